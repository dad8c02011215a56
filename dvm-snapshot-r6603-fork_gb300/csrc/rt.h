// Internal declarations of libdvmh_gb: the GB300 loop-execution runtime.
//
// One process, one GPU.  Device 0 is the host, device 1 the GPU (the
// reference's numbering: rts/dvmh/dvmh_rts.cpp:487-520).  Distributed arrays
// live in pinned host memory and in one device buffer each; actuality is kept
// per array as two flags (host copy current / device copy current) because on
// one device the reference's rectangle sets (rts/dvmh/dvmh_pieces.cpp) only
// ever describe the whole local part.  Loops run through the CUDA handler the
// program registered, on the runtime's stream, in one of three modes:
//   plain    - each loop launched when performed, reduction results copied to
//              the host variable and the stream synchronised at loop end (the
//              reference's per-loop model, rts/dvmh/loop.cpp:2235-2240);
//   async    - each loop launched when performed, reduction results stay on
//              the device until get_actual, no per-loop synchronisation;
//   batched  - loops are queued; at the next synchronisation point the queue
//              (fused where a fusion rule applies) is captured once as a CUDA
//              graph, cached by its signature and replayed afterwards.
#pragma once

#include <cuda_runtime.h>

#include <cstdarg>
#include <cstddef>
#include <cstdint>
#include <cstdio>
#include <map>
#include <string>
#include <vector>

#include "../../include/dvmhlib2.h"
#include "../../include/dvmh_gb.h"

namespace dvmhgb {

constexpr int MAXR = 7;  // maximum array/loop rank (the reference's MAX_ARRAY_RANK)
constexpr int TUNE_NF = 24;  // features per tuner record (DVMHGB_TUNE_NF)

// ---------------------------------------------------------------- errors

[[noreturn]] void fatal(const char *kind, const char *file, int line, const char *fmt, ...);
#define GB_CHECK(cond, ...)                                                         \
    do {                                                                            \
        if (!(cond)) ::dvmhgb::fatal("error", __FILE__, __LINE__, __VA_ARGS__);     \
    } while (0)
#define GB_INTERNAL(cond, ...)                                                      \
    do {                                                                            \
        if (!(cond)) ::dvmhgb::fatal("internal", __FILE__, __LINE__, __VA_ARGS__);  \
    } while (0)
#define GB_CUDA(call)                                                               \
    do {                                                                            \
        cudaError_t e_ = (call);                                                    \
        if (e_ != cudaSuccess)                                                      \
            ::dvmhgb::fatal("cuda", __FILE__, __LINE__, "%s: %s", #call, cudaGetErrorString(e_)); \
    } while (0)

void logmsg(int level, const char *fmt, ...);
enum { LOG_ERROR = 1, LOG_WARN = 2, LOG_INFO = 3, LOG_DEBUG = 4, LOG_TRACE = 5 };

// ---------------------------------------------------------------- settings

enum Mode { MODE_PLAIN = 0, MODE_ASYNC = 1, MODE_BATCHED = 2 };

struct Settings {
    int mode = MODE_BATCHED;
    int logLevel = LOG_ERROR;
    bool syncEachLoop = false;  // DVMH_SYNC_CUDA: synchronise after every loop
    int tuneMode = 0;           // 0 off, 1 exhaustive, 2 model-guided (DVMH_OPT_PARAMS)
    int graphCacheMax = 64;
    bool fuse = true;
    bool defer = true;          // DVMH_GB_DEFER: loops that start a fusion rule may wait in the queue for their second
    bool hostProf = false;      // DVMH_GB_HOSTPROF: time the ABI entry points on the host
    bool autoTfm = true;        // DVMH_GB_AUTOTFM: honour dvmh_loop_autotransform_C (else keep natural layouts)
    bool reduceDeps = false;    // DVMH_REDUCE_DEPS: no dependence on ACROSS axes with one iteration
};
extern Settings settings;

// ---------------------------------------------------------------- host profile
//
// With DVMH_GB_HOSTPROF=1 every profiled entry point accumulates its calls and
// inclusive wall time (steady clock); the table is printed to stderr at exit
// or by dvmhgb_hostprof_dump().  Off, a scope costs one branch.
int profId(const char *name);
struct ProfScope {
    int id;
    long long t0;
    explicit ProfScope(int i);
    ~ProfScope();
};
#define GB_PROF(name)                                                \
    static const int gbProfId_ = ::dvmhgb::profId(name);             \
    ::dvmhgb::ProfScope gbProfScope_(gbProfId_)

// ---------------------------------------------------------------- objects

enum ObjKind : uint32_t {
    K_ARRAY = 0x41525259u,
    K_TEMPLATE = 0x54454d50u,
    K_VAR = 0x56415220u,
    K_REGION = 0x5245474eu,
    K_LOOP = 0x4c4f4f50u,
    K_SPEC = 0x53504543u,
    K_DECL = 0x4445434cu,
};

struct Obj {
    uint32_t kind;
    explicit Obj(uint32_t k) : kind(k) {}
    virtual ~Obj() { kind = 0; }
};

// How the axes of an array, a template or a loop's mapping correspond to the
// axes of the distribution root they are (transitively) aligned with: root
// axis r holds own axis ax[r] (1-based, 0 = none), in direction sign[r].
struct AlignMap {
    const Obj *root = nullptr;
    int rank = 0;  // root rank
    int ax[MAXR] = {};
    int sign[MAXR] = {};
};

struct Array : Obj {
    Array() : Obj(K_ARRAY) {}
    int rank = 0;
    int dtype = rt_UNKNOWN;  // rt_* or rt_UNKNOWN for sized types
    size_t esize = 0;
    long ext[MAXR] = {};
    long shLo[MAXR] = {}, shHi[MAXR] = {};
    bool distributed = false;
    // host copy: dense, pinned
    long hstride[MAXR] = {};
    size_t helems = 0;
    char *host = nullptr;
    // device copy: innermost axis padded to 32 elements (256 B rows for FP64)
    long dstride[MAXR] = {};
    size_t delems = 0;
    char *dev = nullptr;
    char *devAlt = nullptr;  // second buffer for double-buffered (fused) loops and relayouts
    // device layout: natural (tperm all zero) or transformed (rt_layout.h):
    // stored position k holds axis tperm[k] (1-based); tdiag 1 / 2 = the last
    // two stored axes diagonalised (2: slash orientation)
    int tperm[MAXR] = {};
    int tdiag = 0;
    AlignMap align;  // set by dvmh_distribute_C / dvmh_align_C
    bool hostActual = true, devActual = false;
    DvmType *desc = nullptr;
    // a regular variable of the program seen as an array (dvmh_variable_gen_header_C):
    // the host copy is the program's own memory (neither pinned nor freed here) and
    // the header is the runtime's
    bool extHost = false;
    DvmType ownHdr[MAXR + 3] = {};
    std::string name;
    const void *regMark = nullptr;  // the region this array was last registered in
    size_t regIdx = 0;              // and its entry there
    size_t hostBytes() const { return helems * esize; }
    size_t devBytes() const { return delems * esize; }
};

struct Templ : Obj {
    Templ() : Obj(K_TEMPLATE) {}
    int rank = 0;
    long ext[MAXR] = {};
    AlignMap align;  // itself, identity
};

// A regular (non-distributed) variable known to the runtime: scalars and
// blobs registered in regions, reduction variables.
struct Var : Obj {
    Var() : Obj(K_VAR) {}
    const char *addr = nullptr;
    size_t size = 0;
    char *dev = nullptr;
    bool hostActual = true, devActual = false;
    std::string name;
    DvmType hdr[4] = {};  // its rank-0 header (dvmh_variable_gen_header_C with rank 0): hdr[0] = this
};

// An array declared without its size (dvmh_array_declare_C); dvmh_array_alloc_C
// turns it into an Array once the program allocates it.
struct Decl : Obj {
    Decl() : Obj(K_DECL) {}
    int rank = 0;
    DvmType typeSize = 0;
    long ext[MAXR] = {}, shLo[MAXR] = {}, shHi[MAXR] = {};
};

struct Region;
struct Loop;

struct HandlerRef {
    DvmHandlerFunc func = nullptr;
    int nparams = 0;
    void *params[64];
};

struct Reduction {
    int op = 0;        // rf_*
    int vtype = 0;     // rt_*
    size_t esize = 0;  // element size of the value type
    long count = 1;    // array length of the reduction variable
    char *addr = nullptr;
    char *locAddr = nullptr;
    long locSize = 0;
    std::vector<char> init, initLoc;  // host snapshot (reference: DvmhReduction ctor, loop.cpp:17-35)
    Var *var = nullptr;               // registered variable holding addr (device-resident result)
    size_t varOff = 0;
    Var *locVar = nullptr;
    size_t locVarOff = 0;
};

struct Across {
    Array *arr;
    bool isOut;
    long lo[MAXR], hi[MAXR];
};

struct Loop : Obj {
    Loop() : Obj(K_LOOP) {}
    Region *region = nullptr;
    int rank = 0;
    long lo[MAXR] = {}, hi[MAXR] = {}, step[MAXR] = {};
    bool empty = false;
    Array *mapArr = nullptr;
    int arrAxisToLoop[MAXR] = {};  // array axis -> loop axis (1-based), 0 = none
    AlignMap map;                  // distribution root axis -> loop axis (dvmh_loop_map_C)
    std::vector<Reduction> reds;
    std::vector<Across> across;
    long depMask = 0;
    int cudaBlock[3] = {0, 0, 0};
    bool userBlock = false;
    long stage = 0;
    HandlerRef host, cuda;
    bool hasHost = false, hasCuda = false;
    std::string file;
    long line = 0;
    size_t regionElems = 0;  // the most elements of the region's arrays (a queued loop may outlive its region)
};

struct RegionVar {
    Var *var;
    long intent;
};
struct RegionArr {
    Array *arr;
    long intent;
};

struct Region : Obj {
    Region() : Obj(K_REGION) {}
    long flags = 0;
    long targets = 0;
    std::vector<RegionArr> arrays;
    std::vector<RegionVar> vars;
    bool started = false;
};

// Device-side storage of one registered reduction during a handler call.
struct CudaRed {
    int index = 0;  // 1-based
    void **arrPtrSlot = nullptr, **locPtrSlot = nullptr;
    char *items = nullptr, *locItems = nullptr;
    long count = 0;
    bool finished = false;
};

// The loop reference handed to a handler (the reference's DvmhLoopCuda, loop.h:420-473).
struct SpecLoop : Obj {
    SpecLoop() : Obj(K_SPEC) {}
    Loop *loop = nullptr;
    int device = 1;
    cudaStream_t stream = nullptr;
    int block[3] = {0, 0, 0};
    int variant = -1;  // tuner's kernel variant, -1 = handler default
    int layout = -1;   // tuner's layout choice for autotransform (1 transform, 0 natural), -1 none
    void *handler = nullptr;  // the handler running this execution (single, fused or batch)
    uint64_t tkey = 0;        // the tuner's key of this loop shape and handler (0: no variant asked)
    bool exploring = false;   // the variant is one the tuner had not timed yet
    float vf[TUNE_NF] = {};   // features of the loop and the chosen variant
    std::vector<CudaRed> reds;
    std::vector<void *> scratch;  // device allocations owned by this execution
    std::vector<void *> hostScratch;  // pinned host allocations owned by this execution
    std::vector<Array *> swaps;   // arrays whose device buffers swap at loop end
};

// ---------------------------------------------------------------- device layer (rt_device.cu)

struct LayoutDesc;
void launchRelayout(const char *src, const LayoutDesc &from, char *dst, const LayoutDesc &to, size_t esize,
                    cudaStream_t s);

struct Device {
    int ordinal = -1;
    cudaDeviceProp prop{};
    cudaStream_t stream = nullptr;
    int smCount = 0;
    bool ready = false;
    int *statusHost = nullptr;  // mapped pinned word: 0 = fine, else the error a kernel reported
    int *statusDev = nullptr;
};
extern Device gpu;

void deviceInit();
void deviceFinish();
void *devAlloc(size_t bytes);        // caching pool, 256-byte aligned
void devFree(void *p);               // back to the pool
void *hostAlloc(size_t bytes);       // pinned
void hostFree(void *p);
void copyH2D(Array *a);              // whole array, on the stream
void copyD2H(Array *a);              // whole array, on the stream + sync
void copyBoxH2D(Array *a, const long lo[], const long hi[]);
void copyBoxD2H(Array *a, const long lo[], const long hi[]);
void streamSync();

// reduction fold (canonical tree) writing the final value to dst / dstLoc
void launchRedFold(int op, int vtype, long count, long elemCount, const void *items, const void *locItems,
                   long locSize, void *dst, void *dstLoc, cudaStream_t s, std::vector<void *> &scratch);
void fillIdentity(int op, int vtype, void *items, long n, cudaStream_t s);
// one deferred reduction fold (batched handlers): FP64, one element
struct FoldJob {
    int op;
    long count;
    const void *items, *locItems;
    long locSize;
    void *dst, *dstLoc;
    long blockBase;  // first of this job's 2048-item spans in the batch (set by launchRedFoldBatch)
};
bool foldBatchable(int op, int vtype, long count, long elemCount);
void launchRedFoldBatch(const std::vector<FoldJob> &jobs, cudaStream_t s, std::vector<void *> &devScratch,
                        std::vector<void *> &hostScratch);
void identityValue(int op, int vtype, void *out);
size_t typeSize(int vtype);

// ---------------------------------------------------------------- runtime state (rt_core.cpp)

struct State {
    bool inited = false;
    Region *curRegion = nullptr;
    Loop *curLoop = nullptr;
    std::map<const char *, Var *> vars;  // by start address
    std::string file;
    long line = 0;
};
extern State st;

Array *arrayOf(const DvmType desc[], const char *what);
Var *varAt(const void *addr, size_t *off);           // registered variable containing addr, or null
Var *varGet(const void *addr, size_t size);          // existing or new variable for [addr, addr+size)
void ensureDevBuffer(Array *a);
void ensureDevActual(Array *a);
void ensureHostActual(Array *a);
void ensureVarDev(Var *v);
void varH2D(Var *v);
void varD2H(Var *v);
void varForgetStaging(const Var *v);  // the variable is dropped: its pinned staging buffer too
void fillDesc(Array *a);
size_t maxDeviceElems();  // the most device elements of any live array with a device copy
bool isLive(Obj *o, uint32_t kind);
void trackObj(Obj *o);
void untrackObj(Obj *o);
void varDrop(Var *v);     // forget a variable, its device copy and the graphs that name it
bool varInRegion(const Var *v);  // registered in the current region
// a new array on the caller's descriptor, or on its own header for desc == null
// (sizes per axis, shadow widths); no storage yet
Array *arrayNew(DvmType desc[], int rank, DvmType typeSize, const long ext[], const long shLo[], const long shHi[]);
// host storage: `external` (the program's memory) or a pinned buffer of the runtime
void arrayAttachHost(Array *a, char *external);
void arrayRelease(Array *a);  // free the array's buffers and the object (its descriptor is cleared)
void arrayRetarget(Array *a, DvmType desc[]);  // the array is known by another descriptor from now on

// ---------------------------------------------------------------- regular variables (rt_regular.cpp)

// Regular (non-distributed) variables entered into data regions
// (dvmh_data_enter_C / dvmh_data_exit_C) and their runtime forms.
bool regularActual(const void *addr, bool toHost);  // get_actual / actual of a regular array; false if unknown
void regularRegionEnd();  // data exit of the variables a region (or a loop outside regions) entered implicitly

// ---------------------------------------------------------------- loops / batching (rt_loop.cpp)

void queueFlush();  // run or replay everything queued (batched mode)
// run the queued loops up to the last one that names v (a parameter or a
// reduction variable); later loops stay queued
void queueFlushVar(const Var *v);
// the same for the last queued loop that names any variable (a region's end:
// loops over arrays alone may stay queued past it)
void queueFlushVars();
void queueRegionEnded(const Region *r);  // queued loops of an ended region forget it
Var *regularVarOfHeader(const void *p);  // the rank-0 regular variable whose header p is, or null
bool queueBusy();
void loopsAtExit();
void graphsForget(const Obj *a);  // drop the cached graphs that name a freed array or variable
void noteSwap(Array *a);          // a device buffer swap, recorded when a graph is being captured
void noteLayout(Array *a);        // a layout change, likewise
bool inHandlerCall();             // a handler is running
bool transformedInCall(const Array *a);  // autotransformed by the handler running now

// ---------------------------------------------------------------- device layouts (rt_layout.cpp)

bool layoutNatural(const Array *a);
// make the device copy natural again (before copies and hand-written kernels)
void makeNatural(Array *a);
// the reference's choice of layout for an ACROSS loop's array; returns the
// state dvmh_fill_header_C reports (0 natural, 1 permuted, 2 diagonalised)
int autotransform(const Loop *l, Array *a);
int layoutState(const Array *a);
// the loop axis (1-based) that array axis `axis` (0-based) follows, 0 if none
int loopAxisOf(const Loop *l, const Array *a, int axis);
// header coefficients and diagonal parameters of the current device layout
void layoutHeader(const Array *a, long coef[], long ext7[7]);
void alignIdentity(AlignMap &m, const Obj *self, int rank);
const AlignMap *alignOf(const DvmType desc[]);  // of an array or template descriptor (rt_core.cpp)
void alignCompose(AlignMap &out, const AlignMap &target, const int axis[], const int sign[], int targetRank);

// ---------------------------------------------------------------- tuner (rt_tuner.cpp)

bool tunerWants(const Loop *l);  // record timings of this loop shape
// the variant for this execution; sets s->tkey, s->exploring and s->vf
int tunerVariant(SpecLoop *s, int nvariants, int dflt, const float *desc, int ndesc, bool bestOnly);
void tunerPick(Loop *l, int block[3], int *variant);
// a timed execution of a variant-choosing handler
void tunerRecord(uint64_t key, int variant, bool exploring, const float *vf, double seconds);
bool tunerExploring();  // a flush must run without capture: some loop shape still tries variants
void tunerFlushed();    // an uncaptured flush ran
int tunerLayout(const Loop *l, bool explore);  // 1: the reference's transform, 0: natural
void tunerRecordLayout(const Loop *l, int choice, double seconds);

}  // namespace dvmhgb
