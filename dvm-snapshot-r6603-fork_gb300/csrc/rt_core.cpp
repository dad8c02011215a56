// libdvmh_gb core: init/exit, distributed arrays and their descriptors,
// actuality of arrays and variables, shadow renew, regions.
//
// Reference behaviour followed (rts/dvmh/...):
//   dvmh_array_create_C       dvmh2.cpp:546-570  sizes/shadows from varargs, index space [0, size)
//   dvmh_distribute_C/align_C dvmh2.cpp:1330,1564 on one process BLOCK is the identity: the local
//                             part is the whole array, shadows clipped to the bounds
//                             (DvmhData::extendBlock, dvmh_data.cpp:311-320)
//   dvmh_fill_header_C        dvmh_buffer.cpp:149-182 header = {handle, strides[1..rank],
//                             offset of natural base from baseAddr, baseAddr}
//   dvmh_get_natural_base_C   dvmh2.cpp:2190-2203
//   actual / get_actual       dvmh2.cpp:2273-2499 (host copy declared current / made current)
//   dvmh_shadow_renew_C       dvmh2.cpp:2539-2607; with one process the edge set is empty
//                             (doWithEveryEdge, dvmh_data.cpp:373-406): bookkeeping only
//   regions                   dvmh2.cpp:3002-3134, region.cpp:468-578,961
#include <algorithm>
#include <cerrno>
#include <cstdlib>
#include <cstring>
#include <ctime>
#include <unordered_map>
#include <unordered_set>

#include "rt.h"

namespace dvmhgb {

Settings settings;
State st;
std::unordered_set<Obj *> liveObjs;
dvmhgb_stats_t stats;

void fatal(const char *kind, const char *file, int line, const char *fmt, ...) {
    char buf[1024];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof buf, fmt, ap);
    va_end(ap);
    const char *base = strrchr(file, '/');
    fprintf(stderr, "libdvmh_gb %s at %s:%ld (%s:%d): %s\n", kind, st.file.empty() ? "?" : st.file.c_str(), st.line,
            base ? base + 1 : file, line, buf);
    fflush(stderr);
    // DVMH_GB_ERROR_LOG: the same line appended to a file (for hosts that capture stderr)
    if (const char *path = getenv("DVMH_GB_ERROR_LOG")) {
        if (FILE *f = fopen(path, "a")) {
            fprintf(f, "libdvmh_gb %s at %s:%ld (%s:%d): %s\n", kind, st.file.empty() ? "?" : st.file.c_str(),
                    st.line, base ? base + 1 : file, line, buf);
            fclose(f);
        }
    }
    // reference convention: user errors exit(1), internal errors abort (rts/dvmh/dvmh_log.h:75-100)
    if (!strcmp(kind, "internal"))
        abort();
    exit(1);
}

void logmsg(int level, const char *fmt, ...) {
    if (level > settings.logLevel)
        return;
    va_list ap;
    va_start(ap, fmt);
    fprintf(stderr, "[dvmh_gb] ");
    vfprintf(stderr, fmt, ap);
    fprintf(stderr, "\n");
    va_end(ap);
}

// ---------------------------------------------------------------- host profile

namespace {
struct ProfEntry {
    const char *name;
    long calls;
    long long ns;
};
ProfEntry profTable[128];
int profCount = 0;
long long nowNs() {
    struct timespec ts;
    clock_gettime(CLOCK_MONOTONIC, &ts);
    return (long long)ts.tv_sec * 1000000000LL + ts.tv_nsec;
}
void profAtExit() {
    if (settings.hostProf) dvmhgb_hostprof_dump();
}
}  // namespace

int profId(const char *name) {
    if (profCount == 0) atexit(profAtExit);
    if (profCount >= 128) return -1;
    profTable[profCount] = {name, 0, 0};
    return profCount++;
}

ProfScope::ProfScope(int i) : id(settings.hostProf ? i : -1), t0(0) {
    if (id >= 0) t0 = nowNs();
}

ProfScope::~ProfScope() {
    if (id >= 0) {
        profTable[id].calls++;
        profTable[id].ns += nowNs() - t0;
    }
}

size_t typeSize(int vtype) {
    switch (vtype) {
        case rt_CHAR: case rt_UCHAR: return 1;
        case rt_SHORT: case rt_USHORT: return 2;
        case rt_INT: case rt_UINT: case rt_FLOAT: case rt_LOGICAL: return 4;
        case rt_LONG: case rt_ULONG: return sizeof(long);
        case rt_LLONG: case rt_ULLONG: case rt_DOUBLE: case rt_FLOAT_COMPLEX: return 8;
        case rt_DOUBLE_COMPLEX: return 16;
        case rt_POINTER: return sizeof(void *);
        default: return 0;
    }
}

static void loadSettings() {
    const char *m = getenv("DVMH_GB_MODE");
    if (m) {
        if (!strcmp(m, "plain") || !strcmp(m, "0")) settings.mode = MODE_PLAIN;
        else if (!strcmp(m, "async") || !strcmp(m, "1")) settings.mode = MODE_ASYNC;
        else if (!strcmp(m, "batched") || !strcmp(m, "2")) settings.mode = MODE_BATCHED;
        else GB_CHECK(false, "DVMH_GB_MODE must be plain, async or batched (got '%s')", m);
    }
    if (const char *l = getenv("DVMH_LOGLEVEL")) settings.logLevel = atoi(l);
    if (const char *s = getenv("DVMH_SYNC_CUDA")) settings.syncEachLoop = atoi(s) != 0;
    if (const char *t = getenv("DVMH_OPT_PARAMS")) settings.tuneMode = atoi(t);
    if (const char *h = getenv("DVMH_GB_HOSTPROF")) settings.hostProf = atoi(h) != 0;
    if (const char *f = getenv("DVMH_GB_FUSE")) settings.fuse = atoi(f) != 0;
    if (const char *f = getenv("DVMH_GB_DEFER")) settings.defer = atoi(f) != 0;
    if (const char *t = getenv("DVMH_GB_AUTOTFM")) settings.autoTfm = atoi(t) != 0;
    if (const char *r = getenv("DVMH_REDUCE_DEPS")) settings.reduceDeps = atoi(r) != 0;
}

static void track(Obj *o) { liveObjs.insert(o); }
static void untrack(Obj *o) { liveObjs.erase(o); }
bool isLive(Obj *o, uint32_t kind) { return o && liveObjs.count(o) && o->kind == kind; }
void trackObj(Obj *o) { track(o); }
void untrackObj(Obj *o) { untrack(o); }

Array *arrayOf(const DvmType desc[], const char *what) {
    GB_CHECK(desc, "NULL descriptor passed to %s", what);
    Obj *o = (Obj *)desc[0];
    GB_CHECK(isLive(o, K_ARRAY), "%s: descriptor does not refer to a distributed array", what);
    return (Array *)o;
}

// descriptors of the live arrays: handler parameters are checked against this
// registry before any dereference (one hash lookup per parameter)
// (a count: a descriptor's storage may be reused by a new array before the old one is freed)
static std::unordered_map<const void *, int> arrayDescs;

bool isArrayDesc(const void *p) { return arrayDescs.count(p) != 0; }

// ---------------------------------------------------------------- variables

Var *varAt(const void *addr, size_t *off) {
    const char *a = (const char *)addr;
    auto it = st.vars.upper_bound(a);
    if (it == st.vars.begin())
        return nullptr;
    --it;
    Var *v = it->second;
    if (a >= v->addr && a < v->addr + v->size) {
        if (off) *off = (size_t)(a - v->addr);
        return v;
    }
    return nullptr;
}

// forget a variable: its cached graphs, its device copy, its registry entry
static void dropVar(Var *v) {
    streamSync();
    graphsForget(v);
    if (v->dev) devFree(v->dev);
    varForgetStaging(v);
    st.vars.erase(v->addr);
    untrack(v);
    delete v;
}

void varDrop(Var *v) { dropVar(v); }

// A variable known from an earlier region is forgotten because the program
// registers other memory over it.  Its device copy may not hold the only
// current value: the program must have read it back (get_actual) or ended its
// data region first.  The reference reports a changed or overlapping regular
// variable as an error too (rts/dvmh/dvmh2.cpp:1794-1830).
static void checkForgettable(const Var *v, const char *what, const void *addr) {
    GB_CHECK(!v->dev || v->hostActual,
             "%s at %p: the variable '%s' registered there by an earlier region (%zu bytes at %p) has its only "
             "current value on the device; read it back (get_actual) before registering other memory over it",
             what, addr, v->name.c_str(), v->size, (const void *)v->addr);
}

static bool inCurrentRegion(const Var *v) {
    if (st.curRegion)
        for (auto &rv : st.curRegion->vars)
            if (rv.var == v) return true;
    return false;
}

bool varInRegion(const Var *v) { return inCurrentRegion(v); }

// Variables known from earlier regions and loops that overlap [lo, hi), other
// than `keep`: the program's memory there now holds something else, so unless
// the current region registered them they are forgotten, device copies and
// cached graphs with them.
static void dropOverlaps(const char *lo, const char *hi, const Var *keep) {
    auto first = st.vars.upper_bound(lo);
    if (first != st.vars.begin()) --first;
    std::vector<Var *> stale;
    for (auto it = first; it != st.vars.end() && it->first < hi; ++it)
        if (it->second != keep && it->second->addr + it->second->size > lo) stale.push_back(it->second);
    if (stale.empty()) return;
    queueFlush();  // queued loops may still name them
    for (Var *o : stale) {
        GB_CHECK(!inCurrentRegion(o), "variable at %p overlaps the variable '%s' registered in this region",
                 (const void *)lo, o->name.c_str());
        checkForgettable(o, "a variable overlapping it is registered", lo);
        dropVar(o);
    }
}

Var *varGet(const void *addr, size_t size) {
    const char *lo = (const char *)addr, *hi = lo + size;
    auto it = st.vars.find(lo);
    if (it != st.vars.end()) {
        Var *v = it->second;
        // the same extent, or a smaller one inside what this region registered: the same variable
        if (size == v->size || (size < v->size && inCurrentRegion(v))) return v;
        if (size > v->size && inCurrentRegion(v)) {
            // this region registers more of it: the device copy is made anew
            GB_CHECK(!v->dev || v->hostActual, "variable at %p grows (%zu -> %zu bytes) while its device copy is "
                     "newer than the program's", addr, v->size, size);
            dropOverlaps(v->addr + v->size, hi, v);
            if (v->dev) devFree(v->dev);
            v->dev = nullptr;
            v->size = size;
            v->devActual = false;
            v->hostActual = true;
            return v;
        }
        // a different extent at an address known from an earlier region: the program's
        // memory holds a new variable there (an allocation reused), so the old one is
        // forgotten with the others it overlaps; keeping it would copy its old size back
        checkForgettable(v, "a variable of another size is registered", addr);
    }
    dropOverlaps(lo, hi, nullptr);
    Var *v = new Var();
    v->addr = (const char *)addr;
    v->size = size;
    track(v);
    st.vars[v->addr] = v;
    return v;
}

void ensureVarDev(Var *v) {
    if (!v->dev) {
        v->dev = (char *)devAlloc(std::max<size_t>(v->size, 16));
        v->devActual = false;
    }
}

// ---------------------------------------------------------------- arrays

static long roundUp(long v, long m) { return (v + m - 1) / m * m; }

void fillDesc(Array *a) {
    // cdvmh-generated code reads the outer strides from desc[1..rank-1]
    // (converter_main.cpp:1561-1573); the innermost stride is 1.
    DvmType *d = a->desc;
    d[0] = (DvmType)a;
    for (int i = 0; i < a->rank - 1; i++)
        d[i + 1] = a->hstride[i];
    d[a->rank] = 0;
    d[a->rank + 1] = (DvmType)a->host;
}

static void layout(Array *a) {
    long c = 1;
    for (int i = a->rank - 1; i >= 0; i--) {
        a->hstride[i] = c;
        c *= a->ext[i];
    }
    a->helems = (size_t)c;
    // device rows: 16-byte multiple always (vector loads), 256-byte multiple once a row reaches 256 bytes
    long inner = a->ext[a->rank - 1];
    long rowBytes = inner * (long)a->esize;
    long padBytes = a->rank == 1 ? rowBytes : (rowBytes >= 256 ? roundUp(rowBytes, 256) : roundUp(rowBytes, 16));
    long innerPad = (padBytes + (long)a->esize - 1) / (long)a->esize;
    c = 1;
    for (int i = a->rank - 1; i >= 0; i--) {
        a->dstride[i] = c;
        c *= (i == a->rank - 1) ? innerPad : a->ext[i];
    }
    a->delems = (size_t)c;
}

void arrayAttachHost(Array *a, char *external) {
    if (a->host)
        return;
    layout(a);
    if (external) {
        a->host = external;
        a->extHost = true;
    } else {
        size_t bytes = std::max<size_t>(a->hostBytes(), 16);
        a->host = (char *)hostAlloc(bytes);
        memset(a->host, 0, bytes);
    }
    a->distributed = true;
    a->hostActual = true;
    a->devActual = false;
    fillDesc(a);
}

static void allocateHost(Array *a) { arrayAttachHost(a, nullptr); }

void ensureDevBuffer(Array *a) {
    GB_CHECK(a->distributed, "array '%s' is used before it is distributed or aligned", a->name.c_str());
    if (!a->dev) {
        a->dev = (char *)devAlloc(std::max<size_t>(a->devBytes(), 16));
        a->devActual = false;
    }
}

void ensureDevActual(Array *a) {
    ensureDevBuffer(a);
    if (!a->devActual) {
        GB_INTERNAL(a->hostActual, "array '%s' has no current copy", a->name.c_str());
        queueFlush();
        copyH2D(a);
        a->devActual = true;
    }
}

void ensureHostActual(Array *a) {
    if (!a->hostActual) {
        GB_INTERNAL(a->dev && a->devActual, "array '%s' has no current copy", a->name.c_str());
        queueFlush();
        copyD2H(a);
        a->hostActual = true;
    }
}

size_t maxDeviceElems() {
    size_t m = 0;
    for (Obj *o : liveObjs)
        if (o->kind == K_ARRAY && ((Array *)o)->dev) m = std::max(m, ((Array *)o)->delems);
    return m;
}

// ---------------------------------------------------------------- helpers

struct AlignHelper {
    uint32_t magic;
    long axis, mult, summand;
};
static const uint32_t ALIGN_MAGIC = 0x414c4e31u;

static bool boxFromVa(Array *a, long rank, va_list &ap, long lo[], long hi[]) {
    GB_CHECK(rank == a->rank, "rank %ld given for the %d-dimensional array '%s'", rank, a->rank, a->name.c_str());
    bool whole = true;
    for (int i = 0; i < a->rank; i++) {
        long l = (long)va_arg(ap, DvmType), h = (long)va_arg(ap, DvmType);
        lo[i] = (l == (long)UNDEF_BOUND) ? 0 : l;
        hi[i] = (h == (long)UNDEF_BOUND) ? a->ext[i] - 1 : h;
        GB_CHECK(lo[i] >= 0 && hi[i] < a->ext[i], "index out of bounds for array '%s' on axis %d", a->name.c_str(),
                 i + 1);
        if (lo[i] > hi[i]) return false;
        whole = whole && lo[i] == 0 && hi[i] == a->ext[i] - 1;
    }
    return true;
}

// The alignment target's axes, or null for an unknown or undistributed target.
const AlignMap *alignOf(const DvmType desc[]) {
    if (!desc) return nullptr;
    Obj *o = (Obj *)desc[0];
    if (isLive(o, K_ARRAY)) return ((Array *)o)->align.root ? &((Array *)o)->align : nullptr;
    if (isLive(o, K_TEMPLATE)) return &((Templ *)o)->align;
    return nullptr;
}

}  // namespace dvmhgb

using namespace dvmhgb;

extern "C" {

// ---------------------------------------------------------------- init / exit

void dvmh_line_C(DvmType lineNumber, const char fileName[]) {
    st.line = (long)lineNumber;
    if (fileName) st.file = fileName;
}

void dvmh_init_C(DvmType flags, int *pArgc, char ***pArgv) {
    (void)flags;
    (void)pArgc;
    (void)pArgv;
    if (st.inited)
        return;
    loadSettings();
    deviceInit();
    st.inited = true;
    logmsg(LOG_INFO, "initialised on %s (%d SMs), mode %d", gpu.prop.name, gpu.smCount, settings.mode);
    DvmhModuleInitializer::executeInit();  // data enter of the translation units' global variables
}

void dvmh_exit_C(DvmType exitCode) {
    if (st.inited) {
        queueFlush();
        DvmhModuleInitializer::executeFinish();  // data exit of the global variables
        streamSync();
        loopsAtExit();
    }
    fflush(stdout);
    exit((int)exitCode);
}

double dvmh_wtime(void) {
    struct timespec ts;
    clock_gettime(CLOCK_MONOTONIC, &ts);
    return ts.tv_sec + ts.tv_nsec * 1e-9;
}

void dvmh_barrier(void) {
    if (st.inited) {
        queueFlush();
        streamSync();
    }
}

// ---------------------------------------------------------------- arrays, templates, distribution

}  // extern "C"

namespace dvmhgb {

Array *arrayNew(DvmType dvmDesc[], int rank, DvmType typeSize, const long ext[], const long shLo[],
                const long shHi[]) {
    GB_CHECK(rank > 0 && rank <= MAXR, "array rank must be in 1..%d (got %d)", MAXR, rank);
    Array *a = new Array();
    if (!dvmDesc) dvmDesc = a->ownHdr;  // the runtime's own header (a regular variable's array form)
    a->rank = rank;
    if (typeSize <= 0) {
        a->dtype = (int)-typeSize;
        a->esize = dvmhgb::typeSize(a->dtype);
        GB_CHECK(a->esize > 0, "unknown data type %ld", (long)-typeSize);
    } else {
        a->esize = (size_t)typeSize;
    }
    for (int i = 0; i < rank; i++) {
        a->ext[i] = ext[i];
        a->shLo[i] = shLo[i];
        a->shHi[i] = shHi[i];
        GB_CHECK(a->ext[i] > 0, "non-positive size %ld of array on axis %d", a->ext[i], i + 1);
        GB_CHECK(a->shLo[i] >= 0 && a->shHi[i] >= 0, "negative shadow width on axis %d", i + 1);
    }
    a->desc = dvmDesc;
    dvmDesc[0] = (DvmType)a;
    track(a);
    arrayDescs[dvmDesc]++;
    return a;
}

void arrayRelease(Array *a) {
    queueFlush();
    streamSync();
    graphsForget(a);
    if (a->dev) devFree(a->dev);
    if (a->devAlt) devFree(a->devAlt);
    if (a->host && !a->extHost) hostFree(a->host);
    untrack(a);
    if (--arrayDescs[a->desc] <= 0) arrayDescs.erase(a->desc);
    a->desc[0] = 0;
    delete a;
}

void arrayRetarget(Array *a, DvmType desc[]) {
    if (--arrayDescs[a->desc] <= 0) arrayDescs.erase(a->desc);
    a->desc = desc;
    arrayDescs[desc]++;
    if (a->host) fillDesc(a);
    else desc[0] = (DvmType)a;
}

}  // namespace dvmhgb

extern "C" {

void dvmh_array_create_C(DvmType dvmDesc[], DvmType rank, DvmType typeSize, ...) {
    GB_CHECK(st.inited, "LibDVMH is not initialized");
    GB_CHECK(!st.curRegion && !st.curLoop, "dvmh_array_create is not allowed in a region or a parallel loop");
    GB_CHECK(dvmDesc, "NULL descriptor passed to dvmh_array_create");
    GB_CHECK(rank > 0 && rank <= MAXR, "array rank must be in 1..%d (got %ld)", MAXR, (long)rank);
    long ext[MAXR], shLo[MAXR], shHi[MAXR];
    va_list ap;
    va_start(ap, typeSize);
    for (int i = 0; i < rank; i++) {
        ext[i] = (long)va_arg(ap, DvmType);
        shLo[i] = (long)va_arg(ap, DvmType);
        shHi[i] = (long)va_arg(ap, DvmType);
    }
    va_end(ap);
    arrayNew(dvmDesc, (int)rank, typeSize, ext, shLo, shHi);
}

void dvmh_template_create_C(DvmType dvmDesc[], DvmType rank, ...) {
    GB_CHECK(st.inited, "LibDVMH is not initialized");
    GB_CHECK(rank > 0 && rank <= MAXR, "template rank must be in 1..%d", MAXR);
    Templ *t = new Templ();
    t->rank = (int)rank;
    va_list ap;
    va_start(ap, rank);
    for (int i = 0; i < t->rank; i++) t->ext[i] = (long)va_arg(ap, DvmType);
    va_end(ap);
    alignIdentity(t->align, t, t->rank);
    dvmDesc[0] = (DvmType)t;
    track(t);
}

DvmType dvmh_distribution_replicated_(void) { return 0; }
DvmType dvmh_distribution_block_C(DvmType mpsAxis) { return mpsAxis; }

void dvmh_distribute_C(DvmType dvmDesc[], DvmType rank, ...) {
    GB_CHECK(dvmDesc, "NULL descriptor passed to dvmh_distribute");
    Obj *o = (Obj *)dvmDesc[0];
    if (isLive(o, K_TEMPLATE))
        return;  // a template has no storage; one process holds all of it
    Array *a = arrayOf(dvmDesc, "dvmh_distribute");
    GB_CHECK(rank == a->rank, "distribution rank %ld differs from array rank %d", (long)rank, a->rank);
    // one process: BLOCK (and every other rule) maps the whole index space here
    allocateHost(a);
    alignIdentity(a->align, a, a->rank);
}

void dvmh_redistribute_C(DvmType dvmDesc[], DvmType rank, ...) {
    Array *a = arrayOf(dvmDesc, "dvmh_redistribute");
    GB_CHECK(rank == a->rank, "distribution rank differs from array rank");
    allocateHost(a);
}

DvmType dvmh_alignment_linear_C(DvmType axis, DvmType multiplier, DvmType summand) {
    GB_PROF("dvmh_alignment_linear_C");
    AlignHelper *h = new AlignHelper{ALIGN_MAGIC, (long)axis, (long)multiplier, (long)summand};
    return (DvmType)h;
}

static AlignHelper takeAlign(DvmType v) {
    AlignHelper *h = (AlignHelper *)v;
    GB_CHECK(h && h->magic == ALIGN_MAGIC, "invalid alignment helper");
    AlignHelper r = *h;
    h->magic = 0;
    delete h;
    return r;
}

void dvmh_align_C(DvmType dvmDesc[], const DvmType templDesc[], DvmType templRank, ...) {
    Array *a = arrayOf(dvmDesc, "dvmh_align");
    GB_CHECK(templRank >= 0 && templRank <= MAXR, "alignment target rank %ld out of range", (long)templRank);
    int axis[MAXR] = {}, sign[MAXR] = {};
    va_list ap;
    va_start(ap, templRank);
    for (long i = 0; i < templRank; i++) {
        AlignHelper h = takeAlign(va_arg(ap, DvmType));
        GB_CHECK(h.axis == -1 || (h.axis >= 0 && h.axis <= a->rank), "alignment axis %ld out of range", h.axis);
        axis[i] = h.axis > 0 ? (int)h.axis : 0;
        sign[i] = h.mult > 0 ? 1 : (h.mult < 0 ? -1 : 0);
    }
    va_end(ap);
    allocateHost(a);
    if (const AlignMap *t = alignOf(templDesc)) alignCompose(a->align, *t, axis, sign, (int)templRank);
}

void dvmh_array_free_C(DvmType dvmDesc[]) {
    Array *a = arrayOf(dvmDesc, "dvmh_array_free");
    GB_CHECK(!st.curRegion, "dvmh_array_free inside a region");
    GB_CHECK(!a->extHost, "dvmh_array_free: '%s' is a regular variable of the program (it leaves the runtime at "
             "dvmh_data_exit)", a->name.c_str());
    arrayRelease(a);
    dvmDesc[0] = 0;
}

void dvmh_delete_object_(DvmType dvmDesc[]) {
    Obj *o = (Obj *)dvmDesc[0];
    if (isLive(o, K_ARRAY)) {
        dvmh_array_free_C(dvmDesc);
    } else if (isLive(o, K_TEMPLATE)) {
        untrack(o);
        dvmDesc[0] = 0;
        delete o;
    }
}

// ---------------------------------------------------------------- addresses and headers

// A handler that did not ask for a transform of this array, and any caller
// outside handlers, gets the natural device layout.
static void deviceNatural(Array *a) {
    if (layoutNatural(a) || transformedInCall(a)) return;
    if (!inHandlerCall()) queueFlush();  // queued loops first, in their layouts
    makeNatural(a);
}

void *dvmh_get_natural_base_C(DvmType deviceNum, const DvmType dvmDesc[]) {
    GB_CHECK(st.inited, "LibDVMH is not initialized");
    GB_CHECK(deviceNum == 0 || deviceNum == 1, "illegal device number %ld", (long)deviceNum);
    Array *a = arrayOf(dvmDesc, "dvmh_get_natural_base");
    if (deviceNum == 0)
        return a->host;
    deviceNatural(a);
    return a->dev;
}

void *dvmh_get_device_addr_C(DvmType deviceNum, const void *addr) {
    GB_CHECK(deviceNum == 0 || deviceNum == 1, "illegal device number %ld", (long)deviceNum);
    if (deviceNum == 0)
        return (void *)addr;
    size_t off = 0;
    Var *v = varAt(addr, &off);
    GB_CHECK(v && v->dev, "can not get the device address of a variable unknown to the region");
    return v->dev + off;
}

// Header of the array as a handler sees it (rts/dvmh/dvmh2.cpp:2226-2258):
// per-axis coefficients of the device layout (zero for the two diagonal
// axes of a diagonalised copy), the offset from the given base, the base.
// Returns 0 natural, 1 permuted, 2 diagonalised; for 2, extendedParams gets
// x axis, x first index, x extent, y axis, y first index, y extent, slash.
DvmType dvmh_fill_header_C(DvmType deviceNum, const void *baseAddr, const DvmType dvmDesc[], DvmType devHeader[],
                           DvmType extendedParams[]) {
    GB_CHECK(deviceNum == 0 || deviceNum == 1, "illegal device number %ld", (long)deviceNum);
    Array *a = arrayOf(dvmDesc, "dvmh_fill_header");
    GB_CHECK(devHeader, "NULL header passed to dvmh_fill_header");
    long coef[MAXR], ext7[7] = {};
    int state = 0;
    if (deviceNum == 0) {
        for (int i = 0; i < a->rank; i++) coef[i] = a->hstride[i];
    } else {
        deviceNatural(a);
        layoutHeader(a, coef, ext7);
        state = layoutState(a);
    }
    const char *buf = deviceNum == 0 ? a->host : a->dev;
    devHeader[0] = (DvmType)a;
    for (int i = 0; i < a->rank; i++) devHeader[i + 1] = coef[i];
    GB_CHECK(((buf - (const char *)baseAddr) % (long)a->esize) == 0,
             "impossible to express the array relative to the given base");
    devHeader[a->rank + 1] = (DvmType)((buf - (const char *)baseAddr) / (long)a->esize);
    devHeader[a->rank + 2] = (DvmType)baseAddr;
    if (extendedParams && state == 2)
        for (int i = 0; i < 7; i++) extendedParams[i] = ext7[i];
    return state;
}

DvmType dvmh_calc_linear_C(const DvmType dvmDesc[], DvmType rank, ...) {
    Array *a = arrayOf(dvmDesc, "dvmh_calc_linear");
    GB_CHECK(rank == a->rank, "rank mismatch in dvmh_calc_linear");
    va_list ap;
    va_start(ap, rank);
    long lin = 0;
    for (int i = 0; i < a->rank; i++) lin += (long)va_arg(ap, DvmType) * a->hstride[i];
    va_end(ap);
    return lin;
}

void *dvmh_get_element_addr_C(const DvmType dvmDesc[], DvmType rank, ...) {
    Array *a = arrayOf(dvmDesc, "dvmh_get_element_addr");
    GB_CHECK(rank == a->rank, "rank mismatch in dvmh_get_element_addr");
    va_list ap;
    va_start(ap, rank);
    long lin = 0;
    for (int i = 0; i < a->rank; i++) {
        long idx = (long)va_arg(ap, DvmType);
        GB_CHECK(idx >= 0 && idx < a->ext[i], "index out of bounds");
        lin += idx * a->hstride[i];
    }
    va_end(ap);
    return a->host + lin * a->esize;
}

// ---------------------------------------------------------------- actuality

void dvmh_get_actual_variable2_(void *addr) {
    GB_PROF("dvmh_get_actual_variable2_");
    if (!st.inited) return;
    auto it = st.vars.find((const char *)addr);
    if (it == st.vars.end()) {
        regularActual(addr, true);  // a regular array; other unknown variables are current on the host
        return;
    }
    Var *v = it->second;
    if (!v->hostActual) {
        varD2H(v);
        v->hostActual = true;
    }
}

void dvmh_actual_variable2_(const void *addr) {
    GB_PROF("dvmh_actual_variable2_");
    if (!st.inited) return;
    auto it = st.vars.find((const char *)addr);
    if (it == st.vars.end()) {
        regularActual(addr, false);
        return;
    }
    Var *v = it->second;
    v->hostActual = true;
    v->devActual = false;
}

void dvmh_get_actual_array2_(const DvmType dvmDesc[]) {
    GB_PROF("dvmh_get_actual_array2_");
    Array *a = arrayOf(dvmDesc, "dvmh_get_actual_array");
    ensureHostActual(a);
}

void dvmh_actual_array2_(const DvmType dvmDesc[]) {
    GB_PROF("dvmh_actual_array2_");
    Array *a = arrayOf(dvmDesc, "dvmh_actual_array");
    GB_CHECK(a->distributed, "array is not distributed");
    a->hostActual = true;
    a->devActual = false;
}

void dvmh_get_actual_subarray_C(const DvmType dvmDesc[], DvmType rank, ...) {
    Array *a = arrayOf(dvmDesc, "dvmh_get_actual_subarray");
    long lo[MAXR], hi[MAXR];
    va_list ap;
    va_start(ap, rank);
    bool nonEmpty = boxFromVa(a, rank, ap, lo, hi);
    va_end(ap);
    if (!nonEmpty || a->hostActual) return;
    queueFlush();
    copyBoxD2H(a, lo, hi);
}

void dvmh_actual_subarray_C(const DvmType dvmDesc[], DvmType rank, ...) {
    Array *a = arrayOf(dvmDesc, "dvmh_actual_subarray");
    long lo[MAXR], hi[MAXR];
    va_list ap;
    va_start(ap, rank);
    bool nonEmpty = boxFromVa(a, rank, ap, lo, hi);
    va_end(ap);
    if (!nonEmpty) return;
    if (a->dev && a->devActual) {
        // keep the device copy whole: push the updated box now
        queueFlush();
        copyBoxH2D(a, lo, hi);
    } else {
        a->hostActual = true;
    }
}

void dvmh_get_actual_all2_(void) {
    for (Obj *o : std::vector<Obj *>(liveObjs.begin(), liveObjs.end())) {
        if (o->kind == K_ARRAY && ((Array *)o)->distributed) ensureHostActual((Array *)o);
        if (o->kind == K_VAR && !((Var *)o)->hostActual) {
            varD2H((Var *)o);
            ((Var *)o)->hostActual = true;
        }
    }
}

void dvmh_actual_all2_(void) {
    for (Obj *o : liveObjs) {
        if (o->kind == K_ARRAY && ((Array *)o)->distributed) {
            ((Array *)o)->hostActual = true;
            ((Array *)o)->devActual = false;
        }
        if (o->kind == K_VAR) {
            ((Var *)o)->hostActual = true;
            ((Var *)o)->devActual = false;
        }
    }
}

// ---------------------------------------------------------------- shadow renew

void dvmh_shadow_renew_C(const DvmType dvmDesc[], DvmType cornerFlag, DvmType specifiedRank, ...) {
    GB_PROF("dvmh_shadow_renew_C");
    (void)cornerFlag;
    Array *a = arrayOf(dvmDesc, "dvmh_shadow_renew");
    GB_CHECK(specifiedRank == 0 || specifiedRank == a->rank, "shadow renew rank mismatch");
    va_list ap;
    va_start(ap, specifiedRank);
    for (long i = 0; i < specifiedRank; i++) {
        long l = (long)va_arg(ap, DvmType), h = (long)va_arg(ap, DvmType);
        GB_CHECK(l >= 0 && h >= 0 && l <= a->shLo[i] && h <= a->shHi[i],
                 "shadow renew widths exceed the declared widths on axis %ld", i + 1);
    }
    va_end(ap);
    // One process, one device copy: every shadow element is an element of the
    // same buffer, current wherever the array is current.  Nothing moves.
}

// ---------------------------------------------------------------- regions

DvmType dvmh_region_create_C(DvmType regionFlags) {
    GB_PROF("dvmh_region_create_C");
    GB_CHECK(st.inited, "LibDVMH is not initialized");
    GB_CHECK(!st.curRegion, "nested regions are not allowed");
    Region *r = new Region();
    r->flags = (long)regionFlags;
    track(r);
    st.curRegion = r;
    return (DvmType)r;
}

static Region *regionOf(DvmType ref, const char *what) {
    Region *r = (Region *)ref;
    GB_CHECK(isLive(r, K_REGION) && r == st.curRegion, "incorrect region reference passed to %s", what);
    return r;
}

static void regionAddVar(Region *r, Var *v, long intent, const char *varName) {
    if (varName && v->name.empty()) v->name = varName;
    for (auto &rv : r->vars)
        if (rv.var == v) {
            rv.intent |= intent;
            return;
        }
    r->vars.push_back({v, intent});
}

void dvmh_region_register_array_C(DvmType curRegion, DvmType intent, const DvmType dvmDesc[], const char varName[]) {
    GB_PROF("dvmh_region_register_array_C");
    Region *r = regionOf(curRegion, "dvmh_region_register_array");
    GB_CHECK(dvmDesc, "NULL header passed to dvmh_region_register_array");
    Obj *o = (Obj *)dvmDesc[0];
    if (isLive(o, K_TEMPLATE)) return;
    if (isLive(o, K_VAR)) {  // a scalar regular variable (its rank-0 header)
        regionAddVar(r, (Var *)o, (long)intent, varName);
        return;
    }
    Array *a = arrayOf(dvmDesc, "dvmh_region_register_array");
    if (varName && a->name.empty()) a->name = varName;
    if (a->regMark == r && a->regIdx < r->arrays.size() && r->arrays[a->regIdx].arr == a) {
        r->arrays[a->regIdx].intent |= (long)intent;
        return;
    }
    a->regMark = r;
    a->regIdx = r->arrays.size();
    r->arrays.push_back({a, (long)intent});
}

void dvmh_region_register_subarray_C(DvmType curRegion, DvmType intent, const DvmType dvmDesc[], const char varName[],
                                     DvmType rank, ...) {
    // one device copy per array: a sub-array registration maps the whole array
    Array *a = arrayOf(dvmDesc, "dvmh_region_register_subarray");
    GB_CHECK(rank == a->rank, "rank mismatch in dvmh_region_register_subarray");
    dvmh_region_register_array_C(curRegion, intent, dvmDesc, varName);
}

void dvmh_region_register_scalar_C(DvmType curRegion, DvmType intent, const void *addr, DvmType typeSize,
                                   const char varName[]) {
    GB_PROF("dvmh_region_register_scalar_C");
    Region *r = regionOf(curRegion, "dvmh_region_register_scalar");
    GB_CHECK(addr && typeSize > 0, "invalid scalar registration");
    regionAddVar(r, varGet(addr, (size_t)typeSize), (long)intent, varName);
}

void dvmh_region_execute_on_targets_C(DvmType curRegion, DvmType deviceTypes) {
    GB_PROF("dvmh_region_execute_on_targets_C");
    Region *r = regionOf(curRegion, "dvmh_region_execute_on_targets");
    GB_CHECK(deviceTypes & DEVICE_TYPE_CUDA,
             "region targets exclude CUDA: this runtime executes parallel loops on the GPU only");
    r->targets = (long)deviceTypes;
    for (auto &ra : r->arrays) {
        ensureDevBuffer(ra.arr);
        if (ra.intent & (INTENT_IN | INTENT_USE)) ensureDevActual(ra.arr);
    }
    for (auto &rv : r->vars) {
        ensureVarDev(rv.var);
        if ((rv.intent & (INTENT_IN | INTENT_USE)) && !rv.var->devActual) {
            varH2D(rv.var);
            rv.var->devActual = true;
        }
    }
    r->started = true;
}

void dvmh_region_end_C(DvmType curRegion) {
    GB_PROF("dvmh_region_end_C");
    Region *r = regionOf(curRegion, "dvmh_region_end");
    GB_CHECK(!st.curLoop, "region ends inside a parallel loop");
    // every queued loop that names a variable is launched by the region's end:
    // handler parameters may point at variables that live only as long as the
    // region; loops over arrays alone may stay queued (they forget the region)
    queueFlushVars();
    queueRegionEnded(r);
    for (auto &ra : r->arrays)
        if (ra.intent & INTENT_OUT) {
            ra.arr->devActual = true;
            ra.arr->hostActual = false;
        }
    for (auto &rv : r->vars)
        if ((rv.intent & INTENT_OUT) && rv.var->devActual) rv.var->hostActual = false;
    untrack(r);
    st.curRegion = nullptr;
    delete r;
    regularRegionEnd();
}

// ---------------------------------------------------------------- extension API

void dvmhgb_get_stats(dvmhgb_stats_t *out) {
    if (out) *out = stats;
}

void dvmhgb_reset_stats(void) { memset(&stats, 0, sizeof stats); }

void dvmhgb_hostprof_dump(void) {
    fprintf(stderr, "[dvmh_gb host profile] %-40s %10s %12s %10s\n", "entry point", "calls", "total ms", "us/call");
    for (int i = 0; i < profCount; i++)
        if (profTable[i].calls)
            fprintf(stderr, "[dvmh_gb host profile] %-40s %10ld %12.3f %10.3f\n", profTable[i].name, profTable[i].calls,
                    profTable[i].ns * 1e-6, profTable[i].ns * 1e-3 / profTable[i].calls);
}

void dvmhgb_hostprof_reset(void) {
    for (int i = 0; i < profCount; i++) profTable[i].calls = 0, profTable[i].ns = 0;
}

void dvmhgb_count_launches(long n) { stats.kernel_launches += n; }

void *dvmhgb_stream(void) { return (void *)gpu.stream; }

}  // extern "C"
