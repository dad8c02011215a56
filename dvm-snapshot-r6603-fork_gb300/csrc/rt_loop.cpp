// libdvmh_gb loop manager: parallel loops, the handler launcher, the
// in-handler query API, reductions, and batched execution (queue -> fused ->
// captured CUDA graph, cached by signature).
//
// Reference behaviour followed (rts/dvmh/...):
//   dvmh_loop_create_C        dvmh2.cpp:3143-3188; end index normalised to
//                             start + floor((end-start)/step)*step, empty when negative (loop.cpp:556-565)
//   dvmh_loop_map_C           dvmh2.cpp:3210-3303 (array axis -> loop axis correspondence)
//   dvmh_loop_reduction_C     dvmh2.cpp:3343-3362; initial value snapshot (loop.cpp:17-35)
//   dvmh_loop_across_C        dvmh2.cpp:3371-3396; dependency mask (DvmhLoop::renewDependencyMask,
//                             loop.cpp:1117-1150): bit (rank - loopAxis) per axis with a nonzero width
//   dvmh_loop_perform_C       dvmh2.cpp:3769-3969
//   handler launch            DvmhLoopHandler::exec, loop.cpp:442-454; executeFunction, util.cpp:677
//   in-handler queries        dvmh2.cpp:3977-4406
//   CUDA block choice         DvmhLoopCuda::pickBlock (loop.cpp:2134-2199): user block, tuner, the
//                             handler's default, then 256 / 32x8 / 32x4x2 by rank (loop.cpp:1464-1485)
//   change_filled_bounds(2)   dvmh2.cpp:4517-4583
#include <algorithm>
#include <cstring>
#include <list>
#include <unordered_map>
#include <unordered_set>

#include "rt.h"
#include "rt_call.inc"

namespace dvmhgb {

extern dvmhgb_stats_t stats;
bool isArrayDesc(const void *p);

// ---------------------------------------------------------------- rules

struct FusionRule {
    DvmHandlerFunc first, second, fused;
};
static std::vector<FusionRule> fusionRules;
static std::unordered_map<void *, DvmHandlerFunc> batchRules;

// ---------------------------------------------------------------- queue and graph cache

static std::vector<Loop *> queue;

// ---------------------------------------------------------------- handler timing
// With timing on, every handler execution is bracketed by CUDA events on the
// runtime stream (inside a captured graph they become event-record nodes and
// fire on every replay).  Elapsed times are collected at the next stream
// synchronisation and accumulated per handler: the runtime's timing database.
struct TimedExec {
    void *func;
    cudaEvent_t e0, e1;
    Loop *loopCopy;  // loop shape for the tuner (owned), may be null
    int block[3];
    int variant;
    int layout;    // the tuner's layout choice in this execution, -1 none
    bool inGraph;  // owned by a cached graph (reused on every replay)
    uint64_t tkey;   // the tuner's key when the handler chose a variant, else 0
    bool exploring;  // that variant had not been timed before
    float vf[TUNE_NF];
};
struct TimingTotal {
    double ms = 0;
    long count = 0;
};
static std::vector<TimedExec> pendingTimes;
static std::unordered_map<void *, TimingTotal> timingTotals;
static bool timingOn = false;

static cudaEvent_t newEvent() {
    cudaEvent_t e;
    GB_CUDA(cudaEventCreate(&e));
    return e;
}

void collectTimings() {  // called after a stream synchronisation
    for (auto &t : pendingTimes) {
        float ms = 0;
        if (cudaEventElapsedTime(&ms, t.e0, t.e1) == cudaSuccess) {
            TimingTotal &tt = timingTotals[t.func];
            tt.ms += ms;
            tt.count++;
            if (t.tkey) tunerRecord(t.tkey, t.variant, t.exploring, t.vf, ms * 1e-3);
            if (t.loopCopy && t.layout >= 0) tunerRecordLayout(t.loopCopy, t.layout, ms * 1e-3);
        }
        if (!t.inGraph) {
            cudaEventDestroy(t.e0);
            cudaEventDestroy(t.e1);
            delete t.loopCopy;
        }
    }
    pendingTimes.clear();
}

static char graphTimingKey;  // handler key for graphs that ran several handlers

// an array's device layout, as recorded for graph replays
struct LayoutState {
    int perm[MAXR] = {};
    int diag = 0;
    LayoutState() = default;
    explicit LayoutState(const Array *a) : diag(a->tdiag) {
        for (int k = 0; k < MAXR; k++) perm[k] = a->tperm[k];
    }
    void applyTo(Array *a) const {
        for (int k = 0; k < MAXR; k++) a->tperm[k] = perm[k];
        a->tdiag = diag;
    }
};

struct CachedGraph {
    uint64_t key;
    std::vector<uint64_t> sig;
    std::vector<TimedExec> times;  // handlers captured into the graph
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    cudaGraphExec_t exec = nullptr;
    std::vector<void *> scratch;
    std::vector<void *> hostScratch;
    std::vector<Array *> swaps;
    std::vector<std::pair<Array *, LayoutState>> layouts;  // layout changes, in order
    long launches = 0;
};
static std::list<CachedGraph> graphCache;  // most recently used first

bool queueBusy() { return !queue.empty(); }

static void deleteLoop(Loop *l) {
    untrackObj(l);
    delete l;
}

// ---------------------------------------------------------------- helpers

static long floorDiv(long a, long b) {
    long q = a / b, r = a % b;
    return (r != 0 && ((r < 0) != (b < 0))) ? q - 1 : q;
}

static Loop *loopOf(DvmType ref, const char *what) {
    Loop *l = (Loop *)ref;
    GB_CHECK(isLive(l, K_LOOP) && l == st.curLoop, "incorrect loop reference passed to %s", what);
    return l;
}

static SpecLoop *specOf(DvmType ref, const char *what) {
    SpecLoop *s = (SpecLoop *)ref;
    GB_CHECK(isLive(s, K_SPEC), "incorrect loop reference passed to %s (only valid inside a handler)", what);
    return s;
}

// the reference's default block for `rank` free block dimensions (loop.cpp:1464-1485)
static void defaultBlock(int rank, int b[3]) {
    b[0] = b[1] = b[2] = 1;
    if (rank >= 3) { b[0] = 32; b[1] = 4; b[2] = 2; }
    else if (rank == 2) { b[0] = 32; b[1] = 8; }
    else if (rank == 1) { b[0] = 256; }
}

// block dimensions a loop may use: one fewer with dependences (loop.h:257, loop.cpp:2136)
static int freeBlockDims(int loopRank, bool hasDeps) { return loopRank - (hasDeps ? 1 : 0); }

// arrays a loop's handler can touch: its array-descriptor parameters
static void loopArrays(const Loop *l, std::vector<const void *> &out) {
    for (int i = 0; i < l->cuda.nparams; i++)
        if (isArrayDesc(l->cuda.params[i])) out.push_back(l->cuda.params[i]);
}

// ---------------------------------------------------------------- execution of one loop's handler

struct ExecCtx {
    std::vector<TimedExec> *times = nullptr;  // capture: event pairs belong to the graph
    bool capturing = false;
    std::vector<void *> *keep = nullptr;      // scratch kept alive with a cached graph
    std::vector<void *> *keepHost = nullptr;  // pinned host scratch kept with it
    std::vector<Array *> *swaps = nullptr;    // swaps performed (recorded for replays)
    std::vector<std::pair<Array *, LayoutState>> *layouts = nullptr;  // layout changes, likewise
};
static ExecCtx ctx;

// the handler call in progress and the arrays it autotransformed
static int callDepth = 0;
static std::vector<const Array *> callTfm;
bool inHandlerCall() { return callDepth > 0; }
bool transformedInCall(const Array *a) {
    return callDepth > 0 && std::find(callTfm.begin(), callTfm.end(), a) != callTfm.end();
}
struct CallScope {
    CallScope() {
        if (callDepth++ == 0) callTfm.clear();
    }
    ~CallScope() {
        if (--callDepth == 0) callTfm.clear();
    }
};

void noteSwap(Array *a) {
    if (ctx.swaps) ctx.swaps->push_back(a);
}
void noteLayout(Array *a) {
    if (ctx.layouts) ctx.layouts->push_back({a, LayoutState(a)});
}
// reduction folds deferred while a batched handler runs: one launch for all
static bool deferFolds = false;
static std::vector<FoldJob> deferred;

static SpecLoop *newSpec(Loop *l) {
    SpecLoop *s = new SpecLoop();
    s->loop = l;
    s->device = 1;
    s->stream = gpu.stream;
    trackObj(s);
    return s;
}

static void finishSpec(SpecLoop *s) {
    Loop *l = s->loop;
    for (size_t i = 0; i < l->reds.size(); i++) {
        bool done = false;
        for (auto &cr : s->reds)
            if (cr.index == (int)i + 1 && cr.finished) done = true;
        GB_CHECK(done, "CUDA handler of loop at %s:%ld did not finish reduction #%zu (dvmh_loop_cuda_red_finish_C)",
                 l->file.c_str(), l->line, i + 1);
    }
    for (Array *a : s->swaps) {
        std::swap(a->dev, a->devAlt);
        if (ctx.swaps) ctx.swaps->push_back(a);
    }
    for (void *p : s->scratch) {
        if (ctx.keep) ctx.keep->push_back(p);
        else devFree(p);  // one stream: later work is ordered after this loop's kernels
    }
    for (void *p : s->hostScratch) {
        if (ctx.keepHost) ctx.keepHost->push_back(p);
        else {
            streamSync();  // a pending copy may still read it
            hostFree(p);
        }
    }
    untrackObj(s);
    delete s;
}

// Inside a capture no event is recorded (a timing event cannot be captured):
// the handler is noted and the graph launch as a whole is timed instead.
static void timeBegin(TimedExec &t, void *func) {
    t.func = func;
    t.e0 = t.e1 = nullptr;
    t.loopCopy = nullptr;
    t.block[0] = t.block[1] = t.block[2] = 0;
    t.variant = -1;
    t.layout = -1;
    t.inGraph = ctx.capturing;
    t.tkey = 0;
    t.exploring = false;
    if (ctx.capturing) return;
    t.e0 = newEvent();
    t.e1 = newEvent();
    GB_CUDA(cudaEventRecord(t.e0, gpu.stream));
}
// the tuner's choice made in this execution (graph replays are not recorded)
static void timeTuned(TimedExec &t, const SpecLoop *s) {
    if (!s->tkey || ctx.capturing) return;
    t.tkey = s->tkey;
    t.variant = s->variant;
    t.exploring = s->exploring;
    memcpy(t.vf, s->vf, sizeof t.vf);
}

static void timeEnd(TimedExec &t) {
    if (ctx.capturing) {
        if (ctx.times) ctx.times->push_back(t);
        return;
    }
    GB_CUDA(cudaEventRecord(t.e1, gpu.stream));
    pendingTimes.push_back(t);
}

// a launch of a cached graph, timed as a whole when timing is on; the time
// goes to its handler when it ran exactly one
static void launchGraph(CachedGraph &g) {
    GB_PROF("launchGraph");
    bool timed = timingOn && !g.times.empty();
    if (timed) {
        if (!g.e0) {
            g.e0 = newEvent();
            g.e1 = newEvent();
        }
        GB_CUDA(cudaEventRecord(g.e0, gpu.stream));
    }
    GB_CUDA(cudaGraphLaunch(g.exec, gpu.stream));
    if (timed) {
        GB_CUDA(cudaEventRecord(g.e1, gpu.stream));
        TimedExec t = g.times[0];
        if (g.times.size() > 1) t.func = (void *)&graphTimingKey;
        t.e0 = g.e0;
        t.e1 = g.e1;
        t.loopCopy = nullptr;
        t.inGraph = true;
        pendingTimes.push_back(t);
    }
}

static void runSingle(Loop *l) {
    SpecLoop *s = newSpec(l);
    s->handler = (void *)l->cuda.func;
    DvmType ref = (DvmType)s;
    stats.handler_calls++;
    TimedExec t;
    if (timingOn) timeBegin(t, (void *)l->cuda.func);
    {
        CallScope call;
        callWithParams(l->cuda.func, &ref, l->cuda.nparams, l->cuda.params);
    }
    if (timingOn) {
        memcpy(t.block, s->block, sizeof t.block);
        t.variant = s->variant;
        t.layout = s->layout;
        t.loopCopy = (tunerWants(l) && s->layout >= 0) ? new Loop(*l) : nullptr;
        timeTuned(t, s);
        timeEnd(t);
    }
    finishSpec(s);
}

static void runFused(DvmHandlerFunc fused, Loop *a, Loop *b) {
    SpecLoop *sa = newSpec(a), *sb = newSpec(b);
    sa->handler = sb->handler = (void *)fused;
    DvmType refs[2] = {(DvmType)sa, (DvmType)sb};
    void *params[80];
    int n = 0;
    for (int i = 0; i < a->cuda.nparams; i++) params[n++] = a->cuda.params[i];
    for (int i = 0; i < b->cuda.nparams; i++) params[n++] = b->cuda.params[i];
    stats.handler_calls++;
    stats.fused_pairs++;
    TimedExec t;
    if (timingOn) timeBegin(t, (void *)fused);
    {
        CallScope call;
        callWithParams(fused, refs, n, params);
    }
    if (timingOn) {
        timeTuned(t, sa->tkey ? sa : sb);
        timeEnd(t);
    }
    finishSpec(sa);
    finishSpec(sb);
}

static void runBatch(DvmHandlerFunc batched, const std::vector<Loop *> &group) {
    std::vector<DvmType> refs;
    std::vector<SpecLoop *> specs;
    for (Loop *l : group) {
        specs.push_back(newSpec(l));
        specs.back()->handler = (void *)batched;
        refs.push_back((DvmType)specs.back());
    }
    stats.handler_calls++;
    stats.batched_groups++;
    deferFolds = true;
    deferred.clear();
    TimedExec t;
    if (timingOn) timeBegin(t, (void *)batched);
    {
        CallScope call;
        ((void (*)(DvmType *, DvmType))batched)(refs.data(), (DvmType)refs.size());
    }
    deferFolds = false;
    if (!deferred.empty()) launchRedFoldBatch(deferred, gpu.stream, specs[0]->scratch, specs[0]->hostScratch);
    deferred.clear();
    if (timingOn) {
        timeTuned(t, specs[0]);
        timeEnd(t);
    }
    for (SpecLoop *s : specs) finishSpec(s);
}

// Apply fusion and batch rules to the queued loops and run them.
static void runQueued(const std::vector<Loop *> &q) {
    size_t i = 0, n = q.size();
    while (i < n) {
        Loop *l = q[i];
        if (settings.fuse && i + 1 < n) {
            DvmHandlerFunc fused = nullptr;
            for (auto &r : fusionRules)
                if (r.first == l->cuda.func && r.second == q[i + 1]->cuda.func) fused = r.fused;
            // the same region, or a first loop left queued past its region's end (it names arrays only)
            const bool regionsOk = l->region == q[i + 1]->region || l->region == nullptr;
            if (fused && regionsOk && l->cuda.nparams + q[i + 1]->cuda.nparams <= 40) {
                runFused(fused, l, q[i + 1]);
                i += 2;
                continue;
            }
        }
        auto br = batchRules.find((void *)l->cuda.func);
        if (br != batchRules.end()) {
            std::vector<Loop *> group;
            std::unordered_set<const void *> used;
            std::unordered_set<const void *> redAddrs;
            size_t j = i;
            while (j < n && q[j]->cuda.func == l->cuda.func) {
                std::vector<const void *> arrs;
                loopArrays(q[j], arrs);
                bool clash = false;
                for (auto *a : arrs) clash = clash || used.count(a);
                for (auto &r : q[j]->reds) clash = clash || redAddrs.count(r.addr) || (r.locAddr && redAddrs.count(r.locAddr));
                if (clash) break;
                for (auto *a : arrs) used.insert(a);
                for (auto &r : q[j]->reds) {
                    redAddrs.insert(r.addr);
                    if (r.locAddr) redAddrs.insert(r.locAddr);
                }
                group.push_back(q[j]);
                j++;
            }
            if (group.size() > 1) {
                runBatch(br->second, group);
                i = j;
                continue;
            }
        }
        runSingle(l);
        i++;
    }
}

// ---------------------------------------------------------------- batched mode: flush

// DVMH_GB_VARIANT / dvmhgb_force_variant: the value every variant query returns (-1: none)
static int forcedVariant = getenv("DVMH_GB_VARIANT") ? atoi(getenv("DVMH_GB_VARIANT")) : -1;

static void sigAdd(std::vector<uint64_t> &s, uint64_t v) { s.push_back(v); }

static std::vector<uint64_t> signature(const std::vector<Loop *> &q) {
    std::vector<uint64_t> s;
    for (Loop *l : q) {
        sigAdd(s, (uint64_t)l->cuda.func);
        sigAdd(s, (uint64_t)l->cuda.nparams);
        for (int i = 0; i < l->cuda.nparams; i++) {
            sigAdd(s, (uint64_t)l->cuda.params[i]);
            if (isArrayDesc(l->cuda.params[i])) {
                Array *a = (Array *)((const DvmType *)l->cuda.params[i])[0];
                sigAdd(s, (uint64_t)a);  // the object the graph's swap and layout records name
                sigAdd(s, (uint64_t)a->dev);
                sigAdd(s, (uint64_t)a->devAlt);
                uint64_t lay = (uint64_t)a->tdiag;
                for (int k = 0; k < MAXR; k++) lay = lay * 8 + (uint64_t)a->tperm[k];
                sigAdd(s, lay);
            } else {
                size_t off = 0;
                Var *v = varAt(l->cuda.params[i], &off);
                sigAdd(s, (uint64_t)v);
                sigAdd(s, v ? (uint64_t)(v->dev + off) : 0);
            }
        }
        sigAdd(s, (uint64_t)l->rank);
        for (int i = 0; i < l->rank; i++) {
            sigAdd(s, (uint64_t)l->lo[i]);
            sigAdd(s, (uint64_t)l->hi[i]);
            sigAdd(s, (uint64_t)l->step[i]);
        }
        sigAdd(s, (uint64_t)l->depMask);
        for (int i = 0; i < 3; i++) sigAdd(s, (uint64_t)l->cudaBlock[i]);
        for (auto &r : l->reds) {
            sigAdd(s, (uint64_t)r.op);
            sigAdd(s, (uint64_t)r.vtype);
            sigAdd(s, (uint64_t)r.addr);
            sigAdd(s, (uint64_t)r.locAddr);
            sigAdd(s, (uint64_t)r.var);
            sigAdd(s, (uint64_t)r.locVar);
            sigAdd(s, (uint64_t)(r.var ? r.var->dev : nullptr));
            sigAdd(s, (uint64_t)(r.locVar ? r.locVar->dev : nullptr));
        }
    }
    sigAdd(s, (uint64_t)settings.fuse);
    sigAdd(s, (uint64_t)(int64_t)forcedVariant);  // a forced variant is captured anew
    sigAdd(s, (uint64_t)settings.autoTfm);
    return s;
}

static uint64_t hashSig(const std::vector<uint64_t> &s) {
    uint64_t h = 1469598103934665603ull;
    for (uint64_t v : s) {
        h ^= v + 0x9E3779B97F4A7C15ull + (h << 6) + (h >> 2);
        h *= 1099511628211ull;
    }
    return h;
}

static void dropGraph(CachedGraph &g) {
    streamSync();
    if (g.e0) {
        cudaEventDestroy(g.e0);
        cudaEventDestroy(g.e1);
    }
    if (g.exec) cudaGraphExecDestroy(g.exec);
    for (void *p : g.scratch) devFree(p);
    for (void *p : g.hostScratch) hostFree(p);
}

// the variable a queued loop's parameter names -- its address, or the header
// of a rank-0 regular variable -- or null (an array descriptor, no variable)
static const Var *paramVar(const void *p) {
    if (isArrayDesc(p)) return nullptr;
    size_t off = 0;
    if (const Var *v = varAt(p, &off)) return v;
    return regularVarOfHeader(p);
}

// v == nullptr: any parameter that is not an array descriptor counts -- a
// registered variable or not (an unregistered address could die with its
// region just the same)
static bool loopNamesVar(const Loop *l, const Var *v) {
    for (int i = 0; i < l->cuda.nparams; i++) {
        if (v == nullptr) {
            if (!isArrayDesc(l->cuda.params[i])) return true;
            continue;
        }
        if (paramVar(l->cuda.params[i]) == v) return true;
    }
    for (auto &r : l->reds)
        if ((r.var && (v == nullptr || r.var == v)) || (r.locVar && (v == nullptr || r.locVar == v))) return true;
    return false;
}

static void queueFlushPrefix(size_t count);

// A queued loop may wait for a later one only when that can pay: it names no
// variable, and a fusion rule starts with its handler (the next loop may be
// the rule's second).  Every other loop runs at the first flush that reaches it.
static bool deferrable(const Loop *l) {
    if (!settings.defer || !settings.fuse || loopNamesVar(l, nullptr)) return false;
    for (auto &r : fusionRules)
        if (r.first == l->cuda.func) return true;
    return false;
}

void queueFlushVar(const Var *v) {
    size_t last = 0;
    for (size_t i = 0; i < queue.size(); i++)
        if (loopNamesVar(queue[i], v) || !deferrable(queue[i])) last = i + 1;
    if (last) queueFlushPrefix(last);
}

void queueFlushVars() { queueFlushVar(nullptr); }

void queueRegionEnded(const Region *r) {
    for (Loop *l : queue)
        if (l->region == r) l->region = nullptr;
}

void queueFlush() { queueFlushPrefix(queue.size()); }

// Run (or replay) the first `count` queued loops as one group; the rest stay
// queued, in order.  A loop stays queued past a variable's host access or its
// region's end only if it is deferrable (above) and does not name that
// variable (handler parameters may point at variables that live only as long
// as the region; arrays live until they are freed, which flushes everything).
// So a time step's last loop over arrays alone can meet the next step's first
// loop in one group, where a fusion rule joins them.
static void queueFlushPrefix(size_t count) {
    GB_PROF("queueFlush");
    if (queue.empty() || ctx.capturing || count == 0) return;
    if (count > queue.size()) count = queue.size();
    std::vector<Loop *> q(queue.begin(), queue.begin() + (long)count);
    queue.erase(queue.begin(), queue.begin() + (long)count);
    stats.flushes++;
    if (settings.tuneMode && tunerExploring()) {
        // variants are still being tried: run the queue as it is, each handler timed on its own
        runQueued(q);
        tunerFlushed();
        for (Loop *l : q) deleteLoop(l);
        if (settings.syncEachLoop) streamSync();
        return;
    }
    std::vector<uint64_t> sig = signature(q);
    uint64_t key = hashSig(sig);
    for (auto it = graphCache.begin(); it != graphCache.end(); ++it) {
        if (it->key == key && it->sig == sig) {
            launchGraph(*it);
            for (Array *a : it->swaps) std::swap(a->dev, a->devAlt);
            for (auto &pl : it->layouts) pl.second.applyTo(pl.first);
            stats.graph_replays++;
            stats.kernel_launches += it->launches;
            graphCache.splice(graphCache.begin(), graphCache, it);
            for (Loop *l : q) deleteLoop(l);
            if (settings.syncEachLoop) streamSync();
            return;
        }
    }
    CachedGraph g;
    g.key = key;
    g.sig = sig;
    long launchesBefore = stats.kernel_launches;
    ctx.capturing = true;
    ctx.times = &g.times;
    ctx.keep = &g.scratch;
    ctx.keepHost = &g.hostScratch;
    ctx.swaps = &g.swaps;
    ctx.layouts = &g.layouts;
    GB_CUDA(cudaStreamBeginCapture(gpu.stream, cudaStreamCaptureModeRelaxed));
    runQueued(q);
    cudaGraph_t graph = nullptr;
    GB_CUDA(cudaStreamEndCapture(gpu.stream, &graph));
    ctx = ExecCtx();
    GB_CUDA(cudaGraphInstantiate(&g.exec, graph, 0));
    cudaGraphDestroy(graph);
    g.launches = stats.kernel_launches - launchesBefore;
    launchGraph(g);
    stats.graphs_captured++;
    graphCache.push_front(std::move(g));
    while ((int)graphCache.size() > settings.graphCacheMax) {
        dropGraph(graphCache.back());
        graphCache.pop_back();
    }
    for (Loop *l : q) deleteLoop(l);
    if (settings.syncEachLoop) streamSync();
}

// An array or a variable is dropped: no cached graph may name it any more (a
// later object could reuse its descriptor and buffers, and the graph's records
// would then name a dead object).
void graphsForget(const Obj *a) {
    for (auto it = graphCache.begin(); it != graphCache.end();) {
        bool names = std::find(it->sig.begin(), it->sig.end(), (uint64_t)a) != it->sig.end();
        for (const Array *x : it->swaps) names = names || x == a;
        for (auto &pl : it->layouts) names = names || pl.first == a;
        if (names) {
            dropGraph(*it);
            it = graphCache.erase(it);
        } else {
            ++it;
        }
    }
}

void loopsAtExit() {
    for (auto &g : graphCache) dropGraph(g);
    graphCache.clear();
}

// ---------------------------------------------------------------- reduction results after a loop

static void afterReductions(Loop *l, bool toHost) {
    for (auto &r : l->reds) {
        Var *vs[2] = {r.var, r.locVar};
        for (Var *v : vs) {
            if (!v) continue;
            v->devActual = true;
            v->hostActual = false;
            if (toHost) {
                varD2H(v);
                v->hostActual = true;
            }
        }
    }
}

}  // namespace dvmhgb

using namespace dvmhgb;

namespace dvmhgb {
}  // namespace dvmhgb

extern "C" {

// ---------------------------------------------------------------- loop construction

DvmType dvmh_loop_create_C(DvmType curRegion, DvmType rank, ...) {
    GB_PROF("dvmh_loop_create_C");
    GB_CHECK(st.inited, "LibDVMH is not initialized");
    GB_CHECK(!st.curLoop, "nested parallel loops are not allowed");
    GB_CHECK(rank >= 0 && rank <= MAXR, "loop rank must be in 0..%d", MAXR);
    Region *r = (Region *)curRegion;
    GB_CHECK(r == nullptr || (isLive(r, K_REGION) && r == st.curRegion), "incorrect region reference in dvmh_loop_create");
    Loop *l = new Loop();
    l->region = r;
    l->rank = (int)rank;
    l->file = st.file;
    l->line = st.line;
    va_list ap;
    va_start(ap, rank);
    for (int i = 0; i < l->rank; i++) {
        l->lo[i] = (long)va_arg(ap, DvmType);
        l->hi[i] = (long)va_arg(ap, DvmType);
        l->step[i] = (long)va_arg(ap, DvmType);
        GB_CHECK(l->step[i] != 0, "zero loop step on axis %d", i + 1);
        long dist = floorDiv(l->hi[i] - l->lo[i], l->step[i]);
        l->hi[i] = l->lo[i] + dist * l->step[i];
        if (dist < 0) l->empty = true;
        l->arrAxisToLoop[i] = i + 1;
    }
    va_end(ap);
    trackObj(l);
    st.curLoop = l;
    return (DvmType)l;
}

void dvmh_loop_map_C(DvmType curLoop, const DvmType templDesc[], DvmType templRank, ...) {
    GB_PROF("dvmh_loop_map_C");
    Loop *l = loopOf(curLoop, "dvmh_loop_map");
    Obj *o = (Obj *)templDesc[0];
    if (isLive(o, K_ARRAY)) l->mapArr = (Array *)o;
    GB_CHECK(templRank >= 0 && templRank <= MAXR, "mapping target rank %ld out of range", (long)templRank);
    int axis[MAXR] = {}, sign[MAXR] = {};
    va_list ap;
    va_start(ap, templRank);
    for (long i = 0; i < templRank; i++) {
        DvmType hv = va_arg(ap, DvmType);
        struct H { uint32_t magic; long axis, mult, summand; } *h = (H *)hv;
        GB_CHECK(h && h->magic == 0x414c4e31u, "invalid alignment helper in dvmh_loop_map");
        GB_CHECK(h->axis == -1 || (h->axis >= 0 && h->axis <= l->rank), "loop axis %ld out of range", h->axis);
        l->arrAxisToLoop[i] = h->axis > 0 ? (int)h->axis : 0;
        axis[i] = l->arrAxisToLoop[i];
        sign[i] = h->mult > 0 ? 1 : (h->mult < 0 ? -1 : 0);
        h->magic = 0;
        delete h;
    }
    va_end(ap);
    if (const AlignMap *t = alignOf(templDesc)) alignCompose(l->map, *t, axis, sign, (int)templRank);
}

void dvmh_loop_set_cuda_block_C(DvmType curLoop, DvmType xSize, DvmType ySize, DvmType zSize) {
    GB_PROF("dvmh_loop_set_cuda_block_C");
    Loop *l = loopOf(curLoop, "dvmh_loop_set_cuda_block");
    GB_CHECK(xSize >= 1 && ySize >= 1 && zSize >= 1 && xSize * ySize * zSize <= 1024, "invalid CUDA block");
    l->cudaBlock[0] = (int)xSize;
    l->cudaBlock[1] = (int)ySize;
    l->cudaBlock[2] = (int)zSize;
    l->userBlock = true;
}

void dvmh_loop_set_stage_C(DvmType curLoop, DvmType stage) { loopOf(curLoop, "dvmh_loop_set_stage")->stage = stage; }

void dvmh_loop_reduction_C(DvmType curLoop, DvmType redType, void *arrayAddr, DvmType varType, DvmType arrayLength,
                           void *locAddr, DvmType locSize) {
    GB_PROF("dvmh_loop_reduction_C");
    Loop *l = loopOf(curLoop, "dvmh_loop_reduction");
    GB_CHECK(arrayAddr, "NULL reduction variable");
    GB_CHECK(redType >= rf_SUM && redType <= rf_MINLOC, "unknown reduction function %ld", (long)redType);
    GB_CHECK(arrayLength >= 1, "reduction length must be positive");
    bool loc = redType == rf_MINLOC || redType == rf_MAXLOC;
    GB_CHECK(!loc || (locAddr && locSize > 0), "MINLOC/MAXLOC reduction without a location variable");
    Reduction r;
    r.op = (int)redType;
    r.vtype = (int)varType;
    r.esize = typeSize(r.vtype);
    GB_CHECK(r.esize > 0, "unknown reduction variable type %ld", (long)varType);
    r.count = (long)arrayLength;
    r.addr = (char *)arrayAddr;
    r.locAddr = loc ? (char *)locAddr : nullptr;
    r.locSize = loc ? (long)locSize : 0;
    // the reference snapshots the initial value here (loop.cpp:23-29)
    r.init.assign(r.addr, r.addr + r.esize * r.count);
    if (loc) r.initLoc.assign(r.locAddr, r.locAddr + r.locSize * r.count);
    // the result lives in the variable's device copy; a variable the region did
    // not register becomes known here and is written back at loop end.  Such a
    // variable is the program's host memory to the reference, which reads the
    // initial value from it here: while its host copy is current the program
    // may have written it since, so the device copy is refreshed from it; after
    // a loop left a newer result on the device (async and batched modes, no
    // get_actual since), that result is the initial value.  A variable the
    // region registered follows the region's actuality.
    size_t off = 0;
    Var *v = varAt(r.addr, &off);
    if (!v) {
        v = varGet(r.addr, r.esize * r.count);
        off = 0;
    }
    GB_CHECK(off + r.esize * r.count <= v->size, "reduction variable crosses the end of '%s'", v->name.c_str());
    r.var = v;
    r.varOff = off;
    ensureVarDev(v);
    if (!v->devActual || (v->hostActual && !varInRegion(v))) {
        varH2D(v);
        v->devActual = true;
    }
    if (loc) {
        size_t loff = 0;
        Var *lv = varAt(r.locAddr, &loff);
        if (!lv) {
            lv = varGet(r.locAddr, (size_t)(r.locSize * r.count));
            loff = 0;
        }
        r.locVar = lv;
        r.locVarOff = loff;
        ensureVarDev(lv);
        if (!lv->devActual || (lv->hostActual && !varInRegion(lv))) {
            varH2D(lv);
            lv->devActual = true;
        }
    }
    l->reds.push_back(std::move(r));
}

void dvmh_loop_across_C(DvmType curLoop, DvmType isOut, const DvmType dvmDesc[], DvmType rank, ...) {
    GB_PROF("dvmh_loop_across_C");
    Loop *l = loopOf(curLoop, "dvmh_loop_across");
    Array *a = arrayOf(dvmDesc, "dvmh_loop_across");
    GB_CHECK(rank == a->rank, "rank in across directive must be the rank of the array");
    Across ac;
    ac.arr = a;
    ac.isOut = isOut != 0;
    va_list ap;
    va_start(ap, rank);
    for (int i = 0; i < a->rank; i++) {
        ac.lo[i] = (long)va_arg(ap, DvmType);
        ac.hi[i] = (long)va_arg(ap, DvmType);
        GB_CHECK(ac.lo[i] >= 0 && ac.hi[i] >= 0, "negative across width");
    }
    va_end(ap);
    l->across.push_back(ac);
}

void dvmh_loop_shadow_compute_C(DvmType curLoop, const DvmType templDesc[], DvmType specifiedRank, ...) {
    // one device copy: shadow elements computed by the loop are ordinary elements
    (void)loopOf(curLoop, "dvmh_loop_shadow_compute");
    (void)templDesc;
    (void)specifiedRank;
}

DvmType dvmh_handler_func_C(DvmHandlerFunc handlerFunc, DvmType customParamCount, ...) {
    GB_PROF("dvmh_handler_func_C");
    GB_CHECK(handlerFunc, "NULL handler function");
    GB_CHECK(customParamCount >= 0 && customParamCount <= 40, "handler with %ld parameters (at most 40)",
             (long)customParamCount);
    HandlerRef *h = new HandlerRef();
    h->func = handlerFunc;
    h->nparams = (int)customParamCount;
    va_list ap;
    va_start(ap, customParamCount);
    for (int i = 0; i < h->nparams; i++) h->params[i] = va_arg(ap, void *);
    va_end(ap);
    return (DvmType)h;
}

void dvmh_loop_register_handler_C(DvmType curLoop, DvmType deviceType, DvmType handlerType, DvmType handlerHelper) {
    GB_PROF("dvmh_loop_register_handler_C");
    (void)handlerType;
    Loop *l = loopOf(curLoop, "dvmh_loop_register_handler");
    HandlerRef *h = (HandlerRef *)handlerHelper;
    GB_CHECK(h && h->func, "invalid handler helper");
    if (deviceType == DEVICE_TYPE_CUDA) {
        l->cuda = *h;
        l->hasCuda = true;
    } else if (deviceType == DEVICE_TYPE_HOST) {
        l->host = *h;  // kept for completeness; host handlers are not executed by this runtime
        l->hasHost = true;
    } else {
        GB_CHECK(false, "unknown device type %ld", (long)deviceType);
    }
    delete h;
}

void dvmh_loop_perform_C(DvmType curLoop) {
    GB_PROF("dvmh_loop_perform_C");
    Loop *l = loopOf(curLoop, "dvmh_loop_perform");
    if (settings.tuneMode) timingOn = true;  // the tuner learns from recorded timings
    stats.loops_performed++;
    st.curLoop = nullptr;
    GB_CHECK(l->region && l->region->started,
             "parallel loop outside a region: this runtime executes parallel loops on the GPU only, inside regions");
    GB_CHECK(l->hasCuda, "loop at %s:%ld has no CUDA handler: this runtime executes parallel loops on the GPU only",
             l->file.c_str(), l->line);
    // dependency mask from ACROSS widths (loop.cpp:1117-1150): the loop axis each
    // dependent array axis follows; an axis with one iteration keeps its
    // dependence unless DVMH_REDUCE_DEPS asks to drop it, as in the reference
    int firstDep = -1;
    for (auto &ac : l->across)
        for (int j = 0; j < ac.arr->rank; j++)
            if (ac.lo[j] > 0 || ac.hi[j] > 0) {
                int la = loopAxisOf(l, ac.arr, j);
                GB_CHECK(la > 0, "ACROSS array %s has a dependence on axis %d that is not tied to the loop",
                         ac.arr->name.c_str(), j + 1);
                if (firstDep == -1 || la < firstDep) firstDep = la;
                if (!settings.reduceDeps || (!l->empty && l->lo[la - 1] != l->hi[la - 1]))
                    l->depMask |= 1L << (l->rank - la);
            }
    if (firstDep > 0 && l->depMask == 0) l->depMask |= 1L << (l->rank - firstDep);
    if (l->empty) {
        // no iterations: every reduction variable keeps its initial value
        deleteLoop(l);
        return;
    }
    if (settings.mode == MODE_BATCHED) {
        for (auto &ra : l->region->arrays) l->regionElems = std::max(l->regionElems, ra.arr->delems);
        afterReductions(l, false);
        queue.push_back(l);
        return;
    }
    queueFlush();
    runSingle(l);
    afterReductions(l, settings.mode == MODE_PLAIN);
    if (settings.mode == MODE_PLAIN || settings.syncEachLoop) streamSync();
    deleteLoop(l);
}

// ---------------------------------------------------------------- in-handler queries

DvmType dvmh_loop_get_device_num_C(DvmType curLoop) { return specOf(curLoop, "dvmh_loop_get_device_num")->device; }

DvmType dvmh_loop_get_dependency_mask_C(DvmType curLoop) {
    return specOf(curLoop, "dvmh_loop_get_dependency_mask")->loop->depMask;
}

// The handler asks for the layout the reference would choose for this loop
// (rts/dvmh/dvmh2.cpp:4011-4026): the array may stay transformed for the
// rest of this handler call; the header it fills next describes the layout.
DvmType dvmh_loop_autotransform_C(DvmType curLoop, DvmType dvmDesc[]) {
    SpecLoop *s = specOf(curLoop, "dvmh_loop_autotransform");
    Array *a = arrayOf(dvmDesc, "dvmh_loop_autotransform");
    ensureDevBuffer(a);
    if (settings.tuneMode && settings.autoTfm) {
        // the tuner may keep this loop's arrays natural (explores only outside captures)
        if (s->layout < 0) s->layout = tunerLayout(s->loop, !ctx.capturing);
        if (s->layout == 0) {
            makeNatural(a);
            return 0;
        }
    }
    int state = autotransform(s->loop, a);
    if (state != 0) callTfm.push_back(a);
    return state;
}

void dvmh_loop_fill_bounds_C(DvmType curLoop, DvmType boundsLow[], DvmType boundsHigh[], DvmType loopSteps[]) {
    Loop *l = specOf(curLoop, "dvmh_loop_fill_bounds")->loop;
    for (int i = 0; i < l->rank; i++) {
        if (boundsLow) boundsLow[i] = l->lo[i];
        if (boundsHigh) boundsHigh[i] = l->hi[i];
        if (loopSteps) loopSteps[i] = l->step[i];
    }
}

DvmType dvmh_loop_get_slot_count_C(DvmType curLoop) {
    (void)specOf(curLoop, "dvmh_loop_get_slot_count");
    return 1;
}

void dvmh_loop_fill_local_part_C(DvmType curLoop, const DvmType dvmDesc[], DvmType part[]) {
    (void)specOf(curLoop, "dvmh_loop_fill_local_part");
    Array *a = arrayOf(dvmDesc, "dvmh_loop_fill_local_part");
    GB_CHECK(part, "NULL part in dvmh_loop_fill_local_part");
    for (int i = 0; i < a->rank; i++) {  // one process: the whole index space
        part[2 * i] = 0;
        part[2 * i + 1] = a->ext[i] - 1;
    }
}

DvmType dvmh_loop_guess_index_type_C(DvmType curLoop) {
    Loop *l = specOf(curLoop, "dvmh_loop_guess_index_type")->loop;
    // int when every element of the arrays the loop can reach is addressable
    // with int: the region's arrays, or (a loop outside regions) every array
    // with a device copy (dvmh2.cpp:4110-4137)
    size_t maxElems = 0;
    if (l->region)
        for (auto &ra : l->region->arrays) maxElems = std::max(maxElems, ra.arr->delems);
    else
        maxElems = l->regionElems ? l->regionElems : maxDeviceElems();  // queued past the region's end, or outside
    return maxElems < (size_t)2147483647 ? rt_INT : rt_LLONG;
}

static const char *const pickBlockErrors[] = {
    "",
    "Setting CUDA block with more dimensions than the parallel loop has (minus 1 in case of dependency) is prohibited",
    "Block size on an axis is bigger than the device can handle",
    "Block size is bigger than the device can handle",
    "Shared memory amount is insufficient for the CUDA block",
    "Register count is insufficient for the CUDA block",
};

void dvmh_loop_cuda_get_config_C(DvmType curLoop, DvmType sharedPerThread, DvmType regsPerThread, void *inOutThreads,
                                 void *outStream, DvmType *outSharedPerBlock) {
    SpecLoop *s = specOf(curLoop, "dvmh_loop_cuda_get_config");
    Loop *l = s->loop;
    dim3 *t = (dim3 *)inOutThreads;
    int b[3] = {0, 0, 0};
    if (t && t->x >= 1 && t->y >= 1 && t->z >= 1) {  // the handler's own default
        b[0] = (int)t->x;
        b[1] = (int)t->y;
        b[2] = (int)t->z;
    }
    if (l->userBlock) memcpy(b, l->cudaBlock, sizeof b);
    if (!l->userBlock && settings.tuneMode) {
        if (b[0] < 1) defaultBlock(std::min(3, freeBlockDims(l->rank, l->depMask != 0)), b);
        tunerPick(l, b, &s->variant);
    }
    if (sharedPerThread < 0) sharedPerThread = 0;
    dvmhgb_cuda_limits_t lim;
    for (int i = 0; i < 3; i++) lim.maxBlockSize[i] = gpu.prop.maxThreadsDim[i];
    lim.maxThreadsPerBlock = gpu.prop.maxThreadsPerBlock;
    lim.sharedPerBlock = (long)gpu.prop.sharedMemPerBlock;
    lim.regsPerBlock = (long)gpu.prop.regsPerBlock;
    lim.warpSize = gpu.prop.warpSize;
    lim.maxRegsPerThread = 255;
    const int err = dvmhgb_pick_block(l->rank, l->depMask != 0, l->userBlock, b, (long)sharedPerThread,
                                      (long)regsPerThread, &lim);
    GB_CHECK(err == 0, "%s: block (%d, %d, %d), %ld bytes of shared memory and %ld registers per thread",
             pickBlockErrors[err], b[0], b[1], b[2], (long)sharedPerThread, (long)regsPerThread);
    memcpy(s->block, b, sizeof b);
    if (t) {
        t->x = (unsigned)b[0];
        t->y = (unsigned)b[1];
        t->z = (unsigned)b[2];
    }
    if (outStream) *(cudaStream_t *)outStream = s->stream;
    if (outSharedPerBlock) *outSharedPerBlock = (DvmType)b[0] * b[1] * b[2] * sharedPerThread;
}

int dvmhgb_pick_block(int loopRank, int hasDeps, int userBlock, int block[3], long sharedPerThread,
                      long regsPerThread, const dvmhgb_cuda_limits_t *lim) {
    GB_CHECK(block && lim, "NULL argument to dvmhgb_pick_block");
    const int maxBlockRank = freeBlockDims(loopRank, hasDeps != 0);
    if (!(block[0] >= 1 && block[1] >= 1 && block[2] >= 1)) defaultBlock(std::min(3, maxBlockRank), block);
    int blockRank = 3;
    while (blockRank > 0 && block[blockRank - 1] == 1) blockRank--;
    if (blockRank > maxBlockRank) return 1;
    for (int i = 0; i < 3; i++)
        if (block[i] > lim->maxBlockSize[i]) return 2;
    if ((long)block[0] * block[1] * block[2] > lim->maxThreadsPerBlock) return 3;
    // a block that needs more per-block resources than a block can have: one
    // dimension of at most 256 threads, a multiple of the warp size
    auto shrink = [&](long have, long perThread) {
        long n = std::min(256L, have / perThread);
        n = n / lim->warpSize * lim->warpSize;
        block[0] = maxBlockRank >= 1 ? (int)std::max(1L, n) : 1;
        block[1] = block[2] = 1;
    };
    if (sharedPerThread < 0) sharedPerThread = 0;
    if (sharedPerThread > 0 && (long)block[0] * block[1] * block[2] * sharedPerThread > lim->sharedPerBlock) {
        if (userBlock) return 4;
        shrink(lim->sharedPerBlock, sharedPerThread);
    }
    if (regsPerThread <= 0) regsPerThread = lim->maxRegsPerThread;
    if ((long)block[0] * block[1] * block[2] * regsPerThread > lim->regsPerBlock) {
        if (userBlock) return 5;
        shrink(lim->regsPerBlock, regsPerThread);
    }
    return 0;
}

// ---------------------------------------------------------------- reductions inside handlers

static CudaRed &cudaRed(SpecLoop *s, long redIndex, const char *what) {
    GB_CHECK(redIndex >= 1 && redIndex <= (long)s->loop->reds.size(), "invalid reduction number %ld in %s", redIndex,
             what);
    for (auto &cr : s->reds)
        if (cr.index == redIndex) return cr;
    GB_CHECK(false, "%s: reduction #%ld was not registered with dvmh_loop_cuda_register_red_C", what, redIndex);
    return s->reds[0];
}

void dvmh_loop_cuda_register_red_C(DvmType curLoop, DvmType redIndex, void **arrayAddrPtr, void **locAddrPtr) {
    SpecLoop *s = specOf(curLoop, "dvmh_loop_cuda_register_red");
    GB_CHECK(redIndex >= 1 && redIndex <= (long)s->loop->reds.size(), "invalid reduction number %ld", (long)redIndex);
    for (auto &cr : s->reds) GB_CHECK(cr.index != redIndex, "double registration of reduction #%ld", (long)redIndex);
    CudaRed cr;
    cr.index = (int)redIndex;
    cr.arrPtrSlot = arrayAddrPtr;
    cr.locPtrSlot = locAddrPtr;
    s->reds.push_back(cr);
}

// Per-thread starting value: the identity of the operation.  For MAX/MIN/AND/OR
// the reference hands out the initial value instead (loop.cpp:90-93); both give
// the same result because the initial value is combined again at the end.
void dvmh_loop_red_init_C(DvmType curLoop, DvmType redIndex, void *arrayAddr, void *locAddr) {
    SpecLoop *s = specOf(curLoop, "dvmh_loop_red_init");
    GB_CHECK(redIndex >= 1 && redIndex <= (long)s->loop->reds.size(), "invalid reduction number %ld", (long)redIndex);
    Reduction &r = s->loop->reds[redIndex - 1];
    if (arrayAddr)
        for (long i = 0; i < r.count; i++) identityValue(r.op, r.vtype, (char *)arrayAddr + i * r.esize);
    if (locAddr && r.locAddr) memcpy(locAddr, r.initLoc.data(), r.initLoc.size());
}

void dvmh_loop_cuda_red_init_C(DvmType curLoop, DvmType redIndex, void **devArrayAddrPtr, void **devLocAddrPtr) {
    SpecLoop *s = specOf(curLoop, "dvmh_loop_cuda_red_init");
    CudaRed &cr = cudaRed(s, redIndex, "dvmh_loop_cuda_red_init");
    Reduction &r = s->loop->reds[redIndex - 1];
    cr.count = 1;
    cr.items = (char *)devAlloc(r.esize * r.count);
    s->scratch.push_back(cr.items);
    fillIdentity(r.op, r.vtype, cr.items, r.count, s->stream);
    if (devArrayAddrPtr) *devArrayAddrPtr = cr.items;
    if (r.locAddr) {
        cr.locItems = (char *)devAlloc(r.locSize * r.count);
        s->scratch.push_back(cr.locItems);
        GB_CUDA(cudaMemsetAsync(cr.locItems, 0, r.locSize * r.count, s->stream));
    }
    if (devLocAddrPtr) *devLocAddrPtr = cr.locItems;
}

void dvmh_loop_cuda_red_prepare_C(DvmType curLoop, DvmType redIndex, DvmType count, DvmType fillFlag) {
    SpecLoop *s = specOf(curLoop, "dvmh_loop_cuda_red_prepare");
    CudaRed &cr = cudaRed(s, redIndex, "dvmh_loop_cuda_red_prepare");
    GB_CHECK(count > 0, "reduction buffer length must be positive (given %ld)", (long)count);
    Reduction &r = s->loop->reds[redIndex - 1];
    cr.count = (long)count;
    cr.items = (char *)devAlloc(r.esize * r.count * cr.count);
    s->scratch.push_back(cr.items);
    if (fillFlag) fillIdentity(r.op, r.vtype, cr.items, r.count * cr.count, s->stream);
    if (cr.arrPtrSlot) *cr.arrPtrSlot = cr.items;
    if (r.locAddr) {
        cr.locItems = (char *)devAlloc(r.locSize * r.count * cr.count);
        s->scratch.push_back(cr.locItems);
        if (fillFlag) GB_CUDA(cudaMemsetAsync(cr.locItems, 0, r.locSize * r.count * cr.count, s->stream));
        if (cr.locPtrSlot) *cr.locPtrSlot = cr.locItems;
    }
}

void dvmh_loop_cuda_red_finish_C(DvmType curLoop, DvmType redIndex) {
    SpecLoop *s = specOf(curLoop, "dvmh_loop_cuda_red_finish");
    CudaRed &cr = cudaRed(s, redIndex, "dvmh_loop_cuda_red_finish");
    GB_CHECK(cr.items, "reduction #%ld finished before dvmh_loop_cuda_red_prepare_C", (long)redIndex);
    GB_CHECK(!cr.finished, "reduction #%ld finished twice", (long)redIndex);
    Reduction &r = s->loop->reds[redIndex - 1];
    char *dst = r.var->dev + r.varOff;
    char *dstLoc = r.locVar ? r.locVar->dev + r.locVarOff : nullptr;
    if (deferFolds && foldBatchable(r.op, r.vtype, cr.count, r.count))
        deferred.push_back({r.op, cr.count, cr.items, cr.locItems, r.locSize, dst, dstLoc});
    else
        launchRedFold(r.op, r.vtype, cr.count, r.count, cr.items, cr.locItems, r.locSize, dst, dstLoc, s->stream,
                      s->scratch);
    cr.finished = true;
}

void dvmh_loop_red_post_C(DvmType curLoop, DvmType redIndex, const void *arrayAddr, const void *locAddr) {
    (void)curLoop;
    (void)redIndex;
    (void)arrayAddr;
    (void)locAddr;
    GB_CHECK(false, "dvmh_loop_red_post_C belongs to host handlers, which this runtime does not execute");
}

// ---------------------------------------------------------------- axis permutations (dvmh2.cpp:4517-4583)

static int bitCount(long v) {
    int c = 0;
    for (; v; v &= v - 1) c++;
    return c;
}

static void applyPerm(long rank, DvmType *vals, const DvmType *perm) {
    DvmType tmp[MAXR];
    for (long i = 0; i < rank; i++) tmp[i] = vals[perm[i] - 1];
    memcpy(vals, tmp, sizeof(DvmType) * rank);
}

void dvmh_change_filled_bounds_C(DvmType boundsLow[], DvmType boundsHigh[], DvmType loopSteps[], DvmType rank,
                                 DvmType depMask, DvmType idxPerm[]) {
    // dependent axes last; idxPerm: permuted position -> original axis (1-based)
    int depCount = bitCount(depMask);
    long h = rank - depCount, hd = 0;
    for (long i = 1; i <= rank; i++) {
        if ((depMask >> (rank - i)) & 1) idxPerm[h++] = i;
        else idxPerm[hd++] = i;
    }
    if (depCount > 0 && depCount < rank) {
        applyPerm(rank, boundsLow, idxPerm);
        applyPerm(rank, boundsHigh, idxPerm);
        applyPerm(rank, loopSteps, idxPerm);
    }
}

void dvmh_change_filled_bounds2_C(DvmType boundsLow[], DvmType boundsHigh[], DvmType loopSteps[], DvmType rank,
                                  DvmType depMask, DvmType idxPerm[]) {
    // dependent axes first; idxPerm returned 0-based
    int depCount = bitCount(depMask);
    long h = 0, hd = depCount;
    for (long i = 1; i <= rank; i++) {
        if ((depMask >> (rank - i)) & 1) idxPerm[h++] = i;
        else idxPerm[hd++] = i;
    }
    if (depCount > 0 && depCount < rank) {
        applyPerm(rank, boundsLow, idxPerm);
        applyPerm(rank, boundsHigh, idxPerm);
        applyPerm(rank, loopSteps, idxPerm);
    }
    for (long i = 0; i < rank; i++) idxPerm[i]--;
}

// ---------------------------------------------------------------- extension API

void dvmhgb_set_mode(int mode) {
    GB_CHECK(mode >= MODE_PLAIN && mode <= MODE_BATCHED, "unknown mode %d", mode);
    queueFlush();
    settings.mode = mode;
}

int dvmhgb_get_mode(void) { return settings.mode; }

void dvmhgb_set_autotransform(int on) {
    queueFlush();
    settings.autoTfm = on != 0;
}

int dvmhgb_get_autotransform(void) { return settings.autoTfm ? 1 : 0; }

void dvmhgb_set_reduce_dependences(int on) {
    queueFlush();
    settings.reduceDeps = on != 0;
}

void dvmhgb_flush(void) { queueFlush(); }

void dvmhgb_set_deferral(int on) {
    queueFlush();
    settings.defer = on != 0;
}

void dvmhgb_sync(void) {
    queueFlush();
    streamSync();
}

void dvmhgb_register_fusion(DvmHandlerFunc first, DvmHandlerFunc second, DvmHandlerFunc fused) {
    GB_CHECK(first && second && fused, "NULL handler in dvmhgb_register_fusion");
    for (auto &r : fusionRules)
        if (r.first == first && r.second == second) {
            r.fused = fused;
            return;
        }
    fusionRules.push_back({first, second, fused});
}

void dvmhgb_register_batch(DvmHandlerFunc single, DvmHandlerFunc batched) {
    GB_CHECK(single && batched, "NULL handler in dvmhgb_register_batch");
    batchRules[(void *)single] = batched;
}

void dvmhgb_force_variant(int v) { forcedVariant = v < 0 ? -1 : v; }

int dvmhgb_loop_variant_desc(DvmType loopRef, int nvariants, int dflt, const float *desc, int ndesc) {
    SpecLoop *s = specOf(loopRef, "dvmhgb_loop_variant");
    GB_CHECK(nvariants >= 1 && dflt >= 0 && dflt < nvariants, "invalid variant request");
    GB_CHECK(ndesc >= 0 && ndesc <= DVMHGB_VARIANT_NDESC && (ndesc == 0 || desc), "invalid variant description");
    const int forced = forcedVariant;
    int v = s->variant >= 0 ? s->variant : dflt;
    // online tuning explores only in immediate execution (a captured graph keeps its choice)
    if (settings.tuneMode && forced < 0) v = tunerVariant(s, nvariants, dflt, desc, ndesc, ctx.capturing);
    if (forced >= 0) v = forced;
    v = v < nvariants ? v : nvariants - 1;
    s->variant = v;
    return v;
}

int dvmhgb_loop_variant(DvmType loopRef, int nvariants, int dflt) {
    return dvmhgb_loop_variant_desc(loopRef, nvariants, dflt, nullptr, 0);
}

void *dvmhgb_loop_scratch(DvmType loopRef, DvmType bytes) {
    SpecLoop *s = specOf(loopRef, "dvmhgb_loop_scratch");
    GB_CHECK(bytes > 0, "scratch size must be positive");
    void *p = devAlloc((size_t)bytes);
    s->scratch.push_back(p);
    return p;
}

void *dvmhgb_loop_host_scratch(DvmType loopRef, DvmType bytes) {
    SpecLoop *s = specOf(loopRef, "dvmhgb_loop_host_scratch");
    GB_CHECK(bytes > 0, "scratch size must be positive");
    void *p = hostAlloc((size_t)bytes);
    s->hostScratch.push_back(p);
    return p;
}

int *dvmhgb_status_word(void) { return gpu.statusDev; }

void dvmhgb_set_timing(int on) {
    queueFlush();
    timingOn = on != 0;
}

int dvmhgb_timing_get(DvmHandlerFunc handler, double *totalMs, long *count) {
    streamSync();
    auto it = timingTotals.find((void *)handler);
    if (totalMs) *totalMs = it == timingTotals.end() ? 0.0 : it->second.ms;
    if (count) *count = it == timingTotals.end() ? 0 : it->second.count;
    return it == timingTotals.end() ? -1 : 0;
}

void dvmhgb_timing_reset(void) {
    streamSync();
    timingTotals.clear();
}

void *dvmhgb_loop_param(DvmType loopRef, DvmType index) {
    SpecLoop *s = specOf(loopRef, "dvmhgb_loop_param");
    GB_CHECK(index >= 0 && index < s->loop->cuda.nparams, "parameter index %ld out of range", (long)index);
    return s->loop->cuda.params[index];
}

void *dvmhgb_loop_alt_buffer(DvmType loopRef, const DvmType dvmDesc[]) {
    SpecLoop *s = specOf(loopRef, "dvmhgb_loop_alt_buffer");
    Array *a = arrayOf(dvmDesc, "dvmhgb_loop_alt_buffer");
    GB_CHECK(a->dev, "array has no device copy");
    if (!a->devAlt) a->devAlt = (char *)devAlloc(a->devBytes());
    for (Array *x : s->swaps) GB_CHECK(x != a, "alternate buffer requested twice in one loop");
    s->swaps.push_back(a);
    return a->devAlt;
}

}  // extern "C"
