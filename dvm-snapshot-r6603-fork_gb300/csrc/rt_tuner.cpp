// libdvmh_gb tuner: the CUDA-block / kernel-variant autotuner, its timing
// database, and the learned cost model that prunes its search.
//
// Reference counterpart (rts/dvmh/loop.cpp): CudaHandlerOptimizationParams
// (:1464-1575, default blocks 256 / 32x8 / 32x4x2, the serialised block list
// of genParamsRanges :1487-1532), ParamDesc's online search (:1579-1640),
// LoopHandlerPerformanceInfo (:1644-1971, timings recorded per execution),
// DvmhLoopPersistentInfo keyed by the loop's source position (:1975-2062).
// Here:
//   * every timed execution is recorded (features of loop and candidate,
//     seconds) -- the runtime's timing database, also exported for training;
//   * exhaustive tuning (DVMH_OPT_PARAMS=1) tries every candidate of a loop
//     signature once, in successive executions, then keeps the fastest;
//   * model-guided tuning (DVMH_OPT_PARAMS=2) ranks the candidates with the
//     FP32 MLP (csrc/kernels/mlp.cu) and tries only the top k;
//   * for the hand-written kernels the candidates are their variants (how
//     many FP64 operations run on the FP64 unit), chosen online per loop.
#include <algorithm>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <map>
#include <unordered_map>
#include <vector>

#include "rt.h"
#include "../../include/dvmh_gb_kernels.h"

namespace dvmhgb {

extern dvmhgb_stats_t stats;
static float lg(double v) { return (float)std::log2(v > 1 ? v : 1); }

// ---------------------------------------------------------------- timing database

struct Record {
    float f[DVMHGB_TUNE_NF];
    long loopId;
    int cand;
    double seconds;
};
static std::vector<Record> db;

// ---------------------------------------------------------------- online variant tuning of ABI loops

static bool variantModelReady();
static void rankByVariantModel(const std::vector<std::vector<float>> &feats, std::vector<int> &order);

//
// Per loop shape and handler (the tuner's key): the fastest seconds seen for
// each variant.  Exhaustive tuning hands out every untried variant in turn;
// model-guided tuning ranks the variants by the variant model (features of
// the loop and of each variant's description) and hands out only the first
// floor(frac x nvariants) of that order (none: the first is kept untried).
// Afterwards the fastest variant timed is kept; before anything is timed, the
// default (exhaustive) or the model's first choice.

struct VariantState {
    std::map<int, double> best;  // variant -> best seconds seen
    std::map<int, int> runs;     // variant -> timed executions
    int nvariants = 0;
    int chosen = -1;
    std::vector<int> order;      // model-guided: variants fastest first by the model
    int explore = -1;            // variants to try (-1: all)
    bool ranked = false;         // model-guided: the model has ordered the variants
    int explored = 0;            // executions that tried an untried variant
    double exploreSeconds = 0;   // their summed time
    void *handler = nullptr;
};
static std::unordered_map<uint64_t, VariantState> vstate;
static std::vector<uint64_t> vorder;  // keys in the order first seen
static long uncapturedFlushes = 0;    // flushes run eagerly since tuning was reset
static std::vector<Record> vdb;       // the variant database

// timed executions of each variant tried (the fastest counts): one run of a
// variant can carry first-use costs (a second buffer, a stream) or noise.
// Read at every query, so that a tuning session can set it for itself.
static int tuneReps() {
    const char *e = getenv("DVMH_GB_TUNE_REPS");
    const int r = e ? atoi(e) : 2;
    return r < 1 ? 1 : r;
}

static double tuneFrac() {
    static double f = -1;
    if (f < 0) {
        const char *e = getenv("DVMH_GB_TUNE_FRAC");
        f = e ? atof(e) : 0.1;
        if (f < 0) f = 0;
    }
    return f;
}

static uint64_t loopKey(const void *handler, const Loop *l) {
    uint64_t h = (uint64_t)handler * 0x9E3779B97F4A7C15ull;
    for (int i = 0; i < l->rank; i++) h = (h ^ (uint64_t)(l->hi[i] - l->lo[i] + 1)) * 1099511628211ull;
    h ^= (uint64_t)l->depMask;
    return h ? h : 1;
}

// features of a loop and one variant's description
static void variantFeatures(const Loop *l, const float *desc, int ndesc, float *f) {
    memset(f, 0, sizeof(float) * TUNE_NF);
    double total = 1;
    for (int a = 0; a < l->rank; a++) total *= (double)(l->hi[a] - l->lo[a] + 1);
    f[0] = (float)l->rank;
    for (int a = 0; a < 4 && a < l->rank; a++) f[1 + a] = lg((double)(l->hi[a] - l->lo[a] + 1));
    f[5] = lg(total);
    f[6] = (float)(l->depMask != 0);
    f[7] = (float)l->reds.size();
    for (int d = 0; d < ndesc && 8 + d < TUNE_NF; d++) f[8 + d] = desc[d];
}

bool tunerWants(const Loop *l) { return settings.tuneMode != 0 && l->hasCuda; }

void tunerPick(Loop *l, int block[3], int *variant) {
    (void)l;
    (void)block;
    (void)variant;  // the variant is chosen when the handler asks (dvmhgb_loop_variant)
}

static bool tried(const VariantState &vs, int v) {
    auto it = vs.runs.find(v);
    return it != vs.runs.end() && it->second >= tuneReps();
}

static bool explorationDone(const VariantState &vs) {
    if (vs.explore >= 0) {
        for (int i = 0; i < vs.explore; i++)
            if (!tried(vs, vs.order[i])) return false;
        return true;
    }
    for (int v = 0; v < vs.nvariants; v++)
        if (!tried(vs, v)) return false;
    return true;
}

int tunerVariant(SpecLoop *s, int nvariants, int dflt, const float *desc, int ndesc, bool bestOnly) {
    const Loop *l = s->loop;
    const uint64_t key = loopKey(s->handler ? s->handler : (void *)l->cuda.func, l);
    auto found = vstate.find(key);
    if (found == vstate.end()) vorder.push_back(key);
    VariantState &vs = vstate[key];
    vs.handler = s->handler;
    if (vs.nvariants != nvariants) {
        vs = VariantState();
        vs.handler = s->handler;
        vs.nvariants = nvariants;
    }
    // the model ranks the variants at the first query outside a graph capture
    // (its inference runs kernels and reads their result); a query inside a
    // capture gets the default, and the shape counts as exploring until then,
    // so the next flush runs uncaptured
    if (!vs.ranked && !bestOnly && settings.tuneMode == 2 && ndesc > 0 && variantModelReady()) {
        std::vector<std::vector<float>> feats(nvariants, std::vector<float>(TUNE_NF));
        for (int v = 0; v < nvariants; v++) variantFeatures(l, desc + (size_t)v * ndesc, ndesc, feats[v].data());
        rankByVariantModel(feats, vs.order);
        vs.explore = (int)std::floor(tuneFrac() * nvariants);
        vs.ranked = true;
    }
    int v = -1;
    bool exploring = false;
    if (!bestOnly && !explorationDone(vs)) {
        if (vs.explore >= 0) {
            for (int i = 0; i < vs.explore && v < 0; i++)
                if (!tried(vs, vs.order[i])) v = vs.order[i];
        } else {
            for (int c = 0; c < nvariants && v < 0; c++)
                if (!tried(vs, c)) v = c;
        }
        exploring = v >= 0;
    }
    if (v < 0) {
        double bestT = 1e300;
        for (auto &kv : vs.best)
            if (kv.second < bestT) {
                bestT = kv.second;
                v = kv.first;
            }
        if (v < 0) v = vs.explore >= 0 ? vs.order[0] : dflt;
    }
    vs.chosen = v;
    s->tkey = key;
    s->exploring = exploring;
    variantFeatures(l, desc ? desc + (size_t)v * ndesc : nullptr, desc ? ndesc : 0, s->vf);
    s->vf[TUNE_NF - 1] = desc ? s->vf[TUNE_NF - 1] : (float)v;  // no description: the variant number itself
    return v;
}

void tunerRecord(uint64_t key, int variant, bool exploring, const float *vf, double seconds) {
    if (variant < 0) return;
    auto it = vstate.find(key);
    if (it == vstate.end()) return;
    VariantState &vs = it->second;
    auto b = vs.best.find(variant);
    if (b == vs.best.end() || seconds < b->second) vs.best[variant] = seconds;
    vs.runs[variant]++;
    if (exploring) {
        vs.explored++;
        vs.exploreSeconds += seconds;
    }
    Record rec;
    memcpy(rec.f, vf, sizeof rec.f);
    rec.loopId = (long)key;
    rec.cand = variant;
    rec.seconds = seconds;
    vdb.push_back(rec);
}

bool tunerExploring() {
    if (uncapturedFlushes == 0) return true;  // the loops' handlers have not asked yet
    for (auto &kv : vstate)
        if (!explorationDone(kv.second)) return true;
    return false;
}

void tunerFlushed() {
    uncapturedFlushes++;
    streamSync();  // the timings of this flush reach the tuner before the next decision
}

// ---------------------------------------------------------------- online layout tuning of ACROSS loops
//
// For a loop whose handler asks for transforms, the tuner chooses between the
// reference's layout (1) and the natural one (0): in immediate execution it
// runs each twice in a row (the second run of each pays no relayout), then
// keeps the faster; a captured graph takes the best known, or the
// reference's layout before anything is known.

struct LayoutTune {
    double best[2] = {1e300, 1e300};
    int runs[2] = {0, 0};
};
static std::unordered_map<uint64_t, LayoutTune> lstate;
static std::unordered_map<void *, uint64_t> lastLayoutKey;  // handler -> its most recent loop shape

int tunerLayout(const Loop *l, bool explore) {
    LayoutTune &t = lstate[loopKey((void *)l->cuda.func, l)];
    lastLayoutKey[(void *)l->cuda.func] = loopKey((void *)l->cuda.func, l);
    if (explore) {
        if (t.runs[1] < 2) return 1;
        if (t.runs[0] < 2) return 0;
    }
    if (t.runs[0] == 0 || t.runs[1] == 0) return 1;
    return t.best[0] < t.best[1] ? 0 : 1;
}

void tunerRecordLayout(const Loop *l, int choice, double seconds) {
    if (choice < 0 || choice > 1) return;
    LayoutTune &t = lstate[loopKey((void *)l->cuda.func, l)];
    t.runs[choice]++;
    if (seconds < t.best[choice]) t.best[choice] = seconds;
}

// ---------------------------------------------------------------- synthetic loops: candidates, features

static const int BLOCKS[][3] = {{32, 1, 1},  {64, 1, 1},  {128, 1, 1}, {256, 1, 1}, {512, 1, 1}, {1024, 1, 1},
                                {32, 2, 1},  {32, 4, 1},  {32, 8, 1},  {32, 16, 1}, {64, 2, 1},  {64, 4, 1},
                                {64, 8, 1},  {128, 2, 1}, {128, 4, 1}, {16, 16, 1}, {8, 32, 1},  {16, 4, 1},
                                {32, 4, 2},  {32, 8, 2},  {32, 2, 4},  {16, 8, 2},  {64, 2, 2},  {32, 4, 4},
                                {16, 4, 4},  {8, 8, 4},   {64, 4, 2},  {128, 2, 2}};

// The reference's default block for a loop of this rank (loop.cpp:1464-1485).
static void defaultFor(int rank, int b[3]) {
    b[0] = rank == 1 ? 256 : 32;
    b[1] = rank == 1 ? 1 : (rank == 2 ? 8 : 4);
    b[2] = rank >= 3 ? 2 : 1;
}

// Every launchable (block, elements per thread, axis on x) of the loop; when
// there are more than maxOut, an evenly spread subset of them (so that every
// kind of block stays represented), always with the reference's default block.
static int candidates(const dvmhgb_synth_loop *L, dvmhgb_synth_cand *out, int maxOut) {
    std::vector<dvmhgb_synth_cand> all;
    int dflt = -1, db[3];
    defaultFor(L->rank, db);
    for (const auto &b : BLOCKS) {
        if (b[1] > 1 && L->rank < 2) continue;
        if (b[2] > 1 && L->rank < 3 && !L->across) continue;
        // elements per thread 1, 2 (and 4 for rank-1 loops, whose block has one axis: 16+ candidates each)
        for (int ept = 1; ept <= (L->rank == 1 ? 4 : 2); ept *= 2)
            for (int xin = 1; xin >= 0; xin--) {
                if (!xin && (L->rank == 1 || L->across)) continue;
                dvmhgb_synth_cand c{b[0], b[1], b[2], xin, ept};
                if (dvmhgb_synth_items(L, &c) < 0) continue;
                if (b[0] == db[0] && b[1] == db[1] && b[2] == db[2] && xin == 1 && ept == 1) dflt = (int)all.size();
                all.push_back(c);
            }
    }
    const int n = (int)all.size();
    if (maxOut <= 0) return 0;
    if (n <= maxOut) {
        for (int q = 0; q < n; q++) out[q] = all[q];
        return n;
    }
    bool hasDflt = false;
    for (int q = 0; q < maxOut; q++) {
        const int src = (int)((long)q * n / maxOut);
        out[q] = all[src];
        hasDflt = hasDflt || src == dflt;
    }
    if (dflt >= 0 && !hasDflt) out[(int)((long)dflt * maxOut / n)] = all[dflt];  // in its own neighbourhood
    return maxOut;
}


static void features(const dvmhgb_synth_loop *L, const dvmhgb_synth_cand *C, float *f) {
    memset(f, 0, sizeof(float) * DVMHGB_TUNE_NF);
    double total = 1, inner = (double)L->ext[L->rank - 1], outer = (double)L->ext[0];
    for (int a = 0; a < L->rank; a++) total *= (double)L->ext[a];
    int k = 0;
    f[k++] = (float)L->rank;
    for (int a = 0; a < 4; a++) f[k++] = a < L->rank ? lg((double)L->ext[a]) : 0.0f;
    f[k++] = lg(total);
    f[k++] = (float)L->radius;
    f[k++] = (float)L->esize / 4.0f;
    f[k++] = (float)L->isint;
    f[k++] = (float)(L->red == 1);
    f[k++] = (float)(L->red == 2);
    f[k++] = (float)(L->red == 3);
    f[k++] = (float)L->across;
    f[k++] = lg(C->bx);
    f[k++] = lg(C->by);
    f[k++] = lg(C->bz);
    f[k++] = lg((double)C->bx * C->by * C->bz);
    f[k++] = (float)C->ept;
    f[k++] = (float)C->xinner;
    double xext = C->xinner ? inner : outer;
    f[k++] = lg(xext / ((double)C->bx * C->ept));                                 // blocks along x
    f[k++] = lg(std::max(1.0, total / ((double)C->bx * C->by * C->bz * C->ept)));  // blocks in all
    f[k++] = lg(xext) - lg((double)C->bx * C->ept);                               // x fill (waste)
    f[k++] = (float)((long)xext % (C->bx * C->ept) == 0);
    f[k++] = lg(total * (1 + 2 * L->radius * L->rank) * L->esize);                 // bytes touched
}

// ---------------------------------------------------------------- learned model

// the cost model of synthetic candidates, and the variant model of
// variant-choosing handlers: packed MLP parameters (host copy), the
// per-feature normalisation used in training, the parameters on the device
struct Mlp {
    std::vector<float> params, mean, stdv;
    float *dev = nullptr;
    bool empty() const { return params.empty(); }
};
static Mlp model, vmodelStore;

static void rankBy(const Mlp &m, const std::vector<std::vector<float>> &feats, std::vector<int> &order) {
    int n = (int)feats.size();
    order.resize(n);
    for (int i = 0; i < n; i++) order[i] = i;
    if (m.empty() || n == 0) return;
    std::vector<float> X((size_t)n * DVMHGB_TUNE_NF);
    for (int i = 0; i < n; i++)
        for (int j = 0; j < DVMHGB_TUNE_NF; j++)
            X[(size_t)i * DVMHGB_TUNE_NF + j] = (feats[i][j] - m.mean[j]) / m.stdv[j];
    float *dX = (float *)devAlloc(X.size() * sizeof(float));
    float *dY = (float *)devAlloc(n * sizeof(float));
    float *work = (float *)devAlloc(dvmhgb_mlp_work_floats(n) * sizeof(float));
    GB_CUDA(cudaMemcpyAsync(dX, X.data(), X.size() * sizeof(float), cudaMemcpyHostToDevice, gpu.stream));
    GB_CHECK(dvmhgb_mlp_forward(m.dev, dX, n, dY, work, gpu.stream) == 0, "cost model forward failed");
    std::vector<float> y(n);
    GB_CUDA(cudaMemcpyAsync(y.data(), dY, n * sizeof(float), cudaMemcpyDeviceToHost, gpu.stream));
    streamSync();
    devFree(dX);
    devFree(dY);
    devFree(work);
    std::stable_sort(order.begin(), order.end(), [&](int a, int b) { return y[a] < y[b]; });
}

static void rankByModel(const std::vector<std::vector<float>> &feats, std::vector<int> &order) {
    rankBy(model, feats, order);
}
static void rankByVariantModel(const std::vector<std::vector<float>> &feats, std::vector<int> &order) {
    rankBy(vmodelStore, feats, order);
}
static bool variantModelReady() { return !vmodelStore.empty(); }

static void install(Mlp &m, const float *params, const float *mean, const float *stdv) {
    long np = dvmhgb_mlp_nparams();
    m.params.assign(params, params + np);
    m.mean.assign(mean, mean + DVMHGB_TUNE_NF);
    m.stdv.assign(stdv, stdv + DVMHGB_TUNE_NF);
    for (auto &x : m.stdv)
        if (x <= 0) x = 1;
    if (m.dev) devFree(m.dev);
    m.dev = (float *)devAlloc(np * sizeof(float));
    GB_CUDA(cudaMemcpy(m.dev, m.params.data(), np * sizeof(float), cudaMemcpyHostToDevice));
}

}  // namespace dvmhgb

using namespace dvmhgb;

extern "C" {

int dvmhgb_tuner_candidates(const dvmhgb_synth_loop *L, dvmhgb_synth_cand *out, int maxOut) {
    return candidates(L, out, maxOut);
}

void dvmhgb_tuner_features(const dvmhgb_synth_loop *L, const dvmhgb_synth_cand *C, float *f) { features(L, C, f); }

// Runs the synthetic loop with candidate C `reps` times on the runtime stream
// (one untimed warm-up first) and records the fastest into the database.
double dvmhgb_tuner_time_synth(const dvmhgb_synth_loop *L, const dvmhgb_synth_cand *C, long loopId, int cand,
                               int reps) {
    long elems = dvmhgb_synth_elems(L), items = dvmhgb_synth_items(L, C);
    if (elems <= 0 || items < 0) return -1;
    size_t bytes = (size_t)elems * L->esize;
    void *in = devAlloc(bytes), *out = devAlloc(bytes);
    void *it = devAlloc((size_t)std::max(items, 1L) * 8);
    long *locs = (long *)devAlloc((size_t)std::max(items, 1L) * 8);
    GB_CUDA(cudaMemsetAsync(in, 0, bytes, gpu.stream));
    cudaEvent_t e0, e1;
    GB_CUDA(cudaEventCreate(&e0));
    GB_CUDA(cudaEventCreate(&e1));
    double best = 1e300;
    int rc = dvmhgb_synth_run(L, C, in, out, it, locs, gpu.stream);
    for (int r = 0; rc == 0 && r < reps; r++) {
        GB_CUDA(cudaEventRecord(e0, gpu.stream));
        rc = dvmhgb_synth_run(L, C, in, out, it, locs, gpu.stream);
        GB_CUDA(cudaEventRecord(e1, gpu.stream));
        GB_CUDA(cudaEventSynchronize(e1));
        float ms = 0;
        GB_CUDA(cudaEventElapsedTime(&ms, e0, e1));
        best = std::min(best, (double)ms * 1e-3);
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    streamSync();
    devFree(in);
    devFree(out);
    devFree(it);
    devFree(locs);
    if (rc != 0) return -1;
    Record rec;
    features(L, C, rec.f);
    rec.loopId = loopId;
    rec.cand = cand;
    rec.seconds = best;
    db.push_back(rec);
    return best;
}

// All candidates of one loop: buffers allocated once, every candidate run once
// untimed and `reps` times timed back to back, one synchronisation at the end;
// the fastest run of each candidate is recorded.  times[i] = -1 for a
// candidate the launcher rejects.
int dvmhgb_tuner_time_synth_all(const dvmhgb_synth_loop *L, const dvmhgb_synth_cand *cands, int n, long loopId,
                                int reps, double *times) {
    long elems = dvmhgb_synth_elems(L), maxItems = 1;
    for (int i = 0; i < n; i++) maxItems = std::max(maxItems, dvmhgb_synth_items(L, &cands[i]));
    if (elems <= 0 || n < 1 || reps < 1) return -1;
    size_t bytes = (size_t)elems * L->esize;
    void *in = devAlloc(bytes), *out = devAlloc(bytes);
    void *it = devAlloc((size_t)maxItems * 8);
    long *locs = (long *)devAlloc((size_t)maxItems * 8);
    GB_CUDA(cudaMemsetAsync(in, 0, bytes, gpu.stream));
    std::vector<cudaEvent_t> ev((size_t)n * reps * 2);
    for (auto &e : ev) GB_CUDA(cudaEventCreate(&e));
    std::vector<int> ok(n, 1);
    for (int i = 0; i < n; i++) {
        if (dvmhgb_synth_run(L, &cands[i], in, out, it, locs, gpu.stream) != 0) {
            ok[i] = 0;
            continue;
        }
        for (int r = 0; r < reps; r++) {
            GB_CUDA(cudaEventRecord(ev[((size_t)i * reps + r) * 2], gpu.stream));
            dvmhgb_synth_run(L, &cands[i], in, out, it, locs, gpu.stream);
            GB_CUDA(cudaEventRecord(ev[((size_t)i * reps + r) * 2 + 1], gpu.stream));
        }
    }
    streamSync();
    for (int i = 0; i < n; i++) {
        times[i] = -1;
        if (!ok[i]) continue;
        double best = 1e300;
        for (int r = 0; r < reps; r++) {
            float ms = 0;
            GB_CUDA(cudaEventElapsedTime(&ms, ev[((size_t)i * reps + r) * 2], ev[((size_t)i * reps + r) * 2 + 1]));
            best = std::min(best, (double)ms * 1e-3);
        }
        times[i] = best;
        Record rec;
        features(L, &cands[i], rec.f);
        rec.loopId = loopId;
        rec.cand = i;
        rec.seconds = best;
        db.push_back(rec);
    }
    for (auto &e : ev) cudaEventDestroy(e);
    devFree(in);
    devFree(out);
    devFree(it);
    devFree(locs);
    return 0;
}

// The layout the tuner keeps for the most recent loop shape of a handler:
// 0 natural, 1 the reference's transform, -1 while either is unmeasured;
// best[2] (optional) gets the fastest seconds seen with each.
int dvmhgb_tuner_layout(DvmHandlerFunc handler, double best[2]) {
    auto k = lastLayoutKey.find((void *)handler);
    if (k == lastLayoutKey.end()) return -1;
    const LayoutTune &t = lstate[k->second];
    if (best) {
        best[0] = t.runs[0] ? t.best[0] : -1;
        best[1] = t.runs[1] ? t.best[1] : -1;
    }
    if (t.runs[0] < 2 || t.runs[1] < 2) return -1;
    return t.best[0] < t.best[1] ? 0 : 1;
}

void dvmhgb_set_tuning(int mode) {
    GB_CHECK(mode >= 0 && mode <= 2, "unknown tuning mode %d", mode);
    settings.tuneMode = mode;
}

long dvmhgb_tuner_db_size(void) { return (long)db.size(); }

long dvmhgb_tuner_db_export(float *X, double *seconds, long *loopIds, int *cands, long maxRows) {
    long n = std::min(maxRows, (long)db.size());
    for (long i = 0; i < n; i++) {
        if (X) memcpy(X + i * DVMHGB_TUNE_NF, db[i].f, sizeof(float) * DVMHGB_TUNE_NF);
        if (seconds) seconds[i] = db[i].seconds;
        if (loopIds) loopIds[i] = db[i].loopId;
        if (cands) cands[i] = db[i].cand;
    }
    return n;
}

void dvmhgb_tuner_db_clear(void) { db.clear(); }

// Installs the cost model: packed MLP parameters (dvmhgb_mlp_nparams floats)
// and the per-feature normalisation used in training.
int dvmhgb_tuner_set_model(const float *params, const float *mean, const float *stdv) {
    install(model, params, mean, stdv);
    return 0;
}

int dvmhgb_tuner_set_variant_model(const float *params, const float *mean, const float *stdv) {
    install(vmodelStore, params, mean, stdv);
    return 0;
}

long dvmhgb_tuner_vdb_size(void) { return (long)vdb.size(); }

long dvmhgb_tuner_vdb_export(float *X, double *seconds, unsigned long long *keys, int *variants, long maxRows) {
    long n = std::min(maxRows, (long)vdb.size());
    for (long i = 0; i < n; i++) {
        if (X) memcpy(X + i * DVMHGB_TUNE_NF, vdb[i].f, sizeof(float) * DVMHGB_TUNE_NF);
        if (seconds) seconds[i] = vdb[i].seconds;
        if (keys) keys[i] = (unsigned long long)vdb[i].loopId;
        if (variants) variants[i] = vdb[i].cand;
    }
    return n;
}

void dvmhgb_tuner_vdb_clear(void) { vdb.clear(); }

void dvmhgb_tuner_reset(void) {
    queueFlush();
    streamSync();
    vstate.clear();
    vorder.clear();
    lstate.clear();
    lastLayoutKey.clear();
    uncapturedFlushes = 0;
}

long dvmhgb_tuner_variant_count(void) { return (long)vorder.size(); }

int dvmhgb_tuner_exploring(void) {
    streamSync();  // the timings so far reach the tuner
    return settings.tuneMode && tunerExploring() ? 1 : 0;
}

int dvmhgb_tuner_variant_info(long index, DvmHandlerFunc *handler, int *nvariants, int *chosen, double *best,
                              int maxBest, int *explored, double *exploreSeconds) {
    streamSync();
    if (index < 0 || index >= (long)vorder.size()) return -1;
    const VariantState &vs = vstate[vorder[index]];
    if (handler) *handler = (DvmHandlerFunc)vs.handler;
    if (nvariants) *nvariants = vs.nvariants;
    if (chosen) {
        // the variant kept now: the fastest timed, else the default / the model's first
        int v = vs.chosen;
        double bt = 1e300;
        for (auto &kv : vs.best)
            if (kv.second < bt) bt = kv.second, v = kv.first;
        *chosen = v;
    }
    if (best)
        for (int v = 0; v < maxBest && v < vs.nvariants; v++) {
            auto it = vs.best.find(v);
            best[v] = it == vs.best.end() ? -1.0 : it->second;
        }
    if (explored) *explored = vs.explored;
    if (exploreSeconds) *exploreSeconds = vs.exploreSeconds;
    return 0;
}

// Candidate order by predicted time (fastest first) for loop L.
int dvmhgb_tuner_rank(const dvmhgb_synth_loop *L, const dvmhgb_synth_cand *cands, int n, int *order) {
    std::vector<std::vector<float>> feats(n, std::vector<float>(DVMHGB_TUNE_NF));
    for (int i = 0; i < n; i++) features(L, &cands[i], feats[i].data());
    std::vector<int> o;
    rankByModel(feats, o);
    for (int i = 0; i < n; i++) order[i] = o[i];
    return model.empty() ? -1 : 0;
}

}  // extern "C"
