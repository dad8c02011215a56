// Device layouts of distributed arrays: which layout an ACROSS loop's array
// gets (the reference's autotransform, rts/dvmh/dvmh_rts.cpp:1404-1479), the
// relayout that moves a device copy between layouts, and the header a
// handler sees (rts/dvmh/dvmh_buffer.cpp:149-182, rts/dvmh/dvmh2.cpp:2226-2258).
//
// The device copy of an array is natural unless a handler asks for a
// transform (dvmh_loop_autotransform_C).  It stays transformed from loop to
// loop -- an ACROSS time loop pays the relayout once -- and becomes natural
// again, with one more relayout, before anything that expects the natural
// layout touches it: a host<->device copy, a handler that did not ask for the
// transform (every hand-written kernel of this library reads natural rows).
// A relayout writes the second device buffer and swaps the two, so inside a
// captured graph it is a kernel node like any other and the swap and the new
// layout are replayed with the graph.
#include <algorithm>
#include <cstdlib>

#include "rt.h"
#include "rt_layout.h"

namespace dvmhgb {

extern dvmhgb_stats_t stats;

bool layoutNatural(const Array *a) { return a->tperm[0] == 0; }

int layoutState(const Array *a) { return layoutNatural(a) ? 0 : (a->tdiag ? 2 : 1); }

// Where every element of `a` lives under the layout (perm, diag): natural
// (perm[0] == 0) = the padded row-major device layout; otherwise the axes
// stored in the order perm, dense, the last two numbered along diagonals
// when diag != 0.
static LayoutDesc describe(const Array *a, const int perm[], int diag) {
    LayoutDesc L{};
    L.rank = a->rank;
    L.diagUnit = 1;
    for (int i = 0; i < a->rank; i++) L.ext[i] = a->ext[i];
    if (perm[0] == 0) {
        for (int i = 0; i < a->rank; i++) L.coef[i] = a->dstride[i];
        return L;
    }
    const int r = a->rank;
    long c = 1;
    for (int k = r - 1; k >= 0; k--) {
        const int ax = perm[k] - 1;
        L.coef[ax] = (diag && k >= r - 2) ? 0 : c;
        c *= a->ext[ax];
    }
    if (diag) {
        L.diag = 1;
        L.xAxis = perm[r - 1] - 1;
        L.yAxis = perm[r - 2] - 1;
        L.slash = diag == 2;
    }
    return L;
}

// A diagonal plane with a single row or column is the plain order (the slash
// orientation only when the plane has one row); the identity permutation
// without a diagonal is the natural layout (rts/dvmh/dvmh_buffer.cpp:331-352).
static void canonical(const Array *a, int perm[], int &diag) {
    const int r = a->rank;
    if (perm[0] == 0) {
        diag = 0;
        return;
    }
    if (diag) {
        const long Rx = a->ext[perm[r - 1] - 1], Ry = a->ext[perm[r - 2] - 1];
        if ((diag == 1 && (Rx == 1 || Ry == 1)) || (diag == 2 && Ry == 1)) diag = 0;
    }
    bool identity = true;
    for (int k = 0; k < r; k++) identity = identity && perm[k] == k + 1;
    if (identity && !diag)
        for (int k = 0; k < MAXR; k++) perm[k] = 0;
}

// Bring the device copy to the layout (perm, diag).  A device copy that holds
// nothing current changes layout without moving data.
static void setLayout(Array *a, const int permIn[], int diagIn) {
    int perm[MAXR] = {};
    int diag = diagIn;
    if (permIn)
        for (int k = 0; k < a->rank; k++) perm[k] = permIn[k];
    canonical(a, perm, diag);
    bool same = diag == a->tdiag;
    for (int k = 0; k < MAXR; k++) same = same && perm[k] == a->tperm[k];
    if (same) return;
    if (a->dev && a->devActual) {
        const LayoutDesc from = describe(a, a->tperm, a->tdiag), to = describe(a, perm, diag);
        if (!a->devAlt) a->devAlt = (char *)devAlloc(a->devBytes());
        launchRelayout(a->dev, from, a->devAlt, to, a->esize, gpu.stream);
        std::swap(a->dev, a->devAlt);
        noteSwap(a);
        stats.relayouts++;
        logmsg(LOG_DEBUG, "relayout of '%s' to state %d", a->name.c_str(), perm[0] ? (diag ? 2 : 1) : 0);
    }
    for (int k = 0; k < MAXR; k++) a->tperm[k] = perm[k];
    a->tdiag = diag;
    noteLayout(a);
}

void makeNatural(Array *a) {
    if (!layoutNatural(a)) setLayout(a, nullptr, 0);
}

// ---------------------------------------------------------------- alignment

void alignIdentity(AlignMap &m, const Obj *self, int rank) {
    m = AlignMap();
    m.root = self;
    m.rank = rank;
    for (int r = 0; r < rank; r++) {
        m.ax[r] = r + 1;
        m.sign[r] = 1;
    }
}

// `out` aligned with a target whose own axis t (0-based) maps to out's axis
// axis[t] (1-based, <= 0 none) in direction sign[t].
void alignCompose(AlignMap &out, const AlignMap &target, const int axis[], const int sign[], int targetRank) {
    AlignMap m;
    m.root = target.root;
    m.rank = target.rank;
    for (int r = 0; r < target.rank; r++) {
        const int ta = target.ax[r];
        if (ta > 0 && ta <= targetRank && axis[ta - 1] > 0 && sign[ta - 1] != 0) {
            m.ax[r] = axis[ta - 1];
            m.sign[r] = target.sign[r] * sign[ta - 1];
        }
    }
    out = m;
}

// loop axis -> +-array axis (1-based; 0 = no array axis follows that loop axis),
// the direction including the loop step's sign (rts/dvmh/loop.cpp:794-823)
static bool correspondence(const Loop *l, const Array *a, int corr[]) {
    for (int i = 0; i < MAXR; i++) corr[i] = 0;
    if (!l->map.root || l->map.root != a->align.root) return false;
    for (int r = 0; r < l->map.rank; r++) {
        const int la = l->map.ax[r], da = a->align.ax[r];
        if (la > 0 && la <= l->rank && da > 0)
            corr[la - 1] = da * (l->step[la - 1] < 0 ? -1 : 1) * l->map.sign[r] * a->align.sign[r];
    }
    return true;
}

int loopAxisOf(const Loop *l, const Array *a, int axis) {
    if (l->map.root && l->map.root == a->align.root) {
        for (int r = 0; r < l->map.rank; r++)
            if (a->align.ax[r] == axis + 1) return l->map.ax[r] <= l->rank ? l->map.ax[r] : 0;
        return 0;
    }
    // no common distribution root known: the mapped array's own axes
    return axis < MAXR ? l->arrAxisToLoop[axis] : 0;
}

// position (0-based) of the n-th lowest set bit, -1 if there are fewer
static int nthBit(unsigned long v, int n) {
    for (int i = 0; i < 64; i++)
        if ((v >> i) & 1ul)
            if (--n == 0) return i;
    return -1;
}

// ---------------------------------------------------------------- the reference's choice

// With at most one dependence and an independent loop axis, the array axis
// that follows the fastest independent loop axis is stored innermost (its
// cells are the ones a warp updates together).  With two or more
// dependences, the array axes of the two fastest dependent loop axes are
// stored last and numbered along the diagonal the loop sweeps; opposite
// directions of the two give the slash orientation.  Otherwise a diagonal
// is undone when at most one dependence is left.
int autotransform(const Loop *l, Array *a) {
    if (a->rank <= 1) return layoutState(a);
    if (!settings.autoTfm) {
        makeNatural(a);
        return 0;
    }
    const unsigned long dep = (unsigned long)l->depMask;
    const int depCount = __builtin_popcountl(dep);
    int corr[MAXR];
    correspondence(l, a, corr);
    int perm[MAXR] = {};
    for (int k = 0; k < a->rank; k++) perm[k] = layoutNatural(a) ? k + 1 : a->tperm[k];
    const int r = a->rank;
    auto moveTo = [&](int axis, int place) {
        const int at = (int)(std::find(perm, perm + r, axis) - perm);
        std::swap(perm[at], perm[place]);
    };
    bool done = false;
    if (l->rank > depCount && depCount <= 1) {
        const int fastest = l->rank - nthBit(~dep, 1);
        const int da = std::abs(corr[fastest - 1]);
        if (da > 0) {
            moveTo(da, r - 1);
            setLayout(a, perm, 0);
            done = true;
        }
    } else if (depCount >= 2) {
        const int fastest = l->rank - nthBit(dep, 1), prev = l->rank - nthBit(dep, 2);
        const int dx = std::abs(corr[fastest - 1]), dy = std::abs(corr[prev - 1]);
        if (dx > 0 && dy > 0 && dx != dy) {
            moveTo(dx, r - 1);
            moveTo(dy, r - 2);
            const bool slash = (corr[fastest - 1] > 0) != (corr[prev - 1] > 0);
            setLayout(a, perm, slash ? 2 : 1);
            done = true;
        }
    }
    if (!done && depCount <= 1 && a->tdiag) setLayout(a, a->tperm, 0);
    return layoutState(a);
}

// ---------------------------------------------------------------- headers

// Per-axis coefficients of the current device layout and, when diagonalised,
// the plane's description as dvmh_fill_header_C reports it: x axis, its first
// index, its extent, the same for y, and the orientation.
void layoutHeader(const Array *a, long coef[], long ext7[7]) {
    const LayoutDesc L = describe(a, a->tperm, a->tdiag);
    for (int i = 0; i < a->rank; i++) coef[i] = L.coef[i];
    if (L.diag) {
        ext7[0] = L.xAxis + 1;
        ext7[1] = 0;
        ext7[2] = a->ext[L.xAxis];
        ext7[3] = L.yAxis + 1;
        ext7[4] = 0;
        ext7[5] = a->ext[L.yAxis];
        ext7[6] = L.slash;
    }
}

}  // namespace dvmhgb
