// The 3-D Jacobi stencil loop, Out = (6 neighbours of the source) / 6, with the
// source planes staged in shared memory by the Tensor Memory Accelerator and
// the sums in the q61 fixed-point form of softfp64.cuh.  M = 0: the loop
// alone, source A; M = 1: source A_new (below) -- the stencil of the pair
// whose update loop runs beside it; M = 2: the pair fused.  Included by
// jacobi.cu inside its anonymous namespace (TX, TY, Box3, ldOne, inArr3,
// inBox3, st2cs, ctaMax come from there).
//
// Why: the register-resident 2.5-D kernel (planes3) keeps one plane in flight
// per thread; its warps stall on those loads and on the per-plane barrier, and
// every thread spends instructions on addresses, bounds, shuffles and the edge
// columns.  Here one thread of the CTA issues one TMA box copy per plane -- the
// CTA's 64 columns of k with both edge columns and its TY rows of j with both
// halo rows, a (TY + 2) x 68 box starting at k = kb - 2 so that the copy's x
// coordinate stays 16-byte aligned -- into a ring of NS plane slots, several
// planes ahead of the one being computed.  The copy fills every element
// outside the array with 0, the value the loop's neighbours take there.  When a
// plane first becomes the (i+1) neighbour, the CTA converts it in place to q61
// values (each element once) and ORs the range flags; a plane step then reads
// its six neighbours from shared memory with 128-bit loads.
//
// Ring protocol: slot s holds the plane sequence numbers q = s, s + NS, ...
// (plane ib - 1 + q); its mbarrier completes one phase per plane, so the copy
// of q is waited for with parity (q / NS) & 1.  At step t (plane ib + t) the
// CTA waits for q = t + 2, converts it, and meets at one barrier.  After it
// every thread has finished step t - 1, the last reader of q = t - 1, so
// thread 0 issues the copy of q = t - 1 + NS into that slot.  Each thread's
// generic-proxy writes of a slot are followed by a proxy fence before that
// barrier.  Every wait is bounded: after 2 s of the global timer the kernel writes
// DVMHGB_ERR_TMA_TIMEOUT to the status word (when one is given), the CTA
// leaves its loop, and thread 0 waits (bounded again) for the copies still in
// flight before the CTA exits.
//
// Source A_new (M >= 1): B inside the loop box, A outside it -- what the
// stencil reads after the update loop A = B.  A plane outside the box is
// copied from A's tensor map; inside it from B's, and the elements of the box
// copy outside the box in j or k (halo rows and edge columns of the CTAs at
// the box's faces) are replaced by A's values before the conversion.  The
// stencil then reads neither A inside the box nor anything the update writes,
// so the update loop may run at the same time (M = 1).
//
// Fused (M = 2): the chunk's own cells also do the update loop,
// eps = Max(|B - A|, eps); A = B.  Each plane of the chunk
// also brings A's values of the CTA's own 64 x TY cells (a second box of A,
// same mbarrier); before converting its own pair, each thread takes
// |B - A_old| on the FP64 unit (idle beside the q61 sums) into its MAX and
// stores B into A.  Nothing reads A inside the box after that
// store except this CTA's own tile copy, which landed before it.  32 bytes a
// cell: A and B read, A and Out written.
//
// Stencil then update (M = 3): a time step's stencil loop followed by the next
// step's update loop, eps = Max(|B - A|, eps); A = B.  The new B of a cell is
// in a register when its A (the stencil's own source value) is in the slot, so
// the update needs no pass of its own: |B - A| on the FP64 unit, and B stored
// into A's second buffer, which becomes A when the pair ends (A itself is
// still read by the CTAs around).  24 bytes a cell: A read, B and A written.
//
// FP64-unit warps (W > 0): the q61 sums keep the integer pipes busy while the
// FP64 unit idles, so the last W warps of the CTA compute their cells on the
// FP64 unit -- five additions in the source order and RN(sum / 6) by
// sf::div6_fma, three FP64 operations where the integer pipe needs ~40.  They
// read the doubles, so the conversion writes the q61 values into a separate
// ring of QSLOTS planes and leaves the slots as copied (plane q's q61 slot is
// written in step q - 2 and read in steps q - 2 .. q; with four slots its next
// writer, plane q + 4 in step q + 2, comes after the barrier that ends step q).
// The share of cells on the FP64 unit, W / TY, is a launch variant the tuner
// chooses.
//
// Range: as in planes3 -- a plane whose neighbourhood holds a value outside +0
// and [2^-9, 1) is computed on the FP64 unit from global memory, bit for bit
// the same.
namespace tma {

constexpr int BX = 2 * TX + 4;  // k from kb - 2 to kb + 2 TX + 1
constexpr int BY = TY + 2;      // j from jb - 1 to jb + TY
constexpr int BOX_BYTES = BX * BY * 8;
constexpr int SLOT = (BOX_BYTES + 127) / 128 * 128;
constexpr int TILE_BYTES = 2 * TX * TY * 8;  // the CTA's own cells of a plane
constexpr int PAIRS = BX * BY / 2;           // element pairs of a box
constexpr uint64_t WAIT_LIMIT_NS = 2000000000ull;  // a wait gives up after 2 s
constexpr uint32_t SUSPEND_HINT_NS = 1000000;       // a waiting thread sleeps up to 1 ms per poll

constexpr int QSLOTS = 4;  // the q61 ring of the launches with FP64-unit warps
constexpr int slotBytes(bool fused) { return SLOT + (fused ? TILE_BYTES : 0); }
// dynamic shared memory of a launch with NS slots (and FP64-unit warps or
// not): the slots, the q61 ring, the mbarriers and 128 bytes of alignment slack
constexpr int smemBytes(bool fused, int ns, bool fp64warps = false) {
    return ns * slotBytes(fused) + (fp64warps ? QSLOTS * SLOT : 0) + ns * 8 + 128;
}

__device__ __forceinline__ uint32_t smemAddr(const void *p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void mbarInit(uint32_t bar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(bar), "r"(count) : "memory");
}

// one poll: the thread may sleep until the phase completes (or the hint's time passes)
__device__ __forceinline__ bool mbarTryWait(uint32_t bar, uint32_t parity) {
    uint32_t ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2, %3;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(ok)
        : "r"(bar), "r"(parity), "r"(SUSPEND_HINT_NS)
        : "memory");
    return ok != 0;
}

__device__ __forceinline__ uint64_t nowNs() {
    uint64_t t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

// wait for the phase of `parity` to complete, at most WAIT_LIMIT_NS of the
// global timer (the clock is read only once the first poll has failed)
__device__ __forceinline__ bool mbarWait(uint32_t bar, uint32_t parity) {
    if (mbarTryWait(bar, parity)) return true;
    const uint64_t t0 = nowNs();
    while (!mbarTryWait(bar, parity))
        if (nowNs() - t0 > WAIT_LIMIT_NS) return false;
    return true;
}

// thread 0's arrival on the slot's mbarrier, expecting `bytes` of copies
__device__ __forceinline__ void mbarExpect(uint32_t bar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar), "r"(bytes) : "memory");
}

// copy the box at (x, y, z) of the tensor map into dst, completing on the mbarrier
__device__ __forceinline__ void copyBox(const CUtensorMap *map, uint32_t dst, uint32_t bar, int x, int y, int z) {
    asm volatile(
        "cp.async.bulk.tensor.3d.shared::cluster.global.tile.mbarrier::complete_tx::bytes"
        " [%0], [%1, {%2, %3, %4}], [%5];" ::"r"(dst),
        "l"(reinterpret_cast<uint64_t>(map)), "r"(x), "r"(y), "r"(z), "r"(bar)
        : "memory");
}

}  // namespace tma

// mapS: the stencil's source box copies (M = 0: A, else B); mapA (M >= 1):
// A's box copies for planes outside the loop box; mapT (M = 2): A's own-cell
// tiles.  items (M = 2, 3): one MAX partial per CTA; Out2 (M = 3): A's second
// buffer; qe (M = 3): the first qe warps take the update's |B - A| on the
// integer pipe (exact q61 differences), the others on the FP64 unit.
template <int M, int NS, int MINB, int W>
__global__ void __launch_bounds__(TX *TY, MINB)
    kStencil3T(const __grid_constant__ CUtensorMap mapS, const __grid_constant__ CUtensorMap mapA,
               const __grid_constant__ CUtensorMap mapT, double *A, const double *__restrict__ B, double *Out, Box3 b,
               long p0, int ichunk, double *items, int *status, double *Out2, int qe) {
    static_assert(NS >= 4, "the ring holds planes i - 1, i, i + 1 and the slot being refilled");
    static_assert(M >= 0 && M <= 3 && M != 1, "modes 0, 2 and 3");
    constexpr bool S = M == 2, U = M == 2;  // source A_new; the update loop too
    constexpr bool E = M == 3;              // the next step's update loop after the stencil
    constexpr bool QR = W > 0 || E;         // the q61 values in their own ring, the slots keep the doubles
    constexpr int SB = tma::slotBytes(U);
    constexpr int NP = (tma::PAIRS + TX * TY - 1) / (TX * TY);  // box pairs a thread converts
    extern __shared__ unsigned char dyn[];
    unsigned char *base = dyn + ((128u - (tma::smemAddr(dyn) & 127u)) & 127u);
    uint64_t *qring = reinterpret_cast<uint64_t *>(base + NS * SB);  // QR
    uint64_t *bars = reinterpret_cast<uint64_t *>(base + NS * SB + (QR ? tma::QSLOTS * tma::SLOT : 0));
    // the timeout flag, one per parity of the step: a thread sets the flag of
    // its step before the step's barrier and every thread reads it after that
    // barrier, so a flag set in step t + 1 cannot reach a thread still reading
    // step t's
    __shared__ int stopAt[2];
    __shared__ double shr[TY];
    __shared__ sf::Q61Round rtab[sf::Q61_ROUND_ENTRIES];  // the q61 additions' rounding constants

    const int lane = threadIdx.x, ty = threadIdx.y, tid = ty * TX + lane;
    const long kb = 2 * (p0 + (long)blockIdx.x * TX);
    const long jb = b.lo1 + (long)blockIdx.y * TY;
    const long ib = b.lo0 + (long)blockIdx.z * ichunk;
    const long ie = ib + ichunk - 1 < b.hi0 ? ib + ichunk - 1 : b.hi0;
    const int nplanes = (int)(ie - ib + 1), nseq = nplanes + 2;  // planes ib - 1 .. ie + 1
    const long k = kb + 2 * lane, j = jb + ty;
    const bool kI0 = k >= b.lo2 && k <= b.hi2, kI1 = k + 1 >= b.lo2 && k + 1 <= b.hi2, jI = j <= b.hi1;

    auto slotOf = [&](int q) { return reinterpret_cast<uint64_t *>(base + (size_t)(q % NS) * SB); };
    // where plane q's q61 values go: in place, or (W > 0) the q61 ring, the slot keeping the doubles
    auto qslotOf = [&](int q) { return QR ? qring + (size_t)(q % tma::QSLOTS) * (tma::SLOT / 8) : slotOf(q); };
    auto barOf = [&](int q) { return tma::smemAddr(bars + q % NS); };
    auto parityOf = [](int q) { return (uint32_t)((q / NS) & 1); };
    auto planeIn = [&](long z) { return z >= b.lo0 && z <= b.hi0; };
    int issued = 0;  // thread 0: planes issued (q = 0 .. issued - 1)
    auto issue = [&](int q) {
        const long z = ib - 1 + q;
        const uint32_t bar = barOf(q), dst = tma::smemAddr(slotOf(q));
        const bool tile = U && q >= 1 && q <= nplanes;
        tma::mbarExpect(bar, tma::BOX_BYTES + (tile ? tma::TILE_BYTES : 0));
        tma::copyBox(S && !planeIn(z) ? &mapA : &mapS, dst, bar, (int)(kb - 2), (int)(jb - 1), (int)z);
        if (tile) tma::copyBox(&mapT, dst + tma::SLOT, bar, (int)kb, (int)jb, (int)z);
        issued = q + 1;
    };

    // the thread's pairs of a box -- u = 0: its own pair (row ty + 1, pair
    // lane + 1 of the row: the cells whose stencil it computes), u = 1: one of
    // the 84 halo pairs (rows 0 and TY + 1, then the first and last pair of
    // rows 1..TY) for the first 84 threads -- and, source A_new, what they
    // are: bit 0 a pair of the box, bits 1, 2 element 0, 1 outside the loop
    // box but inside the array (A's value replaces B's in the planes inside
    // the box); goff: the pair's offset in a plane
    static_assert(NP == 2 && tma::PAIRS - TX * TY == 2 * (tma::BX / 2) + 2 * TY, "own pairs, then halo pairs");
    int pr[NP];
    unsigned fl[NP];
    long goff[NP];
#pragma unroll
    for (int u = 0; u < NP; u++) {
        constexpr int RP = tma::BX / 2;  // pairs of a row
        int r, cp;
        if (u == 0) {
            r = ty + 1, cp = lane + 1;
        } else if (tid < RP) {
            r = 0, cp = tid;
        } else if (tid < 2 * RP) {
            r = TY + 1, cp = tid - RP;
        } else {
            r = 1 + (tid - 2 * RP) / 2, cp = (tid - 2 * RP) & 1 ? RP - 1 : 0;
        }
        const int p = u == 0 || tid < tma::PAIRS - TX * TY ? r * RP + cp : tma::PAIRS;
        const long jj = jb - 1 + r, kk = kb - 2 + 2 * cp;
        const bool inJ = jj >= b.lo1 && jj <= b.hi1, aJ = jj >= 0 && jj < b.e1;
        const bool ik0 = kk >= b.lo2 && kk <= b.hi2, ik1 = kk + 1 >= b.lo2 && kk + 1 <= b.hi2;
        const bool ak0 = kk >= 0 && kk < b.e2, ak1 = kk + 1 >= 0 && kk + 1 < b.e2;
        pr[u] = p;
        goff[u] = jj * b.s1 + kk;
        fl[u] = p < tma::PAIRS ? 1u : 0u;
        if (S && p < tma::PAIRS) fl[u] |= (aJ && ak0 && !(inJ && ik0) ? 2u : 0u) | (aJ && ak1 && !(inJ && ik1) ? 4u : 0u);
    }
    // fused: the update loop on the thread's own pair -- the cells whose stencil it computes
    const bool ownUpd = U && jI && (kI0 || kI1);
    const int tilePair = ty * TX + lane;
    double *ownA = A + j * b.s1 + k;
    uint64_t mb = 0;    // the update's eps: Max(|B - A|) as a bit pattern (FP64-unit differences)
    uint64_t qmax = 0;  // M = 3: the largest exact q61 difference (warps below qe)
    bool seen = false, qdone = false;

    // wait for plane q (in step q - 2), [fused: do the update of the own pair,
    // replace the elements outside the box], convert it to q61 (in place, or
    // into the q61 ring); the thread's range flag
    auto arrive = [&](int q) -> bool {
        if (!tma::mbarWait(barOf(q), parityOf(q))) {
            if (status) atomicExch(status, DVMHGB_ERR_TMA_TIMEOUT);
            stopAt[q & 1] = 1;  // (q - 2) & 1
        }
        const long z = ib - 1 + q;
        const bool zIn = S && planeIn(z), upd = U && q >= 1 && q <= nplanes;
        bool bad = false;
        ulonglong2 *s2 = reinterpret_cast<ulonglong2 *>(slotOf(q)), *d2 = reinterpret_cast<ulonglong2 *>(qslotOf(q));
        if (U && upd && ownUpd) {  // before this thread's conversion of its own pair overwrites B's doubles
            const ulonglong2 br = s2[pr[0]];
            const ulonglong2 ar = reinterpret_cast<const ulonglong2 *>(slotOf(q) + tma::SLOT / 8)[tilePair];
            const double x = __longlong_as_double((long long)br.x), y = __longlong_as_double((long long)br.y);
            const double ax = __longlong_as_double((long long)ar.x), ay = __longlong_as_double((long long)ar.y);
            // |B - A| on the FP64 unit (idle beside the q61 sums), MAX on the bit patterns
            if (kI0) mb = sf::absmax_bits(sf::nadd(x, -ax), mb);
            if (kI1) mb = sf::absmax_bits(sf::nadd(y, -ay), mb);
            seen = true;
            double *pa = ownA + z * b.s0;
            if (kI0 && kI1) st2cs(pa, make_double2(x, y));
            else if (kI0) pa[0] = x;
            else pa[1] = y;
        }
#pragma unroll
        for (int u = 0; u < NP; u++) {
            if (!(fl[u] & 1u)) continue;
            const ulonglong2 raw = s2[pr[u]];
            double x = __longlong_as_double((long long)raw.x), y = __longlong_as_double((long long)raw.y);
            if (S && zIn && (fl[u] & 6u)) {  // rare: a CTA at a face of the box
                const double *pa = A + z * b.s0 + goff[u];
                if (fl[u] & 2u) x = pa[0];
                if (fl[u] & 4u) y = pa[1];
                if (QR) s2[pr[u]] = make_ulonglong2(sf::bits(x), sf::bits(y));  // the slot keeps the source doubles
            }
            bad |= !sf::q61_ok(x) || !sf::q61_ok(y);
            d2[pr[u]] = make_ulonglong2(sf::q61(x), sf::q61(y));
        }
        // these generic-proxy writes come before the slot's next TMA copy
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
        return bad;
    };
    // the stencil's source at (i, jj, kk) from global memory: A, or fused A_new
    auto src = [&](long i, long jj, long kk) -> double {
        if (!S) return ldOne(A, b, i, jj, kk);
        if (!inArr3(b, i, jj, kk)) return 0.0;
        const long off = i * b.s0 + jj * b.s1 + kk;
        return inBox3(b, i, jj, kk) ? B[off] : A[off];
    };
    auto nativeCell = [&](long i, long kk) -> double {
        const double a = src(i - 1, j, kk), bb = src(i, j - 1, kk), c = src(i, j, kk - 1);
        const double d = src(i, j, kk + 1), e = src(i, j + 1, kk), f = src(i + 1, j, kk);
        return sf::div3p2(sf::nadd(sf::nadd(sf::nadd(sf::nadd(sf::nadd(a, bb), c), d), e), f), 1);
    };

    if (tid < sf::Q61_ROUND_ENTRIES) rtab[tid] = sf::q61_round_entry(tid);
    // 1 and 2 as values the compiler cannot fold (blockDim.x == TX == 32)
    const uint32_t one = blockDim.x >> 5, two = one + one;
    auto add = [&](uint64_t x, uint64_t y) { return sf::q61_add_t(x, y, rtab, one, two); };
    if (tid == 0) {
        stopAt[0] = stopAt[1] = 0;
        for (int s = 0; s < NS; s++) tma::mbarInit(tma::smemAddr(bars + s), 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
        for (int q = 0; q < NS && q < nseq; q++) issue(q);
    }
    __syncthreads();
    // planes ib - 1 and ib; the flags of planes i - 1, i, i + 1 in bits 2, 1, 0 (the first two merged)
    bool bad = arrive(0);
    bad = arrive(1) || bad;
    unsigned flags = __syncthreads_or(bad) ? 3u : 0u;
    bool stop = stopAt[1] != 0;  // (a timeout of q = 0 is seen in step 0)
    const int r0 = (ty + 1) * tma::BX + 2 + 2 * lane;  // the thread's pair in a slot
    double *out = Out + ib * b.s0 + j * b.s1 + k;
    double *const outBase = out, *const out2 = E ? Out2 + ib * b.s0 + j * b.s1 + k : nullptr;
    for (int t = 0; t < nplanes && !stop; t++) {
        const long i = ib + t;
        flags = ((flags << 1) | (__syncthreads_or(arrive(t + 2)) ? 1u : 0u)) & 7u;
        stop = stopAt[t & 1] != 0;
        if (stop) break;
        if (tid == 0 && t >= 1 && t - 1 + NS < nseq) {
            asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
            issue(t - 1 + NS);
        }
        double v0, v1;
        if (flags == 0 && W > 0 && ty >= TY - W) {  // an FP64-unit warp: the doubles of the slots
            const double *pm = reinterpret_cast<const double *>(slotOf(t)) + r0;
            const double *pc = reinterpret_cast<const double *>(slotOf(t + 1)) + r0;
            const double *pp = reinterpret_cast<const double *>(slotOf(t + 2)) + r0;
            const double2 im = *reinterpret_cast<const double2 *>(pm);
            const double2 up = *reinterpret_cast<const double2 *>(pc - tma::BX);
            const double2 own = *reinterpret_cast<const double2 *>(pc);
            const double2 dn = *reinterpret_cast<const double2 *>(pc + tma::BX);
            const double2 ip = *reinterpret_cast<const double2 *>(pp);
            const double left = pc[-1], right = pc[2];
            v0 = sf::div6_fma(((((im.x + up.x) + left) + own.y) + dn.x) + ip.x);
            v1 = sf::div6_fma(((((im.y + up.y) + own.x) + right) + dn.y) + ip.y);
        } else if (flags == 0) {
            const uint64_t *pm = qslotOf(t) + r0, *pc = qslotOf(t + 1) + r0, *pp = qslotOf(t + 2) + r0;
            const ulonglong2 im = *reinterpret_cast<const ulonglong2 *>(pm);
            const ulonglong2 up = *reinterpret_cast<const ulonglong2 *>(pc - tma::BX);
            const ulonglong2 own = *reinterpret_cast<const ulonglong2 *>(pc);
            const ulonglong2 dn = *reinterpret_cast<const ulonglong2 *>(pc + tma::BX);
            const ulonglong2 ip = *reinterpret_cast<const ulonglong2 *>(pp);
            const uint64_t left = pc[-1], right = pc[2];
            // (((((A[i-1] + A[j-1]) + A[k-1]) + A[k+1]) + A[j+1]) + A[i+1]) / 6, left to right
            v0 = sf::q61_div6(add(add(add(add(add(im.x, up.x), left), own.y), dn.x), ip.x));
            v1 = sf::q61_div6(add(add(add(add(add(im.y, up.y), own.x), right), dn.y), ip.y));
            if (E && jI && ty < qe) {
                // the next update's |B - A| as an exact difference of q61 values (A's are the plane's own, B's
                // converted; RN of the largest, once, at the end); a B below the range goes to the FP64 unit
                const bool ok0 = sf::q61_ok(v0), ok1 = sf::q61_ok(v1);
                const uint64_t b0 = sf::q61(v0), b1 = sf::q61(v1);
                const uint64_t d0 = b0 > own.x ? b0 - own.x : own.x - b0, d1 = b1 > own.y ? b1 - own.y : own.y - b1;
                if (kI0 && ok0 && d0 > qmax) qmax = d0;
                if (kI1 && ok1 && d1 > qmax) qmax = d1;
                qdone = ok0 && ok1;
            }
        } else {  // rare: a value outside the fixed-point range near this plane
            v0 = (jI && kI0) ? nativeCell(i, k) : 0.0;
            v1 = (jI && kI1) ? nativeCell(i, k + 1) : 0.0;
        }
        if (jI) {
            if (kI0 && kI1) st2cs(out, make_double2(v0, v1));
            else if (kI0) out[0] = v0;
            else if (kI1) out[1] = v1;
        }
        if (E && jI && !qdone) {  // the next update: eps = Max(|B - A|, eps) on the FP64 unit, A's doubles of the slot
            const double2 a = *reinterpret_cast<const double2 *>(reinterpret_cast<const double *>(slotOf(t + 1)) + r0);
            if (kI0) mb = sf::absmax_bits(sf::nadd(v0, -a.x), mb);
            if (kI1) mb = sf::absmax_bits(sf::nadd(v1, -a.y), mb);
        }
        qdone = false;
        if (E && jI) {  // A = B into A's second buffer
            seen = seen || kI0 || kI1;
            double *o2 = out2 + (out - outBase);
            if (kI0 && kI1) st2cs(o2, make_double2(v0, v1));
            else if (kI0) o2[0] = v0;
            else if (kI1) o2[1] = v1;
        }
        out += b.s0;
    }
    if (U || E) {
        // RN(max |b - a|) of the q61 differences (RN is monotone: the largest, rounded once), with the FP64 part
        const double qd = __ull2double_rn(qmax) * 0x1p-61, f = sf::from(mb);
        double m = seen ? (qd > f ? qd : f) : -__builtin_huge_val();
        m = ctaMax(m, shr);
        if (tid == 0) items[blockIdx.x + gridDim.x * ((long)blockIdx.y + (long)gridDim.y * blockIdx.z)] = m;
    }
    // after a timeout, the copies still in flight land before the CTA's shared memory is released
    if (stop && tid == 0)
        for (int q = issued - NS < 0 ? 0 : issued - NS; q < issued; q++) (void)tma::mbarWait(barOf(q), parityOf(q));
}

// A tensor map of a 3-D array of doubles with extents ext (outermost first)
// and strides st (elements; the innermost is 1), boxes of bx x by x 1.
// Encoded through the driver entry point that the CUDA runtime hands out, so
// the library does not link libcuda.  False when the layout cannot be mapped.
bool encodeMap3(CUtensorMap *map, const double *X, const long ext[3], const long st[3], int bx, int by) {
    using Encode = CUresult (*)(CUtensorMap *, CUtensorMapDataType, cuuint32_t, void *, const cuuint64_t *,
                                const cuuint64_t *, const cuuint32_t *, const cuuint32_t *, CUtensorMapInterleave,
                                CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);
    static std::atomic<Encode> encode{nullptr};
    Encode fn = encode.load();
    if (!fn) {
        void *p = nullptr;
        cudaDriverEntryPointQueryResult q = cudaDriverEntryPointSymbolNotFound;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) !=
                cudaSuccess ||
            q != cudaDriverEntryPointSuccess || !p)
            return false;
        fn = (Encode)p;
        encode.store(fn);
    }
    if (ext[0] < 1 || ext[1] < 1 || ext[2] < 1 || ext[0] > INT32_MAX || ext[1] > INT32_MAX || ext[2] > INT32_MAX)
        return false;
    const cuuint64_t dims[3] = {(cuuint64_t)ext[2], (cuuint64_t)ext[1], (cuuint64_t)ext[0]};
    const cuuint64_t strides[2] = {(cuuint64_t)st[1] * 8, (cuuint64_t)st[0] * 8};
    const cuuint32_t box[3] = {(cuuint32_t)bx, (cuuint32_t)by, 1};
    const cuuint32_t estr[3] = {1, 1, 1};
    return fn(map, CU_TENSOR_MAP_DATA_TYPE_FLOAT64, 3, (void *)X, dims, strides, box, estr,
              CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
              CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}
