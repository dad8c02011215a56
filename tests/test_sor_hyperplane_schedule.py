"""The hyperplane-tile schedule of the SOR wavefront (variants 4 and 5), emulated on the CPU.

The GPU tests check the kernels bit for bit; this test checks the schedule they implement under arbitrary
interleavings, which one GPU run cannot enumerate.  Tiles of ti x tj rows by G hyperplanes i + j + k are listed
plane by plane; up to W tiles are held at once, and at every event a random one of the allowed actions runs: hand
out the next tile (it stages its own rows and +i / +j faces, old values, into its window box), run a held tile whose
five predecessors have released (it stages the -i / -j faces and its rows' position 0, loads the differences its
rows' previous windows carried, takes G skewed steps, stores the cells its successors read and its own carried
differences, and releases), store a released tile's other cells, or close a released tile's residual parts.  Cells a
tile stores after its release are poisoned (NaN) until then.  The array must equal the sequential sweep's and every
residual item the canonical tree's (8-wide parts of k, -0.0 outside the loop box), bit for bit."""
import random

import numpy as np
import pytest


def tree(leaves):
    while len(leaves) > 1:
        leaves = [leaves[q] + leaves[q + 1] for q in range(0, len(leaves), 2)]
    return leaves[0]


def sequential(A, lo, hi, w, G):
    c1, c2 = 1.0 - w, w / 6.0
    sq = {}
    for i in range(lo[0], hi[0] + 1):
        for j in range(lo[1], hi[1] + 1):
            for k in range(lo[2], hi[2] + 1):
                old = A[i, j, k]
                s = ((((A[i - 1, j, k] + A[i + 1, j, k]) + A[i, j - 1, k]) + A[i, j + 1, k]) + A[i, j, k - 1]) + \
                    A[i, j, k + 1]
                nv = c1 * old + c2 * s
                A[i, j, k] = nv
                d = nv - old
                sq[(i, j, k)] = d * d
    parts = 64 // G
    kc0, nparts = parts * (lo[2] // 64), parts * (hi[2] // 64 - lo[2] // 64 + 1)
    items = [tree([sq[(i, j, k)] if lo[2] <= k <= hi[2] else -0.0 for k in range((kc0 + c) * G, (kc0 + c + 1) * G)])
             for i in range(lo[0], hi[0] + 1) for j in range(lo[1], hi[1] + 1) for c in range(nparts)]
    return np.array(items)


def hyperplane(A, lo, hi, w, G, ti, tj, rng, W):
    c1, c2 = 1.0 - w, w / 6.0
    e = A.shape
    na, nb, nk = (hi[0] - lo[0] + ti) // ti, (hi[1] - lo[1] + tj) // tj, hi[2] - lo[2] + 1
    cmin = lambda a, b: (ti * a + tj * b) // G
    cmax = lambda a, b: (ti * a + tj * b + ti + tj - 2 + nk - 1) // G
    exists = lambda a, b, c: 0 <= a < na and 0 <= b < nb and cmin(a, b) <= c <= cmax(a, b)
    tiles = sorted([(a, b, c) for a in range(na) for b in range(nb) for c in range(cmin(a, b), cmax(a, b) + 1)],
                   key=lambda t: (t[0] + t[1] + t[2], t[2], t[0]))
    parts = 64 // G
    kc0, nparts = parts * (lo[2] // 64), parts * (hi[2] // 64 - lo[2] // 64 + 1)
    nj = hi[1] - lo[1] + 1
    items = np.full((hi[0] - lo[0] + 1) * nj * nparts, np.nan)
    carry, released = {}, set()
    ld = lambda i, j, k: A[i, j, k] if (0 <= i < e[0] and 0 <= j < e[1] and 0 <= k < e[2]) else 0.0
    SI, SJ, SK = ti + 2, tj + 2, G + 2

    def window(box, a, b, c, qi, qj, ps):
        ri, rj = ti * a - 1 + qi, tj * b - 1 + qj
        for p in ps:  # window position p: hyperplane G c - 1 + p of row (ri, rj)
            box[qi, qj, p] = ld(lo[0] + ri, lo[1] + rj, lo[2] + G * c - ri - rj - 1 + p)

    def hand_out(t):
        a, b, c = t
        box = np.full((SI, SJ, SK), np.nan)
        for qi in range(1, SI):
            for qj in range(1, SJ):
                window(box, a, b, c, qi, qj, range(1, G + 2))
        return {"t": t, "box": box}

    def ready(h):
        a, b, c = h["t"]
        preds = [(a - 1, b, c), (a - 1, b, c - 1), (a, b - 1, c), (a, b - 1, c - 1), (a, b, c - 1)]
        return all(p in released for p in preds if exists(*p))

    def run(h):
        a, b, c = h["t"]
        box = h["box"]
        for qj in range(1, tj + 1):
            window(box, a, b, c, 0, qj, range(G))
        for qi in range(1, ti + 1):
            window(box, a, b, c, qi, 0, range(G))
            for qj in range(1, tj + 1):
                window(box, a, b, c, qi, qj, [0])
        rows = {}
        for li in range(ti):
            for lj in range(tj):
                ri, rj = ti * a + li, tj * b + lj
                i, j, k0 = lo[0] + ri, lo[1] + rj, lo[2] + G * c - ri - rj
                if i <= hi[0] and j <= hi[1] and k0 <= hi[2]:
                    m = (k0 // G) * G
                    key = ri * nj + rj
                    cin = carry[key] if c != cmin(a, b) else [0.0] * (k0 - m)
                    rows[(li, lj)] = {"key": key, "k0": k0, "m": m, "cin": list(cin), "dv": [0.0] * G}
        for t in range(G):
            new = {}
            for li in range(ti):
                for lj in range(tj):
                    ri, rj = ti * a + li, tj * b + lj
                    rk = G * c + t - ri - rj
                    if lo[0] + ri <= hi[0] and lo[1] + rj <= hi[1] and 0 <= rk < nk:
                        x = box[li + 1, lj + 1]
                        s = ((((box[li, lj + 1, t] + box[li + 2, lj + 1, t + 2]) + box[li + 1, lj, t]) +
                              box[li + 1, lj + 2, t + 2]) + x[t]) + x[t + 2]
                        assert not np.isnan(s) and not np.isnan(x[t + 1])
                        nv = c1 * x[t + 1] + c2 * s
                        new[(li, lj)] = nv
                        rows[(li, lj)]["dv"][t] = nv - x[t + 1]
            for (li, lj), nv in new.items():  # the lanes' writes after the step (warp barrier)
                box[li + 1, lj + 1, t + 1] = nv
        late = []
        for li in range(ti):
            for lj in range(tj):
                ri, rj = ti * a + li, tj * b + lj
                for p in range(1, G + 1):
                    rk = G * c - ri - rj + p - 1
                    if lo[0] + ri <= hi[0] and lo[1] + rj <= hi[1] and 0 <= rk < nk:
                        cell = (lo[0] + ri, lo[1] + rj, lo[2] + rk)
                        if li == ti - 1 or lj == tj - 1 or p == G:
                            A[cell] = box[li + 1, lj + 1, p]
                        else:
                            A[cell] = np.nan
                            late.append((cell, box[li + 1, lj + 1, p]))
        for r in rows.values():
            dl = r["k0"] - r["m"]
            carry[r["key"]] = r["dv"][G - dl:]
        released.add(h["t"])
        h["late"], h["rows"] = late, rows

    def store_late(h):
        for cell, v in h.pop("late"):
            A[cell] = v

    def residual(h):
        a, b, c = h["t"]
        for r in h.pop("rows").values():
            k0, m = r["k0"], r["m"]
            d = r["cin"] + r["dv"]
            leaves = lambda kf, dd: [dd[p] * dd[p] if lo[2] <= kf + p <= hi[2] else -0.0 for p in range(G)]
            P, base = m // G - kc0, r["key"] * nparts
            if c == cmin(a, b):
                for q in range(min(P, nparts)):
                    items[base + q] = -0.0
            if 0 <= P < nparts:
                items[base + P] = tree(leaves(m, d[:G]))
            if k0 + G - 1 >= hi[2]:
                if 0 <= P + 1 < nparts:
                    items[base + P + 1] = tree(leaves(m + G, d[G:] + [np.nan] * (2 * G - len(d))))
                for q in range(max(P + 2, 0), nparts):
                    items[base + q] = -0.0

    nxt, held, done_run = 0, [], []
    while nxt < len(tiles) or held or done_run:
        acts = []
        if nxt < len(tiles) and len(held) + len(done_run) < W:
            acts.append(("take", None))
        acts += [("run", h) for h in held if ready(h)]
        acts += [("late", h) for h in done_run if "late" in h]
        acts += [("res", h) for h in done_run if "rows" in h]
        assert acts, "no action is allowed: the schedule deadlocked"
        kind, h = rng.choice(acts)
        if kind == "take":
            held.append(hand_out(tiles[nxt]))
            nxt += 1
        elif kind == "run":
            held.remove(h)
            run(h)
            done_run.append(h)
        elif kind == "late":
            store_late(h)
        else:
            residual(h)
        done_run = [x for x in done_run if "late" in x or "rows" in x]
    return items


@pytest.mark.parametrize("ti,tj", [(4, 8), (16, 8)])
@pytest.mark.parametrize("shape,lo,hi", [((14, 19, 23), (1, 1, 1), (12, 17, 21)),
                                         ((9, 12, 90), (1, 2, 40), (7, 10, 88)),
                                         ((7, 11, 75), (3, 1, 62), (3, 9, 66))])
def test_schedule_matches_sequential(ti, tj, shape, lo, hi):
    G = 8
    rng = np.random.default_rng(sum(shape) + ti)
    A0 = rng.random(shape) * 2.0 - 0.5
    ref = A0.copy()
    want = sequential(ref, lo, hi, 1.5, G)
    for seed in range(4):  # four random interleavings, up to 9 or 40 tiles held at once
        got = A0.copy()
        items = hyperplane(got, lo, hi, 1.5, G, ti, tj, random.Random(seed * 7919 + ti * 1000 + shape[2]),
                           W=9 if seed % 2 == 0 else 40)
        assert np.array_equal(got.view(np.int64), ref.view(np.int64)), seed
        assert np.array_equal(items.view(np.int64), want.view(np.int64)), seed
