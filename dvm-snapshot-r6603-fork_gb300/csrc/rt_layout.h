// Transformed device layouts of distributed arrays (the reference's
// autotransform: rts/dvmh/dvmh_rts.cpp:1404-1479, rts/dvmh/dvmh_buffer.cpp:90-147).
//
// A device array is either natural (row-major, the innermost row padded, the
// layout every hand-written kernel of this library expects) or transformed:
//   - permuted: the axes stored in another order, dense;
//   - diagonalised: in addition the last two stored axes (y, then x) form a
//     dense Rx x Ry plane numbered along anti-diagonals x + y (or, in the
//     "slash" orientation, along x - y), so that the cells an ACROSS loop
//     with two dependences updates together are adjacent in memory.
// Generated handlers see the layout through dvmh_fill_header_C: per-axis
// coefficients (zero for the two diagonal axes), the return value 0 / 1 / 2
// and, for 2, the plane's axes, extents and orientation.  The numbering is a
// format the generated kernels compute themselves, so it is kept exactly.
#pragma once

#include "../../include/dvmh_gb_layout.h"

#ifdef __CUDACC__
#define GB_HD __host__ __device__ __forceinline__
#else
#define GB_HD inline
#endif

namespace dvmhgb {

constexpr int LAYOUT_MAXR = 7;

// Where element (i_1 .. i_rank) of an array lives in one device buffer:
// sum coef[a] * i_a, plus dvmhgb_diag_index(i_x, i_y) when diagonalised.
struct LayoutDesc {
    int rank;
    long ext[LAYOUT_MAXR];
    long coef[LAYOUT_MAXR];
    int diag;          // 0: none; else the plane of axes xAxis / yAxis (0-based)
    int xAxis, yAxis;
    int slash;
    long diagUnit;     // units per diagonal position (1; the element size when copying bytes)
};

GB_HD long layoutOffset(const LayoutDesc &L, const long idx[]) {
    long off = 0;
    for (int a = 0; a < L.rank; a++) off += L.coef[a] * idx[a];
    if (L.diag) off += L.diagUnit * dvmhgb_diag_index(idx[L.xAxis], idx[L.yAxis], L.ext[L.xAxis], L.ext[L.yAxis], L.slash);
    return off;
}

}  // namespace dvmhgb
