/* Diagonal numbering of a transformed device array, for CUDA handlers that
 * index arrays through dvmh_fill_header_C's description (the role cdvmh's
 * generated kernels give their diagonal-indexing helper).
 *
 * When dvmh_fill_header_C returns 2, element (i_1 .. i_rank) of the array is at
 *   base[ sum_a header[a] * i_a  +  dvmhgb_diag_index(i_x - x_first, i_y - y_first, Rx, Ry, slash) ]
 * with extendedParams = { x axis, x_first, Rx, y axis, y_first, Ry, slash }
 * (axes 1-based) and header[x] = header[y] = 0.  The numbering is the
 * reference's (rts/dvmh/util.cpp:1009-1055): cells ordered by diagonal
 * d = x + y (slash: x + (Ry - 1 - y)), and inside a diagonal along y when the
 * plane is taller than wide (or square, before the main anti-diagonal is
 * passed), along x otherwise. */
#ifndef DVMH_GB_LAYOUT_H
#define DVMH_GB_LAYOUT_H

#ifdef __CUDACC__
#define DVMHGB_HD __host__ __device__ __forceinline__
#else
#define DVMHGB_HD static inline
#endif

/* number of cells (x, y >= 0) with x + y < n */
DVMHGB_HD long dvmhgb_diag_tri(long n) { return n > 0 ? n * (n + 1) / 2 : 0; }

/* position of (x, y) in the diagonal numbering of an Rx x Ry plane; the cells
 * before diagonal d are counted by inclusion-exclusion over the plane's corners */
DVMHGB_HD long dvmhgb_diag_index(long x, long y, long Rx, long Ry, int slash) {
    long d, before, y0, x0;
    int alongY;
    if (slash) y = Ry - 1 - y;
    d = x + y;
    before = dvmhgb_diag_tri(d) - dvmhgb_diag_tri(d - Rx) - dvmhgb_diag_tri(d - Ry) + dvmhgb_diag_tri(d - Rx - Ry);
    alongY = Rx < Ry || (Rx == Ry && d < Rx);
    y0 = d - (Rx - 1) > 0 ? d - (Rx - 1) : 0; /* smallest y on diagonal d */
    x0 = d - (Ry - 1) > 0 ? d - (Ry - 1) : 0; /* smallest x on diagonal d */
    return before + (alongY ? y - y0 : x - x0);
}

#endif
