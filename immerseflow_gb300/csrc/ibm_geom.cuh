// ibm_geom.cuh -- body predicate and grid search shared by the immersed-
// boundary set-up (kernels_ibm.cu) and the per-step geometry of moving bodies
// (kernels_move.cu).  Both files are compiled with -fmad=false and the
// predicate spells out its roundings, so iBlank matches the CPU restatement
// bit for bit.
#pragma once
#include "ifx_dev.h"

namespace ifx {

// Inside the ellipse of centre (cx, cy), axis direction (cs, sn), 1/a^2 and
// 1/b^2: (xr/a)^2 + (yr/b)^2 < 1 in the body frame.
__device__ __forceinline__ int inside_ellipse(double x, double y, double cx, double cy, double cs, double sn,
                                              double ia2, double ib2) {
    const double ddx = __dsub_rn(x, cx);
    const double ddy = __dsub_rn(y, cy);
    const double xr = __dadd_rn(__dmul_rn(ddx, cs), __dmul_rn(ddy, sn));
    const double yr = __dsub_rn(__dmul_rn(ddy, cs), __dmul_rn(ddx, sn));
    const double f = __dadd_rn(__dmul_rn(__dmul_rn(xr, xr), ia2), __dmul_rn(__dmul_rn(yr, yr), ib2));
    return f < 1.0 ? 1 : 0;
}
__device__ __forceinline__ int inside_body(const InstDev& in, double x, double y) {
    return inside_ellipse(x, y, in.bcx, in.bcy, in.bcs, in.bsn, in.bia2, in.bib2);
}

// last index in [1, n-2] with c[idx] <= x (0 if none), as std::upper_bound - 1
__device__ __forceinline__ int ub_index(const double* c, int n, double x) {
    int lo = 1, hi = n - 1;
    while (lo < hi) {
        const int mid = (lo + hi) >> 1;
        if (c[mid] <= x) lo = mid + 1;
        else hi = mid;
    }
    return lo - 1;
}

}  // namespace ifx
