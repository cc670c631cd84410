// frame.h -- grid placement and light frame, FP64, identical on host and device.
//
// Every operation is written through helpers that round on their own (no FMA contraction on the device;
// the host build uses -ffp-contract=off), so the host- and device-computed frames agree bit for bit.
#pragma once

#include <cmath>
#include <cstdint>

#include "../../include/f184gi.h"

#if defined(__CUDACC__)
#define F184_HD __host__ __device__ __forceinline__
#else
#define F184_HD inline
#endif

namespace f184 {

F184_HD double hmul(double a, double b) {
#ifdef __CUDA_ARCH__
    return __dmul_rn(a, b);
#else
    return a * b;
#endif
}
F184_HD double hadd(double a, double b) {
#ifdef __CUDA_ARCH__
    return __dadd_rn(a, b);
#else
    return a + b;
#endif
}
F184_HD double hsub(double a, double b) {
#ifdef __CUDA_ARCH__
    return __dsub_rn(a, b);
#else
    return a - b;
#endif
}
F184_HD double hdiv(double a, double b) {
#ifdef __CUDA_ARCH__
    return __ddiv_rn(a, b);
#else
    return a / b;
#endif
}
F184_HD double hsqrt(double a) {
#ifdef __CUDA_ARCH__
    return __dsqrt_rn(a);
#else
    return std::sqrt(a);
#endif
}
F184_HD double habs(double a) { return a < 0.0 ? -a : a; }

// Grid: cubic, `dim` voxels per axis, 1.5 voxels of margin around the bounds' largest extent, so bounding
// faces pass through voxel centres rather than voxel boundaries.
// Light: orthographic frame around the grid's circumscribed sphere, clip z in [0, 1] along the direction
// of travel; the shadow compare is biased by two voxels.
F184_HD void frame_from_bounds(const float mn[3], const float mx[3], uint32_t dim, const float light_dir[3],
                               f184gi_grid_frame* out) {
    double c[3], ext = 0.0;
    for (int a = 0; a < 3; ++a) {
        double s = hadd(double(mn[a]), double(mx[a]));
        c[a] = hmul(s, 0.5);
        double e = hsub(double(mx[a]), double(mn[a]));
        if (e > ext) ext = e;
    }
    if (!(ext > 0.0)) ext = 1.0;
    double vs = hdiv(ext, double(dim - 3));
    double half = hmul(vs, hmul(double(dim), 0.5));
    for (int a = 0; a < 3; ++a) out->origin[a] = hsub(c[a], half);
    out->voxel_size = vs;
    out->inv_voxel_fixed = hdiv(256.0, vs);
    double L[3] = {double(light_dir[0]), double(light_dir[1]), double(light_dir[2])};
    double l2 = hmul(L[0], L[0]);
    l2 = hadd(l2, hmul(L[1], L[1]));
    l2 = hadd(l2, hmul(L[2], L[2]));
    double len = hsqrt(l2);
    double w[3] = {hdiv(L[0], len), hdiv(L[1], len), hdiv(L[2], len)};
    double h[3] = {0.0, 0.0, 0.0};
    double ax = habs(w[0]), ay = habs(w[1]), az = habs(w[2]);
    if (ax <= ay && ax <= az)
        h[0] = 1.0;
    else if (ay <= az)
        h[1] = 1.0;
    else
        h[2] = 1.0;
    double u[3] = {hsub(hmul(h[1], w[2]), hmul(h[2], w[1])), hsub(hmul(h[2], w[0]), hmul(h[0], w[2])),
                   hsub(hmul(h[0], w[1]), hmul(h[1], w[0]))};
    double ul = hmul(u[0], u[0]);
    ul = hadd(ul, hmul(u[1], u[1]));
    ul = hadd(ul, hmul(u[2], u[2]));
    ul = hsqrt(ul);
    for (int a = 0; a < 3; ++a) u[a] = hdiv(u[a], ul);
    double v[3] = {hsub(hmul(w[1], u[2]), hmul(w[2], u[1])), hsub(hmul(w[2], u[0]), hmul(w[0], u[2])),
                   hsub(hmul(w[0], u[1]), hmul(w[1], u[0]))};
    double R = hmul(half, hsqrt(3.0));
    double R2 = hmul(R, 2.0);
    double* M = out->light_clip;
    for (int a = 0; a < 3; ++a) {
        M[0 + a] = hdiv(u[a], R);
        M[4 + a] = hdiv(v[a], R);
        M[8 + a] = hdiv(w[a], R2);
        M[12 + a] = 0.0;
    }
    double du = hadd(hadd(hmul(u[0], c[0]), hmul(u[1], c[1])), hmul(u[2], c[2]));
    double dv = hadd(hadd(hmul(v[0], c[0]), hmul(v[1], c[1])), hmul(v[2], c[2]));
    double dw = hadd(hadd(hmul(w[0], c[0]), hmul(w[1], c[1])), hmul(w[2], c[2]));
    M[3] = -hdiv(du, R);
    M[7] = -hdiv(dv, R);
    M[11] = hsub(0.5, hdiv(dw, R2));
    M[15] = 1.0;
    out->shadow_bias = hdiv(vs, R);
    for (int a = 0; a < 3; ++a) out->light_dir[a] = w[a];
    // voxel centre (i, j, k) -> light clip row r = base_r + i s_r0 + j s_r1 + k s_r2 (rounded to FP32)
    double hv = hmul(vs, 0.5);
    double c0[3] = {hadd(out->origin[0], hv), hadd(out->origin[1], hv), hadd(out->origin[2], hv)};
    for (int r = 0; r < 3; ++r) {
        const double* Mr = M + 4 * r;
        double base = hadd(hadd(hadd(hmul(Mr[0], c0[0]), hmul(Mr[1], c0[1])), hmul(Mr[2], c0[2])), Mr[3]);
        out->light_vox[4 * r] = float(base);
        for (int a = 0; a < 3; ++a) out->light_vox[4 * r + 1 + a] = float(hmul(Mr[a], vs));
    }
    out->shadow_bias_f = float(out->shadow_bias);
    out->pad_f[0] = out->pad_f[1] = out->pad_f[2] = 0.0f;
}

}  // namespace f184
