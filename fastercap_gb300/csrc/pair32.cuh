// FP32 pre-tests of the element-pair criteria (CAutoRefine::RefineCriteria,
// Solver/Autorefine.cpp:2928-3003) shared by the device link construction and
// the device mesh refinement.
//
// Most pairs are far from every decision boundary of the FP64 test (the rho
// = 2 switch between quadrature and point formula, the threshold e itself),
// so an FP32 evaluation with a bound on its distance to the FP64 value
// decides them; the rest (typically a few per cent) take the FP64 test.
// Bounds are deliberately loose (a factor 4 and more over a first-order
// rounding analysis): a loose bound only sends more pairs to FP64, it never
// changes a decision. Compiled with -fmad=false like the FP64 tests.
#ifndef FCG_PAIR32_CUH
#define FCG_PAIR32_CUH

#include "fc_potential.h"
#include "../host/model.hpp"

namespace fcg {
namespace pair32 {

constexpr float kU = 5.9604645e-8f;  // 2^-24, unit roundoff of float

// unit normal of a dielectric evaluation element (fcg_diel_normal in FP32);
// false when a super node's normal is within rounding of the 1e-12 cut-off
__device__ __forceinline__ bool diel_normal32(unsigned type, const float *n, float &x, float &y, float &z) {
    x = n[0];
    y = n[1];
    z = n[2];
    if (type & FCG_IS_SUPER_NODE) {
        float m = sqrtf(x * x + y * y + z * z);
        const float cut = (float)FCG_PANEL_EPS;
        if (!(fabsf(m - cut) > 1e-5f * cut)) return false;
        if (m < cut) {
            x = y = z = 0.0f;
        } else {
            x /= m;
            y /= m;
            z /= m;
        }
    }
    if ((type & FCG_OUTPERM_NORMAL_DIR) != FCG_OUTPERM_NORMAL_DIR) {
        x = -x;
        y = -y;
        z = -z;
    }
    return true;
}

// rule-2 average over source triangle v (centroid c) of 1/|r - p| or, for a
// field, (r - p).n / |r - p|^3, at r = c + d; `err` bounds the distance to
// fcg_potential_numerical / fcg_enfield_numerical (rule 2)
__device__ __forceinline__ bool quad2_32(float dx, float dy, float dz, const float *v, const float *c, bool efield, float nx,
                                         float ny, float nz, float &val, float &err) {
    float s1x = v[3] - v[0], s1y = v[4] - v[1], s1z = v[5] - v[2];
    float s2x = v[6] - v[3], s2y = v[7] - v[4], s2z = v[8] - v[5];
    float s3x = v[0] - v[6], s3y = v[1] - v[7], s3z = v[2] - v[8];
    float nX = s1y * s2z - s1z * s2y, nY = -s1x * s2z + s1z * s2x, nZ = s1x * s2y - s1y * s2x;
    float mn = sqrtf(nX * nX + nY * nY + nZ * nZ);
    float m1 = sqrtf(s1x * s1x + s1y * s1y + s1z * s1z);
    float m2 = sqrtf(s2x * s2x + s2y * s2y + s2z * s2z);
    float m3 = sqrtf(s3x * s3x + s3y * s3y + s3z * s3z);
    if (!(mn > 0.0f) || !(m1 > 0.0f)) return false;
    float skew = (m1 * m2) / mn;  // 1 / sin of the angle between sides 1 and 2
    float zx = nX / mn, zy = nY / mn, zz = nZ / mn;
    float xx = s1x / m1, xy = s1y / m1, xz = s1z / m1;
    float yx = xy * zz - xz * zy, yy = xz * zx - xx * zz, yz = xx * zy - xy * zx;
    float v01 = m1, v02 = -(s3x * xx + s3y * xy + s3z * xz), v12 = -(s3x * yx + s3y * yy + s3z * yz);
    float ratio = ((v02 - v01) * v12 - v12 * v02) / mn;  // jacobian / (2 area): +-1 up to rounding
    float ox = v[0] - c[0], oy = v[1] - c[1], oz = v[2] - c[2];
    float side = fmaxf(m1, fmaxf(m2, m3));
    float dd = sqrtf(dx * dx + dy * dy + dz * dz);
    // position error of a quadrature point relative to r, against the FP64 path
    float ep = 64.0f * kU * (dd + 3.0f * side * skew);
    const float a = 1.0f / 6.0f, b = 4.0f / 6.0f, w = 1.0f / 3.0f;
    float sum = 0.0f, bnd = 0.0f;
    for (int i = 0; i < 3; i++) {
        float px = i == 0 ? b : a, py = i == 1 ? b : a;
        float p0 = (v01 - v02) * px + v02 * (1.0f - py);
        float p1 = v12 * (1.0f - px - py);
        float ex = dx - (ox + xx * p0 + yx * p1);
        float ey = dy - (oy + xy * p0 + yy * p1);
        float ez = dz - (oz + xz * p0 + yz * p1);
        float r2 = ex * ex + ey * ey + ez * ez;
        float r = sqrtf(r2);
        if (!(r > 2.0f * ep)) return false;  // a point within rounding of r: FP64 decides
        float ir = 1.0f / r;
        if (efield) {
            float t = (ex * nx + ey * ny + ez * nz) * ir * ir * ir;
            sum += w * t;
            bnd += w * (8.0f * ep * ir * ir * ir + 16.0f * kU * ir * ir);
        } else {
            sum += w * ir;
            bnd += w * (4.0f * ep * ir * ir + 16.0f * kU * ir);
        }
    }
    val = sum * ratio;
    err = 4.0f * (bnd * fabsf(ratio) + (64.0f * kU * skew + 1e-6f) * fabsf(val));
    return isfinite(val) && isfinite(err);
}

// one direction of CAutoRefine::RefineCriteria in FP32: the weight of source
// S seen from evaluation element E (d = E.c - S.c), with its error bound
__device__ __forceinline__ bool weight32(const Element &E, const Element &S, float dx, float dy, float dz, float r, bool quad,
                                         float inv_max_area, float inv_max_side, float &cw, float &err) {
    bool diel = (E.type & FCG_IS_DIEL) != 0;
    float nx = 0.0f, ny = 0.0f, nz = 0.0f;
    if (diel && !diel_normal32(E.type, E.n, nx, ny, nz)) return false;
    float pe, pe_err;
    if (quad) {
        if (!quad2_32(dx, dy, dz, S.v, S.c, diel, nx, ny, nz, pe, pe_err)) return false;
    } else {
        float ir = 1.0f / r;
        if (diel) {
            pe = (dx * nx + dy * ny + dz * nz) * ir * ir * ir;
            pe_err = 4.0f * (16.0f * kU * ir * ir + 16.0f * kU * fabsf(pe));
        } else {
            pe = ir;
            pe_err = 16.0f * kU * ir;
        }
    }
    float W = (float)S.area * inv_max_area;
    if (diel) W *= (float)S.maxside * inv_max_side;
    cw = fabsf(pe * W);
    err = pe_err * W + 32.0f * kU * cw + 1e-6f * cw;
    return isfinite(cw) && isfinite(err);
}

// 1 above e, 0 at or below e (the FP64 test splits on c > e), -1 undecided
__device__ __forceinline__ int side_test(float c, float err, float e) {
    if (c - err > e * (1.0f + 4.0f * kU)) return 1;
    if (c + err < e * (1.0f - 4.0f * kU)) return 0;
    return -1;
}

}  // namespace pair32
}  // namespace fcg

#endif
