// Panel-pair potential integrals and element-pair tests shared by the host
// model builder, the device model construction (mesh refinement, link
// construction) and the device coefficient-fill kernels.
//
// Restated from the reference's collocation formulas:
//   potential_opt        CPotential::PotentialOpt        Solver/Potential.cpp:1561-1711
//   potential_numerical  CPotential::PotentialNumerical  Solver/Potential.cpp:2077-2153
//   enfield_numerical    CPotential::EnFieldNumerical    Solver/Potential.cpp:2172-2254
//   quadrature rules 2, 3, 5 of CPotential::InitNumerical Solver/Potential.cpp:112-128,133-149,181-206
//   pot_estimate         CAutoRefine::PotEstimateOpt (one-way, collocation)
//                                                        Solver/Autorefine.cpp:3474-3733
//   self_potential       CAutoRefine::SelfPotential      Solver/Autorefine.cpp:2358-2427
//   diel_normal          CAutoPanel::GetDielNormal       Solver/AutoPanel.h:114-139
//   refine_criteria      CAutoRefine::RefineCriteria     Solver/Autorefine.cpp:2928-3003
//   link_decision        one step of CAutoRefine::RefineMutual  Solver/Autorefine.cpp:3096-3235
//   mesh_decision        one step of CAutoRefine::DiscretizeMutual  Solver/Autorefine.cpp:2638-2730
//   subdivide            CAutoPanel::Subdivide           Solver/AutoPanel.cpp:382-523
//   newell_normal        normal of CAutoPanel::CalcPanelGeomPar  Solver/AutoPanel.cpp:51-104
// plus FP32 forms for the mixed-precision fill (potential32, pot_near32).
//
// Panel vertices, centroids and normals are single precision (as the
// reference stores them); every formula works in double. A difference of two
// float vectors is formed in float and then widened (the rule the model
// builder uses everywhere), a float operand meeting a double one is widened
// first. The order of every floating-point operation follows the reference so
// that host results are bit-reproducible (host code is compiled with
// -ffp-contract=off).
#ifndef FCG_POTENTIAL_H
#define FCG_POTENTIAL_H

#include <math.h>
#include <stdint.h>

#if defined(__CUDACC__)
#define FCG_HD __host__ __device__ __forceinline__
#else
#define FCG_HD inline
#endif

// physical constants as the reference defines them (Solver/Potential.h:41-45)
#define FCG_FOUR_PI_TIMES_E0 1.1126500559756e-10
#define FCG_TWO_TIMES_E0 1.7708375634e-11
#define FCG_POTENTIAL_GEO_EPS 1E-6
#define FCG_PANEL_EPS 1E-12

// element type bits (Solver/AutoElement.h:44-48)
#define FCG_IS_LEAF 1u
#define FCG_IS_DIEL 2u
#define FCG_OUTPERM_NORMAL_DIR 4u
#define FCG_OUTPERM_ELEMENT_LEVEL 8u
#define FCG_IS_SUPER_NODE 128u

struct fcg_d3 {
    double x, y, z;
};

FCG_HD fcg_d3 fcg_mk(double x, double y, double z) { fcg_d3 r; r.x = x; r.y = y; r.z = z; return r; }
FCG_HD fcg_d3 fcg_widen(const float *v) { return fcg_mk((double)v[0], (double)v[1], (double)v[2]); }
// float difference a-b formed in float, then widened
FCG_HD fcg_d3 fcg_fsub(const float *a, const float *b) {
    float x = a[0] - b[0], y = a[1] - b[1], z = a[2] - b[2];
    return fcg_mk((double)x, (double)y, (double)z);
}
FCG_HD double fcg_mod(fcg_d3 a) { return sqrt(a.x * a.x + a.y * a.y + a.z * a.z); }
FCG_HD double fcg_dot(fcg_d3 a, fcg_d3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
FCG_HD fcg_d3 fcg_cross(fcg_d3 a, fcg_d3 b) {
    return fcg_mk(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x);
}

// Quadrature rules in homogeneous triangle coordinates (x, y, 1) with weights.
// rule 2: 3 points, Strang-Fix #1; rule 3: 3 points, Strang-Fix #2;
// rule 5: 6 points, Strang-Fix #4 (the only rules the collocation scheme uses).
FCG_HD int fcg_rule_npts(int rule) { return rule == 5 ? 6 : 3; }
FCG_HD void fcg_rule_point(int rule, int i, double *px, double *py, double *w) {
    if (rule == 2) {
        const double a = 1.0 / 6.0, c = 4.0 / 6.0;
        *px = (i == 0) ? c : a;
        *py = (i == 1) ? c : a;
        *w = 1.0 / 3.0;
    } else if (rule == 3) {
        *px = (i == 0) ? 0.0 : 0.5;
        *py = (i == 1) ? 0.0 : 0.5;
        *w = 1.0 / 3.0;
    } else {
        const double a = 0.659027622374092, b = 0.231933368553031, c = 0.109039009072877;
        const double xs[6] = {a, a, b, b, c, c};
        const double ys[6] = {b, c, a, c, a, b};
        *px = xs[i];
        *py = ys[i];
        *w = 1.0 / 6.0;
    }
}

// Analytic potential at r of a uniform unit charge density on the triangle v
// (9 floats), divided by the triangle area.
FCG_HD double fcg_potential_opt(fcg_d3 r, const float *v) {
    fcg_d3 side[3], rhomp, Pmp[3], Rmp[3], n, rho, l, u;
    double Rmp_norm[3];
    side[0] = fcg_fsub(v + 3, v + 0);
    side[1] = fcg_fsub(v + 6, v + 3);
    side[2] = fcg_fsub(v + 0, v + 6);
    n = fcg_cross(side[0], side[1]);
    double nmod = fcg_mod(n);
    n.x = n.x / nmod;
    n.y = n.y / nmod;
    n.z = n.z / nmod;
    double nr = fcg_dot(n, r);
    rho.x = r.x - n.x * nr;
    rho.y = r.y - n.y * nr;
    rho.z = r.z - n.z * nr;
    for (int i = 0; i < 3; i++) {
        fcg_d3 vi = fcg_widen(v + 3 * i);
        double nv = fcg_dot(n, vi);
        rhomp.x = vi.x - n.x * nv;
        rhomp.y = vi.y - n.y * nv;
        rhomp.z = vi.z - n.z * nv;
        Pmp[i].x = rhomp.x - rho.x;
        Pmp[i].y = rhomp.y - rho.y;
        Pmp[i].z = rhomp.z - rho.z;
        Rmp[i].x = vi.x - r.x;
        Rmp[i].y = vi.y - r.y;
        Rmp[i].z = vi.z - r.z;
        Rmp_norm[i] = fcg_mod(Rmp[i]);
    }
    double d = -fcg_dot(n, Rmp[0]);
    double dnorm = fabs(d);
    double result = 0.0;
    for (int i = 0; i < 3; i++) {
        int j = (i == 2) ? 0 : i + 1;
        double ms = fcg_mod(side[i]);
        l.x = side[i].x / ms;
        l.y = side[i].y / ms;
        l.z = side[i].z / ms;
        u.x = l.y * n.z - l.z * n.y;
        u.y = l.z * n.x - l.x * n.z;
        u.z = l.x * n.y - l.y * n.x;
        double P0signed = fcg_dot(Pmp[j], u);
        double P0 = fabs(P0signed);
        double lplus = fcg_dot(Pmp[j], l);
        double lminus = fcg_dot(Pmp[i], l);
        double R0 = sqrt(P0 * P0 + d * d);
        double lplusabs = fabs(lplus), lminusabs = fabs(lminus);
        // the reference compares the signed values here
        double lmax = (lplus > lminus) ? lplusabs : lminusabs;
        if (P0 / lmax > FCG_POTENTIAL_GEO_EPS && fabs((Rmp_norm[j] + lplus) / lmax) > FCG_POTENTIAL_GEO_EPS &&
            fabs((Rmp_norm[i] + lminus) / lmax) > FCG_POTENTIAL_GEO_EPS) {
            double R0square = R0 * R0;
            double tan1 = atan(P0 * lplus / (R0square + dnorm * Rmp_norm[j]));
            double tan2 = atan(P0 * lminus / (R0square + dnorm * Rmp_norm[i]));
            double ln = log((Rmp_norm[j] + lplus) / (Rmp_norm[i] + lminus));
            double P0sign = (double)((P0signed > 0) - (P0signed < 0));
            result += P0sign * (P0 * ln - dnorm * (tan1 - tan2));
        }
    }
    return (result * 2.0) / nmod;
}

// Local 2D frame of a source triangle for the quadrature formulas.
struct fcg_quad_frame {
    fcg_d3 x, y, v0;
    double vert2d01, vert2d02, vert2d12, jacobian, area;
};

FCG_HD fcg_quad_frame fcg_frame(const float *v) {
    fcg_quad_frame f;
    fcg_d3 side1 = fcg_fsub(v + 3, v + 0);
    fcg_d3 side2 = fcg_fsub(v + 6, v + 3);
    fcg_d3 side3 = fcg_fsub(v + 0, v + 6);
    fcg_d3 normal, z;
    normal.x = side1.y * side2.z - side1.z * side2.y;
    normal.y = -side1.x * side2.z + side1.z * side2.x;
    normal.z = side1.x * side2.y - side1.y * side2.x;
    double mn = fcg_mod(normal);
    z.x = normal.x / mn;
    z.y = normal.y / mn;
    z.z = normal.z / mn;
    double m1 = fcg_mod(side1);
    f.x.x = side1.x / m1;
    f.x.y = side1.y / m1;
    f.x.z = side1.z / m1;
    f.y.x = f.x.y * z.z - f.x.z * z.y;
    f.y.y = f.x.z * z.x - f.x.x * z.z;
    f.y.z = f.x.x * z.y - f.x.y * z.x;
    f.vert2d01 = m1;
    f.vert2d02 = -(side3.x * f.x.x + side3.y * f.x.y + side3.z * f.x.z);
    f.vert2d12 = -(side3.x * f.y.x + side3.y * f.y.y + side3.z * f.y.z);
    f.jacobian = (f.vert2d02 - f.vert2d01) * f.vert2d12 - f.vert2d12 * f.vert2d02;
    f.area = mn / 2.0;
    f.v0 = fcg_widen(v);
    return f;
}

FCG_HD fcg_d3 fcg_frame_point(const fcg_quad_frame &f, double px, double py) {
    // homogeneous third coordinate is 1
    double point0 = (f.vert2d01 - f.vert2d02) * px + f.vert2d02 * (1.0 - py);
    double point1 = f.vert2d12 * (1.0 - px - py);
    fcg_d3 p;
    p.x = f.v0.x + f.x.x * point0 + f.y.x * point1;
    p.y = f.v0.y + f.x.y * point0 + f.y.y * point1;
    p.z = f.v0.z + f.x.z * point0 + f.y.z * point1;
    return p;
}

// Quadrature of 1/|p - r| over the triangle, divided by its area.
FCG_HD double fcg_potential_numerical(fcg_d3 r, const float *v, int rule) {
    fcg_quad_frame f = fcg_frame(v);
    double result = 0.0;
    int np = fcg_rule_npts(rule);
    for (int i = 0; i < np; i++) {
        double px, py, w;
        fcg_rule_point(rule, i, &px, &py, &w);
        fcg_d3 p = fcg_frame_point(f, px, py);
        fcg_d3 dd = fcg_mk(p.x - r.x, p.y - r.y, p.z - r.z);
        double pot = 1 / fcg_mod(dd);
        result += w * pot;
    }
    result *= f.jacobian / 2.0;
    result /= f.area;
    return result;
}

// Quadrature of (r - p).n / |r - p|^3 over the triangle, divided by its area.
FCG_HD double fcg_enfield_numerical(fcg_d3 r, const float *v, fcg_d3 tn, int rule) {
    fcg_quad_frame f = fcg_frame(v);
    double result = 0.0;
    int np = fcg_rule_npts(rule);
    for (int i = 0; i < np; i++) {
        double px, py, w;
        fcg_rule_point(rule, i, &px, &py, &w);
        fcg_d3 p = fcg_frame_point(f, px, py);
        fcg_d3 dist = fcg_mk(r.x - p.x, r.y - p.y, r.z - p.z);
        double rd = fcg_mod(dist);
        double pot = fcg_dot(dist, tn) / (rd * rd * rd);
        result += w * pot;
    }
    result *= f.jacobian / 2.0;
    result /= f.area;
    return result;
}

// Unit normal pointing to the outer-permittivity side of a dielectric element.
// Super nodes store an area-weighted, unnormalised normal.
FCG_HD fcg_d3 fcg_diel_normal(unsigned type, const float *normal) {
    fcg_d3 u;
    if (type & FCG_IS_SUPER_NODE) {
        fcg_d3 n = fcg_widen(normal);
        double m = fcg_mod(n);
        if (m < FCG_PANEL_EPS) u = fcg_mk(0.0, 0.0, 0.0);
        else u = fcg_mk(n.x / m, n.y / m, n.z / m);
    } else {
        u = fcg_widen(normal);
    }
    if ((type & FCG_OUTPERM_NORMAL_DIR) != FCG_OUTPERM_NORMAL_DIR) {
        u.x = -u.x;
        u.y = -u.y;
        u.z = -u.z;
    }
    return u;
}

// Distance band of a panel pair: 0 analytic (rho < 1), 1 rule 5 (rho < 2),
// 2 rule 3 (rho < 4), 3 rule 2 (rho < 10), 4 point formula.
FCG_HD int fcg_band(double rdist, double rmax) {
    double rho = rdist / rmax;
    if (rho < 1.0) return 0;
    if (rho < 2.0) return 1;
    if (rho < 4.0) return 2;
    if (rho < 10.0) return 3;
    return 4;
}

// Coefficient of potential (conductor evaluation element) or of normal
// electric field (dielectric evaluation element) at element 1's centroid due
// to a unit charge spread over element 2.
FCG_HD double fcg_pot_estimate(unsigned type1, const float *c1, const float *n1, double maxside1,
                               const float *c2, const float *v2, double maxside2) {
    fcg_d3 dist = fcg_fsub(c1, c2);
    double rdist = fcg_mod(dist);
    double rmax = (maxside1 > maxside2) ? maxside1 : maxside2;
    int band = fcg_band(rdist, rmax);
    fcg_d3 r1 = fcg_widen(c1);
    if ((type1 & FCG_IS_DIEL) != FCG_IS_DIEL) {
        switch (band) {
        case 0: return fcg_potential_opt(r1, v2) / FCG_FOUR_PI_TIMES_E0;
        case 1: return fcg_potential_numerical(r1, v2, 5) / FCG_FOUR_PI_TIMES_E0;
        case 2: return fcg_potential_numerical(r1, v2, 3) / FCG_FOUR_PI_TIMES_E0;
        case 3: return fcg_potential_numerical(r1, v2, 2) / FCG_FOUR_PI_TIMES_E0;
        default: return 1 / (FCG_FOUR_PI_TIMES_E0 * rdist);
        }
    }
    fcg_d3 nrm = fcg_diel_normal(type1, n1);
    switch (band) {
    case 0: {
        // central difference of the analytic potential across the panel
        double h = rdist / 20;
        fcg_d3 ep = fcg_mk(r1.x + nrm.x * h, r1.y + nrm.y * h, r1.z + nrm.z * h);
        fcg_d3 em = fcg_mk(r1.x - nrm.x * h, r1.y - nrm.y * h, r1.z - nrm.z * h);
        double pp = fcg_potential_opt(ep, v2);
        double pn = fcg_potential_opt(em, v2);
        return (pn - pp) / (2 * h * FCG_FOUR_PI_TIMES_E0);
    }
    case 1: return fcg_enfield_numerical(r1, v2, nrm, 5) / FCG_FOUR_PI_TIMES_E0;
    case 2: return fcg_enfield_numerical(r1, v2, nrm, 3) / FCG_FOUR_PI_TIMES_E0;
    case 3: return fcg_enfield_numerical(r1, v2, nrm, 2) / FCG_FOUR_PI_TIMES_E0;
    default: return fcg_dot(dist, nrm) / (FCG_FOUR_PI_TIMES_E0 * rdist * rdist * rdist);
    }
}

// The source-triangle-only part of fcg_potential_opt (unit normal, its
// modulus, projected vertices, unit edge vectors and in-plane edge normals),
// computed once per triangle so that every near-field evaluation against it
// skips four square roots and twelve divisions. Same operations, same order:
// fcg_potential_opt_tri returns exactly what fcg_potential_opt returns.
struct fcg_tri64 {
    double n[3], nmod, rhomp[9], l[9], u[9], pad;
};

FCG_HD void fcg_tri64_make(const float *v, fcg_tri64 &t) {
    fcg_d3 side[3], n;
    side[0] = fcg_fsub(v + 3, v + 0);
    side[1] = fcg_fsub(v + 6, v + 3);
    side[2] = fcg_fsub(v + 0, v + 6);
    n = fcg_cross(side[0], side[1]);
    double nmod = fcg_mod(n);
    n.x = n.x / nmod;
    n.y = n.y / nmod;
    n.z = n.z / nmod;
    t.n[0] = n.x; t.n[1] = n.y; t.n[2] = n.z;
    t.nmod = nmod;
    for (int i = 0; i < 3; i++) {
        fcg_d3 vi = fcg_widen(v + 3 * i);
        double nv = fcg_dot(n, vi);
        t.rhomp[3 * i] = vi.x - n.x * nv;
        t.rhomp[3 * i + 1] = vi.y - n.y * nv;
        t.rhomp[3 * i + 2] = vi.z - n.z * nv;
        double ms = fcg_mod(side[i]);
        fcg_d3 l = fcg_mk(side[i].x / ms, side[i].y / ms, side[i].z / ms);
        t.l[3 * i] = l.x; t.l[3 * i + 1] = l.y; t.l[3 * i + 2] = l.z;
        t.u[3 * i] = l.y * n.z - l.z * n.y;
        t.u[3 * i + 1] = l.z * n.x - l.x * n.z;
        t.u[3 * i + 2] = l.x * n.y - l.y * n.x;
    }
    t.pad = 0.0;
}

FCG_HD double fcg_potential_opt_tri(fcg_d3 r, const float *v, const fcg_tri64 &t) {
    fcg_d3 n = fcg_mk(t.n[0], t.n[1], t.n[2]), rho, Pmp[3], Rmp[3];
    double Rmp_norm[3];
    double nr = fcg_dot(n, r);
    rho.x = r.x - n.x * nr;
    rho.y = r.y - n.y * nr;
    rho.z = r.z - n.z * nr;
    for (int i = 0; i < 3; i++) {
        fcg_d3 vi = fcg_widen(v + 3 * i);
        Pmp[i].x = t.rhomp[3 * i] - rho.x;
        Pmp[i].y = t.rhomp[3 * i + 1] - rho.y;
        Pmp[i].z = t.rhomp[3 * i + 2] - rho.z;
        Rmp[i].x = vi.x - r.x;
        Rmp[i].y = vi.y - r.y;
        Rmp[i].z = vi.z - r.z;
        Rmp_norm[i] = fcg_mod(Rmp[i]);
    }
    double d = -fcg_dot(n, Rmp[0]);
    double dnorm = fabs(d);
    double result = 0.0;
    for (int i = 0; i < 3; i++) {
        int j = (i == 2) ? 0 : i + 1;
        fcg_d3 l = fcg_mk(t.l[3 * i], t.l[3 * i + 1], t.l[3 * i + 2]);
        fcg_d3 u = fcg_mk(t.u[3 * i], t.u[3 * i + 1], t.u[3 * i + 2]);
        double P0signed = fcg_dot(Pmp[j], u);
        double P0 = fabs(P0signed);
        double lplus = fcg_dot(Pmp[j], l);
        double lminus = fcg_dot(Pmp[i], l);
        double R0 = sqrt(P0 * P0 + d * d);
        double lplusabs = fabs(lplus), lminusabs = fabs(lminus);
        double lmax = (lplus > lminus) ? lplusabs : lminusabs;
        if (P0 / lmax > FCG_POTENTIAL_GEO_EPS && fabs((Rmp_norm[j] + lplus) / lmax) > FCG_POTENTIAL_GEO_EPS &&
            fabs((Rmp_norm[i] + lminus) / lmax) > FCG_POTENTIAL_GEO_EPS) {
            double R0square = R0 * R0;
            double tan1 = atan(P0 * lplus / (R0square + dnorm * Rmp_norm[j]));
            double tan2 = atan(P0 * lminus / (R0square + dnorm * Rmp_norm[i]));
            double ln = log((Rmp_norm[j] + lplus) / (Rmp_norm[i] + lminus));
            double P0sign = (double)((P0signed > 0) - (P0signed < 0));
            result += P0sign * (P0 * ln - dnorm * (tan1 - tan2));
        }
    }
    return (result * 2.0) / t.nmod;
}

// fcg_potential_opt_tri with fewer FP64 divisions and transcendentals, for
// the device fill (FP64 throughput bounds the near field): per edge
//  * the three degeneracy guards x / lmax > eps are tested as x > eps * lmax
//    (same outcome, lmax = 0 included, up to rounding at the threshold);
//  * atan(N1/D1) - atan(N2/D2), with D1, D2 > 0, is the argument of
//    (D1 + i N1)(D2 - i N2): one atan2(N1 D2 - N2 D1, D1 D2 + N1 N2) instead
//    of two atan and two divisions (exact identity; both forms lose the same
//    relative accuracy when the angles nearly cancel). The term is multiplied
//    by |d| and skipped when the field point is in the triangle's plane.
// Results agree with fcg_potential_opt to about 1e-14 relative.
FCG_HD double fcg_potential_opt_fast(fcg_d3 r, const float *v, const fcg_tri64 &t) {
    fcg_d3 n = fcg_mk(t.n[0], t.n[1], t.n[2]), rho, Pmp[3];
    double Rn[3];
    double nr = fcg_dot(n, r);
    rho.x = r.x - n.x * nr;
    rho.y = r.y - n.y * nr;
    rho.z = r.z - n.z * nr;
    fcg_d3 R0v;
    for (int i = 0; i < 3; i++) {
        fcg_d3 vi = fcg_widen(v + 3 * i);
        Pmp[i].x = t.rhomp[3 * i] - rho.x;
        Pmp[i].y = t.rhomp[3 * i + 1] - rho.y;
        Pmp[i].z = t.rhomp[3 * i + 2] - rho.z;
        fcg_d3 Ri = fcg_mk(vi.x - r.x, vi.y - r.y, vi.z - r.z);
        if (i == 0) R0v = Ri;
        Rn[i] = fcg_mod(Ri);
    }
    double d = -fcg_dot(n, R0v);
    double dnorm = fabs(d);
    double result = 0.0;
    for (int i = 0; i < 3; i++) {
        int j = (i == 2) ? 0 : i + 1;
        fcg_d3 l = fcg_mk(t.l[3 * i], t.l[3 * i + 1], t.l[3 * i + 2]);
        fcg_d3 u = fcg_mk(t.u[3 * i], t.u[3 * i + 1], t.u[3 * i + 2]);
        double P0signed = fcg_dot(Pmp[j], u);
        double P0 = fabs(P0signed);
        double lplus = fcg_dot(Pmp[j], l);
        double lminus = fcg_dot(Pmp[i], l);
        double lmax = (lplus > lminus) ? fabs(lplus) : fabs(lminus);
        double ap = Rn[j] + lplus, am = Rn[i] + lminus;
        double tol = FCG_POTENTIAL_GEO_EPS * lmax;
        if (P0 > tol && fabs(ap) > tol && fabs(am) > tol) {
            double R0sq = P0 * P0 + d * d;
            double dt = 0.0;
            if (dnorm > 0.0) {
                double N1 = P0 * lplus, D1 = R0sq + dnorm * Rn[j];
                double N2 = P0 * lminus, D2 = R0sq + dnorm * Rn[i];
                dt = atan2(N1 * D2 - N2 * D1, D1 * D2 + N1 * N2);
            }
            double ln = log(ap / am);
            double P0sign = (double)((P0signed > 0) - (P0signed < 0));
            result += P0sign * (P0 * ln - dnorm * dt);
        }
    }
    return (result * 2.0) / t.nmod;
}

// ---- single-precision analytic potential (mixed-precision near field)
// The potential_opt formula in FP32, in a frame centred on the source
// triangle's centroid and scaled by its largest vertex distance `s` (every
// quantity O(1)); the potential of the scaled problem is s times the
// original. Two rewrites keep FP32 accurate: R + l for l < 0 is formed as
// (P0^2 + d^2) / (R - l) (no cancellation), and the reference's guards
// (P0, R + lplus, R + lminus against 1e-6 lmax) are tested with an error
// bound. When an R + l guard is too close to call in FP32 the evaluation
// reports it and the caller computes that coefficient with the FP64
// formula; an undecidable P0 guard is accepted when the edge's term (which
// is proportional to P0) is below 2e-6 of the scaled potential, since
// keeping or dropping it then changes the result by less than FP32 noise.
struct fcg_tri32 {
    float n[3];      // unit normal
    float inv_s;     // 1 / s
    float w[9];      // vertices - centroid, scaled
    float rp[9];     // the same projected on the plane through the centroid
    float l[9];      // unit edge vectors
    float u[9];      // in-plane edge normals l x n
    float inv_area;  // 1 / area of the scaled triangle
    float pad[3];
};

FCG_HD void fcg_tri32_make(const float *v, const float *c, fcg_tri32 &t) {
    fcg_tri64 T;
    fcg_tri64_make(v, T);
    fcg_d3 cc = fcg_widen(c), n = fcg_mk(T.n[0], T.n[1], T.n[2]);
    fcg_d3 w[3];
    double smax = 0.0;
    for (int i = 0; i < 3; i++) {
        fcg_d3 vi = fcg_widen(v + 3 * i);
        w[i] = fcg_mk(vi.x - cc.x, vi.y - cc.y, vi.z - cc.z);
        double m = fcg_mod(w[i]);
        smax = m > smax ? m : smax;
    }
    double is = smax > 0.0 ? 1.0 / smax : 1.0;
    for (int k = 0; k < 3; k++) t.n[k] = (float)T.n[k];
    t.inv_s = (float)is;
    for (int i = 0; i < 3; i++) {
        fcg_d3 a = fcg_mk(w[i].x * is, w[i].y * is, w[i].z * is);
        double an = fcg_dot(n, a);
        t.w[3 * i] = (float)a.x; t.w[3 * i + 1] = (float)a.y; t.w[3 * i + 2] = (float)a.z;
        t.rp[3 * i] = (float)(a.x - n.x * an);
        t.rp[3 * i + 1] = (float)(a.y - n.y * an);
        t.rp[3 * i + 2] = (float)(a.z - n.z * an);
        for (int k = 0; k < 3; k++) {
            t.l[3 * i + k] = (float)T.l[3 * i + k];
            t.u[3 * i + k] = (float)T.u[3 * i + k];
        }
    }
    t.inv_area = (float)(2.0 / (T.nmod * is * is));
    t.pad[0] = t.pad[1] = t.pad[2] = 0.0f;
}

// potential_opt at r = centroid + (px, py, pz) (unscaled float offsets);
// false when the FP32 evaluation cannot decide a guard the way FP64 would
FCG_HD bool fcg_potential32(float px, float py, float pz, const fcg_tri32 &t, float *out) {
    const float U = 5.9604645e-8f;
    px *= t.inv_s;
    py *= t.inv_s;
    pz *= t.inv_s;
    float nr = t.n[0] * px + t.n[1] * py + t.n[2] * pz;
    float rx = px - t.n[0] * nr, ry = py - t.n[1] * nr, rz = pz - t.n[2] * nr;
    float pm = sqrtf(px * px + py * py + pz * pz);
    float eP = 32.0f * U * (pm + 1.0f);  // absolute error of P0, d, lplus, lminus
    float Pm[9], R[3];
    for (int i = 0; i < 3; i++) {
        Pm[3 * i] = t.rp[3 * i] - rx;
        Pm[3 * i + 1] = t.rp[3 * i + 1] - ry;
        Pm[3 * i + 2] = t.rp[3 * i + 2] - rz;
        float ax = t.w[3 * i] - px, ay = t.w[3 * i + 1] - py, az = t.w[3 * i + 2] - pz;
        R[i] = sqrtf(ax * ax + ay * ay + az * az);
    }
    float d = -(t.n[0] * (t.w[0] - px) + t.n[1] * (t.w[1] - py) + t.n[2] * (t.w[2] - pz));
    float dn = fabsf(d);
    float res = 0.0f;
    for (int i = 0; i < 3; i++) {
        int j = (i == 2) ? 0 : i + 1;
        const float *l = t.l + 3 * i, *u = t.u + 3 * i, *Pj = Pm + 3 * j, *Pi = Pm + 3 * i;
        float P0s = Pj[0] * u[0] + Pj[1] * u[1] + Pj[2] * u[2];
        float P0 = fabsf(P0s);
        float lp = Pj[0] * l[0] + Pj[1] * l[1] + Pj[2] * l[2];
        float lm = Pi[0] * l[0] + Pi[1] * l[1] + Pi[2] * l[2];
        float lmax = (lp > lm) ? fabsf(lp) : fabsf(lm);
        float tol = (float)FCG_POTENTIAL_GEO_EPS * lmax;
        float etol = (float)FCG_POTENTIAL_GEO_EPS * eP + 4.0f * U * tol;
        float R0sq = P0 * P0 + d * d;
        float eR0 = 2.0f * (P0 + dn) * eP + 2.0f * eP * eP + 4.0f * U * R0sq;
        float ap, eap, am, eam;
        if (lp >= 0.0f) { ap = R[j] + lp; eap = 16.0f * U * ap + 2.0f * eP; }
        else { float q = R[j] - lp; ap = R0sq / q; eap = (eR0 + 2.0f * eP * ap) / q + 8.0f * U * ap; }
        if (lm >= 0.0f) { am = R[i] + lm; eam = 16.0f * U * am + 2.0f * eP; }
        else { float q = R[i] - lm; am = R0sq / q; eam = (eR0 + 2.0f * eP * am) / q + 8.0f * U * am; }
        // the R + l guards keep or drop a term whose logarithm diverges: FP32
        // must decide them with certainty
        if (!(fabsf(ap - tol) > 2.0f * (eap + etol)) || !(fabsf(am - tol) > 2.0f * (eam + etol))) return false;
        // the P0 guard keeps or drops a term proportional to P0 (a field point
        // on the edge's line, common between perpendicular faces): when FP32
        // cannot decide it, either choice is fine while the term is negligible
        bool p0_close = !(fabsf(P0 - tol) > 2.0f * (eP + etol));
        bool keep = P0 > tol && ap > tol && am > tol;
        if (keep || (p0_close && ap > tol && am > tol)) {
            float dt = 0.0f;
            if (dn > 0.0f) {
                float N1 = P0 * lp, D1 = R0sq + dn * R[j];
                float N2 = P0 * lm, D2 = R0sq + dn * R[i];
                dt = atan2f(N1 * D2 - N2 * D1, D1 * D2 + N1 * N2);
            }
            float ln = logf(ap / am);
            float sg = (float)((P0s > 0.0f) - (P0s < 0.0f));
            float term = sg * (P0 * ln - dn * dt);
            if (p0_close && !(fabsf(term) < 2e-6f)) return false;
            if (keep) res += term;
        }
    }
    *out = res * t.inv_area * t.inv_s;
    return true;
}

// Near-field coefficient in FP32 (the mixed-precision fill): the analytic
// potential, or for a dielectric evaluation element its central difference
// across the panel; false where an FP64 evaluation must decide a guard.
FCG_HD bool fcg_pot_near32(unsigned type1, const float *c1, const float *n1, const float *c2, const fcg_tri32 &t, float *out) {
    const float k = (float)(1.0 / FCG_FOUR_PI_TIMES_E0);
    float dx = c1[0] - c2[0], dy = c1[1] - c2[1], dz = c1[2] - c2[2];
    float v;
    if ((type1 & FCG_IS_DIEL) != FCG_IS_DIEL) {
        if (!fcg_potential32(dx, dy, dz, t, &v)) return false;
        *out = k * v;
        return true;
    }
    fcg_d3 nrm = fcg_diel_normal(type1, n1);
    float h = sqrtf(dx * dx + dy * dy + dz * dz) / 20.0f;
    float hx = (float)nrm.x * h, hy = (float)nrm.y * h, hz = (float)nrm.z * h;
    float pp, pn;
    if (!fcg_potential32(dx + hx, dy + hy, dz + hz, t, &pp) || !fcg_potential32(dx - hx, dy - hy, dz - hz, t, &pn)) return false;
    *out = k * ((pn - pp) / (2.0f * h));
    return true;
}

// Near-field coefficient with the source triangle's precomputed table.
FCG_HD double fcg_pot_near_tri(unsigned type1, const float *c1, const float *n1, const float *c2, const float *v2,
                               const fcg_tri64 &t) {
    fcg_d3 r1 = fcg_widen(c1);
    if ((type1 & FCG_IS_DIEL) != FCG_IS_DIEL) return fcg_potential_opt_fast(r1, v2, t) / FCG_FOUR_PI_TIMES_E0;
    fcg_d3 dist = fcg_fsub(c1, c2);
    double rdist = fcg_mod(dist);
    fcg_d3 nrm = fcg_diel_normal(type1, n1);
    double h = rdist / 20;
    fcg_d3 ep = fcg_mk(r1.x + nrm.x * h, r1.y + nrm.y * h, r1.z + nrm.z * h);
    fcg_d3 em = fcg_mk(r1.x - nrm.x * h, r1.y - nrm.y * h, r1.z - nrm.z * h);
    double pp = fcg_potential_opt_fast(ep, v2, t);
    double pn = fcg_potential_opt_fast(em, v2, t);
    return (pn - pp) / (2 * h * FCG_FOUR_PI_TIMES_E0);
}

// Near-field (band 0) coefficient: analytic potential, or for a dielectric
// evaluation element the central difference of the analytic potential.
FCG_HD double fcg_pot_near(unsigned type1, const float *c1, const float *n1, const float *c2, const float *v2) {
    fcg_d3 dist = fcg_fsub(c1, c2);
    double rdist = fcg_mod(dist);
    fcg_d3 r1 = fcg_widen(c1);
    if ((type1 & FCG_IS_DIEL) != FCG_IS_DIEL) return fcg_potential_opt(r1, v2) / FCG_FOUR_PI_TIMES_E0;
    fcg_d3 nrm = fcg_diel_normal(type1, n1);
    double h = rdist / 20;
    fcg_d3 ep = fcg_mk(r1.x + nrm.x * h, r1.y + nrm.y * h, r1.z + nrm.z * h);
    fcg_d3 em = fcg_mk(r1.x - nrm.x * h, r1.y - nrm.y * h, r1.z - nrm.z * h);
    double pp = fcg_potential_opt(ep, v2);
    double pn = fcg_potential_opt(em, v2);
    return (pn - pp) / (2 * h * FCG_FOUR_PI_TIMES_E0);
}

// ---- single-precision band classification (mixed-precision fill)
// fcg_band of the float offset (dx, dy, dz) and rmax, decided in single
// precision where that is certain: the FP32 ratio carries a relative error
// below 1e-6, so outside a 1e-5 relative margin around each threshold its
// band is the FP64 band; inside the margin (or for a non-finite ratio) the
// FP64 ratio decides. Returns exactly what fcg_band(fcg_mod(offset), rmax)
// returns.
FCG_HD int fcg_band_exact(float dx, float dy, float dz, double rmax) {
    float d2 = dx * dx + dy * dy + dz * dz;
    float rho = sqrtf(d2) / (float)rmax;
    const float m = 1e-5f;
    bool sure = rho == rho && rho < 3.0e38f && fabsf(rho - 1.0f) > m && fabsf(rho - 2.0f) > 2.0f * m &&
                fabsf(rho - 4.0f) > 4.0f * m && fabsf(rho - 10.0f) > 10.0f * m;
    if (sure) return rho < 1.0f ? 0 : rho < 2.0f ? 1 : rho < 4.0f ? 2 : rho < 10.0f ? 3 : 4;
    double rd = sqrt((double)dx * (double)dx + (double)dy * (double)dy + (double)dz * (double)dz);
    return fcg_band(rd, rmax);
}

// Self coefficient of a leaf panel: collocated analytic potential for a
// conductor panel, field-discontinuity term for a dielectric panel with
// permittivities eb (outer side) and ea (inner side).
FCG_HD double fcg_self_potential(unsigned type, const float *c, const float *v, double area, double eb, double ea) {
    if (type & FCG_IS_DIEL) return (ea + eb) / (FCG_TWO_TIMES_E0 * (eb - ea) * area);
    return fcg_potential_opt(fcg_widen(c), v) / FCG_FOUR_PI_TIMES_E0;
}

// ---------------------------------------------------------------- refinement
// The element-pair tests of the adaptive mesh and of the link construction,
// shared by the host model builder and the device link construction. `E` is
// any element record with float v[9], c[3], n[3], an integer `type`, double
// `area` and `maxside` and int32 `left` / `right` children. Both sides are
// compiled without contraction (host -ffp-contract=off, device -fmad=false);
// the operations are +, -, *, / and sqrt only, so host and device take
// bit-identical decisions.

// Centroid distance vector (float difference, widened), its modulus and the
// larger of the two elements' longest sides (the preamble of
// CAutoRefine::RefineMutual, Solver/Autorefine.cpp:3112-3121).
template <class E>
FCG_HD void fcg_pair_span(const E &A, const E &B, fcg_d3 *dist, double *rdist, double *rmax) {
    *dist = fcg_fsub(A.c, B.c);
    *rdist = fcg_mod(*dist);
    double r1 = A.maxside, r2 = B.maxside;
    *rmax = r1 > r2 ? r1 : r2;
}

// CAutoRefine::RefineCriteria (Solver/Autorefine.cpp:2928-3003): the one-way
// potential estimate of each element at the other's centroid (normal field
// for a dielectric evaluation element; rule-2 quadrature when the centroids
// are closer than twice the larger side, the point formula beyond), weighted
// by the source's area (and longest side, for a dielectric) relative to the
// model's largest. True when either weight exceeds `e`.
template <class E>
FCG_HD bool fcg_refine_criteria(const E &A, const E &B, fcg_d3 dist, double rdist, double rmax, double e, double ccoeff,
                                double max_side, double max_area, double *c1, double *c2) {
    bool force = false;
    fcg_d3 n1 = fcg_diel_normal(A.type, A.n), n2 = fcg_diel_normal(B.type, B.n);
    double pe1, pe2;
    bool d1 = (A.type & FCG_IS_DIEL) != 0, d2 = (B.type & FCG_IS_DIEL) != 0;
    if (rdist / rmax < 2.0) {
        fcg_d3 ca = fcg_widen(A.c), cb = fcg_widen(B.c);
        pe1 = d1 ? fcg_enfield_numerical(ca, B.v, n1, 2) : fcg_potential_numerical(ca, B.v, 2);
        pe2 = d2 ? fcg_enfield_numerical(cb, A.v, n2, 2) : fcg_potential_numerical(cb, A.v, 2);
    } else {
        if (d1) pe1 = (dist.x * n1.x + dist.y * n1.y + dist.z * n1.z) / (rdist * rdist * rdist);
        else pe1 = 1.0 / rdist;
        if (d2) pe2 = (-dist.x * n2.x + -dist.y * n2.y + -dist.z * n2.z) / (rdist * rdist * rdist);
        else pe2 = 1.0 / rdist;
    }
    if (d1) *c1 = fabs(pe1 * B.area * B.maxside / (max_side * max_area * ccoeff));
    else *c1 = fabs(pe1 * B.area / (max_area * ccoeff));
    if (*c1 > e) force = true;
    if (d2) *c2 = fabs(pe2 * A.area * A.maxside / (max_side * max_area * ccoeff));
    else *c2 = fabs(pe2 * A.area / (max_area * ccoeff));
    if (*c2 > e) force = true;
    return force;
}

// One step of CAutoRefine::RefineMutual (Solver/Autorefine.cpp:3096-3235):
// 0 = the pair interacts through one link; 1 = recurse into A's children;
// 2 = recurse into B's children. Two leaves always link; otherwise the pair
// is split when the criteria at link tolerance `eps` fail, on the non-leaf
// side, or on the larger-area side when both have children.
template <class E>
FCG_HD int fcg_link_decision(const E &A, const E &B, double eps, double max_side, double max_area) {
    bool leaf1 = (A.type & FCG_IS_LEAF) != 0, leaf2 = (B.type & FCG_IS_LEAF) != 0;
    if (leaf1 && leaf2) return 0;
    fcg_d3 dist;
    double rdist, rmax, c1, c2;
    fcg_pair_span(A, B, &dist, &rdist, &rmax);
    if (!fcg_refine_criteria(A, B, dist, rdist, rmax, eps, 1.0, max_side, max_area, &c1, &c2)) return 0;
    if (!leaf1 && leaf2) return 1;
    if (leaf1 && !leaf2) return 2;
    return A.area > B.area ? 1 : 2;
}

// ---------------------------------------------------------------- mesh
// Newell normal of a triangle accumulated in float, normalised (in double,
// rounded to float) when its modulus exceeds the panel epsilon; returns the
// modulus (the normal of CAutoPanel::CalcPanelGeomPar, Solver/AutoPanel.cpp:51-104).
FCG_HD double fcg_newell_normal(const float *v, float *n) {
    n[0] = n[1] = n[2] = 0.0f;
    for (int i = 0; i < 3; i++) {
        int j = i + 1 > 2 ? 0 : i + 1;
        const float *a = v + 3 * i, *b = v + 3 * j;
        n[0] += (a[1] - b[1]) * (a[2] + b[2]);
        n[1] += (a[2] - b[2]) * (a[0] + b[0]);
        n[2] += (a[0] - b[0]) * (a[1] + b[1]);
    }
    double m = fcg_mod(fcg_widen(n));
    if (m > FCG_PANEL_EPS) {
        n[0] = (float)(n[0] / m);
        n[1] = (float)(n[1] / m);
        n[2] = (float)(n[2] / m);
    }
    return m;
}

// geometric normal: a panel's own, a super node's from its synthetic triangle
template <class E>
FCG_HD fcg_d3 fcg_geo_normal(const E &e) {
    if (e.type & FCG_IS_SUPER_NODE) {
        float n[3];
        fcg_newell_normal(e.v, n);
        return fcg_widen(n);
    }
    return fcg_widen(e.n);
}

// CAutoPanel::MakeSuperPanel (Solver/AutoPanel.cpp:209-379): the super node
// of two elements: area-weighted centroid and outer-permittivity normal, and
// an equilateral synthetic triangle of the summed area in the plane of that
// normal. Host and device builders share this code (FP64, no contraction),
// so both make the same super nodes bit for bit; lid and rid are the
// children's element ids.
#define FCG_2_DIV_4TH_ROOT_27 0.87738267530166164054614593453133
#define FCG_2_DIV_4TH_ROOT_3 1.5196713713031850946623755013091
#define FCG_M05_PLUS_SQR2_DIV_4 -0.14644660940672623779957781894758
#define FCG_05_PLUS_SQR2_DIV_4 0.85355339059327376220042218105242
#define FCG_SQR2 1.4142135623730950488016887242097
template <class E>
FCG_HD void fcg_make_super(const E &L, const E &R, int lid, int rid, E &e) {
    const bool ld = (L.type & FCG_IS_DIEL) != 0, rd = (R.type & FCG_IS_DIEL) != 0;
    e.type = FCG_IS_LEAF;
    if (ld && rd) e.type |= (FCG_IS_SUPER_NODE | FCG_IS_DIEL | FCG_OUTPERM_NORMAL_DIR);
    else e.type |= FCG_IS_SUPER_NODE;
    e.type &= ~FCG_IS_LEAF;
    e.left = lid;
    e.right = rid;
    e.diel = 0;
    e.area = L.area + R.area;
    fcg_d3 cen = fcg_mk((L.c[0] * L.area + R.c[0] * R.area) / e.area, ((double)L.c[1] * L.area + (double)R.c[1] * R.area) / e.area,
                        ((double)L.c[2] * L.area + (double)R.c[2] * R.area) / e.area);
    e.c[0] = (float)cen.x;
    e.c[1] = (float)cen.y;
    e.c[2] = (float)cen.z;
    fcg_d3 ln = fcg_widen(L.n), rn = fcg_widen(R.n);
    if (!(L.type & FCG_OUTPERM_NORMAL_DIR)) ln = fcg_mk(-ln.x, -ln.y, -ln.z);
    if (!(R.type & FCG_OUTPERM_NORMAL_DIR)) rn = fcg_mk(-rn.x, -rn.y, -rn.z);
    e.n[0] = (float)((ln.x * L.area + rn.x * R.area) / e.area);
    e.n[1] = (float)((ln.y * L.area + rn.y * R.area) / e.area);
    e.n[2] = (float)((ln.z * L.area + rn.z * R.area) / e.area);
    const double modnormal = fcg_mod(fcg_widen(e.n));
    fcg_d3 normal;
    if (modnormal < FCG_PANEL_EPS) {
        if (fabs(ln.x) > FCG_PANEL_EPS) {
            normal.x = (-ln.y - ln.z) / ln.x; normal.y = 1.0; normal.z = 1.0;
        } else if (fabs(ln.y) > FCG_PANEL_EPS) {
            normal.y = (-ln.x - ln.z) / ln.y; normal.x = 1.0; normal.z = 1.0;
        } else if (fabs(ln.z) > FCG_PANEL_EPS) {
            normal.z = (-ln.x - ln.y) / ln.z; normal.x = 1.0; normal.y = 1.0;
        } else {
            const fcg_d3 gl = fcg_geo_normal(L), gr = fcg_geo_normal(R);
            normal = fcg_mk(gl.x * L.area + gr.x * R.area, gl.y * L.area + gr.y * R.area, gl.z * L.area + gr.z * R.area);
            const double m = fcg_mod(normal);
            normal = fcg_mk(normal.x / m, normal.y / m, normal.z / m);
            if (fcg_mod(normal) < FCG_PANEL_EPS) normal = fcg_mk(0.0, 0.0, 1.0);
        }
    } else {
        normal = fcg_mk((double)e.n[0] / modnormal, (double)e.n[1] / modnormal, (double)e.n[2] / modnormal);
    }
    fcg_d3 cm = L.area < R.area ? fcg_fsub(L.c, e.c) : fcg_fsub(R.c, e.c);
    if (fcg_mod(fcg_cross(normal, cm)) < FCG_PANEL_EPS) {
        cm.x = normal.x * 0.5 + normal.y * FCG_M05_PLUS_SQR2_DIV_4 + normal.z * FCG_05_PLUS_SQR2_DIV_4;
        cm.y = normal.x * 0.5 + normal.y * FCG_05_PLUS_SQR2_DIV_4 + normal.z * FCG_M05_PLUS_SQR2_DIV_4;
        cm.z = normal.x * (-FCG_SQR2) + normal.y * 0.5 + normal.z * 0.5;
    }
    fcg_d3 xv = fcg_cross(cm, normal);
    double mx = fcg_mod(xv);
    xv = fcg_mk(xv.x / mx, xv.y / mx, xv.z / mx);
    fcg_d3 yv = fcg_cross(normal, xv);
    double my = fcg_mod(yv);
    yv = fcg_mk(yv.x / my, yv.y / my, yv.z / my);
    const double Rr = FCG_2_DIV_4TH_ROOT_27 * sqrt(e.area);
    const fcg_d3 c = fcg_widen(e.c);
    e.v[0] = (float)(c.x + yv.x * Rr);
    e.v[1] = (float)(c.y + yv.y * Rr);
    e.v[2] = (float)(c.z + yv.z * Rr);
    const double a = FCG_2_DIV_4TH_ROOT_3 * sqrt(e.area);
    e.v[3] = (float)((c.x - yv.x * (Rr / 2.0)) - xv.x * (a / 2.0));
    e.v[4] = (float)((c.y - yv.y * (Rr / 2.0)) - xv.y * (a / 2.0));
    e.v[5] = (float)((c.z - yv.z * (Rr / 2.0)) - xv.z * (a / 2.0));
    e.v[6] = (float)((c.x - yv.x * (Rr / 2.0)) + xv.x * (a / 2.0));
    e.v[7] = (float)((c.y - yv.y * (Rr / 2.0)) + xv.y * (a / 2.0));
    e.v[8] = (float)((c.z - yv.z * (Rr / 2.0)) + xv.z * (a / 2.0));
    e.maxside_idx = 0;
    e.maxside = a;
}

template <class E>
FCG_HD void fcg_centroid3(E &e) {
    float sx = e.v[0] + e.v[3], sy = e.v[1] + e.v[4], sz = e.v[2] + e.v[5];
    sx = sx + e.v[6];
    sy = sy + e.v[7];
    sz = sz + e.v[8];
    e.c[0] = (float)(sx / 3.0);
    e.c[1] = (float)(sy / 3.0);
    e.c[2] = (float)(sz / 3.0);
}

template <class E>
FCG_HD int fcg_max_side3(E &e, double l0, double l1, double l2) {
    if (l0 >= l1 && l0 >= l2) { e.maxside_idx = 0; e.maxside = l0; }
    else if (l1 >= l0 && l1 >= l2) { e.maxside_idx = 1; e.maxside = l1; }
    else { e.maxside_idx = 2; e.maxside = l2; }
    return e.maxside_idx;
}

// CAutoPanel::Subdivide (Solver/AutoPanel.cpp:382-523): bisect a leaf
// triangle across its longest side (midpoint = float sum halved in double,
// rounded to float); the children keep the parent's type, dielectric index
// and normal, halve its area and get their own centroid and longest side.
template <class E>
FCG_HD void fcg_subdivide(const E &P, E &Lc, E &Rc) {
    int ms = P.maxside_idx;
    const float *v0 = P.v, *v1 = P.v + 3, *v2 = P.v + 6;
    const float *a, *b, *o;  // side endpoints a-b, opposite vertex o
    if (ms == 0) { a = v1; b = v0; o = v2; }
    else if (ms == 1) { a = v2; b = v1; o = v0; }
    else { a = v0; b = v2; o = v1; }
    float sx = a[0] + b[0], sy = a[1] + b[1], sz = a[2] + b[2];
    fcg_d3 mid = fcg_mk(sx / 2.0, sy / 2.0, sz / 2.0);
    double newside = fcg_mod(fcg_mk((double)o[0] - mid.x, (double)o[1] - mid.y, (double)o[2] - mid.z));
    double half = P.maxside / 2.0;
    float m[3] = {(float)mid.x, (float)mid.y, (float)mid.z};
    const float *l0, *l1, *l2, *r0, *r1, *r2;
    double lsl[3], rsl[3];
    if (ms == 0) {
        l0 = v0; l1 = m; l2 = v2;
        lsl[0] = half; lsl[1] = newside; lsl[2] = fcg_mod(fcg_fsub(v0, v2));
        r0 = m; r1 = v1; r2 = v2;
        rsl[0] = half; rsl[1] = fcg_mod(fcg_fsub(v2, v1)); rsl[2] = newside;
    } else if (ms == 1) {
        l0 = v1; l1 = m; l2 = v0;
        lsl[0] = half; lsl[1] = newside; lsl[2] = fcg_mod(fcg_fsub(v1, v0));
        r0 = m; r1 = v2; r2 = v0;
        rsl[0] = half; rsl[1] = fcg_mod(fcg_fsub(v0, v2)); rsl[2] = newside;
    } else {
        l0 = v2; l1 = m; l2 = v1;
        lsl[0] = half; lsl[1] = newside; lsl[2] = fcg_mod(fcg_fsub(v2, v1));
        r0 = m; r1 = v0; r2 = v1;
        rsl[0] = half; rsl[1] = fcg_mod(fcg_fsub(v1, v0)); rsl[2] = newside;
    }
    for (int k = 0; k < 3; k++) {
        Lc.v[k] = l0[k]; Lc.v[3 + k] = l1[k]; Lc.v[6 + k] = l2[k];
        Rc.v[k] = r0[k]; Rc.v[3 + k] = r1[k]; Rc.v[6 + k] = r2[k];
        Lc.n[k] = P.n[k];
        Rc.n[k] = P.n[k];
    }
    Lc.type = Rc.type = P.type;
    Lc.diel = Rc.diel = P.diel;
    Lc.area = Rc.area = P.area / 2.0;
    Lc.left = Lc.right = Rc.left = Rc.right = -1;
    fcg_centroid3(Lc);
    fcg_centroid3(Rc);
    fcg_max_side3(Lc, lsl[0], lsl[1], lsl[2]);
    fcg_max_side3(Rc, rsl[0], rsl[1], rsl[2]);
}

// One step of CAutoRefine::DiscretizeMutual (Solver/Autorefine.cpp:2638-2730):
// 0 = the pair is fine enough (c1, c2 hold its weights); 1 / 2 = refine by
// splitting the larger-area element (B on ties). For sibling pairs
// of the self pass (`selfc`) the tolerance is relaxed by the curvature
// coefficient (mesh_curv - 1) (n1.n2 + 1) + 1 of the two geometric normals.
template <class E>
FCG_HD int fcg_mesh_decision(const E &A, const E &B, bool selfc, double e, double mesh_curv, double max_side, double max_area,
                             double *c1, double *c2) {
    fcg_d3 dist;
    double rdist, rmax;
    fcg_pair_span(A, B, &dist, &rdist, &rmax);
    double ccoeff;
    if (selfc) ccoeff = (mesh_curv - 1.0) * (fcg_dot(fcg_geo_normal(A), fcg_geo_normal(B)) + 1.0) + 1.0;
    else ccoeff = 1.0;
    if (!fcg_refine_criteria(A, B, dist, rdist, rmax, e, ccoeff, max_side, max_area, c1, c2)) return 0;
    return A.area > B.area ? 1 : 2;
}

#endif
