/*
 * CPU oracle (test infrastructure only; see fcoracle.h). Plain C restatement of:
 *   pot_opt        CPotential::PotentialOpt        Solver/Potential.cpp:1561-1711
 *   pot_num        CPotential::PotentialNumerical  Solver/Potential.cpp:2077-2153
 *   efield_num     CPotential::EnFieldNumerical    Solver/Potential.cpp:2172-2254
 *   rules 2,3,5    CPotential::InitNumerical       Solver/Potential.cpp:112-128,133-149,181-206
 *   pot_estimate   CAutoRefine::PotEstimateOpt     Solver/Autorefine.cpp:3474-3733
 *   self_pot       CAutoRefine::SelfPotential      Solver/Autorefine.cpp:2358-2427
 *   orc_matvec     CMultHier::MultiplyMatByVec_fast and its three passes
 *                                                  Solver/MultiplyHierarchical.cpp:72-304
 *   gmres          CSolveCap::gmresPrecondSFastAll Solver/SolveCapacitance.cpp:2288-2574
 *   precond        CSolveCap::ComputePrecondVectFast (none / Jacobi / two-level)
 *                                                  Solver/SolveCapacitance.cpp:3458-3598
 *   orc_super_build  two-level preconditioner setup: CSolveCap::MakePreconditioner,
 *                  RecurseComputePrecond, ComputeSuperPrecond, InvertMatrix
 *                                                  Solver/SolveCapacitance.cpp:1061-1133,1876-2066,2116-2258
 *   orc_solve      CSolveCap::Solve                Solver/SolveCapacitance.cpp:1138-1425
 * Vector arithmetic follows the conventions used to compile the reference
 * here: a difference of two single-precision vertices is formed in single
 * precision and widened; everything else is double. Sums are in the
 * reference's order, so results match the reference's own binary bit for bit
 * on the same machine.
 */
#include "fcoracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define FOUR_PI_E0 1.1126500559756e-10
#define TWO_E0 1.7708375634e-11
#define GEO_EPS 1E-6
#define PANEL_EPS 1E-12
#define T_LEAF 1u
#define T_DIEL 2u
#define T_NORMAL_DIR 4u
#define T_SUPER 128u
#define GMRES_ITER_MAX 1000

typedef struct { double x, y, z; } v3;

static v3 mk(double x, double y, double z) { v3 r; r.x = x; r.y = y; r.z = z; return r; }
static v3 wid(const float *f) { return mk(f[0], f[1], f[2]); }
static v3 fsub(const float *a, const float *b) {
    float x = a[0] - b[0], y = a[1] - b[1], z = a[2] - b[2];
    return mk(x, y, z);
}
static double vmod(v3 a) { return sqrt(a.x * a.x + a.y * a.y + a.z * a.z); }
static double vdot(v3 a, v3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }

static double pot_opt(v3 r, const float *vt) {
    v3 side[3], n, rho, Pmp[3], Rmp[3], l, u;
    double Rn[3], result = 0.0;
    int i;
    side[0] = fsub(vt + 3, vt);
    side[1] = fsub(vt + 6, vt + 3);
    side[2] = fsub(vt, vt + 6);
    n = mk(side[0].y * side[1].z - side[0].z * side[1].y, side[0].z * side[1].x - side[0].x * side[1].z,
           side[0].x * side[1].y - side[0].y * side[1].x);
    double nmod = vmod(n);
    n.x = n.x / nmod; n.y = n.y / nmod; n.z = n.z / nmod;
    double nr = vdot(n, r);
    rho = mk(r.x - n.x * nr, r.y - n.y * nr, r.z - n.z * nr);
    for (i = 0; i < 3; i++) {
        v3 vi = wid(vt + 3 * i);
        double nv = vdot(n, vi);
        v3 rh = mk(vi.x - n.x * nv, vi.y - n.y * nv, vi.z - n.z * nv);
        Pmp[i] = mk(rh.x - rho.x, rh.y - rho.y, rh.z - rho.z);
        Rmp[i] = mk(vi.x - r.x, vi.y - r.y, vi.z - r.z);
        Rn[i] = vmod(Rmp[i]);
    }
    double d = -vdot(n, Rmp[0]), dn = fabs(d);
    for (i = 0; i < 3; i++) {
        int j = i == 2 ? 0 : i + 1;
        double ms = vmod(side[i]);
        l = mk(side[i].x / ms, side[i].y / ms, side[i].z / ms);
        u = mk(l.y * n.z - l.z * n.y, l.z * n.x - l.x * n.z, l.x * n.y - l.y * n.x);
        double P0s = vdot(Pmp[j], u), P0 = fabs(P0s);
        double lp = vdot(Pmp[j], l), lm = vdot(Pmp[i], l);
        double R0 = sqrt(P0 * P0 + d * d);
        double lmax = lp > lm ? fabs(lp) : fabs(lm);
        if (P0 / lmax > GEO_EPS && fabs((Rn[j] + lp) / lmax) > GEO_EPS && fabs((Rn[i] + lm) / lmax) > GEO_EPS) {
            double R02 = R0 * R0;
            double t1 = atan(P0 * lp / (R02 + dn * Rn[j]));
            double t2 = atan(P0 * lm / (R02 + dn * Rn[i]));
            double ln = log((Rn[j] + lp) / (Rn[i] + lm));
            double sg = (double)((P0s > 0) - (P0s < 0));
            result += sg * (P0 * ln - dn * (t1 - t2));
        }
    }
    return (result * 2.0) / nmod;
}

static void rule(int r, int i, double *px, double *py, double *w) {
    if (r == 2) {
        double a = 1.0, b = 3.0, c = 4.0, dd = 6.0;
        double xs[3] = {c / dd, a / dd, a / dd}, ys[3] = {a / dd, c / dd, a / dd};
        *px = xs[i]; *py = ys[i]; *w = a / b;
    } else if (r == 3) {
        double xs[3] = {0.0, 0.5, 0.5}, ys[3] = {0.5, 0.0, 0.5};
        *px = xs[i]; *py = ys[i]; *w = 1.0 / 3.0;
    } else {
        double a = 0.659027622374092, b = 0.231933368553031, c = 0.109039009072877;
        double xs[6] = {a, a, b, b, c, c}, ys[6] = {b, c, a, c, a, b};
        *px = xs[i]; *py = ys[i]; *w = 1.0 / 6.0;
    }
}

/* kind 0: potential 1/|p-r|; kind 1: field (r-p).tn/|r-p|^3 */
static double quad(v3 r, const float *vt, int rl, int kind, v3 tn) {
    v3 s1 = fsub(vt + 3, vt), s2 = fsub(vt + 6, vt + 3), s3 = fsub(vt, vt + 6), nrm, z, x, y;
    nrm.x = s1.y * s2.z - s1.z * s2.y;
    nrm.y = -s1.x * s2.z + s1.z * s2.x;
    nrm.z = s1.x * s2.y - s1.y * s2.x;
    double mn = vmod(nrm);
    z = mk(nrm.x / mn, nrm.y / mn, nrm.z / mn);
    double m1 = vmod(s1);
    x = mk(s1.x / m1, s1.y / m1, s1.z / m1);
    y = mk(x.y * z.z - x.z * z.y, x.z * z.x - x.x * z.z, x.x * z.y - x.y * z.x);
    double a01 = m1;
    double a02 = -(s3.x * x.x + s3.y * x.y + s3.z * x.z);
    double a12 = -(s3.x * y.x + s3.y * y.y + s3.z * y.z);
    double jac = (a02 - a01) * a12 - a12 * a02;
    double res = 0.0;
    int np = rl == 5 ? 6 : 3, i;
    for (i = 0; i < np; i++) {
        double px, py, w;
        rule(rl, i, &px, &py, &w);
        double p0 = (a01 - a02) * px + a02 * (1.0 - py);
        double p1 = a12 * (1.0 - px - py);
        v3 p = mk((double)vt[0] + x.x * p0 + y.x * p1, (double)vt[1] + x.y * p0 + y.y * p1, (double)vt[2] + x.z * p0 + y.z * p1);
        double val;
        if (kind == 0) {
            val = 1 / vmod(mk(p.x - r.x, p.y - r.y, p.z - r.z));
        } else {
            v3 dd = mk(r.x - p.x, r.y - p.y, r.z - p.z);
            double rd = vmod(dd);
            val = vdot(dd, tn) / (rd * rd * rd);
        }
        res += w * val;
    }
    res *= jac / 2.0;
    res /= mn / 2.0;
    return res;
}

static v3 diel_normal(unsigned t, const float *n) {
    v3 u;
    if (t & T_SUPER) {
        v3 w = wid(n);
        double m = vmod(w);
        u = m < PANEL_EPS ? mk(0, 0, 0) : mk(w.x / m, w.y / m, w.z / m);
    } else {
        u = wid(n);
    }
    if ((t & T_NORMAL_DIR) != T_NORMAL_DIR) u = mk(-u.x, -u.y, -u.z);
    return u;
}

static double pot_estimate(const orc_model *m, int64_t i, int64_t j) {
    const float *c1 = m->node_centroid + 3 * i, *c2 = m->node_centroid + 3 * j, *v2 = m->node_vertices + 9 * j;
    unsigned t1 = m->node_type[i];
    v3 dist = fsub(c1, c2);
    double rd = vmod(dist);
    double r1 = m->node_maxside[i], r2 = m->node_maxside[j];
    double rmax = r1 > r2 ? r1 : r2;
    v3 p1 = wid(c1), zero = mk(0, 0, 0);
    if ((t1 & T_DIEL) != T_DIEL) {
        if (rd / rmax < 1.0) return pot_opt(p1, v2) / FOUR_PI_E0;
        if (rd / rmax < 2.0) return quad(p1, v2, 5, 0, zero) / FOUR_PI_E0;
        if (rd / rmax < 4.0) return quad(p1, v2, 3, 0, zero) / FOUR_PI_E0;
        if (rd / rmax < 10.0) return quad(p1, v2, 2, 0, zero) / FOUR_PI_E0;
        return 1 / (FOUR_PI_E0 * rd);
    }
    v3 n1 = diel_normal(t1, m->node_normal + 3 * i);
    if (rd / rmax < 1.0) {
        double h = rd / 20;
        v3 ep = mk(p1.x + n1.x * h, p1.y + n1.y * h, p1.z + n1.z * h);
        v3 em = mk(p1.x - n1.x * h, p1.y - n1.y * h, p1.z - n1.z * h);
        double pp = pot_opt(ep, v2), pn = pot_opt(em, v2);
        return (pn - pp) / (2 * h * FOUR_PI_E0);
    }
    if (rd / rmax < 2.0) return quad(p1, v2, 5, 1, n1) / FOUR_PI_E0;
    if (rd / rmax < 4.0) return quad(p1, v2, 3, 1, n1) / FOUR_PI_E0;
    if (rd / rmax < 10.0) return quad(p1, v2, 2, 1, n1) / FOUR_PI_E0;
    return vdot(dist, n1) / (FOUR_PI_E0 * rd * rd * rd);
}

static int32_t *leaf_nodes(const orc_model *m) {
    int32_t *ln = (int32_t *)malloc(sizeof(int32_t) * (size_t)m->n_panels);
    int64_t i;
    for (i = 0; i < m->n_nodes; i++)
        if (m->node_type[i] & T_LEAF) ln[m->node_leaf_first[i]] = (int32_t)i;
    return ln;
}

void orc_fill(const orc_model *m, double *coef, double *self, int threads) {
    int64_t i;
#ifdef _OPENMP
    if (threads > 0) omp_set_num_threads(threads);
#else
    (void)threads;
#endif
#pragma omp parallel for schedule(dynamic, 64)
    for (i = 0; i < m->n_nodes; i++) {
        int64_t l;
        for (l = m->link_ptr[i]; l < m->link_ptr[i + 1]; l++) coef[l] = pot_estimate(m, i, m->link_src[l]);
    }
    int32_t *ln = leaf_nodes(m);
    int32_t c;
    for (c = 0; c < m->n_conductors; c++) {
        int64_t j;
        for (j = m->cond_leaf_first[c]; j < m->cond_leaf_first[c] + m->cond_leaf_count[c]; j++) {
            int64_t nd = ln[j];
            if (m->node_type[nd] & T_DIEL) {
                double eb = m->cond_outperm[c], ea = m->cond_inperm[c];
                self[j] = (ea + eb) / (TWO_E0 * (eb - ea) * m->node_area[nd]);
            } else {
                self[j] = pot_opt(wid(m->node_centroid + 3 * nd), m->node_vertices + 9 * nd) / FOUR_PI_E0;
            }
        }
    }
    free(ln);
}

/* work arrays: charge and potential per node */
static void matvec_ws(const orc_model *m, const double *coef, const double *self, const double *q, double *v,
                      double *chg, double *pot) {
    int64_t i, Nn = m->n_nodes;
    /* up-sweep: post-order, children first */
    for (i = 0; i < Nn; i++) {
        if (m->node_type[i] & T_LEAF) {
            int64_t j = m->node_leaf_first[i];
            chg[i] = q[j];
            pot[i] = self[j] * chg[i];
        } else {
            chg[i] = chg[m->node_left[i]] + chg[m->node_right[i]];
            pot[i] = 0.0;
        }
    }
    /* link sums in stored order */
#pragma omp parallel for schedule(dynamic, 256)
    for (i = 0; i < Nn; i++) {
        int64_t l;
        double p = pot[i];
        for (l = m->link_ptr[i]; l < m->link_ptr[i + 1]; l++) p += chg[m->link_src[l]] * coef[l];
        pot[i] = p;
    }
    /* down-sweep: parents before children */
    for (i = Nn - 1; i >= 0; i--) {
        if (!(m->node_type[i] & T_LEAF)) {
            pot[m->node_left[i]] += pot[i];
            pot[m->node_right[i]] += pot[i];
        } else {
            v[m->node_leaf_first[i]] = pot[i];
        }
    }
}

void orc_matvec(const orc_model *m, const double *coef, const double *self, const double *q, double *v, int threads) {
#ifdef _OPENMP
    if (threads > 0) omp_set_num_threads(threads);
#else
    (void)threads;
#endif
    double *chg = (double *)malloc(sizeof(double) * (size_t)m->n_nodes);
    double *pot = (double *)malloc(sizeof(double) * (size_t)m->n_nodes);
    matvec_ws(m, coef, self, q, v, chg, pot);
    free(chg);
    free(pot);
}

static double norm2(const double *a, int64_t n) {
    double s = 0.0;
    int64_t i;
    for (i = 0; i < n; i++) s += a[i] * a[i];
    return sqrt(s);
}

/* ---- two-level preconditioner setup */

static void super_visit(const orc_model *m, int64_t v, int d, int lev, orc_super *s) {
    int leaf = (m->node_type[v] & T_LEAF) != 0;
    if ((leaf && d <= lev) || (!leaf && d == lev)) {
        s->elem_node[s->m++] = v;
        return;
    }
    super_visit(m, m->node_left[v], d + 1, lev, s);
    super_visit(m, m->node_right[v], d + 1, lev, s);
}

static void lu_inverse(double *a, double *inv, int32_t n) {
    /* LU factorisation with partial pivoting, in place (right-looking, one
     * rank-1 update per column), then the inverse column by column by forward
     * and backward substitution (InvertMatrix, Solver/SolveCapacitance.cpp:2116-2258) */
    int32_t *piv = (int32_t *)malloc(sizeof(int32_t) * (size_t)n);
    double *col = (double *)malloc(sizeof(double) * (size_t)n);
    int32_t j, i, k;
    for (j = 0; j < n; j++) {
        int32_t p = j;
        double best = fabs(a[(size_t)j * n + j]);
        for (i = j + 1; i < n; i++)
            if (fabs(a[(size_t)i * n + j]) > best) { p = i; best = fabs(a[(size_t)i * n + j]); }
        piv[j] = p;
        if (p != j)
            for (k = 0; k < n; k++) {
                double t = a[(size_t)j * n + k];
                a[(size_t)j * n + k] = a[(size_t)p * n + k];
                a[(size_t)p * n + k] = t;
            }
        if (j < n - 1) {
            double r = 1.0 / a[(size_t)j * n + j];
            for (i = j + 1; i < n; i++) a[(size_t)i * n + j] *= r;
            for (i = j + 1; i < n; i++)
                for (k = j + 1; k < n; k++) a[(size_t)i * n + k] -= a[(size_t)i * n + j] * a[(size_t)j * n + k];
        }
    }
    for (k = 0; k < n; k++) {
        for (i = 0; i < n; i++) col[i] = 0.0;
        col[k] = 1.0;
        for (i = 0; i < n; i++) { /* the row swaps, in factorisation order */
            double t = col[i];
            col[i] = col[piv[i]];
            col[piv[i]] = t;
        }
        for (i = 0; i < n; i++) { /* unit lower triangle */
            double sum = col[i];
            for (j = 0; j < i; j++) sum -= a[(size_t)i * n + j] * col[j];
            col[i] = sum;
        }
        for (i = n - 1; i >= 0; i--) { /* upper triangle */
            double sum = col[i];
            for (j = i + 1; j < n; j++) sum -= a[(size_t)i * n + j] * col[j];
            col[i] = sum / a[(size_t)i * n + i];
        }
        for (i = 0; i < n; i++) inv[(size_t)i * n + k] = col[i];
    }
    free(piv);
    free(col);
}

int orc_super_build(const orc_model *m, unsigned dim, orc_super *s) {
    int64_t i, j;
    int32_t c, *parent;
    memset(s, 0, sizeof *s);
    if (dim > 4096) dim = 4096;
    if (dim < 16) dim = 16;
    if ((unsigned)m->n_conductors >= dim) return 0;
    int lev = (int)(unsigned)(log((double)(dim / (unsigned)m->n_conductors)) / log(2.0));
    s->elem_node = (int64_t *)malloc(sizeof(int64_t) * 4096);
    parent = (int32_t *)malloc(sizeof(int32_t) * (size_t)m->n_nodes);
    for (i = 0; i < m->n_nodes; i++) parent[i] = -1;
    for (i = 0; i < m->n_nodes; i++)
        if (!(m->node_type[i] & T_LEAF)) { parent[m->node_left[i]] = (int32_t)i; parent[m->node_right[i]] = (int32_t)i; }
    /* each conductor's tree, in conductor order (roots in leaf order) */
    for (c = 0; c < m->n_conductors; c++)
        for (i = 0; i < m->n_nodes; i++)
            if (parent[i] < 0 && m->node_leaf_first[i] == m->cond_leaf_first[c]) { super_visit(m, i, 0, lev, s); break; }
    free(parent);
    int32_t mm = s->m;
    s->sup_index = (int32_t *)malloc(sizeof(int32_t) * (size_t)m->n_panels);
    s->area = (float *)malloc(sizeof(float) * (size_t)m->n_panels);
    s->dim = (double *)malloc(sizeof(double) * (size_t)mm);
    int32_t *ln = leaf_nodes(m);
    for (i = 0; i < mm; i++) {
        int64_t v = s->elem_node[i];
        s->dim[i] = m->node_area[v];
        for (j = m->node_leaf_first[v]; j < m->node_leaf_first[v] + m->node_leaf_count[v]; j++) s->sup_index[j] = (int32_t)i;
    }
    for (j = 0; j < m->n_panels; j++) s->area[j] = (float)m->node_area[ln[j]];
    free(ln);
    /* super potential matrix: self terms on the diagonal, the one-way
     * estimate both ways off it (ComputeSuperPrecond) */
    double *pm = (double *)malloc(sizeof(double) * (size_t)mm * mm);
    s->minv = (double *)malloc(sizeof(double) * (size_t)mm * mm);
    for (i = 0; i < mm; i++) {
        int64_t v = s->elem_node[i];
        for (c = 0; c < m->n_conductors; c++)
            if (m->node_leaf_first[v] >= m->cond_leaf_first[c] &&
                m->node_leaf_first[v] < m->cond_leaf_first[c] + m->cond_leaf_count[c]) break;
        if (m->node_type[v] & T_DIEL) {
            double eb = m->cond_outperm[c], ea = m->cond_inperm[c];
            pm[(size_t)i * mm + i] = (ea + eb) / (TWO_E0 * (eb - ea) * m->node_area[v]);
        } else {
            pm[(size_t)i * mm + i] = pot_opt(wid(m->node_centroid + 3 * v), m->node_vertices + 9 * v) / FOUR_PI_E0;
        }
        for (j = i + 1; j < mm; j++) {
            pm[(size_t)i * mm + j] = pot_estimate(m, v, s->elem_node[j]);
            pm[(size_t)j * mm + i] = pot_estimate(m, s->elem_node[j], v);
        }
    }
    lu_inverse(pm, s->minv, mm);
    free(pm);
    return mm;
}

void orc_super_free(orc_super *s) {
    free(s->elem_node); free(s->sup_index); free(s->area); free(s->dim); free(s->minv);
    memset(s, 0, sizeof *s);
}

/* two-level preconditioner product (ComputePrecondVectFast, super branch,
 * Solver/SolveCapacitance.cpp:3547-3598): leaf values are averaged into their
 * super element by area, multiplied by the inverse super potential matrix
 * without its diagonal, spread back by area, plus the diagonal term per leaf */
static void super_apply(const orc_super *sp, const double *q, double *out, int64_t n) {
    int32_t mm = sp->m, i, k;
    int64_t j;
    double *pot = (double *)calloc((size_t)mm, sizeof(double)), *chg = (double *)calloc((size_t)mm, sizeof(double));
    for (j = 0; j < n; j++) {
        int32_t e = sp->sup_index[j];
        pot[e] += q[j] * (double)sp->area[j] / sp->dim[e];
    }
    for (i = 0; i < mm; i++)
        for (k = 0; k < mm; k++)
            if (i != k) chg[i] += sp->minv[(size_t)i * mm + k] * pot[k];
    for (j = 0; j < n; j++) {
        int32_t e = sp->sup_index[j];
        out[j] = chg[e] * (double)sp->area[j] / sp->dim[e];
        out[j] += sp->minv[(size_t)e * mm + e] * q[j] * (double)sp->area[j] / sp->dim[e];
    }
    free(pot);
    free(chg);
}

/* pc: 0 none, 1 Jacobi, 2 two-level (sp) */
static void precond(int pc, const double *self, const orc_super *sp, const double *q, double *out, int64_t n) {
    int64_t i;
    if (pc == 2) { super_apply(sp, q, out, n); return; }
    for (i = 0; i < n; i++) out[i] = pc ? q[i] / self[i] : q[i];
}

/* returns the index of the last Arnoldi step (-1 if x0 was accepted); *capped set on non-convergence */
static int gmres(const orc_model *m, const double *coef, const double *self, const orc_super *sp, const double *b, double *x,
                 double tol, int pc, int *capped, double *chg, double *pot) {
    int64_t n = m->n_panels, k;
    int maxit = GMRES_ITER_MAX < n ? GMRES_ITER_MAX : (int)n;
    double *x0 = (double *)calloc((size_t)n, sizeof(double));
    double *vv = (double *)malloc(sizeof(double) * (size_t)n), *w = (double *)malloc(sizeof(double) * (size_t)n);
    double *rr = (double *)malloc(sizeof(double) * (size_t)n), *Pq = (double *)malloc(sizeof(double) * (size_t)n);
    double **Q = (double **)calloc((size_t)maxit + 1, sizeof(double *));
    double **H = (double **)calloc((size_t)maxit + 1, sizeof(double *));
    double *c = (double *)calloc((size_t)maxit + 2, sizeof(double)), *s = (double *)calloc((size_t)maxit + 2, sizeof(double));
    double *g = (double *)calloc((size_t)maxit + 2, sizeof(double)), *z = (double *)calloc((size_t)maxit + 2, sizeof(double));
    double normr, normb;
    int i, j, iteration;
    *capped = 0;
    if (pc) {
        precond(pc, self, sp, b, x0, n);
        matvec_ws(m, coef, self, x0, vv, chg, pot);
        for (k = 0; k < n; k++) rr[k] = b[k] - vv[k];
        normr = norm2(rr, n);
        normb = norm2(b, n);
    } else {
        memcpy(rr, b, sizeof(double) * (size_t)n);
        normr = norm2(rr, n);
        normb = normr;
    }
    Q[0] = (double *)malloc(sizeof(double) * (size_t)n);
    for (k = 0; k < n; k++) Q[0][k] = rr[k] / normr;
    g[0] = normr;
    if (normr / normb < tol) {
        memcpy(x, x0, sizeof(double) * (size_t)n);
        iteration = -1;
        goto done;
    }
    for (i = 0; i < GMRES_ITER_MAX && i < n; i++) {
        H[i] = (double *)calloc((size_t)i + 2, sizeof(double));
        Q[i + 1] = (double *)malloc(sizeof(double) * (size_t)n);
        if (pc) {
            precond(pc, self, sp, Q[i], Pq, n);
            matvec_ws(m, coef, self, Pq, vv, chg, pot);
        } else {
            matvec_ws(m, coef, self, Q[i], vv, chg, pot);
        }
        memcpy(w, vv, sizeof(double) * (size_t)n);
        for (j = 0; j <= i; j++) {
            double d = 0.0;
            for (k = 0; k < n; k++) d += Q[j][k] * w[k];
            H[i][j] = d;
            for (k = 0; k < n; k++) vv[k] = vv[k] - H[i][j] * Q[j][k];
        }
        H[i][i + 1] = norm2(vv, n);
        for (k = 0; k < n; k++) Q[i + 1][k] = vv[k] / H[i][i + 1];
        for (j = 0; j < i; j++) {
            double t1 = H[i][j], t2 = H[i][j + 1];
            H[i][j] = c[j] * t1 - s[j] * t2;
            H[i][j + 1] = c[j] * t2 + s[j] * t1;
        }
        {
            double t1 = H[i][i], t2 = H[i][i + 1];
            double len = sqrt(t1 * t1 + t2 * t2);
            c[i] = t1 / len;
            s[i] = -t2 / len;
            H[i][i] = c[i] * t1 - s[i] * t2;
            H[i][i + 1] = 0;
            t1 = g[i];
            g[i] = c[i] * t1;
            g[i + 1] = s[i] * t1;
        }
        normr = fabs(g[i + 1]) / normb;
        if (normr < tol) break;
    }
    if (i >= GMRES_ITER_MAX || i >= n) {
        *capped = 1;
        i--;
    }
    iteration = i;
    for (j = 0; j <= iteration; j++) z[j] = g[j];
    for (i = iteration; i >= 0; i--) {
        z[i] = z[i] / H[i][i];
        for (j = i - 1; j >= 0; j--) z[j] = z[j] - H[i][j] * z[i];
    }
    for (k = 0; k < n; k++) {
        double t = 0.0;
        for (j = 0; j <= iteration; j++) t += Q[j][k] * z[j];
        vv[k] = t;
    }
    if (pc) {
        precond(pc, self, sp, vv, x, n);
        for (k = 0; k < n; k++) x[k] = x0[k] + x[k];
    } else {
        memcpy(x, vv, sizeof(double) * (size_t)n);
    }
done:
    for (i = 0; i <= maxit; i++) { free(Q[i]); free(H[i]); }
    free(Q); free(H); free(c); free(s); free(g); free(z);
    free(x0); free(vv); free(w); free(rr); free(Pq);
    return iteration;
}

int orc_solve_rows(const orc_model *m, const double *coef, const double *self, double tol, int pc, unsigned super_dim,
                   int row_first, int row_count, double *cap, int *iterations, double *charges, int threads) {
#ifdef _OPENMP
    if (threads > 0) omp_set_num_threads(threads);
#else
    (void)threads;
#endif
    int64_t n = m->n_panels;
    double *b = (double *)calloc((size_t)n, sizeof(double)), *x = (double *)malloc(sizeof(double) * (size_t)n);
    double *chg = (double *)malloc(sizeof(double) * (size_t)m->n_nodes), *pot = (double *)malloc(sizeof(double) * (size_t)m->n_nodes);
    int ncol = 0, row = 0, any_capped = 0;
    orc_super sp;
    memset(&sp, 0, sizeof sp);
    if (pc == 2 && orc_super_build(m, super_dim, &sp) == 0) pc = 0;  /* too many roots: no preconditioner */
    int32_t c, c2;
    for (c = 0; c < m->n_conductors; c++) ncol += m->cond_is_diel[c] ? 0 : 1;
    if (row_count < 0) row_count = ncol;
    int out = 0;  /* rows written so far */
    for (c = 0; c < m->n_conductors; c++) {
        int64_t j;
        int capped, col = 0;
        if (m->cond_is_diel[c]) continue;
        if (row < row_first || row >= row_first + row_count) { row++; continue; }
        for (j = m->cond_leaf_first[c]; j < m->cond_leaf_first[c] + m->cond_leaf_count[c]; j++) b[j] = 1.0;
        int it = gmres(m, coef, self, &sp, b, x, tol, pc, &capped, chg, pot);
        any_capped |= capped;
        if (iterations) iterations[out] = it + 1;
        if (charges) memcpy(charges + (size_t)out * n, x, sizeof(double) * (size_t)n);
        for (c2 = 0; c2 < m->n_conductors; c2++) {
            double acc = 0.0;
            if (m->cond_is_diel[c2]) continue;
            for (j = m->cond_leaf_first[c2]; j < m->cond_leaf_first[c2] + m->cond_leaf_count[c2]; j++)
                acc += m->cond_surf_outperm[m->cond_surf_ptr[c2] + m->leaf_diel[j]] * x[j];
            cap[(size_t)out * ncol + col] = acc;
            col++;
        }
        for (j = m->cond_leaf_first[c]; j < m->cond_leaf_first[c] + m->cond_leaf_count[c]; j++) b[j] = 0.0;
        row++;
        out++;
    }
    free(b); free(x); free(chg); free(pot);
    orc_super_free(&sp);
    return any_capped;
}

int orc_solve_ex(const orc_model *m, const double *coef, const double *self, double tol, int pc, unsigned super_dim,
                 double *cap, int *iterations, double *charges, int threads) {
    return orc_solve_rows(m, coef, self, tol, pc, super_dim, 0, -1, cap, iterations, charges, threads);
}

int orc_solve(const orc_model *m, const double *coef, const double *self, double tol, int pc, double *cap, int *iterations,
              double *charges, int threads) {
    return orc_solve_ex(m, coef, self, tol, pc, 0, cap, iterations, charges, threads);
}
