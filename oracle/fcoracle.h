/*
 * CPU oracle for the capacitance solve hot path (test infrastructure).
 *
 * A plain-C restatement of the reference's algorithm, used only by the tests
 * (as the checker) and by the benchmark's CPU-baseline leg. It is never
 * linked into, or called by, the product library.
 *
 * Pinned against the reference itself: tests/golden holds the outputs of the
 * reference solver compiled from its own sources (oracle/Makefile,
 * oracle/ref_dump.cpp), and tests/test_oracle.py checks this oracle against
 * them (coefficients, matrix-vector products, GMRES iteration counts and the
 * capacitance matrix).
 */
#ifndef FCORACLE_H
#define FCORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct {
    int64_t n_nodes, n_panels, n_links;
    int32_t n_conductors;
    const uint8_t *node_type;
    const int32_t *node_left, *node_right;
    const int64_t *node_leaf_first, *node_leaf_count;
    const float *node_vertices, *node_centroid, *node_normal;
    const double *node_area, *node_maxside;
    const int64_t *link_ptr;
    const int32_t *link_src;
    const uint8_t *leaf_diel;
    const uint8_t *cond_is_diel;
    const int64_t *cond_leaf_first, *cond_leaf_count;
    const double *cond_outperm, *cond_inperm;
    const int32_t *cond_surf_ptr;
    const double *cond_surf_outperm;
} orc_model;

/* link and self coefficients (CAutoRefine::AutoRefineLinks fill pass and SelfPotential) */
void orc_fill(const orc_model *m, double *link_coef, double *self_coef, int threads);
/* v = P q for one vector (CMultHier::MultiplyMatByVec_fast, reference summation order) */
void orc_matvec(const orc_model *m, const double *link_coef, const double *self_coef, const double *q, double *v, int threads);
/* capacitance matrix over the non-dielectric conductors (CSolveCap::Solve + gmresPrecondSFastAll);
 * iterations[c] = Arnoldi steps of conductor c; returns 0, or 1 if some solve hit the cap */
int orc_solve(const orc_model *m, const double *link_coef, const double *self_coef, double tol, int precond, double *cap,
              int *iterations, double *charges, int threads);

/* two-level preconditioner (-ps<dim>): m super elements (nodes at depth
 * log2(dim / conductors) of every conductor's tree, or leaves above it, in
 * depth-first order), the leaf -> element map, leaf areas as float, element
 * areas and the inverse of the m x m super potential matrix (row-major) */
typedef struct {
    int32_t m;
    int64_t *elem_node;
    int32_t *sup_index;
    float *area;
    double *dim;
    double *minv;
} orc_super;
/* returns m; 0 when there are at least `dim` conductors (no two-level preconditioner) */
int orc_super_build(const orc_model *m, unsigned dim, orc_super *s);
void orc_super_free(orc_super *s);
/* orc_solve with precond 2 = two-level of dimension super_dim (falls back to
 * no preconditioner when orc_super_build returns 0) */
int orc_solve_ex(const orc_model *m, const double *link_coef, const double *self_coef, double tol, int precond,
                 unsigned super_dim, double *cap, int *iterations, double *charges, int threads);

/* orc_solve_ex for the rows row_first .. row_first + row_count - 1 of the
 * matrix only (the right-hand sides of those conductors, in solver order;
 * row_count < 0: all): cap receives row_count rows of the full width,
 * iterations and charges one entry per solved row. The reference solves its
 * conductors one after another (Solver/SolveCapacitance.cpp:1138-1425), so
 * the time of a few rows is a fixed share of a whole solve. */
int orc_solve_rows(const orc_model *m, const double *link_coef, const double *self_coef, double tol, int precond,
                   unsigned super_dim, int row_first, int row_count, double *cap, int *iterations, double *charges,
                   int threads);

#ifdef __cplusplus
}
#endif

#endif
