/*
 * fastercap_gb300: C ABI of the GB300 capacitance-solve hot path.
 *
 * The entry points below replace, one for one, the in-process C++ calls the
 * reference FasterCap solver makes on its solve path. All sizes are element
 * counts, all buffers are caller-owned host memory unless stated otherwise,
 * and every function returns an FC_* status with the reference's values
 * (Solver/SolverGlobal.h:39-49). No function aborts the process.
 *
 * Data layout of a model (post-order node array, CSR links by destination):
 *   node i in [0, n_nodes): type bits, children, contiguous leaf range,
 *   links link_ptr[i] .. link_ptr[i+1]-1 with source node link_src[l];
 *   leaf j in [0, n_panels): permittivity index leaf_diel[j];
 *   conductors in solver order (dielectric interfaces first), each owning a
 *   contiguous leaf range.
 */
#ifndef FASTERCAP_GB300_H
#define FASTERCAP_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* status codes (Solver/SolverGlobal.h:39-49) */
#define FCG_NORMAL_END 0
#define FCG_GENERIC_ERROR 1
#define FCG_COMMAND_LINE_ERROR 64
#define FCG_CANNOT_OPEN_FILE 66
#define FCG_OUT_OF_MEMORY 71
#define FCG_FILE_ERROR 74
#define FCG_USER_BREAK 125
/* a CUDA call failed or no usable GPU; the message says which */
#define FCG_DEVICE_ERROR 90
/* a GMRES solve stopped at the iteration cap without converging */
#define FCG_NOT_CONVERGED 91

/* preconditioners (Solver/SolverGlobal.h:62-68) */
#define FCG_PRECOND_NONE 0
#define FCG_PRECOND_JACOBI 1
#define FCG_PRECOND_TWO_LEVEL 2 /* -ps<dim>: the reference's two-level (super) preconditioner */

/* arithmetic of the link coefficients and the link product */
#define FCG_PREC_FP64 0  /* FP64 coefficients, FP64 sums */
#define FCG_PREC_MIXED 1 /* FP32 coefficients and link sums (compensated), FP64 near field, Hessenberg and
                            Givens; the Krylov basis as fcg_solve_options.krylov says */

/* arithmetic of the Krylov basis in mixed precision (FP64 problems: always FP64) */
#define FCG_KRYLOV_PAIR 0 /* basis vectors stored as unevaluated FP32 pairs (about 46 significant bits),
                             Arnoldi dot products, updates and the solution's combination in FP32-pair
                             arithmetic (FP32 pipe) */
#define FCG_KRYLOV_FP64 1 /* basis, dot products, updates and combination in FP64 */

typedef struct fcg_context fcg_context;
typedef struct fcg_model fcg_model;
typedef struct fcg_problem fcg_problem;

/* ---------------------------------------------------------------- model */

/* Mesh and link options: -m, -d, -mc of the reference command line
 * (FasterCapConsole.cpp:136-357, CAutoRefGlobalVars Solver/SolverGlobal.h:162-183). */
typedef struct {
    double mesh_eps;  /* -m  mesh relative refinement value (default 0.1) */
    double eps_ratio; /* -d  link tolerance = eps_ratio * mesh_eps (default 1.0) */
    double mesh_curv; /* -mc mesh curvature coefficient (default 3.0) */
    int verbose;      /* -v */
} fcg_build_options;

/* Flattened model arrays. Pointers are read-only views; lengths follow the counts. */
typedef struct {
    int64_t n_nodes, n_panels, n_links;
    int32_t n_conductors;
    const uint8_t *node_type;          /* [n_nodes] bits: 1 leaf, 2 dielectric, 4 outperm on normal side, 128 super node */
    const int32_t *node_left;          /* [n_nodes] child node or -1 */
    const int32_t *node_right;         /* [n_nodes] */
    const int64_t *node_leaf_first;    /* [n_nodes] first leaf of the node's subtree */
    const int64_t *node_leaf_count;    /* [n_nodes] leaves under the node */
    const float *node_vertices;        /* [n_nodes*9] triangle corners */
    const float *node_centroid;        /* [n_nodes*3] */
    const float *node_normal;          /* [n_nodes*3] (unnormalised for super nodes) */
    const double *node_area;           /* [n_nodes] */
    const double *node_maxside;        /* [n_nodes] */
    const int64_t *link_ptr;           /* [n_nodes+1] */
    const int32_t *link_src;           /* [n_links] */
    const uint8_t *leaf_diel;          /* [n_panels] index into the conductor's outer permittivities */
    const uint8_t *cond_is_diel;       /* [n_conductors] */
    const int64_t *cond_leaf_first;    /* [n_conductors] */
    const int64_t *cond_leaf_count;    /* [n_conductors] */
    const double *cond_outperm;        /* [n_conductors] outer permittivity (dielectric: outperm side) */
    const double *cond_inperm;         /* [n_conductors] inner permittivity (dielectrics only) */
    const int32_t *cond_surf_ptr;      /* [n_conductors+1] offsets into cond_surf_outperm */
    const double *cond_surf_outperm;   /* distinct outer permittivities around each conductor */
} fcg_model_arrays;

typedef struct {
    int64_t n_nodes, n_panels, n_links, input_panels;
    int32_t n_conductors, n_dielectrics, max_level;
    double max_mesh_eps, eps, mesh_eps;
} fcg_model_info;

/* Parse a FastCap-format file and build the refined panel hierarchy and the
 * links. Replaces CAutoRefine::ReadFastCapFile + BuildSuperHierarchy
 * (Solver/Autorefine.cpp:4568, 6410), CAutoRefine::AutoRefinePanels
 * (Solver/Autorefine.cpp:293) and the link-store pass and indexing of
 * CAutoRefine::AutoRefineLinks (Solver/Autorefine.cpp:481-728). */
int fcg_model_build(const char *path, const fcg_build_options *opt, fcg_model **out, char *err, size_t err_len);
/* fcg_model_build with the link construction (the hierarchical traversal of
 * CAutoRefine::RefineMutual / RefineSelf, Solver/Autorefine.cpp:3096-3235,
 * 2115-2229, and the per-node link lists of CAutoRefine::RecurseIndex,
 * Solver/Autorefine.cpp:1173-1220) on the context's GPU. The model is
 * identical to fcg_model_build's, link order included. A NULL context
 * builds on the host. */
int fcg_model_build_on(fcg_context *ctx, const char *path, const fcg_build_options *opt, fcg_model **out, char *err,
                       size_t err_len);
int fcg_model_info_get(const fcg_model *m, fcg_model_info *info);
/* views into the model's arrays (valid until fcg_model_free) */
int fcg_model_arrays_get(const fcg_model *m, fcg_model_arrays *arrays);
/* conductor name in solver order */
const char *fcg_model_conductor_name(const fcg_model *m, int32_t index);
void fcg_model_free(fcg_model *m);

/* Structural checks of caller-built arrays (tree in post-order with
 * contiguous leaf ranges, link offsets, conductor ranges tiling the leaves,
 * permittivity indices) on the host, with the messages fcg_problem_create
 * gives: creation runs the per-node and per-leaf checks on the device
 * before any kernel indexes with the arrays, and range-checks the link
 * sources there. FCG_GENERIC_ERROR with the reason in fcg_last_error().
 * No device needed. */
int fcg_model_arrays_check(const fcg_model_arrays *arrays);

/* Concatenate independent models (geometries) into one model: a forest with
 * no link between geometries, conductors and leaves in model order.
 * geometry_of_conductor (may be NULL) receives, per conductor of the result,
 * the index of the model it came from. Used to solve many geometries with one
 * launch per kernel (fcg_problem_set_geometries). No counterpart in the
 * reference, which solves one geometry per run. */
int fcg_model_concat(const fcg_model *const *models, int32_t n_models, fcg_model **out, int32_t *geometry_of_conductor);

/* ---------------------------------------------------------------- device */

/* One GPU, its streams and the tuned launch shapes. */
int fcg_context_create(int device, fcg_context **out);
void fcg_context_destroy(fcg_context *ctx);
/* last error message of the calling thread */
const char *fcg_last_error(void);
/* the context's default CUDA stream (a cudaStream_t), used by problems
 * created with fcg_problem_create */
void *fcg_context_stream(fcg_context *ctx);

/* Upload a model once (copies the arrays to HBM). Replaces the reference's
 * in-memory link chunks m_dPotCoeffLinks / m_pdPanelPtrLinks
 * (Solver/Autorefine.h:271-272) and node array m_pNodes (Solver/Autorefine.h:283).
 * Arrays in pinned (page-locked) host memory upload fastest: the link
 * sources then go up in chunks that overlap the device-side layout work. */
int fcg_problem_create(fcg_context *ctx, const fcg_model_arrays *arrays, int precision, fcg_problem **out);
/* same, with all of the problem's work on a caller-owned CUDA stream (a
 * cudaStream_t; NULL gives the problem a stream of its own) */
int fcg_problem_create_on_stream(fcg_context *ctx, const fcg_model_arrays *arrays, int precision, void *stream,
                                 fcg_problem **out);
void fcg_problem_destroy(fcg_problem *p);
/* device bytes held by the problem */
int64_t fcg_problem_device_bytes(const fcg_problem *p);

/* Coefficient fill on the GPU: every link coefficient and the self
 * coefficients. Replaces the parallel PotEstimateOpt loop of
 * CAutoRefine::AutoRefineLinks (Solver/Autorefine.cpp:766-840) and the self
 * terms of CAutoRefine::RefineSelf / SelfPotential (Solver/Autorefine.cpp:2115-2229, 2358-2427). */
int fcg_problem_fill(fcg_problem *p);
/* copy coefficients back (FP64 values; mixed precision returns the stored FP32 values widened) */
int fcg_problem_get_coefficients(fcg_problem *p, double *link_coef, double *self_coef);

/* v = P q for k right-hand sides stored [k][n_panels] on the host.
 * Replaces CMultHier::MultiplyMatByVec_fast (Solver/MultiplyHierarchical.cpp:285-304). */
int fcg_problem_matvec(fcg_problem *p, const double *q, double *v, int k);
/* same, with q and v already in device memory */
int fcg_problem_matvec_device(fcg_problem *p, const double *d_q, double *d_v, int k);

/* Same product as fcg_problem_matvec_device for callers that must not
 * allocate device memory when they call it: hosts that reserve all device
 * memory at start-up and forbid allocation afterwards, and hosts whose device
 * memory is owned by another allocator that a cudaMalloc behind its back
 * would break. It calls no cudaMalloc, cudaFree or allocating library
 * routine; the node work arrays live in one fixed 32 MiB device array per GPU
 * (held until the process exits) instead of the problem's workspace.
 * Limit: 8*3 + 4 (mixed) or 8*3 (FP64) bytes per node and padded right-hand
 * side must fit 32 MiB, else FCG_OUT_OF_MEMORY with a message. The first call
 * on a device resolves the array's address and should come before any stream
 * capture. All calls share the array and it keeps the last call's contents
 * (the padding columns the product reads are cleared on every call): calls
 * that overlap on the GPU race and must be serialised by the caller. Runs on
 * the problem's stream and returns after the product completes; while that
 * stream records a CUDA graph it returns once the product's work is queued
 * into the graph (no wait, no profiling events), and each replay computes
 * the product of whatever d_q then holds.
 * No counterpart in the reference (FasterCap never runs without allocation). */
int fcg_problem_matvec_device_noalloc(fcg_problem *p, const double *d_q, double *d_v, int k);

/* GMRES options: -t and -p of the reference command line. */
typedef struct {
    double tol;       /* -t GMRES relative residual tolerance (default 0.01) */
    int precond;      /* FCG_PRECOND_NONE, FCG_PRECOND_JACOBI or FCG_PRECOND_TWO_LEVEL */
    int max_iter;     /* 0: the reference's cap min(1000, n_panels) */
    int rhs_width;    /* right-hand sides per batched solve: 0 = chosen by measurement (mixed problems of
                         at least 4M links; else all conductors, at most 32), 1 = one at a time */
    int precond_dim;  /* two-level dimension (the number of -ps<dim>), clamped to [16, 4096]; 0 = 128 */
    int refine;       /* restarts from the current solution while the true residual |b - A x| / |b| is
                         at or above tol: 0 = default (up to 2 for FCG_PREC_MIXED, none for FP64),
                         -1 = none, n > 0 = up to n */
    int krylov;       /* FCG_PREC_MIXED problems: FCG_KRYLOV_PAIR (0, default) or FCG_KRYLOV_FP64 */
} fcg_solve_options;

/* Declare that the problem holds several independent geometries: conductor c
 * belongs to geometry geometry_of_conductor[c]; every geometry's conductors
 * and leaves must be contiguous (as fcg_model_concat produces them). Each
 * geometry then gets its own GMRES solves (own residuals, Krylov bases,
 * iteration counts) while every product runs once over all geometries.
 * fcg_problem_solve then writes the geometries' capacitance matrices one
 * after another (geometry g: n_g x n_g over its non-dielectric conductors)
 * and iterations per geometry and conductor in the same order. */
int fcg_problem_set_geometries(fcg_problem *p, int32_t n_geometries, const int32_t *geometry_of_conductor);

/* Solve for the capacitance matrix: one right-hand side per conductor, all
 * conductors in one batched right-preconditioned GMRES, C assembled on the
 * device. cap is [n_cond x n_cond] row-major over the non-dielectric
 * conductors in solver order; iterations receives the Arnoldi step count of
 * every right-hand side (may be NULL). Replaces CSolveCap::Solve
 * (Solver/SolveCapacitance.cpp:1138-1425) with gmresPrecondSFastAll
 * (Solver/SolveCapacitance.cpp:2288-2574), the Jacobi and two-level branches
 * of ComputePrecondVectFast (Solver/SolveCapacitance.cpp:3489-3526, 3547-3598)
 * and, for the two-level preconditioner, MakePreconditioner /
 * ComputeSuperPrecond / InvertMatrix (Solver/SolveCapacitance.cpp:1061-1133,
 * 2007-2066, 2116-2258), built on the first solve that asks for it. */
int fcg_problem_solve(fcg_problem *p, const fcg_solve_options *opt, double *cap, int *iterations);
/* the charge vectors of the last batch of right-hand sides, [k][n_panels]
 * (k = the conductors of that batch, all of them up to 32) */
int fcg_problem_get_charges(fcg_problem *p, double *charges);

/* Ask a running or later solve of p to stop: it returns FCG_USER_BREAK at its
 * next Arnoldi step. Safe to call from any thread while the solve runs; the
 * flag stays set for the problem. Replaces the reference's cancellation flag
 * g_bFCContinue polled in the GMRES loop (Solver/SolveCapacitance.cpp:2365). */
int fcg_problem_cancel(fcg_problem *p);

/* Device bytes a problem of this model holds after a solve with `rhs`
 * right-hand sides (min with 32) in at most `iterations` Arnoldi steps: the
 * admission footprint used by the server below. No counterpart in the
 * reference. */
int64_t fcg_problem_estimate_bytes(const fcg_model_arrays *arrays, int precision, int rhs, int iterations);

/* Launch and timing statistics of a problem. With profiling enabled, every
 * link-product launch is bracketed by CUDA events on the problem's stream. */
typedef struct {
    int64_t kernel_launches;  /* kernels launched by the library for this problem */
    int64_t link_launches;    /* link-product (SpMV) launches */
    double link_ms;           /* summed device time of the link-product launches (profiling only) */
    int64_t link_bytes;       /* algorithmic bytes of those launches */
    double fill_ms;           /* device time of the last coefficient fill */
    double solve_ms;          /* device time of the last solve */
    int64_t refine_checks;    /* true-residual checks after GMRES (mixed precision) */
    int64_t refine_cycles;    /* GMRES restarts those checks caused */
    int64_t fill_fp64;        /* last mixed fill: near-field and self coefficients computed by the FP64
                               * formula because FP32 could not decide one of its guards */
    int64_t rhs_width;        /* right-hand sides per batched solve in the last solve (chosen by
                               * measurement when fcg_solve_options.rhs_width is 0) */
} fcg_problem_stats;
int fcg_problem_set_profiling(fcg_problem *p, int enable);
/* Measure the link product's launch shape and the right-hand-side width on
 * first use (default on; mixed problems of at least 4M links). The
 * measurement takes a few tens of launches per shape, which pays when a
 * problem (or problems of the same shape) solve many times; a problem solved
 * once can switch it off and take the built-in rules. Server jobs run with
 * it off. No counterpart in the reference. */
int fcg_problem_set_tuning(fcg_problem *p, int enable);
int fcg_problem_get_stats(fcg_problem *p, fcg_problem_stats *stats);
int fcg_problem_reset_stats(fcg_problem *p);

/* ------------------------------------------------------------ serving */

/* Extraction server on one GPU: jobs (one model each, caller-owned arrays
 * that must stay valid until the job's result is taken) are queued in
 * arrival order and admitted while a slot is free and the sum of admitted
 * footprints (fcg_problem_estimate_bytes) stays within the memory budget;
 * a job larger than the budget runs alone. Every slot is a host thread with
 * its own CUDA stream, so admitted jobs overlap on the device. A job's
 * result does not depend on what else runs (no state is shared between
 * jobs). No counterpart in the reference (one solve per process). */
typedef struct {
    int slots;              /* concurrent jobs (0: 4) */
    int64_t memory_budget;  /* bytes of admitted footprints (0: 80% of free device memory) */
    int iterations_hint;    /* Arnoldi steps assumed by the footprint (0: 64) */
} fcg_server_config;

#define FCG_JOB_QUEUED 0
#define FCG_JOB_RUNNING 1
#define FCG_JOB_DONE 2      /* finished; status in fcg_job_info */
#define FCG_JOB_CANCELLED 3

typedef struct {
    int state;              /* FCG_JOB_* */
    int status;             /* FC_* status of the solve (FCG_USER_BREAK when cancelled) */
    int n_cond;             /* capacitance matrix is n_cond x n_cond */
    int iterations_max;
    int slot;               /* slot that ran the job (-1 if it never ran) */
    int64_t footprint_bytes;
    int64_t device_bytes;   /* bytes the problem actually held */
    double queue_ms;        /* submit -> admission (host clock) */
    double run_ms;          /* admission -> result (host clock) */
    double fill_ms, solve_ms;  /* device time of fill and solve (CUDA events) */
    int64_t kernel_launches;   /* kernels the library launched for the job */
    double build_ms;           /* file jobs: model construction (host clock), part of run_ms */
    int64_t n_panels, n_links; /* size of the job's model */
} fcg_job_info;

typedef struct {
    int slots, running, queued;
    int max_running;        /* most jobs seen running at once */
    int64_t budget, in_use, peak_in_use;
    int64_t submitted, completed;
} fcg_server_stats;

typedef struct fcg_server fcg_server;
int fcg_server_create(fcg_context *ctx, const fcg_server_config *cfg, fcg_server **out);
/* waits for running jobs; queued jobs are cancelled */
void fcg_server_destroy(fcg_server *s);
int fcg_server_submit(fcg_server *s, const fcg_model_arrays *arrays, int precision, const fcg_solve_options *opt,
                      int64_t *job);
/* An extraction request as FasterCap receives one: an input file and the
 * mesh/link switches (-m, -d, -mc). The slot that takes the job builds the
 * model on the server's GPU (fcg_model_build_on: the same model as the
 * reference's ReadFastCapFile + AutoRefinePanels + AutoRefineLinks,
 * Solver/Autorefine.cpp:4568, 293, 481-728), then waits until the model's
 * footprint fits the memory budget (or nothing else holds memory) and
 * solves it like fcg_server_submit's jobs. The file is read when the job
 * starts. The job's matrix size is known once it is done (fcg_server_wait). */
int fcg_server_submit_file(fcg_server *s, const char *path, const fcg_build_options *build, int precision,
                           const fcg_solve_options *opt, int64_t *job);
/* wait until the job is done or cancelled and describe it, keeping its
 * result for fcg_server_result */
int fcg_server_wait(fcg_server *s, int64_t job, fcg_job_info *info);
/* state and timings without waiting */
int fcg_server_poll(fcg_server *s, int64_t job, fcg_job_info *info);
/* wait until the job is done or cancelled, copy its matrix (n_cond^2 values)
 * and iterations (n_cond) if not NULL, and release the job; returns the job's
 * status */
int fcg_server_result(fcg_server *s, int64_t job, double *cap, int *iterations, fcg_job_info *info);
/* a queued job is dropped; a running one stops at its next Arnoldi step */
int fcg_server_cancel(fcg_server *s, int64_t job);
int fcg_server_get_stats(fcg_server *s, fcg_server_stats *stats);

/* ------------------------------------------------------------- driver */

/* Full headless run with the reference's command line (input file and
 * switches), printing the reference's report and "Capacitance matrix is:"
 * block to stdout. Replaces FasterCapConsole::main / CSolveCap::Run
 * (FasterCapConsole.cpp:44-132, Solver/SolveCapacitance.cpp:86-256). */
int fcg_run_command_line(const char *command_line);

#ifdef __cplusplus
}
#endif

#endif
