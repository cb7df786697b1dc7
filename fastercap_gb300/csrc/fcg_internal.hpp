// Internal interfaces between the C ABI layer (host/api.cpp) and the device
// solver (csrc/problem.cu). Not installed; not part of the public header.
#ifndef FCG_INTERNAL_HPP
#define FCG_INTERNAL_HPP

#include <stdint.h>
#include <atomic>
#include <map>
#include <mutex>
#include <vector>
#include <memory>
#include <string>
#include <vector>

#include "../../include/fastercap_gb300.h"

namespace fcg {

// thread-local last error message
void set_error(const std::string &msg);
const char *get_error();

struct DeviceProblem;

// device context: one GPU
struct DeviceContext {
    int device = 0;
    int sm_count = 0;
    size_t smem_optin = 0;  // shared memory a CTA may opt into (bytes)
    size_t free_bytes = 0, total_bytes = 0;
    void *stream = nullptr;  // cudaStream_t owned by the context
    // the handle and every problem created on the context hold a reference;
    // the GPU resources go when the last one is dropped
    std::atomic<int> refs{1};
    // pinned host words for per-iteration readbacks, one 64-byte slot per
    // problem (allocated once: page-locked allocation synchronises the device)
    int *pin = nullptr;
    std::mutex pin_mu;
    std::vector<int> pin_free;
    // link-product launch shapes chosen by measurement, per problem shape
    std::mutex tune_mu;
    std::map<uint64_t, int> tune;
    // pinned staging buffers for uploads from pageable host memory (taken
    // two at a time by a problem creation, allocated on first need)
    std::mutex stage_mu;
    std::vector<void *> stage_free;
    int stage_count = 0;
};
void context_release(DeviceContext &ctx);
void context_unref(DeviceContext *ctx);

int context_init(DeviceContext &ctx, int device);

// structural checks of a model's arrays ("" when valid); no device work
std::string model_check(const fcg_model_arrays &a);

// problem lifetime
int problem_create(DeviceContext &ctx, const fcg_model_arrays &a, int precision, void *stream, DeviceProblem **out);
void problem_destroy(DeviceProblem *p);
int64_t problem_device_bytes(const DeviceProblem *p);
int problem_fill(DeviceProblem *p);
int problem_get_coefficients(DeviceProblem *p, double *link_coef, double *self_coef);
int problem_matvec_host(DeviceProblem *p, const double *q, double *v, int k);
int problem_matvec_device(DeviceProblem *p, const double *d_q, double *d_v, int k);
int problem_matvec_noalloc(DeviceProblem *p, const double *d_q, double *d_v, int k);
// all_charges (optional, host, one geometry): every conductor's charge
// vector, [conductors][n_panels], copied as its batch ends
int problem_solve(DeviceProblem *p, const fcg_solve_options &opt, double *cap, int *iterations, double *all_charges = nullptr);
int problem_get_charges(DeviceProblem *p, double *charges);
int problem_set_geometries(DeviceProblem *p, int n, const int32_t *geom_of_cond);
int problem_n_cond(const DeviceProblem *p);
// request cancellation: the solve returns FCG_USER_BREAK at its next Arnoldi step
void problem_cancel(DeviceProblem *p);
// device bytes a problem of this model will hold after a solve of `rhs`
// right-hand sides in at most `iterations` Arnoldi steps
int64_t problem_estimate_bytes(const fcg_model_arrays &a, int precision, int rhs, int iterations);

// Link construction on the device (csrc/link_build.cu): the traversal of
// the element hierarchy `el` from the root pairs (root_a[i], root_b[i]),
// visited at recursion level root_level[i], in the host builder's order;
// node_of maps element ids to node ids. Fills link_ptr (n_nodes + 1) and
// link_src exactly as the host traversal and its stable bucketing do, and
// max_level with the deepest recursion level of the traversal. With
// device_src the link sources stay in device memory (complete when the call
// returns; freed with the last reference) and link_src is left empty.
struct Element;
int link_build_device(DeviceContext &ctx, const Element *el, int64_t ne, const int32_t *root_a, const int32_t *root_b,
                      const uint16_t *root_level, int64_t n_roots, const int32_t *node_of, int64_t n_nodes, double eps,
                      double max_side, double max_area, std::vector<int64_t> &link_ptr, std::vector<int32_t> &link_src,
                      int &max_level, std::string &err, std::shared_ptr<int32_t> *device_src = nullptr);

// Mesh refinement on the device (csrc/mesh_build.cu): the closure of the
// refinement of the root pairs (root_a[i], root_b[i]) with root_meta[i] =
// recursion level | kMeshSelfPair for pairs of the self pass. `el` (with
// `depth`, every element's depth in its conductor's tree) is replaced by the
// refined hierarchy; max_mesh_eps and max_level receive the largest weight of
// an unrefined pair and the deepest pair level.
constexpr uint16_t kMeshSelfPair = 0x8000;
int mesh_refine_device(DeviceContext &ctx, std::vector<Element> &el, const std::vector<int32_t> &depth,
                       const std::vector<int32_t> &root_a, const std::vector<int32_t> &root_b,
                       const std::vector<uint16_t> &root_meta, double mesh_eps, double mesh_curv, double max_side,
                       double max_area, double &max_mesh_eps, int &max_level, std::string &err);

// Super hierarchy on the device (csrc/super_build.cu): every conductor's
// panels (element ids in `el`, conductors in solver order) split by the host
// recursion's mid-plane rule, the super nodes appended to `el` (made by
// fcg_make_super, the same elements as the host's) and tops[k] set to
// conductor k's root element. FC_FILE_ERROR (with err) for coincident
// centroids or a tree deeper than max_depth.
int super_build_device(DeviceContext &ctx, std::vector<Element> &el, const std::vector<std::vector<int32_t>> &panels,
                       std::vector<int32_t> &tops, int max_depth, std::string &err);

// CUDA streams for host code compiled without the CUDA headers
void *stream_create(int device);
void stream_destroy(int device, void *stream);

// timings of the last fill / solve in milliseconds (CUDA events on the problem's stream)
struct SolveTimings {
    float fill_ms = 0, solve_ms = 0, assemble_ms = 0;
    int iterations_max = 0;
    int64_t refine_checks = 0, refine_cycles = 0;  // true-residual checks, restarts they caused
    int64_t fill_fp64 = 0;  // mixed fill: near-field / self coefficients the FP64 formula decided
    int64_t matvecs = 0;
    int64_t launches = 0, link_launches = 0, link_bytes = 0;
    double link_ms = 0;
    int rhs_width = 0;  // columns per batched solve of the last solve
};
SolveTimings problem_timings(const DeviceProblem *p);
int problem_set_profiling(DeviceProblem *p, bool on);
int problem_set_tuning(DeviceProblem *p, bool on);
void problem_reset_stats(DeviceProblem *p);

}  // namespace fcg

#endif
