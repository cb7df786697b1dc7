// Device-resident capacitance problem for sm_103a: coefficient fill,
// hierarchical matrix-vector product and batched preconditioned GMRES.
//
// Layout in HBM (uploaded once per model, see fcg_problem_create):
//   geo[n_nodes]          80-byte NodeGeo records (vertices, centroid, normal,
//                         type, max side, area): gathered by the fill kernels
//   link_ptr[n_nodes+1]   int64 CSR offsets, links grouped by destination node
//   link_src[n_links]     int32 source node of each link
//   coef64 / coef32       link coefficients (FP64 path / mixed path)
//   self[n_panels]        FP64 self coefficients (also the Jacobi diagonal)
//   sweep plan            the node tree cut into subtrees of <= kBlockLeaves
//                         leaves (one CTA each) plus the "top" nodes above them,
//                         every group listed level by level
// Matrix-vector product v = P q (CMultHier::MultiplyMatByVec_fast,
// Solver/MultiplyHierarchical.cpp:285-304) for k right-hand sides at once:
//   up_block/up_top     node charges Q(node) = Q(left) + Q(right)     (:72-127)
//   spmv                P(node) = sum_l coef[l] * Q(src[l])           (:141-226)
//   down_top/down_block A(node) = P(node) + A(parent); v = self*q + P + A(parent)
//                                                                     (:231-283)
// Node-indexed work arrays hold the k values of one node contiguously.
// GMRES (CSolveCap::gmresPrecondSFastAll, Solver/SolveCapacitance.cpp:2288-2574)
// keeps its Krylov basis as [k][n_panels] vectors: FP64 on the FP64 path,
// FP32 pairs (8 bytes per element too) on the mixed path unless the solve
// asks for FP64 (fcg_solve_options.krylov); Hessenberg columns, Givens
// rotations and norms are FP64 on both.
#include <cuda_runtime.h>
#include <math.h>
#include <stdio.h>
#include <chrono>
#include <string.h>
#include <algorithm>
#include <mutex>
#include <string>
#include <vector>
#include <thread>
#include <type_traits>

#include "fc_potential.h"
#include "fp_bits.cuh"
#include "scan.cuh"
#include "fcg_internal.hpp"

namespace fcg {

#define FCG_CK(call)                                                                         \
    do {                                                                                     \
        cudaError_t e_ = (call);                                                             \
        if (e_ != cudaSuccess) {                                                             \
            set_error(std::string(#call) + " failed: " + cudaGetErrorString(e_));            \
            return FCG_DEVICE_ERROR;                                                         \
        }                                                                                    \
    } while (0)

static const int kBlockLeaves = 256;  // leaves per sweep subtree
static const int kMaxChain = 96;      // ancestors above a sweep subtree
static const int kSweepCols = 4;      // right-hand sides per shared-memory pass of the sweeps
static const int kSweepThreads = 128;  // threads per sweep CTA
static const int kMaxK = 32;          // right-hand sides per matvec batch
static const int kDotChunk = 1024;    // vector elements per CTA in the Krylov kernels
static const int kDotThreads = 128;   // threads per chunk in k_dots
static const int kPinSlots = 1024;    // pinned readback slots per context
static const int kPinSlotInts = 16;
// link words: source node in the low 29 bits, distance band (0..4) in the top 3
static const uint32_t kSrcMask = 0x1FFFFFFFu;
static const int kBandShift = 29;

struct __align__(16) NodeGeo {
    float v[9];
    float c[3];
    float n[3];
    uint32_t type;
    double maxside;
    double area;
};

// Device allocations are stream-ordered (cudaMallocAsync / cudaFreeAsync on
// the problem's stream, from the device's memory pool) inside an AllocScope:
// no allocation or free synchronises the device, so problems on different
// streams (the serving slots) never stall one another. Outside a scope the
// plain calls are used.
static thread_local cudaStream_t t_alloc_stream = NULL;
static thread_local bool t_alloc_async = false;
struct AllocScope {
    cudaStream_t prev;
    bool prev_async;
    explicit AllocScope(cudaStream_t s) : prev(t_alloc_stream), prev_async(t_alloc_async) {
        t_alloc_stream = s;
        t_alloc_async = true;
    }
    ~AllocScope() {
        t_alloc_stream = prev;
        t_alloc_async = prev_async;
    }
};

// device allocation tracked against the problem's byte count
template <class T> static int dalloc(T **p, size_t n, int64_t &bytes) {
    *p = NULL;
    if (n == 0) return FCG_NORMAL_END;
    cudaError_t e = t_alloc_async ? cudaMallocAsync((void **)p, n * sizeof(T), t_alloc_stream)
                                  : cudaMalloc((void **)p, n * sizeof(T));
    if (e != cudaSuccess) {
        cudaGetLastError();
        set_error(std::string("device allocation of ") + std::to_string(n * sizeof(T)) + " bytes failed: " + cudaGetErrorString(e));
        *p = NULL;
        return e == cudaErrorMemoryAllocation ? FCG_OUT_OF_MEMORY : FCG_DEVICE_ERROR;
    }
    bytes += (int64_t)(n * sizeof(T));
    return FCG_NORMAL_END;
}
template <class T> static void dfree(T *&p) {
    if (p) {
        if (t_alloc_async) cudaFreeAsync(p, t_alloc_stream);
        else cudaFree(p);
    }
    p = NULL;
}
template <class T> static int upload(T **p, const T *h, size_t n, int64_t &bytes, cudaStream_t s) {
    int r = dalloc(p, n, bytes);
    if (r != FCG_NORMAL_END) return r;
    if (n) FCG_CK(cudaMemcpyAsync(*p, h, n * sizeof(T), cudaMemcpyHostToDevice, s));
    return FCG_NORMAL_END;
}

// Host-to-device copies during problem creation. From pageable host memory
// the CUDA driver stages a copy synchronously through its own buffers, and
// concurrent creations (the serving slots) queue on that path; a Stager
// instead copies through two pinned buffers of the context, the host filling
// one while the DMA of the other runs, so every creating thread streams at
// its own memcpy speed. Pinned sources go straight to the copy engine.
static const size_t kStageBytes = (size_t)8 << 20;
static const int kStageMax = 32;  // pinned staging buffers per context

struct Stager {
    DeviceContext *ctx = NULL;
    void *buf[2] = {NULL, NULL};
    cudaEvent_t ev[2] = {NULL, NULL};
    int next = 0;
    bool tried = false;
    explicit Stager(DeviceContext &c) : ctx(&c) {}
    // the two buffers, taken from the context (allocated there on first
    // need) when the first pageable copy comes
    void acquire() {
        tried = true;
        std::lock_guard<std::mutex> lk(ctx->stage_mu);
        for (int i = 0; i < 2; i++) {
            if (!ctx->stage_free.empty()) {
                buf[i] = ctx->stage_free.back();
                ctx->stage_free.pop_back();
            } else if (ctx->stage_count < kStageMax && cudaHostAlloc(&buf[i], kStageBytes, cudaHostAllocDefault) == cudaSuccess) {
                ctx->stage_count++;
            } else {
                cudaGetLastError();
                buf[i] = NULL;
            }
            if (buf[i] && cudaEventCreateWithFlags(&ev[i], cudaEventDisableTiming) != cudaSuccess) ev[i] = NULL;
        }
    }
    bool usable() {
        if (!tried) acquire();
        return buf[0] && buf[1] && ev[0] && ev[1];
    }
    // page-locked host memory or device memory: the copy engine reads it directly
    static bool direct(const void *h) {
        cudaPointerAttributes pa;
        bool r = cudaPointerGetAttributes(&pa, h) == cudaSuccess &&
                 (pa.type == cudaMemoryTypeHost || pa.type == cudaMemoryTypeDevice || pa.type == cudaMemoryTypeManaged);
        cudaGetLastError();
        return r;
    }
    cudaError_t copy(void *dst, const void *src, size_t bytes, cudaStream_t s) {
        if (!bytes) return cudaSuccess;
        if (direct(src) || !usable()) return cudaMemcpyAsync(dst, src, bytes, cudaMemcpyDefault, s);
        for (size_t off = 0; off < bytes; off += kStageBytes) {
            size_t n = std::min(kStageBytes, bytes - off);
            int b = next;
            next ^= 1;
            cudaError_t e = cudaEventSynchronize(ev[b]);  // the buffer's previous DMA is done
            if (e != cudaSuccess) return e;
            memcpy(buf[b], (const char *)src + off, n);
            if ((e = cudaMemcpyAsync((char *)dst + off, buf[b], n, cudaMemcpyHostToDevice, s)) != cudaSuccess) return e;
            if ((e = cudaEventRecord(ev[b], s)) != cudaSuccess) return e;
        }
        return cudaSuccess;
    }
    ~Stager() {
        for (int i = 0; i < 2; i++) {
            if (ev[i]) {
                cudaEventSynchronize(ev[i]);
                cudaEventDestroy(ev[i]);
            }
        }
        std::lock_guard<std::mutex> lk(ctx->stage_mu);
        for (int i = 0; i < 2; i++)
            if (buf[i]) ctx->stage_free.push_back(buf[i]);
    }
};

template <class T> static int upload_staged(Stager &st, T **p, const T *h, size_t n, int64_t &bytes, cudaStream_t s) {
    int r = dalloc(p, n, bytes);
    if (r != FCG_NORMAL_END) return r;
    if (n) FCG_CK(st.copy(*p, h, n * sizeof(T), s));
    return FCG_NORMAL_END;
}

// The sweeps' plan. Blocks are the maximal subtrees of at most kBlockLeaves
// leaves (one CTA each); inside a block a node has a local index: leaves
// 0..nl-1 in leaf order, internal nodes nl + their position in the block's
// by-height list. Top nodes (more than kBlockLeaves leaves) form a forest
// over the blocks, listed by height; their children are named by top-local
// indices (block b -> b, top entry t -> n_blocks + t).
struct SweepPlan {
    int n_blocks = 0;
    int n_top = 0, n_top_levels = 0;  // top nodes; heights 0..n_top_levels-1 (top_hptr has n_top_levels + 1 entries)
    int32_t *blk_leaf_first = NULL, *blk_nleaves = NULL, *blk_lvl_first = NULL, *blk_nlvls = NULL, *blk_root = NULL;
    int32_t *blk_node_first = NULL;                 // first entry of the block's internal nodes in lvl_nodes
    int32_t *lvl_ptr = NULL, *lvl_nodes = NULL;
    uint32_t *lvl_kids = NULL;                      // per internal block node: left | right << 16 (local indices)
    int32_t *blk_chain = NULL, *chain = NULL;       // ancestors of every block root, parent first (device labels)
    int32_t *top_nodes = NULL, *top_hptr = NULL;    // top nodes by height (device labels), offsets per height
    int2 *top_kids = NULL;                          // children of every top node (top-local indices)
};

struct DeviceProblem {
    DeviceContext *ctx = NULL;
    int precision = FCG_PREC_FP64;
    int64_t Nn = 0, Np = 0, L = 0;
    int n_cond_all = 0;
    std::vector<int> cond_cols;  // solver-order index of every non-dielectric conductor
    std::vector<int64_t> cond_first, cond_count;
    cudaStream_t stream = NULL;
    bool owns_stream = false;
    cudaEvent_t ev0 = NULL, ev1 = NULL;
    int64_t bytes = 0;
    bool filled = false;
    // near-field (band 0) link list, built on the first fill
    int64_t n_near = -1;
    int32_t *near_link = NULL, *near_row = NULL;
    fcg_tri64 *tri = NULL;    // source-triangle tables for the FP64 near field
    fcg_tri32 *tri32 = NULL;  // scaled FP32 tables for the mixed near field and self terms
    unsigned long long *fill_fp64 = NULL;  // mixed fill: coefficients the FP64 formula decided
    // host copies mapping device rows (height-major labels) back to the model's links
    // (filled on the first coefficient readback)
    std::vector<int64_t> h_ptr_model, h_ptr_dev;
    std::vector<int32_t> h_inv;
    int32_t *inv = NULL;  // device: the model node of every device label
    SolveTimings timings;
    // profiling of the link product: event pairs awaiting readout
    bool profiling = false;
    bool tuning = true;  // measure launch shapes and the right-hand-side width (else the built-in rules)
    std::vector<cudaEvent_t> ev_pool;
    size_t ev_used = 0;

    // model
    NodeGeo *geo = NULL;
    int64_t *link_ptr = NULL;
    uint32_t *link_src = NULL;  // source node | band << kBandShift
    int32_t *leaf_node = NULL, *parent = NULL, *left = NULL, *right = NULL;
    int64_t *node_lfirst = NULL;  // first leaf of every node
    double *leaf_eb = NULL, *leaf_ea = NULL, *leaf_weight = NULL;
    double *coef64 = NULL;
    float *coef32 = NULL;
    double *self = NULL;
    double *rself = NULL;  // mixed path: 1 / self, the Jacobi scaling of the sweeps as a multiply
    float *rself32 = NULL;  // mixed path: 1 / self rounded to FP32 (the up-sweep's leaf charge scale)
    double *srself = NULL;  // mixed path: self * (1 / self) (the down-sweep's leaf term under Jacobi scaling)
    unsigned *status = NULL;
    SweepPlan plan;

    // matvec workspace (kcap values per node)
    int kcap = 0;
    double *Qd = NULL, *Pd = NULL, *Ad = NULL;
    float *Qf = NULL;
    float2 *Pf2 = NULL;
    int spmv_lanes = 32;  // lanes per destination node in the link product (8, 16 or 32)
    int32_t *row_split = NULL;  // multi-right-hand-side link product: CTA b owns rows [row_split[b], row_split[b+1])
    int n_row_split = 0;
    uint64_t tuned = 0;  // bit kp: the launch shape for kp right-hand sides is settled
    int tune_val[64] = {0};  // the settled shape per kp (lanes, or CTA row ranges per SM; 0 = built-in)

    // two-level preconditioner (built for one dimension, kept until another is asked for)
    int sup_dim = -1;  // dimension it was built for (-1: never built)
    int sup_m = 0;     // super elements (0: disabled, at least as many conductors as the dimension)
    int sup_kcap = 0;
    int32_t *sup_index = NULL;
    float *sup_area = NULL;
    int64_t *sup_first = NULL, *sup_count = NULL;
    double *sup_dimv = NULL, *sup_T = NULL, *sup_diag = NULL, *sup_pot = NULL, *sup_chg = NULL;

    // solve geometries (independent models concatenated into one problem)
    int n_geom = 0;
    std::vector<int> geom_cols_ptr;  // cond_cols of geometry g: [geom_cols_ptr[g], geom_cols_ptr[g+1])
    std::vector<int64_t> geom_leaf_first, geom_leaf_count;
    int nch = 0;  // Krylov chunks (never crossing a geometry)
    int32_t *leaf_geom = NULL, *ch_len = NULL, *ch_geom = NULL, *g_ch_first = NULL, *g_ch_count = NULL;
    int64_t *ch_start = NULL;

    // Krylov workspace
    int gk = 0, gS = 0, gM = 0;  // right-hand-side columns, solves, max iterations allocated
    std::vector<double *> V;  // basis vectors, each [gk][Np]
    double **Vptr = NULL;
    int Vptr_cap = 0;
    std::vector<double *> Hc;  // Hessenberg column i: [gS][i + 2]
    std::vector<double *> Hblk;
    double **Hptr = NULL;
    double *cs = NULL, *sn = NULL, *g = NULL, *normb = NULL, *hnorm = NULL, *nrm2 = NULL, *z = NULL;
    double *partial = NULL;
    size_t partial_cap = 0;
    int *active = NULL, *iters = NULL, *capped = NULL, *scap = NULL, *n_active = NULL;
    int *pin = NULL;  // pinned readback slot from the context (NULL: pageable fallback)
    int *pin_dev = NULL;  // the same slot as the device sees it (NULL: no device access)
    int *d_it = NULL;     // device step state: [0] step index, [1] go on, [2] active solves after the step
    double *ptmp = NULL;  // two-level preconditioner output ([k][Np])
    // the Arnoldi loop as one CUDA graph (a while node whose body is one step)
    cudaGraph_t graph = NULL;
    cudaGraphExec_t gexec = NULL;
    std::vector<unsigned char> gkey;
    int g_launches = 0, g_link_launches = 0;
    int64_t g_link_bytes = 0;
    int pin_local[kPinSlotInts];
    std::atomic<int> cancel{0};  // set by fcg_problem_cancel; checked between Arnoldi steps
    double *b = NULL, *x0 = NULL, *w = NULL, *vv = NULL, *x = NULL;
    int x_k = 0;
};

// --------------------------------------------------------------- kernels

// Device node arrays in height-major labels from the caller's post-order
// arrays: geometry, children, parent, leaf map, first leaf of every node.
__global__ void k_build_nodes(int64_t Nn, const int32_t *__restrict__ lab, const uint8_t *__restrict__ type,
                              const float *__restrict__ vert, const float *__restrict__ cent, const float *__restrict__ norm,
                              const double *__restrict__ area, const double *__restrict__ maxside, const int32_t *__restrict__ left,
                              const int32_t *__restrict__ right, const int64_t *__restrict__ leaf_first, NodeGeo *__restrict__ geo,
                              int32_t *__restrict__ dleft, int32_t *__restrict__ dright, int32_t *__restrict__ dparent,
                              int32_t *__restrict__ leaf_node, int64_t *__restrict__ node_lfirst) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < Nn; i += (int64_t)gridDim.x * blockDim.x) {
        int32_t q = lab[i];
        NodeGeo g;
#pragma unroll
        for (int k = 0; k < 9; k++) g.v[k] = vert[9 * i + k];
#pragma unroll
        for (int k = 0; k < 3; k++) { g.c[k] = cent[3 * i + k]; g.n[k] = norm[3 * i + k]; }
        g.type = type[i];
        g.maxside = maxside[i];
        g.area = area[i];
        geo[q] = g;
        int32_t l = left[i], r = right[i];
        dleft[q] = l >= 0 ? lab[l] : -1;
        dright[q] = r >= 0 ? lab[r] : -1;
        if (l >= 0) dparent[lab[l]] = q;
        if (r >= 0) dparent[lab[r]] = q;
        if (type[i] & FCG_IS_LEAF) leaf_node[leaf_first[i]] = q;
        node_lfirst[q] = leaf_first[i];
    }
}

// leaf permittivities: dielectric leaves get (outer, inner), conductor
// leaves the outer permittivity of their surface as the C-assembly weight
__global__ void k_build_leaves(int64_t Np, int n_cond, const int64_t *__restrict__ cfirst, const uint8_t *__restrict__ is_diel,
                               const double *__restrict__ outp, const double *__restrict__ inp, const int32_t *__restrict__ sptr,
                               const double *__restrict__ surf, const uint8_t *__restrict__ leaf_diel, double *__restrict__ eb,
                               double *__restrict__ ea, double *__restrict__ weight) {
    for (int64_t j = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; j < Np; j += (int64_t)gridDim.x * blockDim.x) {
        int lo = 0, hi = n_cond - 1;  // last conductor whose first leaf is <= j
        while (lo < hi) {
            int mid = (lo + hi + 1) >> 1;
            if (cfirst[mid] <= j) lo = mid;
            else hi = mid - 1;
        }
        if (is_diel[lo]) {
            eb[j] = outp[lo];
            ea[j] = inp[lo];
            weight[j] = 0.0;
        } else {
            eb[j] = 0.0;
            ea[j] = 0.0;
            weight[j] = surf[sptr[lo] + leaf_diel[j]];
        }
    }
}

__global__ void k_node_geom(int64_t Nn, const int64_t *__restrict__ node_lfirst, const int32_t *__restrict__ leaf_geom,
                            int32_t *__restrict__ node_geom) {
    for (int64_t v = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; v < Nn; v += (int64_t)gridDim.x * blockDim.x)
        node_geom[v] = leaf_geom[node_lfirst[v]];
}

// Device label, centroid and largest side of a node (model order): all the
// link relabelling and band classification read of a source, one 32-byte
// sector per gather.
struct __align__(32) CentMax {
    float c[3];
    int32_t lab;
    double ms;
    double pad;
};

__global__ void k_cent_max(int64_t Nn, const float *__restrict__ cent, const double *__restrict__ maxside,
                           const int32_t *__restrict__ lab, CentMax *__restrict__ cm) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < Nn; i += (int64_t)gridDim.x * blockDim.x) {
        CentMax r;
        r.c[0] = cent[3 * i];
        r.c[1] = cent[3 * i + 1];
        r.c[2] = cent[3 * i + 2];
        r.lab = lab[i];
        r.ms = maxside[i];
        r.pad = 0.0;
        cm[i] = r;
    }
}

// Links are relabelled in tiles of kRelTile consecutive links (model
// order); tile_row[t] is the row holding the tile's first link.
constexpr int kRelTile = 1024;
constexpr int kRelRows = 256;  // rows a tile keeps in shared memory

__global__ void k_tile_rows(int64_t Nn, const int64_t *__restrict__ ptr_model, int32_t *__restrict__ tile_row) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < Nn; i += (int64_t)gridDim.x * blockDim.x) {
        int64_t a = ptr_model[i], b = ptr_model[i + 1];
        for (int64_t t = (a + kRelTile - 1) / kRelTile; t * kRelTile < b; t++) tile_row[t] = (int32_t)i;
    }
}

// Move every link to its row's device position (height-major label),
// relabel its source and classify its distance band once per problem
// (fcg_band_exact: the FP64 decision of CAutoRefine::PotEstimateOpt,
// Solver/Autorefine.cpp:3495-3505, 3561-3598, from an FP32 ratio where that is
// certain), stored in the source word's top bits; every row's band-0
// (near-field) links are added to ncount (model order, zeroed by the
// caller). The caller's sources are validated here: an index outside
// [0, Nn) is counted in *bad and stored as node 0. A CTA takes tiles
// [t0, t1) of kRelTile links: the rows a tile touches (their offsets,
// device positions and geometry) are staged in shared memory, each thread
// takes four links (coalesced) and finds its row there; a source's label and
// geometry are one 32-byte gather by its model index.
__global__ void __launch_bounds__(256, 5) k_relabel_classify(int64_t Nn, int64_t L, int64_t t0, int64_t t1,
                                                          const int32_t *__restrict__ tile_row, const int64_t *__restrict__ ptr_model,
                                                          const uint32_t *__restrict__ src_model, const int64_t *__restrict__ ptr_dev,
                                                          const CentMax *__restrict__ cm, uint32_t *__restrict__ src_dev,
                                                          unsigned *bad, int32_t *__restrict__ ncount) {
    __shared__ int64_t s_ptr[kRelRows + 1];
    __shared__ int64_t s_o[kRelRows];
    __shared__ CentMax s_cm[kRelRows];
    __shared__ int s_cnt[kRelRows];
    const int tid = threadIdx.x;
    const int64_t ntiles = (L + kRelTile - 1) / kRelTile;
    unsigned nbad = 0;
    for (int64_t t = t0 + blockIdx.x; t < t1; t += gridDim.x) {
        const int64_t lo = t * kRelTile, hi = min(lo + kRelTile, L);
        const int64_t rlo = tile_row[t], rhi = t + 1 < ntiles ? tile_row[t + 1] : Nn - 1;
        const int nr = (int)(rhi - rlo + 1);
        const bool small = nr <= kRelRows;
        uint32_t j[4];
#pragma unroll
        for (int u = 0; u < 4; u++) {
            int64_t l = lo + u * 256 + tid;
            j[u] = l < hi ? src_model[l] : 0u;  // a negative int32 reads as >= Nn
            if (l < hi && j[u] >= (uint64_t)Nn) { nbad++; j[u] = 0; }
        }
        if (small) {
            for (int k = tid; k <= nr; k += blockDim.x) {
                int64_t pk = ptr_model[rlo + k];
                s_ptr[k] = pk;
                if (k < nr) {
                    CentMax d = cm[rlo + k];
                    s_cm[k] = d;
                    s_o[k] = ptr_dev[d.lab] - pk;
                    s_cnt[k] = 0;
                }
            }
        }
        float4 g[4];  // centroid and label bits
        double gms[4];
#pragma unroll
        for (int u = 0; u < 4; u++) {
            g[u] = *reinterpret_cast<const float4 *>(&cm[j[u]]);
            gms[u] = cm[j[u]].ms;
        }
        __syncthreads();
#pragma unroll
        for (int u = 0; u < 4; u++) {
            int64_t l = lo + u * 256 + tid;
            if (l >= hi) continue;
            // the row holding link l: the last row whose first link is <= l
            int64_t row, o;
            CentMax d;
            if (small) {
                int a = 0, b = nr - 1;
                while (a < b) {
                    int m = (a + b + 1) >> 1;
                    if (s_ptr[m] <= l) a = m;
                    else b = m - 1;
                }
                row = a;
                o = s_o[a];
                d = s_cm[a];
            } else {
                int64_t a = rlo, b = rhi;
                while (a < b) {
                    int64_t m = (a + b + 1) >> 1;
                    if (ptr_model[m] <= l) a = m;
                    else b = m - 1;
                }
                row = a;
                d = cm[a];
                o = ptr_dev[d.lab] - ptr_model[a];
            }
            int band = fcg_band_exact(d.c[0] - g[u].x, d.c[1] - g[u].y, d.c[2] - g[u].z, d.ms > gms[u] ? d.ms : gms[u]);
            src_dev[o + l] = __float_as_uint(g[u].w) | ((uint32_t)band << kBandShift);
            if (band == 0) {
                if (small) atomicAdd(&s_cnt[row], 1);
                else atomicAdd(&ncount[row], 1);
            }
        }
        __syncthreads();
        if (small)
            for (int k = tid; k < nr; k += blockDim.x)
                if (s_cnt[k]) atomicAdd(&ncount[rlo + k], s_cnt[k]);
        __syncthreads();  // the next tile reuses the shared arrays
    }
    if (nbad) atomicAdd(bad, nbad);
}

// The near-field list in row order: model row i's band-0 links go to
// [noff[i], noff[i] + ncount[i]) (entries at or beyond cap are dropped; the
// caller then makes room and runs it again). One warp per row.
__global__ void k_near_fill(int64_t Nn, const int64_t *__restrict__ ptr_model, const int32_t *__restrict__ lab,
                            const int64_t *__restrict__ ptr_dev, const uint32_t *__restrict__ src_dev,
                            const int32_t *__restrict__ ncount, const long long *__restrict__ noff, int64_t cap,
                            int32_t *__restrict__ near_link, int32_t *__restrict__ near_row) {
    int lane = threadIdx.x & 31;
    int64_t warp = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
    int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
    for (int64_t i = warp; i < Nn; i += nwarps) {
        if (ncount[i] == 0) continue;
        int32_t q = lab[i];
        int64_t o = ptr_dev[q], len = ptr_model[i + 1] - ptr_model[i], at = noff[i];
        for (int64_t t = 0; t < len; t += 32) {
            int64_t l = t + lane;
            bool nr = l < len && (src_dev[o + l] >> kBandShift) == 0;
            unsigned m = __ballot_sync(0xffffffffu, nr);
            int64_t pos = at + __popc(m & ((1u << lane) - 1u));
            if (nr && pos < cap) {
                near_link[pos] = (int32_t)(o + l);
                near_row[pos] = q;
            }
            at += __popc(m);
        }
    }
}

// Structural checks of the caller's tree, run before any kernel indexes with
// it (the per-node part of the host's model check, same rules): the lowest
// failing node and its reason go to first[0] (node << 8 | code), the leaves
// are counted in first[1].
__global__ void k_check_model(int64_t Nn, int64_t Np, const uint8_t *__restrict__ type, const int32_t *__restrict__ left,
                              const int32_t *__restrict__ right, const int64_t *__restrict__ lf, const int64_t *__restrict__ lc,
                              const int64_t *__restrict__ ptr, unsigned long long *first) {
    unsigned long long nleaf = 0;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < Nn; i += (int64_t)gridDim.x * blockDim.x) {
        int code = 0;
        if (ptr[i + 1] < ptr[i]) {
            code = 1;
        } else if (type[i] & FCG_IS_LEAF) {
            if (left[i] != -1 || right[i] != -1 || lc[i] != 1) code = 2;
            nleaf++;
        } else {
            int32_t l = left[i], r = right[i];
            if (l < 0 || r < 0 || l >= i || r >= i) code = 3;
            else if (lc[i] != lc[l] + lc[r]) code = 4;
            else if (lf[i] != lf[l] || lf[r] != lf[l] + lc[l]) code = 5;
        }
        if (!code && (lf[i] < 0 || lf[i] + lc[i] > Np)) code = 6;
        if (code) atomicMin(&first[0], ((unsigned long long)i << 8) | (unsigned long long)code);
    }
    for (int o = 16; o > 0; o >>= 1) nleaf += __shfl_xor_sync(0xffffffffu, nleaf, o);
    if ((threadIdx.x & 31) == 0 && nleaf) atomicAdd(&first[1], nleaf);
}

// every conductor leaf's permittivity index within its conductor's list (the
// conductors tile the leaves, checked on the host); the lowest failing leaf
// goes to *first
__global__ void k_check_leaves(int64_t Np, int n_cond, const int64_t *__restrict__ cfirst, const uint8_t *__restrict__ is_diel,
                               const int32_t *__restrict__ sptr, const uint8_t *__restrict__ leaf_diel, unsigned long long *first) {
    for (int64_t j = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; j < Np; j += (int64_t)gridDim.x * blockDim.x) {
        int lo = 0, hi = n_cond - 1;  // last conductor whose first leaf is <= j
        while (lo < hi) {
            int mid = (lo + hi + 1) >> 1;
            if (cfirst[mid] <= j) lo = mid;
            else hi = mid - 1;
        }
        if (!is_diel[lo] && (int)leaf_diel[j] >= sptr[lo + 1] - sptr[lo]) atomicMin(first, (unsigned long long)j);
    }
}

// counts tree edges and links whose two nodes lie in different geometries
__global__ void k_check_geometries(int64_t Nn, const int64_t *__restrict__ link_ptr, const uint32_t *__restrict__ link_src,
                                   const int32_t *__restrict__ parent, const int32_t *__restrict__ node_geom, unsigned *bad) {
    unsigned cnt = 0;
    int lane = threadIdx.x & 31;
    int64_t warp = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5, nw = ((int64_t)gridDim.x * blockDim.x) >> 5;
    for (int64_t v = warp; v < Nn; v += nw) {
        int gv = node_geom[v];
        if (lane == 0 && parent[v] >= 0 && node_geom[parent[v]] != gv) cnt++;
        for (int64_t l = link_ptr[v] + lane; l < link_ptr[v + 1]; l += 32)
            if (node_geom[link_src[l] & kSrcMask] != gv) cnt++;
    }
    if (cnt) atomicAdd(bad, cnt);
}

// count the near-field (band 0) links of every row

// Links of bands 1..4 (quadrature and point formulas), FP64 path: the
// reference's formulas, one warp per row.
__global__ void k_fill_far(int64_t Nn, const int64_t *__restrict__ ptr, const uint32_t *__restrict__ src,
                           const NodeGeo *__restrict__ geo, double *__restrict__ c64, unsigned *status) {
    int lane = threadIdx.x & 31;
    int64_t warp = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
    int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
    for (int64_t row = warp; row < Nn; row += nwarps) {
        const NodeGeo g1 = geo[row];
        bool diel = g1.type & FCG_IS_DIEL;
        fcg_d3 n64 = fcg_mk(0, 0, 0);
        if (diel) n64 = fcg_diel_normal(g1.type, g1.n);
        fcg_d3 r1 = fcg_widen(g1.c);
        int64_t s = ptr[row], e = ptr[row + 1];
        for (int64_t l = s + lane; l < e; l += 32) {
            uint32_t w = src[l];
            int band = (int)(w >> kBandShift);
            if (band == 0) continue;
            const NodeGeo &g2 = geo[w & kSrcMask];
            double val;
            if (band == 4) {
                fcg_d3 dist = fcg_fsub(g1.c, g2.c);
                double rd = fcg_mod(dist);
                val = diel ? fcg_dot(dist, n64) / (FCG_FOUR_PI_TIMES_E0 * rd * rd * rd) : 1 / (FCG_FOUR_PI_TIMES_E0 * rd);
            } else {
                int rule = band == 1 ? 5 : (band == 2 ? 3 : 2);
                val = (diel ? fcg_enfield_numerical(r1, g2.v, n64, rule) : fcg_potential_numerical(r1, g2.v, rule)) /
                      FCG_FOUR_PI_TIMES_E0;
            }
            if (!isfinite(val)) atomicOr(status, 1u);
            c64[l] = val;
        }
    }
}

// Mixed-precision far field (bands 1-4): the collocation quadratures of
// CPotential::PotentialNumerical / EnFieldNumerical (Solver/Potential.cpp:2077-2254)
// in FP32 without a per-link frame. A rule point (x, y) of the reference's
// frame (origin v0, x along v1 - v0) is the barycentric point (y, x, 1-x-y)
// of (v0, v1, v2), and the frame's jacobian / (2 area) is exactly 1, so the
// triangle average is the weighted sum over barycentric points: rule 2 the
// three permutations of (2/3, 1/6, 1/6), rule 3 the edge midpoints, rule 5
// the six permutations of its three coordinates. A link evaluates the
// slots of a per-band table (unused slots: the centroid with weight 0) that
// some lane of its warp needs, so the lanes run the same code whatever
// their links' bands; the point formula (band 4) uses the centroid offset.
__global__ void __launch_bounds__(256, 5) k_fill_far32(const int32_t *__restrict__ row_split, const int64_t *__restrict__ ptr,
                                                    const uint32_t *__restrict__ src, const NodeGeo *__restrict__ geo,
                                                    float *__restrict__ c32, unsigned *status) {
    __shared__ float4 tab[5][6];  // [band][slot] = (weight of v0, of v1, of v2, quadrature weight)
    if (threadIdx.x < 30) {
        int band = threadIdx.x / 6, sl = threadIdx.x % 6;
        const float t3 = 1.0f / 3.0f;
        float4 e = make_float4(t3, t3, t3, 0.0f);
        if (band == 4 && sl == 0) e = make_float4(0.0f, 0.0f, 0.0f, 1.0f);
        if (band == 3 && sl < 3) {  // rule 2
            const float a = 1.0f / 6.0f, c = 4.0f / 6.0f;
            e = sl == 0 ? make_float4(a, c, a, t3) : (sl == 1 ? make_float4(c, a, a, t3) : make_float4(a, a, c, t3));
        }
        if (band == 2 && sl < 3)  // rule 3
            e = sl == 0 ? make_float4(0.5f, 0.0f, 0.5f, t3) : (sl == 1 ? make_float4(0.0f, 0.5f, 0.5f, t3) : make_float4(0.5f, 0.5f, 0.0f, t3));
        if (band == 1) {  // rule 5
            const float a = 0.659027622374092f, b = 0.231933368553031f, c = 0.109039009072877f, w = 1.0f / 6.0f;
            const float4 r5[6] = {make_float4(b, a, c, w), make_float4(c, a, b, w), make_float4(a, b, c, w),
                                  make_float4(c, b, a, w), make_float4(a, c, b, w), make_float4(b, c, a, w)};
            e = r5[sl];
        }
        tab[band][sl] = e;
    }
    __syncthreads();
    const float k = (float)(1.0 / FCG_FOUR_PI_TIMES_E0);
    int lane = threadIdx.x & 31;
    // CTA b owns the contiguous rows [row_split[b], row_split[b+1]) (equal
    // link counts), its warps take every eighth row: consecutive rows share
    // most of their sources, so the geometry gathers hit L1 and each source
    // record comes from DRAM about once
    const int r0 = row_split[blockIdx.x], r1 = row_split[blockIdx.x + 1];
    for (int64_t row = r0 + (threadIdx.x >> 5); row < r1; row += blockDim.x >> 5) {
        const NodeGeo &g1 = geo[row];
        bool diel = g1.type & FCG_IS_DIEL;
        float nx = 0.0f, ny = 0.0f, nz = 0.0f;
        if (diel) {
            fcg_d3 n64 = fcg_diel_normal(g1.type, g1.n);
            nx = (float)n64.x; ny = (float)n64.y; nz = (float)n64.z;
        }
        const float c1x = g1.c[0], c1y = g1.c[1], c1z = g1.c[2];
        int64_t s0 = ptr[row], e0 = ptr[row + 1];
        // two links per lane in flight: both source words and both geometry
        // gathers are issued before either is evaluated
        for (int64_t l = s0 + lane; l < e0; l += 64) {
            bool has2 = l + 32 < e0;
            uint32_t wv[2];
            wv[0] = src[l];
            wv[1] = has2 ? src[l + 32] : 0u;  // a band-0 word: skipped below
            float4 A[2], B[2], Cq[2];
#pragma unroll
            for (int u = 0; u < 2; u++) {
                const float4 *G = reinterpret_cast<const float4 *>(geo + (wv[u] & kSrcMask));
                A[u] = G[0];  // v0 v1 v2 (9 floats) and the centroid
                B[u] = G[1];
                Cq[u] = G[2];
            }
#pragma unroll
            for (int u = 0; u < 2; u++) {
                int band = (int)(wv[u] >> kBandShift);
                // quadrature slots with weight (rule 5: 6, rules 2 and 3: 3),
                // the most any lane running here needs: the others have
                // weight 0 and add exactly nothing
                int ns = band == 1 ? 6 : ((band == 2 || band == 3) ? 3 : 0);
                ns = __reduce_max_sync(__activemask(), ns);
                if (band == 0) continue;
                float acc;
                if (band == 4) {
                    // point formula at the source centroid
                    float dx = c1x - Cq[u].y, dy = c1y - Cq[u].z, dz = c1z - Cq[u].w;
                    float ir = rsqrtf(dx * dx + dy * dy + dz * dz);
                    acc = diel ? (dx * nx + dy * ny + dz * nz) * ir * ir * ir : ir;
                } else {
                    // a rule point is the barycentric combination sum t_k v_k
                    // (sum t_k = 1), so the vector from it to the field point is
                    // sum t_k (c1 - v_k)
                    float f0x = c1x - A[u].x, f0y = c1y - A[u].y, f0z = c1z - A[u].z;
                    float f1x = c1x - A[u].w, f1y = c1y - B[u].x, f1z = c1z - B[u].y;
                    float f2x = c1x - B[u].z, f2y = c1y - B[u].w, f2z = c1z - Cq[u].x;
                    acc = 0.0f;
#pragma unroll
                    for (int sl = 0; sl < 6; sl++) {
                        if (sl >= ns) break;
                        float4 t = tab[band][sl];
                        float ex = t.x * f0x + t.y * f1x + t.z * f2x;
                        float ey = t.x * f0y + t.y * f1y + t.z * f2y;
                        float ez = t.x * f0z + t.y * f1z + t.z * f2z;
                        float ir = rsqrtf(ex * ex + ey * ey + ez * ez);
                        float f = diel ? (ex * nx + ey * ny + ez * nz) * ir * ir * ir : ir;
                        acc += t.w * f;
                    }
                }
                float val = k * acc;
                if (!isfinite(val)) atomicOr(status, 1u);
                c32[l + 32 * u] = val;
            }
        }
    }
}

// source-triangle tables of the near-field kernel, one per node
__global__ void k_make_tri(int64_t Nn, const NodeGeo *__restrict__ geo, fcg_tri64 *__restrict__ tri) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < Nn; i += (int64_t)gridDim.x * blockDim.x)
        fcg_tri64_make(geo[i].v, tri[i]);
}

// Near-field links (band 0), FP64 analytic, one thread per listed link.
__global__ void k_fill_near(int64_t n, const int32_t *__restrict__ near_link, const int32_t *__restrict__ near_row,
                            const uint32_t *__restrict__ src, const NodeGeo *__restrict__ geo, const fcg_tri64 *__restrict__ tri,
                            double *__restrict__ c64, float *__restrict__ c32, unsigned *status) {
    for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < n; t += (int64_t)gridDim.x * blockDim.x) {
        int64_t l = near_link[t];
        const NodeGeo &g1 = geo[near_row[t]];
        uint32_t j = src[l] & kSrcMask;
        const NodeGeo &g2 = geo[j];
        double val = fcg_pot_near_tri(g1.type, g1.c, g1.n, g2.c, g2.v, tri[j]);
        if (!isfinite(val)) atomicOr(status, 1u);
        if (c64) c64[l] = val;
        else c32[l] = (float)val;
    }
}

__global__ void __launch_bounds__(128, 8) k_make_tri32(int64_t Nn, const NodeGeo *__restrict__ geo, fcg_tri32 *__restrict__ tri) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < Nn; i += (int64_t)gridDim.x * blockDim.x)
        fcg_tri32_make(geo[i].v, geo[i].c, tri[i]);
}

// FP64 formulas for the mixed fill's few coefficients that FP32 cannot
// decide (kept out of line: they would otherwise set the kernels' registers)
__device__ __noinline__ float near_fp64(unsigned type1, const float *c1, const float *n1, const float *c2, const float *v2) {
    return (float)fcg_pot_near(type1, c1, n1, c2, v2);
}
__device__ __noinline__ double self_fp64(const float *c, const float *v) {
    return fcg_potential_opt(fcg_widen(c), v) / FCG_FOUR_PI_TIMES_E0;
}

// Mixed-precision near-field links: the analytic potential in FP32 in the
// source triangle's scaled frame (fcg_pot_near32), one thread per listed
// link; a link whose guard FP32 cannot decide takes the FP64 formula. Held
// to 64 registers (eight 128-thread CTAs per SM): the few spills cost less
// than the occupancy they buy (sphere fill 0.86 -> 0.77 ms).
__global__ void __launch_bounds__(128, 8) k_fill_near32(int64_t n, const int32_t *__restrict__ near_link, const int32_t *__restrict__ near_row,
                              const uint32_t *__restrict__ src, const NodeGeo *__restrict__ geo, const fcg_tri32 *__restrict__ tri,
                              float *__restrict__ c32, unsigned *status, unsigned long long *fb) {
    for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < n; t += (int64_t)gridDim.x * blockDim.x) {
        int64_t l = near_link[t];
        const NodeGeo &g1 = geo[near_row[t]];
        uint32_t j = src[l] & kSrcMask;
        const NodeGeo &g2 = geo[j];
        float val;
        if (!fcg_pot_near32(g1.type, g1.c, g1.n, g2.c, tri[j], &val)) {
            val = near_fp64(g1.type, g1.c, g1.n, g2.c, g2.v);
            atomicAdd(fb, 1ull);
        }
        if (!isfinite(val)) atomicOr(status, 1u);
        c32[l] = val;
    }
}

// Mixed-precision self terms: conductor leaves by the FP32 analytic potential
// at the own centroid (FP64 where FP32 cannot decide a guard), dielectric
// leaves by their closed form.
__global__ void __launch_bounds__(256, 4) k_fill_self32(int64_t Np, const int32_t *__restrict__ leaf_node, const NodeGeo *__restrict__ geo,
                              const fcg_tri32 *__restrict__ tri, const double *__restrict__ eb, const double *__restrict__ ea,
                              double *__restrict__ self, double *__restrict__ rself, float *__restrict__ rself32,
                              double *__restrict__ srself, unsigned *status, unsigned long long *fb) {
    for (int64_t j = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; j < Np; j += (int64_t)gridDim.x * blockDim.x) {
        int32_t node = leaf_node[j];
        const NodeGeo &g = geo[node];
        double val;
        if (g.type & FCG_IS_DIEL) {
            val = fcg_self_potential(g.type, g.c, g.v, g.area, eb[j], ea[j]);
        } else {
            float v;
            if (fcg_potential32(0.0f, 0.0f, 0.0f, tri[node], &v)) {
                val = (double)(v * (float)(1.0 / FCG_FOUR_PI_TIMES_E0));
            } else {
                val = self_fp64(g.c, g.v);
                atomicAdd(fb, 1ull);
            }
        }
        if (!isfinite(val) || val == 0.0) atomicOr(status, 2u);
        self[j] = val;
        const double r = 1.0 / val;
        rself[j] = r;
        rself32[j] = (float)r;
        srself[j] = val * r;
    }
}

__global__ void k_fill_self(int64_t Np, const int32_t *__restrict__ leaf_node, const NodeGeo *__restrict__ geo,
                            const double *__restrict__ eb, const double *__restrict__ ea, double *__restrict__ self,
                            unsigned *status) {
    for (int64_t j = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; j < Np; j += (int64_t)gridDim.x * blockDim.x) {
        const NodeGeo &g = geo[leaf_node[j]];
        double val;
        if (g.type & FCG_IS_DIEL) {
            val = fcg_self_potential(g.type, g.c, g.v, g.area, eb[j], ea[j]);
        } else {
            // collocation at the own centroid, in the reduced-cost form
            fcg_tri64 t;
            fcg_tri64_make(g.v, t);
            val = fcg_potential_opt_fast(fcg_widen(g.c), g.v, t) / FCG_FOUR_PI_TIMES_E0;
        }
        if (!isfinite(val) || val == 0.0) atomicOr(status, 2u);
        self[j] = val;
    }
}

// Up-sweep (CMultHier::ComputePanelCharges_fast, Solver/MultiplyHierarchical.cpp:72-127),
// in two launches. k_up_blk: one CTA per block; the block's children lists
// (local indices), node labels and level offsets are staged in shared memory
// together with the (optionally Jacobi-scaled) leaf inputs, then every
// internal node sums its two children level by level in shared memory
// (left + right, in FP64), so a level costs a barrier, not a round trip to
// memory. Node charges go to Qf (mixed) or Qd (FP64); the mixed path also
// keeps the block root's FP64 charge for the top pass. Leaf j has device
// label j. Right-hand sides are processed kc at a time; kSweepThreads
// threads per CTA keep every block of a large model resident at once.
// The Arnoldi step's pending normalisation, done by the up-sweep as it reads
// the step's vector (k_scale's work): q = v / |v| for every active solve,
// written back to v and to basis vector *iter (FP64, or an FP32 pair on the
// mixed path); nothing at step 0, whose vector is normalised before the loop.
struct StepScale {
    const double *hn;  // NULL: no normalisation; reciprocals of the norms when recip is set
    int recip;
    const int *active;
    const int32_t *leaf_geom;
    double *const *Vp;
    const int *iter;
    int pair;  // basis vectors as FP32 pairs (the mixed path's FCG_KRYLOV_PAIR)
};

template <bool MIXED>
__global__ void __launch_bounds__(kSweepThreads, 16) k_up_blk(const SweepPlan plan, const double *in, int64_t ld, int k, int kp,
                                                              int kc, const double *__restrict__ diag, int recip,
                                                              double *__restrict__ Qd, float *__restrict__ Qf,
                                                              double *__restrict__ rootq, const StepScale sc) {
    extern __shared__ double sh[];
    double *val = sh;                                                 // (2 kBlockLeaves - 1) x kc
    uint32_t *kids = (uint32_t *)(sh + (2 * kBlockLeaves - 1) * kc);  // kBlockLeaves
    int32_t *lbl = (int32_t *)(kids + kBlockLeaves);                  // kBlockLeaves
    int32_t *lp = lbl + kBlockLeaves;                                 // kBlockLeaves + 1
    const int b = blockIdx.x, tid = threadIdx.x;
    const int lf = plan.blk_leaf_first[b], nl = plan.blk_nleaves[b], lv0 = plan.blk_lvl_first[b], H = plan.blk_nlvls[b];
    const int base = plan.blk_node_first[b], ni = nl - 1;
    for (int t = tid; t < ni; t += blockDim.x) {
        kids[t] = plan.lvl_kids[base + t];
        lbl[t] = plan.lvl_nodes[base + t];
    }
    for (int t = tid; t <= H; t += blockDim.x) lp[t] = plan.lvl_ptr[lv0 + t] - base;
    const int step = sc.hn ? *sc.iter : 0;
    double *Vi = step > 0 ? sc.Vp[step] : NULL;
    for (int c0 = 0; c0 < k; c0 += kc) {
        const int kk = min(kc, k - c0);
        for (int t = tid; t < nl * kk; t += blockDim.x) {
            int r = t / nl, i = t - r * nl;
            int64_t at = (int64_t)(c0 + r) * ld + lf + i;
            double x = in[at];
            if (Vi) {
                int sidx = sc.leaf_geom[lf + i] * k + c0 + r;
                if (sc.active[sidx]) {
                    x = sc.recip ? x * sc.hn[sidx] : x / sc.hn[sidx];
                    const_cast<double *>(in)[at] = x;
                    if (sc.pair) reinterpret_cast<float2 *>(Vi)[at] = d2pair_bits(x);
                    else Vi[at] = x;
                }
            }
            if (diag) x = recip ? x * diag[lf + i] : x / diag[lf + i];
            val[i * kc + r] = x;
            int64_t o = (int64_t)(lf + i) * kp + c0 + r;
            if (!MIXED || ni == 0) Qd[o] = x;
            if (MIXED) Qf[o] = (float)x;
            if (ni == 0) rootq[(int64_t)b * kp + c0 + r] = x;
        }
        __syncthreads();
        for (int h = 0; h < H; h++) {
            const int a = lp[h], cnt = lp[h + 1] - a;
            for (int t = tid; t < cnt * kk; t += blockDim.x) {
                int q = a + t / kk, r = t - (t / kk) * kk;
                uint32_t kd = kids[q];
                double sum = val[(kd & 0xffffu) * kc + r] + val[(kd >> 16) * kc + r];
                val[(nl + q) * kc + r] = sum;
                int64_t o = (int64_t)lbl[q] * kp + c0 + r;
                if (!MIXED || q == ni - 1) Qd[o] = sum;  // the root is the block's last (highest) node
                if (MIXED) Qf[o] = (float)sum;
                if (q == ni - 1) rootq[(int64_t)b * kp + c0 + r] = sum;
            }
            __syncthreads();
        }
    }
}

// k_up_top: one CTA computes every top node from the block roots' FP64
// charges, height by height in shared memory (the host sizes kc so that
// (blocks + top nodes) x kc values fit). k_up_top_global is the same pass
// through device memory for forests too large for shared memory.
template <bool MIXED>
__global__ void __launch_bounds__(1024) k_up_top(const SweepPlan plan, int k, int kp, int kc, const double *__restrict__ rootq,
                                                 double *__restrict__ Qd, float *__restrict__ Qf) {
    extern __shared__ double sh[];
    const int nb = plan.n_blocks, T = plan.n_top, nh = plan.n_top_levels, tid = threadIdx.x;
    double *val = sh;                                        // (nb + T) x kc
    int2 *kids = (int2 *)(sh + (int64_t)(nb + T) * kc);      // T
    int32_t *lbl = (int32_t *)(kids + T);                    // T
    int32_t *hp = lbl + T;                                   // nh + 1
    for (int t = tid; t < T; t += blockDim.x) {
        kids[t] = plan.top_kids[t];
        lbl[t] = plan.top_nodes[t];
    }
    for (int t = tid; t <= nh; t += blockDim.x) hp[t] = plan.top_hptr[t];
    for (int c0 = 0; c0 < k; c0 += kc) {
        const int kk = min(kc, k - c0);
        for (int t = tid; t < nb * kk; t += blockDim.x) {
            int r = t / nb, bb = t - r * nb;
            val[bb * kc + r] = rootq[(int64_t)bb * kp + c0 + r];
        }
        __syncthreads();
        for (int h = 0; h < nh; h++) {
            const int a = hp[h], cnt = hp[h + 1] - a;
            if (cnt == 0) continue;  // uniform: every thread reads the same offsets
            for (int t = tid; t < cnt * kk; t += blockDim.x) {
                int q = a + t / kk, r = t - (t / kk) * kk;
                int2 kd = kids[q];
                double sum = val[(int64_t)kd.x * kc + r] + val[(int64_t)kd.y * kc + r];
                val[(int64_t)(nb + q) * kc + r] = sum;
                int64_t o = (int64_t)lbl[q] * kp + c0 + r;
                if (!MIXED) Qd[o] = sum;
                if (MIXED) Qf[o] = (float)sum;
            }
            __syncthreads();
        }
    }
}

template <bool MIXED>
__global__ void __launch_bounds__(1024) k_up_top_global(const SweepPlan plan, int k, int kp, double *Qd, float *Qf) {
    const int nb = plan.n_blocks, nh = plan.n_top_levels;
    for (int h = 0; h < nh; h++) {
        const int a = plan.top_hptr[h], cnt = plan.top_hptr[h + 1] - a;
        if (cnt == 0) continue;
        for (int t = threadIdx.x; t < cnt * k; t += blockDim.x) {
            int q = a + t / k, r = t - (t / k) * k;
            int2 kd = plan.top_kids[q];
            int32_t l = kd.x < nb ? plan.blk_root[kd.x] : plan.top_nodes[kd.x - nb];
            int32_t rt = kd.y < nb ? plan.blk_root[kd.y] : plan.top_nodes[kd.y - nb];
            double sum = Qd[(int64_t)l * kp + r] + Qd[(int64_t)rt * kp + r];
            int64_t o = (int64_t)plan.top_nodes[q] * kp + r;
            Qd[o] = sum;
            if (MIXED) Qf[o] = (float)sum;
        }
        __syncthreads();  // this level's charges are visible to the CTA's next level
    }
}

__device__ __forceinline__ double pval(const double *P, int64_t i) { return P[i]; }
__device__ __forceinline__ double pval(const float2 *P, int64_t i) {
    float2 v = P[i];
    return (double)v.x + (double)v.y;
}

// Down-sweep (CMultHier::ComputeLeafPotentials_fast, Solver/MultiplyHierarchical.cpp:231-283):
// A(n) = P(n) + A(parent(n)) from the top. One CTA per block: the link
// potentials of the block's nodes and of its root's ancestors, the leaves'
// scaled inputs and self terms are staged in shared memory (each thread
// fetches a node's label and then its potential, so the staging is two
// dependent rounds of loads), the ancestors are summed top down (the
// reference's order), then every internal node, level by level from the
// root, adds its A to its internal children's P (which makes their A) or
// hands it to its leaf children, and every leaf writes
// v = (self * x + P(leaf)) + A(parent(leaf)).
template <class TP>
__global__ void __launch_bounds__(kSweepThreads, 16) k_down_blk(const SweepPlan plan, const double *__restrict__ in, int64_t ld,
                                                                int k, int kp, int kc, const double *__restrict__ diag,
                                                                int recip, const double *__restrict__ self,
                                                                const TP *__restrict__ P, double *__restrict__ out) {
    extern __shared__ double sh[];
    double *pv = sh;                                     // (2 kBlockLeaves - 1) x kc: P, then A of internal nodes
    double *al = pv + (2 * kBlockLeaves - 1) * kc;       // kBlockLeaves x kc: A of each leaf's parent
    double *cp = al + kBlockLeaves * kc;                 // kMaxChain x kc: P of the root's ancestors
    double *ss = cp + kMaxChain * kc;                    // kBlockLeaves: leaf self terms
    uint32_t *kids = (uint32_t *)(ss + kBlockLeaves);    // kBlockLeaves
    int32_t *lp = (int32_t *)(kids + kBlockLeaves);      // kBlockLeaves + 1
    const int b = blockIdx.x, tid = threadIdx.x;
    const int lf = plan.blk_leaf_first[b], nl = plan.blk_nleaves[b], lv0 = plan.blk_lvl_first[b], H = plan.blk_nlvls[b];
    const int base = plan.blk_node_first[b], ni = nl - 1;
    const int ch0 = plan.blk_chain[b], nc = plan.blk_chain[b + 1] - ch0;
    for (int t = tid; t <= H; t += blockDim.x) lp[t] = plan.lvl_ptr[lv0 + t] - base;
    for (int t = tid; t < nl; t += blockDim.x) ss[t] = self[lf + t];
    const bool hasA = ni > 0 || nc > 0;
    for (int c0 = 0; c0 < k; c0 += kc) {
        const int kk = min(kc, k - c0);
        for (int t = tid; t < ni; t += blockDim.x) {
            if (c0 == 0) kids[t] = plan.lvl_kids[base + t];
            int64_t o = (int64_t)plan.lvl_nodes[base + t] * kp + c0;
            for (int r = 0; r < kk; r++) pv[(nl + t) * kc + r] = pval(P, o + r);
        }
        for (int t = tid; t < nc; t += blockDim.x) {
            int64_t o = (int64_t)plan.chain[ch0 + t] * kp + c0;
            for (int r = 0; r < kk; r++) cp[t * kc + r] = pval(P, o + r);
        }
        for (int t = tid; t < nl * kk; t += blockDim.x) {
            int r = t / nl, i = t - r * nl;
            pv[i * kc + r] = pval(P, (int64_t)(lf + i) * kp + c0 + r);
        }
        __syncthreads();
        if (tid < kk && nc > 0) {
            double acc = cp[(nc - 1) * kc + tid];
            for (int j = nc - 2; j >= 0; j--) acc = cp[j * kc + tid] + acc;
            if (ni > 0) pv[(nl + ni - 1) * kc + tid] = pv[(nl + ni - 1) * kc + tid] + acc;  // A of the block root
            else al[tid] = acc;                                                             // a leaf root's parent sum
        }
        __syncthreads();
        for (int h = H - 1; h >= 0; h--) {
            const int a = lp[h], cnt = lp[h + 1] - a;
            for (int t = tid; t < cnt * kk; t += blockDim.x) {
                int q = a + t / kk, r = t - (t / kk) * kk;
                double A = pv[(nl + q) * kc + r];
                uint32_t kd = kids[q];
                int c1 = kd & 0xffffu, c2 = kd >> 16;
                if (c1 < nl) al[c1 * kc + r] = A;
                else pv[c1 * kc + r] = pv[c1 * kc + r] + A;
                if (c2 < nl) al[c2 * kc + r] = A;
                else pv[c2 * kc + r] = pv[c2 * kc + r] + A;
            }
            __syncthreads();
        }
        for (int t = tid; t < nl * kk; t += blockDim.x) {
            int r = t / nl, i = t - r * nl;
            int j = lf + i;
            // the leaf's (scaled) input, read here once instead of staged
            double xv = in[(int64_t)(c0 + r) * ld + j];
            if (diag) xv = recip ? xv * diag[j] : xv / diag[j];
            double v = ss[i] * xv + pv[i * kc + r];
            if (hasA) v = v + al[i * kc + r];
            out[(int64_t)(c0 + r) * ld + j] = v;
        }
        __syncthreads();  // the next pass reuses the shared arrays
    }
}

// ---- mixed-path sweeps in FP32 pairs
//
// GB300 runs FP64 arithmetic and every FP64<->FP32 conversion on its FP64
// pipe, at about 1.6 operations per SM and clock (measured; FP32 about 119):
// the FP64 sweeps spent most of their time there (the down-sweep did six
// FP64 operations or conversions per leaf and right-hand side, four per
// internal node). The mixed path's sweeps therefore sum in unevaluated FP32
// pairs (value = s + c, about 44 significant bits: Knuth's TwoSum for the
// leading parts, then the trailing parts and a Fast2Sum renormalisation) and
// convert with integer operations; FP64 arithmetic is left for the Krylov
// vectors themselves (the step's normalisation, written back to v in FP64
// and to the basis as a pair, and the leaf output v = x * self/diag +
// potential).

// (a.x + a.y) + (b.x + b.y) as a normalised pair
__device__ __forceinline__ float2 f2_add(float2 a, float2 b) {
    const float s = __fadd_rn(a.x, b.x);
    const float bb = __fsub_rn(s, a.x);
    float e = __fadd_rn(__fsub_rn(a.x, __fsub_rn(s, bb)), __fsub_rn(b.x, bb));
    e = __fadd_rn(e, __fadd_rn(a.y, b.y));
    const float h = __fadd_rn(s, e);
    return make_float2(h, __fsub_rn(e, __fsub_rn(h, s)));
}

// acc + a b for pairs a, b: the leading product exactly as p + e (one FMA),
// the cross terms folded into e, p added to the leading sum by TwoSum and
// the rounding errors gathered in the trailing part (Ogita, Rump and
// Oishi's Dot2, 2005, with pair inputs); acc is left unnormalised
__device__ __forceinline__ float2 f2_fma(float2 acc, float2 a, float2 b) {
    const float p = __fmul_rn(a.x, b.x);
    float e = __fmaf_rn(a.x, b.x, -p);
    e = __fmaf_rn(a.x, b.y, e);
    e = __fmaf_rn(a.y, b.x, e);
    const float s = __fadd_rn(acc.x, p);
    const float bb = __fsub_rn(s, acc.x);
    const float err = __fadd_rn(__fsub_rn(acc.x, __fsub_rn(s, bb)), __fsub_rn(p, bb));
    return make_float2(s, __fadd_rn(acc.y, __fadd_rn(err, e)));
}

// The Krylov kernels' element types: the FP64 path keeps the basis and its
// sums in FP64; the mixed path stores basis vectors as FP32 pairs (same
// 8 bytes per element, d2pair_bits) and sums in pairs on the FP32 pipe.
__device__ __forceinline__ double kv_add(double a, double b) { return a + b; }
__device__ __forceinline__ float2 kv_add(float2 a, float2 b) { return f2_add(a, b); }
__device__ __forceinline__ double kv_shfl_xor(double v, int m) { return __shfl_xor_sync(0xffffffffu, v, m); }
__device__ __forceinline__ float2 kv_shfl_xor(float2 v, int m) {
    return make_float2(__shfl_xor_sync(0xffffffffu, v.x, m), __shfl_xor_sync(0xffffffffu, v.y, m));
}
__device__ __forceinline__ double kv_double(double v) { return v; }
__device__ __forceinline__ double kv_double(float2 v) { return pair2d(v); }
template <typename E> __device__ __forceinline__ E kv_zero();
template <> __device__ __forceinline__ double kv_zero<double>() { return 0.0; }
template <> __device__ __forceinline__ float2 kv_zero<float2>() { return make_float2(0.0f, 0.0f); }

// KC consecutive values of a node (KC = 1, 2, 4): vector loads and stores
// where the node's KC values form an aligned 8, 16 or 32-byte group (kp is
// 1, 2 or a multiple of 4 and a pass starts at a multiple of KC)
template <int KC> __device__ __forceinline__ void load_pairs(const float2 *__restrict__ p, float2 *v) {
    if constexpr (KC == 4) {
        const float4 a = reinterpret_cast<const float4 *>(p)[0], b = reinterpret_cast<const float4 *>(p)[1];
        v[0] = make_float2(a.x, a.y); v[1] = make_float2(a.z, a.w); v[2] = make_float2(b.x, b.y); v[3] = make_float2(b.z, b.w);
    } else if constexpr (KC == 2) {
        const float4 a = reinterpret_cast<const float4 *>(p)[0];
        v[0] = make_float2(a.x, a.y); v[1] = make_float2(a.z, a.w);
    } else {
        v[0] = p[0];
    }
}
template <int KC> __device__ __forceinline__ void store_pairs(float2 *p, const float2 *v) {
    if constexpr (KC == 4) {
        reinterpret_cast<float4 *>(p)[0] = make_float4(v[0].x, v[0].y, v[1].x, v[1].y);
        reinterpret_cast<float4 *>(p)[1] = make_float4(v[2].x, v[2].y, v[3].x, v[3].y);
    } else if constexpr (KC == 2) {
        reinterpret_cast<float4 *>(p)[0] = make_float4(v[0].x, v[0].y, v[1].x, v[1].y);
    } else {
        p[0] = v[0];
    }
}
template <int KC> __device__ __forceinline__ void store_leading(float *p, const float2 *v) {
    if constexpr (KC == 4) reinterpret_cast<float4 *>(p)[0] = make_float4(v[0].x, v[1].x, v[2].x, v[3].x);
    else if constexpr (KC == 2) reinterpret_cast<float2 *>(p)[0] = make_float2(v[0].x, v[1].x);
    else p[0] = v[0].x;
}

// Up-sweep, mixed: k_up_blk with the block's sums in FP32 pairs, one thread
// per node carrying KC right-hand sides; CTA (block, y) takes columns
// y*KC .. y*KC+KC-1 of all kp (the padding columns k..kp-1 get zero
// charges), so the column groups of a block run side by side. A leaf's charge is its input
// (normalised in FP64 first when the step asks for it) rounded to FP32,
// times the FP32 Jacobi reciprocal when rs is set; node charges go to Qf
// (the pair's leading part), the block root's pair to rootq for the top
// pass.
template <int KC>
__global__ void __launch_bounds__(kSweepThreads, 8) k_up_blk32(const SweepPlan plan, const double *in, int64_t ld, int k, int kp,
                                                                const float *__restrict__ rs, float *__restrict__ Qf,
                                                                float2 *__restrict__ rootq, const StepScale sc) {
    extern __shared__ __align__(16) float2 shp[];
    float2 *val = shp;                                                // (2 kBlockLeaves - 1) x KC
    uint32_t *kids = (uint32_t *)(shp + (2 * kBlockLeaves - 1) * KC);  // kBlockLeaves
    int32_t *lbl = (int32_t *)(kids + kBlockLeaves);                  // kBlockLeaves
    int32_t *lp = lbl + kBlockLeaves;                                 // kBlockLeaves + 1
    const int b = blockIdx.x, tid = threadIdx.x;
    const int lf = plan.blk_leaf_first[b], nl = plan.blk_nleaves[b], lv0 = plan.blk_lvl_first[b], H = plan.blk_nlvls[b];
    const int base = plan.blk_node_first[b], ni = nl - 1;
    for (int t = tid; t < ni; t += blockDim.x) {
        kids[t] = plan.lvl_kids[base + t];
        lbl[t] = plan.lvl_nodes[base + t];
    }
    for (int t = tid; t <= H; t += blockDim.x) lp[t] = plan.lvl_ptr[lv0 + t] - base;
    const int step = sc.hn ? *sc.iter : 0;
    double *Vi = step > 0 ? sc.Vp[step] : NULL;
    const int c0 = blockIdx.y * KC;
    {
        for (int i = tid; i < nl; i += blockDim.x) {
            const int j = lf + i;
            double x[KC];
#pragma unroll
            for (int r = 0; r < KC; r++) x[r] = c0 + r < k ? in[(int64_t)(c0 + r) * ld + j] : 0.0;
            if (Vi) {
                const int g = sc.leaf_geom[j] * k;
#pragma unroll
                for (int r = 0; r < KC; r++) {
                    if (c0 + r < k && sc.active[g + c0 + r]) {
                        x[r] = sc.recip ? x[r] * sc.hn[g + c0 + r] : x[r] / sc.hn[g + c0 + r];
                        const int64_t at = (int64_t)(c0 + r) * ld + j;
                        const_cast<double *>(in)[at] = x[r];
                        if (sc.pair) reinterpret_cast<float2 *>(Vi)[at] = d2pair_bits(x[r]);
                        else Vi[at] = x[r];
                    }
                }
            }
            const float sj = rs ? rs[j] : 1.0f;
            float2 q[KC];
#pragma unroll
            for (int r = 0; r < KC; r++) q[r] = make_float2(rs ? d2f_bits(x[r]) * sj : d2f_bits(x[r]), 0.0f);
            store_pairs<KC>(val + i * KC, q);
            store_leading<KC>(Qf + (int64_t)j * kp + c0, q);
            if (ni == 0) store_pairs<KC>(rootq + (int64_t)b * kp + c0, q);
        }
        __syncthreads();
        for (int h = 0; h < H; h++) {
            const int a = lp[h], cnt = lp[h + 1] - a;
            for (int t = tid; t < cnt; t += blockDim.x) {
                const int q = a + t;
                const uint32_t kd = kids[q];
                float2 u[KC], w[KC];
                load_pairs<KC>(val + (kd & 0xffffu) * KC, u);
                load_pairs<KC>(val + (kd >> 16) * KC, w);
#pragma unroll
                for (int r = 0; r < KC; r++) u[r] = f2_add(u[r], w[r]);
                store_pairs<KC>(val + (nl + q) * KC, u);
                store_leading<KC>(Qf + (int64_t)lbl[q] * kp + c0, u);
                if (q == ni - 1) store_pairs<KC>(rootq + (int64_t)b * kp + c0, u);  // the root is the block's last (highest) node
            }
            __syncthreads();
        }
    }
}

// Top pass, mixed: k_up_top with FP32 pairs in shared memory, one CTA per
// group of KC right-hand sides, one thread per node.
template <int KC>
__global__ void __launch_bounds__(1024) k_up_top32(const SweepPlan plan, int kp, const float2 *__restrict__ rootq,
                                                   float *__restrict__ Qf) {
    extern __shared__ __align__(16) float2 shp[];
    const int nb = plan.n_blocks, T = plan.n_top, nh = plan.n_top_levels, tid = threadIdx.x;
    float2 *val = shp;                                       // (nb + T) x KC
    int2 *kids = (int2 *)(shp + (int64_t)(nb + T) * KC);     // T
    int32_t *lbl = (int32_t *)(kids + T);                    // T
    int32_t *hp = lbl + T;                                   // nh + 1
    for (int t = tid; t < T; t += blockDim.x) {
        kids[t] = plan.top_kids[t];
        lbl[t] = plan.top_nodes[t];
    }
    for (int t = tid; t <= nh; t += blockDim.x) hp[t] = plan.top_hptr[t];
    const int c0 = blockIdx.x * KC;
    {
        for (int bb = tid; bb < nb; bb += blockDim.x) {
            float2 v[KC];
            load_pairs<KC>(rootq + (int64_t)bb * kp + c0, v);
            store_pairs<KC>(val + bb * KC, v);
        }
        __syncthreads();
        for (int h = 0; h < nh; h++) {
            const int a = hp[h], cnt = hp[h + 1] - a;
            if (cnt == 0) continue;  // uniform: every thread reads the same offsets
            for (int t = tid; t < cnt; t += blockDim.x) {
                const int q = a + t;
                const int2 kd = kids[q];
                float2 u[KC], w[KC];
                load_pairs<KC>(val + (int64_t)kd.x * KC, u);
                load_pairs<KC>(val + (int64_t)kd.y * KC, w);
#pragma unroll
                for (int r = 0; r < KC; r++) u[r] = f2_add(u[r], w[r]);
                store_pairs<KC>(val + (int64_t)(nb + q) * KC, u);
                store_leading<KC>(Qf + (int64_t)lbl[q] * kp + c0, u);
            }
            __syncthreads();
        }
    }
}

// The same pass through device memory (forests too large for shared
// memory): the top nodes' pairs go to Qp (n_nodes x kp).
__global__ void __launch_bounds__(1024) k_up_top32_global(const SweepPlan plan, int kp, const float2 *__restrict__ rootq,
                                                          float2 *Qp, float *__restrict__ Qf) {
    const int nb = plan.n_blocks, nh = plan.n_top_levels;
    for (int h = 0; h < nh; h++) {
        const int a = plan.top_hptr[h], cnt = plan.top_hptr[h + 1] - a;
        if (cnt == 0) continue;
        for (int t = threadIdx.x; t < cnt * kp; t += blockDim.x) {
            int q = a + t / kp, r = t - (t / kp) * kp;
            int2 kd = plan.top_kids[q];
            float2 l = kd.x < nb ? rootq[(int64_t)kd.x * kp + r] : Qp[(int64_t)plan.top_nodes[kd.x - nb] * kp + r];
            float2 rt = kd.y < nb ? rootq[(int64_t)kd.y * kp + r] : Qp[(int64_t)plan.top_nodes[kd.y - nb] * kp + r];
            float2 sum = f2_add(l, rt);
            int64_t o = (int64_t)plan.top_nodes[q] * kp + r;
            Qp[o] = sum;
            Qf[o] = sum.x;
        }
        __syncthreads();  // this level's charges are visible to the CTA's next level
    }
}

// Down-sweep, mixed: k_down_blk with the link potentials (the link
// product's compensated (sum, correction) pairs) propagated in FP32 pairs,
// one thread per node carrying KC right-hand sides; CTA (block, y) takes
// columns y*KC .. y*KC+KC-1. Every internal node, level by level from the
// root, adds its A to both children's P (an internal child's sum is its A,
// a leaf's is its potential P(leaf) + A(parent)); every leaf writes
// v = x * sr + potential in FP64 for its columns below k, sr being the
// leaf's self term times its Jacobi scale.
template <int KC>
__global__ void __launch_bounds__(kSweepThreads, 8) k_down_blk32(const SweepPlan plan, const double *__restrict__ in, int64_t ld,
                                                                 int k, int kp, const double *__restrict__ sr,
                                                                 const float2 *__restrict__ P, double *__restrict__ out) {
    extern __shared__ __align__(16) float2 shp[];
    float2 *pv = shp;                                    // (2 kBlockLeaves - 1) x KC: P, then A (potential at leaves)
    float2 *cp = pv + (2 * kBlockLeaves - 1) * KC;       // kMaxChain x KC: P of the root's ancestors
    double *ss = (double *)(cp + kMaxChain * KC);        // kBlockLeaves: leaf self x scale
    uint32_t *kids = (uint32_t *)(ss + kBlockLeaves);    // kBlockLeaves
    int32_t *lbl = (int32_t *)(kids + kBlockLeaves);     // kBlockLeaves: internal node labels
    int32_t *chl = lbl + kBlockLeaves;                   // kMaxChain: ancestor labels
    int32_t *lp = chl + kMaxChain;                       // kBlockLeaves + 1
    const int b = blockIdx.x, tid = threadIdx.x, c0 = blockIdx.y * KC;
    const int lf = plan.blk_leaf_first[b], nl = plan.blk_nleaves[b], lv0 = plan.blk_lvl_first[b], H = plan.blk_nlvls[b];
    const int base = plan.blk_node_first[b], ni = nl - 1;
    const int ch0 = plan.blk_chain[b], nc = plan.blk_chain[b + 1] - ch0;
    for (int t = tid; t < kBlockLeaves; t += blockDim.x) {
        if (t < ni) {
            kids[t] = plan.lvl_kids[base + t];
            lbl[t] = plan.lvl_nodes[base + t];
        }
        if (t < nl) ss[t] = sr[lf + t];
        if (t < nc) chl[t] = plan.chain[ch0 + t];
    }
    for (int t = tid; t <= H; t += blockDim.x) lp[t] = plan.lvl_ptr[lv0 + t] - base;
    // the leaves' link potentials need no label: load them with the labels
    float2 v[KC];
    for (int i = tid; i < nl; i += blockDim.x) {
        load_pairs<KC>(P + (int64_t)(lf + i) * kp + c0, v);
        store_pairs<KC>(pv + i * KC, v);
    }
    __syncthreads();
    for (int t = tid; t < ni; t += blockDim.x) {
        load_pairs<KC>(P + (int64_t)lbl[t] * kp + c0, v);
        store_pairs<KC>(pv + (nl + t) * KC, v);
    }
    for (int t = tid; t < nc; t += blockDim.x) {
        load_pairs<KC>(P + (int64_t)chl[t] * kp + c0, v);
        store_pairs<KC>(cp + t * KC, v);
    }
    __syncthreads();
    if (tid < KC && nc > 0) {
        float2 acc = cp[(nc - 1) * KC + tid];
        for (int j = nc - 2; j >= 0; j--) acc = f2_add(cp[j * KC + tid], acc);
        // A of the block root (P(leaf) + A(parent) for a single-leaf block)
        pv[(nl + ni - 1) * KC + tid] = f2_add(pv[(nl + ni - 1) * KC + tid], acc);
    }
    __syncthreads();
    for (int h = H - 1; h >= 0; h--) {
        const int a = lp[h], cnt = lp[h + 1] - a;
        for (int t = tid; t < cnt; t += blockDim.x) {
            const int q = a + t;
            float2 A[KC], u[KC];
            load_pairs<KC>(pv + (nl + q) * KC, A);
            const uint32_t kd = kids[q];
            const int c1 = kd & 0xffffu, c2 = kd >> 16;
            load_pairs<KC>(pv + c1 * KC, u);
#pragma unroll
            for (int r = 0; r < KC; r++) u[r] = f2_add(u[r], A[r]);
            store_pairs<KC>(pv + c1 * KC, u);
            load_pairs<KC>(pv + c2 * KC, u);
#pragma unroll
            for (int r = 0; r < KC; r++) u[r] = f2_add(u[r], A[r]);
            store_pairs<KC>(pv + c2 * KC, u);
        }
        __syncthreads();
    }
    for (int i = tid; i < nl; i += blockDim.x) {
        const int j = lf + i;
        double x[KC];
#pragma unroll
        for (int r = 0; r < KC; r++) x[r] = c0 + r < k ? in[(int64_t)(c0 + r) * ld + j] : 0.0;
        float2 pt[KC];
        load_pairs<KC>(pv + i * KC, pt);
        const double sj = ss[i];
#pragma unroll
        for (int r = 0; r < KC; r++)
            if (c0 + r < k) out[(int64_t)(c0 + r) * ld + j] = fma(x[r], sj, f2d_bits(pt[r].x)) + f2d_bits(pt[r].y);
    }
}

// Link product, FP64 (CMultHier::ComputePanelPotentials_2fast,
// Solver/MultiplyHierarchical.cpp:141-226): SW lanes per destination node
// (32/SW nodes per warp in flight), lanes stride over the node's links four
// at a time with independent loads, K right-hand sides per link.
template <int K, int SW>
__global__ void k_spmv64(int64_t Nn, const int64_t *__restrict__ ptr, const uint32_t *__restrict__ src,
                         const double *__restrict__ coef, const double *__restrict__ Q, double *__restrict__ P) {
    const int G = 32 / SW;
    int lane = threadIdx.x & 31, gl = lane % SW;
    int64_t grp = ((blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5) * G + lane / SW;
    int64_t ngrp = (((int64_t)gridDim.x * blockDim.x) >> 5) * G;
    for (int64_t base = grp - lane / SW; base < Nn; base += ngrp) {
        int64_t row = base + lane / SW;
        bool valid = row < Nn;
        double acc[K];
#pragma unroll
        for (int r = 0; r < K; r++) acc[r] = 0.0;
        int s = valid ? (int)ptr[row] : 0, e = valid ? (int)ptr[row + 1] : 0;
        int l = s + gl;
        for (; l + 3 * SW < e; l += 4 * SW) {
            double c[4];
            uint32_t j[4];
#pragma unroll
            for (int u = 0; u < 4; u++) { c[u] = __ldcs(&coef[l + SW * u]); j[u] = __ldcs(&src[l + SW * u]) & kSrcMask; }
#pragma unroll
            for (int u = 0; u < 4; u++) {
                const double *q = Q + (int64_t)j[u] * K;
#pragma unroll
                for (int r = 0; r < K; r++) acc[r] += c[u] * q[r];
            }
        }
        if (l < e) {
            double c[4];
            uint32_t j[4];
#pragma unroll
            for (int u = 0; u < 4; u++) {
                bool ok = l + SW * u < e;
                c[u] = ok ? __ldcs(&coef[l + SW * u]) : 0.0;
                j[u] = ok ? (__ldcs(&src[l + SW * u]) & kSrcMask) : 0u;
            }
#pragma unroll
            for (int u = 0; u < 4; u++) {
                if (l + SW * u < e) {
                    const double *q = Q + (int64_t)j[u] * K;
#pragma unroll
                    for (int r = 0; r < K; r++) acc[r] += c[u] * q[r];
                }
            }
        }
#pragma unroll
        for (int r = 0; r < K; r++) {
#pragma unroll
            for (int o = SW / 2; o > 0; o >>= 1) acc[r] += __shfl_xor_sync(0xffffffffu, acc[r], o);
        }
        if (valid) {
#pragma unroll
            for (int r = 0; r < K; r++)
                if (gl == (r % SW)) P[row * K + r] = acc[r];
        }
    }
}

// Compensated FP32 accumulation (Kahan-Babuska / Neumaier). Each product is
// split exactly into p + e with one FMA (e = c*q - p) and e joins the
// compensation. The row sum leaves the kernel as the unevaluated pair
// (sum, compensation), combined in FP64 by the down-sweep, so that no FP64
// instruction runs in this kernel.
// Compensated FP32 sum: the value is s + c.
struct KSum {
    float s, c;
};
// Neumaier's update, used where two partial sums meet (lane reductions)
__device__ __forceinline__ void kadd(KSum &a, float x) {
    float t = a.s + x;
    if (fabsf(a.s) >= fabsf(x)) a.c += (a.s - t) + x;
    else a.c += (x - t) + a.s;
    a.s = t;
}
// Kahan's update with the product folded in: y = c*q + correction is one
// fused multiply-add (the product's rounding is of the order of the FP32
// coefficient's own), then t = s + y and the new correction is the part of y
// that t lost. Four instructions per link and right-hand side.
__device__ __forceinline__ void kmul_add(KSum &a, float c, float q) {
    float y = fmaf(c, q, a.c);
    float t = a.s + y;
    a.c = y - (t - a.s);
    a.s = t;
}
// Kahan's update with a short plain FP32 sum of products (a group of links):
// the group sum's rounding is of the order of the FP32 coefficients' own, the
// compensation then carries across groups. Four instructions per group.
__device__ __forceinline__ void kgroup_add(KSum &a, float x) {
    float y = x + a.c;
    float t = a.s + y;
    a.c = y - (t - a.s);
    a.s = t;
}

template <int K> __device__ __forceinline__ void load_q(const float *__restrict__ Q, uint32_t j, float *q) {
    if (K % 4 == 0) {
        const float4 *q4 = reinterpret_cast<const float4 *>(Q + (int64_t)j * K);
#pragma unroll
        for (int r = 0; r < K / 4; r++) {
            float4 v = q4[r];
            q[4 * r] = v.x; q[4 * r + 1] = v.y; q[4 * r + 2] = v.z; q[4 * r + 3] = v.w;
        }
    } else {
#pragma unroll
        for (int r = 0; r < K; r++) q[r] = Q[(int64_t)j * K + r];
    }
}

// Link product, mixed: FP32 coefficients and charges streamed, compensated
// FP32 sums; SW lanes per destination node (32/SW nodes per
// warp in flight), four independent links per lane.
template <int K, int SW>
__global__ void k_spmv32(int64_t Nn, const int64_t *__restrict__ ptr, const uint32_t *__restrict__ src,
                         const float *__restrict__ coef, const float *__restrict__ Q, float2 *__restrict__ P) {
    const int G = 32 / SW;
    int lane = threadIdx.x & 31, gl = lane % SW;
    int64_t grp = ((blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5) * G + lane / SW;
    int64_t ngrp = (((int64_t)gridDim.x * blockDim.x) >> 5) * G;
    for (int64_t base = grp - lane / SW; base < Nn; base += ngrp) {
        int64_t row = base + lane / SW;
        bool valid = row < Nn;
        KSum acc[K];
#pragma unroll
        for (int r = 0; r < K; r++) { acc[r].s = 0.f; acc[r].c = 0.f; }
        int s = valid ? (int)ptr[row] : 0, e = valid ? (int)ptr[row + 1] : 0;
        int l = s + gl;
        // four links per lane and pass, their products summed plainly and
        // then added to the compensated sums (kgroup_add)
        for (; l + 3 * SW < e; l += 4 * SW) {
            float c[4];
            uint32_t j[4];
#pragma unroll
            for (int u = 0; u < 4; u++) { c[u] = __ldcs(&coef[l + SW * u]); j[u] = __ldcs(&src[l + SW * u]) & kSrcMask; }
            float t[K];
#pragma unroll
            for (int u = 0; u < 4; u++) {
                float q[K];
                load_q<K>(Q, j[u], q);
#pragma unroll
                for (int r = 0; r < K; r++) t[r] = u == 0 ? c[0] * q[r] : fmaf(c[u], q[r], t[r]);
            }
#pragma unroll
            for (int r = 0; r < K; r++) kgroup_add(acc[r], t[r]);
        }
        if (l < e) {
            // the rest of the row (fewer than 4 links per lane): every load
            // is issued before the first charge is used, as in the loop
            float c[4];
            uint32_t j[4];
#pragma unroll
            for (int u = 0; u < 4; u++) {
                bool ok = l + SW * u < e;
                c[u] = ok ? __ldcs(&coef[l + SW * u]) : 0.f;
                j[u] = ok ? (__ldcs(&src[l + SW * u]) & kSrcMask) : 0u;
            }
            float t[K];
#pragma unroll
            for (int r = 0; r < K; r++) t[r] = 0.f;
#pragma unroll
            for (int u = 0; u < 4; u++) {
                if (l + SW * u < e) {
                    float q[K];
                    load_q<K>(Q, j[u], q);
#pragma unroll
                    for (int r = 0; r < K; r++) t[r] = fmaf(c[u], q[r], t[r]);
                }
            }
#pragma unroll
            for (int r = 0; r < K; r++) kgroup_add(acc[r], t[r]);
        }
#pragma unroll
        for (int r = 0; r < K; r++) {
            KSum a = acc[r];
#pragma unroll
            for (int o = SW / 2; o > 0; o >>= 1) {
                float os = __shfl_xor_sync(0xffffffffu, a.s, o);
                float oc = __shfl_xor_sync(0xffffffffu, a.c, o);
                a.c += oc;
                kadd(a, os);
            }
            acc[r] = a;
        }
        if (valid) {
#pragma unroll
            for (int r = 0; r < K; r++)
                if (gl == (r % SW)) P[row * K + r] = make_float2(acc[r].s, acc[r].c);
        }
    }
}

// Reduction of the link slots of a multi-right-hand-side warp: lane
// li * LPL + ri holds slot li (of LPW) for right-hand-side group ri; after
// the tree, slot 0 holds the sum of all slots (fixed order).
template <int LPL, int LPW> __device__ __forceinline__ void slot_reduce(KSum &a, int lane, int li) {
#pragma unroll
    for (int o = 1; o < LPW; o <<= 1) {
        int from = lane + o * LPL;
        float os = __shfl_sync(0xffffffffu, a.s, from < 32 ? from : lane);
        float oc = __shfl_sync(0xffffffffu, a.c, from < 32 ? from : lane);
        if ((li & (2 * o - 1)) == 0 && li + o < LPW) {
            a.c += oc;
            kadd(a, os);
        }
    }
}
template <int LPL, int LPW> __device__ __forceinline__ double slot_reduce64(double a, int lane, int li) {
#pragma unroll
    for (int o = 1; o < LPW; o <<= 1) {
        int from = lane + o * LPL;
        double oa = __shfl_sync(0xffffffffu, a, from < 32 ? from : lane);
        if ((li & (2 * o - 1)) == 0 && li + o < LPW) a += oa;
    }
    return a;
}

// Link product for K = 4, 8, ..., 32 right-hand sides, mixed: K/4 lanes
// share a link and each owns four right-hand sides (one 16-byte charge
// gather per link); a warp has 32/(K/4) link slots (lanes beyond them idle).
// CTA b owns the contiguous rows [row_split[b], row_split[b+1]) (split for
// equal link counts), its warps take every eighth row: consecutive rows
// share most of their sources, so the gathers hit L1.
template <int K>
__global__ void __launch_bounds__(256) k_spmv32_multi(const int32_t *__restrict__ row_split, const int64_t *__restrict__ ptr,
                                                      const uint32_t *__restrict__ src, const float *__restrict__ coef,
                                                      const float *__restrict__ Q, float2 *__restrict__ P) {
    constexpr int LPL = K / 4, LPW = 32 / LPL;
    // from 20 columns on (at most six slots) a row's slot sums meet in shared
    // memory: lane c < K adds the slots' (sum, correction) pairs of column c
    // in slot order and writes it (fewer instructions than the shuffle tree;
    // with eight or more slots the extra shared-memory wavefronts cost more
    // than they save: 16-column slab product 0.538 -> 0.593 ms)
    constexpr bool SMEM_RED = K >= 20;
    __shared__ __align__(16) KSum red[SMEM_RED ? 8 : 1][SMEM_RED ? LPW * K : 1];
    int lane = threadIdx.x & 31, li = lane / LPL, ri = lane % LPL;
    KSum *wred = red[SMEM_RED ? (threadIdx.x >> 5) : 0];
    bool slot_ok = li < LPW;
    const float4 *Q4 = reinterpret_cast<const float4 *>(Q);
    int r0 = row_split[blockIdx.x], r1 = row_split[blockIdx.x + 1];
    for (int row = r0 + (threadIdx.x >> 5); row < r1; row += 8) {
        KSum acc[4];
#pragma unroll
        for (int r = 0; r < 4; r++) { acc[r].s = 0.f; acc[r].c = 0.f; }
        int s = (int)ptr[row], e = (int)ptr[row + 1];
        int l = s + li;
        if (slot_ok) {
            if constexpr (K >= 16) {
                // four links per slot and pass (four charge gathers in flight
                // per lane), their products summed plainly, then added to
                // the compensated sums (served 22-column requests: 1.5 %
                // faster than two per pass)
                for (; l + 3 * LPW < e; l += 4 * LPW) {
                    float c0 = __ldcs(&coef[l]), c1 = __ldcs(&coef[l + LPW]);
                    float c2 = __ldcs(&coef[l + 2 * LPW]), c3 = __ldcs(&coef[l + 3 * LPW]);
                    uint32_t j0 = __ldcs(&src[l]) & kSrcMask, j1 = __ldcs(&src[l + LPW]) & kSrcMask;
                    uint32_t j2 = __ldcs(&src[l + 2 * LPW]) & kSrcMask, j3 = __ldcs(&src[l + 3 * LPW]) & kSrcMask;
                    float4 q0 = Q4[(int64_t)j0 * LPL + ri], q1 = Q4[(int64_t)j1 * LPL + ri];
                    float4 q2 = Q4[(int64_t)j2 * LPL + ri], q3 = Q4[(int64_t)j3 * LPL + ri];
                    kgroup_add(acc[0], fmaf(c3, q3.x, fmaf(c2, q2.x, fmaf(c1, q1.x, c0 * q0.x))));
                    kgroup_add(acc[1], fmaf(c3, q3.y, fmaf(c2, q2.y, fmaf(c1, q1.y, c0 * q0.y))));
                    kgroup_add(acc[2], fmaf(c3, q3.z, fmaf(c2, q2.z, fmaf(c1, q1.z, c0 * q0.z))));
                    kgroup_add(acc[3], fmaf(c3, q3.w, fmaf(c2, q2.w, fmaf(c1, q1.w, c0 * q0.w))));
                }
            }
            // two links per slot and pass; from 16 columns on (issue bound)
            // their products are summed plainly, then added to the
            // compensated sums (kgroup_add), below that each is (kmul_add)
            for (; l + LPW < e; l += 2 * LPW) {
                float c0 = __ldcs(&coef[l]), c1 = __ldcs(&coef[l + LPW]);
                uint32_t j0 = __ldcs(&src[l]) & kSrcMask, j1 = __ldcs(&src[l + LPW]) & kSrcMask;
                float4 q0 = Q4[(int64_t)j0 * LPL + ri], q1 = Q4[(int64_t)j1 * LPL + ri];
                if constexpr (K >= 16) {
                    kgroup_add(acc[0], fmaf(c1, q1.x, c0 * q0.x));
                    kgroup_add(acc[1], fmaf(c1, q1.y, c0 * q0.y));
                    kgroup_add(acc[2], fmaf(c1, q1.z, c0 * q0.z));
                    kgroup_add(acc[3], fmaf(c1, q1.w, c0 * q0.w));
                } else {
                    kmul_add(acc[0], c0, q0.x); kmul_add(acc[1], c0, q0.y); kmul_add(acc[2], c0, q0.z); kmul_add(acc[3], c0, q0.w);
                    kmul_add(acc[0], c1, q1.x); kmul_add(acc[1], c1, q1.y); kmul_add(acc[2], c1, q1.z); kmul_add(acc[3], c1, q1.w);
                }
            }
            if (l < e) {
                float c0 = __ldcs(&coef[l]);
                uint32_t j0 = __ldcs(&src[l]) & kSrcMask;
                float4 q0 = Q4[(int64_t)j0 * LPL + ri];
                kmul_add(acc[0], c0, q0.x); kmul_add(acc[1], c0, q0.y); kmul_add(acc[2], c0, q0.z); kmul_add(acc[3], c0, q0.w);
            }
        }
        if constexpr (SMEM_RED) {
            if (slot_ok) {
                float4 *o = reinterpret_cast<float4 *>(wred + li * K + 4 * ri);
                o[0] = make_float4(acc[0].s, acc[0].c, acc[1].s, acc[1].c);
                o[1] = make_float4(acc[2].s, acc[2].c, acc[3].s, acc[3].c);
            }
            __syncwarp();
            if (lane < K) {
                KSum a = wred[lane];
#pragma unroll
                for (int q = 1; q < LPW; q++) {
                    const KSum b = wred[q * K + lane];
                    a.c += b.c;
                    kadd(a, b.s);
                }
                P[(int64_t)row * K + lane] = make_float2(a.s, a.c);
            }
            __syncwarp();  // the buffer is reused by the warp's next row
        } else {
#pragma unroll
            for (int r = 0; r < 4; r++) slot_reduce<LPL, LPW>(acc[r], lane, li);
            if (li == 0) {
                float4 *out = reinterpret_cast<float4 *>(P + (int64_t)row * K + 4 * ri);
                out[0] = make_float4(acc[0].s, acc[0].c, acc[1].s, acc[1].c);
                out[1] = make_float4(acc[2].s, acc[2].c, acc[3].s, acc[3].c);
            }
        }
    }
}

// FP64 counterpart: K/2 lanes share a link, each lane owns two right-hand sides.
template <int K>
__global__ void __launch_bounds__(256) k_spmv64_multi(const int32_t *__restrict__ row_split, const int64_t *__restrict__ ptr,
                                                      const uint32_t *__restrict__ src, const double *__restrict__ coef,
                                                      const double *__restrict__ Q, double *__restrict__ P) {
    constexpr int LPL = K / 2, LPW = 32 / LPL;
    int lane = threadIdx.x & 31, li = lane / LPL, ri = lane % LPL;
    bool slot_ok = li < LPW;
    const double2 *Q2 = reinterpret_cast<const double2 *>(Q);
    int r0 = row_split[blockIdx.x], r1 = row_split[blockIdx.x + 1];
    for (int row = r0 + (threadIdx.x >> 5); row < r1; row += 8) {
        double a0 = 0.0, a1 = 0.0;
        int s = (int)ptr[row], e = (int)ptr[row + 1];
        int l = s + li;
        if (slot_ok) {
            for (; l + LPW < e; l += 2 * LPW) {
                double c0 = __ldcs(&coef[l]), c1 = __ldcs(&coef[l + LPW]);
                uint32_t j0 = __ldcs(&src[l]) & kSrcMask, j1 = __ldcs(&src[l + LPW]) & kSrcMask;
                double2 q0 = Q2[(int64_t)j0 * LPL + ri], q1 = Q2[(int64_t)j1 * LPL + ri];
                a0 += c0 * q0.x; a1 += c0 * q0.y;
                a0 += c1 * q1.x; a1 += c1 * q1.y;
            }
            if (l < e) {
                double c0 = __ldcs(&coef[l]);
                double2 q0 = Q2[(int64_t)(__ldcs(&src[l]) & kSrcMask) * LPL + ri];
                a0 += c0 * q0.x; a1 += c0 * q0.y;
            }
        }
        a0 = slot_reduce64<LPL, LPW>(a0, lane, li);
        a1 = slot_reduce64<LPL, LPW>(a1, lane, li);
        if (li == 0) reinterpret_cast<double2 *>(P + (int64_t)row * K)[ri] = make_double2(a0, a1);
    }
}

// ---- two-level preconditioner (CSolveCap::MakePreconditioner,
// ComputeSuperPrecond, InvertMatrix, ComputePrecondVectFast super branch;
// Solver/SolveCapacitance.cpp:1061-1133, 2007-2066, 2116-2258, 3547-3598)

__global__ void k_node_leafflag(int64_t Nn, const NodeGeo *__restrict__ geo, uint8_t *__restrict__ leaf) {
    for (int64_t v = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; v < Nn; v += (int64_t)gridDim.x * blockDim.x)
        leaf[v] = (geo[v].type & FCG_IS_LEAF) ? 1 : 0;
}

// leaf -> element map, leaf areas (single precision, as the reference keeps
// them), element areas
__global__ void k_sup_maps(int m, const int32_t *__restrict__ elem, const int64_t *__restrict__ first,
                           const int64_t *__restrict__ count, const NodeGeo *__restrict__ geo, const int32_t *__restrict__ leaf_node,
                           int32_t *__restrict__ index, float *__restrict__ area, double *__restrict__ dimv) {
    int s = blockIdx.x;
    if (s >= m) return;
    if (threadIdx.x == 0) dimv[s] = geo[elem[s]].area;
    for (int64_t j = first[s] + threadIdx.x; j < first[s] + count[s]; j += blockDim.x) {
        index[j] = s;
        area[j] = (float)geo[leaf_node[j]].area;
    }
}

// super potential matrix A (row-major): self terms on the diagonal, the
// one-way coefficient of element i's evaluation point due to element j off it
__global__ void k_sup_matrix(int m, const int32_t *__restrict__ elem, const int64_t *__restrict__ first,
                             const NodeGeo *__restrict__ geo, const double *__restrict__ leaf_eb, const double *__restrict__ leaf_ea,
                             double *__restrict__ A) {
    int64_t n = (int64_t)m * m;
    for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < n; t += (int64_t)gridDim.x * blockDim.x) {
        int i = (int)(t / m), j = (int)(t - (int64_t)i * m);
        const NodeGeo &gi = geo[elem[i]];
        double v;
        if (i == j) {
            if (gi.type & FCG_IS_DIEL) {
                double eb = leaf_eb[first[i]], ea = leaf_ea[first[i]];
                v = (ea + eb) / (FCG_TWO_TIMES_E0 * (eb - ea) * gi.area);
            } else {
                v = fcg_potential_opt(fcg_widen(gi.c), gi.v) / FCG_FOUR_PI_TIMES_E0;
            }
        } else {
            const NodeGeo &gj = geo[elem[j]];
            v = fcg_pot_estimate(gi.type, gi.c, gi.n, gi.maxside, gj.c, gj.v, gj.maxside);
        }
        A[t] = v;
    }
}

// LU step j, part 1 (one CTA): pivot = first row of largest |A[i][j]|, i >= j;
// swap rows j and pivot; scale the column below the diagonal
__global__ void k_lu_pivot(int m, int j, double *__restrict__ A, int32_t *__restrict__ piv) {
    __shared__ double bv[32];
    __shared__ int bi[32];
    __shared__ int pv;
    double best = -1.0;
    int bidx = m;
    for (int i = j + threadIdx.x; i < m; i += blockDim.x) {
        double a = fabs(A[(int64_t)i * m + j]);
        if (a > best) { best = a; bidx = i; }  // ascending i per thread: first on ties
    }
    for (int o = 16; o > 0; o >>= 1) {
        double ob = __shfl_xor_sync(0xffffffffu, best, o);
        int oi = __shfl_xor_sync(0xffffffffu, bidx, o);
        if (ob > best || (ob == best && oi < bidx)) { best = ob; bidx = oi; }
    }
    int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
    if (lane == 0) { bv[w] = best; bi[w] = bidx; }
    __syncthreads();
    if (threadIdx.x == 0) {
        double b = bv[0];
        int bx = bi[0];
        for (int q = 1; q < (int)(blockDim.x >> 5); q++)
            if (bv[q] > b || (bv[q] == b && bi[q] < bx)) { b = bv[q]; bx = bi[q]; }
        if (bx >= m) bx = j;
        pv = bx;
        piv[j] = bx;
    }
    __syncthreads();
    int pr = pv;
    if (pr != j)
        for (int k = threadIdx.x; k < m; k += blockDim.x) {
            double t = A[(int64_t)j * m + k];
            A[(int64_t)j * m + k] = A[(int64_t)pr * m + k];
            A[(int64_t)pr * m + k] = t;
        }
    __syncthreads();
    if (j < m - 1) {
        double r = 1.0 / A[(int64_t)j * m + j];
        for (int i = j + 1 + threadIdx.x; i < m; i += blockDim.x) A[(int64_t)i * m + j] *= r;
    }
}

// LU step j, part 2: rank-1 update of the trailing block
__global__ void k_lu_update(int m, int j, double *__restrict__ A) {
    int64_t w = m - j - 1, n = w * w;
    for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < n; t += (int64_t)gridDim.x * blockDim.x) {
        int64_t i = j + 1 + t / w, k = j + 1 + t % w;
        A[i * m + k] -= A[i * m + j] * A[(int64_t)j * m + k];
    }
}

// X = the identity with the factorisation's row swaps applied (one CTA)
__global__ void k_perm_identity(int m, const int32_t *__restrict__ piv, int32_t *__restrict__ idx, double *__restrict__ X) {
    if (threadIdx.x == 0) {
        for (int i = 0; i < m; i++) idx[i] = i;
        for (int i = 0; i < m; i++) {
            int t = idx[i];
            idx[i] = idx[piv[i]];
            idx[piv[i]] = t;
        }
    }
    __syncthreads();
    for (int64_t t = threadIdx.x; t < (int64_t)m * m; t += blockDim.x) {
        int i = (int)(t / m), k = (int)(t % m);
        X[t] = idx[i] == k ? 1.0 : 0.0;
    }
}

// forward substitution step i (unit lower factor): rows below i lose L[r][i] * row i
__global__ void k_inv_forward(int m, int i, const double *__restrict__ A, double *__restrict__ X) {
    int64_t n = (int64_t)(m - i - 1) * m;
    for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < n; t += (int64_t)gridDim.x * blockDim.x) {
        int64_t r = i + 1 + t / m, k = t % m;
        X[r * m + k] -= A[r * m + i] * X[(int64_t)i * m + k];
    }
}

// backward substitution step i: row i is divided by U[i][i], rows above lose U[r][i] * row i
__global__ void k_inv_scale(int m, int i, const double *__restrict__ A, double *__restrict__ X) {
    double d = A[(int64_t)i * m + i];
    for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < m; k += gridDim.x * blockDim.x) X[(int64_t)i * m + k] /= d;
}
__global__ void k_inv_backward(int m, int i, const double *__restrict__ A, double *__restrict__ X) {
    int64_t n = (int64_t)i * m;
    for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < n; t += (int64_t)gridDim.x * blockDim.x) {
        int64_t r = t / m, k = t % m;
        X[r * m + k] -= A[r * m + i] * X[(int64_t)i * m + k];
    }
}

// T = X transposed (column-major inverse, coalesced in the product), its
// diagonal, and a count of non-finite entries
__global__ void k_inv_finish(int m, const double *__restrict__ X, double *__restrict__ T, double *__restrict__ diag, unsigned *bad) {
    int64_t n = (int64_t)m * m;
    unsigned nb = 0;
    for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < n; t += (int64_t)gridDim.x * blockDim.x) {
        int64_t r = t / m, k = t % m;
        double v = X[t];
        if (!isfinite(v)) nb++;
        T[k * m + r] = v;
        if (r == k) diag[r] = v;
    }
    if (nb) atomicAdd(bad, nb);
}

// apply, step 1: pot[r][s] = sum over element s's leaves (leaf order) of q * area / dim
__global__ void k_sup_collect(int m, int k, int64_t Np, const int64_t *__restrict__ first, const int64_t *__restrict__ count,
                              const float *__restrict__ area, const double *__restrict__ dimv, const double *__restrict__ in,
                              double *__restrict__ pot) {
    int64_t n = (int64_t)m * k;
    for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < n; t += (int64_t)gridDim.x * blockDim.x) {
        int s = (int)(t % m), r = (int)(t / m);
        const double *q = in + (int64_t)r * Np;
        double acc = 0.0, d = dimv[s];
        for (int64_t j = first[s]; j < first[s] + count[s]; j++) acc += q[j] * (double)area[j] / d;
        pot[t] = acc;
    }
}

// step 2: chg[r][s] = sum over k != s (ascending) of Minv[s][k] * pot[r][k]
__global__ void k_sup_mult(int m, int k, const double *__restrict__ T, const double *__restrict__ pot, double *__restrict__ chg) {
    int64_t n = (int64_t)m * k;
    for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < n; t += (int64_t)gridDim.x * blockDim.x) {
        int s = (int)(t % m), r = (int)(t / m);
        const double *pr = pot + (int64_t)r * m;
        double acc = 0.0;
        for (int q = 0; q < m; q++)
            if (q != s) acc += T[(int64_t)q * m + s] * pr[q];
        chg[t] = acc;
    }
}

// step 3: out = chg * area / dim + Minv[s][s] * q * area / dim per leaf
__global__ void k_sup_spread(int m, int k, int64_t Np, const int32_t *__restrict__ index, const float *__restrict__ area,
                             const double *__restrict__ dimv, const double *__restrict__ diag, const double *__restrict__ chg,
                             const double *__restrict__ in, double *__restrict__ out) {
    int64_t n = (int64_t)k * Np;
    for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < n; t += (int64_t)gridDim.x * blockDim.x) {
        int r = (int)(t / Np);
        int64_t j = t - (int64_t)r * Np;
        int s = index[j];
        double a = (double)area[j], d = dimv[s];
        double v = chg[(int64_t)r * m + s] * a / d;
        v += diag[s] * in[t] * a / d;
        out[t] = v;
    }
}

// ---- Krylov kernels (CSolveCap::gmresPrecondSFastAll, Solver/SolveCapacitance.cpp:2288-2574)
//
// Vectors are [ks][Np]: column r of every vector carries one independent
// solve per geometry g, solve s = g * ks + r, on g's leaf range. Reductions
// run over chunks that never cross a geometry, so every solve has its own dot
// products, norms, Givens rotations, iteration count and convergence test.
// Hessenberg column i of all solves is one array Hc[i] of S * (i + 2) values.

struct SegChunks {
    const int64_t *start;  // first leaf of each chunk
    const int32_t *len;    // leaves in each chunk (<= kDotChunk)
    const int32_t *geom;   // geometry of each chunk
    int n;
};

// b[r][j] = 1 on the leaves of solve (geometry of j, r)'s conductor
__global__ void k_set_rhs(int64_t Np, int ks, const int32_t *__restrict__ leaf_geom, const int64_t *__restrict__ sf,
                          const int64_t *__restrict__ sc, double *__restrict__ b) {
    int64_t n = (int64_t)ks * Np;
    for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < n; t += (int64_t)gridDim.x * blockDim.x) {
        int r = (int)(t / Np);
        int64_t j = t - (int64_t)r * Np;
        int s = leaf_geom[j] * ks + r;
        b[t] = (j >= sf[s] && j < sf[s] + sc[s]) ? 1.0 : 0.0;
    }
}

// y = a / diag (Jacobi) or a copy
__global__ void k_precond(int64_t Np, int k, const double *__restrict__ a, const double *__restrict__ diag, double *__restrict__ y) {
    int64_t n = (int64_t)k * Np;
    for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < n; t += (int64_t)gridDim.x * blockDim.x) {
        int64_t j = t % Np;
        y[t] = diag ? a[t] / diag[j] : a[t];
    }
}

__device__ __forceinline__ double block_sum(double v, double *sh) {
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
    __syncthreads();
    if (lane == 0) sh[w] = v;
    __syncthreads();
    v = (threadIdx.x < (blockDim.x >> 5)) ? sh[threadIdx.x] : 0.0;
    if (w == 0)
        for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

// partial[(r*nvec + j)*nch + c] = <Vj[r], w[r]> over chunk c; the chunk of w
// stays in registers, basis vectors are taken eight at a time with one block
// reduction per group of eight.
__device__ __forceinline__ void reduce_h_warp(int64_t wid, int lane, int i, int ks, int nch, const double *partial,
                                              const int32_t *__restrict__ g_ch_first, const int32_t *__restrict__ g_ch_count,
                                              const int *__restrict__ active, double *const *__restrict__ Hp);

// With fuse_h set, the last CTA to finish (a ticket on *done) also sums the
// Hessenberg column (k_reduce_h's work) and resets *done. kDotThreads
// threads per chunk, each holding kDotChunk / kDotThreads elements of w: on
// GB300 the FP64 pipe bounds the FP64 variant, and the FP64 additions of the
// cross-lane reductions are paid per group of eight vectors, so fewer,
// fuller threads spend a smaller share of the pipe on them. PB (the mixed
// path): basis vectors are FP32 pairs, w is split into pairs once and every
// product and sum is pair arithmetic on the FP32 pipe (f2_fma, f2_add); the
// chunk's sums are rounded to FP64 once.
template <bool PB>
__global__ void __launch_bounds__(kDotThreads) k_dots(int64_t Np, const int *__restrict__ iter, double *const *__restrict__ Vp,
                                                      const double *__restrict__ w, SegChunks ch, int ks,
                                                      const int *__restrict__ active, double *__restrict__ partial, int fuse_h,
                                                      int G, const int32_t *__restrict__ g_ch_first,
                                                      const int32_t *__restrict__ g_ch_count, double *const *__restrict__ Hp,
                                                      int *done) {
    using E = typename std::conditional<PB, float2, double>::type;
    constexpr int NW = kDotThreads / 32, U = kDotChunk / kDotThreads;
    __shared__ E sh[NW][8];
    __shared__ int s_last;
    const int T = 8;
    const int nvec = *iter + 1;
    int r = blockIdx.y, c = blockIdx.x;
    // grid.z splits the basis vectors of a chunk over CTAs (groups of T
    // taken z, z + Z, ...); every (vector, chunk) sum is the same either way.
    // CTAs past the last group have nothing to do but take the ticket.
    const int z = blockIdx.z, Z = gridDim.z;
    if (z * T < nvec && active[ch.geom[c] * ks + r]) {
    int64_t base = ch.start[c];
    int len = ch.len[c];
    E wv[U];
#pragma unroll
    for (int u = 0; u < U; u++) {
        int o = threadIdx.x + u * kDotThreads;
        const double x = (o < len) ? w[(int64_t)r * Np + base + o] : 0.0;
        if constexpr (PB) wv[u] = d2pair_bits(x);
        else wv[u] = x;
    }
    int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    for (int j0 = z * T; j0 < nvec; j0 += Z * T) {
        E acc[T];
#pragma unroll
        for (int t = 0; t < T; t++) {
            acc[t] = kv_zero<E>();
            if (j0 + t < nvec) {
                const E *v = reinterpret_cast<const E *>(Vp[j0 + t]) + (int64_t)r * Np + base;
#pragma unroll
                for (int u = 0; u < U; u++) {
                    int o = threadIdx.x + u * kDotThreads;
                    if constexpr (PB) {
                        if (o < len) acc[t] = f2_fma(acc[t], v[o], wv[u]);
                    } else {
                        if (o < len) acc[t] += v[o] * wv[u];
                    }
                }
            }
        }
        // reduce the eight sums over the warp by halving: each step keeps
        // half of the values and adds the partner lane's copy of them
        // (4 + 2 + 1 exchanges), then the last value over lane pairs: lane l
        // ends with vector 4*bit4 + 2*bit3 + bit2 of its index
#pragma unroll
        for (int q = 0; q < 4; q++) {
            bool hi = lane & 16;
            E send = hi ? acc[q] : acc[q + 4];
            E keep = hi ? acc[q + 4] : acc[q];
            acc[q] = kv_add(keep, kv_shfl_xor(send, 16));
        }
#pragma unroll
        for (int q = 0; q < 2; q++) {
            bool hi = lane & 8;
            E send = hi ? acc[q] : acc[q + 2];
            E keep = hi ? acc[q + 2] : acc[q];
            acc[q] = kv_add(keep, kv_shfl_xor(send, 8));
        }
        {
            bool hi = lane & 4;
            E send = hi ? acc[0] : acc[1];
            E keep = hi ? acc[1] : acc[0];
            acc[0] = kv_add(keep, kv_shfl_xor(send, 4));
        }
        acc[0] = kv_add(acc[0], kv_shfl_xor(acc[0], 2));
        acc[0] = kv_add(acc[0], kv_shfl_xor(acc[0], 1));
        if ((lane & 3) == 0) sh[warp][((lane >> 4) & 1) * 4 + ((lane >> 3) & 1) * 2 + ((lane >> 2) & 1)] = acc[0];
        __syncthreads();
        if (threadIdx.x < T && j0 + threadIdx.x < nvec) {
            E sum = kv_zero<E>();
            for (int ww = 0; ww < NW; ww++) sum = kv_add(sum, sh[ww][threadIdx.x]);
            partial[((int64_t)r * nvec + j0 + threadIdx.x) * ch.n + c] = kv_double(sum);
        }
        __syncthreads();
    }
    }
    if (!fuse_h) return;
    if (threadIdx.x == 0) {
        __threadfence();  // this CTA's partial sums are visible before its ticket
        s_last = atomicAdd(done, 1) == (int)(gridDim.x * gridDim.y * gridDim.z) - 1;
    }
    __syncthreads();
    if (!s_last) return;
    __threadfence();
    const int lane = threadIdx.x & 31;
    for (int64_t wid = threadIdx.x >> 5; wid < (int64_t)nvec * ks * G; wid += blockDim.x >> 5)
        reduce_h_warp(wid, lane, nvec - 1, ks, ch.n, partial, g_ch_first, g_ch_count, active, Hp);
    if (threadIdx.x == 0) *done = 0;
}

// out[sidx*ostride_s + j*ostride_j] = sum of partial[(r*nvec + j)*nch + c]
// over geometry g's chunks, in chunk order; one warp per (j, r, g)
__global__ void k_reduce_seg(int nvec, int ks, int G, int nch, const double *__restrict__ partial,
                             const int32_t *__restrict__ g_ch_first, const int32_t *__restrict__ g_ch_count,
                             const int *__restrict__ active, double *__restrict__ out, int64_t ostride_s, int64_t ostride_j) {
    int64_t wid = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
    int lane = threadIdx.x & 31;
    if (wid >= (int64_t)nvec * ks * G) return;
    int j = (int)(wid % nvec);
    int64_t rg = wid / nvec;
    int r = (int)(rg % ks), g = (int)(rg / ks);
    int sidx = g * ks + r;
    if (active && !active[sidx]) return;
    double sum = 0.0;
    int c0 = g_ch_first[g], cn = g_ch_count[g];
    const double *pp = partial + ((int64_t)r * nvec + j) * nch + c0;
    for (int c = lane; c < cn; c += 32) sum += pp[c];
    for (int o = 16; o > 0; o >>= 1) sum += __shfl_xor_sync(0xffffffffu, sum, o);
    if (lane == 0) out[sidx * ostride_s + j * ostride_j] = sum;
}

// Givens update of Hessenberg column i of active solve sidx; true while the
// solve goes on
// one previous rotation applied to (t1, t2), every product rounded before
// the sum (no contraction: the per-solve and per-warp Givens kernels round
// the same way)
__device__ __forceinline__ double rot_lo(double c, double s, double t1, double t2) {
    return __dsub_rn(__dmul_rn(c, t1), __dmul_rn(s, t2));
}
__device__ __forceinline__ double rot_hi(double c, double s, double t1, double t2) {
    return __dadd_rn(__dmul_rn(c, t2), __dmul_rn(s, t1));
}

// the rest of a solve's Givens step once its column's previous rotations
// are applied (hc[0..i-1] rotated, `carry` the running entry i): the new
// rotation, the right-hand side, the convergence test
__device__ bool givens_finish(int sidx, int i, int M, double *hc, double carry, double hn, double *cs, double *sn, double *g,
                              const double *normb, double tol, const int *scap, int *active, int *iters, int *capped) {
    double *c = cs + (int64_t)sidx * (M + 2), *sv = sn + (int64_t)sidx * (M + 2), *gg = g + (int64_t)sidx * (M + 2);
    hc[i] = carry;
    double t1 = carry, t2 = hn;
    double len = __dsqrt_rn(__dadd_rn(__dmul_rn(t1, t1), __dmul_rn(t2, t2)));
    c[i] = t1 / len;
    sv[i] = -t2 / len;
    hc[i] = rot_lo(c[i], sv[i], t1, t2);
    hc[i + 1] = 0;
    t1 = gg[i];
    gg[i] = c[i] * t1;
    gg[i + 1] = sv[i] * t1;
    double res = fabs(gg[i + 1]) / normb[sidx];
    if (res < tol) {
        active[sidx] = 0;
        iters[sidx] = i;
    } else if (i + 1 >= scap[sidx]) {
        // the solve's iteration cap: keep the last Arnoldi step
        active[sidx] = 0;
        iters[sidx] = i;
        capped[sidx] = 1;
    } else {
        return true;
    }
    return false;
}

__device__ bool givens_one(int sidx, int i, int M, double *const *__restrict__ Hp, double *cs, double *sn, double *g,
                           const double *normb, const double *nrm2, double *hnorm, double *rhnorm, double tol, const int *scap,
                           int *active, int *iters, int *capped) {
    double *hc = Hp[i] + (int64_t)sidx * (i + 2);
    const double *c = cs + (int64_t)sidx * (M + 2), *sv = sn + (int64_t)sidx * (M + 2);
    double hn = sqrt(nrm2[sidx]);
    hnorm[sidx] = hn;
    if (rhnorm) rhnorm[sidx] = 1.0 / hn;
    hc[i + 1] = hn;
    // the previous rotations, in order; the running entry stays in a register
    // so the loads of the next column entries and rotations do not wait on it
    double carry = hc[0];
#pragma unroll 8
    for (int j = 0; j < i; j++) {
        double t1 = carry, t2 = hc[j + 1];
        hc[j] = rot_lo(c[j], sv[j], t1, t2);
        carry = rot_hi(c[j], sv[j], t1, t2);
    }
    return givens_finish(sidx, i, M, hc, carry, hn, cs, sn, g, normb, tol, scap, active, iters, capped);
}

// Givens update of Hessenberg column i of every active solve, one warp per solve: the lanes load 32 entries of the
// column and of the previous rotations at a time, and every lane runs the
// chain of rotations on shuffled values (the same operations in the same
// order as k_givens), so a step waits for memory once per 32 rotations.
__global__ void __launch_bounds__(128) k_givens_warp(int S, const int *__restrict__ iter, int M, double *const *__restrict__ Hp,
                                                     double *cs, double *sn, double *g, const double *normb, const double *nrm2,
                                                     double *hnorm, double *rhnorm, double tol, const int *scap, int *active,
                                                     int *iters, int *capped, int *n_active_all) {
    const int i = *iter;
    const int sidx = (int)((blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5), lane = threadIdx.x & 31;
    if (sidx >= S || !active[sidx]) return;  // the whole warp
    double *hc = Hp[i] + (int64_t)sidx * (i + 2);
    const double *c = cs + (int64_t)sidx * (M + 2), *sv = sn + (int64_t)sidx * (M + 2);
    const double hn = sqrt(nrm2[sidx]);
    double carry = hc[0];
    for (int j0 = 0; j0 < i; j0 += 32) {
        const int j = j0 + lane, cnt = min(32, i - j0);
        double cj = 0.0, sj = 0.0, hj = 0.0, out = 0.0;
        if (j < i) {
            cj = c[j];
            sj = sv[j];
            hj = hc[j + 1];
        }
        for (int q = 0; q < cnt; q++) {
            const double cq = __shfl_sync(0xffffffffu, cj, q), sq = __shfl_sync(0xffffffffu, sj, q);
            const double t1 = carry, t2 = __shfl_sync(0xffffffffu, hj, q);
            const double h = rot_lo(cq, sq, t1, t2);
            carry = rot_hi(cq, sq, t1, t2);
            if (lane == q) out = h;
        }
        __syncwarp();  // every lane has read the entries it overwrites next
        if (j < i) hc[j] = out;
    }
    if (lane != 0) return;
    hnorm[sidx] = hn;
    if (rhnorm) rhnorm[sidx] = 1.0 / hn;
    if (givens_finish(sidx, i, M, hc, carry, hn, cs, sn, g, normb, tol, scap, active, iters, capped))
        atomicAdd(n_active_all + i, 1);
}

// out[r][j] = v[r][j] / hn[solve of (j, r)] for active solves, out = out_fixed
// or basis vector *iter + vofs (as FP32 pairs when PB); v is rewritten with
// the same values in FP64 (it is the input of the next product)
template <bool PB>
__global__ void k_scale(int64_t Np, int ks, double *__restrict__ v, const double *__restrict__ hn, const int *__restrict__ active,
                        const int32_t *__restrict__ leaf_geom, double *__restrict__ out_fixed, double *const *__restrict__ Vp,
                        const int *__restrict__ iter, int vofs) {
    double *out = out_fixed ? out_fixed : Vp[*iter + vofs];
    int64_t n = (int64_t)ks * Np;
    for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < n; t += (int64_t)gridDim.x * blockDim.x) {
        int r = (int)(t / Np);
        int64_t j = t - (int64_t)r * Np;
        int sidx = leaf_geom[j] * ks + r;
        if (active && !active[sidx]) continue;
        double x = v[t] / hn[sidx];
        if constexpr (PB) reinterpret_cast<float2 *>(out)[t] = d2pair_bits(x);
        else out[t] = x;
        v[t] = x;
    }
}

// Hessenberg column *iter of every active solve: out = Hp[i] + sidx*(i+2) + j,
// j < i+1, summed over the solve's geometry chunks (one warp per output)
__device__ __forceinline__ void reduce_h_warp(int64_t wid, int lane, int i, int ks, int nch, const double *partial,
                                              const int32_t *__restrict__ g_ch_first, const int32_t *__restrict__ g_ch_count,
                                              const int *__restrict__ active, double *const *__restrict__ Hp) {
    const int nvec = i + 1;
    int j = (int)(wid % nvec);
    int64_t rg = wid / nvec;
    int r = (int)(rg % ks), g = (int)(rg / ks);
    int sidx = g * ks + r;
    if (!active[sidx]) return;
    double sum = 0.0;
    int c0 = g_ch_first[g], cn = g_ch_count[g];
    const double *pp = partial + ((int64_t)r * nvec + j) * nch + c0;
    for (int c = lane; c < cn; c += 32) sum += __ldcg(&pp[c]);
    for (int o = 16; o > 0; o >>= 1) sum += __shfl_xor_sync(0xffffffffu, sum, o);
    if (lane == 0) Hp[i][(int64_t)sidx * (i + 2) + j] = sum;
}

__global__ void k_reduce_h(int ks, int G, int nch, const int *__restrict__ iter, const double *__restrict__ partial,
                           const int32_t *__restrict__ g_ch_first, const int32_t *__restrict__ g_ch_count,
                           const int *__restrict__ active, double *const *__restrict__ Hp) {
    const int i = *iter, nvec = i + 1;
    int lane = threadIdx.x & 31;
    for (int64_t wid = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5; wid < (int64_t)nvec * ks * G;
         wid += ((int64_t)gridDim.x * blockDim.x) >> 5)
        reduce_h_warp(wid, lane, i, ks, nch, partial, g_ch_first, g_ch_count, active, Hp);
}

// end of an Arnoldi step (one thread): advance the step index; go on while
// a solve is active, the basis has room and no cancellation was asked for.
// Inside the graph's while loop it sets the loop condition.
__device__ void iter_advance_one(int *iter, int i, int na, int cap, const volatile int *cancel, int *state,
                                 cudaGraphConditionalHandle cond, int use_cond) {
    int go = na > 0 && i + 1 < cap && !(cancel && *cancel);
    *iter = i + 1;
    state[0] = go;
    state[1] = na;
    if (use_cond) cudaGraphSetConditional(cond, go ? 1u : 0u);
}

// end of an Arnoldi step (one thread): advance the step index; go on while
// a solve is active, the basis has room and no cancellation was asked for.
// Inside the graph's while loop it sets the loop condition.
__global__ void k_iter_advance(int *iter, const int *__restrict__ n_active, int cap, const volatile int *cancel, int *state,
                               cudaGraphConditionalHandle cond, int use_cond) {
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    int i = *iter;
    iter_advance_one(iter, i, n_active[i], cap, cancel, state, cond, use_cond);
}

// What ends an Arnoldi step (k_reduce_seg of the norms, k_givens,
// k_iter_advance) when the last CTA of k_update runs it.
struct StepEnd {
    int S, ks, G, M, cap, use_cond;
    const int32_t *g_ch_first, *g_ch_count;
    double *const *Hp;
    double *cs, *sn, *g, *nrm2, *hnorm, *rhnorm;
    const double *normb;
    double tol;
    const int *scap;
    int *active, *iters, *capped, *n_active_all, *iter, *state;
    const volatile int *cancel;
    cudaGraphConditionalHandle cond;
};

// one CTA: the norm of every active solve (summed over its geometry's
// chunks in the same order as k_reduce_seg), the Givens update, then the
// step index and the loop condition
__device__ void step_end(const StepEnd &e, int i, double *partial, int nch) {
    __shared__ int s_na;
    const int lane = threadIdx.x & 31;
    if (threadIdx.x == 0) s_na = 0;
    for (int sidx = threadIdx.x >> 5; sidx < e.S; sidx += blockDim.x >> 5) {
        if (!e.active[sidx]) continue;
        int r = sidx % e.ks, gg = sidx / e.ks;
        double sum = 0.0;
        int c0 = e.g_ch_first[gg], cn = e.g_ch_count[gg];
        const double *pp = partial + (int64_t)r * nch + c0;
        for (int c = lane; c < cn; c += 32) sum += __ldcg(&pp[c]);
        for (int o = 16; o > 0; o >>= 1) sum += __shfl_xor_sync(0xffffffffu, sum, o);
        if (lane == 0) e.nrm2[sidx] = sum;
    }
    __syncthreads();
    int na = 0;
    for (int sidx = threadIdx.x; sidx < e.S; sidx += blockDim.x)
        if (e.active[sidx] &&
            givens_one(sidx, i, e.M, e.Hp, e.cs, e.sn, e.g, e.normb, e.nrm2, e.hnorm, e.rhnorm, e.tol, e.scap, e.active, e.iters,
                       e.capped))
            na++;
    if (na) atomicAdd(&s_na, na);
    __syncthreads();
    if (threadIdx.x == 0) {
        e.n_active_all[i] = s_na;
        iter_advance_one(e.iter, i, s_na, e.cap, e.cancel, e.state, e.cond, e.use_cond);
    }
}

// v[r] = w[r] - sum_j h_j V_j[r] with the solve's own h; partial |v|^2 per
// chunk. With fuse_end set, the last CTA to finish (a ticket on *done) also
// ends the Arnoldi step (step_end: norms, Givens, step index) and resets *done.
// PB (the mixed path): basis vectors are FP32 pairs and each element's
// subtraction chain runs in pair arithmetic (w and every h_j split into
// pairs, f2_fma), rounded to FP64 once for v and its norm. QV basis vectors
// are loaded per pass: 8 for small models (few CTAs, so the passes' memory
// waits are the time), else 4; the subtractions are the same either way.
template <bool PB, int QV>
__global__ void __launch_bounds__(256, QV == 8 ? 2 : (PB ? 4 : 1)) k_update(int64_t Np, const int *__restrict__ iter, double *const *__restrict__ Vp, const double *__restrict__ w,
                         double *const *__restrict__ Hp, SegChunks ch, int ks, const int *__restrict__ active,
                         double *__restrict__ v, double *__restrict__ partial, int fuse_end, StepEnd fe, int *done) {
    using E = typename std::conditional<PB, float2, double>::type;
    __shared__ double sh[32];
    __shared__ int s_last;
    const int nvec = *iter + 1;
    int r = blockIdx.y, c = blockIdx.x;
    int sidx = ch.geom[c] * ks + r;
    if (active[sidx]) {
    const double *h = Hp[nvec - 1] + (int64_t)sidx * (nvec + 1);
    int64_t base = ch.start[c];
    int len = ch.len[c];
    // four elements per thread, each its own subtraction chain (in basis
    // order); the elements of four basis vectors are loaded before any of
    // them is used, so one pass waits for memory once per four vectors
    const int U = kDotChunk / 256;
    E x[U];
    int64_t t0 = (int64_t)r * Np + base + threadIdx.x;
#pragma unroll
    for (int u = 0; u < U; u++) {
        const double wd = (threadIdx.x + u * 256 < len) ? w[t0 + u * 256] : 0.0;
        if constexpr (PB) x[u] = d2pair_bits(wd);
        else x[u] = wd;
    }
    for (int j0 = 0; j0 < nvec; j0 += QV) {
        E hv[QV], vv[QV][U];
#pragma unroll
        for (int q = 0; q < QV; q++) {
            const bool okq = j0 + q < nvec;
            const double hq = okq ? h[j0 + q] : 0.0;
            if constexpr (PB) {
                const float2 hp = d2pair_bits(hq);
                hv[q] = make_float2(-hp.x, -hp.y);
            } else {
                hv[q] = hq;
            }
            const E *vj = okq ? reinterpret_cast<const E *>(Vp[j0 + q]) + t0 : NULL;
#pragma unroll
            for (int u = 0; u < U; u++) vv[q][u] = (okq && threadIdx.x + u * 256 < len) ? vj[u * 256] : kv_zero<E>();
        }
#pragma unroll
        for (int q = 0; q < QV; q++)
            if (j0 + q < nvec)
#pragma unroll
                for (int u = 0; u < U; u++)
                    if (threadIdx.x + u * 256 < len) {
                        if constexpr (PB) x[u] = f2_fma(x[u], hv[q], vv[q][u]);
                        else x[u] = x[u] - hv[q] * vv[q][u];
                    }
    }
    double s2 = 0.0;
#pragma unroll
    for (int u = 0; u < U; u++) {
        if (threadIdx.x + u * 256 < len) {
            const double xd = kv_double(x[u]);
            v[t0 + u * 256] = xd;
            s2 += xd * xd;
        }
    }
    s2 = block_sum(s2, sh);
    if (threadIdx.x == 0) partial[(int64_t)r * ch.n + c] = s2;
    }
    if (!fuse_end) return;
    if (threadIdx.x == 0) {
        __threadfence();  // this CTA's partial norm is visible before its ticket
        s_last = atomicAdd(done, 1) == (int)(gridDim.x * gridDim.y) - 1;
    }
    __syncthreads();
    if (!s_last) return;
    __threadfence();
    step_end(fe, nvec - 1, partial, ch.n);
    if (threadIdx.x == 0) *done = 0;
}


// solves whose true residual |b - A x| / |b| is at or above tol
__global__ void k_refine_count(int S, const double *__restrict__ nr2, const double *__restrict__ nb2, double tol, int *count) {
    int sidx = blockIdx.x * blockDim.x + threadIdx.x;
    if (sidx >= S) return;
    double nb = sqrt(nb2[sidx]);
    if (nb > 0.0 && sqrt(nr2[sidx]) / nb >= tol) atomicAdd(count, 1);
}

// back substitution R z = g for every solve, one warp each: column by
// column from the last, the lane that owns z_i divides it by R_ii, then the
// lanes update z_j -= R_ji z_i for all j < i at once (every z_j sees the
// same sequence of updates as in a serial column-oriented sweep)
__global__ void k_backsub(int S, int M, double *const *__restrict__ Hc, const double *g, const int *iters, double *z) {
    const int sidx = (int)((blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5), lane = threadIdx.x & 31;
    if (sidx >= S) return;
    const int it = iters[sidx];
    double *zz = z + (int64_t)sidx * (M + 2);
    const double *gg = g + (int64_t)sidx * (M + 2);
    for (int i = lane; i <= it; i += 32) zz[i] = gg[i];
    __syncwarp();
    for (int i = it; i >= 0; i--) {
        const double *hc = Hc[i] + (int64_t)sidx * (i + 2);
        const double zi = zz[i] / hc[i];
        for (int j = lane; j < i; j += 32) zz[j] = zz[j] - hc[j] * zi;
        if (lane == 0) zz[i] = zi;
        __syncwarp();
    }
}

// y[r][j] = sum_{jv <= iters(s)} z_s[jv] V_jv[r][j] (in pair arithmetic on
// the FP32 pairs of the mixed path's basis when PB)
template <bool PB>
__global__ void k_combine(int64_t Np, int ks, int M, double *const *__restrict__ Vp, const double *__restrict__ z,
                          const int *__restrict__ iters, const int32_t *__restrict__ leaf_geom, double *__restrict__ y) {
    int64_t n = (int64_t)ks * Np;
    for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < n; t += (int64_t)gridDim.x * blockDim.x) {
        int r = (int)(t / Np);
        int64_t j = t - (int64_t)r * Np;
        int sidx = leaf_geom[j] * ks + r;
        int it = iters[sidx];
        if constexpr (PB) {
            // four basis elements loaded before any is used (one wait for
            // memory per four vectors), summed in basis order
            const double *zs = z + (int64_t)sidx * (M + 2);
            float2 sum = make_float2(0.0f, 0.0f);
            int jv = 0;
            for (; jv + 3 <= it; jv += 4) {
                float2 v4[4];
#pragma unroll
                for (int q = 0; q < 4; q++) v4[q] = reinterpret_cast<const float2 *>(Vp[jv + q])[t];
#pragma unroll
                for (int q = 0; q < 4; q++) sum = f2_fma(sum, v4[q], d2pair_bits(zs[jv + q]));
            }
            for (; jv <= it; jv++) sum = f2_fma(sum, reinterpret_cast<const float2 *>(Vp[jv])[t], d2pair_bits(zs[jv]));
            y[t] = pair2d(sum);
        } else {
            double sum = 0.0;
            for (int jv = 0; jv <= it; jv++) sum += Vp[jv][t] * z[(int64_t)sidx * (M + 2) + jv];
            y[t] = sum;
        }
    }
}

// x = x0 + P y (or x0 alone when the initial guess already met the tolerance)
__global__ void k_finish(int64_t Np, int ks, const double *__restrict__ x0, const double *__restrict__ y,
                         const double *__restrict__ diag, const int *__restrict__ iters, const int32_t *__restrict__ leaf_geom,
                         double *__restrict__ x) {
    int64_t n = (int64_t)ks * Np;
    for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < n; t += (int64_t)gridDim.x * blockDim.x) {
        int r = (int)(t / Np);
        int64_t j = t - (int64_t)r * Np;
        if (iters[leaf_geom[j] * ks + r] < 0) { x[t] = x0[t]; continue; }
        double py = diag ? y[t] / diag[j] : y[t];
        x[t] = x0[t] + py;
    }
}

// r = b - w over one chunk, with partial norms of r and b
__global__ void k_residual(int64_t Np, const double *__restrict__ b, const double *__restrict__ wv, SegChunks ch,
                           double *__restrict__ rv, double *__restrict__ pr, double *__restrict__ pb) {
    __shared__ double sh[32];
    int r = blockIdx.y, c = blockIdx.x;
    int64_t base = ch.start[c];
    int len = ch.len[c];
    double s1 = 0.0, s2 = 0.0;
    for (int u = 0; u < kDotChunk / 256; u++) {
        int o = threadIdx.x + u * 256;
        if (o >= len) break;
        int64_t t = (int64_t)r * Np + base + o;
        double bb = b[t];
        double x = wv ? bb - wv[t] : bb;
        rv[t] = x;
        s1 += x * x;
        s2 += bb * bb;
    }
    s1 = block_sum(s1, sh);
    if (threadIdx.x == 0) pr[(int64_t)r * ch.n + c] = s1;
    s2 = block_sum(s2, sh);
    if (threadIdx.x == 0) pb[(int64_t)r * ch.n + c] = s2;
}

__global__ void k_init_state(int S, int M, const double *nr2, const double *nb2, double *normb, double *g, double *hn, double tol,
                             int *active, int *iters, int *capped, int *n_start) {
    int sidx = blockIdx.x * blockDim.x + threadIdx.x;
    if (sidx >= S) return;
    capped[sidx] = 0;
    double nr = sqrt(nr2[sidx]), nb = sqrt(nb2[sidx]);
    normb[sidx] = nb;
    g[(int64_t)sidx * (M + 2)] = nr;
    if (nb == 0.0 || nr / nb < tol) {
        // unused slot, or the initial guess already meets the tolerance
        active[sidx] = 0;
        iters[sidx] = -1;
        hn[sidx] = 1.0;
    } else {
        active[sidx] = 1;
        iters[sidx] = 0;
        hn[sidx] = nr;
        atomicAdd(n_start, 1);
    }
}

// C assembly (CSolveCap::Solve, Solver/SolveCapacitance.cpp:1305-1366):
// entry e = (solve column slot, conductor column) of some geometry,
// C_e = sum over the conductor's leaves of outer permittivity * charge.
// Stage 1: every CTA sums one slice of kAsmChunk leaves of one entry; stage 2
// adds the slices in order (deterministic).
static const int kAsmChunk = 4096;
__global__ void k_assemble_part(int64_t Np, const int32_t *__restrict__ e_slot, const int64_t *__restrict__ e_first,
                                const int64_t *__restrict__ e_count, const double *__restrict__ weight, const double *__restrict__ x,
                                double *__restrict__ part) {
    __shared__ double sh[32];
    int e = blockIdx.x, sl = blockIdx.y;
    int64_t lo = e_first[e] + (int64_t)sl * kAsmChunk, hi = min(e_first[e] + e_count[e], lo + kAsmChunk);
    const double *xr = x + (int64_t)e_slot[e] * Np;
    double s = 0.0;
    for (int64_t j = lo + threadIdx.x; j < hi; j += blockDim.x) s += weight[j] * xr[j];
    s = block_sum(s, sh);
    if (threadIdx.x == 0) part[(int64_t)e * gridDim.y + sl] = s;
}

__global__ void k_assemble_sum(int nentry, int nslice, const double *__restrict__ part, const int64_t *__restrict__ e_out,
                               double *__restrict__ cap) {
    int e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= nentry) return;
    double s = 0.0;
    for (int i = 0; i < nslice; i++) s += part[(int64_t)e * nslice + i];
    cap[e_out[e]] = s;
}

// -------------------------------------------------------------- host side

static int grid_for(int64_t n, int threads, int sms) {
    int64_t g = (n + threads - 1) / threads;
    int64_t cap = (int64_t)sms * 16;
    if (g > cap) g = cap;
    if (g < 1) g = 1;
    return (int)g;
}

int context_init(DeviceContext &ctx, int device) {
    int n = 0;
    cudaError_t e = cudaGetDeviceCount(&n);
    if (e != cudaSuccess || n == 0) {
        set_error(std::string("no CUDA device available: ") + (e == cudaSuccess ? "zero devices" : cudaGetErrorString(e)));
        return FCG_DEVICE_ERROR;
    }
    if (device < 0 || device >= n) { set_error("device index out of range"); return FCG_DEVICE_ERROR; }
    FCG_CK(cudaSetDevice(device));
    cudaDeviceProp prop;
    FCG_CK(cudaGetDeviceProperties(&prop, device));
    ctx.device = device;
    ctx.sm_count = prop.multiProcessorCount;
    ctx.smem_optin = prop.sharedMemPerBlockOptin;
    // the up-sweep's top pass holds the whole top forest in shared memory
    FCG_CK(cudaFuncSetAttribute(k_up_top<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)ctx.smem_optin));
    FCG_CK(cudaFuncSetAttribute(k_up_top<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)ctx.smem_optin));
    FCG_CK(cudaFuncSetAttribute(k_up_top32<1>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)ctx.smem_optin));
    FCG_CK(cudaFuncSetAttribute(k_up_top32<2>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)ctx.smem_optin));
    FCG_CK(cudaFuncSetAttribute(k_up_top32<4>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)ctx.smem_optin));
    FCG_CK(cudaMemGetInfo(&ctx.free_bytes, &ctx.total_bytes));
    cudaStream_t st;
    FCG_CK(cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking));
    ctx.stream = (void *)st;
    // the device's memory pool keeps freed blocks for reuse by later problems
    cudaMemPool_t pool;
    if (cudaDeviceGetDefaultMemPool(&pool, device) == cudaSuccess) {
        uint64_t keep = UINT64_MAX;
        cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &keep);
    }
    if (cudaHostAlloc((void **)&ctx.pin, (size_t)kPinSlots * kPinSlotInts * sizeof(int), cudaHostAllocDefault) != cudaSuccess) {
        ctx.pin = nullptr;
        set_error("cannot allocate pinned host memory");
        return FCG_OUT_OF_MEMORY;
    }
    ctx.pin_free.clear();
    for (int i = kPinSlots - 1; i >= 0; i--) ctx.pin_free.push_back(i);
    return FCG_NORMAL_END;
}

// a pinned slot of kPinSlotInts ints for one problem (NULL when all are taken)
static int *pin_acquire(DeviceContext &ctx) {
    std::lock_guard<std::mutex> lk(ctx.pin_mu);
    if (!ctx.pin || ctx.pin_free.empty()) return NULL;
    int i = ctx.pin_free.back();
    ctx.pin_free.pop_back();
    return ctx.pin + (size_t)i * kPinSlotInts;
}
static void pin_release(DeviceContext &ctx, int *slot) {
    if (!slot || !ctx.pin) return;
    std::lock_guard<std::mutex> lk(ctx.pin_mu);
    ctx.pin_free.push_back((int)((slot - ctx.pin) / kPinSlotInts));
}

void context_unref(DeviceContext *ctx) {
    if (ctx && ctx->refs.fetch_sub(1) == 1) {
        context_release(*ctx);
        delete ctx;
    }
}

void context_release(DeviceContext &ctx) {
    cudaSetDevice(ctx.device);
    if (ctx.stream) {
        cudaStreamSynchronize((cudaStream_t)ctx.stream);
        cudaStreamDestroy((cudaStream_t)ctx.stream);
        ctx.stream = nullptr;
    }
    if (ctx.pin) {
        cudaFreeHost(ctx.pin);
        ctx.pin = nullptr;
    }
    {
        std::lock_guard<std::mutex> lk(ctx.stage_mu);
        for (void *b : ctx.stage_free) cudaFreeHost(b);
        ctx.stage_free.clear();
        ctx.stage_count = 0;
    }
    // hand the pool's unused blocks back
    cudaMemPool_t pool;
    if (cudaDeviceGetDefaultMemPool(&pool, ctx.device) == cudaSuccess) {
        cudaDeviceSynchronize();
        cudaMemPoolTrimTo(pool, 0);
    }
}

// Run fn(begin, end) over [0, n) on up to 16 host threads (chunks of at
// least 32k items; small ranges stay on the calling thread).
template <class F> static void parallel_for(int64_t n, F fn) {
    int nt = (int)std::min<int64_t>(std::max(1u, std::thread::hardware_concurrency()), 16);
    nt = (int)std::min<int64_t>(nt, (n + 32767) / 32768);
    if (nt <= 1) { fn((int64_t)0, n); return; }
    std::vector<std::thread> th;
    int64_t step = (n + nt - 1) / nt;
    for (int t = 1; t < nt; t++) {
        int64_t b = t * step, e = std::min(n, b + step);
        if (b < e) th.emplace_back(fn, b, e);
    }
    fn((int64_t)0, std::min(n, step));
    for (auto &x : th) x.join();
}

// The model checks without a pass over the nodes or leaves: sizes,
// pointers, the ends of link_ptr, the conductors tiling the leaves and their
// permittivities. problem_create runs the per-node and per-leaf checks on
// the device (k_check_model, k_check_leaves) before any kernel indexes with
// the caller's arrays.
static std::string validate_host(const fcg_model_arrays &a) {
    if (a.n_nodes <= 0 || a.n_panels <= 0 || a.n_links < 0 || a.n_conductors <= 0) return "empty model";
    if (a.n_nodes > (int64_t)kSrcMask || a.n_links > 0x7fffffffLL) return "model too large (nodes must fit 29 bits, links 31 bits)";
    if (!a.node_type || !a.node_left || !a.node_right || !a.node_leaf_first || !a.node_leaf_count || !a.node_vertices ||
        !a.node_centroid || !a.node_normal || !a.node_area || !a.node_maxside || !a.link_ptr || (a.n_links && !a.link_src) ||
        !a.leaf_diel || !a.cond_is_diel || !a.cond_leaf_first || !a.cond_leaf_count || !a.cond_outperm || !a.cond_inperm ||
        !a.cond_surf_ptr || !a.cond_surf_outperm)
        return "null model array";
    if (a.link_ptr[0] != 0 || a.link_ptr[a.n_nodes] != a.n_links) return "link_ptr does not span the links";
    int64_t next = 0;
    for (int32_t c = 0; c < a.n_conductors; c++) {
        if (a.cond_leaf_first[c] != next || a.cond_leaf_count[c] <= 0) return "conductor leaf ranges must tile the leaves";
        next += a.cond_leaf_count[c];
        if (a.cond_surf_ptr[c + 1] < a.cond_surf_ptr[c]) return "cond_surf_ptr not monotone";
        if (a.cond_is_diel[c] && a.cond_outperm[c] == a.cond_inperm[c]) return "dielectric interface with equal permittivities";
    }
    if (next != a.n_panels) return "conductor leaf ranges must tile the leaves";
    return "";
}

static const char *node_check_message(int code) {
    switch (code) {
    case 1: return "link_ptr not monotone";
    case 2: return "bad leaf node";
    case 3: return "children must precede their parent (post-order)";
    case 4: return "inconsistent leaf counts";
    case 5: return "leaf ranges are not contiguous";
    default: return "leaf range out of bounds";
    }
}

// the full check on the host (no device work): validate_host, then every
// node (on all host threads; the lowest failing node decides the message)
// and every conductor leaf's permittivity index
static std::string validate(const fcg_model_arrays &a) {
    std::string hs = validate_host(a);
    if (!hs.empty()) return hs;
    std::atomic<int64_t> bad_at{INT64_MAX};
    std::atomic<int64_t> leaves_all{0};
    std::mutex mu;
    int why = 0;
    parallel_for(a.n_nodes, [&](int64_t b, int64_t e) {
        int64_t leaves = 0;
        for (int64_t i = b; i < e; i++) {
            int code = 0;
            if (a.link_ptr[i + 1] < a.link_ptr[i]) {
                code = 1;
            } else if (a.node_type[i] & FCG_IS_LEAF) {
                if (a.node_left[i] != -1 || a.node_right[i] != -1 || a.node_leaf_count[i] != 1) code = 2;
                leaves++;
            } else {
                int32_t l = a.node_left[i], r = a.node_right[i];
                if (l < 0 || r < 0 || l >= i || r >= i) code = 3;
                else if (a.node_leaf_count[i] != a.node_leaf_count[l] + a.node_leaf_count[r]) code = 4;
                else if (a.node_leaf_first[i] != a.node_leaf_first[l] ||
                         a.node_leaf_first[r] != a.node_leaf_first[l] + a.node_leaf_count[l])
                    code = 5;
            }
            if (!code && (a.node_leaf_first[i] < 0 || a.node_leaf_first[i] + a.node_leaf_count[i] > a.n_panels)) code = 6;
            if (code) {
                std::lock_guard<std::mutex> lk(mu);
                if (i < bad_at.load()) { bad_at.store(i); why = code; }
                return;
            }
        }
        leaves_all += leaves;
    });
    if (bad_at.load() != INT64_MAX) return node_check_message(why);
    if (leaves_all.load() != a.n_panels) return "leaf count does not match n_panels";
    for (int32_t c = 0; c < a.n_conductors; c++) {
        if (a.cond_is_diel[c]) continue;
        int32_t ns = a.cond_surf_ptr[c + 1] - a.cond_surf_ptr[c];
        for (int64_t j = a.cond_leaf_first[c]; j < a.cond_leaf_first[c] + a.cond_leaf_count[c]; j++)
            if (a.leaf_diel[j] >= ns) return "leaf permittivity index out of range";
    }
    return "";
}


// FCG_TRACE=1 prints the host phases of problem creation to stderr
struct HostTrace {
    bool on;
    std::chrono::steady_clock::time_point t0, t;
    HostTrace() : on(getenv("FCG_TRACE") != NULL), t0(std::chrono::steady_clock::now()), t(t0) {}
    void mark(const char *what) {
        if (!on) return;
        auto n = std::chrono::steady_clock::now();
        fprintf(stderr, "[fcg] %-24s %8.3f ms (total %8.3f)\n", what, std::chrono::duration<double, std::milli>(n - t).count(),
                std::chrono::duration<double, std::milli>(n - t0).count());
        t = n;
    }
    // device-side marks: an event recorded on a stream, reported (relative
    // to the first mark) once the work has finished
    std::vector<std::pair<const char *, cudaEvent_t>> ev;
    void dmark(const char *what, cudaStream_t st) {
        if (!on) return;
        cudaEvent_t e = NULL;
        if (cudaEventCreate(&e) != cudaSuccess) return;
        cudaEventRecord(e, st);
        ev.push_back({what, e});
    }
    void dreport() {
        if (!on || ev.empty()) return;
        cudaEventSynchronize(ev.back().second);
        for (auto &m : ev) {
            float ms = 0.f;
            cudaEventSynchronize(m.second);
            cudaEventElapsedTime(&ms, ev[0].second, m.second);
            fprintf(stderr, "[fcg]   device %-24s at %8.3f ms\n", m.first, ms);
        }
        for (auto &m : ev) cudaEventDestroy(m.second);
        ev.clear();
    }
    ~HostTrace() {
        for (auto &m : ev) cudaEventDestroy(m.second);
    }
};

// ---- device layout of a problem, from the caller's post-order arrays
// Device node labels are height-major (leaves in leaf order, then every
// height in post-order), rows are offset in that order, and the sweep plan
// cuts the forest into subtrees of at most kBlockLeaves leaves (one CTA
// each in the sweep kernels) whose internal nodes are listed by height. All
// of it is computed here on the device; the host reads back three numbers.

__global__ void k_model_parents(int64_t Nn, const uint8_t *__restrict__ type, const int32_t *__restrict__ left,
                                const int32_t *__restrict__ right, int32_t *__restrict__ par) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < Nn; i += (int64_t)gridDim.x * blockDim.x)
        if (!(type[i] & FCG_IS_LEAF)) {
            par[left[i]] = (int32_t)i;
            par[right[i]] = (int32_t)i;
        }
}

// Heights and leaf counts bottom-up: every leaf climbs while it is the
// second of its parent's two children to arrive (the first one stops), so
// each node is computed once, after both children. Nothing waits.
__global__ void k_heights(int64_t Nn, const uint8_t *__restrict__ type, const int32_t *__restrict__ left,
                          const int32_t *__restrict__ right, const int32_t *__restrict__ par, int32_t *height, int32_t *cnt,
                          int *arrive, int *hmax) {
    int hm = 0;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < Nn; i += (int64_t)gridDim.x * blockDim.x) {
        if (!(type[i] & FCG_IS_LEAF)) continue;
        int32_t n = (int32_t)i;
        int h = 0;
        height[n] = 0;
        cnt[n] = 1;
        for (;;) {
            int32_t q = par[n];
            if (q < 0) break;
            __threadfence();  // this node's values are visible before the arrival is counted
            if (atomicAdd(&arrive[q], 1) == 0) break;
            __threadfence();
            int32_t l = left[q], r = right[q];
            h = 1 + max(__ldcg(&height[l]), __ldcg(&height[r]));
            height[q] = h;
            cnt[q] = __ldcg(&cnt[l]) + __ldcg(&cnt[r]);
            n = q;
        }
        hm = max(hm, h);
    }
    for (int o = 16; o > 0; o >>= 1) hm = max(hm, __shfl_xor_sync(0xffffffffu, hm, o));
    if ((threadIdx.x & 31) == 0) atomicMax(hmax, hm);
}

// entries (height << 32 | node) for the stable sort by height
__global__ void k_height_entries(int64_t Nn, const int32_t *__restrict__ height, unsigned long long *e) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < Nn; i += (int64_t)gridDim.x * blockDim.x)
        e[i] = ((unsigned long long)(uint32_t)height[i] << 32) | (unsigned long long)i;
}

__global__ void k_labels(int64_t Nn, const int32_t *__restrict__ inv, int32_t *__restrict__ lab) {
    for (int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; q < Nn; q += (int64_t)gridDim.x * blockDim.x)
        lab[inv[q]] = (int32_t)q;
}

// the label range [seg_lo[h], seg_hi[h]) of every height h < nseg
__global__ void k_seg_bounds(int64_t Nn, const int32_t *__restrict__ inv, const int32_t *__restrict__ height, int nseg,
                             int32_t *seg_lo, int32_t *seg_hi) {
    for (int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; q < Nn; q += (int64_t)gridDim.x * blockDim.x) {
        int h = height[inv[q]];
        if (h >= nseg) continue;
        if (q == 0 || height[inv[q - 1]] != h) seg_lo[h] = (int32_t)q;
        if (q == Nn - 1 || height[inv[q + 1]] != h) seg_hi[h] = (int32_t)(q + 1);
    }
}

// link count of every row, in label order
__global__ void k_row_lengths(int64_t Nn, const int32_t *__restrict__ inv, const int64_t *__restrict__ ptr_model,
                              int64_t *__restrict__ len) {
    for (int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; q < Nn; q += (int64_t)gridDim.x * blockDim.x) {
        int32_t i = inv[q];
        len[q] = ptr_model[i + 1] - ptr_model[i];
    }
}

// subtree roots: at most kBlockLeaves leaves, the parent above that; marked
// at their first leaf (block ranges tile the leaves, so a scan numbers the
// blocks in leaf order)
__global__ void k_block_flags(int64_t Nn, const int32_t *__restrict__ cnt, const int32_t *__restrict__ par,
                              const int64_t *__restrict__ lf, int32_t *__restrict__ bflag) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < Nn; i += (int64_t)gridDim.x * blockDim.x) {
        int32_t q = par[i];
        if (cnt[i] <= kBlockLeaves && (q < 0 || cnt[q] > kBlockLeaves)) bflag[lf[i]] = 1;
    }
}

__global__ void k_blocks(int64_t Nn, const int32_t *__restrict__ cnt, const int32_t *__restrict__ par,
                         const int32_t *__restrict__ height, const int64_t *__restrict__ lf, const int32_t *__restrict__ lab,
                         const int32_t *__restrict__ bid, SweepPlan pl, int32_t *broot, int32_t *lvl_cnt, int32_t *node_cnt,
                         int32_t *bdepth, int *max_depth) {
    int md = 0;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < Nn; i += (int64_t)gridDim.x * blockDim.x) {
        int32_t q = par[i];
        if (!(cnt[i] <= kBlockLeaves && (q < 0 || cnt[q] > kBlockLeaves))) continue;
        int32_t b = bid[lf[i]];
        pl.blk_leaf_first[b] = (int32_t)lf[i];
        pl.blk_nleaves[b] = cnt[i];
        pl.blk_nlvls[b] = height[i];
        pl.blk_root[b] = lab[i];
        broot[b] = (int32_t)i;
        lvl_cnt[b] = height[i] + 1;
        node_cnt[b] = cnt[i] - 1;
        int depth = 0;  // ancestors above the subtree (the down-sweep's chain)
        for (int32_t a = q; a >= 0 && depth <= kMaxChain; a = par[a]) depth++;
        bdepth[b] = min(depth, kMaxChain + 1);
        md = max(md, depth);
    }
    for (int o = 16; o > 0; o >>= 1) md = max(md, __shfl_xor_sync(0xffffffffu, md, o));
    if ((threadIdx.x & 31) == 0) atomicMax(max_depth, md);
}

// the internal nodes of every block by height: in height-major labels the
// block's nodes of one height are one run of the height's label range (both
// are in post-order), found by binary search for the block's post-order range
__global__ void k_block_levels(int nb, const int32_t *__restrict__ broot, const int32_t *__restrict__ cnt,
                               const int32_t *__restrict__ height, const int32_t *__restrict__ inv, const int32_t *__restrict__ seg_lo,
                               const int32_t *__restrict__ seg_hi, const int32_t *__restrict__ node_off, SweepPlan pl,
                               int32_t *__restrict__ ent_blk, int32_t *__restrict__ pos_of) {
    for (int b = blockIdx.x * blockDim.x + threadIdx.x; b < nb; b += gridDim.x * blockDim.x) {
        int32_t i = broot[b];
        int32_t first = i - (2 * cnt[i] - 1) + 1;
        int H = height[i];
        int32_t off = node_off[b];
        pl.blk_node_first[b] = off;
        int32_t *lp = pl.lvl_ptr + pl.blk_lvl_first[b];
        for (int h = 1; h <= H; h++) {
            int32_t lo = seg_lo[h], hi = seg_hi[h];
            while (lo < hi) {  // first label of height h with post-order index >= first
                int32_t m = lo + ((hi - lo) >> 1);
                if (inv[m] < first) lo = m + 1;
                else hi = m;
            }
            int32_t a0 = lo;
            hi = seg_hi[h];
            while (lo < hi) {  // first label of height h with post-order index > i
                int32_t m = lo + ((hi - lo) >> 1);
                if (inv[m] <= i) lo = m + 1;
                else hi = m;
            }
            lp[h - 1] = off;
            for (int32_t q = a0; q < lo; q++) {
                pl.lvl_nodes[off] = q;
                ent_blk[off] = b;
                pos_of[q] = off;
                off++;
            }
        }
        lp[H] = off;
    }
}

// children of every internal block node as local indices (leaves by leaf
// offset, internal nodes by list position), packed left | right << 16
__global__ void k_block_kids(const long long *__restrict__ n_ent, SweepPlan pl, const int32_t *__restrict__ ent_blk,
                             const int32_t *__restrict__ pos_of, const int32_t *__restrict__ inv, const int32_t *__restrict__ lab,
                             const uint8_t *__restrict__ type, const int32_t *__restrict__ left, const int32_t *__restrict__ right,
                             const int64_t *__restrict__ lf) {
    const int64_t ne = *n_ent;
    for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < ne; e += (int64_t)gridDim.x * blockDim.x) {
        int b = ent_blk[e];
        int32_t i = inv[pl.lvl_nodes[e]];
        int lfb = pl.blk_leaf_first[b], nlb = pl.blk_nleaves[b], base = pl.lvl_ptr[pl.blk_lvl_first[b]];
        int32_t c[2] = {left[i], right[i]};
        uint32_t loc[2];
        for (int u = 0; u < 2; u++)
            loc[u] = (type[c[u]] & FCG_IS_LEAF) ? (uint32_t)(lf[c[u]] - lfb) : (uint32_t)(nlb + pos_of[lab[c[u]]] - base);
        pl.lvl_kids[e] = loc[0] | (loc[1] << 16);
    }
}

// top nodes (more than kBlockLeaves leaves) in label order, which is by
// height; every leaf must carry its own leaf index as label
__global__ void k_top_flags(int64_t Nn, int64_t Np, const int32_t *__restrict__ inv, const int32_t *__restrict__ cnt,
                            const int32_t *__restrict__ leaf_node, int32_t *__restrict__ flag, unsigned *bad) {
    for (int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; q < Nn; q += (int64_t)gridDim.x * blockDim.x) {
        flag[q] = cnt[inv[q]] > kBlockLeaves ? 1 : 0;
        if (q < Np && leaf_node[q] != (int32_t)q) atomicAdd(bad, 1u);
    }
}

__global__ void k_top_list(int64_t Nn, const int32_t *__restrict__ inv, const int32_t *__restrict__ lab, const int32_t *__restrict__ cnt,
                           const int32_t *__restrict__ left, const int32_t *__restrict__ right, const int64_t *__restrict__ lf,
                           const int32_t *__restrict__ bid, const int32_t *__restrict__ tpos, const long long *__restrict__ n_blocks,
                           SweepPlan pl) {
    const int nb = (int)*n_blocks;
    for (int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; q < Nn; q += (int64_t)gridDim.x * blockDim.x) {
        int32_t i = inv[q];
        if (cnt[i] <= kBlockLeaves) continue;
        int t = tpos[q];
        pl.top_nodes[t] = (int32_t)q;
        int32_t c[2] = {left[i], right[i]};
        int loc[2];
        for (int u = 0; u < 2; u++) loc[u] = cnt[c[u]] > kBlockLeaves ? nb + tpos[lab[c[u]]] : bid[lf[c[u]]];
        pl.top_kids[t] = make_int2(loc[0], loc[1]);
    }
}

// offsets of every height in the top list: the top nodes before the
// height's first label
__global__ void k_top_hptr(const int *__restrict__ hmax, int hcap, const int32_t *__restrict__ seg_lo, const int32_t *__restrict__ tpos,
                           const long long *__restrict__ n_top, int32_t *hptr) {
    const int H = *hmax;
    if (H > hcap) return;  // too high: the model is rejected
    for (int h = blockIdx.x * blockDim.x + threadIdx.x; h <= H + 1; h += gridDim.x * blockDim.x)
        hptr[h] = h <= H ? tpos[seg_lo[h]] : (int32_t)*n_top;
}

// the ancestors of every block root, parent first
__global__ void k_chains(int nb, const int32_t *__restrict__ broot, const int32_t *__restrict__ par, const int32_t *__restrict__ lab,
                         SweepPlan pl) {
    for (int b = blockIdx.x * blockDim.x + threadIdx.x; b < nb; b += gridDim.x * blockDim.x) {
        int32_t c = pl.blk_chain[b];
        for (int32_t a = par[broot[b]]; a >= 0; a = par[a]) pl.chain[c++] = lab[a];
        if (b == nb - 1) pl.blk_chain[nb] = c;
    }
}

// Contiguous row ranges of about equal work (links + 8 per row): the first
// row whose work offset reaches b/nb of the total (a binary search per range)
__global__ void k_row_split(int64_t Nn, const int64_t *__restrict__ ptr, int64_t nb, double total, int32_t *split) {
    for (int64_t b = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; b <= nb; b += (int64_t)gridDim.x * blockDim.x) {
        if (b == 0 || b == nb) {
            split[b] = b == 0 ? 0 : (int32_t)Nn;
            continue;
        }
        double target = total * (double)b / (double)nb;
        int64_t lo = 0, hi = Nn;
        while (lo < hi) {
            int64_t m = lo + ((hi - lo) >> 1);
            if ((double)ptr[m] + 8.0 * (double)m < target) lo = m + 1;
            else hi = m;
        }
        split[b] = (int32_t)lo;
    }
}

// Contiguous row ranges of about equal work (links + 8 per row) for the
// multi-right-hand-side link product: ctas ranges (capped so that each has at
// least 64 rows).
static int set_row_split(DeviceProblem *p, int64_t ctas) {
    int64_t Nn = p->Nn, L = p->L;
    int64_t nb = std::max<int64_t>(1, std::min<int64_t>(ctas, (Nn + 63) / 64));
    if (p->row_split && nb == p->n_row_split) return FCG_NORMAL_END;
    dfree(p->row_split);
    p->n_row_split = 0;
    int r = dalloc(&p->row_split, nb + 1, p->bytes);
    if (r != FCG_NORMAL_END) return r;
    k_row_split<<<grid_for(nb + 1, 128, p->ctx->sm_count), 128, 0, p->stream>>>(Nn, p->link_ptr, nb, (double)L + 8.0 * (double)Nn,
                                                                               p->row_split);
    FCG_CK(cudaGetLastError());
    p->timings.launches++;
    p->n_row_split = (int)nb;
    return FCG_NORMAL_END;
}

std::string model_check(const fcg_model_arrays &a) { return validate(a); }

int problem_create(DeviceContext &ctx, const fcg_model_arrays &a, int precision, void *stream, DeviceProblem **out) {
    *out = NULL;
    HostTrace tr;
    std::string bad = validate_host(a);
    tr.mark("validate");
    if (!bad.empty()) { set_error("invalid model: " + bad); return FCG_GENERIC_ERROR; }
    if (precision != FCG_PREC_FP64 && precision != FCG_PREC_MIXED) { set_error("unknown precision"); return FCG_GENERIC_ERROR; }
    FCG_CK(cudaSetDevice(ctx.device));
    DeviceProblem *p = new DeviceProblem();
    p->ctx = &ctx;
    ctx.refs.fetch_add(1);
    p->precision = precision;
    p->pin = pin_acquire(ctx);
    if (p->pin && cudaHostGetDevicePointer((void **)&p->pin_dev, p->pin, 0) != cudaSuccess) {
        cudaGetLastError();
        p->pin_dev = NULL;
    }
    p->Nn = a.n_nodes;
    p->Np = a.n_panels;
    p->L = a.n_links;
    p->n_cond_all = a.n_conductors;
    for (int32_t c = 0; c < a.n_conductors; c++) {
        if (!a.cond_is_diel[c]) p->cond_cols.push_back(c);
        p->cond_first.push_back(a.cond_leaf_first[c]);
        p->cond_count.push_back(a.cond_leaf_count[c]);
    }
    int r = FCG_NORMAL_END;
#define FCG_TRY(x) do { if ((r = (x)) != FCG_NORMAL_END) { problem_destroy(p); return r; } } while (0)
    if (stream) {
        p->stream = (cudaStream_t)stream;
    } else {
        p->owns_stream = true;
        if (cudaStreamCreateWithFlags(&p->stream, cudaStreamNonBlocking) != cudaSuccess) p->stream = NULL;
    }
    if (!p->stream || cudaEventCreate(&p->ev0) != cudaSuccess || cudaEventCreate(&p->ev1) != cudaSuccess) {
        set_error("cannot create stream/events");
        problem_destroy(p);
        return FCG_DEVICE_ERROR;
    }
    cudaStream_t s = p->stream;
    int64_t Nn = a.n_nodes, Np = a.n_panels, L = a.n_links;
    AllocScope alloc_scope(s);
    // Device node labels are height-major (all leaves in leaf order, then
    // every height in post-order): interaction partners have similar heights
    // and are spatially close, so the link product's charge gathers cluster
    // (2.3x fewer distinct sectors than the post-order numbering on a
    // 327k-panel sphere). Rows move as whole units: each row keeps its links
    // in order. Labels, row offsets and the sweep plan are computed on the
    // device from the uploaded arrays (one synchronisation at the end).
    FCG_TRY(dalloc(&p->geo, Nn, p->bytes));
    FCG_TRY(dalloc(&p->parent, Nn, p->bytes));
    FCG_TRY(dalloc(&p->left, Nn, p->bytes));
    FCG_TRY(dalloc(&p->right, Nn, p->bytes));
    FCG_TRY(dalloc(&p->leaf_node, Np, p->bytes));
    FCG_TRY(dalloc(&p->node_lfirst, Nn, p->bytes));
    FCG_TRY(dalloc(&p->leaf_eb, Np, p->bytes));
    FCG_TRY(dalloc(&p->leaf_ea, Np, p->bytes));
    FCG_TRY(dalloc(&p->leaf_weight, Np, p->bytes));
    FCG_TRY(dalloc(&p->link_ptr, Nn + 1, p->bytes));
    FCG_TRY(dalloc(&p->inv, Nn, p->bytes));
    {
        // sweep plan arrays at their bounds (blocks <= leaves; a block's
        // heights <= its leaves - 1, its internal nodes = its leaves - 1)
        SweepPlan &pl = p->plan;
        FCG_TRY(dalloc(&pl.blk_leaf_first, Np, p->bytes));
        FCG_TRY(dalloc(&pl.blk_nleaves, Np, p->bytes));
        FCG_TRY(dalloc(&pl.blk_lvl_first, Np + 1, p->bytes));
        FCG_TRY(dalloc(&pl.blk_nlvls, Np, p->bytes));
        FCG_TRY(dalloc(&pl.blk_root, Np, p->bytes));
        FCG_TRY(dalloc(&pl.lvl_ptr, Np + 1, p->bytes));
        FCG_TRY(dalloc(&pl.lvl_nodes, Np + 1, p->bytes));
        FCG_TRY(dalloc(&pl.lvl_kids, Np + 1, p->bytes));
        FCG_TRY(dalloc(&pl.blk_node_first, Np, p->bytes));
        FCG_TRY(dalloc(&pl.blk_chain, Np + 1, p->bytes));
        FCG_TRY(dalloc(&pl.top_nodes, Np, p->bytes));
        FCG_TRY(dalloc(&pl.top_kids, Np, p->bytes));
        // heights of an accepted tree are below 2^16 and below Np
        FCG_TRY(dalloc(&pl.top_hptr, std::min<int64_t>(Np, 1 << 16) + 2, p->bytes));
    }
    tr.mark("allocate");
    {
        // The caller's node, leaf and link arrays go to the device as they
        // are; kernels check them and build the device layout. The arrays the
        // structural checks read go first, then the checks (their result to a
        // pinned word), then the geometry on the problem's stream and the
        // link sources on a side stream, so the link upload overlaps the
        // layout kernels; the host waits only for the checks before it
        // launches anything that indexes with the caller's arrays.
        const int kMaxHeights = 1 << 16;  // heights sorted in two 8-bit passes
        int64_t tb = 0;
        int32_t *d_left = NULL, *d_right = NULL, *d_sptr = NULL;
        uint8_t *d_type = NULL, *d_cdiel = NULL, *d_ldiel = NULL;
        float *d_vert = NULL, *d_cent = NULL, *d_norm = NULL;
        double *d_area = NULL, *d_maxs = NULL, *d_out = NULL, *d_in = NULL, *d_surf = NULL;
        int64_t *d_lf = NULL, *d_lc = NULL, *d_cf = NULL, *ptr_model = NULL;
        uint32_t *src_model = NULL;
        // layout scratch
        int32_t *d_lab = NULL, *d_par = NULL, *d_height = NULL, *d_cnt = NULL, *seg_lo = NULL, *seg_hi = NULL, *hist = NULL;
        int32_t *bflag = NULL, *bid = NULL, *broot = NULL, *lvl_cnt = NULL, *node_cnt = NULL, *node_off = NULL;
        int32_t *bdep = NULL, *ent_blk = NULL, *pos_of = NULL, *tflag = NULL, *tpos = NULL;
        int *d_arrive = NULL;
        unsigned long long *ent = NULL, *ent2 = NULL, *chk = NULL;
        int32_t *ncount = NULL;                               // near links per model row
        long long *noff = NULL, *sums3 = NULL, *d_near = NULL;  // their offsets, scan scratch of s3, total
        int64_t *rowlen = NULL;
        // scal: [0] blocks, [1] plan levels, [2] block nodes, [3] top nodes, [4] spare, [5] chain entries
        long long *sums = NULL, *scal = NULL;
        int *iscal = NULL;  // [0] max height, [1] max depth above a block
        unsigned *dbad = NULL;  // [0] link sources out of range, [1] leaves not labelled by their leaf index
        unsigned hbad[2] = {0, 0};
        int hscal[2] = {0, 0};
        long long hs[8] = {0, 0, 0, 0, 0, 0, 0, 0};
        long long hblocks[1] = {0};
        unsigned long long hchk_local[4] = {0, 0, 0, 0};
        long long hnear = 0;
        // check results: [0] first bad node << 8 | code, [1] leaves, [2] first bad leaf
        unsigned long long *hchk = p->pin ? (unsigned long long *)p->pin : hchk_local;
        CentMax *d_cm = NULL;
        // link upload; link relabelling (at the device's highest priority: it
        // is the critical path, the layout kernels on s fill in around it)
        cudaStream_t s2 = NULL, s3 = NULL;
        int prio_hi = 0;
        cudaEvent_t ev_alloc = NULL, ev_lab = NULL, ev_rel = NULL;
        // the link sources go up in chunks of whole relabelling tiles; each
        // chunk's relabelling starts when its upload is done. From pageable
        // host memory a copy is staged synchronously, so chunks would only
        // serialise: one copy then.
        const int kLinkChunks = 8;
        const int64_t ntiles = (L + kRelTile - 1) / kRelTile;
        // (pinned host or device memory: the chunks go straight to the copy engine)
        const bool src_pinned = L > 0 && Stager::direct(a.link_src);
        int nchunk = L > 0 ? (src_pinned ? kLinkChunks : 1) : 0;
        std::vector<int64_t> tbound(nchunk + 1, 0);
        std::vector<cudaEvent_t> ev_src(nchunk, (cudaEvent_t)NULL);
        for (int c = 1; c <= nchunk; c++) tbound[c] = ntiles * c / nchunk;
        int32_t *tile_row = NULL;
        int nsurf = a.cond_surf_ptr[a.n_conductors];
        int rr = FCG_NORMAL_END;
        const int64_t ntile_max = devscan::grid_tiles(std::max<int64_t>(Nn, 1) * 1) * devscan::kDigits + 1;
        const int64_t near_cap = L / 16 + 4096;  // near list room; a larger count takes a second pass
        const int sms = ctx.sm_count;
        const int gN = grid_for(Nn, 256, sms);
        if (cudaStreamCreateWithFlags(&s2, cudaStreamNonBlocking) != cudaSuccess ||
            cudaDeviceGetStreamPriorityRange(NULL, &prio_hi) != cudaSuccess ||
            cudaStreamCreateWithPriority(&s3, cudaStreamNonBlocking, prio_hi) != cudaSuccess ||
            cudaEventCreateWithFlags(&ev_alloc, cudaEventDisableTiming) != cudaSuccess ||
            cudaEventCreateWithFlags(&ev_lab, cudaEventDisableTiming) != cudaSuccess ||
            cudaEventCreateWithFlags(&ev_rel, cudaEventDisableTiming) != cudaSuccess) {
            set_error("cannot create the upload stream");
            rr = FCG_DEVICE_ERROR;
        }
        for (int c = 0; c < nchunk && rr == FCG_NORMAL_END; c++)
            if (cudaEventCreateWithFlags(&ev_src[c], cudaEventDisableTiming) != cudaSuccess) {
                set_error("cannot create the upload events");
                rr = FCG_DEVICE_ERROR;
            }
        Stager st(ctx);
#define FCG_UP(ptr, host, n) if (rr == FCG_NORMAL_END) rr = upload_staged(st, &ptr, host, n, tb, s)
#define FCG_AL(ptr, n) if (rr == FCG_NORMAL_END) rr = dalloc(&ptr, (size_t)(n), tb)
        // 1. what the checks read, and the checks
        tr.dmark("start", s);
        FCG_UP(d_type, a.node_type, Nn);
        FCG_UP(d_left, a.node_left, Nn);
        FCG_UP(d_right, a.node_right, Nn);
        FCG_UP(d_lf, a.node_leaf_first, Nn);
        FCG_UP(d_lc, a.node_leaf_count, Nn);
        FCG_UP(ptr_model, a.link_ptr, Nn + 1);
        FCG_UP(d_cf, a.cond_leaf_first, a.n_conductors);
        FCG_UP(d_cdiel, a.cond_is_diel, a.n_conductors);
        FCG_UP(d_sptr, a.cond_surf_ptr, a.n_conductors + 1);
        FCG_UP(d_ldiel, a.leaf_diel, Np);
        FCG_AL(chk, 3);
        if (rr == FCG_NORMAL_END) {
            cudaMemsetAsync(chk, 0xff, 3 * sizeof(unsigned long long), s);
            cudaMemsetAsync(chk + 1, 0, sizeof(unsigned long long), s);
            k_check_model<<<gN, 256, 0, s>>>(Nn, Np, d_type, d_left, d_right, d_lf, d_lc, ptr_model, chk);
            k_check_leaves<<<grid_for(Np, 256, sms), 256, 0, s>>>(Np, a.n_conductors, d_cf, d_cdiel, d_sptr, d_ldiel, chk + 2);
            p->timings.launches += 2;
            if (cudaGetLastError() != cudaSuccess ||
                cudaMemcpyAsync(hchk, chk, 3 * sizeof(unsigned long long), cudaMemcpyDeviceToHost, s) != cudaSuccess ||
                cudaEventRecord(p->ev1, s) != cudaSuccess) {
                set_error("checking the model failed");
                rr = FCG_DEVICE_ERROR;
            }
        }
        // 2. the rest of the model: geometry on s, link sources on s2
        FCG_UP(d_vert, a.node_vertices, 9 * Nn);
        FCG_UP(d_cent, a.node_centroid, 3 * Nn);
        FCG_UP(d_norm, a.node_normal, 3 * Nn);
        FCG_UP(d_area, a.node_area, Nn);
        FCG_UP(d_maxs, a.node_maxside, Nn);
        FCG_UP(d_out, a.cond_outperm, a.n_conductors);
        FCG_UP(d_in, a.cond_inperm, a.n_conductors);
        FCG_UP(d_surf, a.cond_surf_outperm, std::max(nsurf, 1));
        FCG_AL(src_model, L);
        if (rr == FCG_NORMAL_END && L > 0) {
            bool ok = cudaEventRecord(ev_alloc, s) == cudaSuccess && cudaStreamWaitEvent(s2, ev_alloc, 0) == cudaSuccess;
            for (int c = 0; c < nchunk && ok; c++) {
                int64_t lo = tbound[c] * kRelTile, hi = std::min(tbound[c + 1] * kRelTile, L);
                if (hi > lo) ok = st.copy(src_model + lo, a.link_src + lo, (hi - lo) * sizeof(uint32_t), s2) == cudaSuccess;
                ok = ok && cudaEventRecord(ev_src[c], s2) == cudaSuccess;
                if (c == 0) tr.dmark("link chunk 0 uploaded", s2);
            }
            tr.dmark("links uploaded", s2);
            if (!ok) {
                set_error("uploading the links failed");
                rr = FCG_DEVICE_ERROR;
            }
        }
        FCG_AL(d_lab, Nn);
        FCG_AL(d_par, Nn);
        FCG_AL(d_height, Nn);
        FCG_AL(d_cnt, Nn);
        FCG_AL(seg_lo, kMaxHeights);
        FCG_AL(seg_hi, kMaxHeights);
        FCG_AL(hist, ntile_max);
        FCG_AL(ent, Nn);
        FCG_AL(ent2, Nn);
        FCG_AL(rowlen, Nn);
        FCG_AL(sums, devscan::grid_tiles(std::max<int64_t>(Nn, ntile_max)) + 1);
        FCG_AL(scal, 8);
        FCG_AL(iscal, 2);
        FCG_AL(bflag, Np + 1);
        FCG_AL(bid, Np + 1);
        FCG_AL(broot, Np);
        FCG_AL(lvl_cnt, Np + 1);
        FCG_AL(node_cnt, Np + 1);
        FCG_AL(node_off, Np + 1);
        FCG_AL(dbad, 2);
        FCG_AL(bdep, Np + 1);
        FCG_AL(ent_blk, Np + 1);
        FCG_AL(pos_of, Nn);
        FCG_AL(tflag, Nn);
        FCG_AL(tpos, Nn);
        FCG_AL(d_arrive, Nn);
        FCG_AL(d_near, 1);
        FCG_AL(d_cm, Nn);
        FCG_AL(ncount, Nn);
        FCG_AL(noff, Nn);
        FCG_AL(sums3, devscan::grid_tiles(Nn) + 1);
        FCG_AL(tile_row, std::max<int64_t>(ntiles, 1));
#undef FCG_UP
#undef FCG_AL
        if (rr == FCG_NORMAL_END) rr = dalloc(&p->link_src, L, p->bytes);
        if (rr == FCG_NORMAL_END) rr = dalloc(&p->near_link, (size_t)near_cap, p->bytes);
        if (rr == FCG_NORMAL_END) rr = dalloc(&p->near_row, (size_t)near_cap, p->bytes);
        // 3. the checks' verdict before anything indexes with the arrays
        if (rr == FCG_NORMAL_END) {
            if (cudaEventSynchronize(p->ev1) != cudaSuccess) {
                set_error("checking the model failed");
                rr = FCG_DEVICE_ERROR;
            } else if (hchk[0] != ~0ull) {
                set_error(std::string("invalid model: ") + node_check_message((int)(hchk[0] & 255)));
                rr = FCG_GENERIC_ERROR;
            } else if ((int64_t)hchk[1] != Np) {
                set_error("invalid model: leaf count does not match n_panels");
                rr = FCG_GENERIC_ERROR;
            } else if (hchk[2] != ~0ull) {
                set_error("invalid model: leaf permittivity index out of range");
                rr = FCG_GENERIC_ERROR;
            }
        }
        tr.mark("uploads and checks");
        tr.dmark("checks done (host sees)", s);
        if (rr == FCG_NORMAL_END) {
            using namespace devscan;
            cudaMemsetAsync(d_near, 0, sizeof(long long), s);
            cudaMemsetAsync(d_par, 0xff, Nn * sizeof(int32_t), s);     // roots: -1
            cudaMemsetAsync(p->parent, 0xff, Nn * sizeof(int32_t), s);
            cudaMemsetAsync(d_arrive, 0, Nn * sizeof(int), s);
            cudaMemsetAsync(iscal, 0, 2 * sizeof(int), s);
            cudaMemsetAsync(scal, 0, 8 * sizeof(long long), s);
            cudaMemsetAsync(dbad, 0, 2 * sizeof(unsigned), s);
            cudaMemsetAsync(bflag, 0, (Np + 1) * sizeof(int32_t), s);
            k_model_parents<<<gN, 256, 0, s>>>(Nn, d_type, d_left, d_right, d_par);
            k_heights<<<gN, 256, 0, s>>>(Nn, d_type, d_left, d_right, d_par, d_height, d_cnt, d_arrive, iscal);
            // labels: stable sort of the nodes by height (two 8-bit passes)
            k_height_entries<<<gN, 256, 0, s>>>(Nn, d_height, ent);
            {
                unsigned tiles = grid_tiles(Nn);
                int64_t nh = (int64_t)tiles * kDigits;
                unsigned long long *src = ent, *dst = ent2;
                for (int pass = 0; pass < 2; pass++) {
                    int shift = 32 + 8 * pass;
                    k_radix_hist<<<tiles, kThreads, 0, s>>>(Nn, src, shift, hist);
                    exclusive_scan(s, nh, hist, hist, sums, scal + 4);
                    k_radix_scatter<<<tiles, kThreads, 0, s>>>(Nn, src, shift, hist, pass == 1 ? nullptr : dst,
                                                               pass == 1 ? p->inv : nullptr);
                    std::swap(src, dst);
                }
            }
            k_labels<<<gN, 256, 0, s>>>(Nn, p->inv, d_lab);
            k_seg_bounds<<<gN, 256, 0, s>>>(Nn, p->inv, d_height, kMaxHeights, seg_lo, seg_hi);
            // row offsets in label order
            k_row_lengths<<<gN, 256, 0, s>>>(Nn, p->inv, ptr_model, rowlen);
            exclusive_scan(s, Nn, rowlen, p->link_ptr, sums, (long long *)(p->link_ptr + Nn));
            // the links: relabelled and classified on s3, chunk by chunk as
            // their upload completes, next to the rest of the layout on s
            k_cent_max<<<gN, 256, 0, s>>>(Nn, d_cent, d_maxs, d_lab, d_cm);
            p->timings.launches++;
            cudaEventRecord(ev_lab, s);
            cudaStreamWaitEvent(s3, ev_lab, 0);
            if (L > 0) {
                cudaMemsetAsync(ncount, 0, Nn * sizeof(int32_t), s3);
                k_tile_rows<<<gN, 256, 0, s3>>>(Nn, ptr_model, tile_row);
                p->timings.launches++;
            }
            for (int c = 0; c < nchunk; c++) {
                int64_t nt = tbound[c + 1] - tbound[c];
                cudaStreamWaitEvent(s3, ev_src[c], 0);
                if (nt <= 0) continue;
                int grid = (int)std::min<int64_t>(nt, (int64_t)sms * 5);
                k_relabel_classify<<<grid, 256, 0, s3>>>(Nn, L, tbound[c], tbound[c + 1], tile_row, ptr_model, src_model, p->link_ptr,
                                                         d_cm, p->link_src, dbad, ncount);
                p->timings.launches++;
                if (c == 0) tr.dmark("relabel chunk 0", s3);
            }
            if (L > 0) {
                // the near-field list in row order
                int grid = (int)std::min<int64_t>((Nn * 32 + 255) / 256, (int64_t)sms * 32);
                exclusive_scan(s3, Nn, ncount, noff, sums3, d_near);
                k_near_fill<<<grid, 256, 0, s3>>>(Nn, ptr_model, d_lab, p->link_ptr, p->link_src, ncount, noff, near_cap, p->near_link,
                                                  p->near_row);
                p->timings.launches += 4;
            }
            cudaEventRecord(ev_rel, s3);
            tr.dmark("relabel done", s3);
            // the device model
            k_build_nodes<<<gN, 256, 0, s>>>(Nn, d_lab, d_type, d_vert, d_cent, d_norm, d_area, d_maxs, d_left, d_right, d_lf, p->geo,
                                             p->left, p->right, p->parent, p->leaf_node, p->node_lfirst);
            k_build_leaves<<<grid_for(Np, 256, sms), 256, 0, s>>>(Np, a.n_conductors, d_cf, d_cdiel, d_out, d_in, d_sptr, d_surf,
                                                                   d_ldiel, p->leaf_eb, p->leaf_ea, p->leaf_weight);
            // scaled FP32 triangle tables of the mixed near field and self
            // terms (while the links are still uploading)
            if (precision == FCG_PREC_MIXED) {
                rr = dalloc(&p->tri32, Nn, p->bytes);
                if (rr == FCG_NORMAL_END) k_make_tri32<<<grid_for(Nn, 128, sms), 128, 0, s>>>(Nn, p->geo, p->tri32);
                p->timings.launches++;
            }
            // sweep plan: blocks numbered in leaf order, their levels
            k_block_flags<<<gN, 256, 0, s>>>(Nn, d_cnt, d_par, d_lf, bflag);
            exclusive_scan(s, Np, bflag, bid, sums, scal + 0);
            k_blocks<<<gN, 256, 0, s>>>(Nn, d_cnt, d_par, d_height, d_lf, d_lab, bid, p->plan, broot, lvl_cnt, node_cnt, bdep,
                                        iscal + 1);
            tr.dmark("layout kernels", s);
            p->timings.launches += 12;
            if (cudaGetLastError() != cudaSuccess ||
                cudaMemcpyAsync(hblocks, scal, sizeof(long long), cudaMemcpyDeviceToHost, s) != cudaSuccess ||
                cudaStreamSynchronize(s) != cudaSuccess) {
                set_error("building the device model failed");
                rr = FCG_DEVICE_ERROR;
            }
            int nb = (int)hblocks[0];
            if (rr == FCG_NORMAL_END && nb > 0) {
                exclusive_scan(s, nb, lvl_cnt, p->plan.blk_lvl_first, sums, scal + 1);
                exclusive_scan(s, nb, node_cnt, node_off, sums, scal + 2);
                k_block_levels<<<grid_for(nb, 128, sms), 128, 0, s>>>(nb, broot, d_cnt, d_height, p->inv, seg_lo, seg_hi, node_off,
                                                                      p->plan, ent_blk, pos_of);
                k_block_kids<<<grid_for(Np, 256, sms), 256, 0, s>>>(scal + 2, p->plan, ent_blk, pos_of, p->inv, d_lab, d_type, d_left,
                                                                    d_right, d_lf);
                exclusive_scan(s, nb, bdep, p->plan.blk_chain, sums, scal + 5);
                // top nodes by height, their children as top-local indices
                k_top_flags<<<gN, 256, 0, s>>>(Nn, Np, p->inv, d_cnt, p->leaf_node, tflag, dbad + 1);
                exclusive_scan(s, Nn, tflag, tpos, sums, scal + 3);
                k_top_list<<<gN, 256, 0, s>>>(Nn, p->inv, d_lab, d_cnt, d_left, d_right, d_lf, bid, tpos, scal + 0, p->plan);
                k_top_hptr<<<grid_for(std::min<int64_t>(Np, kMaxHeights) + 2, 256, sms), 256, 0, s>>>(
                    iscal + 0, (int)std::min<int64_t>(Np, kMaxHeights) - 1, seg_lo, tpos, scal + 3, p->plan.top_hptr);
                p->timings.launches += 18;
            }
            tr.dmark("plan kernels", s);
            cudaStreamWaitEvent(s, ev_rel, 0);  // the relabelled links
            if (rr == FCG_NORMAL_END &&
                (cudaGetLastError() != cudaSuccess ||
                 cudaMemcpyAsync(&hnear, d_near, sizeof(long long), cudaMemcpyDeviceToHost, s) != cudaSuccess ||
                 cudaMemcpyAsync(hbad, dbad, 2 * sizeof(unsigned), cudaMemcpyDeviceToHost, s) != cudaSuccess ||
                 cudaMemcpyAsync(hscal, iscal, 2 * sizeof(int), cudaMemcpyDeviceToHost, s) != cudaSuccess ||
                 cudaMemcpyAsync(hs, scal, 8 * sizeof(long long), cudaMemcpyDeviceToHost, s) != cudaSuccess ||
                 cudaStreamSynchronize(s) != cudaSuccess)) {
                set_error("building the device model failed");
                rr = FCG_DEVICE_ERROR;
            }
            if (rr == FCG_NORMAL_END) {
                p->plan.n_blocks = nb;
                if (hbad[0]) {
                    set_error("invalid model: " + std::to_string(hbad[0]) + " link sources out of range");
                    rr = FCG_GENERIC_ERROR;
                } else if (hscal[0] >= kMaxHeights || hscal[0] >= Np) {
                    set_error("node tree too high (" + std::to_string(hscal[0]) + " levels)");
                    rr = FCG_GENERIC_ERROR;
                } else if (hscal[1] > kMaxChain) {
                    set_error("node tree too deep above its 256-leaf subtrees (more than " + std::to_string(kMaxChain) + " levels)");
                    rr = FCG_GENERIC_ERROR;
                } else if (hbad[1]) {
                    set_error("invalid model: leaves are not in post-order leaf order");
                    rr = FCG_GENERIC_ERROR;
                }
            }
            if (rr == FCG_NORMAL_END && nb > 0) {
                // the ancestor chains, now that their total is known
                p->plan.n_top = (int)hs[3];
                p->plan.n_top_levels = hscal[0] + 1;
                rr = dalloc(&p->plan.chain, (size_t)std::max<long long>(hs[5], 1), p->bytes);
                if (rr == FCG_NORMAL_END) {
                    k_chains<<<grid_for(nb, 128, sms), 128, 0, s>>>(nb, broot, d_par, d_lab, p->plan);
                    p->timings.launches++;
                    if (cudaGetLastError() != cudaSuccess) {
                        set_error("building the sweep plan failed");
                        rr = FCG_DEVICE_ERROR;
                    }
                }
            }
            if (rr == FCG_NORMAL_END) {
                // the near-field list: complete unless it overflowed its room
                p->n_near = (int64_t)hnear;
                if (p->n_near > near_cap) {
                    dfree(p->near_link);
                    dfree(p->near_row);
                    rr = dalloc(&p->near_link, (size_t)p->n_near, p->bytes);
                    if (rr == FCG_NORMAL_END) rr = dalloc(&p->near_row, (size_t)p->n_near, p->bytes);
                    if (rr == FCG_NORMAL_END) {
                        int grid = (int)std::min<int64_t>((Nn * 32 + 255) / 256, (int64_t)sms * 32);
                        k_near_fill<<<grid, 256, 0, s>>>(Nn, ptr_model, d_lab, p->link_ptr, p->link_src, ncount, noff, p->n_near,
                                                         p->near_link, p->near_row);
                        p->timings.launches++;
                    }
                }
                // per-source FP64 triangle tables of the FP64 near field
                if (rr == FCG_NORMAL_END && precision == FCG_PREC_FP64 && p->n_near > 0) {
                    rr = dalloc(&p->tri, Nn, p->bytes);
                    if (rr == FCG_NORMAL_END) k_make_tri<<<grid_for(Nn, 128, sms), 128, 0, s>>>(Nn, p->geo, p->tri);
                    p->timings.launches++;
                }
                if (rr == FCG_NORMAL_END && cudaGetLastError() != cudaSuccess) {
                    set_error("building the near-field list failed");
                    rr = FCG_DEVICE_ERROR;
                }
            }
        }
        if (s2) cudaStreamSynchronize(s2);  // the link upload reads the caller's array and writes src_model
        if (s3) cudaStreamSynchronize(s3);  // the relabelling reads the scratch freed below
        dfree(d_type); dfree(d_vert); dfree(d_cent); dfree(d_norm); dfree(d_area); dfree(d_maxs);
        dfree(d_left); dfree(d_right); dfree(d_lf); dfree(d_cf); dfree(d_cdiel); dfree(d_out); dfree(d_in);
        dfree(d_sptr); dfree(d_surf); dfree(d_ldiel); dfree(src_model); dfree(ptr_model); dfree(dbad);
        dfree(d_lab); dfree(d_par); dfree(d_height); dfree(d_cnt); dfree(seg_lo); dfree(seg_hi); dfree(hist);
        dfree(ent); dfree(ent2); dfree(rowlen); dfree(sums); dfree(scal); dfree(iscal);
        dfree(bflag); dfree(bid); dfree(broot); dfree(lvl_cnt); dfree(node_cnt); dfree(node_off);
        dfree(bdep); dfree(ent_blk); dfree(pos_of); dfree(tflag); dfree(tpos); dfree(d_arrive);
        dfree(d_lc); dfree(chk); dfree(d_near); dfree(ncount); dfree(noff); dfree(sums3); dfree(tile_row);
        if (ev_alloc) cudaEventDestroy(ev_alloc);
        if (ev_lab) cudaEventDestroy(ev_lab);
        if (ev_rel) cudaEventDestroy(ev_rel);
        if (s3) cudaStreamDestroy(s3);
        dfree(d_cm);
        for (cudaEvent_t e : ev_src)
            if (e) cudaEventDestroy(e);
        if (s2) cudaStreamDestroy(s2);
        if (rr != FCG_NORMAL_END) { problem_destroy(p); return rr; }
    }
    tr.mark("device model and layout");
    tr.dreport();
    FCG_TRY(dalloc(&p->self, Np, p->bytes));
    if (precision == FCG_PREC_MIXED) {
        FCG_TRY(dalloc(&p->rself, Np, p->bytes));
        FCG_TRY(dalloc(&p->rself32, Np, p->bytes));
        FCG_TRY(dalloc(&p->srself, Np, p->bytes));
    }
    if (precision == FCG_PREC_FP64) FCG_TRY(dalloc(&p->coef64, a.n_links, p->bytes));
    else FCG_TRY(dalloc(&p->coef32, a.n_links, p->bytes));
    FCG_TRY(dalloc(&p->status, 1, p->bytes));
    FCG_TRY(dalloc(&p->fill_fp64, 1, p->bytes));
    FCG_TRY(set_row_split(p, (int64_t)ctx.sm_count * 32));
    // lanes per node in the link product: about four links per lane per pass
    {
        double avg = (double)a.n_links / (double)Nn;
        p->spmv_lanes = avg < 40.0 ? 8 : (avg < 160.0 ? 16 : 32);
        const char *env = getenv("FCG_SPMV_LANES");
        if (env && (atoi(env) == 8 || atoi(env) == 16 || atoi(env) == 32)) p->spmv_lanes = atoi(env);
    }
    // the uploads read host vectors that go out of scope: finish them here
    if (cudaStreamSynchronize(s) != cudaSuccess) {
        set_error(std::string("upload failed: ") + cudaGetErrorString(cudaGetLastError()));
        problem_destroy(p);
        return FCG_DEVICE_ERROR;
    }
    tr.mark("rest + sync");
    *out = p;
    return FCG_NORMAL_END;
#undef FCG_TRY
}

static void free_solve_ws(DeviceProblem *p);
static void free_two_level(DeviceProblem *p);

void problem_destroy(DeviceProblem *p) {
    if (!p) return;
    cudaSetDevice(p->ctx->device);
    if (p->stream) cudaStreamSynchronize(p->stream);
    AllocScope alloc_scope(p->stream);
    dfree(p->geo); dfree(p->link_ptr); dfree(p->link_src); dfree(p->leaf_node); dfree(p->parent);
    dfree(p->left); dfree(p->right); dfree(p->node_lfirst); dfree(p->leaf_eb); dfree(p->leaf_ea); dfree(p->leaf_weight);
    dfree(p->coef64); dfree(p->coef32); dfree(p->self); dfree(p->rself); dfree(p->rself32); dfree(p->srself); dfree(p->status);
    dfree(p->near_link); dfree(p->near_row); dfree(p->tri); dfree(p->tri32); dfree(p->fill_fp64);
    SweepPlan &pl = p->plan;
    dfree(pl.blk_leaf_first); dfree(pl.blk_nleaves); dfree(pl.blk_lvl_first); dfree(pl.blk_nlvls); dfree(pl.blk_root);
    dfree(pl.lvl_ptr); dfree(pl.lvl_nodes); dfree(pl.lvl_kids); dfree(pl.blk_node_first); dfree(pl.blk_chain); dfree(pl.chain);
    dfree(pl.top_nodes); dfree(pl.top_kids); dfree(pl.top_hptr); dfree(p->inv);
    dfree(p->Qd); dfree(p->Pd); dfree(p->Ad); dfree(p->Qf); dfree(p->Pf2); dfree(p->row_split);
    free_solve_ws(p);
    dfree(p->partial);
    dfree(p->leaf_geom); dfree(p->ch_start); dfree(p->ch_len); dfree(p->ch_geom); dfree(p->g_ch_first); dfree(p->g_ch_count);
    free_two_level(p);
    if (p->ev0) cudaEventDestroy(p->ev0);
    if (p->ev1) cudaEventDestroy(p->ev1);
    for (size_t i = 0; i < p->ev_pool.size(); i++) cudaEventDestroy(p->ev_pool[i]);
    if (p->stream && p->owns_stream) cudaStreamDestroy(p->stream);
    DeviceContext *ctx = p->ctx;
    pin_release(*ctx, p->pin);
    delete p;
    context_unref(ctx);
}

int64_t problem_device_bytes(const DeviceProblem *p) { return p ? p->bytes : 0; }

void problem_cancel(DeviceProblem *p) {
    if (!p) return;
    p->cancel.store(1);
    // the flag a running graph reads between Arnoldi steps
    if (p->pin) ((volatile int *)p->pin)[4] = 1;
}

int64_t problem_estimate_bytes(const fcg_model_arrays &a, int precision, int rhs, int iterations) {
    int64_t Nn = a.n_nodes, Np = a.n_panels, L = a.n_links;
    int64_t c = precision == FCG_PREC_FP64 ? 8 : 4;
    int k = std::max(1, std::min(rhs, kMaxK));
    int kp = 1;
    while (kp < k) kp <<= 1;
    int64_t nch = (Np + kDotChunk - 1) / kDotChunk + 1;
    // the basis is allocated 16 vectors at a time and, for the graph-run
    // Arnoldi loop, for at least 32 steps (33 vectors) up front
    int64_t steps = std::max(iterations, 32);
    int64_t vecs = ((steps + 1 + 15) / 16) * 16;
    int64_t b = 0;
    b += Nn * (int64_t)(sizeof(NodeGeo) + 8 + 4 * 3 + 4);  // geometry, row pointers, tree, labels
    b += Np * (int64_t)(4 * 7 + 4 + 12 + 4 + 8);          // sweep plan: blocks, levels, children, top forest, chains (typical)
    b += L * (4 + c);                                                  // links
    b += Np * (4 + 8 * 4 + 4);                                         // leaf maps, permittivities, self terms, geometry map
    b += L * 8 + Nn * (int64_t)(precision == FCG_PREC_FP64 ? sizeof(fcg_tri64) : sizeof(fcg_tri32));  // near list (bound) and tables
    b += (int64_t)kp * Nn * (8 * 3 + 4 + 8);                           // matvec node work
    b += (int64_t)k * Np * 8 * (5 + vecs);                             // Krylov vectors and basis
    b += (int64_t)k * (steps + 1) * nch * 8;                           // partial sums
    return b + b / 10;
}

void *stream_create(int device) {
    cudaStream_t s = NULL;
    if (cudaSetDevice(device) != cudaSuccess || cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking) != cudaSuccess) {
        cudaGetLastError();
        return NULL;
    }
    return (void *)s;
}

void stream_destroy(int device, void *stream) {
    if (!stream) return;
    cudaSetDevice(device);
    cudaStreamSynchronize((cudaStream_t)stream);
    cudaStreamDestroy((cudaStream_t)stream);
}
int problem_n_cond(const DeviceProblem *p) { return p ? (int)p->cond_cols.size() : 0; }
SolveTimings problem_timings(const DeviceProblem *p) { return p ? p->timings : SolveTimings(); }

int problem_set_profiling(DeviceProblem *p, bool on) {
    p->profiling = on;
    return FCG_NORMAL_END;
}

int problem_set_tuning(DeviceProblem *p, bool on) {
    p->tuning = on;
    return FCG_NORMAL_END;
}

void problem_reset_stats(DeviceProblem *p) {
    p->timings.launches = p->timings.link_launches = p->timings.link_bytes = 0;
    p->timings.link_ms = 0;
    p->timings.matvecs = 0;
    p->timings.refine_checks = p->timings.refine_cycles = 0;
}

// event pair around one link-product launch (profiling mode)
static void prof_begin(DeviceProblem *p) {
    if (!p->profiling) return;
    if (p->ev_used + 2 > p->ev_pool.size()) {
        for (int i = 0; i < 64; i++) {
            cudaEvent_t e;
            if (cudaEventCreate(&e) != cudaSuccess) return;
            p->ev_pool.push_back(e);
        }
    }
    cudaEventRecord(p->ev_pool[p->ev_used], p->stream);
}
static void prof_end(DeviceProblem *p) {
    if (!p->profiling || p->ev_used + 2 > p->ev_pool.size()) return;
    cudaEventRecord(p->ev_pool[p->ev_used + 1], p->stream);
    p->ev_used += 2;
}
// read the recorded pairs (the stream must be synchronised)
static void prof_collect(DeviceProblem *p) {
    for (size_t i = 0; i + 1 < p->ev_used; i += 2) {
        float ms = 0;
        if (cudaEventElapsedTime(&ms, p->ev_pool[i], p->ev_pool[i + 1]) == cudaSuccess) p->timings.link_ms += ms;
    }
    p->ev_used = 0;
}

static int check_status(DeviceProblem *p, const char *what) {
    unsigned st = 0;
    FCG_CK(cudaMemcpyAsync(&st, p->status, sizeof(unsigned), cudaMemcpyDeviceToHost, p->stream));
    FCG_CK(cudaStreamSynchronize(p->stream));
    if (st) {
        set_error(std::string(what) + ": non-finite or zero coefficient (status " + std::to_string(st) + ")");
        return FCG_GENERIC_ERROR;
    }
    return FCG_NORMAL_END;
}

int problem_fill(DeviceProblem *p) {
    AllocScope alloc_scope(p->stream);
    FCG_CK(cudaSetDevice(p->ctx->device));
    cudaStream_t s = p->stream;
    FCG_CK(cudaMemsetAsync(p->status, 0, sizeof(unsigned), s));
    FCG_CK(cudaMemsetAsync(p->fill_fp64, 0, sizeof(unsigned long long), s));
    FCG_CK(cudaEventRecord(p->ev0, s));
    int sms = p->ctx->sm_count;
    bool mixed = p->precision == FCG_PREC_MIXED;
    if (p->L > 0) {
        int grid = (int)std::min<int64_t>((p->Nn * 32 + 255) / 256, (int64_t)sms * 32);
        if (mixed)
            k_fill_far32<<<p->n_row_split, 256, 0, s>>>(p->row_split, p->link_ptr, p->link_src, p->geo, p->coef32, p->status);
        else k_fill_far<<<grid, 256, 0, s>>>(p->Nn, p->link_ptr, p->link_src, p->geo, p->coef64, p->status);
        FCG_CK(cudaGetLastError());
        p->timings.launches++;
        if (p->n_near > 0) {
            if (mixed)
                k_fill_near32<<<grid_for(p->n_near, 128, sms), 128, 0, s>>>(p->n_near, p->near_link, p->near_row, p->link_src,
                                                                           p->geo, p->tri32, p->coef32, p->status, p->fill_fp64);
            else
                k_fill_near<<<grid_for(p->n_near, 128, sms), 128, 0, s>>>(p->n_near, p->near_link, p->near_row, p->link_src,
                                                                         p->geo, p->tri, p->coef64, p->coef32, p->status);
            FCG_CK(cudaGetLastError());
            p->timings.launches++;
        }
    }
    if (mixed)
        k_fill_self32<<<grid_for(p->Np, 256, sms), 256, 0, s>>>(p->Np, p->leaf_node, p->geo, p->tri32, p->leaf_eb, p->leaf_ea,
                                                               p->self, p->rself, p->rself32, p->srself, p->status,
                                                               p->fill_fp64);
    else
        k_fill_self<<<grid_for(p->Np, 256, sms), 256, 0, s>>>(p->Np, p->leaf_node, p->geo, p->leaf_eb, p->leaf_ea, p->self,
                                                             p->status);
    FCG_CK(cudaGetLastError());
    p->timings.launches++;
    FCG_CK(cudaEventRecord(p->ev1, s));
    unsigned long long fb = 0;
    FCG_CK(cudaMemcpyAsync(&fb, p->fill_fp64, sizeof fb, cudaMemcpyDeviceToHost, s));
    int r = check_status(p, "coefficient fill");
    p->timings.fill_fp64 = (int64_t)fb;
    cudaEventElapsedTime(&p->timings.fill_ms, p->ev0, p->ev1);
    if (r != FCG_NORMAL_END) return r;
    p->filled = true;
    return FCG_NORMAL_END;
}

int problem_get_coefficients(DeviceProblem *p, double *link_coef, double *self_coef) {
    AllocScope alloc_scope(p->stream);
    if (!p->filled) { set_error("coefficients not filled"); return FCG_GENERIC_ERROR; }
    FCG_CK(cudaSetDevice(p->ctx->device));
    if (link_coef && p->L) {
        std::vector<double> dev(p->L);
        if (p->coef64) {
            FCG_CK(cudaMemcpyAsync(dev.data(), p->coef64, p->L * sizeof(double), cudaMemcpyDeviceToHost, p->stream));
            FCG_CK(cudaStreamSynchronize(p->stream));
        } else {
            std::vector<float> tmp(p->L);
            FCG_CK(cudaMemcpyAsync(tmp.data(), p->coef32, p->L * sizeof(float), cudaMemcpyDeviceToHost, p->stream));
            FCG_CK(cudaStreamSynchronize(p->stream));
            for (int64_t l = 0; l < p->L; l++) dev[l] = tmp[l];
        }
        // device rows are in height-major order; return the model's link order
        if (p->h_inv.empty()) {  // the maps between the orders, made on first use
            int64_t Nn = p->Nn;
            p->h_inv.resize(Nn);
            p->h_ptr_dev.resize(Nn + 1);
            FCG_CK(cudaMemcpyAsync(p->h_inv.data(), p->inv, Nn * sizeof(int32_t), cudaMemcpyDeviceToHost, p->stream));
            FCG_CK(cudaMemcpyAsync(p->h_ptr_dev.data(), p->link_ptr, (Nn + 1) * sizeof(int64_t), cudaMemcpyDeviceToHost, p->stream));
            FCG_CK(cudaStreamSynchronize(p->stream));
            std::vector<int64_t> len(Nn);
            for (int64_t q = 0; q < Nn; q++) len[p->h_inv[q]] = p->h_ptr_dev[q + 1] - p->h_ptr_dev[q];
            p->h_ptr_model.assign(Nn + 1, 0);
            for (int64_t i = 0; i < Nn; i++) p->h_ptr_model[i + 1] = p->h_ptr_model[i] + len[i];
        }
        for (int64_t q = 0; q < p->Nn; q++) {
            int64_t i = p->h_inv[q], cnt = p->h_ptr_dev[q + 1] - p->h_ptr_dev[q];
            memcpy(link_coef + p->h_ptr_model[i], dev.data() + p->h_ptr_dev[q], cnt * sizeof(double));
        }
    }
    if (self_coef) {
        FCG_CK(cudaMemcpyAsync(self_coef, p->self, p->Np * sizeof(double), cudaMemcpyDeviceToHost, p->stream));
        FCG_CK(cudaStreamSynchronize(p->stream));
    }
    return FCG_NORMAL_END;
}

// node-work columns for k right-hand sides: 1, 2, else a multiple of four
// (the multi-right-hand-side link product moves four per 16-byte gather)
static int kpad(int k) { return k <= 2 ? k : (k + 3) / 4 * 4; }

static int ensure_matvec_ws(DeviceProblem *p, int kp) {
    if (p->kcap >= kp) return FCG_NORMAL_END;
    dfree(p->Qd); dfree(p->Pd); dfree(p->Ad); dfree(p->Qf); dfree(p->Pf2);
    p->kcap = 0;
    int r;
    size_t n = (size_t)p->Nn * kp;
    if ((r = dalloc(&p->Qd, n, p->bytes))) return r;
    if ((r = dalloc(&p->Ad, n, p->bytes))) return r;
    if (p->precision == FCG_PREC_MIXED) {
        if ((r = dalloc(&p->Qf, n, p->bytes))) return r;
        if ((r = dalloc(&p->Pf2, n, p->bytes))) return r;
    } else {
        if ((r = dalloc(&p->Pd, n, p->bytes))) return r;
    }
    // padding columns (right-hand sides k..kp-1) are read by the link product
    // but never written by the up-sweep: start them at zero; afterwards they
    // only ever hold finite charges, and columns never mix
    FCG_CK(cudaMemsetAsync(p->Qd, 0, n * sizeof(double), p->stream));
    if (p->Qf) FCG_CK(cudaMemsetAsync(p->Qf, 0, n * sizeof(float), p->stream));
    p->kcap = kp;
    return FCG_NORMAL_END;
}

// node work arrays of one product (kp values per node)
struct NodeWork {
    double *Qd;
    float *Qf;
    double *Pd;
    float2 *Pf2;
    double *Ad;  // the block roots' charges in block order (n_blocks x kp of it)
};

// One link-product launch (the kernel follows kp, precision and the
// problem's launch shape: lanes per row, CTA row ranges).
static void launch_link(DeviceProblem *p, const NodeWork &w, int kp, bool mixed) {
    cudaStream_t s = p->stream;
    int64_t rows_per_cta = 8 * (32 / p->spmv_lanes);
    int grid = (int)std::min<int64_t>((p->Nn + rows_per_cta - 1) / rows_per_cta, (int64_t)p->ctx->sm_count * 32);
        int sw = p->spmv_lanes;
#define FCG_SPMV(KK)                                                                                                  \
    do {                                                                                                              \
        if (mixed) {                                                                                                  \
            if (sw == 8) k_spmv32<KK, 8><<<grid, 256, 0, s>>>(p->Nn, p->link_ptr, p->link_src, p->coef32, w.Qf, w.Pf2); \
            else if (sw == 16) k_spmv32<KK, 16><<<grid, 256, 0, s>>>(p->Nn, p->link_ptr, p->link_src, p->coef32, w.Qf, w.Pf2); \
            else k_spmv32<KK, 32><<<grid, 256, 0, s>>>(p->Nn, p->link_ptr, p->link_src, p->coef32, w.Qf, w.Pf2);     \
        } else {                                                                                                      \
            if (sw == 8) k_spmv64<KK, 8><<<grid, 256, 0, s>>>(p->Nn, p->link_ptr, p->link_src, p->coef64, w.Qd, w.Pd); \
            else if (sw == 16) k_spmv64<KK, 16><<<grid, 256, 0, s>>>(p->Nn, p->link_ptr, p->link_src, p->coef64, w.Qd, w.Pd); \
            else k_spmv64<KK, 32><<<grid, 256, 0, s>>>(p->Nn, p->link_ptr, p->link_src, p->coef64, w.Qd, w.Pd);     \
        }                                                                                                             \
    } while (0)
        const int mgrid = p->n_row_split;
        const int32_t *rs = p->row_split;
#define FCG_MULTI32(KK) k_spmv32_multi<KK><<<mgrid, 256, 0, s>>>(rs, p->link_ptr, p->link_src, p->coef32, w.Qf, w.Pf2)
#define FCG_MULTI64(KK) k_spmv64_multi<KK><<<mgrid, 256, 0, s>>>(rs, p->link_ptr, p->link_src, p->coef64, w.Qd, w.Pd)
        if (kp == 1) {
            FCG_SPMV(1);
        } else if (mixed && kp == 2) {
            FCG_SPMV(2);
        } else if (mixed) {
            switch (kp) {
            case 4: FCG_MULTI32(4); break;
            case 8: FCG_MULTI32(8); break;
            case 12: FCG_MULTI32(12); break;
            case 16: FCG_MULTI32(16); break;
            case 20: FCG_MULTI32(20); break;
            case 24: FCG_MULTI32(24); break;
            case 28: FCG_MULTI32(28); break;
            default: FCG_MULTI32(32); break;
            }
        } else {
            switch (kp) {
            case 2: FCG_MULTI64(2); break;
            case 4: FCG_MULTI64(4); break;
            case 8: FCG_MULTI64(8); break;
            case 12: FCG_MULTI64(12); break;
            case 16: FCG_MULTI64(16); break;
            case 20: FCG_MULTI64(20); break;
            case 24: FCG_MULTI64(24); break;
            case 28: FCG_MULTI64(28); break;
            default: FCG_MULTI64(32); break;
            }
        }
#undef FCG_MULTI32
#undef FCG_MULTI64
#undef FCG_SPMV
}

// The launches of one product v = P * (in / diag): up-sweep (blocks, then
// the top forest when there is one), link product, down-sweep. Arrays in/out
// are [k][Np] on the device.
static int launch_matvec(DeviceProblem *p, const NodeWork &w, const double *in, double *out, int k, int kp, const double *diag,
                         const StepScale *scale = NULL) {
    const StepScale sc = scale ? *scale : StepScale{NULL, 0, NULL, NULL, NULL, NULL, 0};
    cudaStream_t s = p->stream;
    bool mixed = p->precision == FCG_PREC_MIXED;
    const SweepPlan &pl = p->plan;
    int64_t Np = p->Np;
    size_t n = (size_t)p->Nn * kp;
    const int kc = std::min(k, kSweepCols);
    const size_t up_smem = (size_t)(2 * kBlockLeaves - 1) * kc * sizeof(double) + (3 * kBlockLeaves + 1) * sizeof(int32_t);
    const size_t down_smem = ((size_t)(3 * kBlockLeaves - 1 + kMaxChain) * kc + kBlockLeaves) * sizeof(double) +
                             (2 * kBlockLeaves + 1) * sizeof(int32_t);
    // the mixed path's Jacobi scaling multiplies by the reciprocals (the
    // FP64 path divides, as the reference does)
    const int recip = mixed && diag == p->self && p->rself ? 1 : 0;
    const double *dg = recip ? p->rself : diag;
    // the mixed path's sweeps in FP32 pairs, for Jacobi scaling (the self
    // terms' reciprocals) or none; any other scaling takes the FP64 sweeps
    if (mixed && (diag == NULL || recip)) {
        // KC right-hand sides per thread and pass (over all kp columns)
        const int KC = kp >= 4 ? 4 : kp;
        const size_t up32 = (size_t)(2 * kBlockLeaves - 1) * KC * sizeof(float2) + (3 * kBlockLeaves + 1) * sizeof(int32_t);
        const size_t down32 = (size_t)(2 * kBlockLeaves - 1 + kMaxChain) * KC * sizeof(float2) + kBlockLeaves * sizeof(double) +
                              (3 * kBlockLeaves + kMaxChain + 1) * sizeof(int32_t);
        const dim3 bgrid(pl.n_blocks, kp / KC);
        float2 *rootq = reinterpret_cast<float2 *>(w.Ad);
        const float *rs = recip ? p->rself32 : NULL;
        const double *sr = recip ? p->srself : p->self;
        if (KC == 4) k_up_blk32<4><<<bgrid, kSweepThreads, up32, s>>>(pl, in, Np, k, kp, rs, w.Qf, rootq, sc);
        else if (KC == 2) k_up_blk32<2><<<bgrid, kSweepThreads, up32, s>>>(pl, in, Np, k, kp, rs, w.Qf, rootq, sc);
        else k_up_blk32<1><<<bgrid, kSweepThreads, up32, s>>>(pl, in, Np, k, kp, rs, w.Qf, rootq, sc);
        FCG_CK(cudaGetLastError());
        int64_t launches = 2;
        if (pl.n_top > 0) {
            size_t fixed = (size_t)pl.n_top * (sizeof(int2) + sizeof(int32_t)) + (size_t)(pl.n_top_levels + 1) * sizeof(int32_t);
            size_t top32 = fixed + (size_t)(pl.n_blocks + pl.n_top) * KC * sizeof(float2);
            if (top32 <= p->ctx->smem_optin) {
                if (KC == 4) k_up_top32<4><<<kp / KC, 1024, top32, s>>>(pl, kp, rootq, w.Qf);
                else if (KC == 2) k_up_top32<2><<<kp / KC, 1024, top32, s>>>(pl, kp, rootq, w.Qf);
                else k_up_top32<1><<<kp / KC, 1024, top32, s>>>(pl, kp, rootq, w.Qf);
            } else {
                k_up_top32_global<<<1, 1024, 0, s>>>(pl, kp, rootq, reinterpret_cast<float2 *>(w.Qd), w.Qf);
            }
            FCG_CK(cudaGetLastError());
            launches++;
        }
        if (p->L > 0) {
            p->timings.link_bytes += p->L * 8 + 8 * (p->Nn + 1) + 12 * (int64_t)k * p->Nn;
            p->timings.link_launches++;
            launches++;
            prof_begin(p);
            launch_link(p, w, kp, true);
            prof_end(p);
            FCG_CK(cudaGetLastError());
        } else {
            FCG_CK(cudaMemsetAsync(w.Pf2, 0, n * sizeof(float2), s));
        }
        if (KC == 4) k_down_blk32<4><<<bgrid, kSweepThreads, down32, s>>>(pl, in, Np, k, kp, sr, w.Pf2, out);
        else if (KC == 2) k_down_blk32<2><<<bgrid, kSweepThreads, down32, s>>>(pl, in, Np, k, kp, sr, w.Pf2, out);
        else k_down_blk32<1><<<bgrid, kSweepThreads, down32, s>>>(pl, in, Np, k, kp, sr, w.Pf2, out);
        FCG_CK(cudaGetLastError());
        p->timings.matvecs++;
        p->timings.launches += launches;
        return FCG_NORMAL_END;
    }
    // w.Ad (n_nodes x kp) holds the block roots' charges in block order
    if (mixed) k_up_blk<true><<<pl.n_blocks, kSweepThreads, up_smem, s>>>(pl, in, Np, k, kp, kc, dg, recip, w.Qd, w.Qf, w.Ad, sc);
    else k_up_blk<false><<<pl.n_blocks, kSweepThreads, up_smem, s>>>(pl, in, Np, k, kp, kc, dg, recip, w.Qd, w.Qf, w.Ad, sc);
    FCG_CK(cudaGetLastError());
    int64_t launches = 2;
    if (pl.n_top > 0) {
        // the top forest in shared memory, as many right-hand sides per pass as fit
        size_t fixed = (size_t)pl.n_top * (sizeof(int2) + sizeof(int32_t)) + (size_t)(pl.n_top_levels + 1) * sizeof(int32_t);
        size_t per_col = (size_t)(pl.n_blocks + pl.n_top) * sizeof(double);
        size_t room = p->ctx->smem_optin > fixed ? p->ctx->smem_optin - fixed : 0;
        int tkc = (int)std::min<size_t>((size_t)k, room / per_col);
        if (tkc >= 1) {
            size_t top_smem = fixed + per_col * tkc;
            if (mixed) k_up_top<true><<<1, 1024, top_smem, s>>>(pl, k, kp, tkc, w.Ad, w.Qd, w.Qf);
            else k_up_top<false><<<1, 1024, top_smem, s>>>(pl, k, kp, tkc, w.Ad, w.Qd, w.Qf);
        } else {
            if (mixed) k_up_top_global<true><<<1, 1024, 0, s>>>(pl, k, kp, w.Qd, w.Qf);
            else k_up_top_global<false><<<1, 1024, 0, s>>>(pl, k, kp, w.Qd, w.Qf);
        }
        FCG_CK(cudaGetLastError());
        launches++;
    }
    if (p->L > 0) {
        // coefficient + source word per link, row offsets, one charge read and
        // one potential write per node and right-hand side
        int64_t cb = mixed ? 4 : 8;
        p->timings.link_bytes += p->L * (cb + 4) + 8 * (p->Nn + 1) + (cb + 8) * (int64_t)k * p->Nn;
        p->timings.link_launches++;
        launches++;
        prof_begin(p);
        launch_link(p, w, kp, mixed);
        prof_end(p);
        FCG_CK(cudaGetLastError());
    } else {
        if (mixed) FCG_CK(cudaMemsetAsync(w.Pf2, 0, n * sizeof(float2), s));
        else FCG_CK(cudaMemsetAsync(w.Pd, 0, n * sizeof(double), s));
    }
    if (mixed) k_down_blk<float2><<<pl.n_blocks, kSweepThreads, down_smem, s>>>(pl, in, Np, k, kp, kc, dg, recip, p->self, w.Pf2, out);
    else k_down_blk<double><<<pl.n_blocks, kSweepThreads, down_smem, s>>>(pl, in, Np, k, kp, kc, dg, recip, p->self, w.Pd, out);
    FCG_CK(cudaGetLastError());
    p->timings.matvecs++;
    p->timings.launches += launches;
    return FCG_NORMAL_END;
}

// Autotuner of the mixed link product's launch shape, per problem shape
// (kp, links per node, node count): lanes per row for one right-hand side
// (8, 16, 32), CTA row ranges for several (SMs x 8..64). Each candidate is
// timed over three launches with CUDA events on the problem's stream; the
// winner is kept in the context, so later problems of the same shape reuse
// it without measuring. Problems under 4M links keep the built-in choice.
// FCG_SPMV_LANES pins the lanes.
static int autotune(DeviceProblem *p, int kp) {
    if (kp >= 64) return FCG_NORMAL_END;
    cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
    if (cudaStreamIsCapturing(p->stream, &cs) != cudaSuccess || cs != cudaStreamCaptureStatusNone) return FCG_NORMAL_END;
    bool single = kp <= 2;
    DeviceContext &ctx = *p->ctx;
    int sms = ctx.sm_count;
    auto apply = [&](int v) -> int {
        p->tune_val[kp] = v;
        if (single) { p->spmv_lanes = v; return FCG_NORMAL_END; }
        return set_row_split(p, (int64_t)sms * v);
    };
    // settled before: put this width's shape back (another width may have
    // set the problem's lanes or row ranges since)
    if ((p->tuned >> kp) & 1u) return p->tune_val[kp] ? apply(p->tune_val[kp]) : FCG_NORMAL_END;
    p->tuned |= 1ull << kp;
    bool mixed = p->precision == FCG_PREC_MIXED;
    if (!mixed || !p->tuning || p->L < (int64_t)4 << 20 || (single && getenv("FCG_SPMV_LANES"))) return FCG_NORMAL_END;
    double avg = (double)p->L / (double)p->Nn;
    uint64_t key = (uint64_t)kp | ((uint64_t)(int)(4.0 * log2(avg + 1.0)) << 8) | ((uint64_t)(int)log2((double)p->Nn) << 16);
    {
        std::lock_guard<std::mutex> lk(ctx.tune_mu);
        auto it = ctx.tune.find(key);
        if (it != ctx.tune.end()) return apply(it->second);
    }
    std::vector<int> cand = single ? std::vector<int>{8, 16, 32} : std::vector<int>{8, 16, 32, 64};
    NodeWork w = {p->Qd, p->Qf, p->Pd, p->Pf2, p->Ad};
    float best_ms = 1e30f;
    int best = single ? p->spmv_lanes : 32;
    cudaEvent_t e0, e1;
    FCG_CK(cudaEventCreate(&e0));
    if (cudaEventCreate(&e1) != cudaSuccess) {
        cudaEventDestroy(e0);
        set_error("cannot create timing events");
        return FCG_DEVICE_ERROR;
    }
    cudaError_t err = cudaSuccess;
    for (int v : cand) {
        int r = apply(v);
        if (r != FCG_NORMAL_END) { cudaEventDestroy(e0); cudaEventDestroy(e1); return r; }
        launch_link(p, w, kp, true);  // warm
        cudaEventRecord(e0, p->stream);
        for (int q = 0; q < 3; q++) launch_link(p, w, kp, true);
        cudaEventRecord(e1, p->stream);
        if ((err = cudaGetLastError()) != cudaSuccess || (err = cudaEventSynchronize(e1)) != cudaSuccess) break;
        float ms = 0;
        cudaEventElapsedTime(&ms, e0, e1);
        p->timings.launches += 4;
        if (ms < best_ms) { best_ms = ms; best = v; }
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (err != cudaSuccess) {
        set_error(std::string("link-product tuning failed: ") + cudaGetErrorString(err));
        return FCG_DEVICE_ERROR;
    }
    {
        std::lock_guard<std::mutex> lk(ctx.tune_mu);
        ctx.tune[key] = best;
    }
    return apply(best);
}

// Right-hand-side width of the batched solves (columns per batch) when the
// caller leaves it open: with more columns per batch the coefficients and
// source words are read once for more columns, but the charge gathers grow
// with the width and stop hitting in L1. Candidates 4, 8, 16 and all of the
// conductors (at most 32); each candidate's link product (in its tuned launch
// shape) is timed over three launches and the width with the least product
// time per solve, ceil(columns / width) x time(width), wins. Mixed problems
// of at least 4M links and more than 4 columns only; the choice is kept in
// the context per problem shape.
static int choose_rhs_width(DeviceProblem *p, int cols, int *width) {
    *width = std::min(cols, kMaxK);
    if (p->precision != FCG_PREC_MIXED || !p->tuning || p->L < ((int64_t)4 << 20) || cols <= 4) return FCG_NORMAL_END;
    cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
    if (cudaStreamIsCapturing(p->stream, &cs) != cudaSuccess || cs != cudaStreamCaptureStatusNone) return FCG_NORMAL_END;
    DeviceContext &ctx = *p->ctx;
    const int full = std::min(cols, kMaxK);
    double avg = (double)p->L / (double)p->Nn;
    uint64_t key = (1ull << 40) | (uint64_t)full | ((uint64_t)(int)(4.0 * log2(avg + 1.0)) << 8) |
                   ((uint64_t)(int)log2((double)p->Nn) << 16);
    {
        std::lock_guard<std::mutex> lk(ctx.tune_mu);
        auto it = ctx.tune.find(key);
        if (it != ctx.tune.end()) { *width = it->second; return FCG_NORMAL_END; }
    }
    std::vector<int> cand;
    for (int w : {4, 8, 16, full})
        if (w <= full && std::find(cand.begin(), cand.end(), w) == cand.end()) cand.push_back(w);
    cudaEvent_t e0, e1;
    FCG_CK(cudaEventCreate(&e0));
    if (cudaEventCreate(&e1) != cudaSuccess) {
        cudaEventDestroy(e0);
        set_error("cannot create timing events");
        return FCG_DEVICE_ERROR;
    }
    // the workspace for the widest candidate serves them all
    int r = ensure_matvec_ws(p, kpad(full));
    double best = 1e300;
    int best_w = full;
    for (size_t i = 0; i < cand.size() && r == FCG_NORMAL_END; i++) {
        int w = cand[i], kp = kpad(w);
        if ((r = autotune(p, kp)) != FCG_NORMAL_END) break;
        NodeWork nw = {p->Qd, p->Qf, p->Pd, p->Pf2, p->Ad};
        launch_link(p, nw, kp, true);  // warm
        cudaEventRecord(e0, p->stream);
        for (int q = 0; q < 3; q++) launch_link(p, nw, kp, true);
        cudaEventRecord(e1, p->stream);
        cudaError_t err = cudaGetLastError();
        if (err == cudaSuccess) err = cudaEventSynchronize(e1);
        if (err != cudaSuccess) {
            set_error(std::string("right-hand-side width tuning failed: ") + cudaGetErrorString(err));
            r = FCG_DEVICE_ERROR;
            break;
        }
        float ms = 0;
        cudaEventElapsedTime(&ms, e0, e1);
        p->timings.launches += 4;
        double cost = (double)((full + w - 1) / w) * ms;
        if (cost < best) { best = cost; best_w = w; }
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (r != FCG_NORMAL_END) return r;
    {
        std::lock_guard<std::mutex> lk(ctx.tune_mu);
        ctx.tune[key] = best_w;
    }
    *width = best_w;
    return FCG_NORMAL_END;
}

// v = P * (in / diag) for k right-hand sides ([k][Np] device arrays)
static int matvec(DeviceProblem *p, const double *in, double *out, int k, const double *diag, const StepScale *scale = NULL) {
    if (k < 1 || k > kMaxK) { set_error("right-hand sides per matvec must be in [1, 32]"); return FCG_GENERIC_ERROR; }
    int kp = kpad(k);
    int r = ensure_matvec_ws(p, kp);
    if (r == FCG_NORMAL_END) r = autotune(p, kp);
    if (r != FCG_NORMAL_END) return r;
    NodeWork w = {p->Qd, p->Qf, p->Pd, p->Pf2, p->Ad};
    return launch_matvec(p, w, in, out, k, kp, diag, scale);
}

int problem_matvec_device(DeviceProblem *p, const double *d_q, double *d_v, int k) {
    AllocScope alloc_scope(p->stream);
    if (!p->filled) { set_error("coefficients not filled"); return FCG_GENERIC_ERROR; }
    FCG_CK(cudaSetDevice(p->ctx->device));
    int r = matvec(p, d_q, d_v, k, NULL);
    if (r != FCG_NORMAL_END) return r;
    FCG_CK(cudaStreamSynchronize(p->stream));
    prof_collect(p);
    return FCG_NORMAL_END;
}

int problem_matvec_host(DeviceProblem *p, const double *q, double *v, int k) {
    AllocScope alloc_scope(p->stream);
    if (!p->filled) { set_error("coefficients not filled"); return FCG_GENERIC_ERROR; }
    FCG_CK(cudaSetDevice(p->ctx->device));
    double *dq = NULL, *dv = NULL;
    int64_t tmp = 0;
    size_t n = (size_t)k * p->Np;
    int r = dalloc(&dq, n, tmp);
    if (r == FCG_NORMAL_END) r = dalloc(&dv, n, tmp);
    if (r == FCG_NORMAL_END && cudaMemcpyAsync(dq, q, n * sizeof(double), cudaMemcpyHostToDevice, p->stream) != cudaSuccess) {
        set_error("copy of q failed");
        r = FCG_DEVICE_ERROR;
    }
    for (int r0 = 0; r == FCG_NORMAL_END && r0 < k; r0 += kMaxK) {
        int kk = std::min(kMaxK, k - r0);
        r = matvec(p, dq + (size_t)r0 * p->Np, dv + (size_t)r0 * p->Np, kk, NULL);
    }
    if (r == FCG_NORMAL_END && (cudaMemcpyAsync(v, dv, n * sizeof(double), cudaMemcpyDeviceToHost, p->stream) != cudaSuccess ||
                                cudaStreamSynchronize(p->stream) != cudaSuccess)) {
        set_error(std::string("matvec failed: ") + cudaGetErrorString(cudaGetLastError()));
        r = FCG_DEVICE_ERROR;
    }
    dfree(dq);
    dfree(dv);
    return r;
}

// ------------------------------------------------------------------ GMRES

// the chunk lists of a single geometry: chunk c covers leaves
// [c * kDotChunk, min((c + 1) * kDotChunk, Np))
__global__ void k_single_geometry_chunks(int64_t Np, int64_t nch, int64_t *start, int32_t *len, int32_t *geom, int32_t *g_first,
                                         int32_t *g_count) {
    for (int64_t c = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; c < nch; c += (int64_t)gridDim.x * blockDim.x) {
        start[c] = c * kDotChunk;
        len[c] = (int32_t)min((int64_t)kDotChunk, Np - c * kDotChunk);
        geom[c] = 0;
        if (c == 0) {
            g_first[0] = 0;
            g_count[0] = (int32_t)nch;
        }
    }
}

int problem_set_geometries(DeviceProblem *p, int n, const int32_t *geom_of_cond) {
    AllocScope alloc_scope(p->stream);
    if (n < 1 || !geom_of_cond) { set_error("need at least one geometry"); return FCG_GENERIC_ERROR; }
    int nc = p->n_cond_all;
    if (nc < 1) { set_error("model has no conductors"); return FCG_GENERIC_ERROR; }
    // conductors of a geometry are contiguous, geometries numbered in order,
    // conductor leaf ranges back to back
    if (geom_of_cond[0] != 0) { set_error("the first conductor must belong to geometry 0"); return FCG_GENERIC_ERROR; }
    for (int c = 1; c < nc; c++) {
        int d = geom_of_cond[c] - geom_of_cond[c - 1];
        if (d != 0 && d != 1) { set_error("geometries must be numbered in conductor order without gaps"); return FCG_GENERIC_ERROR; }
        if (p->cond_first[c] != p->cond_first[c - 1] + p->cond_count[c - 1]) {
            set_error("conductor leaf ranges are not contiguous");
            return FCG_GENERIC_ERROR;
        }
    }
    if (geom_of_cond[nc - 1] != n - 1) { set_error("geometry count does not match the conductor map"); return FCG_GENERIC_ERROR; }
    if (p->cond_first[0] != 0 || p->cond_first[nc - 1] + p->cond_count[nc - 1] != p->Np) {
        set_error("conductor leaf ranges do not cover the panels");
        return FCG_GENERIC_ERROR;
    }
    FCG_CK(cudaSetDevice(p->ctx->device));
    int64_t Np = p->Np, Nn = p->Nn;
    std::vector<int64_t> gfirst(n, -1), gcount(n, 0);
    std::vector<int32_t> leaf_geom(n > 1 ? Np : 0);  // one geometry: all zero, set on the device
    for (int c = 0; c < nc; c++) {
        int g = geom_of_cond[c];
        if (gfirst[g] < 0) gfirst[g] = p->cond_first[c];
        gcount[g] += p->cond_count[c];
        if (n > 1)
            for (int64_t j = p->cond_first[c]; j < p->cond_first[c] + p->cond_count[c]; j++) leaf_geom[j] = g;
    }
    for (int g = 0; g < n; g++)
        if (gcount[g] == 0) { set_error("geometry " + std::to_string(g) + " has no panels"); return FCG_GENERIC_ERROR; }
    std::vector<int> cols_ptr(n + 1, 0);
    for (size_t i = 0; i < p->cond_cols.size(); i++) cols_ptr[geom_of_cond[p->cond_cols[i]] + 1]++;
    for (int g = 0; g < n; g++) cols_ptr[g + 1] += cols_ptr[g];
    // chunks of at most kDotChunk leaves inside each geometry
    std::vector<int64_t> ch_start;
    std::vector<int32_t> ch_len, ch_geom, gch_first(n), gch_count(n);
    for (int g = 0; g < n; g++) {
        gch_first[g] = (int32_t)ch_start.size();
        for (int64_t j = gfirst[g]; j < gfirst[g] + gcount[g]; j += kDotChunk) {
            ch_start.push_back(j);
            ch_len.push_back((int32_t)std::min<int64_t>(kDotChunk, gfirst[g] + gcount[g] - j));
            ch_geom.push_back(g);
        }
        gch_count[g] = (int32_t)ch_start.size() - gch_first[g];
    }
    // every node and link must stay inside one geometry: a product that
    // couples geometries would make the separate solves wrong (nothing to
    // check for a single geometry)
    cudaStream_t s = p->stream;
    int64_t tb = 0;
    int32_t *d_ng = NULL, *d_lg = NULL;
    unsigned *d_bad = NULL;
    int r = FCG_NORMAL_END;
    if (n > 1) r = upload(&d_lg, leaf_geom.data(), Np, tb, s);
    if (n > 1 && r == FCG_NORMAL_END) r = dalloc(&d_ng, Nn, tb);
    if (n > 1 && r == FCG_NORMAL_END) r = dalloc(&d_bad, 1, tb);
    unsigned bad = 0;
    if (n > 1 && r == FCG_NORMAL_END) {
        cudaMemsetAsync(d_bad, 0, sizeof(unsigned), s);
        k_node_geom<<<grid_for(Nn, 256, p->ctx->sm_count), 256, 0, s>>>(Nn, p->node_lfirst, d_lg, d_ng);
        int grid = (int)std::min<int64_t>((Nn * 32 + 255) / 256, (int64_t)p->ctx->sm_count * 32);
        k_check_geometries<<<grid, 256, 0, s>>>(Nn, p->link_ptr, p->link_src, p->parent, d_ng, d_bad);
        if (cudaGetLastError() != cudaSuccess ||
            cudaMemcpyAsync(&bad, d_bad, sizeof(unsigned), cudaMemcpyDeviceToHost, s) != cudaSuccess ||
            cudaStreamSynchronize(s) != cudaSuccess) {
            set_error("geometry check failed");
            r = FCG_DEVICE_ERROR;
        }
    }
    dfree(d_ng);
    dfree(d_lg);
    dfree(d_bad);
    if (r != FCG_NORMAL_END) return r;
    if (bad) {
        set_error(std::to_string(bad) + " tree edges or links connect different geometries");
        return FCG_GENERIC_ERROR;
    }
    dfree(p->leaf_geom); dfree(p->ch_start); dfree(p->ch_len); dfree(p->ch_geom); dfree(p->g_ch_first); dfree(p->g_ch_count);
    p->n_geom = 0;
    if (n == 1) {
        // one geometry: the leaf map and the chunk lists are made on the
        // device, so nothing here waits for the stream's earlier work
        int64_t nc1 = (int64_t)ch_start.size();
        if ((r = dalloc(&p->leaf_geom, Np, p->bytes)) || (r = dalloc(&p->ch_start, nc1, p->bytes)) ||
            (r = dalloc(&p->ch_len, nc1, p->bytes)) || (r = dalloc(&p->ch_geom, nc1, p->bytes)) ||
            (r = dalloc(&p->g_ch_first, 1, p->bytes)) || (r = dalloc(&p->g_ch_count, 1, p->bytes)))
            return r;
        FCG_CK(cudaMemsetAsync(p->leaf_geom, 0, Np * sizeof(int32_t), s));
        k_single_geometry_chunks<<<grid_for(nc1, 256, p->ctx->sm_count), 256, 0, s>>>(Np, nc1, p->ch_start, p->ch_len, p->ch_geom,
                                                                                    p->g_ch_first, p->g_ch_count);
        FCG_CK(cudaGetLastError());
    } else {
        if ((r = upload(&p->leaf_geom, leaf_geom.data(), Np, p->bytes, s)) ||
            (r = upload(&p->ch_start, ch_start.data(), ch_start.size(), p->bytes, s)) ||
            (r = upload(&p->ch_len, ch_len.data(), ch_len.size(), p->bytes, s)) ||
            (r = upload(&p->ch_geom, ch_geom.data(), ch_geom.size(), p->bytes, s)) ||
            (r = upload(&p->g_ch_first, gch_first.data(), n, p->bytes, s)) ||
            (r = upload(&p->g_ch_count, gch_count.data(), n, p->bytes, s)))
            return r;
        FCG_CK(cudaStreamSynchronize(s));
    }
    p->n_geom = n;
    p->nch = (int)ch_start.size();
    p->geom_cols_ptr = cols_ptr;
    p->geom_leaf_first = gfirst;
    p->geom_leaf_count = gcount;
    return FCG_NORMAL_END;
}

static void free_graph(DeviceProblem *p) {
    if (p->gexec) cudaGraphExecDestroy(p->gexec);
    if (p->graph) cudaGraphDestroy(p->graph);
    p->gexec = NULL;
    p->graph = NULL;
    p->gkey.clear();
}

static void free_solve_ws(DeviceProblem *p) {
    free_graph(p);
    dfree(p->d_it); dfree(p->ptmp);
    dfree(p->cs); dfree(p->sn); dfree(p->g); dfree(p->z);
    dfree(p->normb); dfree(p->hnorm); dfree(p->nrm2);
    dfree(p->active); dfree(p->iters); dfree(p->capped); dfree(p->scap); dfree(p->n_active);
    dfree(p->b); dfree(p->x0); dfree(p->w); dfree(p->vv); dfree(p->x);
    for (size_t i = 0; i < p->V.size(); i++) dfree(p->V[i]);
    p->V.clear();
    for (size_t i = 0; i < p->Hblk.size(); i++) dfree(p->Hblk[i]);
    p->Hblk.clear();
    p->Hc.clear();
    dfree(p->Vptr);
    dfree(p->Hptr);
    p->Vptr_cap = 0;
    p->gk = p->gS = p->gM = 0;
}

static int ensure_solve_ws(DeviceProblem *p, int k, int S, int M) {
    int r;
    if (p->gk != k || p->gS != S || p->gM < M) {
        free_solve_ws(p);
        int64_t &B = p->bytes;
        size_t sm = (size_t)S * (M + 2);
        if ((r = dalloc(&p->cs, sm, B)) || (r = dalloc(&p->sn, sm, B)) || (r = dalloc(&p->g, sm, B)) || (r = dalloc(&p->z, sm, B)))
            return r;
        // hnorm: the step's norms, then (mixed path) their reciprocals
        if ((r = dalloc(&p->normb, S, B)) || (r = dalloc(&p->hnorm, 2 * (size_t)S, B)) || (r = dalloc(&p->nrm2, 2 * (size_t)S, B)))
            return r;
        if ((r = dalloc(&p->active, S, B)) || (r = dalloc(&p->iters, S, B)) || (r = dalloc(&p->capped, S, B)) ||
            (r = dalloc(&p->scap, S, B)) || (r = dalloc(&p->n_active, (size_t)M + 2, B)))
            return r;
        size_t n = (size_t)k * p->Np;
        if ((r = dalloc(&p->b, n, B)) || (r = dalloc(&p->x0, n, B)) || (r = dalloc(&p->w, n, B)) || (r = dalloc(&p->vv, n, B)) ||
            (r = dalloc(&p->x, n, B)))
            return r;
        if ((r = dalloc(&p->Vptr, (size_t)M + 2, B)) || (r = dalloc(&p->Hptr, (size_t)M + 2, B))) return r;
        if ((r = dalloc(&p->d_it, 4, B))) return r;
        p->Vptr_cap = M + 2;
        p->gk = k;
        p->gS = S;
        p->gM = M;
        p->x_k = k;
    }
    return FCG_NORMAL_END;
}

// partial sums: grows with the number of basis vectors
static int ensure_partial(DeviceProblem *p, size_t need) {
    if (p->partial_cap >= need) return FCG_NORMAL_END;
    size_t cap = std::max(need, 2 * p->partial_cap);
    FCG_CK(cudaStreamSynchronize(p->stream));
    dfree(p->partial);
    p->partial_cap = 0;
    int r = dalloc(&p->partial, cap, p->bytes);
    if (r == FCG_NORMAL_END) p->partial_cap = cap;
    return r;
}

// make sure basis vector j and Hessenberg column j - 1 exist (allocated in
// groups of 16)
static int ensure_basis(DeviceProblem *p, int j) {
    const int group = 16;
    int r;
    size_t n = (size_t)p->gk * p->Np;
    while ((int)p->V.size() <= j) {
        int start = (int)p->V.size();
        int cnt = std::min(group, p->Vptr_cap - start);
        if (cnt <= 0) { set_error("Krylov basis exhausted"); return FCG_GENERIC_ERROR; }
        double *blk = NULL;
        if ((r = dalloc(&blk, n * cnt, p->bytes))) return r;
        for (int i = 0; i < cnt; i++) p->V.push_back(i == 0 ? blk : NULL);
        std::vector<double *> ptrs(cnt);
        for (int i = 0; i < cnt; i++) ptrs[i] = blk + n * i;
        FCG_CK(cudaMemcpyAsync(p->Vptr + start, ptrs.data(), cnt * sizeof(double *), cudaMemcpyHostToDevice, p->stream));
        // the copy source must outlive the transfer
        FCG_CK(cudaStreamSynchronize(p->stream));
    }
    while ((int)p->Hc.size() < j) {
        int start = (int)p->Hc.size();
        int cnt = std::min(group, p->Vptr_cap - start);
        if (cnt <= 0) { set_error("Hessenberg storage exhausted"); return FCG_GENERIC_ERROR; }
        size_t tot = 0;
        for (int i = 0; i < cnt; i++) tot += (size_t)p->gS * (start + i + 2);
        double *blk = NULL;
        if ((r = dalloc(&blk, tot, p->bytes))) return r;
        p->Hblk.push_back(blk);
        std::vector<double *> ptrs(cnt);
        size_t off = 0;
        for (int i = 0; i < cnt; i++) {
            ptrs[i] = blk + off;
            p->Hc.push_back(blk + off);
            off += (size_t)p->gS * (start + i + 2);
        }
        FCG_CK(cudaMemcpyAsync(p->Hptr + start, ptrs.data(), cnt * sizeof(double *), cudaMemcpyHostToDevice, p->stream));
        FCG_CK(cudaStreamSynchronize(p->stream));
    }
    return FCG_NORMAL_END;
}

// host-side address of basis vector j (V holds group heads; others are offsets)
static double *basis_addr(DeviceProblem *p, int j) {
    int head = j;
    while (p->V[head] == NULL) head--;
    return p->V[head] + (size_t)(j - head) * p->gk * p->Np;
}

static void free_two_level(DeviceProblem *p) {
    dfree(p->sup_index); dfree(p->sup_area); dfree(p->sup_first); dfree(p->sup_count);
    dfree(p->sup_dimv); dfree(p->sup_T); dfree(p->sup_diag); dfree(p->sup_pot); dfree(p->sup_chg);
    p->sup_m = 0;
    p->sup_kcap = 0;
    p->sup_dim = -1;
}

// Build the two-level preconditioner of dimension dim (clamped to
// [16, 4096]). Super elements: in every conductor's tree, the nodes at depth
// log2(dim / conductors) and the leaves above that depth, in leaf order. With
// at least dim conductors it is disabled (sup_m = 0) and the solve runs
// without preconditioner, as the reference does.
static int build_two_level(DeviceProblem *p, int dim) {
    if (dim <= 0) dim = 128;  // the reference's default dimension
    if (dim > 4096) dim = 4096;
    if (dim < 16) dim = 16;
    if (p->sup_dim == dim) return FCG_NORMAL_END;
    free_two_level(p);
    unsigned roots = (unsigned)p->n_cond_all;
    if (roots >= (unsigned)dim) {
        p->sup_dim = dim;
        return FCG_NORMAL_END;
    }
    int lev = (int)(unsigned)(log((double)((unsigned)dim / roots)) / log(2.0));
    cudaStream_t s = p->stream;
    int64_t Nn = p->Nn, Np = p->Np, tb = 0;
    int sms = p->ctx->sm_count;
    int r;
    // tree shape on the host: parents (device labels; a parent's label is
    // larger than its children's), first leaves, leaf flags
    std::vector<int32_t> par(Nn);
    std::vector<int64_t> lf(Nn);
    std::vector<uint8_t> leaf(Nn);
    uint8_t *d_leaf = NULL;
    if ((r = dalloc(&d_leaf, Nn, tb))) return r;
    k_node_leafflag<<<grid_for(Nn, 256, sms), 256, 0, s>>>(Nn, p->geo, d_leaf);
    if (cudaMemcpyAsync(par.data(), p->parent, Nn * sizeof(int32_t), cudaMemcpyDeviceToHost, s) != cudaSuccess ||
        cudaMemcpyAsync(lf.data(), p->node_lfirst, Nn * sizeof(int64_t), cudaMemcpyDeviceToHost, s) != cudaSuccess ||
        cudaMemcpyAsync(leaf.data(), d_leaf, Nn, cudaMemcpyDeviceToHost, s) != cudaSuccess || cudaStreamSynchronize(s) != cudaSuccess) {
        dfree(d_leaf);
        set_error("reading the tree for the two-level preconditioner failed");
        return FCG_DEVICE_ERROR;
    }
    dfree(d_leaf);
    std::vector<int32_t> depth(Nn, 0);
    int64_t nroots = 0;
    for (int64_t v = Nn - 1; v >= 0; v--) {
        if (par[v] < 0) { nroots++; continue; }
        depth[v] = depth[par[v]] + 1;
    }
    if (nroots != (int64_t)roots) {
        set_error("two-level preconditioner: every conductor must have one tree");
        return FCG_GENERIC_ERROR;
    }
    std::vector<std::pair<int64_t, int32_t>> sel;
    for (int64_t v = 0; v < Nn; v++)
        if ((leaf[v] && depth[v] <= lev) || (!leaf[v] && depth[v] == lev)) sel.push_back(std::make_pair(lf[v], (int32_t)v));
    std::sort(sel.begin(), sel.end());
    int m = (int)sel.size();
    std::vector<int32_t> elem(m);
    std::vector<int64_t> first(m), count(m);
    for (int i = 0; i < m; i++) {
        elem[i] = sel[i].second;
        first[i] = sel[i].first;
        count[i] = (i + 1 < m ? sel[i + 1].first : Np) - sel[i].first;
    }
    int32_t *d_elem = NULL, *d_piv = NULL, *d_idx = NULL;
    double *A = NULL, *X = NULL;
    unsigned *d_bad = NULL, bad = 0;
    int64_t &B = p->bytes;
    if ((r = upload(&d_elem, elem.data(), m, tb, s)) || (r = upload(&p->sup_first, first.data(), m, B, s)) ||
        (r = upload(&p->sup_count, count.data(), m, B, s)) || (r = dalloc(&p->sup_index, Np, B)) ||
        (r = dalloc(&p->sup_area, Np, B)) || (r = dalloc(&p->sup_dimv, m, B)) || (r = dalloc(&p->sup_T, (size_t)m * m, B)) ||
        (r = dalloc(&p->sup_diag, m, B)) || (r = dalloc(&A, (size_t)m * m, tb)) || (r = dalloc(&X, (size_t)m * m, tb)) ||
        (r = dalloc(&d_piv, m, tb)) || (r = dalloc(&d_idx, m, tb)) || (r = dalloc(&d_bad, 1, tb))) {
        dfree(d_elem); dfree(A); dfree(X); dfree(d_piv); dfree(d_idx); dfree(d_bad);
        free_two_level(p);
        return r;
    }
    int64_t mm = (int64_t)m * m;
    k_sup_maps<<<m, 128, 0, s>>>(m, d_elem, p->sup_first, p->sup_count, p->geo, p->leaf_node, p->sup_index, p->sup_area,
                                 p->sup_dimv);
    k_sup_matrix<<<grid_for(mm, 128, sms), 128, 0, s>>>(m, d_elem, p->sup_first, p->geo, p->leaf_eb, p->leaf_ea, A);
    for (int j = 0; j < m; j++) {
        k_lu_pivot<<<1, 1024, 0, s>>>(m, j, A, d_piv);
        if (j < m - 1) k_lu_update<<<grid_for((int64_t)(m - j - 1) * (m - j - 1), 256, sms), 256, 0, s>>>(m, j, A);
    }
    k_perm_identity<<<1, 1024, 0, s>>>(m, d_piv, d_idx, X);
    for (int i = 0; i < m - 1; i++) k_inv_forward<<<grid_for((int64_t)(m - i - 1) * m, 256, sms), 256, 0, s>>>(m, i, A, X);
    for (int i = m - 1; i >= 0; i--) {
        k_inv_scale<<<(m + 255) / 256, 256, 0, s>>>(m, i, A, X);
        if (i > 0) k_inv_backward<<<grid_for((int64_t)i * m, 256, sms), 256, 0, s>>>(m, i, A, X);
    }
    cudaMemsetAsync(d_bad, 0, sizeof(unsigned), s);
    k_inv_finish<<<grid_for(mm, 256, sms), 256, 0, s>>>(m, X, p->sup_T, p->sup_diag, d_bad);
    p->timings.launches += 4 + 2 * (int64_t)m + (m - 1) + 2 * (int64_t)m;
    cudaError_t e = cudaGetLastError();
    if (e == cudaSuccess) e = cudaMemcpyAsync(&bad, d_bad, sizeof(unsigned), cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    dfree(d_elem); dfree(A); dfree(X); dfree(d_piv); dfree(d_idx); dfree(d_bad);
    if (e != cudaSuccess) {
        free_two_level(p);
        set_error(std::string("two-level preconditioner setup failed: ") + cudaGetErrorString(e));
        return FCG_DEVICE_ERROR;
    }
    if (bad) {
        free_two_level(p);
        set_error("two-level preconditioner: the super potential matrix is singular");
        return FCG_GENERIC_ERROR;
    }
    p->sup_m = m;
    p->sup_dim = dim;
    return FCG_NORMAL_END;
}

// out = P in for k columns ([k][Np]): Jacobi (diag), two-level, or a copy
static int precond_apply(DeviceProblem *p, int kind, const double *in, double *out, int k) {
    cudaStream_t s = p->stream;
    int64_t Np = p->Np;
    int sms = p->ctx->sm_count;
    int g1 = grid_for((int64_t)k * Np, 256, sms);
    if (kind == FCG_PRECOND_TWO_LEVEL) {
        int m = p->sup_m, r;
        if (p->sup_kcap < k) {
            dfree(p->sup_pot);
            dfree(p->sup_chg);
            p->sup_kcap = 0;
            if ((r = dalloc(&p->sup_pot, (size_t)m * k, p->bytes)) || (r = dalloc(&p->sup_chg, (size_t)m * k, p->bytes))) return r;
            p->sup_kcap = k;
        }
        int gm = grid_for((int64_t)m * k, 128, sms);
        k_sup_collect<<<gm, 128, 0, s>>>(m, k, Np, p->sup_first, p->sup_count, p->sup_area, p->sup_dimv, in, p->sup_pot);
        k_sup_mult<<<gm, 128, 0, s>>>(m, k, p->sup_T, p->sup_pot, p->sup_chg);
        k_sup_spread<<<g1, 256, 0, s>>>(m, k, Np, p->sup_index, p->sup_area, p->sup_dimv, p->sup_diag, p->sup_chg, in, out);
        p->timings.launches += 3;
    } else {
        k_precond<<<g1, 256, 0, s>>>(Np, k, in, kind == FCG_PRECOND_JACOBI ? p->self : NULL, out);
        p->timings.launches++;
    }
    FCG_CK(cudaGetLastError());
    return FCG_NORMAL_END;
}

// ---- one Arnoldi step, enqueued on the problem's stream; the step index is
// read on the device (d_it[0]), so the same launches serve every step and can
// be captured once into a graph.
struct StepArgs {
    int k, S, G, M, nch, cap, pk, pair;  // pair: basis vectors as FP32 pairs
    SegChunks ch;
    const double *diag;
    double tol;
    int use_cond;
    cudaGraphConditionalHandle cond;
};

static int enqueue_step(DeviceProblem *p, const StepArgs &a) {
    cudaStream_t s = p->stream;
    int64_t Np = p->Np;
    int sms = p->ctx->sm_count, r;
    const int g1 = grid_for((int64_t)a.k * Np, 256, sms);
    const int gh = (int)std::min<int64_t>(((int64_t)a.cap * a.k * a.G * 32 + 255) / 256, (int64_t)sms * 32);
    // q_i = v / |v| (the previous step's normalisation, done by the
    // up-sweep for the Jacobi and no-preconditioner paths), w = A P q_i
    const bool fused_scale = a.pk != FCG_PRECOND_TWO_LEVEL;
    if (a.pk == FCG_PRECOND_TWO_LEVEL) {
        if ((r = precond_apply(p, a.pk, p->vv, p->ptmp, a.k)) || (r = matvec(p, p->ptmp, p->w, a.k, NULL))) return r;
    } else {
        // the mixed path multiplies by the reciprocal norms (the FP64 path divides, as the reference does)
        const bool mixed = p->precision == FCG_PREC_MIXED;
        StepScale sc = {mixed ? p->hnorm + a.S : p->hnorm, mixed ? 1 : 0, p->active, p->leaf_geom, p->Vptr, p->d_it, a.pair};
        if ((r = matvec(p, p->vv, p->w, a.k, a.diag, &sc))) return r;
    }
    // classical Gram-Schmidt against q_0..q_i, per solve. The last CTA of
    // k_dots sums the Hessenberg column (four warps, one output after the
    // other) only while that is short: at most 32 outputs (solves x the
    // basis capacity); longer columns take k_reduce_h, one warp per output
    // in parallel, the same sums.
    const bool fuse_h = (int64_t)a.S * a.cap <= 32;
    // basis vectors over grid.z while chunks x columns alone would leave
    // the GPU short of CTAs (small models: fewer than two per SM), up to
    // four CTAs per SM and at most one group of eight vectors per CTA and z
    // (4 conductors, 18.8k panels: 4.9 -> 3.5 ms per fill + solve with the
    // eight-vector passes of k_update below)
    const int dot_ctas = a.nch * a.k;
    const bool small = dot_ctas < 2 * sms;
    const int dz = !small ? 1 : std::max(1, std::min((4 * sms + dot_ctas - 1) / dot_ctas, (a.cap + 7) / 8));
    const dim3 dgrid(a.nch, a.k, dz);
    const bool pair_basis = a.pair != 0;
    if (pair_basis)
        k_dots<true><<<dgrid, kDotThreads, 0, s>>>(Np, p->d_it, p->Vptr, p->w, a.ch, a.k, p->active, p->partial, fuse_h ? 1 : 0,
                                                   a.G, p->g_ch_first, p->g_ch_count, p->Hptr, p->d_it + 3);
    else
        k_dots<false><<<dgrid, kDotThreads, 0, s>>>(Np, p->d_it, p->Vptr, p->w, a.ch, a.k, p->active, p->partial, fuse_h ? 1 : 0,
                                                    a.G, p->g_ch_first, p->g_ch_count, p->Hptr, p->d_it + 3);
    if (!fuse_h)
        k_reduce_h<<<gh, 256, 0, s>>>(a.k, a.G, a.nch, p->d_it, p->partial, p->g_ch_first, p->g_ch_count, p->active, p->Hptr);
    // v = w - sum h_j q_j; for a few solves its last CTA ends the step
    // (norms, Givens, index), for many the three kernels do
    const bool fuse_end = a.S <= 4;
    const volatile int *cancel = p->pin_dev ? p->pin_dev + 4 : NULL;
    double *rhn = p->precision == FCG_PREC_MIXED ? p->hnorm + a.S : NULL;
    StepEnd fe = {a.S, a.k, a.G, a.M, a.cap, a.use_cond, p->g_ch_first, p->g_ch_count, p->Hptr, p->cs, p->sn, p->g, p->nrm2,
                  p->hnorm, rhn, p->normb, a.tol, p->scap, p->active, p->iters, p->capped, p->n_active, p->d_it, p->d_it + 1,
                  cancel, a.cond};
    const dim3 ugrid(a.nch, a.k);
#define FCG_UPDATE(PBV, QV) \
    k_update<PBV, QV><<<ugrid, 256, 0, s>>>(Np, p->d_it, p->Vptr, p->w, p->Hptr, a.ch, a.k, p->active, p->vv, p->partial, \
                                            fuse_end ? 1 : 0, fe, p->d_it + 3)
    if (pair_basis) {
        if (small) FCG_UPDATE(true, 8);
        else FCG_UPDATE(true, 4);
    } else {
        if (small) FCG_UPDATE(false, 8);
        else FCG_UPDATE(false, 4);
    }
#undef FCG_UPDATE
    int launches = 3 + (fuse_h ? 0 : 1);
    if (!fuse_end) {
        const int g1v = (int)(((int64_t)a.k * a.G * 32 + 255) / 256);
        k_reduce_seg<<<g1v, 256, 0, s>>>(1, a.k, a.G, a.nch, p->partial, p->g_ch_first, p->g_ch_count, p->active, p->nrm2, 1, 0);
        k_givens_warp<<<(a.S * 32 + 127) / 128, 128, 0, s>>>(a.S, p->d_it, a.M, p->Hptr, p->cs, p->sn, p->g, p->normb, p->nrm2,
                                                              p->hnorm, rhn, a.tol,
                                    p->scap, p->active, p->iters, p->capped, p->n_active);
        k_iter_advance<<<1, 32, 0, s>>>(p->d_it, p->n_active, a.cap, cancel, p->d_it + 1, a.cond, a.use_cond);
        launches += 3;
    }
    if (!fused_scale) {
        // the two-level path normalises here (its preconditioner reads v first);
        // k_update's step end has already advanced the index, hence Vp[*iter]
        if (pair_basis) k_scale<true><<<g1, 256, 0, s>>>(Np, a.k, p->vv, p->hnorm, p->active, p->leaf_geom, NULL, p->Vptr, p->d_it, 0);
        else k_scale<false><<<g1, 256, 0, s>>>(Np, a.k, p->vv, p->hnorm, p->active, p->leaf_geom, NULL, p->Vptr, p->d_it, 0);
        launches++;
    }
    p->timings.launches += launches;
    FCG_CK(cudaGetLastError());
    return FCG_NORMAL_END;
}

// Build (or reuse) the graph "while (go) { one Arnoldi step }". Everything a
// step reads is in a key; the graph is rebuilt only when the key changes.
static int ensure_step_graph(DeviceProblem *p, StepArgs a) {
    std::vector<unsigned char> key;
    auto put = [&](const void *x, size_t n) { key.insert(key.end(), (const unsigned char *)x, (const unsigned char *)x + n); };
    put(&a.k, sizeof(int) * 8);
    put(&a.ch, sizeof(a.ch));
    put(&a.diag, sizeof(a.diag));
    put(&a.tol, sizeof(a.tol));
    const void *ptrs[] = {p->w, p->vv, p->ptmp, p->partial, p->Vptr, p->Hptr, p->n_active, p->cs, p->sn, p->g, p->normb, p->nrm2,
                          p->hnorm, p->scap, p->active, p->iters, p->capped, p->leaf_geom, p->g_ch_first, p->g_ch_count, p->Qd,
                          p->row_split,
                          p->Qf, p->Pd, p->Pf2, p->Ad, p->sup_T, p->sup_pot, p->sup_chg, p->d_it, p->pin_dev};
    put(ptrs, sizeof(ptrs));
    int ints[] = {p->kcap, p->sup_m, p->sup_kcap, p->spmv_lanes, p->n_row_split, p->profiling ? 1 : 0};
    put(ints, sizeof(ints));
    if (p->gexec && key == p->gkey) return FCG_NORMAL_END;
    free_graph(p);
    cudaGraph_t g = NULL, body = NULL;
    cudaGraphExec_t ge = NULL;
    cudaGraphConditionalHandle h;
    cudaGraphNode_t node;
    cudaGraphNodeParams cp = {};
    cudaError_t e = cudaGraphCreate(&g, 0);
    if (e == cudaSuccess) e = cudaGraphConditionalHandleCreate(&h, g, 1, cudaGraphCondAssignDefault);
    if (e == cudaSuccess) {
        cp.type = cudaGraphNodeTypeConditional;
        cp.conditional.handle = h;
        cp.conditional.type = cudaGraphCondTypeWhile;
        cp.conditional.size = 1;
        e = cudaGraphAddNode(&node, g, NULL, NULL, 0, &cp);
    }
    if (e == cudaSuccess) {
        body = cp.conditional.phGraph_out[0];
        e = cudaStreamBeginCaptureToGraph(p->stream, body, NULL, NULL, 0, cudaStreamCaptureModeThreadLocal);
    }
    if (e != cudaSuccess) {
        cudaGetLastError();
        if (g) cudaGraphDestroy(g);
        set_error(std::string("cannot build the Arnoldi graph: ") + cudaGetErrorString(e));
        return FCG_DEVICE_ERROR;
    }
    // launches made while capturing are not runs: keep the counters as they were
    SolveTimings saved = p->timings;
    a.use_cond = 1;
    a.cond = h;
    int r = enqueue_step(p, a);
    SolveTimings after = p->timings;
    p->timings = saved;
    cudaGraph_t got = NULL;
    e = cudaStreamEndCapture(p->stream, &got);
    if (r == FCG_NORMAL_END && e == cudaSuccess) e = cudaGraphInstantiate(&ge, g, 0);
    if (r != FCG_NORMAL_END || e != cudaSuccess) {
        cudaGetLastError();
        cudaGraphDestroy(g);
        if (r == FCG_NORMAL_END) {
            set_error(std::string("cannot build the Arnoldi graph: ") + cudaGetErrorString(e));
            r = FCG_DEVICE_ERROR;
        }
        return r;
    }
    p->graph = g;
    p->gexec = ge;
    p->gkey = key;
    p->g_launches = (int)(after.launches - saved.launches);
    p->g_link_launches = (int)(after.link_launches - saved.link_launches);
    p->g_link_bytes = after.link_bytes - saved.link_bytes;
    return FCG_NORMAL_END;
}

int problem_solve(DeviceProblem *p, const fcg_solve_options &opt, double *cap, int *iterations, double *all_charges) {
    AllocScope alloc_scope(p->stream);
    if (!p->filled) { set_error("coefficients not filled"); return FCG_GENERIC_ERROR; }
    FCG_CK(cudaSetDevice(p->ctx->device));
    int r;
    if (p->cond_cols.empty()) { set_error("no conductors to solve for"); return FCG_GENERIC_ERROR; }
    if (p->n_geom == 0) {
        std::vector<int32_t> one(p->n_cond_all, 0);
        if ((r = problem_set_geometries(p, 1, one.data()))) return r;
    }
    const int G = p->n_geom;
    const int64_t Np = p->Np;
    const int nch = p->nch;
    if (all_charges && G != 1) { set_error("charge vectors are kept for one geometry only"); return FCG_GENERIC_ERROR; }
    if (opt.krylov != FCG_KRYLOV_PAIR && opt.krylov != FCG_KRYLOV_FP64) {
        set_error("unknown Krylov basis arithmetic " + std::to_string(opt.krylov));
        return FCG_GENERIC_ERROR;
    }
    // the mixed path's Krylov basis as FP32 pairs (FCG_KRYLOV_PAIR): same
    // 8 bytes per element, the Arnoldi kernels on the FP32 pipe
    const bool pair_basis = p->precision == FCG_PREC_MIXED && opt.krylov == FCG_KRYLOV_PAIR;
    // per geometry: columns, output offsets, iteration cap (the reference's
    // min(1000, panels) for the geometry alone)
    std::vector<int> ncol(G);
    std::vector<int64_t> cap_off(G + 1, 0), it_off(G + 1, 0);
    std::vector<int> gcap(G);
    int ks = 0, M = 1;
    for (int g = 0; g < G; g++) {
        ncol[g] = p->geom_cols_ptr[g + 1] - p->geom_cols_ptr[g];
        ks = std::max(ks, ncol[g]);
        cap_off[g + 1] = cap_off[g] + (int64_t)ncol[g] * ncol[g];
        it_off[g + 1] = it_off[g] + ncol[g];
        int64_t c = opt.max_iter > 0 ? opt.max_iter : 1000;
        c = std::min<int64_t>(c, p->geom_leaf_count[g]);
        gcap[g] = (int)std::max<int64_t>(c, 1);
        M = std::max(M, gcap[g]);
    }
    // preconditioner: Jacobi is fused into the product's up-sweep; the
    // two-level one is applied before it (and falls back to none when there
    // are at least as many conductors as its dimension, as in the reference)
    int pk = opt.precond;
    if (pk != FCG_PRECOND_NONE && pk != FCG_PRECOND_JACOBI && pk != FCG_PRECOND_TWO_LEVEL) {
        set_error("unknown preconditioner");
        return FCG_GENERIC_ERROR;
    }
    if (pk == FCG_PRECOND_TWO_LEVEL) {
        if ((r = build_two_level(p, opt.precond_dim))) return r;
        if (p->sup_m == 0) pk = FCG_PRECOND_NONE;
    }
    const double *diag = (pk == FCG_PRECOND_JACOBI) ? p->self : NULL;
    const bool pre = pk != FCG_PRECOND_NONE;
    if (p->pin) ((volatile int *)p->pin)[4] = p->cancel.load() ? 1 : 0;
    cudaStream_t s = p->stream;
    int sms = p->ctx->sm_count;
    SegChunks chunks = {p->ch_start, p->ch_len, p->ch_geom, nch};
    double *d_cap = NULL;
    int64_t tmpb = 0;
    if ((r = dalloc(&d_cap, (size_t)std::max<int64_t>(cap_off[G], 1), tmpb))) return r;
    std::vector<int> h_iters(it_off[G], 0);
    p->timings.iterations_max = 0;
    int status = FCG_NORMAL_END;
    bool any_capped = false;
    float solve_ms_total = 0;
    // columns in batches of at most `width`: batch column r of geometry g is the
    // solve for the geometry's conductor r0 + r
    int width = opt.rhs_width > 0 ? std::min(opt.rhs_width, kMaxK) : kMaxK;
    if (opt.rhs_width == 0 && (r = choose_rhs_width(p, ks, &width)) != FCG_NORMAL_END) return r;
    p->timings.rhs_width = std::min(width, ks);
    for (int r0 = 0; r0 < ks && status == FCG_NORMAL_END; r0 += width) {
        if (p->cancel.load()) { set_error("solve cancelled"); status = FCG_USER_BREAK; break; }
        const int k = std::min(width, ks - r0);
        const int S = G * k;
        std::vector<int64_t> sf(S, 0), sc(S, 0);
        std::vector<int> scap(S);
        std::vector<int32_t> e_slot;
        std::vector<int64_t> e_first, e_count, e_out;
        int64_t maxcount = 1;
        for (int g = 0; g < G; g++) {
            const int *cols = p->cond_cols.data() + p->geom_cols_ptr[g];
            for (int rr = 0; rr < k; rr++) {
                int sidx = g * k + rr;
                scap[sidx] = gcap[g];
                if (r0 + rr >= ncol[g]) continue;
                sf[sidx] = p->cond_first[cols[r0 + rr]];
                sc[sidx] = p->cond_count[cols[r0 + rr]];
                for (int c = 0; c < ncol[g]; c++) {
                    e_slot.push_back(rr);
                    e_first.push_back(p->cond_first[cols[c]]);
                    e_count.push_back(p->cond_count[cols[c]]);
                    e_out.push_back(cap_off[g] + (int64_t)(r0 + rr) * ncol[g] + c);
                    maxcount = std::max(maxcount, p->cond_count[cols[c]]);
                }
            }
        }
        const int nentry = (int)e_slot.size();
        const int nslice = (int)((maxcount + kAsmChunk - 1) / kAsmChunk);
        int64_t *d_sf = NULL, *d_sc = NULL, *d_ef = NULL, *d_ec = NULL, *d_eo = NULL;
        int32_t *d_es = NULL;
        double *d_part = NULL;
        int64_t bb = 0;
        auto free_batch = [&]() {
            cudaStreamSynchronize(s);
            dfree(d_sf); dfree(d_sc); dfree(d_ef); dfree(d_ec); dfree(d_eo); dfree(d_es); dfree(d_part);
        };
        if ((r = ensure_solve_ws(p, k, S, M)) || (r = ensure_partial(p, (size_t)2 * k * nch)) ||
            (r = upload(&d_sf, sf.data(), S, bb, s)) || (r = upload(&d_sc, sc.data(), S, bb, s)) ||
            (r = upload(&d_es, e_slot.data(), nentry, bb, s)) || (r = upload(&d_ef, e_first.data(), nentry, bb, s)) ||
            (r = upload(&d_ec, e_count.data(), nentry, bb, s)) || (r = upload(&d_eo, e_out.data(), nentry, bb, s)) ||
            (r = dalloc(&d_part, (size_t)nentry * nslice, bb))) {
            free_batch();
            status = r;
            break;
        }
        FCG_CK(cudaMemcpyAsync(p->scap, scap.data(), S * sizeof(int), cudaMemcpyHostToDevice, s));
        const int64_t n = (int64_t)k * Np;
        const int g1 = grid_for(n, 256, sms);
        const int gs = (S + 127) / 128;
        auto seg_grid = [&](int nvec) { return (int)(((int64_t)nvec * k * G * 32 + 255) / 256); };
        if ((r = ensure_basis(p, 0))) { free_batch(); status = r; break; }
        cudaEventRecord(p->ev0, s);
        k_set_rhs<<<g1, 256, 0, s>>>(Np, k, p->leaf_geom, d_sf, d_sc, p->b);
        double *V0 = basis_addr(p, 0);
        // GMRES from x0 = P b (or 0), then, for the mixed path, up to `cycles`
        // restarts from the current x while the true residual b - A x (not
        // the recurrence's estimate) is at or above the tolerance
        const int cycles = opt.refine < 0 ? 0 : (opt.refine > 0 ? opt.refine : (p->precision == FCG_PREC_MIXED ? 2 : 0));
        if (pre) {
            if ((r = precond_apply(p, pk, p->b, p->x0, k)) || (r = matvec(p, p->x0, p->w, k, NULL))) {
                free_batch();
                status = r;
                break;
            }
            k_residual<<<dim3(nch, k), 256, 0, s>>>(Np, p->b, p->w, chunks, p->vv, p->partial, p->partial + (size_t)k * nch);
        } else {
            FCG_CK(cudaMemsetAsync(p->x0, 0, n * sizeof(double), s));
            k_residual<<<dim3(nch, k), 256, 0, s>>>(Np, p->b, NULL, chunks, p->vv, p->partial, p->partial + (size_t)k * nch);
        }
        std::vector<int> it_total(S, 0);
        bool notconv = false;
        int *pin = p->pin ? p->pin : p->pin_local;
        for (int cycle = 0; status == FCG_NORMAL_END; cycle++) {
            double *pr = p->partial, *pb = p->partial + (size_t)k * nch;
            k_reduce_seg<<<seg_grid(1), 256, 0, s>>>(1, k, G, nch, pr, p->g_ch_first, p->g_ch_count, NULL, p->nrm2, 1, 0);
            k_reduce_seg<<<seg_grid(1), 256, 0, s>>>(1, k, G, nch, pb, p->g_ch_first, p->g_ch_count, NULL, p->nrm2 + S, 1, 0);
            FCG_CK(cudaMemsetAsync(p->g, 0, (size_t)S * (M + 2) * sizeof(double), s));
            FCG_CK(cudaMemsetAsync(p->n_active, 0, (size_t)(M + 2) * sizeof(int), s));
            k_init_state<<<gs, 128, 0, s>>>(S, M, p->nrm2, p->nrm2 + S, p->normb, p->g, p->hnorm, opt.tol, p->active, p->iters,
                                            p->capped, p->n_active + M + 1);
            if (pair_basis) k_scale<true><<<g1, 256, 0, s>>>(Np, k, p->vv, p->hnorm, NULL, p->leaf_geom, V0, NULL, NULL, 0);
            else k_scale<false><<<g1, 256, 0, s>>>(Np, k, p->vv, p->hnorm, NULL, p->leaf_geom, V0, NULL, NULL, 0);
            FCG_CK(cudaGetLastError());
            p->timings.launches += 7;
            // does any solve need an Arnoldi step? (read below, after the
            // host has prepared the steps while the device works)
            FCG_CK(cudaMemcpyAsync(pin, p->n_active + M + 1, sizeof(int), cudaMemcpyDeviceToHost, s));
            FCG_CK(cudaMemsetAsync(p->d_it, 0, 4 * sizeof(int), s));
            if (pk == FCG_PRECOND_TWO_LEVEL && !p->ptmp && (r = dalloc(&p->ptmp, (size_t)k * Np, p->bytes))) {
                status = r;
                break;
            }
            StepArgs sa = {k, S, G, M, nch, M, pk, pair_basis ? 1 : 0, chunks, diag, opt.tol, 0, 0};
            // the workspace a step touches exists before any capture
            if ((r = ensure_matvec_ws(p, kpad(k))) || (r = autotune(p, kpad(k))) ||
                (pk == FCG_PRECOND_TWO_LEVEL && (r = precond_apply(p, pk, p->vv, p->ptmp, k)))) {
                status = r;
                break;
            }
            const bool use_graph = !p->profiling && getenv("FCG_NO_GRAPH") == NULL;
            if (use_graph) {
                // the first graph launch's basis and graph (a new problem
                // captures and instantiates it here, overlapping the device)
                sa.cap = std::min(M, 32);
                if ((r = ensure_basis(p, sa.cap)) || (r = ensure_partial(p, (size_t)k * sa.cap * nch)) || (r = ensure_step_graph(p, sa))) {
                    status = r;
                    break;
                }
            }
            FCG_CK(cudaStreamSynchronize(s));
            bool any = pin[0] > 0;
            int steps = 0;  // Arnoldi steps taken
            while (any && status == FCG_NORMAL_END) {
                if (use_graph) {
                    // the whole loop in one graph launch, up to the basis capacity
                    int capv = std::min(M, std::max(32, 2 * steps));
                    sa.cap = capv;
                    if ((r = ensure_basis(p, capv)) || (r = ensure_partial(p, (size_t)k * capv * nch)) || (r = ensure_step_graph(p, sa))) {
                        status = r;
                        break;
                    }
                    FCG_CK(cudaGraphLaunch(p->gexec, s));
                    FCG_CK(cudaMemcpyAsync(pin, p->d_it, 3 * sizeof(int), cudaMemcpyDeviceToHost, s));
                    FCG_CK(cudaStreamSynchronize(s));
                    int ran = pin[0] - steps;
                    p->timings.launches += (int64_t)ran * p->g_launches;
                    p->timings.link_launches += (int64_t)ran * p->g_link_launches;
                    p->timings.link_bytes += (int64_t)ran * p->g_link_bytes;
                    p->timings.matvecs += ran;
                    steps = pin[0];
                    // stopped with solves still active: the basis is full (grow it) or a cancel
                    any = pin[2] > 0 && steps < M;
                } else {
                    sa.cap = M;
                    if ((r = ensure_basis(p, steps + 1)) || (r = ensure_partial(p, (size_t)k * (steps + 1) * nch)) ||
                        (r = enqueue_step(p, sa))) {
                        status = r;
                        break;
                    }
                    FCG_CK(cudaMemcpyAsync(pin, p->d_it, 3 * sizeof(int), cudaMemcpyDeviceToHost, s));
                    FCG_CK(cudaStreamSynchronize(s));
                    prof_collect(p);
                    steps = pin[0];
                    any = pin[1] != 0;
                }
                if (p->cancel.load()) { set_error("solve cancelled"); status = FCG_USER_BREAK; break; }
            }
            if (status != FCG_NORMAL_END) break;
            k_backsub<<<(S * 32 + 127) / 128, 128, 0, s>>>(S, M, p->Hptr, p->g, p->iters, p->z);
            if (pair_basis) k_combine<true><<<g1, 256, 0, s>>>(Np, k, M, p->Vptr, p->z, p->iters, p->leaf_geom, p->w);
            else k_combine<false><<<g1, 256, 0, s>>>(Np, k, M, p->Vptr, p->z, p->iters, p->leaf_geom, p->w);
            if (pk == FCG_PRECOND_TWO_LEVEL) {
                if ((r = precond_apply(p, pk, p->w, p->vv, k))) { status = r; break; }
                k_finish<<<g1, 256, 0, s>>>(Np, k, p->x0, p->vv, NULL, p->iters, p->leaf_geom, p->x);
            } else {
                k_finish<<<g1, 256, 0, s>>>(Np, k, p->x0, p->w, diag, p->iters, p->leaf_geom, p->x);
            }
            p->timings.launches += 3;
            {
                std::vector<int> hb(2 * (size_t)S);
                FCG_CK(cudaMemcpyAsync(hb.data(), p->iters, S * sizeof(int), cudaMemcpyDeviceToHost, s));
                FCG_CK(cudaMemcpyAsync(hb.data() + S, p->capped, S * sizeof(int), cudaMemcpyDeviceToHost, s));
                FCG_CK(cudaStreamSynchronize(s));
                // a later cycle that converges clears an earlier cap
                notconv = false;
                for (int q = 0; q < S; q++) {
                    it_total[q] += hb[q] + 1;
                    notconv |= hb[S + q] != 0;
                }
            }
            if (cycle >= cycles) break;
            // true residual of x: r = b - A x, in vv and the chunk partials
            if ((r = matvec(p, p->x, p->w, k, NULL))) { status = r; break; }
            pr = p->partial;
            pb = p->partial + (size_t)k * nch;
            k_residual<<<dim3(nch, k), 256, 0, s>>>(Np, p->b, p->w, chunks, p->vv, pr, pb);
            k_reduce_seg<<<seg_grid(1), 256, 0, s>>>(1, k, G, nch, pr, p->g_ch_first, p->g_ch_count, NULL, p->nrm2, 1, 0);
            k_reduce_seg<<<seg_grid(1), 256, 0, s>>>(1, k, G, nch, pb, p->g_ch_first, p->g_ch_count, NULL, p->nrm2 + S, 1, 0);
            FCG_CK(cudaMemsetAsync(p->n_active + M + 1, 0, sizeof(int), s));
            k_refine_count<<<gs, 128, 0, s>>>(S, p->nrm2, p->nrm2 + S, opt.tol, p->n_active + M + 1);
            p->timings.launches += 4;
            FCG_CK(cudaMemcpyAsync(pin, p->n_active + M + 1, sizeof(int), cudaMemcpyDeviceToHost, s));
            FCG_CK(cudaStreamSynchronize(s));
            p->timings.refine_checks++;
            if (pin[0] == 0) break;
            // restart from x: x0 = x, the residual is already in vv
            p->timings.refine_cycles++;
            FCG_CK(cudaMemcpyAsync(p->x0, p->x, n * sizeof(double), cudaMemcpyDeviceToDevice, s));
        }
        if (status != FCG_NORMAL_END) { free_batch(); break; }
        cudaEventRecord(p->ev1, s);
        if (nentry > 0) {
            k_assemble_part<<<dim3(nentry, nslice), 256, 0, s>>>(Np, d_es, d_ef, d_ec, p->leaf_weight, p->x, d_part);
            k_assemble_sum<<<(nentry + 127) / 128, 128, 0, s>>>(nentry, nslice, d_part, d_eo, d_cap);
        }
        FCG_CK(cudaGetLastError());
        p->timings.launches += nentry > 0 ? 2 : 0;
        FCG_CK(cudaStreamSynchronize(s));
        prof_collect(p);
        float ms = 0;
        cudaEventElapsedTime(&ms, p->ev0, p->ev1);
        solve_ms_total += ms;
        if (all_charges)
            for (int rr = 0; rr < k && r0 + rr < ncol[0]; rr++)
                FCG_CK(cudaMemcpy(all_charges + (size_t)(r0 + rr) * Np, p->x + (size_t)rr * Np, (size_t)Np * sizeof(double),
                                  cudaMemcpyDeviceToHost));
        for (int g = 0; g < G; g++)
            for (int rr = 0; rr < k && r0 + rr < ncol[g]; rr++) {
                int sidx = g * k + rr, it = it_total[sidx];
                h_iters[it_off[g] + r0 + rr] = it;
                p->timings.iterations_max = std::max(p->timings.iterations_max, it);
            }
        free_batch();
        any_capped |= notconv;
    }
    if (status == FCG_NORMAL_END && any_capped) status = FCG_NOT_CONVERGED;
    if (status == FCG_NORMAL_END || status == FCG_NOT_CONVERGED) {
        if (cap && cap_off[G] > 0 &&
            (cudaMemcpyAsync(cap, d_cap, (size_t)cap_off[G] * sizeof(double), cudaMemcpyDeviceToHost, s) != cudaSuccess ||
             cudaStreamSynchronize(s) != cudaSuccess)) {
            set_error("copy of the capacitance matrix failed");
            status = FCG_DEVICE_ERROR;
        } else if (iterations) {
            memcpy(iterations, h_iters.data(), h_iters.size() * sizeof(int));
        }
    }
    p->timings.solve_ms = solve_ms_total;
    p->timings.assemble_ms = 0;
    dfree(d_cap);
    return status;
}

int problem_get_charges(DeviceProblem *p, double *charges) {
    if (!p->x) { set_error("no solve has run"); return FCG_GENERIC_ERROR; }
    FCG_CK(cudaSetDevice(p->ctx->device));
    FCG_CK(cudaMemcpyAsync(charges, p->x, (size_t)p->x_k * p->Np * sizeof(double), cudaMemcpyDeviceToHost, p->stream));
    FCG_CK(cudaStreamSynchronize(p->stream));
    return FCG_NORMAL_END;
}

// ------------------------------------------------------ no-allocation matvec
//
// Some callers cannot allocate device memory at the point where they need a
// product: hosts that reserve all device memory at start-up and forbid
// allocation afterwards (a simulator that has sized its memory pool to the
// whole GPU), or hosts whose device memory belongs to another allocator that
// would not see, and could not account for, a cudaMalloc made behind its
// back. For them, problem_matvec_noalloc runs the same kernels as
// problem_matvec_device with the node work arrays (charges, potentials,
// ancestor sums) placed in this fixed, file-scope device array instead of the
// problem's lazily allocated workspace. Every GPU that loads the library holds
// the array until the process exits. All calls share it, and it keeps the
// previous call's contents: calls that overlap on the GPU (different streams,
// different problems) race on it and must be serialised by the caller.
static const size_t kNoAllocScratchBytes = (size_t)32 << 20;  // 32 MiB per device
static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocScratchBytes];

static const int kMaxDevices = 64;
static void *g_noalloc_addr[kMaxDevices];
static std::mutex g_noalloc_mutex;

// Resolve the device address of the scratch array for the current device
// (once per device; the first call on a device should come before any stream
// capture).
static int noalloc_scratch(int device, unsigned char **out) {
    if (device < 0 || device >= kMaxDevices) { set_error("device index out of range"); return FCG_DEVICE_ERROR; }
    std::lock_guard<std::mutex> lock(g_noalloc_mutex);
    if (!g_noalloc_addr[device]) {
        void *ptr = NULL;
        cudaError_t e = cudaGetSymbolAddress(&ptr, g_noalloc_scratch);
        if (e != cudaSuccess || !ptr) {
            set_error(std::string("cudaGetSymbolAddress of the no-allocation scratch failed: ") + cudaGetErrorString(e));
            return FCG_DEVICE_ERROR;
        }
        g_noalloc_addr[device] = ptr;
    }
    *out = (unsigned char *)g_noalloc_addr[device];
    return FCG_NORMAL_END;
}

static size_t align256(size_t n) { return (n + 255) & ~(size_t)255; }

// bytes of scratch a product with kp padded right-hand sides needs
static size_t noalloc_need(const DeviceProblem *p, int kp) {
    size_t n = (size_t)p->Nn * kp;
    size_t need = 3 * align256(n * sizeof(double));
    if (p->precision == FCG_PREC_MIXED) need += align256(n * sizeof(float));
    return need;
}

int problem_matvec_noalloc(DeviceProblem *p, const double *d_q, double *d_v, int k) {
    if (!p->filled) { set_error("coefficients not filled"); return FCG_GENERIC_ERROR; }
    if (k < 1 || k > kMaxK) { set_error("right-hand sides per matvec must be in [1, 32]"); return FCG_GENERIC_ERROR; }
    int kp = kpad(k);
    size_t need = noalloc_need(p, kp);
    if (need > kNoAllocScratchBytes) {
        set_error("no-allocation matvec: the model needs " + std::to_string(need) + " bytes of node scratch for " +
                  std::to_string(k) + " right-hand side(s), more than the fixed " + std::to_string(kNoAllocScratchBytes) +
                  "-byte array; use fcg_problem_matvec_device or fewer right-hand sides");
        return FCG_OUT_OF_MEMORY;
    }
    FCG_CK(cudaSetDevice(p->ctx->device));
    unsigned char *base = NULL;
    int r = noalloc_scratch(p->ctx->device, &base);
    if (r != FCG_NORMAL_END) return r;
    size_t n = (size_t)p->Nn * kp;
    NodeWork w;
    w.Qd = (double *)base;
    w.Pd = (double *)(base + align256(n * sizeof(double)));
    w.Pf2 = (float2 *)w.Pd;  // the FP64 and mixed potential arrays share the slot (8 bytes per value)
    w.Ad = (double *)(base + 2 * align256(n * sizeof(double)));
    w.Qf = (float *)(base + 3 * align256(n * sizeof(double)));
    cudaStream_t s = p->stream;
    // The link product reads the padding columns k..kp-1 of the charges,
    // which the up-sweep never writes, and the array still holds whatever the
    // last call (any problem, any precision) left there: bits that may not
    // even be a finite number. Columns never mix, so they could not reach the
    // result, but they are cleared anyway so that every value the kernels
    // read is a finite charge (a memset allocates nothing).
    if (kp > k) {
        FCG_CK(cudaMemsetAsync(w.Qd, 0, n * sizeof(double), s));
        if (p->precision == FCG_PREC_MIXED) FCG_CK(cudaMemsetAsync(w.Qf, 0, n * sizeof(float), s));
    }
    // while the caller records a graph on this stream the launches go into
    // the graph: no wait (it would end the recording) and no profiling
    // events (they would time nothing)
    cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
    FCG_CK(cudaStreamIsCapturing(s, &cs));
    const bool recording = cs != cudaStreamCaptureStatusNone;
    const bool profiling = p->profiling;
    if (recording) p->profiling = false;
    r = launch_matvec(p, w, d_q, d_v, k, kp, NULL);
    p->profiling = profiling;
    if (r != FCG_NORMAL_END || recording) return r;
    FCG_CK(cudaStreamSynchronize(s));
    prof_collect(p);  // with profiling on, read back (and release) the link-product events
    return FCG_NORMAL_END;
}

}  // namespace fcg
