// Adaptive mesh refinement on the GPU: CAutoRefine::DiscretizeMutual /
// DiscretizeSelf (Solver/Autorefine.cpp:2638-2795) with CAutoPanel::Subdivide
// (Solver/AutoPanel.cpp:382-523).
//
// The refined mesh does not depend on the order in which element pairs are
// examined. A pair's test (fcg_mesh_decision) reads only the two elements'
// own geometry, never whether they already have children, and a split
// always bisects the same element the same way (fcg_subdivide) and only once.
// So the mesh is the closure of: refine every conductor pair from the two
// conductors' top elements (`selfc` off); refine the two children of every
// internal element, including every element split along the way (`selfc`
// on). The host builder reaches that closure depth first; here the pairs
// advance one level per step:
//   decide   every frontier pair in FP64 (the host builder's own code);
//            non-split pairs update the largest achieved weight, split pairs
//            mark a leaf to bisect
//   number   the marked leaves by an exclusive scan (deterministic ids)
//   bisect   the marked leaves; each new internal element adds the pair of
//            its children, with `selfc`, to the next frontier
//   expand   every split pair into its two children pairs.
// The element ids differ from the host builder's (creation order), but the
// tree, and so the flattened model, is the same. Recursion levels are those
// of the host recursion: a conductor pair starts at level 1, the self pair of
// an element at depth s of its conductor's tree at level s + 2.
//
// Compiled with -fmad=false so that every decision and every bisection
// rounds the way the host builder (-ffp-contract=off) does.
#include <cuda_runtime.h>

#include <stdio.h>
#include <stdlib.h>

#include <algorithm>
#include <string>
#include <vector>

#include "fc_potential.h"
#include "pair32.cuh"
#include "fcg_internal.hpp"
#include "scan.cuh"
#include "../host/model.hpp"

namespace fcg {

using namespace devscan;

namespace {

constexpr int kMaxMeshLevel = 4096;           // the host recursion's limit
constexpr uint16_t kSelfBit = kMeshSelfPair;  // frontier meta: self pass
constexpr uint16_t kLevelMask = 0x7fff;       // frontier meta: recursion level
constexpr int64_t kMaxFrontier = 1ll << 30;   // pairs held at once

static_assert(sizeof(Element) == 96, "element record layout");

// ---- FP32 pre-test of the mesh decision (fcg_mesh_decision), see pair32.cuh

// geometric normal (fcg_geo_normal) in FP32 and a bound on each component's
// distance to the FP64 path's value; false when a super node's Newell modulus
// is within rounding of the normalisation cut-off
__device__ __forceinline__ bool geo_normal32(const Element &e, float &x, float &y, float &z, float &err) {
    if (!(e.type & FCG_IS_SUPER_NODE)) {
        x = e.n[0]; y = e.n[1]; z = e.n[2];
        err = 0.0f;
        return true;
    }
    float n[3];
    n[0] = n[1] = n[2] = 0.0f;
    for (int i = 0; i < 3; i++) {  // the float sums of fcg_newell_normal, same operations
        int j = i + 1 > 2 ? 0 : i + 1;
        const float *a = e.v + 3 * i, *b = e.v + 3 * j;
        n[0] += (a[1] - b[1]) * (a[2] + b[2]);
        n[1] += (a[2] - b[2]) * (a[0] + b[0]);
        n[2] += (a[0] - b[0]) * (a[1] + b[1]);
    }
    float m = sqrtf(n[0] * n[0] + n[1] * n[1] + n[2] * n[2]);
    const float cut = (float)FCG_PANEL_EPS;
    if (!(fabsf(m - cut) > 1e-5f * cut)) return false;
    if (m > cut) {
        x = n[0] / m; y = n[1] / m; z = n[2] / m;
        err = 16.0f * pair32::kU;  // unit components: a few roundings each
    } else {
        x = n[0]; y = n[1]; z = n[2];
        err = 0.0f;  // the same float sums, unnormalised
    }
    return true;
}

// fcg_mesh_decision in FP32: 1 / 2 refine (split the larger-area element),
// 0 no refinement (c1, c2 and their bounds e1, e2 are the pair's weights),
// -1 only the FP64 test can tell
__device__ int mesh_decide32(const Element &A, const Element &B, bool selfc, float e, float mesh_curv, float inv_max_area,
                             float inv_max_side, float &c1, float &e1, float &c2, float &e2) {
    using namespace pair32;
    float dx = A.c[0] - B.c[0], dy = A.c[1] - B.c[1], dz = A.c[2] - B.c[2];  // fcg_fsub's float values
    float r = sqrtf(dx * dx + dy * dy + dz * dz);
    double rm = A.maxside > B.maxside ? A.maxside : B.maxside;
    float rho = r / (float)rm;
    if (!(r > 1e-10f) || !(fabsf(rho - 2.0f) > 1e-5f)) return -1;
    bool quad = rho < 2.0f;
    float cc = 1.0f, cc_err = 0.0f;
    if (selfc) {
        float ax, ay, az, ae, bx, by, bz, be;
        if (!geo_normal32(A, ax, ay, az, ae) || !geo_normal32(B, bx, by, bz, be)) return -1;
        float na = fabsf(ax) + fabsf(ay) + fabsf(az), nb = fabsf(bx) + fabsf(by) + fabsf(bz);
        float dot = ax * bx + ay * by + az * bz;
        float dot_err = ae * nb + be * na + 8.0f * kU * (na * nb);
        cc = (mesh_curv - 1.0f) * (dot + 1.0f) + 1.0f;
        cc_err = (mesh_curv - 1.0f) * dot_err + 8.0f * kU * fabsf(cc) + 8.0f * kU * fabsf(mesh_curv - 1.0f) * (fabsf(dot) + 1.0f);
        if (!(cc - cc_err > 0.0f)) return -1;
    }
    float w1, w1e, w2, w2e;
    if (!weight32(A, B, dx, dy, dz, r, quad, inv_max_area, inv_max_side, w1, w1e)) return -1;
    if (!weight32(B, A, -dx, -dy, -dz, r, quad, inv_max_area, inv_max_side, w2, w2e)) return -1;
    // c = w / cc with the bounds of both factors
    c1 = w1 / cc;
    c2 = w2 / cc;
    e1 = (w1e + c1 * cc_err) / (cc - cc_err) + 8.0f * kU * c1;
    e2 = (w2e + c2 * cc_err) / (cc - cc_err) + 8.0f * kU * c2;
    if (!isfinite(e1) || !isfinite(e2)) return -1;
    int t1 = side_test(c1, e1, e), t2 = side_test(c2, e2, e);
    if (t1 == 1 || t2 == 1) return A.area > B.area ? 1 : 2;
    if (t1 == 0 && t2 == 0) return 0;
    return -1;
}

// Every frontier pair in FP32 where that is certain. Pairs the FP32 test
// cannot decide go to a list for the FP64 test, and so do the kept pairs
// that may hold the largest weight of the model: a kept pair whose upper
// bound is below the largest lower bound already listed cannot (that listed
// pair's exact weight is at least its lower bound), so only pairs near the
// running maximum take the FP64 test for it. `lo_bits` holds that running
// lower bound (bits of a non-negative double).
__global__ void __launch_bounds__(128) k_mesh_decide32(int64_t n, const int2 *__restrict__ pairs, const uint16_t *__restrict__ meta,
                                                       const Element *__restrict__ el, float e, float mesh_curv, float inv_max_area,
                                                       float inv_max_side, uint8_t *flag, uint8_t *split, int32_t *listed,
                                                       unsigned long long *n_listed, unsigned long long *lo_bits,
                                                       int *max_level, unsigned *too_deep) {
    int lvl_max = 0;
    // whole warps stay in the loop while their first pair exists (ballots below)
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i - (threadIdx.x & 31) < n;
         i += (int64_t)gridDim.x * blockDim.x) {
        bool ok = i < n, list = false;
        double lo = 0.0;
        if (ok) {
            int2 pr = pairs[i];
            uint16_t m = meta[i];
            int lvl = m & kLevelMask;
            lvl_max = max(lvl_max, lvl);
            if (lvl > kMaxMeshLevel) {
                atomicOr(too_deep, 1u);
                flag[i] = 0;
            } else {
                const Element &A = el[pr.x], &B = el[pr.y];
                float c1 = 0, e1 = 0, c2 = 0, e2 = 0;
                int f = mesh_decide32(A, B, (m & kSelfBit) != 0, e, mesh_curv, inv_max_area, inv_max_side, c1, e1, c2, e2);
                flag[i] = (uint8_t)(f < 0 ? 0 : f);
                if (f > 0) {
                    int x = f == 1 ? pr.x : pr.y;
                    if (el[x].type & FCG_IS_LEAF) split[x] = 1;
                } else if (f < 0) {
                    list = true;
                } else {
                    // a kept pair: may its exact weight be the model's largest?
                    float hi = 0.0f, l = 0.0f;
                    if (!(A.type & FCG_IS_SUPER_NODE)) { hi = c1 + e1; l = c1 - e1; }
                    if (!(B.type & FCG_IS_SUPER_NODE)) { hi = fmaxf(hi, c2 + e2); l = fmaxf(l, c2 - e2); }
                    double cur = __longlong_as_double((long long)*(volatile unsigned long long *)lo_bits);
                    if (hi > 0.0f && (double)hi >= cur) {
                        list = true;
                        lo = l > 0.0f ? (double)l : 0.0;
                    }
                }
            }
        }
        // warp-aggregated append to the FP64 list, and the running lower bound
        unsigned mk = __ballot_sync(0xffffffffu, list);
        if (mk) {
            int lane = threadIdx.x & 31, leader = __ffs(mk) - 1;
            unsigned long long base = 0;
            if (lane == leader) base = atomicAdd(n_listed, (unsigned long long)__popc(mk));
            base = __shfl_sync(0xffffffffu, base, leader);
            if (list) listed[base + __popc(mk & ((1u << lane) - 1u))] = (int32_t)i;
            for (int o = 16; o > 0; o >>= 1) lo = fmax(lo, __shfl_xor_sync(0xffffffffu, lo, o));
            if (lane == leader && lo > 0.0) atomicMax(lo_bits, (unsigned long long)__double_as_longlong(lo));
        }
    }
    for (int o = 16; o > 0; o >>= 1) lvl_max = max(lvl_max, __shfl_xor_sync(0xffffffffu, lvl_max, o));
    if ((threadIdx.x & 31) == 0) atomicMax(max_level, lvl_max);
}

// the FP64 test (the host builder's own code) for the listed pairs: the
// decision and, for kept pairs, the exact weights behind the model's largest
__global__ void __launch_bounds__(128) k_mesh_decide64(const unsigned long long *__restrict__ n_listed,
                                                       const int32_t *__restrict__ listed, const int2 *__restrict__ pairs,
                                                       const uint16_t *__restrict__ meta, const Element *__restrict__ el,
                                                       double mesh_eps, double mesh_curv, double max_side, double max_area,
                                                       uint8_t *flag, uint8_t *split, unsigned long long *max_eps_bits) {
    int64_t cnt = (int64_t)*n_listed;
    unsigned long long eps_max = 0;
    for (int64_t j = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; j < cnt; j += (int64_t)gridDim.x * blockDim.x) {
        int64_t i = listed[j];
        int2 pr = pairs[i];
        const Element &A = el[pr.x], &B = el[pr.y];
        double c1, c2;
        int f = fcg_mesh_decision(A, B, (meta[i] & kSelfBit) != 0, mesh_eps, mesh_curv, max_side, max_area, &c1, &c2);
        flag[i] = (uint8_t)f;
        if (f) {
            int x = f == 1 ? pr.x : pr.y;
            if (el[x].type & FCG_IS_LEAF) split[x] = 1;
        } else {
            if (!(A.type & FCG_IS_SUPER_NODE) && c1 == c1) eps_max = max(eps_max, (unsigned long long)__double_as_longlong(c1));
            if (!(B.type & FCG_IS_SUPER_NODE) && c2 == c2) eps_max = max(eps_max, (unsigned long long)__double_as_longlong(c2));
        }
    }
    for (int o = 16; o > 0; o >>= 1) eps_max = max(eps_max, __shfl_xor_sync(0xffffffffu, eps_max, o));
    if ((threadIdx.x & 31) == 0 && eps_max) atomicMax(max_eps_bits, eps_max);
}

__global__ void __launch_bounds__(128) k_mesh_decide(int64_t n, const int2 *__restrict__ pairs, const uint16_t *__restrict__ meta,
                                                     const Element *__restrict__ el, double mesh_eps, double mesh_curv,
                                                     double max_side, double max_area, uint8_t *flag, uint8_t *split,
                                                     unsigned long long *max_eps_bits, int *max_level, unsigned *too_deep) {
    int lvl_max = 0;
    // largest weight of the pairs this thread kept, as the bits of a
    // non-negative double (their order is the values' order); one atomic per
    // warp at the end instead of one per pair on a single word
    unsigned long long eps_max = 0;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        int2 pr = pairs[i];
        uint16_t m = meta[i];
        int lvl = m & kLevelMask;
        lvl_max = max(lvl_max, lvl);
        if (lvl > kMaxMeshLevel) {
            atomicOr(too_deep, 1u);
            flag[i] = 0;
            continue;
        }
        const Element &A = el[pr.x], &B = el[pr.y];
        double c1, c2;
        int f = fcg_mesh_decision(A, B, (m & kSelfBit) != 0, mesh_eps, mesh_curv, max_side, max_area, &c1, &c2);
        flag[i] = (uint8_t)f;
        if (f) {
            int x = f == 1 ? pr.x : pr.y;
            if (el[x].type & FCG_IS_LEAF) split[x] = 1;  // many pairs may mark the same leaf
        } else {
            // the largest weight of a pair that needed no refinement (weights are >= 0)
            if (!(A.type & FCG_IS_SUPER_NODE) && c1 == c1) eps_max = max(eps_max, (unsigned long long)__double_as_longlong(c1));
            if (!(B.type & FCG_IS_SUPER_NODE) && c2 == c2) eps_max = max(eps_max, (unsigned long long)__double_as_longlong(c2));
        }
    }
    for (int o = 16; o > 0; o >>= 1) {
        lvl_max = max(lvl_max, __shfl_xor_sync(0xffffffffu, lvl_max, o));
        eps_max = max(eps_max, __shfl_xor_sync(0xffffffffu, eps_max, o));
    }
    if ((threadIdx.x & 31) == 0) {
        atomicMax(max_level, lvl_max);
        if (eps_max) atomicMax(max_eps_bits, eps_max);
    }
}

// bisect the marked leaves into ids ne + 2 rank, ne + 2 rank + 1; the pair of
// the two halves joins the next frontier (self pass) after the split pairs'
// children
__global__ void k_mesh_bisect(int64_t ne, uint8_t *split, const int32_t *__restrict__ rank, Element *el, int32_t *depth,
                              int64_t child_base, int2 *next, uint16_t *next_meta) {
    for (int64_t x = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; x < ne; x += (int64_t)gridDim.x * blockDim.x) {
        if (!split[x]) continue;
        split[x] = 0;
        int64_t k = rank[x];
        int32_t l = (int32_t)(ne + 2 * k), r = l + 1;
        Element P = el[x];
        Element Lc, Rc;
        fcg_subdivide(P, Lc, Rc);
        el[l] = Lc;
        el[r] = Rc;
        int32_t d = depth[x];
        depth[l] = d + 1;
        depth[r] = d + 1;
        el[x].left = l;
        el[x].right = r;
        el[x].type = (uint8_t)(P.type & ~FCG_IS_LEAF);
        next[child_base + k] = make_int2(l, r);
        next_meta[child_base + k] = (uint16_t)(kSelfBit | (uint16_t)min(d + 2, (int)kLevelMask));
    }
}

// children of every split pair at 2 * (exclusive rank among split pairs)
__global__ void __launch_bounds__(kThreads) k_mesh_expand(int64_t n, const int2 *__restrict__ pairs, const uint16_t *__restrict__ meta,
                                                          const uint8_t *__restrict__ flag, const Element *__restrict__ el,
                                                          const long long *__restrict__ tile_off, int2 *next, uint16_t *next_meta) {
    __shared__ long long wt[32];
    int64_t base = (int64_t)blockIdx.x * kTile + (int64_t)threadIdx.x * kItems;
    uint8_t f[kItems];
    long long s = 0;
    for (int j = 0; j < kItems; j++) {
        f[j] = base + j < n ? flag[base + j] : 0;
        s += f[j] != 0;
    }
    long long tot;
    long long r = block_exclusive_scan(s, wt, &tot) + tile_off[blockIdx.x];
    for (int j = 0; j < kItems; j++) {
        int64_t i = base + j;
        if (i >= n) break;
        if (!f[j]) continue;
        int2 pr = pairs[i];
        int2 c0 = pr, c1 = pr;
        if (f[j] == 1) {
            c0.x = el[pr.x].left;
            c1.x = el[pr.x].right;
        } else {
            c0.y = el[pr.y].left;
            c1.y = el[pr.y].right;
        }
        uint16_t m = meta[i];
        uint16_t m1 = (uint16_t)((m & kSelfBit) | (uint16_t)min((m & kLevelMask) + 1, (int)kLevelMask));
        next[2 * r] = c0;
        next[2 * r + 1] = c1;
        next_meta[2 * r] = m1;
        next_meta[2 * r + 1] = m1;
        r++;
    }
}

__global__ void k_count_split(int64_t n, const uint8_t *__restrict__ flag, long long *tile_sums) {
    __shared__ long long wt[32];
    int64_t base = (int64_t)blockIdx.x * kTile + (int64_t)threadIdx.x * kItems;
    long long c = 0;
    for (int j = 0; j < kItems; j++)
        if (base + j < n) c += flag[base + j] != 0;
    c = block_sum(c, wt);
    if (threadIdx.x == 0) tile_sums[blockIdx.x] = c;
}

}  // namespace

#define MB_CK(x)                                                                                     \
    do {                                                                                             \
        cudaError_t e_ = (x);                                                                        \
        if (e_ != cudaSuccess) {                                                                     \
            err = std::string("device mesh refinement: ") + cudaGetErrorString(e_);                  \
            cudaGetLastError();                                                                      \
            return e_ == cudaErrorMemoryAllocation ? FCG_OUT_OF_MEMORY : FCG_DEVICE_ERROR;           \
        }                                                                                            \
    } while (0)

int mesh_refine_device(DeviceContext &ctx, std::vector<Element> &el, const std::vector<int32_t> &depth,
                       const std::vector<int32_t> &root_a, const std::vector<int32_t> &root_b,
                       const std::vector<uint16_t> &root_meta, double mesh_eps, double mesh_curv, double max_side,
                       double max_area, double &max_mesh_eps, int &max_level, std::string &err) {
    MB_CK(cudaSetDevice(ctx.device));
    Bufs B;
    MB_CK(cudaStreamCreateWithFlags(&B.s, cudaStreamNonBlocking));
    cudaStream_t s = B.s;
    const int sms = ctx.sm_count > 0 ? ctx.sm_count : 1;
    const bool trace = getenv("FCG_TRACE") != nullptr;
    // FCG_MESH_FP64=1: every pair through the FP64 test (no FP32 pre-test)
    const bool fp64_only = getenv("FCG_MESH_FP64") != nullptr;
    int64_t ne = (int64_t)el.size();
    int64_t cap = std::max<int64_t>(2 * ne, ne + (1 << 20));
    Element *d_el;
    int32_t *d_depth, *d_rank;
    uint8_t *d_split;
    long long *d_scalars;  // [0] split pairs, [1] marked leaves
    unsigned long long *d_max_eps, *d_lo_bits, *d_n_listed;
    int *d_max_level;
    unsigned *d_too_deep;
    MB_CK(B.alloc(&d_el, (size_t)cap));
    MB_CK(B.alloc(&d_depth, (size_t)cap));
    MB_CK(B.alloc(&d_rank, (size_t)cap));
    MB_CK(B.alloc(&d_split, (size_t)cap));
    MB_CK(B.alloc(&d_scalars, 2));
    MB_CK(B.alloc(&d_max_eps, 1));
    MB_CK(B.alloc(&d_lo_bits, 1));
    MB_CK(B.alloc(&d_n_listed, 1));
    MB_CK(B.alloc(&d_max_level, 1));
    MB_CK(B.alloc(&d_too_deep, 1));
    MB_CK(cudaMemcpyAsync(d_el, el.data(), (size_t)ne * sizeof(Element), cudaMemcpyHostToDevice, s));
    MB_CK(cudaMemcpyAsync(d_depth, depth.data(), (size_t)ne * sizeof(int32_t), cudaMemcpyHostToDevice, s));
    MB_CK(cudaMemsetAsync(d_split, 0, (size_t)cap, s));
    MB_CK(cudaMemsetAsync(d_max_eps, 0, sizeof(unsigned long long), s));
    MB_CK(cudaMemsetAsync(d_lo_bits, 0, sizeof(unsigned long long), s));
    MB_CK(cudaMemsetAsync(d_max_level, 0, sizeof(int), s));
    MB_CK(cudaMemsetAsync(d_too_deep, 0, sizeof(unsigned), s));

    int64_t n = (int64_t)root_a.size();
    int2 *pairs = nullptr;
    uint16_t *meta = nullptr;
    {
        std::vector<int2> h((size_t)n);
        for (int64_t i = 0; i < n; i++) h[(size_t)i] = make_int2(root_a[(size_t)i], root_b[(size_t)i]);
        MB_CK(B.alloc(&pairs, (size_t)n));
        MB_CK(B.alloc(&meta, (size_t)n));
        MB_CK(cudaMemcpyAsync(pairs, h.data(), (size_t)n * sizeof(int2), cudaMemcpyHostToDevice, s));
        MB_CK(cudaMemcpyAsync(meta, root_meta.data(), (size_t)n * sizeof(uint16_t), cudaMemcpyHostToDevice, s));
        MB_CK(cudaStreamSynchronize(s));  // the host vector goes out of scope
    }
    long long tests = 0, steps = 0;
    while (n > 0) {
        steps++;
        tests += n;
        uint8_t *flag;
        int32_t *listed;
        long long *tsums, *esums;
        unsigned tiles = grid_tiles(n), etiles = grid_tiles(ne);
        MB_CK(B.alloc(&flag, (size_t)n));
        MB_CK(B.alloc(&listed, (size_t)n));
        MB_CK(B.alloc(&tsums, tiles));
        MB_CK(B.alloc(&esums, etiles));
        if (fp64_only) {
            k_mesh_decide<<<grid_stride(n, sms, 128), 128, 0, s>>>(n, pairs, meta, d_el, mesh_eps, mesh_curv, max_side, max_area,
                                                                   flag, d_split, d_max_eps, d_max_level, d_too_deep);
        } else {
            // FP32 pre-test, then the FP64 test for the listed pairs
            MB_CK(cudaMemsetAsync(d_n_listed, 0, sizeof(unsigned long long), s));
            k_mesh_decide32<<<grid_stride(n, sms, 128), 128, 0, s>>>(n, pairs, meta, d_el, (float)mesh_eps, (float)mesh_curv,
                                                                     (float)(1.0 / max_area), (float)(1.0 / max_side), flag,
                                                                     d_split, listed, d_n_listed, d_lo_bits, d_max_level,
                                                                     d_too_deep);
            k_mesh_decide64<<<grid_stride(n, sms, 128), 128, 0, s>>>(d_n_listed, listed, pairs, meta, d_el, mesh_eps, mesh_curv,
                                                                     max_side, max_area, flag, d_split, d_max_eps);
        }
        k_count_split<<<tiles, kThreads, 0, s>>>(n, flag, tsums);
        k_scan_sums<<<1, 1024, 0, s>>>(tiles, tsums, d_scalars);
        exclusive_scan(s, ne, d_split, d_rank, esums, d_scalars + 1);
        MB_CK(cudaGetLastError());
        long long h[2];
        unsigned deep = 0;
        MB_CK(cudaMemcpyAsync(h, d_scalars, 2 * sizeof(long long), cudaMemcpyDeviceToHost, s));
        MB_CK(cudaMemcpyAsync(&deep, d_too_deep, sizeof(unsigned), cudaMemcpyDeviceToHost, s));
        MB_CK(cudaStreamSynchronize(s));
        if (deep) {
            err = "mesh refinement recursion too deep (touching or overlapping panels?)";
            return FCG_GENERIC_ERROR;
        }
        const long long n_split_pairs = h[0], n_leaves = h[1];
        const int64_t n_next = 2 * n_split_pairs + n_leaves;
        if (n_next > kMaxFrontier || ne + 2 * n_leaves > 0x7fffffffLL) {
            err = "mesh refinement recursion too deep (touching or overlapping panels?)";
            return FCG_GENERIC_ERROR;
        }
        if (ne + 2 * n_leaves > cap) {  // grow the element arrays
            int64_t ncap = std::max<int64_t>(2 * cap, ne + 2 * n_leaves);
            Element *el2;
            int32_t *depth2, *rank2;
            uint8_t *split2;
            MB_CK(B.alloc(&el2, (size_t)ncap));
            MB_CK(B.alloc(&depth2, (size_t)ncap));
            MB_CK(B.alloc(&rank2, (size_t)ncap));
            MB_CK(B.alloc(&split2, (size_t)ncap));
            MB_CK(cudaMemcpyAsync(el2, d_el, (size_t)ne * sizeof(Element), cudaMemcpyDeviceToDevice, s));
            MB_CK(cudaMemcpyAsync(depth2, d_depth, (size_t)ne * sizeof(int32_t), cudaMemcpyDeviceToDevice, s));
            MB_CK(cudaMemcpyAsync(rank2, d_rank, (size_t)ne * sizeof(int32_t), cudaMemcpyDeviceToDevice, s));
            MB_CK(cudaMemcpyAsync(split2, d_split, (size_t)ne, cudaMemcpyDeviceToDevice, s));
            MB_CK(cudaMemsetAsync(split2 + ne, 0, (size_t)(ncap - ne), s));
            B.release(d_el);
            B.release(d_depth);
            B.release(d_rank);
            B.release(d_split);
            d_el = el2;
            d_depth = depth2;
            d_rank = rank2;
            d_split = split2;
            cap = ncap;
        }
        int2 *next = nullptr;
        uint16_t *next_meta = nullptr;
        if (n_next > 0) {
            MB_CK(B.alloc(&next, (size_t)n_next));
            MB_CK(B.alloc(&next_meta, (size_t)n_next));
        }
        if (n_leaves > 0)
            k_mesh_bisect<<<grid_stride(ne, sms), 256, 0, s>>>(ne, d_split, d_rank, d_el, d_depth, 2 * n_split_pairs, next,
                                                               next_meta);
        if (n_split_pairs > 0) k_mesh_expand<<<tiles, kThreads, 0, s>>>(n, pairs, meta, flag, d_el, tsums, next, next_meta);
        MB_CK(cudaGetLastError());
        B.release(flag);
        B.release(listed);
        B.release(tsums);
        B.release(esums);
        B.release(pairs);
        B.release(meta);
        pairs = next;
        meta = next_meta;
        ne += 2 * n_leaves;
        n = n_next;
    }
    unsigned long long eps_bits = 0;
    MB_CK(cudaMemcpyAsync(&eps_bits, d_max_eps, sizeof(eps_bits), cudaMemcpyDeviceToHost, s));
    MB_CK(cudaMemcpyAsync(&max_level, d_max_level, sizeof(int), cudaMemcpyDeviceToHost, s));
    el.resize((size_t)ne);
    MB_CK(cudaMemcpyAsync(el.data(), d_el, (size_t)ne * sizeof(Element), cudaMemcpyDeviceToHost, s));
    MB_CK(cudaStreamSynchronize(s));
    double me;
    memcpy(&me, &eps_bits, sizeof me);
    max_mesh_eps = me;
    if (trace) fprintf(stderr, "[fcg mesh] %lld steps, %lld pair tests, %lld elements\n", steps, tests, (long long)ne);
    return FCG_NORMAL_END;
}

}  // namespace fcg
