// Link construction on the GPU: the dual-tree traversal of
// CAutoRefine::RefineMutual / RefineSelf (Solver/Autorefine.cpp:3096-3235,
// 2115-2229) and the bucketing of the emitted pairs by destination node
// (the link lists of CAutoRefine::RecurseIndex, Solver/Autorefine.cpp:1173-1220).
//
// Traversal. Every root pair (one per conductor pair, then one per internal
// element for the self interactions, in the host traversal's order) starts a
// binary recursion tree: a pair either links (a leaf of the recursion tree)
// or is replaced by two pairs, the children of one side. The frontier is
// expanded one level per step; the two children of a split pair are placed
// next to each other, in the order of their parents, so each level keeps the
// left-to-right order of the recursion trees. A bottom-up pass counts the
// links under every frontier item and a top-down pass hands out depth-first
// positions (an exclusive scan over the roots, then parent offset / parent
// offset + left child count): the emitted pairs come out in exactly the order
// of the recursive host traversal.
//
// Buckets. Pair k = (a, b) gives the entries (dest a, src b) and (dest b,
// src a); a stable LSD radix sort on the destination (8-bit digits, warp
// match for the stable rank) keeps every row in emission order, which is the
// host builder's stable counting sort.
//
// This file is compiled with -fmad=false so that fcg_link_decision rounds
// every operation the way the host builder (-ffp-contract=off) does: the
// device takes exactly the host's decisions and produces the same arrays.
#include <cuda_runtime.h>

#include <stdio.h>
#include <stdlib.h>

#include <algorithm>
#include <string>
#include <vector>

#include "fc_potential.h"
#include "fcg_internal.hpp"
#include "scan.cuh"
#include "../host/model.hpp"

namespace fcg {

using namespace devscan;

namespace {


static_assert(sizeof(Element) == 96, "element record layout");

// ------------------------------------------------------------------ traversal
// FP32 pre-test. Most pairs are far from every decision boundary of the FP64
// test (the rho = 2 switch between quadrature and point formula, the
// threshold e itself), so an FP32 evaluation with a bound on its distance to
// the FP64 value decides them; the rest (typically a few per cent) take the
// FP64 test. Bounds are deliberately loose (a factor 4 and more over a
// first-order rounding analysis): a loose bound only sends more pairs to
// FP64, it never changes a decision.
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

// fcg_link_decision in FP32, or -1 when only the FP64 test can tell
__device__ int decide32(const Element &A, const Element &B, float e, float inv_max_area, float inv_max_side) {
    bool leaf1 = (A.type & FCG_IS_LEAF) != 0, leaf2 = (B.type & FCG_IS_LEAF) != 0;
    if (leaf1 && leaf2) return 0;
    float dx = A.c[0] - B.c[0], dy = A.c[1] - B.c[1], dz = A.c[2] - B.c[2];  // fcg_fsub's float values
    float r = sqrtf(dx * dx + dy * dy + dz * dz);
    double rm = A.maxside > B.maxside ? A.maxside : B.maxside;
    float rho = r / (float)rm;
    if (!(r > 1e-10f) || !(fabsf(rho - 2.0f) > 1e-5f)) return -1;
    bool quad = rho < 2.0f;
    float c1, e1, c2, e2;
    if (!weight32(A, B, dx, dy, dz, r, quad, inv_max_area, inv_max_side, c1, e1)) return -1;
    if (!weight32(B, A, -dx, -dy, -dz, r, quad, inv_max_area, inv_max_side, c2, e2)) return -1;
    int t1 = side_test(c1, e1, e), t2 = side_test(c2, e2, e);
    if (t1 != 1 && t2 != 1) {
        if (t1 == 0 && t2 == 0) return 0;
        return -1;
    }
    if (!leaf1 && leaf2) return 1;
    if (leaf1 && !leaf2) return 2;
    return A.area > B.area ? 1 : 2;
}

// decide every frontier pair in FP32 where that is certain: 0 link, 1 split
// the first element, 2 the second; undecided pairs go to a list for FP64
__global__ void __launch_bounds__(kThreads) k_decide32(int64_t n, const int2 *__restrict__ pairs, const uint16_t *__restrict__ root_level,
                                                       int depth, const Element *__restrict__ el, float e, float inv_max_area,
                                                       float inv_max_side, uint8_t *flag, int32_t *undecided,
                                                       unsigned long long *n_undecided, int *max_level) {
    int lvl = 0;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i - (threadIdx.x) < n; i += (int64_t)gridDim.x * blockDim.x) {
        int f = 0;
        bool ok = i < n;
        if (ok) {
            int2 pr = pairs[i];
            f = decide32(el[pr.x], el[pr.y], e, inv_max_area, inv_max_side);
            flag[i] = (uint8_t)(f < 0 ? 0 : f);
            lvl = max(lvl, (int)root_level[i] + depth);
        }
        // warp-aggregated append of the undecided pairs
        unsigned m = __ballot_sync(0xffffffffu, ok && f < 0);
        if (m) {
            int lane = threadIdx.x & 31, leader = __ffs(m) - 1;
            unsigned long long base = 0;
            if (lane == leader) base = atomicAdd(n_undecided, (unsigned long long)__popc(m));
            base = __shfl_sync(0xffffffffu, base, leader);
            if (ok && f < 0) undecided[base + __popc(m & ((1u << lane) - 1u))] = (int32_t)i;
        }
    }
    for (int o = 16; o > 0; o >>= 1) lvl = max(lvl, __shfl_xor_sync(0xffffffffu, lvl, o));
    if ((threadIdx.x & 31) == 0) atomicMax(max_level, lvl);
}

// the FP64 test (the host builder's own code) for the undecided pairs
__global__ void __launch_bounds__(128) k_decide64(const unsigned long long *__restrict__ n_undecided, const int32_t *__restrict__ undecided,
                                                  const int2 *__restrict__ pairs, const Element *__restrict__ el, double eps,
                                                  double max_side, double max_area, uint8_t *flag) {
    int64_t m = (int64_t)*n_undecided;
    for (int64_t j = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; j < m; j += (int64_t)gridDim.x * blockDim.x) {
        int32_t i = undecided[j];
        int2 pr = pairs[i];
        flag[i] = (uint8_t)fcg_link_decision(el[pr.x], el[pr.y], eps, max_side, max_area);
    }
}

// per-tile count of split pairs
__global__ void __launch_bounds__(kThreads) k_split_tiles(int64_t n, const uint8_t *__restrict__ flag, long long *tile_sums) {
    __shared__ long long wt[32];
    int64_t base = (int64_t)blockIdx.x * kTile + (int64_t)threadIdx.x * kItems;
    long long splits = 0;
    for (int j = 0; j < kItems; j++)
        if (base + j < n) splits += flag[base + j] != 0;
    splits = block_sum(splits, wt);
    if (threadIdx.x == 0) tile_sums[blockIdx.x] = splits;
}

// children of every split pair into the next level, at 2 * (exclusive rank)
__global__ void __launch_bounds__(kThreads) k_expand(int64_t n, int64_t ne, const int2 *__restrict__ pairs,
                                                     const uint16_t *__restrict__ root_level, const uint8_t *__restrict__ flag,
                                                     const Element *__restrict__ el, const long long *__restrict__ tile_off,
                                                     int32_t *rank, int2 *next, uint16_t *next_level, unsigned *bad) {
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
        if (!f[j]) {
            rank[i] = -1;
            continue;
        }
        int2 pr = pairs[i];
        int2 c0 = pr, c1 = pr;
        if (f[j] == 1) {
            c0.x = el[pr.x].left;
            c1.x = el[pr.x].right;
        } else {
            c0.y = el[pr.y].left;
            c1.y = el[pr.y].right;
        }
        // a split side always has two children; anything else is a corrupt hierarchy
        if (c0.x < 0 || c0.y < 0 || c1.x < 0 || c1.y < 0 || c0.x >= ne || c0.y >= ne || c1.x >= ne || c1.y >= ne) {
            atomicAdd(bad, 1u);
            c0 = c1 = make_int2(0, 0);
        }
        rank[i] = (int32_t)r;
        next[2 * r] = c0;
        next[2 * r + 1] = c1;
        uint16_t rl = root_level[i];
        next_level[2 * r] = rl;
        next_level[2 * r + 1] = rl;
        r++;
    }
}

// links under every item (bottom-up; the deepest level has only links)
__global__ void k_count(int64_t n, const int32_t *__restrict__ rank, const long long *__restrict__ cnt_next, long long *cnt) {
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        int32_t r = rank[i];
        cnt[i] = r < 0 ? 1 : cnt_next[2 * (int64_t)r] + cnt_next[2 * (int64_t)r + 1];
    }
}

// depth-first positions (top-down); `next` holds the next level's counts and
// receives its offsets (each pair of entries is touched by its parent only)
__global__ void k_place(int64_t n, const int2 *__restrict__ pairs, const int32_t *__restrict__ rank, const long long *__restrict__ off,
                        long long *next, int2 *out) {
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        int32_t r = rank[i];
        long long o = off[i];
        if (r < 0) {
            out[o] = pairs[i];
        } else {
            long long c0 = next[2 * (int64_t)r];
            next[2 * (int64_t)r] = o;
            next[2 * (int64_t)r + 1] = o + c0;
        }
    }
}

// ------------------------------------------------------------------ buckets
// pair k -> entries 2k (dest a, src b) and 2k+1 (dest b, src a); node degrees
__global__ void k_entries(int64_t P, const int2 *__restrict__ pairs, const int32_t *__restrict__ node_of,
                          unsigned long long *ent, int *deg) {
    for (int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; k < P; k += (int64_t)gridDim.x * blockDim.x) {
        int2 pr = pairs[k];
        unsigned a = (unsigned)node_of[pr.x], b = (unsigned)node_of[pr.y];
        ent[2 * k] = ((unsigned long long)a << 32) | b;
        ent[2 * k + 1] = ((unsigned long long)b << 32) | a;
        atomicAdd(deg + a, 1);
        atomicAdd(deg + b, 1);
    }
}

// ------------------------------------------------------------------ host side
struct Level {
    int64_t n = 0;
    int2 *pairs = nullptr;
    uint16_t *root_level = nullptr;
    int32_t *rank = nullptr;
    long long *cnt = nullptr;
};


}  // namespace

#define LB_CK(x)                                                                                     \
    do {                                                                                             \
        cudaError_t e_ = (x);                                                                        \
        if (e_ != cudaSuccess) {                                                                     \
            err = std::string("device link construction: ") + cudaGetErrorString(e_);               \
            cudaGetLastError();                                                                      \
            return e_ == cudaErrorMemoryAllocation ? FCG_OUT_OF_MEMORY : FCG_DEVICE_ERROR;           \
        }                                                                                            \
    } while (0)

int link_build_device(DeviceContext &ctx, const Element *el, int64_t ne, const int32_t *root_a, const int32_t *root_b,
                      const uint16_t *root_level, int64_t n_roots, const int32_t *node_of, int64_t n_nodes, double eps,
                      double max_side, double max_area, std::vector<int64_t> &link_ptr, std::vector<int32_t> &link_src,
                      int &max_level, std::string &err) {
    LB_CK(cudaSetDevice(ctx.device));
    Bufs B;
    LB_CK(cudaStreamCreateWithFlags(&B.s, cudaStreamNonBlocking));
    cudaStream_t s = B.s;
    const int sms = ctx.sm_count > 0 ? ctx.sm_count : 1;
    link_ptr.assign((size_t)n_nodes + 1, 0);
    link_src.clear();
    max_level = 0;
    if (n_roots == 0 || n_nodes == 0) return FCG_NORMAL_END;

    Element *d_el;
    int32_t *d_node_of;
    long long *d_scalars;  // [0] scan total, [1] spare
    int *d_max_level;
    unsigned *d_bad;
    unsigned long long *d_undecided;
    const float inv_max_area = (float)(1.0 / max_area), inv_max_side = (float)(1.0 / max_side);
    const bool trace = getenv("FCG_TRACE") != nullptr;
    long long n_tests = 0, n_fp64 = 0;
    LB_CK(B.alloc(&d_undecided, 1));
    LB_CK(B.alloc(&d_el, (size_t)ne));
    LB_CK(B.alloc(&d_node_of, (size_t)ne));
    LB_CK(B.alloc(&d_scalars, 2));
    LB_CK(B.alloc(&d_max_level, 1));
    LB_CK(B.alloc(&d_bad, 1));
    LB_CK(cudaMemcpyAsync(d_el, el, (size_t)ne * sizeof(Element), cudaMemcpyHostToDevice, s));
    LB_CK(cudaMemcpyAsync(d_node_of, node_of, (size_t)ne * sizeof(int32_t), cudaMemcpyHostToDevice, s));
    LB_CK(cudaMemsetAsync(d_max_level, 0, sizeof(int), s));
    LB_CK(cudaMemsetAsync(d_bad, 0, sizeof(unsigned), s));

    // roots
    std::vector<Level> lv(1);
    {
        Level &L0 = lv[0];
        L0.n = n_roots;
        std::vector<int2> h((size_t)n_roots);
        for (int64_t i = 0; i < n_roots; i++) h[(size_t)i] = make_int2(root_a[i], root_b[i]);
        LB_CK(B.alloc(&L0.pairs, (size_t)n_roots));
        LB_CK(B.alloc(&L0.root_level, (size_t)n_roots));
        LB_CK(cudaMemcpyAsync(L0.pairs, h.data(), (size_t)n_roots * sizeof(int2), cudaMemcpyHostToDevice, s));
        LB_CK(cudaMemcpyAsync(L0.root_level, root_level, (size_t)n_roots * sizeof(uint16_t), cudaMemcpyHostToDevice, s));
    }

    // frontier expansion, one level per step
    for (int depth = 0;; depth++) {
        Level &L = lv.back();
        int64_t n = L.n;
        unsigned tiles = grid_tiles(n);
        uint8_t *flag;
        long long *sums;
        int32_t *undecided;
        LB_CK(B.alloc(&flag, (size_t)n));
        LB_CK(B.alloc(&sums, tiles));
        LB_CK(B.alloc(&undecided, (size_t)n));
        LB_CK(B.alloc(&L.rank, (size_t)n));
        LB_CK(cudaMemsetAsync(d_undecided, 0, sizeof(unsigned long long), s));
        k_decide32<<<grid_stride(n, sms), 256, 0, s>>>(n, L.pairs, L.root_level, depth, d_el, (float)eps, inv_max_area,
                                                        inv_max_side, flag, undecided, d_undecided, d_max_level);
        k_decide64<<<grid_stride(n, sms), 128, 0, s>>>(d_undecided, undecided, L.pairs, d_el, eps, max_side, max_area, flag);
        k_split_tiles<<<tiles, kThreads, 0, s>>>(n, flag, sums);
        k_scan_sums<<<1, 1024, 0, s>>>(tiles, sums, d_scalars);
        LB_CK(cudaGetLastError());
        long long level_counts[2] = {0, 0};  // splits, FP64 tests
        LB_CK(cudaMemcpyAsync(&level_counts[0], d_scalars, sizeof(long long), cudaMemcpyDeviceToHost, s));
        LB_CK(cudaMemcpyAsync(&level_counts[1], d_undecided, sizeof(long long), cudaMemcpyDeviceToHost, s));
        LB_CK(cudaStreamSynchronize(s));
        B.release(undecided);
        long long splits = level_counts[0];
        n_tests += n;
        n_fp64 += level_counts[1];
        if (splits > (1ll << 29)) {
            err = "model too large for 32-bit link indices";
            return FCG_OUT_OF_MEMORY;
        }
        Level nx;
        nx.n = 2 * splits;
        if (splits > 0) {
            LB_CK(B.alloc(&nx.pairs, (size_t)nx.n));
            LB_CK(B.alloc(&nx.root_level, (size_t)nx.n));
        }
        k_expand<<<tiles, kThreads, 0, s>>>(n, ne, L.pairs, L.root_level, flag, d_el, sums, L.rank, nx.pairs, nx.root_level, d_bad);
        LB_CK(cudaGetLastError());
        B.release(flag);
        B.release(sums);
        B.release(L.root_level);
        if (splits == 0) break;
        lv.push_back(nx);
    }
    unsigned bad = 0;
    LB_CK(cudaMemcpyAsync(&bad, d_bad, sizeof(unsigned), cudaMemcpyDeviceToHost, s));
    LB_CK(cudaMemcpyAsync(&max_level, d_max_level, sizeof(int), cudaMemcpyDeviceToHost, s));
    LB_CK(cudaStreamSynchronize(s));
    if (bad) {
        err = "device link construction: a split element without two children (" + std::to_string(bad) + " pairs)";
        return FCG_GENERIC_ERROR;
    }
    if (trace)
        fprintf(stderr, "[fcg links] %zu levels, %lld pair tests, %lld (%.2f %%) by the FP64 test\n", lv.size(), n_tests, n_fp64,
                n_tests ? 100.0 * (double)n_fp64 / (double)n_tests : 0.0);

    // links under every item, deepest level first
    for (size_t d = lv.size(); d-- > 0;) {
        Level &L = lv[d];
        LB_CK(B.alloc(&L.cnt, (size_t)L.n));
        const long long *cn = d + 1 < lv.size() ? lv[d + 1].cnt : nullptr;
        k_count<<<grid_stride(L.n, sms), 256, 0, s>>>(L.n, L.rank, cn, L.cnt);
        LB_CK(cudaGetLastError());
    }
    // depth-first positions: scan over the roots, then parent to children
    long long P = 0;
    {
        Level &L0 = lv[0];
        unsigned tiles = grid_tiles(L0.n);
        long long *sums;
        LB_CK(B.alloc(&sums, tiles));
        k_scan_tiles<<<tiles, kThreads, 0, s>>>(L0.n, L0.cnt, sums);
        k_scan_sums<<<1, 1024, 0, s>>>(tiles, sums, d_scalars);
        k_scan_apply<<<tiles, kThreads, 0, s>>>(L0.n, L0.cnt, L0.cnt, sums);
        LB_CK(cudaGetLastError());
        LB_CK(cudaMemcpyAsync(&P, d_scalars, sizeof(long long), cudaMemcpyDeviceToHost, s));
        LB_CK(cudaStreamSynchronize(s));
        B.release(sums);
    }
    if (2 * P > 0x7fffffffLL) {
        err = "model too large for 32-bit link indices";
        return FCG_OUT_OF_MEMORY;
    }
    int2 *emitted;
    LB_CK(B.alloc(&emitted, (size_t)P));
    for (size_t d = 0; d < lv.size(); d++) {
        Level &L = lv[d];
        long long *next = d + 1 < lv.size() ? lv[d + 1].cnt : nullptr;
        k_place<<<grid_stride(L.n, sms), 256, 0, s>>>(L.n, L.pairs, L.rank, L.cnt, next, emitted);
        LB_CK(cudaGetLastError());
    }
    for (Level &L : lv) {
        B.release(L.pairs);
        B.release(L.rank);
        B.release(L.cnt);
    }

    // rows: entries, degrees -> link_ptr, stable radix sort by destination
    const int64_t nent = 2 * P;
    unsigned long long *ent, *ent2 = nullptr;
    int *deg;
    int64_t *d_ptr;
    int32_t *d_src;
    LB_CK(B.alloc(&ent, (size_t)nent));
    LB_CK(B.alloc(&deg, (size_t)n_nodes));
    LB_CK(B.alloc(&d_ptr, (size_t)n_nodes + 1));
    LB_CK(B.alloc(&d_src, (size_t)nent));
    LB_CK(cudaMemsetAsync(deg, 0, (size_t)n_nodes * sizeof(int), s));
    if (P > 0) k_entries<<<grid_stride(P, sms), 256, 0, s>>>(P, emitted, d_node_of, ent, deg);
    LB_CK(cudaGetLastError());
    B.release(emitted);
    {
        unsigned tiles = grid_tiles(n_nodes);
        long long *sums;
        LB_CK(B.alloc(&sums, tiles));
        k_scan_tiles<<<tiles, kThreads, 0, s>>>(n_nodes, deg, sums);
        k_scan_sums<<<1, 1024, 0, s>>>(tiles, sums, (long long *)(d_ptr + n_nodes));
        k_scan_apply<<<tiles, kThreads, 0, s>>>(n_nodes, deg, d_ptr, sums);
        LB_CK(cudaGetLastError());
        B.release(sums);
    }
    B.release(deg);
    if (nent > 0) {
        int bits = 0;
        while (bits < 32 && ((int64_t)1 << bits) < n_nodes) bits++;
        int passes = std::max(1, (bits + 7) / 8);
        unsigned tiles = grid_tiles(nent);
        int64_t nh = (int64_t)tiles * kDigits;
        int *hist;
        long long *hsums;
        unsigned htiles = grid_tiles(nh);
        LB_CK(B.alloc(&hist, (size_t)nh));
        LB_CK(B.alloc(&hsums, htiles));
        if (passes > 1) LB_CK(B.alloc(&ent2, (size_t)nent));
        unsigned long long *src = ent, *dst = ent2;
        for (int pass = 0; pass < passes; pass++) {
            int shift = 32 + 8 * pass;
            bool last = pass == passes - 1;
            k_radix_hist<<<tiles, kThreads, 0, s>>>(nent, src, shift, hist);
            k_scan_tiles<<<htiles, kThreads, 0, s>>>(nh, hist, hsums);
            k_scan_sums<<<1, 1024, 0, s>>>(htiles, hsums, d_scalars + 1);
            k_scan_apply<<<htiles, kThreads, 0, s>>>(nh, hist, hist, hsums);
            k_radix_scatter<<<tiles, kThreads, 0, s>>>(nent, src, shift, hist, last ? nullptr : dst, last ? d_src : nullptr);
            LB_CK(cudaGetLastError());
            std::swap(src, dst);
        }
    }
    link_src.resize((size_t)nent);
    LB_CK(cudaMemcpyAsync(link_ptr.data(), d_ptr, ((size_t)n_nodes + 1) * sizeof(int64_t), cudaMemcpyDeviceToHost, s));
    if (nent > 0) LB_CK(cudaMemcpyAsync(link_src.data(), d_src, (size_t)nent * sizeof(int32_t), cudaMemcpyDeviceToHost, s));
    LB_CK(cudaStreamSynchronize(s));
    if (link_ptr[(size_t)n_nodes] != nent) {
        err = "device link construction: row offsets do not add up to the link count";
        return FCG_GENERIC_ERROR;
    }
    return FCG_NORMAL_END;
}

}  // namespace fcg
