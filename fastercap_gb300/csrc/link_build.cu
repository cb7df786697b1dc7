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
#include <chrono>
#include <string>
#include <vector>

#include "fc_potential.h"
#include "pair32.cuh"
#include "fcg_internal.hpp"
#include "scan.cuh"
#include "../host/model.hpp"

namespace fcg {

using namespace devscan;
using namespace pair32;

namespace {


static_assert(sizeof(Element) == 96, "element record layout");

// ------------------------------------------------------------------ traversal
// FP32 pre-test of every pair (pair32.cuh), FP64 for the undecided ones.

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
                      int &max_level, std::string &err, std::shared_ptr<int32_t> *device_src) {
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
    const auto t_begin = std::chrono::steady_clock::now();
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

    auto t_mark = std::chrono::steady_clock::now();
    auto mark = [&](const char *what) {
        if (!trace) return;
        auto now = std::chrono::steady_clock::now();
        fprintf(stderr, "[fcg links]   %-28s %9.3f ms\n", what, std::chrono::duration<double, std::milli>(now - t_mark).count());
        t_mark = now;
    };
    if (trace) fprintf(stderr, "[fcg links]   traversal                    %9.3f ms\n",
                       std::chrono::duration<double, std::milli>(t_mark - t_begin).count());
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
    if (trace) {
        LB_CK(cudaStreamSynchronize(s));
        mark("placement and row sort");
    }
    LB_CK(cudaMemcpyAsync(link_ptr.data(), d_ptr, ((size_t)n_nodes + 1) * sizeof(int64_t), cudaMemcpyDeviceToHost, s));
    if (device_src) {
        // hand the sources over: off the builder's list, freed by the last owner
        auto it = std::find(B.live.begin(), B.live.end(), (void *)d_src);
        if (it != B.live.end()) B.live.erase(it);
        device_src->reset(d_src, [](int32_t *q) { cudaFreeAsync(q, 0); });
        link_src.clear();
    } else {
        link_src.resize((size_t)nent);
        mark("host link array");
        if (nent > 0) LB_CK(cudaMemcpyAsync(link_src.data(), d_src, (size_t)nent * sizeof(int32_t), cudaMemcpyDeviceToHost, s));
    }
    LB_CK(cudaStreamSynchronize(s));
    mark("download");
    if (link_ptr[(size_t)n_nodes] != nent) {
        err = "device link construction: row offsets do not add up to the link count";
        return FCG_GENERIC_ERROR;
    }
    return FCG_NORMAL_END;
}

}  // namespace fcg
