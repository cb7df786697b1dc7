// Building blocks shared by the device model-construction passes (link
// construction, mesh refinement) and the problem layout: CTA scans, a
// three-phase exclusive scan over device arrays, a stable LSD radix pass on
// the high 32 bits of 64-bit entries and a stream-ordered scratch allocator
// that frees everything it still holds when it goes out of scope. Every
// translation unit gets its own copy (internal linkage).
#ifndef FCG_SCAN_CUH
#define FCG_SCAN_CUH

#include <cuda_runtime.h>
#include <stdint.h>

#include <algorithm>
#include <vector>

namespace fcg {
namespace devscan {
namespace {

constexpr int kThreads = 256;
constexpr int kDigits = 256;
constexpr int kItems = 8;
constexpr int kTile = kThreads * kItems;  // items per CTA in the tiled kernels
constexpr int kWarps = kThreads / 32;

// exclusive scan of one value per thread over the CTA; *total gets the sum
template <class T>
__device__ T block_exclusive_scan(T v, T *warp_tot, T *total) {
    int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    T x = v;
    for (int o = 1; o < 32; o <<= 1) {
        T y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= o) x += y;
    }
    if (lane == 31) warp_tot[w] = x;
    __syncthreads();
    if (w == 0) {
        T t = lane < kWarps ? warp_tot[lane] : T(0);
        for (int o = 1; o < 32; o <<= 1) {
            T y = __shfl_up_sync(0xffffffffu, t, o);
            if (lane >= o) t += y;
        }
        if (lane < kWarps) warp_tot[lane] = t;
    }
    __syncthreads();
    T before = w > 0 ? warp_tot[w - 1] : T(0);
    *total = warp_tot[kWarps - 1];
    __syncthreads();
    return before + x - v;
}

template <class T>
__device__ T block_sum(T v, T *warp_tot) {
    T total;
    block_exclusive_scan(v, warp_tot, &total);
    return total;
}

// ------------------------------------------------------------------ scans
// Three-phase exclusive scan: per-tile sums, one CTA scanning the tile sums,
// then every tile scanned again with its offset. In place is allowed.
template <class TI>
__global__ void __launch_bounds__(kThreads) k_scan_tiles(int64_t n, const TI *__restrict__ in, long long *sums) {
    __shared__ long long wt[32];
    int64_t base = (int64_t)blockIdx.x * kTile + (int64_t)threadIdx.x * kItems;
    long long s = 0;
    for (int j = 0; j < kItems; j++)
        if (base + j < n) s += (long long)in[base + j];
    s = block_sum(s, wt);
    if (threadIdx.x == 0) sums[blockIdx.x] = s;
}

__global__ void __launch_bounds__(1024) k_scan_sums(int64_t m, long long *sums, long long *total) {
    __shared__ long long wt[32];
    long long carry = 0;
    int lane = threadIdx.x & 31, w = threadIdx.x >> 5, nw = blockDim.x >> 5;
    for (int64_t b = 0; b < m; b += blockDim.x) {
        int64_t i = b + threadIdx.x;
        long long v = i < m ? sums[i] : 0;
        long long x = v;
        for (int o = 1; o < 32; o <<= 1) {
            long long y = __shfl_up_sync(0xffffffffu, x, o);
            if (lane >= o) x += y;
        }
        if (lane == 31) wt[w] = x;
        __syncthreads();
        if (w == 0) {
            long long t = lane < nw ? wt[lane] : 0;
            for (int o = 1; o < 32; o <<= 1) {
                long long y = __shfl_up_sync(0xffffffffu, t, o);
                if (lane >= o) t += y;
            }
            if (lane < nw) wt[lane] = t;
        }
        __syncthreads();
        long long before = w > 0 ? wt[w - 1] : 0;
        if (i < m) sums[i] = carry + before + x - v;
        carry += wt[nw - 1];
        __syncthreads();
    }
    if (threadIdx.x == 0) *total = carry;
}

template <class TI, class TO>
__global__ void __launch_bounds__(kThreads) k_scan_apply(int64_t n, const TI *in, TO *out, const long long *__restrict__ sums) {
    __shared__ long long wt[32];
    int64_t base = (int64_t)blockIdx.x * kTile + (int64_t)threadIdx.x * kItems;
    long long v[kItems], s = 0;
    for (int j = 0; j < kItems; j++) {
        v[j] = base + j < n ? (long long)in[base + j] : 0;
        s += v[j];
    }
    long long tot;
    long long run = block_exclusive_scan(s, wt, &tot) + sums[blockIdx.x];
    for (int j = 0; j < kItems; j++) {
        if (base + j < n) out[base + j] = (TO)run;
        run += v[j];
    }
}

inline unsigned grid_tiles(int64_t n) { return (unsigned)std::max<int64_t>((n + kTile - 1) / kTile, 1); }
inline unsigned grid_stride(int64_t n, int sms, int threads = 256) {
    return (unsigned)std::max<int64_t>(std::min<int64_t>((n + threads - 1) / threads, (int64_t)sms * 16), 1);
}

// exclusive scan of in[0..n) into out (in place allowed); the total goes to
// the device word *total. `sums` holds grid_tiles(n) words.
template <class TI, class TO>
inline void exclusive_scan(cudaStream_t s, int64_t n, const TI *in, TO *out, long long *sums, long long *total) {
    unsigned tiles = grid_tiles(n);
    k_scan_tiles<<<tiles, kThreads, 0, s>>>(n, in, sums);
    k_scan_sums<<<1, 1024, 0, s>>>(tiles, sums, total);
    k_scan_apply<<<tiles, kThreads, 0, s>>>(n, in, out, sums);
}

struct Bufs {
    cudaStream_t s = nullptr;
    std::vector<void *> live;
    ~Bufs() {
        if (!s) return;
        for (void *p : live) cudaFreeAsync(p, s);
        cudaStreamSynchronize(s);
        cudaStreamDestroy(s);
    }
    template <class T>
    cudaError_t alloc(T **p, size_t n) {
        *p = nullptr;
        cudaError_t e = cudaMallocAsync((void **)p, std::max<size_t>(n, 1) * sizeof(T), s);
        if (e == cudaSuccess) live.push_back(*p);
        return e;
    }
    template <class T>
    void release(T *&p) {
        if (!p) return;
        auto it = std::find(live.begin(), live.end(), (void *)p);
        if (it != live.end()) live.erase(it);
        cudaFreeAsync(p, s);
        p = nullptr;
    }
};

// digit histogram of one tile, digit-major: hist[digit * ntiles + tile]
__global__ void __launch_bounds__(kThreads) k_radix_hist(int64_t n, const unsigned long long *__restrict__ in, int shift, int *hist) {
    __shared__ int h[kDigits];
    h[threadIdx.x] = 0;
    __syncthreads();
    int64_t t0 = (int64_t)blockIdx.x * kTile;
    for (int j = threadIdx.x; j < kTile; j += kThreads) {
        int64_t i = t0 + j;
        if (i < n) atomicAdd(&h[(int)((in[i] >> shift) & 255)], 1);
    }
    __syncthreads();
    hist[(int64_t)threadIdx.x * gridDim.x + blockIdx.x] = h[threadIdx.x];
}

// stable scatter of one tile by digit. Warp w owns tile items
// [w*256, w*256+256) in eight rounds of 32 consecutive items, so (warp,
// round, lane) is the items' order; inside a round the lanes of one digit
// rank themselves with a warp match, across rounds a per-warp running count
// carries the order, across warps an exclusive prefix per digit.
__global__ void __launch_bounds__(kThreads) k_radix_scatter(int64_t n, const unsigned long long *__restrict__ in, int shift,
                                                            const int *__restrict__ hist_off, unsigned long long *out,
                                                            int32_t *out_src) {
    __shared__ int wcnt[kWarps][kDigits];
    for (int j = threadIdx.x; j < kWarps * kDigits; j += kThreads) (&wcnt[0][0])[j] = 0;
    __syncthreads();
    int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
    int64_t t0 = (int64_t)blockIdx.x * kTile + w * (32 * kItems);
    unsigned long long v[kItems];
    int pos[kItems], dg[kItems];
    for (int r = 0; r < kItems; r++) {
        int64_t i = t0 + r * 32 + lane;
        bool ok = i < n;
        v[r] = ok ? in[i] : 0ull;
        int d = ok ? (int)((v[r] >> shift) & 255) : kDigits + lane;  // lanes past the end match nobody
        unsigned m = __match_any_sync(0xffffffffu, d);
        int rk = __popc(m & ((1u << lane) - 1u));
        pos[r] = ok ? wcnt[w][d] + rk : 0;
        dg[r] = d;
        __syncwarp();
        if (ok && rk == 0) wcnt[w][d] += __popc(m);
        __syncwarp();
    }
    __syncthreads();
    {
        int run = 0;
        for (int ww = 0; ww < kWarps; ww++) {
            int c = wcnt[ww][threadIdx.x];
            wcnt[ww][threadIdx.x] = run;
            run += c;
        }
    }
    __syncthreads();
    for (int r = 0; r < kItems; r++) {
        int64_t i = t0 + r * 32 + lane;
        if (i >= n) break;
        int d = dg[r];
        int64_t dst = (int64_t)hist_off[(int64_t)d * gridDim.x + blockIdx.x] + wcnt[w][d] + pos[r];
        if (out_src) out_src[dst] = (int32_t)(uint32_t)(v[r] & 0xffffffffull);
        else out[dst] = v[r];
    }
}

}  // namespace
}  // namespace devscan
}  // namespace fcg

#endif
