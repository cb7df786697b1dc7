// Super hierarchy on the GPU: CAutoRefine::BuildSuperHierarchy /
// RecurBuild3DSuperHier (Solver/Autorefine.cpp:6410-6629) with
// CAutoPanel::MakeSuperPanel (Solver/AutoPanel.cpp:209-379).
//
// The host recursion splits a conductor's panel set by the mid-plane of the
// bounding box of its panel centroids, across the box's longest side
// (centroid coordinate <= mid goes left), and recurses on both halves; a
// one-panel set is a leaf, a split that leaves one half empty is an error
// (coincident centroids). The tree depends only on the sets: the box, its
// longest side, the mid-plane and each centroid's side do not depend on the
// order of the panels. So every segment of a level is split at once:
//   box      per segment, min/max of the centroids (float atomics on an
//            order-preserving integer encoding: exact, order-free)
//   split    per segment, the longest side and the mid-plane in FP64 as the
//            host computes them
//   count    per panel, its side; per segment, the left count
//   children per segment, two child nodes (and segments for children of more
//            than one panel); the split node gets its super-node element id
//   scatter  every panel to its child segment (positions inside a segment
//            are taken by atomics: any order gives the same sets)
// then the super nodes are made bottom up, one level per launch, by the
// host builder's own fcg_make_super (compiled here with -fmad=false, the host
// with -ffp-contract=off: the same elements bit for bit). Element ids differ
// from the host builder's, the tree does not; the flattened model is the same.
#include <cuda_runtime.h>
#include <stdint.h>
#include <stdio.h>

#include <algorithm>
#include <string>
#include <vector>

#include "fc_potential.h"
#include "fcg_internal.hpp"
#include "scan.cuh"
#include "../host/model.hpp"

namespace fcg {
namespace {

using devscan::Bufs;

// order-preserving encoding of a float as a signed integer (for atomicMin/Max)
__device__ __forceinline__ int f2ord(float f) {
    int i = __float_as_int(f);
    return i >= 0 ? i : i ^ 0x7fffffff;
}
__device__ __forceinline__ float ord2f(int i) { return __int_as_float(i >= 0 ? i : i ^ 0x7fffffff); }

struct SegArrays {
    int32_t *first, *n, *node;
};

__global__ void k_box_init(int nseg, int *bb) {
    int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= nseg) return;
    for (int d = 0; d < 3; d++) {
        bb[s * 6 + d] = 0x7fffffff;       // min
        bb[s * 6 + 3 + d] = (int)0x80000000;  // max
    }
}

__global__ void k_box(int64_t n, const int32_t *__restrict__ perm, const int32_t *__restrict__ segof, const Element *__restrict__ el,
                      int *bb) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const int s = segof[i];
        if (s < 0) continue;
        const float *c = el[perm[i]].c;
        for (int d = 0; d < 3; d++) {
            const int o = f2ord(c[d]);
            atomicMin(&bb[s * 6 + d], o);
            atomicMax(&bb[s * 6 + 3 + d], o);
        }
    }
}

// the host's BBox::max_side and mid-plane: sides compared in FP64 (x on
// ties with y and z, then y on a tie with z), mid = (max + min) / 2
__global__ void k_split(int nseg, const int *__restrict__ bb, int8_t *mc, double *mid, int32_t *left, int32_t *lcur, int32_t *rcur) {
    int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= nseg) return;
    double mn[3], mx[3];
    for (int d = 0; d < 3; d++) {
        mn[d] = (double)ord2f(bb[s * 6 + d]);
        mx[d] = (double)ord2f(bb[s * 6 + 3 + d]);
    }
    const double dx = mx[0] - mn[0], dy = mx[1] - mn[1], dz = mx[2] - mn[2];
    const int m = (dx >= dy && dx >= dz) ? 0 : (dy >= dz ? 1 : 2);
    mc[s] = (int8_t)m;
    mid[s] = (mx[m] + mn[m]) / 2.0;
    left[s] = 0;
    lcur[s] = 0;
    rcur[s] = 0;
}

__global__ void k_count(int64_t n, const int32_t *__restrict__ perm, const int32_t *__restrict__ segof, const Element *__restrict__ el,
                        const int8_t *__restrict__ mc, const double *__restrict__ mid, int32_t *left) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const int s = segof[i];
        if (s < 0) continue;
        if ((double)el[perm[i]].c[mc[s]] <= mid[s]) atomicAdd(&left[s], 1);
    }
}

// per segment: its node becomes internal (gets its super node's element id)
// with two child nodes; children of more than one panel become next-level
// segments. ctr: [0] next segments, [1] nodes, [2] super nodes, [3] error
__global__ void k_children(int nseg, SegArrays cur, SegArrays nxt, const int32_t *__restrict__ left, int32_t *cseg, int32_t *nleft,
                           int32_t *nright, int32_t *nelem, int32_t *nlevel, int level, int32_t elem_base, int *ctr) {
    int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= nseg) return;
    const int nl = left[s], nn = cur.n[s], q = cur.node[s];
    if (nl == 0 || nl == nn) {
        atomicOr(&ctr[3], 1);
        cseg[2 * s] = cseg[2 * s + 1] = -1;
        return;
    }
    const int ql = atomicAdd(&ctr[1], 2), qr = ql + 1;
    nleft[q] = ql;
    nright[q] = qr;
    nelem[q] = elem_base + atomicAdd(&ctr[2], 1);
    nleft[ql] = nright[ql] = nleft[qr] = nright[qr] = -1;
    nlevel[ql] = nlevel[qr] = level + 1;
    const int cf[2] = {cur.first[s], cur.first[s] + nl}, cn[2] = {nl, nn - nl}, cq[2] = {ql, qr};
    for (int h = 0; h < 2; h++) {
        if (cn[h] == 1) {
            cseg[2 * s + h] = -1 - cq[h];  // a leaf child: its node, encoded
        } else {
            const int t = atomicAdd(&ctr[0], 1);
            nxt.first[t] = cf[h];
            nxt.n[t] = cn[h];
            nxt.node[t] = cq[h];
            cseg[2 * s + h] = t;
        }
    }
}

__global__ void k_scatter(int64_t n, const int32_t *__restrict__ perm, const int32_t *__restrict__ segof, const Element *__restrict__ el,
                          SegArrays cur, const int8_t *__restrict__ mc, const double *__restrict__ mid,
                          const int32_t *__restrict__ left, int32_t *lcur, int32_t *rcur, const int32_t *__restrict__ cseg,
                          int32_t *perm2, int32_t *segof2, int32_t *nelem) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const int s = segof[i];
        if (s < 0) {
            perm2[i] = perm[i];
            segof2[i] = -1;
            continue;
        }
        const int32_t id = perm[i];
        const bool l = (double)el[id].c[mc[s]] <= mid[s];
        const int64_t pos = l ? cur.first[s] + atomicAdd(&lcur[s], 1) : cur.first[s] + left[s] + atomicAdd(&rcur[s], 1);
        const int c = cseg[2 * s + (l ? 0 : 1)];
        perm2[pos] = id;
        if (c >= 0) {
            segof2[pos] = c;
        } else {
            segof2[pos] = -1;
            nelem[-1 - c] = id;  // a one-panel child: a leaf
        }
    }
}

// the super nodes of one level, children first (they are one level deeper)
__global__ void k_make(int64_t nq, const int32_t *__restrict__ nlevel, const int32_t *__restrict__ nleft,
                       const int32_t *__restrict__ nright, const int32_t *__restrict__ nelem, int level, Element *el) {
    for (int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; q < nq; q += (int64_t)gridDim.x * blockDim.x) {
        if (nlevel[q] != level || nleft[q] < 0) continue;
        const int32_t lid = nelem[nleft[q]], rid = nelem[nright[q]];
        Element e;
        fcg_make_super(el[lid], el[rid], lid, rid, e);
        el[nelem[q]] = e;
    }
}

int grid_for_n(int64_t n, int sms) { return (int)std::max<int64_t>(1, std::min<int64_t>((n + 255) / 256, (int64_t)sms * 8)); }

}  // namespace

#define SB_CK(x)                                                                                     \
    do {                                                                                             \
        cudaError_t e_ = (x);                                                                        \
        if (e_ != cudaSuccess) {                                                                     \
            err = std::string("device super hierarchy: ") + cudaGetErrorString(e_);                 \
            cudaGetLastError();                                                                      \
            return e_ == cudaErrorMemoryAllocation ? FCG_OUT_OF_MEMORY : FCG_DEVICE_ERROR;           \
        }                                                                                            \
    } while (0)

int super_build_device(DeviceContext &ctx, std::vector<Element> &el, const std::vector<std::vector<int32_t>> &panels,
                       std::vector<int32_t> &tops, int max_depth, std::string &err) {
    SB_CK(cudaSetDevice(ctx.device));
    Bufs B;
    SB_CK(cudaStreamCreateWithFlags(&B.s, cudaStreamNonBlocking));
    cudaStream_t s = B.s;
    const int sms = ctx.sm_count > 0 ? ctx.sm_count : 1;
    const int nc = (int)panels.size();
    std::vector<int32_t> h_perm, h_segof;
    std::vector<int32_t> h_first, h_n, h_node;
    int64_t n = 0, n_super = 0;
    for (int k = 0; k < nc; k++) {
        const int64_t nk = (int64_t)panels[k].size();
        if (nk >= 2) {
            h_first.push_back((int32_t)n);
            h_n.push_back((int32_t)nk);
            h_node.push_back(k);
        }
        for (int32_t id : panels[k]) {
            h_perm.push_back(id);
            h_segof.push_back(nk >= 2 ? (int32_t)h_first.size() - 1 : -1);
        }
        n += nk;
        n_super += nk - 1;
    }
    const int64_t ne = (int64_t)el.size(), nq = 2 * n - nc;
    if (ne + n_super > 0x7fffffffLL) { err = "model too large for 32-bit element ids"; return FCG_OUT_OF_MEMORY; }
    Element *d_el;
    int32_t *d_perm, *d_perm2, *d_segof, *d_segof2, *d_cseg, *d_left, *d_lcur, *d_rcur;
    int32_t *d_nleft, *d_nright, *d_nelem, *d_nlevel;
    int *d_bb, *d_ctr;
    int8_t *d_mc;
    double *d_mid;
    SegArrays cur, nxt;
    const size_t segcap = (size_t)std::max<int64_t>(n, 1);
    SB_CK(B.alloc(&d_el, (size_t)(ne + n_super)));
    SB_CK(B.alloc(&d_perm, (size_t)n));
    SB_CK(B.alloc(&d_perm2, (size_t)n));
    SB_CK(B.alloc(&d_segof, (size_t)n));
    SB_CK(B.alloc(&d_segof2, (size_t)n));
    SB_CK(B.alloc(&d_cseg, 2 * segcap));
    SB_CK(B.alloc(&d_left, segcap));
    SB_CK(B.alloc(&d_lcur, segcap));
    SB_CK(B.alloc(&d_rcur, segcap));
    SB_CK(B.alloc(&d_mc, segcap));
    SB_CK(B.alloc(&d_mid, segcap));
    SB_CK(B.alloc(&d_bb, 6 * segcap));
    SB_CK(B.alloc(&cur.first, segcap));
    SB_CK(B.alloc(&cur.n, segcap));
    SB_CK(B.alloc(&cur.node, segcap));
    SB_CK(B.alloc(&nxt.first, segcap));
    SB_CK(B.alloc(&nxt.n, segcap));
    SB_CK(B.alloc(&nxt.node, segcap));
    SB_CK(B.alloc(&d_nleft, (size_t)nq));
    SB_CK(B.alloc(&d_nright, (size_t)nq));
    SB_CK(B.alloc(&d_nelem, (size_t)nq));
    SB_CK(B.alloc(&d_nlevel, (size_t)nq));
    SB_CK(B.alloc(&d_ctr, 4));
    // roots: node k is conductor k's top; a one-panel conductor's top is its panel
    std::vector<int32_t> h_rl(nc, -1), h_elem(nc, -1), h_lvl(nc, 0);
    for (int k = 0; k < nc; k++)
        if (panels[k].size() == 1) h_elem[k] = panels[k][0];
    SB_CK(cudaMemcpyAsync(d_el, el.data(), (size_t)ne * sizeof(Element), cudaMemcpyHostToDevice, s));
    SB_CK(cudaMemcpyAsync(d_perm, h_perm.data(), (size_t)n * sizeof(int32_t), cudaMemcpyHostToDevice, s));
    SB_CK(cudaMemcpyAsync(d_segof, h_segof.data(), (size_t)n * sizeof(int32_t), cudaMemcpyHostToDevice, s));
    int nseg = (int)h_first.size();
    if (nseg > 0) {
        SB_CK(cudaMemcpyAsync(cur.first, h_first.data(), nseg * sizeof(int32_t), cudaMemcpyHostToDevice, s));
        SB_CK(cudaMemcpyAsync(cur.n, h_n.data(), nseg * sizeof(int32_t), cudaMemcpyHostToDevice, s));
        SB_CK(cudaMemcpyAsync(cur.node, h_node.data(), nseg * sizeof(int32_t), cudaMemcpyHostToDevice, s));
    }
    SB_CK(cudaMemcpyAsync(d_nleft, h_rl.data(), nc * sizeof(int32_t), cudaMemcpyHostToDevice, s));
    SB_CK(cudaMemcpyAsync(d_nright, h_rl.data(), nc * sizeof(int32_t), cudaMemcpyHostToDevice, s));
    SB_CK(cudaMemcpyAsync(d_nelem, h_elem.data(), nc * sizeof(int32_t), cudaMemcpyHostToDevice, s));
    SB_CK(cudaMemcpyAsync(d_nlevel, h_lvl.data(), nc * sizeof(int32_t), cudaMemcpyHostToDevice, s));
    const int h_ctr0[4] = {0, nc, 0, 0};
    SB_CK(cudaMemcpyAsync(d_ctr, h_ctr0, sizeof h_ctr0, cudaMemcpyHostToDevice, s));
    const int gn = grid_for_n(n, sms);
    int level = 0;
    while (nseg > 0) {
        if (level > max_depth) { err = "super hierarchy too deep (coincident panel centroids?)"; return FCG_FILE_ERROR; }
        const int gs = (nseg + 127) / 128;
        SB_CK(cudaMemsetAsync(d_ctr, 0, sizeof(int), s));  // next-level segments
        k_box_init<<<gs, 128, 0, s>>>(nseg, d_bb);
        k_box<<<gn, 256, 0, s>>>(n, d_perm, d_segof, d_el, d_bb);
        k_split<<<gs, 128, 0, s>>>(nseg, d_bb, d_mc, d_mid, d_left, d_lcur, d_rcur);
        k_count<<<gn, 256, 0, s>>>(n, d_perm, d_segof, d_el, d_mc, d_mid, d_left);
        k_children<<<gs, 128, 0, s>>>(nseg, cur, nxt, d_left, d_cseg, d_nleft, d_nright, d_nelem, d_nlevel, level, (int32_t)ne, d_ctr);
        k_scatter<<<gn, 256, 0, s>>>(n, d_perm, d_segof, d_el, cur, d_mc, d_mid, d_left, d_lcur, d_rcur, d_cseg, d_perm2, d_segof2,
                                     d_nelem);
        SB_CK(cudaGetLastError());
        int h_ctr[4];
        SB_CK(cudaMemcpyAsync(h_ctr, d_ctr, sizeof h_ctr, cudaMemcpyDeviceToHost, s));
        SB_CK(cudaStreamSynchronize(s));
        if (h_ctr[3]) { err = "panels with coincident centroids cannot be split into a hierarchy"; return FCG_FILE_ERROR; }
        std::swap(d_perm, d_perm2);
        std::swap(d_segof, d_segof2);
        std::swap(cur, nxt);
        nseg = h_ctr[0];
        level++;
    }
    // super nodes bottom up: level L's nodes have their children at L + 1
    const int gq = grid_for_n(nq, sms);
    for (int L = level - 1; L >= 0; L--) k_make<<<gq, 128, 0, s>>>(nq, d_nlevel, d_nleft, d_nright, d_nelem, L, d_el);
    SB_CK(cudaGetLastError());
    el.resize((size_t)(ne + n_super));
    if (n_super > 0)
        SB_CK(cudaMemcpyAsync(el.data() + ne, d_el + ne, (size_t)n_super * sizeof(Element), cudaMemcpyDeviceToHost, s));
    tops.assign(nc, -1);
    SB_CK(cudaMemcpyAsync(tops.data(), d_nelem, nc * sizeof(int32_t), cudaMemcpyDeviceToHost, s));
    SB_CK(cudaStreamSynchronize(s));
    return FCG_NORMAL_END;
}

}  // namespace fcg
