// Device side of the judged adaptive apply: the bookkeeping of
// TreeBuilder::build (TreeBuilder.cpp:38-87) for a proposed output grid, one
// level after another without returning to the host.
//
// The proposal holds the output nodes level by level; flags[i] bit 0 = node i
// belongs to the judged tree (the roots, and the children of nodes the split
// test refined), bit 1 = the split test refined node i.  Per level:
//   k_compact      work list = kept nodes of the level, in proposal order (the
//                  order in which TreeBuilder creates them)
//   k_cells        band pairs per work entry
//   k_threshold    gThreshold from the tree norm of the levels before
//   ... work list, contraction and reduction as for every level ...
//   k_level_norm   sNorm (first level) and the running wNorm, added in work
//                  order like TreeBuilder, and the tree norm
//   k_judge        split_check (tree_utils.cpp:47-65) of every computed node;
//                  a refined node keeps its proposed children, or marks the
//                  level as missed when it has none
#include <algorithm>

#include "mwgpu_internal.cuh"

namespace mwgpu {

namespace {

__global__ void k_keep_counts(const int *flags, int begin, int n, int *cnt) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) cnt[i] = flags[begin + i] & 1;
}

// koff: exclusive scan of the keep bits of the level (koff[n] = total)
__global__ void k_compact(const int *flags, int begin, int n, const long long *koff, int *work, int *n_work) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n && (flags[begin + i] & 1)) work[koff[i]] = begin + i;
    if (i == 0) *n_work = (int)koff[n];
}

__global__ void k_cells(const int *work, const int *n_work, int cap, const int *cells, int *cnt) {
    const int wi = blockIdx.x * blockDim.x + threadIdx.x;
    if (wi < cap) cnt[wi] = wi < *n_work ? cells[work[wi]] : 0;
}

// ConvolutionCalculator::calcNode gThreshold (:241-248) from the tree norm
__global__ void k_threshold(const double *sq, double prec, int n_terms, double *gthr) {
    double g = *sq;
    if (g > 0.0) g = __dmul_rn(__dmul_rn(prec, 1.0), sqrt(__ddiv_rn(g, (double)n_terms)));
    *gthr = g;
}

// Tree<3>::scalingNorm / waveletNorm of the host, operation by operation
// (explicitly rounded products and sums: no fused multiply-add, like the host
// build), so that the judge decides exactly as the host split test would.
__device__ inline double scaling_norm(const double *nrm) {
    const double s = nrm[0];
    return s >= 0 ? __dmul_rn(s, s) : -1.0;
}

__device__ inline double wavelet_norm(const double *nrm) {
    double w = 0.0;
    for (int c = 1; c < 8; c++) {
        const double v = nrm[c];
        if (v >= 0.0) w = __dadd_rn(w, __dmul_rn(v, v));
        else w = -1.0;
    }
    return w;
}

// state[0] sNorm, state[1] wNorm, state[2] tree norm (also copied to
// sq_level[0..3) of the level); node_terms += items of the level
constexpr int kNormBlock = 1024;
__global__ void __launch_bounds__(kNormBlock) k_level_norm(DevTree g, const int *work, const int *n_work, int first_level, double *state,
                                                           double *sq_level, const long long *g_off, unsigned long long *node_terms) {
    __shared__ double s_sn[kNormBlock], s_wn[kNormBlock];
    const int n = *n_work;
    double sNorm = first_level ? 0.0 : state[0], wNorm = state[1];
    for (int b = 0; b < n; b += kNormBlock) {
        const int i = b + threadIdx.x;
        if (i < n) {
            const double *nrm = g.norms + (size_t)work[i] * 8;
            s_sn[threadIdx.x] = scaling_norm(nrm);
            s_wn[threadIdx.x] = wavelet_norm(nrm);
        }
        __syncthreads();
        if (threadIdx.x == 0) {
            const int e = min(kNormBlock, n - b);
            for (int k = 0; k < e; k++) {
                if (first_level) sNorm = __dadd_rn(sNorm, s_sn[k]);
                wNorm = __dadd_rn(wNorm, s_wn[k]);
            }
        }
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        state[0] = sNorm;
        state[1] = wNorm;
        const double sq = (sNorm < 0.0 || wNorm < 0.0) ? -1.0 : __dadd_rn(sNorm, wNorm);
        state[2] = sq;
        sq_level[0] = sNorm;
        sq_level[1] = wNorm;
        sq_level[2] = sq;
        if (node_terms && g_off) *node_terms += (unsigned long long)g_off[n];
    }
}

// split_check (tree_utils.cpp:47-65) with splitFac = 1; scale_fac[d] =
// 2^(-(n+1)/2) for scale n = root_scale + d (computed on the host)
__global__ void k_judge(DevMRA m, DevTree g, const int *work, const int *n_work, int cap, const double *state, double prec, int abs_prec,
                        const double *scale_fac, int max_scale, int *flags, int level, int *first_miss) {
    const int wi = blockIdx.x * blockDim.x + threadIdx.x;
    if (wi >= cap || wi >= *n_work) return;
    const int i = work[wi];
    const int n = g.idx[i].x;
    if (n + 2 > max_scale) return;
    bool split = false;
    if (prec > 0.0) {
        double t_norm = 1.0;
        const double sq = state[2];
        if (sq > 0.0 && !abs_prec) t_norm = sqrt(sq);
        const double w_thrs = fmax(2.0 * 1.0e-15, __dmul_rn(__dmul_rn(prec, t_norm), scale_fac[n - m.root_scale]));
        const double w_norm = sqrt(wavelet_norm(g.norms + (size_t)i * 8));
        split = w_norm > w_thrs;
    }
    if (!split) return;
    flags[i] |= 2;
    const int c0 = g.child0[i];
    if (c0 < 0) {
        atomicMin(first_miss, level);
        return;
    }
    for (int c = 0; c < 8; c++) flags[c0 + c] |= 1;
}

}  // namespace

void launch_keep_counts(const int *flags, int begin, int n, int *cnt, cudaStream_t s) {
    if (n > 0) k_keep_counts<<<(n + 255) / 256, 256, 0, s>>>(flags, begin, n, cnt);
}

void launch_compact(const int *flags, int begin, int n, const long long *koff, int *work, int *n_work, cudaStream_t s) {
    k_compact<<<(std::max(n, 1) + 255) / 256, 256, 0, s>>>(flags, begin, n, koff, work, n_work);
}

void launch_cells(const int *work, const int *n_work, int cap, const int *cells, int *cnt, cudaStream_t s) {
    if (cap > 0) k_cells<<<(cap + 255) / 256, 256, 0, s>>>(work, n_work, cap, cells, cnt);
}

void launch_threshold(const double *sq, double prec, int n_terms, double *gthr, cudaStream_t s) {
    k_threshold<<<1, 1, 0, s>>>(sq, prec, n_terms, gthr);
}

void launch_level_norm(const DevTree &g, const int *work, const int *n_work, int first_level, double *state, double *sq_level,
                       const long long *g_off, unsigned long long *node_terms, cudaStream_t s) {
    k_level_norm<<<1, kNormBlock, 0, s>>>(g, work, n_work, first_level, state, sq_level, g_off, node_terms);
}

void launch_judge(const DevMRA &m, const DevTree &g, const int *work, const int *n_work, int cap, const double *state, double prec, int abs_prec,
                  const double *scale_fac, int max_scale, int *flags, int level, int *first_miss, cudaStream_t s) {
    if (cap > 0)
        k_judge<<<(cap + 255) / 256, 256, 0, s>>>(m, g, work, n_work, cap, state, prec, abs_prec, scale_fac, max_scale, flags, level, first_miss);
}

}  // namespace mwgpu
