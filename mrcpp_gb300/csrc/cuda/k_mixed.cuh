// Mixed-precision contraction (FP32 products, FP32 partial sums per band
// cell group, FP64 accumulation of the partial sums).
//
// Same screening and term/band selection as the FP64 kernel (k_apply.cu),
// restating ConvolutionCalculator.cpp:224-382; only the arithmetic of the
// component products changes.  One CTA per output node g, 256 threads.
//
// Work of one (f, term) pair is done in two groups of four f components:
//   stage 0  X0[ft][a0]     = O^x_{a0 b0}  applied along x to f_ft
//   stage 1  X1[ft][a0 a1]  = O^y_{a1 b1}  applied along y to X0[ft][a0]
//   stage 2  g[gt]         += O^z_{a2 b2}  applied along z to X1[ft][gt & 3]
// where only the (ft, gt) pairs the screening keeps are formed.  Each 1D
// application is MRCPP's out(K^2 x K) = in^T (K^2 x K) * O (K x K) step; the
// intermediates live in shared memory with rows padded to an odd number of
// 16-byte words (conflict-free float4 row loads), the g accumulators live in
// registers: thread t owns coefficients t + 256 m of the output node.
#pragma once

#include "mwgpu_internal.cuh"

namespace mwgpu {
namespace mixed {

__host__ __device__ constexpr int padded_row(int K) {
    int p = (K + 3) / 4 * 4;
    if ((p / 4) % 2 == 0) p += 4;
    return p;
}

template <int K>
struct Shape {
    static constexpr int K2 = K * K;
    static constexpr int K3 = K * K * K;
    static constexpr int P = padded_row(K);
    static constexpr int BLK = P * K2;                  // one padded K^3 block
    static constexpr int NOUT = (8 * K3 + 255) / 256;    // accumulators per thread
    static constexpr int SMEM_FLOATS = 4 * 2 * BLK + 4 * 4 * BLK + 12 * K2;
};

// out (padded) = apply O along the row axis of `in` (row stride IS), for the
// applies listed in `list` (count n, each entry: in block ptr, out block, O ptr).
template <int K, int IS>
__device__ __forceinline__ void apply_rows(float *__restrict__ out, const float *__restrict__ in, const float *__restrict__ O, int e) {
    using S = Shape<K>;
    // element e of the output block: c = e % K2 (row of in), j = e / K2
    const int c = e % S::K2, j = e / S::K2;
    const float *a = in + IS * c;
    const float *b = O + K * j;
    float s = 0.f;
#pragma unroll
    for (int i = 0; i < K; i++) s = fmaf(a[i], b[i], s);
    // next layout: row (c_hi + K j), position c_lo, row stride P
    const int c_lo = c % K, c_hi = c / K;
    out[c_lo + S::P * (c_hi + K * j)] = s;
}

template <int K>
__global__ void __launch_bounds__(256) k_contract_mixed(DevMRA m, DevOper op, DevTree f, DevTree g, const int *work, int n_work,
                                                        double gthr, LevelStats *stats, int *err) {
    using S = Shape<K>;
    constexpr int K2 = S::K2, K3 = S::K3, P = S::P, BLK = S::BLK, NOUT = S::NOUT;
    extern __shared__ float smf[];
    float *X0 = smf;                  // [4 ft][2 a0] padded blocks
    float *X1 = X0 + 8 * BLK;         // [4 ft][4 (a0,a1)] padded blocks
    float *OB = X1 + 16 * BLK;        // [3 dirs][4 comps] K*K
    __shared__ int s_fid;
    __shared__ double s_fn[8];
    __shared__ unsigned s_mask[2];
    __shared__ unsigned long long s_nt, s_nc;
    const int tid = threadIdx.x;
    const int gi = work[blockIdx.x];
    const int4 gx = g.idx[gi];
    float acc[NOUT];
    double acc64[NOUT];
#pragma unroll
    for (int q = 0; q < NOUT; q++) { acc[q] = 0.f; acc64[q] = 0.0; }
    if (tid == 0) { s_nt = 0; s_nc = 0; }
    __syncthreads();
    const int depth = gx.x - m.root_scale;
    const int w = (depth >= 0 && depth < op.n_band_max) ? op.band_max[depth] : -1;
    unsigned long long nband = 0;
    if (w >= 0 && depth < kMaxDepthRows) {
        int bs[3], be[3], tot = 1;
        const int gl[3] = {gx.y, gx.z, gx.w};
        for (int d = 0; d < 3; d++) {
            int nboxes = m.nbox[d] * (1 << depth), c = m.corner[d] * (1 << depth);
            bs[d] = max(gl[d] - w, c);
            be[d] = min(gl[d] + w, c + nboxes - 1);
            tot *= max(0, be[d] - bs[d] + 1);
        }
        const int nx = be[0] - bs[0] + 1, ny = be[1] - bs[1] + 1;
        const int T = op.n_terms;
        int since_flush = 0;
        for (int q = 0; q < tot; q++) {
            const int fx = bs[0] + q % nx, fy = bs[1] + (q / nx) % ny, fz = bs[2] + q / (nx * ny);
            if (tid == 0) {
                uint64_t key;
                int id = -1;
                if (pack_key(m, gx.x, fx, fy, fz, key)) id = hash_find(f.hkeys, f.hvals, f.hcap, key);
                if (id < 0) atomicOr(err, DE_LOOKUP);
                s_fid = id;
                if (id >= 0)
                    for (int c = 0; c < 8; c++) s_fn[c] = f.norms[(size_t)id * 8 + c];
            }
            __syncthreads();
            const int fid = s_fid;
            if (fid >= 0) {
                nband++;
                const int tl[3] = {fx - gx.y, fy - gx.z, fz - gx.w};
                const int maxdl = max(abs(tl[0]), max(abs(tl[1]), abs(tl[2])));
                const bool gen = fid >= f.cap_real;
                const float *fc = gen ? f.gcoefs32 + (size_t)(fid - f.cap_real) * K3 : f.coefs32 + (size_t)fid * 8 * K3;
                for (int ti = 0; ti < T; ti++) {
                    const int i = op.term_order[depth * T + ti];
                    const int *bwi = op.bw + ((size_t)i * op.max_rows + depth) * 5;
                    if (maxdl > bwi[4]) break;
                    if (tid < 64) {
                        const int ft = tid >> 3, gt = tid & 7;
                        bool pass = true;
                        const double fNorm = s_fn[ft];
                        if (fNorm < kMachineZero) pass = false;
                        if (depth != 0 && ft == 0 && gt == 0) pass = false;
                        double oNorm = 1.0;
                        if (pass) {
                            for (int d = 0; d < 3; d++) {
                                const int a = (gt >> d) & 1, bb = (ft >> d) & 1, idx = 2 * a + bb;
                                if (abs(tl[d]) > bwi[idx]) { pass = false; break; }
                                const int node = op.dep_off[i * op.max_rows + depth] + tl[d] + op.dep_L[i * op.max_rows + depth];
                                oNorm *= op.norms[(size_t)node * 4 + idx];
                            }
                        }
                        if (pass) {
                            const double fThr = (double)op.band_size[((size_t)i * kMaxDepthRows + depth) * 64 + gt * 8 + ft] * fNorm;
                            pass = oNorm * fThr > gthr;
                        }
                        unsigned bal = __ballot_sync(0xffffffffu, pass);
                        if ((tid & 31) == 0) s_mask[tid >> 5] = bal;
                    }
                    // operator blocks of the three directions
                    {
                        const int L0 = op.dep_L[i * op.max_rows + depth], off = op.dep_off[i * op.max_rows + depth];
                        for (int e = tid; e < 12 * K2; e += 256) {
                            const int d = e / (4 * K2), r = e % (4 * K2);
                            const int l = tl[d];
                            float v = 0.f;
                            if (off >= 0 && abs(l) <= L0) v = op.blocks32[(size_t)(off + l + L0) * 4 * K2 + r];
                            OB[e] = v;
                        }
                    }
                    __syncthreads();
                    const unsigned long long mask = (unsigned long long)s_mask[0] | ((unsigned long long)s_mask[1] << 32);
                    if (mask != 0ull) {
                        if (tid == 0) { s_nt++; s_nc += __popcll(mask); }
                        for (int grp = 0; grp < 2; grp++) {
                            const unsigned gmask = (unsigned)((mask >> (32 * grp)) & 0xffffffffull);
                            if (gmask == 0) continue;
                            // stage 0: X0[lft][a0] for needed (ft, a0)
                            // needed bit sets per local ft
                            for (int e = tid; e < 8 * K3; e += 256) {
                                const int ap = e / K3, el = e % K3;
                                const int lft = ap >> 1, a0 = ap & 1, ft = 4 * grp + lft;
                                const unsigned col = (gmask >> (8 * lft)) & 0xffu;
                                const unsigned need = (a0 ? 0xAAu : 0x55u);  // gt with gt&1 == a0
                                if (!(col & need)) continue;
                                apply_rows<K, K>(X0 + ap * BLK, fc + (size_t)ft * K3, OB + 0 * 4 * K2 + (2 * a0 + (ft & 1)) * K2, el);
                            }
                            __syncthreads();
                            // stage 1: X1[lft][s], s = a0 + 2 a1
                            for (int e = tid; e < 16 * K3; e += 256) {
                                const int ap = e / K3, el = e % K3;
                                const int lft = ap >> 2, s = ap & 3, ft = 4 * grp + lft;
                                const unsigned col = (gmask >> (8 * lft)) & 0xffu;
                                const unsigned need = (1u << s) | (1u << (s + 4));
                                if (!(col & need)) continue;
                                apply_rows<K, P>(X1 + ap * BLK, X0 + (lft * 2 + (s & 1)) * BLK, OB + 1 * 4 * K2 + (2 * (s >> 1) + ((ft >> 1) & 1)) * K2, el);
                            }
                            __syncthreads();
                            // stage 2: thread-owned g coefficients e = tid + 256 q
#pragma unroll
                            for (int qq = 0; qq < NOUT; qq++) {
                                const int e = tid + 256 * qq;
                                if (e >= 8 * K3) break;
                                const int gt = e / K3, el = e % K3;
                                const int c = el % K2, j = el / K2;
                                float s = 0.f;
#pragma unroll
                                for (int lft = 0; lft < 4; lft++) {
                                    const int ft = 4 * grp + lft;
                                    if (!((gmask >> (8 * lft + gt)) & 1u)) continue;
                                    const float *a = X1 + (lft * 4 + (gt & 3)) * BLK + P * c;
                                    const float *b = OB + 2 * 4 * K2 + (2 * (gt >> 2) + (ft >> 2)) * K2 + K * j;
#pragma unroll
                                    for (int ii = 0; ii < K; ii++) s = fmaf(a[ii], b[ii], s);
                                }
                                acc[qq] += s;
                            }
                            __syncthreads();
                        }
                    } else {
                        __syncthreads();
                    }
                }
                if (++since_flush >= 8) {
#pragma unroll
                    for (int qq = 0; qq < NOUT; qq++) { acc64[qq] += (double)acc[qq]; acc[qq] = 0.f; }
                    since_flush = 0;
                }
            }
            __syncthreads();  // s_fid / s_fn rewritten next cell
        }
    }
    double *go = g.coefs + (size_t)gi * 8 * K3;
#pragma unroll
    for (int qq = 0; qq < NOUT; qq++) {
        const int e = tid + 256 * qq;
        if (e >= 8 * K3) break;
        go[e] = acc64[qq] + (double)acc[qq];
    }
    __syncthreads();
    // node norms (MWNode::calcNorms) from the stored FP64 coefficients
    __shared__ double red[8][8];
    for (int comp = 0; comp < 8; comp++) {
        double s = 0.0;
        for (int e = tid; e < K3; e += 256) { double v = go[comp * K3 + e]; s += v * v; }
        for (int o = 16; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o);
        if ((tid & 31) == 0) red[comp][tid >> 5] = s;
    }
    __syncthreads();
    if (tid < 8) {
        double t = 0.0;
        for (int wv = 0; wv < 8; wv++) t += red[tid][wv];
        g.norms[(size_t)gi * 8 + tid] = sqrt(t);
    }
    if (tid == 0) {
        atomicAdd(&stats->node_terms, s_nt);
        atomicAdd(&stats->components, s_nc);
        atomicAdd(&stats->band_nodes, nband);
    }
}

}  // namespace mixed
}  // namespace mwgpu
