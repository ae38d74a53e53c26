// Mixed-precision contraction over a work list (FP32 products and FP32 partial
// sums, FP64 accumulation of the partial sums every 16 work items).
//
// One CTA (256 threads = 8 warps) per chunk of the work items of one output
// node g (k_worklist.cu makes the items; the screening of
// ConvolutionCalculator.cpp:224-329 is already in each item's (ft, gt)
// mask).  Two schedules produce the same sum of component products as
// tensorApplyOperComp (ConvolutionCalculator.cpp:333-382):
//
// * block schedule (the mask is the full structural set: every component the
//   band and zero-norm rules allow): the three 1D applications are summed over
//   the input bit of each direction,
//     Y0[a0 b1 b2] = sum_b0 O^x_{a0 b0} f[b0 b1 b2]
//     Y1[a0 a1 b2] = sum_b1 O^y_{a1 b1} Y0[a0 b1 b2]
//     g [a0 a1 a2] += sum_b2 O^z_{a2 b2} Y1[a0 a1 b2]
//   (48 K^4 FMA for a full node instead of 3 K^4 per component), with the
//   s->s product that the reference leaves out at depth > 0 (ft = gt = 0,
//   :261) carried in a separate channel U -> P and dropped at the end;
// * component schedule (a partial mask, from the norm screening): per group of
//   four f components the x and xy intermediates the kept (ft, gt) pairs need.
//
// Every step is one output block out(K^2 x K) = sum_p in_p^T (K^2 x K) O_p (K x K)
// (MRCPP's 1D application).  A warp computes one output block: lane l owns the
// rows c = l + 32 r, keeps a group of JG operator columns in registers and
// reads its rows with vector loads.  Intermediates live in shared memory with
// rows padded to an odd number of 16-byte words.  Warp w accumulates output
// component gt = w of g in registers (lane l: rows l + 32 r, all K columns).
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
    static constexpr int BLK = P * K2;                   // one padded K^3 block
    static constexpr int R = (K2 + 31) / 32;             // rows per lane
    static constexpr int JG = K <= 8 ? (K % 4 == 0 ? 4 : (K % 2 == 0 ? K / 2 : K)) : 2;  // operator columns held in registers
    static constexpr int NBUF = 24;                      // padded blocks in shared memory
    static constexpr int SMEM_FLOATS = NBUF * BLK + 12 * K2 + 2 * 8 * K3;  // + FP64 accumulators
    static constexpr int MIN_BLOCKS = K <= 8 ? 2 : 1;
};

// one output block: out = sum_p O_p applied along the row axis of in_p
struct StageOut {
    float *out;
    const float *in[4];
    const float *o[4];
    int np;
};

// loads K consecutive floats
template <int K, int IS>
__device__ __forceinline__ void load_row(float (&a)[K], const float *base) {
    if constexpr (K % 4 == 0 && IS % 4 == 0) {
#pragma unroll
        for (int i = 0; i < K; i += 4) {
            const float4 v = *reinterpret_cast<const float4 *>(base + i);
            a[i] = v.x;
            a[i + 1] = v.y;
            a[i + 2] = v.z;
            a[i + 3] = v.w;
        }
    } else if constexpr (K % 2 == 0 && IS % 2 == 0) {
#pragma unroll
        for (int i = 0; i < K; i += 2) {
            const float2 v = *reinterpret_cast<const float2 *>(base + i);
            a[i] = v.x;
            a[i + 1] = v.y;
        }
    } else {
#pragma unroll
        for (int i = 0; i < K; i++) a[i] = base[i];
    }
}

// warp-level block step: s[r][j] = sum_p sum_i in_p[i + IS c_r] O_p[i + K j]
template <int K, int IS>
__device__ __forceinline__ void warp_block(const StageOut &x, int lane, float (&s)[Shape<K>::R][K]) {
    using S = Shape<K>;
    constexpr int R = S::R, JG = S::JG;
#pragma unroll
    for (int r = 0; r < R; r++)
#pragma unroll
        for (int j = 0; j < K; j++) s[r][j] = 0.f;
    for (int p = 0; p < x.np; p++) {
        const float *in = x.in[p];
        const float *O = x.o[p];
#pragma unroll
        for (int j0 = 0; j0 < K; j0 += JG) {
            float w[JG][K];
#pragma unroll
            for (int jj = 0; jj < JG; jj++) load_row<K, K>(w[jj], O + K * (j0 + jj));
#pragma unroll
            for (int r = 0; r < R; r++) {
                const int c = lane + 32 * r;
                if (c < S::K2) {
                    float a[K];
                    load_row<K, IS>(a, in + IS * c);
#pragma unroll
                    for (int jj = 0; jj < JG; jj++)
#pragma unroll
                        for (int i = 0; i < K; i++) s[r][j0 + jj] = fmaf(a[i], w[jj][i], s[r][j0 + jj]);
                }
            }
        }
    }
}

template <int K, int IS>
__device__ __forceinline__ void run_stage(const StageOut *so, int nso, int warp, int lane) {
    using S = Shape<K>;
    for (int b = warp; b < nso; b += 8) {
        float s[S::R][K];
        warp_block<K, IS>(so[b], lane, s);
        float *out = so[b].out;
#pragma unroll
        for (int r = 0; r < S::R; r++) {
            const int c = lane + 32 * r;
            if (c < S::K2)
#pragma unroll
                for (int j = 0; j < K; j++) out[(c % K) + S::P * (c / K + K * j)] = s[r][j];
        }
    }
}

// Chunks of the work items of one output node: chunk = (position of g in the
// work list, first item, end item).  The FP64 partial sum of chunk c goes to
// partial[c]; k_reduce_chunks adds the chunks of each g in order
// (deterministic) and computes the node norms.
//
// Without a chunk counter every CTA computes chunk blockIdx.x.  With one, the
// launch is persistent: CTA b starts with chunk b and then takes chunks
// gridDim.x + atomicAdd(counter, 1) until *n_chunks_dev is reached (the
// counter must be 0 at launch), so the grid size does not depend on the work
// list and the number of chunks can be produced on the device.
template <int K>
__global__ void __launch_bounds__(256, Shape<K>::MIN_BLOCKS) k_contract_items(DevMRA m, DevOper op, const DevTree *fs, const DevTree *gs,
                                                                              const int *work_tree, const int *work, const int4 *chunks,
                                                                              const WorkItem *items, double *partial, int *err,
                                                                              const int *n_chunks_dev, int *counter) {
    using S = Shape<K>;
    constexpr int K2 = S::K2, K3 = S::K3, BLK = S::BLK, R = S::R;
    extern __shared__ __align__(16) float smf[];
    float *BUF = smf;                  // NBUF padded blocks
    float *OB = BUF + S::NBUF * BLK;   // [3 dirs][4 comps] K*K, out-of-band blocks zero
    double *G64 = (double *)(OB + 12 * K2);  // FP64 accumulators (thread-owned elements)
    __shared__ StageOut s_so0[9], s_so1[17], s_g[8];
    __shared__ int s_n0, s_n1, s_next;
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int n_chunks = n_chunks_dev ? *n_chunks_dev : (int)gridDim.x;
    for (int cix = blockIdx.x; cix < n_chunks;) {
    const int4 ch = chunks[cix];
    const int gi = work[ch.x];
    const int tree = work_tree[ch.x];
    const int depth = gs[tree].idx[gi].x - m.root_scale;
    const int f_cap_real = fs[tree].cap_real;
    const float *f_coefs32 = fs[tree].coefs32, *f_gcoefs32 = fs[tree].gcoefs32;
    // warp `warp` owns component gt = warp of g: rows lane + 32 r, all columns
    float acc[R][K];
#pragma unroll
    for (int r = 0; r < R; r++)
#pragma unroll
        for (int j = 0; j < K; j++) acc[r][j] = 0.f;
    for (int e = tid; e < 8 * K3; e += 256) G64[e] = 0.0;
    const long long it0 = ch.y, it1 = ch.z;
    int since = 0;
    for (long long it = it0; it < it1; it++) {
        const WorkItem item = items[it];
        const int i = item.term;
        const int *bwi = op.bw + ((size_t)i * op.max_rows + depth) * 5;
        const int L0 = op.dep_L[i * op.max_rows + depth], off = op.dep_off[i * op.max_rows + depth];
        for (int e = tid; e < 12 * K2; e += 256) {
            const int d = e / (4 * K2), r = e % (4 * K2), c = r / K2;
            const int l = item.tl[d];
            float v = 0.f;
            if (off >= 0 && abs(l) <= bwi[c] && abs(l) <= L0) v = op.blocks32[(size_t)(off + l + L0) * 4 * K2 + r];
            OB[e] = v;
        }
        const bool gen = item.fid >= f_cap_real;
        const float *fc = gen ? f_gcoefs32 + (size_t)(item.fid - f_cap_real) * K3 : f_coefs32 + (size_t)item.fid * 8 * K3;
        const bool block = item.flags & 1;
        const float *OX = OB, *OY = OB + 4 * K2, *OZ = OB + 8 * K2;
        if (block) {
            if (tid == 0) {
                bool nz[8], ib[3][4];
                for (int b = 0; b < 8; b++) nz[b] = ((item.mask >> (8 * b)) & 0xffull) != 0ull;
                for (int d = 0; d < 3; d++)
                    for (int c = 0; c < 4; c++) ib[d][c] = abs((int)item.tl[d]) <= bwi[c];
                const bool pure = depth != 0 && nz[0];
                float *Y0 = BUF, *U = BUF + 8 * BLK, *Y1 = BUF + 9 * BLK, *PP = BUF + 17 * BLK;
                bool y0[9], y1[9];
                int n0 = 0, n1 = 0;
                for (int o = 0; o < 8; o++) {
                    const int a0 = o & 1, b1 = (o >> 1) & 1, b2 = o >> 2;
                    StageOut x;
                    x.np = 0;
                    x.out = Y0 + o * BLK;
                    for (int b0 = 0; b0 < 2; b0++) {
                        const int src = b0 + 2 * b1 + 4 * b2;
                        if (!nz[src] || !ib[0][2 * a0 + b0]) continue;
                        if (pure && src == 0 && a0 == 0) continue;  // the s->s path goes through U
                        x.in[x.np] = fc + (size_t)src * K3;
                        x.o[x.np] = OX + (2 * a0 + b0) * K2;
                        x.np++;
                    }
                    y0[o] = x.np > 0;
                    if (x.np) s_so0[n0++] = x;
                }
                y0[8] = pure && ib[0][0];
                if (y0[8]) {
                    StageOut x;
                    x.out = U;
                    x.in[0] = fc;
                    x.o[0] = OX;
                    x.np = 1;
                    s_so0[n0++] = x;
                }
                for (int p = 0; p < 8; p++) {
                    const int a0 = p & 1, a1 = (p >> 1) & 1, b2 = p >> 2;
                    StageOut x;
                    x.np = 0;
                    x.out = Y1 + p * BLK;
                    for (int b1 = 0; b1 < 2; b1++) {
                        const int src = a0 + 2 * b1 + 4 * b2;
                        if (!y0[src] || !ib[1][2 * a1 + b1]) continue;
                        x.in[x.np] = Y0 + src * BLK;
                        x.o[x.np] = OY + (2 * a1 + b1) * K2;
                        x.np++;
                    }
                    if (y0[8] && p == 2 && ib[1][2]) {  // U -> (a0, a1, b2) = (0, 1, 0)
                        x.in[x.np] = U;
                        x.o[x.np] = OY + 2 * K2;
                        x.np++;
                    }
                    y1[p] = x.np > 0;
                    if (x.np) s_so1[n1++] = x;
                }
                y1[8] = y0[8] && ib[1][0];
                if (y1[8]) {
                    StageOut x;
                    x.out = PP;
                    x.in[0] = U;
                    x.o[0] = OY;
                    x.np = 1;
                    s_so1[n1++] = x;
                }
                for (int gt = 0; gt < 8; gt++) {
                    const int a2 = gt >> 2;
                    StageOut x;
                    x.np = 0;
                    x.out = nullptr;
                    for (int b2 = 0; b2 < 2; b2++) {
                        const int src = (gt & 3) + 4 * b2;
                        if (!y1[src] || !ib[2][2 * a2 + b2]) continue;
                        x.in[x.np] = Y1 + src * BLK;
                        x.o[x.np] = OZ + (2 * a2 + b2) * K2;
                        x.np++;
                    }
                    if (y1[8] && gt == 4 && ib[2][2]) {  // P -> (0, 0, 1); P -> (0, 0, 0) is the dropped s->s product
                        x.in[x.np] = PP;
                        x.o[x.np] = OZ + 2 * K2;
                        x.np++;
                    }
                    s_g[gt] = x;
                }
                s_n0 = n0;
                s_n1 = n1;
            }
            __syncthreads();
            run_stage<K, K>(s_so0, s_n0, warp, lane);
            __syncthreads();
            run_stage<K, S::P>(s_so1, s_n1, warp, lane);
            __syncthreads();
            float s[R][K];
            warp_block<K, S::P>(s_g[warp], lane, s);
#pragma unroll
            for (int r = 0; r < R; r++)
#pragma unroll
                for (int j = 0; j < K; j++) acc[r][j] += s[r][j];
        } else {
            for (int grp = 0; grp < 2; grp++) {
                const unsigned gmask = (unsigned)((item.mask >> (32 * grp)) & 0xffffffffull);
                if (gmask == 0) continue;
                if (tid == 0) {
                    float *X0 = BUF, *X1 = BUF + 8 * BLK;
                    int n0 = 0, n1 = 0;
                    for (int lft = 0; lft < 4; lft++) {
                        const int ft = 4 * grp + lft;
                        const unsigned col = (gmask >> (8 * lft)) & 0xffu;
                        for (int a0 = 0; a0 < 2; a0++) {
                            if (!(col & (a0 ? 0xAAu : 0x55u))) continue;
                            StageOut x;
                            x.out = X0 + (lft * 2 + a0) * BLK;
                            x.in[0] = fc + (size_t)ft * K3;
                            x.o[0] = OX + (2 * a0 + (ft & 1)) * K2;
                            x.np = 1;
                            s_so0[n0++] = x;
                        }
                        for (int sidx = 0; sidx < 4; sidx++) {
                            if (!(col & ((1u << sidx) | (1u << (sidx + 4))))) continue;
                            StageOut x;
                            x.out = X1 + (lft * 4 + sidx) * BLK;
                            x.in[0] = X0 + (lft * 2 + (sidx & 1)) * BLK;
                            x.o[0] = OY + (2 * (sidx >> 1) + ((ft >> 1) & 1)) * K2;
                            x.np = 1;
                            s_so1[n1++] = x;
                        }
                    }
                    for (int gt = 0; gt < 8; gt++) {
                        StageOut x;
                        x.np = 0;
                        x.out = nullptr;
                        for (int lft = 0; lft < 4; lft++) {
                            const int ft = 4 * grp + lft;
                            if (!((gmask >> (8 * lft + gt)) & 1u)) continue;
                            x.in[x.np] = X1 + (lft * 4 + (gt & 3)) * BLK;
                            x.o[x.np] = OZ + (2 * (gt >> 2) + (ft >> 2)) * K2;
                            x.np++;
                        }
                        s_g[gt] = x;
                    }
                    s_n0 = n0;
                    s_n1 = n1;
                }
                __syncthreads();
                run_stage<K, K>(s_so0, s_n0, warp, lane);
                __syncthreads();
                run_stage<K, S::P>(s_so1, s_n1, warp, lane);
                __syncthreads();
                float s[R][K];
                warp_block<K, S::P>(s_g[warp], lane, s);
#pragma unroll
                for (int r = 0; r < R; r++)
#pragma unroll
                    for (int j = 0; j < K; j++) acc[r][j] += s[r][j];
                __syncthreads();
            }
        }
        __syncthreads();  // OB, BUF and the stage lists are rewritten by the next item
        if (++since >= 16) {
#pragma unroll
            for (int r = 0; r < R; r++) {
                const int c = lane + 32 * r;
                if (c < K2)
#pragma unroll
                    for (int j = 0; j < K; j++) {
                        G64[warp * K3 + c + K2 * j] += (double)acc[r][j];
                        acc[r][j] = 0.f;
                    }
            }
            since = 0;
        }
    }
    double *go = partial + (size_t)cix * 8 * K3;
#pragma unroll
    for (int r = 0; r < R; r++) {
        const int c = lane + 32 * r;
        if (c < K2)
#pragma unroll
            for (int j = 0; j < K; j++) {
                const int e = warp * K3 + c + K2 * j;
                go[e] = G64[e] + (double)acc[r][j];
            }
    }
    if (!counter) break;
    __syncthreads();  // G64 is cleared with another thread mapping by the next chunk
    if (tid == 0) s_next = (int)gridDim.x + atomicAdd(counter, 1);
    __syncthreads();
    cix = s_next;
    }
}

// g coefficients = sum of the chunk partials of g in chunk order; node norms.
__global__ void __launch_bounds__(256) k_reduce_chunks(const DevTree *gs, const int *work_tree, const int *work, const int *chunk_begin,
                                                       const double *partial, int nc, const int *nw_dev) {
    const int tid = threadIdx.x;
    const int wi = blockIdx.x;
    if (nw_dev && wi >= *nw_dev) return;
    const int gi = work[wi];
    const DevTree &g = gs[work_tree[wi]];
    const int c0 = chunk_begin[wi], c1 = chunk_begin[wi + 1];
    double *go = g.coefs + (size_t)gi * nc;
    const int K3 = nc / 8;
    __shared__ double red[8][8];
    double part[8] = {0, 0, 0, 0, 0, 0, 0, 0};
    for (int e = tid; e < nc; e += 256) {
        double v = 0.0;
        for (int c = c0; c < c1; c++) v += partial[(size_t)c * nc + e];
        go[e] = v;
        part[e / K3] += v * v;
    }
    for (int comp = 0; comp < 8; comp++) {
        double v = part[comp];
        for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
        if ((tid & 31) == 0) red[comp][tid >> 5] = v;
    }
    __syncthreads();
    if (tid < 8) {
        double t = 0.0;
        for (int wv = 0; wv < 8; wv++) t += red[tid][wv];
        g.norms[(size_t)gi * 8 + tid] = sqrt(t);
    }
}

}  // namespace mixed
}  // namespace mwgpu
