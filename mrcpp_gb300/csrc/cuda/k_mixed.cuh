// Mixed-precision contraction over a work list (FP32 products and FP32 partial
// sums, FP64 accumulation of the partial sums every 16 work items).
//
// One CTA (512 threads = 16 warps) per chunk of the work items of one output
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
//   CG f components the x and xy intermediates the kept (ft, gt) pairs need.
//
// Every step is one output block out(K^2 x K) = sum_p in_p^T (K^2 x K) O_p (K x K)
// (MRCPP's 1D application).  A warp task is one output block: lane l owns
// the rows c = l + 32 r and their K outputs, reads its rows with vector loads
// and the operator rows (stored transposed) with broadcast vector loads.
// Blocks live in shared memory with rows padded to an odd number of 16-byte
// words; after the first stage of an item the f node of the next item is
// copied in with cp.async and its operator blocks are gathered, behind the
// second and third stages.  Each warp derives its own tasks from the item's
// mask (no serial list building): three CTA barriers per item of the block
// schedule.  Warp w accumulates component gt = w of g in registers, with a
// compensated (Kahan) FP32 sum for k <= 7, or FP32 sums flushed to FP64
// shared memory every 16 items for larger orders.
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
    static constexpr int R = (K2 + 31) / 32;             // rows per lane: a warp task is a whole output block
    static constexpr int NW = 8, NT = 32 * NW;           // warps, threads
    static constexpr bool KAHAN = K <= 8;                // compensated FP32 accumulators in registers; else FP64 in shared memory
    static constexpr int CG = K >= 10 ? 2 : 4;           // f components per group (component schedule)
    static constexpr int NBUF = CG == 2 ? 18 : 24;       // work blocks
    static constexpr int SMEM_FLOATS = 8 * BLK + NBUF * BLK + 3 * 12 * K2 + (KAHAN ? 0 : 2 * 8 * K3);
    static constexpr int MIN_BLOCKS = 2 * (SMEM_FLOATS * 4 + 1024) <= 228 * 1024 ? 2 : 1;
};

// Row c of a block handled by `lane` in its r-th row slot.  For K = 8 (P = 12)
// the 8-row groups are interleaved so that the 32 scattered stores of
// store_block hit disjoint banks (groups {0,2,4,6} then {1,3,5,7}); row loads
// stay conflict-free (8 consecutive rows per quarter warp).
template <int K>
__device__ __forceinline__ int row_of(int lane, int r) {
    if constexpr (K == 8 && padded_row(K) == 12) return (lane & 7) + 8 * (2 * (lane >> 3) + r);
    else return lane + 32 * r;
}

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

// one warp task: out = sum over the valid slots p (bit p of `valid`) of O_p
// applied along the row axis of in_p (row stride P), rows c = lane + 32 r:
// s[r][j] = sum_p sum_i in_p[i + P c] O_p[i + K j].  The slots are a
// compile-time set so that the pointers stay in registers.
template <int K, int NS>
__device__ __forceinline__ void task_block(const float *const (&in)[NS], const float *const (&O)[NS], unsigned valid, int lane,
                                           float (&s)[Shape<K>::R][K]) {
    using S = Shape<K>;
    constexpr int R = S::R;
#pragma unroll
    for (int r = 0; r < R; r++)
#pragma unroll
        for (int j = 0; j < K; j++) s[r][j] = 0.f;
#pragma unroll
    for (int p = 0; p < NS; p++) {
        if (!((valid >> p) & 1u)) continue;
        float a[R][K];
#pragma unroll
        for (int r = 0; r < R; r++) {
            const int c = row_of<K>(lane, r);
            if (c < S::K2) load_row<K, S::P>(a[r], in[p] + S::P * c);
            else
#pragma unroll
                for (int i = 0; i < K; i++) a[r][i] = 0.f;
        }
        const float *ot = O[p];  // transposed block: row i holds O(i, 0..K-1)
#pragma unroll
        for (int i = 0; i < K; i++) {
            float w[K];
            load_row<K, K>(w, ot + K * i);
#pragma unroll
            for (int r = 0; r < R; r++)
#pragma unroll
                for (int j = 0; j < K; j++) s[r][j] = fmaf(a[r][i], w[j], s[r][j]);
        }
    }
}

// stores a task's rows into an output block (the cyclic axis order of the 1D application)
template <int K>
__device__ __forceinline__ void store_block(float *out, int lane, const float (&s)[Shape<K>::R][K]) {
    using S = Shape<K>;
#pragma unroll
    for (int r = 0; r < S::R; r++) {
        const int c = row_of<K>(lane, r);
        if (c < S::K2)
#pragma unroll
            for (int j = 0; j < K; j++) out[(c % K) + S::P * (c / K + K * j)] = s[r][j];
    }
}

__device__ __forceinline__ void cp_async16(float *dst, const float *src) {
    const unsigned d = (unsigned)__cvta_generic_to_shared(dst);
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(d), "l"(src) : "memory");
}
__device__ __forceinline__ void cp_async4(float *dst, const float *src) {
    const unsigned d = (unsigned)__cvta_generic_to_shared(dst);
    asm volatile("cp.async.ca.shared.global [%0], [%1], 4;\n" ::"r"(d), "l"(src) : "memory");
}
__device__ __forceinline__ void cp_async_wait_all() { asm volatile("cp.async.wait_all;\n" ::: "memory"); }

// copies the f blocks an item needs (mask byte b nonzero) into padded rows
template <int K>
__device__ __forceinline__ void stage_f(float *fb, const WorkItem &item, int f_cap_real, const float *f_coefs32, const float *f_gcoefs32) {
    using S = Shape<K>;
    const bool gen = item.fid >= f_cap_real;
    const float *base = gen ? f_gcoefs32 + (size_t)(item.fid - f_cap_real) * S::K3 : f_coefs32 + (size_t)item.fid * 8 * S::K3;
    if constexpr (K % 4 == 0) {
        constexpr int CH = K / 4, PER = S::K2 * CH;
        for (int t = threadIdx.x; t < 8 * PER; t += S::NT) {
            const int b = t / PER, r = t % PER, c = r / CH, q = r % CH;
            if (((item.mask >> (8 * b)) & 0xffull) == 0ull) continue;
            cp_async16(fb + b * S::BLK + S::P * c + 4 * q, base + (size_t)b * S::K3 + K * c + 4 * q);
        }
    } else {
        for (int t = threadIdx.x; t < 8 * S::K3; t += S::NT) {
            const int b = t / S::K3, r = t % S::K3, c = r / K, i = r % K;
            if (((item.mask >> (8 * b)) & 0xffull) == 0ull) continue;
            cp_async4(fb + b * S::BLK + S::P * c + i, base + (size_t)b * S::K3 + r);
        }
    }
}

// the item's operator blocks [x, y, z][T, C, B, A], zero outside the band,
// each K x K block transposed (row i = O(i, 0..K-1))
template <int K>
__device__ __forceinline__ void stage_ob(float *ob, const DevOper &op, const WorkItem &item, int depth) {
    using S = Shape<K>;
    const int i = item.term;
    const int *bwi = op.bw + ((size_t)i * op.max_rows + depth) * 5;
    const int L0 = op.dep_L[i * op.max_rows + depth], off = op.dep_off[i * op.max_rows + depth];
    for (int e = threadIdx.x; e < 12 * S::K2; e += S::NT) {
        const int d = e / (4 * S::K2), r = e % (4 * S::K2), c = r / S::K2, ij = r % S::K2;
        const int l = d == 0 ? item.tl[0] : (d == 1 ? item.tl[1] : item.tl[2]);
        float v = 0.f;
        if (off >= 0 && abs(l) <= bwi[c] && abs(l) <= L0) v = op.blocks32[(size_t)(off + l + L0) * 4 * S::K2 + r];
        // column-major O(i, j) at i + K j is stored transposed, at j + K i
        ob[e - ij + (ij / K) + K * (ij % K)] = v;
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
__global__ void __launch_bounds__(Shape<K>::NT, Shape<K>::MIN_BLOCKS) k_contract_items(DevMRA m, DevOper op, const DevTree *fs,
                                                                                     const DevTree *gs, const int *work_tree, const int *work,
                                                                                     const int4 *chunks, const WorkItem *items, double *partial,
                                                                                     int *err, const int *n_chunks_dev, int *counter) {
    using S = Shape<K>;
    constexpr int K2 = S::K2, K3 = S::K3, BLK = S::BLK, R = S::R, NW = S::NW, CG = S::CG;
    extern __shared__ __align__(16) float smf[];
    float *FB = smf;                                  // 8 staged f blocks
    float *BUF = FB + 8 * BLK;                        // NBUF work blocks
    float *OBS = BUF + S::NBUF * BLK;                 // 3 x [3 dirs][4 comps] K x K
    double *G64 = (double *)(OBS + 3 * 12 * K2);      // FP64 accumulators (without KAHAN)
    __shared__ int s_next;
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int n_chunks = n_chunks_dev ? *n_chunks_dev : (int)gridDim.x;
    for (int cix = blockIdx.x; cix < n_chunks;) {
        const int4 ch = chunks[cix];
        const int gi = work[ch.x];
        const int tree = work_tree[ch.x];
        const int depth = gs[tree].idx[gi].x - m.root_scale;
        const int f_cap_real = fs[tree].cap_real;
        const float *f_coefs32 = fs[tree].coefs32, *f_gcoefs32 = fs[tree].gcoefs32;
        // warp w owns component gt = w of g: rows lane + 32 r, all columns
        float acc[R][K], cmp[R][K];
#pragma unroll
        for (int r = 0; r < R; r++)
#pragma unroll
            for (int j = 0; j < K; j++) {
                acc[r][j] = 0.f;
                cmp[r][j] = 0.f;
                const int c = row_of<K>(lane, r);
                if (!S::KAHAN && c < K2) G64[warp * K3 + c + K2 * j] = 0.0;
            }
        const int it0 = ch.y, it1 = ch.z;
        if (it0 < it1) {
            const WorkItem first = items[it0];
            stage_f<K>(FB, first, f_cap_real, f_coefs32, f_gcoefs32);
            stage_ob<K>(OBS, op, first, depth);
        }
        cp_async_wait_all();
        __syncthreads();
        int since = 0;
        for (int it = it0; it < it1; it++) {
            const int k = it - it0;
            const WorkItem item = items[it];
            const bool has_next = it + 1 < it1;
            WorkItem nx = item;
            if (has_next) nx = items[it + 1];
            const float *OX = OBS + (k % 3) * 12 * K2, *OY = OX + 4 * K2, *OZ = OX + 8 * K2;
            const int *bwi = op.bw + ((size_t)item.term * op.max_rows + depth) * 5;
            int ib[3] = {0, 0, 0};  // bit c of ib[d]: |l_d| within the band of component c
#pragma unroll
            for (int d = 0; d < 3; d++)
#pragma unroll
                for (int c = 0; c < 4; c++) ib[d] |= (abs((int)item.tl[d]) <= bwi[c]) << c;
            unsigned nzm = 0;
            for (int b = 0; b < 8; b++) nzm |= (((item.mask >> (8 * b)) & 0xffull) != 0ull) << b;
            const bool block = item.flags & 1;
            int last = 0, nsub = 1;
            if (!block) {
                nsub = 8 / CG;
                for (int g = 0; g < nsub; g++)
                    if ((item.mask >> (8 * CG * g)) & ((1ull << (8 * CG)) - 1ull)) last = g;
            }
            for (int sub = 0; sub < nsub; sub++) {
                unsigned long long gbits = 0ull;
                if (!block) {
                    gbits = (item.mask >> (8 * CG * sub)) & ((1ull << (8 * CG)) - 1ull);
                    if (gbits == 0ull) continue;
                }
                float sv[R][K];
                if (block) {
                    const bool pure = depth != 0 && (nzm & 1u);
                    unsigned y0 = 0, y1 = 0;
                    for (int o = 0; o < 8; o++) {
                        const int a0 = o & 1, b12 = o & 6;
                        for (int b0 = 0; b0 < 2; b0++) {
                            const int src = b0 + b12;
                            if (((nzm >> src) & 1u) && ((ib[0] >> (2 * a0 + b0)) & 1) && !(pure && src == 0 && a0 == 0)) y0 |= 1u << o;
                        }
                    }
                    if (pure && (ib[0] & 1)) y0 |= 1u << 8;
                    for (int q = 0; q < 8; q++) {
                        const int a0 = q & 1, a1 = (q >> 1) & 1, b2 = q >> 2;
                        for (int b1 = 0; b1 < 2; b1++)
                            if (((y0 >> (a0 + 2 * b1 + 4 * b2)) & 1u) && ((ib[1] >> (2 * a1 + b1)) & 1)) y1 |= 1u << q;
                        if (q == 2 && ((y0 >> 8) & 1u) && ((ib[1] >> 2) & 1)) y1 |= 1u << q;
                    }
                    if (((y0 >> 8) & 1u) && (ib[1] & 1)) y1 |= 1u << 8;
                    float *Y0 = BUF, *U = BUF + 8 * BLK, *Y1 = BUF + 9 * BLK, *PP = BUF + 17 * BLK;
                    // stage 0: outputs Y0[o] (o < 8) and U (o = 8)
                    for (int o = warp; o < 9; o += NW) {
                        if (!((y0 >> o) & 1u)) continue;
                        const int a0 = o & 1, b12 = o & 6;  // src = b0 + b12
                        const float *in[2] = {FB + b12 * BLK, FB + (b12 + 1) * BLK};
                        const float *O[2] = {OX + 2 * a0 * K2, OX + (2 * a0 + 1) * K2};
                        unsigned valid = 0;
                        for (int b0 = 0; b0 < 2; b0++) {
                            const int src = b0 + b12;
                            if (((nzm >> src) & 1u) && ((ib[0] >> (2 * a0 + b0)) & 1) && !(pure && src == 0 && a0 == 0)) valid |= 1u << b0;
                        }
                        if (o == 8) {  // U = O^x_T f[0]
                            in[0] = FB;
                            O[0] = OX;
                            valid = 1u;
                        }
                        task_block<K, 2>(in, O, valid, lane, sv);
                        store_block<K>(o < 8 ? Y0 + o * BLK : U, lane, sv);
                    }
                    __syncthreads();
                    if (has_next) {  // the staged f block is free: the next item's f and operator blocks
                        stage_f<K>(FB, nx, f_cap_real, f_coefs32, f_gcoefs32);
                        stage_ob<K>(OBS + ((k + 1) % 3) * 12 * K2, op, nx, depth);
                    }
                    // stage 1: outputs Y1[q] (q < 8) and PP (q = 8)
                    for (int q = warp; q < 9; q += NW) {
                        if (!((y1 >> q) & 1u)) continue;
                        const int a0 = q & 1, a1 = (q >> 1) & 1, b2 = q >> 2;
                        const float *in[3] = {Y0 + (a0 + 4 * b2) * BLK, Y0 + (a0 + 2 + 4 * b2) * BLK, U};
                        const float *O[3] = {OY + 2 * a1 * K2, OY + (2 * a1 + 1) * K2, OY + 2 * K2};
                        unsigned valid = 0;
                        for (int b1 = 0; b1 < 2; b1++)
                            if (((y0 >> (a0 + 2 * b1 + 4 * b2)) & 1u) && ((ib[1] >> (2 * a1 + b1)) & 1)) valid |= 1u << b1;
                        if (q == 2 && ((y0 >> 8) & 1u) && ((ib[1] >> 2) & 1)) valid |= 4u;  // U -> (a0, a1, b2) = (0, 1, 0)
                        if (q == 8) {  // P = O^y_T U
                            in[0] = U;
                            O[0] = OY;
                            valid = 1u;
                        }
                        task_block<K, 3>(in, O, valid, lane, sv);
                        store_block<K>(q < 8 ? Y1 + q * BLK : PP, lane, sv);
                    }
                    __syncthreads();
                    // stage 2: g component gt = warp
                    {
                        const int gt = warp, a2 = gt >> 2;
                        const float *in[3] = {Y1 + (gt & 3) * BLK, Y1 + ((gt & 3) + 4) * BLK, PP};
                        const float *O[3] = {OZ + 2 * a2 * K2, OZ + (2 * a2 + 1) * K2, OZ + 2 * K2};
                        unsigned valid = 0;
                        for (int b2 = 0; b2 < 2; b2++)
                            if (((y1 >> ((gt & 3) + 4 * b2)) & 1u) && ((ib[2] >> (2 * a2 + b2)) & 1)) valid |= 1u << b2;
                        // P -> (0, 0, 1); P -> (0, 0, 0) is the dropped s->s product
                        if (gt == 4 && ((y1 >> 8) & 1u) && ((ib[2] >> 2) & 1)) valid |= 4u;
                        task_block<K, 3>(in, O, valid, lane, sv);
                    }
                } else {
                    float *X0 = BUF, *X1 = BUF + 2 * CG * BLK;
                    const int ft0 = CG * sub;
                    // stage 0: X0[(lft, a0)] = O^x_{a0, ft&1} f[ft]
                    for (int jx = warp; jx < 2 * CG; jx += NW) {
                        const int lft = jx >> 1, a0 = jx & 1, ft = ft0 + lft;
                        const unsigned col = (unsigned)((gbits >> (8 * lft)) & 0xffull);
                        if (!(col & (a0 ? 0xAAu : 0x55u))) continue;
                        const float *in[1] = {FB + ft * BLK};
                        const float *O[1] = {OX + (2 * a0 + (ft & 1)) * K2};
                        task_block<K, 1>(in, O, 1u, lane, sv);
                        store_block<K>(X0 + jx * BLK, lane, sv);
                    }
                    __syncthreads();
                    if (sub == last && has_next) {
                        stage_f<K>(FB, nx, f_cap_real, f_coefs32, f_gcoefs32);
                        stage_ob<K>(OBS + ((k + 1) % 3) * 12 * K2, op, nx, depth);
                    }
                    // stage 1: X1[(lft, sidx)] = O^y_{a1, (ft>>1)&1} X0[(lft, a0)], sidx = a0 + 2 a1
                    for (int jx = warp; jx < 4 * CG; jx += NW) {
                        const int lft = jx >> 2, sidx = jx & 3, ft = ft0 + lft;
                        const unsigned col = (unsigned)((gbits >> (8 * lft)) & 0xffull);
                        if (!(col & ((1u << sidx) | (1u << (sidx + 4))))) continue;
                        const float *in[1] = {X0 + (2 * lft + (sidx & 1)) * BLK};
                        const float *O[1] = {OY + (2 * (sidx >> 1) + ((ft >> 1) & 1)) * K2};
                        task_block<K, 1>(in, O, 1u, lane, sv);
                        store_block<K>(X1 + jx * BLK, lane, sv);
                    }
                    __syncthreads();
                    // stage 2: g[gt] += sum over the group's kept (ft, gt) of O^z_{a2, ft>>2} X1[(lft, gt&3)]
                    {
                        const int gt = warp;
                        const float *in[CG];
                        const float *O[CG];
                        unsigned valid = 0;
#pragma unroll
                        for (int lft = 0; lft < CG; lft++) {
                            const int ft = ft0 + lft;
                            in[lft] = X1 + (4 * lft + (gt & 3)) * BLK;
                            O[lft] = OZ + (2 * (gt >> 2) + (ft >> 2)) * K2;
                            if ((gbits >> (8 * lft + gt)) & 1ull) valid |= 1u << lft;
                        }
                        task_block<K, CG>(in, O, valid, lane, sv);
                    }
                    // no barrier before the next group: its stage 0 writes X0, which stage 2
                    // does not read, and its stage 1 writes X1 only after the next barrier
                }
                // accumulate: compensated (Kahan) FP32 sums, or FP32 sums flushed to FP64
#pragma unroll
                for (int r = 0; r < R; r++)
#pragma unroll
                    for (int j = 0; j < K; j++) {
                        if (S::KAHAN) {
                            const float y = sv[r][j] - cmp[r][j];
                            const float t = acc[r][j] + y;
                            cmp[r][j] = (t - acc[r][j]) - y;
                            acc[r][j] = t;
                        } else {
                            acc[r][j] += sv[r][j];
                        }
                    }
            }
            if (!S::KAHAN && ++since >= 16) {
#pragma unroll
                for (int r = 0; r < R; r++) {
                    const int c = row_of<K>(lane, r);
                    if (c < K2)
#pragma unroll
                        for (int j = 0; j < K; j++) {
                            G64[warp * K3 + c + K2 * j] += (double)acc[r][j];
                            acc[r][j] = 0.f;
                        }
                }
                since = 0;
            }
            cp_async_wait_all();
            __syncthreads();  // next item's f and operator blocks ready; work blocks free
        }
        double *go = partial + (size_t)cix * 8 * K3;
#pragma unroll
        for (int r = 0; r < R; r++) {
            const int c = row_of<K>(lane, r);
            if (c < K2)
#pragma unroll
                for (int j = 0; j < K; j++) {
                    const int e = warp * K3 + c + K2 * j;
                    go[e] = S::KAHAN ? (double)acc[r][j] - (double)cmp[r][j] : G64[e] + (double)acc[r][j];
                }
        }
        if (!counter) break;
        __syncthreads();
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
