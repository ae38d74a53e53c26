// Mixed-precision contraction over a work list: FP32 products; per output
// component, a compensated (Kahan) FP32 accumulator in registers for K <= 8,
// and for K > 8 FP32 partial sums added into FP64 accumulators in shared
// memory every 16 work items.
//
// One CTA (256 threads = 8 warps, Shape<K>::NW) per chunk of the work items of
// one output node g (k_worklist.cu makes the items; the screening of
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
    // k = 7: the products run on the tensor cores (mma.sync m16n8k8, TF32 with
    // a hi/lo split of both operands, 3 products per FP32 product); the
    // intermediates are then stored column by column, element (c, j) of an
    // output block at j S1 + (c % 8) + 12 (c / 8), S1 = 100: conflict-free
    // fragment loads and stores
    static constexpr bool MMA = K == 8;
    static constexpr int S1 = 100;
    static constexpr int IB = MMA ? K * S1 : BLK;        // one intermediate block
    static constexpr int SMEM_FLOATS = 8 * BLK + NBUF * IB + 3 * 12 * K2 + (KAHAN ? 0 : 2 * 8 * K3);
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
// adds a task's rows to an output block (same positions as store_block)
template <int K>
__device__ __forceinline__ void add_block(float *out, int lane, const float (&s)[Shape<K>::R][K]) {
    using S = Shape<K>;
#pragma unroll
    for (int r = 0; r < S::R; r++) {
        const int c = row_of<K>(lane, r);
        if (c < S::K2)
#pragma unroll
            for (int j = 0; j < K; j++) out[(c % K) + S::P * (c / K + K * j)] += s[r][j];
    }
}

// ---- tensor-core path (K = 8) ----
__device__ __forceinline__ unsigned to_tf32(float x) {
    unsigned r;
    asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(r) : "f"(x));
    return r;
}

// x = hi + lo, hi = x rounded to TF32 and lo = x - hi exactly (|lo| <= 2^-11 |x|).
// lo goes to the tensor core as an FP32 bit pattern: its use as a TF32
// operand costs at most 2^-11 |lo| <= 2^-22 |x|, the accuracy of a second
// rounding, without the second conversion.
__device__ __forceinline__ void split_tf32(float x, unsigned &hi, unsigned &lo) {
    hi = to_tf32(x);
    lo = __float_as_uint(x - __uint_as_float(hi));
}

// (not volatile: a pure function of its operands, free to be scheduled
// between independent products)
__device__ __forceinline__ void mma_tf32(float (&d)[4], unsigned a0, unsigned a1, unsigned a2, unsigned a3, unsigned b0, unsigned b1) {
    asm("mma.sync.aligned.m16n8k8.row.col.f32.tf32.tf32.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, {%0,%1,%2,%3};\n"
                 : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
                 : "r"(a0), "r"(a1), "r"(a2), "r"(a3), "r"(b0), "r"(b1));
}

// (c, j) of accumulator element e = 4 mt + v of a lane (C fragment of m-tile mt)
__device__ __forceinline__ void mma_cj(int lane, int e, int &c, int &j) {
    const int mt = e >> 2, v = e & 3;
    c = 16 * mt + (lane >> 2) + 8 * (v >> 1);
    j = 2 * (lane & 3) + (v & 1);
}

// One warp task on the tensor cores: the 64 x 8 output block as 4 m-tiles of
// m16n8k8.  A(c, i): staged f (FIN, row c at P c) or an intermediate block
// (element (i + K (c % K), c / K) of its producer at (c / K) S1 + i + 12 (c % K));
// B(i, j) = O(i, j) from the transposed operator block.  s holds the C
// fragments: d[mt][v] = s[mt >> 1][4 (mt & 1) + v].
template <int K, int NS, bool FIN>
__device__ __forceinline__ void task_mma(const float *const (&in)[NS], const float *const (&O)[NS], unsigned valid, int lane,
                                         float (&s)[Shape<K>::R][K]) {
    using S = Shape<K>;
    static_assert(K == 8, "tensor-core path for K = 8");
    const int g = lane >> 2, t = lane & 3;
    // hi.hi products in d, the two correction products in dl: two dependency
    // chains per m-tile
    float d[4][4], dl[4][4];
#pragma unroll
    for (int mt = 0; mt < 4; mt++)
#pragma unroll
        for (int v = 0; v < 4; v++) d[mt][v] = dl[mt][v] = 0.f;
#pragma unroll
    for (int p = 0; p < NS; p++) {
        if (!((valid >> p) & 1u)) continue;
        unsigned bh0, bl0, bh1, bl1;
        split_tf32(O[p][g + K * t], bh0, bl0);
        split_tf32(O[p][g + K * (t + 4)], bh1, bl1);
        // all four m-tiles' A fragments first, then the products m-tile after
        // m-tile, so that consecutive mma instructions are independent
        unsigned ah[4][4], al[4][4];
#pragma unroll
        for (int mt = 0; mt < 4; mt++) {
            float x[4];
            if (FIN) {
                const float *r0 = in[p] + S::P * (16 * mt + g), *r1 = in[p] + S::P * (16 * mt + g + 8);
                x[0] = r0[t];
                x[1] = r1[t];
                x[2] = r0[t + 4];
                x[3] = r1[t + 4];
            } else {
                const float *r0 = in[p] + (2 * mt) * S::S1 + 12 * g, *r1 = in[p] + (2 * mt + 1) * S::S1 + 12 * g;
                x[0] = r0[t];
                x[1] = r1[t];
                x[2] = r0[t + 4];
                x[3] = r1[t + 4];
            }
#pragma unroll
            for (int q = 0; q < 4; q++) split_tf32(x[q], ah[mt][q], al[mt][q]);
        }
#pragma unroll
        for (int mt = 0; mt < 4; mt++) mma_tf32(dl[mt], al[mt][0], al[mt][1], al[mt][2], al[mt][3], bh0, bh1);
#pragma unroll
        for (int mt = 0; mt < 4; mt++) mma_tf32(d[mt], ah[mt][0], ah[mt][1], ah[mt][2], ah[mt][3], bh0, bh1);
#pragma unroll
        for (int mt = 0; mt < 4; mt++) mma_tf32(dl[mt], ah[mt][0], ah[mt][1], ah[mt][2], ah[mt][3], bl0, bl1);
    }
#pragma unroll
    for (int mt = 0; mt < 4; mt++)
#pragma unroll
        for (int v = 0; v < 4; v++) s[mt >> 1][4 * (mt & 1) + v] = d[mt][v] + dl[mt][v];
}

// One m-tile (rows 16 mt .. 16 mt + 15) of a one-input task on the tensor cores:
// the 9th output block of a stage (the U or P channel) is spread over four
// warps this way, so that a stage with 9 outputs on 8 warps takes 1 1/8
// task times instead of 2.
template <int K, bool FIN>
__device__ __forceinline__ void task_mma_tile(const float *in, const float *O, int lane, int mt, float (&d)[4]) {
    using S = Shape<K>;
    const int g = lane >> 2, t = lane & 3;
    unsigned bh0, bl0, bh1, bl1;
    split_tf32(O[g + K * t], bh0, bl0);
    split_tf32(O[g + K * (t + 4)], bh1, bl1);
    float x[4];
    if (FIN) {
        const float *r0 = in + S::P * (16 * mt + g), *r1 = in + S::P * (16 * mt + g + 8);
        x[0] = r0[t];
        x[1] = r1[t];
        x[2] = r0[t + 4];
        x[3] = r1[t + 4];
    } else {
        const float *r0 = in + (2 * mt) * S::S1 + 12 * g, *r1 = in + (2 * mt + 1) * S::S1 + 12 * g;
        x[0] = r0[t];
        x[1] = r1[t];
        x[2] = r0[t + 4];
        x[3] = r1[t + 4];
    }
    unsigned ah[4], al[4];
#pragma unroll
    for (int q = 0; q < 4; q++) split_tf32(x[q], ah[q], al[q]);
#pragma unroll
    for (int v = 0; v < 4; v++) d[v] = 0.f;
    mma_tf32(d, al[0], al[1], al[2], al[3], bh0, bh1);
    mma_tf32(d, ah[0], ah[1], ah[2], ah[3], bl0, bl1);
    mma_tf32(d, ah[0], ah[1], ah[2], ah[3], bh0, bh1);
}
// stores (or adds) the fragment of m-tile mt into an intermediate block
template <int K>
__device__ __forceinline__ void store_or_add_tile(float *out, int lane, int mt, const float (&d)[4], bool add) {
    using S = Shape<K>;
#pragma unroll
    for (int v = 0; v < 4; v++) {
        int c, j;
        mma_cj(lane, 4 * mt + v, c, j);
        float &dst = out[j * S::S1 + (c & 7) + 12 * (c >> 3)];
        dst = add ? dst + d[v] : d[v];
    }
}

// stores C fragments into an intermediate block: element (c, j) at j S1 + (c % 8) + 12 (c / 8)
template <int K>
__device__ __forceinline__ void store_mma(float *out, int lane, const float (&s)[Shape<K>::R][K]) {
    using S = Shape<K>;
#pragma unroll
    for (int e = 0; e < 16; e++) {
        int c, j;
        mma_cj(lane, e, c, j);
        out[j * S::S1 + (c & 7) + 12 * (c >> 3)] = s[e >> 3][e & 7];
    }
}
template <int K>
__device__ __forceinline__ void add_mma(float *out, int lane, const float (&s)[Shape<K>::R][K]) {
    using S = Shape<K>;
#pragma unroll
    for (int e = 0; e < 16; e++) {
        int c, j;
        mma_cj(lane, e, c, j);
        out[j * S::S1 + (c & 7) + 12 * (c >> 3)] += s[e >> 3][e & 7];
    }
}

// one warp task / store on either path
template <int K, int NS, bool FIN>
__device__ __forceinline__ void task(const float *const (&in)[NS], const float *const (&O)[NS], unsigned valid, int lane,
                                     float (&s)[Shape<K>::R][K]) {
    if constexpr (Shape<K>::MMA) task_mma<K, NS, FIN>(in, O, valid, lane, s);
    else task_block<K, NS>(in, O, valid, lane, s);
}
template <int K>
__device__ __forceinline__ void store(float *out, int lane, const float (&s)[Shape<K>::R][K]) {
    if constexpr (Shape<K>::MMA) store_mma<K>(out, lane, s);
    else store_block<K>(out, lane, s);
}
// first contribution of a group to an output block: store; later ones: add
template <int K>
__device__ __forceinline__ void store_or_add(float *out, int lane, const float (&s)[Shape<K>::R][K], bool add) {
    if (add) {
        if constexpr (Shape<K>::MMA) add_mma<K>(out, lane, s);
        else add_block<K>(out, lane, s);
    } else {
        store<K>(out, lane, s);
    }
}
// (c, j) of accumulator element (r, jj) of a lane
template <int K>
__device__ __forceinline__ void acc_cj(int lane, int r, int jj, int &c, int &j) {
    if constexpr (Shape<K>::MMA) mma_cj(lane, r * K + jj, c, j);
    else {
        c = row_of<K>(lane, r);
        j = jj;
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

// stage-1 (bits 17-34) and stage-2 (bits 35-51) input bits of WorkItem::sched
constexpr unsigned long long kStage1Bits = ((1ull << 18) - 1ull) << 17;
constexpr unsigned long long kStage2Bits = ((1ull << 17) - 1ull) << 35;

// block-schedule items whose y and z (resp. z) operator blocks are the same
__device__ __forceinline__ bool same_s1(const WorkItem &a, const WorkItem &b) {
    return (a.flags & 1) && (b.flags & 1) && a.term == b.term && a.tl[1] == b.tl[1] && a.tl[2] == b.tl[2];
}
__device__ __forceinline__ bool same_s2(const WorkItem &a, const WorkItem &b) {
    return (a.flags & 1) && (b.flags & 1) && a.term == b.term && a.tl[2] == b.tl[2];
}

// g accumulators: compensated (Kahan) FP32 sums, or FP32 sums flushed to FP64
template <int K>
__device__ __forceinline__ void accumulate(float (&acc)[Shape<K>::R][K], float (&cmp)[Shape<K>::R][K], const float (&sv)[Shape<K>::R][K]) {
#pragma unroll
    for (int r = 0; r < Shape<K>::R; r++)
#pragma unroll
        for (int j = 0; j < K; j++) {
            if (Shape<K>::KAHAN) {
                const float y = sv[r][j] - cmp[r][j];
                const float t = acc[r][j] + y;
                cmp[r][j] = (t - acc[r][j]) - y;
                acc[r][j] = t;
            } else {
                acc[r][j] += sv[r][j];
            }
        }
}

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

// the item's operator blocks [x, y, z][T, C, B, A] (transposed FP32 copies),
// zero outside the band: cp.async copies of whole blocks
template <int K>
__device__ __forceinline__ void stage_ob(float *ob, const DevOper &op, const WorkItem &item, int depth) {
    using S = Shape<K>;
    const int i = item.term;
    const int *bwi = op.bw + ((size_t)i * op.max_rows + depth) * 5;
    const int L0 = op.dep_L[i * op.max_rows + depth], off = op.dep_off[i * op.max_rows + depth];
    constexpr int CH = S::K2 % 4 == 0 ? 4 : 1, PER = S::K2 / CH;
    for (int e = threadIdx.x; e < 12 * PER; e += S::NT) {
        const int blk = e / PER, q = e % PER, d = blk >> 2, c = blk & 3;
        const int l = d == 0 ? item.tl[0] : (d == 1 ? item.tl[1] : item.tl[2]);
        float *dst = ob + blk * S::K2 + CH * q;
        if (off >= 0 && abs(l) <= bwi[c] && abs(l) <= L0) {
            const float *src = op.blocks32 + (size_t)(off + l + L0) * 4 * S::K2 + c * S::K2 + CH * q;
            if constexpr (CH == 4) cp_async16(dst, src);
            else cp_async4(dst, src);
        } else {
            if constexpr (CH == 4) *reinterpret_cast<float4 *>(dst) = make_float4(0.f, 0.f, 0.f, 0.f);
            else *dst = 0.f;
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
__global__ void __launch_bounds__(Shape<K>::NT, Shape<K>::MIN_BLOCKS) k_contract_items(DevMRA m, DevOper op, const DevTree *fs,
                                                                                     const DevTree *gs, const int *work_tree, const int *work,
                                                                                     const int4 *chunks, const WorkItem *items, double *partial,
                                                                                     int *err, const int *n_chunks_dev, int *counter) {
    using S = Shape<K>;
    constexpr int K2 = S::K2, K3 = S::K3, BLK = S::BLK, IB = S::IB, R = S::R, NW = S::NW, CG = S::CG;
    extern __shared__ __align__(16) float smf[];
    float *FB = smf;                                  // 8 staged f blocks
    float *BUF = FB + 8 * BLK;                        // NBUF work blocks
    float *OBS = BUF + S::NBUF * IB;                  // 3 x [3 dirs][4 comps] K x K
    double *G64 = (double *)(OBS + 3 * 12 * K2);      // FP64 accumulators (without KAHAN)
    __shared__ int s_next;
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int n_chunks = n_chunks_dev ? *n_chunks_dev : (int)gridDim.x;
    for (int cix = blockIdx.x; cix < n_chunks;) {
        const int4 ch = chunks[cix];
        // chunks of type 1 (block-schedule items only, order 7) belong to the tensor-core kernel (k_tc.cu)
        if (ch.w != 1) {
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
            for (int jj = 0; jj < K; jj++) {
                acc[r][jj] = 0.f;
                cmp[r][jj] = 0.f;
                int c, j;
                acc_cj<K>(lane, r, jj, c, j);
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
        // Groups of adjacent block-schedule items (term-major item order):
        // S1 = same (term, l_y, l_z), whose x-step outputs are summed before one
        // y step; S2 = same (term, l_z), whose xy-step outputs are summed before
        // one z step.  O^y and O^z are the same for all items of such a group,
        // so the sums equal the per-item products.  sc1 / sc2: union of the
        // group's stage-1 / stage-2 input bits; w1 / w2: S1 / S2 blocks already
        // written in the group (the first contribution is stored, later ones
        // are added).
        float *S1 = BUF, *S2 = BUF + 9 * IB;
        unsigned long long sc1 = 0ull, sc2 = 0ull;
        unsigned w1 = 0u, w2 = 0u;
        WorkItem prev{};
        for (int it = it0; it < it1; it++) {
            const int k = it - it0;
            const WorkItem item = items[it];
            const bool has_next = it + 1 < it1;
            WorkItem nx = item;
            if (has_next) nx = items[it + 1];
            const float *OX = OBS + (k % 3) * 12 * K2, *OY = OX + 4 * K2, *OZ = OX + 8 * K2;
            const bool block = item.flags & 1;
            float sv[R][K];
            if (block) {
                const bool s1_first = !(k > 0 && same_s1(prev, item)), s1_last = !(has_next && same_s1(item, nx));
                const bool s2_first = !(k > 0 && same_s2(prev, item)), s2_last = !(has_next && same_s2(item, nx));
                // stage structure from the work-list builder (k_worklist.cu)
                const unsigned long long sc = item.sched;
                if (s1_first) {
                    sc1 = 0ull;
                    w1 = 0u;
                }
                if (s2_first) {
                    sc2 = 0ull;
                    w2 = 0u;
                }
                sc1 |= sc & kStage1Bits;
                sc2 |= sc & kStage2Bits;
                // stage 0: outputs Y0[o] (o < 8) and U (o = 8), summed into S1
                unsigned made = (unsigned)((sc >> 16) & 1ull) << 8;
#pragma unroll
                for (int o = 0; o < 8; o++) made |= (((sc >> (2 * o)) & 3ull) ? 1u : 0u) << o;
                for (int o = warp; o < (S::MMA ? 8 : 9); o += NW) {
                    unsigned valid = o < 8 ? (unsigned)((sc >> (2 * o)) & 3ull) : (unsigned)((sc >> 16) & 1ull);
                    if (!valid) continue;
                    const int a0 = o & 1, b12 = o & 6;  // src = b0 + b12
                    const float *in[2] = {FB + b12 * BLK, FB + (b12 + 1) * BLK};
                    const float *O[2] = {OX + 2 * a0 * K2, OX + (2 * a0 + 1) * K2};
                    if (o == 8) {  // U = O^x_T f[0]
                        in[0] = FB;
                        O[0] = OX;
                    }
                    task<K, 2, true>(in, O, valid, lane, sv);
                    store_or_add<K>(S1 + o * IB, lane, sv, (w1 >> o) & 1u);
                }
                if constexpr (S::MMA) {
                    // U = O^x_T f[0]: one m-tile on each of warps 4-7
                    if (((sc >> 16) & 1ull) && warp >= 4) {
                        float d[4];
                        task_mma_tile<K, true>(FB, OX, lane, warp - 4, d);
                        store_or_add_tile<K>(S1 + 8 * IB, lane, warp - 4, d, (w1 >> 8) & 1u);
                    }
                }
                w1 |= made;
                __syncthreads();
                if (has_next) {  // the staged f block is free: the next item's f and operator blocks
                    stage_f<K>(FB, nx, f_cap_real, f_coefs32, f_gcoefs32);
                    stage_ob<K>(OBS + ((k + 1) % 3) * 12 * K2, op, nx, depth);
                }
                if (s1_last) {
                    // stage 1: outputs Y1[q] (q < 8) and PP (q = 8) of the summed S1, summed into S2
                    unsigned made1 = (unsigned)((sc1 >> 34) & 1ull) << 8;
#pragma unroll
                    for (int q = 0; q < 8; q++) made1 |= (((sc1 >> (17 + 2 * q)) & 3ull) || (q == 2 && ((sc1 >> 33) & 1ull)) ? 1u : 0u) << q;
                    for (int q = warp; q < (S::MMA ? 8 : 9); q += NW) {
                        unsigned valid = q < 8 ? (unsigned)((sc1 >> (17 + 2 * q)) & 3ull) | (q == 2 ? (unsigned)((sc1 >> 33) & 1ull) << 2 : 0u)
                                               : (unsigned)((sc1 >> 34) & 1ull);
                        if (!valid) continue;
                        const int a0 = q & 1, a1 = (q >> 1) & 1, b2 = q >> 2;
                        const float *in[3] = {S1 + (a0 + 4 * b2) * IB, S1 + (a0 + 2 + 4 * b2) * IB, S1 + 8 * IB};  // U -> (0, 1, 0)
                        const float *O[3] = {OY + 2 * a1 * K2, OY + (2 * a1 + 1) * K2, OY + 2 * K2};
                        if (q == 8) {  // P = O^y_T U
                            in[0] = S1 + 8 * IB;
                            O[0] = OY;
                        }
                        task<K, 3, false>(in, O, valid, lane, sv);
                        store_or_add<K>(S2 + q * IB, lane, sv, (w2 >> q) & 1u);
                    }
                    if constexpr (S::MMA) {
                        // P = O^y_T U: one m-tile on each of warps 4-7
                        if (((sc1 >> 34) & 1ull) && warp >= 4) {
                            float d[4];
                            task_mma_tile<K, false>(S1 + 8 * IB, OY, lane, warp - 4, d);
                            store_or_add_tile<K>(S2 + 8 * IB, lane, warp - 4, d, (w2 >> 8) & 1u);
                        }
                    }
                    w2 |= made1;
                    __syncthreads();  // S2 complete; S1 free for the next group
                    if (s2_last) {
                        // stage 2: g component gt = warp from the summed S2; P -> (0, 0, 1),
                        // while P -> (0, 0, 0) is the dropped s->s product
                        const int gt = warp, a2 = gt >> 2;
                        const float *in[3] = {S2 + (gt & 3) * IB, S2 + ((gt & 3) + 4) * IB, S2 + 8 * IB};
                        const float *O[3] = {OZ + 2 * a2 * K2, OZ + (2 * a2 + 1) * K2, OZ + 2 * K2};
                        const unsigned valid = (unsigned)((sc2 >> (35 + 2 * gt)) & 3ull) | (gt == 4 ? (unsigned)((sc2 >> 51) & 1ull) << 2 : 0u);
                        task<K, 3, false>(in, O, valid, lane, sv);
                        accumulate<K>(acc, cmp, sv);
                    }
                }
            } else {
                int last = 0;
                constexpr int nsub = 8 / CG;
                for (int g = 0; g < nsub; g++)
                    if ((item.mask >> (8 * CG * g)) & ((1ull << (8 * CG)) - 1ull)) last = g;
                for (int sub = 0; sub < nsub; sub++) {
                    const unsigned long long gbits = (item.mask >> (8 * CG * sub)) & ((1ull << (8 * CG)) - 1ull);
                    if (gbits == 0ull) continue;
                    float *X0 = BUF, *X1 = BUF + 2 * CG * IB;
                    const int ft0 = CG * sub;
                    // stage 0: X0[(lft, a0)] = O^x_{a0, ft&1} f[ft]
                    for (int jx = warp; jx < 2 * CG; jx += NW) {
                        const int lft = jx >> 1, a0 = jx & 1, ft = ft0 + lft;
                        const unsigned col = (unsigned)((gbits >> (8 * lft)) & 0xffull);
                        if (!(col & (a0 ? 0xAAu : 0x55u))) continue;
                        const float *in[1] = {FB + ft * BLK};
                        const float *O[1] = {OX + (2 * a0 + (ft & 1)) * K2};
                        task<K, 1, true>(in, O, 1u, lane, sv);
                        store<K>(X0 + jx * IB, lane, sv);
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
                        const float *in[1] = {X0 + (2 * lft + (sidx & 1)) * IB};
                        const float *O[1] = {OY + (2 * (sidx >> 1) + ((ft >> 1) & 1)) * K2};
                        task<K, 1, false>(in, O, 1u, lane, sv);
                        store<K>(X1 + jx * IB, lane, sv);
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
                            in[lft] = X1 + (4 * lft + (gt & 3)) * IB;
                            O[lft] = OZ + (2 * (gt >> 2) + (ft >> 2)) * K2;
                            if ((gbits >> (8 * lft + gt)) & 1ull) valid |= 1u << lft;
                        }
                        task<K, CG, false>(in, O, valid, lane, sv);
                    }
                    accumulate<K>(acc, cmp, sv);
                    // no barrier before the next group: its stage 0 writes X0, which stage 2
                    // does not read, and its stage 1 writes X1 only after the next barrier
                }
            }
            prev = item;
            if (!S::KAHAN && ++since >= 16) {
#pragma unroll
                for (int r = 0; r < R; r++)
#pragma unroll
                    for (int jj = 0; jj < K; jj++) {
                        int c, j;
                        acc_cj<K>(lane, r, jj, c, j);
                        if (c < K2) G64[warp * K3 + c + K2 * j] += (double)acc[r][jj];
                        acc[r][jj] = 0.f;
                    }
                since = 0;
            }
            cp_async_wait_all();
            __syncthreads();  // next item's f and operator blocks ready; work blocks free
        }
        double *go = partial + (size_t)cix * 8 * K3;
#pragma unroll
        for (int r = 0; r < R; r++)
#pragma unroll
            for (int jj = 0; jj < K; jj++) {
                int c, j;
                acc_cj<K>(lane, r, jj, c, j);
                if (c < K2) {
                    const int e = warp * K3 + c + K2 * j;
                    go[e] = S::KAHAN ? (double)acc[r][jj] - (double)cmp[r][jj] : G64[e] + (double)acc[r][jj];
                }
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
// CTA (wi, comp) handles component comp of work entry wi: each thread sums
// up to 4 coefficients over the chunks with 4 chunks of loads in flight (the
// additions per coefficient stay in chunk order), so coarse levels with few
// g nodes and many chunks each still spread over 8 CTAs per node.
constexpr int kReduceThreads = 128;
// pen_begin / pen_partial (optional): the pencil contraction's task sums of
// each g (k_pencil.cu), added after its chunks, in task order.
__global__ void __launch_bounds__(kReduceThreads) k_reduce_chunks(const DevTree *gs, const int *work_tree, const int *work, const int *chunk_begin,
                                                                  const double *partial, int nc, const int *nw_dev, const int *pen_begin = nullptr,
                                                                  const double *pen_partial = nullptr) {
    constexpr int NT = kReduceThreads, E = 4, U = 4;
    const int tid = threadIdx.x, wi = blockIdx.x, comp = blockIdx.y;
    if (nw_dev && wi >= *nw_dev) return;
    const int gi = work[wi];
    const DevTree &g = gs[work_tree[wi]];
    const int c0 = chunk_begin[wi], c1 = chunk_begin[wi + 1];
    const int K3 = nc / 8;
    const double *src = partial + (size_t)comp * K3;
    double *go = g.coefs + (size_t)gi * nc + (size_t)comp * K3;
    double ss = 0.0;
    for (int e0 = tid; e0 < K3; e0 += E * NT) {
        bool ok[E];
        double v[E];
#pragma unroll
        for (int j = 0; j < E; j++) {
            ok[j] = e0 + j * NT < K3;
            v[j] = 0.0;
        }
        int c = c0;
        for (; c + U <= c1; c += U) {
            double q[U][E];
#pragma unroll
            for (int u = 0; u < U; u++)
#pragma unroll
                for (int j = 0; j < E; j++) q[u][j] = ok[j] ? src[(size_t)(c + u) * nc + e0 + j * NT] : 0.0;
#pragma unroll
            for (int u = 0; u < U; u++)
#pragma unroll
                for (int j = 0; j < E; j++) v[j] += q[u][j];
        }
        for (; c < c1; c++)
#pragma unroll
            for (int j = 0; j < E; j++) v[j] += ok[j] ? src[(size_t)c * nc + e0 + j * NT] : 0.0;
        if (pen_begin) {
            const double *psrc = pen_partial + (size_t)comp * K3;
            for (int t = pen_begin[wi]; t < pen_begin[wi + 1]; t++)
#pragma unroll
                for (int j = 0; j < E; j++) v[j] += ok[j] ? psrc[(size_t)t * nc + e0 + j * NT] : 0.0;
        }
#pragma unroll
        for (int j = 0; j < E; j++)
            if (ok[j]) {
                go[e0 + j * NT] = v[j];
                ss += v[j] * v[j];
            }
    }
    __shared__ double red[NT / 32];
    for (int o = 16; o > 0; o >>= 1) ss += __shfl_down_sync(0xffffffffu, ss, o);
    if ((tid & 31) == 0) red[tid >> 5] = ss;
    __syncthreads();
    if (tid == 0) {
        double t = 0.0;
        for (int wv = 0; wv < NT / 32; wv++) t += red[wv];
        g.norms[(size_t)gi * 8 + comp] = sqrt(t);
    }
}

}  // namespace mixed
}  // namespace mwgpu
