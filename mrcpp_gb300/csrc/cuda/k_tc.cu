// Tensor-core (tcgen05) contraction of the mixed form for order K = 8 (k = 7).
//
// The block schedule of tensorApplyOperComp (ConvolutionCalculator.cpp:333-382,
// per (g, f, term) the three 1D applications of the 2K x 2K operator to the
// (2K)^3 node tensor) as GEMMs on the 5th-generation tensor cores: one thread
// issues tcgen05.mma with both operands in shared memory, the accumulators
// live in tensor memory (TMEM), and the operands are staged with bulk copies
// (cp.async.bulk) that complete on mbarriers.
//
// Work items come in term-major order per output node (k_order_terms), so the
// items of an S1 group (same term, l_y, l_z) differ only in l_x:
//   stage 0 (x): S1 += f_item . O^x(l_x)            for every item of the group
//   stage 1 (y): S2 += S1 . O^y(l_y)                once per S1 group
//   stage 2 (z): g  += S2 . O^z(l_z)                once per S2 group (same term, l_z)
// which is the reference's sum of per-item products regrouped (O^y, O^z are
// the same for all items of a group).  The s->s product that the reference
// leaves out at depth > 0 (:261) is carried in separate channels (U after the
// x step, P after the xy step) and dropped at the last step.
//
// Every GEMM is D[128 x N] += A[128 x 8] B[N x 8]^T (kind::tf32, K-major
// operands without swizzle).  FP32 accuracy from TF32 operands: x = hi + lo
// with hi the TF32 rounding and lo = x - hi exactly; each product is
// lo.hi + hi.lo + hi.hi (the lo.lo term is below 2^-22 relative), so every
// A and B operand exists as a hi and a lo copy.
//
// Stage 0, tile t (b2 = t), rows m = b1 * 64 + (y + 8 z), k-step s = b0 (x):
//   columns 0-7:  a0 = 0 from b0 = 1 (C block)       8-15: a0 = 1 (B, A blocks)
//   columns 16-23: the T block on b0 = 0 (folded into a0 = 0, or the U channel
//   for b1 = b2 = 0 at depth > 0).
// Stage 1, tile t (b2 = t), rows m = a0 * 64 + (x' + 8 z), k = b1 * 8 + y, and
// for tile 0 at depth > 0 a third k-step with U; columns a1 = 0, a1 = 1, P.
// Stage 2, tile t (a0 = t), rows m = a1 * 64 + (x' + 8 y'), k = b2 * 8 + z (+ P);
// columns (a2, z').
// Between stages the threads read the accumulators from TMEM (tcgen05.ld),
// split them into hi / lo and store them transposed into the next stage's A
// operand (bank-conflict-free padded layout).  The per-g result is accumulated
// by the threads in compensated FP32 (Kahan) sums and written per chunk in
// FP64, like the CUDA-core kernel; k_reduce_chunks adds the chunks.
//
// Every wait on an mbarrier is bounded (about one second of clock cycles);
// on expiry the CTA sets DE_TIMEOUT, stops, waits (again bounded) for its
// tensor-core work in flight and frees its TMEM.
#include "mwgpu_internal.cuh"

namespace mwgpu {
namespace tc {

// ---- layouts (bytes) ----
constexpr int A0_REG = 4096;                  // (tile, k-step) region: 2 k-chunks x 16 row groups of 128 B
constexpr int A0_HALF = 4 * A0_REG;           // hi (or lo) of a node: 2 tiles x 2 k-steps
constexpr int A0_BYTES = 2 * A0_HALF;         // 32 KB per staged node
constexpr int A0_LBO = 2048, A0_SBO = 128;
constexpr int AG_BYTES = 2 * A0_REG;          // GenNode buffer: (tile 0, k-step 0), hi + lo
constexpr int B_LBO = 128, B_SBO = 256;       // operator forms: 8 x 8 blocks as 2 core matrices
constexpr int B0_F = 8 * 64, B1_F = 12 * 64, B2_F = 6 * 64;   // floats of one hi (or lo) form
constexpr int F_B0H = 0, F_B0L = B0_F, F_B1H = 2 * B0_F, F_B1L = F_B1H + B1_F, F_B2H = F_B1L + B1_F, F_B2L = F_B2H + B2_F;
static_assert(F_B2L + B2_F == kTcFormFloats, "operator form size");
constexpr int AT_SBO = 144, AT_LBO = 2368;    // transposed stage inputs: padded, conflict-free stores
constexpr int AT_T0 = 6 * AT_LBO, AT_T1 = 4 * AT_LBO, AT_HALF = AT_T0 + AT_T1, AT_BYTES = 2 * AT_HALF;
constexpr int NST = 3;                        // staged items in flight
constexpr int NT = 256;                       // threads: warps w and w + 4 share TMEM lanes 32 (w % 4) ..
// shared memory map
constexpr int SM_A0 = 0;
constexpr int SM_AG = SM_A0 + NST * A0_BYTES;
constexpr int SM_B0 = SM_AG + NST * AG_BYTES;
constexpr int SM_B1 = SM_B0 + NST * 2 * B0_F * 4;
constexpr int SM_B2 = SM_B1 + 2 * B1_F * 4;
constexpr int SM_AT = SM_B2 + 2 * B2_F * 4;
constexpr int SM_BYTES = SM_AT + AT_BYTES;
// TMEM columns
constexpr int TM_S1 = 0, TM_S2 = 128, TM_G = 176, TM_COLS = 256;  // S1: two buffers of 64 columns

__host__ __device__ constexpr uint32_t idesc(int M, int N) {
    // kind::tf32: D f32 (bit 4), A and B tf32 (2 at bits 7 and 10), K-major, N >> 3 at 17, M >> 4 at 24
    return (1u << 4) | (2u << 7) | (2u << 10) | ((uint32_t)(N >> 3) << 17) | ((uint32_t)(M >> 4) << 24);
}

__device__ __forceinline__ uint32_t su32(const void *p) { return (uint32_t)__cvta_generic_to_shared(p); }

// shared-memory matrix descriptor: start, leading (k) and stride (m / n) byte offsets, sm100 version, no swizzle
__device__ __forceinline__ uint64_t sdesc(uint32_t addr, uint32_t lbo, uint32_t sbo) {
    return (uint64_t)((addr >> 4) & 0x3FFFu) | ((uint64_t)((lbo >> 4) & 0x3FFFu) << 16) | ((uint64_t)((sbo >> 4) & 0x3FFFu) << 32) |
           ((uint64_t)1 << 46);
}

__device__ __forceinline__ void mma(uint32_t d, uint64_t a, uint64_t b, uint32_t id, uint32_t acc) {
    asm volatile(
        "{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
        "tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n\t}\n" ::"r"(d),
        "l"(a), "l"(b), "r"(id), "r"(acc));
}
// the three products of a hi / lo pair of operands
__device__ __forceinline__ void mma3(uint32_t d, uint64_t ah, uint64_t al, uint64_t bh, uint64_t bl, uint32_t id, uint32_t acc) {
    mma(d, al, bh, id, acc);
    mma(d, ah, bl, id, 1u);
    mma(d, ah, bh, id, 1u);
}
__device__ __forceinline__ void commit(uint64_t *bar) {
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(su32(bar)) : "memory");
}
__device__ __forceinline__ void bar_init(uint64_t *bar) { asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(su32(bar))); }
__device__ __forceinline__ void expect_tx(uint64_t *bar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(su32(bar)), "r"(bytes) : "memory");
}
__device__ __forceinline__ void bulk(void *dst, const void *src, uint32_t bytes, uint64_t *bar) {
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(su32(dst)), "l"(src),
                 "r"(bytes), "r"(su32(bar))
                 : "memory");
}
// bounded wait for the completion of the phase with the given parity
__device__ __forceinline__ bool bar_wait(uint64_t *bar, uint32_t parity) {
    const long long t0 = clock64();
    while (true) {
        uint32_t ok;
        asm volatile(
            "{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\tselp.u32 %0, 1, 0, p;\n\t}\n"
            : "=r"(ok)
            : "r"(su32(bar)), "r"(parity)
            : "memory");
        if (ok) return true;
        if (clock64() - t0 > (1ll << 31)) return false;
    }
}
__device__ __forceinline__ void fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void fence_async_smem() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }

template <int N>
__device__ __forceinline__ void tmem_ld(uint32_t taddr, float (&v)[N]);
template <>
__device__ __forceinline__ void tmem_ld<32>(uint32_t taddr, float (&v)[32]) {
    uint32_t r[32];
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,%16,%17,%18,%19,%20,%21,%22,%23,%24,"
        "%25,%26,%27,%28,%29,%30,%31}, [%32];"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]), "=r"(r[8]), "=r"(r[9]), "=r"(r[10]),
          "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15]), "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]),
          "=r"(r[21]), "=r"(r[22]), "=r"(r[23]), "=r"(r[24]), "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]),
          "=r"(r[31])
        : "r"(taddr));
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
    for (int i = 0; i < 32; i++) v[i] = __uint_as_float(r[i]);
}
template <>
__device__ __forceinline__ void tmem_ld<16>(uint32_t taddr, float (&v)[16]) {
    uint32_t r[16];
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]), "=r"(r[8]), "=r"(r[9]), "=r"(r[10]),
          "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
        : "r"(taddr));
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
    for (int i = 0; i < 16; i++) v[i] = __uint_as_float(r[i]);
}

// x = hi + lo: hi the TF32 rounding of x, lo the exact remainder
__device__ __forceinline__ void split(float x, float &hi, float &lo) {
    uint32_t h;
    asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(h) : "f"(x));
    hi = __uint_as_float(h);
    lo = x - hi;
}

// byte offset of element (m, k) of a transposed stage input (tile base added by the caller)
__device__ __forceinline__ int at_off(int m, int k) { return (m >> 3) * AT_SBO + (k >> 2) * AT_LBO + (m & 7) * 16 + (k & 3) * 4; }
__device__ __forceinline__ void at_store(unsigned char *at, int tile, int m, int k, float x) {
    float hi, lo;
    split(x, hi, lo);
    const int o = (tile ? AT_T0 : 0) + at_off(m, k);
    *reinterpret_cast<float *>(at + o) = hi;
    *reinterpret_cast<float *>(at + AT_HALF + o) = lo;
}

// operator node of (term, depth, l); the zero record outside the term's cache
__device__ __forceinline__ int oper_node(const DevOper &op, int term, int depth, int l) {
    const int off = op.dep_off[term * op.max_rows + depth], L0 = op.dep_L[term * op.max_rows + depth];
    return (off >= 0 && abs(l) <= L0) ? off + l + L0 : op.n_nodes;
}

__device__ __forceinline__ bool same_s1(const WorkItem &a, const WorkItem &b) {
    return a.term == b.term && a.tl[1] == b.tl[1] && a.tl[2] == b.tl[2];
}
__device__ __forceinline__ bool same_s2(const WorkItem &a, const WorkItem &b) { return a.term == b.term && a.tl[2] == b.tl[2]; }

__global__ void __launch_bounds__(NT, 1) k_contract_tc(DevMRA m, DevOper op, const DevTree *fs, const DevTree *gs, const int *work_tree,
                                                        const int *work, const int4 *chunks, int n_chunks_host, const int *n_chunks_dev,
                                                        const WorkItem *items, double *partial, int *err, int *counter) {
    extern __shared__ __align__(1024) unsigned char sm[];
    __shared__ __align__(8) uint64_t bar_full[NST], bar_mma[NST], bar_s1, bar_s2, bar_b1, bar_b2, bar_end;
    __shared__ uint32_t s_tmem;
    __shared__ int s_next;
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int quarter = warp & 3, half = warp >> 2;  // TMEM lanes 32 quarter .. ; tile = half
    unsigned char *A0 = sm + SM_A0, *AG = sm + SM_AG, *B0 = sm + SM_B0, *B1 = sm + SM_B1, *B2 = sm + SM_B2, *AT = sm + SM_AT;

    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(su32(&s_tmem)), "r"(TM_COLS));
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
    }
    if (tid == 0) {
        for (int i = 0; i < NST; i++) {
            bar_init(&bar_full[i]);
            bar_init(&bar_mma[i]);
        }
        bar_init(&bar_s1);
        bar_init(&bar_s2);
        bar_init(&bar_b1);
        bar_init(&bar_b2);
        bar_init(&bar_end);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    // zero the GenNode buffers (rows of f[2] stay zero) and the transposed
    // inputs (tile-0 rows 64-127 of k-chunks 4, 5 stay zero: U and P exist
    // for a0 = 0 / a1 = 0 only)
    for (int i = tid; i < NST * AG_BYTES / 16; i += NT) reinterpret_cast<float4 *>(AG)[i] = make_float4(0.f, 0.f, 0.f, 0.f);
    for (int i = tid; i < AT_BYTES / 16; i += NT) reinterpret_cast<float4 *>(AT)[i] = make_float4(0.f, 0.f, 0.f, 0.f);
    fence_async_smem();
    fence_before();
    __syncthreads();
    fence_after();
    const uint32_t tmem = s_tmem;
    const uint32_t lane_base = (uint32_t)(32 * quarter) << 16;
    const int n_chunks = n_chunks_dev ? *n_chunks_dev : n_chunks_host;

    // running counters (uniform over the CTA): staged items, stage-1 / stage-2 commits, B1 / B2 copies
    unsigned q = 0, n1 = 0, n2 = 0, nb1 = 0, nb2 = 0;
    // lbad: this thread saw a wait expire; bad: some thread did (CTA-uniform,
    // refreshed with __syncthreads_or, the only value control flow uses)
    bool lbad = false, bad = false;
    auto fail = [&]() {
        atomicOr(err, DE_TIMEOUT);
        lbad = true;
    };

    for (int cix = blockIdx.x; cix < n_chunks && !bad;) {
        const int4 ch = chunks[cix];
        if (ch.w == 1) {
            const int gi = work[ch.x];
            const int tree = work_tree[ch.x];
            const int depth = gs[tree].idx[gi].x - m.root_scale;
            const bool pure = depth > 0;  // the s->s product is left out
            const DevTree &f = fs[tree];
            const int cap_real = f.cap_real;
            const int it0 = ch.y, n = ch.z - ch.y;
            // thread: row r = 32 quarter + lane of tile `half` in every stage
            const int r = 32 * quarter + lane;
            float s1[32], s2[32], acc[16], cmp[16];
#pragma unroll
            for (int j = 0; j < 32; j++) s1[j] = s2[j] = 0.f;
#pragma unroll
            for (int j = 0; j < 16; j++) acc[j] = cmp[j] = 0.f;
            // thread 0: stage item j of this chunk (global index q + j) into buffer (q + j) % NST
            auto fetch = [&](int j) {
                const WorkItem it = items[it0 + j];
                const int b = (int)((q + (unsigned)j) % NST);
                expect_tx(&bar_full[b], (it.fid < cap_real ? (uint32_t)A0_BYTES : 4096u) + 4u * 2 * B0_F);
                if (it.fid < cap_real) {
                    const float *src = f.tc32 + (size_t)it.fid * kTcNodeFloats;
                    bulk(A0 + b * A0_BYTES, src, A0_HALF, &bar_full[b]);
                    bulk(A0 + b * A0_BYTES + A0_HALF, src + 4096, A0_HALF, &bar_full[b]);
                } else {
                    const float *src = f.gtc32 + (size_t)(it.fid - cap_real) * kTcGenFloats;
                    unsigned char *dst = AG + b * AG_BYTES;
                    bulk(dst, src, 1024, &bar_full[b]);
                    bulk(dst + A0_LBO, src + 256, 1024, &bar_full[b]);
                    bulk(dst + A0_REG, src + 512, 1024, &bar_full[b]);
                    bulk(dst + A0_REG + A0_LBO, src + 768, 1024, &bar_full[b]);
                }
                const float *form = op.btc + (size_t)oper_node(op, it.term, depth, it.tl[0]) * kTcFormFloats;
                bulk(B0 + b * 2 * B0_F * 4, form + F_B0H, 2 * B0_F * 4, &bar_full[b]);  // hi and lo forms are adjacent
            };
            if (tid == 0)
                for (int j = 0; j < NST - 1 && j < n; j++) fetch(j);
            WorkItem prev{}, cur{};
            // iteration k issues the x step of item k (TMEM buffer (q + k) & 1) and
            // drains item k - 1 into the register sums s1 (then the y and z steps
            // at the ends of its groups), so that the tensor core works on item k
            // while the threads read item k - 1
            for (int k = 0; k <= n && !bad; k++) {
                if (k < n && tid == 0) {
                    const WorkItem item = items[it0 + k];
                    const unsigned b = (q + (unsigned)k) % NST, ph = ((q + (unsigned)k) / NST) & 1u;
                    const uint32_t d = tmem + TM_S1 + 64 * ((q + (unsigned)k) & 1u);
                    if (!bar_wait(&bar_full[b], ph)) fail();
                    fence_after();
                    if (!lbad) {
                        const uint32_t idn = idesc(128, 32);
                        const uint32_t b_h = su32(B0 + b * 2 * B0_F * 4), b_l = b_h + B0_F * 4;
                        if (item.fid >= cap_real) {
                            const uint32_t a_h = su32(AG + b * AG_BYTES), a_l = a_h + A0_REG;
                            mma3(d, sdesc(a_h, A0_LBO, A0_SBO), sdesc(a_l, A0_LBO, A0_SBO), sdesc(b_h, B_LBO, B_SBO), sdesc(b_l, B_LBO, B_SBO), idn, 0u);
                        } else {
                            const uint32_t a_h = su32(A0 + b * A0_BYTES), a_l = a_h + A0_HALF;
#pragma unroll
                            for (int t = 0; t < 2; t++)
#pragma unroll
                                for (int s = 0; s < 2; s++) {
                                    const uint32_t ao = (2 * t + s) * A0_REG, bo = s * 4 * 256;
                                    mma3(d + 32 * t, sdesc(a_h + ao, A0_LBO, A0_SBO), sdesc(a_l + ao, A0_LBO, A0_SBO), sdesc(b_h + bo, B_LBO, B_SBO),
                                         sdesc(b_l + bo, B_LBO, B_SBO), idn, s > 0 ? 1u : 0u);
                                }
                        }
                    }
                    commit(&bar_mma[b]);  // also after a failed wait, so that the waiters below are released
                    // refill: item k + NST - 1 goes to the buffer of item k - 1, free once its products are done
                    if (k + NST - 1 < n && !lbad) {
                        const unsigned qp = q + (unsigned)k - 1u;
                        if (q + (unsigned)k >= 1u && !bar_wait(&bar_mma[qp % NST], (qp / NST) & 1u)) fail();
                        if (!lbad) fetch(k + NST - 1);
                    }
                }
                if (k == 0) continue;
                // ---- drain item j = k - 1 ----
                const int j = k - 1;
                prev = cur;
                cur = items[it0 + j];
                const bool has_next = j + 1 < n;
                WorkItem nx = cur;
                if (has_next) nx = items[it0 + j + 1];
                const bool s1_first = !(j > 0 && same_s1(prev, cur)), s1_last = !(has_next && same_s1(cur, nx));
                const bool s2_first = !(j > 0 && same_s2(prev, cur)), s2_last = !(has_next && same_s2(cur, nx));
                if (s1_first)
#pragma unroll
                    for (int i = 0; i < 32; i++) s1[i] = 0.f;
                if (s2_first)
#pragma unroll
                    for (int i = 0; i < 32; i++) s2[i] = 0.f;
                {
                    const unsigned qj = q + (unsigned)j;
                    if (!bar_wait(&bar_mma[qj % NST], (qj / NST) & 1u)) fail();
                    fence_after();
                    if (half == 0 || cur.fid < cap_real) {  // GenNode items write tile 0 only
                        float v[32];
                        tmem_ld<32>(tmem + lane_base + TM_S1 + 64 * (qj & 1u) + 32 * half, v);
#pragma unroll
                        for (int i = 0; i < 32; i++) s1[i] += v[i];
                    }
                }
                if (s1_last) {
                    // ---- S1 group complete: stage 1 ----
                    if (n1 > 0 && !bar_wait(&bar_s1, (n1 - 1) & 1u)) fail();  // A1 / B1 free (previous stage 1 done)
                    if (n2 > 0 && !bar_wait(&bar_s2, (n2 - 1) & 1u)) fail();  // (A2 aliases A1)
                    if (tid == 0) {
                        const float *form = op.btc + (size_t)oper_node(op, cur.term, depth, cur.tl[1]) * kTcFormFloats;
                        expect_tx(&bar_b1, 2 * B1_F * 4);
                        bulk(B1, form + F_B1H, 2 * B1_F * 4, &bar_b1);
                    }
                    {
                        // S1 tile t = half (b2 = t), row r = (b1, y, z)
                        const int t = half, b1 = r >> 6, y = r & 7, z = (r >> 3) & 7;
                        const bool u = pure && t == 0 && b1 == 0;
#pragma unroll
                        for (int xo = 0; xo < 8; xo++) {
                            at_store(AT, t, 8 * z + xo, 8 * b1 + y, u ? s1[xo] : s1[xo] + s1[16 + xo]);
                            at_store(AT, t, 64 + 8 * z + xo, 8 * b1 + y, s1[8 + xo]);
                            if (u) at_store(AT, 0, 8 * z + xo, 16 + y, s1[16 + xo]);
                        }
                    }
                    fence_async_smem();
                    fence_before();
                    bad = __syncthreads_or(lbad) != 0 || bad;
                    if (tid == 0 && !bad) {
                        fence_after();
                        if (!bar_wait(&bar_b1, nb1 & 1u)) fail();
                        const uint32_t a_h = su32(AT), a_l = a_h + AT_HALF, b_h = su32(B1), b_l = b_h + B1_F * 4;
#pragma unroll
                        for (int t = 0; t < 2; t++) {
                            const int nks = (t == 0 && pure) ? 3 : 2;
                            const uint32_t idn = idesc(128, t == 0 ? 32 : 16);
                            for (int s = 0; s < nks; s++) {
                                const uint32_t ao = (t ? AT_T0 : 0) + s * 2 * AT_LBO, bo = s * 4 * 256;
                                mma3(tmem + TM_S2 + 32 * t, sdesc(a_h + ao, AT_LBO, AT_SBO), sdesc(a_l + ao, AT_LBO, AT_SBO), sdesc(b_h + bo, B_LBO, B_SBO),
                                     sdesc(b_l + bo, B_LBO, B_SBO), idn, s > 0 ? 1u : 0u);
                            }
                        }
                    }
                    if (tid == 0) commit(&bar_s1);
                    nb1++;
                    n1++;
                    // drain the stage-1 products into the register sums s2
                    if (!bar_wait(&bar_s1, (n1 - 1) & 1u)) fail();
                    fence_after();
                    {
                        if (half == 0) {
                            float v[32];
                            tmem_ld<32>(tmem + lane_base + TM_S2, v);
#pragma unroll
                            for (int i = 0; i < 32; i++) s2[i] += v[i];
                        } else {
                            float v[16];
                            tmem_ld<16>(tmem + lane_base + TM_S2 + 32, v);
#pragma unroll
                            for (int i = 0; i < 16; i++) s2[i] += v[i];
                        }
                    }
                    if (s2_last && !bad) {
                        // ---- S2 group complete: stage 2 ----
                        if (tid == 0) {
                            const float *form = op.btc + (size_t)oper_node(op, cur.term, depth, cur.tl[2]) * kTcFormFloats;
                            expect_tx(&bar_b2, 2 * B2_F * 4);
                            bulk(B2, form + F_B2H, 2 * B2_F * 4, &bar_b2);
                        }
                        {
                            // S2 tile t = half (b2 = t), row r = (a0, z, x')
                            const int t = half, a0 = r >> 6, xo = r & 7, z = (r >> 3) & 7;
                            const bool p = pure && t == 0 && a0 == 0;
#pragma unroll
                            for (int yo = 0; yo < 8; yo++) {
                                at_store(AT, a0, 8 * yo + xo, 8 * t + z, s2[yo]);
                                at_store(AT, a0, 64 + 8 * yo + xo, 8 * t + z, s2[8 + yo]);
                                if (p) at_store(AT, 0, 8 * yo + xo, 16 + z, s2[16 + yo]);
                            }
                        }
                        fence_async_smem();
                        fence_before();
                        bad = __syncthreads_or(lbad) != 0 || bad;
                        if (tid == 0 && !bad) {
                            fence_after();
                            if (!bar_wait(&bar_b2, nb2 & 1u)) fail();
                            const uint32_t a_h = su32(AT), a_l = a_h + AT_HALF, b_h = su32(B2), b_l = b_h + B2_F * 4;
                            const uint32_t idn = idesc(128, 16);
#pragma unroll
                            for (int t = 0; t < 2; t++) {
                                const int nks = (t == 0 && pure) ? 3 : 2;
                                for (int s = 0; s < nks; s++) {
                                    const uint32_t ao = (t ? AT_T0 : 0) + s * 2 * AT_LBO, bo = s * 2 * 256;
                                    mma3(tmem + TM_G + 16 * t, sdesc(a_h + ao, AT_LBO, AT_SBO), sdesc(a_l + ao, AT_LBO, AT_SBO),
                                         sdesc(b_h + bo, B_LBO, B_SBO), sdesc(b_l + bo, B_LBO, B_SBO), idn, s > 0 ? 1u : 0u);
                                }
                            }
                        }
                        if (tid == 0) commit(&bar_s2);
                        nb2++;
                        n2++;
                        if (!bar_wait(&bar_s2, (n2 - 1) & 1u)) fail();
                        fence_after();
                        {
                            // g tile t = half (a0 = t), row r = (a1, y', x'); columns (a2, z')
                            float v[16];
                            tmem_ld<16>(tmem + lane_base + TM_G + 16 * half, v);
#pragma unroll
                            for (int i = 0; i < 16; i++) {
                                const float yv = v[i] - cmp[i];
                                const float tv = acc[i] + yv;
                                cmp[i] = (tv - acc[i]) - yv;
                                acc[i] = tv;
                            }
                        }
                    }
                }
                // every thread has read TMEM buffer (q + j) & 1 before item j + 2 is issued into it
                fence_before();
                bad = __syncthreads_or(lbad) != 0 || bad;
            }
            q += (unsigned)n;
            // partial of this chunk: component gt = a0 + 2 a1 + 4 a2, element x' + 8 y' + 64 z'
            {
                const int a0 = half, a1 = r >> 6, yo = (r >> 3) & 7, xo = r & 7;
                double *go = partial + (size_t)cix * 8 * 512;
#pragma unroll
                for (int j = 0; j < 16; j++) {
                    const int a2 = j >> 3, zo = j & 7, gt = a0 + 2 * a1 + 4 * a2;
                    go[gt * 512 + xo + 8 * yo + 64 * zo] = (double)acc[j] - (double)cmp[j];
                }
            }
        }
        bad = __syncthreads_or(lbad) != 0 || bad;
        if (!counter || bad) break;
        if (tid == 0) s_next = (int)gridDim.x + atomicAdd(counter, 1);
        __syncthreads();
        cix = s_next;
    }
    // wait (bounded) for the tensor-core work still in flight, then free TMEM
    __syncthreads();
    if (tid == 0) {
        fence_after();
        commit(&bar_end);
        bar_wait(&bar_end, 0);
    }
    fence_before();
    __syncthreads();
    fence_after();
    if (warp == 0) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(TM_COLS));
}

// ---- layouts made at upload / GenNode creation ----

// real nodes: element (b, x, yz) of node i -> tile b >> 2, k-step b & 1, row (b >> 1 & 1) 64 + yz, k = x.
// A component whose norm is below MachineZero is stored as zero: the reference
// skips such a component for every output node (ConvolutionCalculator.cpp:258)
__global__ void k_tree_layout(const double *coefs, const double *norms, int first, int n, float *tc) {
    const int i = first + blockIdx.x;
    if (blockIdx.x >= n) return;
    const double *src = coefs + (size_t)i * 4096;
    float *dst = tc + (size_t)i * kTcNodeFloats;
    for (int e = threadIdx.x; e < 4096; e += blockDim.x) {
        const int bb = e >> 9, r = e & 511, x = r & 7, yz = r >> 3;
        const int reg = 2 * (bb >> 2) + (bb & 1), mm = ((bb >> 1) & 1) * 64 + yz;
        const int o = reg * 1024 + (x >> 2) * 512 + (mm >> 3) * 32 + (mm & 7) * 4 + (x & 3);
        float hi, lo;
        split(norms[(size_t)i * 8 + bb] < kMachineZero ? 0.f : (float)src[e], hi, lo);
        dst[o] = hi;
        dst[4096 + o] = lo;
    }
}

// operator forms: slot tables of B0 (2 k-steps x 4), B1 (3 x 4), B2 (3 x 2); -1 = zero block
__constant__ int kSlotB0[8] = {-1, 2, 0, -1, 1, 3, -1, -1};
__constant__ int kSlotB1[12] = {0, 2, -1, -1, 1, 3, -1, -1, -1, 2, 0, -1};
__constant__ int kSlotB2[6] = {0, 2, 1, 3, -1, 2};

__global__ void k_oper_forms(DevOper op, const int4 *node_info, int n_nodes, float *forms) {
    const int nid = blockIdx.x;
    float *out = forms + (size_t)nid * kTcFormFloats;
    int4 ni = make_int4(0, 0, 0, 0);
    const int *w = nullptr;
    if (nid < n_nodes) {
        ni = node_info[nid];
        w = op.bw + ((size_t)ni.x * op.max_rows + ni.y) * 5;
    }
    const double *blk = op.blocks + (size_t)nid * 4 * 64;
    // slot element e = kc 32 + n 4 + kk: B[n][k = 4 kc + kk] = O(x_out = n, x_in = k) = block[k + 8 n]
    for (int e = threadIdx.x; e < (B0_F + B1_F + B2_F); e += blockDim.x) {
        int slot, base, hiofs, loofs;
        if (e < B0_F) {
            slot = kSlotB0[e >> 6];
            base = e;
            hiofs = F_B0H;
            loofs = F_B0L;
        } else if (e < B0_F + B1_F) {
            slot = kSlotB1[(e - B0_F) >> 6];
            base = e - B0_F;
            hiofs = F_B1H;
            loofs = F_B1L;
        } else {
            slot = kSlotB2[(e - B0_F - B1_F) >> 6];
            base = e - B0_F - B1_F;
            hiofs = F_B2H;
            loofs = F_B2L;
        }
        float hi = 0.f, lo = 0.f;
        if (nid < n_nodes && slot >= 0 && w[slot] >= 0 && abs(ni.z) <= w[slot]) {
            const int el = base & 63, kc = el >> 5, nn = (el >> 2) & 7, kk = el & 3;
            split((float)blk[slot * 64 + (4 * kc + kk) + 8 * nn], hi, lo);
        }
        out[hiofs + base] = hi;
        out[loofs + base] = lo;
    }
}

// chunk types: one warp per chunk, grid-stride (the count may be known on the device only)
__global__ void k_chunk_types(int4 *chunks, int n_chunks, const int *n_chunks_dev, const WorkItem *items) {
    const int lane = threadIdx.x & 31, nwarps = gridDim.x * (blockDim.x >> 5);
    const int nc = n_chunks_dev ? *n_chunks_dev : n_chunks;
    for (int c = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5); c < nc; c += nwarps) {
        const int4 ch = chunks[c];
        bool all_block = ch.y < ch.z;
        for (int i0 = ch.y; i0 < ch.z; i0 += 32) {
            const int i = i0 + lane;
            const bool ok = i >= ch.z || (items[i].flags & 1);
            if (!__all_sync(0xffffffffu, ok)) {
                all_block = false;
                break;
            }
        }
        if (lane == 0) chunks[c].w = all_block ? 1 : 0;
    }
}

}  // namespace tc

bool tc_supported(int K) { return K == 8; }

void launch_tc_tree_layout(const DevTree &t, int first, int n, cudaStream_t s) {
    if (n <= 0 || !t.tc32) return;
    tc::k_tree_layout<<<n, 256, 0, s>>>(t.coefs, t.norms, first, n, t.tc32);
}

void launch_tc_oper_forms(const DevOper &op, const int4 *node_info, int n_nodes, float *forms, cudaStream_t s) {
    tc::k_oper_forms<<<n_nodes + 1, 256, 0, s>>>(op, node_info, n_nodes, forms);
}

void launch_chunk_types(int4 *chunks, int n_chunks, const int *n_chunks_dev, const WorkItem *items, cudaStream_t s) {
    if (n_chunks <= 0) return;
    const int blocks = n_chunks_dev ? 4 * 152 : std::min((n_chunks + 7) / 8, 4 * 152);
    tc::k_chunk_types<<<blocks, 256, 0, s>>>(chunks, n_chunks, n_chunks_dev, items);
}

void launch_contract_tc(const DevMRA &m, const DevOper &op, const DevTree *fs, const DevTree *gs, const int *work_tree, const int *work,
                        const int4 *chunks, int n_chunks, const int *n_chunks_dev, const WorkItem *items, double *partial, int *err,
                        int *counter, cudaStream_t s) {
    if (n_chunks <= 0) return;
    static int sms = 0;
    if (sms == 0) {
        int dev = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        cudaFuncSetAttribute(tc::k_contract_tc, cudaFuncAttributeMaxDynamicSharedMemorySize, tc::SM_BYTES);
        if (sms <= 0) sms = 1;
    }
    const int grid = n_chunks_dev ? sms : std::min(sms, n_chunks);
    cudaMemsetAsync(counter, 0, sizeof(int), s);
    tc::k_contract_tc<<<grid, tc::NT, tc::SM_BYTES, s>>>(m, op, fs, gs, work_tree, work, chunks, n_chunks, n_chunks_dev, items, partial, err,
                                                         counter);
}

}  // namespace mwgpu
