// Pencil contraction of the mixed form for order K = 8 (k = 7): the x step
// on the 5th-generation tensor cores (tcgen05) with the operator terms
// stacked along N, the y and z steps as warp-level tensor-core products
// (mma.sync) in the consumer warps, concurrently with the next x step.
//
// What it computes.  For one output node g, one band cell l = (l_x, l_y, l_z)
// and one operator term i, the reference adds (ConvolutionCalculator.cpp:
// 277-382) the three 1D applications
//     g[gt] += O^z_i(l_z) O^y_i(l_y) O^x_i(l_x) f(g + l)[ft]
// over every (ft, gt) component its band and zero-norm rules keep, leaving
// out ft = gt = 0 below the roots (:261).  Without norm screening (levels
// whose gThreshold is negative, ConvolutionCalculator.cpp:241-248 -- the
// fixed-grid applies and the first TreeBuilder iteration) the kept set is
// structural: an operator block (a, b) of a direction takes part iff
// |l_d| <= bw_i[2a+b], and an f component takes part iff its norm is at least
// MachineZero.  Both are folded into the operands (zeroed operator blocks,
// zeroed f components), so the dense block products below equal the sum of
// the reference's component products.  This kernel takes the terms whose band
// width at the depth is at most kPencilMaxW (the item kernel the wider ones).
//
// Schedule.  The cells of one g with the same (l_y, l_z) form a pencil along
// x.  A pencil's f nodes f(g + (l_x, l_y, l_z)) are the A operand of every
// term, so the terms are stacked along N:
//     S1[(y,z)][(j, c)] = sum_{l_x} sum_{x_in} f(l_x)[(y,z)][x_in] B_j(l_x)[c][x_in]
// (tcgen05.mma kind::tf32, M = 128 rows per z half, N = 24 per term, up to 5
// terms per product, K = 8 per instruction, 3 products of TF32 hi / lo parts
// for FP32 accuracy; measured on this GPU a tcgen05.mma costs about 131 cycles
// for any N up to 128 and 170 cycles at N = 256, so only wide N pays, and
// legacy mma.sync shares the same tensor pipe).  The 24 columns of a term are
// its x-step outputs a0 = 0 from b0 = 1 (C block), a0 = 1 (B, A blocks) and
// a0 = 0 from b0 = 0 (T block), so that the s->s path can be split off (U
// channel below).  Per term the consumers then apply the y and z steps with
// warp-level tensor-core products (mma.sync m16n8k8, TF32 hi / lo, 3 products):
//     Y^T[y_out][(x, z)] = O^y[y_out][y_in] S1^T[y_in][(x, z)]
//     G[(x, y)][z_out]  += Y[(x, y)][z_in] O^z[z_out][z_in]^T
// the accumulator fragments of the first product are the A fragments of the
// second (the k index of the z step is permuted to match, and so are the O^z
// fragments), so Y never leaves the registers.
// Below the roots the T-block part of S1 on the (b1, b2) = (0, 0) rows is the
// U channel: it goes through y with the B block (a1 = 1) into Y and with the T
// block into P, and P goes through z with the B block only (a2 = 1), which
// leaves out exactly the T.T.T path from f[0] to g[0].
//
// Roles (128 + 32 x 8 threads): warp 0 lane 0 stages operands with
// cp.async.bulk into mbarrier-tracked slots (a pencil's f nodes once for all
// its term groups, stacked operator forms); warp 1 lane 0 issues the
// tensor-core products and commits into one of two TMEM buffers, so that the
// products of the next unit overlap the consumers; warps 2 and 3 only give
// their registers to the consumers (setmaxnreg); warps 4-11 (consumers; warp
// 4 + w owns x = w and w + 8, so that each has one x of the U channel; or
// warps 4-19 with one x each) read TMEM, transpose S1 through shared memory,
// load their y / z operator fragments (op.pfrag, split and masked at operator
// upload), run the y / z steps and keep the g accumulators (FP32 sums per
// unit, compensated sums over the units) of the task.  A task is (g, l_z): its
// pencils x their term groups ("units", made by the host and
// k_pencil_units); its 8 (k+1)^3 sums go to pen_partial[slot] in FP64, and the
// chunk reduction adds the tasks of g after its chunk partials.
//
// Every wait is bounded (about a second of cycles); on expiry a thread sets
// DE_TIMEOUT, its role stops, the others then time out too, and the CTA
// waits (bounded) for its tensor-core work and frees TMEM.
#include "mwgpu_internal.cuh"

namespace mwgpu {
namespace pencil {

// threads: warpgroup 0 (producer warp, MMA warp, two idle warps), then NCW
// consumer warps (8 or 16: a tile-shape parameter of the plan autotuner; 16
// warps own one x each, 8 warps two)
template <int NCW> __host__ __device__ constexpr int n_threads() { return 128 + 32 * NCW; }
// register split (setmaxnreg): warpgroup 0 hands registers to the consumer
// warpgroups.  The shares must fit in what the CTA is launched with (threads x
// registers per thread): checked on the host before the first launch
// (pencil_shape_ok), since a setmaxnreg.inc that cannot be served waits.
template <int NCW> struct Regs;
template <> struct Regs<8> { static constexpr int prod = 56, cons = 216; };
template <> struct Regs<16> { static constexpr int prod = 40, cons = 104; };
constexpr int GT = kPencilGroup;          // terms per group (per product)
constexpr int CPT = 24;                    // D columns per term
constexpr int NMAX = (GT * CPT + 15) / 16 * 16;   // 128: two D buffers of two tiles fit the 512 TMEM columns
constexpr int NFS = kPencilRing;           // f buffers: a ring through which a unit's x slots pass
constexpr int FREC = kTcNodeFloats * 4;    // bytes of a staged real node (hi 16 KB, lo 16 KB)
constexpr int GREC = 8192;                 // bytes of a staged GenNode (hi 4 KB, lo 4 KB; rows 64-127 zero)
constexpr int BREC = 128 * NMAX;           // bytes of a stacked form (hi s0, hi s1, lo s0, lo s1)
// S1 staging (double-buffered by term): S1[x][y][z] at x XS + y YS + z, U[x][y][z] at
// x US + y UYS + z (strides chosen so that the fragment loads avoid bank conflicts)
constexpr int YS = 24, XS = 16 * YS, UYS = 8, US = 64;
constexpr int S1_FLOATS = 16 * XS + 8 * US;
// shared memory map (bytes)
constexpr int SM_F = 0;                              // NFS real-node buffers
constexpr int SM_G = SM_F + NFS * FREC;              // NFS GenNode buffers (a ring entry's node is real or generated)
constexpr int SM_B = SM_G + NFS * GREC;              // 2 form slots
constexpr int SM_S1 = SM_B + 2 * BREC;               // S1 staging
constexpr int SM_BYTES = SM_S1 + 2 * 4 * S1_FLOATS;
static_assert(SM_BYTES + 1024 <= 227 * 1024, "pencil kernel shared memory");
static_assert(SM_F % 1024 == 0 && SM_G % 1024 == 0 && SM_B % 1024 == 0 && SM_S1 % 16 == 0, "alignment");
constexpr int TM_COLS = 512;                         // D buffer db at column 256 db, tile t at + 128 t
constexpr long long kSpin = 1ll << 31;               // about a second at 2 GHz

__host__ __device__ constexpr uint32_t idesc(int M, int N) {
    // kind::tf32: D f32, A and B tf32, both K-major, N >> 3 at bit 17, M >> 4 at bit 24
    return (1u << 4) | (2u << 7) | (2u << 10) | ((uint32_t)(N >> 3) << 17) | ((uint32_t)(M >> 4) << 24);
}
__device__ __forceinline__ uint32_t su32(const void *p) { return (uint32_t)__cvta_generic_to_shared(p); }
// shared-memory matrix descriptor: no swizzle, K-major; lbo = byte stride between
// the two 16-byte k chunks, sbo = byte stride between 8-row groups
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
__device__ __forceinline__ void commit(uint64_t *bar) {
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(su32(bar)) : "memory");
}
__device__ __forceinline__ void bar_init(uint64_t *bar, int count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(su32(bar)), "r"(count));
}
__device__ __forceinline__ void bar_arrive(uint64_t *bar) {
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(su32(bar)) : "memory");
}
__device__ __forceinline__ void expect_tx(uint64_t *bar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(su32(bar)), "r"(bytes) : "memory");
}
__device__ __forceinline__ void bulk(void *dst, const void *src, uint32_t bytes, uint64_t *bar) {
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(su32(dst)), "l"(src),
                 "r"(bytes), "r"(su32(bar))
                 : "memory");
}
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
        if (clock64() - t0 > kSpin) return false;
    }
}
__device__ __forceinline__ void fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }
template <int NCW> __device__ __forceinline__ void consumers_sync() { asm volatile("bar.sync 1, %0;" ::"n"(32 * NCW) : "memory"); }
// true on every consumer thread iff v is true on all of them (named barrier 1,
// so that control flow around the consumers' barriers stays uniform)
template <int NCW> __device__ __forceinline__ bool consumers_all(bool v) {
    uint32_t r;
    asm volatile(
        "{\n\t.reg .pred p, q;\n\tsetp.ne.u32 q, %1, 0;\n\tbar.red.and.pred p, 1, %2, q;\n\tselp.u32 %0, 1, 0, p;\n\t}\n"
        : "=r"(r)
        : "r"((uint32_t)v), "n"(32 * NCW)
        : "memory");
    return r != 0;
}

__device__ __forceinline__ void tmem_ld4(uint32_t taddr, float (&v)[4]) {
    uint32_t r[4];
    asm volatile("tcgen05.ld.sync.aligned.32x32b.x4.b32 {%0,%1,%2,%3}, [%4];" : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]) : "r"(taddr));
#pragma unroll
    for (int i = 0; i < 4; i++) v[i] = __uint_as_float(r[i]);
}
__device__ __forceinline__ void tmem_ld2(uint32_t taddr, float (&v)[2]) {
    uint32_t r[2];
    asm volatile("tcgen05.ld.sync.aligned.32x32b.x2.b32 {%0,%1}, [%2];" : "=r"(r[0]), "=r"(r[1]) : "r"(taddr));
    v[0] = __uint_as_float(r[0]);
    v[1] = __uint_as_float(r[1]);
}
// n consecutive TMEM columns of this thread's lane (n = 4 or 2)
template <int n> __device__ __forceinline__ void tmem_ldn(uint32_t taddr, float (&v)[n]) {
    if constexpr (n == 4) tmem_ld4(taddr, v);
    else tmem_ld2(taddr, v);
}
__device__ __forceinline__ void tmem_wait_ld() { asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory"); }

// x = hi + lo: hi the TF32 rounding of x, lo the exact remainder
__device__ __forceinline__ void split(float x, float &hi, float &lo) {
    uint32_t h;
    asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(h) : "f"(x));
    hi = __uint_as_float(h);
    lo = x - hi;
}

// (not volatile: a pure function of its operands, so that independent products
// can be scheduled between dependent ones)
__device__ __forceinline__ void mma16(float (&d)[4], const float (&a)[4], const float (&b)[2]) {
    asm("mma.sync.aligned.m16n8k8.row.col.f32.tf32.tf32.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, {%0,%1,%2,%3};\n"
                 : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
                 : "r"(__float_as_uint(a[0])), "r"(__float_as_uint(a[1])), "r"(__float_as_uint(a[2])), "r"(__float_as_uint(a[3])),
                   "r"(__float_as_uint(b[0])), "r"(__float_as_uint(b[1])));
}
// d += a b in FP32 accuracy from TF32 operands: lo.hi + hi.lo + hi.hi
__device__ __forceinline__ void mma3x(float (&d)[4], const float (&ah)[4], const float (&al)[4], const float (&bh)[2], const float (&bl)[2]) {
    mma16(d, al, bh);
    mma16(d, ah, bl);
    mma16(d, ah, bh);
}
// the same with the two correction products in their own accumulator dl (d + dl
// is the sum): two dependency chains instead of one
__device__ __forceinline__ void mma3x2(float (&d)[4], float (&dl)[4], const float (&ah)[4], const float (&al)[4], const float (&bh)[2],
                                       const float (&bl)[2]) {
    mma16(dl, al, bh);
    mma16(d, ah, bh);
    mma16(dl, ah, bl);
}

// padded N of a tensor-core product with n terms (M = 128 needs N % 16 == 0)
__host__ __device__ constexpr int n_pad(int n) { return (CPT * n + 15) / 16 * 16; }

// ---------------------------------------------------------------------------
// Stacked operator forms: per (depth, group, slot b: l_x = 0, -k, +k) the B
// operand of the x step for the group's terms (rows q .. of the depth's term
// rows, band width <= kPencilMaxW, GT per group) that reach |l_x|.  Row
// n = 24 j + c (term j of the group, column c), k = 8 s + q0 (s = b0, the
// input x bit; q0 the input index):
//   c in  0..7:  a0 = 0, p0 = c      from b0 = 1 (C block, idx 1)
//   c in  8..15: a0 = 1, p0 = c - 8  (B block idx 2 from b0 = 0, A block idx 3 from b0 = 1)
//   c in 16..23: a0 = 0, p0 = c - 16 from b0 = 0 (T block, idx 0)
// value = block[q0 + K p0] (MRCPP's K x K column-major block of g = f^T op),
// zero where |l_x| > bw[idx].  Layout per k step s: (n >> 3) 256 + (k >> 2) 128
// + (n & 7) 16 + (k & 3) 4 bytes (LBO 128, SBO 256); hi s0, hi s1, lo s0, lo s1,
// each 32 N_pad bytes.
__global__ void k_stack_forms(DevOper op, const PencilFormJob *jobs, int n_jobs, float *forms) {
    const int jb = blockIdx.x;
    if (jb >= n_jobs) return;
    const PencilFormJob J = jobs[jb];
    const int N = n_pad(J.nt);
    const int T = op.n_terms;
    float *out = forms + J.off;
    const int per = 16 * N;  // elements per hi (or lo) copy: N rows x 16 k
    for (int e = threadIdx.x; e < per; e += blockDim.x) {
        const int n = e >> 4, k = e & 15, s = k >> 3, kl = k & 7;
        float hi = 0.f, lo = 0.f;
        if (n < CPT * J.nt) {
            const int j = n / CPT, c = n % CPT;
            const TermRow row = op.term_rows[(size_t)J.depth * T + J.q + j];
            int idx = -1, p0 = 0;
            if (c < 8) { if (s == 1) idx = 1; p0 = c; }
            else if (c < 16) { idx = s == 0 ? 2 : 3; p0 = c - 8; }
            else { if (s == 0) idx = 0; p0 = c - 16; }
            if (idx >= 0 && row.off >= 0 && abs(J.lx) <= row.L0 && abs(J.lx) <= row.wd[idx]) {
                const double v = op.blocks[((size_t)(row.off + J.lx + row.L0) * 4 + idx) * 64 + kl + 8 * p0];
                split((float)v, hi, lo);
            }
        }
        const int o = s * 8 * N + (n >> 3) * 64 + (kl >> 2) * 32 + (n & 7) * 4 + (kl & 3);
        out[o] = hi;
        out[16 * N + o] = lo;
    }
}

// ---------------------------------------------------------------------------
// The consumers' operator fragments, per (depth, term row r, |l| <= kPencilMaxL) one
// record of kPencilFragFloats, made at operator upload: the TF32 hi / lo parts
// of the blocks in the mma.sync fragment order of each lane, the blocks (a, b)
// outside the band (|l| > bw[2a + b]) zero.  Lane (g, tq), g = lane / 4,
// tq = lane % 4, of a direction's blocks O (blocks32[idx 64 + 8 i + o] = the
// K x K block idx, transposed):
//   y part, per k step s: float4 hi, float4 lo of
//     {O_s[8 tq + g], O_(2+s)[8 tq + g], O_s[8 (tq+4) + g], O_(2+s)[8 (tq+4) + g]}
//     at floats 256 s + 8 lane (the A fragments of the y step);
//   z part, per (a2, s), idx = 2 a2 + s: {hi, hi, lo, lo} of
//     {O_idx[8 (2 tq) + g], O_idx[8 (2 tq + 1) + g]} at floats 512 + 128 idx + 4 lane
//     (the B fragments of the z step, k permuted).
__global__ void k_pencil_frags(DevOper op, float *frags) {
    const int T = op.n_terms;
    const int slot = blockIdx.x, l = slot % kPencilFragL - kPencilMaxL, tr = slot / kPencilFragL, r = tr % T, dd = tr / T;
    const TermRow row = op.term_rows[(size_t)dd * T + r];
    const bool exists = row.off >= 0 && abs(l) <= row.L0;
    const float *blk = exists ? op.blocks32 + (size_t)(row.off + l + row.L0) * 256 : nullptr;
    float *out = frags + (size_t)slot * kPencilFragFloats;
    for (int e = threadIdx.x; e < kPencilFragFloats; e += blockDim.x) {
        float v = 0.f;
        bool lo_part;
        if (e < 512) {
            const int s = e >> 8, lane = (e >> 3) & 31, q = e & 7, qq = q & 3, g = lane >> 2, tq = lane & 3;
            lo_part = q >= 4;
            const int idx = (qq & 1) ? 2 + s : s;
            const int i = (qq & 2) ? tq + 4 : tq;
            if (exists && abs(l) <= row.wd[idx]) v = blk[idx * 64 + 8 * i + g];
        } else {
            const int f = e - 512, idx = f >> 7, lane = (f >> 2) & 31, q = f & 3, g = lane >> 2, tq = lane & 3;
            lo_part = q >= 2;
            if (exists && abs(l) <= row.wd[idx]) v = blk[idx * 64 + 8 * (2 * tq + (q & 1)) + g];
        }
        float hi, lo;
        split(v, hi, lo);
        out[e] = lo_part ? lo : hi;
    }
}

// ---------------------------------------------------------------------------
// Units (PencilUnit, mwgpu_internal.cuh): made on the host from the topology;
// k_pencil_units fills the f nodes of the pencil and what the contraction
// needs to know about them.
using Unit = PencilUnit;

__device__ inline bool node_nonzero(const DevTree &f, int fid) {
    const double *nrm = f.norms + (size_t)fid * 8;
    if (fid >= f.cap_real) return !(nrm[0] < kMachineZero);
    for (int c = 0; c < 8; c++)
        if (!(nrm[c] < kMachineZero)) return true;
    return false;
}

__device__ __forceinline__ int slot_lx(int b) { return b == 0 ? 0 : ((b & 1) ? -((b + 1) >> 1) : (b >> 1)); }

__global__ void k_pencil_units(DevMRA m, const DevTree *fs, const DevTree *gs, const int *work_tree, const int *work, Unit *units, int n_units,
                               int *err) {
    const int u = blockIdx.x * blockDim.x + threadIdx.x;
    if (u >= n_units) return;
    Unit U = units[u];
    const int tr = work_tree[U.wi];
    const DevTree &f = fs[tr];
    const int4 gx = gs[tr].idx[work[U.wi]];
    int flags = 0, w0 = 0, w1 = 0;
    for (int b = 0; b < kPencilSlots; b++) {
        U.fid[b] = -1;
        const int lx = slot_lx(b);
        if (abs(lx) > U.xw || U.ntk[abs(lx)] == 0) continue;
        NodeKey key;
        if (!pack_key(m, gx.x, gx.y + lx, gx.z + U.ly, gx.w + U.lz, key)) continue;  // outside the world
        const int fid = hash_find(f.hkeys, f.hvals, f.hcap, key);
        if (fid < 0) {
            atomicOr(err, DE_LOOKUP);
            continue;
        }
        if (!node_nonzero(f, fid)) continue;
        U.fid[b] = fid;
        const bool gen = fid >= f.cap_real;
        if (gen) flags |= 1 << b;
        // the first product of a tile (slot order) sets how many terms its D holds
        const int n = U.ntk[abs(lx)];
        if (w0 == 0) w0 = n;
        if (w1 == 0 && !gen) w1 = n;
    }
    U.flags = flags;
    U.wt0 = (short)w0;
    U.wt1 = (short)w1;
    units[u] = U;
}

// ---------------------------------------------------------------------------
// The contraction.
template <int NCW>
__global__ void __launch_bounds__(n_threads<NCW>(), 1) k_pencil(DevOper op, const DevTree *fs, const int *work_tree, const Unit *units,
                                                               const int *task_unit, int n_tasks, double *pen_partial, int *err, int *counter) {
    static_assert(NCW == 8 || NCW == 16, "consumer warps");
    constexpr int NT = n_threads<NCW>();
    constexpr int XPW = 16 / NCW;   // x values per consumer warp
    constexpr int CPP = 32 / NCW;   // drained columns of each 8-column block per consumer warp
    extern __shared__ __align__(1024) unsigned char sm[];
    __shared__ __align__(8) uint64_t f_full[NFS], f_empty[NFS], b_full[2], b_empty[2], d_full[2], d_empty[2], bar_end;
    __shared__ uint32_t s_tmem;
    __shared__ int s_task;
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int T = op.n_terms;

    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(su32(&s_tmem)), "r"(TM_COLS));
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
    }
    if (tid == 0) {
        for (int i = 0; i < NFS; i++) {
            bar_init(&f_full[i], 1);
            bar_init(&f_empty[i], 1);
        }
        for (int i = 0; i < 2; i++) {
            bar_init(&b_full[i], 1);
            bar_init(&b_empty[i], 1);
            bar_init(&d_full[i], 1);
            bar_init(&d_empty[i], NCW);
        }
        bar_init(&bar_end, 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    // GenNode slots: rows 64-127 of both k chunks stay zero (only the b1 = 0 rows are copied)
    for (int i = tid; i < NFS * GREC / 16; i += NT) reinterpret_cast<float4 *>(sm + SM_G)[i] = make_float4(0.f, 0.f, 0.f, 0.f);
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    fence_before();
    __syncthreads();
    fence_after();
    const uint32_t tmem = s_tmem;

    // running counters (the producer and the MMA lane walk the same units and nodes)
    unsigned nu = 0;            // units done
    unsigned nb = 0;            // forms
    unsigned nfr = 0;           // f nodes staged (producer) / consumed (MMA) through the ring
    bool lbad = false;
    auto fail = [&]() {
        if (!lbad) atomicOr(err, DE_TIMEOUT);
        lbad = true;
    };
    // consumer warp cw owns x = cw + NCW xi (xi < XPW: with 8 warps one x of the
    // U channel (x < 8) and one without, so that the warps' work per term is
    // even); fragment coordinates g (group), tq (thread in group)
    const int cw = warp >= 4 ? warp - 4 : 0;
    const int fg = lane >> 2, tq = lane & 3;
    auto xof = [&](int xi) { return cw + NCW * xi; };
    float *S1base = reinterpret_cast<float *>(sm + SM_S1);

    // each role runs its own task loop after the register split (the CTA
    // barriers of a task match across the roles: one sync, one reduction)
    if (warp < 4) {
        asm volatile("setmaxnreg.dec.sync.aligned.u32 %0;" ::"n"(Regs<NCW>::prod));
        for (;;) {
            if (tid == 0) s_task = atomicAdd(counter, 1);
            __syncthreads();
            const int task = s_task;
            if (task >= n_tasks) break;
            const int u0 = task_unit[task], u1 = task_unit[task + 1];
            if (warp == 0) {
                // ---------------- producer ----------------
                if (lane == 0 && !lbad) {
                    for (int u = u0; u < u1 && !lbad; u++) {
                        const Unit &U = units[u];
                        const DevTree &f = fs[work_tree[U.wi]];
                        // slot by slot: the f node into the next ring buffer, then the
                        // slot's stacked form (the MMA lane takes them in this order)
                        for (int b = 0; b <= 2 * U.xw && !lbad; b++) {
                            const int fid = U.fid[b];
                            if (fid < 0) continue;
                            const int r = (int)(nfr % NFS);
                            if (nfr >= NFS && !bar_wait(&f_empty[r], ((nfr / NFS) - 1) & 1)) { fail(); break; }
                            if (fid < f.cap_real) {
                                expect_tx(&f_full[r], FREC);
                                bulk(sm + SM_F + r * FREC, f.tc32 + (size_t)fid * kTcNodeFloats, FREC, &f_full[r]);
                            } else {
                                const float *src = f.gtc32 + (size_t)(fid - f.cap_real) * kTcGenFloats;
                                unsigned char *dst = sm + SM_G + r * GREC;
                                expect_tx(&f_full[r], 4096);
                                bulk(dst, src, 1024, &f_full[r]);               // hi, k chunk 0, rows 0-63
                                bulk(dst + 2048, src + 256, 1024, &f_full[r]);  // hi, k chunk 1
                                bulk(dst + 4096, src + 512, 1024, &f_full[r]);  // lo, k chunk 0
                                bulk(dst + 6144, src + 768, 1024, &f_full[r]);  // lo, k chunk 1
                            }
                            nfr++;
                            const int s = nb & 1;
                            if (nb >= 2 && !bar_wait(&b_empty[s], ((nb >> 1) - 1) & 1)) { fail(); break; }
                            const uint32_t bytes = 128u * (uint32_t)n_pad(U.nform[b]);
                            expect_tx(&b_full[s], bytes);
                            bulk(sm + SM_B + s * BREC, op.btc_stack + U.form[b], bytes, &b_full[s]);
                            nb++;
                        }
                        if (lbad) break;
                        nu++;
                    }
                }
            } else if (warp == 1) {
                // ---------------- MMA issue ----------------
                if (lane == 0 && !lbad) {
                    for (int u = u0; u < u1 && !lbad; u++) {
                        const Unit &U = units[u];
                        const DevTree &f = fs[work_tree[U.wi]];
                        const int db = nu & 1;
                        // the consumers have read this D buffer (unit nu - 2)
                        if (nu >= 2 && !bar_wait(&d_empty[db], ((nu >> 1) - 1) & 1)) { fail(); break; }
                        fence_after();
                        const uint32_t dbase = tmem + 256u * db;
                        bool first[2] = {true, true};
                        for (int b = 0; b <= 2 * U.xw && !lbad; b++) {
                            const int fid = U.fid[b];
                            if (fid < 0) continue;
                            const int r = (int)(nfr % NFS);
                            if (!bar_wait(&f_full[r], (nfr / NFS) & 1)) { fail(); break; }
                            const bool gen = fid >= f.cap_real;
                            const uint32_t a_hi = gen ? su32(sm + SM_G + r * GREC) : su32(sm + SM_F + r * FREC);
                            const int nt_tiles = gen ? 1 : 2, nks = gen ? 1 : 2;
                            const int sbix = nb & 1;
                            if (!bar_wait(&b_full[sbix], (nb >> 1) & 1)) { fail(); break; }
                            nb++;
                            fence_after();
                            const int nt = U.ntk[(b + 1) >> 1];
                            const int N = n_pad(nt), NF = n_pad(U.nform[b]);   // product N; the form's own N sets its layout
                            const uint32_t id = idesc(128, N);
                            const uint32_t b_hi = su32(sm + SM_B + sbix * BREC), b_lo = b_hi + 64u * NF;
                            // real nodes: region (tile t, k step s) at (2 t + s) 4 KB, lo at +16 KB;
                            // GenNodes: one region, lo at +4 KB
                            const uint32_t lo_off = gen ? 4096u : 16384u;
                            for (int t = 0; t < nt_tiles; t++)
                                for (int s = 0; s < nks; s++) {
                                    const uint32_t ao = gen ? 0u : (uint32_t)(2 * t + s) * 4096u, bo = (uint32_t)s * 32u * NF;
                                    const uint64_t ah = sdesc(a_hi + ao, 2048, 128), al = sdesc(a_hi + lo_off + ao, 2048, 128);
                                    const uint64_t bh = sdesc(b_hi + bo, 128, 256), bl = sdesc(b_lo + bo, 128, 256);
                                    const uint32_t d = dbase + 128u * t;
                                    const uint32_t acc0 = (first[t] && s == 0) ? 0u : 1u;
                                    mma(d, al, bh, id, acc0);
                                    mma(d, ah, bl, id, 1u);
                                    mma(d, ah, bh, id, 1u);
                                }
                            for (int t = 0; t < nt_tiles; t++) first[t] = false;
                            commit(&b_empty[sbix]);    // the form and the f buffer are free once these products finish
                            commit(&f_empty[r]);
                            nfr++;
                        }
                        commit(&d_full[db]);           // also after a failure, so that the consumers are released
                        nu++;
                    }
                }
            }
            // the producer / MMA lanes other than 0 did not walk the units: bring their counters along
            if (warp <= 1) {
                nu = __shfl_sync(0xffffffffu, nu, 0);
                nb = __shfl_sync(0xffffffffu, nb, 0);
                nfr = __shfl_sync(0xffffffffu, nfr, 0);
            }
            if (__syncthreads_or(lbad) != 0) {
                lbad = true;
                break;
            }
        }
    } else {
        asm volatile("setmaxnreg.inc.sync.aligned.u32 %0;" ::"n"(Regs<NCW>::cons));
        float G[8 * XPW], Gc[8 * XPW];
        for (;;) {
            __syncthreads();
            const int task = s_task;
            if (task >= n_tasks) break;
            const int u0 = task_unit[task], u1 = task_unit[task + 1];
#pragma unroll
            for (int i = 0; i < 8 * XPW; i++) G[i] = Gc[i] = 0.f;
            {
                // ---------------- consumers ----------------
                const int quarter = warp & 3, part = cw >> 2;   // TMEM lanes 32 quarter ..; drained columns CPP part ..
                const int r = 32 * quarter + lane;              // D row of this thread: b1 64 + q1 + 8 q2
                const int b1 = r >> 6, q1 = r & 7, q2 = (r >> 3) & 7;
                const int yrow = 8 * b1 + q1;
                unsigned nterm = 0;   // terms drained (S1 buffer parity)
                for (int u = u0; u < u1; u++) {
                    const int db = nu & 1;
                    bool ok = !lbad;
                    if (ok && !bar_wait(&d_full[db], (nu >> 1) & 1)) { fail(); ok = false; }
                    ok = consumers_all<NCW>(ok);
                    fence_after();
                    const Unit &U = units[u];
                    const int nw = ok ? U.wt0 : 0, wt1 = U.wt1;
                    const bool pure = U.depth > 0;   // the s->s path is left out below the roots
                    float Gu[8 * XPW];   // [xi][a2][v]: unit sums of the z-step fragments
#pragma unroll
                    for (int i = 0; i < 8 * XPW; i++) Gu[i] = 0.f;
                    // S1 columns of one term (both z halves) from TMEM (loading the next
                    // term's columns during this term's products measured 6 % slower)
                    float cC[2][CPP], cA[2][CPP], cT[2][CPP];
                    auto load_term = [&](int j) {
#pragma unroll
                        for (int t = 0; t < 2; t++) {
                            if (j < (t == 0 ? nw : wt1)) {
                                const uint32_t base = tmem + ((uint32_t)(32 * quarter) << 16) + 256u * db + 128u * t + CPT * j;
                                tmem_ldn<CPP>(base + CPP * part, cC[t]);
                                tmem_ldn<CPP>(base + 8 + CPP * part, cA[t]);
                                tmem_ldn<CPP>(base + 16 + CPP * part, cT[t]);
                            } else {
#pragma unroll
                                for (int i = 0; i < CPP; i++) cC[t][i] = cA[t][i] = cT[t][i] = 0.f;
                            }
                        }
                    };
                    bool d_free = false;   // this warp's arrival on d_empty[db] is made
                    for (int j = 0; j < nw && ok; j++, nterm++) {
                        float *S1s = S1base + (nterm & 1) * S1_FLOATS;
                        float *Us = S1s + 16 * XS;
                        // this term's operator fragments (in flight during the drain)
                        const size_t frow = ((size_t)U.depth * T + U.q + j) * kPencilFragL + kPencilMaxL;
                        const float4 *py = reinterpret_cast<const float4 *>(op.pfrag + (frow + U.ly) * kPencilFragFloats);
                        const float4 *pz = reinterpret_cast<const float4 *>(op.pfrag + (frow + U.lz) * kPencilFragFloats) + 128;
                        float4 fy[4], fz[4];
#pragma unroll
                        for (int s = 0; s < 2; s++) {
                            fy[2 * s] = __ldg(py + 64 * s + 2 * lane);
                            fy[2 * s + 1] = __ldg(py + 64 * s + 2 * lane + 1);
                        }
#pragma unroll
                        for (int idx = 0; idx < 4; idx++) fz[idx] = __ldg(pz + 32 * idx + lane);
                        // ---- S1 of term j (both z halves) into shared memory ----
                        load_term(j);
                        tmem_wait_ld();
#pragma unroll
                        for (int t = 0; t < 2; t++) {
                            const int z = 8 * t + q2;
                            const bool u_row = pure && t == 0 && b1 == 0;
#pragma unroll
                            for (int i = 0; i < CPP; i++) {
                                const int xa = CPP * part + i;     // a0 = 0
                                S1s[xa * XS + yrow * YS + z] = u_row ? cC[t][i] : cC[t][i] + cT[t][i];
                                S1s[(8 + xa) * XS + yrow * YS + z] = cA[t][i];
                                if (u_row) Us[xa * US + q1 * UYS + q2] = cT[t][i];
                            }
                        }
                        if (j + 1 == nw) {
                            // the unit's last TMEM columns are read: the D buffer is free
                            fence_before();
                            __syncwarp();
                            if (lane == 0) bar_arrive(&d_empty[db]);
                            d_free = true;
                        }
                        consumers_sync<NCW>();
                        // blocks (a, b) of a direction take part iff |l| <= bw[2a + b]
                        const TermRow row = op.term_rows[(size_t)U.depth * T + U.q + j];
                        unsigned vy = 0, vz = 0;
#pragma unroll
                        for (int c = 0; c < 4; c++) {
                            vy |= (abs(U.ly) <= row.wd[c] ? 1u : 0u) << c;
                            vz |= (abs(U.lz) <= row.wd[c] ? 1u : 0u) << c;
                        }
                        // O^y A fragments per k step s = b1 (block of row half a1: idx 2 a1 + s):
                        // O^y[y_out = (a1, p1)][y_in = (s, q1)] = blocks32[idx 64 + 8 q1 + p1];
                        // O^z B fragments per (a2, s = b2), k permuted: row k = tq <-> z_in = 8 s + 2 tq,
                        // row tq + 4 <-> 8 s + 2 tq + 1; O^z[z_out][z_in] = blocks32[idx 64 + 8 (z_in % 8) + z_out % 8]
                        // (split and masked at operator upload, k_pencil_frags; loaded before the drain)
                        float yah[2][4], yal[2][4], zbh[2][2][2], zbl[2][2][2];
#pragma unroll
                        for (int s = 0; s < 2; s++) {
                            yah[s][0] = fy[2 * s].x; yah[s][1] = fy[2 * s].y; yah[s][2] = fy[2 * s].z; yah[s][3] = fy[2 * s].w;
                            yal[s][0] = fy[2 * s + 1].x; yal[s][1] = fy[2 * s + 1].y; yal[s][2] = fy[2 * s + 1].z; yal[s][3] = fy[2 * s + 1].w;
                        }
#pragma unroll
                        for (int idx = 0; idx < 4; idx++) {
                            const float4 z = fz[idx];
                            zbh[idx >> 1][idx & 1][0] = z.x;
                            zbh[idx >> 1][idx & 1][1] = z.y;
                            zbl[idx >> 1][idx & 1][0] = z.z;
                            zbl[idx >> 1][idx & 1][1] = z.w;
                        }
                        const bool ys[2] = {(vy & 5u) != 0, (vy & 10u) != 0};   // k step s has a block that takes part
                        // ---- y step: C[xi][zb] = Y^T fragment (rows y_out g, g + 8; columns z = 8 zb + 2 tq, +1) ----
                        // B = S1^T: rows k = y_in = 8 s + tq (+4), column n = z = 8 zb + g; all operands
                        // first, then the products with the independent accumulators side by side
                        float C[XPW][2][4], Cl[XPW][2][4], P[XPW][2];
#pragma unroll
                        for (int xi = 0; xi < XPW; xi++)
#pragma unroll
                            for (int zb = 0; zb < 2; zb++)
#pragma unroll
                                for (int v = 0; v < 4; v++) C[xi][zb][v] = Cl[xi][zb][v] = 0.f;
#pragma unroll
                        for (int s = 0; s < 2; s++) {
                            if (!ys[s]) continue;
                            float bh[XPW][2][2], bl[XPW][2][2];
#pragma unroll
                            for (int xi = 0; xi < XPW; xi++)
#pragma unroll
                                for (int zb = 0; zb < 2; zb++) {
                                    const float *src = S1s + xof(xi) * XS + (8 * s + tq) * YS + 8 * zb + fg;
                                    split(src[0], bh[xi][zb][0], bl[xi][zb][0]);
                                    split(src[4 * YS], bh[xi][zb][1], bl[xi][zb][1]);
                                }
#pragma unroll
                            for (int xi = 0; xi < XPW; xi++)
#pragma unroll
                                for (int zb = 0; zb < 2; zb++) mma16(Cl[xi][zb], yal[s], bh[xi][zb]);
#pragma unroll
                            for (int xi = 0; xi < XPW; xi++)
#pragma unroll
                                for (int zb = 0; zb < 2; zb++) mma16(C[xi][zb], yah[s], bh[xi][zb]);
#pragma unroll
                            for (int xi = 0; xi < XPW; xi++)
#pragma unroll
                                for (int zb = 0; zb < 2; zb++) mma16(Cl[xi][zb], yah[s], bl[xi][zb]);
                        }
#pragma unroll
                        for (int xi = 0; xi < XPW; xi++) {
                            const int x = xof(xi);
#pragma unroll
                            for (int zb = 0; zb < 2; zb++)
#pragma unroll
                                for (int v = 0; v < 4; v++) C[xi][zb][v] += Cl[xi][zb][v];
                            P[xi][0] = P[xi][1] = 0.f;
                            // U channel (x < 8, z < 8, y_in < 8): O^y's k step 0 applied to U; the a1 = 0 rows
                            // (T block) are P, the a1 = 1 rows (B block) join Y
                            if (pure && x < 8 && (vy & 5u)) {
                                float bh[2], bl[2], cu[4] = {0.f, 0.f, 0.f, 0.f};
                                split(Us[x * US + tq * UYS + fg], bh[0], bl[0]);
                                split(Us[x * US + (tq + 4) * UYS + fg], bh[1], bl[1]);
                                mma3x(cu, yah[0], yal[0], bh, bl);
                                P[xi][0] = cu[0];
                                P[xi][1] = cu[1];
                                C[xi][0][2] += cu[2];
                                C[xi][0][3] += cu[3];
                            }
                        }
                        // ---- z step: the y-step fragments are the A fragments (k' = tq <-> z = 8 s + 2 tq) ----
                        // split once per (xi, s) for both a2; the products of the (xi, a2) accumulators side by side
                        float Z[XPW][2][4], Zl[XPW][2][4];
#pragma unroll
                        for (int xi = 0; xi < XPW; xi++)
#pragma unroll
                            for (int a2 = 0; a2 < 2; a2++)
#pragma unroll
                                for (int v = 0; v < 4; v++) Z[xi][a2][v] = Zl[xi][a2][v] = 0.f;
#pragma unroll
                        for (int s = 0; s < 2; s++) {
                            const bool zs0 = (vz >> s) & 1u, zs1 = (vz >> (2 + s)) & 1u;
                            if (!zs0 && !zs1) continue;
                            float ah[XPW][4], al[XPW][4];
#pragma unroll
                            for (int xi = 0; xi < XPW; xi++) {
                                split(C[xi][s][0], ah[xi][0], al[xi][0]);
                                split(C[xi][s][2], ah[xi][1], al[xi][1]);
                                split(C[xi][s][1], ah[xi][2], al[xi][2]);
                                split(C[xi][s][3], ah[xi][3], al[xi][3]);
                            }
#pragma unroll
                            for (int xi = 0; xi < XPW; xi++) {
                                if (zs0) mma16(Zl[xi][0], al[xi], zbh[0][s]);
                                if (zs1) mma16(Zl[xi][1], al[xi], zbh[1][s]);
                            }
#pragma unroll
                            for (int xi = 0; xi < XPW; xi++) {
                                if (zs0) mma16(Z[xi][0], ah[xi], zbh[0][s]);
                                if (zs1) mma16(Z[xi][1], ah[xi], zbh[1][s]);
                            }
#pragma unroll
                            for (int xi = 0; xi < XPW; xi++) {
                                if (zs0) mma16(Zl[xi][0], ah[xi], zbl[0][s]);
                                if (zs1) mma16(Zl[xi][1], ah[xi], zbl[1][s]);
                            }
                        }
#pragma unroll
                        for (int xi = 0; xi < XPW; xi++) {
                            const int x = xof(xi);
#pragma unroll
                            for (int a2 = 0; a2 < 2; a2++)
#pragma unroll
                                for (int v = 0; v < 4; v++) Z[xi][a2][v] += Zl[xi][a2][v];
                            // P through z with the B block only (a2 = 1 from b2 = 0): the T.T.T path is left out
                            if (pure && x < 8 && (vy & 1u) && ((vz >> 2) & 1u)) {
                                float ah[4], al[4];
                                split(P[xi][0], ah[0], al[0]);
                                ah[1] = al[1] = 0.f;
                                split(P[xi][1], ah[2], al[2]);
                                ah[3] = al[3] = 0.f;
                                mma3x(Z[xi][1], ah, al, zbh[1][0], zbl[1][0]);
                            }
#pragma unroll
                            for (int a2 = 0; a2 < 2; a2++)
#pragma unroll
                                for (int v = 0; v < 4; v++) Gu[8 * xi + 4 * a2 + v] += Z[xi][a2][v];
                        }
                    }
                    // compensated sums over the units
#pragma unroll
                    for (int e = 0; e < 8 * XPW; e++) {
                        const float yv = Gu[e] - Gc[e];
                        const float tv = G[e] + yv;
                        Gc[e] = (tv - G[e]) - yv;
                        G[e] = tv;
                    }
                    // D is free (if not released after the last term's columns)
                    fence_before();
                    __syncwarp();
                    if (lane == 0 && !d_free) bar_arrive(&d_empty[db]);
                    nu++;
                }
                // the task's sums (slot of its units; every task has one): fragment v of
                // (x, a2): y_out = fg + 8 (v >> 1), z_out = 8 a2 + 2 tq + (v & 1); g component
                // gt = a0 + 2 a1 + 4 a2, element p0 + 8 p1 + 64 p2
                double *go = pen_partial + (size_t)units[u0].task * 4096;
#pragma unroll
                for (int e = 0; e < 8 * XPW; e++) {
                    const int xi = e >> 3, a2 = (e >> 2) & 1, v = e & 3;
                    const int x = xof(xi), a0 = x >> 3, p0 = x & 7, a1 = v >> 1, p1 = fg, p2 = 2 * tq + (v & 1);
                    go[(a0 + 2 * a1 + 4 * a2) * 512 + p0 + 8 * p1 + 64 * p2] = (double)G[e] - (double)Gc[e];
                }
            }
            if (__syncthreads_or(lbad) != 0) {
                lbad = true;
                break;
            }
        }
    }
    // wait (bounded) for the tensor-core work in flight, then free TMEM
    __syncthreads();
    if (tid == 32) {
        fence_after();
        commit(&bar_end);
        bar_wait(&bar_end, 0);
    }
    fence_before();
    __syncthreads();
    fence_after();
    if (warp == 0) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(TM_COLS));
}

// ---------------------------------------------------------------------------
// Work items that the pencil kernel covers (terms of band width <= kPencilMaxW
// at the depth of g) leave the list of the item kernel: per work entry a
// stable compaction.
__device__ __forceinline__ bool kept(const DevOper &op, int depth, const WorkItem &it, int maxw) {
    return op.bw[((size_t)it.term * op.max_rows + depth) * 5 + 4] > maxw;
}

__global__ void k_keep_count(DevMRA m, DevOper op, const DevTree *gs, const int *work_tree, const int *work, const long long *g_off, int n_work,
                             const WorkItem *items, int *keep, const int *nw_dev, int maxw) {
    const int wi = blockIdx.x;
    if (nw_dev && wi >= *nw_dev) {
        if (threadIdx.x == 0) keep[wi] = 0;
        return;
    }
    if (wi >= n_work) return;
    const int depth = gs[work_tree[wi]].idx[work[wi]].x - m.root_scale;
    int c = 0;
    for (long long i = g_off[wi] + threadIdx.x; i < g_off[wi + 1]; i += blockDim.x) c += kept(op, depth, items[i], maxw) ? 1 : 0;
    for (int o = 16; o > 0; o >>= 1) c += __shfl_down_sync(0xffffffffu, c, o);
    __shared__ int red[8];
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = c;
    __syncthreads();
    if (threadIdx.x == 0) {
        int t = 0;
        for (int w = 0; w < (int)(blockDim.x >> 5); w++) t += red[w];
        keep[wi] = t;
    }
}

__global__ void k_keep_fill(DevMRA m, DevOper op, const DevTree *gs, const int *work_tree, const int *work, const long long *g_off,
                            const long long *k_off, int n_work, const WorkItem *in, WorkItem *out, const int *nw_dev, int maxw) {
    const int wi = blockIdx.x;
    if (wi >= n_work || (nw_dev && wi >= *nw_dev)) return;
    const int depth = gs[work_tree[wi]].idx[work[wi]].x - m.root_scale;
    const long long b = g_off[wi], e = g_off[wi + 1];
    long long dst = k_off[wi];
    const int lane = threadIdx.x & 31;
    // one warp keeps the order: ballot prefix per 32 items
    for (long long i0 = b; i0 < e; i0 += 32) {
        const long long i = i0 + lane;
        const bool k = i < e && kept(op, depth, in[i], maxw);
        const unsigned mk = __ballot_sync(0xffffffffu, k);
        if (k) out[dst + __popc(mk & ((1u << lane) - 1u))] = in[i];
        dst += __popc(mk);
    }
}

}  // namespace pencil

bool pencil_supported(int K) { return K == 8 && pencil_shape_ok(kPencilWarpsDefault); }

namespace {
template <int NCW> bool shape_ok_impl() {
    cudaFuncAttributes a{};
    if (cudaFuncGetAttributes(&a, pencil::k_pencil<NCW>) != cudaSuccess) return false;
    return 128 * pencil::Regs<NCW>::prod + 32 * NCW * pencil::Regs<NCW>::cons <= pencil::n_threads<NCW>() * a.numRegs;
}
template <int NCW>
void launch_shape(int grid, const DevOper &op, const DevTree *fs, const int *work_tree, const void *units, const int *task_unit, int n_tasks,
                  double *pen_partial, int *err, int *counter, cudaStream_t s) {
    static bool attr = false;
    if (!attr) {
        cudaFuncSetAttribute(pencil::k_pencil<NCW>, cudaFuncAttributeMaxDynamicSharedMemorySize, pencil::SM_BYTES);
        attr = true;
    }
    pencil::k_pencil<NCW><<<grid, pencil::n_threads<NCW>(), pencil::SM_BYTES, s>>>(op, fs, work_tree, (const pencil::Unit *)units, task_unit,
                                                                                  n_tasks, pen_partial, err, counter);
}
}  // namespace

bool pencil_shape_ok(int consumer_warps) {
    static const bool ok8 = shape_ok_impl<8>(), ok16 = shape_ok_impl<16>();
    return consumer_warps == 16 ? ok16 : consumer_warps == 8 ? ok8 : false;
}

void launch_stack_forms(const DevOper &op, const void *jobs, int n_jobs, float *forms, cudaStream_t s) {
    if (n_jobs <= 0) return;
    pencil::k_stack_forms<<<n_jobs, 256, 0, s>>>(op, (const PencilFormJob *)jobs, n_jobs, forms);
}

void launch_pencil_frags(const DevOper &op, int rows, float *frags, cudaStream_t s) {
    const int n = rows * op.n_terms * kPencilFragL;
    if (n <= 0) return;
    pencil::k_pencil_frags<<<n, 256, 0, s>>>(op, frags);
}

void launch_pencil_units(const DevMRA &m, const DevTree *fs, const DevTree *gs, const int *work_tree, const int *work, void *units, int n_units,
                         int *err, cudaStream_t s) {
    if (n_units <= 0) return;
    pencil::k_pencil_units<<<(n_units + 127) / 128, 128, 0, s>>>(m, fs, gs, work_tree, work, (pencil::Unit *)units, n_units, err);
}

void launch_keep_items(const DevMRA &m, const DevOper &op, const DevTree *gs, const int *work_tree, const int *work, const long long *g_off,
                       int n_work, const WorkItem *in, int *keep, cudaStream_t s, int maxw, const int *nw_dev) {
    if (n_work <= 0) return;
    pencil::k_keep_count<<<n_work, 256, 0, s>>>(m, op, gs, work_tree, work, g_off, n_work, in, keep, nw_dev, maxw);
}

void launch_keep_fill(const DevMRA &m, const DevOper &op, const DevTree *gs, const int *work_tree, const int *work, const long long *g_off,
                      const long long *k_off, int n_work, const WorkItem *in, WorkItem *out, cudaStream_t s, int maxw, const int *nw_dev) {
    if (n_work <= 0) return;
    pencil::k_keep_fill<<<n_work, 32, 0, s>>>(m, op, gs, work_tree, work, g_off, k_off, n_work, in, out, nw_dev, maxw);
}

void launch_pencil(const DevOper &op, const DevTree *fs, const int *work_tree, const void *units, const int *task_unit, int n_tasks,
                   double *pen_partial, int *err, int *counter, cudaStream_t s, int consumer_warps) {
    if (n_tasks <= 0) return;
    static int sms = 0;
    if (sms == 0) {
        int dev = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        if (sms <= 0) sms = 1;
    }
    cudaMemsetAsync(counter, 0, sizeof(int), s);
    const int grid = std::min(sms, n_tasks);
    if (consumer_warps == 16 && pencil_shape_ok(16))
        launch_shape<16>(grid, op, fs, work_tree, units, task_unit, n_tasks, pen_partial, err, counter, s);
    else
        launch_shape<8>(grid, op, fs, work_tree, units, task_unit, n_tasks, pen_partial, err, counter, s);
}

}  // namespace mwgpu
