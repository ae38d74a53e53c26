// Work-list builder: the band traversal and screening of ConvolutionCalculator
// (src/treebuilders/ConvolutionCalculator.cpp:142-329) for a whole level at
// once, one thread per (output node g, band cell f) pair.
//
// For every term whose band reaches f (applyOperComp :277-288) the thread forms
// the 64-bit (ft, gt) component mask from the per-direction band check and the
// norm test of applyOperator (:297-329), in FP64 and in the reference's
// expression order; the band-size factor of :105-139 is rebuilt from the
// direction-0 widths.  Triples with a non-empty mask become work items; their
// number is the node-term count.
//
// COUNT writes the item count of every pair, an exclusive scan gives the write
// positions, FILL writes the items.  Items are ordered by (g, cell, term), the
// order of the reference's loops (cells x fastest, terms by descending width).
//
// Block-schedule items (the mask is the full structural set) carry the input
// structure of the contraction's three stages (`sched`):
//   bits  0-15  stage 0, output o = (a0 b1 b2): input b0 valid at bit 2 o + b0
//   bit  16     the U channel (s->s, x step) exists
//   bits 17-32  stage 1, output q = (a0 a1 b2): input b1 valid at bit 17 + 2 q + b1
//   bit  33     U feeds output q = 2 (a0 = 0, a1 = 1, b2 = 0)
//   bit  34     the P channel (s->s, xy steps) exists
//   bits 35-50  stage 2, component gt: input b2 valid at bit 35 + 2 gt + b2
//   bit  51     P feeds gt = 4
#include "mwgpu_internal.cuh"

namespace mwgpu {

namespace {

// the stage structure of a block-schedule item (bit layout above)
__device__ inline unsigned long long block_schedule(unsigned nzm, const int (&ib)[3], bool pure) {
    unsigned long long sc = 0ull;
    unsigned y0 = 0, y1 = 0;
    for (int o = 0; o < 8; o++) {
        const int a0 = o & 1, b12 = o & 6;
        for (int b0 = 0; b0 < 2; b0++) {
            const int src = b0 + b12;
            if (((nzm >> src) & 1u) && ((ib[0] >> (2 * a0 + b0)) & 1) && !(pure && src == 0 && a0 == 0)) {
                sc |= 1ull << (2 * o + b0);
                y0 |= 1u << o;
            }
        }
    }
    const bool u = pure && (ib[0] & 1);
    if (u) sc |= 1ull << 16;
    for (int q = 0; q < 8; q++) {
        const int a0 = q & 1, a1 = (q >> 1) & 1, b2 = q >> 2;
        for (int b1 = 0; b1 < 2; b1++)
            if (((y0 >> (a0 + 2 * b1 + 4 * b2)) & 1u) && ((ib[1] >> (2 * a1 + b1)) & 1)) {
                sc |= 1ull << (17 + 2 * q + b1);
                y1 |= 1u << q;
            }
    }
    if (u && ((ib[1] >> 2) & 1)) {
        sc |= 1ull << 33;
        y1 |= 1u << 2;
    }
    const bool pp = u && (ib[1] & 1);
    if (pp) sc |= 1ull << 34;
    for (int gt = 0; gt < 8; gt++) {
        const int a2 = gt >> 2;
        for (int b2 = 0; b2 < 2; b2++)
            if (((y1 >> ((gt & 3) + 4 * b2)) & 1u) && ((ib[2] >> (2 * a2 + b2)) & 1)) sc |= 1ull << (35 + 2 * gt + b2);
    }
    if (pp && ((ib[2] >> 2) & 1)) sc |= 1ull << 51;
    return sc;
}

struct PairCtx {
    int wi, fid, depth, tree;
    int tl[3];
};

// locate pair p: work position wi (binary search in pair_off), its tree, band cell and f
__device__ inline bool locate_pair(const DevMRA &m, const DevOper &op, const DevTree *fs, const DevTree *gs, const int *work_tree,
                                   const int *work, const long long *pair_off, int n_work, long long p, PairCtx &pc) {
    int lo = 0, hi = n_work - 1;
    while (lo < hi) {
        int mid = (lo + hi + 1) >> 1;
        if (pair_off[mid] <= p) lo = mid;
        else hi = mid - 1;
    }
    const int wi = lo;
    const int t = work_tree[wi];
    const DevTree &f = fs[t];
    const int4 gx = gs[t].idx[work[wi]];
    const int depth = gx.x - m.root_scale;
    const int w = op.band_max[depth];
    const int gl[3] = {gx.y, gx.z, gx.w};
    int bs[3], be[3];
    for (int d = 0; d < 3; d++) {
        const long long c = (long long)m.corner[d] * (1ll << depth), nboxes = (long long)m.nbox[d] * (1ll << depth);
        bs[d] = (int)max((long long)gl[d] - w, c);
        be[d] = (int)min((long long)gl[d] + w, c + nboxes - 1);
    }
    const long long q = p - pair_off[wi];
    const int nx = be[0] - bs[0] + 1, ny = be[1] - bs[1] + 1;
    const int fx = bs[0] + (int)(q % nx), fy = bs[1] + (int)((q / nx) % ny), fz = bs[2] + (int)(q / ((long long)nx * ny));
    pc.wi = wi;
    pc.tree = t;
    pc.depth = depth;
    pc.tl[0] = fx - gl[0];
    pc.tl[1] = fy - gl[1];
    pc.tl[2] = fz - gl[2];
    NodeKey key;
    pc.fid = -1;
    if (pack_key(m, gx.x, fx, fy, fz, key)) pc.fid = hash_find(f.hkeys, f.hvals, f.hcap, key);
    return pc.fid >= 0;
}

// the reference's FP64 norm test for one component (ConvolutionCalculator.cpp:
// oNorm * fThr > gThreshold, with the products in the same order); kept out of
// line: it only runs for estimates within the FP32 margin of the threshold
__device__ __noinline__ bool exact_pass(const double *onorms, int base, int t0, int t1, int t2, int i0, int i1, int i2, int bsz, double fNorm,
                                        double gthr) {
    double oNorm = 1.0;
    oNorm *= onorms[(size_t)(base + t0) * 4 + i0];
    oNorm *= onorms[(size_t)(base + t1) * 4 + i1];
    oNorm *= onorms[(size_t)(base + t2) * 4 + i2];
    const double fThr = (double)bsz * fNorm;
    return oNorm * fThr > gthr;
}

// Screening of one (pair, term): the (ft, gt) components of the term that
// reach g (mask) and the structural set (smask).  The norm test is
// oNorm * fThr > gThreshold: without screening (gThreshold < 0) every
// structural component passes; otherwise an FP32 estimate decides when it is
// clear of the threshold by far more than its rounding error (2^-12 relative
// against < 2^-20), and the FP64 expression of the reference decides the
// rest.  For 1e-20 < gThreshold < 1e20 an FP32 underflow of one factor can
// only happen for products far below the threshold (the other factors are
// bounded by 1e12).  FP64 arithmetic runs at a small fraction of the FP32
// rate on this part, so the loop works on FP32 copies of the norms; the
// component loops are unrolled so that every table index is a constant.
struct PairNorms {
    float fnf[8];               // f component norms rounded to FP32
    unsigned fnz;               // components with norm >= MachineZero
    unsigned long long fmask;   // (ft, gt) bits with ft in fnz, less (0, 0) below the roots
    float fmx_up;               // FP32 upper bound of the largest f norm
    const double *fn;           // the FP64 norms
};

// (ft, gt) bits (bit ft * 8 + gt) whose operator component in direction D is
// I = 2 gt_D + ft_D
__host__ __device__ constexpr unsigned long long comp_mask(int d, int i) {
    unsigned long long m = 0ull;
    for (int ft = 0; ft < 8; ft++)
        for (int gt = 0; gt < 8; gt++)
            if (2 * ((gt >> d) & 1) + ((ft >> d) & 1) == i) m |= 1ull << (ft * 8 + gt);
    return m;
}
template <int D> struct DirMasks {
    static constexpr unsigned long long m0 = comp_mask(D, 0), m1 = comp_mask(D, 1), m2 = comp_mask(D, 2), m3 = comp_mask(D, 3);
};
// the (ft, gt) bits whose direction-D component is in the band (4-bit mask)
template <int D> __device__ __forceinline__ unsigned long long dir_bits(unsigned m) {
    return ((m & 1u) ? DirMasks<D>::m0 : 0ull) | ((m & 2u) ? DirMasks<D>::m1 : 0ull) | ((m & 4u) ? DirMasks<D>::m2 : 0ull) |
           ((m & 8u) ? DirMasks<D>::m3 : 0ull);
}

__device__ __forceinline__ void term_mask(const DevOper &op, const TermRow &row, const PairCtx &pc, const PairNorms &pn, bool screen, bool fp32,
                                          float thr_hi, float thr_lo, double gthr, unsigned long long &mask, unsigned long long &smask,
                                          unsigned (&inm)[3]) {
    mask = smask = 0ull;
    inm[0] = inm[1] = inm[2] = 0u;
#pragma unroll
    for (int d = 0; d < 3; d++)
#pragma unroll
        for (int c = 0; c < 4; c++) inm[d] |= (abs(pc.tl[d]) <= row.wd[c] ? 1u : 0u) << c;
    // the structural set: every direction's component in its band, f component present
    smask = dir_bits<0>(inm[0]) & dir_bits<1>(inm[1]) & dir_bits<2>(inm[2]) & pn.fmask;
    if (!screen) {
        mask = smask;
        return;
    }
    if (smask == 0ull) return;
    const int L0 = row.L0, off = row.off;
    int fac[4];
#pragma unroll
    for (int c = 0; c < 4; c++) fac[c] = row.wd[c] < 0 ? 1 : 2 * row.wd[c] + 1;
    if (fp32) {
        // bound of every component product of this term: the largest operator
        // norm per direction, band size and f norm; clear of the threshold by
        // far more than the FP32 rounding -> nothing passes
        if (off < 0 || abs(pc.tl[0]) > L0 || abs(pc.tl[1]) > L0 || abs(pc.tl[2]) > L0) return;
        const int fm = max(max(fac[0], fac[1]), max(fac[2], fac[3]));
        const float bound = op.norm_max[off + pc.tl[0] + L0] * op.norm_max[off + pc.tl[1] + L0] * op.norm_max[off + pc.tl[2] + L0] *
                            ((float)(fm * fm * fm * 64) * pn.fmx_up);
        if (bound < thr_lo) return;
    }
    // per direction, for the estimate: FP32 norm x band-size factor (0 outside the band)
    float an[3][4];
#pragma unroll
    for (int d = 0; d < 3; d++)
#pragma unroll
        for (int c = 0; c < 4; c++)
            an[d][c] = (fp32 && ((inm[d] >> c) & 1u)) ? op.norms32[(size_t)(off + pc.tl[d] + L0) * 4 + c] * (float)fac[c] : 0.0f;
#pragma unroll
    for (int ft = 0; ft < 8; ft++) {
        if (((smask >> (8 * ft)) & 0xffull) == 0ull) continue;
        const float ff = 64.0f * pn.fnf[ft];
#pragma unroll
        for (int gt = 0; gt < 8; gt++) {
            const unsigned long long bit = 1ull << (ft * 8 + gt);
            if (!(smask & bit)) continue;
            const int i0 = 2 * (gt & 1) + (ft & 1), i1 = 2 * ((gt >> 1) & 1) + ((ft >> 1) & 1), i2 = 2 * (gt >> 2) + (ft >> 2);
            if (fp32) {
                const float est = (an[0][i0] * an[1][i1]) * (an[2][i2] * ff);
                if (est > thr_hi) {
                    mask |= bit;
                    continue;
                }
                if (est < thr_lo) continue;
            }
            if (exact_pass(op.norms, off + L0, pc.tl[0], pc.tl[1], pc.tl[2], i0, i1, i2, fac[i0] * fac[i1] * fac[i2] * 64, pn.fn[ft], gthr))
                mask |= bit;
        }
    }
}

// One work-list pass over the band pairs (g, f): COUNT stores the number of
// items of each pair, FILL writes them at item_off[p] in term order.  A group
// of G consecutive lanes shares a pair and takes its terms G at a time (lane
// j term base + j), the items of a round placed by a ballot prefix, so that
// small levels (few pairs, all terms) spread over G times more threads; the
// terms are sorted by descending band width, so a pair is finished at its
// first term whose band misses the cell.
// n_pairs / n_work are the launch capacity; with np_dev / nw_dev the actual
// counts come from the device (levels whose work list is made on the device),
// and COUNT writes zero counts for the pairs in [*np_dev, n_pairs).
// lanes per pair: enough threads for the whole GPU (152 SMs x 2048) on small
// levels, one lane per pair once the pairs alone fill it
constexpr long long kPairThreads = 2 * 152LL * 2048;
__host__ __device__ inline int pair_group(long long n_pairs) {
    if (n_pairs * 32 <= kPairThreads) return 32;
    if (n_pairs * 8 <= kPairThreads) return 8;
    if (n_pairs * 4 <= kPairThreads) return 4;
    return 1;
}

// GT > 0: GT lanes per pair; GT == 0: the group size follows the pair count
// read on the device (levels whose work list is made on the device; the grid
// then has at least kPairThreads threads, enough for any count's group)
template <bool FILL, int GT>
__global__ void __launch_bounds__(256) k_pairs(DevMRA m, DevOper op, const DevTree *fs, const DevTree *gs, const int *work_tree, const int *work,
                                               const long long *pair_off, int n_work, long long n_pairs, const double *gthrs, int *counts,
                                               const long long *item_off, WorkItem *items, long long items_cap, unsigned long long *ncomp,
                                               unsigned long long *nband, int *err, const long long *np_dev, const int *nw_dev,
                                               const double *gthr_node) {
    static_assert(GT == 0 || GT == 1 || GT == 4 || GT == 8 || GT == 32, "lane group size");
    const long long gid = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    const long long n_cap = n_pairs;
    if (np_dev) n_pairs = *np_dev;
    if (nw_dev) n_work = *nw_dev;
    const int G = GT > 0 ? GT : pair_group(n_pairs);
    const long long p = gid / G;
    const int j = (int)(gid % G), lane = threadIdx.x & 31;
    int cnt = 0;
    unsigned long long comp = 0, band = 0;
    if (!FILL && np_dev) {
        // the capacity beyond the device count: zero counts, grid-stride
        for (long long q = n_pairs + gid; q < n_cap; q += (long long)gridDim.x * blockDim.x) counts[q] = 0;
    }
    PairCtx pc;
    bool ok = false;
    if (p < n_pairs) {
        ok = locate_pair(m, op, fs, gs, work_tree, work, pair_off, n_work, p, pc);
        if (!ok && j == 0) atomicOr(err, DE_LOOKUP);
    }
    PairNorms pn;
    pn.fnz = 0u;
    pn.fmask = 0ull;
    pn.fmx_up = 0.f;
    pn.fn = nullptr;
    double gthr = 0.0;
    int maxdl = 0;
    if (ok) {
        band = (j == 0);
        const DevTree &f = fs[pc.tree];
        // per work entry where the precision is scaled locally (apply.cpp:221-228)
        gthr = gthr_node ? gthr_node[pc.wi] : gthrs[pc.tree];
        pn.fn = f.norms + (size_t)pc.fid * 8;
        double fmx = 0.0;
#pragma unroll
        for (int c = 0; c < 8; c++) {
            const double v = pn.fn[c];
            pn.fnf[c] = (float)v;
            if (!(v < kMachineZero)) {
                pn.fnz |= 1u << c;
                fmx = fmax(fmx, v);
            }
        }
        pn.fmx_up = nextafterf((float)fmx, INFINITY);
#pragma unroll
        for (int c = 0; c < 8; c++)
            if ((pn.fnz >> c) & 1u) pn.fmask |= 0xffull << (8 * c);
        if (pc.depth != 0) pn.fmask &= ~1ull;  // the (s, s) block only at the roots
        maxdl = max(abs(pc.tl[0]), max(abs(pc.tl[1]), abs(pc.tl[2])));
    }
    const bool screen = !(gthr < 0.0);
    const bool fp32 = gthr > 1e-20 && gthr < 1e20;
    const float thr_hi = (float)(gthr * (1.0 + 1.0 / 4096.0)), thr_lo = (float)(gthr * (1.0 - 1.0 / 4096.0));
    const int T = op.n_terms;
    long long wpos = (FILL && ok) ? item_off[p] : 0;
    bool live = ok && pn.fnz != 0u;
    // FILL with the counts of the COUNT pass: pairs without items are done,
    // the others stop after their last item
    const int target = (FILL && counts && live) ? counts[p] : -1;
    if (FILL && counts && target == 0) live = false;
    if (live && screen && fp32) {
        // the largest per-term bound of this cell over all terms: below the
        // threshold (with room for the FP32 rounding of the per-term bounds,
        // < 2^-21 relative) no term can pass
        const int po = op.pair_bound_off[pc.depth], W = op.band_max[pc.depth];
        if (po >= 0 && maxdl <= W) {
            const int nw = 2 * W + 1;
            const float pbv = op.pair_bound[po + ((pc.tl[0] + W) * nw + (pc.tl[1] + W)) * nw + (pc.tl[2] + W)];
            if (pbv * (64.0f * pn.fmx_up) * (1.0f + 1.0f / 1048576.0f) < thr_lo) live = false;
        }
    }
    for (int base = 0; base < T; base += G) {
        const int ti = base + j;
        bool active = live && ti < T;
        TermRow row;
        if (active) {
            row = op.term_rows[(size_t)pc.depth * T + ti];
            active = maxdl <= row.bw_max;
        }
        if (G == 1) {
            if (!active) break;
        } else if (!__any_sync(0xffffffffu, active)) {
            break;
        }
        unsigned long long mask = 0ull, smask = 0ull;
        unsigned inm[3] = {0u, 0u, 0u};
        if (active) term_mask(op, row, pc, pn, screen, fp32, thr_hi, thr_lo, gthr, mask, smask, inm);
        const bool pass = mask != 0ull;
        long long pos = wpos;
        int n_round = pass ? 1 : 0;
        if (G > 1) {
            const unsigned b = __ballot_sync(0xffffffffu, pass);
            const unsigned grp = G == 32 ? b : (b >> (lane & ~(G - 1))) & (unsigned)((1ull << G) - 1ull);  // G: 4, 8 or 32
            pos = wpos + __popc(grp & ((1u << j) - 1u));
            n_round = __popc(grp);
        }
        if (pass) {
            if (FILL) {
                WorkItem it;
                it.mask = mask;
                it.fid = pc.fid;
                it.term = (short)row.term;
                it.tl[0] = (short)pc.tl[0];
                it.tl[1] = (short)pc.tl[1];
                it.tl[2] = (short)pc.tl[2];
                it.flags = (mask == smask) ? 1 : 0;
                it.pad = 0;
                it.sched = 0ull;
                if (it.flags) {
                    unsigned nzm = 0;
                    for (int b = 0; b < 8; b++) nzm |= (((mask >> (8 * b)) & 0xffull) != 0ull) << b;
                    const int ib[3] = {(int)inm[0], (int)inm[1], (int)inm[2]};
                    it.sched = block_schedule(nzm, ib, pc.depth != 0 && (nzm & 1u));
                }
                if (pos < items_cap) items[pos] = it;
                else atomicOr(err, DE_POOL_FULL);
            } else {
                comp += __popcll(mask);
            }
        }
        wpos += n_round;
        cnt += n_round;
        if (FILL && target > 0 && cnt >= target) live = false;
    }
    if (!FILL && j == 0 && p < n_pairs) counts[p] = cnt;
    if (!FILL) {
        for (int o = 16; o > 0; o >>= 1) {
            comp += __shfl_down_sync(0xffffffffu, comp, o);
            band += __shfl_down_sync(0xffffffffu, band, o);
        }
        if (lane == 0 && (comp || band)) {
            atomicAdd(ncomp, comp);
            atomicAdd(nband, band);
        }
    }
}


// exclusive scan of int counts into long long offsets: per-block scan, scan of
// the block sums (one block), add.
constexpr int kScanBlock = 1024;

__global__ void k_scan_local(const int *in, long long *out, long long n, long long *block_sums) {
    __shared__ long long s[kScanBlock];
    const long long base = blockIdx.x * (long long)kScanBlock;
    const int t = threadIdx.x;
    long long v = (base + t < n) ? in[base + t] : 0;
    s[t] = v;
    __syncthreads();
    for (int o = 1; o < kScanBlock; o <<= 1) {
        long long x = t >= o ? s[t - o] : 0;
        __syncthreads();
        s[t] += x;
        __syncthreads();
    }
    if (base + t < n) out[base + t] = s[t] - v;
    if (t == kScanBlock - 1) block_sums[blockIdx.x] = s[t];
}

__global__ void k_scan_sums(long long *block_sums, int nb, long long *total) {
    __shared__ long long s[kScanBlock];
    long long carry = 0;
    for (int b0 = 0; b0 < nb; b0 += kScanBlock) {
        const int t = threadIdx.x;
        long long v = (b0 + t < nb) ? block_sums[b0 + t] : 0;
        s[t] = v;
        __syncthreads();
        for (int o = 1; o < kScanBlock; o <<= 1) {
            long long x = t >= o ? s[t - o] : 0;
            __syncthreads();
            s[t] += x;
            __syncthreads();
        }
        if (b0 + t < nb) block_sums[b0 + t] = carry + s[t] - v;
        long long last = s[kScanBlock - 1];
        __syncthreads();
        carry += last;
    }
    if (threadIdx.x == 0) *total = carry;
}

__global__ void k_scan_add(long long *out, long long n, const long long *block_sums, const long long *total) {
    const long long i = blockIdx.x * (long long)kScanBlock + threadIdx.x;
    if (i < n) out[i] += block_sums[blockIdx.x];
    if (i == n) out[n] = *total;
}

// per-g item offsets: g_off[wi] = item_off[pair_off[wi]]
// per work entry the offset of its first item, clamped to the item capacity:
// when a list outgrows its buffer (the fill flags DE_POOL_FULL and writes no
// item beyond it) the passes that read the items stay inside it
__global__ void k_gather_goff(const long long *item_off, const long long *pair_off, int n_work, long long *g_off, const int *nw_dev,
                              long long cap) {
    const int wi = blockIdx.x * blockDim.x + threadIdx.x;
    if (nw_dev) n_work = *nw_dev;
    if (wi <= n_work) g_off[wi] = min(item_off[pair_off[wi]], cap);
}

// Term-major order of the work items of each output node: a stable counting
// sort by term of the items [g_off[wi], g_off[wi + 1]) of `in` (cell-major
// from k_pairs: band cells z slowest, x fastest) into the same range of
// `out`.  The items of one term then follow the band cells in z, y, x order,
// so that the items with the same (term, l_y, l_z), and the runs of those
// with the same (term, l_z), are adjacent: the contraction sums their
// x-step (and xy-step) intermediates before the remaining 1D applications.
// One CTA per output node; per tile of 256 items a warp ranks the items of
// each term with __match_any_sync and the warps' counts give the offsets.
__global__ void __launch_bounds__(kOrderThreads) k_order_terms(const long long *g_off, int n_work, const WorkItem *in, WorkItem *out,
                                                                int n_terms, int *err, const int *nw_dev) {
    constexpr int NWARP = kOrderThreads / 32;
    __shared__ int base[kOrderMaxTerms];
    __shared__ int wcnt[NWARP][kOrderMaxTerms];
    if (nw_dev) n_work = *nw_dev;
    const int wi = blockIdx.x;
    if (wi >= n_work) return;
    const long long b = g_off[wi], e = g_off[wi + 1];
    if (b == e) return;
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    for (int t = tid; t < kOrderMaxTerms; t += kOrderThreads) {
        base[t] = 0;
        for (int w = 0; w < NWARP; w++) wcnt[w][t] = 0;
    }
    __syncthreads();
    for (long long i = b + tid; i < e; i += kOrderThreads) {
        const int t = in[i].term;
        if (t >= 0 && t < n_terms) atomicAdd(&base[t], 1);
        else atomicOr(err, DE_RANGE);
    }
    __syncthreads();
    if (tid == 0) {
        int s = 0;
        for (int t = 0; t < n_terms; t++) {
            const int c = base[t];
            base[t] = s;
            s += c;
        }
    }
    __syncthreads();
    for (long long t0 = b; t0 < e; t0 += kOrderThreads) {
        const long long i = t0 + tid;
        WorkItem it;
        int term = -1;
        if (i < e) {
            it = in[i];
            term = it.term;
            if (term < 0 || term >= n_terms) term = -1;
        }
        const unsigned peers = __match_any_sync(0xffffffffu, term);
        const int rank = __popc(peers & ((1u << lane) - 1u));
        if (term >= 0 && rank == 0) wcnt[warp][term] = __popc(peers);
        __syncthreads();
        if (term >= 0) {
            long long pos = base[term] + rank;
            for (int w = 0; w < warp; w++) pos += wcnt[w][term];
            if (b + pos < e) out[b + pos] = it;
        }
        __syncthreads();
        for (int t = tid; t < n_terms; t += kOrderThreads) {
            int s = 0;
            for (int w = 0; w < NWARP; w++) {
                s += wcnt[w][t];
                wcnt[w][t] = 0;
            }
            base[t] += s;
        }
        __syncthreads();
    }
}

// chunks of at most `per` items per work entry (at least one, so that every
// output node gets its reduction input)
__device__ inline long long chunk_len(const long long *g_off, int n_work, long long per) {
    if (per > 0) return per;
    const long long total = g_off[n_work];
    return max(8LL, (total + kChunkTarget - 1) / kChunkTarget);
}

__global__ void k_chunk_count(const long long *g_off, int n_work, long long per, int *counts, const int *nw_dev) {
    const int wi = blockIdx.x * blockDim.x + threadIdx.x;
    if (wi >= n_work) return;
    if (nw_dev && wi >= *nw_dev) {
        counts[wi] = 0;
        return;
    }
    per = chunk_len(g_off, nw_dev ? *nw_dev : n_work, per);
    const long long len = g_off[wi + 1] - g_off[wi];
    counts[wi] = len == 0 ? 1 : (int)((len + per - 1) / per);
}

__global__ void k_chunk_fill(const long long *g_off, const long long *c_off, int n_work, long long per, int4 *chunks, int *chunk_begin,
                             int cap, int *n_chunks, int *err, const int *nw_dev) {
    const int wi = blockIdx.x * blockDim.x + threadIdx.x;
    if (nw_dev) n_work = *nw_dev;
    if (n_work == 0 && wi == 0) {
        chunk_begin[0] = 0;
        *n_chunks = 0;
    }
    if (wi >= n_work) return;
    per = chunk_len(g_off, n_work, per);
    const long long b = g_off[wi], e = g_off[wi + 1];
    long long c = c_off[wi];
    chunk_begin[wi] = (int)c;
    if (wi == n_work - 1) {
        const long long tot = c_off[n_work];
        chunk_begin[n_work] = (int)tot;
        *n_chunks = (int)(tot < (long long)cap ? tot : (long long)cap);
        if (tot > cap) atomicOr(err, DE_POOL_FULL);
    }
    if (b == e) {
        if (c < cap) chunks[c] = make_int4(wi, (int)b, (int)e, 0);
        return;
    }
    for (long long x = b; x < e; x += per, c++)
        if (c < cap) chunks[c] = make_int4(wi, (int)x, (int)min(e, x + per), 0);
}


}  // namespace

void launch_pairs_count(const DevMRA &m, const DevOper &op, const DevTree *fs, const DevTree *gs, const int *work_tree, const int *work,
                        const long long *pair_off, int n_work, long long n_pairs, const double *gthrs, int *counts, unsigned long long *ncomp,
                        unsigned long long *nband, int *err, cudaStream_t s, const long long *np_dev, const int *nw_dev,
                        const double *gthr_node) {
    if (n_pairs <= 0) return;
    auto go = [&](auto kern, int g) {
        kern<<<(unsigned)((n_pairs * g + 255) / 256), 256, 0, s>>>(m, op, fs, gs, work_tree, work, pair_off, n_work, n_pairs, gthrs, counts, nullptr,
                                                                  nullptr, 0, ncomp, nband, err, np_dev, nw_dev, gthr_node);
    };
    auto kern_dev_false = [&](long long thr) {
        k_pairs<false, 0><<<(unsigned)((thr + 255) / 256), 256, 0, s>>>(m, op, fs, gs, work_tree, work, pair_off, n_work, n_pairs, gthrs, counts,
                                                                       nullptr, nullptr, 0, ncomp, nband, err, np_dev, nw_dev, gthr_node);
    };
    if (np_dev) {
        // group size from the device count: at least kPairThreads threads
        const long long thr = std::max(n_pairs * pair_group(n_pairs), kPairThreads);
        kern_dev_false(thr);
        return;
    }
    switch (pair_group(n_pairs)) {
        case 32: go(k_pairs<false, 32>, 32); break;
        case 8: go(k_pairs<false, 8>, 8); break;
        case 4: go(k_pairs<false, 4>, 4); break;
        default: go(k_pairs<false, 1>, 1); break;
    }
}

void launch_pairs_fill(const DevMRA &m, const DevOper &op, const DevTree *fs, const DevTree *gs, const int *work_tree, const int *work,
                       const long long *pair_off, int n_work, long long n_pairs, const double *gthrs, const int *counts_in, const long long *item_off,
                       WorkItem *items, long long items_cap, int *err, cudaStream_t s, const long long *np_dev, const int *nw_dev,
                       const double *gthr_node) {
    if (n_pairs <= 0) return;
    int *counts = const_cast<int *>(counts_in);  // read only in FILL
    auto go = [&](auto kern, int g) {
        kern<<<(unsigned)((n_pairs * g + 255) / 256), 256, 0, s>>>(m, op, fs, gs, work_tree, work, pair_off, n_work, n_pairs, gthrs, counts, item_off,
                                                                  items, items_cap, nullptr, nullptr, err, np_dev, nw_dev, gthr_node);
    };
    auto kern_dev_true = [&](long long thr) {
        k_pairs<true, 0><<<(unsigned)((thr + 255) / 256), 256, 0, s>>>(m, op, fs, gs, work_tree, work, pair_off, n_work, n_pairs, gthrs, counts,
                                                                      item_off, items, items_cap, nullptr, nullptr, err, np_dev, nw_dev, gthr_node);
    };
    if (np_dev) {
        // group size from the device count: at least kPairThreads threads
        const long long thr = std::max(n_pairs * pair_group(n_pairs), kPairThreads);
        kern_dev_true(thr);
        return;
    }
    switch (pair_group(n_pairs)) {
        case 32: go(k_pairs<true, 32>, 32); break;
        case 8: go(k_pairs<true, 8>, 8); break;
        case 4: go(k_pairs<true, 4>, 4); break;
        default: go(k_pairs<true, 1>, 1); break;
    }
}

void launch_chunk_count(const long long *g_off, int n_work, long long per, int *counts, cudaStream_t s, const int *nw_dev) {
    k_chunk_count<<<(n_work + 255) / 256, 256, 0, s>>>(g_off, n_work, per, counts, nw_dev);
}

void launch_chunk_fill(const long long *g_off, const long long *c_off, int n_work, long long per, int4 *chunks, int *chunk_begin, int cap,
                       int *n_chunks, int *err, cudaStream_t s, const int *nw_dev) {
    k_chunk_fill<<<(n_work + 255) / 256, 256, 0, s>>>(g_off, c_off, n_work, per, chunks, chunk_begin, cap, n_chunks, err, nw_dev);
}

long long scan_blocks(long long n) { return (n + kScanBlock - 1) / kScanBlock; }

void launch_scan(const int *in, long long *out, long long n, long long *block_sums, long long *total, cudaStream_t s) {
    const long long nb = scan_blocks(n + 1);
    k_scan_local<<<(unsigned)nb, kScanBlock, 0, s>>>(in, out, n, block_sums);
    k_scan_sums<<<1, kScanBlock, 0, s>>>(block_sums, (int)nb, total);
    k_scan_add<<<(unsigned)nb, kScanBlock, 0, s>>>(out, n, block_sums, total);
}

void launch_gather_goff(const long long *item_off, const long long *pair_off, int n_work, long long *g_off, cudaStream_t s, const int *nw_dev,
                        long long cap) {
    k_gather_goff<<<(n_work + 1 + 255) / 256, 256, 0, s>>>(item_off, pair_off, n_work, g_off, nw_dev, cap);
}

bool term_order_supported(int n_terms) { return n_terms > 0 && n_terms <= kOrderMaxTerms; }

void launch_order_terms(const long long *g_off, int n_work, const WorkItem *in, WorkItem *out, int n_terms, int *err, cudaStream_t s,
                        const int *nw_dev) {
    if (n_work <= 0) return;
    k_order_terms<<<n_work, kOrderThreads, 0, s>>>(g_off, n_work, in, out, n_terms, err, nw_dev);
}

}  // namespace mwgpu
