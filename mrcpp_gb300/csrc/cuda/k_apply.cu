// Operator application kernels: band lookup pre-pass and the FP64 per-node
// contraction.
//
// The contraction restates ConvolutionCalculator (src/treebuilders/
// ConvolutionCalculator.cpp) for one output node g per CTA:
//   band box          makeOperBand/fillOperBand            :142-222
//   f/g components    calcNode loop over ft, gt            :252-265  (ft=gt=0 only at depth 0)
//   term skip         applyOperComp maxDeltaL > bw.max     :277-288
//   screening         applyOperator band + norm test       :297-329
//   contraction       tensorApplyOperComp, 3 x g = f^T O   :333-382
// Work per (f, term) is re-associated: for each f component ft the
// direction-x and direction-y intermediates are shared between the g
// components that need them; the arithmetic of each component product is
// the same three 1D applications.
#include "mwgpu_internal.cuh"

#include <cstdlib>

namespace mwgpu {

namespace {

// out[c + K2*j] (+)= sum_i in[i + K*c] * F[i + K*j], products and sums in TC;
// the result is converted to TO (accumulated in TO when ADD).
template <bool ADD, typename TC, typename TI, typename TO>
__device__ __forceinline__ void tapply(TO *out, const TI *in, const double *F, int K, int tid, int nthr) {
    const int K2 = K * K, K3 = K2 * K;
    for (int e = tid; e < K3; e += nthr) {
        int c = e % K2, j = e / K2;
        const TI *a = in + K * c;
        const double *b = F + K * j;
        TC s = (TC)0;
        for (int i = 0; i < K; i++) s = fma((TC)a[i], (TC)__ldg(b + i), s);
        if (ADD) out[c + K2 * j] += (TO)s;
        else out[c + K2 * j] = (TO)s;
    }
}

// the block schedule runs where its 18 K^3 doubles of shared memory fit: K <= 11
constexpr int kBlockMaxK = 11;

// One stage of the block schedule: up to 5 output blocks, each the sum of up
// to 3 one-axis applications out[q] (=|+=) sum_p in[q][p]^T O[q][p] (the cyclic
// axis order of tapply), all outputs in one pass of the CTA.  The operands are
// listed in shared memory by thread 0.
struct StageList {
    const double *in[5][3];
    const double *O[5][3];
    double *out[5];
    int np[5];
    int nout;
};

// Thread t owns output column j = t % K of every block and rows c = t / K +
// m (nthr / K): the operator column of the current input stays in registers,
// and the K threads that share a row c read the same shared-memory words (the
// rows of consecutive threads would be K doubles apart, a 16-way bank
// conflict for K = 8).  The inputs of an output are added one after the other
// by the thread that owns the element.
template <bool ADD, int KM>
__device__ __forceinline__ void stage_apply(const StageList &st, int K, int tid, int nthr) {
    const int K2 = K * K;
    const int groups = nthr / K;  // threads per column
    const int j = tid % K, c0 = tid / K;
    if (c0 >= groups) return;
    for (int q = 0; q < st.nout; q++) {
        const int np = st.np[q];
        double *out = st.out[q] + K2 * j;
        if (np == 0) {
            if (!ADD)
                for (int c = c0; c < K2; c += groups) out[c] = 0.0;
            continue;
        }
        for (int p = 0; p < np; p++) {
            double b[KM];
#pragma unroll
            for (int i = 0; i < KM; i++) b[i] = i < K ? __ldg(st.O[q][p] + K * j + i) : 0.0;
            const double *in = st.in[q][p];
            const bool store = !ADD && p == 0;
            for (int c = c0; c < K2; c += groups) {
                const double *a = in + K * c;
                double s = 0.0;
#pragma unroll
                for (int i = 0; i < KM; i++)
                    if (i < K) s = fma(a[i], b[i], s);
                if (store) out[c] = s;
                else out[c] += s;
            }
        }
    }
}

// stage_apply with the operator columns sized for K
template <bool ADD>
__device__ __forceinline__ void stage_apply_k(const StageList &st, int K, int tid, int nthr) {
    switch (K) {
        case 2: stage_apply<ADD, 2>(st, K, tid, nthr); break;
        case 4: stage_apply<ADD, 4>(st, K, tid, nthr); break;
        case 6: stage_apply<ADD, 6>(st, K, tid, nthr); break;
        case 8: stage_apply<ADD, 8>(st, K, tid, nthr); break;
        case 10: stage_apply<ADD, 10>(st, K, tid, nthr); break;
        default: stage_apply<ADD, kBlockMaxK>(st, K, tid, nthr); break;
    }
}

struct Box {
    int s[3], e[3];
    int total;
};

__device__ inline bool band_box(const DevMRA &m, const DevOper &op, int4 g, int &depth, Box &b) {
    depth = g.x - m.root_scale;
    int w = (depth >= 0 && depth < op.n_band_max) ? op.band_max[depth] : -1;
    if (op.band_dir >= 0) w = op.band_dir_w;  // derivative: one direction
    if (w < 0) return false;
    int gl[3] = {g.y, g.z, g.w};
    b.total = 1;
    for (int d = 0; d < 3; d++) {
        // world bounds at this depth (64-bit: nbox 2^30 exceeds int)
        const long long c = (long long)m.corner[d] * (1ll << depth), nboxes = (long long)m.nbox[d] * (1ll << depth);
        const int wd = (op.band_dir < 0 || op.band_dir == d) ? w : 0;
        b.s[d] = (int)max((long long)gl[d] - wd, c);
        b.e[d] = (int)min((long long)gl[d] + wd, c + nboxes - 1);
        b.total *= (b.e[d] - b.s[d] + 1);
    }
    return b.total > 0;
}

__device__ inline void box_cell(const Box &b, int q, int &x, int &y, int &z) {
    int nx = b.e[0] - b.s[0] + 1, ny = b.e[1] - b.s[1] + 1;
    x = b.s[0] + q % nx;
    y = b.s[1] + (q / nx) % ny;
    z = b.s[2] + q / (nx * ny);
}

__global__ void k_band_missing(DevMRA m, DevOper op, DevTree f, DevTree g, const int *work, int n_work, NodeKey *pkeys,
                               int *pvals, int phcap, NodeKey *plist, int *pcount, int pcap, int *err) {
    int gi = work[blockIdx.x];
    int4 gx = g.idx[gi];
    int depth;
    Box b;
    if (!band_box(m, op, gx, depth, b)) return;
    for (int q = threadIdx.x; q < b.total; q += blockDim.x) {
        int x, y, z;
        box_cell(b, q, x, y, z);
        NodeKey key;
        if (!pack_key(m, gx.x, x, y, z, key)) { atomicOr(err, DE_RANGE); continue; }
        if (hash_find(f.hkeys, f.hvals, f.hcap, key) >= 0) continue;
        bool full = false;
        if (hash_insert(pkeys, pvals, phcap, key, 0, &full)) {
            int pos = atomicAdd(pcount, 1);
            if (pos < pcap) plist[pos] = key;
        }
        if (full) atomicOr(err, DE_HASH_FULL);
    }
}

// One CTA per output node.  Shared memory: g accumulator 8K^3, then either
// the per-component intermediates (x 2K^3, xy 4K^3) or, with `block`, the
// block schedule's 10K^3.
//
// Two schedules give the sum of the kept component products of
// tensorApplyOperComp:
// * block schedule, for a (f, term) whose kept components are all the
//   structural ones (band widths, zero-norm f components, the depth rule;
//   every item of a level without norm screening): per output x-bit a0,
//     Y0[b1 b2]    = sum_b0 O^x_{a0 b0} f[b0 b1 b2]
//     Y1[a1 b2]    = sum_b1 O^y_{a1 b1} Y0[b1 b2]
//     g[a0 a1 a2] += sum_b2 O^z_{a2 b2} Y1[a1 b2]
//   (48 K^4 FMA for a full node-term, against 112 K^4 for the per-component
//   schedule), operator blocks outside their band and zero-norm f
//   components left out of the sums.  At depth > 0 the (s, s) product
//   (ft = gt = 0, ConvolutionCalculator.cpp:261) is not in the sums: f[000]'s
//   x-step into a0 = 0 is kept apart as U0, enters the y step only toward
//   a1 = 1, U1 = O^y_00 U0 enters the z step only toward a2 = 1, and the
//   remaining O^z_00 U1 is never formed;
// * per-component schedule otherwise: for each f component ft the x and xy
//   intermediates shared by the kept g components.
// TC is the type of the 1D products and of the x / xy intermediates of the
// per-component schedule (double: the plain form).
template <typename TC>
// With nw_dev / gthr_dev the number of work entries and the threshold come from
// the device (the grid is then a capacity); gthr_node holds one threshold per
// work entry where the precision is scaled per output node (apply.cpp:221-228).
__global__ void __launch_bounds__(256) k_contract(DevMRA m, DevOper op, DevTree f, DevTree g, const int *work, int n_work,
                                                  double gthr, LevelStats *stats, int *err, const int *nw_dev, const double *gthr_dev,
                                                  const double *gthr_node, bool block) {
    if (nw_dev && (int)blockIdx.x >= *nw_dev) return;
    if (gthr_dev) gthr = *gthr_dev;
    if (gthr_node) gthr = gthr_node[blockIdx.x];
    extern __shared__ double sm[];
    const int K = m.K, K2 = K * K, K3 = m.kp1_d, tid = threadIdx.x, nthr = blockDim.x;
    double *gacc = sm;
    TC *X0 = (TC *)(gacc + 8 * K3);
    TC *X1 = X0 + 2 * K3;
    double *Y0 = gacc + 8 * K3, *Y1 = Y0 + 4 * K3, *U0 = Y1 + 4 * K3, *U1 = U0 + K3;
    __shared__ int s_fid;
    __shared__ double s_fn[8];
    __shared__ unsigned s_mask[2], s_smask[2];
    __shared__ unsigned long long s_nt, s_nc;
    __shared__ StageList s_st;
    const int gi = work[blockIdx.x];
    const int4 gx = g.idx[gi];
    for (int e = tid; e < 8 * K3; e += nthr) gacc[e] = 0.0;
    if (tid == 0) { s_nt = 0; s_nc = 0; }
    __syncthreads();
    int depth;
    Box b;
    unsigned long long nband = 0;
    if (band_box(m, op, gx, depth, b) && depth < kMaxDepthRows) {
        const int T = op.n_terms;
        for (int q = 0; q < b.total; q++) {
            int fx, fy, fz;
            box_cell(b, q, fx, fy, fz);
            if (tid == 0) {
                NodeKey key;
                int id = -1;
                if (pack_key(m, gx.x, fx, fy, fz, key)) id = hash_find(f.hkeys, f.hvals, f.hcap, key);
                if (id < 0) atomicOr(err, DE_LOOKUP);
                s_fid = id;
                if (id >= 0)
                    for (int c = 0; c < 8; c++) s_fn[c] = f.norms[(size_t)id * 8 + c];
            }
            __syncthreads();
            const int fid = s_fid;
            if (fid < 0) { __syncthreads(); continue; }
            nband++;
            const int tl[3] = {fx - gx.y, fy - gx.z, fz - gx.w};
            const int maxdl = max(abs(tl[0]), max(abs(tl[1]), abs(tl[2])));
            const bool gen = fid >= f.cap_real;
            const double *fc = gen ? f.gcoefs + (size_t)(fid - f.cap_real) * K3 : f.coefs + (size_t)fid * 8 * K3;
            for (int ti = 0; ti < T; ti++) {
                const int i = op.term_order[depth * T + ti];
                const int *bwi = op.bw + ((size_t)i * op.max_rows + depth) * 5;
                if (maxdl > bwi[4]) break;  // terms sorted by descending max width at this depth
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
                    const bool structural = pass;
                    if (pass) {
                        const double fThr = (double)op.band_size[((size_t)i * kMaxDepthRows + depth) * 64 + gt * 8 + ft] * fNorm;
                        const double upper = oNorm * fThr;
                        pass = upper > gthr;
                    }
                    unsigned bal = __ballot_sync(0xffffffffu, pass), sbal = __ballot_sync(0xffffffffu, structural);
                    if ((tid & 31) == 0) {
                        s_mask[tid >> 5] = bal;
                        s_smask[tid >> 5] = sbal;
                    }
                }
                __syncthreads();
                const unsigned long long mask = (unsigned long long)s_mask[0] | ((unsigned long long)s_mask[1] << 32);
                const unsigned long long smask = (unsigned long long)s_smask[0] | ((unsigned long long)s_smask[1] << 32);
                if (mask == 0ull) { __syncthreads(); continue; }
                if (tid == 0) { s_nt++; s_nc += __popcll(mask); }
                const int L0 = op.dep_L[i * op.max_rows + depth];
                const int off = op.dep_off[i * op.max_rows + depth];
                const double *ob[3];
                for (int d = 0; d < 3; d++) ob[d] = op.blocks + (size_t)(off + tl[d] + L0) * 4 * K2;
                if (block && mask == smask) {
                    // f components present and operator blocks inside their band
                    auto fon = [&](int ft) { return !(s_fn[ft] < kMachineZero); };
                    auto oon = [&](int d, int a, int bb) { return abs(tl[d]) <= bwi[2 * a + bb]; };
                    const bool excl = depth != 0;
                    for (int a0 = 0; a0 < 2; a0++) {
                        // x step: Y0[b1 b2] (+ U0 for the excluded path)
                        if (tid == 0) {
                            StageList &st = s_st;
                            st.nout = 0;
                            for (int q = 0; q < 4; q++) {
                                int np = 0;
                                for (int b0 = 0; b0 < 2; b0++) {
                                    const int ft = b0 + 2 * q;
                                    if (!fon(ft) || !oon(0, a0, b0) || (excl && a0 == 0 && ft == 0)) continue;
                                    st.in[q][np] = fc + (size_t)ft * K3;
                                    st.O[q][np] = ob[0] + (2 * a0 + b0) * K2;
                                    np++;
                                }
                                st.np[q] = np;
                                st.out[q] = Y0 + q * K3;
                            }
                            st.nout = 4;
                            if (excl && a0 == 0) {
                                st.np[4] = (fon(0) && oon(0, 0, 0)) ? 1 : 0;
                                st.in[4][0] = fc;
                                st.O[4][0] = ob[0];
                                st.out[4] = U0;
                                st.nout = 5;
                            }
                        }
                        __syncthreads();
                        stage_apply_k<false>(s_st, K, tid, nthr);
                        __syncthreads();
                        // y step: Y1[a1 b2] = sum_b1 O^y_{a1 b1} Y0[b1 b2] (+ U0 toward a1 = 1; U1 = O^y_00 U0)
                        if (tid == 0) {
                            StageList &st = s_st;
                            for (int q = 0; q < 4; q++) {
                                const int a1 = q & 1, b2 = q >> 1;
                                int np = 0;
                                for (int b1 = 0; b1 < 2; b1++) {
                                    if (!oon(1, a1, b1)) continue;
                                    st.in[q][np] = Y0 + (b1 + 2 * b2) * K3;
                                    st.O[q][np] = ob[1] + (2 * a1 + b1) * K2;
                                    np++;
                                }
                                if (excl && a0 == 0 && a1 == 1 && b2 == 0 && oon(1, 1, 0)) {
                                    st.in[q][np] = U0;
                                    st.O[q][np] = ob[1] + 2 * K2;
                                    np++;
                                }
                                st.np[q] = np;
                                st.out[q] = Y1 + q * K3;
                            }
                            st.nout = 4;
                            if (excl && a0 == 0) {
                                st.np[4] = oon(1, 0, 0) ? 1 : 0;
                                st.in[4][0] = U0;
                                st.O[4][0] = ob[1];
                                st.out[4] = U1;
                                st.nout = 5;
                            }
                        }
                        __syncthreads();
                        stage_apply_k<false>(s_st, K, tid, nthr);
                        __syncthreads();
                        // z step: g[a0 a1 a2] += sum_b2 O^z_{a2 b2} Y1[a1 b2] (+ U1 toward a2 = 1)
                        if (tid == 0) {
                            StageList &st = s_st;
                            for (int q = 0; q < 4; q++) {
                                const int a1 = q & 1, a2 = q >> 1;
                                int np = 0;
                                for (int b2 = 0; b2 < 2; b2++) {
                                    if (!oon(2, a2, b2)) continue;
                                    st.in[q][np] = Y1 + (a1 + 2 * b2) * K3;
                                    st.O[q][np] = ob[2] + (2 * a2 + b2) * K2;
                                    np++;
                                }
                                if (excl && a0 == 0 && a1 == 0 && a2 == 1 && oon(2, 1, 0)) {
                                    st.in[q][np] = U1;
                                    st.O[q][np] = ob[2] + 2 * K2;
                                    np++;
                                }
                                st.np[q] = np;
                                st.out[q] = gacc + (a0 + 2 * a1 + 4 * a2) * K3;
                            }
                            st.nout = 4;
                        }
                        __syncthreads();
                        stage_apply_k<true>(s_st, K, tid, nthr);
                        __syncthreads();
                    }
                    continue;
                }
                for (int ft = 0; ft < 8; ft++) {
                    const unsigned gm = (unsigned)((mask >> (8 * ft)) & 0xffull);
                    if (gm == 0) continue;
                    const double *fin = fc + (size_t)ft * K3;
                    const int b0 = ft & 1, b1 = (ft >> 1) & 1, b2 = (ft >> 2) & 1;
                    unsigned need0 = 0, need1 = 0;
                    for (int gt = 0; gt < 8; gt++)
                        if (gm & (1u << gt)) { need0 |= 1u << (gt & 1); need1 |= 1u << (gt & 3); }
                    for (int a0 = 0; a0 < 2; a0++)
                        if (need0 & (1u << a0)) tapply<false, TC>(X0 + a0 * K3, fin, ob[0] + (2 * a0 + b0) * K2, K, tid, nthr);
                    __syncthreads();
                    for (int s = 0; s < 4; s++)
                        if (need1 & (1u << s)) tapply<false, TC>(X1 + s * K3, X0 + (s & 1) * K3, ob[1] + (2 * (s >> 1) + b1) * K2, K, tid, nthr);
                    __syncthreads();
                    for (int gt = 0; gt < 8; gt++)
                        if (gm & (1u << gt)) tapply<true, TC>(gacc + gt * K3, X1 + (gt & 3) * K3, ob[2] + (2 * (gt >> 2) + b2) * K2, K, tid, nthr);
                    __syncthreads();
                }
            }
            __syncthreads();  // s_fid / s_fn are rewritten for the next band cell
        }
    }
    __syncthreads();
    double *go = g.coefs + (size_t)gi * 8 * K3;
    for (int e = tid; e < 8 * K3; e += nthr) go[e] = gacc[e];
    // node norms (MWNode::calcNorms)
    __shared__ double red[8][8];
    for (int comp = 0; comp < 8; comp++) {
        double s = 0.0;
        for (int e = tid; e < K3; e += nthr) { double v = gacc[comp * K3 + e]; s += v * v; }
        for (int o = 16; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o);
        if ((tid & 31) == 0) red[comp][tid >> 5] = s;
    }
    __syncthreads();
    if (tid < 8) {
        double t = 0.0;
        for (int w = 0; w < nthr / 32; w++) t += red[tid][w];
        g.norms[(size_t)gi * 8 + tid] = sqrt(t);
    }
    if (tid == 0) {
        atomicAdd(&stats->node_terms, s_nt);
        atomicAdd(&stats->components, s_nc);
        atomicAdd(&stats->band_nodes, nband);
    }
}


// DerivativeCalculator::calcNode(gNode) (DerivativeCalculator.cpp:113-151) for
// one output node per CTA: the band along dir (makeOperBand :153-176), per
// (f, ft, gt) the checks of applyOperator (:199-241: the component's band width
// in every direction, the identity -- T or A block at l = 0 -- off the apply
// direction), the 1D application along dir (tensorApplyOperComp :245-268 with
// identity factors), division by sf^order and the node norms.  FP64.
__global__ void __launch_bounds__(256) k_deriv(DevMRA m, DevOper op, DevTree f, DevTree g, const int *work, int n_work, int order,
                                               LevelStats *stats, int *err) {
    extern __shared__ double sm[];
    const int K = m.K, K2 = K * K, K3 = m.kp1_d, tid = threadIdx.x, nthr = blockDim.x;
    const int dir = op.band_dir, width = op.band_dir_w;
    double *acc = sm;
    __shared__ double red[8][8];
    const int gi = work[blockIdx.x];
    const int4 gx = g.idx[gi];
    const int depth = gx.x - m.root_scale;
    for (int e = tid; e < 8 * K3; e += nthr) acc[e] = 0.0;
    __syncthreads();
    unsigned long long nt = 0, nc = 0, nb = 0;
    if (depth >= 0 && depth < op.max_rows && dir >= 0 && dir < 3) {
        const int gl[3] = {gx.y, gx.z, gx.w};
        const int *bw = op.bw + (size_t)depth * 5;  // term 0
        const int off = op.dep_off[depth], L0 = op.dep_L[depth];
        for (int w = -width; w <= width; w++) {
            int fl[3] = {gl[0], gl[1], gl[2]};
            fl[dir] += w;
            const long long c0 = (long long)m.corner[dir] * (1ll << depth), nbx = (long long)m.nbox[dir] * (1ll << depth);
            if ((long long)gl[dir] + w < c0 || (long long)gl[dir] + w >= c0 + nbx) continue;  // outside the world (getRootIndex < 0)
            NodeKey key;
            if (!pack_key(m, gx.x, fl[0], fl[1], fl[2], key)) {
                if (tid == 0) atomicOr(err, DE_RANGE);
                continue;
            }
            const int fid = hash_find(f.hkeys, f.hvals, f.hcap, key);
            if (fid < 0) {
                if (tid == 0) atomicOr(err, DE_LOOKUP);
                continue;
            }
            nb++;
            const bool gen = fid >= f.cap_real;
            const double *fc = gen ? f.gcoefs + (size_t)(fid - f.cap_real) * K3 : f.coefs + (size_t)fid * 8 * K3;
            const double *fn = f.norms + (size_t)fid * 8;
            bool any = false;
            for (int ft = 0; ft < 8; ft++) {
                if (fn[ft] < kMachineZero || (gen && ft > 0)) continue;
                for (int gt = 0; gt < 8; gt++) {
                    bool ok = true;
                    int oi_dir = 0;
                    for (int d = 0; d < 3; d++) {
                        const int oi = 2 * ((gt >> d) & 1) + ((ft >> d) & 1);
                        const int l = d == dir ? w : 0;
                        if (abs(l) > bw[oi]) { ok = false; break; }
                        if (d == dir) oi_dir = oi;
                        else if (!(oi == 0 || oi == 3)) { ok = false; break; }
                    }
                    if (!ok || off < 0 || abs(w) > L0) continue;
                    any = true;
                    nc++;
                    const double *O = op.blocks + ((size_t)(off + w + L0) * 4 + oi_dir) * K2;
                    const double *src = fc + (size_t)ft * K3;
                    double *dst = acc + (size_t)gt * K3;
                    // g(.., j, ..) += sum_i O(i, j) f(.., i, ..) along dir (column-major O, g = f^T O)
                    for (int e = tid; e < K3; e += nthr) {
                        int cd[3] = {e % K, (e / K) % K, e / K2};
                        const int j = cd[dir];
                        double s = 0.0;
                        for (int i = 0; i < K; i++) {
                            cd[dir] = i;
                            s += O[i + K * j] * src[cd[0] + K * cd[1] + K2 * cd[2]];
                        }
                        dst[e] += s;
                    }
                }
            }
            if (any) nt++;
        }
    }
    __syncthreads();  // the accumulator's elements were owned per (gt, e); below per flat index
    // division by the scaling factor to the operator order, coefficients and norms
    double sfo = 1.0;
    for (int i = 0; i < order; i++) sfo *= m.sf;
    double *go = g.coefs + (size_t)gi * 8 * K3;
    double part[8];
    for (int c = 0; c < 8; c++) part[c] = 0.0;
    for (int e = tid; e < 8 * K3; e += nthr) {
        const double v = acc[e] / sfo;
        go[e] = v;
        part[e / K3] += v * v;
    }
    for (int c = 0; c < 8; c++)
        for (int o = 16; o > 0; o >>= 1) part[c] += __shfl_down_sync(0xffffffffu, part[c], o);
    if ((tid & 31) == 0)
        for (int c = 0; c < 8; c++) red[tid >> 5][c] = part[c];
    __syncthreads();
    if (tid < 8) {
        double t = 0.0;
        for (int w = 0; w < (nthr + 31) / 32; w++) t += red[w][tid];
        g.norms[(size_t)gi * 8 + tid] = sqrt(t);
    }
    if (tid == 0) {
        atomicAdd(&stats->node_terms, nt);
        atomicAdd(&stats->components, nc);
        atomicAdd(&stats->band_nodes, nb);
    }
}

}  // namespace

void launch_deriv(const DevMRA &m, const DevOper &op, const DevTree &f, DevTree g, const int *work, int n_work, int order, LevelStats *stats,
                  int *err, cudaStream_t s) {
    if (n_work <= 0) return;
    const size_t smem = sizeof(double) * 8 * m.kp1_d;
    if (smem > 48 * 1024) cudaFuncSetAttribute(k_deriv, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    k_deriv<<<n_work, 256, smem, s>>>(m, op, f, g, work, n_work, order, stats, err);
}

void launch_band_missing(const DevMRA &m, const DevOper &op, const DevTree &f, const DevTree &g, const int *work, int n_work,
                         NodeKey *pkeys, int *pvals, int phcap, NodeKey *plist, int *pcount, int pcap, int *err, cudaStream_t s) {
    if (n_work <= 0) return;
    k_band_missing<<<n_work, 256, 0, s>>>(m, op, f, g, work, n_work, pkeys, pvals, phcap, plist, pcount, pcap, err);
}

void launch_contract_fp64(const DevMRA &m, const DevOper &op, const DevTree &f, DevTree g, const int *work, int n_work,
                          double gthr, LevelStats *stats, int *err, cudaStream_t s, const int *nw_dev, const double *gthr_dev,
                          const double *gthr_node) {
    if (n_work <= 0) return;
    // the block schedule where its 18 K^3 doubles fit (orders up to 10)
    const bool block = m.K <= kBlockMaxK && sizeof(double) * 18 * (size_t)m.kp1_d <= 227 * 1024 && !std::getenv("MWGPU_FP64_COMPONENTS");
    size_t smem = sizeof(double) * (block ? 18 : 14) * m.kp1_d;
    if (smem > 48 * 1024) cudaFuncSetAttribute(k_contract<double>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    k_contract<double><<<n_work, 256, smem, s>>>(m, op, f, g, work, n_work, gthr, stats, err, nw_dev, gthr_dev, gthr_node, block);
}

}  // namespace mwgpu
