// Tree kernels: node lookup table, GenNode generation, node norms and the
// whole-tree multiwavelet transforms.
//
// Reference behaviour restated here:
//   GenNodes        MWTree::getNode -> MWNode::retrieveNode -> threadSafeGenChildren
//                   -> tree_utils::mw_transform(readOnlyScaling)  (src/trees/MWTree.cpp:340-352,
//                   src/trees/MWNode.cpp:410-418, 1097-1120, src/utils/tree_utils.cpp:113-216)
//   node norms      MWNode::calcNorms / calcComponentNorm (src/trees/MWNode.cpp:609-655)
//   TopDown (add)   MWTree::mwTransformDown -> MWNode::giveChildrenCoefs(false) (MWTree.cpp:194-216)
//   BottomUp        MWTree::mwTransformUp -> FunctionNode<3>::reCompress -> mw_transform_back
//                   (MWTree.cpp:166-181, FunctionNode.cpp:391-409, tree_utils.cpp:229-301)
// The 1D step everywhere is math_utils::apply_filter: out(K^2 x K) = in^T (K^2 x K) * F.
#include <algorithm>
#include <cstdint>
#include <cstdlib>

#include "mwgpu_internal.cuh"

namespace mwgpu {

namespace {

constexpr int kTransformThreads = 1024;

// out[c + K2*j] (+)= sum_i in[i + K*c] * F[i + K*j]
// (consecutive threads take consecutive j of one row c: the row is a broadcast
// read and the filter columns hit distinct banks)
template <bool ADD>
__device__ __forceinline__ void dapply(double *out, const double *in, const double *F, int K, int tid, int nthr) {
    const int K2 = K * K, K3 = K2 * K;
    for (int e = tid; e < K3; e += nthr) {
        int c = e / K, j = e % K;
        const double *a = in + K * c;
        const double *b = F + K * j;
        double s = 0.0;
        for (int i = 0; i < K; i++) s = fma(a[i], b[i], s);
        if (ADD) out[c + K2 * j] += s;
        else out[c + K2 * j] = s;
    }
}

__device__ inline const double *filt(const DevMRA &m, int op, int fidx) { return m.filt + ((size_t)op * 4 + fidx) * m.K * m.K; }

__global__ void k_hash_build(DevMRA m, DevTree t, int first, int count, int *err) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= count) return;
    int id = first + i;
    int4 x = t.idx[id];
    NodeKey key;
    if (!pack_key(m, x.x, x.y, x.z, x.w, key)) { atomicOr(err, DE_RANGE); return; }
    bool full = false;
    hash_insert(t.hkeys, t.hvals, t.hcap, key, id, &full);
    if (full) atomicOr(err, DE_HASH_FULL);
}

// One CTA per pending GenNode: walk up to the nearest node present in the
// lookup table, then reconstruct down along the path to the requested child.
__global__ void k_gen_nodes(DevMRA m, DevTree f, const NodeKey *plist, int n_pend, int gen_base, int *err, bool real_only) {
    extern __shared__ double sm[];
    const int K = m.K, K3 = m.kp1_d;
    double *b0 = sm;           // 4 K^3
    double *b1 = sm + 4 * K3;  // 4 K^3
    __shared__ int s_anc, s_ancn;
    int p = blockIdx.x;
    if (p >= n_pend) return;
    int n, l0, l1, l2;
    unpack_key(m, plist[p], n, l0, l1, l2);
    if (threadIdx.x == 0) {
        s_anc = -1;
        s_ancn = 0;
        for (int a = n - 1; a >= m.root_scale; a--) {
            int sh = n - a;
            NodeKey key;
            if (!pack_key(m, a, l0 >> sh, l1 >> sh, l2 >> sh, key)) break;
            int id = hash_find(f.hkeys, f.hvals, f.hcap, key);
            if (id >= 0 && (!real_only || id < f.cap_real)) { s_anc = id; s_ancn = a; break; }
        }
    }
    __syncthreads();
    int anc = s_anc, an = s_ancn;
    if (anc < 0) {
        if (threadIdx.x == 0) atomicOr(err, DE_LOOKUP);
        return;
    }
    const int tid = threadIdx.x, nthr = blockDim.x;
    const double *src;
    bool real = anc < f.cap_real;
    // first step
    {
        int sh = n - an - 1;
        int c0 = (l0 >> sh) & 1, c1 = (l1 >> sh) & 1, c2 = (l2 >> sh) & 1;
        if (real) {
            const double *in = f.coefs + (size_t)anc * 8 * K3;
            // stage 0: tmp[(c0,b1,b2)] for the 4 (b1,b2), slot q = b1 + 2*b2
            for (int q = 0; q < 4; q++) {
                int ftlo = 2 * q;  // b0 = 0, bits b1,b2 from q
                dapply<false>(b0 + q * K3, in + (size_t)ftlo * K3, filt(m, 1, 2 * c0 + 0), K, tid, nthr);
            }
            __syncthreads();
            for (int q = 0; q < 4; q++) dapply<true>(b0 + q * K3, in + (size_t)(2 * q + 1) * K3, filt(m, 1, 2 * c0 + 1), K, tid, nthr);
            __syncthreads();
            // stage 1: tmp2[(c0,c1,b2)], slot b2
            for (int b2 = 0; b2 < 2; b2++) dapply<false>(b1 + b2 * K3, b0 + (0 + 2 * b2) * K3, filt(m, 1, 2 * c1 + 0), K, tid, nthr);
            __syncthreads();
            for (int b2 = 0; b2 < 2; b2++) dapply<true>(b1 + b2 * K3, b0 + (1 + 2 * b2) * K3, filt(m, 1, 2 * c1 + 1), K, tid, nthr);
            __syncthreads();
            // stage 2
            dapply<false>(b0, b1, filt(m, 1, 2 * c2 + 0), K, tid, nthr);
            __syncthreads();
            dapply<true>(b0, b1 + K3, filt(m, 1, 2 * c2 + 1), K, tid, nthr);
            __syncthreads();
        } else {
            const double *in = f.gcoefs + (size_t)(anc - f.cap_real) * K3;
            dapply<false>(b1, in, filt(m, 1, 2 * c0), K, tid, nthr);
            __syncthreads();
            dapply<false>(b1 + K3, b1, filt(m, 1, 2 * c1), K, tid, nthr);
            __syncthreads();
            dapply<false>(b0, b1 + K3, filt(m, 1, 2 * c2), K, tid, nthr);
            __syncthreads();
        }
        src = b0;
    }
    // remaining steps from scaling-only parents
    for (int a = an + 1; a < n; a++) {
        int sh = n - a - 1;
        int c0 = (l0 >> sh) & 1, c1 = (l1 >> sh) & 1, c2 = (l2 >> sh) & 1;
        dapply<false>(b1, src, filt(m, 1, 2 * c0), K, tid, nthr);
        __syncthreads();
        dapply<false>(b1 + K3, b1, filt(m, 1, 2 * c1), K, tid, nthr);
        __syncthreads();
        dapply<false>(b0, b1 + K3, filt(m, 1, 2 * c2), K, tid, nthr);
        __syncthreads();
        src = b0;
    }
    int slot = gen_base + p;
    if (slot >= f.cap_gen) {
        if (tid == 0) atomicOr(err, DE_POOL_FULL);
        return;
    }
    double *out = f.gcoefs + (size_t)slot * K3;
    float *out32 = f.gcoefs32 + (size_t)slot * K3;
    float *tc = f.gtc32 ? f.gtc32 + (size_t)slot * kTcGenFloats : nullptr;
    for (int e = tid; e < K3; e += nthr) {
        out[e] = src[e];
        out32[e] = (float)src[e];
        if (tc) tc_gen_store(tc, e, (float)src[e]);
    }
    // scaling norm (GenNode wavelet norms are zero)
    __shared__ double red[32];
    double s = 0.0;
    for (int e = tid; e < K3; e += nthr) s += src[e] * src[e];
    for (int o = 16; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o);
    if ((tid & 31) == 0) red[tid >> 5] = s;
    __syncthreads();
    if (tid == 0) {
        double t = 0.0;
        for (int w = 0; w < (nthr + 31) / 32; w++) t += red[w];
        double *nr = f.norms + (size_t)(f.cap_real + slot) * 8;
        nr[0] = sqrt(t);
        for (int c = 1; c < 8; c++) nr[c] = 0.0;
        f.idx[f.cap_real + slot] = make_int4(n, l0, l1, l2);
    }
}

__global__ void k_gen_insert(DevMRA m, DevTree f, const NodeKey *plist, int n_pend, int gen_base, int *err) {
    int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= n_pend) return;
    bool full = false;
    hash_insert(f.hkeys, f.hvals, f.hcap, plist[p], f.cap_real + gen_base + p, &full);
    if (full) atomicOr(err, DE_HASH_FULL);
}

__device__ void block_norms(const double *c, int K3, double *nr, int tid, int nthr) {
    __shared__ double red[8][32];
    for (int comp = 0; comp < 8; comp++) {
        double s = 0.0;
        for (int e = tid; e < K3; e += nthr) { double v = c[comp * K3 + e]; s += v * v; }
        for (int o = 16; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o);
        if ((tid & 31) == 0) red[comp][tid >> 5] = s;
    }
    __syncthreads();
    if (tid < 8) {
        double t = 0.0;
        for (int w = 0; w < (nthr + 31) / 32; w++) t += red[tid][w];
        nr[tid] = sqrt(t);
    }
    __syncthreads();
}

// Node norms with warp w summing component w (256 threads): FP64 arithmetic is
// slow on this part, so each lane does K^3/32 products and one shuffle tree.
__device__ __forceinline__ void block_norms8(const double *c, int K3, double *nr, int tid) {
    const int w = tid >> 5, lane = tid & 31;
    double s = 0.0;
    for (int e = lane; e < K3; e += 32) {
        const double v = c[(size_t)w * K3 + e];
        s += v * v;
    }
    for (int o = 16; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o);
    if (lane == 0) nr[w] = sqrt(s);
}

__global__ void k_node_norms(DevMRA m, DevTree t, const int *nodes, int n) {
    int i = nodes[blockIdx.x];
    block_norms(t.coefs + (size_t)i * 8 * m.kp1_d, m.kp1_d, t.norms + (size_t)i * 8, threadIdx.x, blockDim.x);
}

// TopDown: parent (s,d) -> children scaling, added (overwrite=false) or assigned.
// With ptree set, parent j belongs to tree ts[ptree[j]] (several trees per launch).
__global__ void k_mw_down(DevMRA m, DevTree t0, const DevTree *ts, const int *ptree, const int *parents, int n, bool overwrite) {
    extern __shared__ double sm[];
    const DevTree t = ptree ? ts[ptree[blockIdx.x]] : t0;
    const int K = m.K, K3 = m.kp1_d, tid = threadIdx.x, nthr = blockDim.x;
    double *t1 = sm, *t2 = sm + 8 * K3;
    int p = parents[blockIdx.x];
    int c0 = t.child0[p];
    if (c0 < 0) return;
    const double *in = t.coefs + (size_t)p * 8 * K3;
    // stage 0 (direction x)
    for (int gt = 0; gt < 8; gt++) {
        dapply<false>(t1 + gt * K3, in + (size_t)(gt & ~1) * K3, filt(m, 1, 2 * (gt & 1) + 0), K, tid, nthr);
    }
    __syncthreads();
    for (int gt = 0; gt < 8; gt++) dapply<true>(t1 + gt * K3, in + (size_t)(gt | 1) * K3, filt(m, 1, 2 * (gt & 1) + 1), K, tid, nthr);
    __syncthreads();
    // stage 1 (direction y)
    for (int gt = 0; gt < 8; gt++) dapply<false>(t2 + gt * K3, t1 + (gt & ~2) * K3, filt(m, 1, 2 * ((gt >> 1) & 1) + 0), K, tid, nthr);
    __syncthreads();
    for (int gt = 0; gt < 8; gt++) dapply<true>(t2 + gt * K3, t1 + (gt | 2) * K3, filt(m, 1, 2 * ((gt >> 1) & 1) + 1), K, tid, nthr);
    __syncthreads();
    // stage 2 (direction z) straight into the children scaling blocks
    for (int gt = 0; gt < 8; gt++) {
        double *o = t.coefs + (size_t)(c0 + gt) * 8 * K3;
        if (overwrite) {
            for (int e = tid; e < 8 * K3; e += nthr) o[e] = 0.0;
            __syncthreads();
            dapply<false>(o, t2 + (gt & ~4) * K3, filt(m, 1, 2 * ((gt >> 2) & 1) + 0), K, tid, nthr);
        } else {
            dapply<true>(o, t2 + (gt & ~4) * K3, filt(m, 1, 2 * ((gt >> 2) & 1) + 0), K, tid, nthr);
        }
    }
    __syncthreads();
    for (int gt = 0; gt < 8; gt++) {
        double *o = t.coefs + (size_t)(c0 + gt) * 8 * K3;
        dapply<true>(o, t2 + (gt | 4) * K3, filt(m, 1, 2 * ((gt >> 2) & 1) + 1), K, tid, nthr);
    }
    __syncthreads();
    for (int gt = 0; gt < 8; gt++) block_norms(t.coefs + (size_t)(c0 + gt) * 8 * K3, K3, t.norms + (size_t)(c0 + gt) * 8, tid, nthr);
}

// BottomUp: 8 children scaling blocks -> parent (s,d), then parent norms.
__global__ void k_mw_up(DevMRA m, DevTree t0, const DevTree *ts, const int *ptree, const int *parents, int n) {
    extern __shared__ double sm[];
    const DevTree t = ptree ? ts[ptree[blockIdx.x]] : t0;
    const int K = m.K, K3 = m.kp1_d, tid = threadIdx.x, nthr = blockDim.x;
    double *t1 = sm, *t2 = sm + 8 * K3;
    int p = parents[blockIdx.x];
    int c0 = t.child0[p];
    if (c0 < 0) return;
    for (int ct = 0; ct < 8; ct++) {
        const double *cs = t.coefs + (size_t)(c0 + ct) * 8 * K3;
        for (int e = tid; e < K3; e += nthr) t1[ct * K3 + e] = cs[e];
    }
    __syncthreads();
    double *bufs[2] = {t1, t2};
    for (int d = 0; d < 3; d++) {
        double *in = bufs[d & 1], *out = bufs[(d + 1) & 1];
        int mask = 1 << d;
        for (int gt = 0; gt < 8; gt++)
            dapply<false>(out + gt * K3, in + (gt & ~mask) * K3, filt(m, 0, 2 * ((gt >> d) & 1) + 0), K, tid, nthr);
        __syncthreads();
        for (int gt = 0; gt < 8; gt++)
            dapply<true>(out + gt * K3, in + (gt | mask) * K3, filt(m, 0, 2 * ((gt >> d) & 1) + 1), K, tid, nthr);
        __syncthreads();
    }
    double *pc = t.coefs + (size_t)p * 8 * K3;
    for (int e = tid; e < 8 * K3; e += nthr) pc[e] = t2[e];
    __syncthreads();
    block_norms(pc, K3, t.norms + (size_t)p * 8, tid, nthr);
}

// ProjectionCalculator::calcNode (ProjectionCalculator.cpp:34-51) for one node
// per CTA, of a sum of Gaussians c_g exp(-a_g |r - R_g|^2): the function at the
// quadrature points of the 8 children (MWNode::getExpandedChildPts,
// MWNode.cpp:854-935; x fastest), cvTransform(Backward) (MWNode.cpp:448-490:
// the value-to-coefficient map along each direction, times
// sqrt(sf^3 2^(-3 (n+1)))), the compression of the 8 child blocks
// (mwTransform(Compression)) and the node norms.  FP64.  gauss: [n][5] =
// coefficient, exponent, position; or values: the function at those points,
// 8 (k+1)^3 per node in the same order (evaluated by the caller).
__global__ void k_project(DevMRA m, DevTree t, const int *nodes, int n, const double *gauss, int ng, const double *vc_map, const double *roots,
                          const double *values) {
    extern __shared__ double sm[];
    const int K = m.K, K3 = m.kp1_d, tid = threadIdx.x, nthr = blockDim.x;
    double *t1 = sm, *t2 = sm + 8 * K3;
    const int i = nodes[blockIdx.x];
    const int4 nd = t.idx[i];
    const double sfac = exp2(-(double)(nd.x + 1));
    const int lq[3] = {nd.y, nd.z, nd.w};
    for (int e = tid; e < 8 * K3; e += nthr) {
        if (values) {
            t1[e] = values[(size_t)blockIdx.x * 8 * K3 + e];
            continue;
        }
        const int ct = e / K3, p = e % K3;
        double r[3];
        int rem = p;
        for (int d = 0; d < 3; d++) {
            const int q = rem % K;
            rem /= K;
            r[d] = m.sf * (sfac * (roots[q] + 2.0 * lq[d] + ((ct >> d) & 1)));
        }
        double v = 0.0;
        for (int g = 0; g < ng; g++) {
            const double *G = gauss + 5 * g;
            const double dx = r[0] - G[2], dy = r[1] - G[3], dz = r[2] - G[4];
            v += G[0] * exp(-G[1] * (dx * dx + dy * dy + dz * dz));
        }
        t1[e] = v;
    }
    __syncthreads();
    // cvTransform(Backward): the K x K value-to-coefficient map along x, y, z of every child block
    double *bufs[2] = {t1, t2};
    for (int d = 0; d < 3; d++) {
        double *in = bufs[d & 1], *out = bufs[(d + 1) & 1];
        for (int ct = 0; ct < 8; ct++) dapply<false>(out + ct * K3, in + ct * K3, vc_map, K, tid, nthr);
        __syncthreads();
    }
    // result in t2; scale: sqrt(sf^3 / 2^(3 (n+1)))
    const double two_fac = sqrt(m.sf * m.sf * m.sf / exp2(3.0 * (nd.x + 1)));
    for (int e = tid; e < 8 * K3; e += nthr) t1[e] = two_fac * t2[e];
    __syncthreads();
    // mwTransform(Compression): 8 child scaling blocks -> s + d of the node
    for (int d = 0; d < 3; d++) {
        double *in = bufs[d & 1], *out = bufs[(d + 1) & 1];
        const int mask = 1 << d;
        for (int gt = 0; gt < 8; gt++)
            dapply<false>(out + gt * K3, in + (gt & ~mask) * K3, filt(m, 0, 2 * ((gt >> d) & 1) + 0), K, tid, nthr);
        __syncthreads();
        for (int gt = 0; gt < 8; gt++)
            dapply<true>(out + gt * K3, in + (gt | mask) * K3, filt(m, 0, 2 * ((gt >> d) & 1) + 1), K, tid, nthr);
        __syncthreads();
    }
    double *pc = t.coefs + (size_t)i * 8 * K3;
    for (int e = tid; e < 8 * K3; e += nthr) pc[e] = t2[e];
    __syncthreads();
    block_norms(pc, K3, t.norms + (size_t)i * 8, tid, nthr);
}

// The three directional filter stages of a node transform in shared memory:
// op 0 compresses 8 child scaling blocks into s + d, op 1 reconstructs
// (tree_utils::mw_transform / mw_transform_back, tree_utils.cpp:113-301).
// in: t1, result in t2 (t1 is overwritten).
__device__ void node_mw3(const DevMRA &m, int op, double *t1, double *t2, int tid, int nthr) {
    const int K = m.K, K3 = m.kp1_d;
    double *bufs[2] = {t1, t2};
    for (int d = 0; d < 3; d++) {
        double *in = bufs[d & 1], *out = bufs[(d + 1) & 1];
        const int mask = 1 << d;
        for (int gt = 0; gt < 8; gt++) dapply<false>(out + gt * K3, in + (gt & ~mask) * K3, filt(m, op, 2 * ((gt >> d) & 1) + 0), K, tid, nthr);
        __syncthreads();
        for (int gt = 0; gt < 8; gt++) dapply<true>(out + gt * K3, in + (gt | mask) * K3, filt(m, op, 2 * ((gt >> d) & 1) + 1), K, tid, nthr);
        __syncthreads();
    }
}

// cvTransform (MWNode.cpp:448-490) of 8 child blocks with the K x K map S along
// x, y, z, times fac: in t1, result in t2
__device__ void node_cv(const DevMRA &m, const double *S, double fac, double *t1, double *t2, int tid, int nthr) {
    const int K = m.K, K3 = m.kp1_d;
    double *bufs[2] = {t1, t2};
    for (int d = 0; d < 3; d++) {
        double *in = bufs[d & 1], *out = bufs[(d + 1) & 1];
        for (int ct = 0; ct < 8; ct++) dapply<false>(out + ct * K3, in + ct * K3, S, K, tid, nthr);
        __syncthreads();
    }
    for (int e = tid; e < 8 * K3; e += nthr) t2[e] *= fac;
    __syncthreads();
}

// AdditionCalculator / MultiplicationCalculator::calcNode (AdditionCalculator.h:42-66,
// MultiplicationCalculator.h:42-72) for one output node per CTA and inputs
// ins[0..n_in) with factors c[j]: the input node of the same index (a GenNode
// made beforehand where the input tree has none: scaling block only).  Sum:
// out = sum_j c_j in_j in the compressed form.  Product: every input node is
// reconstructed to its children's scaling blocks and transformed to values at
// the children's quadrature points (cvTransform Forward), the values are
// multiplied, transformed back (Backward) and compressed.  FP64; node norms.
template <bool MUL>
__global__ void k_combine(DevMRA m, const DevTree *ins, const double *c, int n_in, DevTree out, const int *nodes, int n, const double *cv_map,
                          const double *vc_map, int *err) {
    extern __shared__ double sm[];
    const int K3 = m.kp1_d, tid = threadIdx.x, nthr = blockDim.x;
    double *acc = sm, *t1 = sm + 8 * K3, *t2 = sm + 16 * K3;
    const int i = nodes[blockIdx.x];
    const int4 nd = out.idx[i];
    const double fw = sqrt(exp2(3.0 * (nd.x + 1)) / (m.sf * m.sf * m.sf));
    for (int e = tid; e < 8 * K3; e += nthr) acc[e] = MUL ? 1.0 : 0.0;
    __syncthreads();
    NodeKey key;
    const bool kok = pack_key(m, nd.x, nd.y, nd.z, nd.w, key);
    for (int j = 0; j < n_in; j++) {
        const DevTree &f = ins[j];
        const int fid = kok ? hash_find(f.hkeys, f.hvals, f.hcap, key) : -1;
        if (fid < 0) {
            if (tid == 0) atomicOr(err, DE_LOOKUP);
            continue;
        }
        const bool gen = fid >= f.cap_real;
        const double *fc = gen ? f.gcoefs + (size_t)(fid - f.cap_real) * K3 : f.coefs + (size_t)fid * 8 * K3;
        if (!MUL) {
            for (int e = tid; e < 8 * K3; e += nthr) acc[e] += c[j] * ((gen && e >= K3) ? 0.0 : fc[e]);
            continue;
        }
        for (int e = tid; e < 8 * K3; e += nthr) t1[e] = (gen && e >= K3) ? 0.0 : fc[e];
        __syncthreads();
        node_mw3(m, 1, t1, t2, tid, nthr);        // children's scaling blocks in t2
        for (int e = tid; e < 8 * K3; e += nthr) t1[e] = t2[e];
        __syncthreads();
        node_cv(m, cv_map, fw, t1, t2, tid, nthr);  // values in t2
        for (int e = tid; e < 8 * K3; e += nthr) acc[e] *= c[j] * t2[e];
        __syncthreads();
    }
    __syncthreads();
    double *oc = out.coefs + (size_t)i * 8 * K3;
    if (MUL) {
        for (int e = tid; e < 8 * K3; e += nthr) t1[e] = acc[e];
        __syncthreads();
        node_cv(m, vc_map, 1.0 / fw, t1, t2, tid, nthr);  // coefficients of the children in t2
        for (int e = tid; e < 8 * K3; e += nthr) t1[e] = t2[e];
        __syncthreads();
        node_mw3(m, 0, t1, t2, tid, nthr);                // compressed in t2
        for (int e = tid; e < 8 * K3; e += nthr) oc[e] = t2[e];
    } else {
        for (int e = tid; e < 8 * K3; e += nthr) oc[e] = acc[e];
    }
    __syncthreads();
    block_norms(oc, K3, out.norms + (size_t)i * 8, tid, nthr);
}

// The transforms of the mixed form: the same three filter stages with FP32
// products in shared memory, the children / parent coefficients kept in FP64.
template <bool ADD>
__device__ __forceinline__ void fapply(float *out, const float *in, const float *F, int K, int tid, int nthr) {
    const int K2 = K * K, K3 = K2 * K;
    for (int e = tid; e < K3; e += nthr) {
        const int c = e / K, j = e % K;
        const float *a = in + K * c;
        const float *b = F + K * j;
        float s = 0.f;
        for (int i = 0; i < K; i++) s = fmaf(a[i], b[i], s);
        if (ADD) out[c + K2 * j] += s;
        else out[c + K2 * j] = s;
    }
}

// filters of op (0 compression, 1 reconstruction) as floats: F[fidx * K2 + ...]
__device__ __forceinline__ void load_filters32(float *F, const DevMRA &m, int op, int tid, int nthr) {
    const int n = 4 * m.K * m.K;
    const double *src = m.filt + (size_t)op * n;
    for (int e = tid; e < n; e += nthr) F[e] = (float)src[e];
}

// One 1D filter stage over the 8 blocks of a node, both inputs of an output in
// one pass: out[gt] = in[gt & ~m] F[2 b] + in[gt | m] F[2 b + 1], m = 1 << d,
// b = bit d of gt (the sums of fapply<false> then fapply<true>, bit for bit).
// All threads of the block share the 8 (k+1)^3 outputs.
__device__ __forceinline__ void fstage8(float *out, const float *in, const float *F, int d, int K, int tid, int nthr) {
    const int K2 = K * K, K3 = K2 * K, m = 1 << d;
    for (int e = tid; e < 8 * K3; e += nthr) {
        const int gt = e / K3, r = e - gt * K3, c = r / K, j = r - c * K;
        const int b = (gt >> d) & 1;
        const float *a0 = in + (size_t)(gt & ~m) * K3 + K * c, *a1 = in + (size_t)(gt | m) * K3 + K * c;
        const float *f0 = F + (2 * b) * K2 + K * j, *f1 = F + (2 * b + 1) * K2 + K * j;
        float s0 = 0.f, s1 = 0.f;
        for (int i = 0; i < K; i++) {
            s0 = fmaf(a0[i], f0[i], s0);
            s1 = fmaf(a1[i], f1[i], s1);
        }
        out[(size_t)gt * K3 + c + K2 * j] = s0 + s1;
    }
}

// out[q] = in[2q] F0 + in[2q+1] F1 for q < nout (one filter direction applied
// to nout pairs of blocks, both inputs of an output in one pass)
__device__ __forceinline__ void fpairs(float *out, const float *in, int nout, const float *F0, const float *F1, int K, int tid, int nthr) {
    const int K2 = K * K, K3 = K2 * K;
    for (int e = tid; e < nout * K3; e += nthr) {
        const int q = e / K3, r = e - q * K3, c = r / K, j = r - c * K;
        const float *a0 = in + (size_t)(2 * q) * K3 + K * c, *a1 = a0 + K3;
        const float *f0 = F0 + K * j, *f1 = F1 + K * j;
        float s0 = 0.f, s1 = 0.f;
        for (int i = 0; i < K; i++) {
            s0 = fmaf(a0[i], f0[i], s0);
            s1 = fmaf(a1[i], f1[i], s1);
        }
        out[(size_t)q * K3 + c + K2 * j] = s0 + s1;
    }
}

// (one CTA of kTransformThreads per parent: the levels of a tree are short,
// so the latency of one parent is the launch's time)
__global__ void __launch_bounds__(kTransformThreads) k_mw_down32(DevMRA m, DevTree t0, const DevTree *ts, const int *ptree, const int *parents,
                                                                int n, bool overwrite) {
    extern __shared__ float sm32[];
    const DevTree t = ptree ? ts[ptree[blockIdx.x]] : t0;
    const int K = m.K, K3 = m.kp1_d, tid = threadIdx.x, nthr = blockDim.x;
    float *t1 = sm32, *t2 = t1 + 8 * K3, *F = t2 + 8 * K3;
    const int p = parents[blockIdx.x];
    const int c0 = t.child0[p];
    if (c0 < 0) return;
    const double *in = t.coefs + (size_t)p * 8 * K3;
    for (int e = tid; e < 8 * K3; e += nthr) t2[e] = (float)in[e];
    load_filters32(F, m, 1, tid, nthr);
    __syncthreads();
    fstage8(t1, t2, F, 0, K, tid, nthr);
    __syncthreads();
    fstage8(t2, t1, F, 1, K, tid, nthr);
    __syncthreads();
    fstage8(t1, t2, F, 2, K, tid, nthr);
    __syncthreads();
    // child gt receives the scaling block t1[gt] (its wavelet blocks are untouched: only the scaling part is passed down)
    for (int e = tid; e < 8 * K3; e += nthr) {
        const int gt = e / K3, r = e % K3;
        double *o = t.coefs + (size_t)(c0 + gt) * 8 * K3;
        if (overwrite) {
            // overwrite: the child's whole block is replaced by its scaling part
            for (int cc = 0; cc < 8; cc++)
                if (cc == 0) o[r] = (double)t1[e];
                else o[cc * K3 + r] = 0.0;
        } else {
            o[r] += (double)t1[e];
        }
    }
    __syncthreads();
    // only the scaling component of a child changed: warp w < 8 recomputes the
    // scaling norm of child w (the wavelet norms stay, or are 0 when overwritten)
    if (tid < 256) {
        const int w = tid >> 5, lane = tid & 31;
        const double *cc = t.coefs + (size_t)(c0 + w) * 8 * K3;
        double s = 0.0;
        for (int e = lane; e < K3; e += 32) s += cc[e] * cc[e];
        for (int o = 16; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o);
        double *nr = t.norms + (size_t)(c0 + w) * 8;
        if (lane == 0) nr[0] = sqrt(s);
        if (overwrite && lane >= 1 && lane < 8) nr[lane] = 0.0;
    }
}

__global__ void __launch_bounds__(kTransformThreads) k_mw_up32(DevMRA m, DevTree t0, const DevTree *ts, const int *ptree, const int *parents,
                                                              int n) {
    extern __shared__ float sm32[];
    const DevTree t = ptree ? ts[ptree[blockIdx.x]] : t0;
    const int K = m.K, K3 = m.kp1_d, tid = threadIdx.x, nthr = blockDim.x;
    float *t1 = sm32, *t2 = t1 + 8 * K3, *F = t2 + 8 * K3;
    const int p = parents[blockIdx.x];
    const int c0 = t.child0[p];
    if (c0 < 0) return;
    for (int e = tid; e < 8 * K3; e += nthr) t1[e] = (float)t.coefs[(size_t)(c0 + e / K3) * 8 * K3 + e % K3];
    load_filters32(F, m, 0, tid, nthr);
    __syncthreads();
    fstage8(t2, t1, F, 0, K, tid, nthr);
    __syncthreads();
    fstage8(t1, t2, F, 1, K, tid, nthr);
    __syncthreads();
    fstage8(t2, t1, F, 2, K, tid, nthr);
    __syncthreads();
    double *pc = t.coefs + (size_t)p * 8 * K3;
    for (int e = tid; e < 8 * K3; e += nthr) pc[e] = (double)t2[e];
    __syncthreads();
    if (tid < 256) block_norms8(pc, K3, t.norms + (size_t)p * 8, tid);
}

// GenNodes of the mixed form: the path reconstruction of k_gen_nodes with FP32
// products (filters and buffers in shared memory), starting from the FP32 copy
// of the real ancestor or from an FP32 GenNode.  The result goes to gcoefs32
// (read by the mixed contraction) and, widened, to gcoefs; the scaling norm is
// accumulated in FP64.  The intermediate steps stay in FP32, so a chain through
// stored GenNodes gives the same values as one walk from the real ancestor.
__global__ void k_gen_nodes32(DevMRA m, DevTree f, const NodeKey *plist, int n_pend, int gen_base, int *err, bool real_only) {
    extern __shared__ float sg32[];
    const int K = m.K, K2 = K * K, K3 = m.kp1_d;
    float *b0 = sg32, *b1 = b0 + 4 * K3, *F = b1 + 4 * K3;  // F: the 4 reconstruction filters
    __shared__ int s_anc, s_ancn;
    const int p = blockIdx.x;
    if (p >= n_pend) return;
    int n, l0, l1, l2;
    unpack_key(m, plist[p], n, l0, l1, l2);
    const int tid = threadIdx.x, nthr = blockDim.x;
    if (tid == 0) {
        s_anc = -1;
        s_ancn = 0;
        for (int a = n - 1; a >= m.root_scale; a--) {
            const int sh = n - a;
            NodeKey key;
            if (!pack_key(m, a, l0 >> sh, l1 >> sh, l2 >> sh, key)) break;
            const int id = hash_find(f.hkeys, f.hvals, f.hcap, key);
            if (id >= 0 && (!real_only || id < f.cap_real)) {
                s_anc = id;
                s_ancn = a;
                break;
            }
        }
    }
    load_filters32(F, m, 1, tid, nthr);
    __syncthreads();
    const int anc = s_anc, an = s_ancn;
    if (anc < 0) {
        if (tid == 0) atomicOr(err, DE_LOOKUP);
        return;
    }
    const float *src;
    {
        const int sh = n - an - 1;
        const int c0 = (l0 >> sh) & 1, c1 = (l1 >> sh) & 1, c2 = (l2 >> sh) & 1;
        if (anc < f.cap_real) {
            // from the real ancestor's 8 components: x, y, z with both inputs of
            // an output in one pass (the sums of fapply<false> then fapply<true>)
            const float *in = f.coefs32 + (size_t)anc * 8 * K3;
            fpairs(b0, in, 4, F + (2 * c0) * K2, F + (2 * c0 + 1) * K2, K, tid, nthr);
            __syncthreads();
            fpairs(b1, b0, 2, F + (2 * c1) * K2, F + (2 * c1 + 1) * K2, K, tid, nthr);
            __syncthreads();
            fpairs(b0, b1, 1, F + (2 * c2) * K2, F + (2 * c2 + 1) * K2, K, tid, nthr);
            __syncthreads();
        } else {
            const float *in = f.gcoefs32 + (size_t)(anc - f.cap_real) * K3;
            fapply<false>(b1, in, F + (2 * c0) * K2, K, tid, nthr);
            __syncthreads();
            fapply<false>(b1 + K3, b1, F + (2 * c1) * K2, K, tid, nthr);
            __syncthreads();
            fapply<false>(b0, b1 + K3, F + (2 * c2) * K2, K, tid, nthr);
            __syncthreads();
        }
        src = b0;
    }
    for (int a = an + 1; a < n; a++) {
        const int sh = n - a - 1;
        const int c0 = (l0 >> sh) & 1, c1 = (l1 >> sh) & 1, c2 = (l2 >> sh) & 1;
        fapply<false>(b1, src, F + (2 * c0) * K2, K, tid, nthr);
        __syncthreads();
        fapply<false>(b1 + K3, b1, F + (2 * c1) * K2, K, tid, nthr);
        __syncthreads();
        fapply<false>(b0, b1 + K3, F + (2 * c2) * K2, K, tid, nthr);
        __syncthreads();
        src = b0;
    }
    const int slot = gen_base + p;
    if (slot >= f.cap_gen) {
        if (tid == 0) atomicOr(err, DE_POOL_FULL);
        return;
    }
    double *out = f.gcoefs + (size_t)slot * K3;
    float *out32 = f.gcoefs32 + (size_t)slot * K3;
    float *tc = f.gtc32 ? f.gtc32 + (size_t)slot * kTcGenFloats : nullptr;
    double s = 0.0;
    for (int e = tid; e < K3; e += nthr) {
        const float v = src[e];
        out32[e] = v;
        out[e] = (double)v;
        if (tc) tc_gen_store(tc, e, v);
        s += (double)v * (double)v;
    }
    __shared__ double red[32];
    for (int o = 16; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o);
    if ((tid & 31) == 0) red[tid >> 5] = s;
    __syncthreads();
    if (tid == 0) {
        double t = 0.0;
        for (int w = 0; w < (nthr + 31) / 32; w++) t += red[w];
        double *nr = f.norms + (size_t)(f.cap_real + slot) * 8;
        nr[0] = sqrt(t);
        for (int c = 1; c < 8; c++) nr[c] = 0.0;
        f.idx[f.cap_real + slot] = make_int4(n, l0, l1, l2);
    }
}

// GenNodes of the mixed form, one parent (family) per CTA: the children
// fam_slots[8 q + c] >= 0 of parent fam_keys[q] (c = x bit | y bit << 1 |
// z bit << 2) from the parent's nearest real ancestor.  The x- and y-step
// blocks are computed once for the children that share them; each child's
// value is the same sequence of filter products as in k_gen_nodes32 (real
// parent: the two-input steps from its 8 components; otherwise the parent's
// scaling block along the path, then one-input steps), so the values are
// bit-identical to it.  Shared memory: three regions of 8 blocks + filters.
__global__ void k_gen_family32(DevMRA m, DevTree f, const NodeKey *fam_keys, const int *fam_slots, int n_fam, const int *n_fam_dev, int gen_base,
                               bool real_only, int *err) {
    extern __shared__ float sh_fam[];
    const int K = m.K, K2 = K * K, K3 = m.kp1_d;
    float *R0 = sh_fam, *R1 = R0 + 8 * K3, *R2 = R1 + 8 * K3, *F = R2 + 8 * K3;
    __shared__ int s_anc, s_ancn, s_slot[8];
    __shared__ double red[32];
    const int q = blockIdx.x;
    if (q >= (n_fam_dev ? min(n_fam, *n_fam_dev) : n_fam)) return;
    int n, l0, l1, l2;  // the parent
    unpack_key(m, fam_keys[q], n, l0, l1, l2);
    const int tid = threadIdx.x, nthr = blockDim.x;
    if (tid < 8) s_slot[tid] = fam_slots[8 * q + tid];
    if (tid == 0) {
        s_anc = -1;
        s_ancn = 0;
        for (int a = n; a >= m.root_scale; a--) {
            const int sh = n - a;
            NodeKey key;
            if (!pack_key(m, a, l0 >> sh, l1 >> sh, l2 >> sh, key)) break;
            const int id = hash_find(f.hkeys, f.hvals, f.hcap, key);
            if (id >= 0 && (!real_only || id < f.cap_real)) {
                s_anc = id;
                s_ancn = a;
                break;
            }
        }
    }
    load_filters32(F, m, 1, tid, nthr);
    __syncthreads();
    const int anc = s_anc, an = s_ancn;
    if (anc < 0) {
        if (tid == 0) atomicOr(err, DE_LOOKUP);
        return;
    }
    const bool anc_real = anc < f.cap_real;
    unsigned need = 0, need_x = 0, need_xy = 0;
    for (int c = 0; c < 8; c++)
        if (s_slot[c] >= 0) {
            need |= 1u << c;
            need_x |= 1u << (c & 1);
            need_xy |= 1u << (c & 3);
        }
    const float *child[8];
    if (an == n && anc_real) {
        // real parent: x, y, z steps with both inputs of an output in one pass
        const float *in = f.coefs32 + (size_t)anc * 8 * K3;
        for (int c0 = 0; c0 < 2; c0++)
            if (need_x >> c0 & 1) fpairs(R0 + 4 * c0 * K3, in, 4, F + (2 * c0) * K2, F + (2 * c0 + 1) * K2, K, tid, nthr);
        __syncthreads();
        for (int c01 = 0; c01 < 4; c01++)
            if (need_xy >> c01 & 1) {
                const int c0 = c01 & 1, c1 = c01 >> 1;
                fpairs(R1 + 2 * c01 * K3, R0 + 4 * c0 * K3, 2, F + (2 * c1) * K2, F + (2 * c1 + 1) * K2, K, tid, nthr);
            }
        __syncthreads();
        for (int c = 0; c < 8; c++) {
            child[c] = R2 + c * K3;
            if (need >> c & 1) fpairs(R2 + c * K3, R1 + 2 * (c & 3) * K3, 1, F + (2 * (c >> 2)) * K2, F + (2 * (c >> 2) + 1) * K2, K, tid, nthr);
        }
        __syncthreads();
    } else {
        // the parent's scaling block: a GenNode's own block, or along the path
        // from the ancestor (its 8 components if real, its scaling block if a GenNode)
        const float *src;
        float *dst = R1;
        if (an == n) {
            src = f.gcoefs32 + (size_t)(anc - f.cap_real) * K3;
        } else {
            const int sh = n - an;  // the path bit at level an + 1
            const int c0 = (l0 >> (sh - 1)) & 1, c1 = (l1 >> (sh - 1)) & 1, c2 = (l2 >> (sh - 1)) & 1;
            if (anc_real) {
                const float *in = f.coefs32 + (size_t)anc * 8 * K3;
                fpairs(R0, in, 4, F + (2 * c0) * K2, F + (2 * c0 + 1) * K2, K, tid, nthr);
                __syncthreads();
                fpairs(R1, R0, 2, F + (2 * c1) * K2, F + (2 * c1 + 1) * K2, K, tid, nthr);
                __syncthreads();
                fpairs(R2, R1, 1, F + (2 * c2) * K2, F + (2 * c2 + 1) * K2, K, tid, nthr);
                __syncthreads();
            } else {
                const float *in = f.gcoefs32 + (size_t)(anc - f.cap_real) * K3;
                fapply<false>(R1, in, F + (2 * c0) * K2, K, tid, nthr);
                __syncthreads();
                fapply<false>(R1 + K3, R1, F + (2 * c1) * K2, K, tid, nthr);
                __syncthreads();
                fapply<false>(R2, R1 + K3, F + (2 * c2) * K2, K, tid, nthr);
                __syncthreads();
            }
            src = R2;
        }
        for (int a = an + 1; a < n; a++) {
            const int sh = n - a - 1;
            const int c0 = (l0 >> sh) & 1, c1 = (l1 >> sh) & 1, c2 = (l2 >> sh) & 1;
            fapply<false>(R0, src, F + (2 * c0) * K2, K, tid, nthr);
            __syncthreads();
            fapply<false>(R0 + K3, R0, F + (2 * c1) * K2, K, tid, nthr);
            __syncthreads();
            fapply<false>(dst, R0 + K3, F + (2 * c2) * K2, K, tid, nthr);
            __syncthreads();
            src = dst;
            dst = dst == R1 ? R2 : R1;
        }
        // children of the parent block src: one-input steps; results in the other region
        for (int c0 = 0; c0 < 2; c0++)
            if (need_x >> c0 & 1) fapply<false>(R0 + c0 * K3, src, F + (2 * c0) * K2, K, tid, nthr);
        __syncthreads();
        for (int c01 = 0; c01 < 4; c01++)
            if (need_xy >> c01 & 1) fapply<false>(R0 + (2 + c01) * K3, R0 + (c01 & 1) * K3, F + (2 * (c01 >> 1)) * K2, K, tid, nthr);
        __syncthreads();
        for (int c = 0; c < 8; c++) {
            child[c] = dst + c * K3;
            if (need >> c & 1) fapply<false>(dst + c * K3, R0 + (2 + (c & 3)) * K3, F + (2 * (c >> 2)) * K2, K, tid, nthr);
        }
        __syncthreads();
    }
    for (int c = 0; c < 8; c++) {
        if (s_slot[c] < 0) continue;
        const int slot = gen_base + s_slot[c];
        if (slot >= f.cap_gen) {
            if (tid == 0) atomicOr(err, DE_POOL_FULL);
            continue;
        }
        const float *v = child[c];
        double *out = f.gcoefs + (size_t)slot * K3;
        float *out32 = f.gcoefs32 + (size_t)slot * K3;
        float *tc = f.gtc32 ? f.gtc32 + (size_t)slot * kTcGenFloats : nullptr;
        double s2 = 0.0;
        for (int e = tid; e < K3; e += nthr) {
            const float x = v[e];
            out32[e] = x;
            out[e] = (double)x;
            if (tc) tc_gen_store(tc, e, x);
            s2 += (double)x * (double)x;
        }
        for (int o = 16; o > 0; o >>= 1) s2 += __shfl_down_sync(0xffffffffu, s2, o);
        if ((tid & 31) == 0) red[tid >> 5] = s2;
        __syncthreads();
        if (tid == 0) {
            double t = 0.0;
            for (int w = 0; w < (nthr + 31) / 32; w++) t += red[w];
            double *nr = f.norms + (size_t)(f.cap_real + slot) * 8;
            nr[0] = sqrt(t);
            for (int cc = 1; cc < 8; cc++) nr[cc] = 0.0;
            f.idx[f.cap_real + slot] = make_int4(n + 1, 2 * l0 + (c & 1), 2 * l1 + ((c >> 1) & 1), 2 * l2 + (c >> 2));
        }
        __syncthreads();
    }
}

__global__ void k_to_float(const double *src, float *dst, size_t n) {
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) dst[i] = (float)src[i];
}

// FP64 node coefficients read straight from page-locked host memory (its
// device mapping), written as the device FP64 array and its FP32 copy in one
// pass; n_pairs pairs of doubles
__global__ void k_host_in(const double2 *__restrict__ src, double2 *__restrict__ dst, float2 *__restrict__ dst32, size_t n_pairs) {
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n_pairs; i += (size_t)gridDim.x * blockDim.x) {
        const double2 v = src[i];
        dst[i] = v;
        if (dst32) dst32[i] = make_float2((float)v.x, (float)v.y);
    }
}

__global__ void k_gather_norms_multi(const DevTree *gs, const int *work_tree, const int *work, int n, double *dst) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n * 8) return;
    const int w = i / 8;
    dst[i] = gs[work_tree[w]].norms[(size_t)work[w] * 8 + (i % 8)];
}

// device time stamp (PTX %globaltimer, nanoseconds)
__global__ void k_stamp(unsigned long long *t) {
    unsigned long long v;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(v));
    *t = v;
}

__global__ void k_copy_nodes(DevTree src, DevTree dst, const int *sid, const int *did, int n, int nc) {
    const int j = blockIdx.x;
    if (j >= n) return;
    const double *a = src.coefs + (size_t)sid[j] * nc;
    const int d = did ? did[j] : j;  // without did: row j
    double *b = dst.coefs + (size_t)d * nc;
    for (int e = threadIdx.x; e < nc; e += blockDim.x) b[e] = a[e];
    if (threadIdx.x < 8) dst.norms[(size_t)d * 8 + threadIdx.x] = src.norms[(size_t)sid[j] * 8 + threadIdx.x];
}

}  // namespace

void launch_copy_nodes(const DevTree &src, const DevTree &dst, const int *sid, const int *did, int n, int nc, cudaStream_t s) {
    if (n > 0) k_copy_nodes<<<n, 256, 0, s>>>(src, dst, sid, did, n, nc);
}

void launch_stamp(unsigned long long *t, cudaStream_t s) { k_stamp<<<1, 1, 0, s>>>(t); }

void launch_gather_norms(const DevTree *gs, const int *work_tree, const int *work, int n, double *dst, cudaStream_t s) {
    if (n <= 0) return;
    k_gather_norms_multi<<<(n * 8 + 255) / 256, 256, 0, s>>>(gs, work_tree, work, n, dst);
}

bool host_in_supported(const double *host, size_t n, const double **dev) {
    if (std::getenv("MWGPU_H2D_DMA") || n % 2 != 0 || ((uintptr_t)host & 15) != 0) return false;
    cudaPointerAttributes a{};
    if (cudaPointerGetAttributes(&a, host) != cudaSuccess) {
        cudaGetLastError();
        return false;
    }
    if (a.type != cudaMemoryTypeHost || a.devicePointer == nullptr || ((uintptr_t)a.devicePointer & 15) != 0) return false;
    *dev = (const double *)a.devicePointer;
    return true;
}

void launch_host_in(const double *src_dev, double *dst, float *dst32, size_t n, cudaStream_t s) {
    if (n == 0) return;
    k_host_in<<<4 * 152, 512, 0, s>>>((const double2 *)src_dev, (double2 *)dst, (float2 *)dst32, n / 2);
}

void launch_to_float(const double *src, float *dst, size_t n, cudaStream_t s) {
    if (n == 0) return;
    int blocks = (int)std::min<size_t>((n + 255) / 256, 152 * 16);
    k_to_float<<<blocks, 256, 0, s>>>(src, dst, n);
}

void launch_hash_build(const DevMRA &m, DevTree t, int first, int count, int *err, cudaStream_t s) {
    if (count <= 0) return;
    k_hash_build<<<(count + 255) / 256, 256, 0, s>>>(m, t, first, count, err);
}

void launch_gen_nodes(const DevMRA &m, DevTree f, const NodeKey *plist, int n_pend, int gen_base, int *err, cudaStream_t s, bool real_only,
                      bool fp32) {
    if (n_pend <= 0) return;
    if (fp32) {
        const size_t smem = sizeof(float) * (8 * (size_t)m.kp1_d + 4 * m.K * m.K);
        if (smem > 48 * 1024) cudaFuncSetAttribute(k_gen_nodes32, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        k_gen_nodes32<<<n_pend, 256, smem, s>>>(m, f, plist, n_pend, gen_base, err, real_only);
        return;
    }
    size_t smem = sizeof(double) * 8 * m.kp1_d;
    if (smem > 48 * 1024) cudaFuncSetAttribute(k_gen_nodes, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    k_gen_nodes<<<n_pend, 128, smem, s>>>(m, f, plist, n_pend, gen_base, err, real_only);
}

void launch_gen_family32(const DevMRA &m, DevTree f, const NodeKey *fam_keys, const int *fam_slots, int n_fam, const int *n_fam_dev, int gen_base,
                         bool real_only, int *err, cudaStream_t s) {
    if (n_fam <= 0) return;
    const size_t smem = sizeof(float) * (24 * (size_t)m.kp1_d + 4 * m.K * m.K);
    if (smem > 48 * 1024) cudaFuncSetAttribute(k_gen_family32, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    k_gen_family32<<<n_fam, 256, smem, s>>>(m, f, fam_keys, fam_slots, n_fam, n_fam_dev, gen_base, real_only, err);
}

// Families of the pending GenNode keys plist[0..n) on the device: the parent
// keys go into a table whose value is the pending index of the inserting key
// (the family's leader); leaders are numbered; every key takes its child slot.
__device__ inline bool parent_of(const DevMRA &m, const NodeKey &k, NodeKey &pk, int &c) {
    int n, l0, l1, l2;
    unpack_key(m, k, n, l0, l1, l2);
    c = (l0 & 1) | ((l1 & 1) << 1) | ((l2 & 1) << 2);
    return pack_key(m, n - 1, l0 >> 1, l1 >> 1, l2 >> 1, pk);
}

__global__ void k_fam_insert(DevMRA m, const NodeKey *plist, int n, NodeKey *fkeys, int *fvals, int fcap, int *err) {
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= n) return;
    NodeKey pk;
    int c;
    if (!parent_of(m, plist[p], pk, c)) {
        atomicOr(err, DE_RANGE);
        return;
    }
    bool full = false;
    hash_insert(fkeys, fvals, fcap, pk, p, &full);
    if (full) atomicOr(err, DE_HASH_FULL);
}

__global__ void k_fam_number(DevMRA m, const NodeKey *plist, int n, const NodeKey *fkeys, const int *fvals, int fcap, int *famid, NodeKey *fam_keys,
                             int *fam_count) {
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= n) return;
    NodeKey pk;
    int c;
    if (!parent_of(m, plist[p], pk, c)) return;
    if (hash_find(fkeys, fvals, fcap, pk) != p) return;
    const int fam = atomicAdd(fam_count, 1);
    famid[p] = fam;
    fam_keys[fam] = pk;
}

__global__ void k_fam_place(DevMRA m, const NodeKey *plist, int n, const NodeKey *fkeys, const int *fvals, int fcap, const int *famid, int *fam_slots,
                            int *err) {
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= n) return;
    NodeKey pk;
    int c;
    if (!parent_of(m, plist[p], pk, c)) return;
    const int leader = hash_find(fkeys, fvals, fcap, pk);
    if (leader < 0 || leader >= n) {
        atomicOr(err, DE_LOOKUP);
        return;
    }
    fam_slots[8 * (size_t)famid[leader] + c] = p;
}

void launch_gen_families(const DevMRA &m, const NodeKey *plist, int n, NodeKey *fkeys, int *fvals, int fcap, int *famid, NodeKey *fam_keys,
                         int *fam_slots, int *fam_count, int *err, cudaStream_t s) {
    if (n <= 0) return;
    const int b = (n + 255) / 256;
    k_fam_insert<<<b, 256, 0, s>>>(m, plist, n, fkeys, fvals, fcap, err);
    k_fam_number<<<b, 256, 0, s>>>(m, plist, n, fkeys, fvals, fcap, famid, fam_keys, fam_count);
    k_fam_place<<<b, 256, 0, s>>>(m, plist, n, fkeys, fvals, fcap, famid, fam_slots, err);
}

void launch_gen_insert(const DevMRA &m, DevTree f, const NodeKey *plist, int n_pend, int gen_base, int *err, cudaStream_t s) {
    if (n_pend <= 0) return;
    k_gen_insert<<<(n_pend + 255) / 256, 256, 0, s>>>(m, f, plist, n_pend, gen_base, err);
}

void launch_node_norms(const DevMRA &m, DevTree t, const int *nodes, int n, cudaStream_t s) {
    if (n <= 0) return;
    k_node_norms<<<n, 128, 0, s>>>(m, t, nodes, n);
}

void launch_mw_down(const DevMRA &m, DevTree t, const DevTree *ts, const int *ptree, const int *parents, int n, bool overwrite, cudaStream_t s,
                    bool fp32) {
    if (n <= 0) return;
    if (fp32) {
        const size_t sm = sizeof(float) * (16 * (size_t)m.kp1_d + 4 * m.K * m.K);
        if (sm > 48 * 1024) cudaFuncSetAttribute(k_mw_down32, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
        k_mw_down32<<<n, kTransformThreads, sm, s>>>(m, t, ts, ptree, parents, n, overwrite);
        return;
    }
    size_t smem = sizeof(double) * 16 * m.kp1_d;
    if (smem > 48 * 1024) cudaFuncSetAttribute(k_mw_down, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    k_mw_down<<<n, 256, smem, s>>>(m, t, ts, ptree, parents, n, overwrite);
}

void launch_project(const DevMRA &m, DevTree t, const int *nodes, int n, const double *gauss, int ng, const double *vc_map,
                    const double *roots, cudaStream_t s, const double *values) {
    if (n <= 0) return;
    const size_t smem = sizeof(double) * 16 * m.kp1_d;
    if (smem > 48 * 1024) cudaFuncSetAttribute(k_project, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    k_project<<<n, 256, smem, s>>>(m, t, nodes, n, gauss, ng, vc_map, roots, values);
}

void launch_combine(const DevMRA &m, bool mul, const DevTree *ins, const double *c, int n_in, DevTree out, const int *nodes, int n,
                    const double *cv_map, const double *vc_map, int *err, cudaStream_t s) {
    if (n <= 0) return;
    const size_t smem = sizeof(double) * 24 * m.kp1_d;
    auto kern = mul ? k_combine<true> : k_combine<false>;
    if (smem > 48 * 1024) cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    kern<<<n, 256, smem, s>>>(m, ins, c, n_in, out, nodes, n, cv_map, vc_map, err);
}

void launch_mw_up(const DevMRA &m, DevTree t, const DevTree *ts, const int *ptree, const int *parents, int n, cudaStream_t s, bool fp32) {
    if (n <= 0) return;
    if (fp32) {
        const size_t sm = sizeof(float) * (16 * (size_t)m.kp1_d + 4 * m.K * m.K);
        if (sm > 48 * 1024) cudaFuncSetAttribute(k_mw_up32, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
        k_mw_up32<<<n, kTransformThreads, sm, s>>>(m, t, ts, ptree, parents, n);
        return;
    }
    size_t smem = sizeof(double) * 16 * m.kp1_d;
    if (smem > 48 * 1024) cudaFuncSetAttribute(k_mw_up, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    k_mw_up<<<n, 256, smem, s>>>(m, t, ts, ptree, parents, n);
}

}  // namespace mwgpu
