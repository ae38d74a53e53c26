// Internal device-side structures of the mwgpu library (not part of the C-ABI).
//
// HBM layout
//   operator tables: one array of operator nodes for all terms; node = 4 K*K
//     blocks (T,C,B,A; column-major K x K) + 4 component norms; per
//     (term, depth) the offset of translation l = -L and L.
//   trees: node index (scale, l0, l1, l2) as int4, 8 K^3 doubles per real
//     node (compressed s+d form, component c at c*K^3, x fastest), 8 norms per
//     node; GenNodes (scaling-only nodes made by reconstruction) live in a
//     separate pool of K^3 doubles per node, ids >= capacity_real.
//   lookup: open-addressing hash keyed by (depth, translation offsets).
#pragma once

#include <cstdint>
#include <cuda_bf16.h>
#include <cuda_runtime.h>

namespace mwgpu {

constexpr int kMaxDepthRows = 30;   // ConvolutionCalculator band-size rows (MaxDepth)
constexpr double kMachineZero = 1.0e-14;
// Node key of the lookup tables: depth d and the three translation offsets
// from the world corner, t_i = l_i - corner_i 2^d (0 <= t_i < nbox_i 2^d):
// lo = t0 | t1 << 32, hi = t2 | d << 32.  Every node index the reference can
// form (depth <= 30 below the root scale, 32-bit translations) has a key; a
// slot with every bit set is empty.
struct __align__(16) NodeKey {
    unsigned long long lo, hi;
};
__host__ __device__ inline bool operator==(const NodeKey &a, const NodeKey &b) { return a.lo == b.lo && a.hi == b.hi; }
__host__ __device__ inline bool key_empty(const NodeKey &k) { return k.lo == ~0ull && k.hi == ~0ull; }
// chunk length of the mixed contraction: max(8, ceil(items / kChunkTarget))
constexpr long long kChunkTarget = 8 * 304;
// term-major ordering of the work items (k_order_terms): threads, most terms
constexpr int kOrderThreads = 256, kOrderMaxTerms = 256;
// learned-grid network: features, hidden width, parameter count
constexpr int kMlpFeatures = 8, kMlpHidden = 64;
constexpr int kMlpParams = kMlpHidden * kMlpFeatures + kMlpHidden + kMlpHidden * kMlpHidden + kMlpHidden + kMlpHidden + 1;

struct DevMRA {
    int K, kp1_d, root_scale, max_scale;
    int corner[3], nbox[3];
    double sf;
    const double *filt;  // [2 ops][4 filters][K*K] column-major; op 0 = compression, 1 = reconstruction
};

// one operator term at one depth, in the per-depth term order (descending
// band width): term index, translation range and node offset of its cache,
// band widths of the 4 components and their maximum
struct __align__(16) TermRow {
    int term, L0, off, bw_max;
    int wd[4];
};

struct DevOper {
    int n_terms, K;
    int max_rows;               // rows of per-term tables (= kMaxDepthRows + 1)
    const int *term_depth;      // [T]
    const int *dep_off;         // [T * max_rows] node offset of l = -L, -1 beyond term depth
    const int *dep_L;           // [T * max_rows]
    const double *blocks;       // [nodes * 4 * K * K]
    const double *norms;        // [nodes * 4]
    const int *bw;              // [T * max_rows * 5] band widths at the apply precision (-1 beyond)
    const int *band_size;       // [T * kMaxDepthRows * 64] ConvolutionCalculator band-size factors
    const int *band_max;        // [max_rows]
    const int *term_order;      // [max_rows * T] terms sorted by descending bw max at depth
    int n_band_max;
    const float *blocks32;      // FP32 copy of blocks (mixed form), each K x K block transposed
    const float *norm_max;      // [nodes] upper bound of the 4 component norms (FP32, rounded up)
    const float *norms32;       // [nodes * 4] norms rounded to FP32 (screening estimates)
    const TermRow *term_rows;   // [max_rows * T] term_order with the per-term tables of each depth
    // per depth d with band_max[d] = W >= 0: for every cell (a, b, c) in
    // [-W, W]^3 (a slowest) the largest per-term screening bound over the terms
    // (prod_d norm_max(l_d) * fm^3, FP32 rounded up); pair_bound_off[d] = -1: none
    const float *pair_bound;
    const int *pair_bound_off;  // [max_rows]
    // K = 8: per operator node (and a zero record after the last) the B
    // operands of the tensor-core contraction (k_tc.cu), TF32 hi and lo parts,
    // with the blocks outside the band zeroed; null otherwise
    const float *btc;
    // K = 8: stacked x-step forms of the pencil contraction (k_pencil.cu), per
    // (depth, term group, x slot); null otherwise
    const float *btc_stack;
    // K = 8: the y- and z-step operator fragments of the pencil contraction per
    // (depth, term row, l = -kPencilMaxL .. kPencilMaxL): 1024 floats each
    // (k_pencil.cu); null otherwise
    const float *pfrag;
    int n_nodes;
    // derivative operators (DerivativeCalculator::makeOperBand): the band runs
    // along band_dir only, band_dir_w wide; -1: the convolution band box
    int band_dir, band_dir_w;
};

struct DevTree {
    int n_real, cap_real;        // real nodes
    int n_gen, cap_gen;          // generated scaling-only nodes
    int4 *idx;                   // [cap_real + cap_gen] (scale, l0, l1, l2)
    double *coefs;               // [cap_real * 8 K^3]
    double *gcoefs;              // [cap_gen * K^3]
    double *norms;               // [(cap_real + cap_gen) * 8]
    int *child0;                 // [cap_real] first child id or -1
    float *coefs32;              // input trees: FP32 copy of coefs (mixed form)
    float *gcoefs32;             // input trees: FP32 copy of gcoefs
    float *tc32;                 // K = 8 input trees: TF32 hi / lo of every node in the tensor-core layout (k_tc.cu)
    float *gtc32;                // K = 8 input trees: the same for the scaling block of every GenNode
    NodeKey *hkeys;              // [hcap]
    int *hvals;                  // [hcap]
    int hcap;                    // power of two
};

__host__ __device__ inline bool pack_key(const DevMRA &m, int n, int l0, int l1, int l2, NodeKey &key) {
    const int d = n - m.root_scale;
    if (d < 0 || d > 30) return false;
    const int l[3] = {l0, l1, l2};
    unsigned long long t[3];
    for (int i = 0; i < 3; i++) {
        const long long v = (long long)l[i] - (long long)m.corner[i] * (1ll << d);
        if (v < 0 || v >= (long long)m.nbox[i] * (1ll << d) || v > 0xffffffffll) return false;
        t[i] = (unsigned long long)v;
    }
    key.lo = t[0] | t[1] << 32;
    key.hi = t[2] | (unsigned long long)d << 32;
    return true;
}

__host__ __device__ inline void unpack_key(const DevMRA &m, const NodeKey &key, int &n, int &l0, int &l1, int &l2) {
    const int d = (int)(key.hi >> 32);
    n = m.root_scale + d;
    l0 = (int)((long long)(key.lo & 0xffffffffull) + (long long)m.corner[0] * (1ll << d));
    l1 = (int)((long long)(key.lo >> 32) + (long long)m.corner[1] * (1ll << d));
    l2 = (int)((long long)(key.hi & 0xffffffffull) + (long long)m.corner[2] * (1ll << d));
}

__host__ __device__ inline uint32_t hash_slot(const NodeKey &key, int hcap) {
    // both words folded, then the 64-bit finaliser of MurmurHash3 (every key
    // bit reaches every slot bit)
    uint64_t h = key.lo ^ (key.hi * 0x9E3779B97F4A7C15ull);
    h ^= h >> 33;
    h *= 0xFF51AFD7ED558CCDull;
    h ^= h >> 33;
    h *= 0xC4CEB9FE1A85EC53ull;
    h ^= h >> 33;
    return (uint32_t)(h & (uint64_t)(hcap - 1));
}

__device__ inline int hash_find(const NodeKey *keys, const int *vals, int hcap, const NodeKey &key) {
    uint32_t s = hash_slot(key, hcap);
    for (int probe = 0; probe < hcap; probe++) {
        const NodeKey k = keys[s];
        if (k == key) return vals[s];
        if (key_empty(k)) return -1;
        s = (s + 1) & (hcap - 1);
    }
    return -1;
}

// 128-bit compare-and-swap of a global table slot (PTX atom.cas.b128, sm_90
// and later); returns the slot's previous content.
__device__ inline NodeKey key_cas(NodeKey *slot, const NodeKey &cmp, const NodeKey &val) {
    NodeKey old;
    asm volatile(
        "{\n\t.reg .b128 d, b, c;\n\tmov.b128 b, {%2, %3};\n\tmov.b128 c, {%4, %5};\n\t"
        "atom.global.cas.b128 d, [%6], b, c;\n\tmov.b128 {%0, %1}, d;\n}\n"
        : "=l"(old.lo), "=l"(old.hi)
        : "l"(cmp.lo), "l"(cmp.hi), "l"(val.lo), "l"(val.hi), "l"(slot)
        : "memory");
    return old;
}

// Inserts key; returns true if this call inserted it. Bounded probing.
__device__ inline bool hash_insert(NodeKey *keys, int *vals, int hcap, const NodeKey &key, int val, bool *full) {
    const NodeKey empty{~0ull, ~0ull};
    uint32_t s = hash_slot(key, hcap);
    for (int probe = 0; probe < hcap; probe++) {
        const NodeKey prev = key_cas(&keys[s], empty, key);
        if (key_empty(prev)) { vals[s] = val; return true; }
        if (prev == key) return false;
        s = (s + 1) & (hcap - 1);
    }
    *full = true;
    return false;
}

// error flags written by kernels (host reads them after each phase)
enum DevError { DE_LOOKUP = 1, DE_HASH_FULL = 2, DE_POOL_FULL = 4, DE_RANGE = 8, DE_TIMEOUT = 16 };

// One (output node, input node, term) triple with its contracted (ft, gt)
// components: bit ft*8+gt of mask.  flags bit 0: the mask equals the
// structural set (every component the band and zero-norm rules allow), so
// the components may be summed blockwise.
struct WorkItem {
    unsigned long long mask;   // contracted (ft, gt) components, bit 8 ft + gt
    unsigned long long sched;  // block schedule: valid inputs of every stage output (see k_worklist.cu)
    int fid;
    short term;
    short tl[3];
    short flags;               // bit 0: block schedule
    short pad;
};

struct LevelStats {
    unsigned long long node_terms;   // (g, f, term) triples with >= 1 contracted component
    unsigned long long components;   // contracted (g, f, term, ft, gt) components
    unsigned long long band_nodes;   // (g, f) pairs visited
    unsigned long long gen_nodes;    // GenNodes created
};

// One unit of the pencil contraction (k_pencil.cu): output node g (work entry
// wi), pencil (l_y, l_z), and a group of up to kPencilGroup operator terms: the
// terms of the depth in descending band width that reach the pencil
// (w >= max(|l_y|, |l_z|)), from term row q on.  Slot b of the x window is
// l_x = 0 (b = 0), -k (b = 2k - 1), +k (b = 2k), |l_x| <= xw; ntk[k] of the
// unit's terms reach |l_x| = k.  The host fills the topology part, the device
// the f nodes (k_pencil_units).  The pencil path takes the terms whose band
// width at the depth is at most kPencilMaxW (then every |l_d| <= that); the
// wider terms stay with the item kernel.  The kernel stages a unit's f nodes
// slot by slot through a ring of kPencilRing buffers (shared memory holds
// three 32 KB nodes next to the other buffers).
constexpr int kPencilMaxW = 4;
constexpr int kPencilMaxL = kPencilMaxW;
// two configurations of the pencil path: the terms of band width <= 1 (levels
// built per call: few units, cheap to make on the host) or <= kPencilMaxW
// (plans: units made once)
constexpr int kPencilCfgs = 2;
constexpr int kPencilCfgW[kPencilCfgs] = {1, kPencilMaxW};
constexpr int kPencilSlots = 2 * kPencilMaxL + 1;
constexpr int kPencilRing = 3;
// operator fragment records per (depth, term row): l = -kPencilMaxL .. kPencilMaxL
constexpr int kPencilFragL = 2 * kPencilMaxL + 1;
struct PencilUnit {
    long long form[kPencilSlots];   // float offsets of the stacked x-step forms of the slots
    int fid[kPencilSlots];          // f nodes of the slots (-1: none, outside the world or zero norm)
    int task;                       // partial slot of the task (work entry, l_z)
    int wi;                         // work entry of g
    int flags;                      // bit b: fid[b] is a GenNode
    short depth, q, nt, xw;         // q: term row of the group's first term at the depth
    short ntk[kPencilMaxL + 1];     // terms reaching |l_x| = k
    short nform[kPencilSlots];      // terms of each slot's stacked form (its layout)
    short wt0, wt1;                 // terms whose products tile 0 / tile 1 of D hold
    short pflags;                   // bit 0: first group of its pencil, bit 1: last (a pencil's groups are consecutive)
    signed char ly, lz;
};

// kernel launchers (k_apply.cu / k_tree.cu)
void launch_band_missing(const DevMRA &m, const DevOper &op, const DevTree &f, const DevTree &g, const int *work, int n_work,
                         NodeKey *pkeys, int *pvals, int phcap, NodeKey *plist, int *pcount, int pcap, int *err, cudaStream_t s);
// real_only: reconstruct from the nearest real ancestor even where a GenNode
// ancestor exists (GenNodes that are rewritten by the same launch)
// GenNodes of the pending keys plist[0..n_pend) into slots gen_base + p
// (fp32: FP32 products, the GenNodes of the mixed form)
void launch_gen_nodes(const DevMRA &m, DevTree f, const NodeKey *plist, int n_pend, int gen_base, int *err, cudaStream_t s,
                      bool real_only = false, bool fp32 = false);
// Mixed-form GenNodes grouped by parent (one CTA per parent, the requested
// children fam_slots[8 q + c] >= 0; values bit-identical to launch_gen_nodes)
// (n_fam_dev: the family count on the device, n_fam an upper bound; slots
// gen_base + fam_slots[...]; real_only as for launch_gen_nodes)
void launch_gen_family32(const DevMRA &m, DevTree f, const NodeKey *fam_keys, const int *fam_slots, int n_fam, const int *n_fam_dev, int gen_base,
                         bool real_only, int *err, cudaStream_t s);
// families of the pending keys plist[0..n) on the device (fkeys: a table of
// fcap >= 2 n slots, all bits set; fam_slots: 8 n entries of -1; fam_count 0)
void launch_gen_families(const DevMRA &m, const NodeKey *plist, int n, NodeKey *fkeys, int *fvals, int fcap, int *famid, NodeKey *fam_keys,
                         int *fam_slots, int *fam_count, int *err, cudaStream_t s);
void launch_gen_insert(const DevMRA &m, DevTree f, const NodeKey *plist, int n_pend, int gen_base, int *err, cudaStream_t s);
// DerivativeCalculator::calcNode for the work entries (output leaves): band along
// op.band_dir, 1D application of term 0 with the identity elsewhere, divided by
// sf^order; FP64
void launch_deriv(const DevMRA &m, const DevOper &op, const DevTree &f, DevTree g, const int *work, int n_work, int order, LevelStats *stats,
                  int *err, cudaStream_t s);
void launch_contract_fp64(const DevMRA &m, const DevOper &op, const DevTree &f, DevTree g, const int *work, int n_work,
                          double gthr, LevelStats *stats, int *err, cudaStream_t s, const int *nw_dev = nullptr,
                          const double *gthr_dev = nullptr, const double *gthr_node = nullptr);
bool mixed_supported(int K);
void launch_pairs_count(const DevMRA &m, const DevOper &op, const DevTree *fs, const DevTree *gs, const int *work_tree, const int *work,
                        const long long *pair_off, int n_work, long long n_pairs, const double *gthrs, int *counts, unsigned long long *ncomp,
                        unsigned long long *nband, int *err, cudaStream_t s, const long long *np_dev = nullptr, const int *nw_dev = nullptr,
                        const double *gthr_node = nullptr);
// FILL: counts are the COUNT pass's per-pair item counts (pairs without items
// are skipped; may be null)
void launch_pairs_fill(const DevMRA &m, const DevOper &op, const DevTree *fs, const DevTree *gs, const int *work_tree, const int *work,
                       const long long *pair_off, int n_work, long long n_pairs, const double *gthrs, const int *counts, const long long *item_off,
                       WorkItem *items, long long items_cap, int *err, cudaStream_t s, const long long *np_dev = nullptr, const int *nw_dev = nullptr,
                       const double *gthr_node = nullptr);
// chunking of the work list on the device (graph-capturable levels); per <= 0:
// the chunk length follows from the item count on the device (kChunkTarget)
void launch_chunk_count(const long long *g_off, int n_work, long long per, int *counts, cudaStream_t s, const int *nw_dev = nullptr);
void launch_chunk_fill(const long long *g_off, const long long *c_off, int n_work, long long per, int4 *chunks, int *chunk_begin, int cap,
                       int *n_chunks, int *err, cudaStream_t s, const int *nw_dev = nullptr);
// tc_counter: a device int for the tensor-core kernel's chunk counter (order 7; null: CUDA cores only)
void launch_items(const DevMRA &m, const DevOper &op, const DevTree *fs, const DevTree *gs, const int *work_tree, const int *work,
                  const int4 *chunks, int n_chunks, const WorkItem *items, double *partial, int *err, const int *n_chunks_dev, int *counter,
                  int *tc_counter, cudaStream_t s);
// pen_begin / pen_partial: task sums of the pencil contraction per work entry (optional)
void launch_reduce_chunks(const DevMRA &m, const DevTree *gs, const int *work_tree, const int *work, int n_work, const int *chunk_begin,
                          const double *partial, cudaStream_t s, const int *nw_dev = nullptr, const int *pen_begin = nullptr,
                          const double *pen_partial = nullptr);
// CTAs of the contraction kernel of order K resident on one SM (0 if unknown)
int contract_items_resident(int K);
long long scan_blocks(long long n);
void launch_scan(const int *in, long long *out, long long n, long long *block_sums, long long *total, cudaStream_t s);
// cap: the capacity of the item buffer the offsets index (offsets beyond it are clamped)
void launch_gather_goff(const long long *item_off, const long long *pair_off, int n_work, long long *g_off, cudaStream_t s, const int *nw_dev = nullptr,
                        long long cap = 0x7fffffffffffffffLL);
// term-major order of each output node's items (in -> out, same ranges); only
// for operators of at most kOrderMaxTerms terms
bool term_order_supported(int n_terms);
void launch_order_terms(const long long *g_off, int n_work, const WorkItem *in, WorkItem *out, int n_terms, int *err, cudaStream_t s,
                        const int *nw_dev = nullptr);
void launch_contract_items(const DevMRA &m, const DevOper &op, const DevTree *fs, const DevTree *gs, const int *work_tree, const int *work,
                           int n_work, const int4 *chunks, int n_chunks, const int *chunk_begin, const WorkItem *items, double *partial, int *err,
                           int *tc_counter, cudaStream_t s);
// copies coefficients and norms of nodes sid[j] of src to nodes did[j] of dst
void launch_copy_nodes(const DevTree &src, const DevTree &dst, const int *sid, const int *did, int n, int nc, cudaStream_t s);
// writes the device's nanosecond timer (usable inside CUDA graphs)
void launch_stamp(unsigned long long *t, cudaStream_t s);
void launch_gather_norms(const DevTree *gs, const int *work_tree, const int *work, int n, double *dst, cudaStream_t s);
void launch_node_norms(const DevMRA &m, DevTree t, const int *nodes, int n, cudaStream_t s);
// fp32: FP32 filter products (the mixed form), coefficients stay FP64
void launch_mw_down(const DevMRA &m, DevTree t, const DevTree *ts, const int *ptree, const int *parents, int n, bool overwrite, cudaStream_t s,
                    bool fp32 = false);
void launch_mw_up(const DevMRA &m, DevTree t, const DevTree *ts, const int *ptree, const int *parents, int n, cudaStream_t s, bool fp32 = false);
void launch_to_float(const double *src, float *dst, size_t n, cudaStream_t s);
// host arrays in page-locked memory that the device can read: their device
// address (*dev) for launch_host_in (MWGPU_H2D_DMA=1: copy engine instead)
bool host_in_supported(const double *host, size_t n, const double **dev);
// n doubles from a device-mapped host array into dst and its FP32 copy dst32 (may be null)
void launch_host_in(const double *src_dev, double *dst, float *dst32, size_t n, cudaStream_t s);
// AdditionCalculator / MultiplicationCalculator::calcNode for the given output
// nodes over the input trees ins[0..n_in) (device array) with factors c (device)
void launch_combine(const DevMRA &m, bool mul, const DevTree *ins, const double *c, int n_in, DevTree out, const int *nodes, int n,
                    const double *cv_map, const double *vc_map, int *err, cudaStream_t s);
// ProjectionCalculator::calcNode of a Gaussian sum (gauss [ng][5]: coefficient,
// exponent, position) for the given nodes; vc_map (K x K) and roots (K) of the basis
// peak-rate probes of the FP64 pipes (k_rates.cu)
void launch_rate_dfma(double *out, int blocks, int iters, cudaStream_t s);
void launch_rate_dmma(double *out, int blocks, int iters, cudaStream_t s);
double rate_dfma_flops(int blocks, int iters);
double rate_dmma_flops(int blocks, int iters);
int rate_threads();
// values: the function at the children's quadrature points (8 (k+1)^3 per node), or null for the Gaussians
void launch_project(const DevMRA &m, DevTree t, const int *nodes, int n, const double *gauss, int ng, const double *vc_map,
                    const double *roots, cudaStream_t s, const double *values = nullptr);
void launch_hash_build(const DevMRA &m, DevTree t, int first, int count, int *err, cudaStream_t s);

// learned grid (k_mlp.cu)
size_t mlp_train_smem();
void launch_mlp_infer(const float *X, int n, const __nv_bfloat16 *wb, float *prob, cudaStream_t s);
void launch_mlp_train_tile(const float *X, const float *Y, const int *idx, int base, int count, const __nv_bfloat16 *wb, float pos_weight,
                           float inv_wsum, float *partial, float *loss_partial, cudaStream_t s);
void launch_mlp_reduce(const float *partial, const float *loss_partial, int tiles, float *grad, float *loss, cudaStream_t s);
void launch_mlp_adam(float *master, float *m1, float *m2, const float *grad, __nv_bfloat16 *wb, float lr, float beta1, float beta2, float eps,
                     float c1, float c2, cudaStream_t s);
void launch_mlp_to_bf16(const float *src, __nv_bfloat16 *dst, int n, cudaStream_t s);
void launch_mlp_features(const DevMRA &m, const DevTree &f, const int4 *nodes, int n, const int *band_w, const int *terms, int rows, double ftot,
                         float *X, cudaStream_t s);

// tensor-core contraction of order K = 8 (k_tc.cu)
constexpr int kTcNodeFloats = 8192;   // tc32 per real node: hi then lo, 4096 floats each
constexpr int kTcGenFloats = 1024;    // gtc32 per GenNode: scaling block, hi then lo
constexpr int kTcFormFloats = 3328;   // btc per operator node
bool tc_supported(int K);
// element e = x + 8 (y + 8 z) of a GenNode's scaling block into its gtc32 record (hi, lo)
__device__ inline void tc_gen_store(float *rec, int e, float v) {
    const int x = e & 7, yz = e >> 3;
    const int o = (x >> 2) * 256 + (yz >> 3) * 32 + (yz & 7) * 4 + (x & 3);
    unsigned h;
    asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(h) : "f"(v));
    const float hi = __uint_as_float(h);
    rec[o] = hi;
    rec[512 + o] = v - hi;
}
// layout of real nodes [first, first + n) of an input tree from its FP64 coefficients
void launch_tc_tree_layout(const DevTree &t, int first, int n, cudaStream_t s);
// operator forms: node_info[j] = (term, depth, l) of operator node j; writes n_nodes + 1 records
void launch_tc_oper_forms(const DevOper &op, const int4 *node_info, int n_nodes, float *forms, cudaStream_t s);
// chunk types: .w = 1 where every item of the chunk is a block-schedule item
void launch_chunk_types(int4 *chunks, int n_chunks, const int *n_chunks_dev, const WorkItem *items, cudaStream_t s);
// contraction of the type-1 chunks on the tensor cores (persistent; counter zeroed here)
void launch_contract_tc(const DevMRA &m, const DevOper &op, const DevTree *fs, const DevTree *gs, const int *work_tree, const int *work,
                        const int4 *chunks, int n_chunks, const int *n_chunks_dev, const WorkItem *items, double *partial, int *err,
                        int *counter, cudaStream_t s);

// pencil contraction (k_pencil.cu)
constexpr int kPencilGroup = 5;   // operator terms per tensor-core product (24 columns each)
bool pencil_supported(int K);
// stacked form jobs; forms get 128 pad16(24 nt) bytes each
struct PencilFormJob {
    int depth, q, lx, nt;   // q: term row of the group's first term
    long long off;
};
void launch_stack_forms(const DevOper &op, const void *jobs, int n_jobs, float *forms, cudaStream_t s);
// the pencil contraction's y / z operator fragments (op.pfrag layout): rows x T x kPencilFragL records
constexpr int kPencilFragFloats = 1024;
void launch_pencil_frags(const DevOper &op, int rows, float *frags, cudaStream_t s);
void launch_pencil_units(const DevMRA &m, const DevTree *fs, const DevTree *gs, const int *work_tree, const int *work, void *units, int n_units,
                         int *err, cudaStream_t s);
// per work entry the number of its items whose term is wider than kPencilMaxW
// at the entry's depth (those the item kernel keeps), and their compaction
// (maxw: the widest band the pencil kernel takes, kPencilCfgW of the configuration)
void launch_keep_items(const DevMRA &m, const DevOper &op, const DevTree *gs, const int *work_tree, const int *work, const long long *g_off,
                       int n_work, const WorkItem *in, int *keep, cudaStream_t s, int maxw, const int *nw_dev = nullptr);
void launch_keep_fill(const DevMRA &m, const DevOper &op, const DevTree *gs, const int *work_tree, const int *work, const long long *g_off,
                      const long long *k_off, int n_work, const WorkItem *in, WorkItem *out, cudaStream_t s, int maxw, const int *nw_dev = nullptr);
// persistent; counter: a device int (zeroed here); pen_partial: 8 K^3 doubles per task;
// consumer_warps: 8 or 16 (the CTA shape; kPencilWarpsDefault where nothing was tuned)
constexpr int kPencilWarpsDefault = 8;
// the CTA shape's register split fits the registers the kernel is launched with
bool pencil_shape_ok(int consumer_warps);
void launch_pencil(const DevOper &op, const DevTree *fs, const int *work_tree, const void *units, const int *task_unit, int n_tasks,
                   double *pen_partial, int *err, int *counter, cudaStream_t s, int consumer_warps = kPencilWarpsDefault);

// judged adaptive apply (k_judged.cu)
void launch_keep_counts(const int *flags, int begin, int n, int *cnt, cudaStream_t s);
void launch_compact(const int *flags, int begin, int n, const long long *koff, int *work, int *n_work, cudaStream_t s);
void launch_cells(const int *work, const int *n_work, int cap, const int *cells, int *cnt, cudaStream_t s);
void launch_threshold(const double *sq, double prec, int n_terms, double *gthr, cudaStream_t s);
void launch_level_norm(const DevTree &g, const int *work, const int *n_work, int first_level, double *state, double *sq_level,
                       const long long *g_off, unsigned long long *node_terms, cudaStream_t s);
void launch_judge(const DevMRA &m, const DevTree &g, const int *work, const int *n_work, int cap, const double *state, double prec, int abs_prec,
                  const double *scale_fac, int max_scale, int *flags, int level, int *first_miss, cudaStream_t s);

}  // namespace mwgpu
