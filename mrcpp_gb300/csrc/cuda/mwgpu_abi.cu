// C-ABI implementation (include/mwgpu.h): device memory, uploads, per-level
// operator application and whole-tree transforms.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdlib>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <mutex>
#include <string>
#include <type_traits>
#include <vector>

#include "../../../include/mwgpu.h"
#include "mwgpu_internal.cuh"

using namespace mwgpu;

namespace {
thread_local std::string g_init_error;
constexpr double kMachinePrec = 1.0e-15;
}  // namespace

struct mwgpu_ctx {
    int device = 0;
    int precision = MWGPU_PREC_FP64;
    cudaStream_t stream = nullptr;
    cudaEvent_t ev0 = nullptr, ev1 = nullptr, ev2 = nullptr;
    std::string err;
    int *d_err = nullptr;
    LevelStats *d_stats = nullptr;
    int *d_work = nullptr;
    int work_cap = 0;
    // pending GenNode set
    uint64_t *d_pkeys = nullptr;
    int *d_pvals = nullptr;
    int phcap = 0;
    uint64_t *d_plist = nullptr;
    int pcap = 0;
    int *d_pcount = nullptr;
    int *d_list = nullptr;  // parent lists for transforms
    int list_cap = 0;
    cudaEvent_t marks[16] = {};
    // work list of the mixed form
    WorkItem *d_items = nullptr;
    long long items_cap = 0;
    long long *d_pair_off = nullptr, pair_off_cap = 0;
    int *d_pcounts = nullptr;
    long long pcounts_cap = 0;
    long long *d_item_off = nullptr, item_off_cap = 0;
    long long *d_scan = nullptr, scan_cap = 0;
    long long *d_goff = nullptr, goff_cap = 0;
    int4 *d_chunks = nullptr;
    int *d_chunk_begin = nullptr;
    int chunks_cap = 0;
    double *d_partial = nullptr;
    size_t partial_cap = 0;  // doubles
    unsigned long long launches = 0;
    void *d_scrub = nullptr;
    size_t scrub_bytes = 0;
};

struct mwgpu_oper {
    DevMRA mra{};
    double *d_filt = nullptr;
    DevOper op{};
    std::vector<void *> allocs;
    int n_rows = 0;
    std::vector<int> widths;    // [T * n_rows * 5]
    std::vector<int> band_max;  // [n_rows]
};

struct mwgpu_tree {
    DevMRA mra{};
    double *d_filt = nullptr;
    DevTree t{};
    std::vector<int4> h_idx;
    std::vector<int> h_child0;
    bool is_input = false;
};

#define MW_CK(call)                                                                                 \
    do {                                                                                            \
        cudaError_t e_ = (call);                                                                    \
        if (e_ != cudaSuccess) {                                                                    \
            ctx->err = std::string(#call) + ": " + cudaGetErrorString(e_);                          \
            return (e_ == cudaErrorMemoryAllocation) ? MWGPU_ERR_OOM : MWGPU_ERR_DEVICE;            \
        }                                                                                           \
    } while (0)

#define MW_ARG(cond, msg)                     \
    do {                                      \
        if (!(cond)) {                        \
            ctx->err = msg;                   \
            return MWGPU_ERR_BAD_ARG;         \
        }                                     \
    } while (0)

namespace {

mwgpu_status make_mra(mwgpu_ctx *ctx, const mwgpu_mra_desc *d, DevMRA &m, double **filt) {
    MW_ARG(d && d->filters, "null MRA descriptor");
    MW_ARG(d->order >= 0 && d->order < 32, "invalid order");
    m.K = d->order + 1;
    m.kp1_d = m.K * m.K * m.K;
    m.root_scale = d->root_scale;
    m.max_scale = d->max_scale;
    for (int i = 0; i < 3; i++) {
        m.corner[i] = d->corner[i];
        m.nbox[i] = d->nbox[i];
        MW_ARG(d->nbox[i] > 0, "invalid box count");
    }
    m.sf = d->sf;
    size_t bytes = sizeof(double) * 8 * m.K * m.K;
    MW_CK(cudaMalloc(filt, bytes));
    MW_CK(cudaMemcpy(*filt, d->filters, bytes, cudaMemcpyHostToDevice));
    m.filt = *filt;
    return MWGPU_OK;
}

template <class T> mwgpu_status dev_alloc(mwgpu_ctx *ctx, T **p, size_t n) {
    *p = nullptr;
    if (n == 0) n = 1;
    MW_CK(cudaMalloc((void **)p, sizeof(T) * n));
    return MWGPU_OK;
}

int next_pow2(long long x) {
    int p = 1;
    while (p < x) p <<= 1;
    return p;
}

// (re)allocates the hash of tree t for `entries` entries and reinserts all nodes.
mwgpu_status rebuild_hash(mwgpu_ctx *ctx, mwgpu_tree *tr, long long entries) {
    DevTree &t = tr->t;
    int hcap = next_pow2(std::max<long long>(1024, 2 * entries + 16));
    if (hcap != t.hcap) {
        if (t.hkeys) cudaFree(t.hkeys);
        if (t.hvals) cudaFree(t.hvals);
        t.hkeys = nullptr;
        t.hvals = nullptr;
        if (auto s = dev_alloc(ctx, &t.hkeys, hcap)) return s;
        if (auto s = dev_alloc(ctx, &t.hvals, hcap)) return s;
        t.hcap = hcap;
    }
    MW_CK(cudaMemsetAsync(t.hkeys, 0xFF, sizeof(uint64_t) * hcap, ctx->stream));
    MW_CK(cudaMemsetAsync(ctx->d_err, 0, sizeof(int), ctx->stream));
    launch_hash_build(tr->mra, t, 0, t.n_real, ctx->d_err, ctx->stream);
    ctx->launches += t.n_real > 0;
    if (t.n_gen > 0) launch_hash_build(tr->mra, t, t.cap_real, t.n_gen, ctx->d_err, ctx->stream);
    ctx->launches += t.n_gen > 0;
    int herr = 0;
    MW_CK(cudaMemcpyAsync(&herr, ctx->d_err, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
    MW_CK(cudaStreamSynchronize(ctx->stream));
    if (herr) {
        ctx->err = "node index outside the lookup range or lookup table full (error " + std::to_string(herr) + ")";
        return MWGPU_ERR_BAD_ARG;
    }
    return MWGPU_OK;
}

// grows the real-node arrays of an output tree to hold `need` nodes
mwgpu_status grow_real(mwgpu_ctx *ctx, mwgpu_tree *tr, int need) {
    DevTree &t = tr->t;
    if (need <= t.cap_real) return MWGPU_OK;
    int cap = std::max(need, t.cap_real * 2);
    const size_t nc = 8 * (size_t)tr->mra.kp1_d;
    int4 *idx;
    double *coefs, *norms;
    int *child0;
    if (auto s = dev_alloc(ctx, &idx, cap)) return s;
    if (auto s = dev_alloc(ctx, &coefs, (size_t)cap * nc)) return s;
    if (auto s = dev_alloc(ctx, &norms, (size_t)cap * 8)) return s;
    if (auto s = dev_alloc(ctx, &child0, cap)) return s;
    MW_CK(cudaMemsetAsync(coefs, 0, sizeof(double) * cap * nc, ctx->stream));
    if (t.n_real > 0) {
        MW_CK(cudaMemcpyAsync(idx, t.idx, sizeof(int4) * t.n_real, cudaMemcpyDeviceToDevice, ctx->stream));
        MW_CK(cudaMemcpyAsync(coefs, t.coefs, sizeof(double) * t.n_real * nc, cudaMemcpyDeviceToDevice, ctx->stream));
        MW_CK(cudaMemcpyAsync(norms, t.norms, sizeof(double) * t.n_real * 8, cudaMemcpyDeviceToDevice, ctx->stream));
        MW_CK(cudaMemcpyAsync(child0, t.child0, sizeof(int) * t.n_real, cudaMemcpyDeviceToDevice, ctx->stream));
    }
    MW_CK(cudaStreamSynchronize(ctx->stream));
    cudaFree(t.idx);
    cudaFree(t.coefs);
    cudaFree(t.norms);
    cudaFree(t.child0);
    t.idx = idx;
    t.coefs = coefs;
    t.norms = norms;
    t.child0 = child0;
    t.cap_real = cap;
    return MWGPU_OK;
}

// grows the GenNode pool of an input tree (ids cap_real + j)
mwgpu_status grow_gen(mwgpu_ctx *ctx, mwgpu_tree *tr, int need) {
    DevTree &t = tr->t;
    if (need <= t.cap_gen) return MWGPU_OK;
    int cap = std::max(need, std::max(1024, t.cap_gen * 2));
    const size_t K3 = tr->mra.kp1_d;
    int tot = t.cap_real + cap;
    int4 *idx;
    double *g, *norms;
    float *g32;
    if (auto s = dev_alloc(ctx, &idx, tot)) return s;
    if (auto s = dev_alloc(ctx, &norms, (size_t)tot * 8)) return s;
    if (auto s = dev_alloc(ctx, &g, (size_t)cap * K3)) return s;
    if (auto s = dev_alloc(ctx, &g32, (size_t)cap * K3)) return s;
    MW_CK(cudaMemcpyAsync(idx, t.idx, sizeof(int4) * (t.cap_real + t.n_gen), cudaMemcpyDeviceToDevice, ctx->stream));
    MW_CK(cudaMemcpyAsync(norms, t.norms, sizeof(double) * 8 * (t.cap_real + t.n_gen), cudaMemcpyDeviceToDevice, ctx->stream));
    if (t.n_gen > 0) {
        MW_CK(cudaMemcpyAsync(g, t.gcoefs, sizeof(double) * K3 * t.n_gen, cudaMemcpyDeviceToDevice, ctx->stream));
        MW_CK(cudaMemcpyAsync(g32, t.gcoefs32, sizeof(float) * K3 * t.n_gen, cudaMemcpyDeviceToDevice, ctx->stream));
    }
    MW_CK(cudaStreamSynchronize(ctx->stream));
    cudaFree(t.idx);
    cudaFree(t.norms);
    if (t.gcoefs) cudaFree(t.gcoefs);
    if (t.gcoefs32) cudaFree(t.gcoefs32);
    t.idx = idx;
    t.norms = norms;
    t.gcoefs = g;
    t.gcoefs32 = g32;
    t.cap_gen = cap;
    return MWGPU_OK;
}

mwgpu_status ensure_work(mwgpu_ctx *ctx, int n) {
    if (n <= ctx->work_cap) return MWGPU_OK;
    if (ctx->d_work) cudaFree(ctx->d_work);
    ctx->work_cap = std::max(n, 2 * ctx->work_cap);
    return dev_alloc(ctx, &ctx->d_work, ctx->work_cap);
}

mwgpu_status ensure_pending(mwgpu_ctx *ctx, int phcap, int pcap) {
    if (phcap > ctx->phcap) {
        if (ctx->d_pkeys) cudaFree(ctx->d_pkeys);
        if (ctx->d_pvals) cudaFree(ctx->d_pvals);
        if (auto s = dev_alloc(ctx, &ctx->d_pkeys, phcap)) return s;
        if (auto s = dev_alloc(ctx, &ctx->d_pvals, phcap)) return s;
        ctx->phcap = phcap;
    }
    if (pcap > ctx->pcap) {
        if (ctx->d_plist) cudaFree(ctx->d_plist);
        if (auto s = dev_alloc(ctx, &ctx->d_plist, pcap)) return s;
        ctx->pcap = pcap;
    }
    return MWGPU_OK;
}

mwgpu_status check_err(mwgpu_ctx *ctx, const char *phase) {
    int herr = 0;
    MW_CK(cudaMemcpyAsync(&herr, ctx->d_err, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
    MW_CK(cudaStreamSynchronize(ctx->stream));
    if (herr) {
        ctx->err = std::string(phase) + ": device error flags " + std::to_string(herr);
        return MWGPU_ERR_INTERNAL;
    }
    return MWGPU_OK;
}

void free_tree(mwgpu_tree *tr);

// grows a device buffer of T to at least n elements (contents not kept)
template <class T> mwgpu_status grow_buf(mwgpu_ctx *ctx, T **p, long long *cap, long long n) {
    if (n <= *cap) return MWGPU_OK;
    if (*p) cudaFree(*p);
    *p = nullptr;
    *cap = std::max(n, 2 * *cap);
    return dev_alloc(ctx, p, (size_t)*cap);
}

// Mixed form: work list (pair counts, scan, fill) then the contraction over
// chunks of items and the per-node reduction.  node_terms is returned in *hs.
mwgpu_status run_mixed(mwgpu_ctx *ctx, const mwgpu_oper *o, mwgpu_tree *inp, mwgpu_tree *out, const int *d_work, const int *node_ix, int n,
                       double gthr, LevelStats *hs) {
    // (g, band cell) pairs: the band boxes of makeOperBand, clipped to the world
    std::vector<long long> poff(n + 1, 0);
    const DevMRA &m = o->mra;
    for (int wi = 0; wi < n; wi++) {
        const int4 gx = out->h_idx[node_ix[wi]];
        const int depth = gx.x - m.root_scale;
        long long cells = 0;
        if (depth >= 0 && depth < o->op.n_band_max && depth < kMaxDepthRows && o->band_max[depth] >= 0) {
            const int w = o->band_max[depth];
            const int gl[3] = {gx.y, gx.z, gx.w};
            cells = 1;
            for (int d = 0; d < 3; d++) {
                long long nboxes = (long long)m.nbox[d] << depth, c = (long long)m.corner[d] << depth;
                long long s0 = std::max<long long>(gl[d] - w, c), e0 = std::min<long long>(gl[d] + w, c + nboxes - 1);
                cells *= std::max<long long>(0, e0 - s0 + 1);
            }
        }
        poff[wi + 1] = poff[wi] + cells;
    }
    const long long np = poff[n];
    if (auto s = grow_buf(ctx, &ctx->d_pair_off, &ctx->pair_off_cap, n + 1)) return s;
    if (auto s = grow_buf(ctx, &ctx->d_pcounts, &ctx->pcounts_cap, np + 1)) return s;
    if (auto s = grow_buf(ctx, &ctx->d_item_off, &ctx->item_off_cap, np + 1)) return s;
    if (auto s = grow_buf(ctx, &ctx->d_scan, &ctx->scan_cap, scan_blocks(np + 1) + 2)) return s;
    if (auto s = grow_buf(ctx, &ctx->d_goff, &ctx->goff_cap, n + 1)) return s;
    MW_CK(cudaMemcpyAsync(ctx->d_pair_off, poff.data(), sizeof(long long) * (n + 1), cudaMemcpyHostToDevice, ctx->stream));
    LevelStats *dst = ctx->d_stats;
    launch_pairs_count(m, o->op, inp->t, out->t, d_work, ctx->d_pair_off, n, np, gthr, ctx->d_pcounts, &dst->components, &dst->band_nodes,
                       ctx->d_err, ctx->stream);
    long long *d_total = ctx->d_scan + (ctx->scan_cap - 1);
    launch_scan(ctx->d_pcounts, ctx->d_item_off, np, ctx->d_scan, d_total, ctx->stream);
    launch_gather_goff(ctx->d_item_off, ctx->d_pair_off, n, ctx->d_goff, ctx->stream);
    ctx->launches += 5;
    std::vector<long long> offs(n + 1);
    MW_CK(cudaMemcpyAsync(offs.data(), ctx->d_goff, sizeof(long long) * (n + 1), cudaMemcpyDeviceToHost, ctx->stream));
    MW_CK(cudaStreamSynchronize(ctx->stream));
    const long long total = offs[n];
    if (total > 0x7fffffffLL) {
        ctx->err = "work list of more than 2^31 items";
        return MWGPU_ERR_BAD_ARG;
    }
    if (total > ctx->items_cap) {
        if (ctx->d_items) cudaFree(ctx->d_items);
        ctx->d_items = nullptr;
        ctx->items_cap = std::max(total, 2 * ctx->items_cap);
        if (auto s = dev_alloc(ctx, &ctx->d_items, (size_t)ctx->items_cap)) return s;
    }
    launch_pairs_fill(m, o->op, inp->t, out->t, d_work, ctx->d_pair_off, n, np, gthr, ctx->d_item_off, ctx->d_items, ctx->d_err, ctx->stream);
    ctx->launches++;
    // chunks of about the same number of items, several waves of CTAs
    long long per = std::max<long long>(8, (total + 8 * 304 - 1) / (8 * 304));
    if (const char *e = std::getenv("MWGPU_CHUNK_ITEMS")) per = std::max<long long>(1, std::atoll(e));
    std::vector<int4> chunks;
    std::vector<int> cbeg(n + 1, 0);
    for (int i = 0; i < n; i++) {
        cbeg[i] = (int)chunks.size();
        long long b = offs[i], e = offs[i + 1];
        if (b == e) chunks.push_back(make_int4(i, (int)b, (int)e, 0));
        for (long long c = b; c < e; c += per) chunks.push_back(make_int4(i, (int)c, (int)std::min(e, c + per), 0));
    }
    cbeg[n] = (int)chunks.size();
    const int nch = (int)chunks.size();
    if (nch > ctx->chunks_cap || n + 1 > ctx->chunks_cap) {
        if (ctx->d_chunks) cudaFree(ctx->d_chunks);
        if (ctx->d_chunk_begin) cudaFree(ctx->d_chunk_begin);
        ctx->d_chunks = nullptr;
        ctx->d_chunk_begin = nullptr;
        ctx->chunks_cap = std::max(std::max(nch, n + 1), 2 * ctx->chunks_cap);
        if (auto s = dev_alloc(ctx, &ctx->d_chunks, ctx->chunks_cap)) return s;
        if (auto s = dev_alloc(ctx, &ctx->d_chunk_begin, ctx->chunks_cap)) return s;
    }
    const size_t need = (size_t)nch * 8 * (size_t)o->mra.kp1_d;  // doubles
    if (need > ctx->partial_cap) {
        if (ctx->d_partial) cudaFree(ctx->d_partial);
        ctx->d_partial = nullptr;
        ctx->partial_cap = std::max(need, 2 * ctx->partial_cap);
        if (auto s = dev_alloc(ctx, &ctx->d_partial, ctx->partial_cap)) return s;
    }
    MW_CK(cudaMemcpyAsync(ctx->d_chunks, chunks.data(), sizeof(int4) * nch, cudaMemcpyHostToDevice, ctx->stream));
    MW_CK(cudaMemcpyAsync(ctx->d_chunk_begin, cbeg.data(), sizeof(int) * (n + 1), cudaMemcpyHostToDevice, ctx->stream));
    MW_CK(cudaEventRecord(ctx->ev1, ctx->stream));
    launch_contract_items(o->mra, o->op, inp->t, out->t, d_work, n, ctx->d_chunks, nch, ctx->d_chunk_begin, ctx->d_items, ctx->d_partial,
                          ctx->d_err, ctx->stream);
    ctx->launches += 3;
    MW_CK(cudaStreamSynchronize(ctx->stream));  // host vectors above must outlive the copies
    hs->node_terms = (unsigned long long)total;
    return MWGPU_OK;
}

mwgpu_status make_tree(mwgpu_ctx *ctx, const mwgpu_mra_desc *mra, const mwgpu_tree_desc *d, bool input, mwgpu_tree **out) {
    MW_ARG(out && d && d->n_nodes > 0 && d->idx && d->child0, "invalid tree descriptor");
    auto *tr = new mwgpu_tree();
    tr->is_input = input;
    if (auto s = make_mra(ctx, mra, tr->mra, &tr->d_filt)) { delete tr; return s; }
    DevTree &t = tr->t;
    const int n = d->n_nodes;
    const size_t nc = 8 * (size_t)tr->mra.kp1_d;
    t.n_real = n;
    t.cap_real = input ? n : std::max(n, 64);
    t.n_gen = 0;
    t.cap_gen = 0;
    int tot = t.cap_real;
    tr->h_idx.resize(n);
    tr->h_child0.assign(d->child0, d->child0 + n);
    for (int i = 0; i < n; i++) tr->h_idx[i] = make_int4(d->idx[4 * i], d->idx[4 * i + 1], d->idx[4 * i + 2], d->idx[4 * i + 3]);
    mwgpu_status s;
    if ((s = dev_alloc(ctx, &t.idx, tot)) || (s = dev_alloc(ctx, &t.coefs, (size_t)tot * nc)) || (s = dev_alloc(ctx, &t.norms, (size_t)tot * 8)) ||
        (s = dev_alloc(ctx, &t.child0, tot))) {
        delete tr;
        return s;
    }
    MW_CK(cudaMemcpyAsync(t.idx, tr->h_idx.data(), sizeof(int4) * n, cudaMemcpyHostToDevice, ctx->stream));
    MW_CK(cudaMemcpyAsync(t.child0, d->child0, sizeof(int) * n, cudaMemcpyHostToDevice, ctx->stream));
    if (d->coefs) MW_CK(cudaMemcpyAsync(t.coefs, d->coefs, sizeof(double) * n * nc, cudaMemcpyHostToDevice, ctx->stream));
    else MW_CK(cudaMemsetAsync(t.coefs, 0, sizeof(double) * tot * nc, ctx->stream));
    if (input) {
        // FP32 copy read by the mixed form
        if ((s = dev_alloc(ctx, &t.coefs32, (size_t)n * nc))) { free_tree(tr); return s; }
        launch_to_float(t.coefs, t.coefs32, (size_t)n * nc, ctx->stream);
        ctx->launches++;
    }
    if (d->norms) {
        MW_CK(cudaMemcpyAsync(t.norms, d->norms, sizeof(double) * n * 8, cudaMemcpyHostToDevice, ctx->stream));
    } else if (d->coefs) {
        std::vector<int> all(n);
        for (int i = 0; i < n; i++) all[i] = i;
        if ((s = ensure_work(ctx, n))) { delete tr; return s; }
        MW_CK(cudaMemcpyAsync(ctx->d_work, all.data(), sizeof(int) * n, cudaMemcpyHostToDevice, ctx->stream));
        launch_node_norms(tr->mra, t, ctx->d_work, n, ctx->stream);
        ctx->launches++;
    } else {
        MW_CK(cudaMemsetAsync(t.norms, 0, sizeof(double) * tot * 8, ctx->stream));
    }
    if ((s = rebuild_hash(ctx, tr, n))) { delete tr; return s; }
    *out = tr;
    return MWGPU_OK;
}

void free_tree(mwgpu_tree *tr) {
    if (!tr) return;
    DevTree &t = tr->t;
    cudaFree(t.idx);
    cudaFree(t.coefs);
    cudaFree(t.norms);
    cudaFree(t.child0);
    if (t.gcoefs) cudaFree(t.gcoefs);
    if (t.coefs32) cudaFree(t.coefs32);
    if (t.gcoefs32) cudaFree(t.gcoefs32);
    if (t.hkeys) cudaFree(t.hkeys);
    if (t.hvals) cudaFree(t.hvals);
    if (tr->d_filt) cudaFree(tr->d_filt);
    delete tr;
}

}  // namespace

extern "C" {

mwgpu_status mwgpu_init(mwgpu_ctx **out, const mwgpu_config *cfg) {
    if (!out) { g_init_error = "null context pointer"; return MWGPU_ERR_BAD_ARG; }
    *out = nullptr;
    int ndev = 0;
    cudaError_t e = cudaGetDeviceCount(&ndev);
    if (e != cudaSuccess || ndev == 0) {
        g_init_error = std::string("no CUDA device: ") + (e != cudaSuccess ? cudaGetErrorString(e) : "count is 0");
        return MWGPU_ERR_NO_DEVICE;
    }
    auto *ctx = new mwgpu_ctx();
    ctx->device = cfg ? cfg->device : 0;
    ctx->precision = cfg ? cfg->precision : MWGPU_PREC_FP64;
    if (ctx->device < 0 || ctx->device >= ndev) {
        g_init_error = "invalid device ordinal";
        delete ctx;
        return MWGPU_ERR_BAD_ARG;
    }
    if (cudaSetDevice(ctx->device) != cudaSuccess || cudaStreamCreateWithFlags(&ctx->stream, cudaStreamNonBlocking) != cudaSuccess ||
        cudaEventCreate(&ctx->ev0) != cudaSuccess || cudaEventCreate(&ctx->ev1) != cudaSuccess || cudaEventCreate(&ctx->ev2) != cudaSuccess ||
        cudaMalloc(&ctx->d_err, sizeof(int)) != cudaSuccess || cudaMalloc(&ctx->d_stats, sizeof(LevelStats)) != cudaSuccess ||
        cudaMalloc(&ctx->d_pcount, sizeof(int)) != cudaSuccess) {
        g_init_error = std::string("device initialisation failed: ") + cudaGetErrorString(cudaGetLastError());
        delete ctx;
        return MWGPU_ERR_DEVICE;
    }
    cudaMemset(ctx->d_err, 0, sizeof(int));
    *out = ctx;
    return MWGPU_OK;
}

mwgpu_status mwgpu_destroy(mwgpu_ctx *ctx) {
    if (!ctx) return MWGPU_ERR_BAD_ARG;
    cudaSetDevice(ctx->device);
    cudaStreamSynchronize(ctx->stream);
    for (void *p : {(void *)ctx->d_err, (void *)ctx->d_stats, (void *)ctx->d_work, (void *)ctx->d_pkeys, (void *)ctx->d_pvals,
                    (void *)ctx->d_plist, (void *)ctx->d_pcount, (void *)ctx->d_list, (void *)ctx->d_items, (void *)ctx->d_chunks,
                    (void *)ctx->d_chunk_begin, (void *)ctx->d_partial, (void *)ctx->d_pair_off, (void *)ctx->d_pcounts,
                    (void *)ctx->d_item_off, (void *)ctx->d_scan, (void *)ctx->d_goff})
        if (p) cudaFree(p);
    for (auto &e : ctx->marks)
        if (e) cudaEventDestroy(e);
    if (ctx->d_scrub) cudaFree(ctx->d_scrub);
    cudaEventDestroy(ctx->ev0);
    cudaEventDestroy(ctx->ev1);
    cudaEventDestroy(ctx->ev2);
    cudaStreamDestroy(ctx->stream);
    delete ctx;
    return MWGPU_OK;
}

const char *mwgpu_last_error(const mwgpu_ctx *ctx) { return ctx ? ctx->err.c_str() : g_init_error.c_str(); }

mwgpu_status mwgpu_set_precision(mwgpu_ctx *ctx, int precision) {
    if (!ctx) return MWGPU_ERR_BAD_ARG;
    MW_ARG(precision == MWGPU_PREC_FP64 || precision == MWGPU_PREC_MIXED, "invalid precision mode");
    ctx->precision = precision;
    return MWGPU_OK;
}

mwgpu_status mwgpu_upload_operator(mwgpu_ctx *ctx, const mwgpu_mra_desc *mra, const mwgpu_oper_desc *d, double prec, mwgpu_oper **out) {
    if (!ctx) return MWGPU_ERR_BAD_ARG;
    MW_ARG(out && d && d->n_terms > 0 && d->depth && d->max_transl && d->blocks && d->norms, "invalid operator descriptor");
    MW_ARG(mra && d->order == mra->order, "operator order differs from the MRA order");
    cudaSetDevice(ctx->device);
    auto *o = new mwgpu_oper();
    if (auto s = make_mra(ctx, mra, o->mra, &o->d_filt)) { delete o; return s; }
    const int T = d->n_terms, K = d->order + 1, K2 = K * K;
    if (prec < 0.0) prec = d->build_prec;
    int maxDepth = 0;
    for (int t = 0; t < T; t++) maxDepth = std::max(maxDepth, d->depth[t]);
    const int rows = std::max(maxDepth + 1, kMaxDepthRows + 1);
    o->n_rows = rows;
    std::vector<int> dep_off((size_t)T * rows, -1), dep_L((size_t)T * rows, 0);
    std::vector<int> bw((size_t)T * rows * 5, -1);
    size_t node = 0, tl = 0;
    for (int t = 0; t < T; t++) {
        for (int dd = 0; dd < d->depth[t]; dd++) {
            int L = d->max_transl[tl + dd];
            dep_off[(size_t)t * rows + dd] = (int)node;
            dep_L[(size_t)t * rows + dd] = L;
            // OperatorTree::calcBandWidth
            int l = 0;
            bool done = false;
            while (!done) {
                done = true;
                size_t nid = node + (size_t)(l + L);
                double thrs = std::max(kMachinePrec, prec / (8.0 * (1 << dd)));
                for (int c = 0; c < 4; c++) {
                    if (d->norms[nid * 4 + c] > thrs) {
                        int *w = &bw[((size_t)t * rows + dd) * 5];
                        w[c] = l;
                        if (l > w[4]) w[4] = l;
                        done = false;
                    }
                }
                if (++l > L) break;
            }
            node += 2 * (size_t)L + 1;
        }
        tl += d->depth[t];
    }
    // MWOperator::calcBandWidths: band_max over terms and components, rows 0..maxDepth
    std::vector<int> band_max(rows, -1);
    for (int t = 0; t < T; t++)
        for (int n = 0; n <= d->depth[t]; n++)
            for (int c = 0; c < 4; c++) band_max[n] = std::max(band_max[n], bw[((size_t)t * rows + n) * 5 + c]);
    // ConvolutionCalculator::calcBandSizeFactor (direction-0 widths only)
    std::vector<int> bsz((size_t)T * kMaxDepthRows * 64, 0);
    for (int t = 0; t < T; t++)
        for (int dd = 0; dd < kMaxDepthRows; dd++)
            for (int gt = 0; gt < 8; gt++)
                for (int ft = 0; ft < 8; ft++) {
                    int tot = 1;
                    for (int i = 0; i < 3; i++) {
                        int oIdx = 2 * ((gt >> i) & 1) + ((ft >> i) & 1);
                        int width = dd < rows ? bw[((size_t)t * rows + dd) * 5 + oIdx] : -1;
                        if (dd > d->depth[t]) width = -1;
                        if (width < 0) continue;
                        tot *= 2 * width + 1;
                    }
                    bsz[((size_t)t * kMaxDepthRows + dd) * 64 + gt * 8 + ft] = tot * 64;
                }
    // terms ordered by descending max width per depth (stable)
    std::vector<int> order((size_t)rows * T);
    for (int dd = 0; dd < rows; dd++) {
        std::vector<int> idx(T);
        for (int t = 0; t < T; t++) idx[t] = t;
        std::stable_sort(idx.begin(), idx.end(), [&](int a, int b) {
            return bw[((size_t)a * rows + dd) * 5 + 4] > bw[((size_t)b * rows + dd) * 5 + 4];
        });
        for (int t = 0; t < T; t++) order[(size_t)dd * T + t] = idx[t];
    }
    o->widths = bw;
    o->band_max = band_max;
    auto up = [&](auto **dst, const auto *src, size_t n) -> mwgpu_status {
        using E = std::remove_pointer_t<std::remove_reference_t<decltype(*dst)>>;
        if (auto s = dev_alloc(ctx, (E **)dst, n)) return s;
        o->allocs.push_back((void *)*dst);
        MW_CK(cudaMemcpy((void *)*dst, src, sizeof(E) * n, cudaMemcpyHostToDevice));
        return MWGPU_OK;
    };
    int *p_td, *p_off, *p_L, *p_bw, *p_bsz, *p_bm, *p_ord;
    double *p_blk, *p_nrm;
    std::vector<float> blk32(node * 4 * K2);
    for (size_t q = 0; q < blk32.size(); q++) blk32[q] = (float)d->blocks[q];
    float *p_blk32;
    mwgpu_status s;
    if ((s = up(&p_td, d->depth, T)) || (s = up(&p_off, dep_off.data(), dep_off.size())) || (s = up(&p_L, dep_L.data(), dep_L.size())) ||
        (s = up(&p_bw, bw.data(), bw.size())) || (s = up(&p_bsz, bsz.data(), bsz.size())) || (s = up(&p_bm, band_max.data(), band_max.size())) ||
        (s = up(&p_ord, order.data(), order.size())) || (s = up(&p_blk, d->blocks, node * 4 * K2)) || (s = up(&p_nrm, d->norms, node * 4)) ||
        (s = up(&p_blk32, blk32.data(), blk32.size()))) {
        for (void *p : o->allocs) cudaFree(p);
        delete o;
        return s;
    }
    o->op.n_terms = T;
    o->op.K = K;
    o->op.max_rows = rows;
    o->op.term_depth = p_td;
    o->op.dep_off = p_off;
    o->op.dep_L = p_L;
    o->op.blocks = p_blk;
    o->op.norms = p_nrm;
    o->op.bw = p_bw;
    o->op.band_size = p_bsz;
    o->op.band_max = p_bm;
    o->op.term_order = p_ord;
    o->op.n_band_max = maxDepth + 1;
    o->op.blocks32 = p_blk32;
    *out = o;
    return MWGPU_OK;
}

mwgpu_status mwgpu_free_operator(mwgpu_ctx *ctx, mwgpu_oper *o) {
    if (!ctx || !o) return MWGPU_ERR_BAD_ARG;
    for (void *p : o->allocs) cudaFree(p);
    if (o->d_filt) cudaFree(o->d_filt);
    delete o;
    return MWGPU_OK;
}

mwgpu_status mwgpu_operator_bandwidths(mwgpu_ctx *ctx, const mwgpu_oper *o, int *n_rows, int *widths, int *band_max) {
    if (!ctx || !o || !n_rows) return MWGPU_ERR_BAD_ARG;
    *n_rows = o->n_rows;
    if (widths) std::memcpy(widths, o->widths.data(), sizeof(int) * o->widths.size());
    if (band_max) std::memcpy(band_max, o->band_max.data(), sizeof(int) * o->band_max.size());
    return MWGPU_OK;
}

mwgpu_status mwgpu_upload_tree(mwgpu_ctx *ctx, const mwgpu_mra_desc *mra, const mwgpu_tree_desc *d, mwgpu_tree **out) {
    if (!ctx) return MWGPU_ERR_BAD_ARG;
    MW_ARG(d && d->coefs, "input tree needs coefficients");
    cudaSetDevice(ctx->device);
    return make_tree(ctx, mra, d, true, out);
}

mwgpu_status mwgpu_create_tree(mwgpu_ctx *ctx, const mwgpu_mra_desc *mra, const mwgpu_tree_desc *d, mwgpu_tree **out) {
    if (!ctx) return MWGPU_ERR_BAD_ARG;
    cudaSetDevice(ctx->device);
    return make_tree(ctx, mra, d, false, out);
}

mwgpu_status mwgpu_tree_add_nodes(mwgpu_ctx *ctx, mwgpu_tree *tr, int n, const int *idx, int n_parents, const int *parent_ids,
                                  const int *parent_child0) {
    if (!ctx || !tr) return MWGPU_ERR_BAD_ARG;
    MW_ARG(!tr->is_input, "cannot add nodes to an input tree");
    MW_ARG(n >= 0 && (n == 0 || idx), "invalid node list");
    cudaSetDevice(ctx->device);
    DevTree &t = tr->t;
    int old = t.n_real;
    if (auto s = grow_real(ctx, tr, old + n)) return s;
    for (int i = 0; i < n; i++) {
        tr->h_idx.push_back(make_int4(idx[4 * i], idx[4 * i + 1], idx[4 * i + 2], idx[4 * i + 3]));
        tr->h_child0.push_back(-1);
    }
    for (int p = 0; p < n_parents; p++) {
        MW_ARG(parent_ids[p] >= 0 && parent_ids[p] < old + n, "invalid parent id");
        tr->h_child0[parent_ids[p]] = parent_child0[p];
    }
    if (n > 0) MW_CK(cudaMemcpyAsync(t.idx + old, tr->h_idx.data() + old, sizeof(int4) * n, cudaMemcpyHostToDevice, ctx->stream));
    MW_CK(cudaMemcpyAsync(t.child0, tr->h_child0.data(), sizeof(int) * (old + n), cudaMemcpyHostToDevice, ctx->stream));
    t.n_real = old + n;
    if (2LL * t.n_real + 16 > t.hcap) return rebuild_hash(ctx, tr, t.n_real);
    if (n > 0) {
        MW_CK(cudaMemsetAsync(ctx->d_err, 0, sizeof(int), ctx->stream));
        launch_hash_build(tr->mra, t, old, n, ctx->d_err, ctx->stream);
        ctx->launches++;
        return check_err(ctx, "tree_add_nodes");
    }
    return MWGPU_OK;
}

mwgpu_status mwgpu_tree_size(const mwgpu_tree *tr, int *n) {
    if (!tr || !n) return MWGPU_ERR_BAD_ARG;
    *n = tr->t.n_real;
    return MWGPU_OK;
}

mwgpu_status mwgpu_free_tree(mwgpu_ctx *ctx, mwgpu_tree *tr) {
    if (!ctx || !tr) return MWGPU_ERR_BAD_ARG;
    cudaSetDevice(ctx->device);
    cudaStreamSynchronize(ctx->stream);
    free_tree(tr);
    return MWGPU_OK;
}

mwgpu_status mwgpu_apply_level(mwgpu_ctx *ctx, const mwgpu_oper *o, mwgpu_tree *inp, mwgpu_tree *out, const int *node_ix, int n,
                               double prec, double out_sqnorm, double *norms_out, mwgpu_level_stats *stats) {
    if (!ctx) return MWGPU_ERR_BAD_ARG;
    MW_ARG(o && inp && out && inp->is_input && !out->is_input, "invalid operator or trees");
    MW_ARG(n >= 0 && (n == 0 || node_ix), "invalid node list");
    MW_ARG(inp->mra.K == o->op.K && out->mra.K == o->op.K, "order mismatch");
    cudaSetDevice(ctx->device);
    if (stats) std::memset(stats, 0, sizeof(*stats));
    if (n == 0) return MWGPU_OK;
    for (int i = 0; i < n; i++) MW_ARG(node_ix[i] >= 0 && node_ix[i] < out->t.n_real, "node index out of range");
    if (auto s = ensure_work(ctx, n)) return s;
    MW_CK(cudaEventRecord(ctx->ev0, ctx->stream));
    MW_CK(cudaMemcpyAsync(ctx->d_work, node_ix, sizeof(int) * n, cudaMemcpyHostToDevice, ctx->stream));
    MW_CK(cudaMemsetAsync(ctx->d_err, 0, sizeof(int), ctx->stream));
    MW_CK(cudaMemsetAsync(ctx->d_stats, 0, sizeof(LevelStats), ctx->stream));
    // GenNodes needed by the operator bands of this level
    int pcount = 0;
    for (int attempt = 0; attempt < 8; attempt++) {
        if (auto s = ensure_pending(ctx, std::max(ctx->phcap, 1 << 16), std::max(ctx->pcap, 1 << 15))) return s;
        MW_CK(cudaMemsetAsync(ctx->d_pkeys, 0xFF, sizeof(uint64_t) * ctx->phcap, ctx->stream));
        MW_CK(cudaMemsetAsync(ctx->d_pcount, 0, sizeof(int), ctx->stream));
        launch_band_missing(o->mra, o->op, inp->t, out->t, ctx->d_work, n, ctx->d_pkeys, ctx->d_pvals, ctx->phcap, ctx->d_plist,
                            ctx->d_pcount, ctx->pcap, ctx->d_err, ctx->stream);
        ctx->launches++;
        int herr = 0;
        MW_CK(cudaMemcpyAsync(&pcount, ctx->d_pcount, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
        MW_CK(cudaMemcpyAsync(&herr, ctx->d_err, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
        MW_CK(cudaStreamSynchronize(ctx->stream));
        if (herr & DE_RANGE) { ctx->err = "band index outside the lookup range"; return MWGPU_ERR_INTERNAL; }
        bool hfull = herr & DE_HASH_FULL;
        if (!hfull && pcount <= ctx->pcap) break;
        MW_CK(cudaMemsetAsync(ctx->d_err, 0, sizeof(int), ctx->stream));
        if (auto s = ensure_pending(ctx, hfull ? ctx->phcap * 4 : next_pow2(4LL * pcount), std::max(pcount + 1024, ctx->pcap))) return s;
        if (attempt == 7) { ctx->err = "pending GenNode set did not fit"; return MWGPU_ERR_OOM; }
    }
    if (pcount > 0) {
        DevTree &f = inp->t;
        if (auto s = grow_gen(ctx, inp, f.n_gen + pcount)) return s;
        if (2LL * (f.n_real + f.n_gen + pcount) + 16 > f.hcap)
            if (auto s = rebuild_hash(ctx, inp, (long long)f.n_real + f.n_gen + pcount)) return s;
        launch_gen_nodes(inp->mra, f, ctx->d_plist, pcount, f.n_gen, ctx->d_err, ctx->stream);
        launch_gen_insert(inp->mra, f, ctx->d_plist, pcount, f.n_gen, ctx->d_err, ctx->stream);
        ctx->launches += 2;
        f.n_gen += pcount;
    }
    double gthr = out_sqnorm;
    if (gthr > 0.0) gthr = prec * 1.0 * std::sqrt(gthr / (double)o->op.n_terms);
    if (ctx->precision == MWGPU_PREC_MIXED && !mixed_supported(o->op.K)) {
        ctx->err = "mixed form supports orders k = 1..11";
        return MWGPU_ERR_BAD_ARG;
    }
    LevelStats mixed_nt{};
    if (ctx->precision == MWGPU_PREC_MIXED) {
        if (auto s = run_mixed(ctx, o, inp, out, ctx->d_work, node_ix, n, gthr, &mixed_nt)) return s;
    } else {
        MW_CK(cudaEventRecord(ctx->ev1, ctx->stream));
        launch_contract_fp64(o->mra, o->op, inp->t, out->t, ctx->d_work, n, gthr, ctx->d_stats, ctx->d_err, ctx->stream);
        ctx->launches++;
    }
    MW_CK(cudaGetLastError());
    MW_CK(cudaEventRecord(ctx->ev2, ctx->stream));
    LevelStats hs{};
    MW_CK(cudaMemcpyAsync(&hs, ctx->d_stats, sizeof(LevelStats), cudaMemcpyDeviceToHost, ctx->stream));
    if (norms_out) {
        // gather the norms of the computed nodes
        std::vector<double> all((size_t)out->t.n_real * 8);
        MW_CK(cudaMemcpyAsync(all.data(), out->t.norms, sizeof(double) * all.size(), cudaMemcpyDeviceToHost, ctx->stream));
        if (auto s = check_err(ctx, "apply_level")) return s;
        for (int i = 0; i < n; i++) std::memcpy(norms_out + 8 * (size_t)i, &all[(size_t)node_ix[i] * 8], sizeof(double) * 8);
    } else if (auto s = check_err(ctx, "apply_level")) {
        return s;
    }
    if (ctx->precision == MWGPU_PREC_MIXED) hs.node_terms = mixed_nt.node_terms;
    if (stats) {
        stats->node_terms = hs.node_terms;
        stats->components = hs.components;
        stats->band_nodes = hs.band_nodes;
        stats->gen_nodes = (unsigned long long)pcount;
        float ms = 0.f;
        cudaEventElapsedTime(&ms, ctx->ev0, ctx->ev2);
        stats->device_ms = ms;
        cudaEventElapsedTime(&ms, ctx->ev1, ctx->ev2);
        stats->contract_ms = ms;
    }
    return MWGPU_OK;
}

mwgpu_status mwgpu_transform(mwgpu_ctx *ctx, mwgpu_tree *tr, int direction, int overwrite) {
    if (!ctx || !tr) return MWGPU_ERR_BAD_ARG;
    MW_ARG(direction == MWGPU_TOPDOWN || direction == MWGPU_BOTTOMUP, "invalid transform direction");
    MW_ARG(!(direction == MWGPU_BOTTOMUP && !overwrite), "BottomUp transform always overwrites");
    cudaSetDevice(ctx->device);
    const int n = tr->t.n_real;
    // parents per depth (breadth-first order from the roots)
    std::vector<int> depth(n, -1);
    std::vector<std::vector<int>> levels;
    for (int i = 0; i < n; i++) depth[i] = tr->h_idx[i].x - tr->mra.root_scale;
    int maxd = 0;
    for (int i = 0; i < n; i++) maxd = std::max(maxd, depth[i]);
    levels.resize(maxd + 1);
    for (int i = 0; i < n; i++)
        if (tr->h_child0[i] >= 0 && depth[i] >= 0) levels[depth[i]].push_back(i);
    std::vector<int> flat;
    std::vector<std::pair<int, int>> ranges;
    for (auto &l : levels) { ranges.push_back({(int)flat.size(), (int)l.size()}); flat.insert(flat.end(), l.begin(), l.end()); }
    if (flat.empty()) return MWGPU_OK;
    if ((int)flat.size() > ctx->list_cap) {
        if (ctx->d_list) cudaFree(ctx->d_list);
        ctx->list_cap = (int)flat.size() * 2;
        if (auto s = dev_alloc(ctx, &ctx->d_list, ctx->list_cap)) return s;
    }
    MW_CK(cudaMemcpyAsync(ctx->d_list, flat.data(), sizeof(int) * flat.size(), cudaMemcpyHostToDevice, ctx->stream));
    if (direction == MWGPU_TOPDOWN) {
        for (auto &r : ranges) {
            launch_mw_down(tr->mra, tr->t, ctx->d_list + r.first, r.second, overwrite != 0, ctx->stream);
            ctx->launches += r.second > 0;
        }
    } else {
        for (int l = (int)ranges.size() - 1; l >= 0; l--) {
            launch_mw_up(tr->mra, tr->t, ctx->d_list + ranges[l].first, ranges[l].second, ctx->stream);
            ctx->launches += ranges[l].second > 0;
        }
    }
    MW_CK(cudaGetLastError());
    MW_CK(cudaStreamSynchronize(ctx->stream));
    return MWGPU_OK;
}

mwgpu_status mwgpu_download_tree(mwgpu_ctx *ctx, const mwgpu_tree *tr, double *coefs, double *norms) {
    if (!ctx || !tr) return MWGPU_ERR_BAD_ARG;
    cudaSetDevice(ctx->device);
    const size_t n = tr->t.n_real, nc = 8 * (size_t)tr->mra.kp1_d;
    if (coefs) MW_CK(cudaMemcpyAsync(coefs, tr->t.coefs, sizeof(double) * n * nc, cudaMemcpyDeviceToHost, ctx->stream));
    if (norms) MW_CK(cudaMemcpyAsync(norms, tr->t.norms, sizeof(double) * n * 8, cudaMemcpyDeviceToHost, ctx->stream));
    MW_CK(cudaStreamSynchronize(ctx->stream));
    return MWGPU_OK;
}

mwgpu_status mwgpu_sync(mwgpu_ctx *ctx) {
    if (!ctx) return MWGPU_ERR_BAD_ARG;
    MW_CK(cudaStreamSynchronize(ctx->stream));
    return MWGPU_OK;
}

mwgpu_status mwgpu_tree_clear_generated(mwgpu_ctx *ctx, mwgpu_tree *tr) {
    if (!ctx || !tr) return MWGPU_ERR_BAD_ARG;
    MW_ARG(tr->is_input, "only input trees hold GenNodes");
    cudaSetDevice(ctx->device);
    if (tr->t.n_gen == 0) return MWGPU_OK;
    tr->t.n_gen = 0;
    return rebuild_hash(ctx, tr, tr->t.n_real);
}

mwgpu_status mwgpu_timer_mark(mwgpu_ctx *ctx, int slot) {
    if (!ctx) return MWGPU_ERR_BAD_ARG;
    MW_ARG(slot >= 0 && slot < 16, "timer slot out of range");
    cudaSetDevice(ctx->device);
    if (!ctx->marks[slot]) MW_CK(cudaEventCreate(&ctx->marks[slot]));
    MW_CK(cudaEventRecord(ctx->marks[slot], ctx->stream));
    return MWGPU_OK;
}

mwgpu_status mwgpu_timer_elapsed(mwgpu_ctx *ctx, int a, int b, double *ms) {
    if (!ctx || !ms) return MWGPU_ERR_BAD_ARG;
    MW_ARG(a >= 0 && a < 16 && b >= 0 && b < 16 && ctx->marks[a] && ctx->marks[b], "timer slot not recorded");
    MW_CK(cudaEventSynchronize(ctx->marks[b]));
    float f = 0.f;
    MW_CK(cudaEventElapsedTime(&f, ctx->marks[a], ctx->marks[b]));
    *ms = f;
    return MWGPU_OK;
}

mwgpu_status mwgpu_launch_count(const mwgpu_ctx *ctx, unsigned long long *count) {
    if (!ctx || !count) return MWGPU_ERR_BAD_ARG;
    *count = ctx->launches;
    return MWGPU_OK;
}

mwgpu_status mwgpu_scrub_l2(mwgpu_ctx *ctx, size_t bytes) {
    if (!ctx) return MWGPU_ERR_BAD_ARG;
    cudaSetDevice(ctx->device);
    if (bytes > ctx->scrub_bytes) {
        if (ctx->d_scrub) cudaFree(ctx->d_scrub);
        ctx->d_scrub = nullptr;
        MW_CK(cudaMalloc(&ctx->d_scrub, bytes));
        ctx->scrub_bytes = bytes;
    }
    MW_CK(cudaMemsetAsync(ctx->d_scrub, (int)(ctx->launches & 0xff), bytes, ctx->stream));
    return MWGPU_OK;
}

}  // extern "C"

// ---------------------------------------------------------------------------
// Allocation-free level computation.
//
// For callers that must not allocate device memory while they run a level:
// code inside a framework whose caching allocator owns the device memory (a
// stray cudaMalloc outside it fragments the pool and can fail once the pool
// has claimed the free memory), and latency-critical loops where cudaMalloc /
// cudaFree would synchronise the device.  mwgpu_apply_level keeps its work
// list, error flag and counters in context buffers that it grows with
// cudaMalloc when a level is larger than any before; this variant keeps them
// in one file-scope device array of fixed size instead.
// ---------------------------------------------------------------------------
namespace {

constexpr int kStaticMaxNodes = 65536;  // largest node list one call accepts
constexpr int kStaticMaxDevices = 64;

struct StaticScratch {
    int work[kStaticMaxNodes];              // node indices of the level
    double norms[(size_t)kStaticMaxNodes * 8];  // component norms staged for the host
    LevelStats stats;                       // counters, zeroed by every call
    int err;                                // device error flags, zeroed by every call
};

// 4.5 MiB per device, held from library load until process exit.  Host code
// must not pass `g_static_scratch` itself to a kernel: on the host that name
// is only a stand-in for the device symbol; its device address comes from
// cudaGetSymbolAddress below.
static __device__ __align__(256) StaticScratch g_static_scratch;

std::mutex g_static_mu;
StaticScratch *g_static_addr[kStaticMaxDevices] = {};

__global__ void k_gather_norms(const double *norms, const int *work, int n, double *dst) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n * 8) return;
    dst[i] = norms[(size_t)work[i / 8] * 8 + (i % 8)];
}

}  // namespace

extern "C" mwgpu_status mwgpu_apply_level_static(mwgpu_ctx *ctx, const mwgpu_oper *o, const mwgpu_tree *inp, mwgpu_tree *out,
                                                 const int *node_ix, int n, double prec, double out_sqnorm, double *norms_out,
                                                 mwgpu_level_stats *stats) {
    if (!ctx) return MWGPU_ERR_BAD_ARG;
    MW_ARG(o && inp && out && inp->is_input && !out->is_input, "invalid operator or trees");
    MW_ARG(n >= 0 && (n == 0 || node_ix), "invalid node list");
    MW_ARG(n <= kStaticMaxNodes, "mwgpu_apply_level_static accepts at most 65536 nodes per call");
    MW_ARG(inp->mra.K == o->op.K && out->mra.K == o->op.K, "order mismatch");
    MW_ARG(ctx->device >= 0 && ctx->device < kStaticMaxDevices, "device ordinal beyond the static scratch table");
    MW_ARG(ctx->precision == MWGPU_PREC_FP64, "mwgpu_apply_level_static computes the FP64 form only");
    for (int i = 0; i < n; i++) MW_ARG(node_ix[i] >= 0 && node_ix[i] < out->t.n_real, "node index out of range");
    MW_CK(cudaSetDevice(ctx->device));
    if (stats) std::memset(stats, 0, sizeof(*stats));
    if (n == 0) return MWGPU_OK;
    // once per device, with the device current: the device address of the array
    StaticScratch *sc = nullptr;
    {
        std::lock_guard<std::mutex> lk(g_static_mu);
        if (!g_static_addr[ctx->device]) {
            void *p = nullptr;
            cudaError_t e = cudaGetSymbolAddress(&p, g_static_scratch);
            if (e != cudaSuccess || !p) {
                ctx->err = std::string("cudaGetSymbolAddress(static scratch): ") + cudaGetErrorString(e);
                return MWGPU_ERR_DEVICE;
            }
            g_static_addr[ctx->device] = (StaticScratch *)p;
        }
        sc = g_static_addr[ctx->device];
    }
    MW_CK(cudaEventRecord(ctx->ev0, ctx->stream));
    MW_CK(cudaMemcpyAsync(sc->work, node_ix, sizeof(int) * n, cudaMemcpyHostToDevice, ctx->stream));
    MW_CK(cudaMemsetAsync(&sc->err, 0, sizeof(int), ctx->stream));
    MW_CK(cudaMemsetAsync(&sc->stats, 0, sizeof(LevelStats), ctx->stream));
    double gthr = out_sqnorm;
    if (gthr > 0.0) gthr = prec * 1.0 * std::sqrt(gthr / (double)o->op.n_terms);
    MW_CK(cudaEventRecord(ctx->ev1, ctx->stream));
    // GenNodes are not made here: every band node must already be in the input
    // tree's lookup table (a band node that is missing sets DE_LOOKUP)
    launch_contract_fp64(o->mra, o->op, inp->t, out->t, sc->work, n, gthr, &sc->stats, &sc->err, ctx->stream);
    ctx->launches++;
    MW_CK(cudaGetLastError());
    MW_CK(cudaEventRecord(ctx->ev2, ctx->stream));
    if (norms_out) {
        k_gather_norms<<<(n * 8 + 255) / 256, 256, 0, ctx->stream>>>(out->t.norms, sc->work, n, sc->norms);
        ctx->launches++;
        MW_CK(cudaGetLastError());
        MW_CK(cudaMemcpyAsync(norms_out, sc->norms, sizeof(double) * 8 * (size_t)n, cudaMemcpyDeviceToHost, ctx->stream));
    }
    LevelStats hs{};
    int herr = 0;
    MW_CK(cudaMemcpyAsync(&hs, &sc->stats, sizeof(LevelStats), cudaMemcpyDeviceToHost, ctx->stream));
    MW_CK(cudaMemcpyAsync(&herr, &sc->err, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
    MW_CK(cudaStreamSynchronize(ctx->stream));
    if (herr & DE_LOOKUP) {
        ctx->err = "apply_level_static: a band node is missing from the input tree (run mwgpu_apply_level once on these nodes first)";
        return MWGPU_ERR_BAD_ARG;
    }
    if (herr) {
        ctx->err = "apply_level_static: device error flags " + std::to_string(herr);
        return MWGPU_ERR_INTERNAL;
    }
    if (stats) {
        stats->node_terms = hs.node_terms;
        stats->components = hs.components;
        stats->band_nodes = hs.band_nodes;
        stats->gen_nodes = 0;
        float ms = 0.f;
        cudaEventElapsedTime(&ms, ctx->ev0, ctx->ev2);
        stats->device_ms = ms;
        cudaEventElapsedTime(&ms, ctx->ev1, ctx->ev2);
        stats->contract_ms = ms;
    }
    return MWGPU_OK;
}
