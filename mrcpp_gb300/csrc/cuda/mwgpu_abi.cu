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

#include "abi_state.cuh"

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
    if (auto s = pool_alloc(ctx, filt, (size_t)8 * m.K * m.K)) return s;
    MW_CK(cudaMemcpyAsync(*filt, d->filters, bytes, cudaMemcpyHostToDevice, ctx->stream));
    m.filt = *filt;
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
        pool_free(ctx, t.hkeys);
        pool_free(ctx, t.hvals);
        t.hkeys = nullptr;
        t.hvals = nullptr;
        if (auto s = pool_alloc(ctx, &t.hkeys, hcap)) return s;
        if (auto s = pool_alloc(ctx, &t.hvals, hcap)) return s;
        t.hcap = hcap;
    }
    MW_CK(cudaMemsetAsync(t.hkeys, 0xFF, sizeof(NodeKey) * hcap, ctx->stream));
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
    if (auto s = pool_alloc(ctx, &idx, cap)) return s;
    if (auto s = pool_alloc(ctx, &coefs, (size_t)cap * nc)) return s;
    if (auto s = pool_alloc(ctx, &norms, (size_t)cap * 8)) return s;
    if (auto s = pool_alloc(ctx, &child0, cap)) return s;
    MW_CK(cudaMemsetAsync(coefs, 0, sizeof(double) * cap * nc, ctx->stream));
    if (t.n_real > 0) {
        MW_CK(cudaMemcpyAsync(idx, t.idx, sizeof(int4) * t.n_real, cudaMemcpyDeviceToDevice, ctx->stream));
        MW_CK(cudaMemcpyAsync(coefs, t.coefs, sizeof(double) * t.n_real * nc, cudaMemcpyDeviceToDevice, ctx->stream));
        MW_CK(cudaMemcpyAsync(norms, t.norms, sizeof(double) * t.n_real * 8, cudaMemcpyDeviceToDevice, ctx->stream));
        MW_CK(cudaMemcpyAsync(child0, t.child0, sizeof(int) * t.n_real, cudaMemcpyDeviceToDevice, ctx->stream));
    }
    // (stream order: the old blocks are reused only after these copies)
    pool_free(ctx, t.idx);
    pool_free(ctx, t.coefs);
    pool_free(ctx, t.norms);
    pool_free(ctx, t.child0);
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
    float *g32, *gtc = nullptr;
    if (auto s = pool_alloc(ctx, &idx, tot)) return s;
    if (auto s = pool_alloc(ctx, &norms, (size_t)tot * 8)) return s;
    if (auto s = pool_alloc(ctx, &g, (size_t)cap * K3)) return s;
    if (auto s = pool_alloc(ctx, &g32, (size_t)cap * K3)) return s;
    if (t.tc32)
        if (auto s = pool_alloc(ctx, &gtc, (size_t)cap * mwgpu::kTcGenFloats)) return s;
    MW_CK(cudaMemcpyAsync(idx, t.idx, sizeof(int4) * (t.cap_real + t.n_gen), cudaMemcpyDeviceToDevice, ctx->stream));
    MW_CK(cudaMemcpyAsync(norms, t.norms, sizeof(double) * 8 * (t.cap_real + t.n_gen), cudaMemcpyDeviceToDevice, ctx->stream));
    if (t.n_gen > 0) {
        MW_CK(cudaMemcpyAsync(g, t.gcoefs, sizeof(double) * K3 * t.n_gen, cudaMemcpyDeviceToDevice, ctx->stream));
        MW_CK(cudaMemcpyAsync(g32, t.gcoefs32, sizeof(float) * K3 * t.n_gen, cudaMemcpyDeviceToDevice, ctx->stream));
        if (gtc && t.gtc32)
            MW_CK(cudaMemcpyAsync(gtc, t.gtc32, sizeof(float) * mwgpu::kTcGenFloats * t.n_gen, cudaMemcpyDeviceToDevice, ctx->stream));
    }
    pool_free(ctx, t.idx);
    pool_free(ctx, t.norms);
    pool_free(ctx, t.gcoefs);
    pool_free(ctx, t.gcoefs32);
    if (t.gtc32) pool_free(ctx, t.gtc32);
    t.idx = idx;
    t.norms = norms;
    t.gcoefs = g;
    t.gcoefs32 = g32;
    t.gtc32 = gtc;
    t.cap_gen = cap;
    return MWGPU_OK;
}

mwgpu_status ensure_work(mwgpu_ctx *ctx, int n) {
    if (n <= ctx->work_cap) return MWGPU_OK;
    if (ctx->d_work) cudaFree(ctx->d_work);
    if (ctx->d_wtree) cudaFree(ctx->d_wtree);
    ctx->d_work = ctx->d_wtree = nullptr;
    ctx->work_cap = std::max(n, 2 * ctx->work_cap);
    if (auto s = dev_alloc(ctx, &ctx->d_work, ctx->work_cap)) return s;
    return dev_alloc(ctx, &ctx->d_wtree, ctx->work_cap);
}

mwgpu_status ensure_trees(mwgpu_ctx *ctx, int nt) {
    if (nt <= ctx->trees_cap) return MWGPU_OK;
    for (void *p : {(void *)ctx->d_fs, (void *)ctx->d_gs, (void *)ctx->d_gthr, (void *)ctx->d_pcount})
        if (p) cudaFree(p);
    ctx->d_fs = ctx->d_gs = nullptr;
    ctx->d_gthr = nullptr;
    ctx->d_pcount = nullptr;
    ctx->trees_cap = std::max(nt, 2 * ctx->trees_cap);
    if (auto s = dev_alloc(ctx, &ctx->d_fs, ctx->trees_cap)) return s;
    if (auto s = dev_alloc(ctx, &ctx->d_gs, ctx->trees_cap)) return s;
    if (auto s = dev_alloc(ctx, &ctx->d_gthr, ctx->trees_cap)) return s;
    if (auto s = dev_alloc(ctx, &ctx->d_pcount, ctx->trees_cap)) return s;
    ctx->pcount_cap = ctx->trees_cap;
    return MWGPU_OK;
}

// pending GenNode sets of nt trees: tree t uses hash slots [t phcap, (t+1) phcap)
// and list slots [t pcap, (t+1) pcap)
mwgpu_status ensure_pending(mwgpu_ctx *ctx, int phcap, int pcap, int nt) {
    if (phcap > ctx->phcap || (long long)phcap * nt > ctx->ph_total) {
        if (ctx->d_pkeys) cudaFree(ctx->d_pkeys);
        if (ctx->d_pvals) cudaFree(ctx->d_pvals);
        ctx->d_pkeys = nullptr;
        ctx->d_pvals = nullptr;
        ctx->phcap = std::max(phcap, ctx->phcap);
        ctx->ph_total = (long long)ctx->phcap * nt;
        if (auto s = dev_alloc(ctx, &ctx->d_pkeys, (size_t)ctx->ph_total)) return s;
        if (auto s = dev_alloc(ctx, &ctx->d_pvals, (size_t)ctx->ph_total)) return s;
    }
    if (pcap > ctx->pcap || (long long)pcap * nt > ctx->pl_total) {
        if (ctx->d_plist) cudaFree(ctx->d_plist);
        ctx->d_plist = nullptr;
        ctx->pcap = std::max(pcap, ctx->pcap);
        ctx->pl_total = (long long)ctx->pcap * nt;
        if (auto s = dev_alloc(ctx, &ctx->d_plist, (size_t)ctx->pl_total)) return s;
    }
    return MWGPU_OK;
}

mwgpu_status check_err(mwgpu_ctx *ctx, const char *phase) {
    int herr = 0;
    MW_CK(cudaMemcpyAsync(&herr, ctx->d_err, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
    MW_CK(cudaStreamSynchronize(ctx->stream));
    if (herr) {
        ctx->err = std::string(phase) + ": device error flags " + std::to_string(herr);
        return (herr & mwgpu::DE_TIMEOUT) ? MWGPU_ERR_TIMEOUT : MWGPU_ERR_INTERNAL;
    }
    return MWGPU_OK;
}

void free_tree(mwgpu_ctx *ctx, mwgpu_tree *tr);

// grows a device buffer of T to at least n elements (contents not kept)
template <class T> mwgpu_status grow_buf(mwgpu_ctx *ctx, T **p, long long *cap, long long n) {
    if (n <= *cap) return MWGPU_OK;
    if (*p) cudaFree(*p);
    *p = nullptr;
    *cap = std::max(n, 2 * *cap);
    return dev_alloc(ctx, p, (size_t)*cap);
}

// One level over nt (input, output) tree pairs that share an operator.  The
// work entries are grouped by tree: entries seg[t] .. seg[t+1]-1 are nodes of
// output tree t.
struct Level {
    const mwgpu_oper *o = nullptr;
    int nt = 0;
    mwgpu_tree *const *inps = nullptr;
    mwgpu_tree *const *outs = nullptr;
    int n = 0;
    std::vector<int> node, tree, order;  // grouped entries; order[j] = caller position of entry j
    std::vector<int> seg;
    std::vector<double> gthr;
    // precision scaled per output node (the precTrees form of apply): one
    // factor per grouped entry, and the thresholds made from them; empty: 1
    std::vector<double> pfac, gnode;
    std::vector<DevTree> fs, gs;
    // derivative levels: band direction (-1: convolution), band width, operator order
    int band_dir = -1, band_w = 0, deriv_order = 0;
    DevOper op() const {
        DevOper d = o->op;
        d.band_dir = band_dir;
        d.band_dir_w = band_w;
        return d;
    }
};

// (g, band cell) pairs of every work entry: the band boxes of makeOperBand
// (ConvolutionCalculator.cpp:142-222), clipped to the world; poff[n] = total
void pair_offsets(const Level &lv, std::vector<long long> &poff) {
    const mwgpu_oper *o = lv.o;
    const DevMRA &m = o->mra;
    const int n = lv.n;
    poff.assign(n + 1, 0);
    for (int wi = 0; wi < n; wi++) {
        const int4 gx = lv.outs[lv.tree[wi]]->h_idx[lv.node[wi]];
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
}

// The pencil contraction (k_pencil.cu) takes the terms of band width <=
// kPencilMaxW on levels without norm screening (every gThreshold negative:
// fixed grids, first TreeBuilder iterations), order 7, input trees with their
// TF32 operands; the item kernel keeps the wider terms.  MWGPU_NO_PENCIL
// selects the item kernel for everything (the same sums).
bool use_pencil(const Level &lv) {
    const mwgpu_oper *o = lv.o;
    if (!pencil_supported(o->op.K) || !o->op.btc_stack || !o->op.pfrag || lv.band_dir >= 0 || std::getenv("MWGPU_NO_PENCIL")) return false;
    for (double g : lv.gthr)
        if (!(g < 0.0)) return false;
    for (double g : lv.gnode)
        if (!(g < 0.0)) return false;
    for (int t = 0; t < lv.nt; t++)
        if (!lv.inps[t]->t.tc32) return false;
    return true;
}

// Consumer warps of the pencil kernel (its CTA shape) where no autotuning
// chose them: MWGPU_PENCIL_WARPS = 8 or 16, else the default.
int pencil_warps() {
    if (const char *e = std::getenv("MWGPU_PENCIL_WARPS")) {
        const int w = std::atoi(e);
        if ((w == 8 || w == 16) && pencil_shape_ok(w)) return w;
    }
    return kPencilWarpsDefault;
}

// Units of the pencil contraction from the topology: per work entry the tasks
// (l_z in the world) with their pencils (l_y in the world) and term groups;
// tasks in descending size (the persistent kernel takes them in this order),
// each with its partial slot (slots of a work entry consecutive, pen_begin).
struct PencilPlan {
    std::vector<PencilUnit> flat;   // units in creation order, task t's at flat[tstart[t] .. tstart[t+1])
    std::vector<int> tstart, ord;   // ord: the tasks in processing order
    std::vector<int> task_unit;     // first unit of every processed task, + total
    std::vector<int> pen_begin;     // per work entry its first slot, + total
    int n_tasks = 0;
    size_t n_units = 0;
    // the units in processing order of their tasks into dst[0 .. n_units)
    void emit(PencilUnit *dst) const {
        for (int k = 0; k < n_tasks; k++) {
            const int t = ord[k];
            std::copy(flat.begin() + tstart[t], flat.begin() + tstart[t + 1], dst + task_unit[k]);
        }
    }
};

// Pencil configuration of a level: per-call levels take the terms of band
// width <= 1 (their units are made on the host on every call, and the wider
// terms would multiply them), plans the terms up to kPencilMaxW (units made
// once; measured on the bench level: 2.64 ms for the contraction against 3.14
// ms with the narrow terms only).
constexpr int kLevelPencilCfg = 0, kPlanPencilCfg = 1;

void pencil_build(const Level &lv, PencilPlan &pp, int cfg) {
    const mwgpu_oper *o = lv.o;
    const DevMRA &m = o->mra;
    const int G = o->pen_groups, n = lv.n;
    constexpr int G5 = mwgpu::kPencilGroup, NK = mwgpu::kPencilMaxL + 1, NS = mwgpu::kPencilSlots;
    std::vector<PencilUnit> &flat = pp.flat;
    std::vector<int> &tstart = pp.tstart;
    std::vector<long long> cost;
    flat.clear();
    tstart.clear();
    pp.pen_begin.assign(n + 1, 0);
    for (int wi = 0; wi < n; wi++) {
        pp.pen_begin[wi] = (int)tstart.size();
        const int4 gx = lv.outs[lv.tree[wi]]->h_idx[lv.node[wi]];
        const int depth = gx.x - m.root_scale;
        if (depth < 0 || depth >= o->n_rows || o->band_max[depth] < 0) continue;
        const mwgpu_oper::PenCfg &pc = o->pen[cfg];
        const int *tk = &pc.tk[(size_t)depth * NK];
        if (tk[0] == 0) continue;
        const int W = std::min(o->band_max[depth], mwgpu::kPencilCfgW[cfg]);
        auto inworld = [&](int d, long long l) {
            const long long c = (long long)m.corner[d] << depth, nb = (long long)m.nbox[d] << depth;
            return l >= c && l < c + nb;
        };
        const int gl[3] = {gx.y, gx.z, gx.w};
        for (int lz = -W; lz <= W; lz++) {
            if (!inworld(2, (long long)gl[2] + lz)) continue;
            const size_t first = flat.size();
            const int task = (int)tstart.size();
            long long c = 0;
            for (int ly = -W; ly <= W; ly++) {
                if (!inworld(1, (long long)gl[1] + ly)) continue;
                const int mm = std::max(std::abs(ly), std::abs(lz));
                const int tm = tk[mm];
                for (int q = 0; q * G5 < tm; q++) {
                    PencilUnit U{};
                    U.pflags = 3;   // the kernel stages every unit's f nodes
                    U.task = task;
                    U.wi = wi;
                    U.depth = (short)depth;
                    U.ly = (signed char)ly;
                    U.lz = (signed char)lz;
                    U.q = (short)(pc.r0[depth] + G5 * q);
                    U.nt = (short)std::min(G5, tm - G5 * q);
                    int xw = 0;
                    for (int k = 0; k < NK; k++) {
                        U.ntk[k] = (short)std::min((int)U.nt, std::max(0, tk[k] - G5 * q));
                        if (U.ntk[k] > 0) xw = k;
                    }
                    U.xw = (short)xw;
                    for (int b = 0; b < NS; b++) {
                        const size_t ix = ((size_t)depth * G + q) * NS + b;
                        U.form[b] = pc.form[ix];
                        U.nform[b] = pc.nform[ix];
                        U.fid[b] = -1;
                        if ((b + 1) / 2 <= xw) c += 2;   // tensor-core products
                    }
                    flat.push_back(U);
                    c += 3 * U.nt;                       // y / z steps
                }
            }
            if (flat.size() == first) continue;
            tstart.push_back((int)first);
            cost.push_back(c);
        }
    }
    tstart.push_back((int)flat.size());
    pp.n_tasks = (int)cost.size();
    pp.pen_begin[n] = pp.n_tasks;
    // tasks in descending cost (the persistent kernel takes them in this order)
    std::vector<int> &ord = pp.ord;
    ord.resize(pp.n_tasks);
    for (int i = 0; i < pp.n_tasks; i++) ord[i] = i;
    std::stable_sort(ord.begin(), ord.end(), [&](int a, int b) { return cost[a] > cost[b]; });
    pp.task_unit.assign(pp.n_tasks + 1, 0);
    size_t pos = 0;
    for (int k = 0; k < pp.n_tasks; k++) {
        pp.task_unit[k] = (int)pos;
        pos += (size_t)(tstart[ord[k] + 1] - tstart[ord[k]]);
    }
    pp.task_unit[pp.n_tasks] = (int)pos;
    pp.n_units = pos;
}

// Mixed form: work list (pair counts, scan, fill) then the contraction over
// chunks of items and the per-node reduction.  node_terms is returned in *hs.
mwgpu_status run_mixed(mwgpu_ctx *ctx, const Level &lv, LevelStats *hs) {
    const mwgpu_oper *o = lv.o;
    const int n = lv.n;
    const DevMRA &m = o->mra;
    std::vector<long long> poff;
    pair_offsets(lv, poff);
    const long long np = poff[n];
    if (auto s = grow_buf(ctx, &ctx->d_pair_off, &ctx->pair_off_cap, n + 1)) return s;
    if (auto s = grow_buf(ctx, &ctx->d_pcounts, &ctx->pcounts_cap, np + 1)) return s;
    if (auto s = grow_buf(ctx, &ctx->d_item_off, &ctx->item_off_cap, np + 1)) return s;
    if (auto s = grow_buf(ctx, &ctx->d_scan, &ctx->scan_cap, scan_blocks(np + 1) + 2)) return s;
    if (auto s = grow_buf(ctx, &ctx->d_goff, &ctx->goff_cap, n + 1)) return s;
    MW_CK(cudaMemcpyAsync(ctx->d_pair_off, poff.data(), sizeof(long long) * (n + 1), cudaMemcpyHostToDevice, ctx->stream));
    LevelStats *dst = ctx->d_stats;
    const double *gnode = lv.gnode.empty() ? nullptr : ctx->d_gnode;
    launch_pairs_count(m, o->op, ctx->d_fs, ctx->d_gs, ctx->d_wtree, ctx->d_work, ctx->d_pair_off, n, np, ctx->d_gthr, ctx->d_pcounts,
                       &dst->components, &dst->band_nodes, ctx->d_err, ctx->stream, nullptr, nullptr, gnode);
    long long *d_total = ctx->d_scan + (ctx->scan_cap - 1);
    launch_scan(ctx->d_pcounts, ctx->d_item_off, np, ctx->d_scan, d_total, ctx->stream);
    launch_gather_goff(ctx->d_item_off, ctx->d_pair_off, n, ctx->d_goff, ctx->stream);
    ctx->launches += 5;
    // the pencil units depend on the topology only: built on the host while the
    // device counts the work list, uploaded behind it
    const bool pencil = use_pencil(lv);
    static thread_local PencilPlan pp;  // rebuilt every level, its host vectors kept between levels
    if (pencil) {
        pencil_build(lv, pp, kLevelPencilCfg);
        const long long nu = (long long)pp.n_units;
        if (auto s = grow_buf(ctx, &ctx->d_units, &ctx->units_cap, std::max(nu, 1LL))) return s;
        if (auto s = grow_buf(ctx, &ctx->d_task_unit, &ctx->task_unit_cap, pp.n_tasks + 1)) return s;
        if (auto s = grow_buf(ctx, &ctx->d_pen_begin, &ctx->pen_begin_cap, n + 1)) return s;
        const size_t pneed = (size_t)std::max(pp.n_tasks, 1) * 8 * (size_t)o->mra.kp1_d;
        if (pneed > ctx->pen_partial_cap) {
            if (ctx->d_pen_partial) cudaFree(ctx->d_pen_partial);
            ctx->d_pen_partial = nullptr;
            ctx->pen_partial_cap = std::max(pneed, 2 * ctx->pen_partial_cap);
            if (auto s = dev_alloc(ctx, &ctx->d_pen_partial, ctx->pen_partial_cap)) return s;
        }
        if (!ctx->d_pen_counter)
            if (auto s = dev_alloc(ctx, &ctx->d_pen_counter, 1)) return s;
        if (nu > 0) {
            // through a page-locked staging buffer (a copy from pageable memory
            // blocks the host at a fraction of the link's rate); the previous
            // level's copy out of it ended at that level's stream synchronisation
            if ((size_t)nu > ctx->h_units_cap) {
                const size_t cap = std::max((size_t)nu, 2 * ctx->h_units_cap);
                if (ctx->h_units) cudaFreeHost(ctx->h_units);
                ctx->h_units = nullptr;
                ctx->h_units_cap = 0;
                if (cudaHostAlloc((void **)&ctx->h_units, sizeof(PencilUnit) * cap, cudaHostAllocDefault) == cudaSuccess)
                    ctx->h_units_cap = cap;
                else
                    (void)cudaGetLastError(), ctx->h_units = nullptr;
            }
            std::vector<PencilUnit> pageable;
            PencilUnit *hu = ctx->h_units;
            if (!hu) {
                pageable.resize(nu);
                hu = pageable.data();
            }
            pp.emit(hu);
            MW_CK(cudaMemcpyAsync(ctx->d_units, hu, sizeof(PencilUnit) * nu, cudaMemcpyHostToDevice, ctx->stream));
            if (!ctx->h_units) MW_CK(cudaStreamSynchronize(ctx->stream));
        }
        MW_CK(cudaMemcpyAsync(ctx->d_task_unit, pp.task_unit.data(), sizeof(int) * (pp.n_tasks + 1), cudaMemcpyHostToDevice, ctx->stream));
        MW_CK(cudaMemcpyAsync(ctx->d_pen_begin, pp.pen_begin.data(), sizeof(int) * (n + 1), cudaMemcpyHostToDevice, ctx->stream));
    }
    std::vector<long long> offs(n + 1);
    MW_CK(cudaMemcpyAsync(offs.data(), ctx->d_goff, sizeof(long long) * (n + 1), cudaMemcpyDeviceToHost, ctx->stream));
    MW_CK(cudaStreamSynchronize(ctx->stream));
    const long long total = offs[n];
    if (total > 0x7fffffffLL) {
        ctx->err = "work list of more than 2^31 items";
        return MWGPU_ERR_BAD_ARG;
    }
    if (total > ctx->items_cap) {
        for (WorkItem **p : {&ctx->d_items, &ctx->d_items_cm}) {
            if (*p) cudaFree(*p);
            *p = nullptr;
        }
        ctx->items_cap = std::max(total, 2 * ctx->items_cap);
        if (auto s = dev_alloc(ctx, &ctx->d_items, (size_t)ctx->items_cap)) return s;
        if (auto s = dev_alloc(ctx, &ctx->d_items_cm, (size_t)ctx->items_cap)) return s;
    }
    // cell-major items from the builder, then term-major per output node
    const bool order = term_order_supported(o->op.n_terms);
    launch_pairs_fill(m, o->op, ctx->d_fs, ctx->d_gs, ctx->d_wtree, ctx->d_work, ctx->d_pair_off, n, np, ctx->d_gthr, ctx->d_pcounts, ctx->d_item_off,
                      order ? ctx->d_items_cm : ctx->d_items, ctx->items_cap, ctx->d_err, ctx->stream, nullptr, nullptr, gnode);
    if (order) launch_order_terms(ctx->d_goff, n, ctx->d_items_cm, ctx->d_items, o->op.n_terms, ctx->d_err, ctx->stream);
    ctx->launches += 1 + (order ? 1 : 0);
    // pencil path: the items of the wider terms stay with the item kernel (stable compaction into d_items_cm)
    const WorkItem *kitems = ctx->d_items;
    if (pencil) {
        if (auto s = grow_buf(ctx, &ctx->d_keep, &ctx->keep_cap, n + 1)) return s;
        if (auto s = grow_buf(ctx, &ctx->d_keep_off, &ctx->keep_off_cap, n + 1)) return s;
        if (auto s = grow_buf(ctx, &ctx->d_scan, &ctx->scan_cap, std::max(scan_blocks(np + 1), scan_blocks(n + 1)) + 2)) return s;
        launch_keep_items(m, o->op, ctx->d_gs, ctx->d_wtree, ctx->d_work, ctx->d_goff, n, ctx->d_items, ctx->d_keep, ctx->stream,
                          mwgpu::kPencilCfgW[kLevelPencilCfg]);
        launch_scan(ctx->d_keep, ctx->d_keep_off, n, ctx->d_scan, ctx->d_scan + (ctx->scan_cap - 1), ctx->stream);
        launch_keep_fill(m, o->op, ctx->d_gs, ctx->d_wtree, ctx->d_work, ctx->d_goff, ctx->d_keep_off, n, ctx->d_items, ctx->d_items_cm,
                         ctx->stream, mwgpu::kPencilCfgW[kLevelPencilCfg]);
        ctx->launches += 5;
        MW_CK(cudaMemcpyAsync(offs.data(), ctx->d_keep_off, sizeof(long long) * (n + 1), cudaMemcpyDeviceToHost, ctx->stream));
        kitems = ctx->d_items_cm;
        MW_CK(cudaStreamSynchronize(ctx->stream));
    }
    // chunks of about the same number of items, several waves of CTAs
    const long long kept = offs[n];
    long long per = std::max<long long>(8, (kept + kChunkTarget - 1) / kChunkTarget);
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
    // the tensor-core kernel only where every input tree carries its TF32 operands
    bool tc_ok = true;
    for (int t = 0; t < lv.nt; t++) tc_ok = tc_ok && lv.inps[t]->t.tc32 != nullptr;
    if (pencil) {
        // the wider terms' items (chunks; a chunk of an entry without kept items is empty), the pencils, then both sums
        launch_items(o->mra, o->op, ctx->d_fs, ctx->d_gs, ctx->d_wtree, ctx->d_work, ctx->d_chunks, nch, kitems, ctx->d_partial, ctx->d_err,
                     nullptr, nullptr, tc_ok ? ctx->d_tc_counter : nullptr, ctx->stream);
        launch_pencil_units(o->mra, ctx->d_fs, ctx->d_gs, ctx->d_wtree, ctx->d_work, ctx->d_units, (int)pp.n_units, ctx->d_err, ctx->stream);
        launch_pencil(o->op, ctx->d_fs, ctx->d_wtree, ctx->d_units, ctx->d_task_unit, pp.n_tasks, ctx->d_pen_partial, ctx->d_err,
                      ctx->d_pen_counter, ctx->stream, pencil_warps());
        launch_reduce_chunks(o->mra, ctx->d_gs, ctx->d_wtree, ctx->d_work, n, ctx->d_chunk_begin, ctx->d_partial, ctx->stream, nullptr,
                             ctx->d_pen_begin, ctx->d_pen_partial);
        ctx->launches += 4;
    } else {
        launch_contract_items(o->mra, o->op, ctx->d_fs, ctx->d_gs, ctx->d_wtree, ctx->d_work, n, ctx->d_chunks, nch, ctx->d_chunk_begin,
                              ctx->d_items, ctx->d_partial, ctx->d_err, tc_ok ? ctx->d_tc_counter : nullptr, ctx->stream);
        ctx->launches += 2;
    }
    // (the chunk arrays came from pageable memory: the copies read them before returning)
    hs->node_terms = (unsigned long long)total;
    return MWGPU_OK;
}

mwgpu_status make_tree(mwgpu_ctx *ctx, const mwgpu_mra_desc *mra, const mwgpu_tree_desc *d, bool input, mwgpu_tree **out) {
    MW_ARG(out && d && d->n_nodes > 0 && d->idx && d->child0, "invalid tree descriptor");
    PhaseTrace trace(ctx, input ? "upload_tree" : "create_tree");
    auto *tr = new mwgpu_tree();
    tr->is_input = input;
    if (auto s = make_mra(ctx, mra, tr->mra, &tr->d_filt)) { free_tree(ctx, tr); return s; }
    tr->h_filt.assign(mra->filters, mra->filters + 8 * tr->mra.K * tr->mra.K);
    DevTree &t = tr->t;
    const int n = d->n_nodes;
    const size_t nc = 8 * (size_t)tr->mra.kp1_d;
    t.n_real = n;
    t.cap_real = input ? n : std::max(n, 512);  // output trees grow by the split step: room for a few levels
    t.n_gen = 0;
    t.cap_gen = 0;
    int tot = t.cap_real;
    tr->h_idx.resize(n);
    tr->h_child0.assign(d->child0, d->child0 + n);
    for (int i = 0; i < n; i++) tr->h_idx[i] = make_int4(d->idx[4 * i], d->idx[4 * i + 1], d->idx[4 * i + 2], d->idx[4 * i + 3]);
    mwgpu_status s;
    if ((s = pool_alloc(ctx, &t.idx, tot)) || (s = pool_alloc(ctx, &t.coefs, (size_t)tot * nc)) || (s = pool_alloc(ctx, &t.norms, (size_t)tot * 8)) ||
        (s = pool_alloc(ctx, &t.child0, tot))) {
        free_tree(ctx, tr);
        return s;
    }
    trace.mark("alloc");
    MW_CK(cudaMemcpyAsync(t.idx, tr->h_idx.data(), sizeof(int4) * n, cudaMemcpyHostToDevice, ctx->stream));
    MW_CK(cudaMemcpyAsync(t.child0, d->child0, sizeof(int) * n, cudaMemcpyHostToDevice, ctx->stream));
    // page-locked host coefficients of an input tree are read by a kernel that
    // writes the FP64 array and its FP32 copy in one pass
    const double *hdev = nullptr;
    const bool hin = input && d->coefs && host_in_supported(d->coefs, (size_t)n * nc, &hdev);
    if (d->coefs && !hin) MW_CK(cudaMemcpyAsync(t.coefs, d->coefs, sizeof(double) * n * nc, cudaMemcpyHostToDevice, ctx->stream));
    else if (!d->coefs) MW_CK(cudaMemsetAsync(t.coefs, 0, sizeof(double) * tot * nc, ctx->stream));
    trace.mark("coefs");
    if (input) {
        // FP32 copy read by the mixed form
        if ((s = pool_alloc(ctx, &t.coefs32, (size_t)n * nc))) { free_tree(ctx, tr); return s; }
        if (hin) launch_host_in(hdev, t.coefs, t.coefs32, (size_t)n * nc, ctx->stream);
        else launch_to_float(t.coefs, t.coefs32, (size_t)n * nc, ctx->stream);
        ctx->launches++;
        // TF32 hi / lo operands of the tensor-core x step (order 7; made below, once the norms are there)
        if (mwgpu::tc_supported(tr->mra.K) && n > 0)
            if ((s = pool_alloc(ctx, &t.tc32, (size_t)n * mwgpu::kTcNodeFloats))) { free_tree(ctx, tr); return s; }
    }
    if (d->norms) {
        MW_CK(cudaMemcpyAsync(t.norms, d->norms, sizeof(double) * n * 8, cudaMemcpyHostToDevice, ctx->stream));
    } else if (d->coefs) {
        std::vector<int> all(n);
        for (int i = 0; i < n; i++) all[i] = i;
        if ((s = ensure_work(ctx, n))) { free_tree(ctx, tr); return s; }
        MW_CK(cudaMemcpyAsync(ctx->d_work, all.data(), sizeof(int) * n, cudaMemcpyHostToDevice, ctx->stream));
        launch_node_norms(tr->mra, t, ctx->d_work, n, ctx->stream);
        ctx->launches++;
    } else {
        MW_CK(cudaMemsetAsync(t.norms, 0, sizeof(double) * tot * 8, ctx->stream));
    }
    if (input && t.tc32) {
        mwgpu::launch_tc_tree_layout(t, 0, n, ctx->stream);
        ctx->launches++;
    }
    trace.mark("fp32_norms");
    // only input trees are looked up by node index (band cells, GenNode
    // ancestors); output trees are addressed by position
    if (input && (s = rebuild_hash(ctx, tr, n))) { free_tree(ctx, tr); return s; }
    trace.mark("hash");
    // the host arrays may be page-locked, so the copies run asynchronously:
    // they are read in full before the call returns
    if (!input) MW_CK(cudaStreamSynchronize(ctx->stream));
    *out = tr;
    return MWGPU_OK;
}

void free_tree(mwgpu_ctx *ctx, mwgpu_tree *tr) {
    if (!tr) return;
    DevTree &t = tr->t;
    for (void *p : {(void *)t.idx, (void *)t.coefs, (void *)t.norms, (void *)t.child0, (void *)t.gcoefs, (void *)t.coefs32, (void *)t.gcoefs32, (void *)t.tc32, (void *)t.gtc32,
                    (void *)t.hkeys, (void *)t.hvals, (void *)tr->d_filt})
        pool_free(ctx, p);
    delete tr;
}

}  // namespace

namespace {

// GenNodes the operator bands of the work entries need, every tree at once
// (MWTree::getNode, MWTree.cpp:340-352); ctx->d_work / d_wtree hold the entries.
mwgpu_status gen_pass(mwgpu_ctx *ctx, const Level &lv, std::vector<int> &pcount, unsigned long long &gen_total) {
    const mwgpu_oper *o = lv.o;
    const int nt = lv.nt;
    // GenNodes follow the level's precision mode (FP32 products in the mixed
    // form); ones made in the other mode are dropped first, so that a result
    // does not depend on which applies ran on the tree before (trees held by
    // a plan keep theirs: the plan remakes them on every execution)
    const bool fp32 = ctx->precision == MWGPU_PREC_MIXED;
    for (int t = 0; t < nt; t++) {
        mwgpu_tree *inp = lv.inps[t];
        if (inp->t.n_gen > 0 && inp->gen_prec != ctx->precision && inp->plans == 0) {
            inp->t.n_gen = 0;
            if (auto s = rebuild_hash(ctx, inp, inp->t.n_real)) return s;
        }
    }
    pcount.assign(nt, 0);
    for (int attempt = 0; attempt < 8; attempt++) {
        if (auto s = ensure_pending(ctx, std::max(ctx->phcap, 1 << 16), std::max(ctx->pcap, 1 << 15), nt)) return s;
        MW_CK(cudaMemsetAsync(ctx->d_pkeys, 0xFF, sizeof(NodeKey) * ctx->phcap * nt, ctx->stream));
        MW_CK(cudaMemsetAsync(ctx->d_pcount, 0, sizeof(int) * nt, ctx->stream));
        for (int t = 0; t < nt; t++) {
            const int b = lv.seg[t], e = lv.seg[t + 1];
            if (b == e) continue;
            launch_band_missing(o->mra, lv.op(), lv.inps[t]->t, lv.outs[t]->t, ctx->d_work + b, e - b, ctx->d_pkeys + (size_t)t * ctx->phcap,
                                ctx->d_pvals + (size_t)t * ctx->phcap, ctx->phcap, ctx->d_plist + (size_t)t * ctx->pcap, ctx->d_pcount + t,
                                ctx->pcap, ctx->d_err, ctx->stream);
            ctx->launches++;
        }
        int herr = 0;
        MW_CK(cudaMemcpyAsync(pcount.data(), ctx->d_pcount, sizeof(int) * nt, cudaMemcpyDeviceToHost, ctx->stream));
        MW_CK(cudaMemcpyAsync(&herr, ctx->d_err, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
        MW_CK(cudaStreamSynchronize(ctx->stream));
        if (herr & DE_RANGE) { ctx->err = "band index outside the lookup range"; return MWGPU_ERR_INTERNAL; }
        const bool hfull = herr & DE_HASH_FULL;
        const int pmax = *std::max_element(pcount.begin(), pcount.end());
        if (!hfull && pmax <= ctx->pcap) break;
        MW_CK(cudaMemsetAsync(ctx->d_err, 0, sizeof(int), ctx->stream));
        if (auto s = ensure_pending(ctx, hfull ? ctx->phcap * 4 : next_pow2(4LL * pmax), std::max(pmax + 1024, ctx->pcap), nt)) return s;
        if (attempt == 7) { ctx->err = "pending GenNode set did not fit"; return MWGPU_ERR_OOM; }
    }
    gen_total = 0;
    for (int t = 0; t < nt; t++) {
        if (pcount[t] == 0) continue;
        mwgpu_tree *inp = lv.inps[t];
        DevTree &f = inp->t;
        if (auto s = grow_gen(ctx, inp, f.n_gen + pcount[t])) return s;
        if (2LL * (f.n_real + f.n_gen + pcount[t]) + 16 > f.hcap)
            if (auto s = rebuild_hash(ctx, inp, (long long)f.n_real + f.n_gen + pcount[t])) return s;
        const NodeKey *pl = ctx->d_plist + (size_t)t * ctx->pcap;
        if (fp32 && !std::getenv("MWGPU_GEN_PER_NODE")) {
            // GenNodes by parent (k_gen_family32): families formed on the device
            const int n = pcount[t];
            long long fcap = 64;
            while (fcap < 2LL * n + 16) fcap *= 2;
            if (auto s = grow_buf(ctx, &ctx->d_fkeys, &ctx->fkeys_cap, fcap)) return s;
            if (auto s = grow_buf(ctx, &ctx->d_fvals, &ctx->fvals_cap, fcap)) return s;
            if (auto s = grow_buf(ctx, &ctx->d_famid, &ctx->famid_cap, n)) return s;
            if (auto s = grow_buf(ctx, &ctx->d_fam_keys, &ctx->fam_keys_cap, n)) return s;
            if (auto s = grow_buf(ctx, &ctx->d_fam_slots, &ctx->fam_slots_cap, 8LL * n)) return s;
            if (auto s = grow_buf(ctx, &ctx->d_fam_count, &ctx->fam_count_cap, 1)) return s;
            MW_CK(cudaMemsetAsync(ctx->d_fkeys, 0xFF, sizeof(NodeKey) * fcap, ctx->stream));
            MW_CK(cudaMemsetAsync(ctx->d_fam_slots, 0xFF, sizeof(int) * 8 * (size_t)n, ctx->stream));
            MW_CK(cudaMemsetAsync(ctx->d_fam_count, 0, sizeof(int), ctx->stream));
            launch_gen_families(inp->mra, pl, n, ctx->d_fkeys, ctx->d_fvals, (int)fcap, ctx->d_famid, ctx->d_fam_keys, ctx->d_fam_slots,
                                ctx->d_fam_count, ctx->d_err, ctx->stream);
            launch_gen_family32(inp->mra, f, ctx->d_fam_keys, ctx->d_fam_slots, n, ctx->d_fam_count, f.n_gen, false, ctx->d_err, ctx->stream);
            ctx->launches += 4;
        } else {
            launch_gen_nodes(inp->mra, f, pl, pcount[t], f.n_gen, ctx->d_err, ctx->stream, false, fp32);
            ctx->launches++;
        }
        launch_gen_insert(inp->mra, f, pl, pcount[t], f.n_gen, ctx->d_err, ctx->stream);
        ctx->launches++;
        f.n_gen += pcount[t];
        gen_total += pcount[t];
        inp->gen_prec = ctx->precision;
    }
    return MWGPU_OK;
}

// Everything of one level after validation: GenNodes of every input tree,
// per-tree thresholds, the contraction and the norm gather.
mwgpu_status level_run(mwgpu_ctx *ctx, Level &lv, const double *sqnorms, double prec, double *norms_out, mwgpu_level_stats *stats,
                       std::vector<int> *pcount_out = nullptr) {
    const mwgpu_oper *o = lv.o;
    const int n = lv.n, nt = lv.nt;
    PhaseTrace tr(ctx, "apply_level");
    if (auto s = ensure_work(ctx, n)) return s;
    if (auto s = ensure_trees(ctx, nt)) return s;
    MW_CK(cudaEventRecord(ctx->ev0, ctx->stream));
    MW_CK(cudaMemcpyAsync(ctx->d_work, lv.node.data(), sizeof(int) * n, cudaMemcpyHostToDevice, ctx->stream));
    MW_CK(cudaMemcpyAsync(ctx->d_wtree, lv.tree.data(), sizeof(int) * n, cudaMemcpyHostToDevice, ctx->stream));
    MW_CK(cudaMemsetAsync(ctx->d_err, 0, sizeof(int), ctx->stream));
    MW_CK(cudaMemsetAsync(ctx->d_stats, 0, sizeof(LevelStats), ctx->stream));
    std::vector<int> pcount;
    unsigned long long gen_total = 0;
    tr.mark("setup");
    if (auto s = gen_pass(ctx, lv, pcount, gen_total)) return s;
    tr.mark("gen");
    if (pcount_out) *pcount_out = pcount;
    // per-tree screening threshold (ConvolutionCalculator.cpp:240-246); with
    // per-node factors (apply.cpp:221-228) one threshold per work entry,
    // prec * precFac * sqrt(|g|^2 / nTerms) in the reference's order
    lv.gthr.assign(nt, 0.0);
    for (int t = 0; t < nt; t++) {
        double g = sqnorms[t];
        if (g > 0.0) g = prec * 1.0 * std::sqrt(g / (double)o->op.n_terms);
        lv.gthr[t] = g;
    }
    lv.gnode.clear();
    if (!lv.pfac.empty()) {
        lv.gnode.resize(n);
        for (int j = 0; j < n; j++) {
            double g = sqnorms[lv.tree[j]];
            if (g > 0.0) g = prec * lv.pfac[j] * std::sqrt(g / (double)o->op.n_terms);
            lv.gnode[j] = g;
        }
        if (auto s = grow_buf(ctx, &ctx->d_gnode, &ctx->gnode_cap, n)) return s;
        MW_CK(cudaMemcpyAsync(ctx->d_gnode, lv.gnode.data(), sizeof(double) * n, cudaMemcpyHostToDevice, ctx->stream));
    }
    lv.fs.resize(nt);
    lv.gs.resize(nt);
    for (int t = 0; t < nt; t++) {
        lv.fs[t] = lv.inps[t]->t;
        lv.gs[t] = lv.outs[t]->t;
    }
    MW_CK(cudaMemcpyAsync(ctx->d_fs, lv.fs.data(), sizeof(DevTree) * nt, cudaMemcpyHostToDevice, ctx->stream));
    MW_CK(cudaMemcpyAsync(ctx->d_gs, lv.gs.data(), sizeof(DevTree) * nt, cudaMemcpyHostToDevice, ctx->stream));
    MW_CK(cudaMemcpyAsync(ctx->d_gthr, lv.gthr.data(), sizeof(double) * nt, cudaMemcpyHostToDevice, ctx->stream));
    LevelStats mixed_nt{};
    if (lv.band_dir >= 0) {
        MW_CK(cudaEventRecord(ctx->ev1, ctx->stream));
        launch_deriv(o->mra, lv.op(), lv.inps[0]->t, lv.outs[0]->t, ctx->d_work, n, lv.deriv_order, ctx->d_stats, ctx->d_err, ctx->stream);
        ctx->launches++;
    } else if (ctx->precision == MWGPU_PREC_MIXED) {
        if (auto s = run_mixed(ctx, lv, &mixed_nt)) return s;
    } else {
        MW_CK(cudaEventRecord(ctx->ev1, ctx->stream));
        for (int t = 0; t < nt; t++) {
            const int b = lv.seg[t], e = lv.seg[t + 1];
            if (b == e) continue;
            launch_contract_fp64(o->mra, o->op, lv.inps[t]->t, lv.outs[t]->t, ctx->d_work + b, e - b, lv.gthr[t], ctx->d_stats, ctx->d_err,
                                 ctx->stream, nullptr, nullptr, lv.gnode.empty() ? nullptr : ctx->d_gnode + b);
            ctx->launches++;
        }
    }
    MW_CK(cudaGetLastError());
    tr.mark("contract");
    MW_CK(cudaEventRecord(ctx->ev2, ctx->stream));
    LevelStats hs{};
    MW_CK(cudaMemcpyAsync(&hs, ctx->d_stats, sizeof(LevelStats), cudaMemcpyDeviceToHost, ctx->stream));
    std::vector<double> staged;
    if (norms_out) {
        if (auto s = grow_buf(ctx, &ctx->d_nstage, &ctx->nstage_cap, 8LL * n)) return s;
        launch_gather_norms(ctx->d_gs, ctx->d_wtree, ctx->d_work, n, ctx->d_nstage, ctx->stream);
        ctx->launches++;
        staged.resize((size_t)8 * n);
        MW_CK(cudaMemcpyAsync(staged.data(), ctx->d_nstage, sizeof(double) * 8 * n, cudaMemcpyDeviceToHost, ctx->stream));
    }
    if (auto s = check_err(ctx, "apply_level")) return s;
    tr.mark("result");
    if (norms_out)
        for (int j = 0; j < n; j++) std::memcpy(norms_out + 8 * (size_t)lv.order[j], &staged[8 * (size_t)j], sizeof(double) * 8);
    if (ctx->precision == MWGPU_PREC_MIXED && lv.band_dir < 0) hs.node_terms = mixed_nt.node_terms;
    if (stats) {
        stats->node_terms = hs.node_terms;
        stats->components = hs.components;
        stats->band_nodes = hs.band_nodes;
        stats->gen_nodes = gen_total;
        float ms = 0.f;
        cudaEventElapsedTime(&ms, ctx->ev0, ctx->ev2);
        stats->device_ms = ms;
        cudaEventElapsedTime(&ms, ctx->ev1, ctx->ev2);
        stats->contract_ms = ms;
    }
    return MWGPU_OK;
}

// TopDown / BottomUp of nt trees with the same MRA: one launch per depth for
// all trees (MWTree.cpp:166-216).
mwgpu_status transform_impl(mwgpu_ctx *ctx, int nt, mwgpu_tree *const *trees, int direction, int overwrite) {
    MW_ARG(direction == MWGPU_TOPDOWN || direction == MWGPU_BOTTOMUP, "invalid transform direction");
    MW_ARG(!(direction == MWGPU_BOTTOMUP && !overwrite), "BottomUp transform always overwrites");
    for (int t = 0; t < nt; t++) {
        MW_ARG(trees[t], "null tree");
        MW_ARG(trees[t]->h_filt == trees[0]->h_filt && trees[t]->mra.root_scale == trees[0]->mra.root_scale, "trees of a batch need the same MRA");
        for (int u = 0; u < t; u++) MW_ARG(trees[u] != trees[t], "trees of a batch must be distinct");
    }
    cudaSetDevice(ctx->device);
    // parents per depth (breadth-first order from the roots), all trees
    std::vector<std::vector<int2>> levels;
    for (int t = 0; t < nt; t++) {
        const mwgpu_tree *tr = trees[t];
        const int n = tr->t.n_real;
        for (int i = 0; i < n; i++) {
            const int depth = tr->h_idx[i].x - tr->mra.root_scale;
            if (tr->h_child0[i] < 0 || depth < 0) continue;
            if ((int)levels.size() <= depth) levels.resize(depth + 1);
            levels[depth].push_back(make_int2(t, i));
        }
    }
    std::vector<int> flat, ftree;
    std::vector<std::pair<int, int>> ranges;
    for (auto &l : levels) {
        ranges.push_back({(int)flat.size(), (int)l.size()});
        for (auto &e : l) {
            ftree.push_back(e.x);
            flat.push_back(e.y);
        }
    }
    if (flat.empty()) return MWGPU_OK;
    if ((int)flat.size() > ctx->list_cap) {
        if (ctx->d_list) cudaFree(ctx->d_list);
        if (ctx->d_ltree) cudaFree(ctx->d_ltree);
        ctx->d_list = ctx->d_ltree = nullptr;
        ctx->list_cap = (int)flat.size() * 2;
        if (auto s = dev_alloc(ctx, &ctx->d_list, ctx->list_cap)) return s;
        if (auto s = dev_alloc(ctx, &ctx->d_ltree, ctx->list_cap)) return s;
    }
    MW_CK(cudaMemcpyAsync(ctx->d_list, flat.data(), sizeof(int) * flat.size(), cudaMemcpyHostToDevice, ctx->stream));
    const DevTree *ts = nullptr;
    const int *ptree = nullptr;
    std::vector<DevTree> h_ts;
    if (nt > 1) {
        if (auto s = ensure_trees(ctx, nt)) return s;
        for (int t = 0; t < nt; t++) h_ts.push_back(trees[t]->t);
        MW_CK(cudaMemcpyAsync(ctx->d_gs, h_ts.data(), sizeof(DevTree) * nt, cudaMemcpyHostToDevice, ctx->stream));
        MW_CK(cudaMemcpyAsync(ctx->d_ltree, ftree.data(), sizeof(int) * ftree.size(), cudaMemcpyHostToDevice, ctx->stream));
        ts = ctx->d_gs;
        ptree = ctx->d_ltree;
    }
    const DevMRA &m = trees[0]->mra;
    const DevTree &t0 = trees[0]->t;
    const bool fp32 = ctx->precision == MWGPU_PREC_MIXED;  // FP32 filter products in the mixed form
    if (direction == MWGPU_TOPDOWN) {
        for (auto &r : ranges) {
            launch_mw_down(m, t0, ts, ptree ? ptree + r.first : nullptr, ctx->d_list + r.first, r.second, overwrite != 0, ctx->stream, fp32);
            ctx->launches += r.second > 0;
        }
    } else {
        for (int l = (int)ranges.size() - 1; l >= 0; l--) {
            launch_mw_up(m, t0, ts, ptree ? ptree + ranges[l].first : nullptr, ctx->d_list + ranges[l].first, ranges[l].second, ctx->stream, fp32);
            ctx->launches += ranges[l].second > 0;
        }
    }
    MW_CK(cudaGetLastError());
    MW_CK(cudaStreamSynchronize(ctx->stream));
    return MWGPU_OK;
}

// Validation shared by the single-tree, batched and planned level calls;
// groups the work entries by tree (stable).
mwgpu_status make_level(mwgpu_ctx *ctx, const mwgpu_oper *o, int nt, mwgpu_tree *const *inps, mwgpu_tree *const *outs, const int *work_tree,
                        const int *node_ix, int n, Level &lv) {
    MW_ARG(o, "invalid operator or trees");
    for (int t = 0; t < nt; t++) {
        MW_ARG(inps[t] && outs[t] && inps[t]->is_input && !outs[t]->is_input, "invalid operator or trees");
        MW_ARG(inps[t]->mra.K == o->op.K && outs[t]->mra.K == o->op.K, "order mismatch");
        for (int u = 0; u < t; u++) MW_ARG(inps[u] != inps[t] && outs[u] != outs[t], "trees of a batch must be distinct");
        MW_ARG(inps[t]->plans == 0 && outs[t]->plans == 0, "tree is held by a plan (destroy the plan first)");
    }
    MW_ARG(n >= 0 && (n == 0 || node_ix), "invalid node list");
    if (ctx->precision == MWGPU_PREC_MIXED && !mixed_supported(o->op.K)) {
        ctx->err = "mixed form supports orders k = 1..9";
        return MWGPU_ERR_BAD_ARG;
    }
    lv.o = o;
    lv.nt = nt;
    lv.inps = inps;
    lv.outs = outs;
    lv.n = n;
    lv.seg.assign(nt + 1, 0);
    for (int i = 0; i < n; i++) {
        const int t = work_tree ? work_tree[i] : 0;
        MW_ARG(t >= 0 && t < nt, "work tree index out of range");
        MW_ARG(node_ix[i] >= 0 && node_ix[i] < outs[t]->t.n_real, "node index out of range");
        lv.seg[t + 1]++;
    }
    for (int t = 0; t < nt; t++) lv.seg[t + 1] += lv.seg[t];
    lv.node.resize(n);
    lv.tree.resize(n);
    lv.order.resize(n);
    std::vector<int> pos(lv.seg.begin(), lv.seg.end() - 1);
    for (int i = 0; i < n; i++) {
        const int t = work_tree ? work_tree[i] : 0;
        const int j = pos[t]++;
        lv.node[j] = node_ix[i];
        lv.tree[j] = t;
        lv.order[j] = i;
    }
    return MWGPU_OK;
}

mwgpu_status level_entry(mwgpu_ctx *ctx, const mwgpu_oper *o, int nt, mwgpu_tree *const *inps, mwgpu_tree *const *outs, const int *work_tree,
                         const int *node_ix, int n, double prec, const double *sqnorms, double *norms_out, mwgpu_level_stats *stats,
                         const double *prec_fac = nullptr) {
    Level lv;
    if (auto s = make_level(ctx, o, nt, inps, outs, work_tree, node_ix, n, lv)) return s;
    if (prec_fac) {
        for (int i = 0; i < n; i++) MW_ARG(prec_fac[i] >= 0.0, "precision factors must be >= 0 (1 / the largest norm of the precision trees)");
        lv.pfac.resize(n);
        for (int j = 0; j < n; j++) lv.pfac[j] = prec_fac[lv.order[j]];
    }
    cudaSetDevice(ctx->device);
    if (stats) std::memset(stats, 0, sizeof(*stats));
    if (n == 0) return MWGPU_OK;
    return level_run(ctx, lv, sqnorms, prec, norms_out, stats);
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
        cudaMalloc(&ctx->d_tc_counter, sizeof(int)) != cudaSuccess) {
        g_init_error = std::string("device initialisation failed: ") + cudaGetErrorString(cudaGetLastError());
        delete ctx;
        return MWGPU_ERR_DEVICE;
    }
    cudaMemset(ctx->d_err, 0, sizeof(int));
    // freed tree storage stays cached for reuse up to a quarter of the device
    // (a batch of input trees is re-uploaded every step); an allocation that
    // fails returns the whole cache to the device first
    size_t free_b = 0, total_b = 0;
    if (cudaMemGetInfo(&free_b, &total_b) == cudaSuccess && total_b > 0) ctx->pool.limit = std::max<size_t>(size_t(1) << 30, total_b / 4);
    *out = ctx;
    return MWGPU_OK;
}

mwgpu_status mwgpu_destroy(mwgpu_ctx *ctx) {
    if (!ctx) return MWGPU_ERR_BAD_ARG;
    cudaSetDevice(ctx->device);
    cudaStreamSynchronize(ctx->stream);
    for (void *p : {(void *)ctx->d_err, (void *)ctx->d_stats, (void *)ctx->d_tc_counter, (void *)ctx->d_proj, (void *)ctx->d_work, (void *)ctx->d_pkeys, (void *)ctx->d_fkeys, (void *)ctx->d_fam_keys, (void *)ctx->d_fvals, (void *)ctx->d_famid, (void *)ctx->d_fam_slots, (void *)ctx->d_fam_count, (void *)ctx->d_pvals,
                    (void *)ctx->d_plist, (void *)ctx->d_pcount, (void *)ctx->d_list, (void *)ctx->d_items, (void *)ctx->d_items_cm, (void *)ctx->d_chunks,
                    (void *)ctx->d_chunk_begin, (void *)ctx->d_partial, (void *)ctx->d_pair_off, (void *)ctx->d_pcounts,
                    (void *)ctx->d_item_off, (void *)ctx->d_scan, (void *)ctx->d_goff, (void *)ctx->d_wtree, (void *)ctx->d_fs,
                    (void *)ctx->d_gs, (void *)ctx->d_gthr, (void *)ctx->d_nstage, (void *)ctx->d_ltree, (void *)ctx->d_units,
                    (void *)ctx->d_task_unit, (void *)ctx->d_pen_partial, (void *)ctx->d_pen_begin, (void *)ctx->d_keep, (void *)ctx->d_keep_off,
                    (void *)ctx->d_pen_counter, (void *)ctx->d_gnode})
        if (p) cudaFree(p);
    pool_trim(ctx);
    for (auto &e : ctx->marks)
        if (e) cudaEventDestroy(e);
    if (ctx->d_scrub) cudaFree(ctx->d_scrub);
    if (ctx->d_arena) cudaFree(ctx->d_arena);
    if (ctx->h_units) cudaFreeHost(ctx->h_units);
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
    // FP32 copy for the mixed form, each K x K block transposed (row i = O(i, 0..K-1))
    std::vector<float> blk32(node * 4 * K2);
    for (size_t q = 0; q < blk32.size(); q++) {
        const size_t b = q / K2, ij = q % K2;  // column-major O(i, j) at i + K j
        blk32[b * K2 + (ij / K) + K * (ij % K)] = (float)d->blocks[q];
    }
    // per operator node an upper bound of its 4 component norms (screening bound)
    std::vector<float> nmax(node);
    for (size_t q = 0; q < node; q++) {
        double mx = 0.0;
        for (int c = 0; c < 4; c++) mx = std::max(mx, d->norms[q * 4 + c]);
        nmax[q] = std::nextafter((float)mx, INFINITY);
    }
    std::vector<TermRow> trows((size_t)rows * T);
    for (int dd = 0; dd < rows; dd++)
        for (int ti = 0; ti < T; ti++) {
            const int i = order[(size_t)dd * T + ti];
            TermRow &r = trows[(size_t)dd * T + ti];
            r.term = i;
            r.L0 = dep_L[(size_t)i * rows + dd];
            r.off = dep_off[(size_t)i * rows + dd];
            r.bw_max = bw[((size_t)i * rows + dd) * 5 + 4];
            for (int c = 0; c < 4; c++) r.wd[c] = bw[((size_t)i * rows + dd) * 5 + c];
        }
    TermRow *p_trows;
    // pair screening table: per depth and band cell the largest per-term bound
    std::vector<int> pb_off(rows, -1);
    std::vector<float> pb;
    for (int dd = 0; dd <= maxDepth && dd < rows; dd++) {
        const int W = band_max[dd];
        if (W < 0) continue;
        const int nw = 2 * W + 1;
        const size_t cells = (size_t)nw * nw * nw;
        if (pb.size() + cells > ((size_t)1 << 26)) break;
        std::vector<double> tab(cells, 0.0), v(nw);
        for (int t = 0; t < T; t++) {
            const int off = dep_off[(size_t)t * rows + dd], L0 = dep_L[(size_t)t * rows + dd];
            const int *w = &bw[((size_t)t * rows + dd) * 5];
            if (off < 0 || w[4] < 0) continue;
            int fm = 1;
            for (int c = 0; c < 4; c++) fm = std::max(fm, w[c] < 0 ? 1 : 2 * w[c] + 1);
            const double f3 = (double)fm * fm * fm;
            for (int l = -W; l <= W; l++) v[l + W] = (std::abs(l) <= L0 && std::abs(l) <= w[4]) ? (double)nmax[off + l + L0] : 0.0;
            for (int a = 0; a < nw; a++) {
                if (v[a] == 0.0) continue;
                for (int b = 0; b < nw; b++) {
                    const double ab = v[a] * v[b] * f3;
                    if (ab == 0.0) continue;
                    double *row = &tab[((size_t)a * nw + b) * nw];
                    for (int c = 0; c < nw; c++) row[c] = std::max(row[c], ab * v[c]);
                }
            }
        }
        pb_off[dd] = (int)pb.size();
        for (double x : tab) pb.push_back(x > 0.0 ? std::nextafter((float)(x * (1.0 + 1e-14)), INFINITY) : 0.0f);
    }
    float *p_pb;
    int *p_pboff;
    std::vector<float> nrm32(node * 4);
    for (size_t q = 0; q < nrm32.size(); q++) nrm32[q] = (float)d->norms[q];
    float *p_blk32, *p_nmax, *p_nrm32;
    mwgpu_status s;
    if ((s = up(&p_td, d->depth, T)) || (s = up(&p_off, dep_off.data(), dep_off.size())) || (s = up(&p_L, dep_L.data(), dep_L.size())) ||
        (s = up(&p_bw, bw.data(), bw.size())) || (s = up(&p_bsz, bsz.data(), bsz.size())) || (s = up(&p_bm, band_max.data(), band_max.size())) ||
        (s = up(&p_ord, order.data(), order.size())) || (s = up(&p_blk, d->blocks, node * 4 * K2)) || (s = up(&p_nrm, d->norms, node * 4)) ||
        (s = up(&p_blk32, blk32.data(), blk32.size())) || (s = up(&p_nmax, nmax.data(), nmax.size())) ||
        (s = up(&p_nrm32, nrm32.data(), nrm32.size())) || (s = up(&p_trows, trows.data(), trows.size())) ||
        (s = up(&p_pb, pb.data(), pb.size())) || (s = up(&p_pboff, pb_off.data(), pb_off.size()))) {
        for (void *p : o->allocs) cudaFree(p);
        pool_free(ctx, o->d_filt);
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
    o->op.norm_max = p_nmax;
    o->op.norms32 = p_nrm32;
    o->op.term_rows = p_trows;
    o->op.pair_bound = p_pb;
    o->op.pair_bound_off = p_pboff;
    o->op.n_nodes = (int)node;
    o->op.btc = nullptr;
    o->op.btc_stack = nullptr;
    o->op.pfrag = nullptr;
    o->op.band_dir = -1;
    o->op.band_dir_w = 0;
    if (mwgpu::tc_supported(K)) {
        // B operands of the tensor-core contraction per operator node (band zeroed) + a zero record
        std::vector<int4> ninfo(node);
        size_t nd = 0;
        for (int t = 0; t < T; t++)
            for (int dd = 0; dd < d->depth[t]; dd++) {
                const int L = dep_L[(size_t)t * rows + dd];
                for (int l = -L; l <= L; l++) ninfo[nd++] = make_int4(t, dd, l, 0);
            }
        int4 *p_ni = nullptr;
        float *p_btc = nullptr;
        if ((s = up(&p_ni, ninfo.data(), ninfo.size())) || (s = dev_alloc(ctx, &p_btc, (node + 1) * (size_t)mwgpu::kTcFormFloats))) {
            for (void *p : o->allocs) cudaFree(p);
            pool_free(ctx, o->d_filt);
            delete o;
            return s;
        }
        o->allocs.push_back((void *)p_btc);
        mwgpu::launch_tc_oper_forms(o->op, p_ni, (int)node, p_btc, ctx->stream);
        MW_CK(cudaStreamSynchronize(ctx->stream));
        o->op.btc = p_btc;
    }
    if (mwgpu::pencil_supported(K)) {
        // stacked x-step forms of the pencil contraction, per configuration c:
        // per depth the terms of band width <= kPencilCfgW[c] (after the wider
        // ones in term-row order), in groups of kPencilGroup, for every x slot
        // (l_x = 0, -k, +k) the group's terms with band width >= k
        constexpr int G5 = mwgpu::kPencilGroup, NK = mwgpu::kPencilMaxL + 1, NS = mwgpu::kPencilSlots;
        const int G = (T + G5 - 1) / G5;
        o->pen_groups = G;
        std::vector<mwgpu::PencilFormJob> jobs;
        long long fl = 0;
        for (int c = 0; c < mwgpu::kPencilCfgs; c++) {
            mwgpu_oper::PenCfg &pc = o->pen[c];
            const int maxw = mwgpu::kPencilCfgW[c];
            pc.tk.assign((size_t)rows * NK, 0);
            pc.r0.assign(rows, 0);
            pc.form.assign((size_t)rows * G * NS, -1);
            pc.nform.assign((size_t)rows * G * NS, 0);
            for (int dd = 0; dd < rows; dd++) {
                int r0 = 0;
                for (int ti = 0; ti < T; ti++) {
                    const TermRow &tr = trows[(size_t)dd * T + ti];
                    if (tr.off < 0) continue;
                    if (tr.bw_max > maxw) {
                        r0++;
                        continue;
                    }
                    for (int k = 0; k < NK; k++)
                        if (tr.bw_max >= k) pc.tk[(size_t)dd * NK + k]++;
                }
                pc.r0[dd] = r0;
                const int t0 = pc.tk[(size_t)dd * NK];
                for (int q = 0; q * G5 < t0; q++)
                    for (int b = 0; b < NS; b++) {
                        const int k = (b + 1) / 2, lx = b == 0 ? 0 : ((b & 1) ? -k : k);
                        const int nt = std::max(0, std::min(G5, pc.tk[(size_t)dd * NK + k] - G5 * q));
                        if (nt <= 0) continue;
                        const size_t ix = ((size_t)dd * G + q) * NS + b;
                        pc.form[ix] = fl;
                        pc.nform[ix] = (short)nt;
                        jobs.push_back({dd, r0 + G5 * q, lx, nt, fl});
                        fl += 32LL * ((24 * nt + 15) / 16 * 16);
                    }
            }
        }
        mwgpu::PencilFormJob *p_jobs = nullptr;
        float *p_stack = nullptr;
        if ((s = up(&p_jobs, jobs.data(), jobs.size())) || (s = dev_alloc(ctx, &p_stack, (size_t)std::max(fl, 1LL)))) {
            for (void *p : o->allocs) cudaFree(p);
            pool_free(ctx, o->d_filt);
            delete o;
            return s;
        }
        o->allocs.push_back((void *)p_stack);
        mwgpu::launch_stack_forms(o->op, p_jobs, (int)jobs.size(), p_stack, ctx->stream);
        MW_CK(cudaStreamSynchronize(ctx->stream));
        MW_CK(cudaGetLastError());
        o->op.btc_stack = p_stack;
        // the y / z operator fragments of the consumers, per (depth, term row, l in the pencil band)
        float *p_frag = nullptr;
        if ((s = dev_alloc(ctx, &p_frag, (size_t)rows * T * mwgpu::kPencilFragL * mwgpu::kPencilFragFloats))) {
            for (void *p : o->allocs) cudaFree(p);
            pool_free(ctx, o->d_filt);
            delete o;
            return s;
        }
        o->allocs.push_back((void *)p_frag);
        mwgpu::launch_pencil_frags(o->op, rows, p_frag, ctx->stream);
        MW_CK(cudaStreamSynchronize(ctx->stream));
        MW_CK(cudaGetLastError());
        o->op.pfrag = p_frag;
    }
    *out = o;
    return MWGPU_OK;
}

mwgpu_status mwgpu_free_operator(mwgpu_ctx *ctx, mwgpu_oper *o) {
    if (!ctx || !o) return MWGPU_ERR_BAD_ARG;
    for (void *p : o->allocs) cudaFree(p);
    pool_free(ctx, o->d_filt);
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
    MW_ARG(tr->plans == 0, "tree is held by a plan (destroy the plan first)");
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
    // (copies from pageable memory read their source before returning)
    return MWGPU_OK;
}

mwgpu_status mwgpu_tree_size(const mwgpu_tree *tr, int *n) {
    if (!tr || !n) return MWGPU_ERR_BAD_ARG;
    *n = tr->t.n_real;
    return MWGPU_OK;
}

mwgpu_status mwgpu_free_tree(mwgpu_ctx *ctx, mwgpu_tree *tr) {
    if (!ctx || !tr) return MWGPU_ERR_BAD_ARG;
    MW_ARG(tr->plans == 0, "tree is held by a plan (destroy the plan first)");
    cudaSetDevice(ctx->device);
    free_tree(ctx, tr);
    return MWGPU_OK;
}

mwgpu_status mwgpu_apply_level(mwgpu_ctx *ctx, const mwgpu_oper *o, mwgpu_tree *inp, mwgpu_tree *out, const int *node_ix, int n,
                               double prec, double out_sqnorm, double *norms_out, mwgpu_level_stats *stats) {
    if (!ctx) return MWGPU_ERR_BAD_ARG;
    mwgpu_tree *inps[1] = {inp}, *outs[1] = {out};
    return level_entry(ctx, o, 1, inps, outs, nullptr, node_ix, n, prec, &out_sqnorm, norms_out, stats);
}

mwgpu_status mwgpu_apply_level_scaled(mwgpu_ctx *ctx, const mwgpu_oper *o, mwgpu_tree *inp, mwgpu_tree *out, const int *node_ix, int n,
                                      double prec, double out_sqnorm, const double *prec_fac, double *norms_out, mwgpu_level_stats *stats) {
    if (!ctx) return MWGPU_ERR_BAD_ARG;
    MW_ARG(n == 0 || prec_fac, "null precision factors");
    mwgpu_tree *inps[1] = {inp}, *outs[1] = {out};
    return level_entry(ctx, o, 1, inps, outs, nullptr, node_ix, n, prec, &out_sqnorm, norms_out, stats, prec_fac);
}

mwgpu_status mwgpu_combine_level(mwgpu_ctx *ctx, int op, int n_in, mwgpu_tree *const *inps, const double *c, const double *cv_map, const double *vc_map,
                                 mwgpu_tree *out, const int *node_ix, int n, double *norms_out) {
    if (!ctx) return MWGPU_ERR_BAD_ARG;
    MW_ARG(op == MWGPU_COMBINE_ADD || op == MWGPU_COMBINE_MULTIPLY, "invalid combine operation");
    MW_ARG(n_in >= 1 && inps && c && cv_map && vc_map, "invalid inputs or basis tables");
    MW_ARG(out && !out->is_input, "the result is an output tree");
    for (int j = 0; j < n_in; j++) MW_ARG(inps[j] && inps[j]->is_input && inps[j]->mra.K == out->mra.K && inps[j]->plans == 0, "invalid input tree");
    MW_ARG(n >= 0 && (n == 0 || node_ix), "invalid node list");
    for (int i = 0; i < n; i++) MW_ARG(node_ix[i] >= 0 && node_ix[i] < out->t.n_real, "node index out of range");
    cudaSetDevice(ctx->device);
    if (n == 0) return MWGPU_OK;
    // GenNodes of the inputs where the output has a node they lack (getNode):
    // the band machinery with a one-cell band, one segment per input
    mwgpu_oper cell{};
    cell.mra = out->mra;
    cell.op.band_dir = 0;
    cell.op.band_dir_w = 0;
    Level lv;
    lv.o = &cell;
    lv.nt = n_in;
    lv.inps = inps;
    std::vector<mwgpu_tree *> outs(n_in, out);
    lv.outs = outs.data();
    lv.n = n * n_in;
    lv.band_dir = 0;
    lv.band_w = 0;
    lv.seg.resize(n_in + 1);
    for (int j = 0; j <= n_in; j++) lv.seg[j] = j * n;
    for (int j = 0; j < n_in; j++)
        for (int i = 0; i < n; i++) {
            lv.node.push_back(node_ix[i]);
            lv.tree.push_back(j);
        }
    const int prev = ctx->precision;
    ctx->precision = MWGPU_PREC_FP64;
    auto restore = [&](mwgpu_status s) {
        ctx->precision = prev;
        return s;
    };
    if (auto s = ensure_work(ctx, lv.n)) return restore(s);
    if (auto s = ensure_trees(ctx, n_in)) return restore(s);
    MW_CK(cudaMemcpyAsync(ctx->d_work, lv.node.data(), sizeof(int) * lv.n, cudaMemcpyHostToDevice, ctx->stream));
    MW_CK(cudaMemcpyAsync(ctx->d_wtree, lv.tree.data(), sizeof(int) * lv.n, cudaMemcpyHostToDevice, ctx->stream));
    MW_CK(cudaMemsetAsync(ctx->d_err, 0, sizeof(int), ctx->stream));
    std::vector<int> pcount;
    unsigned long long gen_total = 0;
    if (auto s = gen_pass(ctx, lv, pcount, gen_total)) return restore(s);
    ctx->precision = prev;
    std::vector<DevTree> fs(n_in);
    for (int j = 0; j < n_in; j++) fs[j] = inps[j]->t;
    const int K = out->mra.K;
    if (auto s = grow_buf(ctx, &ctx->d_proj, &ctx->proj_cap, (long long)n_in + 2LL * K * K)) return s;
    double *d_c = ctx->d_proj, *d_cv = d_c + n_in, *d_vc = d_cv + K * K;
    MW_CK(cudaMemcpyAsync(ctx->d_fs, fs.data(), sizeof(DevTree) * n_in, cudaMemcpyHostToDevice, ctx->stream));
    MW_CK(cudaMemcpyAsync(d_c, c, sizeof(double) * n_in, cudaMemcpyHostToDevice, ctx->stream));
    MW_CK(cudaMemcpyAsync(d_cv, cv_map, sizeof(double) * K * K, cudaMemcpyHostToDevice, ctx->stream));
    MW_CK(cudaMemcpyAsync(d_vc, vc_map, sizeof(double) * K * K, cudaMemcpyHostToDevice, ctx->stream));
    launch_combine(out->mra, op == MWGPU_COMBINE_MULTIPLY, ctx->d_fs, d_c, n_in, out->t, ctx->d_work, n, d_cv, d_vc, ctx->d_err, ctx->stream);
    ctx->launches++;
    if (norms_out) {
        if (auto s = grow_buf(ctx, &ctx->d_nstage, &ctx->nstage_cap, 8LL * n)) return s;
        std::vector<int> zeros(n, 0);
        MW_CK(cudaMemcpyAsync(ctx->d_wtree, zeros.data(), sizeof(int) * n, cudaMemcpyHostToDevice, ctx->stream));
        MW_CK(cudaMemcpyAsync(ctx->d_gs, &out->t, sizeof(DevTree), cudaMemcpyHostToDevice, ctx->stream));
        launch_gather_norms(ctx->d_gs, ctx->d_wtree, ctx->d_work, n, ctx->d_nstage, ctx->stream);
        ctx->launches++;
        MW_CK(cudaMemcpyAsync(norms_out, ctx->d_nstage, sizeof(double) * 8 * n, cudaMemcpyDeviceToHost, ctx->stream));
    }
    return check_err(ctx, "combine level");
}

// The level of a projection: the Gaussians (n_gauss > 0) evaluated on the
// device, or the function values the caller evaluated (values).
static mwgpu_status project_level(mwgpu_ctx *ctx, mwgpu_tree *tree, int n_gauss, const double *gauss, const double *values, const double *vc_map,
                                  const double *roots, const int *node_ix, int n, double *norms_out) {
    if (!ctx) return MWGPU_ERR_BAD_ARG;
    MW_ARG(tree && !tree->is_input, "projection writes an output tree");
    MW_ARG(n_gauss >= 0 && (n_gauss == 0 || gauss) && vc_map && roots, "invalid Gaussian list or basis tables");
    MW_ARG(n >= 0 && (n == 0 || node_ix), "invalid node list");
    MW_ARG(n == 0 || !values || n_gauss == 0, "Gaussians or values, not both");
    for (int i = 0; i < n; i++) MW_ARG(node_ix[i] >= 0 && node_ix[i] < tree->t.n_real, "node index out of range");
    cudaSetDevice(ctx->device);
    if (n == 0) return MWGPU_OK;
    const int K = tree->mra.K;
    const long long nval = values ? (long long)n * 8 * tree->mra.kp1_d : 0;
    const long long need = 5LL * std::max(n_gauss, 1) + (long long)K * K + K + nval;
    if (auto s = grow_buf(ctx, &ctx->d_proj, &ctx->proj_cap, need)) return s;
    if (auto s = ensure_work(ctx, n)) return s;
    double *d_g = ctx->d_proj, *d_vc = d_g + 5 * std::max(n_gauss, 1), *d_roots = d_vc + K * K, *d_val = d_roots + K;
    if (n_gauss > 0) MW_CK(cudaMemcpyAsync(d_g, gauss, sizeof(double) * 5 * n_gauss, cudaMemcpyHostToDevice, ctx->stream));
    if (values) MW_CK(cudaMemcpyAsync(d_val, values, sizeof(double) * nval, cudaMemcpyHostToDevice, ctx->stream));
    MW_CK(cudaMemcpyAsync(d_vc, vc_map, sizeof(double) * K * K, cudaMemcpyHostToDevice, ctx->stream));
    MW_CK(cudaMemcpyAsync(d_roots, roots, sizeof(double) * K, cudaMemcpyHostToDevice, ctx->stream));
    MW_CK(cudaMemcpyAsync(ctx->d_work, node_ix, sizeof(int) * n, cudaMemcpyHostToDevice, ctx->stream));
    launch_project(tree->mra, tree->t, ctx->d_work, n, d_g, n_gauss, d_vc, d_roots, ctx->stream, values ? d_val : nullptr);
    ctx->launches++;
    if (norms_out) {
        if (auto s = grow_buf(ctx, &ctx->d_nstage, &ctx->nstage_cap, 8LL * n)) return s;
        if (auto s = ensure_trees(ctx, 1)) return s;
        std::vector<int> zeros(n, 0);
        MW_CK(cudaMemcpyAsync(ctx->d_wtree, zeros.data(), sizeof(int) * n, cudaMemcpyHostToDevice, ctx->stream));
        MW_CK(cudaMemcpyAsync(ctx->d_gs, &tree->t, sizeof(DevTree), cudaMemcpyHostToDevice, ctx->stream));
        launch_gather_norms(ctx->d_gs, ctx->d_wtree, ctx->d_work, n, ctx->d_nstage, ctx->stream);
        ctx->launches++;
        MW_CK(cudaMemcpyAsync(norms_out, ctx->d_nstage, sizeof(double) * 8 * n, cudaMemcpyDeviceToHost, ctx->stream));
    }
    MW_CK(cudaGetLastError());
    MW_CK(cudaStreamSynchronize(ctx->stream));
    return MWGPU_OK;
}

mwgpu_status mwgpu_project_level(mwgpu_ctx *ctx, mwgpu_tree *tree, int n_gauss, const double *gauss, const double *vc_map, const double *roots,
                                 const int *node_ix, int n, double *norms_out) {
    return project_level(ctx, tree, n_gauss, gauss, nullptr, vc_map, roots, node_ix, n, norms_out);
}

mwgpu_status mwgpu_project_level_values(mwgpu_ctx *ctx, mwgpu_tree *tree, const double *values, const double *vc_map, const double *roots,
                                        const int *node_ix, int n, double *norms_out) {
    if (!ctx) return MWGPU_ERR_BAD_ARG;
    MW_ARG(n == 0 || values, "null values");
    return project_level(ctx, tree, 0, nullptr, values, vc_map, roots, node_ix, n, norms_out);
}

mwgpu_status mwgpu_apply_derivative(mwgpu_ctx *ctx, const mwgpu_oper *o, mwgpu_tree *inp, mwgpu_tree *out, const int *node_ix, int n, int dir,
                                    int order, mwgpu_level_stats *stats) {
    if (!ctx) return MWGPU_ERR_BAD_ARG;
    MW_ARG(dir >= 0 && dir < 3, "derivative direction must be 0, 1 or 2");
    MW_ARG(order >= 1, "derivative order must be >= 1");
    MW_ARG(o && o->op.n_terms == 1, "a derivative operator has one term");
    Level lv;
    mwgpu_tree *ins[1] = {inp}, *outs[1] = {out};
    // the FP64 form: GenNodes in FP64 as well, whatever the context's mode
    const int prev = ctx->precision;
    ctx->precision = MWGPU_PREC_FP64;
    mwgpu_status s = make_level(ctx, o, 1, ins, outs, nullptr, node_ix, n, lv);
    if (s == MWGPU_OK) {
        // DerivativeCalculator::makeOperBand: width = the operator's largest band width
        int w = -1;
        for (int b : o->band_max) w = std::max(w, b);
        lv.band_dir = dir;
        lv.band_w = std::max(w, 0);
        lv.deriv_order = order;
        cudaSetDevice(ctx->device);
        if (stats) std::memset(stats, 0, sizeof(*stats));
        const double zero = 0.0;
        if (n > 0) s = level_run(ctx, lv, &zero, 0.0, nullptr, stats);
    }
    ctx->precision = prev;
    return s;
}

mwgpu_status mwgpu_apply_level_batch(mwgpu_ctx *ctx, const mwgpu_oper *o, int n_trees, mwgpu_tree *const *inps, mwgpu_tree *const *outs,
                                     const int *work_tree, const int *node_ix, int n, double prec, const double *out_sqnorms,
                                     double *norms_out, mwgpu_level_stats *stats) {
    if (!ctx) return MWGPU_ERR_BAD_ARG;
    MW_ARG(n_trees >= 1 && inps && outs && out_sqnorms, "invalid tree arrays");
    MW_ARG(n == 0 || work_tree, "null work_tree");
    return level_entry(ctx, o, n_trees, inps, outs, work_tree, node_ix, n, prec, out_sqnorms, norms_out, stats);
}

mwgpu_status mwgpu_transform(mwgpu_ctx *ctx, mwgpu_tree *tr, int direction, int overwrite) {
    if (!ctx || !tr) return MWGPU_ERR_BAD_ARG;
    mwgpu_tree *trees[1] = {tr};
    return transform_impl(ctx, 1, trees, direction, overwrite);
}

mwgpu_status mwgpu_transform_batch(mwgpu_ctx *ctx, int n_trees, mwgpu_tree *const *trees, int direction, int overwrite) {
    if (!ctx) return MWGPU_ERR_BAD_ARG;
    MW_ARG(n_trees >= 1 && trees, "invalid tree array");
    return transform_impl(ctx, n_trees, trees, direction, overwrite);
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

mwgpu_status mwgpu_download_nodes(mwgpu_ctx *ctx, const mwgpu_tree *tr, int n, const int *ids, double *coefs, double *norms) {
    if (!ctx || !tr) return MWGPU_ERR_BAD_ARG;
    MW_ARG(n >= 0 && (n == 0 || ids), "null node list");
    for (int j = 0; j < n; j++) MW_ARG(ids[j] >= 0 && ids[j] < tr->t.n_real, "node id out of range");
    if (n == 0 || (!coefs && !norms)) return MWGPU_OK;
    cudaSetDevice(ctx->device);
    const size_t nc = 8 * (size_t)tr->mra.kp1_d;
    if (auto s = ensure_work(ctx, n)) return s;
    DevTree stage{};
    if (auto s = pool_alloc(ctx, &stage.coefs, (size_t)n * nc)) return s;
    if (auto s = pool_alloc(ctx, &stage.norms, (size_t)n * 8)) {
        pool_free(ctx, stage.coefs);
        return s;
    }
    MW_CK(cudaMemcpyAsync(ctx->d_work, ids, sizeof(int) * n, cudaMemcpyHostToDevice, ctx->stream));
    launch_copy_nodes(tr->t, stage, ctx->d_work, nullptr, n, (int)nc, ctx->stream);
    ctx->launches++;
    cudaError_t e = cudaSuccess;
    if (coefs) e = cudaMemcpyAsync(coefs, stage.coefs, sizeof(double) * n * nc, cudaMemcpyDeviceToHost, ctx->stream);
    if (norms && e == cudaSuccess) e = cudaMemcpyAsync(norms, stage.norms, sizeof(double) * n * 8, cudaMemcpyDeviceToHost, ctx->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
    pool_free(ctx, stage.coefs);
    pool_free(ctx, stage.norms);
    MW_CK(e);
    return MWGPU_OK;
}

mwgpu_status mwgpu_sync(mwgpu_ctx *ctx) {
    if (!ctx) return MWGPU_ERR_BAD_ARG;
    MW_CK(cudaStreamSynchronize(ctx->stream));
    return MWGPU_OK;
}

mwgpu_status mwgpu_tree_update_coefs(mwgpu_ctx *ctx, mwgpu_tree *tr, const double *coefs, const double *norms) {
    if (!ctx || !tr || !coefs) return MWGPU_ERR_BAD_ARG;
    MW_ARG(tr->is_input, "only input trees take new coefficients");
    cudaSetDevice(ctx->device);
    PhaseTrace trace(ctx, "update_coefs");
    DevTree &t = tr->t;
    const int n = t.n_real;
    const size_t nc = 8 * (size_t)tr->mra.kp1_d;
    // page-locked host arrays are read by a kernel that writes both device copies
    const double *hdev = nullptr;
    if (host_in_supported(coefs, (size_t)n * nc, &hdev)) {
        launch_host_in(hdev, t.coefs, t.coefs32, (size_t)n * nc, ctx->stream);
        ctx->launches += 1;
        trace.mark("coefs_fp32");
    } else {
        MW_CK(cudaMemcpyAsync(t.coefs, coefs, sizeof(double) * n * nc, cudaMemcpyHostToDevice, ctx->stream));
        trace.mark("coefs");
        launch_to_float(t.coefs, t.coefs32, (size_t)n * nc, ctx->stream);
        ctx->launches += 1;
    }
    if (norms) {
        MW_CK(cudaMemcpyAsync(t.norms, norms, sizeof(double) * n * 8, cudaMemcpyHostToDevice, ctx->stream));
    } else {
        std::vector<int> all(n);
        for (int i = 0; i < n; i++) all[i] = i;
        if (auto s = ensure_work(ctx, n)) return s;
        MW_CK(cudaMemcpyAsync(ctx->d_work, all.data(), sizeof(int) * n, cudaMemcpyHostToDevice, ctx->stream));
        launch_node_norms(tr->mra, t, ctx->d_work, n, ctx->stream);
        ctx->launches++;
    }
    if (t.tc32) {
        mwgpu::launch_tc_tree_layout(t, 0, n, ctx->stream);
        ctx->launches++;
    }
    MW_CK(cudaStreamSynchronize(ctx->stream));
    trace.mark("fp32_tf32_norms");
    // GenNodes hold values of the old coefficients: a plan recomputes its own,
    // otherwise they are dropped and made again by the next level
    if (tr->plans == 0 && t.n_gen > 0) {
        t.n_gen = 0;
        return rebuild_hash(ctx, tr, n);
    }
    return MWGPU_OK;
}

mwgpu_status mwgpu_tree_clear_generated(mwgpu_ctx *ctx, mwgpu_tree *tr) {
    if (!ctx || !tr) return MWGPU_ERR_BAD_ARG;
    MW_ARG(tr->is_input, "only input trees hold GenNodes");
    MW_ARG(tr->plans == 0, "tree is held by a plan (destroy the plan first)");
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
    MW_ARG(inp->plans == 0 && out->plans == 0, "tree is held by a plan (destroy the plan first)");
    // GenNodes made by a mixed-form level hold FP32-product values; the FP64
    // contraction must not read them
    MW_ARG(inp->t.n_gen == 0 || inp->gen_prec == MWGPU_PREC_FP64,
           "the input tree's GenNodes were made by the mixed form: run mwgpu_apply_level in FP64 on these nodes first");
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

// ---------------------------------------------------------------------------
// Level plans: one level over a batch of trees whose node lists stay fixed
// (apply with maxIter = 0 onto given output grids, or the repeated applies of
// a fixed-grid SCF loop).  What depends only on the topology is prepared once:
// the GenNode keys and slots, the band pair offsets, buffer capacities and the
// chunk length (chosen by timing candidates).  What depends on values -- the
// GenNode coefficients, screening and work list, contraction, reduction,
// norms and the transforms -- is captured as one CUDA graph and recomputed on
// every execution.
// ---------------------------------------------------------------------------
struct mwgpu_plan {
    const mwgpu_oper *o = nullptr;
    int nt = 0, n = 0, precision = 0, flags = 0;
    std::vector<mwgpu_tree *> inps, outs;
    std::vector<int> seg;
    std::vector<double> gthr;
    // precision scaled per output node (the precTrees form of apply): one
    // factor per grouped entry, and the thresholds made from them; empty: 1
    std::vector<double> pfac, gnode;
    std::vector<void *> allocs;
    int *d_work = nullptr, *d_wtree = nullptr;
    DevTree *d_fs = nullptr, *d_gs = nullptr;
    double *d_gthr = nullptr;
    long long np = 0;
    long long *d_pair_off = nullptr, *d_item_off = nullptr, *d_scan = nullptr, *d_goff = nullptr, *d_coff = nullptr, *d_cscan = nullptr;
    long long scan_n = 0, cscan_n = 0;
    int *d_pcounts = nullptr, *d_ccount = nullptr;
    WorkItem *d_items = nullptr, *d_items_cm = nullptr;  // term-major / cell-major (null: no reordering)
    long long items_cap = 0;
    int4 *d_chunks = nullptr;
    int *d_chunk_begin = nullptr, *d_nchunks = nullptr, *d_counter = nullptr;
    int chunks_cap = 0;
    double *d_partial = nullptr;
    LevelStats *d_stats = nullptr;
    int *d_err = nullptr;
    unsigned long long *d_stamps = nullptr;  // level start, contraction start / end, level end, pencil kernel start / end (ns)
    std::vector<NodeKey *> d_gkeys;
    std::vector<int> gcount;
    // mixed form: the GenNodes grouped by parent (keys, 8 slots per parent)
    std::vector<NodeKey *> d_fam_keys;
    std::vector<int *> d_fam_slots;
    std::vector<int> fcount;
    int *d_list = nullptr, *d_ltree = nullptr;
    std::vector<std::pair<int, int>> ranges;
    long long per = 0;
    int grid = 0;
    cudaEvent_t e1 = nullptr, e2 = nullptr;  // autotuning timers (outside the graph)
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    unsigned long long launches_per_exec = 0;
    // autotuning candidates: chunk length, schedule (1: pencil + item kernels,
    // 0: item kernel alone) and the contraction's time
    std::vector<double> tune_ms;
    std::vector<long long> tune_per;
    std::vector<int> tune_pencil;
    int tune_choice = -1;
    // pencil contraction (unscreened order-7 levels): kept items of the item
    // kernel (their offsets per entry), units and task sums
    bool pencil = false;
    // the pencil configuration covers every term of every entry (pen_all_ok);
    // pen_all: the executions leave the item list unfilled.  Set for the
    // captured graph only: the autotuning candidates of the item kernel alone
    // read the list that the passes before them fill
    bool pen_all_ok = false, pen_all = false;
    int pen_warps = kPencilWarpsDefault;     // consumer warps of the pencil kernel
    int *d_keep = nullptr;
    long long *d_keep_off = nullptr, *d_kscan = nullptr;
    long long kscan_n = 0;
    PencilUnit *d_units = nullptr;
    int n_units = 0, n_tasks = 0;
    int *d_task_unit = nullptr, *d_pen_begin = nullptr, *d_pen_counter = nullptr;
    double *d_pen_partial = nullptr;
    unsigned long long pen_node_terms = 0;   // last checked execution: node-terms of the pencil kernel
    double pen_ms = 0.0;                     // and its device time
};

namespace {

template <class T> mwgpu_status plan_alloc(mwgpu_ctx *ctx, mwgpu_plan *pl, T **p, size_t n) {
    if (auto s = dev_alloc(ctx, p, n)) return s;
    pl->allocs.push_back((void *)*p);
    return MWGPU_OK;
}

void plan_free(mwgpu_plan *pl) {
    if (!pl) return;
    if (pl->exec) cudaGraphExecDestroy(pl->exec);
    if (pl->graph) cudaGraphDestroy(pl->graph);
    for (cudaEvent_t e : {pl->e1, pl->e2})
        if (e) cudaEventDestroy(e);
    for (void *p : pl->allocs) cudaFree(p);
    delete pl;
}

// chunking + contraction + reduction of a planned mixed level (no host sync)
// reduce: the whole contraction with the reduction (the level); otherwise the
// contraction alone between the plan's events e1 and e2 (autotuning)
void plan_contract(mwgpu_ctx *ctx, mwgpu_plan *pl, long long per, bool reduce) {
    const mwgpu_oper *o = pl->o;
    cudaStream_t st = ctx->stream;
    // with the pencil contraction the item kernel takes the compacted items of the wider terms
    const long long *goff = pl->pencil ? pl->d_keep_off : pl->d_goff;
    const WorkItem *items = pl->pencil ? pl->d_items_cm : pl->d_items;
    launch_chunk_count(goff, pl->n, per, pl->d_ccount, st);
    launch_scan(pl->d_ccount, pl->d_coff, pl->n, pl->d_cscan, pl->d_cscan + (pl->cscan_n - 1), st);
    launch_chunk_fill(goff, pl->d_coff, pl->n, per, pl->d_chunks, pl->d_chunk_begin, pl->chunks_cap, pl->d_nchunks, pl->d_err, st);
    cudaMemsetAsync(pl->d_counter, 0, sizeof(int), st);
    if (reduce) launch_stamp(pl->d_stamps + 1, st);
    else cudaEventRecord(pl->e1, st);
    bool tc_ok = true;
    for (int t = 0; t < pl->nt; t++) tc_ok = tc_ok && pl->inps[t]->t.tc32 != nullptr;
    launch_items(o->mra, o->op, pl->d_fs, pl->d_gs, pl->d_wtree, pl->d_work, pl->d_chunks, pl->grid, items, pl->d_partial, pl->d_err,
                 pl->d_nchunks, pl->d_counter, tc_ok ? pl->d_counter + 1 : nullptr, st);
    if (pl->pencil) {
        launch_pencil_units(o->mra, pl->d_fs, pl->d_gs, pl->d_wtree, pl->d_work, pl->d_units, pl->n_units, pl->d_err, st);
        if (reduce) launch_stamp(pl->d_stamps + 4, st);
        launch_pencil(o->op, pl->d_fs, pl->d_wtree, pl->d_units, pl->d_task_unit, pl->n_tasks, pl->d_pen_partial, pl->d_err, pl->d_pen_counter,
                      st, pl->pen_warps);
        if (reduce) launch_stamp(pl->d_stamps + 5, st);
        ctx->launches += reduce ? 5 : 3;
    }
    if (reduce)
        launch_reduce_chunks(o->mra, pl->d_gs, pl->d_wtree, pl->d_work, pl->n, pl->d_chunk_begin, pl->d_partial, st, nullptr,
                             pl->pencil ? pl->d_pen_begin : nullptr, pl->pencil ? pl->d_pen_partial : nullptr);
    ctx->launches += 6 + (reduce ? 2 : 0);
}

// the whole level on the context stream, without host synchronisation
void plan_sequence(mwgpu_ctx *ctx, mwgpu_plan *pl) {
    const mwgpu_oper *o = pl->o;
    cudaStream_t st = ctx->stream;
    launch_stamp(pl->d_stamps + 0, st);
    ctx->launches++;
    cudaMemsetAsync(pl->d_err, 0, sizeof(int), st);
    cudaMemsetAsync(pl->d_stats, 0, sizeof(LevelStats), st);
    // GenNode values from the current input coefficients (slots fixed at plan time)
    for (int t = 0; t < pl->nt; t++) {
        if (pl->gcount[t] == 0) continue;
        if (!pl->fcount.empty() && pl->fcount[t] > 0)
            launch_gen_family32(pl->inps[t]->mra, pl->inps[t]->t, pl->d_fam_keys[t], pl->d_fam_slots[t], pl->fcount[t], nullptr, 0, true, pl->d_err,
                                st);
        else
            launch_gen_nodes(pl->inps[t]->mra, pl->inps[t]->t, pl->d_gkeys[t], pl->gcount[t], 0, pl->d_err, st, true,
                             pl->precision == MWGPU_PREC_MIXED);
        ctx->launches++;
    }
    if (pl->precision == MWGPU_PREC_MIXED) {
        LevelStats *dst = pl->d_stats;
        launch_pairs_count(o->mra, o->op, pl->d_fs, pl->d_gs, pl->d_wtree, pl->d_work, pl->d_pair_off, pl->n, pl->np, pl->d_gthr, pl->d_pcounts,
                           &dst->components, &dst->band_nodes, pl->d_err, st);
        launch_scan(pl->d_pcounts, pl->d_item_off, pl->np, pl->d_scan, pl->d_scan + (pl->scan_n - 1), st);
        launch_gather_goff(pl->d_item_off, pl->d_pair_off, pl->n, pl->d_goff, st, nullptr, pl->items_cap);
        // the count pass gives the node-terms and the screening statistics; the
        // items themselves only where the item kernel has terms to take
        const bool fill = !(pl->pencil && pl->pen_all);
        const bool ordered = term_order_supported(o->op.n_terms);
        if (fill) {
            launch_pairs_fill(o->mra, o->op, pl->d_fs, pl->d_gs, pl->d_wtree, pl->d_work, pl->d_pair_off, pl->n, pl->np, pl->d_gthr,
                              pl->d_pcounts, pl->d_item_off, ordered ? pl->d_items_cm : pl->d_items, pl->items_cap, pl->d_err, st);
            if (ordered) launch_order_terms(pl->d_goff, pl->n, pl->d_items_cm, pl->d_items, o->op.n_terms, pl->d_err, st);
        }
        ctx->launches += 5 + (fill ? 1 + (ordered ? 1 : 0) : 0);
        if (pl->pencil && fill) {
            launch_keep_items(o->mra, o->op, pl->d_gs, pl->d_wtree, pl->d_work, pl->d_goff, pl->n, pl->d_items, pl->d_keep, st,
                              mwgpu::kPencilCfgW[kPlanPencilCfg]);
            launch_scan(pl->d_keep, pl->d_keep_off, pl->n, pl->d_kscan, pl->d_kscan + (pl->kscan_n - 1), st);
            launch_keep_fill(o->mra, o->op, pl->d_gs, pl->d_wtree, pl->d_work, pl->d_goff, pl->d_keep_off, pl->n, pl->d_items, pl->d_items_cm, st,
                             mwgpu::kPencilCfgW[kPlanPencilCfg]);
            ctx->launches += 5;
        } else if (pl->pencil) {
            cudaMemsetAsync(pl->d_keep_off, 0, sizeof(long long) * (pl->n + 1), st);   // no item is left to the item kernel
        }
        plan_contract(ctx, pl, pl->per, true);
    } else {
        launch_stamp(pl->d_stamps + 1, st);
        ctx->launches++;
        for (int t = 0; t < pl->nt; t++) {
            const int b = pl->seg[t], e = pl->seg[t + 1];
            if (b == e) continue;
            launch_contract_fp64(o->mra, o->op, pl->inps[t]->t, pl->outs[t]->t, pl->d_work + b, e - b, pl->gthr[t], pl->d_stats, pl->d_err, st);
            ctx->launches++;
        }
    }
    launch_stamp(pl->d_stamps + 2, st);
    ctx->launches++;
    if (pl->flags & MWGPU_PLAN_TRANSFORMS) {
        const mwgpu_tree *t0 = pl->outs[0];
        for (auto &r : pl->ranges) {
            launch_mw_down(t0->mra, t0->t, pl->d_gs, pl->d_ltree + r.first, pl->d_list + r.first, r.second, false, st,
                           pl->precision == MWGPU_PREC_MIXED);
            ctx->launches += r.second > 0;
        }
        for (int l = (int)pl->ranges.size() - 1; l >= 0; l--) {
            launch_mw_up(t0->mra, t0->t, pl->d_gs, pl->d_ltree + pl->ranges[l].first, pl->d_list + pl->ranges[l].first, pl->ranges[l].second, st,
                         pl->precision == MWGPU_PREC_MIXED);
            ctx->launches += pl->ranges[l].second > 0;
        }
    }
    launch_stamp(pl->d_stamps + 3, st);
    ctx->launches++;
}

mwgpu_status plan_check(mwgpu_ctx *ctx, mwgpu_plan *pl, mwgpu_level_stats *stats) {
    int herr = 0;
    LevelStats hs{};
    long long total = 0;
    unsigned long long stamps[6] = {0, 0, 0, 0, 0, 0};
    long long kept = 0;
    MW_CK(cudaMemcpyAsync(stamps, pl->d_stamps, sizeof(stamps), cudaMemcpyDeviceToHost, ctx->stream));
    MW_CK(cudaMemcpyAsync(&herr, pl->d_err, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
    MW_CK(cudaMemcpyAsync(&hs, pl->d_stats, sizeof(LevelStats), cudaMemcpyDeviceToHost, ctx->stream));
    if (pl->precision == MWGPU_PREC_MIXED)
        MW_CK(cudaMemcpyAsync(&total, pl->d_goff + pl->n, sizeof(long long), cudaMemcpyDeviceToHost, ctx->stream));
    if (pl->pencil) MW_CK(cudaMemcpyAsync(&kept, pl->d_keep_off + pl->n, sizeof(long long), cudaMemcpyDeviceToHost, ctx->stream));
    MW_CK(cudaStreamSynchronize(ctx->stream));
    if (pl->pencil) {
        pl->pen_node_terms = (unsigned long long)(total - kept);
        pl->pen_ms = (double)(stamps[5] - stamps[4]) * 1e-6;
    }
    if (herr & DE_POOL_FULL) {
        ctx->err = "plan: the work list outgrew the planned capacity (input values changed the screening); create a new plan";
        return MWGPU_ERR_OOM;
    }
    if (herr) {
        ctx->err = "plan: device error flags " + std::to_string(herr);
        return MWGPU_ERR_INTERNAL;
    }
    if (stats) {
        std::memset(stats, 0, sizeof(*stats));
        stats->node_terms = pl->precision == MWGPU_PREC_MIXED ? (unsigned long long)total : hs.node_terms;
        stats->components = hs.components;
        stats->band_nodes = hs.band_nodes;
        unsigned long long g = 0;
        for (int c : pl->gcount) g += c;
        stats->gen_nodes = g;
        stats->device_ms = (double)(stamps[3] - stamps[0]) * 1e-6;
        stats->contract_ms = (double)(stamps[2] - stamps[1]) * 1e-6;
    }
    return MWGPU_OK;
}

}  // namespace

extern "C" mwgpu_status mwgpu_plan_create(mwgpu_ctx *ctx, const mwgpu_oper *o, int n_trees, mwgpu_tree *const *inps, mwgpu_tree *const *outs,
                                          const int *work_tree, const int *node_ix, int n, double prec, const double *out_sqnorms, int flags,
                                          mwgpu_plan **out) {
    if (!ctx) return MWGPU_ERR_BAD_ARG;
    MW_ARG(out && n_trees >= 1 && inps && outs && out_sqnorms, "invalid plan arguments");
    MW_ARG(n > 0, "a plan needs at least one node");
    *out = nullptr;
    Level lv;
    if (auto s = make_level(ctx, o, n_trees, inps, outs, work_tree, node_ix, n, lv)) return s;
    cudaSetDevice(ctx->device);
    if (flags & MWGPU_PLAN_TRANSFORMS) {
        // the transforms rewrite every node: the plan must compute all of them
        for (int t = 0; t < n_trees; t++) {
            const int cnt = lv.seg[t + 1] - lv.seg[t];
            MW_ARG(cnt == outs[t]->t.n_real, "a plan with transforms must compute every node of its output trees");
            std::vector<char> seen(outs[t]->t.n_real, 0);
            for (int j = lv.seg[t]; j < lv.seg[t + 1]; j++) {
                MW_ARG(!seen[lv.node[j]], "a node appears twice in the plan");
                seen[lv.node[j]] = 1;
            }
        }
    }
    for (int t = 0; t < n_trees; t++)
        MW_ARG(outs[t]->h_filt == outs[0]->h_filt && outs[t]->mra.root_scale == outs[0]->mra.root_scale, "trees of a plan need the same MRA");
    // a fresh GenNode set that belongs to the plan
    for (int t = 0; t < n_trees; t++)
        if (inps[t]->t.n_gen > 0) {
            inps[t]->t.n_gen = 0;
            if (auto s = rebuild_hash(ctx, inps[t], inps[t]->t.n_real)) return s;
        }
    // eager level: makes the GenNodes, gives the work-list size and the result
    std::vector<int> pcount;
    mwgpu_level_stats st0{};
    if (auto s = level_run(ctx, lv, out_sqnorms, prec, nullptr, &st0, &pcount)) return s;

    auto *pl = new mwgpu_plan();
    pl->o = o;
    pl->nt = n_trees;
    pl->n = n;
    pl->precision = ctx->precision;
    pl->flags = flags;
    pl->inps.assign(inps, inps + n_trees);
    pl->outs.assign(outs, outs + n_trees);
    pl->seg = lv.seg;
    pl->gthr = lv.gthr;
    auto fail = [&](mwgpu_status s) {
        plan_free(pl);
        return s;
    };
    mwgpu_status s;
    if ((s = plan_alloc(ctx, pl, &pl->d_work, n)) || (s = plan_alloc(ctx, pl, &pl->d_wtree, n)) || (s = plan_alloc(ctx, pl, &pl->d_fs, n_trees)) ||
        (s = plan_alloc(ctx, pl, &pl->d_gs, n_trees)) || (s = plan_alloc(ctx, pl, &pl->d_gthr, n_trees)) ||
        (s = plan_alloc(ctx, pl, &pl->d_stats, 1)) || (s = plan_alloc(ctx, pl, &pl->d_err, 1)) || (s = plan_alloc(ctx, pl, &pl->d_stamps, 6)))
        return fail(s);
    if (cudaEventCreate(&pl->e1) != cudaSuccess || cudaEventCreate(&pl->e2) != cudaSuccess) {
        ctx->err = "plan: event creation failed";
        return fail(MWGPU_ERR_DEVICE);
    }
    MW_CK(cudaMemcpyAsync(pl->d_work, lv.node.data(), sizeof(int) * n, cudaMemcpyHostToDevice, ctx->stream));
    MW_CK(cudaMemcpyAsync(pl->d_wtree, lv.tree.data(), sizeof(int) * n, cudaMemcpyHostToDevice, ctx->stream));
    MW_CK(cudaMemcpyAsync(pl->d_fs, lv.fs.data(), sizeof(DevTree) * n_trees, cudaMemcpyHostToDevice, ctx->stream));
    MW_CK(cudaMemcpyAsync(pl->d_gs, lv.gs.data(), sizeof(DevTree) * n_trees, cudaMemcpyHostToDevice, ctx->stream));
    MW_CK(cudaMemcpyAsync(pl->d_gthr, lv.gthr.data(), sizeof(double) * n_trees, cudaMemcpyHostToDevice, ctx->stream));
    // GenNode keys of every input tree (slots 0 .. count-1 after the reset above)
    pl->gcount = pcount;
    pl->d_gkeys.assign(n_trees, nullptr);
    for (int t = 0; t < n_trees; t++) {
        if (pcount[t] == 0) continue;
        if ((s = plan_alloc(ctx, pl, &pl->d_gkeys[t], pcount[t]))) return fail(s);
        MW_CK(cudaMemcpyAsync(pl->d_gkeys[t], ctx->d_plist + (size_t)t * ctx->pcap, sizeof(NodeKey) * pcount[t], cudaMemcpyDeviceToDevice,
                              ctx->stream));
    }
    // mixed form: GenNodes grouped by parent, so that the children of a parent
    // share its x and y steps (k_gen_family32); the slots stay those above
    if (pl->precision == MWGPU_PREC_MIXED && !std::getenv("MWGPU_GEN_PER_NODE")) {
        pl->fcount.assign(n_trees, 0);
        pl->d_fam_keys.assign(n_trees, nullptr);
        pl->d_fam_slots.assign(n_trees, nullptr);
        for (int t = 0; t < n_trees; t++) {
            if (pcount[t] == 0) continue;
            const DevMRA &m = pl->inps[t]->mra;
            std::vector<NodeKey> keys(pcount[t]);
            MW_CK(cudaMemcpyAsync(keys.data(), pl->d_gkeys[t], sizeof(NodeKey) * pcount[t], cudaMemcpyDeviceToHost, ctx->stream));
            MW_CK(cudaStreamSynchronize(ctx->stream));
            std::vector<NodeKey> fkeys;
            std::vector<int> fslots;
            std::unordered_map<unsigned long long, std::vector<int>> by_parent;  // parent key hash -> families
            for (int p = 0; p < pcount[t]; p++) {
                int n, l0, l1, l2;
                unpack_key(m, keys[p], n, l0, l1, l2);
                NodeKey pk;
                if (!pack_key(m, n - 1, l0 >> 1, l1 >> 1, l2 >> 1, pk)) {
                    ctx->err = "plan: a GenNode without a parent in the world";
                    return fail(MWGPU_ERR_BAD_ARG);
                }
                const int c = (l0 & 1) | ((l1 & 1) << 1) | ((l2 & 1) << 2);
                auto &cand = by_parent[pk.lo * 0x9E3779B97F4A7C15ull ^ pk.hi];
                int fam = -1;
                for (int q : cand)
                    if (fkeys[q] == pk) fam = q;
                if (fam < 0) {
                    fam = (int)fkeys.size();
                    fkeys.push_back(pk);
                    fslots.insert(fslots.end(), 8, -1);
                    cand.push_back(fam);
                }
                fslots[8 * (size_t)fam + c] = p;
            }
            pl->fcount[t] = (int)fkeys.size();
            if ((s = plan_alloc(ctx, pl, &pl->d_fam_keys[t], fkeys.size())) || (s = plan_alloc(ctx, pl, &pl->d_fam_slots[t], fslots.size())))
                return fail(s);
            MW_CK(cudaMemcpyAsync(pl->d_fam_keys[t], fkeys.data(), sizeof(NodeKey) * fkeys.size(), cudaMemcpyHostToDevice, ctx->stream));
            MW_CK(cudaMemcpyAsync(pl->d_fam_slots[t], fslots.data(), sizeof(int) * fslots.size(), cudaMemcpyHostToDevice, ctx->stream));
            MW_CK(cudaStreamSynchronize(ctx->stream));
        }
    }
    // transforms: parents per depth over all output trees
    if (flags & MWGPU_PLAN_TRANSFORMS) {
        std::vector<std::vector<int2>> levels;
        for (int t = 0; t < n_trees; t++) {
            const mwgpu_tree *tr = outs[t];
            for (int i = 0; i < tr->t.n_real; i++) {
                const int depth = tr->h_idx[i].x - tr->mra.root_scale;
                if (tr->h_child0[i] < 0 || depth < 0) continue;
                if ((int)levels.size() <= depth) levels.resize(depth + 1);
                levels[depth].push_back(make_int2(t, i));
            }
        }
        std::vector<int> flat, ftree;
        for (auto &l : levels) {
            pl->ranges.push_back({(int)flat.size(), (int)l.size()});
            for (auto &e : l) {
                ftree.push_back(e.x);
                flat.push_back(e.y);
            }
        }
        if ((s = plan_alloc(ctx, pl, &pl->d_list, flat.size())) || (s = plan_alloc(ctx, pl, &pl->d_ltree, flat.size()))) return fail(s);
        if (!flat.empty()) {
            MW_CK(cudaMemcpyAsync(pl->d_list, flat.data(), sizeof(int) * flat.size(), cudaMemcpyHostToDevice, ctx->stream));
            MW_CK(cudaMemcpyAsync(pl->d_ltree, ftree.data(), sizeof(int) * ftree.size(), cudaMemcpyHostToDevice, ctx->stream));
        }
        MW_CK(cudaStreamSynchronize(ctx->stream));
    }
    if (pl->precision == MWGPU_PREC_MIXED) {
        std::vector<long long> poff;
        pair_offsets(lv, poff);
        pl->np = poff[n];
        const long long total = (long long)st0.node_terms;
        pl->items_cap = total + total / 4 + 1024;
        pl->scan_n = scan_blocks(pl->np + 1) + 2;
        pl->cscan_n = scan_blocks(n + 1) + 2;
        int dev_sm = 0;
        cudaDeviceGetAttribute(&dev_sm, cudaDevAttrMultiProcessorCount, ctx->device);
        const int res = std::max(1, contract_items_resident(o->op.K));
        pl->grid = std::max(1, dev_sm) * res;
        const long long per_min = std::max<long long>(4, pl->items_cap / (16LL * pl->grid) / 2);
        const long long ccap = (long long)n + pl->items_cap / per_min + 1;
        if (ccap > 0x7fffffffLL || pl->items_cap > 0x7fffffffLL) {
            ctx->err = "plan: work list too large";
            return fail(MWGPU_ERR_BAD_ARG);
        }
        pl->chunks_cap = (int)ccap;
        if ((s = plan_alloc(ctx, pl, &pl->d_pair_off, n + 1)) || (s = plan_alloc(ctx, pl, &pl->d_pcounts, pl->np + 1)) ||
            (s = plan_alloc(ctx, pl, &pl->d_item_off, pl->np + 1)) || (s = plan_alloc(ctx, pl, &pl->d_scan, pl->scan_n)) ||
            (s = plan_alloc(ctx, pl, &pl->d_goff, n + 1)) || (s = plan_alloc(ctx, pl, &pl->d_ccount, n + 1)) ||
            (s = plan_alloc(ctx, pl, &pl->d_coff, n + 1)) || (s = plan_alloc(ctx, pl, &pl->d_cscan, pl->cscan_n)) ||
            (s = plan_alloc(ctx, pl, &pl->d_items, pl->items_cap)) || (s = plan_alloc(ctx, pl, &pl->d_chunks, pl->chunks_cap)) ||
            (s = plan_alloc(ctx, pl, &pl->d_chunk_begin, n + 1)) || (s = plan_alloc(ctx, pl, &pl->d_nchunks, 1)) ||
            (s = plan_alloc(ctx, pl, &pl->d_counter, 2)) ||
            (s = plan_alloc(ctx, pl, &pl->d_partial, (size_t)pl->chunks_cap * 8 * o->mra.kp1_d)))
            return fail(s);
        pl->pencil = use_pencil(lv);
        pl->pen_warps = pencil_warps();
        if (pl->pencil) {
            // every term at the depth of every entry within the plan configuration's band
            // width (MWGPU_PLAN_FILL=1 keeps the fill, to compare both forms)
            // A term wider than that makes no item below the roots when its blocks
            // other than (s, s) are outside its band at every translation: the
            // work list leaves the (s, s) block out there, and every other
            // component pair takes a non-(s, s) block in some direction.
            const int R = o->n_rows, T = o->op.n_terms;
            std::vector<signed char> wide(R, -1);   // per depth: -1 unknown, 0 / 1
            auto depth_wide = [&](int depth) {
                if (depth < 0 || depth >= R) return false;
                if (wide[depth] < 0) {
                    wide[depth] = 0;
                    for (int t = 0; t < T; t++) {
                        const int *w = &o->widths[((size_t)t * R + depth) * 5];
                        if (w[4] <= mwgpu::kPencilCfgW[kPlanPencilCfg]) continue;
                        if (depth != 0 && std::max(w[1], std::max(w[2], w[3])) < 0) continue;
                        wide[depth] = 1;
                        break;
                    }
                }
                return wide[depth] != 0;
            };
            pl->pen_all_ok = std::getenv("MWGPU_PLAN_FILL") == nullptr;
            for (int wi = 0; wi < n && pl->pen_all_ok; wi++)
                if (depth_wide(lv.outs[lv.tree[wi]]->h_idx[lv.node[wi]].x - o->mra.root_scale)) pl->pen_all_ok = false;
        }
        if ((term_order_supported(o->op.n_terms) || pl->pencil) && (s = plan_alloc(ctx, pl, &pl->d_items_cm, pl->items_cap))) return fail(s);
        if (pl->pencil) {
            PencilPlan pp;
            pencil_build(lv, pp, kPlanPencilCfg);
            std::vector<PencilUnit> units(pp.n_units);
            pp.emit(units.data());
            pl->n_units = (int)pp.n_units;
            pl->n_tasks = pp.n_tasks;
            pl->kscan_n = scan_blocks(n + 1) + 2;
            if ((s = plan_alloc(ctx, pl, &pl->d_keep, n + 1)) || (s = plan_alloc(ctx, pl, &pl->d_keep_off, n + 1)) ||
                (s = plan_alloc(ctx, pl, &pl->d_kscan, pl->kscan_n)) || (s = plan_alloc(ctx, pl, &pl->d_units, std::max(pl->n_units, 1))) ||
                (s = plan_alloc(ctx, pl, &pl->d_task_unit, pp.n_tasks + 1)) || (s = plan_alloc(ctx, pl, &pl->d_pen_begin, n + 1)) ||
                (s = plan_alloc(ctx, pl, &pl->d_pen_counter, 1)) ||
                (s = plan_alloc(ctx, pl, &pl->d_pen_partial, (size_t)std::max(pp.n_tasks, 1) * 8 * o->mra.kp1_d)))
                return fail(s);
            if (pl->n_units > 0)
                MW_CK(cudaMemcpyAsync(pl->d_units, units.data(), sizeof(PencilUnit) * pl->n_units, cudaMemcpyHostToDevice, ctx->stream));
            MW_CK(cudaMemcpyAsync(pl->d_task_unit, pp.task_unit.data(), sizeof(int) * (pp.n_tasks + 1), cudaMemcpyHostToDevice, ctx->stream));
            MW_CK(cudaMemcpyAsync(pl->d_pen_begin, pp.pen_begin.data(), sizeof(int) * (n + 1), cudaMemcpyHostToDevice, ctx->stream));
        }
        MW_CK(cudaMemcpyAsync(pl->d_pair_off, poff.data(), sizeof(long long) * (n + 1), cudaMemcpyHostToDevice, ctx->stream));
        MW_CK(cudaStreamSynchronize(ctx->stream));
        // chunk length: candidates around the default, each timed on the full
        // contraction of this level (after one untimed work-list pass)
        pl->per = std::max<long long>(8, (total + 8LL * pl->grid - 1) / (8LL * pl->grid));
        plan_sequence(ctx, pl);
        if ((s = plan_check(ctx, pl, nullptr))) return fail(s);
        const bool tune = (flags & MWGPU_PLAN_AUTOTUNE) != 0 && total > 0;
        if (tune) {
            // the schedule of the contraction (pencil + item kernels where the
            // level allows the pencil kernel, with 8 or 16 consumer warps per
            // pencil CTA, or the item kernel alone) and the chunk length of the
            // persistent item kernel (2 to 16 waves of the grid over its
            // items), each candidate timed on the whole contraction of this level
            const bool can_pencil = pl->pencil;
            const long long kept = can_pencil ? std::max<long long>(1, total - (long long)pl->pen_node_terms) : total;
            double best = 1e300;
            long long best_per = pl->per;
            int best_sched = pl->pencil ? (pl->pen_warps == 16 ? 2 : 1) : 0;
            std::vector<int> scheds{0};
            if (can_pencil) scheds = pencil_shape_ok(16) ? std::vector<int>{1, 2, 0} : std::vector<int>{1, 0};
            for (int pen : scheds) {
                pl->pencil = pen != 0;
                pl->pen_warps = pen == 2 ? 16 : 8;
                const long long base = pen ? kept : total;
                for (int waves : {2, 4, 8, 16}) {
                    const long long per = std::max<long long>(per_min, (base + (long long)waves * pl->grid - 1) / ((long long)waves * pl->grid));
                    float ms = 0.f;
                    for (int rep = 0; rep < 2; rep++) {
                        plan_contract(ctx, pl, per, false);
                        MW_CK(cudaEventRecord(pl->e2, ctx->stream));
                        MW_CK(cudaEventSynchronize(pl->e2));
                        float m1 = 0.f;
                        MW_CK(cudaEventElapsedTime(&m1, pl->e1, pl->e2));
                        ms = rep == 0 ? m1 : std::min(ms, m1);
                        if (m1 > 250.f) break;  // long launches: one timing is enough
                    }
                    int herr = 0;
                    MW_CK(cudaMemcpy(&herr, pl->d_err, sizeof(int), cudaMemcpyDeviceToHost));
                    if (herr) {
                        ctx->err = "plan autotuning: device error flags " + std::to_string(herr);
                        return fail((herr & DE_TIMEOUT) ? MWGPU_ERR_TIMEOUT : MWGPU_ERR_INTERNAL);
                    }
                    pl->tune_per.push_back(per);
                    pl->tune_pencil.push_back(pen);
                    pl->tune_ms.push_back(ms);
                    if (ms < best) {
                        best = ms;
                        best_per = per;
                        best_sched = pen;
                        pl->tune_choice = (int)pl->tune_ms.size() - 1;
                    }
                }
            }
            pl->per = best_per;
            pl->pencil = best_sched != 0;
            pl->pen_warps = best_sched == 2 ? 16 : 8;
            // the trees hold what every execution leaves (same schedule and chunking)
            plan_sequence(ctx, pl);
            if ((s = plan_check(ctx, pl, nullptr))) return fail(s);
        }
    } else {
        // one eager pass: the trees hold what every execution leaves (with the transforms)
        plan_sequence(ctx, pl);
        if ((s = plan_check(ctx, pl, nullptr))) return fail(s);
    }
    // capture the level as one graph
    pl->pen_all = pl->pen_all_ok;
    unsigned long long l0 = ctx->launches;
    MW_CK(cudaStreamBeginCapture(ctx->stream, cudaStreamCaptureModeRelaxed));
    plan_sequence(ctx, pl);
    cudaError_t ce = cudaStreamEndCapture(ctx->stream, &pl->graph);
    pl->launches_per_exec = ctx->launches - l0;
    ctx->launches = l0;
    if (ce != cudaSuccess) {
        ctx->err = std::string("plan: graph capture failed: ") + cudaGetErrorString(ce);
        return fail(MWGPU_ERR_DEVICE);
    }
    ce = cudaGraphInstantiate(&pl->exec, pl->graph, 0);
    if (ce != cudaSuccess) {
        ctx->err = std::string("plan: graph instantiation failed: ") + cudaGetErrorString(ce);
        return fail(MWGPU_ERR_DEVICE);
    }
    for (auto *t : pl->inps) t->plans++;
    for (auto *t : pl->outs) t->plans++;
    *out = pl;
    return MWGPU_OK;
}

extern "C" mwgpu_status mwgpu_plan_execute(mwgpu_ctx *ctx, mwgpu_plan *pl, mwgpu_level_stats *stats) {
    if (!ctx || !pl) return MWGPU_ERR_BAD_ARG;
    cudaSetDevice(ctx->device);
    MW_CK(cudaGraphLaunch(pl->exec, ctx->stream));
    ctx->launches += pl->launches_per_exec;
    if (!stats) return MWGPU_OK;
    return plan_check(ctx, pl, stats);
}

extern "C" mwgpu_status mwgpu_plan_check(mwgpu_ctx *ctx, mwgpu_plan *pl, mwgpu_level_stats *stats) {
    if (!ctx || !pl) return MWGPU_ERR_BAD_ARG;
    cudaSetDevice(ctx->device);
    return plan_check(ctx, pl, stats);
}

extern "C" mwgpu_status mwgpu_plan_info(const mwgpu_plan *pl, long long *chunk_items, int *grid, int *n_candidates, long long *cand_items,
                                        double *cand_ms, unsigned long long *launches) {
    if (!pl) return MWGPU_ERR_BAD_ARG;
    if (chunk_items) *chunk_items = pl->per;
    if (grid) *grid = pl->grid;
    if (launches) *launches = pl->launches_per_exec;
    if (n_candidates) {
        const int nc = (int)pl->tune_per.size();
        if (cand_items)
            for (int i = 0; i < std::min(nc, *n_candidates); i++) cand_items[i] = pl->tune_per[i];
        if (cand_ms)
            for (int i = 0; i < std::min(nc, *n_candidates); i++) cand_ms[i] = pl->tune_ms[i];
        *n_candidates = nc;
    }
    return MWGPU_OK;
}

extern "C" mwgpu_status mwgpu_fp64_pipe_rates(mwgpu_ctx *ctx, double *dfma_tflops, double *dmma_tflops) {
    if (!ctx || !dfma_tflops || !dmma_tflops) return MWGPU_ERR_BAD_ARG;
    cudaSetDevice(ctx->device);
    int sms = 0;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, ctx->device);
    const int blocks = std::max(1, sms) * 4, iters = 2048;
    double *out = nullptr;
    MW_CK(cudaMalloc(&out, sizeof(double) * (size_t)blocks * rate_threads()));
    cudaEvent_t a, b;
    cudaEventCreate(&a);
    cudaEventCreate(&b);
    auto timed = [&](bool dmma) {
        float best = 1e30f;
        for (int rep = 0; rep < 3; rep++) {
            cudaEventRecord(a, ctx->stream);
            if (dmma) launch_rate_dmma(out, blocks, iters, ctx->stream);
            else launch_rate_dfma(out, blocks, iters, ctx->stream);
            cudaEventRecord(b, ctx->stream);
            cudaEventSynchronize(b);
            float ms = 0.f;
            cudaEventElapsedTime(&ms, a, b);
            if (rep > 0) best = std::min(best, ms);  // the first launch warms up
        }
        return best;
    };
    const float t_dfma = timed(false), t_dmma = timed(true);
    const cudaError_t e = cudaGetLastError();
    cudaEventDestroy(a);
    cudaEventDestroy(b);
    cudaFree(out);
    ctx->launches += 6;
    if (e != cudaSuccess) {
        ctx->err = std::string("fp64 pipe rates: ") + cudaGetErrorString(e);
        return MWGPU_ERR_DEVICE;
    }
    *dfma_tflops = rate_dfma_flops(blocks, iters) / (t_dfma * 1e-3) / 1e12;
    *dmma_tflops = rate_dmma_flops(blocks, iters) / (t_dmma * 1e-3) / 1e12;
    return MWGPU_OK;
}

extern "C" mwgpu_status mwgpu_plan_tuning(const mwgpu_plan *pl, int *n_candidates, long long *chunk_items, int *schedule, double *ms,
                                          int *chosen) {
    if (!pl || !n_candidates) return MWGPU_ERR_BAD_ARG;
    const int nc = (int)pl->tune_per.size();
    for (int i = 0; i < std::min(nc, *n_candidates); i++) {
        if (chunk_items) chunk_items[i] = pl->tune_per[i];
        if (schedule) schedule[i] = pl->tune_pencil[i];
        if (ms) ms[i] = pl->tune_ms[i];
    }
    if (chosen) *chosen = pl->tune_choice;
    *n_candidates = nc;
    return MWGPU_OK;
}

extern "C" mwgpu_status mwgpu_plan_pencil_info(const mwgpu_plan *pl, unsigned long long *node_terms, double *ms) {
    if (!pl || !node_terms || !ms) return MWGPU_ERR_BAD_ARG;
    *node_terms = pl->pencil ? pl->pen_node_terms : 0ull;
    *ms = pl->pencil ? pl->pen_ms : 0.0;
    return MWGPU_OK;
}

extern "C" mwgpu_status mwgpu_plan_destroy(mwgpu_ctx *ctx, mwgpu_plan *pl) {
    if (!ctx) return MWGPU_ERR_BAD_ARG;
    if (!pl) return MWGPU_OK;
    cudaSetDevice(ctx->device);
    cudaStreamSynchronize(ctx->stream);
    for (auto *t : pl->inps) t->plans--;
    for (auto *t : pl->outs) t->plans--;
    plan_free(pl);
    return MWGPU_OK;
}

// ---------------------------------------------------------------------------
// Judged adaptive apply over a proposed output grid (mwgpu_apply_judged).
// ---------------------------------------------------------------------------
namespace {

// bump allocator over ctx->d_arena: first a sizing pass (base == nullptr),
// then the carving pass
struct Carver {
    char *base = nullptr;
    size_t off = 0;
    template <class T> T *take(size_t n) {
        off = (off + 255) & ~(size_t)255;
        T *p = base ? (T *)(base + off) : nullptr;
        off += sizeof(T) * std::max<size_t>(n, 1);
        return p;
    }
};

}  // namespace

extern "C" mwgpu_status mwgpu_apply_judged(mwgpu_ctx *ctx, const mwgpu_oper *o, mwgpu_tree *inp, mwgpu_tree *out, int n_levels,
                                           const int *level_begin, double prec, int abs_prec, int first_level, const double *state_in,
                                           int transforms, int *flags_out, int *first_miss_out, double *sq_levels, mwgpu_level_stats *stats) {
    if (!ctx) return MWGPU_ERR_BAD_ARG;
    MW_ARG(o && inp && out && level_begin && flags_out && first_miss_out && state_in, "null argument");
    MW_ARG(first_level >= 0 && first_level < n_levels, "first level out of range");
    MW_ARG(n_levels >= 1 && level_begin[0] == 0 && level_begin[n_levels] == out->t.n_real, "level ranges must cover the output tree");
    for (int j = 0; j < n_levels; j++) MW_ARG(level_begin[j + 1] > level_begin[j], "empty proposal level");
    const int N = out->t.n_real;
    // levels and children: children of level j are consecutive in level j+1
    for (int j = 0; j < n_levels; j++)
        for (int i = level_begin[j]; i < level_begin[j + 1]; i++) {
            const int c0 = out->h_child0[i];
            MW_ARG(c0 < 0 || (c0 >= level_begin[j + 1] && j + 1 < n_levels && c0 + 8 <= level_begin[j + 2]),
                   "proposed children must lie in the next level");
        }
    PhaseTrace tr(ctx, "apply_judged");
    std::vector<int> all(N);
    for (int i = 0; i < N; i++) all[i] = i;
    mwgpu_tree *inps[1] = {inp}, *outs[1] = {out};
    Level lv;
    if (auto s = make_level(ctx, o, 1, inps, outs, nullptr, all.data(), N, lv)) return s;
    cudaSetDevice(ctx->device);
    if (stats) std::memset(stats, 0, sizeof(*stats));
    const bool mixed = ctx->precision == MWGPU_PREC_MIXED;
    const DevMRA &m = o->mra;
    if (auto s = ensure_work(ctx, N)) return s;
    if (auto s = ensure_trees(ctx, 1)) return s;
    MW_CK(cudaEventRecord(ctx->ev0, ctx->stream));
    MW_CK(cudaMemcpyAsync(ctx->d_work, all.data(), sizeof(int) * N, cudaMemcpyHostToDevice, ctx->stream));
    MW_CK(cudaMemsetAsync(ctx->d_wtree, 0, sizeof(int) * N, ctx->stream));
    MW_CK(cudaMemsetAsync(ctx->d_err, 0, sizeof(int), ctx->stream));
    MW_CK(cudaMemsetAsync(ctx->d_stats, 0, sizeof(LevelStats), ctx->stream));
    // GenNodes for every proposed node (a superset of what the judged tree needs)
    std::vector<int> pcount;
    unsigned long long gen_total = 0;
    tr.mark("setup");
    if (auto s = gen_pass(ctx, lv, pcount, gen_total)) return s;
    tr.mark("gen");
    lv.fs.assign(1, inp->t);
    lv.gs.assign(1, out->t);
    MW_CK(cudaMemcpyAsync(ctx->d_fs, lv.fs.data(), sizeof(DevTree), cudaMemcpyHostToDevice, ctx->stream));
    MW_CK(cudaMemcpyAsync(ctx->d_gs, lv.gs.data(), sizeof(DevTree), cudaMemcpyHostToDevice, ctx->stream));
    // band pairs per proposed node; per level the largest counts any judged subset can reach
    std::vector<long long> poff;
    pair_offsets(lv, poff);
    std::vector<int> cells(N);
    for (int i = 0; i < N; i++) cells[i] = (int)(poff[i + 1] - poff[i]);
    std::vector<long long> lvl_pairs(n_levels, 0), lvl_items(n_levels, 0);
    for (int j = 0; j < n_levels; j++) lvl_pairs[j] = poff[level_begin[j + 1]] - poff[level_begin[j]];
    int grid = 0, dev_sm = 0;
    long long max_pairs = 0, max_items = 0, max_chunks = 0;
    int max_level = 0;
    for (int j = 0; j < n_levels; j++) max_level = std::max(max_level, level_begin[j + 1] - level_begin[j]);
    for (auto v : lvl_pairs) max_pairs = std::max(max_pairs, v);
    std::vector<long long> lvl_per(n_levels, 8);
    const int T = o->op.n_terms;
    const bool order = term_order_supported(T);  // term-major work items (mixed form)
    // Work-list capacity per level: every (pair, term) of the level as an item
    // while that stays within kJudgedItemBudget (no host round trip); beyond
    // it, or when a level overflows it, the exact bound from an unscreened
    // count pass (one synchronisation) and the pass runs again.
    constexpr long long kJudgedItemBudget = 1LL << 25;
    const bool estimate_fits = max_pairs * T <= kJudgedItemBudget;
    if (mixed) {
        cudaDeviceGetAttribute(&dev_sm, cudaDevAttrMultiProcessorCount, ctx->device);
        grid = std::max(1, dev_sm) * std::max(1, contract_items_resident(o->op.K));
    }
    int first_miss = 0x7fffffff;
    for (int attempt = 0;; attempt++) {
    const bool exact = attempt > 0 || !estimate_fits;
    max_items = max_chunks = 0;
    if (mixed && !exact) {
        for (int j = 0; j < n_levels; j++) {
            lvl_items[j] = lvl_pairs[j] * T;
            lvl_per[j] = 0;
            max_items = std::max(max_items, lvl_items[j]);
            max_chunks = std::max(max_chunks, (long long)(level_begin[j + 1] - level_begin[j]) + kChunkTarget + 1);
        }
    }
    if (mixed && exact) {
        // items per proposed node without norm screening (an upper bound of every level's work list)
        if (auto s = grow_buf(ctx, &ctx->d_pair_off, &ctx->pair_off_cap, N + 1)) return s;
        if (auto s = grow_buf(ctx, &ctx->d_pcounts, &ctx->pcounts_cap, poff[N] + 1)) return s;
        if (auto s = grow_buf(ctx, &ctx->d_item_off, &ctx->item_off_cap, poff[N] + 1)) return s;
        if (auto s = grow_buf(ctx, &ctx->d_scan, &ctx->scan_cap, scan_blocks(poff[N] + 1) + 2)) return s;
        if (auto s = grow_buf(ctx, &ctx->d_goff, &ctx->goff_cap, N + 1)) return s;
        const double neg = -HUGE_VAL;
        MW_CK(cudaMemcpyAsync(ctx->d_gthr, &neg, sizeof(double), cudaMemcpyHostToDevice, ctx->stream));
        MW_CK(cudaMemcpyAsync(ctx->d_pair_off, poff.data(), sizeof(long long) * (N + 1), cudaMemcpyHostToDevice, ctx->stream));
        LevelStats *dst = ctx->d_stats;
        launch_pairs_count(m, o->op, ctx->d_fs, ctx->d_gs, ctx->d_wtree, ctx->d_work, ctx->d_pair_off, N, poff[N], ctx->d_gthr, ctx->d_pcounts,
                           &dst->components, &dst->band_nodes, ctx->d_err, ctx->stream);
        launch_scan(ctx->d_pcounts, ctx->d_item_off, poff[N], ctx->d_scan, ctx->d_scan + (ctx->scan_cap - 1), ctx->stream);
        launch_gather_goff(ctx->d_item_off, ctx->d_pair_off, N, ctx->d_goff, ctx->stream);
        ctx->launches += 5;
        std::vector<long long> ub(N + 1);
        MW_CK(cudaMemcpyAsync(ub.data(), ctx->d_goff, sizeof(long long) * (N + 1), cudaMemcpyDeviceToHost, ctx->stream));
        MW_CK(cudaMemsetAsync(ctx->d_stats, 0, sizeof(LevelStats), ctx->stream));
        if (auto s = check_err(ctx, "judged apply (work-list bound)")) return s;
        // chunk length from the level's item count on the device (the rule of
        // the host-driven levels, so that both give the same sums): at most
        // n + kChunkTarget + 1 chunks
        for (int j = 0; j < n_levels; j++) {
            lvl_items[j] = ub[level_begin[j + 1]] - ub[level_begin[j]];
            lvl_per[j] = 0;
            max_items = std::max(max_items, lvl_items[j]);
            max_chunks = std::max(max_chunks, (long long)(level_begin[j + 1] - level_begin[j]) + kChunkTarget + 1);
        }
        if (max_items > 0x7fffffffLL || max_chunks > 0x7fffffffLL) {
            ctx->err = "judged apply: work list too large";
            return MWGPU_ERR_BAD_ARG;
        }
    }
    tr.mark("bound");
    // scratch, sized then carved
    const int rows = std::max(m.max_scale - m.root_scale + 2, 1);
    auto carve = [&](Carver &c) {
        struct B {
            int *flags, *kcnt, *work, *nwork, *ccnt, *pcounts, *chunk_begin, *nchunks, *counter, *first_miss, *cells;
            long long *koff, *kscan, *pair_off, *pscan, *item_off, *iscan, *goff, *coff, *cscan;
            int4 *chunks;
            WorkItem *items, *items_cm;
            double *partial, *state, *sq, *scale_fac;
            unsigned long long *node_terms;
        } b{};
        b.flags = c.take<int>(N);
        b.cells = c.take<int>(N);
        b.kcnt = c.take<int>(max_level + 1);
        b.koff = c.take<long long>(max_level + 1);
        b.kscan = c.take<long long>(scan_blocks(max_level + 1) + 2);
        b.work = c.take<int>(max_level + 1);
        b.nwork = c.take<int>(1);
        b.ccnt = c.take<int>(max_level + 1);
        b.pair_off = c.take<long long>(max_level + 1);
        b.pscan = c.take<long long>(scan_blocks(max_level + 1) + 2);
        b.pcounts = c.take<int>(max_pairs + 1);
        b.item_off = c.take<long long>(max_pairs + 1);
        b.iscan = c.take<long long>(scan_blocks(max_pairs + 1) + 2);
        b.goff = c.take<long long>(max_level + 1);
        b.coff = c.take<long long>(max_level + 1);
        b.cscan = c.take<long long>(scan_blocks(max_level + 1) + 2);
        b.chunks = c.take<int4>(mixed ? max_chunks : 1);
        b.chunk_begin = c.take<int>(max_level + 1);
        b.nchunks = c.take<int>(1);
        b.counter = c.take<int>(2);  // CUDA-core and tensor-core chunk counters
        b.items = c.take<WorkItem>(mixed ? max_items : 1);
        b.items_cm = c.take<WorkItem>(mixed && order ? max_items : 1);
        b.partial = c.take<double>(mixed ? (size_t)max_chunks * 8 * m.kp1_d : 1);
        b.state = c.take<double>(3);
        b.sq = c.take<double>(3 * (size_t)n_levels);
        b.scale_fac = c.take<double>(rows);
        b.first_miss = c.take<int>(1);
        b.node_terms = c.take<unsigned long long>(1);
        return b;
    };
    Carver sizing;
    carve(sizing);
    if (sizing.off > ctx->arena_bytes) {
        if (ctx->d_arena) cudaFree(ctx->d_arena);
        ctx->d_arena = nullptr;
        ctx->arena_bytes = 0;
        MW_CK(cudaMalloc(&ctx->d_arena, sizing.off));
        ctx->arena_bytes = sizing.off;
    }
    Carver cv;
    cv.base = (char *)ctx->d_arena;
    auto b = carve(cv);
    // initial state: the levels before first_level are the judged tree already
    // computed (kept; refined where they have children), first_level is kept;
    // TreeBuilder's sNorm, wNorm and tree norm after the levels before
    std::vector<int> h_flags(N, 0);
    for (int j = 0; j < first_level; j++)
        for (int i = level_begin[j]; i < level_begin[j + 1]; i++) h_flags[i] = 1 | (out->h_child0[i] >= 0 ? 2 : 0);
    for (int i = level_begin[first_level]; i < level_begin[first_level + 1]; i++) h_flags[i] = 1;
    std::vector<double> fac(rows);
    for (int d = 0; d < rows; d++) fac[d] = std::pow(2.0, -(0.5 * 1.0 * (m.root_scale + d + 1)));
    const double state0[3] = {state_in[0], state_in[1], state_in[2]};
    const int big = 0x7fffffff;
    MW_CK(cudaMemcpyAsync(b.flags, h_flags.data(), sizeof(int) * N, cudaMemcpyHostToDevice, ctx->stream));
    MW_CK(cudaMemcpyAsync(b.cells, cells.data(), sizeof(int) * N, cudaMemcpyHostToDevice, ctx->stream));
    MW_CK(cudaMemcpyAsync(b.scale_fac, fac.data(), sizeof(double) * rows, cudaMemcpyHostToDevice, ctx->stream));
    MW_CK(cudaMemcpyAsync(b.state, state0, sizeof(state0), cudaMemcpyHostToDevice, ctx->stream));
    MW_CK(cudaMemcpyAsync(b.first_miss, &big, sizeof(int), cudaMemcpyHostToDevice, ctx->stream));
    MW_CK(cudaMemsetAsync(b.node_terms, 0, sizeof(unsigned long long), ctx->stream));
    tr.mark("arena");
    MW_CK(cudaEventRecord(ctx->ev1, ctx->stream));
    cudaStream_t st = ctx->stream;
    for (int j = first_level; j < n_levels; j++) {
        const int lb = level_begin[j], nl = level_begin[j + 1] - lb;
        launch_keep_counts(b.flags, lb, nl, b.kcnt, st);
        launch_scan(b.kcnt, b.koff, nl, b.kscan, b.kscan + (scan_blocks(max_level + 1) + 1), st);
        launch_compact(b.flags, lb, nl, b.koff, b.work, b.nwork, st);
        launch_threshold(b.state + 2, prec, T, ctx->d_gthr, st);
        ctx->launches += 6;
        if (mixed) {
            const long long pc = lvl_pairs[j];
            launch_cells(b.work, b.nwork, nl, b.cells, b.ccnt, st);
            launch_scan(b.ccnt, b.pair_off, nl, b.pscan, b.pscan + (scan_blocks(max_level + 1) + 1), st);
            const long long *np_dev = b.pair_off + nl;
            LevelStats *dst = ctx->d_stats;
            launch_pairs_count(m, o->op, ctx->d_fs, ctx->d_gs, ctx->d_wtree, b.work, b.pair_off, nl, pc, ctx->d_gthr, b.pcounts, &dst->components,
                               &dst->band_nodes, ctx->d_err, st, np_dev, b.nwork);
            launch_scan(b.pcounts, b.item_off, pc, b.iscan, b.iscan + (scan_blocks(max_pairs + 1) + 1), st);
            launch_gather_goff(b.item_off, b.pair_off, nl, b.goff, st, b.nwork, lvl_items[j]);
            launch_chunk_count(b.goff, nl, lvl_per[j], b.ccnt, st, b.nwork);
            launch_scan(b.ccnt, b.coff, nl, b.cscan, b.cscan + (scan_blocks(max_level + 1) + 1), st);
            const int ccap = (int)((long long)nl + kChunkTarget + 1);
            launch_chunk_fill(b.goff, b.coff, nl, lvl_per[j], b.chunks, b.chunk_begin, ccap, b.nchunks, ctx->d_err, st, b.nwork);
            launch_pairs_fill(m, o->op, ctx->d_fs, ctx->d_gs, ctx->d_wtree, b.work, b.pair_off, nl, pc, ctx->d_gthr, b.pcounts, b.item_off,
                              order ? b.items_cm : b.items, lvl_items[j], ctx->d_err, st, np_dev, b.nwork);
            if (order) launch_order_terms(b.goff, nl, b.items_cm, b.items, T, ctx->d_err, st, b.nwork);
            MW_CK(cudaMemsetAsync(b.counter, 0, sizeof(int), st));
            launch_items(m, o->op, ctx->d_fs, ctx->d_gs, ctx->d_wtree, b.work, b.chunks, grid, b.items, b.partial, ctx->d_err, b.nchunks, b.counter,
                         inp->t.tc32 ? b.counter + 1 : nullptr, st);
            launch_reduce_chunks(m, ctx->d_gs, ctx->d_wtree, b.work, nl, b.chunk_begin, b.partial, st, b.nwork);
            launch_level_norm(out->t, b.work, b.nwork, j == 0, b.state, b.sq + 3 * j, b.goff, b.node_terms, st);  // sNorm: level 0 only
            ctx->launches += 17 + (order ? 1 : 0);
        } else {
            launch_contract_fp64(m, o->op, inp->t, out->t, b.work, nl, 0.0, ctx->d_stats, ctx->d_err, st, b.nwork, ctx->d_gthr);
            launch_level_norm(out->t, b.work, b.nwork, j == 0, b.state, b.sq + 3 * j, nullptr, nullptr, st);
            ctx->launches += 2;
        }
        launch_judge(m, out->t, b.work, b.nwork, nl, b.state, prec, abs_prec, b.scale_fac, m.max_scale, b.flags, j, b.first_miss, st);
        ctx->launches++;
        if (tr.on) tr.mark("L" + std::to_string(j));
    }
    MW_CK(cudaGetLastError());
    MW_CK(cudaEventRecord(ctx->ev2, ctx->stream));
    if (mixed && !exact) {
        int herr = 0;
        MW_CK(cudaMemcpyAsync(&herr, ctx->d_err, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
        MW_CK(cudaStreamSynchronize(ctx->stream));
        if (herr == DE_POOL_FULL) {
            // a level's work list outgrew the estimate: exact bound, again
            // (the pass only overwrites what it computes)
            MW_CK(cudaMemsetAsync(ctx->d_err, 0, sizeof(int), ctx->stream));
            MW_CK(cudaMemsetAsync(ctx->d_stats, 0, sizeof(LevelStats), ctx->stream));
            tr.mark("overflow");
            continue;
        }
    }
    first_miss = big;
    unsigned long long nt_mixed = 0;
    LevelStats hs{};
    MW_CK(cudaMemcpyAsync(flags_out, b.flags, sizeof(int) * N, cudaMemcpyDeviceToHost, st));
    MW_CK(cudaMemcpyAsync(&first_miss, b.first_miss, sizeof(int), cudaMemcpyDeviceToHost, st));
    MW_CK(cudaMemcpyAsync(&nt_mixed, b.node_terms, sizeof(nt_mixed), cudaMemcpyDeviceToHost, st));
    MW_CK(cudaMemcpyAsync(&hs, ctx->d_stats, sizeof(hs), cudaMemcpyDeviceToHost, st));
    std::vector<double> sqv(3 * (size_t)n_levels);
    MW_CK(cudaMemcpyAsync(sqv.data(), b.sq, sizeof(double) * 3 * n_levels, cudaMemcpyDeviceToHost, st));
    if (auto s = check_err(ctx, "judged apply")) return s;
    tr.mark("result");
    if (sq_levels) std::memcpy(sq_levels, sqv.data(), sizeof(double) * 3 * n_levels);
    *first_miss_out = first_miss == big ? -1 : first_miss;
    if (stats) {
        stats->node_terms = mixed ? nt_mixed : hs.node_terms;
        stats->components = hs.components;
        stats->band_nodes = hs.band_nodes;
        stats->gen_nodes = gen_total;
        float ms = 0.f;
        cudaEventElapsedTime(&ms, ctx->ev0, ctx->ev2);
        stats->device_ms = ms;
        cudaEventElapsedTime(&ms, ctx->ev1, ctx->ev2);
        stats->contract_ms = ms;
    }
    break;
    }
    cudaStream_t st = ctx->stream;
    if (transforms && first_miss == 0x7fffffff) {
        // TopDown(add) and BottomUp over the judged tree: its parents are the refined nodes
        std::vector<std::vector<int>> levels(n_levels);
        for (int j = 0; j < n_levels; j++)
            for (int i = level_begin[j]; i < level_begin[j + 1]; i++)
                if ((flags_out[i] & 3) == 3) levels[j].push_back(i);
        std::vector<int> flat;
        std::vector<std::pair<int, int>> ranges;
        for (auto &l : levels) {
            ranges.push_back({(int)flat.size(), (int)l.size()});
            flat.insert(flat.end(), l.begin(), l.end());
        }
        if (!flat.empty()) {
            if ((int)flat.size() > ctx->list_cap) {
                if (ctx->d_list) cudaFree(ctx->d_list);
                if (ctx->d_ltree) cudaFree(ctx->d_ltree);
                ctx->d_list = ctx->d_ltree = nullptr;
                ctx->list_cap = (int)flat.size() * 2;
                if (auto s = dev_alloc(ctx, &ctx->d_list, ctx->list_cap)) return s;
                if (auto s = dev_alloc(ctx, &ctx->d_ltree, ctx->list_cap)) return s;
            }
            MW_CK(cudaMemcpyAsync(ctx->d_list, flat.data(), sizeof(int) * flat.size(), cudaMemcpyHostToDevice, st));
            for (auto &r : ranges) {
                launch_mw_down(out->mra, out->t, nullptr, nullptr, ctx->d_list + r.first, r.second, false, st, mixed);
                ctx->launches += r.second > 0;
            }
            for (int l = (int)ranges.size() - 1; l >= 0; l--) {
                launch_mw_up(out->mra, out->t, nullptr, nullptr, ctx->d_list + ranges[l].first, ranges[l].second, st, mixed);
                ctx->launches += ranges[l].second > 0;
            }
            MW_CK(cudaGetLastError());
            MW_CK(cudaStreamSynchronize(st));
        }
        tr.mark("transforms");
    }
    return MWGPU_OK;
}

extern "C" mwgpu_status mwgpu_tree_copy_nodes(mwgpu_ctx *ctx, const mwgpu_tree *src, mwgpu_tree *dst, int n, const int *src_ids,
                                              const int *dst_ids) {
    if (!ctx || !src || !dst) return MWGPU_ERR_BAD_ARG;
    MW_ARG(n >= 0 && (n == 0 || (src_ids && dst_ids)), "invalid node lists");
    MW_ARG(src->mra.K == dst->mra.K, "order mismatch");
    MW_ARG(dst->plans == 0, "tree is held by a plan (destroy the plan first)");
    for (int i = 0; i < n; i++)
        MW_ARG(src_ids[i] >= 0 && src_ids[i] < src->t.n_real && dst_ids[i] >= 0 && dst_ids[i] < dst->t.n_real, "node index out of range");
    if (n == 0) return MWGPU_OK;
    cudaSetDevice(ctx->device);
    if (auto s = ensure_work(ctx, n)) return s;
    MW_CK(cudaMemcpyAsync(ctx->d_work, src_ids, sizeof(int) * n, cudaMemcpyHostToDevice, ctx->stream));
    MW_CK(cudaMemcpyAsync(ctx->d_wtree, dst_ids, sizeof(int) * n, cudaMemcpyHostToDevice, ctx->stream));
    launch_copy_nodes(src->t, dst->t, ctx->d_work, ctx->d_wtree, n, 8 * src->mra.kp1_d, ctx->stream);
    ctx->launches++;
    MW_CK(cudaGetLastError());
    MW_CK(cudaStreamSynchronize(ctx->stream));
    return MWGPU_OK;
}
