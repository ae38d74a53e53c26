// C interface of the host mirror (include/mwhost.h) and mrcpp::apply driven
// through the device C-ABI (include/mwgpu.h).
//
// mwh_apply follows src/treebuilders/apply.cpp:68-93: calcBandWidths, the
// TreeBuilder loop of TreeBuilder.cpp:38-87 with WaveletAdaptor splitting
// (WaveletAdaptor.h:51-54, TreeAdaptor.h:41-52), then TopDown(add) and
// BottomUp transforms and the final square norm.  The per-node work of each
// iteration (ConvolutionCalculator::calcNodeVector) runs on the GPU.
#include <algorithm>
#include <atomic>
#include <chrono>
#include <fstream>
#include <sstream>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <map>
#include <mutex>
#include <string>

#include "../../../include/mwhost.h"
#include "mw_host.h"

using namespace mwh;

struct mwh_mra {
    MRA<3> m;
};
// A host tree and the device copy of it as an apply input (NodeAllocator's
// device mirror, NodeAllocator.cpp:108-113): made by the first apply that
// reads the tree, reused while `version` is unchanged (every host entry that
// changes the tree bumps it), freed with the tree.
struct mwh_tree {
    std::unique_ptr<Tree<3>> t;
    unsigned long long version = 1;
    mwgpu_tree *dev = nullptr;
    unsigned long long dev_version = 0;
    size_t dev_nodes = 0;
    const double *dev_data = nullptr;
};
struct mwh_oper {
    std::unique_ptr<ConvolutionOperator> op;
    std::vector<int> depth, max_transl;
    std::vector<double> blocks, norms;
};

namespace {

// Phase timing of a host entry point when the environment sets MWGPU_TRACE
// (every mark drains the device stream; one line to stderr per call).
struct HostTrace {
    mwgpu_ctx *ctx = nullptr;
    const char *fn;
    bool on;
    std::chrono::steady_clock::time_point t0, last;
    std::string line;
    explicit HostTrace(const char *f) : fn(f), on(std::getenv("MWGPU_TRACE") != nullptr) {
        if (on) t0 = last = std::chrono::steady_clock::now();
    }
    void mark(const std::string &phase) {
        if (!on) return;
        if (ctx) mwgpu_sync(ctx);
        const auto now = std::chrono::steady_clock::now();
        char buf[96];
        std::snprintf(buf, sizeof(buf), " %s=%.3f", phase.c_str(), std::chrono::duration<double, std::milli>(now - last).count());
        line += buf;
        last = now;
    }
    ~HostTrace() {
        if (on)
            std::fprintf(stderr, "[mwh] %s%s total=%.3f ms\n", fn, line.c_str(),
                         std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count());
    }
};

thread_local std::string g_err;
std::mutex g_gpu_mu;
mwgpu_ctx *g_ctx = nullptr;
struct OperKey {
    const mwh_oper *op;
    double prec;
    bool operator<(const OperKey &o) const { return op != o.op ? op < o.op : prec < o.prec; }
};
std::map<OperKey, mwgpu_oper *> g_oper_cache;

int fail(int code, const std::string &msg) {
    g_err = msg;
    return code;
}

template <class F> int guard(F &&f) {
    try {
        return f();
    } catch (const Error &e) {
        return fail(e.code ? e.code : 1, e.what());
    } catch (const std::exception &e) {
        return fail(MWGPU_ERR_INTERNAL, e.what());
    }
}

void fill_desc(const MRA<3> &m, mwgpu_mra_desc *d, double *filters) {
    d->order = m.order();
    d->root_scale = m.rootScale();
    for (int i = 0; i < 3; i++) {
        d->corner[i] = m.world.corner[i];
        d->nbox[i] = m.world.nbox[i];
    }
    d->max_scale = m.maxScale();
    d->sf = m.world.sf[0];
    const int K = m.kp1();
    for (int op = 0; op < 2; op++)
        for (int f = 0; f < 4; f++)
            std::memcpy(filters + ((size_t)op * 4 + f) * K * K, m.basis->sub[op][f].data(), sizeof(double) * K * K);
    d->filters = filters;
}

// flat copy of the non-generated nodes in breadth-first order
void export_tree(const Tree<3> &t, std::vector<int> &order, std::vector<int> &idx, std::vector<int> &child0) {
    order.clear();
    for (auto &lvl : t.nodesByDepth(false))
        for (int i : lvl) order.push_back(i);
    std::vector<int> pos(t.nodes.size(), -1);
    for (size_t j = 0; j < order.size(); j++) pos[order[j]] = (int)j;
    idx.resize(order.size() * 4);
    child0.assign(order.size(), -1);
    for (size_t j = 0; j < order.size(); j++) {
        const auto &n = t.nodes[order[j]];
        idx[4 * j] = n.n;
        idx[4 * j + 1] = n.l[0];
        idx[4 * j + 2] = n.l[1];
        idx[4 * j + 3] = n.l[2];
        if (n.child0 >= 0 && !t.isGen(n.child0)) child0[j] = pos[n.child0];
    }
}

mwgpu_ctx *gpu_ctx(int precision) {
    if (!g_ctx) {
        mwgpu_config cfg{};
        const char *dev = std::getenv("MWGPU_DEVICE");
        cfg.device = dev ? std::atoi(dev) : 0;
        cfg.precision = precision;
        if (int s = mwgpu_init(&g_ctx, &cfg)) throw Error(s, std::string("GPU initialisation failed: ") + mwgpu_last_error(nullptr));
    }
    mwgpu_set_precision(g_ctx, precision);
    return g_ctx;
}

void ck(int s, const char *what) {
    if (s) throw Error(s, std::string(what) + ": " + mwgpu_last_error(g_ctx));
}

// operator tables on the device, cached per (operator, apply precision)
mwgpu_oper *device_operator(mwgpu_ctx *ctx, const mwgpu_mra_desc &md, mwh_oper *operp, double prec) {
    auto it = g_oper_cache.find({operp, prec});
    if (it != g_oper_cache.end()) return it->second;
    mwgpu_oper *dop = nullptr;
    mwgpu_oper_desc od{};
    mwh_oper_desc(operp, &od);
    ck(mwgpu_upload_operator(ctx, &md, &od, prec, &dop), "upload operator");
    g_oper_cache[{operp, prec}] = dop;
    return dop;
}

// Topology of a grid proposal: node index and first child only, children
// appended 8 at a time in the order of Tree::createChildren (no coefficient
// storage, unlike a Tree, whose nodes each carry 8 (k+1)^3 zeroed doubles).
struct GridSketch {
    struct Node {
        int n;
        int l[3];
        int child0;
    };
    std::vector<Node> nodes;
    // the roots of a fresh tree, in its order
    explicit GridSketch(const Tree<3> &fresh) {
        nodes.reserve(4 * fresh.nodes.size() + 64);
        for (const auto &nd : fresh.nodes) nodes.push_back({nd.n, {nd.l[0], nd.l[1], nd.l[2]}, -1});
    }
    void createChildren(int i) {
        const Node p = nodes[i];
        nodes[i].child0 = (int)nodes.size();
        for (int c = 0; c < Tree<3>::tDim; c++)
            nodes.push_back({p.n + 1, {2 * p.l[0] + (c & 1), 2 * p.l[1] + ((c >> 1) & 1), 2 * p.l[2] + ((c >> 2) & 1)}, -1});
    }
};

// State of one output tree inside apply: the TreeBuilder loop of
// TreeBuilder.cpp:38-87 (sNorm from the first iteration, cumulative wNorm,
// maxIter, WaveletAdaptor split), advanced one iteration at a time so that
// several trees can share every device level call.
struct BuildState {
    Tree<3> *tree = nullptr;
    mwgpu_tree *dinp = nullptr, *dout = nullptr;
    std::vector<int> work;
    double sNorm = 0.0, wNorm = 0.0;
    int iter = 0;
    size_t synced = 0;
};

mwgpu_tree *upload_input(mwgpu_ctx *ctx, const mwgpu_mra_desc &md, const Tree<3> &inp, mwh_apply_stats &acc) {
    bool any_gen = false;
    for (size_t i = 0; i < inp.nodes.size() && !any_gen; i++) any_gen = inp.isGen((int)i);
    if (!any_gen) {
        // the device tree takes the host node order: the coefficients go up
        // straight from the tree's own storage (lookups are by node index key)
        const size_t n = inp.nodes.size();
        std::vector<int> idx(4 * n), child0(n);
        std::vector<double> norms(8 * n);
        for (size_t i = 0; i < n; i++) {
            const auto &nd = inp.nodes[i];
            idx[4 * i] = nd.n;
            for (int d = 0; d < 3; d++) idx[4 * i + 1 + d] = nd.l[d];
            child0[i] = nd.child0;
            std::memcpy(&norms[8 * i], nd.norms, sizeof(double) * 8);
        }
        mwgpu_tree_desc fd{(int)n, idx.data(), child0.data(), inp.coefs.data(), norms.data()};
        mwgpu_tree *dinp = nullptr;
        ck(mwgpu_upload_tree(ctx, &md, &fd, &dinp), "upload input tree");
        acc.h2d_bytes += (unsigned long long)(n * inp.nCoefs + norms.size()) * 8 + (idx.size() + child0.size()) * 4;
        return dinp;
    }
    std::vector<int> order, idx, child0;
    export_tree(inp, order, idx, child0);
    std::vector<double> coefs(order.size() * (size_t)inp.nCoefs), norms(order.size() * 8);
    for (size_t j = 0; j < order.size(); j++) {
        std::memcpy(&coefs[j * inp.nCoefs], inp.c(order[j]), sizeof(double) * inp.nCoefs);
        std::memcpy(&norms[j * 8], inp.nodes[order[j]].norms, sizeof(double) * 8);
    }
    mwgpu_tree_desc fd{(int)order.size(), idx.data(), child0.data(), coefs.data(), norms.data()};
    mwgpu_tree *dinp = nullptr;
    ck(mwgpu_upload_tree(ctx, &md, &fd, &dinp), "upload input tree");
    acc.h2d_bytes += (unsigned long long)(coefs.size() + norms.size()) * 8 + (idx.size() + child0.size()) * 4;
    return dinp;
}

// the tree changes: its device input copy is stale.  Versions come from one
// counter, so that (tree, version) never repeats, even for a tree allocated
// where a freed one was.
std::atomic<unsigned long long> g_version_clock{1};
void touch(mwh_tree *t) {
    if (t) t->version = ++g_version_clock;
}

// the device input copy of a host tree: reused while the tree is unchanged,
// else (re)uploaded; owned by the tree
mwgpu_tree *resident_input(mwgpu_ctx *ctx, const mwgpu_mra_desc &md, mwh_tree *inp, mwh_apply_stats &acc) {
    const Tree<3> &t = *inp->t;
    if (inp->dev && inp->dev_version == inp->version && inp->dev_nodes == t.nodes.size() && inp->dev_data == t.coefs.data()) return inp->dev;
    if (inp->dev) mwgpu_free_tree(ctx, inp->dev);
    inp->dev = nullptr;
    inp->dev = upload_input(ctx, md, t, acc);
    inp->dev_version = inp->version;
    inp->dev_nodes = t.nodes.size();
    inp->dev_data = t.coefs.data();
    return inp->dev;
}

// output tree: the host ids are the device ids (nodes are only appended)
mwgpu_tree *create_output(mwgpu_ctx *ctx, const mwgpu_mra_desc &md, Tree<3> &out, mwh_apply_stats &acc) {
    out.clearGenerated();
    std::vector<int> oidx(out.nodes.size() * 4), oc0(out.nodes.size(), -1);
    for (size_t i = 0; i < out.nodes.size(); i++) {
        oidx[4 * i] = out.nodes[i].n;
        for (int d = 0; d < 3; d++) oidx[4 * i + 1 + d] = out.nodes[i].l[d];
        oc0[i] = out.nodes[i].child0;
    }
    mwgpu_tree_desc gd{(int)out.nodes.size(), oidx.data(), oc0.data(), nullptr, nullptr};
    mwgpu_tree *dout = nullptr;
    ck(mwgpu_create_tree(ctx, &md, &gd, &dout), "create output tree");
    acc.h2d_bytes += (oidx.size() + oc0.size()) * 4;
    return dout;
}

// Fixed-grid applies (maxIter = 0 onto fresh output grids: no norm
// screening), of one (input, output) pair or a batch of them, that repeat
// with the same operator, output grids and input topologies -- the applies of
// an SCF loop once its grids have settled -- replay
// a level plan (mwgpu_plan: GenNode values, work list, contraction, reduction,
// TopDown and BottomUp as one CUDA graph) instead of building the level again.
// A plan owns device copies of its input and output trees (the input tree's
// resident copy moves to a new plan when it is current); new input values go
// into the plan's input copy (mwgpu_tree_update_coefs).  The first apply of a
// kind creates the plan (with the autotuner: about 30 timed contractions);
// up to kPlanCache plans are kept, the least recently used is dropped.
// MWH_NO_PLAN_CACHE=1 builds every level instead.
struct PlanTree {
    unsigned long long out_hash = 0, inp_hash = 0;
    size_t out_n = 0, inp_n = 0;
    const mwh_tree *inp = nullptr;     // the input whose values the input copy holds
    unsigned long long inp_version = 0;
    const double *inp_data = nullptr;
    mwgpu_tree *dinp = nullptr, *dout = nullptr;
};
struct PlanEntry {
    const mwgpu_oper *dop = nullptr;
    int precision = 0;
    double prec = 0.0;
    std::vector<PlanTree> trees;       // the (input, output) pairs of the batch
    mwgpu_plan *plan = nullptr;
    unsigned long long used = 0;
};
constexpr size_t kPlanCache = 4;
std::vector<PlanEntry> g_plans;
unsigned long long g_plan_clock = 0;

// FNV-1a over the topology in storage order (node index and first child)
unsigned long long topo_hash(const Tree<3> &t) {
    unsigned long long h = 1469598103934665603ull;
    auto mix = [&](unsigned v) {
        h ^= v;
        h *= 1099511628211ull;
    };
    for (const auto &nd : t.nodes) {
        mix((unsigned)nd.n);
        for (int d = 0; d < 3; d++) mix((unsigned)nd.l[d]);
        mix((unsigned)nd.child0);
    }
    mix((unsigned)t.nodes.size());
    return h;
}

void plan_entry_free(mwgpu_ctx *ctx, PlanEntry &e) {
    if (e.plan) mwgpu_plan_destroy(ctx, e.plan);
    for (auto &t : e.trees) {
        if (t.dout) mwgpu_free_tree(ctx, t.dout);
        if (t.dinp) mwgpu_free_tree(ctx, t.dinp);
    }
    e = PlanEntry{};
}

// the plans that use a device operator (before it is freed)
void drop_plans(mwgpu_ctx *ctx, const mwgpu_oper *dop) {
    for (size_t i = 0; i < g_plans.size();) {
        if (g_plans[i].dop == dop) {
            plan_entry_free(ctx, g_plans[i]);
            g_plans.erase(g_plans.begin() + i);
        } else {
            i++;
        }
    }
}

// The fixed-grid apply of nt (input, output) pairs through a cached plan;
// false where it does not apply (then the caller builds the levels).  Same
// results as the built level: the plan's level is the level
// mwgpu_apply_level_batch computes on these nodes.
bool apply_planned(mwgpu_ctx *ctx, const mwgpu_mra_desc &md, mwgpu_oper *dop, double prec, int precision, int nt, mwh_tree **outs,
                   mwh_tree **inps, mwh_apply_stats &acc, HostTrace &ht) {
    if (std::getenv("MWH_NO_PLAN_CACHE")) return false;
    std::vector<PlanTree> key(nt);
    for (int t = 0; t < nt; t++) {
        Tree<3> &out = *outs[t]->t;
        const Tree<3> &inp = *inps[t]->t;
        out.clearGenerated();
        if (!(out.squareNorm < 0.0) || out.nodes.empty()) return false;
        for (size_t i = 0; i < inp.nodes.size(); i++)
            if (inp.isGen((int)i)) return false;
        key[t].out_hash = topo_hash(out);
        key[t].inp_hash = topo_hash(inp);
        key[t].out_n = out.nodes.size();
        key[t].inp_n = inp.nodes.size();
    }
    ht.mark("key");
    auto same = [&](const PlanEntry &x) {
        if (x.dop != dop || x.precision != precision || x.prec != prec || (int)x.trees.size() != nt) return false;
        for (int t = 0; t < nt; t++)
            if (x.trees[t].out_hash != key[t].out_hash || x.trees[t].inp_hash != key[t].inp_hash || x.trees[t].out_n != key[t].out_n ||
                x.trees[t].inp_n != key[t].inp_n)
                return false;
        return true;
    };
    PlanEntry *e = nullptr;
    for (auto &x : g_plans)
        if (same(x)) e = &x;
    acc.planned = 1;
    if (!e) {
        if (g_plans.size() >= kPlanCache) {
            auto lru = std::min_element(g_plans.begin(), g_plans.end(), [](const PlanEntry &a, const PlanEntry &b) { return a.used < b.used; });
            plan_entry_free(ctx, *lru);
            g_plans.erase(lru);
        }
        PlanEntry ne;
        ne.dop = dop;
        ne.precision = precision;
        ne.prec = prec;
        ne.trees = key;
        try {
            std::vector<int> wtree, work;
            std::vector<double> sq(nt);
            std::vector<mwgpu_tree *> dins(nt), douts(nt);
            for (int t = 0; t < nt; t++) {
                PlanTree &pt = ne.trees[t];
                mwh_tree *inpp = inps[t];
                const Tree<3> &inp = *inpp->t;
                Tree<3> &out = *outs[t]->t;
                // the tree's current device copy moves to the plan (no second
                // upload); otherwise the plan uploads its own
                if (inpp->dev && inpp->dev_version == inpp->version && inpp->dev_nodes == pt.inp_n && inpp->dev_data == inp.coefs.data()) {
                    pt.dinp = inpp->dev;
                    inpp->dev = nullptr;
                    inpp->dev_version = 0;
                } else {
                    pt.dinp = upload_input(ctx, md, inp, acc);
                }
                pt.dout = create_output(ctx, md, out, acc);
                pt.inp = inpp;
                pt.inp_version = inpp->version;
                pt.inp_data = inp.coefs.data();
                dins[t] = pt.dinp;
                douts[t] = pt.dout;
                sq[t] = out.squareNorm;
                // ConvolutionCalculator::getInitialWorkVector: all nodes of the output tree
                for (auto &lvl : out.nodesByDepth(false))
                    for (int i : lvl) {
                        wtree.push_back(t);
                        work.push_back(i);
                    }
            }
            ck(mwgpu_plan_create(ctx, dop, nt, dins.data(), douts.data(), wtree.data(), work.data(), (int)work.size(), prec, sq.data(),
                                 MWGPU_PLAN_TRANSFORMS | MWGPU_PLAN_AUTOTUNE, &ne.plan),
               "create level plan");
        } catch (...) {
            plan_entry_free(ctx, ne);
            throw;
        }
        g_plans.push_back(ne);
        e = &g_plans.back();
        acc.planned = 2;
    } else {
        // new input values, same topology: into the plan's input copies
        std::vector<double> norms;
        for (int t = 0; t < nt; t++) {
            PlanTree &pt = e->trees[t];
            mwh_tree *inpp = inps[t];
            const Tree<3> &inp = *inpp->t;
            if (pt.inp == inpp && pt.inp_version == inpp->version && pt.inp_data == inp.coefs.data()) continue;
            const size_t n_in = inp.nodes.size();
            norms.resize(8 * n_in);
            for (size_t i = 0; i < n_in; i++) std::memcpy(&norms[8 * i], inp.nodes[i].norms, sizeof(double) * 8);
            ck(mwgpu_tree_update_coefs(ctx, pt.dinp, inp.coefs.data(), norms.data()), "update input values");
            acc.h2d_bytes += (unsigned long long)(n_in * (size_t)inp.nCoefs + norms.size()) * 8;
            pt.inp = inpp;
            pt.inp_version = inpp->version;
            pt.inp_data = inp.coefs.data();
        }
    }
    ht.mark(acc.planned == 2 ? "plan" : "input");
    e->used = ++g_plan_clock;
    mwgpu_level_stats ls{};
    ck(mwgpu_plan_execute(ctx, e->plan, &ls), "execute level plan");
    ht.mark("level");
    int out_nodes = 0;
    std::vector<double> nn;
    for (int t = 0; t < nt; t++) {
        Tree<3> &out = *outs[t]->t;
        nn.resize(out.nodes.size() * 8);
        ck(mwgpu_download_tree(ctx, e->trees[t].dout, out.coefs.data(), nn.data()), "download output tree");
        acc.d2h_bytes += (unsigned long long)(out.coefs.size() + nn.size()) * 8;
        for (size_t i = 0; i < out.nodes.size(); i++) {
            double s2 = 0.0;
            for (int c = 0; c < 8; c++) {
                out.nodes[i].norms[c] = nn[i * 8 + c];
                s2 += nn[i * 8 + c] * nn[i * 8 + c];
            }
            out.nodes[i].squareNorm = s2;
            out.nodes[i].flags |= F_HASCOEFS;
        }
        out.calcSquareNorm();
        out_nodes += (int)out.nodes.size();
    }
    ht.mark("download");
    acc.node_terms = ls.node_terms;
    acc.components = ls.components;
    acc.band_nodes = ls.band_nodes;
    acc.gen_nodes = ls.gen_nodes;
    acc.device_ms = ls.device_ms;
    acc.contract_ms = ls.contract_ms;
    acc.iterations = 1;
    acc.out_nodes = out_nodes;
    return true;
}

// children made by the split step are mirrored to the device before the next
// iteration computes them
void sync_new(mwgpu_ctx *ctx, BuildState &b, mwh_apply_stats &acc) {
    const Tree<3> &t = *b.tree;
    if (t.nodes.size() <= b.synced) return;
    int n = (int)(t.nodes.size() - b.synced);
    std::vector<int> nidx(4 * (size_t)n), pids, pc0;
    for (int j = 0; j < n; j++) {
        const auto &nd = t.nodes[b.synced + j];
        nidx[4 * j] = nd.n;
        for (int d = 0; d < 3; d++) nidx[4 * j + 1 + d] = nd.l[d];
        if (nd.parent >= 0 && t.nodes[nd.parent].child0 == (int)(b.synced + j)) {
            pids.push_back(nd.parent);
            pc0.push_back(t.nodes[nd.parent].child0);
        }
    }
    ck(mwgpu_tree_add_nodes(ctx, b.dout, n, nidx.data(), (int)pids.size(), pids.data(), pc0.data()), "add output nodes");
    acc.h2d_bytes += (nidx.size() + pids.size() + pc0.size()) * 4 + t.nodes.size() * 4;
    b.synced = t.nodes.size();
}

// The precision function of the precTrees form of apply (apply.cpp:221-229):
// precFac(idx) = 1 / max_i sqrt(getNode(idx).getMaxSquareNorm()) over the
// precision trees after makeMaxSquareNorms; 1 without precision trees.  A node
// a precision tree lacks is generated for its norm alone (the tree is read only).
struct PrecScale {
    std::vector<const Tree<3> *> trees;
    std::vector<std::vector<double>> msq;
    double operator()(int n, const int *l) const {
        if (trees.empty()) return 1.0;
        double maxNorm = 0.0;
        for (size_t i = 0; i < trees.size(); i++) {
            const int id = trees[i]->find(n, l);
            const double v = id >= 0 ? msq[i][id] : trees[i]->genScaledSquareNorm(n, l);
            maxNorm = std::max(maxNorm, std::sqrt(v));
        }
        return 1.0 / maxNorm;
    }
};

// mrcpp::apply (apply.cpp:68-93) for nt independent (out, inp) pairs with one
// operator.  Each TreeBuilder iteration of all trees still building is one
// device level call; the transforms of all trees share their launches.
// scale (nt = 1 only): the precTrees form (apply.cpp:214-251), the precision
// scaled per output node in the screening and in the split test.
int apply_impl(double prec, int nt, mwh_tree **outs, mwh_oper *operp, mwh_tree **inps, int max_iter, int abs_prec, int precision,
               mwh_apply_stats *stats, const PrecScale *scale = nullptr) {
    if (scale && nt != 1) return fail(1, "precision trees need a single (out, inp) pair");
    ConvolutionOperator &op = *operp->op;
    for (int t = 0; t < nt; t++) {
        if (!(*outs[t]->t->mra == *inps[t]->t->mra)) return fail(1, "Incompatible MRA");
        if (!(*outs[t]->t->mra == op.mra)) return fail(1, "Operator MRA differs from the function MRA");
    }
    auto t0 = std::chrono::steady_clock::now();
    std::lock_guard<std::mutex> lk(g_gpu_mu);
    mwgpu_ctx *ctx = gpu_ctx(precision);
    const MRA<3> &mra = *outs[0]->t->mra;
    std::vector<double> filters(8 * (size_t)mra.kp1() * mra.kp1());
    mwgpu_mra_desc md{};
    fill_desc(mra, &md, filters.data());

    mwgpu_oper *dop = device_operator(ctx, md, operp, prec);
    HostTrace ht("apply");
    ht.ctx = ctx;
    mwh_apply_stats acc{};
    unsigned long long l0 = 0, l1 = 0;
    mwgpu_launch_count(ctx, &l0);
    std::vector<BuildState> bs(nt);
    for (int t = 0; t < nt; t++) touch(outs[t]);
    if (!scale && max_iter == 0 && apply_planned(ctx, md, dop, prec, precision, nt, outs, inps, acc, ht)) {
        ht.mark("norms");
        mwgpu_launch_count(ctx, &l1);
        acc.launches = l1 - l0;
        acc.wall_ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
        if (stats) *stats = acc;
        return 0;
    }
    // the input trees' device copies belong to the trees
    auto release = [&] {
        for (auto &b : bs) {
            if (b.dout) mwgpu_free_tree(ctx, b.dout);
            b.dout = b.dinp = nullptr;
        }
    };
    try {
        for (int t = 0; t < nt; t++) {
            BuildState &b = bs[t];
            b.tree = outs[t]->t.get();
            // room for the refinement without moving the coefficients on every
            // growth step (untouched capacity costs no memory; a fixed grid
            // does not grow)
            if (max_iter != 0) {
                const size_t guess = b.tree->nodes.size() + 2 * inps[t]->t->nodes.size() + 4096;
                b.tree->nodes.reserve(guess);
                b.tree->coefs.reserve(guess * (size_t)b.tree->nCoefs);
            }
            b.dinp = resident_input(ctx, md, inps[t], acc);
            // each apply makes its own GenNodes, as the reference deletes them at
            // the end of apply (apply.cpp:86-87): statistics do not depend on
            // earlier applies
            ck(mwgpu_tree_clear_generated(ctx, b.dinp), "clear generated nodes");
            ht.mark("input");
            b.dout = create_output(ctx, md, *b.tree, acc);
            ht.mark("output");
            b.synced = b.tree->nodes.size();
            // ConvolutionCalculator::getInitialWorkVector: all nodes of the output tree
            for (auto &lvl : b.tree->nodesByDepth(false))
                for (int i : lvl) b.work.push_back(i);
        }
        ht.mark("upload");
        std::vector<int> wtree, wnode;
        std::vector<double> sq(nt), nbuf, pfac;
        std::vector<mwgpu_tree *> dins(nt), douts(nt);
        for (int t = 0; t < nt; t++) {
            dins[t] = bs[t].dinp;
            douts[t] = bs[t].dout;
        }
        while (true) {
            wtree.clear();
            wnode.clear();
            for (int t = 0; t < nt; t++) {
                BuildState &b = bs[t];
                if (b.work.empty()) continue;
                sync_new(ctx, b, acc);
                for (int i : b.work) {
                    wtree.push_back(t);
                    wnode.push_back(i);
                }
            }
            if (wnode.empty()) break;
            for (int t = 0; t < nt; t++) sq[t] = bs[t].tree->squareNorm;
            const int n = (int)wnode.size();
            nbuf.resize((size_t)n * 8);
            mwgpu_level_stats ls{};
            if (scale) {
                pfac.resize(n);
                for (int j = 0; j < n; j++) {
                    const auto &nd = bs[0].tree->nodes[wnode[j]];
                    pfac[j] = (*scale)(nd.n, nd.l);
                }
                ck(mwgpu_apply_level_scaled(ctx, dop, dins[0], douts[0], wnode.data(), n, prec, sq[0], pfac.data(), nbuf.data(), &ls),
                   "apply level");
                acc.h2d_bytes += (unsigned long long)n * 8;
            } else if (nt == 1)
                ck(mwgpu_apply_level(ctx, dop, dins[0], douts[0], wnode.data(), n, prec, sq[0], nbuf.data(), &ls), "apply level");
            else
                ck(mwgpu_apply_level_batch(ctx, dop, nt, dins.data(), douts.data(), wtree.data(), wnode.data(), n, prec, sq.data(), nbuf.data(),
                                           &ls),
                   "apply level");
            ht.mark("level" + std::to_string(acc.iterations));
            acc.h2d_bytes += (unsigned long long)n * (nt == 1 ? 4 : 8);
            acc.d2h_bytes += (unsigned long long)n * 8 * 8;
            for (int j = 0; j < n; j++) {
                Tree<3> &t = *bs[wtree[j]].tree;
                auto &nd = t.nodes[wnode[j]];
                double s2 = 0.0;
                for (int c = 0; c < 8; c++) {
                    nd.norms[c] = nbuf[(size_t)j * 8 + c];
                    s2 += nd.norms[c] * nd.norms[c];
                }
                nd.squareNorm = s2;
                nd.flags |= F_HASCOEFS;
            }
            acc.node_terms += ls.node_terms;
            acc.components += ls.components;
            acc.band_nodes += ls.band_nodes;
            acc.gen_nodes += ls.gen_nodes;
            acc.device_ms += ls.device_ms;
            acc.contract_ms += ls.contract_ms;
            acc.iterations++;
            // TreeBuilder::build bookkeeping and split, per tree (TreeBuilder.cpp:49-80)
            for (int t = 0; t < nt; t++) {
                BuildState &b = bs[t];
                if (b.work.empty()) continue;
                Tree<3> &tree = *b.tree;
                if (b.iter == 0) {
                    b.sNorm = 0.0;
                    for (int i : b.work)
                        if (tree.depth(i) >= 0) b.sNorm += tree.scalingNorm(i);
                }
                for (int i : b.work)
                    if (tree.depth(i) >= 0) b.wNorm += tree.waveletNorm(i);
                tree.squareNorm = (b.sNorm < 0.0 || b.wNorm < 0.0) ? -1.0 : b.sNorm + b.wNorm;
                if (b.iter >= max_iter && max_iter >= 0) b.work.clear();
                std::vector<int> next;
                for (size_t j = 0; j < b.work.size(); j++) {
                    const int i = b.work[j];
                    if (tree.isBranch(i)) continue;
                    if (tree.nodes[i].n + 2 > mra.maxScale()) continue;
                    // WaveletAdaptor::splitNode: prec * precFac (WaveletAdaptor.h:51-54)
                    const double p = scale ? prec * pfac[j] : prec;
                    if (split_check(tree, i, p, 1.0, abs_prec != 0)) {
                        tree.createChildren(i, false);
                        int c0 = tree.nodes[i].child0;
                        for (int c = 0; c < Tree<3>::tDim; c++) next.push_back(c0 + c);
                    }
                }
                b.work.swap(next);
                b.iter++;
            }
        }
        for (auto &b : bs) sync_new(ctx, b, acc);
        ht.mark("split");
        auto t1 = std::chrono::steady_clock::now();
        if (nt == 1) {
            ck(mwgpu_transform(ctx, douts[0], MWGPU_TOPDOWN, 0), "TopDown transform");
            ck(mwgpu_transform(ctx, douts[0], MWGPU_BOTTOMUP, 1), "BottomUp transform");
        } else {
            ck(mwgpu_transform_batch(ctx, nt, douts.data(), MWGPU_TOPDOWN, 0), "TopDown transform");
            ck(mwgpu_transform_batch(ctx, nt, douts.data(), MWGPU_BOTTOMUP, 1), "BottomUp transform");
        }
        ht.mark("transforms");
        int out_nodes = 0;
        for (auto &b : bs) {
            Tree<3> &out = *b.tree;
            std::vector<double> nn(out.nodes.size() * 8);
            ck(mwgpu_download_tree(ctx, b.dout, out.coefs.data(), nn.data()), "download output tree");
            acc.d2h_bytes += (unsigned long long)(out.coefs.size() + nn.size()) * 8;
            for (size_t i = 0; i < out.nodes.size(); i++) {
                double s2 = 0.0;
                for (int c = 0; c < 8; c++) {
                    out.nodes[i].norms[c] = nn[i * 8 + c];
                    s2 += nn[i * 8 + c] * nn[i * 8 + c];
                }
                out.nodes[i].squareNorm = s2;
                out.nodes[i].flags |= F_HASCOEFS;
            }
            out.calcSquareNorm();
            out_nodes += (int)out.nodes.size();
        }
        ht.mark("download");
        auto t2 = std::chrono::steady_clock::now();
        acc.transform_ms = std::chrono::duration<double, std::milli>(t2 - t1).count();
        acc.out_nodes = out_nodes;
    } catch (...) {
        release();
        throw;
    }
    mwgpu_launch_count(ctx, &l1);
    acc.launches = l1 - l0;
    release();
    acc.wall_ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
    if (stats) *stats = acc;
    return 0;
}
// CopyAdaptor (CopyAdaptor.cpp:55-71) with TreeBuilder: refine `out` wherever a
// child of a node, shifted by up to bw[d] boxes in direction d, is a node of `inp`
void copy_adapt(Tree<3> &out, const Tree<3> &inp, const int bw[3]) {
    const int maxScale = out.mra->maxScale();
    std::vector<int> work = out.endNodes(), next;
    while (!work.empty()) {
        next.clear();
        for (int i : work) {
            if (out.isBranch(i) || out.nodes[i].n + 2 > maxScale) continue;
            const auto nd = out.nodes[i];
            bool split = false;
            for (int c = 0; c < 8 && !split; c++) {
                const int cl[3] = {2 * nd.l[0] + (c & 1), 2 * nd.l[1] + ((c >> 1) & 1), 2 * nd.l[2] + ((c >> 2) & 1)};
                for (int d = 0; d < 3 && !split; d++)
                    for (int w = -bw[d]; w <= bw[d] && !split; w++) {
                        int l[3] = {cl[0], cl[1], cl[2]};
                        l[d] += w;
                        const int id = inp.find(nd.n + 1, l);
                        split = id >= 0 && !inp.isGen(id);
                    }
            }
            if (!split) continue;
            out.createChildren(i, false);
            const int c0 = out.nodes[i].child0;
            for (int c = 0; c < 8; c++) next.push_back(c0 + c);
        }
        work.swap(next);
    }
}

// apply(out, DerivativeOperator, inp, dir) (apply.cpp:379-412): the output grid is
// the input grid widened by the band along dir, the end nodes are computed on
// the device, then BottomUp and the square norm
int apply_derivative_impl(mwh_tree *outp, mwh_oper *operp, mwh_tree *inpp, int dir, mwh_apply_stats *stats) {
    ConvolutionOperator &op = *operp->op;
    if (op.derivOrder <= 0) return fail(1, "not a derivative operator");
    if (dir < 0 || dir > 2) return fail(1, "invalid apply direction");
    if (!(*outp->t->mra == *inpp->t->mra)) return fail(1, "Incompatible MRA");
    if (!(*outp->t->mra == op.mra)) return fail(1, "Operator MRA differs from the function MRA");
    Tree<3> &out = *outp->t;
    for (size_t i = 0; i < out.nodes.size(); i++)
        if (out.isBranch((int)i)) return fail(1, "the output function must contain only empty root nodes");
    auto t0 = std::chrono::steady_clock::now();
    // oper.calcBandWidths(1.0): band widths 0 or 1
    op.calcBandWidths(1.0);
    int bw[3] = {0, 0, 0};
    bw[dir] = std::max(op.getMaxBandWidth(-1), 0);
    copy_adapt(out, *inpp->t, bw);
    std::lock_guard<std::mutex> lk(g_gpu_mu);
    mwgpu_ctx *ctx = gpu_ctx(MWGPU_PREC_FP64);
    const MRA<3> &mra = *out.mra;
    std::vector<double> filters(8 * (size_t)mra.kp1() * mra.kp1());
    mwgpu_mra_desc md{};
    fill_desc(mra, &md, filters.data());
    mwgpu_oper *dop = device_operator(ctx, md, operp, 1.0);
    mwh_apply_stats acc{};
    unsigned long long l0 = 0, l1 = 0;
    mwgpu_launch_count(ctx, &l0);
    mwgpu_tree *dinp = nullptr, *dout = nullptr;
    try {
        dinp = upload_input(ctx, md, *inpp->t, acc);
        dout = create_output(ctx, md, out, acc);
        // DerivativeCalculator::getInitialWorkVector: the end nodes
        std::vector<int> work = out.endNodes();
        mwgpu_level_stats ls{};
        ck(mwgpu_apply_derivative(ctx, dop, dinp, dout, work.data(), (int)work.size(), dir, op.derivOrder, &ls), "apply derivative");
        ck(mwgpu_transform(ctx, dout, MWGPU_BOTTOMUP, 1), "BottomUp transform");
        std::vector<double> nn(out.nodes.size() * 8);
        ck(mwgpu_download_tree(ctx, dout, out.coefs.data(), nn.data()), "download output tree");
        acc.d2h_bytes += (unsigned long long)(out.coefs.size() + nn.size()) * 8;
        for (size_t i = 0; i < out.nodes.size(); i++) {
            double s2 = 0.0;
            for (int c = 0; c < 8; c++) {
                out.nodes[i].norms[c] = nn[i * 8 + c];
                s2 += nn[i * 8 + c] * nn[i * 8 + c];
            }
            out.nodes[i].squareNorm = s2;
            out.nodes[i].flags |= F_HASCOEFS;
        }
        out.calcSquareNorm();
        acc.node_terms = ls.node_terms;
        acc.components = ls.components;
        acc.band_nodes = ls.band_nodes;
        acc.gen_nodes = ls.gen_nodes;
        acc.device_ms = ls.device_ms;
        acc.contract_ms = ls.contract_ms;
        acc.iterations = 1;
        acc.out_nodes = (int)out.nodes.size();
    } catch (...) {
        if (dout) mwgpu_free_tree(ctx, dout);
        if (dinp) mwgpu_free_tree(ctx, dinp);
        throw;
    }
    mwgpu_free_tree(ctx, dout);
    mwgpu_free_tree(ctx, dinp);
    mwgpu_launch_count(ctx, &l1);
    acc.launches = l1 - l0;
    acc.wall_ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
    if (stats) *stats = acc;
    return 0;
}

// project(prec, out, GaussExp, maxIter, absPrec) (project.cpp:47-66) with the
// node computations on the device: TreeBuilder + WaveletAdaptor on the host,
// ProjectionCalculator::calcNode per iteration through mwgpu_project_level,
// BottomUp on the device, then the coefficients come back
// func (optional): any function, evaluated on the host at the children's
// quadrature points of each level (the RepresentableFunction of
// ProjectionCalculator), in batches of at most kProjectBatch points; the
// transforms and norms of the level run on the device
int project_device_impl(double prec, Tree<3> &tree, int n, const double *coef, const double *ex, const double *pos, int max_iter, bool abs_prec,
                        mwh_apply_stats *stats, const BatchFunc *func = nullptr) {
    auto t0 = std::chrono::steady_clock::now();
    std::vector<double> gauss(5 * (size_t)n);
    for (int j = 0; j < n; j++) {
        gauss[5 * j] = coef[j];
        gauss[5 * j + 1] = ex[j];
        for (int d = 0; d < 3; d++) gauss[5 * j + 2 + d] = pos[3 * j + d];
    }
    const MRA<3> &mra = *tree.mra;
    const ScalingBasis &basis = *mra.basis;
    std::lock_guard<std::mutex> lk(g_gpu_mu);
    mwgpu_ctx *ctx = gpu_ctx(MWGPU_PREC_FP64);
    std::vector<double> filters(8 * (size_t)mra.kp1() * mra.kp1());
    mwgpu_mra_desc md{};
    fill_desc(mra, &md, filters.data());
    mwh_apply_stats acc{};
    BuildState b;
    b.tree = &tree;
    tree.clearGenerated();
    b.dout = create_output(ctx, md, tree, acc);
    b.synced = tree.nodes.size();
    try {
        std::vector<double> nbuf, pts, vals;
        const int K = mra.kp1(), K3 = K * K * K;
        auto calc = [&](Tree<3> &t, const std::vector<int> &work) {
            sync_new(ctx, b, acc);
            nbuf.resize(8 * work.size());
            if (func) {
                // MWNode::getExpandedChildPts (MWNode.cpp:854-935), scaled by the world's factors
                const size_t np = work.size() * 8 * (size_t)K3;
                pts.resize(3 * np);
                vals.resize(np);
                for (size_t j = 0; j < work.size(); j++) {
                    const auto &nd = t.nodes[work[j]];
                    const double h = std::ldexp(1.0, -(nd.n + 1));
                    for (int e = 0; e < 8 * K3; e++) {
                        const int ct = e / K3, q = e % K3;
                        const int qd[3] = {q % K, (q / K) % K, q / (K * K)};
                        for (int d = 0; d < 3; d++)
                            pts[3 * (j * 8 * K3 + e) + d] = mra.world.sf[d] * (h * (basis.roots[qd[d]] + 2.0 * nd.l[d] + ((ct >> d) & 1)));
                    }
                }
                for (size_t b0 = 0; b0 < np; b0 += kProjectBatch) {
                    const size_t nb = std::min(kProjectBatch, np - b0);
                    (*func)((long long)nb, pts.data() + 3 * b0, vals.data() + b0);
                }
                acc.h2d_bytes += np * 8;
                ck(mwgpu_project_level_values(ctx, b.dout, vals.data(), basis.vcMap.data(), basis.roots.data(), work.data(), (int)work.size(),
                                              nbuf.data()),
                   "projection level");
            } else {
                ck(mwgpu_project_level(ctx, b.dout, n, gauss.data(), basis.vcMap.data(), basis.roots.data(), work.data(), (int)work.size(),
                                       nbuf.data()),
                   "projection level");
            }
            for (size_t j = 0; j < work.size(); j++) {
                auto &nd = t.nodes[work[j]];
                double s2 = 0.0;
                for (int c = 0; c < 8; c++) {
                    nd.norms[c] = nbuf[8 * j + c];
                    s2 += nd.norms[c] * nd.norms[c];
                }
                nd.squareNorm = s2;
                nd.flags |= F_HASCOEFS;
            }
            acc.iterations++;
        };
        auto split = [prec, abs_prec](const Tree<3> &t, int i) { return split_check(t, i, prec, 1.0, abs_prec); };
        tree_build<3>(tree, tree.endNodes(), calc, split, max_iter, mra.maxScale());
        sync_new(ctx, b, acc);
        ck(mwgpu_transform(ctx, b.dout, MWGPU_BOTTOMUP, 1), "BottomUp transform");
        std::vector<double> nn(tree.nodes.size() * 8);
        ck(mwgpu_download_tree(ctx, b.dout, tree.coefs.data(), nn.data()), "download projected tree");
        for (size_t i = 0; i < tree.nodes.size(); i++) {
            double s2 = 0.0;
            for (int c = 0; c < 8; c++) {
                tree.nodes[i].norms[c] = nn[i * 8 + c];
                s2 += nn[i * 8 + c] * nn[i * 8 + c];
            }
            tree.nodes[i].squareNorm = s2;
            tree.nodes[i].flags |= F_HASCOEFS;
        }
        tree.calcSquareNorm();
    } catch (...) {
        mwgpu_free_tree(ctx, b.dout);
        throw;
    }
    mwgpu_free_tree(ctx, b.dout);
    acc.out_nodes = (int)tree.nodes.size();
    acc.wall_ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
    if (stats) *stats = acc;
    return 0;
}

// add (add.cpp:58-83) / multiply (multiply.cpp:70-101, WaveletAdaptor) with
// the node computations on the device: TreeBuilder + WaveletAdaptor on the
// host, AdditionCalculator / MultiplicationCalculator::calcNode per iteration
// through mwgpu_combine_level, BottomUp on the device
// max_norms: multiply's MultiplicationAdaptor (multiply.cpp:104-108,
// MultiplicationAdaptor.h:45-65) instead of the wavelet adaptor: a node splits
// when maxW0 maxS1 + maxW1 maxS0 + maxW0 maxW1 > prec (max norms of the two
// inputs at the node after makeMaxSquareNorms; a node an input lacks has its
// generated scaling norm and no wavelet norm) and one input has children
// there.  (The reference counts an input node with generated children as
// a branch too; on an output tree that starts from its root nodes no such node
// is tested, so the rules agree.)
int combine_device_impl(int op, double prec, Tree<3> &out, int n, const double *c, mwh_tree *const *inps, int max_iter, bool abs_prec,
                        mwh_apply_stats *stats, bool max_norms = false) {
    for (int j = 0; j < n; j++)
        if (!(*inps[j]->t->mra == *out.mra)) return fail(1, "Incompatible MRA");
    if (max_norms && (op != MWGPU_COMBINE_MULTIPLY || n != 2)) return fail(1, "Invalid tree vec size: the max-norm adaptor multiplies two functions");
    std::vector<double> msq[2], mwsq[2];
    if (max_norms)
        for (int j = 0; j < 2; j++) {
            msq[j] = inps[j]->t->maxSquareNorms();
            mwsq[j] = inps[j]->t->maxWSquareNorms();
        }
    auto t0 = std::chrono::steady_clock::now();
    const MRA<3> &mra = *out.mra;
    const ScalingBasis &basis = *mra.basis;
    std::lock_guard<std::mutex> lk(g_gpu_mu);
    mwgpu_ctx *ctx = gpu_ctx(MWGPU_PREC_FP64);
    std::vector<double> filters(8 * (size_t)mra.kp1() * mra.kp1());
    mwgpu_mra_desc md{};
    fill_desc(mra, &md, filters.data());
    mwh_apply_stats acc{};
    std::vector<mwgpu_tree *> dins(n, nullptr);
    BuildState b;
    b.tree = &out;
    auto release = [&] {
        if (b.dout) mwgpu_free_tree(ctx, b.dout);
        for (auto *d : dins)
            if (d) mwgpu_free_tree(ctx, d);
    };
    try {
        for (int j = 0; j < n; j++) dins[j] = upload_input(ctx, md, *inps[j]->t, acc);
        out.clearGenerated();
        b.dout = create_output(ctx, md, out, acc);
        b.synced = out.nodes.size();
        std::vector<double> nbuf;
        auto calc = [&](Tree<3> &t, const std::vector<int> &work) {
            sync_new(ctx, b, acc);
            nbuf.resize(8 * work.size());
            ck(mwgpu_combine_level(ctx, op, n, dins.data(), c, basis.cvMap.data(), basis.vcMap.data(), b.dout, work.data(), (int)work.size(),
                                   nbuf.data()),
               op == MWGPU_COMBINE_ADD ? "addition level" : "multiplication level");
            for (size_t j = 0; j < work.size(); j++) {
                auto &nd = t.nodes[work[j]];
                double s2 = 0.0;
                for (int q = 0; q < 8; q++) {
                    nd.norms[q] = nbuf[8 * j + q];
                    s2 += nd.norms[q] * nd.norms[q];
                }
                nd.squareNorm = s2;
                nd.flags |= F_HASCOEFS;
            }
            acc.iterations++;
        };
        auto split = [&](const Tree<3> &t, int i) {
            if (!max_norms) return split_check(t, i, prec, 1.0, abs_prec);
            const auto &nd = t.nodes[i];
            double S[2], W[2];
            bool leaf[2];
            for (int j = 0; j < 2; j++) {
                const Tree<3> &f = *inps[j]->t;
                const int id = f.find(nd.n, nd.l);
                if (id >= 0) {
                    S[j] = std::sqrt(msq[j][id]);
                    W[j] = std::sqrt(mwsq[j][id]);
                    const int c0 = f.nodes[id].child0;
                    leaf[j] = c0 < 0 || f.isGen(c0);
                } else {
                    S[j] = std::sqrt(f.genScaledSquareNorm(nd.n, nd.l));
                    W[j] = 0.0;
                    leaf[j] = true;
                }
            }
            const double multNorm = W[0] * S[1] + W[1] * S[0] + W[0] * W[1];
            return multNorm > prec && !(leaf[0] && leaf[1]);
        };
        tree_build<3>(out, out.endNodes(), calc, split, max_iter, mra.maxScale());
        sync_new(ctx, b, acc);
        ck(mwgpu_transform(ctx, b.dout, MWGPU_BOTTOMUP, 1), "BottomUp transform");
        std::vector<double> nn(out.nodes.size() * 8);
        ck(mwgpu_download_tree(ctx, b.dout, out.coefs.data(), nn.data()), "download result tree");
        for (size_t i = 0; i < out.nodes.size(); i++) {
            double s2 = 0.0;
            for (int q = 0; q < 8; q++) {
                out.nodes[i].norms[q] = nn[i * 8 + q];
                s2 += nn[i * 8 + q] * nn[i * 8 + q];
            }
            out.nodes[i].squareNorm = s2;
            out.nodes[i].flags |= F_HASCOEFS;
        }
        out.calcSquareNorm();
    } catch (...) {
        release();
        throw;
    }
    release();
    acc.out_nodes = (int)out.nodes.size();
    acc.wall_ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
    if (stats) *stats = acc;
    return 0;
}

}  // namespace

extern "C" {

const char *mwh_last_error(void) { return g_err.c_str(); }

int mwh_set_table_path(const char *path) {
    if (!path) return fail(1, "null path");
    set_table_path(path);
    return 0;
}

int mwh_mra_create(int type, int order, int root_scale, const int *corner, const int *nbox, double sf, int max_depth, mwh_mra **out) {
    return guard([&] {
        if (!out || !corner || !nbox) return fail(1, "null argument");
        BoundingBox<3> b(root_scale, {corner[0], corner[1], corner[2]}, {nbox[0], nbox[1], nbox[2]}, {sf, sf, sf});
        *out = new mwh_mra{MRA<3>(b, type, order, max_depth)};
        return 0;
    });
}

int mwh_mra_from_bounds(int type, int order, int lb, int ub, int max_depth, mwh_mra **out) {
    return guard([&] {
        if (!out) return fail(1, "null argument");
        *out = new mwh_mra{MRA<3>(BoundingBox<3>::fromBounds(lb, ub), type, order, max_depth)};
        return 0;
    });
}

void mwh_mra_free(mwh_mra *m) { delete m; }

int mwh_mra_desc(const mwh_mra *m, mwgpu_mra_desc *d, double *filters) {
    if (!m || !d || !filters) return fail(1, "null argument");
    fill_desc(m->m, d, filters);
    return 0;
}

int mwh_mra_maps(const mwh_mra *m, double *cv_map, double *vc_map, double *roots, double *weights) {
    if (!m) return fail(1, "null MRA");
    const ScalingBasis &b = *m->m.basis;
    const size_t K = b.K;
    if (cv_map) std::memcpy(cv_map, b.cvMap.data(), sizeof(double) * K * K);
    if (vc_map) std::memcpy(vc_map, b.vcMap.data(), sizeof(double) * K * K);
    if (roots) std::memcpy(roots, b.roots.data(), sizeof(double) * K);
    if (weights) std::memcpy(weights, b.weights.data(), sizeof(double) * K);
    return 0;
}

int mwh_mra_distances(const mwh_mra *m, double eps, double *r_min, double *r_max) {
    if (!m || !(eps > 0.0)) return fail(1, "invalid MRA distance arguments");
    if (r_min) *r_min = m->m.calcMinDistance(eps);
    if (r_max) *r_max = m->m.calcMaxDistance();
    return 0;
}

int mwh_tree_create(const mwh_mra *m, mwh_tree **out) {
    return guard([&] {
        if (!m || !out) return fail(1, "null argument");
        *out = new mwh_tree{std::make_unique<Tree<3>>(m->m)};
        touch(*out);
        return 0;
    });
}

void mwh_tree_free(mwh_tree *t) {
    if (!t) return;
    if (t->dev) {
        std::lock_guard<std::mutex> lk(g_gpu_mu);
        if (g_ctx) mwgpu_free_tree(g_ctx, t->dev);
    }
    delete t;
}

static GaussExp<3> make_gexp(int n, const double *coef, const double *ex, const double *pos) {
    GaussExp<3> g;
    for (int i = 0; i < n; i++) g.funcs.push_back(GaussFunc<3>(ex[i], coef[i], {pos[3 * i], pos[3 * i + 1], pos[3 * i + 2]}));
    return g;
}

int mwh_build_grid_gauss(mwh_tree *t, int n, const double *coef, const double *ex, const double *pos) {
    touch(t);
    return guard([&] {
        if (!t || n < 0 || (n > 0 && (!coef || !ex || !pos))) return fail(1, "invalid Gaussian list");
        build_grid(*t->t, make_gexp(n, coef, ex, pos));
        return 0;
    });
}

int mwh_project_gauss(double prec, mwh_tree *t, int n, const double *coef, const double *ex, const double *pos, int max_iter, int abs_prec) {
    touch(t);
    return guard([&] {
        if (!t || n < 0 || (n > 0 && (!coef || !ex || !pos))) return fail(1, "invalid Gaussian list");
        auto g = make_gexp(n, coef, ex, pos);
        project<3>(prec, *t->t, [&g](const double *r) { return g.evalf(r); }, max_iter, abs_prec != 0);
        return 0;
    });
}

int mwh_project_func(double prec, mwh_tree *t, mwh_func f, void *user, int max_iter, int abs_prec) {
    touch(t);
    return guard([&] {
        if (!t || !f) return fail(1, "invalid projection arguments");
        project_batched<3>(prec, *t->t, [f, user](long long n, const double *r, double *v) { f(n, r, v, user); }, max_iter, abs_prec != 0);
        return 0;
    });
}

int mwh_project_func_device(double prec, mwh_tree *t, mwh_func f, void *user, int max_iter, int abs_prec, mwh_apply_stats *stats) {
    touch(t);
    return guard([&] {
        if (!t || !f) return fail(1, "null argument");
        BatchFunc bf = [f, user](long long n, const double *r, double *v) { f(n, r, v, user); };
        return project_device_impl(prec, *t->t, 0, nullptr, nullptr, nullptr, max_iter, abs_prec != 0, stats, &bf);
    });
}

int mwh_project_gauss_device(double prec, mwh_tree *t, int n, const double *coef, const double *ex, const double *pos, int max_iter, int abs_prec,
                             mwh_apply_stats *stats) {
    touch(t);
    return guard([&] {
        if (!t || n < 0 || (n > 0 && (!coef || !ex || !pos))) return fail(1, "invalid Gaussian list");
        return project_device_impl(prec, *t->t, n, coef, ex, pos, max_iter, abs_prec != 0, stats);
    });
}

int mwh_add(double prec, mwh_tree *out, int n, const double *c, mwh_tree *const *inps, int max_iter, int abs_prec, mwh_apply_stats *stats) {
    touch(out);
    return guard([&] {
        if (!out || n < 1 || !c || !inps) return fail(1, "invalid sum");
        for (int j = 0; j < n; j++)
            if (!inps[j]) return fail(1, "null input tree");
        return combine_device_impl(MWGPU_COMBINE_ADD, prec, *out->t, n, c, inps, max_iter, abs_prec != 0, stats);
    });
}

int mwh_multiply_max_norms(double prec, mwh_tree *out, int n, const double *c, mwh_tree *const *inps, int max_iter, mwh_apply_stats *stats) {
    touch(out);
    return guard([&] {
        if (!out || n < 1 || !c || !inps) return fail(1, "null argument");
        for (int j = 0; j < n; j++)
            if (!inps[j] || inps[j] == out) return fail(1, "invalid input tree");
        return combine_device_impl(MWGPU_COMBINE_MULTIPLY, prec, *out->t, n, c, inps, max_iter, false, stats, true);
    });
}

int mwh_multiply(double prec, mwh_tree *out, int n, const double *c, mwh_tree *const *inps, int max_iter, int abs_prec, mwh_apply_stats *stats) {
    touch(out);
    return guard([&] {
        if (!out || n < 1 || !c || !inps) return fail(1, "invalid product");
        for (int j = 0; j < n; j++)
            if (!inps[j]) return fail(1, "null input tree");
        return combine_device_impl(MWGPU_COMBINE_MULTIPLY, prec, *out->t, n, c, inps, max_iter, abs_prec != 0, stats);
    });
}

int mwh_copy_grid(mwh_tree *out, const mwh_tree *inp) {
    touch(out);
    return guard([&] {
        if (!out || !inp) return fail(1, "null argument");
        copy_grid(*out->t, *inp->t);
        return 0;
    });
}

int mwh_tree_info(const mwh_tree *t, int *n, double *sq) {
    if (!t) return fail(1, "null tree");
    int c = 0;
    for (size_t i = 0; i < t->t->nodes.size(); i++)
        if (!t->t->isGen((int)i)) c++;
    if (n) *n = c;
    if (sq) *sq = t->t->squareNorm;
    return 0;
}

int mwh_tree_rescale(mwh_tree *t, double c) {
    touch(t);
    return guard([&] {
        if (!t) return fail(1, "null tree");
        auto &tr = *t->t;
        const size_t nc = (size_t)tr.nCoefs;
        for (size_t i = 0; i < tr.nodes.size(); i++) {
            if (tr.isGen((int)i) || !(tr.nodes[i].flags & F_HASCOEFS)) continue;
            double *x = tr.c((int)i);
            for (size_t j = 0; j < nc; j++) x[j] *= c;
            tr.calcNorms((int)i);
        }
        tr.calcSquareNorm();
        return 0;
    });
}

int mwh_tree_export(const mwh_tree *t, int *idx, int *child0, double *coefs, double *norms) {
    return guard([&] {
        if (!t) return fail(1, "null tree");
        std::vector<int> order, ix, c0;
        export_tree(*t->t, order, ix, c0);
        if (idx) std::memcpy(idx, ix.data(), sizeof(int) * ix.size());
        if (child0) std::memcpy(child0, c0.data(), sizeof(int) * c0.size());
        const size_t nc = t->t->nCoefs;
        for (size_t j = 0; j < order.size(); j++) {
            if (coefs) std::memcpy(coefs + j * nc, t->t->c(order[j]), sizeof(double) * nc);
            if (norms) std::memcpy(norms + j * 8, t->t->nodes[order[j]].norms, sizeof(double) * 8);
        }
        return 0;
    });
}

int mwh_tree_import(mwh_tree *t, int n, const int *idx, const int *child0, const double *coefs, double square_norm) {
    touch(t);
    return guard([&] {
        if (!t || n <= 0 || !idx || !child0) return fail(1, "invalid flat tree");
        auto nt = std::make_unique<Tree<3>>(*t->t->mra);
        // the flat tree lists the roots first, in the same order as the MRA
        std::vector<int> map(n, -1);
        for (size_t r = 0; r < nt->roots.size(); r++) {
            if ((int)r >= n) return fail(1, "flat tree misses roots");
            int id = nt->find(idx[4 * r], &idx[4 * r + 1]);
            if (id < 0) return fail(1, "flat tree roots do not match the MRA");
            map[r] = id;
        }
        for (int j = 0; j < n; j++) {
            if (map[j] < 0) return fail(1, "flat tree is not in parent-before-child order");
            if (child0[j] >= 0) {
                nt->createChildren(map[j], false);
                int c0 = nt->nodes[map[j]].child0;
                for (int c = 0; c < 8; c++) {
                    if (child0[j] + c >= n) return fail(1, "child index out of range");
                    map[child0[j] + c] = c0 + c;
                }
            }
        }
        for (int j = 0; j < n; j++) {
            if (coefs) std::memcpy(nt->c(map[j]), coefs + (size_t)j * nt->nCoefs, sizeof(double) * nt->nCoefs);
            nt->nodes[map[j]].flags |= F_HASCOEFS;
            nt->calcNorms(map[j]);
        }
        nt->squareNorm = square_norm;
        t->t = std::move(nt);
        return 0;
    });
}

// ---- tree files: a flat, versioned layout (FunctionTree::saveTree / loadTree,
// FunctionTree.cpp:378-435, write the node allocator's raw chunks instead) ----
namespace {
const char kTreeMagic[8] = {'M', 'W', 'T', 'R', 'E', 'E', 0, 1};
// header: magic, then int32 dimension, basis type, order, root scale, corner[3],
// nbox[3], max depth, then double sf[3], square norm, then int64 node count;
// body: int32 idx[n][4] (scale, l0, l1, l2), int32 child0[n], double coefs[n][8 (k+1)^3]
// (compressed s+d form), nodes parents before children, roots first; little-endian
struct TreeHeader {
    int32_t dim, type, order, root_scale, corner[3], nbox[3], max_depth;
    double sf[3], square_norm;
    int64_t n;
};
std::string tree_path(const char *file) { return std::string(file) + ".mwtree"; }
}  // namespace

int mwh_tree_save(const mwh_tree *t, const char *file) {
    return guard([&] {
        if (!t || !file) return fail(1, "null argument");
        const Tree<3> &tr = *t->t;
        std::vector<int> order, ix, c0;
        export_tree(tr, order, ix, c0);
        const MRA<3> &m = *tr.mra;
        TreeHeader h{};
        h.dim = 3;
        h.type = m.basis->type;
        h.order = m.order();
        h.root_scale = m.rootScale();
        for (int d = 0; d < 3; d++) {
            h.corner[d] = m.world.corner[d];
            h.nbox[d] = m.world.nbox[d];
            h.sf[d] = m.world.sf[d];
        }
        h.max_depth = m.maxDepth;
        h.square_norm = tr.squareNorm;
        h.n = (int64_t)order.size();
        const std::string path = tree_path(file);
        FILE *fh = std::fopen(path.c_str(), "wb");
        if (!fh) return fail(1, "unable to open " + path + " for writing");
        bool ok = std::fwrite(kTreeMagic, 1, 8, fh) == 8 && std::fwrite(&h, sizeof(h), 1, fh) == 1 &&
                  std::fwrite(ix.data(), sizeof(int), ix.size(), fh) == ix.size() && std::fwrite(c0.data(), sizeof(int), c0.size(), fh) == c0.size();
        for (size_t j = 0; ok && j < order.size(); j++) ok = std::fwrite(tr.c(order[j]), sizeof(double), tr.nCoefs, fh) == tr.nCoefs;
        ok = (std::fclose(fh) == 0) && ok;
        if (!ok) return fail(1, "write error on " + path);
        return 0;
    });
}

int mwh_tree_load(mwh_tree *t, const char *file) {
    touch(t);
    return guard([&] {
        if (!t || !file) return fail(1, "null argument");
        const std::string path = tree_path(file);
        FILE *fh = std::fopen(path.c_str(), "rb");
        if (!fh) return fail(1, "unable to open " + path);
        char magic[8];
        TreeHeader h{};
        bool ok = std::fread(magic, 1, 8, fh) == 8 && std::memcmp(magic, kTreeMagic, 8) == 0 && std::fread(&h, sizeof(h), 1, fh) == 1;
        if (!ok) {
            std::fclose(fh);
            return fail(1, path + " is not a tree file of this format");
        }
        // the tree must have the MRA the file was written with (loadTree's requirement)
        const MRA<3> &m = *t->t->mra;
        bool same = h.dim == 3 && h.type == m.basis->type && h.order == m.order() && h.root_scale == m.rootScale() && h.max_depth == m.maxDepth;
        for (int d = 0; d < 3; d++) same = same && h.corner[d] == m.world.corner[d] && h.nbox[d] == m.world.nbox[d] && h.sf[d] == m.world.sf[d];
        if (!same) {
            std::fclose(fh);
            return fail(1, "the MRA of " + path + " differs from the tree's");
        }
        if (h.n <= 0 || h.n > (int64_t)1 << 31) {
            std::fclose(fh);
            return fail(1, "invalid node count in " + path);
        }
        const size_t n = (size_t)h.n, nc = t->t->nCoefs;
        std::vector<int> ix(4 * n), c0(n);
        std::vector<double> coefs(n * nc);
        ok = std::fread(ix.data(), sizeof(int), ix.size(), fh) == ix.size() && std::fread(c0.data(), sizeof(int), n, fh) == n &&
             std::fread(coefs.data(), sizeof(double), coefs.size(), fh) == coefs.size();
        std::fclose(fh);
        if (!ok) return fail(1, path + " is truncated");
        return mwh_tree_import(t, (int)n, ix.data(), c0.data(), coefs.data(), h.square_norm);
    });
}

double mwh_dot(const mwh_tree *a, const mwh_tree *b) { return (a && b) ? dot(*a->t, *b->t) : 0.0; }
double mwh_evalf(const mwh_tree *t, double x, double y, double z) {
    double r[3] = {x, y, z};
    return t ? evalf(*t->t, r) : 0.0;
}
double mwh_integrate(const mwh_tree *t) { return t ? integrate(*t->t) : 0.0; }

static void finish_oper(mwh_oper *o) {
    auto &op = *o->op;
    o->depth.clear();
    o->max_transl.clear();
    o->blocks.clear();
    o->norms.clear();
    for (auto &t : op.terms) {
        o->depth.push_back(t.depth);
        o->max_transl.insert(o->max_transl.end(), t.maxTransl.begin(), t.maxTransl.end());
        o->blocks.insert(o->blocks.end(), t.blocks.begin(), t.blocks.end());
        o->norms.insert(o->norms.end(), t.norms.begin(), t.norms.end());
    }
}

int mwh_poisson(const mwh_mra *m, double prec, mwh_oper **out) {
    return guard([&] {
        if (!m || !out || !(prec > 0.0)) return fail(1, "invalid Poisson operator arguments");
        auto *o = new mwh_oper{make_poisson(m->m, prec), {}, {}, {}, {}};
        finish_oper(o);
        *out = o;
        return 0;
    });
}

int mwh_helmholtz(const mwh_mra *m, double mu, double prec, mwh_oper **out) {
    return guard([&] {
        if (!m || !out || !(prec > 0.0) || !(mu > 0.0)) return fail(1, "invalid Helmholtz operator arguments");
        auto *o = new mwh_oper{make_helmholtz(m->m, mu, prec), {}, {}, {}, {}};
        finish_oper(o);
        *out = o;
        return 0;
    });
}

int mwh_convolution(const mwh_mra *m, int n, const double *exps, const double *coefs, double prec, mwh_oper **out) {
    return guard([&] {
        if (!m || !out || n < 1 || !exps || !coefs || !(prec > 0.0)) return fail(1, "invalid convolution operator arguments");
        std::vector<GaussFunc<1>> kernel;
        for (int i = 0; i < n; i++) {
            if (!(exps[i] > 0.0)) return fail(1, "kernel exponents must be positive");
            kernel.emplace_back(exps[i], coefs[i]);
        }
        auto *o = new mwh_oper{make_convolution(m->m, kernel, prec), {}, {}, {}, {}};
        finish_oper(o);
        *out = o;
        return 0;
    });
}

int mwh_abgv(const mwh_mra *m, double a, double b, mwh_oper **out) {
    return guard([&] {
        if (!m || !out) return fail(1, "invalid ABGV operator arguments");
        auto *o = new mwh_oper{make_abgv(m->m, a, b), {}, {}, {}, {}};
        finish_oper(o);
        *out = o;
        return 0;
    });
}

int mwh_deriv_tables(const mwh_mra *m, int order, const double *s_p1, const double *s_0, const double *s_m1, mwh_oper **out) {
    return guard([&] {
        if (!m || !out || !s_p1 || !s_0 || !s_m1 || order < 1) return fail(1, "invalid derivative table arguments");
        const int K = m->m.kp1();
        Mat a(K, K), b(K, K), c(K, K);
        for (int i = 0; i < K; i++)
            for (int j = 0; j < K; j++) {
                a(i, j) = s_p1[i * K + j];
                b(i, j) = s_0[i * K + j];
                c(i, j) = s_m1[i * K + j];
            }
        auto *o = new mwh_oper{make_table_derivative(m->m, order, a, b, c), {}, {}, {}, {}};
        finish_oper(o);
        *out = o;
        return 0;
    });
}

// PHCalculator::readSMatrix / BSCalculator::readSMatrix (PHCalculator.cpp:44-74,
// BSCalculator.cpp:44-74): the file holds, for (k+1) = 2, 3, ..., a line with
// k+1 and then 3(k+1) rows of k+1 numbers: S_+1, S_0, S_-1
static int read_deriv_tables(const std::string &file, int K, int kp1_end, Mat &s_p1, Mat &s_0, Mat &s_m1) {
    std::ifstream ifs(file.c_str());
    if (!ifs) return fail(1, "Failed to open file: " + file);
    for (int kp1 = 2; kp1 < kp1_end; kp1++) {
        std::string line;
        std::getline(ifs, line);
        std::istringstream head(line);
        int order = -1;
        head >> order;
        if (order != kp1) return fail(1, "Orders do not match in " + file);
        Mat data(3 * kp1, kp1);
        for (int i = 0; i < 3 * kp1; i++) {
            std::getline(ifs, line);
            std::istringstream row(line);
            for (int j = 0; j < kp1; j++) row >> data(i, j);
            if (!row) return fail(1, "Malformed table in " + file);
        }
        if (kp1 == K) {
            s_p1 = Mat(K, K);
            s_0 = Mat(K, K);
            s_m1 = Mat(K, K);
            for (int i = 0; i < K; i++)
                for (int j = 0; j < K; j++) {
                    s_p1(i, j) = data(i, j);
                    s_0(i, j) = data(K + i, j);
                    s_m1(i, j) = data(2 * K + i, j);
                }
            return 0;
        }
    }
    return fail(1, "Scaling order not supported");
}

static int table_operator(const mwh_mra *m, int order, const char *filter_dir, bool ph, mwh_oper **out) {
    return guard([&] {
        if (!m || !out) return fail(1, "null argument");
        const int max_order = ph ? 2 : 3;
        if (order < 1 || order > max_order) return fail(1, ph ? "PH derivative order must be 1 or 2" : "B-spline derivative order must be 1, 2 or 3");
        std::string dir = filter_dir ? filter_dir : "";
        if (dir.empty()) {
            const char *env = std::getenv("MWFILTERS_DIR");
            if (env) dir = env;
        }
        if (dir.empty()) return fail(1, "no filter directory (argument or MWFILTERS_DIR)");
        const char t = m->m.basis->type == Legendre ? 'L' : 'I';
        const std::string file = dir + "/" + t + (ph ? "_ph_deriv_" : "_b-spline-deriv") + std::to_string(order) + ".txt";
        Mat a, b, c;
        if (int rc = read_deriv_tables(file, m->m.kp1(), ph ? 30 : 21, a, b, c)) return rc;
        auto *o = new mwh_oper{make_table_derivative(m->m, order, a, b, c), {}, {}, {}, {}};
        finish_oper(o);
        *out = o;
        return 0;
    });
}

int mwh_ph(const mwh_mra *m, int order, const char *filter_dir, mwh_oper **out) { return table_operator(m, order, filter_dir, true, out); }
int mwh_bs(const mwh_mra *m, int order, const char *filter_dir, mwh_oper **out) { return table_operator(m, order, filter_dir, false, out); }

int mwh_apply_derivative(mwh_tree *out, mwh_oper *oper, mwh_tree *inp, int dir, mwh_apply_stats *stats) {
    touch(out);
    return guard([&] {
        if (!out || !oper || !inp) return fail(1, "null argument");
        return apply_derivative_impl(out, oper, inp, dir, stats);
    });
}

void mwh_oper_free(mwh_oper *o) {
    if (!o) return;
    std::lock_guard<std::mutex> lk(g_gpu_mu);
    for (auto it = g_oper_cache.begin(); it != g_oper_cache.end();) {
        if (it->first.op == o) {
            if (g_ctx) {
                drop_plans(g_ctx, it->second);
                mwgpu_free_operator(g_ctx, it->second);
            }
            it = g_oper_cache.erase(it);
        } else {
            ++it;
        }
    }
    delete o;
}

int mwh_oper_info(const mwh_oper *o, int *n_terms, int *n_nodes, int *n_rows) {
    if (!o) return fail(1, "null operator");
    if (n_terms) *n_terms = (int)o->depth.size();
    if (n_nodes) *n_nodes = (int)o->norms.size() / 4;
    if (n_rows) *n_rows = (int)o->max_transl.size();
    return 0;
}

int mwh_oper_export(const mwh_oper *o, int *depth, int *max_transl, double *blocks, double *norms, double *kexp, double *kcoef) {
    if (!o) return fail(1, "null operator");
    if (depth) std::memcpy(depth, o->depth.data(), sizeof(int) * o->depth.size());
    if (max_transl) std::memcpy(max_transl, o->max_transl.data(), sizeof(int) * o->max_transl.size());
    if (blocks) std::memcpy(blocks, o->blocks.data(), sizeof(double) * o->blocks.size());
    if (norms) std::memcpy(norms, o->norms.data(), sizeof(double) * o->norms.size());
    for (size_t i = 0; i < o->op->kernel.size(); i++) {
        if (kexp) kexp[i] = o->op->kernel[i].alpha[0];
        if (kcoef) kcoef[i] = o->op->kernel[i].coef;
    }
    return 0;
}

int mwh_oper_desc(const mwh_oper *o, mwgpu_oper_desc *d) {
    if (!o || !d) return fail(1, "null argument");
    d->n_terms = (int)o->depth.size();
    d->order = o->op->mra.order();
    d->depth = o->depth.data();
    d->max_transl = o->max_transl.data();
    d->blocks = o->blocks.data();
    d->norms = o->norms.data();
    d->build_prec = o->op->buildPrec;
    return 0;
}

int mwh_poisson_kernel(double eps, double r_min, double r_max, int cap, double *exps, double *coefs) {
    return guard([&] {
        auto k = poisson_kernel(eps, r_min, r_max);
        for (int i = 0; i < (int)k.size() && i < cap; i++) {
            if (exps) exps[i] = k[i].alpha[0];
            if (coefs) coefs[i] = k[i].coef;
        }
        return (int)k.size();
    });
}

int mwh_helmholtz_kernel(double mu, double eps, double r_min, double r_max, int cap, double *exps, double *coefs) {
    return guard([&] {
        auto k = helmholtz_kernel(mu, eps, r_min, r_max);
        for (int i = 0; i < (int)k.size() && i < cap; i++) {
            if (exps) exps[i] = k[i].alpha[0];
            if (coefs) coefs[i] = k[i].coef;
        }
        return (int)k.size();
    });
}

int mwh_apply(double prec, mwh_tree *outp, mwh_oper *operp, mwh_tree *inpp, int max_iter, int abs_prec, int precision, mwh_apply_stats *stats) {
    return guard([&] {
        if (!outp || !operp || !inpp) return fail(1, "null argument");
        mwh_tree *outs[1] = {outp}, *inps[1] = {inpp};
        return apply_impl(prec, 1, outs, operp, inps, max_iter, abs_prec, precision, stats);
    });
}

int mwh_apply_prec(double prec, mwh_tree *outp, mwh_oper *operp, mwh_tree *inpp, int n_prec, mwh_tree *const *prec_trees, int max_iter,
                   int abs_prec, int precision, mwh_apply_stats *stats) {
    return guard([&] {
        if (!outp || !operp || !inpp || n_prec < 0 || (n_prec > 0 && !prec_trees)) return fail(1, "null argument");
        PrecScale ps;
        for (int i = 0; i < n_prec; i++) {
            if (!prec_trees[i]) return fail(1, "null argument");
            if (prec_trees[i] == outp) return fail(1, "the output tree cannot be a precision tree");
            if (!(*prec_trees[i]->t->mra == *outp->t->mra)) return fail(1, "Incompatible MRA");
            ps.trees.push_back(prec_trees[i]->t.get());
            ps.msq.push_back(prec_trees[i]->t->maxSquareNorms());  // makeMaxSquareNorms (apply.cpp:221)
        }
        mwh_tree *outs[1] = {outp}, *inps[1] = {inpp};
        return apply_impl(prec, 1, outs, operp, inps, max_iter, abs_prec, precision, stats, &ps);
    });
}

int mwh_prec_factors(int n_prec, mwh_tree *const *prec_trees, int n, const int *idx, double *fac) {
    return guard([&] {
        if (n_prec < 0 || (n_prec > 0 && !prec_trees) || n < 0 || (n > 0 && (!idx || !fac))) return fail(1, "null argument");
        PrecScale ps;
        for (int i = 0; i < n_prec; i++) {
            if (!prec_trees[i]) return fail(1, "null argument");
            if (i > 0 && !(*prec_trees[i]->t->mra == *prec_trees[0]->t->mra)) return fail(1, "Incompatible MRA");
            ps.trees.push_back(prec_trees[i]->t.get());
            ps.msq.push_back(prec_trees[i]->t->maxSquareNorms());
        }
        for (int j = 0; j < n; j++) fac[j] = ps(idx[4 * j], idx + 4 * j + 1);
        return 0;
    });
}

int mwh_apply_batch(double prec, int n, mwh_tree **outs, mwh_oper *operp, mwh_tree **inps, int max_iter, int abs_prec, int precision,
                    mwh_apply_stats *stats) {
    return guard([&] {
        if (n < 1 || !outs || !inps || !operp) return fail(1, "null argument");
        for (int t = 0; t < n; t++) {
            if (!outs[t] || !inps[t]) return fail(1, "null argument");
            for (int u = 0; u < t; u++)
                if (outs[u] == outs[t] || inps[u] == inps[t] || outs[u] == inps[t]) return fail(1, "trees of a batch must be distinct");
        }
        return apply_impl(prec, n, outs, operp, inps, max_iter, abs_prec, precision, stats);
    });
}


struct mwh_mlp {
    std::vector<float> params;
    mwgpu_mlp *dev = nullptr;
};

int mwh_mlp_create(const float *params, mwh_mlp **out) {
    return guard([&] {
        if (!params || !out) return fail(1, "null argument");
        *out = new mwh_mlp{std::vector<float>(params, params + MWGPU_MLP_PARAMS), nullptr};
        return 0;
    });
}

void mwh_mlp_free(mwh_mlp *m) {
    if (!m) return;
    if (m->dev && g_ctx) {
        std::lock_guard<std::mutex> lk(g_gpu_mu);
        mwgpu_mlp_destroy(g_ctx, m->dev);
    }
    delete m;
}

int mwh_grid_features(double prec, mwh_tree *gridp, mwh_oper *operp, mwh_tree *inpp, float *x, float *y) {
    return guard([&] {
        if (!gridp || !operp || !inpp || !x) return fail(1, "null argument");
        Tree<3> &grid = *gridp->t;
        Tree<3> &inp = *inpp->t;
        std::lock_guard<std::mutex> lk(g_gpu_mu);
        mwgpu_ctx *ctx = gpu_ctx(MWGPU_PREC_FP64);
        const MRA<3> &mra = *inp.mra;
        std::vector<double> filters(8 * (size_t)mra.kp1() * mra.kp1());
        mwgpu_mra_desc md{};
        fill_desc(mra, &md, filters.data());
        mwgpu_oper *dop = device_operator(ctx, md, operp, prec);
        mwh_apply_stats acc{};
        mwgpu_tree *dinp = upload_input(ctx, md, inp, acc);
        // rows in the order of the tree export (breadth first)
        std::vector<int> order, gidx, gc0;
        export_tree(grid, order, gidx, gc0);
        const int n = (int)order.size();
        std::vector<int> idx(4 * (size_t)n);
        for (int j = 0; j < n; j++) {
            const auto &nd = grid.nodes[order[j]];
            idx[4 * j] = nd.n;
            for (int d = 0; d < 3; d++) idx[4 * j + 1 + d] = nd.l[d];
            if (y) y[j] = gc0[j] >= 0 ? 1.f : 0.f;
        }
        int st = mwgpu_mlp_features(ctx, dop, dinp, std::sqrt(std::max(inp.squareNorm, 0.0)), idx.data(), n, x);
        mwgpu_free_tree(ctx, dinp);
        ck(st, "grid features");
        return 0;
    });
}

int mwh_apply_learned(double prec, mwh_tree *outp, mwh_oper *operp, mwh_tree *inpp, const mwh_mlp *mlpc, double threshold, int full_levels,
                      int abs_prec, int precision, mwh_learned_stats *stats) {
    touch(outp);
    return guard([&] {
        if (!outp || !operp || !inpp || !mlpc) return fail(1, "null argument");
        mwh_mlp *mlp = const_cast<mwh_mlp *>(mlpc);
        Tree<3> &out = *outp->t;
        Tree<3> &inp = *inpp->t;
        mwh_learned_stats ls{};
        ls.first_miss = -1;
        // only a fresh output tree (the roots) can take a proposal
        bool fresh = true;
        for (auto &nd : out.nodes) fresh = fresh && nd.child0 < 0 && nd.n == out.mra->rootScale();
        if (!fresh) {
            mwh_tree *o1[1] = {outp}, *i1[1] = {inpp};
            int rc = apply_impl(prec, 1, o1, operp, i1, -1, abs_prec, precision, &ls.apply);
            ls.fallback = 1;
            if (stats) *stats = ls;
            return rc;
        }
        auto t0 = std::chrono::steady_clock::now();
        std::lock_guard<std::mutex> lk(g_gpu_mu);
        mwgpu_ctx *ctx = gpu_ctx(precision);
        const MRA<3> &mra = *out.mra;
        std::vector<double> filters(8 * (size_t)mra.kp1() * mra.kp1());
        mwgpu_mra_desc md{};
        fill_desc(mra, &md, filters.data());
        mwgpu_oper *dop = device_operator(ctx, md, operp, prec);
        if (!mlp->dev) ck(mwgpu_mlp_create(ctx, mlp->params.data(), &mlp->dev), "network upload");
        HostTrace ht("apply_learned");
        ht.ctx = ctx;
        mwh_apply_stats acc{};
        unsigned long long l0 = 0, l1 = 0;
        mwgpu_launch_count(ctx, &l0);
        mwgpu_tree *dinp = nullptr, *dprop = nullptr, *dold = nullptr;
        // The proposal, level by level.  `prop` holds the judged tree of the
        // levels before `first` (exact) and the proposed levels after it; its
        // node order is TreeBuilder's (levels, each in the order of the parents).
        GridSketch prop(out);
        std::vector<int> level_begin, flags;
        std::vector<double> norm_levels, norms;
        try {
            dinp = resident_input(ctx, md, inpp, acc);
            ck(mwgpu_tree_clear_generated(ctx, dinp), "clear generated nodes");
            ht.mark("upload");
            const double f_norm = std::sqrt(std::max(inp.squareNorm, 0.0));
            const size_t max_nodes = std::max<size_t>(4096, 4 * inp.nodes.size());
            std::vector<int> idx;
            std::vector<float> pr;
            // extends the proposal below the nodes `cur` (one level), predicting level by level
            auto propose = [&](std::vector<int> cur) {
                while (!cur.empty()) {
                    level_begin.push_back(level_begin.back() + (int)cur.size());
                    const int lvl = (int)level_begin.size() - 2;
                    const int n = (int)cur.size();
                    std::vector<int> refine;
                    if (lvl < full_levels) {
                        for (int i : cur)
                            if (prop.nodes[i].n + 2 <= mra.maxScale()) refine.push_back(i);
                    } else {
                        idx.resize(4 * (size_t)n);
                        for (int j = 0; j < n; j++) {
                            const auto &nd = prop.nodes[cur[j]];
                            idx[4 * j] = nd.n;
                            for (int d = 0; d < 3; d++) idx[4 * j + 1 + d] = nd.l[d];
                        }
                        pr.resize(n);
                        const auto tp = std::chrono::steady_clock::now();
                        ck(mwgpu_mlp_predict(ctx, mlp->dev, dop, dinp, f_norm, idx.data(), n, pr.data()), "grid prediction");
                        ls.predict_ms += std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - tp).count();
                        ls.host_round_trips += 1;
                        for (int j = 0; j < n; j++)
                            if (pr[j] > threshold && prop.nodes[cur[j]].n + 2 <= mra.maxScale()) refine.push_back(cur[j]);
                    }
                    ls.proposal_levels++;
                    // a proposal larger than the budget stops here (the judge then
                    // reports the first level it would have needed)
                    if (prop.nodes.size() + Tree<3>::tDim * refine.size() > max_nodes) break;
                    std::vector<int> next;
                    for (int i : refine) {
                        prop.createChildren(i);
                        const int c0 = prop.nodes[i].child0;
                        for (int c = 0; c < Tree<3>::tDim; c++) next.push_back(c0 + c);
                    }
                    cur.swap(next);
                }
            };
            std::vector<int> roots;
            for (size_t i = 0; i < prop.nodes.size(); i++) roots.push_back((int)i);
            level_begin.push_back(0);
            propose(roots);
            ht.mark("propose");
            ls.proposal_nodes = (int)prop.nodes.size();
            double state[3] = {0.0, 0.0, out.squareNorm};
            int first = 0;
            std::vector<int> src_prev;  // node of the previous device proposal for every node of prop (-1: new)
            for (int pass = 0;; pass++) {
                // the proposal as a device tree; the judged levels before `first` are copied over
                std::vector<int> pidx(prop.nodes.size() * 4), pc0(prop.nodes.size(), -1);
                for (size_t i = 0; i < prop.nodes.size(); i++) {
                    pidx[4 * i] = prop.nodes[i].n;
                    for (int d = 0; d < 3; d++) pidx[4 * i + 1 + d] = prop.nodes[i].l[d];
                    pc0[i] = prop.nodes[i].child0;
                }
                mwgpu_tree_desc gd{(int)prop.nodes.size(), pidx.data(), pc0.data(), nullptr, nullptr};
                dold = dprop;
                dprop = nullptr;
                ck(mwgpu_create_tree(ctx, &md, &gd, &dprop), "create proposal tree");
                acc.h2d_bytes += (pidx.size() + pc0.size()) * 4;
                if (dold) {
                    std::vector<int> a, b;
                    for (int i = 0; i < level_begin[first]; i++) {
                        a.push_back(src_prev[i]);
                        b.push_back(i);
                    }
                    ck(mwgpu_tree_copy_nodes(ctx, dold, dprop, (int)a.size(), a.data(), b.data()), "copy judged levels");
                    mwgpu_free_tree(ctx, dold);
                    dold = nullptr;
                }
                ht.mark("tree" + std::to_string(pass));
                const int nlev = (int)level_begin.size() - 1;
                flags.assign(prop.nodes.size(), 0);
                norm_levels.assign(3 * (size_t)nlev, 0.0);
                int miss = -1;
                mwgpu_level_stats st{};
                const auto tj = std::chrono::steady_clock::now();
                ck(mwgpu_apply_judged(ctx, dop, dinp, dprop, nlev, level_begin.data(), prec, abs_prec, first, state, 1, flags.data(), &miss,
                                      norm_levels.data(), &st),
                   "judged apply");
                ls.judged_ms += std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - tj).count();
                ht.mark("judged" + std::to_string(pass));
                ls.host_round_trips += 1;
                acc.node_terms += st.node_terms;
                acc.components += st.components;
                acc.band_nodes += st.band_nodes;
                acc.gen_nodes += st.gen_nodes;
                acc.device_ms += st.device_ms;
                acc.contract_ms += st.contract_ms;
                acc.iterations += 1;
                acc.d2h_bytes += flags.size() * 4;
                if (pass == 0) ls.first_miss = miss;
                if (miss < 0) break;
                // a refinement the proposal missed at level `miss`: the judged tree
                // up to there is kept, all children of the refined nodes of that
                // level are added, the network proposes below them, next pass
                ls.fallback = 1;
                GridSketch next(out);
                std::vector<int> map(prop.nodes.size(), -1), nsrc;
                for (size_t i = 0; i < next.nodes.size(); i++) {
                    map[i] = (int)i;
                    nsrc.push_back((int)i);
                }
                // nlb[j + 1] = end of level j of `next` (iteration j creates level j + 1)
                std::vector<int> nlb{0, (int)next.nodes.size()}, frontier;
                for (int j = 0; j <= miss; j++) {
                    for (int i = level_begin[j]; i < level_begin[j + 1]; i++) {
                        if ((flags[i] & 3) != 3) continue;
                        const int oi = map[i];
                        next.createChildren(oi);
                        const int c0 = next.nodes[oi].child0, p0 = prop.nodes[i].child0;
                        for (int c = 0; c < Tree<3>::tDim; c++) {
                            nsrc.push_back(j < miss && p0 >= 0 ? p0 + c : -1);
                            if (j < miss && p0 >= 0) map[p0 + c] = c0 + c;
                            if (j == miss) frontier.push_back(c0 + c);
                        }
                    }
                    nlb.push_back((int)nsrc.size());
                }
                // levels 0 .. miss stay; the frontier (level miss + 1) is proposed next
                level_begin.assign(nlb.begin(), nlb.begin() + (miss + 2));
                prop = std::move(next);
                src_prev = nsrc;
                state[0] = norm_levels[3 * miss];
                state[1] = norm_levels[3 * miss + 1];
                state[2] = norm_levels[3 * miss + 2];
                first = miss + 1;
                propose(frontier);
                ht.mark("propose" + std::to_string(pass + 1));
                ls.proposal_nodes += (int)prop.nodes.size() - level_begin[first];
            }
        } catch (...) {
            if (dprop) mwgpu_free_tree(ctx, dprop);
            if (dold) mwgpu_free_tree(ctx, dold);
            throw;
        }
        // the judged tree, created in TreeBuilder's order (the host ids of the plain apply)
        std::vector<int> map(prop.nodes.size(), -1);
        for (size_t i = 0; i < out.nodes.size(); i++) map[i] = (int)i;
        const int nlev = (int)level_begin.size() - 1;
        {
            size_t n_keep = 0;
            for (size_t i = 0; i < prop.nodes.size(); i++) n_keep += flags[i] & 1;
            out.nodes.reserve(n_keep);
            out.coefs.reserve(n_keep * (size_t)out.nCoefs);
        }
        int kept = 0;
        for (int j = 0; j < nlev; j++)
            for (int i = level_begin[j]; i < level_begin[j + 1]; i++) {
                if (!(flags[i] & 1)) continue;
                kept++;
                if ((flags[i] & 3) != 3) continue;
                const int oi = map[i];
                out.createChildren(oi, false);
                const int c0 = out.nodes[oi].child0, p0 = prop.nodes[i].child0;
                for (int c = 0; c < Tree<3>::tDim; c++) map[p0 + c] = c0 + c;
            }
        ls.kept_nodes = kept;
        ht.mark("out_tree");
        // the kept nodes, gathered on the device in the output tree's order,
        // straight into its coefficient storage
        std::vector<int> src(out.nodes.size(), -1);
        for (size_t i = 0; i < prop.nodes.size(); i++)
            if (map[i] >= 0 && (flags[i] & 1)) src[map[i]] = (int)i;
        for (size_t oi = 0; oi < src.size(); oi++)
            if (src[oi] < 0) throw Error(6, "judged tree: output node without a computed source");
        norms.resize(src.size() * 8);
        try {
            ck(mwgpu_download_nodes(ctx, dprop, (int)src.size(), src.data(), out.coefs.data(), norms.data()), "download output tree");
        } catch (...) {
            mwgpu_free_tree(ctx, dprop);
            throw;
        }
        acc.d2h_bytes += (src.size() * (size_t)out.nCoefs + norms.size()) * 8;
        ls.host_round_trips += 1;
        mwgpu_free_tree(ctx, dprop);  // the input tree keeps its device copy
        mwgpu_launch_count(ctx, &l1);
        acc.launches = l1 - l0;
        ht.mark("download");
        for (size_t oi = 0; oi < src.size(); oi++) {
            double s2 = 0.0;
            for (int c = 0; c < 8; c++) {
                out.nodes[oi].norms[c] = norms[oi * 8 + c];
                s2 += norms[oi * 8 + c] * norms[oi * 8 + c];
            }
            out.nodes[oi].squareNorm = s2;
            out.nodes[oi].flags |= F_HASCOEFS;
        }
        out.calcSquareNorm();
        acc.out_nodes = (int)out.nodes.size();
        acc.wall_ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
        ls.apply = acc;
        if (stats) *stats = ls;
        return 0;
    });
}

}  // extern "C"
