// C interface of the host mirror (include/mwhost.h) and mrcpp::apply driven
// through the device C-ABI (include/mwgpu.h).
//
// mwh_apply follows src/treebuilders/apply.cpp:68-93: calcBandWidths, the
// TreeBuilder loop of TreeBuilder.cpp:38-87 with WaveletAdaptor splitting
// (WaveletAdaptor.h:51-54, TreeAdaptor.h:41-52), then TopDown(add) and
// BottomUp transforms and the final square norm.  The per-node work of each
// iteration (ConvolutionCalculator::calcNodeVector) runs on the GPU.
#include <algorithm>
#include <chrono>
#include <map>
#include <mutex>

#include "../../../include/mwhost.h"
#include "mw_host.h"

using namespace mwh;

struct mwh_mra {
    MRA<3> m;
};
struct mwh_tree {
    std::unique_ptr<Tree<3>> t;
};
struct mwh_oper {
    std::unique_ptr<ConvolutionOperator> op;
    std::vector<int> depth, max_transl;
    std::vector<double> blocks, norms;
};

namespace {
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

int mwh_tree_create(const mwh_mra *m, mwh_tree **out) {
    return guard([&] {
        if (!m || !out) return fail(1, "null argument");
        *out = new mwh_tree{std::make_unique<Tree<3>>(m->m)};
        return 0;
    });
}

void mwh_tree_free(mwh_tree *t) { delete t; }

static GaussExp<3> make_gexp(int n, const double *coef, const double *ex, const double *pos) {
    GaussExp<3> g;
    for (int i = 0; i < n; i++) g.funcs.push_back(GaussFunc<3>(ex[i], coef[i], {pos[3 * i], pos[3 * i + 1], pos[3 * i + 2]}));
    return g;
}

int mwh_build_grid_gauss(mwh_tree *t, int n, const double *coef, const double *ex, const double *pos) {
    return guard([&] {
        if (!t || n < 0 || (n > 0 && (!coef || !ex || !pos))) return fail(1, "invalid Gaussian list");
        build_grid(*t->t, make_gexp(n, coef, ex, pos));
        return 0;
    });
}

int mwh_project_gauss(double prec, mwh_tree *t, int n, const double *coef, const double *ex, const double *pos, int max_iter, int abs_prec) {
    return guard([&] {
        if (!t || n < 0 || (n > 0 && (!coef || !ex || !pos))) return fail(1, "invalid Gaussian list");
        auto g = make_gexp(n, coef, ex, pos);
        project<3>(prec, *t->t, [&g](const double *r) { return g.evalf(r); }, max_iter, abs_prec != 0);
        return 0;
    });
}

int mwh_copy_grid(mwh_tree *out, const mwh_tree *inp) {
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

void mwh_oper_free(mwh_oper *o) {
    if (!o) return;
    std::lock_guard<std::mutex> lk(g_gpu_mu);
    for (auto it = g_oper_cache.begin(); it != g_oper_cache.end();) {
        if (it->first.op == o) {
            if (g_ctx) mwgpu_free_operator(g_ctx, it->second);
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
        Tree<3> &out = *outp->t;
        Tree<3> &inp = *inpp->t;
        ConvolutionOperator &op = *operp->op;
        if (!(*out.mra == *inp.mra)) return fail(1, "Incompatible MRA");
        if (!(*out.mra == op.mra)) return fail(1, "Operator MRA differs from the function MRA");
        auto t0 = std::chrono::steady_clock::now();
        std::lock_guard<std::mutex> lk(g_gpu_mu);
        mwgpu_ctx *ctx = gpu_ctx(precision);
        const MRA<3> &mra = *out.mra;
        std::vector<double> filters(8 * (size_t)mra.kp1() * mra.kp1());
        mwgpu_mra_desc md{};
        fill_desc(mra, &md, filters.data());

        // operator tables on the device, cached per (operator, apply precision)
        mwgpu_oper *dop = nullptr;
        auto it = g_oper_cache.find({operp, prec});
        if (it != g_oper_cache.end()) {
            dop = it->second;
        } else {
            mwgpu_oper_desc od{};
            mwh_oper_desc(operp, &od);
            ck(mwgpu_upload_operator(ctx, &md, &od, prec, &dop), "upload operator");
            g_oper_cache[{operp, prec}] = dop;
        }

        // input tree
        std::vector<int> order, idx, child0;
        export_tree(inp, order, idx, child0);
        std::vector<double> coefs(order.size() * (size_t)inp.nCoefs), norms(order.size() * 8);
        for (size_t j = 0; j < order.size(); j++) {
            std::memcpy(&coefs[j * inp.nCoefs], inp.c(order[j]), sizeof(double) * inp.nCoefs);
            std::memcpy(&norms[j * 8], inp.nodes[order[j]].norms, sizeof(double) * 8);
        }
        mwgpu_tree_desc fd{(int)order.size(), idx.data(), child0.data(), coefs.data(), norms.data()};
        mwgpu_tree *dinp = nullptr, *dout = nullptr;
        ck(mwgpu_upload_tree(ctx, &md, &fd, &dinp), "upload input tree");

        // output tree: the host ids are the device ids (nodes are only appended)
        out.clearGenerated();
        std::vector<int> oidx(out.nodes.size() * 4), oc0(out.nodes.size(), -1);
        for (size_t i = 0; i < out.nodes.size(); i++) {
            oidx[4 * i] = out.nodes[i].n;
            for (int d = 0; d < 3; d++) oidx[4 * i + 1 + d] = out.nodes[i].l[d];
            oc0[i] = out.nodes[i].child0;
        }
        mwgpu_tree_desc gd{(int)out.nodes.size(), oidx.data(), oc0.data(), nullptr, nullptr};
        int st = mwgpu_create_tree(ctx, &md, &gd, &dout);
        if (st) {
            mwgpu_free_tree(ctx, dinp);
            ck(st, "create output tree");
        }
        mwh_apply_stats acc{};
        unsigned long long l0 = 0, l1 = 0;
        mwgpu_launch_count(ctx, &l0);
        acc.h2d_bytes = (unsigned long long)(coefs.size() + norms.size()) * 8 + (idx.size() + child0.size()) * 4 +
                        (oidx.size() + oc0.size()) * 4;
        try {
            // ConvolutionCalculator::getInitialWorkVector: all nodes of the output tree
            std::vector<int> work;
            for (auto &lvl : out.nodesByDepth(false))
                for (int i : lvl) work.push_back(i);
            std::vector<double> nbuf;
            auto calc = [&](Tree<3> &t, const std::vector<int> &w) {
                nbuf.resize(w.size() * 8);
                mwgpu_level_stats ls{};
                ck(mwgpu_apply_level(ctx, dop, dinp, dout, w.data(), (int)w.size(), prec, t.squareNorm, nbuf.data(), &ls), "apply level");
                acc.h2d_bytes += w.size() * 4;
                acc.d2h_bytes += (unsigned long long)t.nodes.size() * 8 * 8;
                for (size_t j = 0; j < w.size(); j++) {
                    double sq = 0.0;
                    for (int c = 0; c < 8; c++) {
                        t.nodes[w[j]].norms[c] = nbuf[j * 8 + c];
                        sq += nbuf[j * 8 + c] * nbuf[j * 8 + c];
                    }
                    t.nodes[w[j]].squareNorm = sq;
                    t.nodes[w[j]].flags |= F_HASCOEFS;
                }
                acc.node_terms += ls.node_terms;
                acc.components += ls.components;
                acc.band_nodes += ls.band_nodes;
                acc.gen_nodes += ls.gen_nodes;
                acc.device_ms += ls.device_ms;
                acc.contract_ms += ls.contract_ms;
                acc.iterations++;
            };
            size_t synced = out.nodes.size();
            auto split = [&](const Tree<3> &t, int i) { return split_check(t, i, prec, 1.0, abs_prec != 0); };
            // children made by the split step are mirrored to the device before
            // the next iteration computes them (host ids == device ids)
            auto sync_new = [&](const Tree<3> &t) {
                if (t.nodes.size() <= synced) return;
                int n = (int)(t.nodes.size() - synced);
                std::vector<int> nidx(4 * (size_t)n), pids, pc0;
                for (int j = 0; j < n; j++) {
                    const auto &nd = t.nodes[synced + j];
                    nidx[4 * j] = nd.n;
                    for (int d = 0; d < 3; d++) nidx[4 * j + 1 + d] = nd.l[d];
                    if (nd.parent >= 0 && t.nodes[nd.parent].child0 == (int)(synced + j)) {
                        pids.push_back(nd.parent);
                        pc0.push_back(t.nodes[nd.parent].child0);
                    }
                }
                ck(mwgpu_tree_add_nodes(ctx, dout, n, nidx.data(), (int)pids.size(), pids.data(), pc0.data()), "add output nodes");
                acc.h2d_bytes += (nidx.size() + pids.size() + pc0.size()) * 4 + t.nodes.size() * 4;
                synced = t.nodes.size();
            };
            auto calc_sync = [&](Tree<3> &t, const std::vector<int> &w) {
                sync_new(t);
                calc(t, w);
            };
            tree_build<3>(out, work, calc_sync, split, max_iter, mra.maxScale());
            sync_new(out);
            auto t1 = std::chrono::steady_clock::now();
            ck(mwgpu_transform(ctx, dout, MWGPU_TOPDOWN, 0), "TopDown transform");
            ck(mwgpu_transform(ctx, dout, MWGPU_BOTTOMUP, 1), "BottomUp transform");
            std::vector<double> nn(out.nodes.size() * 8);
            ck(mwgpu_download_tree(ctx, dout, out.coefs.data(), nn.data()), "download output tree");
            acc.d2h_bytes += (unsigned long long)(out.coefs.size() + nn.size()) * 8;
            auto t2 = std::chrono::steady_clock::now();
            acc.transform_ms = std::chrono::duration<double, std::milli>(t2 - t1).count();
            for (size_t i = 0; i < out.nodes.size(); i++) {
                double sq = 0.0;
                for (int c = 0; c < 8; c++) {
                    out.nodes[i].norms[c] = nn[i * 8 + c];
                    sq += nn[i * 8 + c] * nn[i * 8 + c];
                }
                out.nodes[i].squareNorm = sq;
                out.nodes[i].flags |= F_HASCOEFS;
            }
            out.calcSquareNorm();
        } catch (...) {
            mwgpu_free_tree(ctx, dout);
            mwgpu_free_tree(ctx, dinp);
            throw;
        }
        mwgpu_launch_count(ctx, &l1);
        acc.launches = l1 - l0;
        mwgpu_free_tree(ctx, dout);
        mwgpu_free_tree(ctx, dinp);
        acc.out_nodes = (int)out.nodes.size();
        acc.wall_ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
        if (stats) *stats = acc;
        return 0;
    });
}

}  // extern "C"
