// Gaussians, grid building, projection and a few tree utilities of the host
// mirror.
//
// Follows src/functions/GaussFunc.cpp:47-110, src/functions/Gaussian.cpp:116-135
// (visibility/zero tests), src/treebuilders/grid.cpp:78-124 (build_grid with
// AnalyticAdaptor.h:38-49), src/treebuilders/project.cpp:41-66 and
// ProjectionCalculator.cpp:34-51, src/trees/MWNode.cpp:448-490 (cvTransform),
// :854-935 (child quadrature points), src/treebuilders/grid.cpp:220 (copy_grid).
#include "mw_host.h"

#include <algorithm>

namespace mwh {

template <int D> double GaussFunc<D>::evalf(const double *r) const {
    double q2 = 0.0, p2 = 1.0;
    for (int d = 0; d < D; d++) {
        double q = r[d] - pos[d];
        q2 += alpha[d] * q * q;
        if (power[d] == 1) p2 *= q;
        else if (power[d] > 1) p2 *= std::pow(q, power[d]);
    }
    return coef * p2 * std::exp(-q2);
}

template <int D> bool GaussFunc<D>::isVisibleAtScale(int scale, int nQuadPts) const {
    for (int d = 0; d < D; d++) {
        double stdDeviation = std::pow(2.0 * alpha[d], -0.5);
        int visibleScale = static_cast<int>(-std::floor(std::log2(nQuadPts * 0.5 * stdDeviation)));
        if (scale < visibleScale) return false;
    }
    return true;
}

template <int D> bool GaussFunc<D>::isZeroOnInterval(const double *a, const double *b) const {
    for (int i = 0; i < D; i++) {
        double stdDeviation = std::pow(2.0 * alpha[i], -0.5);
        double gaussBoxMin = pos[i] - 5.0 * stdDeviation;
        double gaussBoxMax = pos[i] + 5.0 * stdDeviation;
        if (a[i] > gaussBoxMax || b[i] < gaussBoxMin) return true;
    }
    return false;
}

template <int D> double GaussFunc<D>::calcSquareNorm() const {
    double norm = 1.0;
    for (int d = 0; d < D; d++) {
        double a = 2.0 * alpha[d];
        double sq = 1.0;
        int p = power[d];
        if (p > 0) {
            int i = 2 * p - 1;
            while (i > 0) { sq = i * sq / (2.0 * a); i -= 2; }
        }
        sq *= std::sqrt(pi / a);
        norm *= sq;
    }
    return norm * coef * coef;
}

template <int D> static void node_bounds(const Tree<D> &t, int i, double *lb, double *ub) {
    const auto &w = t.mra->world;
    double two_n = std::pow(2.0, -t.nodes[i].n);
    for (int d = 0; d < D; d++) {
        lb[d] = w.sf[d] * two_n * t.nodes[i].l[d];
        ub[d] = w.sf[d] * two_n * (t.nodes[i].l[d] + 1);
    }
}

template <int D> static void build_grid_one(Tree<D> &tree, const GaussFunc<D> &f) {
    int maxScale = tree.mra->maxScale();
    std::vector<int> work = tree.endNodes();
    auto calc = [](Tree<D> &, const std::vector<int> &) {};
    auto split = [&f](const Tree<D> &t, int i) {
        int scale = t.nodes[i].n;
        if (f.isVisibleAtScale(scale, t.K)) return false;
        double lb[3], ub[3];
        node_bounds(t, i, lb, ub);
        if (f.isZeroOnInterval(lb, ub)) return false;
        return true;
    };
    // DefaultCalculator leaves norms undefined, so TreeBuilder sees -1 norms.
    tree_build<D>(tree, work, calc, split, -1, maxScale);
}

template <int D> void build_grid(Tree<D> &tree, const GaussFunc<D> &f) { build_grid_one(tree, f); }
template <int D> void build_grid(Tree<D> &tree, const GaussExp<D> &f) {
    for (auto &g : f.funcs) build_grid_one(tree, g);
}

// ProjectionCalculator::calcNode for node i.
// The tDim * kp1_d points of node i at which ProjectionCalculator::calcNode
// evaluates the function (ProjectionCalculator.cpp:34-51): the quadrature
// points of the children, child by child, x fastest
// (math_utils::tensor_expand_coords_3D); r holds 3 doubles per point.
template <int D> static void node_points(const Tree<D> &t, int i, double *r) {
    const auto &b = *t.mra->basis;
    const auto &w = t.mra->world;
    const int K = t.K, kp1_d = t.kp1_d, tDim = Tree<D>::tDim;
    const auto &nd = t.nodes[i];
    const double sFac = std::pow(2.0, -(nd.n + 1));
    std::vector<double> prim((size_t)D * 2 * K);
    for (int d = 0; d < D; d++)
        for (int q = 0; q < K; q++) {
            prim[(size_t)d * 2 * K + q] = sFac * (b.roots[q] + 2.0 * nd.l[d]);
            prim[(size_t)d * 2 * K + K + q] = sFac * (b.roots[q] + 2.0 * nd.l[d] + 1.0);
        }
    for (int ct = 0; ct < tDim; ct++)
        for (int p = 0; p < kp1_d; p++) {
            int rem = p;
            double *x = r + 3 * ((size_t)ct * kp1_d + p);
            x[0] = x[1] = x[2] = 0.0;
            for (int d = 0; d < D; d++) {
                const int q = rem % K, bit = (ct >> d) & 1;
                rem /= K;
                x[d] = w.sf[d] * prim[(size_t)d * 2 * K + bit * K + q];
            }
        }
}

// Node i from its function values at node_points (in its coefficient storage):
// cvTransform(Backward), the 2^{-D(n+1)/2} scaling, compression and norms
// (ProjectionCalculator.cpp:40-50).
template <int D> static void node_from_values(Tree<D> &t, int i) {
    const auto &b = *t.mra->basis;
    const auto &w = t.mra->world;
    const int K = t.K, kp1_d = t.kp1_d, tDim = Tree<D>::tDim;
    const auto &nd = t.nodes[i];
    double *coefs = t.c(i);
    std::vector<double> tmp(t.nCoefs);
    double *in = coefs, *out = tmp.data();
    int kp1_dm1 = kp1_d / K;
    for (int d = 0; d < D; d++) {
        for (int ct = 0; ct < tDim; ct++) apply_filter(out + (size_t)ct * kp1_d, in + (size_t)ct * kp1_d, b.vcMap, K, kp1_dm1, false);
        std::swap(in, out);
    }
    double sf_prod = 1.0;
    for (int d = 0; d < D; d++) sf_prod *= w.sf[d];
    if (sf_prod <= MachineZero) sf_prod = 1.0;
    double two_fac = std::pow(2.0, D * (nd.n + 1)) / sf_prod;
    two_fac = std::sqrt(1.0 / two_fac);
    if (D % 2 == 1) {
        for (int j = 0; j < t.nCoefs; j++) coefs[j] = two_fac * in[j];
    } else {
        for (int j = 0; j < t.nCoefs; j++) coefs[j] *= two_fac;
    }
    t.mwTransformNode(i, Compression);
    t.nodes[i].flags |= F_HASCOEFS;
    t.calcNorms(i);
}

template <int D> static void project_node(Tree<D> &t, int i, const std::function<double(const double *)> &f) {
    const int n = Tree<D>::tDim * t.kp1_d;
    std::vector<double> r(3 * (size_t)n);
    node_points(t, i, r.data());
    double *coefs = t.c(i);
    for (int p = 0; p < n; p++) coefs[p] = f(r.data() + 3 * (size_t)p);
    node_from_values(t, i);
}

template <int D> void project(double prec, Tree<D> &tree, const std::function<double(const double *)> &f, int maxIter, bool absPrec) {
    int maxScale = tree.mra->maxScale();
    std::vector<int> work = tree.endNodes();
    auto calc = [&f](Tree<D> &t, const std::vector<int> &w) {
        // coefficient storage may grow only in the split step, so nodes can be
        // computed in parallel here
#pragma omp parallel for schedule(dynamic)
        for (size_t j = 0; j < w.size(); j++) project_node(t, w[j], f);
    };
    auto split = [prec, absPrec](const Tree<D> &t, int i) { return split_check(t, i, prec, 1.0, absPrec); };
    tree_build<D>(tree, work, calc, split, maxIter, maxScale);
    tree.mwTransformUp();
    tree.calcSquareNorm();
}

// project() for a function evaluated on many points per call: the points of
// a level's nodes are gathered (at most kProjectBatch per call), the callback
// fills the values, the node computations run in parallel.
template <int D> void project_batched(double prec, Tree<D> &tree, const BatchFunc &f, int maxIter, bool absPrec) {
    int maxScale = tree.mra->maxScale();
    std::vector<int> work = tree.endNodes();
    auto calc = [&f](Tree<D> &t, const std::vector<int> &w) {
        const size_t per = (size_t)Tree<D>::tDim * t.kp1_d;
        const size_t nodes_per_call = std::max<size_t>(1, kProjectBatch / per);
        std::vector<double> r, v;
        for (size_t j0 = 0; j0 < w.size(); j0 += nodes_per_call) {
            const size_t nj = std::min(nodes_per_call, w.size() - j0);
            r.resize(3 * per * nj);
            v.assign(per * nj, 0.0);
#pragma omp parallel for schedule(static)
            for (size_t j = 0; j < nj; j++) node_points(t, w[j0 + j], r.data() + 3 * per * j);
            f((long long)(per * nj), r.data(), v.data());
#pragma omp parallel for schedule(dynamic)
            for (size_t j = 0; j < nj; j++) {
                std::copy(v.begin() + per * j, v.begin() + per * (j + 1), t.c(w[j0 + j]));
                node_from_values(t, w[j0 + j]);
            }
        }
    };
    auto split = [prec, absPrec](const Tree<D> &t, int i) { return split_check(t, i, prec, 1.0, absPrec); };
    tree_build<D>(tree, work, calc, split, maxIter, maxScale);
    tree.mwTransformUp();
    tree.calcSquareNorm();
}

template <int D> void copy_grid(Tree<D> &out, const Tree<D> &inp) {
    if (!(*out.mra == *inp.mra)) throw Error(1, "Incompatible MRA");
    Tree<D> fresh(*inp.mra);
    // breadth-first copy of the non-generated topology
    std::vector<std::pair<int, int>> stack;
    for (size_t r = 0; r < inp.roots.size(); r++) stack.push_back({inp.roots[r], fresh.roots[r]});
    while (!stack.empty()) {
        auto [a, b] = stack.back();
        stack.pop_back();
        int c0 = inp.nodes[a].child0;
        if (c0 >= 0 && !inp.isGen(c0)) {
            fresh.createChildren(b, false);
            int d0 = fresh.nodes[b].child0;
            for (int c = 0; c < Tree<D>::tDim; c++) stack.push_back({c0 + c, d0 + c});
        }
    }
    fresh.squareNorm = -1.0;
    out = std::move(fresh);
}

template <int D> double dot(const Tree<D> &a, const Tree<D> &b) {
    const int kp1_d = a.kp1_d, tDim = Tree<D>::tDim;
    double s = 0.0;
    for (size_t r = 0; r < a.roots.size(); r++) {
        const double *x = a.c(a.roots[r]), *y = b.c(b.roots[r]);
        for (int j = 0; j < kp1_d; j++) s += x[j] * y[j];
    }
    for (size_t i = 0; i < a.nodes.size(); i++) {
        if (a.isGen((int)i)) continue;
        const auto &n = a.nodes[i];
        int j = b.find(n.n, n.l);
        if (j < 0 || b.isGen(j)) continue;
        const double *x = a.c((int)i), *y = b.c(j);
        for (int q = kp1_d; q < tDim * kp1_d; q++) s += x[q] * y[q];
    }
    return s;
}

template <int D> double evalf(const Tree<D> &t, const double *r) {
    const auto &w = t.mra->world;
    const auto &b = *t.mra->basis;
    int l[3] = {0, 0, 0};
    for (int d = 0; d < D; d++) {
        double x = r[d];
        if (x < w.lower(d) || x >= w.upper(d)) return 0.0;
        l[d] = (int)std::floor(x / w.unitLength(d));
    }
    int i = t.find(w.scale, l);
    if (i < 0) return 0.0;
    while (t.nodes[i].child0 >= 0 && !t.isGen(t.nodes[i].child0)) {
        int c = 0;
        int n1 = t.nodes[i].n + 1;
        for (int d = 0; d < D; d++) {
            int ld = (int)std::floor(r[d] / (w.sf[d] * std::pow(2.0, -n1)));
            c |= (ld & 1) << d;
        }
        i = t.nodes[i].child0 + c;
    }
    const auto &nd = t.nodes[i];
    const int K = t.K;
    std::vector<double> phi((size_t)D * K);
    double fac = 1.0;
    for (int d = 0; d < D; d++) {
        double two_n = std::pow(2.0, nd.n);
        double xl = r[d] / w.sf[d] * two_n - nd.l[d];
        for (int q = 0; q < K; q++) phi[(size_t)d * K + q] = b.eval(q, xl);
        fac *= std::sqrt(two_n / w.sf[d]);
    }
    const double *s = t.c(i);
    double v = 0.0;
    for (int p = 0; p < t.kp1_d; p++) {
        double term = s[p];
        int rem = p;
        for (int d = 0; d < D; d++) { term *= phi[(size_t)d * K + rem % K]; rem /= K; }
        v += term;
    }
    return fac * v;
}

template <int D> double integrate(const Tree<D> &t) {
    const auto &w = t.mra->world;
    const auto &b = *t.mra->basis;
    const int K = t.K;
    std::vector<double> ip(K);
    for (int q = 0; q < K; q++) ip[q] = (b.type == Legendre) ? (q == 0 ? 1.0 : 0.0) : std::sqrt(b.weights[q]);
    double s = 0.0;
    for (int r : t.roots) {
        double fac = 1.0;
        for (int d = 0; d < D; d++) fac *= std::sqrt(w.sf[d] * std::pow(2.0, -t.nodes[r].n));
        const double *c = t.c(r);
        double v = 0.0;
        for (int p = 0; p < t.kp1_d; p++) {
            double term = c[p];
            int rem = p;
            for (int d = 0; d < D; d++) { term *= ip[rem % K]; rem /= K; }
            v += term;
        }
        s += fac * v;
    }
    return s;
}

#define MWH_PINST(D)                                                                                      \
    template struct GaussFunc<D>;                                                                         \
    template void build_grid<D>(Tree<D> &, const GaussFunc<D> &);                                         \
    template void build_grid<D>(Tree<D> &, const GaussExp<D> &);                                          \
    template void project<D>(double, Tree<D> &, const std::function<double(const double *)> &, int, bool); \
    template void project_batched<D>(double, Tree<D> &, const BatchFunc &, int, bool); \
    template void copy_grid<D>(Tree<D> &, const Tree<D> &);                                               \
    template double dot<D>(const Tree<D> &, const Tree<D> &);                                             \
    template double evalf<D>(const Tree<D> &, const double *);                                            \
    template double integrate<D>(const Tree<D> &);
MWH_PINST(1)
MWH_PINST(2)
MWH_PINST(3)

}  // namespace mwh
