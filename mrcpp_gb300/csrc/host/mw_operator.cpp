// Construction of the separated convolution operators (host, one-time).
//
// Follows src/operators/PoissonKernel.cpp:48-86, HelmholtzKernel.cpp:47-80,
// PoissonOperator.cpp:40-55, HelmholtzOperator.cpp:41-56,
// ConvolutionOperator.cpp:51-142, MWOperator.cpp:35-129,
// src/treebuilders/CrossCorrelationCalculator.cpp:36-96, OperatorAdaptor.h:32-49,
// src/trees/OperatorNode.cpp:56-80 (component norms),
// src/trees/OperatorTree.cpp:109-134 (band width), :200-238 (node cache).
#include "mw_host.h"

namespace mwh {

namespace {
constexpr double root_pi = 1.7724538509055160273;  // api/constants.h
}  // namespace

// 1/r and exp(-mu r)/r as sums of Gaussians from a truncated trapezoidal
// rule in s after the substitution that turns the kernel's integral
// representation into a sum of Gaussians in r (PoissonKernel.cpp:48-86,
// HelmholtzKernel.cpp:47-80).  The steps, the operation order and the long
// double literals are the reference's: the number of terms and every exponent
// depend on their rounding, and the reference's tests pin the term counts
// (26 for Poisson at 1e-5, 33 for Helmholtz).  Lengths are in units of
// r_max; the rule runs over s in [s_lo, s_hi] with step `step`, end points
// at half weight.
std::vector<GaussFunc<1>> poisson_kernel(double epsilon, double r_min, double r_max) {
    std::vector<GaussFunc<1>> out;
    const double r_rel = r_min / r_max, unit = r_max;
    // where the integrand has decayed below epsilon at both ends
    double t_lo = 1.0L;
    while ((2.0 * t_lo * std::exp(-t_lo)) > epsilon) t_lo *= 1.1L;
    double t_hi = 1.0L;
    while ((std::sqrt(t_hi) * std::exp(-t_hi) / r_rel) > epsilon) t_hi *= 1.1L;
    const double s_lo = -std::log(2.0 * t_lo);
    const double s_hi = std::log(t_hi / (r_rel * r_rel)) / 2.0;
    const double step = 1.0 / (0.2L - 0.47L * std::log10(epsilon));
    const int n_terms = static_cast<int>(std::ceil((s_hi - s_lo) / step) + 1);
    if (n_terms > MaxSepRank) throw Error(1, "Maximum separation rank exceeded.");
    for (int k = 0; k < n_terms; k++) {
        const double s = s_lo + step * k;
        const double sh = std::sinh(s), ch = std::cosh(s);
        const double w = 1.0 + std::exp(-sh);
        double alpha = 4.0L * (sh + std::log(w)) * (sh + std::log(w));
        double beta = step * (4.0L / root_pi) * ch / w;
        alpha *= 1.0 / (unit * unit);
        beta *= 1.0 / unit;
        if (k == 0 || k == (n_terms - 1)) beta *= 1.0 / 2.0;
        out.push_back(GaussFunc<1>(alpha, beta));
    }
    return out;
}

std::vector<GaussFunc<1>> helmholtz_kernel(double mu, double epsilon, double r_min, double r_max) {
    std::vector<GaussFunc<1>> out;
    const double r_rel = r_min / r_max, unit = r_max;
    const double mu_u = mu * unit;  // mu in units of r_max
    const double t = std::max((-2.5L * std::log(epsilon)), 5.0L);
    const double s_lo = -std::log(4 * t / (mu_u * mu_u)) / 2;
    const double s_hi = std::log(t / (r_rel * r_rel)) / 2;
    const double step = 1.0 / (0.20L - 0.47L * std::log10(epsilon));
    const int n_terms = static_cast<int>(std::ceil((s_hi - s_lo) / step) + 1);
    if (n_terms > MaxSepRank) throw Error(1, "Maximum separation rank exceeded.");
    for (int k = 0; k < n_terms; k++) {
        const double s = s_lo + step * k;
        const double two_s_neg = -s * 2.0;
        const double log_w = -mu_u * mu_u * std::exp(two_s_neg) / 4.0 + s;
        double beta = (step * (2.0 / root_pi) * std::exp(log_w));
        const double two_s = 2.0L * s;
        double alpha = std::exp(two_s);
        alpha *= 1.0 / (unit * unit);
        beta *= 1.0 / unit;
        if (k == 0 || k == (n_terms - 1)) beta *= 1.0 / 2.0;
        out.push_back(GaussFunc<1>(alpha, beta));
    }
    return out;
}

// OperatorNode::calcComponentNorm
static double oper_component_norm(const Tree<2> &t, int node, int comp, double normPrec) {
    int depth = t.depth(node);
    double thrs = std::max(MachinePrec, normPrec / (8.0 * (1 << depth)));
    const int K = t.K;
    const double *m = t.c(node) + (size_t)comp * K * K;
    double sq = 0.0;
    for (int j = 0; j < K * K; j++) sq += m[j] * m[j];
    double vecNorm = std::sqrt(sq);
    double norm = 0.0;
    if (vecNorm > thrs) {
        double infNorm = 0.0, oneNorm = 0.0;
        for (int r = 0; r < K; r++) {
            double s = 0.0;
            for (int c = 0; c < K; c++) s += std::fabs(m[r + K * c]);
            infNorm = std::max(infNorm, s);
        }
        for (int c = 0; c < K; c++) {
            double s = 0.0;
            for (int r = 0; r < K; r++) s += std::fabs(m[r + K * c]);
            oneNorm = std::max(oneNorm, s);
        }
        if (std::sqrt(infNorm * oneNorm) > thrs) {
            double twoNorm = vecNorm;
            if (twoNorm > thrs) norm = twoNorm;
        }
    }
    return norm;
}

// OperatorTree::setupOperNodeCache (OperatorTree.cpp:200-238): per depth the
// nodes (0, i) for l = -i and (i, 0) for l = i, l in [-L, L]
static OperatorTerm term_from_tree(Tree<2> &otree, int operRoot, int K) {
    OperatorTerm term;
    auto levels = otree.nodesByDepth(false);
    int nScales = (int)levels.size();
    term.depth = nScales;
    term.maxTransl.assign(nScales, 0);
    for (int n = 0; n < nScales; n++)
        for (int i : levels[n]) {
            term.maxTransl[n] = std::max(term.maxTransl[n], std::abs(otree.nodes[i].l[0]));
            term.maxTransl[n] = std::max(term.maxTransl[n], std::abs(otree.nodes[i].l[1]));
        }
    std::vector<std::vector<int>> cache(nScales);
    for (int n = 0; n < nScales; n++) {
        int scale = operRoot + n;
        int L = term.maxTransl[n];
        cache[n].assign(2 * L + 1, -1);
        for (int i = L; i >= 0; i--) {
            int l[2] = {0, i};
            cache[n][L - i] = otree.getNode(scale, l, false);
        }
        for (int i = 1; i <= L; i++) {
            int l[2] = {i, 0};
            cache[n][L + i] = otree.getNode(scale, l, false);
        }
    }
    size_t total = 0;
    term.offset.resize(nScales);
    for (int n = 0; n < nScales; n++) { term.offset[n] = total; total += cache[n].size(); }
    term.blocks.assign(total * 4 * K * K, 0.0);
    term.norms.assign(total * 4, 0.0);
    for (int n = 0; n < nScales; n++)
        for (size_t j = 0; j < cache[n].size(); j++) {
            int node = cache[n][j];
            if (node < 0) continue;  // not in the tree: a zero node
            size_t idx = term.offset[n] + j;
            std::memcpy(&term.blocks[idx * 4 * K * K], otree.c(node), sizeof(double) * 4 * K * K);
            for (int c = 0; c < 4; c++) term.norms[idx * 4 + c] = otree.nodes[node].norms[c];
        }
    return term;
}

void build_operator_terms(ConvolutionOperator &op, double k_prec, double o_prec) {
    const MRA<3> &mra = op.mra;
    const auto &box = mra.world;
    const int type = mra.basis->type;
    const int k = mra.order();
    int reach = op.operReach + 1;
    if (reach < 0)
        for (int d = 0; d < 3; d++)
            if (box.size(d) > reach) reach = box.size(d);
    double sf = box.sf[0];
    // kernel MRA (ConvolutionOperator::getKernelMRA) and operator MRA (MWOperator::getOperatorMRA)
    MRA<1> kmra(BoundingBox<1>(op.operRoot, {-reach}, {2 * reach}, {sf}), type, 2 * k + 1);
    MRA<2> omra(BoundingBox<2>(op.operRoot, {0, 0}, {reach, reach}, {sf, sf}), type, k);
    const int K = k + 1, Kp = 2 * K;
    Mat Lm = table(2, type, k), Rm = table(3, type, k);
    for (auto *M : {&Lm, &Rm})
        for (auto &x : M->a)
            if (std::fabs(x) < MachinePrec) x = 0.0;

    op.terms.clear();
    for (const auto &g : op.kernel) {
        GaussFunc<1> kf = g;
        kf.coef = std::copysign(std::pow(std::fabs(g.coef), 1.0 / 3.0), g.coef);
        Tree<1> ktree(kmra);
        build_grid(ktree, kf);
        project<1>(k_prec, ktree, [&kf](const double *r) { return kf.evalf(r); });

        Tree<2> otree(omra);
        otree.componentNorm = [o_prec](const Tree<2> &t, int i, int c) { return oper_component_norm(t, i, c, o_prec); };
        auto calc = [&](Tree<2> &t, const std::vector<int> &work) {
            for (int node : work) {
                double *coefs = t.c(node);
                std::fill(coefs, coefs + t.nCoefs, 0.0);
                int scale = t.nodes[node].n + 1;
                for (int i = 0; i < 4; i++) {
                    int l0 = 2 * t.nodes[node].l[0] + (i & 1);
                    int l1 = 2 * t.nodes[node].l[1] + ((i >> 1) & 1);
                    int la[1] = {l1 - l0 - 1}, lb[1] = {l1 - l0};
                    int na = ktree.getNode(scale, la, true);
                    int nb = ktree.getNode(scale, lb, true);
                    const double *sa = ktree.c(na), *sb = ktree.c(nb);
                    for (int r = 0; r < K * K; r++) {
                        double va = 0.0, vb = 0.0;
                        for (int p = 0; p < Kp; p++) va += Lm(r, p) * sa[p];
                        for (int p = 0; p < Kp; p++) vb += Rm(r, p) * sb[p];
                        coefs[i * K * K + r] = va + vb;
                    }
                }
                double two_n = std::pow(2.0, -scale / 2.0);
                for (int j = 0; j < t.nCoefs; j++) coefs[j] = std::sqrt(sf) * two_n * coefs[j];
                t.mwTransformNode(node, Compression);
                t.nodes[node].flags |= F_HASCOEFS;
                t.calcNorms(node);
            }
        };
        auto split = [](const Tree<2> &t, int i) {
            const auto &n = t.nodes[i];
            bool chkTransl = (n.l[0] == 0 || n.l[1] == 0);
            bool chkCompNorm = false;
            for (int c = 1; c < 4; c++)
                if (n.norms[c] > 0.0) chkCompNorm = true;
            return chkTransl && chkCompNorm;
        };
        tree_build<2>(otree, otree.endNodes(), calc, split, -1, omra.maxScale());
        otree.mwTransformUp();

        op.terms.push_back(term_from_tree(otree, op.operRoot, K));
    }
    op.bandPrec = -2.0;
}

void ConvolutionOperator::calcBandWidths(double prec) {
    if (prec == bandPrec && !bandMax.empty()) return;
    int maxDepth = 0;
    for (auto &t : terms) {
        double p = prec < 0.0 ? buildPrec : prec;
        t.bw.w.assign(t.depth + 1, {-1, -1, -1, -1, -1});
        for (int depth = 0; depth < t.depth; depth++) {
            int l = 0;
            bool done = false;
            while (!done) {
                done = true;
                size_t idx = t.nodeIndex(depth, l);
                double thrs = std::max(MachinePrec, p / (8.0 * (1 << depth)));
                for (int c = 0; c < 4; c++)
                    if (t.norms[idx * 4 + c] > thrs) {
                        t.bw.setWidth(depth, c, l);
                        done = false;
                    }
                if (++l > t.maxTransl[depth]) break;
            }
        }
        if (t.bw.depth() > maxDepth) maxDepth = t.bw.depth();
    }
    bandMax.assign(maxDepth + 1, -1);
    for (auto &t : terms)
        for (int n = 0; n <= t.bw.depth(); n++)
            for (int j = 0; j < 4; j++) bandMax[n] = std::max(bandMax[n], t.bw.getWidth(n, j));
    bandPrec = prec;
}

int ConvolutionOperator::getMaxBandWidth(int depth) const {
    if (depth < 0) {
        int m = -1;
        for (int w : bandMax) m = std::max(m, w);
        return m;
    }
    if (depth < (int)bandMax.size()) return bandMax[depth];
    return -1;
}

std::unique_ptr<ConvolutionOperator> make_convolution(const MRA<3> &mra, const std::vector<GaussFunc<1>> &kernel, double prec) {
    auto op = std::make_unique<ConvolutionOperator>();
    op->mra = mra;
    op->operRoot = mra.rootScale();
    op->buildPrec = prec;
    op->kernel = kernel;
    build_operator_terms(*op, prec / 10.0, prec);
    return op;
}

// P'_m(t) = sum over k = m-1, m-3, ... >= 0 of (2k+1) P_k(t)
static double legendre_deriv(int m, double t) {
    double p0 = 1.0, p1 = t, s = 0.0;
    for (int k = 0; k < m; k++) {
        const double pk = k == 0 ? p0 : p1;
        if ((m - 1 - k) % 2 == 0) s += (2.0 * k + 1.0) * pk;
        if (k >= 1) {
            const double p2 = ((2.0 * k + 1.0) * t * p1 - k * p0) / (k + 1.0);
            p0 = p1;
            p1 = p2;
        }
    }
    return s;
}

// ABGVOperator (ABGVOperator.cpp:45-71): the operator tree of the first
// derivative with boundary parameters a, b, node by node from
// ABGVCalculator::calcNode (ABGVCalculator.cpp:118-170), refined along the
// diagonal only (BandWidthAdaptor.h:35-52: split where l0 = 0 and 2 |dl| <= bw).
// A derivative operator from its blocks: the operator tree of
// DerivativeOperator::initialize (ABGVOperator.cpp:45-71, PHOperator.cpp:46-68,
// BSOperator.cpp:46-68): nodes with l = l1 - l0 in {-1, 0, 1} get the blocks
// `fill` writes (component c, element (i, j) at c K^2 + i K + j), scaled by
// 2^(order (n+1)) and compressed (the calculators' calcNode); the tree is
// refined by BandWidthAdaptor(bw) (BandWidthAdaptor.h:45-50).
static std::unique_ptr<ConvolutionOperator> make_derivative(const MRA<3> &mra, int order, int bw,
                                                            const std::function<void(int, double *)> &fill) {
    auto op = std::make_unique<ConvolutionOperator>();
    op->mra = mra;
    op->operRoot = mra.rootScale();
    op->operReach = 1;
    op->buildPrec = MachineZero;
    op->derivOrder = order;
    const ScalingBasis &basis = *mra.basis;
    const double sf = mra.world.sf[0];
    MRA<2> omra(BoundingBox<2>(op->operRoot, {0, 0}, {op->operReach + 1, op->operReach + 1}, {sf, sf}), basis.type, mra.order());
    Tree<2> otree(omra);
    otree.componentNorm = [](const Tree<2> &t, int i, int c) { return oper_component_norm(t, i, c, MachineZero); };
    auto calc = [&](Tree<2> &t, const std::vector<int> &work) {
        for (int node : work) {
            double *coefs = t.c(node);
            std::fill(coefs, coefs + t.nCoefs, 0.0);
            const auto &nd = t.nodes[node];
            const int l = nd.l[1] - nd.l[0];
            if (l >= -1 && l <= 1) fill(l, coefs);
            const double two_np1 = std::pow(2.0, order * (nd.n + 1));
            for (int j = 0; j < t.nCoefs; j++) coefs[j] *= two_np1;
            t.mwTransformNode(node, Compression);
            t.nodes[node].flags |= F_HASCOEFS;
            t.calcNorms(node);
        }
    };
    auto split = [bw](const Tree<2> &t, int i) {
        const auto &n = t.nodes[i];
        return n.l[0] == 0 && 2 * std::abs(n.l[0] - n.l[1]) <= bw;
    };
    tree_build<2>(otree, otree.endNodes(), calc, split, -1, omra.maxScale());
    op->terms.push_back(term_from_tree(otree, op->operRoot, mra.kp1()));
    op->bandPrec = -2.0;
    return op;
}

std::unique_ptr<ConvolutionOperator> make_abgv(const MRA<3> &mra, double a, double b) {
    const int bw = (std::fabs(a) > MachineZero || std::fabs(b) > MachineZero) ? 1 : 0;
    const ScalingBasis &basis = *mra.basis;
    const int K = mra.kp1(), type = basis.type;
    // value vectors and K matrix (ABGVCalculator.cpp:48-116)
    std::vector<double> v0(K), v1(K);
    Mat Km(K, K);
    if (type == Legendre) {
        for (int i = 0; i < K; i++) {
            const double c = std::sqrt(2.0 * i + 1.0);
            v1[i] = c;
            v0[i] = (i % 2) ? -c : c;
        }
        for (int i = 0; i < K; i++)
            for (int j = i; j < K; j++)
                if ((i - j) % 2 != 0) Km(j, i) = 2.0 * std::sqrt(2.0 * i + 1.0) * std::sqrt(2.0 * j + 1.0);
    } else {
        for (int i = 0; i < K; i++) {
            v0[i] = basis.eval(i, 0.0);
            v1[i] = basis.eval(i, 1.0);
        }
        // K(i, j) = 2 sqrt(w_j) p_i'(r_j), where p_i' is the derivative of
        // phi_i(x) = sqrt(w_i) sum_m L_m(r_i) L_m(x), L_m(x) = sqrt(2m+1) P_m(2x - 1),
        // taken with respect to the polynomial's own argument 2x - 1
        // (Polynomial::calcDerivative, Polynomial.cpp:222-236): half of d/dx, so
        // K(i, j) is the integral of phi_i' phi_j over [0, 1], as in the Legendre case
        for (int i = 0; i < K; i++)
            for (int j = 0; j < K; j++) {
                double d = 0.0;
                for (int mm = 0; mm < K; mm++)
                    d += legendre_scaled(mm, basis.roots[i]) * std::sqrt(2.0 * mm + 1.0) * legendre_deriv(mm, 2.0 * basis.roots[j] - 1.0);
                Km(i, j) = 2.0 * std::sqrt(basis.weights[j]) * std::sqrt(basis.weights[i]) * d;
            }
    }
    const int K2 = K * K;
    auto fill = [&](int l, double *coefs) {
        switch (l) {
            case 1:
                if (b > MachineZero)
                    for (int i = 0; i < K; i++)
                        for (int j = 0; j < K; j++) coefs[1 * K2 + i * K + j] = -b * v0[i] * v1[j];
                break;
            case 0:
                for (int i = 0; i < K; i++)
                    for (int j = 0; j < K; j++) {
                        const double diag = (1.0 - a) * v1[i] * v1[j] - (1.0 - b) * v0[i] * v0[j] - Km(i, j);
                        coefs[0 * K2 + i * K + j] = diag;
                        coefs[1 * K2 + i * K + j] = a * v1[i] * v0[j];
                        coefs[2 * K2 + i * K + j] = -b * v0[i] * v1[j];
                        coefs[3 * K2 + i * K + j] = diag;
                    }
                break;
            default:  // l = -1
                if (a > MachineZero)
                    for (int i = 0; i < K; i++)
                        for (int j = 0; j < K; j++) coefs[2 * K2 + i * K + j] = a * v1[i] * v0[j];
                break;
        }
    };
    return make_derivative(mra, 1, bw, fill);
}

std::unique_ptr<ConvolutionOperator> make_table_derivative(const MRA<3> &mra, int order, const Mat &s_p1, const Mat &s_0, const Mat &s_m1) {
    const int K = mra.kp1(), K2 = K * K;
    if (s_p1.rows != K || s_p1.cols != K || s_0.rows != K || s_0.cols != K || s_m1.rows != K || s_m1.cols != K)
        throw Error(1, "derivative tables must be (k+1) x (k+1)");
    // PHCalculator::calcNode / BSCalculator::calcNode (PHCalculator.cpp:80-127, BSCalculator.cpp:83-127)
    auto fill = [&](int l, double *coefs) {
        for (int i = 0; i < K; i++)
            for (int j = 0; j < K; j++) {
                const int e = i * K + j;
                if (l == 1) {
                    coefs[1 * K2 + e] = s_p1(i, j);
                } else if (l == 0) {
                    coefs[0 * K2 + e] = s_0(i, j);
                    coefs[1 * K2 + e] = s_m1(i, j);
                    coefs[2 * K2 + e] = s_p1(i, j);
                    coefs[3 * K2 + e] = s_0(i, j);
                } else {
                    coefs[2 * K2 + e] = s_m1(i, j);
                }
            }
    };
    return make_derivative(mra, order, 1, fill);
}

std::unique_ptr<ConvolutionOperator> make_poisson(const MRA<3> &mra, double prec) {
    double k_prec = prec / 10.0;
    double r_min = mra.calcMinDistance(k_prec);
    double r_max = mra.calcMaxDistance();
    return make_convolution(mra, poisson_kernel(k_prec, r_min, r_max), prec);
}

std::unique_ptr<ConvolutionOperator> make_helmholtz(const MRA<3> &mra, double mu, double prec) {
    double k_prec = prec / 10.0;
    double r_min = mra.calcMinDistance(k_prec);
    double r_max = mra.calcMaxDistance();
    return make_convolution(mra, helmholtz_kernel(mu, k_prec, r_min, r_max), prec);
}

}  // namespace mwh
