// Adaptive tree container, per-node multiwavelet transforms, norms and the
// level-synchronous build loop of the host mirror.
//
// Follows src/trees/MWTree.cpp:109-216, 340-352 (square norm, BottomUp/TopDown,
// getNode with generation), src/trees/MWNode.cpp:312-335 (giveChildrenCoefs),
// :557-595 (mwTransform), :609-669 (norms, reCompress), :1097-1120
// (retrieveNode), src/trees/FunctionNode.cpp:255-328 (create/gen children),
// src/utils/tree_utils.cpp:47-65 (split_check), :113-216 (mw_transform),
// src/treebuilders/TreeBuilder.cpp:38-87 and TreeAdaptor.h:41-52.
#include "mw_host.h"

namespace mwh {

template <int D> Tree<D>::Tree(const MRA<D> &m) : mra(&m) {
    K = m.kp1();
    kp1_d = 1;
    for (int d = 0; d < D; d++) kp1_d *= K;
    nCoefs = tDim * kp1_d;
    const auto &w = m.world;
    int nr = w.totBoxes();
    for (int b = 0; b < nr; b++) {
        int l[3] = {0, 0, 0};
        int rem = b;
        for (int d = 0; d < D; d++) { l[d] = w.corner[d] + rem % w.nbox[d]; rem /= w.nbox[d]; }
        int id = addNode(w.scale, l, -1, F_ROOT);
        roots.push_back(id);
    }
}

template <int D> int Tree<D>::addNode(int n, const int *l, int parent, int flags) {
    Node nd{};
    nd.n = n;
    for (int d = 0; d < 3; d++) nd.l[d] = d < D ? l[d] : 0;
    nd.parent = parent;
    nd.child0 = -1;
    nd.flags = flags;
    for (int c = 0; c < tDim; c++) nd.norms[c] = -1.0;
    nd.squareNorm = -1.0;
    int id = (int)nodes.size();
    nodes.push_back(nd);
    coefs.resize(coefs.size() + nCoefs, 0.0);
    NodeKey k{n, {nd.l[0], nd.l[1], nd.l[2]}};
    index[k] = id;
    return id;
}

template <int D> int Tree<D>::find(int n, const int *l) const {
    NodeKey k{n, {l[0], D > 1 ? l[1] : 0, D > 2 ? l[2] : 0}};
    auto it = index.find(k);
    return it == index.end() ? -1 : it->second;
}

template <int D> void Tree<D>::createChildren(int i, bool gen) {
    if (nodes[i].child0 >= 0) throw Error(1, "Node already has children");
    int first = -1;
    for (int c = 0; c < tDim; c++) {
        int l[3] = {0, 0, 0};
        for (int d = 0; d < D; d++) l[d] = 2 * nodes[i].l[d] + ((c >> d) & 1);
        int id = addNode(nodes[i].n + 1, l, i, gen ? F_GEN : 0);
        if (c == 0) first = id;
    }
    nodes[i].child0 = first;
    nodes[i].flags |= F_BRANCH;
}

template <int D> int Tree<D>::rootIndexOf(int n, const int *l) const {
    const auto &w = mra->world;
    int shift = n - w.scale;
    int b = 0, stride = 1;
    for (int d = 0; d < D; d++) {
        int lr = shift >= 0 ? (l[d] >> shift) : l[d];
        int off = lr - w.corner[d];
        if (off < 0 || off >= w.nbox[d]) return -1;
        b += off * stride;
        stride *= w.nbox[d];
    }
    return roots[b];
}

template <int D> int Tree<D>::getNode(int n, const int *l, bool genFlag) {
    int id = find(n, l);
    if (id >= 0) return id;
    int cur = rootIndexOf(n, l);
    if (cur < 0) throw Error(1, "node index outside the world box");
    while (nodes[cur].n < n) {
        if (nodes[cur].child0 < 0) {
            createChildren(cur, genFlag);
            giveChildrenCoefs(cur, true);
        }
        int shift = n - nodes[cur].n - 1;
        int c = 0;
        for (int d = 0; d < D; d++) c |= ((l[d] >> shift) & 1) << d;
        cur = nodes[cur].child0 + c;
    }
    return cur;
}

// tree_utils::mw_transform (tree_utils.cpp:113-216): parent (s,d) -> children
// scaling blocks, children at stride `stride`; readOnlyScaling for GenNodes.
template <int D>
static void mw_transform(const ScalingBasis &b, const double *in, double *out, bool readOnlyScaling, int stride, bool overwrite) {
    const int K = b.K, tDim = 1 << D;
    int kp1_d = 1;
    for (int d = 0; d < D; d++) kp1_d *= K;
    int kp1_dm1 = kp1_d / K;
    std::vector<double> t1((size_t)kp1_d * tDim), t2((size_t)kp1_d * tDim);
    const double *src = in;
    int srcStride = kp1_d;
    for (int i = 0; i < D; i++) {
        int mask = 1 << i;
        int ftlim = readOnlyScaling ? (1 << i) : tDim;
        bool last = (i == D - 1);
        double *dst = (i % 2 == 0) ? t1.data() : t2.data();
        for (int gt = 0; gt < tDim; gt++) {
            double *o = last ? out + (size_t)gt * stride : dst + (size_t)gt * kp1_d;
            bool add = last ? !overwrite : false;
            for (int ft = 0; ft < ftlim; ft++) {
                if ((gt | mask) != (ft | mask)) continue;
                const double *x = src + (size_t)ft * srcStride;
                int fidx = 2 * ((gt >> i) & 1) + ((ft >> i) & 1);
                apply_filter(o, x, b.sub[Reconstruction][fidx], K, kp1_dm1, add);
                add = true;
            }
        }
        src = dst;
        srcStride = kp1_d;
    }
}

template <int D> void Tree<D>::giveChildrenCoefs(int i, bool overwrite) {
    int c0 = nodes[i].child0;
    if (c0 < 0) throw Error(1, "giveChildrenCoefs on leaf");
    if (overwrite)
        for (int c = 0; c < tDim; c++) std::fill(this->c(c0 + c), this->c(c0 + c) + nCoefs, 0.0);
    mw_transform<D>(*mra->basis, this->c(i), this->c(c0), isGen(i), nCoefs, overwrite);
    for (int c = 0; c < tDim; c++) {
        nodes[c0 + c].flags |= F_HASCOEFS;
        calcNorms(c0 + c);
    }
}

template <int D> std::vector<double> Tree<D>::maxNorms(bool wavelet) const {
    std::vector<double> msq(nodes.size(), -1.0);
    auto scaled = [this, wavelet](int i) {
        double sq = 0.0;
        for (int c = wavelet ? 1 : 0; c < tDim; c++) sq += nodes[i].norms[c] * nodes[i].norms[c];
        return std::ldexp(1.0, D * nodes[i].n) * sq;
    };
    // deepest level first, so that every child is done before its parent
    const auto levels = nodesByDepth(true);
    for (auto it = levels.rbegin(); it != levels.rend(); ++it)
        for (int i : *it) {
            double m = scaled(i);
            const int c0 = nodes[i].child0;
            if (!isGen(i) && c0 >= 0 && !isGen(c0))
                for (int c = 0; c < tDim; c++) m = std::max(m, msq[c0 + c]);
            msq[i] = m;
        }
    return msq;
}

template <int D> double Tree<D>::genScaledSquareNorm(int n, const int *l) const {
    int cur = rootIndexOf(n, l);
    if (cur < 0) throw Error(1, "node index outside the world box");
    std::vector<double> blk(c(cur), c(cur) + nCoefs), kids((size_t)tDim * nCoefs);
    bool gen = isGen(cur);
    int at = nodes[cur].n;
    while (at < n) {
        const int shift = n - at - 1;
        int ci = 0;
        for (int d = 0; d < D; d++) ci |= ((l[d] >> shift) & 1) << d;
        const int c0 = (cur >= 0) ? nodes[cur].child0 : -1;
        if (c0 >= 0) {
            cur = c0 + ci;
            blk.assign(c(cur), c(cur) + nCoefs);
            gen = isGen(cur);
        } else {
            // giveChildrenCoefs(overwrite = true) of a leaf: children scaling blocks
            std::fill(kids.begin(), kids.end(), 0.0);
            mw_transform<D>(*mra->basis, blk.data(), kids.data(), gen, nCoefs, true);
            blk.assign(kids.begin() + (size_t)ci * nCoefs, kids.begin() + (size_t)(ci + 1) * nCoefs);
            gen = true;
            cur = -1;
        }
        at++;
    }
    double sq;
    if (cur >= 0) {
        sq = 0.0;
        for (int c = 0; c < tDim; c++) sq += nodes[cur].norms[c] * nodes[cur].norms[c];
    } else {
        // calcNorms of a GenNode: the scaling component only
        double s = 0.0;
        for (int j = 0; j < kp1_d; j++) s += blk[j] * blk[j];
        const double nrm = std::sqrt(s);
        sq = nrm * nrm;
    }
    return std::ldexp(1.0, D * n) * sq;
}

template <int D> void Tree<D>::calcNorms(int i) {
    double sq = 0.0;
    for (int c = 0; c < tDim; c++) {
        double nrm;
        if (componentNorm) {
            nrm = componentNorm(*this, i, c);
        } else if (isGen(i) && c != 0) {
            nrm = 0.0;
        } else {
            const double *x = this->c(i) + (size_t)c * kp1_d;
            double s = 0.0;
            for (int j = 0; j < kp1_d; j++) s += x[j] * x[j];
            nrm = std::sqrt(s);
        }
        nodes[i].norms[c] = nrm;
        sq += nrm * nrm;
    }
    nodes[i].squareNorm = sq;
}

template <int D> double Tree<D>::waveletNorm(int i) const {
    double w = 0.0;
    for (int c = 1; c < tDim; c++) {
        double n = nodes[i].norms[c];
        if (n >= 0.0) w += n * n;
        else w = -1.0;
    }
    return w;
}

template <int D> void Tree<D>::mwTransformNode(int i, int op) {
    const auto &b = *mra->basis;
    int kp1_dm1 = kp1_d / K;
    std::vector<double> tmp(nCoefs);
    double *in = this->c(i), *out = tmp.data();
    for (int d = 0; d < D; d++) {
        int mask = 1 << d;
        for (int gt = 0; gt < tDim; gt++) {
            double *o = out + (size_t)gt * kp1_d;
            bool add = false;
            for (int ft = 0; ft < tDim; ft++) {
                if ((gt | mask) != (ft | mask)) continue;
                int fidx = 2 * ((gt >> d) & 1) + ((ft >> d) & 1);
                apply_filter(o, in + (size_t)ft * kp1_d, b.sub[op][fidx], K, kp1_dm1, add);
                add = true;
            }
        }
        std::swap(in, out);
    }
    if (D % 2 == 1) std::memcpy(this->c(i), in, sizeof(double) * nCoefs);
}

template <int D> void Tree<D>::reCompress(int i) {
    int c0 = nodes[i].child0;
    if (c0 < 0) return;
    double *p = this->c(i);
    for (int c = 0; c < tDim; c++) std::memcpy(p + (size_t)c * kp1_d, this->c(c0 + c), sizeof(double) * kp1_d);
    mwTransformNode(i, Compression);
    nodes[i].flags |= F_HASCOEFS;
    calcNorms(i);
}

template <int D> std::vector<std::vector<int>> Tree<D>::nodesByDepth(bool includeGen) const {
    std::vector<std::vector<int>> out;
    // breadth-first from the roots, so that each level keeps parent order
    std::vector<int> level = roots;
    while (!level.empty()) {
        std::vector<int> next;
        std::vector<int> keep;
        for (int i : level) {
            if (!includeGen && isGen(i)) continue;
            keep.push_back(i);
            if (nodes[i].child0 >= 0)
                for (int c = 0; c < tDim; c++) next.push_back(nodes[i].child0 + c);
        }
        if (keep.empty()) break;
        out.push_back(keep);
        level.swap(next);
    }
    return out;
}

template <int D> std::vector<int> Tree<D>::endNodes() const {
    std::vector<int> out;
    for (auto &lvl : nodesByDepth(false))
        for (int i : lvl) {
            int c0 = nodes[i].child0;
            if (c0 < 0 || isGen(c0)) out.push_back(i);
        }
    return out;
}

template <int D> void Tree<D>::mwTransformUp() {
    auto table = nodesByDepth(false);
    for (int n = (int)table.size() - 2; n >= 0; n--)
        for (int i : table[n]) {
            int c0 = nodes[i].child0;
            if (c0 >= 0 && !isGen(c0)) reCompress(i);
        }
}

template <int D> void Tree<D>::mwTransformDown(bool overwrite) {
    auto table = nodesByDepth(false);
    for (auto &lvl : table)
        for (int i : lvl) {
            int c0 = nodes[i].child0;
            if (c0 >= 0 && !isGen(c0)) giveChildrenCoefs(i, overwrite);
        }
}

template <int D> void Tree<D>::calcSquareNorm() {
    double s = 0.0;
    for (int i : endNodes()) s += nodes[i].squareNorm;
    squareNorm = s;
}

template <int D> void Tree<D>::clearGenerated() {
    // Rebuild without GenNodes (FunctionTree::deleteGenerated); nothing to do
    // (and no copy of the coefficients) when the tree holds none.
    bool any = false;
    for (size_t i = 0; i < nodes.size() && !any; i++) any = isGen((int)i);
    if (!any) return;
    std::vector<int> remap(nodes.size(), -1);
    std::vector<Node> nn;
    CoefVector nc;
    for (size_t i = 0; i < nodes.size(); i++) {
        if (isGen((int)i)) continue;
        remap[i] = (int)nn.size();
        nn.push_back(nodes[i]);
        nc.insert(nc.end(), c((int)i), c((int)i) + nCoefs);
    }
    for (auto &n : nn) {
        if (n.parent >= 0) n.parent = remap[n.parent];
        if (n.child0 >= 0) {
            n.child0 = remap[n.child0];
            if (n.child0 < 0) n.flags &= ~F_BRANCH;
        }
    }
    for (auto &r : roots) r = remap[r];
    nodes.swap(nn);
    coefs.swap(nc);
    index.clear();
    for (size_t i = 0; i < nodes.size(); i++) index[NodeKey{nodes[i].n, {nodes[i].l[0], nodes[i].l[1], nodes[i].l[2]}}] = (int)i;
}

template <int D> bool split_check(const Tree<D> &t, int node, double prec, double splitFac, bool absPrec) {
    bool split = false;
    if (prec > 0.0) {
        double t_norm = 1.0;
        double sq_norm = t.squareNorm;
        if (sq_norm > 0.0 && !absPrec) t_norm = std::sqrt(sq_norm);
        double scale_fac = 1.0;
        if (splitFac > MachineZero) {
            double expo = 0.5 * splitFac * (t.nodes[node].n + 1);
            scale_fac = std::pow(2.0, -expo);
        }
        double w_thrs = std::max(2.0 * MachinePrec, prec * t_norm * scale_fac);
        double w_norm = std::sqrt(t.waveletNorm(node));
        if (w_norm > w_thrs) split = true;
    }
    return split;
}

template <int D>
void tree_build(Tree<D> &tree, std::vector<int> work, const std::function<void(Tree<D> &, const std::vector<int> &)> &calc,
                const std::function<bool(const Tree<D> &, int)> &split, int maxIter, int maxScale) {
    double sNorm = 0.0, wNorm = 0.0;
    int iter = 0;
    while (!work.empty()) {
        calc(tree, work);
        if (iter == 0) {
            sNorm = 0.0;
            for (int i : work)
                if (tree.depth(i) >= 0) sNorm += tree.scalingNorm(i);
        }
        for (int i : work)
            if (tree.depth(i) >= 0) wNorm += tree.waveletNorm(i);
        tree.squareNorm = (sNorm < 0.0 || wNorm < 0.0) ? -1.0 : sNorm + wNorm;
        if (iter >= maxIter && maxIter >= 0) work.clear();
        std::vector<int> next;
        for (int i : work) {
            if (tree.isBranch(i)) continue;
            if (tree.nodes[i].n + 2 > maxScale) continue;
            if (split(tree, i)) {
                tree.createChildren(i, false);
                int c0 = tree.nodes[i].child0;
                for (int c = 0; c < Tree<D>::tDim; c++) next.push_back(c0 + c);
            }
        }
        work.swap(next);
        iter++;
    }
}

#define MWH_INST(D)                                                                                                   \
    template struct Tree<D>;                                                                                          \
    template bool split_check<D>(const Tree<D> &, int, double, double, bool);                                         \
    template void tree_build<D>(Tree<D> &, std::vector<int>, const std::function<void(Tree<D> &, const std::vector<int> &)> &, \
                                const std::function<bool(const Tree<D> &, int)> &, int, int);
MWH_INST(1)
MWH_INST(2)
MWH_INST(3)

}  // namespace mwh
