// Host-side mirror of MRCPP's data model for the operator-application path.
//
// This is the C++ layer that sits above the C-ABI (include/mwgpu.h).  It keeps
// the objects MRCPP keeps on the host -- MultiResolutionAnalysis, FunctionTree,
// OperatorTree, the Gaussian kernels -- and builds inputs (projection) and
// operators (kernel projection + cross correlation) exactly as the reference
// does.  The operator application itself never runs here: apply() hands every
// level to the GPU (mw_apply.cpp).
//
// Reference files followed (paths inside MRChemSoft/mrcpp):
//   src/trees/BoundingBox.cpp:47-80, 229-239     world box, scales, scaling factor
//   src/trees/MultiResolutionAnalysis.h:59-65    max scale, r_min
//   src/core/{Legendre,Interpolating}Basis.cpp   scaling bases, cv maps
//   src/core/MWFilter.cpp:100-133, 200-251       filters and sub-filter selection
//   src/utils/math_utils.cpp:175-194             apply_filter
//   src/trees/MWNode.cpp:448-669                 cv/mw transforms, norms
//   src/treebuilders/TreeBuilder.cpp:38-87       adaptive build loop
//   src/utils/tree_utils.cpp:47-65               split check
#pragma once

#include <array>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <functional>
#include <memory>
#include <stdexcept>
#include <string>
#include <unordered_map>
#include <vector>

namespace mwh {

constexpr double MachineZero = 1.0e-14;  // api/constants.h
constexpr double MachinePrec = 1.0e-15;
constexpr int MaxDepth = 30;
constexpr int MaxSepRank = 1000;
constexpr double pi = 3.14159265358979323846;

// Storage of tree coefficients.  Blocks of at least host_block_min() bytes are
// asked of host_block_alloc first: page-locked host memory kept in a cache
// (mw_pinned.cpp), so that whole-tree copies between host and device run as
// direct DMA instead of through the driver's pageable staging buffers.  When
// page-locked memory cannot be had (no device) the C heap serves.
size_t host_block_min();
void *host_block_alloc(size_t bytes);            // nullptr: declined
bool host_block_release(void *p, size_t bytes);  // false: not a page-locked block

template <class T> struct CoefAllocator {
    using value_type = T;
    CoefAllocator() noexcept = default;
    template <class U> CoefAllocator(const CoefAllocator<U> &) noexcept {}
    T *allocate(size_t n) {
        const size_t bytes = n * sizeof(T);
        if (bytes >= host_block_min())
            if (void *p = host_block_alloc(bytes)) return static_cast<T *>(p);
        return std::allocator<T>().allocate(n);
    }
    void deallocate(T *p, size_t n) noexcept {
        const size_t bytes = n * sizeof(T);
        if (bytes >= host_block_min() && host_block_release(p, bytes)) return;
        std::allocator<T>().deallocate(p, n);
    }
    template <class U> bool operator==(const CoefAllocator<U> &) const noexcept { return true; }
    template <class U> bool operator!=(const CoefAllocator<U> &) const noexcept { return false; }
};
using CoefVector = std::vector<double, CoefAllocator<double>>;

enum BasisType { Legendre = 0, Interpol = 1 };
enum Operation { Compression = 0, Reconstruction = 1 };

struct Error : std::runtime_error {
    int code;
    Error(int c, const std::string &m) : std::runtime_error(m), code(c) {}
};

// ---------------------------------------------------------------------------
// Tables (filters, cross correlation) generated by data/gen_mwtables.py.
// ---------------------------------------------------------------------------
struct Mat {  // column-major dense matrix
    int rows = 0, cols = 0;
    std::vector<double> a;
    Mat() = default;
    Mat(int r, int c) : rows(r), cols(c), a((size_t)r * c, 0.0) {}
    double &operator()(int i, int j) { return a[i + (size_t)rows * j]; }
    double operator()(int i, int j) const { return a[i + (size_t)rows * j]; }
    const double *data() const { return a.data(); }
    Mat transpose() const {
        Mat t(cols, rows);
        for (int i = 0; i < rows; i++)
            for (int j = 0; j < cols; j++) t(j, i) = (*this)(i, j);
        return t;
    }
};

// Returns a table (row-major in the file, returned as Mat) or throws.
const Mat &table(int kind, int type, int k);
void set_table_path(const std::string &path);

// Scaling basis of order k (K = k+1 functions), with quadrature and filters.
struct ScalingBasis {
    int type = Interpol, order = 0, K = 1;
    std::vector<double> roots, weights;  // Gauss-Legendre on [0,1], ascending
    Mat vcMap, cvMap;                    // value->coef (Backward) and coef->value (Forward)
    Mat H0, H1, G0, G1;                  // two-scale filters
    Mat sub[2][4];                       // [Compression|Reconstruction][2*gt_bit + ft_bit]
    ScalingBasis() = default;
    ScalingBasis(int type, int order);
    double eval(int j, double x) const;  // phi_j(x), x in [0,1]
};
const ScalingBasis &get_basis(int type, int order);
// sqrt(2j+1) P_j(2x - 1): the Legendre scaling function j on [0, 1]
double legendre_scaled(int j, double x);

// Gauss-Legendre nodes/weights on [0,1] computed in double (ascending).
void gauss_legendre01(int n, std::vector<double> &x, std::vector<double> &w);

// g(K^{D-1} x K) (=|+=) f^T (K^{D-1} x K) * F(K x K), MRCPP's apply_filter.
void apply_filter(double *out, const double *in, const Mat &F, int K, int Kdm1, bool add);

// ---------------------------------------------------------------------------
// World box and MRA
// ---------------------------------------------------------------------------
template <int D> struct BoundingBox {
    int scale = 0;
    std::array<int, D> corner{};
    std::array<int, D> nbox{};
    std::array<double, D> sf{};
    BoundingBox() { nbox.fill(1); sf.fill(1.0); }
    BoundingBox(int n, const std::array<int, D> &l, const std::array<int, D> &nb, const std::array<double, D> &s)
        : scale(n), corner(l), nbox(nb), sf(s) {}
    // MRCPP BoundingBox({lb, ub}) constructor (BoundingBox.cpp:47-80)
    static BoundingBox fromBounds(int lb, int ub);
    int size(int d) const { return nbox[d]; }
    int totBoxes() const { int t = 1; for (int d = 0; d < D; d++) t *= nbox[d]; return t; }
    double unitLength(int d) const { return sf[d] * std::pow(2.0, -scale); }
    double lower(int d) const { return corner[d] * unitLength(d); }
    double upper(int d) const { return lower(d) + unitLength(d) * nbox[d]; }
    bool operator==(const BoundingBox &o) const { return scale == o.scale && corner == o.corner && nbox == o.nbox && sf == o.sf; }
};

template <int D> struct MRA {
    BoundingBox<D> world;
    const ScalingBasis *basis = nullptr;
    int maxDepth = MaxDepth;
    MRA() = default;
    MRA(const BoundingBox<D> &b, int type, int order, int depth = MaxDepth) : world(b), basis(&get_basis(type, order)), maxDepth(depth) {
        if (depth > MaxDepth) throw Error(1, "Beyond MaxDepth");
    }
    int order() const { return basis->order; }
    int kp1() const { return basis->K; }
    int rootScale() const { return world.scale; }
    int maxScale() const { return world.scale + maxDepth; }
    double calcMinDistance(double eps) const { return std::sqrt(eps * std::pow(2.0, -maxScale())); }
    double calcMaxDistance() const {
        double s = 0.0;
        for (int d = 0; d < D; d++) { double x = world.upper(d) - world.lower(d); s += x * x; }
        return std::sqrt(s);
    }
    bool operator==(const MRA &o) const { return world == o.world && basis == o.basis && maxDepth == o.maxDepth; }
};

// ---------------------------------------------------------------------------
// Adaptive 2^D-tree with flat node storage.
// ---------------------------------------------------------------------------
struct NodeKey {
    int n;
    int l[3];
    bool operator==(const NodeKey &o) const { return n == o.n && l[0] == o.l[0] && l[1] == o.l[1] && l[2] == o.l[2]; }
};
struct NodeKeyHash {
    size_t operator()(const NodeKey &k) const {
        uint64_t h = (uint64_t)(uint32_t)k.n * 0x9E3779B97F4A7C15ull;
        for (int d = 0; d < 3; d++) { h ^= (uint64_t)(uint32_t)k.l[d] + 0x9E3779B97F4A7C15ull + (h << 6) + (h >> 2); }
        return (size_t)h;
    }
};

enum NodeFlags { F_BRANCH = 1, F_GEN = 2, F_HASCOEFS = 4, F_ROOT = 8 };

template <int D> struct Tree {
    static constexpr int tDim = 1 << D;
    struct Node {
        int n;
        int l[3];
        int parent;
        int child0;  // first of tDim contiguous children, -1 if leaf
        int flags;
        double norms[1 << D];
        double squareNorm;
    };
    const MRA<D> *mra;
    int K, kp1_d, nCoefs;
    std::vector<Node> nodes;
    CoefVector coefs;  // nodes.size() * nCoefs
    std::unordered_map<NodeKey, int, NodeKeyHash> index;
    std::vector<int> roots;
    double squareNorm = -1.0;

    explicit Tree(const MRA<D> &m);
    int addNode(int n, const int *l, int parent, int flags);
    int find(int n, const int *l) const;
    double *c(int i) { return coefs.data() + (size_t)i * nCoefs; }
    const double *c(int i) const { return coefs.data() + (size_t)i * nCoefs; }
    bool isBranch(int i) const { return nodes[i].flags & F_BRANCH; }
    bool isGen(int i) const { return nodes[i].flags & F_GEN; }
    int depth(int i) const { return nodes[i].n - mra->rootScale(); }
    void createChildren(int i, bool gen = false);
    // MWTree::getNode: returns node, generating missing ones by reconstruction.
    // gen=true marks new nodes as GenNodes (FunctionTree), false as real nodes
    // (OperatorNode::genChildren).
    int getNode(int n, const int *l, bool genFlag = true);
    int rootIndexOf(int n, const int *l) const;
    void giveChildrenCoefs(int i, bool overwrite);
    void calcNorms(int i);  // plain vector norms of each component (MWNode::calcComponentNorm)
    double scalingNorm(int i) const { double s = nodes[i].norms[0]; return s >= 0 ? s * s : -1.0; }
    double waveletNorm(int i) const;
    void mwTransformNode(int i, int op);  // MWNode::mwTransform, in place
    void reCompress(int i);               // children scaling -> parent s+d
    void mwTransformUp();                 // BottomUp
    void mwTransformDown(bool overwrite); // TopDown
    void calcSquareNorm();
    std::vector<std::vector<int>> nodesByDepth(bool includeGen = false) const;
    std::vector<int> endNodes() const;
    void clearGenerated();
    // MWNode::getMaxSquareNorm of every node after MWTree::makeMaxSquareNorms
    // (MWTree.cpp:536-543, MWNode.cpp:1257-1269, MWNode.h:84,212): the largest
    // 2^(D n) |node|^2 over the node and its real descendants; GenNodes get
    // their own scaled square norm
    std::vector<double> maxSquareNorms() const { return maxNorms(false); }
    // the same over the wavelet part alone (maxWSquareNorm, MWNode.h:85,213)
    std::vector<double> maxWSquareNorms() const { return maxNorms(true); }
    std::vector<double> maxNorms(bool wavelet) const;
    // the scaled square norm 2^(D n) |s|^2 of the node (n, l) where it is
    // missing: its scaling block made from the deepest existing ancestor as
    // getNode would generate it (the tree is not changed)
    double genScaledSquareNorm(int n, const int *l) const;
    // norm override hook (OperatorNode::calcComponentNorm); nullptr = plain
    std::function<double(const Tree &, int, int)> componentNorm;
};

// MRCPP TreeBuilder::build loop (TreeBuilder.cpp:38-87).  calc computes the
// nodes in work (coefs + norms); split decides refinement of one node.
template <int D>
void tree_build(Tree<D> &tree, std::vector<int> work, const std::function<void(Tree<D> &, const std::vector<int> &)> &calc,
                const std::function<bool(const Tree<D> &, int)> &split, int maxIter, int maxScale);

// tree_utils::split_check (tree_utils.cpp:47-65)
template <int D> bool split_check(const Tree<D> &t, int node, double prec, double splitFac, bool absPrec);

// ---------------------------------------------------------------------------
// Gaussians (src/functions/GaussFunc.cpp, Gaussian.cpp)
// ---------------------------------------------------------------------------
template <int D> struct GaussFunc {
    double coef = 1.0;
    std::array<double, D> alpha{};
    std::array<double, D> pos{};
    std::array<int, D> power{};
    GaussFunc() = default;
    GaussFunc(double a, double c, const std::array<double, D> &p = {}) : coef(c), pos(p) { alpha.fill(a); power.fill(0); }
    double evalf(const double *r) const;
    bool isVisibleAtScale(int scale, int nQuadPts) const;
    bool isZeroOnInterval(const double *a, const double *b) const;
    double calcSquareNorm() const;
};
template <int D> struct GaussExp {
    std::vector<GaussFunc<D>> funcs;
    double evalf(const double *r) const { double s = 0; for (auto &g : funcs) s += g.evalf(r); return s; }
};

// build_grid (grid.cpp:78-124) and project (project.cpp:41-66)
template <int D> void build_grid(Tree<D> &tree, const GaussFunc<D> &f);
template <int D> void build_grid(Tree<D> &tree, const GaussExp<D> &f);
template <int D> void project(double prec, Tree<D> &tree, const std::function<double(const double *)> &f, int maxIter = -1, bool absPrec = false);
// a function of n points (3 doubles each) writing n values
using BatchFunc = std::function<void(long long n, const double *r, double *values)>;
constexpr size_t kProjectBatch = size_t(1) << 20;  // points per callback call
template <int D> void project_batched(double prec, Tree<D> &tree, const BatchFunc &f, int maxIter = -1, bool absPrec = false);
// copy_grid (grid.cpp:220): out gets the topology of inp, no coefficients
template <int D> void copy_grid(Tree<D> &out, const Tree<D> &inp);
// dot product of two compressed trees (multiply.cpp:286)
template <int D> double dot(const Tree<D> &a, const Tree<D> &b);
// pointwise evaluation from the leaf scaling coefficients
template <int D> double evalf(const Tree<D> &t, const double *r);
template <int D> double integrate(const Tree<D> &t);

// ---------------------------------------------------------------------------
// Convolution operators (src/operators)
// ---------------------------------------------------------------------------
struct BandWidth {  // src/trees/BandWidth.h:37-61
    std::vector<std::array<int, 5>> w;  // rows 0..depth
    int depth() const { return (int)w.size() - 1; }
    int getWidth(int d, int idx) const { return (d > depth() || d < 0) ? -1 : w[d][idx]; }
    int getMaxWidth(int d) const { return getWidth(d, 4); }
    void setWidth(int d, int idx, int wd) { w[d][idx] = wd; if (wd > w[d][4]) w[d][4] = wd; }
};

// One operator term: the 2D operator tree reduced to what apply() reads,
// namely the node cache of OperatorTree::setupOperNodeCache
// (OperatorTree.cpp:200-238): per depth, nodes for l in [-L, L].
struct OperatorTerm {
    int depth = 0;                       // number of scales (nodesAtDepth.size())
    std::vector<int> maxTransl;          // per depth
    std::vector<size_t> offset;          // per depth: index of node l=-L in blocks/norms
    std::vector<double> blocks;          // per node 4*K*K (T,C,B,A), column-major K x K each
    std::vector<double> norms;           // per node 4 component norms
    BandWidth bw;                        // at the last calcBandWidth precision
    size_t nodeIndex(int d, int l) const { return offset[d] + (size_t)(l + maxTransl[d]); }
};

struct ConvolutionOperator {
    MRA<3> mra;
    int operRoot = 0;
    int operReach = -10;
    double buildPrec = -1.0;
    std::vector<GaussFunc<1>> kernel;    // separated Gaussian expansion
    std::vector<OperatorTerm> terms;     // one per kernel term (isotropic: same in x,y,z)
    std::vector<int> bandMax;            // MWOperator::band_max
    double bandPrec = -2.0;              // precision of the current band widths
    int derivOrder = 0;                  // DerivativeOperator::getOrder (0: a convolution)
    int K() const { return mra.kp1(); }
    int size() const { return (int)terms.size(); }
    void calcBandWidths(double prec);    // MWOperator.cpp:78-108
    int getMaxBandWidth(int depth) const;
};

// PoissonKernel.cpp:48-86, HelmholtzKernel.cpp:47-80
std::vector<GaussFunc<1>> poisson_kernel(double epsilon, double r_min, double r_max);
std::vector<GaussFunc<1>> helmholtz_kernel(double mu, double epsilon, double r_min, double r_max);
// PoissonOperator.cpp:40-55, HelmholtzOperator.cpp:41-56
std::unique_ptr<ConvolutionOperator> make_poisson(const MRA<3> &mra, double prec);
std::unique_ptr<ConvolutionOperator> make_helmholtz(const MRA<3> &mra, double mu, double prec);
// ABGVOperator(mra, a, b) (ABGVOperator.cpp:45-71): first derivative, band 0 (a = b = 0) or 1
std::unique_ptr<ConvolutionOperator> make_abgv(const MRA<3> &mra, double a, double b);
// PHOperator / BSOperator (PHOperator.cpp:46-68, BSOperator.cpp:46-68): derivative
// of order `order` from the tables S_+1, S_0, S_-1 ((k+1) x (k+1), element (i, j)
// as PHCalculator / BSCalculator read it) of the basis
std::unique_ptr<ConvolutionOperator> make_table_derivative(const MRA<3> &mra, int order, const Mat &s_p1, const Mat &s_0, const Mat &s_m1);
// ConvolutionOperator(mra, kernel, prec) (ConvolutionOperator.cpp:51-62)
std::unique_ptr<ConvolutionOperator> make_convolution(const MRA<3> &mra, const std::vector<GaussFunc<1>> &kernel, double prec);
// ConvolutionOperator::initialize (ConvolutionOperator.cpp:78-108), k_prec/o_prec given
void build_operator_terms(ConvolutionOperator &op, double k_prec, double o_prec);

}  // namespace mwh
