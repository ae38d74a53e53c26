/*
 * mwhost.h -- C interface of the host-side mirror of MRCPP used to drive the
 * GPU path without MRCPP itself: MultiResolutionAnalysis<3>, FunctionTree<3>,
 * GaussFunc/GaussExp projection, PoissonOperator/HelmholtzOperator
 * construction and mrcpp::apply.  Names and argument meaning follow the
 * reference API:
 *   mwh_apply          mrcpp::apply(prec, out, oper, inp, maxIter, absPrec)   src/treebuilders/apply.h:41
 *   mwh_apply_prec     mrcpp::apply(prec, out, oper, inp, precTrees, ...)      src/treebuilders/apply.h:43
 *   mwh_ph, mwh_bs     mrcpp::PHOperator / BSOperator(MRA, order)              src/operators/PHOperator.h, BSOperator.h
 *   mwh_apply_batch    a loop of mrcpp::apply over functions, one device pass
 *   mwh_poisson        mrcpp::PoissonOperator(MRA, prec)                       src/operators/PoissonOperator.h:44
 *   mwh_helmholtz      mrcpp::HelmholtzOperator(MRA, mu, prec)                 src/operators/HelmholtzOperator.h:44
 *   mwh_project_gauss  mrcpp::build_grid + mrcpp::project                      src/treebuilders/grid.h, project.h
 *   mwh_copy_grid      mrcpp::copy_grid                                         src/treebuilders/grid.h
 *   mwh_dot            mrcpp::dot(FunctionTree, FunctionTree)                  src/treebuilders/multiply.h
 * Every function returns 0 on success, a nonzero mwgpu_status-like code on
 * error; mwh_last_error() gives the message (the reference aborts instead).
 */
#ifndef MWHOST_H
#define MWHOST_H

#include "mwgpu.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct mwh_mra mwh_mra;
typedef struct mwh_tree mwh_tree;
typedef struct mwh_oper mwh_oper;

typedef struct {
    unsigned long long node_terms; /* summed over levels */
    unsigned long long components;
    unsigned long long band_nodes;
    unsigned long long gen_nodes;
    int iterations;                /* TreeBuilder iterations */
    int out_nodes;                 /* nodes of the output tree */
    double device_ms;              /* device time of all levels */
    double contract_ms;            /* device time of the contraction kernels */
    double transform_ms;           /* wall time of the TopDown + BottomUp transforms */
    double wall_ms;                /* wall time of the whole apply */
    unsigned long long launches;   /* kernels launched by this apply */
    unsigned long long h2d_bytes;  /* host-to-device bytes copied by this apply */
    unsigned long long d2h_bytes;  /* device-to-host bytes copied by this apply */
    int planned;                   /* 1: a fixed-grid apply replayed a cached level plan,
                                      2: it created that plan, 0: built the level */
} mwh_apply_stats;

const char *mwh_last_error(void);
/* Path of the MW table file (filters, cross correlation); default: found next to the library. */
int mwh_set_table_path(const char *path);

/* MultiResolutionAnalysis<3>(BoundingBox<3>(n, corner, nbox, {sf,sf,sf}), basis(type, order), max_depth);
 * type 0 = Legendre, 1 = Interpolating. */
int mwh_mra_create(int type, int order, int root_scale, const int *corner, const int *nbox, double sf, int max_depth, mwh_mra **out);
/* MultiResolutionAnalysis<3>({lb, ub}, ...) (BoundingBox.cpp:47-80) */
int mwh_mra_from_bounds(int type, int order, int lb, int ub, int max_depth, mwh_mra **out);
void mwh_mra_free(mwh_mra *mra);
/* MRA descriptor for the C-ABI; filters must hold 8*(k+1)^2 doubles. */
int mwh_mra_desc(const mwh_mra *mra, mwgpu_mra_desc *desc, double *filters);

/* The scaling basis's coefficient-to-value and value-to-coefficient maps
 * (K x K, column-major) and its quadrature roots and weights on [0, 1]
 * (ScalingBasis::getCVMap, src/core/ScalingBasis.h). */
int mwh_mra_maps(const mwh_mra *mra, double *cv_map, double *vc_map, double *roots, double *weights);
/* MultiResolutionAnalysis::calcMinDistance(eps) and calcMaxDistance()
 * (src/trees/MultiResolutionAnalysis.h:65-66): the kernel range of an operator. */
int mwh_mra_distances(const mwh_mra *mra, double eps, double *r_min, double *r_max);
int mwh_tree_create(const mwh_mra *mra, mwh_tree **out);
void mwh_tree_free(mwh_tree *tree);
/* Tree coefficients of 4 MiB and more live in page-locked host memory (so the
 * device copies of an apply run as DMA), freed blocks in a size-keyed cache;
 * MWH_PAGEABLE=1 keeps them on the C heap.  Reports the page-locked bytes in
 * trees and idle in the cache; returns 1 when page-locked memory is in use, -1
 * when it is declined (no device, or MWH_PAGEABLE=1), 0 before the first
 * large tree.  No reference counterpart (its trees are pageable). */
int mwh_pinned_stats(unsigned long long *live_bytes, unsigned long long *idle_bytes);
/* n Gaussians coef * exp(-exp * |r - pos|^2) (pos: 3n doubles). */
int mwh_build_grid_gauss(mwh_tree *tree, int n, const double *coef, const double *exp, const double *pos);
int mwh_project_gauss(double prec, mwh_tree *tree, int n, const double *coef, const double *exp, const double *pos, int max_iter,
                      int abs_prec);
/* project(prec, tree, GaussExp, maxIter, absPrec) (src/treebuilders/project.cpp:47-66)
 * with the node computations (ProjectionCalculator::calcNode) and the final
 * BottomUp on the device (mwgpu_project_level); the split test and tree
 * growth stay on the host.  stats: iterations, output nodes, wall time
 * (optional). */
int mwh_project_gauss_device(double prec, mwh_tree *tree, int n, const double *coef, const double *exp, const double *pos, int max_iter,
                             int abs_prec, mwh_apply_stats *stats);
/* project(prec, tree, std::function<double(const Coord<3> &)>, maxIter, absPrec)
 * (src/treebuilders/project.cpp:59-63, 85-102) for a host function that is evaluated
 * on many points per call: f(n, r, values, user) writes the values at the n
 * points r (3 doubles each).  The points of a TreeBuilder iteration are
 * passed in calls of at most 2^20 points; the node computations
 * (ProjectionCalculator::calcNode) and the final BottomUp run on the host. */
typedef void (*mwh_func)(long long n, const double *r, double *values, void *user);
int mwh_project_func(double prec, mwh_tree *tree, mwh_func f, void *user, int max_iter, int abs_prec);
/* The same with the node computations on the device: per TreeBuilder
 * iteration f is evaluated on the host at every child quadrature point of the
 * level (mwgpu_project_level_values), the transforms, norms and the final
 * BottomUp run on the GPU. */
int mwh_project_func_device(double prec, mwh_tree *tree, mwh_func f, void *user, int max_iter, int abs_prec, mwh_apply_stats *stats);
/* add(prec, out, FunctionTreeVector, maxIter, absPrec) (src/treebuilders/add.cpp:58-83)
 * and multiply(prec, out, FunctionTreeVector, maxIter, absPrec) with the
 * wavelet adaptor (multiply.cpp:70-101): out = sum_j c[j] inps[j] or
 * prod_j c[j] inps[j], built adaptively from out's current grid; node
 * computations and BottomUp on the device (mwgpu_combine_level). */
int mwh_add(double prec, mwh_tree *out, int n, const double *c, mwh_tree *const *inps, int max_iter, int abs_prec, mwh_apply_stats *stats);
int mwh_multiply(double prec, mwh_tree *out, int n, const double *c, mwh_tree *const *inps, int max_iter, int abs_prec, mwh_apply_stats *stats);
/* multiply(..., useMaxNorms = true) (multiply.cpp:104-108): the grid is
 * refined by MultiplicationAdaptor (MultiplicationAdaptor.h:45-65) from the
 * two inputs' max norms (makeMaxSquareNorms); n must be 2. */
int mwh_multiply_max_norms(double prec, mwh_tree *out, int n, const double *c, mwh_tree *const *inps, int max_iter, mwh_apply_stats *stats);
int mwh_copy_grid(mwh_tree *out, const mwh_tree *inp);
/* FunctionTree::rescale(c) (src/trees/FunctionTree.cpp:651-668): every stored
 * coefficient times c, norms and square norm recomputed. */
int mwh_tree_rescale(mwh_tree *tree, double c);
/* node count (non-generated nodes) and tree square norm */
int mwh_tree_info(const mwh_tree *tree, int *n_nodes, double *square_norm);
/* flat copy: idx[4n], child0[n] (local numbering), coefs[n*8K^3], norms[n*8]; any may be NULL */
int mwh_tree_export(const mwh_tree *tree, int *idx, int *child0, double *coefs, double *norms);
/* replaces the tree with the given flat tree (same layout as export; roots first) */
int mwh_tree_import(mwh_tree *tree, int n, const int *idx, const int *child0, const double *coefs, double square_norm);
/* Tree files ("<file>.mwtree"): replaces FunctionTree::saveTree / loadTree
 * (src/trees/FunctionTree.cpp:378-435), which dump the node allocator's
 * chunks (layout-bound).  This format is flat and versioned: header (MRA:
 * basis, order, world box, max depth; square norm; node count), then node
 * indices, first-child indices and the compressed coefficients, parents
 * before children, little-endian.  load requires the tree's MRA to equal the
 * file's (as loadTree does) and replaces the tree's nodes. */
int mwh_tree_save(const mwh_tree *tree, const char *file);
int mwh_tree_load(mwh_tree *tree, const char *file);
double mwh_dot(const mwh_tree *a, const mwh_tree *b);
double mwh_evalf(const mwh_tree *tree, double x, double y, double z);
double mwh_integrate(const mwh_tree *tree);

int mwh_poisson(const mwh_mra *mra, double prec, mwh_oper **out);
int mwh_helmholtz(const mwh_mra *mra, double mu, double prec, mwh_oper **out);
/* ConvolutionOperator<3>(mra, kernel, prec) (src/operators/ConvolutionOperator.cpp:51-62):
 * the operator of the 1D Gaussian kernel sum_i coefs[i] exp(-exps[i] x^2)
 * (e.g. from mwh_poisson_kernel / mwh_helmholtz_kernel), kernel projected at
 * prec / 10, operator built at prec. */
int mwh_convolution(const mwh_mra *mra, int n, const double *exps, const double *coefs, double prec, mwh_oper **out);
/* ABGVOperator(mra, a, b) (src/operators/ABGVOperator.cpp:45-71): first
 * derivative; a = b = 0 center difference (band 0), a = b = 0.5 central
 * difference (band 1). */
int mwh_abgv(const mwh_mra *mra, double a, double b, mwh_oper **out);
void mwh_oper_free(mwh_oper *oper);
/* number of terms, total operator nodes, total (term, depth) rows */
int mwh_oper_info(const mwh_oper *oper, int *n_terms, int *n_nodes, int *n_rows);
/* flat node caches: depth[T], max_transl[rows], blocks[nodes*4K^2], norms[nodes*4],
 * kernel exponents/coefficients[T]; any may be NULL */
int mwh_oper_export(const mwh_oper *oper, int *depth, int *max_transl, double *blocks, double *norms, double *kexp, double *kcoef);
/* operator descriptor pointing into the operator's own arrays (valid while oper lives) */
int mwh_oper_desc(const mwh_oper *oper, mwgpu_oper_desc *desc);
/* kernel of PoissonKernel/HelmholtzKernel alone (no trees): returns the term count,
 * fills exps/coefs when non-NULL (cap entries) */
int mwh_poisson_kernel(double eps, double r_min, double r_max, int cap, double *exps, double *coefs);
int mwh_helmholtz_kernel(double mu, double eps, double r_min, double r_max, int cap, double *exps, double *coefs);

/* mrcpp::apply on the GPU: precision = MWGPU_PREC_FP64 or MWGPU_PREC_MIXED. */
int mwh_apply(double prec, mwh_tree *out, mwh_oper *oper, mwh_tree *inp, int max_iter, int abs_prec, int precision, mwh_apply_stats *stats);
/* Derivative operators from tabulated blocks: PHOperator(MRA, order)
 * (src/operators/PHOperator.cpp:40-68, Holoborodko's smoothing derivative,
 * order 1 or 2) and BSOperator(MRA, order) (BSOperator.cpp:40-68, B-spline
 * derivative, order 1, 2 or 3).  Their S_+1, S_0, S_-1 tables are read from
 * the reference's filter files <L|I>_ph_deriv_<order>.txt /
 * <L|I>_b-spline-deriv<order>.txt in filter_dir (NULL: the MWFILTERS_DIR
 * environment variable, as details::find_filters); mwh_deriv_tables takes the
 * three (k+1) x (k+1) tables directly (row-major, element (i, j) as the
 * calculators read it).  Apply with mwh_apply_derivative. */
int mwh_ph(const mwh_mra *mra, int order, const char *filter_dir, mwh_oper **out);
int mwh_bs(const mwh_mra *mra, int order, const char *filter_dir, mwh_oper **out);
int mwh_deriv_tables(const mwh_mra *mra, int order, const double *s_p1, const double *s_0, const double *s_m1, mwh_oper **out);
/* mrcpp::apply(prec, out, oper, inp, precTrees, maxIter, absPrec)
 * (src/treebuilders/apply.h:43, apply.cpp:214-251): the precision of output
 * node idx is scaled by precFac(idx) = 1 / max_i sqrt(getMaxSquareNorm) of the
 * node idx of precision tree i after makeMaxSquareNorms (MWTree.cpp:536-543;
 * the largest 2^(3n) |node|^2 over the node and its descendants), in the
 * screening threshold (mwgpu_apply_level_scaled) and in the split test
 * (WaveletAdaptor.h:51-54).  A node missing from a precision tree is generated
 * for its norm (the precision trees are not changed).  n_prec = 0 gives
 * precFac = 1, the plain apply. */
int mwh_apply_prec(double prec, mwh_tree *out, mwh_oper *oper, mwh_tree *inp, int n_prec, mwh_tree *const *prec_trees, int max_iter,
                   int abs_prec, int precision, mwh_apply_stats *stats);
/* The precision function of that form alone (the lambda of apply.cpp:222-229):
 * fac[j] = precFac of the node idx[4j..4j+3] = (n, l0, l1, l2). */
int mwh_prec_factors(int n_prec, mwh_tree *const *prec_trees, int n, const int *idx, double *fac);
/* apply(out, DerivativeOperator, inp, dir) (src/treebuilders/apply.cpp:379-412):
 * out must hold only its root nodes; its grid becomes the input grid widened
 * by the operator band along dir (CopyAdaptor), the end nodes are computed on
 * the device (mwgpu_apply_derivative, FP64), then BottomUp. */
int mwh_apply_derivative(mwh_tree *out, mwh_oper *oper, mwh_tree *inp, int dir, mwh_apply_stats *stats);
/* n independent applies of one operator, outs[t] = oper(inps[t]) (the loop over
 * functions around mrcpp::apply, apply.h:41), advanced in lockstep: each
 * TreeBuilder iteration of all trees is one mwgpu_apply_level_batch call and
 * the transforms of all trees share their launches.  Every output equals the
 * one mwh_apply gives for its pair.  Trees must be distinct; stats are summed. */
int mwh_apply_batch(double prec, int n, mwh_tree **outs, mwh_oper *oper, mwh_tree **inps, int max_iter, int abs_prec, int precision,
                    mwh_apply_stats *stats);

/* Learned output grid (no reference counterpart): the network proposes the
 * output grid level by level (features + inference on the GPU; the first
 * full_levels levels are refined without asking it), then a
 * mwgpu_apply_judged pass computes and judges it with the split test.  When
 * the judge refines a node of level j that the proposal did not, levels 0..j
 * are kept, all children of the refined nodes of level j are added, the
 * network proposes below them and another judged pass continues from level
 * j+1 (fallback = 1, first_miss = j of the first pass).  The result equals
 * mwh_apply(prec, out, oper, inp, -1, abs_prec, precision).  `out` must be a
 * fresh tree (root nodes only), else the plain apply runs. */
typedef struct mwh_mlp mwh_mlp;
typedef struct {
    mwh_apply_stats apply;   /* of the judged pass (or of the plain fallback) */
    int proposal_nodes, proposal_levels, kept_nodes, first_miss, fallback, host_round_trips;
    double predict_ms, judged_ms;
} mwh_learned_stats;
int mwh_mlp_create(const float *params, mwh_mlp **out);
void mwh_mlp_free(mwh_mlp *mlp);
int mwh_apply_learned(double prec, mwh_tree *out, mwh_oper *oper, mwh_tree *inp, const mwh_mlp *mlp, double threshold, int full_levels,
                      int abs_prec, int precision, mwh_learned_stats *stats);
/* Training data: features (n*8) of every node of `grid` (e.g. the output of a
 * plain apply of oper on inp) in the order of the tree export (breadth first),
 * and labels (1 = the node has children).  n = number of nodes of grid. */
int mwh_grid_features(double prec, mwh_tree *grid, mwh_oper *oper, mwh_tree *inp, float *x, float *y);

#ifdef __cplusplus
}
#endif

#endif /* MWHOST_H */
