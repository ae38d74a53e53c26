/*
 * mwgpu.h -- C-ABI of the GB300 operator-application library.
 *
 * This is the boundary MRCPP's host code binds to.  The host keeps its
 * FunctionTree / OperatorTree objects (src/trees/FunctionTree.h,
 * src/trees/OperatorTree.h) and hands flat copies of them to the device:
 * operator node caches once per (operator, apply precision), the input tree
 * once per apply, and the output tree level by level.  The GPU side replaces
 * ConvolutionCalculator::calcNodeVector (src/treebuilders/TreeCalculator.h:39-50
 * via ConvolutionCalculator.cpp:224-382) and the two whole-tree transforms of
 * apply (src/treebuilders/apply.cpp:82-84).  Only D = 3, T = double is
 * accelerated.  There is no CPU fallback: every entry point needs a CUDA
 * device and returns MWGPU_ERR_NO_DEVICE without one.
 *
 * Conventions
 *   - plain pointers and sizes, host memory unless stated otherwise;
 *   - a node index is 4 ints (scale, l0, l1, l2) like mrcpp::NodeIndex<3>
 *     (src/trees/NodeIndex.h:39-97);
 *   - a node's coefficients are 8*(k+1)^3 doubles, component c (bit d set =
 *     wavelet in direction d) at c*(k+1)^3, x fastest inside a component, the
 *     layout of MWNode::coefs (src/trees/MWNode.h:183, FunctionNode.cpp:77-83);
 *   - an operator node is 4*(k+1)^2 doubles (T, C, B, A; each (k+1)x(k+1)
 *     column-major) plus 4 component norms, the layout of OperatorNode::coefs
 *     (src/trees/OperatorNode.cpp:96-104);
 *   - every call returns an mwgpu_status; MWGPU_OK = 0.  The reference aborts on
 *     errors (MSG_ABORT, src/utils/Printer.h:159-170); here the caller gets a
 *     code and mwgpu_last_error() gives the message.
 */
#ifndef MWGPU_H
#define MWGPU_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef int mwgpu_status;
#define MWGPU_OK 0
#define MWGPU_ERR_BAD_ARG 1
#define MWGPU_ERR_OOM 2
#define MWGPU_ERR_DEVICE 3
#define MWGPU_ERR_TIMEOUT 4
#define MWGPU_ERR_NO_DEVICE 5
#define MWGPU_ERR_INTERNAL 6

#define MWGPU_PREC_FP64 0  /* plain form: FP64 throughout */
#define MWGPU_PREC_MIXED 1 /* mixed form: FP32 contractions, FP64 accumulation */

#define MWGPU_TOPDOWN 0
#define MWGPU_BOTTOMUP 1

typedef struct mwgpu_ctx mwgpu_ctx;
typedef struct mwgpu_oper mwgpu_oper;
typedef struct mwgpu_tree mwgpu_tree;

typedef struct {
    int device;         /* CUDA device ordinal */
    int precision;      /* MWGPU_PREC_FP64 or MWGPU_PREC_MIXED */
    int reserved[6];
} mwgpu_config;

/* World box + basis: mrcpp::MultiResolutionAnalysis<3>
 * (src/trees/MultiResolutionAnalysis.h:59-65, BoundingBox.cpp:47-80). */
typedef struct {
    int order;          /* k; K = k+1 */
    int root_scale;
    int corner[3];
    int nbox[3];
    int max_scale;      /* root_scale + max depth */
    double sf;          /* uniform scaling factor */
    /* 8 (k+1)x(k+1) column-major filters: compression H0t,H1t,G0t,G1t then
     * reconstruction H0,G0,H1,G1 (MWFilter::getSubFilter, MWFilter.cpp:100-133) */
    const double *filters;
} mwgpu_mra_desc;

/* Operator node caches of a ConvolutionOperator<3> (MWOperator::oper_exp,
 * isotropic; OperatorTree::setupOperNodeCache, OperatorTree.cpp:200-238).
 * For term t and depth d < depth[t] the nodes for l = -L..L, L =
 * max_transl[sum(depth[0..t-1]) + d], are stored consecutively. */
typedef struct {
    int n_terms;
    int order;
    const int *depth;        /* [n_terms] number of operator scales per term */
    const int *max_transl;   /* [sum depth] */
    const double *blocks;    /* [nodes * 4 * K*K] */
    const double *norms;     /* [nodes * 4], OperatorNode::calcComponentNorm */
    double build_prec;       /* norm precision of the operator trees */
} mwgpu_oper_desc;

/* Flat FunctionTree<3>.  child0[i] = index of the first of the 8 contiguous
 * children of node i, or -1 for a leaf. */
typedef struct {
    int n_nodes;
    const int *idx;          /* [n_nodes * 4] */
    const int *child0;       /* [n_nodes] */
    const double *coefs;     /* [n_nodes * 8K^3] or NULL (zeros) */
    const double *norms;     /* [n_nodes * 8] or NULL (computed on the device) */
} mwgpu_tree_desc;

/* Counters of one level (OperatorStatistics, OperatorStatistics.cpp:84-105). */
typedef struct {
    unsigned long long node_terms;   /* (g, f, term) triples with >= 1 contracted component */
    unsigned long long components;   /* contracted (g, f, term, ft, gt) component products */
    unsigned long long band_nodes;   /* (g, f) pairs inside the operator band */
    unsigned long long gen_nodes;    /* input GenNodes created */
    double device_ms;                /* device time of the level (CUDA events) */
    double contract_ms;              /* device time of the contraction kernel */
} mwgpu_level_stats;

/* Context on one device.  Replaces nothing in the reference (MRCPP has no
 * device state); owns the stream and scratch buffers. */
mwgpu_status mwgpu_init(mwgpu_ctx **ctx, const mwgpu_config *cfg);
mwgpu_status mwgpu_destroy(mwgpu_ctx *ctx);
/* Message of the last failed call on this context (or of the last failed
 * mwgpu_init when ctx is NULL). */
const char *mwgpu_last_error(const mwgpu_ctx *ctx);
mwgpu_status mwgpu_set_precision(mwgpu_ctx *ctx, int precision);

/* Uploads the operator node caches and derives, for apply precision `prec`,
 * the band widths (MWOperator::calcBandWidths, MWOperator.cpp:78-108 and
 * OperatorTree::calcBandWidth, OperatorTree.cpp:109-134) and the band-size
 * factors (ConvolutionCalculator::initBandSizes, ConvolutionCalculator.cpp:105-139).
 * prec < 0 uses build_prec. */
mwgpu_status mwgpu_upload_operator(mwgpu_ctx *ctx, const mwgpu_mra_desc *mra, const mwgpu_oper_desc *oper, double prec,
                                   mwgpu_oper **out);
mwgpu_status mwgpu_free_operator(mwgpu_ctx *ctx, mwgpu_oper *oper);
/* Band widths at the uploaded precision: widths[t * (rows) * 5 + d * 5 + c]
 * (c = T,C,B,A,max), rows = *n_rows, and band_max[rows]. Either pointer may be
 * NULL to query n_rows only. */
mwgpu_status mwgpu_operator_bandwidths(mwgpu_ctx *ctx, const mwgpu_oper *oper, int *n_rows, int *widths, int *band_max);

/* Input tree (the `inp` of apply, compressed s+d form, all nodes).  GenNodes
 * the operator band needs are created on the device from these nodes, like
 * MWTree::getNode (MWTree.cpp:340-352); the host never sees them, matching
 * inp.deleteGenerated() at the end of apply (apply.cpp:86-87).  The host
 * arrays may be pageable or page-locked (page-locked ones copy as DMA); either
 * way they are read in full before the call returns, as in create_tree,
 * tree_update_coefs, download_tree and download_nodes. */
mwgpu_status mwgpu_upload_tree(mwgpu_ctx *ctx, const mwgpu_mra_desc *mra, const mwgpu_tree_desc *tree, mwgpu_tree **out);
/* Output tree with the given topology and zero coefficients. */
mwgpu_status mwgpu_create_tree(mwgpu_ctx *ctx, const mwgpu_mra_desc *mra, const mwgpu_tree_desc *tree, mwgpu_tree **out);
/* Appends nodes (e.g. the children made by TreeAdaptor::splitNodeVector,
 * TreeAdaptor.h:41-52) and sets child0 of their parents. The new nodes get
 * indices n_nodes .. n_nodes+n-1 in order. */
mwgpu_status mwgpu_tree_add_nodes(mwgpu_ctx *ctx, mwgpu_tree *tree, int n, const int *idx, int n_parents, const int *parent_ids,
                                  const int *parent_child0);
mwgpu_status mwgpu_tree_size(const mwgpu_tree *tree, int *n_nodes);
mwgpu_status mwgpu_free_tree(mwgpu_ctx *ctx, mwgpu_tree *tree);

/* One TreeBuilder iteration of apply: computes the nodes out[node_ix[0..n)]
 * (ConvolutionCalculator::calcNode for each, ConvolutionCalculator.cpp:224-274)
 * with the screening threshold that calcNode derives from out_sqnorm
 * (:241-248; out_sqnorm <= 0 disables norm screening exactly like the
 * reference).  Coefficients stay on the device; norms_out (n*8 doubles, may be
 * NULL) receives the component norms the split test needs. */
mwgpu_status mwgpu_apply_level(mwgpu_ctx *ctx, const mwgpu_oper *oper, mwgpu_tree *inp, mwgpu_tree *out, const int *node_ix, int n,
                               double prec, double out_sqnorm, double *norms_out, mwgpu_level_stats *stats);
/* mwgpu_apply_level with the precision scaled per output node: the
 * calculator's precision function (ConvolutionCalculator::setPrecFunction,
 * ConvolutionCalculator.h:43, set by the precTrees form of apply,
 * apply.cpp:214-251) evaluated by the caller, prec_fac[i] for node node_ix[i].
 * Node i is screened with gThreshold = prec * prec_fac[i] *
 * sqrt(out_sqnorm / nTerms) (ConvolutionCalculator.cpp:244-245).  Factors
 * must be >= 0 (+inf allowed: a node whose precision trees are zero there
 * keeps no component); else MWGPU_ERR_BAD_ARG before any device work. */
mwgpu_status mwgpu_apply_level_scaled(mwgpu_ctx *ctx, const mwgpu_oper *oper, mwgpu_tree *inp, mwgpu_tree *out, const int *node_ix, int n,
                                      double prec, double out_sqnorm, const double *prec_fac, double *norms_out, mwgpu_level_stats *stats);

/* Whole-tree transform of the output tree: MWGPU_TOPDOWN with overwrite = 0
 * adds the coarse-scale contributions downwards (MWTree::mwTransformDown,
 * MWTree.cpp:194-216); MWGPU_BOTTOMUP recompresses (MWTree::mwTransformUp,
 * MWTree.cpp:166-181). */
mwgpu_status mwgpu_transform(mwgpu_ctx *ctx, mwgpu_tree *tree, int direction, int overwrite);

/* Sum / product level: replaces AdditionCalculator::calcNode
 * (src/treebuilders/AdditionCalculator.h:42-66) or MultiplicationCalculator::calcNode
 * (MultiplicationCalculator.h:42-72) for the nodes node_ix[0..n) of `out`:
 * out = sum_j c[j] inps[j] (compressed coefficients) or the pointwise product
 * prod_j c[j] inps[j] at the children's quadrature points (reconstruction,
 * cvTransform with the basis's cv_map / vc_map (K x K, column-major),
 * compression).  Missing input nodes become GenNodes (getNode).  FP64; node
 * norms to norms_out (8 per node, optional).  The caller's TreeBuilder loop
 * does the split test and the final BottomUp (add.cpp, multiply.cpp). */
#define MWGPU_COMBINE_ADD 0
#define MWGPU_COMBINE_MULTIPLY 1
mwgpu_status mwgpu_combine_level(mwgpu_ctx *ctx, int op, int n_in, mwgpu_tree *const *inps, const double *c, const double *cv_map, const double *vc_map,
                                 mwgpu_tree *out, const int *node_ix, int n, double *norms_out);

/* Projection level: replaces ProjectionCalculator::calcNode
 * (src/treebuilders/ProjectionCalculator.cpp:34-51) for the nodes
 * node_ix[0..n) of `tree` (an output tree), for a sum of Gaussians
 * gauss[j] = {coefficient, exponent, x, y, z}: values at the children's
 * quadrature points, cvTransform(Backward) with the basis's value-to-coefficient
 * map vc_map (K x K, column-major) and quadrature roots (K, on [0, 1]),
 * compression, node norms (norms_out: 8 per node, optional).  FP64.  The
 * caller's TreeBuilder loop does the split test and the final BottomUp
 * (project.cpp:47-66). */
mwgpu_status mwgpu_project_level(mwgpu_ctx *ctx, mwgpu_tree *tree, int n_gauss, const double *gauss, const double *vc_map, const double *roots,
                                 const int *node_ix, int n, double *norms_out);
/* The same level for any function the caller can evaluate (the
 * RepresentableFunction of ProjectionCalculator, ProjectionCalculator.cpp:
 * 40-43, lives on the host): values[8 (k+1)^3 j + (k+1)^3 ct + qx + (k+1) qy
 * + (k+1)^2 qz] = f at the point of child ct of node node_ix[j], coordinate d
 * = sf 2^-(n+1) (root[q_d] + 2 l_d + bit_d(ct)) (MWNode::getExpandedChildPts,
 * MWNode.cpp:854-935). */
mwgpu_status mwgpu_project_level_values(mwgpu_ctx *ctx, mwgpu_tree *tree, const double *values, const double *vc_map, const double *roots,
                                        const int *node_ix, int n, double *norms_out);

/* Derivative level: replaces DerivativeCalculator::calcNodeVector
 * (src/treebuilders/DerivativeCalculator.cpp:113-151) for the output end nodes
 * node_ix[0..n) of `out` (a grid made by CopyAdaptor, CopyAdaptor.cpp:55-71):
 * per node the input nodes within the operator band along `dir` (GenNodes made
 * as needed), the 1D application of the one-term derivative operator along dir
 * with the identity in the other directions, division by sf^order, node norms.
 * FP64 in every precision mode.  The caller then runs the BottomUp transform
 * (apply.cpp:379-412). */
mwgpu_status mwgpu_apply_derivative(mwgpu_ctx *ctx, const mwgpu_oper *oper, mwgpu_tree *inp, mwgpu_tree *out, const int *node_ix, int n, int dir,
                                    int order, mwgpu_level_stats *stats);

/* Batched level: one TreeBuilder iteration of n_trees independent applies of
 * the same operator (the loop over functions that calls mrcpp::apply once per
 * function, apply.cpp:68-93), computed by one work list and one contraction
 * launch.  Entry i computes node node_ix[i] of outs[work_tree[i]] from
 * inps[work_tree[i]] with the screening threshold of out_sqnorms[work_tree[i]];
 * norms_out (n*8, may be NULL) is in entry order.  Input and output trees of a
 * batch must be distinct.  Results equal n_trees calls of mwgpu_apply_level. */
mwgpu_status mwgpu_apply_level_batch(mwgpu_ctx *ctx, const mwgpu_oper *oper, int n_trees, mwgpu_tree *const *inps, mwgpu_tree *const *outs,
                                     const int *work_tree, const int *node_ix, int n, double prec, const double *out_sqnorms,
                                     double *norms_out, mwgpu_level_stats *stats);
/* mwgpu_transform of several distinct trees with the same MRA, one launch per
 * depth for all of them. */
mwgpu_status mwgpu_transform_batch(mwgpu_ctx *ctx, int n_trees, mwgpu_tree *const *trees, int direction, int overwrite);

/* Level plans.  No counterpart in the reference (each mrcpp::apply rebuilds
 * its bands, apply.cpp:68-93).  For levels whose node lists stay fixed: apply
 * with maxIter = 0 onto given output grids (the fixed-grid apply of
 * apply.cpp:68-93 with copy_grid), over one or many functions, possibly
 * repeated as input values change (a fixed-grid SCF loop).
 *
 * mwgpu_plan_create computes the level once (same arguments and results as
 * mwgpu_apply_level_batch, in the context precision) and keeps what depends
 * only on the topology: the input trees' GenNode keys and slots (earlier
 * GenNodes of the input trees are dropped first), the band pair offsets,
 * buffer capacities (work list: 1.25x the planned size) and, with
 * MWGPU_PLAN_AUTOTUNE, the schedule of the contraction (for order 7 on
 * levels without norm screening: pencil and item kernels, or the item
 * kernel alone) and the chunk length of the persistent item kernel, chosen
 * by timing every combination on the whole contraction of this level.  The level is then captured as
 * one CUDA graph: GenNode values from the current input coefficients,
 * screening and work list, contraction (one persistent launch for all trees),
 * chunk reduction and norms, and with MWGPU_PLAN_TRANSFORMS the TopDown(add)
 * and BottomUp transforms of all output trees (the node list must then hold
 * every node of every output tree once).
 *
 * mwgpu_plan_execute replays the graph on the context stream.  With stats it
 * waits and returns them (and the device status); without, it returns at once
 * and mwgpu_plan_check later waits and reports.  While a plan exists its trees
 * may not be changed structurally: level calls, mwgpu_tree_add_nodes,
 * mwgpu_tree_clear_generated and mwgpu_free_tree on them return
 * MWGPU_ERR_BAD_ARG.  New input coefficients for the same topology go in with
 * mwgpu_tree_update_coefs.  If they change the screening so much that the work
 * list outgrows its capacity, execute/check return MWGPU_ERR_OOM: create a new
 * plan. */
typedef struct mwgpu_plan mwgpu_plan;
#define MWGPU_PLAN_TRANSFORMS 1
#define MWGPU_PLAN_AUTOTUNE 2
mwgpu_status mwgpu_plan_create(mwgpu_ctx *ctx, const mwgpu_oper *oper, int n_trees, mwgpu_tree *const *inps, mwgpu_tree *const *outs,
                               const int *work_tree, const int *node_ix, int n, double prec, const double *out_sqnorms, int flags,
                               mwgpu_plan **plan);
mwgpu_status mwgpu_plan_execute(mwgpu_ctx *ctx, mwgpu_plan *plan, mwgpu_level_stats *stats);
mwgpu_status mwgpu_plan_check(mwgpu_ctx *ctx, mwgpu_plan *plan, mwgpu_level_stats *stats);
/* Pencil contraction of the last checked execution of a plan (mwgpu_plan_check):
 * the node-terms it computed (those of the operator terms of band width <= 4,
 * on levels without norm screening) and its device time in ms; 0 and 0 when the
 * plan does not use it.  No reference counterpart (a measurement of the GPU
 * schedule of calcNodeVector, ConvolutionCalculator.cpp:224-382). */
mwgpu_status mwgpu_plan_pencil_info(const mwgpu_plan *plan, unsigned long long *node_terms, double *ms);

/* Chunk length and persistent grid in use, the timed candidates (n_candidates:
 * in = room in the arrays, out = number tried) and kernel launches per execution. */
mwgpu_status mwgpu_plan_info(const mwgpu_plan *plan, long long *chunk_items, int *grid, int *n_candidates, long long *cand_items,
                             double *cand_ms, unsigned long long *launches);
/* The autotuning candidates of a plan: per candidate the chunk length, the
 * schedule (1: pencil kernel with 8 consumer warps per CTA + item kernel,
 * 2: the same with 16 consumer warps, 0: item kernel alone) and the time of
 * the contraction in ms; chosen = the index in use (-1 without autotuning).
 * n_candidates: in = room in the arrays (any may be NULL), out = number tried. */
mwgpu_status mwgpu_plan_tuning(const mwgpu_plan *plan, int *n_candidates, long long *chunk_items, int *schedule, double *ms, int *chosen);

/* Peak FP64 rates of this GPU in TFLOP/s, measured with CUDA events: chains of
 * independent DFMA per thread, and of mma.sync m8n8k4 f64 (DMMA) per warp, 4
 * CTAs of 256 threads per SM.  No reference counterpart: the measurement
 * behind the FP64 form's choice of pipe (it runs on DFMA). */
mwgpu_status mwgpu_fp64_pipe_rates(mwgpu_ctx *ctx, double *dfma_tflops, double *dmma_tflops);
mwgpu_status mwgpu_plan_destroy(mwgpu_ctx *ctx, mwgpu_plan *plan);
/* New coefficients (and norms, or NULL to compute them) of all nodes of an
 * input tree with unchanged topology; refreshes the FP32 copy.  GenNodes are
 * recomputed by the next level call or plan execution. */
mwgpu_status mwgpu_tree_update_coefs(mwgpu_ctx *ctx, mwgpu_tree *tree, const double *coefs, const double *norms);

/* Copies coefficients and/or norms of all real nodes back (either may be NULL). */
mwgpu_status mwgpu_download_tree(mwgpu_ctx *ctx, const mwgpu_tree *tree, double *coefs, double *norms);
/* Copies coefficients and/or norms of the real nodes ids[0..n) back, node
 * ids[j] to row j (gathered on the device: one transfer of n rows). */
mwgpu_status mwgpu_download_nodes(mwgpu_ctx *ctx, const mwgpu_tree *tree, int n, const int *ids, double *coefs, double *norms);

/* Synchronises the context stream; returns device errors. */
mwgpu_status mwgpu_sync(mwgpu_ctx *ctx);

/* Drops the GenNodes made by earlier mwgpu_apply_level calls on an input tree
 * (FunctionTree::deleteGenerated, called by apply at apply.cpp:86-87). */
mwgpu_status mwgpu_tree_clear_generated(mwgpu_ctx *ctx, mwgpu_tree *tree);

/* Device timers: records CUDA event `slot` (0..15) on the context stream;
 * elapsed time between two recorded slots. No reference counterpart (MRCPP's
 * Timer, src/utils/Timer.h:40-58, is host-only). */
mwgpu_status mwgpu_timer_mark(mwgpu_ctx *ctx, int slot);
mwgpu_status mwgpu_timer_elapsed(mwgpu_ctx *ctx, int slot0, int slot1, double *ms);
/* Number of kernels this context has launched so far. */
mwgpu_status mwgpu_launch_count(const mwgpu_ctx *ctx, unsigned long long *count);
/* Writes `bytes` of device scratch on the context stream (evicts L2 between
 * timed repetitions). */
mwgpu_status mwgpu_scrub_l2(mwgpu_ctx *ctx, size_t bytes);

/* Learned output grid.  No counterpart in the reference.  A 3-layer, 64-wide
 * network (BF16 weights, FP32 arithmetic) that predicts for an output node of
 * apply whether the wavelet-norm split test (tree_utils::split_check,
 * tree_utils.cpp:47-65) will refine it; mwgpu_apply_judged runs the split test
 * itself, so the prediction changes how many host round trips the apply
 * needs, never its result.
 * Parameters: MWGPU_MLP_PARAMS floats, W1[64][8], b1[64], W2[64][64], b2[64],
 * W3[64], b3 (W[out][in], row-major).  Features: MWGPU_MLP_FEATURES floats per
 * node (depth/16; log10 of the input's wavelet norm at the node relative to
 * f_norm /8; log10 of the input norm summed over the operator band box /8;
 * operator terms reaching the depth /100; translation parities; 1 / 0.5 / 0
 * if the input has a branch node / a leaf / no node there). */
typedef struct mwgpu_mlp mwgpu_mlp;
#define MWGPU_MLP_FEATURES 8
#define MWGPU_MLP_PARAMS 4801
mwgpu_status mwgpu_mlp_create(mwgpu_ctx *ctx, const float *params, mwgpu_mlp **mlp);
mwgpu_status mwgpu_mlp_destroy(mwgpu_ctx *ctx, mwgpu_mlp *mlp);
/* FP32 master parameters and/or their BF16 copy (either may be NULL). */
mwgpu_status mwgpu_mlp_get(mwgpu_ctx *ctx, const mwgpu_mlp *mlp, float *params, uint16_t *bf16);
/* Features of n nodes (idx: n*4 ints) against input tree inp; x: n*8 floats. */
mwgpu_status mwgpu_mlp_features(mwgpu_ctx *ctx, const mwgpu_oper *oper, const mwgpu_tree *inp, double f_norm, const int *idx, int n,
                                float *x);
/* Features + inference in one call (device buffers kept in the network):
 * P(split) of n nodes (idx: n*4 ints) against input tree inp. */
mwgpu_status mwgpu_mlp_predict(mwgpu_ctx *ctx, mwgpu_mlp *mlp, const mwgpu_oper *oper, const mwgpu_tree *inp, double f_norm, const int *idx,
                               int n, float *prob);
/* P(split) of n feature rows. */
mwgpu_status mwgpu_mlp_infer(mwgpu_ctx *ctx, const mwgpu_mlp *mlp, const float *x, int n, float *prob);
/* Gradient (MWGPU_MLP_PARAMS floats) and value of the weighted binary cross
 * entropy over n samples (labels 0/1, weight pos_weight for label 1). */
mwgpu_status mwgpu_mlp_grad(mwgpu_ctx *ctx, const mwgpu_mlp *mlp, const float *x, const float *y, int n, float pos_weight, float *grad,
                            float *loss);
/* Adam training on the device: `epochs` passes over the n samples in seeded
 * random order, mini-batches of `batch`; epoch_loss (may be NULL) gets the
 * mean batch loss of every epoch. */
mwgpu_status mwgpu_mlp_train(mwgpu_ctx *ctx, mwgpu_mlp *mlp, const float *x, const float *y, int n, int epochs, int batch, float lr,
                             float pos_weight, unsigned seed, float *epoch_loss);

/* Adaptive apply over a proposed output grid, judged on the device.  No
 * counterpart in the reference; it runs the TreeBuilder loop of apply
 * (TreeBuilder.cpp:38-87 with WaveletAdaptor, tree_utils.cpp:47-65) for all
 * levels without returning to the host.  `out` holds the proposal: level 0 =
 * the root nodes of a fresh output tree, every proposed split has its 8
 * children (child0) in the next level, and the nodes are ordered by level,
 * each level in the order of its parents (the order TreeBuilder creates
 * nodes): nodes level_begin[j] .. level_begin[j+1]-1 form level j.
 * Level j computes the nodes the split test kept (the nodes of first_level,
 * then the children of refined nodes) with the screening threshold of the tree
 * norm of the levels before, adds their norms to the tree norm in
 * TreeBuilder's order and judges them with split_check (prec, abs_prec,
 * splitFac 1).  Levels before first_level are a judged tree computed earlier
 * (their coefficients already in `out`; refined = has children); state_in =
 * TreeBuilder's sNorm, wNorm and tree norm after them ({0, 0, out's tree norm}
 * for first_level 0).  flags_out[i]: bit 0 = node of the judged tree, bit 1 =
 * refined.  first_miss = the first level where a refined node had no proposed
 * children (-1: none); the result is then exact up to that level only.  With
 * `transforms` and no miss, TopDown(add) and BottomUp run over the judged
 * tree.  norm_levels (3*n_levels, may be NULL) gets sNorm, wNorm and the tree
 * norm after each computed level (to continue after a miss).  Equal to
 * mwgpu_apply_level driven by the host TreeBuilder on the judged tree
 * whenever first_miss is -1. */
mwgpu_status mwgpu_apply_judged(mwgpu_ctx *ctx, const mwgpu_oper *oper, mwgpu_tree *inp, mwgpu_tree *out, int n_levels,
                                const int *level_begin, double prec, int abs_prec, int first_level, const double *state_in, int transforms,
                                int *flags_out, int *first_miss, double *norm_levels, mwgpu_level_stats *stats);
/* Copies coefficients and norms of nodes src_ids[j] of src to dst_ids[j] of dst. */
mwgpu_status mwgpu_tree_copy_nodes(mwgpu_ctx *ctx, const mwgpu_tree *src, mwgpu_tree *dst, int n, const int *src_ids, const int *dst_ids);

/* Allocation-free variant of mwgpu_apply_level.  No counterpart in the
 * reference (MRCPP allocates on the host as it goes).  For callers that must
 * not allocate device memory while a level runs -- code inside a framework
 * whose caching allocator owns the device memory, or a latency-critical loop
 * where cudaMalloc/cudaFree would synchronise the device.  Its work list,
 * error flag, counters and norm staging live in a fixed 4.5 MiB device array
 * that every GPU loading the library holds until exit; it calls no cudaMalloc,
 * cudaFree or other allocating routine.
 *   - FP64 form only (the context precision must be MWGPU_PREC_FP64);
 *   - n <= 65536 nodes, else MWGPU_ERR_BAD_ARG;
 *   - it creates no GenNodes: every node of the operator bands must already be
 *     in the input tree (run mwgpu_apply_level once on the same nodes first,
 *     in the FP64 form: GenNodes made by the mixed form are rejected), else
 *     MWGPU_ERR_BAD_ARG; when a band node turns out to be missing during the
 *     contraction the call returns MWGPU_ERR_BAD_ARG after the kernel has
 *     run, and the listed output nodes are then undefined;
 *   - trees held by a plan are rejected (MWGPU_ERR_BAD_ARG);
 *   - the first call on a device looks up the array's device address; make
 *     that first call before any stream capture;
 *   - all calls share the one array: calls that overlap on the GPU (other host
 *     threads, other contexts on the same device) race.  Each call clears the
 *     counters and the error flag it uses before its kernels run.
 * Same arguments and results as mwgpu_apply_level otherwise. */
mwgpu_status mwgpu_apply_level_static(mwgpu_ctx *ctx, const mwgpu_oper *oper, const mwgpu_tree *inp, mwgpu_tree *out,
                                      const int *node_ix, int n, double prec, double out_sqnorm, double *norms_out,
                                      mwgpu_level_stats *stats);

#ifdef __cplusplus
}
#endif

#endif /* MWGPU_H */
