/*
 * CPU oracle for mrcpp::apply (test infrastructure only; see oracle_apply.c).
 */
#ifndef ORACLE_APPLY_H
#define ORACLE_APPLY_H

#ifdef __cplusplus
extern "C" {
#endif

typedef struct {
    int order;          /* k */
    int root_scale;
    int corner[3];
    int nbox[3];
    int max_scale;
    double sf;
    /* 8 (k+1)^2 column-major filters: compression H0t,H1t,G0t,G1t, reconstruction H0,G0,H1,G1 */
    const double *filters;
} oracle_mra;

typedef struct {
    int n_terms;
    int order;
    const int *depth;      /* [n_terms] operator scales per term */
    const int *max_transl; /* [sum depth] */
    const double *blocks;  /* per node 4 (k+1)^2, nodes l = -L..L per (term, depth) */
    const double *norms;   /* per node 4 */
    double build_prec;
} oracle_oper;

typedef struct {
    int n_nodes;
    const int *idx;        /* [n*4] scale, l0, l1, l2; roots first, parents before children */
    const int *child0;     /* [n] */
    const double *coefs;   /* [n*8K^3] (input tree) */
    const double *norms;   /* [n*8] (input tree) */
} oracle_tree;

typedef struct oracle_result oracle_result;

/* apply(prec, out, oper, inp, max_iter, abs_prec) starting from the topology out0
 * whose square norm is out_sqnorm (-1 for a fresh or copied grid). */
int oracle_apply(const oracle_mra *mra, const oracle_oper *oper, const oracle_tree *inp, const oracle_tree *out0, double out_sqnorm,
                 double prec, int max_iter, int abs_prec, int nthreads, int count_terms, oracle_result **res);
int oracle_apply_sampled(const oracle_mra *mra, const oracle_oper *oper, const oracle_tree *inp, const oracle_tree *out0, double out_sqnorm,
                         double prec, int max_iter, int abs_prec, int nthreads, int count_terms, int sample, oracle_result **res);
/* apply(out, DerivativeOperator, inp, dir): out0 holds the output roots; the
 * grid is copy-adapted from inp along dir, end nodes computed, then BottomUp. */
/* the precTrees form of apply (apply.cpp:214-251): n_prec precision trees
 * (coefficients and norms); n_prec = 0 is oracle_apply_sampled */
int oracle_apply_prec(const oracle_mra *mra, const oracle_oper *oper, const oracle_tree *inp, const oracle_tree *out0, double out_sqnorm,
                      double prec, int max_iter, int abs_prec, int nthreads, int count_terms, int sample, int n_prec,
                      const oracle_tree *prec_trees, oracle_result **res);
/* project(prec, out0's grid, f): f(n, r[3 n], v[n], user) evaluates the function */
typedef void (*oracle_func)(long long n, const double *r, double *v, void *user);
int oracle_project(const oracle_mra *mra, const double *vc_map, const double *roots, const oracle_tree *out0, double prec, int max_iter,
                   int abs_prec, oracle_func f, void *user, oracle_result **res);
int oracle_apply_derivative(const oracle_mra *mra, const oracle_oper *oper, const oracle_tree *inp, const oracle_tree *out0, int dir, int order,
                            int nthreads, oracle_result **res);
/* add (op 0) / multiply (op 1): out = sum / product of c[j] inps[j], adaptive
 * from out0's end nodes at prec; cv_map / vc_map the basis's value maps. */
int oracle_combine(const oracle_mra *mra, int op, int n_in, const oracle_tree *inps, const double *c, const double *cv_map, const double *vc_map,
                   const oracle_tree *out0, double prec, int max_iter, int abs_prec, oracle_result **res);
/* use_max_norms = 1: multiply of two functions with the max-norm adaptor */
int oracle_combine_ex(const oracle_mra *mra, int op, int n_in, const oracle_tree *inps, const double *c, const double *cv_map,
                      const double *vc_map, const oracle_tree *out0, double prec, int max_iter, int abs_prec, int use_max_norms,
                      oracle_result **res);
int oracle_result_info(const oracle_result *r, int *n_nodes, double *square_norm, unsigned long long *node_terms,
                       unsigned long long *components, int *iterations);
int oracle_result_export(const oracle_result *r, int *idx, int *child0, double *coefs, double *norms);
void oracle_result_free(oracle_result *r);

#ifdef __cplusplus
}
#endif

#endif
