// C-ABI of the learned output-grid network (include/mwgpu.h, mwgpu_mlp_*):
// parameters on the device, node features, inference, gradients and Adam
// training with the kernels of k_mlp.cu.
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <random>
#include <vector>

#include "abi_state.cuh"

using namespace mwgpu;

struct mwgpu_mlp {
    float *master = nullptr;          // FP32 parameters
    float *m1 = nullptr, *m2 = nullptr;  // Adam moments
    __nv_bfloat16 *wb = nullptr;      // BF16 copy used by the forward passes
    long long steps = 0;              // Adam steps taken
    // buffers of mwgpu_mlp_predict, grown as needed
    int4 *p_nodes = nullptr;
    float *p_x = nullptr, *p_prob = nullptr;
    int p_cap = 0;
    int *p_tab = nullptr;  // band widths and term counts per depth
    int p_rows = 0;
};

namespace {

// scratch of one call: features / labels / permutation / gradient partials
struct MlpScratch {
    float *x = nullptr, *y = nullptr, *prob = nullptr, *partial = nullptr, *loss_partial = nullptr, *grad = nullptr, *loss = nullptr;
    int *perm = nullptr;
    int4 *nodes = nullptr;
    int *band_w = nullptr, *terms = nullptr;
    std::vector<void *> all;
    ~MlpScratch() {
        for (void *p : all) cudaFree(p);
    }
};

template <class T> mwgpu_status scratch(mwgpu_ctx *ctx, MlpScratch &s, T **p, size_t n) {
    if (auto st = dev_alloc(ctx, p, n)) return st;
    s.all.push_back((void *)*p);
    return MWGPU_OK;
}

constexpr int kTile = 128;

}  // namespace

extern "C" {

mwgpu_status mwgpu_mlp_create(mwgpu_ctx *ctx, const float *params, mwgpu_mlp **out) {
    if (!ctx || !params || !out) return MWGPU_ERR_BAD_ARG;
    cudaSetDevice(ctx->device);
    auto *m = new mwgpu_mlp();
    mwgpu_status s;
    if ((s = dev_alloc(ctx, &m->master, kMlpParams)) || (s = dev_alloc(ctx, &m->m1, kMlpParams)) || (s = dev_alloc(ctx, &m->m2, kMlpParams)) ||
        (s = dev_alloc(ctx, &m->wb, kMlpParams))) {
        mwgpu_mlp_destroy(ctx, m);
        return s;
    }
    MW_CK(cudaMemcpyAsync(m->master, params, sizeof(float) * kMlpParams, cudaMemcpyHostToDevice, ctx->stream));
    MW_CK(cudaMemsetAsync(m->m1, 0, sizeof(float) * kMlpParams, ctx->stream));
    MW_CK(cudaMemsetAsync(m->m2, 0, sizeof(float) * kMlpParams, ctx->stream));
    launch_mlp_to_bf16(m->master, m->wb, kMlpParams, ctx->stream);
    ctx->launches++;
    MW_CK(cudaGetLastError());
    MW_CK(cudaStreamSynchronize(ctx->stream));
    *out = m;
    return MWGPU_OK;
}

mwgpu_status mwgpu_mlp_destroy(mwgpu_ctx *ctx, mwgpu_mlp *m) {
    if (!ctx) return MWGPU_ERR_BAD_ARG;
    if (!m) return MWGPU_OK;
    cudaSetDevice(ctx->device);
    cudaStreamSynchronize(ctx->stream);
    for (void *p : {(void *)m->master, (void *)m->m1, (void *)m->m2, (void *)m->wb, (void *)m->p_nodes, (void *)m->p_x, (void *)m->p_prob,
                    (void *)m->p_tab})
        if (p) cudaFree(p);
    delete m;
    return MWGPU_OK;
}

mwgpu_status mwgpu_mlp_get(mwgpu_ctx *ctx, const mwgpu_mlp *m, float *params, uint16_t *bf16) {
    if (!ctx || !m) return MWGPU_ERR_BAD_ARG;
    cudaSetDevice(ctx->device);
    if (params) MW_CK(cudaMemcpyAsync(params, m->master, sizeof(float) * kMlpParams, cudaMemcpyDeviceToHost, ctx->stream));
    if (bf16) MW_CK(cudaMemcpyAsync(bf16, m->wb, sizeof(uint16_t) * kMlpParams, cudaMemcpyDeviceToHost, ctx->stream));
    MW_CK(cudaStreamSynchronize(ctx->stream));
    return MWGPU_OK;
}

mwgpu_status mwgpu_mlp_features(mwgpu_ctx *ctx, const mwgpu_oper *o, const mwgpu_tree *inp, double f_norm, const int *idx, int n, float *x) {
    if (!ctx || !o || !inp || !x) return MWGPU_ERR_BAD_ARG;
    MW_ARG(n >= 0 && (n == 0 || idx), "invalid node list");
    MW_ARG(inp->is_input, "features are computed against an input tree");
    if (n == 0) return MWGPU_OK;
    cudaSetDevice(ctx->device);
    // per depth: band half width and the number of terms whose band reaches it
    const int rows = o->n_rows, T = o->op.n_terms;
    std::vector<int> bw(rows), terms(rows, 0);
    for (int d = 0; d < rows; d++) {
        bw[d] = o->band_max[d];
        for (int t = 0; t < T; t++) terms[d] += o->widths[((size_t)t * rows + d) * 5 + 4] >= 0;
    }
    std::vector<int4> nodes(n);
    for (int i = 0; i < n; i++) nodes[i] = make_int4(idx[4 * i], idx[4 * i + 1], idx[4 * i + 2], idx[4 * i + 3]);
    MlpScratch s;
    mwgpu_status st;
    if ((st = scratch(ctx, s, &s.nodes, n)) || (st = scratch(ctx, s, &s.band_w, rows)) || (st = scratch(ctx, s, &s.terms, rows)) ||
        (st = scratch(ctx, s, &s.x, (size_t)n * kMlpFeatures)))
        return st;
    MW_CK(cudaMemcpyAsync(s.nodes, nodes.data(), sizeof(int4) * n, cudaMemcpyHostToDevice, ctx->stream));
    MW_CK(cudaMemcpyAsync(s.band_w, bw.data(), sizeof(int) * rows, cudaMemcpyHostToDevice, ctx->stream));
    MW_CK(cudaMemcpyAsync(s.terms, terms.data(), sizeof(int) * rows, cudaMemcpyHostToDevice, ctx->stream));
    launch_mlp_features(inp->mra, inp->t, s.nodes, n, s.band_w, s.terms, rows, f_norm, s.x, ctx->stream);
    ctx->launches++;
    MW_CK(cudaGetLastError());
    MW_CK(cudaMemcpyAsync(x, s.x, sizeof(float) * n * kMlpFeatures, cudaMemcpyDeviceToHost, ctx->stream));
    MW_CK(cudaStreamSynchronize(ctx->stream));
    return MWGPU_OK;
}

mwgpu_status mwgpu_mlp_infer(mwgpu_ctx *ctx, const mwgpu_mlp *m, const float *x, int n, float *prob) {
    if (!ctx || !m || !prob) return MWGPU_ERR_BAD_ARG;
    MW_ARG(n >= 0 && (n == 0 || x), "invalid sample list");
    if (n == 0) return MWGPU_OK;
    cudaSetDevice(ctx->device);
    MlpScratch s;
    mwgpu_status st;
    if ((st = scratch(ctx, s, &s.x, (size_t)n * kMlpFeatures)) || (st = scratch(ctx, s, &s.prob, n))) return st;
    MW_CK(cudaMemcpyAsync(s.x, x, sizeof(float) * n * kMlpFeatures, cudaMemcpyHostToDevice, ctx->stream));
    launch_mlp_infer(s.x, n, m->wb, s.prob, ctx->stream);
    ctx->launches++;
    MW_CK(cudaGetLastError());
    MW_CK(cudaMemcpyAsync(prob, s.prob, sizeof(float) * n, cudaMemcpyDeviceToHost, ctx->stream));
    MW_CK(cudaStreamSynchronize(ctx->stream));
    return MWGPU_OK;
}

mwgpu_status mwgpu_mlp_grad(mwgpu_ctx *ctx, const mwgpu_mlp *m, const float *x, const float *y, int n, float pos_weight, float *grad,
                            float *loss) {
    if (!ctx || !m || !x || !y || !grad) return MWGPU_ERR_BAD_ARG;
    MW_ARG(n > 0, "empty batch");
    cudaSetDevice(ctx->device);
    double wsum = 0.0;
    for (int i = 0; i < n; i++) wsum += y[i] > 0.5f ? pos_weight : 1.0f;
    const int tiles = (n + kTile - 1) / kTile;
    MlpScratch s;
    mwgpu_status st;
    if ((st = scratch(ctx, s, &s.x, (size_t)n * kMlpFeatures)) || (st = scratch(ctx, s, &s.y, n)) ||
        (st = scratch(ctx, s, &s.partial, (size_t)tiles * kMlpParams)) || (st = scratch(ctx, s, &s.loss_partial, tiles)) ||
        (st = scratch(ctx, s, &s.grad, kMlpParams)) || (st = scratch(ctx, s, &s.loss, 1)))
        return st;
    MW_CK(cudaMemcpyAsync(s.x, x, sizeof(float) * n * kMlpFeatures, cudaMemcpyHostToDevice, ctx->stream));
    MW_CK(cudaMemcpyAsync(s.y, y, sizeof(float) * n, cudaMemcpyHostToDevice, ctx->stream));
    launch_mlp_train_tile(s.x, s.y, nullptr, 0, n, m->wb, pos_weight, (float)(1.0 / wsum), s.partial, s.loss_partial, ctx->stream);
    launch_mlp_reduce(s.partial, s.loss_partial, tiles, s.grad, s.loss, ctx->stream);
    ctx->launches += 2;
    MW_CK(cudaGetLastError());
    MW_CK(cudaMemcpyAsync(grad, s.grad, sizeof(float) * kMlpParams, cudaMemcpyDeviceToHost, ctx->stream));
    float l = 0.f;
    MW_CK(cudaMemcpyAsync(&l, s.loss, sizeof(float), cudaMemcpyDeviceToHost, ctx->stream));
    MW_CK(cudaStreamSynchronize(ctx->stream));
    if (loss) *loss = l;
    return MWGPU_OK;
}

mwgpu_status mwgpu_mlp_train(mwgpu_ctx *ctx, mwgpu_mlp *m, const float *x, const float *y, int n, int epochs, int batch, float lr,
                             float pos_weight, unsigned seed, float *epoch_loss) {
    if (!ctx || !m || !x || !y) return MWGPU_ERR_BAD_ARG;
    MW_ARG(n > 0 && epochs >= 0 && batch > 0, "invalid training arguments");
    cudaSetDevice(ctx->device);
    const int tiles_max = (std::min(batch, n) + kTile - 1) / kTile;
    const int nbatch = (n + batch - 1) / batch;
    MlpScratch s;
    mwgpu_status st;
    if ((st = scratch(ctx, s, &s.x, (size_t)n * kMlpFeatures)) || (st = scratch(ctx, s, &s.y, n)) || (st = scratch(ctx, s, &s.perm, n)) ||
        (st = scratch(ctx, s, &s.partial, (size_t)tiles_max * kMlpParams)) || (st = scratch(ctx, s, &s.loss_partial, tiles_max)) ||
        (st = scratch(ctx, s, &s.grad, kMlpParams)) || (st = scratch(ctx, s, &s.loss, nbatch)))
        return st;
    MW_CK(cudaMemcpyAsync(s.x, x, sizeof(float) * n * kMlpFeatures, cudaMemcpyHostToDevice, ctx->stream));
    MW_CK(cudaMemcpyAsync(s.y, y, sizeof(float) * n, cudaMemcpyHostToDevice, ctx->stream));
    std::mt19937 rng(seed);
    std::vector<int> perm(n);
    std::vector<float> bl(nbatch);
    const float beta1 = 0.9f, beta2 = 0.999f, eps = 1e-8f;
    for (int e = 0; e < epochs; e++) {
        for (int i = 0; i < n; i++) perm[i] = i;
        std::shuffle(perm.begin(), perm.end(), rng);
        MW_CK(cudaMemcpyAsync(s.perm, perm.data(), sizeof(int) * n, cudaMemcpyHostToDevice, ctx->stream));
        for (int b = 0; b < nbatch; b++) {
            const int base = b * batch, cnt = std::min(batch, n - base);
            double wsum = 0.0;
            for (int i = base; i < base + cnt; i++) wsum += y[perm[i]] > 0.5f ? pos_weight : 1.0f;
            launch_mlp_train_tile(s.x, s.y, s.perm, base, cnt, m->wb, pos_weight, (float)(1.0 / wsum), s.partial, s.loss_partial, ctx->stream);
            launch_mlp_reduce(s.partial, s.loss_partial, (cnt + kTile - 1) / kTile, s.grad, s.loss + b, ctx->stream);
            m->steps++;
            const float c1 = 1.f - std::pow(beta1, (float)m->steps), c2 = 1.f - std::pow(beta2, (float)m->steps);
            launch_mlp_adam(m->master, m->m1, m->m2, s.grad, m->wb, lr, beta1, beta2, eps, c1, c2, ctx->stream);
            ctx->launches += 3;
        }
        MW_CK(cudaGetLastError());
        MW_CK(cudaMemcpyAsync(bl.data(), s.loss, sizeof(float) * nbatch, cudaMemcpyDeviceToHost, ctx->stream));
        MW_CK(cudaStreamSynchronize(ctx->stream));  // the permutation buffer is rewritten by the next epoch
        if (epoch_loss) {
            double a = 0.0;
            for (int b = 0; b < nbatch; b++) a += bl[b];
            epoch_loss[e] = (float)(a / nbatch);
        }
    }
    return MWGPU_OK;
}

mwgpu_status mwgpu_mlp_predict(mwgpu_ctx *ctx, mwgpu_mlp *m, const mwgpu_oper *o, const mwgpu_tree *inp, double f_norm, const int *idx, int n,
                               float *prob) {
    if (!ctx || !m || !o || !inp || !prob) return MWGPU_ERR_BAD_ARG;
    MW_ARG(n >= 0 && (n == 0 || idx), "invalid node list");
    MW_ARG(inp->is_input, "features are computed against an input tree");
    if (n == 0) return MWGPU_OK;
    cudaSetDevice(ctx->device);
    const int rows = o->n_rows, T = o->op.n_terms;
    std::vector<int> tab(2 * (size_t)rows, 0);
    for (int d = 0; d < rows; d++) {
        tab[d] = o->band_max[d];
        for (int t = 0; t < T; t++) tab[rows + d] += o->widths[((size_t)t * rows + d) * 5 + 4] >= 0;
    }
    if (n > m->p_cap) {
        for (void *p : {(void *)m->p_nodes, (void *)m->p_x, (void *)m->p_prob})
            if (p) cudaFree(p);
        m->p_nodes = nullptr;
        m->p_x = m->p_prob = nullptr;
        m->p_cap = 0;
        const int cap = std::max(n, 1024);
        mwgpu_status st;
        if ((st = dev_alloc(ctx, &m->p_nodes, cap)) || (st = dev_alloc(ctx, &m->p_x, (size_t)cap * kMlpFeatures)) ||
            (st = dev_alloc(ctx, &m->p_prob, cap)))
            return st;
        m->p_cap = cap;
    }
    if (rows > m->p_rows) {
        if (m->p_tab) cudaFree(m->p_tab);
        m->p_tab = nullptr;
        m->p_rows = 0;
        if (auto st = dev_alloc(ctx, &m->p_tab, 2 * (size_t)rows)) return st;
        m->p_rows = rows;
    }
    std::vector<int4> nodes(n);
    for (int i = 0; i < n; i++) nodes[i] = make_int4(idx[4 * i], idx[4 * i + 1], idx[4 * i + 2], idx[4 * i + 3]);
    MW_CK(cudaMemcpyAsync(m->p_nodes, nodes.data(), sizeof(int4) * n, cudaMemcpyHostToDevice, ctx->stream));
    MW_CK(cudaMemcpyAsync(m->p_tab, tab.data(), sizeof(int) * 2 * rows, cudaMemcpyHostToDevice, ctx->stream));
    launch_mlp_features(inp->mra, inp->t, m->p_nodes, n, m->p_tab, m->p_tab + rows, rows, f_norm, m->p_x, ctx->stream);
    launch_mlp_infer(m->p_x, n, m->wb, m->p_prob, ctx->stream);
    ctx->launches += 2;
    MW_CK(cudaGetLastError());
    MW_CK(cudaMemcpyAsync(prob, m->p_prob, sizeof(float) * n, cudaMemcpyDeviceToHost, ctx->stream));
    MW_CK(cudaStreamSynchronize(ctx->stream));
    return MWGPU_OK;
}

}  // extern "C"
