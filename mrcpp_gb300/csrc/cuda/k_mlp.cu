// Learned output grid: a 3-layer, 64-wide multilayer perceptron that predicts,
// for a node of the output tree of apply, whether the wavelet-norm split test
// (tree_utils::split_check, tree_utils.cpp:47-65) will refine it.  Nothing in
// the reference corresponds to it; the split test itself stays the judge.
//
//   features x (8)  ->  h1 = relu(W1 x + b1) (64)  ->  h2 = relu(W2 h1 + b2) (64)
//                   ->  z = W3 . h2 + b3,   P(split) = sigmoid(z)
//
// Weights are BF16 for the forward passes (an FP32 master copy is updated by
// Adam); products and sums are FP32.  Training minimises the weighted binary
// cross entropy  sum_s w_s [max(z,0) - z y + log(1 + exp(-|z|))] / sum_s w_s,
// w_s = pos_weight for split nodes, 1 otherwise.
//
// Features of a node (n, l) against the input tree f (relative to the total
// norm |f| of f, base-10 logarithms):
//   0  depth / 16
//   1  log10 |f(n,l)| / 8: the wavelet norm of f's node, or, where f has no
//      node there, the nearest stored ancestor's norm times 2^(-3(n-a)/2) (its
//      norm spread over the 8^(n-a) descendants)
//   2  log10 of the total-norm estimate summed over the operator band box at
//      this depth (half width min(band_max, 3), clipped to the world) / 8
//   3  operator terms whose band reaches this depth / 100
//   4-6  translation parity l_d mod 2
//   7  f at (n, l): 1 = a node with children, 0.5 = a leaf, 0 = no node
#include <cuda_bf16.h>

#include "mwgpu_internal.cuh"

namespace mwgpu {
namespace mlp {

constexpr int F = kMlpFeatures, H = kMlpHidden;
constexpr int OFF_W1 = 0, OFF_B1 = OFF_W1 + H * F, OFF_W2 = OFF_B1 + H, OFF_B2 = OFF_W2 + H * H, OFF_W3 = OFF_B2 + H, OFF_B3 = OFF_W3 + H;
static_assert(OFF_B3 + 1 == kMlpParams, "parameter layout");
constexpr int TILE = 128;  // samples per CTA in training
constexpr int HP = H + 1;  // padded row of the per-sample activations

__device__ __forceinline__ float bf(const __nv_bfloat16 v) { return __bfloat162float(v); }

// loads the BF16 weights into shared memory as floats
__device__ __forceinline__ void load_weights(float *w, const __nv_bfloat16 *wb) {
    for (int i = threadIdx.x; i < kMlpParams; i += blockDim.x) w[i] = bf(wb[i]);
}

// forward pass of one sample; h1, h2 may be null (inference)
__device__ __forceinline__ float forward(const float *w, const float *x, float *h1s, float *h2s) {
    float h1[H];
#pragma unroll 4
    for (int j = 0; j < H; j++) {
        float a = w[OFF_B1 + j];
#pragma unroll
        for (int i = 0; i < F; i++) a = fmaf(w[OFF_W1 + j * F + i], x[i], a);
        h1[j] = fmaxf(a, 0.f);
        if (h1s) h1s[j] = h1[j];
    }
    float z = w[OFF_B3];
    for (int j = 0; j < H; j++) {
        float a = w[OFF_B2 + j];
#pragma unroll
        for (int i = 0; i < H; i++) a = fmaf(w[OFF_W2 + j * H + i], h1[i], a);
        const float h = fmaxf(a, 0.f);
        if (h2s) h2s[j] = h;
        z = fmaf(w[OFF_W3 + j], h, z);
    }
    return z;
}

__global__ void __launch_bounds__(128) k_infer(const float *X, int n, const __nv_bfloat16 *wb, float *prob) {
    extern __shared__ float w[];
    load_weights(w, wb);
    __syncthreads();
    for (int s = blockIdx.x * blockDim.x + threadIdx.x; s < n; s += gridDim.x * blockDim.x) {
        float x[F];
#pragma unroll
        for (int i = 0; i < F; i++) x[i] = X[(size_t)s * F + i];
        const float z = forward(w, x, nullptr, nullptr);
        prob[s] = 1.f / (1.f + expf(-z));
    }
}

// One tile of TILE samples (sample ids idx[base + s], or base + s without idx):
// forward, backward, and the tile's parameter gradients and loss.
__global__ void __launch_bounds__(TILE) k_train_tile(const float *X, const float *Y, const int *idx, int base, int count,
                                                     const __nv_bfloat16 *wb, float pos_weight, float inv_wsum, float *partial,
                                                     float *loss_partial) {
    extern __shared__ float sm[];
    float *w = sm;                      // kMlpParams
    float *xs = w + kMlpParams;         // [TILE][F]
    float *h1 = xs + TILE * F;          // [TILE][HP]
    float *h2 = h1 + TILE * HP;         // [TILE][HP]
    float *d2 = h2 + TILE * HP;         // [TILE][HP]
    float *d1 = d2 + TILE * HP;         // [TILE][HP]
    float *dz = d1 + TILE * HP;         // [TILE]
    float *ls = dz + TILE;              // [TILE]
    load_weights(w, wb);
    const int s = threadIdx.x;
    const int t0 = blockIdx.x * TILE;
    const bool valid = t0 + s < count;
    const int sid = valid ? (idx ? idx[base + t0 + s] : base + t0 + s) : 0;
    for (int i = 0; i < F; i++) xs[s * F + i] = valid ? X[(size_t)sid * F + i] : 0.f;
    __syncthreads();
    float loss = 0.f, g = 0.f;
    if (valid) {
        const float z = forward(w, xs + s * F, h1 + s * HP, h2 + s * HP);
        const float y = Y[sid];
        const float ws = (y > 0.5f ? pos_weight : 1.f) * inv_wsum;
        loss = ws * (fmaxf(z, 0.f) - z * y + log1pf(expf(-fabsf(z))));
        const float p = 1.f / (1.f + expf(-z));
        g = ws * (p - y);
    } else {
        for (int j = 0; j < H; j++) h1[s * HP + j] = h2[s * HP + j] = 0.f;
    }
    dz[s] = g;
    ls[s] = loss;
    // dh2 = g W3 (h2 > 0); dh1 = W2^T dh2 (h1 > 0)
    for (int j = 0; j < H; j++) d2[s * HP + j] = h2[s * HP + j] > 0.f ? g * w[OFF_W3 + j] : 0.f;
    for (int i = 0; i < H; i++) {
        float a = 0.f;
        for (int j = 0; j < H; j++) a = fmaf(w[OFF_W2 + j * H + i], d2[s * HP + j], a);
        d1[s * HP + i] = h1[s * HP + i] > 0.f ? a : 0.f;
    }
    __syncthreads();
    // parameter gradients of the tile, summed over its samples in order
    float *out = partial + (size_t)blockIdx.x * kMlpParams;
    for (int p = threadIdx.x; p < kMlpParams; p += TILE) {
        float a = 0.f;
        if (p < OFF_B1) {
            const int j = p / F, i = p % F;
            for (int q = 0; q < TILE; q++) a = fmaf(d1[q * HP + j], xs[q * F + i], a);
        } else if (p < OFF_W2) {
            const int j = p - OFF_B1;
            for (int q = 0; q < TILE; q++) a += d1[q * HP + j];
        } else if (p < OFF_B2) {
            const int j = (p - OFF_W2) / H, i = (p - OFF_W2) % H;
            for (int q = 0; q < TILE; q++) a = fmaf(d2[q * HP + j], h1[q * HP + i], a);
        } else if (p < OFF_W3) {
            const int j = p - OFF_B2;
            for (int q = 0; q < TILE; q++) a += d2[q * HP + j];
        } else if (p < OFF_B3) {
            const int i = p - OFF_W3;
            for (int q = 0; q < TILE; q++) a = fmaf(dz[q], h2[q * HP + i], a);
        } else {
            for (int q = 0; q < TILE; q++) a += dz[q];
        }
        out[p] = a;
    }
    if (threadIdx.x == 0) {
        float l = 0.f;
        for (int q = 0; q < TILE; q++) l += ls[q];
        loss_partial[blockIdx.x] = l;
    }
}

// grad[p] = sum over tiles in order; loss = sum of the tile losses
__global__ void k_reduce_grad(const float *partial, const float *loss_partial, int tiles, float *grad, float *loss) {
    for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < kMlpParams; p += gridDim.x * blockDim.x) {
        float a = 0.f;
        for (int t = 0; t < tiles; t++) a += partial[(size_t)t * kMlpParams + p];
        grad[p] = a;
    }
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        float l = 0.f;
        for (int t = 0; t < tiles; t++) l += loss_partial[t];
        *loss = l;
    }
}

// Adam (Kingma & Ba 2015) on the FP32 master weights, then the BF16 copy
__global__ void k_adam(float *master, float *m1, float *m2, const float *grad, __nv_bfloat16 *wb, float lr, float beta1, float beta2,
                       float eps, float c1, float c2) {
    for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < kMlpParams; p += gridDim.x * blockDim.x) {
        const float gp = grad[p];
        const float a = beta1 * m1[p] + (1.f - beta1) * gp;
        const float b = beta2 * m2[p] + (1.f - beta2) * gp * gp;
        m1[p] = a;
        m2[p] = b;
        const float v = master[p] - lr * (a / c1) / (sqrtf(b / c2) + eps);
        master[p] = v;
        wb[p] = __float2bfloat16_rn(v);
    }
}

__global__ void k_to_bf16(const float *src, __nv_bfloat16 *dst, int n) {
    for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < n; p += gridDim.x * blockDim.x) dst[p] = __float2bfloat16_rn(src[p]);
}

// norm of f around (n, l): the stored node (wavelet part only if `wavelet`),
// else the nearest stored ancestor's total norm spread over its descendants;
// 0 outside the world.  *stored: 0 none, 1 leaf, 2 node with children.
__device__ inline double norm_estimate(const DevMRA &m, const DevTree &f, int n, int l0, int l1, int l2, bool wavelet, int *stored) {
    *stored = 0;
    for (int a = n; a >= m.root_scale; a--) {
        const int sh = n - a;
        NodeKey key;
        if (!pack_key(m, a, l0 >> sh, l1 >> sh, l2 >> sh, key)) return 0.0;
        const int id = hash_find(f.hkeys, f.hvals, f.hcap, key);
        if (id >= 0 && id < f.cap_real) {
            double s = 0.0;
            for (int c = (wavelet && sh == 0) ? 1 : 0; c < 8; c++) {
                const double v = f.norms[(size_t)id * 8 + c];
                s += v * v;
            }
            if (sh == 0) *stored = f.child0[id] >= 0 ? 2 : 1;
            // 2^(-1.5 sh) as a power of two times 1 or 2^(-1/2)
            return ldexp(sqrt(s) * ((sh & 1) ? 0.70710678118654752440 : 1.0), -((3 * sh) / 2));
        }
    }
    return 0.0;
}

// one CTA of kFeatureThreads per node: the band cells spread over all its
// threads (each walks up to the nearest stored ancestor of its cells), the
// band sum reduced in a fixed order
constexpr int kFeatureThreads = 128;
__global__ void __launch_bounds__(kFeatureThreads) k_features(DevMRA m, DevTree f, const int4 *nodes, int n, const int *band_w, const int *terms,
                                                              int rows, double ftot, float *X) {
    const int node = blockIdx.x, tid = threadIdx.x, lane = tid & 31;
    if (node >= n) return;
    const int4 g = nodes[node];
    const int depth = g.x - m.root_scale;
    const int dr = min(max(depth, 0), rows - 1);
    const int w = min(max(band_w[dr], 0), 3);
    const int gl[3] = {g.y, g.z, g.w};
    int bs[3], be[3];
    for (int d = 0; d < 3; d++) {
        const int nb = m.nbox[d] << max(depth, 0), c = m.corner[d] << max(depth, 0);
        bs[d] = max(gl[d] - w, c);
        be[d] = min(gl[d] + w, c + nb - 1);
    }
    const int nx = be[0] - bs[0] + 1, ny = be[1] - bs[1] + 1, nz = be[2] - bs[2] + 1;
    const int cells = max(nx, 0) * max(ny, 0) * max(nz, 0);
    double band = 0.0;
    for (int q = tid; q < cells; q += kFeatureThreads) {
        int st;
        band += norm_estimate(m, f, g.x, bs[0] + q % nx, bs[1] + (q / nx) % ny, bs[2] + q / (nx * ny), false, &st);
    }
    for (int o = 16; o > 0; o >>= 1) band += __shfl_down_sync(0xffffffffu, band, o);
    __shared__ double red[kFeatureThreads / 32];
    if (lane == 0) red[tid >> 5] = band;
    __syncthreads();
    if (tid == 0) {
        double tot = 0.0;
        for (int i = 0; i < kFeatureThreads / 32; i++) tot += red[i];
        int st;
        const double own = norm_estimate(m, f, g.x, g.y, g.z, g.w, true, &st);
        const double inv = ftot > 0.0 ? 1.0 / ftot : 1.0;
        float *x = X + (size_t)node * F;
        x[0] = (float)depth / 16.f;
        x[1] = (float)(log10(fmax(own * inv, 1e-30)) / 8.0);
        x[2] = (float)(log10(fmax(tot * inv, 1e-30)) / 8.0);
        x[3] = (float)terms[dr] / 100.f;
        x[4] = (float)(g.y & 1);
        x[5] = (float)(g.z & 1);
        x[6] = (float)(g.w & 1);
        x[7] = 0.5f * (float)st;
    }
}

}  // namespace mlp

size_t mlp_train_smem() {
    return sizeof(float) * (kMlpParams + mlp::TILE * mlp::F + 4 * mlp::TILE * mlp::HP + 2 * mlp::TILE);
}

void launch_mlp_infer(const float *X, int n, const __nv_bfloat16 *wb, float *prob, cudaStream_t s) {
    if (n <= 0) return;
    const int blocks = std::min((n + 127) / 128, 152 * 8);
    mlp::k_infer<<<blocks, 128, sizeof(float) * kMlpParams, s>>>(X, n, wb, prob);
}

void launch_mlp_train_tile(const float *X, const float *Y, const int *idx, int base, int count, const __nv_bfloat16 *wb, float pos_weight,
                           float inv_wsum, float *partial, float *loss_partial, cudaStream_t s) {
    if (count <= 0) return;
    const size_t smem = mlp_train_smem();
    cudaFuncSetAttribute(mlp::k_train_tile, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    const int tiles = (count + mlp::TILE - 1) / mlp::TILE;
    mlp::k_train_tile<<<tiles, mlp::TILE, smem, s>>>(X, Y, idx, base, count, wb, pos_weight, inv_wsum, partial, loss_partial);
}

void launch_mlp_reduce(const float *partial, const float *loss_partial, int tiles, float *grad, float *loss, cudaStream_t s) {
    mlp::k_reduce_grad<<<(kMlpParams + 255) / 256, 256, 0, s>>>(partial, loss_partial, tiles, grad, loss);
}

void launch_mlp_adam(float *master, float *m1, float *m2, const float *grad, __nv_bfloat16 *wb, float lr, float beta1, float beta2, float eps,
                     float c1, float c2, cudaStream_t s) {
    mlp::k_adam<<<(kMlpParams + 255) / 256, 256, 0, s>>>(master, m1, m2, grad, wb, lr, beta1, beta2, eps, c1, c2);
}

void launch_mlp_to_bf16(const float *src, __nv_bfloat16 *dst, int n, cudaStream_t s) {
    mlp::k_to_bf16<<<(n + 255) / 256, 256, 0, s>>>(src, dst, n);
}

void launch_mlp_features(const DevMRA &m, const DevTree &f, const int4 *nodes, int n, const int *band_w, const int *terms, int rows, double ftot,
                         float *X, cudaStream_t s) {
    if (n <= 0) return;
    mlp::k_features<<<n, mlp::kFeatureThreads, 0, s>>>(m, f, nodes, n, band_w, terms, rows, ftot, X);
}

}  // namespace mwgpu
