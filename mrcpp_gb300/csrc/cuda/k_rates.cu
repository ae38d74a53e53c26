// Peak issue rates of the two FP64 paths of this GPU, measured (no reference
// counterpart): chains of independent DFMA per thread, and chains of
// mma.sync.aligned.m8n8k4.f64 (DMMA) per warp.  The FP64 form of the
// contraction is bound by whichever pipe it runs on, so the faster of the two
// is the one to use; mwgpu_fp64_pipe_rates reports both.
#include "mwgpu_internal.cuh"

namespace mwgpu {
namespace {

constexpr int kRateThreads = 256;

__global__ void __launch_bounds__(kRateThreads) k_rate_dfma(double *out, int iters, double a, double b) {
    double x[8];
#pragma unroll
    for (int i = 0; i < 8; i++) x[i] = threadIdx.x * 1e-9 + i;
    for (int it = 0; it < iters; it++)
#pragma unroll
        for (int i = 0; i < 8; i++) x[i] = fma(x[i], a, b);
    double s = 0.0;
#pragma unroll
    for (int i = 0; i < 8; i++) s += x[i];
    out[blockIdx.x * blockDim.x + threadIdx.x] = s;
}

__global__ void __launch_bounds__(kRateThreads) k_rate_dmma(double *out, int iters, double a, double b) {
    double d[4][2];
#pragma unroll
    for (int i = 0; i < 4; i++) {
        d[i][0] = threadIdx.x * 1e-9 + i;
        d[i][1] = i;
    }
    const double av = a + threadIdx.x * 1e-12, bv = b;
    for (int it = 0; it < iters; it++)
#pragma unroll
        for (int i = 0; i < 4; i++)
            asm volatile("mma.sync.aligned.m8n8k4.row.col.f64.f64.f64.f64 {%0,%1}, {%2}, {%3}, {%0,%1};\n"
                         : "+d"(d[i][0]), "+d"(d[i][1])
                         : "d"(av), "d"(bv));
    double s = 0.0;
#pragma unroll
    for (int i = 0; i < 4; i++) s += d[i][0] + d[i][1];
    out[blockIdx.x * blockDim.x + threadIdx.x] = s;
}

}  // namespace

// blocks of kRateThreads threads, `iters` steps each: FLOP counts per launch
void launch_rate_dfma(double *out, int blocks, int iters, cudaStream_t s) {
    k_rate_dfma<<<blocks, kRateThreads, 0, s>>>(out, iters, 0.999999, 1e-7);
}
void launch_rate_dmma(double *out, int blocks, int iters, cudaStream_t s) {
    k_rate_dmma<<<blocks, kRateThreads, 0, s>>>(out, iters, 0.999999, 1e-7);
}
double rate_dfma_flops(int blocks, int iters) { return 2.0 * 8 * (double)iters * blocks * kRateThreads; }
double rate_dmma_flops(int blocks, int iters) { return 2.0 * 8 * 8 * 4 * 4 * (double)iters * blocks * (kRateThreads / 32); }
int rate_threads() { return kRateThreads; }

}  // namespace mwgpu
