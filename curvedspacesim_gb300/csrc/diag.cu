// Device diagnostics: the measured FP64 FMA issue rate used as the denominator of the geodesic kernel's FP64
// roofline (the measured peaks cover HBM copy bandwidth and BF16 tensor throughput only).
#include "cssg_internal.cuh"
#include "window.cuh"

namespace {

__global__ void __launch_bounds__(256) fp64_fma_chain(double* out, int iters, double a, double b)
{
    // 8 independent dependent chains per thread keep the FP64 pipe busy without touching memory
    double x0 = threadIdx.x * 1e-9, x1 = x0 + 1, x2 = x0 + 2, x3 = x0 + 3, x4 = x0 + 4, x5 = x0 + 5, x6 = x0 + 6,
           x7 = x0 + 7;
    for (int i = 0; i < iters; ++i) {
        x0 = fma(x0, a, b);
        x1 = fma(x1, a, b);
        x2 = fma(x2, a, b);
        x3 = fma(x3, a, b);
        x4 = fma(x4, a, b);
        x5 = fma(x5, a, b);
        x6 = fma(x6, a, b);
        x7 = fma(x7, a, b);
    }
    double s = x0 + x1 + x2 + x3 + x4 + x5 + x6 + x7;
    if (s == 12345.678) out[0] = s;  // keeps the chains alive
}

}  // namespace

extern "C" int cssg_diag_fp64_peak(cssg_ctx* ctx, double* gflops)
{
    if (!ctx || !gflops) return cssg_bad_args("cssg_diag_fp64_peak");
    DeviceScope scope(ctx->device);
    CSSG_CUDA(scope.err);
    int sms = 0;
    CSSG_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, ctx->device));
    double* out = nullptr;
    CSSG_CUDA(cudaMallocAsync((void**)&out, sizeof(double), ctx->stream));
    cudaEvent_t e0, e1;
    CSSG_CUDA(cudaEventCreate(&e0));
    CSSG_CUDA(cudaEventCreate(&e1));
    const int blocks = sms * 8, threads = 256, iters = 4096;
    fp64_fma_chain<<<blocks, threads, 0, ctx->stream>>>(out, iters, 0.999999, 1e-7);  // warm-up
    CSSG_CUDA(cudaEventRecord(e0, ctx->stream));
    fp64_fma_chain<<<blocks, threads, 0, ctx->stream>>>(out, iters, 0.999999, 1e-7);
    CSSG_CUDA(cudaEventRecord(e1, ctx->stream));
    CSSG_CUDA(cudaEventSynchronize(e1));
    float ms = 0;
    CSSG_CUDA(cudaEventElapsedTime(&ms, e0, e1));
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    CSSG_CUDA(cudaFreeAsync(out, ctx->stream));
    double flops = 2.0 * 8.0 * (double)iters * blocks * threads;
    *gflops = flops / (ms * 1e-3) / 1e9;
    return CSSG_OK;
}

namespace {
__global__ void reciprocal_kernel(int n, const double* __restrict__ x, double* __restrict__ out)
{
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) out[i] = rcp_nr(x[i]);
}
}  // namespace

// The propagation's reciprocal (rcp_nr) on n device values, for accuracy tests.
extern "C" int cssg_diag_reciprocal(cssg_ctx* ctx, int n, const double* x, double* out)
{
    if (!ctx || n < 0 || (n > 0 && (!x || !out))) {
        cssg_set_error("cssg_diag_reciprocal: bad arguments");
        return CSSG_ERR_ARG;
    }
    DeviceScope scope(ctx->device);
    CSSG_CUDA(scope.err);
    if (n) reciprocal_kernel<<<(n + 255) / 256, 256, 0, ctx->stream>>>(n, x, out);
    CSSG_CUDA(cudaGetLastError());
    return CSSG_OK;
}

extern "C" int cssg_diag_flops_per_window(void) { return kFlopsPerWindow; }
