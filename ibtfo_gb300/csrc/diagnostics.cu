// Diagnostics with no reference counterpart: the FP64 pipe rate of the
// current GPU, and an evaluator of the fp64_fast / FP32 form's reciprocal and
// square root for error-bound tests.
//
// FP64 pipe rate.  The plain FP64 sweep is bound by the FP64 pipe rather than
// by HBM, so its roofline denominator is the pipe's instruction rate.  The
// kernel keeps every warp slot busy with independent DFMA chains (eight per
// thread, 2,048 threads per SM) and little else: per iteration a thread
// issues eight DFMA and two integer instructions.  The rate it reports is
// FP64 thread instructions per second (one DFMA = one pipe instruction = two
// flops), the unit of the sweep's FP64 instruction count (DADD + DMUL + DFMA
// thread instructions per launch).
#include <cuda_runtime.h>

#include "../../include/ibtfo.h"
#include "internal.h"
#include "physics_fast.cuh"

namespace ibtfo {
void set_last_error(const char *msg);
}

namespace {
constexpr int kChains = 8;
constexpr int kThreads = 256;
constexpr int kCtasPerSm = 8;

__global__ void __launch_bounds__(kThreads) fp64_fma_chains_kernel(double *sink, int iters, double a, double b)
{
    double x[kChains];
#pragma unroll
    for (int k = 0; k < kChains; k++)
        x[k] = 1.0 + 1e-3 * (double)(threadIdx.x + k);
    for (int i = 0; i < iters; i++)
    {
#pragma unroll
        for (int k = 0; k < kChains; k++)
            x[k] = fma(x[k], a, b);
    }
    double s = 0.0;
#pragma unroll
    for (int k = 0; k < kChains; k++)
        s += x[k];
    // never true for the arguments below (the chains stay near 1): keeps the
    // chains live without a store per thread
    if (s == -1.0)
        sink[blockIdx.x * blockDim.x + threadIdx.x] = s;
}

// y[i] = f(x[i]) for the function selected by `fn` (IBTFO_MATH_*)
__global__ void fast_math_kernel(int fn, const double *__restrict__ x, double *__restrict__ y, int n)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n)
        return;
    const double v = x[i];
    double r = 0.0;
    switch (fn)
    {
    case IBTFO_MATH_RCP_F64: r = ibtfo::rcp_t(v); break;
    case IBTFO_MATH_SQRT_F64: r = ibtfo::sqrt_t(v); break;
    case IBTFO_MATH_RCP_F32: r = (double)ibtfo::rcp_t((float)v); break;
    case IBTFO_MATH_SQRT_F32: r = (double)ibtfo::sqrt_t((float)v); break;
    case IBTFO_MATH_DIV_F64: r = 1.0 / v; break;
    case IBTFO_MATH_LIBSQRT_F64: r = sqrt(v); break;
    case IBTFO_MATH_DIV_F32: r = (double)(1.0f / (float)v); break;
    default: r = sqrtf((float)v); break;
    }
    y[i] = r;
}

struct DevBuf
{
    void *p = nullptr;
    ~DevBuf()
    {
        if (p)
            cudaFree(p);
    }
};
} // namespace

extern "C" ibtfo_status ibtfo_fp64_pipe_rate(int iters, double *inst_per_s, double *seconds)
{
    using namespace ibtfo;
    if (!inst_per_s || iters < 1 || iters > (1 << 20))
    {
        set_last_error("ibtfo_fp64_pipe_rate: need inst_per_s and 1 <= iters <= 2^20");
        return IBTFO_EINVAL;
    }
    int dev = 0, sms = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e == cudaSuccess)
        e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    const int grid = sms * kCtasPerSm;
    DevBuf sink;
    cudaStream_t s = nullptr;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    if (e == cudaSuccess)
        e = cudaMalloc(&sink.p, (size_t)grid * kThreads * sizeof(double));
    if (e == cudaSuccess)
        e = cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking);
    if (e == cudaSuccess)
        e = cudaEventCreate(&e0);
    if (e == cudaSuccess)
        e = cudaEventCreate(&e1);
    float ms = 0.0f;
    if (e == cudaSuccess)
    {
        // a = 1 - 2^-20, b = 2^-20: every chain moves toward the fixed point 1
        // (no overflow, no subnormals)
        const double a = 1.0 - 0x1p-20, b = 0x1p-20;
        double *out = static_cast<double *>(sink.p);
        fp64_fma_chains_kernel<<<grid, kThreads, 0, s>>>(out, iters / 8 + 1, a, b); // warm-up
        cudaEventRecord(e0, s);
        fp64_fma_chains_kernel<<<grid, kThreads, 0, s>>>(out, iters, a, b);
        cudaEventRecord(e1, s);
        count_launch(2);
        e = cudaEventSynchronize(e1);
        if (e == cudaSuccess)
            e = cudaEventElapsedTime(&ms, e0, e1);
    }
    if (e0)
        cudaEventDestroy(e0);
    if (e1)
        cudaEventDestroy(e1);
    if (s)
        cudaStreamDestroy(s);
    if (e != cudaSuccess || !(ms > 0.0f))
    {
        set_last_error(e != cudaSuccess ? cudaGetErrorString(e) : "ibtfo_fp64_pipe_rate: zero elapsed time");
        return IBTFO_ECUDA;
    }
    const double inst = (double)grid * kThreads * kChains * (double)iters;
    *inst_per_s = inst / (ms * 1e-3);
    if (seconds)
        *seconds = ms * 1e-3;
    return IBTFO_OK;
}

extern "C" ibtfo_status ibtfo_fast_math_eval(int fn, const double *x, double *y, int n)
{
    using namespace ibtfo;
    if (!x || !y || n < 1 || fn < 0 || fn > IBTFO_MATH_LIBSQRT_F32)
    {
        set_last_error("ibtfo_fast_math_eval: need x, y, n >= 1 and a known function");
        return IBTFO_EINVAL;
    }
    const size_t bytes = (size_t)n * sizeof(double);
    DevBuf dx, dy;
    cudaError_t e = cudaMalloc(&dx.p, bytes);
    if (e == cudaSuccess)
        e = cudaMalloc(&dy.p, bytes);
    if (e == cudaSuccess)
        e = cudaMemcpy(dx.p, x, bytes, cudaMemcpyHostToDevice);
    if (e == cudaSuccess)
    {
        fast_math_kernel<<<(n + 255) / 256, 256>>>(fn, static_cast<const double *>(dx.p), static_cast<double *>(dy.p),
                                                   n);
        count_launch();
        e = cudaGetLastError();
    }
    if (e == cudaSuccess)
        e = cudaMemcpy(y, dy.p, bytes, cudaMemcpyDeviceToHost);
    if (e != cudaSuccess)
    {
        set_last_error(cudaGetErrorString(e));
        return IBTFO_ECUDA;
    }
    return IBTFO_OK;
}
