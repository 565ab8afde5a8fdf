// probes.cu -- small device kernels used by the tests and the benchmark:
// elementwise hmath evaluation (host/device bit-equality checks) and an
// FP64 issue-rate probe (the FP64 roofline denominator).
#include <cstdint>

#include "fp64i.h"
#include "hmath.h"

namespace mhm {

__global__ void hmath_eval_kernel(int op, int64_t n, const double *x, const double *y, double *out)
{
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const double v = x[i];
    out[i] = op == 0 ? hm_log(v) : op == 1 ? hm_exp(v) : op == 2 ? hm_pow(v, y[i]) : hm_div(v, y[i]);
}

// 8 independent DFMA chains per thread keep the FP64 pipe busy; the result is
// stored so the chains are not removed.
__global__ void fp64_probe_kernel(int64_t iters, double *sink)
{
    const int64_t tid = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    double a0 = 1.0 + tid * 1e-9, a1 = a0 + 1e-3, a2 = a0 + 2e-3, a3 = a0 + 3e-3;
    double a4 = a0 + 4e-3, a5 = a0 + 5e-3, a6 = a0 + 6e-3, a7 = a0 + 7e-3;
    const double b = 0.999999999, c = 1e-12;
    for (int64_t i = 0; i < iters; ++i) {
        a0 = fma(a0, b, c);
        a1 = fma(a1, b, c);
        a2 = fma(a2, b, c);
        a3 = fma(a3, b, c);
        a4 = fma(a4, b, c);
        a5 = fma(a5, b, c);
        a6 = fma(a6, b, c);
        a7 = fma(a7, b, c);
    }
    sink[tid] = a0 + a1 + a2 + a3 + a4 + a5 + a6 + a7;
}

cudaError_t launch_hmath_eval(int op, int64_t n, const double *x, const double *y, double *out, cudaStream_t s)
{
    if (n == 0) return cudaSuccess;
    hmath_eval_kernel<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(op, n, x, y, out);
    return cudaGetLastError();
}

cudaError_t launch_fp64_probe(int64_t iters, int blocks, int threads, double *sink, cudaStream_t s)
{
    fp64_probe_kernel<<<blocks, threads, 0, s>>>(iters, sink);
    return cudaGetLastError();
}

} // namespace mhm
