// pnjl_probe.cu -- pipe-throughput probes used as roofline denominators.
//
// Each probe runs independent dependency chains of one instruction type on every lane of a
// full grid (a multiple of the SM count) and reports operations per second from CUDA-event
// time.  kind 0: FP64 FMA, 1: FP32 FMA, 2: FP32 ex2.approx (the SFU).  The chains are
// seeded from the thread index and written back so the compiler cannot drop them.
// kind 3: FP64 FMA chains on lane 0 of every warp only (the other lanes are predicated off),
// reported per active lane -- whether the FP64 pipe skips inactive lanes.
//
// Also the element-wise check of the FP64 functions of the certification pass
// (pnjl_f64.cuh) against the library functions, for the tests.
#include <cuda_runtime.h>

#include <vector>

#include "../../include/pnjl_cuda.h"
#include "pnjl_f64.cuh"
#include "pnjl_host_common.h"

namespace pnjl {

template <typename R>
__global__ void __launch_bounds__(256) fma_probe(R *out, int iters, R a, R b, int lanes) {
    if ((int)(threadIdx.x & 31) >= lanes) return;
    R x[8];
#pragma unroll
    for (int k = 0; k < 8; ++k) x[k] = (R)(threadIdx.x + k) * (R)1e-3;
    for (int i = 0; i < iters; ++i) {
#pragma unroll
        for (int k = 0; k < 8; ++k) x[k] = x[k] * a + b;
    }
    R s = 0;
#pragma unroll
    for (int k = 0; k < 8; ++k) s += x[k];
    out[blockIdx.x * blockDim.x + threadIdx.x] = s;
}

__global__ void __launch_bounds__(256) ex2_probe(float *out, int iters) {
    float x[8];
#pragma unroll
    for (int k = 0; k < 8; ++k) x[k] = -(float)(threadIdx.x + k) * 1e-4f;
    for (int i = 0; i < iters; ++i) {
#pragma unroll
        for (int k = 0; k < 8; ++k) {
            float y;
            asm volatile("ex2.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x[k]));
            x[k] = -y;  // stays in (-1, 0]: 2^x in (0.5, 1]
        }
    }
    float s = 0;
#pragma unroll
    for (int k = 0; k < 8; ++k) s += x[k];
    out[blockIdx.x * blockDim.x + threadIdx.x] = s;
}

// y[i] = f(x[i]): fn 0 exp_nonpos, 1 rcp_normal, 2 rsqrt_normal, 3 exp, 4 1/x, 5 rsqrt,
// 6 ff_exp, 7 ff_log (of x as a float-float pair, returned as hi + lo)
__global__ void __launch_bounds__(256) f64_math_kernel(int fn, int64_t n, const double *x, double *y,
                                                       const float *tab_global) {
    __shared__ __align__(16) float tabf[kExpTableFloats];
    for (int i = threadIdx.x; i < kExpTableFloats; i += blockDim.x) tabf[i] = tab_global[i];
    __syncthreads();
    const double *tab = (const double *)(tabf + kExp64Offset);
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const double v = x[i];
        double r;
        switch (fn) {
            case 0: r = exp_nonpos(v, tab); break;
            case 1: r = rcp_normal(v); break;
            case 2: r = rsqrt_normal(v); break;
            case 3: r = exp(v); break;
            case 4: r = 1.0 / v; break;
            case 5: r = rsqrt(v); break;
            case 6: r = ff_to_double(ff_exp(ff_from_double(v), tabf)); break;
            default: r = ff_to_double(ff_log(ff_from_double(v), tabf)); break;
        }
        y[i] = r;
    }
}

}  // namespace pnjl

extern "C" int pnjl_f64_math_impl(int device, int fn, int64_t n, const double *x, double *y) {
    if (fn < 0 || fn > 7 || n < 0 || (n > 0 && (!x || !y))) return PNJL_ERR_INVALID_ARGUMENT;
    if (n == 0) return PNJL_OK;
    if (cudaSetDevice(device) != cudaSuccess) return PNJL_ERR_CUDA;
    std::vector<float> tabs(pnjl::kExpTableFloats);
    pnjl::ff_exp_tables(tabs.data());
    double *d = nullptr;
    const size_t bytes = (size_t)n * sizeof(double);
    if (cudaMalloc(&d, 2 * bytes + pnjl::kExpTableFloats * sizeof(float)) != cudaSuccess) return PNJL_ERR_OUT_OF_MEMORY;
    double *dx = d, *dy = d + n;
    float *dt = (float *)(d + 2 * n);
    cudaError_t e = cudaMemcpy(dx, x, bytes, cudaMemcpyHostToDevice);
    if (e == cudaSuccess)
        e = cudaMemcpy(dt, tabs.data(), pnjl::kExpTableFloats * sizeof(float), cudaMemcpyHostToDevice);
    if (e == cudaSuccess) {
        const int64_t blocks = std::min<int64_t>((n + 255) / 256, 4096);
        pnjl::f64_math_kernel<<<(int)blocks, 256>>>(fn, n, dx, dy, dt);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaMemcpy(y, dy, bytes, cudaMemcpyDeviceToHost);
    cudaFree(d);
    return e == cudaSuccess ? PNJL_OK : PNJL_ERR_CUDA;
}

extern "C" int pnjl_probe_peak_impl(int device, int kind, double *ops_per_s) {
    if (!ops_per_s || kind < 0 || kind > 3) return PNJL_ERR_INVALID_ARGUMENT;
    if (cudaSetDevice(device) != cudaSuccess) return PNJL_ERR_CUDA;
    int sms = 0;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device);
    const int blocks = sms * 8, threads = 256;
    void *buf = nullptr;
    if (cudaMalloc(&buf, (size_t)blocks * threads * sizeof(double)) != cudaSuccess) return PNJL_ERR_OUT_OF_MEMORY;
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    const int iters = kind == 0 ? 2048 : (kind == 3 ? 8192 : 16384);
    float best = 1e30f;
    for (int rep = 0; rep < 4; ++rep) {
        cudaEventRecord(e0);
        if (kind == 0) pnjl::fma_probe<double><<<blocks, threads>>>((double *)buf, iters, 0.999999, 1e-7, 32);
        else if (kind == 1) pnjl::fma_probe<float><<<blocks, threads>>>((float *)buf, iters, 0.9999f, 1e-5f, 32);
        else if (kind == 3) pnjl::fma_probe<double><<<blocks, threads>>>((double *)buf, iters, 0.999999, 1e-7, 1);
        else pnjl::ex2_probe<<<blocks, threads>>>((float *)buf, iters);
        cudaEventRecord(e1);
        cudaEventSynchronize(e1);
        float ms = 0.f;
        cudaEventElapsedTime(&ms, e0, e1);
        if (rep > 0 && ms < best) best = ms;  // first launch is the warm-up
    }
    cudaError_t err = cudaGetLastError();
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    cudaFree(buf);
    if (err != cudaSuccess) return PNJL_ERR_CUDA;
    const double lanes = kind == 3 ? (double)blocks * threads / 32.0 : (double)blocks * threads;
    const double ops = lanes * iters * 8.0 * (kind == 2 ? 1.0 : 2.0);
    *ops_per_s = ops / (best * 1e-3);
    return PNJL_OK;
}
