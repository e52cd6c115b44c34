// Pipe calibration: throughput of FMA and of each transcendental / division
// in FP64 and FP32 on this GPU.  The roofline of the RPMD kernels is the FP64
// (plain form) or FP32 (mixed form) pipe, and the algorithmic work of the
// reference formulas counts each exp, pow, division ... once; these timings
// turn those counts into FMA-equivalents measured on the same device.
#include <cuda_runtime.h>

#include "../../include/caracal_gb300.h"

namespace {

constexpr int kChains = 8;

template <class F> __device__ inline F op_apply(int op, F x);

template <>
__device__ inline double op_apply<double>(int op, double x) {
  switch (op) {
    case CR_CALIB_FMA: return fma(x, 0.999999, 1e-7);
    case CR_CALIB_DIV: return 1.0000001 / x;
    case CR_CALIB_SQRT: return sqrt(x) + 0.25;
    case CR_CALIB_EXP: return exp(-x);
    case CR_CALIB_LOG: return log(x + 2.0);
    case CR_CALIB_POW: return pow(x + 1.5, -0.7);
    case CR_CALIB_SIN: return sin(x) + 0.5;
    case CR_CALIB_COS: return cos(x);
    case CR_CALIB_ACOS: return acos(0.5 * x) * 0.3;
    case CR_CALIB_ERF: return erf(x) + 0.1;
    case CR_CALIB_TANH: return tanh(x) + 0.2;
    case CR_CALIB_COSH: return cosh(x) - 0.9;
    default: return x;
  }
}

template <>
__device__ inline float op_apply<float>(int op, float x) {
  switch (op) {
    case CR_CALIB_FMA: return fmaf(x, 0.999999f, 1e-7f);
    case CR_CALIB_DIV: return 1.0000001f / x;
    case CR_CALIB_SQRT: return sqrtf(x) + 0.25f;
    case CR_CALIB_EXP: return expf(-x);
    case CR_CALIB_LOG: return logf(x + 2.0f);
    case CR_CALIB_POW: return powf(x + 1.5f, -0.7f);
    case CR_CALIB_SIN: return sinf(x) + 0.5f;
    case CR_CALIB_COS: return cosf(x);
    case CR_CALIB_ACOS: return acosf(0.5f * x) * 0.3f;
    case CR_CALIB_ERF: return erff(x) + 0.1f;
    case CR_CALIB_TANH: return tanhf(x) + 0.2f;
    case CR_CALIB_COSH: return coshf(x) - 0.9f;
    default: return x;
  }
}

template <class F, int OP>
__global__ void calib_kernel(F* out, int iters) {
  F x[kChains];
#pragma unroll
  for (int c = 0; c < kChains; ++c) x[c] = F(0.5) + F(1e-3) * F(c) + F(1e-7) * F(threadIdx.x);
  for (int it = 0; it < iters; ++it) {
#pragma unroll
    for (int c = 0; c < kChains; ++c) x[c] = op_apply<F>(OP, x[c]);
  }
  F s = F(0);
#pragma unroll
  for (int c = 0; c < kChains; ++c) s += x[c];
  if (s == F(-12345)) out[blockIdx.x * blockDim.x + threadIdx.x] = s;  // keeps the work alive
}

// FP64 tensor-core throughput: kChains independent m8n8k4 accumulations per
// warp (A 8x4 row, B 4x8 col: one double of each per thread, D 8x8: two).
__global__ void calib_dmma_kernel(double* out, int iters) {
  const double a = 1e-3 + 1e-9 * threadIdx.x, b = 1e-3;
  double d0[kChains], d1[kChains];
#pragma unroll
  for (int c = 0; c < kChains; ++c) {
    d0[c] = 1e-3 * c;
    d1[c] = 0.0;
  }
  for (int it = 0; it < iters; ++it) {
#pragma unroll
    for (int c = 0; c < kChains; ++c)
      asm volatile("mma.sync.aligned.m8n8k4.row.col.f64.f64.f64.f64 {%0, %1}, {%2}, {%3}, {%0, %1};\n"
                   : "+d"(d0[c]), "+d"(d1[c])
                   : "d"(a), "d"(b));
  }
  double s = 0.0;
#pragma unroll
  for (int c = 0; c < kChains; ++c) s += d0[c] + d1[c];
  if (s == -12345.0) out[blockIdx.x * blockDim.x + threadIdx.x] = s;  // keeps the work alive
}

template <class F>
int run_one(int op, int iters, float* ms) {
  int dev = 0, sms = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return CR_ERR_NO_DEVICE;
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  const int block = 256, grid = sms * 8;
  F* out = nullptr;
  if (cudaMalloc(&out, (size_t)grid * block * sizeof(F)) != cudaSuccess) return CR_ERR_CUDA;
  cudaEvent_t a, b;
  cudaEventCreate(&a);
  cudaEventCreate(&b);
  auto launch = [&]() {
    switch (op) {
      case CR_CALIB_FMA: calib_kernel<F, CR_CALIB_FMA><<<grid, block>>>(out, iters); break;
      case CR_CALIB_DIV: calib_kernel<F, CR_CALIB_DIV><<<grid, block>>>(out, iters); break;
      case CR_CALIB_SQRT: calib_kernel<F, CR_CALIB_SQRT><<<grid, block>>>(out, iters); break;
      case CR_CALIB_EXP: calib_kernel<F, CR_CALIB_EXP><<<grid, block>>>(out, iters); break;
      case CR_CALIB_LOG: calib_kernel<F, CR_CALIB_LOG><<<grid, block>>>(out, iters); break;
      case CR_CALIB_POW: calib_kernel<F, CR_CALIB_POW><<<grid, block>>>(out, iters); break;
      case CR_CALIB_SIN: calib_kernel<F, CR_CALIB_SIN><<<grid, block>>>(out, iters); break;
      case CR_CALIB_COS: calib_kernel<F, CR_CALIB_COS><<<grid, block>>>(out, iters); break;
      case CR_CALIB_ACOS: calib_kernel<F, CR_CALIB_ACOS><<<grid, block>>>(out, iters); break;
      case CR_CALIB_ERF: calib_kernel<F, CR_CALIB_ERF><<<grid, block>>>(out, iters); break;
      case CR_CALIB_TANH: calib_kernel<F, CR_CALIB_TANH><<<grid, block>>>(out, iters); break;
      case CR_CALIB_COSH: calib_kernel<F, CR_CALIB_COSH><<<grid, block>>>(out, iters); break;
      case CR_CALIB_DMMA:
        if constexpr (sizeof(F) == 8) calib_dmma_kernel<<<grid, block>>>(out, iters);
        break;
      default: break;
    }
  };
  launch();  // warm-up
  cudaEventRecord(a);
  launch();
  cudaEventRecord(b);
  cudaError_t err = cudaEventSynchronize(b);
  cudaEventElapsedTime(ms, a, b);
  cudaEventDestroy(a);
  cudaEventDestroy(b);
  cudaFree(out);
  return err == cudaSuccess ? CR_OK : CR_ERR_CUDA;
}

}  // namespace

extern "C" int cr_calibrate_op(int fp64, int op, int iters, double* ops_per_s) {
  if (!ops_per_s || op < CR_CALIB_FMA || op > CR_CALIB_DMMA || iters < 1) return CR_ERR_ARG;
  if (op == CR_CALIB_DMMA && !fp64) return CR_ERR_ARG;
  int n = 0;
  if (cudaGetDeviceCount(&n) != cudaSuccess || n == 0) return CR_ERR_NO_DEVICE;
  float ms = 0.f;
  int rc = fp64 ? run_one<double>(op, iters, &ms) : run_one<float>(op, iters, &ms);
  if (rc) return rc;
  int dev = 0, sms = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  double total = (double)sms * 8 * 256 * kChains * (double)iters;
  if (op == CR_CALIB_DMMA) total = total / 32.0 * 256.0;  // per warp instruction: 8 x 8 x 4 multiply-adds
  *ops_per_s = total / (ms * 1e-3);
  return CR_OK;
}
