// rsg_pipes.cu -- issue rates of the arithmetic pipes the RSG step leans on,
// measured on the current device (pn_measure_pipe_rates).
//
// The FP64 form of the step is bound by GB300's FP64 pipe and the FP32 and
// double-float forms by FP32 issue; how to split work between the pipes (and
// what a conversion between double and float costs) is read from these
// rates rather than assumed.  Each measurement is a throughput kernel: every
// thread runs eight independent dependency chains of one operation, a full
// grid of resident blocks keeps every scheduler busy, and the rate is
// chain-operations / CUDA-event time (best of three).  The conversions are
// inline PTX (cvt) that the compiler cannot fold; each carries two integer
// instructions that turn its result back into the next input.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdint>

namespace pn {
namespace {

constexpr int kChains = 8;
constexpr int kThreads = 256;

enum PipeOp { kDfma = 0, kDadd = 1, kFfma = 2, kCvtF64toF32 = 3, kCvtF32toF64 = 4, kIadd = 5, kOps = 6 };

__device__ __forceinline__ float cvt_f32_f64(double d) {
  float f;
  asm volatile("cvt.rn.f32.f64 %0, %1;" : "=f"(f) : "d"(d));
  return f;
}
__device__ __forceinline__ double cvt_f64_f32(float f) {
  double d;
  asm volatile("cvt.f64.f32 %0, %1;" : "=d"(d) : "f"(f));
  return d;
}

template <int OP>
__global__ void __launch_bounds__(kThreads) k_pipe(int iters, float seed, double *sink) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  double d[kChains];
  float f[kChains];
  uint32_t u[kChains];
#pragma unroll
  for (int c = 0; c < kChains; c++) {
    f[c] = seed + 1e-3f * (float)(t & 255) + 0.01f * (float)c;
    d[c] = (double)f[c];
    u[c] = (uint32_t)t * 2654435761u + (uint32_t)c;
  }
  const double da = 0.9999999, db = 1e-9;
  const float fa = 0.999999f, fb = 1e-7f;
  for (int n = 0; n < iters; n++) {
#pragma unroll
    for (int c = 0; c < kChains; c++) {
      if constexpr (OP == kDfma) d[c] = fma(d[c], da, db);
      else if constexpr (OP == kDadd) d[c] = d[c] + db;
      else if constexpr (OP == kFfma) f[c] = fmaf(f[c], fa, fb);
      else if constexpr (OP == kCvtF64toF32) {
        // f = (float)d; the next d is f's value again (positive floats: the
        // exponent rebiased, the significand moved into the high word)
        f[c] = cvt_f32_f64(d[c]);
        d[c] = __hiloint2double((__float_as_int(f[c]) >> 3) + 0x38000000, 0);
      } else if constexpr (OP == kCvtF32toF64) {
        d[c] = cvt_f64_f32(f[c]);
        f[c] = __int_as_float((__double2hiint(d[c]) - 0x38000000) << 3);
      } else {
        u[c] = (u[c] ^ 0x9e3779b9u) + (uint32_t)n;
      }
    }
  }
  double acc = 0.0;
#pragma unroll
  for (int c = 0; c < kChains; c++) acc += d[c] + (double)f[c] + (double)u[c];
  if (acc == -1.0) sink[t] = acc;  // never true: keeps the chains live
}

template <int OP>
cudaError_t time_op(int blocks, int iters, double *sink, cudaEvent_t e0, cudaEvent_t e1, float *ms) {
  k_pipe<OP><<<blocks, kThreads>>>(iters, 1.0f, sink);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  if ((e = cudaEventRecord(e0)) != cudaSuccess) return e;
  k_pipe<OP><<<blocks, kThreads>>>(iters, 1.0f, sink);
  if ((e = cudaGetLastError()) != cudaSuccess) return e;
  if ((e = cudaEventRecord(e1)) != cudaSuccess) return e;
  if ((e = cudaEventSynchronize(e1)) != cudaSuccess) return e;
  return cudaEventElapsedTime(ms, e0, e1);
}

template <int OP>
cudaError_t rate_of(int blocks, double *sink, cudaEvent_t e0, cudaEvent_t e1, double *rate) {
  // size the loop for about 10 ms, then take the best of three
  int iters = 256;
  float ms = 0.f;
  cudaError_t e = time_op<OP>(blocks, iters, sink, e0, e1, &ms);
  if (e != cudaSuccess) return e;
  const double scale = 10.0 / std::max(ms, 1e-3f);
  iters = (int)std::min(1 << 24, std::max(256, (int)(iters * scale)));
  float best = 1e30f;
  for (int r = 0; r < 3; r++) {
    if ((e = time_op<OP>(blocks, iters, sink, e0, e1, &ms)) != cudaSuccess) return e;
    best = std::min(best, ms);
  }
  *rate = (double)blocks * kThreads * (double)iters * kChains / (best * 1e-3);
  return cudaSuccess;
}

}  // namespace

cudaError_t measure_pipe_rates(double *rates, int n) {
  int dev = 0, sms = 0, per_sm = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e == cudaSuccess) e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  if (e == cudaSuccess) e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_pipe<kDfma>, kThreads, 0);
  if (e != cudaSuccess) return e;
  const int blocks = sms * std::max(per_sm, 1);
  double *sink = nullptr;
  if ((e = cudaMalloc(&sink, sizeof(double) * (size_t)blocks * kThreads)) != cudaSuccess) return e;
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  e = cudaEventCreate(&e0);
  if (e == cudaSuccess) e = cudaEventCreate(&e1);
  double r[kOps] = {};
  if (e == cudaSuccess) e = rate_of<kDfma>(blocks, sink, e0, e1, &r[kDfma]);
  if (e == cudaSuccess) e = rate_of<kDadd>(blocks, sink, e0, e1, &r[kDadd]);
  if (e == cudaSuccess) e = rate_of<kFfma>(blocks, sink, e0, e1, &r[kFfma]);
  if (e == cudaSuccess) e = rate_of<kCvtF64toF32>(blocks, sink, e0, e1, &r[kCvtF64toF32]);
  if (e == cudaSuccess) e = rate_of<kCvtF32toF64>(blocks, sink, e0, e1, &r[kCvtF32toF64]);
  if (e == cudaSuccess) e = rate_of<kIadd>(blocks, sink, e0, e1, &r[kIadd]);
  if (e0) cudaEventDestroy(e0);
  if (e1) cudaEventDestroy(e1);
  cudaFree(sink);
  if (e != cudaSuccess) return e;
  for (int k = 0; k < std::min(n, (int)kOps); k++) rates[k] = r[k];
  return cudaSuccess;
}

}  // namespace pn
