// selftest.cu -- oeb_selftest_fp64: the integer-pipe FP64 multiply, division, addition,
// subtraction and square root (precision.cuh: fp64::mul, div, add, isub, sqrt) against the
// FP64 instructions on seeded random operands, on the device.
#include <cuda_runtime.h>
#include <stdint.h>

#include "oeb_common.cuh"
#include "precision.cuh"

namespace oeb {
namespace {

__device__ __forceinline__ uint64_t splitmix(uint64_t x) {
  x += 0x9E3779B97F4A7C15ull;
  x = (x ^ (x >> 30)) * 0xBF58476D1CE4E5B9ull;
  x = (x ^ (x >> 27)) * 0x94D049BB133111EBull;
  return x ^ (x >> 31);
}

// One operand of distribution `mode` from the hash h.
__device__ double operand(uint64_t h, int mode) {
  uint64_t m = h & 0xFFFFFFFFFFFFFull;
  const uint64_t sign = h & 0x8000000000000000ull;
  const uint64_t g = splitmix(h);
  uint64_t e;
  switch (mode) {
    case 0:
      return __longlong_as_double((long long)h);
    case 1:
      e = 1023 - 40 + g % 81;
      break;
    case 2:
      e = (g & 1) ? 1 + (g >> 1) % 60 : 2046 - (g >> 1) % 60;
      break;
    case 3:
      e = 1 + g % 2046;
      m &= ~((1ull << ((g >> 40) % 52)) - 1);
      break;
    default:
      e = 1023 - 5 + g % 11;
      m = (g & 4) ? (m | 0xFFFFF00000000ull) : (m & 0xFF);
      break;
  }
  return __longlong_as_double((long long)(sign | (e << 52) | m));
}

__global__ void selftest_kernel(int op, uint64_t seed, int64_t n, int mode, unsigned long long* bad,
                                unsigned long long* first) {
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < n; t += stride) {
    const uint64_t h = splitmix(seed ^ (uint64_t)t);
    double a, b;
    if (mode == 5 && op == 4) {  // exact squares
      const double q = (double)(1 + h % 100000000);
      a = __dmul_rn(q, q);
      b = 0.0;
    } else if (mode == 5) {  // b times a small integer over b: exact quotients and quotients near 1
      b = operand(splitmix(h + 17), 1);
      a = __dmul_rn(b, (double)(1 + h % 1000));
    } else if (mode == 6) {  // a + (-a (1 + small)): cancellation of all but a few bits
      a = operand(h, 1);
      b = -__dmul_rn(a, 1.0 + ldexp((double)(h % 1024), -52 + (int)(h % 7)));
    } else if (mode == 7) {  // b = a 2^-k with its low bits changed: every alignment shift
      a = operand(h, 1);
      const double s2 = ldexp(a, -(int)(splitmix(h) % 70));
      b = __longlong_as_double(__double_as_longlong((h & 1) ? -s2 : s2) ^ (long long)(splitmix(h + 3) & 0xFF));
    } else {
      a = operand(h, mode);
      b = operand(splitmix(h + 17), mode);
    }
    double want, got;
    switch (op) {
      case 0: want = __dmul_rn(a, b); got = fp64::mul(a, b); break;
      case 1: want = __ddiv_rn(a, b); got = fp64::div(a, b); break;
      case 2: want = __dadd_rn(a, b); got = fp64::add(a, b); break;
      case 3: want = __dsub_rn(a, b); got = isub(F64i(a), F64i(b)).v; break;
      default: want = __dsqrt_rn(a); got = fp64::sqrt(a); break;
    }
    const unsigned long long bw = (unsigned long long)__double_as_longlong(want);
    const unsigned long long bg = (unsigned long long)__double_as_longlong(got);
    if (bw != bg && !(want != want && got != got)) {
      if (atomicAdd(bad, 1ull) == 0ull) {
        first[0] = (unsigned long long)__double_as_longlong(a);
        first[1] = (unsigned long long)__double_as_longlong(b);
        first[2] = bw;
        first[3] = bg;
      }
    }
  }
}

// The FP64 pipe's issue rate: every thread runs kChains independent chains of FP64 additions
// (each addition waits only for the one before it in its chain), enough warps to fill every SM.
// The sum is stored where nothing reads it only if it is an impossible value, so that the
// additions are not removed.
constexpr int kChains = 8;
__global__ void fp64_add_rate_kernel(int iters, double step, double* sink) {
  double x[kChains];
#pragma unroll
  for (int c = 0; c < kChains; ++c) x[c] = (double)(threadIdx.x + c);
#pragma unroll 1
  for (int i = 0; i < iters; ++i) {
#pragma unroll
    for (int c = 0; c < kChains; ++c) x[c] = __dadd_rn(x[c], step);
  }
  double t = 0.0;
#pragma unroll
  for (int c = 0; c < kChains; ++c) t = __dadd_rn(t, x[c]);
  if (t == -1.0) sink[blockIdx.x] = t;  // never true for these operands
}

}  // namespace
}  // namespace oeb

extern "C" oeb_status oeb_probe_fp64_add_rate(double* adds_per_second, double* adds_per_launch) {
  if (!adds_per_second) return OEB_ERR_NULL;
  int dev = 0, sms = 1;
  OEB_CUDA_TRY(cudaGetDevice(&dev));
  OEB_CUDA_TRY(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
  const int ctas = sms * 8, threads = 256, iters = 1 << 14;
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  OEB_CUDA_TRY(cudaEventCreate(&e0));
  cudaError_t e = cudaEventCreate(&e1);
  float best = 0.f;
  for (int rep = 0; rep < 4 && e == cudaSuccess; ++rep) {  // the first launch is the warm-up
    cudaEventRecord(e0, 0);
    oeb::fp64_add_rate_kernel<<<ctas, threads>>>(iters, 0.5, nullptr);
    e = cudaGetLastError();
    if (e != cudaSuccess) break;
    oeb::count_launches(1);
    cudaEventRecord(e1, 0);
    e = cudaEventSynchronize(e1);
    float ms = 0.f;
    if (e == cudaSuccess) cudaEventElapsedTime(&ms, e0, e1);
    if (rep > 0 && (best == 0.f || ms < best)) best = ms;
  }
  cudaEventDestroy(e0);
  if (e1) cudaEventDestroy(e1);
  if (e != cudaSuccess) return oeb::cuda_fail(e);
  const double adds = (double)ctas * threads * iters * oeb::kChains;
  *adds_per_second = best > 0.f ? adds / (best * 1e-3) : 0.0;
  if (adds_per_launch) *adds_per_launch = adds;
  return OEB_OK;
}

extern "C" oeb_status oeb_selftest_fp64(int op, int64_t pairs, uint64_t seed, int mode, uint64_t* mismatches,
                                        uint64_t* first) {
  if (!mismatches) return OEB_ERR_NULL;
  if (op < 0 || op > 4 || pairs < 0 || mode < 0 || mode > 7) return OEB_ERR_ARGUMENT;
  unsigned long long* d = nullptr;
  OEB_CUDA_TRY(cudaMalloc(&d, 5 * sizeof(unsigned long long)));
  cudaError_t e = cudaMemset(d, 0, 5 * sizeof(unsigned long long));
  if (e == cudaSuccess && pairs > 0) {
    int dev = 0, sms = 1;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    oeb::selftest_kernel<<<sms * 8, 256>>>(op, seed, pairs, mode, d, d + 1);
    e = cudaGetLastError();
    if (e == cudaSuccess) oeb::count_launches(1);
  }
  unsigned long long h[5] = {0, 0, 0, 0, 0};
  if (e == cudaSuccess) e = cudaMemcpy(h, d, sizeof(h), cudaMemcpyDeviceToHost);
  cudaFree(d);
  if (e != cudaSuccess) return oeb::cuda_fail(e);
  *mismatches = h[0];
  if (first)
    for (int i = 0; i < 4; ++i) first[i] = h[1 + i];
  return OEB_OK;
}
