// selftest.cu -- oeb_selftest_fp64: the integer-pipe FP64 multiply, division, addition,
// subtraction and square root (precision.cuh: fp64::mul, div, add, isub, sqrt) against the
// FP64 instructions on seeded random operands, on the device; and two measurements of the
// GPU the design rests on: the FP64 pipe's addition rate (oeb_probe_fp64_add_rate) and
// i-neighbours read through L1 against warp shuffles (oeb_probe_shuffle_neighbours).
#include <cuda_runtime.h>
#include <stdint.h>
#include <string.h>

#include <vector>

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

// The same for each FP64 operation the stencils use (oeb_probe_fp64_rate): OP 0 addition, 1
// multiplication, 2 fused multiply-add, 3 division, 4 square root (the division and the square
// root are the compiler's instruction sequences).  The operands keep every chain finite and
// normal.
template <int OP>
__global__ void fp64_op_rate_kernel(int iters, double step, double* sink) {
  double x[kChains];
#pragma unroll
  for (int c = 0; c < kChains; ++c) x[c] = 1.0 + 0.125 * (double)(threadIdx.x + c);
#pragma unroll 1
  for (int i = 0; i < iters; ++i) {
#pragma unroll
    for (int c = 0; c < kChains; ++c) {
      if (OP == 0) x[c] = __dadd_rn(x[c], step);
      if (OP == 1) x[c] = __dmul_rn(x[c], 1.0 + step);
      if (OP == 2) x[c] = __fma_rn(x[c], 1.0 - step, step);
      if (OP == 3) x[c] = __ddiv_rn(x[c], 1.0 + step);
      if (OP == 4) x[c] = __dsqrt_rn(x[c] + 1.0);
    }
  }
  double t = 0.0;
#pragma unroll
  for (int c = 0; c < kChains; ++c) t = __dadd_rn(t, x[c]);
  if (t == -1.0) sink[blockIdx.x] = t;  // never true for these operands
}

// ---- i-neighbours through L1 or through warp shuffles (oeb_probe_shuffle_neighbours) --
// FP32 fields of a 256 x 256 x 80 interior with a 3-cell halo, one CTA of 32 x 8 threads a
// 32 x 32 tile and k-level, four rows a thread.
constexpr int kPNX = 256, kPNY = 256, kPNZ = 80, kPH = 3;
constexpr int kPSX = kPNX + 2 * kPH, kPSY = kPNY + 2 * kPH;
constexpr long kPSK = (long)kPSX * kPSY;
constexpr size_t kPCells = (size_t)kPSK * (kPNZ + 2 * kPH);

__device__ __forceinline__ long probe_offset(int i, int j, int k) {
  return (long)(k + kPH) * kPSK + (long)(j + kPH) * kPSX + i + kPH;
}

// the 5-point laplacian, its i-neighbours loaded (through L1)
__global__ void probe_lap_l1(const float* __restrict__ in, float* __restrict__ out) {
  const int i = blockIdx.x * 32 + threadIdx.x, k = blockIdx.z;
  for (int r = 0; r < 4; ++r) {
    const long o = probe_offset(i, blockIdx.y * 32 + threadIdx.y + 8 * r, k);
    const float c = __ldg(in + o);
    out[o] = ((__ldg(in + o - 1) - c) + (__ldg(in + o + 1) - c)) + ((__ldg(in + o + kPSX) - c) + (__ldg(in + o - kPSX) - c));
  }
}

// the same, its i-neighbours shuffled from the adjacent lanes; lanes 0 and 31 load the
// warp's two outer cells
__global__ void probe_lap_shfl(const float* __restrict__ in, float* __restrict__ out) {
  const int lane = threadIdx.x, i = blockIdx.x * 32 + lane, k = blockIdx.z;
  for (int r = 0; r < 4; ++r) {
    const long o = probe_offset(i, blockIdx.y * 32 + threadIdx.y + 8 * r, k);
    const float c = __ldg(in + o);
    const float e = (lane == 0 || lane == 31) ? __ldg(in + o + (lane == 0 ? -1 : 1)) : 0.f;
    float w = __shfl_up_sync(0xffffffffu, c, 1), x = __shfl_down_sync(0xffffffffu, c, 1);
    const float e0 = __shfl_sync(0xffffffffu, e, 0), e31 = __shfl_sync(0xffffffffu, e, 31);
    if (lane == 0) w = e0;
    if (lane == 31) x = e31;
    out[o] = ((w - c) + (x - c)) + ((__ldg(in + o + kPSX) - c) + (__ldg(in + o - kPSX) - c));
  }
}

// a 7-cell window along i (the shape of the fifth-order advection sums), loaded
__device__ __constant__ float kProbeCoef[7] = {1.f / 30, -0.25f, 1.f, -1.f / 3, -0.5f, 1.f / 20, 0.1f};
__global__ void probe_win_l1(const float* __restrict__ in, float* __restrict__ out) {
  const int i = blockIdx.x * 32 + threadIdx.x, k = blockIdx.z;
  for (int r = 0; r < 4; ++r) {
    const long o = probe_offset(i, blockIdx.y * 32 + threadIdx.y + 8 * r, k);
    float s = 0.f;
#pragma unroll
    for (int d = -3; d <= 3; ++d) s = s + kProbeCoef[d + 3] * __ldg(in + o + d);
    out[o] = s;
  }
}

// the same window shuffled: lane l holds cells i0-3+l and (l < 6) i0+29+l of its row
__global__ void probe_win_shfl(const float* __restrict__ in, float* __restrict__ out) {
  const int lane = threadIdx.x, k = blockIdx.z;
  for (int r = 0; r < 4; ++r) {
    const long row = probe_offset(blockIdx.x * 32, blockIdx.y * 32 + threadIdx.y + 8 * r, k);
    const float a = __ldg(in + row - 3 + lane);
    const float b = lane < 6 ? __ldg(in + row + 29 + lane) : 0.f;
    float s = 0.f;
#pragma unroll
    for (int d = -3; d <= 3; ++d) {
      const int src = lane + d + 3;
      const float va = __shfl_sync(0xffffffffu, a, src & 31);
      const float vb = __shfl_sync(0xffffffffu, b, (src - 32) & 31);
      s = s + kProbeCoef[d + 3] * (src < 32 ? va : vb);
    }
    out[row + lane] = s;
  }
}

}  // namespace
}  // namespace oeb

extern "C" oeb_status oeb_probe_shuffle_neighbours(double* us, uint64_t* mismatches) {
  if (!us || !mismatches) return OEB_ERR_NULL;
  using namespace oeb;
  constexpr int kCopies = 12;  // 12 input copies of 23.6 MB: more than the L2, launches rotate over them
  float *in = nullptr, *o1 = nullptr, *o2 = nullptr;
  cudaError_t e = cudaMalloc(&in, kPCells * sizeof(float) * kCopies);
  if (e == cudaSuccess) e = cudaMalloc(&o1, kPCells * sizeof(float));
  if (e == cudaSuccess) e = cudaMalloc(&o2, kPCells * sizeof(float));
  std::vector<float> h(kPCells), r1, r2;
  uint64_t x = 0x243F6A8885A308D3ull;
  for (float& v : h) {  // xorshift values in [0, 1)
    x ^= x << 13;
    x ^= x >> 7;
    x ^= x << 17;
    v = (float)(x >> 40) / (float)(1u << 24);
  }
  for (int c = 0; c < kCopies && e == cudaSuccess; ++c)
    e = cudaMemcpy(in + c * kPCells, h.data(), kPCells * sizeof(float), cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaMemset(o1, 0, kPCells * sizeof(float));
  if (e == cudaSuccess) e = cudaMemset(o2, 0, kPCells * sizeof(float));
  const dim3 grid(kPNX / 32, kPNY / 32, kPNZ), block(32, 8);
  using Kern = void (*)(const float*, float*);
  const Kern pairs[2][2] = {{probe_lap_l1, probe_lap_shfl}, {probe_win_l1, probe_win_shfl}};
  // the two forms of each stencil give the same bits
  for (int p = 0; p < 2 && e == cudaSuccess; ++p) {
    pairs[p][0]<<<grid, block>>>(in, o1);
    pairs[p][1]<<<grid, block>>>(in, o2);
    count_launches(2);
    e = cudaDeviceSynchronize();
    r1.resize(kPCells);
    r2.resize(kPCells);
    if (e == cudaSuccess) e = cudaMemcpy(r1.data(), o1, kPCells * sizeof(float), cudaMemcpyDeviceToHost);
    if (e == cudaSuccess) e = cudaMemcpy(r2.data(), o2, kPCells * sizeof(float), cudaMemcpyDeviceToHost);
    uint64_t bad = 0;
    for (size_t q = 0; q < kPCells; ++q) bad += memcmp(&r1[q], &r2[q], sizeof(float)) != 0;
    mismatches[p] = bad;
  }
  // each form: the best of three averages over 60 back-to-back launches, after 5 warm-up launches
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  if (e == cudaSuccess) e = cudaEventCreate(&e0);
  if (e == cudaSuccess) e = cudaEventCreate(&e1);
  for (int f = 0; f < 4 && e == cudaSuccess; ++f) {
    const Kern kern = pairs[f / 2][f % 2];
    float best = 0.f;
    for (int rep = 0; rep < 3 && e == cudaSuccess; ++rep) {
      for (int w = 0; w < 5; ++w) kern<<<grid, block>>>(in + (w % kCopies) * kPCells, o1);
      cudaEventRecord(e0, 0);
      for (int r = 0; r < 60; ++r) kern<<<grid, block>>>(in + (r % kCopies) * kPCells, o1);
      cudaEventRecord(e1, 0);
      count_launches(65);
      e = cudaEventSynchronize(e1);
      float ms = 0.f;
      if (e == cudaSuccess) cudaEventElapsedTime(&ms, e0, e1);
      if (best == 0.f || ms < best) best = ms;
    }
    us[f] = best / 60.0 * 1e3;
  }
  if (e0) cudaEventDestroy(e0);
  if (e1) cudaEventDestroy(e1);
  cudaFree(in);
  cudaFree(o1);
  cudaFree(o2);
  return e == cudaSuccess ? OEB_OK : cuda_fail(e);
}

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

extern "C" oeb_status oeb_probe_fp64_rate(int op, double* ops_per_second, double* ops_per_launch) {
  if (!ops_per_second) return OEB_ERR_NULL;
  if (op < 0 || op > 4) return OEB_ERR_ARGUMENT;
  using Kern = void (*)(int, double, double*);
  const Kern kerns[5] = {oeb::fp64_op_rate_kernel<0>, oeb::fp64_op_rate_kernel<1>, oeb::fp64_op_rate_kernel<2>,
                         oeb::fp64_op_rate_kernel<3>, oeb::fp64_op_rate_kernel<4>};
  int dev = 0, sms = 1;
  OEB_CUDA_TRY(cudaGetDevice(&dev));
  OEB_CUDA_TRY(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
  // the division and the square root are sequences of several instructions: fewer iterations
  const int ctas = sms * 8, threads = 256, iters = op >= 3 ? 1 << 11 : 1 << 14;
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  OEB_CUDA_TRY(cudaEventCreate(&e0));
  cudaError_t e = cudaEventCreate(&e1);
  float best = 0.f;
  for (int rep = 0; rep < 4 && e == cudaSuccess; ++rep) {  // the first launch is the warm-up
    cudaEventRecord(e0, 0);
    kerns[op]<<<ctas, threads>>>(iters, 1.0 / 1024.0, nullptr);
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
  const double ops = (double)ctas * threads * iters * oeb::kChains;
  *ops_per_second = best > 0.f ? ops / (best * 1e-3) : 0.0;
  if (ops_per_launch) *ops_per_launch = ops;
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
