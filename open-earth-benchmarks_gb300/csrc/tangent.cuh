// tangent.cuh -- running a stencil kernel on dual numbers: the tangent-linear entry points.
//
// oeb_<k>_tl_<f64|f32>(dy..., x..., dx..., scalars) computes dy = J(x) dx, the stencil's
// Jacobian at the state x applied to the perturbation dx of its active inputs, with every
// branch frozen at x.  The kernel is the forward kernel instantiated with Dual<T>:
//   1. each input field is packed into a Dual array in the field's own layout (value from x,
//      derivative from dx for active inputs, 0 for parameters), in device scratch
//      (scratch_alloc: the stream-ordered pool, or a batch plan's arena);
//   2. the forward kernel runs on the Dual arrays;
//   3. the derivative part of each output is copied to dy over the output's written box.
// Scratch is returned to the pool on every exit path.
#pragma once

#include <algorithm>
#include <vector>

#include "dual.cuh"
#include "oeb_common.cuh"
#include "stencil_util.cuh"

namespace oeb {

constexpr int kFlatThreads = kTX * kTY;

template <class T>
struct pack_dual_kernel {
  static __device__ __forceinline__ void run(const uint3& blk, Dual<T>* __restrict__ out, const T* __restrict__ v,
                                             const T* __restrict__ d, int64_t n) {
    const int64_t e = (int64_t)blk.x * kFlatThreads + threadIdx.y * kTX + threadIdx.x;
    if (e < n) out[e] = Dual<T>(v[e], d ? d[e] : T(0));
  }
};

// dy(box) = derivative part of y(box); box = [-ilo, nx+ihi) x [-jlo, ny+jhi) x [-klo, nz+khi)
template <class T>
struct unpack_deriv_kernel {
  static __device__ __forceinline__ void run(const uint3& blk, T* __restrict__ dy, const Dual<T>* __restrict__ y,
                                             int ni, int nj, int nk, int64_t sj, int64_t sk) {
    const int64_t n = (int64_t)ni * nj * nk;
    const int64_t e = (int64_t)blk.x * kFlatThreads + threadIdx.y * kTX + threadIdx.x;
    if (e >= n) return;
    const int64_t i = e % ni, r = e / ni, j = r % nj, k = r / nj;
    const int64_t o = i + j * sj + k * sk;
    dy[o] = y[o].d;
  }
};

inline dim3 flat_grid(int64_t n) { return dim3((unsigned)((n + kFlatThreads - 1) / kFlatThreads)); }

// Device scratch of one tangent-linear call.
template <class T>
class DualArrays {
 public:
  explicit DualArrays(cudaStream_t s) : s_(s) {}
  ~DualArrays() {
    for (void* p : bufs_) scratch_free(p, s_);
  }

  // Dual copy of the field described by `x` (derivative from `dx` if given, else 0), in
  // x's layout; returns the address of the Dual at x's interior origin.
  template <class M>
  oeb_status pack(const M* x, const M* dx, Dual<T>** origin) {
    const T* start = (x->allocated && x->allocated <= x->aligned) ? x->allocated : x->aligned;
    int64_t last = 0;
    for (size_t r = 0; r < sizeof(x->sizes) / sizeof(x->sizes[0]); ++r) last += (x->sizes[r] - 1) * x->strides[r];
    const int64_t n = (int64_t)(x->aligned - start) + last + 1;
    if (dx) {
      for (size_t r = 0; r < sizeof(x->sizes) / sizeof(x->sizes[0]); ++r)
        if (dx->sizes[r] != x->sizes[r] || dx->strides[r] != x->strides[r]) return OEB_ERR_LAYOUT;
      if (dx->offset != x->offset || (dx->aligned - dx->allocated) != (x->aligned - x->allocated))
        return OEB_ERR_LAYOUT;
    }
    void* buf = nullptr;
    OEB_TRY(scratch_alloc(&buf, (size_t)n * sizeof(Dual<T>), s_));
    bufs_.push_back(buf);
    Dual<T>* base = static_cast<Dual<T>*>(buf);
    const T* dstart = dx ? ((dx->allocated && dx->allocated <= dx->aligned) ? dx->allocated : dx->aligned) : nullptr;
    OEB_TRY(launch<pack_dual_kernel<T>>(flat_grid(n), 0, s_, base, start, dstart, n));
    *origin = base + (x->aligned - start) + x->offset;
    return OEB_OK;
  }

  // Uninitialised Dual array in y's layout, for an output.
  template <class M>
  oeb_status alloc(const M* y, Dual<T>** origin) {
    return pack_impl_alloc(y, origin);
  }

  // dy over `box` from the derivative part of the Dual output at `origin`.
  oeb_status unpack(T* dy_origin, const Dual<T>* origin, const oeb_domain& d, const Reach& r, int64_t sj,
                    int64_t sk) {
    const int ni = (int)(d.nx + r.ilo + r.ihi), nj = (int)(d.ny + r.jlo + r.jhi), nk = (int)(d.nz + r.klo + r.khi);
    const int64_t first = -(int64_t)r.ilo - (int64_t)r.jlo * sj - (int64_t)r.klo * sk;
    const int64_t n = (int64_t)ni * nj * nk;
    return launch<unpack_deriv_kernel<T>>(flat_grid(n), 0, s_, dy_origin + first, origin + first, ni, nj, nk, sj, sk);
  }

 private:
  template <class M>
  oeb_status pack_impl_alloc(const M* y, Dual<T>** origin) {
    const T* start = (y->allocated && y->allocated <= y->aligned) ? y->allocated : y->aligned;
    int64_t last = 0;
    for (size_t r = 0; r < 3; ++r) last += (y->sizes[r] - 1) * y->strides[r];
    const int64_t n = (int64_t)(y->aligned - start) + last + 1;
    void* buf = nullptr;
    OEB_TRY(scratch_alloc(&buf, (size_t)n * sizeof(Dual<T>), s_));
    bufs_.push_back(buf);
    *origin = static_cast<Dual<T>*>(buf) + (y->aligned - start) + y->offset;
    return OEB_OK;
  }

  cudaStream_t s_;
  std::vector<void*> bufs_;
};

}  // namespace oeb
