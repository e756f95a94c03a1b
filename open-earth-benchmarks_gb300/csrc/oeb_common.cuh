// oeb_common.cuh -- shared host/device pieces of the GB300 stencil library.
//
// Field layout (the reference's Storage<T,3>, include/util.h:24-31 and :82-94):
//   element (i,j,k) = aligned[offset + strides[2]*i + strides[1]*j + strides[0]*k]
// A validated field becomes a Grid view: a pointer to its interior origin (i,j,k) = (0,0,0)
// plus the row stride sj = strides[1] and the plane stride sk = strides[0]; strides[2] must
// be 1.  All 3-D fields of one call share sj and sk, so one index serves every field.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <atomic>
#include <initializer_list>

#include "../../include/oeb_gb300.h"

namespace oeb {

// ---------------------------------------------------------------------------------------
// Host side: status bookkeeping
// ---------------------------------------------------------------------------------------

// Records a CUDA error for oeb_last_cuda_error() and returns OEB_ERR_CUDA.
oeb_status cuda_fail(cudaError_t err);
// Checks the launch just made (cudaGetLastError) and counts it.
oeb_status after_launch();
void count_launches(uint64_t n);
// Launches issued while this thread captures a graph are tallied apart (recorded, not run).
void capture_count_begin();
uint64_t capture_count_end();
bool capture_counting();
// While a ValidateOnly guard is alive on this thread, entry points return after validating
// their descriptors, before any CUDA call (used by the host-buffer path to reject bad
// descriptors before it allocates or copies anything).
bool validating();
struct ValidateOnly {
  ValidateOnly();
  ~ValidateOnly();
};
#define OEB_RETURN_IF_VALIDATING() \
  do {                             \
    if (oeb::validating()) return OEB_OK; \
  } while (0)

// While a HostInPlace guard is alive on this thread, the fields the entry points receive are
// host memory the device reads in place (the host entry points' direct mode); the kernels that
// stage their tiles with cp.async then keep to ordinary loads, which are what that mode was
// measured and tested with.
bool fields_in_host_memory();
struct HostInPlace {
  HostInPlace();
  ~HostInPlace();
};

// Raises a kernel's dynamic shared-memory limit to `bytes` on the current device, once per
// (kernel, device); thread-safe.
oeb_status ensure_dyn_smem(const void* kernel, int bytes);
// The library's stream-ordered device memory pool for the current device.
oeb_status device_pool(cudaMemPool_t* out);

#define OEB_TRY(expr)                   \
  do {                                  \
    oeb_status _st = (expr);            \
    if (_st != OEB_OK) return _st;      \
  } while (0)

#define OEB_CUDA_TRY(expr)                         \
  do {                                             \
    cudaError_t _e = (expr);                       \
    if (_e != cudaSuccess) return oeb::cuda_fail(_e); \
  } while (0)

// ---------------------------------------------------------------------------------------
// Host side: descriptor validation
// ---------------------------------------------------------------------------------------

// Cells a kernel touches beyond the interior [0,nx) x [0,ny) x [0,nz), per side.  For inputs
// this is the read reach, for outputs the written box.
struct Reach {
  int ilo, ihi, jlo, jhi, klo, khi;
};
constexpr Reach kInterior{0, 0, 0, 0, 0, 0};

// Validated view of one 3-D field.
template <class T>
struct Grid {
  T* origin;      // address of (0,0,0)
  int64_t sj;     // strides[1]
  int64_t sk;     // strides[0]
  const char* lo; // first byte touched
  const char* hi; // one past the last byte touched
};

// Validated view of one 1-D (per-latitude, indexed by j) field.
template <class T>
struct Line {
  const T* origin;
  int64_t s;
  const char* lo;
  const char* hi;
};

oeb_status check_domain(const oeb_domain* dom);

template <class T, class M>
oeb_status check_field3(const M* m, const oeb_domain& d, const Reach& r, Grid<T>* g);

// While a ReachLog is installed on the calling thread, check_field3 records the reach each
// 3-D descriptor is validated against (the host entry points learn from it which k-planes of
// an input the kernel reads, and copy only those).
struct ReachLog {
  static constexpr int kMax = 32;
  const void* desc[kMax];
  Reach reach[kMax];
  int n = 0;
  // the reach recorded for `m` (the union if it was validated more than once), or false
  bool find(const void* m, Reach* out) const;
};
void set_reach_log(ReachLog* log);
template <class T, class M>
oeb_status check_field1(const M* m, const oeb_domain& d, int jlo, int jhi, Line<T>* l);

// All 3-D fields of one call must share (sj, sk).
template <class T>
oeb_status check_same_strides(std::initializer_list<const Grid<T>*> grids);
// No output may overlap another output or any input.
oeb_status check_no_alias(std::initializer_list<const char*> out_ranges, std::initializer_list<const char*> in_ranges);

template <class T>
inline const char* lo_of(const Grid<T>& g) { return g.lo; }

// ---------------------------------------------------------------------------------------
// Device side
// ---------------------------------------------------------------------------------------

// Interior extents and the shared strides, passed by value to every kernel.
struct Dims {
  int nx, ny, nz;
  int64_t sj, sk;
};

}  // namespace oeb
