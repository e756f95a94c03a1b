// abi_common.cu -- status strings, error bookkeeping, descriptor validation and device
// storage allocation for the C ABI declared in include/oeb_gb300.h.
#include <stdio.h>
#include <string.h>

#include <algorithm>
#include <atomic>
#include <limits>
#include <mutex>
#include <set>
#include <utility>
#include <vector>

#include "oeb_common.cuh"
#include "launch.cuh"
#include "stage.cuh"

namespace oeb {

namespace {
thread_local char g_last_cuda_error[256] = "";
thread_local int g_validate_only = 0;
thread_local ReachLog* t_reach_log = nullptr;
std::atomic<uint64_t> g_launches{0};
}  // namespace

bool validating() { return g_validate_only > 0; }
void set_reach_log(ReachLog* log) { t_reach_log = log; }

bool ReachLog::find(const void* m, Reach* out) const {
  bool found = false;
  for (int q = 0; q < n; ++q) {
    if (desc[q] != m) continue;
    const Reach& r = reach[q];
    if (!found) {
      *out = r;
    } else {
      out->ilo = std::max(out->ilo, r.ilo), out->ihi = std::max(out->ihi, r.ihi);
      out->jlo = std::max(out->jlo, r.jlo), out->jhi = std::max(out->jhi, r.jhi);
      out->klo = std::max(out->klo, r.klo), out->khi = std::max(out->khi, r.khi);
    }
    found = true;
  }
  return found;
}
ValidateOnly::ValidateOnly() { ++g_validate_only; }
ValidateOnly::~ValidateOnly() { --g_validate_only; }

oeb_status cuda_fail(cudaError_t err) {
  snprintf(g_last_cuda_error, sizeof(g_last_cuda_error), "%s: %s", cudaGetErrorName(err), cudaGetErrorString(err));
  return OEB_ERR_CUDA;
}

namespace {
// Launches issued by this thread while it captures a graph: recorded, not run.
thread_local bool t_capturing = false;
thread_local uint64_t t_captured = 0;
}  // namespace

void count_launches(uint64_t n) {
  if (t_capturing)
    t_captured += n;
  else
    g_launches.fetch_add(n, std::memory_order_relaxed);
}
void capture_count_begin() {
  t_capturing = true;
  t_captured = 0;
}
uint64_t capture_count_end() {
  t_capturing = false;
  return t_captured;
}
bool capture_counting() { return t_capturing; }

namespace {
thread_local Recorder* t_recorder = nullptr;
std::atomic<int> g_kb_override{0};
}  // namespace

int kb_override() { return g_kb_override.load(std::memory_order_relaxed); }

namespace {
std::atomic<int> g_shape_override{0};
}  // namespace
int shape_override() { return g_shape_override.load(std::memory_order_relaxed); }
std::atomic<int> g_fusion_override{OEB_FUSE_HADV_UPDATE};  // oeb_set_fusion
std::atomic<int> g_adjoint_tiles{1};
int adjoint_tiles() { return g_adjoint_tiles.load(std::memory_order_relaxed); }
int fusion_override() { return g_fusion_override.load(std::memory_order_relaxed); }

namespace {
thread_local int t_host_in_place = 0;
}  // namespace
bool fields_in_host_memory() { return t_host_in_place > 0; }
HostInPlace::HostInPlace() { ++t_host_in_place; }
HostInPlace::~HostInPlace() { --t_host_in_place; }

// SMs of each device, read once (cudaDevAttrMultiProcessorCount); 0 until read.
namespace {
constexpr int kMaxDevices = 64;
std::atomic<int> g_sms[kMaxDevices];
}  // namespace

int staged_kb(int tiles, int nz, int ctas_per_sm) {
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0) dev = 0;
  int sms = dev < kMaxDevices ? g_sms[dev].load(std::memory_order_relaxed) : 0;
  if (sms < 1) {
    if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || sms < 1) sms = 1;
    if (dev < kMaxDevices) g_sms[dev].store(sms, std::memory_order_relaxed);
  }
  // the most k-chunks per tile that still fit every CTA into one wave, then levels per chunk
  const long slots = (long)sms * (ctas_per_sm > 0 ? ctas_per_sm : 1);
  long chunks = tiles > 0 ? slots / tiles : 1;
  if (chunks < 1) chunks = 1;
  if (chunks > nz) chunks = nz;
  const long kb = (nz + chunks - 1) / (chunks > 0 ? chunks : 1);
  return (int)(kb < 1 ? 1 : kb);
}

Recorder* recorder() { return t_recorder; }
void set_recorder(Recorder* r) { t_recorder = r; }

oeb_status scratch_alloc(void** p, size_t bytes, cudaStream_t st) {
  *p = nullptr;
  if (Recorder* r = t_recorder) {
    const size_t at = (r->used + 255) & ~size_t(255);
    if (r->arena && at + bytes > r->arena_bytes) return OEB_ERR_TOO_LARGE;
    // sizing pass: placeholder addresses, never dereferenced (nothing is launched)
    *p = r->arena ? static_cast<void*>(r->arena + at) : reinterpret_cast<void*>(uintptr_t(4096) + at);
    r->live.push_back({at, false});
    r->used = at + bytes;
    if (r->used > r->peak) r->peak = r->used;
    return OEB_OK;
  }
  cudaMemPool_t pool;
  OEB_TRY(device_pool(&pool));
  const cudaError_t e = cudaMallocFromPoolAsync(p, bytes, pool, st);
  if (e != cudaSuccess) {
    cuda_fail(e);
    return OEB_ERR_ALLOC;
  }
  return OEB_OK;
}

void scratch_free(void* p, cudaStream_t st) {
  if (!p) return;
  if (Recorder* r = t_recorder) {
    const uintptr_t base = r->arena ? reinterpret_cast<uintptr_t>(r->arena) : uintptr_t(4096);
    const size_t at = reinterpret_cast<uintptr_t>(p) - base;
    for (auto& a : r->live)
      if (a.first == at) a.second = true;
    while (!r->live.empty() && r->live.back().second) {
      r->used = r->live.back().first;
      r->live.pop_back();
    }
    return;
  }
  cudaFreeAsync(p, st);
}

oeb_status after_launch() {
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return cuda_fail(e);
  count_launches(1);
  return OEB_OK;
}

oeb_status ensure_dyn_smem(const void* kernel, int bytes) {
  static std::mutex mu;
  static std::set<std::pair<const void*, int>> done;
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return cuda_fail(e);
  std::lock_guard<std::mutex> lock(mu);
  if (done.count({kernel, dev})) return OEB_OK;
  e = cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
  if (e != cudaSuccess) return cuda_fail(e);
  done.insert({kernel, dev});
  return OEB_OK;
}

// One stream-ordered memory pool per device for the library's own scratch (host staging,
// tangent-linear dual arrays), kept for the life of the process with the release threshold
// at the maximum so repeated calls reuse the same device memory.
oeb_status device_pool(cudaMemPool_t* out) {
  static std::mutex mu;
  static std::vector<cudaMemPool_t> pools;
  int dev = 0;
  OEB_CUDA_TRY(cudaGetDevice(&dev));
  std::lock_guard<std::mutex> lock(mu);
  if ((int)pools.size() <= dev) pools.resize(dev + 1, nullptr);
  if (!pools[dev]) {
    cudaMemPoolProps props = {};
    props.allocType = cudaMemAllocationTypePinned;
    props.location.type = cudaMemLocationTypeDevice;
    props.location.id = dev;
    cudaMemPool_t p = nullptr;
    OEB_CUDA_TRY(cudaMemPoolCreate(&p, &props));
    uint64_t threshold = ~0ull;
    OEB_CUDA_TRY(cudaMemPoolSetAttribute(p, cudaMemPoolAttrReleaseThreshold, &threshold));
    // memory freed on one stream is never reused by an allocation on another through an
    // inserted dependency (the pool grows instead): asynchronous host calls allocate on the
    // copy-in stream and free on the caller's, and must not serialise the two
    int no = 0;
    OEB_CUDA_TRY(cudaMemPoolSetAttribute(p, cudaMemPoolReuseAllowInternalDependencies, &no));
    pools[dev] = p;
  }
  *out = pools[dev];
  return OEB_OK;
}

oeb_status check_domain(const oeb_domain* dom) {
  if (!dom) return OEB_ERR_NULL;
  const int64_t lim = std::numeric_limits<int32_t>::max() / 2;
  if (dom->nx < 1 || dom->ny < 1 || dom->nz < 1) return OEB_ERR_DOMAIN;
  if (dom->nx > lim || dom->ny > lim || dom->nz > lim) return OEB_ERR_DOMAIN;
  return OEB_OK;
}

// A descriptor is accepted when strides[2] == 1, rows do not overlap
// (strides[1] >= sizes[2]) and planes do not overlap (strides[0] >= strides[1]*sizes[1]).
// Its offset then splits uniquely into the halo widths hk*strides[0] + hj*strides[1] + hi,
// as allocateStorage builds it (include/util.h:136).  The required box must lie inside
// [-h, size-h) on each axis.
template <class T, class M>
oeb_status check_field3(const M* m, const oeb_domain& d, const Reach& r, Grid<T>* g) {
  if (!m || !m->aligned) return OEB_ERR_NULL;
  if (reinterpret_cast<uintptr_t>(m->aligned) % alignof(T) != 0) return OEB_ERR_ALIGNMENT;
  const int64_t szk = m->sizes[0], szj = m->sizes[1], szi = m->sizes[2];
  const int64_t sk = m->strides[0], sj = m->strides[1], si = m->strides[2];
  if (si != 1) return OEB_ERR_LAYOUT;
  if (szi < 1 || szj < 1 || szk < 1) return OEB_ERR_LAYOUT;
  if (sj < szi || sk < sj * szj) return OEB_ERR_LAYOUT;
  // 32-bit in-plane index arithmetic in the kernels.
  if (sk > std::numeric_limits<int32_t>::max()) return OEB_ERR_DOMAIN;
  if (m->offset < 0) return OEB_ERR_HALO;
  const int64_t hk = m->offset / sk;
  const int64_t rem = m->offset % sk;
  const int64_t hj = rem / sj;
  const int64_t hi = rem % sj;
  if (hi >= szi || hj >= szj || hk >= szk) return OEB_ERR_HALO;
  // box [-lo, n-1+hi] on each axis must fit in [-h, size-h-1]
  if (r.ilo > hi || r.jlo > hj || r.klo > hk) return OEB_ERR_HALO;
  if (d.nx + r.ihi > szi - hi || d.ny + r.jhi > szj - hj || d.nz + r.khi > szk - hk) return OEB_ERR_HALO;
  if (ReachLog* log = t_reach_log) {
    if (log->n < ReachLog::kMax) {
      log->desc[log->n] = m;
      log->reach[log->n++] = r;
    }
  }
  g->origin = m->aligned + m->offset;
  g->sj = sj;
  g->sk = sk;
  const int64_t first = -(int64_t)r.ilo - (int64_t)r.jlo * sj - (int64_t)r.klo * sk;
  const int64_t last = (d.nx - 1 + r.ihi) + (d.ny - 1 + r.jhi) * sj + (d.nz - 1 + r.khi) * sk;
  g->lo = reinterpret_cast<const char*>(g->origin + first);
  g->hi = reinterpret_cast<const char*>(g->origin + last + 1);
  return OEB_OK;
}

template <class T, class M>
oeb_status check_field1(const M* m, const oeb_domain& d, int jlo, int jhi, Line<T>* l) {
  if (!m || !m->aligned) return OEB_ERR_NULL;
  if (reinterpret_cast<uintptr_t>(m->aligned) % alignof(T) != 0) return OEB_ERR_ALIGNMENT;
  const int64_t s = m->strides[0];
  if (s < 1 || m->sizes[0] < 1) return OEB_ERR_LAYOUT;
  if (m->offset < 0 || m->offset % s != 0) return OEB_ERR_HALO;
  const int64_t h = m->offset / s;
  if (jlo > h || d.ny + jhi > m->sizes[0] - h) return OEB_ERR_HALO;
  l->origin = m->aligned + m->offset;
  l->s = s;
  l->lo = reinterpret_cast<const char*>(l->origin - (int64_t)jlo * s);
  l->hi = reinterpret_cast<const char*>(l->origin + (d.ny - 1 + jhi) * s + 1);
  return OEB_OK;
}

template <class T>
oeb_status check_same_strides(std::initializer_list<const Grid<T>*> grids) {
  const Grid<T>* first = *grids.begin();
  for (const Grid<T>* g : grids)
    if (g->sj != first->sj || g->sk != first->sk) return OEB_ERR_LAYOUT;
  return OEB_OK;
}

// Ranges come as flat lists of (lo, hi) pairs.
oeb_status check_no_alias(std::initializer_list<const char*> outs, std::initializer_list<const char*> ins) {
  std::vector<const char*> o(outs), in(ins);
  for (size_t a = 0; a + 1 < o.size(); a += 2) {
    for (size_t b = a + 2; b + 1 < o.size(); b += 2)
      if (o[a] < o[b + 1] && o[b] < o[a + 1]) return OEB_ERR_ALIAS;
    for (size_t b = 0; b + 1 < in.size(); b += 2)
      if (o[a] < in[b + 1] && in[b] < o[a + 1]) return OEB_ERR_ALIAS;
  }
  return OEB_OK;
}

template oeb_status check_field3<double, oeb_memref3d_f64>(const oeb_memref3d_f64*, const oeb_domain&, const Reach&,
                                                          Grid<double>*);
template oeb_status check_field3<float, oeb_memref3d_f32>(const oeb_memref3d_f32*, const oeb_domain&, const Reach&,
                                                         Grid<float>*);
template oeb_status check_field1<double, oeb_memref1d_f64>(const oeb_memref1d_f64*, const oeb_domain&, int, int,
                                                          Line<double>*);
template oeb_status check_field1<float, oeb_memref1d_f32>(const oeb_memref1d_f32*, const oeb_domain&, int, int,
                                                         Line<float>*);
template oeb_status check_same_strides<double>(std::initializer_list<const Grid<double>*>);
template oeb_status check_same_strides<float>(std::initializer_list<const Grid<float>*>);

}  // namespace oeb

// ---------------------------------------------------------------------------------------
// C ABI: information, errors, storage
// ---------------------------------------------------------------------------------------

extern "C" int oeb_abi_version(void) { return 10000; }

extern "C" const char* oeb_status_string(int status) {
  switch (status) {
    case OEB_OK: return "ok";
    case OEB_ERR_NULL: return "a required descriptor or pointer is NULL";
    case OEB_ERR_DOMAIN: return "invalid interior extents";
    case OEB_ERR_LAYOUT: return "unsupported or mismatched field layout";
    case OEB_ERR_HALO: return "field halo smaller than the kernel's reach";
    case OEB_ERR_ALIGNMENT: return "pointer not aligned to its element size";
    case OEB_ERR_CUDA: return "CUDA runtime error";
    case OEB_ERR_ALLOC: return "allocation failed";
    case OEB_ERR_ALIAS: return "an output overlaps another field";
    case OEB_ERR_UNSUPPORTED: return "unsupported kernel or variant";
    case OEB_ERR_TIMEOUT: return "bounded device wait gave up";
    case OEB_ERR_TOO_LARGE: return "request exceeds a fixed capacity";
    case OEB_ERR_ARGUMENT: return "scalar argument out of range";
    default: return "unknown status";
  }
}

extern "C" const char* oeb_last_cuda_error(void) { return oeb::g_last_cuda_error; }

extern "C" uint64_t oeb_launch_count(void) { return oeb::g_launches.load(std::memory_order_relaxed); }

extern "C" int oeb_is_device_pointer(const void* p) {
  if (!p) return 0;
  cudaPointerAttributes attr;
  cudaError_t e = cudaPointerGetAttributes(&attr, p);
  if (e != cudaSuccess) {
    cudaGetLastError();  // unregistered host memory on some drivers: clear the sticky-free error
    return 0;
  }
  return (attr.type == cudaMemoryTypeDevice || attr.type == cudaMemoryTypeManaged) ? 1 : 0;
}

extern "C" oeb_status oeb_stream_synchronize(void* stream) {
  cudaError_t e = cudaStreamSynchronize((cudaStream_t)stream);
  return e == cudaSuccess ? OEB_OK : oeb::cuda_fail(e);
}

namespace {

template <class T, class M>
oeb_status alloc3(int64_t nx, int64_t ny, int64_t nz, int64_t halo, int64_t pitch_multiple, M* out) {
  if (!out) return OEB_ERR_NULL;
  if (nx < 1 || ny < 1 || nz < 1 || halo < 0 || pitch_multiple < 1) return OEB_ERR_ARGUMENT;
  const int64_t szi = nx + 2 * halo, szj = ny + 2 * halo, szk = nz + 2 * halo;
  const int64_t pitch = (szi + pitch_multiple - 1) / pitch_multiple * pitch_multiple;
  const int64_t n = pitch * szj * szk;
  void* p = nullptr;
  cudaError_t e = cudaMalloc(&p, (size_t)n * sizeof(T));
  if (e != cudaSuccess) {
    oeb::cuda_fail(e);
    return OEB_ERR_ALLOC;
  }
  out->allocated = static_cast<T*>(p);
  out->aligned = static_cast<T*>(p);
  out->sizes[0] = szk;
  out->sizes[1] = szj;
  out->sizes[2] = szi;
  out->strides[2] = 1;
  out->strides[1] = pitch;
  out->strides[0] = pitch * szj;
  out->offset = halo * out->strides[0] + halo * out->strides[1] + halo;  // util.h:136
  return OEB_OK;
}

template <class T, class M>
oeb_status alloc1(int64_t n, int64_t halo, M* out) {
  if (!out) return OEB_ERR_NULL;
  if (n < 1 || halo < 0) return OEB_ERR_ARGUMENT;
  void* p = nullptr;
  cudaError_t e = cudaMalloc(&p, (size_t)(n + 2 * halo) * sizeof(T));
  if (e != cudaSuccess) {
    oeb::cuda_fail(e);
    return OEB_ERR_ALLOC;
  }
  out->allocated = static_cast<T*>(p);
  out->aligned = static_cast<T*>(p);
  out->sizes[0] = n + 2 * halo;
  out->strides[0] = 1;
  out->offset = halo;  // util.h:105
  return OEB_OK;
}

}  // namespace

extern "C" oeb_status oeb_storage3d_alloc_f64(int64_t nx, int64_t ny, int64_t nz, int64_t halo, int64_t pm,
                                              oeb_memref3d_f64* out) {
  return alloc3<double>(nx, ny, nz, halo, pm, out);
}
extern "C" oeb_status oeb_storage1d_alloc_f64(int64_t n, int64_t halo, oeb_memref1d_f64* out) {
  return alloc1<double>(n, halo, out);
}
extern "C" oeb_status oeb_storage3d_alloc_f32(int64_t nx, int64_t ny, int64_t nz, int64_t halo, int64_t pm,
                                              oeb_memref3d_f32* out) {
  return alloc3<float>(nx, ny, nz, halo, pm, out);
}
extern "C" oeb_status oeb_storage1d_alloc_f32(int64_t n, int64_t halo, oeb_memref1d_f32* out) {
  return alloc1<float>(n, halo, out);
}

// All four descriptor types start with {allocated, aligned}; freeing needs only those.
extern "C" oeb_status oeb_storage_free(void* memref) {
  if (!memref) return OEB_ERR_NULL;
  void** ptrs = static_cast<void**>(memref);
  if (ptrs[0]) {
    cudaError_t e = cudaFree(ptrs[0]);
    if (e != cudaSuccess) return oeb::cuda_fail(e);
  }
  ptrs[0] = nullptr;
  ptrs[1] = nullptr;
  return OEB_OK;
}

// Bytes from `allocated` to one past the last element of the descriptor's box; the box
// starts at aligned[0] for every allocateStorage-style descriptor (include/util.h:136-139).
template <class M, class T>
static int64_t span_bytes(const M* m) {
  if (!m || !m->aligned || !m->allocated) return 0;
  const int64_t last = (m->sizes[0] - 1) * m->strides[0] + (m->sizes[1] - 1) * m->strides[1] +
                       (m->sizes[2] - 1) * m->strides[2];
  return (int64_t)((m->aligned + last + 1) - m->allocated) * (int64_t)sizeof(T);
}

extern "C" int64_t oeb_memref3d_span_bytes_f64(const oeb_memref3d_f64* m) { return span_bytes<oeb_memref3d_f64, double>(m); }
extern "C" int64_t oeb_memref3d_span_bytes_f32(const oeb_memref3d_f32* m) { return span_bytes<oeb_memref3d_f32, float>(m); }

extern "C" oeb_status oeb_set_tile_shape(int shape) {
  if (shape < 0 || shape >= oeb::kShapes) return OEB_ERR_ARGUMENT;
  oeb::g_shape_override.store(shape, std::memory_order_relaxed);
  return OEB_OK;
}

extern "C" oeb_status oeb_set_adjoint_tiles(int on) {
  if (on != 0 && on != 1) return OEB_ERR_ARGUMENT;
  oeb::g_adjoint_tiles.store(on, std::memory_order_relaxed);
  return OEB_OK;
}

extern "C" oeb_status oeb_set_fusion(int mask) {
  if (mask & ~OEB_FUSE_ALL) return OEB_ERR_ARGUMENT;
  oeb::g_fusion_override.store(mask, std::memory_order_relaxed);
  return OEB_OK;
}

extern "C" oeb_status oeb_set_kblock(int kb) {
  if (kb < 0 || kb > 1024) return OEB_ERR_ARGUMENT;
  oeb::g_kb_override.store(kb, std::memory_order_relaxed);
  return OEB_OK;
}

// ---- whole-field transfers (oeb_upload* / oeb_download*) ------------------------------
// A field made by allocateStorage (include/util.h:99-148) moves to or from its device twin as
// one copy of its elements: from aligned[0] (element (0,0,0) of the box, halo included) to one
// past the last element, row padding included.  What lies between allocated and aligned is
// unused padding in allocateStorage (aligned = allocated + 32 - halo, util.h:139) and none in
// oeb_storage*_alloc (aligned = allocated), so it is neither compared nor copied.  Both
// descriptors must have the same offset, sizes and strides; cudaMemcpyDefault lets either
// side be host (pageable or pinned) or device memory.
namespace {

template <class T, int R, class M>
oeb_status transfer(const M* dst, const M* src, void* stream) {
  if (!dst || !src || !dst->aligned || !src->aligned) return OEB_ERR_NULL;
  if (dst->offset != src->offset) return OEB_ERR_LAYOUT;
  int64_t last = 0;
  for (int r = 0; r < R; ++r) {
    if (dst->sizes[r] != src->sizes[r] || dst->strides[r] != src->strides[r]) return OEB_ERR_LAYOUT;
    if (dst->sizes[r] < 1 || dst->strides[r] < 1) return OEB_ERR_LAYOUT;
    last += (dst->sizes[r] - 1) * dst->strides[r];
  }
  const int64_t elems = last + 1;
  const uintptr_t a = (uintptr_t)dst->aligned, b = (uintptr_t)src->aligned, n = (uintptr_t)elems * sizeof(T);
  if (a < b + n && b < a + n) return OEB_ERR_ALIAS;
  const cudaError_t e = cudaMemcpyAsync((void*)dst->aligned, src->aligned, (size_t)elems * sizeof(T),
                                        cudaMemcpyDefault, (cudaStream_t)stream);
  return e == cudaSuccess ? OEB_OK : oeb::cuda_fail(e);
}

}  // namespace

extern "C" oeb_status oeb_upload3d_f64(const oeb_memref3d_f64* dev, const oeb_memref3d_f64* host, void* stream) {
  return transfer<double, 3>(dev, host, stream);
}
extern "C" oeb_status oeb_download3d_f64(const oeb_memref3d_f64* host, const oeb_memref3d_f64* dev, void* stream) {
  return transfer<double, 3>(host, dev, stream);
}
extern "C" oeb_status oeb_upload1d_f64(const oeb_memref1d_f64* dev, const oeb_memref1d_f64* host, void* stream) {
  return transfer<double, 1>(dev, host, stream);
}
extern "C" oeb_status oeb_download1d_f64(const oeb_memref1d_f64* host, const oeb_memref1d_f64* dev, void* stream) {
  return transfer<double, 1>(host, dev, stream);
}
extern "C" oeb_status oeb_upload3d_f32(const oeb_memref3d_f32* dev, const oeb_memref3d_f32* host, void* stream) {
  return transfer<float, 3>(dev, host, stream);
}
extern "C" oeb_status oeb_download3d_f32(const oeb_memref3d_f32* host, const oeb_memref3d_f32* dev, void* stream) {
  return transfer<float, 3>(host, dev, stream);
}
extern "C" oeb_status oeb_upload1d_f32(const oeb_memref1d_f32* dev, const oeb_memref1d_f32* host, void* stream) {
  return transfer<float, 1>(dev, host, stream);
}
extern "C" oeb_status oeb_download1d_f32(const oeb_memref1d_f32* host, const oeb_memref1d_f32* dev, void* stream) {
  return transfer<float, 1>(host, dev, stream);
}
