// host_staging.cu -- host-buffer entry points oeb_<k>_f64_host.
//
// These take the same descriptors as the device entry points, but pointing to HOST memory
// (for instance fields made by the reference's allocateStorage, include/util.h:126-141),
// and return when the outputs are in host memory.  Cells outside the written boxes are
// never written, as in the reference.
//
// Direct mode (the default where it applies): when the device can address every field in
// place -- a GB300 with its Grace host reads and writes pageable host memory over NVLink-C2C
// through the host's page tables; elsewhere page-locked memory mapped at the same address --
// the call runs the device entry point on the host descriptors themselves.  The stencils'
// loads and stores cross the link as the kernel runs: no staging copies, and the transfers
// overlap the arithmetic.
//
// Staged mode (other memory, or oeb_set_host_direct(0)): every field goes through device
// memory from a library-owned stream-ordered pool, in a three-stage pipeline over k-slabs of the domain, on two copy streams of the
// library and the caller's stream:
//   copy-in   the inputs in k order: slab s needs every level up to its top + 1 (no stencil
//             reads further in k), which in the k-major layout is a prefix of each field's
//             span, so the inputs go up in prefix chunks, each byte once;
//   compute   the device entry point on descriptors shifted to the slab (origin + k0 planes,
//             nz = the slab's levels), as soon as its chunk is in;
//   copy-out  each output's written box for the slab (cudaMemcpy3DAsync), as soon as the
//             slab is computed.
// Host-to-device and device-to-host copies run on separate copy engines and overlap the
// kernels, so a call costs about its largest stage instead of their sum.  Pinned host memory
// makes the copies DMA transfers; pageable memory also works.
#include <algorithm>
#include <atomic>
#include <mutex>
#include <vector>

#include "oeb_reach.cuh"

namespace oeb {
namespace {

template <class T>
const T* span_start(const T* allocated, const T* aligned) {
  return (allocated && allocated <= aligned) ? allocated : aligned;
}

// Number of elements from the span start to one past the descriptor's last element; the
// descriptor's box starts at aligned[0] (include/util.h:136-139).
template <class M>
int64_t span_elems3(const M* m) {
  const int64_t last = (m->sizes[0] - 1) * m->strides[0] + (m->sizes[1] - 1) * m->strides[1] +
                       (m->sizes[2] - 1) * m->strides[2];
  return (int64_t)(m->aligned - span_start(m->allocated, m->aligned)) + last + 1;
}
template <class M>
int64_t span_elems1(const M* m) {
  return (int64_t)(m->aligned - span_start(m->allocated, m->aligned)) + (m->sizes[0] - 1) * m->strides[0] + 1;
}

template <class M>
bool sane3(const M* m) {
  return m && m->aligned && m->sizes[0] > 0 && m->sizes[1] > 0 && m->sizes[2] > 0 && m->strides[0] > 0 &&
         m->strides[1] > 0 && m->strides[2] > 0;
}
template <class M>
bool sane1(const M* m) {
  return m && m->aligned && m->sizes[0] > 0 && m->strides[0] > 0;
}

template <class M3>
struct OutSpec {
  const M3* host;
  Reach box;
};

// Stream-ordered staging of one call.  Device buffers are returned to the pool on every
// exit path, after all work that uses them has been enqueued.
template <class T>
class Stager {
 public:
  Stager(cudaStream_t s, cudaMemPool_t pool) : s_(s), free_(s), pool_(pool) {}
  ~Stager() {
    for (void* p : bufs_) cudaFreeAsync(p, free_);
  }
  // Returns the buffers on `s` instead (a stream ordered after every use of them).
  void release_on(cudaStream_t s) { free_ = s; }

  // A device buffer for the span of `host`; `dev` is `host` rebased onto it.
  template <class M>
  oeb_status alloc(const M* host, int64_t elems, M* dev) {
    void* buf = nullptr;
    const size_t bytes = (size_t)elems * sizeof(T);
    cudaError_t e = cudaMallocFromPoolAsync(&buf, bytes, pool_, s_);
    if (e != cudaSuccess) {
      cuda_fail(e);
      return OEB_ERR_ALLOC;
    }
    bufs_.push_back(buf);
    const T* start = span_start(host->allocated, host->aligned);
    *dev = *host;
    T* base = static_cast<T*>(buf);
    dev->aligned = base + (host->aligned - start);
    dev->allocated = base;
    return OEB_OK;
  }

 private:
  cudaStream_t s_, free_;
  cudaMemPool_t pool_;
  std::vector<void*> bufs_;
};

// Copies the written box of one output from device to host.
template <class T, class M3>
oeb_status copy_box_back(const M3* host, const M3* dev, const oeb_domain& d, const Reach& r, cudaStream_t s) {
  const int64_t sj = host->strides[1], sk = host->strides[0];
  const int64_t first = host->offset - r.ilo - r.jlo * sj - r.klo * sk;
  const size_t width = (size_t)(d.nx + r.ilo + r.ihi) * sizeof(T);
  const size_t rows = (size_t)(d.ny + r.jlo + r.jhi);
  const size_t planes = (size_t)(d.nz + r.klo + r.khi);
  T* hsrc = host->aligned + first;
  T* dsrc = dev->aligned + first;
  if (sk % sj == 0) {
    cudaMemcpy3DParms p = {};
    p.srcPtr = make_cudaPitchedPtr(dsrc, (size_t)sj * sizeof(T), width, (size_t)(sk / sj));
    p.dstPtr = make_cudaPitchedPtr(hsrc, (size_t)sj * sizeof(T), width, (size_t)(sk / sj));
    p.extent = make_cudaExtent(width, rows, planes);
    p.kind = cudaMemcpyDeviceToHost;
    OEB_CUDA_TRY(cudaMemcpy3DAsync(&p, s));
  } else {
    for (size_t k = 0; k < planes; ++k)
      OEB_CUDA_TRY(cudaMemcpy2DAsync(hsrc + k * sk, (size_t)sj * sizeof(T), dsrc + k * sk, (size_t)sj * sizeof(T),
                                     width, rows, cudaMemcpyDeviceToHost, s));
  }
  return OEB_OK;
}

constexpr int kMaxFields = 16;
constexpr int kMaxSlabs = 8;
constexpr int64_t kMinPipelinedBytes = int64_t(8) << 20;  // smaller calls run as one slab
std::atomic<int> g_host_slabs{0};                          // oeb_set_host_slabs (0: automatic)

// The copy streams and events of the staged calls on one device, created once.  Calls on a
// device are serialised by `mu` (each is synchronous anyway).
struct StageStreams {
  std::mutex mu;
  cudaStream_t in = nullptr, out = nullptr;
  cudaEvent_t ev_in[kMaxSlabs], ev_comp[kMaxSlabs];
};

oeb_status stage_streams(StageStreams** out) {
  static std::mutex mu;
  static std::vector<StageStreams*> per_device;
  int dev = 0;
  OEB_CUDA_TRY(cudaGetDevice(&dev));
  std::lock_guard<std::mutex> lock(mu);
  if ((int)per_device.size() <= dev) per_device.resize(dev + 1, nullptr);
  if (!per_device[dev]) {
    StageStreams* ss = new StageStreams();
    cudaError_t e = cudaStreamCreateWithFlags(&ss->in, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&ss->out, cudaStreamNonBlocking);
    for (int q = 0; q < kMaxSlabs && e == cudaSuccess; ++q) {
      e = cudaEventCreateWithFlags(&ss->ev_in[q], cudaEventDisableTiming);
      if (e == cudaSuccess) e = cudaEventCreateWithFlags(&ss->ev_comp[q], cudaEventDisableTiming);
    }
    if (e != cudaSuccess) return cuda_fail(e);  // the partial set is kept out of use
    per_device[dev] = ss;
  }
  *out = per_device[dev];
  return OEB_OK;
}

std::atomic<int> g_host_direct{1};  // oeb_set_host_direct
std::atomic<int> g_host_async{0};   // oeb_set_host_async

// Whether the current device can address host memory at `p` in place: it reads pageable
// memory through the host's page tables (cudaDevAttrPageableMemoryAccess, the NVLink-C2C
// systems), or `p` is page-locked memory mapped at the same address.
bool device_addressable(const void* p) {
  static std::mutex mu;
  static std::vector<int> pageable;  // per device: -1 unknown, 0 / 1
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return false;
  {
    std::lock_guard<std::mutex> lock(mu);
    if ((int)pageable.size() <= dev) pageable.resize(dev + 1, -1);
    if (pageable[dev] < 0) {
      int v = 0;
      pageable[dev] = cudaDeviceGetAttribute(&v, cudaDevAttrPageableMemoryAccess, dev) == cudaSuccess && v == 1;
    }
    if (pageable[dev]) return true;
  }
  cudaPointerAttributes a;
  if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
    cudaGetLastError();
    return false;
  }
  return a.type == cudaMemoryTypeHost && a.devicePointer == p;
}

template <class M>
M shift_k(const M& m, int64_t k0) {
  M r = m;
  r.offset += k0 * m.strides[0];
  return r;
}

// Stages the inputs (3-D and 1-D) and outputs of one call and runs `launch(d3, d1, o3, dom,
// stream)` on the device descriptors, slab by slab, with the copies overlapped.
template <class T, class M3, class M1, class Launch>
oeb_status run_host(const oeb_domain* dom, void* stream, std::initializer_list<const M3*> in3,
                    std::initializer_list<const M1*> in1, std::initializer_list<OutSpec<M3>> out3, Launch&& launch) {
  OEB_TRY(check_domain(dom));
  for (const M3* m : in3)
    if (!sane3(m)) return m ? OEB_ERR_LAYOUT : OEB_ERR_NULL;
  for (const M1* m : in1)
    if (!sane1(m)) return m ? OEB_ERR_LAYOUT : OEB_ERR_NULL;
  for (const OutSpec<M3>& o : out3)
    if (!sane3(o.host)) return o.host ? OEB_ERR_LAYOUT : OEB_ERR_NULL;
  if (in3.size() > (size_t)kMaxFields || in1.size() > (size_t)kMaxFields || out3.size() > (size_t)kMaxFields)
    return OEB_ERR_TOO_LARGE;
  M3 d3[kMaxFields];
  M1 d1[kMaxFields];
  M3 o3[kMaxFields];
  const M3* h3[kMaxFields];
  int n3 = 0, n1 = 0, no = 0;
  for (const M3* m : in3) h3[n3] = m, d3[n3++] = *m;
  for (const M1* m : in1) d1[n1++] = *m;
  for (const OutSpec<M3>& o : out3) o3[no++] = *o.host;
  ReachLog reach;
  {
    // Validate the host descriptors with the device entry point's own checks, before any
    // allocation or copy (the descriptors are identical up to the base pointers); the checks
    // record each input's reach
    ValidateOnly guard;
    set_reach_log(&reach);
    const oeb_status vst = launch(d3, d1, o3, dom, stream);
    set_reach_log(nullptr);
    OEB_TRY(vst);
  }
  // Direct: the kernels read and write the host fields in place over the host link -- no
  // staging copies, and the transfers overlap the arithmetic by construction.  Asynchronous
  // calls always stage: copy engines pipelined across calls move the data faster than
  // kernels reading the host fields one call after another (measured: 3.2 vs 2.5 GPts/s on
  // the ten-stencil step).
  const bool async = g_host_async.load(std::memory_order_relaxed) != 0;
  bool direct = g_host_direct.load(std::memory_order_relaxed) != 0 && !async;
  for (int q = 0; q < n3 && direct; ++q) direct = device_addressable(d3[q].aligned);
  for (int q = 0; q < n1 && direct; ++q) direct = device_addressable(d1[q].aligned);
  for (int q = 0; q < no && direct; ++q) direct = device_addressable(o3[q].aligned);
  if (direct) {
    oeb_status st;
    {
      HostInPlace in_place;
      st = launch(d3, d1, o3, dom, stream);
    }
    const cudaError_t e = cudaStreamSynchronize((cudaStream_t)stream);
    if (st == OEB_OK && e != cudaSuccess) st = cuda_fail(e);
    return st;
  }
  StageStreams* ss = nullptr;
  OEB_TRY(stage_streams(&ss));
  std::lock_guard<std::mutex> lock(ss->mu);
  cudaStream_t sc = (cudaStream_t)stream;
  cudaMemPool_t pool = nullptr;
  OEB_TRY(device_pool(&pool));
  int64_t span[kMaxFields];
  int64_t bytes = 0;
  for (int n = 0; n < n3; ++n) bytes += (span[n] = span_elems3(h3[n])) * (int64_t)sizeof(T);
  const int want = g_host_slabs.load(std::memory_order_relaxed);
  // automatic: one slab for small calls and for asynchronous ones (they pipeline across
  // calls, and every slab costs a copy per field to enqueue), else kMaxSlabs
  const int slabs = (int)std::min<int64_t>(
      want > 0 ? want : ((bytes < kMinPipelinedBytes || async) ? 1 : kMaxSlabs), dom->nz);
  oeb_status st = OEB_OK;
  {
    Stager<T> stage(ss->in, pool);  // buffers go back to the pool on ss->in, after the final sync
    for (int n = 0; n < n3 && st == OEB_OK; ++n) st = stage.alloc(h3[n], span[n], &d3[n]);
    int n = 0;
    for (const M1* m : in1) {
      if (st != OEB_OK) break;
      st = stage.alloc(m, span_elems1(m), &d1[n]);
      if (st == OEB_OK)
        st = cudaMemcpyAsync(d1[n].allocated, span_start(m->allocated, m->aligned), span_elems1(m) * sizeof(T),
                             cudaMemcpyHostToDevice, ss->in) == cudaSuccess
                 ? OEB_OK
                 : cuda_fail(cudaGetLastError());
      ++n;
    }
    n = 0;
    for (const OutSpec<M3>& o : out3) {
      if (st != OEB_OK) break;
      st = stage.alloc(o.host, span_elems3(o.host), &o3[n++]);
    }
    // each input's copy range (elements from its span start): the k-planes its kernel reads,
    // -klo .. nz+khi-1 of its validated reach (every row of them), else the whole span
    int64_t copied[kMaxFields] = {0}, need_end[kMaxFields];
    for (int q = 0; q < n3; ++q) {
      const M3* h = h3[q];
      need_end[q] = span[q];
      Reach r;
      if (reach.find(&d3[q], &r)) {
        // rounded out to 64 KB of the span (the copy engines move whole pages faster)
        constexpr int64_t kAlign = 65536 / (int64_t)sizeof(T);
        const int64_t sk = h->strides[0], hk = h->offset / sk;
        const int64_t base = (int64_t)(h->aligned - span_start(h->allocated, h->aligned));
        copied[q] = std::max<int64_t>(0, (base + (hk - r.klo) * sk) / kAlign * kAlign);
        need_end[q] = std::min<int64_t>(span[q], (base + (hk + dom->nz + r.khi) * sk + kAlign - 1) / kAlign * kAlign);
      }
    }
    for (int s = 0; s < slabs && st == OEB_OK; ++s) {
      const int64_t k0 = dom->nz * s / slabs, k1 = dom->nz * (s + 1) / slabs;
      // copy-in: every input's prefix up to level k1 (the slab's top + 1), whole on the last slab
      for (int q = 0; q < n3 && st == OEB_OK; ++q) {
        const M3* h = h3[q];
        const T* hstart = span_start(h->allocated, h->aligned);
        const int64_t end = s == slabs - 1 ? need_end[q]
                                           : std::min(need_end[q], (int64_t)(h->aligned - hstart) + h->offset +
                                                                       (k1 + 1) * h->strides[0]);
        if (end > copied[q]) {
          if (cudaMemcpyAsync(d3[q].allocated + copied[q], hstart + copied[q], (size_t)(end - copied[q]) * sizeof(T),
                              cudaMemcpyHostToDevice, ss->in) != cudaSuccess)
            st = cuda_fail(cudaGetLastError());
          copied[q] = end;
        }
      }
      if (st != OEB_OK) break;
      // (errors end the loop through `st`: the synchronisation below always runs before the
      // buffers go back to the pool)
      if (cudaEventRecord(ss->ev_in[s], ss->in) != cudaSuccess || cudaStreamWaitEvent(sc, ss->ev_in[s], 0) != cudaSuccess) {
        st = cuda_fail(cudaGetLastError());
        break;
      }
      // compute the slab
      M3 s3[kMaxFields], so[kMaxFields];
      for (int q = 0; q < n3; ++q) s3[q] = shift_k(d3[q], k0);
      for (int q = 0; q < no; ++q) so[q] = shift_k(o3[q], k0);
      const oeb_domain ds{dom->nx, dom->ny, k1 - k0};
      st = launch(s3, d1, so, &ds, stream);
      if (st != OEB_OK) break;
      if (!async && (cudaEventRecord(ss->ev_comp[s], sc) != cudaSuccess ||
                     cudaStreamWaitEvent(ss->out, ss->ev_comp[s], 0) != cudaSuccess)) {
        st = cuda_fail(cudaGetLastError());
        break;
      }
      // copy-out: the slab's part of every output's written box
      int q = 0;
      for (const OutSpec<M3>& o : out3) {
        const M3 hs = shift_k(*o.host, k0);
        st = copy_box_back<T>(&hs, &so[q++], ds, o.box, async ? sc : ss->out);
        if (st != OEB_OK) break;
      }
    }
    if (async && st == OEB_OK) {
      // complete when `stream` is: the copy-out ran on it, after the compute; the buffers
      // go back to the pool on it, after the copy-out (every other use of them precedes it),
      // so the next call's copy-in (ss->in) overlaps this call's compute and copy-out
      stage.release_on(sc);
    }
    if (!async || st != OEB_OK) {
      const cudaError_t e1 = cudaStreamSynchronize(ss->out);
      const cudaError_t e2 = cudaStreamSynchronize(sc);
      const cudaError_t e3 = cudaStreamSynchronize(ss->in);
      if (st == OEB_OK && (e1 != cudaSuccess || e2 != cudaSuccess || e3 != cudaSuccess))
        st = cuda_fail(e1 != cudaSuccess ? e1 : e2 != cudaSuccess ? e2 : e3);
    }
  }  // device buffers returned to the pool here (stream-ordered on ss->in, or on `stream` when asynchronous)
  return st;
}

}  // namespace
}  // namespace oeb

using namespace oeb;

#define OEB_HM3(S) oeb_memref3d_##S
#define OEB_HM1(S) oeb_memref1d_##S

#define OEB_HOST_ENTRIES(S, T) \
extern "C" oeb_status oeb_laplace_##S##_host(const OEB_HM3(S)* in, const OEB_HM3(S)* out, const oeb_domain* dom, void* stream) { \
  return run_host<T, OEB_HM3(S), OEB_HM1(S)>(dom, stream, {in}, {}, {{out, kInterior}}, \
                                  [&](const OEB_HM3(S)* i3, const OEB_HM1(S)*, const OEB_HM3(S)* o3, const oeb_domain* dm, void* sm) { \
                                    return oeb_laplace_##S(&i3[0], &o3[0], dm, sm); \
                                  }); \
} \
 \
extern "C" oeb_status oeb_hdiffsa_##S##_host(const OEB_HM3(S)* out, const OEB_HM3(S)* in, const OEB_HM3(S)* mask, const OEB_HM1(S)* crlato, \
                                           const OEB_HM1(S)* crlatu, const oeb_domain* dom, void* stream) { \
  return run_host<T, OEB_HM3(S), OEB_HM1(S)>(dom, stream, {in, mask}, {crlato, crlatu}, {{out, kInterior}}, \
                                  [&](const OEB_HM3(S)* i3, const OEB_HM1(S)* i1, const OEB_HM3(S)* o3, const oeb_domain* dm, void* sm) { \
                                    return oeb_hdiffsa_##S(&o3[0], &i3[0], &i3[1], &i1[0], &i1[1], dm, sm); \
                                  }); \
} \
 \
extern "C" oeb_status oeb_hdiffsmag_##S##_host(const OEB_HM3(S)* uout, const OEB_HM3(S)* vout, const OEB_HM3(S)* uin, const OEB_HM3(S)* vin, \
                                             const OEB_HM3(S)* mask, const OEB_HM1(S)* crlavo, const OEB_HM1(S)* crlavu, const OEB_HM1(S)* crlato, \
                                             const OEB_HM1(S)* crlatu, const OEB_HM1(S)* acrlat0, T eddlat, T eddlon, \
                                             T tau_smag, T weight_smag, const oeb_domain* dom, \
                                             void* stream) { \
  return run_host<T, OEB_HM3(S), OEB_HM1(S)>( \
      dom, stream, {uin, vin, mask}, {crlavo, crlavu, crlato, crlatu, acrlat0}, {{uout, kInterior}, {vout, kInterior}}, \
      [&](const OEB_HM3(S)* i3, const OEB_HM1(S)* i1, const OEB_HM3(S)* o3, const oeb_domain* dm, void* sm) { \
        return oeb_hdiffsmag_##S(&o3[0], &o3[1], &i3[0], &i3[1], &i3[2], &i1[0], &i1[1], &i1[2], &i1[3], &i1[4], \
                                 eddlat, eddlon, tau_smag, weight_smag, dm, sm); \
      }); \
} \
 \
extern "C" oeb_status oeb_hadvuv_##S##_host(const OEB_HM3(S)* uout, const OEB_HM3(S)* vout, const OEB_HM3(S)* uin, const OEB_HM3(S)* vin, \
                                          const OEB_HM1(S)* acrlat0, const OEB_HM1(S)* acrlat1, const OEB_HM1(S)* tgrlatda0, \
                                          const OEB_HM1(S)* tgrlatda1, T eddlat, T eddlon, const oeb_domain* dom, \
                                          void* stream) { \
  return run_host<T, OEB_HM3(S), OEB_HM1(S)>(dom, stream, {uin, vin}, {acrlat0, acrlat1, tgrlatda0, tgrlatda1}, \
                                  {{uout, kInterior}, {vout, kInterior}}, \
                                  [&](const OEB_HM3(S)* i3, const OEB_HM1(S)* i1, const OEB_HM3(S)* o3, const oeb_domain* dm, void* sm) { \
                                    return oeb_hadvuv_##S(&o3[0], &o3[1], &i3[0], &i3[1], &i1[0], &i1[1], &i1[2], \
                                                          &i1[3], eddlat, eddlon, dm, sm); \
                                  }); \
} \
 \
extern "C" oeb_status oeb_hadvuv5th_##S##_host(const OEB_HM3(S)* uout, const OEB_HM3(S)* vout, const OEB_HM3(S)* uin, const OEB_HM3(S)* vin, \
                                             const OEB_HM1(S)* acrlat0, const OEB_HM1(S)* acrlat1, const OEB_HM1(S)* tgrlatda0, \
                                             const OEB_HM1(S)* tgrlatda1, T eddlat, T eddlon, const oeb_domain* dom, \
                                             void* stream) { \
  return run_host<T, OEB_HM3(S), OEB_HM1(S)>(dom, stream, {uin, vin}, {acrlat0, acrlat1, tgrlatda0, tgrlatda1}, \
                                  {{uout, kInterior}, {vout, kInterior}}, \
                                  [&](const OEB_HM3(S)* i3, const OEB_HM1(S)* i1, const OEB_HM3(S)* o3, const oeb_domain* dm, void* sm) { \
                                    return oeb_hadvuv5th_##S(&o3[0], &o3[1], &i3[0], &i3[1], &i1[0], &i1[1], &i1[2], \
                                                             &i1[3], eddlat, eddlon, dm, sm); \
                                  }); \
} \
 \
extern "C" oeb_status oeb_fastwavesuv_##S##_host(const OEB_HM3(S)* uout, const OEB_HM3(S)* vout, const OEB_HM3(S)* uin, const OEB_HM3(S)* vin, \
                                               const OEB_HM3(S)* utens, const OEB_HM3(S)* vtens, const OEB_HM3(S)* wgtfac, const OEB_HM3(S)* ppuv, \
                                               const OEB_HM3(S)* hhl, const OEB_HM3(S)* rho, const OEB_HM1(S)* fx, T edadlat, T dt, \
                                               const oeb_domain* dom, void* stream) { \
  return run_host<T, OEB_HM3(S), OEB_HM1(S)>(dom, stream, {uin, vin, utens, vtens, wgtfac, ppuv, hhl, rho}, {fx}, \
                                  {{uout, kInterior}, {vout, kInterior}}, \
                                  [&](const OEB_HM3(S)* i3, const OEB_HM1(S)* i1, const OEB_HM3(S)* o3, const oeb_domain* dm, void* sm) { \
                                    return oeb_fastwavesuv_##S(&o3[0], &o3[1], &i3[0], &i3[1], &i3[2], &i3[3], &i3[4], \
                                                               &i3[5], &i3[6], &i3[7], &i1[0], edadlat, dt, dm, \
                                                               sm); \
                                  }); \
} \
 \
extern "C" oeb_status oeb_uvbke_##S##_host(const OEB_HM3(S)* ub, const OEB_HM3(S)* vb, const OEB_HM3(S)* uc, const OEB_HM3(S)* vc, const OEB_HM3(S)* cosa, \
                                         const OEB_HM3(S)* rsina, double dt5, const oeb_domain* dom, void* stream) { \
  return run_host<T, OEB_HM3(S), OEB_HM1(S)>(dom, stream, {uc, vc, cosa, rsina}, {}, {{ub, kInterior}, {vb, kInterior}}, \
                                  [&](const OEB_HM3(S)* i3, const OEB_HM1(S)*, const OEB_HM3(S)* o3, const oeb_domain* dm, void* sm) { \
                                    return oeb_uvbke_##S(&o3[0], &o3[1], &i3[0], &i3[1], &i3[2], &i3[3], dt5, dm, \
                                                         sm); \
                                  }); \
} \
 \
extern "C" oeb_status oeb_nh_p_grad_##S##_host(const OEB_HM3(S)* uout, const OEB_HM3(S)* vout, const OEB_HM3(S)* uin, const OEB_HM3(S)* vin, \
                                             const OEB_HM3(S)* rdx, const OEB_HM3(S)* rdy, const OEB_HM3(S)* gz, const OEB_HM3(S)* pp, const OEB_HM3(S)* pk3, \
                                             const OEB_HM3(S)* wk1, T dt, const oeb_domain* dom, void* stream) { \
  return run_host<T, OEB_HM3(S), OEB_HM1(S)>(dom, stream, {uin, vin, rdx, rdy, gz, pp, pk3, wk1}, {}, \
                                  {{uout, kInterior}, {vout, kInterior}}, \
                                  [&](const OEB_HM3(S)* i3, const OEB_HM1(S)*, const OEB_HM3(S)* o3, const oeb_domain* dm, void* sm) { \
                                    return oeb_nh_p_grad_##S(&o3[0], &o3[1], &i3[0], &i3[1], &i3[2], &i3[3], &i3[4], \
                                                             &i3[5], &i3[6], &i3[7], dt, dm, sm); \
                                  }); \
} \
 \
extern "C" oeb_status oeb_p_grad_c_##S##_host(const OEB_HM3(S)* uout, const OEB_HM3(S)* vout, const OEB_HM3(S)* uin, const OEB_HM3(S)* vin, \
                                            const OEB_HM3(S)* rdxc, const OEB_HM3(S)* rdyc, const OEB_HM3(S)* delpc, const OEB_HM3(S)* gz, \
                                            const OEB_HM3(S)* pkc, T dt2, const oeb_domain* dom, void* stream) { \
  return run_host<T, OEB_HM3(S), OEB_HM1(S)>(dom, stream, {uin, vin, rdxc, rdyc, delpc, gz, pkc}, {}, \
                                  {{uout, kInterior}, {vout, kInterior}}, \
                                  [&](const OEB_HM3(S)* i3, const OEB_HM1(S)*, const OEB_HM3(S)* o3, const oeb_domain* dm, void* sm) { \
                                    return oeb_p_grad_c_##S(&o3[0], &o3[1], &i3[0], &i3[1], &i3[2], &i3[3], &i3[4], \
                                                            &i3[5], &i3[6], dt2, dm, sm); \
                                  }); \
} \
 \
extern "C" oeb_status oeb_fvtp2d_##S##_host(const OEB_HM3(S)* q_i, const OEB_HM3(S)* q_j, const OEB_HM3(S)* fx1, const OEB_HM3(S)* fx2, const OEB_HM3(S)* fy1, \
                                          const OEB_HM3(S)* fy2, const OEB_HM3(S)* q, const OEB_HM3(S)* crx, const OEB_HM3(S)* cry, const OEB_HM3(S)* ra_x, \
                                          const OEB_HM3(S)* ra_y, const OEB_HM3(S)* xfx, const OEB_HM3(S)* yfx, const OEB_HM3(S)* area, T p1, \
                                          T p2, const oeb_domain* dom, void* stream) { \
  return run_host<T, OEB_HM3(S), OEB_HM1(S)>( \
      dom, stream, {q, crx, cry, ra_x, ra_y, xfx, yfx, area}, {}, \
      {{q_i, kFvQi}, {q_j, kFvQj}, {fx1, kInterior}, {fx2, kFvFx2}, {fy1, kInterior}, {fy2, kFvFy2}}, \
      [&](const OEB_HM3(S)* i3, const OEB_HM1(S)*, const OEB_HM3(S)* o3, const oeb_domain* dm, void* sm) { \
        return oeb_fvtp2d_##S(&o3[0], &o3[1], &o3[2], &o3[3], &o3[4], &o3[5], &i3[0], &i3[1], &i3[2], &i3[3], &i3[4], \
                              &i3[5], &i3[6], &i3[7], p1, p2, dm, sm); \
      }); \
}

OEB_HOST_ENTRIES(f64, double)
OEB_HOST_ENTRIES(f32, float)

extern "C" oeb_status oeb_set_host_slabs(int slabs) {
  if (slabs < 0 || slabs > oeb::kMaxSlabs) return OEB_ERR_ARGUMENT;
  oeb::g_host_slabs.store(slabs, std::memory_order_relaxed);
  return OEB_OK;
}

extern "C" oeb_status oeb_set_host_direct(int enable) {
  if (enable != 0 && enable != 1) return OEB_ERR_ARGUMENT;
  oeb::g_host_direct.store(enable, std::memory_order_relaxed);
  return OEB_OK;
}

extern "C" oeb_status oeb_set_host_async(int enable) {
  if (enable != 0 && enable != 1) return OEB_ERR_ARGUMENT;
  oeb::g_host_async.store(enable, std::memory_order_relaxed);
  return OEB_OK;
}
