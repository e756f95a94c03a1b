// launch.cuh -- the one way this library launches a kernel, and the batched persistent form.
//
// Every kernel is a Body: a struct with `static __device__ void run(uint3 blk, A... a)` that
// does the work of the CTA `blk` of its grid (the code that would read blockIdx).  launch<Body>
// either runs it as an ordinary grid (grid_kernel, blk = blockIdx), or -- while a Recorder is
// installed on the calling thread -- records the grid and the arguments instead.  A batch plan
// (batch.cu) records the same sequence of calls for many ensemble members and then replays
// each recorded position as ONE persistent launch over all members: batch_kernel, whose CTAs
// walk a list of (member, tile) items -- or runs every member's whole step in one launch of the
// step kernel (step.cu), which calls the bodies that declare a kStepOp.  The bodies never read
// blockIdx or gridDim, so a tile computes the same results in every form.
//
// Every kernel instantiated for double runs as the same kernel instantiated for F64i
// (precision.cuh): double arithmetic with the multiplications on the integer pipe, bit for
// bit the same results.  launch() rebinds the Body and reinterprets its arguments (double,
// double*, and structs or pointers of a template over double) as their F64i twins, which
// have the same layout.
//
// Scratch memory of a call (adjoint terms, dual-number arrays) comes from scratch_alloc: the
// library's stream-ordered pool normally, the plan's arena while recording (so that it lives
// as long as the plan).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>
#include <string.h>

#include <type_traits>
#include <utility>
#include <vector>

#include "oeb_common.cuh"
#include "precision.cuh"

namespace oeb {

constexpr int kLaunchTX = 32, kLaunchTY = 8;  // every CTA is 32 x 8 threads

// ---- argument packs (trivially copyable, identical layout on host and device) -------
template <class... A>
struct Pack;
template <>
struct Pack<> {};
template <class H, class... R>
struct Pack<H, R...> {
  H h;
  Pack<R...> r;
};

inline Pack<> make_pack() { return {}; }
template <class H, class... R>
Pack<H, R...> make_pack(H h, R... r) {
  return Pack<H, R...>{h, make_pack(r...)};
}

template <class Body, class... Done>
__device__ __forceinline__ void call_pack(const uint3& blk, const Pack<>&, const Done&... d) {
  Body::run(blk, d...);
}
template <class Body, class H, class... R, class... Done>
__device__ __forceinline__ void call_pack(const uint3& blk, const Pack<H, R...>& p, const Done&... d) {
  call_pack<Body>(blk, p.r, d..., p.h);
}

// ---- kernels ----------------------------------------------------------------------------
template <class Body, class... A>
__global__ void __launch_bounds__(kLaunchTX* kLaunchTY) grid_kernel(A... a) {
  Body::run(blockIdx, a...);
}

// The same for a body that declares kMinCtas > 0: the compiler keeps its registers low
// enough for that many CTAs per SM.
template <class Body, int N, class... A>
__global__ void __launch_bounds__(kLaunchTX* kLaunchTY, N) grid_kernel_bound(A... a) {
  Body::run(blockIdx, a...);
}

template <class Body, class = void>
struct MinCtas {
  static constexpr int value = 0;
};
template <class Body>
struct MinCtas<Body, std::void_t<decltype(Body::kMinCtas)>> {
  static constexpr int value = Body::kMinCtas;
};

// The tile shape a body was instantiated with (kShape, see tuned_shape), 0 for bodies that
// take no shape.
template <class Body, class = void>
struct ShapeOf {
  static constexpr int value = 0;
};
template <class Body>
struct ShapeOf<Body, std::void_t<decltype(Body::kShape)>> {
  static constexpr int value = Body::kShape;
};

// The grid kernel of Body over arguments A...
template <class Body, class... A>
constexpr auto grid_entry() {
  if constexpr (MinCtas<Body>::value > 0)
    return &grid_kernel_bound<Body, MinCtas<Body>::value, A...>;
  else
    return &grid_kernel<Body, A...>;
}

// ---- the one-launch step (step.cu) --------------------------------------------------------
// A batch plan can also run every member's whole step as ONE persistent launch of the step
// kernel, which calls the bodies of the chained step from a single switch.  A body that may
// run there declares `static constexpr int kStepOp = step_op<T>(kOp...)`: an id unique over
// both precisions.  Bodies without one (or instantiated for another T, e.g. Dual) are -1.
enum StepOpBase : int {
  kOpCombine,
  kOpFwsFwd,
  kOpFwsAdjTerms,
  kOpFwsAdj,       // fastwavesuv_adj_kernel<T, 0>: the march over the terms pass's coefficients
  kOpFwsAdjFused,  // fastwavesuv_adj_kernel<T, 1>: the march that forms them itself
  kOpHadv5Fwd,     // + tile shape (3 shapes)
  kOpHadv5AdjTerms = kOpHadv5Fwd + 3,  // + tile shape
  kOpHadv5AdjGather = kOpHadv5AdjTerms + 3,
  kOpSmagFwd,
  kOpSmagAdjTerms,
  kOpSmagAdjTs,
  kOpSmagAdjGather,
  kOpSmagAdjFused,
  kOpFvQ,
  kOpFvFlux,
  kOpFvFused,
  kOpFvAdjQij,
  kOpFvAdjF2,
  kOpFvAdjQ,
  kOpHadv5AdjTiled,  // hadv_adj_f32<5>: the FP32 advection adjoint in one tiled launch
  kStepOpBases
};
template <class T>
constexpr int step_op(int base) {
  return base < 0 ? -1 : std::is_same<T, F64i>::value ? 2 * base : std::is_same<T, float>::value ? 2 * base + 1 : -1;
}
constexpr int kStepOps = 2 * kStepOpBases;

template <class Body, class = void>
struct StepOpOf {
  static constexpr int value = -1;
};
template <class Body>
struct StepOpOf<Body, std::void_t<decltype(Body::kStepOp)>> {
  static constexpr int value = Body::kStepOp;
};

// The argument pack of a body's run() parameters (after the tile index), decayed: what the
// step kernel reads.  A recording converts the call's arguments to these types on the host,
// as an ordinary launch converts them when it calls run().
template <class... P>
Pack<std::decay_t<P>...> run_pack_of(void (*)(const uint3&, P...));
template <class Body>
using RunPack = decltype(run_pack_of(&Body::run));
template <class P>
struct PackFrom;
template <class... P>
struct PackFrom<Pack<P...>> {
  template <class... A>
  static Pack<P...> make(A... a) {
    static_assert(sizeof...(A) == sizeof...(P), "run() takes a different number of arguments");
    return make_pack(static_cast<P>(a)...);
  }
};

// One item per (member, tile); tiles[m] = {first item of member m, tiles along x, along y}.
struct BatchTile {
  int first, gx, gy, pad;
};

template <class Body, class... A>
__global__ void __launch_bounds__(kLaunchTX* kLaunchTY)
    batch_kernel(const BatchTile* __restrict__ tiles, int members, int total, const Pack<A...>* __restrict__ args) {
  for (int item = blockIdx.x; item < total; item += gridDim.x) {
    int lo = 0, hi = members - 1;  // last member whose first item is <= item
    while (lo < hi) {
      const int mid = (lo + hi + 1) >> 1;
      if (tiles[mid].first <= item) lo = mid; else hi = mid - 1;
    }
    const BatchTile t = tiles[lo];
    const int local = item - t.first;
    const int plane = t.gx * t.gy;
    const uint3 blk = make_uint3((unsigned)(local % t.gx), (unsigned)((local % plane) / t.gx),
                                 (unsigned)(local / plane));
    const Pack<A...> a = args[lo];
    call_pack<Body>(blk, a);
    __syncthreads();  // the next item reuses the shared memory
  }
}

// ---- recording ----------------------------------------------------------------------------
// Launches one recorded position for `members` members: tiles and args are device arrays.
using BatchLaunchFn = oeb_status (*)(const BatchTile* tiles, int members, int total, const void* args, size_t smem,
                                     int ctas, cudaStream_t st);
// CTAs of batch_kernel that fit on one SM with `smem` dynamic shared memory.
using BatchOccupancyFn = int (*)(size_t smem);

// Launches one recorded call as an ordinary grid from its argument pack (host memory).
using GridLaunchFn = oeb_status (*)(const void* args, dim3 grid, size_t smem, cudaStream_t st);

struct LaunchRecord {
  BatchLaunchFn launcher;  // also identifies the kernel (Body and argument types)
  int shape_tag = 0;       // the body's tile shape (ShapeOf); 0 for bodies that take none
  GridLaunchFn grid_launcher;
  BatchOccupancyFn occupancy;
  dim3 grid;
  size_t smem;
  std::vector<unsigned char> args;  // Pack<A...>
  int step_op = -1;                      // the body's kStepOp (-1: the step kernel cannot run it)
  std::vector<unsigned char> step_args;  // RunPack<Body>, for the step kernel
};

struct Recorder {
  std::vector<LaunchRecord> records;
  char* arena = nullptr;  // scratch arena (nullptr: sizing pass, addresses are placeholders)
  size_t arena_bytes = 0;
  size_t used = 0;  // top of the arena stack
  size_t peak = 0;  // the most it held
  // live allocations, oldest first: {offset, freed}.  A call's scratch is freed when the call
  // returns; the stack pops every freed allocation on its top, so later calls reuse the space
  // (safe: a batch runs each recorded launch for all members before the next one).
  std::vector<std::pair<size_t, bool>> live;
  int kb = 0;     // k-levels per CTA for the kernels that take one (0: their default)
  int shape = 0;  // tile shape for the kernels that take one (0: their default; tuned_shape)
  int fusion = 0;  // fusion grouping of the chained step (tuned_fusion)
};

Recorder* recorder();             // the calling thread's recorder, or nullptr
void set_recorder(Recorder* r);  // installs (or with nullptr removes) it
// k-levels per CTA set by oeb_set_kblock (0: none).
int kb_override();
// Whether the FP32 adjoints that have a tiled one-launch form use it (oeb_set_adjoint_tiles;
// default 1).
int adjoint_tiles();
// k-levels per CTA: the recorder's choice while recording, else oeb_set_kblock's, else `def`.
inline int tuned_kb(int def) {
  const Recorder* r = recorder();
  if (r && r->kb > 0) return r->kb;
  const int o = kb_override();
  return o > 0 ? o : def;
}

// Tile shapes of the pointwise bodies that take one: 0 = 32 x 32 (the default), 1 = 32 x 8,
// 2 = 64 x 16 (i x j cells a CTA of 32 x 8 threads covers).
constexpr int kShapes = 3;
int shape_override();  // set by oeb_set_tile_shape (0: none)
// The tile shape: the recorder's while recording, else oeb_set_tile_shape's.
inline int tuned_shape() {
  const Recorder* r = recorder();
  if (r) return r->shape;
  return shape_override();
}

// Fusion groupings of the chained step, a bit mask (OEB_FUSE_* in oeb_gb300.h): which stages
// run as one kernel.  The recorder's while recording (a batch plan's grouping), else
// oeb_set_fusion's (OEB_FUSE_HADV_UPDATE by default).
int fusion_override();
inline int tuned_fusion() {
  const Recorder* r = recorder();
  if (r) return r->fusion;
  return fusion_override();
}

oeb_status scratch_alloc(void** p, size_t bytes, cudaStream_t st);
void scratch_free(void* p, cudaStream_t st);

template <class Body, class... A>
oeb_status batch_launch(const BatchTile* tiles, int members, int total, const void* args, size_t smem, int ctas,
                        cudaStream_t st) {
  if (smem > 48 * 1024) OEB_TRY(ensure_dyn_smem((const void*)batch_kernel<Body, A...>, (int)smem));
  batch_kernel<Body, A...><<<ctas, dim3(kLaunchTX, kLaunchTY), smem, st>>>(
      tiles, members, total, static_cast<const Pack<A...>*>(args));
  return after_launch();
}

template <class Body, class... Done>
void launch_unpacked(dim3 grid, size_t smem, cudaStream_t st, const Pack<>&, const Done&... d) {
  grid_entry<Body, Done...>()<<<grid, dim3(kLaunchTX, kLaunchTY), smem, st>>>(d...);
}
template <class Body, class H, class... R, class... Done>
void launch_unpacked(dim3 grid, size_t smem, cudaStream_t st, const Pack<H, R...>& p, const Done&... d) {
  launch_unpacked<Body>(grid, smem, st, p.r, d..., p.h);
}

template <class Body, class... A>
oeb_status grid_launch_packed(const void* args, dim3 grid, size_t smem, cudaStream_t st) {
  if (smem > 48 * 1024) OEB_TRY(ensure_dyn_smem((const void*)grid_entry<Body, A...>(), (int)smem));
  launch_unpacked<Body>(grid, smem, st, *static_cast<const Pack<A...>*>(args));
  return after_launch();
}

template <class Body, class... A>
int batch_occupancy(size_t smem) {
  if (smem > 48 * 1024 && ensure_dyn_smem((const void*)batch_kernel<Body, A...>, (int)smem) != OEB_OK) return 1;
  int n = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, batch_kernel<Body, A...>, kLaunchTX * kLaunchTY, smem) !=
          cudaSuccess ||
      n < 1)
    n = 1;
  return n;
}

// ---- double -> F64i ----------------------------------------------------------------------
template <class B>
struct Rebind {
  using type = B;
  static constexpr bool on = false;
};
template <template <class> class K>
struct Rebind<K<double>> {
  using type = K<F64i>;
  static constexpr bool on = true;
};
template <template <class, int> class K, int N>
struct Rebind<K<double, N>> {
  using type = K<F64i, N>;
  static constexpr bool on = true;
};
template <template <class, int, int> class K, int N, int M>
struct Rebind<K<double, N, M>> {
  using type = K<F64i, N, M>;
  static constexpr bool on = true;
};

template <class A>
struct ArgMap {
  using type = A;
  static A conv(A a) { return a; }
};
template <>
struct ArgMap<double> {
  using type = F64i;
  static F64i conv(double a) { return F64i(a); }
};
template <>
struct ArgMap<double*> {
  using type = F64i*;
  static F64i* conv(double* a) { return reinterpret_cast<F64i*>(a); }
};
template <>
struct ArgMap<const double*> {
  using type = const F64i*;
  static const F64i* conv(const double* a) { return reinterpret_cast<const F64i*>(a); }
};
template <template <class> class X>
struct ArgMap<X<double>> {
  using type = X<F64i>;
  static X<F64i> conv(const X<double>& a) {
    static_assert(sizeof(X<F64i>) == sizeof(X<double>), "F64i twin must have the same layout");
    X<F64i> r;
    memcpy(static_cast<void*>(&r), &a, sizeof(r));
    return r;
  }
};
template <template <class> class X>
struct ArgMap<X<double>*> {
  using type = X<F64i>*;
  static X<F64i>* conv(X<double>* a) { return reinterpret_cast<X<F64i>*>(a); }
};
template <template <class> class X>
struct ArgMap<const X<double>*> {
  using type = const X<F64i>*;
  static const X<F64i>* conv(const X<double>* a) { return reinterpret_cast<const X<F64i>*>(a); }
};

template <class Body, class... A>
oeb_status launch_as(dim3 grid, size_t smem, cudaStream_t st, A... a) {
  if (grid.x == 0 || grid.y == 0 || grid.z == 0) return OEB_OK;
  if (Recorder* r = recorder()) {
    LaunchRecord rec;
    rec.launcher = &batch_launch<Body, A...>;
    rec.shape_tag = ShapeOf<Body>::value;
    rec.grid_launcher = &grid_launch_packed<Body, A...>;
    rec.occupancy = &batch_occupancy<Body, A...>;
    rec.grid = grid;
    rec.smem = smem;
    const Pack<A...> p = make_pack(a...);
    rec.args.resize(sizeof(p));
    memcpy(rec.args.data(), &p, sizeof(p));
    if constexpr (StepOpOf<Body>::value >= 0) {
      const RunPack<Body> rp = PackFrom<RunPack<Body>>::make(a...);
      rec.step_op = StepOpOf<Body>::value;
      rec.step_args.resize(sizeof(rp));
      memcpy(rec.step_args.data(), &rp, sizeof(rp));
    }
    r->records.push_back(std::move(rec));
    return OEB_OK;
  }
  if (smem > 48 * 1024) OEB_TRY(ensure_dyn_smem((const void*)grid_entry<Body, A...>(), (int)smem));
  grid_entry<Body, A...>()<<<grid, dim3(kLaunchTX, kLaunchTY), smem, st>>>(a...);
  return after_launch();
}

template <class Body, class... A>
oeb_status launch(dim3 grid, size_t smem, cudaStream_t st, A... a) {
  if constexpr (Rebind<Body>::on) {
    return launch_as<typename Rebind<Body>::type, typename ArgMap<A>::type...>(grid, smem, st, ArgMap<A>::conv(a)...);
  } else {
    return launch_as<Body, A...>(grid, smem, st, a...);
  }
}

}  // namespace oeb
