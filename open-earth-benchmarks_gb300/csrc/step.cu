// step.cu -- the step kernel: the chained step of every member of a batch, forward and adjoint,
// in ONE persistent launch (the tables and the protocol are described in step.cuh).
//
// The kernel calls the bodies of the chained step from one switch, so this file includes the
// stencil files with OEB_BODIES_ONLY: their bodies and device helpers, each file in a namespace
// of its own, without their entry points.  Each body is compiled here as it is in its own file
// (the same source, the same flags: --fmad=false), so a tile computes the same bits in either
// kernel.  Each body is a non-inlined function: the kernel is a loop around the switch, and the
// register count is the largest body's.
//
// Memory ordering between the tasks of a member: a CTA that finishes a tile synchronises its
// threads and then, from one thread, fences at GPU scope and counts the tile done (a release);
// a CTA whose task waits reads that count with ld.acquire.gpu from one thread, then
// synchronises its threads before any of them reads the previous task's outputs.
// Later tasks read what earlier tasks of this launch wrote: every body's loads are coherent
// here (ld() in stencil_util.cuh), not the non-coherent path of the single-kernel builds.
#define OEB_COHERENT_LOADS 1

#include <algorithm>

#include "launch.cuh"
#include "step.cuh"

// CTAs an SM the kernel is compiled for: 2 leaves every body its registers (the heaviest, the
// advection adjoint's terms, take 128); 3 and 4 cap them at 80 and 64, which spills a little
// in the heaviest bodies.  The library is built with all three (step_c2.o, step_c3.o,
// step_c4.o); the form autotuner times each.  Every name this file defines carries the
// count, so the three objects link side by side.
#ifndef OEB_STEP_MIN_CTAS
#define OEB_STEP_MIN_CTAS 2
#endif
#define OEB_STEP_CAT2(a, b) a##b
#define OEB_STEP_CAT(a, b) OEB_STEP_CAT2(a, b)

#define OEB_BODIES_ONLY 1
#define OEB_BODIES_NS OEB_STEP_CAT(step_fws_c, OEB_STEP_MIN_CTAS)
#include "k_fastwavesuv.cu"
#undef OEB_BODIES_NS
#define OEB_BODIES_NS OEB_STEP_CAT(step_fv_c, OEB_STEP_MIN_CTAS)
#include "k_fvtp2d.cu"
#undef OEB_BODIES_NS
#define OEB_BODIES_NS OEB_STEP_CAT(step_hd_c, OEB_STEP_MIN_CTAS)
#include "k_hdiff.cu"
#undef OEB_BODIES_NS
#define OEB_BODIES_NS OEB_STEP_CAT(step_pw_c, OEB_STEP_MIN_CTAS)
#include "k_pointwise.cu"
#undef OEB_BODIES_NS
#define OEB_BODIES_NS OEB_STEP_CAT(step_ch_c, OEB_STEP_MIN_CTAS)
#include "chain.cu"
#undef OEB_BODIES_NS

namespace oeb {
namespace step_fws = OEB_STEP_CAT(step_fws_c, OEB_STEP_MIN_CTAS);
namespace step_fv = OEB_STEP_CAT(step_fv_c, OEB_STEP_MIN_CTAS);
namespace step_hd = OEB_STEP_CAT(step_hd_c, OEB_STEP_MIN_CTAS);
namespace step_pw = OEB_STEP_CAT(step_pw_c, OEB_STEP_MIN_CTAS);
namespace step_ch = OEB_STEP_CAT(step_ch_c, OEB_STEP_MIN_CTAS);
namespace OEB_STEP_CAT(step_c, OEB_STEP_MIN_CTAS) {

template <class... B>
struct OpList {};

// Every body the chained step records, in both precisions (FP64 runs as F64i), with the FP32
// adjoints in either form (oeb_set_adjoint_tiles).
using StepBodies = OpList<
    step_ch::combine_kernel<F64i>, step_ch::combine_kernel<float>,
    step_fws::fastwavesuv_kernel<F64i>, step_fws::fastwavesuv_kernel<float>,
    step_fws::fastwavesuv_adj_terms_kernel<F64i>, step_fws::fastwavesuv_adj_kernel<F64i, 0>,
    step_fws::fastwavesuv_adj_kernel<float, 1>,
    step_pw::hadv_kernel<F64i, 5, 0>, step_pw::hadv_kernel<F64i, 5, 1>, step_pw::hadv_kernel<F64i, 5, 2>,
    step_pw::hadv_kernel<float, 5, 0>, step_pw::hadv_kernel<float, 5, 1>, step_pw::hadv_kernel<float, 5, 2>,
    step_pw::hadv_adj_terms_kernel<F64i, 5, 0>, step_pw::hadv_adj_terms_kernel<F64i, 5, 1>,
    step_pw::hadv_adj_terms_kernel<F64i, 5, 2>, step_pw::hadv_adj_terms_kernel<float, 5, 0>,
    step_pw::hadv_adj_terms_kernel<float, 5, 1>, step_pw::hadv_adj_terms_kernel<float, 5, 2>,
    step_pw::hadv_adj_gather_kernel<F64i, 5>, step_pw::hadv_adj_gather_kernel<float, 5>,
    step_hd::hdiffsmag_kernel<F64i>, step_hd::hdiffsmag_kernel<float>,
    step_hd::hdiffsmag_adj_terms_kernel<F64i>, step_hd::hdiffsmag_adj_ts_kernel<F64i>,
    step_hd::hdiffsmag_adj_gather_kernel<F64i>, step_hd::hdiffsmag_adj_f32,
    step_hd::hdiffsmag_adj_terms_kernel<float>, step_hd::hdiffsmag_adj_ts_kernel<float>,
    step_hd::hdiffsmag_adj_gather_kernel<float>, step_pw::hadv_adj_f32<5>,
    step_fws::fastwavesuv_adj_terms_kernel<float>, step_fws::fastwavesuv_adj_kernel<float, 0>,
    step_fv::fvtp2d_q_kernel<F64i>, step_fv::fvtp2d_q_kernel<float>, step_fv::fvtp2d_flux_kernel<F64i>,
    step_fv::fvtp2d_fused_kernel<float>, step_fv::fvtp2d_adj_qij_kernel<F64i>,
    step_fv::fvtp2d_adj_qij_kernel<float>, step_fv::fvtp2d_adj_f2_kernel<F64i>,
    step_fv::fvtp2d_adj_f2_kernel<float>, step_fv::fvtp2d_adj_q_kernel<F64i>,
    step_fv::fvtp2d_adj_q_kernel<float>>;

template <class... B>
constexpr bool ids_valid(OpList<B...>) {
  const int ids[] = {B::kStepOp...};
  for (size_t i = 0; i < sizeof...(B); ++i) {
    if (ids[i] < 0 || ids[i] >= kStepOps) return false;
    for (size_t j = 0; j < i; ++j)
      if (ids[i] == ids[j]) return false;
  }
  return true;
}
static_assert(ids_valid(StepBodies{}), "every body of the step kernel needs a distinct kStepOp");

template <class... B>
bool has_id(int op, OpList<B...>) {
  return ((op == B::kStepOp) || ...);
}

// One tile of a body, its arguments read from the table.
template <class Body>
__device__ __noinline__ void op_call(const uint3& blk, const unsigned char* args) {
  const RunPack<Body> p = *reinterpret_cast<const RunPack<Body>*>(args);
  call_pack<Body>(blk, p);
}

template <class... B>
__device__ __forceinline__ void dispatch(int op, const uint3& blk, const unsigned char* args, OpList<B...>) {
  (void)(((op == B::kStepOp) && (op_call<B>(blk, args), true)) || ...);
}

__device__ __forceinline__ unsigned ld_acquire(const unsigned* p) {
  unsigned v;
  asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}

__device__ __forceinline__ unsigned long long now_ns() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

// Polls of one wait at most, whatever the timer reads: with the sleep between polls, several
// seconds.
constexpr unsigned kMaxPolls = 1u << 25;

// Waits (one thread) until `need` tiles of task `dep` are done.  False if the wait gave up --
// past the plan's limit, or because another CTA's wait gave up first; the first to give up
// sets the status word and records its task.
// A wait that had to poll adds its duration (in us) and one to the run's wait statistics.
__device__ bool wait_done(const StepParams& P, int dep, unsigned need, int task) {
  if (ld_acquire(P.done + dep) >= need) return true;
  const unsigned long long t0 = now_ns();
  for (unsigned n = 0; n < kMaxPolls; ++n) {
    __nanosleep(128);
    if (ld_acquire(P.done + dep) >= need) {
      atomicAdd(P.ctl + 3, (unsigned)((now_ns() - t0) >> 10));
      atomicAdd(P.ctl + 4, 1u);
      return true;
    }
    if (*(volatile unsigned*)(P.ctl + 1) != 0u) return false;
    if (now_ns() - t0 > P.wait_ns) break;
  }
  if (atomicCAS(P.ctl + 1, 0u, (unsigned)OEB_ERR_TIMEOUT) == 0u) atomicExch(P.ctl + 2, (unsigned)task);
  return false;
}

constexpr int kStepMinCtas = OEB_STEP_MIN_CTAS;

__global__ void __launch_bounds__(kLaunchTX* kLaunchTY, kStepMinCtas) step_kernel(const StepParams P) {
  __shared__ int s_task, s_item;
  const bool lead = threadIdx.x == 0 && threadIdx.y == 0;
  for (;;) {
    if (lead) {
      int task = -1, item = -1;
      if (*(volatile unsigned*)(P.ctl + 1) == 0u) {
        item = (int)atomicAdd(P.ctl, 1u);
        if (item < P.total) {
          int lo = 0, hi = P.ntasks - 1;  // the last task whose first item is <= item
          while (lo < hi) {
            const int mid = (lo + hi + 1) >> 1;
            if (P.tasks[mid].first <= item) lo = mid; else hi = mid - 1;
          }
          task = lo;
          const int dep = P.tasks[lo].dep;
          if (dep >= 0 && !wait_done(P, dep, P.tasks[lo].need, lo)) task = -1;
        }
      }
      s_task = task;
      s_item = item;
    }
    __syncthreads();
    const int task = s_task;
    if (task < 0) return;
    const StepTask t = P.tasks[task];
    const int local = s_item - t.first;
    const int plane = t.gx * t.gy;
    const uint3 blk = make_uint3((unsigned)(local % t.gx), (unsigned)((local % plane) / t.gx),
                                 (unsigned)(local / plane));
    dispatch(t.op, blk, P.table + t.args, StepBodies{});
    __syncthreads();  // the tile's writes are done, and the shared memory is free again
    if (lead) {
      __threadfence();
      atomicAdd(P.done + task, 1u);
    }
  }
}

}  // namespace step_cN
using namespace OEB_STEP_CAT(step_c, OEB_STEP_MIN_CTAS);

oeb_status OEB_STEP_CAT(step_launch_c, OEB_STEP_MIN_CTAS)(const StepParams& p, int ctas, size_t smem,
                                                          cudaStream_t st) {
  if (smem > 48 * 1024) OEB_TRY(ensure_dyn_smem((const void*)step_kernel, (int)smem));
  step_kernel<<<ctas, dim3(kLaunchTX, kLaunchTY), smem, st>>>(p);
  return after_launch();
}

int OEB_STEP_CAT(step_occupancy_c, OEB_STEP_MIN_CTAS)(size_t smem) {
  if (smem > 48 * 1024 && ensure_dyn_smem((const void*)step_kernel, (int)smem) != OEB_OK) return 1;
  int n = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, step_kernel, kLaunchTX * kLaunchTY, smem) != cudaSuccess ||
      n < 1)
    n = 1;
  return n;
}

#if OEB_STEP_MIN_CTAS == 2
bool step_has_op(int op) { return has_id(op, StepBodies{}); }
#endif

}  // namespace oeb
