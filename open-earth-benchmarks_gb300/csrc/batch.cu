// batch.cu -- batched ensembles: the chained step of many uneven members as persistent launches.
//
// A batch plan is built in three passes over the members (each member has its own chain
// plan, i.e. its own workspace):
//   1. sizing: every member's forward and adjoint step is recorded with a placeholder arena,
//      which measures the scratch the adjoint stencils take (the arena is a stack: a call's
//      scratch is reused by the next call);
//   2. recording: the same calls with the member's region of the real arena; every kernel
//      launch of the step becomes a LaunchRecord (grid, dynamic shared memory, arguments);
//   3. tables: position p of the recorded sequences is the same kernel for every member of
//      one precision, so for each position and precision the plan uploads one table of
//      (member, tile) items -- members largest first -- and one array of argument packs.
// A run replays the positions in order, each as one batch_kernel launch (launch.cuh) whose
// CTAs walk the items; FP64 members on the caller's stream, FP32 members on a second stream.
//
// The autotuner records the step again with other k-blockings (kb: k-levels per tile of the
// kernels that take one) and times, for every position and precision, each kb in three forms:
// the batched launch as a single persistent wave (occupancy x SMs CTAs), the batched launch
// with one CTA per tile, and plain per-member launches of the recorded grids (the same tiles,
// one ordinary launch per member: no item search, arguments in the kernel's parameter space).
// It keeps the fastest, so a tuned plan is never slower, position by position, than launching
// the members one by one.
//
// The one-launch form (oeb_batch_set_form) runs a whole run as ONE launch of the step kernel
// (step.cu): every member's recorded launches, forward then adjoint, become tasks in one ticket
// order, each waiting on the device (bounded) for its member's previous task.
#include <algorithm>
#include <new>
#include <vector>

#include "launch.cuh"
#include "oeb_common.cuh"
#include "step.cuh"

namespace {

struct Member {
  int elem = 8;
  oeb_domain dom{};
  oeb_chain_scalars s{};
  // descriptor copies, so the plan can record again (autotuning) after the caller's structs
  // are gone; the fields structs below point into these
  std::vector<oeb_memref3d_f64> d3;
  std::vector<oeb_memref1d_f64> d1;
  std::vector<oeb_memref3d_f32> f3;
  std::vector<oeb_memref1d_f32> f1;
  oeb_chain_fields_f64 fields64{};
  oeb_chain_fields_f32 fields32{};
  oeb_memref3d_f64 io64[10]{};  // uout vout fx1 fy1 uoutb voutb fx1b fy1b ub vb
  oeb_memref3d_f32 io32[10]{};
  oeb_chain_plan* chain = nullptr;
  size_t arena_off = 0, arena_size = 0;
};

// One batched launch of a run.
struct Slot {
  oeb::BatchLaunchFn fn = nullptr;
  oeb::GridLaunchFn gfn = nullptr;
  int side = 0;  // 0: FP64 members on the caller's stream, 1: FP32 members on the plan's stream
  int members = 0, total = 0;
  size_t smem = 0;
  int occupancy = 1;
  size_t tiles_off = 0, args_off = 0;  // into the device table buffer
  int ctas = 0;
  int kb = 0;
  int shape = 0;      // the tile shape the slot was recorded with (tuned_shape)
  int shape_tag = 0;  // its kernel's shape (0: the kernel takes none, so `shape` made no difference)
  bool per_member = false;  // run as one ordinary launch per member
  // per member, in slot order: grid, dynamic shared memory and argument pack (host copy)
  std::vector<dim3> grids;
  std::vector<size_t> smems, arg_offs;
  std::vector<unsigned char> host_args;
};

}  // namespace

struct oeb_batch_plan {
  int modes = 0;
  int device = 0;
  int sms = 0;
  std::vector<Member> members;
  char* arena = nullptr;
  size_t arena_bytes = 0;
  char* tables = nullptr;
  size_t table_bytes = 0;
  std::vector<Slot> slots;  // forward positions, then adjoint positions
  cudaStream_t side = nullptr;
  cudaEvent_t fork = nullptr, join = nullptr;
  // the one-launch form (step.cu): every member's step in one launch of the step kernel
  int fusion = 0;         // the fusion grouping its launches were recorded with (OEB_FUSE_*)
  size_t base_slots = 0;  // slots of the grouping 0 (in the signature, which any grouping shares)
  int form = OEB_BATCH_FORM_PER_LAUNCH;
  int one_kb = -1;          // the k-blocking its tasks were recorded with (-1: not built)
  char* one_buf = nullptr;  // tasks, argument packs, then the done counters and control words
  size_t one_bytes = 0, one_done_off = 0, one_ctl_off = 0;
  int one_tasks = 0, one_total = 0, one_ctas = 0;
  int one_per_sm = 2;  // the step kernel build: CTAs an SM (2, 3 or 4)
  size_t one_smem = 0;
  oeb::StepTask one_first{};  // task 0 as built (oeb_batch_withhold changes it on the device)
  bool withheld = false;
  unsigned long long wait_ns = 2000000000ull;
};

namespace oeb {
namespace {

constexpr int kModes[2] = {OEB_CHAIN_FORWARD, OEB_CHAIN_ADJOINT};

template <class M3, class M1, class F>
void copy_fields(const F* src, std::vector<M3>& d3, std::vector<M1>& d1, F* dst) {
  d3.reserve(17);
  d1.reserve(10);
  auto c3 = [&](const M3* m) -> const M3* {
    if (!m) return nullptr;
    d3.push_back(*m);
    return &d3.back();
  };
  auto c1 = [&](const M1* m) -> const M1* {
    if (!m) return nullptr;
    d1.push_back(*m);
    return &d1.back();
  };
  dst->u = c3(src->u);
  dst->v = c3(src->v);
  dst->utens = c3(src->utens);
  dst->vtens = c3(src->vtens);
  dst->wgtfac = c3(src->wgtfac);
  dst->ppuv = c3(src->ppuv);
  dst->hhl = c3(src->hhl);
  dst->rho = c3(src->rho);
  dst->fx = c1(src->fx);
  dst->acrlat0 = c1(src->acrlat0);
  dst->acrlat1 = c1(src->acrlat1);
  dst->tgrlatda0 = c1(src->tgrlatda0);
  dst->tgrlatda1 = c1(src->tgrlatda1);
  dst->mask = c3(src->mask);
  dst->crlavo = c1(src->crlavo);
  dst->crlavu = c1(src->crlavu);
  dst->crlato = c1(src->crlato);
  dst->crlatu = c1(src->crlatu);
  dst->smag_acrlat0 = c1(src->smag_acrlat0);
  dst->crx = c3(src->crx);
  dst->cry = c3(src->cry);
  dst->ra_x = c3(src->ra_x);
  dst->ra_y = c3(src->ra_y);
  dst->xfx = c3(src->xfx);
  dst->yfx = c3(src->yfx);
  dst->area = c3(src->area);
}

template <class M3>
oeb_status copy_io(const oeb_batch_member& src, int modes, M3* io) {
  const void* p[10] = {src.uout, src.vout, src.fx1, src.fy1, src.uoutb, src.voutb, src.fx1b, src.fy1b, src.ub, src.vb};
  for (int q = 0; q < 10; ++q) {
    const bool needed = q < 4 ? (modes & OEB_CHAIN_FORWARD) : (modes & OEB_CHAIN_ADJOINT);
    if (!p[q]) {
      if (needed) return OEB_ERR_NULL;
      continue;
    }
    io[q] = *static_cast<const M3*>(p[q]);
  }
  return OEB_OK;
}

// Records member m's step for `mode` into rec (launches nothing).
oeb_status record(Member& m, int mode, Recorder* rec) {
  set_recorder(rec);
  oeb_status st;
  if (m.elem == 8) {
    const oeb_memref3d_f64* io = m.io64;
    st = mode == OEB_CHAIN_FORWARD
             ? oeb_chain_forward_f64(m.chain, &m.fields64, &m.s, &io[0], &io[1], &io[2], &io[3], nullptr)
             : oeb_chain_adj_f64(m.chain, &m.fields64, &m.s, &io[4], &io[5], &io[6], &io[7], &io[8], &io[9], nullptr);
  } else {
    const oeb_memref3d_f32* io = m.io32;
    st = mode == OEB_CHAIN_FORWARD
             ? oeb_chain_forward_f32(m.chain, &m.fields32, &m.s, &io[0], &io[1], &io[2], &io[3], nullptr)
             : oeb_chain_adj_f32(m.chain, &m.fields32, &m.s, &io[4], &io[5], &io[6], &io[7], &io[8], &io[9], nullptr);
  }
  set_recorder(nullptr);
  return st;
}

// Recorded sequences of every member for every mode in the plan, with k-blocking kb and tile
// shape `shape`.
oeb_status record_all(oeb_batch_plan* p, int kb, int shape, std::vector<std::vector<std::vector<LaunchRecord>>>* out) {
  out->assign(2, {});
  for (int mi = 0; mi < 2; ++mi) {
    if (!(p->modes & kModes[mi])) continue;
    (*out)[mi].resize(p->members.size());
    for (size_t i = 0; i < p->members.size(); ++i) {
      Member& m = p->members[i];
      Recorder rec;
      rec.kb = kb;
      rec.shape = shape;
      rec.fusion = p->fusion;
      rec.arena = p->arena + m.arena_off;
      rec.arena_bytes = m.arena_size;
      OEB_TRY(record(m, kModes[mi], &rec));
      (*out)[mi][i] = std::move(rec.records);
    }
  }
  return OEB_OK;
}

// Slots and host tables of one recording: for every position, one slot per precision.  The
// members of one precision record the same launches; the two precisions may record different
// numbers of them (FP32 fvtp2d is one launch, FP64 two), so positions count per precision.
oeb_status build_slots(oeb_batch_plan* p, const std::vector<std::vector<std::vector<LaunchRecord>>>& seq, int kb,
                       int shape, std::vector<Slot>* slots, std::vector<char>* host, size_t base) {
  for (int mi = 0; mi < 2; ++mi) {
    if (!(p->modes & kModes[mi])) continue;
    const auto& per = seq[mi];
    std::vector<int> members_of[2];
    size_t len_of[2] = {0, 0};
    for (int side = 0; side < 2; ++side) {
      for (size_t i = 0; i < p->members.size(); ++i)
        if (p->members[i].elem == (side ? 4 : 8)) members_of[side].push_back((int)i);
      if (members_of[side].empty()) continue;
      len_of[side] = per[members_of[side][0]].size();
      for (int i : members_of[side])
        if (per[i].size() != len_of[side]) return OEB_ERR_UNSUPPORTED;
    }
    const size_t len = std::max(len_of[0], len_of[1]);
    for (size_t pos = 0; pos < len; ++pos) {
      for (int side = 0; side < 2; ++side) {
        if (pos >= len_of[side]) continue;
        std::vector<int> who = members_of[side];
        const LaunchRecord& r0 = per[who[0]][pos];
        for (int i : who)
          if (per[i][pos].launcher != r0.launcher || per[i][pos].args.size() != r0.args.size())
            return OEB_ERR_UNSUPPORTED;
        auto tiles_of = [&](int i) {
          const dim3 g = per[i][pos].grid;
          return (int64_t)g.x * g.y * g.z;
        };
        std::stable_sort(who.begin(), who.end(), [&](int a, int b) { return tiles_of(a) > tiles_of(b); });
        Slot sl;
        sl.fn = r0.launcher;
        sl.gfn = r0.grid_launcher;
        sl.side = side;
        sl.members = (int)who.size();
        sl.smem = 0;
        sl.kb = kb;
        sl.shape = shape;
        sl.shape_tag = r0.shape_tag;
        int64_t total = 0;
        std::vector<BatchTile> tiles;
        std::vector<char> args;
        for (int i : who) {
          const LaunchRecord& r = per[i][pos];
          tiles.push_back(BatchTile{(int)total, (int)r.grid.x, (int)r.grid.y, 0});
          total += tiles_of(i);
          args.insert(args.end(), r.args.begin(), r.args.end());
          sl.smem = std::max(sl.smem, r.smem);
          sl.grids.push_back(r.grid);
          sl.smems.push_back(r.smem);
          const size_t at = (sl.host_args.size() + 15) & ~size_t(15);  // packs 16-byte aligned
          sl.host_args.resize(at + r.args.size());
          memcpy(sl.host_args.data() + at, r.args.data(), r.args.size());
          sl.arg_offs.push_back(at);
        }
        if (total > INT32_MAX) return OEB_ERR_TOO_LARGE;
        sl.total = (int)total;
        sl.occupancy = r0.occupancy(sl.smem);
        sl.ctas = std::min<int64_t>(total, (int64_t)sl.occupancy * p->sms);
        auto put = [&](const void* src, size_t n) {
          const size_t at = (host->size() + 255) & ~size_t(255);
          host->resize(at + n);
          memcpy(host->data() + at, src, n);
          return base + at;
        };
        sl.tiles_off = put(tiles.data(), tiles.size() * sizeof(BatchTile));
        sl.args_off = put(args.data(), args.size());
        slots->push_back(sl);
      }
    }
  }
  return OEB_OK;
}

// Replaces the plan's device tables by `host`.  The new buffer is allocated and filled
// first, and the old one freed only after the device is idle (a run in flight may still read
// it): on any error the plan keeps its tables, which still match its slots.
oeb_status upload(oeb_batch_plan* p, const std::vector<char>& host) {
  char* tables = nullptr;
  cudaError_t e = cudaMalloc(&tables, std::max<size_t>(host.size(), 256));
  if (e != cudaSuccess) {
    cuda_fail(e);
    return OEB_ERR_ALLOC;
  }
  e = cudaMemcpy(tables, host.data(), host.size(), cudaMemcpyHostToDevice);
  if (e == cudaSuccess && p->tables) e = cudaDeviceSynchronize();
  if (e != cudaSuccess) {
    cudaFree(tables);
    return cuda_fail(e);
  }
  if (p->tables) cudaFree(p->tables);
  p->tables = tables;
  p->table_bytes = host.size();
  return OEB_OK;
}

oeb_status run_slot(oeb_batch_plan* p, const Slot& sl, int ctas, bool per_member, cudaStream_t main) {
  const cudaStream_t s = sl.side ? p->side : main;
  if (per_member) {
    for (size_t i = 0; i < sl.grids.size(); ++i)
      OEB_TRY(sl.gfn(sl.host_args.data() + sl.arg_offs[i], sl.grids[i], sl.smems[i], s));
    return OEB_OK;
  }
  return sl.fn(reinterpret_cast<const BatchTile*>(p->tables + sl.tiles_off), sl.members, sl.total,
               p->tables + sl.args_off, sl.smem, ctas, s);
}

// ---- the one-launch form --------------------------------------------------------------
// The ticket order of the members' tasks: member m has counts[m] tasks, taken in order; the
// result lists (member, position) pairs by the fraction of its member's step each task ends
// ((position + 1/2) / count), larger members (points) first at equal fractions.  Every
// member's tasks keep their order, so a task's predecessor always holds an earlier ticket.
std::vector<std::pair<int, int>> step_order(const std::vector<int>& counts, const std::vector<int64_t>& points) {
  const int nm = (int)counts.size();
  std::vector<int> by(nm), rank(nm);
  for (int i = 0; i < nm; ++i) by[i] = i;
  std::stable_sort(by.begin(), by.end(), [&](int a, int b) { return points[a] > points[b]; });
  for (int r = 0; r < nm; ++r) rank[by[r]] = r;
  struct Pending {
    int member, pos;
    double key;
  };
  std::vector<Pending> all;
  for (int i = 0; i < nm; ++i)
    for (int q = 0; q < counts[i]; ++q) all.push_back(Pending{i, q, (q + 0.5) / (double)counts[i]});
  std::stable_sort(all.begin(), all.end(), [&](const Pending& a, const Pending& b) {
    if (a.key != b.key) return a.key < b.key;
    return rank[a.member] < rank[b.member];
  });
  std::vector<std::pair<int, int>> out;
  out.reserve(all.size());
  for (const Pending& a : all) out.emplace_back(a.member, a.pos);
  return out;
}

// Records every member's step with k-blocking kb (the default tile shape) and builds the
// step kernel's tables: each member's launches, forward then adjoint, become its tasks, each
// waiting for the member's previous one.  The tasks of all members are merged in the order of
// the fraction of its member's step a task ends, larger members first at equal fractions;
// every member's tasks keep their order, which is all the step kernel needs (step.cuh).  The
// new tables are uploaded into a buffer of their own and replace the old ones only when all
// is done, so a failure leaves the plan as it was.
oeb_status build_one(oeb_batch_plan* p, int kb) {
  std::vector<std::vector<std::vector<LaunchRecord>>> seq;
  OEB_TRY(record_all(p, kb, 0, &seq));
  const int nm = (int)p->members.size();
  std::vector<std::vector<const LaunchRecord*>> lists(nm);  // each member's launches, forward then adjoint
  std::vector<int> counts(nm);
  std::vector<int64_t> points(nm);
  size_t smem = 0;
  for (int i = 0; i < nm; ++i) {
    for (int mi = 0; mi < 2; ++mi)
      if (p->modes & kModes[mi])
        for (const LaunchRecord& r : seq[mi][i]) lists[i].push_back(&r);
    for (const LaunchRecord* r : lists[i]) {
      if (r->step_op < 0 || !step_has_op(r->step_op)) return OEB_ERR_UNSUPPORTED;
      smem = std::max(smem, r->smem);
    }
    counts[i] = (int)lists[i].size();
    points[i] = (int64_t)p->members[i].dom.nx * p->members[i].dom.ny * p->members[i].dom.nz;
  }
  const std::vector<std::pair<int, int>> order = step_order(counts, points);
  if (order.empty()) return OEB_ERR_UNSUPPORTED;
  const int ntasks = (int)order.size();
  std::vector<StepTask> tasks(ntasks);
  std::vector<int> last(nm, -1);
  std::vector<char> packs;
  int64_t total = 0;
  for (int t = 0; t < ntasks; ++t) {
    struct {
      int member;
      const LaunchRecord* r;
    } a{order[t].first, lists[order[t].first][order[t].second]};
    const dim3 g = a.r->grid;
    const int64_t tiles = (int64_t)g.x * g.y * g.z;
    if (tiles > INT32_MAX || total + tiles > INT32_MAX) return OEB_ERR_TOO_LARGE;
    StepTask& k = tasks[t];
    k.first = (int)total;
    k.tiles = (int)tiles;
    k.gx = (int)g.x;
    k.gy = (int)g.y;
    k.op = a.r->step_op;
    k.dep = last[a.member];
    k.need = k.dep >= 0 ? (unsigned)tasks[k.dep].tiles : 0u;
    const size_t at = (packs.size() + 15) & ~size_t(15);  // packs 16-byte aligned
    packs.resize(at + a.r->step_args.size());
    memcpy(packs.data() + at, a.r->step_args.data(), a.r->step_args.size());
    k.args = (int64_t)at;  // made absolute below
    last[a.member] = t;
    total += tiles;
  }
  auto up = [](size_t n) { return (n + 255) & ~size_t(255); };
  const size_t tasks_bytes = up(sizeof(StepTask) * ntasks);
  const size_t done_off = tasks_bytes + up(packs.size());
  const size_t ctl_off = done_off + up(sizeof(unsigned) * (ntasks + 1));
  const size_t bytes = ctl_off + up(sizeof(unsigned) * kStepCtlWords);
  for (StepTask& k : tasks) k.args += (int64_t)tasks_bytes;
  std::vector<char> host(done_off, 0);
  memcpy(host.data(), tasks.data(), sizeof(StepTask) * ntasks);
  memcpy(host.data() + tasks_bytes, packs.data(), packs.size());
  char* buf = nullptr;
  cudaError_t e = cudaMalloc(&buf, bytes);
  if (e != cudaSuccess) {
    cuda_fail(e);
    return OEB_ERR_ALLOC;
  }
  e = cudaMemcpy(buf, host.data(), host.size(), cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaMemset(buf + done_off, 0, bytes - done_off);
  if (e == cudaSuccess && p->one_buf) e = cudaDeviceSynchronize();
  if (e != cudaSuccess) {
    cudaFree(buf);
    return cuda_fail(e);
  }
  if (p->one_buf) cudaFree(p->one_buf);
  p->one_buf = buf;
  p->one_bytes = bytes;
  p->one_done_off = done_off;
  p->one_ctl_off = ctl_off;
  p->one_tasks = ntasks;
  p->one_total = (int)total;
  p->one_smem = smem;
  p->one_ctas = step_occupancy(p->one_per_sm, smem) * p->sms;
  p->one_first = tasks[0];
  p->one_kb = kb;
  p->withheld = false;
  return OEB_OK;
}

oeb_status run_one(oeb_batch_plan* p, cudaStream_t st) {
  OEB_CUDA_TRY(cudaMemsetAsync(p->one_buf + p->one_done_off, 0, p->one_bytes - p->one_done_off, st));
  StepParams P;
  P.tasks = reinterpret_cast<const StepTask*>(p->one_buf);
  P.ntasks = p->one_tasks;
  P.total = p->one_total;
  P.table = reinterpret_cast<const unsigned char*>(p->one_buf);
  P.done = reinterpret_cast<unsigned*>(p->one_buf + p->one_done_off);
  P.ctl = reinterpret_cast<unsigned*>(p->one_buf + p->one_ctl_off);
  P.wait_ns = p->wait_ns;
  return step_launch(p->one_per_sm, P, p->one_ctas, p->one_smem, st);
}

oeb_status run_per_launch(oeb_batch_plan* p, cudaStream_t st);

oeb_status run(oeb_batch_plan* p, cudaStream_t st) {
  if (p->form == OEB_BATCH_FORM_ONE_LAUNCH) return run_one(p, st);
  return run_per_launch(p, st);
}

// The step kernel build with `per_sm` CTAs an SM, sized to fill every SM.
void use_variant(oeb_batch_plan* p, int per_sm) {
  p->one_per_sm = per_sm;
  if (p->one_buf) p->one_ctas = step_occupancy(per_sm, p->one_smem) * p->sms;
}

oeb_status set_form(oeb_batch_plan* p, int form, int kb, int per_sm) {
  if (form != OEB_BATCH_FORM_PER_LAUNCH && form != OEB_BATCH_FORM_ONE_LAUNCH) return OEB_ERR_ARGUMENT;
  if (form == OEB_BATCH_FORM_ONE_LAUNCH) {
    if (kb != 0 && kb != 1 && kb != 2 && kb != 4 && kb != 8) return OEB_ERR_ARGUMENT;
    if (per_sm == 0) per_sm = 2;
    if (!step_variant(per_sm)) return OEB_ERR_ARGUMENT;
    const int prev = p->one_per_sm;
    p->one_per_sm = per_sm;
    if (kb != p->one_kb) {
      const oeb_status b = build_one(p, kb);
      if (b != OEB_OK) {
        p->one_per_sm = prev;
        return b;
      }
    }
    use_variant(p, per_sm);
  }
  p->form = form;
  return OEB_OK;
}

// Times a whole run of the plan as it stands, `reps` times after one untimed run.
oeb_status time_runs(oeb_batch_plan* p, cudaStream_t st, int reps, float* ms) {
  cudaEvent_t e0, e1;
  OEB_CUDA_TRY(cudaEventCreate(&e0));
  if (cudaEventCreate(&e1) != cudaSuccess) {
    cudaEventDestroy(e0);
    return cuda_fail(cudaGetLastError());
  }
  oeb_status r = run(p, st);
  if (r == OEB_OK && cudaEventRecord(e0, st) != cudaSuccess) r = cuda_fail(cudaGetLastError());
  for (int i = 0; i < reps && r == OEB_OK; ++i) r = run(p, st);
  if (r == OEB_OK && (cudaEventRecord(e1, st) != cudaSuccess || cudaEventSynchronize(e1) != cudaSuccess))
    r = cuda_fail(cudaGetLastError());
  if (r == OEB_OK) {
    cudaEventElapsedTime(ms, e0, e1);
    *ms /= (float)reps;
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  return r;
}

// The launch form and, for the one-launch form, the k-blocking and the step kernel build, by
// timing whole runs: the per-launch form as the plan stands (with the choices of
// oeb_batch_autotune, if it ran), then the one-launch form with every k-blocking the
// recordings take, each with every build (2, 3, 4 CTAs an SM).  Keeps the fastest.
oeb_status autotune_form(oeb_batch_plan* p, cudaStream_t st, float* best_ms_out) {
  constexpr int kReps = 3;
  const int kbs[] = {0, 1, 2, 4, 8};
  float best_ms = 0.f;
  p->form = OEB_BATCH_FORM_PER_LAUNCH;
  OEB_TRY(time_runs(p, st, kReps, &best_ms));
  int best_form = OEB_BATCH_FORM_PER_LAUNCH, best_kb = p->one_kb, best_per_sm = p->one_per_sm;
  for (int kb : kbs) {
    const oeb_status b = kb == p->one_kb ? OEB_OK : build_one(p, kb);
    if (b == OEB_ERR_UNSUPPORTED) break;
    OEB_TRY(b);
    p->form = OEB_BATCH_FORM_ONE_LAUNCH;
    for (int per_sm = 2; per_sm <= 4; ++per_sm) {
      use_variant(p, per_sm);
      float ms = 0.f;
      OEB_TRY(time_runs(p, st, kReps, &ms));
      if (ms < best_ms) {
        best_ms = ms;
        best_form = OEB_BATCH_FORM_ONE_LAUNCH;
        best_kb = kb;
        best_per_sm = per_sm;
      }
    }
  }
  if (best_form == OEB_BATCH_FORM_ONE_LAUNCH && best_kb != p->one_kb) OEB_TRY(build_one(p, best_kb));
  use_variant(p, best_per_sm);
  p->form = best_form;
  if (best_ms_out) *best_ms_out = best_ms;
  return OEB_OK;
}

// The status word of the last one-launch run: 0, or OEB_ERR_TIMEOUT and the task whose wait
// gave up.  Waits for the device to be idle first.
oeb_status step_status(oeb_batch_plan* p, int* status, int* task) {
  *status = 0;
  if (task) *task = -1;
  if (!p->one_buf) return OEB_OK;
  unsigned ctl[kStepCtlWords];
  OEB_CUDA_TRY(cudaDeviceSynchronize());
  OEB_CUDA_TRY(cudaMemcpy(ctl, p->one_buf + p->one_ctl_off, sizeof(ctl), cudaMemcpyDeviceToHost));
  *status = (int)ctl[1];
  if (task && ctl[1] != 0u) *task = (int)ctl[2];
  return OEB_OK;
}

// The wait statistics of the last one-launch run: the time its CTAs spent in waits that had
// to poll (us, summed over CTAs) and the number of such waits.
oeb_status step_waits(oeb_batch_plan* p, uint64_t* wait_us, uint64_t* waits) {
  *wait_us = 0;
  *waits = 0;
  if (!p->one_buf) return OEB_OK;
  unsigned ctl[kStepCtlWords];
  OEB_CUDA_TRY(cudaDeviceSynchronize());
  OEB_CUDA_TRY(cudaMemcpy(ctl, p->one_buf + p->one_ctl_off, sizeof(ctl), cudaMemcpyDeviceToHost));
  *wait_us = ctl[3];
  *waits = ctl[4];
  return OEB_OK;
}

// Makes the first task of the one-launch form wait for a count that nothing writes (on), or
// restores it (off): a run then ends with OEB_ERR_TIMEOUT after the wait limit.
oeb_status withhold(oeb_batch_plan* p, int on) {
  if (!p->one_buf) return OEB_ERR_ARGUMENT;
  StepTask t = p->one_first;
  if (on) {
    t.dep = p->one_tasks;  // done[ntasks]: never written
    t.need = 1u;
  }
  OEB_CUDA_TRY(cudaDeviceSynchronize());
  OEB_CUDA_TRY(cudaMemcpy(p->one_buf, &t, sizeof(t), cudaMemcpyHostToDevice));
  p->withheld = on != 0;
  return OEB_OK;
}

oeb_status run_per_launch(oeb_batch_plan* p, cudaStream_t st) {
  OEB_CUDA_TRY(cudaEventRecord(p->fork, st));
  OEB_CUDA_TRY(cudaStreamWaitEvent(p->side, p->fork, 0));
  for (const Slot& sl : p->slots) OEB_TRY(run_slot(p, sl, sl.ctas, sl.per_member, st));
  OEB_CUDA_TRY(cudaEventRecord(p->join, p->side));
  OEB_CUDA_TRY(cudaStreamWaitEvent(st, p->join, 0));
  return OEB_OK;
}

void destroy(oeb_batch_plan* p) {
  if (!p) return;
  cudaSetDevice(p->device);
  cudaDeviceSynchronize();
  for (Member& m : p->members)
    if (m.chain) oeb_chain_plan_destroy(m.chain);
  if (p->arena) cudaFree(p->arena);
  if (p->tables) cudaFree(p->tables);
  if (p->one_buf) cudaFree(p->one_buf);
  if (p->fork) cudaEventDestroy(p->fork);
  if (p->join) cudaEventDestroy(p->join);
  if (p->side) cudaStreamDestroy(p->side);
  delete p;
}

oeb_status create(const oeb_batch_member* in, int count, int modes, oeb_batch_plan** out) {
  if (!in || !out) return OEB_ERR_NULL;
  *out = nullptr;
  if (count < 1) return OEB_ERR_ARGUMENT;
  modes &= OEB_CHAIN_FORWARD | OEB_CHAIN_ADJOINT;
  if (!modes) return OEB_ERR_ARGUMENT;
  oeb_batch_plan* p = new (std::nothrow) oeb_batch_plan();
  if (!p) return OEB_ERR_ALLOC;
  p->modes = modes;
  auto fail = [&](oeb_status st) {
    destroy(p);
    return st;
  };
  if (cudaGetDevice(&p->device) != cudaSuccess ||
      cudaDeviceGetAttribute(&p->sms, cudaDevAttrMultiProcessorCount, p->device) != cudaSuccess)
    return fail(cuda_fail(cudaGetLastError()));
  if (cudaStreamCreateWithFlags(&p->side, cudaStreamNonBlocking) != cudaSuccess ||
      cudaEventCreateWithFlags(&p->fork, cudaEventDisableTiming) != cudaSuccess ||
      cudaEventCreateWithFlags(&p->join, cudaEventDisableTiming) != cudaSuccess)
    return fail(cuda_fail(cudaGetLastError()));
  p->members.resize(count);
  for (int i = 0; i < count; ++i) {
    const oeb_batch_member& src = in[i];
    Member& m = p->members[i];
    if (src.elem_size != 8 && src.elem_size != 4) return fail(OEB_ERR_ARGUMENT);
    if (!src.fields) return fail(OEB_ERR_NULL);
    m.elem = src.elem_size;
    m.dom = src.dom;
    m.s = src.scalars;
    oeb_status st;
    if (m.elem == 8) {
      copy_fields(static_cast<const oeb_chain_fields_f64*>(src.fields), m.d3, m.d1, &m.fields64);
      st = copy_io(src, modes, m.io64);
      if (st == OEB_OK) {
        if (!m.fields64.u) return fail(OEB_ERR_NULL);
        st = oeb_chain_plan_create_f64(m.fields64.u, &m.dom, modes, &m.chain);
      }
    } else {
      copy_fields(static_cast<const oeb_chain_fields_f32*>(src.fields), m.f3, m.f1, &m.fields32);
      st = copy_io(src, modes, m.io32);
      if (st == OEB_OK) {
        if (!m.fields32.u) return fail(OEB_ERR_NULL);
        st = oeb_chain_plan_create_f32(m.fields32.u, &m.dom, modes, &m.chain);
      }
    }
    if (st != OEB_OK) return fail(st);
  }
  // 1. sizing: each member's scratch peak over its recorded calls
  size_t arena = 0;
  for (Member& m : p->members) {
    size_t need = 0;
    for (int mode : kModes) {
      if (!(modes & mode)) continue;
      Recorder rec;
      const oeb_status st = record(m, mode, &rec);
      if (st != OEB_OK) return fail(st);
      need = std::max(need, rec.peak);
    }
    m.arena_off = arena;
    m.arena_size = need;
    arena += (need + 255) & ~size_t(255);
  }
  p->arena_bytes = arena;
  if (arena) {
    const cudaError_t e = cudaMalloc(&p->arena, arena);
    if (e != cudaSuccess) {
      cuda_fail(e);
      return fail(OEB_ERR_ALLOC);
    }
  }
  // 2. recording and 3. tables, default k-blocking
  std::vector<std::vector<std::vector<LaunchRecord>>> seq;
  oeb_status st = record_all(p, 0, 0, &seq);
  std::vector<char> host;
  if (st == OEB_OK) st = build_slots(p, seq, 0, 0, &p->slots, &host, 0);
  if (st == OEB_OK) st = upload(p, host);
  if (st != OEB_OK) return fail(st);
  p->base_slots = p->slots.size();
  *out = p;
  return OEB_OK;
}

oeb_status autotune_slots(oeb_batch_plan* p, cudaStream_t st) {
  const int kbs[] = {1, 2, 4, 8};
  constexpr int kReps = 3;
  // every candidate's slots -- each k-blocking with each tile shape -- in one table buffer
  std::vector<std::vector<Slot>> cand;
  std::vector<char> host;
  for (int shape = 0; shape < kShapes; ++shape) {
    for (int kb : kbs) {
      std::vector<std::vector<std::vector<LaunchRecord>>> seq;
      OEB_TRY(record_all(p, kb, shape, &seq));
      std::vector<Slot> slots;
      OEB_TRY(build_slots(p, seq, kb, shape, &slots, &host, 0));
      if (slots.size() != p->slots.size()) return OEB_ERR_UNSUPPORTED;
      cand.push_back(std::move(slots));
    }
  }
  OEB_TRY(upload(p, host));
  // the default choice of every slot: kb = 4, the default shape, one persistent wave
  std::vector<Slot> best = cand[2];
  // buffers hold the data of a complete run before single launches are timed
  for (size_t i = 0; i < best.size(); ++i) best[i].ctas = std::min(best[i].total, best[i].occupancy * p->sms);
  p->slots = best;
  OEB_TRY(run_per_launch(p, st));
  OEB_CUDA_TRY(cudaStreamSynchronize(st));
  OEB_CUDA_TRY(cudaStreamSynchronize(p->side));
  cudaEvent_t e0, e1;
  OEB_CUDA_TRY(cudaEventCreate(&e0));
  OEB_CUDA_TRY(cudaEventCreate(&e1));
  oeb_status result = OEB_OK;
  for (size_t i = 0; i < best.size() && result == OEB_OK; ++i) {
    float best_ms = -1.f;
    for (auto& c : cand) {
      const Slot& sl = c[i];
      // a shape other than the default changes nothing for a kernel that takes none
      if (sl.shape != 0 && sl.shape_tag == 0) continue;
      const cudaStream_t s = sl.side ? p->side : st;
      // persistent wave, one CTA per tile (batched launches), then per-member launches
      const int wave = std::min(sl.total, sl.occupancy * p->sms);
      const int options[3] = {wave, sl.total, 0};
      for (int o = 0; o < 3 && result == OEB_OK; ++o) {
        if (o == 1 && options[1] == options[0]) continue;
        const bool per_member = o == 2;
        result = run_slot(p, sl, options[o], per_member, st);  // warm-up
        if (result != OEB_OK) break;
        cudaEventRecord(e0, s);
        for (int r = 0; r < kReps && result == OEB_OK; ++r) result = run_slot(p, sl, options[o], per_member, st);
        cudaEventRecord(e1, s);
        if (cudaEventSynchronize(e1) != cudaSuccess) result = cuda_fail(cudaGetLastError());
        float ms = 0.f;
        cudaEventElapsedTime(&ms, e0, e1);
        if (result == OEB_OK && (best_ms < 0.f || ms < best_ms)) {
          best_ms = ms;
          best[i] = sl;
          best[i].ctas = per_member ? wave : options[o];
          best[i].per_member = per_member;
        }
      }
      if (result != OEB_OK) break;
    }
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  OEB_TRY(result);
  p->slots = best;
  return OEB_OK;
}

// ---- tuning records ------------------------------------------------------------------
// A record keeps the autotuner's choices so that a later process can reuse them without
// timing anything: three ints a slot, in run order -- the slot's kb, its tile shape, and its
// launch form (kFormWave: one persistent wave; kFormPerTile: one CTA per tile;
// kFormPerMember: one ordinary launch per member).  The wave's CTA count is taken from the
// device the record is applied on.  kb is one of the values a plan records with: 0 (every
// kernel's own default, as at creation) or 1, 2, 4, 8 (the autotuner's candidates); the shape
// is 0 .. kShapes-1 (tuned_shape).
constexpr int kFormWave = 0, kFormPerTile = 1, kFormPerMember = 2;

int wave_ctas(const oeb_batch_plan* p, const Slot& sl) { return std::min(sl.total, sl.occupancy * p->sms); }

bool recorded_kb(int kb) { return kb == 0 || kb == 1 || kb == 2 || kb == 4 || kb == 8; }

// FNV-1a over what fixes the plan's launch sequence: modes, then every member's element
// size and domain in order, then the slot count.
uint64_t signature(const oeb_batch_plan* p) {
  uint64_t h = 1469598103934665603ull;
  auto mix = [&](int64_t v) {
    for (int b = 0; b < 8; ++b) {
      h ^= (uint64_t)((v >> (8 * b)) & 0xff);
      h *= 1099511628211ull;
    }
  };
  mix(p->modes);
  mix((int64_t)p->members.size());
  for (const Member& m : p->members) {
    mix(m.elem);
    mix(m.dom.nx);
    mix(m.dom.ny);
    mix(m.dom.nz);
  }
  mix((int64_t)p->base_slots);
  return h;
}

oeb_status tuning_get(const oeb_batch_plan* p, int* rec, int capacity, int* count) {
  if (!count) return OEB_ERR_NULL;
  *count = (int)p->slots.size();
  if (!rec) return OEB_OK;
  if (capacity < *count) return OEB_ERR_TOO_LARGE;
  for (size_t i = 0; i < p->slots.size(); ++i) {
    const Slot& sl = p->slots[i];
    rec[3 * i] = sl.kb;
    rec[3 * i + 1] = sl.shape;
    rec[3 * i + 2] = sl.per_member ? kFormPerMember : (sl.ctas == wave_ctas(p, sl) ? kFormWave : kFormPerTile);
  }
  return OEB_OK;
}

// Records the step with every kb the record names, builds their slots into one new table
// buffer, and only then replaces the plan's tables and slots: on any error the plan is left
// as it was.
oeb_status tuning_apply(oeb_batch_plan* p, const int* rec, int count) {
  if (!rec) return OEB_ERR_NULL;
  if (count != (int)p->slots.size()) return OEB_ERR_ARGUMENT;
  std::vector<std::pair<int, int>> recs;  // the (kb, shape) pairs the record names
  for (int i = 0; i < count; ++i) {
    const int kb = rec[3 * i], shape = rec[3 * i + 1], form = rec[3 * i + 2];
    if (!recorded_kb(kb) || shape < 0 || shape >= kShapes || form < kFormWave || form > kFormPerMember)
      return OEB_ERR_ARGUMENT;
    if (std::find(recs.begin(), recs.end(), std::make_pair(kb, shape)) == recs.end()) recs.push_back({kb, shape});
  }
  std::vector<std::vector<Slot>> cand;
  std::vector<char> host;
  for (const auto& ks : recs) {
    std::vector<std::vector<std::vector<LaunchRecord>>> seq;
    OEB_TRY(record_all(p, ks.first, ks.second, &seq));
    std::vector<Slot> slots;
    OEB_TRY(build_slots(p, seq, ks.first, ks.second, &slots, &host, 0));
    if (slots.size() != p->slots.size()) return OEB_ERR_UNSUPPORTED;
    cand.push_back(std::move(slots));
  }
  std::vector<Slot> next(count);
  for (int i = 0; i < count; ++i) {
    const size_t c = (size_t)(std::find(recs.begin(), recs.end(), std::make_pair(rec[3 * i], rec[3 * i + 1])) -
                              recs.begin());
    Slot sl = cand[c][i];
    const int form = rec[3 * i + 2];
    sl.per_member = form == kFormPerMember;
    sl.ctas = form == kFormPerTile ? sl.total : wave_ctas(p, sl);
    next[i] = std::move(sl);
  }
  OEB_TRY(upload(p, host));
  p->slots = std::move(next);
  return OEB_OK;
}

// Records the step with fusion grouping `mask` and replaces the plan's launches by its
// default choices (kb 0, the default shape, one persistent wave), as at creation.  The
// one-launch tables, if built, are rebuilt for the new grouping; if that fails they are
// dropped (and a one-launch plan falls back to the per-launch form).  On any earlier error
// the plan is unchanged.
oeb_status set_fusion(oeb_batch_plan* p, int mask) {
  if (mask & ~OEB_FUSE_ALL) return OEB_ERR_ARGUMENT;
  const int prev = p->fusion;
  p->fusion = mask;
  std::vector<std::vector<std::vector<LaunchRecord>>> seq;
  std::vector<Slot> slots;
  std::vector<char> host;
  oeb_status st = record_all(p, 0, 0, &seq);
  if (st == OEB_OK) st = build_slots(p, seq, 0, 0, &slots, &host, 0);
  if (st == OEB_OK) st = upload(p, host);
  if (st != OEB_OK) {
    p->fusion = prev;
    return st;
  }
  p->slots = std::move(slots);
  if (p->one_buf) {
    st = build_one(p, p->one_kb);
    if (st != OEB_OK) {
      cudaDeviceSynchronize();
      cudaFree(p->one_buf);
      p->one_buf = nullptr;
      p->one_bytes = 0;
      p->one_kb = -1;
      p->form = OEB_BATCH_FORM_PER_LAUNCH;
      return st;
    }
  }
  return OEB_OK;
}

// The autotuner: for each fusion grouping, the per-launch choices (autotune_slots) and the
// time of a whole run with them; keeps the grouping whose run is faster, with its choices.
// Times the per-launch form whatever the plan's form; leaves the form as it was.
oeb_status autotune(oeb_batch_plan* p, cudaStream_t st) {
  const int form = p->form;
  p->form = OEB_BATCH_FORM_PER_LAUNCH;
  const int masks[] = {0, OEB_FUSE_HADV_UPDATE};
  float best_ms = -1.f;
  int best_mask = p->fusion;
  std::vector<int> best_rec;
  oeb_status r = OEB_OK;
  for (int mask : masks) {
    r = set_fusion(p, mask);
    if (r == OEB_OK) r = autotune_slots(p, st);
    float ms = 0.f;
    if (r == OEB_OK) r = time_runs(p, st, 3, &ms);
    if (r != OEB_OK) break;
    if (best_ms < 0.f || ms < best_ms) {
      best_ms = ms;
      best_mask = mask;
      int n = 0;
      tuning_get(p, nullptr, 0, &n);
      best_rec.assign(3 * (size_t)n, 0);
      r = tuning_get(p, best_rec.data(), n, &n);
      if (r != OEB_OK) break;
    }
  }
  if (r == OEB_OK && best_mask != p->fusion) {
    r = set_fusion(p, best_mask);
    if (r == OEB_OK) r = tuning_apply(p, best_rec.data(), (int)(best_rec.size() / 3));
  }
  if (p->one_buf) p->form = form;
  return r;
}

// Makes the plan's device current for the lifetime of the guard and restores the caller's
// device afterwards: the entry points that allocate, copy or launch run on the device the plan
// was created on, whichever device the calling thread has current.
class PlanDevice {
 public:
  explicit PlanDevice(const oeb_batch_plan* p) {
    ok_ = cudaGetDevice(&prev_) == cudaSuccess && (prev_ == p->device || cudaSetDevice(p->device) == cudaSuccess);
    switched_ = ok_ && prev_ != p->device;
  }
  ~PlanDevice() {
    if (switched_) cudaSetDevice(prev_);
  }
  bool ok() const { return ok_; }

 private:
  int prev_ = 0;
  bool ok_ = false, switched_ = false;
};

}  // namespace
}  // namespace oeb

using namespace oeb;

extern "C" oeb_status oeb_batch_plan_create(const oeb_batch_member* members, int count, int modes,
                                            oeb_batch_plan** out) {
  return create(members, count, modes, out);
}

extern "C" oeb_status oeb_batch_run(oeb_batch_plan* p, void* stream) {
  if (!p) return OEB_ERR_NULL;
  PlanDevice on(p);
  if (!on.ok()) return cuda_fail(cudaGetLastError());
  return run(p, (cudaStream_t)stream);
}

extern "C" oeb_status oeb_batch_autotune(oeb_batch_plan* p, void* stream) {
  if (!p) return OEB_ERR_NULL;
  PlanDevice on(p);
  if (!on.ok()) return cuda_fail(cudaGetLastError());
  return autotune(p, (cudaStream_t)stream);
}

extern "C" oeb_status oeb_batch_signature(const oeb_batch_plan* p, uint64_t* out) {
  if (!p || !out) return OEB_ERR_NULL;
  *out = signature(p);
  return OEB_OK;
}

extern "C" oeb_status oeb_batch_tuning_get(const oeb_batch_plan* p, int* record, int capacity, int* count) {
  if (!p) return OEB_ERR_NULL;
  return tuning_get(p, record, capacity, count);
}

extern "C" oeb_status oeb_batch_tuning_apply(oeb_batch_plan* p, const int* record, int count) {
  if (!p) return OEB_ERR_NULL;
  PlanDevice on(p);
  if (!on.ok()) return cuda_fail(cudaGetLastError());
  return tuning_apply(p, record, count);
}

extern "C" int oeb_batch_launches(const oeb_batch_plan* p) {
  if (p && p->form == OEB_BATCH_FORM_ONE_LAUNCH) return 1;
  int n = 0;
  if (p)
    for (const Slot& sl : p->slots) n += sl.per_member ? (int)sl.grids.size() : 1;
  return n;
}

extern "C" int64_t oeb_batch_points(const oeb_batch_plan* p) {
  int64_t n = 0;
  if (p)
    for (const Member& m : p->members) n += m.dom.nx * m.dom.ny * m.dom.nz;
  return n;
}

extern "C" size_t oeb_batch_plan_bytes(const oeb_batch_plan* p) {
  if (!p) return 0;
  size_t n = p->arena_bytes + p->table_bytes + p->one_bytes;
  for (const Member& m : p->members) n += oeb_chain_plan_bytes(m.chain);
  return n;
}

extern "C" oeb_status oeb_batch_plan_destroy(oeb_batch_plan* p) {
  if (!p) return OEB_ERR_NULL;
  destroy(p);
  return OEB_OK;
}

extern "C" oeb_status oeb_batch_set_form(oeb_batch_plan* p, int form, int kb, int ctas_per_sm) {
  if (!p) return OEB_ERR_NULL;
  PlanDevice on(p);
  if (!on.ok()) return cuda_fail(cudaGetLastError());
  return set_form(p, form, kb, ctas_per_sm);
}

extern "C" oeb_status oeb_batch_get_form(const oeb_batch_plan* p, int* form, int* kb, int* ctas_per_sm) {
  if (!p || !form || !kb || !ctas_per_sm) return OEB_ERR_NULL;
  const bool one = p->form == OEB_BATCH_FORM_ONE_LAUNCH;
  *form = p->form;
  *kb = one ? p->one_kb : -1;
  *ctas_per_sm = one ? p->one_per_sm : -1;
  return OEB_OK;
}

extern "C" oeb_status oeb_batch_step_waits(oeb_batch_plan* p, uint64_t* wait_us, uint64_t* waits) {
  if (!p || !wait_us || !waits) return OEB_ERR_NULL;
  PlanDevice on(p);
  if (!on.ok()) return cuda_fail(cudaGetLastError());
  return step_waits(p, wait_us, waits);
}

extern "C" oeb_status oeb_batch_autotune_form(oeb_batch_plan* p, void* stream, float* ms) {
  if (!p) return OEB_ERR_NULL;
  PlanDevice on(p);
  if (!on.ok()) return cuda_fail(cudaGetLastError());
  return autotune_form(p, (cudaStream_t)stream, ms);
}

extern "C" oeb_status oeb_batch_step_status(oeb_batch_plan* p, int* status, int* task) {
  if (!p || !status) return OEB_ERR_NULL;
  PlanDevice on(p);
  if (!on.ok()) return cuda_fail(cudaGetLastError());
  return step_status(p, status, task);
}

extern "C" oeb_status oeb_batch_set_wait_limit(oeb_batch_plan* p, uint64_t ns) {
  if (!p) return OEB_ERR_NULL;
  if (ns == 0) return OEB_ERR_ARGUMENT;
  p->wait_ns = ns;
  return OEB_OK;
}

extern "C" oeb_status oeb_batch_withhold(oeb_batch_plan* p, int on) {
  if (!p) return OEB_ERR_NULL;
  PlanDevice dev(p);
  if (!dev.ok()) return cuda_fail(cudaGetLastError());
  return withhold(p, on);
}

extern "C" oeb_status oeb_batch_set_fusion(oeb_batch_plan* p, int mask) {
  if (!p) return OEB_ERR_NULL;
  PlanDevice on(p);
  if (!on.ok()) return cuda_fail(cudaGetLastError());
  return set_fusion(p, mask);
}

extern "C" oeb_status oeb_batch_get_fusion(const oeb_batch_plan* p, int* mask) {
  if (!p || !mask) return OEB_ERR_NULL;
  *mask = p->fusion;
  return OEB_OK;
}

extern "C" oeb_status oeb_batch_step_order(int members, const int* counts, const int64_t* points, int* member,
                                           int* position, int* dep) {
  if (!counts || !points || !member || !position || !dep) return OEB_ERR_NULL;
  if (members < 1) return OEB_ERR_ARGUMENT;
  std::vector<int> c(counts, counts + members);
  for (int v : c)
    if (v < 0) return OEB_ERR_ARGUMENT;
  const auto order = oeb::step_order(c, std::vector<int64_t>(points, points + members));
  std::vector<int> last(members, -1);
  for (size_t t = 0; t < order.size(); ++t) {
    member[t] = order[t].first;
    position[t] = order[t].second;
    dep[t] = last[order[t].first];
    last[order[t].first] = (int)t;
  }
  return OEB_OK;
}
