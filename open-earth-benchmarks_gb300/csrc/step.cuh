// step.cuh -- the one-launch step: tables a batch plan builds and the launch of the step kernel.
//
// A batch plan (batch.cu) can run the chained step of every member, forward then adjoint, as
// ONE launch of step_kernel (step.cu).  Each member's recorded launches become tasks, in the
// member's order; a task is (body, argument pack, tiles).  The plan lists every member's tasks
// in one sequence in which each task comes after its member's previous task.  The kernel's
// CTAs take the items (task, tile) of that sequence in order, from a ticket counter; an item
// waits, before it runs, until every tile of its member's previous task is done.  Because a
// CTA holding ticket t waits only on items with smaller tickets, and every smaller ticket is
// held by a CTA that is already running, the waits always end -- whatever number of CTAs is
// resident.  Each wait is bounded all the same: past the plan's limit the CTA sets the status
// word to OEB_ERR_TIMEOUT and every CTA returns at its next item.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "oeb_common.cuh"

namespace oeb {

struct StepTask {
  int first;      // the task's first item (ticket)
  int tiles;      // its items
  int gx, gy;     // tiles along x and y (along z: tiles / (gx gy))
  int op;         // the body (kStepOp)
  int dep;        // the task it waits for: its member's previous task (-1: none)
  unsigned need;  // tiles of `dep` that must be done
  int pad;
  int64_t args;   // byte offset of the body's RunPack in the table
};

// Control words of a run, zeroed before it: the ticket counter, the status (0, or
// OEB_ERR_TIMEOUT once a wait gave up), the task whose wait gave up, the time CTAs spent in
// waits that had to poll (us, summed over CTAs), the number of such waits, and spares.
constexpr int kStepCtlWords = 8;

struct StepParams {
  const StepTask* tasks;
  int ntasks;
  int total;                   // items over all tasks
  const unsigned char* table;  // argument packs
  unsigned* done;              // per task: tiles done; done[ntasks] is never written
  unsigned* ctl;               // kStepCtlWords words
  unsigned long long wait_ns;  // the longest a CTA waits for one task
};

// The step kernel is built for 2, 3 and 4 CTAs an SM (registers capped at 128, 80, 64).
// step_launch_cN launches that build with `ctas` CTAs and `smem` bytes of dynamic shared
// memory; step_occupancy_cN is its CTAs an SM with `smem` bytes.
oeb_status step_launch_c2(const StepParams& p, int ctas, size_t smem, cudaStream_t st);
oeb_status step_launch_c3(const StepParams& p, int ctas, size_t smem, cudaStream_t st);
oeb_status step_launch_c4(const StepParams& p, int ctas, size_t smem, cudaStream_t st);
int step_occupancy_c2(size_t smem);
int step_occupancy_c3(size_t smem);
int step_occupancy_c4(size_t smem);
// Whether the step kernel holds the body with this kStepOp.
bool step_has_op(int op);

inline bool step_variant(int per_sm) { return per_sm >= 2 && per_sm <= 4; }
inline oeb_status step_launch(int per_sm, const StepParams& p, int ctas, size_t smem, cudaStream_t st) {
  return per_sm == 4 ? step_launch_c4(p, ctas, smem, st)
                     : per_sm == 3 ? step_launch_c3(p, ctas, smem, st) : step_launch_c2(p, ctas, smem, st);
}
inline int step_occupancy(int per_sm, size_t smem) {
  return per_sm == 4 ? step_occupancy_c4(smem) : per_sm == 3 ? step_occupancy_c3(smem) : step_occupancy_c2(smem);
}

}  // namespace oeb
