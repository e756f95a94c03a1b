// oeb_driver_f64.cpp -- the GPU driver's kernels with ElementType = double: a driver in the style of
// the reference's src/<k>.cpp (globals, then the Storage types, then the kernel headers), whose
// kernel headers are the drop-in ones (include/oeb/<k>.h) over device-resident fields.
#include <string>
#include <utility>

#include "driver_api.h"

typedef double ElementType;
#include "driver_storage.h"
typedef Storage<ElementType, 1> Storage1D;
typedef Storage<ElementType, 3> Storage3D;

// driver globals of the reference (src/uvbke.cpp:11-12, src/fvtp2d.cpp:11-12)
static const double dt5 = 0.5 * 225.0;
#define p1 ElementType(0.583333)
#define p2 ElementType(0.083333)

// calls return as soon as their kernels are queued; the driver times them with CUDA events
#define OEB_DROPIN_ASYNC
#include "fastwavesuv.h"
#include "fvtp2d.h"
#include "hadvuv.h"
#include "hadvuv5th.h"
#include "hdiffsa.h"
#include "hdiffsmag.h"
#include "laplace.h"
#include "nh_p_grad.h"
#include "p_grad_c.h"
#include "uvbke.h"

// the adjoint entry points of this precision (include/oeb_gb300.h)
#define OEB_DRIVER_ADJ(k) oeb_##k##_adj_f64
#include "driver_kernels.inc"

bool oeb_driver_run_f64(const char* kernel, int algo, int count, bool adjoint, bool keep, oeb_driver::Result* r) {
  return run_kernel(kernel, algo, count, adjoint, keep, r);
}
