// oeb_reach.cuh -- written boxes of the outputs that extend past the interior, shared by the
// device entry points and the host-buffer staging path (which copies back exactly these
// boxes, so host cells the reference would not write stay untouched).
#pragma once

#include "oeb_common.cuh"

namespace oeb {

// fvtp2d (kernels/fvtp2d.h): q_i on i in [-3,N+2), j in [0,N) (:46-47); q_j on i in [0,N),
// j in [-3,N+2) (:122-123); fx2 on i in [0,N+1), j in [-3,N+2) (:102-103); fy2 on
// i in [-3,N+2), j in [0,N+1) (:26-27).  Reach{ilo, ihi, jlo, jhi, klo, khi} counts cells
// beyond [0,N) on each side.
constexpr Reach kFvQi{3, 2, 0, 0, 0, 0};
constexpr Reach kFvQj{0, 0, 3, 2, 0, 0};
constexpr Reach kFvFx2{0, 1, 3, 2, 0, 0};
constexpr Reach kFvFy2{3, 2, 0, 1, 0, 0};

}  // namespace oeb
