// driver_api.h -- what the GPU driver's main() needs from its two precision translation units.
#ifndef OEB_DRIVER_API_H
#define OEB_DRIVER_API_H

#include <cstdint>

// the globals every reference driver defines (src/<k>.cpp:4-7); set by main() from the CLI
extern int64_t domain_size;
extern int64_t domain_height;
extern int64_t halo_width;

namespace oeb_driver {
struct Result;
}

// adjoint: each timed call is the forward variant followed by oeb_<kernel>_adj_<precision>,
// seeded with the forward outputs.  keep: the semantic outputs' interiors are copied to
// r->outputs after the timed calls.
bool oeb_driver_run_f64(const char* kernel, int algo, int count, bool adjoint, bool keep, oeb_driver::Result* r);
bool oeb_driver_run_f32(const char* kernel, int algo, int count, bool adjoint, bool keep, oeb_driver::Result* r);
// The device-to-device copy rate of the current GPU in GB/s (read + write bytes), measured once.
double oeb_driver_copy_gbs();

#endif  // OEB_DRIVER_API_H
