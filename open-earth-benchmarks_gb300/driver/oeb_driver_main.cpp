// oeb_driver -- the reference's kernel drivers on the GPU.
//
//   oeb_driver <kernel> [ALGO [domain_size domain_height]] [--f32] [--adjoint] [--count N] [--json]
//   oeb_driver all      [ALGO [domain_size domain_height]] [...]
//
// <kernel> and the positional arguments are those of the reference's ./<kernel> (src/<k>.cpp:
// ALGO 0 default, 1 fullfusion, 2 partialfusion, 3 openmp; domain_size = nx = ny, domain_height
// = nz; halo 4; the same input fills and scalars).  "all" runs the ten kernels in the order of
// the reference's run_all.sh.  Every variant runs the library's one GPU kernel per stencil,
// through the drop-in headers on device-resident fields.  Output: the reference's lines
// (ALGO, domain_size, domain_height, then "<name>: T ms / C count, avg A ms" per kernel, or
// "Unknown ALGO" for a variant the kernel lacks, as the reference prints it) and, with --json,
// one JSON line per kernel with GPts/s and algorithmic HBM GB/s.  --adjoint (not in the
// reference, which has no adjoints) times each call as the forward variant followed by the
// kernel's adjoint, for hdiffsmag, hadvuv, hadvuv5th, fastwavesuv and fvtp2d; any other
// kernel prints "<kernel>: no adjoint" and is skipped.  Exit status 1 for a usage error or an
// unknown kernel name.
#include <algorithm>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "driver_api.h"
#include "driver_storage.h"

int64_t domain_size = 64;  // the reference drivers' defaults (src/<k>.cpp:4-7)
int64_t domain_height = 60;
int64_t halo_width = 4;

namespace {

const char* kAll[] = {"fastwavesuv", "fvtp2d", "hadvuv", "hadvuv5th", "hdiffsa", "hdiffsmag",
                      "laplace",     "nh_p_grad", "p_grad_c", "uvbke"};
// the kernels with an adjoint entry point (include/oeb_gb300.h)
const char* kAdjoint[] = {"fastwavesuv", "fvtp2d", "hadvuv", "hadvuv5th", "hdiffsmag"};

bool listed(const char* const* b, const char* const* e, const std::string& name) {
  return std::find_if(b, e, [&](const char* k) { return name == k; }) != e;
}

int usage() {
  std::fprintf(stderr,
               "Usage: oeb_driver <kernel|all> [ALGO [domain_size domain_height]] [--f32] [--adjoint] [--count N] "
               "[--json]\n");
  return 1;
}

}  // namespace

int main(int argc, char** argv) {
  std::vector<const char*> pos;
  bool f32 = false, json = false, adjoint = false;
  int count = 1000;  // the reference drivers' count (src/<k>.cpp:7)
  for (int a = 1; a < argc; ++a) {
    if (!std::strcmp(argv[a], "--f32")) {
      f32 = true;
    } else if (!std::strcmp(argv[a], "--adjoint")) {
      adjoint = true;
    } else if (!std::strcmp(argv[a], "--json")) {
      json = true;
    } else if (!std::strcmp(argv[a], "--count") && a + 1 < argc) {
      count = std::atoi(argv[++a]);
    } else if (argv[a][0] == '-' && argv[a][1] == '-') {
      return usage();
    } else {
      pos.push_back(argv[a]);
    }
  }
  if (pos.empty() || pos.size() == 3 || pos.size() > 4 || count < 1) return usage();
  const std::string kernel = pos[0];
  int algo = 0;
  if (pos.size() >= 2) algo = std::atoi(pos[1]);
  if (pos.size() == 4) {
    domain_size = std::atoll(pos[2]);
    domain_height = std::atoll(pos[3]);
  }
  if (domain_size < 1 || domain_height < 1) return usage();
  std::printf("ALGO: %d\ndomain_size: %lld\ndomain_height: %lld\n", algo, (long long)domain_size,
              (long long)domain_height);
  std::vector<std::string> names;
  if (kernel == "all")
    names.assign(std::begin(kAll), std::end(kAll));
  else
    names.push_back(kernel);
  int status = 0;
  for (const std::string& name : names) {
    if (adjoint && listed(std::begin(kAll), std::end(kAll), name) &&
        !listed(std::begin(kAdjoint), std::end(kAdjoint), name)) {
      std::printf("%s: no adjoint\n", name.c_str());
      continue;
    }
    oeb_driver::Result r{};
    const bool ok = f32 ? oeb_driver_run_f32(name.c_str(), algo, count, adjoint, &r)
                        : oeb_driver_run_f64(name.c_str(), algo, count, adjoint, &r);
    if (!ok) {
      if (!listed(std::begin(kAll), std::end(kAll), name)) {
        std::fprintf(stderr, "oeb_driver: unknown kernel %s\n", name.c_str());
        status = 1;
      } else {
        std::printf("Unknown ALGO\n");  // as the reference's drivers print it, and carry on
      }
      continue;
    }
    const std::string label =
        name + (r.variant[0] ? std::string(" ") + r.variant : std::string()) + (r.adjoint ? " + adjoint" : "");
    std::printf("%s: %f ms / %d count, avg %f ms\n", label.c_str(), r.total_ms, r.count, r.total_ms / r.count);
    if (json) {
      const double s = r.total_ms * 1e-3 / r.count;
      const double bytes = (double)r.fields * (double)r.points * (f32 ? 4.0 : 8.0);
      std::printf(
          "{\"kernel\": \"%s\", \"variant\": \"%s\", \"mode\": \"%s\", \"precision\": \"%s\", "
          "\"domain\": [%lld, %lld, %lld], \"halo\": %lld, \"count\": %d, \"ms_per_call\": %.6f, \"gpts\": %.4f, "
          "\"hbm_gbs\": %.1f}\n",
          name.c_str(), r.variant[0] ? r.variant : "default", r.adjoint ? "forward+adjoint" : "forward",
          f32 ? "f32" : "f64", (long long)domain_size,
          (long long)domain_size, (long long)domain_height, (long long)halo_width, r.count, s * 1e3,
          (double)r.points / s / 1e9, bytes / s / 1e9);
    }
    std::fflush(stdout);
  }
  return status;
}
