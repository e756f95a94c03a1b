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
// one JSON line per kernel with GPts/s, algorithmic HBM GB/s and their fraction of this GPU's
// device-to-device copy rate (measured by the driver, once); FP32 lines add the normwise
// max and rms error of the semantic outputs against the FP64 run of the same variant on the
// same fills (the FP64 stencils give the reference's results bit for bit).  --adjoint (not in
// the reference, which has no adjoints) times each call as the forward variant followed by the
// kernel's adjoint.  Exit status 1 for a usage error or an unknown kernel name.
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include <cuda_runtime.h>

#include "driver_api.h"
#include "driver_storage.h"

int64_t domain_size = 64;  // the reference drivers' defaults (src/<k>.cpp:4-7)
int64_t domain_height = 60;
int64_t halo_width = 4;

namespace {

const char* kAll[] = {"fastwavesuv", "fvtp2d", "hadvuv", "hadvuv5th", "hdiffsa", "hdiffsmag",
                      "laplace",     "nh_p_grad", "p_grad_c", "uvbke"};

// Normwise errors of `got` against `ref` over all outputs: max |e| / max |ref| and
// rms(e) / max |ref|, the worst output's.
void errors(const std::vector<std::vector<double>>& got, const std::vector<std::vector<double>>& ref, double* mx,
            double* rms) {
  *mx = *rms = 0.0;
  for (size_t o = 0; o < got.size() && o < ref.size(); ++o) {
    double scale = 0.0, emax = 0.0, esq = 0.0;
    for (double v : ref[o]) scale = std::max(scale, std::fabs(v));
    for (size_t c = 0; c < got[o].size(); ++c) {
      const double e = std::fabs(got[o][c] - ref[o][c]);
      emax = std::max(emax, e);
      esq += e * e;
    }
    if (scale > 0.0 && !got[o].empty()) {
      *mx = std::max(*mx, emax / scale);
      *rms = std::max(*rms, std::sqrt(esq / (double)got[o].size()) / scale);
    }
  }
}

bool listed(const char* const* b, const char* const* e, const std::string& name) {
  return std::find_if(b, e, [&](const char* k) { return name == k; }) != e;
}

}  // namespace

double oeb_driver_copy_gbs() {
  static double gbs = -1.0;
  if (gbs >= 0.0) return gbs;
  gbs = 0.0;
  const size_t bytes = size_t(1) << 30;  // 1 GiB each way, far above the L2
  void *a = nullptr, *b = nullptr;
  if (cudaMalloc(&a, bytes) != cudaSuccess || cudaMalloc(&b, bytes) != cudaSuccess) {
    cudaFree(a);
    cudaGetLastError();
    return gbs;
  }
  cudaMemset(a, 0, bytes);
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  float best = 0.f;
  for (int rep = 0; rep < 6; ++rep) {
    cudaEventRecord(e0, 0);
    cudaMemcpyAsync(b, a, bytes, cudaMemcpyDeviceToDevice, 0);
    cudaEventRecord(e1, 0);
    cudaEventSynchronize(e1);
    float ms = 0.f;
    cudaEventElapsedTime(&ms, e0, e1);
    if (rep > 0 && (best == 0.f || ms < best)) best = ms;  // the first copy is the warm-up
  }
  if (best > 0.f) gbs = 2.0 * (double)bytes / (best * 1e-3) / 1e9;
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaFree(a);
  cudaFree(b);
  return gbs;
}

namespace {

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
    oeb_driver::Result r{};
    const bool errs = json && f32;
    const bool ok = f32 ? oeb_driver_run_f32(name.c_str(), algo, count, adjoint, errs, &r)
                        : oeb_driver_run_f64(name.c_str(), algo, count, adjoint, false, &r);
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
      const double copy = oeb_driver_copy_gbs();
      std::string err;
      if (errs) {
        oeb_driver::Result ref{};
        oeb_driver_run_f64(name.c_str(), algo, 1, false, true, &ref);
        double mx = 0.0, rms = 0.0;
        errors(r.outputs, ref.outputs, &mx, &rms);
        char buf[160];
        std::snprintf(buf, sizeof buf, ", \"max_rel_err_vs_f64\": %.3e, \"rms_rel_err_vs_f64\": %.3e", mx, rms);
        err = buf;
      }
      std::printf(
          "{\"kernel\": \"%s\", \"variant\": \"%s\", \"mode\": \"%s\", \"precision\": \"%s\", "
          "\"domain\": [%lld, %lld, %lld], \"halo\": %lld, \"count\": %d, \"ms_per_call\": %.6f, \"gpts\": %.4f, "
          "\"hbm_gbs\": %.1f, \"copy_gbs\": %.1f, \"hbm_frac_of_copy\": %.4f%s}\n",
          name.c_str(), r.variant[0] ? r.variant : "default", r.adjoint ? "forward+adjoint" : "forward",
          f32 ? "f32" : "f64", (long long)domain_size,
          (long long)domain_size, (long long)domain_height, (long long)halo_width, r.count, s * 1e3,
          (double)r.points / s / 1e9, bytes / s / 1e9, copy, copy > 0.0 ? bytes / s / 1e9 / copy : 0.0, err.c_str());
    }
    std::fflush(stdout);
  }
  return status;
}
