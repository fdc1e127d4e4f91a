/* Benchmark driver: builds one synthetic workload through the meep:: C++ API
 * (meep_gb300/workloads/cases.hpp) and times the stepping path.
 *
 *   bench_main <workload> <warmup> <steps> [e2e_steps] [total_steps]
 *
 * Prints one JSON object:
 *   device_ms  time of `steps` consecutive steps on the engine's stream
 *              (CUDA events around one batched call; fields already resident)
 *   e2e_ms     wall time of `e2e_steps` iterations of the public API call
 *              sequence fields::step() + dft_flux::flux() (the flux spectrum is
 *              copied to host every step)
 *   flux       the flux spectrum after total_steps steps (the run continues,
 *              untimed, after the timed parts), for precision comparisons
 * Built against the CUDA engine (meep_gb300/lib) or, for the CPU baseline,
 * against the CPU oracle (oracle/_build); the code is the same.
 */
#include <meep.hpp>

#include <chrono>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>

#include "cases.hpp"

using namespace workloads;

int main(int argc, char **argv) {
  if (argc < 4) {
    fprintf(stderr, "usage: %s workload warmup steps [e2e_steps]\n", argv[0]);
    return 2;
  }
  std::string name = argv[1];
  int warm = atoi(argv[2]), steps = atoi(argv[3]);
  int e2e_steps = argc > 4 ? atoi(argv[4]) : steps;
  int total_steps = argc > 5 ? atoi(argv[5]) : 0;
  meep::verbosity = 0;
  auto t0 = std::chrono::steady_clock::now();
  std::unique_ptr<Workload> wl;
  if (name == "vec3d_full") wl = make_vec3d(256, 256, 256, 20.0, 0.8, 60, 42, 200, 50);
  else if (name == "vec3d_mid") wl = make_vec3d(128, 128, 128, 20.0, 0.8, 30, 42, 100, 50);
  else if (name == "vec3d_rot") wl = make_vec3d(256, 256, 256, 20.0, 0.8, 60, 42, 200, 50, true);
  else if (name == "tm2d_full") wl = make_tm2d(512, 512, 16.0, 1.0, 40, 1234, 400, 51, 0);
  else if (name == "disp3d_full") wl = make_disp3d(384, 384, 192, 20.0, 0.8, 200, 1);
  else if (name == "disp3d_mid") wl = make_disp3d(192, 192, 96, 20.0, 0.8, 200, 1);
  else {
    fprintf(stderr, "unknown workload %s\n", name.c_str());
    return 2;
  }
  fields &f = *wl->f;
  for (int i = 0; i < warm; i++)
    f.step();
  double setup_s = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
  // device-resident timing: one batched call of `steps` steps
  double device_ms = 0;
  long long l0 = f.kernel_launches();
  // wall-clock bounds of the timed region (seconds since the epoch), so that
  // clock samples taken by an outside sampler can be matched to it
  double wall0 = 0, wall1 = 0;
  auto epoch_s = [] {
    return std::chrono::duration<double>(std::chrono::system_clock::now().time_since_epoch()).count();
  };
  if (steps > 0) {
    wall0 = epoch_s();
    meep::step_n(f, steps);
    device_ms = f.last_step_ms();
    wall1 = epoch_s();
  }
  long long launches = f.kernel_launches() - l0;
  // end-to-end through the public API: step + flux spectrum to host
  double e2e_ms = 0, checksum = 0;
  if (e2e_steps > 0) {
    auto a = std::chrono::steady_clock::now();
    for (int i = 0; i < e2e_steps; i++) {
      f.step();
      if (wl->flux) {
        double *F = wl->flux->flux();
        checksum += F[0];
        delete[] F;
      }
      else {
        meep::sync_dfts(f);
        checksum += std::real(wl->dftf->chunks->dft[0]);
      }
    }
    e2e_ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - a).count();
  }
  if (total_steps > f.t) meep::step_n(f, total_steps - f.t);
  std::string flux = "[]";
  if (wl->flux) {
    double *F = wl->flux->flux();
    flux = "[";
    for (int i = 0; i < wl->nfreq; i++) {
      char buf[64];
      snprintf(buf, sizeof(buf), "%s%.17g", i ? ", " : "", F[i]);
      flux += buf;
    }
    flux += "]";
    delete[] F;
  }
  printf("{\"workload\": \"%s\", \"cells\": %.0f, \"realnum_bytes\": %d, \"warmup\": %d, "
         "\"steps\": %d, \"e2e_steps\": %d, \"device_ms\": %.6f, \"e2e_ms\": %.6f, "
         "\"launches\": %lld, \"nfreq\": %d, \"setup_s\": %.3f, \"checksum\": %.17g, \"t\": %d, "
         "\"timed_wall\": [%.6f, %.6f], \"flux\": %s}\n",
         name.c_str(), wl->cells(), (int)sizeof(meep::realnum), warm, steps, e2e_steps, device_ms,
         e2e_ms, launches, wl->nfreq, setup_s, checksum, f.t, wall0, wall1, flux.c_str());
  return 0;
}
