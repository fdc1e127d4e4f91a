/* Benchmark driver: builds one synthetic workload through the meep:: C++ API
 * (meep_gb300/workloads/cases.hpp) and times the stepping path.
 *
 *   bench_main [--align-dft] <workload> <warmup> <steps> [e2e_steps] [total_steps] [dft_file]
 *
 * --align-dft lengthens the warm-up so that the timed steps end on a DFT
 * sample step (a multiple of the first monitor's decimation; of 64 samples,
 * one tensor-core block, when a single-precision monitor samples every step),
 * so the timed window holds the DFT work it is credited with.
 *
 * Prints one JSON object:
 *   device_ms  time of `steps` consecutive steps on the engine's stream
 *              (CUDA events around one batched call; fields already resident)
 *   e2e_ms     wall time of `e2e_steps` iterations of the public API call
 *              sequence fields::step() + dft_flux::flux() (the flux spectrum is
 *              copied to host every step)
 *   flux       the flux spectrum after total_steps steps (the run continues,
 *              untimed, after the timed parts), for precision comparisons
 *   dft_file   (optional) the DFT-fields sums of a dft_fields workload after
 *              total_steps steps, written as complex doubles, point-major
 *              (frequency fastest), chunk after chunk (get_dft_data order)
 * Built against the CUDA engine (meep_gb300/lib) or, for the CPU baseline,
 * against the CPU oracle (oracle/_build); the code is the same.
 */
#include <meep.hpp>

#include <chrono>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "cases.hpp"

using namespace workloads;

int main(int argc, char **argv) {
  bool align = false;
  if (argc > 1 && std::string(argv[1]) == "--align-dft") {
    align = true;
    argv++;
    argc--;
  }
  if (argc < 4) {
    fprintf(stderr, "usage: %s [--align-dft] workload warmup steps [e2e_steps] [total_steps] [dft_file]\n",
            argv[0]);
    return 2;
  }
  std::string name = argv[1];
  int warm = atoi(argv[2]), steps = atoi(argv[3]);
  int e2e_steps = argc > 4 ? atoi(argv[4]) : steps;
  int total_steps = argc > 5 ? atoi(argv[5]) : 0;
  const char *dft_file = argc > 6 ? argv[6] : nullptr;
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
  const dft_chunk *first = wl->flux ? wl->flux->E : (wl->dftf ? wl->dftf->chunks : nullptr);
  const int decimation = first ? first->get_decimation_factor() : 0;
  const int warm_requested = warm;
  if (align && decimation > 0 && steps > 0) {
    const int period = decimation * (sizeof(realnum) == 4 && decimation == 1 ? 64 : 1);
    warm += (period - (warm + steps) % period) % period;
  }
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
    // steps return once queued: the timed region ends when the last one has run
    f.last_step_ms();
    e2e_ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - a).count();
  }
  if (total_steps > f.t) meep::step_n(f, total_steps - f.t);
  if (dft_file && wl->dftf) {
    // the running sums in double (get_dft_data), not the realnum chunk copies
    std::vector<std::complex<double>> buf(dft_data_size(wl->dftf->chunks));
    get_dft_data(wl->dftf->chunks, buf.data(), buf.size());
    FILE *fp = fopen(dft_file, "wb");
    if (!fp || fwrite(buf.data(), sizeof(std::complex<double>), buf.size(), fp) != buf.size()) {
      fprintf(stderr, "cannot write %s\n", dft_file);
      return 1;
    }
    fclose(fp);
  }
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
  printf("{\"workload\": \"%s\", \"cells\": %.0f, \"realnum_bytes\": %d, \"warmup\": %d, \"warmup_requested\": %d, "
         "\"steps\": %d, \"e2e_steps\": %d, \"device_ms\": %.6f, \"e2e_ms\": %.6f, "
         "\"launches\": %lld, \"nfreq\": %d, \"setup_s\": %.3f, \"checksum\": %.17g, \"t\": %d, "
         "\"timed_wall\": [%.6f, %.6f], \"dft_decimation\": %d, \"flux\": %s}\n",
         name.c_str(), wl->cells(), (int)sizeof(meep::realnum), warm, warm_requested, steps, e2e_steps, device_ms,
         e2e_ms, launches, wl->nfreq, setup_s, checksum, f.t, wall0, wall1, decimation, flux.c_str());
  return 0;
}
