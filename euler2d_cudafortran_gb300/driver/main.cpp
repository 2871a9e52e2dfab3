// main.cpp -- the HydroRun driver of serial_ref/main.f90 on the GB300 library.
//
//   euler2d_gb300 test.nml [--percall] [--binary-vtk] [--no-io] [--sync-io] [--outdir DIR]
//
// Same sequence as serial_ref/main.f90:36-95: read the namelist, print the
// parameters, init_implode, initial compute_dt, make_boundaries, then the
// step loop with output every nOutput steps, the final output of u, the
// timer summary and the Perf line in Mcell-updates/s.  `t` is never advanced
// by the reference, so the loop runs nStepmax steps whatever tEnd is.
//
// Between two outputs the steps run on the device without host round trips
// (e2d_advance); --percall calls compute_dt + godunov_unsplit every step as
// the reference does.  Both give the same states and dt sequence.
//
// Output is asynchronous unless --sync-io: the state is snapshotted on the
// device in stream order, copied to pinned host memory on a copy stream and
// written to its VTK file by a writer thread, while the next steps run; the
// "io time" is then the time the step loop waits for output.
#include <chrono>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <thread>
#include <vector>

#include "euler2d_gb300.h"
#include "namelist.h"
#include "vtk.h"

namespace {

using clk = std::chrono::steady_clock;

struct Timer {
  double elapsed = 0;
  clk::time_point t0;
  void start() { t0 = clk::now(); }
  void stop() { elapsed += std::chrono::duration<double>(clk::now() - t0).count(); }
};

int die(const char* what, int rc) {
  std::fprintf(stderr, "euler2d_gb300: %s failed (%d): %s\n", what, rc, e2d_last_error());
  return 1;
}

}  // namespace

int main(int argc, char** argv) {
  std::string nml, outdir = ".";
  bool percall = false, binary = false, no_io = false, parse_only = false, sync_io = false;
  for (int k = 1; k < argc; ++k) {
    if (!std::strcmp(argv[k], "--percall")) percall = true;
    else if (!std::strcmp(argv[k], "--binary-vtk")) binary = true;
    else if (!std::strcmp(argv[k], "--no-io")) no_io = true;
    else if (!std::strcmp(argv[k], "--sync-io")) sync_io = true;
    else if (!std::strcmp(argv[k], "--parse-only")) parse_only = true;
    else if (!std::strcmp(argv[k], "--outdir") && k + 1 < argc) outdir = argv[++k];
    else nml = argv[k];
  }
  if (nml.empty()) {
    std::printf(" You should provide an input parameter file (with a namelist)\n Usage:\n    ./euler2d_gb300 param.nml\n");
    return 0;
  }
  RunConfig cfg;
  std::string err = read_namelist(nml, &cfg);
  if (!err.empty()) {
    std::fprintf(stderr, "%s\n", err.c_str());
    return 1;
  }
  const e2d_params& p = cfg.p;
  if (parse_only) {  // the parameters as read, for tests of the namelist reader
    std::printf("{\"tEnd\": %.17g, \"nStepmax\": %d, \"nOutput\": %d, \"nx\": %d, \"ny\": %d, "
                "\"gamma0\": %.17g, \"cfl\": %.17g, \"smallr\": %.17g, \"smallc\": %.17g, "
                "\"niter_riemann\": %d, \"iorder\": %d, \"slope_type\": %d, \"boundary_type_xmin\": %d, "
                "\"boundary_type_xmax\": %d, \"boundary_type_ymin\": %d, \"boundary_type_ymax\": %d, "
                "\"implementationVersion\": %d, \"riemann_solver\": %d, \"precision\": %d}\n",
                cfg.tEnd, cfg.nStepmax, cfg.nOutput, p.nx, p.ny, p.gamma0, p.cfl, p.smallr, p.smallc,
                p.niter_riemann, p.iorder, p.slope_type, p.boundary_type_xmin, p.boundary_type_xmax,
                p.boundary_type_ymin, p.boundary_type_ymax, p.implementation_version, p.riemann_solver, p.precision);
    return 0;
  }
  const int isize = p.nx + 4, jsize = p.ny + 4;
  std::printf(" Simulation run parameters:\n nx : %d\n ny : %d\n dx : %.17g\n dy : %.17g\n", p.nx, p.ny, 1.0 / p.nx,
              1.0 / p.ny);
  std::printf(" imin : 1 imax : %d\n jmin : 1 jmax : %d\n", isize, jsize);
  std::printf(" nStepmax,tEnd,nOutput : %d %g %d\n", cfg.nStepmax, cfg.tEnd, cfg.nOutput);
  std::printf(" gamma0,cfl : %g %g\n smallr,smallc,niter_riemann : %g %g %d\n iorder,slope_type : %d %d\n",
              p.gamma0, p.cfl, p.smallr, p.smallc, p.niter_riemann, p.iorder, p.slope_type);
  int arith = E2D_ARITH_EXACT;
  e2d_arithmetic(&arith);
  std::printf(" Using implementation version %d, %s Riemann solver, %s, %s arithmetic\n", p.implementation_version,
              p.riemann_solver == E2D_RIEMANN_HLLC ? "HLLC" : "approximate", p.precision == 8 ? "FP64" : "FP32",
              arith == E2D_ARITH_FMA ? "fused multiply-add" : "exact");

  e2d_run* run = nullptr;
  int rc = e2d_create(&p, &run);
  if (rc) return die("e2d_create", rc);
  rc = e2d_init_implode(run);
  if (rc) return die("init_implode", rc);
  size_t state_bytes = 0;
  e2d_get_sizes(run, nullptr, nullptr, &state_bytes);
  std::vector<unsigned char> host(sync_io ? state_bytes : 0);
  void* pinned = nullptr;
  if (!sync_io && (rc = e2d_host_alloc(state_bytes, &pinned))) return die("host_alloc", rc);

  double dtd = 0;
  float dtf = 0;
  void* dtp = p.precision == 8 ? (void*)&dtd : (void*)&dtf;
  auto dt_value = [&]() { return p.precision == 8 ? dtd : (double)dtf; };
  rc = e2d_compute_dt(run, 0, dtp);
  if (rc) return die("compute_dt", rc);
  std::printf(" Initial value for dt %.17g\n", dt_value());
  rc = e2d_make_boundaries(run, 0);
  if (rc) return die("make_boundaries", rc);

  std::printf(" Start computation....\n");
  Timer total, io;
  total.start();
  int nStep = 0;
  const double t = 0.0;  // never advanced (serial_ref/main.f90:53)
  std::thread writer;
  int writer_rc = 0;
  auto output = [&](int which, int step) -> int {
    io.start();
    int r = 0;
    if (sync_io) {
      r = e2d_download_state(run, which, host.data());
      if (!r && !no_io && save_vtk(outdir, step, host.data(), p.nx, p.ny, p.precision, !binary).empty())
        std::fprintf(stderr, "cannot write VTK output in %s\n", outdir.c_str());
    } else {
      if (writer.joinable()) writer.join();  // the previous file is written, the buffer free
      r = writer_rc ? writer_rc : e2d_begin_download(run, which, pinned);
      if (!r)
        writer = std::thread([&, step]() {
          writer_rc = e2d_wait_download(run);
          if (!writer_rc && !no_io && save_vtk(outdir, step, pinned, p.nx, p.ny, p.precision, !binary).empty())
            std::fprintf(stderr, "cannot write VTK output in %s\n", outdir.c_str());
        });
    }
    io.stop();
    return r;
  };
  std::vector<double> dtlog8;
  std::vector<float> dtlog4;
  while (t < cfg.tEnd && nStep < cfg.nStepmax) {
    if (nStep % cfg.nOutput == 0) {
      std::printf(" Output results at step %d dt %.17g\n", nStep, dt_value());
      if ((rc = output(nStep % 2, nStep))) return die("download_state", rc);
    }
    if (percall) {
      if ((rc = e2d_compute_dt(run, nStep % 2, dtp))) return die("compute_dt", rc);
      if ((rc = e2d_godunov_unsplit(run, nStep, dt_value()))) return die("godunov_unsplit", rc);
      ++nStep;
    } else {
      int chunk = cfg.nOutput - nStep % cfg.nOutput;
      if (nStep + chunk > cfg.nStepmax) chunk = cfg.nStepmax - nStep;
      void* log = nullptr;
      if (p.precision == 8) { dtlog8.resize(chunk); log = dtlog8.data(); }
      else { dtlog4.resize(chunk); log = dtlog4.data(); }
      if ((rc = e2d_advance(run, nStep, chunk, log))) return die("advance", rc);
      if (p.precision == 8) dtd = dtlog8[chunk - 1];
      else dtf = dtlog4[chunk - 1];
      nStep += chunk;
    }
  }
  std::printf(" Output results at step %d dt %.17g\n", nStep, dt_value());
  // serial_ref/main.f90:81 always writes u (stale after an odd number of steps)
  if ((rc = output(0, nStep))) return die("download_state", rc);
  if (writer.joinable()) {
    io.start();
    writer.join();
    io.stop();
  }
  if (writer_rc) return die("wait_download", writer_rc);
  e2d_synchronize(run);
  total.stop();
  e2d_host_free(pinned);
  unsigned health = 0;
  e2d_get_health(run, &health);
  e2d_destroy(run);
  if (health) std::printf(" health flags : %u\n", health);
  std::printf(" total      time : %.6f secondes\n", total.elapsed);
  std::printf(" io         time : %.6f secondes %.3f %%\n", io.elapsed, 100 * io.elapsed / total.elapsed);
  const double compute = total.elapsed - io.elapsed;
  std::printf(" Perf             : %.3f  number of Mcell-updates/s\n",
              1.0 * nStep * isize * jsize / compute * 1e-6);
  std::printf(" Perf (interior)  : %.3f  number of Mcell-updates/s\n", 1.0 * nStep * p.nx * p.ny / compute * 1e-6);
  return 0;
}
