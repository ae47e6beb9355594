// les_main.cpp -- the reference's main program (main.f95) on the GB300 solver library.
//
// A drop-in for the les_main executable for users without the Fortran build: the same
// set-up, time loop and output files, driven through the C-ABI of include/les_gpu.h.
//
//   set (set.f95:44-95)          n0, n1, nmax, dt and the data file names, from the
//                                command line (defaults: the reference's)
//   grid, init, feedbfm, ifdata  les_gpu_setup_scenario: the seeded synthetic scenario
//                                (the GIS inputs are absent); --restart reads data30 and
//                                data31 as ifdata does with ical = 1 (ifdata.f95:252-480)
//   the loop (main.f95:247-327)  time = float(n-1)*dt; the whole step on the device
//                                (run_LES_kernel, main.f95:251) or, with --per-stage, the
//                                seven subroutine calls of main.f95:260-296 with their
//                                times (the TIMINGS build's "Time for state i" lines);
//                                press's and adam's data20/data21 and centre print every
//                                1000 steps and at nmax (press.f95:197-216, adam.f95:20-27);
//                                ifdata_out (anime.f95:326); aveflow with data10/data11 at
//                                nmax (aveflow.f95:5-344)
//
// Files go to --out (default ./data, the directory of set.f95:44-50's paths); data30/31
// go to --out as well (the reference writes them to the working directory).  There is
// no CPU fallback: without a GPU the library refuses to create the domain and this
// program exits with status 1.
#include <sys/stat.h>

#include <chrono>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "les_gpu.h"

namespace {

struct Options {
  int im = 150, jm = 150, km = 90;
  int n0 = 1, n1 = 1, nmax = 10;  // set.f95:82-85
  float dt = 0.05f;               // set.f95:89
  unsigned long long seed = 1;
  float coverage = 0.30f, direction = 0.f, u_ref = 5.f;
  std::string out = "./data";
  std::string restart30, restart31;
  bool per_stage = false, aveflow = true, little_endian = false, fixed_sor = false, quiet = false;
};

void usage(FILE *f) {
  std::fprintf(f,
               "usage: les_main [--dims IMxJMxKM] [--n0 N] [--n1 N] [--nmax N] [--dt S] [--seed S]\n"
               "                [--coverage F] [--direction DEG] [--speed M/S] [--out DIR]\n"
               "                [--restart DATA30 DATA31] [--per-stage] [--no-aveflow] [--fixed-sor]\n"
               "                [--little-endian] [--quiet]\n"
               "The time loop of MPI-LES's main.f95 on the GPU (one domain, one GPU).\n");
}

bool parse(int argc, char **argv, Options *o) {
  for (int a = 1; a < argc; ++a) {
    const std::string k = argv[a];
    auto val = [&](void) -> const char * { return a + 1 < argc ? argv[++a] : nullptr; };
    const char *v = nullptr;
    if (k == "--help" || k == "-h") {
      usage(stdout);
      std::exit(0);
    } else if (k == "--dims") {
      if (!(v = val()) || std::sscanf(v, "%dx%dx%d", &o->im, &o->jm, &o->km) != 3) return false;
    } else if (k == "--n0") {
      if (!(v = val())) return false;
      o->n0 = std::atoi(v);
    } else if (k == "--n1") {
      if (!(v = val())) return false;
      o->n1 = std::atoi(v);
    } else if (k == "--nmax") {
      if (!(v = val())) return false;
      o->nmax = std::atoi(v);
    } else if (k == "--dt") {
      if (!(v = val())) return false;
      o->dt = std::strtof(v, nullptr);
    } else if (k == "--seed") {
      if (!(v = val())) return false;
      o->seed = std::strtoull(v, nullptr, 10);
    } else if (k == "--coverage") {
      if (!(v = val())) return false;
      o->coverage = std::strtof(v, nullptr);
    } else if (k == "--direction") {
      if (!(v = val())) return false;
      o->direction = std::strtof(v, nullptr);
    } else if (k == "--speed") {
      if (!(v = val())) return false;
      o->u_ref = std::strtof(v, nullptr);
    } else if (k == "--out") {
      if (!(v = val())) return false;
      o->out = v;
    } else if (k == "--restart") {
      if (a + 2 >= argc) return false;
      o->restart30 = argv[++a];
      o->restart31 = argv[++a];
    } else if (k == "--per-stage") {
      o->per_stage = true;
    } else if (k == "--no-aveflow") {
      o->aveflow = false;
    } else if (k == "--fixed-sor") {
      o->fixed_sor = true;
    } else if (k == "--little-endian") {
      o->little_endian = true;
    } else if (k == "--quiet") {
      o->quiet = true;
    } else {
      return false;
    }
  }
  return o->im > 0 && o->jm > 0 && o->km > 0 && o->n0 >= 1 && o->nmax >= o->n0 && o->n1 >= 1 && o->dt > 0.f;
}

les_handle *g_h = nullptr;

// Report a failed call with the library's message and stop (the reference stops too).
void check(int rc, const char *what) {
  if (rc == LES_OK) return;
  char msg[512] = "";
  if (g_h) les_gpu_last_error(g_h, msg, sizeof msg);
  std::fprintf(stderr, "les_main: %s failed (status %d)%s%s\n", what, rc, *msg ? ": " : "", msg);
  if (g_h) les_gpu_destroy(g_h);
  std::exit(1);
}

float at(int field, int i, int j, int k) {
  const int lb[3] = {i, j, k};
  float x = 0.f;
  check(les_gpu_download(g_h, field, &x, lb, lb), "download");
  return x;
}

double now() {
  return std::chrono::duration<double>(std::chrono::steady_clock::now().time_since_epoch()).count();
}

}  // namespace

int main(int argc, char **argv) {
  Options o;
  if (!parse(argc, argv, &o)) {
    usage(stderr);
    return 2;
  }
  const int flags = o.little_endian ? LES_IO_LITTLE_ENDIAN : 0;
  ::mkdir(o.out.c_str(), 0755);  // may exist already; a failed open reports the rest

  // set.f95:89-95 and press.f95:43-45
  les_dims dims = {o.im, o.jm, o.km};
  les_params prm = {o.dt, 1.1763f, 15.83f * 1e-6f, -10.f, -1.f, 1.f, 1e-4f, 50, o.fixed_sor ? 1 : 0, 0};
  check(les_gpu_create(&dims, &prm, &g_h), "les_gpu_create (is a GPU present?)");

  les_scenario sc;
  std::memset(&sc, 0, sizeof sc);
  sc.im = o.im; sc.jm = o.jm; sc.km = o.km;
  sc.dx = 4.f; sc.dy = 4.f; sc.dz_law = 1; sc.dz0 = 2.f; sc.dz_ratio = 1.04f;
  sc.seed = o.seed; sc.coverage = o.coverage; sc.fp_min = 5; sc.fp_max = 20; sc.h_min = 10.f; sc.h_max = 60.f;
  sc.inflow_law = 1; sc.u_ref = o.u_ref; sc.z_ref = 100.f; sc.pl_exp = 0.2f; sc.direction_deg = o.direction;
  sc.noise = 1e-3f;
  check(les_gpu_setup_scenario(g_h, &sc), "set-up");
  if (!o.restart30.empty()) {
    int nr = 0;
    float tr = 0.f;
    check(les_gpu_read_restart(g_h, o.restart30.c_str(), o.restart31.c_str(), &nr, &tr), "restart read");
    if (!o.quiet) std::printf("ifdata: restart from step %d, time %g\n", nr, (double)tr);
  }
  if (!o.quiet)
    std::printf("MAIN: running GB300 LES code for %d time steps, domain = %d x %d x %d\n", o.nmax - o.n0 + 1,
                o.im, o.jm, o.km);

  const std::string d20 = o.out + "/data20", d21 = o.out + "/data21";
  const std::string d10 = o.out + "/data10", d11 = o.out + "/data11";
  static const char *kStage[7] = {"velnw", "bondv1", "velfg", "feedbf", "les", "adam", "press"};
  double stage_s[7] = {0, 0, 0, 0, 0, 0, 0};
  const double t_loop = now();
  for (int n = o.n0; n <= o.nmax; ++n) {
    const float time = (float)(n - 1) * o.dt;  // main.f95:248
    if (o.per_stage) {
      for (int s = 0; s < 7; ++s) {
        const double t0 = now();
        int rc;
        switch (s) {
          case 0: rc = les_gpu_velnw(g_h); break;
          case 1: rc = les_gpu_bondv1(g_h, n); break;
          case 2: rc = les_gpu_velfg(g_h); break;
          case 3: rc = les_gpu_feedbf(g_h); break;
          case 4: rc = les_gpu_les(g_h); break;
          case 5: rc = les_gpu_adam(g_h); break;
          default: rc = les_gpu_press(g_h, n, o.nmax); break;
        }
        check(rc, kStage[s]);
        check(les_gpu_sync(g_h), kStage[s]);
        stage_s[s] += now() - t0;
      }
    } else {
      check(les_gpu_step(g_h, n, o.nmax), "step");
    }
    if (n % 1000 == 0 || n == o.nmax) {  // press.f95:197-216 and adam.f95:20-27
      const int ic = o.im / 2, jc = o.jm / 2, kc = o.km / 2;
      if (!o.quiet)
        std::printf(" timestep: %d pressure at centre: %g vel at centre: %g %g %g\n", n / 1000,
                    (double)at(LES_FIELD_P, ic, jc, kc), (double)at(LES_FIELD_U, ic, jc, kc),
                    (double)at(LES_FIELD_V, ic, jc, kc), (double)at(LES_FIELD_W, ic, jc, kc));
      check(les_gpu_write_data21(g_h, d21.c_str(), flags), "data21");
      check(les_gpu_write_data20(g_h, d20.c_str(), flags), "data20");
    }
    int wrote = 0;
    check(les_gpu_ifdata_out(g_h, o.out.c_str(), n, o.n1, o.nmax, time, flags, &wrote), "ifdata_out");
    if (o.aveflow) {
      check(les_gpu_aveflow(g_h, n, o.n1, o.nmax), "aveflow");
      if (n == o.nmax) {
        check(les_gpu_write_data10(g_h, d10.c_str(), flags), "data10");
        check(les_gpu_write_data11(g_h, d11.c_str(), flags), "data11");
      }
    }
  }
  check(les_gpu_sync(g_h), "sync");
  const double wall = now() - t_loop;
  long long bad = 0;
  check(les_gpu_check_finite(g_h, &bad), "check_finite");
  double diag[5];
  check(les_gpu_diag(g_h, diag), "diag");
  const double cells = (double)o.im * o.jm * o.km, steps = o.nmax - o.n0 + 1;
  if (o.per_stage && !o.quiet)
    for (int s = 0; s < 7; ++s)
      std::printf("Time for state %2d = %9.3f ms  (%s, per step, with a synchronisation)\n", s + 1,
                  1e3 * stage_s[s] / steps, kStage[s]);
  std::printf("les_main: %d steps of %d x %d x %d in %.3f s, %.4g cell-steps/s (output included); "
              "last press: %d SOR iterations, residual %.6g; non-finite values: %lld\n",
              (int)steps, o.im, o.jm, o.km, wall, cells * steps / wall, (int)diag[0], diag[1], bad);
  les_gpu_destroy(g_h);
  return bad ? 3 : 0;
}
