// ph4_gpu_main.cc -- TEST INFRASTRUCTURE ONLY: the drop-in link check.
//
// main() around ph4_harness.cc's ph4ref_run, for the build of the UNMODIFIED
// ph4 objects in GPU mode (-DGPU -DNOMPI, oracle/Makefile target "link"):
// jdata/idata then reach gravity only through ph4's own GRAPE-6 glue
// (src/amuse_ph4/src/gpu.cc:36-492 via the by-value wrappers of grape.cc),
// and those calls resolve to this repository's libsapporo.so.
//
// Usage: ph4_gpu_run [n] [t_end]  -- a uniform sphere of n equal masses
// (drand48, seed 1), eps2 = 1e-4, eta = 0.01; prints E0, E1, block steps.
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <vector>

extern "C" int ph4ref_run(int n, const double *mass, const int *ids, const double *pos,
                          const double *vel, double eps2, double eta, double t_end,
                          double *pos_out, double *vel_out, double *acc_out,
                          double *jerk_out, double *pot_out, double *time_out,
                          double *step_out, double *stats);

int main(int argc, char **argv) {
  const int n = argc > 1 ? atoi(argv[1]) : 256;
  const double t_end = argc > 2 ? atof(argv[2]) : 0.0625;
  if (n < 2) return 2;
  srand48(1);
  std::vector<double> m(n, 1.0 / n), x(3 * n), v(3 * n), out(3 * n * 4 + 3 * n);
  std::vector<int> ids(n);
  for (int j = 0; j < n; j++) {
    ids[j] = j + 1;
    double r2;
    do {
      for (int k = 0; k < 3; k++) x[3 * j + k] = 2 * drand48() - 1;
      r2 = x[3 * j] * x[3 * j] + x[3 * j + 1] * x[3 * j + 1] + x[3 * j + 2] * x[3 * j + 2];
    } while (r2 > 1);
    for (int k = 0; k < 3; k++) v[3 * j + k] = 0.3 * (2 * drand48() - 1);
  }
  std::vector<double> po(3 * n), vo(3 * n), ao(3 * n), jo(3 * n), pot(n), t(n), dt(n);
  double stats[5];
  ph4ref_run(n, m.data(), ids.data(), x.data(), v.data(), 1e-4, 0.01, t_end, po.data(),
             vo.data(), ao.data(), jo.data(), pot.data(), t.data(), dt.data(), stats);
  printf("E0 %.15g E1 %.15g dE/E %.3e blocks %.0f t %.6g\n", stats[0], stats[1],
         std::fabs((stats[1] - stats[0]) / stats[0]), stats[4], stats[3]);
  return 0;
}
