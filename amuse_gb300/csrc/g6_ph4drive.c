/*
 * g6_ph4drive.c -- a caller of the GRAPE-6 ABI, written the way ph4 calls
 * it (src/amuse_ph4/src/gpu.cc).  It is not part of libsapporo.so; tests and
 * the benchmark's end-to-end leg use it so that the library is exercised by
 * C loops over host arrays, as in the worker process, rather than by one
 * Python call per particle.
 *
 *   drv_load   jdata::initialize_gpu  (gpu.cc:36-92):  one g6_set_j_particle
 *              per j, slot = j, index = id[j], a2 = acc/2, j6 = jerk/6, k18 = 0.
 *   drv_update idata::update_gpu      (gpu.cc:163-230): the same for a list.
 *   drv_force  idata::get_partial_acc_and_jerk_on_gpu (gpu.cc:302-408):
 *              g6_set_ti, then i-chunks of g6_npipes(): g6calc_firsthalf +
 *              g6calc_lasthalf (or lasthalf2 when neighbours are wanted).
 */
#include <stdlib.h>

#include "g6.h"

static int clusterid = 0;

int drv_load(int n, const int *ids, const double *t, const double *dt, const double *m,
             const double (*pos)[3], const double (*vel)[3], const double (*acc)[3],
             const double (*jerk)[3]) {
  double a2[3], j6[3], k18[3] = {0, 0, 0};
  for (int j = 0; j < n; j++) {
    for (int k = 0; k < 3; k++) {
      a2[k] = acc ? acc[j][k] / 2 : 0.0;
      j6[k] = jerk ? jerk[j][k] / 6 : 0.0;
    }
    int addr = j, idx = ids[j];
    double tj = t ? t[j] : 0.0, dtj = dt ? dt[j] : 0.0, mj = m[j];
    int rc = g6_set_j_particle_(&clusterid, &addr, &idx, &tj, &dtj, &mj, k18, j6, a2,
                                (double *)vel[j], (double *)pos[j]);
    if (rc) return rc;
  }
  return 0;
}

int drv_update(int nlist, const int *slots, const int *ids, const double *t, const double *dt,
               const double *m, const double (*pos)[3], const double (*vel)[3],
               const double (*acc)[3], const double (*jerk)[3]) {
  double a2[3], j6[3], k18[3] = {0, 0, 0};
  for (int q = 0; q < nlist; q++) {
    const int j = slots[q];
    for (int k = 0; k < 3; k++) {
      a2[k] = acc[j][k] / 2;
      j6[k] = jerk[j][k] / 6;
    }
    int addr = j, idx = ids[j];
    double tj = t[j], dtj = dt[j], mj = m[j];
    int rc = g6_set_j_particle_(&clusterid, &addr, &idx, &tj, &dtj, &mj, k18, j6, a2,
                                (double *)vel[j], (double *)pos[j]);
    if (rc) return rc;
  }
  return 0;
}

int drv_force(int nj, double ti, double eps2, int ni, const int *ids, const double (*ipos)[3],
              const double (*ivel)[3], const double *h2in, double (*acc)[3], double (*jerk)[3],
              double *pot, int *nn, int want_nn) {
  const int npipes = g6_npipes_();
  double *h2 = (double *)malloc(sizeof(double) * (size_t)npipes);
  double(*a2)[3] = (double(*)[3])malloc(sizeof(double) * 3 * (size_t)npipes);
  double(*j6)[3] = (double(*)[3])malloc(sizeof(double) * 3 * (size_t)npipes);
  if (!h2 || !a2 || !j6) {
    free(h2); free(a2); free(j6);
    return G6_ERR_NOMEM;
  }
  for (int i = 0; i < npipes; i++) {
    h2[i] = eps2;
    for (int k = 0; k < 3; k++) a2[i][k] = j6[i][k] = 0;
  }
  int rc = g6_set_ti_(&clusterid, &ti);
  for (int i = 0; i < ni && rc == 0; i += npipes) {
    int nni = ni - i < npipes ? ni - i : npipes;
    if (h2in)
      for (int q = 0; q < nni; q++) h2[q] = h2in[i + q];
    int njj = nj;
    double e2 = eps2;
    g6calc_firsthalf_(&clusterid, &njj, &nni, (int *)ids + i, (double(*)[3])ipos + i,
                      (double(*)[3])ivel + i, a2, j6, pot + i, &e2, h2);
    if (want_nn)
      rc = g6calc_lasthalf2_(&clusterid, &njj, &nni, (int *)ids + i, (double(*)[3])ipos + i,
                             (double(*)[3])ivel + i, &e2, h2, acc + i, jerk + i, pot + i,
                             nn + i);
    else
      rc = g6calc_lasthalf_(&clusterid, &njj, &nni, (int *)ids + i, (double(*)[3])ipos + i,
                            (double(*)[3])ivel + i, &e2, h2, acc + i, jerk + i, pot + i);
  }
  free(h2);
  free(a2);
  free(j6);
  return rc;
}
