/*
 * g6_oracle.c -- TEST INFRASTRUCTURE ONLY (the oracle).
 *
 * A plain-C restatement of AMUSE ph4's FP64 CPU Hermite path, used by the
 * test-suite, by __graft_entry__.smoke() and by bench.py's CPU-baseline leg
 * as the checker.  Nothing in the shipped library links, loads or calls this
 * file; the product (libsapporo.so) has no CPU force path at all.
 *
 * Every function follows the reference loop-for-loop so that, compiled with
 * -O2 -ffp-contract=off, it is bit-identical to the unmodified ph4 objects
 * (pinned by tests/test_oracle.py against fixtures generated from
 * the reference build, see oracle/Makefile target `ref`).
 *
 *   orc_force          src/amuse_ph4/src/idata.cc:147-237   (get_partial_acc_and_jerk)
 *   orc_predict        src/amuse_ph4/src/jdata.cc:710-750   (predict_all)
 *   orc_correct        src/amuse_ph4/src/idata.cc:399-514   (correct + Aarseth step)
 *   orc_initial_step   src/amuse_ph4/src/jdata.cc:503-564   (set_initial_timestep)
 *   orc_run            src/amuse_ph4/src/jdata.cc:752-795 + idata.cc:832-881
 *                      (block-step loop of interface.cc:614-711, CPU mode,
 *                      manage_encounters = 0)
 *   orc_run_enc        the same loop with idata::check_encounters
 *                      (idata.cc:620-700) after every block and the
 *                      COLLISION_DETECTION stopping condition of
 *                      jdata::advance_and_check_encounter (jdata.cc:797-850)
 *   orc_hermite_fixed  src/amuse_hermite/interface.cc:266-281,387-552
 *                      (shared fixed-step Hermite, test_mode)
 *   orc_knn            src/amuse_ph4/src/gpu.cc:534-558 (save_neighbors:
 *                      all other particles by squared distance, the first
 *                      knn kept), over the whole j-system
 */
#include <math.h>
#include <pthread.h>
#include <stdlib.h>
#include <string.h>

#define ORC_TINY (1.0 / 4503599627370496.0) /* 2^-52, stdinc.h:33 */
#define ORC_INF 1.0e300                     /* stdinc.h:32 */

/* ------------------------------------------------------------------ */
/* Force: idata::get_partial_acc_and_jerk (idata.cc:147-237).          */
/* j-arrays are the predicted j-system; i-arrays the predicted i's.     */
/* nn[i] is a j index (-1 if none); dnn[i] = sqrt(min r2).             */
/* ------------------------------------------------------------------ */
static void force_range(int i0, int i1, int nj, const double *mass,
                        const double *jpos, const double *jvel, double eps2,
                        const double *ipos, const double *ivel, double *acc,
                        double *jerk, double *pot, int *nn, double *dnn) {
  double dx[3], dv[3], r2, xv, r2i, ri, mri, mr3i, a3;
  for (int i = i0; i < i1; i++) {
    double lpot = 0, ldnn = ORC_INF;
    int lnn = -1;
    double la[3] = {0, 0, 0}, lj[3] = {0, 0, 0};
    for (int j = 0; j < nj; j++) {
      if (mass[j] > ORC_TINY) {
        r2 = xv = 0;
        for (int k = 0; k < 3; k++) {
          dx[k] = jpos[3 * j + k] - ipos[3 * i + k];
          dv[k] = jvel[3 * j + k] - ivel[3 * i + k];
          r2 += dx[k] * dx[k];
          xv += dx[k] * dv[k];
        }
        r2i = 1 / (r2 + eps2 + ORC_TINY);
        ri = sqrt(r2i);
        mri = mass[j] * ri;
        mr3i = mri * r2i;
        a3 = -3 * xv * r2i;
        if (r2 > ORC_TINY) {
          lpot -= mri;
          if (r2 < ldnn) {
            ldnn = r2;
            lnn = j;
          }
        }
        for (int k = 0; k < 3; k++) {
          la[k] += mr3i * dx[k];
          lj[k] += mr3i * (dv[k] + a3 * dx[k]);
        }
      }
    }
    pot[i] = lpot;
    for (int k = 0; k < 3; k++) {
      acc[3 * i + k] = la[k];
      jerk[3 * i + k] = lj[k];
    }
    if (nn) nn[i] = lnn;
    if (dnn) dnn[i] = sqrt(ldnn);
  }
}

void orc_force(int nj, const double *mass, const double *jpos,
               const double *jvel, double eps2, int ni, const double *ipos,
               const double *ivel, double *acc, double *jerk, double *pot,
               int *nn, double *dnn) {
  force_range(0, ni, nj, mass, jpos, jvel, eps2, ipos, ivel, acc, jerk, pot,
              nn, dnn);
}

/* Multi-threaded wrapper: k threads over disjoint i-ranges, each running
   the same scalar loop (the reference has no threading; this is the
   all-cores CPU baseline). */
struct force_job {
  int i0, i1, nj;
  const double *mass, *jpos, *jvel, *ipos, *ivel;
  double eps2;
  double *acc, *jerk, *pot, *dnn;
  int *nn;
};

static void *force_thread(void *arg) {
  struct force_job *f = (struct force_job *)arg;
  force_range(f->i0, f->i1, f->nj, f->mass, f->jpos, f->jvel, f->eps2,
              f->ipos, f->ivel, f->acc, f->jerk, f->pot, f->nn, f->dnn);
  return NULL;
}

int orc_force_mt(int nthreads, int nj, const double *mass, const double *jpos,
                 const double *jvel, double eps2, int ni, const double *ipos,
                 const double *ivel, double *acc, double *jerk, double *pot,
                 int *nn, double *dnn) {
  if (nthreads < 1) nthreads = 1;
  if (nthreads > ni) nthreads = ni > 0 ? ni : 1;
  pthread_t *th = (pthread_t *)malloc(sizeof(pthread_t) * nthreads);
  struct force_job *jobs =
      (struct force_job *)malloc(sizeof(struct force_job) * nthreads);
  if (!th || !jobs) {
    free(th);
    free(jobs);
    return -1;
  }
  int started = 0;
  for (int t = 0; t < nthreads; t++) {
    struct force_job f = {(int)((long long)ni * t / nthreads),
                          (int)((long long)ni * (t + 1) / nthreads),
                          nj, mass, jpos, jvel, ipos, ivel, eps2,
                          acc, jerk, pot, dnn, nn};
    jobs[t] = f;
    if (pthread_create(&th[t], NULL, force_thread, &jobs[t]) == 0)
      started = t + 1;
    else
      break;
  }
  for (int t = 0; t < started; t++) pthread_join(th[t], NULL);
  /* Any range that could not get a thread runs on this one. */
  for (int t = started; t < nthreads; t++) force_thread(&jobs[t]);
  free(th);
  free(jobs);
  return nthreads;
}

/* ------------------------------------------------------------------ */
/* Predictor: jdata::predict_all (jdata.cc:710-750); identical to the   */
/* GPU-mode i-predictor idata::predict (idata.cc:346-365).              */
/* ------------------------------------------------------------------ */
void orc_predict(int n, double t, const double *time, const double *pos,
                 const double *vel, const double *acc, const double *jerk,
                 double *pred_pos, double *pred_vel) {
  for (int j = 0; j < n; j++) {
    double dt = t - time[j];
    if (dt == 0) {
      for (int k = 0; k < 3; k++) {
        pred_pos[3 * j + k] = pos[3 * j + k];
        pred_vel[3 * j + k] = vel[3 * j + k];
      }
    } else {
      for (int k = 0; k < 3; k++) {
        pred_pos[3 * j + k] =
            pos[3 * j + k] +
            dt * (vel[3 * j + k] +
                  0.5 * dt * (acc[3 * j + k] + dt * jerk[3 * j + k] / 3));
        pred_vel[3 * j + k] =
            vel[3 * j + k] + dt * (acc[3 * j + k] + 0.5 * dt * jerk[3 * j + k]);
      }
    }
  }
}

/* ------------------------------------------------------------------ */
/* Corrector + Aarseth step: idata::correct (idata.cc:399-514).         */
/* ipos/ivel hold the predicted values on entry, corrected on exit.     */
/* itime/itimestep are updated in place.                                */
/* ------------------------------------------------------------------ */
void orc_correct(int ni, double tnext, double eta, double *itime,
                 double *itimestep, double *ipos, double *ivel,
                 const double *old_acc, const double *old_jerk,
                 const double *iacc, const double *ijerk) {
  for (int i = 0; i < ni; i++) {
    double dt = tnext - itime[i];
    double dt2 = dt * dt;
    double a2 = 0, j2 = 0, k2 = 0, l2 = 0;
    for (int k = 0; k < 3; k++) {
      double alpha = -3 * (old_acc[3 * i + k] - iacc[3 * i + k]) -
                     dt * (2 * old_jerk[3 * i + k] + ijerk[3 * i + k]);
      double beta = 2 * (old_acc[3 * i + k] - iacc[3 * i + k]) +
                    dt * (old_jerk[3 * i + k] + ijerk[3 * i + k]);
      ipos[3 * i + k] += (alpha / 12 + beta / 20) * dt2;
      ivel[3 * i + k] += (alpha / 3 + beta / 4) * dt;
      a2 += pow(iacc[3 * i + k], 2);
      j2 += pow(dt * ijerk[3 * i + k], 2);
      k2 += pow(2 * alpha, 2);
      l2 += pow(6 * beta, 2);
    }
    double newstep = eta * dt * sqrt((sqrt(a2 * k2) + j2) / (sqrt(j2 * l2) + k2));
    int exponent;
    double oldstep2 = itimestep[i] / (2 * frexp(itimestep[i], &exponent));
    while (fmod(tnext, oldstep2) != 0) oldstep2 /= 2;
    if (newstep < oldstep2) {
      newstep = oldstep2 / 2;
    } else {
      double t2 = 2 * oldstep2;
      if (newstep >= t2 && fmod(tnext, t2) == 0)
        newstep = t2;
      else
        newstep = oldstep2;
    }
    itime[i] = tnext;
    itimestep[i] = newstep;
  }
}

/* ------------------------------------------------------------------ */
/* Initial step: jdata::set_initial_timestep (jdata.cc:503-564), with   */
/* all steps forced to zero first (force_initial_timestep, :566-580).   */
/* ------------------------------------------------------------------ */
static int cmp_double(const void *a, const void *b) {
  double x = *(const double *)a, y = *(const double *)b;
  return (x > y) - (x < y);
}

void orc_initial_step(int n, double system_time, double eta, double fac,
                      double limit, double limitm, const double *acc,
                      const double *jerk, double *timestep) {
  for (int j = 0; j < n; j++) {
    double a2 = 0, j2 = 0;
    for (int k = 0; k < 3; k++) {
      a2 += pow(acc[3 * j + k], 2);
      j2 += pow(jerk[3 * j + k], 2);
    }
    double firststep;
    if (eta == 0.0)
      firststep = limit;
    else if (a2 == 0.0 || j2 == 0.0)
      firststep = fac * eta;
    else
      firststep = fac * eta * sqrt(a2 / j2);
    if (isnan(firststep)) firststep = fac * eta;
    int exponent;
    firststep /= 2 * frexp(firststep, &exponent);
    while (fmod(system_time, firststep) != 0) firststep /= 2;
    while (firststep > limit) firststep /= 2;
    timestep[j] = firststep;
  }
  if (limitm > 0 && n > 0) {
    double *tmp = (double *)malloc(sizeof(double) * n);
    memcpy(tmp, timestep, sizeof(double) * n);
    qsort(tmp, n, sizeof(double), cmp_double);
    double dtmax = limitm * tmp[n / 2];
    free(tmp);
    for (int j = 0; j < n; j++)
      while (timestep[j] > dtmax) timestep[j] /= 2;
  }
}

/* ------------------------------------------------------------------ */
/* Energy: jdata::get_energy(false) (jdata.cc:582-680): pot via the     */
/* force path at system_time, kin from predicted velocities.            */
/* ------------------------------------------------------------------ */
static double energy_at(int n, double t, const double *mass, const double *time,
                        const double *pos, const double *vel, const double *acc,
                        const double *jerk, double eps2, double *scratch,
                        int nthreads) {
  double *pp = scratch, *pv = scratch + 3 * n, *a = scratch + 6 * n,
         *jk = scratch + 9 * n, *pot = scratch + 12 * n;
  orc_predict(n, t, time, pos, vel, acc, jerk, pp, pv);
  orc_force_mt(nthreads, n, mass, pp, pv, eps2, n, pp, pv, a, jk, pot, NULL,
               NULL);
  double pot2 = 0, kin2 = 0;
  for (int i = 0; i < n; i++) pot2 += mass[i] * pot[i];
  for (int j = 0; j < n; j++) {
    double v2 = 0;
    for (int k = 0; k < 3; k++) v2 += pow(pv[3 * j + k], 2);
    kin2 += mass[j] * v2;
  }
  return pot2 / 2 + kin2 / 2;
}

/* ------------------------------------------------------------------ */
/* Full block-step run, CPU mode, one process, manage_encounters = 0:  */
/* commit_particles (interface.cc:317-347) then evolve_model            */
/* (interface.cc:614-711) -> jdata::advance (jdata.cc:752-795) ->        */
/* idata::advance (idata.cc:832-881).  The block is found with the O(N) */
/* search of idata::set_list (idata.cc:796-806, the "#if 0" branch);     */
/* it selects the same set as the list scheduler, and each particle's   */
/* update is independent of the order within the block.                 */
/* State arrays are updated in place; returns block steps taken.        */
/* stats (optional, length 4): E0, E1, total particle steps, t_final.   */
/* ------------------------------------------------------------------ */
/* Encounter check modes (bits), shared with the library's g6x_set_encounters. */
#define ORC_ENC_CHECK 1     /* run idata::check_encounters after every block */
#define ORC_ENC_STOP_COLL 2 /* stop as COLLISION_DETECTION does (vr test) */
#define ORC_ENC_STOP_CLOSE 4 /* stop when a close pair (rmin) is found */
#define ORC_ENC_EPS 0.001   /* jdata.cc:797 (from couple/multiples.py) */

/* idata::check_encounters (idata.cc:620-700) in CPU mode for one block:
   nn/dnn are the block's nearest neighbours (j indices) and distances from
   the force loop.  The first i (block order = slot order here) with the
   largest rmin/dnn, resp. (R_i + R_nn)/dnn, wins; a pair is reported when
   that ratio is >= 1.  ph4 tests the mass of i as imass[i], which CPU mode
   never fills; the nn of a CPU-mode force always has mass > 2^-52, so the
   test passes either way.  enc[0..5]: close pair (slots), collision pair
   (slots), rmax_close, rmax_coll. */
static void check_encounters(int ni, const int *ilist, const int *inn,
                             const double *idnn, const double *mass,
                             const double *radius, double rmin, double *enc) {
  double rmax_close = 0, rmax_coll = 0;
  int imax_close = -1, imax_coll = -1;
  for (int i = 0; i < ni; i++) {
    int jnn = inn[i];
    if (jnn < 0) continue;
    if (mass[jnn] > ORC_TINY || mass[ilist[i]] > ORC_TINY) {
      double r = rmin / idnn[i];
      if (r > rmax_close) {
        rmax_close = r;
        imax_close = i;
      }
      r = (radius[ilist[i]] + radius[jnn]) / idnn[i];
      if (r > rmax_coll) {
        rmax_coll = r;
        imax_coll = i;
      }
    }
  }
  enc[0] = enc[1] = enc[2] = enc[3] = -1;
  if (rmax_close >= 1) {
    enc[0] = ilist[imax_close];
    enc[1] = inn[imax_close];
  }
  if (rmax_coll >= 1) {
    enc[2] = ilist[imax_coll];
    enc[3] = inn[imax_coll];
  }
  enc[4] = rmax_close;
  enc[5] = rmax_coll;
}

/* The COLLISION_DETECTION test of jdata::advance_and_check_encounter
   (jdata.cc:822-848) on the current (corrected) state of the pair. */
static int collision_approaching(const double *pos, const double *vel, int j1,
                                 int j2) {
  double r = 0, v = 0, vr = 0;
  for (int k = 0; k < 3; k++) {
    double dx = pos[3 * j1 + k] - pos[3 * j2 + k];
    double dv = vel[3 * j1 + k] - vel[3 * j2 + k];
    r += dx * dx;
    v += dv * dv;
    vr += dx * dv;
  }
  r = sqrt(r);
  v = sqrt(v);
  return vr < ORC_ENC_EPS * r * v;
}

static long run_impl(int n, const double *mass, double *pos, double *vel,
                     double eps2, double eta, double t_end, int nthreads,
                     double *acc, double *jerk, double *pot, double *time,
                     double *timestep, double *stats, long max_blocks,
                     const double *radius, int enc_mode, double rmin,
                     double *enc_out) {
  double *pp = (double *)malloc(sizeof(double) * 3 * n);
  double *pv = (double *)malloc(sizeof(double) * 3 * n);
  double *scratch = (double *)malloc(sizeof(double) * 13 * n);
  int *ilist = (int *)malloc(sizeof(int) * n);
  double *ip = (double *)malloc(sizeof(double) * 3 * n);
  double *iv = (double *)malloc(sizeof(double) * 3 * n);
  double *oa = (double *)malloc(sizeof(double) * 3 * n);
  double *oj = (double *)malloc(sizeof(double) * 3 * n);
  double *ia = (double *)malloc(sizeof(double) * 3 * n);
  double *ij = (double *)malloc(sizeof(double) * 3 * n);
  double *ipot = (double *)malloc(sizeof(double) * n);
  double *it = (double *)malloc(sizeof(double) * n);
  double *its = (double *)malloc(sizeof(double) * n);
  int *inn = (int *)malloc(sizeof(int) * n);
  double *idnn = (double *)malloc(sizeof(double) * n);
  double enc[6] = {-1, -1, -1, -1, 0, 0};
  int stopped = 0;
  /* jdata::initialize_arrays (jdata.cc:426): rmin = 2/nj by default. */
  if (rmin <= 0 && n > 0) rmin = 2. / n;
  double system_time = 0;
  /* commit_particles: initialize_arrays (time = 0, acc = jerk = 0),
     predict_all(0, true), idata::setup -> forces on all, scatter. */
  for (int j = 0; j < n; j++) {
    time[j] = 0;
    timestep[j] = 0;
  }
  memset(acc, 0, sizeof(double) * 3 * n);
  memset(jerk, 0, sizeof(double) * 3 * n);
  orc_predict(n, 0.0, time, pos, vel, acc, jerk, pp, pv);
  orc_force_mt(nthreads, n, mass, pp, pv, eps2, n, pp, pv, acc, jerk, pot,
               NULL, NULL);
  /* force_initial_timestep(0.0625, 0.03125, 8.0) (interface.cc:29-31). */
  orc_initial_step(n, 0.0, eta, 0.0625, 0.03125, 8.0, acc, jerk, timestep);
  double e0 = energy_at(n, system_time, mass, time, pos, vel, acc, jerk, eps2,
                        scratch, nthreads);
  long blocks = 0;
  double steps = 0;
  while (system_time < t_end && (max_blocks <= 0 || blocks < max_blocks)) {
    double tnext = ORC_INF;
    for (int j = 0; j < n; j++)
      if (time[j] + timestep[j] < tnext) tnext = time[j] + timestep[j];
    int ni = 0;
    for (int j = 0; j < n; j++)
      if (time[j] + timestep[j] == tnext) ilist[ni++] = j;
    orc_predict(n, tnext, time, pos, vel, acc, jerk, pp, pv);
    for (int i = 0; i < ni; i++) {
      int j = ilist[i];
      it[i] = time[j];
      its[i] = timestep[j];
      for (int k = 0; k < 3; k++) {
        ip[3 * i + k] = pp[3 * j + k];
        iv[3 * i + k] = pv[3 * j + k];
        oa[3 * i + k] = acc[3 * j + k];
        oj[3 * i + k] = jerk[3 * j + k];
      }
    }
    orc_force_mt(nthreads, n, mass, pp, pv, eps2, ni, ip, iv, ia, ij, ipot,
                 enc_mode ? inn : NULL, enc_mode ? idnn : NULL);
    orc_correct(ni, tnext, eta, it, its, ip, iv, oa, oj, ia, ij);
    for (int i = 0; i < ni; i++) {
      int j = ilist[i];
      pot[j] = ipot[i];
      time[j] = it[i];
      timestep[j] = its[i];
      for (int k = 0; k < 3; k++) {
        pos[3 * j + k] = ip[3 * i + k];
        vel[3 * j + k] = iv[3 * i + k];
        acc[3 * j + k] = ia[3 * i + k];
        jerk[3 * j + k] = ij[3 * i + k];
      }
    }
    blocks++;
    steps += ni;
    system_time = tnext;
    if (enc_mode) {
      check_encounters(ni, ilist, inn, idnn, mass, radius, rmin, enc);
      if ((enc_mode & ORC_ENC_STOP_COLL) && enc[2] >= 0 &&
          collision_approaching(pos, vel, (int)enc[2], (int)enc[3]))
        stopped = 1;
      if ((enc_mode & ORC_ENC_STOP_CLOSE) && enc[0] >= 0) stopped |= 2;
      if (stopped) break;
    }
  }
  double e1 = energy_at(n, system_time, mass, time, pos, vel, acc, jerk, eps2,
                        scratch, nthreads);
  if (stats) {
    stats[0] = e0;
    stats[1] = e1;
    stats[2] = steps;
    stats[3] = system_time;
  }
  if (enc_out) {
    for (int k = 0; k < 6; k++) enc_out[k] = enc[k];
    enc_out[6] = stopped;
    enc_out[7] = rmin;
  }
  free(pp); free(pv); free(scratch); free(ilist); free(ip); free(iv);
  free(oa); free(oj); free(ia); free(ij); free(ipot); free(it); free(its);
  free(inn); free(idnn);
  return blocks;
}

long orc_run(int n, const double *mass, double *pos, double *vel, double eps2,
             double eta, double t_end, int nthreads, double *acc, double *jerk,
             double *pot, double *time, double *timestep, double *stats,
             long max_blocks) {
  return run_impl(n, mass, pos, vel, eps2, eta, t_end, nthreads, acc, jerk,
                  pot, time, timestep, stats, max_blocks, NULL, 0, 0.0, NULL);
}

/* orc_run with the encounter check after every block.  radius[n] (ph4's
   particle radius), enc_mode (ORC_ENC_* bits), rmin (<= 0: 2/n).
   enc_out[8]: close pair (slots, -1 none), collision pair (slots),
   rmax_close, rmax_coll of the last block, stopped (1 collision, 2 close),
   rmin used.  A stop ends the run after that block, as the ph4 worker's
   evolve_model does (interface.cc:667-668). */
long orc_run_enc(int n, const double *mass, const double *radius, double *pos,
                 double *vel, double eps2, double eta, double t_end,
                 int nthreads, double *acc, double *jerk, double *pot,
                 double *time, double *timestep, double *stats,
                 long max_blocks, int enc_mode, double rmin, double *enc_out) {
  return run_impl(n, mass, pos, vel, eps2, eta, t_end, nthreads, acc, jerk,
                  pot, time, timestep, stats, max_blocks, radius, enc_mode,
                  rmin, enc_out);
}

/* ------------------------------------------------------------------ */
/* smallN's few-body integrator without the unperturbed-binary tree   */
/* (smallN with dt_crit = 0): all bodies are top-level nodes.           */
/*   calculate_top_level_acc_and_jerk  smallN.cc:318-363 (pairs i<j,   */
/*       get_pairwise_acc_and_jerk_CPT smallN.cc:121-273, leaf = node), */
/*   kepler_step_sq                    smallN.cc:85-116,               */
/*   take_a_step                       smallN.cc:553-682 (n_iter       */
/*       iterations of the time-symmetrised corrector),                */
/*   correct_acc_and_jerk / correct_pos_and_vel smallN.cc:487-531,     */
/*   predict_loworder                  hdyn.h:192-201,                 */
/*   smallN_evolve loop                smallN.cc:906-1117.             */
/* Vector operations follow vec.h (dot = (a0 b0 + a1 b1) + a2 b2, v/s   */
/* per component).  State in place; returns the number of steps.       */
/* ------------------------------------------------------------------ */
typedef struct {
  double m, pos[3], vel[3], pp[3], pv[3], acc[3], jerk[3], oacc[3], ojerk[3];
  double t_pred;
} sn_body;

static double sn_forces(int n, sn_body *b) {
  for (int i = 0; i < n; i++)
    for (int k = 0; k < 3; k++) b[i].acc[k] = b[i].jerk[k] = 0;
  double min_ts2 = ORC_INF;
  for (int i = 0; i < n; i++)
    for (int j = i + 1; j < n; j++) {
      double dx[3], dv[3];
      for (int k = 0; k < 3; k++) {
        dx[k] = b[j].pp[k] - b[i].pp[k] + 0.0;
        dv[k] = b[j].pv[k] - b[i].pv[k] + 0.0;
      }
      double d2 = dx[0] * dx[0] + dx[1] * dx[1] + dx[2] * dx[2];
      double d = sqrt(d2);
      double d3 = d2 * d;
      double xv = dx[0] * dv[0] + dx[1] * dv[1] + dx[2] * dv[2];
      double force[3], jerk[3];
      for (int k = 0; k < 3; k++) {
        double iforce = b[j].m * dx[k] / d3;
        double ijerk = b[j].m * (dv[k] / d3 - 3 * dx[k] * xv / (d3 * d2));
        force[k] = b[i].m * iforce;
        jerk[k] = b[i].m * ijerk;
      }
      /* kepler_step_sq(d2, d3, mi + mj, |vj - vi|^2) */
      double mass = b[j].m + b[i].m;
      double dvc[3];
      for (int k = 0; k < 3; k++) dvc[k] = b[j].pv[k] - b[i].pv[k];
      double vel2 = dvc[0] * dvc[0] + dvc[1] * dvc[1] + dvc[2] * dvc[2];
      double dtff2 = 0.5 * d3 / mass;
      double dtv2 = d2 / fabs(vel2);
      double ts2 = fmin(dtff2, dtv2);
      double mi = 1 / b[i].m, mj = 1 / b[j].m;
      for (int k = 0; k < 3; k++) {
        b[i].acc[k] += mi * force[k];
        b[i].jerk[k] += mi * jerk[k];
        b[j].acc[k] += -mj * force[k];
        b[j].jerk[k] += -mj * jerk[k];
      }
      if (ts2 < min_ts2) min_ts2 = ts2;
    }
  return min_ts2;
}

long orc_smalln(int n, const double *mass, double *pos, double *vel, double eta, int n_iter,
                double t_end, double *t_out, long max_steps) {
  sn_body *b = (sn_body *)calloc((size_t)n, sizeof(sn_body));
  for (int i = 0; i < n; i++) {
    b[i].m = mass[i];
    b[i].t_pred = -1;
    for (int k = 0; k < 3; k++) {
      b[i].pos[k] = pos[3 * i + k];
      b[i].vel[k] = vel[3 * i + k];
      b[i].pp[k] = b[i].pos[k]; /* init_pred */
      b[i].pv[k] = b[i].vel[k];
    }
  }
  double t = 0, root_t_pred = -1;
  double dt = eta * sqrt(sn_forces(n, b));
  long steps = 0;
  while (t < t_end && (max_steps <= 0 || steps < max_steps)) {
    /* take_a_step */
    double tn = t + dt;
    if (tn != root_t_pred) { /* predict_loworder_all */
      for (int i = 0; i < n; i++) {
        if (tn != b[i].t_pred) {
          double h = tn - t, h3 = h / 3, h2 = h / 2;
          for (int k = 0; k < 3; k++) {
            b[i].pp[k] = ((b[i].ojerk[k] * h3 + b[i].oacc[k]) * h2 + b[i].vel[k]) * h + b[i].pos[k];
            b[i].pv[k] = (b[i].ojerk[k] * h2 + b[i].oacc[k]) * h + b[i].vel[k];
          }
          b[i].t_pred = tn;
        }
      }
      root_t_pred = tn;
    }
    for (int i = 0; i < n; i++)
      for (int k = 0; k < 3; k++) {
        b[i].oacc[k] = b[i].acc[k];
        b[i].ojerk[k] = b[i].jerk[k];
      }
    double new_dt = dt, end_dt = dt;
    for (int it = 0; it <= n_iter; it++) {
      double prev = new_dt;
      end_dt = eta * sqrt(sn_forces(n, b));
      if (it < n_iter) {
        new_dt = 0.5 * (dt + end_dt);
        new_dt = dt + 0.5 * (end_dt - dt) * (new_dt / prev);
      }
      for (int i = 0; i < n; i++) {
        if (new_dt != prev) { /* correct_acc_and_jerk(new_dt, prev) */
          double dt_off = new_dt - 0.5 * prev;
          double theta = 0.5 * prev;
          double tau = dt_off / theta;
          double inv_theta = 1 / theta;
          double tau2 = tau * tau, tau3 = tau2 * tau;
          for (int k = 0; k < 3; k++) {
            double pa = b[i].acc[k], pj = b[i].jerk[k];
            double oa = b[i].oacc[k], oj = b[i].ojerk[k];
            b[i].acc[k] = 0.25 * (oa * (2 - 3 * tau + tau3) + pa * (2 + 3 * tau - tau3) +
                                  oj * theta * (1 - tau - tau2 + tau3) +
                                  pj * theta * (-1 - tau + tau2 + tau3));
            b[i].jerk[k] = 0.25 * (oa * inv_theta * 3 * (-1 + tau2) + pa * inv_theta * 3 * (1 - tau2) +
                                   oj * (-1 - 2 * tau + 3 * tau2) + pj * (-1 + 2 * tau + 3 * tau2));
          }
        }
        /* correct_pos_and_vel(new_dt) */
        double nd2 = new_dt * new_dt;
        for (int k = 0; k < 3; k++) {
          b[i].pv[k] = b[i].vel[k] + new_dt * (b[i].acc[k] + b[i].oacc[k]) / 2 -
                       nd2 * (b[i].jerk[k] - b[i].ojerk[k]) / 12;
          b[i].pp[k] = b[i].pos[k] + new_dt * (b[i].pv[k] + b[i].vel[k]) / 2 -
                       nd2 * (b[i].acc[k] - b[i].oacc[k]) / 12;
        }
      }
    }
    for (int i = 0; i < n; i++)
      for (int k = 0; k < 3; k++) {
        b[i].pos[k] = b[i].pp[k];
        b[i].vel[k] = b[i].pv[k];
      }
    dt = end_dt;
    t = t + new_dt;
    steps++;
  }
  for (int i = 0; i < n; i++)
    for (int k = 0; k < 3; k++) {
      pos[3 * i + k] = b[i].pos[k];
      vel[3 * i + k] = b[i].vel[k];
    }
  if (t_out) *t_out = t;
  free(b);
  return steps;
}

/* ------------------------------------------------------------------ */
/* Fixed-step shared Hermite: the hermite code in test_mode            */
/* (calculate_step returns dt_param, interface.cc:618-637):            */
/*   hf_forces    get_acc_jerk_pot_coll   interface.cc:387-533         */
/*                (symmetric j > i pair loop; note rv_r2 = (r.v)/r^2   */
/*                uses the UNsoftened r^2 while r3 is softened)        */
/*   predict      predict_step            interface.cc:266-281         */
/*   correct      correct_step            interface.cc:536-552         */
/*   step loop    evolve_step             interface.cc:558-616         */
/* pos/vel in place; acc/jerk (may be NULL) receive the final forces.  */
/* ------------------------------------------------------------------ */
static void hf_forces(int n, const double *mass, const double *pos, const double *vel,
                      double eps2, double *acc, double *jerk) {
  for (int i = 0; i < n; i++)
    for (int k = 0; k < 3; k++) acc[3 * i + k] = jerk[3 * i + k] = 0;
  for (int i = 0; i < n; i++)
    for (int j = i + 1; j < n; j++) {
      double rji[3], vji[3];
      for (int k = 0; k < 3; k++) {
        rji[k] = pos[3 * j + k] - pos[3 * i + k];
        vji[k] = vel[3 * j + k] - vel[3 * i + k];
      }
      double r2 = 0, rv_r2 = 0;
      for (int k = 0; k < 3; k++) {
        r2 += rji[k] * rji[k];
        rv_r2 += rji[k] * vji[k];
      }
      rv_r2 /= r2;
      r2 += eps2;
      double r = sqrt(r2);
      double r3 = r * r2;
      double da[3], dj[3];
      for (int k = 0; k < 3; k++) {
        da[k] = rji[k] / r3;
        dj[k] = (vji[k] - 3 * rv_r2 * rji[k]) / r3;
      }
      for (int k = 0; k < 3; k++) {
        acc[3 * i + k] += mass[j] * da[k];
        acc[3 * j + k] -= mass[i] * da[k];
        jerk[3 * i + k] += mass[j] * dj[k];
        jerk[3 * j + k] -= mass[i] * dj[k];
      }
    }
}

void orc_hermite_fixed(int n, const double *mass, double *pos, double *vel, double eps2,
                       double dt, int nsteps, double *acc_out, double *jerk_out) {
  size_t b = sizeof(double) * 3 * (size_t)n;
  double *acc = (double *)malloc(b), *jerk = (double *)malloc(b);
  double *op = (double *)malloc(b), *ov = (double *)malloc(b);
  double *oa = (double *)malloc(b), *oj = (double *)malloc(b);
  hf_forces(n, mass, pos, vel, eps2, acc, jerk);
  for (int s = 0; s < nsteps; s++) {
    memcpy(op, pos, b);
    memcpy(ov, vel, b);
    memcpy(oa, acc, b);
    memcpy(oj, jerk, b);
    for (int e = 0; e < 3 * n; e++) {
      pos[e] += vel[e] * dt + acc[e] * dt * dt / 2 + jerk[e] * dt * dt * dt / 6;
      vel[e] += acc[e] * dt + jerk[e] * dt * dt / 2;
    }
    hf_forces(n, mass, pos, vel, eps2, acc, jerk);
    for (int e = 0; e < 3 * n; e++) {
      vel[e] = ov[e] + (oa[e] + acc[e]) * dt / 2 + (oj[e] - jerk[e]) * dt * dt / 12;
      pos[e] = op[e] + (ov[e] + vel[e]) * dt / 2 + (oa[e] - acc[e]) * dt * dt / 12;
    }
  }
  if (acc_out) memcpy(acc_out, acc, b);
  if (jerk_out) memcpy(jerk_out, jerk, b);
  free(acc); free(jerk); free(op); free(ov); free(oa); free(oj);
}

/* ------------------------------------------------------------------ */
/* k nearest neighbours: save_neighbors (gpu.cc:534-558) applied to the  */
/* complete list of other particles, as get_densities_on_gpu            */
/* (gpu.cc:568-866) intends: r_sq = sum_k (pos[i][k] - pos[j][k])^2 in   */
/* component order, ascending; ties (which std::sort leaves unordered)  */
/* to the smaller index.  pos[n][3] are the (predicted) positions.       */
/* out_j[ni][k] (-1 past the last), out_d2[ni][k] (+inf there).          */
/* ------------------------------------------------------------------ */
void orc_knn(int n, const double *pos, int k, int ni, const int *slots,
             int *out_j, double *out_d2) {
  for (int q = 0; q < ni; q++) {
    const int i = slots[q];
    int *lj = out_j + (size_t)q * k;
    double *ld = out_d2 + (size_t)q * k;
    int cnt = 0;
    for (int j = 0; j < n; j++) {
      if (j == i) continue;
      double r_sq = 0;
      for (int c = 0; c < 3; c++) {
        double d = pos[3 * i + c] - pos[3 * j + c];
        r_sq += d * d;
      }
      if (cnt == k && !(r_sq < ld[k - 1] || (r_sq == ld[k - 1] && j < lj[k - 1])))
        continue;
      int p = cnt < k ? cnt : k - 1;
      while (p > 0 && (r_sq < ld[p - 1] || (r_sq == ld[p - 1] && j < lj[p - 1]))) {
        ld[p] = ld[p - 1];
        lj[p] = lj[p - 1];
        p--;
      }
      ld[p] = r_sq;
      lj[p] = j;
      if (cnt < k) cnt++;
    }
    for (int p = cnt; p < k; p++) {
      lj[p] = -1;
      ld[p] = INFINITY;
    }
  }
}

/* ------------------------------------------------------------------ */
/* smallN with unperturbed binaries: smallN.cc:906-1117 with           */
/* smallN_unpert.cc:44-88 (is_unperturbed_and_approaching), :233-360   */
/* (create_binary), :367-460 (time_to_radius, dt_perturbers), :567-774 */
/* (extend_or_end_binary) and smallN.cc:127-240 (forces between        */
/* top-level nodes resolved into their leaves), :380-470 (components   */
/* advanced on their Kepler orbits).  The binary tree is one level     */
/* deep, as smallN builds it.  Differences, stated:                    */
/*   - the two-body motion comes from a universal-variable Kepler      */
/*     propagator (Stumpff functions, Newton on the universal anomaly; */
/*     the published two-body solution), not smallN's kepler class;    */
/*   - the energy correction at the end of a partially unperturbed     */
/*     segment rescales the relative velocity to absorb the change of  */
/*     the tidal potential (the form smallN_unpert.cc:612-625 keeps    */
/*     under #if 0); the angular-momentum term is not applied;         */
/*   - the perturber of a candidate pair is searched among top-level   */
/*     nodes (smallN_unpert.cc:65-75 walks all leaves, whose           */
/*     positions under a binary node are relative to it).              */
/* pos/vel in place (all n bodies resolved at the end); returns steps. */
/* ------------------------------------------------------------------ */
#define SNU_NB 8 /* binaries per system at most */

typedef struct {
  int li, lj;           /* leader slot (holds the CM node) and companion */
  double mi, mj;        /* component masses */
  double r0[3], v0[3];  /* relative state x_j - x_i at time t0 */
  double t0, t_pred;    /* reference time, end of the unperturbed segment */
  double tidal;         /* tidal potential at the start of the segment */
  int full;             /* fully unperturbed: components frozen at r0, v0 */
} snu_bin;

/* Stumpff functions C(z) = (1 - cos sqrt z) / z and S(z) = (sqrt z -
 * sin sqrt z) / z^(3/2) (continued to z < 0 with cosh, sinh).  Near z = 0
 * their Taylor series (terms to z^6, below 1e-17 relative for |z| < 0.1);
 * elsewhere C through 2 sin^2(s/2), which does not cancel. */
static double snu_stumpff_c(double z) {
  if (z > 0.1) {
    double h = sin(0.5 * sqrt(z));
    return 2 * h * h / z;
  }
  if (z < -0.1) {
    double h = sinh(0.5 * sqrt(-z));
    return 2 * h * h / -z;
  }
  return 1.0 / 2 +
         z * (-1.0 / 24 +
              z * (1.0 / 720 +
                   z * (-1.0 / 40320 +
                        z * (1.0 / 3628800 + z * (-1.0 / 479001600 + z / 87178291200.0)))));
}
static double snu_stumpff_s(double z) {
  if (z > 0.1) {
    double s = sqrt(z);
    return (s - sin(s)) / (s * s * s);
  }
  if (z < -0.1) {
    double s = sqrt(-z);
    return (sinh(s) - s) / (s * s * s);
  }
  return 1.0 / 6 +
         z * (-1.0 / 120 +
              z * (1.0 / 5040 +
                   z * (-1.0 / 362880 +
                        z * (1.0 / 39916800 + z * (-1.0 / 6227020800.0 + z / 1307674368000.0)))));
}

/* Two-body relative motion over dt (mu = G M): universal variables.  The
 * universal anomaly x solves F(x) = (r0.v0/sqrt(mu)) x^2 C + (1 - alpha r0)
 * x^3 S + r0 x - sqrt(mu) dt = 0, and dF/dx is the separation r(x) > 0, so
 * F increases monotonically: the root is bracketed (doubling out from the
 * mean-motion guess) and found by Newton steps that fall back to bisection
 * when a step leaves the bracket or does not halve the previous one.  A
 * plain Newton iteration from the mean-motion guess diverges on eccentric
 * orbits near pericentre. */
static void snu_kepler(double mu, const double r0[3], const double v0[3], double dt, double r[3],
                       double v[3]) {
  double rn = sqrt(r0[0] * r0[0] + r0[1] * r0[1] + r0[2] * r0[2]);
  double v2 = v0[0] * v0[0] + v0[1] * v0[1] + v0[2] * v0[2];
  double rv = r0[0] * v0[0] + r0[1] * v0[1] + r0[2] * v0[2];
  double alpha = 2 / rn - v2 / mu, smu = sqrt(mu), c1 = rv / smu, c2 = 1 - alpha * rn;
  if (dt == 0) {
    for (int k = 0; k < 3; k++) r[k] = r0[k], v[k] = v0[k];
    return;
  }
#define SNU_F(xx) \
  (c1 * (xx) * (xx) * snu_stumpff_c(alpha * (xx) * (xx)) + \
   c2 * (xx) * (xx) * (xx) * snu_stumpff_s(alpha * (xx) * (xx)) + rn * (xx) - smu * dt)
  double x0 = alpha > 0 ? smu * dt * alpha : smu * dt / rn; /* same sign as dt */
  double lo, hi;
  if (dt > 0) {
    lo = 0, hi = x0;
    for (int k = 0; k < 200 && SNU_F(hi) < 0; k++) lo = hi, hi *= 2;
  } else {
    hi = 0, lo = x0;
    for (int k = 0; k < 200 && SNU_F(lo) > 0; k++) hi = lo, lo *= 2;
  }
#undef SNU_F
  double x = x0 > lo && x0 < hi ? x0 : 0.5 * (lo + hi);
  double step_old = hi - lo, step = step_old;
  for (int it = 0; it < 200; it++) {
    double z = alpha * x * x, C = snu_stumpff_c(z), S = snu_stumpff_s(z);
    double F = c1 * x * x * C + c2 * x * x * x * S + rn * x - smu * dt;
    double dF = c1 * x * (1 - z * S) + c2 * x * x * C + rn;
    if (F == 0) break;
    if (F < 0) lo = x; else hi = x;
    double xn = x - F / dF;
    if (!(xn > lo && xn < hi) || fabs(2 * F) > fabs(step_old * dF)) {
      step_old = step;
      step = 0.5 * (hi - lo);
      xn = lo + step;
    } else {
      step_old = step;
      step = F / dF;
    }
    if (fabs(xn - x) <= 1e-15 * fabs(xn)) {
      x = xn;
      break;
    }
    x = xn;
  }
  double z = alpha * x * x, C = snu_stumpff_c(z), S = snu_stumpff_s(z);
  double f = 1 - x * x * C / rn, g = dt - x * x * x * S / smu;
  for (int k = 0; k < 3; k++) r[k] = f * r0[k] + g * v0[k];
  double rr = sqrt(r[0] * r[0] + r[1] * r[1] + r[2] * r[2]);
  double fd = smu / (rr * rn) * (alpha * x * x * x * S - x), gd = 1 - x * x * C / rr;
  for (int k = 0; k < 3; k++) v[k] = fd * r0[k] + gd * v0[k];
}

/* The propagator, exported for the tests. */
void orc_kepler(double mu, const double *r0, const double *v0, double dt, double *r, double *v) {
  snu_kepler(mu, r0, v0, dt, r, v);
}

/* Time to the next pericentre and the period (inf unless bound) of the
 * relative orbit; returns 0 if the pair is not approaching its pericentre
 * (smallN_unpert.cc:252-266: mean anomaly >= 0). */
static int snu_peri(double mu, const double r[3], const double v[3], double *dt_peri,
                    double *period) {
  double rn = sqrt(r[0] * r[0] + r[1] * r[1] + r[2] * r[2]);
  double v2 = v[0] * v[0] + v[1] * v[1] + v[2] * v[2];
  double rv = r[0] * v[0] + r[1] * v[1] + r[2] * v[2];
  if (rv >= 0) return 0;
  double alpha = 2 / rn - v2 / mu;
  double h[3] = {r[1] * v[2] - r[2] * v[1], r[2] * v[0] - r[0] * v[2], r[0] * v[1] - r[1] * v[0]};
  double p = (h[0] * h[0] + h[1] * h[1] + h[2] * h[2]) / mu;
  double e = sqrt(fmax(0.0, 1 - p * alpha));
  *period = INFINITY;
  if (fabs(alpha) * rn < 1e-8 || e < 1e-12) { /* ~parabolic (Barker) or degenerate */
    double D = rv / sqrt(mu * p);
    *dt_peri = -0.5 * sqrt(p * p * p / mu) * (D + D * D * D / 3);
    if (alpha > 0) *period = 2 * M_PI / sqrt(mu * alpha * alpha * alpha);
    return *dt_peri > 0;
  }
  double M, n;
  if (alpha > 0) {
    double a = 1 / alpha;
    double cE = (1 - rn * alpha) / e, sE = rv / (e * sqrt(mu * a));
    double E = atan2(sE, cE);
    M = E - e * sin(E);
    n = sqrt(mu * alpha * alpha * alpha);
    *period = 2 * M_PI / n;
  } else {
    double sF = rv / (e * sqrt(-mu / alpha));
    double F = asinh(sF);
    M = e * sF - F;
    n = sqrt(-mu * alpha * alpha * alpha);
  }
  if (M >= 0) return 0;
  *dt_peri = -M / n;
  return 1;
}

typedef struct {
  int n, nb;
  int node[64];      /* node (leader slot) of each slot; -1: companion slot */
  snu_bin b[SNU_NB];
  int bin_of[64];    /* binary index of a leader slot, -1: single */
  double lx[64][3], lv[64][3]; /* predicted leaves of binary members */
} snu_tree;

/* Predicted leaves of binary q at time t from its CM's predicted state
 * (smallN.cc:380-470: Kepler motion; frozen when fully unperturbed). */
static void snu_resolve(snu_tree *T, const sn_body *b, int q, double t) {
  const snu_bin *B = &T->b[q];
  double r[3], v[3];
  if (B->full)
    for (int k = 0; k < 3; k++) r[k] = B->r0[k], v[k] = B->v0[k];
  else
    snu_kepler(B->mi + B->mj, B->r0, B->v0, t - B->t0, r, v);
  double M = B->mi + B->mj, fi = B->mj / M, fj = B->mi / M;
  const sn_body *C = &b[B->li];
  for (int k = 0; k < 3; k++) {
    T->lx[B->li][k] = C->pp[k] - fi * r[k];
    T->lv[B->li][k] = C->pv[k] - fi * v[k];
    T->lx[B->lj][k] = C->pp[k] + fj * r[k];
    T->lv[B->lj][k] = C->pv[k] + fj * v[k];
  }
}

/* Resolved forces on top-level nodes (smallN.cc:127-240, 316-363);
 * returns min step^2, and the node pair that set it. */
static double snu_forces(snu_tree *T, sn_body *b, int *imin, int *jmin) {
  int n = T->n;
  double lx[64][3], lv[64][3], lm[64];
  int ln[64];
  for (int s = 0; s < n; s++) {
    int leader = T->node[s] >= 0 ? T->node[s] : -1;
    if (leader < 0) { /* a companion: find its binary */
      for (int q = 0; q < T->nb; q++)
        if (T->b[q].lj == s) leader = T->b[q].li;
    }
    ln[s] = leader;
    int q = T->bin_of[leader];
    if (q >= 0) {
      lm[s] = s == T->b[q].li ? T->b[q].mi : T->b[q].mj;
      for (int k = 0; k < 3; k++) lx[s][k] = T->lx[s][k], lv[s][k] = T->lv[s][k];
    } else {
      lm[s] = b[s].m;
      for (int k = 0; k < 3; k++) lx[s][k] = b[s].pp[k], lv[s][k] = b[s].pv[k];
    }
  }
  for (int i = 0; i < n; i++)
    for (int k = 0; k < 3; k++) b[i].acc[k] = b[i].jerk[k] = 0;
  /* the leaves of each top-level node, in ascending order (the order the
     sums below take them in) */
  int mem[64][64], nm[64];
  for (int s = 0; s < n; s++) nm[s] = 0;
  for (int s = 0; s < n; s++)
    if (ln[s] >= 0) mem[ln[s]][nm[ln[s]]++] = s;
  double min_ts2 = ORC_INF;
  *imin = *jmin = -1;
  for (int A = 0; A < n; A++) {
    if (T->node[A] != A) continue; /* top-level nodes are their own leader */
    for (int Bn = A + 1; Bn < n; Bn++) {
      if (T->node[Bn] != Bn) continue;
      double F[3] = {0, 0, 0}, J[3] = {0, 0, 0}, mind2 = ORC_INF;
      for (int ia = 0; ia < nm[A]; ia++) {
        const int a = mem[A][ia];
        double fi[3] = {0, 0, 0}, ji[3] = {0, 0, 0};
        for (int ic = 0; ic < nm[Bn]; ic++) {
          const int c = mem[Bn][ic];
          double dx[3], dv[3];
          for (int k = 0; k < 3; k++) dx[k] = lx[c][k] - lx[a][k], dv[k] = lv[c][k] - lv[a][k];
          double d2 = dx[0] * dx[0] + dx[1] * dx[1] + dx[2] * dx[2];
          double d = sqrt(d2), d3 = d2 * d;
          double xv = dx[0] * dv[0] + dx[1] * dv[1] + dx[2] * dv[2];
          for (int k = 0; k < 3; k++) {
            fi[k] += lm[c] * dx[k] / d3;
            ji[k] += lm[c] * (dv[k] / d3 - 3 * dx[k] * xv / (d3 * d2));
          }
          if (d2 < mind2) mind2 = d2;
        }
        for (int k = 0; k < 3; k++) F[k] += lm[a] * fi[k], J[k] += lm[a] * ji[k];
      }
      double dvc[3];
      for (int k = 0; k < 3; k++) dvc[k] = b[Bn].pv[k] - b[A].pv[k];
      double vel2 = dvc[0] * dvc[0] + dvc[1] * dvc[1] + dvc[2] * dvc[2];
      double md = sqrt(mind2);
      double ts2 = fmin(0.5 * mind2 * md / (b[A].m + b[Bn].m), mind2 / fabs(vel2));
      for (int k = 0; k < 3; k++) {
        b[A].acc[k] += F[k] / b[A].m;
        b[A].jerk[k] += J[k] / b[A].m;
        b[Bn].acc[k] -= F[k] / b[Bn].m;
        b[Bn].jerk[k] -= J[k] / b[Bn].m;
      }
      if (ts2 < min_ts2) {
        min_ts2 = ts2;
        *imin = A;
        *jmin = Bn;
      }
    }
  }
  return min_ts2;
}

static double snu_dist(const double a[3], const double b[3]) {
  double d[3] = {a[0] - b[0], a[1] - b[1], a[2] - b[2]};
  return sqrt(d[0] * d[0] + d[1] * d[1] + d[2] * d[2]);
}

/* Tidal potential of the other top-level nodes on leaves (xi, xj) around
 * the CM xc (smallN_unpert.cc:17-40). */
static double snu_tidal(const snu_tree *T, const sn_body *b, int self, double mi, double mj,
                        const double xi[3], const double xj[3], const double xc[3],
                        int skip) {
  double phi = 0, mc = mi + mj;
  for (int k = 0; k < T->n; k++) {
    if (T->node[k] != k || k == self || k == skip) continue;
    phi += b[k].m * (-mi / snu_dist(xi, b[k].pos) - mj / snu_dist(xj, b[k].pos) +
                     mc / snu_dist(xc, b[k].pos));
  }
  return phi;
}

static double snu_time_to_radius(double dr, double vr, double ar) {
  if (dr <= 0) return 0;
  double dt = ORC_INF;
  if (vr < 0) dt = -dr / vr;
  if (ar < 0) dt = fmin(dt, sqrt(-2 * dr / ar));
  return dt;
}

long orc_smalln_unpert(int n, const double *mass, double *pos, double *vel, double eta,
                       int n_iter, double t_end, double dt_crit, double r2_crit, double gamma,
                       int allow_full, double *t_out, long max_steps, int *nbin_out) {
  if (n > 64) return -1;
  const double gamma2 = gamma * gamma, gamma_inv3 = pow(fmax(gamma2, 1e-120), -1.0 / 6);
  sn_body *b = (sn_body *)calloc((size_t)n, sizeof(sn_body));
  snu_tree T;
  memset(&T, 0, sizeof(T));
  T.n = n;
  for (int i = 0; i < n; i++) {
    T.node[i] = i;
    T.bin_of[i] = -1;
    b[i].m = mass[i];
    for (int k = 0; k < 3; k++) {
      b[i].pos[k] = b[i].pp[k] = pos[3 * i + k];
      b[i].vel[k] = b[i].pv[k] = vel[3 * i + k];
    }
  }
  int bim, bjm, nbin_made = 0;
  double t = 0;
  double dt = eta * sqrt(snu_forces(&T, b, &bim, &bjm));
  long steps = 0;
  while (t < t_end && (max_steps <= 0 || steps < max_steps)) {
    /* take_a_step (smallN.cc:553-682) with the unperturbed limit */
    double lim = ORC_INF;
    for (int q = 0; q < T.nb; q++) lim = fmin(lim, T.b[q].t_pred - t);
    int nit = n_iter;
    if (dt >= lim) {
      dt = lim;
      nit = 0;
    }
    /* predict_loworder_all (hdyn.h:192-201: with the stored old force) */
    double tn = t + dt, h = dt, h3 = h / 3, h2 = h / 2;
    for (int i = 0; i < n; i++) {
      if (T.node[i] != i) continue;
      for (int k = 0; k < 3; k++) {
        b[i].pp[k] = ((b[i].ojerk[k] * h3 + b[i].oacc[k]) * h2 + b[i].vel[k]) * h + b[i].pos[k];
        b[i].pv[k] = (b[i].ojerk[k] * h2 + b[i].oacc[k]) * h + b[i].vel[k];
      }
    }
    /* store_old_force */
    double oa[64][3], oj[64][3];
    for (int i = 0; i < n; i++)
      for (int k = 0; k < 3; k++) oa[i][k] = b[i].acc[k], oj[i][k] = b[i].jerk[k];
    for (int q = 0; q < T.nb; q++) snu_resolve(&T, b, q, tn);
    double new_dt = dt, end_dt = dt;
    for (int it = 0; it <= nit; it++) {
      double prev = new_dt;
      end_dt = eta * sqrt(snu_forces(&T, b, &bim, &bjm));
      if (it < nit) {
        new_dt = 0.5 * (dt + end_dt);
        new_dt = dt + 0.5 * (end_dt - dt) * (new_dt / prev);
        if (new_dt >= lim) {
          new_dt = lim;
          nit = 0;
        }
      }
      for (int i = 0; i < n; i++) {
        if (T.node[i] != i) continue;
        if (new_dt != prev) {
          double dt_off = new_dt - 0.5 * prev, theta = 0.5 * prev, tau = dt_off / theta;
          double inv_theta = 1 / theta, tau2 = tau * tau, tau3 = tau2 * tau;
          for (int k = 0; k < 3; k++) {
            double pa = b[i].acc[k], pj = b[i].jerk[k];
            b[i].acc[k] = 0.25 * (oa[i][k] * (2 - 3 * tau + tau3) + pa * (2 + 3 * tau - tau3) +
                                  oj[i][k] * theta * (1 - tau - tau2 + tau3) +
                                  pj * theta * (-1 - tau + tau2 + tau3));
            b[i].jerk[k] = 0.25 * (oa[i][k] * inv_theta * 3 * (-1 + tau2) +
                                   pa * inv_theta * 3 * (1 - tau2) +
                                   oj[i][k] * (-1 - 2 * tau + 3 * tau2) +
                                   pj * (-1 + 2 * tau + 3 * tau2));
          }
        }
        double nd2 = new_dt * new_dt;
        for (int k = 0; k < 3; k++) {
          b[i].pv[k] = b[i].vel[k] + new_dt * (b[i].acc[k] + oa[i][k]) / 2 -
                       nd2 * (b[i].jerk[k] - oj[i][k]) / 12;
          b[i].pp[k] = b[i].pos[k] + new_dt * (b[i].pv[k] + b[i].vel[k]) / 2 -
                       nd2 * (b[i].acc[k] - oa[i][k]) / 12;
        }
      }
      for (int q = 0; q < T.nb; q++) snu_resolve(&T, b, q, t + new_dt);
    }
    for (int i = 0; i < n; i++) {
      if (T.node[i] != i) continue;
      for (int k = 0; k < 3; k++) {
        b[i].pos[k] = b[i].pp[k];
        b[i].vel[k] = b[i].pv[k];
        b[i].oacc[k] = oa[i][k];
        b[i].ojerk[k] = oj[i][k];
      }
    }
    dt = end_dt;
    t = t + new_dt;
    steps++;

    /* tree changes (smallN.cc:1022-1060) */
    int changed = 0;
    /* is_unperturbed_and_approaching (smallN_unpert.cc:44-88) + create_binary */
    if (bim >= 0 && dt <= dt_crit && T.bin_of[bim] < 0 && T.bin_of[bjm] < 0 && T.nb < SNU_NB) {
      int i = bim, j = bjm;
      double dx[3], dvv[3];
      for (int k = 0; k < 3; k++) dx[k] = b[i].pos[k] - b[j].pos[k], dvv[k] = b[i].vel[k] - b[j].vel[k];
      double d2 = dx[0] * dx[0] + dx[1] * dx[1] + dx[2] * dx[2];
      double rv = dx[0] * dvv[0] + dx[1] * dvv[1] + dx[2] * dvv[2];
      if (d2 <= r2_crit && rv <= 0) {
        double M = b[i].m + b[j].m, cm[3], cmv[3];
        for (int k = 0; k < 3; k++) {
          cm[k] = (b[i].m * b[i].pos[k] + b[j].m * b[j].pos[k]) / M;
          cmv[k] = (b[i].m * b[i].vel[k] + b[j].m * b[j].vel[k]) / M;
        }
        double maxp = 0, nnd2 = 0;
        int kk = -1;
        for (int k2 = 0; k2 < n; k2++) {
          if (T.node[k2] != k2 || k2 == i || k2 == j) continue;
          double e2 = 0;
          for (int k = 0; k < 3; k++) e2 += (b[k2].pos[k] - cm[k]) * (b[k2].pos[k] - cm[k]);
          double p2 = b[k2].m * b[k2].m / e2;
          if (p2 > maxp) maxp = p2, nnd2 = e2, kk = k2;
        }
        int unp = 1;
        if (kk >= 0) {
          double g2 = 4 * pow(b[kk].m / M, 2) * pow(d2 / nnd2, 3);
          unp = g2 < gamma2;
        }
        double r[3], v[3], dtp, per;
        for (int k = 0; k < 3; k++) r[k] = b[j].pos[k] - b[i].pos[k], v[k] = b[j].vel[k] - b[i].vel[k];
        if (unp && snu_peri(M, r, v, &dtp, &per)) {
          snu_bin *B = &T.b[T.nb];
          B->li = i;
          B->lj = j;
          B->mi = b[i].m;
          B->mj = b[j].m;
          for (int k = 0; k < 3; k++) B->r0[k] = r[k], B->v0[k] = v[k];
          B->t0 = t;
          B->t_pred = 2 * (t + dtp) - t;
          B->full = 0;
          B->tidal = snu_tidal(&T, b, i, b[i].m, b[j].m, b[i].pos, b[j].pos, cm, j);
          b[i].m = M;
          for (int k = 0; k < 3; k++) {
            b[i].pos[k] = b[i].pp[k] = cm[k];
            b[i].vel[k] = b[i].pv[k] = cmv[k];
            b[i].oacc[k] = b[i].ojerk[k] = 0; /* a new node */
          }
          T.node[j] = -1;
          T.bin_of[i] = T.nb;
          T.nb++;
          nbin_made++;
          changed = 1;
        }
      }
    }
    /* extend_or_end_binary for segments that end now */
    for (int q = 0; q < T.nb; q++) {
      snu_bin *B = &T.b[q];
      if (B->t_pred > t) continue;
      int i = B->li, j = B->lj;
      double M = B->mi + B->mj, r[3], v[3];
      if (B->full)
        for (int k = 0; k < 3; k++) r[k] = B->r0[k], v[k] = B->v0[k];
      else
        snu_kepler(M, B->r0, B->v0, t - B->t0, r, v);
      double xi[3], xj[3];
      for (int k = 0; k < 3; k++) {
        xi[k] = b[i].pos[k] - B->mj / M * r[k];
        xj[k] = b[i].pos[k] + B->mi / M * r[k];
      }
      double tid = snu_tidal(&T, b, i, B->mi, B->mj, xi, xj, b[i].pos, j);
      if (!B->full) {
        double mu = B->mi * B->mj / M, v2 = v[0] * v[0] + v[1] * v[1] + v[2] * v[2];
        double fac = 1 - 2 * (tid - B->tidal) / (mu * v2);
        if (fac > 0)
          for (int k = 0; k < 3; k++) v[k] *= sqrt(fac);
      }
      /* extension by whole periods while no perturber can arrive
         (dt_perturbers, smallN_unpert.cc:402-460) */
      double rn = sqrt(r[0] * r[0] + r[1] * r[1] + r[2] * r[2]);
      double v2 = v[0] * v[0] + v[1] * v[1] + v[2] * v[2];
      double alpha = 2 / rn - v2 / M;
      double dtp = -1, period = ORC_INF;
      if (allow_full && alpha > 0) {
        double a = 1 / alpha;
        period = 2 * M_PI / sqrt(M * alpha * alpha * alpha);
        dtp = ORC_INF;
        for (int k2 = 0; k2 < n; k2++) {
          if (T.node[k2] != k2 || k2 == i) continue;
          double rp = gamma_inv3 * a * cbrt(2 * b[k2].m / M);
          double dp[3], dvl[3], da[3];
          for (int k = 0; k < 3; k++) {
            dp[k] = b[k2].pos[k] - b[i].pos[k];
            dvl[k] = b[k2].vel[k] - b[i].vel[k];
            da[k] = b[k2].acc[k] - b[i].acc[k];
          }
          double dr = sqrt(dp[0] * dp[0] + dp[1] * dp[1] + dp[2] * dp[2]);
          double vr = (dvl[0] * dp[0] + dvl[1] * dp[1] + dvl[2] * dp[2]) / dr;
          double ar = (da[0] * dp[0] + da[1] * dp[1] + da[2] * dp[2]) / dr;
          double tr = snu_time_to_radius(dr - rp, vr, ar);
          if (tr < dtp) dtp = tr;
          if (tr <= 0) break;
        }
        dtp *= 0.5;
      }
      if (dtp >= period) {
        B->t_pred += floor(dtp / period) * period;
        B->full = 1;
        B->tidal = tid;
        for (int k = 0; k < 3; k++) B->r0[k] = r[k], B->v0[k] = v[k];
        B->t0 = t;
        continue;
      }
      /* terminate: the components become top-level nodes again */
      b[j].m = B->mj;
      b[i].m = B->mi;
      double cx[3], cv[3];
      for (int k = 0; k < 3; k++) cx[k] = b[i].pos[k], cv[k] = b[i].vel[k];
      for (int k = 0; k < 3; k++) {
        b[i].pos[k] = b[i].pp[k] = cx[k] - B->mj / M * r[k];
        b[i].vel[k] = b[i].pv[k] = cv[k] - B->mj / M * v[k];
        b[j].pos[k] = b[j].pp[k] = cx[k] + B->mi / M * r[k];
        b[j].vel[k] = b[j].pv[k] = cv[k] + B->mi / M * v[k];
        b[i].oacc[k] = b[i].ojerk[k] = b[j].oacc[k] = b[j].ojerk[k] = 0;
      }
      T.node[j] = j;
      T.bin_of[i] = -1;
      T.b[q] = T.b[T.nb - 1];
      if (q < T.nb - 1) T.bin_of[T.b[q].li] = q;
      T.nb--;
      q--;
      changed = 1;
    }
    if (changed) {
      for (int i = 0; i < n; i++)
        for (int k = 0; k < 3; k++) b[i].pp[k] = b[i].pos[k], b[i].pv[k] = b[i].vel[k];
      for (int q = 0; q < T.nb; q++) snu_resolve(&T, b, q, t);
      dt = eta * sqrt(snu_forces(&T, b, &bim, &bjm));
    }
  }
  /* resolve the binaries left at the end into their components */
  for (int q = 0; q < T.nb; q++) {
    snu_bin *B = &T.b[q];
    int i = B->li, j = B->lj;
    double M = B->mi + B->mj, r[3], v[3];
    if (B->full)
      for (int k = 0; k < 3; k++) r[k] = B->r0[k], v[k] = B->v0[k];
    else
      snu_kepler(M, B->r0, B->v0, t - B->t0, r, v);
    for (int k = 0; k < 3; k++) {
      double cx = b[i].pos[k], cv = b[i].vel[k];
      b[i].pos[k] = cx - B->mj / M * r[k];
      b[i].vel[k] = cv - B->mj / M * v[k];
      b[j].pos[k] = cx + B->mi / M * r[k];
      b[j].vel[k] = cv + B->mi / M * v[k];
    }
  }
  for (int i = 0; i < n; i++)
    for (int k = 0; k < 3; k++) {
      pos[3 * i + k] = b[i].pos[k];
      vel[3 * i + k] = b[i].vel[k];
    }
  if (t_out) *t_out = t;
  if (nbin_out) *nbin_out = nbin_made;
  free(b);
  return steps;
}
