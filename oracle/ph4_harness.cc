// ph4_harness.cc -- TEST INFRASTRUCTURE ONLY.
//
// A small C-ABI driver around the UNMODIFIED ph4 objects (compiled from the
// reference sources by oracle/Makefile into oracle/_ref/libph4ref.so).  It
// drives jdata/idata/scheduler the way the ph4 worker does
// (src/amuse_ph4/interface.cc:82-119 initialize_code, :317-347
// commit_particles, :614-711 evolve_model), in CPU mode (no -DGPU), one
// process (-DNOMPI), with manage_encounters = 0 so that eps2 = 0 runs never
// enter resolve_encounter (jdata.cc:859-863).  It is used only to generate
// golden fixtures and to pin the C restatement in g6_oracle.c.
#include <cstdio>
#include <cstring>
#include <iostream>

#include "hdyn.h"
#include "idata.h"
#include "jdata.h"
#include "scheduler.h"
#include "stopcond.h"

extern "C" {

// Force only: the j-system is given already predicted; ph4's
// idata::get_partial_acc_and_jerk (idata.cc:147-237) runs on it unchanged.
// nn[i] is a j index, dnn[i] the nearest-neighbour distance.
int ph4ref_force(int nj, const double *mass, const double *jpos,
                 const double *jvel, double eps2, int ni, const double *ipos,
                 const double *ivel, double *acc, double *jerk, double *pot,
                 int *nn, double *dnn) {
  static jdata *jd = NULL;
  static idata *id = NULL;
  static int cap_j = 0;
  if (!jd) {
    jd = new jdata;
    std::streambuf *old = std::cout.rdbuf(NULL);
    id = new idata(NULL);  // prints a notice about the NULL jdata pointer
    std::cout.rdbuf(old);
  }
  if (nj > cap_j) {
    // Leaked on purpose: jdata::cleanup() expects arrays made by
    // add_particle(); this harness owns only what it touches.
    jd->mass = new real[nj];
    jd->pred_pos = new real[nj][3];
    jd->pred_vel = new real[nj][3];
    cap_j = nj;
  }
  jd->nj = nj;
  jd->eps2 = eps2;
  for (int j = 0; j < nj; j++) {
    jd->mass[j] = mass[j];
    for (int k = 0; k < 3; k++) {
      jd->pred_pos[j][k] = jpos[3 * j + k];
      jd->pred_vel[j][k] = jvel[3 * j + k];
    }
  }
  id->jdat = jd;
  id->set_ni(ni);
  id->ni = ni;
  for (int i = 0; i < ni; i++) {
    id->ilist[i] = i;
    for (int k = 0; k < 3; k++) {
      id->ipos[i][k] = ipos[3 * i + k];
      id->ivel[i][k] = ivel[3 * i + k];
    }
  }
  id->get_partial_acc_and_jerk();
  for (int i = 0; i < ni; i++) {
    pot[i] = id->ipot[i];
    nn[i] = id->inn[i];
    dnn[i] = id->idnn[i];
    for (int k = 0; k < 3; k++) {
      acc[3 * i + k] = id->iacc[i][k];
      jerk[3 * i + k] = id->ijerk[i][k];
    }
  }
  return 0;
}

// Corrector + Aarseth step on a list, through ph4's idata::correct
// (idata.cc:399-514).  ipos/ivel: predicted in, corrected out.
int ph4ref_correct(int ni, double tnext, double eta, double *itime,
                   double *itimestep, double *ipos, double *ivel,
                   const double *old_acc, const double *old_jerk,
                   const double *iacc, const double *ijerk) {
  static jdata *jd = NULL;
  static idata *id = NULL;
  if (!jd) {
    jd = new jdata;
    std::streambuf *old = std::cout.rdbuf(NULL);
    id = new idata(NULL);
    std::cout.rdbuf(old);
  }
  jd->eta = eta;
  id->jdat = jd;
  id->set_ni(ni);
  id->ni = ni;
  for (int i = 0; i < ni; i++) {
    id->itime[i] = itime[i];
    id->itimestep[i] = itimestep[i];
    for (int k = 0; k < 3; k++) {
      id->ipos[i][k] = ipos[3 * i + k];
      id->ivel[i][k] = ivel[3 * i + k];
      id->old_acc[i][k] = old_acc[3 * i + k];
      id->old_jerk[i][k] = old_jerk[3 * i + k];
      id->iacc[i][k] = iacc[3 * i + k];
      id->ijerk[i][k] = ijerk[3 * i + k];
    }
  }
  id->correct(tnext);
  for (int i = 0; i < ni; i++) {
    itime[i] = id->itime[i];
    itimestep[i] = id->itimestep[i];
    for (int k = 0; k < 3; k++) {
      ipos[3 * i + k] = id->ipos[i][k];
      ivel[3 * i + k] = id->ivel[i][k];
    }
  }
  return 0;
}

// Full run: initialize_code + add_particle + commit_particles +
// evolve_model(t_end), CPU mode.  State is returned in j order (the order
// particles were added).  stats: E0, E1, total_steps, system_time,
// block_steps.
int ph4ref_run(int n, const double *mass, const int *ids, const double *pos,
               const double *vel, double eps2, double eta, double t_end,
               double *pos_out, double *vel_out, double *acc_out,
               double *jerk_out, double *pot_out, double *time_out,
               double *step_out, double *stats) {
  std::streambuf *old = std::cout.rdbuf(NULL);  // ph4 is chatty on cout
  jdata *jd = new jdata;
  jd->setup_gpu();
  jd->system_time = 0;
  jd->sync_time = 0;
  jd->set_manage_encounters(0);
  jd->eps2 = eps2;
  jd->eta = eta;
  for (int j = 0; j < n; j++) {
    vec p(pos[3 * j], pos[3 * j + 1], pos[3 * j + 2]);
    vec v(vel[3 * j], vel[3 * j + 1], vel[3 * j + 2]);
    jd->add_particle(mass[j], 0.0, p, v, ids[j]);
  }
  // commit_particles (interface.cc:317-347); sync_times() is a no-op here.
  jd->initialize_arrays();
  idata *id = new idata(jd);
  jd->force_initial_timestep(0.0625, 0.03125, 8.0);
  scheduler *s = new scheduler(jd);
  double e0 = jd->get_energy();
  // evolve_model (interface.cc:614-711), no force_sync.
  while (jd->system_time < t_end)
    if (jd->advance_and_check_encounter()) break;
  double e1 = jd->get_energy();
  std::cout.rdbuf(old);
  for (int j = 0; j < n; j++) {
    pot_out[j] = jd->pot[j];
    time_out[j] = jd->time[j];
    step_out[j] = jd->timestep[j];
    for (int k = 0; k < 3; k++) {
      pos_out[3 * j + k] = jd->pos[j][k];
      vel_out[3 * j + k] = jd->vel[j][k];
      acc_out[3 * j + k] = jd->acc[j][k];
      jerk_out[3 * j + k] = jd->jerk[j][k];
    }
  }
  stats[0] = e0;
  stats[1] = e1;
  stats[2] = jd->total_steps;
  stats[3] = jd->system_time;
  stats[4] = jd->block_steps;
  (void)s;
  (void)id;
  // jdata/idata/scheduler are leaked: ph4's cleanup paths assume the
  // worker process exits afterwards.
  return 0;
}

// Full run with the COLLISION_DETECTION stopping condition enabled, as the
// ph4 worker sets it up (interface.cc:106 set_support_for_condition, :629
// reset_stopping_conditions, :667-668 the evolve loop): particles carry a
// radius; after every block idata::check_encounters (idata.cc:620-700) runs
// and jdata::advance_and_check_encounter (jdata.cc:797-850) stops the run
// when the collision pair is approaching.  enc_out: close1, close2, coll1,
// coll2 (ids from the last block, -1 none), stopping condition set (0/1),
// its two particle ids, rmin.  stats as ph4ref_run.  stop_on_close also ends
// the loop after the first block that reports a close pair (jd->close1, the
// pair ph4 hands to resolve_encounter when it manages encounters itself).
int ph4ref_run_coll(int n, const double *mass, const double *radius, const int *ids,
                    const double *pos, const double *vel, double eps2, double eta,
                    double t_end, int stop_on_close, double *pos_out, double *vel_out,
                    double *time_out, double *step_out, double *stats, double *enc_out) {
  std::streambuf *old = std::cout.rdbuf(NULL);
  set_support_for_condition(COLLISION_DETECTION);
  enable_stopping_condition(COLLISION_DETECTION);
  reset_stopping_conditions();
  jdata *jd = new jdata;
  jd->setup_gpu();
  jd->system_time = 0;
  jd->sync_time = 0;
  jd->set_manage_encounters(0);
  jd->eps2 = eps2;
  jd->eta = eta;
  for (int j = 0; j < n; j++) {
    vec p(pos[3 * j], pos[3 * j + 1], pos[3 * j + 2]);
    vec v(vel[3 * j], vel[3 * j + 1], vel[3 * j + 2]);
    jd->add_particle(mass[j], radius[j], p, v, ids[j]);
  }
  jd->initialize_arrays();
  idata *id = new idata(jd);
  jd->force_initial_timestep(0.0625, 0.03125, 8.0);
  scheduler *s = new scheduler(jd);
  double e0 = jd->get_energy();
  jd->coll1 = jd->coll2 = -1;
  jd->close1 = jd->close2 = -1;
  while (jd->system_time < t_end) {
    if (jd->advance_and_check_encounter()) break;
    if (stop_on_close && jd->close1 >= 0) break;
  }
  int set = 0, p0 = -1, p1 = -1;
  is_stopping_condition_set(COLLISION_DETECTION, &set);
  if (set) {
    get_stopping_condition_particle_index(0, 0, &p0);
    get_stopping_condition_particle_index(0, 1, &p1);
  }
  enc_out[0] = jd->close1;
  enc_out[1] = jd->close2;
  enc_out[2] = jd->coll1;
  enc_out[3] = jd->coll2;
  enc_out[4] = set;
  enc_out[5] = p0;
  enc_out[6] = p1;
  enc_out[7] = jd->rmin;
  double e1 = jd->get_energy();
  disable_stopping_condition(COLLISION_DETECTION);
  reset_stopping_conditions();
  std::cout.rdbuf(old);
  for (int j = 0; j < n; j++) {
    time_out[j] = jd->time[j];
    step_out[j] = jd->timestep[j];
    for (int k = 0; k < 3; k++) {
      pos_out[3 * j + k] = jd->pos[j][k];
      vel_out[3 * j + k] = jd->vel[j][k];
    }
  }
  stats[0] = e0;
  stats[1] = e1;
  stats[2] = jd->total_steps;
  stats[3] = jd->system_time;
  stats[4] = jd->block_steps;
  (void)s;
  (void)id;
  return 0;
}

// smallN (src/amuse_ph4/src/smallN.cc smallN_evolve) on one system, set up
// as the smallN worker does (src/amuse_smalln/interface.cc:61-85,
// src/amuse_smalln/src/smallN_interface.cc:8-36), with dt_crit given
// (0 disables the unperturbed-binary tree).  State in place.
int ph4ref_smalln(int n, const double *mass, double *pos, double *vel, double eta,
                  double t_end, double dt_crit, double *t_out) {
  std::streambuf *old = std::cout.rdbuf(NULL);
  hdyn *b = new hdyn;
  b->set_eta(eta);
  b->set_gamma(1e-6);
  b->set_system_time(0.0);
  b->set_allow_full_unperturbed(1);
  b->set_cm_index(100000);
  b->set_dt_crit(dt_crit);
  b->set_n_iter(2);
  hdyn *prev = NULL;
  for (int i = 0; i < n; i++) {
    hdyn *bn = new hdyn;
    bn->set_mass(mass[i]);
    bn->set_radius(0.0);
    bn->set_pos(vec(pos[3 * i], pos[3 * i + 1], pos[3 * i + 2]));
    bn->set_vel(vec(vel[3 * i], vel[3 * i + 1], vel[3 * i + 2]));
    bn->set_index(i + 1);
    bn->set_parent(b);
    if (!prev) {
      b->set_oldest_daughter(bn);
    } else {
      bn->set_older_sister(prev);
      prev->set_younger_sister(bn);
    }
    prev = bn;
  }
  smallN_evolve(b, t_end, _INFINITY_, _INFINITY_, _INFINITY_, 0, "");
  // Report every leaf by its index; the leaves of a binary node hold
  // positions relative to it (smallN.cc:427-436), so add the node's.
  // Returns the number of binary nodes left at the end.
  int nbin = 0;
  for_all_daughters(hdyn, b, bi) {
    hdyn *od = bi->get_oldest_daughter();
    if (od) {
      nbin++;
      for (hdyn *leaf = od; leaf; leaf = leaf->get_younger_sister()) {
        vec p = bi->get_pos() + leaf->get_pos(), v = bi->get_vel() + leaf->get_vel();
        const int i = leaf->get_index() - 1;
        for (int k = 0; k < 3; k++) {
          pos[3 * i + k] = p[k];
          vel[3 * i + k] = v[k];
        }
      }
      continue;
    }
    vec p = bi->get_pos(), v = bi->get_vel();
    const int i = bi->get_index() - 1;
    for (int k = 0; k < 3; k++) {
      pos[3 * i + k] = p[k];
      vel[3 * i + k] = v[k];
    }
  }
  *t_out = b->get_system_time();
  std::cout.rdbuf(old);
  return nbin;
}

// smallN's structure analysis (src/amuse_ph4/src/analyze.cc check_structure,
// get_tree) on a flat system of n leaves: returns over (0-3; 2 is the
// quasi-stable termination, which depends on the calls before this one) and
// writes the decomposed tree as text, a binary as "(first,second)" of
// 0-based body indices in daughter order, top-level nodes separated by
// spaces.
static int describe_ref(hdyn *b, char *s, int cap) {
  hdyn *od = b->get_oldest_daughter();
  if (!od) return snprintf(s, cap > 0 ? cap : 0, "%d", b->get_index() - 1);
  int w = snprintf(s, cap > 0 ? cap : 0, "(");
  w += describe_ref(od, s + w, cap > w ? cap - w : 0);
  w += snprintf(s + w, cap > w ? cap - w : 0, ",");
  w += describe_ref(od->get_younger_sister(), s + w, cap > w ? cap - w : 0);
  w += snprintf(s + w, cap > w ? cap - w : 0, ")");
  return w;
}

int ph4ref_check_structure(int n, const double *mass, const double *pos, const double *vel,
                           char *summary, int cap) {
  std::streambuf *old = std::cout.rdbuf(NULL);
  hdyn *b = new hdyn;
  b->set_system_time(0.0);
  hdyn *prev = NULL;
  for (int i = 0; i < n; i++) {
    hdyn *bn = new hdyn;
    bn->set_mass(mass[i]);
    bn->set_pos(vec(pos[3 * i], pos[3 * i + 1], pos[3 * i + 2]));
    bn->set_vel(vec(vel[3 * i], vel[3 * i + 1], vel[3 * i + 2]));
    bn->set_index(i + 1);
    bn->set_parent(b);
    if (!prev) {
      b->set_oldest_daughter(bn);
    } else {
      bn->set_older_sister(prev);
      prev->set_younger_sister(bn);
    }
    prev = bn;
  }
  const int over = check_structure(b, _INFINITY_, 0);
  hdyn *t = get_tree(b);
  int w = 0;
  if (cap > 0) summary[0] = 0;
  for_all_daughters(hdyn, t, bi) {
    if (w > 0) w += snprintf(summary + w, cap > w ? cap - w : 0, " ");
    w += describe_ref(bi, summary + w, cap > w ? cap - w : 0);
  }
  rmtree(t);
  rmtree(b);
  std::cout.rdbuf(old);
  return over;
}

}  // extern "C"
