/*
 * g6.h -- public C ABI of libsapporo.so (GB300 / sm_103a build).
 *
 * Part 1 is the GRAPE-6 API exactly as AMUSE's callers bind it: the 16
 * trailing-underscore, all-pointer symbols of lib/sapporo_light/g6lib.h:5-51
 * (sapporoG6lib.cpp:5-78), used by phiGRAPE through gfortran name mangling
 * and by ph4 through its by-value wrappers (src/amuse_ph4/src/grape.h).
 * Part 2 is the by-value set of ph4's grape.h / lib/g6lib/g6lib.h:58-128,
 * exported as WEAK symbols (ph4 defines its own strong copies in grape.cc).
 * Part 3 is the extension API (g6x_*), which has no GRAPE-6 counterpart:
 * device-resident state, the FP64 corrector / block-step driver, precision
 * selection and statistics.
 *
 * Conventions (shared by all parts): arrays `double x[][3]` are row-major
 * [n][3] (= Fortran x(3,n)); 0 means success and a negative value an error
 * (the reference exits the process instead, sapporo.cpp:26-27,76-79,255-257);
 * one context per process; not re-entrant.
 */
#ifndef G6_GB300_H
#define G6_GB300_H

#ifdef __cplusplus
extern "C" {
#endif

/* Error codes. */
#define G6_OK 0
#define G6_ERR_NOT_OPEN (-1)   /* g6_open not called / failed */
#define G6_ERR_ARG (-2)        /* bad argument (address, ni > npipes, ...) */
#define G6_ERR_CUDA (-3)       /* CUDA runtime error */
#define G6_ERR_NOMEM (-4)      /* device or pinned allocation failed */
#define G6_ERR_DEVICE (-5)     /* no such CUDA device */
#define G6_ERR_KERNEL (-6)     /* a kernel reported a timeout (error word) */
#define G6_ERR_STATE (-7)      /* call out of order (e.g. lasthalf w/o firsthalf) */

/* ---------------- Part 1: GRAPE-6 ABI (pointer arguments) ---------------- */

/* sapporo.cpp:19-41: select CUDA device *id, allocate the j-store. */
int g6_open_(int *id);
/* sapporo.cpp:43-56: release device memory. */
int g6_close_(int *id);
/* sapporo.cpp:64-66: max i-particles per g6calc call (<= 16384 by
   default, phiGRAPE's NGP bound; env G6_NPIPES overrides). */
int g6_npipes_(void);
/* sapporoG6lib.cpp:10-11: accepted and ignored. */
int g6_set_tunit_(double *);
int g6_set_xunit_(double *);
/* sapporo.cpp:58-62: time to which j-particles are predicted. */
int g6_set_ti_(int *id, double *ti);
/* sapporo.cpp:68-112: stage one j record for slot *address; index = id used
   for self-exclusion and returned as neighbour; a2 = acc/2, j6 = jerk/6,
   k18 (snap/18) is ignored as in the reference. */
int g6_set_j_particle_(int *cluster_id, int *address, int *index, double *tj, double *dtj,
                       double *mass, double k18[3], double j6[3], double a2[3], double v[3],
                       double x[3]);
/* sapporo.cpp:114-152: start the force on ni i-particles from j slots
   [0, nj) predicted to the last set_ti (pending j updates applied first).
   aold/j6old/phiold are ignored as in the reference; h2 is the neighbour
   radius^2 (used by the neighbour-list API).  Asynchronous. */
void g6calc_firsthalf_(int *cluster_id, int *nj, int *ni, int index[], double xi[][3],
                       double vi[][3], double aold[][3], double j6old[][3], double phiold[],
                       double *eps2, double h2[]);
/* sapporo.cpp:154-182: wait and OVERWRITE acc, jerk, pot of the ni
   i-particles of the preceding firsthalf. */
int g6calc_lasthalf_(int *cluster_id, int *nj, int *ni, int index[], double xi[][3],
                     double vi[][3], double *eps2, double h2[], double acc[][3],
                     double jerk[][3], double pot[]);
/* sapporo.cpp:185-232: as lasthalf, plus nnbindex[i] = index (id) of the
   nearest j (self excluded), -1 if none. */
int g6calc_lasthalf2_(int *cluster_id, int *nj, int *ni, int index[], double xi[][3],
                      double vi[][3], double *eps2, double h2[], double acc[][3],
                      double jerk[][3], double pot[], int *inn);
/* sapporoG6lib.cpp:58-61: no-ops returning 0. */
int g6_initialize_jp_buffer_(int *cluster_id, int *buf_size);
int g6_flush_jp_buffer_(int *cluster_id);
int g6_reset_(int *cluster_id);
int g6_reset_fofpga_(int *cluster_id);
/* sapporo.cpp:234-246: fetch the neighbour lists (r^2 <= h2[i], self
   excluded) of the last force call; returns 1 if any list overflowed its
   G6_NGB_MAX entries, 0 otherwise. */
int g6_read_neighbour_list_(int *cluster_id);
/* sapporo.cpp:248-272: copy the sorted neighbour ids of i-particle *ipipe
   into neighbour_list (at most *maxlength), set *n_neighbours; returns 1
   on overflow. */
int g6_get_neighbour_list_(int *cluster_id, int *ipipe, int *maxlength, int *n_neighbours,
                           int neighbour_list[]);

#define G6_NGB_MAX 256 /* per-i neighbour capacity (sapporo_defs.h NGB_PP) */

/* ---------------- Part 2: by-value forms (weak) ---------------------------- */

int g6_open(int id);
int g6_close(int id);
int g6_npipes(void);
int g6_set_tunit(double t);
int g6_set_xunit(double x);
int g6_set_ti(int id, double ti);
int g6_set_j_particle(int cluster_id, int address, int index, double tj, double dtj, double mass,
                      double k18[3], double j6[3], double a2[3], double v[3], double x[3]);
void g6calc_firsthalf(int cluster_id, int nj, int ni, int index[], double xi[][3],
                      double vi[][3], double aold[][3], double j6old[][3], double phiold[],
                      double eps2, double h2[]);
int g6calc_lasthalf(int cluster_id, int nj, int ni, int index[], double xi[][3], double vi[][3],
                    double eps2, double h2[], double acc[][3], double jerk[][3], double pot[]);
int g6calc_lasthalf2(int cluster_id, int nj, int ni, int index[], double xi[][3],
                     double vi[][3], double eps2, double h2[], double acc[][3],
                     double jerk[][3], double pot[], int inn[]);
int g6_initialize_jp_buffer(int cluster_id, int buf_size);
int g6_flush_jp_buffer(int cluster_id);
int g6_reset(int cluster_id);
int g6_reset_fofpga(int cluster_id);
int g6_read_neighbour_list(int cluster_id);
int g6_get_neighbour_list(int cluster_id, int ipipe, int maxlength, int *n_neighbours,
                          int neighbour_list[]);

/* ---------------- Part 3: extension API (no GRAPE-6 counterpart) ---------- */

#define G6X_SPLIT 0 /* double-single positions, FP32 pair arithmetic (default) */
#define G6X_FP64 1  /* plain FP64 pair arithmetic */

/* Precision of subsequent force evaluations. */
int g6x_set_precision(int prec);
int g6x_get_precision(void);
/* Split precision: every force call ends with a refinement pass.
   - Nearest neighbour: the FP32 argmin is kept only where a proven FP32
     error bound separates it from every other j; otherwise the candidates
     within the bound are ranked by ph4's FP64 r^2 (first slot on equal
     values), so nn is ph4's nearest neighbour.
   - Condition number: i-particles whose kappa = sum m/(r^2+eps^2) / |acc|
     exceeds the limit (default 48, env G6_KAPPA; 0 disables both passes)
     get acc and pot recomputed in FP64 from the same records (the jerk
     keeps its split value).
   - Dominant term: i-particles below that limit whose largest single term
     m/(r^2+eps^2) may exceed |acc| get acc and pot recomputed from the
     same FP32 pair terms with compensated sums, the terms above 0.02 |acc|
     in FP64.
   g6x_refine_stats reports the last call's queue: out = {particles queued,
   of which for kappa, largest queue that overflowed the 16384 entries since
   the last read (then nothing was refined in that call), of which for a
   dominant term}. */
int g6x_set_refine(double kappa);
int g6x_refine_stats(int out[4]);
/* Test hook for the force kernel's bounded waits: with on != 0, the next
   force call's first CTA waits for its first j-tile on a barrier that
   nothing arrives on, with a 20 ms limit instead of 2 s.  The wait expires,
   the CTA raises its abort flag, drains the copies it issued and sets the
   error word, so that call returns G6_ERR_KERNEL (no trap, no unbounded
   spin); the hook then clears itself and later calls run normally. */
int g6x_test_wait_expiry(int on);
/* Change the i-chunk bound reported by g6_npipes (1 .. 1<<20). */
int g6x_set_npipes(int npipes);
/* Last error message ("" if none). */
const char *g6x_last_error(void);

/* Bulk-load n particles into slots [0, n) from host arrays (replaces n
   g6_set_j_particle calls); acc/jerk unscaled.  Resets the device run. */
int g6x_load(int n, const int *ids, const double *mass, const double (*x)[3],
             const double (*v)[3], const double (*acc)[3], const double (*jerk)[3],
             const double *t, const double *dt);
/* Read the device j-state of slots [0, n) back to host arrays (any may be
   NULL). */
int g6x_read(int n, double (*x)[3], double (*v)[3], double (*acc)[3], double (*jerk)[3],
             double *pot, double *t, double *dt, int *nn);

/* Blocking force on ni explicit i-particles (host arrays) against slots
   [0, nj) predicted to ti.  self_slot[i] (or NULL) is the slot to exclude;
   nn[i] is a j SLOT (-1 none); nn_r2[i] = its squared distance r^2 (FP64
   value rounded to FP32); either may be NULL.  Any ni (no npipes bound). */
int g6x_force(double ti, double eps2, int nj, int ni, const double (*xi)[3],
              const double (*vi)[3], const int *self_slot, double (*acc)[3],
              double (*jerk)[3], double *pot, int *nn, float *nn_r2);
/* Same with all arrays in device memory (no host copies, asynchronous on the
   library stream unless sync != 0). */
int g6x_force_dev(double ti, double eps2, int nj, int ni, const double *d_xi,
                  const double *d_vi, const int *d_self_slot, double *d_acc, double *d_jerk,
                  double *d_pot, int *d_nn, float *d_nn_r2, int sync);
/* As g6x_force_dev, but the call allocates no device memory: no reference
   counterpart (the GRAPE-6 library has nothing like it).  For callers that
   may not allocate during the call -- device memory owned and budgeted by a
   host framework, or step loops that cannot absorb cudaMalloc's implicit
   synchronisation.  The split-j partial sums use a fixed 16 MiB array that
   every GPU loading the library holds until exit; g6_open takes it and looks
   up its device address (after a device reset, g6_close and g6_open again),
   and allocates the fixed refinement queue the call also uses.  A call
   whose launch shape needs more scratch, or whose nj exceeds the j-store
   already allocated, or with more staged j updates than the update buffer
   holds, returns G6_ERR_ARG instead of allocating.  All calls share the
   array: calls that overlap on the GPU race and must not be issued. */
int g6x_force_dev_noalloc(double ti, double eps2, int nj, int ni, const double *d_xi,
                          const double *d_vi, const int *d_self_slot, double *d_acc,
                          double *d_jerk, double *d_pot, int *d_nn, int sync);
/* Force on the device-resident slots d_ilist[0..ni) predicted to ti (i data
   taken from the predicted j records; self excluded by slot). */
int g6x_force_slots(double ti, double eps2, int nj, int ni, const int *d_ilist, double *d_acc,
                    double *d_jerk, double *d_pot, int *d_nn, int sync);

/* Device-resident ph4-style integration of the loaded particles:
   g6x_run_init  -- forces at t = 0 and initial steps (jdata.cc:503-580),
   g6x_run       -- block steps (predict all j, force on the block, FP64
                    corrector + Aarseth step) until system time >= t_end
                    or, if *blocks > 0 on entry, after *blocks block steps;
                    *blocks returns the block steps taken,
   g6x_energy    -- kinetic and potential energy at the system time,
   g6x_step_all  -- one shared step of all particles to tnext (the
                    benchmark step: predict + force on all + correct). */
int g6x_run_init(double eps2, double eta);
int g6x_run(double t_end, long long *blocks, double *particle_steps);
/* Host-side account of the last g6x_run: out = {block steps, wall ms, ms
   spent waiting in the per-block synchronisation, particle steps}. */
int g6x_run_stats(double out[4]);
/* Encounter check in g6x_run (replaces ph4's idata::check_encounters,
   src/amuse_ph4/src/idata.cc:620-700, and the COLLISION_DETECTION stopping
   condition of jdata::advance_and_check_encounter, jdata.cc:797-850).
   With G6_ENC_CHECK the force of every block also finds each particle's
   nearest neighbour; over the block, the particle with the largest
   rmin/dnn gives the close pair and the one with the largest
   (R_i + R_nn)/dnn the collision pair, each when that ratio is >= 1 (dnn in
   FP64 from both particles predicted to the block time; ties go to the
   smaller slot, where ph4 takes the first in its scheduler's list).
   G6_ENC_STOP_COLLISION ends g6x_run after a block whose collision pair is
   approaching (vr < 0.001 r v on the corrected state), as ph4's worker
   ends evolve_model; G6_ENC_STOP_CLOSE after any block with a close pair
   (for a caller that resolves encounters itself).  Stop bits imply CHECK.
   rmin <= 0 selects ph4's default 2/n (jdata.cc:426).  Radii are set by
   slot (default 0).  g6x_encounter reports the last checked block: ids =
   {close1, close2, coll1, coll2} (particle ids, -1 none), out = {stop bits
   (1 collision, 2 close), block time, rmax_close, rmax_coll}. */
#define G6_ENC_CHECK 1
#define G6_ENC_STOP_COLLISION 2
#define G6_ENC_STOP_CLOSE 4
int g6x_set_encounters(int mode, double rmin);
int g6x_set_radius(int n, const double *radius);
int g6x_encounter(int ids[4], double out[4]);
/* The k (1..32) nearest neighbours of each listed slot among the j-slots
   [0, nj), positions predicted to t with ph4's predictor: the lists that
   ph4's get_densities_on_gpu (src/amuse_ph4/src/gpu.cc:568-866) builds
   from GRAPE neighbour lists and reduces with save_neighbors
   (gpu.cc:534-558) to the knn nearest, sorted by squared distance.  Exact
   in FP64 (an FP32 pre-filter with a proven error slack rejects only
   particles farther than the current k-th); ties go to the smaller slot.
   Host arrays: slots[ni]; out ids[ni][k] (particle ids, -1 when fewer than
   k others exist), d2[ni][k] squared distances (+inf there).  Blocking. */
int g6x_knn(int k, int nj, double t, int ni, const int *slots, int *ids, double *d2);
int g6x_energy(double *kinetic, double *potential);
int g6x_step_all(double tnext);
/* FP64 corrector + Aarseth step (idata.cc:399-514) applied on the device to
   the listed slots with the given new acc/jerk (host arrays, [ni][3]);
   positions/velocities are predicted from the stored state to tnext first
   (idata.cc:346-365).  Blocking. */
int g6x_correct(int ni, const int *slots, double tnext, double eta, const double (*acc)[3],
                const double (*jerk)[3]);
double g6x_system_time(void);

/* Statistics of the last force call: out[0] predictor ms, out[1] force ms
   (incl. second pass), out[2] pair interactions, out[3] JL, out[4] nsplit,
   out[5] grid.x, out[6] predictor bytes, out[7] nj.  Timing is measured
   with CUDA events only while g6x_timing(1) is set. */
int g6x_timing(int on);
int g6x_stats(double out[8]);
/* The same, n values at most (up to 10): out[8] the force kernel's ms (with
   its split-j merge), out[9] the refinement pass's ms (out[1] = out[8] +
   out[9] for split-precision calls). */
int g6x_stats_n(double *out, int n);
/* Launch shape override for the following force calls: jl j-lanes per
   i-particle (a power of two up to 256) and nsplit j-ranges, each 0 for the
   cost model's choice (the default).  For tuning and measurement; results do
   not depend on the shape beyond the FP32 summation order. */
int g6x_set_shape(int jl, int nsplit);

/* Structure of one few-body system (n <= 64 bodies, G = 1, positions and
   velocities in any common frame) and whether its interaction is over, as
   smallN's check_structure decides it (src/amuse_ph4/src/analyze.cc:
   866-1070) for the multiples hand-off: bodies are paired into binaries by
   relative energy (only lightly perturbed pairs), escapers and stability
   are flagged, and the interaction is over when every top-level node is
   escaping and stable.  Host code; no device is needed.
   top_of[n] (optional) receives, per body, the smallest body index of its
   top-level node; summary (optional) the structure as text, a binary as
   "(first,second)" of body indices, top-level nodes separated by spaces.
   Returns bit 0 = over, bit 1 = a multiple above a binary was judged by the
   published Mardling-Aarseth criterion (smallN consults Mardling's nstab
   there, which this library does not restate), bit 2 = every top-level node
   escaping, stable or not (smallN's quasi-stable ending needs it together
   with a history of the grouping, which the caller keeps), or G6_ERR_ARG. */
int g6x_check_structure(int n, const double *mass, const double *pos, const double *vel,
                        int *top_of, char *summary, int summary_cap);

/* g6x_check_structure for nsys systems of n_per_sys[s] bodies stored back to
   back, on nthreads host threads (<= 0: one per online core).  flags[s]
   receives system s's return value; top_of (optional) the per-body values,
   indices local to each system; top_rank (optional) per body the position
   of its top-level node in the tree's order (two checks with equal top_rank
   have the same top-level grouping in the same order: smallN's "state");
   summary (optional) nsys strings of summary_cap bytes each.  Returns 0, or
   the first system's error. */
int g6x_check_structure_batch(int nsys, const int *n_per_sys, const double *mass,
                              const double *pos, const double *vel, int *flags, int *top_of,
                              int *top_rank, char *summary, int summary_cap, int nthreads);

/* Batched few-body systems (the encounters AMUSE's multiples module hands
   to smallN): nsys independent systems of n_per_sys[s] bodies (2..64),
   stored back to back in mass/pos/vel, each integrated to t_end[s] with
   smallN's time-symmetrised shared-step Hermite scheme and Kepler step
   criterion (src/amuse_ph4/src/smallN.cc:85-116,318-363,487-682) without
   the unperturbed-binary tree, in one persistent kernel fed by a device work
   queue (largest systems first) and replayed from a CUDA graph.  mode
   (argument `exact`): G6_BATCH_EXACT reproduces smallN's floating-point
   operations bit for bit; G6_BATCH_FAST uses one FP64 reciprocal square
   root per pair; G6_BATCH_SPLIT keeps state, predictor and corrector in
   FP64 and evaluates the pair terms in FP32 from double-single positions
   (relative force error ~1e-7).  pos/vel are overwritten; optional
   outputs: t_final[s], steps[s], wall_ms[s] (GPU time from the first to the
   last step of system s), status[s] (0 done, 1 step budget max_steps
   exhausted), *elapsed_ms (whole launch). */
#define G6_BATCH_FAST 0
#define G6_BATCH_EXACT 1
#define G6_BATCH_SPLIT 2
int g6x_batch_run(int nsys, const int *n_per_sys, const double *t_end, const double *mass,
                  double (*pos)[3], double (*vel)[3], double eta, int n_iter,
                  long long max_steps, int exact, double *t_final, long long *steps,
                  double *wall_ms, int *status, double *elapsed_ms);
/* Launch shape of g6x_batch_run: warps (= systems in flight) per CTA and
   CTAs per SM. */
int g6x_batch_config(int warps_per_cta, int ctas_per_sm);
/* smallN's unperturbed binaries in the batch (fast and split modes; the
   exact mode refuses them): after each step the pair that set the step
   becomes a binary node when approaching, within sqrt(r2_crit), its step
   below dt_crit and its tidal parameter below gamma (smallN_unpert.cc:
   44-88); its centre of mass is integrated, its components follow the
   Kepler orbit to the same separation past pericentre, where the change of
   the tidal potential is absorbed and the binary is extended by whole
   periods (allow_full) or dissolved.  smallN's worker defaults: dt_crit
   1e-3, r2_crit 1e-2, gamma 1e-6, allow_full 1 (src/amuse_ph4/src/hdyn.cc:
   10-14, src/amuse_smalln/interface.cc:72).  At most 8 binaries per system
   at a time; with them on, at most 4 warps per CTA.  g6x_batch_binaries
   reads the number of binaries each system of the last run made. */
int g6x_batch_unperturbed(int on, double dt_crit, double r2_crit, double gamma, int allow_full);
int g6x_batch_binaries(int nsys, int *nbin);
/* Autotuner: time the candidate shapes on the given systems (end times
   scaled by frac; the inputs are not modified) and keep the fastest;
   out = {warps per CTA, CTAs per SM, ms}. */
int g6x_batch_tune(int nsys, const int *n_per_sys, const double *t_end, const double *mass,
                   const double (*pos)[3], const double (*vel)[3], double eta, int n_iter,
                   int exact, double frac, double out[3]);

/* Fixed-step Hermite integration and its adjoint (no reference
   counterpart in the GRAPE-6 ABI: the scheme is the hermite code's,
   src/amuse_hermite/interface.cc:266-281 predict_step and :536-552
   correct_step, with this library's force).  All arrays are device
   pointers, particle-major [n][3] doubles (m: [n]); every call blocks.
   g6x_fixed_force         -- (a, j) of all n bodies at (x, v); precision as
                              set by g6x_set_precision; overwrites the j
                              records (a later g6_ call re-predicts).
   g6x_fixed_step          -- one step of size h in place on (x, v, a, j);
                              xp/vp receive the predicted state the force
                              was evaluated at (needed by the adjoint).
   g6x_force_vjp           -- cotangents (gx, gv, gm) of the force's inputs
                              given cotangents (la, lj) of (acc, jerk).
   g6x_fixed_step_adjoint  -- the adjoint of one g6x_fixed_step, in place on
                              the state cotangents (lx, lv, la, lj); lm
                              accumulates the mass cotangent; work holds 7n
                              doubles.
   g6x_fixed_run           -- nsteps steps with one host synchronisation;
                              optionally keeps every step's predicted state
                              (xp_all/vp_all: [nsteps][n][3], or both NULL).
   g6x_fixed_adjoint_run   -- the adjoints of nsteps steps, last first, at
                              the predicted states g6x_fixed_run kept. */
/* Jerk form of the fixed-step force (and of its derivatives):
   G6_JERK_HERMITE (default) -- the hermite code's, whose (r.v) factor is
     divided by the unsoftened r^2 (interface.cc:440-449,486);
   G6_JERK_SOFTENED          -- ph4's / this library's g6 force, the exact
     time derivative of the softened acceleration.  Equal when eps2 = 0. */
#define G6_JERK_HERMITE 0
#define G6_JERK_SOFTENED 1
int g6x_set_fixed_jerk(int form);
int g6x_fixed_force(int n, double eps2, const double *d_x, const double *d_v, const double *d_m,
                    double *d_a, double *d_j);
int g6x_fixed_step(int n, double h, double eps2, double *d_x, double *d_v, double *d_a,
                   double *d_j, const double *d_m, double *d_xp, double *d_vp);
int g6x_force_vjp(int n, double eps2, const double *d_x, const double *d_v, const double *d_m,
                  const double *d_la, const double *d_lj, double *d_gx, double *d_gv,
                  double *d_gm);
int g6x_fixed_step_adjoint(int n, double h, double eps2, const double *d_xp, const double *d_vp,
                           const double *d_m, double *d_lx, double *d_lv, double *d_la,
                           double *d_lj, double *d_lm, double *d_work);
int g6x_fixed_run(int n, double h, double eps2, int nsteps, double *d_x, double *d_v,
                  double *d_a, double *d_j, const double *d_m, double *d_xp_all,
                  double *d_vp_all);
int g6x_fixed_adjoint_run(int n, double h, double eps2, int nsteps, const double *d_xp_all,
                          const double *d_vp_all, const double *d_m, double *d_lx, double *d_lv,
                          double *d_la, double *d_lj, double *d_lm, double *d_work);

/* Device pointers of the predicted j records (for tools) and the stream. */
void *g6x_stream(void);

#ifdef __cplusplus
}
#endif
#endif
