/*
 * g6_dev.h -- internal interface between the C host library (g6_host.c)
 * and the CUDA launchers (kern_*.cu).  Plain C; not installed.
 *
 * HBM layout of the j-system (capacity `cap` slots, a multiple of G6_TILE):
 *   t, dt, m, pot           double[cap]
 *   x, v, a, j              double[3*cap], component-major: x[k*cap + slot]
 *   id, nn                  int[cap]
 *   jp                      predicted records, one per slot, padded to the
 *                           next multiple of G6_TILE with zero-mass records
 *                           far away:
 *                             split: 48 B per slot, stored in pairs of slots
 *                                    (2p, 2p+1) with every field a float2
 *                                    {slot 2p, slot 2p+1}, 96 B per pair:
 *                                    [xh yh zh m][xl yl zl ml][vx vy vz 0]
 *                                    (the force kernel's packed f32x2 loads;
 *                                    m + ml is the FP64 mass to 2^-48, the
 *                                    force kernel uses m, the refinement
 *                                    pass both)
 *                             fp64 : 64 B {x,y,z,m}{vx,vy,vz,0}
 * Accelerations and jerks are stored unscaled (the GRAPE-6 a/2, j/6 inputs
 * are rescaled on the host), so the device predictor evaluates exactly
 * ph4's expression (jdata.cc:736-744).
 */
#ifndef G6_DEV_H
#define G6_DEV_H

#include <cuda_runtime_api.h>

#ifdef __cplusplus
extern "C" {
#endif

#define G6_TILE 256 /* j records per shared-memory tile */

enum { G6_PREC_SPLIT = 0, G6_PREC_FP64 = 1 };

typedef struct {
  int cap;
  double *t, *dt, *m, *pot;
  double *x, *v, *a, *j;
  int *id, *nn;
  void *jp_split; /* 48 B records */
  void *jp_f64;   /* 64 B records */
} g6_jstate;

/* One staged j-update (g6_set_j_particle), 128 B. */
typedef struct {
  int addr, id;
  double t, dt, m;
  double x[3], v[3], a[3], j[3];
} g6_jupd;

/* One force evaluation. i-particles are either given explicitly
 * (ipos/ivel, FP64, [ni][3]) or, when ilist != NULL, are the j-slots in
 * ilist predicted to the same time (ipos/ivel ignored).  iself[i] is the
 * j slot to exclude (the particle itself) or -1.                         */
typedef struct {
  int ni, nj, prec;
  double eps2;
  const double *ipos, *ivel; /* device, [ni][3] */
  const int *ilist;          /* device, [ni] or NULL */
  const int *iself;          /* device, [ni] or NULL (then = ilist) */
  const g6_jstate *js;       /* j-system (device pointers inside) */
  double ti;                 /* prediction time (for ilist mode) */
  /* outputs (device) */
  double *acc, *jerk, *pot;  /* [ni][3], [ni][3], [ni] */
  int *nn;                   /* [ni] nearest j slot (-1 none) */
  float *nn_r2;              /* [ni] (r^2 + eps^2) of nn, or NULL */
  /* scratch for split-j partial sums (device) */
  void *scratch;
  size_t scratch_bytes;
  int *err; /* device error word (0 = ok) */
  /* launch shape override (0 = automatic) */
  int force_jl, force_nsplit;
  int want_nn; /* 0: nn[] = -1 (no nearest-neighbour search) */
  int hjerk;   /* 1: jerk as the hermite code forms it, (r.v) / r^2 with the
                  unsoftened r^2 (src/amuse_hermite/interface.cc:440-449,486);
                  needs want_nn = 0 and force_jl 0 or 1 */
  /* split precision only: the refinement pass (kern_force.cu, refine_kernel)
     that makes the nearest neighbour exact and redoes ill-conditioned sums
     in FP64.  refine: a g6k_refine_bytes() device buffer, zeroed once at
     allocation (NULL: no refinement, and the split-j merge runs as a second
     kernel); kappa: condition number above which acc and pot are redone in
     FP64 (0: never; < 0: no refinement pass at all, the buffer then only
     holds the force kernel's split-merge tickets). */
  void *refine;
  double kappa;
  /* test hook: the first CTA waits for its first tile on a barrier that
     nothing arrives on, with a 20 ms limit, so the bounded wait expires and
     the call ends with the error word set (no trap, no unbounded spin) */
  int stall_test;
  /* optional: recorded on the stream between the force kernel (with its
     split-j merge) and the refinement pass, to time the two apart */
  cudaEvent_t ev_mid;
} g6_force_args;

/* Size of the refinement buffer (fixed; allocated once per context). */
size_t g6k_refine_bytes(void);
/* Last refinement: out[0] particles queued, out[1] of them because of the
   condition number, out[2] the largest queue that overflowed (0: none),
   out[3] of them because of a dominant term.  */
int g6k_refine_read(const void *refine, int out[4], cudaStream_t st);

/* Launch shape actually used (reported by g6k_force). */
typedef struct {
  int jl, nsplit, grid_x, grid_y, threads;
} g6_shape;

size_t g6k_scratch_bytes(int ni, int nj, int prec, int nn, int force_jl, int force_nsplit);
int g6k_sm_count(void);

int g6k_scatter(const g6_jstate *js, const g6_jupd *d_upd, int n, cudaStream_t st);
int g6k_predict(const g6_jstate *js, int nj, double ti, int prec, cudaStream_t st);
int g6k_force(const g6_force_args *a, g6_shape *shape, cudaStream_t st);

/* FP64 Hermite corrector + Aarseth step on the listed slots (in place):
 * idata.cc:399-514.  acc/jerk are the new values at tnext, [ni][3]. */
int g6k_correct(const g6_jstate *js, int ni, const int *ilist, double tnext,
                double eta, const double *acc, const double *jerk,
                const double *pot, const int *nn, cudaStream_t st);
/* Encounter check of one block (idata::check_encounters, idata.cc:620-700)
 * and the stopping decision after its corrector (jdata.cc:797-850).         */
typedef struct {
  double rmax_close, rmax_coll; /* largest rmin/dnn and (R_i + R_nn)/dnn */
  double t;                     /* time of the block */
  int close_slot[2], coll_slot[2];
  int close_id[2], coll_id[2];  /* -1: no pair */
  int stopped;                  /* 1 collision, 2 close pair (bits) */
  int pad;
} g6_enc;
/* A block whose stopping decision (g6k_enc_decide) is still to be taken. */
typedef struct {
  g6_enc *enc; /* NULL: none */
  int mode;
  double t;
  int *flag;
} g6_enc_decision_args;
/* Pre-corrector pass over the block: nn[i] is the nearest j slot of ilist[i]
 * from the force; distances are recomputed in FP64 from both particles
 * predicted to tnext.  part_d >= 2 * ceil(ni/32), part_i >= 4 * ceil(ni/32),
 * *counter == 0 on entry (left 0).                                           */
int g6k_enc_check(const g6_jstate *js, const double *rad, int ni, const int *ilist,
                  const int *nn, double tnext, double rmin, double *part_d, int *part_i,
                  unsigned *counter, g6_enc *enc, cudaStream_t st);
/* Post-corrector: ids of the pairs, the collision test on the corrected
 * state, stop bits into enc->stopped and *flag.                              */
int g6k_enc_decide(const g6_jstate *js, g6_enc *enc, int mode, double tnext, int *flag,
                    cudaStream_t st);
/* g6x_run's two-kernel scheduler: sched_reset once per run (dmin2[0..1] =
 * +inf, *d_ni = 0); per block sched_first (min of t + dt into dmin, *d_ni
 * = 0, the pending stopping decision) then list_predict (kern_predict.cu:
 * the slots with t + dt == tnext into d_ilist / *d_ni, tnext into *d_tnext,
 * all j predicted to tnext in precision prec, *dmin_next = +inf).        */
int g6k_sched_reset(unsigned long long *dmin2, int *d_ni, cudaStream_t st);
int g6k_sched_first(const g6_jstate *js, int nj, unsigned long long *dmin, int *d_ni,
                    const g6_enc_decision_args *decision, cudaStream_t st);
int g6k_list_predict(const g6_jstate *js, int nj, int prec, const unsigned long long *dmin,
                     unsigned long long *dmin_next, int *d_ilist, int *d_ni, double *d_tnext,
                     cudaStream_t st);
/* k nearest neighbours (kern_knn.cu): for each of ni listed slots, the k
 * (1..G6_KNN_MAX) nearest other j in [0, nj) by FP64 distance of the
 * positions predicted to t, ties to the smaller slot.  The split records
 * must hold the j-system predicted to t.  ids (particle ids, -1 when fewer
 * than k others) and d2 (+inf there) are [ni][k] device arrays.          */
#define G6_KNN_MAX 32
size_t g6k_knn_scratch_bytes(int nj, int ni, int k);
int g6k_knn(const g6_jstate *js, int nj, double t, int k, int ni, const int *slots, int *ids,
            double *d2, void *scratch, size_t scratch_bytes, cudaStream_t st);
/* Initial time steps (jdata.cc:503-564 without the median limit). */
int g6k_initial_step(const g6_jstate *js, int nj, double eta, double fac,
                     double limit, double system_time, cudaStream_t st);
/* Kinetic energy and sum m*pot (predicted to t) -> d_out[0..1]. */
int g6k_energy_sums(const g6_jstate *js, int nj, double t, const double *pot_i,
                    double *d_out, cudaStream_t st);
/* Plain copy of acc/jerk/pot/time into the j-state for ilist (t, dt untouched
 * except time = t0), used after the initial force evaluation. */
int g6k_store_forces(const g6_jstate *js, int ni, const int *ilist,
                     const double *acc, const double *jerk, const double *pot,
                     const int *nn, cudaStream_t st);

#ifdef __cplusplus
}
#endif

#ifdef __CUDACC__
/* ph4's prediction of one position component, x + dt*(v + 0.5*dt*(a +
   dt*j/3)) with its rounding order and no contraction (predict_all,
   src/amuse_ph4/src/jdata.cc:736-744; the host i-prediction idata.cc:346-365
   is the same expression); dt == 0 copies. */
__device__ __forceinline__ double g6_predict_x(double x, double v, double a, double j,
                                               double dt) {
  if (dt == 0) return x;
  const double hdt = __dmul_rn(0.5, dt);
  return __dadd_rn(
      x, __dmul_rn(dt, __dadd_rn(v, __dmul_rn(hdt, __dadd_rn(a, __ddiv_rn(__dmul_rn(dt, j), 3.0))))));
}
/* ph4's predicted velocity component, v + dt*(a + 0.5*dt*j) (jdata.cc:741-743). */
__device__ __forceinline__ double g6_predict_v(double v, double a, double j, double dt) {
  if (dt == 0) return v;
  return __dadd_rn(v, __dmul_rn(dt, __dadd_rn(a, __dmul_rn(__dmul_rn(0.5, dt), j))));
}
/* Split-record field f of slot s (f: 0 xh, 1 yh, 2 zh, 3 m, 4 xl, 5 yl,
   6 zl, 7 pad, 8 vx, 9 vy, 10 vz, 11 pad) in the pair layout above. */
__device__ __forceinline__ float *g6_split_field(void *base, int s, int f) {
  return (float *)base + (size_t)(s >> 1) * 24 + (f >> 2) * 8 + (f & 3) * 2 + (s & 1);
}
__device__ __forceinline__ float g6_split_get(const void *base, int s, int f) {
  return *g6_split_field((void *)base, s, f);
}
__device__ __forceinline__ void g6_split_store(void *base, int s, float xh, float yh, float zh,
                                               float m, float ml, float xl, float yl, float zl,
                                               float vx, float vy, float vz) {
  float *p = (float *)base + (size_t)(s >> 1) * 24 + (s & 1);
  p[0] = xh; p[2] = yh; p[4] = zh; p[6] = m;
  p[8] = xl; p[10] = yl; p[12] = zl; p[14] = ml;
  p[16] = vx; p[18] = vy; p[20] = vz; p[22] = 0.f;
}
#endif
#endif
