// kern_step.cu -- FP64 kernels around the force evaluation for the
// device-resident block-step driver (extension API):
//
//   correct_kernel   Hermite corrector + Aarseth step with power-of-2
//                    quantisation, src/amuse_ph4/src/idata.cc:399-514.
//                    The i-particle prediction it corrects is ph4's host
//                    i-prediction (idata.cc:346-365).  Written with explicit
//                    round-to-nearest intrinsics (no contraction into FMA)
//                    so that it rounds exactly like the x86 CPU code.
//   schedule kernels tnext = min_j (t_j + dt_j) and the list of slots with
//                    t_j + dt_j == tnext (the block of scheduler::get_list,
//                    src/amuse_ph4/src/scheduler.cc:66-79).
//   initial_step     jdata::set_initial_timestep (jdata.cc:503-564).
//   energy sums      sum m |v_p|^2 and sum m pot (jdata.cc:582-680).
//   encounter check  idata::check_encounters (idata.cc:620-700) over a
//                    block, and the COLLISION_DETECTION test of
//                    jdata::advance_and_check_encounter (jdata.cc:797-850).
#include "pdl.cuh"
#include <cuda_runtime.h>
#include <limits.h>
#include <stdint.h>

#include "g6_dev.h"

namespace {

constexpr int PT = 256;

__device__ __forceinline__ double dmul(double a, double b) { return __dmul_rn(a, b); }
__device__ __forceinline__ double dadd(double a, double b) { return __dadd_rn(a, b); }
__device__ __forceinline__ double dsub(double a, double b) { return __dsub_rn(a, b); }
__device__ __forceinline__ double ddiv(double a, double b) { return __ddiv_rn(a, b); }

// fmod(t, p) == 0 for p a positive normal power of two, without the
// iterative double-precision fmod: t = m * 2^e (m an integer) is a multiple
// of p = 2^k exactly when e + (trailing zero bits of m) >= k.  Any other p
// goes to fmod.  Infinite or NaN t: fmod is NaN, so "not a multiple".
__device__ __forceinline__ bool multiple_of_pow2(double t, double p) {
  const unsigned long long pb = (unsigned long long)__double_as_longlong(p);
  const int pe = (int)((pb >> 52) & 0x7ff);
  if (pe == 0 || pe == 0x7ff || (pb & 0x000fffffffffffffull) || (pb >> 63))
    return fmod(t, p) == 0;
  const unsigned long long tb = (unsigned long long)__double_as_longlong(t) & 0x7fffffffffffffffull;
  if (tb == 0) return true;
  const int te = (int)(tb >> 52);
  if (te == 0x7ff) return false;
  unsigned long long m = tb & 0x000fffffffffffffull;
  int e;
  if (te == 0) {
    e = -1074;
  } else {
    m |= 1ull << 52;
    e = te - 1075;
  }
  const int tz = __ffsll((long long)m) - 1;
  return e + tz >= pe - 1023;
}

// Four lanes per particle: lane k < 3 corrects component k (the divides of
// the three components run in parallel, which is what bounds a small block's
// latency), and the squared norms are summed in component order after a
// shuffle, exactly as the scalar loop adds them, so the result stays
// bit-identical with ph4.  Lane 3 only takes part in the shuffles.
__global__ void correct_kernel(g6_jstate js, int ni, const int *__restrict__ ilist, double tnext,
                               double eta, const double *__restrict__ acc,
                               const double *__restrict__ jerk, const double *__restrict__ pot,
                               const int *__restrict__ nn) {
  pdl_wait();
  pdl_trigger();
  const int g = blockIdx.x * blockDim.x + threadIdx.x;
  const int i = g >> 2;
  const int k = g & 3;
  const int lane = threadIdx.x & 31;
  const int base = lane & ~3;
  const bool active = i < ni;  // whole groups of 4 agree
  const int ii = active ? i : 0;
  const int s = ilist[ii];
  const int cap = js.cap;
  const double t0 = js.t[s];
  const double dt = dsub(tnext, t0);
  const double dt2 = dmul(dt, dt);
  const int kc = k < 3 ? k : 2;
  double xp, vp, pa2 = 0, pj2 = 0, pk2 = 0, pl2 = 0;
  {
    const double x = js.x[kc * cap + s], v = js.v[kc * cap + s];
    const double oa = js.a[kc * cap + s], oj = js.j[kc * cap + s];
    if (dt == 0) {
      xp = x;
      vp = v;
    } else {
      // x + dt*(v + 0.5*dt*(a + dt*j/3)),  v + dt*(a + 0.5*dt*j)
      const double hdt = dmul(0.5, dt);
      xp = dadd(x, dmul(dt, dadd(v, dmul(hdt, dadd(oa, ddiv(dmul(dt, oj), 3.0))))));
      vp = dadd(v, dmul(dt, dadd(oa, dmul(hdt, oj))));
    }
    const double ia = acc[3 * ii + kc], ij = jerk[3 * ii + kc];
    const double da = dsub(oa, ia);
    const double alpha = dsub(dmul(-3.0, da), dmul(dt, dadd(dmul(2.0, oj), ij)));
    const double beta = dadd(dmul(2.0, da), dmul(dt, dadd(oj, ij)));
    xp = dadd(xp, dmul(dadd(ddiv(alpha, 12.0), ddiv(beta, 20.0)), dt2));
    vp = dadd(vp, dmul(dadd(ddiv(alpha, 3.0), ddiv(beta, 4.0)), dt));
    pa2 = dmul(ia, ia);
    const double dj = dmul(dt, ij);
    pj2 = dmul(dj, dj);
    const double ak = dmul(2.0, alpha);
    pk2 = dmul(ak, ak);
    const double bl = dmul(6.0, beta);
    pl2 = dmul(bl, bl);
  }
  // a2 = ((0 + p0) + p1) + p2, as the scalar component loop accumulates
  double a2 = 0, j2 = 0, k2 = 0, l2 = 0;
#pragma unroll
  for (int c = 0; c < 3; c++) {
    a2 = dadd(a2, __shfl_sync(0xffffffffu, pa2, base + c));
    j2 = dadd(j2, __shfl_sync(0xffffffffu, pj2, base + c));
    k2 = dadd(k2, __shfl_sync(0xffffffffu, pk2, base + c));
    l2 = dadd(l2, __shfl_sync(0xffffffffu, pl2, base + c));
  }
  if (!active) return;
  if (k < 3) {
    js.x[k * cap + s] = xp;
    js.v[k * cap + s] = vp;
    js.a[k * cap + s] = acc[3 * i + k];
    js.j[k * cap + s] = jerk[3 * i + k];
    return;
  }
  // lane 3: the Aarseth step with power-of-two quantisation
  double newstep = dmul(dmul(eta, dt),
                        __dsqrt_rn(ddiv(dadd(__dsqrt_rn(dmul(a2, k2)), j2),
                                        dadd(__dsqrt_rn(dmul(j2, l2)), k2))));
  const double olds = js.dt[s];
  int expo;
  double oldstep2 = ddiv(olds, dmul(2.0, frexp(olds, &expo)));
  for (int guard = 0; guard < 1100 && !multiple_of_pow2(tnext, oldstep2); guard++)
    oldstep2 = ddiv(oldstep2, 2.0);
  if (newstep < oldstep2) {
    newstep = ddiv(oldstep2, 2.0);
  } else {
    const double t2 = dmul(2.0, oldstep2);
    if (newstep >= t2 && multiple_of_pow2(tnext, t2))
      newstep = t2;
    else
      newstep = oldstep2;
  }
  js.t[s] = tnext;
  js.dt[s] = newstep;
  if (pot) js.pot[s] = pot[i];
  if (nn) js.nn[s] = nn[i];
}

// ---- encounter check ----
// A candidate pair (i slot s, its nearest neighbour j) with its ratio r.
// ph4 keeps the first i of its list with the largest r (strict >); the
// block list here has no fixed order, so ties go to the smaller slot, which
// is the first in slot order.
struct EncC {
  double r;
  int s, j;
};

__device__ __forceinline__ void enc_take(EncC &a, const EncC &b) {
  if (b.r > a.r || (b.r == a.r && b.s < a.s)) a = b;
}

__device__ __forceinline__ EncC enc_shfl(const EncC &c, int o) {
  EncC d;
  d.r = __shfl_xor_sync(0xffffffffu, c.r, o);
  d.s = __shfl_xor_sync(0xffffffffu, c.s, o);
  d.j = __shfl_xor_sync(0xffffffffu, c.j, o);
  return d;
}

// Both candidates reduced over the CTA (at most 8 warps); the result is
// valid in thread 0.
__device__ void enc_block_reduce(EncC &c0, EncC &c1) {
  __shared__ EncC sh[2][8];
  for (int o = 16; o > 0; o >>= 1) {
    enc_take(c0, enc_shfl(c0, o));
    enc_take(c1, enc_shfl(c1, o));
  }
  const int w = threadIdx.x >> 5;
  if ((threadIdx.x & 31) == 0) {
    sh[0][w] = c0;
    sh[1][w] = c1;
  }
  __syncthreads();
  if (threadIdx.x == 0)
    for (int k = 1; k < (int)(blockDim.x >> 5); k++) {
      enc_take(c0, sh[0][k]);
      enc_take(c1, sh[1][k]);
    }
  __syncthreads();
}

// Four lanes per block particle, as in the corrector (FP64 runs at 2 lanes
// per SM here, so a block's FP64 work has to spread over many SMs): lane
// k < 3 predicts component k of the particle and of its nearest neighbour
// to tnext and forms dx_k^2; the group sums them in component order (ph4
// CPU mode: idnn = sqrt of the force loop's min r^2 over the predicted
// j-system).  The group's first lane forms r_close = rmin / dnn and r_coll
// = (R_i + R_nn) / dnn for pairs with at least one massive member.  Each
// CTA leaves its best two candidates in part_*; the last CTA to finish
// (atomic ticket) reduces them and writes the block's result.
__global__ void enc_check_kernel(g6_jstate js, const double *__restrict__ rad, int ni,
                                 const int *__restrict__ ilist, const int *__restrict__ nn,
                                 double tnext, double rmin, double *part_d, int *part_i,
                                 unsigned *counter, g6_enc *enc) {
  const double tiny = 1.0 / 4503599627370496.0;  // 2^-52 (stdinc.h)
  const int g = blockIdx.x * blockDim.x + threadIdx.x;
  const int i = g >> 2;
  const int k = g & 3;
  const int base = (threadIdx.x & 31) & ~3;
  const int ii = i < ni ? i : 0;
  const int s = ilist[ii];
  const int jn = nn[ii];
  const bool valid = i < ni && jn >= 0 && (js.m[jn] > tiny || js.m[s] > tiny);
  double p = 0;
  if (valid && k < 3) {
    const int cap = js.cap;
    const int a = k * cap + s, b = k * cap + jn;
    const double xi = g6_predict_x(js.x[a], js.v[a], js.a[a], js.j[a], dsub(tnext, js.t[s]));
    const double xj = g6_predict_x(js.x[b], js.v[b], js.a[b], js.j[b], dsub(tnext, js.t[jn]));
    const double dx = dsub(xj, xi);
    p = dmul(dx, dx);
  }
  double r2 = 0;
#pragma unroll
  for (int c = 0; c < 3; c++) r2 = dadd(r2, __shfl_sync(0xffffffffu, p, base + c));
  EncC cc = {0.0, INT_MAX, -1}, cl = {0.0, INT_MAX, -1};
  if (valid && k == 0) {
    const double dnn = __dsqrt_rn(r2);
    cc.r = ddiv(rmin, dnn);
    cc.s = s;
    cc.j = jn;
    cl.r = ddiv(dadd(rad[s], rad[jn]), dnn);
    cl.s = s;
    cl.j = jn;
  }
  enc_block_reduce(cc, cl);
  __shared__ bool last;
  if (threadIdx.x == 0) {
    part_d[2 * blockIdx.x] = cc.r;
    part_d[2 * blockIdx.x + 1] = cl.r;
    part_i[4 * blockIdx.x] = cc.s;
    part_i[4 * blockIdx.x + 1] = cc.j;
    part_i[4 * blockIdx.x + 2] = cl.s;
    part_i[4 * blockIdx.x + 3] = cl.j;
    __threadfence();
    last = atomicAdd(counter, 1u) == gridDim.x - 1;
  }
  __syncthreads();
  if (!last) return;
  __threadfence();
  EncC a = {0.0, INT_MAX, -1}, b = {0.0, INT_MAX, -1};
  for (int q = threadIdx.x; q < (int)gridDim.x; q += blockDim.x) {
    const EncC ka = {__ldcg(part_d + 2 * q), __ldcg(part_i + 4 * q), __ldcg(part_i + 4 * q + 1)};
    const EncC kb = {__ldcg(part_d + 2 * q + 1), __ldcg(part_i + 4 * q + 2),
                     __ldcg(part_i + 4 * q + 3)};
    enc_take(a, ka);
    enc_take(b, kb);
  }
  enc_block_reduce(a, b);
  if (threadIdx.x == 0) {
    enc->rmax_close = a.r;
    enc->rmax_coll = b.r;
    const bool close = a.r >= 1.0, coll = b.r >= 1.0;
    enc->close_slot[0] = close ? a.s : -1;
    enc->close_slot[1] = close ? a.j : -1;
    enc->coll_slot[0] = coll ? b.s : -1;
    enc->coll_slot[1] = coll ? b.j : -1;
    *counter = 0;
  }
}

// After the corrector: the pair ids, and ph4's COLLISION_DETECTION test on
// the current state of the pair, vr < EPS r v with EPS = 0.001
// (jdata.cc:797,822-848).  mode bits: 2 stop on an approaching collision
// pair, 4 stop on any close pair.  One thread.
__device__ void enc_decide(const g6_jstate &js, g6_enc *enc, int mode, double t, int *flag) {
  const int cap = js.cap;
  for (int p = 0; p < 2; p++) {
    enc->close_id[p] = enc->close_slot[p] >= 0 ? js.id[enc->close_slot[p]] : -1;
    enc->coll_id[p] = enc->coll_slot[p] >= 0 ? js.id[enc->coll_slot[p]] : -1;
  }
  int stop = 0;
  if ((mode & 2) && enc->coll_slot[0] >= 0) {
    const int j1 = enc->coll_slot[0], j2 = enc->coll_slot[1];
    double r = 0, v = 0, vr = 0;
    for (int k = 0; k < 3; k++) {
      const double dx = dsub(js.x[k * cap + j1], js.x[k * cap + j2]);
      const double dv = dsub(js.v[k * cap + j1], js.v[k * cap + j2]);
      r = dadd(r, dmul(dx, dx));
      v = dadd(v, dmul(dv, dv));
      vr = dadd(vr, dmul(dx, dv));
    }
    r = __dsqrt_rn(r);
    v = __dsqrt_rn(v);
    if (vr < dmul(dmul(0.001, r), v)) stop |= 1;
  }
  if ((mode & 4) && enc->close_slot[0] >= 0) stop |= 2;
  enc->stopped = stop;
  enc->t = t;
  *flag = stop;
}

__global__ void enc_decide_kernel(g6_jstate js, g6_enc *enc, int mode, double t, int *flag) {
  if (threadIdx.x == 0 && blockIdx.x == 0) enc_decide(js, enc, mode, t, flag);
}

__global__ void store_kernel(g6_jstate js, int ni, const int *__restrict__ ilist,
                             const double *__restrict__ acc, const double *__restrict__ jerk,
                             const double *__restrict__ pot, const int *__restrict__ nn) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= ni) return;
  const int s = ilist[i];
  const int cap = js.cap;
#pragma unroll
  for (int k = 0; k < 3; k++) {
    js.a[k * cap + s] = acc[3 * i + k];
    js.j[k * cap + s] = jerk[3 * i + k];
  }
  if (pot) js.pot[s] = pot[i];
  if (nn) js.nn[s] = nn[i];
}

// t + dt >= 0 always, so the IEEE bit pattern orders like an unsigned int.
// First kernel of a block in g6x_run: the minimum of t + dt (into dmin,
// which the previous block's list_predict_kernel reset to +inf), the block
// count reset (the host has read the previous count), and the previous
// block's encounter stopping decision (after that block's corrector).
__global__ void sched_min_first(g6_jstate js, int nj, unsigned long long *dmin, int *dni,
                                g6_enc_decision_args v) {
  pdl_wait();
  pdl_trigger();
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    *dni = 0;
    if (v.enc) enc_decide(js, v.enc, v.mode, v.t, v.flag);
  }
  __shared__ unsigned long long w[PT / 32];
  unsigned long long m = 0x7ff0000000000000ull;
  for (int s = blockIdx.x * blockDim.x + threadIdx.x; s < nj; s += gridDim.x * blockDim.x) {
    const unsigned long long b = __double_as_longlong(js.t[s] + js.dt[s]);
    m = b < m ? b : m;
  }
  for (int o = 16; o > 0; o >>= 1) {
    const unsigned long long x = __shfl_xor_sync(0xffffffffu, m, o);
    m = x < m ? x : m;
  }
  if ((threadIdx.x & 31) == 0) w[threadIdx.x >> 5] = m;
  __syncthreads();
  if (threadIdx.x == 0) {
    for (int k = 1; k < PT / 32; k++) m = w[k] < m ? w[k] : m;
    atomicMin(dmin, m);
  }
}

__global__ void sched_reset(unsigned long long *dmin, int *dni) {
  dmin[0] = dmin[1] = 0x7ff0000000000000ull;
  *dni = 0;
}

__global__ void initial_step_kernel(g6_jstate js, int nj, double eta, double fac, double limit,
                                    double system_time) {
  const int s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= nj) return;
  const int cap = js.cap;
  double a2 = 0, j2 = 0;
#pragma unroll
  for (int k = 0; k < 3; k++) {
    const double a = js.a[k * cap + s], j = js.j[k * cap + s];
    a2 = dadd(a2, dmul(a, a));
    j2 = dadd(j2, dmul(j, j));
  }
  double fs;
  if (eta == 0.0)
    fs = limit;
  else if (a2 == 0.0 || j2 == 0.0)
    fs = dmul(fac, eta);
  else
    fs = dmul(dmul(fac, eta), __dsqrt_rn(ddiv(a2, j2)));
  if (isnan(fs)) fs = dmul(fac, eta);
  int expo;
  fs = ddiv(fs, dmul(2.0, frexp(fs, &expo)));
  for (int g = 0; g < 1100 && !multiple_of_pow2(system_time, fs); g++) fs = ddiv(fs, 2.0);
  for (int g = 0; g < 1100 && fs > limit; g++) fs = ddiv(fs, 2.0);
  js.dt[s] = fs;
  js.t[s] = system_time;
}

__global__ void clamp_step_kernel(g6_jstate js, int nj, double dtmax) {
  const int s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= nj) return;
  double d = js.dt[s];
  for (int g = 0; g < 1100 && d > dtmax; g++) d = ddiv(d, 2.0);
  js.dt[s] = d;
}

// Per-block partial sums of m|v_p|^2 and m*pot, in fixed order.
__global__ void energy_partial(g6_jstate js, int nj, double t, const double *__restrict__ pot,
                               double *part) {
  __shared__ double sk[PT], sp[PT];
  const int cap = js.cap;
  double kin = 0, pe = 0;
  const int s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s < nj) {
    const double m = js.m[s];
    const double dt = t - js.t[s];
    double v2 = 0;
    for (int k = 0; k < 3; k++) {
      double v = js.v[k * cap + s];
      if (dt != 0) {
        const double a = js.a[k * cap + s], j = js.j[k * cap + s];
        v = dadd(v, dmul(dt, dadd(a, dmul(dmul(0.5, dt), j))));
      }
      v2 = dadd(v2, dmul(v, v));
    }
    kin = dmul(m, v2);
    pe = pot ? dmul(m, pot[s]) : 0.0;
  }
  sk[threadIdx.x] = kin;
  sp[threadIdx.x] = pe;
  __syncthreads();
  for (int o = PT / 2; o > 0; o >>= 1) {
    if (threadIdx.x < o) {
      sk[threadIdx.x] += sk[threadIdx.x + o];
      sp[threadIdx.x] += sp[threadIdx.x + o];
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    part[2 * blockIdx.x] = sk[0];
    part[2 * blockIdx.x + 1] = sp[0];
  }
}

__global__ void energy_final(const double *part, int nb, double *out) {
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  double k = 0, p = 0;
  for (int b = 0; b < nb; b++) {
    k += part[2 * b];
    p += part[2 * b + 1];
  }
  out[0] = k;
  out[1] = p;
}

}  // namespace

extern "C" int g6k_correct(const g6_jstate *js, int ni, const int *ilist, double tnext,
                           double eta, const double *acc, const double *jerk, const double *pot,
                           const int *nn, cudaStream_t st) {
  if (ni <= 0) return 0;
  // 4 lanes per particle, 32 particles per 128-thread block
  return launch_pdl(correct_kernel, dim3((ni + 31) / 32), dim3(128), 0, st, *js, ni, ilist, tnext,
                    eta, acc, jerk, pot, nn) == cudaSuccess
             ? 0
             : -3;
}

extern "C" int g6k_store_forces(const g6_jstate *js, int ni, const int *ilist, const double *acc,
                                const double *jerk, const double *pot, const int *nn,
                                cudaStream_t st) {
  if (ni <= 0) return 0;
  store_kernel<<<(ni + PT - 1) / PT, PT, 0, st>>>(*js, ni, ilist, acc, jerk, pot, nn);
  return cudaGetLastError() == cudaSuccess ? 0 : -3;
}

// g6x_run's scheduler, in two kernels per block with the predictor:
// g6k_sched_reset once before the loop (both parities' minima +inf), then
// per block g6k_sched_first (minimum into dmin[parity]) and
// g6k_list_predict (kern_predict.cu: the block list, tnext, the prediction,
// and dmin[1 - parity] reset for the next block).
extern "C" int g6k_sched_reset(unsigned long long *dmin2, int *d_ni, cudaStream_t st) {
  sched_reset<<<1, 1, 0, st>>>(dmin2, d_ni);
  return cudaGetLastError() == cudaSuccess ? 0 : -3;
}

extern "C" int g6k_sched_first(const g6_jstate *js, int nj, unsigned long long *dmin, int *d_ni,
                               const g6_enc_decision_args *decision, cudaStream_t st) {
  if (nj <= 0) return -1;
  int grid = (nj + PT - 1) / PT;
  const int cap_grid = 4 * g6k_sm_count();
  if (grid > cap_grid) grid = cap_grid;
  g6_enc_decision_args v;
  if (decision) {
    v = *decision;
  } else {
    v.enc = NULL;
    v.mode = 0;
    v.t = 0;
    v.flag = NULL;
  }
  return launch_pdl(sched_min_first, dim3(grid), dim3(PT), 0, st, *js, nj, dmin, d_ni, v) ==
                 cudaSuccess
             ? 0
             : -3;
}

extern "C" int g6k_enc_check(const g6_jstate *js, const double *rad, int ni, const int *ilist,
                             const int *nn, double tnext, double rmin, double *part_d,
                             int *part_i, unsigned *counter, g6_enc *enc, cudaStream_t st) {
  if (ni <= 0) return 0;
  // 4 lanes per particle, 32 particles per 128-thread block
  enc_check_kernel<<<(ni + 31) / 32, 128, 0, st>>>(*js, rad, ni, ilist, nn, tnext, rmin, part_d,
                                                   part_i, counter, enc);
  return cudaGetLastError() == cudaSuccess ? 0 : -3;
}

extern "C" int g6k_enc_decide(const g6_jstate *js, g6_enc *enc, int mode, double tnext,
                               int *flag, cudaStream_t st) {
  enc_decide_kernel<<<1, 32, 0, st>>>(*js, enc, mode, tnext, flag);
  return cudaGetLastError() == cudaSuccess ? 0 : -3;
}

extern "C" int g6k_initial_step(const g6_jstate *js, int nj, double eta, double fac, double limit,
                                double system_time, cudaStream_t st) {
  if (nj <= 0) return 0;
  initial_step_kernel<<<(nj + PT - 1) / PT, PT, 0, st>>>(*js, nj, eta, fac, limit, system_time);
  return cudaGetLastError() == cudaSuccess ? 0 : -3;
}

extern "C" int g6k_clamp_steps(const g6_jstate *js, int nj, double dtmax, cudaStream_t st) {
  if (nj <= 0) return 0;
  clamp_step_kernel<<<(nj + PT - 1) / PT, PT, 0, st>>>(*js, nj, dtmax);
  return cudaGetLastError() == cudaSuccess ? 0 : -3;
}

// d_out must hold 2 + 2*ceil(nj/256) doubles; results in d_out[0..1].
extern "C" int g6k_energy_sums(const g6_jstate *js, int nj, double t, const double *pot_i,
                               double *d_out, cudaStream_t st) {
  if (nj <= 0) return 0;
  const int nb = (nj + PT - 1) / PT;
  energy_partial<<<nb, PT, 0, st>>>(*js, nj, t, pot_i, d_out + 2);
  energy_final<<<1, 32, 0, st>>>(d_out + 2, nb, d_out);
  return cudaGetLastError() == cudaSuccess ? 0 : -3;
}
