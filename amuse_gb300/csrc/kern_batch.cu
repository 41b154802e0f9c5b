// kern_batch.cu -- many independent few-body systems in one persistent
// launch (the encounters that AMUSE's multiples module hands to smallN).
//
// Each warp takes a system from a device work queue (an atomic counter over
// a host-chosen order, largest systems first), integrates it to its end
// time, writes it back and takes the next one, so uneven systems balance
// themselves.  The integrator is smallN's (src/amuse_ph4/src/smallN.cc):
// without the unperturbed-binary tree in batch_kernel (its EXACT mode is
// bit-identical to smallN with dt_crit = 0), with it in batch_unp_kernel
// (below) -- a shared-step, time-symmetrised
// 4th-order Hermite scheme --
//   predict_loworder (hdyn.h:192-201) from the stored old acc/jerk,
//   n_iter + 1 force evaluations per step, each followed by
//   correct_acc_and_jerk / correct_pos_and_vel (smallN.cc:487-531) for the
//   iterated step new_dt (smallN.cc:617-660),
//   step from the Kepler criterion eta * sqrt(min over pairs of
//   min(0.5 r^3 / (m_i + m_j), r^2 / v^2)) (smallN.cc:85-116, :318-363).
// State is FP64.  Lane l owns bodies l and l + 32 (n <= 64).
//
// EXACT = true evaluates every expression with the same IEEE operations, in
// the same order, as smallN on the CPU (each pair in its (i < j) orientation,
// contributions accumulated in smallN's pair order, no fused multiply-adds,
// IEEE divides and square roots), so results are bit-identical to smallN.
// MODE_FAST uses one reciprocal square root per pair and FMAs (about 7x
// fewer FP64 instructions; results differ from smallN at the last-bit
// level, which chaotic systems amplify).
// MODE_SPLIT keeps the state, the predictor and the corrector in FP64 but
// evaluates the pair terms in FP32 from double-single positions (the
// relative position is exact to FP32 precision of |r|, as in the g6 force
// kernel) and FP32 velocities, with one rsqrt.approx per pair: GB300 runs
// FP32 at 64x its FP64 rate, and the pair terms are the O(n^2) part.
#include <cuda_runtime.h>
#include <stdint.h>

namespace {

constexpr int MAXN = 64;
constexpr int WARPS_MAX = 8;
enum { MODE_FAST = 0, MODE_EXACT = 1, MODE_SPLIT = 2 };


__device__ __forceinline__ double ADD(double a, double b) { return __dadd_rn(a, b); }
__device__ __forceinline__ double SUB(double a, double b) { return __dsub_rn(a, b); }
__device__ __forceinline__ double MUL(double a, double b) { return __dmul_rn(a, b); }
__device__ __forceinline__ double DIV(double a, double b) { return __ddiv_rn(a, b); }

struct Body {
  double m, inv_m;
  double pos[3], vel[3], pp[3], pv[3], acc[3], jerk[3], oacc[3], ojerk[3];
};

struct WarpSmem {
  union {
    struct {
      double pp[MAXN][3];
      double pv[MAXN][3];
    } d;
    struct {  // MODE_SPLIT: double-single positions, FP32 velocities
      float ph[MAXN][3];
      float pl[MAXN][3];
      float vf[MAXN][3];
    } f;
  };
  double m[MAXN];
  float mf[MAXN];
};

// 1/sqrt(x): FP32 MUFU seed, two Newton-Raphson steps.
__device__ __forceinline__ double rsqrt64(double x) {
  double y = (double)rsqrtf((float)x);
  const double hx = 0.5 * x;
  y = y * fma(-hx * y, y, 1.5);
  y = y * fma(-hx * y, y, 1.5);
  return y;
}

// Contribution of the pair (a, b), a < b in smallN's orientation, to body
// `me` (me == a or me == b), plus the pair's Kepler time-step^2.
template <bool EXACT>
__device__ __forceinline__ double pair_term(const WarpSmem &S, int a, int b, bool me_is_a,
                                            double inv_me, double acc[3], double jerk[3]) {
  const double ma = S.m[a], mb = S.m[b];
  double dx[3], dv[3];
#pragma unroll
  for (int k = 0; k < 3; k++) {
    dx[k] = SUB(S.d.pp[b][k], S.d.pp[a][k]);
    dv[k] = SUB(S.d.pv[b][k], S.d.pv[a][k]);
  }
  if (EXACT) {
    const double d2 = ADD(ADD(MUL(dx[0], dx[0]), MUL(dx[1], dx[1])), MUL(dx[2], dx[2]));
    const double d = __dsqrt_rn(d2);
    const double d3 = MUL(d2, d);
    const double xv = ADD(ADD(MUL(dx[0], dv[0]), MUL(dx[1], dv[1])), MUL(dx[2], dv[2]));
    const double d5 = MUL(d3, d2);
    const double s = me_is_a ? inv_me : -inv_me;
#pragma unroll
    for (int k = 0; k < 3; k++) {
      const double iforce = DIV(MUL(mb, dx[k]), d3);
      const double ijerk = MUL(mb, SUB(DIV(dv[k], d3), DIV(MUL(MUL(3.0, dx[k]), xv), d5)));
      const double force = MUL(ma, iforce);
      const double jk = MUL(ma, ijerk);
      acc[k] = ADD(acc[k], MUL(s, force));
      jerk[k] = ADD(jerk[k], MUL(s, jk));
    }
    const double mass = ADD(mb, ma);
    const double vel2 = ADD(ADD(MUL(dv[0], dv[0]), MUL(dv[1], dv[1])), MUL(dv[2], dv[2]));
    const double dtff2 = DIV(MUL(0.5, d3), mass);
    const double dtv2 = DIV(d2, fabs(vel2));
    return fmin(dtff2, dtv2);
  } else {
    const double d2 = dx[0] * dx[0] + dx[1] * dx[1] + dx[2] * dx[2];
    const double rinv = rsqrt64(d2);
    const double rinv2 = rinv * rinv;
    const double rinv3 = rinv * rinv2;
    const double xv = dx[0] * dv[0] + dx[1] * dv[1] + dx[2] * dv[2];
    const double mo = me_is_a ? mb : -ma;  // force/m_me on me
    const double f = mo * rinv3;
    const double a3 = -3.0 * xv * rinv2;
#pragma unroll
    for (int k = 0; k < 3; k++) {
      acc[k] = fma(f, dx[k], acc[k]);
      jerk[k] = fma(f, fma(a3, dx[k], dv[k]), jerk[k]);
    }
    (void)inv_me;
    const double vel2 = dv[0] * dv[0] + dv[1] * dv[1] + dv[2] * dv[2];
    const double d3 = d2 * d2 * rinv;
    const double dtff2 = 0.5 * d3 / (ma + mb);
    const double dtv2 = d2 / vel2;
    return fmin(dtff2, dtv2);
  }
}

__device__ __forceinline__ float rsqrt_approx(float x) {
  float y;
  asm("rsqrt.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
  return y;
}

// MODE_SPLIT pair term: contribution of j to body i, and the pair's Kepler
// step^2.  FP32 unless the pair is closer than 1e-9 (d^2 < 1e-18): there
// m / d^3 times a relative velocity ~ sqrt(M / d) can leave the FP32 range,
// so such (rare) pairs are evaluated in FP64 into separate accumulators.
// The pair j == i (self) is evaluated too, with its contribution masked to
// zero and its step to +inf, so the j loop has no divergent skip.  The step
// quotients use the approximate division (split mode is not bit-exact with
// anything, and the step only has to follow the criterion closely).
__device__ __forceinline__ float pair_split(const WarpSmem &S, int i, int j, float acc[3],
                                            float jerk[3], double accd[3], double jerkd[3]) {
  const bool self = j == i;
  float dx[3], dv[3];
#pragma unroll
  for (int k = 0; k < 3; k++) {
    dx[k] = __fadd_rn(__fsub_rn(S.f.ph[j][k], S.f.ph[i][k]), __fsub_rn(S.f.pl[j][k], S.f.pl[i][k]));
    dv[k] = S.f.vf[j][k] - S.f.vf[i][k];
  }
  const float d2 = fmaf(dx[2], dx[2], fmaf(dx[1], dx[1], dx[0] * dx[0]));
  const float v2 = fmaf(dv[2], dv[2], fmaf(dv[1], dv[1], dv[0] * dv[0]));
  const float mt = S.mf[i] + S.mf[j];
  if (self || d2 >= 1e-18f) {
    const float rinv = self ? 0.f : rsqrt_approx(d2);
    const float rinv2 = rinv * rinv;
    const float f = S.mf[j] * rinv * rinv2;
    const float xv = fmaf(dx[2], dv[2], fmaf(dx[1], dv[1], dx[0] * dv[0]));
    const float a3 = -3.0f * xv * rinv2;
#pragma unroll
    for (int k = 0; k < 3; k++) {
      acc[k] = fmaf(f, dx[k], acc[k]);
      jerk[k] = fmaf(f, fmaf(a3, dx[k], dv[k]), jerk[k]);
    }
    const float ts = fminf(__fdividef(0.5f * d2 * (d2 * rinv), mt), __fdividef(d2, v2));
    return self ? __int_as_float(0x7f800000) : ts;
  }
  double X[3], W[3];
#pragma unroll
  for (int k = 0; k < 3; k++) {
    X[k] = (double)dx[k];
    W[k] = (double)dv[k];
  }
  const double dd2 = X[0] * X[0] + X[1] * X[1] + X[2] * X[2];
  const double d = sqrt(dd2);
  const double rinv2 = 1.0 / dd2;
  const double f = (double)S.mf[j] * rinv2 / d;
  const double a3 = -3.0 * (X[0] * W[0] + X[1] * W[1] + X[2] * W[2]) * rinv2;
#pragma unroll
  for (int k = 0; k < 3; k++) {
    accd[k] += f * X[k];
    jerkd[k] += f * (a3 * X[k] + W[k]);
  }
  const double vv = W[0] * W[0] + W[1] * W[1] + W[2] * W[2];
  return (float)fmin(0.5 * dd2 * d / (double)mt, dd2 / vv);
}

// acc/jerk of the lane's bodies from the predicted state in S; returns the
// system's min Kepler step^2 (warp-uniform).
template <int MODE>
__device__ double forces(const WarpSmem &S, int n, int lane, Body B[2]) {
  constexpr bool EXACT = MODE == MODE_EXACT;
  double ts2 = __longlong_as_double(0x7ff0000000000000ll);
#pragma unroll
  for (int q = 0; q < 2; q++) {
    const int i = lane + 32 * q;
#pragma unroll
    for (int k = 0; k < 3; k++) B[q].acc[k] = B[q].jerk[k] = 0.0;
    if (i >= n) continue;
    if (MODE == MODE_SPLIT) {
      float a[3] = {0.f, 0.f, 0.f}, jk[3] = {0.f, 0.f, 0.f};
      double ad[3] = {0.0, 0.0, 0.0}, jd[3] = {0.0, 0.0, 0.0};
      float m2 = __int_as_float(0x7f800000);
      for (int j = 0; j < n; j++) m2 = fminf(m2, pair_split(S, i, j, a, jk, ad, jd));
#pragma unroll
      for (int k = 0; k < 3; k++) {
        B[q].acc[k] = (double)a[k] + ad[k];
        B[q].jerk[k] = (double)jk[k] + jd[k];
      }
      ts2 = fmin(ts2, (double)m2);
    } else if (EXACT) {
      // smallN's pair order: (j, i) for j < i first, then (i, j) for j > i,
      // each pair in its (i < j) orientation.
      for (int j = 0; j < i; j++)
        ts2 = fmin(ts2, pair_term<true>(S, j, i, false, B[q].inv_m, B[q].acc, B[q].jerk));
      for (int j = i + 1; j < n; j++)
        ts2 = fmin(ts2, pair_term<true>(S, i, j, true, B[q].inv_m, B[q].acc, B[q].jerk));
    } else {
      // orientation-free (same instruction stream in every lane)
      for (int j = 0; j < n; j++) {
        if (j == i) continue;
        ts2 = fmin(ts2, pair_term<false>(S, i, j, true, B[q].inv_m, B[q].acc, B[q].jerk));
      }
    }
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) ts2 = fmin(ts2, __shfl_xor_sync(0xffffffffu, ts2, o));
  return ts2;
}

template <int MODE>
__device__ __forceinline__ void publish(WarpSmem &S, int n, int lane, const Body B[2]) {
  __syncwarp();
#pragma unroll
  for (int q = 0; q < 2; q++) {
    const int i = lane + 32 * q;
    if (i < n) {
#pragma unroll
      for (int k = 0; k < 3; k++) {
        if (MODE == MODE_SPLIT) {
          const float h = __double2float_rn(B[q].pp[k]);
          S.f.ph[i][k] = h;
          S.f.pl[i][k] = __double2float_rn(B[q].pp[k] - (double)h);
          S.f.vf[i][k] = __double2float_rn(B[q].pv[k]);
        } else {
          S.d.pp[i][k] = B[q].pp[k];
          S.d.pv[i][k] = B[q].pv[k];
        }
      }
    }
  }
  __syncwarp();
}

template <int MODE>
__global__ void batch_kernel(const int *__restrict__ order, const int *__restrict__ off,
                             const double *__restrict__ t_end_s, const double *__restrict__ mass,
                             double *pos, double *vel, double eta, int n_iter,
                             long long max_steps, int *queue, double *t_out, long long *steps_out,
                             unsigned long long *wall_ns, int *status) {
  constexpr bool EXACT = MODE == MODE_EXACT;
  __shared__ WarpSmem smem[WARPS_MAX];
  const int lane = threadIdx.x & 31;
  const int w = threadIdx.x >> 5;
  WarpSmem &S = smem[w];
  const int nsys = queue[1];  // written by the host before the launch
  while (true) {
    int q = 0;
    if (lane == 0) q = atomicAdd(queue, 1);
    q = __shfl_sync(0xffffffffu, q, 0);
    if (q >= nsys) break;
    const int s = order[q];
    unsigned long long t0;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t0));
    const int base = off[s];
    const int n = off[s + 1] - base;
    const double t_end = t_end_s[s];
    if (n < 2 || n > MAXN) {
      if (lane == 0) {
        status[s] = 2;  // unsupported size (host also checks)
        steps_out[s] = 0;
        t_out[s] = 0.0;
      }
      continue;
    }
    Body B[2];
#pragma unroll
    for (int qq = 0; qq < 2; qq++) {
      const int i = lane + 32 * qq;
      const int ii = i < n ? i : 0;
      B[qq].m = mass[base + ii];
      B[qq].inv_m = EXACT ? DIV(1.0, B[qq].m) : 1.0 / B[qq].m;
#pragma unroll
      for (int k = 0; k < 3; k++) {
        B[qq].pos[k] = pos[3 * (base + ii) + k];
        B[qq].vel[k] = vel[3 * (base + ii) + k];
        B[qq].pp[k] = B[qq].pos[k];  // init_pred
        B[qq].pv[k] = B[qq].vel[k];
        B[qq].oacc[k] = B[qq].ojerk[k] = 0.0;  // hdyn() zeroes them
      }
      if (i < n) {
        S.m[i] = B[qq].m;
        S.mf[i] = __double2float_rn(B[qq].m);
      }
    }
    publish<MODE>(S, n, lane, B);
    double t = 0.0, t_pred = -1.0;
    double dt = EXACT ? MUL(eta, __dsqrt_rn(forces<MODE>(S, n, lane, B)))
                      : eta * sqrt(forces<MODE>(S, n, lane, B));
    long long nsteps = 0;
    int st = 0;
    while (t < t_end) {
      if (nsteps >= max_steps) {
        st = 1;  // step budget exhausted
        break;
      }
      const double tn = EXACT ? ADD(t, dt) : t + dt;
      if (tn != t_pred) {  // predict_loworder_all
        const double h = EXACT ? SUB(tn, t) : tn - t;
        const double h3 = EXACT ? DIV(h, 3.0) : h / 3.0;
        const double h2 = EXACT ? DIV(h, 2.0) : h * 0.5;
#pragma unroll
        for (int qq = 0; qq < 2; qq++) {
#pragma unroll
          for (int k = 0; k < 3; k++) {
            const double oj = B[qq].ojerk[k], oa = B[qq].oacc[k];
            if (EXACT) {
              B[qq].pp[k] = ADD(MUL(ADD(MUL(ADD(MUL(oj, h3), oa), h2), B[qq].vel[k]), h), B[qq].pos[k]);
              B[qq].pv[k] = ADD(MUL(ADD(MUL(oj, h2), oa), h), B[qq].vel[k]);
            } else {
              B[qq].pp[k] = fma(fma(fma(oj, h3, oa), h2, B[qq].vel[k]), h, B[qq].pos[k]);
              B[qq].pv[k] = fma(fma(oj, h2, oa), h, B[qq].vel[k]);
            }
          }
        }
        t_pred = tn;
      }
#pragma unroll
      for (int qq = 0; qq < 2; qq++)
#pragma unroll
        for (int k = 0; k < 3; k++) {
          B[qq].oacc[k] = B[qq].acc[k];
          B[qq].ojerk[k] = B[qq].jerk[k];
        }
      double new_dt = dt, end_dt = dt;
      for (int it = 0; it <= n_iter; it++) {
        const double prev = new_dt;
        publish<MODE>(S, n, lane, B);
        const double ts2 = forces<MODE>(S, n, lane, B);
        end_dt = EXACT ? MUL(eta, __dsqrt_rn(ts2)) : eta * sqrt(ts2);
        if (it < n_iter) {
          if (EXACT) {
            new_dt = MUL(0.5, ADD(dt, end_dt));
            new_dt = ADD(dt, MUL(MUL(0.5, SUB(end_dt, dt)), DIV(new_dt, prev)));
          } else {
            new_dt = 0.5 * (dt + end_dt);
            new_dt = dt + 0.5 * (end_dt - dt) * (new_dt / prev);
          }
        }
        const bool cj = new_dt != prev;
        double tau = 0, tau2 = 0, tau3 = 0, theta = 0, inv_theta = 0;
        if (cj) {
          if (EXACT) {
            const double dt_off = SUB(new_dt, MUL(0.5, prev));
            theta = MUL(0.5, prev);
            tau = DIV(dt_off, theta);
            inv_theta = DIV(1.0, theta);
            tau2 = MUL(tau, tau);
            tau3 = MUL(tau2, tau);
          } else {
            theta = 0.5 * prev;
            tau = (new_dt - theta) / theta;
            inv_theta = 1.0 / theta;
            tau2 = tau * tau;
            tau3 = tau2 * tau;
          }
        }
        const double nd2 = EXACT ? MUL(new_dt, new_dt) : new_dt * new_dt;
#pragma unroll
        for (int qq = 0; qq < 2; qq++) {
          Body &b = B[qq];
#pragma unroll
          for (int k = 0; k < 3; k++) {
            if (cj) {  // correct_acc_and_jerk(new_dt, prev)
              const double pa = b.acc[k], pj = b.jerk[k], oa = b.oacc[k], oj = b.ojerk[k];
              if (EXACT) {
                const double c1 = ADD(SUB(2.0, MUL(3.0, tau)), tau3);
                const double c2 = SUB(ADD(2.0, MUL(3.0, tau)), tau3);
                const double c3 = ADD(SUB(SUB(1.0, tau), tau2), tau3);
                const double c4 = ADD(ADD(SUB(-1.0, tau), tau2), tau3);
                b.acc[k] = MUL(0.25, ADD(ADD(ADD(MUL(oa, c1), MUL(pa, c2)), MUL(MUL(oj, theta), c3)),
                                         MUL(MUL(pj, theta), c4)));
                const double e1 = ADD(-1.0, tau2), e2 = SUB(1.0, tau2);
                const double e3 = ADD(SUB(-1.0, MUL(2.0, tau)), MUL(3.0, tau2));
                const double e4 = ADD(ADD(-1.0, MUL(2.0, tau)), MUL(3.0, tau2));
                b.jerk[k] = MUL(0.25, ADD(ADD(ADD(MUL(MUL(MUL(oa, inv_theta), 3.0), e1),
                                                  MUL(MUL(MUL(pa, inv_theta), 3.0), e2)),
                                              MUL(oj, e3)),
                                          MUL(pj, e4)));
              } else {
                b.acc[k] = 0.25 * (oa * (2 - 3 * tau + tau3) + pa * (2 + 3 * tau - tau3) +
                                   oj * theta * (1 - tau - tau2 + tau3) +
                                   pj * theta * (-1 - tau + tau2 + tau3));
                b.jerk[k] = 0.25 * (oa * inv_theta * 3 * (-1 + tau2) + pa * inv_theta * 3 * (1 - tau2) +
                                    oj * (-1 - 2 * tau + 3 * tau2) + pj * (-1 + 2 * tau + 3 * tau2));
              }
            }
            // correct_pos_and_vel(new_dt)
            if (EXACT) {
              b.pv[k] = SUB(ADD(b.vel[k], DIV(MUL(new_dt, ADD(b.acc[k], b.oacc[k])), 2.0)),
                            DIV(MUL(nd2, SUB(b.jerk[k], b.ojerk[k])), 12.0));
              b.pp[k] = SUB(ADD(b.pos[k], DIV(MUL(new_dt, ADD(b.pv[k], b.vel[k])), 2.0)),
                            DIV(MUL(nd2, SUB(b.acc[k], b.oacc[k])), 12.0));
            } else {
              b.pv[k] = b.vel[k] + new_dt * (b.acc[k] + b.oacc[k]) * 0.5 -
                        nd2 * (b.jerk[k] - b.ojerk[k]) * (1.0 / 12.0);
              b.pp[k] = b.pos[k] + new_dt * (b.pv[k] + b.vel[k]) * 0.5 -
                        nd2 * (b.acc[k] - b.oacc[k]) * (1.0 / 12.0);
            }
          }
        }
      }
#pragma unroll
      for (int qq = 0; qq < 2; qq++)
#pragma unroll
        for (int k = 0; k < 3; k++) {
          B[qq].pos[k] = B[qq].pp[k];
          B[qq].vel[k] = B[qq].pv[k];
        }
      dt = end_dt;
      t = EXACT ? ADD(t, new_dt) : t + new_dt;
      nsteps++;
    }
#pragma unroll
    for (int qq = 0; qq < 2; qq++) {
      const int i = lane + 32 * qq;
      if (i < n) {
#pragma unroll
        for (int k = 0; k < 3; k++) {
          pos[3 * (base + i) + k] = B[qq].pos[k];
          vel[3 * (base + i) + k] = B[qq].vel[k];
        }
      }
    }
    if (lane == 0) {
      unsigned long long t1;
      asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t1));
      t_out[s] = t;
      steps_out[s] = nsteps;
      wall_ns[s] = t1 - t0;
      status[s] = st;
    }
    __syncwarp();
  }
}

// ---------------------------------------------------------------------------
// Unperturbed binaries (smallN's default treatment: src/amuse_ph4/src/
// smallN.cc:1022-1060 and smallN_unpert.cc): after each step the pair that
// set the time step becomes a binary node when it is approaching, closer
// than r_crit, its step is below dt_crit and the strongest perturber's
// tidal parameter gamma^2 = 4 (m_k/M)^2 (r^2/d_k^2)^3 is below gamma^2_unpert
// (smallN_unpert.cc:44-88).  Its centre of mass is integrated like a body;
// its components follow the two-body orbit (universal-variable Kepler
// propagation) and are resolved for every force evaluation (forces between
// top-level nodes are sums over their leaves, smallN.cc:127-240; the step
// criterion takes the closest leaf pair with the nodes' masses and
// velocities).  The unperturbed segment ends at the time the orbit returns
// to the same separation past pericentre (smallN_unpert.cc:252-266, 335);
// there the change of the tidal potential is absorbed into the relative
// velocity, and the binary is either extended by whole periods (frozen
// components) while no perturber can arrive (dt_perturbers,
// smallN_unpert.cc:402-460, 682-704) or dissolved.  The same algorithm, with
// the same stated differences from smallN, is the oracle's
// orc_smalln_unpert.  FAST (FP64 pair terms) and SPLIT (FP32 pair terms)
// modes; all tree decisions are taken redundantly by every lane of the
// warp from shared data, so they are warp-uniform.
constexpr int NB = 8;             // binaries per system at most
constexpr int WARPS_MAX_UNP = 4;  // shared memory per warp is larger here

struct BinRec {
  int li, lj, full, pad;
  double mi, mj, r0[3], v0[3], t0, tpred, tidal;
  // the last Kepler solution (universal anomaly, its dt, the separation):
  // the next solve starts from it (dtw = 0: none yet)
  double xw, dtw, rw;
};

struct UnpParams {
  double dt_crit, r2_crit, gamma2, gamma_inv3;
  int allow_full;
};

struct UnpSmem {
  union {  // leaves for the force loop; node positions/velocities for the tree logic
    struct {
      double pp[MAXN][3];
      double pv[MAXN][3];
    } d;
    struct {
      float ph[MAXN][3];
      float pl[MAXN][3];
      float vf[MAXN][3];
    } f;
  } A;
  double la[MAXN][3], lj[MAXN][3];  // leaf forces, then node accelerations
  double m[MAXN];                    // leaf masses
  float mf[MAXN];
  double nm[MAXN];                   // node masses (at node slots)
  float nmf[MAXN];                   // the same in FP32 (split mode's step criterion)
  double cv[MAXN][3];                // node predicted velocities (at node slots)
  float cvf[MAXN][3];
  int nd[MAXN];                      // node (leader slot) of every leaf slot
  BinRec bin[NB];
  int nb;
};

// Stumpff functions C(z) = (1 - cos sqrt z) / z, S(z) = (sqrt z - sin sqrt z)
// / z^(3/2) (cosh, sinh for z < 0), both from one sincos (one exp) of
// sqrt(|z|) / 2: 1 - cos s = 2 sin^2(s/2) (no cancellation), sin s = 2
// sin(s/2) cos(s/2).  Taylor series to z^6 for |z| < 0.1 (below 1e-17
// relative).  FP64 transcendentals run at the FP64 rate, so one call per
// Newton step rather than two.
__device__ __forceinline__ void kst_cs(double z, double &C, double &S) {
  if (z > 0.1) {
    const double s = sqrt(z);
    double sh, ch;
    sincos(0.5 * s, &sh, &ch);
    C = 2.0 * sh * sh / z;
    S = (s - 2.0 * sh * ch) / (s * z);
  } else if (z < -0.1) {
    const double s = sqrt(-z), e = exp(0.5 * s), ei = 1.0 / e;
    const double sh = 0.5 * (e - ei), ch = 0.5 * (e + ei);
    C = 2.0 * sh * sh / -z;
    S = (2.0 * sh * ch - s) / (s * -z);
  } else {
    C = 1.0 / 2 +
        z * (-1.0 / 24 +
             z * (1.0 / 720 +
                  z * (-1.0 / 40320 +
                       z * (1.0 / 3628800 + z * (-1.0 / 479001600 + z / 87178291200.0)))));
    S = 1.0 / 6 +
        z * (-1.0 / 120 +
             z * (1.0 / 5040 +
                  z * (-1.0 / 362880 +
                       z * (1.0 / 39916800 + z * (-1.0 / 6227020800.0 + z / 1307674368000.0)))));
  }
}

// Two-body relative motion over dt (mu = G M), universal variables: the
// universal anomaly x solves
//   F(x) = (r0.v0 / sqrt(mu)) x^2 C(z) + (1 - alpha r0) x^3 S(z) + r0 x - sqrt(mu) dt = 0,
// z = alpha x^2, whose derivative is the separation r(x) > 0.  F being
// monotonic, the root is bracketed and found by Newton steps that fall back
// to bisection when a step leaves the bracket or does not halve the one
// before last (a plain Newton iteration diverges on eccentric orbits near
// pericentre).  The first guess is the mean-motion one, or, with a warm
// start (*dtw > 0: the solution xw at dtw, separation rw, of the same
// orbit), xw + sqrt(mu) (dt - dtw) / rw (dx/dt = sqrt(mu) / r); x grows with
// dt, so xw then also bounds the root from one side.  The C and S of the
// step whose correction is below 1e-15 x give the f and g functions.
__device__ void kep_prop(double mu, const double r0[3], const double v0[3], double dt,
                         double r[3], double v[3], double *xw = nullptr, double *dtw = nullptr,
                         double *rw = nullptr) {
  const double rn = sqrt(r0[0] * r0[0] + r0[1] * r0[1] + r0[2] * r0[2]);
  const double v2 = v0[0] * v0[0] + v0[1] * v0[1] + v0[2] * v0[2];
  const double rv = r0[0] * v0[0] + r0[1] * v0[1] + r0[2] * v0[2];
  const double alpha = 2.0 / rn - v2 / mu, smu = sqrt(mu);
  const double c1 = rv / smu, c2 = 1.0 - alpha * rn;
  if (dt == 0.0) {
    for (int k = 0; k < 3; k++) r[k] = r0[k], v[k] = v0[k];
    return;
  }
  auto Fx = [&](double x) {
    double C, S;
    kst_cs(alpha * x * x, C, S);
    return c1 * x * x * C + c2 * x * x * x * S + rn * x - smu * dt;
  };
  const bool warm = xw && *dtw > 0.0 && dt > 0.0;
  const double inf = __longlong_as_double(0x7ff0000000000000ll);
  double x0 = alpha > 0.0 ? smu * dt * alpha : smu * dt / rn;  // sign of dt
  double lo, hi;
  if (warm) {
    // The root lies above xw when dt >= dtw (F(xw) <= 0), else in (0, xw).
    // No evaluation before the first Newton step: with hi = +inf, steps from
    // below (F < 0, dF > 0) only move up, until one lands above the root and
    // bounds it.
    x0 = *xw + smu * (dt - *dtw) / *rw;
    lo = dt >= *dtw ? *xw : 0.0;
    hi = dt >= *dtw ? inf : *xw;
    if (!(x0 > lo && x0 < hi)) x0 = hi < inf ? 0.5 * (lo + hi) : lo + fabs(lo) + 1e-300;
  } else if (dt > 0.0) {
    lo = 0.0, hi = x0;
    for (int k = 0; k < 200 && Fx(hi) < 0.0; k++) lo = hi, hi *= 2.0;
  } else {
    hi = 0.0, lo = x0;
    for (int k = 0; k < 200 && Fx(lo) > 0.0; k++) hi = lo, lo *= 2.0;
  }
  double x = x0 > lo && x0 < hi ? x0 : 0.5 * (lo + hi);
  double step_old = hi - lo, step = step_old, C = 0.5, S = 1.0 / 6;
  for (int it = 0; it < 200; it++) {
    const double z = alpha * x * x;
    kst_cs(z, C, S);
    const double F = c1 * x * x * C + c2 * x * x * x * S + rn * x - smu * dt;
    const double dF = c1 * x * (1.0 - z * S) + c2 * x * x * C + rn;
    if (F == 0.0 || fabs(F) <= 1e-15 * fabs(x * dF)) break;  // x is the root: C, S belong to it
    if (F < 0.0)
      lo = x;
    else
      hi = x;
    double xn = x - F / dF;
    if (hi < inf && (!(xn > lo && xn < hi) || fabs(2.0 * F) > fabs(step_old * dF))) {
      step_old = step;
      step = 0.5 * (hi - lo);
      xn = lo + step;
    } else {
      step_old = step;
      step = F / dF;
    }
    if (xn == x) break;
    x = xn;
  }
  const double f = 1.0 - x * x * C / rn, g = dt - x * x * x * S / smu;
  for (int k = 0; k < 3; k++) r[k] = f * r0[k] + g * v0[k];
  const double rr = sqrt(r[0] * r[0] + r[1] * r[1] + r[2] * r[2]);
  const double fd = smu / (rr * rn) * (alpha * x * x * x * S - x), gd = 1.0 - x * x * C / rr;
  for (int k = 0; k < 3; k++) v[k] = fd * r0[k] + gd * v0[k];
  if (xw && dt > 0.0) {
    *xw = x;
    *dtw = dt;
    *rw = rr;
  }
}

// Time to the next pericentre (0: not approaching it) and the period (inf
// unless bound): mean anomaly from the eccentric (hyperbolic) anomaly;
// Barker's equation near e = 1.
__device__ int kep_peri(double mu, const double r[3], const double v[3], double *dt_peri,
                        double *period) {
  const double rn = sqrt(r[0] * r[0] + r[1] * r[1] + r[2] * r[2]);
  const double v2 = v[0] * v[0] + v[1] * v[1] + v[2] * v[2];
  const double rv = r[0] * v[0] + r[1] * v[1] + r[2] * v[2];
  *period = __longlong_as_double(0x7ff0000000000000ll);
  if (rv >= 0.0) return 0;
  const double alpha = 2.0 / rn - v2 / mu;
  const double h0 = r[1] * v[2] - r[2] * v[1], h1 = r[2] * v[0] - r[0] * v[2],
               h2 = r[0] * v[1] - r[1] * v[0];
  const double p = (h0 * h0 + h1 * h1 + h2 * h2) / mu;
  const double e = sqrt(fmax(0.0, 1.0 - p * alpha));
  if (fabs(alpha) * rn < 1e-8 || e < 1e-12) {
    const double D = rv / sqrt(mu * p);
    *dt_peri = -0.5 * sqrt(p * p * p / mu) * (D + D * D * D / 3.0);
    if (alpha > 0.0) *period = 2.0 * M_PI / sqrt(mu * alpha * alpha * alpha);
    return *dt_peri > 0.0;
  }
  double M, n;
  if (alpha > 0.0) {
    const double a = 1.0 / alpha;
    const double E = atan2(rv / (e * sqrt(mu * a)), (1.0 - rn * alpha) / e);
    M = E - e * sin(E);
    n = sqrt(mu * alpha * alpha * alpha);
    *period = 2.0 * M_PI / n;
  } else {
    const double sF = rv / (e * sqrt(-mu / alpha));
    M = e * sF - asinh(sF);
    n = sqrt(-mu * alpha * alpha * alpha);
  }
  if (M >= 0.0) return 0;
  *dt_peri = -M / n;
  return 1;
}

__device__ __forceinline__ double dist3(const double a[3], const double b[3]) {
  const double d0 = a[0] - b[0], d1 = a[1] - b[1], d2 = a[2] - b[2];
  return sqrt(d0 * d0 + d1 * d1 + d2 * d2);
}

// The relative state of a binary at time t (frozen when fully unperturbed).
__device__ __forceinline__ void bin_rel(const BinRec &b, double t, double r[3], double v[3]) {
  if (b.full) {
    for (int k = 0; k < 3; k++) r[k] = b.r0[k], v[k] = b.v0[k];
  } else {
    kep_prop(b.mi + b.mj, b.r0, b.v0, t - b.t0, r, v);
  }
}
// The same, starting the Kepler solve from the binary's last solution and
// keeping this one (the force evaluations: a few per step, at nearby times).
__device__ __forceinline__ void bin_rel_warm(BinRec &b, double t, double r[3], double v[3]) {
  if (b.full) {
    for (int k = 0; k < 3; k++) r[k] = b.r0[k], v[k] = b.v0[k];
  } else {
    kep_prop(b.mi + b.mj, b.r0, b.v0, t - b.t0, r, v, &b.xw, &b.dtw, &b.rw);
  }
}

// Warp-wide sum and minimum (xor butterfly: every lane ends with the same
// value, a + b being b + a).
__device__ __forceinline__ double warp_sum(double x) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) x += __shfl_xor_sync(0xffffffffu, x, o);
  return x;
}
__device__ __forceinline__ double warp_min(double x) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) x = fmin(x, __shfl_xor_sync(0xffffffffu, x, o));
  return x;
}

// Tidal potential of the other top-level nodes on leaves (xi, xj) around
// the centre of mass xc (smallN_unpert.cc:17-40); node positions in S.A.d.
// The whole warp calls it (uniform arguments); each lane sums its two node
// slots (the tree's loops over nodes run at 1/32 of the FP64 work per lane).
__device__ double tidal_pot(const UnpSmem &S, int n, int lane, int li, int lj, double mi,
                            double mj, const double xi[3], const double xj[3],
                            const double xc[3]) {
  double phi = 0.0;
#pragma unroll
  for (int q = 0; q < 2; q++) {
    const int k = lane + 32 * q;
    if (k >= n || S.nd[k] != k || k == li || k == lj) continue;
    phi += S.nm[k] * (-mi / dist3(xi, S.A.d.pp[k]) - mj / dist3(xj, S.A.d.pp[k]) +
                      (mi + mj) / dist3(xc, S.A.d.pp[k]));
  }
  return warp_sum(phi);
}

template <int MODE>
__device__ __forceinline__ void unp_store_leaf(UnpSmem &S, int s, const double x[3],
                                               const double v[3]) {
  if (MODE == MODE_SPLIT) {
    for (int k = 0; k < 3; k++) {
      const float h = __double2float_rn(x[k]);
      S.A.f.ph[s][k] = h;
      S.A.f.pl[s][k] = __double2float_rn(x[k] - (double)h);
      S.A.f.vf[s][k] = __double2float_rn(v[k]);
    }
  } else {
    for (int k = 0; k < 3; k++) S.A.d.pp[s][k] = x[k], S.A.d.pv[s][k] = v[k];
  }
}

// Resolved forces on the top-level nodes from the predicted states in B:
// returns the system's min step^2 (warp-uniform) and the node pair setting it.
template <int MODE>
__device__ double unp_forces(UnpSmem &S, int n, int lane, Body B[2], double t, int *imin,
                             int *jmin) {
  __syncwarp();
  // publish: node slots of this lane (singles: their leaf; leaders: both leaves)
#pragma unroll
  for (int q = 0; q < 2; q++) {
    const int s = lane + 32 * q;
    if (s >= n || S.nd[s] != s) continue;
    for (int k = 0; k < 3; k++) {
      S.cv[s][k] = B[q].pv[k];
      S.cvf[s][k] = __double2float_rn(B[q].pv[k]);
    }
    S.nm[s] = B[q].m;
    S.nmf[s] = __double2float_rn(B[q].m);
    int qb = -1;
    for (int b = 0; b < S.nb; b++)
      if (S.bin[b].li == s) qb = b;
    if (qb < 0) {
      unp_store_leaf<MODE>(S, s, B[q].pp, B[q].pv);
    } else {
      BinRec &bb = S.bin[qb];  // this lane's binary (its leader slot is the lane's)
      double r[3], v[3], xi[3], vi[3], xj[3], vj[3];
      bin_rel_warm(bb, t, r, v);
      const double M = bb.mi + bb.mj, fi = bb.mj / M, fj = bb.mi / M;
      for (int k = 0; k < 3; k++) {
        xi[k] = B[q].pp[k] - fi * r[k];
        vi[k] = B[q].pv[k] - fi * v[k];
        xj[k] = B[q].pp[k] + fj * r[k];
        vj[k] = B[q].pv[k] + fj * v[k];
      }
      unp_store_leaf<MODE>(S, bb.li, xi, vi);
      unp_store_leaf<MODE>(S, bb.lj, xj, vj);
    }
  }
  __syncwarp();
  double ts2 = __longlong_as_double(0x7ff0000000000000ll);
  int pmin = 0x7fffffff;  // node pair id a * MAXN + b (a < b) of ts2
  double la[2][3], lj[2][3];
#pragma unroll
  for (int q = 0; q < 2; q++) {
    const int i = lane + 32 * q;
    for (int k = 0; k < 3; k++) la[q][k] = lj[q][k] = 0.0;
    if (i >= n) continue;
    const int ni = S.nd[i];
    if (MODE == MODE_SPLIT) {
      // FP32 throughout the loop (FP64 runs at 1/64 of the FP32 rate): the
      // pairs within one node (the leaf itself, its binary companion) are
      // evaluated with their terms masked to zero and their step to +inf,
      // so the loop does not diverge; the smallest step and its node pair
      // are kept in FP32 and merged into the FP64 minimum afterwards.
      float a[3] = {0.f, 0.f, 0.f}, jk[3] = {0.f, 0.f, 0.f};
      float tsq = __int_as_float(0x7f800000);
      int pq = 0x7fffffff;
      for (int j = 0; j < n; j++) {
        const int nj = S.nd[j];
        const bool same = nj == ni;
        float dx[3], dv[3], dc[3];
        for (int k = 0; k < 3; k++) {
          dx[k] = __fadd_rn(__fsub_rn(S.A.f.ph[j][k], S.A.f.ph[i][k]),
                            __fsub_rn(S.A.f.pl[j][k], S.A.f.pl[i][k]));
          dv[k] = S.A.f.vf[j][k] - S.A.f.vf[i][k];
          dc[k] = S.cvf[nj][k] - S.cvf[ni][k];
        }
        const float d2 = fmaf(dx[2], dx[2], fmaf(dx[1], dx[1], dx[0] * dx[0]));
        const float v2 = fmaf(dc[2], dc[2], fmaf(dc[1], dc[1], dc[0] * dc[0]));
        const float mt = S.nmf[ni] + S.nmf[nj];
        float ts;
        if (same || d2 >= 1e-18f) {
          const float rinv = same ? 0.f : rsqrt_approx(d2);
          const float rinv2 = rinv * rinv;
          const float f = S.mf[j] * rinv * rinv2;
          const float xv = fmaf(dx[2], dv[2], fmaf(dx[1], dv[1], dx[0] * dv[0]));
          const float a3 = -3.0f * xv * rinv2;
          for (int k = 0; k < 3; k++) {
            a[k] = fmaf(f, dx[k], a[k]);
            jk[k] = fmaf(f, fmaf(a3, dx[k], dv[k]), jk[k]);
          }
          ts = same ? __int_as_float(0x7f800000)
                    : fminf(__fdividef(0.5f * d2 * (d2 * rinv), mt), __fdividef(d2, v2));
        } else {  // too close for FP32: FP64
          double X[3], W[3];
          for (int k = 0; k < 3; k++) X[k] = (double)dx[k], W[k] = (double)dv[k];
          const double dd2 = X[0] * X[0] + X[1] * X[1] + X[2] * X[2];
          const double d = sqrt(dd2), ri2 = 1.0 / dd2, fd = S.m[j] * ri2 / d;
          const double a3 = -3.0 * (X[0] * W[0] + X[1] * W[1] + X[2] * W[2]) * ri2;
          for (int k = 0; k < 3; k++) {
            la[q][k] += fd * X[k];
            lj[q][k] += fd * (a3 * X[k] + W[k]);
          }
          ts = (float)fmin(0.5 * dd2 * d / (double)mt, dd2 / (double)v2);
        }
        const int pid = ni < nj ? ni * MAXN + nj : nj * MAXN + ni;
        if (ts < tsq || (ts == tsq && pid < pq)) {
          tsq = ts;
          pq = pid;
        }
      }
      if ((double)tsq < ts2 || ((double)tsq == ts2 && pq < pmin)) {
        ts2 = (double)tsq;
        pmin = pq;
      }
      for (int k = 0; k < 3; k++) la[q][k] += (double)a[k], lj[q][k] += (double)jk[k];
    } else {
      for (int j = 0; j < n; j++) {
        const int nj = S.nd[j];
        if (nj == ni) continue;
        double dx[3], dv[3], dc[3];
        for (int k = 0; k < 3; k++) {
          dx[k] = S.A.d.pp[j][k] - S.A.d.pp[i][k];
          dv[k] = S.A.d.pv[j][k] - S.A.d.pv[i][k];
          dc[k] = S.cv[nj][k] - S.cv[ni][k];
        }
        const double d2 = dx[0] * dx[0] + dx[1] * dx[1] + dx[2] * dx[2];
        const double rinv = rsqrt64(d2);
        const double rinv2 = rinv * rinv;
        const double f = S.m[j] * rinv * rinv2;
        const double a3 = -3.0 * (dx[0] * dv[0] + dx[1] * dv[1] + dx[2] * dv[2]) * rinv2;
        for (int k = 0; k < 3; k++) {
          la[q][k] = fma(f, dx[k], la[q][k]);
          lj[q][k] = fma(f, fma(a3, dx[k], dv[k]), lj[q][k]);
        }
        const double v2 = dc[0] * dc[0] + dc[1] * dc[1] + dc[2] * dc[2];
        const double d3 = d2 * d2 * rinv;
        const double ts = fmin(0.5 * d3 / (S.nm[ni] + S.nm[nj]), d2 / v2);
        const int pid = ni < nj ? ni * MAXN + nj : nj * MAXN + ni;
        if (ts < ts2 || (ts == ts2 && pid < pmin)) {
          ts2 = ts;
          pmin = pid;
        }
      }
    }
  }
  __syncwarp();
#pragma unroll
  for (int q = 0; q < 2; q++) {
    const int i = lane + 32 * q;
    if (i < n)
      for (int k = 0; k < 3; k++) S.la[i][k] = la[q][k], S.lj[i][k] = lj[q][k];
  }
  __syncwarp();
  // node forces: mass-weighted leaf forces
#pragma unroll
  for (int q = 0; q < 2; q++) {
    const int s = lane + 32 * q;
    for (int k = 0; k < 3; k++) B[q].acc[k] = B[q].jerk[k] = 0.0;
    if (s >= n || S.nd[s] != s) continue;
    int qb = -1;
    for (int b = 0; b < S.nb; b++)
      if (S.bin[b].li == s) qb = b;
    if (qb < 0) {
      for (int k = 0; k < 3; k++) B[q].acc[k] = S.la[s][k], B[q].jerk[k] = S.lj[s][k];
    } else {
      const BinRec &bb = S.bin[qb];
      const double M = bb.mi + bb.mj;
      for (int k = 0; k < 3; k++) {
        B[q].acc[k] = (bb.mi * S.la[bb.li][k] + bb.mj * S.la[bb.lj][k]) / M;
        B[q].jerk[k] = (bb.mi * S.lj[bb.li][k] + bb.mj * S.lj[bb.lj][k]) / M;
      }
    }
  }
  for (int o = 16; o > 0; o >>= 1) {
    const double ot = __shfl_xor_sync(0xffffffffu, ts2, o);
    const int op = __shfl_xor_sync(0xffffffffu, pmin, o);
    if (ot < ts2 || (ot == ts2 && op < pmin)) {
      ts2 = ot;
      pmin = op;
    }
  }
  *imin = pmin == 0x7fffffff ? -1 : pmin / MAXN;
  *jmin = pmin == 0x7fffffff ? -1 : pmin % MAXN;
  return ts2;
}

// Node states (after a step) into shared memory for the tree logic: positions
// and velocities in A.d, accelerations in la, masses in nm.
__device__ __forceinline__ void unp_publish_nodes(UnpSmem &S, int n, int lane, const Body B[2]) {
  __syncwarp();
#pragma unroll
  for (int q = 0; q < 2; q++) {
    const int s = lane + 32 * q;
    if (s >= n || S.nd[s] != s) continue;
    for (int k = 0; k < 3; k++) {
      S.A.d.pp[s][k] = B[q].pos[k];
      S.A.d.pv[s][k] = B[q].vel[k];
      S.la[s][k] = B[q].acc[k];
    }
    S.nm[s] = B[q].m;
  }
  __syncwarp();
}

__device__ __forceinline__ void body_set(Body &b, double m, const double x[3], const double v[3]) {
  b.m = m;
  b.inv_m = 1.0 / m;
  for (int k = 0; k < 3; k++) {
    b.pos[k] = b.pp[k] = x[k];
    b.vel[k] = b.pv[k] = v[k];
    b.oacc[k] = b.ojerk[k] = 0.0;  // a node the tree has just made
  }
}

// The tree changes after a step (smallN.cc:1022-1060): binary creation from
// the pair that set the step, then the end of every segment due now.  Every
// lane evaluates the same decisions from shared data; lane 0 writes the
// shared records, the owners of the slots update their bodies.  Returns 0
// (no change), 1 (changed), 3 (changed, a binary made).
__device__ int unp_tree(UnpSmem &S, int n, int lane, Body B[2], double t, double dt_nat, int bim,
                        int bjm, const UnpParams &P) {
  unp_publish_nodes(S, n, lane, B);
  int changed = 0;
  // --- creation (is_unperturbed_and_approaching, create_binary)
  if (bim >= 0 && S.nb < NB && dt_nat <= P.dt_crit) {
    bool leaves = true;
    for (int b = 0; b < S.nb; b++)
      if (S.bin[b].li == bim || S.bin[b].li == bjm) leaves = false;
    const int i = bim, j = bjm;
    const double *xi = S.A.d.pp[i], *xj = S.A.d.pp[j], *vi = S.A.d.pv[i], *vj = S.A.d.pv[j];
    double r[3], v[3];
    for (int k = 0; k < 3; k++) r[k] = xj[k] - xi[k], v[k] = vj[k] - vi[k];
    const double d2 = r[0] * r[0] + r[1] * r[1] + r[2] * r[2];
    const double rv = r[0] * v[0] + r[1] * v[1] + r[2] * v[2];
    if (leaves && d2 <= P.r2_crit && rv <= 0.0) {
      const double mi = S.nm[i], mj = S.nm[j], M = mi + mj;
      double cm[3], cmv[3];
      for (int k = 0; k < 3; k++) {
        cm[k] = (mi * xi[k] + mj * xj[k]) / M;
        cmv[k] = (mi * vi[k] + mj * vj[k]) / M;
      }
      // the strongest perturber (largest m^2 / d^2 from the CM; the first
      // node on ties): each lane its two node slots, then a warp argmax
      double maxp = 0.0, nnd2 = 0.0, mk = 0.0;
      int kk = 0x7fffffff;
#pragma unroll
      for (int q = 0; q < 2; q++) {
        const int k2 = lane + 32 * q;
        if (k2 >= n || S.nd[k2] != k2 || k2 == i || k2 == j) continue;
        double e2 = 0.0;
        for (int k = 0; k < 3; k++) e2 += (S.A.d.pp[k2][k] - cm[k]) * (S.A.d.pp[k2][k] - cm[k]);
        const double p2 = S.nm[k2] * S.nm[k2] / e2;
        if (p2 > maxp) maxp = p2, nnd2 = e2, mk = S.nm[k2], kk = k2;
      }
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) {
        const double op = __shfl_xor_sync(0xffffffffu, maxp, o);
        const double od = __shfl_xor_sync(0xffffffffu, nnd2, o);
        const double om = __shfl_xor_sync(0xffffffffu, mk, o);
        const int ok = __shfl_xor_sync(0xffffffffu, kk, o);
        if (op > maxp || (op == maxp && ok < kk)) maxp = op, nnd2 = od, mk = om, kk = ok;
      }
      bool unp = true;
      if (maxp > 0.0) {
        const double q = d2 / nnd2;
        unp = 4.0 * (mk / M) * (mk / M) * q * q * q < P.gamma2;
      }
      double dtp, per;
      if (unp && kep_peri(M, r, v, &dtp, &per)) {
        double pxi[3], pxj[3];
        for (int k = 0; k < 3; k++) pxi[k] = xi[k], pxj[k] = xj[k];
        const double tid = tidal_pot(S, n, lane, i, j, mi, mj, pxi, pxj, cm);
        __syncwarp();
        if (lane == 0) {
          BinRec &b = S.bin[S.nb];
          b.li = i;
          b.lj = j;
          b.full = 0;
          b.mi = mi;
          b.mj = mj;
          for (int k = 0; k < 3; k++) b.r0[k] = r[k], b.v0[k] = v[k];
          b.t0 = t;
          b.dtw = 0.0;
          b.tpred = 2.0 * (t + dtp) - t;
          b.tidal = tid;
          S.nd[j] = i;
          S.nm[i] = M;
          for (int k = 0; k < 3; k++) S.A.d.pp[i][k] = cm[k], S.A.d.pv[i][k] = cmv[k];
          S.nb++;
        }
#pragma unroll
        for (int q = 0; q < 2; q++)
          if (lane + 32 * q == i) body_set(B[q], M, cm, cmv);
        __syncwarp();
        changed = 3;
      }
    }
  }
  // --- segments ending now (extend_or_end_binary)
  for (int qb = 0; qb < S.nb; qb++) {
    const BinRec bb = S.bin[qb];
    if (bb.tpred > t) continue;
    const int i = bb.li, j = bb.lj;
    const double M = bb.mi + bb.mj;
    double r[3], v[3], xi[3], xj[3], xc[3], vc[3];
    BinRec bw = bb;  // warm-started solve on a copy (every lane, same values)
    bin_rel_warm(bw, t, r, v);
    for (int k = 0; k < 3; k++) xc[k] = S.A.d.pp[i][k], vc[k] = S.A.d.pv[i][k];
    for (int k = 0; k < 3; k++) {
      xi[k] = xc[k] - bb.mj / M * r[k];
      xj[k] = xc[k] + bb.mi / M * r[k];
    }
    const double tid = tidal_pot(S, n, lane, i, j, bb.mi, bb.mj, xi, xj, xc);
    if (!bb.full) {
      const double mu = bb.mi * bb.mj / M, v2 = v[0] * v[0] + v[1] * v[1] + v[2] * v[2];
      const double fac = 1.0 - 2.0 * (tid - bb.tidal) / (mu * v2);
      if (fac > 0.0) {
        const double sf = sqrt(fac);
        for (int k = 0; k < 3; k++) v[k] *= sf;
      }
    }
    const double rn = sqrt(r[0] * r[0] + r[1] * r[1] + r[2] * r[2]);
    const double alpha = 2.0 / rn - (v[0] * v[0] + v[1] * v[1] + v[2] * v[2]) / M;
    double dtp = -1.0, period = __longlong_as_double(0x7ff0000000000000ll);
    if (P.allow_full && alpha > 0.0) {
      const double a = 1.0 / alpha;
      period = 2.0 * M_PI / sqrt(M * alpha * alpha * alpha);
      // time for any other node to come within the perturbation radius
      // (dt_perturbers): each lane its two node slots, then a warp minimum
      dtp = __longlong_as_double(0x7ff0000000000000ll);
#pragma unroll
      for (int q = 0; q < 2; q++) {
        const int k2 = lane + 32 * q;
        if (k2 >= n || S.nd[k2] != k2 || k2 == i) continue;
        const double rp = P.gamma_inv3 * a * cbrt(2.0 * S.nm[k2] / M);
        double dp[3], dvl[3], da[3];
        for (int k = 0; k < 3; k++) {
          dp[k] = S.A.d.pp[k2][k] - xc[k];
          dvl[k] = S.A.d.pv[k2][k] - vc[k];
          da[k] = S.la[k2][k] - S.la[i][k];
        }
        const double dr = sqrt(dp[0] * dp[0] + dp[1] * dp[1] + dp[2] * dp[2]);
        const double vr = (dvl[0] * dp[0] + dvl[1] * dp[1] + dvl[2] * dp[2]) / dr;
        const double ar = (da[0] * dp[0] + da[1] * dp[1] + da[2] * dp[2]) / dr;
        const double dd = dr - rp;
        double tr = 0.0;  // time_to_radius (smallN_unpert.cc:367-392)
        if (dd > 0.0) {
          tr = __longlong_as_double(0x7ff0000000000000ll);
          if (vr < 0.0) tr = -dd / vr;
          if (ar < 0.0) tr = fmin(tr, sqrt(-2.0 * dd / ar));
        }
        if (tr < dtp) dtp = tr;
      }
      dtp = 0.5 * warp_min(dtp);
    }
    __syncwarp();
    if (dtp >= period) {  // extend by whole periods, components frozen
      if (lane == 0) {
        BinRec &b = S.bin[qb];
        b.tpred += floor(dtp / period) * period;
        b.full = 1;
        b.tidal = tid;
        for (int k = 0; k < 3; k++) b.r0[k] = r[k], b.v0[k] = v[k];
        b.t0 = t;
        b.dtw = 0.0;
      }
      __syncwarp();
      continue;
    }
    // dissolve: the components become top-level nodes again
    double yi[3], yj[3], wi[3], wj[3];
    for (int k = 0; k < 3; k++) {
      yi[k] = xc[k] - bb.mj / M * r[k];
      yj[k] = xc[k] + bb.mi / M * r[k];
      wi[k] = vc[k] - bb.mj / M * v[k];
      wj[k] = vc[k] + bb.mi / M * v[k];
    }
#pragma unroll
    for (int q = 0; q < 2; q++) {
      if (lane + 32 * q == i) body_set(B[q], bb.mi, yi, wi);
      if (lane + 32 * q == j) body_set(B[q], bb.mj, yj, wj);
    }
    __syncwarp();
    if (lane == 0) {
      for (int k = 0; k < 3; k++) {
        S.A.d.pp[i][k] = yi[k];
        S.A.d.pv[i][k] = wi[k];
        S.A.d.pp[j][k] = yj[k];
        S.A.d.pv[j][k] = wj[k];
      }
      S.nd[j] = j;
      S.nm[i] = bb.mi;
      S.nm[j] = bb.mj;
      S.bin[qb] = S.bin[S.nb - 1];
      S.nb--;
    }
    __syncwarp();
    qb--;
    changed |= 1;
  }
  return changed;
}

template <int MODE>
__global__ void batch_unp_kernel(const int *__restrict__ order, const int *__restrict__ off,
                                 const double *__restrict__ t_end_s, const double *__restrict__ mass,
                                 double *pos, double *vel, double eta, int n_iter,
                                 long long max_steps, int *queue, double *t_out,
                                 long long *steps_out, unsigned long long *wall_ns, int *status,
                                 int *nbin_out, UnpParams P) {
  __shared__ UnpSmem smem[WARPS_MAX_UNP];
  const int lane = threadIdx.x & 31;
  const int w = threadIdx.x >> 5;
  UnpSmem &S = smem[w];
  const int nsys = queue[1];  // written by the host before the launch
  while (true) {
    int qq0 = 0;
    if (lane == 0) qq0 = atomicAdd(queue, 1);
    qq0 = __shfl_sync(0xffffffffu, qq0, 0);
    if (qq0 >= nsys) break;
    const int s = order[qq0];
    unsigned long long t0;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t0));
    const int base = off[s];
    const int n = off[s + 1] - base;
    const double t_end = t_end_s[s];
    if (n < 2 || n > MAXN) {
      if (lane == 0) {
        status[s] = 2;
        steps_out[s] = 0;
        t_out[s] = 0.0;
        nbin_out[s] = 0;
      }
      continue;
    }
    Body B[2];
    __syncwarp();
#pragma unroll
    for (int q = 0; q < 2; q++) {
      const int i = lane + 32 * q;
      const int ii = i < n ? i : 0;
      double x[3], v[3];
      for (int k = 0; k < 3; k++) x[k] = pos[3 * (base + ii) + k], v[k] = vel[3 * (base + ii) + k];
      body_set(B[q], mass[base + ii], x, v);
      if (i < n) {
        S.m[i] = B[q].m;
        S.mf[i] = __double2float_rn(B[q].m);
        S.nd[i] = i;
      }
    }
    if (lane == 0) S.nb = 0;
    __syncwarp();
    int bim, bjm, made = 0;
    double t = 0.0;
    double dt = eta * sqrt(unp_forces<MODE>(S, n, lane, B, t, &bim, &bjm));
    long long nsteps = 0;
    int st = 0;
    while (t < t_end) {
      if (nsteps >= max_steps) {
        st = 1;
        break;
      }
      double lim = __longlong_as_double(0x7ff0000000000000ll);
      for (int b = 0; b < S.nb; b++) lim = fmin(lim, S.bin[b].tpred - t);
      int nit = n_iter;
      if (dt >= lim) {
        dt = lim;
        nit = 0;
      }
      // predict_loworder (hdyn.h:192-201: with the stored old force)
      const double h = dt, h3 = h / 3.0, h2 = h * 0.5;
#pragma unroll
      for (int q = 0; q < 2; q++) {
        if (lane + 32 * q >= n || S.nd[lane + 32 * q] != lane + 32 * q) continue;
        for (int k = 0; k < 3; k++) {
          const double oj = B[q].ojerk[k], oa = B[q].oacc[k];
          B[q].pp[k] = fma(fma(fma(oj, h3, oa), h2, B[q].vel[k]), h, B[q].pos[k]);
          B[q].pv[k] = fma(fma(oj, h2, oa), h, B[q].vel[k]);
        }
      }
#pragma unroll
      for (int q = 0; q < 2; q++)
        for (int k = 0; k < 3; k++) B[q].oacc[k] = B[q].acc[k], B[q].ojerk[k] = B[q].jerk[k];
      double new_dt = dt, end_dt = dt;
      for (int it = 0; it <= nit; it++) {
        const double prev = new_dt;
        const double ts2 = unp_forces<MODE>(S, n, lane, B, t + new_dt, &bim, &bjm);
        end_dt = eta * sqrt(ts2);
        if (it < nit) {
          new_dt = 0.5 * (dt + end_dt);
          new_dt = dt + 0.5 * (end_dt - dt) * (new_dt / prev);
          if (new_dt >= lim) {
            new_dt = lim;
            nit = 0;
          }
        }
        const bool cj = new_dt != prev;
        double tau = 0, tau2 = 0, tau3 = 0, theta = 0, inv_theta = 0;
        if (cj) {
          theta = 0.5 * prev;
          tau = (new_dt - theta) / theta;
          inv_theta = 1.0 / theta;
          tau2 = tau * tau;
          tau3 = tau2 * tau;
        }
        const double nd2 = new_dt * new_dt;
#pragma unroll
        for (int q = 0; q < 2; q++) {
          Body &b = B[q];
          for (int k = 0; k < 3; k++) {
            if (cj) {
              const double pa = b.acc[k], pj = b.jerk[k], oa = b.oacc[k], oj = b.ojerk[k];
              b.acc[k] = 0.25 * (oa * (2 - 3 * tau + tau3) + pa * (2 + 3 * tau - tau3) +
                                 oj * theta * (1 - tau - tau2 + tau3) +
                                 pj * theta * (-1 - tau + tau2 + tau3));
              b.jerk[k] = 0.25 * (oa * inv_theta * 3 * (-1 + tau2) + pa * inv_theta * 3 * (1 - tau2) +
                                  oj * (-1 - 2 * tau + 3 * tau2) + pj * (-1 + 2 * tau + 3 * tau2));
            }
            b.pv[k] = b.vel[k] + new_dt * (b.acc[k] + b.oacc[k]) * 0.5 -
                      nd2 * (b.jerk[k] - b.ojerk[k]) * (1.0 / 12.0);
            b.pp[k] = b.pos[k] + new_dt * (b.pv[k] + b.vel[k]) * 0.5 -
                      nd2 * (b.acc[k] - b.oacc[k]) * (1.0 / 12.0);
          }
        }
      }
#pragma unroll
      for (int q = 0; q < 2; q++)
        for (int k = 0; k < 3; k++) B[q].pos[k] = B[q].pp[k], B[q].vel[k] = B[q].pv[k];
      dt = end_dt;
      t = t + new_dt;
      nsteps++;
      const int tc = unp_tree(S, n, lane, B, t, dt, bim, bjm, P);
      if (tc) {
        if (tc & 2) made++;
        dt = eta * sqrt(unp_forces<MODE>(S, n, lane, B, t, &bim, &bjm));
      }
    }
    // resolve the binaries left at the end into their components
    __syncwarp();
#pragma unroll
    for (int q = 0; q < 2; q++) {
      const int i = lane + 32 * q;
      if (i >= n || S.nd[i] != i) continue;
      int qb = -1;
      for (int b = 0; b < S.nb; b++)
        if (S.bin[b].li == i) qb = b;
      if (qb < 0) {
        for (int k = 0; k < 3; k++) {
          pos[3 * (base + i) + k] = B[q].pos[k];
          vel[3 * (base + i) + k] = B[q].vel[k];
        }
      } else {
        const BinRec &bb = S.bin[qb];
        double r[3], v[3];
        bin_rel(bb, t, r, v);
        const double M = bb.mi + bb.mj;
        for (int k = 0; k < 3; k++) {
          pos[3 * (base + bb.li) + k] = B[q].pos[k] - bb.mj / M * r[k];
          vel[3 * (base + bb.li) + k] = B[q].vel[k] - bb.mj / M * v[k];
          pos[3 * (base + bb.lj) + k] = B[q].pos[k] + bb.mi / M * r[k];
          vel[3 * (base + bb.lj) + k] = B[q].vel[k] + bb.mi / M * v[k];
        }
      }
    }
    if (lane == 0) {
      unsigned long long t1;
      asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t1));
      t_out[s] = t;
      steps_out[s] = nsteps;
      wall_ns[s] = t1 - t0;
      status[s] = st;
      nbin_out[s] = made;
    }
    __syncwarp();
  }
}

__global__ void queue_reset(int *queue) { queue[0] = 0; }

}  // namespace

extern "C" int g6k_batch_max_n(void) { return MAXN; }

// One persistent launch: grid = ctas_per_sm * SMs, warps_per_cta warps each.
// Resets the queue counter first (same stream), so the pair can be captured
// in a CUDA graph and replayed.  queue[0] is the counter, queue[1] the number
// of systems, which the host writes before each replay (a graph then serves
// every batch size).
extern "C" int g6k_batch_launch(const int *order, const int *off, const double *t_end,
                                const double *mass, double *pos, double *vel, double eta,
                                int n_iter, long long max_steps, int exact, int warps_per_cta,
                                int ctas, int *queue, double *t_out, long long *steps_out,
                                unsigned long long *wall_ns, int *status, cudaStream_t st) {
  if (warps_per_cta < 1 || warps_per_cta > WARPS_MAX || ctas < 1) return -2;
  if (exact < MODE_FAST || exact > MODE_SPLIT) return -2;
  queue_reset<<<1, 1, 0, st>>>(queue);
#define G6_BATCH(M)                                                                           \
  batch_kernel<M><<<ctas, 32 * warps_per_cta, 0, st>>>(order, off, t_end, mass, pos, vel,       \
                                                       eta, n_iter, max_steps, queue, t_out,    \
                                                       steps_out, wall_ns, status)
  if (exact == MODE_EXACT)
    G6_BATCH(MODE_EXACT);
  else if (exact == MODE_SPLIT)
    G6_BATCH(MODE_SPLIT);
  else
    G6_BATCH(MODE_FAST);
#undef G6_BATCH
  return cudaGetLastError() == cudaSuccess ? 0 : -3;
}

// The same with smallN's unperturbed binaries (FAST or SPLIT pair terms):
// dt_crit, r2_crit, gamma and allow_full as smallN's set_dt_crit,
// set_r2_crit, set_gamma, set_allow_full_unperturbed; nbin_out[s] counts the
// binaries made in system s.
extern "C" int g6k_batch_launch_unp(const int *order, const int *off,
                                    const double *t_end, const double *mass, double *pos,
                                    double *vel, double eta, int n_iter, long long max_steps,
                                    int mode, int warps_per_cta, int ctas, double dt_crit,
                                    double r2_crit, double gamma, int allow_full, int *queue,
                                    double *t_out, long long *steps_out,
                                    unsigned long long *wall_ns, int *status, int *nbin_out,
                                    cudaStream_t st) {
  if (warps_per_cta < 1 || warps_per_cta > WARPS_MAX_UNP || ctas < 1) return -2;
  if (mode != MODE_FAST && mode != MODE_SPLIT) return -2;
  UnpParams P;
  P.dt_crit = dt_crit;
  P.r2_crit = r2_crit;
  P.gamma2 = gamma * gamma;
  P.gamma_inv3 = pow(fmax(P.gamma2, 1e-120), -1.0 / 6.0);
  P.allow_full = allow_full;
  queue_reset<<<1, 1, 0, st>>>(queue);
  if (mode == MODE_SPLIT)
    batch_unp_kernel<MODE_SPLIT><<<ctas, 32 * warps_per_cta, 0, st>>>(
        order, off, t_end, mass, pos, vel, eta, n_iter, max_steps, queue, t_out, steps_out,
        wall_ns, status, nbin_out, P);
  else
    batch_unp_kernel<MODE_FAST><<<ctas, 32 * warps_per_cta, 0, st>>>(
        order, off, t_end, mass, pos, vel, eta, n_iter, max_steps, queue, t_out, steps_out,
        wall_ns, status, nbin_out, P);
  return cudaGetLastError() == cudaSuccess ? 0 : -3;
}
