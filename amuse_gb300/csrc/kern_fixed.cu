// kern_fixed.cu -- fixed-step Hermite integration and its adjoint.
//
// Forward step (the hermite code's scheme, src/amuse_hermite/interface.cc:
// predict_step :266-281, correct_step :536-552), state (x, v, a, j), step h:
//   xp = x + v h + a h^2/2 + j h^3/6,   vp = v + a h + j h^2/2
//   (a1, j1) = F(xp, vp; m)              (the library's force kernel)
//   v' = v + (a + a1) h/2 + (j - j1) h^2/12
//   x' = x + (v + v') h/2 + (a - a1) h^2/12,   (a, j) <- (a1, j1)
// F is ph4's pair force: a_k = sum_j m_j r s^-3/2, j_k = sum_j m_j (v s^-3/2
// - 3 (r.v) r s^-5/2), r = x_j - x_k, v = v_j - v_k, s = r^2 + eps^2.
//
// Adjoint of one step, given the adjoints (Lx', Lv', La', Lj') of its
// outputs (exact-arithmetic derivative of the map above):
//   Lvt = Lv' + Lx' h/2
//   La1 = La' - Lx' h^2/12 + Lvt h/2,   Lj1 = Lj' - Lvt h^2/12
//   (gxp, gvp, gm) = VJP_F(xp, vp, m; La1, Lj1)
//   Lx = Lx' + gxp
//   Lv = Lx' h/2 + Lvt + gxp h + gvp
//   La = Lx' h^2/12 + Lvt h/2 + gxp h^2/2 + gvp h
//   Lj = Lvt h^2/12 + gxp h^3/6 + gvp h^2/2,     Lm += gm
// Force VJP for body k, from its side of each pair (r = x_j - x_k, ...):
//   c = m_k Lam_j - m_j Lam_k  (Lam = (La1, Lj1)),  lam = c_a, mu = c_j
//   gx_k += lam s^-3/2 - 3 (r.lam) r s^-5/2
//           - 3 [(mu.v) r + (mu.r) v + (r.v) mu] s^-5/2 + 15 (r.v)(mu.r) r s^-7/2
//   gv_k += mu s^-3/2 - 3 (r.mu) r s^-5/2
//   gm_k -= La1_j . r s^-3/2 + Lj1_j . (v s^-3/2 - 3 (r.v) r s^-5/2)
// (the pair Jacobians are even in (r, v), which gives the c combination).
// With the hermite code's jerk form (r.v divided by the unsoftened q = r^2,
// src/amuse_hermite/interface.cc:440-449,486) the jerk terms become
//   gx_k += -3 (mu.v) r s^-5/2 - 3 [(mu.r) v + (r.v) mu] q^-1 s^-3/2
//           + 3 (r.v)(mu.r) r (2 q^-2 s^-3/2 + 3 q^-1 s^-5/2)
//   gv_k += mu s^-3/2 - 3 (r.mu) r q^-1 s^-3/2
//   gm_k -= ... + Lj1_j . (v s^-3/2 - 3 (r.v) r q^-1 s^-3/2)
// (q = s recovers the softened form).
// The VJP runs in split precision (double-single r, FP32 pair math, per-tile
// FP32 partials folded into FP64 totals) or in FP64.
#include <cuda_runtime.h>

#include "f32x2.cuh"
#include "g6_dev.h"

struct __align__(32) G6D4 {
  double x, y, z, w;
};

namespace {

constexpr int PT = 256;
constexpr int VT = 128;  // VJP threads per CTA
constexpr int VTILE = 128;

__global__ void records_kernel(int n, int n_pad, const double *__restrict__ x,
                               const double *__restrict__ v, const double *__restrict__ m,
                               int prec, void *jp_split, void *jp_f64) {
  const int s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= n_pad) return;
  double xp[3], vp[3], mm;
  if (s < n) {
    for (int k = 0; k < 3; k++) {
      xp[k] = x[3 * s + k];
      vp[k] = v[3 * s + k];
    }
    mm = m[s];
  } else {
    for (int k = 0; k < 3; k++) {
      xp[k] = 1.0e18;
      vp[k] = 0.0;
    }
    mm = 0.0;
  }
  if (prec == G6_PREC_FP64) {
    G6D4 *r = reinterpret_cast<G6D4 *>(jp_f64) + 2 * (size_t)s;
    r[0] = G6D4{xp[0], xp[1], xp[2], mm};
    r[1] = G6D4{vp[0], vp[1], vp[2], 0.0};
  } else {
    float h[3], l[3];
    for (int k = 0; k < 3; k++) {
      h[k] = __double2float_rn(xp[k]);
      l[k] = __double2float_rn(xp[k] - (double)h[k]);
    }
    const float mh = __double2float_rn(mm);
    g6_split_store(jp_split, s, h[0], h[1], h[2], mh, __double2float_rn(mm - (double)mh), l[0],
                   l[1], l[2], __double2float_rn(vp[0]), __double2float_rn(vp[1]),
                   __double2float_rn(vp[2]));
  }
}

__global__ void predict_kernel(int n, double h, const double *__restrict__ x,
                               const double *__restrict__ v, const double *__restrict__ a,
                               const double *__restrict__ j, double *xp, double *vp) {
  const int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= 3 * n) return;
  // hermite predict_step: pos += vel*dt + acc*dt*dt/2 + jerk*dt*dt*dt/6
  xp[e] = x[e] + (v[e] * h + a[e] * h * h / 2 + j[e] * h * h * h / 6);
  vp[e] = v[e] + (a[e] * h + j[e] * h * h / 2);
}

__global__ void correct_kernel(int n, double h, double *x, double *v, double *a, double *j,
                               const double *__restrict__ a1, const double *__restrict__ j1) {
  const int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= 3 * n) return;
  const double v0 = v[e], a0 = a[e], jj0 = j[e], an = a1[e], jn = j1[e];
  // hermite correct_step
  const double vn = v0 + (a0 + an) * h / 2 + (jj0 - jn) * h * h / 12;
  x[e] = x[e] + (v0 + vn) * h / 2 + (a0 - an) * h * h / 12;
  v[e] = vn;
  a[e] = an;
  j[e] = jn;
}

// Adjoint, first half: step-output adjoints in (lx, lv, la, lj) become the
// corrector's input-adjoint contributions (in place); la1/lj1 receive the
// adjoints of the force outputs (the VJP's cotangents).
__global__ void adj_pre_kernel(int n, double h, double *lx, double *lv, double *la, double *lj,
                               double *la1, double *lj1) {
  const int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= 3 * n) return;
  const double Lx = lx[e], Lv = lv[e], La = la[e], Lj = lj[e];
  const double Lvt = Lv + Lx * h / 2;
  la1[e] = La - Lx * h * h / 12 + Lvt * h / 2;
  lj1[e] = Lj - Lvt * h * h / 12;
  lx[e] = Lx;
  lv[e] = Lx * h / 2 + Lvt;
  la[e] = Lx * h * h / 12 + Lvt * h / 2;
  lj[e] = Lvt * h * h / 12;
}

// Adjoint, second half: add the predictor's pull-back of (gxp, gvp).
// lm (if not NULL) accumulates the mass cotangent gm.
__global__ void adj_post_kernel(int n, double h, double *lx, double *lv, double *la, double *lj,
                                const double *__restrict__ gxp, const double *__restrict__ gvp,
                                double *lm, const double *__restrict__ gm) {
  const int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= 3 * n) return;
  if (lm && e < n) lm[e] += gm[e];
  const double gx = gxp[e], gv = gvp[e];
  lx[e] += gx;
  lv[e] += gx * h + gv;
  la[e] += gx * h * h / 2 + gv * h;
  lj[e] += gx * h * h * h / 6 + gv * h * h / 2;
}

// ---- force VJP, FP64 ----
struct VRecD {
  double x[3], v[3], m, la[3], lj[3];
};

// One body k per thread, j in shared-memory tiles of VTILE, the j range
// split over gridDim.y CTA rows; m < 0 marks padding.
template <bool HJ>
__global__ void __launch_bounds__(VT) vjp_f64_kernel(int n, double eps2,
                                                     const double *__restrict__ x,
                                                     const double *__restrict__ v,
                                                     const double *__restrict__ m,
                                                     const double *__restrict__ la1,
                                                     const double *__restrict__ lj1, int jsplit,
                                                     double *part /* [nsplit][n][7] */) {
  __shared__ VRecD td[VTILE];
  eps2 += 1.0 / 4503599627370496.0;  // the force kernel's softening (+2^-52, as ph4)
  const int k = blockIdx.x * VT + threadIdx.x;
  const bool valid = k < n;
  const int kk = valid ? k : 0;
  const int j0 = blockIdx.y * jsplit;
  const int j1 = min(n, j0 + jsplit);
  const double xk[3] = {x[3 * kk], x[3 * kk + 1], x[3 * kk + 2]};
  const double vk[3] = {v[3 * kk], v[3 * kk + 1], v[3 * kk + 2]};
  const double mk = m[kk];
  const double lak[3] = {la1[3 * kk], la1[3 * kk + 1], la1[3 * kk + 2]};
  const double ljk[3] = {lj1[3 * kk], lj1[3 * kk + 1], lj1[3 * kk + 2]};
  double tot[7] = {0, 0, 0, 0, 0, 0, 0};  // gx[3], gv[3], gm
  for (int t0 = j0; t0 < j1; t0 += VTILE) {
    __syncthreads();
    for (int q = threadIdx.x; q < VTILE; q += VT) {
      const int jj = t0 + q;
      VRecD &r = td[q];
      if (jj < j1) {
        for (int c = 0; c < 3; c++) {
          r.x[c] = x[3 * jj + c];
          r.v[c] = v[3 * jj + c];
          r.la[c] = la1[3 * jj + c];
          r.lj[c] = lj1[3 * jj + c];
        }
        r.m = m[jj];
      } else {
        for (int c = 0; c < 3; c++) r.x[c] = r.v[c] = r.la[c] = r.lj[c] = 0.0;
        r.m = -1.0;
      }
    }
    __syncthreads();
    double acc[7] = {0, 0, 0, 0, 0, 0, 0};
    for (int q = 0; q < VTILE; q++) {
      const VRecD &r = td[q];
      if (r.m < 0.0 || t0 + q == k) continue;
      double R[3], V[3], lam[3], mu[3];
      for (int c = 0; c < 3; c++) {
        R[c] = r.x[c] - xk[c];
        V[c] = r.v[c] - vk[c];
        lam[c] = mk * r.la[c] - r.m * lak[c];
        mu[c] = mk * r.lj[c] - r.m * ljk[c];
      }
      const double s = R[0] * R[0] + R[1] * R[1] + R[2] * R[2] + eps2;
      const double si = 1.0 / s, s1 = sqrt(si);
      const double s3 = s1 * si, s5 = s3 * si, s7 = s5 * si;
      const double rl = R[0] * lam[0] + R[1] * lam[1] + R[2] * lam[2];
      const double rm = R[0] * mu[0] + R[1] * mu[1] + R[2] * mu[2];
      const double vm = V[0] * mu[0] + V[1] * mu[1] + V[2] * mu[2];
      const double rv = R[0] * V[0] + R[1] * V[1] + R[2] * V[2];
      // qs = q^-1 s^-3/2 (s^-5/2 in the softened form), c7 = 15 s^-7/2 resp.
      // 3 (2 q^-2 s^-3/2 + 3 q^-1 s^-5/2)
      double qs, c7;
      if (HJ) {
        const double qi = 1.0 / (R[0] * R[0] + R[1] * R[1] + R[2] * R[2]);
        qs = qi * s3;
        c7 = 3.0 * (2.0 * qi * qs + 3.0 * qi * s5);
      } else {
        qs = s5;
        c7 = 15.0 * s7;
      }
      const double cr = -3.0 * (rl * s5 + vm * s5) + rv * rm * c7;
      for (int c = 0; c < 3; c++) {
        acc[c] += lam[c] * s3 + cr * R[c] - 3.0 * qs * (rm * V[c] + rv * mu[c]);
        acc[3 + c] += mu[c] * s3 - 3.0 * rm * qs * R[c];
      }
      const double ga = (r.la[0] * R[0] + r.la[1] * R[1] + r.la[2] * R[2]) * s3;
      const double lv = r.lj[0] * V[0] + r.lj[1] * V[1] + r.lj[2] * V[2];
      const double lr = r.lj[0] * R[0] + r.lj[1] * R[1] + r.lj[2] * R[2];
      acc[6] -= ga + lv * s3 - 3.0 * rv * lr * qs;
    }
    for (int c = 0; c < 7; c++) tot[c] += acc[c];
  }
  if (valid) {
    double *p = part + ((size_t)blockIdx.y * n + k) * 7;
    for (int c = 0; c < 7; c++) p[c] = tot[c];
  }
}

// ---- split-precision force VJP, packed f32x2, register-blocked ----
// Records come in pairs of consecutive bodies, every field a float2 (body
// 2p, body 2p+1), 128 B per pair: xh yh zh m xl yl zl vx vy vz la0 la1 la2
// lj0 lj1 lj2.  Each add/sub/mul/fma.rn.f32x2 evaluates one body k against
// two bodies j; each thread owns VIPT bodies k (values duplicated into both
// halves), so every shared-memory record pair serves 2 x VIPT pairs.
// Padding records (zero mass and cotangents, far away) contribute exactly
// zero.  The self pair also contributes exactly zero: r = v = 0 and
// lam = m_k La_j - m_j La_k cancels bit for bit (two rounded products, no
// contraction); with the hermite jerk form the 1/r^2 factor is set to 0
// there.
constexpr int VF = 16;  // fields per body
struct __align__(16) VJPair {
  float2 f[VF];
};
constexpr int VIPT = 2;
constexpr int VT2 = 128;

__device__ __forceinline__ float rsqrt_approx(float x) {
  float y;
  asm("rsqrt.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
  return y;
}
__device__ __forceinline__ float rcp_approx(float x) {
  float y;
  asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
  return y;
}

__global__ void vjp_records_kernel(int n, int n_pad, const double *__restrict__ x,
                                   const double *__restrict__ v, const double *__restrict__ m,
                                   const double *__restrict__ la1, const double *__restrict__ lj1,
                                   VJPair *rec) {
  const int s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= n_pad) return;
  float f[VF];
  if (s < n) {
    for (int k = 0; k < 3; k++) {
      f[k] = __double2float_rn(x[3 * s + k]);
      f[4 + k] = __double2float_rn(x[3 * s + k] - (double)f[k]);
      f[7 + k] = __double2float_rn(v[3 * s + k]);
      f[10 + k] = __double2float_rn(la1[3 * s + k]);
      f[13 + k] = __double2float_rn(lj1[3 * s + k]);
    }
    f[3] = __double2float_rn(m[s]);
  } else {
    for (int k = 0; k < VF; k++) f[k] = 0.f;
    f[0] = f[1] = f[2] = 1.0e18f;
  }
  float *dst = reinterpret_cast<float *>(rec + (s >> 1)) + (s & 1);
  for (int k = 0; k < VF; k++) dst[2 * k] = f[k];
}

template <bool HJ>
__global__ void __launch_bounds__(VT2) vjp_split_kernel(int n, float eps2, const VJPair *__restrict__ rec,
                                                        int jsplit, int n_pad,
                                                        double *part /* [nsplit][n][7] */) {
  __shared__ VJPair tile[VTILE / 2];
  f2x xh[VIPT][3], xl[VIPT][3], vk[VIPT][3], mk[VIPT], lak[VIPT][3], ljk[VIPT][3];
  int kk[VIPT];
#pragma unroll
  for (int q = 0; q < VIPT; q++) {
    kk[q] = blockIdx.x * (VT2 * VIPT) + q * VT2 + threadIdx.x;
    const int k = kk[q] < n_pad ? kk[q] : 0;
    const float *src = reinterpret_cast<const float *>(rec + (k >> 1)) + (k & 1);
#pragma unroll
    for (int c = 0; c < 3; c++) {
      xh[q][c] = f2_dup(src[2 * c]);
      xl[q][c] = f2_dup(src[2 * (4 + c)]);
      vk[q][c] = f2_dup(src[2 * (7 + c)]);
      lak[q][c] = f2_dup(src[2 * (10 + c)]);
      ljk[q][c] = f2_dup(src[2 * (13 + c)]);
    }
    mk[q] = f2_dup(src[2 * 3]);
  }
  double tot[VIPT][7];
#pragma unroll
  for (int q = 0; q < VIPT; q++)
#pragma unroll
    for (int c = 0; c < 7; c++) tot[q][c] = 0.0;
  const f2x e2 = f2_dup(eps2);
  const f2x m3 = f2_dup(-3.0f);
  const int j0 = blockIdx.y * jsplit;
  const int j1 = min(n_pad, j0 + jsplit);
  for (int t0 = j0; t0 < j1; t0 += VTILE) {
    __syncthreads();
    for (int q = threadIdx.x; q < VTILE / 2; q += VT2) tile[q] = rec[t0 / 2 + q];
    __syncthreads();
    f2x g[VIPT][7];
#pragma unroll
    for (int q = 0; q < VIPT; q++)
#pragma unroll
      for (int c = 0; c < 7; c++) g[q][c] = 0ull;
#pragma unroll 2
    for (int jj = 0; jj < VTILE / 2; jj++) {
      const VJPair &r = tile[jj];
      f2x xhj[3], xlj[3], vj[3], laj[3], ljj[3];
#pragma unroll
      for (int c = 0; c < 3; c++) {
        xhj[c] = f2_of(r.f[c]);
        xlj[c] = f2_of(r.f[4 + c]);
        vj[c] = f2_of(r.f[7 + c]);
        laj[c] = f2_of(r.f[10 + c]);
        ljj[c] = f2_of(r.f[13 + c]);
      }
      const f2x mj = f2_of(r.f[3]);
#pragma unroll
      for (int q = 0; q < VIPT; q++) {
        f2x R[3], V[3], lam[3], mu[3];
#pragma unroll
        for (int c = 0; c < 3; c++) {
          R[c] = f2_add(f2_sub(xhj[c], xh[q][c]), f2_sub(xlj[c], xl[q][c]));
          V[c] = f2_sub(vj[c], vk[q][c]);
          lam[c] = f2_sub(f2_mul(mk[q], laj[c]), f2_mul(mj, lak[q][c]));
          mu[c] = f2_sub(f2_mul(mk[q], ljj[c]), f2_mul(mj, ljk[q][c]));
        }
        const f2x s = f2_fma(R[2], R[2], f2_fma(R[1], R[1], f2_fma(R[0], R[0], e2)));
        float sa, sb;
        f2_unpack(s, sa, sb);
        const f2x s1 = f2_pack(rsqrt_approx(sa), rsqrt_approx(sb));
        const f2x si = f2_mul(s1, s1);
        const f2x s3 = f2_mul(s1, si), s5 = f2_mul(s3, si);
        const f2x rl = f2_fma(R[2], lam[2], f2_fma(R[1], lam[1], f2_mul(R[0], lam[0])));
        const f2x rm = f2_fma(R[2], mu[2], f2_fma(R[1], mu[1], f2_mul(R[0], mu[0])));
        const f2x vm = f2_fma(V[2], mu[2], f2_fma(V[1], mu[1], f2_mul(V[0], mu[0])));
        const f2x rv = f2_fma(R[2], V[2], f2_fma(R[1], V[1], f2_mul(R[0], V[0])));
        f2x qs, c7;
        if (HJ) {
          const f2x r2u = f2_fma(R[2], R[2], f2_fma(R[1], R[1], f2_mul(R[0], R[0])));
          float ua, ub;
          f2_unpack(r2u, ua, ub);
          const f2x qi = f2_pack(ua > 0.f ? rcp_approx(ua) : 0.f, ub > 0.f ? rcp_approx(ub) : 0.f);
          qs = f2_mul(qi, s3);
          c7 = f2_mul(qi, f2_fma(f2_dup(6.0f), qs, f2_mul(f2_dup(9.0f), s5)));
        } else {
          qs = s5;
          c7 = f2_mul(f2_dup(15.0f), f2_mul(s5, si));
        }
        const f2x q3 = f2_mul(m3, qs);
        const f2x cr = f2_fma(f2_mul(rv, rm), c7, f2_mul(m3, f2_mul(f2_add(rl, vm), s5)));
        const f2x w = f2_mul(q3, rm);
#pragma unroll
        for (int c = 0; c < 3; c++) {
          const f2x u = f2_fma(rm, V[c], f2_mul(rv, mu[c]));
          g[q][c] = f2_fma(q3, u, f2_fma(cr, R[c], f2_fma(lam[c], s3, g[q][c])));
          g[q][3 + c] = f2_fma(w, R[c], f2_fma(mu[c], s3, g[q][3 + c]));
        }
        const f2x ga = f2_fma(laj[2], R[2], f2_fma(laj[1], R[1], f2_mul(laj[0], R[0])));
        const f2x lv = f2_fma(ljj[2], V[2], f2_fma(ljj[1], V[1], f2_mul(ljj[0], V[0])));
        const f2x lr = f2_fma(ljj[2], R[2], f2_fma(ljj[1], R[1], f2_mul(ljj[0], R[0])));
        g[q][6] = f2_sub(g[q][6], f2_fma(f2_add(ga, lv), s3, f2_mul(f2_mul(q3, rv), lr)));
      }
    }
#pragma unroll
    for (int q = 0; q < VIPT; q++)
#pragma unroll
      for (int c = 0; c < 7; c++) {
        float lo, hi;
        f2_unpack(g[q][c], lo, hi);
        tot[q][c] += (double)lo + (double)hi;
      }
  }
#pragma unroll
  for (int q = 0; q < VIPT; q++) {
    if (kk[q] < n) {
      double *p = part + ((size_t)blockIdx.y * n + kk[q]) * 7;
#pragma unroll
      for (int c = 0; c < 7; c++) p[c] = tot[q][c];
    }
  }
}

__global__ void vjp_reduce_kernel(int n, int nsplit, const double *__restrict__ part, double *gx,
                                  double *gv, double *gm) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= n) return;
  double t[7] = {0, 0, 0, 0, 0, 0, 0};
  for (int s = 0; s < nsplit; s++)
    for (int c = 0; c < 7; c++) t[c] += part[((size_t)s * n + k) * 7 + c];
  for (int c = 0; c < 3; c++) {
    gx[3 * k + c] = t[c];
    gv[3 * k + c] = t[3 + c];
  }
  gm[k] = t[6];
}

}  // namespace

extern "C" int g6k_fixed_records(const g6_jstate *js, int n, const double *x, const double *v,
                                 const double *m, int prec, cudaStream_t st) {
  const int n_pad = (n + G6_TILE - 1) / G6_TILE * G6_TILE;
  if (n <= 0 || n_pad > js->cap) return -1;
  records_kernel<<<(n_pad + PT - 1) / PT, PT, 0, st>>>(n, n_pad, x, v, m, prec, js->jp_split,
                                                     js->jp_f64);
  return cudaGetLastError() == cudaSuccess ? 0 : -3;
}

extern "C" int g6k_fixed_predict(int n, double h, const double *x, const double *v,
                                 const double *a, const double *j, double *xp, double *vp,
                                 cudaStream_t st) {
  predict_kernel<<<(3 * n + PT - 1) / PT, PT, 0, st>>>(n, h, x, v, a, j, xp, vp);
  return cudaGetLastError() == cudaSuccess ? 0 : -3;
}

extern "C" int g6k_fixed_correct(int n, double h, double *x, double *v, double *a, double *j,
                                 const double *a1, const double *j1, cudaStream_t st) {
  correct_kernel<<<(3 * n + PT - 1) / PT, PT, 0, st>>>(n, h, x, v, a, j, a1, j1);
  return cudaGetLastError() == cudaSuccess ? 0 : -3;
}

extern "C" int g6k_fixed_adj_pre(int n, double h, double *lx, double *lv, double *la, double *lj,
                                 double *la1, double *lj1, cudaStream_t st) {
  adj_pre_kernel<<<(3 * n + PT - 1) / PT, PT, 0, st>>>(n, h, lx, lv, la, lj, la1, lj1);
  return cudaGetLastError() == cudaSuccess ? 0 : -3;
}

extern "C" int g6k_fixed_adj_post(int n, double h, double *lx, double *lv, double *la,
                                  double *lj, const double *gxp, const double *gvp, double *lm,
                                  const double *gm, cudaStream_t st) {
  adj_post_kernel<<<(3 * n + PT - 1) / PT, PT, 0, st>>>(n, h, lx, lv, la, lj, gxp, gvp, lm, gm);
  return cudaGetLastError() == cudaSuccess ? 0 : -3;
}

// Launch shapes.  FP64: one body per thread, j split over 1/4/8 CTA rows.
// Split: VIPT bodies per thread, j split so that there are >= 4 CTAs per SM.
static void vjp_shape(int n, int prec, int *nsplit, int *jsplit, int *n_pad) {
  *n_pad = (n + VTILE - 1) / VTILE * VTILE;
  if (prec == G6_PREC_FP64) {
    *nsplit = n >= 8192 ? 8 : (n >= 1024 ? 4 : 1);
    *jsplit = (n + *nsplit - 1) / *nsplit;
    return;
  }
  static int sms = 0;  // SM count of the (single) device, looked up once
  if (sms <= 0) {
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess ||
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess ||
        sms <= 0)
      sms = 152;
  }
  const int gx = (n + VT2 * VIPT - 1) / (VT2 * VIPT);
  const int tiles = *n_pad / VTILE;
  int ns = (4 * sms + gx - 1) / gx;
  if (ns > tiles) ns = tiles;
  if (ns < 1) ns = 1;
  const int tp = (tiles + ns - 1) / ns;  // tiles per split
  *jsplit = tp * VTILE;
  *nsplit = (tiles + tp - 1) / tp;
}

// Scratch: the split records (n_pad x 64 B), then the partials
// (nsplit x n x 7 doubles); the larger of the two precisions' needs.
extern "C" size_t g6k_vjp_scratch_bytes(int n) {
  size_t need = 0;
  for (int prec = 0; prec < 2; prec++) {
    int ns, js, np;
    vjp_shape(n, prec, &ns, &js, &np);
    const size_t b = (size_t)np * (sizeof(VJPair) / 2) + (size_t)ns * (size_t)n * 7 * sizeof(double);
    if (b > need) need = b;
  }
  return need;
}

// hjerk: differentiate the hermite code's jerk form instead of the softened
// one (must match the force the forward step used).
extern "C" int g6k_force_vjp(int n, double eps2, int prec, int hjerk, const double *x,
                             const double *v, const double *m, const double *la1,
                             const double *lj1, double *gx, double *gv, double *gm, void *scratch,
                             cudaStream_t st) {
  if (n <= 0) return 0;
  int nsplit, jsplit, n_pad;
  vjp_shape(n, prec, &nsplit, &jsplit, &n_pad);
  VJPair *rec = reinterpret_cast<VJPair *>(scratch);
  double *part = reinterpret_cast<double *>(reinterpret_cast<char *>(scratch) +
                                            (size_t)n_pad * (sizeof(VJPair) / 2));
  if (prec == G6_PREC_FP64) {
    dim3 grid((n + VT - 1) / VT, nsplit);
#define G6_VJP(H) vjp_f64_kernel<H><<<grid, VT, 0, st>>>(n, eps2, x, v, m, la1, lj1, jsplit, part)
    if (hjerk) G6_VJP(true);
    else G6_VJP(false);
#undef G6_VJP
  } else {
    vjp_records_kernel<<<(n_pad + PT - 1) / PT, PT, 0, st>>>(n, n_pad, x, v, m, la1, lj1, rec);
    const float e2 = (float)eps2 + (float)(1.0 / 4503599627370496.0);
    dim3 grid((n + VT2 * VIPT - 1) / (VT2 * VIPT), nsplit);
    if (hjerk)
      vjp_split_kernel<true><<<grid, VT2, 0, st>>>(n, e2, rec, jsplit, n_pad, part);
    else
      vjp_split_kernel<false><<<grid, VT2, 0, st>>>(n, e2, rec, jsplit, n_pad, part);
  }
  vjp_reduce_kernel<<<(n + 127) / 128, 128, 0, st>>>(n, nsplit, part, gx, gv, gm);
  return cudaGetLastError() == cudaSuccess ? 0 : -3;
}
