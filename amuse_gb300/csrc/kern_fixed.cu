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
    float4 *r = reinterpret_cast<float4 *>(jp_split) + 3 * (size_t)s;
    r[0] = make_float4(h[0], h[1], h[2], __double2float_rn(mm));
    r[1] = make_float4(l[0], l[1], l[2], 0.f);
    r[2] = make_float4(__double2float_rn(vp[0]), __double2float_rn(vp[1]),
                       __double2float_rn(vp[2]), 0.f);
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

// ---- force VJP ----
struct VRec {  // one j in shared memory
  float xh, yh, zh, xl, yl, zl, vx, vy, vz, m;
  float la[3], lj[3];
};
struct VRecD {
  double x[3], v[3], m, la[3], lj[3];
};

template <bool F64, bool HJ>
__global__ void __launch_bounds__(VT) vjp_kernel(int n, double eps2, const double *__restrict__ x,
                                                 const double *__restrict__ v,
                                                 const double *__restrict__ m,
                                                 const double *__restrict__ la1,
                                                 const double *__restrict__ lj1, int jsplit,
                                                 double *part /* [nsplit][n][7] */) {
  __shared__ VRec ts[F64 ? 1 : VTILE];
  __shared__ VRecD td[F64 ? VTILE : 1];
  eps2 += 1.0 / 4503599627370496.0;  // the force kernel's softening (+2^-52, as ph4)
  const int k = blockIdx.x * VT + threadIdx.x;
  const bool valid = k < n;
  const int kk = valid ? k : 0;
  const int j0 = blockIdx.y * jsplit;
  const int j1 = min(n, j0 + jsplit);
  // own data
  const double xk[3] = {x[3 * kk], x[3 * kk + 1], x[3 * kk + 2]};
  const double vk[3] = {v[3 * kk], v[3 * kk + 1], v[3 * kk + 2]};
  const double mk = m[kk];
  const double lak[3] = {la1[3 * kk], la1[3 * kk + 1], la1[3 * kk + 2]};
  const double ljk[3] = {lj1[3 * kk], lj1[3 * kk + 1], lj1[3 * kk + 2]};
  float xkh[3], xkl[3];
  for (int q = 0; q < 3; q++) {
    xkh[q] = __double2float_rn(xk[q]);
    xkl[q] = __double2float_rn(xk[q] - (double)xkh[q]);
  }
  double tot[7] = {0, 0, 0, 0, 0, 0, 0};  // gx[3], gv[3], gm
  for (int t0 = j0; t0 < j1; t0 += VTILE) {
    __syncthreads();
    for (int q = threadIdx.x; q < VTILE; q += VT) {
      const int jj = t0 + q;
      if (F64) {
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
          r.m = -1.0;  // marks padding
        }
      } else {
        VRec &r = ts[q];
        if (jj < j1) {
          const double X[3] = {x[3 * jj], x[3 * jj + 1], x[3 * jj + 2]};
          r.xh = __double2float_rn(X[0]);
          r.yh = __double2float_rn(X[1]);
          r.zh = __double2float_rn(X[2]);
          r.xl = __double2float_rn(X[0] - (double)r.xh);
          r.yl = __double2float_rn(X[1] - (double)r.yh);
          r.zl = __double2float_rn(X[2] - (double)r.zh);
          r.vx = __double2float_rn(v[3 * jj]);
          r.vy = __double2float_rn(v[3 * jj + 1]);
          r.vz = __double2float_rn(v[3 * jj + 2]);
          r.m = __double2float_rn(m[jj]);
          for (int c = 0; c < 3; c++) {
            r.la[c] = __double2float_rn(la1[3 * jj + c]);
            r.lj[c] = __double2float_rn(lj1[3 * jj + c]);
          }
        } else {
          r.xh = r.yh = r.zh = 1.0e18f;
          r.xl = r.yl = r.zl = r.vx = r.vy = r.vz = 0.f;
          r.m = -1.0f;
          for (int c = 0; c < 3; c++) r.la[c] = r.lj[c] = 0.f;
        }
      }
    }
    __syncthreads();
    if (F64) {
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
    } else {
      float acc[7] = {0, 0, 0, 0, 0, 0, 0};
      const float lamk[3] = {(float)lak[0], (float)lak[1], (float)lak[2]};
      const float muk[3] = {(float)ljk[0], (float)ljk[1], (float)ljk[2]};
      const float mkf = (float)mk;
      const float vkf[3] = {(float)vk[0], (float)vk[1], (float)vk[2]};
      const float e2 = (float)eps2;
      for (int q = 0; q < VTILE; q++) {
        const VRec &r = ts[q];
        if (r.m < 0.f || t0 + q == k) continue;
        const float R[3] = {__fadd_rn(__fsub_rn(r.xh, xkh[0]), __fsub_rn(r.xl, xkl[0])),
                            __fadd_rn(__fsub_rn(r.yh, xkh[1]), __fsub_rn(r.yl, xkl[1])),
                            __fadd_rn(__fsub_rn(r.zh, xkh[2]), __fsub_rn(r.zl, xkl[2]))};
        const float V[3] = {r.vx - vkf[0], r.vy - vkf[1], r.vz - vkf[2]};
        float lam[3], mu[3];
        for (int c = 0; c < 3; c++) {
          lam[c] = mkf * r.la[c] - r.m * lamk[c];
          mu[c] = mkf * r.lj[c] - r.m * muk[c];
        }
        const float s = fmaf(R[0], R[0], fmaf(R[1], R[1], fmaf(R[2], R[2], e2)));
        const float s1 = rsqrtf(s);
        const float si = s1 * s1;
        const float s3 = s1 * si, s5 = s3 * si, s7 = s5 * si;
        const float rl = R[0] * lam[0] + R[1] * lam[1] + R[2] * lam[2];
        const float rm = R[0] * mu[0] + R[1] * mu[1] + R[2] * mu[2];
        const float vm = V[0] * mu[0] + V[1] * mu[1] + V[2] * mu[2];
        const float rv = R[0] * V[0] + R[1] * V[1] + R[2] * V[2];
        float qs, c7;
        if (HJ) {
          const float qi = __frcp_rn(R[0] * R[0] + R[1] * R[1] + R[2] * R[2]);
          qs = qi * s3;
          c7 = 3.0f * (2.0f * qi * qs + 3.0f * qi * s5);
        } else {
          qs = s5;
          c7 = 15.0f * s7;
        }
        const float cr = -3.0f * (rl * s5 + vm * s5) + rv * rm * c7;
        for (int c = 0; c < 3; c++) {
          acc[c] += lam[c] * s3 + cr * R[c] - 3.0f * qs * (rm * V[c] + rv * mu[c]);
          acc[3 + c] += mu[c] * s3 - 3.0f * rm * qs * R[c];
        }
        const float ga = (r.la[0] * R[0] + r.la[1] * R[1] + r.la[2] * R[2]) * s3;
        const float lv = r.lj[0] * V[0] + r.lj[1] * V[1] + r.lj[2] * V[2];
        const float lr = r.lj[0] * R[0] + r.lj[1] * R[1] + r.lj[2] * R[2];
        acc[6] -= ga + lv * s3 - 3.0f * rv * lr * qs;
      }
      for (int c = 0; c < 7; c++) tot[c] += (double)acc[c];
    }
  }
  if (valid) {
    double *p = part + ((size_t)blockIdx.y * n + k) * 7;
    for (int c = 0; c < 7; c++) p[c] = tot[c];
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

// part must hold nsplit * n * 7 doubles; nsplit = ceil(n / jsplit).
extern "C" size_t g6k_vjp_scratch_bytes(int n) {
  const int nsplit = n >= 8192 ? 8 : (n >= 1024 ? 4 : 1);
  return (size_t)nsplit * (size_t)n * 7 * sizeof(double);
}

// hjerk: differentiate the hermite code's jerk form instead of the softened
// one (must match the force the forward step used).
extern "C" int g6k_force_vjp(int n, double eps2, int prec, int hjerk, const double *x,
                             const double *v, const double *m, const double *la1,
                             const double *lj1, double *gx, double *gv, double *gm, double *part,
                             cudaStream_t st) {
  if (n <= 0) return 0;
  const int nsplit = n >= 8192 ? 8 : (n >= 1024 ? 4 : 1);
  const int jsplit = (n + nsplit - 1) / nsplit;
  dim3 grid((n + VT - 1) / VT, nsplit);
#define G6_VJP(F, H) vjp_kernel<F, H><<<grid, VT, 0, st>>>(n, eps2, x, v, m, la1, lj1, jsplit, part)
  if (prec == G6_PREC_FP64) {
    if (hjerk) G6_VJP(true, true);
    else G6_VJP(true, false);
  } else {
    if (hjerk) G6_VJP(false, true);
    else G6_VJP(false, false);
  }
#undef G6_VJP
  vjp_reduce_kernel<<<(n + 127) / 128, 128, 0, st>>>(n, nsplit, part, gx, gv, gm);
  return cudaGetLastError() == cudaSuccess ? 0 : -3;
}
