// kern_predict.cu -- j-update scatter and the FP64 j-predictor.
//
// Scatter: staged g6_set_j_particle records (128 B each) land in their j
// slot (the role of lib/sapporo_light/dev_evaluate_gravity.cu:322-348).
//
// Predictor: every j slot in [0, nj) is predicted to t_i in FP64 with ph4's
// expression (src/amuse_ph4/src/jdata.cc:736-744):
//   x_p = x + dt (v + dt/2 (a + dt j/3)),  v_p = v + dt (a + dt j/2),
// copied unchanged when dt = 0 (for the FP64 records with ph4's rounding
// order, bit for bit; the split records' double-single rounding hides the
// difference, so there the compiler may contract), then packed for the
// force kernel:
//   split: x_p as a double-single pair (hi = rn(x_p), lo = rn(x_p - hi)),
//          v_p and m in FP32                      -> 48 B record
//   fp64 : x_p, v_p, m in FP64                     -> 64 B record
// Slots [nj, roundup(nj, G6_TILE)) get zero-mass records far away so the force
// kernel streams whole tiles.  Streams 15 doubles + 1 int per slot
// (coalesced, component-major arrays) and writes one record.
#include "pdl.cuh"
#include <cuda_runtime.h>

#include "g6_dev.h"

// 32-byte aligned FP64 quadruple (CUDA 13 deprecates the unaligned double4).
struct __align__(32) G6D4 {
  double x, y, z, w;
};
__host__ __device__ __forceinline__ G6D4 g6d4(double x, double y, double z, double w) {
  G6D4 r;
  r.x = x; r.y = y; r.z = z; r.w = w;
  return r;
}

namespace {

constexpr int PT = 256;
constexpr double FAR = 1.0e18;

__global__ void scatter_kernel(g6_jstate js, const g6_jupd *__restrict__ upd, int n) {
  const int u = blockIdx.x * blockDim.x + threadIdx.x;
  if (u >= n) return;
  const g6_jupd r = upd[u];
  const int s = r.addr;
  if (s < 0 || s >= js.cap) return;  // host validates; never write out of range
  const int cap = js.cap;
  js.t[s] = r.t;
  js.dt[s] = r.dt;
  js.m[s] = r.m;
  js.id[s] = r.id;
#pragma unroll
  for (int k = 0; k < 3; k++) {
    js.x[k * cap + s] = r.x[k];
    js.v[k * cap + s] = r.v[k];
    js.a[k * cap + s] = r.a[k];
    js.j[k * cap + s] = r.j[k];
  }
}

// Predict slot s (< nj: ph4's expression in FP64; nj <= s < nj_pad: a
// zero-mass record far away) and store its force record.
template <int PREC>
__device__ __forceinline__ void predict_one(const g6_jstate &js, int s, int nj, double ti) {
  const int cap = js.cap;
  double xp[3], vp[3], m;
  if (s < nj) {
    m = js.m[s];
    const double dt = ti - js.t[s];
    if (dt == 0) {
#pragma unroll
      for (int k = 0; k < 3; k++) {
        xp[k] = js.x[k * cap + s];
        vp[k] = js.v[k * cap + s];
      }
    } else if (PREC == G6_PREC_FP64) {
      // the FP64 records (plain FP64 kernel, GPU oracle) carry ph4's
      // expression with its rounding order, bit for bit
#pragma unroll
      for (int k = 0; k < 3; k++) {
        const double x = js.x[k * cap + s], v = js.v[k * cap + s];
        const double a = js.a[k * cap + s], j = js.j[k * cap + s];
        xp[k] = g6_predict_x(x, v, a, j, dt);
        vp[k] = g6_predict_v(v, a, j, dt);
      }
    } else {
#pragma unroll
      for (int k = 0; k < 3; k++) {
        const double x = js.x[k * cap + s], v = js.v[k * cap + s];
        const double a = js.a[k * cap + s], j = js.j[k * cap + s];
        xp[k] = x + dt * (v + 0.5 * dt * (a + dt * j * (1.0 / 3.0)));
        vp[k] = v + dt * (a + 0.5 * dt * j);
      }
    }
  } else {
    m = 0.0;
#pragma unroll
    for (int k = 0; k < 3; k++) {
      xp[k] = FAR;
      vp[k] = 0.0;
    }
  }
  if (PREC == G6_PREC_SPLIT) {
    float h[3], l[3];
#pragma unroll
    for (int k = 0; k < 3; k++) {
      h[k] = __double2float_rn(xp[k]);
      l[k] = __double2float_rn(xp[k] - (double)h[k]);
    }
    const float mh = __double2float_rn(m);
    g6_split_store(js.jp_split, s, h[0], h[1], h[2], mh, __double2float_rn(m - (double)mh), l[0],
                   l[1], l[2], __double2float_rn(vp[0]), __double2float_rn(vp[1]),
                   __double2float_rn(vp[2]));
  } else {
    G6D4 *rec = reinterpret_cast<G6D4 *>(js.jp_f64) + 2 * (size_t)s;
    rec[0] = g6d4(xp[0], xp[1], xp[2], m);
    rec[1] = g6d4(vp[0], vp[1], vp[2], 0.0);
  }
}

template <int PREC>
__global__ void __launch_bounds__(PT) predict_kernel(g6_jstate js, int nj, int nj_pad, double ti) {
  const int s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= nj_pad) return;
  predict_one<PREC>(js, s, nj, ti);
}

// The block scheduler's second kernel fused with the predictor: the block
// time tn is the minimum of t + dt found by sched_min_first (bits in
// *dmin); each thread lists its slot if t + dt == tn (the block: ph4's
// scheduler, src/amuse_ph4/src/scheduler.cc) and predicts it to tn.
// *dmin_next, the other parity's minimum, is reset to +inf for the next
// block.
template <int PREC>
__global__ void __launch_bounds__(PT) list_predict_kernel(g6_jstate js, int nj, int nj_pad,
                                                          const unsigned long long *dmin,
                                                          unsigned long long *dmin_next,
                                                          int *ilist, int *dni, double *dtnext) {
  pdl_wait();
  pdl_trigger();
  const int s = blockIdx.x * blockDim.x + threadIdx.x;
  const double tn = __longlong_as_double((long long)*dmin);
  if (s == 0) {
    *dtnext = tn;
    *dmin_next = 0x7ff0000000000000ull;
  }
  if (s >= nj_pad) return;
  if (s < nj && js.t[s] + js.dt[s] == tn) ilist[atomicAdd(dni, 1)] = s;
  predict_one<PREC>(js, s, nj, tn);
}

}  // namespace

extern "C" int g6k_scatter(const g6_jstate *js, const g6_jupd *d_upd, int n, cudaStream_t st) {
  if (n <= 0) return 0;
  scatter_kernel<<<(n + PT - 1) / PT, PT, 0, st>>>(*js, d_upd, n);
  return cudaGetLastError() == cudaSuccess ? 0 : -3;
}

extern "C" int g6k_predict(const g6_jstate *js, int nj, double ti, int prec, cudaStream_t st) {
  if (nj <= 0) return 0;
  const int nj_pad = (nj + G6_TILE - 1) / G6_TILE * G6_TILE;
  if (nj_pad > js->cap) return -1;
  const int grid = (nj_pad + PT - 1) / PT;
  if (prec == G6_PREC_FP64)
    predict_kernel<G6_PREC_FP64><<<grid, PT, 0, st>>>(*js, nj, nj_pad, ti);
  else
    predict_kernel<G6_PREC_SPLIT><<<grid, PT, 0, st>>>(*js, nj, nj_pad, ti);
  return cudaGetLastError() == cudaSuccess ? 0 : -3;
}

extern "C" int g6k_list_predict(const g6_jstate *js, int nj, int prec,
                                const unsigned long long *dmin, unsigned long long *dmin_next,
                                int *d_ilist, int *d_ni, double *d_tnext, cudaStream_t st) {
  if (nj <= 0) return 0;
  const int nj_pad = (nj + G6_TILE - 1) / G6_TILE * G6_TILE;
  if (nj_pad > js->cap) return -1;
  const int grid = (nj_pad + PT - 1) / PT;
  const cudaError_t e =
      prec == G6_PREC_FP64
          ? launch_pdl(list_predict_kernel<G6_PREC_FP64>, dim3(grid), dim3(PT), 0, st, *js, nj,
                       nj_pad, dmin, dmin_next, d_ilist, d_ni, d_tnext)
          : launch_pdl(list_predict_kernel<G6_PREC_SPLIT>, dim3(grid), dim3(PT), 0, st, *js, nj,
                       nj_pad, dmin, dmin_next, d_ilist, d_ni, d_tnext);
  return e == cudaSuccess ? 0 : -3;
}
