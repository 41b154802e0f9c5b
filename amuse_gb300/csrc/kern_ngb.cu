// kern_ngb.cu -- neighbour lists for g6_read_neighbour_list / g6_get_neighbour_list.
//
// For each i-particle of the last g6calc call: ids of all j in [0, nj) with
// |x_j - x_i|^2 <= h2[i], the i-particle itself excluded (the list part of
// lib/sapporo_light/dev_evaluate_gravity.cu:60-73 and :305-319).  One CTA
// per i-particle scans the predicted j records; hits are appended through a
// shared counter (order is arbitrary, the host sorts as the reference does,
// sapporo.cpp:270).  out row i = [count, id_0 .. id_{maxn-1}]; count may
// exceed maxn (overflow).
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

constexpr int NB = 256;

template <int PREC>
__global__ void __launch_bounds__(NB) ngb_kernel(g6_jstate js, int nj, const double *ipos,
                                                 const double *h2, const int *iself, int *out,
                                                 int maxn) {
  __shared__ int cnt;
  const int i = blockIdx.x;
  if (threadIdx.x == 0) cnt = 0;
  __syncthreads();
  const double xi = ipos[3 * i], yi = ipos[3 * i + 1], zi = ipos[3 * i + 2];
  const double r2max = h2[i];
  const int self = iself ? iself[i] : -1;
  int *row = out + (size_t)i * (maxn + 1);
  for (int j = threadIdx.x; j < nj; j += NB) {
    double dx, dy, dz;
    if (PREC == G6_PREC_SPLIT) {
      const void *b = js.jp_split;
      dx = ((double)g6_split_get(b, j, 0) + (double)g6_split_get(b, j, 4)) - xi;
      dy = ((double)g6_split_get(b, j, 1) + (double)g6_split_get(b, j, 5)) - yi;
      dz = ((double)g6_split_get(b, j, 2) + (double)g6_split_get(b, j, 6)) - zi;
    } else {
      const G6D4 p = reinterpret_cast<const G6D4 *>(js.jp_f64)[2 * (size_t)j];
      dx = p.x - xi;
      dy = p.y - yi;
      dz = p.z - zi;
    }
    const double r2 = dx * dx + dy * dy + dz * dz;
    if (r2 <= r2max && j != self) {
      const int k = atomicAdd(&cnt, 1);
      if (k < maxn) row[1 + k] = js.id[j];
    }
  }
  __syncthreads();
  if (threadIdx.x == 0) row[0] = cnt;
}

}  // namespace

extern "C" int g6k_neighbours(const g6_jstate *js, int nj, int ni, int prec, const double *ipos,
                              const double *h2, const int *iself, int *out, int maxn,
                              cudaStream_t st) {
  if (ni <= 0 || nj <= 0) return 0;
  if (prec == G6_PREC_FP64)
    ngb_kernel<G6_PREC_FP64><<<ni, NB, 0, st>>>(*js, nj, ipos, h2, iself, out, maxn);
  else
    ngb_kernel<G6_PREC_SPLIT><<<ni, NB, 0, st>>>(*js, nj, ipos, h2, iself, out, maxn);
  return cudaGetLastError() == cudaSuccess ? 0 : -3;
}
