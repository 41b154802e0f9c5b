// kern_knn.cu -- the k nearest neighbours of listed particles (extension
// call g6x_knn), exact in FP64.
//
// ph4's jdata::get_densities_on_gpu (src/amuse_ph4/src/gpu.cc:568-866)
// gathers, through the GRAPE neighbour-list calls and a retry loop on the
// search radii, the knn = 12 nearest neighbours of every particle:
// save_neighbors (gpu.cc:534-558) sorts all other particles by the squared
// distance sum_k (x_i,k - x_j,k)^2 and keeps the first knn.  Here one pass
// over the j-system finds them directly:
//
//   filter  the FP32 squared distance from the double-single split records,
//           two j per packed f32x2 instruction, against a bound T(B) above
//           the FP32 value of every j that is not farther than the current
//           k-th neighbour B (bound below), so no neighbour is lost;
//   accept  the FP64 squared distance ((0 + d0^2) + d1^2) + d2^2, as
//           save_neighbors sums it, from both particles' positions predicted
//           with ph4's expression; insertion into a per-thread list sorted by
//           (d^2, slot) in shared memory.
//
// Filter bound.  With X >= max |coordinate| over the j-system, each FP32
// difference dx_f of the split records obeys |dx_f - dx| <= 2^-22 |dx| + E,
// E = 2^-30 X (double-single representation 2^-48 X per position, three
// FP32 roundings, and a few ulps between the split predictor's FMA form and
// ph4's expression).  The FMA chain for the square sum adds 3 roundings.  So
// d^2 <= B implies d_f^2 <= (1 + 2^-19) B + 3.5 E sqrt(B) + 3.1 E^2, and the
// filter keeps every j with d_f^2 <= T(B) = (1 + 2^-16) B + 4 E sqrt(B) +
// 4 E^2 (rounded up to FP32).
//
// j is split across CTAs (grid.y) when few particles are listed; a second
// kernel merges the per-split lists (each sorted by (d^2, slot)), so the
// result does not depend on the split.
#include <cuda_runtime.h>
#include <limits.h>
#include <math.h>

#include "f32x2.cuh"
#include "g6_dev.h"

namespace {

constexpr int KT = 128;            // threads per CTA, one listed particle each
constexpr int KTJ = G6_TILE;       // j per shared-memory tile
constexpr int KRPT = KTJ / 2;      // split record pairs per tile
constexpr int KMAXSPLIT = 64;      // j-splits at most

// One pair of consecutive split records (the layout in g6_dev.h).
struct __align__(16) PairRec {
  float2 xh, yh, zh, m, xl, yl, zl, pad0, vx, vy, vz, pad1;
};
static_assert(sizeof(PairRec) == 96, "split record pair");

struct KArgs {
  g6_jstate js;
  int nj, ni, k, nsplit, jsplit;
  const int *slots;     // [ni]
  const double *pos64;  // [nj][4]: ph4-predicted x, y, z
  const unsigned *xmax; // FP32 bits of max |xh| over j < nj
  double *part_d;       // [nsplit][ni][k]
  int *part_s;          // [nsplit][ni][k]
};

__global__ void knn_xmax_kernel(g6_jstate js, int nj, unsigned *xmax) {
  float m = 0.f;
  for (int s = blockIdx.x * blockDim.x + threadIdx.x; s < nj; s += gridDim.x * blockDim.x) {
    m = fmaxf(m, fabsf(g6_split_get(js.jp_split, s, 0)));
    m = fmaxf(m, fabsf(g6_split_get(js.jp_split, s, 1)));
    m = fmaxf(m, fabsf(g6_split_get(js.jp_split, s, 2)));
  }
  for (int o = 16; o > 0; o >>= 1) m = fmaxf(m, __shfl_xor_sync(0xffffffffu, m, o));
  if ((threadIdx.x & 31) == 0) atomicMax(xmax, __float_as_uint(m));  // m >= 0: bits order
}

// ph4-predicted FP64 positions of all j (save_neighbors' coordinates).
__global__ void knn_pos_kernel(g6_jstate js, int nj, double t, double *pos64) {
  const int s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= nj) return;
  const int cap = js.cap;
  const double dt = __dsub_rn(t, js.t[s]);
#pragma unroll
  for (int k = 0; k < 3; k++) {
    const int a = k * cap + s;
    pos64[4 * (size_t)s + k] = g6_predict_x(js.x[a], js.v[a], js.a[a], js.j[a], dt);
  }
  pos64[4 * (size_t)s + 3] = 0.0;
}

__device__ __forceinline__ bool knn_less(double da, int sa, double db, int sb) {
  return da < db || (da == db && sa < sb);
}

__device__ __forceinline__ float knn_bound(double B, double E) {
  const double T = (1.0 + 1.0 / 65536.0) * B + 4.0 * E * sqrt(B) + 4.0 * E * E;
  return __double2float_ru(T);
}

__global__ void __launch_bounds__(KT) knn_kernel(KArgs ka) {
  extern __shared__ __align__(16) unsigned char smem[];
  PairRec *tile = reinterpret_cast<PairRec *>(smem);
  double *ld = reinterpret_cast<double *>(tile + KRPT);  // [k][KT]
  int *ls = reinterpret_cast<int *>(ld + ka.k * KT);      // [k][KT]
  const int tid = threadIdx.x;
  const int i = blockIdx.x * KT + tid;
  const bool active = i < ka.ni;
  const int self = active ? ka.slots[i] : -1;
  const int K = ka.k;

  f2x xh = 0, yh = 0, zh = 0, xl = 0, yl = 0, zl = 0;
  double xi0 = 0, xi1 = 0, xi2 = 0;
  if (active) {
    const void *r = ka.js.jp_split;
    xh = f2_dup(g6_split_get(r, self, 0));
    yh = f2_dup(g6_split_get(r, self, 1));
    zh = f2_dup(g6_split_get(r, self, 2));
    xl = f2_dup(g6_split_get(r, self, 4));
    yl = f2_dup(g6_split_get(r, self, 5));
    zl = f2_dup(g6_split_get(r, self, 6));
    xi0 = ka.pos64[4 * (size_t)self];
    xi1 = ka.pos64[4 * (size_t)self + 1];
    xi2 = ka.pos64[4 * (size_t)self + 2];
  }
  const double E = (double)__uint_as_float(*ka.xmax) * (1.0 + 1.0 / 1048576.0) *
                   (1.0 / 1073741824.0);  // 2^-30 X
  int cnt = 0;
  float T = __int_as_float(0x7f800000);  // +inf until the list is full

  const int j0 = blockIdx.y * ka.jsplit;
  int j1 = j0 + ka.jsplit;
  if (j1 > ka.nj) j1 = ka.nj;
  const PairRec *gj = reinterpret_cast<const PairRec *>(ka.js.jp_split);

  for (int tj = j0; tj < j1; tj += KTJ) {
    // cooperative copy of one tile: KRPT pair records, 16 B per load
    {
      const float4 *src = reinterpret_cast<const float4 *>(gj + tj / 2);
      float4 *dst = reinterpret_cast<float4 *>(tile);
      for (int q = tid; q < KRPT * 6; q += KT) dst[q] = src[q];
    }
    __syncthreads();
    if (active) {
      const int npair = (j1 - tj + 1) / 2 < KRPT ? (j1 - tj + 1) / 2 : KRPT;
      for (int p = 0; p < npair; p++) {
        const PairRec &r = tile[p];
        const f2x dx = f2_add(f2_sub(f2_of(r.xh), xh), f2_sub(f2_of(r.xl), xl));
        const f2x dy = f2_add(f2_sub(f2_of(r.yh), yh), f2_sub(f2_of(r.yl), yl));
        const f2x dz = f2_add(f2_sub(f2_of(r.zh), zh), f2_sub(f2_of(r.zl), zl));
        const f2x r2 = f2_fma(dz, dz, f2_fma(dy, dy, f2_mul(dx, dx)));
        float ra, rb;
        f2_unpack(r2, ra, rb);
        if (fminf(ra, rb) > T) continue;
#pragma unroll
        for (int h = 0; h < 2; h++) {
          const int j = tj + 2 * p + h;
          if ((h ? rb : ra) > T || j >= j1 || j == self) continue;
          const double d0 = __dsub_rn(xi0, ka.pos64[4 * (size_t)j]);
          const double d1 = __dsub_rn(xi1, ka.pos64[4 * (size_t)j + 1]);
          const double d2 = __dsub_rn(xi2, ka.pos64[4 * (size_t)j + 2]);
          const double d = __dadd_rn(__dadd_rn(__dmul_rn(d0, d0), __dmul_rn(d1, d1)),
                                     __dmul_rn(d2, d2));
          if (cnt == K && !knn_less(d, j, ld[(K - 1) * KT + tid], ls[(K - 1) * KT + tid]))
            continue;
          int q = cnt < K ? cnt : K - 1;
          while (q > 0 && knn_less(d, j, ld[(q - 1) * KT + tid], ls[(q - 1) * KT + tid])) {
            ld[q * KT + tid] = ld[(q - 1) * KT + tid];
            ls[q * KT + tid] = ls[(q - 1) * KT + tid];
            q--;
          }
          ld[q * KT + tid] = d;
          ls[q * KT + tid] = j;
          if (cnt < K) cnt++;
          if (cnt == K) T = knn_bound(ld[(K - 1) * KT + tid], E);
        }
      }
    }
    __syncthreads();
  }
  if (!active) return;
  const size_t o = ((size_t)blockIdx.y * ka.ni + i) * K;
  for (int q = 0; q < K; q++) {
    ka.part_d[o + q] = q < cnt ? ld[q * KT + tid] : __longlong_as_double(0x7ff0000000000000ll);
    ka.part_s[o + q] = q < cnt ? ls[q * KT + tid] : INT_MAX;
  }
}

// Per listed particle: merge the nsplit sorted lists, map slots to ids.
__global__ void knn_merge_kernel(g6_jstate js, int ni, int k, int nsplit,
                                 const double *__restrict__ part_d,
                                 const int *__restrict__ part_s, int *ids, double *d2) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= ni) return;
  int head[KMAXSPLIT];
  for (int s = 0; s < nsplit; s++) head[s] = 0;
  for (int q = 0; q < k; q++) {
    int best = -1;
    double bd = 0;
    int bs = INT_MAX;
    for (int s = 0; s < nsplit; s++) {
      if (head[s] >= k) continue;
      const size_t o = ((size_t)s * ni + i) * k + head[s];
      const double d = part_d[o];
      const int sl = part_s[o];
      if (sl == INT_MAX) continue;
      if (best < 0 || knn_less(d, sl, bd, bs)) {
        best = s;
        bd = d;
        bs = sl;
      }
    }
    if (best < 0) {
      ids[(size_t)i * k + q] = -1;
      d2[(size_t)i * k + q] = __longlong_as_double(0x7ff0000000000000ll);
    } else {
      head[best]++;
      ids[(size_t)i * k + q] = js.id[bs];
      d2[(size_t)i * k + q] = bd;
    }
  }
}

void knn_shape(int ni, int nj, int *nsplit, int *jsplit) {
  const int ntiles = (nj + KTJ - 1) / KTJ;
  const int gx = (ni + KT - 1) / KT;
  const int want = 4 * g6k_sm_count();
  int ns = (want + gx - 1) / gx;
  if (ns > KMAXSPLIT) ns = KMAXSPLIT;
  if (ns > ntiles) ns = ntiles;
  if (ns < 1) ns = 1;
  const int tp = (ntiles + ns - 1) / ns;
  *jsplit = tp * KTJ;
  *nsplit = (ntiles + tp - 1) / tp;
}

size_t align256(size_t b) { return (b + 255) / 256 * 256; }

}  // namespace

extern "C" size_t g6k_knn_scratch_bytes(int nj, int ni, int k) {
  int nsplit, jsplit;
  knn_shape(ni, nj, &nsplit, &jsplit);
  return align256(sizeof(double) * 4 * (size_t)nj) + align256(sizeof(unsigned)) +
         align256(sizeof(double) * (size_t)nsplit * ni * k) +
         align256(sizeof(int) * (size_t)nsplit * ni * k);
}

// The split records must hold the j-system predicted to t (g6k_predict,
// G6_PREC_SPLIT); slots, ids and d2 are device arrays.
extern "C" int g6k_knn(const g6_jstate *js, int nj, double t, int k, int ni, const int *slots,
                       int *ids, double *d2, void *scratch, size_t scratch_bytes,
                       cudaStream_t st) {
  if (ni <= 0) return 0;
  if (nj <= 0 || k < 1 || k > G6_KNN_MAX) return -2;
  if (scratch_bytes < g6k_knn_scratch_bytes(nj, ni, k)) return -4;
  int nsplit, jsplit;
  knn_shape(ni, nj, &nsplit, &jsplit);
  char *p = static_cast<char *>(scratch);
  double *pos64 = reinterpret_cast<double *>(p);
  p += align256(sizeof(double) * 4 * (size_t)nj);
  unsigned *xmax = reinterpret_cast<unsigned *>(p);
  p += align256(sizeof(unsigned));
  double *part_d = reinterpret_cast<double *>(p);
  p += align256(sizeof(double) * (size_t)nsplit * ni * k);
  int *part_s = reinterpret_cast<int *>(p);

  const size_t smem = sizeof(PairRec) * KRPT + (sizeof(double) + sizeof(int)) * (size_t)k * KT;
  static bool attr = false;
  if (!attr) {
    const int most = (int)(sizeof(PairRec) * KRPT + (sizeof(double) + sizeof(int)) *
                                                        (size_t)G6_KNN_MAX * KT);
    if (cudaFuncSetAttribute(knn_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, most) !=
        cudaSuccess)
      return -3;
    attr = true;
  }
  if (cudaMemsetAsync(xmax, 0, sizeof(unsigned), st) != cudaSuccess) return -3;
  knn_xmax_kernel<<<2 * g6k_sm_count(), 256, 0, st>>>(*js, nj, xmax);
  knn_pos_kernel<<<(nj + 255) / 256, 256, 0, st>>>(*js, nj, t, pos64);
  KArgs ka;
  ka.js = *js;
  ka.nj = nj;
  ka.ni = ni;
  ka.k = k;
  ka.nsplit = nsplit;
  ka.jsplit = jsplit;
  ka.slots = slots;
  ka.pos64 = pos64;
  ka.xmax = xmax;
  ka.part_d = part_d;
  ka.part_s = part_s;
  dim3 grid((ni + KT - 1) / KT, nsplit);
  knn_kernel<<<grid, KT, smem, st>>>(ka);
  knn_merge_kernel<<<(ni + 127) / 128, 128, 0, st>>>(*js, ni, k, nsplit, part_d, part_s, ids,
                                                      d2);
  return cudaGetLastError() == cudaSuccess ? 0 : -3;
}
