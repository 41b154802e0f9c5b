// kern_knn.cu -- the k nearest neighbours of listed particles (extension
// call g6x_knn), exact in FP64.
//
// ph4's jdata::get_densities_on_gpu (src/amuse_ph4/src/gpu.cc:568-866)
// gathers, through the GRAPE neighbour-list calls and a retry loop on the
// search radii, the knn = 12 nearest neighbours of every particle:
// save_neighbors (gpu.cc:534-558) sorts all other particles by the squared
// distance sum_k (x_i,k - x_j,k)^2 and keeps the first knn.  Here:
//
//   knn_kernel     one thread per listed particle streams the split records
//                  (j split across CTAs when few particles are listed) and
//                  keeps, in shared memory, the k + KEXTRA smallest FP32
//                  double-single squared distances (two j per packed f32x2
//                  instruction; no FP64 in the loop), then writes the FP64
//                  squared distances of those candidates, summed in
//                  component order as save_neighbors sums them, from
//                  positions predicted with ph4's expression;
//   knn_merge      per particle: sorts each split's candidates by (d^2,
//                  slot), proves that no particle left out can be among the
//                  k nearest (gap test below), and merges the splits;
//   knn_exact      particles whose gap test failed (many FP32-equal
//                  distances at the cut, e.g. a lattice) are redone with an
//                  FP64 distance for every j that passes the filter bound.
//
// Filter bound.  With X >= max |coordinate| over the j-system, each FP32
// difference dx_f of the split records obeys |dx_f - dx| <= 2^-22 |dx| + E,
// E = 2^-30 X (double-single representation 2^-48 X per position, three
// FP32 roundings, and a few ulps between the split predictor's FMA form and
// ph4's expression).  The FMA chain for the square sum adds 3 roundings.  So
// d^2 <= D implies d_f^2 <= T(D) = (1 + 2^-16) D + 4 E sqrt(D) + 4 E^2.
// Gap test: the candidates are the particles with the smallest FP32 keys,
// every other j has d_f^2 >= F (the largest kept key); if T(d_k^2) < F for
// the k-th exact distance d_k^2 among the candidates, every other j has
// d^2 > d_k^2, so the candidates hold the exact k nearest.
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
constexpr int KEXTRA = 8;          // candidates kept beyond k
constexpr int KPMAX = G6_KNN_MAX + KEXTRA;

// One pair of consecutive split records (the layout in g6_dev.h).
struct __align__(16) PairRec {
  float2 xh, yh, zh, m, xl, yl, zl, pad0, vx, vy, vz, pad1;
};
static_assert(sizeof(PairRec) == 96, "split record pair");

struct KArgs {
  g6_jstate js;
  int nj, ni, k, kp, nsplit, jsplit;
  const int *slots;      // [ni]
  const double *pos64;   // [nj][4]: ph4-predicted x, y, z
  const unsigned *xmax;  // FP32 bits of max |xh| over j < nj
  double *cand_d;        // [nsplit][ni][kp] exact d^2 of the candidates
  int *cand_s;           // [nsplit][ni][kp] their slots
  int *cand_n;           // [nsplit][ni] candidates kept
  float *cand_f;         // [nsplit][ni] largest FP32 key kept (+inf: all kept)
  int *flag;             // [ni] gap test failed
  int *ids;              // [ni][k] out
  double *d2;            // [ni][k] out
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

// Squared distances are >= +0, so their IEEE bits order like the values:
// the sort keys compare as integers (FP64 compares issue at the FP64 rate).
__device__ __forceinline__ unsigned long long kbits(double d) {
  return (unsigned long long)__double_as_longlong(d);
}
__device__ __forceinline__ bool kless(unsigned long long a, int sa, unsigned long long b,
                                      int sb) {
  return a < b || (a == b && sa < sb);
}

__device__ __forceinline__ double knn_E(const unsigned *xmax) {
  return (double)__uint_as_float(*xmax) * (1.0 + 1.0 / 1048576.0) * (1.0 / 1073741824.0);
}

// T(D) of the header, rounded up to FP32.
__device__ __forceinline__ float knn_bound(double D, double E) {
  const double T = (1.0 + 1.0 / 65536.0) * D + 4.0 * E * sqrt(D) + 4.0 * E * E;
  return __double2float_ru(T);
}

// FP64 squared distance, summed in component order (save_neighbors).
__device__ __forceinline__ double knn_d2(const double *pos64, double x0, double x1, double x2,
                                         int j) {
  const double d0 = __dsub_rn(x0, pos64[4 * (size_t)j]);
  const double d1 = __dsub_rn(x1, pos64[4 * (size_t)j + 1]);
  const double d2 = __dsub_rn(x2, pos64[4 * (size_t)j + 2]);
  return __dadd_rn(__dadd_rn(__dmul_rn(d0, d0), __dmul_rn(d1, d1)), __dmul_rn(d2, d2));
}

struct IPos {
  f2x xh, yh, zh, xl, yl, zl;
  double x0, x1, x2;
};

__device__ __forceinline__ IPos knn_ipos(const KArgs &ka, int self) {
  IPos p;
  const void *r = ka.js.jp_split;
  p.xh = f2_dup(g6_split_get(r, self, 0));
  p.yh = f2_dup(g6_split_get(r, self, 1));
  p.zh = f2_dup(g6_split_get(r, self, 2));
  p.xl = f2_dup(g6_split_get(r, self, 4));
  p.yl = f2_dup(g6_split_get(r, self, 5));
  p.zl = f2_dup(g6_split_get(r, self, 6));
  p.x0 = ka.pos64[4 * (size_t)self];
  p.x1 = ka.pos64[4 * (size_t)self + 1];
  p.x2 = ka.pos64[4 * (size_t)self + 2];
  return p;
}

// FP32 squared distances of one record pair (two j) to the particle.
__device__ __forceinline__ void knn_r2f(const PairRec &r, const IPos &p, float &ra, float &rb) {
  const f2x dx = f2_add(f2_sub(f2_of(r.xh), p.xh), f2_sub(f2_of(r.xl), p.xl));
  const f2x dy = f2_add(f2_sub(f2_of(r.yh), p.yh), f2_sub(f2_of(r.yl), p.yl));
  const f2x dz = f2_add(f2_sub(f2_of(r.zh), p.zh), f2_sub(f2_of(r.zl), p.zl));
  f2_unpack(f2_fma(dz, dz, f2_fma(dy, dy, f2_mul(dx, dx))), ra, rb);
}

__device__ __forceinline__ void knn_load_tile(PairRec *tile, const PairRec *gj, int tj) {
  const float4 *src = reinterpret_cast<const float4 *>(gj + tj / 2);
  float4 *dst = reinterpret_cast<float4 *>(tile);
  for (int q = threadIdx.x; q < KRPT * 6; q += KT) dst[q] = src[q];
}

// Candidate pass: the kp smallest FP32 keys (ties to the smaller slot) of
// this split's j range, then their exact FP64 squared distances.
__global__ void __launch_bounds__(KT) knn_kernel(KArgs ka) {
  extern __shared__ __align__(16) unsigned char smem[];
  PairRec *tile = reinterpret_cast<PairRec *>(smem);
  float *lf = reinterpret_cast<float *>(tile + KRPT);  // [kp][KT]
  int *ls = reinterpret_cast<int *>(lf + ka.kp * KT);   // [kp][KT]
  const int tid = threadIdx.x;
  const int i = blockIdx.x * KT + tid;
  const bool active = i < ka.ni;
  const int self = active ? ka.slots[i] : -1;
  const int KP = ka.kp;
  IPos ip;
  if (active) ip = knn_ipos(ka, self);
  int cnt = 0;
  float F = __int_as_float(0x7f800000);  // largest kept key once the list is full

  const int j0 = blockIdx.y * ka.jsplit;
  const int j1 = min(j0 + ka.jsplit, ka.nj);
  const PairRec *gj = reinterpret_cast<const PairRec *>(ka.js.jp_split);
  for (int tj = j0; tj < j1; tj += KTJ) {
    knn_load_tile(tile, gj, tj);
    __syncthreads();
    if (active) {
      // Two record pairs (four j) per step: two independent FP32 chains and
      // one early-out test.  The kept set does not depend on the order in
      // which candidates arrive.
      const int npair = min(KRPT, (j1 - tj + 1) / 2);
      for (int p = 0; p < npair; p += 2) {
        float rr[4];
        knn_r2f(tile[p], ip, rr[0], rr[1]);
        if (p + 1 < npair) {
          knn_r2f(tile[p + 1], ip, rr[2], rr[3]);
        } else {
          rr[2] = rr[3] = __int_as_float(0x7f800000);
        }
        if (fminf(fminf(rr[0], rr[1]), fminf(rr[2], rr[3])) > F) continue;
#pragma unroll
        for (int h = 0; h < 4; h++) {
          const int j = tj + 2 * p + h;
          const float r = rr[h];
          if ((h >= 2 && p + 1 >= npair) || r > F || j >= j1 || j == self) continue;
          if (cnt == KP) {
            const float lr = lf[(KP - 1) * KT + tid];
            if (!(r < lr || (r == lr && j < ls[(KP - 1) * KT + tid]))) continue;
          }
          int q = cnt < KP ? cnt : KP - 1;
          while (q > 0) {
            const float pr = lf[(q - 1) * KT + tid];
            const int ps = ls[(q - 1) * KT + tid];
            if (!(r < pr || (r == pr && j < ps))) break;
            lf[q * KT + tid] = pr;
            ls[q * KT + tid] = ps;
            q--;
          }
          lf[q * KT + tid] = r;
          ls[q * KT + tid] = j;
          if (cnt < KP) cnt++;
          if (cnt == KP) F = lf[(KP - 1) * KT + tid];
        }
      }
    }
    __syncthreads();
  }
  if (!active) return;
  const size_t o = (size_t)blockIdx.y * ka.ni + i;
  ka.cand_n[o] = cnt;
  ka.cand_f[o] = cnt == KP ? F : __int_as_float(0x7f800000);
  for (int q = 0; q < cnt; q++) {
    const int j = ls[q * KT + tid];
    ka.cand_d[o * KP + q] = knn_d2(ka.pos64, ip.x0, ip.x1, ip.x2, j);
    ka.cand_s[o * KP + q] = j;
  }
}

// Per listed particle: exact sort of each split's candidates, the gap test,
// and the merge of the splits' k nearest.
__global__ void knn_merge_kernel(KArgs ka) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= ka.ni) return;
  const int K = ka.k, KP = ka.kp;
  const double E = knn_E(ka.xmax);
  unsigned long long ck[KPMAX], gk[G6_KNN_MAX], tk[G6_KNN_MAX];
  int cs[KPMAX], gs[G6_KNN_MAX], ts[G6_KNN_MAX];
  int gn = 0;
  bool ok = true;
  for (int sp = 0; sp < ka.nsplit; sp++) {
    const size_t o = (size_t)sp * ka.ni + i;
    const int n = ka.cand_n[o];
    for (int q = 0; q < n; q++) {  // insertion sort by (d^2, slot)
      const unsigned long long key = kbits(ka.cand_d[o * KP + q]);
      const int sl = ka.cand_s[o * KP + q];
      int r = q;
      while (r > 0 && kless(key, sl, ck[r - 1], cs[r - 1])) {
        ck[r] = ck[r - 1];
        cs[r] = cs[r - 1];
        r--;
      }
      ck[r] = key;
      cs[r] = sl;
    }
    const float F = ka.cand_f[o];
    if (n == KP && !(knn_bound(__longlong_as_double((long long)ck[K - 1]), E) < F)) ok = false;
    // merge the split's first min(K, n) into the running k nearest
    const int m = n < K ? n : K;
    int a = 0, b = 0, t = 0;
    while (t < K && (a < gn || b < m)) {
      if (b >= m || (a < gn && kless(gk[a], gs[a], ck[b], cs[b]))) {
        tk[t] = gk[a];
        ts[t++] = gs[a++];
      } else {
        tk[t] = ck[b];
        ts[t++] = cs[b++];
      }
    }
    for (int q = 0; q < t; q++) {
      gk[q] = tk[q];
      gs[q] = ts[q];
    }
    gn = t;
  }
  ka.flag[i] = ok ? 0 : 1;
  for (int q = 0; q < K; q++) {
    ka.ids[(size_t)i * K + q] = q < gn ? ka.js.id[gs[q]] : -1;
    ka.d2[(size_t)i * K + q] =
        q < gn ? __longlong_as_double((long long)gk[q]) : __longlong_as_double(0x7ff0000000000000ll);
  }
}

// Particles whose gap test failed: one pass over all j with an FP64
// distance for every j that passes the filter bound T(current k-th), and a
// sorted list of the k nearest in shared memory.  CTAs without such a
// particle return at once.
__global__ void __launch_bounds__(KT) knn_exact_kernel(KArgs ka) {
  extern __shared__ __align__(16) unsigned char smem[];
  PairRec *tile = reinterpret_cast<PairRec *>(smem);
  unsigned long long *lk = reinterpret_cast<unsigned long long *>(tile + KRPT);  // [k][KT]
  int *ls = reinterpret_cast<int *>(lk + ka.k * KT);                               // [k][KT]
  const int tid = threadIdx.x;
  const int i = blockIdx.x * KT + tid;
  const bool mine = i < ka.ni && ka.flag[i];
  if (!__syncthreads_or(mine)) return;
  const int self = mine ? ka.slots[i] : -1;
  const int K = ka.k;
  IPos ip;
  if (mine) ip = knn_ipos(ka, self);
  const double E = knn_E(ka.xmax);
  int cnt = 0;
  float T = __int_as_float(0x7f800000);
  const PairRec *gj = reinterpret_cast<const PairRec *>(ka.js.jp_split);
  for (int tj = 0; tj < ka.nj; tj += KTJ) {
    knn_load_tile(tile, gj, tj);
    __syncthreads();
    if (mine) {
      const int npair = min(KRPT, (ka.nj - tj + 1) / 2);
      for (int p = 0; p < npair; p++) {
        float ra, rb;
        knn_r2f(tile[p], ip, ra, rb);
        if (fminf(ra, rb) > T) continue;
        for (int h = 0; h < 2; h++) {
          const int j = tj + 2 * p + h;
          if ((h ? rb : ra) > T || j >= ka.nj || j == self) continue;
          const unsigned long long key = kbits(knn_d2(ka.pos64, ip.x0, ip.x1, ip.x2, j));
          if (cnt == K && !kless(key, j, lk[(K - 1) * KT + tid], ls[(K - 1) * KT + tid]))
            continue;
          int q = cnt < K ? cnt : K - 1;
          while (q > 0 && kless(key, j, lk[(q - 1) * KT + tid], ls[(q - 1) * KT + tid])) {
            lk[q * KT + tid] = lk[(q - 1) * KT + tid];
            ls[q * KT + tid] = ls[(q - 1) * KT + tid];
            q--;
          }
          lk[q * KT + tid] = key;
          ls[q * KT + tid] = j;
          if (cnt < K) cnt++;
          if (cnt == K)
            T = knn_bound(__longlong_as_double((long long)lk[(K - 1) * KT + tid]), E);
        }
      }
    }
    __syncthreads();
  }
  if (!mine) return;
  for (int q = 0; q < K; q++) {
    ka.ids[(size_t)i * K + q] = q < cnt ? ka.js.id[ls[q * KT + tid]] : -1;
    ka.d2[(size_t)i * K + q] = q < cnt ? __longlong_as_double((long long)lk[q * KT + tid])
                                       : __longlong_as_double(0x7ff0000000000000ll);
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

struct Layout {
  size_t pos64, xmax, cand_d, cand_s, cand_n, cand_f, flag, total;
};

Layout knn_layout(int nj, int ni, int k, int nsplit) {
  const size_t kp = (size_t)k + KEXTRA, nc = (size_t)nsplit * ni;
  Layout L;
  L.pos64 = 0;
  L.xmax = L.pos64 + align256(sizeof(double) * 4 * (size_t)nj);
  L.cand_d = L.xmax + align256(sizeof(unsigned));
  L.cand_s = L.cand_d + align256(sizeof(double) * nc * kp);
  L.cand_n = L.cand_s + align256(sizeof(int) * nc * kp);
  L.cand_f = L.cand_n + align256(sizeof(int) * nc);
  L.flag = L.cand_f + align256(sizeof(float) * nc);
  L.total = L.flag + align256(sizeof(int) * (size_t)ni);
  return L;
}

}  // namespace

extern "C" size_t g6k_knn_scratch_bytes(int nj, int ni, int k) {
  int nsplit, jsplit;
  knn_shape(ni, nj, &nsplit, &jsplit);
  return knn_layout(nj, ni, k, nsplit).total;
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
  const Layout L = knn_layout(nj, ni, k, nsplit);
  char *p = static_cast<char *>(scratch);
  static bool attr = false;
  if (!attr) {
    const int fast = (int)(sizeof(PairRec) * KRPT + (sizeof(float) + sizeof(int)) * KPMAX * KT);
    const int exact =
        (int)(sizeof(PairRec) * KRPT + (sizeof(double) + sizeof(int)) * G6_KNN_MAX * KT);
    if (cudaFuncSetAttribute(knn_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, fast) !=
            cudaSuccess ||
        cudaFuncSetAttribute(knn_exact_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             exact) != cudaSuccess)
      return -3;
    attr = true;
  }
  KArgs ka;
  ka.js = *js;
  ka.nj = nj;
  ka.ni = ni;
  ka.k = k;
  ka.kp = k + KEXTRA;
  ka.nsplit = nsplit;
  ka.jsplit = jsplit;
  ka.slots = slots;
  ka.pos64 = reinterpret_cast<const double *>(p + L.pos64);
  ka.xmax = reinterpret_cast<const unsigned *>(p + L.xmax);
  ka.cand_d = reinterpret_cast<double *>(p + L.cand_d);
  ka.cand_s = reinterpret_cast<int *>(p + L.cand_s);
  ka.cand_n = reinterpret_cast<int *>(p + L.cand_n);
  ka.cand_f = reinterpret_cast<float *>(p + L.cand_f);
  ka.flag = reinterpret_cast<int *>(p + L.flag);
  ka.ids = ids;
  ka.d2 = d2;
  if (cudaMemsetAsync(p + L.xmax, 0, sizeof(unsigned), st) != cudaSuccess) return -3;
  knn_xmax_kernel<<<2 * g6k_sm_count(), 256, 0, st>>>(*js, nj,
                                                      reinterpret_cast<unsigned *>(p + L.xmax));
  knn_pos_kernel<<<(nj + 255) / 256, 256, 0, st>>>(*js, nj, t,
                                                   reinterpret_cast<double *>(p + L.pos64));
  const size_t smem_fast = sizeof(PairRec) * KRPT + (sizeof(float) + sizeof(int)) * ka.kp * KT;
  const size_t smem_exact = sizeof(PairRec) * KRPT + (sizeof(double) + sizeof(int)) * k * KT;
  const int gx = (ni + KT - 1) / KT;
  knn_kernel<<<dim3(gx, nsplit), KT, smem_fast, st>>>(ka);
  knn_merge_kernel<<<(ni + 127) / 128, 128, 0, st>>>(ka);
  knn_exact_kernel<<<gx, KT, smem_exact, st>>>(ka);
  return cudaGetLastError() == cudaSuccess ? 0 : -3;
}
