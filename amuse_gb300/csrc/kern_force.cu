// kern_force.cu -- the i-block Hermite force kernel (acc, jerk, pot, nearest
// neighbour) for sm_103a, in two arithmetic policies:
//
//   split: positions as double-single (hi+lo float pairs), relative
//          position formed by (xj_hi - xi_hi) + (xj_lo - xi_lo), all pair
//          arithmetic in FP32 (one MUFU rsqrt per pair), per-tile FP32
//          partial sums folded into compensated (TwoSum) hi/lo totals.
//          The j records are stored in pairs (every field a float2 of two
//          consecutive j), so each packed f32x2 instruction (add/sub/mul/fma
//          .rn.f32x2) evaluates one i against two j: half the issue slots of
//          scalar code for the same FP32 work.
//   fp64:  the same pair formula in plain FP64 (the "plain FP64 GPU"
//          kernel; also the GPU-side oracle at N=2^20).
//
// The pair formula is ph4's (src/amuse_ph4/src/idata.cc:188-226):
//   dx = xj - xi, dv = vj - vi, r2 = |dx|^2 + eps2 (+2^-52 as ph4),
//   rinv = r2^-1/2, mr3i = m rinv^3,
//   acc += mr3i dx, jerk += mr3i (dv - 3 (dx.dv)/r2 dx), pot -= m rinv,
//   nn = argmin r2 over j != self (first j on ties).
// The GRAPE-6 semantics of the g6 API excludes the i-particle itself by
// identity (lib/sapporo_light/dev_evaluate_gravity.cu:80-84 compares ids);
// here the host resolves id -> j slot once per call and the kernel skips
// that slot.
//
// Structure (one CTA = 128 threads = 4 warps; 2 i-particles per thread in
// split precision, 3 CTAs per SM; 4 in FP64):
//   * j-tiles of 256 records are streamed HBM/L2 -> shared memory with
//     cp.async.bulk (TMA, non-tensor) completing on an mbarrier; warps
//     consume the ring independently (no CTA barrier in the loop).
//   * JL j-lanes share each i-particle (JL = 1 for large i-blocks, up to
//     128 for tiny ones); j is also split across CTAs (grid.y) so that small
//     active blocks still fill all 152 SMs.
//   * Lanes of one i merge with warp shuffles (plus shared memory across
//     warps for JL > 32); CTAs of one i merge in a second pass kernel, in
//     fixed order, with float-float (split) or FP64 adds: deterministic.
//   * Nearest neighbour (optional, a template flag): the hot loop keeps only
//     a running min of r2 (one FMNMX per pair) and the tile where it last
//     improved; after the loop that tile is re-read from L2 and re-scanned
//     with bit-identical arithmetic to find the index.
//   * A tile that holds the self slot of one of the warp's i-particles takes
//     a checked copy of the loop (rinv = 0, r2 -> +inf for self).
#include <cuda_runtime.h>
#include <stdint.h>

#include "f32x2.cuh"
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

// Tuning constants (compile-time; the defaults are the measured best).
#ifndef G6_NT
#define G6_NT 128
#endif
#ifndef G6_IPT
#define G6_IPT 2
#endif
#ifndef G6_UNROLL
#define G6_UNROLL 4
#endif
#ifndef G6_MINB
#define G6_MINB 3
#endif
#ifndef G6_IPT_F64
#define G6_IPT_F64 4
#endif
constexpr int NT = G6_NT;    // threads per CTA
constexpr int TJ = G6_TILE;  // j records per tile
// i-particles per thread: the split kernel's packed f32x2 pair terms need
// twice the registers per i, so it holds fewer i than the FP64 kernel.
constexpr int IPT_SPLIT = G6_IPT;
constexpr int IPT_F64 = G6_IPT_F64;
constexpr int UNROLL = G6_UNROLL;  // j-loop unroll factor
constexpr int JLMAX = TJ < NT ? TJ : NT;  // j-lanes per i at most
constexpr unsigned long long WAIT_NS = 2000000000ull;  // 2 s bound per wait

enum { ERR_TMA_TIMEOUT = 1, ERR_SHAPE = 2 };

// Split records come in pairs of consecutive j slots, every field a float2
// {j even, j odd} (the global layout the predictor writes, g6_dev.h), so a
// packed f32x2 instruction evaluates two j at once.
struct __align__(16) RecS {
  float2 xh, yh, zh, m, xl, yl, zl, pad0, vx, vy, vz, pad1;
};
struct __align__(32) RecD {
  G6D4 p, v;
};
static_assert(sizeof(RecS) == 96, "split record pair");
static_assert(sizeof(RecD) == 64, "fp64 record");

// ---------------------------------------------------------------- PTX ---
__device__ __forceinline__ uint32_t smem_u32(const void *p) {
  return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}
__device__ __forceinline__ unsigned long long gtimer() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}
__device__ __forceinline__ void mbar_init(uint64_t *bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count)
               : "memory");
}
__device__ __forceinline__ void fence_barrier_init() {
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}
__device__ __forceinline__ void mbar_expect_tx(uint64_t *bar, uint32_t bytes) {
  asm volatile(
      "mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)),
      "r"(bytes)
      : "memory");
}
__device__ __forceinline__ void tma_load_1d(void *dst, const void *src, uint32_t bytes,
                                            uint64_t *bar) {
  asm volatile(
      "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, "
      "[%3];" ::"r"(smem_u32(dst)),
      "l"(src), "r"(bytes), "r"(smem_u32(bar))
      : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(uint64_t *bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
      "selp.u32 %0, 1, 0, p;\n\t}"
      : "=r"(ok)
      : "r"(smem_u32(bar)), "r"(parity)
      : "memory");
  return ok != 0;
}
// Bounded wait that also gives up when another warp of the CTA raised
// *abort (false in both cases).
__device__ __forceinline__ bool mbar_wait_abortable(uint64_t *bar, uint32_t parity,
                                                    volatile int *abort) {
  if (mbar_try_wait(bar, parity)) return true;
  const unsigned long long t0 = gtimer();
  while (true) {
    if (mbar_try_wait(bar, parity)) return true;
    if (*abort) return false;
    if (gtimer() - t0 > WAIT_NS) return false;
  }
}
// Bounded wait: false after WAIT_NS of global time.
__device__ __forceinline__ bool mbar_wait_bounded(uint64_t *bar, uint32_t parity) {
  if (mbar_try_wait(bar, parity)) return true;
  const unsigned long long t0 = gtimer();
  while (true) {
    if (mbar_try_wait(bar, parity)) return true;
    if (gtimer() - t0 > WAIT_NS) return false;
  }
}

// One MUFU.RSQ, flush-to-zero (r2 >= eps2 + 2^-52 is never subnormal).
// (A Newton step after it costs 13% and does not change the block-step
// behaviour measured at eta = 0.01..0.14, so there is none.)
__device__ __forceinline__ float rsqrt_approx(float x) {
  float y;
  asm("rsqrt.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
  return y;
}

// One MUFU.RCP, flush-to-zero.
__device__ __forceinline__ float rcp_approx(float x) {
  float y;
  asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
  return y;
}

// ------------------------------------------------------- float-float ---
// Knuth TwoSum folded into a (hi, lo) accumulator.
__device__ __forceinline__ void ff_acc(float &hi, float &lo, float p) {
  const float s = __fadd_rn(hi, p);
  const float bb = __fsub_rn(s, hi);
  const float e = __fadd_rn(__fsub_rn(hi, __fsub_rn(s, bb)), __fsub_rn(p, bb));
  hi = s;
  lo = __fadd_rn(lo, e);
}
// (ah, al) += (bh, bl), renormalised.
__device__ __forceinline__ void ff_add(float &ah, float &al, float bh, float bl) {
  const float s = __fadd_rn(ah, bh);
  const float bb = __fsub_rn(s, ah);
  float e = __fadd_rn(__fsub_rn(ah, __fsub_rn(s, bb)), __fsub_rn(bh, bb));
  e = __fadd_rn(e, __fadd_rn(al, bl));
  ah = __fadd_rn(s, e);
  al = __fsub_rn(e, __fsub_rn(ah, s));
}

// ------------------------------------------------------------ policies ---
struct SplitP {
  using Rec = RecS;
  using R = float;
  static constexpr int JPR = 2;     // j per record (packed pair)
  static constexpr int IPT = IPT_SPLIT;
  static constexpr int NSTAGE = 3;  // TMA ring depth (3 x 12 KB)
  static constexpr int MINB = G6_MINB;  // resident CTAs per SM
  struct I {  // i values duplicated into both halves
    f2x xh, yh, zh, xl, yl, zl, vx, vy, vz;
  };
  struct Part {  // per-fold-period partial sums, one per half
    f2x a[3], j[3], p;
  };
  struct Tot {  // compensated totals
    float ah[3], al[3], jh[3], jl[3], ph, pl;
  };
  struct Out {  // partial record exchanged between CTAs, 64 B
    float2 a[3], j[3], p;
    float nnr2;
    int nn;
  };
  __device__ static void split(double d, float &h, float &l) {
    h = __double2float_rn(d);
    l = __double2float_rn(d - (double)h);
  }
  __device__ static I dup(float xh, float yh, float zh, float xl, float yl, float zl, float vx,
                          float vy, float vz) {
    I s;
    s.xh = f2_pack(xh, xh); s.yh = f2_pack(yh, yh); s.zh = f2_pack(zh, zh);
    s.xl = f2_pack(xl, xl); s.yl = f2_pack(yl, yl); s.zl = f2_pack(zl, zl);
    s.vx = f2_pack(vx, vx); s.vy = f2_pack(vy, vy); s.vz = f2_pack(vz, vz);
    return s;
  }
  __device__ static I load_i_explicit(const double *p, const double *v) {
    float xh, yh, zh, xl, yl, zl;
    split(p[0], xh, xl);
    split(p[1], yh, yl);
    split(p[2], zh, zl);
    return dup(xh, yh, zh, xl, yl, zl, __double2float_rn(v[0]), __double2float_rn(v[1]),
               __double2float_rn(v[2]));
  }
  __device__ static I load_i_slot(const void *recs, int slot) {
    return dup(g6_split_get(recs, slot, 0), g6_split_get(recs, slot, 1),
               g6_split_get(recs, slot, 2), g6_split_get(recs, slot, 4),
               g6_split_get(recs, slot, 5), g6_split_get(recs, slot, 6),
               g6_split_get(recs, slot, 8), g6_split_get(recs, slot, 9),
               g6_split_get(recs, slot, 10));
  }
  __device__ static void zero(Part &q) {
#pragma unroll
    for (int k = 0; k < 3; k++) q.a[k] = q.j[k] = 0ull;
    q.p = 0ull;
  }
  __device__ static void zero(Tot &t) {
#pragma unroll
    for (int k = 0; k < 3; k++) t.ah[k] = t.al[k] = t.jh[k] = t.jl[k] = 0.f;
    t.ph = t.pl = 0.f;
  }
  __device__ static void fold(Tot &t, const Part &q) {
#pragma unroll
    for (int k = 0; k < 3; k++) {
      ff_acc(t.ah[k], t.al[k], f2_lo(q.a[k]));
      ff_acc(t.ah[k], t.al[k], f2_hi(q.a[k]));
      ff_acc(t.jh[k], t.jl[k], f2_lo(q.j[k]));
      ff_acc(t.jh[k], t.jl[k], f2_hi(q.j[k]));
    }
    ff_acc(t.ph, t.pl, f2_lo(q.p));
    ff_acc(t.ph, t.pl, f2_hi(q.p));
  }
  // r^2 + eps^2 of both j of a record (the nearest-neighbour key): the main
  // loop and the re-scan use this same arithmetic, so the keys are
  // bit-identical.
  __device__ static __forceinline__ f2x r2e(const I &s, const Rec &r, f2x eps2, f2x &dx, f2x &dy,
                                            f2x &dz) {
    dx = f2_add(f2_sub(f2_of(r.xh), s.xh), f2_sub(f2_of(r.xl), s.xl));
    dy = f2_add(f2_sub(f2_of(r.yh), s.yh), f2_sub(f2_of(r.yl), s.yl));
    dz = f2_add(f2_sub(f2_of(r.zh), s.zh), f2_sub(f2_of(r.zl), s.zl));
    return f2_fma(dz, dz, f2_fma(dy, dy, f2_fma(dx, dx, eps2)));
  }
  // Both j of record r on one i.  selfrel = (self slot) - (slot of the
  // record's first j): half h is the i itself when selfrel == h (CHECK only).
  // HJ: the jerk as the hermite code forms it (src/amuse_hermite/
  // interface.cc:440-449,469-486): the (r.v) factor divided by the
  // UNsoftened r^2.
  template <bool CHECK, bool NN, bool HJ = false>
  __device__ static __forceinline__ void pair(const I &s, const Rec &r, f2x eps2, Part &q,
                                              float &nnmin, int selfrel) {
    f2x dx, dy, dz;
    const f2x r2 = r2e(s, r, eps2, dx, dy, dz);
    const float r2a = f2_lo(r2), r2b = f2_hi(r2);
    float ra = rsqrt_approx(r2a), rb = rsqrt_approx(r2b);
    if (CHECK) {
      ra = selfrel == 0 ? 0.f : ra;
      rb = selfrel == 1 ? 0.f : rb;
      if (NN) {
        const float inf = __int_as_float(0x7f800000);
        nnmin = fminf(nnmin, fminf(selfrel == 0 ? inf : r2a, selfrel == 1 ? inf : r2b));
      }
    } else if (NN) {
      nnmin = fminf(nnmin, fminf(r2a, r2b));
    }
    const f2x rinv = f2_pack(ra, rb);
    const f2x dvx = f2_sub(f2_of(r.vx), s.vx);
    const f2x dvy = f2_sub(f2_of(r.vy), s.vy);
    const f2x dvz = f2_sub(f2_of(r.vz), s.vz);
    const f2x rv = f2_fma(dz, dvz, f2_fma(dy, dvy, f2_mul(dx, dvx)));
    const f2x rinv2 = f2_mul(rinv, rinv);
    const f2x mri = f2_mul(f2_of(r.m), rinv);
    const f2x mr3i = f2_mul(mri, rinv2);
    const f2x m3 = f2_pack(-3.0f, -3.0f);
    f2x a3;
    if (HJ) {
      const f2x r2u = f2_fma(dz, dz, f2_fma(dy, dy, f2_mul(dx, dx)));
      float ia = rcp_approx(f2_lo(r2u)), ib = rcp_approx(f2_hi(r2u));
      if (CHECK) {
        ia = selfrel == 0 ? 0.f : ia;
        ib = selfrel == 1 ? 0.f : ib;
      }
      a3 = f2_mul(m3, f2_mul(rv, f2_pack(ia, ib)));
    } else {
      a3 = f2_mul(m3, f2_mul(rv, rinv2));
    }
    q.a[0] = f2_fma(mr3i, dx, q.a[0]);
    q.a[1] = f2_fma(mr3i, dy, q.a[1]);
    q.a[2] = f2_fma(mr3i, dz, q.a[2]);
    q.j[0] = f2_fma(mr3i, f2_fma(a3, dx, dvx), q.j[0]);
    q.j[1] = f2_fma(mr3i, f2_fma(a3, dy, dvy), q.j[1]);
    q.j[2] = f2_fma(mr3i, f2_fma(a3, dz, dvz), q.j[2]);
    q.p = f2_add(q.p, mri);
  }
  // Nearest-neighbour re-scan of one record: the first of its j (in slot
  // order) whose key equals best and that is not the i itself.
  __device__ static __forceinline__ bool rescan(const I &s, const Rec &r, f2x eps2, float best,
                                                int slot0, int self, int &idx) {
    f2x dx, dy, dz;
    const f2x r2 = r2e(s, r, eps2, dx, dy, dz);
    if (f2_lo(r2) == best && slot0 != self) {
      idx = slot0;
      return true;
    }
    if (f2_hi(r2) == best && slot0 + 1 != self) {
      idx = slot0 + 1;
      return true;
    }
    return false;
  }
  __device__ static f2x eps(double eps2) {
    const float e = (float)eps2 + (float)(1.0 / 4503599627370496.0);  // + 2^-52 (ph4)
    return f2_pack(e, e);
  }
  __device__ static void to_out(const Tot &t, float nnr2, int nn, Out &o) {
#pragma unroll
    for (int k = 0; k < 3; k++) {
      o.a[k] = make_float2(t.ah[k], t.al[k]);
      o.j[k] = make_float2(t.jh[k], t.jl[k]);
    }
    o.p = make_float2(t.ph, t.pl);
    o.nnr2 = nnr2;
    o.nn = nn;
  }
  __device__ static void merge(Out &a, const Out &b) {
#pragma unroll
    for (int k = 0; k < 3; k++) {
      ff_add(a.a[k].x, a.a[k].y, b.a[k].x, b.a[k].y);
      ff_add(a.j[k].x, a.j[k].y, b.j[k].x, b.j[k].y);
    }
    ff_add(a.p.x, a.p.y, b.p.x, b.p.y);
    if (b.nnr2 < a.nnr2 || (b.nnr2 == a.nnr2 && b.nn < a.nn)) {
      a.nnr2 = b.nnr2;
      a.nn = b.nn;
    }
  }
  __device__ static void write_final(const Out &o, int i, double *acc, double *jerk,
                                     double *pot) {
#pragma unroll
    for (int k = 0; k < 3; k++) {
      acc[3 * i + k] = (double)o.a[k].x + (double)o.a[k].y;
      jerk[3 * i + k] = (double)o.j[k].x + (double)o.j[k].y;
    }
    pot[i] = -((double)o.p.x + (double)o.p.y);
  }
};

struct F64P {
  using Rec = RecD;
  using R = double;
  static constexpr int JPR = 1;     // j per record
  static constexpr int IPT = IPT_F64;
  static constexpr int NSTAGE = 2;  // TMA ring depth (2 x 16 KB)
  static constexpr int MINB = 1;
  struct I {
    double x, y, z, vx, vy, vz;
  };
  struct Part {
    double a[3], j[3], p;
  };
  struct Tot {
    double a[3], j[3], p;
  };
  struct Out {  // 80 B
    double a[3], j[3], p;
    double nnr2;
    int nn, pad;
  };
  __device__ static I load_i_explicit(const double *p, const double *v) {
    I s;
    s.x = p[0]; s.y = p[1]; s.z = p[2];
    s.vx = v[0]; s.vy = v[1]; s.vz = v[2];
    return s;
  }
  __device__ static I load_i_slot(const void *recs, int slot) {
    const Rec &r = reinterpret_cast<const Rec *>(recs)[slot];
    I s;
    s.x = r.p.x; s.y = r.p.y; s.z = r.p.z;
    s.vx = r.v.x; s.vy = r.v.y; s.vz = r.v.z;
    return s;
  }
  __device__ static double eps(double eps2) { return eps2 + 1.0 / 4503599627370496.0; }
  __device__ static void zero(Part &q) {
#pragma unroll
    for (int k = 0; k < 3; k++) q.a[k] = q.j[k] = 0.0;
    q.p = 0.0;
  }
  __device__ static void zero(Tot &t) {
#pragma unroll
    for (int k = 0; k < 3; k++) t.a[k] = t.j[k] = 0.0;
    t.p = 0.0;
  }
  __device__ static void fold(Tot &t, const Part &q) {
#pragma unroll
    for (int k = 0; k < 3; k++) {
      t.a[k] += q.a[k];
      t.j[k] += q.j[k];
    }
    t.p += q.p;
  }
  __device__ static __forceinline__ double r2e(const I &s, const Rec &r, double eps2,
                                               double &dx, double &dy, double &dz) {
    dx = r.p.x - s.x;
    dy = r.p.y - s.y;
    dz = r.p.z - s.z;
    double r2 = __fma_rn(dx, dx, eps2);
    r2 = __fma_rn(dy, dy, r2);
    return __fma_rn(dz, dz, r2);
  }
  // 1/sqrt(x) in FP64: FP32 MUFU seed, then two Newton-Raphson steps
  // y <- y (3 - x y^2) / 2 (quadratic convergence: 2^-22 -> 2^-44 -> 2^-88).
  __device__ static __forceinline__ double rsqrt64(double x) {
    double y = (double)rsqrtf((float)x);
    const double hx = 0.5 * x;
    y = y * __fma_rn(-hx * y, y, 1.5);
    y = y * __fma_rn(-hx * y, y, 1.5);
    return y;
  }
  template <bool CHECK, bool NN, bool HJ = false>
  __device__ static __forceinline__ void pair(const I &s, const Rec &r, double eps2, Part &q,
                                              double &nnmin, int selfrel) {
    const bool is_self = CHECK && selfrel == 0;
    double dx, dy, dz;
    const double r2 = r2e(s, r, eps2, dx, dy, dz);
    double rinv = rsqrt64(r2);
    if (CHECK) {
      rinv = is_self ? 0.0 : rinv;
      if (NN) nnmin = fmin(nnmin, is_self ? __longlong_as_double(0x7ff0000000000000ll) : r2);
    } else if (NN) {
      nnmin = fmin(nnmin, r2);
    }
    const double dvx = r.v.x - s.vx, dvy = r.v.y - s.vy, dvz = r.v.z - s.vz;
    const double rv = dx * dvx + dy * dvy + dz * dvz;
    const double rinv2 = rinv * rinv;
    const double mri = r.p.w * rinv;
    const double mr3i = mri * rinv2;
    double a3;
    if (HJ) {
      const double r2u = dx * dx + dy * dy + dz * dz;
      a3 = (CHECK && is_self) ? 0.0 : -3.0 * (rv / r2u);
    } else {
      a3 = -3.0 * (rv * rinv2);
    }
    q.a[0] = fma(mr3i, dx, q.a[0]);
    q.a[1] = fma(mr3i, dy, q.a[1]);
    q.a[2] = fma(mr3i, dz, q.a[2]);
    q.j[0] = fma(mr3i, fma(a3, dx, dvx), q.j[0]);
    q.j[1] = fma(mr3i, fma(a3, dy, dvy), q.j[1]);
    q.j[2] = fma(mr3i, fma(a3, dz, dvz), q.j[2]);
    q.p += mri;
  }
  __device__ static __forceinline__ bool rescan(const I &s, const Rec &r, double eps2,
                                                double best, int slot0, int self, int &idx) {
    double dx, dy, dz;
    if (r2e(s, r, eps2, dx, dy, dz) == best && slot0 != self) {
      idx = slot0;
      return true;
    }
    return false;
  }
  __device__ static void to_out(const Tot &t, double nnr2, int nn, Out &o) {
#pragma unroll
    for (int k = 0; k < 3; k++) {
      o.a[k] = t.a[k];
      o.j[k] = t.j[k];
    }
    o.p = t.p;
    o.nnr2 = nnr2;
    o.nn = nn;
    o.pad = 0;
  }
  __device__ static void merge(Out &a, const Out &b) {
#pragma unroll
    for (int k = 0; k < 3; k++) {
      a.a[k] += b.a[k];
      a.j[k] += b.j[k];
    }
    a.p += b.p;
    if (b.nnr2 < a.nnr2 || (b.nnr2 == a.nnr2 && b.nn < a.nn)) {
      a.nnr2 = b.nnr2;
      a.nn = b.nn;
    }
  }
  __device__ static void write_final(const Out &o, int i, double *acc, double *jerk,
                                     double *pot) {
#pragma unroll
    for (int k = 0; k < 3; k++) {
      acc[3 * i + k] = o.a[k];
      jerk[3 * i + k] = o.j[k];
    }
    pot[i] = -o.p;
  }
};

// Shuffle helpers for Out (field by field).
template <class O>
__device__ __forceinline__ O shfl_xor_out(const O &o, int m) {
  O r;
  const int *src = reinterpret_cast<const int *>(&o);
  int *dst = reinterpret_cast<int *>(&r);
#pragma unroll
  for (int w = 0; w < (int)(sizeof(O) / 4); w++) dst[w] = __shfl_xor_sync(0xffffffffu, src[w], m);
  return r;
}

struct KParams {
  int ni, nj, nsplit, jsplit;  // jsplit: j per CTA-split (multiple of TJ)
  double eps2;
  const double *ipos, *ivel;
  const int *ilist, *iself;
  const void *jrec;
  double *acc, *jerk, *pot;
  int *nn;
  float *nn_r2;
  void *part;  // [nsplit][ni_pad] Out records when nsplit > 1
  int ni_pad;
  int *err;
  int want_nn;
  int hjerk;  // the hermite code's jerk form (JL = 1, no nn only)
};

// Number of j per thread between compensated folds.
constexpr int FOLD_J = 64;

template <class P, int JL, bool NN, bool HJ = false>
__global__ void __launch_bounds__(NT, P::MINB) force_kernel(KParams kp) {
  constexpr int NSTAGE = P::NSTAGE;
  using Rec = typename P::Rec;
  using R = typename P::R;
  constexpr int JPR = P::JPR;            // j per record
  constexpr int IPT = P::IPT;            // i-particles per thread
  constexpr int RPT = TJ / JPR;          // records per tile
  constexpr int NIL = NT / JL;           // i-lanes per CTA
  constexpr int ISLOTS = NIL * IPT;      // i-particles per CTA
  constexpr int JPT = RPT / JL;          // records per thread per tile
  constexpr int FOLD_TILES = (FOLD_J / (JPT * JPR)) > 0 ? (FOLD_J / (JPT * JPR)) : 1;
  static_assert(JL >= 1 && JL <= JLMAX && JL <= RPT && (RPT % JL) == 0, "JL");

  __shared__ __align__(128) Rec tiles[NSTAGE][RPT];
  __shared__ __align__(8) uint64_t full[NSTAGE];
  __shared__ int released[NSTAGE];
  __shared__ int issued_s;
  __shared__ volatile int abort_s;

  const int tid = threadIdx.x;
  const int jl = tid % JL;
  const int il = tid / JL;
  const int lane = tid & 31;

  // ---- i-particles of this thread ----
  typename P::I I[IPT];
  int self[IPT];
  bool valid[IPT];
#pragma unroll
  for (int k = 0; k < IPT; k++) {
    const int i = blockIdx.x * ISLOTS + k * NIL + il;
    valid[k] = i < kp.ni;
    const int ii = valid[k] ? i : 0;
    if (kp.ilist) {
      const int slot = kp.ilist[ii];
      I[k] = P::load_i_slot(kp.jrec, slot);
      self[k] = valid[k] ? (kp.iself ? kp.iself[ii] : slot) : -1;
    } else {
      I[k] = P::load_i_explicit(kp.ipos + 3 * ii, kp.ivel + 3 * ii);
      self[k] = valid[k] && kp.iself ? kp.iself[ii] : -1;
    }
  }

  // ---- j-range of this CTA ----
  const int js = blockIdx.y * kp.jsplit;
  int je = js + kp.jsplit;
  const int nj_pad = (kp.nj + TJ - 1) / TJ * TJ;
  if (je > nj_pad) je = nj_pad;
  const int ntiles = je > js ? (je - js) / TJ : 0;
  const Rec *gj = reinterpret_cast<const Rec *>(kp.jrec) + js / JPR;

  constexpr int NWARP = NT / 32;
  if (tid == 0) {
#pragma unroll
    for (int s = 0; s < NSTAGE; s++) {
      mbar_init(&full[s], 1);
      released[s] = 0;
    }
    issued_s = ntiles < NSTAGE ? ntiles : NSTAGE;
    abort_s = 0;
    fence_barrier_init();
  }
  __syncthreads();
  if (tid == 0) {
    for (int s = 0; s < NSTAGE && s < ntiles; s++) {
      mbar_expect_tx(&full[s], RPT * sizeof(Rec));
      tma_load_1d(&tiles[s][0], gj + s * RPT, RPT * sizeof(Rec), &full[s]);
    }
  }

  const auto eps2 = P::eps(kp.eps2);  // eps^2 + 2^-52 (ph4)
  typename P::Part q[IPT];
  typename P::Tot T[IPT];
  R nnmin[IPT], nnbest[IPT];
  int nnidx[IPT], besttile[IPT];
#pragma unroll
  for (int k = 0; k < IPT; k++) {
    P::zero(q[k]);
    P::zero(T[k]);
    nnmin[k] = nnbest[k] = (R)__int_as_float(0x7f800000);
    nnidx[k] = -1;
    besttile[k] = -1;
  }

  // Warps consume tiles independently: no CTA barrier in the loop.  Each
  // warp releases a stage after reading it; the warp whose release completes
  // a use of the stage (all NWARP warps done) refills it with tile t+NSTAGE.
  // The per-stage release counter only grows: use k of stage s ends when it
  // reaches (k+1)*NWARP.
  bool failed = false;
  for (int t = 0; t < ntiles; t++) {
    const int s = t % NSTAGE;
    const bool ok = mbar_wait_abortable(&full[s], (t / NSTAGE) & 1, &abort_s);
    if (!__all_sync(0xffffffffu, ok)) {
      failed = true;
      if (lane == 0) abort_s = 1;
      break;
    }
    const Rec *tile = &tiles[s][0];
    const int tj0 = js + t * TJ;

    // Does this tile hold the self slot of any i of this warp?
    bool mine = false;
#pragma unroll
    for (int k = 0; k < IPT; k++) mine |= (unsigned)(self[k] - tj0) < (unsigned)TJ;
    const bool slow = __any_sync(0xffffffffu, mine);

    if (!slow) {
#pragma unroll UNROLL
      for (int u = 0; u < JPT; u++) {
        const Rec r = tile[jl + JL * u];
#pragma unroll
        for (int k = 0; k < IPT; k++)
          P::template pair<false, NN, HJ>(I[k], r, eps2, q[k], nnmin[k], 0);
      }
    } else {
      for (int u = 0; u < JPT; u++) {
        const int jj = jl + JL * u;
        const Rec r = tile[jj];
#pragma unroll
        for (int k = 0; k < IPT; k++)
          P::template pair<true, NN, HJ>(I[k], r, eps2, q[k], nnmin[k],
                                         self[k] - (tj0 + JPR * jj));
      }
    }

    // Nearest neighbour: remember the tile in which the running min last
    // improved (strict <, so the earliest tile wins ties); its index within
    // the tile is recovered once, after the loop.
#pragma unroll
    for (int k = 0; k < IPT; k++) {
      if (!NN) break;
      const bool imp = nnmin[k] < nnbest[k];
      nnbest[k] = imp ? nnmin[k] : nnbest[k];
      besttile[k] = imp ? t : besttile[k];
    }

    if ((t + 1) % FOLD_TILES == 0) {
#pragma unroll
      for (int k = 0; k < IPT; k++) {
        P::fold(T[k], q[k]);
        P::zero(q[k]);
      }
    }

    // Release stage s; the last releaser refills it.
    __syncwarp();
    if (lane == 0) {
      __threadfence_block();
      const int c = atomicAdd(&released[s], 1);
      if (c == (t / NSTAGE + 1) * NWARP - 1 && t + NSTAGE < ntiles) {
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
        mbar_expect_tx(&full[s], RPT * sizeof(Rec));
        tma_load_1d(&tiles[s][0], gj + (t + NSTAGE) * RPT, RPT * sizeof(Rec), &full[s]);
        atomicMax(&issued_s, t + NSTAGE + 1);
      }
    }
  }

  if (__syncthreads_or(failed)) {
    // Drain the copies still in flight (bounded) before the CTA leaves.
    if (tid == 0) {
      atomicOr(kp.err, ERR_TMA_TIMEOUT);
      const int hi = issued_s;
      for (int u = hi - NSTAGE > 0 ? hi - NSTAGE : 0; u < hi; u++)
        (void)mbar_wait_bounded(&full[u % NSTAGE], (u / NSTAGE) & 1);
    }
    return;
  }

  // ---- nearest neighbour: find the first j of the best tile (this lane's
  // j subset) whose r^2 equals the running min, with the same arithmetic,
  // reading the records back from global memory (L2). ----
#pragma unroll
  for (int k = 0; k < IPT; k++) {
    if (!NN || besttile[k] < 0) continue;
    const Rec *g = gj + besttile[k] * RPT;
    const int tj0 = js + besttile[k] * TJ;
    bool found = false;
    for (int u = 0; u < JPT && !found; u++) {
      const int jj = jl + JL * u;
      found = P::rescan(I[k], g[jj], eps2, nnbest[k], tj0 + JPR * jj, self[k], nnidx[k]);
    }
  }

  // ---- merge: fold remainders, then j-lanes, then (maybe) CTAs ----
  typename P::Out o[IPT];
#pragma unroll
  for (int k = 0; k < IPT; k++) {
    P::fold(T[k], q[k]);
    P::to_out(T[k], nnbest[k], nnidx[k], o[k]);
  }
  if (JL > 1) {
#pragma unroll
    for (int m = 1; m < (JL < 32 ? JL : 32); m <<= 1) {
#pragma unroll
      for (int k = 0; k < IPT; k++) {
        typename P::Out other = shfl_xor_out(o[k], m);
        // Lower lane first keeps the order fixed.
        if (lane & m) {
          P::merge(other, o[k]);
          o[k] = other;
        } else {
          P::merge(o[k], other);
        }
      }
    }
  }
  (void)lane;
  if (JL > 32) {
    // Cross-warp: warps w0..w0+JL/32-1 own one i-lane group.
    __syncthreads();
    typename P::Out *buf = reinterpret_cast<typename P::Out *>(&tiles[0][0]);
    static_assert(sizeof(typename P::Out) * IPT * (NT / 32) <= sizeof(Rec) * RPT * NSTAGE, "smem");
    const int warp = tid >> 5;
    if (lane == 0) {
#pragma unroll
      for (int k = 0; k < IPT; k++) buf[warp * IPT + k] = o[k];
    }
    __syncthreads();
    if (jl == 0) {
      constexpr int WPG = JL / 32;
#pragma unroll
      for (int k = 0; k < IPT; k++) {
        typename P::Out acc = buf[warp * IPT + k];
        for (int w = 1; w < WPG; w++) P::merge(acc, buf[(warp + w) * IPT + k]);
        o[k] = acc;
      }
    }
  }
  if (jl != 0) return;
#pragma unroll
  for (int k = 0; k < IPT; k++) {
    if (!valid[k]) continue;
    const int i = blockIdx.x * ISLOTS + k * NIL + il;
    if (kp.nsplit == 1) {
      P::write_final(o[k], i, kp.acc, kp.jerk, kp.pot);
      if (kp.nn) kp.nn[i] = (o[k].nn >= 0 && o[k].nn < kp.nj) ? o[k].nn : -1;
      if (kp.nn_r2) kp.nn_r2[i] = (float)o[k].nnr2;
    } else {
      reinterpret_cast<typename P::Out *>(kp.part)[(size_t)blockIdx.y * kp.ni_pad + i] = o[k];
    }
  }
}

// Second pass: merge the nsplit partial records of each i in split order
// (one thread per i; for large blocks).
template <class P>
__global__ void reduce_kernel(KParams kp) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= kp.ni) return;
  const typename P::Out *part = reinterpret_cast<const typename P::Out *>(kp.part);
  typename P::Out o = part[i];
  for (int s = 1; s < kp.nsplit; s++) P::merge(o, part[(size_t)s * kp.ni_pad + i]);
  P::write_final(o, i, kp.acc, kp.jerk, kp.pot);
  if (kp.nn) kp.nn[i] = (o.nn >= 0 && o.nn < kp.nj) ? o.nn : -1;
  if (kp.nn_r2) kp.nn_r2[i] = (float)o.nnr2;
}

// The same merge with one warp per i, for small blocks, where the splits are
// many and the i few (a thread walking 128 splits alone took ~90 us): lane l
// merges splits l, l+32, ... in order, then the lanes merge in a fixed
// shuffle-down tree.  Deterministic for a given (ni, nsplit).
template <class P>
__global__ void reduce_warp_kernel(KParams kp) {
  const int i = (int)((blockIdx.x * (size_t)blockDim.x + threadIdx.x) >> 5);
  const int lane = threadIdx.x & 31;
  if (i >= kp.ni) return;  // whole warps exit together
  const typename P::Out *part = reinterpret_cast<const typename P::Out *>(kp.part);
  typename P::Out o = part[(size_t)(lane < kp.nsplit ? lane : 0) * kp.ni_pad + i];
  for (int s = lane + 32; s < kp.nsplit; s += 32) P::merge(o, part[(size_t)s * kp.ni_pad + i]);
  const int have = kp.nsplit < 32 ? kp.nsplit : 32;  // lanes holding a partial
#pragma unroll
  for (int off = 16; off > 0; off >>= 1) {
    typename P::Out b;
    const int *src = reinterpret_cast<const int *>(&o);
    int *dst = reinterpret_cast<int *>(&b);
#pragma unroll
    for (int w = 0; w < (int)(sizeof(b) / 4); w++)
      dst[w] = __shfl_down_sync(0xffffffffu, src[w], off);
    if (lane < off && lane + off < have) P::merge(o, b);
  }
  if (lane == 0) {
    P::write_final(o, i, kp.acc, kp.jerk, kp.pot);
    if (kp.nn) kp.nn[i] = (o.nn >= 0 && o.nn < kp.nj) ? o.nn : -1;
    if (kp.nn_r2) kp.nn_r2[i] = (float)o.nnr2;
  }
}

int g_sms = 0;

int sm_count() {
  if (g_sms == 0) {
    int dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&g_sms, cudaDevAttrMultiProcessorCount, dev);
    if (g_sms <= 0) g_sms = 152;
  }
  return g_sms;
}

// Launch shape: JL from the i-block size, nsplit so that the grid covers
// about two resident CTAs per SM, with at least 4 tiles per split.
// Launch shape from a small cost model.  A CTA streams tiles_per tiles of
// its j-range; per tile each thread spends ~A issue slots of fixed work
// (wait, release, bookkeeping) plus B per j-record for its IPT i-particles
// (JPT = 256/JL records), plus F per CTA (i-loads, lane merges, output).
// Resident CTAs run in waves of MINB per SM, so
//   cost = waves * (tiles_per * (A + B * JPT) + F) * (1 + 0.002 * nsplit)
// (the last factor charges the partial-sum traffic of the second pass).
// Candidates: JL from the smallest that does not waste CTA i-slots up to
// 256 (more j-lanes = more CTAs for small blocks), and every distinct split
// count up to 4 resident waves' worth.  Large blocks (a full wave of CTAs at
// JL = 1) stay at JL = 1.  The last few shapes are cached (block steps
// repeat the same ni).
struct ShapeKey {
  int ni, nj, prec, fjl, fns;
  int jl, nsplit, jsplit;
};
ShapeKey g_shape_cache[256];

void choose_shape(int ni, int nj, int prec, int force_jl, int force_nsplit, int *jl_out,
                  int *nsplit_out, int *jsplit_out) {
  const unsigned h = ((unsigned)ni * 2654435761u ^ (unsigned)nj * 40503u ^ (unsigned)prec) & 255u;
  ShapeKey &c = g_shape_cache[h];
  if (c.ni == ni && c.nj == nj && c.prec == prec && c.fjl == force_jl && c.fns == force_nsplit &&
      c.jl > 0) {
    *jl_out = c.jl;
    *nsplit_out = c.nsplit;
    *jsplit_out = c.jsplit;
    return;
  }
  const int ntiles = nj > 0 ? (nj + TJ - 1) / TJ : 1;
  const int minb = prec == G6_PREC_FP64 ? F64P::MINB : SplitP::MINB;
  const int slots = minb * sm_count();
  const double A = 150.0, F = 3000.0;
  // per j and i: ~20 issue slots split (packed j pairs), ~37 x 32 FP64
  const int IPT = prec == G6_PREC_FP64 ? IPT_F64 : IPT_SPLIT;
  const double B = (prec == G6_PREC_FP64 ? 32.0 * 37.0 : 20.0) * IPT;
  int jl0 = 1;
  while (jl0 < JLMAX && (NT / (jl0 * 2)) * IPT >= ni && ni > 0) jl0 *= 2;
  int jl_lo = jl0, jl_hi = JLMAX;
  if (force_jl > 0) jl_lo = jl_hi = force_jl;
  else if (jl0 == 1 && (ni + (NT * IPT) - 1) / (NT * IPT) >= slots) jl_hi = 1;
  const int max_ns = ntiles < 4 * slots ? ntiles : 4 * slots;
  // Split counts: all small ones, then those from small tiles_per; each is
  // normalised to (tiles per split, splits), and repeats are dropped (a
  // repeat has the same cost and cannot win the strict comparison below).
  int cand_tp[512], cand_ns[512];
  int nc = 0;
  {
    int raw[512];
    int nr = 0;
    if (force_nsplit > 0) {
      raw[nr++] = force_nsplit;
    } else {
      for (int q = 1; q <= 128 && q <= max_ns; q++) raw[nr++] = q;
      for (int tp = 1; tp <= 256 && nr < 512; tp++) {
        const int q = (ntiles + tp - 1) / tp;
        if (q > 128 && q <= max_ns) raw[nr++] = q;
      }
    }
    for (int k = 0; k < nr; k++) {
      int ns = raw[k] < 1 ? 1 : raw[k];
      if (ns > ntiles) ns = ntiles;
      const int tp = (ntiles + ns - 1) / ns;
      if (nc > 0 && cand_tp[nc - 1] == tp) continue;
      cand_tp[nc] = tp;
      cand_ns[nc] = (ntiles + tp - 1) / tp;
      nc++;
    }
  }
  double best = 1e300;
  int bjl = jl_lo, bns = 1;
  for (int jl = jl_lo; jl <= jl_hi; jl *= 2) {
    const int islots = (NT / jl) * IPT;
    const long long gx = (ni + islots - 1) / islots;
    for (int k = 0; k < nc; k++) {
      const int tp = cand_tp[k], ns = cand_ns[k];
      const long long ctas = gx * ns;
      const long long waves = (ctas + slots - 1) / slots;
      const double cost =
          (double)waves * (tp * (A + B * (double)(TJ / jl)) + F) * (1.0 + 0.002 * ns);
      if (cost < best * 0.999) {
        best = cost;
        bjl = jl;
        bns = ns;
      }
    }
  }
  const int tp = (ntiles + bns - 1) / bns;
  *jl_out = bjl;
  *nsplit_out = (ntiles + tp - 1) / tp;
  *jsplit_out = tp * TJ;
  c.ni = ni;
  c.nj = nj;
  c.prec = prec;
  c.fjl = force_jl;
  c.fns = force_nsplit;
  c.jl = *jl_out;
  c.nsplit = *nsplit_out;
  c.jsplit = *jsplit_out;
}

template <class P>
int launch(const KParams &kp, int jl, int gx, cudaStream_t st) {
  dim3 grid(gx, kp.nsplit), block(NT);
  // Without nearest neighbours only the large-block shape has its own
  // instantiation; small blocks are latency-bound and keep the nn code.
  if (kp.hjerk) {
    if (jl != 1 || kp.want_nn) return -2;
    force_kernel<P, 1, false, true><<<grid, block, 0, st>>>(kp);
  } else switch (jl) {
#define G6_CASE(J)                                            \
  case J:                                                     \
    if (kp.want_nn)                                           \
      force_kernel<P, J, true><<<grid, block, 0, st>>>(kp);  \
    else                                                      \
      force_kernel<P, J, false><<<grid, block, 0, st>>>(kp); \
    break;
    G6_CASE(1)
    G6_CASE(2)
    G6_CASE(4)
    G6_CASE(8)
    G6_CASE(16)
    G6_CASE(32)
    G6_CASE(64)
    G6_CASE(128)
#if G6_NT >= 256
    G6_CASE(256)
#endif
#undef G6_CASE
    default:
      return -2;
  }
  if (kp.nsplit > 1) {
    if (kp.ni < 4096)
      reduce_warp_kernel<P><<<(kp.ni + 3) / 4, 128, 0, st>>>(kp);
    else
      reduce_kernel<P><<<(kp.ni + 127) / 128, 128, 0, st>>>(kp);
  }
  return cudaGetLastError() == cudaSuccess ? 0 : -3;
}

}  // namespace

extern "C" int g6k_sm_count(void) { return sm_count(); }

extern "C" size_t g6k_scratch_bytes(int ni, int nj, int prec, int force_jl, int force_nsplit) {
  int jl, nsplit, jsplit;
  choose_shape(ni, nj, prec, force_jl, force_nsplit, &jl, &nsplit, &jsplit);
  if (nsplit <= 1) return 0;
  const size_t rec = prec == G6_PREC_FP64 ? sizeof(F64P::Out) : sizeof(SplitP::Out);
  return (size_t)nsplit * (size_t)ni * rec;
}

extern "C" int g6k_force(const g6_force_args *a, g6_shape *shape, cudaStream_t st) {
  if (a->ni <= 0) return 0;
  if (a->nj <= 0 || !a->acc || !a->jerk || !a->pot || !a->js || !a->err) return -1;
  if (!a->ilist && (!a->ipos || !a->ivel)) return -1;
  if (a->hjerk && (a->want_nn || (a->force_jl != 0 && a->force_jl != 1))) return -2;
  int jl, nsplit, jsplit;
  choose_shape(a->ni, a->nj, a->prec, a->hjerk ? 1 : a->force_jl, a->force_nsplit, &jl, &nsplit,
               &jsplit);
  if (jl < 1 || jl > JLMAX || (jl & (jl - 1))) return -2;
  KParams kp;
  kp.ni = a->ni;
  kp.nj = a->nj;
  kp.nsplit = nsplit;
  kp.jsplit = jsplit;
  kp.eps2 = a->eps2;
  kp.ipos = a->ipos;
  kp.ivel = a->ivel;
  kp.ilist = a->ilist;
  kp.iself = a->iself;
  kp.acc = a->acc;
  kp.jerk = a->jerk;
  kp.pot = a->pot;
  kp.nn = a->nn;
  kp.nn_r2 = a->nn_r2;
  kp.part = a->scratch;
  kp.ni_pad = a->ni;
  kp.err = a->err;
  kp.want_nn = a->want_nn;
  kp.hjerk = a->hjerk;
  const size_t need = nsplit > 1 ? g6k_scratch_bytes(a->ni, a->nj, a->prec, jl, nsplit) : 0;
  if (need > a->scratch_bytes) return -4;
  const int islots = (NT / jl) * (a->prec == G6_PREC_FP64 ? IPT_F64 : IPT_SPLIT);
  const int gx = (a->ni + islots - 1) / islots;
  if (shape) {
    shape->jl = jl;
    shape->nsplit = nsplit;
    shape->grid_x = gx;
    shape->grid_y = nsplit;
    shape->threads = NT;
  }
  if (a->prec == G6_PREC_FP64) {
    kp.jrec = a->js->jp_f64;
    return launch<F64P>(kp, jl, gx, st);
  }
  kp.jrec = a->js->jp_split;
  return launch<SplitP>(kp, jl, gx, st);
}

// ---------------------------------------------------------------------------
// Fixed scratch for callers that cannot allocate device memory.
//
// The split-j partial sums normally live in a buffer that the host library
// grows with cudaMalloc on demand.  g6k_force_static instead places them in
// this file-scope array, which every GPU that loads the library holds (16 MiB)
// until the process exits.  Its device address is looked up once per device,
// on the first call made with that device current.  Every call shares the
// array: nothing in it has to start at zero (each partial record is written
// by exactly one CTA before the second pass reads it), and calls that overlap
// on the GPU (different streams, or host threads) race on it.
#define G6_STATIC_SCRATCH_BYTES (16u << 20)
static __device__ __align__(256) unsigned char g6_static_scratch[G6_STATIC_SCRATCH_BYTES];

extern "C" size_t g6k_static_scratch_capacity(void) { return G6_STATIC_SCRATCH_BYTES; }

// Returns 0, -1/-2/-3 as g6k_force, -4 when the launch shape needs more than
// G6_STATIC_SCRATCH_BYTES of scratch (*need_out tells how much), -5 when the
// array's device address cannot be obtained.
extern "C" int g6k_force_static(const g6_force_args *a, g6_shape *shape, cudaStream_t st,
                                size_t *need_out) {
  static void *addr[64];
  static int have[64];
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return -5;
  if (!have[dev]) {
    void *p = nullptr;
    if (cudaGetSymbolAddress(&p, g6_static_scratch) != cudaSuccess || p == nullptr) return -5;
    addr[dev] = p;
    have[dev] = 1;
  }
  const size_t need = g6k_scratch_bytes(a->ni, a->nj, a->prec, a->hjerk ? 1 : a->force_jl,
                                        a->force_nsplit);
  if (need_out) *need_out = need;
  if (need > G6_STATIC_SCRATCH_BYTES) return -4;
  g6_force_args b = *a;
  b.scratch = addr[dev];
  b.scratch_bytes = G6_STATIC_SCRATCH_BYTES;
  return g6k_force(&b, shape, st);
}
