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
#include "pdl.cuh"
#include <cuda_runtime.h>
#include <stddef.h>
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
#ifndef G6_UNROLL_NN
#define G6_UNROLL_NN 4  // j-loop unroll factor of the nearest-neighbour variant
#endif
#ifndef G6_ACHUNK
#define G6_ACHUNK 0  // split: fold the acceleration partials with the jerk's
#endif
#ifndef G6_UNROLL
#define G6_UNROLL 8
#endif
#ifndef G6_MINB
#define G6_MINB 3
#endif
#ifndef G6_IPT_F64
#define G6_IPT_F64 4
#endif
#ifndef G6_XMERGE_MAX
#define G6_XMERGE_MAX 2  // split merge in the force kernel up to this many i per group
#endif
#ifndef G6_JCHUNK
#define G6_JCHUNK 32  // split: records per jerk fold
#endif
#ifndef G6_TOT_SMEM
#define G6_TOT_SMEM 2  // split: compensated totals in shared memory (2: with NN only)
#endif
constexpr int NT = G6_NT;    // threads per CTA
constexpr int TJ = G6_TILE;  // j records per tile
// i-particles per thread: the split kernel's packed f32x2 pair terms need
// twice the registers per i, so it holds fewer i than the FP64 kernel.
constexpr int IPT_SPLIT = G6_IPT;
constexpr int IPT_F64 = G6_IPT_F64;
constexpr int UNROLL = G6_UNROLL;  // j-loop unroll factor (the best measured:
                                    // 8 plain, 4 with the nearest neighbour)
constexpr int JLMAX = TJ < NT ? TJ : NT;  // j-lanes per i at most
constexpr unsigned long long WAIT_NS = 2000000000ull;  // 2 s bound per wait
constexpr unsigned long long STALL_TEST_NS = 20000000ull;  // 20 ms under the test hook

enum { ERR_TMA_TIMEOUT = 1, ERR_SHAPE = 2 };

// Split records come in pairs of consecutive j slots, every field a float2
// {j even, j odd} (the global layout the predictor writes, g6_dev.h), so a
// packed f32x2 instruction evaluates two j at once.
struct __align__(16) RecS {
  float2 xh, yh, zh, m, xl, yl, zl, ml, vx, vy, vz, pad1;  // ml: the mass's low part
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
// *abort (false in both cases, or after limit_ns of global time).
__device__ __forceinline__ bool mbar_wait_abortable(uint64_t *bar, uint32_t parity,
                                                    volatile int *abort,
                                                    unsigned long long limit_ns) {
  if (mbar_try_wait(bar, parity)) return true;
  const unsigned long long t0 = gtimer();
  while (true) {
    if (mbar_try_wait(bar, parity)) return true;
    if (*abort) return false;
    if (gtimer() - t0 > limit_ns) return false;
  }
}
// Bounded wait: false after limit_ns of global time.
__device__ __forceinline__ bool mbar_wait_bounded(uint64_t *bar, uint32_t parity,
                                                  unsigned long long limit_ns) {
  if (mbar_try_wait(bar, parity)) return true;
  const unsigned long long t0 = gtimer();
  while (true) {
    if (mbar_try_wait(bar, parity)) return true;
    if (gtimer() - t0 > limit_ns) return false;
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

// max(a, b, c) and min(a, b, c) in one ALU instruction each (3-input
// max.f32 / min.f32).
__device__ __forceinline__ float fmax3(float a, float b, float c) {
  float r;
  asm("max.f32 %0, %1, %2, %3;" : "=f"(r) : "f"(a), "f"(b), "f"(c));
  return r;
}
__device__ __forceinline__ float fmin3(float a, float b, float c) {
  float r;
  asm("min.f32 %0, %1, %2, %3;" : "=f"(r) : "f"(a), "f"(b), "f"(c));
  return r;
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

struct KParams;

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
    f2x a[3], j[3], p, s;
  };
  struct Tot {  // compensated totals (s: plain sum, an estimate), largest chunk of s
    float ah[3], al[3], jh[3], jl[3], ph, pl, s, mt, pad;  // 17 words: odd stride
  };
  struct Out {  // partial record exchanged between CTAs, 80 B
    float2 a[3], j[3], p;
    float nnr2;   // smallest nearest-neighbour key (r^2 + eps^2, FP32)
    float nnr2b;  // second smallest key over the other j
    float s1;     // sum of m / (r^2 + eps^2): the condition number's numerator
    float mt;     // largest partial sum of s over 32 j: bounds the largest term
    int nn;
    int pad;
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
    q.s = 0ull;
  }
  __device__ static void zero(Tot &t) {
#pragma unroll
    for (int k = 0; k < 3; k++) t.ah[k] = t.al[k] = t.jh[k] = t.jl[k] = 0.f;
    t.ph = t.pl = 0.f;
    t.s = t.mt = 0.f;
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
    fold_s(t, q);
  }
  // The condition number's sum arrives in chunks of at most 32 j per half
  // (the jerk fold period): the largest chunk bounds the largest single term
  // m / (r^2 + eps^2) from above, for the price of one 3-input maximum per
  // chunk rather than per pair.
  __device__ static __forceinline__ void fold_s(Tot &t, const Part &q) {
    t.s += f2_lo(q.s) + f2_hi(q.s);
    t.mt = fmax3(t.mt, f2_lo(q.s), f2_hi(q.s));
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
  //
  // NN keeps the smallest key of the tile (nnmin, one 3-input minimum per j pair); the
  // kernel turns the tile minima into the smallest and second smallest key
  // over all j, whose gap decides whether the FP32 argmin is provably ph4's
  // FP64 nearest neighbour (finish() below).  Without HJ the sum of
  // m / (r^2 + eps^2) (Part::s) is kept for the condition number of the
  // acceleration sum.
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
        nnmin = fmin3(nnmin, selfrel == 0 ? inf : r2a, selfrel == 1 ? inf : r2b);
      }
    } else if (NN) {
      nnmin = fmin3(nnmin, r2a, r2b);
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
    if (!HJ) q.s = f2_fma(mri, rinv, q.s);  // the condition number's sum
  }
  // Nearest-neighbour re-scan of one record of the best tile: the first j
  // (in slot order) whose key equals best and that is not the i itself
  // becomes idx; every other key lowers m2 (the second smallest key).
  __device__ static __forceinline__ void rescan(const I &s, const Rec &r, f2x eps2, float best,
                                                int slot0, int self, int &idx, float &m2) {
    f2x dx, dy, dz;
    const f2x r2 = r2e(s, r, eps2, dx, dy, dz);
    const float kk[2] = {f2_lo(r2), f2_hi(r2)};
#pragma unroll
    for (int h = 0; h < 2; h++) {
      if (slot0 + h == self) continue;
      if (idx < 0 && kk[h] == best)
        idx = slot0 + h;
      else
        m2 = fminf(m2, kk[h]);
    }
  }
  // Mid-tile fold of the jerk partial sums (and of the condition number's
  // chunk): the jerk sum cancels more than the others, so it is folded every
  // JCHUNK records.
  static constexpr bool JFOLD = true;
  // shared-memory totals free registers: they pay off in the nearest-
  // neighbour variant, not in the plain one (measured)
  template <bool NN>
  __host__ __device__ static constexpr bool tot_shared() {
    return G6_TOT_SMEM == 1 || (G6_TOT_SMEM == 2 && NN);
  }
  __device__ static void fold_jerk(Tot &t, Part &q) {
    fold_s(t, q);
    q.s = 0ull;
#pragma unroll
    for (int k = 0; k < 3; k++) {
      ff_acc(t.jh[k], t.jl[k], f2_lo(q.j[k]));
      ff_acc(t.jh[k], t.jl[k], f2_hi(q.j[k]));
      q.j[k] = 0ull;
      if (G6_ACHUNK) {
        ff_acc(t.ah[k], t.al[k], f2_lo(q.a[k]));
        ff_acc(t.ah[k], t.al[k], f2_hi(q.a[k]));
        q.a[k] = 0ull;
      }
    }
  }
  __device__ static f2x eps(double eps2) {
    const float e = (float)eps2 + (float)(1.0 / 4503599627370496.0);  // + 2^-52 (ph4)
    return f2_pack(e, e);
  }
  __device__ static void to_out(const Tot &t, float nnr2, float nnr2b, int nn, Out &o) {
#pragma unroll
    for (int k = 0; k < 3; k++) {
      o.a[k] = make_float2(t.ah[k], t.al[k]);
      o.j[k] = make_float2(t.jh[k], t.jl[k]);
    }
    o.p = make_float2(t.ph, t.pl);
    o.nnr2 = nnr2;
    o.nnr2b = nnr2b;
    o.s1 = t.s;
    o.mt = t.mt;
    o.nn = nn;
    o.pad = 0;
  }
  __device__ static void merge(Out &a, const Out &b) {
#pragma unroll
    for (int k = 0; k < 3; k++) {
      ff_add(a.a[k].x, a.a[k].y, b.a[k].x, b.a[k].y);
      ff_add(a.j[k].x, a.j[k].y, b.j[k].x, b.j[k].y);
    }
    ff_add(a.p.x, a.p.y, b.p.x, b.p.y);
    a.s1 += b.s1;
    a.mt = fmaxf(a.mt, b.mt);
    // second smallest of the four keys: min(max of the minima, min of the seconds)
    const float m2 = fminf(fmaxf(a.nnr2, b.nnr2), fminf(a.nnr2b, b.nnr2b));
    if (b.nnr2 < a.nnr2 || (b.nnr2 == a.nnr2 && b.nn < a.nn)) {
      a.nnr2 = b.nnr2;
      a.nn = b.nn;
    }
    a.nnr2b = m2;
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
  __device__ static void finish(const Out &o, int i, const KParams &kp);
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
  struct Out {  // 72 B
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
  // ph4's nearest-neighbour key: the unsoftened r^2 summed in component
  // order without contraction (idata.cc:200-205,214-218), so the argmin
  // (first slot on equal keys) is ph4's nn bit for bit.
  __device__ static __forceinline__ double nnkey(double dx, double dy, double dz) {
    return __dadd_rn(__dadd_rn(__dmul_rn(dx, dx), __dmul_rn(dy, dy)), __dmul_rn(dz, dz));
  }
  template <bool CHECK, bool NN, bool HJ = false>
  __device__ static __forceinline__ void pair(const I &s, const Rec &r, double eps2, Part &q,
                                              double &nnmin, int selfrel) {
    const bool is_self = CHECK && selfrel == 0;
    double dx, dy, dz;
    const double r2 = r2e(s, r, eps2, dx, dy, dz);
    double rinv = rsqrt64(r2);
    if (CHECK) rinv = is_self ? 0.0 : rinv;
    if (NN) {
      const double key = nnkey(dx, dy, dz);
      nnmin = fmin(nnmin, is_self ? __longlong_as_double(0x7ff0000000000000ll) : key);
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
  __device__ static __forceinline__ void rescan(const I &s, const Rec &r, double eps2,
                                                double best, int slot0, int self, int &idx,
                                                double &m2) {
    (void)m2;  // the FP64 key is ph4's own: no gap to prove
    double dx, dy, dz;
    (void)r2e(s, r, eps2, dx, dy, dz);
    if (idx < 0 && slot0 != self && nnkey(dx, dy, dz) == best) idx = slot0;
  }
  static constexpr bool JFOLD = false;
  template <bool NN>
  __host__ __device__ static constexpr bool tot_shared() {
    return false;
  }
  __device__ static void fold_jerk(Tot &, Part &) {}
  __device__ static void to_out(const Tot &t, double nnr2, double nnr2b, int nn, Out &o) {
    (void)nnr2b;
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
  __device__ static void finish(const Out &o, int i, const KParams &kp);
};

// A partial record written by another CTA of this launch: read around L1.
template <class O>
__device__ __forceinline__ O load_out_cg(const O *p) {
  O r;
  const int *src = reinterpret_cast<const int *>(p);
  int *dst = reinterpret_cast<int *>(&r);
#pragma unroll
  for (int w = 0; w < (int)(sizeof(O) / 4); w++) dst[w] = __ldcg(src + w);
  return r;
}

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
  // nearest-neighbour proof and refinement queue (split precision)
  g6_jstate js;   // FP64 state: ph4-predicted positions of i and nn
  double ti;      // prediction time of the records
  void *refine;   // refinement buffer (NULL: none)
  double kappa2;  // squared condition-number limit (0: no FP64 redo)
  // bounded waits: limit per wait; stall (test hook) makes CTA (0, 0) wait
  // for its first tile on a barrier that nothing arrives on
  unsigned long long wait_ns;
  int stall;
  unsigned *xtick;  // per-i-group tickets for the in-kernel split merge (NULL: second pass)
};

// ------------------------------------------------ nearest neighbour proof ---
//
// ph4's nearest neighbour (idata.cc:200-226) is the j with the smallest FP64
// r^2 = (dx^2 + dy^2) + dz^2 of the ph4-predicted positions, the first j on
// equal values.  The split kernel ranks j by the FP32 key k = r^2 + eps^2
// of the double-single records.  Bound (the argument of kern_knn.cu, with
// the softening added first in the FMA chain): with X >= |coordinate| of i
// and of every j within distance sqrt(D) of i, E = 2^-30 X and e the FP32
// softening, any j with ph4 r^2 <= D has
//     k <= Tk(D) = (1 + 2^-16)(D + e) + 4 E sqrt(D) + 4 E^2.
// So if the second smallest key m2 exceeds Tk(D_f), D_f the FP64 r^2 of the
// FP32 argmin j_f, every other j has ph4 r^2 > D_f and j_f is ph4's nearest
// neighbour.  X = max |x_i| + sqrt(D_f) covers every j that could beat it.
// Otherwise (near-equal keys, e.g. distance ties) the i-particle is queued
// and refine_kernel ranks every j with k <= Tk(D_f) in FP64.
//
// ---------------------------------------------- condition-number refinement
//
// The FP32 pair terms carry a few ulps each, so the relative error of the
// acceleration grows with the condition number of its sum,
// kappa = sum m / (r^2 + eps^2) / |a| (about 1e-8 kappa at N = 2^20; the
// particles near the centre of a cluster, where the pulls cancel, reach
// kappa ~ 100-300), and with the largest single term over |a|, whose own
// error does not average out (a massive neighbour pulling against the rest
// of the cluster).  i-particles with kappa above the caller's limit are
// queued (REF_ACC), and refine_kernel recomputes their acceleration and
// potential in FP64 from the same records (double-single positions exact in
// FP64).  Those with kappa below it but a largest term (bounded by the
// largest partial sum over 32 j of one thread) above MU0 |a| are queued for
// the cheaper REF_MT pass: the sum redone with the kernel's FP32 pair terms
// but compensated (TwoSum) accumulation, every term above TAU |a| replaced
// by its FP64 value.  That removes the dominant terms' own errors and the
// FP32 partial sums' roundings relative to them, which are what does not
// average out there; the remaining terms are each below TAU |a|, so their
// random errors add up to ~1e-7 sqrt(TAU kappa) |a|.  Common in clusters
// with a mass spectrum (a massive star near the i), REF_MT costs ~50 FP32
// operations per pair where REF_ACC costs ~20 FP64 ones (each 1/64 the
// FP32 rate).  In both the jerk keeps its split value.
//
// Refinement buffer (g6k_refine_bytes, zeroed once): a header, the queue
// (i, reason, key bound), per-entry tickets, per-(entry, chunk) partial
// records, and the force kernel's per-i-group tickets for its in-kernel
// split merge.  refine_kernel leaves the header's count at zero.
constexpr int RCAP = 16384;    // queue entries
constexpr int RPCAP = 32768;   // partial records (entries x chunks)
constexpr int RCHMAX = 64;     // j-chunks per entry at most
constexpr int RNT = 256;       // refine_kernel threads per CTA
constexpr int XTMAX = 8192;    // i-groups (grid.x) whose split merge runs in the force kernel
enum { REF_ACC = 1, REF_NN = 2, REF_MT = 4 };
// Largest single term over |a| above which the sum is redone (REF_MT): a
// term carries up to ~7e-7 relative error (three times the 1.25e-7 of the
// MUFU reciprocal square root, measured over all FP32 inputs in [1, 4), plus
// the roundings of r^2, the differences and the products), and a partial
// sum holding it rounds every later term to its own ulp.  At 1.5 a particle
// with a term of 1.4 |a| reached 1.23e-6 (a star pulling against a cluster,
// 6000 bodies); at 1.0 the worst left unrefined is one term's error.
constexpr double MU0 = 1.0;
// Terms above TAU |a| are evaluated in FP64 in the REF_MT pass.  A warp
// takes the FP64 branch whenever one of its lanes does, at 1/64 of the FP32
// rate, so TAU is kept where few terms reach it: at 0.02 the remaining
// terms' random errors stay below ~1e-7 sqrt(0.02 kappa) |a| (C2 at 65536
// Salpeter: the same largest error as at 0.005, and the block loop 2 %
// faster).
#ifndef G6_REF_UNITS
#define G6_REF_UNITS 4  // refine_kernel: (entry, j-chunk) units per CTA to aim for
#endif
#ifndef G6_TAU
#define G6_TAU 0.02f
#endif
constexpr float TAU = G6_TAU;

struct RefHdr {
  unsigned count;     // entries queued by this call (reset by refine_kernel)
  unsigned done;      // refine_kernel CTAs finished
  unsigned overflow;  // largest count that exceeded RCAP (sticky until read)
  unsigned last;      // count of the last refinement
  unsigned last_acc;  // of which queued for the condition number
  unsigned nacc;      // REF_ACC entries queued by this call
  unsigned nmt;       // REF_MT entries queued by this call
  unsigned last_mt;   // of the last refinement
};
struct RefPart {  // one j-chunk of one entry, FP64
  double a[3], p, r2;
  int slot, pad;
};
struct RefBuf {
  RefHdr h;
  int list[RCAP];
  int mode[RCAP];
  float thr[RCAP];     // REF_NN: the FP32 key bound
  float thr_mt[RCAP];  // REF_MT: TAU |a|
  unsigned ticket[RCAP];
  RefPart part[RPCAP];
  unsigned xtick[XTMAX];  // force kernel: CTAs of an i-group done (reset by the last)
};

__device__ __forceinline__ double dsub(double a, double b) { return __dsub_rn(a, b); }

// FP64 position of j slot s predicted to ti with ph4's expression.
__device__ __forceinline__ void jpos64(const g6_jstate &js, double ti, int s, double x[3]) {
  const int cap = js.cap;
  const double dt = dsub(ti, js.t[s]);
#pragma unroll
  for (int k = 0; k < 3; k++)
    x[k] = g6_predict_x(js.x[k * cap + s], js.v[k * cap + s], js.a[k * cap + s],
                        js.j[k * cap + s], dt);
}
// FP64 position of i-particle i as ph4 holds it: the caller's point, or the
// listed slot predicted to ti.
__device__ __forceinline__ void ipos64(const KParams &kp, int i, double x[3]) {
  if (kp.ilist) {
    jpos64(kp.js, kp.ti, kp.ilist[i], x);
  } else {
#pragma unroll
    for (int k = 0; k < 3; k++) x[k] = kp.ipos[3 * i + k];
  }
}
// ph4's r^2 of j relative to i (dx = x_j - x_i), component order, no FMA.
__device__ __forceinline__ double ph4_r2(const double xi[3], const double xj[3]) {
  const double d0 = dsub(xj[0], xi[0]), d1 = dsub(xj[1], xi[1]), d2 = dsub(xj[2], xi[2]);
  return __dadd_rn(__dadd_rn(__dmul_rn(d0, d0), __dmul_rn(d1, d1)), __dmul_rn(d2, d2));
}
// Tk(D) of the header, rounded up to FP32.
__device__ __forceinline__ float nn_bound(double D, double e, const double xi[3]) {
  const double sD = sqrt(D);
  const double X = fmax(fabs(xi[0]), fmax(fabs(xi[1]), fabs(xi[2]))) + sD * (1.0 + 1.0 / 1048576.0);
  const double E = X * (1.0 + 1.0 / 1048576.0) * (1.0 / 1073741824.0);
  const double T = (1.0 + 1.0 / 65536.0) * (D + e) + 4.0 * E * sD + 4.0 * E * E;
  return __double2float_ru(T);
}
// The FP32 softening of the split key (SplitP::eps), as a double.
__device__ __forceinline__ double split_eps(double eps2) {
  return (double)((float)eps2 + (float)(1.0 / 4503599627370496.0));
}

__device__ __forceinline__ void ref_enqueue(void *buf, int i, int mode, float thr,
                                            float thr_mt) {
  RefBuf *b = reinterpret_cast<RefBuf *>(buf);
  const unsigned e = atomicAdd(&b->h.count, 1u);
  if (mode & REF_ACC) atomicAdd(&b->h.nacc, 1u);
  if (mode & REF_MT) atomicAdd(&b->h.nmt, 1u);
  if (e < (unsigned)RCAP) {
    b->list[e] = i;
    b->mode[e] = mode;
    b->thr[e] = thr;
    b->thr_mt[e] = thr_mt;
  }
}

__device__ __noinline__ void SplitP::finish(const Out &o, int i, const KParams &kp) {
  write_final(o, i, kp.acc, kp.jerk, kp.pot);
  int mode = 0;
  float thr = 0.f, thr_mt = 0.f;
  if (kp.refine && kp.kappa2 > 0.0) {
    double a2 = 0.0;
#pragma unroll
    for (int k = 0; k < 3; k++) {
      const double a = (double)o.a[k].x + (double)o.a[k].y;
      a2 += a * a;
    }
    const double s1 = (double)o.s1, mt = (double)o.mt;
    if (s1 * s1 > kp.kappa2 * a2) {
      mode |= REF_ACC;
    } else if (mt * mt > MU0 * MU0 * a2) {
      mode |= REF_MT;
      thr_mt = (float)((double)TAU * sqrt(a2));
    }
  }
  const int nn = (o.nn >= 0 && o.nn < kp.nj) ? o.nn : -1;
  if (kp.want_nn) {
    float r2out = __int_as_float(0x7f800000);
    if (nn >= 0) {
      double xi[3], xj[3];
      ipos64(kp, i, xi);
      jpos64(kp.js, kp.ti, nn, xj);
      const double D = ph4_r2(xi, xj);
      r2out = (float)D;
      const float T = nn_bound(D, split_eps(kp.eps2), xi);
      if (kp.refine && !(o.nnr2b > T)) {
        mode |= REF_NN;
        thr = T;
      }
    }
    if (kp.nn) kp.nn[i] = nn;
    if (kp.nn_r2) kp.nn_r2[i] = r2out;
  } else if (kp.nn) {
    kp.nn[i] = -1;
  }
  if (mode) ref_enqueue(kp.refine, i, mode, thr, thr_mt);
}

__device__ __noinline__ void F64P::finish(const Out &o, int i, const KParams &kp) {
  write_final(o, i, kp.acc, kp.jerk, kp.pot);
  const int nn = (o.nn >= 0 && o.nn < kp.nj) ? o.nn : -1;
  if (kp.nn) kp.nn[i] = kp.want_nn ? nn : -1;
  if (kp.nn_r2) kp.nn_r2[i] = nn >= 0 ? (float)o.nnr2 : __int_as_float(0x7f800000);
}

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
  constexpr int JCHUNK = JPT < G6_JCHUNK ? JPT : G6_JCHUNK;  // records per jerk fold (split)
  static_assert(JL >= 1 && JL <= JLMAX && JL <= RPT && (RPT % JL) == 0, "JL");

  __shared__ __align__(128) Rec tiles[NSTAGE][RPT];
  __shared__ __align__(8) uint64_t full[NSTAGE];
  __shared__ __align__(8) uint64_t never;  // test hook: no arrival ever
  __shared__ int released[NSTAGE];
  __shared__ int issued_s;
  __shared__ volatile int abort_s;

  const int tid = threadIdx.x;
  const int jl = tid % JL;
  const int il = tid / JL;
  const int lane = tid & 31;
  pdl_wait();  // the predictor's records and the block list are complete

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
    mbar_init(&never, 1);
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
  // Compensated totals: in shared memory for the split nearest-neighbour
  // variant (touched once per fold; it frees registers for the pair loop),
  // in registers otherwise.  Layout [k][thread]: 17-word records,
  // conflict-free.
  constexpr bool TSH = P::template tot_shared<NN>();
  __shared__ typename P::Tot tot_sh[TSH ? IPT * NT : 1];
  typename P::Tot tot_reg[TSH ? 1 : IPT];
  auto T = [&](int k) -> typename P::Tot & {
    if constexpr (TSH)
      return tot_sh[k * NT + threadIdx.x];
    else
      return tot_reg[k];
  };
  R nnmin[IPT], nnbest[IPT], nnm2[IPT];
  int nnidx[IPT], besttile[IPT];
#pragma unroll
  for (int k = 0; k < IPT; k++) {
    P::zero(q[k]);
    P::zero(T(k));
    nnmin[k] = nnbest[k] = nnm2[k] = (R)__int_as_float(0x7f800000);
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
    const bool stall = kp.stall && t == 0 && blockIdx.x == 0 && blockIdx.y == 0;
    const bool ok = stall ? mbar_wait_abortable(&never, 0, &abort_s, kp.wait_ns)
                          : mbar_wait_abortable(&full[s], (t / NSTAGE) & 1, &abort_s, kp.wait_ns);
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

    // JCHUNK records between jerk folds (split: the jerk partials are
    // folded more often than the rest; the last chunk folds with the tile).
    if (!slow) {
#pragma unroll 1
      for (int ub = 0; ub < JPT; ub += JCHUNK) {
        constexpr int UNR = NN ? G6_UNROLL_NN : UNROLL;
#pragma unroll UNR
        for (int u = ub; u < ub + JCHUNK; u++) {
          const Rec r = tile[jl + JL * u];
#pragma unroll
          for (int k = 0; k < IPT; k++)
            P::template pair<false, NN, HJ>(I[k], r, eps2, q[k], nnmin[k], 0);
        }
        if (P::JFOLD && ub + JCHUNK < JPT) {
#pragma unroll
          for (int k = 0; k < IPT; k++) P::fold_jerk(T(k), q[k]);
        }
      }
    } else {
      for (int u = 0; u < JPT; u++) {
        const int jj = jl + JL * u;
        const Rec r = tile[jj];
#pragma unroll
        for (int k = 0; k < IPT; k++)
          P::template pair<true, NN, HJ>(I[k], r, eps2, q[k], nnmin[k],
                                         self[k] - (tj0 + JPR * jj));
        if (P::JFOLD && (u + 1) % JCHUNK == 0 && u + 1 < JPT) {
#pragma unroll
          for (int k = 0; k < IPT; k++) P::fold_jerk(T(k), q[k]);
        }
      }
    }

    // Nearest neighbour: nnmin holds this tile's smallest key.  Keep the
    // smallest over the tiles (nnbest) and the tile where it occurs (strict
    // <, so the earliest tile wins ties; the index within the tile is
    // recovered once, after the loop), and fold the larger of the tile's
    // and the running minimum into the second smallest key (nnm2).
#pragma unroll
    for (int k = 0; k < IPT; k++) {
      if (!NN) break;
      const R tmin = nnmin[k];
      nnm2[k] = fmin(nnm2[k], fmax(tmin, nnbest[k]));
      const bool imp = tmin < nnbest[k];
      nnbest[k] = imp ? tmin : nnbest[k];
      besttile[k] = imp ? t : besttile[k];
      nnmin[k] = (R)__int_as_float(0x7f800000);
    }

    if ((t + 1) % FOLD_TILES == 0) {
#pragma unroll
      for (int k = 0; k < IPT; k++) {
        P::fold(T(k), q[k]);
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

  pdl_trigger();  // j loop done: the next kernel of the chain may be scheduled
  if (__syncthreads_or(failed)) {
    // Drain the copies still in flight (bounded) before the CTA leaves.
    if (tid == 0) {
      atomicOr(kp.err, ERR_TMA_TIMEOUT);
      const int hi = issued_s;
      for (int u = hi - NSTAGE > 0 ? hi - NSTAGE : 0; u < hi; u++)
        (void)mbar_wait_bounded(&full[u % NSTAGE], (u / NSTAGE) & 1, kp.wait_ns);
      // Still count this CTA in its i-group, so that the group's ticket
      // returns to zero for the next launch (the results are void: the
      // error word is set).
      if (kp.nsplit > 1 && kp.xtick &&
          atomicAdd(&kp.xtick[blockIdx.x], 1u) == (unsigned)(kp.nsplit - 1))
        kp.xtick[blockIdx.x] = 0u;
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
    for (int u = 0; u < JPT; u++) {
      const int jj = jl + JL * u;
      P::rescan(I[k], g[jj], eps2, nnbest[k], tj0 + JPR * jj, self[k], nnidx[k], nnm2[k]);
    }
  }

  // ---- merge: fold remainders, then j-lanes, then (maybe) CTAs ----
  typename P::Out o[IPT];
#pragma unroll
  for (int k = 0; k < IPT; k++) {
    P::fold(T(k), q[k]);
    P::to_out(T(k), nnbest[k], nnm2[k], nnidx[k], o[k]);
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
  if (jl == 0) {
#pragma unroll
    for (int k = 0; k < IPT; k++) {
      if (!valid[k]) continue;
      const int i = blockIdx.x * ISLOTS + k * NIL + il;
      if (kp.nsplit == 1) {
        P::finish(o[k], i, kp);
      } else {
        reinterpret_cast<typename P::Out *>(kp.part)[(size_t)blockIdx.y * kp.ni_pad + i] = o[k];
      }
    }
  }
  if (kp.nsplit == 1 || !kp.xtick) return;

  // ---- split merge in the last CTA of the i-group (no second launch): the
  // CTA whose ticket completes the group merges the nsplit partial records
  // of each of the group's i, a warp per i, lane l taking splits l, l+32, ...
  // in order and the lanes merging in a fixed shuffle-down tree (as
  // reduce_warp_kernel).  The ticket is reset for the next launch. ----
  __shared__ int last_s;
  __threadfence();
  __syncthreads();
  if (tid == 0) last_s = atomicAdd(&kp.xtick[blockIdx.x], 1u) == (unsigned)(kp.nsplit - 1);
  __syncthreads();
  if (!last_s) return;
  __threadfence();
  using Out = typename P::Out;
  const Out *part = reinterpret_cast<const Out *>(kp.part);
  const int warp = tid >> 5;
  const int i0 = blockIdx.x * ISLOTS;
  for (int qq = warp; qq < ISLOTS; qq += NWARP) {
    const int i = i0 + qq;
    if (i >= kp.ni) break;
    Out m = load_out_cg(part + (size_t)(lane < kp.nsplit ? lane : 0) * kp.ni_pad + i);
    for (int sp = lane + 32; sp < kp.nsplit; sp += 32)
      P::merge(m, load_out_cg(part + (size_t)sp * kp.ni_pad + i));
    const int have = kp.nsplit < 32 ? kp.nsplit : 32;
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) {
      Out b;
      const int *src = reinterpret_cast<const int *>(&m);
      int *dst = reinterpret_cast<int *>(&b);
#pragma unroll
      for (int w = 0; w < (int)(sizeof(Out) / 4); w++)
        dst[w] = __shfl_down_sync(0xffffffffu, src[w], off);
      if (lane < off && lane + off < have) P::merge(m, b);
    }
    if (lane == 0) P::finish(m, i, kp);
  }
  if (tid == 0) kp.xtick[blockIdx.x] = 0u;
}

// Second pass: merge the nsplit partial records of each i in split order
// (one thread per i; for large blocks).
template <class P>
__global__ void reduce_kernel(KParams kp) {
  pdl_wait();
  pdl_trigger();
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= kp.ni) return;
  const typename P::Out *part = reinterpret_cast<const typename P::Out *>(kp.part);
  typename P::Out o = part[i];
  for (int s = 1; s < kp.nsplit; s++) P::merge(o, part[(size_t)s * kp.ni_pad + i]);
  P::finish(o, i, kp);
}

// The same merge with one warp per i, for small blocks, where the splits are
// many and the i few (a thread walking 128 splits alone took ~90 us): lane l
// merges splits l, l+32, ... in order, then the lanes merge in a fixed
// shuffle-down tree.  Deterministic for a given (ni, nsplit).
template <class P>
__global__ void reduce_warp_kernel(KParams kp) {
  pdl_wait();
  pdl_trigger();
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
  if (lane == 0) P::finish(o, i, kp);
}

// FP64 redo of the queued i-particles (see "nearest neighbour proof" and
// "condition-number refinement" above).  A persistent grid walks the
// (entry, j-chunk) units; each CTA reduces its unit in a fixed order and the
// CTA that completes an entry's last chunk (atomic ticket) merges the chunks
// in chunk order and overwrites that particle's results.  The chunk count
// depends only on the number of queued entries, so results are
// deterministic.  The last CTA to finish resets the queue.
//
// 1/sqrt(x): FP32 MUFU seed (relative error < 2^-22) and one Newton step,
// relative error < 2^-42, far below the 1e-6 the pass is for.
__device__ __forceinline__ double refine_rsqrt(double x) {
  double y = (double)rsqrt_approx((float)x);
  return y * __fma_rn(-0.5 * x * y, y, 1.5);
}

// One j of a REF_MT entry: the force kernel's FP32 term (same operations,
// so the same value up to the final product's rounding) into compensated
// FP32 sums, or, above thr = TAU |a|, the FP64 term into the FP64 sums.
__device__ __forceinline__ void mt_term(float xh, float yh, float zh, float m, float ml, float xl,
                                        float yl, float zl, const float ih[3], const float il[3],
                                        const double xi[3], float e32, double eps2, float thr,
                                        double sa[3], double &sp, float ah[3], float al[3],
                                        float &ph, float &pl) {
  const float jh[3] = {xh, yh, zh}, jl[3] = {xl, yl, zl};
  float d[3];
#pragma unroll
  for (int k = 0; k < 3; k++) d[k] = __fadd_rn(__fsub_rn(jh[k], ih[k]), __fsub_rn(jl[k], il[k]));
  const float r2f = __fmaf_rn(d[2], d[2], __fmaf_rn(d[1], d[1], __fmaf_rn(d[0], d[0], e32)));
  const float rinv = rsqrt_approx(r2f);
  const float mri = __fmul_rn(m, rinv);
  if (__fmul_rn(mri, rinv) > thr) {
    double dx[3];
#pragma unroll
    for (int k = 0; k < 3; k++) dx[k] = ((double)jh[k] + (double)jl[k]) - xi[k];
    const double r2 = __fma_rn(dx[2], dx[2], __fma_rn(dx[1], dx[1], __fma_rn(dx[0], dx[0], eps2)));
    const double ri = refine_rsqrt(r2);
    const double mr = ((double)m + (double)ml) * ri;
    const double mr3 = mr * (ri * ri);
#pragma unroll
    for (int k = 0; k < 3; k++) sa[k] = __fma_rn(mr3, dx[k], sa[k]);
    sp += mr;
  } else {
    // the FP32 term with the mass's high part, compensated; its low part
    // (2^-24 of the term) goes straight into the low words
    const float r3 = __fmul_rn(rinv, __fmul_rn(rinv, rinv));
    const float mr3i = __fmul_rn(mri, __fmul_rn(rinv, rinv));
    const float lr3 = __fmul_rn(ml, r3);
#pragma unroll
    for (int k = 0; k < 3; k++) {
      ff_acc(ah[k], al[k], __fmul_rn(mr3i, d[k]));
      al[k] = __fmaf_rn(lr3, d[k], al[k]);
    }
    ff_acc(ph, pl, mri);
    pl = __fmaf_rn(ml, rinv, pl);
  }
}

__global__ void __launch_bounds__(RNT) refine_kernel(KParams kp) {
  pdl_wait();
  pdl_trigger();
  RefBuf *b = reinterpret_cast<RefBuf *>(kp.refine);
  __shared__ unsigned s_cnt;
  __shared__ double s_sum[RNT / 32][5];
  __shared__ int s_slot[RNT / 32];
  __shared__ int s_last;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  if (tid == 0) s_cnt = *reinterpret_cast<volatile unsigned *>(&b->h.count);
  __syncthreads();
  const unsigned cnt = s_cnt;
  if (cnt == 0) {  // nothing queued (most calls): record that and leave
    if (blockIdx.x == 0 && tid == 0) b->h.last = b->h.last_acc = b->h.last_mt = 0u;
    return;
  }
  const int ne = cnt > (unsigned)RCAP ? 0 : (int)cnt;
  if (cnt > (unsigned)RCAP && blockIdx.x == 0 && tid == 0) atomicMax(&b->h.overflow, cnt);
  int nch = 1;
  if (ne > 0) {
    // About one unit per CTA while the entries are few (each unit then
    // covers more j and the CTA reduces once); four per CTA once they are
    // many, for balance (measured on config 2's blocks: 8 entries 34 -> 24
    // us, 25 entries 68 -> 40 us at one per CTA; 366 entries 282 us at four,
    // 652 us at one)
    const int upc = ne * 4 > (int)gridDim.x ? G6_REF_UNITS : 1;
    nch = (upc * (int)gridDim.x + ne - 1) / ne;
    nch = min(nch, RCHMAX);
    nch = min(nch, RPCAP / ne);
    nch = min(nch, max(1, kp.nj / 1024));
    nch = max(nch, 1);
  }
  const int units = ne * nch;
  const double eps2 = kp.eps2 + 1.0 / 4503599627370496.0;  // ph4's + 2^-52
  const float e32 = (float)split_eps(kp.eps2);
  const double inf = __longlong_as_double(0x7ff0000000000000ll);
  const void *rec = kp.jrec;
  for (int u = blockIdx.x; u < units; u += gridDim.x) {
    const int e = u / nch, c = u - e * nch;
    const int i = b->list[e];
    const int mode = b->mode[e];
    const float thr = b->thr[e], thr_mt = b->thr_mt[e];
    // chunk c: record pairs [p0, p1) (j from 2 p0 to 2 p1, nj at most)
    const int npair = (kp.nj + 1) >> 1;
    const int p0 = (int)((long long)npair * c / nch);
    const int p1 = (int)((long long)npair * (c + 1) / nch);
    const int j0 = 2 * p0;
    const int j1 = 2 * p1 < kp.nj ? 2 * p1 : kp.nj;
    // The i-particle in the split kernel's own representation (double-single
    // position), so that an i and a j copy of it at the same place give
    // dx = 0 exactly, as there.
    int self;
    double xi[3], xi64[3];
    float ih[3], il[3];
    if (kp.ilist) {
      const int slot = kp.ilist[i];
      self = kp.iself ? kp.iself[i] : slot;
#pragma unroll
      for (int k = 0; k < 3; k++) {
        ih[k] = g6_split_get(rec, slot, k);
        il[k] = g6_split_get(rec, slot, 4 + k);
      }
    } else {
      self = kp.iself ? kp.iself[i] : -1;
#pragma unroll
      for (int k = 0; k < 3; k++) SplitP::split(kp.ipos[3 * i + k], ih[k], il[k]);
    }
#pragma unroll
    for (int k = 0; k < 3; k++) xi[k] = (double)ih[k] + (double)il[k];
    if (mode & REF_NN) ipos64(kp, i, xi64);
    double sa[3] = {0.0, 0.0, 0.0}, sp = 0.0;
    float ah[3] = {0.f, 0.f, 0.f}, al[3] = {0.f, 0.f, 0.f}, ph = 0.f, pl = 0.f;  // REF_MT
    double br2 = inf;
    int bslot = -1;
    if (mode == REF_MT) {
      // the common case alone: whole record pairs in four 16-byte loads,
      // two pairs in flight per thread
      const float4 *q4 = reinterpret_cast<const float4 *>(rec);
#pragma unroll 2
      for (int rp = p0 + tid; rp < p1; rp += RNT) {
        const float4 A = __ldg(q4 + 6 * rp), B = __ldg(q4 + 6 * rp + 1);
        const float4 C = __ldg(q4 + 6 * rp + 2), D = __ldg(q4 + 6 * rp + 3);
        if (2 * rp != self && 2 * rp < kp.nj)
          mt_term(A.x, A.z, B.x, B.z, D.z, C.x, C.z, D.x, ih, il, xi, e32, eps2, thr_mt, sa, sp,
                  ah, al, ph, pl);
        if (2 * rp + 1 != self && 2 * rp + 1 < kp.nj)
          mt_term(A.y, A.w, B.y, B.w, D.w, C.y, C.w, D.y, ih, il, xi, e32, eps2, thr_mt, sa, sp,
                  ah, al, ph, pl);
      }
    }
    for (int j = j0 + tid; mode != REF_MT && j < j1; j += RNT) {
      if (j == self) continue;
      if (mode & REF_MT)
        mt_term(g6_split_get(rec, j, 0), g6_split_get(rec, j, 1), g6_split_get(rec, j, 2),
                g6_split_get(rec, j, 3), g6_split_get(rec, j, 7), g6_split_get(rec, j, 4),
                g6_split_get(rec, j, 5), g6_split_get(rec, j, 6), ih, il, xi, e32, eps2, thr_mt,
                sa, sp, ah, al, ph, pl);
      if (mode & REF_ACC) {  // acceleration and potential; the jerk stays
        double dx[3];
#pragma unroll
        for (int k = 0; k < 3; k++)
          dx[k] = ((double)g6_split_get(rec, j, k) + (double)g6_split_get(rec, j, 4 + k)) - xi[k];
        const double m = (double)g6_split_get(rec, j, 3) + (double)g6_split_get(rec, j, 7);
        const double r2 = __fma_rn(dx[2], dx[2], __fma_rn(dx[1], dx[1], __fma_rn(dx[0], dx[0], eps2)));
        const double rinv = refine_rsqrt(r2);
        const double mri = m * rinv;
        const double mr3i = mri * (rinv * rinv);
#pragma unroll
        for (int k = 0; k < 3; k++) sa[k] = __fma_rn(mr3i, dx[k], sa[k]);
        sp += mri;
      }
      if (mode & REF_NN) {
        float d[3];
#pragma unroll
        for (int k = 0; k < 3; k++)
          d[k] = __fadd_rn(__fsub_rn(g6_split_get(rec, j, k), ih[k]),
                           __fsub_rn(g6_split_get(rec, j, 4 + k), il[k]));
        const float key = __fmaf_rn(d[2], d[2], __fmaf_rn(d[1], d[1], __fmaf_rn(d[0], d[0], e32)));
        if (key <= thr) {
          double xj[3];
          jpos64(kp.js, kp.ti, j, xj);
          const double r2 = ph4_r2(xi64, xj);
          if (r2 < br2 || (r2 == br2 && j < bslot)) {
            br2 = r2;
            bslot = j;
          }
        }
      }
    }
    if (mode & REF_MT) {
#pragma unroll
      for (int k = 0; k < 3; k++) sa[k] += (double)ah[k] + (double)al[k];
      sp += (double)ph + (double)pl;
    }
    // fixed-order reduction: shuffle-down tree, then warps in order
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) {
#pragma unroll
      for (int k = 0; k < 3; k++) sa[k] += __shfl_down_sync(0xffffffffu, sa[k], off);
      sp += __shfl_down_sync(0xffffffffu, sp, off);
      const double or2 = __shfl_down_sync(0xffffffffu, br2, off);
      const int os = __shfl_down_sync(0xffffffffu, bslot, off);
      if (or2 < br2 || (or2 == br2 && os >= 0 && (bslot < 0 || os < bslot))) {
        br2 = or2;
        bslot = os;
      }
    }
    if (lane == 0) {
      for (int k = 0; k < 3; k++) s_sum[warp][k] = sa[k];
      s_sum[warp][3] = sp;
      s_sum[warp][4] = br2;
      s_slot[warp] = bslot;
    }
    __syncthreads();
    if (tid == 0) {
      RefPart q;
      for (int k = 0; k < 3; k++) q.a[k] = 0.0;
      q.p = 0.0;
      q.r2 = inf;
      q.slot = -1;
      q.pad = 0;
      for (int w = 0; w < RNT / 32; w++) {
        for (int k = 0; k < 3; k++) q.a[k] += s_sum[w][k];
        q.p += s_sum[w][3];
        if (s_slot[w] >= 0 && (s_sum[w][4] < q.r2 || (s_sum[w][4] == q.r2 && s_slot[w] < q.slot))) {
          q.r2 = s_sum[w][4];
          q.slot = s_slot[w];
        }
      }
      b->part[e * nch + c] = q;
      __threadfence();
      s_last = atomicAdd(&b->ticket[e], 1u) == (unsigned)(nch - 1);
    }
    __syncthreads();
    // The CTA that completed the entry merges its chunks: warp 0, lane l
    // taking chunks l and l + 32, then a fixed shuffle tree (the result does
    // not depend on which CTA finished last).
    if (s_last && warp == 0) {
      __threadfence();
      const volatile RefPart *vp = b->part + (size_t)e * nch;
      double fa[3] = {0.0, 0.0, 0.0}, fp = 0.0, fr2 = inf;
      int fs = -1;
      for (int cc = lane; cc < nch; cc += 32) {
        for (int k = 0; k < 3; k++) fa[k] += vp[cc].a[k];
        fp += vp[cc].p;
        const int sl = vp[cc].slot;
        const double r2 = vp[cc].r2;
        if (sl >= 0 && (r2 < fr2 || (r2 == fr2 && sl < fs))) {
          fr2 = r2;
          fs = sl;
        }
      }
#pragma unroll
      for (int off = 16; off > 0; off >>= 1) {
#pragma unroll
        for (int k = 0; k < 3; k++) fa[k] += __shfl_down_sync(0xffffffffu, fa[k], off);
        fp += __shfl_down_sync(0xffffffffu, fp, off);
        const double or2 = __shfl_down_sync(0xffffffffu, fr2, off);
        const int os = __shfl_down_sync(0xffffffffu, fs, off);
        if (os >= 0 && (or2 < fr2 || (or2 == fr2 && (fs < 0 || os < fs)))) {
          fr2 = or2;
          fs = os;
        }
      }
      if (lane == 0) {
        if (mode & (REF_ACC | REF_MT)) {
          for (int k = 0; k < 3; k++) kp.acc[3 * i + k] = fa[k];
          kp.pot[i] = -fp;
        }
        if ((mode & REF_NN) && fs >= 0) {
          if (kp.nn) kp.nn[i] = fs;
          if (kp.nn_r2) kp.nn_r2[i] = (float)fr2;
        }
        b->ticket[e] = 0u;
      }
    }
    __syncthreads();
  }
  __syncthreads();
  if (tid == 0) {
    __threadfence();
    const unsigned d = atomicAdd(&b->h.done, 1u);
    if (d == gridDim.x - 1) {
      b->h.last = cnt;
      b->h.last_acc = b->h.nacc;
      b->h.last_mt = b->h.nmt;
      b->h.count = 0u;
      b->h.nacc = 0u;
      b->h.nmt = 0u;
      b->h.done = 0u;
      __threadfence();
    }
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
  int ni, nj, prec, nn, fjl, fns;
  int jl, nsplit, jsplit;
};
ShapeKey g_shape_cache[256];

void choose_shape(int ni, int nj, int prec, int nn, int force_jl, int force_nsplit, int *jl_out,
                  int *nsplit_out, int *jsplit_out) {
  nn = nn ? 1 : 0;
  const unsigned h =
      ((unsigned)ni * 2654435761u ^ (unsigned)nj * 40503u ^ (unsigned)prec ^ (unsigned)nn * 97u) &
      255u;
  ShapeKey &c = g_shape_cache[h];
  if (c.ni == ni && c.nj == nj && c.prec == prec && c.nn == nn && c.fjl == force_jl &&
      c.fns == force_nsplit && c.jl > 0) {
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
      // Where the i-groups alone do not fill the GPU, CTAs are kept to at
      // most 128 tiles (256 with the nearest neighbour, whose CTAs each
      // re-scan a best tile at the end): many short CTAs balance over the
      // SMs as slots free up, better than a few long ones in one wave
      // (measured, 16384 i against 2^20 j: 0.674 of peak at 7 splits of 586
      // tiles, 0.700 at 38 or 57 splits; the wave count does not capture
      // it; with nn at 65536 i: 0.690 at 16 splits, 0.685 at 32).
      if (gx < slots && tp > (nn ? 256 : 128) && k + 1 < nc) continue;
      // j-lanes (JL > 1) cost a few per cent per pair in large blocks
      // (measured at 65536 i: JL = 2 ran 3 % slower than JL = 1 without the
      // nearest neighbour and 6 % slower with it), where JL = 1 fills the
      // GPU by splitting j alone
      const double jl_pen = (jl > 1 && ni >= 16384) ? 1.05 : 1.0;
      // each split adds per-CTA start-up, a partial record per i to write
      // and merge, and (nearest neighbour) a re-scan of its best tile: 0.2 %
      // per split against j sets of up to 2048 tiles (measured: 65536 i
      // against 2^18 j ran 2 % slower at 16 splits than at 7), proportionally
      // less against larger ones (2^20 j: 16 splits beat 7 by 1.5 %)
      const double split_pen = 0.002 * ns * (ntiles > 2048 ? 2048.0 / ntiles : 1.0);
      const double cost = (double)waves * (tp * (A + B * (double)(TJ / jl)) + F) *
                          (1.0 + split_pen) * jl_pen;
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
  c.nn = nn;
  c.fjl = force_jl;
  c.fns = force_nsplit;
  c.jl = *jl_out;
  c.nsplit = *nsplit_out;
  c.jsplit = *jsplit_out;
}

template <class P>
int launch(const KParams &kp, int jl, int gx, cudaStream_t st, cudaEvent_t ev_mid) {
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
  if (kp.nsplit > 1 && !kp.xtick) {
    if (kp.ni < 4096)
      launch_pdl(reduce_warp_kernel<P>, dim3((kp.ni + 3) / 4), dim3(128), 0, st, kp);
    else
      launch_pdl(reduce_kernel<P>, dim3((kp.ni + 127) / 128), dim3(128), 0, st, kp);
  }
  if (ev_mid) cudaEventRecord(ev_mid, st);
  // refine_kernel: units of (entry, j-chunk), at most RCHMAX chunks per
  // entry and ni entries, so small blocks get a small grid
  if (kp.refine) {
    const long long cap = (long long)kp.ni * RCHMAX;
    const int grid = cap < 2LL * sm_count() ? (int)cap : 2 * sm_count();
    launch_pdl(refine_kernel, dim3(grid), dim3(RNT), 0, st, kp);
  }
  return cudaGetLastError() == cudaSuccess ? 0 : -3;
}

}  // namespace

extern "C" int g6k_sm_count(void) { return sm_count(); }

extern "C" size_t g6k_refine_bytes(void) { return sizeof(RefBuf); }

extern "C" int g6k_refine_read(const void *refine, int out[4], cudaStream_t st) {
  RefHdr h;
  if (cudaMemcpyAsync(&h, refine, sizeof(h), cudaMemcpyDeviceToHost, st) != cudaSuccess ||
      cudaStreamSynchronize(st) != cudaSuccess)
    return -3;
  out[0] = (int)h.last;
  out[1] = (int)h.last_acc;
  out[2] = (int)h.overflow;
  out[3] = (int)h.last_mt;
  if (h.overflow) {
    const unsigned zero = 0;
    cudaMemcpyAsync(reinterpret_cast<char *>(const_cast<void *>(refine)) +
                        offsetof(RefHdr, overflow),
                    &zero, sizeof(zero), cudaMemcpyHostToDevice, st);
    cudaStreamSynchronize(st);
  }
  return 0;
}

extern "C" size_t g6k_scratch_bytes(int ni, int nj, int prec, int nn, int force_jl,
                                    int force_nsplit) {
  int jl, nsplit, jsplit;
  choose_shape(ni, nj, prec, nn, force_jl, force_nsplit, &jl, &nsplit, &jsplit);
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
  choose_shape(a->ni, a->nj, a->prec, a->want_nn, a->hjerk ? 1 : a->force_jl, a->force_nsplit,
               &jl, &nsplit, &jsplit);
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
  kp.js = *a->js;
  kp.ti = a->ti;
  // The refinement pass serves the split kernel's g6 results; the hermite
  // jerk form and callers passing kappa < 0 (the fixed-step path) keep plain
  // split arithmetic.
  kp.refine =
      (a->prec == G6_PREC_SPLIT && !a->hjerk && a->kappa >= 0.0) ? a->refine : nullptr;
  kp.kappa2 = a->kappa > 0.0 ? a->kappa * a->kappa : 0.0;
  kp.stall = a->stall_test;
  kp.wait_ns = a->stall_test ? STALL_TEST_NS : WAIT_NS;
  const size_t need =
      nsplit > 1 ? g6k_scratch_bytes(a->ni, a->nj, a->prec, a->want_nn, jl, nsplit) : 0;
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
  // The in-kernel split merge runs in the one CTA that completes an i-group,
  // a warp per i: it saves a launch where the group holds one or two i
  // (JL = 128), but with more i per group that CTA's warps merge them one
  // after another and the tail outlasts a second launch that gives every i
  // its own warp (measured, force with merge: 722 i at JL = 4, 136 us in the
  // kernel against 83 us with the second launch; 64 i at JL = 32, 44 us
  // against 32 us; 1 i at JL = 128, 21 us against 24 us).
  kp.xtick = (a->refine && nsplit > 1 && gx <= XTMAX && islots <= G6_XMERGE_MAX)
                 ? reinterpret_cast<RefBuf *>(a->refine)->xtick
                 : nullptr;
  if (a->prec == G6_PREC_FP64) {
    kp.jrec = a->js->jp_f64;
    return launch<F64P>(kp, jl, gx, st, a->ev_mid);
  }
  kp.jrec = a->js->jp_split;
  return launch<SplitP>(kp, jl, gx, st, a->ev_mid);
}

// ---------------------------------------------------------------------------
// Fixed scratch for callers that cannot allocate device memory.
//
// The split-j partial sums normally live in a buffer that the host library
// grows with cudaMalloc on demand.  g6k_force_static instead places them in
// this file-scope array, which every GPU that loads the library holds (16 MiB)
// until the process exits.  Host code cannot use the array's name as a device
// address: g6k_static_scratch_addr looks the address up (cudaGetSymbolAddress)
// with the caller's device current; the host library does that once in
// g6_open and keeps it in its context until g6_close (a device reset needs
// g6_close + g6_open).  The lookup also loads this module, so the array is
// taken at g6_open, not at the first call.  Every call shares the array:
// nothing in it has to start at zero (each partial record is written by
// exactly one CTA before it is read), and calls that overlap on the GPU
// (different streams, or host threads) race on it.
#define G6_STATIC_SCRATCH_BYTES (16u << 20)
static __device__ __align__(256) unsigned char g6_static_scratch[G6_STATIC_SCRATCH_BYTES];

extern "C" size_t g6k_static_scratch_capacity(void) { return G6_STATIC_SCRATCH_BYTES; }

// 0 and the array's device address on the current device, or -5.
extern "C" int g6k_static_scratch_addr(void **out) {
  void *p = nullptr;
  if (cudaGetSymbolAddress(&p, g6_static_scratch) != cudaSuccess || p == nullptr) return -5;
  *out = p;
  return 0;
}

// Returns 0, -1/-2/-3 as g6k_force, -4 when the launch shape needs more than
// G6_STATIC_SCRATCH_BYTES of scratch (*need_out tells how much), -5 without
// the array's address (static_addr from g6k_static_scratch_addr).
extern "C" int g6k_force_static(const g6_force_args *a, void *static_addr, g6_shape *shape,
                                cudaStream_t st, size_t *need_out) {
  if (!static_addr) return -5;
  const size_t need = g6k_scratch_bytes(a->ni, a->nj, a->prec, a->want_nn,
                                        a->hjerk ? 1 : a->force_jl,
                                        a->force_nsplit);
  if (need_out) *need_out = need;
  if (need > G6_STATIC_SCRATCH_BYTES) return -4;
  g6_force_args b = *a;
  b.scratch = static_addr;
  b.scratch_bytes = G6_STATIC_SCRATCH_BYTES;
  return g6k_force(&b, shape, st);
}
