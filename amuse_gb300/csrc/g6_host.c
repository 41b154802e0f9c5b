/*
 * g6_host.c -- host side of libsapporo.so (C11 + CUDA runtime C API).
 *
 * Implements the GRAPE-6 ABI of include/g6.h on one GPU.  Mirrors the
 * behaviour of the reference host library (lib/sapporo_light/sapporo.cpp,
 * send_fetch_data.cpp) with these differences by design:
 *   - the j-store grows on demand (no nj_max = 131072 cap, sapporo.cpp:30);
 *   - j updates are staged in pinned memory, deduplicated per slot with an
 *     O(1) slot index (the reference uses a std::map, sapporo.cpp:83-110) and
 *     applied with one copy + one scatter kernel per force call;
 *   - inputs and outputs move with one asynchronous copy each way;
 *   - errors return negative codes instead of exit(-1).
 * There is no CPU force path: every force is computed by the CUDA kernels.
 */
#define _POSIX_C_SOURCE 200112L /* clock_gettime */
#include <math.h>
#include <stdarg.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <time.h>

#include <cuda_runtime_api.h>

#include "g6.h"
#include "g6_dev.h"

int g6k_clamp_steps(const g6_jstate *js, int nj, double dtmax, cudaStream_t st);
int g6k_static_scratch_addr(void **out);
int g6k_neighbours(const g6_jstate *js, int nj, int ni, int prec, const double *ipos,
                   const double *h2, const int *iself, int *out, int maxn, cudaStream_t st);

#define G6_DEFAULT_CAP 131072
#define G6_DEFAULT_NPIPES 16384
/* Condition-number limit above which split acc/pot are redone in FP64
   (kern_force.cu: "condition-number refinement"). */
#define G6_DEFAULT_KAPPA 48.0

/* ------------------------------------------------------------ id map --- */
/* Open addressing id -> slot (ids are arbitrary ints). */
typedef struct {
  int *key, *val;
  int cap, n;
} idmap;

static unsigned hash_int(int k) {
  unsigned x = (unsigned)k;
  x ^= x >> 16;
  x *= 0x7feb352du;
  x ^= x >> 15;
  x *= 0x846ca68bu;
  x ^= x >> 16;
  return x;
}

static void idmap_free(idmap *m) {
  free(m->key);
  free(m->val);
  memset(m, 0, sizeof(*m));
}

static int idmap_put(idmap *m, int k, int v);

static int idmap_grow(idmap *m) {
  idmap n;
  n.cap = m->cap ? 2 * m->cap : 1024;
  n.n = 0;
  n.key = (int *)malloc(sizeof(int) * n.cap);
  n.val = (int *)malloc(sizeof(int) * n.cap);
  if (!n.key || !n.val) {
    free(n.key);
    free(n.val);
    return -1;
  }
  for (int i = 0; i < n.cap; i++) n.val[i] = -1;
  for (int i = 0; i < m->cap; i++)
    if (m->val[i] >= 0) idmap_put(&n, m->key[i], m->val[i]); /* drops erased entries */
  idmap_free(m);
  *m = n;
  return 0;
}

static int idmap_put(idmap *m, int k, int v) {
  if (2 * (m->n + 1) > m->cap && idmap_grow(m) != 0) return -1;
  unsigned h = hash_int(k) & (unsigned)(m->cap - 1);
  /* val == -1: empty; val < -1: erased entry (kept so probe chains hold). */
  while (m->val[h] != -1 && m->key[h] != k) h = (h + 1) & (unsigned)(m->cap - 1);
  if (m->val[h] == -1) m->n++;
  m->key[h] = k;
  m->val[h] = v;
  return 0;
}

static int idmap_get(const idmap *m, int k) {
  if (m->cap == 0) return -1;
  unsigned h = hash_int(k) & (unsigned)(m->cap - 1);
  while (m->val[h] != -1) {
    if (m->key[h] == k) return m->val[h] >= 0 ? m->val[h] : -1;
    h = (h + 1) & (unsigned)(m->cap - 1);
  }
  return -1;
}

/* ----------------------------------------------------------- context --- */
typedef struct {
  int is_open, device, npipes, prec;
  cudaStream_t st;
  cudaEvent_t ev_done, ev_upd, ev_t0, ev_t1, ev_t2, ev_tm;
  g6_jstate js;
  /* host mirrors (size cap) */
  int *slot_id, *stage_pos;
  idmap ids;
  /* staged j updates (pinned) */
  g6_jupd *h_upd, *d_upd;
  int n_upd, cap_upd, cap_dupd, upd_inflight;
  /* time / prediction state */
  double ti;
  int pred_valid, pred_nj, pred_prec;
  double pred_t;
  /* i / out buffers: pinned host block + device block, capacity cap_i */
  int cap_i;
  void *h_in, *d_in;   /* [ipos 3n][ivel 3n][h2 n] doubles, [iself n] ints */
  void *h_out, *d_out; /* [err 2 ints][acc 3n][jerk 3n][pot n] doubles, [nn n] ints, [nnr2 n] floats */
  int *d_err;
  void *d_scratch;
  size_t scratch_bytes;
  /* pending g6calc */
  int pending, pending_ni, pending_nj;
  int *pending_ids; /* copy of index[] for the neighbour-list API */
  int pending_cap;
  /* device run (extension API) */
  int run_n;
  double run_t, run_eps2, run_eta;
  int *d_ilist, *d_ni;
  double *d_tnext, *d_sched, *d_esum, *d_racc, *d_rjerk, *d_rpot;
  void *d_mail, *h_mail; /* 16 B {tnext, ni, stop}: device copy and pinned host copy */
  int *d_rnn;
  int run_cap;
  /* encounter check in g6x_run (idata::check_encounters) */
  int enc_mode;
  double enc_rmin;
  double *d_rad; /* particle radii by slot, rad_cap entries */
  int rad_cap;
  g6_enc *d_enc;
  double *d_encp_d;
  int *d_encp_i;
  unsigned *d_enc_ctr;
  int enc_cap; /* CTAs the partial buffers hold */
  /* k nearest neighbours (g6x_knn) */
  void *d_knn;
  size_t knn_bytes;
  /* split-precision refinement queue (nearest-neighbour proof, FP64 redo of
     ill-conditioned sums) and the force kernel's split-merge tickets: fixed
     size, allocated at open */
  void *d_refine;
  double kappa;
  /* device address of the no-allocation entry point's fixed scratch array,
     looked up at open with the library's device current */
  void *d_static;
  /* test hook: the next force call's first CTA waits on a barrier that
     nothing arrives on (g6x_test_wait_expiry) */
  int stall_next;
  /* statistics */
  int timing;
  double st_predict_ms, st_force_ms, st_pairs, st_pred_bytes, st_nj;
  double st_kernel_ms, st_refine_ms; /* force_ms split at the refinement pass */
  int shape_jl, shape_ns;            /* launch shape override (0: the cost model's) */
  g6_shape shape;
  int predicted_this_call;
  char err[256];
} g6ctx;

static g6ctx G;
static int ilist_identity_n; /* d_ilist holds 0..n-1 for this n (0: unknown) */

static void seterr(const char *fmt, ...) {
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(G.err, sizeof(G.err), fmt, ap);
  va_end(ap);
  fprintf(stderr, "libsapporo(gb300): %s\n", G.err);
}

#define CK(call)                                                   \
  do {                                                             \
    cudaError_t e_ = (call);                                       \
    if (e_ != cudaSuccess) {                                       \
      seterr("%s failed: %s", #call, cudaGetErrorString(e_));      \
      return G6_ERR_CUDA;                                          \
    }                                                              \
  } while (0)

static void *pin_alloc(size_t bytes) {
  void *p = NULL;
  if (cudaHostAlloc(&p, bytes ? bytes : 16, cudaHostAllocDefault) != cudaSuccess) return NULL;
  return p;
}

static void free_jstate(g6_jstate *js) {
  cudaFree(js->t); cudaFree(js->dt); cudaFree(js->m); cudaFree(js->pot);
  cudaFree(js->x); cudaFree(js->v); cudaFree(js->a); cudaFree(js->j);
  cudaFree(js->id); cudaFree(js->nn);
  cudaFree(js->jp_split); cudaFree(js->jp_f64);
  memset(js, 0, sizeof(*js));
}

/* Grow the j-store to hold at least `need` slots (contents preserved). */
static int grow_j(int need) {
  if (need <= G.js.cap) return 0;
  int cap = G.js.cap ? G.js.cap : G6_DEFAULT_CAP;
  while (cap < need) cap *= 2;
  cap = (cap + G6_TILE - 1) / G6_TILE * G6_TILE;
  g6_jstate n;
  memset(&n, 0, sizeof(n));
  n.cap = cap;
  size_t d = sizeof(double) * (size_t)cap;
  int ok = cudaMalloc((void **)&n.t, d) == cudaSuccess &&
           cudaMalloc((void **)&n.dt, d) == cudaSuccess &&
           cudaMalloc((void **)&n.m, d) == cudaSuccess &&
           cudaMalloc((void **)&n.pot, d) == cudaSuccess &&
           cudaMalloc((void **)&n.x, 3 * d) == cudaSuccess &&
           cudaMalloc((void **)&n.v, 3 * d) == cudaSuccess &&
           cudaMalloc((void **)&n.a, 3 * d) == cudaSuccess &&
           cudaMalloc((void **)&n.j, 3 * d) == cudaSuccess &&
           cudaMalloc((void **)&n.id, sizeof(int) * (size_t)cap) == cudaSuccess &&
           cudaMalloc((void **)&n.nn, sizeof(int) * (size_t)cap) == cudaSuccess &&
           cudaMalloc(&n.jp_split, 48 * (size_t)cap) == cudaSuccess &&
           cudaMalloc(&n.jp_f64, 64 * (size_t)cap) == cudaSuccess;
  if (!ok) {
    free_jstate(&n);
    seterr("cannot allocate j-store for %d slots", cap);
    return G6_ERR_NOMEM;
  }
  cudaMemsetAsync(n.t, 0, d, G.st);
  cudaMemsetAsync(n.dt, 0, d, G.st);
  cudaMemsetAsync(n.m, 0, d, G.st);
  cudaMemsetAsync(n.pot, 0, d, G.st);
  cudaMemsetAsync(n.x, 0, 3 * d, G.st);
  cudaMemsetAsync(n.v, 0, 3 * d, G.st);
  cudaMemsetAsync(n.a, 0, 3 * d, G.st);
  cudaMemsetAsync(n.j, 0, 3 * d, G.st);
  cudaMemsetAsync(n.id, 0xff, sizeof(int) * (size_t)cap, G.st);
  cudaMemsetAsync(n.nn, 0xff, sizeof(int) * (size_t)cap, G.st);
  if (G.js.cap) {
    size_t od = sizeof(double) * (size_t)G.js.cap;
    cudaMemcpyAsync(n.t, G.js.t, od, cudaMemcpyDeviceToDevice, G.st);
    cudaMemcpyAsync(n.dt, G.js.dt, od, cudaMemcpyDeviceToDevice, G.st);
    cudaMemcpyAsync(n.m, G.js.m, od, cudaMemcpyDeviceToDevice, G.st);
    cudaMemcpyAsync(n.pot, G.js.pot, od, cudaMemcpyDeviceToDevice, G.st);
    for (int k = 0; k < 3; k++) {
      cudaMemcpyAsync(n.x + (size_t)k * cap, G.js.x + (size_t)k * G.js.cap, od,
                      cudaMemcpyDeviceToDevice, G.st);
      cudaMemcpyAsync(n.v + (size_t)k * cap, G.js.v + (size_t)k * G.js.cap, od,
                      cudaMemcpyDeviceToDevice, G.st);
      cudaMemcpyAsync(n.a + (size_t)k * cap, G.js.a + (size_t)k * G.js.cap, od,
                      cudaMemcpyDeviceToDevice, G.st);
      cudaMemcpyAsync(n.j + (size_t)k * cap, G.js.j + (size_t)k * G.js.cap, od,
                      cudaMemcpyDeviceToDevice, G.st);
    }
    cudaMemcpyAsync(n.id, G.js.id, sizeof(int) * (size_t)G.js.cap, cudaMemcpyDeviceToDevice, G.st);
    cudaMemcpyAsync(n.nn, G.js.nn, sizeof(int) * (size_t)G.js.cap, cudaMemcpyDeviceToDevice, G.st);
  }
  CK(cudaStreamSynchronize(G.st));
  int *sid = (int *)realloc(G.slot_id, sizeof(int) * (size_t)cap);
  int *spos = (int *)realloc(G.stage_pos, sizeof(int) * (size_t)cap);
  if (!sid || !spos) {
    if (sid) G.slot_id = sid;
    if (spos) G.stage_pos = spos;
    free_jstate(&n);
    seterr("host allocation failed");
    return G6_ERR_NOMEM;
  }
  for (int s = G.js.cap; s < cap; s++) {
    sid[s] = -1;
    spos[s] = -1;
  }
  G.slot_id = sid;
  G.stage_pos = spos;
  free_jstate(&G.js);
  G.js = n;
  G.pred_valid = 0;
  return 0;
}

static int ensure_io(int ni) {
  if (ni <= G.cap_i) return 0;
  int cap = G.cap_i ? G.cap_i : 1024;
  while (cap < ni) cap *= 2;
  size_t in_b = (size_t)cap * (7 * sizeof(double) + sizeof(int));
  size_t out_b = 16 + (size_t)cap * (7 * sizeof(double) + sizeof(int) + sizeof(float));
  if (G.h_in) cudaFreeHost(G.h_in);
  if (G.h_out) cudaFreeHost(G.h_out);
  cudaFree(G.d_in);
  cudaFree(G.d_out);
  G.h_in = G.h_out = G.d_in = G.d_out = NULL;
  G.cap_i = 0;
  G.h_in = pin_alloc(in_b);
  G.h_out = pin_alloc(out_b);
  if (!G.h_in || !G.h_out || cudaMalloc(&G.d_in, in_b) != cudaSuccess ||
      cudaMalloc(&G.d_out, out_b) != cudaSuccess) {
    seterr("cannot allocate i/o buffers for %d i-particles", cap);
    return G6_ERR_NOMEM;
  }
  CK(cudaMemsetAsync(G.d_out, 0, out_b, G.st));
  G.d_err = (int *)G.d_out;
  G.cap_i = cap;
  int *pid = (int *)realloc(G.pending_ids, sizeof(int) * (size_t)cap);
  if (!pid) return G6_ERR_NOMEM;
  G.pending_ids = pid;
  G.pending_cap = cap;
  return 0;
}

/* Views into the i/o blocks for capacity cap_i. */
#define IN_POS(b) ((double *)(b))
#define IN_VEL(b) ((double *)(b) + 3 * (size_t)G.cap_i)
#define IN_H2(b) ((double *)(b) + 6 * (size_t)G.cap_i)
#define IN_SELF(b) ((int *)((double *)(b) + 7 * (size_t)G.cap_i))
#define OUT_ERR(b) ((int *)(b))
#define OUT_ACC(b) ((double *)((char *)(b) + 16))
#define OUT_JERK(b) (OUT_ACC(b) + 3 * (size_t)G.cap_i)
#define OUT_POT(b) (OUT_ACC(b) + 6 * (size_t)G.cap_i)
#define OUT_NN(b) ((int *)(OUT_ACC(b) + 7 * (size_t)G.cap_i))
#define OUT_NNR2(b) ((float *)(OUT_NN(b) + (size_t)G.cap_i))

static int ensure_scratch(size_t bytes) {
  if (bytes <= G.scratch_bytes) return 0;
  cudaFree(G.d_scratch);
  G.d_scratch = NULL;
  G.scratch_bytes = 0;
  size_t b = bytes + bytes / 4;
  if (cudaMalloc(&G.d_scratch, b) != cudaSuccess) {
    seterr("cannot allocate %zu B of split-j scratch", b);
    return G6_ERR_NOMEM;
  }
  G.scratch_bytes = b;
  return 0;
}

static int check_open(void) {
  if (!G.is_open) {
    seterr("library not opened (g6_open)");
    return G6_ERR_NOT_OPEN;
  }
  return 0;
}

/* Apply staged j updates: one H2D copy + one scatter kernel. */
static int flush_updates(void) {
  if (G.n_upd == 0) return 0;
  if (G.n_upd > G.cap_dupd) {
    cudaFree(G.d_upd);
    G.d_upd = NULL;
    G.cap_dupd = 0;
    int c = G.cap_upd;
    if (cudaMalloc((void **)&G.d_upd, sizeof(g6_jupd) * (size_t)c) != cudaSuccess) {
      seterr("cannot allocate update buffer");
      return G6_ERR_NOMEM;
    }
    G.cap_dupd = c;
  }
  CK(cudaMemcpyAsync(G.d_upd, G.h_upd, sizeof(g6_jupd) * (size_t)G.n_upd,
                     cudaMemcpyHostToDevice, G.st));
  CK(cudaEventRecord(G.ev_upd, G.st));
  G.upd_inflight = 1;
  int rc = g6k_scatter(&G.js, G.d_upd, G.n_upd, G.st);
  if (rc) {
    seterr("scatter launch failed");
    return G6_ERR_CUDA;
  }
  for (int u = 0; u < G.n_upd; u++) G.stage_pos[G.h_upd[u].addr] = -1;
  G.n_upd = 0;
  G.pred_valid = 0;
  return 0;
}

static int predict_if_needed(int nj) {
  G.predicted_this_call = 0;
  if (G.pred_valid && G.pred_t == G.ti && G.pred_nj == nj && G.pred_prec == G.prec) return 0;
  int need = (nj + G6_TILE - 1) / G6_TILE * G6_TILE;
  int rc = grow_j(need);
  if (rc) return rc;
  if (G.timing) cudaEventRecord(G.ev_t0, G.st);
  if (g6k_predict(&G.js, nj, G.ti, G.prec, G.st)) {
    seterr("predictor launch failed");
    return G6_ERR_CUDA;
  }
  if (G.timing) cudaEventRecord(G.ev_t1, G.st);
  G.predicted_this_call = 1;
  G.pred_valid = 1;
  G.pred_t = G.ti;
  G.pred_nj = nj;
  G.pred_prec = G.prec;
  return 0;
}

/* The refinement pass of split-precision g6 forces (the fixed-step path
   passes kappa < 0 and keeps plain split arithmetic).  The buffer is passed
   in every case: the force kernel also keeps its split-merge tickets there. */
static void refine_args(g6_force_args *a) {
  a->refine = G.d_refine;
  if (a->kappa >= 0.0) a->kappa = G.kappa;
}

/* Run one force evaluation whose inputs are already on the device. */
static int run_force(g6_force_args *a) {
  if (!a->force_jl && !a->hjerk) a->force_jl = G.shape_jl;
  if (!a->force_nsplit) a->force_nsplit = G.shape_ns;
  size_t need = g6k_scratch_bytes(a->ni, a->nj, a->prec, a->want_nn, a->hjerk ? 1 : a->force_jl,
                                  a->force_nsplit);
  int rc = ensure_scratch(need);
  if (rc) return rc;
  refine_args(a);
  a->stall_test = G.stall_next;
  G.stall_next = 0;
  a->scratch = G.d_scratch;
  a->scratch_bytes = G.scratch_bytes;
  a->js = &G.js;
  a->err = G.d_err;
  if (G.timing) {
    if (!G.predicted_this_call) cudaEventRecord(G.ev_t1, G.st);
  }
  a->ev_mid = G.timing ? G.ev_tm : NULL;
  rc = g6k_force(a, &G.shape, G.st);
  if (rc) {
    seterr("force launch failed (%d)", rc);
    return G6_ERR_CUDA;
  }
  if (G.timing) cudaEventRecord(G.ev_t2, G.st);
  G.st_pairs = (double)a->ni * (double)(a->nj > 0 ? a->nj - 1 : 0);
  G.st_nj = a->nj;
  G.st_pred_bytes = G.predicted_this_call
                        ? (double)a->nj * (15.0 * 8.0 + (G.prec == G6_PREC_FP64 ? 64.0 : 48.0))
                        : 0.0;
  return 0;
}

static void collect_timing(void) {
  if (!G.timing) return;
  float ms = 0;
  G.st_predict_ms = 0;
  if (G.predicted_this_call && cudaEventElapsedTime(&ms, G.ev_t0, G.ev_t1) == cudaSuccess)
    G.st_predict_ms = ms;
  if (cudaEventElapsedTime(&ms, G.ev_t1, G.ev_t2) == cudaSuccess) G.st_force_ms = ms;
  G.st_kernel_ms = G.st_force_ms;
  G.st_refine_ms = 0;
  if (cudaEventElapsedTime(&ms, G.ev_t1, G.ev_tm) == cudaSuccess) {
    G.st_kernel_ms = ms;
    G.st_refine_ms = G.st_force_ms - ms;
  }
}

/* ===================================================== Part 1: g6 ABI === */

int g6_open_(int *id) {
  int dev = id ? *id : 0;
  if (G.is_open) return 0;
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev <= 0) {
    seterr("no CUDA device found");
    return G6_ERR_DEVICE;
  }
  if (dev < 0 || dev >= ndev) {
    seterr("cluster id %d: no such CUDA device (have %d)", dev, ndev);
    return G6_ERR_DEVICE;
  }
  memset(&G, 0, sizeof(G));
  G.device = dev;
  CK(cudaSetDevice(dev));
  CK(cudaStreamCreateWithFlags(&G.st, cudaStreamNonBlocking));
  CK(cudaEventCreateWithFlags(&G.ev_done, cudaEventDisableTiming));
  CK(cudaEventCreateWithFlags(&G.ev_upd, cudaEventDisableTiming));
  CK(cudaEventCreate(&G.ev_t0));
  CK(cudaEventCreate(&G.ev_t1));
  CK(cudaEventCreate(&G.ev_t2));
  CK(cudaEventCreate(&G.ev_tm));
  G.npipes = G6_DEFAULT_NPIPES;
  const char *e = getenv("G6_NPIPES");
  if (e && atoi(e) > 0 && atoi(e) <= (1 << 20)) G.npipes = atoi(e);
  G.prec = G6_PREC_SPLIT;
  e = getenv("G6_PRECISION");
  if (e && (!strcmp(e, "fp64") || !strcmp(e, "FP64"))) G.prec = G6_PREC_FP64;
  G.kappa = G6_DEFAULT_KAPPA;
  e = getenv("G6_KAPPA");
  if (e && atof(e) >= 0.0) G.kappa = atof(e);
  G.is_open = 1;
  int rc = grow_j(G6_DEFAULT_CAP);
  if (rc == 0) rc = ensure_io(G.npipes < 4096 ? G.npipes : 4096);
  if (rc == 0) {
    if (cudaMalloc(&G.d_refine, g6k_refine_bytes()) != cudaSuccess ||
        cudaMemset(G.d_refine, 0, g6k_refine_bytes()) != cudaSuccess) {
      seterr("cannot allocate the refinement buffer");
      rc = G6_ERR_NOMEM;
    }
  }
  /* Loads the force module, so its fixed 16 MiB array is taken here. */
  if (rc == 0 && g6k_static_scratch_addr(&G.d_static) != 0) {
    seterr("cannot obtain the device address of the fixed scratch array");
    rc = G6_ERR_CUDA;
  }
  if (rc) {
    g6_close_(id);
    return rc;
  }
  return 0;
}

static void ngb_free(void);
static void batch_free(void);
static void fixed_free(void);

int g6_close_(int *id) {
  (void)id;
  if (!G.is_open) return 0;
  cudaStreamSynchronize(G.st);
  ngb_free();
  batch_free();
  fixed_free();
  free_jstate(&G.js);
  if (G.h_upd) cudaFreeHost(G.h_upd);
  if (G.h_in) cudaFreeHost(G.h_in);
  if (G.h_out) cudaFreeHost(G.h_out);
  cudaFree(G.d_upd); cudaFree(G.d_in); cudaFree(G.d_out); cudaFree(G.d_scratch);
  cudaFree(G.d_ilist); cudaFree(G.d_mail); cudaFree(G.d_sched);
  if (G.h_mail) cudaFreeHost(G.h_mail);
  cudaFree(G.d_esum); cudaFree(G.d_racc); cudaFree(G.d_rjerk); cudaFree(G.d_rpot);
  cudaFree(G.d_rnn);
  cudaFree(G.d_rad); cudaFree(G.d_enc); cudaFree(G.d_encp_d); cudaFree(G.d_encp_i);
  cudaFree(G.d_enc_ctr);
  cudaFree(G.d_knn);
  cudaFree(G.d_refine);
  cudaEventDestroy(G.ev_done); cudaEventDestroy(G.ev_upd);
  cudaEventDestroy(G.ev_t0); cudaEventDestroy(G.ev_t1); cudaEventDestroy(G.ev_t2);
  cudaEventDestroy(G.ev_tm);
  cudaStreamDestroy(G.st);
  free(G.slot_id);
  free(G.stage_pos);
  free(G.pending_ids);
  idmap_free(&G.ids);
  memset(&G, 0, sizeof(G));
  ilist_identity_n = 0;
  return 0;
}

int g6_npipes_(void) { return G.is_open ? G.npipes : G6_DEFAULT_NPIPES; }
int g6_set_tunit_(double *t) { (void)t; return 0; }
int g6_set_xunit_(double *x) { (void)x; return 0; }

int g6_set_ti_(int *id, double *ti) {
  (void)id;
  int rc = check_open();
  if (rc) return rc;
  G.ti = *ti;
  return 0;
}

int g6_set_j_particle_(int *cluster_id, int *address, int *index, double *tj, double *dtj,
                       double *mass, double k18[3], double j6[3], double a2[3], double v[3],
                       double x[3]) {
  (void)cluster_id;
  (void)k18;
  int rc = check_open();
  if (rc) return rc;
  const int addr = *address;
  if (addr < 0) {
    seterr("g6_set_j_particle: negative address %d", addr);
    return G6_ERR_ARG;
  }
  if (addr >= G.js.cap) {
    rc = grow_j(addr + 1);
    if (rc) return rc;
  }
  if (G.upd_inflight) {
    /* The previous staging buffer may still be in flight. */
    cudaEventSynchronize(G.ev_upd);
    G.upd_inflight = 0;
  }
  int pos = G.stage_pos[addr];
  if (pos < 0) {
    if (G.n_upd == G.cap_upd) {
      int c = G.cap_upd ? 2 * G.cap_upd : 4096;
      g6_jupd *nb = (g6_jupd *)pin_alloc(sizeof(g6_jupd) * (size_t)c);
      if (!nb) {
        seterr("cannot allocate pinned staging (%d records)", c);
        return G6_ERR_NOMEM;
      }
      if (G.h_upd) {
        memcpy(nb, G.h_upd, sizeof(g6_jupd) * (size_t)G.n_upd);
        cudaFreeHost(G.h_upd);
      }
      G.h_upd = nb;
      G.cap_upd = c;
    }
    pos = G.n_upd++;
    G.stage_pos[addr] = pos;
  }
  g6_jupd *r = &G.h_upd[pos];
  r->addr = addr;
  r->id = *index;
  r->t = *tj;
  r->dt = *dtj;
  r->m = *mass;
  for (int k = 0; k < 3; k++) {
    r->x[k] = x[k];
    r->v[k] = v[k];
    r->a[k] = a2[k] * 2.0;
    r->j[k] = j6[k] * 6.0;
  }
  if (G.slot_id[addr] != *index) {
    if (G.slot_id[addr] >= 0 && idmap_get(&G.ids, G.slot_id[addr]) == addr)
      idmap_put(&G.ids, G.slot_id[addr], -2 - addr); /* tombstone: not found */
    G.slot_id[addr] = *index;
    if (idmap_put(&G.ids, *index, addr)) {
      seterr("id map allocation failed");
      return G6_ERR_NOMEM;
    }
  }
  return 0;
}

/* The explicit-i force call with host arrays runs in two phases, so that
 * the kernel knows whether the caller wants nearest neighbours:
 *   stage_force_host  (g6calc_firsthalf): apply staged j updates, predict
 *                      the j-system, copy the i-particles to the device;
 *   launch_force_host (g6calc_lasthalf / lasthalf2): launch the force kernel
 *                      with or without the nearest-neighbour search, then
 *                      copy the results back.
 * Both AMUSE callers issue lasthalf right after firsthalf (ph4 gpu.cc:394-407,
 * phiGRAPE gravity.F:104-111), so nothing overlaps in between either way. */
static int staged, staged_ni, staged_nj;
static double staged_eps2;

static int stage_force_host(int nj, int ni, const int *index, const double *xi,
                            const double *vi, const int *self_slot, double eps2,
                            const double *h2) {
  int rc = check_open();
  if (rc) return rc;
  if (G.pending) {
    cudaEventSynchronize(G.ev_done);
    G.pending = 0;
  }
  staged = 0;
  if (nj < 0 || ni < 0) {
    seterr("negative nj/ni");
    return G6_ERR_ARG;
  }
  if (ni > 0 && nj == 0) {
    seterr("nj = 0");
    return G6_ERR_ARG;
  }
  if (ni > 0) {
    rc = ensure_io(ni);
    if (rc) return rc;
    rc = flush_updates();
    if (rc) return rc;
    rc = predict_if_needed(nj);
    if (rc) return rc;
    memcpy(IN_POS(G.h_in), xi, sizeof(double) * 3 * (size_t)ni);
    memcpy(IN_VEL(G.h_in), vi, sizeof(double) * 3 * (size_t)ni);
    if (h2)
      memcpy(IN_H2(G.h_in), h2, sizeof(double) * (size_t)ni);
    else
      for (int i = 0; i < ni; i++) IN_H2(G.h_in)[i] = 0.0;
    int *hs = IN_SELF(G.h_in);
    if (self_slot) {
      memcpy(hs, self_slot, sizeof(int) * (size_t)ni);
    } else {
      for (int i = 0; i < ni; i++) {
        int s = idmap_get(&G.ids, index[i]);
        hs[i] = (s >= 0 && s < nj) ? s : -1;
      }
    }
    /* One copy of the live prefix of each input section. */
    CK(cudaMemcpyAsync(IN_POS(G.d_in), IN_POS(G.h_in), sizeof(double) * 3 * (size_t)ni,
                       cudaMemcpyHostToDevice, G.st));
    CK(cudaMemcpyAsync(IN_VEL(G.d_in), IN_VEL(G.h_in), sizeof(double) * 3 * (size_t)ni,
                       cudaMemcpyHostToDevice, G.st));
    CK(cudaMemcpyAsync(IN_SELF(G.d_in), hs, sizeof(int) * (size_t)ni, cudaMemcpyHostToDevice,
                       G.st));
    if (index && ni <= G.pending_cap) memcpy(G.pending_ids, index, sizeof(int) * (size_t)ni);
  }
  G.pending_nj = nj;
  staged = 1;
  staged_ni = ni;
  staged_nj = nj;
  staged_eps2 = eps2;
  return 0;
}

static int launch_force_host(int want_nn) {
  if (!staged) {
    seterr("lasthalf without firsthalf");
    return G6_ERR_STATE;
  }
  staged = 0;
  const int ni = staged_ni;
  G.pending = 1;
  G.pending_ni = ni;
  if (ni == 0) return 0;
  g6_force_args a;
  memset(&a, 0, sizeof(a));
  a.ni = ni;
  a.nj = staged_nj;
  a.prec = G.prec;
  a.eps2 = staged_eps2;
  a.ipos = IN_POS(G.d_in);
  a.ivel = IN_VEL(G.d_in);
  a.iself = IN_SELF(G.d_in);
  a.ti = G.ti;
  a.acc = OUT_ACC(G.d_out);
  a.jerk = OUT_JERK(G.d_out);
  a.pot = OUT_POT(G.d_out);
  a.nn = OUT_NN(G.d_out);
  a.nn_r2 = OUT_NNR2(G.d_out);
  a.want_nn = want_nn;
  int rc = run_force(&a);
  if (rc) {
    G.pending = 0;
    return rc;
  }
  /* Error word + live prefix of each output section. */
  CK(cudaMemcpyAsync(G.h_out, G.d_out, 16, cudaMemcpyDeviceToHost, G.st));
  CK(cudaMemcpyAsync(OUT_ACC(G.h_out), OUT_ACC(G.d_out), sizeof(double) * 3 * (size_t)ni,
                     cudaMemcpyDeviceToHost, G.st));
  CK(cudaMemcpyAsync(OUT_JERK(G.h_out), OUT_JERK(G.d_out), sizeof(double) * 3 * (size_t)ni,
                     cudaMemcpyDeviceToHost, G.st));
  CK(cudaMemcpyAsync(OUT_POT(G.h_out), OUT_POT(G.d_out), sizeof(double) * (size_t)ni,
                     cudaMemcpyDeviceToHost, G.st));
  if (want_nn) {
    CK(cudaMemcpyAsync(OUT_NN(G.h_out), OUT_NN(G.d_out), sizeof(int) * (size_t)ni,
                       cudaMemcpyDeviceToHost, G.st));
    CK(cudaMemcpyAsync(OUT_NNR2(G.h_out), OUT_NNR2(G.d_out), sizeof(float) * (size_t)ni,
                       cudaMemcpyDeviceToHost, G.st));
  }
  CK(cudaEventRecord(G.ev_done, G.st));
  return 0;
}

static int finish_force(int ni) {
  if (!G.pending) {
    seterr("lasthalf without firsthalf");
    return G6_ERR_STATE;
  }
  if (ni != G.pending_ni) {
    cudaEventSynchronize(G.ev_done);
    G.pending = 0;
    seterr("lasthalf ni=%d differs from firsthalf ni=%d", ni, G.pending_ni);
    return G6_ERR_ARG;
  }
  cudaError_t e = ni > 0 ? cudaEventSynchronize(G.ev_done) : cudaSuccess;
  G.pending = 0;
  if (e != cudaSuccess) {
    seterr("force call failed: %s", cudaGetErrorString(e));
    return G6_ERR_CUDA;
  }
  collect_timing();
  if (ni > 0 && OUT_ERR(G.h_out)[0] != 0) {
    seterr("force kernel reported error word 0x%x", OUT_ERR(G.h_out)[0]);
    cudaMemsetAsync(G.d_err, 0, sizeof(int), G.st);
    return G6_ERR_KERNEL;
  }
  return 0;
}

static int firsthalf_rc;

void g6calc_firsthalf_(int *cluster_id, int *nj, int *ni, int index[], double xi[][3],
                       double vi[][3], double aold[][3], double j6old[][3], double phiold[],
                       double *eps2, double h2[]) {
  (void)cluster_id;
  (void)aold;
  (void)j6old;
  (void)phiold;
  if (G.is_open && *ni > G.npipes) {
    seterr("g6calc_firsthalf: ni=%d > npipes=%d", *ni, G.npipes);
    staged = 0;
    firsthalf_rc = G6_ERR_ARG;
    return;
  }
  firsthalf_rc = stage_force_host(*nj, *ni, index, &xi[0][0], &vi[0][0], NULL, *eps2, h2);
}

static int lasthalf_common(int ni, int want_nn, double acc[][3], double jerk[][3],
                           double pot[]) {
  if (firsthalf_rc) {
    int rc = firsthalf_rc;
    firsthalf_rc = 0;
    return rc;
  }
  int rc = launch_force_host(want_nn);
  if (rc) return rc;
  rc = finish_force(ni);
  if (rc) return rc;
  memcpy(&acc[0][0], OUT_ACC(G.h_out), sizeof(double) * 3 * (size_t)ni);
  memcpy(&jerk[0][0], OUT_JERK(G.h_out), sizeof(double) * 3 * (size_t)ni);
  memcpy(pot, OUT_POT(G.h_out), sizeof(double) * (size_t)ni);
  return 0;
}

int g6calc_lasthalf_(int *cluster_id, int *nj, int *ni, int index[], double xi[][3],
                     double vi[][3], double *eps2, double h2[], double acc[][3],
                     double jerk[][3], double pot[]) {
  (void)cluster_id; (void)nj; (void)index; (void)xi; (void)vi; (void)eps2; (void)h2;
  return lasthalf_common(*ni, 0, acc, jerk, pot);
}

int g6calc_lasthalf2_(int *cluster_id, int *nj, int *ni, int index[], double xi[][3],
                      double vi[][3], double *eps2, double h2[], double acc[][3],
                      double jerk[][3], double pot[], int *inn) {
  (void)cluster_id; (void)nj; (void)index; (void)xi; (void)vi; (void)eps2; (void)h2;
  int rc = lasthalf_common(*ni, 1, acc, jerk, pot);
  if (rc) return rc;
  const int *nn = OUT_NN(G.h_out);
  for (int i = 0; i < *ni; i++) inn[i] = nn[i] >= 0 ? G.slot_id[nn[i]] : -1;
  return 0;
}

int g6_initialize_jp_buffer_(int *cluster_id, int *buf_size) {
  (void)cluster_id;
  (void)buf_size;
  return 0;
}
int g6_flush_jp_buffer_(int *cluster_id) { (void)cluster_id; return 0; }
int g6_reset_(int *cluster_id) { (void)cluster_id; return 0; }
int g6_reset_fofpga_(int *cluster_id) { (void)cluster_id; return 0; }

/* ---- neighbour lists (sapporo.cpp:234-272) ---- */
/* Computed on demand from the i-particles of the last g6calc call: a
   separate pass over the predicted j records (r^2 <= h2[i], self
   excluded), so the force kernel carries no list logic. */
static int *h_ngb, *d_ngb;
static int ngb_cap, ngb_ni, ngb_valid;

static void ngb_free(void) {
  if (h_ngb) cudaFreeHost(h_ngb);
  cudaFree(d_ngb);
  h_ngb = NULL;
  d_ngb = NULL;
  ngb_cap = ngb_ni = ngb_valid = 0;
}

int g6_read_neighbour_list_(int *cluster_id) {
  (void)cluster_id;
  int rc = check_open();
  if (rc) return rc;
  if (G.pending) {
    seterr("g6_read_neighbour_list before g6calc_lasthalf");
    return G6_ERR_STATE;
  }
  const int ni = G.pending_ni;
  if (ni <= 0) return 0;
  const size_t per = (size_t)(G6_NGB_MAX + 1);
  if (ni > ngb_cap) {
    if (h_ngb) cudaFreeHost(h_ngb);
    cudaFree(d_ngb);
    h_ngb = (int *)pin_alloc(sizeof(int) * per * (size_t)ni);
    if (!h_ngb || cudaMalloc((void **)&d_ngb, sizeof(int) * per * (size_t)ni) != cudaSuccess) {
      ngb_cap = 0;
      seterr("cannot allocate neighbour lists");
      return G6_ERR_NOMEM;
    }
    ngb_cap = ni;
  }
  CK(cudaMemcpyAsync(IN_H2(G.d_in), IN_H2(G.h_in), sizeof(double) * (size_t)ni,
                     cudaMemcpyHostToDevice, G.st));
  if (g6k_neighbours(&G.js, G.pending_nj, ni, G.prec, IN_POS(G.d_in), IN_H2(G.d_in),
                     IN_SELF(G.d_in), d_ngb, G6_NGB_MAX, G.st)) {
    seterr("neighbour kernel launch failed");
    return G6_ERR_CUDA;
  }
  CK(cudaMemcpyAsync(h_ngb, d_ngb, sizeof(int) * per * (size_t)ni, cudaMemcpyDeviceToHost, G.st));
  CK(cudaStreamSynchronize(G.st));
  ngb_ni = ni;
  ngb_valid = 1;
  int overflow = 0;
  for (int i = 0; i < ni; i++)
    if (h_ngb[per * i] > G6_NGB_MAX) overflow = 1;
  return overflow;
}

static int cmp_int(const void *a, const void *b) {
  int x = *(const int *)a, y = *(const int *)b;
  return (x > y) - (x < y);
}

int g6_get_neighbour_list_(int *cluster_id, int *ipipe, int *maxlength, int *n_neighbours,
                           int neighbour_list[]) {
  (void)cluster_id;
  if (!ngb_valid) {
    seterr("g6_get_neighbour_list before g6_read_neighbour_list");
    return G6_ERR_STATE;
  }
  if (*ipipe < 0 || *ipipe >= ngb_ni) {
    seterr("g6_get_neighbour_list: ipipe=%d out of range [0,%d)", *ipipe, ngb_ni);
    return G6_ERR_ARG;
  }
  const int *row = h_ngb + (size_t)(G6_NGB_MAX + 1) * (size_t)(*ipipe);
  int len = row[0];
  int overflow = len > G6_NGB_MAX;
  if (len > G6_NGB_MAX) len = G6_NGB_MAX;
  int n = len < *maxlength ? len : *maxlength;
  if (len > *maxlength) overflow = 1;
  memcpy(neighbour_list, row + 1, sizeof(int) * (size_t)(n > 0 ? n : 0));
  qsort(neighbour_list, (size_t)(n > 0 ? n : 0), sizeof(int), cmp_int);
  *n_neighbours = n;
  return overflow;
}

/* ================================================ Part 2: by-value ===== */
#define WEAK __attribute__((weak))
WEAK int g6_open(int id) { return g6_open_(&id); }
WEAK int g6_close(int id) { return g6_close_(&id); }
WEAK int g6_npipes(void) { return g6_npipes_(); }
WEAK int g6_set_tunit(double t) { return g6_set_tunit_(&t); }
WEAK int g6_set_xunit(double x) { return g6_set_xunit_(&x); }
WEAK int g6_set_ti(int id, double ti) { return g6_set_ti_(&id, &ti); }
WEAK int g6_set_j_particle(int cluster_id, int address, int index, double tj, double dtj,
                           double mass, double k18[3], double j6[3], double a2[3], double v[3],
                           double x[3]) {
  return g6_set_j_particle_(&cluster_id, &address, &index, &tj, &dtj, &mass, k18, j6, a2, v, x);
}
WEAK void g6calc_firsthalf(int cluster_id, int nj, int ni, int index[], double xi[][3],
                           double vi[][3], double aold[][3], double j6old[][3], double phiold[],
                           double eps2, double h2[]) {
  g6calc_firsthalf_(&cluster_id, &nj, &ni, index, xi, vi, aold, j6old, phiold, &eps2, h2);
}
WEAK int g6calc_lasthalf(int cluster_id, int nj, int ni, int index[], double xi[][3],
                         double vi[][3], double eps2, double h2[], double acc[][3],
                         double jerk[][3], double pot[]) {
  return g6calc_lasthalf_(&cluster_id, &nj, &ni, index, xi, vi, &eps2, h2, acc, jerk, pot);
}
WEAK int g6calc_lasthalf2(int cluster_id, int nj, int ni, int index[], double xi[][3],
                          double vi[][3], double eps2, double h2[], double acc[][3],
                          double jerk[][3], double pot[], int inn[]) {
  return g6calc_lasthalf2_(&cluster_id, &nj, &ni, index, xi, vi, &eps2, h2, acc, jerk, pot, inn);
}
WEAK int g6_initialize_jp_buffer(int cluster_id, int buf_size) {
  return g6_initialize_jp_buffer_(&cluster_id, &buf_size);
}
WEAK int g6_flush_jp_buffer(int cluster_id) { return g6_flush_jp_buffer_(&cluster_id); }
WEAK int g6_reset(int cluster_id) { return g6_reset_(&cluster_id); }
WEAK int g6_reset_fofpga(int cluster_id) { return g6_reset_fofpga_(&cluster_id); }
WEAK int g6_read_neighbour_list(int cluster_id) { return g6_read_neighbour_list_(&cluster_id); }
WEAK int g6_get_neighbour_list(int cluster_id, int ipipe, int maxlength, int *n_neighbours,
                               int neighbour_list[]) {
  return g6_get_neighbour_list_(&cluster_id, &ipipe, &maxlength, n_neighbours, neighbour_list);
}

/* ============================================== Part 3: extension ====== */

int g6x_set_precision(int prec) {
  if (prec != G6X_SPLIT && prec != G6X_FP64) return G6_ERR_ARG;
  G.prec = prec;
  return 0;
}
int g6x_get_precision(void) { return G.prec; }
int g6x_set_shape(int jl, int nsplit) {
  if (jl < 0 || jl > 256 || (jl & (jl - 1)) || nsplit < 0) return G6_ERR_ARG;
  G.shape_jl = jl;
  G.shape_ns = nsplit;
  return 0;
}
int g6x_set_refine(double kappa) {
  if (!(kappa >= 0.0)) return G6_ERR_ARG;
  G.kappa = kappa;
  return 0;
}
int g6x_test_wait_expiry(int on) {
  int rc = check_open();
  if (rc) return rc;
  G.stall_next = on ? 1 : 0;
  return 0;
}
int g6x_refine_stats(int out[4]) {
  int rc = check_open();
  if (rc) return rc;
  if (g6k_refine_read(G.d_refine, out, G.st)) {
    seterr("cannot read the refinement queue");
    return G6_ERR_CUDA;
  }
  return 0;
}
int g6x_set_npipes(int npipes) {
  if (npipes < 1 || npipes > (1 << 20)) return G6_ERR_ARG;
  G.npipes = npipes;
  return 0;
}
const char *g6x_last_error(void) { return G.err; }
void *g6x_stream(void) { return (void *)G.st; }
int g6x_timing(int on) {
  G.timing = on ? 1 : 0;
  return 0;
}
int g6x_stats_n(double *out, int n) {
  if (!out || n < 0) return G6_ERR_ARG;
  if (G.timing && G.is_open) {
    cudaEventSynchronize(G.ev_t2);
    collect_timing();
  }
  const double v[10] = {G.st_predict_ms, G.st_force_ms, G.st_pairs, G.shape.jl,
                        G.shape.nsplit,  G.shape.grid_x, G.st_pred_bytes, G.st_nj,
                        G.st_kernel_ms,  G.st_refine_ms};
  for (int k = 0; k < n && k < 10; k++) out[k] = v[k];
  return 0;
}
int g6x_stats(double out[8]) { return g6x_stats_n(out, 8); }

int g6x_load(int n, const int *ids, const double *mass, const double (*x)[3],
             const double (*v)[3], const double (*acc)[3], const double (*jerk)[3],
             const double *t, const double *dt) {
  int rc = check_open();
  if (rc) return rc;
  if (n <= 0) return G6_ERR_ARG;
  rc = grow_j((n + G6_TILE - 1) / G6_TILE * G6_TILE);
  if (rc) return rc;
  /* Staged updates for these slots are superseded. */
  if (G.upd_inflight) {
    cudaEventSynchronize(G.ev_upd);
    G.upd_inflight = 0;
  }
  for (int u = 0; u < G.n_upd; u++) G.stage_pos[G.h_upd[u].addr] = -1;
  G.n_upd = 0;
  const size_t nd = sizeof(double) * (size_t)n;
  const int cap = G.js.cap;
  double *tmp = (double *)malloc(nd);
  if (!tmp) return G6_ERR_NOMEM;
  CK(cudaMemcpy(G.js.m, mass, nd, cudaMemcpyHostToDevice));
  if (t) {
    CK(cudaMemcpy(G.js.t, t, nd, cudaMemcpyHostToDevice));
  } else {
    CK(cudaMemset(G.js.t, 0, nd));
  }
  if (dt) {
    CK(cudaMemcpy(G.js.dt, dt, nd, cudaMemcpyHostToDevice));
  } else {
    CK(cudaMemset(G.js.dt, 0, nd));
  }
  const double(*src[4])[3] = {x, v, acc, jerk};
  double *dst[4] = {G.js.x, G.js.v, G.js.a, G.js.j};
  for (int q = 0; q < 4; q++) {
    for (int k = 0; k < 3; k++) {
      for (int s = 0; s < n; s++) tmp[s] = src[q] ? src[q][s][k] : 0.0;
      CK(cudaMemcpy(dst[q] + (size_t)k * cap, tmp, nd, cudaMemcpyHostToDevice));
    }
  }
  free(tmp);
  idmap_free(&G.ids);
  for (int s = 0; s < n; s++) {
    G.slot_id[s] = ids ? ids[s] : s;
    if (idmap_put(&G.ids, G.slot_id[s], s)) return G6_ERR_NOMEM;
  }
  for (int s = n; s < G.js.cap; s++) G.slot_id[s] = -1; /* slots beyond n are unused */
  CK(cudaMemcpy(G.js.id, G.slot_id, sizeof(int) * (size_t)n, cudaMemcpyHostToDevice));
  G.pred_valid = 0;
  G.run_n = n;
  G.run_t = 0;
  return 0;
}

int g6x_read(int n, double (*x)[3], double (*v)[3], double (*acc)[3], double (*jerk)[3],
             double *pot, double *t, double *dt, int *nn) {
  int rc = check_open();
  if (rc) return rc;
  if (n <= 0 || n > G.js.cap) return G6_ERR_ARG;
  CK(cudaStreamSynchronize(G.st));
  const size_t nd = sizeof(double) * (size_t)n;
  const int cap = G.js.cap;
  if (pot) CK(cudaMemcpy(pot, G.js.pot, nd, cudaMemcpyDeviceToHost));
  if (t) CK(cudaMemcpy(t, G.js.t, nd, cudaMemcpyDeviceToHost));
  if (dt) CK(cudaMemcpy(dt, G.js.dt, nd, cudaMemcpyDeviceToHost));
  if (nn) CK(cudaMemcpy(nn, G.js.nn, sizeof(int) * (size_t)n, cudaMemcpyDeviceToHost));
  double(*dst[4])[3] = {x, v, acc, jerk};
  const double *src[4] = {G.js.x, G.js.v, G.js.a, G.js.j};
  double *tmp = (double *)malloc(nd);
  if (!tmp) return G6_ERR_NOMEM;
  for (int q = 0; q < 4; q++) {
    if (!dst[q]) continue;
    for (int k = 0; k < 3; k++) {
      CK(cudaMemcpy(tmp, src[q] + (size_t)k * cap, nd, cudaMemcpyDeviceToHost));
      for (int s = 0; s < n; s++) dst[q][s][k] = tmp[s];
    }
  }
  free(tmp);
  return 0;
}

int g6x_force(double ti, double eps2, int nj, int ni, const double (*xi)[3],
              const double (*vi)[3], const int *self_slot, double (*acc)[3],
              double (*jerk)[3], double *pot, int *nn, float *nn_r2) {
  int rc = check_open();
  if (rc) return rc;
  G.ti = ti;
  int *self = NULL;
  if (!self_slot) {
    /* explicit points: nothing excluded */
    self = (int *)malloc(sizeof(int) * (size_t)(ni > 0 ? ni : 1));
    if (!self) return G6_ERR_NOMEM;
    for (int i = 0; i < ni; i++) self[i] = -1;
  }
  rc = stage_force_host(nj, ni, NULL, &xi[0][0], &vi[0][0], self_slot ? self_slot : self, eps2,
                        NULL);
  free(self);
  if (rc) return rc;
  rc = launch_force_host(nn != NULL || nn_r2 != NULL);
  if (rc) return rc;
  rc = finish_force(ni);
  if (rc) return rc;
  if (acc) memcpy(&acc[0][0], OUT_ACC(G.h_out), sizeof(double) * 3 * (size_t)ni);
  if (jerk) memcpy(&jerk[0][0], OUT_JERK(G.h_out), sizeof(double) * 3 * (size_t)ni);
  if (pot) memcpy(pot, OUT_POT(G.h_out), sizeof(double) * (size_t)ni);
  if (nn) memcpy(nn, OUT_NN(G.h_out), sizeof(int) * (size_t)ni);
  if (nn_r2) memcpy(nn_r2, OUT_NNR2(G.h_out), sizeof(float) * (size_t)ni);
  return 0;
}

static int read_err_word(void) {
  int herr = 0;
  if (G.d_err && cudaMemcpy(&herr, G.d_err, sizeof(int), cudaMemcpyDeviceToHost) == cudaSuccess &&
      herr) {
    seterr("force kernel reported error word 0x%x", herr);
    cudaMemset(G.d_err, 0, sizeof(int));
    return G6_ERR_KERNEL;
  }
  return 0;
}

int g6x_force_dev(double ti, double eps2, int nj, int ni, const double *d_xi,
                  const double *d_vi, const int *d_self_slot, double *d_acc, double *d_jerk,
                  double *d_pot, int *d_nn, float *d_nn_r2, int sync) {
  int rc = check_open();
  if (rc) return rc;
  if (ni <= 0 || nj <= 0) return ni == 0 ? 0 : G6_ERR_ARG;
  G.ti = ti;
  rc = ensure_io(1);
  if (rc) return rc;
  rc = flush_updates();
  if (rc) return rc;
  rc = predict_if_needed(nj);
  if (rc) return rc;
  g6_force_args a;
  memset(&a, 0, sizeof(a));
  a.ni = ni;
  a.nj = nj;
  a.prec = G.prec;
  a.eps2 = eps2;
  a.ipos = d_xi;
  a.ivel = d_vi;
  a.iself = d_self_slot;
  a.ti = ti;
  a.acc = d_acc;
  a.jerk = d_jerk;
  a.pot = d_pot;
  a.nn = d_nn;
  a.nn_r2 = d_nn_r2;
  a.want_nn = d_nn != NULL || d_nn_r2 != NULL;
  rc = run_force(&a);
  if (rc) return rc;
  if (sync) {
    CK(cudaStreamSynchronize(G.st));
    collect_timing();
    return read_err_word();
  }
  return 0;
}

int g6x_force_slots(double ti, double eps2, int nj, int ni, const int *d_ilist, double *d_acc,
                    double *d_jerk, double *d_pot, int *d_nn, int sync) {
  int rc = check_open();
  if (rc) return rc;
  if (ni <= 0 || nj <= 0) return ni == 0 ? 0 : G6_ERR_ARG;
  G.ti = ti;
  rc = ensure_io(1);
  if (rc) return rc;
  rc = flush_updates();
  if (rc) return rc;
  rc = predict_if_needed(nj);
  if (rc) return rc;
  g6_force_args a;
  memset(&a, 0, sizeof(a));
  a.ni = ni;
  a.nj = nj;
  a.prec = G.prec;
  a.eps2 = eps2;
  a.ilist = d_ilist;
  a.ti = ti;
  a.acc = d_acc;
  a.jerk = d_jerk;
  a.pot = d_pot;
  a.nn = d_nn;
  a.want_nn = d_nn != NULL;
  rc = run_force(&a);
  if (rc) return rc;
  if (sync) {
    CK(cudaStreamSynchronize(G.st));
    collect_timing();
    return read_err_word();
  }
  return 0;
}

/* ---- device-resident block-step driver ---- */

static int ensure_run_buffers(int n) {
  if (n <= G.run_cap) return 0;
  cudaFree(G.d_ilist); cudaFree(G.d_mail); cudaFree(G.d_sched);
  cudaFree(G.d_esum); cudaFree(G.d_racc); cudaFree(G.d_rjerk); cudaFree(G.d_rpot);
  cudaFree(G.d_rnn);
  G.d_mail = NULL;
  G.d_ni = NULL;
  G.d_tnext = NULL;
  G.run_cap = 0;
  ilist_identity_n = 0;
  size_t nd = sizeof(double) * (size_t)n;
  int ok = cudaMalloc((void **)&G.d_ilist, sizeof(int) * (size_t)n) == cudaSuccess &&
           cudaMalloc(&G.d_mail, 16) == cudaSuccess &&
           (G.h_mail || cudaHostAlloc(&G.h_mail, 16, cudaHostAllocDefault) == cudaSuccess) &&
           cudaMalloc((void **)&G.d_sched, sizeof(double) * 4) == cudaSuccess &&
           cudaMalloc((void **)&G.d_esum, sizeof(double) * (size_t)(4 + 2 * (n / 256 + 2))) ==
               cudaSuccess &&
           cudaMalloc((void **)&G.d_racc, 3 * nd) == cudaSuccess &&
           cudaMalloc((void **)&G.d_rjerk, 3 * nd) == cudaSuccess &&
           cudaMalloc((void **)&G.d_rpot, nd) == cudaSuccess &&
           cudaMalloc((void **)&G.d_rnn, sizeof(int) * (size_t)n) == cudaSuccess;
  if (!ok) {
    seterr("cannot allocate run buffers");
    return G6_ERR_NOMEM;
  }
  G.d_tnext = (double *)G.d_mail;
  G.d_ni = (int *)((char *)G.d_mail + 8);
  CK(cudaMemset(G.d_mail, 0, 16));
  G.run_cap = n;
  return 0;
}

/* ---- encounter check (extension API) ---- */

/* Radii by slot, at least n entries; entries added are zero. */
static int ensure_radius(int n) {
  if (n <= G.rad_cap) return 0;
  double *r = NULL;
  CK(cudaMalloc((void **)&r, sizeof(double) * (size_t)n));
  CK(cudaMemset(r, 0, sizeof(double) * (size_t)n));
  if (G.d_rad) {
    CK(cudaMemcpy(r, G.d_rad, sizeof(double) * (size_t)G.rad_cap, cudaMemcpyDeviceToDevice));
    cudaFree(G.d_rad);
  }
  G.d_rad = r;
  G.rad_cap = n;
  return 0;
}

static int ensure_enc_buffers(int n) {
  const int grid = (n + 31) / 32; /* enc_check_kernel: 32 particles per CTA */
  int rc = ensure_radius(n);
  if (rc) return rc;
  if (!G.d_enc) {
    g6_enc e;
    memset(&e, 0, sizeof(e));
    e.close_slot[0] = e.close_slot[1] = e.coll_slot[0] = e.coll_slot[1] = -1;
    e.close_id[0] = e.close_id[1] = e.coll_id[0] = e.coll_id[1] = -1;
    CK(cudaMalloc((void **)&G.d_enc, sizeof(g6_enc)));
    CK(cudaMemcpy(G.d_enc, &e, sizeof(e), cudaMemcpyHostToDevice));
    CK(cudaMalloc((void **)&G.d_enc_ctr, sizeof(unsigned)));
    CK(cudaMemset(G.d_enc_ctr, 0, sizeof(unsigned)));
  }
  if (grid > G.enc_cap) {
    cudaFree(G.d_encp_d);
    cudaFree(G.d_encp_i);
    G.d_encp_d = NULL;
    G.d_encp_i = NULL;
    G.enc_cap = 0;
    CK(cudaMalloc((void **)&G.d_encp_d, sizeof(double) * 2 * (size_t)grid));
    CK(cudaMalloc((void **)&G.d_encp_i, sizeof(int) * 4 * (size_t)grid));
    G.enc_cap = grid;
  }
  return 0;
}

int g6x_set_encounters(int mode, double rmin) {
  int rc = check_open();
  if (rc) return rc;
  if (mode & ~(G6_ENC_CHECK | G6_ENC_STOP_COLLISION | G6_ENC_STOP_CLOSE)) {
    seterr("g6x_set_encounters: unknown mode bits %#x", mode);
    return G6_ERR_ARG;
  }
  if (mode & (G6_ENC_STOP_COLLISION | G6_ENC_STOP_CLOSE)) mode |= G6_ENC_CHECK;
  if (!(rmin >= 0)) {
    seterr("g6x_set_encounters: rmin %g", rmin);
    return G6_ERR_ARG;
  }
  G.enc_mode = mode;
  G.enc_rmin = rmin;
  return 0;
}

int g6x_set_radius(int n, const double *radius) {
  int rc = check_open();
  if (rc) return rc;
  if (n < 0 || (n > 0 && !radius)) return G6_ERR_ARG;
  if (n == 0) return 0;
  rc = ensure_radius(n);
  if (rc) return rc;
  CK(cudaMemcpy(G.d_rad, radius, sizeof(double) * (size_t)n, cudaMemcpyHostToDevice));
  return 0;
}

/* ---- k nearest neighbours (extension API) ---- */
int g6x_knn(int k, int nj, double t, int ni, const int *slots, int *ids, double *d2) {
  int rc = check_open();
  if (rc) return rc;
  if (k < 1 || k > G6_KNN_MAX || ni < 0 || nj < 1 || nj > G.js.cap || (ni > 0 && !slots)) {
    seterr("g6x_knn: k=%d nj=%d ni=%d", k, nj, ni);
    return G6_ERR_ARG;
  }
  if (ni == 0) return 0;
  if (!ids || !d2) return G6_ERR_ARG;
  for (int i = 0; i < ni; i++)
    if (slots[i] < 0 || slots[i] >= nj) {
      seterr("g6x_knn: slot %d out of [0, %d)", slots[i], nj);
      return G6_ERR_ARG;
    }
  rc = flush_updates();
  if (rc) return rc;
  /* the filter reads the split records: predict them to t */
  if (g6k_predict(&G.js, nj, t, G6_PREC_SPLIT, G.st)) return G6_ERR_CUDA;
  G.pred_valid = 0;
  const size_t io = (sizeof(int) * 2 + sizeof(double)) * (size_t)ni * (size_t)k + 256;
  const size_t need = g6k_knn_scratch_bytes(nj, ni, k) + io + sizeof(int) * (size_t)ni + 512;
  if (need > G.knn_bytes) {
    cudaFree(G.d_knn);
    G.d_knn = NULL;
    G.knn_bytes = 0;
    CK(cudaMalloc(&G.d_knn, need));
    G.knn_bytes = need;
  }
  char *p = (char *)G.d_knn;
  int *d_slots = (int *)p;
  p += ((sizeof(int) * (size_t)ni + 255) / 256) * 256;
  int *d_ids = (int *)p;
  p += ((sizeof(int) * (size_t)ni * k + 255) / 256) * 256;
  double *d_d2 = (double *)p;
  p += ((sizeof(double) * (size_t)ni * k + 255) / 256) * 256;
  const size_t rest = G.knn_bytes - (size_t)(p - (char *)G.d_knn);
  CK(cudaMemcpyAsync(d_slots, slots, sizeof(int) * (size_t)ni, cudaMemcpyHostToDevice, G.st));
  rc = g6k_knn(&G.js, nj, t, k, ni, d_slots, d_ids, d_d2, p, rest, G.st);
  if (rc) {
    seterr("knn launch failed (%d)", rc);
    return G6_ERR_CUDA;
  }
  CK(cudaMemcpyAsync(ids, d_ids, sizeof(int) * (size_t)ni * k, cudaMemcpyDeviceToHost, G.st));
  CK(cudaMemcpyAsync(d2, d_d2, sizeof(double) * (size_t)ni * k, cudaMemcpyDeviceToHost, G.st));
  CK(cudaStreamSynchronize(G.st));
  return 0;
}

int g6x_encounter(int ids[4], double out[4]) {
  int rc = check_open();
  if (rc) return rc;
  g6_enc e;
  memset(&e, 0, sizeof(e));
  e.close_id[0] = e.close_id[1] = e.coll_id[0] = e.coll_id[1] = -1;
  if (G.d_enc) {
    CK(cudaStreamSynchronize(G.st));
    CK(cudaMemcpy(&e, G.d_enc, sizeof(e), cudaMemcpyDeviceToHost));
  }
  if (ids) {
    ids[0] = e.close_id[0];
    ids[1] = e.close_id[1];
    ids[2] = e.coll_id[0];
    ids[3] = e.coll_id[1];
  }
  if (out) {
    out[0] = e.stopped;
    out[1] = e.t;
    out[2] = e.rmax_close;
    out[3] = e.rmax_coll;
  }
  return 0;
}

static int identity_list(int n) {
  if (ilist_identity_n == n) return 0;
  int *h = (int *)malloc(sizeof(int) * (size_t)n);
  if (!h) return G6_ERR_NOMEM;
  for (int s = 0; s < n; s++) h[s] = s;
  cudaError_t e = cudaMemcpy(G.d_ilist, h, sizeof(int) * (size_t)n, cudaMemcpyHostToDevice);
  free(h);
  ilist_identity_n = e == cudaSuccess ? n : 0;
  return e == cudaSuccess ? 0 : G6_ERR_CUDA;
}

static int cmp_dbl(const void *a, const void *b) {
  double x = *(const double *)a, y = *(const double *)b;
  return (x > y) - (x < y);
}

int g6x_run_init(double eps2, double eta) {
  int rc = check_open();
  if (rc) return rc;
  const int n = G.run_n;
  if (n <= 0) return G6_ERR_STATE;
  rc = ensure_run_buffers(n);
  if (rc) return rc;
  rc = identity_list(n);
  if (rc) return rc;
  G.run_eps2 = eps2;
  G.run_eta = eta;
  G.run_t = 0;
  /* idata::setup: forces on all at t = 0 (commit_particles). */
  rc = g6x_force_slots(0.0, eps2, n, n, G.d_ilist, G.d_racc, G.d_rjerk, G.d_rpot, G.d_rnn, 0);
  if (rc) return rc;
  if (g6k_store_forces(&G.js, n, G.d_ilist, G.d_racc, G.d_rjerk, G.d_rpot, G.d_rnn, G.st))
    return G6_ERR_CUDA;
  /* force_initial_timestep(0.0625, 0.03125, 8.0) (interface.cc:29-31). */
  if (g6k_initial_step(&G.js, n, eta, 0.0625, 0.03125, 0.0, G.st)) return G6_ERR_CUDA;
  double *h = (double *)malloc(sizeof(double) * (size_t)n);
  if (!h) return G6_ERR_NOMEM;
  CK(cudaMemcpyAsync(h, G.js.dt, sizeof(double) * (size_t)n, cudaMemcpyDeviceToHost, G.st));
  CK(cudaStreamSynchronize(G.st));
  qsort(h, (size_t)n, sizeof(double), cmp_dbl);
  const double dtmax = 8.0 * h[n / 2];
  free(h);
  if (g6k_clamp_steps(&G.js, n, dtmax, G.st)) return G6_ERR_CUDA;
  G.pred_valid = 0;
  CK(cudaStreamSynchronize(G.st));
  return read_err_word();
}

static double run_stats[4]; /* last g6x_run: blocks, wall ms, ms waiting in syncs, steps */

static double now_ms(void) {
  struct timespec ts;
  clock_gettime(CLOCK_MONOTONIC, &ts);
  return ts.tv_sec * 1e3 + ts.tv_nsec * 1e-6;
}

int g6x_run_stats(double out[4]) {
  if (!out) return G6_ERR_ARG;
  memcpy(out, run_stats, sizeof(run_stats));
  return 0;
}

int g6x_run(double t_end, long long *blocks, double *particle_steps) {
  int rc = check_open();
  if (rc) return rc;
  const double w0 = now_ms();
  double wsync = 0;
  const int n = G.run_n;
  if (n <= 0 || G.run_cap < n) return G6_ERR_STATE;
  const long long max_blocks = blocks && *blocks > 0 ? *blocks : -1;
  long long nb = 0;
  double ns = 0;
  int hbuf[2];
  double tn;
  /* Encounter check: the force also finds each block particle's nearest
     neighbour and a pass before the corrector evaluates ph4's criteria.  The
     stopping test on the corrected pair runs in the first kernel of the next
     block's scheduler (or after the loop), and its stop bits reach the host
     in that block's mailbox copy, before that block's force is launched. */
  const int enc = G.enc_mode;
  const double rmin = G.enc_rmin > 0 ? G.enc_rmin : 2.0 / n; /* jdata.cc:426 */
  int *d_stop = (int *)((char *)G.d_mail + 12);
  if (enc) {
    rc = ensure_enc_buffers(n);
    if (rc) return rc;
    CK(cudaMemsetAsync(d_stop, 0, sizeof(int), G.st));
  }
  g6_enc_decision_args pend; /* the last block's stopping decision, taken by the next schedule */
  memset(&pend, 0, sizeof(pend));
  /* Per block: sched_first (min of t + dt), list_predict (the block list,
     tnext, all j predicted to tnext), the mailbox copy and the one host
     synchronisation, then the force on the block (split merge in the force
     kernel, refinement pass), [encounter check], corrector.  The two
     minima alternate by block parity: each list_predict resets the other. */
  unsigned long long *dmin2 = (unsigned long long *)G.d_sched;
  int parity = 0;
  if (g6k_sched_reset(dmin2, G.d_ni, G.st)) return G6_ERR_CUDA;
  while (G.run_t < t_end && nb != max_blocks) {
    ilist_identity_n = 0;
    if (g6k_sched_first(&G.js, n, dmin2 + parity, G.d_ni, pend.enc ? &pend : NULL, G.st) ||
        g6k_list_predict(&G.js, n, G.prec, dmin2 + parity, dmin2 + (parity ^ 1), G.d_ilist,
                         G.d_ni, G.d_tnext, G.st))
      return G6_ERR_CUDA;
    parity ^= 1;
    pend.enc = NULL;
    /* one 16-byte copy into pinned memory: the only host round trip per block */
    CK(cudaMemcpyAsync(G.h_mail, G.d_mail, 16, cudaMemcpyDeviceToHost, G.st));
    const double s0 = now_ms();
    CK(cudaStreamSynchronize(G.st));
    wsync += now_ms() - s0;
    memcpy(&tn, G.h_mail, sizeof(double));
    memcpy(hbuf, (const char *)G.h_mail + 8, 2 * sizeof(int));
    if (enc && hbuf[1]) break; /* the previous block met a stopping condition */
    const int ni = hbuf[0];
    if (ni <= 0 || ni > n || !(tn > G.run_t)) {
      seterr("scheduler produced ni=%d tnext=%.17g at t=%.17g", ni, tn, G.run_t);
      return G6_ERR_STATE;
    }
    /* list_predict has predicted every j to tn */
    G.pred_valid = 1;
    G.pred_t = tn;
    G.pred_nj = n;
    G.pred_prec = G.prec;
    rc = g6x_force_slots(tn, G.run_eps2, n, ni, G.d_ilist, G.d_racc, G.d_rjerk, G.d_rpot,
                         enc ? G.d_rnn : NULL, 0);
    if (rc) return rc;
    if (enc && g6k_enc_check(&G.js, G.d_rad, ni, G.d_ilist, G.d_rnn, tn, rmin, G.d_encp_d,
                             G.d_encp_i, G.d_enc_ctr, G.d_enc, G.st))
      return G6_ERR_CUDA;
    if (g6k_correct(&G.js, ni, G.d_ilist, tn, G.run_eta, G.d_racc, G.d_rjerk, G.d_rpot,
                    enc ? G.d_rnn : NULL, G.st))
      return G6_ERR_CUDA;
    if (enc) {
      pend.enc = G.d_enc;
      pend.mode = enc;
      pend.t = tn;
      pend.flag = d_stop;
    }
    G.pred_valid = 0; /* j-state changed */
    G.run_t = tn;
    nb++;
    ns += ni;
  }
  /* the loop ended on time or block count: the last block's stopping decision */
  if (pend.enc && g6k_enc_decide(&G.js, pend.enc, pend.mode, pend.t, pend.flag, G.st))
    return G6_ERR_CUDA;
  CK(cudaStreamSynchronize(G.st));
  run_stats[0] = (double)nb;
  run_stats[1] = now_ms() - w0;
  run_stats[2] = wsync;
  run_stats[3] = ns;
  if (blocks) *blocks = nb;
  if (particle_steps) *particle_steps = ns;
  return read_err_word();
}

int g6x_correct(int ni, const int *slots, double tnext, double eta, const double (*acc)[3],
                const double (*jerk)[3]) {
  int rc = check_open();
  if (rc) return rc;
  if (ni <= 0) return 0;
  if (ni > G.js.cap) return G6_ERR_ARG;
  for (int i = 0; i < ni; i++)
    if (slots[i] < 0 || slots[i] >= G.js.cap) {
      seterr("g6x_correct: slot %d out of range", slots[i]);
      return G6_ERR_ARG;
    }
  rc = ensure_run_buffers(ni > G.run_n ? ni : (G.run_n > 0 ? G.run_n : ni));
  if (rc) return rc;
  ilist_identity_n = 0;
  CK(cudaMemcpyAsync(G.d_ilist, slots, sizeof(int) * (size_t)ni, cudaMemcpyHostToDevice, G.st));
  CK(cudaMemcpyAsync(G.d_racc, acc, sizeof(double) * 3 * (size_t)ni, cudaMemcpyHostToDevice,
                     G.st));
  CK(cudaMemcpyAsync(G.d_rjerk, jerk, sizeof(double) * 3 * (size_t)ni, cudaMemcpyHostToDevice,
                     G.st));
  if (g6k_correct(&G.js, ni, G.d_ilist, tnext, eta, G.d_racc, G.d_rjerk, NULL, NULL, G.st))
    return G6_ERR_CUDA;
  G.pred_valid = 0;
  CK(cudaStreamSynchronize(G.st));
  return 0;
}

int g6x_step_all(double tnext) {
  int rc = check_open();
  if (rc) return rc;
  const int n = G.run_n;
  if (n <= 0 || G.run_cap < n) return G6_ERR_STATE;
  rc = identity_list(n);
  if (rc) return rc;
  rc = g6x_force_slots(tnext, G.run_eps2, n, n, G.d_ilist, G.d_racc, G.d_rjerk, G.d_rpot,
                       NULL, 0);
  if (rc) return rc;
  if (g6k_correct(&G.js, n, G.d_ilist, tnext, G.run_eta, G.d_racc, G.d_rjerk, G.d_rpot,
                  NULL, G.st))
    return G6_ERR_CUDA;
  G.pred_valid = 0;
  G.run_t = tnext;
  return 0;
}

double g6x_system_time(void) { return G.run_t; }

int g6x_energy(double *kinetic, double *potential) {
  int rc = check_open();
  if (rc) return rc;
  const int n = G.run_n;
  if (n <= 0 || G.run_cap < n) return G6_ERR_STATE;
  /* jdata::get_energy: pot of all particles predicted to system time. */
  rc = identity_list(n);
  if (rc) return rc;
  rc = g6x_force_slots(G.run_t, G.run_eps2, n, n, G.d_ilist, G.d_racc, G.d_rjerk, G.d_rpot,
                       NULL, 0);
  if (rc) return rc;
  if (g6k_energy_sums(&G.js, n, G.run_t, G.d_rpot, G.d_esum, G.st)) return G6_ERR_CUDA;
  double h[2];
  CK(cudaMemcpyAsync(h, G.d_esum, sizeof(h), cudaMemcpyDeviceToHost, G.st));
  CK(cudaStreamSynchronize(G.st));
  if (kinetic) *kinetic = h[0] / 2;
  if (potential) *potential = h[1] / 2;
  return read_err_word();
}

/* ---- force without any device allocation ----
 * For callers that must not allocate device memory during the call: code
 * whose device memory is owned and budgeted by a host framework (the
 * framework hands out every buffer, so a library cudaMalloc would either fail
 * or break its accounting), or code that cannot tolerate the implicit device
 * synchronisation and latency of cudaMalloc/cudaFree in its step loop.  The
 * j-system must already be resident (loaded and sized by earlier calls); the
 * split-j partial sums go to a fixed 16 MiB device array inside the library
 * instead of the growable scratch buffer.  That array is taken, and its device
 * address looked up, in g6_open; the refinement queue is allocated there too.
 * Calls needing more than that, a larger j-store, or a larger update buffer
 * are refused, never allocated. */
size_t g6k_static_scratch_capacity(void);
int g6k_force_static(const g6_force_args *a, void *static_addr, g6_shape *shape,
                     cudaStream_t st, size_t *need_out);

int g6x_force_dev_noalloc(double ti, double eps2, int nj, int ni, const double *d_xi,
                          const double *d_vi, const int *d_self_slot, double *d_acc,
                          double *d_jerk, double *d_pot, int *d_nn, int sync) {
  int rc = check_open();
  if (rc) return rc;
  if (ni < 0 || nj < 0) return G6_ERR_ARG;
  if (ni == 0) return 0;
  if (nj == 0 || !d_xi || !d_vi || !d_acc || !d_jerk || !d_pot) {
    seterr("g6x_force_dev_noalloc: nj = 0 or a NULL input/output pointer");
    return G6_ERR_ARG;
  }
  const int nj_pad = (nj + G6_TILE - 1) / G6_TILE * G6_TILE;
  if (nj_pad > G.js.cap) {
    seterr("g6x_force_dev_noalloc: nj=%d exceeds the j-store (%d slots); it would need an "
           "allocation", nj, G.js.cap);
    return G6_ERR_ARG;
  }
  if (G.n_upd > G.cap_dupd) {
    seterr("g6x_force_dev_noalloc: %d staged j updates exceed the update buffer (%d); it would "
           "need an allocation", G.n_upd, G.cap_dupd);
    return G6_ERR_ARG;
  }
  if (!G.d_err) {
    seterr("g6x_force_dev_noalloc: library i/o buffers missing");
    return G6_ERR_STATE;
  }
  G.ti = ti;
  rc = flush_updates(); /* copies into the existing update buffer only */
  if (rc) return rc;
  rc = predict_if_needed(nj); /* the j-store already holds nj_pad slots */
  if (rc) return rc;
  g6_force_args a;
  memset(&a, 0, sizeof(a));
  a.ni = ni;
  a.nj = nj;
  a.prec = G.prec;
  a.eps2 = eps2;
  a.ipos = d_xi;
  a.ivel = d_vi;
  a.iself = d_self_slot;
  a.ti = ti;
  a.acc = d_acc;
  a.jerk = d_jerk;
  a.pot = d_pot;
  a.nn = d_nn;
  a.want_nn = d_nn != NULL;
  a.js = &G.js;
  a.err = G.d_err;
  refine_args(&a); /* fixed buffer, allocated at open */
  size_t need = 0;
  if (G.timing && !G.predicted_this_call) cudaEventRecord(G.ev_t1, G.st);
  a.ev_mid = G.timing ? G.ev_tm : NULL;
  rc = g6k_force_static(&a, G.d_static, &G.shape, G.st, &need);
  if (rc == -4) {
    seterr("g6x_force_dev_noalloc: ni=%d, nj=%d needs %zu B of split-j scratch, more than the "
           "fixed %zu B; use g6x_force_dev or fewer i-particles per call", ni, nj, need,
           g6k_static_scratch_capacity());
    return G6_ERR_ARG;
  }
  if (rc) {
    seterr("g6x_force_dev_noalloc: launch failed (%d)", rc);
    return G6_ERR_CUDA;
  }
  if (G.timing) cudaEventRecord(G.ev_t2, G.st);
  G.st_pairs = (double)ni * (double)(nj - 1);
  G.st_nj = nj;
  G.st_pred_bytes = G.predicted_this_call
                        ? (double)nj * (15.0 * 8.0 + (G.prec == G6_PREC_FP64 ? 64.0 : 48.0))
                        : 0.0;
  if (sync) {
    CK(cudaStreamSynchronize(G.st));
    collect_timing();
    return read_err_word();
  }
  return 0;
}

/* ===================================== batched few-body systems ======= */
/* Many independent systems (n <= 64 each) integrated with smallN's scheme
 * in one persistent kernel fed by a device work queue (kern_batch.cu).  The
 * queue-reset + kernel pair is captured in a CUDA graph, re-captured only
 * when buffers or parameters change.  Launch shape (warps per CTA, CTAs per
 * SM) comes from g6x_batch_tune or defaults to 4 x 2. */
int g6k_batch_max_n(void);
int g6k_batch_launch_unp(const int *order, const int *off, const double *t_end,
                         const double *mass, double *pos, double *vel, double eta, int n_iter,
                         long long max_steps, int mode, int warps_per_cta, int ctas,
                         double dt_crit, double r2_crit, double gamma, int allow_full, int *queue,
                         double *t_out, long long *steps_out, unsigned long long *wall_ns,
                         int *status, int *nbin_out, cudaStream_t st);
int g6k_batch_launch(const int *order, const int *off, const double *t_end,
                     const double *mass, double *pos, double *vel, double eta, int n_iter,
                     long long max_steps, int exact, int warps_per_cta, int ctas, int *queue,
                     double *t_out, long long *steps_out, unsigned long long *wall_ns,
                     int *status, cudaStream_t st);

static struct {
  int cap_sys, cap_body;
  int *d_order, *d_off, *d_queue, *d_status;
  double *d_tend, *d_mass, *d_pos, *d_vel, *d_tout;
  long long *d_steps;
  unsigned long long *d_wall;
  int wpc, cps; /* warps per CTA, CTAs per SM */
  cudaGraphExec_t gexec;
  int g_exact, g_niter, g_wpc, g_cps;
  double g_eta;
  long long g_maxsteps;
  void *g_key;
  /* smallN's unperturbed binaries (g6x_batch_unperturbed) */
  int unp, unp_full;
  double unp_dt_crit, unp_r2_crit, unp_gamma;
  int *d_nbin;
  int g_unp;
} BT = {0, 0, NULL, NULL, NULL, NULL, NULL, NULL, NULL, NULL, NULL, NULL, NULL, 4, 2,
        NULL, 0, 0, 0, 0, 0.0, 0, NULL, 0, 0, 0.0, 0.0, 0.0, NULL, 0};

static void batch_free(void) {
  cudaFree(BT.d_order); cudaFree(BT.d_off); cudaFree(BT.d_queue); cudaFree(BT.d_status);
  cudaFree(BT.d_tend); cudaFree(BT.d_mass); cudaFree(BT.d_pos); cudaFree(BT.d_vel);
  cudaFree(BT.d_tout); cudaFree(BT.d_steps); cudaFree(BT.d_wall); cudaFree(BT.d_nbin);
  if (BT.gexec) cudaGraphExecDestroy(BT.gexec);
  const int wpc = BT.wpc, cps = BT.cps, unp = BT.unp, full = BT.unp_full;
  const double dc = BT.unp_dt_crit, r2 = BT.unp_r2_crit, g = BT.unp_gamma;
  memset(&BT, 0, sizeof(BT));
  BT.wpc = wpc;
  BT.cps = cps;
  BT.unp = unp;
  BT.unp_full = full;
  BT.unp_dt_crit = dc;
  BT.unp_r2_crit = r2;
  BT.unp_gamma = g;
}

static int batch_ensure(int nsys, int nbody) {
  if (nsys > BT.cap_sys) {
    cudaFree(BT.d_order); cudaFree(BT.d_off); cudaFree(BT.d_tend); cudaFree(BT.d_tout);
    cudaFree(BT.d_steps); cudaFree(BT.d_wall); cudaFree(BT.d_status); cudaFree(BT.d_nbin);
    BT.cap_sys = 0;
    size_t s = (size_t)nsys;
    if (cudaMalloc((void **)&BT.d_order, sizeof(int) * s) != cudaSuccess ||
        cudaMalloc((void **)&BT.d_off, sizeof(int) * (s + 1)) != cudaSuccess ||
        cudaMalloc((void **)&BT.d_tend, sizeof(double) * s) != cudaSuccess ||
        cudaMalloc((void **)&BT.d_tout, sizeof(double) * s) != cudaSuccess ||
        cudaMalloc((void **)&BT.d_steps, sizeof(long long) * s) != cudaSuccess ||
        cudaMalloc((void **)&BT.d_wall, sizeof(unsigned long long) * s) != cudaSuccess ||
        cudaMalloc((void **)&BT.d_status, sizeof(int) * s) != cudaSuccess ||
        cudaMalloc((void **)&BT.d_nbin, sizeof(int) * s) != cudaSuccess) {
      seterr("cannot allocate batch buffers for %d systems", nsys);
      return G6_ERR_NOMEM;
    }
    BT.cap_sys = nsys;
  }
  if (nbody > BT.cap_body) {
    cudaFree(BT.d_mass); cudaFree(BT.d_pos); cudaFree(BT.d_vel);
    BT.cap_body = 0;
    size_t b = (size_t)nbody;
    if (cudaMalloc((void **)&BT.d_mass, sizeof(double) * b) != cudaSuccess ||
        cudaMalloc((void **)&BT.d_pos, sizeof(double) * 3 * b) != cudaSuccess ||
        cudaMalloc((void **)&BT.d_vel, sizeof(double) * 3 * b) != cudaSuccess) {
      seterr("cannot allocate batch buffers for %d bodies", nbody);
      return G6_ERR_NOMEM;
    }
    BT.cap_body = nbody;
  }
  /* [0] the work counter, [1] the number of systems of the current launch */
  if (!BT.d_queue && cudaMalloc((void **)&BT.d_queue, 2 * sizeof(int)) != cudaSuccess)
    return G6_ERR_NOMEM;
  return 0;
}

static int cmp_desc_n(const void *a, const void *b) {
  const int *x = (const int *)a, *y = (const int *)b; /* (n, index) pairs */
  if (x[0] != y[0]) return y[0] - x[0];
  return x[1] - y[1];
}

/* Launch through a (cached) CUDA graph: queue reset + persistent kernel.
   The kernel reads the number of systems from the device, so one graph
   serves every batch size (a multiples hand-off shrinks the batch at every
   increment). */
static int batch_graph_launch(int nsys, double eta, int n_iter, long long max_steps, int exact) {
  const int ctas = BT.cps * g6k_sm_count();
  const int unp = BT.unp && exact != G6_BATCH_EXACT;
  CK(cudaMemcpyAsync(BT.d_queue + 1, &nsys, sizeof(int), cudaMemcpyHostToDevice, G.st));
  if (!BT.gexec || BT.g_exact != exact || BT.g_niter != n_iter ||
      BT.g_eta != eta || BT.g_maxsteps != max_steps || BT.g_wpc != BT.wpc ||
      BT.g_cps != BT.cps || BT.g_key != (void *)BT.d_pos || BT.g_unp != unp) {
    if (BT.gexec) {
      cudaGraphExecDestroy(BT.gexec);
      BT.gexec = NULL;
    }
    cudaGraph_t g;
    CK(cudaStreamBeginCapture(G.st, cudaStreamCaptureModeThreadLocal));
    int rc = unp ? g6k_batch_launch_unp(BT.d_order, BT.d_off, BT.d_tend, BT.d_mass,
                                        BT.d_pos, BT.d_vel, eta, n_iter, max_steps, exact,
                                        BT.wpc, ctas, BT.unp_dt_crit, BT.unp_r2_crit,
                                        BT.unp_gamma, BT.unp_full, BT.d_queue, BT.d_tout,
                                        BT.d_steps, BT.d_wall, BT.d_status, BT.d_nbin, G.st)
                 : g6k_batch_launch(BT.d_order, BT.d_off, BT.d_tend, BT.d_mass, BT.d_pos,
                                    BT.d_vel, eta, n_iter, max_steps, exact, BT.wpc, ctas,
                                    BT.d_queue, BT.d_tout, BT.d_steps, BT.d_wall, BT.d_status,
                                    G.st);
    cudaError_t e = cudaStreamEndCapture(G.st, &g);
    if (rc || e != cudaSuccess) {
      seterr("batch graph capture failed (%d, %s)", rc, cudaGetErrorString(e));
      return G6_ERR_CUDA;
    }
    e = cudaGraphInstantiate(&BT.gexec, g, 0);
    cudaGraphDestroy(g);
    if (e != cudaSuccess) {
      seterr("batch graph instantiate failed: %s", cudaGetErrorString(e));
      BT.gexec = NULL;
      return G6_ERR_CUDA;
    }
    BT.g_exact = exact;
    BT.g_niter = n_iter;
    BT.g_eta = eta;
    BT.g_maxsteps = max_steps;
    BT.g_wpc = BT.wpc;
    BT.g_cps = BT.cps;
    BT.g_key = (void *)BT.d_pos;
    BT.g_unp = unp;
  }
  CK(cudaGraphLaunch(BT.gexec, G.st));
  return 0;
}

int g6x_batch_unperturbed(int on, double dt_crit, double r2_crit, double gamma, int allow_full) {
  if (on && !(dt_crit >= 0 && r2_crit >= 0 && gamma > 0)) return G6_ERR_ARG;
  BT.unp = on ? 1 : 0;
  BT.unp_dt_crit = dt_crit;
  BT.unp_r2_crit = r2_crit;
  BT.unp_gamma = gamma;
  BT.unp_full = allow_full ? 1 : 0;
  return 0;
}

int g6x_batch_binaries(int nsys, int *nbin) {
  int rc = check_open();
  if (rc) return rc;
  if (nsys <= 0 || nsys > BT.cap_sys || !nbin || !BT.d_nbin) return G6_ERR_ARG;
  CK(cudaMemcpy(nbin, BT.d_nbin, sizeof(int) * (size_t)nsys, cudaMemcpyDeviceToHost));
  return 0;
}

int g6x_batch_config(int warps_per_cta, int ctas_per_sm) {
  if (warps_per_cta < 1 || warps_per_cta > 8 || ctas_per_sm < 1 || ctas_per_sm > 16)
    return G6_ERR_ARG;
  BT.wpc = warps_per_cta;
  BT.cps = ctas_per_sm;
  return 0;
}

int g6x_batch_run(int nsys, const int *n_per_sys, const double *t_end, const double *mass,
                  double (*pos)[3], double (*vel)[3], double eta, int n_iter,
                  long long max_steps, int exact, double *t_final, long long *steps,
                  double *wall_ms, int *status, double *elapsed_ms) {
  int rc = check_open();
  if (rc) return rc;
  if (nsys <= 0 || !n_per_sys || !t_end || !mass || !pos || !vel || n_iter < 0 || eta <= 0 ||
      exact < G6_BATCH_FAST || exact > G6_BATCH_SPLIT)
    return G6_ERR_ARG;
  if (BT.unp && exact == G6_BATCH_EXACT) {
    seterr("g6x_batch_run: the exact mode reproduces smallN without unperturbed binaries; "
           "switch them off (g6x_batch_unperturbed) or use the fast or split mode");
    return G6_ERR_ARG;
  }
  if (BT.unp && BT.wpc > 4) {
    seterr("g6x_batch_run: with unperturbed binaries at most 4 warps per CTA");
    return G6_ERR_ARG;
  }
  const int maxn = g6k_batch_max_n();
  int *off = (int *)malloc(sizeof(int) * (size_t)(nsys + 1));
  int *pairs = (int *)malloc(sizeof(int) * 2 * (size_t)nsys);
  int *order = (int *)malloc(sizeof(int) * (size_t)nsys);
  if (!off || !pairs || !order) {
    free(off); free(pairs); free(order);
    return G6_ERR_NOMEM;
  }
  off[0] = 0;
  for (int s = 0; s < nsys; s++) {
    if (n_per_sys[s] < 2 || n_per_sys[s] > maxn) {
      seterr("g6x_batch_run: system %d has n=%d (supported 2..%d)", s, n_per_sys[s], maxn);
      free(off); free(pairs); free(order);
      return G6_ERR_ARG;
    }
    off[s + 1] = off[s] + n_per_sys[s];
    pairs[2 * s] = n_per_sys[s];
    pairs[2 * s + 1] = s;
  }
  /* largest systems first: the queue then balances like LPT scheduling */
  qsort(pairs, (size_t)nsys, 2 * sizeof(int), cmp_desc_n);
  for (int q = 0; q < nsys; q++) order[q] = pairs[2 * q + 1];
  const int nb = off[nsys];
  rc = batch_ensure(nsys, nb);
  if (rc == 0) {
    cudaMemcpyAsync(BT.d_order, order, sizeof(int) * (size_t)nsys, cudaMemcpyHostToDevice, G.st);
    cudaMemcpyAsync(BT.d_off, off, sizeof(int) * (size_t)(nsys + 1), cudaMemcpyHostToDevice, G.st);
    cudaMemcpyAsync(BT.d_tend, t_end, sizeof(double) * (size_t)nsys, cudaMemcpyHostToDevice, G.st);
    cudaMemcpyAsync(BT.d_mass, mass, sizeof(double) * (size_t)nb, cudaMemcpyHostToDevice, G.st);
    cudaMemcpyAsync(BT.d_pos, &pos[0][0], sizeof(double) * 3 * (size_t)nb, cudaMemcpyHostToDevice,
                    G.st);
    cudaMemcpyAsync(BT.d_vel, &vel[0][0], sizeof(double) * 3 * (size_t)nb, cudaMemcpyHostToDevice,
                    G.st);
    cudaEventRecord(G.ev_t0, G.st);
    rc = batch_graph_launch(nsys, eta, n_iter, max_steps > 0 ? max_steps : (1LL << 40), exact);
    cudaEventRecord(G.ev_t1, G.st);
  }
  free(off); free(pairs); free(order);
  if (rc) return rc;
  CK(cudaMemcpyAsync(&pos[0][0], BT.d_pos, sizeof(double) * 3 * (size_t)nb, cudaMemcpyDeviceToHost,
                     G.st));
  CK(cudaMemcpyAsync(&vel[0][0], BT.d_vel, sizeof(double) * 3 * (size_t)nb, cudaMemcpyDeviceToHost,
                     G.st));
  unsigned long long *wall = (unsigned long long *)malloc(sizeof(unsigned long long) * (size_t)nsys);
  if (!wall) return G6_ERR_NOMEM;
  CK(cudaMemcpyAsync(wall, BT.d_wall, sizeof(unsigned long long) * (size_t)nsys,
                     cudaMemcpyDeviceToHost, G.st));
  if (t_final)
    CK(cudaMemcpyAsync(t_final, BT.d_tout, sizeof(double) * (size_t)nsys, cudaMemcpyDeviceToHost,
                       G.st));
  if (steps)
    CK(cudaMemcpyAsync(steps, BT.d_steps, sizeof(long long) * (size_t)nsys,
                       cudaMemcpyDeviceToHost, G.st));
  if (status)
    CK(cudaMemcpyAsync(status, BT.d_status, sizeof(int) * (size_t)nsys, cudaMemcpyDeviceToHost,
                       G.st));
  cudaError_t e = cudaStreamSynchronize(G.st);
  if (e != cudaSuccess) {
    free(wall);
    seterr("batch run failed: %s", cudaGetErrorString(e));
    return G6_ERR_CUDA;
  }
  if (wall_ms)
    for (int s = 0; s < nsys; s++) wall_ms[s] = (double)wall[s] * 1e-6;
  free(wall);
  if (elapsed_ms) {
    float ms = 0;
    cudaEventElapsedTime(&ms, G.ev_t0, G.ev_t1);
    *elapsed_ms = ms;
  }
  return 0;
}

/* Autotuner: time every (warps per CTA, CTAs per SM) shape whose warps fit
 * the register file on a copy of the given systems (shortened to frac of
 * their end time) and keep the fastest.  out[0..2] = best wpc, cps, ms. */
int g6x_batch_tune(int nsys, const int *n_per_sys, const double *t_end, const double *mass,
                   const double (*pos)[3], const double (*vel)[3], double eta, int n_iter,
                   int exact, double frac, double out[3]) {
  int rc = check_open();
  if (rc) return rc;
  if (nsys <= 0 || frac <= 0) return G6_ERR_ARG;
  int nb = 0;
  for (int s = 0; s < nsys; s++) nb += n_per_sys[s];
  double *te = (double *)malloc(sizeof(double) * (size_t)nsys);
  double(*p)[3] = (double(*)[3])malloc(sizeof(double) * 3 * (size_t)nb);
  double(*v)[3] = (double(*)[3])malloc(sizeof(double) * 3 * (size_t)nb);
  if (!te || !p || !v) {
    free(te); free(p); free(v);
    return G6_ERR_NOMEM;
  }
  for (int s = 0; s < nsys; s++) te[s] = t_end[s] * frac;
  static const int shapes[][2] = {{1, 8}, {2, 4}, {2, 6}, {4, 2}, {4, 3}, {8, 1}, {1, 4},
                                  {2, 2}, {4, 1}, {1, 12}, {3, 4}, {6, 2}};
  const int nshape = (int)(sizeof(shapes) / sizeof(shapes[0]));
  double best = 1e300;
  int bw = BT.wpc, bc = BT.cps;
  for (int k = 0; k < nshape; k++) {
    if (BT.unp && shapes[k][0] > 4) continue; /* that kernel holds 4 warps per CTA at most */
    memcpy(p, pos, sizeof(double) * 3 * (size_t)nb);
    memcpy(v, vel, sizeof(double) * 3 * (size_t)nb);
    BT.wpc = shapes[k][0];
    BT.cps = shapes[k][1];
    double ms = 0;
    rc = g6x_batch_run(nsys, n_per_sys, te, mass, p, v, eta, n_iter, 0, exact, NULL, NULL, NULL,
                       NULL, &ms);
    if (rc) break;
    if (ms < best) {
      best = ms;
      bw = shapes[k][0];
      bc = shapes[k][1];
    }
  }
  free(te); free(p); free(v);
  BT.wpc = bw;
  BT.cps = bc;
  if (out) {
    out[0] = bw;
    out[1] = bc;
    out[2] = best;
  }
  return rc;
}

/* ============================== fixed-step Hermite and its adjoint ===== */
/* Building blocks on device arrays ([n][3] doubles) for the differentiable
 * fixed-step integrator (amuse_gb300/adjoint.py drives them from a
 * torch.autograd.Function).  All calls are blocking. */
int g6k_fixed_records(const g6_jstate *js, int n, const double *x, const double *v,
                      const double *m, int prec, cudaStream_t st);
int g6k_fixed_predict(int n, double h, const double *x, const double *v, const double *a,
                      const double *j, double *xp, double *vp, cudaStream_t st);
int g6k_fixed_correct(int n, double h, double *x, double *v, double *a, double *j,
                      const double *a1, const double *j1, cudaStream_t st);
int g6k_fixed_adj_pre(int n, double h, double *lx, double *lv, double *la, double *lj,
                      double *la1, double *lj1, cudaStream_t st);
int g6k_fixed_adj_post(int n, double h, double *lx, double *lv, double *la, double *lj,
                       const double *gxp, const double *gvp, double *lm, const double *gm,
                       cudaStream_t st);
size_t g6k_vjp_scratch_bytes(int n);
int g6k_force_vjp(int n, double eps2, int prec, int hjerk, const double *x, const double *v,
                  const double *m, const double *la1, const double *lj1, double *gx, double *gv,
                  double *gm, void *scratch, cudaStream_t st);

static double *fx_a1, *fx_j1, *fx_xp, *fx_vp;
static void *fx_part;
static size_t fx_part_bytes;
static int fx_cap;
static int fx_form = G6_JERK_HERMITE;

static void fixed_free(void) {
  cudaFree(fx_a1); cudaFree(fx_j1); cudaFree(fx_xp); cudaFree(fx_vp); cudaFree(fx_part);
  fx_a1 = fx_j1 = fx_xp = fx_vp = NULL;
  fx_part = NULL;
  fx_cap = 0;
  fx_part_bytes = 0;
}

int g6x_set_fixed_jerk(int form) {
  if (form != G6_JERK_HERMITE && form != G6_JERK_SOFTENED) return G6_ERR_ARG;
  fx_form = form;
  return 0;
}

/* a1/j1 hold n bodies; the VJP scratch is sized for this n's launch shape
   (its split count depends on n, so a smaller n can need more). */
static int fixed_buffers(int n) {
  const size_t need = g6k_vjp_scratch_bytes(n);
  if (n <= fx_cap && fx_part && need <= fx_part_bytes) return 0;
  const int cap = n > fx_cap ? n : fx_cap;
  const size_t bytes = need > fx_part_bytes ? need : fx_part_bytes;
  cudaFree(fx_a1); cudaFree(fx_j1); cudaFree(fx_xp); cudaFree(fx_vp); cudaFree(fx_part);
  fx_a1 = fx_j1 = fx_xp = fx_vp = NULL;
  fx_part = NULL;
  fx_cap = 0;
  fx_part_bytes = 0;
  if (cudaMalloc((void **)&fx_a1, sizeof(double) * 3 * (size_t)cap) != cudaSuccess ||
      cudaMalloc((void **)&fx_j1, sizeof(double) * 3 * (size_t)cap) != cudaSuccess ||
      cudaMalloc((void **)&fx_xp, sizeof(double) * 3 * (size_t)cap) != cudaSuccess ||
      cudaMalloc((void **)&fx_vp, sizeof(double) * 3 * (size_t)cap) != cudaSuccess ||
      cudaMalloc(&fx_part, bytes) != cudaSuccess) {
    seterr("cannot allocate fixed-step buffers for n=%d", n);
    return G6_ERR_NOMEM;
  }
  fx_cap = cap;
  fx_part_bytes = bytes;
  return 0;
}

/* The fixed-step calls enqueue on the library stream; the public entry
   points below synchronise once at their end and then check the force
   kernel's error word. */
static int fixed_force_async(int n, double eps2, const double *d_x, const double *d_v,
                             const double *d_m, double *d_a, double *d_j) {
  int rc = grow_j((n + G6_TILE - 1) / G6_TILE * G6_TILE);
  if (rc) return rc;
  rc = ensure_run_buffers(n);
  if (rc) return rc;
  rc = identity_list(n);
  if (rc) return rc;
  if (g6k_fixed_records(&G.js, n, d_x, d_v, d_m, G.prec, G.st)) return G6_ERR_CUDA;
  G.pred_valid = 0; /* the records no longer hold a prediction of the j-state */
  g6_force_args a;
  memset(&a, 0, sizeof(a));
  a.ni = n;
  a.nj = n;
  a.prec = G.prec;
  a.eps2 = eps2;
  a.ilist = G.d_ilist;
  a.acc = d_a;
  a.jerk = d_j;
  a.pot = G.d_rpot;
  a.hjerk = fx_form == G6_JERK_HERMITE;
  a.kappa = -1.0; /* the adjoint differentiates plain split arithmetic */
  return run_force(&a);
}

static int fixed_step_async(int n, double h, double eps2, double *d_x, double *d_v, double *d_a,
                            double *d_j, const double *d_m, double *d_xp, double *d_vp) {
  if (g6k_fixed_predict(n, h, d_x, d_v, d_a, d_j, d_xp, d_vp, G.st)) return G6_ERR_CUDA;
  int rc = fixed_force_async(n, eps2, d_xp, d_vp, d_m, fx_a1, fx_j1);
  if (rc) return rc;
  if (g6k_fixed_correct(n, h, d_x, d_v, d_a, d_j, fx_a1, fx_j1, G.st)) return G6_ERR_CUDA;
  return 0;
}

static int fixed_step_adjoint_async(int n, double h, double eps2, const double *d_xp,
                                    const double *d_vp, const double *d_m, double *d_lx,
                                    double *d_lv, double *d_la, double *d_lj, double *d_lm,
                                    double *d_work) {
  double *gxp = d_work, *gvp = d_work + 3 * (size_t)n, *gm = d_work + 6 * (size_t)n;
  if (g6k_fixed_adj_pre(n, h, d_lx, d_lv, d_la, d_lj, fx_a1, fx_j1, G.st)) return G6_ERR_CUDA;
  if (g6k_force_vjp(n, eps2, G.prec, fx_form == G6_JERK_HERMITE, d_xp, d_vp, d_m, fx_a1, fx_j1,
                    gxp, gvp, gm, fx_part, G.st))
    return G6_ERR_CUDA;
  if (g6k_fixed_adj_post(n, h, d_lx, d_lv, d_la, d_lj, gxp, gvp, d_lm, gm, G.st))
    return G6_ERR_CUDA;
  return 0;
}

static int fixed_finish(void) {
  CK(cudaStreamSynchronize(G.st));
  return read_err_word();
}

/* acc/jerk of all n bodies at (x, v) (split or FP64 per g6x_set_precision). */
int g6x_fixed_force(int n, double eps2, const double *d_x, const double *d_v, const double *d_m,
                    double *d_a, double *d_j) {
  int rc = check_open();
  if (rc) return rc;
  if (n <= 0) return G6_ERR_ARG;
  rc = fixed_force_async(n, eps2, d_x, d_v, d_m, d_a, d_j);
  return rc ? rc : fixed_finish();
}

/* One fixed step in place on (x, v, a, j); xp/vp receive the predicted
 * positions and velocities the force was evaluated at. */
int g6x_fixed_step(int n, double h, double eps2, double *d_x, double *d_v, double *d_a,
                   double *d_j, const double *d_m, double *d_xp, double *d_vp) {
  int rc = check_open();
  if (rc) return rc;
  if (n <= 0 || !d_xp || !d_vp) return G6_ERR_ARG;
  rc = fixed_buffers(n);
  if (rc) return rc;
  rc = fixed_step_async(n, h, eps2, d_x, d_v, d_a, d_j, d_m, d_xp, d_vp);
  return rc ? rc : fixed_finish();
}

/* nsteps fixed steps in place, one host synchronisation at the end.  If
 * d_xp_all/d_vp_all are not NULL they receive the predicted states of every
 * step ([nsteps][n][3] each); otherwise library scratch is used. */
int g6x_fixed_run(int n, double h, double eps2, int nsteps, double *d_x, double *d_v,
                  double *d_a, double *d_j, const double *d_m, double *d_xp_all,
                  double *d_vp_all) {
  int rc = check_open();
  if (rc) return rc;
  if (n <= 0 || nsteps < 0 || (!d_xp_all) != (!d_vp_all)) return G6_ERR_ARG;
  rc = fixed_buffers(n);
  if (rc) return rc;
  for (int s = 0; s < nsteps; s++) {
    const size_t o = d_xp_all ? 3 * (size_t)n * (size_t)s : 0;
    rc = fixed_step_async(n, h, eps2, d_x, d_v, d_a, d_j, d_m, d_xp_all ? d_xp_all + o : fx_xp,
                          d_vp_all ? d_vp_all + o : fx_vp);
    if (rc) return rc;
  }
  return fixed_finish();
}

/* Vector-Jacobian product of the force at (x, v): given cotangents la/lj of
 * (acc, jerk), gx/gv/gm receive the cotangents of x, v, m. */
int g6x_force_vjp(int n, double eps2, const double *d_x, const double *d_v, const double *d_m,
                  const double *d_la, const double *d_lj, double *d_gx, double *d_gv,
                  double *d_gm) {
  int rc = check_open();
  if (rc) return rc;
  if (n <= 0) return G6_ERR_ARG;
  rc = fixed_buffers(n);
  if (rc) return rc;
  if (g6k_force_vjp(n, eps2, G.prec, fx_form == G6_JERK_HERMITE, d_x, d_v, d_m, d_la, d_lj, d_gx,
                    d_gv, d_gm, fx_part, G.st))
    return G6_ERR_CUDA;
  return fixed_finish();
}

/* Adjoint of one fixed step (in place on lx, lv, la, lj; gm accumulates
 * into d_lm) at the predicted state (xp, vp) the forward step used. */
int g6x_fixed_step_adjoint(int n, double h, double eps2, const double *d_xp, const double *d_vp,
                           const double *d_m, double *d_lx, double *d_lv, double *d_la,
                           double *d_lj, double *d_lm, double *d_work /* [7n] */) {
  int rc = check_open();
  if (rc) return rc;
  if (n <= 0 || !d_work) return G6_ERR_ARG;
  rc = fixed_buffers(n);
  if (rc) return rc;
  rc = fixed_step_adjoint_async(n, h, eps2, d_xp, d_vp, d_m, d_lx, d_lv, d_la, d_lj, d_lm,
                                d_work);
  return rc ? rc : fixed_finish();
}

/* The adjoints of nsteps consecutive steps, last step first, at the
 * predicted states d_xp_all/d_vp_all ([nsteps][n][3], as g6x_fixed_run
 * wrote them); one host synchronisation at the end. */
int g6x_fixed_adjoint_run(int n, double h, double eps2, int nsteps, const double *d_xp_all,
                          const double *d_vp_all, const double *d_m, double *d_lx, double *d_lv,
                          double *d_la, double *d_lj, double *d_lm, double *d_work) {
  int rc = check_open();
  if (rc) return rc;
  if (n <= 0 || nsteps < 0 || !d_work || !d_xp_all || !d_vp_all) return G6_ERR_ARG;
  rc = fixed_buffers(n);
  if (rc) return rc;
  for (int s = nsteps - 1; s >= 0; s--) {
    const size_t o = 3 * (size_t)n * (size_t)s;
    rc = fixed_step_adjoint_async(n, h, eps2, d_xp_all + o, d_vp_all + o, d_m, d_lx, d_lv, d_la,
                                  d_lj, d_lm, d_work);
    if (rc) return rc;
  }
  return fixed_finish();
}
