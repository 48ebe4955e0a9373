/*
 * xpbd_oracle_c.c -- CPU oracle for the RDC-XPBD substep, TEST INFRASTRUCTURE ONLY.
 *
 * A plain-C (pthreads) restatement of the reference solver
 * (RaymondMcGuire/rdc-xpbd-taichi, xpbd_gpu/neohookean_solver.py and
 * xpbd_gpu/xpbd_base.py) in FP32, the reference's arithmetic type, for the
 * timed CPU baseline and as a second checker next to oracle/xpbd_oracle.py,
 * and (built with -DOC_DOUBLE) in FP64 as the float64 reference run of large
 * meshes.
 * Only the tests and bench.py's CPU legs load it.  Parity of this file is
 * checked against the NumPy oracle, which is pinned to the reference's own
 * code (tests/golden/).
 *
 * Threads split every tet and vertex loop into static ranges.  The Jacobi
 * scatter of the reference (ti.atomic_add, neohookean_solver.py:443-451) is
 * restated deterministically: each tet writes its four corner contributions,
 * then each vertex sums its corners in ascending (tet, corner) order, which is
 * the order of a sequential scatter.  The residual sum is accumulated in FP64
 * per thread and combined in thread order.
 */
#include <math.h>
#include <pthread.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

/* Arithmetic type: FP32 (the reference's) by default; -DOC_DOUBLE builds the
 * same restatement in FP64 (the float64 reference run).  The SDF table and the
 * solver constants stay FP32 in both builds. */
#ifdef OC_DOUBLE
typedef double real;
#define FABS fabs
#define SQRT sqrt
#define EXP exp
#define FMAX fmax
#define FMIN fmin
#define EPS 1e-12 /* xpbd_gpu/constants.py:3 */
#else
typedef float real;
#define FABS fabsf
#define SQRT sqrtf
#define EXP expf
#define FMAX fmaxf
#define FMIN fminf
#define EPS 1e-12f /* xpbd_gpu/constants.py:3 */
#endif

typedef struct {
  int kind; /* 0 plane, 1 sphere, 2 cube (sdf.py:60-124) */
  int fixed;
  float a[3], b[3], vel[3];
} oc_sdf;

typedef struct {
  float mu, lambda, gravity[3], damping, relax_h, relax_d, gamma;
  int cheb, warmup, block, iters, precise;
  double rho_min, rho_max, rho_beta;
} oc_params;

typedef struct {
  int V, T, n_sdf, nthreads;
  const oc_params* p;
  const oc_sdf* sdf;
  const int* tets;     /* [T][4] */
  const real* dm;     /* [T][9] inv_Dm row-major */
  const real* v0;     /* [T] */
  const real* inv_m;  /* [V] */
  const int* csr_off;  /* [V+1] vertex -> (tet*4+corner), ascending */
  const int* csr_slot; /* [4T] */
  real *x, *v, *xp, *yprev, *ycurr, *post; /* [V][3] */
  real* lam;          /* [T][2] */
  real* corner;       /* [4T][4] */
  double* part;        /* [nthreads][3] */
  real dt;
  int first;
} oc_state;

/* ---------------- a minimal static-range thread pool ---------------- */
typedef void (*oc_fn)(oc_state* s, int lo, int hi, int tid);
typedef struct {
  pthread_t th[256];
  int n;
  pthread_mutex_t mu;
  pthread_cond_t go, done;
  int gen, pending, quit;
  oc_fn fn;
  oc_state* s;
  int N;
} oc_pool;

typedef struct {
  oc_pool* pool;
  int tid;
} oc_worker;

static void* oc_worker_main(void* arg) {
  oc_worker* w = (oc_worker*)arg;
  oc_pool* P = w->pool;
  int seen = 0;
  for (;;) {
    pthread_mutex_lock(&P->mu);
    while (P->gen == seen && !P->quit) pthread_cond_wait(&P->go, &P->mu);
    if (P->quit) {
      pthread_mutex_unlock(&P->mu);
      return NULL;
    }
    seen = P->gen;
    oc_fn fn = P->fn;
    oc_state* s = P->s;
    int N = P->N;
    pthread_mutex_unlock(&P->mu);
    const int n = P->n + 1;
    const int lo = (int)((long long)N * w->tid / n), hi = (int)((long long)N * (w->tid + 1) / n);
    fn(s, lo, hi, w->tid);
    pthread_mutex_lock(&P->mu);
    if (--P->pending == 0) pthread_cond_signal(&P->done);
    pthread_mutex_unlock(&P->mu);
  }
}

static void oc_run_par(oc_pool* P, oc_fn fn, oc_state* s, int N) {
  if (P->n == 0) {
    fn(s, 0, N, 0);
    return;
  }
  pthread_mutex_lock(&P->mu);
  P->fn = fn;
  P->s = s;
  P->N = N;
  P->pending = P->n;
  P->gen++;
  pthread_cond_broadcast(&P->go);
  pthread_mutex_unlock(&P->mu);
  const int n = P->n + 1;
  fn(s, (int)((long long)N * P->n / n), N, P->n); /* the caller takes the last range */
  pthread_mutex_lock(&P->mu);
  while (P->pending) pthread_cond_wait(&P->done, &P->mu);
  pthread_mutex_unlock(&P->mu);
}

/* ---------------- SDFs (sdf.py) ---------------- */
static real sdf_dist(const oc_sdf* s, const real* p) {
  if (s->kind == 0) return (p[0] - s->a[0]) * s->b[0] + (p[1] - s->a[1]) * s->b[1] + (p[2] - s->a[2]) * s->b[2];
  if (s->kind == 1) {
    real d0 = p[0] - s->a[0], d1 = p[1] - s->a[1], d2 = p[2] - s->a[2];
    return SQRT(d0 * d0 + d1 * d1 + d2 * d2) - s->b[0];
  }
  real d0 = FABS(p[0] - s->a[0]) - s->b[0], d1 = FABS(p[1] - s->a[1]) - s->b[1], d2 = FABS(p[2] - s->a[2]) - s->b[2];
  real m0 = FMAX(d0, 0.f), m1 = FMAX(d1, 0.f), m2 = FMAX(d2, 0.f);
  return SQRT(m0 * m0 + m1 * m1 + m2 * m2) + FMIN(FMAX(d0, FMAX(d1, d2)), 0.f);
}

static void sdf_normal(const oc_sdf* s, const real* p, real* n) {
  if (s->kind == 0) {
    n[0] = s->b[0]; n[1] = s->b[1]; n[2] = s->b[2];
    return;
  }
  real d[3] = {p[0] - s->a[0], p[1] - s->a[1], p[2] - s->a[2]};
  if (s->kind == 1) { /* normalized(EPS): v / (|v| + EPS) */
    real inv = 1.f / (SQRT(d[0] * d[0] + d[1] * d[1] + d[2] * d[2]) + EPS);
    n[0] = d[0] * inv; n[1] = d[1] * inv; n[2] = d[2] * inv;
    return;
  }
  int ax = 0;
  if (FABS(d[1]) > FABS(d[0])) ax = 1;
  if (FABS(d[2]) > FABS(d[ax])) ax = 2;
  n[0] = n[1] = n[2] = 0.f;
  n[ax] = d[ax] > 0.f ? 1.f : -1.f;
}

/* apply_external_forces (xpbd_base.py:139-146) + solve_sdf_collision (:162-178) */
static void phase_begin(oc_state* s, int lo, int hi, int tid) {
  const oc_params* p = s->p;
  for (int i = lo; i < hi; ++i) {
    real* v = s->v + 3 * i;
    real* x = s->x + 3 * i;
    real* q = s->xp + 3 * i;
    const real w = s->inv_m[i];
    if (w > 0.f)
      for (int k = 0; k < 3; ++k) v[k] += p->gravity[k] * s->dt;
    for (int k = 0; k < 3; ++k) q[k] = x[k] + v[k] * s->dt;
    if (w > 0.f)
      for (int k = 0; k < s->n_sdf; ++k) {
        const oc_sdf* sd = s->sdf + k;
        const real phi = sdf_dist(sd, q);
        if (phi < 0.f) {
          real n[3];
          sdf_normal(sd, q, n);
          const real dotnv = n[0] * (sd->vel[0] - v[0]) + n[1] * (sd->vel[1] - v[1]) + n[2] * (sd->vel[2] - v[2]);
          if (dotnv > 0.f || sd->fixed) {
            const real pen = -sdf_dist(sd, q);
            if (pen > 0.f)
              for (int c = 0; c < 3; ++c) q[c] += n[c] * pen;
          }
        }
      }
    for (int k = 0; k < 3; ++k) {
      s->yprev[3 * i + k] = q[k];
    }
  }
}

static void tet_F(const oc_state* s, const real* pos, int t, real F[9]) {
  const int* id = s->tets + 4 * t;
  const real* P0 = pos + 3 * id[0];
  real e[3][3];
  for (int c = 0; c < 3; ++c) {
    const real* Pc = pos + 3 * id[c + 1];
    for (int r = 0; r < 3; ++r) e[r][c] = Pc[r] - P0[r];
  }
  const real* dm = s->dm + 9 * t;
  for (int r = 0; r < 3; ++r)
    for (int c = 0; c < 3; ++c) F[3 * r + c] = e[r][0] * dm[c] + e[r][1] * dm[3 + c] + e[r][2] * dm[6 + c];
}

static void invariants(int precise, const real F[9], real* CD, real* CH) {
  if (precise) {
    real g00 = F[0] - 1.f, g11 = F[4] - 1.f, g22 = F[8] - 1.f, g01 = F[1], g02 = F[2], g10 = F[3], g12 = F[5],
          g20 = F[6], g21 = F[7];
    real tr = g00 + g11 + g22;
    real gg = g00 * g00 + g01 * g01 + g02 * g02 + g10 * g10 + g11 * g11 + g12 * g12 + g20 * g20 + g21 * g21 + g22 * g22;
    *CD = 2.f * tr + gg;
    real m2 = (g00 * g11 - g01 * g10) + (g00 * g22 - g02 * g20) + (g11 * g22 - g12 * g21);
    real dg = g00 * (g11 * g22 - g21 * g12) - g10 * (g01 * g22 - g21 * g02) + g20 * (g01 * g12 - g11 * g02);
    *CH = tr + (m2 + dg);
  } else {
    real q = 0.f;
    for (int k = 0; k < 9; ++k) q += F[k] * F[k];
    *CD = q - 3.f;
    *CH = F[0] * (F[4] * F[8] - F[7] * F[5]) - F[3] * (F[1] * F[8] - F[7] * F[2]) + F[6] * (F[1] * F[5] - F[4] * F[2]) - 1.f;
  }
}

static void corner_grads(const real gF[9], const real* dm, real g[4][3]) {
  for (int c = 0; c < 3; ++c)
    for (int r = 0; r < 3; ++r) g[c + 1][r] = gF[3 * r] * dm[3 * c] + gF[3 * r + 1] * dm[3 * c + 1] + gF[3 * r + 2] * dm[3 * c + 2];
  for (int r = 0; r < 3; ++r) g[0][r] = -(g[1][r] + g[2][r] + g[3][r]);
}

static real dot3(const real* a, const real* b) { return a[0] * b[0] + a[1] * b[1] + a[2] * b[2]; }

/* solve_neohookean_block (neohookean_solver.py:358-451) / split pair (:144-254) */
static void phase_project(oc_state* s, int lo, int hi, int tid) {
  const oc_params* p = s->p;
  const real dt2 = s->dt * s->dt;
  for (int t = lo; t < hi; ++t) {
    const int* id = s->tets + 4 * t;
    const real* dm = s->dm + 9 * t;
    real w[4];
    for (int c = 0; c < 4; ++c) w[c] = s->inv_m[id[c]];
    real F[9], CD, CH;
    tet_F(s, s->xp, t, F);
    invariants(p->precise, F, &CD, &CH);
    real gF[9], H[9], gD[4][3], gH[4][3];
    for (int k = 0; k < 9; ++k) gF[k] = F[k] * 2.f;
    corner_grads(gF, dm, gD);
    /* columns of F: F_j = (F[j], F[3+j], F[6+j]); cof = [F1 x F2, F2 x F0, F0 x F1] */
    const real c0[3] = {F[0], F[3], F[6]}, c1[3] = {F[1], F[4], F[7]}, c2[3] = {F[2], F[5], F[8]};
    const real x0[3] = {c1[1] * c2[2] - c1[2] * c2[1], c1[2] * c2[0] - c1[0] * c2[2], c1[0] * c2[1] - c1[1] * c2[0]};
    const real x1[3] = {c2[1] * c0[2] - c2[2] * c0[1], c2[2] * c0[0] - c2[0] * c0[2], c2[0] * c0[1] - c2[1] * c0[0]};
    const real x2[3] = {c0[1] * c1[2] - c0[2] * c1[1], c0[2] * c1[0] - c0[0] * c1[2], c0[0] * c1[1] - c0[1] * c1[0]};
    for (int r = 0; r < 3; ++r) {
      H[3 * r] = x0[r];
      H[3 * r + 1] = x1[r];
      H[3 * r + 2] = x2[r];
    }
    corner_grads(H, dm, gH);
    real* L = s->lam + 2 * t;
    if (s->first) L[0] = L[1] = 0.f; /* neohookean_solver.py:458-459 */
    const real aD = 1.f / (p->mu * s->v0[t]) / dt2, aH = 1.f / (p->lambda * s->v0[t]) / dt2;
    real dp[4][3], cnt;
    if (p->block) {
      real A11 = 0.f, A22 = 0.f, A12 = 0.f;
      for (int c = 0; c < 4; ++c) {
        A11 += w[c] * dot3(gD[c], gD[c]);
        A22 += w[c] * dot3(gH[c], gH[c]);
        A12 += w[c] * dot3(gD[c], gH[c]);
      }
      A11 += aD;
      A22 += aH;
      real b1 = -(CD + aD * L[0]), b2 = -(CH + aH * L[1]);
      /* solve2x2_pivot_lu (:331-356) */
      real M00 = A11, M01 = A12, M10 = A12, M11 = A22, r0 = b1, r1 = b2, dD = 0.f, dH = 0.f;
      int ok = 1;
      if (FABS(M00) < FABS(M10)) {
        real tmp = M00; M00 = M10; M10 = tmp;
        tmp = M01; M01 = M11; M11 = tmp;
        tmp = r0; r0 = r1; r1 = tmp;
      }
      if (FABS(M00) < EPS) ok = 0;
      if (ok) {
        real m = M10 / M00, M11_ = M11 - m * M01, r1_ = r1 - m * r0;
        if (FABS(M11_) < EPS) ok = 0;
        else {
          dH = r1_ / M11_;
          dD = (r0 - M01 * dH) / M00;
        }
      }
      if (!ok) { /* :425-432 */
        dD = FABS(A11) > EPS ? b1 / A11 : 0.f;
        dH = FABS(A22) > EPS ? b2 / A22 : 0.f;
      }
      L[0] += dD;
      L[1] += dH;
      for (int c = 0; c < 4; ++c)
        for (int r = 0; r < 3; ++r) dp[c][r] = w[c] * (gD[c][r] * dD + gH[c][r] * dH);
      cnt = 1.f;
    } else {
      real wsH = 0.f, wsD = 0.f;
      for (int c = 0; c < 4; ++c) {
        wsH += w[c] * dot3(gH[c], gH[c]);
        wsD += w[c] * dot3(gD[c], gD[c]);
      }
      real dlH = 0.f, dlD = 0.f, cH = 0.f, cD = 0.f;
      if (wsH > EPS) {
        dlH = -(CH + aH * L[1]) / (wsH + aH) * p->relax_h;
        cH = 1.f;
      }
      if (wsD > EPS) {
        dlD = -(CD + aD * L[0]) / (wsD + aD) * p->relax_d;
        cD = 1.f;
      }
      L[0] += dlD;
      L[1] += dlH;
      for (int c = 0; c < 4; ++c)
        for (int r = 0; r < 3; ++r) dp[c][r] = dlH * w[c] * gH[c][r] + dlD * w[c] * gD[c][r];
      cnt = cH + cD;
    }
    for (int c = 0; c < 4; ++c) {
      real* o = s->corner + 4 * (4 * t + c);
      o[0] = dp[c][0];
      o[1] = dp[c][1];
      o[2] = dp[c][2];
      o[3] = cnt;
    }
  }
}

/* post_solve (:115-119): sequential-order sum of the corner contributions */
static void phase_gather(oc_state* s, int lo, int hi, int tid) {
  for (int i = lo; i < hi; ++i) {
    real d[4] = {0.f, 0.f, 0.f, 0.f};
    for (int k = s->csr_off[i]; k < s->csr_off[i + 1]; ++k) {
      const real* c = s->corner + 4 * s->csr_slot[k];
      d[0] += c[0]; d[1] += c[1]; d[2] += c[2]; d[3] += c[3];
    }
    for (int r = 0; r < 3; ++r) {
      s->ycurr[3 * i + r] = s->xp[3 * i + r];
      s->post[3 * i + r] = s->xp[3 * i + r] + (d[3] > 0.f ? d[r] / d[3] : 0.f);
    }
  }
}

/* compute_xpbd_residual (:298-329), FP64 per-thread sums */
static void phase_residual(oc_state* s, int lo, int hi, int tid) {
  const oc_params* p = s->p;
  const real dt2 = s->dt * s->dt;
  double sum = 0.0;
  for (int t = lo; t < hi; ++t) {
    real F[9], CD, CH;
    tet_F(s, s->post, t, F);
    invariants(p->precise, F, &CD, &CH);
    const real aD = 1.f / (p->mu * s->v0[t]) / dt2, aH = 1.f / (p->lambda * s->v0[t]) / dt2;
    const real rD = CD + aD * s->lam[2 * t], rH = CH + aH * s->lam[2 * t + 1];
    sum += (double)SQRT(rD * rD + rH * rH);
  }
  s->part[3 * tid] = sum;
}

static real g_omega; /* set per iteration before phase_cheb */

/* _chebyshev_update (:131-137) + rotation (:139-142); without Chebyshev the post positions */
static void phase_cheb(oc_state* s, int lo, int hi, int tid) {
  const real g = s->p->gamma, om = g_omega;
  for (int i = lo; i < hi; ++i)
    for (int r = 0; r < 3; ++r) {
      const int k = 3 * i + r;
      if (s->p->cheb) {
        const real xn = g * (s->post[k] - s->ycurr[k]) + s->ycurr[k];
        s->xp[k] = s->yprev[k] + om * (xn - s->yprev[k]);
        s->yprev[k] = s->ycurr[k];
      } else {
        s->xp[k] = s->post[k];
      }
    }
}

/* advance (xpbd_base.py:148-160) */
static void phase_end(oc_state* s, int lo, int hi, int tid) {
  const real e = EXP(-s->dt * s->p->damping);
  for (int i = lo; i < hi; ++i) {
    if (s->inv_m[i] <= 0.f) continue;
    for (int r = 0; r < 3; ++r) {
      const int k = 3 * i + r;
      s->v[k] = (s->xp[k] - s->x[k]) / s->dt * e;
      s->x[k] = s->xp[k];
    }
  }
}

/*
 * Run `n_frames` frames of `frame_dt` in chunks of `dt` (neohookean_solver.py:562-587).
 * x, v: [V][3] in/out.  rho_hat: in/out (persists across calls).  r_hat_hist:
 * optional, receives r_hat of every iteration of every frame.  Returns 0.
 */
int oc_run(int V, int T, real* x, real* v, const int* tets, const real* inv_Dm, const real* V0,
           const real* inv_m, const oc_sdf* sdfs, int n_sdf, const oc_params* p, double frame_dt, double dt,
           int substeps, int n_frames, double* rho_hat, int nthreads, double* r_hat_hist) {
  if (V <= 0 || T <= 0 || nthreads < 1) return 1;
  if (nthreads > 256) nthreads = 256;
  oc_state s;
  memset(&s, 0, sizeof(s));
  s.V = V; s.T = T; s.n_sdf = n_sdf; s.p = p; s.sdf = sdfs; s.tets = tets; s.dm = inv_Dm; s.v0 = V0;
  s.inv_m = inv_m; s.x = x; s.v = v; s.nthreads = nthreads;
  int* off = (int*)calloc((size_t)V + 1, sizeof(int));
  int* slot = (int*)malloc(sizeof(int) * 4 * (size_t)T);
  for (long long k = 0; k < 4ll * T; ++k) off[tets[k] + 1]++;
  for (int i = 0; i < V; ++i) off[i + 1] += off[i];
  int* fill = (int*)malloc(sizeof(int) * (size_t)V);
  memcpy(fill, off, sizeof(int) * (size_t)V);
  for (long long k = 0; k < 4ll * T; ++k) slot[fill[tets[k]]++] = (int)k;
  free(fill);
  s.csr_off = off; s.csr_slot = slot;
  s.xp = (real*)malloc(sizeof(real) * 3 * V);
  s.yprev = (real*)malloc(sizeof(real) * 3 * V);
  s.ycurr = (real*)malloc(sizeof(real) * 3 * V);
  s.post = (real*)malloc(sizeof(real) * 3 * V);
  s.lam = (real*)calloc(2 * (size_t)T, sizeof(real));
  s.corner = (real*)malloc(sizeof(real) * 16 * (size_t)T);
  s.part = (double*)calloc(3 * 256, sizeof(double));
  oc_pool pool;
  memset(&pool, 0, sizeof(pool));
  pool.n = nthreads - 1;
  pthread_mutex_init(&pool.mu, NULL);
  pthread_cond_init(&pool.go, NULL);
  pthread_cond_init(&pool.done, NULL);
  oc_worker workers[256];
  for (int k = 0; k < pool.n; ++k) {
    workers[k].pool = &pool;
    workers[k].tid = k;
    pthread_create(&pool.th[k], NULL, oc_worker_main, &workers[k]);
  }
  long long rec = 0;
  for (int f = 0; f < n_frames; ++f) {
    double left = frame_dt;
    while (left > 0.0) {
      const double dt0 = dt < left ? dt : left;
      left -= dt0;
      s.dt = (real)(dt0 / substeps);
      for (int sub = 0; sub < substeps; ++sub) {
        oc_run_par(&pool, phase_begin, &s, V);
        double prev = -1.0, omega = 1.0;
        for (int it = 0; it < p->iters; ++it) {
          s.first = it == 0;
          oc_run_par(&pool, phase_project, &s, T);
          oc_run_par(&pool, phase_gather, &s, V);
          if (p->cheb) {
            memset(s.part, 0, sizeof(double) * 3 * 256);
            oc_run_par(&pool, phase_residual, &s, T);
            double S = 0.0;
            for (int k = 0; k < nthreads; ++k) S += s.part[3 * k];
            const double r_hat = S / T;
            if (r_hat_hist) r_hat_hist[rec++] = r_hat;
            if (prev > 1e-12) { /* neohookean_solver.py:498-504 */
              double ri = r_hat / (prev + 1e-12);
              ri = ri < p->rho_min ? p->rho_min : (ri > p->rho_max ? p->rho_max : ri);
              *rho_hat = (1.0 - p->rho_beta) * *rho_hat + p->rho_beta * ri;
            }
            prev = r_hat;
            const double r2 = *rho_hat * *rho_hat; /* :538-546 */
            if (it < p->warmup) omega = 1.0;
            else if (it == p->warmup) omega = 2.0 / (2.0 - r2);
            else omega = 4.0 / (4.0 - r2 * omega);
          }
          g_omega = (real)omega;
          oc_run_par(&pool, phase_cheb, &s, V);
        }
        oc_run_par(&pool, phase_end, &s, V);
      }
    }
  }
  pthread_mutex_lock(&pool.mu);
  pool.quit = 1;
  pthread_cond_broadcast(&pool.go);
  pthread_mutex_unlock(&pool.mu);
  for (int k = 0; k < pool.n; ++k) pthread_join(pool.th[k], NULL);
  free(off); free(slot); free(s.xp); free(s.yprev); free(s.ycurr); free(s.post); free(s.lam); free(s.corner);
  free(s.part);
  return 0;
}
