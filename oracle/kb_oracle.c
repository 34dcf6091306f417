/*
 * kb_oracle.c -- TEST INFRASTRUCTURE ONLY.  FP64 CPU restatement of KitBase.jl's
 * discrete-velocity-method time step (1D2F1V, 2D2F2V), used as the parity
 * checker of the CUDA library and as the timed CPU baseline.  Nothing in the
 * product links or calls this file.
 *
 * PARITY UNPINNED: KitBase.jl is Julia, Julia is absent from every machine this
 * project builds on, and the reference test suite holds no golden vectors for
 * this path (test/test_flux.jl, test/test_step.jl and test/test_solver_*.jl
 * assert nothing).  The restatement is pinned by invariants and known answers
 * instead (Gaussian moments vs quadrature, Maxwellian fixed points, telescoping
 * conservation, Sod at small Kn vs the exact Riemann solution) -- see tests/.
 *
 * Structure follows the reference stage by stage and keeps its storage: every
 * cell owns w, prim, sw, h, b, sh, sb; every face owns fw, fh, fb
 * (ControlVolume2F / Interface2F, src/Struct/struct_ctr.jl:94-117,
 * src/Struct/struct_face.jl:56-65).  Sums use Julia's pairwise order
 * (Base.mapreduce_impl: block 1024, split at the midpoint) with a sequential
 * base case.  File:line citations are into the reference tree.
 */
#include "../include/kitgpu.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define MAXV 4

typedef struct kbo {
  kb_config_t c;
  int D, NW;             /* dimension, length of w / prim */
  int nxt, nyt, ncell;   /* cells incl. ghosts */
  int nvel;              /* nu * nv */
  double dx, dy;         /* uniform cell sizes */
  double *u, *v, *wt;    /* velocity tables */
  double *w, *prim, *sw; /* [cell][4], sw [cell][2][4] */
  double *h, *b;         /* [cell][nvel] */
  double *sh, *sb;       /* [cell][2][nvel] */
  int nfx, nfy;
  double *fwx, *fhx, *fbx; /* x faces [(nx+1)*ny] */
  double *fwy, *fhy, *fby; /* y faces [nx*(ny+1)] */
  unsigned char *fdonex, *fdoney; /* face computed in the last evolve */
  double *wall[4];               /* [nface_side][4] global frame */
  double *tmp;                   /* per-thread scratch [nthreads][8*nvel] */
  int ntmp;
} kbo_t;

/* ------------------------------------------------------------------ sums */

/* Julia Base pairwise reduction: src base/reduce.jl mapreduce_impl, blksize 1024. */
static double psum(const double* a, long n) {
  if (n <= 1024) {
    double s = 0.0;
    for (long i = 0; i < n; ++i) s += a[i];
    return s;
  }
  long mid = (n - 1) >> 1; /* first half holds mid+1 elements */
  return psum(a, mid + 1) + psum(a + mid + 1, n - mid - 1);
}

/* ------------------------------------------------------------- physics */

/* heaviside, src/Math/math_general.jl:13 */
static inline double heaviside(double x) { return x >= 0 ? 1.0 : 0.0; }

/* sign as used by fortsign, src/Math/math_general.jl:20 */
static inline double jsign(double y) { return y > 0 ? 1.0 : (y < 0 ? -1.0 : y); }

/* vanleer, src/Reconstruction/recon_limiter.jl:17-19 */
static inline double vanleer(double sL, double sR) {
  return (jsign(sL) + jsign(sR)) * fabs(sL) * fabs(sR) / (fabs(sL) + fabs(sR) + 1.e-7);
}

/* conserve_prim!, src/Theory/theory_macro.jl:185-206 */
static void conserve_prim(const double* W, int nw, double g, double* prim) {
  if (nw == 3) {
    prim[0] = W[0];
    prim[1] = W[1] / W[0];
    prim[2] = 0.5 * W[0] / (g - 1.0) / (W[2] - 0.5 * (W[1] * W[1]) / W[0]);
  } else {
    prim[0] = W[0];
    prim[1] = W[1] / W[0];
    prim[2] = W[2] / W[0];
    prim[3] = 0.5 * W[0] / (g - 1.0) / (W[3] - 0.5 * (W[1] * W[1] + W[2] * W[2]) / W[0]);
  }
}

/* prim_conserve!, src/Theory/theory_macro.jl:10-33 */
static void prim_conserve(const double* p, int nw, double g, double* W) {
  if (nw == 3) {
    W[0] = p[0];
    W[1] = p[0] * p[1];
    W[2] = 0.5 * p[0] / p[2] / (g - 1.0) + 0.5 * p[0] * (p[1] * p[1]);
  } else {
    W[0] = p[0];
    W[1] = p[0] * p[1];
    W[2] = p[0] * p[2];
    W[3] = 0.5 * p[0] / p[3] / (g - 1.0) + 0.5 * p[0] * (p[1] * p[1] + p[2] * p[2]);
  }
}

/* vhs_collision_time, src/Theory/theory_relaxation.jl:28,35-36 */
static inline double vhs_time(const double* prim, int nw, double mu, double om) {
  return mu * 2.0 * pow(prim[nw - 1], 1.0 - om) / prim[0];
}

/* gauss_moments(prim, inK), src/Theory/theory_moments.jl:10-86.  Mu, MuL, MuR,
 * Mv hold orders 0..6, Mxi orders 0..2. */
static void gauss_moments(const double* prim, int nw, double inK, double* Mu, double* Mv,
                          double* Mxi, double* MuL, double* MuR) {
  double l = prim[nw - 1], U = prim[1];
  MuL[0] = 0.5 * erfc(-sqrt(l) * U);
  MuL[1] = U * MuL[0] + 0.5 * exp(-l * (U * U)) / sqrt(M_PI * l);
  MuR[0] = 0.5 * erfc(sqrt(l) * U);
  MuR[1] = U * MuR[0] - 0.5 * exp(-l * (U * U)) / sqrt(M_PI * l);
  for (int i = 2; i <= 6; ++i) {
    MuL[i] = U * MuL[i - 1] + 0.5 * (i - 1) * MuL[i - 2] / l;
    MuR[i] = U * MuR[i - 1] + 0.5 * (i - 1) * MuR[i - 2] / l;
  }
  for (int i = 0; i <= 6; ++i) Mu[i] = MuL[i] + MuR[i];
  if (nw == 4) {
    double V = prim[2];
    Mv[0] = 1.0;
    Mv[1] = V;
    for (int i = 2; i <= 6; ++i) Mv[i] = V * Mv[i - 1] + 0.5 * (i - 1) * Mv[i - 2] / l;
  }
  Mxi[0] = 1.0;
  Mxi[1] = 0.5 * inK / l;
  Mxi[2] = (inK * inK + 2.0 * inK) / (4.0 * (l * l));
}

/* moments_conserve(Mu, Mxi, alpha, delta), src/Theory/theory_moments.jl:98-108 */
static void mc1(const double* Mu, const double* Mxi, int a, int d, double* uv) {
  uv[0] = Mu[a] * Mxi[d / 2];
  uv[1] = Mu[a + 1] * Mxi[d / 2];
  uv[2] = 0.5 * (Mu[a + 2] * Mxi[d / 2] + Mu[a] * Mxi[(d + 2) / 2]);
}

/* moments_conserve(Mu, Mv, Mxi, alpha, beta, delta), src/Theory/theory_moments.jl:113-145 */
static void mc2(const double* Mu, const double* Mv, const double* Mxi, int a, int bb, int d,
                double* uv) {
  uv[0] = Mu[a] * Mv[bb] * Mxi[d / 2];
  uv[1] = Mu[a + 1] * Mv[bb] * Mxi[d / 2];
  uv[2] = Mu[a] * Mv[bb + 1] * Mxi[d / 2];
  uv[3] = 0.5 * (Mu[a + 2] * Mv[bb] * Mxi[d / 2] + Mu[a] * Mv[bb + 2] * Mxi[d / 2] +
                 Mu[a] * Mv[bb] * Mxi[(d + 2) / 2]);
}

/* moments_conserve_slope, src/Theory/theory_moments.jl:335-369 */
static void mcs1(const double* a, const double* Mu, const double* Mxi, int al, double* out) {
  double t0[3], t1[3], t2[3], t3[3];
  mc1(Mu, Mxi, al, 0, t0);
  mc1(Mu, Mxi, al + 1, 0, t1);
  mc1(Mu, Mxi, al + 2, 0, t2);
  mc1(Mu, Mxi, al, 2, t3);
  for (int k = 0; k < 3; ++k)
    out[k] = a[0] * t0[k] + a[1] * t1[k] + 0.5 * a[2] * t2[k] + 0.5 * a[2] * t3[k];
}

static void mcs2(const double* a, const double* Mu, const double* Mv, const double* Mxi, int al,
                 int be, double* out) {
  double t0[4], t1[4], t2[4], t3[4], t4[4], t5[4];
  mc2(Mu, Mv, Mxi, al, be, 0, t0);
  mc2(Mu, Mv, Mxi, al + 1, be, 0, t1);
  mc2(Mu, Mv, Mxi, al, be + 1, 0, t2);
  mc2(Mu, Mv, Mxi, al + 2, be, 0, t3);
  mc2(Mu, Mv, Mxi, al, be + 2, 0, t4);
  mc2(Mu, Mv, Mxi, al, be, 2, t5);
  for (int k = 0; k < 4; ++k)
    out[k] = a[0] * t0[k] + a[1] * t1[k] + a[2] * t2[k] + 0.5 * a[3] * t3[k] +
             0.5 * a[3] * t4[k] + 0.5 * a[3] * t5[k];
}

/* pdf_slope(prim, sw, inK), src/Theory/theory_pdf.jl:11-49 */
static void pdf_slope(const double* p, const double* s, int nw, double inK, double* sl) {
  if (nw == 3) {
    sl[2] = 4.0 * (p[2] * p[2]) / (inK + 1.0) / p[0] *
            (2.0 * s[2] - 2.0 * p[1] * s[1] + s[0] * ((p[1] * p[1]) - 0.5 * (inK + 1.0) / p[2]));
    sl[1] = 2.0 * p[2] / p[0] * (s[1] - p[1] * s[0]) - p[1] * sl[2];
    sl[0] = s[0] / p[0] - p[1] * sl[1] - 0.5 * ((p[1] * p[1]) + 0.5 * (inK + 1.0) / p[2]) * sl[2];
  } else {
    sl[3] = 4.0 * (p[3] * p[3]) / (inK + 2.0) / p[0] *
            (2.0 * s[3] - 2.0 * p[1] * s[1] - 2.0 * p[2] * s[2] +
             s[0] * ((p[1] * p[1]) + (p[2] * p[2]) - 0.5 * (inK + 2.0) / p[3]));
    sl[2] = 2.0 * p[3] / p[0] * (s[2] - p[2] * s[0]) - p[2] * sl[3];
    sl[1] = 2.0 * p[3] / p[0] * (s[1] - p[1] * s[0]) - p[1] * sl[3];
    sl[0] = s[0] / p[0] - p[1] * sl[1] - p[2] * sl[2] -
            0.5 * ((p[1] * p[1]) + (p[2] * p[2]) + 0.5 * (inK + 2.0) / p[3]) * sl[3];
  }
}

/* local_frame / global_frame for w of length 4, src/Geometry/geo_general.jl:115-153 */
static void local_frame(const double* w, const double* n, double* L) {
  L[0] = w[0];
  L[1] = w[1] * n[0] + w[2] * n[1];
  L[2] = w[2] * n[0] - w[1] * n[1];
  L[3] = w[3];
}
static void global_frame(const double* w, const double* n, double* G) {
  G[0] = w[0];
  G[1] = w[1] * n[0] - w[2] * n[1];
  G[2] = w[1] * n[1] + w[2] * n[0];
  G[3] = w[3];
}

/* ------------------------------------------------------------ indexing */

static inline long cidx(const kbo_t* o, int i, int j) { /* 1-based physical i, j */
  return (long)(j - 1 + o->c.ngy) * o->nxt + (i - 1 + o->c.ngx);
}
static inline double* SW(const kbo_t* o, long c, int d) { return o->sw + (c * 2 + d) * 4; }
static inline double* SH(const kbo_t* o, long c, int d) {
  return o->sh + (c * 2 + d) * (long)o->nvel;
}
static inline double* SB(const kbo_t* o, long c, int d) {
  return o->sb + (c * 2 + d) * (long)o->nvel;
}
static inline double* Hc(const kbo_t* o, long c) { return o->h + c * (long)o->nvel; }
static inline double* Bc(const kbo_t* o, long c) { return o->b + c * (long)o->nvel; }

static double* scratch(kbo_t* o) {
  int t = 0;
#ifdef _OPENMP
  t = omp_get_thread_num();
#endif
  return o->tmp + (long)t * 16 * o->nvel;
}

/* ------------------------------------------------------------ lifecycle */

kbo_t* kbo_create(const kb_config_t* cfg, const double* u, const double* v, const double* wt) {
  kbo_t* o = (kbo_t*)calloc(1, sizeof(kbo_t));
  o->c = *cfg;
  o->D = cfg->dim;
  o->NW = cfg->dim + 2;
  o->nxt = cfg->nx + 2 * cfg->ngx;
  o->nyt = cfg->dim == 2 ? cfg->ny + 2 * cfg->ngy : 1;
  if (cfg->dim == 1) {
    o->c.ny = 1;
    o->c.ngy = 0;
  }
  o->ncell = o->nxt * o->nyt;
  o->nvel = cfg->nu * (cfg->dim == 2 ? cfg->nv : 1);
  o->dx = (cfg->x1 - cfg->x0) / cfg->nx;
  o->dy = cfg->dim == 2 ? (cfg->y1 - cfg->y0) / cfg->ny : 0.0;
  long nv = o->nvel, nc = o->ncell;
  o->u = malloc(sizeof(double) * nv);
  o->v = calloc(nv, sizeof(double));
  o->wt = malloc(sizeof(double) * nv);
  memcpy(o->u, u, sizeof(double) * nv);
  if (v && cfg->dim == 2) memcpy(o->v, v, sizeof(double) * nv);
  memcpy(o->wt, wt, sizeof(double) * nv);
  o->w = calloc(nc * 4, sizeof(double));
  o->prim = calloc(nc * 4, sizeof(double));
  o->sw = calloc(nc * 8, sizeof(double));
  o->h = calloc(nc * nv, sizeof(double));
  o->b = calloc(nc * nv, sizeof(double));
  o->sh = calloc(nc * 2 * nv, sizeof(double));
  o->sb = calloc(nc * 2 * nv, sizeof(double));
  int nx = o->c.nx, ny = o->c.ny;
  o->nfx = (nx + 1) * ny;
  o->nfy = o->D == 2 ? nx * (ny + 1) : 0;
  o->fwx = calloc((long)o->nfx * 4, sizeof(double));
  o->fhx = calloc((long)o->nfx * nv, sizeof(double));
  o->fbx = calloc((long)o->nfx * nv, sizeof(double));
  o->fdonex = calloc(o->nfx, 1);
  if (o->nfy) {
    o->fwy = calloc((long)o->nfy * 4, sizeof(double));
    o->fhy = calloc((long)o->nfy * nv, sizeof(double));
    o->fby = calloc((long)o->nfy * nv, sizeof(double));
    o->fdoney = calloc(o->nfy, 1);
  }
  for (int s = 0; s < 4; ++s) {
    int n = s < 2 ? ny : nx;
    o->wall[s] = calloc((long)n * 4, sizeof(double));
  }
  int nt = 1;
#ifdef _OPENMP
  nt = omp_get_max_threads();
#endif
  o->ntmp = nt;
  o->tmp = malloc(sizeof(double) * (long)nt * 16 * nv);
  return o;
}

void kbo_destroy(kbo_t* o) {
  if (!o) return;
  free(o->u); free(o->v); free(o->wt);
  free(o->w); free(o->prim); free(o->sw);
  free(o->h); free(o->b); free(o->sh); free(o->sb);
  free(o->fwx); free(o->fhx); free(o->fbx); free(o->fdonex);
  free(o->fwy); free(o->fhy); free(o->fby); free(o->fdoney);
  for (int s = 0; s < 4; ++s) free(o->wall[s]);
  free(o->tmp);
  free(o);
}

void kbo_set_threads(int n) {
#ifdef _OPENMP
  omp_set_num_threads(n);
#else
  (void)n;
#endif
}

int kbo_max_threads(void) {
#ifdef _OPENMP
  return omp_get_max_threads();
#else
  return 1;
#endif
}

int kbo_set_wall(kbo_t* o, int side, const double* prim) {
  int n = side < 2 ? o->c.ny : o->c.nx;
  for (int f = 0; f < n; ++f)
    for (int k = 0; k < o->NW; ++k) o->wall[side][f * 4 + k] = prim[f * o->NW + k];
  return 0;
}

int kbo_set_state(kbo_t* o, const double* w, const double* prim, const double* h,
                  const double* b) {
  for (long c = 0; c < o->ncell; ++c)
    for (int k = 0; k < o->NW; ++k) {
      o->w[c * 4 + k] = w[c * o->NW + k];
      o->prim[c * 4 + k] = prim[c * o->NW + k];
    }
  memcpy(o->h, h, sizeof(double) * o->ncell * (long)o->nvel);
  memcpy(o->b, b, sizeof(double) * o->ncell * (long)o->nvel);
  memset(o->sw, 0, sizeof(double) * o->ncell * 8);
  memset(o->sh, 0, sizeof(double) * o->ncell * 2 * (long)o->nvel);
  memset(o->sb, 0, sizeof(double) * o->ncell * 2 * (long)o->nvel);
  return 0;
}

int kbo_get_state(const kbo_t* o, double* w, double* prim, double* h, double* b) {
  for (long c = 0; c < o->ncell; ++c)
    for (int k = 0; k < o->NW; ++k) {
      if (w) w[c * o->NW + k] = o->w[c * 4 + k];
      if (prim) prim[c * o->NW + k] = o->prim[c * 4 + k];
    }
  if (h) memcpy(h, o->h, sizeof(double) * o->ncell * (long)o->nvel);
  if (b) memcpy(b, o->b, sizeof(double) * o->ncell * (long)o->nvel);
  return 0;
}

/* ----------------------------------------------------------- timestep */

/* timestep, src/Solver/solver_main.jl:240-288 (1D), :290-342 (2D).  The
 * reference reduces tmax with a racy max under @threads; here it is serial. */
double kbo_timestep(const kbo_t* o, double cfl, double sim_time, double max_time) {
  double tmax = 0.0;
  int nx = o->c.nx, ny = o->c.ny;
  for (int j = 1; j <= ny; ++j)
    for (int i = 1; i <= nx; ++i) {
      const double* p = o->prim + cidx(o, i, j) * 4;
      double sos = pow(0.5 * o->c.gamma / p[o->NW - 1], 0.5);
      if (o->D == 1) {
        double vmax = fmax(o->c.umax, fabs(p[1])) + sos;
        tmax = fmax(tmax, vmax / o->dx);
      } else {
        double umax = fmax(o->c.umax, fabs(p[1])) + sos;
        double vmax = fmax(o->c.vmax, fabs(p[2])) + sos;
        tmax = fmax(tmax, umax / o->dx + vmax / o->dy);
      }
    }
  double dt = cfl / tmax;
  return dt < (max_time - sim_time) ? dt : max_time - sim_time;
}

/* ------------------------------------------------------- reconstruction */

/* reconstruct3! along a line of three cells (src/Reconstruction/reconstruction.jl:136-151) */
static void recon3(double* s, const double* qL, const double* qN, const double* qR, long n,
                   double dL, double dR) {
  for (long k = 0; k < n; ++k) {
    double sL = (qN[k] - qL[k]) / dL;
    double sR = (qR[k] - qN[k]) / dR;
    s[k] = vanleer(sL, sR);
  }
}
/* reconstruct2!, src/Reconstruction/reconstruction.jl:48-50 */
static void recon2(double* s, const double* qL, const double* qR, long n, double d) {
  for (long k = 0; k < n; ++k) s[k] = (qR[k] - qL[k]) / d;
}

/* reconstruct! 1D2F (src/Solver/solver_reconstruction.jl:101-153) and
 * 2D2F (:475-620). */
/* per-thread scratch sized for the current OpenMP team (threads may change
 * between calls through kbo_set_threads) */
static void ensure_scratch(kbo_t* o) {
  int nt = 1;
#ifdef _OPENMP
  nt = omp_get_max_threads();
#endif
  if (nt > o->ntmp) {
    free(o->tmp);
    o->tmp = malloc(sizeof(double) * (long)nt * 16 * o->nvel);
    o->ntmp = nt;
  }
}

void kbo_reconstruct(kbo_t* o) {
  if (o->c.interp_order == 1) return;
  int nx = o->c.nx, ny = o->c.ny, NW = o->NW;
  long nv = o->nvel;
  if (o->D == 1) {
    int i0 = o->c.ngx > 0 ? 1 : 2, i1 = o->c.ngx > 0 ? nx : nx - 1;
    double d = 0.5 * (o->dx + o->dx);
#pragma omp parallel for schedule(static)
    for (int i = i0; i <= i1; ++i) {
      long c = cidx(o, i, 1), cl = cidx(o, i - 1, 1), cr = cidx(o, i + 1, 1);
      recon3(SW(o, c, 0), o->w + cl * 4, o->w + c * 4, o->w + cr * 4, NW, d, d);
      recon3(SH(o, c, 0), Hc(o, cl), Hc(o, c), Hc(o, cr), nv, d, d);
      recon3(SB(o, c, 0), Bc(o, cl), Bc(o, c), Bc(o, cr), nv, d, d);
    }
    return;
  }
  double dX = 0.5 * (o->dx + o->dx), dY = 0.5 * (o->dy + o->dy);
#pragma omp parallel for schedule(static)
  for (int j = 1; j <= ny; ++j)
    for (int i = 1; i <= nx; ++i) {
      long c = cidx(o, i, j);
      /* x direction: one-sided at i = 1, nx; three-cell inside */
      if (i == 1 || i == nx) {
        long a = cidx(o, i == 1 ? 1 : nx - 1, j), bq = cidx(o, i == 1 ? 2 : nx, j);
        recon2(SW(o, c, 0), o->w + a * 4, o->w + bq * 4, NW, dX);
        recon2(SH(o, c, 0), Hc(o, a), Hc(o, bq), nv, dX);
        recon2(SB(o, c, 0), Bc(o, a), Bc(o, bq), nv, dX);
      } else {
        long cl = cidx(o, i - 1, j), cr = cidx(o, i + 1, j);
        recon3(SW(o, c, 0), o->w + cl * 4, o->w + c * 4, o->w + cr * 4, NW, dX, dX);
        recon3(SH(o, c, 0), Hc(o, cl), Hc(o, c), Hc(o, cr), nv, dX, dX);
        recon3(SB(o, c, 0), Bc(o, cl), Bc(o, c), Bc(o, cr), nv, dX, dX);
      }
      /* y direction */
      if (j == 1 || j == ny) {
        long a = cidx(o, i, j == 1 ? 1 : ny - 1), bq = cidx(o, i, j == 1 ? 2 : ny);
        recon2(SW(o, c, 1), o->w + a * 4, o->w + bq * 4, NW, dY);
        recon2(SH(o, c, 1), Hc(o, a), Hc(o, bq), nv, dY);
        recon2(SB(o, c, 1), Bc(o, a), Bc(o, bq), nv, dY);
      } else {
        long cd = cidx(o, i, j - 1), cu = cidx(o, i, j + 1);
        recon3(SW(o, c, 1), o->w + cd * 4, o->w + c * 4, o->w + cu * 4, NW, dY, dY);
        recon3(SH(o, c, 1), Hc(o, cd), Hc(o, c), Hc(o, cu), nv, dY, dY);
        recon3(SB(o, c, 1), Bc(o, cd), Bc(o, c), Bc(o, cu), nv, dY, dY);
      }
    }
}

/* --------------------------------------------------------------- fluxes */

typedef struct {
  const double *hL, *bL, *hR, *bR, *shL, *sbL, *shR, *sbR; /* face states (reconstructed) */
  const double *un, *ut;                                 /* face-frame velocities */
  double wL[4], wR[4];                                   /* face-frame w states */
  double dxL, dxR, len;
} face_in_t;

/* flux_kfvs! 2F1V (src/Flux/flux_kfvs.jl:303-337) and 2F2V (:654-700) */
static void flux_kfvs(kbo_t* o, const face_in_t* F, double dt, double* fw, double* fh,
                      double* fb) {
  long nv = o->nvel;
  double* t = scratch(o);
  for (long k = 0; k < nv; ++k) {
    double d = heaviside(F->un[k]);
    double h = F->hL[k] * d + F->hR[k] * (1.0 - d);
    double b = F->bL[k] * d + F->bR[k] * (1.0 - d);
    double sh = F->shL[k] * d + F->shR[k] * (1.0 - d);
    double sb = F->sbL[k] * d + F->sbR[k] * (1.0 - d);
    double u = F->un[k];
    fh[k] = dt * u * h - 0.5 * (dt * dt) * (u * u) * sh;
    fb[k] = dt * u * b - 0.5 * (dt * dt) * (u * u) * sb;
    if (o->D == 2) {
      fh[k] *= F->len;
      fb[k] *= F->len;
    }
  }
  /* flux_conserve!, src/Theory/theory_moments.jl:376-416 */
  const double* w = o->wt;
  for (long k = 0; k < nv; ++k) t[k] = w[k] * fh[k];
  fw[0] = psum(t, nv);
  for (long k = 0; k < nv; ++k) t[k] = F->un[k] * w[k] * fh[k];
  fw[1] = psum(t, nv);
  if (o->D == 1) {
    for (long k = 0; k < nv; ++k) t[k] = (F->un[k] * F->un[k]) * w[k] * fh[k];
    double a = psum(t, nv);
    for (long k = 0; k < nv; ++k) t[k] = w[k] * fb[k];
    fw[2] = 0.5 * (a + psum(t, nv));
  } else {
    for (long k = 0; k < nv; ++k) t[k] = F->ut[k] * w[k] * fh[k];
    fw[2] = psum(t, nv);
    for (long k = 0; k < nv; ++k)
      t[k] = ((F->un[k] * F->un[k]) + (F->ut[k] * F->ut[k])) * w[k] * fh[k];
    double a = psum(t, nv);
    for (long k = 0; k < nv; ++k) t[k] = w[k] * fb[k];
    fw[3] = 0.5 * (a + psum(t, nv));
  }
}

/* interface equilibrium shared by KCU and UGKS (flux_kcu.jl:480-495, flux_ugks.jl:47-56) */
static void interface_prim(const kbo_t* o, const double* wL, const double* wR, double* primL,
                           double* primR, double* w, double* prim) {
  int NW = o->NW;
  double K = o->c.K, g = o->c.gamma;
  double Mu[7], Mv[7], Mxi[3], MuL[7], MuR[7], M1[4], M2[4];
  conserve_prim(wL, NW, g, primL);
  conserve_prim(wR, NW, g, primR);
  gauss_moments(primL, NW, K, Mu, Mv, Mxi, MuL, MuR);
  if (NW == 3) mc1(MuL, Mxi, 0, 0, M1); else mc2(MuL, Mv, Mxi, 0, 0, 0, M1);
  gauss_moments(primR, NW, K, Mu, Mv, Mxi, MuL, MuR);
  if (NW == 3) mc1(MuR, Mxi, 0, 0, M2); else mc2(MuR, Mv, Mxi, 0, 0, 0, M2);
  for (int k = 0; k < NW; ++k) w[k] = primL[0] * M1[k] + primR[0] * M2[k];
  conserve_prim(w, NW, g, prim);
}

/* flux_kcu! 1D2F1V (src/Flux/flux_kcu.jl:463-530) and 2D2F2V (:898-970) */
static void flux_kcu(kbo_t* o, const face_in_t* F, double dt, double* fw, double* fh,
                     double* fb) {
  int NW = o->NW;
  long nv = o->nvel;
  double K = o->c.K;
  double primL[4] = {0}, primR[4] = {0}, w[4] = {0}, prim[4] = {0};
  interface_prim(o, F->wL, F->wR, primL, primR, w, prim);
  double tau = vhs_time(prim, NW, o->c.mu_ref, o->c.omega);
  tau += fabs(primL[0] / primL[NW - 1] - primR[0] / primR[NW - 1]) /
         (primL[0] / primL[NW - 1] + primR[0] / primR[NW - 1]) * dt * 2.0;
  double Mt[2];
  Mt[1] = tau * (1.0 - exp(-dt / tau));
  Mt[0] = dt - Mt[1];
  double Mu[7], Mv[7], Mxi[3], MuL[7], MuR[7], Muv[4];
  gauss_moments(prim, NW, K, Mu, Mv, Mxi, MuL, MuR);
  double len = o->D == 2 ? F->len : 1.0;
  if (NW == 3) {
    mc1(Mu, Mxi, 1, 0, Muv);
    for (int k = 0; k < 3; ++k) fw[k] = Mt[0] * prim[0] * Muv[k];
  } else {
    mc2(Mu, Mv, Mxi, 1, 0, 0, Muv);
    for (int k = 0; k < 4; ++k) fw[k] = Mt[0] * prim[0] * Muv[k] * len;
  }
  double* H = scratch(o) + 2 * nv;
  double* B = H + nv;
  double* hh = B + nv;
  double* bb = hh + nv;
  double* t = scratch(o);
  for (long k = 0; k < nv; ++k) {
    double u = F->un[k];
    if (NW == 3)
      H[k] = prim[0] * sqrt(prim[2] / M_PI) * exp(-prim[2] * ((u - prim[1]) * (u - prim[1])));
    else {
      double vv = F->ut[k];
      H[k] = prim[0] * (prim[3] / M_PI) *
             exp(-prim[3] * ((u - prim[1]) * (u - prim[1]) + (vv - prim[2]) * (vv - prim[2])));
    }
    B[k] = H[k] * K / (2.0 * prim[NW - 1]);
    double d = heaviside(u);
    hh[k] = F->hL[k] * d + F->hR[k] * (1.0 - d);
    bb[k] = F->bL[k] * d + F->bR[k] * (1.0 - d);
  }
  const double* om = o->wt;
  const double *u = F->un, *v = F->ut;
  if (NW == 3) {
    for (long k = 0; k < nv; ++k) t[k] = om[k] * u[k] * hh[k];
    fw[0] += Mt[1] * psum(t, nv);
    for (long k = 0; k < nv; ++k) t[k] = om[k] * (u[k] * u[k]) * hh[k];
    fw[1] += Mt[1] * psum(t, nv);
    for (long k = 0; k < nv; ++k) t[k] = om[k] * (u[k] * u[k] * u[k]) * hh[k];
    double a = psum(t, nv);
    for (long k = 0; k < nv; ++k) t[k] = om[k] * u[k] * bb[k];
    fw[2] += Mt[1] * 0.5 * (a + psum(t, nv));
    for (long k = 0; k < nv; ++k) {
      fh[k] = Mt[0] * u[k] * H[k] + Mt[1] * u[k] * hh[k];
      fb[k] = Mt[0] * u[k] * B[k] + Mt[1] * u[k] * bb[k];
    }
  } else {
    for (long k = 0; k < nv; ++k) t[k] = om[k] * u[k] * hh[k];
    fw[0] += Mt[1] * psum(t, nv) * len;
    for (long k = 0; k < nv; ++k) t[k] = om[k] * (u[k] * u[k]) * hh[k];
    fw[1] += Mt[1] * psum(t, nv) * len;
    for (long k = 0; k < nv; ++k) t[k] = om[k] * v[k] * u[k] * hh[k];
    fw[2] += Mt[1] * psum(t, nv) * len;
    for (long k = 0; k < nv; ++k) t[k] = om[k] * u[k] * ((u[k] * u[k]) + (v[k] * v[k])) * hh[k];
    double a = psum(t, nv);
    for (long k = 0; k < nv; ++k) t[k] = om[k] * u[k] * bb[k];
    fw[3] += Mt[1] * 0.5 * (a + psum(t, nv)) * len;
    for (long k = 0; k < nv; ++k) {
      fh[k] = (Mt[0] * u[k] * H[k] + Mt[1] * u[k] * hh[k]) * len;
      fb[k] = (Mt[0] * u[k] * B[k] + Mt[1] * u[k] * bb[k]) * len;
    }
  }
}

/* flux_ugks! 1D2F1V (src/Flux/flux_ugks.jl:8-114) and 2D2F2V (:121-253).  The
 * reference has no Interface2F-level wrapper for UGKS; the face states follow
 * the reconstructed-state convention of the KCU wrappers (flux_kcu.jl:46-102,
 * :149-191) and the 3F UGKS call of solver_evolution.jl:278-314: w and h are
 * the face-reconstructed states, dxL/dxR are the half cell widths. */
static void flux_ugks(kbo_t* o, const face_in_t* F, double dt, double* fw, double* fh,
                      double* fb) {
  int NW = o->NW;
  long nv = o->nvel;
  double K = o->c.K;
  double primL[4] = {0}, primR[4] = {0}, w[4] = {0}, prim[4] = {0};
  interface_prim(o, F->wL, F->wR, primL, primR, w, prim);
  double dL[4] = {0}, dR[4] = {0}, aL[4] = {0}, aR[4] = {0}, aT[4] = {0};
  for (int k = 0; k < NW; ++k) {
    dL[k] = (w[k] - F->wL[k]) / F->dxL;
    dR[k] = (F->wR[k] - w[k]) / F->dxR;
  }
  pdf_slope(prim, dL, NW, K, aL);
  pdf_slope(prim, dR, NW, K, aR);
  double Mu[7], Mv[7], Mxi[3], MuL[7], MuR[7];
  gauss_moments(prim, NW, K, Mu, Mv, Mxi, MuL, MuR);
  double MauL[4], MauR[4], MauT[4], Muv[4], tmp[4];
  if (NW == 3) {
    mcs1(aL, MuL, Mxi, 1, MauL);
    mcs1(aR, MuR, Mxi, 1, MauR);
  } else {
    mcs2(aL, MuL, Mv, Mxi, 1, 0, MauL);
    mcs2(aR, MuR, Mv, Mxi, 1, 0, MauR);
  }
  for (int k = 0; k < NW; ++k) tmp[k] = -prim[0] * (MauL[k] + MauR[k]);
  pdf_slope(prim, tmp, NW, K, aT);

  double tau = vhs_time(prim, NW, o->c.mu_ref, o->c.omega);
  double Mt[5];
  Mt[3] = tau * (1.0 - exp(-dt / tau));
  Mt[4] = -tau * dt * exp(-dt / tau) + tau * Mt[3];
  Mt[0] = dt - Mt[3];
  Mt[1] = -tau * Mt[0] + Mt[4];
  Mt[2] = (dt * dt) / 2.0 - tau * Mt[0];

  if (NW == 3) {
    mc1(Mu, Mxi, 1, 0, Muv);
    mcs1(aL, MuL, Mxi, 2, MauL);
    mcs1(aR, MuR, Mxi, 2, MauR);
    mcs1(aT, Mu, Mxi, 1, MauT);
  } else {
    mc2(Mu, Mv, Mxi, 1, 0, 0, Muv);
    mcs2(aL, MuL, Mv, Mxi, 2, 0, MauL);
    mcs2(aR, MuR, Mv, Mxi, 2, 0, MauR);
    mcs2(aT, Mu, Mv, Mxi, 1, 0, MauT);
  }
  for (int k = 0; k < NW; ++k)
    fw[k] = Mt[0] * prim[0] * Muv[k] + Mt[1] * prim[0] * (MauL[k] + MauR[k]) +
            Mt[2] * prim[0] * MauT[k];

  double* t = scratch(o);
  double* H = t + nv;
  double* B = H + nv;
  double* hh = B + nv;
  double* bb = hh + nv;
  double* sh = bb + nv;
  double* sb = sh + nv;
  const double *u = F->un, *v = F->ut, *om = o->wt;
  for (long k = 0; k < nv; ++k) {
    double uu = u[k];
    if (NW == 3)
      H[k] = prim[0] * sqrt(prim[2] / M_PI) * exp(-prim[2] * ((uu - prim[1]) * (uu - prim[1])));
    else {
      double vv = v[k];
      H[k] = prim[0] * (prim[3] / M_PI) *
             exp(-prim[3] * ((uu - prim[1]) * (uu - prim[1]) + (vv - prim[2]) * (vv - prim[2])));
    }
    B[k] = H[k] * K / (2.0 * prim[NW - 1]);
    double d = heaviside(uu);
    hh[k] = F->hL[k] * d + F->hR[k] * (1.0 - d);
    bb[k] = F->bL[k] * d + F->bR[k] * (1.0 - d);
    sh[k] = F->shL[k] * d + F->shR[k] * (1.0 - d);
    sb[k] = F->sbL[k] * d + F->sbR[k] * (1.0 - d);
  }
  double a, c2;
  if (NW == 3) {
    for (long k = 0; k < nv; ++k) t[k] = om[k] * u[k] * hh[k];
    a = psum(t, nv);
    for (long k = 0; k < nv; ++k) t[k] = om[k] * (u[k] * u[k]) * sh[k];
    fw[0] += Mt[3] * a - Mt[4] * psum(t, nv);
    for (long k = 0; k < nv; ++k) t[k] = om[k] * (u[k] * u[k]) * hh[k];
    a = psum(t, nv);
    for (long k = 0; k < nv; ++k) t[k] = om[k] * (u[k] * u[k] * u[k]) * sh[k];
    fw[1] += Mt[3] * a - Mt[4] * psum(t, nv);
    for (long k = 0; k < nv; ++k) t[k] = om[k] * (u[k] * u[k] * u[k]) * hh[k];
    a = psum(t, nv);
    for (long k = 0; k < nv; ++k) t[k] = om[k] * u[k] * bb[k];
    a = a + psum(t, nv);
    for (long k = 0; k < nv; ++k) t[k] = om[k] * (u[k] * u[k] * u[k] * u[k]) * sh[k];
    c2 = psum(t, nv);
    for (long k = 0; k < nv; ++k) t[k] = om[k] * (u[k] * u[k]) * sb[k];
    c2 = c2 + psum(t, nv);
    fw[2] += Mt[3] * 0.5 * a - Mt[4] * 0.5 * c2;
    for (long k = 0; k < nv; ++k) {
      double uu = u[k], d = heaviside(uu), Hk = H[k], Bk = B[k], u2 = uu * uu;
      fh[k] = Mt[0] * uu * Hk +
              Mt[1] * u2 * (aL[0] * Hk + aL[1] * uu * Hk + 0.5 * aL[2] * (u2 * Hk + Bk)) * d +
              Mt[1] * u2 * (aR[0] * Hk + aR[1] * uu * Hk + 0.5 * aR[2] * (u2 * Hk + Bk)) * (1.0 - d) +
              Mt[2] * uu * (aT[0] * Hk + aT[1] * uu * Hk + 0.5 * aT[2] * (u2 * Hk + Bk)) +
              Mt[3] * uu * hh[k] - Mt[4] * u2 * sh[k];
      fb[k] = Mt[0] * uu * Bk +
              Mt[1] * u2 * (aL[0] * Bk + aL[1] * uu * Bk + 0.5 * aL[2] * (u2 * Bk + Mxi[2] * Hk)) * d +
              Mt[1] * u2 * (aR[0] * Bk + aR[1] * uu * Bk + 0.5 * aR[2] * (u2 * Bk + Mxi[2] * Hk)) * (1.0 - d) +
              Mt[2] * uu * (aT[0] * Bk + aT[1] * uu * Bk + 0.5 * aT[2] * (u2 * Bk + Mxi[2] * Hk)) +
              Mt[3] * uu * bb[k] - Mt[4] * u2 * sb[k];
    }
  } else {
    for (long k = 0; k < nv; ++k) t[k] = om[k] * u[k] * hh[k];
    a = psum(t, nv);
    for (long k = 0; k < nv; ++k) t[k] = om[k] * (u[k] * u[k]) * sh[k];
    fw[0] += Mt[3] * a - Mt[4] * psum(t, nv);
    for (long k = 0; k < nv; ++k) t[k] = om[k] * (u[k] * u[k]) * hh[k];
    a = psum(t, nv);
    for (long k = 0; k < nv; ++k) t[k] = om[k] * (u[k] * u[k] * u[k]) * sh[k];
    fw[1] += Mt[3] * a - Mt[4] * psum(t, nv);
    for (long k = 0; k < nv; ++k) t[k] = om[k] * v[k] * u[k] * hh[k];
    a = psum(t, nv);
    for (long k = 0; k < nv; ++k) t[k] = om[k] * v[k] * (u[k] * u[k]) * sh[k];
    fw[2] += Mt[3] * a - Mt[4] * psum(t, nv);
    for (long k = 0; k < nv; ++k) t[k] = om[k] * u[k] * ((u[k] * u[k]) + (v[k] * v[k])) * hh[k];
    a = psum(t, nv);
    for (long k = 0; k < nv; ++k) t[k] = om[k] * u[k] * bb[k];
    a = a + psum(t, nv);
    for (long k = 0; k < nv; ++k)
      t[k] = om[k] * (u[k] * u[k]) * ((u[k] * u[k]) + (v[k] * v[k])) * sh[k];
    c2 = psum(t, nv);
    for (long k = 0; k < nv; ++k) t[k] = om[k] * (u[k] * u[k]) * sb[k];
    c2 = c2 + psum(t, nv);
    fw[3] += Mt[3] * 0.5 * a - Mt[4] * 0.5 * c2;
    for (long k = 0; k < nv; ++k) {
      double uu = u[k], vv = v[k], d = heaviside(uu), Hk = H[k], Bk = B[k], u2 = uu * uu;
      double c2k = u2 + vv * vv;
      fh[k] = Mt[0] * uu * Hk +
              Mt[1] * u2 *
                  (aL[0] * Hk + aL[1] * uu * Hk + aL[2] * vv * Hk + 0.5 * aL[3] * (c2k * Hk + Bk)) * d +
              Mt[1] * u2 *
                  (aR[0] * Hk + aR[1] * uu * Hk + aR[2] * vv * Hk + 0.5 * aR[3] * (c2k * Hk + Bk)) *
                  (1.0 - d) +
              Mt[2] * uu *
                  (aT[0] * Hk + aT[1] * uu * Hk + aT[2] * vv * Hk + 0.5 * aT[3] * (c2k * Hk + Bk)) +
              Mt[3] * uu * hh[k] - Mt[4] * u2 * sh[k];
      fb[k] = Mt[0] * uu * Bk +
              Mt[1] * u2 *
                  (aL[0] * Bk + aL[1] * uu * Bk + aL[2] * vv * Bk +
                   0.5 * aL[3] * (c2k * Bk + Mxi[2] * Hk)) * d +
              Mt[1] * u2 *
                  (aR[0] * Bk + aR[1] * uu * Bk + aR[2] * vv * Bk +
                   0.5 * aR[3] * (c2k * Bk + Mxi[2] * Hk)) * (1.0 - d) +
              Mt[2] * uu *
                  (aT[0] * Bk + aT[1] * uu * Bk + aT[2] * vv * Bk +
                   0.5 * aT[3] * (c2k * Bk + Mxi[2] * Hk)) +
              Mt[3] * uu * bb[k] - Mt[4] * u2 * sb[k];
    }
    for (int k = 0; k < 4; ++k) fw[k] *= F->len;
    for (long k = 0; k < nv; ++k) {
      fh[k] *= F->len;
      fb[k] *= F->len;
    }
  }
}

/* flux_boundary_maxwell! 1D2F1V (src/Flux/flux_boundary.jl:39-61) and 2D2F2V
 * (:190-220).  un/ut are the face-frame velocities, bc the face-frame wall prim. */
/* ------------------------------------------------------------- 1F models
 * One distribution f per cell (ControlVolume1F / Interface1F,
 * src/Struct/struct_ctr.jl, struct_face.jl), held in the h arrays of this
 * oracle; b is unused.  Restated from the reference's 1F functions, not
 * derived from the 2F ones above. */

/* flux_kfvs! 1F1V (src/Flux/flux_kfvs.jl:238-262) and 1F2V (:615-650), with
 * flux_conserve! 1f1v / 1f2v (src/Theory/theory_moments.jl:387-391, :401-406) */
static void flux_kfvs_1f(kbo_t* o, const face_in_t* F, double dt, double* fw, double* ff) {
  long nv = o->nvel;
  double* t = scratch(o);
  const double* om = o->wt;
  for (long k = 0; k < nv; ++k) {
    double d = heaviside(F->un[k]);
    double f = F->hL[k] * d + F->hR[k] * (1.0 - d);
    double sf = F->shL[k] * d + F->shR[k] * (1.0 - d);
    double u = F->un[k];
    ff[k] = dt * u * f - 0.5 * (dt * dt) * (u * u) * sf;
    if (o->D == 2) ff[k] *= F->len;
  }
  for (long k = 0; k < nv; ++k) t[k] = om[k] * ff[k];
  fw[0] = psum(t, nv);
  for (long k = 0; k < nv; ++k) t[k] = F->un[k] * om[k] * ff[k];
  fw[1] = psum(t, nv);
  if (o->D == 1) {
    for (long k = 0; k < nv; ++k) t[k] = (F->un[k] * F->un[k]) * om[k] * ff[k];
    fw[2] = 0.5 * psum(t, nv);
  } else {
    for (long k = 0; k < nv; ++k) t[k] = F->ut[k] * om[k] * ff[k];
    fw[2] = psum(t, nv);
    for (long k = 0; k < nv; ++k)
      t[k] = ((F->un[k] * F->un[k]) + (F->ut[k] * F->ut[k])) * om[k] * ff[k];
    fw[3] = 0.5 * psum(t, nv);
  }
}

/* flux_kcu! 1D1F1V (src/Flux/flux_kcu.jl:241-303) and 2D1F2V (:828-894):
 * interface equilibrium from the half-range moments of both sides, M0 part
 * of fw from moments_conserve (with the internal degrees of freedom inK),
 * f0 part from the upwind f, ff = Mt1 u g + Mt2 u f (x len in 2D). */
static void flux_kcu_1f(kbo_t* o, const face_in_t* F, double dt, double* fw, double* ff) {
  int NW = o->NW;
  long nv = o->nvel;
  double K = o->c.K;
  double primL[4] = {0}, primR[4] = {0}, w[4] = {0}, prim[4] = {0};
  interface_prim(o, F->wL, F->wR, primL, primR, w, prim);
  double tau = vhs_time(prim, NW, o->c.mu_ref, o->c.omega);
  tau += fabs(primL[0] / primL[NW - 1] - primR[0] / primR[NW - 1]) /
         (primL[0] / primL[NW - 1] + primR[0] / primR[NW - 1]) * dt * 2.0;
  double Mt[2];
  Mt[1] = tau * (1.0 - exp(-dt / tau)); /* f0 */
  Mt[0] = dt - Mt[1];                   /* M0 */
  double Mu[7], Mv[7], Mxi[3], MuL[7], MuR[7], Muv[4];
  gauss_moments(prim, NW, K, Mu, Mv, Mxi, MuL, MuR);
  double len = o->D == 2 ? F->len : 1.0;
  if (NW == 3) {
    mc1(Mu, Mxi, 1, 0, Muv);
    for (int k = 0; k < 3; ++k) fw[k] = Mt[0] * prim[0] * Muv[k];
  } else {
    mc2(Mu, Mv, Mxi, 1, 0, 0, Muv);
    for (int k = 0; k < 4; ++k) fw[k] = Mt[0] * prim[0] * Muv[k] * len;
  }
  double* g = scratch(o) + 2 * nv;
  double* f = g + nv;
  double* t = scratch(o);
  const double *u = F->un, *v = F->ut, *om = o->wt;
  for (long k = 0; k < nv; ++k) {
    if (NW == 3)
      g[k] = prim[0] * sqrt(prim[2] / M_PI) * exp(-prim[2] * ((u[k] - prim[1]) * (u[k] - prim[1])));
    else
      g[k] = prim[0] * (prim[3] / M_PI) *
             exp(-prim[3] * ((u[k] - prim[1]) * (u[k] - prim[1]) + (v[k] - prim[2]) * (v[k] - prim[2])));
    double d = heaviside(u[k]);
    f[k] = F->hL[k] * d + F->hR[k] * (1.0 - d);
  }
  for (long k = 0; k < nv; ++k) t[k] = om[k] * u[k] * f[k];
  fw[0] += Mt[1] * psum(t, nv) * len;
  for (long k = 0; k < nv; ++k) t[k] = om[k] * (u[k] * u[k]) * f[k];
  fw[1] += Mt[1] * psum(t, nv) * len;
  if (NW == 3) {
    for (long k = 0; k < nv; ++k) t[k] = om[k] * (u[k] * u[k] * u[k]) * f[k];
    fw[2] += Mt[1] * 0.5 * psum(t, nv);
  } else {
    for (long k = 0; k < nv; ++k) t[k] = om[k] * v[k] * u[k] * f[k];
    fw[2] += Mt[1] * psum(t, nv) * len;
    for (long k = 0; k < nv; ++k) t[k] = om[k] * u[k] * ((u[k] * u[k]) + (v[k] * v[k])) * f[k];
    fw[3] += Mt[1] * 0.5 * psum(t, nv) * len;
  }
  for (long k = 0; k < nv; ++k) ff[k] = (Mt[0] * u[k] * g[k] + Mt[1] * u[k] * f[k]) * len;
}

/* flux_boundary_maxwell! 2D1F2V (src/Flux/flux_boundary.jl:158-186), face frame. */
static void flux_maxwell_1f(kbo_t* o, const double* bc, const double* fc, const double* un,
                            const double* ut, double dt, double len, int rot, double* fw,
                            double* ff) {
  long nv = o->nvel;
  double* t = scratch(o);
  double* fW = t + nv;
  const double* om = o->wt;
  for (long k = 0; k < nv; ++k) t[k] = om[k] * un[k] * fc[k] * (1.0 - heaviside(un[k] * rot));
  double SF = psum(t, nv);
  double lw = bc[3];
  for (long k = 0; k < nv; ++k)
    t[k] = om[k] * un[k] *
           exp(-lw * ((un[k] - bc[1]) * (un[k] - bc[1]) + (ut[k] - bc[2]) * (ut[k] - bc[2]))) *
           heaviside(un[k] * rot);
  double SG = (lw / M_PI) * psum(t, nv);
  double prim[4] = {-SF / SG, bc[1], bc[2], bc[3]};
  for (long k = 0; k < nv; ++k) {
    double H = prim[0] * (prim[3] / M_PI) *
               exp(-prim[3] * ((un[k] - prim[1]) * (un[k] - prim[1]) + (ut[k] - prim[2]) * (ut[k] - prim[2])));
    double d = heaviside(un[k] * rot);
    fW[k] = H * d + fc[k] * (1.0 - d);
  }
  /* discrete_moments(f, u, w, n) = sum(w .* u.^n .* f) (theory_moments.jl:432-437) */
  for (long k = 0; k < nv; ++k) t[k] = om[k] * un[k] * fW[k];
  fw[0] = psum(t, nv) * len * dt;
  for (long k = 0; k < nv; ++k) t[k] = om[k] * (un[k] * un[k]) * fW[k];
  fw[1] = psum(t, nv) * len * dt;
  for (long k = 0; k < nv; ++k) t[k] = om[k] * ut[k] * (fW[k] * un[k]);
  fw[2] = psum(t, nv) * len * dt;
  for (long k = 0; k < nv; ++k) t[k] = om[k] * un[k] * (fW[k] * ((un[k] * un[k]) + (ut[k] * ut[k])));
  fw[3] = 0.5 * psum(t, nv) * len * dt;
  for (long k = 0; k < nv; ++k) ff[k] = un[k] * fW[k] * len * dt;
}

static void flux_maxwell(kbo_t* o, const double* bc, const double* hc, const double* bcell,
                         const double* un, const double* ut, double dt, double len, int rot,
                         double* fw, double* fh, double* fb) {
  long nv = o->nvel;
  int NW = o->NW;
  double K = o->c.K;
  double* t = scratch(o);
  double* hW = t + nv;
  double* bW = hW + nv;
  const double* om = o->wt;
  for (long k = 0; k < nv; ++k) t[k] = om[k] * un[k] * hc[k] * (1.0 - heaviside(un[k] * rot));
  double SF = psum(t, nv);
  double lw = bc[NW - 1];
  for (long k = 0; k < nv; ++k) {
    double d = heaviside(un[k] * rot);
    double e = NW == 3 ? exp(-lw * ((un[k] - bc[1]) * (un[k] - bc[1])))
                       : exp(-lw * ((un[k] - bc[1]) * (un[k] - bc[1]) +
                                    (ut[k] - bc[2]) * (ut[k] - bc[2])));
    t[k] = om[k] * un[k] * e * d;
  }
  double SG = (NW == 3 ? pow(lw / M_PI, 0.5) : (lw / M_PI)) * psum(t, nv);
  double prim[4] = {0, 0, 0, 0};
  prim[0] = -SF / SG;
  for (int k = 1; k < NW; ++k) prim[k] = bc[k];
  for (long k = 0; k < nv; ++k) {
    double H;
    if (NW == 3)
      H = prim[0] * sqrt(prim[2] / M_PI) * exp(-prim[2] * ((un[k] - prim[1]) * (un[k] - prim[1])));
    else
      H = prim[0] * (prim[3] / M_PI) *
          exp(-prim[3] * ((un[k] - prim[1]) * (un[k] - prim[1]) +
                          (ut[k] - prim[2]) * (ut[k] - prim[2])));
    double B = H * K / (2.0 * prim[NW - 1]);
    double d = heaviside(un[k] * rot);
    hW[k] = H * d + hc[k] * (1.0 - d);
    bW[k] = B * d + bcell[k] * (1.0 - d);
  }
  double s = NW == 3 ? dt : len * dt;
  for (long k = 0; k < nv; ++k) t[k] = om[k] * un[k] * hW[k];
  fw[0] = psum(t, nv) * s;
  for (long k = 0; k < nv; ++k) t[k] = om[k] * (un[k] * un[k]) * hW[k];
  fw[1] = psum(t, nv) * s;
  if (NW == 3) {
    for (long k = 0; k < nv; ++k) t[k] = om[k] * un[k] * (hW[k] * (un[k] * un[k]));
    double a = psum(t, nv);
    for (long k = 0; k < nv; ++k) t[k] = om[k] * un[k] * bW[k];
    fw[2] = (0.5 * a + 0.5 * psum(t, nv)) * s;
  } else {
    for (long k = 0; k < nv; ++k) t[k] = om[k] * ut[k] * (hW[k] * un[k]);
    fw[2] = psum(t, nv) * s;
    for (long k = 0; k < nv; ++k)
      t[k] = om[k] * un[k] * (hW[k] * ((un[k] * un[k]) + (ut[k] * ut[k])));
    double a = psum(t, nv);
    for (long k = 0; k < nv; ++k) t[k] = om[k] * un[k] * bW[k];
    fw[3] = (0.5 * a + 0.5 * psum(t, nv)) * s;
  }
  for (long k = 0; k < nv; ++k) {
    fh[k] = un[k] * hW[k] * s;
    fb[k] = un[k] * bW[k] * s;
  }
}

/* face-normal geometry of the uniform Cartesian mesh.  Face lengths are the
 * vertex distances of PSpace2D (src/Geometry/geo_struct.jl:101-107): the
 * distance between y - dy/2 and y + dy/2 of the left cell row. */
static double xface_len(const kbo_t* o, int j) {
  double y = o->c.y0 + (j - 0.5) * o->dy;
  return fabs((y + 0.5 * o->dy) - (y - 0.5 * o->dy));
}
static double yface_len(const kbo_t* o, int i) {
  double x = o->c.x0 + (i - 0.5) * o->dx;
  return fabs((x + 0.5 * o->dx) - (x - 0.5 * o->dx));
}

/* One interior face: left cell cl, right cell cr, direction d (0 = x, 1 = y). */
static void interior_face(kbo_t* o, long cl, long cr, int d, double len, double dt, double* fw,
                          double* fh, double* fb) {
  long nv = o->nvel;
  int NW = o->NW;
  double* buf = scratch(o) + 8 * nv; /* hL, bL, hR, bR, un, ut */
  double *hL = buf, *bL = hL + nv, *hR = bL + nv, *bR = hR + nv, *un = bR + nv, *ut = un + nv;
  double dxL = 0.5 * (d == 0 ? o->dx : o->dy), dxR = dxL;
  const double *shL = SH(o, cl, d), *sbL = SB(o, cl, d), *shR = SH(o, cr, d), *sbR = SB(o, cr, d);
  const double *h0 = Hc(o, cl), *b0 = Bc(o, cl), *h1 = Hc(o, cr), *b1 = Bc(o, cr);
  double n[2] = {d == 0 ? 1.0 : 0.0, d == 0 ? 0.0 : 1.0};
  for (long k = 0; k < nv; ++k) {
    if (o->c.flux == KB_FLUX_KFVS) {
      hL[k] = h0[k] + shL[k] * dxL;
      bL[k] = b0[k] + sbL[k] * dxL;
      hR[k] = h1[k] - shR[k] * dxR;
      bR[k] = b1[k] - sbR[k] * dxR;
    } else {
      hL[k] = h0[k] + dxL * shL[k];
      bL[k] = b0[k] + dxL * sbL[k];
      hR[k] = h1[k] - dxR * shR[k];
      bR[k] = b1[k] - dxR * sbR[k];
    }
    if (NW == 3) {
      un[k] = o->u[k];
      ut[k] = 0.0;
    } else {
      un[k] = o->u[k] * n[0] + o->v[k] * n[1];
      ut[k] = o->v[k] * n[0] - o->u[k] * n[1];
    }
  }
  face_in_t F;
  F.hL = hL; F.bL = bL; F.hR = hR; F.bR = bR;
  F.shL = shL; F.sbL = sbL; F.shR = shR; F.sbR = sbR;
  F.un = un; F.ut = ut;
  F.dxL = dxL; F.dxR = dxR; F.len = len;
  if (o->c.flux != KB_FLUX_KFVS) {
    const double *wl = o->w + cl * 4, *wr = o->w + cr * 4;
    const double *swl = SW(o, cl, d), *swr = SW(o, cr, d);
    double a[4], c[4];
    for (int k = 0; k < NW; ++k) {
      a[k] = NW == 3 ? wl[k] + swl[k] * dxL : wl[k] + dxL * swl[k];
      c[k] = NW == 3 ? wr[k] - swr[k] * dxR : wr[k] - dxR * swr[k];
    }
    if (NW == 4) {
      local_frame(a, n, F.wL);
      local_frame(c, n, F.wR);
    } else {
      memcpy(F.wL, a, sizeof(a));
      memcpy(F.wR, c, sizeof(c));
    }
  }
  double fwl[4] = {0, 0, 0, 0};
  if (o->c.nf == 1) { /* 1F: ff in fh, no fb */
    if (o->c.flux == KB_FLUX_KFVS) flux_kfvs_1f(o, &F, dt, fwl, fh);
    else flux_kcu_1f(o, &F, dt, fwl, fh);
    memset(fb, 0, sizeof(double) * nv);
  } else if (o->c.flux == KB_FLUX_KFVS) flux_kfvs(o, &F, dt, fwl, fh, fb);
  else if (o->c.flux == KB_FLUX_KCU) flux_kcu(o, &F, dt, fwl, fh, fb);
  else flux_ugks(o, &F, dt, fwl, fh, fb);
  if (NW == 4) global_frame(fwl, n, fw);
  else memcpy(fw, fwl, sizeof(double) * 3);
}

/* evolve! 1D2F (src/Solver/solver_evolution.jl:64-89) + evolve_boundary!
 * (src/Solver/evolve_boundary.jl:4-47); 2D2F (:608-679) + (:52-178). */
void kbo_evolve(kbo_t* o, double dt) {
  ensure_scratch(o);
  int nx = o->c.nx, ny = o->c.ny;
  long nv = o->nvel;
  int i0 = o->c.ngx > 0 ? 1 : 2, i1 = o->c.ngx > 0 ? nx + 1 : nx;
  memset(o->fdonex, 0, o->nfx);
  if (o->D == 1) {
#pragma omp parallel for schedule(dynamic, 4)
    for (int i = i0; i <= i1; ++i) {
      long f = i - 1;
      interior_face(o, cidx(o, i - 1, 1), cidx(o, i, 1), 0, 1.0, dt, o->fwx + f * 4,
                    o->fhx + f * nv, o->fbx + f * nv);
      o->fdonex[f] = 1;
    }
    for (int s = 0; s < 2; ++s) {
      if (o->c.bc[s] != KB_BC_MAXWELL) continue;
      int i = s == 0 ? 1 : nx;
      long f = s == 0 ? 0 : nx;
      long c = cidx(o, i, 1);
      flux_maxwell(o, o->wall[s], Hc(o, c), Bc(o, c), o->u, o->v, dt, 1.0, s == 0 ? 1 : -1,
                   o->fwx + f * 4, o->fhx + f * nv, o->fbx + f * nv);
      o->fdonex[f] = 1;
    }
    return;
  }
  int j0 = o->c.ngy > 0 ? 1 : 2, j1 = o->c.ngy > 0 ? ny + 1 : ny;
  memset(o->fdoney, 0, o->nfy);
#pragma omp parallel for schedule(dynamic, 1)
  for (int j = 1; j <= ny; ++j)
    for (int i = i0; i <= i1; ++i) {
      long f = (long)(j - 1) * (nx + 1) + (i - 1);
      interior_face(o, cidx(o, i - 1, j), cidx(o, i, j), 0, xface_len(o, j), dt, o->fwx + f * 4,
                    o->fhx + f * nv, o->fbx + f * nv);
      o->fdonex[f] = 1;
    }
#pragma omp parallel for schedule(dynamic, 1)
  for (int j = j0; j <= j1; ++j)
    for (int i = 1; i <= nx; ++i) {
      long f = (long)(j - 1) * nx + (i - 1);
      interior_face(o, cidx(o, i, j - 1), cidx(o, i, j), 1, yface_len(o, i), dt, o->fwy + f * 4,
                    o->fhy + f * nv, o->fby + f * nv);
      o->fdoney[f] = 1;
    }
  /* Maxwell walls: every normal points along +x or +y, so rot = +1 on the
   * left / bottom wall and -1 on the right / top wall. */
  for (int s = 0; s < 4; ++s) {
    if (o->c.bc[s] != KB_BC_MAXWELL) continue;
    int nside = s < 2 ? ny : nx;
#pragma omp parallel for schedule(dynamic, 1)
    for (int q = 1; q <= nside; ++q) {
      double n[2], bcl[4], fwl[4];
      double* un = scratch(o) + 8 * nv;
      double* ut = un + nv;
      long c, f;
      double len;
      double *fw, *fh, *fb;
      if (s < 2) {
        n[0] = 1.0; n[1] = 0.0;
        int i = s == 0 ? 1 : nx;
        c = cidx(o, i, q);
        f = (long)(q - 1) * (nx + 1) + (s == 0 ? 0 : nx);
        len = o->dy;
        fw = o->fwx + f * 4; fh = o->fhx + f * nv; fb = o->fbx + f * nv;
        o->fdonex[f] = 1;
      } else {
        n[0] = 0.0; n[1] = 1.0;
        int j = s == 2 ? 1 : ny;
        c = cidx(o, q, j);
        f = (long)(s == 2 ? 0 : ny) * nx + (q - 1);
        len = o->dx;
        fw = o->fwy + f * 4; fh = o->fhy + f * nv; fb = o->fby + f * nv;
        o->fdoney[f] = 1;
      }
      for (long k = 0; k < nv; ++k) {
        un[k] = o->u[k] * n[0] + o->v[k] * n[1];
        ut[k] = o->v[k] * n[0] - o->u[k] * n[1];
      }
      local_frame(o->wall[s] + (long)(q - 1) * 4, n, bcl);
      if (o->c.nf == 1) {
        flux_maxwell_1f(o, bcl, Hc(o, c), un, ut, dt, len, (s == 0 || s == 2) ? 1 : -1, fwl, fh);
        memset(fb, 0, sizeof(double) * nv);
      } else {
        flux_maxwell(o, bcl, Hc(o, c), Bc(o, c), un, ut, dt, len, (s == 0 || s == 2) ? 1 : -1,
                     fwl, fh, fb);
      }
      global_frame(fwl, n, fw);
    }
  }
}

/* ----------------------------------------------------------------- update */

/* step! 1D2F1V (src/Solver/step_2f.jl:6-64) and 2D2F2V (:179-249).  Faces are
 * given as (fw, fh, fb) quadruples L, R, D, U; RES / AVG receive this cell's
 * (w - w_old)^2 and |w|. */
static void step_cell(kbo_t* o, long c, const double* const* fwv, const double* const* fhv,
                      const double* const* fbv, double ds, double dt, int coll, double* res,
                      double* avg) {
  int NW = o->NW;
  long nv = o->nvel;
  double K = o->c.K, g = o->c.gamma, Pr = o->c.Pr;
  double *w = o->w + c * 4, *prim = o->prim + c * 4, *h = Hc(o, c), *b = Bc(o, c);
  const double *u = o->u, *v = o->v, *om = o->wt;
  double* t = scratch(o);
  double* SHs = t + nv;
  double* SBs = SHs + nv;
  double w_old[4];
  memcpy(w_old, w, sizeof(w_old));
  if (coll == KB_COLL_SHAKHOV) {
    double q[2];
    if (NW == 3) {
      for (long k = 0; k < nv; ++k) {
        double cu = u[k] - prim[1];
        t[k] = om[k] * cu * (cu * cu) * h[k];
      }
      double a = psum(t, nv);
      for (long k = 0; k < nv; ++k) t[k] = om[k] * (u[k] - prim[1]) * b[k];
      q[0] = 0.5 * (a + psum(t, nv));
      for (long k = 0; k < nv; ++k) {
        double cu = u[k] - prim[1];
        double MH = prim[0] * sqrt(prim[2] / M_PI) * exp(-prim[2] * (cu * cu));
        double MB = MH * K / (2.0 * prim[2]);
        double f = 0.8 * (1.0 - Pr) * (prim[2] * prim[2]) / prim[0] * cu * q[0];
        SHs[k] = f * (2.0 * prim[2] * (cu * cu) + K - 5.0) * MH;
        SBs[k] = f * (2.0 * prim[2] * (cu * cu) + K - 3.0) * MB;
      }
    } else {
      for (int m = 0; m < 2; ++m) {
        for (long k = 0; k < nv; ++k) {
          double cu = u[k] - prim[1], cv = v[k] - prim[2];
          double cm = m == 0 ? cu : cv;
          t[k] = om[k] * cm * ((cu * cu) + (cv * cv)) * h[k];
        }
        double a = psum(t, nv);
        for (long k = 0; k < nv; ++k) t[k] = om[k] * ((m == 0 ? u[k] - prim[1] : v[k] - prim[2])) * b[k];
        q[m] = 0.5 * (a + psum(t, nv));
      }
      for (long k = 0; k < nv; ++k) {
        double cu = u[k] - prim[1], cv = v[k] - prim[2];
        double MH = prim[0] * (prim[3] / M_PI) * exp(-prim[3] * ((cu * cu) + (cv * cv)));
        double MB = MH * K / (2.0 * prim[3]);
        double f = 0.8 * (1.0 - Pr) * (prim[3] * prim[3]) / prim[0] * (cu * q[0] + cv * q[1]);
        SHs[k] = f * (2.0 * prim[3] * ((cu * cu) + (cv * cv)) + K - 5.0) * MH;
        SBs[k] = f * (2.0 * prim[3] * ((cu * cu) + (cv * cv)) + K - 3.0) * MB;
      }
    }
  } else {
    for (long k = 0; k < nv; ++k) SHs[k] = SBs[k] = 0.0;
  }
  for (int k = 0; k < NW; ++k) {
    if (NW == 3) w[k] += (fwv[0][k] - fwv[1][k]) / ds;
    else w[k] += (fwv[0][k] - fwv[1][k] + fwv[2][k] - fwv[3][k]) / ds;
  }
  conserve_prim(w, NW, g, prim);
  for (int k = 0; k < NW; ++k) {
    res[k] = (w[k] - w_old[k]) * (w[k] - w_old[k]);
    avg[k] = fabs(w[k]);
  }
  double tau = vhs_time(prim, NW, o->c.mu_ref, o->c.omega);
  for (long k = 0; k < nv; ++k) {
    double MH;
    if (NW == 3)
      MH = prim[0] * sqrt(prim[2] / M_PI) * exp(-prim[2] * ((u[k] - prim[1]) * (u[k] - prim[1])));
    else
      MH = prim[0] * (prim[3] / M_PI) *
           exp(-prim[3] * ((u[k] - prim[1]) * (u[k] - prim[1]) + (v[k] - prim[2]) * (v[k] - prim[2])));
    double MB = MH * K / (2.0 * prim[NW - 1]);
    MH += SHs[k];
    MB += SBs[k];
    if (NW == 3) {
      h[k] = (h[k] + (fhv[0][k] - fhv[1][k]) / ds + dt / tau * MH) / (1.0 + dt / tau);
      b[k] = (b[k] + (fbv[0][k] - fbv[1][k]) / ds + dt / tau * MB) / (1.0 + dt / tau);
    } else {
      h[k] = (h[k] + (fhv[0][k] - fhv[1][k] + fhv[2][k] - fhv[3][k]) / ds + dt / tau * MH) /
             (1.0 + dt / tau);
      b[k] = (b[k] + (fbv[0][k] - fbv[1][k] + fbv[2][k] - fbv[3][k]) / ds + dt / tau * MB) /
             (1.0 + dt / tau);
    }
  }
}

/* step! 1D1F1V (src/Solver/step_1f.jl:6-58) and 2D1F2V (:164-224): f in h.
 * Shakhov (1D): q = heat_flux(f, prim, u, w) (theory_moments.jl:522),
 * S = shakhov(u, M, q, prim, Pr) (theory_equilibrium.jl:178-186).  The
 * reference's 2D1F2V Shakhov branch names an undefined b (step_1f.jl:194),
 * so 2D1F2V runs BGK only. */
static void step_cell_1f(kbo_t* o, long c, const double* const* fwv, const double* const* ffv,
                         double ds, double dt, int coll, double* res, double* avg) {
  int NW = o->NW;
  long nv = o->nvel;
  double g = o->c.gamma, Pr = o->c.Pr;
  double *w = o->w + c * 4, *prim = o->prim + c * 4, *f = Hc(o, c);
  const double *u = o->u, *v = o->v, *om = o->wt;
  double* t = scratch(o);
  double* S = t + nv;
  double w_old[4];
  memcpy(w_old, w, sizeof(w_old));
  if (coll == KB_COLL_SHAKHOV && NW == 3) {
    for (long k = 0; k < nv; ++k) {
      double cu = u[k] - prim[1];
      t[k] = om[k] * cu * (cu * cu) * f[k];
    }
    double q = 0.5 * psum(t, nv);
    for (long k = 0; k < nv; ++k) {
      double cu = u[k] - prim[1];
      double M = prim[0] * sqrt(prim[2] / M_PI) * exp(-prim[2] * (cu * cu));
      S[k] = 0.8 * (1.0 - Pr) * (prim[2] * prim[2]) / prim[0] * cu * q *
             (2.0 * prim[2] * (cu * cu) - 5.0) * M;
    }
  } else {
    for (long k = 0; k < nv; ++k) S[k] = 0.0;
  }
  for (int k = 0; k < NW; ++k) {
    if (NW == 3) w[k] += (fwv[0][k] - fwv[1][k]) / ds;
    else w[k] += (fwv[0][k] - fwv[1][k] + fwv[2][k] - fwv[3][k]) / ds;
  }
  conserve_prim(w, NW, g, prim);
  for (int k = 0; k < NW; ++k) {
    res[k] = (w[k] - w_old[k]) * (w[k] - w_old[k]);
    avg[k] = fabs(w[k]);
  }
  double tau = vhs_time(prim, NW, o->c.mu_ref, o->c.omega);
  for (long k = 0; k < nv; ++k) {
    double M;
    if (NW == 3)
      M = prim[0] * sqrt(prim[2] / M_PI) * exp(-prim[2] * ((u[k] - prim[1]) * (u[k] - prim[1])));
    else
      M = prim[0] * (prim[3] / M_PI) *
          exp(-prim[3] * ((u[k] - prim[1]) * (u[k] - prim[1]) + (v[k] - prim[2]) * (v[k] - prim[2])));
    M += S[k];
    if (NW == 3)
      f[k] = (f[k] + (ffv[0][k] - ffv[1][k]) / ds + dt / tau * M) / (1.0 + dt / tau);
    else
      f[k] = (f[k] + (ffv[0][k] - ffv[1][k] + ffv[2][k] - ffv[3][k]) / ds + dt / tau * M) /
             (1.0 + dt / tau);
  }
}

static void copy_ctr(kbo_t* o, long dst, long src) { /* copy_ctr!, src/Struct/struct.jl:55-66 */
  memcpy(o->w + dst * 4, o->w + src * 4, sizeof(double) * 4);
  memcpy(o->prim + dst * 4, o->prim + src * 4, sizeof(double) * 4);
  memcpy(o->sw + dst * 8, o->sw + src * 8, sizeof(double) * 8);
  memcpy(Hc(o, dst), Hc(o, src), sizeof(double) * o->nvel);
  memcpy(Bc(o, dst), Bc(o, src), sizeof(double) * o->nvel);
}

/* update! 1D (src/Solver/solver_update.jl:61-93) + update_boundary!
 * (src/Solver/update_boundary.jl:6-61); 2D (:193-246) + (:172-306). */
void kbo_update(kbo_t* o, double dt, double* residual) {
  ensure_scratch(o);
  int nx = o->c.nx, ny = o->c.ny, NW = o->NW;
  long nv = o->nvel;
  int coll = o->c.collision;
  double* res = calloc((long)o->ncell * 8, sizeof(double)); /* res[4], avg[4] per cell */
  unsigned char* grp = calloc(o->ncell, 1); /* 0 untouched, 1 interior, 2+s boundary side s */
  if (o->D == 1) {
    for (int i = 2; i <= nx - 1; ++i) grp[cidx(o, i, 1)] = 1;
    if (o->c.bc[0] != KB_BC_FIX) grp[cidx(o, 1, 1)] = 2;
    if (o->c.bc[1] != KB_BC_FIX) grp[cidx(o, nx, 1)] = 3;
  } else {
    for (int j = 2; j <= ny - 1; ++j)
      for (int i = 2; i <= nx - 1; ++i) grp[cidx(o, i, j)] = 1;
    if (o->c.bc[0] != KB_BC_FIX) for (int j = 1; j <= ny; ++j) grp[cidx(o, 1, j)] = 2;
    if (o->c.bc[1] != KB_BC_FIX) for (int j = 1; j <= ny; ++j) grp[cidx(o, nx, j)] = 3;
    if (o->c.bc[2] != KB_BC_FIX) for (int i = 2; i <= nx - 1; ++i) grp[cidx(o, i, 1)] = 4;
    if (o->c.bc[3] != KB_BC_FIX) for (int i = 2; i <= nx - 1; ++i) grp[cidx(o, i, ny)] = 5;
  }
#pragma omp parallel for schedule(dynamic, 1)
  for (int j = 1; j <= ny; ++j)
    for (int i = 1; i <= nx; ++i) {
      long c = cidx(o, i, j);
      if (!grp[c]) continue;
      const double *fwv[4] = {0, 0, 0, 0}, *fhv[4] = {0, 0, 0, 0}, *fbv[4] = {0, 0, 0, 0};
      long fl = (long)(j - 1) * (nx + 1) + (i - 1), fr = fl + 1;
      fwv[0] = o->fwx + fl * 4; fhv[0] = o->fhx + fl * nv; fbv[0] = o->fbx + fl * nv;
      fwv[1] = o->fwx + fr * 4; fhv[1] = o->fhx + fr * nv; fbv[1] = o->fbx + fr * nv;
      double ds = o->dx;
      if (o->D == 2) {
        long fd = (long)(j - 1) * nx + (i - 1), fu = fd + nx;
        fwv[2] = o->fwy + fd * 4; fhv[2] = o->fhy + fd * nv; fbv[2] = o->fby + fd * nv;
        fwv[3] = o->fwy + fu * 4; fhv[3] = o->fhy + fu * nv; fbv[3] = o->fby + fu * nv;
        ds = o->dx * o->dy;
      }
      /* 1D boundary cells are stepped without the collision keyword, i.e. BGK
       * (src/Solver/update_boundary.jl:33,38) */
      int cc = (o->D == 1 && grp[c] >= 2) ? KB_COLL_BGK : coll;
      if (o->c.nf == 1) step_cell_1f(o, c, fwv, fhv, ds, dt, cc, res + c * 8, res + c * 8 + 4);
      else step_cell(o, c, fwv, fhv, fbv, ds, dt, cc, res + c * 8, res + c * 8 + 4);
    }
  /* residuals in cell order (the reference sums racily under @threads) */
  double sR[4] = {0}, sA[4] = {0}, bR[4] = {0}, bA[4] = {0};
  for (int j = 1; j <= ny; ++j)
    for (int i = 1; i <= nx; ++i) {
      long c = cidx(o, i, j);
      if (!grp[c]) continue;
      for (int k = 0; k < NW; ++k) {
        if (grp[c] == 1) { sR[k] += res[c * 8 + k]; sA[k] += res[c * 8 + 4 + k]; }
        else { bR[k] += res[c * 8 + k]; bA[k] += res[c * 8 + 4 + k]; }
      }
    }
  double ncell = o->D == 1 ? (double)nx : (double)nx * ny;
  for (int k = 0; k < NW; ++k) {
    double r = sqrt(sR[k] * ncell) / (sA[k] + 1.e-7);
    r += sqrt(bR[k] * 2) / (bA[k] + 1.e-7);
    if (residual) residual[k] = r;
  }
  free(res);
  free(grp);
  /* ghost fill: bc_extra! / bc_period! (src/Boundary/bc_extra.jl, bc_period.jl) */
  int ngx = o->c.ngx, ngy = o->c.ngy;
  if (o->D == 1) {
    if (o->c.bc[0] == KB_BC_PERIOD) {
      for (int k = 1; k <= ngx; ++k) {
        copy_ctr(o, cidx(o, 1 - k, 1), cidx(o, nx + 1 - k, 1));
        copy_ctr(o, cidx(o, nx + k, 1), cidx(o, k, 1));
      }
    } else if (o->c.bc[0] == KB_BC_EXTRA) {
      for (int k = 1; k <= ngx; ++k) copy_ctr(o, cidx(o, 1 - k, 1), cidx(o, 1, 1));
    }
    if (o->c.bc[1] == KB_BC_EXTRA)
      for (int k = 1; k <= ngx; ++k) copy_ctr(o, cidx(o, nx + k, 1), cidx(o, nx, 1));
    return;
  }
  if (o->c.bc[0] == KB_BC_EXTRA)
    for (int j = 1 - ngy; j <= ny + ngy; ++j)
      for (int k = 1; k <= ngx; ++k) copy_ctr(o, cidx(o, 1 - k, j), cidx(o, 1, j));
  if (o->c.bc[1] == KB_BC_EXTRA)
    for (int j = 1 - ngy; j <= ny + ngy; ++j)
      for (int k = 1; k <= ngx; ++k) copy_ctr(o, cidx(o, nx + k, j), cidx(o, nx, j));
  if (o->c.bc[2] == KB_BC_EXTRA)
    for (int k = 1; k <= ngy; ++k)
      for (int i = 1 - ngx; i <= nx + ngx; ++i) copy_ctr(o, cidx(o, i, 1 - k), cidx(o, i, 1));
  if (o->c.bc[3] == KB_BC_EXTRA)
    for (int k = 1; k <= ngy; ++k)
      for (int i = 1 - ngx; i <= nx + ngx; ++i) copy_ctr(o, cidx(o, i, ny + k), cidx(o, i, ny));
}

void kbo_step(kbo_t* o, double dt, int nsteps, double* residual) {
  for (int s = 0; s < nsteps; ++s) {
    kbo_reconstruct(o);
    kbo_evolve(o, dt);
    kbo_update(o, dt, residual);
  }
}

/* Faces of the last evolve in the kb_download_faces layout (global-frame fw). */
int kbo_get_faces(const kbo_t* o, double* fw, double* fh, double* fb) {
  long nv = o->nvel;
  int NW = o->NW;
  for (long f = 0; f < o->nfx + o->nfy; ++f) {
    int x = f < o->nfx;
    long g = x ? f : f - o->nfx;
    int done = x ? o->fdonex[g] : o->fdoney[g];
    const double* w = (x ? o->fwx : o->fwy) + g * 4;
    const double* hh = (x ? o->fhx : o->fhy) + g * nv;
    const double* bb = (x ? o->fbx : o->fby) + g * nv;
    for (int k = 0; k < NW; ++k)
      if (fw) fw[f * NW + k] = done ? w[k] : 0.0;
    for (long k = 0; k < nv; ++k) {
      if (fh) fh[f * nv + k] = done ? hh[k] : 0.0;
      if (fb) fb[f * nv + k] = done ? bb[k] : 0.0;
    }
  }
  return 0;
}

/* Slopes in the kb_download_slopes layout: sw [cell][dim][NW], sh/sb [cell][dim][nvel]. */
int kbo_get_slopes(const kbo_t* o, double* sw, double* sh, double* sb) {
  long nv = o->nvel;
  int D = o->D, NW = o->NW;
  for (long c = 0; c < o->ncell; ++c)
    for (int d = 0; d < D; ++d) {
      if (sw)
        for (int k = 0; k < NW; ++k) sw[(c * D + d) * NW + k] = SW(o, c, d)[k];
      if (sh) memcpy(sh + (c * D + d) * nv, SH(o, c, d), sizeof(double) * nv);
      if (sb) memcpy(sb + (c * D + d) * nv, SB(o, c, d), sizeof(double) * nv);
    }
  return 0;
}

/* ------------------------------------------------ pointwise entry points */

void kbo_gauss_moments(const double* prim, int nw, double inK, double* Mu, double* Mv,
                       double* Mxi, double* MuL, double* MuR) {
  gauss_moments(prim, nw, inK, Mu, Mv, Mxi, MuL, MuR);
}
void kbo_conserve_prim(const double* w, int nw, double g, double* prim) {
  conserve_prim(w, nw, g, prim);
}
void kbo_prim_conserve(const double* prim, int nw, double g, double* w) {
  prim_conserve(prim, nw, g, w);
}
void kbo_pdf_slope(const double* prim, const double* sw, int nw, double inK, double* sl) {
  pdf_slope(prim, sw, nw, inK, sl);
}
double kbo_vanleer(double sL, double sR) { return vanleer(sL, sR); }
double kbo_psum(const double* a, long n) { return psum(a, n); }
