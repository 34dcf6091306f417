/* kb_oracle_us.c -- TEST INFRASTRUCTURE ONLY: FP64 C restatement of
 * KitBase.jl's unstructured DVM step (2D2F2V and 2D1F2V on triangle meshes),
 * the multithreaded counterpart of oracle/oracle_us.py (same formulas, same
 * mesh tables, built by oracle_us.py from the points and triangles
 * independently of the product's host code).  Only tests/ and bench.py's CPU
 * baseline load it.
 *
 * PARITY UNPINNED: the reference cannot run here and its unstructured test
 * (test/test_unstructure.jl) asserts nothing.
 *
 * Restated (file:line of the reference):
 *  - evolve! US2F / US1F, KFVS branch, first-order face states
 *    (src/Solver/solver_evolution.jl:872-1035) with flux_kfvs! 2F2V / 1F2V
 *    (src/Flux/flux_kfvs.jl:615-700), flux_conserve!
 *    (src/Theory/theory_moments.jl:409-414) and global_frame
 *    (src/Geometry/geo_general.jl:6-26);
 *  - update! US2F / US1F (src/Solver/solver_update.jl:359-471) with the
 *    triangle step! (src/Solver/step_2f.jl:256-326, src/Solver/step_1f.jl:228-285),
 *    heat_flux and shakhov 2F2V (src/Theory/theory_moments.jl:567-578,
 *    src/Theory/theory_equilibrium.jl:227-238);
 *  - update_boundary! US2F / US1F (src/Solver/update_boundary.jl:546-594);
 *  - timestep for unstructured cells (src/Solver/solver_main.jl:398-420).
 * Velocity sums use Julia's pairwise reduction (psum, as in kb_oracle.c).
 */
#include <math.h>
#include <omp.h>
#include <stdlib.h>
#include <string.h>

typedef struct {
  int nc, nface, nv, coll, nfm; /* nfm: 2 (h, b) or 1 (f) */
  double K, gamma, mu, omega, Pr;
  const int* fcell;  /* [nface][2] first cell, second cell or -1 */
  const int* cface;  /* [nc][3] */
  const int* nb;     /* [nc][3] -1 where none */
  const int* ctype;  /* [nc] */
  const double* fn;  /* [nface][2] normal from the first to the second cell */
  const double* flen;
  const double* dirc; /* [nc][3] orientation sign of each face for the cell */
  const double* area;
  const double* dxmin;
  const double *u, *v, *wt;
  double *w, *prim, *h, *b; /* [nc][4], [nc][4], [nc][nv] x 2 */
  double *fw, *fh, *fb;     /* [nface][4], [nface][nv] x 2 */
  double *cres;             /* [nc][8] */
  double* tmp;              /* per-thread scratch [threads][6 nv] */
  int ntmp;
} kbou_t;

static double usum(const double* a, long n) {
  if (n <= 1024) {
    double s = 0.0;
    for (long i = 0; i < n; ++i) s += a[i];
    return s;
  }
  long mid = (n - 1) >> 1;
  return usum(a, mid + 1) + usum(a + mid + 1, n - mid - 1);
}

/* conserve_prim 2D, src/Theory/theory_macro.jl:185-206 */
static void us_conserve_prim(const double* w, double g, double* p) {
  p[0] = w[0];
  p[1] = w[1] / w[0];
  p[2] = w[2] / w[0];
  p[3] = 0.5 * w[0] / (g - 1.0) / (w[3] - 0.5 * (w[1] * w[1] + w[2] * w[2]) / w[0]);
}

void* kbou_create(int nc, int nface, const int* fcell, const int* cface, const int* nb, const int* ctype,
                  const double* fn, const double* flen, const double* dirc, const double* area,
                  const double* dxmin, int nv, const double* u, const double* v, const double* wt,
                  double K, double gamma, double mu, double omega, double Pr, int coll, int nfm) {
  kbou_t* o = (kbou_t*)calloc(1, sizeof(kbou_t));
  if (!o) return NULL;
  o->nc = nc;
  o->nface = nface;
  o->nv = nv;
  o->coll = coll;
  o->nfm = nfm;
  o->K = K;
  o->gamma = gamma;
  o->mu = mu;
  o->omega = omega;
  o->Pr = Pr;
  o->fcell = fcell;
  o->cface = cface;
  o->nb = nb;
  o->ctype = ctype;
  o->fn = fn;
  o->flen = flen;
  o->dirc = dirc;
  o->area = area;
  o->dxmin = dxmin;
  o->u = u;
  o->v = v;
  o->wt = wt;
  o->w = (double*)calloc((size_t)nc * 4, sizeof(double));
  o->prim = (double*)calloc((size_t)nc * 4, sizeof(double));
  o->h = (double*)calloc((size_t)nc * nv, sizeof(double));
  o->b = (double*)calloc((size_t)nc * nv, sizeof(double));
  o->fw = (double*)calloc((size_t)nface * 4, sizeof(double));
  o->fh = (double*)calloc((size_t)nface * nv, sizeof(double));
  o->fb = (double*)calloc((size_t)nface * nv, sizeof(double));
  o->cres = (double*)calloc((size_t)nc * 8, sizeof(double));
  o->ntmp = omp_get_max_threads();
  o->tmp = (double*)calloc((size_t)o->ntmp * 6 * nv, sizeof(double));
  return o;
}

void kbou_destroy(void* p) {
  kbou_t* o = (kbou_t*)p;
  if (!o) return;
  free(o->w);
  free(o->prim);
  free(o->h);
  free(o->b);
  free(o->fw);
  free(o->fh);
  free(o->fb);
  free(o->cres);
  free(o->tmp);
  free(o);
}

void kbou_set_state(void* p, const double* w, const double* prim, const double* h, const double* b) {
  kbou_t* o = (kbou_t*)p;
  memcpy(o->w, w, sizeof(double) * 4 * (size_t)o->nc);
  memcpy(o->prim, prim, sizeof(double) * 4 * (size_t)o->nc);
  memcpy(o->h, h, sizeof(double) * (size_t)o->nc * o->nv);
  memcpy(o->b, b, sizeof(double) * (size_t)o->nc * o->nv);
}

void kbou_get_state(void* p, double* w, double* prim, double* h, double* b) {
  kbou_t* o = (kbou_t*)p;
  memcpy(w, o->w, sizeof(double) * 4 * (size_t)o->nc);
  memcpy(prim, o->prim, sizeof(double) * 4 * (size_t)o->nc);
  memcpy(h, o->h, sizeof(double) * (size_t)o->nc * o->nv);
  memcpy(b, o->b, sizeof(double) * (size_t)o->nc * o->nv);
}

/* timestep: cfl / max over cells of sqrt(umax^2 + vmax^2) / min dx with
 * umax = u1 + c, vmax = v1 + c, clipped to max_time - t */
double kbou_timestep(void* p, double cfl, double t, double tmax_time, double u1, double v1) {
  kbou_t* o = (kbou_t*)p;
  double tm = 0.0;
  for (int c = 0; c < o->nc; ++c) {
    const double sos = pow(0.5 * o->gamma / o->prim[4 * c + 3], 0.5);
    const double um = u1 + sos, vm = v1 + sos;
    const double r = sqrt(um * um + vm * vm) / o->dxmin[c];
    if (r > tm) tm = r;
  }
  const double dt = cfl / tm;
  return dt < tmax_time - t ? dt : tmax_time - t;
}

static void us_evolve(kbou_t* o, double dt) {
  const int nv = o->nv;
#pragma omp parallel for schedule(static)
  for (int f = 0; f < o->nface; ++f) {
    double* t = o->tmp + (size_t)omp_get_thread_num() * 6 * nv;
    double* fw = o->fw + 4L * f;
    double* fh = o->fh + (size_t)f * nv;
    double* fb = o->fb + (size_t)f * nv;
    const int c1 = o->fcell[2 * f], c2 = o->fcell[2 * f + 1];
    if (c2 < 0) {  /* boundary face: no flux (cell types 0, 1, 3) */
      fw[0] = fw[1] = fw[2] = fw[3] = 0.0;
      memset(fh, 0, sizeof(double) * nv);
      memset(fb, 0, sizeof(double) * nv);
      continue;
    }
    const double n1 = o->fn[2 * f], n2 = o->fn[2 * f + 1], len = o->flen[f];
    const double *hL = o->h + (size_t)c1 * nv, *hR = o->h + (size_t)c2 * nv;
    const double *bL = o->b + (size_t)c1 * nv, *bR = o->b + (size_t)c2 * nv;
    double *s0 = t, *s1 = t + nv, *s2 = t + 2 * nv, *s3 = t + 3 * nv, *s4 = t + 4 * nv;
    for (int k = 0; k < nv; ++k) {
      const double vn = o->u[k] * n1 + o->v[k] * n2;
      const double vt = o->v[k] * n1 - o->u[k] * n2;
      const double d = vn >= 0.0 ? 1.0 : 0.0; /* heaviside */
      const double hh = hL[k] * d + hR[k] * (1.0 - d);
      fh[k] = (dt * vn * hh - 0.5 * dt * dt * vn * vn * 0.0) * len;
      if (o->nfm == 2) {
        const double bb = bL[k] * d + bR[k] * (1.0 - d);
        fb[k] = (dt * vn * bb - 0.5 * dt * dt * vn * vn * 0.0) * len;
      } else {
        fb[k] = 0.0;
      }
      s0[k] = o->wt[k] * fh[k];
      s1[k] = vn * o->wt[k] * fh[k];
      s2[k] = vt * o->wt[k] * fh[k];
      s3[k] = (vn * vn + vt * vt) * o->wt[k] * fh[k];
      s4[k] = o->wt[k] * fb[k];
    }
    const double a0 = usum(s0, nv), a1 = usum(s1, nv), a2 = usum(s2, nv);
    const double a3 = o->nfm == 2 ? 0.5 * (usum(s3, nv) + usum(s4, nv)) : 0.5 * usum(s3, nv);
    fw[0] = a0;
    fw[1] = a1 * n1 - a2 * n2;
    fw[2] = a1 * n2 + a2 * n1;
    fw[3] = a3;
  }
}

static void us_update(kbou_t* o, double dt, double* res) {
  const int nv = o->nv;
  const double K = o->K, Pr = o->Pr;
#pragma omp parallel for schedule(static)
  for (int c = 0; c < o->nc; ++c) {
    double* cr = o->cres + 8L * c;
    if (o->ctype[c] != 0 && o->ctype[c] != 2) {
      for (int k = 0; k < 8; ++k) cr[k] = 0.0;
      continue;
    }
    double* t = o->tmp + (size_t)omp_get_thread_num() * 6 * nv;
    double *w = o->w + 4L * c, *p = o->prim + 4L * c;
    double *h = o->h + (size_t)c * nv, *b = o->b + (size_t)c * nv;
    const int* fs = o->cface + 3 * c;
    const double* dc = o->dirc + 3 * c;
    const double area = o->area[c];
    double q0 = 0.0, q1 = 0.0;
    const double rho_o = p[0], U_o = p[1], V_o = p[2], lam_o = p[3];
    if (o->coll == 1) { /* heat_flux 2F2V of the old state */
      double *a = t, *bq = t + nv, *e = t + 2 * nv, *fq = t + 3 * nv;
      for (int k = 0; k < nv; ++k) {
        const double cu = o->u[k] - U_o, cv = o->v[k] - V_o, c2 = cu * cu + cv * cv;
        a[k] = o->wt[k] * cu * c2 * h[k];
        bq[k] = o->wt[k] * cu * b[k];
        e[k] = o->wt[k] * cv * c2 * h[k];
        fq[k] = o->wt[k] * cv * b[k];
      }
      q0 = 0.5 * (usum(a, nv) + usum(bq, nv));
      q1 = 0.5 * (usum(e, nv) + usum(fq, nv));
    }
    double wo[4];
    for (int k = 0; k < 4; ++k) {
      wo[k] = w[k];
      w[k] -= (o->fw[4L * fs[0] + k] * dc[0] + o->fw[4L * fs[1] + k] * dc[1] + o->fw[4L * fs[2] + k] * dc[2]) /
              area;
    }
    us_conserve_prim(w, o->gamma, p);
    for (int k = 0; k < 4; ++k) {
      cr[k] = (w[k] - wo[k]) * (w[k] - wo[k]);
      cr[4 + k] = fabs(w[k]);
    }
    const double tau = o->mu * 2.0 * pow(p[3], 1.0 - o->omega) / p[0];
    const double kk = dt / tau;
    const double *f0h = o->fh + (size_t)fs[0] * nv, *f1h = o->fh + (size_t)fs[1] * nv,
                 *f2h = o->fh + (size_t)fs[2] * nv;
    const double *f0b = o->fb + (size_t)fs[0] * nv, *f1b = o->fb + (size_t)fs[1] * nv,
                 *f2b = o->fb + (size_t)fs[2] * nv;
    for (int k = 0; k < nv; ++k) {
      const double du = o->u[k] - p[1], dv = o->v[k] - p[2];
      double MH = p[0] * (p[3] / M_PI) * exp(-p[3] * (du * du + dv * dv));
      double MB = o->nfm == 2 ? MH * K / (2.0 * p[3]) : 0.0;
      if (o->coll == 1) {
        const double cu = o->u[k] - U_o, cv = o->v[k] - V_o, c2 = cu * cu + cv * cv;
        const double MHo = rho_o * (lam_o / M_PI) * exp(-lam_o * c2);
        const double MBo = MHo * K / (2.0 * lam_o);
        const double fac = 0.8 * (1.0 - Pr) * lam_o * lam_o / rho_o * (cu * q0 + cv * q1);
        MH += fac * (2.0 * lam_o * c2 + K - 5.0) * MHo;
        MB += fac * (2.0 * lam_o * c2 + K - 3.0) * MBo;
      }
      h[k] = (h[k] - (f0h[k] * dc[0] + f1h[k] * dc[1] + f2h[k] * dc[2]) / area + kk * MH) / (1.0 + kk);
      if (o->nfm == 2)
        b[k] = (b[k] - (f0b[k] * dc[0] + f1b[k] * dc[1] + f2b[k] * dc[2]) / area + kk * MB) / (1.0 + kk);
    }
  }
  /* residual in cell order */
  double sr[4] = {0, 0, 0, 0}, sa[4] = {0, 0, 0, 0};
  for (int c = 0; c < o->nc; ++c)
    for (int k = 0; k < 4; ++k) {
      sr[k] += o->cres[8L * c + k];
      sa[k] += o->cres[8L * c + 4 + k];
    }
  for (int k = 0; k < 4; ++k) res[k] = sqrt(sr[k] * o->nc) / (sa[k] + 1.e-7);
  /* update_boundary!: extrapolated cells in cell order, mean of the first two neighbours */
  for (int c = 0; c < o->nc; ++c) {
    if (o->ctype[c] != 3) continue;
    int id[2], m = 0;
    for (int j = 0; j < 3 && m < 2; ++j)
      if (o->nb[3 * c + j] != -1) id[m++] = o->nb[3 * c + j];
    for (int k = 0; k < 4; ++k) o->w[4L * c + k] = 0.5 * (o->w[4L * id[0] + k] + o->w[4L * id[1] + k]);
    for (int k = 0; k < nv; ++k) {
      o->h[(size_t)c * nv + k] = 0.5 * (o->h[(size_t)id[0] * nv + k] + o->h[(size_t)id[1] * nv + k]);
      if (o->nfm == 2)
        o->b[(size_t)c * nv + k] = 0.5 * (o->b[(size_t)id[0] * nv + k] + o->b[(size_t)id[1] * nv + k]);
    }
    us_conserve_prim(o->w + 4L * c, o->gamma, o->prim + 4L * c);
  }
}

void kbou_step(void* p, double dt, int n, double* res) {
  kbou_t* o = (kbou_t*)p;
  double r[4] = {0, 0, 0, 0};
  if (omp_get_max_threads() > o->ntmp) { /* the thread count grew since creation */
    free(o->tmp);
    o->ntmp = omp_get_max_threads();
    o->tmp = (double*)calloc((size_t)o->ntmp * 6 * o->nv, sizeof(double));
  }
  for (int s = 0; s < n; ++s) {
    us_evolve(o, dt);
    us_update(o, dt, r);
  }
  if (res)
    for (int k = 0; k < 4; ++k) res[k] = r[k];
}
