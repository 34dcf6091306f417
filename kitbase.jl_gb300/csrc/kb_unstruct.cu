// kb_unstruct.cu -- the DVM step of 2D2F2V solves on triangle meshes
// (KitBase's unstructured 2F path: evolve! US2F,
// src/Solver/solver_evolution.jl:945-1035; update! US2F,
// src/Solver/solver_update.jl:414-471; triangle step!,
// src/Solver/step_2f.jl:256-326; update_boundary! US2F,
// src/Solver/update_boundary.jl:575-594; timestep for unstructured cells,
// src/Solver/solver_main.jl:398-420).
//
// Cells and faces are gathered through index tables, so each step is three
// kernels: one CTA per face forms the first-order KFVS fluxes fh, fb of every
// velocity (stored per face) and their moments fw; one CTA per stepped cell
// applies the triangle update (w from the three faces' fw with their
// orientation signs, then the BGK / Shakhov relaxation of h, b from the three
// faces' fh, fb, in place); one CTA walks the extrapolated boundary cells in
// cell order and sets each to the mean of its two neighbours.  The plain
// form computes in FP64 throughout; the FP32 split form stores h, b and the
// face fluxes in FP32 and keeps fw, w, prim and all moments in FP64.
#include <cuda_runtime.h>

#include <string>
#include <vector>

#include "../../include/kitgpu.h"
#include "kb_device.cuh"
#include "kb_kernels.cuh"

namespace kb {

struct UsDev {
  int ncell, nface, nvel, vstride, coll, navg;
  const int* face_cells;     // [nface][2], -1 where no cell
  const int* cell_faces;     // [ncell][3]
  const int* cell_nb;        // [ncell][3], -1 where no cell
  const int* cell_type;      // [ncell]: 0 stepped, 1 fixed, 3 mean of two neighbours
  const int* avg_list;       // type-3 cells in cell order [navg]
  const double* face_n;      // [nface][2]
  const double* face_len;    // [nface]
  const double* cell_area;   // [ncell]
  const double* cell_mindx;  // [ncell] smallest centre-to-edge distance
  const double* u;
  const double* v;
  const double* wt;
  double* w;      // [ncell][4]
  double* prim;   // [ncell][4]
  void* h;        // [ncell][vstride]
  void* b;
  void* fh;       // [nface][vstride]
  void* fb;
  double* fw;     // [nface][4] global frame
  double* cres;   // [ncell][8]: (w - w_old)^2, |w| of the last step
  double* tmax;   // [1]
  double* residual;  // [4]
  int* status;
  double K, gamma, mu_ref, omega, Pr, umax, vmax;
};

constexpr int US_T = 128;

// fixed-order tree sum over the CTA (deterministic)
__device__ __forceinline__ double us_block_sum(double x, double* red) {
  red[threadIdx.x] = x;
  __syncthreads();
  for (int s = US_T / 2; s >= 1; s >>= 1) {
    if (threadIdx.x < s) red[threadIdx.x] += red[threadIdx.x + s];
    __syncthreads();
  }
  const double r = red[0];
  __syncthreads();
  return r;
}

// flux_kfvs! 2F2V (src/Flux/flux_kfvs.jl:654-700) of first-order face states
// with flux_conserve! (src/Theory/theory_moments.jl:409-414), then
// global_frame (src/Geometry/geo_general.jl:6-26).  Faces without two cells
// are not used by any stepped cell and carry zero flux.
template <typename R>
__global__ void __launch_bounds__(US_T) k_us_face(UsDev d, double dt) {
  __shared__ double red[US_T];
  const int f = blockIdx.x;
  const int cl = d.face_cells[2 * f], cr = d.face_cells[2 * f + 1];
  R* Fh = (R*)d.fh + (long)f * d.vstride;
  R* Fb = (R*)d.fb + (long)f * d.vstride;
  if (cl < 0 || cr < 0) {
    for (int v = threadIdx.x; v < d.nvel; v += US_T) {
      Fh[v] = R(0);
      Fb[v] = R(0);
    }
    if (threadIdx.x < 4) d.fw[4 * f + threadIdx.x] = 0.0;
    return;
  }
  const double n1 = d.face_n[2 * f], n2 = d.face_n[2 * f + 1], len = d.face_len[f];
  const R* HL = (const R*)d.h + (long)cl * d.vstride;
  const R* BL = (const R*)d.b + (long)cl * d.vstride;
  const R* HR = (const R*)d.h + (long)cr * d.vstride;
  const R* BR = (const R*)d.b + (long)cr * d.vstride;
  double s[5] = {0.0, 0.0, 0.0, 0.0, 0.0};
  for (int v = threadIdx.x; v < d.nvel; v += US_T) {
    const double u = d.u[v], vv = d.v[v];
    const double vn = __dadd_rn(__dmul_rn(u, n1), __dmul_rn(vv, n2));
    const double vt = __dsub_rn(__dmul_rn(vv, n1), __dmul_rn(u, n2));
    const bool up = vn >= 0.0;  // heaviside(0) = 1
    R fh, fb;
    if (sizeof(R) == 8) {
      const double hs = up ? (double)HL[v] : (double)HR[v];
      const double bs = up ? (double)BL[v] : (double)BR[v];
      fh = R(__dmul_rn(__dmul_rn(__dmul_rn(dt, vn), hs), len));
      fb = R(__dmul_rn(__dmul_rn(__dmul_rn(dt, vn), bs), len));
    } else {
      const float hs = up ? (float)HL[v] : (float)HR[v];
      const float bs = up ? (float)BL[v] : (float)BR[v];
      const float tl = float(dt * len * vn);
      fh = R(tl * hs);
      fb = R(tl * bs);
    }
    Fh[v] = fh;
    Fb[v] = fb;
    const double om = d.wt[v];
    const double wf = om * (double)fh;
    s[0] += wf;
    s[1] += vn * wf;
    s[2] += vt * wf;
    s[3] += (vn * vn + vt * vt) * wf;
    s[4] += om * (double)fb;
  }
  double S[5];
#pragma unroll
  for (int k = 0; k < 5; ++k) S[k] = us_block_sum(s[k], red);
  if (threadIdx.x == 0) {
    const double l1 = S[1], l2 = S[2];
    d.fw[4 * f + 0] = S[0];
    d.fw[4 * f + 1] = l1 * n1 - l2 * n2;
    d.fw[4 * f + 2] = l1 * n2 + l2 * n1;
    d.fw[4 * f + 3] = 0.5 * (S[3] + S[4]);
  }
}

// step! 2D2F2V on a triangle (src/Solver/step_2f.jl:256-326) for the cells
// update! US2F steps (cellType 0, src/Solver/solver_update.jl:428-462); the
// orientation sign of face j is +1 when the face normal points out of the
// cell (the cell is the first of the face's two cells) and -1 otherwise.
template <typename R>
__global__ void __launch_bounds__(US_T) k_us_cell(UsDev d, double dt) {
  __shared__ double red[US_T];
  __shared__ double sh[16];
  const int c = blockIdx.x;
  double* cr = d.cres + 8L * c;
  if (d.cell_type[c] != 0) {
    if (threadIdx.x < 8) cr[threadIdx.x] = 0.0;
    return;
  }
  int fj[3];
  double sg[3];
#pragma unroll
  for (int j = 0; j < 3; ++j) {
    fj[j] = d.cell_faces[3 * c + j];
    // a boundary face's normal points into its only cell
    sg[j] = (d.face_cells[2 * fj[j]] == c && d.face_cells[2 * fj[j] + 1] != -1) ? 1.0 : -1.0;
  }
  const double area = d.cell_area[c];
  double* w = d.w + 4L * c;
  double* p = d.prim + 4L * c;
  const double rho_o = p[0], U_o = p[1], V_o = p[2], lam_o = p[3];
  R* H = (R*)d.h + (long)c * d.vstride;
  R* B = (R*)d.b + (long)c * d.vstride;
  const bool shak = d.coll == COLL_SHAKHOV;
  double q0 = 0.0, q1 = 0.0;
  if (shak) {  // heat_flux 2F2V of the old state (src/Theory/theory_moments.jl:567-578)
    double a0 = 0.0, a1 = 0.0;
    for (int v = threadIdx.x; v < d.nvel; v += US_T) {
      const double cu = d.u[v] - U_o, cv = d.v[v] - V_o, om = d.wt[v];
      const double c2 = cu * cu + cv * cv, hv = (double)H[v], bv = (double)B[v];
      a0 += om * cu * c2 * hv + om * cu * bv;
      a1 += om * cv * c2 * hv + om * cv * bv;
    }
    q0 = 0.5 * us_block_sum(a0, red);
    q1 = 0.5 * us_block_sum(a1, red);
  }
  __syncthreads();  // every thread has read the old prim before thread 0 replaces it
  if (threadIdx.x == 0) {
    double wo[4];
    for (int k = 0; k < 4; ++k) wo[k] = w[k];
    for (int k = 0; k < 4; ++k)
      w[k] -= (d.fw[4 * fj[0] + k] * sg[0] + d.fw[4 * fj[1] + k] * sg[1] +
               d.fw[4 * fj[2] + k] * sg[2]) / area;
    double pn[4];
    conserve_prim<false>(w, 4, d.gamma, pn);
    for (int k = 0; k < 4; ++k) {
      p[k] = pn[k];
      cr[k] = (w[k] - wo[k]) * (w[k] - wo[k]);
      cr[4 + k] = fabs(w[k]);
    }
    if (!(pn[0] > 0.0) || !(pn[3] > 0.0) || !isfinite(pn[0]) || !isfinite(pn[3])) atomicOr(d.status, 1);
    const double tau = d.mu_ref * 2.0 * pow(pn[3], 1.0 - d.omega) / pn[0];
    for (int k = 0; k < 4; ++k) sh[k] = pn[k];
    sh[4] = dt / tau;
  }
  __syncthreads();
  const double rho = sh[0], U = sh[1], V = sh[2], lam = sh[3], k = sh[4];
  const double rn = rho * (lam / PI), cB = d.K / (2.0 * lam);
  const double orn = rho_o * (lam_o / PI), ocB = d.K / (2.0 * lam_o);
  const double sfac = 0.8 * (1.0 - d.Pr) * (lam_o * lam_o) / rho_o;
  const R* F0h = (const R*)d.fh + (long)fj[0] * d.vstride;
  const R* F1h = (const R*)d.fh + (long)fj[1] * d.vstride;
  const R* F2h = (const R*)d.fh + (long)fj[2] * d.vstride;
  const R* F0b = (const R*)d.fb + (long)fj[0] * d.vstride;
  const R* F1b = (const R*)d.fb + (long)fj[1] * d.vstride;
  const R* F2b = (const R*)d.fb + (long)fj[2] * d.vstride;
  for (int v = threadIdx.x; v < d.nvel; v += US_T) {
    const double u = d.u[v], vv = d.v[v];
    const double du = u - U, dv = vv - V;
    double MH = rn * exp(-lam * (du * du + dv * dv));
    double MB = MH * cB;
    if (shak) {
      const double cu = u - U_o, cv = vv - V_o, c2 = cu * cu + cv * cv;
      const double MHo = orn * exp(-lam_o * c2), MBo = MHo * ocB;
      const double fq = sfac * (cu * q0 + cv * q1);
      MH += fq * (2.0 * lam_o * c2 + d.K - 5.0) * MHo;
      MB += fq * (2.0 * lam_o * c2 + d.K - 3.0) * MBo;
    }
    const double dh = ((double)F0h[v] * sg[0] + (double)F1h[v] * sg[1] + (double)F2h[v] * sg[2]) / area;
    const double db = ((double)F0b[v] * sg[0] + (double)F1b[v] * sg[1] + (double)F2b[v] * sg[2]) / area;
    H[v] = R(((double)H[v] - dh + k * MH) / (1.0 + k));
    B[v] = R(((double)B[v] - db + k * MB) / (1.0 + k));
  }
}

// update_boundary! US2F (src/Solver/update_boundary.jl:575-594): each
// extrapolated cell becomes the mean of its two neighbours, in cell order
// (a later cell sees the new value of an earlier one), one CTA in sequence.
template <typename R>
__global__ void __launch_bounds__(US_T) k_us_avg(UsDev d) {
  for (int a = 0; a < d.navg; ++a) {
    const int c = d.avg_list[a];
    int id[2] = {c, c}, m = 0;
    for (int j = 0; j < 3; ++j)
      if (d.cell_nb[3 * c + j] != -1 && m < 2) id[m++] = d.cell_nb[3 * c + j];
    if (threadIdx.x == 0) {
      double* w = d.w + 4L * c;
      for (int k = 0; k < 4; ++k) w[k] = 0.5 * (d.w[4L * id[0] + k] + d.w[4L * id[1] + k]);
      double pn[4];
      conserve_prim<false>(w, 4, d.gamma, pn);
      for (int k = 0; k < 4; ++k) d.prim[4L * c + k] = pn[k];
    }
    R* H = (R*)d.h;
    R* B = (R*)d.b;
    const long o = (long)c * d.vstride, o0 = (long)id[0] * d.vstride, o1 = (long)id[1] * d.vstride;
    for (int v = threadIdx.x; v < d.nvel; v += US_T) {
      H[o + v] = R(0.5 * ((double)H[o0 + v] + (double)H[o1 + v]));
      B[o + v] = R(0.5 * ((double)B[o0 + v] + (double)B[o1 + v]));
    }
    __syncthreads();
  }
}

// residual of update! US2F: sqrt(sum (w - w_old)^2 * ncell) / (sum |w| + 1e-7)
// over the stepped cells (src/Solver/solver_update.jl:465-467); chunked sums
// in cell order, then a fixed tree (deterministic)
__global__ void __launch_bounds__(US_T) k_us_residual(UsDev d) {
  __shared__ double red[US_T];
  const int per = (d.ncell + US_T - 1) / US_T;
  const int c0 = threadIdx.x * per, c1 = min(d.ncell, c0 + per);
  for (int k = 0; k < 4; ++k) {
    double r = 0.0, a = 0.0;
    for (int c = c0; c < c1; ++c) {
      r += d.cres[8L * c + k];
      a += d.cres[8L * c + 4 + k];
    }
    const double Rs = us_block_sum(r, red), As = us_block_sum(a, red);
    if (threadIdx.x == 0) d.residual[k] = sqrt(Rs * d.ncell) / (As + 1.e-7);
  }
}

// timestep for unstructured cells (src/Solver/solver_main.jl:398-420):
// max over cells of sqrt(umax^2 + vmax^2) / min(dx), umax = u1 + c.
__global__ void k_us_tmax(UsDev d) {
  __shared__ double red[256];
  double m = 0.0;
  for (int c = blockIdx.x * blockDim.x + threadIdx.x; c < d.ncell; c += gridDim.x * blockDim.x) {
    const double sos = pow(0.5 * d.gamma / d.prim[4L * c + 3], 0.5);
    const double um = d.umax + sos, vm = d.vmax + sos;
    m = fmax(m, sqrt(um * um + vm * vm) / d.cell_mindx[c]);
  }
  red[threadIdx.x] = m;
  __syncthreads();
  for (int s = 128; s >= 1; s >>= 1) {
    if (threadIdx.x < s) red[threadIdx.x] = fmax(red[threadIdx.x], red[threadIdx.x + s]);
    __syncthreads();
  }
  if (threadIdx.x == 0)
    atomicMax((unsigned long long*)d.tmax, (unsigned long long)__double_as_longlong(red[0]));
}

template <typename R>
__global__ void k_us_in(R* dst, const double* src, long ncell, int nvel, int vstride) {
  const long c = blockIdx.x;
  for (int v = threadIdx.x; v < vstride; v += blockDim.x)
    dst[c * vstride + v] = v < nvel ? R(src[c * nvel + v]) : R(0);
}
template <typename R>
__global__ void k_us_out(double* dst, const R* src, long ncell, int nvel, int vstride) {
  const long c = blockIdx.x;
  for (int v = threadIdx.x; v < nvel; v += blockDim.x) dst[c * nvel + v] = (double)src[c * vstride + v];
}

}  // namespace kb

struct kb_us {
  kb::UsDev d;
  int prec = 0;
  cudaStream_t stream = nullptr;
  std::vector<void*> allocs;
  int64_t launches = 0;
  double* stage = nullptr;
};

static int usfail(int code, const std::string& m) {
  kb::set_error(m);
  return code;
}

static int usalloc(kb_us* U, void** p, size_t bytes) {
  if (cudaMalloc(p, bytes ? bytes : 16) != cudaSuccess) {
    cudaGetLastError();
    return usfail(KB_ERR_NOMEM, "unstructured solve: cudaMalloc failed");
  }
  U->allocs.push_back(*p);
  return KB_OK;
}

extern "C" int kb_us_destroy(kb_us_t* U) {
  if (!U) return KB_OK;
  if (U->stream) cudaStreamSynchronize(U->stream);
  for (void* p : U->allocs) cudaFree(p);
  if (U->stream) cudaStreamDestroy(U->stream);
  delete U;
  return KB_OK;
}

extern "C" int kb_us_create(const kb_config_t* cfg, int32_t ncell, int32_t nface,
                            const int32_t* face_cells, const int32_t* cell_faces,
                            const int32_t* cell_nb, const int32_t* cell_type,
                            const double* face_n, const double* face_len, const double* cell_area,
                            const double* cell_mindx, const double* u, const double* v,
                            const double* weights, kb_us_t** out) {
  if (!cfg || !out || !face_cells || !cell_faces || !cell_nb || !cell_type || !face_n ||
      !face_len || !cell_area || !cell_mindx || !u || !v || !weights || ncell < 1 || nface < 3)
    return usfail(KB_ERR_ARG, "kb_us_create: null argument or empty mesh");
  if (cfg->dim != 2 || cfg->nf == 1) return usfail(KB_ERR_CONFIG, "unstructured solves are 2D2F2V");
  if (cfg->flux != KB_FLUX_KFVS)
    return usfail(KB_ERR_CONFIG, "unstructured solves use KFVS (evolve! US2F computes fluxes for :kfvs only)");
  if (cfg->interp_order != 1)
    return usfail(KB_ERR_CONFIG,
                  "unstructured solves are first order: the reference's slopes divide by the x / y "
                  "offsets of neighbouring cell centres (reconstruct4!), which vanish on general meshes");
  if (cfg->collision < 0 || cfg->collision > 1) return usfail(KB_ERR_CONFIG, "unknown collision");
  if (cfg->precision != KB_PREC_FP64 && cfg->precision != KB_PREC_FP32)
    return usfail(KB_ERR_CONFIG, "unknown precision");
  if (cfg->nu < 1 || cfg->nv < 1) return usfail(KB_ERR_CONFIG, "empty velocity grid");
  if (!(cfg->gamma > 1.0) || !(cfg->mu_ref > 0.0)) return usfail(KB_ERR_CONFIG, "invalid gas properties");
  for (int f = 0; f < nface; ++f)
    if (face_cells[2 * f] < 0 || face_cells[2 * f] >= ncell || face_cells[2 * f + 1] < -1 ||
        face_cells[2 * f + 1] >= ncell)
      return usfail(KB_ERR_ARG, "face_cells out of range");
  std::vector<int> avg;
  for (int c = 0; c < ncell; ++c) {
    const int t = cell_type[c];
    if (t == 2)
      return usfail(KB_ERR_CONFIG,
                    "cell type 2 (Maxwell wall) is not offered: the reference's US2F evolve! calls "
                    "flux_boundary_maxwell! with an argument list no method takes");
    if (t != 0 && t != 1 && t != 3) return usfail(KB_ERR_CONFIG, "cell types are 0, 1 or 3");
    int nb = 0;
    for (int j = 0; j < 3; ++j) {
      const int f = cell_faces[3 * c + j];
      if (f < 0 || f >= nface) return usfail(KB_ERR_ARG, "cell_faces out of range");
      if (face_cells[2 * f] != c && face_cells[2 * f + 1] != c)
        return usfail(KB_ERR_ARG, "cell_faces and face_cells disagree");
      if (cell_nb[3 * c + j] < -1 || cell_nb[3 * c + j] >= ncell)
        return usfail(KB_ERR_ARG, "cell_neighbors out of range");
      nb += cell_nb[3 * c + j] >= 0;
    }
    if (t == 0 && nb != 3) return usfail(KB_ERR_CONFIG, "a stepped cell (type 0) needs three neighbours");
    if (t == 3) {
      if (nb < 2) return usfail(KB_ERR_CONFIG, "an extrapolated cell (type 3) needs two neighbours");
      avg.push_back(c);
    }
  }
  kb_us* U = new kb_us();
  kb::UsDev& d = U->d;
  U->prec = cfg->precision;
  d.ncell = ncell;
  d.nface = nface;
  d.nvel = cfg->nu * cfg->nv;
  d.vstride = (d.nvel + 3) / 4 * 4;
  d.coll = cfg->collision;
  d.navg = (int)avg.size();
  d.K = cfg->K;
  d.gamma = cfg->gamma;
  d.mu_ref = cfg->mu_ref;
  d.omega = cfg->omega;
  d.Pr = cfg->Pr;
  d.umax = cfg->umax;
  d.vmax = cfg->vmax;
  auto bail = [&](int rc) {
    kb_us_destroy(U);
    return rc;
  };
  if (cudaStreamCreateWithFlags(&U->stream, cudaStreamNonBlocking) != cudaSuccess)
    return bail(usfail(KB_ERR_CUDA, "cudaStreamCreate failed"));
  const size_t esz = U->prec == KB_PREC_FP64 ? 8 : 4;
  void* p;
  int rc;
#define USALLOC(dst, T, count)                                                        \
  if ((rc = usalloc(U, &p, sizeof(T) * (size_t)(count))) != KB_OK) return bail(rc); \
  dst = (T*)p;
  int *fc, *cf, *nbp, *ct, *al, *st;
  double *fn, *fl, *ca, *cm, *du, *dv, *dw, *tm, *res;
  USALLOC(fc, int, 2 * nface);
  USALLOC(cf, int, 3 * ncell);
  USALLOC(nbp, int, 3 * ncell);
  USALLOC(ct, int, ncell);
  USALLOC(al, int, avg.size() + 1);
  USALLOC(st, int, 1);
  USALLOC(fn, double, 2 * nface);
  USALLOC(fl, double, nface);
  USALLOC(ca, double, ncell);
  USALLOC(cm, double, ncell);
  USALLOC(du, double, d.nvel);
  USALLOC(dv, double, d.nvel);
  USALLOC(dw, double, d.nvel);
  USALLOC(tm, double, 1);
  USALLOC(res, double, 4);
  USALLOC(d.w, double, 4L * ncell);
  USALLOC(d.prim, double, 4L * ncell);
  USALLOC(d.fw, double, 4L * nface);
  USALLOC(d.cres, double, 8L * ncell);
  USALLOC(U->stage, double, (long)ncell * d.nvel);
#undef USALLOC
  for (void** q : {&d.h, &d.b})
    if ((rc = usalloc(U, q, esz * (size_t)ncell * d.vstride)) != KB_OK) return bail(rc);
  for (void** q : {&d.fh, &d.fb})
    if ((rc = usalloc(U, q, esz * (size_t)nface * d.vstride)) != KB_OK) return bail(rc);
  bool ok = true;
  auto up = [&](void* dst, const void* src, size_t bytes) {
    ok &= cudaMemcpy(dst, src, bytes, cudaMemcpyHostToDevice) == cudaSuccess;
  };
  up(fc, face_cells, sizeof(int) * 2 * nface);
  up(cf, cell_faces, sizeof(int) * 3 * ncell);
  up(nbp, cell_nb, sizeof(int) * 3 * ncell);
  up(ct, cell_type, sizeof(int) * ncell);
  if (!avg.empty()) up(al, avg.data(), sizeof(int) * avg.size());
  up(fn, face_n, sizeof(double) * 2 * nface);
  up(fl, face_len, sizeof(double) * nface);
  up(ca, cell_area, sizeof(double) * ncell);
  up(cm, cell_mindx, sizeof(double) * ncell);
  up(du, u, sizeof(double) * d.nvel);
  up(dv, v, sizeof(double) * d.nvel);
  up(dw, weights, sizeof(double) * d.nvel);
  ok &= cudaMemset(st, 0, sizeof(int)) == cudaSuccess;
  ok &= cudaMemset(d.cres, 0, sizeof(double) * 8L * ncell) == cudaSuccess;
  if (!ok) return bail(usfail(KB_ERR_CUDA, "kb_us_create: copy failed"));
  d.face_cells = fc;
  d.cell_faces = cf;
  d.cell_nb = nbp;
  d.cell_type = ct;
  d.avg_list = al;
  d.status = st;
  d.face_n = fn;
  d.face_len = fl;
  d.cell_area = ca;
  d.cell_mindx = cm;
  d.u = du;
  d.v = dv;
  d.wt = dw;
  d.tmax = tm;
  d.residual = res;
  *out = U;
  return KB_OK;
}

extern "C" int kb_us_upload(kb_us_t* U, const double* w, const double* prim, const double* h,
                            const double* b) {
  if (!U || !w || !prim || !h || !b) return usfail(KB_ERR_ARG, "kb_us_upload: null argument");
  const kb::UsDev& d = U->d;
  bool ok = cudaMemcpy(d.w, w, sizeof(double) * 4L * d.ncell, cudaMemcpyHostToDevice) == cudaSuccess &&
            cudaMemcpy(d.prim, prim, sizeof(double) * 4L * d.ncell, cudaMemcpyHostToDevice) == cudaSuccess;
  for (int k = 0; k < 2 && ok; ++k) {
    ok &= cudaMemcpy(U->stage, k == 0 ? h : b, sizeof(double) * (size_t)d.ncell * d.nvel,
                     cudaMemcpyHostToDevice) == cudaSuccess;
    void* dst = k == 0 ? d.h : d.b;
    if (U->prec == KB_PREC_FP64)
      kb::k_us_in<double><<<d.ncell, 128, 0, U->stream>>>((double*)dst, U->stage, d.ncell, d.nvel, d.vstride);
    else
      kb::k_us_in<float><<<d.ncell, 128, 0, U->stream>>>((float*)dst, U->stage, d.ncell, d.nvel, d.vstride);
    U->launches++;
    ok &= cudaStreamSynchronize(U->stream) == cudaSuccess;
  }
  ok &= cudaMemset(d.status, 0, sizeof(int)) == cudaSuccess;
  if (!ok) return usfail(KB_ERR_CUDA, "kb_us_upload failed");
  return KB_OK;
}

extern "C" int kb_us_download(kb_us_t* U, double* w, double* prim, double* h, double* b) {
  if (!U) return usfail(KB_ERR_ARG, "kb_us_download: null handle");
  const kb::UsDev& d = U->d;
  bool ok = cudaStreamSynchronize(U->stream) == cudaSuccess;
  if (w) ok &= cudaMemcpy(w, d.w, sizeof(double) * 4L * d.ncell, cudaMemcpyDeviceToHost) == cudaSuccess;
  if (prim) ok &= cudaMemcpy(prim, d.prim, sizeof(double) * 4L * d.ncell, cudaMemcpyDeviceToHost) == cudaSuccess;
  for (int k = 0; k < 2 && ok; ++k) {
    double* dst = k == 0 ? h : b;
    if (!dst) continue;
    const void* src = k == 0 ? d.h : d.b;
    if (U->prec == KB_PREC_FP64)
      kb::k_us_out<double><<<d.ncell, 128, 0, U->stream>>>(U->stage, (const double*)src, d.ncell, d.nvel, d.vstride);
    else
      kb::k_us_out<float><<<d.ncell, 128, 0, U->stream>>>(U->stage, (const float*)src, d.ncell, d.nvel, d.vstride);
    U->launches++;
    ok &= cudaStreamSynchronize(U->stream) == cudaSuccess;
    ok &= cudaMemcpy(dst, U->stage, sizeof(double) * (size_t)d.ncell * d.nvel, cudaMemcpyDeviceToHost) ==
          cudaSuccess;
  }
  if (!ok) return usfail(KB_ERR_CUDA, "kb_us_download failed");
  return KB_OK;
}

extern "C" int kb_us_timestep(kb_us_t* U, double cfl, double sim_time, double max_time,
                              double* dt_out) {
  if (!U || !dt_out) return usfail(KB_ERR_ARG, "kb_us_timestep: null argument");
  const kb::UsDev& d = U->d;
  bool ok = cudaMemsetAsync(d.tmax, 0, sizeof(double), U->stream) == cudaSuccess;
  kb::k_us_tmax<<<(d.ncell + 255) / 256, 256, 0, U->stream>>>(d);
  U->launches++;
  double tmax = 0.0;
  ok &= cudaStreamSynchronize(U->stream) == cudaSuccess;
  ok &= cudaMemcpy(&tmax, d.tmax, sizeof(double), cudaMemcpyDeviceToHost) == cudaSuccess;
  if (!ok || !(tmax > 0.0)) return usfail(KB_ERR_CUDA, "kb_us_timestep failed");
  const double dt = cfl / tmax;
  *dt_out = dt < max_time - sim_time ? dt : max_time - sim_time;
  return KB_OK;
}

extern "C" int kb_us_step(kb_us_t* U, double dt, int32_t nsteps, double* residual) {
  if (!U || nsteps < 0) return usfail(KB_ERR_ARG, "kb_us_step: bad argument");
  const kb::UsDev& d = U->d;
  for (int s = 0; s < nsteps; ++s) {
    if (U->prec == KB_PREC_FP64) {
      kb::k_us_face<double><<<d.nface, kb::US_T, 0, U->stream>>>(d, dt);
      kb::k_us_cell<double><<<d.ncell, kb::US_T, 0, U->stream>>>(d, dt);
      if (d.navg) kb::k_us_avg<double><<<1, kb::US_T, 0, U->stream>>>(d);
    } else {
      kb::k_us_face<float><<<d.nface, kb::US_T, 0, U->stream>>>(d, dt);
      kb::k_us_cell<float><<<d.ncell, kb::US_T, 0, U->stream>>>(d, dt);
      if (d.navg) kb::k_us_avg<float><<<1, kb::US_T, 0, U->stream>>>(d);
    }
    U->launches += d.navg ? 3 : 2;
  }
  kb::k_us_residual<<<1, kb::US_T, 0, U->stream>>>(d);
  U->launches++;
  if (cudaStreamSynchronize(U->stream) != cudaSuccess)
    return usfail(KB_ERR_CUDA, std::string("kb_us_step: ") + cudaGetErrorString(cudaGetLastError()));
  int st = 0;
  cudaMemcpy(&st, d.status, sizeof(int), cudaMemcpyDeviceToHost);
  if (residual) cudaMemcpy(residual, d.residual, sizeof(double) * 4, cudaMemcpyDeviceToHost);
  if (st) return usfail(KB_ERR_NUMERIC, "non-finite or non-positive density / lambda in an unstructured solve");
  return KB_OK;
}

extern "C" int kb_us_info(kb_us_t* U, int64_t* launches) {
  if (!U || !launches) return usfail(KB_ERR_ARG, "kb_us_info: null argument");
  *launches = U->launches;
  return KB_OK;
}
