// kb_kernels.cu -- sm_103a kernels of the DVM time step (1D2F1V, 2D2F2V).
//
// One step is: [w slopes] -> [face parameters] -> face moments (fw) ->
// [Maxwell walls] -> [Shakhov heat flux] -> cell parameters (w, prim, tau,
// residual partials) -> pointwise update of h, b -> [ghost fill] -> residual.
// The pointwise face fluxes fh, fb are never stored: the update kernel forms
// them again from the neighbour cells, so h and b are read from HBM and
// written once per step apart from stencil re-reads that hit L2.
#include <cuda_runtime.h>
#include <stdio.h>

#include "kb_kernels.cuh"

namespace kb {

// ----------------------------------------------------------------- helpers

__host__ __device__ inline int face_count(const Geo& g) {
  return (g.nx + 1) * g.ny + (g.D == 2 ? g.nx * (g.ny + 1) : 0);
}

// Face f -> direction d, left cell, right cell (cell indices incl. ghosts),
// index i (x position of the face / cell), j, and the step between cells along d.
struct FaceGeo {
  int d, cL, cR, step, iL, iR;  // iL/iR: index along d of the two cells
  int fi, fj;                   // face coordinates
};
__host__ __device__ inline FaceGeo face_geo(const Geo& g, int f) {
  FaceGeo r;
  int nfx = (g.nx + 1) * g.ny;
  if (f < nfx) {
    r.d = 0;
    r.fi = f % (g.nx + 1);
    r.fj = f / (g.nx + 1);
    r.cL = cell_index(g, r.fi - 1, r.fj);
    r.cR = r.cL + 1;
    r.step = 1;
    r.iL = r.fi - 1;
    r.iR = r.fi;
  } else {
    int q = f - nfx;
    r.d = 1;
    r.fi = q % g.nx;
    r.fj = q / g.nx;
    r.cL = cell_index(g, r.fi, r.fj - 1);
    r.cR = cell_index(g, r.fi, r.fj);
    r.step = g.nxt;
    r.iL = r.fj - 1;
    r.iR = r.fj;
  }
  return r;
}

// Face length: vertex distance of PSpace2D (src/Geometry/geo_struct.jl:101-107);
// for x faces it depends on the row, for y faces on the column.
__host__ __device__ inline double face_len(const Geo& g, int d, int fi, int fj) {
  if (g.D == 1) return 1.0;
  if (d == 0) {
    double y = g.y0 + (fj + 1 - 0.5) * g.dy;
    return fabs((y + 0.5 * g.dy) - (y - 0.5 * g.dy));
  }
  double x = g.x0 + (fi + 1 - 0.5) * g.dx;
  return fabs((x + 0.5 * g.dx) - (x - 0.5 * g.dx));
}

// Classification of every face (0 not computed, 1 interior flux, 2 Maxwell wall):
// evolve! computes faces idx0:idx1 (all faces when ghosts exist, interior
// faces otherwise; src/Solver/solver_evolution.jl:64-89, :608-679) and
// evolve_boundary! replaces the wall faces (src/Solver/evolve_boundary.jl).
void face_kinds_host(const Geo& g, signed char* kind) {
  int n = face_count(g);
  for (int f = 0; f < n; ++f) {
    FaceGeo r = face_geo(g, f);
    int pos = r.d == 0 ? r.fi : r.fj;
    int nn = r.d == 0 ? g.nx : g.ny;
    int ng = r.d == 0 ? g.ngx : g.ngy;
    signed char k = 1;
    if ((pos == 0 || pos == nn) && ng == 0) k = 0;
    int side = r.d == 0 ? (pos == 0 ? 0 : (pos == nn ? 1 : -1)) : (pos == 0 ? 2 : (pos == nn ? 3 : -1));
    if (side >= 0 && g.bc[side] == BC_MAXWELL) k = 2;
    kind[f] = k;
  }
}

template <typename R>
__device__ __forceinline__ R dscale(double d);
template <>
__device__ __forceinline__ double dscale<double>(double d) { return d; }
template <>
__device__ __forceinline__ float dscale<float>(double d) { return float(1.0 / d); }

template <typename R>
__device__ __forceinline__ const R* vtab(const DevState& s, int which);
template <>
__device__ __forceinline__ const double* vtab<double>(const DevState& s, int which) {
  return which == 0 ? s.u : (which == 1 ? s.v : s.wt);
}
template <>
__device__ __forceinline__ const float* vtab<float>(const DevState& s, int which) {
  return which == 0 ? s.uf : (which == 1 ? s.vf : s.wtf);
}

// Upwind face state of one distribution at one velocity: the reconstructed
// value of the upwind cell (h + s dx/2 from the left, h - s dx/2 from the
// right) and that cell's slope (flux_kfvs.jl:35-63 / :98-140 wrappers).
template <typename R>
__device__ __forceinline__ R upwind_state(const R* __restrict__ q, long vs, int up, int step,
                                          int rule, bool left, int v, R dsc, R dxh, R& slope) {
  R q0 = q[(long)up * vs + v];
  R qm = (rule == 1 || rule == 3) ? q[(long)(up - step) * vs + v] : R(0);
  R qp = (rule == 1 || rule == 2) ? q[(long)(up + step) * vs + v] : R(0);
  R s = slope_of<R>(rule, qm, q0, qp, dsc);
  slope = s;
  return left ? q0 + s * dxh : q0 - s * dxh;
}

// Per-face coefficients in the storage precision.
template <typename R>
struct FP {
  R rho_n, U, V, lam, cB, Mxi2, len;
  R Mt[5];
  R aL[4], aR[4], aT[4];
};
template <typename R>
__device__ __forceinline__ FP<R> load_fp(const DevState& s, int f);
template <>
__device__ __forceinline__ FP<double> load_fp<double>(const DevState& s, int f) {
  const FaceParam& p = s.fp[f];
  FP<double> r;
  double lam = p.prim[3];
  r.rho_n = s.g.D == 1 ? p.prim[0] * sqrt(lam / PI) : p.prim[0] * (lam / PI);
  r.U = p.prim[1];
  r.V = p.prim[2];
  r.lam = lam;
  r.cB = s.g.K / (2.0 * lam);
  r.Mxi2 = p.Mxi2;
  r.len = p.len;
  for (int k = 0; k < 5; ++k) r.Mt[k] = p.Mt[k];
  for (int k = 0; k < 4; ++k) {
    r.aL[k] = p.aL[k];
    r.aR[k] = p.aR[k];
    r.aT[k] = p.aT[k];
  }
  return r;
}
template <>
__device__ __forceinline__ FP<float> load_fp<float>(const DevState& s, int f) {
  const FaceParamF& p = s.fpf[f];
  FP<float> r;
  r.rho_n = p.rho_n;
  r.U = p.U;
  r.V = p.V;
  r.lam = p.lam;
  r.cB = p.cB;
  r.Mxi2 = p.Mxi2;
  r.len = p.len;
  for (int k = 0; k < 5; ++k) r.Mt[k] = p.Mt[k];
  for (int k = 0; k < 4; ++k) {
    r.aL[k] = p.aL[k];
    r.aR[k] = p.aR[k];
    r.aT[k] = p.aT[k];
  }
  return r;
}

// Pointwise interface flux at one velocity (face-local frame).  Returns the
// full fluxes fh, fb and the transport parts Th, Tb whose moments form the
// discrete part of fw.
//   KFVS  flux_kfvs.jl:303-337 (1D), :654-700 (2D)
//   KCU   flux_kcu.jl:463-530 (1D), :898-970 (2D)
//   UGKS  flux_ugks.jl:8-114 (1D), :121-253 (2D)
template <typename R, int FLUX, int D>
__device__ __forceinline__ void face_flux(const FP<R>& P, R dt, R un, R ut, bool pos, R h, R b,
                                          R sh, R sb, R& fh, R& fb, R& Th, R& Tb) {
  if (FLUX == FLUX_KFVS) {
    R a = dt * un;
    R c = R(0.5) * (dt * dt) * (un * un);
    fh = a * h - c * sh;
    fb = a * b - c * sb;
    if (D == 2) {
      fh *= P.len;
      fb *= P.len;
    }
    Th = fh;
    Tb = fb;
  } else {
    R du = un - P.U;
    R e = du * du;
    if (D == 2) {
      R dv = ut - P.V;
      e += dv * dv;
    }
    R H = P.rho_n * mexp(-P.lam * e);
    R B = H * P.cB;
    if (FLUX == FLUX_KCU) {
      Th = P.Mt[1] * un * h;
      Tb = P.Mt[1] * un * b;
      fh = P.Mt[0] * un * H + Th;
      fb = P.Mt[0] * un * B + Tb;
    } else {
      Th = P.Mt[3] * un * h - P.Mt[4] * (un * un) * sh;
      Tb = P.Mt[3] * un * b - P.Mt[4] * (un * un) * sb;
      const R* a = pos ? P.aL : P.aR;
      R c2 = un * un;
      if (D == 2) c2 += ut * ut;
      R lin = a[0] + a[1] * un;
      R linT = P.aT[0] + P.aT[1] * un;
      R aE = a[D + 1], tE = P.aT[D + 1];
      if (D == 2) {
        lin += a[2] * ut;
        linT += P.aT[2] * ut;
      }
      // (c2 H + B) = (c2 + cB) H ; (c2 B + Mxi2 H) = (cB c2 + Mxi2) H
      R ph = lin + R(0.5) * aE * (c2 + P.cB);
      R pT = linT + R(0.5) * tE * (c2 + P.cB);
      R pb = P.cB * lin + R(0.5) * aE * (P.cB * c2 + P.Mxi2);
      R pTb = P.cB * linT + R(0.5) * tE * (P.cB * c2 + P.Mxi2);
      R m2 = P.Mt[1] * (un * un);
      R m3 = P.Mt[2] * un;
      R m1 = P.Mt[0] * un;
      fh = H * (m1 + m2 * ph + m3 * pT) + Th;
      fb = H * (m1 * P.cB + m2 * pb + m3 * pTb) + Tb;
    }
    if (D == 2) {
      fh *= P.len;
      fb *= P.len;
    }
  }
}

// ------------------------------------------------------------ w slopes

// reconstruct! for w (src/Solver/solver_reconstruction.jl:111-122 1D, :496-537 2D):
// one thread per (physical cell, direction).
__global__ void k_wslope(DevState s) {
  const Geo& g = s.g;
  int t = blockIdx.x * blockDim.x + threadIdx.x;
  int n = g.nx * g.ny;
  if (t >= n * g.D) return;
  int d = t / n, c0 = t % n;
  int i = c0 % g.nx, j = c0 / g.nx;
  int c = cell_index(g, i, j);
  int rule = slope_rule(g, d, d == 0 ? i : j);
  int step = d == 0 ? 1 : g.nxt;
  double dd = d == 0 ? g.dx : g.dy;  // 0.5 * (dx[i-1] + dx[i]) on a uniform mesh
  double* out = s.sw + ((long)c * 2 + d) * 4;
  for (int k = 0; k < g.NW; ++k) {
    double q0 = s.w[(long)c * 4 + k];
    double qm = (rule == 1 || rule == 3) ? s.w[(long)(c - step) * 4 + k] : 0.0;
    double qp = (rule == 1 || rule == 2) ? s.w[(long)(c + step) * 4 + k] : 0.0;
    out[k] = slope_of<double>(rule, qm, q0, qp, dd);
  }
}

// ------------------------------------------------------- face parameters

// Interface equilibrium from the two half Maxwellians (flux_kcu.jl:480-495,
// flux_ugks.jl:47-56), then the KCU / UGKS time integrals, UGKS slopes and
// the analytic part of fw.  One thread per face.
template <int FLUX>
__global__ void k_face_param(DevState s, double dt) {
  const Geo& g = s.g;
  int f = blockIdx.x * blockDim.x + threadIdx.x;
  if (f >= s.nface_x + s.nface_y) return;
  if (s.kind[f] != 1) return;
  FaceGeo r = face_geo(g, f);
  int NW = g.NW;
  double dxh = 0.5 * (r.d == 0 ? g.dx : g.dy);
  double len = face_len(g, r.d, r.fi, r.fj);
  FaceParam P;
  for (int k = 0; k < 4; ++k) {
    P.prim[k] = 0;
    P.aL[k] = P.aR[k] = P.aT[k] = P.fwa[k] = 0;
  }
  for (int k = 0; k < 5; ++k) P.Mt[k] = 0;
  P.len = len;
  P.Mxi2 = 0;
  P.pad = 0;
  if (FLUX == FLUX_KFVS) {
    P.mult = 1.0;
  } else {
    // face states of w (local frame): w + dx/2 sw from the left, w - dx/2 sw from the right
    double wl[4], wr[4], wL[4], wR[4];
    const double* sl = s.sw + ((long)r.cL * 2 + r.d) * 4;
    const double* sr = s.sw + ((long)r.cR * 2 + r.d) * 4;
    for (int k = 0; k < 4; ++k) {
      wl[k] = k < NW ? s.w[(long)r.cL * 4 + k] + dxh * sl[k] : 0.0;
      wr[k] = k < NW ? s.w[(long)r.cR * 4 + k] - dxh * sr[k] : 0.0;
    }
    if (NW == 4 && r.d == 1) {  // local_frame with n = (0, 1)
      wL[0] = wl[0]; wL[1] = wl[2]; wL[2] = -wl[1]; wL[3] = wl[3];
      wR[0] = wr[0]; wR[1] = wr[2]; wR[2] = -wr[1]; wR[3] = wr[3];
    } else {
      for (int k = 0; k < 4; ++k) { wL[k] = wl[k]; wR[k] = wr[k]; }
    }
    double pL[4], pR[4], wi[4], p[4], M1[4], M2[4];
    conserve_prim(wL, NW, g.gamma, pL);
    conserve_prim(wR, NW, g.gamma, pR);
    GM m;
    gauss_moments(pL, NW, g.K, m);
    moments_conserve(m.MuL, m.Mv, m.Mxi, NW, 0, 0, 0, M1);
    gauss_moments(pR, NW, g.K, m);
    moments_conserve(m.MuR, m.Mv, m.Mxi, NW, 0, 0, 0, M2);
    for (int k = 0; k < 4; ++k) wi[k] = k < NW ? pL[0] * M1[k] + pR[0] * M2[k] : 0.0;
    conserve_prim(wi, NW, g.gamma, p);
    double lam = p[NW - 1];
    P.prim[0] = p[0];
    P.prim[1] = p[1];
    P.prim[2] = NW == 4 ? p[2] : 0.0;
    P.prim[3] = lam;
    double tau = vhs_time(p[0], lam, g.mu_ref, g.omega);
    GM mi;
    if (FLUX == FLUX_KCU) {
      tau += fabs(pL[0] / pL[NW - 1] - pR[0] / pR[NW - 1]) /
             (pL[0] / pL[NW - 1] + pR[0] / pR[NW - 1]) * dt * 2.0;
      P.Mt[1] = tau * (1.0 - exp(-dt / tau));
      P.Mt[0] = dt - P.Mt[1];
      gauss_moments(p, NW, g.K, mi);
      double Muv[4];
      moments_conserve(mi.Mu, mi.Mv, mi.Mxi, NW, 1, 0, 0, Muv);
      for (int k = 0; k < NW; ++k) P.fwa[k] = P.Mt[0] * p[0] * Muv[k] * len;
      P.mult = len;
    } else {
      double dL[4], dR[4];
      for (int k = 0; k < 4; ++k) {
        dL[k] = k < NW ? (wi[k] - wL[k]) / dxh : 0.0;
        dR[k] = k < NW ? (wR[k] - wi[k]) / dxh : 0.0;
      }
      double aL[4], aR[4], aT[4];
      pdf_slope(p, dL, NW, g.K, aL);
      pdf_slope(p, dR, NW, g.K, aR);
      gauss_moments(p, NW, g.K, mi);
      double MauL[4], MauR[4], MauT[4], Muv[4], tmp[4];
      moments_conserve_slope(aL, mi.MuL, mi.Mv, mi.Mxi, NW, 1, MauL);
      moments_conserve_slope(aR, mi.MuR, mi.Mv, mi.Mxi, NW, 1, MauR);
      for (int k = 0; k < 4; ++k) tmp[k] = -p[0] * (MauL[k] + MauR[k]);
      pdf_slope(p, tmp, NW, g.K, aT);
      double ex = exp(-dt / tau);
      double Mt[5];
      Mt[3] = tau * (1.0 - ex);
      Mt[4] = -tau * dt * ex + tau * Mt[3];
      Mt[0] = dt - Mt[3];
      Mt[1] = -tau * Mt[0] + Mt[4];
      Mt[2] = (dt * dt) / 2.0 - tau * Mt[0];
      moments_conserve(mi.Mu, mi.Mv, mi.Mxi, NW, 1, 0, 0, Muv);
      moments_conserve_slope(aL, mi.MuL, mi.Mv, mi.Mxi, NW, 2, MauL);
      moments_conserve_slope(aR, mi.MuR, mi.Mv, mi.Mxi, NW, 2, MauR);
      moments_conserve_slope(aT, mi.Mu, mi.Mv, mi.Mxi, NW, 1, MauT);
      for (int k = 0; k < NW; ++k)
        P.fwa[k] = (Mt[0] * p[0] * Muv[k] + Mt[1] * p[0] * (MauL[k] + MauR[k]) +
                    Mt[2] * p[0] * MauT[k]) * len;
      for (int k = 0; k < 5; ++k) P.Mt[k] = Mt[k];
      // slopes stored with the energy slope at index D+1 for both dimensions
      for (int k = 0; k < 4; ++k) {
        P.aL[k] = aL[k];
        P.aR[k] = aR[k];
        P.aT[k] = aT[k];
      }
      P.Mxi2 = mi.Mxi[2];
      P.mult = len;
    }
  }
  s.fp[f] = P;
  FaceParamF F;
  double lam = P.prim[3] > 0 ? P.prim[3] : 1.0;
  F.rho_n = float(g.D == 1 ? P.prim[0] * sqrt(lam / PI) : P.prim[0] * (lam / PI));
  F.U = float(P.prim[1]);
  F.V = float(P.prim[2]);
  F.lam = float(P.prim[3]);
  F.cB = float(g.K / (2.0 * lam));
  for (int k = 0; k < 5; ++k) F.Mt[k] = float(P.Mt[k]);
  for (int k = 0; k < 4; ++k) {
    F.aL[k] = float(P.aL[k]);
    F.aR[k] = float(P.aR[k]);
    F.aT[k] = float(P.aT[k]);
  }
  F.Mxi2 = float(P.Mxi2);
  F.len = float(len);
  F.pad[0] = F.pad[1] = 0.f;
  s.fpf[f] = F;
}

// ------------------------------------------------------------ face moments

// fw of interior faces: analytic part + moments of the transport part of the
// pointwise flux (flux_conserve!, src/Theory/theory_moments.jl:376-416, and
// the fw updates of flux_kcu! / flux_ugks!), rotated to the global frame.
// One warp per face; lanes stride over velocities.
template <typename R, int D, int FLUX>
__global__ void __launch_bounds__(256) k_face_moments(DevState s, double dt) {
  const Geo& g = s.g;
  int f = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  int lane = threadIdx.x & 31;
  if (f >= s.nface_x + s.nface_y) return;
  if (s.kind[f] != 1) return;
  FaceGeo r = face_geo(g, f);
  FP<R> P = load_fp<R>(s, f);
  const R* H = (const R*)s.h[s.cur];
  const R* Bq = (const R*)s.b[s.cur];
  const R* U = vtab<R>(s, 0);
  const R* V = vtab<R>(s, 1);
  const R* W = vtab<R>(s, 2);
  long vs = g.vstride;
  int ruleL = slope_rule(g, r.d, r.iL), ruleR = slope_rule(g, r.d, r.iR);
  R dsc = dscale<R>(r.d == 0 ? g.dx : g.dy);
  R dxh = R(0.5 * (r.d == 0 ? g.dx : g.dy));
  R rdt = R(dt);
  Acc<R> a0, a1, a2, a3;
  for (int v = lane; v < g.nvel; v += 32) {
    R un, ut;
    if (D == 1) {
      un = U[v];
      ut = R(0);
    } else if (r.d == 0) {
      un = U[v];
      ut = V[v];
    } else {
      un = V[v];
      ut = -U[v];
    }
    bool pos = un >= R(0);
    int up = pos ? r.cL : r.cR;
    int rule = pos ? ruleL : ruleR;
    R sh, sb;
    R h = upwind_state<R>(H, vs, up, r.step, rule, pos, v, dsc, dxh, sh);
    R b = upwind_state<R>(Bq, vs, up, r.step, rule, pos, v, dsc, dxh, sb);
    R fh, fb, Th, Tb;
    if (FLUX == FLUX_KFVS) {
      face_flux<R, FLUX, D>(P, rdt, un, ut, pos, h, b, sh, sb, fh, fb, Th, Tb);
    } else if (FLUX == FLUX_KCU) {
      Th = P.Mt[1] * un * h;
      Tb = P.Mt[1] * un * b;
    } else {
      Th = P.Mt[3] * un * h - P.Mt[4] * (un * un) * sh;
      Tb = P.Mt[3] * un * b - P.Mt[4] * (un * un) * sb;
    }
    R wT = W[v] * Th;
    a0.add(wT);
    a1.add(wT * un);
    R c2 = un * un;
    if (D == 2) {
      a2.add(wT * ut);
      c2 += ut * ut;
    }
    a3.add(wT * c2 + W[v] * Tb);
  }
  double S0 = a0.total(), S1 = a1.total(), S2 = D == 2 ? a2.total() : 0.0, S3 = a3.total();
  if (lane == 0) {
    const FaceParam& p = s.fp[f];
    double m = p.mult;
    double fl[4];
    if (D == 1) {
      fl[0] = p.fwa[0] + m * S0;
      fl[1] = p.fwa[1] + m * S1;
      fl[2] = p.fwa[2] + m * (0.5 * S3);
      fl[3] = 0.0;
    } else {
      fl[0] = p.fwa[0] + m * S0;
      fl[1] = p.fwa[1] + m * S1;
      fl[2] = p.fwa[2] + m * S2;
      fl[3] = p.fwa[3] + m * (0.5 * S3);
    }
    double* out = s.fw + (long)f * 4;
    if (D == 2 && r.d == 1) {  // global_frame with n = (0, 1)
      out[0] = fl[0];
      out[1] = -fl[2];
      out[2] = fl[1];
      out[3] = fl[3];
    } else {
      for (int k = 0; k < 4; ++k) out[k] = fl[k];
    }
  }
}

// ------------------------------------------------------------ Maxwell walls

// flux_boundary_maxwell! 1D2F1V (src/Flux/flux_boundary.jl:39-61) and 2D2F2V
// (:190-220) in the face-local frame; rot = +1 on the left / bottom wall and
// -1 on the right / top wall (src/Solver/evolve_boundary.jl).  One warp per
// wall face: pass 1 finds the wall density, pass 2 the moments of h_wall.
template <typename R, int D>
__global__ void __launch_bounds__(256) k_wall(DevState s, double dt) {
  const Geo& g = s.g;
  int f = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  int lane = threadIdx.x & 31;
  if (f >= s.nface_x + s.nface_y) return;
  if (s.kind[f] != 2) return;
  FaceGeo r = face_geo(g, f);
  int pos = r.d == 0 ? r.fi : r.fj;
  int rot = pos == 0 ? 1 : -1;
  int c = pos == 0 ? r.cR : r.cL;  // the interior cell next to the wall
  const double* wp = s.wall + (long)f * 4;
  double bw[4];
  if (D == 1) {
    bw[0] = wp[0]; bw[1] = wp[1]; bw[2] = 0.0; bw[3] = wp[2];
  } else if (r.d == 0) {
    bw[0] = wp[0]; bw[1] = wp[1]; bw[2] = wp[2]; bw[3] = wp[3];
  } else {
    bw[0] = wp[0]; bw[1] = wp[2]; bw[2] = -wp[1]; bw[3] = wp[3];
  }
  double lw = bw[3];
  const R* H = (const R*)s.h[s.cur];
  const R* Bq = (const R*)s.b[s.cur];
  const R* U = vtab<R>(s, 0);
  const R* V = vtab<R>(s, 1);
  const R* W = vtab<R>(s, 2);
  long vs = g.vstride;
  R Uw = R(bw[1]), Vw = R(bw[2]), Lw = R(lw);
  Acc<R> sf, sg;
  for (int v = lane; v < g.nvel; v += 32) {
    R un, ut;
    if (D == 1) { un = U[v]; ut = R(0); }
    else if (r.d == 0) { un = U[v]; ut = V[v]; }
    else { un = V[v]; ut = -U[v]; }
    bool in = un * R(rot) >= R(0);
    R du = un - Uw, e = du * du;
    if (D == 2) { R dv = ut - Vw; e += dv * dv; }
    if (in) sg.add(W[v] * un * mexp(-Lw * e));
    else sf.add(W[v] * un * H[(long)c * vs + v]);
  }
  double SF = sf.total(), SG = sg.total();
  SG *= D == 1 ? sqrt(lw / PI) : (lw / PI);
  double rho = -SF / SG;
  double len = D == 2 ? (r.d == 0 ? g.dy : g.dx) : 1.0;
  double sc = D == 2 ? len * dt : dt;
  R rn = R(D == 1 ? rho * sqrt(lw / PI) : rho * (lw / PI));
  R cB = R(g.K / (2.0 * lw));
  Acc<R> a0, a1, a2, a3;
  for (int v = lane; v < g.nvel; v += 32) {
    R un, ut;
    if (D == 1) { un = U[v]; ut = R(0); }
    else if (r.d == 0) { un = U[v]; ut = V[v]; }
    else { un = V[v]; ut = -U[v]; }
    bool in = un * R(rot) >= R(0);
    R hw, bwv;
    if (in) {
      R du = un - Uw, e = du * du;
      if (D == 2) { R dv = ut - Vw; e += dv * dv; }
      hw = rn * mexp(-Lw * e);
      bwv = hw * cB;
    } else {
      hw = H[(long)c * vs + v];
      bwv = Bq[(long)c * vs + v];
    }
    R t = W[v] * un * hw;
    a0.add(t);
    a1.add(t * un);
    R c2 = un * un;
    if (D == 2) { a2.add(t * ut); c2 += ut * ut; }
    a3.add(t * c2 + W[v] * un * bwv);
  }
  double S0 = a0.total(), S1 = a1.total(), S2 = D == 2 ? a2.total() : 0.0, S3 = a3.total();
  if (lane == 0) {
    s.rhow[f] = rho;
    double fl[4] = {S0 * sc, S1 * sc, 0.0, 0.0};
    if (D == 1) {
      fl[2] = 0.5 * S3 * sc;
    } else {
      fl[2] = S2 * sc;
      fl[3] = 0.5 * S3 * sc;
    }
    double* out = s.fw + (long)f * 4;
    if (D == 2 && r.d == 1) {
      out[0] = fl[0]; out[1] = -fl[2]; out[2] = fl[1]; out[3] = fl[3];
    } else {
      for (int k = 0; k < 4; ++k) out[k] = fl[k];
    }
  }
}

// ------------------------------------------------------- cell parameters

// Update group of a physical cell: 0 fixed (copied), 1 interior, 2 boundary
// (update! loops 2:nx-1 / 2:nx-1 x 2:ny-1, update_boundary! the rest when the
// side is not :fix; src/Solver/solver_update.jl, update_boundary.jl).
__device__ inline int update_group(const Geo& g, int i, int j) {
  if (g.D == 1) {
    if (i >= 1 && i <= g.nx - 2) return 1;
    if (i == 0 && g.bc[0] != BC_FIX) return 2;
    if (i == g.nx - 1 && g.bc[1] != BC_FIX) return 2;
    return 0;
  }
  if (i >= 1 && i <= g.nx - 2 && j >= 1 && j <= g.ny - 2) return 1;
  if (i == 0) return g.bc[0] != BC_FIX ? 2 : 0;
  if (i == g.nx - 1) return g.bc[1] != BC_FIX ? 2 : 0;
  if (j == 0) return g.bc[2] != BC_FIX ? 2 : 0;
  return g.bc[3] != BC_FIX ? 2 : 0;
}

// heat_flux 2F1V / 2F2V (src/Theory/theory_moments.jl:530-531, :567-578) of the
// old state.  One warp per updated cell (Shakhov only).
template <typename R, int D>
__global__ void __launch_bounds__(256) k_cell_q(DevState s) {
  const Geo& g = s.g;
  int t = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  int lane = threadIdx.x & 31;
  if (t >= g.nx * g.ny) return;
  int i = t % g.nx, j = t / g.nx;
  int grp = update_group(g, i, j);
  if (!grp) return;
  int coll = (D == 1 && grp == 2) ? COLL_BGK : s.coll;
  if (coll != COLL_SHAKHOV) return;
  int c = cell_index(g, i, j);
  const R* H = (const R*)s.h[s.cur] + (long)c * g.vstride;
  const R* Bq = (const R*)s.b[s.cur] + (long)c * g.vstride;
  const R* U = vtab<R>(s, 0);
  const R* V = vtab<R>(s, 1);
  const R* W = vtab<R>(s, 2);
  R Uc = R(s.prim[(long)c * 4 + 1]);
  R Vc = R(D == 2 ? s.prim[(long)c * 4 + 2] : 0.0);
  Acc<R> a0, a1;
  for (int v = lane; v < g.nvel; v += 32) {
    R cu = U[v] - Uc;
    if (D == 1) {
      a0.add(W[v] * cu * (cu * cu) * H[v] + W[v] * cu * Bq[v]);
    } else {
      R cv = V[v] - Vc;
      R c2 = cu * cu + cv * cv;
      a0.add(W[v] * cu * c2 * H[v] + W[v] * cu * Bq[v]);
      a1.add(W[v] * cv * c2 * H[v] + W[v] * cv * Bq[v]);
    }
  }
  double q0 = a0.total(), q1 = D == 2 ? a1.total() : 0.0;
  if (lane == 0) {
    s.q[(long)c * 2 + 0] = 0.5 * q0;
    s.q[(long)c * 2 + 1] = 0.5 * q1;
  }
}

// step! scalar part (src/Solver/step_2f.jl:6-64, :179-249): Shakhov factors of
// the old state, w += flux divergence, prim, tau, residual terms.  One thread
// per physical cell; each block writes its residual partials in a fixed order.
template <int D>
__global__ void __launch_bounds__(256) k_cell_param(DevState s, double dt) {
  const Geo& g = s.g;
  __shared__ double red[256][8];
  __shared__ int isb[256];
  int t = blockIdx.x * blockDim.x + threadIdx.x;
  double rr[8] = {0, 0, 0, 0, 0, 0, 0, 0};
  int grp = 0;
  if (t < g.nx * g.ny) {
    int i = t % g.nx, j = t / g.nx;
    int c = cell_index(g, i, j);
    grp = update_group(g, i, j);
    CellParam P;
    P.upd = grp ? 1 : 0;
    int coll = (D == 1 && grp == 2) ? COLL_BGK : s.coll;
    P.coll = coll;
    double* w = s.w + (long)c * 4;
    double* p = s.prim + (long)c * 4;
    int NW = g.NW;
    double lo = p[NW - 1];
    P.o_rho_n = D == 1 ? p[0] * sqrt(lo / PI) : p[0] * (lo / PI);
    P.oU = p[1];
    P.oV = D == 2 ? p[2] : 0.0;
    P.olam = lo;
    P.ocB = g.K / (2.0 * lo);
    P.sfac = 0.8 * (1.0 - g.Pr) * (lo * lo) / p[0];
    P.q0 = s.q[(long)c * 2 + 0];
    P.q1 = s.q[(long)c * 2 + 1];
    if (grp) {
      double wo[4] = {w[0], w[1], w[2], w[3]};
      double ds;
      const double *fL, *fR, *fD = nullptr, *fU = nullptr;
      int fx = j * (g.nx + 1) + i;
      fL = s.fw + (long)fx * 4;
      fR = s.fw + (long)(fx + 1) * 4;
      if (D == 1) {
        ds = g.dx;
        for (int k = 0; k < 3; ++k) w[k] += (fL[k] - fR[k]) / ds;
      } else {
        int fy = s.nface_x + j * g.nx + i;
        fD = s.fw + (long)fy * 4;
        fU = s.fw + (long)(fy + g.nx) * 4;
        ds = g.dx * g.dy;
        for (int k = 0; k < 4; ++k) w[k] += (fL[k] - fR[k] + fD[k] - fU[k]) / ds;
      }
      double pn[4];
      conserve_prim(w, NW, g.gamma, pn);
      for (int k = 0; k < NW; ++k) p[k] = pn[k];
      for (int k = 0; k < NW; ++k) {
        double dw = w[k] - wo[k];
        rr[k] = dw * dw;
        rr[4 + k] = fabs(w[k]);
      }
      double lam = pn[NW - 1];
      double tau = vhs_time(pn[0], lam, g.mu_ref, g.omega);
      P.rho_n = D == 1 ? pn[0] * sqrt(lam / PI) : pn[0] * (lam / PI);
      P.U = pn[1];
      P.V = D == 2 ? pn[2] : 0.0;
      P.lam = lam;
      P.cB = g.K / (2.0 * lam);
      P.dtau = dt / tau;
      P.inv = 1.0 / (1.0 + dt / tau);
      bool bad = !(pn[0] > 0.0) || !(lam > 0.0) || !isfinite(pn[0]) || !isfinite(lam) ||
                 !isfinite(pn[1]);
      if (bad) atomicOr(s.status, 1);
    } else {
      P.rho_n = P.U = P.V = P.lam = P.cB = P.dtau = 0.0;
      P.inv = 1.0;
    }
    s.cp[c] = P;
    CellParamF F;
    F.rho_n = float(P.rho_n);
    F.U = float(P.U);
    F.V = float(P.V);
    F.lam = float(P.lam);
    F.cB = float(P.cB);
    F.dtau = float(P.dtau);
    F.inv = float(P.inv);
    F.o_rho_n = float(P.o_rho_n);
    F.oU = float(P.oU);
    F.oV = float(P.oV);
    F.olam = float(P.olam);
    F.ocB = float(P.ocB);
    F.sf0 = float(P.sfac * P.q0);
    F.sf1 = float(P.sfac * P.q1);
    F.upd = P.upd;
    F.coll = P.coll;
    s.cpf[c] = F;
  }
  // deterministic block partials: interior (grp 1) and boundary (grp 2) sums
  for (int half = 0; half < 2; ++half) {
    bool take = grp == half + 1;
    for (int k = 0; k < 8; ++k) red[threadIdx.x][k] = take ? rr[k] : 0.0;
    isb[threadIdx.x] = 0;
    __syncthreads();
    for (int st = 128; st >= 1; st >>= 1) {
      if (threadIdx.x < st)
        for (int k = 0; k < 8; ++k) red[threadIdx.x][k] += red[threadIdx.x + st][k];
      __syncthreads();
    }
    if (threadIdx.x == 0)
      for (int k = 0; k < 8; ++k) s.blockres[(long)blockIdx.x * 16 + half * 8 + k] = red[0][k];
    __syncthreads();
  }
}

// residual = sqrt(sumRes N) / (sumAvg + 1e-7) + sqrt(boundary sumRes 2) / (...)
// (src/Solver/solver_update.jl:86-88, :239-241; update_boundary.jl:41-44, :284-288).
__global__ void k_residual(DevState s) {
  __shared__ double red[256][16];
  double acc[16];
  for (int k = 0; k < 16; ++k) acc[k] = 0.0;
  for (int b = threadIdx.x; b < s.res_blocks; b += blockDim.x)
    for (int k = 0; k < 16; ++k) acc[k] += s.blockres[(long)b * 16 + k];
  for (int k = 0; k < 16; ++k) red[threadIdx.x][k] = acc[k];
  __syncthreads();
  for (int st = 128; st >= 1; st >>= 1) {
    if (threadIdx.x < st)
      for (int k = 0; k < 16; ++k) red[threadIdx.x][k] += red[threadIdx.x + st][k];
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    const Geo& g = s.g;
    double n = g.D == 1 ? double(g.nx) : double(g.nx) * g.ny;
    for (int k = 0; k < 4; ++k) {
      double r = sqrt(red[0][k] * n) / (red[0][4 + k] + 1.e-7);
      r += sqrt(red[0][8 + k] * 2) / (red[0][12 + k] + 1.e-7);
      s.residual[k] = r;
    }
  }
}

// ------------------------------------------------------------ cell update

template <typename R>
struct CP {
  R rho_n, U, V, lam, cB, dtau, inv, o_rho_n, oU, oV, olam, ocB, s0, s1;
  int upd, coll;
};
template <typename R>
__device__ __forceinline__ CP<R> load_cp(const DevState& s, int c);
template <>
__device__ __forceinline__ CP<double> load_cp<double>(const DevState& s, int c) {
  const CellParam& p = s.cp[c];
  CP<double> r;
  r.rho_n = p.rho_n; r.U = p.U; r.V = p.V; r.lam = p.lam; r.cB = p.cB;
  r.dtau = p.dtau; r.inv = p.inv;
  r.o_rho_n = p.o_rho_n; r.oU = p.oU; r.oV = p.oV; r.olam = p.olam; r.ocB = p.ocB;
  r.s0 = p.sfac * p.q0; r.s1 = p.sfac * p.q1;
  r.upd = p.upd; r.coll = p.coll;
  return r;
}
template <>
__device__ __forceinline__ CP<float> load_cp<float>(const DevState& s, int c) {
  const CellParamF& p = s.cpf[c];
  CP<float> r;
  r.rho_n = p.rho_n; r.U = p.U; r.V = p.V; r.lam = p.lam; r.cB = p.cB;
  r.dtau = p.dtau; r.inv = p.inv;
  r.o_rho_n = p.o_rho_n; r.oU = p.oU; r.oV = p.oV; r.olam = p.olam; r.ocB = p.ocB;
  r.s0 = p.sf0; r.s1 = p.sf1;
  r.upd = p.upd; r.coll = p.coll;
  return r;
}

// Pointwise flux of one face of cell c at velocity v (the face is left of c
// when `right` is false).
template <typename R, int D, int FLUX>
__device__ __forceinline__ void cell_face_flux(const DevState& s, const R* H, const R* Bq,
                                               int f, int kind, const FP<R>& P, int c, int d,
                                               bool right, int v, R un, R ut, R dt, R& fh,
                                               R& fb) {
  const Geo& g = s.g;
  long vs = g.vstride;
  if (kind == 0) {
    fh = R(0);
    fb = R(0);
    return;
  }
  if (kind == 2) {
    // wall flux u h_wall len dt, h_wall = wall Maxwellian on incoming velocities
    int rot = right ? -1 : 1;
    bool in = un * R(rot) >= R(0);
    const double* wp = s.wall + (long)f * 4;
    double lw = D == 1 ? wp[2] : wp[3];
    R sc = R(D == 2 ? (d == 0 ? g.dy : g.dx) * (double)dt : (double)dt);
    R hw, bw;
    if (in) {
      double Uw = d == 0 ? wp[1] : wp[2];
      double Vw = D == 1 ? 0.0 : (d == 0 ? wp[2] : -wp[1]);
      double rho = s.rhow[f];
      R rn = R(D == 1 ? rho * sqrt(lw / PI) : rho * (lw / PI));
      R du = un - R(Uw), e = du * du;
      if (D == 2) { R dv = ut - R(Vw); e += dv * dv; }
      hw = rn * mexp(-R(lw) * e);
      bw = hw * R(g.K / (2.0 * lw));
    } else {
      hw = H[(long)c * vs + v];
      bw = Bq[(long)c * vs + v];
    }
    fh = un * hw * sc;
    fb = un * bw * sc;
    return;
  }
  FaceGeo r = face_geo(g, f);
  bool pos = un >= R(0);
  int up = pos ? r.cL : r.cR;
  int rule = slope_rule(g, d, pos ? r.iL : r.iR);
  R dsc = dscale<R>(d == 0 ? g.dx : g.dy);
  R dxh = R(0.5 * (d == 0 ? g.dx : g.dy));
  R sh, sb;
  R h = upwind_state<R>(H, vs, up, r.step, rule, pos, v, dsc, dxh, sh);
  R b = upwind_state<R>(Bq, vs, up, r.step, rule, pos, v, dsc, dxh, sb);
  R Th, Tb;
  face_flux<R, FLUX, D>(P, dt, un, ut, pos, h, b, sh, sb, fh, fb, Th, Tb);
}

// Pointwise part of step!: h = (h + flux divergence / ds + dt/tau (M + S)) /
// (1 + dt/tau) with the new Maxwellian M and the Shakhov term S of the old
// state (src/Solver/step_2f.jl:56-63, :240-248).  One warp per cell
// (ghost and fixed cells are copied to the output buffer).
template <typename R, int D, int FLUX>
__global__ void __launch_bounds__(256) k_update(DevState s, double dt) {
  const Geo& g = s.g;
  int c = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  int lane = threadIdx.x & 31;
  if (c >= s.ncell) return;
  const R* H = (const R*)s.h[s.cur];
  const R* Bq = (const R*)s.b[s.cur];
  R* Ho = (R*)s.h[s.cur ^ 1];
  R* Bo = (R*)s.b[s.cur ^ 1];
  long vs = g.vstride;
  int ci = c % g.nxt - g.ngx, cj = c / g.nxt - g.ngy;
  bool phys = ci >= 0 && ci < g.nx && cj >= 0 && cj < g.ny;
  CP<R> C;
  if (phys) C = load_cp<R>(s, c);
  if (!phys || !C.upd) {
    for (int v = lane; v < g.nvel; v += 32) {
      Ho[(long)c * vs + v] = H[(long)c * vs + v];
      Bo[(long)c * vs + v] = Bq[(long)c * vs + v];
    }
    return;
  }
  int fxL = cj * (g.nx + 1) + ci, fxR = fxL + 1;
  int fyD = s.nface_x + cj * g.nx + ci, fyU = fyD + g.nx;
  int kL = s.kind[fxL], kR = s.kind[fxR];
  int kD = D == 2 ? s.kind[fyD] : 0, kU = D == 2 ? s.kind[fyU] : 0;
  FP<R> PL, PR, PD, PU;
  if (kL == 1) PL = load_fp<R>(s, fxL);
  if (kR == 1) PR = load_fp<R>(s, fxR);
  if (D == 2) {
    if (kD == 1) PD = load_fp<R>(s, fyD);
    if (kU == 1) PU = load_fp<R>(s, fyU);
  }
  const R* U = vtab<R>(s, 0);
  const R* V = vtab<R>(s, 1);
  R rdt = R(dt);
  R ids = dscale<R>(D == 1 ? g.dx : g.dx * g.dy);
  double dsd = D == 1 ? g.dx : g.dx * g.dy;
  R Kf = R(g.K);
  bool shak = C.coll == COLL_SHAKHOV;
  for (int v = lane; v < g.nvel; v += 32) {
    R u = U[v];
    R vv = D == 2 ? V[v] : R(0);
    R fhL, fbL, fhR, fbR, fhD = 0, fbD = 0, fhU = 0, fbU = 0;
    cell_face_flux<R, D, FLUX>(s, H, Bq, fxL, kL, PL, c, 0, false, v, u, vv, rdt, fhL, fbL);
    cell_face_flux<R, D, FLUX>(s, H, Bq, fxR, kR, PR, c, 0, true, v, u, vv, rdt, fhR, fbR);
    if (D == 2) {
      cell_face_flux<R, D, FLUX>(s, H, Bq, fyD, kD, PD, c, 1, false, v, vv, -u, rdt, fhD, fbD);
      cell_face_flux<R, D, FLUX>(s, H, Bq, fyU, kU, PU, c, 1, true, v, vv, -u, rdt, fhU, fbU);
    }
    R du = u - C.U, e = du * du;
    if (D == 2) { R dv = vv - C.V; e += dv * dv; }
    R MH = C.rho_n * mexp(-C.lam * e);
    R MB = MH * Kf / (R(2) * C.lam);
    if (shak) {
      R ou = u - C.oU, oe = ou * ou, cq = ou * C.s0;
      if (D == 2) {
        R ov = vv - C.oV;
        oe += ov * ov;
        cq += ov * C.s1;
      }
      R OH = C.o_rho_n * mexp(-C.olam * oe);
      R OB = OH * Kf / (R(2) * C.olam);
      R tl = R(2) * C.olam * oe + Kf;
      MH += cq * (tl - R(5)) * OH;
      MB += cq * (tl - R(3)) * OB;
    }
    R h0 = H[(long)c * vs + v], b0 = Bq[(long)c * vs + v];
    R dh, db;
    if (D == 1) {
      dh = fhL - fhR;
      db = fbL - fbR;
    } else {
      dh = fhL - fhR + fhD - fhU;
      db = fbL - fbR + fbD - fbU;
    }
    R hn, bn;
    if (sizeof(R) == 8) {
      hn = (h0 + dh / R(dsd) + C.dtau * MH) / (R(1) + C.dtau);
      bn = (b0 + db / R(dsd) + C.dtau * MB) / (R(1) + C.dtau);
    } else {
      hn = (h0 + dh * ids + C.dtau * MH) * C.inv;
      bn = (b0 + db * ids + C.dtau * MB) * C.inv;
    }
    Ho[(long)c * vs + v] = hn;
    Bo[(long)c * vs + v] = bn;
  }
}

// ------------------------------------------------------------ ghost fill

// copy_ctr! of w, prim, sw, h, b (src/Struct/struct.jl:55-66) for bc_extra!
// (src/Boundary/bc_extra.jl) and 1D bc_period! (src/Boundary/bc_period.jl:10-19)
// in the new buffers.  pass 0: x sides, pass 1: y sides.  One block per ghost cell.
template <typename R>
__global__ void k_ghost(DevState s, int pass) {
  const Geo& g = s.g;
  int t = blockIdx.x;
  int dst = -1, src = -1;
  if (pass == 0) {
    int nrow = g.D == 2 ? g.nyt : 1;
    int per = 2 * g.ngx;
    if (t >= per * nrow) return;
    int jj = t / per, k = t % per;
    int j = jj - g.ngy;
    if (k < g.ngx) {  // left ghost 1-k-1 (0-based: -1-k)
      int gi = -1 - k;
      if (g.bc[0] == BC_EXTRA) src = cell_index(g, 0, j);
      else if (g.bc[0] == BC_PERIOD && g.D == 1) src = cell_index(g, g.nx - 1 - k, j);
      if (src >= 0) dst = cell_index(g, gi, j);
    } else {
      int kk = k - g.ngx;
      int gi = g.nx + kk;
      if (g.bc[1] == BC_EXTRA) src = cell_index(g, g.nx - 1, j);
      else if (g.bc[0] == BC_PERIOD && g.D == 1) src = cell_index(g, kk, j);
      if (src >= 0) dst = cell_index(g, gi, j);
    }
  } else {
    int per = 2 * g.ngy;
    if (t >= per * g.nxt) return;
    int ii = t / per, k = t % per;
    int i = ii - g.ngx;
    if (k < g.ngy) {
      if (g.bc[2] == BC_EXTRA) { src = cell_index(g, i, 0); dst = cell_index(g, i, -1 - k); }
    } else {
      int kk = k - g.ngy;
      if (g.bc[3] == BC_EXTRA) { src = cell_index(g, i, g.ny - 1); dst = cell_index(g, i, g.ny + kk); }
    }
  }
  if (dst < 0) return;
  R* Ho = (R*)s.h[s.cur ^ 1];
  R* Bo = (R*)s.b[s.cur ^ 1];
  long vs = g.vstride;
  for (int v = threadIdx.x; v < g.nvel; v += blockDim.x) {
    Ho[(long)dst * vs + v] = Ho[(long)src * vs + v];
    Bo[(long)dst * vs + v] = Bo[(long)src * vs + v];
  }
  if (threadIdx.x < 4) {
    s.w[(long)dst * 4 + threadIdx.x] = s.w[(long)src * 4 + threadIdx.x];
    s.prim[(long)dst * 4 + threadIdx.x] = s.prim[(long)src * 4 + threadIdx.x];
  }
  if (threadIdx.x < 8) s.sw[(long)dst * 8 + threadIdx.x] = s.sw[(long)src * 8 + threadIdx.x];
}

// ------------------------------------------------------------- dumps

template <typename R, int D, int FLUX>
__global__ void k_faces_dump(DevState s, double dt, double* fh_out, double* fb_out) {
  const Geo& g = s.g;
  int f = blockIdx.x;
  if (f >= s.nface_x + s.nface_y) return;
  int kind = s.kind[f];
  FaceGeo r = face_geo(g, f);
  const R* H = (const R*)s.h[s.cur];
  const R* Bq = (const R*)s.b[s.cur];
  const R* U = vtab<R>(s, 0);
  const R* V = vtab<R>(s, 1);
  FP<R> P;
  if (kind == 1) P = load_fp<R>(s, f);
  int pos0 = r.d == 0 ? r.fi : r.fj;
  bool right = pos0 != 0;  // wall faces: the cell is on the left of the right / top wall
  int c = (kind == 2 && pos0 == 0) ? r.cR : r.cL;
  for (int v = threadIdx.x; v < g.nvel; v += blockDim.x) {
    R un, ut;
    if (D == 1) { un = U[v]; ut = R(0); }
    else if (r.d == 0) { un = U[v]; ut = V[v]; }
    else { un = V[v]; ut = -U[v]; }
    R fh = 0, fb = 0;
    if (kind != 0)
      cell_face_flux<R, D, FLUX>(s, H, Bq, f, kind, P, c, r.d, right, v, un, ut, R(dt), fh, fb);
    fh_out[(long)f * g.nvel + v] = double(fh);
    fb_out[(long)f * g.nvel + v] = double(fb);
  }
}

template <typename R>
__global__ void k_slopes_dump(DevState s, double* sh, double* sb) {
  const Geo& g = s.g;
  int c = blockIdx.x;
  int d = blockIdx.y;
  if (c >= s.ncell) return;
  int ci = c % g.nxt - g.ngx, cj = c / g.nxt - g.ngy;
  bool phys = ci >= 0 && ci < g.nx && cj >= 0 && cj < g.ny;
  int rule = phys ? slope_rule(g, d, d == 0 ? ci : cj) : 0;
  int step = d == 0 ? 1 : g.nxt;
  const R* H = (const R*)s.h[s.cur];
  const R* Bq = (const R*)s.b[s.cur];
  long vs = g.vstride;
  R dsc = dscale<R>(d == 0 ? g.dx : g.dy);
  for (int v = threadIdx.x; v < g.nvel; v += blockDim.x) {
    R t;
    R vh = upwind_state<R>(H, vs, c, step, rule, true, v, dsc, R(0), t);
    (void)vh;
    sh[((long)c * g.D + d) * g.nvel + v] = double(t);
    upwind_state<R>(Bq, vs, c, step, rule, true, v, dsc, R(0), t);
    sb[((long)c * g.D + d) * g.nvel + v] = double(t);
  }
}

// --------------------------------------------------------- conversions

__global__ void k_conv_in_d(double* dst, const double* src, long ncell, int nvel, int vs) {
  long t = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= ncell * nvel) return;
  long c = t / nvel;
  int v = (int)(t % nvel);
  dst[c * vs + v] = src[t];
}
__global__ void k_conv_in_f(float* dst, const double* src, long ncell, int nvel, int vs) {
  long t = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= ncell * nvel) return;
  long c = t / nvel;
  int v = (int)(t % nvel);
  dst[c * vs + v] = (float)src[t];
}
__global__ void k_conv_out_d(double* dst, const double* src, long ncell, int nvel, int vs) {
  long t = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= ncell * nvel) return;
  long c = t / nvel;
  int v = (int)(t % nvel);
  dst[t] = src[c * vs + v];
}
__global__ void k_conv_out_f(double* dst, const float* src, long ncell, int nvel, int vs) {
  long t = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= ncell * nvel) return;
  long c = t / nvel;
  int v = (int)(t % nvel);
  dst[t] = (double)src[c * vs + v];
}
__global__ void k_pack_w(double* dst4, const double* src, long ncell, int nw) {
  long c = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= ncell) return;
  for (int k = 0; k < 4; ++k) dst4[c * 4 + k] = k < nw ? src[c * nw + k] : 0.0;
}

// timestep: max over physical cells (src/Solver/solver_main.jl:240-342); one block.
__global__ void k_timestep(DevState s, double umax, double vmax, double* out) {
  __shared__ double red[256];
  const Geo& g = s.g;
  double m = 0.0;
  for (int t = threadIdx.x; t < g.nx * g.ny; t += blockDim.x) {
    int i = t % g.nx, j = t / g.nx;
    const double* p = s.prim + (long)cell_index(g, i, j) * 4;
    double sos = pow(0.5 * g.gamma / p[g.NW - 1], 0.5);
    double v;
    if (g.D == 1) v = (fmax(umax, fabs(p[1])) + sos) / g.dx;
    else v = (fmax(umax, fabs(p[1])) + sos) / g.dx + (fmax(vmax, fabs(p[2])) + sos) / g.dy;
    m = fmax(m, v);
  }
  red[threadIdx.x] = m;
  __syncthreads();
  for (int st = 128; st >= 1; st >>= 1) {
    if (threadIdx.x < st) red[threadIdx.x] = fmax(red[threadIdx.x], red[threadIdx.x + st]);
    __syncthreads();
  }
  if (threadIdx.x == 0) *out = red[0];
}

// ------------------------------------------------------------- launchers

static inline unsigned nblk(long n, int bs) { return (unsigned)((n + bs - 1) / bs); }

int launch_reconstruct(DevState& s, cudaStream_t st) {
  if (s.flux == FLUX_KFVS) return 0;  // KFVS reads no w slopes
  long n = (long)s.g.nx * s.g.ny * s.g.D;
  if (s.g.interp == 1) return 0;
  k_wslope<<<nblk(n, 128), 128, 0, st>>>(s);
  return 1;
}

template <typename R, int D>
static int evolve_t(DevState& s, double dt, cudaStream_t st) {
  int nf = s.nface_x + s.nface_y;
  int n = 0;
  switch (s.flux) {
    case FLUX_KFVS: k_face_param<FLUX_KFVS><<<nblk(nf, 128), 128, 0, st>>>(s, dt); break;
    case FLUX_KCU: k_face_param<FLUX_KCU><<<nblk(nf, 128), 128, 0, st>>>(s, dt); break;
    default: k_face_param<FLUX_UGKS><<<nblk(nf, 128), 128, 0, st>>>(s, dt); break;
  }
  ++n;
  unsigned gb = nblk((long)nf * 32, 256);
  switch (s.flux) {
    case FLUX_KFVS: k_face_moments<R, D, FLUX_KFVS><<<gb, 256, 0, st>>>(s, dt); break;
    case FLUX_KCU: k_face_moments<R, D, FLUX_KCU><<<gb, 256, 0, st>>>(s, dt); break;
    default: k_face_moments<R, D, FLUX_UGKS><<<gb, 256, 0, st>>>(s, dt); break;
  }
  ++n;
  bool wall = false;
  for (int k = 0; k < 2 * D; ++k) wall |= s.g.bc[k] == BC_MAXWELL;
  if (wall) {
    k_wall<R, D><<<gb, 256, 0, st>>>(s, dt);
    ++n;
  }
  return n;
}

int launch_evolve(DevState& s, double dt, cudaStream_t st) {
  if (s.prec == 0) return s.g.D == 1 ? evolve_t<double, 1>(s, dt, st) : evolve_t<double, 2>(s, dt, st);
  return s.g.D == 1 ? evolve_t<float, 1>(s, dt, st) : evolve_t<float, 2>(s, dt, st);
}

template <typename R, int D>
static int update_t(DevState& s, double dt, cudaStream_t st) {
  int n = 0;
  long ncp = (long)s.g.nx * s.g.ny;
  if (s.coll == COLL_SHAKHOV) {
    k_cell_q<R, D><<<nblk(ncp * 32, 256), 256, 0, st>>>(s);
    ++n;
  }
  k_cell_param<D><<<s.res_blocks, 256, 0, st>>>(s, dt);
  ++n;
  unsigned gb = nblk((long)s.ncell * 32, 256);
  switch (s.flux) {
    case FLUX_KFVS: k_update<R, D, FLUX_KFVS><<<gb, 256, 0, st>>>(s, dt); break;
    case FLUX_KCU: k_update<R, D, FLUX_KCU><<<gb, 256, 0, st>>>(s, dt); break;
    default: k_update<R, D, FLUX_UGKS><<<gb, 256, 0, st>>>(s, dt); break;
  }
  ++n;
  s.cur ^= 1;
  bool fill = false;
  for (int k = 0; k < 2 * D; ++k) fill |= s.g.bc[k] == BC_EXTRA || s.g.bc[k] == BC_PERIOD;
  if (fill) {
    // the ghost kernels write into buffer cur^1 of their DevState copy: pass
    // a copy that still points at the pre-swap index so they fill the new state
    DevState t = s;
    t.cur ^= 1;
    int nrow = D == 2 ? s.g.nyt : 1;
    if (s.g.ngx > 0) { k_ghost<R><<<2 * s.g.ngx * nrow, 128, 0, st>>>(t, 0); ++n; }
    if (D == 2 && s.g.ngy > 0) { k_ghost<R><<<2 * s.g.ngy * s.g.nxt, 128, 0, st>>>(t, 1); ++n; }
  }
  k_residual<<<1, 256, 0, st>>>(s);
  ++n;
  return n;
}

int launch_update(DevState& s, double dt, cudaStream_t st) {
  if (s.prec == 0) return s.g.D == 1 ? update_t<double, 1>(s, dt, st) : update_t<double, 2>(s, dt, st);
  return s.g.D == 1 ? update_t<float, 1>(s, dt, st) : update_t<float, 2>(s, dt, st);
}

template <typename R, int D>
static int faces_dump_t(DevState& s, double dt, double* fh, double* fb, cudaStream_t st) {
  int nf = s.nface_x + s.nface_y;
  switch (s.flux) {
    case FLUX_KFVS: k_faces_dump<R, D, FLUX_KFVS><<<nf, 128, 0, st>>>(s, dt, fh, fb); break;
    case FLUX_KCU: k_faces_dump<R, D, FLUX_KCU><<<nf, 128, 0, st>>>(s, dt, fh, fb); break;
    default: k_faces_dump<R, D, FLUX_UGKS><<<nf, 128, 0, st>>>(s, dt, fh, fb); break;
  }
  return 1;
}

int launch_faces_dump(DevState& s, double dt, double* fh, double* fb, cudaStream_t st) {
  if (s.prec == 0)
    return s.g.D == 1 ? faces_dump_t<double, 1>(s, dt, fh, fb, st) : faces_dump_t<double, 2>(s, dt, fh, fb, st);
  return s.g.D == 1 ? faces_dump_t<float, 1>(s, dt, fh, fb, st) : faces_dump_t<float, 2>(s, dt, fh, fb, st);
}

int launch_slopes_dump(DevState& s, double* sh, double* sb, cudaStream_t st) {
  dim3 grid(s.ncell, s.g.D);
  if (s.prec == 0) k_slopes_dump<double><<<grid, 128, 0, st>>>(s, sh, sb);
  else k_slopes_dump<float><<<grid, 128, 0, st>>>(s, sh, sb);
  return 1;
}

int launch_convert_in(void* dst, int prec, const double* src, long ncell, int nvel, int vstride,
                      cudaStream_t st) {
  long n = ncell * nvel;
  if (n == 0) return 0;
  if (prec == 0) k_conv_in_d<<<nblk(n, 256), 256, 0, st>>>((double*)dst, src, ncell, nvel, vstride);
  else k_conv_in_f<<<nblk(n, 256), 256, 0, st>>>((float*)dst, src, ncell, nvel, vstride);
  return 1;
}

int launch_convert_out(double* dst, int prec, const void* src, long ncell, int nvel, int vstride,
                       cudaStream_t st) {
  long n = ncell * nvel;
  if (n == 0) return 0;
  if (prec == 0) k_conv_out_d<<<nblk(n, 256), 256, 0, st>>>(dst, (const double*)src, ncell, nvel, vstride);
  else k_conv_out_f<<<nblk(n, 256), 256, 0, st>>>(dst, (const float*)src, ncell, nvel, vstride);
  return 1;
}

int launch_pack_w(double* dst4, const double* src, long ncell, int nw, cudaStream_t st) {
  k_pack_w<<<nblk(ncell, 256), 256, 0, st>>>(dst4, src, ncell, nw);
  return 1;
}

int launch_timestep(const DevState& s, double umax, double vmax, double* out, cudaStream_t st) {
  k_timestep<<<1, 256, 0, st>>>(s, umax, vmax, out);
  return 1;
}

}  // namespace kb
