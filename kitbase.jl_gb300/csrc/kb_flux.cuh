// kb_flux.cuh -- device helpers shared by the DVM kernels: face geometry,
// upwind face states, per-face / per-cell coefficients and the pointwise
// interface fluxes of KFVS, KCU and UGKS.
#pragma once

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
  r.cB = s.g.Kb / (2.0 * lam);
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


}  // namespace kb
