// kb_kernels.cu -- sm_103a kernels of the DVM time step (1D2F1V, 2D2F2V).
//
// One step is: [w slopes] -> [face parameters] -> face moments (fw) ->
// [Maxwell walls] -> [Shakhov heat flux] -> cell parameters (w, prim, tau,
// residual partials) -> pointwise update of h, b -> [ghost fill] -> residual.
// The pointwise face fluxes fh, fb are never stored: the update kernel forms
// them again from the neighbour cells, so h and b are read from HBM and
// written once per step apart from stencil re-reads that hit L2.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdint>
#include <mutex>
#include <set>
#include <utility>
#include <stdio.h>

#include "kb_kernels.cuh"
#include "kb_flux.cuh"

namespace kb {

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

// ------------------------------------------------------------ w slopes

// reconstruct! for w (src/Solver/solver_reconstruction.jl:111-122 1D, :496-537 2D):
// one thread per (physical cell, direction).
// FAST (the FP32 split form): one reciprocal of the cell size per thread in
// place of two FP64 divisions per component.
template <bool FAST, bool GRP = false>
__global__ void k_wslope(DevState sp) {
  int lb;
  const int gr = group_member<GRP, GK_WSLOPE>(sp, lb);
  KB_GROUP_STATE(GRP, sp, gr);
  const Geo& g = s.g;
  int t = lb * blockDim.x + threadIdx.x;
  int n = g.nx * g.ny;
  if (t >= n * g.D) return;
  int d = t / n, c0 = t % n;
  int i = c0 % g.nx, j = c0 / g.nx;
  int c = cell_index(g, i, j);
  int rule = slope_rule(g, d, d == 0 ? i : j);
  int step = d == 0 ? 1 : g.nxt;
  double dd = d == 0 ? g.dx : g.dy;  // 0.5 * (dx[i-1] + dx[i]) on a uniform mesh
  double* out = s.sw + ((long)c * 2 + d) * 4;
  const double rd = FAST ? 1.0 / dd : 0.0;
  for (int k = 0; k < g.NW; ++k) {
    double q0 = s.w[(long)c * 4 + k];
    double qm = (rule == 1 || rule == 3) ? s.w[(long)(c - step) * 4 + k] : 0.0;
    double qp = (rule == 1 || rule == 2) ? s.w[(long)(c + step) * 4 + k] : 0.0;
    if (FAST) {
      const double a = (q0 - qm) * rd, b = (qp - q0) * rd;
      out[k] = rule == 1 ? vanleer(a, b) : (rule == 2 ? b : (rule == 3 ? a : 0.0));
    } else {
      out[k] = slope_of<double>(rule, qm, q0, qp, dd);
    }
  }
}

// ------------------------------------------------------- face parameters

// log2-form exponent of rho (lam/pi)^(D/2) exp(-lam ((un-U)^2 + (ut-V)^2)) as
// E.x + E.y un + E.z ut + E.w c2.
// FAST (the FP32 split form): log2 of the density factor in FP32.
template <bool FAST = false>
__device__ inline float4 maxwell_exp2(double rho_n, double U, double V, double lam) {
  float4 E;
  const double l2r = rho_n > 0.0 ? (FAST ? double(log2f(float(rho_n))) : log2(rho_n)) : 0.0;
  E.x = rho_n > 0.0 ? float(l2r - lam * (U * U + V * V) * LOG2E) : -200.f;
  E.y = float(2.0 * lam * U * LOG2E);
  E.z = float(2.0 * lam * V * LOG2E);
  E.w = float(-lam * LOG2E);
  return E;
}

// FP32 monomial coefficients of the interface flux (see FaceCoef32).
template <bool FAST = false>
__device__ __forceinline__ FaceCoef32 face_coef32(const Geo& g, const FaceParam& P, int flux, double dd) {
  FaceCoef32 c;
  float4 z = make_float4(0.f, 0.f, 0.f, 0.f);
  c.E = c.T = c.G = c.Cp = c.Dp = c.Cm = c.Dm = z;
  double len = P.len;
  c.T.x = float(P.tr[0]);
  c.T.y = float(P.tr[1] / dd);
  if (flux == FLUX_KFVS) return c;
  double lam = P.prim[3], rho = P.prim[0];
  double rho_n = g.D == 1 ? rho * t_sqrt<FAST>(lam / PI) : rho * (lam / PI);
  c.E = maxwell_exp2<FAST>(rho_n, P.prim[1], P.prim[2], lam);
  double cB = g.Kb / (2.0 * lam);
  const double* Mt = P.Mt;
  if (flux == FLUX_KCU) {
    c.T.z = float(Mt[0] * len);
    c.T.w = float(Mt[0] * cB * len);
    return c;
  }
  // the energy slope sits at index D + 1; selected between constant indices
  // (a run-time index would place the slope arrays in local memory)
  const double* t = P.aT;
  const double tt = g.D == 2 ? t[2] : 0.0, te = g.D == 2 ? t[3] : t[2], Mxi2 = P.Mxi2;
  c.T.z = float((Mt[0] + Mt[2] * (t[0] + 0.5 * te * cB)) * len);
  c.T.w = float((Mt[0] * cB + Mt[2] * (cB * t[0] + 0.5 * te * Mxi2)) * len);
  c.G.x = float(Mt[2] * tt * len);
  c.G.y = float(0.5 * Mt[2] * te * len);
  c.G.z = float(Mt[2] * cB * tt * len);
  c.G.w = float(0.5 * Mt[2] * cB * te * len);
  // one upwind side's slope terms (a = aL for un >= 0, aR otherwise)
  auto side = [&](const double (&a)[4], float4& C, float4& Dd) {
    const double at = g.D == 2 ? a[2] : 0.0, ae = g.D == 2 ? a[3] : a[2];
    C.x = float((Mt[1] * (a[0] + 0.5 * ae * cB) + Mt[2] * t[1]) * len);
    C.y = float(Mt[1] * a[1] * len);
    C.z = float(Mt[1] * at * len);
    C.w = float(0.5 * Mt[1] * ae * len);
    Dd.x = float((Mt[1] * (cB * a[0] + 0.5 * ae * Mxi2) + Mt[2] * cB * t[1]) * len);
    Dd.y = float(Mt[1] * cB * a[1] * len);
    Dd.z = float(Mt[1] * cB * at * len);
    Dd.w = float(0.5 * Mt[1] * cB * ae * len);
  };
  side(P.aL, c.Cp, c.Dp);
  side(P.aR, c.Cm, c.Dm);
  return c;
}

// Interface equilibrium from the two half Maxwellians (flux_kcu.jl:480-495,
// flux_ugks.jl:47-56), then the KCU / UGKS time integrals, UGKS slopes and
// the analytic part of fw.  One thread per face.
// FAST: the FP32 split form (transcendentals in FP32, see t_exp).
template <int D, int FLUX, bool FAST, bool GRP = false>
__global__ void k_face_param(DevState sp, double dt_arg) {
  int lb;
  const int gr = group_member<GRP, GK_FACE>(sp, lb);
  KB_GROUP_STATE(GRP, sp, gr);
  const double dt = GRP ? sp.grp->dt[gr] : dt_arg;
  const Geo& g = s.g;
  int f = lb * blockDim.x + threadIdx.x;
  if (f >= s.nface_x + s.nface_y) return;
  if (s.kind[f] != 1) return;
  FaceGeo r = face_geo(g, f);
  constexpr int NW = D + 2;
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
  P.tr[0] = P.tr[1] = 0;
  if (FLUX == FLUX_KFVS) {
    P.mult = 1.0;
    P.tr[0] = dt * len;
    P.tr[1] = 0.5 * (dt * dt) * len;
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
    conserve_prim<FAST>(wL, NW, g.gamma, pL);
    conserve_prim<FAST>(wR, NW, g.gamma, pR);
    GM m;
    gauss_moments<FAST>(pL, NW, g.K, m, 1);
    moments_conserve(m.MuL, m.Mv, m.Mxi, NW, 0, 0, 0, M1);
    gauss_moments<FAST>(pR, NW, g.K, m, 2);
    moments_conserve(m.MuR, m.Mv, m.Mxi, NW, 0, 0, 0, M2);
    for (int k = 0; k < 4; ++k) wi[k] = k < NW ? pL[0] * M1[k] + pR[0] * M2[k] : 0.0;
    conserve_prim<FAST>(wi, NW, g.gamma, p);
    double lam = p[NW - 1];
    P.prim[0] = p[0];
    P.prim[1] = p[1];
    P.prim[2] = NW == 4 ? p[2] : 0.0;
    P.prim[3] = lam;
    double tau = vhs_time<FAST>(p[0], lam, g.mu_ref, g.omega);
    GM mi;
    if (FLUX == FLUX_KCU) {
      tau += fabs(pL[0] / pL[NW - 1] - pR[0] / pR[NW - 1]) /
             (pL[0] / pL[NW - 1] + pR[0] / pR[NW - 1]) * dt * 2.0;
      P.Mt[1] = tau * (1.0 - t_exp<FAST>(-dt / tau));
      P.Mt[0] = dt - P.Mt[1];
      gauss_moments<FAST>(p, NW, g.K, mi);
      double Muv[4];
      moments_conserve(mi.Mu, mi.Mv, mi.Mxi, NW, 1, 0, 0, Muv);
      for (int k = 0; k < NW; ++k) P.fwa[k] = P.Mt[0] * p[0] * Muv[k] * len;
      P.mult = len;
      P.tr[0] = P.Mt[1] * len;
    } else {
      double dL[4], dR[4];
      const double rdx = FAST ? 1.0 / dxh : 0.0;
      for (int k = 0; k < 4; ++k) {
        dL[k] = k < NW ? (FAST ? (wi[k] - wL[k]) * rdx : (wi[k] - wL[k]) / dxh) : 0.0;
        dR[k] = k < NW ? (FAST ? (wR[k] - wi[k]) * rdx : (wR[k] - wi[k]) / dxh) : 0.0;
      }
      double aL[4], aR[4], aT[4];
      pdf_slope<FAST>(p, dL, NW, g.K, aL);
      pdf_slope<FAST>(p, dR, NW, g.K, aR);
      gauss_moments<FAST>(p, NW, g.K, mi);
      double MauL[4], MauR[4], MauT[4], Muv[4], tmp[4];
      moments_conserve_slope(aL, mi.MuL, mi.Mv, mi.Mxi, NW, 1, MauL);
      moments_conserve_slope(aR, mi.MuR, mi.Mv, mi.Mxi, NW, 1, MauR);
      for (int k = 0; k < 4; ++k) tmp[k] = -p[0] * (MauL[k] + MauR[k]);
      pdf_slope<FAST>(p, tmp, NW, g.K, aT);
      double ex = t_exp<FAST>(-dt / tau);
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
      P.tr[0] = Mt[3] * len;
      P.tr[1] = Mt[4] * len;
    }
  }
  s.fp[f] = P;
  s.fc[f] = face_coef32<FAST>(g, P, FLUX, r.d == 0 ? g.dx : g.dy);
  FaceParamF F;
  double lam = P.prim[3] > 0 ? P.prim[3] : 1.0;
  F.rho_n = float(g.D == 1 ? P.prim[0] * sqrt(lam / PI) : P.prim[0] * (lam / PI));
  F.U = float(P.prim[1]);
  F.V = float(P.prim[2]);
  F.lam = float(P.prim[3]);
  F.cB = float(g.Kb / (2.0 * lam));
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

// ------------------------------------------------------------ Maxwell walls

// flux_boundary_maxwell! 1D2F1V (src/Flux/flux_boundary.jl:39-61) and 2D2F2V
// (:190-220) in the face-local frame; rot = +1 on the left / bottom wall and
// -1 on the right / top wall (src/Solver/evolve_boundary.jl).  One CTA of
// WALL_T threads per wall face (DevState::wall_list): the velocities are
// shared by all its warps, each warp sums its part, and thread 0 adds the
// warps' sums in warp order (deterministic) and finishes the face.
constexpr int WALL_T = 128;
template <typename R, int D, bool GRP = false>
__global__ void __launch_bounds__(WALL_T) k_wall(DevState sp, double dt_arg) {
  __shared__ double part[WALL_T / 32][8];
  int lb;
  const int gr = group_member<GRP, GK_WALL>(sp, lb);
  KB_GROUP_STATE(GRP, sp, gr);
  const double dt = GRP ? sp.grp->dt[gr] : dt_arg;
  const Geo& g = s.g;
  const int f = s.wall_list[lb];
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
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
  // One pass: the outgoing half from the interior cell's h, b; the incoming
  // half as moments of the unit-density wall Maxwellian, scaled by the wall
  // density afterwards in FP64.  The mass flux S0 = SF + rho_n * I0 then
  // cancels to FP64 round-off by construction (the density is chosen so that
  // no mass crosses the wall), also when h is stored in FP32.
  Acc<R> o0, o1, o2, o3, i0, i1, i2, i3;
  for (int v = threadIdx.x; v < g.nvel; v += WALL_T) {
    R un, ut;
    if (D == 1) { un = U[v]; ut = R(0); }
    else if (r.d == 0) { un = U[v]; ut = V[v]; }
    else { un = V[v]; ut = -U[v]; }
    const bool in = un * R(rot) >= R(0);
    R c2 = un * un;
    if (D == 2) c2 += ut * ut;
    if (in) {
      R du = un - Uw, e = du * du;
      if (D == 2) { R dv = ut - Vw; e += dv * dv; }
      const R t = W[v] * un * mexp(-Lw * e);
      i0.add(t);
      i1.add(t * un);
      if (D == 2) i2.add(t * ut);
      i3.add(t * c2);
    } else {
      const R t = W[v] * un * H[(long)c * vs + v];
      o0.add(t);
      o1.add(t * un);
      if (D == 2) o2.add(t * ut);
      o3.add(t * c2 + W[v] * un * Bq[(long)c * vs + v]);
    }
  }
  {
    const double t0 = o0.total(), t1 = o1.total(), t2 = D == 2 ? o2.total() : 0.0, t3 = o3.total();
    const double t4 = i0.total(), t5 = i1.total(), t6 = D == 2 ? i2.total() : 0.0, t7 = i3.total();
    if (lane == 0) {
      part[wid][0] = t0; part[wid][1] = t1; part[wid][2] = t2; part[wid][3] = t3;
      part[wid][4] = t4; part[wid][5] = t5; part[wid][6] = t6; part[wid][7] = t7;
    }
  }
  __syncthreads();
  if (threadIdx.x != 0) return;
  double T[8];
  for (int k = 0; k < 8; ++k) {
    T[k] = part[0][k];
    for (int w = 1; w < WALL_T / 32; ++w) T[k] += part[w][k];
  }
  const double norm = D == 1 ? sqrt(lw / PI) : (lw / PI);
  const double SF = T[0], I0 = T[4];
  const double rho = -SF / (I0 * norm);
  const double rn = rho * norm;  // wall density times the Maxwellian's normalisation
  const double cBw = g.Kb / (2.0 * lw);
  double len = D == 2 ? (r.d == 0 ? g.dy : g.dx) : 1.0;
  double sc = D == 2 ? len * dt : dt;
  const double S0 = SF + rn * I0;
  const double S1 = T[1] + rn * T[5];
  const double S2 = D == 2 ? T[2] + rn * T[6] : 0.0;
  const double S3 = T[3] + rn * (T[7] + cBw * I0);
  s.rhow[f] = rho;
  FaceCoef32 wc;
  float4 z = make_float4(0.f, 0.f, 0.f, 0.f);
  wc.G = wc.Cp = wc.Dp = wc.Cm = wc.Dm = z;
  wc.E = maxwell_exp2(D == 1 ? rho * sqrt(lw / PI) : rho * (lw / PI), bw[1], bw[2], lw);
  wc.T = make_float4(float(sc), 0.f, float(g.Kb / (2.0 * lw)), float(rot));
  s.fc[f] = wc;
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

// step! scalar part (src/Solver/step_2f.jl:6-64, :179-249): Shakhov factors of
// the old state, w += flux divergence, prim, tau, residual terms.  One thread
// per physical cell; each block writes its residual partials in a fixed order.
// FAST (the FP32 split form): tau, the density factors and the exponent
// offsets of the coefficient blocks with FP32 transcendentals, conserve_prim
// by reciprocals (see t_exp); w and prim stay FP64.  BS threads per block
// (32 on small grids, 256 otherwise: DevState::cell_bs).
template <int D, bool FAST, int BS, bool GRP = false>
__global__ void __launch_bounds__(BS) k_cell_param(DevState sp, double dt_arg) {
  int lb;
  const int gr = group_member<GRP, GK_CELL>(sp, lb);
  KB_GROUP_STATE(GRP, sp, gr);
  const double dt = GRP ? sp.grp->dt[gr] : dt_arg;
  const Geo& g = s.g;
  __shared__ double red[BS][8];
  int t = lb * BS + threadIdx.x;
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
    constexpr int NW = D + 2;  // compile-time, so the small arrays stay in registers
    double lo = p[NW - 1];
    P.o_rho_n = D == 1 ? p[0] * t_sqrt<FAST>(lo / PI) : p[0] * (lo / PI);
    P.oU = p[1];
    P.oV = D == 2 ? p[2] : 0.0;
    P.olam = lo;
    P.ocB = g.Kb / (2.0 * lo);
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
      conserve_prim<FAST>(w, NW, g.gamma, pn);
      for (int k = 0; k < NW; ++k) p[k] = pn[k];
      for (int k = 0; k < NW; ++k) {
        double dw = w[k] - wo[k];
        rr[k] = dw * dw;
        rr[4 + k] = fabs(w[k]);
      }
      double lam = pn[NW - 1];
      double tau = vhs_time<FAST>(pn[0], lam, g.mu_ref, g.omega);
      P.rho_n = D == 1 ? pn[0] * t_sqrt<FAST>(lam / PI) : pn[0] * (lam / PI);
      P.U = pn[1];
      P.V = D == 2 ? pn[2] : 0.0;
      P.lam = lam;
      P.cB = g.Kb / (2.0 * lam);
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
    CellCoef32 K;
    float4 z = make_float4(0.f, 0.f, 0.f, 0.f);
    K.EM = K.EO = K.Q = K.TL = z;
    if (P.upd) {
      K.EM = maxwell_exp2<FAST>(P.rho_n, P.U, P.V, P.lam);
      double ds = D == 1 ? g.dx : g.dx * g.dy;
      K.A = make_float4(float(P.cB), float(P.dtau), float(P.inv), float(1.0 / ds));
      if (P.coll == COLL_SHAKHOV) {
        K.EO = maxwell_exp2<FAST>(P.o_rho_n, P.oU, P.oV, P.olam);
        double s0 = P.sfac * P.q0, s1 = P.sfac * P.q1;
        K.Q = make_float4(float(-(s0 * P.oU + s1 * P.oV)), float(s0), float(s1), float(P.ocB));
        double l2 = 2.0 * P.olam;
        K.TL = make_float4(float(l2 * (P.oU * P.oU + P.oV * P.oV) + g.Kb), float(-2.0 * l2 * P.oU),
                           float(-2.0 * l2 * P.oV), float(l2));
      } else {
        K.EO.x = -200.f;
      }
    } else {
      K.EM.x = -200.f;
      K.EO.x = -200.f;
      K.A = make_float4(0.f, 0.f, 1.f, 0.f);
    }
    s.cc[c] = K;
  }
  // deterministic block partials: interior (grp 1) and boundary (grp 2) sums
  for (int half = 0; half < 2; ++half) {
    bool take = grp == half + 1;
    for (int k = 0; k < 8; ++k) red[threadIdx.x][k] = take ? rr[k] : 0.0;
    __syncthreads();
    for (int st = BS / 2; st >= 1; st >>= 1) {
      if (threadIdx.x < st)
        for (int k = 0; k < 8; ++k) red[threadIdx.x][k] += red[threadIdx.x + st][k];
      __syncthreads();
    }
    if (threadIdx.x == 0)
      for (int k = 0; k < 8; ++k) s.blockres[(long)lb * 16 + half * 8 + k] = red[0][k];
    __syncthreads();
  }
}

// residual = sqrt(sumRes N) / (sumAvg + 1e-7) + sqrt(boundary sumRes 2) / (...)
// (src/Solver/solver_update.jl:86-88, :239-241; update_boundary.jl:41-44, :284-288).
template <bool GRP = false>
__global__ void k_residual(DevState sp) {
  int lb;
  const int gr = group_member<GRP, GK_RES>(sp, lb);
  KB_GROUP_STATE(GRP, sp, gr);
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

// Per-face constants of the update loop, built once per warp so the velocity
// loop runs in the storage precision only.
template <typename R>
struct FaceCtx {
  int kind;             // 0 none, 1 interior, 2 wall
  int cL, cR, step;     // cells on both sides and the cell step along the normal
  int ruleL, ruleR;     // slope rules of the two cells along the normal
  R dsc, dxh;           // 1/dx (FP32) or dx (FP64), dx/2
  FP<R> P;              // interior coefficients
  R wU, wV, wlam, wrn, wcB, wsc;  // wall: velocity, lambda, rho (lam/pi)^(D/2), K/(2 lam), len dt
  int rot;
};

template <typename R, int D>
__device__ __forceinline__ FaceCtx<R> make_ctx(const DevState& s, int f, int kind, bool right,
                                               double dt) {
  const Geo& g = s.g;
  FaceCtx<R> x;
  x.kind = kind;
  FaceGeo r = face_geo(g, f);
  x.cL = r.cL;
  x.cR = r.cR;
  x.step = r.step;
  x.ruleL = slope_rule(g, r.d, r.iL);
  x.ruleR = slope_rule(g, r.d, r.iR);
  double dd = r.d == 0 ? g.dx : g.dy;
  x.dsc = dscale<R>(dd);
  x.dxh = R(0.5 * dd);
  x.rot = right ? -1 : 1;
  if (kind == 1) x.P = load_fp<R>(s, f);
  if (kind == 2) {
    const double* wp = s.wall + (long)f * 4;
    double lw = D == 1 ? wp[2] : wp[3];
    double rho = s.rhow[f];
    x.wU = R(r.d == 0 ? wp[1] : wp[2]);
    x.wV = R(D == 1 ? 0.0 : (r.d == 0 ? wp[2] : -wp[1]));
    x.wlam = R(lw);
    x.wrn = R(D == 1 ? rho * sqrt(lw / PI) : rho * (lw / PI));
    x.wcB = R(g.Kb / (2.0 * lw));
    x.wsc = R(D == 2 ? (r.d == 0 ? g.dy : g.dx) * dt : dt);
  }
  return x;
}

// Pointwise flux of one face at velocity v (face-local velocities un, ut);
// c is the interior cell next to a wall face.
template <typename R, int D, int FLUX>
__device__ __forceinline__ void ctx_flux(const FaceCtx<R>& x, const R* __restrict__ H,
                                         const R* __restrict__ Bq, long vs, int c, int v,
                                         R un, R ut, R dt, R& fh, R& fb) {
  if (x.kind == 0) {
    fh = R(0);
    fb = R(0);
    return;
  }
  if (x.kind == 2) {
    // u h_wall len dt with h_wall the wall Maxwellian on incoming velocities
    bool in = un * R(x.rot) >= R(0);
    R hw, bw;
    if (in) {
      R du = un - x.wU, e = du * du;
      if (D == 2) {
        R dv = ut - x.wV;
        e += dv * dv;
      }
      hw = x.wrn * mexp(-x.wlam * e);
      bw = hw * x.wcB;
    } else {
      hw = H[(long)c * vs + v];
      bw = Bq[(long)c * vs + v];
    }
    fh = un * hw * x.wsc;
    fb = un * bw * x.wsc;
    return;
  }
  bool pos = un >= R(0);
  int up = pos ? x.cL : x.cR;
  int rule = pos ? x.ruleL : x.ruleR;
  R sh, sb;
  R h = upwind_state<R>(H, vs, up, x.step, rule, pos, v, x.dsc, x.dxh, sh);
  R b = upwind_state<R>(Bq, vs, up, x.step, rule, pos, v, x.dsc, x.dxh, sb);
  R Th, Tb;
  face_flux<R, FLUX, D>(x.P, dt, un, ut, pos, h, b, sh, sb, fh, fb, Th, Tb);
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
  int pos0 = r.d == 0 ? r.fi : r.fj;
  bool right = pos0 != 0;  // wall faces: the cell is on the left of the right / top wall
  int c = (kind == 2 && pos0 == 0) ? r.cR : r.cL;
  FaceCtx<R> X = make_ctx<R, D>(s, f, kind, right, dt);
  for (int v = threadIdx.x; v < g.nvel; v += blockDim.x) {
    R un, ut;
    if (D == 1) { un = U[v]; ut = R(0); }
    else if (r.d == 0) { un = U[v]; ut = V[v]; }
    else { un = V[v]; ut = -U[v]; }
    R fh = 0, fb = 0;
    ctx_flux<R, D, FLUX>(X, H, Bq, g.vstride, c, v, un, ut, R(dt), fh, fb);
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

// Row copy with conversion between the host layout ([cell][nvel], FP64) and
// the device layout ([cell][vstride], storage precision); a block converts cpb
// consecutive cells, threads striding over velocities (no index division).
template <typename DT, typename ST>
__global__ void k_conv(DT* __restrict__ dst, const ST* __restrict__ src, long ncell, int nvel,
                       int dvs, int svs, int cpb) {
  const long c0 = (long)blockIdx.x * cpb;
  for (int r = 0; r < cpb; ++r) {
    const long c = c0 + r;
    if (c >= ncell) return;
    for (int v = threadIdx.x; v < nvel; v += blockDim.x) dst[c * dvs + v] = (DT)src[c * svs + v];
  }
}
// The same conversion when both layouts are one dense array (nvel equal to
// the device row stride): element pairs, CONV_U of them per thread with all
// loads issued before the first store.  Across the host link (page-locked
// host arrays read or written in place) each load waits microseconds, so
// the bandwidth is the number of bytes in flight: 16-byte FP64 pairs, eight
// per thread.
constexpr int CONV_T = 256, CONV_U = 8;
template <typename T> struct ConvPair;
template <> struct ConvPair<float> {
  using T = float2;
  __device__ static float2 make(double a, double b) { return make_float2((float)a, (float)b); }
};
template <> struct ConvPair<double> {
  using T = double2;
  __device__ static double2 make(double a, double b) { return make_double2(a, b); }
};
template <typename DT, typename ST>
__global__ void __launch_bounds__(CONV_T) k_conv_flat(DT* __restrict__ dst, const ST* __restrict__ src,
                                                      long npair) {
  using S2 = typename ConvPair<ST>::T;
  using D2 = typename ConvPair<DT>::T;
  const long p0 = (long)blockIdx.x * (CONV_T * CONV_U) + threadIdx.x;
  S2 v[CONV_U];
#pragma unroll
  for (int u = 0; u < CONV_U; ++u) {
    const long p = p0 + (long)u * CONV_T;
    if (p < npair) v[u] = ((const S2*)src)[p];
  }
#pragma unroll
  for (int u = 0; u < CONV_U; ++u) {
    const long p = p0 + (long)u * CONV_T;
    if (p < npair) ((D2*)dst)[p] = ConvPair<DT>::make((double)v[u].x, (double)v[u].y);
  }
}
// Dense, even-length arrays whose pair loads and stores are aligned take the
// pair kernel.
static bool conv_flat_ok(const void* dst, size_t desz, const void* src, size_t sesz, int nvel, int vstride) {
  return nvel == vstride && nvel % 2 == 0 && (uintptr_t)dst % (2 * desz) == 0 &&
         (uintptr_t)src % (2 * sesz) == 0;
}
template <typename DT, typename ST>
static void conv_flat(DT* dst, const ST* src, long n, cudaStream_t st) {
  const long npair = n / 2;
  const unsigned nb = (unsigned)((npair + CONV_T * CONV_U - 1) / (CONV_T * CONV_U));
  k_conv_flat<DT, ST><<<nb, CONV_T, 0, st>>>(dst, src, npair);
}

__global__ void k_pack_w(double* dst4, const double* src, long ncell, int nw) {
  long c = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= ncell) return;
  for (int k = 0; k < 4; ++k) dst4[c * 4 + k] = k < nw ? src[c * nw + k] : 0.0;
}

// timestep: max over physical cells (src/Solver/solver_main.jl:240-342); one block.
// Maximum over the physical cells of the CFL rate; each block reduces its
// cells, then one atomic max per block on the bit pattern (the rates are
// positive, so their IEEE bits order like unsigned integers and the result
// does not depend on the order of the blocks).
__global__ void k_timestep(DevState s, double umax, double vmax, double* out) {
  __shared__ double red[256];
  const Geo& g = s.g;
  double m = 0.0;
  const long n = (long)g.nx * g.ny;
  for (long t = (long)blockIdx.x * blockDim.x + threadIdx.x; t < n; t += (long)gridDim.x * blockDim.x) {
    int i = (int)(t % g.nx), j = (int)(t / g.nx);
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
  if (threadIdx.x == 0)
    atomicMax((unsigned long long*)out, (unsigned long long)__double_as_longlong(red[0]));
}

// Equilibrium initial distributions of init_fvm (src/Solver/solver_init.jl:
// 119-141, :285-325): h = maxwellian(u, prim) (src/Theory/theory_equilibrium.jl:
// 8-25), b = h K / (2 lambda), for every cell incl. ghosts.  One block per cell.
template <typename R>
__global__ void k_init_eq(DevState s, R* __restrict__ H, R* __restrict__ Bq) {
  const Geo& g = s.g;
  const long c = blockIdx.x;
  const double* p = s.prim + c * 4;
  const double rho = p[0], U = p[1], V = g.D == 2 ? p[2] : 0.0, lam = p[g.NW - 1];
  const double rn = g.D == 1 ? rho * sqrt(lam / PI) : rho * (lam / PI);
  const double cB = g.Kb / (2.0 * lam);
  const long vs = g.vstride;
  for (int v = threadIdx.x; v < g.nvel; v += blockDim.x) {
    const double du = s.u[v] - U;
    double e = du * du;
    if (g.D == 2) {
      const double dv = s.v[v] - V;
      e += dv * dv;
    }
    const double M = rn * exp(-lam * e);
    H[c * vs + v] = (R)M;
    Bq[c * vs + v] = (R)(M * cB);
  }
}

// ------------------------------------------------------------- launchers

static inline unsigned nblk(long n, int bs) { return (unsigned)((n + bs - 1) / bs); }

// Every kernel of a step asks for the largest shared-memory carveout, the one
// the two HBM passes need for their rings.  An SM holds CTAs of kernels with
// different carveouts only after it drains and reconfigures, so when many
// solves share the GPU (a served stream: one CUDA stream per solve) a single
// carveout for all step kernels lets their CTAs share SMs.  Set once per
// kernel and device, on the first (uncaptured) launch.
void prefer_max_shared(const void* fn) {
  static std::mutex m;
  static std::set<std::pair<const void*, int>> done;
  int dev = 0;
  cudaGetDevice(&dev);
  std::lock_guard<std::mutex> lock(m);
  if (done.insert(std::make_pair(fn, dev)).second)
    cudaFuncSetAttribute(fn, cudaFuncAttributePreferredSharedMemoryCarveout,
                         cudaSharedmemCarveoutMaxShared);
}

// Threads per block of the one-thread-per-item FP64 kernels (w slopes, face
// parameters): one warp per block while the items fill fewer than two
// 128-thread blocks per multiprocessor, so a small grid spreads its FP64 work
// over more multiprocessors' FP64 pipes instead of queueing on a few.
static inline int item_bs(const DevState& s, long n) { return n < 2L * s.sm_count * 128 ? 32 : 128; }

int launch_reconstruct(DevState& s, cudaStream_t st) {
  if (s.flux == FLUX_KFVS) return 0;  // KFVS reads no w slopes
  long n = (long)s.g.nx * s.g.ny * s.g.D;
  if (s.g.interp == 1) return 0;
  const int bs = item_bs(s, n);
  void (*fn)(DevState) = s.prec != 0 ? k_wslope<true> : k_wslope<false>;
  prefer_max_shared((const void*)fn);
  fn<<<nblk(n, bs), bs, 0, st>>>(s);
  return 1;
}

template <int D>
static void (*face_param_fn(int flux, bool fast))(DevState, double) {
  switch (flux) {
    case FLUX_KFVS: return fast ? k_face_param<D, FLUX_KFVS, true> : k_face_param<D, FLUX_KFVS, false>;
    case FLUX_KCU: return fast ? k_face_param<D, FLUX_KCU, true> : k_face_param<D, FLUX_KCU, false>;
    default: return fast ? k_face_param<D, FLUX_UGKS, true> : k_face_param<D, FLUX_UGKS, false>;
  }
}

int launch_face_param(DevState& s, double dt, cudaStream_t st) {
  int nf = s.nface_x + s.nface_y;
  const bool fast = s.prec != 0;
  const int bs = item_bs(s, nf);
  void (*fn)(DevState, double) = s.g.D == 2 ? face_param_fn<2>(s.flux, fast) : face_param_fn<1>(s.flux, fast);
  prefer_max_shared((const void*)fn);
  fn<<<nblk(nf, bs), bs, 0, st>>>(s, dt);
  return 1;
}

int launch_wall(DevState& s, double dt, cudaStream_t st) {
  if (s.nwall == 0) return 0;
  void (*fn)(DevState, double);
  if (s.g.D == 1) fn = s.prec == 0 ? k_wall<double, 1> : k_wall<float, 1>;
  else fn = s.prec == 0 ? k_wall<double, 2> : k_wall<float, 2>;
  prefer_max_shared((const void*)fn);
  fn<<<(unsigned)s.nwall, WALL_T, 0, st>>>(s, dt);
  return 1;
}

int launch_evolve(DevState& s, double dt, cudaStream_t st) {
  int n = launch_face_param(s, dt, st);
  n += launch_moments(s, st);
  n += launch_wall(s, dt, st);
  return n;
}

template <int BS>
static void cell_param_bs(DevState& s, double dt, cudaStream_t st) {
  const bool fast = s.prec != 0;
  void (*fn)(DevState, double);
  if (s.g.D == 1) fn = fast ? k_cell_param<1, true, BS> : k_cell_param<1, false, BS>;
  else fn = fast ? k_cell_param<2, true, BS> : k_cell_param<2, false, BS>;
  prefer_max_shared((const void*)fn);
  fn<<<s.res_blocks, BS, 0, st>>>(s, dt);
}

int launch_cell_param(DevState& s, double dt, cudaStream_t st) {
  if (s.cell_bs == 32) cell_param_bs<32>(s, dt, st);
  else cell_param_bs<256>(s, dt, st);
  return 1;
}

template <typename R, int D>
static int finish_t(DevState& s, cudaStream_t st) {
  int n = 0;
  s.cur ^= 1;
  bool fill = false;
  for (int k = 0; k < 2 * D; ++k) fill |= s.g.bc[k] == BC_EXTRA || s.g.bc[k] == BC_PERIOD;
  if (fill) {
    // the ghost kernels write into buffer cur^1 of their DevState copy: pass
    // a copy that still points at the pre-swap index so they fill the new state
    DevState t = s;
    t.cur ^= 1;
    int nrow = D == 2 ? s.g.nyt : 1;
    prefer_max_shared((const void*)k_ghost<R>);
    if (s.g.ngx > 0) { k_ghost<R><<<2 * s.g.ngx * nrow, 128, 0, st>>>(t, 0); ++n; }
    if (D == 2 && s.g.ngy > 0) { k_ghost<R><<<2 * s.g.ngy * s.g.nxt, 128, 0, st>>>(t, 1); ++n; }
  }
  prefer_max_shared((const void*)k_residual<false>);
  k_residual<false><<<1, 256, 0, st>>>(s);
  ++n;
  return n;
}

// ---- grouped launches (kb_group.cu): the per-face / per-cell kernels of one
// step of the 2D FP32 form over all members of a group; ls.grp points at
// the step's member table, the block counts are the members' summed.
void group_small(int kind, const DevState& ls, int flux, int blocks, cudaStream_t st) {
  if (blocks <= 0) return;
  const void* fn = nullptr;
  switch (kind) {
    case GK_WSLOPE:
      fn = (const void*)k_wslope<true, true>;
      prefer_max_shared(fn);
      k_wslope<true, true><<<blocks, 32, 0, st>>>(ls);
      break;
    case GK_FACE: {
      void (*f)(DevState, double) = flux == FLUX_KFVS ? k_face_param<2, FLUX_KFVS, true, true>
                                    : flux == FLUX_KCU ? k_face_param<2, FLUX_KCU, true, true>
                                                       : k_face_param<2, FLUX_UGKS, true, true>;
      prefer_max_shared((const void*)f);
      f<<<blocks, 32, 0, st>>>(ls, 0.0);
      break;
    }
    case GK_WALL:
      fn = (const void*)k_wall<float, 2, true>;
      prefer_max_shared(fn);
      k_wall<float, 2, true><<<blocks, WALL_T, 0, st>>>(ls, 0.0);
      break;
    case GK_CELL:
      fn = (const void*)k_cell_param<2, true, 32, true>;
      prefer_max_shared(fn);
      k_cell_param<2, true, 32, true><<<blocks, 32, 0, st>>>(ls, 0.0);
      break;
    case GK_RES:
      fn = (const void*)k_residual<true>;
      prefer_max_shared(fn);
      k_residual<true><<<blocks, 256, 0, st>>>(ls);
      break;
    default:
      break;
  }
}

int launch_finish(DevState& s, cudaStream_t st) {
  if (s.prec == 0) return s.g.D == 1 ? finish_t<double, 1>(s, st) : finish_t<double, 2>(s, st);
  return s.g.D == 1 ? finish_t<float, 1>(s, st) : finish_t<float, 2>(s, st);
}

int launch_update(DevState& s, double dt, cudaStream_t st) {
  int n = launch_cell_param(s, dt, st);
  n += launch_march(s, dt, st);
  n += launch_finish(s, st);
  return n;
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
  if (ncell * nvel == 0) return 0;
  if (conv_flat_ok(dst, prec == 0 ? 8 : 4, src, 8, nvel, vstride)) {
    if (prec == 0) conv_flat((double*)dst, src, ncell * nvel, st);
    else conv_flat((float*)dst, src, ncell * nvel, st);
    return 1;
  }
  const int cpb = std::max(1, 2048 / nvel);
  const unsigned nb = (unsigned)((ncell + cpb - 1) / cpb);
  if (prec == 0) k_conv<double, double><<<nb, 256, 0, st>>>((double*)dst, src, ncell, nvel, vstride, nvel, cpb);
  else k_conv<float, double><<<nb, 256, 0, st>>>((float*)dst, src, ncell, nvel, vstride, nvel, cpb);
  return 1;
}

int launch_convert_out(double* dst, int prec, const void* src, long ncell, int nvel, int vstride,
                       cudaStream_t st) {
  if (ncell * nvel == 0) return 0;
  if (conv_flat_ok(dst, 8, src, prec == 0 ? 8 : 4, nvel, vstride)) {
    if (prec == 0) conv_flat(dst, (const double*)src, ncell * nvel, st);
    else conv_flat(dst, (const float*)src, ncell * nvel, st);
    return 1;
  }
  const int cpb = std::max(1, 2048 / nvel);
  const unsigned nb = (unsigned)((ncell + cpb - 1) / cpb);
  if (prec == 0)
    k_conv<double, double><<<nb, 256, 0, st>>>(dst, (const double*)src, ncell, nvel, nvel, vstride, cpb);
  else
    k_conv<double, float><<<nb, 256, 0, st>>>(dst, (const float*)src, ncell, nvel, nvel, vstride, cpb);
  return 1;
}

int launch_pack_w(double* dst4, const double* src, long ncell, int nw, cudaStream_t st) {
  k_pack_w<<<nblk(ncell, 256), 256, 0, st>>>(dst4, src, ncell, nw);
  return 1;
}

int launch_timestep(const DevState& s, double umax, double vmax, double* out, cudaStream_t st) {
  cudaMemsetAsync(out, 0, sizeof(double), st);
  const long n = (long)s.g.nx * s.g.ny;
  const unsigned nb = (unsigned)std::min<long>(1184, std::max<long>(1, (n + 255) / 256));
  k_timestep<<<nb, 256, 0, st>>>(s, umax, vmax, out);
  return 1;
}

int launch_init_equilibrium(DevState& s, cudaStream_t st) {
  if (s.prec == 0) k_init_eq<double><<<s.ncell, 128, 0, st>>>(s, (double*)s.h[0], (double*)s.b[0]);
  else k_init_eq<float><<<s.ncell, 128, 0, st>>>(s, (float*)s.h[0], (float*)s.b[0]);
  return 1;
}

}  // namespace kb
