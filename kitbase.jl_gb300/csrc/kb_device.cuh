// kb_device.cuh -- device-side data layout and pointwise physics of the DVM step.
//
// Layout in HBM (one handle):
//   h, b   [cell][vstride] of T (double for KB_PREC_FP64, float for KB_PREC_FP32),
//          velocity index fastest (v = iu + nu*iv), vstride = nvel rounded up to 4;
//          two copies (ping-pong) because the update reads neighbour cells.
//   w, prim [cell][4] double (1D uses 3 entries), sw [cell][2][4] double.
//   per face: FaceParam (interface equilibrium, time integrals, UGKS slopes) and
//   fw [face][4] double in the global frame.
//   per cell: CellParam (new Maxwellian, collision factors, Shakhov coefficients).
// Cells are ordered x fastest with ghost layers included; x faces ((nx+1)*ny,
// i fastest) and y faces (nx*(ny+1)).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

namespace kb {

constexpr double PI = 3.141592653589793238462643383279502884;
constexpr double LOG2E = 1.442695040888963407359924681001892137;

enum { FLUX_KFVS = 0, FLUX_KCU = 1, FLUX_UGKS = 2 };
enum { COLL_BGK = 0, COLL_SHAKHOV = 1 };
enum { BC_FIX = 0, BC_EXTRA = 1, BC_PERIOD = 2, BC_MAXWELL = 3 };

// Geometry of one solve, passed by value to every kernel.
struct Geo {
  int D, NW;
  int nx, ny, ngx, ngy, nxt, nyt;
  int nu, nvel, vstride;
  int interp;  // 1 or 2
  int bc[4];
  double dx, dy, x0, y0;
  double K, gamma, mu_ref, omega, Pr;
  // K in the terms of the second distribution b (its equilibrium
  // B = H K / (2 lambda), the Shakhov factor 2 lambda c^2 + K - 5): K for the
  // 2F models, 0 for the 1F models, which carry no b (src/Solver/step_1f.jl)
  double Kb;
  int nf;  // distributions per cell: 2 (h, b) or 1 (f, held in h; b stays 0)
};

// Interface quantities of one face in the face-local frame.  KFVS uses only
// `mult`; KCU adds the equilibrium part (prim, Mt[0..1], fwa); UGKS all of it.
struct FaceParam {
  double prim[4];   // rho, U_n, U_t, lambda at the interface (1D: U_t = 0)
  double Mt[5];     // time integration coefficients
  double aL[4], aR[4], aT[4];
  double fwa[4];    // analytic (equilibrium) part of fw, local frame, times len
  double mult;      // factor applied to the discrete moments (len or 1)
  double len;       // face length (1 in 1D)
  double Mxi2;      // <xi^4> moment of the interface Maxwellian
  double tr[2];     // transport coefficients incl. len: Th = tr0 un h_face - tr1 un^2 sh
};

// FP32 copy of the per-v coefficients of FaceParam, read by the FP32 kernels.
struct FaceParamF {
  float rho_n;      // rho * (lambda/pi)^(D/2)
  float U, V, lam;  // interface velocity (local frame) and lambda
  float cB;         // K / (2 lambda)
  float Mt[5];
  float aL[4], aR[4], aT[4];
  float Mxi2;
  float len;
  float pad[2];
};

// Per-cell quantities of the update: new Maxwellian, relaxation factor,
// Shakhov coefficients at the old state.
struct CellParam {
  double rho_n, U, V, lam, cB;  // new Maxwellian: rho*(lam/pi)^(D/2), U, V, lambda, K/(2 lambda)
  double dtau;                  // dt / tau
  double inv;                   // 1 / (1 + dt / tau)
  double o_rho_n, oU, oV, olam, ocB;  // old Maxwellian (Shakhov term)
  double sfac;                  // 0.8 (1 - Pr) lambda^2 / rho (old)
  double q0, q1;                // old heat flux
  int upd;                      // 0: copied unchanged, 1: stepped
  int coll;                     // collision model used for this cell
};

struct CellParamF {
  float rho_n, U, V, lam, cB, dtau, inv;
  float o_rho_n, oU, oV, olam, ocB, sf0, sf1;  // sf0/1 = sfac * q0/1
  int upd, coll;
};

// FP32 coefficient block of one face for the velocity-owning kernels.  With
// face-frame velocity (un, ut), c2 = un^2 + ut^2 and the monomials
// m = (un, un^2, un^3, un^2 ut, un^2 c2, un ut, un c2):
//   H  = 2^(E.x + E.y un + E.z ut + E.w c2)            (interface Maxwellian)
//   fh = H (C1 m1 + ... + C7 m7) + T.x un h_f - T.y un^2 dh
//   fb = H (D1 m1 + ... + D7 m7) + T.x un b_f - T.y un^2 db
// where h_f is the upwind face value and dh the unscaled van Leer slope
// (slope * dx), T.y already divided by dx; len is folded in.  C2..C5 and
// D2..D5 depend on the upwind side (aL for un >= 0, aR otherwise).
// For a Maxwell wall face: E is the wall Maxwellian, T.x = len dt,
// T.z = K / (2 lambda_w), T.w = rot.
struct __align__(16) FaceCoef32 {
  float4 E;
  float4 T;   // T3, T4 / dx, C1, D1
  float4 G;   // C6, C7, D6, D7
  float4 Cp;  // C2..C5 for un >= 0
  float4 Dp;  // D2..D5 for un >= 0
  float4 Cm;  // C2..C5 for un < 0
  float4 Dm;  // D2..D5 for un < 0
};

// FP32 coefficients of the pointwise cell update (velocity (u, v), c2):
//   M   = 2^(EM.x + EM.y u + EM.z v + EM.w c2),  MB = M A.x
//   OH  = 2^(EO.x + EO.y u + EO.z v + EO.w c2)   (old Maxwellian, Shakhov)
//   cq  = Q.x + Q.y u + Q.z v,  tl = TL.x + TL.y u + TL.z v + TL.w c2
//   MH += cq (tl - 5) OH,  MB += cq (tl - 3) OH Q.w
//   h   = (h + div * A.w + A.y MH) * A.z
// Cells left unchanged carry A = (0, 0, 1, 0), Q = 0 and EM.x = -200.
struct __align__(16) CellCoef32 {
  float4 EM;
  float4 A;   // cB, dt/tau, 1/(1 + dt/tau), 1/ds
  float4 EO;
  float4 Q;   // Q0, Q1, Q2, old cB
  float4 TL;
};

__host__ __device__ inline int cell_index(const Geo& g, int i, int j) {
  return (j + g.ngy) * g.nxt + (i + g.ngx);
}

// Slope rule along one direction for a cell with 0-based index i (ghosts
// outside [0, n)): 0 none, 1 van Leer (reconstruct3!), 2 forward difference,
// 3 backward difference (reconstruct2! at 2D boundaries).  Follows
// reconstruct! 1D2F (src/Solver/solver_reconstruction.jl:101-153) and 2D2F
// (:475-620): 1D without ghosts leaves cells 1 and nx at zero slope; 2D uses
// one-sided slopes at i = 1 and i = nx; ghost cells keep zero h / b slopes.
__host__ __device__ inline int slope_rule(const Geo& g, int d, int i) {
  if (g.interp == 1) return 0;
  int n = d == 0 ? g.nx : g.ny;
  int ng = d == 0 ? g.ngx : g.ngy;
  if (i < 0 || i >= n) return 0;
  if (g.D == 1) {
    if (ng == 0 && (i == 0 || i == n - 1)) return 0;
    return 1;
  }
  if (i == 0) return 2;
  if (i == n - 1) return 3;
  return 1;
}

// ---------------------------------------------------------------- limiter

// vanleer (src/Reconstruction/recon_limiter.jl:17-19) with fortsign = |1|*sign(y)
template <typename R>
__device__ __forceinline__ R jsign(R y) {
  return y > R(0) ? R(1) : (y < R(0) ? R(-1) : y);
}
template <typename R>
__device__ __forceinline__ R vanleer(R sL, R sR) {
  R aL = fabs(sL), aR = fabs(sR);
  return (jsign(sL) + jsign(sR)) * aL * aR / (aL + aR + R(1.e-7));
}

// Slope of one distribution value at a cell given its neighbours.
template <typename R>
__device__ __forceinline__ R slope_of(int rule, R qm, R q0, R qp, R inv_d) {
  if (rule == 1) return vanleer((q0 - qm) * inv_d, (qp - q0) * inv_d);
  if (rule == 2) return (qp - q0) * inv_d;
  if (rule == 3) return (q0 - qm) * inv_d;
  return R(0);
}
template <>
__device__ __forceinline__ double slope_of<double>(int rule, double qm, double q0, double qp,
                                                   double d) {
  // FP64 path divides like the reference: (q0 - qm) / dx
  if (rule == 1) return vanleer((q0 - qm) / d, (qp - q0) / d);
  if (rule == 2) return (qp - q0) / d;
  if (rule == 3) return (q0 - qm) / d;
  return 0.0;
}

// ---------------------------------------------------- scalar FP64 physics

// conserve_prim!, src/Theory/theory_macro.jl:185-206.  FAST (the FP32 split
// form) multiplies by 1 / rho instead of dividing: GB300 runs FP64 at 1/64 of
// the FP32 rate and each FP64 division costs several FP64 operations.
template <bool FAST = false>
__device__ inline void conserve_prim(const double* W, int nw, double g, double* p) {
  if (FAST) {
    const double r = 1.0 / W[0];
    p[0] = W[0];
    p[1] = W[1] * r;
    if (nw == 3) {
      p[2] = 0.5 * W[0] / ((g - 1.0) * (W[2] - 0.5 * (W[1] * W[1]) * r));
      p[3] = 0.0;
    } else {
      p[2] = W[2] * r;
      p[3] = 0.5 * W[0] / ((g - 1.0) * (W[3] - 0.5 * (W[1] * W[1] + W[2] * W[2]) * r));
    }
    return;
  }
  if (nw == 3) {
    p[0] = W[0];
    p[1] = W[1] / W[0];
    p[2] = 0.5 * W[0] / (g - 1.0) / (W[2] - 0.5 * (W[1] * W[1]) / W[0]);
    p[3] = 0.0;
  } else {
    p[0] = W[0];
    p[1] = W[1] / W[0];
    p[2] = W[2] / W[0];
    p[3] = 0.5 * W[0] / (g - 1.0) / (W[3] - 0.5 * (W[1] * W[1] + W[2] * W[2]) / W[0]);
  }
}

// Transcendental functions of the face and cell parameters.  FAST (the FP32
// split form, whose fluxes are FP32 anyway) evaluates them in FP32 and widens
// the result; otherwise the FP64 library functions.  Arithmetic, divisions
// and the moment recursions stay FP64 either way.
template <bool FAST>
__device__ __forceinline__ double t_exp(double x) { return FAST ? (double)expf((float)x) : exp(x); }
template <bool FAST>
__device__ __forceinline__ double t_erfc(double x) { return FAST ? (double)erfcf((float)x) : erfc(x); }
template <bool FAST>
__device__ __forceinline__ double t_sqrt(double x) { return FAST ? (double)sqrtf((float)x) : sqrt(x); }
template <bool FAST>
__device__ __forceinline__ double t_pow(double x, double y) {
  return FAST ? (double)powf((float)x, (float)y) : pow(x, y);
}

// vhs_collision_time, src/Theory/theory_relaxation.jl:28
template <bool FAST = false>
__device__ inline double vhs_time(double rho, double lam, double mu, double om) {
  return mu * 2.0 * t_pow<FAST>(lam, 1.0 - om) / rho;
}

// Moments of the Gaussian: orders 0..6 of the full / left / right half
// range in u, orders 0..6 in v, orders 0..2 of the internal energy
// (gauss_moments, src/Theory/theory_moments.jl:10-86).
struct GM {
  double Mu[7], MuL[7], MuR[7], Mv[7], Mxi[3];
};

// half: 1 the left half range only (MuL, Mv, Mxi), 2 the right half only,
// 3 everything.  1 / (2 lambda) is formed once and multiplied in.
template <bool FAST = false>
__device__ inline void gauss_moments(const double* p, int nw, double inK, GM& m, int half = 3) {
  double l = p[nw - 1], U = p[1];
  const double hl = 0.5 / l;
  const double sl = t_sqrt<FAST>(l);
  // e = exp(-l U^2) / (2 sqrt(pi l)); FAST evaluates it in FP32 like its exp
  const double e = FAST ? double(0.5f * expf(float(-l * (U * U))) * rsqrtf(float(PI * l)))
                        : 0.5 * exp(-l * (U * U)) / sqrt(PI * l);
  if (half & 1) {
    m.MuL[0] = 0.5 * t_erfc<FAST>(-sl * U);
    m.MuL[1] = U * m.MuL[0] + e;
    for (int i = 2; i <= 6; ++i) m.MuL[i] = U * m.MuL[i - 1] + (i - 1) * hl * m.MuL[i - 2];
  }
  if (half & 2) {
    m.MuR[0] = 0.5 * t_erfc<FAST>(sl * U);
    m.MuR[1] = U * m.MuR[0] - e;
    for (int i = 2; i <= 6; ++i) m.MuR[i] = U * m.MuR[i - 1] + (i - 1) * hl * m.MuR[i - 2];
  }
  if (half == 3)
    for (int i = 0; i <= 6; ++i) m.Mu[i] = m.MuL[i] + m.MuR[i];
  double V = nw == 4 ? p[2] : 0.0;
  m.Mv[0] = 1.0;
  m.Mv[1] = V;
  for (int i = 2; i <= 6; ++i) m.Mv[i] = V * m.Mv[i - 1] + (i - 1) * hl * m.Mv[i - 2];
  m.Mxi[0] = 1.0;
  m.Mxi[1] = inK * hl;
  m.Mxi[2] = (inK * inK + 2.0 * inK) * (hl * hl);
}

// moments_conserve(Mu[, Mv], Mxi, alpha[, beta], delta) for the internal-energy
// forms (src/Theory/theory_moments.jl:98-145).  In 1D Mv is ignored.
__device__ inline void moments_conserve(const double* Mu, const double* Mv, const double* Mxi,
                                        int nw, int a, int bb, int d, double* uv) {
  if (nw == 3) {
    uv[0] = Mu[a] * Mxi[d / 2];
    uv[1] = Mu[a + 1] * Mxi[d / 2];
    uv[2] = 0.5 * (Mu[a + 2] * Mxi[d / 2] + Mu[a] * Mxi[(d + 2) / 2]);
    uv[3] = 0.0;
  } else {
    uv[0] = Mu[a] * Mv[bb] * Mxi[d / 2];
    uv[1] = Mu[a + 1] * Mv[bb] * Mxi[d / 2];
    uv[2] = Mu[a] * Mv[bb + 1] * Mxi[d / 2];
    uv[3] = 0.5 * (Mu[a + 2] * Mv[bb] * Mxi[d / 2] + Mu[a] * Mv[bb + 2] * Mxi[d / 2] +
                   Mu[a] * Mv[bb] * Mxi[(d + 2) / 2]);
  }
}

// moments_conserve_slope (src/Theory/theory_moments.jl:335-369)
__device__ inline void moments_conserve_slope(const double* a, const double* Mu,
                                              const double* Mv, const double* Mxi, int nw,
                                              int al, double* out) {
  double t0[4], t1[4], t2[4], t3[4], t4[4], t5[4];
  if (nw == 3) {
    moments_conserve(Mu, Mv, Mxi, 3, al, 0, 0, t0);
    moments_conserve(Mu, Mv, Mxi, 3, al + 1, 0, 0, t1);
    moments_conserve(Mu, Mv, Mxi, 3, al + 2, 0, 0, t2);
    moments_conserve(Mu, Mv, Mxi, 3, al, 0, 2, t3);
    for (int k = 0; k < 3; ++k)
      out[k] = a[0] * t0[k] + a[1] * t1[k] + 0.5 * a[2] * t2[k] + 0.5 * a[2] * t3[k];
    out[3] = 0.0;
  } else {
    moments_conserve(Mu, Mv, Mxi, 4, al, 0, 0, t0);
    moments_conserve(Mu, Mv, Mxi, 4, al + 1, 0, 0, t1);
    moments_conserve(Mu, Mv, Mxi, 4, al, 1, 0, t2);
    moments_conserve(Mu, Mv, Mxi, 4, al + 2, 0, 0, t3);
    moments_conserve(Mu, Mv, Mxi, 4, al, 2, 0, t4);
    moments_conserve(Mu, Mv, Mxi, 4, al, 0, 2, t5);
    for (int k = 0; k < 4; ++k)
      out[k] = a[0] * t0[k] + a[1] * t1[k] + a[2] * t2[k] + 0.5 * a[3] * t3[k] +
               0.5 * a[3] * t4[k] + 0.5 * a[3] * t5[k];
  }
}

// pdf_slope(prim, sw, inK) (src/Theory/theory_pdf.jl:11-49); FAST forms the
// three reciprocals once (see conserve_prim)
template <bool FAST = false>
__device__ inline void pdf_slope(const double* p, const double* s, int nw, double inK,
                                 double* sl) {
  if (FAST) {
    const int e = nw - 1;  // energy slot
    const double r0 = 1.0 / p[0], rl = 1.0 / p[e], rk = 1.0 / (inK + double(nw - 2));
    const double U = p[1], V = nw == 4 ? p[2] : 0.0, sv = nw == 4 ? s[2] : 0.0;
    const double q2 = U * U + V * V, c = 0.5 * (inK + double(nw - 2)) * rl;
    const double se = 4.0 * (p[e] * p[e]) * rk * r0 *
                      (2.0 * s[e] - 2.0 * U * s[1] - 2.0 * V * sv + s[0] * (q2 - c));
    const double tl = 2.0 * p[e] * r0;
    const double s1 = tl * (s[1] - U * s[0]) - U * se;
    const double s2 = tl * (sv - V * s[0]) - V * se;
    sl[0] = s[0] * r0 - U * s1 - V * s2 - 0.5 * (q2 + c) * se;
    sl[1] = s1;
    if (nw == 4) {
      sl[2] = s2;
      sl[3] = se;
    } else {
      sl[2] = se;
      sl[3] = 0.0;
    }
    return;
  }
  if (nw == 3) {
    sl[2] = 4.0 * (p[2] * p[2]) / (inK + 1.0) / p[0] *
            (2.0 * s[2] - 2.0 * p[1] * s[1] + s[0] * ((p[1] * p[1]) - 0.5 * (inK + 1.0) / p[2]));
    sl[1] = 2.0 * p[2] / p[0] * (s[1] - p[1] * s[0]) - p[1] * sl[2];
    sl[0] = s[0] / p[0] - p[1] * sl[1] - 0.5 * ((p[1] * p[1]) + 0.5 * (inK + 1.0) / p[2]) * sl[2];
    sl[3] = 0.0;
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

// ------------------------------------------- compensated FP32 accumulation

// Double-float accumulator: (hi, lo) with |lo| <= ulp(hi)/2 after each add.
// Knuth's TwoSum makes every addition error-free, so the pair carries about
// 44 significant bits; it is converted exactly to FP64 (hi + lo) before the
// FP64 combination across threads.
struct DF {
  float hi, lo;
};
__device__ __forceinline__ void df_add(DF& a, float x) {
  float s = a.hi + x;
  float bp = s - a.hi;
  float e = (a.hi - (s - bp)) + (x - bp);
  a.hi = s;
  a.lo += e;
}
__device__ __forceinline__ DF df_merge(DF a, DF b) {
  float s = a.hi + b.hi;
  float bp = s - a.hi;
  float e = (a.hi - (s - bp)) + (b.hi - bp);
  e += a.lo + b.lo;
  float hi = s + e;
  float lo = e - (hi - s);
  DF r;
  r.hi = hi;
  r.lo = lo;
  return r;
}
__device__ __forceinline__ DF df_shfl_xor(DF a, int m) {
  DF r;
  r.hi = __shfl_xor_sync(0xffffffffu, a.hi, m);
  r.lo = __shfl_xor_sync(0xffffffffu, a.lo, m);
  return r;
}
__device__ __forceinline__ double df_warp_sum(DF a) {
#pragma unroll
  for (int m = 16; m >= 1; m >>= 1) a = df_merge(a, df_shfl_xor(a, m));
  return (double)a.hi + (double)a.lo;
}

__device__ __forceinline__ double warp_sum(double x) {
#pragma unroll
  for (int m = 16; m >= 1; m >>= 1) x += __shfl_xor_sync(0xffffffffu, x, m);
  return x;
}

// Accumulator selected by the storage type: FP64 path sums in double, FP32
// path in compensated double-float.
template <typename R>
struct Acc;
template <>
struct Acc<double> {
  double s;
  __device__ __forceinline__ Acc() : s(0.0) {}
  __device__ __forceinline__ void add(double x) { s += x; }
  __device__ __forceinline__ double total() { return warp_sum(s); }
};
template <>
struct Acc<float> {
  DF s;
  __device__ __forceinline__ Acc() { s.hi = 0.f; s.lo = 0.f; }
  __device__ __forceinline__ void add(float x) { df_add(s, x); }
  __device__ __forceinline__ double total() { return df_warp_sum(s); }
};

// exp of a Maxwellian exponent: accurate FP64 exp on the FP64 path, ex2.approx
// with a pre-scaled argument on the FP32 path.
__device__ __forceinline__ double mexp(double x) { return exp(x); }
__device__ __forceinline__ float mexp(float x) { return exp2f(x * float(LOG2E)); }

}  // namespace kb
