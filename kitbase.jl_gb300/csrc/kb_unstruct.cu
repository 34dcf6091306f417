// kb_unstruct.cu -- the DVM step of 2D2F2V solves on triangle meshes
// (KitBase's unstructured 2F path: evolve! US2F,
// src/Solver/solver_evolution.jl:945-1035; update! US2F,
// src/Solver/solver_update.jl:414-471; triangle step!,
// src/Solver/step_2f.jl:256-326; update_boundary! US2F,
// src/Solver/update_boundary.jl:575-594; timestep for unstructured cells,
// src/Solver/solver_main.jl:398-420).
//
// One fused kernel per step, one CTA per stepped cell: the CTA reads its own
// h, b and its three neighbours' (gathered through the index tables), forms
// the first-order KFVS flux of each of its three faces for every velocity and
// the faces' moments fw (block sums), updates w and prim, and relaxes h, b
// with the fluxes formed again in a second sweep (the neighbours' values are
// then in L1).  The face fluxes are never stored: each interior face is
// formed by both of its cells, with the same inputs, the same operation
// order (explicitly rounded operations, no contraction) and the same
// velocity partition of the block sums, so both sides see bit-identical fw
// and the update stays conservative.  New h, b go to the other buffer of a
// ping-pong pair (neighbours must read the old state); fixed cells hold the
// same values in both.  The extrapolated boundary cells are then set in
// dependency levels (see kb_us_create) that reproduce the reference's
// sequential cell-order loop.  The plain form computes in FP64 throughout;
// the FP32 split form stores h, b and forms the per-velocity arithmetic in
// FP32, with the block sums in compensated double-float and fw, w, prim, tau
// in FP64.  DRAM traffic per step is one read and one write of the stepped
// cells' h, b (the neighbours' re-reads hit L2 for meshes numbered with
// locality), 16 B per cell-velocity in the FP32 form.
// 2D1F2V (cfg->nf = 1: evolve! / update! / update_boundary! US1F, the
// 2D1F2V triangle step!, src/Solver/step_1f.jl:228-285) runs the same
// kernels with b held at zero and its equilibrium K / (2 lambda) M replaced
// by 0, which reduces every term to the 1F formula (flux_kfvs! 1F2V,
// src/Flux/flux_kfvs.jl:615-650).
#include <cuda_runtime.h>

#include <algorithm>
#include <string>
#include <vector>

#include "../../include/kitgpu.h"
#include "kb_device.cuh"
#include "kb_kernels.cuh"

namespace kb {

// FP64 face record of a stepped cell (32-byte aligned, one vector load pair)
struct alignas(32) UsG64 {
  double n1, n2, len, sgn;
};

struct UsDev {
  int ncell, nface, nvel, vstride, coll, nstep, navg;
  const int* cell_nb;        // [ncell][3], -1 where no cell
  const int* cell_type;      // [ncell]: 0 stepped, 1 fixed, 3 mean of two neighbours
  const int4* step_rec;      // [nstep] stepped (type-0) cell, its neighbours over its faces 0..2
  const float4* step_geo32;  // [nstep][3] per face: n1, n2, len, sg |n|^2 (FP32 form)
  const UsG64* step_geo64;   // [nstep][3] the same in FP64
  const int* avg_list;       // type-3 cells by dependency level [navg]
  const double* cell_iarea;  // [ncell] 1 / area (one IEEE division per cell, on the host)
  const double* cell_mindx;  // [ncell] smallest centre-to-edge distance
  const double* u;           // velocity grid, FP64
  const double* v;
  const double* wt;
  const float* uf;           // and its FP32 copies for the FP32 form
  const float* vf;
  const float* wtf;
  double* w;      // [ncell][4]
  double* prim;   // [ncell][4]
  double* bres;   // [step CTAs][8]: sums of (w - w_old)^2, |w| over each CTA's cells, last step
  double* tmax;   // [1]
  double* residual;  // [4]
  int* status;
  double K, Kb, gamma, mu_ref, omega, Pr, umax, vmax;  // Kb = K (2F) or 0 (1F: b absent)
};

constexpr int US_T = 128;
constexpr int US_W = US_T / 32;
constexpr int US_BLK = 8;  // velocities summed plainly before a compensated flush

// explicitly rounded arithmetic (never contracted), so that both cells of a
// face form its flux and moments bit-identically
__device__ __forceinline__ double rmul(double a, double b) { return __dmul_rn(a, b); }
__device__ __forceinline__ double radd(double a, double b) { return __dadd_rn(a, b); }
__device__ __forceinline__ double rsub(double a, double b) { return __dsub_rn(a, b); }
__device__ __forceinline__ double rfma(double a, double b, double c) { return __fma_rn(a, b, c); }
__device__ __forceinline__ float rmul(float a, float b) { return __fmul_rn(a, b); }
__device__ __forceinline__ float radd(float a, float b) { return __fadd_rn(a, b); }
__device__ __forceinline__ float rsub(float a, float b) { return __fsub_rn(a, b); }
__device__ __forceinline__ float rfma(float a, float b, float c) { return __fmaf_rn(a, b, c); }

// Per cell and velocity, the signed sums over the cell's three faces of
// the first-order KFVS fluxes (flux_kfvs! 2F2V / 1F2V of first-order states,
// src/Flux/flux_kfvs.jl:615-700; heaviside(0) = 1):
//   Dh = sum_j sg_j fh_j,  Db = sum_j sg_j fb_j,  Dn = sum_j sg_j |n_j|^2 fh_j
// with sg_j = +1 where the normal points out of the cell.  The reference
// forms each face's moments fw in the face frame (vn, vt) and rotates them
// back (global_frame, src/Geometry/geo_general.jl:6-26); with its normals of
// length |n| = |d| / (|d| + 1e-6) that equals |n|^2 times the global-frame
// moments, so the cell's sum_j sg_j fw_j is
//   (sum w Dh, sum u w Dn, sum v w Dn, (sum c^2 w Dn + sum w Db) / 2).
// Each face flux is formed with explicitly rounded operations (never
// contracted) from the same inputs in both of its cells, so both see the
// same per-velocity values.
template <typename R>
struct UsFace {
  R n1, n2, a, l;  // flux = ((a vn) s) l: FP64 a = dt, l = len; FP32 a = dt len, l = 1
  R sg, sgn;       // sg and sg |n|^2
  int nb;          // the other cell
  bool left;       // the cell is the face's first cell
};

template <typename R>
__device__ __forceinline__ void us_flux(const UsFace<R>& F, R u, R v, R hc, R bc, R hn, R bn,
                                        R& fh, R& fb) {
  const R vn = rfma(u, F.n1, rmul(v, F.n2));
  const bool own = (vn >= R(0)) == F.left;
  const R hs = own ? hc : hn, bs = own ? bc : bn;
  const R av = rmul(F.a, vn);
  if (sizeof(R) == 8) {
    fh = rmul(rmul(av, hs), F.l);
    fb = rmul(rmul(av, bs), F.l);
  } else {
    fh = rmul(av, hs);
    fb = rmul(av, bs);
  }
}

constexpr int US_CB = 32;   // most cells of one CTA (one lane each in the cell phase)
constexpr int US_NM = 8;    // block sums per cell: 5 moments, 2 heat-flux sums, 1 spare
constexpr int US_NP = 16;   // per-cell parameters of the relaxation

// warp reduce-scatter of 8 per-lane partial sums (FP64, or double-float in
// the FP32 form): three halving exchanges leave lane l with the partial of
// sum (l >> 2) & 7 over its 8-lane group, two more finish it; lanes with
// (l & 3) == 0 then hold the 8 totals.
__device__ __forceinline__ double us_merge(double a, double b) { return a + b; }
__device__ __forceinline__ DF us_merge(DF a, DF b) { return df_merge(a, b); }
__device__ __forceinline__ double us_shfl(double a, int m) { return __shfl_xor_sync(0xffffffffu, a, m); }
__device__ __forceinline__ DF us_shfl(DF a, int m) { return df_shfl_xor(a, m); }
__device__ __forceinline__ double us_value(double a) { return a; }
__device__ __forceinline__ double us_value(DF a) { return (double)a.hi + (double)a.lo; }
template <typename V>
__device__ __forceinline__ double us_reduce8(const V (&x)[8], int lane) {
  const bool b4 = lane & 16, b3 = lane & 8, b2 = lane & 4;
  V y[4], z[2];
#pragma unroll
  for (int k = 0; k < 4; ++k) y[k] = us_merge(b4 ? x[k + 4] : x[k], us_shfl(b4 ? x[k] : x[k + 4], 16));
#pragma unroll
  for (int k = 0; k < 2; ++k) z[k] = us_merge(b3 ? y[k + 2] : y[k], us_shfl(b3 ? y[k] : y[k + 2], 8));
  V t = us_merge(b2 ? z[1] : z[0], us_shfl(b2 ? z[0] : z[1], 4));
  t = us_merge(t, us_shfl(t, 2));
  t = us_merge(t, us_shfl(t, 1));
  return us_value(t);
}

template <typename R> struct Vec2;
template <> struct Vec2<float> { using T = float2; };
template <> struct Vec2<double> { using T = double2; };

// Packed FP32 pair arithmetic (one instruction for both velocities of a
// lane's pair) and the base-2 exponential of a pre-scaled argument.
__device__ __forceinline__ float2 p2add(float2 a, float2 b) { return __fadd2_rn(a, b); }
__device__ __forceinline__ float2 p2mul(float2 a, float2 b) { return __fmul2_rn(a, b); }
__device__ __forceinline__ float2 p2fma(float2 a, float2 b, float2 c) { return __ffma2_rn(a, b, c); }
__device__ __forceinline__ float2 p2sub(float2 a, float2 b) {
  unsigned long long A = *reinterpret_cast<unsigned long long*>(&a);
  unsigned long long B = *reinterpret_cast<unsigned long long*>(&b), C;
  asm("sub.rn.f32x2 %0, %1, %2;" : "=l"(C) : "l"(A), "l"(B));
  return *reinterpret_cast<float2*>(&C);
}
__device__ __forceinline__ float2 p2s(float x) { return make_float2(x, x); }
__device__ __forceinline__ float us_ex2(float x) {
  float y;
  asm("ex2.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
  return y;
}
__device__ __forceinline__ float2 p2ex2(float2 a) { return make_float2(us_ex2(a.x), us_ex2(a.y)); }

// Outward first-order KFVS flux of one face for a velocity pair, FP32 form:
// with vo = u no1 + v no2 the normal velocity along the cell's outward
// normal (sg n) and ao = (dt len) vo, the flux out of the cell is
// max(ao, 0) h_cell + min(ao, 0) h_neighbour (heaviside(0) = 1 and a zero
// normal velocity carries nothing).  Its neighbour forms exactly the
// negated value (negation is exact), so both cells of a face agree bit for
// bit.
__device__ __forceinline__ void us_flux2(float no1, float no2, float a, float2 u2, float2 v2, float2 hc,
                                         float2 bc, float2 hn, float2 bn, float2& fh, float2& fb) {
  const float2 ao = p2mul(p2s(a), p2fma(u2, p2s(no1), p2mul(v2, p2s(no2))));
  const float2 ap = make_float2(fmaxf(ao.x, 0.f), fmaxf(ao.y, 0.f));
  const float2 am = make_float2(fminf(ao.x, 0.f), fminf(ao.y, 0.f));
  fh = p2fma(ap, hc, p2mul(am, hn));
  fb = p2fma(ap, bc, p2mul(am, bn));
}

// A stepped cell's face geometry: normal, length and sg |n|^2 (its sign is
// the orientation: + where the cell is the face's first cell)
template <typename R>
struct UsGeo {
  R n1, n2, len, sgn;
};

// Stage the records of a CTA's nloc cells (cell, neighbours, per-face
// geometry) into shared memory: one coalesced read per CTA, so the warps'
// cell loops hold no prefetched record in registers.
__device__ __forceinline__ void us_stage_rec(const UsDev& d, int c0, int nloc, int4* RS, float4* GS) {
  for (int t = threadIdx.x; t < nloc; t += US_T) RS[t] = __ldg(d.step_rec + c0 + t);
  for (int t = threadIdx.x; t < 3 * nloc; t += US_T) GS[t] = __ldg(d.step_geo32 + 3L * c0 + t);
}
__device__ __forceinline__ void us_stage_rec(const UsDev& d, int c0, int nloc, int4* RS, UsG64* GS) {
  for (int t = threadIdx.x; t < nloc; t += US_T) RS[t] = __ldg(d.step_rec + c0 + t);
  for (int t = threadIdx.x; t < 3 * nloc; t += US_T) GS[t] = d.step_geo64[3L * c0 + t];
}
__device__ __forceinline__ void us_geo(const float4& q, UsGeo<float>& g) {
  g.n1 = q.x;
  g.n2 = q.y;
  g.len = q.z;
  g.sgn = q.w;
}
__device__ __forceinline__ void us_geo(const UsG64& q, UsGeo<double>& g) {
  g.n1 = q.n1;
  g.n2 = q.n2;
  g.len = q.len;
  g.sgn = q.sgn;
}
template <typename R> struct UsGeoRow;
template <> struct UsGeoRow<float> { using T = float4; };
template <> struct UsGeoRow<double> { using T = UsG64; };

// One CTA of US_T threads steps cb consecutive cells of the step list:
// (1) each warp takes cells wid, wid + 4, ..., forms Dh, Db (kept in shared
// memory, two velocities per lane and iteration) and the cell's velocity
// sums (blocked, compensated in the FP32 form); (2) warp 0 does each cell's
// FP64 algebra on its own lane (w update, conserve_prim, residual partials,
// tau, equilibrium and Shakhov parameters); (3) the warps relax h, b of
// their cells.  The FP32 form takes its face geometry from an FP32 table and
// evaluates the cell's transcendentals in FP32 (GB300 runs FP64 at a small
// fraction of the FP32 rate, so per-cell FP64 work is kept to the lane-per-
// cell phase).  Launch bounds: the FP32 form fits 7 CTAs per SM (BGK, 72
// registers) or 6 (Shakhov, whose heat-flux sums need more registers; 7 would
// spill); the FP64 form 3.
template <typename R, bool SHAK>
__global__ void __launch_bounds__(US_T, sizeof(R) == 4 ? (SHAK ? 6 : 7) : 3)
    k_us_step(UsDev d, double dt, int cb, const R* __restrict__ hin,
                                                  const R* __restrict__ bin, R* __restrict__ hout,
                                                  R* __restrict__ bout) {
  using R2 = typename Vec2<R>::T;
  constexpr bool FAST = sizeof(R) == 4;
  extern __shared__ __align__(16) unsigned char us_smem[];
  double* S = (double*)us_smem;                  // [cb][US_NM]
  R* P = (R*)(S + cb * US_NM);                   // [cb][US_NP] (room for doubles)
  R* D = (R*)(S + cb * (US_NM + US_NP));         // [cb][2][vstride]: Dh, Db
  using GR = typename UsGeoRow<R>::T;
  GR* GS = (GR*)(D + (long)cb * 2 * d.vstride);  // [cb][3] face geometry
  int4* RS = (int4*)(GS + 3 * cb);               // [cb] cell and neighbours
  const int tid = threadIdx.x, lane = tid & 31, wid = tid >> 5;
  const int c0 = blockIdx.x * cb;
  const int nloc = min(cb, d.nstep - c0);
  const R2* U2 = (const R2*)(FAST ? (const void*)d.uf : (const void*)d.u);
  const R2* V2 = (const R2*)(FAST ? (const void*)d.vf : (const void*)d.v);
  const R2* W2 = (const R2*)(FAST ? (const void*)d.wtf : (const void*)d.wt);
  const long vs = d.vstride;
  const int np = d.vstride >> 1;
  constexpr bool shak = SHAK;
  const R rdt = R(dt);

  // (1) face fluxes and velocity sums.  The records of the CTA's cells (the
  // cell, its three neighbours, and per face n1, n2, len and sg |n|^2) are
  // staged in shared memory first.
  us_stage_rec(d, c0, nloc, RS, GS);
  __syncthreads();
  for (int i = wid; i < nloc; i += US_W) {
    const int4 rec = RS[i];
    const int c = rec.x;
    UsFace<R> F[3];
#pragma unroll
    for (int j = 0; j < 3; ++j) {
      UsGeo<R> geo;
      us_geo(GS[3 * i + j], geo);
      F[j].n1 = geo.n1;
      F[j].n2 = geo.n2;
      F[j].a = FAST ? rmul(rdt, geo.len) : R(dt);
      F[j].l = FAST ? R(1) : geo.len;
      F[j].sgn = geo.sgn;
      F[j].left = geo.sgn > R(0);
      F[j].sg = F[j].left ? R(1) : R(-1);
    }
    F[0].nb = rec.y;
    F[1].nb = rec.z;
    F[2].nb = rec.w;
    const R2* Hc = (const R2*)(hin + (long)c * vs);
    const R2* Bc = (const R2*)(bin + (long)c * vs);
    const R2* H0 = (const R2*)(hin + (long)F[0].nb * vs);
    const R2* B0 = (const R2*)(bin + (long)F[0].nb * vs);
    const R2* H1 = (const R2*)(hin + (long)F[1].nb * vs);
    const R2* B1 = (const R2*)(bin + (long)F[1].nb * vs);
    const R2* H2 = (const R2*)(hin + (long)F[2].nb * vs);
    const R2* B2 = (const R2*)(bin + (long)F[2].nb * vs);
    R Uo = R(0), Vo = R(0);
    if (shak) {
      Uo = R(d.prim[4L * c + 1]);
      Vo = R(d.prim[4L * c + 2]);
    }
    R2* Dh = (R2*)(D + (long)i * 2 * vs);
    R2* Db = (R2*)(D + (long)i * 2 * vs + vs);
    R pp[US_NM];
    Acc<R> acc[US_NM];
#pragma unroll
    for (int k = 0; k < US_NM; ++k) pp[k] = R(0);
    int blk = 0;
    if constexpr (FAST) {
      float no[3][2], aa[3], nn[3];
#pragma unroll
      for (int j = 0; j < 3; ++j) {
        no[j][0] = F[j].left ? F[j].n1 : -F[j].n1;
        no[j][1] = F[j].left ? F[j].n2 : -F[j].n2;
        aa[j] = F[j].a;
        nn[j] = fabsf(F[j].sgn);
      }
      float2 Pk[US_NM];
#pragma unroll
      for (int k = 0; k < US_NM; ++k) Pk[k] = make_float2(0.f, 0.f);
      const float2 Uo2 = p2s(Uo), Vo2 = p2s(Vo);
      for (int q = lane; q < np; q += 32) {
        const float2 u2 = U2[q], v2 = V2[q], w2 = W2[q];
        const float2 hc2 = Hc[q], bc2 = Bc[q];
        const float2 h0 = H0[q], b0 = B0[q], h1 = H1[q], b1 = B1[q], h2 = H2[q], b2 = B2[q];
        float2 fh, fb, dh2, db2, dn2;
        us_flux2(no[0][0], no[0][1], aa[0], u2, v2, hc2, bc2, h0, b0, fh, fb);
        dh2 = fh;
        db2 = fb;
        dn2 = p2mul(p2s(nn[0]), fh);
        us_flux2(no[1][0], no[1][1], aa[1], u2, v2, hc2, bc2, h1, b1, fh, fb);
        dh2 = p2add(dh2, fh);
        db2 = p2add(db2, fb);
        dn2 = p2fma(p2s(nn[1]), fh, dn2);
        us_flux2(no[2][0], no[2][1], aa[2], u2, v2, hc2, bc2, h2, b2, fh, fb);
        dh2 = p2add(dh2, fh);
        db2 = p2add(db2, fb);
        dn2 = p2fma(p2s(nn[2]), fh, dn2);
        Dh[q] = dh2;
        Db[q] = db2;
        const float2 wn = p2mul(w2, dn2);
        Pk[0] = p2fma(w2, dh2, Pk[0]);
        Pk[1] = p2fma(u2, wn, Pk[1]);
        Pk[2] = p2fma(v2, wn, Pk[2]);
        Pk[3] = p2fma(p2fma(u2, u2, p2mul(v2, v2)), wn, Pk[3]);
        Pk[4] = p2fma(w2, db2, Pk[4]);
        if (shak) {  // heat_flux 2F2V of the old state (src/Theory/theory_moments.jl:567-578)
          const float2 cu = p2sub(u2, Uo2), cv = p2sub(v2, Vo2);
          const float2 t = p2mul(w2, p2fma(p2fma(cu, cu, p2mul(cv, cv)), hc2, bc2));
          Pk[5] = p2fma(cu, t, Pk[5]);
          Pk[6] = p2fma(cv, t, Pk[6]);
        }
      }
      // the pair partials (np / 32 pairs per lane) enter the compensated
      // cross-lane sums
#pragma unroll
      for (int k = 0; k < US_NM; ++k) {
        acc[k].add(Pk[k].x);
        acc[k].add(Pk[k].y);
      }
    } else
    for (int q = lane; q < np; q += 32) {
      const R2 u2 = U2[q], v2 = V2[q], w2 = W2[q];
      const R2 hc2 = Hc[q], bc2 = Bc[q];
      const R2 h0 = H0[q], b0 = B0[q], h1 = H1[q], b1 = B1[q], h2 = H2[q], b2 = B2[q];
      R2 dh2, db2;
#pragma unroll
      for (int e = 0; e < 2; ++e) {
        const R u = e ? u2.y : u2.x, vv = e ? v2.y : v2.x, om = e ? w2.y : w2.x;
        const R hc = e ? hc2.y : hc2.x, bc = e ? bc2.y : bc2.x;
        R fh0, fb0, fh1, fb1, fh2, fb2;
        us_flux(F[0], u, vv, hc, bc, e ? h0.y : h0.x, e ? b0.y : b0.x, fh0, fb0);
        us_flux(F[1], u, vv, hc, bc, e ? h1.y : h1.x, e ? b1.y : b1.x, fh1, fb1);
        us_flux(F[2], u, vv, hc, bc, e ? h2.y : h2.x, e ? b2.y : b2.x, fh2, fb2);
        const R dh = F[0].sg * fh0 + F[1].sg * fh1 + F[2].sg * fh2;
        const R db = F[0].sg * fb0 + F[1].sg * fb1 + F[2].sg * fb2;
        const R dn = F[0].sgn * fh0 + F[1].sgn * fh1 + F[2].sgn * fh2;
        if (e) { dh2.y = dh; db2.y = db; } else { dh2.x = dh; db2.x = db; }
        const R wn = om * dn;
        pp[0] += om * dh;
        pp[1] += u * wn;
        pp[2] += vv * wn;
        pp[3] += (u * u + vv * vv) * wn;
        pp[4] += om * db;
        if (shak) {  // heat_flux 2F2V of the old state (src/Theory/theory_moments.jl:567-578)
          const R cu = u - Uo, cv = vv - Vo;
          const R t = om * ((cu * cu + cv * cv) * hc + bc);
          pp[5] += cu * t;
          pp[6] += cv * t;
        }
      }
      Dh[q] = dh2;
      Db[q] = db2;
      if (++blk == US_BLK) {
#pragma unroll
        for (int k = 0; k < US_NM; ++k) {
          acc[k].add(pp[k]);
          pp[k] = R(0);
        }
        blk = 0;
      }
    }
    decltype(acc[0].s) x[US_NM];
#pragma unroll
    for (int k = 0; k < US_NM; ++k) {
      acc[k].add(pp[k]);
      x[k] = acc[k].s;
    }
    const double t = us_reduce8(x, lane);
    if ((lane & 3) == 0) S[i * US_NM + (lane >> 2)] = t;
  }
  __syncthreads();

  // (2) the cell algebra, one lane per cell (step! 2D2F2V on a triangle,
  // src/Solver/step_2f.jl:256-326; 2D1F2V src/Solver/step_1f.jl:228-285)
  if (wid == 0) {
    double rr[8] = {0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0};
    if (lane < nloc) {
      const int c = RS[lane].x;
      const double* Sc = S + lane * US_NM;
      double* w = d.w + 4L * c;
      double* p = d.prim + 4L * c;
      const double rho_o = p[0], U_o = p[1], V_o = p[2], lam_o = p[3];
      const double ia = d.cell_iarea[c];
      const double A[4] = {Sc[0], Sc[1], Sc[2], 0.5 * (Sc[3] + Sc[4])};
      double wo[4], pn[4];
      for (int k = 0; k < 4; ++k) {
        wo[k] = w[k];
        w[k] -= A[k] * ia;
      }
      conserve_prim<FAST>(w, 4, d.gamma, pn);
      for (int k = 0; k < 4; ++k) {
        p[k] = pn[k];
        rr[k] = (w[k] - wo[k]) * (w[k] - wo[k]);
        rr[4 + k] = fabs(w[k]);
      }
      if (!(pn[0] > 0.0) || !(pn[3] > 0.0) || !isfinite(pn[0]) || !isfinite(pn[3])) atomicOr(d.status, 1);
      R* Pc = P + lane * US_NP;
      if constexpr (FAST) {
        // The relaxation's FP32 coefficients are formed in FP32: FP64
        // division runs on GB300's slow FP64 pipe while the CTA's other
        // warps wait at the barrier.
        const float rho = (float)pn[0], lam = (float)pn[3], Kb = (float)d.Kb;
        const float tau = (float)(2.0 * d.mu_ref) * powf(lam, (float)(1.0 - d.omega)) / rho;
        const float k = (float)dt / tau;
        Pc[0] = rho * (lam * (float)(1.0 / PI));  // Maxwellian amplitude
        Pc[1] = R(pn[1]);
        Pc[2] = R(pn[2]);
        Pc[3] = lam;
        Pc[4] = Kb / (2.f * lam);  // B / H
        Pc[5] = k;
        Pc[6] = 1.f / (1.f + k);
        Pc[7] = R(ia);
        if (shak) {  // shakhov 2F2V of the old state (src/Theory/theory_equilibrium.jl:227-238)
          const float ro = (float)rho_o, lo = (float)lam_o;
          const float sfac = (float)(0.8 * (1.0 - d.Pr)) * (lo * lo) / ro;
          Pc[8] = sfac * 0.5f * (float)Sc[5];
          Pc[9] = sfac * 0.5f * (float)Sc[6];
          Pc[10] = ro * (lo * (float)(1.0 / PI));
          Pc[11] = Kb / (2.f * lo);
          Pc[12] = lo;
          Pc[13] = R(U_o);
          Pc[14] = R(V_o);
        }
      } else {
        const double k = dt / vhs_time<FAST>(pn[0], pn[3], d.mu_ref, d.omega);
        Pc[0] = R(pn[0] * (pn[3] / PI));  // Maxwellian amplitude
        Pc[1] = R(pn[1]);
        Pc[2] = R(pn[2]);
        Pc[3] = R(pn[3]);
        Pc[4] = R(d.Kb / (2.0 * pn[3]));  // B / H
        Pc[5] = R(k);
        Pc[6] = R(1.0 / (1.0 + k));
        Pc[7] = R(ia);
        if (shak) {  // shakhov 2F2V of the old state (src/Theory/theory_equilibrium.jl:227-238)
          const double sfac = 0.8 * (1.0 - d.Pr) * (lam_o * lam_o) / rho_o;
          Pc[8] = R(sfac * 0.5 * Sc[5]);
          Pc[9] = R(sfac * 0.5 * Sc[6]);
          Pc[10] = R(rho_o * (lam_o / PI));
          Pc[11] = R(d.Kb / (2.0 * lam_o));
          Pc[12] = R(lam_o);
          Pc[13] = R(U_o);
          Pc[14] = R(V_o);
        }
      }
    }
    // residual partials of update! (src/Solver/solver_update.jl:465-467)
    // summed over the CTA's cells in a fixed order
    const double t = us_reduce8(rr, lane);
    if ((lane & 3) == 0) d.bres[8L * blockIdx.x + (lane >> 2)] = t;
  }
  __syncthreads();

  // (3) relaxation of h, b
  const R Km5 = R(d.Kb - 5.0), Km3 = R(d.Kb - 3.0);
  for (int i = wid; i < nloc; i += US_W) {
    const int c = RS[i].x;
    const R* Pc = P + i * US_NP;
    const R rn = Pc[0], U = Pc[1], V = Pc[2], lam = Pc[3], cB = Pc[4];
    const R kk = Pc[5], i1k = Pc[6], ia = Pc[7];
    R fq0 = R(0), fq1 = R(0), orn = R(0), ocB = R(0), olam = R(0), Uo = R(0), Vo = R(0);
    if (shak) {
      fq0 = Pc[8];
      fq1 = Pc[9];
      orn = Pc[10];
      ocB = Pc[11];
      olam = Pc[12];
      Uo = Pc[13];
      Vo = Pc[14];
    }
    const R2* Hc = (const R2*)(hin + (long)c * vs);
    const R2* Bc = (const R2*)(bin + (long)c * vs);
    const R2* Dh = (const R2*)(D + (long)i * 2 * vs);
    const R2* Db = (const R2*)(D + (long)i * 2 * vs + vs);
    R2* Ho = (R2*)(hout + (long)c * vs);
    R2* Bo = (R2*)(bout + (long)c * vs);
    if constexpr (FAST) {
      const float nl = -float(LOG2E) * lam, onl = -float(LOG2E) * olam;
      for (int q = lane; q < np; q += 32) {
        const float2 u2 = U2[q], v2 = V2[q], hc2 = Hc[q], bc2 = Bc[q], dh2 = Dh[q], db2 = Db[q];
        const float2 du = p2sub(u2, p2s(U)), dv = p2sub(v2, p2s(V));
        float2 MH = p2mul(p2s(rn), p2ex2(p2mul(p2s(nl), p2fma(du, du, p2mul(dv, dv)))));
        float2 MB = p2mul(p2s(cB), MH);
        if (shak) {
          const float2 cu = p2sub(u2, p2s(Uo)), cv = p2sub(v2, p2s(Vo));
          const float2 c2 = p2fma(cu, cu, p2mul(cv, cv));
          const float2 MHo = p2mul(p2s(orn), p2ex2(p2mul(p2s(onl), c2)));
          const float2 fq = p2fma(p2s(fq0), cu, p2mul(p2s(fq1), cv));
          const float2 tl = p2mul(p2s(2.f * olam), c2);
          MH = p2fma(p2mul(fq, p2add(tl, p2s(Km5))), MHo, MH);
          MB = p2fma(p2mul(fq, p2add(tl, p2s(Km3))), p2mul(p2s(ocB), MHo), MB);
        }
        Ho[q] = p2mul(p2fma(p2s(kk), MH, p2fma(dh2, p2s(-ia), hc2)), p2s(i1k));
        Bo[q] = p2mul(p2fma(p2s(kk), MB, p2fma(db2, p2s(-ia), bc2)), p2s(i1k));
      }
    } else
    for (int q = lane; q < np; q += 32) {
      const R2 u2 = U2[q], v2 = V2[q], hc2 = Hc[q], bc2 = Bc[q], dh2 = Dh[q], db2 = Db[q];
      R2 ho, bo;
#pragma unroll
      for (int e = 0; e < 2; ++e) {
        const R u = e ? u2.y : u2.x, vv = e ? v2.y : v2.x;
        const R du = u - U, dv = vv - V;
        R MH = rn * mexp(-lam * (du * du + dv * dv));
        R MB = MH * cB;
        if (shak) {
          const R cu = u - Uo, cv = vv - Vo, c2 = cu * cu + cv * cv;
          const R MHo = orn * mexp(-olam * c2), MBo = MHo * ocB;
          const R fq = fq0 * cu + fq1 * cv;
          const R tl = R(2) * olam * c2;
          MH += fq * (tl + Km5) * MHo;
          MB += fq * (tl + Km3) * MBo;
        }
        const R hn = ((e ? hc2.y : hc2.x) - (e ? dh2.y : dh2.x) * ia + kk * MH) * i1k;
        const R bn = ((e ? bc2.y : bc2.x) - (e ? db2.y : db2.x) * ia + kk * MB) * i1k;
        if (e) { ho.y = hn; bo.y = bn; } else { ho.x = hn; bo.x = bn; }
      }
      Ho[q] = ho;
      Bo[q] = bo;
    }
  }
}

// update_boundary! US2F (src/Solver/update_boundary.jl:575-594) for the
// extrapolated cells of one dependency level: each becomes the mean of its
// first two neighbours.  The reference runs this loop in cell order, so a
// cell sees the new value of an earlier extrapolated neighbour and the old
// value of a later one; levels are built so that the earlier ones are done
// and the later ones not yet, and a later one's old h, b are read from the
// input buffer (its output slot is written in a later level).
template <typename R>
__global__ void __launch_bounds__(US_T) k_us_avg(UsDev d, int first, const R* __restrict__ hin,
                                                 const R* __restrict__ bin, R* hout, R* bout) {
  const int c = d.avg_list[first + blockIdx.x];
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
  const long vs = d.vstride;
  const bool old0 = d.cell_type[id[0]] == 3 && id[0] > c, old1 = d.cell_type[id[1]] == 3 && id[1] > c;
  const R* H0 = (old0 ? hin : hout) + id[0] * vs;
  const R* B0 = (old0 ? bin : bout) + id[0] * vs;
  const R* H1 = (old1 ? hin : hout) + id[1] * vs;
  const R* B1 = (old1 ? bin : bout) + id[1] * vs;
  R* H = hout + (long)c * vs;
  R* B = bout + (long)c * vs;
  for (int v = threadIdx.x; v < d.nvel; v += US_T) {
    H[v] = R(0.5) * (H0[v] + H1[v]);
    B[v] = R(0.5) * (B0[v] + B1[v]);
  }
}

// residual of update! US2F: sqrt(sum (w - w_old)^2 * ncell) / (sum |w| + 1e-7)
// over the stepped cells (src/Solver/solver_update.jl:465-467) from the step
// CTAs' partials: strided sums, then a fixed tree (deterministic)
__global__ void __launch_bounds__(256) k_us_residual(UsDev d, int nblk) {
  __shared__ double red[8][256];
  double a[8] = {0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0};
  for (int b = threadIdx.x; b < nblk; b += 256)
    for (int k = 0; k < 8; ++k) a[k] += d.bres[8L * b + k];
  for (int k = 0; k < 8; ++k) red[k][threadIdx.x] = a[k];
  __syncthreads();
  for (int s = 128; s >= 1; s >>= 1) {
    if (threadIdx.x < s)
      for (int k = 0; k < 8; ++k) red[k][threadIdx.x] += red[k][threadIdx.x + s];
    __syncthreads();
  }
  if (threadIdx.x < 4)
    d.residual[threadIdx.x] = sqrt(red[threadIdx.x][0] * d.ncell) / (red[4 + threadIdx.x][0] + 1.e-7);
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

// FP64 host rows [ncell][nvel] <-> device rows [ncell][vstride] (both
// buffers of the ping-pong pair on upload)
template <typename R>
__global__ void k_us_in(R* dst0, R* dst1, const double* src, int nvel, int vstride) {
  const long c = blockIdx.x;
  for (int v = threadIdx.x; v < vstride; v += blockDim.x) {
    const R x = v < nvel ? R(src[c * nvel + v]) : R(0);
    dst0[c * vstride + v] = x;
    dst1[c * vstride + v] = x;
  }
}
template <typename R>
__global__ void k_us_out(double* dst, const R* src, int nvel, int vstride) {
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
  void* h[2] = {nullptr, nullptr};  // ping-pong pairs; cur holds the state
  void* b[2] = {nullptr, nullptr};
  int cur = 0;
  std::vector<int> level_first;  // avg_list offsets of the dependency levels (+ end)
  int cb = 1;                    // stepped cells per CTA
  int nblk = 0;                  // CTAs of the last step launch (residual partial rows)
  size_t smem = 0;               // dynamic shared memory of the step kernel
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

// Dependency levels of the extrapolated (type-3) cells.  update_boundary!
// sets them one after another in cell order, each from its first two
// neighbours, so a cell c that reads an earlier type-3 cell must come after
// it and one that reads a later type-3 cell must come before it (it sees the
// old value).  Both constraints point from the lower to the higher cell
// index, so levels by longest path in index order make every level free of
// such pairs, and running the levels in order reproduces the loop.
static std::vector<int> us_levels(int ncell, const int32_t* cell_nb, const int32_t* cell_type,
                                  std::vector<int>& order, std::vector<int>& first) {
  std::vector<int> lvl(ncell, 0), minl(ncell, 1);
  int top = 0;
  for (int c = 0; c < ncell; ++c) {
    if (cell_type[c] != 3) continue;
    int ids[2], m = 0;
    for (int j = 0; j < 3 && m < 2; ++j)
      if (cell_nb[3 * c + j] != -1) ids[m++] = cell_nb[3 * c + j];
    int l = minl[c];
    for (int k = 0; k < m; ++k)
      if (cell_type[ids[k]] == 3 && ids[k] < c) l = std::max(l, lvl[ids[k]] + 1);
    lvl[c] = l;
    for (int k = 0; k < m; ++k)
      if (cell_type[ids[k]] == 3 && ids[k] > c) minl[ids[k]] = std::max(minl[ids[k]], l + 1);
    top = std::max(top, l);
  }
  first.assign(top + 2, 0);
  for (int c = 0; c < ncell; ++c)
    if (cell_type[c] == 3) first[lvl[c] + 1]++;
  for (int l = 1; l <= top + 1; ++l) first[l] += first[l - 1];
  order.assign(first[top + 1], 0);
  std::vector<int> pos(first.begin(), first.end());
  for (int c = 0; c < ncell; ++c)
    if (cell_type[c] == 3) order[pos[lvl[c]]++] = c;
  // level 0 is empty (levels start at 1)
  first.erase(first.begin());
  return lvl;
}

// Cells per CTA of the step kernel and its shared memory: the per-velocity
// flux sums of cb cells (2 nvel values each) plus the per-cell sums,
// parameters and staged records (cell, neighbours, face geometry).  cb = 0 picks the largest count up to 32 within 32 KB of flux
// sums (at least one cell).
static int us_set_cells_per_cta(kb_us* U, int cb) {
  const kb::UsDev& d = U->d;
  const size_t esz = U->prec == KB_PREC_FP64 ? 8 : 4;
  const size_t per = 2 * (size_t)d.vstride * esz + sizeof(int4) + 12 * esz;
  if (cb == 0) cb = (int)std::max<size_t>(1, std::min<size_t>(kb::US_CB, (32u << 10) / per));
  if (cb < 1 || cb > kb::US_CB) return usfail(KB_ERR_ARG, "cells per CTA must be 1 .. 32");
  const size_t smem = (sizeof(double) * (kb::US_NM + kb::US_NP) + per) * cb;
  int dev = 0, maxs = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&maxs, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
  if (smem > (size_t)maxs)
    return usfail(KB_ERR_CONFIG, "velocity grid too large for the unstructured step's shared memory");
  const bool sk = d.coll == KB_COLL_SHAKHOV;
  const void* fn = U->prec == KB_PREC_FP64 ? (sk ? (const void*)kb::k_us_step<double, true>
                                                 : (const void*)kb::k_us_step<double, false>)
                                           : (sk ? (const void*)kb::k_us_step<float, true>
                                                 : (const void*)kb::k_us_step<float, false>);
  cudaError_t e = cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) {
    cudaGetLastError();
    return usfail(KB_ERR_CUDA, "kb_us: cudaFuncSetAttribute failed");
  }
  U->cb = cb;
  U->smem = smem;
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
  if (cfg->dim != 2) return usfail(KB_ERR_CONFIG, "unstructured solves are 2D (2D2F2V or 2D1F2V)");
  if (cfg->nf == 1 && cfg->collision != KB_COLL_BGK)
    return usfail(KB_ERR_CONFIG,
                  "2D1F2V unstructured solves are BGK: the reference's triangle step! for 2D1F2V reads "
                  "h and b, which it does not have, under Shakhov");
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
  std::vector<int> steps;
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
      const int n = cell_nb[3 * c + j];
      if (n < -1 || n >= ncell) return usfail(KB_ERR_ARG, "cell_neighbors out of range");
      if (n != (face_cells[2 * f] == c ? face_cells[2 * f + 1] : face_cells[2 * f]))
        return usfail(KB_ERR_ARG, "cell_neighbors and face_cells disagree");
      nb += n >= 0;
    }
    if (t == 0) {
      if (nb != 3) return usfail(KB_ERR_CONFIG, "a stepped cell (type 0) needs three neighbours");
      steps.push_back(c);
    }
    if (t == 3 && nb < 2)
      return usfail(KB_ERR_CONFIG, "an extrapolated cell (type 3) needs two neighbours");
  }
  std::vector<int> avg, first;
  us_levels(ncell, cell_nb, cell_type, avg, first);
  kb_us* U = new kb_us();
  kb::UsDev& d = U->d;
  U->prec = cfg->precision;
  U->level_first = first;
  d.ncell = ncell;
  d.nface = nface;
  d.nvel = cfg->nu * cfg->nv;
  d.vstride = (d.nvel + 3) / 4 * 4;
  d.coll = cfg->collision;
  d.nstep = (int)steps.size();
  d.navg = (int)avg.size();
  d.K = cfg->K;
  d.Kb = cfg->nf == 1 ? 0.0 : cfg->K;
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
  int *nbp, *ct, *al, *st;
  int4* srec;
  float4* sg32;
  kb::UsG64* sg64;
  double *ca, *cm, *du, *dv, *dw, *tm, *res;
  float *fu, *fv, *fwt;
  USALLOC(nbp, int, 3 * ncell);
  USALLOC(ct, int, ncell);
  USALLOC(srec, int4, steps.size() + 1);
  USALLOC(sg32, float4, 3 * steps.size() + 1);
  USALLOC(sg64, kb::UsG64, 3 * steps.size() + 1);
  USALLOC(al, int, avg.size() + 1);
  USALLOC(st, int, 1);
  USALLOC(ca, double, ncell);
  USALLOC(cm, double, ncell);
  USALLOC(du, double, d.vstride);
  USALLOC(dv, double, d.vstride);
  USALLOC(dw, double, d.vstride);
  USALLOC(fu, float, d.vstride);
  USALLOC(fv, float, d.vstride);
  USALLOC(fwt, float, d.vstride);
  USALLOC(tm, double, 1);
  USALLOC(res, double, 4);
  USALLOC(d.w, double, 4L * ncell);
  USALLOC(d.prim, double, 4L * ncell);
  USALLOC(d.bres, double, 8L * std::max(1, (int)steps.size()));
  USALLOC(U->stage, double, (long)ncell * d.nvel);
#undef USALLOC
  for (void** q : {&U->h[0], &U->h[1], &U->b[0], &U->b[1]})
    if ((rc = usalloc(U, q, esz * (size_t)ncell * d.vstride)) != KB_OK) return bail(rc);
  // velocity grid padded to vstride with zero weights (the padding carries
  // no moment), in FP64 and FP32
  const size_t VS = d.vstride;
  std::vector<double> f64(3 * VS, 0.0);
  std::vector<float> f32(3 * VS, 0.0f);
  for (int k = 0; k < d.nvel; ++k) {
    f64[k] = u[k];
    f64[VS + k] = v[k];
    f64[2 * VS + k] = weights[k];
    f32[k] = (float)u[k];
    f32[VS + k] = (float)v[k];
    f32[2 * VS + k] = (float)weights[k];
  }
  // stepped-cell records: the cell, its neighbours, and per face n1, n2,
  // len and sg |n|^2 with sg = +1 where the cell is the face's first cell
  std::vector<int4> r4(steps.size());
  std::vector<float4> g32(3 * steps.size());
  std::vector<kb::UsG64> g64(3 * steps.size());
  for (size_t k = 0; k < steps.size(); ++k) {
    const int c = steps[k];
    int nbj[3];
    for (int j = 0; j < 3; ++j) {
      const int f = cell_faces[3 * c + j];
      const bool left = face_cells[2 * f] == c;
      nbj[j] = left ? face_cells[2 * f + 1] : face_cells[2 * f];
      const double n1 = face_n[2 * f], n2 = face_n[2 * f + 1];
      const double sgn = (left ? 1.0 : -1.0) * (n1 * n1 + n2 * n2);
      g32[3 * k + j] = make_float4((float)n1, (float)n2, (float)face_len[f], (float)sgn);
      g64[3 * k + j] = kb::UsG64{n1, n2, face_len[f], sgn};
    }
    r4[k] = make_int4(c, nbj[0], nbj[1], nbj[2]);
  }
  bool ok = true;
  auto up = [&](void* dst, const void* src, size_t bytes) {
    ok &= cudaMemcpy(dst, src, bytes, cudaMemcpyHostToDevice) == cudaSuccess;
  };
  up(nbp, cell_nb, sizeof(int) * 3 * ncell);
  up(ct, cell_type, sizeof(int) * ncell);
  if (!steps.empty()) {
    up(srec, r4.data(), sizeof(int4) * steps.size());
    up(sg32, g32.data(), sizeof(float4) * g32.size());
    up(sg64, g64.data(), sizeof(kb::UsG64) * g64.size());
  }
  if (!avg.empty()) up(al, avg.data(), sizeof(int) * avg.size());
  {
    std::vector<double> ia(ncell);
    for (long i = 0; i < ncell; ++i) ia[i] = 1.0 / cell_area[i];
    up(ca, ia.data(), sizeof(double) * ncell);
  }
  up(cm, cell_mindx, sizeof(double) * ncell);
  up(du, f64.data(), sizeof(double) * VS);
  up(dv, f64.data() + VS, sizeof(double) * VS);
  up(dw, f64.data() + 2 * VS, sizeof(double) * VS);
  up(fu, f32.data(), sizeof(float) * VS);
  up(fv, f32.data() + VS, sizeof(float) * VS);
  up(fwt, f32.data() + 2 * VS, sizeof(float) * VS);
  ok &= cudaMemset(st, 0, sizeof(int)) == cudaSuccess;
  ok &= cudaMemset(d.bres, 0, sizeof(double) * 8L * std::max(1, (int)steps.size())) == cudaSuccess;
  if (!ok) return bail(usfail(KB_ERR_CUDA, "kb_us_create: copy failed"));
  if ((rc = us_set_cells_per_cta(U, 0)) != KB_OK) return bail(rc);
  d.cell_nb = nbp;
  d.cell_type = ct;
  d.step_rec = srec;
  d.step_geo32 = sg32;
  d.step_geo64 = sg64;
  d.avg_list = al;
  d.status = st;
  d.cell_iarea = ca;
  d.cell_mindx = cm;
  d.u = du;
  d.v = dv;
  d.wt = dw;
  d.uf = fu;
  d.vf = fv;
  d.wtf = fwt;
  d.tmax = tm;
  d.residual = res;
  *out = U;
  return KB_OK;
}

extern "C" int kb_us_upload(kb_us_t* U, const double* w, const double* prim, const double* h,
                            const double* b) {
  if (!U || !w || !prim || !h || !b) return usfail(KB_ERR_ARG, "kb_us_upload: null argument");
  const kb::UsDev& d = U->d;
  bool ok = cudaStreamSynchronize(U->stream) == cudaSuccess &&
            cudaMemcpy(d.w, w, sizeof(double) * 4L * d.ncell, cudaMemcpyHostToDevice) == cudaSuccess &&
            cudaMemcpy(d.prim, prim, sizeof(double) * 4L * d.ncell, cudaMemcpyHostToDevice) == cudaSuccess;
  for (int k = 0; k < 2 && ok; ++k) {
    ok &= cudaMemcpy(U->stage, k == 0 ? h : b, sizeof(double) * (size_t)d.ncell * d.nvel,
                     cudaMemcpyHostToDevice) == cudaSuccess;
    void** dst = k == 0 ? U->h : U->b;
    if (U->prec == KB_PREC_FP64)
      kb::k_us_in<double><<<d.ncell, 128, 0, U->stream>>>((double*)dst[0], (double*)dst[1], U->stage,
                                                          d.nvel, d.vstride);
    else
      kb::k_us_in<float><<<d.ncell, 128, 0, U->stream>>>((float*)dst[0], (float*)dst[1], U->stage,
                                                         d.nvel, d.vstride);
    U->launches++;
    ok &= cudaStreamSynchronize(U->stream) == cudaSuccess;
  }
  U->cur = 0;
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
    const void* src = k == 0 ? U->h[U->cur] : U->b[U->cur];
    if (U->prec == KB_PREC_FP64)
      kb::k_us_out<double><<<d.ncell, 128, 0, U->stream>>>(U->stage, (const double*)src, d.nvel, d.vstride);
    else
      kb::k_us_out<float><<<d.ncell, 128, 0, U->stream>>>(U->stage, (const float*)src, d.nvel, d.vstride);
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

template <typename R>
static void us_enqueue_step(kb_us* U, double dt) {
  const kb::UsDev& d = U->d;
  const R* hin = (const R*)U->h[U->cur];
  const R* bin = (const R*)U->b[U->cur];
  R* hout = (R*)U->h[U->cur ^ 1];
  R* bout = (R*)U->b[U->cur ^ 1];
  if (d.nstep) {
    const int grid = (d.nstep + U->cb - 1) / U->cb;
    U->nblk = grid;
    if (d.coll == KB_COLL_SHAKHOV)
      kb::k_us_step<R, true><<<grid, kb::US_T, U->smem, U->stream>>>(d, dt, U->cb, hin, bin, hout, bout);
    else
      kb::k_us_step<R, false><<<grid, kb::US_T, U->smem, U->stream>>>(d, dt, U->cb, hin, bin, hout, bout);
    U->launches++;
  }
  for (size_t l = 0; l + 1 < U->level_first.size(); ++l) {
    const int n = U->level_first[l + 1] - U->level_first[l];
    if (n == 0) continue;
    kb::k_us_avg<R><<<n, kb::US_T, 0, U->stream>>>(d, U->level_first[l], hin, bin, hout, bout);
    U->launches++;
  }
  U->cur ^= 1;
}

extern "C" int kb_us_step(kb_us_t* U, double dt, int32_t nsteps, double* residual) {
  if (!U || nsteps < 0) return usfail(KB_ERR_ARG, "kb_us_step: bad argument");
  const kb::UsDev& d = U->d;
  for (int s = 0; s < nsteps; ++s) {
    if (U->prec == KB_PREC_FP64)
      us_enqueue_step<double>(U, dt);
    else
      us_enqueue_step<float>(U, dt);
  }
  kb::k_us_residual<<<1, 256, 0, U->stream>>>(d, U->nblk);
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

extern "C" int kb_us_set_tuning(kb_us_t* U, int32_t cells_per_cta) {
  if (!U) return usfail(KB_ERR_ARG, "kb_us_set_tuning: null handle");
  if (cudaStreamSynchronize(U->stream) != cudaSuccess) return usfail(KB_ERR_CUDA, "kb_us_set_tuning");
  return us_set_cells_per_cta(U, cells_per_cta);
}

extern "C" int kb_us_get_tuning(kb_us_t* U, int32_t* cells_per_cta) {
  if (!U || !cells_per_cta) return usfail(KB_ERR_ARG, "kb_us_get_tuning: null argument");
  *cells_per_cta = U->cb;
  return KB_OK;
}

extern "C" int kb_us_stream(kb_us_t* U, void** stream) {
  if (!U || !stream) return usfail(KB_ERR_ARG, "kb_us_stream: null argument");
  *stream = (void*)U->stream;
  return KB_OK;
}
