// kb_batch.cuh -- device side of the batched 1D2F1V solves: the ragged
// layout (BatchDev) and the fused FP32 segment kernel, a template over the
// segment length and the CTA size so that the autotuner can choose them
// (instantiated in kb_batch_seg_a.cu / kb_batch_seg_b.cu).
#pragma once

#include <cuda_runtime.h>

#include <type_traits>
#include <vector>

#include "kb_device.cuh"
#include "kb_kernels.cuh"
#include "kb_tma.cuh"

namespace kb {

struct BatchDev {
  int n;                 // instances
  const int* order;      // processing order (largest first)
  const int* nx;         // physical cells
  const int* ng;         // ghost layers
  const int* nu;         // velocities
  const int* nus;        // row stride of the distributions: nu rounded up to 4
  const long* cell_off;  // first cell (incl. ghosts)
  const long* elem_off;  // first distribution element
  const int* vel_off;    // velocity table offset
  const double* dx;      // cell size
  const double* dt;      // time step
  const double* mu;      // reference viscosity
  const double* u;       // velocity tables (FP64)
  const double* wt;
  const float* uf;       // FP32 copies
  const float* ul;       // u - uf: the FP32 velocities as hi + lo pairs
  const float* wtf;
  double* w;             // [cell][4] (3 used)
  double* prim;          // [cell][4]
  double* fw;            // [instance faces][4] scratch: face flux per instance (nx+1 each)
  const long* face_off;
  double* q;             // [cell] old heat flux
  double* cp;            // [cell][16] cell coefficients (see k_batch_step)
  float* mc;             // [cell][8] FP32 Maxwellian coefficients of the cell's current prim
                         // (SegMax: rn, U hi, lambda, K / (2 lambda), U lo), kept with prim
  double* residual;      // [n][4]
  int* active;           // [n] 1 while not converged
  int* counter;          // work counter
  int* status;
  // FP32 segment form: segment k covers cells [seg_i0[k], seg_i0[k] + SEG) of
  // instance seg_b[k]; an instance's segments are consecutive from
  // seg_first[b] (nseg[b] of them)
  const int* seg_b;
  const int* seg_i0;
  const int* seg_first;
  const int* nseg;
  double* respart;       // [segments][8] residual partial sums
  int nseg_all;          // segments of the current segment length
  int sst_max;           // largest shared-memory row stride of the batch (floats)
  int nu4_max;           // largest velocity count, rounded up to 4
  double K, gamma, omega, Pr, tol;
  int coll;
};

template <typename R>
__device__ __forceinline__ R bvl(int rule, R qm, R q0, R qp, R epsd) {
  R a = q0 - qm, b = qp - q0;
  if (rule == 1) return (a * fabs(b) + b * fabs(a)) / (fabs(a) + fabs(b) + epsd);
  return R(0);
}
// FP32 form: one reciprocal and one multiply (subnormals flushed), the
// division the FP32 passes of the 2D solver use as well
template <>
__device__ __forceinline__ float bvl<float>(int rule, float qm, float q0, float qp, float epsd) {
  float a = q0 - qm, b = qp - q0;
  if (rule != 1) return 0.f;
  float r;
  asm("div.approx.ftz.f32 %0, %1, %2;"
      : "=f"(r)
      : "f"(a * fabsf(b) + b * fabsf(a)), "f"(fabsf(a) + fabsf(b) + epsd));
  return r;
}

// 1D slope rule: van Leer everywhere inside when ghosts exist, boundary cells
// flat without ghosts (src/Solver/solver_reconstruction.jl:101-153).
__device__ __forceinline__ int brule(int i, int nx, int ng) {
  if (i < 0 || i >= nx) return 0;
  if (ng == 0 && (i == 0 || i == nx - 1)) return 0;
  return 1;
}

template <typename R>
struct BSum;
template <>
struct BSum<float> {
  float p;
  DF d;
  __device__ __forceinline__ void init() { p = 0.f; d.hi = d.lo = 0.f; }
  __device__ __forceinline__ void add(float x) { p += x; }
  __device__ __forceinline__ void flush() { df_add(d, p); p = 0.f; }
  __device__ __forceinline__ double get() { flush(); return (double)d.hi + (double)d.lo; }
};
template <>
struct BSum<double> {
  double p;
  __device__ __forceinline__ void init() { p = 0.0; }
  __device__ __forceinline__ void add(double x) { p += x; }
  __device__ __forceinline__ void flush() {}
  __device__ __forceinline__ double get() { return p; }
};

template <typename R>
__device__ __forceinline__ const R* btab(const BatchDev& B, int which);
template <>
__device__ __forceinline__ const double* btab<double>(const BatchDev& B, int which) {
  return which == 0 ? B.u : B.wt;
}
template <>
__device__ __forceinline__ const float* btab<float>(const BatchDev& B, int which) {
  return which == 0 ? B.uf : B.wtf;
}


// e^x on the MUFU unit (2^(x log2 e), results below 2^-126 flushed to zero)
__device__ __forceinline__ float fexp(float x) {
  float y;
  asm("ex2.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x * 1.4426950408889634f));
  return y;
}

// The FP32 Maxwellian of the segment kernel's relaxation and of the
// device-built equilibrium state (kb_batch_init_equilibrium, kb_pool_add):
// rn 2^(-lambda du^2 log2 e) with du = (u - U_hi) + (u_lo - U_lo).  Both
// use this one function, so a uniform equilibrium state is an exact fixed
// point of the FP32 update: fixed boundary cells and the cells next to them
// then agree bit for bit, and no FP32 rounding drift enters the FP64 w
// there (which, at high Mach number, the kinetic energy would amplify in T).
__device__ __forceinline__ float seg_maxwell(float u, float ulo, float rn, float Uh, float Ul,
                                             float lam) {
  const float du = (u - Uh) + (ulo - Ul);
  return rn * fexp(-lam * du * du);
}

// FP32 coefficients of one cell's Maxwellian from its FP64 prim [rho, U,
// lambda]: density factor rn = rho sqrt(lambda / pi), U as an FP32 pair,
// lambda, K / (2 lambda), each formed in FP64 and rounded once.
struct SegMax {
  float rn, Uh, Ul, lam, cB;
  __device__ __forceinline__ void set(const double* p, double K) {
    rn = float(p[0] * sqrt(p[2] * (1.0 / PI)));
    Uh = float(p[1]);
    Ul = float(p[1] - (double)Uh);
    lam = float(p[2]);
    cB = float(K / (2.0 * p[2]));
  }
};

// The cell's FP32 Maxwellian coefficients into B.mc (kept with its prim).
__device__ __forceinline__ void seg_store_coef(const BatchDev& B, long cell, const SegMax& m) {
  float4* mcc = (float4*)(B.mc + cell * 8);
  mcc[0] = make_float4(m.rn, m.Uh, m.lam, m.cB);
  mcc[1] = make_float4(m.Ul, 0.f, 0.f, 0.f);
}

// Equilibrium h, b of cell c (0-based incl. ghosts) of instance b into both
// FP32 buffers (init_fvm, src/Solver/solver_init.jl:119-141); row padding zero.
__device__ __forceinline__ void seg_init_cell(const BatchDev& B, int b, int c, float* H0, float* B0,
                                              float* H1, float* B1) {
  SegMax m;
  m.set(B.prim + (B.cell_off[b] + c) * 4, B.K);
  if (threadIdx.x == 0) seg_store_coef(B, B.cell_off[b] + c, m);
  const int nu = B.nu[b], ns = B.nus[b];
  const long e = B.elem_off[b] + (long)c * ns;
  const float* uf = B.uf + B.vel_off[b];
  const float* ul = B.ul + B.vel_off[b];
  for (int v = threadIdx.x; v < ns; v += blockDim.x) {
    float hv = 0.f, bv = 0.f;
    if (v < nu) {
      hv = seg_maxwell(uf[v], ul[v], m.rn, m.Uh, m.Ul, m.lam);
      bv = hv * m.cB;
    }
    H0[e + v] = hv;
    B0[e + v] = bv;
    H1[e + v] = hv;
    B1[e + v] = bv;
  }
}

// ---- FP32 form: one CTA per segment of SEG cells, the whole step fused.
// In 1D an instance has at most 256 velocities, so a segment's stencil window
// (SEG + 4 cells x all velocities, h and b) fits in shared memory: the face
// moments of the segment's faces, the new w / prim / tau of its cells and
// the pointwise update all need only the old state inside that window, so
// the step is one pass over HBM (each value read once, plus a 2-cell halo on
// each side, and written once).  The window arrives by bulk async copies, one
// per row, into rows whose stride is = 4 (mod 32) floats so that the face
// threads read without bank conflicts.  Per-instance residuals are summed
// by k_batch_seg_res after the step, in segment order (deterministic).
constexpr int SEG_MAXNU = 256;
constexpr int SEG_CC = 4;  // float4 coefficient blocks per cell
__host__ __device__ inline int seg_stride(int nus) { return (nus + 31) / 32 * 32 + 4; }
// Thread mapping of a segment CTA of SEG cells and T threads: FT threads per
// face in the face-moment phase (SEG + 1 faces), QT threads per cell in the
// heat-flux phase (warps 1 .. NWH), one lane per cell of warp 0 in the cell
// phase, one thread per velocity in the pointwise phase.
template <int SEG, int T>
struct SegShape {
  static constexpr int ROWS = SEG + 4;  // window cells
  static constexpr int FT = T / (SEG + 1);
  static constexpr int QRAW = (T - 32) / SEG;
  static constexpr int QT = QRAW >= 8 ? 8 : (QRAW >= 4 ? 4 : (QRAW >= 2 ? 2 : 1));
  static constexpr int NWH = (QT * SEG + 31) / 32;
  static_assert(SEG <= 32 && T % 32 == 0 && FT >= 1 && QRAW >= 1 && 1 + NWH <= T / 32,
                "segment shape");
};
// Dynamic shared memory of a segment CTA, sized by the batch's largest row
// stride and velocity count: h and b windows, velocity tables (hi, weight,
// lo), fw, the 16-byte aligned cell coefficients, the face-moment partials
// and the old prim of the stepped cells.
template <int SEG, int T>
__host__ __device__ inline int seg_smem(int sst_max, int nu4_max) {
  return 2 * (SEG + 4) * sst_max * 4 + 3 * nu4_max * 4 + (SEG + 1) * 3 * 8 + 16 +
         SEG * SEG_CC * 16 + T * 6 * 4 + SEG * 3 * 8 + 8 * 8;
}
template <int SEG, int T>
__host__ __device__ inline int seg_smem_max() {
  return seg_smem<SEG, T>(seg_stride((SEG_MAXNU + 3) / 4 * 4), SEG_MAXNU);
}

// Segment k covers cells [seg_i0[k], seg_i0[k] + SEG) of instance seg_b[k].
// A CTA takes segments k = blockIdx.x, blockIdx.x + gridDim.x, ...: one
// segment each when the grid has a CTA per segment, or a persistent loop
// when the grid is the number of CTAs that fit on the GPU at once.
template <int SEG, int SEG_T>
__global__ void __launch_bounds__(SEG_T) k_batch_seg(BatchDev B, const float* __restrict__ Hin,
                                                     const float* __restrict__ Bin,
                                                     float* __restrict__ Hout,
                                                     float* __restrict__ Bout) {
  using SH = SegShape<SEG, SEG_T>;
  constexpr int SEG_ROWS = SH::ROWS;
  constexpr int SEG_FT = SH::FT;
  constexpr int QT = SH::QT;
  extern __shared__ __align__(16) unsigned char sm[];
  __shared__ unsigned long long bar;
  __shared__ float sconst[4];  // T3, T4, 1/dx, 1e-7 dx
  // GB300 runs FP64 at 1/64 of the FP32 rate: FP64 work below is done by as
  // few warps as possible (the per-instance constants by one thread, the
  // cell update and its residual by the first warp)
  const int tid = threadIdx.x, lane = tid & 31, wid = tid >> 5;
  if (tid == 0) {
    mbar_init(&bar, 1);
    fence_async_smem();
  }
  __syncthreads();
  unsigned phase = 0;  // completed window copies of this CTA (mbarrier parity)
  for (int k = blockIdx.x; k < B.nseg_all; k += gridDim.x) {
  const int b = B.seg_b[k], i0 = B.seg_i0[k];
  const int nx = B.nx[b], ng = B.ng[b], nu = B.nu[b], ns = B.nus[b];
  const int i1 = min(i0 + SEG, nx);
  const long c0 = B.cell_off[b], e0 = B.elem_off[b];
  const float* Hi = Hin + e0;
  const float* Bi = Bin + e0;
  float* Ho = Hout + e0;
  float* Bo = Bout + e0;
  if (!B.active[b]) {  // converged: carry this segment's cells over
    for (long t = tid; t < (long)(i1 - i0) * ns; t += SEG_T) {
      const long o = (long)(i0 + ng) * ns + t;
      Ho[o] = Hi[o];
      Bo[o] = Bi[o];
    }
    continue;  // CTA-uniform
  }
  const int sst = seg_stride(ns);
  float* sH = (float*)sm;
  float* sB = sH + SEG_ROWS * B.sst_max;
  float* sU = sB + SEG_ROWS * B.sst_max;
  float* sW = sU + B.nu4_max;
  float* sUl = sW + B.nu4_max;               // low parts of the velocities
  double* sfw = (double*)(sUl + B.nu4_max);  // [SEG + 1][3]
  // [SEG][SEG_CC] float4 cell coefficients, 16-byte aligned
  float4* scc = (float4*)(((unsigned long long)(sfw + (SEG + 1) * 3) + 15) & ~15ull);
  float* sred = (float*)(scc + SEG * SEG_CC);  // [SEG_T][6]: face-moment DF partials
  // window rows r0 .. r1-1 (cells incl. ghosts), smem row = cell - r0
  const int r0 = max(i0 - 2, -ng), r1 = min(i1 + 2, nx + ng), nrow = r1 - r0;
  if (tid < 32) {
    if (lane == 0) mbar_expect(&bar, 2u * nrow * ns * 4u);
    __syncwarp();
    for (int r = lane; r < 2 * nrow; r += 32) {
      const int row = r >> 1;
      const float* src = ((r & 1) ? Bi : Hi) + (long)(r0 + row + ng) * ns;
      float* dst = ((r & 1) ? sB : sH) + row * sst;
      bulk_g2s(dst, src, (unsigned)ns * 4u, &bar);
    }
  }
  for (int v = tid; v < nu; v += SEG_T) {
    sU[v] = B.uf[B.vel_off[b] + v];
    sUl[v] = B.ul[B.vel_off[b] + v];
    sW[v] = B.wtf[B.vel_off[b] + v];
  }
  if (tid == 0) {
    const double dx0 = B.dx[b], dt0 = B.dt[b];
    sconst[0] = float(dt0);
    sconst[1] = float(0.5 * dt0 * dt0 / dx0);
    sconst[2] = float(1.0 / dx0);
    sconst[3] = float(1.e-7 * dx0);
  }
  // one thread waits for the window; the others wait at the CTA barrier
  const bool ok = tid == 0 ? mbar_wait(&bar, phase & 1) : true;
  if (__syncthreads_or(!ok)) {  // CTA-uniform: bounded clean-up, then leave
    if (tid == 0) {
      atomicOr(B.status, 2);
      mbar_wait(&bar, phase & 1);
    }
    return;
  }
  ++phase;
  const float epsd = sconst[3];
  const float T3 = sconst[0], T4 = sconst[1];
  auto rowH = [&](int c) { return sH + (c - r0) * sst; };
  auto rowB = [&](int c) { return sB + (c - r0) * sst; };

  // ---- face moments of faces fa .. fb: SEG_FT threads per face (velocities
  // v = q mod SEG_FT), so the SEG + 1 faces keep all four warps busy
  const int fa = max(i0, 1), fb = min(i1, nx - 1);
  const int ca = max(i0, 1), cb = min(i1, nx - 1);  // stepped cells [ca, cb)
  {
    const int j = tid / SEG_FT, q = tid - j * SEG_FT;
    const int f = fa + j;
    // Each moment term enters as an exact pair: the FP32 products w fh,
    // w fh u, w fh u^2, w fb with their rounding errors (FMA), added with
    // error-free sums (TwoSum).  In a supersonic flow the energy flux is
    // large and the flux difference between a cell's two faces small, so
    // FP32 rounding of the terms or of running partial sums would enter w as
    // a bias of relative size ~1e-7 of the flux every step -- amplified in
    // T = 1 / (2 lambda) by the kinetic-to-thermal energy ratio (~35 at
    // Mach 8), it grew to 1e-5 of T within a few hundred steps.
    DF m0, m1, m2;
    m0.hi = m0.lo = m1.hi = m1.lo = m2.hi = m2.lo = 0.f;
    float l0 = 0.f, l1 = 0.f, l2 = 0.f;  // sums of the products' rounding errors
    if (j <= SEG && f <= fb) {
      const int iL = f - 1, iR = f;
      const int rL = brule(iL, nx, ng), rR = brule(iR, nx, ng);
      for (int v = q; v < nu; v += SEG_FT) {
        const float u = sU[v];
        const bool pos = u >= 0.f;
        const int c = pos ? iL : iR;
        const int r = pos ? rL : rR;
        const float* hc = rowH(c);
        const float* bc = rowB(c);
        const float h0 = hc[v], b0 = bc[v];
        float sh = 0.f, sb = 0.f;
        if (r == 1) {
          sh = bvl<float>(1, hc[v - sst], h0, hc[v + sst], epsd);
          sb = bvl<float>(1, bc[v - sst], b0, bc[v + sst], epsd);
        }
        const float side = pos ? 0.5f : -0.5f;
        const float hf = h0 + side * sh, bf = b0 + side * sb;
        const float fh = T3 * u * hf - T4 * (u * u) * sh;
        const float fbb = T3 * u * bf - T4 * (u * u) * sb;
        // rounded products that the compiler may not fuse into a later add
        // (a fused product would no longer match its error term)
        const float wv = sW[v];
        const float t0 = __fmul_rn(wv, fh), e0 = fmaf(wv, fh, -t0);  // w fh = t0 + e0 exactly
        const float t1 = __fmul_rn(t0, u), e1 = fmaf(t0, u, -t1);
        const float c1 = fmaf(e0, u, e1);                            // w fh u = t1 + c1
        const float t2 = __fmul_rn(t1, u), e2 = fmaf(t1, u, -t2);
        const float tb = __fmul_rn(wv, fbb), eb = fmaf(wv, fbb, -tb);
        df_add(m0, t0);
        df_add(m1, t1);
        df_add(m2, t2);
        df_add(m2, tb);
        l0 += e0;
        l1 += c1;
        l2 += fmaf(c1, u, e2) + eb;                       // w (fh u^2 + fb) = t2 + tb + ...
      }
    }
    // each thread's pairs, merged per face below in thread order: both
    // segments that share a face map it to the same threads q, so they
    // compute bit-identical fw (conservation holds exactly)
    float* o = sred + tid * 6;
    o[0] = m0.hi;
    o[1] = m0.lo + l0;
    o[2] = m1.hi;
    o[3] = m1.lo + l1;
    o[4] = m2.hi;
    o[5] = m2.lo + l2;
  }
  // the old prim of the stepped cells, read before warp 0 overwrites it
  // (warps 1 and 2 need the old U while warp 0 updates the cells)
  double* spo = (double*)(sred + SEG_T * 6);  // [SEG][3] rho, U, lambda
  if (tid < cb - ca) {
    const double* p = B.prim + (c0 + ca + tid + ng) * 4;
    spo[tid * 3 + 0] = p[0];
    spo[tid * 3 + 1] = p[1];
    spo[tid * 3 + 2] = p[2];
  }
  __syncthreads();  // face partials and old prim in shared memory
  // Warp 0: merge the face moments, then the FP64 cell update; warps 1 and 2
  // meanwhile: the old heat flux (Shakhov) of the stepped cells.
  if (wid == 0) {
    // residual terms of the cell: a convergence monitor, summed in FP32 below
    float rr[6] = {0, 0, 0, 0, 0, 0};
    // face f = fa + jf, moment m: the SEG_FT partials of its threads, in order
    for (int t0 = lane; t0 < 3 * (SEG + 1); t0 += 32) {
      const int jf = t0 / 3, m = t0 - 3 * jf;
      if (fa + jf <= fb) {
        const float* o = sred + jf * SEG_FT * 6 + 2 * m;
        DF d;
        d.hi = o[0];
        d.lo = o[1];
        for (int t = 1; t < SEG_FT; ++t) {
          DF e;
          e.hi = o[6 * t];
          e.lo = o[6 * t + 1];
          d = df_merge(d, e);
        }
        const double v = (double)d.hi + (double)d.lo;
        sfw[jf * 3 + m] = m == 2 ? 0.5 * v : v;
      }
    }
    __syncwarp();
    // ---- cell parameters of the stepped cells (one lane per cell, FP64)
    if (lane < cb - ca) {
      const double dx = B.dx[b], dt = B.dt[b];
      const int i = ca + lane;
      const long c = c0 + i + ng;
      double* w = B.w + c * 4;
      double* p = B.prim + c * 4;
      const double* fL = sfw + (i - fa) * 3;
      const double* fR = sfw + (i + 1 - fa) * 3;
      double wo[3] = {w[0], w[1], w[2]};
      const double rho_o = spo[lane * 3 + 0], Uo = spo[lane * 3 + 1], lo = spo[lane * 3 + 2];
      const double idx = 1.0 / dx;
      for (int m = 0; m < 3; ++m) w[m] += (fL[m] - fR[m]) * idx;
      double pn[4];
      conserve_prim<true>(w, 3, B.gamma, pn);
      p[0] = pn[0];
      p[1] = pn[1];
      p[2] = pn[2];
      for (int m = 0; m < 3; ++m) {
        double d = w[m] - wo[m];
        rr[m] = float(d * d);
        rr[3 + m] = float(fabs(w[m]));
      }
      double lam = pn[2];
      if (!(pn[0] > 0.0) || !(lam > 0.0) || !isfinite(pn[0]) || !isfinite(lam)) atomicOr(B.status, 1);
      // w, prim and q stay FP64; the coefficients below feed only the FP32
      // pointwise update.  The Maxwellian's density factor, U and lambda are
      // formed in FP64 and rounded once, and U is carried as an FP32 pair
      // (hi + lo) so that u - U is exact to FP32 rounding of the difference:
      // at high Mach the energy is mostly kinetic, and an FP32-rounded U or
      // density factor would bias the moments of the equilibrium by more
      // than the FP32 split form's 1e-5 budget in T.  tau only sets the
      // relaxation rate and is formed in FP32 (GB300's FP64 rate is 1/64 of
      // its FP32 rate).
      const float rf = float(pn[0]), lf = float(lam);
      const float tau = float(B.mu[b]) * 2.f * powf(lf, float(1.0 - B.omega)) / rf;
      const float dtt = float(dt) / tau;
      const double Kd = B.K;
      float4* kc = scc + lane * SEG_CC;
      // the old Maxwellian's coefficients are the ones this cell's update
      // formed from the same prim one step earlier (or the set-up formed from
      // the initial prim): read instead of recomputed, which saves an FP64
      // square root and division per cell, bit for bit the same values
      float4* mcc = (float4*)(B.mc + c * 8);
      const float4 mo = mcc[0];
      const float mUl = mcc[1].x;
      // new Maxwellian: density factor, U (hi), lambda, K / (2 lambda)
      SegMax mn;
      mn.set(pn, Kd);
      kc[0] = make_float4(mn.rn, mn.Uh, mn.lam, mn.cB);
      // dt / tau, 1 / (1 + dt / tau), old Maxwellian (Shakhov) density factor and U (hi)
      kc[1] = make_float4(dtt, 1.f / (1.f + dtt), mo.x, mo.y);
      // old lambda, K / (2 lambda); .z (the Shakhov heat-flux factor) comes
      // from warps 1-2; .w the low part of U
      float* k2 = (float*)(kc + 2);
      k2[0] = mo.z;
      k2[1] = mo.w;
      k2[3] = mn.Ul;
      kc[3] = make_float4(mUl, 0.f, 0.f, 0.f);
      mcc[0] = make_float4(mn.rn, mn.Uh, mn.lam, mn.cB);
      mcc[1] = make_float4(mn.Ul, 0.f, 0.f, 0.f);
    }
    // residual partial sums of the segment, in a fixed shuffle order (FP32:
    // GB300's FP64 pipe would make this tree the longest chain of the phase)
#pragma unroll
    for (int m = 0; m < 6; ++m) {
#pragma unroll
      for (int o = 16; o >= 1; o >>= 1) rr[m] += __shfl_xor_sync(0xffffffffu, rr[m], o);
    }
    // this segment's residual partial sums (k_batch_seg_res adds them up)
    if (lane == 0) {
      double* pr = B.respart + (long)k * 8;
#pragma unroll
      for (int m = 0; m < 6; ++m) pr[m] = (double)rr[m];
    }
  } else if (wid <= SH::NWH) {
    // ---- old heat flux of the stepped cells, QT threads per cell, and the
    // Shakhov factor 0.8 (1 - Pr) lambda^2 / rho q of the cell coefficients
    const int lt = tid - 32, jc = lt / QT, q = lt % QT;
    const int i = ca + jc;
    float qf = 0.f;
    if (B.coll == COLL_SHAKHOV) {
      BSum<float> sm4;
      sm4.init();
      if (i < cb) {
        const double Ud = spo[jc * 3 + 1];
        const float Uc = float(Ud), Ul = float(Ud - (double)Uc);  // U as an FP32 pair
        const float* hc = rowH(i);
        const float* bc = rowB(i);
        int it = 0;
        for (int v = q; v < nu; v += QT, ++it) {
          const float cu = (sU[v] - Uc) + (sUl[v] - Ul);
          sm4.add(sW[v] * cu * (cu * cu * hc[v] + bc[v]));
          if ((it & 7) == 7) sm4.flush();
        }
      }
      sm4.flush();
      DF d = sm4.d;
#pragma unroll
      for (int m = 1; m < QT; m <<= 1) d = df_merge(d, df_shfl_xor(d, m));
      if (i < cb) {
        const double qc = 0.5 * ((double)d.hi + (double)d.lo);
        const float rof = float(spo[jc * 3 + 0]), lof = float(spo[jc * 3 + 2]);
        qf = float(0.8 * (1.0 - B.Pr)) * (lof * lof) / rof * float(qc);
      }
    }
    if (q == 0 && jc < SEG && i < cb) ((float*)(scc + jc * SEG_CC + 2))[2] = qf;
  }
  __syncthreads();  // cell coefficients ready for the pointwise update
  // ---- pointwise KFVS flux + relaxation, one thread per velocity.  Every
  // upwind cell of a segment away from ghost-less ends takes the van Leer
  // slope, so that form skips the per-face slope rule.
  const float idx = sconst[2];
  const bool all_vl = ng > 0 || (ca >= 2 && cb <= nx - 2);
  auto pointwise = [&](auto vl_tag) {
    constexpr bool VL = decltype(vl_tag)::value;
    for (int v = tid; v < nu; v += SEG_T) {
      const float u = sU[v], ulo = sUl[v];
      const bool pos = u >= 0.f;
      const float side = pos ? 0.5f : -0.5f;
      const float Tu = T3 * u, Tuu = T4 * (u * u);
      if (i0 == 0) {  // fixed end cells keep their state
        Ho[(long)ng * ns + v] = rowH(0)[v];
        Bo[(long)ng * ns + v] = rowB(0)[v];
      }
      if (i1 == nx) {
        Ho[(long)(nx - 1 + ng) * ns + v] = rowH(nx - 1)[v];
        Bo[(long)(nx - 1 + ng) * ns + v] = rowB(nx - 1)[v];
      }
      // flux through face f, whose upwind cell row starts at hc / bc
      auto face = [&](int f, const float* hc, const float* bc, float& fh, float& fbv) {
        const float h0 = hc[0], b0 = bc[0];
        float sh = 0.f, sb = 0.f;
        if (VL || brule(pos ? f - 1 : f, nx, ng) == 1) {
          sh = bvl<float>(1, hc[-sst], h0, hc[sst], epsd);
          sb = bvl<float>(1, bc[-sst], b0, bc[sst], epsd);
        }
        fh = Tu * (h0 + side * sh) - Tuu * sh;
        fbv = Tu * (b0 + side * sb) - Tuu * sb;
      };
      if (ca >= cb) continue;
      // hr / br: row of cell i at this velocity; the upwind cell of face i + 1
      // is i (pos) or i + 1
      const int up = pos ? 0 : sst;
      const float* hr = rowH(ca) + v;
      const float* br = rowB(ca) + v;
      float fhL, fbL;
      face(ca, hr - sst + up, br - sst + up, fhL, fbL);
      float* ph = Ho + (long)(ca + ng) * ns + v;
      float* pb = Bo + (long)(ca + ng) * ns + v;
      const float4* kc = scc;
      for (int i = ca; i < cb; ++i, hr += sst, br += sst, ph += ns, pb += ns, kc += SEG_CC) {
        float fhR, fbR;
        face(i + 1, hr + up, br + up, fhR, fbR);
        const float4 k0 = kc[0], k1 = kc[1], k2 = kc[2];
        const float h0 = hr[0], b0 = br[0];
        const float M = seg_maxwell(u, ulo, k0.x, k0.y, k2.w, k0.z);
        float MH = M, MB = M * k0.w;
        if (B.coll == COLL_SHAKHOV) {
          const float ou = (u - k1.w) + (ulo - kc[3].x);
          const float OH = k1.z * fexp(-k2.x * ou * ou);
          const float cq = k2.z * ou;
          const float tl = 2.f * k2.x * ou * ou + float(B.K);
          MH += cq * (tl - 5.f) * OH;
          MB += cq * (tl - 3.f) * OH * k2.y;
        }
        // (h + div + dt/tau MH) / (1 + dt/tau) written as a correction of h,
        // so that an equilibrium cell (MH == h, div == 0) stays bit-exact
        *ph = h0 + ((fhL - fhR) * idx + k1.x * (MH - h0)) * k1.y;
        *pb = b0 + ((fbL - fbR) * idx + k1.x * (MB - b0)) * k1.y;
        fhL = fhR;
        fbL = fbR;
      }
    }
  };
  if (all_vl) pointwise(std::true_type{});
  else pointwise(std::false_type{});
  __syncthreads();  // the window and coefficients are reused by the next segment
  }
}


// One compiled shape of the segment kernel.
struct SegVariant {
  int seg, threads;
  const void* fn;                 // k_batch_seg<seg, threads>
  int (*smem)(int sst_max, int nu4_max);
  int smem_max;
};
void seg_variants_a(std::vector<SegVariant>& out);
void seg_variants_b(std::vector<SegVariant>& out);

}  // namespace kb
