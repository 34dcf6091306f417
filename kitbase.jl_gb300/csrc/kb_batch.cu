// kb_batch.cu -- many independent 1D2F1V solves (uneven cell counts and
// velocity grids) advanced by ONE persistent kernel launch per time step.
//
// Ragged layout: instance b owns cells [cell_off[b], cell_off[b] + nxt[b])
// (ghosts included) and a velocity table at vel_off[b] of length nu[b]; its
// distributions start at elem_off[b] in the flat h / b arrays and are
// [cell][nus[b]] (velocity fastest, rows padded to a multiple of 4 values so
// every row starts 16-byte aligned for bulk copies).  Each step runs three
// phases per instance:
//   A  face moments fw (blocked compensated sums over velocities) and the
//      old heat flux q
//   C  cell parameters: w, prim, tau, residual terms, the instance's
//      residual and convergence flag
//   D  pointwise KFVS flux + BGK / Shakhov relaxation (one thread per
//      velocity, marching the cells)
// FP32 split form: k_batch_seg fuses A, C and D for one 16-cell segment of
// one instance per CTA (one pass over HBM), and k_batch_seg_res forms each
// instance's residual from its segments' partial sums.  FP64 form
// (k_batch_step, the comparator): a CTA takes whole instances from a work
// counter (largest first).
// Covers the configuration of the batched shock-structure ensemble: KFVS,
// BGK or Shakhov, fixed boundaries, van Leer, up to 256 velocities.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <numeric>
#include <string>
#include <vector>

#include "../../include/kitgpu.h"
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

template <typename R, int BS>
__global__ void __launch_bounds__(BS) k_batch_step(BatchDev B, const R* __restrict__ Hin,
                                                    const R* __restrict__ Bin, R* __restrict__ Hout,
                                                    R* __restrict__ Bout) {
  __shared__ int s_b;
  __shared__ double red[BS / 32][8];
  const int tid = threadIdx.x, lane = tid & 31, wid = tid >> 5;
  for (;;) {
    if (tid == 0) s_b = atomicAdd(B.counter, 1);
    __syncthreads();
    const int slot = s_b;
    __syncthreads();
    if (slot >= B.n) return;
    const int b = B.order[slot];
    const int nx = B.nx[b], ng = B.ng[b], nu = B.nu[b], ns = B.nus[b];
    const long c0 = B.cell_off[b], e0 = B.elem_off[b];
    const int nxt = nx + 2 * ng;
    const R* Hi = Hin + e0;
    const R* Bi = Bin + e0;
    R* Ho = Hout + e0;
    R* Bo = Bout + e0;
    if (!B.active[b]) {  // converged: carry the state over
      for (long k = tid; k < (long)nxt * ns; k += BS) {
        Ho[k] = Hi[k];
        Bo[k] = Bi[k];
      }
      continue;
    }
    const R* U = btab<R>(B, 0) + B.vel_off[b];
    const R* W = btab<R>(B, 1) + B.vel_off[b];
    const double dx = B.dx[b], dt = B.dt[b];
    const R epsd = R(1.e-7 * dx);
    double* fw = B.fw + B.face_off[b] * 4;
    // ---- A: face moments (faces 1 .. nx-1 bound the stepped cells) and q
    const R T3 = R(dt), T4 = R(0.5 * dt * dt / dx);
    for (int f = 1 + tid; f <= nx - 1; f += BS) {
      BSum<R> s0, s1, s2;
      s0.init();
      s1.init();
      s2.init();
      const int iL = f - 1, iR = f;
      const int rL = brule(iL, nx, ng), rR = brule(iR, nx, ng);
      const R* hL = Hi + (long)(iL + ng) * ns;
      const R* bL = Bi + (long)(iL + ng) * ns;
      for (int v = 0; v < nu; ++v) {
        R u = U[v];
        bool pos = u >= R(0);
        const R* hc = pos ? hL : hL + ns;
        const R* bc = pos ? bL : bL + ns;
        int r = pos ? rL : rR;
        R h0 = hc[v], b0 = bc[v];
        R sh = R(0), sb = R(0);
        if (r == 1) {
          sh = bvl<R>(1, hc[v - ns], h0, hc[v + ns], epsd);
          sb = bvl<R>(1, bc[v - ns], b0, bc[v + ns], epsd);
        }
        R side = pos ? R(0.5) : R(-0.5);
        R hf = h0 + side * sh, bf = b0 + side * sb;
        R fh = T3 * u * hf - T4 * (u * u) * sh;
        R fb = T3 * u * bf - T4 * (u * u) * sb;
        R wf = W[v] * fh;
        s0.add(wf);
        s1.add(wf * u);
        s2.add(wf * u * u + W[v] * fb);
        if ((v & 7) == 7) {
          s0.flush();
          s1.flush();
          s2.flush();
        }
      }
      double* o = fw + (long)f * 4;
      o[0] = s0.get();
      o[1] = s1.get();
      o[2] = 0.5 * s2.get();
    }
    if (B.coll == COLL_SHAKHOV) {
      for (int i = 1 + tid; i <= nx - 2; i += BS) {
        BSum<R> s;
        s.init();
        const R* hc = Hi + (long)(i + ng) * ns;
        const R* bc = Bi + (long)(i + ng) * ns;
        R Uc = R(B.prim[(c0 + i + ng) * 4 + 1]);
        for (int v = 0; v < nu; ++v) {
          R cu = U[v] - Uc;
          s.add(W[v] * cu * (cu * cu * hc[v] + bc[v]));
          if ((v & 7) == 7) s.flush();
        }
        B.q[c0 + i + ng] = 0.5 * s.get();
      }
    }
    __syncthreads();
    // ---- C: cell parameters of the stepped cells 1 .. nx-2 (fixed ends)
    double rr[6] = {0, 0, 0, 0, 0, 0};
    for (int i = 1 + tid; i <= nx - 2; i += BS) {
      const long c = c0 + i + ng;
      double* w = B.w + c * 4;
      double* p = B.prim + c * 4;
      const double* fL = fw + (long)i * 4;
      const double* fR = fw + (long)(i + 1) * 4;
      double wo[3] = {w[0], w[1], w[2]};
      double lo = p[2], rho_o = p[0], Uo = p[1];
      for (int k = 0; k < 3; ++k) w[k] += (fL[k] - fR[k]) / dx;
      double pn[4];
      conserve_prim(w, 3, B.gamma, pn);
      p[0] = pn[0];
      p[1] = pn[1];
      p[2] = pn[2];
      for (int k = 0; k < 3; ++k) {
        double d = w[k] - wo[k];
        rr[k] += d * d;
        rr[3 + k] += fabs(w[k]);
      }
      double lam = pn[2];
      double tau = vhs_time(pn[0], lam, B.mu[b], B.omega);
      if (!(pn[0] > 0.0) || !(lam > 0.0) || !isfinite(pn[0]) || !isfinite(lam)) atomicOr(B.status, 1);
      double* k = B.cp + c * 16;
      k[0] = pn[0] * sqrt(lam / PI);  // new Maxwellian
      k[1] = pn[1];
      k[2] = lam;
      k[3] = B.K / (2.0 * lam);
      k[4] = dt / tau;
      k[5] = 1.0 / (1.0 + dt / tau);
      k[6] = rho_o * sqrt(lo / PI);  // old Maxwellian (Shakhov)
      k[7] = Uo;
      k[8] = lo;
      k[9] = B.K / (2.0 * lo);
      k[10] = B.coll == COLL_SHAKHOV ? 0.8 * (1.0 - B.Pr) * (lo * lo) / rho_o * B.q[c] : 0.0;
    }
    // residual (src/Solver/solver_update.jl:86-88; fixed ends add zero)
    for (int k = 0; k < 6; ++k) {
#pragma unroll
      for (int m = 16; m >= 1; m >>= 1) rr[k] += __shfl_xor_sync(0xffffffffu, rr[k], m);
    }
    if (lane == 0)
      for (int k = 0; k < 6; ++k) red[wid][k] = rr[k];
    __syncthreads();
    if (tid == 0) {
      double t[6] = {0, 0, 0, 0, 0, 0};
      for (int w8 = 0; w8 < BS / 32; ++w8)
        for (int k = 0; k < 6; ++k) t[k] += red[w8][k];
      double mx = 0.0;
      for (int k = 0; k < 3; ++k) {
        // fixed ends contribute sqrt(0 * 2) / (0 + 1e-7) = 0 (update_boundary.jl:41-44)
        double r = sqrt(t[k] * nx) / (t[3 + k] + 1.e-7);
        B.residual[b * 4 + k] = r;
        mx = fmax(mx, r);
      }
      if (mx < B.tol) B.active[b] = 0;
    }
    __syncthreads();
    // ---- D: pointwise update, one thread per velocity marching the cells
    for (int v = tid; v < nu; v += BS) {
      const R u = U[v];
      const bool pos = u >= R(0);
      const R side = pos ? R(0.5) : R(-0.5);
      auto at = [&](const R* q, int i) { return q[(long)(i + ng) * ns + v]; };
      // fixed end cells keep their state
      Ho[(long)ng * ns + v] = at(Hi, 0);
      Bo[(long)ng * ns + v] = at(Bi, 0);
      Ho[(long)(nx - 1 + ng) * ns + v] = at(Hi, nx - 1);
      Bo[(long)(nx - 1 + ng) * ns + v] = at(Bi, nx - 1);
      // window: cells i-1, i, i+1 around the upwind cell of face i (between i-1 and i)
      auto face = [&](int f, R& fh, R& fb) {
        int up = pos ? f - 1 : f;
        int r = brule(up, nx, ng);
        R h0 = at(Hi, up), b0 = at(Bi, up);
        R sh = R(0), sb = R(0);
        if (r == 1) {
          sh = bvl<R>(1, at(Hi, up - 1), h0, at(Hi, up + 1), epsd);
          sb = bvl<R>(1, at(Bi, up - 1), b0, at(Bi, up + 1), epsd);
        }
        R hf = h0 + side * sh, bf = b0 + side * sb;
        fh = T3 * u * hf - T4 * (u * u) * sh;
        fb = T3 * u * bf - T4 * (u * u) * sb;
      };
      R fhL, fbL;
      face(1, fhL, fbL);
      for (int i = 1; i <= nx - 2; ++i) {
        R fhR, fbR;
        face(i + 1, fhR, fbR);
        const long c = c0 + i + ng;
        const double* k = B.cp + c * 16;
        R h0 = at(Hi, i), b0 = at(Bi, i);
        R du = u - R(k[1]);
        R M = R(k[0]) * mexp(-R(k[2]) * du * du);
        R MH = M, MB = M * R(k[3]);
        if (B.coll == COLL_SHAKHOV) {
          R ou = u - R(k[7]);
          R OH = R(k[6]) * mexp(-R(k[8]) * ou * ou);
          R cq = R(k[10]) * ou;
          R tl = R(2) * R(k[8]) * ou * ou + R(B.K);
          MH += cq * (tl - R(5)) * OH;
          MB += cq * (tl - R(3)) * OH * R(k[9]);
        }
        R dtau = R(k[4]);
        R hn, bn;
        if (sizeof(R) == 8) {
          hn = (h0 + (fhL - fhR) / R(dx) + dtau * MH) / (R(1) + dtau);
          bn = (b0 + (fbL - fbR) / R(dx) + dtau * MB) / (R(1) + dtau);
        } else {
          R idx = R(1.0 / dx), inv = R(k[5]);
          hn = (h0 + (fhL - fhR) * idx + dtau * MH) * inv;
          bn = (b0 + (fbL - fbR) * idx + dtau * MB) * inv;
        }
        Ho[(long)(i + ng) * ns + v] = hn;
        Bo[(long)(i + ng) * ns + v] = bn;
        fhL = fhR;
        fbL = fbR;
      }
    }
    __syncthreads();
  }
}

// e^x on the MUFU unit (2^(x log2 e), results below 2^-126 flushed to zero)
__device__ __forceinline__ float fexp(float x) {
  float y;
  asm("ex2.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x * 1.4426950408889634f));
  return y;
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
constexpr int SEG = 16;
constexpr int SEG_T = 128;
constexpr int SEG_ROWS = SEG + 4;
constexpr int SEG_MAXNU = 256;
__host__ __device__ inline int seg_stride(int nus) { return (nus + 31) / 32 * 32 + 4; }
constexpr int SEG_FT = SEG_T / (SEG + 1);  // threads per face in the face-moment phase
static_assert(SEG_FT >= 1 && SEG * 8 <= SEG_T, "thread groups of the moment phases");
// Dynamic shared memory of a segment CTA, sized by the batch's largest row
// stride and velocity count: h and b windows, velocity tables, fw, the
// 16-byte aligned cell coefficients, the face-moment partials and the old
// prim of the stepped cells.
constexpr int SEG_CC = 4;  // float4 coefficient blocks per cell
__host__ __device__ inline int seg_smem(int sst_max, int nu4_max) {
  return 2 * SEG_ROWS * sst_max * 4 + 3 * nu4_max * 4 + (SEG + 1) * 3 * 8 + 16 +
         SEG * SEG_CC * 16 + SEG_T * 6 * 4 + SEG * 3 * 8 + 8 * 8;
}
constexpr int SEG_SMEM_MAX = 2 * SEG_ROWS * ((SEG_MAXNU + 31) / 32 * 32 + 4) * 4 +
                             3 * SEG_MAXNU * 4 + (SEG + 1) * 3 * 8 + 16 + SEG * SEG_CC * 16 +
                             SEG_T * 6 * 4 + SEG * 3 * 8 + 8 * 8;

__global__ void __launch_bounds__(SEG_T) k_batch_seg(BatchDev B, const float* __restrict__ Hin,
                                                     const float* __restrict__ Bin,
                                                     float* __restrict__ Hout,
                                                     float* __restrict__ Bout) {
  extern __shared__ __align__(16) unsigned char sm[];
  __shared__ unsigned long long bar;
  __shared__ float sconst[4];  // T3, T4, 1/dx, 1e-7 dx
  // GB300 runs FP64 at 1/64 of the FP32 rate: FP64 work below is done by as
  // few warps as possible (the per-instance constants by one thread, the
  // cell update and its residual by the first warp)
  const int tid = threadIdx.x, lane = tid & 31, wid = tid >> 5;
  const int k = blockIdx.x;
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
    return;
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
  if (tid == 0) {
    mbar_init(&bar, 1);
    fence_async_smem();
  }
  __syncthreads();
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
  const bool ok = tid == 0 ? mbar_wait(&bar, 0) : true;
  if (__syncthreads_or(!ok)) {  // CTA-uniform: bounded clean-up, then leave
    if (tid == 0) {
      atomicOr(B.status, 2);
      mbar_wait(&bar, 0);
    }
    return;
  }
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
    BSum<float> s0, s1, s2;
    s0.init();
    s1.init();
    s2.init();
    if (j <= SEG && f <= fb) {
      const int iL = f - 1, iR = f;
      const int rL = brule(iL, nx, ng), rR = brule(iR, nx, ng);
      int it = 0;
      for (int v = q; v < nu; v += SEG_FT, ++it) {
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
        const float wf = sW[v] * fh;
        s0.add(wf);
        s1.add(wf * u);
        s2.add(wf * u * u + sW[v] * fbb);
        if ((it & 7) == 7) {
          s0.flush();
          s1.flush();
          s2.flush();
        }
      }
    }
    // each thread's compensated partials, merged per face below in thread
    // order: both segments that share a face map it to the same threads q,
    // so they compute bit-identical fw (conservation holds exactly)
    s0.flush();
    s1.flush();
    s2.flush();
    float* o = sred + tid * 6;
    o[0] = s0.d.hi;
    o[1] = s0.d.lo;
    o[2] = s1.d.hi;
    o[3] = s1.d.lo;
    o[4] = s2.d.hi;
    o[5] = s2.d.lo;
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
  static_assert(SEG <= 32 && 4 * SEG <= 64, "cell update on warp 0, heat flux on warps 1-2");
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
      const float Uh = float(pn[1]), oUh = float(Uo);
      float4* kc = scc + lane * SEG_CC;
      // new Maxwellian: density factor, U (hi), lambda, K / (2 lambda)
      kc[0] = make_float4(float(pn[0] * sqrt(lam * (1.0 / PI))), Uh, lf, float(Kd / (2.0 * lam)));
      // dt / tau, 1 / (1 + dt / tau), old Maxwellian (Shakhov) density factor and U (hi)
      kc[1] = make_float4(dtt, 1.f / (1.f + dtt), float(rho_o * sqrt(lo * (1.0 / PI))), oUh);
      // old lambda, K / (2 lambda); .z (the Shakhov heat-flux factor) comes
      // from warps 1-2; .w the low part of U
      float* k2 = (float*)(kc + 2);
      k2[0] = float(lo);
      k2[1] = float(Kd / (2.0 * lo));
      k2[3] = float(pn[1] - (double)Uh);
      kc[3] = make_float4(float(Uo - (double)oUh), 0.f, 0.f, 0.f);
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
  } else if (wid <= 2) {
    // ---- old heat flux of the stepped cells, 4 threads per cell, and the
    // Shakhov factor 0.8 (1 - Pr) lambda^2 / rho q of the cell coefficients
    const int lt = tid - 32, jc = lt >> 2, q = lt & 3;
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
        for (int v = q; v < nu; v += 4, ++it) {
          const float cu = (sU[v] - Uc) + (sUl[v] - Ul);
          sm4.add(sW[v] * cu * (cu * cu * hc[v] + bc[v]));
          if ((it & 7) == 7) sm4.flush();
        }
      }
      sm4.flush();
      DF d = sm4.d;
#pragma unroll
      for (int m = 1; m <= 2; m <<= 1) d = df_merge(d, df_shfl_xor(d, m));
      if (i < cb) {
        const double qc = 0.5 * ((double)d.hi + (double)d.lo);
        const float rof = float(spo[jc * 3 + 0]), lof = float(spo[jc * 3 + 2]);
        qf = float(0.8 * (1.0 - B.Pr)) * (lof * lof) / rof * float(qc);
      }
    }
    if (q == 0 && i < cb) ((float*)(scc + jc * SEG_CC + 2))[2] = qf;
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
        const float du = (u - k0.y) + (ulo - k2.w);
        const float M = k0.x * fexp(-k0.z * du * du);
        float MH = M, MB = M * k0.w;
        if (B.coll == COLL_SHAKHOV) {
          const float ou = (u - k1.w) + (ulo - kc[3].x);
          const float OH = k1.z * fexp(-k2.x * ou * ou);
          const float cq = k2.z * ou;
          const float tl = 2.f * k2.x * ou * ou + float(B.K);
          MH += cq * (tl - 5.f) * OH;
          MB += cq * (tl - 3.f) * OH * k2.y;
        }
        *ph = (h0 + (fhL - fhR) * idx + k1.x * MH) * k1.y;
        *pb = (b0 + (fbL - fbR) * idx + k1.x * MB) * k1.y;
        fhL = fhR;
        fbL = fbR;
      }
    }
  };
  if (all_vl) pointwise(std::true_type{});
  else pointwise(std::false_type{});
}

// Residual of each active instance of the segment form
// (src/Solver/solver_update.jl:86-88) and its convergence flag.  One warp per
// instance: lane l adds the partial sums of segments l, l + 32, ... in order,
// then a fixed shuffle tree combines the lanes (deterministic).  Launched
// after k_batch_seg on the same stream, so no segment CTA waits on a fence or
// an atomic counter of the others.
__global__ void k_batch_seg_res(BatchDev B) {
  const int b = (int)((blockIdx.x * (long)blockDim.x + threadIdx.x) >> 5), lane = threadIdx.x & 31;
  if (b >= B.n || !B.active[b]) return;  // warp-uniform
  double t[6] = {0, 0, 0, 0, 0, 0};
  const int s0 = B.seg_first[b], s1 = s0 + B.nseg[b];
  for (int sgi = s0 + lane; sgi < s1; sgi += 32)
    for (int m = 0; m < 6; ++m) t[m] += B.respart[(long)sgi * 8 + m];
#pragma unroll
  for (int m = 0; m < 6; ++m) t[m] = warp_sum(t[m]);
  if (lane == 0) {
    double mx = 0.0;
    for (int m = 0; m < 3; ++m) {
      const double r = sqrt(t[m] * B.nx[b]) / (t[3 + m] + 1.e-7);
      B.residual[b * 4 + m] = r;
      mx = fmax(mx, r);
    }
    if (mx < B.tol) B.active[b] = 0;
  }
}

__global__ void k_batch_timestep(BatchDev B, const double* umax, double cfl, double* dt_out) {
  const int b = blockIdx.x;
  __shared__ double red[256];
  const int nx = B.nx[b], ng = B.ng[b];
  double m = 0.0;
  for (int i = threadIdx.x; i < nx; i += blockDim.x) {
    const double* p = B.prim + (B.cell_off[b] + i + ng) * 4;
    double sos = pow(0.5 * B.gamma / p[2], 0.5);
    m = fmax(m, (fmax(umax[b], fabs(p[1])) + sos) / B.dx[b]);
  }
  red[threadIdx.x] = m;
  __syncthreads();
  for (int s = blockDim.x / 2; s >= 1; s >>= 1) {
    if (threadIdx.x < s) red[threadIdx.x] = fmax(red[threadIdx.x], red[threadIdx.x + s]);
    __syncthreads();
  }
  if (threadIdx.x == 0) dt_out[b] = cfl / red[0];
}

template <typename R>
__global__ void k_batch_convert(R* dst, const double* src, long n) {
  long t = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t < n) dst[t] = (R)src[t];
}
template <typename R>
__global__ void k_batch_back(double* dst, const R* src, long n) {
  long t = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t < n) dst[t] = (double)src[t];
}

}  // namespace kb

// ---------------------------------------------------------------- C ABI

struct kb_batch {
  kb::BatchDev d;
  int prec = 0;
  int n = 0;
  long ncell = 0, nelem = 0, nface = 0, nvel = 0;
  void* h[2] = {nullptr, nullptr};
  void* bq[2] = {nullptr, nullptr};
  int cur = 0;
  cudaStream_t stream = nullptr;
  std::vector<void*> allocs;
  std::vector<int> nx, ng, nu, nus;
  std::vector<long> cell_off, elem_off, dense_off;  // dense_off: caller layout [cell][nu]
  long ndense = 0, nseg = 0;
  double* d_stage = nullptr;
  double* d_umax = nullptr;
  cudaGraphExec_t graph = nullptr;
  int graph_cur = -1;
  int grid = 0;
  int64_t launches = 0;
};

static int bfail(int code, const std::string& m) {
  kb::set_error(m);
  return code;
}

static int balloc(kb_batch* B, void** p, size_t bytes) {
  if (bytes == 0) bytes = 16;
  if (cudaMalloc(p, bytes) != cudaSuccess) {
    cudaGetLastError();
    return bfail(KB_ERR_NOMEM, "cudaMalloc failed (" + std::to_string(bytes) + " bytes)");
  }
  B->allocs.push_back(*p);
  return KB_OK;
}

extern "C" int kb_batch_destroy(kb_batch_t* B) {
  if (!B) return KB_OK;
  if (B->stream) cudaStreamSynchronize(B->stream);
  if (B->graph) cudaGraphExecDestroy(B->graph);
  for (void* p : B->allocs) cudaFree(p);
  if (B->stream) cudaStreamDestroy(B->stream);
  delete B;
  return KB_OK;
}

extern "C" int kb_batch_create(const kb_config_t* base, int32_t n, const int32_t* nx,
                               const int32_t* ngx, const int32_t* nu, const double* x0,
                               const double* x1, const double* umax, const double* mu_ref,
                               const double* u_all, const double* w_all, kb_batch_t** out) {
  if (!base || n <= 0 || !nx || !ngx || !nu || !x0 || !x1 || !umax || !mu_ref || !u_all ||
      !w_all || !out)
    return bfail(KB_ERR_ARG, "kb_batch_create: null argument or empty batch");
  if (base->dim != 1 || base->nf == 1) return bfail(KB_ERR_CONFIG, "batched solves are 1D2F1V");
  if (base->flux != KB_FLUX_KFVS) return bfail(KB_ERR_CONFIG, "batched solves use KFVS");
  if (base->bc[0] != KB_BC_FIX || base->bc[1] != KB_BC_FIX)
    return bfail(KB_ERR_CONFIG, "batched solves use fixed boundaries");
  if (base->interp_order != 2) return bfail(KB_ERR_CONFIG, "batched solves use van Leer slopes");
  if (base->precision != KB_PREC_FP64 && base->precision != KB_PREC_FP32)
    return bfail(KB_ERR_CONFIG, "unknown precision");
  for (int b = 0; b < n; ++b) {
    if (nx[b] < 3 || nu[b] < 1 || nu[b] > 256 || ngx[b] < 0 || ngx[b] > 2 || !(x1[b] > x0[b]))
      return bfail(KB_ERR_CONFIG, "instance " + std::to_string(b) +
                                      ": need nx >= 3, 1 <= nu <= 256, 0 <= ng <= 2, x1 > x0");
  }
  kb_batch* B = new kb_batch();
  B->prec = base->precision;
  B->n = n;
  B->nx.assign(nx, nx + n);
  B->ng.assign(ngx, ngx + n);
  B->nu.assign(nu, nu + n);
  std::vector<long> face_off(n), vel_off_l(n);
  std::vector<int> vel_off(n);
  std::vector<double> dx(n), dt(n, 0.0), mu(mu_ref, mu_ref + n);
  B->cell_off.resize(n);
  B->elem_off.resize(n);
  long cells = 0, elems = 0, faces = 0, vels = 0;
  B->nus.resize(n);
  B->dense_off.resize(n);
  std::vector<int> seg_b, seg_i0, seg_first(n), nseg(n);
  long dense = 0;
  for (int b = 0; b < n; ++b) {
    B->cell_off[b] = cells;
    B->elem_off[b] = elems;
    B->dense_off[b] = dense;
    face_off[b] = faces;
    vel_off[b] = (int)vels;
    long nxt = nx[b] + 2 * ngx[b];
    B->nus[b] = (nu[b] + 3) / 4 * 4;
    cells += nxt;
    elems += nxt * B->nus[b];
    dense += nxt * nu[b];
    faces += nx[b] + 1;
    vels += nu[b];
    dx[b] = (x1[b] - x0[b]) / nx[b];
    seg_first[b] = (int)seg_b.size();
    nseg[b] = (nx[b] + kb::SEG - 1) / kb::SEG;
    for (int k = 0; k < nseg[b]; ++k) {
      seg_b.push_back(b);
      seg_i0.push_back(k * kb::SEG);
    }
  }
  B->ndense = dense;
  B->nseg = (long)seg_b.size();
  B->ncell = cells;
  B->nelem = elems;
  B->nface = faces;
  B->nvel = vels;
  // largest instances first
  std::vector<int> order(n);
  std::iota(order.begin(), order.end(), 0);
  std::stable_sort(order.begin(), order.end(), [&](int a, int c) {
    return (long)nx[a] * nu[a] > (long)nx[c] * nu[c];
  });
  auto fail_out = [&](int rc) {
    kb_batch_destroy(B);
    return rc;
  };
  if (cudaStreamCreateWithFlags(&B->stream, cudaStreamNonBlocking) != cudaSuccess)
    return fail_out(bfail(KB_ERR_CUDA, "cudaStreamCreate failed"));
  void* p;
  int rc;
#define BALLOC(dst, T, count)                                              \
  if ((rc = balloc(B, &p, sizeof(T) * (size_t)(count))) != KB_OK) return fail_out(rc); \
  dst = (T*)p;
  int *d_order, *d_nx, *d_ng, *d_nu, *d_vo, *d_active, *d_counter, *d_status;
  int *d_nus, *d_segb, *d_segi0, *d_segfirst, *d_nseg;
  double* d_respart;
  long *d_co, *d_eo, *d_fo;
  double *d_dx, *d_dt, *d_mu, *d_u, *d_w, *d_wv, *d_prim, *d_fw, *d_q, *d_cp, *d_res;
  float *d_uf, *d_wf, *d_ul;
  BALLOC(d_order, int, n);
  BALLOC(d_nx, int, n);
  BALLOC(d_ng, int, n);
  BALLOC(d_nu, int, n);
  BALLOC(d_nus, int, n);
  BALLOC(d_segb, int, B->nseg);
  BALLOC(d_segi0, int, B->nseg);
  BALLOC(d_segfirst, int, n);
  BALLOC(d_nseg, int, n);
  BALLOC(d_respart, double, B->nseg * 8);
  BALLOC(d_vo, int, n);
  BALLOC(d_active, int, n);
  BALLOC(d_counter, int, 2);
  BALLOC(d_status, int, 1);
  BALLOC(d_co, long, n);
  BALLOC(d_eo, long, n);
  BALLOC(d_fo, long, n);
  BALLOC(d_dx, double, n);
  BALLOC(d_dt, double, n);
  BALLOC(d_mu, double, n);
  BALLOC(d_u, double, vels);
  BALLOC(d_wv, double, vels);
  BALLOC(d_uf, float, vels);
  BALLOC(d_ul, float, vels);
  BALLOC(d_wf, float, vels);
  BALLOC(d_w, double, cells * 4);
  BALLOC(d_prim, double, cells * 4);
  BALLOC(d_fw, double, faces * 4);
  BALLOC(d_q, double, cells);
  BALLOC(d_cp, double, cells * 16);
  BALLOC(d_res, double, (size_t)n * 4);
  BALLOC(B->d_umax, double, n);
  size_t esz = B->prec == KB_PREC_FP64 ? 8 : 4;
  for (int k = 0; k < 2; ++k) {
    if ((rc = balloc(B, &B->h[k], esz * elems)) != KB_OK) return fail_out(rc);
    if ((rc = balloc(B, &B->bq[k], esz * elems)) != KB_OK) return fail_out(rc);
  }
  BALLOC(B->d_stage, double, elems);
  // padding values of the distribution rows stay zero in both buffers
  for (int k = 0; k < 2; ++k) {
    cudaMemset(B->h[k], 0, esz * elems);
    cudaMemset(B->bq[k], 0, esz * elems);
  }
#undef BALLOC
  std::vector<float> uf(u_all, u_all + vels), wf(w_all, w_all + vels), ul(vels);
  for (long k = 0; k < vels; ++k) ul[k] = float(u_all[k] - (double)uf[k]);
  std::vector<int> ones(n, 1);
  bool ok = true;
  ok &= cudaMemcpy(d_order, order.data(), sizeof(int) * n, cudaMemcpyHostToDevice) == cudaSuccess;
  ok &= cudaMemcpy(d_nx, nx, sizeof(int) * n, cudaMemcpyHostToDevice) == cudaSuccess;
  ok &= cudaMemcpy(d_ng, ngx, sizeof(int) * n, cudaMemcpyHostToDevice) == cudaSuccess;
  ok &= cudaMemcpy(d_nu, nu, sizeof(int) * n, cudaMemcpyHostToDevice) == cudaSuccess;
  ok &= cudaMemcpy(d_nus, B->nus.data(), sizeof(int) * n, cudaMemcpyHostToDevice) == cudaSuccess;
  ok &= cudaMemcpy(d_segb, seg_b.data(), sizeof(int) * B->nseg, cudaMemcpyHostToDevice) == cudaSuccess;
  ok &= cudaMemcpy(d_segi0, seg_i0.data(), sizeof(int) * B->nseg, cudaMemcpyHostToDevice) == cudaSuccess;
  ok &= cudaMemcpy(d_segfirst, seg_first.data(), sizeof(int) * n, cudaMemcpyHostToDevice) == cudaSuccess;
  ok &= cudaMemcpy(d_nseg, nseg.data(), sizeof(int) * n, cudaMemcpyHostToDevice) == cudaSuccess;
  ok &= cudaMemset(d_respart, 0, sizeof(double) * B->nseg * 8) == cudaSuccess;
  ok &= cudaMemcpy(d_vo, vel_off.data(), sizeof(int) * n, cudaMemcpyHostToDevice) == cudaSuccess;
  ok &= cudaMemcpy(d_active, ones.data(), sizeof(int) * n, cudaMemcpyHostToDevice) == cudaSuccess;
  ok &= cudaMemcpy(d_co, B->cell_off.data(), sizeof(long) * n, cudaMemcpyHostToDevice) == cudaSuccess;
  ok &= cudaMemcpy(d_eo, B->elem_off.data(), sizeof(long) * n, cudaMemcpyHostToDevice) == cudaSuccess;
  ok &= cudaMemcpy(d_fo, face_off.data(), sizeof(long) * n, cudaMemcpyHostToDevice) == cudaSuccess;
  ok &= cudaMemcpy(d_dx, dx.data(), sizeof(double) * n, cudaMemcpyHostToDevice) == cudaSuccess;
  ok &= cudaMemcpy(d_dt, dt.data(), sizeof(double) * n, cudaMemcpyHostToDevice) == cudaSuccess;
  ok &= cudaMemcpy(d_mu, mu.data(), sizeof(double) * n, cudaMemcpyHostToDevice) == cudaSuccess;
  ok &= cudaMemcpy(d_u, u_all, sizeof(double) * vels, cudaMemcpyHostToDevice) == cudaSuccess;
  ok &= cudaMemcpy(d_wv, w_all, sizeof(double) * vels, cudaMemcpyHostToDevice) == cudaSuccess;
  ok &= cudaMemcpy(d_uf, uf.data(), sizeof(float) * vels, cudaMemcpyHostToDevice) == cudaSuccess;
  ok &= cudaMemcpy(d_ul, ul.data(), sizeof(float) * vels, cudaMemcpyHostToDevice) == cudaSuccess;
  ok &= cudaMemcpy(d_wf, wf.data(), sizeof(float) * vels, cudaMemcpyHostToDevice) == cudaSuccess;
  ok &= cudaMemcpy(B->d_umax, umax, sizeof(double) * n, cudaMemcpyHostToDevice) == cudaSuccess;
  ok &= cudaMemset(d_status, 0, sizeof(int)) == cudaSuccess;
  ok &= cudaMemset(d_q, 0, sizeof(double) * cells) == cudaSuccess;
  ok &= cudaMemset(d_fw, 0, sizeof(double) * faces * 4) == cudaSuccess;
  ok &= cudaMemset(d_res, 0, sizeof(double) * n * 4) == cudaSuccess;
  if (!ok) return fail_out(bfail(KB_ERR_CUDA, "batch table upload failed"));
  kb::BatchDev& d = B->d;
  d.n = n;
  d.order = d_order;
  d.nx = d_nx;
  d.ng = d_ng;
  d.nu = d_nu;
  d.nus = d_nus;
  d.seg_b = d_segb;
  d.seg_i0 = d_segi0;
  d.seg_first = d_segfirst;
  d.nseg = d_nseg;
  d.respart = d_respart;
  d.sst_max = 4;
  d.nu4_max = 4;
  for (int b = 0; b < n; ++b) {
    d.sst_max = std::max(d.sst_max, kb::seg_stride(B->nus[b]));
    d.nu4_max = std::max(d.nu4_max, B->nus[b]);
  }
  d.cell_off = d_co;
  d.elem_off = d_eo;
  d.vel_off = d_vo;
  d.dx = d_dx;
  d.dt = d_dt;
  d.mu = d_mu;
  d.u = d_u;
  d.wt = d_wv;
  d.uf = d_uf;
  d.ul = d_ul;
  d.wtf = d_wf;
  d.w = d_w;
  d.prim = d_prim;
  d.fw = d_fw;
  d.face_off = d_fo;
  d.q = d_q;
  d.cp = d_cp;
  d.residual = d_res;
  d.active = d_active;
  d.counter = d_counter;
  d.status = d_status;
  d.K = base->K;
  d.gamma = base->gamma;
  d.omega = base->omega;
  d.Pr = base->Pr;
  d.tol = 0.0;
  d.coll = base->collision;
  int dev = 0, sms = 1, per = 1;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  if (B->prec == KB_PREC_FP64)
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, kb::k_batch_step<double, 256>, 256, 0);
  else
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, kb::k_batch_step<float, 256>, 256, 0);
  B->grid = std::min(n, std::max(1, sms * per));
  // the segment kernel's dynamic shared memory limit, raised on this device
  // once per batch here rather than at launch (launches may sit inside a
  // stream capture, and batches may be driven from several host threads)
  if (B->prec == KB_PREC_FP32 &&
      cudaFuncSetAttribute(kb::k_batch_seg, cudaFuncAttributeMaxDynamicSharedMemorySize,
                           kb::SEG_SMEM_MAX) != cudaSuccess)
    return fail_out(bfail(KB_ERR_CUDA, "kb_batch_create: shared-memory attribute refused"));
  *out = B;
  return KB_OK;
}

extern "C" int kb_batch_upload(kb_batch_t* B, const double* w, const double* prim,
                               const double* h, const double* bq) {
  if (!B || !w || !prim || !h || !bq) return bfail(KB_ERR_ARG, "kb_batch_upload: null argument");
  std::vector<double> w4(B->ncell * 4, 0.0), p4(B->ncell * 4, 0.0);
  for (long c = 0; c < B->ncell; ++c)
    for (int k = 0; k < 3; ++k) {
      w4[c * 4 + k] = w[c * 3 + k];
      p4[c * 4 + k] = prim[c * 3 + k];
    }
  if (cudaMemcpy(B->d.w, w4.data(), sizeof(double) * w4.size(), cudaMemcpyHostToDevice) != cudaSuccess ||
      cudaMemcpy(B->d.prim, p4.data(), sizeof(double) * p4.size(), cudaMemcpyHostToDevice) != cudaSuccess)
    return bfail(KB_ERR_CUDA, "kb_batch_upload: copy failed");
  const long n = B->nelem;
  const unsigned g = (unsigned)((n + 255) / 256);
  std::vector<double> pad(n, 0.0);  // caller rows of nu values -> padded rows
  for (int which = 0; which < 2; ++which) {
    const double* src = which == 0 ? h : bq;
    for (int b = 0; b < B->n; ++b) {
      const long nxt = B->nx[b] + 2 * B->ng[b];
      for (long c = 0; c < nxt; ++c)
        std::memcpy(&pad[B->elem_off[b] + c * B->nus[b]], src + B->dense_off[b] + c * B->nu[b],
                    sizeof(double) * B->nu[b]);
    }
    if (cudaMemcpy(B->d_stage, pad.data(), sizeof(double) * n, cudaMemcpyHostToDevice) != cudaSuccess)
      return bfail(KB_ERR_CUDA, "kb_batch_upload: copy failed");
    for (int k = 0; k < 2; ++k) {
      void* dst = which == 0 ? B->h[k] : B->bq[k];
      if (B->prec == KB_PREC_FP64)
        kb::k_batch_convert<double><<<g, 256, 0, B->stream>>>((double*)dst, B->d_stage, n);
      else
        kb::k_batch_convert<float><<<g, 256, 0, B->stream>>>((float*)dst, B->d_stage, n);
      B->launches++;
    }
    cudaStreamSynchronize(B->stream);
  }
  std::vector<int> ones(B->n, 1);
  cudaMemcpy((void*)B->d.active, ones.data(), sizeof(int) * B->n, cudaMemcpyHostToDevice);
  cudaMemset(B->d.status, 0, sizeof(int));
  B->cur = 0;
  if (cudaGetLastError() != cudaSuccess) return bfail(KB_ERR_CUDA, "kb_batch_upload failed");
  return KB_OK;
}

extern "C" int kb_batch_download(kb_batch_t* B, double* w, double* prim, double* h, double* bq) {
  if (!B) return bfail(KB_ERR_ARG, "kb_batch_download: null handle");
  cudaStreamSynchronize(B->stream);
  if (w || prim) {
    std::vector<double> w4(B->ncell * 4), p4(B->ncell * 4);
    cudaMemcpy(w4.data(), B->d.w, sizeof(double) * w4.size(), cudaMemcpyDeviceToHost);
    cudaMemcpy(p4.data(), B->d.prim, sizeof(double) * p4.size(), cudaMemcpyDeviceToHost);
    for (long c = 0; c < B->ncell; ++c)
      for (int k = 0; k < 3; ++k) {
        if (w) w[c * 3 + k] = w4[c * 4 + k];
        if (prim) prim[c * 3 + k] = p4[c * 4 + k];
      }
  }
  const long n = B->nelem;
  const unsigned g = (unsigned)((n + 255) / 256);
  std::vector<double> pad(n);
  for (int which = 0; which < 2; ++which) {
    double* dst = which == 0 ? h : bq;
    if (!dst) continue;
    const void* src = which == 0 ? B->h[B->cur] : B->bq[B->cur];
    if (B->prec == KB_PREC_FP64)
      kb::k_batch_back<double><<<g, 256, 0, B->stream>>>(B->d_stage, (const double*)src, n);
    else
      kb::k_batch_back<float><<<g, 256, 0, B->stream>>>(B->d_stage, (const float*)src, n);
    B->launches++;
    cudaStreamSynchronize(B->stream);
    cudaMemcpy(pad.data(), B->d_stage, sizeof(double) * n, cudaMemcpyDeviceToHost);
    for (int b = 0; b < B->n; ++b) {
      const long nxt = B->nx[b] + 2 * B->ng[b];
      for (long c = 0; c < nxt; ++c)
        std::memcpy(dst + B->dense_off[b] + c * B->nu[b], &pad[B->elem_off[b] + c * B->nus[b]],
                    sizeof(double) * B->nu[b]);
    }
  }
  if (cudaGetLastError() != cudaSuccess) return bfail(KB_ERR_CUDA, "kb_batch_download failed");
  return KB_OK;
}

extern "C" int kb_batch_timestep(kb_batch_t* B, double cfl, double* dt_out) {
  if (!B) return bfail(KB_ERR_ARG, "kb_batch_timestep: null handle");
  kb::k_batch_timestep<<<B->n, 256, 0, B->stream>>>(B->d, B->d_umax, cfl, (double*)B->d.dt);
  B->launches++;
  cudaStreamSynchronize(B->stream);
  if (dt_out) cudaMemcpy(dt_out, B->d.dt, sizeof(double) * B->n, cudaMemcpyDeviceToHost);
  if (cudaGetLastError() != cudaSuccess) return bfail(KB_ERR_CUDA, "kb_batch_timestep failed");
  return KB_OK;
}

extern "C" int kb_batch_set_dt(kb_batch_t* B, const double* dt) {
  if (!B || !dt) return bfail(KB_ERR_ARG, "kb_batch_set_dt: null argument");
  if (cudaMemcpy((void*)B->d.dt, dt, sizeof(double) * B->n, cudaMemcpyHostToDevice) != cudaSuccess)
    return bfail(KB_ERR_CUDA, "kb_batch_set_dt failed");
  return KB_OK;
}

// Kernels batch_launch issues per step: the FP32 segment form adds the
// per-instance residual kernel.
static int batch_kernels_per_step(const kb_batch* B) { return B->prec == KB_PREC_FP32 ? 2 : 1; }

static void batch_launch(kb_batch* B, int cur) {
  if (B->prec == KB_PREC_FP32) {  // fused segments (one pass over HBM)
    const int smem = kb::seg_smem(B->d.sst_max, B->d.nu4_max);
    kb::k_batch_seg<<<(unsigned)B->nseg, kb::SEG_T, smem, B->stream>>>(
        B->d, (const float*)B->h[cur], (const float*)B->bq[cur], (float*)B->h[cur ^ 1],
        (float*)B->bq[cur ^ 1]);
    kb::k_batch_seg_res<<<(unsigned)((B->n + 3) / 4), 128, 0, B->stream>>>(B->d);
    return;
  }
  cudaMemsetAsync(B->d.counter, 0, sizeof(int), B->stream);
  if (B->prec == KB_PREC_FP64)
    kb::k_batch_step<double, 256><<<B->grid, 256, 0, B->stream>>>(
        B->d, (const double*)B->h[cur], (const double*)B->bq[cur], (double*)B->h[cur ^ 1],
        (double*)B->bq[cur ^ 1]);
  else
    kb::k_batch_step<float, 256><<<B->grid, 256, 0, B->stream>>>(
        B->d, (const float*)B->h[cur], (const float*)B->bq[cur], (float*)B->h[cur ^ 1],
        (float*)B->bq[cur ^ 1]);
}

// Two steps (ping and pong) captured once as a CUDA graph and replayed.
static int batch_graph(kb_batch* B) {
  if (B->graph && B->graph_cur == B->cur) return KB_OK;
  if (B->graph) {
    cudaGraphExecDestroy(B->graph);
    B->graph = nullptr;
  }
  cudaGraph_t g;
  if (cudaStreamBeginCapture(B->stream, cudaStreamCaptureModeThreadLocal) != cudaSuccess)
    return bfail(KB_ERR_CUDA, "graph capture failed to start");
  batch_launch(B, B->cur);
  batch_launch(B, B->cur ^ 1);
  if (cudaStreamEndCapture(B->stream, &g) != cudaSuccess)
    return bfail(KB_ERR_CUDA, "graph capture failed");
  cudaError_t e = cudaGraphInstantiate(&B->graph, g, 0);
  cudaGraphDestroy(g);
  if (e != cudaSuccess) return bfail(KB_ERR_CUDA, "graph instantiation failed");
  B->graph_cur = B->cur;
  return KB_OK;
}

extern "C" int kb_batch_step(kb_batch_t* B, int32_t nsteps, double tol, double* residual,
                             int32_t* active) {
  if (!B) return bfail(KB_ERR_ARG, "kb_batch_step: null handle");
  if (nsteps < 0) return bfail(KB_ERR_ARG, "kb_batch_step: nsteps must be >= 0");
  if (B->d.tol != tol) {
    B->d.tol = tol;
    if (B->graph) {
      cudaGraphExecDestroy(B->graph);
      B->graph = nullptr;
    }
  }
  int rc = batch_graph(B);
  if (rc != KB_OK) return rc;
  int pairs = nsteps / 2;
  for (int k = 0; k < pairs; ++k) {
    if (cudaGraphLaunch(B->graph, B->stream) != cudaSuccess)
      return bfail(KB_ERR_CUDA, "graph launch failed");
    B->launches += 2 * batch_kernels_per_step(B);
  }
  if (nsteps & 1) {
    batch_launch(B, B->cur);
    B->launches += batch_kernels_per_step(B);
    B->cur ^= 1;
  }
  if (cudaStreamSynchronize(B->stream) != cudaSuccess)
    return bfail(KB_ERR_CUDA, std::string("batch step failed: ") + cudaGetErrorString(cudaGetLastError()));
  if (residual)
    cudaMemcpy(residual, B->d.residual, sizeof(double) * 4 * B->n, cudaMemcpyDeviceToHost);
  if (active) cudaMemcpy(active, B->d.active, sizeof(int) * B->n, cudaMemcpyDeviceToHost);
  int st = 0;
  cudaMemcpy(&st, B->d.status, sizeof(int), cudaMemcpyDeviceToHost);
  if (st) return bfail(KB_ERR_NUMERIC, "non-finite or non-positive density / lambda in a batched solve");
  return KB_OK;
}

extern "C" int kb_batch_info(kb_batch_t* B, int64_t* elems, int64_t* launches) {
  if (!B) return bfail(KB_ERR_ARG, "kb_batch_info: null handle");
  if (elems) *elems = B->nelem;
  if (launches) *launches = B->launches;
  return KB_OK;
}
