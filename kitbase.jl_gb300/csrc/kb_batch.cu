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
#include <map>
#include <cstring>
#include <numeric>
#include <string>
#include <vector>

#include "../../include/kitgpu.h"
#include "kb_batch.cuh"

namespace kb {

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

__global__ void k_batch_timestep(BatchDev B, const double* umax, double cfl, double* dt_out,
                                 int b0 = 0) {
  const int b = b0 + blockIdx.x;
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

// Equilibrium h, b of instances' cells into both FP32 buffers with the
// relaxation's own FP32 Maxwellian (seg_init_cell): blockIdx.y = instance
// b0 + y, blockIdx.x = cell.
__global__ void k_batch_init_eq32(BatchDev B, int b0, float* H0, float* B0, float* H1, float* B1) {
  const int b = b0 + blockIdx.y;
  if ((int)blockIdx.x >= B.nx[b] + 2 * B.ng[b]) return;
  seg_init_cell(B, b, blockIdx.x, H0, B0, H1, B1);
}

// FP32 Maxwellian coefficients of every cell from its prim (after a host
// upload of prim): blockIdx.y = instance, one thread per cell.
__global__ void k_batch_mcache(BatchDev B) {
  const int b = blockIdx.y;
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= B.nx[b] + 2 * B.ng[b]) return;
  const long cell = B.cell_off[b] + c;
  SegMax m;
  m.set(B.prim + cell * 4, B.K);
  seg_store_coef(B, cell, m);
}

// FP64 form: h = maxwellian(u, prim), b = h K / (2 lambda) in FP64
// (src/Theory/theory_equilibrium.jl:8-13) into both buffers.
__global__ void k_batch_init_eq64(BatchDev B, double* H0, double* B0, double* H1, double* B1) {
  const int b = blockIdx.y;
  if ((int)blockIdx.x >= B.nx[b] + 2 * B.ng[b]) return;
  const double* p = B.prim + (B.cell_off[b] + blockIdx.x) * 4;
  const double rn = p[0] * sqrt(p[2] / PI), cB = B.K / (2.0 * p[2]);
  const int nu = B.nu[b], ns = B.nus[b];
  const long e = B.elem_off[b] + (long)blockIdx.x * ns;
  const double* u = B.u + B.vel_off[b];
  for (int v = threadIdx.x; v < ns; v += blockDim.x) {
    double hv = 0.0, bv = 0.0;
    if (v < nu) {
      const double du = u[v] - p[1];
      hv = rn * exp(-p[2] * du * du);
      bv = hv * cB;
    }
    H0[e + v] = hv;
    B0[e + v] = bv;
    H1[e + v] = hv;
    B1[e + v] = bv;
  }
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
  // FP32 segment kernel: shape (cells per segment, threads, persistent grid)
  // and its launch; segment tables are rebuilt when the shape changes
  int seg = 16, seg_t = 128, persist = 0;
  const void* seg_fn = nullptr;
  int seg_smem = 0, seg_grid = 0;
  int* d_segb = nullptr;
  int* d_segi0 = nullptr;
  int* d_segfirst = nullptr;
  int* d_nseg = nullptr;
  long seg_cap = 0;  // capacity of the segment tables (segments of 8 cells)
  // pool form (kb_pool_*): instance slots that requests join and leave, and
  // first-fit allocators of the cell, element and velocity ranges
  bool pool = false;
  std::vector<char> used;
  std::map<long, long> free_cells, free_elems, free_vels;  // offset -> length
  std::vector<long> vel_off_h;
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

// Compiled shapes of the FP32 segment kernel (kb_batch_seg_a.cu, _b.cu).
static const std::vector<kb::SegVariant>& seg_variants() {
  static const std::vector<kb::SegVariant> v = [] {
    std::vector<kb::SegVariant> out;
    kb::seg_variants_a(out);
    kb::seg_variants_b(out);
    return out;
  }();
  return v;
}

// Select the segment kernel's shape: segment tables for `seg` cells per
// segment (instances in processing order, their segments consecutive),
// the kernel's shared-memory limit, and the grid -- one CTA per segment, or
// (persist) as many CTAs as fit on the GPU at once, each looping over
// segments.  Runs outside any stream capture; invalidates the step graph.
static int batch_set_shape(kb_batch* B, int seg, int threads, int persist) {
  const kb::SegVariant* var = nullptr;
  for (const auto& v : seg_variants())
    if (v.seg == seg && v.threads == threads) var = &v;
  if (!var) return bfail(KB_ERR_ARG, "batch shape: no segment kernel for " + std::to_string(seg) +
                                         " cells x " + std::to_string(threads) + " threads");
  std::vector<int> seg_b, seg_i0, seg_first(B->n), nseg(B->n);
  for (int b = 0; b < B->n; ++b) {
    seg_first[b] = (int)seg_b.size();
    nseg[b] = B->pool && !B->used[b] ? 0 : (B->nx[b] + seg - 1) / seg;
    for (int k = 0; k < nseg[b]; ++k) {
      seg_b.push_back(b);
      seg_i0.push_back(k * seg);
    }
  }
  if ((long)seg_b.size() > B->seg_cap) return bfail(KB_ERR_ARG, "batch shape: segment table overflow");
  cudaStreamSynchronize(B->stream);
  bool ok = true;
  ok &= cudaMemcpy(B->d_segb, seg_b.data(), sizeof(int) * seg_b.size(), cudaMemcpyHostToDevice) == cudaSuccess;
  ok &= cudaMemcpy(B->d_segi0, seg_i0.data(), sizeof(int) * seg_i0.size(), cudaMemcpyHostToDevice) == cudaSuccess;
  ok &= cudaMemcpy(B->d_segfirst, seg_first.data(), sizeof(int) * B->n, cudaMemcpyHostToDevice) == cudaSuccess;
  ok &= cudaMemcpy(B->d_nseg, nseg.data(), sizeof(int) * B->n, cudaMemcpyHostToDevice) == cudaSuccess;
  const int smem = var->smem(B->d.sst_max, B->d.nu4_max);
  ok &= cudaFuncSetAttribute(var->fn, cudaFuncAttributeMaxDynamicSharedMemorySize, var->smem_max) ==
        cudaSuccess;
  // the carveout of every step kernel (kb::prefer_max_shared): a pool that
  // shares the GPU with other solves' streams keeps their CTAs on common SMs
  kb::prefer_max_shared(var->fn);
  kb::prefer_max_shared((const void*)kb::k_batch_seg_res);
  int per = 0, dev = 0, sms = 1;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  ok &= cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, var->fn, threads, smem) == cudaSuccess;
  if (!ok || per < 1) {
    cudaGetLastError();
    return bfail(KB_ERR_CUDA, "batch shape: segment tables or kernel attributes refused");
  }
  B->nseg = (long)seg_b.size();
  B->d.nseg_all = (int)B->nseg;
  B->seg = seg;
  B->seg_t = threads;
  B->persist = persist ? 1 : 0;
  B->seg_fn = var->fn;
  B->seg_smem = smem;
  B->seg_grid = persist ? (int)std::min<long>(B->nseg, (long)sms * per) : (int)B->nseg;
  if (B->pool && persist) B->seg_grid = sms * per;  // fixed, whatever the membership
  if (B->graph) {
    cudaGraphExecDestroy(B->graph);
    B->graph = nullptr;
  }
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
  long dense = 0;
  long seg_cap = 0;
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
    seg_cap += (nx[b] + 7) / 8;  // the shortest segment length the tuner offers
  }
  B->ndense = dense;
  B->seg_cap = seg_cap;
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
  float *d_uf, *d_wf, *d_ul, *d_mc;
  BALLOC(d_order, int, n);
  BALLOC(d_nx, int, n);
  BALLOC(d_ng, int, n);
  BALLOC(d_nu, int, n);
  BALLOC(d_nus, int, n);
  BALLOC(d_segb, int, B->seg_cap);
  BALLOC(d_segi0, int, B->seg_cap);
  BALLOC(d_segfirst, int, n);
  BALLOC(d_nseg, int, n);
  BALLOC(d_respart, double, B->seg_cap * 8);
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
  BALLOC(d_mc, float, cells * 8);
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
  ok &= cudaMemset(d_respart, 0, sizeof(double) * B->seg_cap * 8) == cudaSuccess;
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
  B->d_segb = d_segb;
  B->d_segi0 = d_segi0;
  B->d_segfirst = d_segfirst;
  B->d_nseg = d_nseg;
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
  d.mc = d_mc;
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
  if (B->prec == KB_PREC_FP32 && (rc = batch_set_shape(B, 16, 128, 0)) != KB_OK)
    return fail_out(rc);
  *out = B;
  return KB_OK;
}

extern "C" int kb_batch_upload(kb_batch_t* B, const double* w, const double* prim,
                               const double* h, const double* bq) {
  if (B && B->pool) return bfail(KB_ERR_STATE, "pools move state per slot (kb_pool_add / kb_pool_download)");
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
  if (B->prec == KB_PREC_FP32) {  // the FP32 step reads each cell's Maxwellian coefficients
    int maxc = 1;
    for (int b = 0; b < B->n; ++b) maxc = std::max(maxc, B->nx[b] + 2 * B->ng[b]);
    kb::k_batch_mcache<<<dim3((unsigned)((maxc + 127) / 128), (unsigned)B->n), 128, 0, B->stream>>>(B->d);
    B->launches++;
    cudaStreamSynchronize(B->stream);
  }
  std::vector<int> ones(B->n, 1);
  cudaMemcpy((void*)B->d.active, ones.data(), sizeof(int) * B->n, cudaMemcpyHostToDevice);
  cudaMemset(B->d.status, 0, sizeof(int));
  B->cur = 0;
  if (cudaGetLastError() != cudaSuccess) return bfail(KB_ERR_CUDA, "kb_batch_upload failed");
  return KB_OK;
}

extern "C" int kb_batch_init_equilibrium(kb_batch_t* B, const double* w, const double* prim) {
  if (B && B->pool) return bfail(KB_ERR_STATE, "pools move state per slot (kb_pool_add / kb_pool_download)");
  if (!B || !w || !prim) return bfail(KB_ERR_ARG, "kb_batch_init_equilibrium: null argument");
  std::vector<double> w4(B->ncell * 4, 0.0), p4(B->ncell * 4, 0.0);
  for (long c = 0; c < B->ncell; ++c)
    for (int k = 0; k < 3; ++k) {
      w4[c * 4 + k] = w[c * 3 + k];
      p4[c * 4 + k] = prim[c * 3 + k];
    }
  if (cudaMemcpy(B->d.w, w4.data(), sizeof(double) * w4.size(), cudaMemcpyHostToDevice) != cudaSuccess ||
      cudaMemcpy(B->d.prim, p4.data(), sizeof(double) * p4.size(), cudaMemcpyHostToDevice) != cudaSuccess)
    return bfail(KB_ERR_CUDA, "kb_batch_init_equilibrium: copy failed");
  int maxc = 1;
  for (int b = 0; b < B->n; ++b) maxc = std::max(maxc, B->nx[b] + 2 * B->ng[b]);
  const dim3 grid((unsigned)maxc, (unsigned)B->n);
  if (B->prec == KB_PREC_FP64)
    kb::k_batch_init_eq64<<<grid, 128, 0, B->stream>>>(B->d, (double*)B->h[0], (double*)B->bq[0],
                                                       (double*)B->h[1], (double*)B->bq[1]);
  else
    kb::k_batch_init_eq32<<<grid, 128, 0, B->stream>>>(B->d, 0, (float*)B->h[0], (float*)B->bq[0],
                                                       (float*)B->h[1], (float*)B->bq[1]);
  B->launches++;
  std::vector<int> ones(B->n, 1);
  cudaMemcpyAsync((void*)B->d.active, ones.data(), sizeof(int) * B->n, cudaMemcpyHostToDevice, B->stream);
  cudaMemsetAsync(B->d.status, 0, sizeof(int), B->stream);
  if (cudaStreamSynchronize(B->stream) != cudaSuccess)
    return bfail(KB_ERR_CUDA, std::string("kb_batch_init_equilibrium: ") +
                                  cudaGetErrorString(cudaGetLastError()));
  B->cur = 0;
  return KB_OK;
}

extern "C" int kb_batch_download(kb_batch_t* B, double* w, double* prim, double* h, double* bq) {
  if (B && B->pool) return bfail(KB_ERR_STATE, "pools move state per slot (kb_pool_add / kb_pool_download)");
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
  if (B && B->pool) return bfail(KB_ERR_STATE, "pool time steps are set per slot by kb_pool_add");
  if (!B) return bfail(KB_ERR_ARG, "kb_batch_timestep: null handle");
  kb::k_batch_timestep<<<B->n, 256, 0, B->stream>>>(B->d, B->d_umax, cfl, (double*)B->d.dt);
  B->launches++;
  cudaStreamSynchronize(B->stream);
  if (dt_out) cudaMemcpy(dt_out, B->d.dt, sizeof(double) * B->n, cudaMemcpyDeviceToHost);
  if (cudaGetLastError() != cudaSuccess) return bfail(KB_ERR_CUDA, "kb_batch_timestep failed");
  return KB_OK;
}

extern "C" int kb_batch_set_dt(kb_batch_t* B, const double* dt) {
  if (B && B->pool) return bfail(KB_ERR_STATE, "pool time steps are set per slot by kb_pool_add");
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
    const float* hin = (const float*)B->h[cur];
    const float* bin = (const float*)B->bq[cur];
    float* hout = (float*)B->h[cur ^ 1];
    float* bout = (float*)B->bq[cur ^ 1];
    void* args[] = {(void*)&B->d, (void*)&hin, (void*)&bin, (void*)&hout, (void*)&bout};
    if (B->seg_grid > 0)  // an empty pool has no segments
      cudaLaunchKernel(B->seg_fn, dim3((unsigned)B->seg_grid), dim3((unsigned)B->seg_t), args,
                       (size_t)B->seg_smem, B->stream);
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

extern "C" int kb_batch_set_tuning(kb_batch_t* B, const int32_t* params, int32_t n) {
  if (!B || !params || n < 1) return bfail(KB_ERR_ARG, "kb_batch_set_tuning: null argument");
  if (B->prec != KB_PREC_FP32) return KB_OK;  // the FP64 comparator has one shape
  const int seg = params[0] > 0 ? params[0] : 16;
  const int thr = n > 1 && params[1] > 0 ? params[1] : 128;
  const int per = n > 2 ? params[2] : 0;
  return batch_set_shape(B, seg, thr, per);
}

extern "C" int kb_batch_get_tuning(kb_batch_t* B, int32_t* params, int32_t n) {
  if (!B || !params) return bfail(KB_ERR_ARG, "kb_batch_get_tuning: null argument");
  const int32_t v[3] = {B->seg, B->seg_t, B->persist};
  for (int k = 0; k < n && k < 3; ++k) params[k] = v[k];
  return KB_OK;
}

extern "C" int kb_batch_info(kb_batch_t* B, int64_t* elems, int64_t* launches) {
  if (!B) return bfail(KB_ERR_ARG, "kb_batch_info: null handle");
  if (elems) *elems = B->nelem;
  if (launches) *launches = B->launches;
  return KB_OK;
}

// ----------------------------------------------------------------- pool
// Continuous batching of 1D2F1V solves: a pool of instance slots with
// capacity fixed at creation; a request joins between steps (kb_pool_add
// places it in free cell / element / velocity ranges, builds its equilibrium
// state on the device and computes its time step) and leaves between steps
// (kb_pool_remove frees its ranges); kb_batch_step advances every resident
// instance with the same fused launch per step.  Only the segment tables and
// the per-slot scalars change on a join or leave (small host-to-device
// copies); the step graph is re-captured at the next step.

static long range_alloc(std::map<long, long>& fr, long n) {
  for (auto it = fr.begin(); it != fr.end(); ++it) {
    if (it->second >= n) {
      const long off = it->first, len = it->second;
      fr.erase(it);
      if (len > n) fr[off + n] = len - n;
      return off;
    }
  }
  return -1;
}

static void range_free(std::map<long, long>& fr, long off, long n) {
  auto it = fr.emplace(off, n).first;
  auto nx = std::next(it);
  if (nx != fr.end() && it->first + it->second == nx->first) {
    it->second += nx->second;
    fr.erase(nx);
  }
  if (it != fr.begin()) {
    auto pv = std::prev(it);
    if (pv->first + pv->second == it->first) {
      pv->second += it->second;
      fr.erase(it);
    }
  }
}

extern "C" int kb_pool_create(const kb_config_t* base, int32_t max_instances, int64_t max_cells,
                              int32_t max_nu, kb_batch_t** out) {
  if (!base || !out || max_instances < 1 || max_cells < 3 * (int64_t)max_instances || max_nu < 1)
    return bfail(KB_ERR_ARG, "kb_pool_create: null argument or empty capacity");
  if (base->dim != 1 || base->nf == 1) return bfail(KB_ERR_CONFIG, "pooled solves are 1D2F1V");
  if (base->precision != KB_PREC_FP32) return bfail(KB_ERR_CONFIG, "pooled solves use the FP32 split form");
  if (base->flux != KB_FLUX_KFVS) return bfail(KB_ERR_CONFIG, "pooled solves use KFVS");
  if (base->bc[0] != KB_BC_FIX || base->bc[1] != KB_BC_FIX)
    return bfail(KB_ERR_CONFIG, "pooled solves use fixed boundaries");
  if (max_nu > kb::SEG_MAXNU) return bfail(KB_ERR_CONFIG, "pooled solves have at most 256 velocities");
  // placeholder instances of max_nu velocities and max_cells cells in all
  // size the arrays (cells x max_nu distribution values, n x max_nu
  // velocities); their slots are then released
  const int n = max_instances;
  std::vector<int32_t> nx(n, 3), ng(n, 0), nu(n, max_nu);
  nx[0] = (int32_t)(max_cells - 3 * (int64_t)(n - 1));
  std::vector<double> x0(n, 0.0), x1(n, 1.0), um(n, 1.0), mu(n, base->mu_ref);
  std::vector<double> uu((size_t)n * max_nu, 0.0), ww((size_t)n * max_nu, 1.0);
  kb_config_t c = *base;
  c.nu = max_nu;
  kb_batch_t* B = nullptr;
  int rc = kb_batch_create(&c, n, nx.data(), ng.data(), nu.data(), x0.data(), x1.data(),
                           um.data(), mu.data(), uu.data(), ww.data(), &B);
  if (rc != KB_OK) return rc;
  B->pool = true;
  B->used.assign(n, 0);
  B->free_cells[0] = B->ncell;
  B->free_elems[0] = B->nelem;
  B->free_vels[0] = B->nvel;
  B->vel_off_h.assign(n, 0);
  std::vector<int> zeros(n, 0);
  cudaMemcpy((void*)B->d.active, zeros.data(), sizeof(int) * n, cudaMemcpyHostToDevice);
  for (int b = 0; b < n; ++b) B->nx[b] = 0;
  rc = batch_set_shape(B, 16, 128, 1);
  if (rc != KB_OK) {
    kb_batch_destroy(B);
    return rc;
  }
  *out = B;
  return KB_OK;
}

template <typename T>
static bool put1(const T* dev, int b, T v) {
  return cudaMemcpy((void*)(dev + b), &v, sizeof(T), cudaMemcpyHostToDevice) == cudaSuccess;
}

extern "C" int kb_pool_add(kb_batch_t* B, int32_t nx, int32_t ngx, int32_t nu, double x0, double x1,
                           double umax, double mu_ref, const double* u, const double* wts,
                           const double* w, const double* prim, double cfl, int32_t* slot,
                           double* dt_out) {
  if (!B || !B->pool || !u || !wts || !w || !prim || !slot) return bfail(KB_ERR_ARG, "kb_pool_add: null argument");
  if (nx < 3 || ngx < 0 || ngx > 2 || nu < 1 || nu > (int)B->d.nu4_max || !(x1 > x0) || !(cfl > 0.0))
    return bfail(KB_ERR_CONFIG, "kb_pool_add: invalid instance");
  int b = -1;
  for (int k = 0; k < B->n && b < 0; ++k)
    if (!B->used[k]) b = k;
  if (b < 0) return bfail(KB_ERR_NOMEM, "kb_pool_add: no free slot");
  const long nxt = nx + 2 * ngx, nus = (nu + 3) / 4 * 4;
  const long co = range_alloc(B->free_cells, nxt);
  const long eo = co < 0 ? -1 : range_alloc(B->free_elems, nxt * nus);
  const long vo = eo < 0 ? -1 : range_alloc(B->free_vels, nu);
  if (vo < 0) {
    if (eo >= 0) range_free(B->free_elems, eo, nxt * nus);
    if (co >= 0) range_free(B->free_cells, co, nxt);
    return bfail(KB_ERR_NOMEM, "kb_pool_add: the pool's cell or velocity capacity is used up");
  }
  cudaStreamSynchronize(B->stream);
  B->used[b] = 1;
  B->nx[b] = nx;
  B->ng[b] = ngx;
  B->nu[b] = nu;
  B->nus[b] = (int)nus;
  B->cell_off[b] = co;
  B->elem_off[b] = eo;
  B->vel_off_h[b] = vo;
  const double dx = (x1 - x0) / nx;
  bool ok = put1(B->d.nx, b, (int)nx) && put1(B->d.ng, b, (int)ngx) && put1(B->d.nu, b, (int)nu) &&
            put1(B->d.nus, b, (int)nus) && put1(B->d.cell_off, b, co) && put1(B->d.elem_off, b, eo) &&
            put1(B->d.vel_off, b, (int)vo) && put1(B->d.dx, b, dx) && put1(B->d.mu, b, mu_ref) &&
            put1((const double*)B->d_umax, b, umax);
  std::vector<float> uf(nu), ul(nu), wf(nu);
  for (int k = 0; k < nu; ++k) {
    uf[k] = float(u[k]);
    ul[k] = float(u[k] - (double)uf[k]);
    wf[k] = float(wts[k]);
  }
  ok &= cudaMemcpy((void*)(B->d.u + vo), u, sizeof(double) * nu, cudaMemcpyHostToDevice) == cudaSuccess;
  ok &= cudaMemcpy((void*)(B->d.wt + vo), wts, sizeof(double) * nu, cudaMemcpyHostToDevice) == cudaSuccess;
  ok &= cudaMemcpy((void*)(B->d.uf + vo), uf.data(), sizeof(float) * nu, cudaMemcpyHostToDevice) == cudaSuccess;
  ok &= cudaMemcpy((void*)(B->d.ul + vo), ul.data(), sizeof(float) * nu, cudaMemcpyHostToDevice) == cudaSuccess;
  ok &= cudaMemcpy((void*)(B->d.wtf + vo), wf.data(), sizeof(float) * nu, cudaMemcpyHostToDevice) == cudaSuccess;
  std::vector<double> w4(nxt * 4, 0.0), p4(nxt * 4, 0.0);
  for (long c = 0; c < nxt; ++c)
    for (int k = 0; k < 3; ++k) {
      w4[c * 4 + k] = w[c * 3 + k];
      p4[c * 4 + k] = prim[c * 3 + k];
    }
  ok &= cudaMemcpy(B->d.w + co * 4, w4.data(), sizeof(double) * w4.size(), cudaMemcpyHostToDevice) == cudaSuccess;
  ok &= cudaMemcpy(B->d.prim + co * 4, p4.data(), sizeof(double) * p4.size(), cudaMemcpyHostToDevice) == cudaSuccess;
  if (!ok) return bfail(KB_ERR_CUDA, "kb_pool_add: copy failed");
  kb::k_batch_init_eq32<<<dim3((unsigned)nxt, 1), 128, 0, B->stream>>>(
      B->d, b, (float*)B->h[0], (float*)B->bq[0], (float*)B->h[1], (float*)B->bq[1]);
  kb::k_batch_timestep<<<1, 256, 0, B->stream>>>(B->d, B->d_umax, cfl, (double*)B->d.dt, b);
  B->launches += 2;
  double dt = 0.0;
  ok &= cudaStreamSynchronize(B->stream) == cudaSuccess;
  ok &= cudaMemcpy(&dt, B->d.dt + b, sizeof(double), cudaMemcpyDeviceToHost) == cudaSuccess;
  ok &= put1((const int*)B->d.active, b, 1);
  const double zero4[4] = {0, 0, 0, 0};
  ok &= cudaMemcpy(B->d.residual + (long)b * 4, zero4, sizeof(zero4), cudaMemcpyHostToDevice) == cudaSuccess;
  if (!ok) {
    cudaGetLastError();
    return bfail(KB_ERR_CUDA, "kb_pool_add: device set-up failed");
  }
  int rc = batch_set_shape(B, B->seg, B->seg_t, B->persist);
  if (rc != KB_OK) return rc;
  *slot = b;
  if (dt_out) *dt_out = dt;
  return KB_OK;
}

extern "C" int kb_pool_remove(kb_batch_t* B, int32_t slot) {
  if (!B || !B->pool || slot < 0 || slot >= B->n || !B->used[slot])
    return bfail(KB_ERR_ARG, "kb_pool_remove: no such slot");
  cudaStreamSynchronize(B->stream);
  const long nxt = B->nx[slot] + 2 * B->ng[slot];
  range_free(B->free_cells, B->cell_off[slot], nxt);
  range_free(B->free_elems, B->elem_off[slot], nxt * B->nus[slot]);
  range_free(B->free_vels, B->vel_off_h[slot], B->nu[slot]);
  B->used[slot] = 0;
  B->nx[slot] = 0;
  if (!put1((const int*)B->d.active, slot, 0)) return bfail(KB_ERR_CUDA, "kb_pool_remove: copy failed");
  return batch_set_shape(B, B->seg, B->seg_t, B->persist);
}

extern "C" int kb_pool_download(kb_batch_t* B, int32_t slot, double* w, double* prim, double* h,
                                double* bq) {
  if (!B || !B->pool || slot < 0 || slot >= B->n || !B->used[slot])
    return bfail(KB_ERR_ARG, "kb_pool_download: no such slot");
  cudaStreamSynchronize(B->stream);
  const long nxt = B->nx[slot] + 2 * B->ng[slot], co = B->cell_off[slot];
  const int nu = B->nu[slot], nus = B->nus[slot];
  bool ok = true;
  if (w || prim) {
    std::vector<double> a4(nxt * 4);
    for (int which = 0; which < 2; ++which) {
      double* dst = which == 0 ? w : prim;
      if (!dst) continue;
      ok &= cudaMemcpy(a4.data(), (which == 0 ? B->d.w : B->d.prim) + co * 4, sizeof(double) * a4.size(),
                       cudaMemcpyDeviceToHost) == cudaSuccess;
      for (long c = 0; c < nxt; ++c)
        for (int k = 0; k < 3; ++k) dst[c * 3 + k] = a4[c * 4 + k];
    }
  }
  const long ne = nxt * nus, eo = B->elem_off[slot];
  std::vector<double> stage(ne);
  for (int which = 0; which < 2; ++which) {
    double* dst = which == 0 ? h : bq;
    if (!dst) continue;
    const float* src = (const float*)(which == 0 ? B->h[B->cur] : B->bq[B->cur]) + eo;
    kb::k_batch_back<float><<<(unsigned)((ne + 255) / 256), 256, 0, B->stream>>>(B->d_stage, src, ne);
    B->launches++;
    ok &= cudaStreamSynchronize(B->stream) == cudaSuccess;
    ok &= cudaMemcpy(stage.data(), B->d_stage, sizeof(double) * ne, cudaMemcpyDeviceToHost) == cudaSuccess;
    for (long c = 0; c < nxt; ++c) std::memcpy(dst + c * nu, &stage[c * nus], sizeof(double) * nu);
  }
  if (!ok) return bfail(KB_ERR_CUDA, "kb_pool_download: copy failed");
  return KB_OK;
}
