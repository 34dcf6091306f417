// kb_march.cuh -- the two HBM passes of one DVM time step (kernel templates;
// instantiated per precision and flux in kb_march_*.cu so they compile in parallel).
//
// Pass A (k_mom): fw of every interior face and the old heat flux q of every
// cell.  A warp owns a line segment of TS faces (along x or y) and loops over
// ALL velocities, lanes striding by 32; the cells of the segment stencil are
// held in a register window, so each cell value is loaded once per segment
// and each van Leer slope is formed once.  Per-lane partial sums are
// compensated (FP32 blocks flushed into double-float accumulators on the FP32
// path) and combined once per face by a fixed shuffle tree, so fw is
// deterministic and each face has exactly one writer.
//
// Pass B (k_march): the pointwise update of h and b.  A thread owns one
// velocity; a CTA owns a strip of TX columns, a chunk of rows and a chunk of
// velocities and marches up the rows with a four-row register window.  Every
// x-face and y-face flux is evaluated once per velocity and added to both
// neighbouring cells, so h and b are read once (plus a 4-cell x halo per row)
// and written once.
#pragma once

#include <cuda.h>
#include <cuda_runtime.h>

#include <mutex>
#include <type_traits>

#include "kb_kernels.cuh"
#include "kb_flux.cuh"
#include "kb_tma.cuh"

namespace kb {

// van Leer slope times dx, from raw differences: dx * vanleer(a/dx, b/dx)
// = (a|b| + b|a|) / (|a| + |b| + 1e-7 dx) (src/Reconstruction/recon_limiter.jl:17-19);
// rules 2 / 3 are the one-sided reconstruct2! differences.
// x / y as one reciprocal and one multiply, subnormal inputs and results
// flushed to zero (the non-flushing form adds range fix-ups to every call).
__device__ __forceinline__ float fdiv_ftz(float x, float y) {
  float r;
  asm("div.approx.ftz.f32 %0, %1, %2;" : "=f"(r) : "f"(x), "f"(y));
  return r;
}
__device__ __forceinline__ float vl_diff(int rule, float qm, float q0, float qp, float epsd) {
  float a = q0 - qm, b = qp - q0;
  if (rule == 1) return fdiv_ftz(a * fabsf(b) + b * fabsf(a), fabsf(a) + fabsf(b) + epsd);
  if (rule == 2) return b;
  if (rule == 3) return a;
  return 0.f;
}
__device__ __forceinline__ double vl_diff(int rule, double qm, double q0, double qp, double epsd) {
  double a = q0 - qm, b = qp - q0;
  if (rule == 1) return (a * fabs(b) + b * fabs(a)) / (fabs(a) + fabs(b) + epsd);
  if (rule == 2) return b;
  if (rule == 3) return a;
  return 0.0;
}

// 2^x on the MUFU unit (flushes results below 2^-126 to zero).
__device__ __forceinline__ float ex2(float x) {
  float y;
  asm("ex2.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
  return y;
}

// Rule-dispatching slope; FAST = interior cell (van Leer only).
template <bool FAST, typename R>
__device__ __forceinline__ R slope(int rule, R qm, R q0, R qp, R epsd) {
  if (FAST) return vl_diff(1, qm, q0, qp, epsd);
  return vl_diff(rule, qm, q0, qp, epsd);
}

template <typename R>
__device__ __forceinline__ R ldq(const R* __restrict__ q, long idx, bool ok) {
  return ok ? __ldg(q + idx) : R(0);
}

// Blocked compensated accumulator: plain partial sums, flushed into a
// double-float (TwoSum) accumulator; FP64 path sums in double directly.
template <typename R>
struct BAcc;
template <>
struct BAcc<float> {
  float p;
  DF d;
  __device__ __forceinline__ void init() { p = 0.f; d.hi = 0.f; d.lo = 0.f; }
  __device__ __forceinline__ void add(float x) { p += x; }
  __device__ __forceinline__ void flush() { df_add(d, p); p = 0.f; }
  __device__ __forceinline__ double total() { flush(); return df_warp_sum(d); }
};
template <>
struct BAcc<double> {
  double p;
  __device__ __forceinline__ void init() { p = 0.0; }
  __device__ __forceinline__ void add(double x) { p += x; }
  __device__ __forceinline__ void flush() {}
  __device__ __forceinline__ double total() { return warp_sum(p); }
};

// ------------------------------------------------------------------ pass A

// DIR 0: x faces, segments along x in each row; DIR 1: y faces, segments
// along y in each column.  Face f of a segment sits between cells p-1 and p
// along the line with p = p0 + f; cells p0-2 .. p0+TS+1 form the window.
template <typename R, int D, int FLUX, int TS, bool SHAK, int DIR>
__global__ void __launch_bounds__(128) k_mom(DevState s) {
  const Geo& g = s.g;
  const int lane = threadIdx.x & 31;
  const int gw = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int n = DIR == 0 ? g.nx : g.ny;          // cells along the line
  const int ng = DIR == 0 ? g.ngx : g.ngy;
  const int nlines = DIR == 0 ? g.ny : g.nx;
  const int nseg = (n + TS - 1) / TS;
  if (gw >= nseg * nlines) return;
  const int line = gw / nseg, sg = gw - line * nseg;
  const int p0 = sg * TS;
  const int ncell = min(TS, n - p0);
  const int nf = ncell + (sg == nseg - 1 ? 1 : 0);  // faces p0 .. p0+nf-1
  const long vs = g.vstride;
  const R* __restrict__ H = (const R*)s.h[s.cur];
  const R* __restrict__ Bq = (const R*)s.b[s.cur];
  const R* __restrict__ U = vtab<R>(s, 0);
  const R* __restrict__ V = vtab<R>(s, 1);
  const R* __restrict__ W = vtab<R>(s, 2);
  const double dd = DIR == 0 ? g.dx : g.dy;
  const R epsd = R(1.e-7 * dd);

  long base[TS + 4];
  bool ex[TS + 4];
  int rule[TS + 4];
#pragma unroll
  for (int w = 0; w < TS + 4; ++w) {
    int p = p0 - 2 + w;
    ex[w] = p >= -ng && p < n + ng;
    int c = DIR == 0 ? cell_index(g, p, line) : cell_index(g, line, p);
    base[w] = ex[w] ? (long)c * vs : 0;
    rule[w] = slope_rule(g, DIR, p);
  }
  int fidx[TS + 1];
  bool act[TS + 1];
  R t3[TS + 1], t4[TS + 1];
#pragma unroll
  for (int f = 0; f < TS + 1; ++f) {
    int p = p0 + f;
    fidx[f] = DIR == 0 ? line * (g.nx + 1) + p : s.nface_x + p * g.nx + line;
    act[f] = f < nf && s.kind[fidx[f]] == 1;
    t3[f] = R(0);
    t4[f] = R(0);
    if (act[f]) {
      const FaceParam& P = s.fp[fidx[f]];
      t3[f] = R(P.tr[0]);
      t4[f] = R(P.tr[1] / dd);
    }
  }
  R oU[TS], oV[TS];
  if (SHAK) {
#pragma unroll
    for (int c = 0; c < TS; ++c) {
      int cc = base[c + 2] / vs;
      oU[c] = R(s.prim[(long)cc * 4 + 1]);
      oV[c] = R(D == 2 ? s.prim[(long)cc * 4 + 2] : 0.0);
    }
  }
  BAcc<R> acc[TS + 1][4];
  BAcc<R> qa[SHAK ? TS : 1][2];
#pragma unroll
  for (int f = 0; f < TS + 1; ++f)
#pragma unroll
    for (int k = 0; k < 4; ++k) acc[f][k].init();
#pragma unroll
  for (int c = 0; c < (SHAK ? TS : 1); ++c) {
    qa[c][0].init();
    qa[c][1].init();
  }

  auto run = [&](auto fast_tag) {
  constexpr bool FAST = decltype(fast_tag)::value;
  int it = 0;
  for (int v0 = 0; v0 < g.nvel; v0 += 32, ++it) {
    const int v = v0 + lane;
    const bool ok = v < g.nvel;
    R u = ok ? U[v] : R(0);
    R vv = (ok && D == 2) ? V[v] : R(0);
    R om = ok ? W[v] : R(0);
    R un = DIR == 0 ? u : vv;
    R ut = DIR == 0 ? vv : -u;
    R hx[TS + 4], bx[TS + 4];
#pragma unroll
    for (int w = 0; w < TS + 4; ++w) {
      hx[w] = ldq(H, base[w] + v, (FAST || ex[w]) && ok);
      bx[w] = ldq(Bq, base[w] + v, (FAST || ex[w]) && ok);
    }
    R dh[TS + 2], db[TS + 2];  // slopes of cells w = 1 .. TS+2
#pragma unroll
    for (int w = 1; w <= TS + 2; ++w) {
      dh[w - 1] = slope<FAST>(rule[w], hx[w - 1], hx[w], hx[w + 1], epsd);
      db[w - 1] = slope<FAST>(rule[w], bx[w - 1], bx[w], bx[w + 1], epsd);
    }
    const bool pos = un >= R(0);
    const R c2 = un * un + ut * ut;
    const R un2 = un * un;
#pragma unroll
    for (int f = 0; f < TS + 1; ++f) {
      if (FAST ? f == TS : !act[f]) continue;
      R hu = pos ? hx[f + 1] : hx[f + 2];
      R bu = pos ? bx[f + 1] : bx[f + 2];
      R su = pos ? dh[f] : dh[f + 1];
      R sb = pos ? db[f] : db[f + 1];
      R hf = hu + (pos ? R(0.5) : R(-0.5)) * su;
      R bf = bu + (pos ? R(0.5) : R(-0.5)) * sb;
      R Th = t3[f] * un * hf - t4[f] * un2 * su;
      R Tb = t3[f] * un * bf - t4[f] * un2 * sb;
      R wT = om * Th;
      acc[f][0].add(wT);
      acc[f][1].add(wT * un);
      if (D == 2) acc[f][2].add(wT * ut);
      acc[f][3].add(wT * c2 + om * Tb);
    }
    if (SHAK) {
#pragma unroll
      for (int c = 0; c < TS; ++c) {
        R cu = u - oU[c];
        R cv = vv - oV[c];
        R c2o = cu * cu + cv * cv;
        R hc = hx[c + 2], bc = bx[c + 2];
        qa[c][0].add(om * cu * c2o * hc + om * cu * bc);
        if (D == 2) qa[c][1].add(om * cv * c2o * hc + om * cv * bc);
      }
    }
    if ((it & 3) == 3) {
#pragma unroll
      for (int f = 0; f < TS + 1; ++f)
#pragma unroll
        for (int k = 0; k < 4; ++k) acc[f][k].flush();
#pragma unroll
      for (int c = 0; c < (SHAK ? TS : 1); ++c) {
        qa[c][0].flush();
        qa[c][1].flush();
      }
    }
  }
  };
  bool fast = g.interp == 2 && p0 >= 2 && p0 + TS <= n - 2 && nf == TS;
#pragma unroll
  for (int f = 0; f < TS; ++f) fast = fast && act[f];
  if (fast) run(std::true_type{});
  else run(std::false_type{});
#pragma unroll
  for (int f = 0; f < TS + 1; ++f) {
    if (!act[f]) continue;
    double S0 = acc[f][0].total(), S1 = acc[f][1].total();
    double S2 = D == 2 ? acc[f][2].total() : 0.0;
    double S3 = acc[f][3].total();
    if (lane == 0) {
      const FaceParam& P = s.fp[fidx[f]];
      double fl[4];
      fl[0] = P.fwa[0] + S0;
      fl[1] = P.fwa[1] + S1;
      if (D == 1) {
        fl[2] = P.fwa[2] + 0.5 * S3;
        fl[3] = 0.0;
      } else {
        fl[2] = P.fwa[2] + S2;
        fl[3] = P.fwa[3] + 0.5 * S3;
      }
      double* out = s.fw + (long)fidx[f] * 4;
      if (DIR == 1) {  // global_frame with n = (0, 1)
        out[0] = fl[0];
        out[1] = -fl[2];
        out[2] = fl[1];
        out[3] = fl[3];
      } else {
        out[0] = fl[0];
        out[1] = fl[1];
        out[2] = fl[2];
        out[3] = fl[3];
      }
    }
  }
  if (SHAK) {
#pragma unroll
    for (int c = 0; c < TS; ++c) {
      double q0 = qa[c][0].total();
      double q1 = D == 2 ? qa[c][1].total() : 0.0;
      if (lane == 0 && c < ncell) {
        long cc = base[c + 2] / vs;
        s.q[cc * 2 + 0] = 0.5 * q0;
        s.q[cc * 2 + 1] = 0.5 * q1;
      }
    }
  }
}

// Pass A, FP32 form: the stencil window of a CTA segment (4 warps x TS faces
// along one line) is streamed through shared memory in chunks of MOM_VC
// velocities, MOM_P chunks in flight: one TMA tensor box per distribution
// (velocities x window cells of the line; cells outside the grid read as
// zero) plus three bulk copies of the velocity tables per chunk, so the DRAM
// latency is covered by the copies already issued instead of by registers.
// A fifth (producer) warp issues the copies; each consumer warp reads its
// TS+4 window cells from shared memory, lanes over velocities, and releases a
// stage through its own mbarrier arrival, so consumer warps never wait on
// one another.
constexpr int MOM_VC = KB_TMA_VBOX;  // velocities per staged chunk (one TMA box)
constexpr int MOM_P = 3;     // chunks in flight
template <int TS>
struct MomStage {
  static constexpr int NF = 4 * TS;     // faces per CTA segment
  static constexpr int NWIN = NF + 4;   // window cells p0-2 .. p0+NF+1
  static constexpr int BOX = NWIN * MOM_VC;                // one distribution: [cell][v]
  static constexpr int FLOATS = 2 * BOX + 3 * MOM_VC;      // h box, b box, then u, v, w
  // stages, then full[MOM_P], empty[MOM_P] mbarriers and a failure flag
  static constexpr int BYTES = MOM_P * FLOATS * 4 + 16 * MOM_P + 16;
};
constexpr int MOM_THREADS = 160;  // 4 consumer warps + 1 producer warp

template <int D, int FLUX, int TS, bool SHAK, int DIR, bool GRP = false>
__global__ void __launch_bounds__(MOM_THREADS) k_mom_st(const __grid_constant__ CUtensorMap tmh,
                                                        const __grid_constant__ CUtensorMap tmb,
                                                        DevState sp) {
  using R = float;
  int lb;
  const int gr = group_member<GRP, DIR == 0 ? GK_MOMX : GK_MOMY>(sp, lb);
  KB_GROUP_STATE(GRP, sp, gr);
  // a grouped launch reads each member's tensor maps from global memory
  const CUtensorMap* mh = GRP ? sp.grp->maps + gr * 6 + DIR * 2 : &tmh;
  const CUtensorMap* mb = GRP ? sp.grp->maps + gr * 6 + DIR * 2 + 1 : &tmb;
  if (GRP && threadIdx.x == 4 * 32) {  // the producer warp's issuing lane
    tmap_acquire(mh);
    tmap_acquire(mb);
  }
  using SL = MomStage<TS>;
  extern __shared__ __align__(1024) unsigned char smemA[];
  float* stg = (float*)smemA;
  unsigned long long* full = (unsigned long long*)(smemA + MOM_P * SL::FLOATS * 4);
  unsigned long long* empty = full + MOM_P;
  int* bad = (int*)(empty + MOM_P);
  constexpr int PRODUCER = 4;
  const Geo& g = s.g;
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  const int n = DIR == 0 ? g.nx : g.ny;  // cells along the line
  const int ng = DIR == 0 ? g.ngx : g.ngy;
  const int nseg = (n + SL::NF - 1) / SL::NF;
  const int line = lb / nseg, sgi = lb - line * nseg;
  const int p0 = sgi * SL::NF;      // first face of the CTA segment
  const int p0w = p0 + wid * TS;    // first face of this warp
  const int ncell = wid == PRODUCER ? 0 : max(0, min(TS, n - p0w));
  const int nf = ncell > 0 ? ncell + (p0w + ncell == n ? 1 : 0) : 0;  // faces p0w .. p0w+nf-1
  const int vs = g.vstride;
  const double dd = DIR == 0 ? g.dx : g.dy;
  const R epsd = R(1.e-7 * dd);
  const int nchunk = (g.nvel + MOM_VC - 1) / MOM_VC;

  // window cell w of the CTA (p = p0 - 2 + w): existence and cell index
  auto win_cell = [&](int w, bool& e) {
    const int p = p0 - 2 + w;
    e = p >= -ng && p < n + ng;
    return DIR == 0 ? cell_index(g, p, line) : cell_index(g, line, p);
  };
  if (threadIdx.x == 0) {
    for (int k = 0; k < MOM_P; ++k) {
      mbar_init(&full[k], 1);
      mbar_init(&empty[k], PRODUCER);
    }
    *bad = 0;
  }
  fence_async_smem();
  __syncthreads();

  // tensor coordinates (velocity, column, row) of the window's first cell
  const int cx = DIR == 0 ? p0 - 2 + g.ngx : line + g.ngx;
  const int cy = DIR == 0 ? line + g.ngy : p0 - 2 + g.ngy;
  auto issue = [&](int k) {  // producer lane 0: chunk k into stage k % MOM_P
    float* S = stg + (k % MOM_P) * SL::FLOATS;
    unsigned long long* bar = &full[k % MOM_P];
    const int v0 = k * MOM_VC;
    const unsigned cb = (unsigned)min(MOM_VC, vs - v0) * 4u;  // a multiple of 16
    if (lane == 0) {
      mbar_expect(bar, 2u * SL::BOX * 4u + 3u * cb);
      tma_load_3d(S, mh, v0, cx, cy, bar);
      tma_load_3d(S + SL::BOX, mb, v0, cx, cy, bar);
      for (int t = 0; t < 3; ++t) bulk_g2s(S + 2 * SL::BOX + t * MOM_VC, vtab<R>(s, t) + v0, cb, bar);
    }
    __syncwarp();
  };

  // this warp's faces and window (wl = 0 .. TS+3 <-> CTA window cell wid*TS + wl)
  int rule[TS + 4];
#pragma unroll
  for (int w = 0; w < TS + 4; ++w) rule[w] = slope_rule(g, DIR, p0w - 2 + w);
  int fidx[TS + 1];
  bool act[TS + 1];
  R t3[TS + 1], t4[TS + 1];
#pragma unroll
  for (int f = 0; f < TS + 1; ++f) {
    int p = p0w + f;
    fidx[f] = DIR == 0 ? line * (g.nx + 1) + p : s.nface_x + p * g.nx + line;
    act[f] = f < nf && s.kind[fidx[f]] == 1;
    t3[f] = R(0);
    t4[f] = R(0);
    if (act[f]) {
      const FaceParam& P = s.fp[fidx[f]];
      t3[f] = R(P.tr[0]);
      t4[f] = R(P.tr[1] / dd);
    }
  }
  R oU[TS], oV[TS];
  if (SHAK) {
#pragma unroll
    for (int c = 0; c < TS; ++c) {
      bool e;
      const int cc = win_cell(wid * TS + c + 2, e);
      oU[c] = e ? R(s.prim[(long)cc * 4 + 1]) : R(0);
      oV[c] = (e && D == 2) ? R(s.prim[(long)cc * 4 + 2]) : R(0);
    }
  }
  BAcc<R> acc[TS + 1][4];
  BAcc<R> qa[SHAK ? TS : 1][2];
#pragma unroll
  for (int f = 0; f < TS + 1; ++f)
#pragma unroll
    for (int k = 0; k < 4; ++k) acc[f][k].init();
#pragma unroll
  for (int c = 0; c < (SHAK ? TS : 1); ++c) {
    qa[c][0].init();
    qa[c][1].init();
  }

  bool fast = g.interp == 2 && p0w >= 2 && p0w + TS <= n - 2 && nf == TS;
#pragma unroll
  for (int f = 0; f < TS; ++f) fast = fast && act[f];
  // One velocity of this warp's faces.  SG 0: upwind side per lane; SG 1 / 2:
  // every lane of the warp has un >= 0 / un < 0, so only the upwind cells'
  // slopes are formed and only the window cells they touch are read.
  auto one = [&](const float* S, const float* Sw, int vl, auto fast_tag, auto sign_tag) {
    constexpr bool FAST = decltype(fast_tag)::value;
    constexpr int SG = decltype(sign_tag)::value;
    const R u = S[2 * SL::BOX + vl];
    const R vv = D == 2 ? S[2 * SL::BOX + MOM_VC + vl] : R(0);
    const R om = S[2 * SL::BOX + 2 * MOM_VC + vl];
    const R un = DIR == 0 ? u : vv;
    const R ut = DIR == 0 ? vv : -u;
    constexpr int WLO = SG == 2 ? 1 : 0, WHI = SG == 1 ? TS + 1 : (SG == 2 ? TS + 2 : TS + 3);
    R hx[TS + 4], bx[TS + 4];
#pragma unroll
    for (int w = WLO; w <= WHI; ++w) {
      hx[w] = Sw[w * MOM_VC + vl];
      bx[w] = Sw[SL::BOX + w * MOM_VC + vl];
    }
    const bool pos = SG == 0 ? un >= R(0) : SG == 1;
    const R c2 = un * un + ut * ut;
    const R un2 = un * un;
#pragma unroll
    for (int f = 0; f < TS + 1; ++f) {
      if (FAST ? f == TS : !act[f]) continue;
      R hu, bu, su, sb;
      if (SG == 1 || (SG == 0 && FAST)) {
        // upwind cell w = f + 1 (pos) or f + 2 (neg), its slope from three values
        const int w = SG == 1 ? f + 1 : f + 2;
        if (SG == 1) {
          hu = hx[w];
          bu = bx[w];
          su = slope<FAST>(rule[w], hx[w - 1], hx[w], hx[w + 1], epsd);
          sb = slope<FAST>(rule[w], bx[w - 1], bx[w], bx[w + 1], epsd);
        } else {
          const R hm = pos ? hx[f] : hx[f + 1], h0 = pos ? hx[f + 1] : hx[f + 2],
                  hp = pos ? hx[f + 2] : hx[f + 3];
          const R bm = pos ? bx[f] : bx[f + 1], b0 = pos ? bx[f + 1] : bx[f + 2],
                  bp = pos ? bx[f + 2] : bx[f + 3];
          hu = h0;
          bu = b0;
          su = slope<FAST>(1, hm, h0, hp, epsd);
          sb = slope<FAST>(1, bm, b0, bp, epsd);
        }
      } else if (SG == 2) {
        const int w = f + 2;
        hu = hx[w];
        bu = bx[w];
        su = slope<FAST>(rule[w], hx[w - 1], hx[w], hx[w + 1], epsd);
        sb = slope<FAST>(rule[w], bx[w - 1], bx[w], bx[w + 1], epsd);
      } else {
        // boundary segment, mixed signs: both candidate cells' rules apply
        const int wl = f + 1, wr = f + 2;
        const R sl = slope<FAST>(rule[wl], hx[wl - 1], hx[wl], hx[wl + 1], epsd);
        const R sr = slope<FAST>(rule[wr], hx[wr - 1], hx[wr], hx[wr + 1], epsd);
        const R tl = slope<FAST>(rule[wl], bx[wl - 1], bx[wl], bx[wl + 1], epsd);
        const R tr = slope<FAST>(rule[wr], bx[wr - 1], bx[wr], bx[wr + 1], epsd);
        hu = pos ? hx[wl] : hx[wr];
        bu = pos ? bx[wl] : bx[wr];
        su = pos ? sl : sr;
        sb = pos ? tl : tr;
      }
      R hf = hu + (pos ? R(0.5) : R(-0.5)) * su;
      R bf = bu + (pos ? R(0.5) : R(-0.5)) * sb;
      R Th = t3[f] * un * hf - t4[f] * un2 * su;
      R Tb = t3[f] * un * bf - t4[f] * un2 * sb;
      R wT = om * Th;
      acc[f][0].add(wT);
      acc[f][1].add(wT * un);
      if (D == 2) acc[f][2].add(wT * ut);
      acc[f][3].add(wT * c2 + om * Tb);
    }
    if (SHAK) {
#pragma unroll
      for (int c = 0; c < TS; ++c) {
        R cu = u - oU[c];
        R cv = vv - oV[c];
        R c2o = cu * cu + cv * cv;
        R hc = hx[c + 2], bc = bx[c + 2];
        qa[c][0].add(om * cu * c2o * hc + om * cu * bc);
        if (D == 2) qa[c][1].add(om * cv * c2o * hc + om * cv * bc);
      }
    }
  };
  // one staged chunk of this warp's faces (FAST: interior van Leer window)
  auto body = [&](const float* S, int k, auto fast_tag) {
    constexpr bool FAST = decltype(fast_tag)::value;
    using I0 = std::integral_constant<int, 0>;
    const float* Sw = S + wid * TS * MOM_VC;  // this warp's window cell 0 (h; b at + BOX)
    // iterations holding at least one velocity: the same count on every lane,
    // so the whole warp reaches each ballot
    const int mmax = min(MOM_VC / 32, (g.nvel - k * MOM_VC + 31) / 32);
#pragma unroll
    for (int m = 0; m < MOM_VC / 32; ++m) {
      if (m >= mmax) break;
      const int vl = m * 32 + lane;
      const bool valid = k * MOM_VC + vl < g.nvel;
      if (FAST) {
        const R un = S[2 * SL::BOX + (DIR == 0 ? 0 : MOM_VC) + vl];
        const unsigned ap = __ballot_sync(0xffffffffu, !valid || un >= R(0));
        const unsigned an = __ballot_sync(0xffffffffu, !valid || un < R(0));
        if (valid) {
          if (ap == 0xffffffffu) one(S, Sw, vl, fast_tag, std::integral_constant<int, 1>{});
          else if (an == 0xffffffffu) one(S, Sw, vl, fast_tag, std::integral_constant<int, 2>{});
          else one(S, Sw, vl, fast_tag, I0{});
        }
      } else if (valid) {
        one(S, Sw, vl, fast_tag, I0{});
      }
    }
    // flush the FP32 partials (16 velocities per lane) into the compensated
    // sums; the interior form never touches the segment's last face
    if ((k & 3) == 3) {
#pragma unroll
      for (int f = 0; f < (FAST ? TS : TS + 1); ++f)
#pragma unroll
        for (int q = 0; q < 4; ++q) acc[f][q].flush();
#pragma unroll
      for (int c = 0; c < (SHAK ? TS : 1); ++c) {
        qa[c][0].flush();
        qa[c][1].flush();
      }
    }
  };
  volatile int* vbad = bad;
  if (wid == PRODUCER) {
    for (int k = 0; k < nchunk; ++k) {
      if (k >= MOM_P) {
        // stage k % MOM_P is free once all consumer warps released chunk k - MOM_P
        int ok = 1, stop = 0;
        if (lane == 0) {
          ok = mbar_wait(&empty[k % MOM_P], ((k / MOM_P) - 1) & 1);
          stop = *vbad;
        }
        ok = __shfl_sync(0xffffffffu, ok, 0);  // one decision for the whole warp
        stop = __shfl_sync(0xffffffffu, stop, 0);
        if (!ok || stop) {  // stop issuing: consumers then skip their waits
          if (lane == 0 && !ok) {
            atomicOr(bad, 1);
            atomicOr(s.status, 2);
          }
          break;
        }
        if (lane == 0) fence_async_smem();
        __syncwarp();
      }
      issue(k);
    }
  } else {
    for (int k = 0; k < nchunk; ++k) {
      bool ok = *vbad == 0;
      if (ok) {
        ok = mbar_wait(&full[k % MOM_P], (k / MOM_P) & 1);
        if (!ok) {
          atomicOr(bad, 1);
          atomicOr(s.status, 2);
        }
      }
      ok = __all_sync(0xffffffffu, ok);
      const float* S = stg + (k % MOM_P) * SL::FLOATS;
      if (ok && nf > 0) {
        if (fast) body(S, k, std::true_type{});
        else body(S, k, std::false_type{});
      }
      __syncwarp();
      if (lane == 0) mbar_arrive(&empty[k % MOM_P]);
    }
  }
  __syncthreads();
  if (*vbad) {
    // copies of the last chunks issued may still land: wait (bounded) for
    // each stage's latest phase before the shared memory is released
    if (threadIdx.x == 0)
      for (int k = max(0, nchunk - MOM_P); k < nchunk; ++k)
        mbar_wait(&full[k % MOM_P], (k / MOM_P) & 1);
    return;
  }
#pragma unroll
  for (int f = 0; f < TS + 1; ++f) {
    if (!act[f]) continue;
    double S0 = acc[f][0].total(), S1 = acc[f][1].total();
    double S2 = D == 2 ? acc[f][2].total() : 0.0;
    double S3 = acc[f][3].total();
    if (lane == 0) {
      const FaceParam& P = s.fp[fidx[f]];
      double fl[4];
      fl[0] = P.fwa[0] + S0;
      fl[1] = P.fwa[1] + S1;
      if (D == 1) {
        fl[2] = P.fwa[2] + 0.5 * S3;
        fl[3] = 0.0;
      } else {
        fl[2] = P.fwa[2] + S2;
        fl[3] = P.fwa[3] + 0.5 * S3;
      }
      double* out = s.fw + (long)fidx[f] * 4;
      if (DIR == 1) {  // global_frame with n = (0, 1)
        out[0] = fl[0];
        out[1] = -fl[2];
        out[2] = fl[1];
        out[3] = fl[3];
      } else {
        out[0] = fl[0];
        out[1] = fl[1];
        out[2] = fl[2];
        out[3] = fl[3];
      }
    }
  }
  if (SHAK) {
#pragma unroll
    for (int c = 0; c < TS; ++c) {
      double q0 = qa[c][0].total();
      double q1 = D == 2 ? qa[c][1].total() : 0.0;
      if (lane == 0 && c < ncell) {
        bool e;
        const long cc = win_cell(wid * TS + c + 2, e);
        s.q[cc * 2 + 0] = 0.5 * q0;
        s.q[cc * 2 + 1] = 0.5 * q1;
      }
    }
  }
}

// ------------------------------------------------------------------ pass B

// Per-face evaluation state of one thread (one velocity, static upwind side).
template <typename R>
struct FEv;

// FP32: monomial form of FaceCoef32.
constexpr bool FLUX_NEEDS_G = true;
template <>
struct FEv<float> {
  float4 E, T, G, C, Dd;
  int kind;
  // c: this face's coefficient block (global or staged in shared memory)
  __device__ __forceinline__ void load_interior(const FaceCoef32& c, bool pos) {
    kind = 1;
    E = c.E;
    T = c.T;
    if (FLUX_NEEDS_G) {
      G = c.G;
      const float4* cd = pos ? &c.Cp : &c.Cm;
      C = cd[0];
      Dd = cd[1];
    }
  }
  __device__ __forceinline__ void load(const FaceCoef32& c, int kd, bool pos) {
    kind = kd;
    if (kind == 0) return;
    E = c.E;
    T = c.T;
    if (kind == 1) {
      G = c.G;
      C = pos ? c.Cp : c.Cm;
      Dd = pos ? c.Dp : c.Dm;
    }
  }
};

// FP64: direct formulas of the reference with the interface prim.
template <>
struct FEv<double> {
  FP<double> P;
  double dd;  // cell size along the face normal
  double wU, wV, wlam, wrn, wcB, wsc, rot;
  int kind;
  __device__ __forceinline__ void load(const DevState& s, int f, bool pos) {
    (void)pos;
    kind = s.kind[f];
    if (kind == 0) return;
    const Geo& g = s.g;
    FaceGeo r = face_geo(g, f);
    dd = r.d == 0 ? g.dx : g.dy;
    if (kind == 1) {
      P = load_fp<double>(s, f);
    } else {
      const double* wp = s.wall + (long)f * 4;
      double lw = g.D == 1 ? wp[2] : wp[3];
      double rho = s.rhow[f];
      wU = r.d == 0 ? wp[1] : wp[2];
      wV = g.D == 1 ? 0.0 : (r.d == 0 ? wp[2] : -wp[1]);
      wlam = lw;
      wrn = g.D == 1 ? rho * sqrt(lw / PI) : rho * (lw / PI);
      wcB = g.Kb / (2.0 * lw);
      wsc = g.D == 2 ? (r.d == 0 ? g.dy : g.dx) : 1.0;
      int p0 = r.d == 0 ? r.fi : r.fj;
      rot = p0 == 0 ? 1.0 : -1.0;
    }
  }
};

// Velocity of one face direction: normal and tangential components, |c|^2
// and un^2.  The UGKS polynomial in (un, ut, c2) is evaluated in Horner form
// from these, so no higher monomials are held.
template <typename R>
struct Mono {
  R un, ut, c2, n2;
  __device__ __forceinline__ void set(R a, R b) {
    un = a;
    ut = b;
    c2 = a * a + b * b;
    n2 = a * a;
  }
};

// Interface flux of one face at this thread's velocity.  hu, bu: upwind cell
// values; su, sb: upwind slopes times dx; side = +0.5 when the upwind cell is
// on the left, -0.5 on the right; hc, bc: the interior cell of a wall face.
template <int D, int FLUX, bool FAST = false>
__device__ __forceinline__ void eval_face(const FEv<float>& e, const Mono<float>& M, float side,
                                          float hu, float bu, float su, float sb, float hc,
                                          float bc, double dt, float& fh, float& fb) {
  (void)dt;
  if (!FAST && e.kind == 0) {
    fh = 0.f;
    fb = 0.f;
    return;
  }
  const float un = M.un;
  if (!FAST && e.kind == 2) {
    // u h_wall len dt, h_wall the wall Maxwellian on incoming velocities
    // (src/Flux/flux_boundary.jl:39-61, :190-220)
    bool in = un * e.T.w >= 0.f;
    float hw, bw;
    if (in) {
      hw = ex2(e.E.x + e.E.y * un + e.E.z * M.ut + e.E.w * M.c2);
      bw = hw * e.T.z;
    } else {
      hw = hc;
      bw = bc;
    }
    fh = un * hw * e.T.x;
    fb = un * bw * e.T.x;
    return;
  }
  const float hf = hu + side * su;
  const float bf = bu + side * sb;
  const float a = e.T.x * un;
  const float c = e.T.y * M.n2;
  fh = a * hf - c * su;
  fb = a * bf - c * sb;
  if (FLUX == FLUX_KFVS) return;
  const float Hm = ex2(e.E.x + e.E.y * un + e.E.z * M.ut + e.E.w * M.c2);
  // un (T.z + un (C.x + C.y un + C.z ut + C.w c2) + G.x ut + G.y c2), b with T.w, Dd, G.zw
  float ph = e.T.z, pb = e.T.w;
  if (FLUX == FLUX_UGKS) {
    float ih = e.C.x + e.C.y * un + e.C.w * M.c2;
    float ib = e.Dd.x + e.Dd.y * un + e.Dd.w * M.c2;
    if (D == 2) {
      ih += e.C.z * M.ut;
      ib += e.Dd.z * M.ut;
    }
    ph += un * ih + e.G.x * M.ut + e.G.y * M.c2;
    pb += un * ib + e.G.z * M.ut + e.G.w * M.c2;
  }
  const float Hu = Hm * un;
  fh += Hu * ph;
  fb += Hu * pb;
}

template <int D, int FLUX, bool FAST = false>
__device__ __forceinline__ void eval_face(const FEv<double>& e, const Mono<double>& M,
                                          double side, double hu, double bu, double su,
                                          double sb, double hc, double bc, double dt,
                                          double& fh, double& fb) {
  if (!FAST && e.kind == 0) {
    fh = 0.0;
    fb = 0.0;
    return;
  }
  const double un = M.un, ut = M.ut;
  if (!FAST && e.kind == 2) {
    bool in = un * e.rot >= 0.0;
    double hw, bw;
    if (in) {
      double du = un - e.wU, ee = du * du;
      if (D == 2) {
        double dv = ut - e.wV;
        ee += dv * dv;
      }
      hw = e.wrn * exp(-e.wlam * ee);
      bw = hw * e.wcB;
    } else {
      hw = hc;
      bw = bc;
    }
    fh = un * hw * e.wsc * dt;
    fb = un * bw * e.wsc * dt;
    return;
  }
  const double hf = hu + side * su;
  const double bf = bu + side * sb;
  double Th, Tb;
  face_flux<double, FLUX, D>(e.P, dt, un, ut, side > 0.0, hf, bf, su / e.dd, sb / e.dd, fh, fb,
                             Th, Tb);
}

// Pointwise relaxation of one cell value (step!, src/Solver/step_2f.jl:32-63, :210-248).
__device__ __forceinline__ void relax(const CellCoef32& k, bool shak, float u, float vv,
                                      float c2, float h0, float b0, float dh, float db,
                                      float& hn, float& bn) {
  float M = ex2(k.EM.x + k.EM.y * u + k.EM.z * vv + k.EM.w * c2);
  float MH = M, MB = M * k.A.x;
  if (shak) {
    float OH = ex2(k.EO.x + k.EO.y * u + k.EO.z * vv + k.EO.w * c2);
    float cq = (k.Q.x + k.Q.y * u + k.Q.z * vv) * OH;
    float tl = k.TL.x + k.TL.y * u + k.TL.z * vv + k.TL.w * c2;
    MH += cq * (tl - 5.f);
    MB += cq * (tl - 3.f) * k.Q.w;
  }
  hn = (h0 + dh * k.A.w + k.A.y * MH) * k.A.z;
  bn = (b0 + db * k.A.w + k.A.y * MB) * k.A.z;
}

__device__ __forceinline__ void relax(const CP<double>& C, double ds, double u, double vv,
                                      double Kf, int D, double h0, double b0, double dh,
                                      double db, double& hn, double& bn) {
  if (!C.upd) {
    hn = h0;
    bn = b0;
    return;
  }
  double du = u - C.U, e = du * du;
  if (D == 2) {
    double dv = vv - C.V;
    e += dv * dv;
  }
  double MH = C.rho_n * exp(-C.lam * e);
  double MB = MH * Kf / (2.0 * C.lam);
  if (C.coll == COLL_SHAKHOV) {
    double ou = u - C.oU, oe = ou * ou, cq = ou * C.s0;
    if (D == 2) {
      double ov = vv - C.oV;
      oe += ov * ov;
      cq += ov * C.s1;
    }
    double OH = C.o_rho_n * exp(-C.olam * oe);
    double OB = OH * Kf / (2.0 * C.olam);
    double tl = 2.0 * C.olam * oe + Kf;
    MH += cq * (tl - 5.0) * OH;
    MB += cq * (tl - 3.0) * OB;
  }
  hn = (h0 + dh / ds + C.dtau * MH) / (1.0 + C.dtau);
  bn = (b0 + db / ds + C.dtau * MB) / (1.0 + C.dtau);
}

// Load face f's evaluation state: FP32 from its coefficient block c (global
// memory or staged in shared memory), FP64 from the FaceParam table.
template <bool FAST>
__device__ __forceinline__ void face_load(FEv<float>& e, const DevState& s, int f,
                                          const FaceCoef32& c, bool pos) {
  if (FAST) e.load_interior(c, pos);
  else e.load(c, s.kind[f], pos);
}
template <bool FAST>
__device__ __forceinline__ void face_load(FEv<double>& e, const DevState& s, int f,
                                          const FaceCoef32& c, bool pos) {
  (void)c;
  e.load(s, f, pos);
}

// Shared-memory staging of the FP32 coefficient blocks of a pass-B strip:
// rows are staged CH at a time into two buffers (double buffering) by bulk
// async copies issued from warp 0, each buffer completing on its own mbarrier.
// Per row of a buffer: x faces [TX+1], y faces above the row [TX], cells [TX].
constexpr int MARCH_CH = 8;
template <int TX>
struct MarchStage {
  static constexpr int XF = 0;
  static constexpr int YF = (TX + 1) * (int)sizeof(FaceCoef32);
  static constexpr int CC = YF + TX * (int)sizeof(FaceCoef32);
  static constexpr int ROW = CC + TX * (int)sizeof(CellCoef32);
  static constexpr int BUF = MARCH_CH * ROW;
  static constexpr int Y0 = TX * (int)sizeof(FaceCoef32);  // y faces below the first row
  // [y faces below the first row][buffer 0][buffer 1][2 mbarriers]
  static constexpr int BYTES = Y0 + 2 * BUF + 16;
};
static_assert(sizeof(FaceCoef32) % 16 == 0 && sizeof(CellCoef32) % 16 == 0,
              "bulk copies need 16-byte multiples");

// Pass B: one thread per velocity, CTA = (strip of TX columns, RY rows,
// BS velocities).  Window rows wh[0..3] = rows j-1 .. j+2 of the strip; the
// next window row and the next row's 4-cell x halo are loaded one iteration
// ahead so their latency overlaps the current row's arithmetic.  In the 2D
// FP32 form the per-face / per-cell coefficient blocks of the strip arrive in
// shared memory by bulk async copies, a chunk of rows ahead of their use, so
// the row body waits on no global load but the distributions.  Threads past
// the last velocity compute on a clamped velocity and store nothing, so every
// thread reaches every barrier.
template <typename R, int D, int FLUX, int TX, int BS>
__global__ void __launch_bounds__(BS, (sizeof(R) == 4 && TX < 4 ? 384 : 256) / BS) k_march(DevState s, double dt, int RY) {
  constexpr bool STAGE = sizeof(R) == 4 && D == 2;
  using SL = MarchStage<TX>;
  extern __shared__ __align__(16) unsigned char smem[];
  const Geo& g = s.g;
  const int vraw = blockIdx.z * BS + threadIdx.x;
  const bool vok = vraw < g.nvel;
  const int v = vok ? vraw : g.nvel - 1;
  const int i0 = blockIdx.x * TX;
  const int ncol = min(TX, g.nx - i0);
  const int j0 = D == 2 ? blockIdx.y * RY : 0;
  int j1 = D == 2 ? min(g.ny, j0 + RY) : 1;
  const int vs = g.vstride;
  const R* __restrict__ H = (const R*)s.h[s.cur];
  const R* __restrict__ Bq = (const R*)s.b[s.cur];
  R* __restrict__ Ho = (R*)s.h[s.cur ^ 1];
  R* __restrict__ Bo = (R*)s.b[s.cur ^ 1];

  // ---- coefficient staging (2D FP32)
  const int nchunk = (j1 - j0 + MARCH_CH - 1) / MARCH_CH;
  unsigned long long* bars = (unsigned long long*)(smem + SL::BYTES - 16);
  int failed = -1;  // chunk whose copies missed the deadline
  auto issue = [&](int ch) {  // warp 0: copy chunk ch into buffer ch & 1
    unsigned char* buf = smem + SL::Y0 + (ch & 1) * SL::BUF;
    const int r0 = j0 + ch * MARCH_CH;
    const int nr = min(MARCH_CH, j1 - r0);
    const unsigned xb = (ncol + 1) * sizeof(FaceCoef32), yb = ncol * sizeof(FaceCoef32),
                   cb = ncol * sizeof(CellCoef32);
    unsigned bytes = nr * (xb + yb + cb);
    if (ch == 0) bytes += yb;
    const int lane = threadIdx.x;
    if (lane == 0) mbar_expect(&bars[ch & 1], bytes);
    __syncwarp();
    if (lane < nr) {
      const int j = r0 + lane;
      unsigned char* row = buf + lane * SL::ROW;
      bulk_g2s(row + SL::XF, s.fc + (long)j * (g.nx + 1) + i0, xb, &bars[ch & 1]);
      bulk_g2s(row + SL::YF, s.fc + s.nface_x + (long)(j + 1) * g.nx + i0, yb, &bars[ch & 1]);
      bulk_g2s(row + SL::CC, s.cc + cell_index(g, i0, j), cb, &bars[ch & 1]);
    }
    if (ch == 0 && lane == 0)
      bulk_g2s(smem, s.fc + s.nface_x + (long)j0 * g.nx + i0, yb, &bars[0]);
  };
  // wait for chunk ch; the outcome is made CTA-uniform, and after a timeout
  // the CTA stops issuing copies and leaves the row loop
  auto await = [&](int ch) {
    const bool ok = mbar_wait(&bars[ch & 1], (ch >> 1) & 1);
    if (__syncthreads_or(!ok)) {
      failed = ch;
      if (threadIdx.x == 0) atomicOr(s.status, 2);
    }
  };
  if (STAGE) {
    if (threadIdx.x == 0) {
      mbar_init(&bars[0], 1);
      mbar_init(&bars[1], 1);
      fence_async_smem();
    }
    __syncthreads();
    if (threadIdx.x < 32) {
      issue(0);
      if (nchunk > 1) issue(1);
    }
  }

  const R u = vtab<R>(s, 0)[v];
  const R vv = D == 2 ? vtab<R>(s, 1)[v] : R(0);
  Mono<R> MX, MY;
  MX.set(u, vv);
  if (D == 2) MY.set(vv, -u);
  const bool px = u >= R(0), py = vv >= R(0);
  const R sys = py ? R(0.5) : R(-0.5);
  const R epsx = R(1.e-7 * g.dx), epsy = R(1.e-7 * g.dy);
  const bool shak = s.coll == COLL_SHAKHOV;
  const double ds = D == 1 ? g.dx : g.dx * g.dy;
  const double Kf = g.Kb;

  bool exx[TX + 4];
  int rx[TX + 4];
  int coff[TX + 4];  // offset of (column, v) inside a row
#pragma unroll
  for (int w = 0; w < TX + 4; ++w) {
    int i = i0 - 2 + w;
    exx[w] = i >= -g.ngx && i < g.nx + g.ngx;
    rx[w] = slope_rule(g, 0, i);
    coff[w] = exx[w] ? (i + g.ngx) * vs + v : 0;
  }
  const long rows = (long)g.nxt * vs;
  auto rowok = [&](int j) { return j >= -g.ngy && j < g.ny + g.ngy; };
  auto tile = [&](int j, R* th, R* tb) {
    const bool rk = rowok(j);
    const long ro = rk ? (long)(j + g.ngy) * rows : 0;
#pragma unroll
    for (int c = 0; c < TX; ++c) {
      const bool e = rk && exx[c + 2];
      th[c] = ldq(H + ro, coff[c + 2], e);
      tb[c] = ldq(Bq + ro, coff[c + 2], e);
    }
  };
  auto halo = [&](int j, R* hh, R* hb) {
    const bool rk = rowok(j);
    const long ro = rk ? (long)(j + g.ngy) * rows : 0;
#pragma unroll
    for (int k = 0; k < 4; ++k) {
      const int w = k < 2 ? k : TX + k;
      hh[k] = ldq(H + ro, coff[w], rk && exx[w]);
      hb[k] = ldq(Bq + ro, coff[w], rk && exx[w]);
    }
  };
  // coefficient blocks of row j: the staged copies, or the global tables
  auto stage_row = [&](int j) -> const unsigned char* {
    const int r = j - j0;
    return smem + SL::Y0 + ((r / MARCH_CH) & 1) * SL::BUF + (r % MARCH_CH) * SL::ROW;
  };
  auto xcoef = [&](int j) -> const FaceCoef32* {
    if (STAGE) return (const FaceCoef32*)(stage_row(j) + SL::XF);
    return s.fc + (long)j * (g.nx + 1) + i0;
  };
  auto ycoef = [&](int j) -> const FaceCoef32* {  // y faces above row j
    if (STAGE) return (const FaceCoef32*)(stage_row(j) + SL::YF);
    return s.fc + s.nface_x + (long)(j + 1) * g.nx + i0;
  };
  auto ccoef = [&](int j) -> const CellCoef32* {
    if (STAGE) return (const CellCoef32*)(stage_row(j) + SL::CC);
    return s.cc + cell_index(g, i0, j);
  };

  R wh[4][TX], wb[4][TX];
  R nh[TX], nb[TX];
  R hh[4], hb[4], nhh[4], nhb[4];
  R fyh[TX], fyb[TX];
  if (D == 2) {
    // prologue: rows j0-2 .. j0+2, the halo of row j0 and the y face below row j0
    R ph[TX], pb[TX];
    tile(j0 - 2, ph, pb);
#pragma unroll
    for (int k = 0; k < 4; ++k) tile(j0 - 1 + k, wh[k], wb[k]);
    halo(j0, hh, hb);
    if (STAGE) {
      await(0);
      if (failed >= 0) j1 = j0;  // no rows: straight to the bounded clean-up
    }
    const FaceCoef32* y0c =
        STAGE ? (const FaceCoef32*)smem : s.fc + s.nface_x + (long)j0 * g.nx + i0;
    const int rlo = slope_rule(g, 1, j0 - 1), rhi = slope_rule(g, 1, j0);
#pragma unroll
    for (int c = 0; c < TX; ++c) {
      FEv<R> e;
      e.kind = 0;
      if (c < ncol) face_load<false>(e, s, s.nface_x + j0 * g.nx + i0 + c, y0c[c], py);
      R hu, bu, su, sb;
      if (py) {
        hu = wh[0][c];
        bu = wb[0][c];
        su = vl_diff(rlo, ph[c], wh[0][c], wh[1][c], epsy);
        sb = vl_diff(rlo, pb[c], wb[0][c], wb[1][c], epsy);
      } else {
        hu = wh[1][c];
        bu = wb[1][c];
        su = vl_diff(rhi, wh[0][c], wh[1][c], wh[2][c], epsy);
        sb = vl_diff(rhi, wb[0][c], wb[1][c], wb[2][c], epsy);
      }
      eval_face<D, FLUX>(e, MY, sys, hu, bu, su, sb, wh[1][c], wb[1][c], dt, fyh[c], fyb[c]);
    }
  } else {
    tile(0, wh[1], wb[1]);
    halo(0, hh, hb);
  }

  auto row = [&](int j, auto fast_tag, auto sign_tag) {
    constexpr bool FAST = decltype(fast_tag)::value;
    constexpr int SG = decltype(sign_tag)::value;
    // compile-time upwind sides when the warp's velocities share their signs
    const bool qx = SG == 0 ? px : (SG == 1 || SG == 2);
    const bool qy = SG == 0 ? py : (SG == 1 || SG == 3);
    const R qxs = qx ? R(0.5) : R(-0.5), qys = qy ? R(0.5) : R(-0.5);
    const FaceCoef32* xc = xcoef(j);
    const FaceCoef32* yc = ycoef(j);
    const CellCoef32* cc = ccoef(j);
    // prefetch the next window row and the next row's halo
    if (D == 2 && j + 1 < j1) {
      tile(j + 3, nh, nb);
      halo(j + 1, nhh, nhb);
    }
    R xh[TX + 4], xb[TX + 4];
#pragma unroll
    for (int c = 0; c < TX; ++c) {
      xh[c + 2] = wh[1][c];
      xb[c + 2] = wb[1][c];
    }
#pragma unroll
    for (int k = 0; k < 2; ++k) {
      xh[k] = hh[k];
      xb[k] = hb[k];
      xh[TX + 2 + k] = hh[2 + k];
      xb[TX + 2 + k] = hb[2 + k];
    }
    // y faces above row j
    R fyh2[TX], fyb2[TX];
    if (D == 2) {
      const int rlo = slope_rule(g, 1, j), rhi = slope_rule(g, 1, j + 1);
#pragma unroll
      for (int c = 0; c < TX; ++c) {
        FEv<R> e;
        e.kind = 0;
        if (FAST || c < ncol)
          face_load<FAST>(e, s, s.nface_x + (j + 1) * g.nx + i0 + c, yc[c], qy);
        R hu, bu, su, sb;
        if (qy) {
          hu = wh[1][c];
          bu = wb[1][c];
          su = slope<FAST>(rlo, wh[0][c], wh[1][c], wh[2][c], epsy);
          sb = slope<FAST>(rlo, wb[0][c], wb[1][c], wb[2][c], epsy);
        } else {
          hu = wh[2][c];
          bu = wb[2][c];
          su = slope<FAST>(rhi, wh[1][c], wh[2][c], wh[3][c], epsy);
          sb = slope<FAST>(rhi, wb[1][c], wb[2][c], wb[3][c], epsy);
        }
        eval_face<D, FLUX, FAST>(e, MY, qys, hu, bu, su, sb, wh[1][c], wb[1][c], dt, fyh2[c],
                                 fyb2[c]);
      }
    }
    // x slopes of cells w = 1 .. TX+2 and the x faces of row j
    R dh[TX + 2], db[TX + 2];
#pragma unroll
    for (int w = 1; w <= TX + 2; ++w) {
      dh[w - 1] = slope<FAST>(rx[w], xh[w - 1], xh[w], xh[w + 1], epsx);
      db[w - 1] = slope<FAST>(rx[w], xb[w - 1], xb[w], xb[w + 1], epsx);
    }
    R fxh[TX + 1], fxb[TX + 1];
#pragma unroll
    for (int f = 0; f <= TX; ++f) {
      FEv<R> e;
      e.kind = 0;
      const int fi = i0 + f;
      if (FAST || f <= ncol) face_load<FAST>(e, s, j * (g.nx + 1) + fi, xc[f], qx);
      R hu = qx ? xh[f + 1] : xh[f + 2];
      R bu = qx ? xb[f + 1] : xb[f + 2];
      R su = qx ? dh[f] : dh[f + 1];
      R sb = qx ? db[f] : db[f + 1];
      R hc = fi == 0 ? xh[f + 2] : xh[f + 1];
      R bc = fi == 0 ? xb[f + 2] : xb[f + 1];
      eval_face<D, FLUX, FAST>(e, MX, qxs, hu, bu, su, sb, hc, bc, dt, fxh[f], fxb[f]);
    }
    // update the cells of row j
    const long ro = (long)(j + g.ngy) * rows;
#pragma unroll
    for (int c = 0; c < TX; ++c) {
      if (!FAST && c >= ncol) continue;
      R dhh = fxh[c] - fxh[c + 1];
      R dbb = fxb[c] - fxb[c + 1];
      if (D == 2) {
        dhh = dhh + fyh[c] - fyh2[c];
        dbb = dbb + fyb[c] - fyb2[c];
      }
      R hn, bn;
      if constexpr (sizeof(R) == 4) {
        const CellCoef32 k = cc[c];
        relax(k, shak, u, vv, MX.c2, xh[c + 2], xb[c + 2], dhh, dbb, hn, bn);
      } else {
        const CP<double> C = load_cp<double>(s, cell_index(g, i0 + c, j));
        relax(C, ds, u, vv, Kf, D, xh[c + 2], xb[c + 2], dhh, dbb, hn, bn);
      }
      if (vok) {
        Ho[ro + coff[c + 2]] = hn;
        Bo[ro + coff[c + 2]] = bn;
      }
    }
    if (D == 2) {
#pragma unroll
      for (int c = 0; c < TX; ++c) {
        wh[0][c] = wh[1][c];
        wb[0][c] = wb[1][c];
        wh[1][c] = wh[2][c];
        wb[1][c] = wb[2][c];
        wh[2][c] = wh[3][c];
        wb[2][c] = wb[3][c];
        wh[3][c] = nh[c];
        wb[3][c] = nb[c];
        fyh[c] = fyh2[c];
        fyb[c] = fyb2[c];
      }
#pragma unroll
      for (int k = 0; k < 4; ++k) {
        hh[k] = nhh[k];
        hb[k] = nhb[k];
      }
    }
  };
  const bool fastx = g.interp == 2 && i0 >= 2 && i0 + TX <= g.nx - 2;
  // warp-uniform velocity signs select a sign-specialised interior row body
  const unsigned bx = __ballot_sync(0xffffffffu, px), by = __ballot_sync(0xffffffffu, py);
  const int sg = (bx != 0 && bx != 0xffffffffu) || (by != 0 && by != 0xffffffffu)
                     ? 0 : (bx != 0 ? (by != 0 ? 1 : 2) : (by != 0 ? 3 : 4));
  using T0 = std::integral_constant<int, 0>;
  for (int j = j0; j < j1; ++j) {
    if (STAGE) {
      const int r = j - j0;
      if (r > 0 && r % MARCH_CH == 0) {
        const int ch = r / MARCH_CH;
        // buffer (ch + 1) & 1 is free once every thread finished chunk ch - 1
        if (ch + 1 < nchunk) {
          __syncthreads();
          if (threadIdx.x < 32) {
            if (threadIdx.x == 0) fence_async_smem();
            __syncwarp();
            issue(ch + 1);
          }
        }
        await(ch);
        if (failed >= 0) break;
      }
    }
    if (fastx && (D == 1 || (j >= 1 && j <= g.ny - 3))) {
      // sign-specialised rows only in the FP32 path (the FP64 path is
      // bound by the FP64 pipe, not by selects)
      if constexpr (sizeof(R) == 4) {
        switch (sg) {
          case 1: row(j, std::true_type{}, std::integral_constant<int, 1>{}); break;
          case 2: row(j, std::true_type{}, std::integral_constant<int, 2>{}); break;
          case 3: row(j, std::true_type{}, std::integral_constant<int, 3>{}); break;
          case 4: row(j, std::true_type{}, std::integral_constant<int, 4>{}); break;
          default: row(j, std::true_type{}, T0{}); break;
        }
      } else {
        row(j, std::true_type{}, T0{});
      }
    } else {
      row(j, std::false_type{}, T0{});
    }
  }
  if (STAGE && failed >= 0) {
    // copies of the failed chunk and of the one issued after it may still
    // land: wait (bounded) for them before the shared memory is released
    mbar_wait(&bars[failed & 1], (failed >> 1) & 1);
    if (failed + 1 < nchunk) mbar_wait(&bars[(failed + 1) & 1], ((failed + 1) >> 1) & 1);
  }
}

// ------------------------------------------------- pass B, FP32 2D (TMA rows)

// Shared-memory ring of the 2D FP32 update: one slot per grid row of the
// strip.  The slots' h and b boxes (TX+4 columns incl. the 2-cell x halo on
// each side, M3_BS velocities; [column][velocity]) come first, each box on a
// multiple of 1 KB; then the slots' coefficient blocks (x faces [TX+1], y
// faces above the row [TX], cells [TX]), packed at 16-byte multiples so that
// no padding sits between slots.
constexpr int M3_BS = KB_TMA_VBOX;  // velocities (threads) per CTA, one TMA box
template <int TX, int NS>
struct M3Layout {
  static constexpr int W = TX + 4;
  static constexpr int BOX = W * M3_BS * 4;
  static constexpr int DSLOT = 2 * BOX;  // h box, then b box
  static constexpr int XF = 0;           // offsets within a coefficient slot
  static constexpr int YF = XF + (TX + 1) * (int)sizeof(FaceCoef32);
  static constexpr int CC = YF + TX * (int)sizeof(FaceCoef32);
  static constexpr int CSLOT = CC + TX * (int)sizeof(CellCoef32);
  static constexpr int COEF = NS * DSLOT;         // first coefficient slot
  static constexpr int BARS = COEF + NS * CSLOT;  // full[NS], empty[NS], failure flag
  static constexpr int BYTES = BARS + 16 * NS + 16;
};

// Pass B in the 2D FP32 form.  Thread = one velocity; CTA = 128 velocities x
// a strip of TX columns x RY rows, marching up the rows.  Rows arrive by TMA
// (h and b boxes) plus bulk copies (coefficients) into a ring of NS slots,
// NS - 4 rows ahead of the 4-row stencil window: at the start of row j,
// thread 0 refills the slot of row j - 2 once every warp has released it
// (per-slot "empty" mbarriers), so only thread 0 ever waits on other warps
// and the window costs no registers.  Each
// x face and y face is evaluated once per velocity and feeds both neighbours.
template <int FLUX, int TX, int NS, bool GRP = false>
__global__ void __launch_bounds__(M3_BS) k_march3(const __grid_constant__ CUtensorMap tmh,
                                                  const __grid_constant__ CUtensorMap tmb,
                                                  DevState sp, int RY) {
  static_assert(NS >= 6, "the ring holds the 4-row window plus at least one row ahead");
  int lb;
  const int gr = group_member<GRP, GK_MARCH>(sp, lb);
  KB_GROUP_STATE(GRP, sp, gr);
  const CUtensorMap* mh = GRP ? sp.grp->maps + gr * 6 + 4 : &tmh;
  const CUtensorMap* mb = GRP ? sp.grp->maps + gr * 6 + 5 : &tmb;
  if (GRP && threadIdx.x == 0) {  // the issuing thread
    tmap_acquire(mh);
    tmap_acquire(mb);
  }
  // block coordinates (velocity box, strip, row block) in the member's own grid
  int bx = blockIdx.x, by = blockIdx.y, bz = blockIdx.z;
  if (GRP) {
    const int gx = (s.g.nvel + M3_BS - 1) / M3_BS, gy = (s.g.nx + TX - 1) / TX;
    bx = lb % gx;
    by = (lb / gx) % gy;
    bz = lb / (gx * gy);
  }
  using L = M3Layout<TX, NS>;
  constexpr int D = 2;
  extern __shared__ __align__(1024) unsigned char smem3[];
  unsigned long long* full = (unsigned long long*)(smem3 + L::BARS);
  unsigned long long* empty = full + NS;
  int* bad = (int*)(empty + NS);
  volatile int* vbad = bad;
  const Geo& g = s.g;
  const int tid = threadIdx.x, lane = tid & 31;
  const int v0 = bx * M3_BS;
  const int vraw = v0 + tid;
  const bool vok = vraw < g.nvel;
  const int v = vok ? vraw : g.nvel - 1;
  const int i0 = by * TX;
  const int ncol = min(TX, g.nx - i0);
  const int j0 = bz * RY;
  const int j1 = min(g.ny, j0 + RY);
  const int q0 = j0 - 2;    // first staged row
  const int qend = j1 + 1;  // last staged row
  const int vs = g.vstride;
  float* __restrict__ Ho = (float*)s.h[s.cur ^ 1];
  float* __restrict__ Bo = (float*)s.b[s.cur ^ 1];

  auto slot = [&](int q) -> const unsigned char* { return smem3 + ((q - q0) % NS) * L::DSLOT; };
  auto cslot = [&](int q) -> const unsigned char* {
    return smem3 + L::COEF + ((q - q0) % NS) * L::CSLOT;
  };
  auto issue = [&](int q) {  // thread 0: grid row q and its coefficient blocks
    const int r = q - q0;
    unsigned char* S = smem3 + (r % NS) * L::DSLOT;
    unsigned char* C = smem3 + L::COEF + (r % NS) * L::CSLOT;
    unsigned long long* bar = &full[r % NS];
    const bool hy = q >= j0 - 1 && q <= j1 - 1, hx = q >= j0 && q <= j1 - 1;
    const unsigned xb = (ncol + 1) * sizeof(FaceCoef32), yb = ncol * sizeof(FaceCoef32),
                   cb = ncol * sizeof(CellCoef32);
    mbar_expect(bar, 2 * L::BOX + (hy ? yb : 0u) + (hx ? xb + cb : 0u));
    tma_load_3d(S, mh, v0, i0 - 2 + g.ngx, q + g.ngy, bar);
    tma_load_3d(S + L::BOX, mb, v0, i0 - 2 + g.ngx, q + g.ngy, bar);
    if (hx) {
      bulk_g2s(C + L::XF, s.fc + (long)q * (g.nx + 1) + i0, xb, bar);
      bulk_g2s(C + L::CC, s.cc + cell_index(g, i0, q), cb, bar);
    }
    if (hy) bulk_g2s(C + L::YF, s.fc + s.nface_x + (long)(q + 1) * g.nx + i0, yb, bar);
  };
  // every thread waits for row q itself; after any timeout the copies stop
  // and the remaining waits are skipped (the status word reports it)
  auto await_row = [&](int q) {
    if (*vbad) return;
    const int r = q - q0;
    if (!mbar_wait(&full[r % NS], (r / NS) & 1)) {
      atomicOr(bad, 1);
      atomicOr(s.status, 2);
    }
  };
  auto release_row = [&](int q) {  // this warp no longer reads row q
    __syncwarp();
    if (lane == 0) mbar_arrive(&empty[(q - q0) % NS]);
  };

  int issued = 0;  // rows issued so far (thread 0)
  if (tid == 0) {
    for (int k = 0; k < NS; ++k) {
      mbar_init(&full[k], 1);
      mbar_init(&empty[k], M3_BS / 32);
    }
    *bad = 0;
    fence_async_smem();
  }
  __syncthreads();
  if (tid == 0)
    for (int q = q0; q <= qend && q < q0 + NS; ++q, ++issued) issue(q);

  const float u = s.uf[v], vv = s.vf[v];
  Mono<float> MX, MY;
  MX.set(u, vv);
  MY.set(vv, -u);
  const bool px = u >= 0.f, py = vv >= 0.f;
  const float sx = px ? 0.5f : -0.5f, sy = py ? 0.5f : -0.5f;
  const float epsx = float(1.e-7 * g.dx), epsy = float(1.e-7 * g.dy);
  const bool shak = s.coll == COLL_SHAKHOV;
  const int shx = px ? 0 : 1;  // x window shift: face f's upwind cell is window k = f + 1
  int rxs[TX + 3];             // x slope rule of window k (column k + shx)
#pragma unroll
  for (int k = 0; k < TX + 3; ++k) rxs[k] = slope_rule(g, 0, i0 - 2 + k + shx);
  const long rowstride = (long)g.nxt * vs;

  auto Hv = [&](const unsigned char* S, int w) { return ((const float*)S)[w * M3_BS + tid]; };
  auto Bv = [&](const unsigned char* S, int w) {
    return ((const float*)(S + L::BOX))[w * M3_BS + tid];
  };
  // flux through the y face of column c between rows ql and ql + 1
  auto yface = [&](int ql, int c, auto fast_tag, float& fh, float& fb) {
    constexpr bool FAST = decltype(fast_tag)::value;
    fh = 0.f;
    fb = 0.f;
    if (!FAST && c >= ncol) return;
    const int qa = py ? ql - 1 : ql;  // stencil rows qa .. qa + 2, upwind cell qa + 1
    const unsigned char* S0 = slot(qa);
    const unsigned char* S1 = slot(qa + 1);
    const unsigned char* S2 = slot(qa + 2);
    const int w = c + 2;
    const float h0 = Hv(S1, w), b0 = Bv(S1, w);
    const int rule = FAST ? 1 : slope_rule(g, 1, qa + 1);
    const float su = vl_diff(rule, Hv(S0, w), h0, Hv(S2, w), epsy);
    const float sb = vl_diff(rule, Bv(S0, w), b0, Bv(S2, w), epsy);
    FEv<float> e;
    const FaceCoef32* yc = (const FaceCoef32*)(cslot(ql) + L::YF);
    face_load<FAST>(e, s, s.nface_x + (ql + 1) * g.nx + i0 + c, yc[c], py);
    float hc = 0.f, bc = 0.f;
    if (!FAST) {  // interior cell of a wall face
      const unsigned char* Si = slot(ql + 1 == 0 ? ql + 1 : ql);
      hc = Hv(Si, w);
      bc = Bv(Si, w);
    }
    eval_face<D, FLUX, FAST>(e, MY, sy, h0, b0, su, sb, hc, bc, 0.0, fh, fb);
  };

  float fyh[TX], fyb[TX];  // flux through the y faces below the current row
  await_row(q0);
  await_row(q0 + 1);
  await_row(q0 + 2);
  await_row(q0 + 3);
  {
    const bool fast = g.interp == 2 && i0 >= 2 && i0 + TX <= g.nx - 2 && j0 >= 2 && j0 <= g.ny - 2;
#pragma unroll
    for (int c = 0; c < TX; ++c) {
      if (fast) yface(j0 - 1, c, std::true_type{}, fyh[c], fyb[c]);
      else yface(j0 - 1, c, std::false_type{}, fyh[c], fyb[c]);
    }
  }
  release_row(q0);

  auto row = [&](int j, auto fast_tag) {
    constexpr bool FAST = decltype(fast_tag)::value;
    const unsigned char* Sj = slot(j);
    // y faces above row j
    float fyh2[TX], fyb2[TX];
#pragma unroll
    for (int c = 0; c < TX; ++c) yface(j, c, fast_tag, fyh2[c], fyb2[c]);
    // x window of row j, shifted to the upwind side, and the x faces
    float xs[TX + 3], xt[TX + 3];
#pragma unroll
    for (int k = 0; k < TX + 3; ++k) {
      xs[k] = Hv(Sj, k + shx);
      xt[k] = Bv(Sj, k + shx);
    }
    const FaceCoef32* xc = (const FaceCoef32*)(cslot(j) + L::XF);
    float fxh[TX + 1], fxb[TX + 1];
#pragma unroll
    for (int f = 0; f <= TX; ++f) {
      fxh[f] = 0.f;
      fxb[f] = 0.f;
      if (!FAST && f > ncol) continue;
      const float su = slope<FAST>(rxs[f + 1], xs[f], xs[f + 1], xs[f + 2], epsx);
      const float sb = slope<FAST>(rxs[f + 1], xt[f], xt[f + 1], xt[f + 2], epsx);
      FEv<float> e;
      const int fi = i0 + f;
      face_load<FAST>(e, s, j * (g.nx + 1) + fi, xc[f], px);
      float hc = 0.f, bc = 0.f;
      if (!FAST) {  // interior cell of a wall face
        hc = Hv(Sj, fi == 0 ? f + 2 : f + 1);
        bc = Bv(Sj, fi == 0 ? f + 2 : f + 1);
      }
      eval_face<D, FLUX, FAST>(e, MX, sx, xs[f + 1], xt[f + 1], su, sb, hc, bc, 0.0, fxh[f],
                               fxb[f]);
    }
    // relax and store the cells of row j
    const CellCoef32* cc = (const CellCoef32*)(cslot(j) + L::CC);
    const long ro = (long)(j + g.ngy) * rowstride + (long)(i0 + g.ngx) * vs + v;
#pragma unroll
    for (int c = 0; c < TX; ++c) {
      if (!FAST && c >= ncol) continue;
      const float dhh = fxh[c] - fxh[c + 1] + fyh[c] - fyh2[c];
      const float dbb = fxb[c] - fxb[c + 1] + fyb[c] - fyb2[c];
      float hn, bn;
      const CellCoef32 k = cc[c];
      relax(k, shak, u, vv, MX.c2, Hv(Sj, c + 2), Bv(Sj, c + 2), dhh, dbb, hn, bn);
      if (vok) {
        Ho[ro + (long)c * vs] = hn;
        Bo[ro + (long)c * vs] = bn;
      }
    }
#pragma unroll
    for (int c = 0; c < TX; ++c) {
      fyh[c] = fyh2[c];
      fyb[c] = fyb2[c];
    }
  };

  const bool fastx = g.interp == 2 && i0 >= 2 && i0 + TX <= g.nx - 2;
  for (int j = j0; j < j1; ++j) {
    if (tid == 0 && *vbad == 0) {
      // refill the slot of row q - NS = j - 2, which every warp released at
      // the end of row j - 1: the ring then runs NS - 4 rows ahead
      const int q = j + NS - 2;
      if (q <= qend) {
        const int r = q - q0;
        if (mbar_wait(&empty[r % NS], ((r - NS) / NS) & 1)) {
          fence_async_smem();
          issue(q);
          ++issued;
        } else {
          atomicOr(bad, 1);
          atomicOr(s.status, 2);
        }
      }
    }
    await_row(j + 2);
    if (fastx && j >= 1 && j <= g.ny - 3) row(j, std::true_type{});
    else row(j, std::false_type{});
    release_row(j - 1);
  }
  __syncthreads();
  if (*vbad && tid == 0) {
    // copies of the last rows issued may still land: wait (bounded) for each
    // slot's latest row before the shared memory is released
    for (int r = max(0, issued - NS); r < issued; ++r) mbar_wait(&full[r % NS], (r / NS) & 1);
  }
}

// ------------------------------------ pass B, FP32 2D, two velocities per thread

// Packed FP32 pair arithmetic (one instruction for both lanes of a float2).
__device__ __forceinline__ float2 f2add(float2 a, float2 b) { return __fadd2_rn(a, b); }
__device__ __forceinline__ float2 f2mul(float2 a, float2 b) { return __fmul2_rn(a, b); }
__device__ __forceinline__ float2 f2fma(float2 a, float2 b, float2 c) { return __ffma2_rn(a, b, c); }
__device__ __forceinline__ float2 f2sub(float2 a, float2 b) {
  unsigned long long A = *reinterpret_cast<unsigned long long*>(&a);
  unsigned long long B = *reinterpret_cast<unsigned long long*>(&b), C;
  asm("sub.rn.f32x2 %0, %1, %2;" : "=l"(C) : "l"(A), "l"(B));
  return *reinterpret_cast<float2*>(&C);
}
__device__ __forceinline__ float2 f2s(float s) { return make_float2(s, s); }
__device__ __forceinline__ float2 f2ex2(float2 a) { return make_float2(ex2(a.x), ex2(a.y)); }

// van Leer slope (times dx) of a pair, interior cells (rule 1)
__device__ __forceinline__ float2 vl2(float2 qm, float2 q0, float2 qp, float epsd) {
  const float2 a = f2sub(q0, qm), b = f2sub(qp, q0);
  const float2 A = make_float2(fabsf(a.x), fabsf(a.y)), B = make_float2(fabsf(b.x), fabsf(b.y));
  const float2 num = f2fma(b, A, f2mul(a, B));
  const float2 den = f2add(f2add(A, B), f2s(epsd));
  return make_float2(fdiv_ftz(num.x, den.x), fdiv_ftz(num.y, den.y));
}
// general slope of a pair: per-lane rules (boundary cells)
__device__ __forceinline__ float2 slope2(int r0, int r1, float2 qm, float2 q0, float2 qp,
                                         float epsd) {
  if (r0 == 1 && r1 == 1) return vl2(qm, q0, qp, epsd);
  return make_float2(vl_diff(r0, qm.x, q0.x, qp.x, epsd), vl_diff(r1, qm.y, q0.y, qp.y, epsd));
}

struct Mono2 {
  float2 un, ut, c2, n2;
  __device__ __forceinline__ void set(float2 a, float2 b) {
    un = a;
    ut = b;
    c2 = f2fma(a, a, f2mul(b, b));
    n2 = f2mul(a, a);
  }
  __device__ __forceinline__ Mono<float> lane(int k) const {
    Mono<float> M;
    M.un = k ? un.y : un.x;
    M.ut = k ? ut.y : ut.x;
    M.c2 = k ? c2.y : c2.x;
    M.n2 = k ? n2.y : n2.x;
    return M;
  }
};

// interface flux of an interior face for a velocity pair (same formulas as
// eval_face); non-interior faces go lane by lane through eval_face
template <int D, int FLUX, bool FAST>
__device__ __forceinline__ void eval_face2(const FEv<float>& e, const Mono2& M, float2 side,
                                           float2 hu, float2 bu, float2 su, float2 sb,
                                           float2 hc, float2 bc, float2& fh, float2& fb) {
  if (!FAST && e.kind != 1) {
    eval_face<D, FLUX>(e, M.lane(0), side.x, hu.x, bu.x, su.x, sb.x, hc.x, bc.x, 0.0, fh.x, fb.x);
    eval_face<D, FLUX>(e, M.lane(1), side.y, hu.y, bu.y, su.y, sb.y, hc.y, bc.y, 0.0, fh.y, fb.y);
    return;
  }
  const float2 hf = f2fma(side, su, hu), bf = f2fma(side, sb, bu);
  const float2 a = f2mul(f2s(e.T.x), M.un);
  const float2 c = f2mul(f2s(-e.T.y), M.n2);
  fh = f2fma(c, su, f2mul(a, hf));
  fb = f2fma(c, sb, f2mul(a, bf));
  if (FLUX == FLUX_KFVS) return;
  const float2 Hm = f2ex2(
      f2fma(f2s(e.E.w), M.c2, f2fma(f2s(e.E.z), M.ut, f2fma(f2s(e.E.y), M.un, f2s(e.E.x)))));
  float2 ph = f2s(e.T.z), pb = f2s(e.T.w);
  if (FLUX == FLUX_UGKS) {
    float2 ih = f2fma(f2s(e.C.w), M.c2, f2fma(f2s(e.C.y), M.un, f2s(e.C.x)));
    float2 ib = f2fma(f2s(e.Dd.w), M.c2, f2fma(f2s(e.Dd.y), M.un, f2s(e.Dd.x)));
    if (D == 2) {
      ih = f2fma(f2s(e.C.z), M.ut, ih);
      ib = f2fma(f2s(e.Dd.z), M.ut, ib);
    }
    ph = f2fma(f2s(e.G.y), M.c2, f2fma(f2s(e.G.x), M.ut, f2fma(M.un, ih, ph)));
    pb = f2fma(f2s(e.G.w), M.c2, f2fma(f2s(e.G.z), M.ut, f2fma(M.un, ib, pb)));
  }
  const float2 Hu = f2mul(Hm, M.un);
  fh = f2fma(Hu, ph, fh);
  fb = f2fma(Hu, pb, fb);
}

// pointwise relaxation of a velocity pair (same formulas as relax)
__device__ __forceinline__ void relax2(const CellCoef32& k, bool shak, float2 u, float2 vv,
                                       float2 c2, float2 h0, float2 b0, float2 dh, float2 db,
                                       float2& hn, float2& bn) {
  const float2 M = f2ex2(
      f2fma(f2s(k.EM.w), c2, f2fma(f2s(k.EM.z), vv, f2fma(f2s(k.EM.y), u, f2s(k.EM.x)))));
  float2 MH = M, MB = f2mul(M, f2s(k.A.x));
  if (shak) {
    const float2 OH = f2ex2(
        f2fma(f2s(k.EO.w), c2, f2fma(f2s(k.EO.z), vv, f2fma(f2s(k.EO.y), u, f2s(k.EO.x)))));
    const float2 cq = f2mul(f2fma(f2s(k.Q.z), vv, f2fma(f2s(k.Q.y), u, f2s(k.Q.x))), OH);
    const float2 tl =
        f2fma(f2s(k.TL.w), c2, f2fma(f2s(k.TL.z), vv, f2fma(f2s(k.TL.y), u, f2s(k.TL.x))));
    MH = f2fma(cq, f2add(tl, f2s(-5.f)), MH);
    MB = f2fma(f2mul(cq, f2add(tl, f2s(-3.f))), f2s(k.Q.w), MB);
  }
  hn = f2mul(f2fma(f2s(k.A.y), MH, f2fma(dh, f2s(k.A.w), h0)), f2s(k.A.z));
  bn = f2mul(f2fma(f2s(k.A.y), MB, f2fma(db, f2s(k.A.w), b0)), f2s(k.A.z));
}

// Pass B in the 2D FP32 form with two adjacent velocities per thread: the
// same ring, rows and faces as k_march3, with packed FP32-pair arithmetic, so
// each face's coefficients, each slot lookup and each barrier operation serve
// two velocities.  A CTA of 64 threads covers the 128 velocities of a box.
constexpr int M4_THREADS = M3_BS / 2;
// Two groups (TX 4, NS 6): 128 registers a thread and 57 KB of shared memory
// let four CTAs (16 warps) share an SM.
template <int FLUX, int TX, int NS, int G>
__global__ void __launch_bounds__(M4_THREADS * G, G == 2 ? 4 : 1) k_march4(const __grid_constant__ CUtensorMap tmh,
                                                       const __grid_constant__ CUtensorMap tmb,
                                                       DevState s, int RY) {
  static_assert(NS >= 6, "the ring holds the 4-row window plus at least one row ahead");
  using L = M3Layout<TX, NS>;
  constexpr int D = 2;
  extern __shared__ __align__(1024) unsigned char smem4[];
  unsigned long long* full = (unsigned long long*)(smem4 + L::BARS);
  unsigned long long* empty = full + NS;
  int* bad = (int*)(empty + NS);
  volatile int* vbad = bad;
  const Geo& g = s.g;
  const int tid = threadIdx.x, lane = tid & 31;
  // G groups of 64 threads split the strip's columns: group tid / 64 owns
  // columns cg .. cg + TXG - 1; every group covers all 128 velocities
  constexpr int TXG = TX / G;
  const int lt = tid % M4_THREADS, cg = (tid / M4_THREADS) * TXG;
  const int v0 = blockIdx.x * M3_BS;
  const int va = v0 + 2 * lt, vb = va + 1;  // this thread's velocities
  const bool oka = va < g.nvel, okb = vb < g.nvel;
  const int ia = oka ? va : g.nvel - 1, ib = okb ? vb : g.nvel - 1;
  const int i0 = blockIdx.y * TX;
  const int ncol = min(TX, g.nx - i0);
  const int j0 = blockIdx.z * RY;
  const int j1 = min(g.ny, j0 + RY);
  const int q0 = j0 - 2;
  const int qend = j1 + 1;
  const int vs = g.vstride;
  float* __restrict__ Ho = (float*)s.h[s.cur ^ 1];
  float* __restrict__ Bo = (float*)s.b[s.cur ^ 1];

  auto slot = [&](int q) -> const unsigned char* { return smem4 + ((q - q0) % NS) * L::DSLOT; };
  auto cslot = [&](int q) -> const unsigned char* {
    return smem4 + L::COEF + ((q - q0) % NS) * L::CSLOT;
  };
  auto issue = [&](int q) {
    const int r = q - q0;
    unsigned char* S = smem4 + (r % NS) * L::DSLOT;
    unsigned char* C = smem4 + L::COEF + (r % NS) * L::CSLOT;
    unsigned long long* bar = &full[r % NS];
    const bool hy = q >= j0 - 1 && q <= j1 - 1, hx = q >= j0 && q <= j1 - 1;
    const unsigned xb = (ncol + 1) * sizeof(FaceCoef32), yb = ncol * sizeof(FaceCoef32),
                   cb = ncol * sizeof(CellCoef32);
    mbar_expect(bar, 2 * L::BOX + (hy ? yb : 0u) + (hx ? xb + cb : 0u));
    tma_load_3d(S, &tmh, v0, i0 - 2 + g.ngx, q + g.ngy, bar);
    tma_load_3d(S + L::BOX, &tmb, v0, i0 - 2 + g.ngx, q + g.ngy, bar);
    if (hx) {
      bulk_g2s(C + L::XF, s.fc + (long)q * (g.nx + 1) + i0, xb, bar);
      bulk_g2s(C + L::CC, s.cc + cell_index(g, i0, q), cb, bar);
    }
    if (hy) bulk_g2s(C + L::YF, s.fc + s.nface_x + (long)(q + 1) * g.nx + i0, yb, bar);
  };
  auto await_row = [&](int q) {
    if (*vbad) return;
    const int r = q - q0;
    if (!mbar_wait(&full[r % NS], (r / NS) & 1)) {
      atomicOr(bad, 1);
      atomicOr(s.status, 2);
    }
  };
  auto release_row = [&](int q) {
    __syncwarp();
    if (lane == 0) mbar_arrive(&empty[(q - q0) % NS]);
  };

  int issued = 0;
  if (tid == 0) {
    for (int k = 0; k < NS; ++k) {
      mbar_init(&full[k], 1);
      mbar_init(&empty[k], M4_THREADS * G / 32);
    }
    *bad = 0;
    fence_async_smem();
  }
  __syncthreads();
  if (tid == 0)
    for (int q = q0; q <= qend && q < q0 + NS; ++q, ++issued) issue(q);

  const float2 u = make_float2(s.uf[ia], s.uf[ib]), vv = make_float2(s.vf[ia], s.vf[ib]);
  Mono2 MX, MY;
  MX.set(u, vv);
  MY.set(vv, make_float2(-u.x, -u.y));
  const bool pxa = u.x >= 0.f, pxb = u.y >= 0.f, pya = vv.x >= 0.f, pyb = vv.y >= 0.f;
  const float2 sx = make_float2(pxa ? 0.5f : -0.5f, pxb ? 0.5f : -0.5f);
  const float2 sy = make_float2(pya ? 0.5f : -0.5f, pyb ? 0.5f : -0.5f);
  const float epsx = float(1.e-7 * g.dx), epsy = float(1.e-7 * g.dy);
  const bool shak = s.coll == COLL_SHAKHOV;
  const int sha = pxa ? 0 : 1, shb = pxb ? 0 : 1;  // x window shift per lane
  const bool samex = sha == shb, samey = pya == pyb;
  int rxa[TXG + 3], rxb[TXG + 3];
#pragma unroll
  for (int k = 0; k < TXG + 3; ++k) {
    rxa[k] = slope_rule(g, 0, i0 - 2 + cg + k + sha);
    rxb[k] = slope_rule(g, 0, i0 - 2 + cg + k + shb);
  }
  const long rowstride = (long)g.nxt * vs;

  // values of this thread's pair in column w of a slot: both lanes from the
  // same column (one 64-bit load) or each lane from its own column
  auto Hp = [&](const unsigned char* S, int w) {
    return *(const float2*)((const float*)S + w * M3_BS + 2 * lt);
  };
  auto Bp = [&](const unsigned char* S, int w) {
    return *(const float2*)((const float*)(S + L::BOX) + w * M3_BS + 2 * lt);
  };
  auto H2 = [&](const unsigned char* Sa, int wa, const unsigned char* Sb, int wb) {
    return make_float2(((const float*)Sa)[wa * M3_BS + 2 * lt],
                       ((const float*)Sb)[wb * M3_BS + 2 * lt + 1]);
  };
  auto B2 = [&](const unsigned char* Sa, int wa, const unsigned char* Sb, int wb) {
    return make_float2(((const float*)(Sa + L::BOX))[wa * M3_BS + 2 * lt],
                       ((const float*)(Sb + L::BOX))[wb * M3_BS + 2 * lt + 1]);
  };

  auto yface = [&](int ql, int c, auto fast_tag, auto same_tag, float2& fh, float2& fb) {
    constexpr bool FAST = decltype(fast_tag)::value;
    constexpr bool SAME = decltype(same_tag)::value;  // both lanes share their upwind sides
    fh = f2s(0.f);
    fb = f2s(0.f);
    if (!FAST && cg + c >= ncol) return;
    const int w = cg + c + 2;
    const int qa = pya ? ql - 1 : ql, qb = pyb ? ql - 1 : ql;  // stencil rows start
    float2 hm, h0, hp, bm, b0, bp;
    if (SAME) {
      const unsigned char* S0 = slot(qa);
      const unsigned char* S1 = slot(qa + 1);
      const unsigned char* S2 = slot(qa + 2);
      hm = Hp(S0, w); h0 = Hp(S1, w); hp = Hp(S2, w);
      bm = Bp(S0, w); b0 = Bp(S1, w); bp = Bp(S2, w);
    } else {
      hm = H2(slot(qa), w, slot(qb), w); h0 = H2(slot(qa + 1), w, slot(qb + 1), w);
      hp = H2(slot(qa + 2), w, slot(qb + 2), w);
      bm = B2(slot(qa), w, slot(qb), w); b0 = B2(slot(qa + 1), w, slot(qb + 1), w);
      bp = B2(slot(qa + 2), w, slot(qb + 2), w);
    }
    float2 su, sb;
    if (FAST) {
      su = vl2(hm, h0, hp, epsy);
      sb = vl2(bm, b0, bp, epsy);
    } else {
      const int ra = slope_rule(g, 1, qa + 1), rb = slope_rule(g, 1, qb + 1);
      su = slope2(ra, rb, hm, h0, hp, epsy);
      sb = slope2(ra, rb, bm, b0, bp, epsy);
    }
    FEv<float> e;
    const FaceCoef32* yc = (const FaceCoef32*)(cslot(ql) + L::YF);
    if (FAST) e.load_interior(yc[cg + c], true);
    else e.load(yc[cg + c], s.kind[s.nface_x + (ql + 1) * g.nx + i0 + cg + c], true);
    if (FLUX != FLUX_KFVS && (FAST || e.kind == 1)) {
      // the upwind-dependent coefficients of each lane
      const float4* cpa = pya ? &yc[cg + c].Cp : &yc[cg + c].Cm;
      if (!SAME) {  // mixed pair: evaluate lane by lane
        FEv<float> ea = e, eb = e;
        ea.C = (pya ? yc[cg + c].Cp : yc[cg + c].Cm);
        ea.Dd = (pya ? yc[cg + c].Dp : yc[cg + c].Dm);
        eb.C = (pyb ? yc[cg + c].Cp : yc[cg + c].Cm);
        eb.Dd = (pyb ? yc[cg + c].Dp : yc[cg + c].Dm);
        eval_face<D, FLUX>(ea, MY.lane(0), sy.x, h0.x, b0.x, su.x, sb.x, 0.f, 0.f, 0.0, fh.x, fb.x);
        eval_face<D, FLUX>(eb, MY.lane(1), sy.y, h0.y, b0.y, su.y, sb.y, 0.f, 0.f, 0.0, fh.y, fb.y);
        return;
      }
      e.C = cpa[0];
      e.Dd = cpa[1];
    }
    float2 hc = f2s(0.f), bc = f2s(0.f);
    if (!FAST) {
      const unsigned char* Si = slot(ql + 1 == 0 ? ql + 1 : ql);
      hc = Hp(Si, w);
      bc = Bp(Si, w);
    }
    eval_face2<D, FLUX, FAST>(e, MY, sy, h0, b0, su, sb, hc, bc, fh, fb);
  };

  float2 fyh[TXG], fyb[TXG];
  await_row(q0);
  await_row(q0 + 1);
  await_row(q0 + 2);
  await_row(q0 + 3);
  const bool same = samex && samey;
  {
    const bool fast = g.interp == 2 && i0 >= 2 && i0 + TX <= g.nx - 2 && j0 >= 2 && j0 <= g.ny - 2;
#pragma unroll
    for (int c = 0; c < TXG; ++c) {
      if (fast && same) yface(j0 - 1, c, std::true_type{}, std::true_type{}, fyh[c], fyb[c]);
      else yface(j0 - 1, c, std::false_type{}, std::false_type{}, fyh[c], fyb[c]);
    }
  }
  release_row(q0);

  auto row = [&](int j, auto fast_tag, auto same_tag) {
    constexpr bool FAST = decltype(fast_tag)::value;
    constexpr bool SAME = decltype(same_tag)::value;
    const unsigned char* Sj = slot(j);
    float2 fyh2[TXG], fyb2[TXG];
#pragma unroll
    for (int c = 0; c < TXG; ++c) yface(j, c, fast_tag, same_tag, fyh2[c], fyb2[c]);
    // x window of row j shifted to each lane's upwind side
    float2 xs[TXG + 3], xt[TXG + 3];
    if (SAME) {
#pragma unroll
      for (int k = 0; k < TXG + 3; ++k) {
        xs[k] = Hp(Sj, cg + k + sha);
        xt[k] = Bp(Sj, cg + k + sha);
      }
    } else {
#pragma unroll
      for (int k = 0; k < TXG + 3; ++k) {
        xs[k] = H2(Sj, cg + k + sha, Sj, cg + k + shb);
        xt[k] = B2(Sj, cg + k + sha, Sj, cg + k + shb);
      }
    }
    const FaceCoef32* xc = (const FaceCoef32*)(cslot(j) + L::XF);
    float2 fxh[TXG + 1], fxb[TXG + 1];
#pragma unroll
    for (int f = 0; f <= TXG; ++f) {
      fxh[f] = f2s(0.f);
      fxb[f] = f2s(0.f);
      if (!FAST && cg + f > ncol) continue;
      float2 su, sb;
      if (FAST) {
        su = vl2(xs[f], xs[f + 1], xs[f + 2], epsx);
        sb = vl2(xt[f], xt[f + 1], xt[f + 2], epsx);
      } else {
        su = slope2(rxa[f + 1], rxb[f + 1], xs[f], xs[f + 1], xs[f + 2], epsx);
        sb = slope2(rxa[f + 1], rxb[f + 1], xt[f], xt[f + 1], xt[f + 2], epsx);
      }
      const int fi = i0 + cg + f;
      FEv<float> e;
      if (FAST) e.load_interior(xc[cg + f], true);
      else e.load(xc[cg + f], s.kind[j * (g.nx + 1) + fi], true);
      if (FLUX != FLUX_KFVS && (FAST || e.kind == 1)) {
        if (!SAME) {  // mixed pair: evaluate lane by lane
          FEv<float> ea = e, eb = e;
          ea.C = (pxa ? xc[cg + f].Cp : xc[cg + f].Cm);
          ea.Dd = (pxa ? xc[cg + f].Dp : xc[cg + f].Dm);
          eb.C = (pxb ? xc[cg + f].Cp : xc[cg + f].Cm);
          eb.Dd = (pxb ? xc[cg + f].Dp : xc[cg + f].Dm);
          eval_face<D, FLUX>(ea, MX.lane(0), sx.x, xs[f + 1].x, xt[f + 1].x, su.x, sb.x, 0.f,
                             0.f, 0.0, fxh[f].x, fxb[f].x);
          eval_face<D, FLUX>(eb, MX.lane(1), sx.y, xs[f + 1].y, xt[f + 1].y, su.y, sb.y, 0.f,
                             0.f, 0.0, fxh[f].y, fxb[f].y);
          continue;
        }
        const float4* cp = pxa ? &xc[cg + f].Cp : &xc[cg + f].Cm;
        e.C = cp[0];
        e.Dd = cp[1];
      }
      float2 hc = f2s(0.f), bc = f2s(0.f);
      if (!FAST) {
        hc = Hp(Sj, cg + (fi == 0 ? f + 2 : f + 1));
        bc = Bp(Sj, cg + (fi == 0 ? f + 2 : f + 1));
      }
      eval_face2<D, FLUX, FAST>(e, MX, sx, xs[f + 1], xt[f + 1], su, sb, hc, bc, fxh[f], fxb[f]);
    }
    const CellCoef32* cc = (const CellCoef32*)(cslot(j) + L::CC);
    const long ro = (long)(j + g.ngy) * rowstride + (long)(i0 + g.ngx) * vs + va;
#pragma unroll
    for (int c = 0; c < TXG; ++c) {
      if (!FAST && cg + c >= ncol) continue;
      const float2 dhh = f2sub(f2add(f2sub(fxh[c], fxh[c + 1]), fyh[c]), fyh2[c]);
      const float2 dbb = f2sub(f2add(f2sub(fxb[c], fxb[c + 1]), fyb[c]), fyb2[c]);
      float2 hn, bn;
      relax2(cc[cg + c], shak, u, vv, MX.c2, Hp(Sj, cg + c + 2), Bp(Sj, cg + c + 2), dhh, dbb,
             hn, bn);
      float* ph = Ho + ro + (long)(cg + c) * vs;
      float* pb = Bo + ro + (long)(cg + c) * vs;
      if (okb) {
        *(float2*)ph = hn;
        *(float2*)pb = bn;
      } else if (oka) {
        ph[0] = hn.x;
        pb[0] = bn.x;
      }
    }
#pragma unroll
    for (int c = 0; c < TXG; ++c) {
      fyh[c] = fyh2[c];
      fyb[c] = fyb2[c];
    }
  };

  const bool fastx = g.interp == 2 && i0 >= 2 && i0 + TX <= g.nx - 2;
  for (int j = j0; j < j1; ++j) {
    if (tid == 0 && *vbad == 0) {
      const int q = j + NS - 2;  // into the slot of row j - 2 (see k_march3)
      if (q <= qend) {
        const int r = q - q0;
        if (mbar_wait(&empty[r % NS], ((r - NS) / NS) & 1)) {
          fence_async_smem();
          issue(q);
          ++issued;
        } else {
          atomicOr(bad, 1);
          atomicOr(s.status, 2);
        }
      }
    }
    await_row(j + 2);
    // warps whose pairs all share their upwind sides run only the packed body
    if (fastx && j >= 1 && j <= g.ny - 3 && same) row(j, std::true_type{}, std::true_type{});
    else row(j, std::false_type{}, std::false_type{});
    release_row(j - 1);
  }
  __syncthreads();
  if (*vbad && tid == 0) {
    for (int r = max(0, issued - NS); r < issued; ++r) mbar_wait(&full[r % NS], (r / NS) & 1);
  }
}

// ----------------------------------------------------------- launch helpers

constexpr int TS_MOM = 4;    // faces per warp in pass A
constexpr int TX_MARCH = 4;  // columns per strip in pass B (FP32)
constexpr int RY_MARCH = 32;

static inline unsigned nblk2(long n, int bs) { return (unsigned)((n + bs - 1) / bs); }

// FP32 pass A: one CTA (4 warps) per segment of 4 TS faces along a line;
// its dynamic shared memory exceeds the default 48 KB for TS = 4, so the
// limit is raised once per device.
template <int D, int FLUX, int TS, bool SHAK, int DIR>
static void mom_st_go(DevState& s, cudaStream_t st) {
  const Geo& g = s.g;
  using SL = MomStage<TS>;
  const int n = DIR == 0 ? g.nx : g.ny, nlines = DIR == 0 ? g.ny : g.nx;
  const long nblk = (long)nlines * ((n + SL::NF - 1) / SL::NF);
  auto kern = k_mom_st<D, FLUX, TS, SHAK, DIR>;
  const CUtensorMap* tm =
      (const CUtensorMap*)s.tmaps + 8 + ((DIR * 2 + (TS == 4 ? 1 : 0)) * 2 + s.cur) * 2;
  static std::once_flag once[64];  // per device; thread-safe for concurrent host threads
  int dev = 0;
  cudaGetDevice(&dev);
  std::call_once(once[dev & 63], [&] {
    if (SL::BYTES > 48 * 1024)
      cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, SL::BYTES);
    cudaFuncSetAttribute(kern, cudaFuncAttributePreferredSharedMemoryCarveout,
                         cudaSharedmemCarveoutMaxShared);
  });
  kern<<<(unsigned)nblk, MOM_THREADS, SL::BYTES, st>>>(tm[0], tm[1], s);
}

template <typename R, int D, int FLUX, int TS>
static int mom_go(DevState& s, cudaStream_t st) {
  const Geo& g = s.g;
  if constexpr (sizeof(R) == 4) {
    if (s.coll == COLL_SHAKHOV) mom_st_go<D, FLUX, TS, true, 0>(s, st);
    else mom_st_go<D, FLUX, TS, false, 0>(s, st);
    if (D == 2) mom_st_go<D, FLUX, TS, false, 1>(s, st);
    return D == 2 ? 2 : 1;
  }
  int n = 0;
  long wx = (long)((g.nx + TS - 1) / TS) * g.ny;
  prefer_max_shared((const void*)k_mom<R, D, FLUX, TS, true, 0>);
  prefer_max_shared((const void*)k_mom<R, D, FLUX, TS, false, 0>);
  prefer_max_shared((const void*)k_mom<R, D, FLUX, TS, false, 1>);
  if (s.coll == COLL_SHAKHOV)
    k_mom<R, D, FLUX, TS, true, 0><<<nblk2(wx * 32, 128), 128, 0, st>>>(s);
  else
    k_mom<R, D, FLUX, TS, false, 0><<<nblk2(wx * 32, 128), 128, 0, st>>>(s);
  ++n;
  if (D == 2) {
    long wy = (long)((g.ny + TS - 1) / TS) * g.nx;
    k_mom<R, D, FLUX, TS, false, 1><<<nblk2(wy * 32, 128), 128, 0, st>>>(s);
    ++n;
  }
  return n;
}

template <typename R, int D, int FLUX>
static int mom_t(DevState& s, cudaStream_t st) {
  // 8: both face directions in one launch over row rings (2D FP32, BGK)
  if (sizeof(R) == 4 && D == 2 && s.tune[KB_TUNE_MOM_TS] == 8 && s.coll == COLL_BGK && s.mpart)
    return moments_ring(s, st);
  if (s.tune[KB_TUNE_MOM_TS] == 2) return mom_go<R, D, FLUX, 2>(s, st);
  return mom_go<R, D, FLUX, TS_MOM>(s, st);
}

template <typename R, int D, int FLUX, int TX, int BS>
static void march_go(DevState& s, double dt, cudaStream_t st) {
  const Geo& g = s.g;
  const int ry = s.tune[KB_TUNE_MARCH_RY] > 0 ? s.tune[KB_TUNE_MARCH_RY] : RY_MARCH;
  dim3 grid((g.nx + TX - 1) / TX, D == 2 ? (g.ny + ry - 1) / ry : 1, (g.nvel + BS - 1) / BS);
  const int smem = sizeof(R) == 4 && D == 2 ? MarchStage<TX>::BYTES : 0;
  prefer_max_shared((const void*)k_march<R, D, FLUX, TX, BS>);
  k_march<R, D, FLUX, TX, BS><<<grid, BS, smem, st>>>(s, dt, ry);
}

// FP32 2D pass B (k_march3): the tensor maps of the current h / b buffers for
// this strip width; the ring needs more than the default 48 KB of shared
// memory, so the limit is raised once per device.
template <int FLUX, int TX, int NS, int G>
static void march3_go(DevState& s, cudaStream_t st) {
  constexpr bool PAIR = G > 0;  // G groups of 64 threads, two velocities each
  const Geo& g = s.g;
  using L = M3Layout<TX, NS>;
  const int ry = s.tune[KB_TUNE_MARCH_RY] > 0 ? s.tune[KB_TUNE_MARCH_RY] : RY_MARCH;
  const CUtensorMap* tm = (const CUtensorMap*)s.tmaps + ((TX == 4 ? 1 : 0) * 2 + s.cur) * 2;
  void (*kern)(CUtensorMap, CUtensorMap, DevState, int);
  if constexpr (PAIR) kern = k_march4<FLUX, TX, NS, G>;
  else kern = k_march3<FLUX, TX, NS>;
  static std::once_flag once[64];  // per device; thread-safe for concurrent host threads
  int dev = 0;
  cudaGetDevice(&dev);
  std::call_once(once[dev & 63], [&] {
    cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, L::BYTES);
    // all of the unified L1 / shared storage as shared memory: the ring is the
    // kernel's only reuse, so residency counts for more than L1 cache
    cudaFuncSetAttribute(kern, cudaFuncAttributePreferredSharedMemoryCarveout,
                         cudaSharedmemCarveoutMaxShared);
  });
  dim3 grid((g.nvel + M3_BS - 1) / M3_BS, (g.nx + TX - 1) / TX, (g.ny + ry - 1) / ry);
  kern<<<grid, PAIR ? M4_THREADS * G : M3_BS, L::BYTES, st>>>(tm[0], tm[1], s, ry);
}

// FP32: the autotuned shapes (TX 2 or 4 columns, 64 or 128 threads);
// FP64: one shape (two columns keep the FP64 update free of spills).
template <typename R, int D, int FLUX>
static int march_t(DevState& s, double dt, cudaStream_t st) {
  if constexpr (sizeof(R) == 8) {
    march_go<R, D, FLUX, 2, 64>(s, dt, st);
  } else {
    const int tx = s.tune[KB_TUNE_MARCH_TX] > 0 ? s.tune[KB_TUNE_MARCH_TX] : TX_MARCH;
    const int bs = s.tune[KB_TUNE_MARCH_BS] > 0 ? s.tune[KB_TUNE_MARCH_BS] : 128;
    if constexpr (D == 2) {
      // bs 64: two velocities per thread, one 64-thread group per strip
      // (k_march4); tx 4 + bs 64 splits the strip between two groups; bs 128:
      // one velocity per thread (k_march3)
      if (bs == 64) {
        if (tx == 2) march3_go<FLUX, 2, 8, 1>(s, st);
        else march3_go<FLUX, 4, 6, 2>(s, st);
      } else {
        if (tx == 2) march3_go<FLUX, 2, 8, 0>(s, st);
        else march3_go<FLUX, 4, 7, 0>(s, st);
      }
    } else {
      if (tx == 2) {
        if (bs == 64) march_go<R, D, FLUX, 2, 64>(s, dt, st);
        else march_go<R, D, FLUX, 2, 128>(s, dt, st);
      } else {
        if (bs == 64) march_go<R, D, FLUX, 4, 64>(s, dt, st);
        else march_go<R, D, FLUX, 4, 128>(s, dt, st);
      }
    }
  }
  return 1;
}

}  // namespace kb

// One precision x flux: the pass A and pass B launchers of both dimensions.
#define KB_MARCH_INSTANCE(R, FLUX, NAME)                                          \
  namespace kb {                                                                \
  int moments_##NAME(DevState& s, cudaStream_t st) {                            \
    return s.g.D == 1 ? mom_t<R, 1, FLUX>(s, st) : mom_t<R, 2, FLUX>(s, st);     \
  }                                                                             \
  int march_##NAME(DevState& s, double dt, cudaStream_t st) {                   \
    return s.g.D == 1 ? march_t<R, 1, FLUX>(s, dt, st) : march_t<R, 2, FLUX>(s, dt, st); \
  }                                                                             \
  }
