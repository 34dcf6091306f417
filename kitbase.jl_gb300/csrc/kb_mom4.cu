// kb_mom4.cu -- pass A of the 2D FP32 step (face moments fw) in one launch
// over row rings, both face directions from one read of h and b.
//
// The two-launch form (k_mom_st, kb_march.cuh) streams every distribution
// twice per step, once along x lines and once along y lines.  This form
// uses the row ring of the pointwise update (k_march4): a CTA owns 128
// velocities of a strip of TX columns and RY rows and marches up the rows;
// rows arrive by TMA (h and b boxes of TX + 4 columns, the x halo included)
// with the rows' face coefficient blocks, and at row j it forms, for its two
// velocities per thread, the free-transport flux moments of the x faces of
// row j and of the y faces between rows j and j + 1 (upwind value plus the
// van Leer slope of the upwind cell, evolve! / flux_kfvs! / flux_kcu! /
// flux_ugks! free-transport part, the same arithmetic as k_mom_st).  The
// 16 per-thread sums of a row (4 moments of 2 x faces and 2 y faces of the
// thread's group) are reduced over the warp's 64 velocities by an FP32
// pairwise warp reduce-scatter and written as one partial per (velocity box,
// warp of the group, face), so no warp waits on another; k_mom_fin then adds
// all partials of a face in double-float in a fixed order (deterministic),
// adds the analytic part of fw and rotates y faces to the global frame.  BGK only: the Shakhov heat flux of the old state stays
// with the two-launch form.
#include <mutex>

#include "kb_march.cuh"

namespace kb {

template <int TX, int NS>
struct MALayout {
  static constexpr int W = TX + 4;
  static constexpr int BOX = W * M3_BS * 4;
  static constexpr int DSLOT = 2 * BOX;  // h box, then b box
  static constexpr int XF = 0;           // x faces of the row [TX + 1]
  static constexpr int YF = (TX + 1) * (int)sizeof(FaceCoef32);  // y faces above the row [TX]
  static constexpr int CSLOT = YF + TX * (int)sizeof(FaceCoef32);
  static constexpr int COEF = NS * DSLOT;
  static constexpr int BARS = COEF + NS * CSLOT;
  static constexpr int BYTES = BARS + 16 * NS + 16;
};

// Warp reduce-scatter of 16 per-lane values: four halving exchanges leave
// lanes 2k and 2k + 1 with the partial of value k over their half of the
// warp, the last exchange completes it.  Plain FP32 pairwise sums (5 levels
// over the warp's 64 velocities); the partials of the velocity boxes and
// warps are then added in double-float by k_mom_fin.
__device__ __forceinline__ float ma_reduce16(const float (&x)[16], int lane) {
  const bool b4 = lane & 16, b3 = lane & 8, b2 = lane & 4, b1 = lane & 2;
  float y[8], z[4], t[2];
#pragma unroll
  for (int k = 0; k < 8; ++k)
    y[k] = (b4 ? x[k + 8] : x[k]) + __shfl_xor_sync(0xffffffffu, b4 ? x[k] : x[k + 8], 16);
#pragma unroll
  for (int k = 0; k < 4; ++k) z[k] = (b3 ? y[k + 4] : y[k]) + __shfl_xor_sync(0xffffffffu, b3 ? y[k] : y[k + 4], 8);
#pragma unroll
  for (int k = 0; k < 2; ++k) t[k] = (b2 ? z[k + 2] : z[k]) + __shfl_xor_sync(0xffffffffu, b2 ? z[k] : z[k + 2], 4);
  const float r = (b1 ? t[1] : t[0]) + __shfl_xor_sync(0xffffffffu, b1 ? t[0] : t[1], 2);
  return r + __shfl_xor_sync(0xffffffffu, r, 1);
}

// Free-transport moments of one face for a velocity pair (k_mom_st's
// per-velocity terms): Th = t3 un hf - t4 un^2 s, hf = hu +- s / 2, and
// (sum w Th, sum w Th un, sum w Th ut, sum w (Th c^2 + Tb)).
__device__ __forceinline__ float4 ma_moments(float t3, float t4, const Mono2& M, float2 side, float2 om,
                                             float2 h0, float2 b0, float2 su, float2 sb) {
  const float2 hf = f2fma(side, su, h0), bf = f2fma(side, sb, b0);
  const float2 a = f2mul(f2s(t3), M.un);
  const float2 c = f2mul(f2s(-t4), M.n2);
  const float2 Th = f2fma(c, su, f2mul(a, hf));
  const float2 Tb = f2fma(c, sb, f2mul(a, bf));
  const float2 wT = f2mul(om, Th);
  const float2 m1 = f2mul(wT, M.un), m2 = f2mul(wT, M.ut);
  const float2 m3 = f2fma(wT, M.c2, f2mul(om, Tb));
  return make_float4(wT.x + wT.y, m1.x + m1.y, m2.x + m2.y, m3.x + m3.y);
}

// G groups of 64 threads (two velocities each) split the strip's TX columns,
// TX / G = 2 columns per group.
template <int TX, int NS, int G>
__global__ void __launch_bounds__(M4_THREADS * G, G == 2 ? 4 : 8)
    k_mom4(const __grid_constant__ CUtensorMap tmh, const __grid_constant__ CUtensorMap tmb,
           DevState s, int RY) {
  static_assert(NS >= 6 && TX / G == 2, "ring of at least 6 rows; two columns per group");
  using L = MALayout<TX, NS>;
  constexpr int TXG = TX / G;
  extern __shared__ __align__(1024) unsigned char smemM[];
  unsigned long long* full = (unsigned long long*)(smemM + L::BARS);
  unsigned long long* empty = full + NS;
  int* bad = (int*)(empty + NS);
  volatile int* vbad = bad;
  const Geo& g = s.g;
  const int tid = threadIdx.x, lane = tid & 31;
  const int grp = tid / M4_THREADS, lt = tid % M4_THREADS, cg = grp * TXG;
  const bool w1 = (lt >> 5) == 1;  // second warp of the group
  const int ck = blockIdx.x, v0 = ck * M3_BS;
  const int va = v0 + 2 * lt, vb = va + 1;
  const bool oka = va < g.nvel, okb = vb < g.nvel;
  const int ia = oka ? va : g.nvel - 1, ib = okb ? vb : g.nvel - 1;
  const int i0 = blockIdx.y * TX;
  const int ncol = min(TX, g.nx - i0);
  const int j0 = blockIdx.z * RY;
  const int j1 = min(g.ny, j0 + RY);
  const int q0 = j0 - 2;
  const int qend = j1 + 1;
  const long nface = (long)s.nface_x + s.nface_y;

  auto slot = [&](int q) -> const unsigned char* { return smemM + ((q - q0) % NS) * L::DSLOT; };
  auto cslot = [&](int q) -> const unsigned char* {
    return smemM + L::COEF + ((q - q0) % NS) * L::CSLOT;
  };
  auto issue = [&](int q) {
    const int r = q - q0;
    unsigned char* S = smemM + (r % NS) * L::DSLOT;
    unsigned char* C = smemM + L::COEF + (r % NS) * L::CSLOT;
    unsigned long long* bar = &full[r % NS];
    const bool hy = q >= j0 - 1 && q <= j1 - 1, hx = q >= j0 && q <= j1 - 1;
    const unsigned xb = (ncol + 1) * sizeof(FaceCoef32), yb = ncol * sizeof(FaceCoef32);
    mbar_expect(bar, 2 * L::BOX + (hy ? yb : 0u) + (hx ? xb : 0u));
    tma_load_3d(S, &tmh, v0, i0 - 2 + g.ngx, q + g.ngy, bar);
    tma_load_3d(S + L::BOX, &tmb, v0, i0 - 2 + g.ngx, q + g.ngy, bar);
    if (hx) bulk_g2s(C + L::XF, s.fc + (long)q * (g.nx + 1) + i0, xb, bar);
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
  const float2 om = make_float2(oka ? s.wtf[ia] : 0.f, okb ? s.wtf[ib] : 0.f);
  Mono2 MX, MY;
  MX.set(u, vv);
  MY.set(vv, make_float2(-u.x, -u.y));
  const bool pxa = u.x >= 0.f, pxb = u.y >= 0.f, pya = vv.x >= 0.f, pyb = vv.y >= 0.f;
  const float2 sx = make_float2(pxa ? 0.5f : -0.5f, pxb ? 0.5f : -0.5f);
  const float2 sy = make_float2(pya ? 0.5f : -0.5f, pyb ? 0.5f : -0.5f);
  const float epsx = float(1.e-7 * g.dx), epsy = float(1.e-7 * g.dy);
  const int sha = pxa ? 0 : 1, shb = pxb ? 0 : 1;
  const bool samex = sha == shb, samey = pya == pyb;
  int rxa[TXG + 3], rxb[TXG + 3];
#pragma unroll
  for (int k = 0; k < TXG + 3; ++k) {
    rxa[k] = slope_rule(g, 0, i0 - 2 + cg + k + sha);
    rxb[k] = slope_rule(g, 0, i0 - 2 + cg + k + shb);
  }
  auto Hp = [&](const unsigned char* S, int w) {
    return *(const float2*)((const float*)S + w * M3_BS + 2 * lt);
  };
  auto Bp = [&](const unsigned char* S, int w) {
    return *(const float2*)((const float*)(S + L::BOX) + w * M3_BS + 2 * lt);
  };
  auto H2 = [&](const unsigned char* Sa, int wa, const unsigned char* Sb, int wb) {
    return make_float2(((const float*)Sa)[wa * M3_BS + 2 * lt], ((const float*)Sb)[wb * M3_BS + 2 * lt + 1]);
  };
  auto B2 = [&](const unsigned char* Sa, int wa, const unsigned char* Sb, int wb) {
    return make_float2(((const float*)(Sa + L::BOX))[wa * M3_BS + 2 * lt],
                       ((const float*)(Sb + L::BOX))[wb * M3_BS + 2 * lt + 1]);
  };

  // moments of the y face above row ql in column c of the group
  auto yface = [&](int ql, int c, auto fast_tag, auto same_tag) -> float4 {
    constexpr bool FAST = decltype(fast_tag)::value;
    constexpr bool SAME = decltype(same_tag)::value;
    if (!FAST && cg + c >= ncol) return make_float4(0.f, 0.f, 0.f, 0.f);
    const int w = cg + c + 2;
    const int qa = pya ? ql - 1 : ql, qb = pyb ? ql - 1 : ql;
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
    const float4 T = ((const FaceCoef32*)(cslot(ql) + L::YF))[cg + c].T;
    return ma_moments(T.x, T.y, MY, sy, om, h0, b0, su, sb);
  };
  // moments of x face f (0 .. TXG) of the group in row j, window xs / xt
  auto xface = [&](int f, const float2* xs, const float2* xt, const FaceCoef32* xc,
                   auto fast_tag) -> float4 {
    constexpr bool FAST = decltype(fast_tag)::value;
    float2 su, sb;
    if (FAST) {
      su = vl2(xs[f], xs[f + 1], xs[f + 2], epsx);
      sb = vl2(xt[f], xt[f + 1], xt[f + 2], epsx);
    } else {
      su = slope2(rxa[f + 1], rxb[f + 1], xs[f], xs[f + 1], xs[f + 2], epsx);
      sb = slope2(rxa[f + 1], rxb[f + 1], xt[f], xt[f + 1], xt[f + 2], epsx);
    }
    const float4 T = xc[cg + f].T;
    return ma_moments(T.x, T.y, MX, sx, om, xs[f + 1], xt[f + 1], su, sb);
  };

  // reduce a warp's 16 row values over its 64 velocities and write the
  // owned faces' partials (one per warp: velocity box ck, half w1): values
  // 4 f + m (x faces f = 0, 1 of row jx) and 8 + 4 c + m (y faces of y-face
  // row yr, i.e. between grid rows yr - 1 and yr, columns c); jx < 0 or
  // yr < 0: none.  No warp waits on another.
  float2* __restrict__ mypart = s.mpart + ((long)ck * 2 + (w1 ? 1 : 0)) * nface * 4;
  auto flush = [&](const float (&x)[16], int jx, int yr) {
    const float r = ma_reduce16(x, lane);
    const int k = lane >> 1, m = k & 3;
    if ((lane & 1) == 0) {
      long f = -1;
      if (k < 8) {
        const int col = cg + (k >> 2);
        if (jx >= 0 && col < ncol) f = (long)jx * (g.nx + 1) + i0 + col;
      } else {
        const int col = cg + ((k - 8) >> 2);
        if (yr >= 0 && col < ncol) f = s.nface_x + (long)yr * g.nx + i0 + col;
      }
      if (f >= 0) mypart[f * 4 + m] = make_float2(r, 0.f);
    }
  };
  // the grid's last x face (i = nx), owned by the group holding column nx - 1
  const bool has_last = i0 + ncol == g.nx && cg < ncol && cg + TXG >= ncol;
  auto flush_last = [&](float4 o4, int j) {
    float x[16];
#pragma unroll
    for (int k = 4; k < 16; ++k) x[k] = 0.f;
    x[0] = o4.x;
    x[1] = o4.y;
    x[2] = o4.z;
    x[3] = o4.w;
    const float r = ma_reduce16(x, lane);
    const int k = lane >> 1;
    if ((lane & 1) == 0 && k < 4) mypart[((long)j * (g.nx + 1) + g.nx) * 4 + k] = make_float2(r, 0.f);
  };

  await_row(q0);
  await_row(q0 + 1);
  await_row(q0 + 2);
  await_row(q0 + 3);
  const bool same = samex && samey;
  {
    // the y faces between rows j0 - 1 and j0
    const bool fast = g.interp == 2 && i0 >= 2 && i0 + TX <= g.nx - 2 && j0 >= 2 && j0 <= g.ny - 2;
    float x[16];
#pragma unroll
    for (int k = 0; k < 8; ++k) x[k] = 0.f;
#pragma unroll
    for (int c = 0; c < TXG; ++c) {
      const float4 y = fast && same ? yface(j0 - 1, c, std::true_type{}, std::true_type{})
                                    : yface(j0 - 1, c, std::false_type{}, std::false_type{});
      x[8 + 4 * c] = y.x;
      x[9 + 4 * c] = y.y;
      x[10 + 4 * c] = y.z;
      x[11 + 4 * c] = y.w;
    }
    flush(x, -1, j0);
  }
  release_row(q0);

  auto row = [&](int j, auto fast_tag, auto same_tag) {
    constexpr bool FAST = decltype(fast_tag)::value;
    constexpr bool SAME = decltype(same_tag)::value;
    const unsigned char* Sj = slot(j);
    float x[16];
#pragma unroll
    for (int c = 0; c < TXG; ++c) {
      const float4 y = yface(j, c, fast_tag, same_tag);
      x[8 + 4 * c] = y.x;
      x[9 + 4 * c] = y.y;
      x[10 + 4 * c] = y.z;
      x[11 + 4 * c] = y.w;
    }
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
#pragma unroll
    for (int f = 0; f < TXG; ++f) {
      const float4 o = (!FAST && cg + f >= ncol) ? make_float4(0.f, 0.f, 0.f, 0.f)
                                                 : xface(f, xs, xt, xc, fast_tag);
      x[4 * f] = o.x;
      x[4 * f + 1] = o.y;
      x[4 * f + 2] = o.z;
      x[4 * f + 3] = o.w;
    }
    // the y faces above row j belong to this block when row j + 1 does, or
    // when they are the grid's top faces
    flush(x, j, (j + 1 < j1 || j + 1 == g.ny) ? j + 1 : -1);
    if (!FAST && has_last) {  // face index ncol - cg, 1 or 2 (compile-time window offsets)
      const float4 o = ncol - cg == 1 ? xface(1, xs, xt, xc, std::false_type{})
                                      : xface(2, xs, xt, xc, std::false_type{});
      flush_last(o, j);
    }
  };

  const bool fastx = g.interp == 2 && i0 >= 2 && i0 + TX <= g.nx - 2;
  for (int j = j0; j < j1; ++j) {
    if (tid == 0 && *vbad == 0) {
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
    if (fastx && j >= 1 && j <= g.ny - 3 && same && !has_last) row(j, std::true_type{}, std::true_type{});
    else row(j, std::false_type{}, std::false_type{});
    release_row(j - 1);
  }
  __syncthreads();
  if (*vbad && tid == 0) {
    for (int r = max(0, issued - NS); r < issued; ++r) mbar_wait(&full[r % NS], (r / NS) & 1);
  }
}

// fw of every interior face: the analytic part plus the partials of all
// velocity boxes in box order, y faces rotated to the global frame
// (global_frame with n = (0, 1)).
__global__ void k_mom_fin(DevState s, int nchunk) {
  const long nface = (long)s.nface_x + s.nface_y;
  const long f = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (f >= nface || s.kind[f] != 1) return;
  DF a[4];
#pragma unroll
  for (int m = 0; m < 4; ++m) a[m].hi = a[m].lo = 0.f;
  for (int k = 0; k < 2 * nchunk; ++k) {  // box k / 2, half k % 2
    const float4* p = (const float4*)(s.mpart + ((long)k * nface + f) * 4);
    const float4 x = p[0], y = p[1];
    DF d;
    d.hi = x.x; d.lo = x.y; a[0] = df_merge(a[0], d);
    d.hi = x.z; d.lo = x.w; a[1] = df_merge(a[1], d);
    d.hi = y.x; d.lo = y.y; a[2] = df_merge(a[2], d);
    d.hi = y.z; d.lo = y.w; a[3] = df_merge(a[3], d);
  }
  const FaceParam& P = s.fp[f];
  const double S0 = (double)a[0].hi + a[0].lo, S1 = (double)a[1].hi + a[1].lo;
  const double S2 = (double)a[2].hi + a[2].lo, S3 = (double)a[3].hi + a[3].lo;
  const double fl0 = P.fwa[0] + S0, fl1 = P.fwa[1] + S1, fl2 = P.fwa[2] + S2;
  const double fl3 = P.fwa[3] + 0.5 * S3;
  double* out = s.fw + f * 4;
  if (f >= s.nface_x) {
    out[0] = fl0;
    out[1] = -fl2;
    out[2] = fl1;
    out[3] = fl3;
  } else {
    out[0] = fl0;
    out[1] = fl1;
    out[2] = fl2;
    out[3] = fl3;
  }
}

// Pass A in the row-ring form: the TMA maps of the update pass for 4-column
// strips (box 128 velocities x 8 columns x 1 row), RY rows per CTA.
int moments_ring(DevState& s, cudaStream_t st) {
  constexpr int TX = 4, NS = 6, G = 2;
  using L = MALayout<TX, NS>;
  const Geo& g = s.g;
  const int ry = s.tune[KB_TUNE_MARCH_RY] > 0 ? s.tune[KB_TUNE_MARCH_RY] : 64;
  const CUtensorMap* tm = (const CUtensorMap*)s.tmaps + (1 * 2 + s.cur) * 2;
  auto kern = k_mom4<TX, NS, G>;
  static std::once_flag once[64];
  int dev = 0;
  cudaGetDevice(&dev);
  std::call_once(once[dev & 63], [&] {
    cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, L::BYTES);
    cudaFuncSetAttribute(kern, cudaFuncAttributePreferredSharedMemoryCarveout,
                         cudaSharedmemCarveoutMaxShared);
  });
  prefer_max_shared((const void*)k_mom_fin);
  const int nchunk = (g.nvel + M3_BS - 1) / M3_BS;
  dim3 grid(nchunk, (g.nx + TX - 1) / TX, (g.ny + ry - 1) / ry);
  kern<<<grid, M4_THREADS * G, L::BYTES, st>>>(tm[0], tm[1], s, ry);
  const long nface = (long)s.nface_x + s.nface_y;
  k_mom_fin<<<(unsigned)((nface + 255) / 256), 256, 0, st>>>(s, nchunk);
  return 2;
}

}  // namespace kb
