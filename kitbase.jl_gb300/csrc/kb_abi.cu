// kb_abi.cu -- extern "C" entry points of libkitgpu (declared in include/kitgpu.h).
//
// A handle owns its device buffers and one CUDA stream.  Distributions live in
// HBM in the layout of kb_device.cuh and stay resident across calls; only
// kb_upload_state / kb_download_state move them across PCIe / C2C.
#include <cuda.h>
#include <cudaTypedefs.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/kitgpu.h"
#include "kb_handle.h"
#include "kb_kernels.cuh"

using kb::DevState;
using kb::Geo;



static thread_local std::string g_err;

static int fail(int code, const std::string& msg) {
  g_err = msg;
  return code;
}

void kb::set_error(const std::string& msg) { g_err = msg; }

// Encode the TMA descriptors of the FP32 form: each distribution buffer is a
// 3D tensor (velocity, column, row) incl. ghosts.  Update-pass boxes are 128
// velocities x (strip width + 4) columns x 1 row; moment-pass boxes are 128
// velocities x (4 x faces per warp + 4) cells along x or along y.  Coordinates
// outside the tensor read as zero, which is what both passes expect beyond the
// grid.
static int make_tmaps(kb_handle* h) {
  void* fn = nullptr;
  cudaDriverEntryPointQueryResult q;
  if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &fn, 12000, cudaEnableDefault,
                                       &q) != cudaSuccess ||
      q != cudaDriverEntryPointSuccess || !fn)
    return fail(KB_ERR_CUDA, "cuTensorMapEncodeTiled is not available from the driver");
  auto encode = (PFN_cuTensorMapEncodeTiled_v12000)fn;
  const Geo& g = h->s.g;
  const cuuint64_t dims[3] = {(cuuint64_t)g.vstride, (cuuint64_t)g.nxt, (cuuint64_t)g.nyt};
  const cuuint64_t strides[2] = {(cuuint64_t)g.vstride * 4, (cuuint64_t)g.vstride * 4 * g.nxt};
  const cuuint32_t estr[3] = {1, 1, 1};
  auto make = [&](int idx, const cuuint32_t* box, int k, int d) {
    CUresult r = encode(&h->tmaps[idx], CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 3,
                        d == 0 ? h->s.h[k] : h->s.b[k], dims, strides, box, estr,
                        CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
                        CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    return r == CUDA_SUCCESS;
  };
  bool ok = true;
  for (int t = 0; t < 2 && g.D == 2; ++t) {
    const cuuint32_t box[3] = {kb::KB_TMA_VBOX, (cuuint32_t)(t == 0 ? 2 + 4 : 4 + 4), 1};
    for (int k = 0; k < 2; ++k)
      for (int d = 0; d < 2; ++d) ok = ok && make((t * 2 + k) * 2 + d, box, k, d);
  }
  for (int dir = 0; dir < g.D; ++dir)
    for (int t = 0; t < 2; ++t) {
      const cuuint32_t nwin = 4 * (t == 0 ? 2 : 4) + 4;
      const cuuint32_t box[3] = {kb::KB_TMA_VBOX, dir == 0 ? nwin : 1u, dir == 0 ? 1u : nwin};
      for (int k = 0; k < 2; ++k)
        for (int d = 0; d < 2; ++d) ok = ok && make(8 + ((dir * 2 + t) * 2 + k) * 2 + d, box, k, d);
    }
  if (!ok) return fail(KB_ERR_CUDA, "cuTensorMapEncodeTiled failed");
  h->s.tmaps = &h->tmaps[0];
  return KB_OK;
}

#define KB_CUDA(call)                                                                   \
  do {                                                                                  \
    cudaError_t e_ = (call);                                                            \
    if (e_ != cudaSuccess)                                                              \
      return fail(KB_ERR_CUDA, std::string(#call) + ": " + cudaGetErrorString(e_));    \
  } while (0)

static int dev_alloc(kb_handle* h, void** p, size_t bytes) {
  if (bytes == 0) bytes = 16;
  cudaError_t e = cudaMalloc(p, bytes);
  if (e != cudaSuccess) {
    cudaGetLastError();
    return fail(KB_ERR_NOMEM, std::string("cudaMalloc(") + std::to_string(bytes) +
                                  " bytes): " + cudaGetErrorString(e));
  }
  h->allocs.push_back(*p);
  h->bytes += (int64_t)bytes;
  return KB_OK;
}

#define KB_TRY(x)               \
  do {                          \
    int r_ = (x);               \
    if (r_ != KB_OK) return r_; \
  } while (0)

static int check_launch(kb_handle* h, int n) {
  h->launches += n;
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return fail(KB_ERR_CUDA, std::string("kernel launch: ") + cudaGetErrorString(e));
  return KB_OK;
}

static int sync(kb_handle* h) {
  cudaError_t e = cudaStreamSynchronize(h->stream);
  if (e != cudaSuccess) return fail(KB_ERR_CUDA, std::string("stream sync: ") + cudaGetErrorString(e));
  return KB_OK;
}

extern "C" {

const char* kb_version(void) { return "kitgpu 0.1.0 (sm_103a)"; }

const char* kb_last_error(void) { return g_err.c_str(); }

static int validate(const kb_config_t* c) {
  if (c->dim != 1 && c->dim != 2) return fail(KB_ERR_CONFIG, "dim must be 1 or 2");
  if (c->nx < 3) return fail(KB_ERR_CONFIG, "nx must be >= 3");
  if (c->dim == 2 && c->ny < 3) return fail(KB_ERR_CONFIG, "ny must be >= 3 in 2D");
  if (c->nu < 1 || (c->dim == 2 && c->nv < 1)) return fail(KB_ERR_CONFIG, "empty velocity grid");
  if (c->ngx < 0 || c->ngx > 2 || (c->dim == 2 && (c->ngy < 0 || c->ngy > 2)))
    return fail(KB_ERR_CONFIG, "ghost layers must be in [0, 2]");
  if (c->flux < 0 || c->flux > 2) return fail(KB_ERR_CONFIG, "unknown flux");
  if (c->nf < 0 || c->nf > 2) return fail(KB_ERR_CONFIG, "nf must be 1 (1F) or 2 (2F)");
  if (c->nf == 1 && c->flux == KB_FLUX_UGKS)
    return fail(KB_ERR_CONFIG, "the 1F models take KFVS or KCU (the reference has no 1F UGKS step)");
  if (c->nf == 1 && c->dim == 1 && (c->bc[0] == KB_BC_MAXWELL || c->bc[1] == KB_BC_MAXWELL))
    return fail(KB_ERR_CONFIG,
                "1D1F1V has no Maxwell wall in the reference (evolve_boundary! covers the 2F "
                "cells only, src/Solver/evolve_boundary.jl:4-47)");
  if (c->nf == 1 && c->dim == 2 && c->collision == KB_COLL_SHAKHOV)
    return fail(KB_ERR_CONFIG,
                "2D1F2V runs BGK only: the reference's Shakhov branch of its step! reads an "
                "undefined b (src/Solver/step_1f.jl:194)");
  if (c->collision < 0 || c->collision > 1) return fail(KB_ERR_CONFIG, "unknown collision");
  if (c->interp_order != 1 && c->interp_order != 2)
    return fail(KB_ERR_CONFIG, "interp_order must be 1 or 2");
  if (c->precision != KB_PREC_FP64 && c->precision != KB_PREC_FP32)
    return fail(KB_ERR_CONFIG, "unknown precision");
  int nside = 2 * c->dim;
  for (int k = 0; k < nside; ++k)
    if (c->bc[k] < 0 || c->bc[k] > 3) return fail(KB_ERR_CONFIG, "unknown boundary condition");
  if (c->dim == 1) {
    for (int k = 0; k < 2; ++k)
      if ((c->bc[k] == KB_BC_EXTRA || c->bc[k] == KB_BC_PERIOD) && c->ngx < 1)
        return fail(KB_ERR_CONFIG,
                    "extra / period boundaries need ghost cells (nxg >= 1): without them the "
                    "reference steps the boundary cells with never-computed faces");
    if ((c->bc[0] == KB_BC_PERIOD) != (c->bc[1] == KB_BC_PERIOD))
      return fail(KB_ERR_CONFIG, "period must be set on both sides");
  } else {
    for (int k = 1; k < 4; ++k)
      if (c->bc[k] != c->bc[0])
        return fail(KB_ERR_CONFIG, "2D boundaries must be the same on all four sides");
    if (c->bc[0] == KB_BC_PERIOD)
      return fail(KB_ERR_CONFIG,
                  "2D period is not supported: the reference fills only the left / bottom "
                  "ghost layers (src/Boundary/bc_period.jl:25-40)");
    if (c->bc[0] == KB_BC_EXTRA && (c->ngx < 1 || c->ngy < 1))
      return fail(KB_ERR_CONFIG, "extra boundaries need ghost cells (nxg, nyg >= 1)");
  }
  if (!(c->x1 > c->x0) || (c->dim == 2 && !(c->y1 > c->y0)))
    return fail(KB_ERR_CONFIG, "empty physical domain");
  if (!(c->gamma > 1.0) || !(c->mu_ref > 0.0) || c->K < 0.0)
    return fail(KB_ERR_CONFIG, "invalid gas properties");
  return KB_OK;
}

int kb_create(const kb_config_t* cfg, const double* u, const double* v, const double* weights,
              kb_handle_t** out) {
  if (!cfg || !u || !weights || !out) return fail(KB_ERR_ARG, "kb_create: null argument");
  if (cfg->dim == 2 && !v) return fail(KB_ERR_ARG, "kb_create: v table required in 2D");
  KB_TRY(validate(cfg));
  kb_handle* h = new kb_handle();
  h->cfg = *cfg;
  if (h->cfg.dim == 1) {
    h->cfg.ny = 1;
    h->cfg.ngy = 0;
    h->cfg.nv = 1;
  }
  const kb_config_t& c = h->cfg;
  Geo& g = h->s.g;
  g.D = c.dim;
  g.NW = c.dim + 2;
  g.nx = c.nx;
  g.ny = c.ny;
  g.ngx = c.ngx;
  g.ngy = c.ngy;
  g.nxt = c.nx + 2 * c.ngx;
  g.nyt = c.dim == 2 ? c.ny + 2 * c.ngy : 1;
  g.nu = c.nu;
  g.nvel = c.nu * c.nv;
  g.vstride = (g.nvel + 3) / 4 * 4;
  g.interp = c.interp_order;
  for (int k = 0; k < 4; ++k) g.bc[k] = k < 2 * c.dim ? c.bc[k] : KB_BC_FIX;
  g.dx = (c.x1 - c.x0) / c.nx;
  g.dy = c.dim == 2 ? (c.y1 - c.y0) / c.ny : 1.0;
  g.x0 = c.x0;
  g.y0 = c.dim == 2 ? c.y0 : 0.0;
  g.K = c.K;
  g.nf = c.nf == 1 ? 1 : 2;
  g.Kb = g.nf == 1 ? 0.0 : c.K;
  g.gamma = c.gamma;
  g.mu_ref = c.mu_ref;
  g.omega = c.omega;
  g.Pr = c.Pr;
  h->nvel = g.nvel;
  h->vstride = g.vstride;
  h->ncell = (long)g.nxt * g.nyt;
  h->s.ncell = (int)h->ncell;
  h->s.nface_x = (c.nx + 1) * g.ny;
  h->s.nface_y = c.dim == 2 ? c.nx * (c.ny + 1) : 0;
  h->nface = h->s.nface_x + h->s.nface_y;
  h->s.prec = c.precision;
  h->s.flux = c.flux;
  h->s.coll = c.collision;
  h->s.cur = 0;
  {
    // GB300 runs FP64 at a small fraction of its FP32 rate, and the cell
    // parameters are FP64 work per cell: a grid with fewer than two full
    // 256-thread blocks per multiprocessor spreads its cells one warp per
    // block so that more FP64 pipes share them (the block count also fixes
    // the order of the residual's partial sums)
    int dev = 0, sms = 1;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    h->s.sm_count = sms > 0 ? sms : 1;
    const long cells = (long)c.nx * g.ny;
    h->s.cell_bs = cells < 2L * h->s.sm_count * 256 ? 32 : 256;
    h->s.res_blocks = (int)((cells + h->s.cell_bs - 1) / h->s.cell_bs);
  }
  for (int k = 0; k < kb::TUNE_N; ++k) h->s.tune[k] = 0;

  int rc = KB_OK;
  auto bail = [&](int r) {
    kb_destroy(h);
    return r;
  };
  if (cudaGetDevice(&h->device) != cudaSuccess) return bail(fail(KB_ERR_CUDA, "no CUDA device"));
  if (cudaStreamCreateWithFlags(&h->stream, cudaStreamNonBlocking) != cudaSuccess)
    return bail(fail(KB_ERR_CUDA, "cudaStreamCreate failed"));

  size_t esz = c.precision == KB_PREC_FP64 ? 8 : 4;
  size_t dist = (size_t)h->ncell * g.vstride * esz;
  void* p;
#define ALLOC(ptr, type, n)                                        \
  if ((rc = dev_alloc(h, &p, sizeof(type) * (size_t)(n))) != KB_OK) \
    return bail(rc);                                               \
  ptr = (type*)p;
  ALLOC(h->s.u, double, g.vstride);
  ALLOC(h->s.v, double, g.vstride);
  ALLOC(h->s.wt, double, g.vstride);
  ALLOC(h->s.uf, float, g.vstride);
  ALLOC(h->s.vf, float, g.vstride);
  ALLOC(h->s.wtf, float, g.vstride);
  for (int k = 0; k < 2; ++k) {
    if ((rc = dev_alloc(h, &h->s.h[k], dist)) != KB_OK) return bail(rc);
    if ((rc = dev_alloc(h, &h->s.b[k], dist)) != KB_OK) return bail(rc);
    cudaMemset(h->s.h[k], 0, dist);
    cudaMemset(h->s.b[k], 0, dist);
  }
  ALLOC(h->s.w, double, h->ncell * 4);
  ALLOC(h->s.prim, double, h->ncell * 4);
  ALLOC(h->s.sw, double, h->ncell * 8);
  ALLOC(h->s.fp, kb::FaceParam, h->nface);
  ALLOC(h->s.fpf, kb::FaceParamF, h->nface);
  ALLOC(h->s.fw, double, (size_t)h->nface * 4);
  ALLOC(h->s.wall, double, (size_t)h->nface * 4);
  ALLOC(h->s.rhow, double, h->nface);
  ALLOC(h->s.kind, signed char, h->nface);
  ALLOC(h->s.q, double, h->ncell * 2);
  ALLOC(h->s.cp, kb::CellParam, h->ncell);
  ALLOC(h->s.cpf, kb::CellParamF, h->ncell);
  ALLOC(h->s.fc, kb::FaceCoef32, h->nface);
  ALLOC(h->s.cc, kb::CellCoef32, h->ncell);
  ALLOC(h->s.blockres, double, (size_t)h->s.res_blocks * 16);
  h->s.mpart = nullptr;
  h->s.grp = nullptr;
  if (c.precision == KB_PREC_FP32 && g.D == 2) {
    const size_t nbox = (size_t)(g.nvel + kb::KB_TMA_VBOX - 1) / kb::KB_TMA_VBOX;
    ALLOC(h->s.mpart, float2, 2 * nbox * h->nface * 4);  // two warps per face and box
  }
  ALLOC(h->s.residual, double, 4);
  ALLOC(h->s.status, int, 1);
  ALLOC(h->d_scalar, double, 8);
  h->stage_elems = std::min<long>(h->ncell * (long)g.nvel, 32L << 20);
  h->stage_elems = std::max<long>(h->stage_elems, h->ncell * 4);
  ALLOC(h->d_stage, double, h->stage_elems);
#undef ALLOC
  h->s.tmaps = nullptr;
  if (c.precision == KB_PREC_FP32 && (rc = make_tmaps(h)) != KB_OK) return bail(rc);
  cudaMemset(h->s.sw, 0, sizeof(double) * h->ncell * 8);
  cudaMemset(h->s.q, 0, sizeof(double) * h->ncell * 2);
  cudaMemset(h->s.w, 0, sizeof(double) * h->ncell * 4);
  cudaMemset(h->s.prim, 0, sizeof(double) * h->ncell * 4);
  cudaMemset(h->s.fw, 0, sizeof(double) * h->nface * 4);
  cudaMemset(h->s.wall, 0, sizeof(double) * h->nface * 4);
  cudaMemset(h->s.rhow, 0, sizeof(double) * h->nface);
  cudaMemset(h->s.status, 0, sizeof(int));
  cudaMemset(h->s.fc, 0, sizeof(kb::FaceCoef32) * h->nface);
  cudaMemset(h->s.cc, 0, sizeof(kb::CellCoef32) * h->ncell);
  cudaMemset(h->s.fp, 0, sizeof(kb::FaceParam) * h->nface);
  cudaMemset(h->s.residual, 0, sizeof(double) * 4);

  // velocity tables (padded entries have zero weight)
  std::vector<double> hu(g.vstride, 0.0), hv(g.vstride, 0.0), hw(g.vstride, 0.0);
  std::vector<float> fu(g.vstride, 0.f), fv(g.vstride, 0.f), fw(g.vstride, 0.f);
  for (int k = 0; k < g.nvel; ++k) {
    hu[k] = u[k];
    hv[k] = c.dim == 2 ? v[k] : 0.0;
    hw[k] = weights[k];
    fu[k] = (float)hu[k];
    fv[k] = (float)hv[k];
    fw[k] = (float)hw[k];
  }
  if (cudaMemcpy((void*)h->s.u, hu.data(), sizeof(double) * g.vstride, cudaMemcpyHostToDevice) ||
      cudaMemcpy((void*)h->s.v, hv.data(), sizeof(double) * g.vstride, cudaMemcpyHostToDevice) ||
      cudaMemcpy((void*)h->s.wt, hw.data(), sizeof(double) * g.vstride, cudaMemcpyHostToDevice) ||
      cudaMemcpy((void*)h->s.uf, fu.data(), sizeof(float) * g.vstride, cudaMemcpyHostToDevice) ||
      cudaMemcpy((void*)h->s.vf, fv.data(), sizeof(float) * g.vstride, cudaMemcpyHostToDevice) ||
      cudaMemcpy((void*)h->s.wtf, fw.data(), sizeof(float) * g.vstride, cudaMemcpyHostToDevice))
    return bail(fail(KB_ERR_CUDA, "velocity table upload failed"));
  std::vector<signed char> kinds(h->nface);
  kb::face_kinds_host(g, kinds.data());
  if (cudaMemcpy(h->s.kind, kinds.data(), h->nface, cudaMemcpyHostToDevice) != cudaSuccess)
    return bail(fail(KB_ERR_CUDA, "face kind upload failed"));
  {
    // the wall faces, one CTA each in k_wall
    std::vector<int> walls;
    for (int f = 0; f < h->nface; ++f)
      if (kinds[f] == 2) walls.push_back(f);
    h->s.nwall = (int)walls.size();
    h->s.wall_list = nullptr;
    if (!walls.empty()) {
      if ((rc = dev_alloc(h, &p, sizeof(int) * walls.size())) != KB_OK) return bail(rc);
      h->s.wall_list = (int*)p;
      if (cudaMemcpy(h->s.wall_list, walls.data(), sizeof(int) * walls.size(), cudaMemcpyHostToDevice) !=
          cudaSuccess)
        return bail(fail(KB_ERR_CUDA, "wall face list upload failed"));
    }
  }
  // the set-up copies above are synchronous; wait for this handle's stream
  // only, so that creating a handle never waits for other solves' work
  if (cudaStreamSynchronize(h->stream) != cudaSuccess || cudaGetLastError() != cudaSuccess)
    return bail(fail(KB_ERR_CUDA, "init failed"));
  *out = h;
  return KB_OK;
}

int kb_destroy(kb_handle_t* h) {
  if (!h) return KB_OK;
  if (h->stream) cudaStreamSynchronize(h->stream);
  for (cudaEvent_t e : h->events) cudaEventDestroy(e);
  if (h->ev_done) cudaEventDestroy(h->ev_done);
  for (int k = 0; k < 2; ++k) {
    if (h->agraph[k]) cudaGraphExecDestroy(h->agraph[k]);
    if (h->sgraph[k]) cudaGraphExecDestroy(h->sgraph[k]);
  }
  if (h->h_res) cudaFreeHost(h->h_res);
  for (void* p : h->allocs) cudaFree(p);
  if (h->stream) cudaStreamDestroy(h->stream);
  delete h;
  return KB_OK;
}

int kb_set_wall(kb_handle_t* h, int side, const double* host_prim) {
  if (!h || !host_prim) return fail(KB_ERR_ARG, "kb_set_wall: null argument");
  const Geo& g = h->s.g;
  if (side < 0 || side >= 2 * g.D) return fail(KB_ERR_ARG, "kb_set_wall: side out of range");
  int n = side < 2 ? g.ny : g.nx;
  std::vector<double> buf((size_t)h->nface * 4);
  KB_CUDA(cudaMemcpy(buf.data(), h->s.wall, sizeof(double) * buf.size(), cudaMemcpyDeviceToHost));
  for (int q = 0; q < n; ++q) {
    int f;
    if (side == 0) f = q * (g.nx + 1);
    else if (side == 1) f = q * (g.nx + 1) + g.nx;
    else if (side == 2) f = h->s.nface_x + q;
    else f = h->s.nface_x + g.ny * g.nx + q;
    for (int k = 0; k < 4; ++k) buf[(size_t)f * 4 + k] = k < g.NW ? host_prim[q * g.NW + k] : 0.0;
    if (!(host_prim[q * g.NW + g.NW - 1] > 0.0))
      return fail(KB_ERR_ARG, "kb_set_wall: wall lambda must be positive");
  }
  KB_CUDA(cudaMemcpy(h->s.wall, buf.data(), sizeof(double) * buf.size(), cudaMemcpyHostToDevice));
  return KB_OK;
}

// Device address of page-locked host memory (the host pointer's mapping under
// unified addressing), or null for pageable memory.
static void* device_view(const void* p) {
  cudaPointerAttributes a;
  if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
    cudaGetLastError();
    return nullptr;
  }
  return a.type == cudaMemoryTypeHost ? a.devicePointer : nullptr;
}

// distributions host (double, [ncell][nvel]) <-> device (padded, precision).
// Page-locked host arrays are converted in place by one kernel that reads
// (or writes) them over the host link directly; pageable ones go through the
// device staging buffer in chunks.
static int dist_in(kb_handle* h, void* dst, const double* src) {
  if (const void* dv = device_view(src))
    return check_launch(h, kb::launch_convert_in(dst, h->s.prec, (const double*)dv, h->ncell,
                                                 h->nvel, h->vstride, h->stream));
  long per = std::max<long>(1, h->stage_elems / h->nvel);
  size_t esz = h->s.prec == KB_PREC_FP64 ? 8 : 4;
  for (long c0 = 0; c0 < h->ncell; c0 += per) {
    long n = std::min(per, h->ncell - c0);
    KB_CUDA(cudaMemcpyAsync(h->d_stage, src + c0 * h->nvel, sizeof(double) * n * h->nvel,
                            cudaMemcpyHostToDevice, h->stream));
    char* d = (char*)dst + (size_t)c0 * h->vstride * esz;
    KB_TRY(check_launch(h, kb::launch_convert_in(d, h->s.prec, h->d_stage, n, h->nvel, h->vstride, h->stream)));
  }
  return KB_OK;
}

static int dist_out(kb_handle* h, double* dst, const void* src) {
  if (void* dv = device_view(dst)) {
    KB_TRY(check_launch(h, kb::launch_convert_out((double*)dv, h->s.prec, src, h->ncell, h->nvel,
                                                  h->vstride, h->stream)));
    return sync(h);
  }
  long per = std::max<long>(1, h->stage_elems / h->nvel);
  size_t esz = h->s.prec == KB_PREC_FP64 ? 8 : 4;
  for (long c0 = 0; c0 < h->ncell; c0 += per) {
    long n = std::min(per, h->ncell - c0);
    const char* s = (const char*)src + (size_t)c0 * h->vstride * esz;
    KB_TRY(check_launch(h, kb::launch_convert_out(h->d_stage, h->s.prec, s, n, h->nvel, h->vstride, h->stream)));
    KB_CUDA(cudaMemcpyAsync(dst + c0 * h->nvel, h->d_stage, sizeof(double) * n * h->nvel,
                            cudaMemcpyDeviceToHost, h->stream));
    KB_TRY(sync(h));
  }
  return KB_OK;
}

int kb_upload_state(kb_handle_t* h, const double* w, const double* prim, const double* hdist,
                    const double* bdist) {
  if (!h || !w || !prim || !hdist || (!bdist && h->s.g.nf != 1))
    return fail(KB_ERR_ARG, "kb_upload_state: null argument");
  int NW = h->s.g.NW;
  std::vector<double> w4((size_t)h->ncell * 4, 0.0), p4((size_t)h->ncell * 4, 0.0);
  for (long c = 0; c < h->ncell; ++c)
    for (int k = 0; k < NW; ++k) {
      w4[c * 4 + k] = w[c * NW + k];
      p4[c * 4 + k] = prim[c * NW + k];
    }
  KB_CUDA(cudaMemcpyAsync(h->s.w, w4.data(), sizeof(double) * w4.size(), cudaMemcpyHostToDevice, h->stream));
  KB_CUDA(cudaMemcpyAsync(h->s.prim, p4.data(), sizeof(double) * p4.size(), cudaMemcpyHostToDevice, h->stream));
  KB_CUDA(cudaMemsetAsync(h->s.sw, 0, sizeof(double) * h->ncell * 8, h->stream));
  KB_CUDA(cudaMemsetAsync(h->s.status, 0, sizeof(int), h->stream));
  h->s.cur = 0;
  KB_TRY(dist_in(h, h->s.h[0], hdist));
  if (bdist) {
    KB_TRY(dist_in(h, h->s.b[0], bdist));
  } else {  // 1F: no second distribution
    KB_CUDA(cudaMemsetAsync(h->s.b[0], 0, (size_t)h->ncell * h->vstride * (h->s.prec == KB_PREC_FP64 ? 8 : 4),
                            h->stream));
  }
  // both ping-pong buffers start equal: ghost cells of fix / Maxwell solves are
  // never rewritten, so the second buffer must hold them too
  size_t dist = (size_t)h->ncell * h->vstride * (h->s.prec == KB_PREC_FP64 ? 8 : 4);
  KB_CUDA(cudaMemcpyAsync(h->s.h[1], h->s.h[0], dist, cudaMemcpyDeviceToDevice, h->stream));
  KB_CUDA(cudaMemcpyAsync(h->s.b[1], h->s.b[0], dist, cudaMemcpyDeviceToDevice, h->stream));
  KB_TRY(sync(h));
  h->evolved = false;
  return KB_OK;
}

int kb_init_equilibrium(kb_handle_t* h, const double* w, const double* prim) {
  if (!h || !w || !prim) return fail(KB_ERR_ARG, "kb_init_equilibrium: null argument");
  int NW = h->s.g.NW;
  for (long c = 0; c < h->ncell; ++c)
    if (!(prim[c * NW] > 0.0) || !(prim[c * NW + NW - 1] > 0.0))
      return fail(KB_ERR_ARG, "kb_init_equilibrium: density and lambda must be positive");
  std::vector<double> w4((size_t)h->ncell * 4, 0.0), p4((size_t)h->ncell * 4, 0.0);
  for (long c = 0; c < h->ncell; ++c)
    for (int k = 0; k < NW; ++k) {
      w4[c * 4 + k] = w[c * NW + k];
      p4[c * 4 + k] = prim[c * NW + k];
    }
  KB_CUDA(cudaMemcpyAsync(h->s.w, w4.data(), sizeof(double) * w4.size(), cudaMemcpyHostToDevice, h->stream));
  KB_CUDA(cudaMemcpyAsync(h->s.prim, p4.data(), sizeof(double) * p4.size(), cudaMemcpyHostToDevice, h->stream));
  KB_CUDA(cudaMemsetAsync(h->s.sw, 0, sizeof(double) * h->ncell * 8, h->stream));
  KB_CUDA(cudaMemsetAsync(h->s.status, 0, sizeof(int), h->stream));
  h->s.cur = 0;
  KB_TRY(check_launch(h, kb::launch_init_equilibrium(h->s, h->stream)));
  size_t dist = (size_t)h->ncell * h->vstride * (h->s.prec == KB_PREC_FP64 ? 8 : 4);
  KB_CUDA(cudaMemcpyAsync(h->s.h[1], h->s.h[0], dist, cudaMemcpyDeviceToDevice, h->stream));
  KB_CUDA(cudaMemcpyAsync(h->s.b[1], h->s.b[0], dist, cudaMemcpyDeviceToDevice, h->stream));
  KB_TRY(sync(h));
  h->evolved = false;
  return KB_OK;
}

int kb_download_state(kb_handle_t* h, double* w, double* prim, double* hdist, double* bdist) {
  if (!h) return fail(KB_ERR_ARG, "kb_download_state: null handle");
  int NW = h->s.g.NW;
  KB_TRY(sync(h));
  if (w || prim) {
    std::vector<double> w4((size_t)h->ncell * 4), p4((size_t)h->ncell * 4);
    KB_CUDA(cudaMemcpy(w4.data(), h->s.w, sizeof(double) * w4.size(), cudaMemcpyDeviceToHost));
    KB_CUDA(cudaMemcpy(p4.data(), h->s.prim, sizeof(double) * p4.size(), cudaMemcpyDeviceToHost));
    for (long c = 0; c < h->ncell; ++c)
      for (int k = 0; k < NW; ++k) {
        if (w) w[c * NW + k] = w4[c * 4 + k];
        if (prim) prim[c * NW + k] = p4[c * 4 + k];
      }
  }
  if (hdist) KB_TRY(dist_out(h, hdist, h->s.h[h->s.cur]));
  if (bdist) KB_TRY(dist_out(h, bdist, h->s.b[h->s.cur]));
  return KB_OK;
}

int kb_timestep(kb_handle_t* h, double cfl, double sim_time, double max_time, double* dt_out) {
  if (!h || !dt_out) return fail(KB_ERR_ARG, "kb_timestep: null argument");
  KB_TRY(check_launch(h, kb::launch_timestep(h->s, h->cfg.umax, h->cfg.vmax, h->d_scalar, h->stream)));
  double tmax = 0.0;
  KB_CUDA(cudaMemcpyAsync(&tmax, h->d_scalar, sizeof(double), cudaMemcpyDeviceToHost, h->stream));
  KB_TRY(sync(h));
  double dt = cfl / tmax;
  *dt_out = dt < (max_time - sim_time) ? dt : max_time - sim_time;
  return KB_OK;
}

int kb_reconstruct(kb_handle_t* h) {
  if (!h) return fail(KB_ERR_ARG, "kb_reconstruct: null handle");
  KB_TRY(check_launch(h, kb::launch_reconstruct(h->s, h->stream)));
  return sync(h);
}

int kb_evolve(kb_handle_t* h, double dt) {
  if (!h) return fail(KB_ERR_ARG, "kb_evolve: null handle");
  if (!(dt > 0.0)) return fail(KB_ERR_ARG, "kb_evolve: dt must be positive");
  KB_TRY(check_launch(h, kb::launch_evolve(h->s, dt, h->stream)));
  KB_TRY(sync(h));
  h->evolved = true;
  return KB_OK;
}

// Status word of the device state: bit 0 a non-physical state after a step,
// bit 1 a bounded device wait (bulk-copy staging) that gave up.
static int status_error(int st) {
  if (st & 2) return fail(KB_ERR_TIMEOUT, "a device wait for staged coefficients timed out");
  if (st) return fail(KB_ERR_NUMERIC, "non-finite or non-positive density / lambda after a step");
  return KB_OK;
}

static int read_residual(kb_handle* h, double* residual) {
  double r[4];
  int st = 0;
  KB_CUDA(cudaMemcpyAsync(r, h->s.residual, sizeof(r), cudaMemcpyDeviceToHost, h->stream));
  KB_CUDA(cudaMemcpyAsync(&st, h->s.status, sizeof(int), cudaMemcpyDeviceToHost, h->stream));
  KB_TRY(sync(h));
  if (residual)
    for (int k = 0; k < h->s.g.NW; ++k) residual[k] = r[k];
  return status_error(st);
}

int kb_update(kb_handle_t* h, double dt, double* residual) {
  if (!h) return fail(KB_ERR_ARG, "kb_update: null handle");
  if (!h->evolved) return fail(KB_ERR_STATE, "kb_update: call kb_evolve first");
  KB_TRY(check_launch(h, kb::launch_update(h->s, dt, h->stream)));
  h->evolved = false;
  return read_residual(h, residual);
}

// One step as kernel groups with an event after each group (stage k ends at
// event k+1).
static int timed_step(kb_handle* h, double dt, cudaEvent_t* ev) {
  cudaStream_t st = h->stream;
  int n = 0;
  cudaEventRecord(ev[0], st);
  n += kb::launch_reconstruct(h->s, st);
  cudaEventRecord(ev[1], st);
  n += kb::launch_face_param(h->s, dt, st);
  cudaEventRecord(ev[2], st);
  n += kb::launch_moments(h->s, st);
  cudaEventRecord(ev[3], st);
  n += kb::launch_wall(h->s, dt, st);
  cudaEventRecord(ev[4], st);
  n += kb::launch_cell_param(h->s, dt, st);
  cudaEventRecord(ev[5], st);
  n += kb::launch_march(h->s, dt, st);
  cudaEventRecord(ev[6], st);
  n += kb::launch_finish(h->s, st);
  cudaEventRecord(ev[7], st);
  return n;
}

static int enqueue_steps(kb_handle* h, double dt, int nsteps);
static void drop_step_graphs(kb_handle* h);

// Two steps from the current buffer recorded as a CUDA graph for kb_step,
// cached per starting buffer and dt; null when recording failed (the caller
// then steps eagerly).
static cudaGraphExec_t step_pair_graph(kb_handle* h, double dt) {
  const int c = h->s.cur;
  if (h->sgraph_dt != dt) {
    drop_step_graphs(h);
    h->sgraph_dt = dt;
  }
  if (h->sgraph[c]) return h->sgraph[c];
  cudaGraph_t gr = nullptr;
  bool ok = cudaStreamBeginCapture(h->stream, cudaStreamCaptureModeThreadLocal) == cudaSuccess;
  const int n = ok ? enqueue_steps(h, dt, 2) : 0;
  ok = cudaStreamEndCapture(h->stream, &gr) == cudaSuccess && ok;
  h->s.cur = c;  // two recorded steps leave the buffer index where it was
  if (ok && cudaGraphInstantiate(&h->sgraph[c], gr, 0) == cudaSuccess) {
    h->sgraph_launches = n;
  } else {
    h->sgraph[c] = nullptr;
  }
  if (gr) cudaGraphDestroy(gr);
  cudaGetLastError();  // a failed recording only means eager steps
  return h->sgraph[c];
}

int kb_step(kb_handle_t* h, double dt, int32_t nsteps, double* residual) {
  if (!h) return fail(KB_ERR_ARG, "kb_step: null handle");
  if (!(dt > 0.0)) return fail(KB_ERR_ARG, "kb_step: dt must be positive");
  if (nsteps < 0) return fail(KB_ERR_ARG, "kb_step: nsteps must be >= 0");
  if (h->timing) {
    size_t need = (size_t)nsteps * (KB_NSTAGE + 1);
    while (h->events.size() < need) {
      cudaEvent_t e;
      KB_CUDA(cudaEventCreate(&e));
      h->events.push_back(e);
    }
    for (int s = 0; s < nsteps; ++s)
      KB_TRY(check_launch(h, timed_step(h, dt, &h->events[(size_t)s * (KB_NSTAGE + 1)])));
    KB_TRY(sync(h));
    for (int s = 0; s < nsteps; ++s) {
      cudaEvent_t* ev = &h->events[(size_t)s * (KB_NSTAGE + 1)];
      for (int k = 0; k < KB_NSTAGE; ++k) {
        float ms = 0.f;
        KB_CUDA(cudaEventElapsedTime(&ms, ev[k], ev[k + 1]));
        h->stage_ms[k] += ms;
        h->stage_n[k] += 1;
      }
    }
  } else {
    // A long run replays two steps recorded as a CUDA graph: one graph
    // launch per two steps instead of ~16 kernel launches, so small solves
    // are bound by their kernels rather than by launch latency.  The first
    // two steps run eagerly (modules load and function attributes are set
    // outside any capture); results are those of the eager steps, bit for bit.
    int s = 0;
    auto eager = [&]() -> int {
      int n = kb::launch_reconstruct(h->s, h->stream);
      n += kb::launch_evolve(h->s, dt, h->stream);
      n += kb::launch_update(h->s, dt, h->stream);
      return check_launch(h, n);
    };
    for (; s < nsteps && s < 2; ++s) KB_TRY(eager());
    if (nsteps - s >= 4) {
      cudaGraphExec_t gx = step_pair_graph(h, dt);
      for (; gx && s + 2 <= nsteps; s += 2) {
        KB_CUDA(cudaGraphLaunch(gx, h->stream));
        h->launches += h->sgraph_launches;
      }
    }
    for (; s < nsteps; ++s) KB_TRY(eager());
  }
  h->evolved = false;
  return read_residual(h, residual);
}

int kb_step_cfl(kb_handle_t* h, double cfl, double sim_time, double max_time, int32_t nsteps,
                double* time_out, double* residual) {
  if (!h || !time_out) return fail(KB_ERR_ARG, "kb_step_cfl: null argument");
  if (!(cfl > 0.0) || nsteps < 0) return fail(KB_ERR_ARG, "kb_step_cfl: cfl must be positive, nsteps >= 0");
  double t = sim_time;
  double r[4] = {0.0, 0.0, 0.0, 0.0};
  // stop at max_time (within rounding of the accumulated time)
  const double t_eps = 1e-14 * fabs(max_time);
  for (int s = 0; s < nsteps && t < max_time - t_eps; ++s) {
    double dt = 0.0;
    KB_TRY(kb_timestep(h, cfl, t, max_time, &dt));  // device CFL reduction of the current state
    if (!(dt > 0.0)) break;
    KB_TRY(kb_step(h, dt, 1, r));
    t += dt;
  }
  *time_out = t;
  if (residual)
    for (int k = 0; k < h->s.g.NW; ++k) residual[k] = r[k];
  return KB_OK;
}

// Forget the recorded step graphs of kb_step_async.
static void drop_graphs(kb_handle* h) {
  for (int k = 0; k < 2; ++k)
    if (h->agraph[k]) {
      cudaGraphExecDestroy(h->agraph[k]);
      h->agraph[k] = nullptr;
    }
}

static void drop_step_graphs(kb_handle* h) {
  for (int k = 0; k < 2; ++k)
    if (h->sgraph[k]) {
      cudaGraphExecDestroy(h->sgraph[k]);
      h->sgraph[k] = nullptr;
    }
}

// nsteps steps enqueued kernel by kernel on the handle stream.
static int enqueue_steps(kb_handle* h, double dt, int nsteps) {
  int n = 0;
  for (int s = 0; s < nsteps; ++s) {
    n += kb::launch_reconstruct(h->s, h->stream);
    n += kb::launch_evolve(h->s, dt, h->stream);
    n += kb::launch_update(h->s, dt, h->stream);
  }
  return n;
}

int kb_step_async(kb_handle_t* h, double dt, int32_t nsteps) {
  if (!h) return fail(KB_ERR_ARG, "kb_step_async: null handle");
  if (!(dt > 0.0)) return fail(KB_ERR_ARG, "kb_step_async: dt must be positive");
  if (nsteps < 0) return fail(KB_ERR_ARG, "kb_step_async: nsteps must be >= 0");
  if (!h->h_res) {
    KB_CUDA(cudaMallocHost((void**)&h->h_res, sizeof(double) * 5));
    KB_CUDA(cudaEventCreateWithFlags(&h->ev_done, cudaEventDisableTiming));
  }
  // A served request advances in equal chunks with one dt, so the chunk's
  // ~8 kernels per step are recorded once per starting buffer as a CUDA graph
  // and replayed: one launch per chunk instead of hundreds keeps the host
  // from becoming the bottleneck when many small solves share the GPU.  The
  // first chunk of a shape runs eagerly (module loading and function
  // attributes happen outside a capture) and is recorded for the next one.
  const int c = h->s.cur;
  if (nsteps > 0 && h->agraph[c] && h->agraph_dt == dt && h->agraph_n == nsteps) {
    KB_CUDA(cudaGraphLaunch(h->agraph[c], h->stream));
    h->launches += h->agraph_launches;
    h->s.cur = c ^ (nsteps & 1);
  } else {
    // record only a chunk shape seen twice in a row (a request's last, shorter
    // chunk is not worth a recording)
    const bool again = h->agraph_dt == dt && h->agraph_n == nsteps;
    if (!again) {
      drop_graphs(h);
      h->agraph_dt = dt;
      h->agraph_n = nsteps;
    }
    KB_TRY(check_launch(h, enqueue_steps(h, dt, nsteps)));
    if (again && nsteps > 0 && !h->agraph[c]) {
      // record the same chunk from buffer c for the next calls
      const int after = h->s.cur;
      h->s.cur = c;
      cudaGraph_t gr = nullptr;
      bool ok = cudaStreamBeginCapture(h->stream, cudaStreamCaptureModeThreadLocal) == cudaSuccess;
      int n = ok ? enqueue_steps(h, dt, nsteps) : 0;
      ok = cudaStreamEndCapture(h->stream, &gr) == cudaSuccess && ok;
      if (ok && cudaGraphInstantiate(&h->agraph[c], gr, 0) == cudaSuccess) {
        h->agraph_launches = n;
      } else {
        h->agraph[c] = nullptr;
      }
      if (gr) cudaGraphDestroy(gr);
      cudaGetLastError();  // a failed recording only means no replay
      h->s.cur = after;
    }
  }
  KB_CUDA(cudaMemcpyAsync(h->h_res, h->s.residual, sizeof(double) * 4, cudaMemcpyDeviceToHost,
                          h->stream));
  KB_CUDA(cudaMemcpyAsync(h->h_res + 4, h->s.status, sizeof(int), cudaMemcpyDeviceToHost,
                          h->stream));
  KB_CUDA(cudaEventRecord(h->ev_done, h->stream));
  h->pending = true;
  h->evolved = false;
  return KB_OK;
}

int kb_query(kb_handle_t* h, double* residual, int32_t* ready) {
  if (!h || !ready) return fail(KB_ERR_ARG, "kb_query: null argument");
  if (!h->pending) {
    *ready = 1;
    return KB_OK;
  }
  cudaError_t e = cudaEventQuery(h->ev_done);
  if (e == cudaErrorNotReady) {
    *ready = 0;
    return KB_OK;
  }
  if (e != cudaSuccess) return fail(KB_ERR_CUDA, std::string("kb_query: ") + cudaGetErrorString(e));
  *ready = 1;
  h->pending = false;
  if (residual)
    for (int k = 0; k < h->s.g.NW; ++k) residual[k] = h->h_res[k];
  int st = 0;
  std::memcpy(&st, h->h_res + 4, sizeof(int));
  return status_error(st);
}

int kb_set_timing(kb_handle_t* h, int enable) {
  if (!h) return fail(KB_ERR_ARG, "kb_set_timing: null handle");
  h->timing = enable != 0;
  for (int k = 0; k < KB_NSTAGE; ++k) {
    h->stage_ms[k] = 0.0;
    h->stage_n[k] = 0;
  }
  return KB_OK;
}

int kb_get_timing(kb_handle_t* h, double* ms, int64_t* count) {
  if (!h || !ms) return fail(KB_ERR_ARG, "kb_get_timing: null argument");
  for (int k = 0; k < KB_NSTAGE; ++k) {
    ms[k] = h->stage_ms[k];
    if (count) count[k] = h->stage_n[k];
  }
  return KB_OK;
}

int kb_set_tuning(kb_handle_t* h, const int32_t* params, int32_t n) {
  if (!h || (!params && n > 0)) return fail(KB_ERR_ARG, "kb_set_tuning: null argument");
  if (n < 0 || n > kb::TUNE_N) return fail(KB_ERR_ARG, "kb_set_tuning: bad parameter count");
  for (int k = 0; k < n; ++k) {
    int p = params[k];
    bool ok = true;
    if (k == kb::KB_TUNE_MARCH_TX) ok = p == 0 || p == 2 || p == 4;
    if (k == kb::KB_TUNE_MARCH_RY) ok = p >= 0 && p <= 4096;
    if (k == kb::KB_TUNE_MARCH_BS) ok = p == 0 || p == 64 || p == 128;
    if (k == kb::KB_TUNE_MOM_TS) ok = p == 0 || p == 2 || p == 4 || p == 8;
    if (!ok) return fail(KB_ERR_ARG, "kb_set_tuning: value out of range for parameter " + std::to_string(k));
  }
  for (int k = 0; k < n; ++k) h->s.tune[k] = params[k];
  drop_graphs(h);  // recorded launch shapes are stale
  drop_step_graphs(h);
  return KB_OK;
}

int kb_get_tuning(kb_handle_t* h, int32_t* params, int32_t n) {
  if (!h || !params) return fail(KB_ERR_ARG, "kb_get_tuning: null argument");
  for (int k = 0; k < n && k < kb::TUNE_N; ++k) params[k] = h->s.tune[k];
  return KB_OK;
}

int kb_get_stream(kb_handle_t* h, void** stream) {
  if (!h || !stream) return fail(KB_ERR_ARG, "kb_get_stream: null argument");
  *stream = (void*)h->stream;
  return KB_OK;
}

int kb_download_faces(kb_handle_t* h, double dt, double* fw, double* fh, double* fb) {
  if (!h) return fail(KB_ERR_ARG, "kb_download_faces: null handle");
  const Geo& g = h->s.g;
  KB_TRY(sync(h));
  if (fw) {
    std::vector<double> f4((size_t)h->nface * 4);
    std::vector<signed char> kinds(h->nface);
    KB_CUDA(cudaMemcpy(f4.data(), h->s.fw, sizeof(double) * f4.size(), cudaMemcpyDeviceToHost));
    KB_CUDA(cudaMemcpy(kinds.data(), h->s.kind, h->nface, cudaMemcpyDeviceToHost));
    for (int f = 0; f < h->nface; ++f)
      for (int k = 0; k < g.NW; ++k) fw[(size_t)f * g.NW + k] = kinds[f] ? f4[(size_t)f * 4 + k] : 0.0;
  }
  if (fh || fb) {
    double *dfh = nullptr, *dfb = nullptr;
    size_t n = (size_t)h->nface * g.nvel;
    KB_CUDA(cudaMalloc(&dfh, sizeof(double) * n));
    if (cudaMalloc(&dfb, sizeof(double) * n) != cudaSuccess) {
      cudaFree(dfh);
      return fail(KB_ERR_NOMEM, "kb_download_faces: allocation failed");
    }
    int rc = check_launch(h, kb::launch_faces_dump(h->s, dt, dfh, dfb, h->stream));
    if (rc == KB_OK) rc = sync(h);
    if (rc == KB_OK && fh && cudaMemcpy(fh, dfh, sizeof(double) * n, cudaMemcpyDeviceToHost) != cudaSuccess)
      rc = fail(KB_ERR_CUDA, "kb_download_faces: copy failed");
    if (rc == KB_OK && fb && cudaMemcpy(fb, dfb, sizeof(double) * n, cudaMemcpyDeviceToHost) != cudaSuccess)
      rc = fail(KB_ERR_CUDA, "kb_download_faces: copy failed");
    cudaFree(dfh);
    cudaFree(dfb);
    return rc;
  }
  return KB_OK;
}

int kb_upload_slopes(kb_handle_t* h, const double* sw) {
  if (!h || !sw) return fail(KB_ERR_ARG, "kb_upload_slopes: null argument");
  const Geo& g = h->s.g;
  KB_TRY(sync(h));
  std::vector<double> s8((size_t)h->ncell * 8, 0.0);
  for (long c = 0; c < h->ncell; ++c)
    for (int d = 0; d < g.D; ++d)
      for (int k = 0; k < g.NW; ++k) s8[(size_t)c * 8 + d * 4 + k] = sw[((size_t)c * g.D + d) * g.NW + k];
  KB_CUDA(cudaMemcpy(h->s.sw, s8.data(), sizeof(double) * s8.size(), cudaMemcpyHostToDevice));
  return KB_OK;
}

int kb_download_slopes(kb_handle_t* h, double* sw, double* sh, double* sb) {
  if (!h) return fail(KB_ERR_ARG, "kb_download_slopes: null handle");
  const Geo& g = h->s.g;
  KB_TRY(sync(h));
  if (sw) {
    std::vector<double> s8((size_t)h->ncell * 8);
    KB_CUDA(cudaMemcpy(s8.data(), h->s.sw, sizeof(double) * s8.size(), cudaMemcpyDeviceToHost));
    for (long c = 0; c < h->ncell; ++c)
      for (int d = 0; d < g.D; ++d)
        for (int k = 0; k < g.NW; ++k) sw[((size_t)c * g.D + d) * g.NW + k] = s8[(size_t)c * 8 + d * 4 + k];
  }
  if (sh || sb) {
    double *dsh = nullptr, *dsb = nullptr;
    size_t n = (size_t)h->ncell * g.D * g.nvel;
    KB_CUDA(cudaMalloc(&dsh, sizeof(double) * n));
    if (cudaMalloc(&dsb, sizeof(double) * n) != cudaSuccess) {
      cudaFree(dsh);
      return fail(KB_ERR_NOMEM, "kb_download_slopes: allocation failed");
    }
    int rc = check_launch(h, kb::launch_slopes_dump(h->s, dsh, dsb, h->stream));
    if (rc == KB_OK) rc = sync(h);
    if (rc == KB_OK && sh && cudaMemcpy(sh, dsh, sizeof(double) * n, cudaMemcpyDeviceToHost) != cudaSuccess)
      rc = fail(KB_ERR_CUDA, "kb_download_slopes: copy failed");
    if (rc == KB_OK && sb && cudaMemcpy(sb, dsb, sizeof(double) * n, cudaMemcpyDeviceToHost) != cudaSuccess)
      rc = fail(KB_ERR_CUDA, "kb_download_slopes: copy failed");
    cudaFree(dsh);
    cudaFree(dsb);
    return rc;
  }
  return KB_OK;
}

int kb_status(kb_handle_t* h) {
  if (!h) return fail(KB_ERR_ARG, "kb_status: null handle");
  int st = 0;
  KB_CUDA(cudaMemcpyAsync(&st, h->s.status, sizeof(int), cudaMemcpyDeviceToHost, h->stream));
  KB_TRY(sync(h));
  return (st & 2) ? KB_ERR_TIMEOUT : st ? KB_ERR_NUMERIC : KB_OK;
}

int kb_device_bytes(kb_handle_t* h, int64_t* bytes) {
  if (!h || !bytes) return fail(KB_ERR_ARG, "kb_device_bytes: null argument");
  *bytes = h->bytes;
  return KB_OK;
}

int kb_launch_count(kb_handle_t* h, int64_t* count) {
  if (!h || !count) return fail(KB_ERR_ARG, "kb_launch_count: null argument");
  *count = h->launches;
  return KB_OK;
}

}  // extern "C"
