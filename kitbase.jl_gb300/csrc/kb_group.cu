// kb_group.cu -- continuous batching of 2D solves: every member of a group is
// advanced by ONE launch of each step kernel (kb_group_* in include/kitgpu.h).
//
// A served stream holds many small 2D solves (lid-driven cavities of 16^2 to
// 128^2 cells); launched one handle at a time, each step of each solve is a
// chain of eight small kernels that leaves most of the GPU idle.  A group
// concatenates its members' blocks: launch k of a step covers the blocks of
// kernel k of every member, a block finds its member by a binary search over
// the members' first blocks (GroupTab::start) and then runs exactly the block
// it runs in the member's own launch, reading the member's device state, time
// step and TMA maps from the group's tables.  Results are bit-identical to
// the member stepped alone with the same launch shapes.  Members join and
// leave between chunks of steps; each keeps its own buffers, so a member can
// be downloaded or stepped on its own again after leaving.
//
// Covered form: 2D FP32 split, KCU flux (the served cavities), BGK or Shakhov,
// boundaries without ghost fill (fix / Maxwell walls), with the launch shapes
// the server gives 2D solves: pass A along lines with 2 faces per warp, pass B
// in 2-column strips of 8 rows with one velocity per thread.
#include <cuda.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <cstring>
#include <mutex>
#include <string>
#include <vector>

#include "../../include/kitgpu.h"
#include "kb_handle.h"
#include "kb_march.cuh"

using kb::DevState;
using kb::GroupTab;

namespace {

constexpr int G_TS = 2;                     // pass A faces per warp
constexpr int G_TX = 2, G_NS = 8, G_RY = 8;  // pass B strip columns, ring rows, rows per CTA

int gfail(int code, const std::string& m) {
  kb::set_error(m);
  return code;
}

// residual[4] and status of every member into one array (one copy to the host)
__global__ void k_group_gather(const DevState* states, int n, double* out) {
  const int r = blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= n) return;
  const DevState& s = states[r];
  for (int k = 0; k < 4; ++k) out[r * 5 + k] = s.residual[k];
  out[r * 5 + 4] = (double)*s.status;
}

template <bool SHAK, int DIR>
void launch_mom(const DevState& ls, int blocks, cudaStream_t st) {
  using SL = kb::MomStage<G_TS>;
  auto kern = kb::k_mom_st<2, kb::FLUX_KCU, G_TS, SHAK, DIR, true>;
  static std::once_flag once[64];
  int dev = 0;
  cudaGetDevice(&dev);
  std::call_once(once[dev & 63], [&] {
    cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, SL::BYTES);
    cudaFuncSetAttribute(kern, cudaFuncAttributePreferredSharedMemoryCarveout,
                         cudaSharedmemCarveoutMaxShared);
  });
  CUtensorMap unused;  // the grouped kernel reads the members' maps from the table
  std::memset(&unused, 0, sizeof(unused));
  kern<<<(unsigned)blocks, kb::MOM_THREADS, SL::BYTES, st>>>(unused, unused, ls);
}

void launch_march(const DevState& ls, int blocks, cudaStream_t st) {
  using L = kb::M3Layout<G_TX, G_NS>;
  auto kern = kb::k_march3<kb::FLUX_KCU, G_TX, G_NS, true>;
  static std::once_flag once[64];
  int dev = 0;
  cudaGetDevice(&dev);
  std::call_once(once[dev & 63], [&] {
    cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, L::BYTES);
    cudaFuncSetAttribute(kern, cudaFuncAttributePreferredSharedMemoryCarveout,
                         cudaSharedmemCarveoutMaxShared);
  });
  CUtensorMap unused;
  std::memset(&unused, 0, sizeof(unused));
  kern<<<(unsigned)blocks, kb::M3_BS, L::BYTES, st>>>(unused, unused, ls, G_RY);
}

}  // namespace

struct kb_group {
  int device = 0;
  int cap = 0;
  int flux = -1, coll = -1;
  cudaStream_t stream = nullptr;
  std::vector<kb_handle*> mem;
  std::vector<double> dt;
  bool dirty = true;    // tables out of date (membership changed)
  int parity = 0;       // steps since the tables were built, mod 2
  bool pending = false; // a chunk whose residuals have not been collected
  int blocks[kb::GK_N] = {0};
  DevState ls[2];       // launch states: grp -> the table of each buffer parity
  // device tables
  GroupTab* d_tab = nullptr;       // [2]
  DevState* d_states = nullptr;    // [2][cap]
  CUtensorMap* d_maps = nullptr;   // [2][cap][6]
  double* d_dt = nullptr;          // [cap]
  int* d_start = nullptr;          // [GK_N][cap + 1]
  double* d_res = nullptr;         // [cap][5]
  double* h_res = nullptr;         // pinned [cap][5]
  cudaEvent_t ev = nullptr;
  int64_t launches = 0;
};

static void group_free(kb_group* G) {
  if (G->stream) cudaStreamSynchronize(G->stream);
  cudaFree(G->d_tab);
  cudaFree(G->d_states);
  cudaFree(G->d_maps);
  cudaFree(G->d_dt);
  cudaFree(G->d_start);
  cudaFree(G->d_res);
  if (G->h_res) cudaFreeHost(G->h_res);
  if (G->ev) cudaEventDestroy(G->ev);
  if (G->stream) cudaStreamDestroy(G->stream);
  delete G;
}

// Per-member block counts of each kernel kind, prefix sums, and both parity
// tables (member states with the buffer index of that parity, their TMA maps).
static int group_build(kb_group* G) {
  const int n = (int)G->mem.size();
  std::vector<int> start((size_t)kb::GK_N * (n + 1), 0);
  std::vector<DevState> st((size_t)2 * G->cap);
  std::vector<CUtensorMap> maps((size_t)2 * G->cap * 6);
  for (int r = 0; r < n; ++r) {
    kb_handle* h = G->mem[r];
    const kb::Geo& g = h->s.g;
    const long cells = (long)g.nx * g.ny;
    int nb[kb::GK_N];
    nb[kb::GK_WSLOPE] = g.interp == 2 && G->flux != kb::FLUX_KFVS ? (int)((cells * 2 + 31) / 32) : 0;
    nb[kb::GK_FACE] = (h->s.nface_x + h->s.nface_y + 31) / 32;
    nb[kb::GK_MOMX] = g.ny * ((g.nx + 4 * G_TS - 1) / (4 * G_TS));
    nb[kb::GK_MOMY] = g.nx * ((g.ny + 4 * G_TS - 1) / (4 * G_TS));
    nb[kb::GK_WALL] = h->s.nwall;
    nb[kb::GK_CELL] = h->s.res_blocks;
    nb[kb::GK_MARCH] = ((g.nvel + kb::M3_BS - 1) / kb::M3_BS) * ((g.nx + G_TX - 1) / G_TX) *
                       ((g.ny + G_RY - 1) / G_RY);
    nb[kb::GK_RES] = 1;
    for (int k = 0; k < kb::GK_N; ++k) start[(size_t)k * (n + 1) + r + 1] = start[(size_t)k * (n + 1) + r] + nb[k];
    const CUtensorMap* tm = h->tmaps;
    for (int p = 0; p < 2; ++p) {
      // the member's state with the buffer that is current at this parity
      // in slot 0 (the grouped kernels take cur as the constant 0)
      const int c = h->s.cur ^ p;
      DevState s = h->s;
      s.h[0] = h->s.h[c];
      s.h[1] = h->s.h[c ^ 1];
      s.b[0] = h->s.b[c];
      s.b[1] = h->s.b[c ^ 1];
      s.cur = 0;
      s.grp = nullptr;
      st[(size_t)p * G->cap + r] = s;
      CUtensorMap* m = &maps[((size_t)p * G->cap + r) * 6];
      m[0] = tm[8 + ((0 * 2 + 0) * 2 + c) * 2];  // pass A x faces, 2 faces per warp: h
      m[1] = tm[8 + ((0 * 2 + 0) * 2 + c) * 2 + 1];
      m[2] = tm[8 + ((1 * 2 + 0) * 2 + c) * 2];  // pass A y faces
      m[3] = tm[8 + ((1 * 2 + 0) * 2 + c) * 2 + 1];
      m[4] = tm[(0 * 2 + c) * 2];  // pass B, 2-column strips
      m[5] = tm[(0 * 2 + c) * 2 + 1];
    }
  }
  for (int k = 0; k < kb::GK_N; ++k) G->blocks[k] = start[(size_t)k * (n + 1) + n];
  GroupTab tab[2];
  for (int p = 0; p < 2; ++p) {
    tab[p].n = n;
    tab[p].states = G->d_states + (size_t)p * G->cap;
    tab[p].dt = G->d_dt;
    tab[p].maps = G->d_maps + (size_t)p * G->cap * 6;
    tab[p].start = G->d_start;
  }
  bool ok = true;
  ok &= cudaMemcpy(G->d_states, st.data(), sizeof(DevState) * st.size(), cudaMemcpyHostToDevice) == cudaSuccess;
  ok &= cudaMemcpy(G->d_maps, maps.data(), sizeof(CUtensorMap) * maps.size(), cudaMemcpyHostToDevice) == cudaSuccess;
  ok &= cudaMemcpy(G->d_dt, G->dt.data(), sizeof(double) * std::max(n, 1), cudaMemcpyHostToDevice) == cudaSuccess;
  ok &= cudaMemcpy(G->d_start, start.data(), sizeof(int) * start.size(), cudaMemcpyHostToDevice) == cudaSuccess;
  ok &= cudaMemcpy(G->d_tab, tab, sizeof(tab), cudaMemcpyHostToDevice) == cudaSuccess;
  if (!ok) {
    cudaGetLastError();
    return gfail(KB_ERR_CUDA, "kb_group: table upload failed");
  }
  for (int p = 0; p < 2; ++p) {
    G->ls[p] = n > 0 ? G->mem[0]->s : DevState{};
    G->ls[p].grp = G->d_tab + p;
  }
  G->parity = 0;
  G->dirty = false;
  return KB_OK;
}

extern "C" {

int kb_group_create(int32_t capacity, kb_group_t** out) {
  if (!out || capacity < 1 || capacity > 4096) return gfail(KB_ERR_ARG, "kb_group_create: capacity in 1..4096");
  kb_group* G = new kb_group();
  G->cap = capacity;
  cudaGetDevice(&G->device);
  bool ok = cudaStreamCreateWithFlags(&G->stream, cudaStreamNonBlocking) == cudaSuccess;
  ok = ok && cudaMalloc(&G->d_tab, sizeof(GroupTab) * 2) == cudaSuccess;
  ok = ok && cudaMalloc(&G->d_states, sizeof(DevState) * 2 * capacity) == cudaSuccess;
  ok = ok && cudaMalloc(&G->d_maps, sizeof(CUtensorMap) * 2 * capacity * 6) == cudaSuccess;
  ok = ok && cudaMalloc(&G->d_dt, sizeof(double) * capacity) == cudaSuccess;
  ok = ok && cudaMalloc(&G->d_start, sizeof(int) * kb::GK_N * (capacity + 1)) == cudaSuccess;
  ok = ok && cudaMalloc(&G->d_res, sizeof(double) * 5 * capacity) == cudaSuccess;
  ok = ok && cudaMallocHost(&G->h_res, sizeof(double) * 5 * capacity) == cudaSuccess;
  ok = ok && cudaEventCreateWithFlags(&G->ev, cudaEventDisableTiming) == cudaSuccess;
  if (!ok) {
    cudaGetLastError();
    group_free(G);
    return gfail(KB_ERR_NOMEM, "kb_group_create: allocation failed");
  }
  *out = G;
  return KB_OK;
}

int kb_group_destroy(kb_group_t* G) {
  if (G) group_free(G);
  return KB_OK;
}

int kb_group_add(kb_group_t* G, kb_handle_t* h, double dt) {
  if (!G || !h) return gfail(KB_ERR_ARG, "kb_group_add: null argument");
  if (G->pending) return gfail(KB_ERR_STATE, "kb_group_add: collect the running chunk (kb_group_query) first");
  if (!(dt > 0.0)) return gfail(KB_ERR_ARG, "kb_group_add: dt must be positive");
  if ((int)G->mem.size() >= G->cap) return gfail(KB_ERR_ARG, "kb_group_add: group is full");
  if (std::find(G->mem.begin(), G->mem.end(), h) != G->mem.end())
    return gfail(KB_ERR_ARG, "kb_group_add: already a member");
  const kb_config_t& c = h->cfg;
  if (c.dim != 2 || c.precision != KB_PREC_FP32)
    return gfail(KB_ERR_CONFIG, "kb_group_add: groups hold 2D FP32-split solves");
  if (c.flux != KB_FLUX_KCU) return gfail(KB_ERR_CONFIG, "kb_group_add: groups hold KCU solves");
  for (int k = 0; k < 4; ++k)
    if (c.bc[k] == KB_BC_EXTRA || c.bc[k] == KB_BC_PERIOD)
      return gfail(KB_ERR_CONFIG, "kb_group_add: boundaries with ghost fill are not grouped");
  if (h->s.cell_bs != 32)
    return gfail(KB_ERR_CONFIG, "kb_group_add: grid too large for a group (cell blocks of 256)");
  if (!G->mem.empty() && c.collision != G->coll)
    return gfail(KB_ERR_CONFIG, "kb_group_add: all members share the collision model");
  if (cudaStreamSynchronize(h->stream) != cudaSuccess) {
    cudaGetLastError();
    return gfail(KB_ERR_CUDA, "kb_group_add: the handle's own work failed");
  }
  G->flux = c.flux;
  G->coll = c.collision;
  G->mem.push_back(h);
  G->dt.push_back(dt);
  G->dirty = true;
  return KB_OK;
}

int kb_group_remove(kb_group_t* G, kb_handle_t* h) {
  if (!G || !h) return gfail(KB_ERR_ARG, "kb_group_remove: null argument");
  if (G->pending) return gfail(KB_ERR_STATE, "kb_group_remove: collect the running chunk (kb_group_query) first");
  auto it = std::find(G->mem.begin(), G->mem.end(), h);
  if (it == G->mem.end()) return gfail(KB_ERR_ARG, "kb_group_remove: not a member");
  G->dt.erase(G->dt.begin() + (it - G->mem.begin()));
  G->mem.erase(it);
  G->dirty = true;
  return KB_OK;
}

int kb_group_step_async(kb_group_t* G, int32_t nsteps) {
  if (!G) return gfail(KB_ERR_ARG, "kb_group_step_async: null group");
  if (nsteps < 0) return gfail(KB_ERR_ARG, "kb_group_step_async: nsteps must be >= 0");
  if (G->pending) return gfail(KB_ERR_STATE, "kb_group_step_async: collect the running chunk first");
  const int n = (int)G->mem.size();
  if (n == 0) return KB_OK;
  if (G->dirty) {
    int rc = group_build(G);
    if (rc != KB_OK) return rc;
  }
  const bool shak = G->coll == KB_COLL_SHAKHOV;
  int64_t nl = 0;
  for (int k = 0; k < nsteps; ++k) {
    const DevState& ls = G->ls[(G->parity + k) & 1];
    kb::group_small(kb::GK_WSLOPE, ls, G->flux, G->blocks[kb::GK_WSLOPE], G->stream);
    kb::group_small(kb::GK_FACE, ls, G->flux, G->blocks[kb::GK_FACE], G->stream);
    if (shak) launch_mom<true, 0>(ls, G->blocks[kb::GK_MOMX], G->stream);
    else launch_mom<false, 0>(ls, G->blocks[kb::GK_MOMX], G->stream);
    launch_mom<false, 1>(ls, G->blocks[kb::GK_MOMY], G->stream);
    kb::group_small(kb::GK_WALL, ls, G->flux, G->blocks[kb::GK_WALL], G->stream);
    kb::group_small(kb::GK_CELL, ls, G->flux, G->blocks[kb::GK_CELL], G->stream);
    launch_march(ls, G->blocks[kb::GK_MARCH], G->stream);
    kb::group_small(kb::GK_RES, ls, G->flux, G->blocks[kb::GK_RES], G->stream);
    nl += 6 + (G->blocks[kb::GK_WSLOPE] > 0) + (G->blocks[kb::GK_WALL] > 0);
  }
  // the members' current buffers moved with the steps
  G->parity = (G->parity + nsteps) & 1;
  for (kb_handle* h : G->mem) {
    h->s.cur ^= (nsteps & 1);
    h->evolved = false;
  }
  k_group_gather<<<(n + 63) / 64, 64, 0, G->stream>>>(G->d_states, n, G->d_res);
  ++nl;
  cudaMemcpyAsync(G->h_res, G->d_res, sizeof(double) * 5 * n, cudaMemcpyDeviceToHost, G->stream);
  cudaEventRecord(G->ev, G->stream);
  G->launches += nl;
  G->pending = true;
  const cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return gfail(KB_ERR_CUDA, std::string("kb_group_step_async: ") + cudaGetErrorString(e));
  return KB_OK;
}

int kb_group_query(kb_group_t* G, double* residual, int32_t* status, int32_t* ready) {
  if (!G || !ready) return gfail(KB_ERR_ARG, "kb_group_query: null argument");
  *ready = 1;
  if (!G->pending) return KB_OK;
  const cudaError_t q = cudaEventQuery(G->ev);
  if (q == cudaErrorNotReady) {
    *ready = 0;
    return KB_OK;
  }
  G->pending = false;
  if (q != cudaSuccess) {
    cudaGetLastError();
    return gfail(KB_ERR_CUDA, std::string("kb_group_query: ") + cudaGetErrorString(q));
  }
  const int n = (int)G->mem.size();
  for (int r = 0; r < n; ++r) {
    if (residual)
      for (int k = 0; k < 4; ++k) residual[r * 4 + k] = G->h_res[r * 5 + k];
    if (status) {
      const int st = (int)G->h_res[r * 5 + 4];
      status[r] = (st & 2) ? KB_ERR_TIMEOUT : st ? KB_ERR_NUMERIC : KB_OK;
    }
  }
  return KB_OK;
}

int kb_group_info(kb_group_t* G, int32_t* members, int64_t* launches) {
  if (!G) return gfail(KB_ERR_ARG, "kb_group_info: null group");
  if (members) *members = (int32_t)G->mem.size();
  if (launches) *launches = G->launches;
  return KB_OK;
}

}  // extern "C"
