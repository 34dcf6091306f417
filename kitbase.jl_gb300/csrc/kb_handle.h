// kb_handle.h -- the solver handle behind kb_handle_t (private to the library:
// kb_abi.cu owns it, kb_group.cu steps several handles in shared launches).
#pragma once

#include <cuda.h>
#include <cuda_runtime.h>

#include <cstdint>
#include <vector>

#include "../../include/kitgpu.h"
#include "kb_kernels.cuh"

struct kb_handle {
  kb_config_t cfg;
  kb::DevState s;
  cudaStream_t stream = nullptr;
  int device = 0;
  int nvel = 0, vstride = 0;
  long ncell = 0;
  int nface = 0;
  int64_t bytes = 0;
  int64_t launches = 0;
  std::vector<void*> allocs;
  double* d_stage = nullptr;  // host-layout staging buffer for up/downloads
  long stage_elems = 0;
  double* d_scalar = nullptr; // [8] scratch scalars
  bool evolved = false;
  // asynchronous stepping (kb_step_async / kb_query)
  double* h_res = nullptr;    // pinned host copy of residual[4] + status
  cudaEvent_t ev_done = nullptr;
  bool pending = false;
  // chunks of kb_step_async replayed as CUDA graphs: one executable graph per
  // starting buffer index, valid for one (dt, nsteps) and the current tuning
  cudaGraphExec_t agraph[2] = {nullptr, nullptr};
  // kb_step's long runs: two steps recorded per starting buffer for one dt
  cudaGraphExec_t sgraph[2] = {nullptr, nullptr};
  double sgraph_dt = 0.0;
  int64_t sgraph_launches = 0;
  double agraph_dt = 0.0;
  int agraph_n = 0;
  int64_t agraph_launches = 0;
  // per-stage kernel timing (kb_set_timing): CUDA events on the handle stream
  bool timing = false;
  std::vector<cudaEvent_t> events;
  double stage_ms[KB_NSTAGE] = {0};
  int64_t stage_n[KB_NSTAGE] = {0};
  // TMA descriptors of the FP32 form: [0, 8) the 2D update, [strip width 2, 4]
  // [buffer][h, b]; [8, 24) the moment pass, [direction][faces per warp 2, 4]
  // [buffer][h, b]
  CUtensorMap tmaps[24];
};
