// kb_kernels.cuh -- launch interface between the C ABI (kb_abi.cu) and the
// DVM kernels (kb_kernels.cu).
#pragma once

#include <cuda.h>

#include <string>

#include "kb_device.cuh"

namespace kb {

// Velocities per TMA box of the FP32 passes: the tensor maps (kb_abi.cu) and
// the shared-memory stages of both passes (kb_march.cuh) are sized by it.
constexpr int KB_TMA_VBOX = 128;

// Record the message returned by kb_last_error() for this host thread.
void set_error(const std::string& msg);

// Tunable launch shapes (kb_set_tuning); 0 selects the built-in default.
enum { KB_TUNE_MARCH_TX = 0, KB_TUNE_MARCH_RY = 1, KB_TUNE_MARCH_BS = 2, KB_TUNE_MOM_TS = 3,
       TUNE_N = 4 };

struct GroupTab;

// Device buffers of one solve (owned by kb_handle, see kb_abi.cu).
struct DevState {
  Geo g;
  int tune[TUNE_N];
  int prec;   // 0: FP64, 1: FP32 split
  int flux, coll;
  const double* u;  // velocity tables [vstride]
  const double* v;
  const double* wt;
  const float* uf;
  const float* vf;
  const float* wtf;
  void* h[2];       // [ncell][vstride] (double or float)
  void* b[2];
  int cur;          // index of the current state in h / b
  double* w;        // [ncell][4]
  double* prim;     // [ncell][4]
  double* sw;       // [ncell][2][4]
  FaceParam* fp;    // [nface]
  FaceParamF* fpf;  // [nface]
  double* fw;       // [nface][4] global frame
  double* wall;     // [nface][4] wall prim, global frame (only wall faces read)
  double* rhow;     // [nface] Maxwell wall density
  signed char* kind;  // [nface] 0 none, 1 interior, 2 wall
  int* wall_list;   // [nwall] indices of the wall faces (kind 2), in face order
  int nwall;
  double* q;        // [ncell][2]
  CellParam* cp;    // [ncell]
  CellParamF* cpf;  // [ncell]
  FaceCoef32* fc;   // [nface] FP32 coefficient blocks
  CellCoef32* cc;   // [ncell] FP32 cell coefficients
  double* blockres; // [nblocks][16] residual partials
  float2* mpart;    // [velocity boxes][2][nface][4] pass-A partials of the row-ring form
                    // (double-float hi, lo); null where that form is not offered
  double* residual; // [4]
  int* status;      // [1]
  // host pointer to the TMA descriptors (CUtensorMap) of the FP32 form (the
  // layout is documented at kb_handle::tmaps); unused by device code
  const void* tmaps;
  int nface_x, nface_y;
  int ncell;
  int res_blocks;   // number of blocks of k_cell_param
  int cell_bs;      // threads per block of k_cell_param (32 or 256)
  const GroupTab* grp;  // device table of a grouped launch (kb_group_*), else null
  int sm_count;     // multiprocessors of the device: small grids spread their
                    // FP64-heavy per-face / per-cell threads over more of them
};

// Ask for the largest shared-memory carveout for kernel fn on the current
// device (once per kernel and device; see kb_kernels.cu).
void prefer_max_shared(const void* fn);

// One launch of a step kernel over the members of a group of 2D solves
// (kb_group_*): member r owns blocks [start[k][r], start[k][r + 1]) of the
// launch of kernel kind k, and runs there exactly the blocks it runs in its
// own launch, so its results are bit-identical alone and in the group.
enum { GK_WSLOPE = 0, GK_FACE, GK_MOMX, GK_MOMY, GK_WALL, GK_CELL, GK_MARCH, GK_RES, GK_N };
struct GroupTab {
  int n;                    // members
  const DevState* states;   // [n] member states, buffer index of this step
  const double* dt;         // [n] member time steps
  const CUtensorMap* maps;  // [n][6] TMA maps of this step: pass A x (h, b), y (h, b), pass B (h, b)
  const int* start;         // [GK_N][n + 1] first block of each member per kernel kind
};

// The member a block of a grouped launch belongs to, and the block's index in
// that member's own launch (a plain launch: member 0, the block itself).
template <bool GRP, int KIND>
__device__ __forceinline__ int group_member(const DevState& sp, int& lb) {
  if constexpr (!GRP) {
    lb = blockIdx.x;
    return 0;
  } else {
    const GroupTab& t = *sp.grp;
    const int* st = t.start + KIND * (t.n + 1);
    const int b = blockIdx.x;
    int lo = 0, hi = t.n - 1;  // the last member whose first block is <= b
    while (lo < hi) {
      const int mid = (lo + hi + 1) >> 1;
      if (st[mid] <= b) lo = mid;
      else hi = mid - 1;
    }
    lb = b - st[lo];
    return lo;
  }
}
// The state a kernel body reads as `s`: the launch's own parameter, or in a
// grouped launch a private copy of the member's state.  The group's tables
// hold each member's state with its current buffer in slot 0 (cur = 0), and
// the copy sets cur to the constant 0, so that `s.h[s.cur ^ 1]` and the like
// index with constants and the copy's fields stay in registers.
#define KB_GROUP_STATE(GRP, sp, gr)           \
  DevState s_member_;                         \
  if constexpr (GRP) {                        \
    s_member_ = (sp).grp->states[gr];         \
    s_member_.cur = 0;                        \
  }                                           \
  const DevState& s = (GRP) ? s_member_ : (sp)

// Grouped launch of a per-face / per-cell step kernel (kind GK_WSLOPE,
// GK_FACE, GK_WALL, GK_CELL or GK_RES) over `blocks` blocks (kb_kernels.cu).
void group_small(int kind, const DevState& ls, int flux, int blocks, cudaStream_t st);

// Face classification for the current configuration (host computes, uploads).
void face_kinds_host(const Geo& g, signed char* kind);

// One time step (reconstruct! -> evolve! -> update!) on `stream`.
// Returns the number of kernel launches.
int launch_reconstruct(DevState& s, cudaStream_t st);
int launch_evolve(DevState& s, double dt, cudaStream_t st);
int launch_update(DevState& s, double dt, cudaStream_t st);

// The same step split into its kernel groups (per-stage timing):
// evolve = face_param + moments + wall; update = cell_param + march + finish.
int launch_face_param(DevState& s, double dt, cudaStream_t st);
int launch_wall(DevState& s, double dt, cudaStream_t st);
int launch_cell_param(DevState& s, double dt, cudaStream_t st);
int launch_finish(DevState& s, cudaStream_t st);

// Pass A (face moments, heat flux) and pass B (pointwise update), kb_march.cu.
int launch_moments(DevState& s, cudaStream_t st);
// Pass A of the 2D FP32 BGK step in one launch over row rings plus the
// partial sum (kb_mom4.cu); returns the number of launches.
int moments_ring(DevState& s, cudaStream_t st);
int launch_march(DevState& s, double dt, cudaStream_t st);

// Materialise face fluxes fh / fb (double) of the current state, and slopes.
int launch_faces_dump(DevState& s, double dt, double* fh, double* fb, cudaStream_t st);
int launch_slopes_dump(DevState& s, double* sh, double* sb, cudaStream_t st);

// Conversion kernels for upload / download of distributions.
int launch_convert_in(void* dst, int prec, const double* src, long ncell, int nvel, int vstride,
                      cudaStream_t st);
int launch_convert_out(double* dst, int prec, const void* src, long ncell, int nvel,
                       int vstride, cudaStream_t st);
int launch_pack_w(double* dst4, const double* src, long ncell, int nw, cudaStream_t st);

// Equilibrium h, b of every cell from its prim into buffer 0.
int launch_init_equilibrium(DevState& s, cudaStream_t st);

// CFL time step (timestep, src/Solver/solver_main.jl:240-342): tmax into out.
int launch_timestep(const DevState& s, double umax, double vmax, double* out, cudaStream_t st);

}  // namespace kb
