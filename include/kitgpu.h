/*
 * kitgpu.h -- C ABI of the GB300 (sm_103a) discrete-velocity-method time step.
 *
 * This library replaces the Julia CPU hot path of KitBase.jl (v0.9.31) for the
 * reduced-distribution forms 1D2F1V and 2D2F2V:
 *   reconstruct!  src/Solver/solver_reconstruction.jl:101-153 (1D), :475-620 (2D)
 *   evolve!       src/Solver/solver_evolution.jl:64-89 (1D), :608-679 (2D)
 *                 + evolve_boundary! src/Solver/evolve_boundary.jl:4-178
 *   update!       src/Solver/solver_update.jl:61-93 (1D), :193-246 (2D)
 *                 + update_boundary! src/Solver/update_boundary.jl:6-61, :172-306
 *   step!         src/Solver/step_2f.jl:6-64 (1D2F1V), :179-249 (2D2F2V)
 * with the kinetic fluxes flux_kfvs!, flux_kcu!, flux_ugks! and
 * flux_boundary_maxwell! (src/Flux/flux_*.jl files) and BGK / Shakhov relaxation.
 *
 * Conventions
 *  - Every function returns an int status: KB_OK (0) or a negative KB_ERR_*.
 *    kb_last_error() returns a thread-local message for the last failure.
 *  - Plain pointers and sizes only.  All pointers named host_* or documented as
 *    host arrays point to host memory; the library copies them.
 *  - Cell order: x fastest, ghost layers included:
 *        cell = (j + ngy) * (nx + 2*ngx) + (i + ngx),  i in [-ngx, nx+ngx), j likewise
 *    (0-based; the reference's 1-based ctr[i, j] is cell (i-1, j-1)).
 *    This is the column-major order of the reference's OffsetArray{ControlVolume2F}.
 *  - Velocity order: iu fastest, v = iu + nu * iv (column-major order of the
 *    reference's u[i, j] matrices, src/Phase/phase_velocity.jl:128-258).
 *  - Per-cell vectors: w and prim have dim + 2 entries (3 in 1D, 4 in 2D).
 *  - A handle owns one CUDA stream.  A handle is not thread-safe; separate
 *    handles may be driven from separate host threads.
 */
#ifndef KITGPU_H
#define KITGPU_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define KB_OK 0
#define KB_ERR_ARG (-1)       /* bad argument (null pointer, out-of-range value) */
#define KB_ERR_CONFIG (-2)    /* unsupported or inconsistent configuration */
#define KB_ERR_CUDA (-3)      /* CUDA runtime failure (message in kb_last_error) */
#define KB_ERR_NUMERIC (-4)   /* non-finite or non-positive rho / lambda after a step */
#define KB_ERR_TIMEOUT (-5)   /* a bounded device wait gave up */
#define KB_ERR_NOMEM (-6)     /* device allocation failed */
#define KB_ERR_STATE (-7)     /* call order violated (e.g. update before evolve) */

/* flux solver: KS.set.flux, dispatched at src/Solver/solver_evolution.jl:80 */
enum { KB_FLUX_KFVS = 0, KB_FLUX_KCU = 1, KB_FLUX_UGKS = 2 };
/* collision model: KS.set.collision, tested at src/Solver/step_2f.jl:34 */
enum { KB_COLL_BGK = 0, KB_COLL_SHAKHOV = 1 };
/* boundary condition per side: KS.set.boundary (src/Solver/update_boundary.jl) */
enum { KB_BC_FIX = 0, KB_BC_EXTRA = 1, KB_BC_PERIOD = 2, KB_BC_MAXWELL = 3 };
/* storage / arithmetic form of the distributions */
enum {
  KB_PREC_FP64 = 0,  /* plain form: everything in FP64 */
  KB_PREC_FP32 = 1   /* h, b and pointwise fluxes in FP32; moments, w, prim, q in FP64 */
};

/* Solver configuration: the fields of Setup / PSpace / Gas that the DVM step reads
 * (src/Struct/struct_setup.jl:106-119, src/Geometry/geo_struct.jl:10-186,
 *  src/Struct/struct_property.jl:51-64). */
typedef struct kb_config {
  int32_t dim;           /* 1 (1D2F1V) or 2 (2D2F2V) */
  int32_t nx, ny;        /* physical cells; ny = 1 in 1D */
  int32_t ngx, ngy;      /* ghost layers (nxg, nyg); ngy = 0 in 1D */
  int32_t nu, nv;        /* velocity points per axis; nv = 1 in 1D */
  int32_t flux;          /* KB_FLUX_* */
  int32_t collision;     /* KB_COLL_* */
  int32_t bc[4];         /* x-left, x-right, y-down, y-up (1D uses bc[0], bc[1]) */
  int32_t interp_order;  /* 1: no reconstruction, 2: van Leer slopes */
  int32_t precision;     /* KB_PREC_* */
  double x0, x1, y0, y1; /* physical domain; cells are uniform */
  double umax, vmax;     /* vs.u1 / vs.v1, used by the CFL time step */
  double K;              /* internal degrees of freedom (inK) */
  double gamma;          /* heat capacity ratio */
  double mu_ref;         /* reference viscosity (ref_vhs_vis) */
  double omega;          /* VHS viscosity index (gas.omega) */
  double Pr;             /* Prandtl number */
  int32_t nf;            /* distributions per cell: 2 (or 0) for the 2F models 1D2F1V /
                            2D2F2V (h, b); 1 for the 1F models 1D1F1V / 2D1F2V (f only,
                            passed as h; b is absent: NULL on upload, zero on download).
                            1F takes KFVS or KCU (src/Flux/flux_kfvs.jl:238-262, :615-650;
                            src/Flux/flux_kcu.jl:241-303, :828-894; step!
                            src/Solver/step_1f.jl) */
} kb_config_t;

typedef struct kb_handle kb_handle_t;

/* Library version string. */
const char* kb_version(void);

/* Message describing the last failing call on this host thread. */
const char* kb_last_error(void);

/* Build a solver on the current CUDA device.  u, v, weights are host arrays of
 * nu*nv velocity abscissae and quadrature weights (VSpace1D / VSpace2D fields);
 * v may be NULL in 1D.  Replaces SolverSet construction + init_fvm storage
 * (src/Solver/solver_set.jl:73-117, src/Solver/solver_init.jl:119-141, :285-325). */
int kb_create(const kb_config_t* cfg, const double* u, const double* v,
              const double* weights, kb_handle_t** out);

/* Release every device allocation of the handle. */
int kb_destroy(kb_handle_t* h);

/* Maxwell wall primitive states for one side, in the global frame, one per
 * boundary face: side 0/1 (x-left/right) take ny faces, side 2/3 (y-down/up)
 * take nx faces; each face has dim+2 values [rho, U, (V,) lambda] (rho unused).
 * These are the values KS.ib.bc(xc, yc, p) returns at the face midpoints
 * (src/Solver/evolve_boundary.jl:4-178). */
int kb_set_wall(kb_handle_t* h, int side, const double* host_prim);

/* Copy the whole cell state (all cells incl. ghosts) host -> device.
 * w, prim: [ncell][dim+2]; h, b: [ncell][nu*nv].  FP32 handles round h, b
 * on the device.  Replaces the deep copies in ControlVolume(W, PRIM, H, B, ND)
 * (src/Struct/struct_ctr.jl:207-241). */
int kb_upload_state(kb_handle_t* h, const double* w, const double* prim,
                    const double* hdist, const double* bdist);

/* Set every cell (incl. ghosts) to its equilibrium: w and prim from the host
 * ([ncell][dim+2]), h = maxwellian(u, prim) and b = h K / (2 lambda) computed on
 * the device, the way init_fvm builds them (src/Solver/solver_init.jl:119-141,
 * :285-325; src/Theory/theory_equilibrium.jl:8-25).  Moves only w and prim
 * across the bus, so a new solve starts without a host-built distribution. */
int kb_init_equilibrium(kb_handle_t* h, const double* w, const double* prim);

/* Copy the whole cell state device -> host (same layout as kb_upload_state).
 * Any pointer may be NULL to skip that field.  Feeds write_jld / extract_sol. */
int kb_download_state(kb_handle_t* h, double* w, double* prim, double* hdist,
                      double* bdist);

/* CFL time step of the current state: timestep(KS, ctr, simTime)
 * (src/Solver/solver_main.jl:240-288 1D, :290-342 2D). */
int kb_timestep(kb_handle_t* h, double cfl, double sim_time, double max_time,
                double* dt_out);

/* CFL rate of a state held in the CALLER's device memory, for callers that
 * cannot allocate device memory (a host whose device memory belongs to its
 * own pool, or a service that has already accounted every byte): the call
 * makes no allocation of any kind.  No counterpart in the reference.
 *   d_prim  device array [cells incl. ghosts][dim+2], same order as
 *           kb_upload_state's prim; only physical cells are read;
 *   d_tmax  device double receiving max over cells of
 *           (max(umax,|U|) + c)/dx (+ (max(vmax,|V|) + c)/dy in 2D), so that
 *           dt = cfl / tmax as in kb_timestep;
 *   stream  cudaStream_t (NULL: default stream); the call only enqueues.
 * Per-block partial maxima live in one fixed device array compiled into the
 * library (8 KB, held by every GPU that loads it until exit); grids above
 * KB_NOALLOC_MAX_CELLS physical cells are rejected with KB_ERR_ARG.  Every
 * call reuses that array: calls that overlap on the GPU race.  The first call
 * on a device looks up the array's device address; make that first call
 * before any stream capture.  That address is kept for the life of the
 * process: do not use this call again after a reset of its device
 * (cudaDeviceReset, CUDA.jl device_reset!).  A CUDA error already pending on
 * the calling thread is reported as KB_ERR_CUDA and left in place. */
#define KB_NOALLOC_MAX_CELLS 2097152
int kb_timestep_noalloc(const kb_config_t* cfg, const double* d_prim, double* d_tmax,
                        void* stream);

/* reconstruct!: van Leer slopes of w for every cell.  The slopes of h and b
 * are formed on the fly inside kb_evolve / kb_update, so this stage only
 * refreshes the w slopes that KCU / UGKS read. */
int kb_reconstruct(kb_handle_t* h);

/* evolve!: interface fluxes fw of every face (flux chosen by cfg.flux) plus
 * Maxwell wall fluxes.  Requires kb_reconstruct first when interp_order = 2. */
int kb_evolve(kb_handle_t* h, double dt);

/* update!: finite-volume update of w, BGK / Shakhov relaxation of h and b,
 * boundary cells and ghost fill.  residual (host, dim+2 doubles, may be NULL)
 * receives the residual of this step (src/Solver/solver_update.jl:86-88). */
int kb_update(kb_handle_t* h, double dt, double* residual);

/* nsteps fused time steps reconstruct! -> evolve! -> update! with a fixed dt.
 * residual (host, dim+2 doubles, may be NULL) receives the last step's residual.
 * Replaces the body of the solve! loop (src/Solver/solver_main.jl:32-72). */
int kb_step(kb_handle_t* h, double dt, int32_t nsteps, double* residual);

/* nsteps steps, each with its own dt: before every step the CFL rate of the
 * current state is reduced on the device (as kb_timestep: timestep,
 * src/Solver/solver_main.jl:240-342) and dt = cfl / rate, clipped to
 * max_time - t; stops early once t reaches max_time.  time_out receives the
 * simulated time reached, residual (may be NULL) the last step's residual.
 * The per-step dt option of the time loop; solve! itself keeps the dt of the
 * initial state (src/Solver/solver_main.jl:12-76). */
int kb_step_cfl(kb_handle_t* h, double cfl, double sim_time, double max_time, int32_t nsteps,
                double* time_out, double* residual);

/* Asynchronous form of kb_step for serving many solves at once: enqueue
 * nsteps steps on the handle's stream and return immediately; the residual of
 * the last step is copied to pinned host memory behind the steps.  kb_query
 * sets *ready = 1 once they finished (then fills residual, dim+2 doubles, may
 * be NULL) and 0 while they run.  No reference counterpart: the reference's
 * solve! blocks until maxTime. */
int kb_step_async(kb_handle_t* h, double dt, int32_t nsteps);
int kb_query(kb_handle_t* h, double* residual, int32_t* ready);

/* Face fluxes of the last kb_evolve, materialised for inspection: fw in the
 * global frame [nface][dim+2], fh, fb [nface][nu*nv].  x faces first
 * ((nx+1)*ny, i fastest), then y faces (nx*(ny+1)).  Faces that the
 * reference never computes for this configuration are returned as zero.
 * Any pointer may be NULL.  (face.fw / face.fh / face.fb of Interface2F,
 * src/Struct/struct_face.jl:56-65.) */
int kb_download_faces(kb_handle_t* h, double dt, double* fw, double* fh, double* fb);

/* Slopes sw [ncell][dim][dim+2], sh, sb [ncell][dim][nu*nv] as reconstruct!
 * would store them (ctr.sw / ctr.sh / ctr.sb; 2D slopes use the last index
 * for the direction, src/Data/data_array.jl:15-50).  Any pointer may be NULL. */
int kb_download_slopes(kb_handle_t* h, double* sw, double* sh, double* sb);

/* Restore the w slopes sw [ncell][dim][dim+2] (layout of kb_download_slopes),
 * e.g. from a checkpoint.  reconstruct! recomputes them for the cells it
 * updates; ghost cells keep the slopes bc_extra! copied into them the step
 * before (src/Boundary/bc_extra.jl:10-50), which is state a restart needs
 * (ctr.sw of ControlVolume2F, src/Struct/struct_ctr.jl:94-117). */
int kb_upload_slopes(kb_handle_t* h, const double* sw);

/* Status word of the handle: KB_OK, KB_ERR_NUMERIC once a step produced a
 * non-finite or non-positive density / lambda, or KB_ERR_TIMEOUT once a
 * bounded device wait (coefficient staging of the update pass) gave up. */
int kb_status(kb_handle_t* h);

/* Groups of 2D solves advanced together (continuous batching of served 2D
 * requests; no reference counterpart -- the reference runs each solve! on
 * its own, src/Solver/solver_main.jl:12-150).  A group advances all of its
 * member handles with ONE launch of each step kernel per step; a member's
 * result is bit-identical to stepping it alone with the launch shapes the
 * group uses (kb_set_tuning 2, 8, 128, 2: 2-column strips of 8 rows, one
 * velocity per thread, pass A with 2 faces per warp).  Members: 2D FP32-split
 * KCU solves, BGK or Shakhov (one model per group), without ghost-filled
 * boundaries, small enough for 32-thread cell blocks (fewer than two
 * 256-thread blocks per multiprocessor).  Members join and leave between
 * chunks (after kb_group_query reported the chunk done); while in a group a
 * handle must not be stepped on its own, and it must leave the group before
 * kb_destroy.  A group has its own stream and, like a handle, is not
 * thread-safe.
 *   kb_group_create    capacity = most members at a time
 *   kb_group_add       member with its time step dt (KB_ERR_CONFIG when the
 *                      solve is not covered)
 *   kb_group_step_async  enqueue nsteps steps of every member
 *   kb_group_query     *ready = 1 once the chunk finished; residual [n][4]
 *                      and status [n] (KB_OK / KB_ERR_NUMERIC /
 *                      KB_ERR_TIMEOUT) in member order (order of joining,
 *                      members that left removed); either may be NULL
 *   kb_group_info      members and kernel launches so far */
typedef struct kb_group kb_group_t;
int kb_group_create(int32_t capacity, kb_group_t** out);
int kb_group_destroy(kb_group_t* g);
int kb_group_add(kb_group_t* g, kb_handle_t* h, double dt);
int kb_group_remove(kb_group_t* g, kb_handle_t* h);
int kb_group_step_async(kb_group_t* g, int32_t nsteps);
int kb_group_query(kb_group_t* g, double* residual, int32_t* status, int32_t* ready);
int kb_group_info(kb_group_t* g, int32_t* members, int64_t* launches);

/* Test of the bounded device waits, no reference counterpart: one CTA waits
 * through the same bounded mbarrier wait the staging kernels use, on a phase
 * that nothing completes.  The wait gives up after limit_s (0 < limit_s <= 2)
 * and the call returns KB_ERR_TIMEOUT with *status_out = 2 (the status bit
 * the staging kernels set) and *waited_s = how long the wait took; the CUDA
 * context stays usable.  Either pointer may be NULL.  Allocates 16 bytes of
 * device memory for the result; runs on the default stream and synchronizes. */
int kb_wait_probe(double limit_s, int32_t* status_out, double* waited_s);

/* Device bytes held by the handle. */
int kb_device_bytes(kb_handle_t* h, int64_t* bytes);

/* Number of kernel launches issued by this handle since creation. */
int kb_launch_count(kb_handle_t* h, int64_t* count);

/* Per-stage kernel timing of kb_step, measured with CUDA events on the
 * handle's stream.  Stages: 0 w slopes (reconstruct!), 1 face parameters,
 * 2 face moments (fw, heat flux), 3 Maxwell walls, 4 cell parameters
 * (w, prim, tau), 5 pointwise update of h and b, 6 ghost fill + residual.
 * kb_set_timing(h, 1) enables and resets the counters; kb_get_timing returns
 * the accumulated milliseconds and step counts per stage.  No reference
 * counterpart (the reference only wraps solve! in @showprogress). */
#define KB_NSTAGE 7
int kb_set_timing(kb_handle_t* h, int enable);
int kb_get_timing(kb_handle_t* h, double* ms, int64_t* count);

/* Launch shapes of the two HBM passes, chosen by the autotuner (kitgpu.tune):
 * params[0] columns per strip of the update pass (2, 4), params[1] rows
 * per CTA of the update pass (1..4096), params[2] update-pass form (64: two
 * velocities per thread in packed FP32 pairs -- the 2D FP32 form -- or 64
 * threads per CTA elsewhere; 128: one velocity per thread, 128 threads),
 * params[3] faces per warp of the moment pass (2, 4) along x and y lines,
 * or 8: both face directions in one launch over the update pass's row rings
 * (2D FP32 BGK; other solves keep the line form).  0 keeps the default.
 * No reference counterpart. */
#define KB_NTUNE 4
int kb_set_tuning(kb_handle_t* h, const int32_t* params, int32_t n);
int kb_get_tuning(kb_handle_t* h, int32_t* params, int32_t n);

/* The cudaStream_t (as void*) the handle launches on, so callers can order
 * their own work or CUDA events against it. */
int kb_get_stream(kb_handle_t* h, void** stream);

/* ------------------------------------------------------------------ batch
 * Many independent 1D2F1V solves with uneven cell counts and velocity grids,
 * advanced by one fused kernel launch per step over a flattened ragged index
 * (the FP32 split form adds a small per-instance residual kernel), two steps
 * captured as a CUDA graph.  Each instance is what the
 * reference would run as its own solve! (src/Solver/solver_main.jl:12-76) with
 * KFVS, BGK / Shakhov, fixed boundaries and van Leer slopes; a launch is the
 * loop of that call over all instances.  Instance b has nx[b] cells (plus
 * ngx[b] ghost layers per side) on [x0[b], x1[b]] and nu[b] <= 256 velocities;
 * u_all / w_all concatenate the velocity tables.  States concatenate the
 * instances: w, prim [cells][3], h, b [cells][nu of its instance]. */
typedef struct kb_batch kb_batch_t;
int kb_batch_create(const kb_config_t* base, int32_t n, const int32_t* nx, const int32_t* ngx,
                    const int32_t* nu, const double* x0, const double* x1, const double* umax,
                    const double* mu_ref, const double* u_all, const double* w_all,
                    kb_batch_t** out);
int kb_batch_destroy(kb_batch_t* b);
int kb_batch_upload(kb_batch_t* b, const double* w, const double* prim, const double* hdist,
                    const double* bdist);
int kb_batch_download(kb_batch_t* b, double* w, double* prim, double* hdist, double* bdist);
/* w, prim of every cell (same layout as kb_batch_upload) with h, b built on
 * the device as each cell's equilibrium (init_fvm, src/Solver/solver_init.jl:
 * 119-141).  The FP32 split form evaluates that Maxwellian with the same
 * FP32 function as its relaxation, so a uniform equilibrium region (such as
 * the fixed upstream state of a shock) stays bit-exact instead of drifting
 * by FP32 rounding. */
int kb_batch_init_equilibrium(kb_batch_t* b, const double* w, const double* prim);
/* Per-instance CFL time step (timestep, src/Solver/solver_main.jl:240-288). */
int kb_batch_timestep(kb_batch_t* b, double cfl, double* dt_out);
int kb_batch_set_dt(kb_batch_t* b, const double* dt);
/* nsteps steps; an instance whose residual max falls below tol stops (its
 * state is carried unchanged).  residual [n][4] and active [n] may be NULL. */
int kb_batch_step(kb_batch_t* b, int32_t nsteps, double tol, double* residual, int32_t* active);
int kb_batch_info(kb_batch_t* b, int64_t* elems, int64_t* launches);
/* Shape of the FP32 batch step kernel, chosen by the autotuner (kitgpu.tune):
 * params[0] cells per segment (8, 16, 32), params[1] threads per CTA (64, 128,
 * 256; compiled pairs: 8x64, 16x64, 16x128, 16x256, 32x128, 32x256), params[2]
 * 1 for a persistent grid (as many CTAs as fit on the GPU, each looping over
 * segments) or 0 for one CTA per segment.  Call outside stream capture; the
 * FP64 batch ignores it.  No reference counterpart. */
int kb_batch_set_tuning(kb_batch_t* b, const int32_t* params, int32_t n);
int kb_batch_get_tuning(kb_batch_t* b, int32_t* params, int32_t n);

/* ------------------------------------------------------------------- pool
 * Continuous batching of 1D2F1V solves for a serving loop: a batch whose
 * instances join and leave between steps.  kb_pool_create reserves
 * max_instances slots, max_cells cells (ghosts included) and max_nu
 * velocities per instance (FP32 split form, KFVS, fixed boundaries, as the
 * batch above).  kb_pool_add places one solve in free ranges: velocity table
 * u / weights (nu each), cells w / prim [nx + 2 ngx][3] (init_fvm's state; h
 * and b are built on the device as its equilibrium), the time step
 * cfl / max((max(umax, |U|) + c) / dx) of timestep (src/Solver/solver_main.jl:
 * 240-288) returned in *dt_out; *slot receives the instance index used by
 * the residual / active arrays of kb_batch_step.  kb_pool_remove releases a
 * slot; kb_pool_download reads one slot's state (w, prim [ncell][3], h, b
 * [ncell][nu]; any pointer may be NULL).  kb_batch_step advances every
 * resident solve with one fused launch per step; kb_batch_set_tuning picks
 * the kernel shape; kb_batch_destroy frees the pool.  The whole-batch
 * upload / download / timestep / set_dt calls are refused on a pool.  Each
 * resident solve is what the reference would run as its own solve!
 * (src/Solver/solver_main.jl:12-76); no single reference counterpart. */
int kb_pool_create(const kb_config_t* base, int32_t max_instances, int64_t max_cells,
                   int32_t max_nu, kb_batch_t** out);
int kb_pool_add(kb_batch_t* b, int32_t nx, int32_t ngx, int32_t nu, double x0, double x1,
                double umax, double mu_ref, const double* u, const double* weights,
                const double* w, const double* prim, double cfl, int32_t* slot, double* dt_out);
int kb_pool_remove(kb_batch_t* b, int32_t slot);
int kb_pool_download(kb_batch_t* b, int32_t slot, double* w, double* prim, double* hdist,
                     double* bdist);

/* ----------------------------------------------------------- unstructured
 * 2D2F2V on a triangle mesh: evolve! US2F (src/Solver/solver_evolution.jl:
 * 945-1035), update! US2F (src/Solver/solver_update.jl:414-471) with the
 * triangle step! (src/Solver/step_2f.jl:256-326), update_boundary! US2F
 * (src/Solver/update_boundary.jl:575-594) and the unstructured timestep
 * (src/Solver/solver_main.jl:398-420).  First-order KFVS, BGK or Shakhov,
 * FP64 or the FP32 split form.  cfg->nf = 1 gives 2D1F2V (evolve! US1F
 * :872-947, update! US1F src/Solver/solver_update.jl:359-403, the 2D1F2V
 * triangle step! src/Solver/step_1f.jl:228-285, update_boundary! US1F
 * src/Solver/update_boundary.jl:546-566): BGK only, b held at zero.
 * cfg supplies dim = 2, nf, nu, nv, collision,
 * precision, umax, vmax and the gas (K, gamma, mu_ref, omega, Pr), with
 * flux = KFVS and interp_order = 1 (other choices: KB_ERR_CONFIG).  Mesh
 * arrays (0-based): face_cells [nface][2] (-1: no cell), cell_faces and
 * cell_neighbors [ncell][3], cell_type [ncell] (0 stepped, 1 fixed, 3 set to
 * the mean of its two neighbours after each step; 2, a Maxwell wall cell, is
 * refused: the reference's call for it matches no method), face normals
 * [nface][2] pointing from the first to the second cell, face lengths, cell
 * areas and the smallest centre-to-edge distance of each cell; u, v, weights
 * the velocity grid (nu*nv).  State: w, prim [ncell][4], h, b [ncell][nu*nv]. */
typedef struct kb_us kb_us_t;
int kb_us_create(const kb_config_t* cfg, int32_t ncell, int32_t nface, const int32_t* face_cells,
                 const int32_t* cell_faces, const int32_t* cell_neighbors, const int32_t* cell_type,
                 const double* face_n, const double* face_len, const double* cell_area,
                 const double* cell_mindx, const double* u, const double* v,
                 const double* weights, kb_us_t** out);
int kb_us_destroy(kb_us_t* us);
int kb_us_upload(kb_us_t* us, const double* w, const double* prim, const double* hdist,
                 const double* bdist);
int kb_us_download(kb_us_t* us, double* w, double* prim, double* hdist, double* bdist);
int kb_us_timestep(kb_us_t* us, double cfl, double sim_time, double max_time, double* dt_out);
/* nsteps steps with a fixed dt; residual (host, 4 doubles, may be NULL)
 * receives the last step's residual (src/Solver/solver_update.jl:465-467). */
int kb_us_step(kb_us_t* us, double dt, int32_t nsteps, double* residual);
int kb_us_info(kb_us_t* us, int64_t* launches);
/* Kernel shape of the step: stepped cells per CTA (1..32; 0 = the default,
 * as many as fit 32 KB of per-velocity flux sums).  No reference
 * counterpart (launch tuning). */
int kb_us_set_tuning(kb_us_t* us, int32_t cells_per_cta);
int kb_us_get_tuning(kb_us_t* us, int32_t* cells_per_cta);
/* The CUDA stream (cudaStream_t) the solve's kernels run on, for timing
 * with events or ordering the caller's own work; no reference counterpart. */
int kb_us_stream(kb_us_t* us, void** stream);

#ifdef __cplusplus
}
#endif

#endif /* KITGPU_H */
