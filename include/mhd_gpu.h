/*
 * mhd_gpu.h -- C ABI of the GB300 (sm_103a) per-timestep ideal-MHD update.
 *
 * The reference program (mhd3d3.f90, module globals + `call step`) has no
 * plugin or FFI layer: the seam is the argument-less `call step` at
 * mhd3d3.f90:3286, which reads and writes the module `fields` (mhd3d3.f90:251-316),
 * the `pars` scalars (mhd3d3.f90:65-104) and the block geometry dxblock..dzblock
 * (mhd3d3.f90:114-119).  The entry points below replace that seam one for one:
 *
 *   mhd_init   <- the end of `initialization` (mhd3d3.f90:3327-3377): the driver
 *                 hands over the initialised, ghost-inclusive FP64 fields.
 *   mhd_step   <- `call step` (mhd3d3.f90:3286 -> step, mhd3d3.f90:3585-3600).
 *   mhd_fetch  <- the module arrays read by `outputxyz` (mhd3d3.f90:3091-3109)
 *                 and by `diag_rho_neg` / `diag_overflow` (mhd3d3.f90:3143-3160).
 *   mhd_free   <- `termination` / `dealloc_fields` (mhd3d3.f90:3936-3943, 319-337).
 *
 * Array convention (identical to the Fortran module arrays, mhd3d3.f90:287-290):
 * FP64, column-major (x fastest), ghost-inclusive extents with ng = nord/2
 * ghost layers per side and nx = nx0 + nord (same for y, z):
 *   cell arrays  rho,vx,vy,vz,p,bx,by,bz : (nx, ny, nz)
 *   face arrays  bi : (nx+1, ny, nz)   bj : (nx, ny+1, nz)   bk : (nx, ny, nz+1)
 * Geometry: the reference's dxblock(i,j,k) depends on i only (init_geom,
 * mhd3d3.f90:3473-3486), so it is passed as 1-D arrays dx[nx], dy[ny], dz[nz].
 *
 * All functions return 0 (MHD_OK) on success or a negative MHD_E* code.
 * Nothing here blocks forever: device waits are bounded (MHD_E_TIMEOUT).
 */
#ifndef MHD_GPU_H
#define MHD_GPU_H

#include <stdint.h>
#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

/* reconop values (mhd3d3.f90:78-79, 833-860) plus the MC-limited TVD variant */
enum { MHD_RECON_PDM = 1, MHD_RECON_TVD = 2, MHD_RECON_WENO5 = 3, MHD_RECON_MPWENO5 = 4,
       MHD_RECON_TVD_MC = 5 };
/* stepop values (mhd3d3.f90:3585-3600) */
enum { MHD_STEP_AB2 = 1, MHD_STEP_RK2 = 2, MHD_STEP_RK3 = 3 };
/* Edge EMF: MHD_EMF_LFM is get_eijk_LFM, the one the reference calls
 * (mhd3d3.f90:1754-1856); MHD_EMF_YEE is get_eijk_Yee (1654-1752, with
 * get_v_center 2562-2592), whose calls the reference keeps commented out
 * (3354, 3621).  Yee runs on Cartesian meshes only. */
enum { MHD_EMF_LFM = 0, MHD_EMF_YEE = 1 };
/* per-axis boundary kinds */
enum { MHD_BC_PERIODIC = 0,   /* periodic Cartesian topology (mhd3d2.f90:3063-3064) */
       MHD_BC_EVEN = 1,       /* even mirror of every variable (mhd3d3.f90:781-819, bc=0) */
       MHD_BC_REFLECT = 2,    /* even mirror, normal velocity odd (mhd3d2.f90:713,720) */
       MHD_BC_OUTFLOW = 3 };  /* zero-gradient copy of the boundary cell / face */
enum { MHD_FP64 = 0, MHD_FP32 = 1 };
/* dt_mode: 0 = as the reference (RK: fixed deck tau, mhd3d3.f90:3656-3661;
 *              AB: CFL dt, mhd3d3.f90:3609), 1 = CFL dt for every stepop */
enum { MHD_DT_REFERENCE = 0, MHD_DT_CFL = 1 };

/* status bits returned by mhd_step (device-side checks of the reference's
 * diag_rho_neg / diag_overflow, mhd3d3.f90:3143-3160, and its CFL warning,
 * mhd3d3.f90:3658-3660) */
enum {
  MHD_ST_NAN        = 1u << 0,  /* NaN in rho, p or v (any cell incl. ghosts) */
  MHD_ST_NEG_RHO    = 1u << 1,  /* rho < 0 somewhere (diag_rho_neg) */
  MHD_ST_NEG_P      = 1u << 2,  /* p < 0 somewhere */
  MHD_ST_CFL        = 1u << 3,  /* CFL dt < fixed tau (the reference only prints) */
  MHD_ST_TIMEOUT    = 1u << 4,  /* a bounded device wait gave up */
  MHD_ST_CUDA_ERROR = 1u << 5   /* a CUDA call failed; see mhd_last_error */
};

enum { MHD_OK = 0, MHD_E_ARG = -1, MHD_E_CUDA = -2, MHD_E_NOMEM = -3,
       MHD_E_TIMEOUT = -4, MHD_E_STATE = -5 };

typedef struct mhd_params {
  int32_t nx0, ny0, nz0;   /* interior cells per axis (one rank: nx0 = nx0G) */
  int32_t nord;            /* stencil order, ng = nord/2 (comp_pars, mhd3d3.f90:208) */
  int32_t reconop;         /* MHD_RECON_* */
  int32_t stepop;          /* MHD_STEP_* */
  int32_t bc[3];           /* MHD_BC_* for x, y, z */
  int32_t precision;       /* MHD_FP64 or MHD_FP32 */
  int32_t dt_mode;         /* MHD_DT_* */
  int32_t tvd_shift;       /* TVD corner stencils: 0 = shifts ignored as in
                              mhd3d3.f90:1187-1237, 1 = honoured as in mhd3d2.f90:1152-1199 */
  double gam;              /* 5/3 in the reference (mhd3d3.f90:51) */
  double cfl, pdmb, eps, alpha, beta;   /* namelist `free` (mhd3d3.f90:91,156) */
  double tau;              /* deck tau (namelist `list`); AB priming dt if > 0 */
  int32_t emf;             /* MHD_EMF_*: edge EMF scheme */
  int32_t reserved[7];
} mhd_params;

/* Create a solver on the current CUDA device from the driver's initialised
 * fields.  The ghost fill and get_bxyz of `initialization`
 * (mhd3d3.f90:3349-3351) are re-applied on the device.  Returns MHD_E_ARG for
 * an unsupported deck (nord odd, nord < 8 with PDM, nord < 6 with WENO, ...). */
int mhd_init(const mhd_params* prm,
             const double* rho, const double* vx, const double* vy, const double* vz,
             const double* p, const double* bi, const double* bj, const double* bk,
             const double* dx, const double* dy, const double* dz, void** handle);

/* Curvilinear metric mode (no reference counterpart: the reference mesh is
 * Cartesian, init_geom mhd3d3.f90:3473-3486).  xn, yn, zn are the physical
 * coordinates of the ghost-inclusive mesh nodes, each (nx+1, ny+1, nz+1) in
 * Fortran order; phi_i/j/k are the magnetic fluxes B.A through the faces
 * (same extents as bi/bj/bk).  The library computes the FP64 metric (face
 * area vectors and normals, cell volumes, edge lengths) on the device.
 * Fluxes go through the face area vectors, the conserved update divides by
 * the cell volume and CT advances the face fluxes by the circulation of E.dl,
 * so every term reduces to the Cartesian scheme on a rectilinear mesh.
 * mhd_fetch then returns the face fluxes in bi/bj/bk and the cell-centred B
 * in bx/by/bz; mhd_diagnostics uses the cell volumes.  Returns MHD_E_ARG for a
 * mesh with a non-positive interior cell volume. */
int mhd_init_mapped(const mhd_params* prm,
                    const double* rho, const double* vx, const double* vy, const double* vz,
                    const double* p, const double* phi_i, const double* phi_j, const double* phi_k,
                    const double* xn, const double* yn, const double* zn, void** handle);

/* One time step (replaces `call step`, mhd3d3.f90:3286).  tau_inout is the
 * driver's module `tau` (may be NULL).  On entry: an RK step with the
 * reference dt mode takes the fixed deck dt (tau = tau0, mhd3d3.f90:3656-3661),
 * and a positive *tau_inout that differs from the handle's fixed dt becomes
 * that fixed dt before the step (as mhd_set_tau, in stream order); AB steps
 * and MHD_DT_CFL take the CFL dt (get_dt) and ignore the input, as the
 * reference overwrites tau there.  On return *tau_inout holds the dt the step
 * used (the module `tau` after the step) and *status (if non-NULL) the
 * MHD_ST_* bits of the checks made during it.  Synchronous with respect to
 * the handle's stream when either pointer is non-NULL. */
int mhd_step(void* handle, double* tau_inout, uint32_t* status);

/* n steps back to back without host synchronisation in between (the driver's
 * inner `do nt=1,nts` loop, mhd3d3.f90:3284-3288).  status accumulates;
 * tau_out is output only (the dt of the last step). */
int mhd_step_n(void* handle, int32_t nsteps, double* tau_out, uint32_t* status);

/* Copy the current state back into ghost-inclusive FP64 Fortran arrays.  Any
 * pointer may be NULL to skip that field.  Synchronous. */
int mhd_fetch(void* handle, double* rho, double* vx, double* vy, double* vz,
              double* p, double* bx, double* by, double* bz,
              double* bi, double* bj, double* bk);

/* FP64 diagnostics of the current state: out[0] = mass = sum rho dV,
 * out[1] = total energy sum (rho v^2/2 + p/(gam-1) + B^2/2) dV, both with
 * compensated (Neumaier) summation over interior cells, out[2] = max |div B|
 * over interior cells from face B, out[3] = min rho (incl. ghosts),
 * out[4] = CFL dt (mhd3d3.f90:1608-1639). No reference counterpart except
 * out[3] (diag_rho_neg) and out[4] (get_dt). */
int mhd_diagnostics(void* handle, double out[5]);

/* Build a CUDA graph of n steps and replay it (graph-captured variant of
 * mhd_step_n; same results). */
int mhd_step_graph(void* handle, int32_t nsteps, double* tau_out, uint32_t* status);

/* Set the dt used by the next RK step (the driver's deck `tau`), e.g. after a
 * restart. */
int mhd_set_tau(void* handle, double tau);

/* Per-launch-family timing: when on, mhd_step_n brackets every launch family
 * with CUDA events on the handle's stream (no extra synchronisation);
 * mhd_last_timings then returns the summed device time of the last
 * mhd_step_n call in ms: [x fluxes, y fluxes, z fluxes + conserved update,
 * emf, face-B update, fill + bxyz, dt (+ save / predictor), unused]. */
int mhd_set_profiling(void* handle, int32_t on);
int mhd_last_timings(void* handle, float out_ms[8]);

/* Enqueue nsteps (graph-replayed when use_graph != 0) between two CUDA events
 * recorded on the handle's stream; *ms = their elapsed device time. */
int mhd_time_steps(void* handle, int32_t nsteps, int32_t use_graph, float* ms);

int mhd_free(void* handle);

/* Human-readable text of the last error on this thread. */
const char* mhd_last_error(void);

/* Bound, in seconds, on every host wait for the device in this process
 * (default 600).  A wait that runs out returns MHD_E_TIMEOUT, sets
 * MHD_ST_TIMEOUT in *status, and leaves the enqueued work running: the handle
 * stays usable and the next waiting call picks up where it ended. */
int mhd_set_wait_bound(double seconds);

/* Device 0's SM count, compute capability (major, minor) and maximum SM clock
 * in MHz, for roofline denominators (no reference counterpart). */
int mhd_device_info(int32_t out[4]);

/* ---- checkpoint / restart (no counterpart in the reference, which only
 * plans one: mhd3d3.f90:16, 63, 88) ------------------------------------
 * mhd_checkpoint_save writes everything a step depends on: the parameter
 * block, the device scalars (tau, tau0), the cell primitives, the face B
 * (bi, bj, bk; the reference's HDF5 frames keep only cell B) and, for AB,
 * the previous level; in the handle's own precision, so a run resumed with
 * mhd_checkpoint_load continues bit for bit.  Format: 16-byte magic
 * "MHDGB300CKPT0001", uint32 version, uint32 sizeof(mhd_params), the
 * mhd_params, 4 doubles (tau, tau0, dt_cfl, ab_coef), uint32 element size,
 * uint32 array count, then per array uint32 id + uint64 bytes + the raw
 * padded device array (ids 0-10 state, 100-110 AB previous level), and last
 * id 999 with the FP64 cell widths dx|dy|dz.  Little-endian. */
int mhd_checkpoint_save(void* handle, const char* path);
int mhd_checkpoint_load(const char* path, void** handle);

/* ---- kernel-level entry points used by the parity tests --------------- */

/* Face fluxes of the current state, as get_flux_stress (mhd3d3.f90:2385-2560)
 * leaves them: for dir d in {0,1,2} and q in {rho, rvx, rvy, rvz, eng,
 * stress_x, stress_y, stress_z}, out[(d*8+q)*nface_d ...] with the reference's
 * interior extents (nx0+1,ny0,nz0) / (nx0,ny0+1,nz0) / (nx0,ny0,nz0+1). */
int mhd_debug_fluxes(void* handle, double* out);

/* Edge EMFs of the current state, as get_eijk_LFM (mhd3d3.f90:1754-1856):
 * ei (nx0,ny0+1,nz0+1), ej (nx0+1,ny0,nz0+1), ek (nx0+1,ny0+1,nz0). */
int mhd_debug_emf(void* handle, double* ei, double* ej, double* ek);

/* ---- allocation-free diagnostics (no counterpart in the reference) ----
 *
 * For callers that cannot allocate device memory when they need the
 * diagnostics: a driver whose device memory is all owned by its own pool, a
 * latency-critical loop that must not take the implicit device
 * synchronisation of cudaMalloc/cudaFree, or a process capped by MPS/MIG
 * limits.  Same five outputs as mhd_diagnostics on a Cartesian grid (cell
 * widths dx, dy, dz), computed from arrays the caller already holds on the
 * device; the call allocates nothing.  Curvilinear (mhd_init_mapped) grids
 * are not covered: their diagnostics use cell volumes and face areas, so use
 * mhd_diagnostics there.
 *
 * All array arguments are DEVICE pointers to FP64, ghost-inclusive, Fortran-
 * ordered arrays of the layout mhd_init takes from the host (cell arrays
 * (nx,ny,nz), bi (nx+1,ny,nz), bj (nx,ny+1,nz), bk (nx,ny,nz+1); dx/dy/dz of
 * length nx/ny/nz).  Only nx0, ny0, nz0, nord, gam and cfl of *prm are read.
 * out is a DEVICE pointer to 5 doubles, written on `stream` (a cudaStream_t,
 * NULL for the legacy default stream); the call returns without waiting.
 *
 * Scratch: a file-scope device array of 2048 x 7 doubles (112 KB) that every
 * GPU loading this library keeps until the process exits; grids with more
 * than 2048 z planes (nz0 + nord) are rejected with MHD_E_ARG.  All calls share
 * that array, so calls whose kernels overlap on the GPU (different streams,
 * or other host threads, on the same device) race: order them on one stream.
 * The first call on each device looks up the array's device address with
 * that device current; make that first call before any stream capture.  The
 * address is cached for the life of the process: after a cudaDeviceReset of
 * a device, do not call this entry point on it again.
 * Errors: a CUDA error already pending from the caller's own work is
 * reported as MHD_E_CUDA and left pending (cudaPeekAtLastError); a failed
 * launch of this call is reported as MHD_E_CUDA and cleared. */
int mhd_diagnostics_noalloc(const mhd_params* prm, const double* rho, const double* vx,
                            const double* vy, const double* vz, const double* p,
                            const double* bi, const double* bj, const double* bk,
                            const double* dx, const double* dy, const double* dz,
                            double* out, void* stream);

/* ---- batched ensemble of independent grids -------------------------- */

/* Advance `ngrids` independent solvers (same precision, any sizes) by nsteps
 * each in one CUDA graph (no reference counterpart: the reference runs one
 * grid per job).  Cartesian PDM grids that share an RK stepper, dt mode and
 * limiter constants run every stage as one launch per kernel family over all
 * grids (with the launch shapes of the first grid); other ensembles get one
 * graph branch per grid.  Each grid's result is bit-for-bit what stepping it
 * alone gives.  Graphs are cached per (grids, nsteps). */
int mhd_ensemble_step(void** handles, int32_t ngrids, int32_t nsteps, uint32_t* status);

/* The same ensemble steps as mhd_ensemble_step, with *ms the device time of
 * the ensemble graph: two CUDA events on the stream that carries it (the
 * first grid's), recorded right before and after its launch. */
int mhd_ensemble_time(void** handles, int32_t ngrids, int32_t nsteps, float* ms);

/* Tile autotuner (no reference counterpart).  Times the launch-shape variants
 * compiled for the FP32 Cartesian paths -- y/z face-tile length 4, 8 or 16 (8
 * only outside PDM)
 * or 32 (32: column sweeps of 32-cell segments with a register window) and
 * the PDM EMF shape: 4 or 8 (shared-memory tiles, ei tile 4x4 or 8x8 edges)
 * or 1 (slice streams: one edge column per thread, the default) -- on the
 * handle's own grid, `reps` timed runs each, keeps the fastest and writes it
 * to out[0] (tile length) and out[1] (EMF shape).  The timed launches touch
 * only scratch arrays, so the state is unchanged, and every choice gives
 * bit-identical steps.  Other
 * handles keep their fixed shapes (returned in out). */
int mhd_autotune(void* handle, int32_t reps, int32_t out[2]);

/* The same for a batched ensemble: times the batched launches over all grids
 * and gives every grid the fastest shapes. */
int mhd_ensemble_autotune(void** handles, int32_t ngrids, int32_t reps, int32_t out[2]);

/* Sets the launch shapes directly (no timing): face-tile length 4, 8, 16 or
 * 32 and EMF shape 4, 8 or 1, for a reproducible configuration (profiling, or
 * shapes found by an earlier mhd_autotune).  Handles outside the tunable
 * path (FP64, metric mode, other reconstructions) accept only their fixed
 * shapes.  Every choice gives bit-identical steps. */
int mhd_set_tiles(void* handle, int32_t face_tile, int32_t ei_tile);

/* ---- learned coarse-grid correction (BF16 tcgen05) ---------------------- */

/* Kernel-level check of the tensor-core GEMM primitive the MLP kernels are
 * built from: C[M x N] = A[M x K] B[N x K]^T with BF16 A and B (host arrays,
 * row-major, K contiguous, raw bf16 bits) and FP32 C; N and K multiples of 16
 * up to 256.  No reference counterpart. */
int mhd_tc_gemm_test(const uint16_t* a, const uint16_t* b, float* c, int32_t M, int32_t N, int32_t K);

/* Learned coarse-grid correction (no reference counterpart).  A per-cell MLP,
 * 216 inputs (3x3x3 stencil of the 8 conserved variables rho, rho v, hydro
 * energy, cell B, normalised) -> 64 -> 64 (GELU) -> 8 outputs (5 conserved
 * hydro increments and a cell-centred vector-potential increment, times a
 * per-output scale).  Weights are FP32 masters with BF16 copies; every GEMM of
 * training and inference runs on the tcgen05 tensor cores with FP32
 * accumulation.  Parameters are one flat FP32 vector: W1[64][256] b1[64]
 * W2[64][64] b2[64] W3[16][64] b3[16] (21648 floats; inputs 216..255 and
 * outputs 8..15 are padding). */
int mhd_mlp_create(const float* params, void** mlp);
/* Read (params_out) and/or replace (params_in) the parameters; either may be NULL. */
int mhd_mlp_params(void* mlp, float* params_out, const float* params_in);
/* Feature normalisation (mean, std per variable) and output scales. */
int mhd_mlp_set_norm(void* mlp, const float* mean8, const float* std8, const float* scale8);
/* Training set: n rows of 256 BF16 features (raw bits) and 8 FP32 targets. */
int mhd_mlp_set_data(void* mlp, const uint16_t* x, const float* t, int64_t n);
/* Gradient of the mean squared error over rows [offset, offset+count) of the
 * training set (no update): grad_out[21648], *loss_out the mean loss. */
int mhd_mlp_grad(void* mlp, int64_t offset, int32_t count, float* grad_out, float* loss_out);
/* iters Adam steps on random minibatches of `batch` rows; *loss_out is the
 * mean minibatch loss of the last iterations. */
int mhd_mlp_train(void* mlp, int32_t iters, int32_t batch, float lr, uint64_t seed, float* loss_out);
/* Raw network outputs y[n][8] for feature rows x[n][256] (BF16 bits). */
int mhd_mlp_forward(void* mlp, const uint16_t* x, int64_t n, float* y);
/* Apply the correction once to an FP32 Cartesian periodic RK grid (the state
 * after a step): hydro increments per cell (a cell whose corrected density or
 * pressure would not be positive keeps its state) and face B += curl of the
 * edge-averaged vector potential, so div B stays at round-off. */
int mhd_mlp_apply(void* handle, void* mlp);
/* nsteps x (mhd_step + mhd_mlp_apply), one host synchronisation at the end. */
int mhd_step_corrected(void* handle, void* mlp, int32_t nsteps, double* tau_out, uint32_t* status);
int mhd_mlp_free(void* mlp);

#ifdef __cplusplus
}
#endif

#endif /* MHD_GPU_H */
