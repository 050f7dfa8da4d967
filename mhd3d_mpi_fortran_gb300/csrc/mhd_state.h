// Device-side state of one solver handle and the launcher interface shared by
// the precision-specific translation units (mhd_fp32.cu, mhd_fp64.cu) and the
// C-ABI layer (mhd_api.cu).
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>
#include <string>
#include <vector>

namespace mhd {

// Per-axis ghost-image tables for the fused fill (host side of ghost_src).
std::vector<int> ghost_maps(int nx0, int ny0, int nz0, int ng, const int bc[3]);

// Text returned by mhd_last_error() on this thread (library-internal).
__attribute__((visibility("hidden"))) void set_last_error(const std::string& msg);

// Ghost-inclusive grid.  Cell arrays have (nx,ny,nz) elements, face arrays one
// more along their own axis; every array of a handle uses the same padded
// strides, element (i,j,k) (0-based, ghost-inclusive) at i + px*(j + py*k).
// The face at the low side of cell c along an axis is stored at index c, as
// are the flux through it and, for edges, the edge at the low sides of c.
struct Geom {
  int nx0, ny0, nz0;   // interior cells
  int ng, nord;        // ghost layers, nord = 2*ng
  int nx, ny, nz;      // cells incl. ghosts (nx0 + nord)
  int px, py, pz;      // strides: px >= nx+1 (multiple of 32), py = ny+1, pz = nz+1
  long long plane;     // px*py
  long long vol;       // plane*pz
};

// Scalars that live on the device so that a step never waits on the host.
struct Scal {
  double tau;                    // dt of the current step (module `tau`)
  double tau0;                   // previous dt (AB) / fixed deck dt (RK)
  double dt_cfl;                 // last CFL dt (get_dt)
  double ab_coef;                // tau/tau0/2 of advance_predictor_ab
  unsigned long long dtmin_bits; // running min of the CFL reduction (+inf between steps)
  unsigned int status;           // MHD_ST_* bits
  unsigned int pend_status;      // status bits of the state the next step starts from
  unsigned long long dtnext_bits; // CFL dt of that state (min over cells, +inf when empty)
};
// form of an RK first stage that also stores U^n (the input state) for the
// later stages' combines
constexpr int FORM_SAVE = -2;

// Curvilinear metric (metric mode only; FP64 in both precisions), computed
// once on the device from the node coordinates.  Same padded layout as the
// fields: a face at the index of the cell on its high side (the cell whose
// low face it is), an edge at the index of its upper cell.
struct Metric {
  const double* nrm[3][3];  // unit normals of the low faces [face axis][component]
  const double* am[3];      // face area magnitudes |A|
  const double* vol;        // cell volumes V
  const double* rvol;       // 1/V
  const double* eb[3][3];   // cell edge vectors (face-centroid differences) [axis][component]
  const double* nb[3][3];   // mean unit normal of the two a-faces of a cell [axis][component]
  const double* sa;         // sum over a of |mean area vector of the a-faces| (CFL)
  const double* ge[3];      // per edge family: g_e = |A1|_e |A2|_e / Vbar_e
  const double* dl[3];      // per edge family: edge length
};

// Raw device arrays the geometry kernels write (the const views above alias them).
struct MetricOut {
  double *nrm[3][3], *am[3], *vol, *rvol, *eb[3][3], *nb[3][3], *sa, *ge[3], *dl[3];
};
constexpr int kMetricArrays = 9 + 3 + 2 + 9 + 9 + 1 + 3 + 3;

// Geometry of a mapped grid from ghost-inclusive node coordinates stored in
// the padded layout (node (i,j,k) at i + px*(j + py*k)); FP64, no FMA.
// Writes the minimum interior cell volume to *min_vol (device).
void metric_geometry(const Geom& g, const double* X, const double* Y, const double* Z, const MetricOut& m,
                     double* min_vol, cudaStream_t st);

template <typename T>
struct Dev {
  Geom g;
  int recon, stepop, tvd_shift, dt_mode;
  int bc[3];
  T gam, pdmb, eps, alpha, beta, cfl;
  // state of the current level; the cell primitives and the face B are
  // double-buffered: the z-flux kernel writes the new primitives into o*, the
  // CT kernel the new face B into ob* (swapped after each stage), so no kernel
  // reads an element another thread of it is updating
  T *rho, *vx, *vy, *vz, *p, *bi, *bj, *bk, *bx, *by, *bz;
  T *orho, *ovx, *ovy, *ovz, *op;
  T *obi, *obj, *obk;
  T* dU[8];    // x+y flux divergence per cell {rho, rvx, rvy, rvz, eng, s_x, s_y, s_z}
  // previous level: RK {rho, rvx, rvy, rvz, eng, bi, bj, bk};
  //                 AB {rho, vx, vy, vz, p, bi, bj, bk, bx, by, bz}
  T* q[11];
  // AB predicted half step {rho, vx, vy, vz, p, bi, bj, bk, bx, by, bz}
  T* h[11];
  T* F[3][8];  // face fluxes [axis][rho, rvx, rvy, rvz, eng, s_x, s_y, s_z]
  T* E[3];     // edge EMFs ei, ej, ek
  T* vf;       // |v| + |B|/sqrt(rho) of the stage input
  const double *dx, *dy, *dz;  // FP64 cell widths (ghost-inclusive, 1-D)
  const T *wx, *wy, *wz;       // the same widths in T (FP32 path: converted once)
  const T *rwx, *rwy, *rwz;    // reciprocal widths (FP32 path; unused in FP64)
  Scal* sc;
  const int* gmap;             // per-axis ghost-image tables (cell x,y,z; face x,y,z), each n+2
  unsigned int* partial;       // per-block scratch of the CFL reduction
  unsigned int* counter;
  // metric mode: geometry, and the per-stage normal velocities w^a (cells)
  // and face-normal field b_a = Phi_a/|A_a| (faces) of the EMF
  Metric m;
  T* mw[3];
  T* mbn[3];
  // launch shapes (host side only): y/z face-tile length and EMF shape (ei
  // tile 4 or 8, or kEmfStream), chosen by the autotuner for the FP32 Cartesian
  // PDM path
  int tile_td, tile_ey;
  int emf;           // edge EMF scheme: 0 LFM, 1 Yee
  T* ye[12];         // Yee split electric fields, [x, y, z edges][pp, np, pn, nn] (emf = 1)
};

// The same handle with the two halves of its double-buffered arrays exchanged.
template <typename T>
inline Dev<T> other_half(Dev<T> d) {
  T* t;
  t = d.rho; d.rho = d.orho; d.orho = t;
  t = d.vx; d.vx = d.ovx; d.ovx = t;
  t = d.vy; d.vy = d.ovy; d.ovy = t;
  t = d.vz; d.vz = d.ovz; d.ovz = t;
  t = d.p; d.p = d.op; d.op = t;
  t = d.bi; d.bi = d.obi; d.obi = t;
  t = d.bj; d.bj = d.obj; d.obj = t;
  t = d.bk; d.bk = d.obk; d.obk = t;
  return d;
}

// Stage-input view: which arrays feed the EMF and flux kernels (RK: the
// state; AB: the predicted half step, mhd3d3.f90:3622-3624).
template <typename T>
struct Inp {
  const T *rho, *vx, *vy, *vz, *p, *bx, *by, *bz, *bi, *bj, *bk;
};

// M: curvilinear metric mode (face fluxes Phi in bi/bj/bk, area-weighted
// fluxes, E.dl circulation); instantiated in mhd_metric_fp32.cu /
// mhd_metric_fp64.cu.  M = false is the reference's Cartesian scheme.
template <typename T, bool M = false>
struct Launch {
  static void bxyz_vf(const Dev<T>& d, bool want_vf, cudaStream_t st);
  // ghost fill + get_bxyz + vf in one pass
  // dt_next (Cartesian): also the CFL dt and status of every cell for the
  // next step (the accumulators emptied first), as the step's dt pass gives them
  static void fill_bxyz(const Dev<T>& d, bool want_vf, cudaStream_t st, bool dt_next = false);
  // mode: 0 RK fixed, 1 CFL, 2 AB, 3 read only; save: also store RK U^n
  static void cfl(const Dev<T>& d, int mode, cudaStream_t st, bool save = false);
  // tau selection from the CFL dt and status that the previous step's last
  // stage accumulated for this state (Scal::dtnext_bits, pend_status); with
  // recompute, from a dt pass over the current state instead (first step,
  // or after the state changed between steps)
  static void cfl_folded(const Dev<T>& d, int mode, bool recompute, cudaStream_t st);
  static void save_prev(const Dev<T>& d, cudaStream_t st);
  static void predictor_ab(const Dev<T>& d, cudaStream_t st);
  // face fluxes of all three axes into F (kernel-level debug entry point)
  static void fluxes(const Dev<T>& d, const Inp<T>& in, cudaStream_t st);
  static void emf(const Dev<T>& d, const Inp<T>& in, cudaStream_t st);
  // hydro part of a stage, part 0: x faces; 1: y march (x+y divergence);
  // 2: z march with the conserved update and combine, new primitives into d.o*.
  // form: -1 none (stage 1 / AB), 0 (Xp+X)/den, 1 (c*Xp+X)/den, 2 (Xp+c*X)/den
  static void hydro(const Dev<T>& d, const Inp<T>& in, int part, int form, double c, double den, bool ab,
                    cudaStream_t st);
  // constrained-transport face-B update + combine (into the other half)
  static void ct(const Dev<T>& d, int form, double c, double den, cudaStream_t st);
  // Cartesian: CT + get_bxyz + vf over the interior cells in one pass, then
  // the ghost fill of the new half (d is the stage's view, as for ct)
  // dt_next: also accumulate the CFL dt and status of the new state (all
  // cells, ghosts included) for the next step
  static void ct_fill(const Dev<T>& d, int form, double c, double den, bool want_vf, cudaStream_t st,
                      bool dt_next = false);
  static void fill(const Dev<T>& d, cudaStream_t st);
  static void diagnostics(const Dev<T>& d, double* out5_dev, cudaStream_t st);
};

// Batched ensemble (Cartesian, PDM, RK2/RK3): each launch family covers every
// grid of the batch in one flattened 1-D launch.  A family's per-grid block
// grid is exactly the one its single-grid launcher uses; map[f] lists
// {grid, bx, by, bz} for every block of the launch, grid after grid.
enum BatchFam {
  BF_CFL, BF_FLUX_X, BF_FLUX_Y, BF_FLUX_Z, BF_EMF_I, BF_EMF_J, BF_EMF_K, BF_EMF_R, BF_CT, BF_FILL, BF_COUNT
};

struct BatchView {
  const void* tab[2];       // device Dev<T>[ngrids] for the two halves of the primitive buffers
  const int4* map[BF_COUNT];
  int nblk[BF_COUNT];
  int ngrids;
  double pdmb, eps, alpha, beta;  // limiter constants shared by the batch
  int tvd_shift;
  int tile_td, tile_ey;           // launch shapes shared by the batch
};

template <typename T>
struct Batch {
  // blocks (x, y, z) of family f for one grid with the given tiles
  static dim3 dims(int fam, const Geom& g, int td, int ey);
  // get_dt + advance_previous of every grid (RK); mode as Launch::cfl
  static void cfl(const BatchView& v, int sel, int mode, cudaStream_t st);
  // one RK stage of every grid: emf, fluxes + update, ct (on tab[sel]), then
  // fill + bxyz + vf on tab[sel ^ 1], the half the stage wrote
  static void stage(const BatchView& v, int sel, int form, double c, double den, cudaStream_t st);
  // parts of a stage, bit mask: 1 EMF, 2 fluxes + conserved update (writes
  // only scratch and the other half), 4 face-B update + fill (state)
  static void parts(const BatchView& v, int sel, int which, int form, double c, double den, cudaStream_t st);
};

// Normalisation of the learned correction: features (U - mean) / std per
// conserved variable, outputs times scale.
struct MlpNorm {
  float mean[8], std[8], scale[8];
};
// Apply the learned correction of MLP handle h to the interior of an FP32
// Cartesian periodic grid (mhd_mlp.cu); the caller refills the ghosts.
int mlp_correct(void* h, Dev<float>& d, cudaStream_t st);
// MHD_E_TIMEOUT if an MLP kernel recorded a wait that gave up, else MHD_OK.
int mlp_status(void* h);

// Tile lengths the autotuner tries (FP32 Cartesian PDM).
constexpr int kSweepTile = 32;  // face-shape value of the column sweeps
constexpr int kTileTD[4] = {4, 8, 16, kSweepTile};
constexpr int kEmfStream = 1;   // EMF-shape value of the slice-streamed EMF families
// Slice-streamed EMF launch shape (compile-time knobs): warps per block
// (edges along the warp axis), the blocks a family's launch aims at, and the
// shortest segment of the stream axis.  The EMF families run beside the face
// fluxes on a second stream, so a launch of about two blocks per SM, each
// streaming a long segment, leaves the flux kernels room.
#ifndef MHD_EMF_NW
#define MHD_EMF_NW 8
#endif
#ifndef MHD_EMF_BLOCKS
#define MHD_EMF_BLOCKS 304
#endif
#ifndef MHD_EMF_SEG_MIN
#define MHD_EMF_SEG_MIN 16
#endif
// Edge positions per segment for a family with nx0 x nW0 edge columns and
// nS0 + 1 edge positions along the stream axis.
__host__ __device__ inline int emf_stream_seg(int nx0, int nW0, int nS0) {
  const int cols = ((nx0 + 31) / 32) * ((nW0 + MHD_EMF_NW - 1) / MHD_EMF_NW);
  const int nseg = (MHD_EMF_BLOCKS + cols / 2) / cols;
  const int seg = (nS0 + 1) / (nseg > 1 ? nseg : 1);
  return seg > MHD_EMF_SEG_MIN ? seg : MHD_EMF_SEG_MIN;
}
// Segments along the stream axis: nseg of seg edge positions, the last one taking the rest.
__host__ __device__ inline int emf_stream_segs(int nS0, int seg) { return (nS0 + 1) / seg > 1 ? (nS0 + 1) / seg : 1; }
constexpr int kTileEY[3] = {4, 8, kEmfStream};

}  // namespace mhd
