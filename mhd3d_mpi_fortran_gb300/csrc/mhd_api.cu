// C ABI of the GB300 MHD step (declared in include/mhd_gpu.h).  Host-side
// sequencing of one time step on one CUDA stream; every kernel is in
// mhd_kernels.cuh, instantiated per precision in mhd_fp32.cu / mhd_fp64.cu
// (Cartesian) and mhd_metric_fp32.cu / mhd_metric_fp64.cu (curvilinear
// metric mode, handles made by mhd_init_mapped).
//
// Step sequence (reference routine -> launches):
//   step_rk2/rk3 (mhd3d3.f90:3648-3792):
//     get_dt + advance_previous -> Launch::cfl(save);
//     per stage: get_eijk_LFM -> emf; get_flux_stress + advance_corrector1/2
//     + combines -> hydro (x faces, y faces, z faces + update);
//     advance_bijk + combine -> ct; fill_hydro_mpi/fill_mag_mpi + get_bxyz
//     -> fill_bxyz.
//   step_ab (mhd3d3.f90:3602-3644):
//     get_dt -> cfl(AB); advance_predictor_ab -> predictor_ab; emf(h);
//     hydro(h); ct; fill_bxyz.
#include <cuda_runtime.h>
#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <string>
#include <thread>
#include <vector>
#include <atomic>
#include <map>
#include <mutex>
#include <unistd.h>

#include "../../include/mhd_gpu.h"
#include "mhd_state.h"

using namespace mhd;

namespace {

thread_local std::string g_err;

int fail(int code, const std::string& msg) {
  g_err = msg;
  return code;
}

#define CK(call)                                                                         \
  do {                                                                                   \
    cudaError_t e_ = (call);                                                             \
    if (e_ != cudaSuccess)                                                               \
      return fail(MHD_E_CUDA, std::string(#call) + ": " + cudaGetErrorString(e_));       \
  } while (0)

// Bound on any host wait for the device (mhd_set_wait_bound), seconds.
std::atomic<double> g_wait_seconds{600.0};

std::atomic<unsigned long long> g_next_uid{1};

struct Handle {
  unsigned long long uid = 0;  // never reused: keys the ensemble graph cache
  mhd_params prm{};
  Geom g{};
  int fp32 = 0;
  cudaStream_t st = nullptr;
  cudaStream_t st2 = nullptr;  // side stream: the EMF families run on it beside the face fluxes
  cudaEvent_t ev_fork = nullptr, ev_join = nullptr;
  void* buf = nullptr;
  size_t bytes = 0;
  double* geo = nullptr;       // dx | dy | dz (FP64)
  Scal* sc = nullptr;          // device scalars
  Scal* sc_h = nullptr;        // pinned mirror
  double* diag = nullptr;      // device diagnostics buffer
  double* diag_h = nullptr;    // pinned
  Dev<float> df{};
  Dev<double> dd{};
  bool profile = false;
  float tms[8] = {0, 0, 0, 0, 0, 0, 0, 0};
  cudaEvent_t ev[16] = {};
  std::vector<cudaEvent_t> pool;
  std::vector<int> fam;
  int par = 0;                 // which half of the double-buffered primitives is current
  // the previous RK step (or the learned correction's refill) left the CFL dt
  // and status of the current state in Scal::dtnext_bits / pend_status;
  // cleared when the state changes otherwise between steps (init, load,
  // batched steps)
  bool prepared = false;
  int tile_td = 8, tile_ey = 8;  // launch shapes (autotuned for FP32 Cartesian PDM)
  float* geoT = nullptr;       // FP32 copy of the cell widths
  int* gmap = nullptr;         // ghost-image tables
  bool metric = false;         // curvilinear metric mode (mhd_init_mapped)
  double* met = nullptr;       // FP64 metric arrays (kMetricArrays x vol)
  std::vector<double> nodes;   // host copy of the node coordinates (checkpoints)
  // graphs keyed by (nsteps, starting parity + 2 prepared) -> (exec, parity + 2 prepared after replay)
  std::map<std::pair<int, int>, std::pair<cudaGraphExec_t, int>> graphs;
};

size_t round_up(size_t a, size_t b) { return (a + b - 1) / b * b; }

int wait_stream(Handle* h) {
  cudaEvent_t e;
  CK(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
  CK(cudaEventRecord(e, h->st));
  auto t0 = std::chrono::steady_clock::now();
  for (;;) {
    cudaError_t q = cudaEventQuery(e);
    if (q == cudaSuccess) break;
    if (q != cudaErrorNotReady) {
      cudaEventDestroy(e);
      return fail(MHD_E_CUDA, std::string("device error: ") + cudaGetErrorString(q));
    }
    double el = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    if (el > g_wait_seconds.load(std::memory_order_relaxed)) {
      cudaEventDestroy(e);
      return fail(MHD_E_TIMEOUT, "device did not finish within the wait bound");
    }
    std::this_thread::sleep_for(std::chrono::microseconds(el < 0.01 ? 20 : 500));
  }
  cudaEventDestroy(e);
  return MHD_OK;
}

// ---- precision-generic step body -------------------------------------
template <typename T>
Inp<T> state_inp(const Dev<T>& d) {
  return Inp<T>{d.rho, d.vx, d.vy, d.vz, d.p, d.bx, d.by, d.bz, d.bi, d.bj, d.bk};
}
template <typename T>
Inp<T> half_inp(const Dev<T>& d) {
  return Inp<T>{d.h[0], d.h[1], d.h[2], d.h[3], d.h[4], d.h[8], d.h[9], d.h[10], d.h[5], d.h[6], d.h[7]};
}

// Launch-family recorder: in profile mode every family is bracketed by a pair
// of CUDA events on the stream (no synchronisation); pairs are resolved after
// the call.  Families: 0 x fluxes, 1 y fluxes (+x divergence), 2 z fluxes +
// conserved update, 3 emf, 4 ct (face B) with the fill + bxyz that follows it
// (one fused family since both run in Launch::ct_fill), 5 unused, 6
// dt/save/predict.
struct Rec {
  Handle* h = nullptr;
  cudaStream_t st = nullptr;
  std::vector<cudaEvent_t>* pool = nullptr;
  std::vector<int>* fam = nullptr;
  size_t used = 0;
  void begin() {
    if (!pool) return;
    while (pool->size() < used + 2) {
      cudaEvent_t e;
      cudaEventCreate(&e);
      pool->push_back(e);
    }
    cudaEventRecord((*pool)[used], st);
  }
  void end(int f) {
    if (!pool) return;
    cudaEventRecord((*pool)[used + 1], st);
    fam->push_back(f);
    used += 2;
  }
};

template <typename T>
Dev<T>& dev(Handle* h);
template <>
Dev<float>& dev<float>(Handle* h) { return h->df; }
template <>
Dev<double>& dev<double>(Handle* h) { return h->dd; }

// The handle's Dev with the current half of the primitive buffers in front.
template <typename T>
Dev<T> at_par(const Dev<T>& base, int par) {
  return par ? other_half(base) : base;
}

// The EMF families and the face-flux kernels of a stage read the same stage
// input and write disjoint arrays (E; F, dU and the other half of the
// primitives), so the EMF runs on the side stream between a fork and a join
// event while the fluxes run on st; CT, which reads both, follows the join.
// In graph capture the fork and join become the graph's dependencies.  The
// family recorder (profile mode) keeps one stream so that its event pairs
// time one family each.
template <typename T, bool M>
void emf_and_fluxes(Handle* h, const Dev<T>& d, const Inp<T>& in, int form, double c, double den, bool ab,
                    cudaStream_t st, Rec& R) {
  typedef Launch<T, M> L;
  if (R.pool || !h->st2) {
    R.begin(); L::emf(d, in, st); R.end(3);
    for (int part = 0; part < 3; ++part) {
      R.begin(); L::hydro(d, in, part, form, c, den, ab, st); R.end(part);
    }
    return;
  }
  cudaEventRecord(h->ev_fork, st);
  cudaStreamWaitEvent(h->st2, h->ev_fork, 0);
  L::emf(d, in, h->st2);
  for (int part = 0; part < 3; ++part) L::hydro(d, in, part, form, c, den, ab, st);
  cudaEventRecord(h->ev_join, h->st2);
  cudaStreamWaitEvent(st, h->ev_join, 0);
}

template <typename T, bool M>
void enqueue_step(Handle* h, int& par, cudaStream_t st, Rec* r = nullptr) {
  typedef Launch<T, M> L;
  Rec none;
  Rec& R = r ? *r : none;
  const Dev<T>& base = dev<T>(h);
  const mhd_params& p = h->prm;
  if (p.stepop == MHD_STEP_AB2) {
    Dev<T> d = at_par(base, par);
    R.begin(); L::cfl(d, 2, st); L::predictor_ab(d, st); R.end(6);
    Inp<T> in = half_inp(d);
    emf_and_fluxes<T, M>(h, d, in, -1, 0.0, 1.0, true, st, R);
    R.begin(); L::ct_fill(d, -1, 0.0, 1.0, false, st); R.end(4);
    par ^= 1;
    h->prepared = false;
    return;
  }
  // Cartesian RK: U^n is stored by the first stage and the CFL dt of the next
  // step's state accumulated by the last one (no separate pass over the
  // state); the metric mode keeps the CFL pass that also stores U^n.
  constexpr bool fold = !M;
  {
    Dev<T> d = at_par(base, par);
    R.begin();
    if (fold) L::cfl_folded(d, p.dt_mode == MHD_DT_CFL ? 1 : 0, !h->prepared, st);
    else L::cfl(d, p.dt_mode == MHD_DT_CFL ? 1 : 0, st, true);
    R.end(6);
  }
  int nst = (p.stepop == MHD_STEP_RK2) ? 2 : 3;
  for (int s = 1; s <= nst; ++s) {
    int form = fold ? FORM_SAVE : -1;
    double c = 0.0, den = 1.0;
    if (s > 1) {
      if (nst == 2) { form = 0; den = 2.0; }
      else if (s == 2) { form = 1; c = 3.0; den = 4.0; }
      else { form = 2; c = 2.0; den = 3.0; }
    }
    Dev<T> d = at_par(base, par);
    Inp<T> in = state_inp(d);
    emf_and_fluxes<T, M>(h, d, in, form, c, den, false, st, R);
    R.begin(); L::ct_fill(d, form, c, den, true, st, fold && s == nst); R.end(4);
    par ^= 1;
  }
  h->prepared = fold;
}

// Cartesian or metric step of a handle.
template <typename T>
void enqueue_any(Handle* h, int& par, cudaStream_t st, Rec* r = nullptr) {
  if (h->metric) enqueue_step<T, true>(h, par, st, r);
  else enqueue_step<T, false>(h, par, st, r);
}

inline void set_widths(Handle* h, Dev<double>& d) {
  d.wx = d.dx; d.wy = d.dy; d.wz = d.dz;
  d.rwx = d.dx; d.rwy = d.dy; d.rwz = d.dz;
}
inline void set_widths(Handle* h, Dev<float>& d) {
  const Geom& g = h->g;
  const int n = g.nx + g.ny + g.nz;
  d.wx = h->geoT; d.wy = h->geoT + g.nx; d.wz = h->geoT + g.nx + g.ny;
  d.rwx = h->geoT + n; d.rwy = h->geoT + n + g.nx; d.rwz = h->geoT + n + g.nx + g.ny;
}

template <typename T>
void carve(Handle* h, Dev<T>& d, char* base) {
  const Geom& g = h->g;
  size_t n = (size_t)g.vol;
  T* a = (T*)base;
  auto next = [&]() { T* r = a; a += n; return r; };
  d.g = g;
  d.recon = h->prm.reconop;
  d.stepop = h->prm.stepop;
  d.tvd_shift = h->prm.tvd_shift;
  d.dt_mode = h->prm.dt_mode;
  for (int i = 0; i < 3; ++i) d.bc[i] = h->prm.bc[i];
  d.gam = (T)h->prm.gam; d.pdmb = (T)h->prm.pdmb; d.eps = (T)h->prm.eps;
  d.alpha = (T)h->prm.alpha; d.beta = (T)h->prm.beta; d.cfl = (T)h->prm.cfl;
  d.rho = next(); d.vx = next(); d.vy = next(); d.vz = next(); d.p = next();
  d.bi = next(); d.bj = next(); d.bk = next(); d.bx = next(); d.by = next(); d.bz = next();
  d.orho = next(); d.ovx = next(); d.ovy = next(); d.ovz = next(); d.op = next();
  d.obi = next(); d.obj = next(); d.obk = next();
  for (int q = 0; q < 8; ++q) d.dU[q] = next();
  int nq = (h->prm.stepop == MHD_STEP_AB2) ? 11 : 8;
  for (int i = 0; i < 11; ++i) d.q[i] = (i < nq) ? next() : nullptr;
  for (int i = 0; i < 11; ++i) d.h[i] = (h->prm.stepop == MHD_STEP_AB2) ? next() : nullptr;
  // x-face fluxes only: the y / z faces are consumed inside the sweeps / face
  // tiles; the kernel-level debug entry point gives them scratch of its own
  for (int q = 0; q < 8; ++q) d.F[0][q] = next();
  for (int ax = 1; ax < 3; ++ax)
    for (int q = 0; q < 8; ++q) d.F[ax][q] = nullptr;
  for (int e = 0; e < 3; ++e) d.E[e] = next();
  d.vf = next();
  d.dx = h->geo; d.dy = h->geo + g.nx; d.dz = h->geo + g.nx + g.ny;
  set_widths(h, d);
  d.sc = h->sc;
  d.gmap = h->gmap;
  d.partial = nullptr;
  d.counter = nullptr;
  d.m = Metric{};
  d.tile_td = h->tile_td;
  d.tile_ey = h->tile_ey;
  for (int a = 0; a < 3; ++a) {
    d.mw[a] = h->metric ? next() : nullptr;
    d.mbn[a] = h->metric ? next() : nullptr;
  }
  d.emf = h->prm.emf;
  for (int q = 0; q < 12; ++q) d.ye[q] = (h->prm.emf == MHD_EMF_YEE) ? next() : nullptr;
  if (h->metric) {
    const double* mb = h->met;
    auto nm = [&]() { const double* r = mb; mb += n; return r; };
    Metric& m = d.m;
    for (int a = 0; a < 3; ++a)
      for (int q = 0; q < 3; ++q) m.nrm[a][q] = nm();
    for (int a = 0; a < 3; ++a) m.am[a] = nm();
    m.vol = nm();
    m.rvol = nm();
    for (int a = 0; a < 3; ++a)
      for (int q = 0; q < 3; ++q) m.eb[a][q] = nm();
    for (int a = 0; a < 3; ++a)
      for (int q = 0; q < 3; ++q) m.nb[a][q] = nm();
    m.sa = nm();
    for (int e = 0; e < 3; ++e) m.ge[e] = nm();
    for (int e = 0; e < 3; ++e) m.dl[e] = nm();
  }
}

// The writable view of the metric block carved as carve() lays it out.
MetricOut metric_out(Handle* h) {
  const size_t n = (size_t)h->g.vol;
  double* mb = h->met;
  auto nm = [&]() { double* r = mb; mb += n; return r; };
  MetricOut m;
  for (int a = 0; a < 3; ++a)
    for (int q = 0; q < 3; ++q) m.nrm[a][q] = nm();
  for (int a = 0; a < 3; ++a) m.am[a] = nm();
  m.vol = nm();
  m.rvol = nm();
  for (int a = 0; a < 3; ++a)
    for (int q = 0; q < 3; ++q) m.eb[a][q] = nm();
  for (int a = 0; a < 3; ++a)
    for (int q = 0; q < 3; ++q) m.nb[a][q] = nm();
  m.sa = nm();
  for (int e = 0; e < 3; ++e) m.ge[e] = nm();
  for (int e = 0; e < 3; ++e) m.dl[e] = nm();
  return m;
}

size_t n_arrays(const mhd_params& p, bool metric) {
  size_t n = 11 + 5 + 3 + 8 + ((p.stepop == MHD_STEP_AB2) ? 22 : 8) + 8 + 3 + 1 + (metric ? 6 : 0) +
             ((p.emf == MHD_EMF_YEE) ? 12 : 0);
  return n;
}

// host FP64 Fortran array (ex,ey,ez) -> padded T on the host; rows in parallel
template <typename T>
void pack(const Geom& g, const double* src, int ex, int ey, int ez, T* dst) {
#pragma omp parallel for schedule(static)
  for (int k = 0; k < ez; ++k)
    for (int j = 0; j < ey; ++j) {
      const double* s = src + (size_t)ex * ((size_t)j + (size_t)ey * k);
      T* d = dst + (size_t)g.px * ((size_t)j + (size_t)g.py * k);
      for (int i = 0; i < ex; ++i) d[i] = (T)s[i];
    }
}

// Host FP64 Fortran arrays (ex, ey, ez) <-> the padded device arrays, with the
// conversion on the device: the FP64 array is copied as it is (pageable
// copies run at the link rate on Grace-Blackwell, about 190 GB/s measured)
// into the face-flux scratch, which holds no live data outside a step, and a
// kernel converts it into (or out of) the padded layout.  Padding elements
// are never read by the kernels; the device buffer is zeroed at allocation.
template <typename T>
__global__ void k_from_f64(const double* __restrict__ src, int ex, int ey, int px, long long plane,
                           T* __restrict__ dst) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const int j = blockIdx.y, k = blockIdx.z;
  if (i < ex) dst[i + (long long)px * j + plane * k] = (T)src[i + (long long)ex * (j + (long long)ey * k)];
}
template <typename T>
__global__ void k_to_f64(const T* __restrict__ src, int ex, int ey, int px, long long plane,
                         double* __restrict__ dst) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const int j = blockIdx.y, k = blockIdx.z;
  if (i < ex) dst[i + (long long)ex * (j + (long long)ey * k)] = (double)src[i + (long long)px * j + plane * k];
}

template <typename T>
double* f64_scratch(const Dev<T>& d) {
  return reinterpret_cast<double*>(d.F[0][0]);  // 8 x vol x sizeof(T) bytes, >= one FP64 array
}

template <typename T>
int upload(Handle* h, const double* const* arrs) {
  const Geom& g = h->g;
  Dev<T>& d = dev<T>(h);
  T* dsts[8] = {d.rho, d.vx, d.vy, d.vz, d.p, d.bi, d.bj, d.bk};
  int ext[8][3] = {{g.nx, g.ny, g.nz}, {g.nx, g.ny, g.nz}, {g.nx, g.ny, g.nz}, {g.nx, g.ny, g.nz},
                   {g.nx, g.ny, g.nz}, {g.nx + 1, g.ny, g.nz}, {g.nx, g.ny + 1, g.nz},
                   {g.nx, g.ny, g.nz + 1}};
  double* scratch = f64_scratch(d);
  for (int a = 0; a < 8; ++a) {
    const int ex = ext[a][0], ey = ext[a][1], ez = ext[a][2];
    CK(cudaMemcpyAsync(scratch, arrs[a], sizeof(double) * (size_t)ex * ey * ez, cudaMemcpyHostToDevice, h->st));
    k_from_f64<T><<<dim3((ex + 255) / 256, ey, ez), 256, 0, h->st>>>(scratch, ex, ey, g.px, g.plane, dsts[a]);
  }
  CK(cudaGetLastError());
  return wait_stream(h);
}

template <typename T, bool M>
int init_device(Handle* h) {
  Dev<T>& d = dev<T>(h);
  cudaStream_t st = h->st;
  Launch<T, M>::fill(d, st);
  Launch<T, M>::bxyz_vf(d, h->prm.stepop != MHD_STEP_AB2, st);
  if (h->prm.stepop == MHD_STEP_AB2) {
    if (!(h->prm.tau > 0.0)) Launch<T, M>::cfl(d, 1, st);  // prime with the CFL dt (mhd3d2)
    T* x[11] = {d.rho, d.vx, d.vy, d.vz, d.p, d.bi, d.bj, d.bk, d.bx, d.by, d.bz};
    for (int a = 0; a < 11; ++a)
      CK(cudaMemcpyAsync(d.q[a], x[a], (size_t)h->g.vol * sizeof(T), cudaMemcpyDeviceToDevice, st));
  }
  CK(cudaGetLastError());
  return wait_stream(h);
}

template <typename T>
int do_steps(Handle* h, int n) {
  if (h->profile) {
    for (int i = 0; i < 8; ++i) h->tms[i] = 0;
    Rec r;
    r.h = h; r.st = h->st; r.pool = &h->pool; r.fam = &h->fam;
    h->fam.clear();
    for (int s = 0; s < n; ++s) enqueue_any<T>(h, h->par, h->st, &r);
    CK(cudaGetLastError());
    int rc = wait_stream(h);
    if (rc) return rc;
    for (size_t i = 0; i < h->fam.size(); ++i) {
      float ms = 0;
      cudaEventElapsedTime(&ms, h->pool[2 * i], h->pool[2 * i + 1]);
      h->tms[h->fam[i]] += ms;
    }
    return MHD_OK;
  }
  for (int s = 0; s < n; ++s) enqueue_any<T>(h, h->par, h->st);
  CK(cudaGetLastError());
  return MHD_OK;
}

int finish(Handle* h, double* tau_out, uint32_t* status) {
  if (!tau_out && !status) return MHD_OK;
  CK(cudaMemcpyAsync(h->sc_h, h->sc, sizeof(Scal), cudaMemcpyDeviceToHost, h->st));
  CK(cudaMemsetAsync(&h->sc->status, 0, sizeof(unsigned int), h->st));
  int rc = wait_stream(h);
  if (rc) {
    if (status) *status = MHD_ST_TIMEOUT | (rc == MHD_E_CUDA ? MHD_ST_CUDA_ERROR : 0);
    return rc;
  }
  if (tau_out) *tau_out = h->sc_h->tau;
  if (status) *status = h->sc_h->status;
  return MHD_OK;
}

int validate(const mhd_params* p) {
  if (!p) return fail(MHD_E_ARG, "null params");
  if (p->nx0 < 1 || p->ny0 < 1 || p->nz0 < 1) return fail(MHD_E_ARG, "grid sizes must be positive");
  if (p->nord <= 0 || (p->nord & 1)) return fail(MHD_E_ARG, "nord must be even and positive");
  if (p->reconop < 1 || p->reconop > 5) return fail(MHD_E_ARG, "reconop must be 1..5");
  if (p->stepop < 1 || p->stepop > 3) return fail(MHD_E_ARG, "stepop must be 1..3");
  if (p->emf != MHD_EMF_LFM && p->emf != MHD_EMF_YEE) return fail(MHD_E_ARG, "emf must be 0 (LFM) or 1 (Yee)");
  int need = (p->reconop == 1) ? 8 : (p->reconop == 3 || p->reconop == 4) ? 6 : 4;
  if (p->nord < need) return fail(MHD_E_ARG, "nord too small for the reconstruction stencil");
  int ng = p->nord / 2;
  for (int a = 0; a < 3; ++a) {
    if (p->bc[a] < 0 || p->bc[a] > 3) return fail(MHD_E_ARG, "bc must be 0..3");
    int n0 = a == 0 ? p->nx0 : a == 1 ? p->ny0 : p->nz0;
    if (n0 < ng) return fail(MHD_E_ARG, "each axis needs at least ng interior cells");
  }
  if (p->precision != MHD_FP32 && p->precision != MHD_FP64) return fail(MHD_E_ARG, "precision 0 or 1");
  if (!(p->gam > 1.0)) return fail(MHD_E_ARG, "gam must exceed 1");
  if (p->stepop != MHD_STEP_AB2 && p->dt_mode == MHD_DT_REFERENCE && !(p->tau > 0.0))
    return fail(MHD_E_ARG, "RK with the reference dt needs tau > 0");
  return MHD_OK;
}

}  // namespace

void mhd::set_last_error(const std::string& msg) { g_err = msg; }

// Host twin of the device ghost_src: image of index x on an axis with n0
// interior cells (cell axis) or n0+1 interior faces (face axis).
static int host_ghost_src(int x, int ng, int n0, bool face, int kind) {
  const int hi = face ? ng + n0 : ng + n0 - 1;
  if (x >= ng && x <= hi) return x;
  const bool lo = x < ng;
  if (kind == MHD_BC_PERIODIC) return lo ? x + n0 : x - n0;
  if (kind == MHD_BC_OUTFLOW) return lo ? ng : hi;
  if (!face) return lo ? 2 * ng - 1 - x : 2 * n0 + 2 * ng - 1 - x;
  return lo ? 2 * ng - x : 2 * n0 + 2 * ng - x;
}

std::vector<int> mhd::ghost_maps(int nx0, int ny0, int nz0, int ng, const int bc[3]) {
  const int n0[3] = {nx0, ny0, nz0};
  std::vector<int> m;
  for (int face = 0; face < 2; ++face)
    for (int a = 0; a < 3; ++a) {
      const int n = n0[a] + 2 * ng;  // cells incl. ghosts; faces are n+1
      for (int x = 0; x < n + 2; ++x) {
        const bool valid = face ? x <= n : x < n;
        m.push_back(valid ? host_ghost_src(x, ng, n0[a], face != 0, bc[a]) : 0);
      }
    }
  return m;
}

// Entry points: C linkage comes from their declarations in mhd_gpu.h.

const char* mhd_last_error(void) { return g_err.c_str(); }

int mhd_set_wait_bound(double seconds) {
  if (!(seconds > 0.0) || !std::isfinite(seconds)) return fail(MHD_E_ARG, "wait bound must be positive and finite");
  g_wait_seconds.store(seconds, std::memory_order_relaxed);
  return MHD_OK;
}

int mhd_device_info(int32_t out[4]) {
  if (!out) return fail(MHD_E_ARG, "null output");
  int v[4] = {0, 0, 0, 0};
  CK(cudaDeviceGetAttribute(&v[0], cudaDevAttrMultiProcessorCount, 0));
  CK(cudaDeviceGetAttribute(&v[1], cudaDevAttrComputeCapabilityMajor, 0));
  CK(cudaDeviceGetAttribute(&v[2], cudaDevAttrComputeCapabilityMinor, 0));
  CK(cudaDeviceGetAttribute(&v[3], cudaDevAttrClockRate, 0));  // kHz
  out[0] = v[0]; out[1] = v[1]; out[2] = v[2]; out[3] = v[3] / 1000;
  return MHD_OK;
}

// Handle with its device buffers allocated and cleared, scalars set from prm,
// but no fields uploaded yet.
static int create_handle(const mhd_params* prm, const double* dx, const double* dy, const double* dz,
                         Handle** out, bool metric = false) {
  *out = nullptr;
  Handle* h = new Handle();
  h->uid = g_next_uid++;
  h->prm = *prm;
  h->fp32 = (prm->precision == MHD_FP32);
  h->metric = metric;
  // the column sweeps are the fastest FP32 face shape at production sizes; the
  // slice-streamed EMF when its ei launch has at least 256 blocks (about
  // 128^3 and up; 96^3 measured even), the 8x8 ei tiles on smaller grids (the
  // autotuner may still pick others)
  h->tile_td = (h->fp32 && !metric) ? kSweepTile : 8;
  Geom& g = h->g;
  g.nx0 = prm->nx0; g.ny0 = prm->ny0; g.nz0 = prm->nz0;
  {
    const long long eb = (long long)((g.nx0 + 31) / 32) * ((g.ny0 + MHD_EMF_NW - 1) / MHD_EMF_NW) *
                         emf_stream_segs(g.nz0, emf_stream_seg(g.nx0, g.ny0, g.nz0));
    h->tile_ey = (h->fp32 && !metric) ? (eb >= 256 ? kEmfStream : 8) : h->fp32 ? 8 : 4;
  }
  g.nord = prm->nord; g.ng = prm->nord / 2;
  g.nx = g.nx0 + g.nord; g.ny = g.ny0 + g.nord; g.nz = g.nz0 + g.nord;
  g.px = (int)round_up((size_t)g.nx + 1, 32);
  g.py = g.ny + 1;
  g.pz = g.nz + 1;
  g.plane = (long long)g.px * g.py;
  g.vol = g.plane * g.pz;
  if (g.vol >= (1LL << 31)) {
    delete h;
    return fail(MHD_E_ARG, "grid too large for 32-bit indexing");
  }
  size_t es = h->fp32 ? sizeof(float) : sizeof(double);
  h->bytes = n_arrays(*prm, metric) * (size_t)g.vol * es;
  auto bail = [&](int code, const std::string& m) {
    mhd_free(h);
    return fail(code, m);
  };
  if (cudaStreamCreateWithFlags(&h->st, cudaStreamNonBlocking) != cudaSuccess ||
      cudaStreamCreateWithFlags(&h->st2, cudaStreamNonBlocking) != cudaSuccess ||
      cudaEventCreateWithFlags(&h->ev_fork, cudaEventDisableTiming) != cudaSuccess ||
      cudaEventCreateWithFlags(&h->ev_join, cudaEventDisableTiming) != cudaSuccess)
    return bail(MHD_E_CUDA, "stream create failed");
  if (cudaMalloc(&h->buf, h->bytes) != cudaSuccess) return bail(MHD_E_NOMEM, "device allocation failed");
  if (metric && cudaMalloc(&h->met, sizeof(double) * kMetricArrays * (size_t)g.vol) != cudaSuccess)
    return bail(MHD_E_NOMEM, "device allocation of the metric failed");
  if (cudaMalloc(&h->geo, sizeof(double) * (g.nx + g.ny + g.nz)) != cudaSuccess ||
      cudaMalloc(&h->sc, sizeof(Scal)) != cudaSuccess ||
      cudaMalloc(&h->diag, sizeof(double) * (8 + 5 * 152 * 2)) != cudaSuccess)
    return bail(MHD_E_NOMEM, "device allocation failed");
  if (cudaMallocHost(&h->sc_h, sizeof(Scal)) != cudaSuccess ||
      cudaMallocHost(&h->diag_h, sizeof(double) * 8) != cudaSuccess)
    return bail(MHD_E_NOMEM, "pinned allocation failed");
  for (int i = 0; i < 16; ++i) cudaEventCreate(&h->ev[i]);
  if (cudaMemsetAsync(h->buf, 0, h->bytes, h->st) != cudaSuccess) return bail(MHD_E_CUDA, "memset failed");
  std::vector<double> geo((size_t)g.nx + g.ny + g.nz);
  std::memcpy(geo.data(), dx, sizeof(double) * g.nx);
  std::memcpy(geo.data() + g.nx, dy, sizeof(double) * g.ny);
  std::memcpy(geo.data() + g.nx + g.ny, dz, sizeof(double) * g.nz);
  for (double v : geo)
    if (!(v > 0.0)) return bail(MHD_E_ARG, "cell widths must be positive (diag_geom)");
  if (cudaMemcpy(h->geo, geo.data(), sizeof(double) * geo.size(), cudaMemcpyHostToDevice) != cudaSuccess)
    return bail(MHD_E_CUDA, "geometry upload failed");
  {
    // FP32 widths and their reciprocals (1/dx computed in FP64, rounded once)
    std::vector<float> gf(geo.begin(), geo.end());
    for (double v : geo) gf.push_back((float)(1.0 / v));
    if (cudaMalloc(&h->geoT, sizeof(float) * gf.size()) != cudaSuccess ||
        cudaMemcpy(h->geoT, gf.data(), sizeof(float) * gf.size(), cudaMemcpyHostToDevice) != cudaSuccess)
      return bail(MHD_E_NOMEM, "geometry upload failed");
  }
  {
    std::vector<int> gm = mhd::ghost_maps(g.nx0, g.ny0, g.nz0, g.ng, prm->bc);
    if (cudaMalloc(&h->gmap, sizeof(int) * gm.size()) != cudaSuccess ||
        cudaMemcpy(h->gmap, gm.data(), sizeof(int) * gm.size(), cudaMemcpyHostToDevice) != cudaSuccess)
      return bail(MHD_E_NOMEM, "ghost map upload failed");
  }
  Scal s{};
  s.tau = prm->tau;
  s.tau0 = prm->tau;
  s.dt_cfl = 0.0;
  s.ab_coef = 0.0;
  double inf = INFINITY;
  std::memcpy(&s.dtmin_bits, &inf, sizeof(double));
  std::memcpy(&s.dtnext_bits, &inf, sizeof(double));
  s.status = 0;
  s.pend_status = 0;
  if (cudaMemcpy(h->sc, &s, sizeof(Scal), cudaMemcpyHostToDevice) != cudaSuccess)
    return bail(MHD_E_CUDA, "scalar upload failed");
  if (h->fp32) carve<float>(h, h->df, (char*)h->buf);
  else carve<double>(h, h->dd, (char*)h->buf);
  *out = h;
  return MHD_OK;
}

int mhd_init(const mhd_params* prm, const double* rho, const double* vx, const double* vy,
             const double* vz, const double* p, const double* bi, const double* bj, const double* bk,
             const double* dx, const double* dy, const double* dz, void** handle) {
  if (!handle) return fail(MHD_E_ARG, "null handle pointer");
  *handle = nullptr;
  int rc = validate(prm);
  if (rc) return rc;
  if (!rho || !vx || !vy || !vz || !p || !bi || !bj || !bk || !dx || !dy || !dz)
    return fail(MHD_E_ARG, "null field pointer");
  Handle* h = nullptr;
  rc = create_handle(prm, dx, dy, dz, &h);
  if (rc) return rc;
  const double* arrs[8] = {rho, vx, vy, vz, p, bi, bj, bk};
  rc = h->fp32 ? upload<float>(h, arrs) : upload<double>(h, arrs);
  if (rc) { std::string m = g_err; mhd_free(h); return fail(rc, m); }
  rc = h->fp32 ? init_device<float, false>(h) : init_device<double, false>(h);
  if (rc) { std::string m = g_err; mhd_free(h); return fail(rc, m); }
  *handle = h;
  return MHD_OK;
}

// Metric mode: upload the node coordinates, compute the FP64 metric on the
// device, reject meshes with a non-positive interior cell volume.
static int setup_metric(Handle* h, const double* const xyz[3]) {
  const Geom& g = h->g;
  const size_t nn = (size_t)(g.nx + 1) * (g.ny + 1) * (g.nz + 1);
  h->nodes.resize(3 * nn);
  for (int a = 0; a < 3; ++a) std::memcpy(h->nodes.data() + a * nn, xyz[a], nn * sizeof(double));
  for (double v : h->nodes)
    if (!std::isfinite(v)) return fail(MHD_E_ARG, "node coordinates must be finite");
  double* dn = nullptr;
  double* mv = nullptr;
  CK(cudaMalloc(&dn, sizeof(double) * 3 * (size_t)g.vol + sizeof(double)));
  mv = dn + 3 * (size_t)g.vol;
  int rc = MHD_OK;
  if (cudaMemsetAsync(dn, 0, sizeof(double) * 3 * (size_t)g.vol, h->st) != cudaSuccess)
    rc = fail(MHD_E_CUDA, "metric set-up memset failed");
  std::vector<double> stage(rc ? 0 : (size_t)g.vol);
  for (int a = 0; a < 3 && rc == MHD_OK; ++a) {
    pack<double>(g, h->nodes.data() + a * nn, g.nx + 1, g.ny + 1, g.nz + 1, stage.data());
    if (cudaMemcpyAsync(dn + a * (size_t)g.vol, stage.data(), sizeof(double) * (size_t)g.vol,
                        cudaMemcpyHostToDevice, h->st) != cudaSuccess ||
        cudaStreamSynchronize(h->st) != cudaSuccess)
      rc = fail(MHD_E_CUDA, "node coordinate upload failed");
  }
  double vmin = 0.0;
  if (rc == MHD_OK) {
    metric_geometry(g, dn, dn + (size_t)g.vol, dn + 2 * (size_t)g.vol, metric_out(h), mv, h->st);
    if (cudaGetLastError() != cudaSuccess) rc = fail(MHD_E_CUDA, "metric kernels failed to launch");
  }
  if (rc == MHD_OK) {
    if (cudaMemcpyAsync(&vmin, mv, sizeof(double), cudaMemcpyDeviceToHost, h->st) != cudaSuccess)
      rc = fail(MHD_E_CUDA, "metric read-back failed");
    else rc = wait_stream(h);
  }
  cudaFree(dn);
  if (rc) return rc;
  if (!(vmin > 0.0)) return fail(MHD_E_ARG, "mapped grid has a non-positive cell volume");
  // the Dev views were carved before the metric existed: refresh them
  if (h->fp32) carve<float>(h, h->df, (char*)h->buf);
  else carve<double>(h, h->dd, (char*)h->buf);
  return MHD_OK;
}

int mhd_init_mapped(const mhd_params* prm, const double* rho, const double* vx, const double* vy,
                    const double* vz, const double* p, const double* phi_i, const double* phi_j,
                    const double* phi_k, const double* xn, const double* yn, const double* zn, void** handle) {
  if (!handle) return fail(MHD_E_ARG, "null handle pointer");
  *handle = nullptr;
  int rc = validate(prm);
  if (rc) return rc;
  if (prm->emf == MHD_EMF_YEE) return fail(MHD_E_ARG, "the Yee EMF runs on Cartesian meshes only");
  if (!rho || !vx || !vy || !vz || !p || !phi_i || !phi_j || !phi_k || !xn || !yn || !zn)
    return fail(MHD_E_ARG, "null field pointer");
  const int nx = prm->nx0 + prm->nord, ny = prm->ny0 + prm->nord, nz = prm->nz0 + prm->nord;
  std::vector<double> ones((size_t)nx + ny + nz, 1.0);
  Handle* h = nullptr;
  rc = create_handle(prm, ones.data(), ones.data() + nx, ones.data() + nx + ny, &h, true);
  if (rc) return rc;
  const double* xyz[3] = {xn, yn, zn};
  rc = setup_metric(h, xyz);
  if (rc) { std::string m = g_err; mhd_free(h); return fail(rc, m); }
  const double* arrs[8] = {rho, vx, vy, vz, p, phi_i, phi_j, phi_k};
  rc = h->fp32 ? upload<float>(h, arrs) : upload<double>(h, arrs);
  if (rc) { std::string m = g_err; mhd_free(h); return fail(rc, m); }
  rc = h->fp32 ? init_device<float, true>(h) : init_device<double, true>(h);
  if (rc) { std::string m = g_err; mhd_free(h); return fail(rc, m); }
  *handle = h;
  return MHD_OK;
}

// ---- checkpoint / restart
static const char kMagic[17] = "MHDGB300CKPT0001";

template <typename T>
static void ckpt_arrays(Handle* h, std::vector<std::pair<uint32_t, void*>>& out) {
  Dev<T> d = at_par(dev<T>(h), h->par);
  T* st[11] = {d.rho, d.vx, d.vy, d.vz, d.p, d.bi, d.bj, d.bk, d.bx, d.by, d.bz};
  for (uint32_t a = 0; a < 11; ++a) out.push_back({a, (void*)st[a]});
  if (h->prm.stepop == MHD_STEP_AB2)
    for (uint32_t a = 0; a < 11; ++a) out.push_back({100 + a, (void*)d.q[a]});
}

int mhd_checkpoint_save(void* handle, const char* path) {
  Handle* h = (Handle*)handle;
  if (!h || !path) return fail(MHD_E_ARG, "null argument");
  int rc = wait_stream(h);
  if (rc) return rc;
  FILE* f = std::fopen(path, "wb");
  if (!f) return fail(MHD_E_ARG, std::string("cannot open ") + path);
  std::vector<std::pair<uint32_t, void*>> arrs;
  if (h->fp32) ckpt_arrays<float>(h, arrs);
  else ckpt_arrays<double>(h, arrs);
  CK(cudaMemcpy(h->sc_h, h->sc, sizeof(Scal), cudaMemcpyDeviceToHost));
  // version 2: metric mode, with the node coordinates as record 200
  const uint32_t ver = h->metric ? 2 : 1, psz = (uint32_t)sizeof(mhd_params);
  const uint32_t es = h->fp32 ? 4 : 8, na = (uint32_t)arrs.size() + 1 + (h->metric ? 1 : 0);
  const double sc4[4] = {h->sc_h->tau, h->sc_h->tau0, h->sc_h->dt_cfl, h->sc_h->ab_coef};
  bool ok = std::fwrite(kMagic, 1, 16, f) == 16 && std::fwrite(&ver, 4, 1, f) == 1 &&
            std::fwrite(&psz, 4, 1, f) == 1 && std::fwrite(&h->prm, sizeof(mhd_params), 1, f) == 1 &&
            std::fwrite(sc4, 8, 4, f) == 4 && std::fwrite(&es, 4, 1, f) == 1 && std::fwrite(&na, 4, 1, f) == 1;
  const size_t bytes = (size_t)h->g.vol * es;
  std::vector<char> buf(ok ? bytes : 0);
  for (auto& a : arrs) {
    if (!ok) break;
    if (cudaMemcpy(buf.data(), a.second, bytes, cudaMemcpyDeviceToHost) != cudaSuccess) { ok = false; break; }
    const uint64_t nb = bytes;
    ok = std::fwrite(&a.first, 4, 1, f) == 1 && std::fwrite(&nb, 8, 1, f) == 1 &&
         std::fwrite(buf.data(), 1, bytes, f) == bytes;
  }
  if (ok) {  // FP64 cell widths, id 999
    const size_t ng = (size_t)h->g.nx + h->g.ny + h->g.nz;
    std::vector<double> w(ng);
    ok = cudaMemcpy(w.data(), h->geo, ng * 8, cudaMemcpyDeviceToHost) == cudaSuccess;
    const uint32_t id = 999;
    const uint64_t nb = ng * 8;
    ok = ok && std::fwrite(&id, 4, 1, f) == 1 && std::fwrite(&nb, 8, 1, f) == 1 &&
         std::fwrite(w.data(), 8, ng, f) == ng;
  }
  if (ok && h->metric) {  // node coordinates X | Y | Z (FP64, ghost-inclusive, Fortran order)
    const uint32_t id = 200;
    const uint64_t nb = h->nodes.size() * 8;
    ok = std::fwrite(&id, 4, 1, f) == 1 && std::fwrite(&nb, 8, 1, f) == 1 &&
         std::fwrite(h->nodes.data(), 8, h->nodes.size(), f) == h->nodes.size();
  }
  ok = (std::fclose(f) == 0) && ok;
  if (!ok) return fail(MHD_E_ARG, std::string("checkpoint write failed: ") + path);
  return MHD_OK;
}

int mhd_checkpoint_load(const char* path, void** handle) {
  if (!path || !handle) return fail(MHD_E_ARG, "null argument");
  *handle = nullptr;
  FILE* f = std::fopen(path, "rb");
  if (!f) return fail(MHD_E_ARG, std::string("cannot open ") + path);
  char magic[16];
  uint32_t ver = 0, psz = 0, es = 0, na = 0;
  mhd_params prm{};
  double sc4[4];
  bool ok = std::fread(magic, 1, 16, f) == 16 && std::memcmp(magic, kMagic, 16) == 0 &&
            std::fread(&ver, 4, 1, f) == 1 && (ver == 1 || ver == 2) && std::fread(&psz, 4, 1, f) == 1 &&
            psz == sizeof(mhd_params) && std::fread(&prm, sizeof(mhd_params), 1, f) == 1 &&
            std::fread(sc4, 8, 4, f) == 4 && std::fread(&es, 4, 1, f) == 1 && std::fread(&na, 4, 1, f) == 1;
  if (!ok || validate(&prm) != MHD_OK || es != (prm.precision == MHD_FP32 ? 4u : 8u)) {
    std::fclose(f);
    return fail(MHD_E_ARG, std::string("not a compatible checkpoint: ") + path);
  }
  // geometry is not stored: widths come back from the widths array below
  const int nx = prm.nx0 + prm.nord, ny = prm.ny0 + prm.nord, nz = prm.nz0 + prm.nord;
  std::vector<double> ones((size_t)nx + ny + nz, 1.0);
  Handle* h = nullptr;
  const bool metric = (ver == 2);
  const size_t nnodes = (size_t)(nx + 1) * (ny + 1) * (nz + 1);
  int rc = create_handle(&prm, ones.data(), ones.data() + nx, ones.data() + nx + ny, &h, metric);
  if (rc) { std::fclose(f); return rc; }
  std::vector<std::pair<uint32_t, void*>> arrs;
  if (h->fp32) ckpt_arrays<float>(h, arrs);
  else ckpt_arrays<double>(h, arrs);
  const size_t bytes = (size_t)h->g.vol * es;
  std::vector<char> buf(std::max(bytes, metric ? 3 * nnodes * 8 : (size_t)0));
  size_t loaded = 0;
  for (uint32_t n = 0; n < na && ok; ++n) {
    uint32_t id = 0;
    uint64_t nb = 0;
    ok = std::fread(&id, 4, 1, f) == 1 && std::fread(&nb, 8, 1, f) == 1 &&
         (nb == bytes || (id == 999 && nb == ((size_t)nx + ny + nz) * 8) ||
          (metric && id == 200 && nb == 3 * nnodes * 8)) &&
         std::fread(buf.data(), 1, nb, f) == nb;
    if (!ok) break;
    void* dst = nullptr;
    if (id == 200) {  // node coordinates: rebuild the metric
      const double* nd = (const double*)buf.data();
      const double* xyz[3] = {nd, nd + nnodes, nd + 2 * nnodes};
      ok = setup_metric(h, xyz) == MHD_OK;
      ++loaded;
      continue;
    }
    if (id == 999) {  // cell widths (FP64)
      const size_t ng = (size_t)nx + ny + nz;
      ok = cudaMemcpy(h->geo, buf.data(), ng * 8, cudaMemcpyHostToDevice) == cudaSuccess;
      std::vector<float> gf(ng * 2);
      const double* w = (const double*)buf.data();
      for (size_t i = 0; i < ng; ++i) { gf[i] = (float)w[i]; gf[ng + i] = (float)(1.0 / w[i]); }
      ok = ok && cudaMemcpy(h->geoT, gf.data(), gf.size() * 4, cudaMemcpyHostToDevice) == cudaSuccess;
      ++loaded;
      continue;
    }
    for (auto& a : arrs)
      if (a.first == id) dst = a.second;
    if (!dst) { ok = false; break; }
    ok = cudaMemcpy(dst, buf.data(), bytes, cudaMemcpyHostToDevice) == cudaSuccess;
    ++loaded;
  }
  std::fclose(f);
  if (!ok || loaded != arrs.size() + 1 + (metric ? 1 : 0)) {
    mhd_free(h);
    return fail(MHD_E_ARG, std::string("checkpoint is truncated or inconsistent: ") + path);
  }
  Scal s{};
  s.tau = sc4[0]; s.tau0 = sc4[1]; s.dt_cfl = sc4[2]; s.ab_coef = sc4[3];
  double inf = INFINITY;
  std::memcpy(&s.dtmin_bits, &inf, sizeof(double));
  std::memcpy(&s.dtnext_bits, &inf, sizeof(double));
  if (cudaMemcpy(h->sc, &s, sizeof(Scal), cudaMemcpyHostToDevice) != cudaSuccess) {
    mhd_free(h);
    return fail(MHD_E_CUDA, "scalar upload failed");
  }
  // vf (and cell B) as the end of the saved step left them: the same fused
  // kernel the step runs, on the restored fields
  const bool want_vf = prm.stepop != MHD_STEP_AB2;
  if (h->fp32) {
    if (metric) Launch<float, true>::fill_bxyz(h->df, want_vf, h->st);
    else Launch<float>::fill_bxyz(h->df, want_vf, h->st);
  } else {
    if (metric) Launch<double, true>::fill_bxyz(h->dd, want_vf, h->st);
    else Launch<double>::fill_bxyz(h->dd, want_vf, h->st);
  }
  rc = wait_stream(h);
  if (rc) {
    std::string m = g_err;
    mhd_free(h);
    return fail(rc, m);
  }
  *handle = h;
  return MHD_OK;
}

int mhd_step_n(void* handle, int32_t nsteps, double* tau_out, uint32_t* status) {
  Handle* h = (Handle*)handle;
  if (!h) return fail(MHD_E_ARG, "null handle");
  if (nsteps < 0) return fail(MHD_E_ARG, "nsteps < 0");
  int rc = h->fp32 ? do_steps<float>(h, nsteps) : do_steps<double>(h, nsteps);
  if (rc) {
    if (status) *status = MHD_ST_CUDA_ERROR;
    return rc;
  }
  return finish(h, tau_out, status);
}

// Sets the fixed RK dt (Scal::tau, Scal::tau0) in stream order, without a host wait.
__global__ void k_set_tau(Scal* sc, double tau) {
  sc->tau = tau;
  sc->tau0 = tau;
}

int mhd_step(void* handle, double* tau_inout, uint32_t* status) {
  Handle* h = (Handle*)handle;
  if (!h) return fail(MHD_E_ARG, "null handle");
  // tau in: the driver's module tau.  RK steps with the reference dt take the
  // fixed deck dt tau0 (step_rk2/3, mhd3d3.f90:3656-3661); a positive value
  // that differs from it becomes the new fixed dt before the step.  AB steps
  // and the CFL dt mode compute their dt on the device (get_dt) and ignore it.
  if (tau_inout && *tau_inout > 0.0 && std::isfinite(*tau_inout) && h->prm.stepop != MHD_STEP_AB2 &&
      h->prm.dt_mode == MHD_DT_REFERENCE && *tau_inout != h->prm.tau) {
    k_set_tau<<<1, 1, 0, h->st>>>(h->sc, *tau_inout);
    CK(cudaGetLastError());
    h->prm.tau = *tau_inout;
  }
  return mhd_step_n(handle, 1, tau_inout, status);
}

static int graph_for(Handle* h, int nsteps, cudaGraphExec_t* out);

int mhd_step_graph(void* handle, int32_t nsteps, double* tau_out, uint32_t* status) {
  Handle* h = (Handle*)handle;
  if (!h) return fail(MHD_E_ARG, "null handle");
  if (nsteps <= 0) return fail(MHD_E_ARG, "nsteps must be positive");
  cudaGraphExec_t ex = nullptr;
  int rc = graph_for(h, nsteps, &ex);
  if (rc) return rc;
  CK(cudaGraphLaunch(ex, h->st));
  return finish(h, tau_out, status);
}

static int graph_for(Handle* h, int nsteps, cudaGraphExec_t* out) {
  // the first captured step differs when the state was changed between steps
  auto key = std::make_pair(nsteps, h->par + (h->prepared ? 2 : 0));
  auto it = h->graphs.find(key);
  if (it != h->graphs.end()) {
    *out = it->second.first;
    h->par = it->second.second & 1;  // the replay leaves this half current
    h->prepared = (it->second.second & 2) != 0;
    return MHD_OK;
  }
  cudaGraph_t gr;
  cudaGraphExec_t ex;
  int par = h->par;
  CK(cudaStreamBeginCapture(h->st, cudaStreamCaptureModeThreadLocal));
  for (int s = 0; s < nsteps; ++s) {
    if (h->fp32) enqueue_any<float>(h, par, h->st);
    else enqueue_any<double>(h, par, h->st);
  }
  CK(cudaStreamEndCapture(h->st, &gr));
  CK(cudaGraphInstantiate(&ex, gr, 0));
  cudaGraphDestroy(gr);
  h->graphs[key] = std::make_pair(ex, par + (h->prepared ? 2 : 0));
  h->par = par;
  *out = ex;
  return MHD_OK;
}

int mhd_time_steps(void* handle, int32_t nsteps, int32_t use_graph, float* ms) {
  Handle* h = (Handle*)handle;
  if (!h || !ms || nsteps <= 0) return fail(MHD_E_ARG, "bad arguments");
  cudaGraphExec_t ex = nullptr;
  if (use_graph) {
    int rc = graph_for(h, nsteps, &ex);
    if (rc) return rc;
  }
  CK(cudaEventRecord(h->ev[0], h->st));
  if (use_graph) {
    CK(cudaGraphLaunch(ex, h->st));
  } else {
    int rc = h->fp32 ? do_steps<float>(h, nsteps) : do_steps<double>(h, nsteps);
    if (rc) return rc;
  }
  CK(cudaEventRecord(h->ev[1], h->st));
  int rc = wait_stream(h);
  if (rc) return rc;
  CK(cudaEventElapsedTime(ms, h->ev[0], h->ev[1]));
  return MHD_OK;
}

int mhd_set_tau(void* handle, double tau) {
  Handle* h = (Handle*)handle;
  if (!h || !(tau > 0.0)) return fail(MHD_E_ARG, "bad handle or tau");
  int rc = wait_stream(h);
  if (rc) return rc;
  CK(cudaMemcpy(h->sc_h, h->sc, sizeof(Scal), cudaMemcpyDeviceToHost));
  h->sc_h->tau = tau;
  h->sc_h->tau0 = tau;
  CK(cudaMemcpy(h->sc, h->sc_h, sizeof(Scal), cudaMemcpyHostToDevice));
  h->prm.tau = tau;
  return MHD_OK;
}

int mhd_set_profiling(void* handle, int32_t on) {
  Handle* h = (Handle*)handle;
  if (!h) return fail(MHD_E_ARG, "null handle");
  h->profile = on != 0;
  return MHD_OK;
}

int mhd_last_timings(void* handle, float out_ms[8]) {
  Handle* h = (Handle*)handle;
  if (!h || !out_ms) return fail(MHD_E_ARG, "null argument");
  for (int i = 0; i < 8; ++i) out_ms[i] = h->tms[i];
  return MHD_OK;
}

// Writes the first byte of every page of a caller's output array on all host
// threads.  A copy into pages the process has not touched yet would take
// their first-touch faults one at a time inside the copy; already-mapped pages
// cost one store each.  The array is overwritten right after.
static void prefault(double* p, size_t bytes) {
  const size_t page = (size_t)sysconf(_SC_PAGESIZE);
  char* c = reinterpret_cast<char*>(p);
  const long long npg = (long long)((bytes + page - 1) / page);
#pragma omp parallel for schedule(static)
  for (long long k = 0; k < npg; ++k) c[(size_t)k * page] = 0;
}

// Device-side conversion to FP64, then a copy straight into the caller's arrays.
template <typename T>
static int fetch_t(Handle* h, double* const* outs) {
  const Geom& g = h->g;
  Dev<T> d = at_par(dev<T>(h), h->par);
  const T* srcs[11] = {d.rho, d.vx, d.vy, d.vz, d.p, d.bx, d.by, d.bz, d.bi, d.bj, d.bk};
  int ext[11][3];
  for (int a = 0; a < 8; ++a) { ext[a][0] = g.nx; ext[a][1] = g.ny; ext[a][2] = g.nz; }
  ext[8][0] = g.nx + 1; ext[8][1] = g.ny; ext[8][2] = g.nz;
  ext[9][0] = g.nx; ext[9][1] = g.ny + 1; ext[9][2] = g.nz;
  ext[10][0] = g.nx; ext[10][1] = g.ny; ext[10][2] = g.nz + 1;
  double* scratch = f64_scratch(d);
  for (int a = 0; a < 11; ++a)
    if (outs[a]) prefault(outs[a], sizeof(double) * (size_t)ext[a][0] * ext[a][1] * ext[a][2]);
  for (int a = 0; a < 11; ++a) {
    if (!outs[a]) continue;
    const int ex = ext[a][0], ey = ext[a][1], ez = ext[a][2];
    k_to_f64<T><<<dim3((ex + 255) / 256, ey, ez), 256, 0, h->st>>>(srcs[a], ex, ey, g.px, g.plane, scratch);
    CK(cudaMemcpyAsync(outs[a], scratch, sizeof(double) * (size_t)ex * ey * ez, cudaMemcpyDeviceToHost, h->st));
  }
  CK(cudaGetLastError());
  return wait_stream(h);
}

int mhd_fetch(void* handle, double* rho, double* vx, double* vy, double* vz, double* p, double* bx,
              double* by, double* bz, double* bi, double* bj, double* bk) {
  Handle* h = (Handle*)handle;
  if (!h) return fail(MHD_E_ARG, "null handle");
  double* outs[11] = {rho, vx, vy, vz, p, bx, by, bz, bi, bj, bk};
  return h->fp32 ? fetch_t<float>(h, outs) : fetch_t<double>(h, outs);
}

template <typename T, bool M>
static int diag_t(Handle* h, double out[5]) {
  Dev<T> d = at_par(dev<T>(h), h->par);
  Launch<T, M>::diagnostics(d, h->diag, h->st);
  CK(cudaGetLastError());
  CK(cudaMemcpyAsync(h->diag_h, h->diag, sizeof(double) * 4, cudaMemcpyDeviceToHost, h->st));
  int rc = wait_stream(h);
  if (rc) return rc;
  for (int i = 0; i < 4; ++i) out[i] = h->diag_h[i];
  // CFL dt of the current state: the dt kernel in "peek" mode (status kept)
  Launch<T, M>::cfl(d, 3, h->st);
  CK(cudaMemcpyAsync(h->sc_h, h->sc, sizeof(Scal), cudaMemcpyDeviceToHost, h->st));
  rc = wait_stream(h);
  if (rc) return rc;
  out[4] = h->sc_h->dt_cfl;
  return MHD_OK;
}

int mhd_diagnostics(void* handle, double out[5]) {
  Handle* h = (Handle*)handle;
  if (!h || !out) return fail(MHD_E_ARG, "null argument");
  if (h->metric) return h->fp32 ? diag_t<float, true>(h, out) : diag_t<double, true>(h, out);
  return h->fp32 ? diag_t<float, false>(h, out) : diag_t<double, false>(h, out);
}

template <typename T, bool M>
static int dbg_flux_t(Handle* h, double* out) {
  const Geom& g = h->g;
  Dev<T> d = at_par(dev<T>(h), h->par);
  // the y / z face fluxes go to scratch of this call (the handle keeps none)
  T* yz = nullptr;
  if (cudaMalloc(&yz, 16 * (size_t)g.vol * sizeof(T)) != cudaSuccess)
    return fail(MHD_E_NOMEM, "debug fluxes: device allocation failed");
  for (int ax = 1; ax < 3; ++ax)
    for (int q = 0; q < 8; ++q) d.F[ax][q] = yz + (size_t)((ax - 1) * 8 + q) * (size_t)g.vol;
  struct Free {
    T* p;
    ~Free() { cudaFree(p); }
  } release{yz};
  Launch<T, M>::fluxes(d, state_inp(d), h->st);
  CK(cudaGetLastError());
  std::vector<T> host((size_t)g.vol);
  size_t off = 0;
  for (int ax = 0; ax < 3; ++ax) {
    int ex = g.nx0 + (ax == 0), ey = g.ny0 + (ax == 1), ez = g.nz0 + (ax == 2);
    for (int q = 0; q < 8; ++q) {
      CK(cudaMemcpyAsync(host.data(), d.F[ax][q], (size_t)g.vol * sizeof(T), cudaMemcpyDeviceToHost, h->st));
      int rc = wait_stream(h);
      if (rc) return rc;
      for (int k = 0; k < ez; ++k)
        for (int j = 0; j < ey; ++j)
          for (int i = 0; i < ex; ++i)
            out[off + i + (size_t)ex * (j + (size_t)ey * k)] =
                (double)host[(size_t)(i + g.ng) + (size_t)g.px * ((j + g.ng) + (size_t)g.py * (k + g.ng))];
      off += (size_t)ex * ey * ez;
    }
  }
  return MHD_OK;
}

int mhd_debug_fluxes(void* handle, double* out) {
  Handle* h = (Handle*)handle;
  if (!h || !out) return fail(MHD_E_ARG, "null argument");
  if (h->metric) return h->fp32 ? dbg_flux_t<float, true>(h, out) : dbg_flux_t<double, true>(h, out);
  return h->fp32 ? dbg_flux_t<float, false>(h, out) : dbg_flux_t<double, false>(h, out);
}

template <typename T, bool M>
static int dbg_emf_t(Handle* h, double* const* outs) {
  const Geom& g = h->g;
  Dev<T> d = at_par(dev<T>(h), h->par);
  Launch<T, M>::bxyz_vf(d, true, h->st);
  Launch<T, M>::emf(d, state_inp(d), h->st);
  CK(cudaGetLastError());
  std::vector<T> host((size_t)g.vol);
  for (int e = 0; e < 3; ++e) {
    if (!outs[e]) continue;
    int ex = g.nx0 + (e != 0), ey = g.ny0 + (e != 1), ez = g.nz0 + (e != 2);
    CK(cudaMemcpyAsync(host.data(), d.E[e], (size_t)g.vol * sizeof(T), cudaMemcpyDeviceToHost, h->st));
    int rc = wait_stream(h);
    if (rc) return rc;
    for (int k = 0; k < ez; ++k)
      for (int j = 0; j < ey; ++j)
        for (int i = 0; i < ex; ++i)
          outs[e][i + (size_t)ex * (j + (size_t)ey * k)] =
              (double)host[(size_t)(i + g.ng) + (size_t)g.px * ((j + g.ng) + (size_t)g.py * (k + g.ng))];
  }
  return MHD_OK;
}

int mhd_debug_emf(void* handle, double* ei, double* ej, double* ek) {
  Handle* h = (Handle*)handle;
  if (!h) return fail(MHD_E_ARG, "null handle");
  double* outs[3] = {ei, ej, ek};
  if (h->metric) return h->fp32 ? dbg_emf_t<float, true>(h, outs) : dbg_emf_t<double, true>(h, outs);
  return h->fp32 ? dbg_emf_t<float, false>(h, outs) : dbg_emf_t<double, false>(h, outs);
}

// ---- ensembles
// Device tables of a batched ensemble (see Batch in mhd_state.h).
struct BatchBufs {
  void* tabs = nullptr;
  int4* maps = nullptr;
  BatchView view{};
};

// Grids that can share one batched launch per kernel family: same precision,
// Cartesian, PDM, the same RK stepper, dt mode and limiter constants.
static bool batchable(Handle* const* hs, int n) {
  const mhd_params& a = hs[0]->prm;
  if (hs[0]->metric || a.reconop != MHD_RECON_PDM || a.emf != MHD_EMF_LFM ||
      (a.stepop != MHD_STEP_RK2 && a.stepop != MHD_STEP_RK3))
    return false;
  for (int i = 1; i < n; ++i) {
    const mhd_params& b = hs[i]->prm;
    if (hs[i]->metric || hs[i]->fp32 != hs[0]->fp32 || b.reconop != a.reconop || b.stepop != a.stepop ||
        b.dt_mode != a.dt_mode || b.pdmb != a.pdmb || b.eps != a.eps || b.alpha != a.alpha || b.beta != a.beta ||
        b.tvd_shift != a.tvd_shift || b.emf != a.emf)
      return false;
  }
  return true;
}

template <typename T>
static int build_batch(Handle* const* hs, int n, BatchBufs& b) {
  std::vector<Dev<T>> tab(2 * (size_t)n);
  for (int i = 0; i < n; ++i) {
    tab[i] = at_par(dev<T>(hs[i]), hs[i]->par);
    tab[n + i] = at_par(dev<T>(hs[i]), hs[i]->par ^ 1);
  }
  std::vector<int4> map;
  size_t off[BF_COUNT];
  for (int f = 0; f < BF_COUNT; ++f) {
    off[f] = map.size();
    for (int i = 0; i < n; ++i) {
      const dim3 dd = Batch<T>::dims(f, hs[i]->g, hs[0]->tile_td, hs[0]->tile_ey);
      for (unsigned z = 0; z < dd.z; ++z)
        for (unsigned y = 0; y < dd.y; ++y)
          for (unsigned x = 0; x < dd.x; ++x) map.push_back(make_int4(i, (int)x, (int)y, (int)z));
    }
    const size_t nb = map.size() - off[f];
    if (nb >= (size_t)INT32_MAX) return fail(MHD_E_ARG, "ensemble too large for one launch per kernel family");
    b.view.nblk[f] = (int)nb;
  }
  CK(cudaMalloc(&b.tabs, sizeof(Dev<T>) * tab.size()));
  CK(cudaMalloc(&b.maps, sizeof(int4) * map.size()));
  CK(cudaMemcpy(b.tabs, tab.data(), sizeof(Dev<T>) * tab.size(), cudaMemcpyHostToDevice));
  CK(cudaMemcpy(b.maps, map.data(), sizeof(int4) * map.size(), cudaMemcpyHostToDevice));
  b.view.tab[0] = b.tabs;
  b.view.tab[1] = (const Dev<T>*)b.tabs + n;
  for (int f = 0; f < BF_COUNT; ++f) b.view.map[f] = b.maps + off[f];
  b.view.ngrids = n;
  const mhd_params& p = hs[0]->prm;
  b.view.pdmb = p.pdmb; b.view.eps = p.eps; b.view.alpha = p.alpha; b.view.beta = p.beta;
  b.view.tvd_shift = p.tvd_shift;
  b.view.tile_td = hs[0]->tile_td;
  b.view.tile_ey = hs[0]->tile_ey;
  return MHD_OK;
}

// nsteps RK steps of every grid of a batch; returns the number of half swaps.
// The EMF families of a stage run on the side stream st2 beside the face
// fluxes (they read the same stage input and write disjoint arrays), joined
// before CT, as a single grid's stage runs them.
template <typename T>
static int enqueue_batch(const BatchView& v, int stepop, int dt_mode, int nsteps, cudaStream_t st,
                         cudaStream_t st2, cudaEvent_t fork, cudaEvent_t join) {
  int flips = 0;
  const int nst = (stepop == MHD_STEP_RK2) ? 2 : 3;
  for (int s = 0; s < nsteps; ++s) {
    Batch<T>::cfl(v, flips & 1, dt_mode == MHD_DT_CFL ? 1 : 0, st);
    for (int k = 1; k <= nst; ++k) {
      int form = -1;
      double c = 0.0, den = 1.0;
      if (k > 1) {
        if (nst == 2) { form = 0; den = 2.0; }
        else if (k == 2) { form = 1; c = 3.0; den = 4.0; }
        else { form = 2; c = 2.0; den = 3.0; }
      }
      const int sel = flips & 1;
      // (a failed record or wait surfaces when the capture ends)
      cudaEventRecord(fork, st);
      cudaStreamWaitEvent(st2, fork, 0);
      Batch<T>::parts(v, sel, 1, form, c, den, st2);
      Batch<T>::parts(v, sel, 2, form, c, den, st);
      cudaEventRecord(join, st2);
      cudaStreamWaitEvent(st, join, 0);
      Batch<T>::parts(v, sel, 4, form, c, den, st);
      ++flips;
    }
  }
  return flips;
}

// Graph of nsteps steps of every grid: batched (one launch per kernel family
// over all grids) when the grids allow it, else one branch per grid.
static int capture_ensemble(const std::vector<Handle*>& hs, int nsteps, cudaGraphExec_t* ex,
                            std::vector<int>& pars, BatchBufs& bufs) {
  Handle* h0 = hs[0];
  const int n = (int)hs.size();
  pars.resize(n);
  cudaGraph_t gr = nullptr;
  if (batchable(hs.data(), n)) {
    int rc = h0->fp32 ? build_batch<float>(hs.data(), n, bufs) : build_batch<double>(hs.data(), n, bufs);
    if (rc) return rc;
    CK(cudaStreamBeginCapture(h0->st, cudaStreamCaptureModeThreadLocal));
    const int flips =
        h0->fp32 ? enqueue_batch<float>(bufs.view, h0->prm.stepop, h0->prm.dt_mode, nsteps, h0->st, h0->st2,
                                        h0->ev_fork, h0->ev_join)
                 : enqueue_batch<double>(bufs.view, h0->prm.stepop, h0->prm.dt_mode, nsteps, h0->st, h0->st2,
                                         h0->ev_fork, h0->ev_join);
    CK(cudaStreamEndCapture(h0->st, &gr));
    for (int i = 0; i < n; ++i) pars[i] = hs[i]->par ^ (flips & 1);
  } else {
    cudaEvent_t fork;
    CK(cudaEventCreateWithFlags(&fork, cudaEventDisableTiming));
    std::vector<cudaEvent_t> joins(n, nullptr);
    CK(cudaStreamBeginCapture(h0->st, cudaStreamCaptureModeThreadLocal));
    cudaEventRecord(fork, h0->st);
    for (int i = 1; i < n; ++i) cudaStreamWaitEvent(hs[i]->st, fork, 0);
    for (int i = 0; i < n; ++i) {
      Handle* h = hs[i];
      int par = h->par;
      for (int s = 0; s < nsteps; ++s) {
        if (h->fp32) enqueue_any<float>(h, par, h->st);
        else enqueue_any<double>(h, par, h->st);
      }
      pars[i] = par;
      if (i > 0) {
        cudaEventCreateWithFlags(&joins[i], cudaEventDisableTiming);
        cudaEventRecord(joins[i], h->st);
        cudaStreamWaitEvent(h0->st, joins[i], 0);
      }
    }
    cudaError_t e = cudaStreamEndCapture(h0->st, &gr);
    for (int i = 1; i < n; ++i)
      if (joins[i]) cudaEventDestroy(joins[i]);
    cudaEventDestroy(fork);
    if (e != cudaSuccess) return fail(MHD_E_CUDA, std::string("ensemble capture: ") + cudaGetErrorString(e));
  }
  cudaError_t e = cudaGraphInstantiate(ex, gr, 0);
  cudaGraphDestroy(gr);
  if (e != cudaSuccess) return fail(MHD_E_CUDA, std::string("ensemble graph: ") + cudaGetErrorString(e));
  return MHD_OK;
}

// Cached ensemble graphs, keyed by (grid uid, half) pairs, nsteps and the
// launch shapes; entries holding a grid are dropped when it is freed.
struct EnsEntry {
  cudaGraphExec_t ex = nullptr;
  std::vector<int> par_end;
  BatchBufs bufs;
};
static std::mutex g_ens_mu;
static std::map<std::vector<unsigned long long>, EnsEntry> g_ens_cache;

static void ens_release(EnsEntry& en) {
  if (en.ex) cudaGraphExecDestroy(en.ex);
  if (en.bufs.tabs) cudaFree(en.bufs.tabs);
  if (en.bufs.maps) cudaFree(en.bufs.maps);
  en = EnsEntry{};
}

// Drop every cached ensemble graph that steps grid `uid`.
static void ens_forget(unsigned long long uid) {
  std::lock_guard<std::mutex> lk(g_ens_mu);
  for (auto it = g_ens_cache.begin(); it != g_ens_cache.end();) {
    bool has = false;
    const auto& k = it->first;
    for (size_t i = 0; i + 2 < k.size(); i += 2) has = has || k[i] == uid;
    if (has) {
      ens_release(it->second);
      it = g_ens_cache.erase(it);
    } else {
      ++it;
    }
  }
}

// Ensemble: nsteps steps of every grid in one CUDA graph on the first grid's
// stream; graphs cached per (grids, their current halves, nsteps, shapes).
// Enqueues the graph (after the work already queued on every grid's stream)
// and returns; ev_after (optional) is recorded right after it.
static int ens_launch(void** handles, int32_t ngrids, int32_t nsteps, std::vector<Handle*>& hs,
                      cudaEvent_t ev_before, cudaEvent_t ev_after) {
  if (!handles || ngrids <= 0 || nsteps <= 0) return fail(MHD_E_ARG, "bad ensemble arguments");
  hs.assign(ngrids, nullptr);
  for (int i = 0; i < ngrids; ++i) {
    Handle* h = (Handle*)handles[i];
    if (!h) return fail(MHD_E_ARG, "null handle in ensemble");
    if (h->fp32 != ((Handle*)handles[0])->fp32) return fail(MHD_E_ARG, "ensemble grids must share the precision");
    for (int j = 0; j < i; ++j)
      if (hs[j] == h) return fail(MHD_E_ARG, "a grid appears twice in the ensemble");
    hs[i] = h;
  }
  Handle* h0 = hs[0];
  std::lock_guard<std::mutex> lk(g_ens_mu);
  std::vector<unsigned long long> key;
  for (Handle* h : hs) {
    key.push_back(h->uid);
    key.push_back((unsigned long long)h->par);
  }
  key.push_back((unsigned long long)nsteps);
  key.push_back((unsigned long long)(h0->tile_td * 64 + h0->tile_ey));  // the batch's launch shapes
  auto it = g_ens_cache.find(key);
  if (it == g_ens_cache.end()) {
    EnsEntry en;
    int rc = capture_ensemble(hs, nsteps, &en.ex, en.par_end, en.bufs);
    if (rc) {
      ens_release(en);
      return rc;
    }
    it = g_ens_cache.emplace(key, en).first;
  }
  // order the graph after work already queued on every grid's own stream
  for (int i = 1; i < ngrids; ++i) {
    cudaEvent_t e;
    CK(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
    CK(cudaEventRecord(e, hs[i]->st));
    CK(cudaStreamWaitEvent(h0->st, e, 0));
    cudaEventDestroy(e);
  }
  for (int i = 0; i < ngrids; ++i) {
    hs[i]->par = it->second.par_end[i];
    hs[i]->prepared = false;  // batched steps run their own CFL pass
  }
  if (ev_before) CK(cudaEventRecord(ev_before, h0->st));
  CK(cudaGraphLaunch(it->second.ex, h0->st));
  if (ev_after) CK(cudaEventRecord(ev_after, h0->st));
  return MHD_OK;
}

int mhd_ensemble_step(void** handles, int32_t ngrids, int32_t nsteps, uint32_t* status) {
  std::vector<Handle*> hs;
  int rc = ens_launch(handles, ngrids, nsteps, hs, nullptr, nullptr);
  if (rc) return rc;
  // h0's stream carries the whole graph: waiting on it first covers every grid
  uint32_t acc = 0;
  for (int i = 0; i < ngrids; ++i) {
    uint32_t st = 0;
    int rc = finish(hs[i], nullptr, &st);
    if (rc) return rc;
    acc |= st;
  }
  if (status) *status = acc;
  return MHD_OK;
}

// The same nsteps-step ensemble graph as mhd_ensemble_step, bracketed by two
// CUDA events on the stream that carries it; *ms = their elapsed device time.
int mhd_ensemble_time(void** handles, int32_t ngrids, int32_t nsteps, float* ms) {
  if (!ms) return fail(MHD_E_ARG, "null output");
  if (!handles || ngrids <= 0 || !handles[0]) return fail(MHD_E_ARG, "bad ensemble arguments");
  Handle* h0 = (Handle*)handles[0];
  std::vector<Handle*> hs;
  int rc = ens_launch(handles, ngrids, nsteps, hs, h0->ev[2], h0->ev[3]);
  if (rc) return rc;
  for (Handle* h : hs) {  // read back and clear each grid's status, as mhd_ensemble_step does
    uint32_t st = 0;
    rc = finish(h, nullptr, &st);
    if (rc) return rc;
  }
  CK(cudaEventElapsedTime(ms, h0->ev[2], h0->ev[3]));
  return MHD_OK;
}

// ---- tile autotuner
// Device time (ms) of `reps` runs of fn on stream st, the minimum over runs.
template <typename Fn>
static float time_min(cudaStream_t st, int reps, Fn fn) {
  cudaEvent_t a, b;
  cudaEventCreate(&a);
  cudaEventCreate(&b);
  float best = INFINITY;
  fn();  // warm-up (and first-launch attributes)
  for (int r = 0; r < reps; ++r) {
    cudaEventRecord(a, st);
    fn();
    cudaEventRecord(b, st);
    if (cudaEventSynchronize(b) != cudaSuccess) break;
    float ms = 0;
    cudaEventElapsedTime(&ms, a, b);
    best = ms < best ? ms : best;
  }
  cudaEventDestroy(a);
  cudaEventDestroy(b);
  return best;
}

static void drop_graphs(Handle* h) {
  for (auto& kv : h->graphs) cudaGraphExecDestroy(kv.second.first);
  h->graphs.clear();
}

// FP32 Cartesian PDM: face tiles 4/8/16 or the column sweeps, EMF as ei tiles
// 4x4/8x8 or slice streams; the other FP32 Cartesian reconstructions: face tile
// 8 (4 and 16 run as 8) or the column sweeps (their EMF launch shapes are
// fixed, the EMF value is ignored).
static bool tunable(const Handle* h) { return h->fp32 && !h->metric; }

int mhd_autotune(void* handle, int32_t reps, int32_t out[2]) {
  Handle* h = (Handle*)handle;
  if (!h || reps <= 0) return fail(MHD_E_ARG, "bad autotune arguments");
  if (tunable(h)) {
    int rc = wait_stream(h);
    if (rc) return rc;
    // The timed launches (EMF, face fluxes + update) write only scratch (E,
    // F, dU) and the other half of the double buffer, so the state a step
    // starts from is untouched; every tile choice gives the same bits.  Each
    // (face shape, EMF shape) pair is timed as a stage runs it: the EMF
    // families on the side stream beside the face fluxes (a shape that is
    // faster alone is not always the faster one there).
    float best = INFINITY;
    int pick_td = h->tile_td, pick_ey = h->tile_ey;
    for (int td : kTileTD) {
      for (int ey : kTileEY) {
        h->tile_td = td;
        h->tile_ey = ey;
        carve<float>(h, h->df, (char*)h->buf);
        Dev<float> d = at_par(h->df, h->par);
        const Inp<float> in = state_inp(d);
        Rec none;
        const float ms =
            time_min(h->st, reps, [&] { emf_and_fluxes<float, false>(h, d, in, -1, 0.0, 1.0, false, h->st, none); });
        if (ms < best) { best = ms; pick_td = td; pick_ey = ey; }
      }
    }
    h->tile_td = pick_td;
    h->tile_ey = pick_ey;
    carve<float>(h, h->df, (char*)h->buf);
    drop_graphs(h);
    CK(cudaGetLastError());
  }
  if (out) { out[0] = h->tile_td; out[1] = h->tile_ey; }
  return MHD_OK;
}

int mhd_set_tiles(void* handle, int32_t face_tile, int32_t ei_tile) {
  Handle* h = (Handle*)handle;
  if (!h) return fail(MHD_E_ARG, "null handle");
  if (!tunable(h)) {
    if (face_tile != h->tile_td || ei_tile != h->tile_ey)
      return fail(MHD_E_ARG, "this handle's launch shapes are fixed");
    return MHD_OK;
  }
  bool ok_td = false, ok_ey = false;
  for (int td : kTileTD) ok_td |= td == face_tile;
  for (int ey : kTileEY) ok_ey |= ey == ei_tile;
  if (!ok_td || !ok_ey)
    return fail(MHD_E_ARG, "face tile must be 4, 8, 16 or 32 and EMF shape 4, 8 (ei tile) or 1 (slice streams)");
  int rc = wait_stream(h);
  if (rc) return rc;
  h->tile_td = face_tile;
  h->tile_ey = ei_tile;
  carve<float>(h, h->df, (char*)h->buf);
  drop_graphs(h);
  return MHD_OK;
}

int mhd_ensemble_autotune(void** handles, int32_t ngrids, int32_t reps, int32_t out[2]) {
  if (!handles || ngrids <= 0 || reps <= 0) return fail(MHD_E_ARG, "bad autotune arguments");
  std::vector<Handle*> hs(ngrids);
  for (int i = 0; i < ngrids; ++i) {
    hs[i] = (Handle*)handles[i];
    if (!hs[i]) return fail(MHD_E_ARG, "null handle in ensemble");
  }
  Handle* h0 = hs[0];
  if (tunable(h0) && batchable(hs.data(), ngrids)) {
    for (Handle* h : hs) {
      int rc = wait_stream(h);
      if (rc) return rc;
    }
    // each (face shape, EMF shape) pair timed as a batched stage runs it: the
    // EMF families on the side stream beside the face fluxes
    int best_td = h0->tile_td, best_ey = h0->tile_ey;
    float best = INFINITY;
    for (int td : kTileTD) {
      for (int ey : kTileEY) {
        for (Handle* h : hs) { h->tile_td = td; h->tile_ey = ey; }
        BatchBufs b;
        int rc = build_batch<float>(hs.data(), ngrids, b);
        if (rc == MHD_OK) {
          const float ms = time_min(h0->st, reps, [&] {
            cudaEventRecord(h0->ev_fork, h0->st);
            cudaStreamWaitEvent(h0->st2, h0->ev_fork, 0);
            Batch<float>::parts(b.view, 0, 1, -1, 0.0, 1.0, h0->st2);
            Batch<float>::parts(b.view, 0, 2, -1, 0.0, 1.0, h0->st);
            cudaEventRecord(h0->ev_join, h0->st2);
            cudaStreamWaitEvent(h0->st, h0->ev_join, 0);
          });
          if (ms < best) { best = ms; best_td = td; best_ey = ey; }
        }
        cudaFree(b.tabs);
        cudaFree(b.maps);
        if (rc) return rc;
      }
    }
    for (Handle* h : hs) {
      h->tile_td = best_td;
      h->tile_ey = best_ey;
      carve<float>(h, h->df, (char*)h->buf);
      drop_graphs(h);
    }
    CK(cudaGetLastError());
  }
  if (out) { out[0] = h0->tile_td; out[1] = h0->tile_ey; }
  return MHD_OK;
}

// ---- learned coarse-grid correction
int mhd_mlp_apply(void* handle, void* mlp) {
  Handle* h = (Handle*)handle;
  if (!h || !mlp) return fail(MHD_E_ARG, "null argument");
  if (!h->fp32 || h->metric || h->prm.stepop == MHD_STEP_AB2)
    return fail(MHD_E_ARG, "the learned correction runs on FP32 Cartesian grids with an RK stepper");
  for (int a = 0; a < 3; ++a)
    if (h->prm.bc[a] != MHD_BC_PERIODIC) return fail(MHD_E_ARG, "the learned correction needs periodic axes");
  Dev<float> d = at_par(h->df, h->par);
  int rc = mlp_correct(mlp, d, h->st);
  if (rc) return rc;
  // the refill of the corrected state also gives the next step its CFL dt
  Launch<float>::fill_bxyz(d, true, h->st, true);
  h->prepared = true;
  CK(cudaGetLastError());
  return MHD_OK;
}

int mhd_step_corrected(void* handle, void* mlp, int32_t nsteps, double* tau_out, uint32_t* status) {
  Handle* h = (Handle*)handle;
  if (!h || !mlp || nsteps < 0) return fail(MHD_E_ARG, "bad arguments");
  for (int s = 0; s < nsteps; ++s) {
    int rc = do_steps<float>(h, 1);
    if (!rc) rc = mhd_mlp_apply(handle, mlp);
    if (rc) {
      if (status) *status = MHD_ST_CUDA_ERROR;
      return rc;
    }
  }
  int rc = finish(h, tau_out, status);
  if (rc) return rc;
  return mlp_status(mlp);
}

int mhd_free(void* handle) {
  Handle* h = (Handle*)handle;
  if (!h) return MHD_OK;
  if (h->st) cudaStreamSynchronize(h->st);
  ens_forget(h->uid);
  for (auto& kv : h->graphs) cudaGraphExecDestroy(kv.second.first);
  for (int i = 0; i < 16; ++i)
    if (h->ev[i]) cudaEventDestroy(h->ev[i]);
  for (cudaEvent_t e : h->pool) cudaEventDestroy(e);
  if (h->buf) cudaFree(h->buf);
  if (h->geo) cudaFree(h->geo);
  if (h->geoT) cudaFree(h->geoT);
  if (h->gmap) cudaFree(h->gmap);
  if (h->met) cudaFree(h->met);
  if (h->sc) cudaFree(h->sc);
  if (h->diag) cudaFree(h->diag);
  if (h->sc_h) cudaFreeHost(h->sc_h);
  if (h->diag_h) cudaFreeHost(h->diag_h);
  if (h->st) cudaStreamDestroy(h->st);
  if (h->st2) cudaStreamDestroy(h->st2);
  if (h->ev_fork) cudaEventDestroy(h->ev_fork);
  if (h->ev_join) cudaEventDestroy(h->ev_join);
  delete h;
  return MHD_OK;
}
