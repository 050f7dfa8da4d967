// Allocation-free diagnostics of caller-owned device arrays.
//
// Some callers of this library cannot allocate device memory at the moment
// they want the diagnostics:
// * a driver that has handed all device memory to its own pool (one
//   preallocated slab per rank) and keeps it there;
// * code that runs between launches of a latency-critical loop, where an
//   implicit device synchronisation from cudaMalloc/cudaFree would stall the
//   pipeline;
// * a process capped by MPS or MIG limits that reserved everything at start.
//
// mhd_diagnostics_noalloc computes the same five numbers as mhd_diagnostics,
// on arrays the caller already owns on the device, and allocates nothing. Its
// only scratch is the file-scope array below: one 7-double record per z plane,
// at most kMaxPlanes planes.  Every GPU that loads this library holds the
// array until the process exits.
#include <cuda_runtime.h>
#include <math.h>
#include <mutex>
#include <string>

#include "../../include/mhd_gpu.h"
#include "mhd_state.h"

namespace {

constexpr int kMaxPlanes = 2048;  // ghost-inclusive z planes (nz0 + nord)
constexpr int kRec = 7;           // mass (sum, comp.), energy (sum, comp.), max|div B|, min rho, CFL dt
constexpr int kMaxDevices = 64;
constexpr int kThreads = 256;

static __device__ __align__(256) double g_plane_scratch[kMaxPlanes * kRec];

struct DD2 {
  double s, c;
};
__device__ __forceinline__ DD2 add_dd(DD2 x, DD2 y) {
  double s = x.s + y.s;
  double bb = s - x.s;
  double e = (x.s - (s - bb)) + (y.s - bb);
  e += x.c + y.c;
  double s2 = s + e;
  double b2 = s2 - s;
  double e2 = (s - (s2 - b2)) + (e - b2);
  return DD2{s2, e2};
}

struct Dims {
  int nx0, ny0, nz0, ng, nx, ny, nz;
  double gam, cfl;
};

// One block per ghost-inclusive z plane.  Every slot of the scratch that the
// final pass reads is written here first, so nothing needs clearing.
__global__ void __launch_bounds__(kThreads) k_plane(Dims d, const double* __restrict__ rho,
                                                    const double* __restrict__ vx, const double* __restrict__ vy,
                                                    const double* __restrict__ vz, const double* __restrict__ p,
                                                    const double* __restrict__ bi, const double* __restrict__ bj,
                                                    const double* __restrict__ bk, const double* __restrict__ dxa,
                                                    const double* __restrict__ dya, const double* __restrict__ dza,
                                                    double* part) {
  const int k = blockIdx.x;
  const int ncell = d.nx * d.ny;
  const bool kin = k >= d.ng && k < d.ng + d.nz0;
  const double gm1 = d.gam - 1.0;
  DD2 ms{0, 0}, es{0, 0};
  double dmax = 0.0, rmin = INFINITY, tmin = INFINITY;
  for (int t = threadIdx.x; t < ncell; t += blockDim.x) {
    const int i = t % d.nx, j = t / d.nx;
    const long long c = (long long)i + (long long)d.nx * (j + (long long)d.ny * k);
    const long long ci = (long long)i + (long long)(d.nx + 1) * (j + (long long)d.ny * k);
    const long long cj = (long long)i + (long long)d.nx * (j + (long long)(d.ny + 1) * k);
    const double r0 = rho[c], p0 = p[c], u = vx[c], v = vy[c], w = vz[c];
    // cell-centred B as get_bxyz (mhd3d3.f90:2118-2128)
    const double a = 0.5 * (bi[ci + 1] + bi[ci]);
    const double b = 0.5 * (bj[cj + d.nx] + bj[cj]);
    const double cc = 0.5 * (bk[c + (long long)d.nx * d.ny] + bk[c]);
    rmin = r0 < rmin ? r0 : rmin;
    // get_dt (mhd3d3.f90:1608-1639), every cell incl. ghosts
    const double vv = sqrt(u * u + v * v + w * w);
    const double btot = sqrt(a * a + b * b + cc * cc);
    const double valf = btot / sqrt(r0);
    const double vs = sqrt(d.gam * p0 / r0);
    const double vcfl = vv + sqrt(valf * valf + vs * vs);
    const double dt = d.cfl / (vcfl / dxa[i] + vcfl / dya[j] + vcfl / dza[k]);
    tmin = dt < tmin ? dt : tmin;
    if (kin && i >= d.ng && i < d.ng + d.nx0 && j >= d.ng && j < d.ng + d.ny0) {
      const double dv = dxa[i] * dya[j] * dza[k];
      ms = add_dd(ms, DD2{r0 * dv, 0.0});
      const double e = 0.5 * r0 * (u * u + v * v + w * w) + p0 / gm1 + 0.5 * (a * a + b * b + cc * cc);
      es = add_dd(es, DD2{e * dv, 0.0});
      const double db = (bi[ci + 1] - bi[ci]) / dxa[i] + (bj[cj + d.nx] - bj[cj]) / dya[j] +
                        (bk[c + (long long)d.nx * d.ny] - bk[c]) / dza[k];
      const double adb = fabs(db);
      dmax = adb > dmax ? adb : dmax;
    }
  }
  __shared__ double sh[kRec][kThreads];
  const int tid = threadIdx.x;
  sh[0][tid] = ms.s; sh[1][tid] = ms.c; sh[2][tid] = es.s; sh[3][tid] = es.c;
  sh[4][tid] = dmax; sh[5][tid] = rmin; sh[6][tid] = tmin;
  __syncthreads();
  for (int wdt = kThreads / 2; wdt > 0; wdt >>= 1) {
    if (tid < wdt) {
      DD2 x = add_dd(DD2{sh[0][tid], sh[1][tid]}, DD2{sh[0][tid + wdt], sh[1][tid + wdt]});
      DD2 y = add_dd(DD2{sh[2][tid], sh[3][tid]}, DD2{sh[2][tid + wdt], sh[3][tid + wdt]});
      sh[0][tid] = x.s; sh[1][tid] = x.c; sh[2][tid] = y.s; sh[3][tid] = y.c;
      sh[4][tid] = sh[4][tid] > sh[4][tid + wdt] ? sh[4][tid] : sh[4][tid + wdt];
      sh[5][tid] = sh[5][tid] < sh[5][tid + wdt] ? sh[5][tid] : sh[5][tid + wdt];
      sh[6][tid] = sh[6][tid] < sh[6][tid + wdt] ? sh[6][tid] : sh[6][tid + wdt];
    }
    __syncthreads();
  }
  if (tid < kRec) part[(long long)k * kRec + tid] = sh[tid][0];
}

// Plane records combined in plane order (deterministic).
__global__ void k_final(const double* part, int nz, double* out) {
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  DD2 m{0, 0}, e{0, 0};
  double dm = 0.0, rm = INFINITY, tm = INFINITY;
  for (int k = 0; k < nz; ++k) {
    const double* r = part + (long long)k * kRec;
    m = add_dd(m, DD2{r[0], r[1]});
    e = add_dd(e, DD2{r[2], r[3]});
    dm = r[4] > dm ? r[4] : dm;
    rm = r[5] < rm ? r[5] : rm;
    tm = r[6] < tm ? r[6] : tm;
  }
  out[0] = m.s + m.c;
  out[1] = e.s + e.c;
  out[2] = dm;
  out[3] = rm;
  out[4] = tm;
}

int fail_na(int code, const std::string& m) {
  mhd::set_last_error(m);  // read back with mhd_last_error()
  return code;
}

// Device address of the scratch array, looked up once per device with that
// device current (cudaGetSymbolAddress), then cached for the life of the
// process.  A cudaDeviceReset destroys the context the address belongs to,
// so the cache does not survive one (documented in mhd_gpu.h).
int scratch_for_current_device(double** out) {
  static std::mutex mu;
  static double* ptr[kMaxDevices] = {};
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return fail_na(MHD_E_CUDA, std::string("cudaGetDevice: ") + cudaGetErrorString(e));
  if (dev < 0 || dev >= kMaxDevices) return fail_na(MHD_E_ARG, "device ordinal out of range");
  std::lock_guard<std::mutex> lock(mu);
  if (!ptr[dev]) {
    double* p = nullptr;
    e = cudaGetSymbolAddress((void**)&p, g_plane_scratch);
    if (e != cudaSuccess || !p)
      return fail_na(MHD_E_CUDA, std::string("cudaGetSymbolAddress: ") + cudaGetErrorString(e));
    ptr[dev] = p;
  }
  *out = ptr[dev];
  return MHD_OK;
}

}  // namespace

int mhd_diagnostics_noalloc(const mhd_params* prm, const double* rho, const double* vx, const double* vy,
                            const double* vz, const double* p, const double* bi, const double* bj,
                            const double* bk, const double* dx, const double* dy, const double* dz,
                            double* out, void* stream) {
  if (!prm || !rho || !vx || !vy || !vz || !p || !bi || !bj || !bk || !dx || !dy || !dz || !out)
    return fail_na(MHD_E_ARG, "null argument");
  if (prm->nx0 < 1 || prm->ny0 < 1 || prm->nz0 < 1 || prm->nord < 0 || (prm->nord & 1))
    return fail_na(MHD_E_ARG, "bad grid sizes");
  Dims d;
  d.nx0 = prm->nx0; d.ny0 = prm->ny0; d.nz0 = prm->nz0; d.ng = prm->nord / 2;
  d.nx = d.nx0 + prm->nord; d.ny = d.ny0 + prm->nord; d.nz = d.nz0 + prm->nord;
  d.gam = prm->gam; d.cfl = prm->cfl;
  if (d.nz > kMaxPlanes)
    return fail_na(MHD_E_ARG, "grid has " + std::to_string(d.nz) + " z planes (nz0 + nord); the allocation-free "
                   "diagnostics hold at most " + std::to_string(kMaxPlanes));
  if ((long long)d.nx * d.ny >= (1LL << 31)) return fail_na(MHD_E_ARG, "z plane larger than 2^31 cells");
  // An error the caller's own work left pending is reported, and left pending
  // for the caller, rather than taken for a failure of these launches.
  cudaError_t e = cudaPeekAtLastError();
  if (e != cudaSuccess)
    return fail_na(MHD_E_CUDA, std::string("an earlier CUDA error is pending (left for the caller): ") +
                                   cudaGetErrorString(e));
  double* scratch = nullptr;
  int rc = scratch_for_current_device(&scratch);
  if (rc) return rc;
  cudaStream_t st = (cudaStream_t)stream;
  k_plane<<<d.nz, kThreads, 0, st>>>(d, rho, vx, vy, vz, p, bi, bj, bk, dx, dy, dz, scratch);
  k_final<<<1, 1, 0, st>>>(scratch, d.nz, out);
  e = cudaGetLastError();
  if (e != cudaSuccess) return fail_na(MHD_E_CUDA, std::string("launch: ") + cudaGetErrorString(e));
  return MHD_OK;
}
