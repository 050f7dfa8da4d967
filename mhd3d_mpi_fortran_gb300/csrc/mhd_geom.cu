// Curvilinear metric of a mapped grid (metric mode), computed once on the
// device from the ghost-inclusive node coordinates.  FP64, built with
// -fmad=false: every quantity is rounded exactly as the CPU oracle's
// metric_geometry / edge_metric write it, so the FP64 metric mode agrees with
// the oracle to the last bit.  No counterpart in the reference, whose mesh is
// Cartesian (dxblock/dyblock/dzblock, mhd3d3.f90:3473-3486).
//
// Definitions (node P(i,j,k); 0-based, ghost-inclusive; face (ax,i,j,k) is the
// low face normal to ax of cell (i,j,k); t1 = ax+1, t2 = ax+2 cyclic):
//   A      = 0.5 (P(+t1+t2) - P) x (P(+t2) - P(+t1))   face area vector
//   |A|, n = A/|A|
//   C      = mean of the face's 4 nodes                 face centroid
//   V      = (1/3) sum over the 6 faces of C . A_out    (divergence theorem)
//   e_a    = C(high a-face) - C(low a-face)             cell edge vector
//   nbar_a = Abar/|Abar|, Abar = mean of the two a-face area vectors
//   sa     = sum_a |Abar_a|
//   g_e    = (mean |A| of the two a1 faces at the edge) (same for a2) / (mean V of its 4 cells)
//   dl_e   = |P(c + e) - P(c)|
#include <cuda_runtime.h>
#include <cmath>

#include "mhd_state.h"

namespace mhd {
namespace {

struct Nodes {
  const double *X, *Y, *Z;
};

__device__ __forceinline__ long long ix(const Geom& g, int i, int j, int k) {
  return (long long)i + (long long)g.px * ((long long)j + (long long)g.py * (long long)k);
}

__device__ __forceinline__ void node(const Nodes& N, const Geom& g, int i, int j, int k, double* x) {
  const long long c = ix(g, i, j, k);
  x[0] = N.X[c];
  x[1] = N.Y[c];
  x[2] = N.Z[c];
}

__device__ __forceinline__ void off(int ax, int o, int* d) {
  d[0] = d[1] = d[2] = 0;
  d[ax] = o;
}

// Face area vector of the low face normal to ax of cell (i,j,k).
__device__ void face_area(const Nodes& N, const Geom& g, int ax, int i, int j, int k, double* A) {
  const int t1 = (ax + 1) % 3, t2 = (ax + 2) % 3;
  int a[3] = {i, j, k}, b[3] = {i, j, k}, c0[3] = {i, j, k}, c1[3] = {i, j, k};
  b[t1] += 1; b[t2] += 1;  // P(+t1+t2)
  c0[t1] += 1;             // P(+t1)
  c1[t2] += 1;             // P(+t2)
  double p0[3], p1[3], q0[3], q1[3];
  node(N, g, a[0], a[1], a[2], p0);
  node(N, g, b[0], b[1], b[2], p1);
  node(N, g, c0[0], c0[1], c0[2], q0);
  node(N, g, c1[0], c1[1], c1[2], q1);
  double d1[3], d2[3];
  for (int q = 0; q < 3; ++q) {
    d1[q] = p1[q] - p0[q];
    d2[q] = q1[q] - q0[q];
  }
  A[0] = 0.5 * (d1[1] * d2[2] - d1[2] * d2[1]);
  A[1] = 0.5 * (d1[2] * d2[0] - d1[0] * d2[2]);
  A[2] = 0.5 * (d1[0] * d2[1] - d1[1] * d2[0]);
}

__device__ void face_centroid(const Nodes& N, const Geom& g, int ax, int i, int j, int k, double* C) {
  const int t1 = (ax + 1) % 3, t2 = (ax + 2) % 3;
  int b[3] = {i, j, k}, c[3] = {i, j, k}, d[3] = {i, j, k};
  b[t1] += 1;
  c[t1] += 1; c[t2] += 1;
  d[t2] += 1;
  double pa[3], pb[3], pc[3], pd[3];
  node(N, g, i, j, k, pa);
  node(N, g, b[0], b[1], b[2], pb);
  node(N, g, c[0], c[1], c[2], pc);
  node(N, g, d[0], d[1], d[2], pd);
  for (int q = 0; q < 3; ++q) C[q] = 0.25 * (pa[q] + pb[q] + pc[q] + pd[q]);
}

// Pass 1: area vectors (held in nrm until pass 3) and magnitudes of every face.
__global__ void k_geom_faces(Geom g, Nodes N, MetricOut m) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const int j = blockIdx.y * blockDim.y + threadIdx.y;
  const int k = blockIdx.z;
  if (i > g.nx || j > g.ny || k > g.nz) return;
  const long long c = ix(g, i, j, k);
  for (int ax = 0; ax < 3; ++ax) {
    const int lim[3] = {g.nx + (ax == 0), g.ny + (ax == 1), g.nz + (ax == 2)};
    if (i >= lim[0] || j >= lim[1] || k >= lim[2]) continue;
    double A[3];
    face_area(N, g, ax, i, j, k, A);
    m.nrm[ax][0][c] = A[0];
    m.nrm[ax][1][c] = A[1];
    m.nrm[ax][2][c] = A[2];
    m.am[ax][c] = sqrt(A[0] * A[0] + A[1] * A[1] + A[2] * A[2]);
  }
}

// Pass 2: cell volumes, edge vectors, mean unit normals, CFL area sums.
__global__ void k_geom_cells(Geom g, Nodes N, MetricOut m) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const int j = blockIdx.y * blockDim.y + threadIdx.y;
  const int k = blockIdx.z;
  if (i >= g.nx || j >= g.ny || k >= g.nz) return;
  const long long c = ix(g, i, j, k);
  double v = 0.0, s = 0.0;
  for (int ax = 0; ax < 3; ++ax) {
    int hi[3] = {i, j, k};
    hi[ax] += 1;
    const long long ch = ix(g, hi[0], hi[1], hi[2]);
    double Clo[3], Chi[3];
    face_centroid(N, g, ax, i, j, k, Clo);
    face_centroid(N, g, ax, hi[0], hi[1], hi[2], Chi);
    const double slo = Clo[0] * m.nrm[ax][0][c] + Clo[1] * m.nrm[ax][1][c] + Clo[2] * m.nrm[ax][2][c];
    const double shi = Chi[0] * m.nrm[ax][0][ch] + Chi[1] * m.nrm[ax][1][ch] + Chi[2] * m.nrm[ax][2][ch];
    v = v + (shi - slo);
    for (int q = 0; q < 3; ++q) m.eb[ax][q][c] = Chi[q] - Clo[q];
    double Ab[3];
    for (int q = 0; q < 3; ++q) Ab[q] = 0.5 * (m.nrm[ax][q][c] + m.nrm[ax][q][ch]);
    const double mm = sqrt(Ab[0] * Ab[0] + Ab[1] * Ab[1] + Ab[2] * Ab[2]);
    for (int q = 0; q < 3; ++q) m.nb[ax][q][c] = Ab[q] / mm;
    s = s + mm;
  }
  const double V = v / 3.0;
  m.vol[c] = V;
  m.rvol[c] = 1.0 / V;
  m.sa[c] = s;
}

// Pass 3: edge factors and lengths; unit normals replace the area vectors.
__global__ void k_geom_edges(Geom g, Nodes N, MetricOut m) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const int j = blockIdx.y * blockDim.y + threadIdx.y;
  const int k = blockIdx.z;
  if (i > g.nx || j > g.ny || k > g.nz) return;
  const long long c = ix(g, i, j, k);
  const int x3[3] = {i, j, k};
  if (i < g.nx && j < g.ny && k < g.nz) {
    for (int e = 0; e < 3; ++e) {
      const int a1 = (e + 1) % 3, a2 = (e + 2) % 3;
      if (x3[a1] < 1 || x3[a2] < 1) continue;
      int d1[3], d2[3];
      off(a1, 1, d1);
      off(a2, 1, d2);
      const long long s1 = ix(g, d1[0], d1[1], d1[2]), s2 = ix(g, d2[0], d2[1], d2[2]);
      const long long m1 = c - s1, m2 = c - s2, m12 = c - s1 - s2;
      const double vb = 0.25 * (m.vol[m12] + m.vol[m2] + m.vol[c] + m.vol[m1]);
      const double a1b = 0.5 * (m.am[a1][m2] + m.am[a1][c]);
      const double a2b = 0.5 * (m.am[a2][m1] + m.am[a2][c]);
      m.ge[e][c] = a1b * a2b / vb;
      int ce[3] = {i, j, k};
      ce[e] += 1;
      double p0[3], p1[3];
      node(N, g, i, j, k, p0);
      node(N, g, ce[0], ce[1], ce[2], p1);
      m.dl[e][c] = sqrt((p1[0] - p0[0]) * (p1[0] - p0[0]) + (p1[1] - p0[1]) * (p1[1] - p0[1]) +
                        (p1[2] - p0[2]) * (p1[2] - p0[2]));
    }
  }
  for (int ax = 0; ax < 3; ++ax) {
    const int lim[3] = {g.nx + (ax == 0), g.ny + (ax == 1), g.nz + (ax == 2)};
    if (i >= lim[0] || j >= lim[1] || k >= lim[2]) continue;
    const double a = m.am[ax][c];
    for (int q = 0; q < 3; ++q) m.nrm[ax][q][c] = m.nrm[ax][q][c] / a;
  }
}

// Minimum volume over the interior cells (one block; set-up only).
__global__ void k_min_vol(Geom g, const double* vol, double* out) {
  const long long n = (long long)g.nx0 * g.ny0 * g.nz0;
  double mn = INFINITY;
  for (long long t = threadIdx.x; t < n; t += blockDim.x) {
    const int i = (int)(t % g.nx0) + g.ng;
    const long long r = t / g.nx0;
    const int j = (int)(r % g.ny0) + g.ng;
    const int k = (int)(r / g.ny0) + g.ng;
    const double v = vol[ix(g, i, j, k)];
    mn = (v < mn || v != v) ? v : mn;
  }
  __shared__ double sm[1024];
  sm[threadIdx.x] = mn;
  __syncthreads();
  for (int w = blockDim.x / 2; w > 0; w >>= 1) {
    if ((int)threadIdx.x < w) {
      const double o = sm[threadIdx.x + w];
      if (o < sm[threadIdx.x] || o != o) sm[threadIdx.x] = o;
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) *out = sm[0];
}

}  // namespace

void metric_geometry(const Geom& g, const double* X, const double* Y, const double* Z, const MetricOut& m,
                     double* min_vol, cudaStream_t st) {
  Nodes N{X, Y, Z};
  dim3 b(64, 4, 1);
  dim3 gr((g.nx + 1 + b.x - 1) / b.x, (g.ny + 1 + b.y - 1) / b.y, g.nz + 1);
  k_geom_faces<<<gr, b, 0, st>>>(g, N, m);
  k_geom_cells<<<gr, b, 0, st>>>(g, N, m);
  k_geom_edges<<<gr, b, 0, st>>>(g, N, m);
  k_min_vol<<<1, 1024, 0, st>>>(g, m.vol, min_vol);
}

}  // namespace mhd
