// ORACLE -- test infrastructure only.  Nothing in the product path may link,
// import or call this file; it is the CPU checker for the GPU library.
//
// A CPU FP64 restatement of the reference's per-timestep MHD update
// (tiegcm/mhd3d_mpi_fortran, mhd3d3.f90 unless stated otherwise).  Every routine
// keeps the reference's array-at-a-time structure (one pass per Fortran
// statement or forall) and the reference's expression order, so that FP64
// results agree with the GPU FP64 mode to the last bit apart from exp/erfc
// (glibc here, CUDA's libdevice there).  Built with -ffp-contract=off: no FMA.
// A second, fused mode (oracle_set_fused) evaluates the face and edge passes
// one x line at a time from the cell arrays, without the array passes'
// temporaries; it calls the same element functions in the same order and so
// gives the array passes' results bit for bit -- it is the faster CPU
// baseline, not a second specification.
//
// Parity pinning: the reference ships no tests or golden vectors and its
// Fortran cannot be compiled here (no gfortran/ifort, MPI or HDF5), so this
// restatement is pinned only by the invariants the reference's own artefacts
// imply (point symmetry of Orszag-Tang, process_mhd_2d.m:95-102; shock-tube
// axis permutation, mhd3d3.f90:3523-3569; div B from CT, mhd3d3.f90:3909-3933;
// periodic mass conservation).  "Parity unpinned" against a reference binary.
//
// Single-rank semantics: one MPI rank with xprocs=yprocs=zprocs=1.  The halo
// SENDRECVs then exchange with PROC_NULL (walls, mhd3d3.f90:3228-3256, then the
// mirror overwrites the ghosts) or with the rank itself (periodic topology of
// mhd3d2.f90:3063-3064, a plain wrap); MPI_REDUCE/BCAST of dt are identities.

#include <cmath>
#include <cstddef>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <vector>
#include <algorithm>
#include <omp.h>

#include "../include/mhd_gpu.h"

namespace {

// Fortran-style 3-D array: 1-based, column-major.
struct A3 {
  int n1 = 0, n2 = 0, n3 = 0;
  std::vector<double> v;
  A3() {}
  A3(int a, int b, int c) { alloc(a, b, c); }
  void alloc(int a, int b, int c) {
    n1 = a; n2 = b; n3 = c;
    v.assign((size_t)a * b * c, 0.0);
  }
  inline double& operator()(int i, int j, int k) {
    return v[(size_t)(i - 1) + (size_t)n1 * ((size_t)(j - 1) + (size_t)n2 * (size_t)(k - 1))];
  }
  inline double operator()(int i, int j, int k) const {
    return v[(size_t)(i - 1) + (size_t)n1 * ((size_t)(j - 1) + (size_t)n2 * (size_t)(k - 1))];
  }
};

// Fortran intrinsics.  sign(1,x): +1 for x >= 0 including -0.0 (ifort default).
inline double fsign1(double x) { return (x >= 0.0) ? 1.0 : -1.0; }
inline double fmax2(double a, double b) { return (a > b) ? a : b; }
inline double fmin2(double a, double b) { return (a < b) ? a : b; }

#define FOR3(a, b, c) \
  _Pragma("omp parallel for schedule(static)") \
  for (int k = 1; k <= (c); ++k) for (int j = 1; j <= (b); ++j) for (int i = 1; i <= (a); ++i)

struct Oracle {
  // pars (mhd3d3.f90:33-104)
  int nx0, ny0, nz0, nord, ng, nx, ny, nz, reconop, stepop, bc[3], dt_mode, tvd_shift, emf = 0;
  double gam, cfl, pdmb, eps, alpha, beta, tau, tau0, pi;
  std::vector<double> dxv, dyv, dzv;  // dxblock(i,j,k) = dxv[i-1]
  // fields (mhd3d3.f90:251-283)
  A3 rho, vx, vy, vz, p, bx, by, bz, bi, bj, bk, ei, ej, ek;
  A3 rhovx, rhovy, rhovz, eng, rho0, rhovx0, rhovy0, rhovz0, eng0;
  A3 rhop, vxp, vyp, vzp, pp, bxp, byp, bzp, bip, bjp, bkp;
  A3 rhoh, vxh, vyh, vzh, ph, bxh, byh, bzh, bih, bjh, bkh;
  A3 rhovxp, rhovyp, rhovzp, rhovxh, rhovyh, rhovzh, engp;
  A3 flux[3][8];  // [dir][rho, rvx, rvy, rvz, eng, stress_x, stress_y, stress_z]
  uint32_t status = 0;

  // ---- curvilinear (metric) mode: no reference counterpart; this oracle is
  // its specification.  Face fields bi/bj/bk hold the magnetic flux
  // Phi = B.A through each face; fluxes are multiplied by face areas and the
  // update divided by cell volumes; CT is the circulation of E.dl.  On a
  // Cartesian mesh every term reduces to the reference's formula.
  bool metric = false;
  A3 X[3];               // node coordinates (nx+1, ny+1, nz+1)
  A3 Af[3][3];           // [face axis][component] low-face area vectors (face extents)
  A3 vol;                // cell volumes (nx, ny, nz)
  A3 eb[3][3];           // [axis][component] cell edge vectors (face-centroid differences)
  A3 w[3];               // v . (mean unit normal of the a-faces), per stage

  double dxb(int i, int, int) const { return dxv[i - 1]; }
  double dyb(int, int j, int) const { return dyv[j - 1]; }
  double dzb(int, int, int k) const { return dzv[k - 1]; }

  // ------------------------------------------------------------------ fills
  // One rank, so the SENDRECVs of fillx_center (mhd3d3.f90:346-390) either
  // wrap (periodic) or are replaced by the wall mirror.  Periodic:
  //   aa(1:ng) = aa(lnx-nord+1:lnx-ng); aa(lnx-ng+1:lnx) = aa(ng+1:nord)
  // Even/odd wall (xbc=0/1): aa(i) = +-aa(nord+1-i); aa(lnx+1-i) = +-aa(lnx-nord+i).
  // Outflow (no reference counterpart): copy of the first/last interior cell.
  // axis: 0,1,2; face: this array's own staggering axis (fillx_face,
  // mhd3d3.f90:482-524: aa(1:ng)=aa(lnx-nord:lnx-ng-1), aa(lnx-ng+1:lnx)=
  // aa(ng+2:nord+1); walls aa(i)=+-aa(nord+2-i), aa(n+2-i)=+-aa(n0+i)).
  void fill_axis(A3& a, int axis, bool face, double sgn) {
    int n[3] = {a.n1, a.n2, a.n3};
    int n0 = (axis == 0) ? nx0 : (axis == 1) ? ny0 : nz0;
    int nn = n[axis];  // lnx (cell) or lnx = n+1 (face)
    int kind = bc[axis];
    int e1 = n[(axis + 1) % 3], e2 = n[(axis + 2) % 3];
    auto at = [&](int g, int u, int w) -> double& {
      if (axis == 0) return a(g, u, w);
      if (axis == 1) return a(w, g, u);
      return a(u, w, g);
    };
    // map: for a ghost index g, the source index and sign
    auto src = [&](int g, int& s, double& f) {
      f = 1.0;
      if (kind == MHD_BC_PERIODIC) {
        if (!face) s = (g <= ng) ? g + n0 : g - n0;      // lnx-nord+g = n0+g
        else s = (g <= ng) ? g + n0 : g - n0;            // lnx-nord-1+g = n0+g
      } else if (kind == MHD_BC_OUTFLOW) {
        if (!face) s = (g <= ng) ? ng + 1 : ng + n0;
        else s = (g <= ng) ? ng + 1 : ng + n0 + 1;
      } else {
        if (!face) s = (g <= ng) ? nord + 1 - g : 2 * n0 + nord + 1 - g;  // lnx+1-i <- lnx-nord+i
        else s = (g <= ng) ? nord + 2 - g : 2 * n0 + nord + 2 - g;        // nx+2-i <- nx0+i
        f = sgn;
      }
    };
    std::vector<int> gl;
    for (int g = 1; g <= ng; ++g) gl.push_back(g);
    int hi0 = face ? ng + n0 + 2 : ng + n0 + 1;
    for (int g = hi0; g <= nn; ++g) gl.push_back(g);
    // Periodic: the left block is filled first, then the right one reads
    // aa(ng+1:nord) (interior); walls: both blocks read interior only.
    for (int g : gl) {
      int s; double f;
      src(g, s, f);
#pragma omp parallel for schedule(static)
      for (int w = 1; w <= e2; ++w)
        for (int u = 1; u <= e1; ++u) {
          double val = at(s, u, w);
          at(g, u, w) = (f == 1.0) ? val : -val;
        }
    }
  }
  double vsign(int var, int axis) {
    // REFLECT: normal velocity odd (mhd3d2.f90:713 vx in x, 720 vy in y)
    if (bc[axis] != MHD_BC_REFLECT) return 1.0;
    return (var == axis + 1) ? -1.0 : 1.0;
  }
  // fill_hydro_mpi (mhd3d3.f90:781-801): x for all, then y, then z.
  void fill_hydro() {
    A3* h[5] = {&rho, &p, &vx, &vy, &vz};
    int var[5] = {0, 4, 1, 2, 3};
    for (int ax = 0; ax < 3; ++ax)
      for (int q = 0; q < 5; ++q) fill_axis(*h[q], ax, false, vsign(var[q], ax));
  }
  // fill_mag_mpi (mhd3d3.f90:803-819)
  void fill_mag() {
    for (int ax = 0; ax < 3; ++ax) {
      fill_axis(bi, ax, ax == 0, 1.0);
      fill_axis(bj, ax, ax == 1, 1.0);
      fill_axis(bk, ax, ax == 2, 1.0);
    }
  }

  // ---------------------------------------------------------- reconstruction
  // 8-point centred interpolant (interp_pdm, mhd3d3.f90:862-924)
  static inline double tap8(double a0, double a1, double a2, double a3, double a4,
                            double a5, double a6, double a7) {
    double s = -3.0 * a0;
    s = s + 29.0 * a1;
    s = s - 139.0 * a2;
    s = s + 533.0 * a3;
    s = s + 533.0 * a4;
    s = s - 139.0 * a5;
    s = s + 29.0 * a6;
    s = s - 3.0 * a7;
    return s / 840.0;
  }

  // Gather helper for dir 1..6 (dirs 4..6 keep the transverse extents, untruncated).
  // Returns f at offset m along the recon axis for output element (i,j,k),
  // including the PDM2 stencil shifts (snx,sny,snz).
  inline double gat(const A3& f, int dir, int i, int j, int k, int m, int snx, int sny, int snz) const {
    switch (dir) {
      case 1: return f(ng + i + m + snx, ng + j + sny, ng + k + snz);
      case 2: return f(ng + i + snx, ng + j + m + sny, ng + k + snz);
      case 3: return f(ng + i + snx, ng + j + sny, ng + k + m + snz);
      case 4: return f(ng + i + m + snx, j, k);
      case 5: return f(i, ng + j + m + sny, k);
      default: return f(i, j, ng + k + m + snz);
    }
  }

  void interp_pdm(const A3& f, A3& fi, int lnx, int lny, int lnz, int dir) {
    FOR3(lnx, lny, lnz) {
      fi(i, j, k) = tap8(gat(f, dir, i, j, k, -4, 0, 0, 0), gat(f, dir, i, j, k, -3, 0, 0, 0),
                         gat(f, dir, i, j, k, -2, 0, 0, 0), gat(f, dir, i, j, k, -1, 0, 0, 0),
                         gat(f, dir, i, j, k, 0, 0, 0, 0), gat(f, dir, i, j, k, 1, 0, 0, 0),
                         gat(f, dir, i, j, k, 2, 0, 0, 0), gat(f, dir, i, j, k, 3, 0, 0, 0));
    }
  }

  // interp2_pdm (mhd3d3.f90:926-989): two-pass 8-tap interpolant to edges.
  void interp2_pdm(const A3& f, A3& fi, int dir) {
    if (dir == 1) {  // fi (nx0,ny0+1,nz0+1): y then z
      A3 g(nx0, ny0 + 1, nz);
      FOR3(nx0, ny0 + 1, nz) {
        g(i, j, k) = tap8(f(ng + i, ng + j - 4, k), f(ng + i, ng + j - 3, k), f(ng + i, ng + j - 2, k),
                          f(ng + i, ng + j - 1, k), f(ng + i, ng + j, k), f(ng + i, ng + j + 1, k),
                          f(ng + i, ng + j + 2, k), f(ng + i, ng + j + 3, k));
      }
      FOR3(nx0, ny0 + 1, nz0 + 1) {
        fi(i, j, k) = tap8(g(i, j, ng + k - 4), g(i, j, ng + k - 3), g(i, j, ng + k - 2), g(i, j, ng + k - 1),
                           g(i, j, ng + k), g(i, j, ng + k + 1), g(i, j, ng + k + 2), g(i, j, ng + k + 3));
      }
    } else if (dir == 2) {  // fi (nx0+1,ny0,nz0+1): z then x
      A3 g(nx, ny0, nz0 + 1);
      FOR3(nx, ny0, nz0 + 1) {
        g(i, j, k) = tap8(f(i, ng + j, ng + k - 4), f(i, ng + j, ng + k - 3), f(i, ng + j, ng + k - 2),
                          f(i, ng + j, ng + k - 1), f(i, ng + j, ng + k), f(i, ng + j, ng + k + 1),
                          f(i, ng + j, ng + k + 2), f(i, ng + j, ng + k + 3));
      }
      FOR3(nx0 + 1, ny0, nz0 + 1) {
        fi(i, j, k) = tap8(g(ng + i - 4, j, k), g(ng + i - 3, j, k), g(ng + i - 2, j, k), g(ng + i - 1, j, k),
                           g(ng + i, j, k), g(ng + i + 1, j, k), g(ng + i + 2, j, k), g(ng + i + 3, j, k));
      }
    } else {  // fi (nx0+1,ny0+1,nz0): x then y
      A3 g(nx0 + 1, ny, nz0);
      FOR3(nx0 + 1, ny, nz0) {
        g(i, j, k) = tap8(f(ng + i - 4, j, ng + k), f(ng + i - 3, j, ng + k), f(ng + i - 2, j, ng + k),
                          f(ng + i - 1, j, ng + k), f(ng + i, j, ng + k), f(ng + i + 1, j, ng + k),
                          f(ng + i + 2, j, ng + k), f(ng + i + 3, j, ng + k));
      }
      FOR3(nx0 + 1, ny0 + 1, nz0) {
        fi(i, j, k) = tap8(g(i, ng + j - 4, k), g(i, ng + j - 3, k), g(i, ng + j - 2, k), g(i, ng + j - 1, k),
                           g(i, ng + j, k), g(i, ng + j + 1, k), g(i, ng + j + 2, k), g(i, ng + j + 3, k));
      }
    }
  }

  // interp_tvd (mhd3d3.f90:991-1035): 2-point mean
  void interp_tvd(const A3& f, A3& fi, int lnx, int lny, int lnz, int dir) {
    FOR3(lnx, lny, lnz) {
      fi(i, j, k) = (gat(f, dir, i, j, k, -1, 0, 0, 0) + gat(f, dir, i, j, k, 0, 0, 0, 0)) / 2.0;
    }
  }

  // interp2_tvd (mhd3d3.f90:1037-1067): 4-cell mean at the edge
  void interp2_tvd(const A3& f, A3& fi, int dir) {
    if (dir == 1) {
      FOR3(nx0, ny0 + 1, nz0 + 1) {
        fi(i, j, k) = (f(ng + i, ng + j - 1, ng + k - 1) + f(ng + i, ng + j, ng + k - 1) +
                       f(ng + i, ng + j, ng + k) + f(ng + i, ng + j - 1, ng + k)) / 4.0;
      }
    } else if (dir == 2) {
      FOR3(nx0 + 1, ny0, nz0 + 1) {
        fi(i, j, k) = (f(ng + i - 1, ng + j, ng + k - 1) + f(ng + i - 1, ng + j, ng + k) +
                       f(ng + i, ng + j, ng + k) + f(ng + i, ng + j, ng + k - 1)) / 4.0;
      }
    } else {
      FOR3(nx0 + 1, ny0 + 1, nz0) {
        fi(i, j, k) = (f(ng + i - 1, ng + j - 1, ng + k) + f(ng + i, ng + j - 1, ng + k) +
                       f(ng + i, ng + j, ng + k) + f(ng + i - 1, ng + j, ng + k)) / 4.0;
      }
    }
  }

  // PDM2 (mhd3d3.f90:1069-1172): partial-donor limiter of the interpolant fi,
  // one element (the array form below and the fused step share it).
  inline void pdm2_el(double fm2, double fm1, double f0, double fp1, double fi, double& fl, double& fr) const {
    double maxf = fmax2(fm1, f0);
    double minf = fmin2(fm1, f0);
    double fii = fmax2(minf, fmin2(fi, maxf));
    double dfm = pdmb * (fm1 - fm2);
    double df0 = pdmb * (f0 - fm1);
    double dfp = pdmb * (fp1 - f0);
    double sm = fsign1(dfm), s0 = fsign1(df0), sp = fsign1(dfp);
    dfm = std::fabs(dfm);
    dfp = std::fabs(dfp);
    double qm = std::fabs(sm + s0);
    double qp = std::fabs(s0 + sp);
    double dfl = fii - fm1;
    double dfr = f0 - fii;
    fl = fii - s0 * fmax2(0.0, std::fabs(dfl) - qm * dfm);
    fr = fii + s0 * fmax2(0.0, std::fabs(dfr) - qp * dfp);
  }
  void PDM2(A3& fleft, A3& fright, const A3& f, const A3& fi, int lnx, int lny, int lnz,
            int snx, int sny, int snz, int dir) {
    FOR3(lnx, lny, lnz) {
      double fl, fr;
      pdm2_el(gat(f, dir, i, j, k, -2, snx, sny, snz), gat(f, dir, i, j, k, -1, snx, sny, snz),
              gat(f, dir, i, j, k, 0, snx, sny, snz), gat(f, dir, i, j, k, 1, snx, sny, snz), fi(i, j, k), fl, fr);
      fleft(i, j, k) = fl;
      fright(i, j, k) = fr;
    }
  }

  // TVD (mhd3d3.f90:1174-1250, van Leer).  mhd3d3 ignores the stencil shifts
  // (mhd3d3.f90:1187-1237); mhd3d2 honours them (mhd3d2.f90:1152-1199):
  // tvd_shift selects.  mc=true: the MC limiter variant (no reference
  // counterpart) phi(a) = max(0, min(2a, (1+a)/2, 2)).
  void TVD(A3& fleft, A3& fright, const A3& f, const A3& fi, int lnx, int lny, int lnz,
           int snx, int sny, int snz, int dir, bool mc) {
    if (!tvd_shift) { snx = 0; sny = 0; snz = 0; }
    FOR3(lnx, lny, lnz) {
      double fl, fr;
      tvd_el(gat(f, dir, i, j, k, -2, snx, sny, snz), gat(f, dir, i, j, k, -1, snx, sny, snz),
             gat(f, dir, i, j, k, 0, snx, sny, snz), gat(f, dir, i, j, k, 1, snx, sny, snz), fi(i, j, k), mc, fl, fr);
      fleft(i, j, k) = fl;
      fright(i, j, k) = fr;
    }
  }
  inline void tvd_el(double fm2, double fm1, double f0, double fp1, double fi, bool mc, double& fl,
                     double& fr) const {
    double a = (fm1 - fm2) / (f0 - fm1 + eps);
    double b = mc ? mclim(a) : (a + std::fabs(a)) / (1.0 + std::fabs(a));
    fl = fm1 - b * (fm1 - fi);
    a = (f0 - fp1) / (fm1 - f0 + eps);
    b = mc ? mclim(a) : (a + std::fabs(a)) / (1.0 + std::fabs(a));
    fr = f0 - b * (f0 - fi);
  }
  // MC limiter in the same form: with fi the 2-point mean, fleft = fm1 -
  // b*(fm1-fi) = fm1 + b/2*(f0-fm1), so b is the limiter phi(a) itself (van
  // Leer's b above is phi_vL(a)); MC: phi(a) = max(0, min(2a, (1+a)/2, 2)).
  static double mclim(double a) {
    return fmax2(0.0, fmin2(fmin2(2.0 * a, 0.5 * (1.0 + a)), 2.0));
  }

  // WENO5 (mhd3d3.f90:1252-1378), one face element
  static inline void weno5_pt(double fm3, double fm2, double fm1, double f0, double fp1, double fp2,
                              double eps, double& fl, double& fr) {
    const double c13 = 13.0 / 12.0;
    double h0 = (2.0 * fm3 - 7.0 * fm2 + 11.0 * fm1) / 6.0;
    double h1 = (-fm2 + 5.0 * fm1 + 2.0 * f0) / 6.0;
    double h2 = (2.0 * fm1 + 5.0 * f0 - fp1) / 6.0;
    double t, u;
    t = fm3 - 2.0 * fm2 + fm1; u = fm3 - 4.0 * fm2 + 3.0 * fm1;
    double s0 = c13 * (t * t) + 0.25 * (u * u);
    t = fm2 - 2.0 * fm1 + f0; u = fm2 - f0;
    double s1 = c13 * (t * t) + 0.25 * (u * u);
    t = fm1 - 2.0 * f0 + fp1; u = 3.0 * fm1 - 4.0 * f0 + fp1;
    double s2 = c13 * (t * t) + 0.25 * (u * u);
    s0 = 0.1 / ((eps + s0) * (eps + s0));
    s1 = 0.6 / ((eps + s1) * (eps + s1));
    s2 = 0.3 / ((eps + s2) * (eps + s2));
    double sum = s0 + s1 + s2;
    double w0 = s0 / sum, w1 = s1 / sum, w2 = s2 / sum;
    fl = w0 * h0 + w1 * h1 + w2 * h2;
    h0 = (2.0 * fp2 - 7.0 * fp1 + 11.0 * f0) / 6.0;
    h1 = (-fp1 + 5.0 * f0 + 2.0 * fm1) / 6.0;
    h2 = (2.0 * f0 + 5.0 * fm1 - fm2) / 6.0;
    t = fp2 - 2.0 * fp1 + f0; u = fp2 - 4.0 * fp1 + 3.0 * f0;
    s0 = c13 * (t * t) + 0.25 * (u * u);
    t = fp1 - 2.0 * f0 + fm1; u = fp1 - fm1;
    s1 = c13 * (t * t) + 0.25 * (u * u);
    t = f0 - 2.0 * fm1 + fm2; u = 3.0 * f0 - 4.0 * fm1 + fm2;
    s2 = c13 * (t * t) + 0.25 * (u * u);
    s0 = 0.1 / ((eps + s0) * (eps + s0));
    s1 = 0.6 / ((eps + s1) * (eps + s1));
    s2 = 0.3 / ((eps + s2) * (eps + s2));
    sum = s0 + s1 + s2;
    w0 = s0 / sum; w1 = s1 / sum; w2 = s2 / sum;
    fr = w0 * h0 + w1 * h1 + w2 * h2;
  }

  // minmod / median (mhd3d3.f90:1380-1403)
  static inline double minmod(double a, double b) {
    return 0.5 * (fsign1(a) + fsign1(b)) * fmin2(std::fabs(a), std::fabs(b));
  }
  static inline double median(double a, double b, double c) { return a + minmod(b - a, c - a); }

  // MP bound of one side (MPWENO5, mhd3d3.f90:1530-1591); for the left state
  // (a3..b1) = (fm3,fm2,fm1,f0,fp1), for the right (fp2,fp1,f0,fm1,fm2).
  static inline double mp_side(double w, double a3, double a2, double a1, double b0, double b1,
                               double alpha, double beta) {
    double h0 = a3 - 2.0 * a2 + a1;
    double h1 = a2 - 2.0 * a1 + b0;
    double h2 = a1 - 2.0 * b0 + b1;
    double s2 = 4.0 * h1 - h2;
    double s0 = 4.0 * h2 - h1;
    double s1 = minmod(s2, s0);
    s2 = minmod(h1, h2);
    s0 = minmod(s1, s2);
    double w2 = 4.0 * h0 - h1;
    double w0 = 4.0 * h1 - h0;
    double w1 = minmod(w2, w0);
    w2 = minmod(h0, h1);
    w0 = minmod(w1, w2);
    s1 = a1 + alpha * (a1 - a2);
    s2 = 0.5 * (a1 + b0 - s0);
    s0 = 0.5 * (3.0 * a1 - a2) + beta * w0 / 3.0;
    w1 = fmin2(fmin2(a1, b0), s2);
    w2 = fmin2(fmin2(a1, s1), s0);
    w0 = fmax2(w1, w2);
    h1 = fmax2(fmax2(a1, b0), s2);
    h2 = fmax2(fmax2(a1, s1), s0);
    h0 = fmin2(h1, h2);
    return median(w, w0, h0);
  }

  void WENO5(A3& fleft, A3& fright, const A3& f, int lnx, int lny, int lnz, int dir, bool mp) {
    FOR3(lnx, lny, lnz) {
      double fm3 = gat(f, dir, i, j, k, -3, 0, 0, 0);
      double fm2 = gat(f, dir, i, j, k, -2, 0, 0, 0);
      double fm1 = gat(f, dir, i, j, k, -1, 0, 0, 0);
      double f0 = gat(f, dir, i, j, k, 0, 0, 0, 0);
      double fp1 = gat(f, dir, i, j, k, 1, 0, 0, 0);
      double fp2 = gat(f, dir, i, j, k, 2, 0, 0, 0);
      double fl, fr;
      weno5_pt(fm3, fm2, fm1, f0, fp1, fp2, eps, fl, fr);
      if (mp) {  // MPWENO5 (mhd3d3.f90:1405-1596)
        fl = mp_side(fl, fm3, fm2, fm1, f0, fp1, alpha, beta);
        fr = mp_side(fr, fp2, fp1, f0, fm1, fm2, alpha, beta);
      }
      fleft(i, j, k) = fl;
      fright(i, j, k) = fr;
    }
  }

  // reconstruct_3d (mhd3d3.f90:833-860)
  void reconstruct_3d(A3& fleft, A3& fright, const A3& f, int lnx, int lny, int lnz, int dir) {
    fleft.alloc(lnx, lny, lnz);
    fright.alloc(lnx, lny, lnz);
    if (reconop == 1) {
      A3 fi(lnx, lny, lnz);
      interp_pdm(f, fi, lnx, lny, lnz, dir);
      PDM2(fleft, fright, f, fi, lnx, lny, lnz, 0, 0, 0, dir);
    } else if (reconop == 2 || reconop == 5) {
      A3 fi(lnx, lny, lnz);
      interp_tvd(f, fi, lnx, lny, lnz, dir);
      TVD(fleft, fright, f, fi, lnx, lny, lnz, 0, 0, 0, dir, reconop == 5);
    } else {
      WENO5(fleft, fright, f, lnx, lny, lnz, dir, reconop == 4);
    }
  }

  // --------------------------------------------------------------- get_*
  // get_dt (mhd3d3.f90:1608-1639): CFL dt, minval over all cells incl. ghosts
  double get_dt() {
    if (metric) return get_dt_metric();
    double m = INFINITY;
#pragma omp parallel for reduction(min : m) schedule(static)
    for (int k = 1; k <= nz; ++k)
      for (int j = 1; j <= ny; ++j)
        for (int i = 1; i <= nx; ++i) {
          double v = std::sqrt(vx(i, j, k) * vx(i, j, k) + vy(i, j, k) * vy(i, j, k) + vz(i, j, k) * vz(i, j, k));
          double btot = std::sqrt(bx(i, j, k) * bx(i, j, k) + by(i, j, k) * by(i, j, k) + bz(i, j, k) * bz(i, j, k));
          double valf = btot / std::sqrt(rho(i, j, k));
          double vs = std::sqrt(gam * p(i, j, k) / rho(i, j, k));
          double vcfl = v + std::sqrt(valf * valf + vs * vs);
          double dt = cfl / (vcfl / dxb(i, j, k) + vcfl / dyb(i, j, k) + vcfl / dzb(i, j, k));
          m = (dt < m) ? dt : m;
        }
    return m;
  }

  // get_conserve (mhd3d3.f90:1641-1650)
  void get_conserve() {
    FOR3(nx, ny, nz) {
      double r = rho(i, j, k), u = vx(i, j, k), v = vy(i, j, k), w = vz(i, j, k);
      rho0(i, j, k) = r;
      rhovx0(i, j, k) = r * u;
      rhovy0(i, j, k) = r * v;
      rhovz0(i, j, k) = r * w;
      eng0(i, j, k) = 0.5 * r * (u * u + v * v + w * w) + p(i, j, k) / (gam - 1.0);
    }
  }

  // Quadrant selection by the sign of dif and the 4-quadrant mean of
  // get_vav_center2corner (mhd3d3.f90:2056-2108), one element
  inline double corner_blend_el(const A3& lv, int dir, int i, int j, int k, double a00_0, double a00_1,
                                double a10_0, double a10_1, double a01_0, double a01_1, double a11_0,
                                double a11_1) const {
    double d00, d10, d01, d11;
    const int G = ng;
    if (dir == 1) {
      d00 = std::fabs(lv(i + G, j + G - 2, k + G - 1) - lv(i + G, j + G - 1, k + G - 1)) -
            std::fabs(lv(i + G, j + G - 1, k + G - 2) - lv(i + G, j + G - 1, k + G - 1));
      d10 = std::fabs(lv(i + G, j + G + 1, k + G - 1) - lv(i + G, j + G, k + G - 1)) -
            std::fabs(lv(i + G, j + G, k + G - 2) - lv(i + G, j + G, k + G - 1));
      d01 = std::fabs(lv(i + G, j + G - 2, k + G) - lv(i + G, j + G - 1, k + G)) -
            std::fabs(lv(i + G, j + G - 1, k + G + 1) - lv(i + G, j + G - 1, k + G));
      d11 = std::fabs(lv(i + G, j + G + 1, k + G) - lv(i + G, j + G, k + G)) -
            std::fabs(lv(i + G, j + G, k + G + 1) - lv(i + G, j + G, k + G));
    } else if (dir == 2) {
      d00 = std::fabs(lv(i + G - 1, j + G, k + G - 2) - lv(i + G - 1, j + G, k + G - 1)) -
            std::fabs(lv(i + G - 2, j + G, k + G - 1) - lv(i + G - 1, j + G, k + G - 1));
      d10 = std::fabs(lv(i + G - 1, j + G, k + G + 1) - lv(i + G - 1, j + G, k + G)) -
            std::fabs(lv(i + G - 2, j + G, k + G) - lv(i + G - 1, j + G, k + G));
      d01 = std::fabs(lv(i + G, j + G, k + G - 2) - lv(i + G, j + G, k + G - 1)) -
            std::fabs(lv(i + G + 1, j + G, k + G - 1) - lv(i + G, j + G, k + G - 1));
      d11 = std::fabs(lv(i + G, j + G, k + G + 1) - lv(i + G, j + G, k + G)) -
            std::fabs(lv(i + G + 1, j + G, k + G) - lv(i + G, j + G, k + G));
    } else {
      d00 = std::fabs(lv(i + G - 2, j + G - 1, k + G) - lv(i + G - 1, j + G - 1, k + G)) -
            std::fabs(lv(i + G - 1, j + G - 2, k + G) - lv(i + G - 1, j + G - 1, k + G));
      d10 = std::fabs(lv(i + G + 1, j + G - 1, k + G) - lv(i + G, j + G - 1, k + G)) -
            std::fabs(lv(i + G, j + G - 2, k + G) - lv(i + G, j + G - 1, k + G));
      d01 = std::fabs(lv(i + G - 2, j + G, k + G) - lv(i + G - 1, j + G, k + G)) -
            std::fabs(lv(i + G - 1, j + G + 1, k + G) - lv(i + G - 1, j + G, k + G));
      d11 = std::fabs(lv(i + G + 1, j + G, k + G) - lv(i + G, j + G, k + G)) -
            std::fabs(lv(i + G, j + G + 1, k + G) - lv(i + G, j + G, k + G));
    }
    return blend4(d00, d10, d01, d11, a00_0, a00_1, a10_0, a10_1, a01_0, a01_1, a11_0, a11_1);
  }
  static inline double blend4(double d00, double d10, double d01, double d11, double a00_0, double a00_1,
                              double a10_0, double a10_1, double a01_0, double a01_1, double a11_0,
                              double a11_1) {
    d00 = fsign1(d00); d10 = fsign1(d10); d01 = fsign1(d01); d11 = fsign1(d11);
    double v00 = (1.0 + d00) / 2.0 * a00_0 + (1.0 - d00) / 2.0 * a00_1;
    double v10 = (1.0 + d10) / 2.0 * a10_0 + (1.0 - d10) / 2.0 * a10_1;
    double v01 = (1.0 + d01) / 2.0 * a01_0 + (1.0 - d01) / 2.0 * a01_1;
    double v11 = (1.0 + d11) / 2.0 * a11_0 + (1.0 - d11) / 2.0 * a11_1;
    return 0.25 * (v00 + v01 + v10 + v11);
  }

  // get_vav_center2corner (mhd3d3.f90:1858-2116)
  void get_vav_center2corner(const A3& lv, A3& vav, int dir) {
    int ii = nx0 + 1, jj = ny0 + 1, kk = nz0 + 1;
    if (dir == 1) ii = nx0;
    else if (dir == 2) jj = ny0;
    else kk = nz0;
    A3 v00_0(ii, jj, kk), v00_1(ii, jj, kk), v10_0(ii, jj, kk), v10_1(ii, jj, kk);
    A3 v01_0(ii, jj, kk), v01_1(ii, jj, kk), v11_0(ii, jj, kk), v11_1(ii, jj, kk);
    if (reconop == 1 || reconop == 2 || reconop == 5) {
      A3 vi(ii, jj, kk);
      bool tvd = (reconop != 1), mc = (reconop == 5);
      if (!tvd) interp2_pdm(lv, vi, dir);
      else interp2_tvd(lv, vi, dir);
      auto L = [&](A3& a, A3& b, int sx, int sy, int sz, int d) {
        if (!tvd) PDM2(a, b, lv, vi, ii, jj, kk, sx, sy, sz, d);
        else TVD(a, b, lv, vi, ii, jj, kk, sx, sy, sz, d, mc);
      };
      if (dir == 1) {
        L(v00_0, v10_0, 0, 0, -1, 2);
        L(v00_1, v01_1, 0, -1, 0, 3);
        L(v10_1, v11_1, 0, 0, 0, 3);
        L(v01_0, v11_0, 0, 0, 0, 2);
      } else if (dir == 2) {
        L(v00_0, v10_0, -1, 0, 0, 3);
        L(v00_1, v01_1, 0, 0, -1, 1);
        L(v10_1, v11_1, 0, 0, 0, 1);
        L(v01_0, v11_0, 0, 0, 0, 3);
      } else {
        L(v00_0, v10_0, 0, -1, 0, 1);
        L(v00_1, v01_1, -1, 0, 0, 2);
        L(v10_1, v11_1, 0, 0, 0, 2);
        L(v01_0, v11_0, 0, 0, 0, 1);
      }
    } else {
      // WENO5 / MPWENO5 two-level reconstruction (mhd3d3.f90:1925-2049 /
      // 1989-2049).  vi is the full (nx,ny,nz) scratch; only its rows / planes
      // written just before each use are read.
      bool mp = (reconop == 4);
      A3 vi(nx, ny, nz), lvl, lvr;
      auto W = [&](A3& a, A3& b, const A3& f, int l1, int l2, int l3, int d) {
        a.alloc(l1, l2, l3);
        b.alloc(l1, l2, l3);
        WENO5(a, b, f, l1, l2, l3, d, mp);
      };
      auto rows_y = [&](const A3& src) {
        FOR3(nx, jj, nz) { vi(i, ng + j, k) = src(i, j, k); }
      };
      auto planes_z = [&](const A3& src) {
        FOR3(nx, ny, kk) { vi(i, j, ng + k) = src(i, j, k); }
      };
      auto cols_x = [&](const A3& src) {
        FOR3(ii, ny, nz) { vi(ng + i, j, k) = src(i, j, k); }
      };
      if (dir == 1) {
        W(lvl, lvr, lv, nx, jj, nz, 5);
        rows_y(lvl); W(v00_1, v01_1, vi, ii, jj, kk, 3);
        rows_y(lvr); W(v10_1, v11_1, vi, ii, jj, kk, 3);
        W(lvl, lvr, lv, nx, ny, kk, 6);
        planes_z(lvl); W(v00_0, v01_0, vi, ii, jj, kk, 2);
        planes_z(lvr); W(v10_0, v11_0, vi, ii, jj, kk, 2);
      } else if (dir == 2) {
        W(lvl, lvr, lv, nx, ny, kk, 6);
        planes_z(lvl); W(v00_1, v01_1, vi, ii, jj, kk, 1);
        planes_z(lvr); W(v10_1, v11_1, vi, ii, jj, kk, 1);
        W(lvl, lvr, lv, ii, ny, nz, 4);
        cols_x(lvl); W(v00_0, v01_0, vi, ii, jj, kk, 3);
        cols_x(lvr); W(v10_0, v11_0, vi, ii, jj, kk, 3);
      } else {
        W(lvl, lvr, lv, ii, ny, nz, 4);
        cols_x(lvl); W(v00_1, v01_1, vi, ii, jj, kk, 2);
        cols_x(lvr); W(v10_1, v11_1, vi, ii, jj, kk, 2);
        W(lvl, lvr, lv, nx, jj, nz, 5);
        rows_y(lvl); W(v00_0, v01_0, vi, ii, jj, kk, 1);
        rows_y(lvr); W(v10_0, v11_0, vi, ii, jj, kk, 1);
      }
    }
    // quadrant selection by the sign of dif (mhd3d3.f90:2056-2108)
    vav.alloc(ii, jj, kk);
    FOR3(ii, jj, kk) {
      vav(i, j, k) = corner_blend_el(lv, dir, i, j, k, v00_0(i, j, k), v00_1(i, j, k), v10_0(i, j, k),
                                     v10_1(i, j, k), v01_0(i, j, k), v01_1(i, j, k), v11_0(i, j, k),
                                     v11_1(i, j, k));
    }
  }

  // The edge EMF of get_eijk_LFM (mhd3d3.f90:1806-1856) from its corner
  // velocities and face-B states, one element.
  inline double edge_emf_el(int kkk, int i, int j, int k, double v1av, double v2av, double b1l, double b1r,
                            double b2l, double b2r, const A3& vf) const {
    const int G = ng;
    double eta;
    if (kkk == 1)
      eta = 0.25 * (vf(i + G, j + G - 1, k + G - 1) + vf(i + G, j + G, k + G - 1) + vf(i + G, j + G, k + G) +
                    vf(i + G, j + G - 1, k + G));
    else if (kkk == 2)
      eta = 0.25 * (vf(i + G - 1, j + G, k + G - 1) + vf(i + G - 1, j + G, k + G) + vf(i + G, j + G, k + G) +
                    vf(i + G, j + G, k + G - 1));
    else
      eta = 0.25 * (vf(i + G - 1, j + G - 1, k + G) + vf(i + G, j + G - 1, k + G) + vf(i + G, j + G, k + G) +
                    vf(i + G - 1, j + G, k + G));
    return edge_combine(v1av, v2av, b1l, b1r, b2l, b2r, eta);
  }
  static inline double edge_combine(double v1av, double v2av, double b1l, double b1r, double b2l, double b2r,
                                    double eta) {
    double sig1 = fsign1(v1av), sig2 = fsign1(v2av);
    double b1u = (1.0 + sig2) / 2.0 * b1l + (1.0 - sig2) / 2.0 * b1r;
    double b2u = (1.0 + sig1) / 2.0 * b2l + (1.0 - sig1) / 2.0 * b2r;
    double dum = -v1av * b2u + v2av * b1u;
    return dum + eta * (b1l + b2r - b1r - b2l);
  }

  // get_eijk_LFM (mhd3d3.f90:1754-1856)
  void get_eijk_LFM(const A3& lrho, const A3& lvx, const A3& lvy, const A3& lvz, const A3& lp,
                    const A3& lbx, const A3& lby, const A3& lbz, const A3& lbi, const A3& lbj,
                    const A3& lbk) {
    (void)lp;
    if (metric) {
      get_eijk_metric(lrho, lvx, lvy, lvz, lbx, lby, lbz, lbi, lbj, lbk);
      return;
    }
    if (fused_edges()) {
      get_eijk_LFM_fused(lrho, lvx, lvy, lvz, lbx, lby, lbz, lbi, lbj, lbk);
      return;
    }
    A3 vf(nx, ny, nz);
    FOR3(nx, ny, nz) {
      double u = lvx(i, j, k), v = lvy(i, j, k), w = lvz(i, j, k);
      double a = lbx(i, j, k), b = lby(i, j, k), c = lbz(i, j, k);
      vf(i, j, k) = std::sqrt(u * u + v * v + w * w) + std::sqrt((a * a + b * b + c * c) / lrho(i, j, k));
    }
    for (int kkk = 1; kkk <= 3; ++kkk) {
      int ii = nx0 + 1, jj = ny0 + 1, kk = nz0 + 1, d1, d2;
      const A3 *v1, *v2, *b1, *b2;
      if (kkk == 1) { ii = nx0; v1 = &lvy; v2 = &lvz; b1 = &lbj; b2 = &lbk; d1 = 3; d2 = 2; }
      else if (kkk == 2) { jj = ny0; v1 = &lvz; v2 = &lvx; b1 = &lbk; b2 = &lbi; d1 = 1; d2 = 3; }
      else { kk = nz0; v1 = &lvx; v2 = &lvy; b1 = &lbi; b2 = &lbj; d1 = 2; d2 = 1; }
      A3 v1av, v2av, b1l, b1r, b2l, b2r;
      get_vav_center2corner(*v1, v1av, kkk);
      get_vav_center2corner(*v2, v2av, kkk);
      reconstruct_3d(b1l, b1r, *b1, ii, jj, kk, d1);
      reconstruct_3d(b2l, b2r, *b2, ii, jj, kk, d2);
      A3& e = (kkk == 1) ? ei : (kkk == 2) ? ej : ek;
      e.alloc(ii, jj, kk);
      FOR3(ii, jj, kk) {
        e(i, j, k) = edge_emf_el(kkk, i, j, k, v1av(i, j, k), v2av(i, j, k), b1l(i, j, k), b1r(i, j, k),
                                 b2l(i, j, k), b2r(i, j, k), vf);
      }
    }
  }

  // get_bxyz (mhd3d3.f90:2118-2128)
  void get_bxyz() {
    if (metric) {
      get_bxyz_metric();
      return;
    }
    FOR3(nx, ny, nz) {
      bx(i, j, k) = 0.5 * (bi(i + 1, j, k) + bi(i, j, k));
      by(i, j, k) = 0.5 * (bj(i, j + 1, k) + bj(i, j, k));
      bz(i, j, k) = 0.5 * (bk(i, j, k + 1) + bk(i, j, k));
    }
  }

  // get_eijk_Yee (mhd3d3.f90:1654-1752) with get_v_center (2562-2592, the
  // element formula of get_v_face): split electric fields of the Gaussian
  // velocity moments of every cell, each reconstructed to the edges in two
  // passes -- the left face state for a + moment, the right one for a -
  // moment -- and summed.  The reference keeps its calls commented out
  // (3354, 3621); emf = MHD_EMF_YEE selects it here.
  void get_eijk_Yee(const A3& lrho, const A3& lvx, const A3& lvy, const A3& lvz, const A3& lp,
                    const A3& lbx, const A3& lby, const A3& lbz) {
    A3 e[3][4];  // [x, y, z][pp, np, pn, nn]
    for (int f = 0; f < 3; ++f)
      for (int q = 0; q < 4; ++q) e[f][q].alloc(nx, ny, nz);
    FOR3(nx, ny, nz) {
      const double bxc = lbx(i, j, k), byc = lby(i, j, k), bzc = lbz(i, j, k);
      const double bsq = bxc * bxc + byc * byc + bzc * bzc;
      const double lam = lrho(i, j, k) / (2. * lp(i, j, k) + bsq);
      double x0p, x0n, x1p, x1n, y0p, y0n, y1p, y1n, z0p, z0n, z1p, z1n;
      v_face(lam, lvx(i, j, k), x0p, x0n, x1p, x1n);
      v_face(lam, lvy(i, j, k), y0p, y0n, y1p, y1n);
      v_face(lam, lvz(i, j, k), z0p, z0n, z1p, z1n);
      e[2][0](i, j, k) = bxc * x0p * y1p - byc * x1p * y0p;
      e[2][1](i, j, k) = bxc * x0n * y1p - byc * x1n * y0p;
      e[2][2](i, j, k) = bxc * x0p * y1n - byc * x1p * y0n;
      e[2][3](i, j, k) = bxc * x0n * y1n - byc * x1n * y0n;
      e[0][0](i, j, k) = byc * y0p * z1p - bzc * y1p * z0p;
      e[0][1](i, j, k) = byc * y0n * z1p - bzc * y1n * z0p;
      e[0][2](i, j, k) = byc * y0p * z1n - bzc * y1p * z0n;
      e[0][3](i, j, k) = byc * y0n * z1n - bzc * y1n * z0n;
      e[1][0](i, j, k) = bzc * z0p * x1p - bxc * z1p * x0p;
      e[1][1](i, j, k) = bzc * z0n * x1p - bxc * z1n * x0p;
      e[1][2](i, j, k) = bzc * z0p * x1n - bxc * z1p * x0n;
      e[1][3](i, j, k) = bzc * z0n * x1n - bxc * z1n * x0n;
    }
    // family kkk: first pass along d1 over (l1), second along d2 over (l2)
    for (int kkk = 1; kkk <= 3; ++kkk) {
      int d1, d2, l1[3], l2[3], oe[3];
      if (kkk == 1) {
        d1 = 5; d2 = 6; l1[0] = nx; l1[1] = ny0 + 1; l1[2] = nz; l2[0] = nx; l2[1] = ny0 + 1; l2[2] = nz0 + 1;
      } else if (kkk == 2) {
        d1 = 6; d2 = 4; l1[0] = nx; l1[1] = ny; l1[2] = nz0 + 1; l2[0] = nx0 + 1; l2[1] = ny; l2[2] = nz0 + 1;
      } else {
        d1 = 4; d2 = 5; l1[0] = nx0 + 1; l1[1] = ny; l1[2] = nz; l2[0] = nx0 + 1; l2[1] = ny0 + 1; l2[2] = nz;
      }
      A3* F = e[kkk - 1];
      A3 qpp, qpn, qnp, qnn, dum;
      reconstruct_3d(qpp, dum, F[0], l1[0], l1[1], l1[2], d1);
      reconstruct_3d(qpn, dum, F[2], l1[0], l1[1], l1[2], d1);
      reconstruct_3d(dum, qnn, F[3], l1[0], l1[1], l1[2], d1);
      reconstruct_3d(dum, qnp, F[1], l1[0], l1[1], l1[2], d1);
      A3 epp, enp, enn, epn, d2m;
      reconstruct_3d(epp, d2m, qpp, l2[0], l2[1], l2[2], d2);
      reconstruct_3d(enp, d2m, qnp, l2[0], l2[1], l2[2], d2);
      reconstruct_3d(d2m, enn, qnn, l2[0], l2[1], l2[2], d2);
      reconstruct_3d(d2m, epn, qpn, l2[0], l2[1], l2[2], d2);
      oe[0] = (kkk == 1) ? ng : 0; oe[1] = (kkk == 2) ? ng : 0; oe[2] = (kkk == 3) ? ng : 0;
      A3& E = (kkk == 1) ? ei : (kkk == 2) ? ej : ek;
      E.alloc(kkk == 1 ? nx0 : nx0 + 1, kkk == 2 ? ny0 : ny0 + 1, kkk == 3 ? nz0 : nz0 + 1);
      FOR3(E.n1, E.n2, E.n3) {
        const int a = i + oe[0], b = j + oe[1], c = k + oe[2];
        E(i, j, k) = epp(a, b, c) + enp(a, b, c) + epn(a, b, c) + enn(a, b, c);
      }
    }
  }
  // get_v_face (mhd3d3.f90:2594-2615), element form
  inline void v_face(double llam, double lv, double& v0p, double& v0n, double& v1p, double& v1n) const {
    double a = std::sqrt(llam);
    double b = 0.5 * std::exp(-llam * (lv * lv)) / a / std::sqrt(pi);
    v0p = 0.5 * std::erfc(-a * lv);
    v0n = 0.5 * std::erfc(a * lv);
    v1p = lv * v0p + b;
    v1n = lv * v0n - b;
  }

  // The Gaussian-split flux of one face (get_flux_stress, mhd3d3.f90:2418-2558)
  // from its left and right states {rho, vx, vy, vz, p, bx, by, bz}: o = {rho,
  // rho vx, rho vy, rho vz, energy, stress x, y, z} fluxes along axis kkk.
  inline void flux_el(int kkk, const double* L, const double* R, double* o) const {
    double v0p, v0n, v1p, v1n;
    // left flux
    double r = L[0], u = L[1], v = L[2], w = L[3], pp_ = L[4];
    double b1 = L[5], b2 = L[6], b3 = L[7];
    double vn = (kkk == 1) ? u : (kkk == 2) ? v : w;
    double bn = (kkk == 1) ? b1 : (kkk == 2) ? b2 : b3;
    double leng = 0.5 * r * (u * u + v * v + w * w) + pp_ / (gam - 1.0);
    double llam = r / (2.0 * pp_);
    v_face(llam, vn, v0p, v0n, v1p, v1n);
    double rp = r * v1p;
    double rvxp = r * u * v1p, rvyp = r * v * v1p, rvzp = r * w * v1p;
    double ep = (leng + 0.5 * pp_) * v1p;
    if (kkk == 1) rvxp = rvxp + pp_ * v0p;
    else if (kkk == 2) rvyp = rvyp + pp_ * v0p;
    else rvzp = rvzp + pp_ * v0p;
    ep = ep + 0.5 * pp_ * vn * v0p;
    double lbsq = b1 * b1 + b2 * b2 + b3 * b3;
    llam = r / (2.0 * pp_ + lbsq);
    v_face(llam, vn, v0p, v0n, v1p, v1n);
    double sxp = ((kkk == 1) ? (0.5 * lbsq - b1 * b1) : (-b1 * bn)) * v0p;
    double syp = ((kkk == 2) ? (0.5 * lbsq - b2 * b2) : (-b2 * bn)) * v0p;
    double szp = ((kkk == 3) ? (0.5 * lbsq - b3 * b3) : (-b3 * bn)) * v0p;
    // right flux
    r = R[0]; u = R[1]; v = R[2]; w = R[3]; pp_ = R[4];
    b1 = R[5]; b2 = R[6]; b3 = R[7];
    vn = (kkk == 1) ? u : (kkk == 2) ? v : w;
    bn = (kkk == 1) ? b1 : (kkk == 2) ? b2 : b3;
    leng = 0.5 * r * (u * u + v * v + w * w) + pp_ / (gam - 1.0);
    llam = r / (2.0 * pp_);
    v_face(llam, vn, v0p, v0n, v1p, v1n);
    double rn = r * v1n;
    double rvxn = r * u * v1n, rvyn = r * v * v1n, rvzn = r * w * v1n;
    double en = (leng + 0.5 * pp_) * v1n;
    if (kkk == 1) rvxn = rvxn + pp_ * v0n;
    else if (kkk == 2) rvyn = rvyn + pp_ * v0n;
    else rvzn = rvzn + pp_ * v0n;
    en = en + 0.5 * pp_ * vn * v0n;
    lbsq = b1 * b1 + b2 * b2 + b3 * b3;
    llam = r / (2.0 * pp_ + lbsq);
    v_face(llam, vn, v0p, v0n, v1p, v1n);
    double sxn = ((kkk == 1) ? (0.5 * lbsq - b1 * b1) : (-b1 * bn)) * v0n;
    double syn = ((kkk == 2) ? (0.5 * lbsq - b2 * b2) : (-b2 * bn)) * v0n;
    double szn = ((kkk == 3) ? (0.5 * lbsq - b3 * b3) : (-b3 * bn)) * v0n;
    o[0] = rp + rn;
    o[1] = rvxp + rvxn;
    o[2] = rvyp + rvyn;
    o[3] = rvzp + rvzn;
    o[4] = ep + en;
    o[5] = sxp + sxn;
    o[6] = syp + syn;
    o[7] = szp + szn;
  }

  // get_flux_stress (mhd3d3.f90:2385-2560)
  void get_flux_stress(const A3& lrho, const A3& lvx, const A3& lvy, const A3& lvz, const A3& lp,
                       const A3& lbx, const A3& lby, const A3& lbz) {
    if (metric) {
      get_flux_stress_metric(lrho, lvx, lvy, lvz, lp, lbx, lby, lbz);
      return;
    }
    if (fused) {
      get_flux_stress_fused(lrho, lvx, lvy, lvz, lp, lbx, lby, lbz);
      return;
    }
    for (int kkk = 1; kkk <= 3; ++kkk) {
      int ii = nx0, jj = ny0, kk = nz0;
      if (kkk == 1) ii = nx0 + 1;
      if (kkk == 2) jj = ny0 + 1;
      if (kkk == 3) kk = nz0 + 1;
      A3 rhol, rhor, vxl, vxr, vyl, vyr, vzl, vzr, pl, pr, bxl, bxr, byl, byr, bzl, bzr;
      reconstruct_3d(rhol, rhor, lrho, ii, jj, kk, kkk);
      reconstruct_3d(vxl, vxr, lvx, ii, jj, kk, kkk);
      reconstruct_3d(vyl, vyr, lvy, ii, jj, kk, kkk);
      reconstruct_3d(vzl, vzr, lvz, ii, jj, kk, kkk);
      reconstruct_3d(pl, pr, lp, ii, jj, kk, kkk);
      reconstruct_3d(bxl, bxr, lbx, ii, jj, kk, kkk);
      reconstruct_3d(byl, byr, lby, ii, jj, kk, kkk);
      reconstruct_3d(bzl, bzr, lbz, ii, jj, kk, kkk);
      A3* out = flux[kkk - 1];
      for (int q = 0; q < 8; ++q) out[q].alloc(ii, jj, kk);
      FOR3(ii, jj, kk) {
        const double L[8] = {rhol(i, j, k), vxl(i, j, k), vyl(i, j, k), vzl(i, j, k),
                             pl(i, j, k),   bxl(i, j, k), byl(i, j, k), bzl(i, j, k)};
        const double R[8] = {rhor(i, j, k), vxr(i, j, k), vyr(i, j, k), vzr(i, j, k),
                             pr(i, j, k),   bxr(i, j, k), byr(i, j, k), bzr(i, j, k)};
        double o[8];
        flux_el(kkk, L, R, o);
        for (int q = 0; q < 8; ++q) out[q](i, j, k) = o[q];
      }
    }
  }

  // ------------------------------------------------- fused (optimised) mode
  // One pass per face family and per edge family: every reconstruction is
  // evaluated where it is used, from the cell arrays, with no face, edge or
  // interpolant temporaries (the array passes above allocate and stream about
  // thirty of them per stage).  Each element calls the same element functions
  // as the array passes in the same order, so the two modes give identical
  // bits.  Cartesian meshes; the edge pass covers PDM / TVD / TVD-MC (the
  // two-level WENO corner reconstruction is not separable per edge and keeps
  // its array form), the face pass every reconstruction.
  bool fused = false;

  // Address of f(i, j, k) and the element stride along axis dir (1, 2, 3).
  static inline const double* at(const A3& f, int i, int j, int k) {
    return f.v.data() + ((size_t)(i - 1) + (size_t)f.n1 * ((size_t)(j - 1) + (size_t)f.n2 * (size_t)(k - 1)));
  }
  static inline ptrdiff_t stride(const A3& f, int dir) {
    return dir == 1 ? 1 : dir == 2 ? (ptrdiff_t)f.n1 : (ptrdiff_t)f.n1 * f.n2;
  }

  // reconstruct_3d (mhd3d3.f90:833-860) along one line of n elements: element
  // t reconstructs from c[t + m * s], m = -3..2, s the stride of the recon
  // axis.  One loop per reconstruction, no branches inside: it vectorises.
  template <int RECON>
  void recon_line(const double* c, ptrdiff_t s, int n, double* __restrict L, double* __restrict R) const {
    for (int t = 0; t < n; ++t) {
      const double* e = c + t;
      if constexpr (RECON == 1) {
        double fi = tap8(e[-4 * s], e[-3 * s], e[-2 * s], e[-s], e[0], e[s], e[2 * s], e[3 * s]);
        pdm2_el(e[-2 * s], e[-s], e[0], e[s], fi, L[t], R[t]);
      } else if constexpr (RECON == 2 || RECON == 5) {
        double fi = (e[-s] + e[0]) / 2.0;
        tvd_el(e[-2 * s], e[-s], e[0], e[s], fi, RECON == 5, L[t], R[t]);
      } else {
        double fm3 = e[-3 * s], fm2 = e[-2 * s], fm1 = e[-s], f0 = e[0], fp1 = e[s], fp2 = e[2 * s], fl, fr;
        weno5_pt(fm3, fm2, fm1, f0, fp1, fp2, eps, fl, fr);
        if constexpr (RECON == 4) {
          fl = mp_side(fl, fm3, fm2, fm1, f0, fp1, alpha, beta);
          fr = mp_side(fr, fp2, fp1, f0, fm1, fm2, alpha, beta);
        }
        L[t] = fl;
        R[t] = fr;
      }
    }
  }
  void recon_line_any(const double* c, ptrdiff_t s, int n, double* L, double* R) const {
    switch (reconop) {
      case 1: recon_line<1>(c, s, n, L, R); break;
      case 2: recon_line<2>(c, s, n, L, R); break;
      case 3: recon_line<3>(c, s, n, L, R); break;
      case 4: recon_line<4>(c, s, n, L, R); break;
      default: recon_line<5>(c, s, n, L, R); break;
    }
  }

  // get_vav_center2corner (mhd3d3.f90:1858-2116) along one line of n edges
  // (PDM / TVD).  Element t sits at c + t; sp and sq are the strides of the
  // edge's two transverse axes in the reference's order (edges along x: y, z;
  // along y: z, x; along z: x, y) -- interp2's first and second pass, the
  // limiters' axes and the quadrant differences all follow from them.
  // w: scratch of 17 lines.
  template <int RECON>
  void corner_line(const double* c, ptrdiff_t sp, ptrdiff_t sq, int n, double* __restrict out,
                   double* __restrict w, int W) const {
    double* vi = w;
    if constexpr (RECON == 1) {  // interp2_pdm: 8-tap along p, then along q
      double* g = w + W;
      for (int q = 0; q < 8; ++q) {
        const double* r = c + (q - 4) * sq;
        double* gq = g + q * W;
        for (int t = 0; t < n; ++t) {
          const double* e = r + t;
          gq[t] = tap8(e[-4 * sp], e[-3 * sp], e[-2 * sp], e[-sp], e[0], e[sp], e[2 * sp], e[3 * sp]);
        }
      }
      for (int t = 0; t < n; ++t)
        vi[t] = tap8(g[t], g[W + t], g[2 * W + t], g[3 * W + t], g[4 * W + t], g[5 * W + t], g[6 * W + t],
                     g[7 * W + t]);
    } else {  // interp2_tvd: 4-cell mean
      for (int t = 0; t < n; ++t) {
        const double* e = c + t;
        vi[t] = (e[-sp - sq] + e[-sq] + e[0] + e[-sp]) / 4.0;
      }
    }
    // the four limited pairs: (base shift, axis) = (-q, p), (-p, q), (0, q), (0, p);
    // TVD without the stencil-shift option drops the shifts
    const bool shift = (RECON == 1) || tvd_shift;
    double *a00_0 = w + 9 * W, *a10_0 = w + 10 * W, *a00_1 = w + 11 * W, *a01_1 = w + 12 * W;
    double *a10_1 = w + 13 * W, *a11_1 = w + 14 * W, *a01_0 = w + 15 * W, *a11_0 = w + 16 * W;
    auto lim = [&](const double* b, ptrdiff_t s, double* A, double* B) {
      for (int t = 0; t < n; ++t) {
        const double* e = b + t;
        if constexpr (RECON == 1) pdm2_el(e[-2 * s], e[-s], e[0], e[s], vi[t], A[t], B[t]);
        else tvd_el(e[-2 * s], e[-s], e[0], e[s], vi[t], RECON == 5, A[t], B[t]);
      }
    };
    lim(shift ? c - sq : c, sp, a00_0, a10_0);
    lim(shift ? c - sp : c, sq, a00_1, a01_1);
    lim(c, sq, a10_1, a11_1);
    lim(c, sp, a01_0, a11_0);
    // quadrant selection (mhd3d3.f90:2056-2108)
    for (int t = 0; t < n; ++t) {
      const double* e = c + t;
      double d00 = std::fabs(e[-2 * sp - sq] - e[-sp - sq]) - std::fabs(e[-sp - 2 * sq] - e[-sp - sq]);
      double d10 = std::fabs(e[sp - sq] - e[-sq]) - std::fabs(e[-2 * sq] - e[-sq]);
      double d01 = std::fabs(e[-2 * sp] - e[-sp]) - std::fabs(e[-sp + sq] - e[-sp]);
      double d11 = std::fabs(e[sp] - e[0]) - std::fabs(e[sq] - e[0]);
      out[t] = blend4(d00, d10, d01, d11, a00_0[t], a00_1[t], a10_0[t], a10_1[t], a01_0[t], a01_1[t], a11_0[t],
                      a11_1[t]);
    }
  }
  void corner_line_any(const double* c, ptrdiff_t sp, ptrdiff_t sq, int n, double* out, double* w, int W) const {
    if (reconop == 1) corner_line<1>(c, sp, sq, n, out, w, W);
    else if (reconop == 2) corner_line<2>(c, sp, sq, n, out, w, W);
    else corner_line<5>(c, sp, sq, n, out, w, W);
  }

  bool fused_edges() const { return fused && !metric && (reconop == 1 || reconop == 2 || reconop == 5); }

  // Runs body(j, k, buf, W) over the (j, k) lines of a jj x kk family, OpenMP
  // over k; buf holds nq per-thread line buffers of W = nx + 1 entries.
  template <class Body> void lines(int jj, int kk, int nq, Body body) {
    const int W = nx + 1;
#pragma omp parallel
    {
      std::vector<double> buf((size_t)nq * W);
#pragma omp for schedule(static)
      for (int k = 1; k <= kk; ++k)
        for (int j = 1; j <= jj; ++j) body(j, k, buf.data(), W);
    }
  }

  // get_eijk_LFM in one pass per edge family.  Per x line of edges: the two
  // corner velocities and the two face-B states into line buffers (unit-stride
  // loops over i that the compiler vectorises), then the edge combine.
  void get_eijk_LFM_fused(const A3& lrho, const A3& lvx, const A3& lvy, const A3& lvz, const A3& lbx,
                          const A3& lby, const A3& lbz, const A3& lbi, const A3& lbj, const A3& lbk) {
    A3 vf(nx, ny, nz);
    FOR3(nx, ny, nz) {
      double u = lvx(i, j, k), v = lvy(i, j, k), w = lvz(i, j, k);
      double a = lbx(i, j, k), b = lby(i, j, k), c = lbz(i, j, k);
      vf(i, j, k) = std::sqrt(u * u + v * v + w * w) + std::sqrt((a * a + b * b + c * c) / lrho(i, j, k));
    }
    for (int kkk = 1; kkk <= 3; ++kkk) {
      int ii = nx0 + 1, jj = ny0 + 1, kk = nz0 + 1, d1, d2;
      const A3 *v1, *v2, *b1, *b2;
      if (kkk == 1) { ii = nx0; v1 = &lvy; v2 = &lvz; b1 = &lbj; b2 = &lbk; d1 = 3; d2 = 2; }
      else if (kkk == 2) { jj = ny0; v1 = &lvz; v2 = &lvx; b1 = &lbk; b2 = &lbi; d1 = 1; d2 = 3; }
      else { kk = nz0; v1 = &lvx; v2 = &lvy; b1 = &lbi; b2 = &lbj; d1 = 2; d2 = 1; }
      A3& e = (kkk == 1) ? ei : (kkk == 2) ? ej : ek;
      e.alloc(ii, jj, kk);
      const ptrdiff_t sp = stride(vf, kkk == 1 ? 2 : kkk == 2 ? 3 : 1);
      const ptrdiff_t sq = stride(vf, kkk == 1 ? 3 : kkk == 2 ? 1 : 2);
      lines(jj, kk, 6 + 17, [&](int j, int k, double* b, int W) {
        double *v1a = b, *v2a = b + W, *b1l = b + 2 * W, *b1r = b + 3 * W, *b2l = b + 4 * W, *b2r = b + 5 * W;
        corner_line_any(at(*v1, ng + 1, ng + j, ng + k), sp, sq, ii, v1a, b + 6 * W, W);
        corner_line_any(at(*v2, ng + 1, ng + j, ng + k), sp, sq, ii, v2a, b + 6 * W, W);
        recon_line_any(at(*b1, ng + 1, ng + j, ng + k), stride(*b1, d1), ii, b1l, b1r);
        recon_line_any(at(*b2, ng + 1, ng + j, ng + k), stride(*b2, d2), ii, b2l, b2r);
        const double* cv = at(vf, ng + 1, ng + j, ng + k);
        double* eo = &e(1, j, k);
        for (int t = 0; t < ii; ++t) {
          const double* v = cv + t;
          const double eta = 0.25 * (v[-sp - sq] + v[-sq] + v[0] + v[-sp]);
          eo[t] = edge_combine(v1a[t], v2a[t], b1l[t], b1r[t], b2l[t], b2r[t], eta);
        }
      });
    }
  }

  // get_flux_stress in one pass per face family: per x line of faces the 16
  // reconstructed states into line buffers, then the fluxes.
  void get_flux_stress_fused(const A3& lrho, const A3& lvx, const A3& lvy, const A3& lvz, const A3& lp,
                             const A3& lbx, const A3& lby, const A3& lbz) {
    const A3* src[8] = {&lrho, &lvx, &lvy, &lvz, &lp, &lbx, &lby, &lbz};
    for (int kkk = 1; kkk <= 3; ++kkk) {
      int ii = nx0, jj = ny0, kk = nz0;
      if (kkk == 1) ii = nx0 + 1;
      if (kkk == 2) jj = ny0 + 1;
      if (kkk == 3) kk = nz0 + 1;
      A3* out = flux[kkk - 1];
      for (int q = 0; q < 8; ++q) out[q].alloc(ii, jj, kk);
      lines(jj, kk, 16, [&](int j, int k, double* b, int W) {
        for (int q = 0; q < 8; ++q)
          recon_line_any(at(*src[q], ng + 1, ng + j, ng + k), stride(*src[q], kkk), ii, b + q * W, b + (8 + q) * W);
        for (int i = 1; i <= ii; ++i) {
          double L[8], R[8], o[8];
          for (int q = 0; q < 8; ++q) {
            L[q] = b[q * W + i - 1];
            R[q] = b[(8 + q) * W + i - 1];
          }
          flux_el(kkk, L, R, o);
          for (int q = 0; q < 8; ++q) out[q](i, j, k) = o[q];
        }
      });
    }
  }

  // ------------------------------------------------------------ advance_*
  // advance_previous (mhd3d3.f90:3794-3819)
  void advance_previous() {
    rhop = rho; bip = bi; bjp = bj; bkp = bk;
    if (stepop == 1) {
      vxp = vx; vyp = vy; vzp = vz; pp = p; bxp = bx; byp = by; bzp = bz;
    } else {
      FOR3(nx, ny, nz) {
        double r = rho(i, j, k), u = vx(i, j, k), v = vy(i, j, k), w = vz(i, j, k);
        rhovxp(i, j, k) = r * u;
        rhovyp(i, j, k) = r * v;
        rhovzp(i, j, k) = r * w;
        engp(i, j, k) = 0.5 * r * (u * u + v * v + w * w) + p(i, j, k) / (gam - 1.0);
      }
    }
  }

  // advance_predictor_ab (mhd3d3.f90:3821-3840)
  void advance_predictor_ab() {
    double c = tau / tau0 / 2.0;
    auto pr = [&](A3& h, const A3& x, const A3& xp) {
      h.alloc(x.n1, x.n2, x.n3);
#pragma omp parallel for schedule(static)
      for (size_t n = 0; n < x.v.size(); ++n) h.v[n] = x.v[n] + c * (x.v[n] - xp.v[n]);
    };
    pr(rhoh, rho, rhop); pr(vxh, vx, vxp); pr(vyh, vy, vyp); pr(vzh, vz, vzp); pr(ph, p, pp);
    pr(bxh, bx, bxp); pr(byh, by, byp); pr(bzh, bz, bzp);
    pr(bih, bi, bip); pr(bjh, bj, bjp); pr(bkh, bk, bkp);
    advance_previous();
  }

  // advance_corrector1 (mhd3d3.f90:3842-3878)
  void advance_corrector1() {
    A3* F = flux[0]; A3* Gf = flux[1]; A3* H = flux[2];
    const int G = ng;
    if (metric) advance_corrector_metric(1);
    else FOR3(nx0, ny0, nz0) {
      double dx = dxb(G + i, G + j, G + k), dy = dyb(G + i, G + j, G + k), dz = dzb(G + i, G + j, G + k);
      auto d = [&](int q) {
        return (F[q](i + 1, j, k) - F[q](i, j, k)) / dx + (Gf[q](i, j + 1, k) - Gf[q](i, j, k)) / dy +
               (H[q](i, j, k + 1) - H[q](i, j, k)) / dz;
      };
      rho(G + i, G + j, G + k) = rho0(G + i, G + j, G + k) - tau * d(0);
      eng(G + i, G + j, G + k) = eng0(G + i, G + j, G + k) - tau * d(4);
      rhovx(G + i, G + j, G + k) = rhovx0(G + i, G + j, G + k) - tau * d(1);
      rhovy(G + i, G + j, G + k) = rhovy0(G + i, G + j, G + k) - tau * d(2);
      rhovz(G + i, G + j, G + k) = rhovz0(G + i, G + j, G + k) - tau * d(3);
    }
    if (stepop == 1) {
      FOR3(nx, ny, nz) {
        double a = rhovx(i, j, k), b = rhovy(i, j, k), c = rhovz(i, j, k);
        p(i, j, k) = (gam - 1.0) * (eng(i, j, k) - 0.5 * (a * a + b * b + c * c) / rho(i, j, k));
      }
    }
  }

  // advance_corrector2 (mhd3d3.f90:3880-3907)
  void advance_corrector2() {
    A3* F = flux[0]; A3* Gf = flux[1]; A3* H = flux[2];
    const int G = ng;
    if (metric) advance_corrector_metric(2);
    else FOR3(nx0, ny0, nz0) {
      double dx = dxb(G + i, G + j, G + k), dy = dyb(G + i, G + j, G + k), dz = dzb(G + i, G + j, G + k);
      auto d = [&](int q) {
        return (F[q](i + 1, j, k) - F[q](i, j, k)) / dx + (Gf[q](i, j + 1, k) - Gf[q](i, j, k)) / dy +
               (H[q](i, j, k + 1) - H[q](i, j, k)) / dz;
      };
      rhovx(G + i, G + j, G + k) = rhovx(G + i, G + j, G + k) - tau * d(5);
      rhovy(G + i, G + j, G + k) = rhovy(G + i, G + j, G + k) - tau * d(6);
      rhovz(G + i, G + j, G + k) = rhovz(G + i, G + j, G + k) - tau * d(7);
    }
    if (stepop == 1) vel_from_mom();
  }
  void vel_from_mom() {
    FOR3(nx, ny, nz) {
      vx(i, j, k) = rhovx(i, j, k) / rho(i, j, k);
      vy(i, j, k) = rhovy(i, j, k) / rho(i, j, k);
      vz(i, j, k) = rhovz(i, j, k) / rho(i, j, k);
    }
  }

  // advance_bijk (mhd3d3.f90:3909-3933)
  void advance_bijk() {
    if (metric) {
      advance_bijk_metric();
      return;
    }
    const int G = ng;
    FOR3(nx0 + 1, ny0, nz0) {
      bi(G + i, G + j, G + k) = bi(G + i, G + j, G + k) -
          tau * ((ek(i, j + 1, k) - ek(i, j, k)) / dyb(G + i, G + j, G + k) -
                 (ej(i, j, k + 1) - ej(i, j, k)) / dzb(G + i, G + j, G + k));
    }
    FOR3(nx0, ny0 + 1, nz0) {
      bj(G + i, G + j, G + k) = bj(G + i, G + j, G + k) -
          tau * ((ei(i, j, k + 1) - ei(i, j, k)) / dzb(G + i, G + j, G + k) -
                 (ek(i + 1, j, k) - ek(i, j, k)) / dxb(G + i, G + j, G + k));
    }
    FOR3(nx0, ny0, nz0 + 1) {
      bk(G + i, G + j, G + k) = bk(G + i, G + j, G + k) -
          tau * ((ej(i + 1, j, k) - ej(i, j, k)) / dxb(G + i, G + j, G + k) -
                 (ei(i, j + 1, k) - ei(i, j, k)) / dyb(G + i, G + j, G + k));
    }
  }

  // elementwise whole-array helpers for the stage combines
  template <class Fn> void each(A3& a, Fn fn) {
#pragma omp parallel for schedule(static)
    for (size_t n = 0; n < a.v.size(); ++n) a.v[n] = fn(n);
  }

  // Stage combine of step_rk2 / step_rk3 (mhd3d3.f90:3670-3705, 3741-3789).
  // c0,c1,den: X = (c0*Xp + c1*X)/den in the reference's operand order;
  // form 0: (Xp+X)/den, 1: (c0*Xp+X)/den, 2: (Xp+c1*X)/den.
  double comb(int form, double c, double xp, double x, double den) const {
    if (form == 0) return (xp + x) / den;
    if (form == 1) return (c * xp + x) / den;
    return (xp + c * x) / den;
  }

  void edge_emf(const A3& lrho, const A3& lvx, const A3& lvy, const A3& lvz, const A3& lp, const A3& lbx,
                const A3& lby, const A3& lbz, const A3& lbi, const A3& lbj, const A3& lbk) {
    if (emf == MHD_EMF_YEE) get_eijk_Yee(lrho, lvx, lvy, lvz, lp, lbx, lby, lbz);
    else get_eijk_LFM(lrho, lvx, lvy, lvz, lp, lbx, lby, lbz, lbi, lbj, lbk);
  }

  void rk_stage(int s, int nst) {
    get_conserve();
    edge_emf(rho, vx, vy, vz, p, bx, by, bz, bi, bj, bk);
    get_flux_stress(rho, vx, vy, vz, p, bx, by, bz);
    advance_corrector1();
    int form = -1; double c = 0, den = 1;
    if (s > 1) {
      if (nst == 2) { form = 0; den = 2.0; }
      else if (s == 2) { form = 1; c = 3.0; den = 4.0; }
      else { form = 2; c = 2.0; den = 3.0; }
    }
    if (form < 0) {
      rhovxh = rhovx; rhovyh = rhovy; rhovzh = rhovz;
    } else {
      each(rho, [&](size_t n) { return comb(form, c, rhop.v[n], rho.v[n], den); });
      rhovxh.alloc(nx, ny, nz); rhovyh.alloc(nx, ny, nz); rhovzh.alloc(nx, ny, nz);
      each(rhovxh, [&](size_t n) { return comb(form, c, rhovxp.v[n], rhovx.v[n], den); });
      each(rhovyh, [&](size_t n) { return comb(form, c, rhovyp.v[n], rhovy.v[n], den); });
      each(rhovzh, [&](size_t n) { return comb(form, c, rhovzp.v[n], rhovz.v[n], den); });
      each(eng, [&](size_t n) { return comb(form, c, engp.v[n], eng.v[n], den); });
    }
    each(p, [&](size_t n) {
      double a = rhovxh.v[n], b = rhovyh.v[n], cc = rhovzh.v[n];
      return (gam - 1.0) * (eng.v[n] - 0.5 * (a * a + b * b + cc * cc) / rho.v[n]);
    });
    advance_corrector2();
    if (form >= 0) {
      each(rhovx, [&](size_t n) { return comb(form, c, rhovxp.v[n], rhovx.v[n], den); });
      each(rhovy, [&](size_t n) { return comb(form, c, rhovyp.v[n], rhovy.v[n], den); });
      each(rhovz, [&](size_t n) { return comb(form, c, rhovzp.v[n], rhovz.v[n], den); });
    }
    vel_from_mom();
    advance_bijk();
    if (form >= 0) {
      each(bi, [&](size_t n) { return comb(form, c, bip.v[n], bi.v[n], den); });
      each(bj, [&](size_t n) { return comb(form, c, bjp.v[n], bj.v[n], den); });
      each(bk, [&](size_t n) { return comb(form, c, bkp.v[n], bk.v[n], den); });
    }
    fill_hydro();
    fill_mag();
    get_bxyz();
  }


  // ------------------------------------------------------------ metric mode
  static inline void cross(const double* a, const double* b, double* c) {
    c[0] = a[1] * b[2] - a[2] * b[1];
    c[1] = a[2] * b[0] - a[0] * b[2];
    c[2] = a[0] * b[1] - a[1] * b[0];
  }
  // node (i,j,k) coordinate vector
  inline void node(int i, int j, int k, double* x) const {
    x[0] = X[0](i, j, k); x[1] = X[1](i, j, k); x[2] = X[2](i, j, k);
  }
  // Face area vector 0.5*(d1 x d2) of the low face normal to `ax` of cell
  // (i,j,k) (face-array index), from its four nodes (diagonals d1, d2).
  void face_area(int ax, int i, int j, int k, double* A) const {
    double p0[3], p1[3], q0[3], q1[3], d1[3], d2[3];
    if (ax == 0) { node(i, j, k, p0); node(i, j + 1, k + 1, p1); node(i, j + 1, k, q0); node(i, j, k + 1, q1); }
    else if (ax == 1) { node(i, j, k, p0); node(i + 1, j, k + 1, p1); node(i, j, k + 1, q0); node(i + 1, j, k, q1); }
    else { node(i, j, k, p0); node(i + 1, j + 1, k, p1); node(i + 1, j, k, q0); node(i, j + 1, k, q1); }
    for (int c = 0; c < 3; ++c) { d1[c] = p1[c] - p0[c]; d2[c] = q1[c] - q0[c]; }
    cross(d1, d2, A);
    for (int c = 0; c < 3; ++c) A[c] = 0.5 * A[c];
  }
  // centroid (mean of the 4 nodes) of the low face normal to `ax`
  void face_centroid(int ax, int i, int j, int k, double* C) const {
    int o1[3] = {0, 0, 0}, o2[3] = {0, 0, 0};
    o1[(ax + 1) % 3] = 1;
    o2[(ax + 2) % 3] = 1;
    double a[3], b[3], c[3], d[3];
    node(i, j, k, a);
    node(i + o1[0], j + o1[1], k + o1[2], b);
    node(i + o1[0] + o2[0], j + o1[1] + o2[1], k + o1[2] + o2[2], c);
    node(i + o2[0], j + o2[1], k + o2[2], d);
    for (int q = 0; q < 3; ++q) C[q] = 0.25 * (a[q] + b[q] + c[q] + d[q]);
  }
  void metric_geometry() {
    int fe[3][3] = {{nx + 1, ny, nz}, {nx, ny + 1, nz}, {nx, ny, nz + 1}};
    for (int ax = 0; ax < 3; ++ax)
      for (int c = 0; c < 3; ++c) Af[ax][c].alloc(fe[ax][0], fe[ax][1], fe[ax][2]);
    for (int ax = 0; ax < 3; ++ax) {
      for (int k = 1; k <= fe[ax][2]; ++k)
        for (int j = 1; j <= fe[ax][1]; ++j)
          for (int i = 1; i <= fe[ax][0]; ++i) {
            double A[3];
            face_area(ax, i, j, k, A);
            for (int c = 0; c < 3; ++c) Af[ax][c](i, j, k) = A[c];
          }
    }
    vol.alloc(nx, ny, nz);
    for (int a = 0; a < 3; ++a)
      for (int c = 0; c < 3; ++c) eb[a][c].alloc(nx, ny, nz);
    for (int k = 1; k <= nz; ++k)
      for (int j = 1; j <= ny; ++j)
        for (int i = 1; i <= nx; ++i) {
          // V = (1/3) sum over faces of centroid . outward area
          double v = 0.0;
          for (int ax = 0; ax < 3; ++ax) {
            int hi[3] = {i, j, k};
            hi[ax] += 1;
            double Clo[3], Chi[3];
            face_centroid(ax, i, j, k, Clo);
            face_centroid(ax, hi[0], hi[1], hi[2], Chi);
            double slo = Clo[0] * Af[ax][0](i, j, k) + Clo[1] * Af[ax][1](i, j, k) + Clo[2] * Af[ax][2](i, j, k);
            double shi = Chi[0] * Af[ax][0](hi[0], hi[1], hi[2]) + Chi[1] * Af[ax][1](hi[0], hi[1], hi[2]) +
                         Chi[2] * Af[ax][2](hi[0], hi[1], hi[2]);
            v = v + (shi - slo);
            for (int c = 0; c < 3; ++c) eb[ax][c](i, j, k) = Chi[c] - Clo[c];
          }
          vol(i, j, k) = v / 3.0;
        }
  }
  double amag(int ax, int i, int j, int k) const {
    double a = Af[ax][0](i, j, k), b = Af[ax][1](i, j, k), c = Af[ax][2](i, j, k);
    return std::sqrt(a * a + b * b + c * c);
  }
  // cell-averaged area vector of the a-faces of cell (i,j,k)
  void abar(int ax, int i, int j, int k, double* A) const {
    int hi[3] = {i, j, k};
    hi[ax] += 1;
    for (int c = 0; c < 3; ++c) A[c] = 0.5 * (Af[ax][c](i, j, k) + Af[ax][c](hi[0], hi[1], hi[2]));
  }

  // B = sum_a (Phi_a averaged over the two a-faces / V) * (cell edge vector along a)
  void get_bxyz_metric() {
    A3* F[3] = {&bi, &bj, &bk};
    A3* B[3] = {&bx, &by, &bz};
    FOR3(nx, ny, nz) {
      double ph[3];
      for (int a = 0; a < 3; ++a) {
        int hi[3] = {i, j, k};
        hi[a] += 1;
        ph[a] = 0.5 * ((*F[a])(hi[0], hi[1], hi[2]) + (*F[a])(i, j, k)) / vol(i, j, k);
      }
      for (int c = 0; c < 3; ++c)
        (*B[c])(i, j, k) = ph[0] * eb[0][c](i, j, k) + ph[1] * eb[1][c](i, j, k) + ph[2] * eb[2][c](i, j, k);
    }
  }

  // CFL dt with 1/dx_a -> |abar_a| / V
  double get_dt_metric() {
    double m = INFINITY;
#pragma omp parallel for reduction(min : m) schedule(static)
    for (int k = 1; k <= nz; ++k)
      for (int j = 1; j <= ny; ++j)
        for (int i = 1; i <= nx; ++i) {
          double v = std::sqrt(vx(i, j, k) * vx(i, j, k) + vy(i, j, k) * vy(i, j, k) + vz(i, j, k) * vz(i, j, k));
          double btot = std::sqrt(bx(i, j, k) * bx(i, j, k) + by(i, j, k) * by(i, j, k) + bz(i, j, k) * bz(i, j, k));
          double valf = btot / std::sqrt(rho(i, j, k));
          double vs = std::sqrt(gam * p(i, j, k) / rho(i, j, k));
          double vcfl = v + std::sqrt(valf * valf + vs * vs);
          double s = 0.0;
          for (int a = 0; a < 3; ++a) {
            double A[3];
            abar(a, i, j, k, A);
            s = s + std::sqrt(A[0] * A[0] + A[1] * A[1] + A[2] * A[2]);
          }
          double dt = cfl / (vcfl * s / vol(i, j, k));
          m = (dt < m) ? dt : m;
        }
    return m;
  }

  // Face fluxes in metric form: the reference's Gaussian-split formulas with the
  // face normal n = A/|A| in place of the axis, vector momentum and stress, and
  // every flux multiplied by |A| (stored in `flux`, interior extents).
  void get_flux_stress_metric(const A3& lrho, const A3& lvx, const A3& lvy, const A3& lvz, const A3& lp,
                              const A3& lbx, const A3& lby, const A3& lbz) {
    for (int kkk = 1; kkk <= 3; ++kkk) {
      int ii = nx0, jj = ny0, kk = nz0;
      if (kkk == 1) ii = nx0 + 1;
      if (kkk == 2) jj = ny0 + 1;
      if (kkk == 3) kk = nz0 + 1;
      A3 L[8], R[8];
      const A3* src[8] = {&lrho, &lvx, &lvy, &lvz, &lp, &lbx, &lby, &lbz};
      for (int v = 0; v < 8; ++v) reconstruct_3d(L[v], R[v], *src[v], ii, jj, kk, kkk);
      A3* out = flux[kkk - 1];
      for (int q = 0; q < 8; ++q) out[q].alloc(ii, jj, kk);
      const int ax = kkk - 1;
      FOR3(ii, jj, kk) {
        const int fi = ng + i, fj = ng + j, fk = ng + k;  // face-array index of this face
        double A[3] = {Af[ax][0](fi, fj, fk), Af[ax][1](fi, fj, fk), Af[ax][2](fi, fj, fk)};
        double am = std::sqrt(A[0] * A[0] + A[1] * A[1] + A[2] * A[2]);
        double n[3] = {A[0] / am, A[1] / am, A[2] / am};
        double tot[8] = {0, 0, 0, 0, 0, 0, 0, 0};
        for (int side = 0; side < 2; ++side) {
          const A3* S = side == 0 ? L : R;
          double r = S[0](i, j, k), u[3] = {S[1](i, j, k), S[2](i, j, k), S[3](i, j, k)}, pr = S[4](i, j, k);
          double b[3] = {S[5](i, j, k), S[6](i, j, k), S[7](i, j, k)};
          double vn = u[0] * n[0] + u[1] * n[1] + u[2] * n[2];
          double bn = b[0] * n[0] + b[1] * n[1] + b[2] * n[2];
          double leng = 0.5 * r * (u[0] * u[0] + u[1] * u[1] + u[2] * u[2]) + pr / (gam - 1.0);
          double v0p, v0n, v1p, v1n;
          v_face(r / (2.0 * pr), vn, v0p, v0n, v1p, v1n);
          double v0 = side == 0 ? v0p : v0n, v1 = side == 0 ? v1p : v1n;
          double f[8];
          f[0] = r * v1;
          for (int c = 0; c < 3; ++c) f[1 + c] = r * u[c] * v1 + pr * n[c] * v0;
          f[4] = (leng + 0.5 * pr) * v1 + 0.5 * pr * vn * v0;
          double lbsq = b[0] * b[0] + b[1] * b[1] + b[2] * b[2];
          v_face(r / (2.0 * pr + lbsq), vn, v0p, v0n, v1p, v1n);
          v0 = side == 0 ? v0p : v0n;
          for (int c = 0; c < 3; ++c) f[5 + c] = (0.5 * lbsq * n[c] - b[c] * bn) * v0;
          for (int q = 0; q < 8; ++q) tot[q] = tot[q] + f[q];
        }
        for (int q = 0; q < 8; ++q) out[q](i, j, k) = tot[q] * am;
      }
    }
  }

  // w^a = v . nbar_a per cell, nbar_a = abar_a / |abar_a| the mean unit
  // normal of the a-faces (the velocity normal to those faces)
  void get_w(const A3& lvx, const A3& lvy, const A3& lvz) {
    for (int a = 0; a < 3; ++a) w[a].alloc(nx, ny, nz);
    for (int a = 0; a < 3; ++a) {
      FOR3(nx, ny, nz) {
        double A[3];
        abar(a, i, j, k, A);
        double m = std::sqrt(A[0] * A[0] + A[1] * A[1] + A[2] * A[2]);
        w[a](i, j, k) = lvx(i, j, k) * (A[0] / m) + lvy(i, j, k) * (A[1] / m) + lvz(i, j, k) * (A[2] / m);
      }
    }
  }

  // Edge circulation E.dl in metric form.  The reference's procedure runs on
  // normal components: w^a (corner-limited like v) and the face-normal field
  // b_a = Phi_a / |A_a| (reconstructed to the edge and upwinded like bi/bj/bk):
  //   E.dl = g_e (-w1 b2u + w2 b1u) + eta |dl_e| (b1l + b2r - b1r - b2l),
  //   g_e = |A1|_e |A2|_e / Vbar_e,
  // |A1|_e, |A2|_e the mean magnitudes of the two a1 (a2) faces that share
  // the edge and Vbar_e the mean volume of its 4 cells.  On a Cartesian mesh
  // g_e = |dl_e| = the edge length and E.dl = E dl of get_eijk_LFM.
  void get_eijk_metric(const A3& lrho, const A3& lvx, const A3& lvy, const A3& lvz, const A3& lbx,
                       const A3& lby, const A3& lbz, const A3& lbi, const A3& lbj, const A3& lbk) {
    A3 vf(nx, ny, nz);
    FOR3(nx, ny, nz) {
      double u = lvx(i, j, k), v = lvy(i, j, k), ww = lvz(i, j, k);
      double a = lbx(i, j, k), b = lby(i, j, k), c = lbz(i, j, k);
      vf(i, j, k) = std::sqrt(u * u + v * v + ww * ww) + std::sqrt((a * a + b * b + c * c) / lrho(i, j, k));
    }
    get_w(lvx, lvy, lvz);
    const A3* fb[3] = {&lbi, &lbj, &lbk};
    A3 bn[3];
    for (int a = 0; a < 3; ++a) {
      const A3& F = *fb[a];
      bn[a].alloc(F.n1, F.n2, F.n3);
      FOR3(F.n1, F.n2, F.n3) { bn[a](i, j, k) = F(i, j, k) / amag(a, i, j, k); }
    }
    for (int kkk = 1; kkk <= 3; ++kkk) {
      const int e = kkk - 1, a1 = (e + 1) % 3, a2 = (e + 2) % 3;
      int ii = nx0 + 1, jj = ny0 + 1, kk = nz0 + 1;
      if (e == 0) ii = nx0;
      else if (e == 1) jj = ny0;
      else kk = nz0;
      // b1 = normal field of the a1 faces reconstructed along a2, b2 = that
      // of the a2 faces along a1 (the reference's d1 / d2)
      A3 w1av, w2av, b1l, b1r, b2l, b2r;
      get_vav_center2corner(w[a1], w1av, kkk);
      get_vav_center2corner(w[a2], w2av, kkk);
      reconstruct_3d(b1l, b1r, bn[a1], ii, jj, kk, a2 + 1);
      reconstruct_3d(b2l, b2r, bn[a2], ii, jj, kk, a1 + 1);
      A3& E = (e == 0) ? ei : (e == 1) ? ej : ek;
      E.alloc(ii, jj, kk);
      FOR3(ii, jj, kk) {
        double ga, dl;
        edge_metric(e, ng + i, ng + j, ng + k, ga, dl);
        int c[3] = {ng + i, ng + j, ng + k};  // upper cell of the edge
        int m1[3] = {c[0], c[1], c[2]}, m2[3] = {c[0], c[1], c[2]}, m12[3] = {c[0], c[1], c[2]};
        m1[a1] -= 1; m2[a2] -= 1; m12[a1] -= 1; m12[a2] -= 1;
        double sig1 = fsign1(w1av(i, j, k)), sig2 = fsign1(w2av(i, j, k));
        double b1u = (1.0 + sig2) / 2.0 * b1l(i, j, k) + (1.0 - sig2) / 2.0 * b1r(i, j, k);
        double b2u = (1.0 + sig1) / 2.0 * b2l(i, j, k) + (1.0 - sig1) / 2.0 * b2r(i, j, k);
        double dum = -w1av(i, j, k) * b2u + w2av(i, j, k) * b1u;
        double eta = 0.25 * (vf(m12[0], m12[1], m12[2]) + vf(m2[0], m2[1], m2[2]) + vf(c[0], c[1], c[2]) +
                             vf(m1[0], m1[1], m1[2]));
        E(i, j, k) = ga * dum + eta * dl * (b1l(i, j, k) + b2r(i, j, k) - b1r(i, j, k) - b2l(i, j, k));
      }
    }
  }

  // g_e and |dl_e| of the e-directed edge whose upper cell is c = (ci,cj,ck)
  void edge_metric(int e, int ci, int cj, int ck, double& ga, double& dl) const {
    const int a1 = (e + 1) % 3, a2 = (e + 2) % 3;
    int c[3] = {ci, cj, ck};
    int m1[3] = {ci, cj, ck}, m2[3] = {ci, cj, ck}, m12[3] = {ci, cj, ck};
    m1[a1] -= 1; m2[a2] -= 1; m12[a1] -= 1; m12[a2] -= 1;
    double vb = 0.25 * (vol(m12[0], m12[1], m12[2]) + vol(m2[0], m2[1], m2[2]) + vol(c[0], c[1], c[2]) +
                        vol(m1[0], m1[1], m1[2]));
    double a1b = 0.5 * (amag(a1, m2[0], m2[1], m2[2]) + amag(a1, c[0], c[1], c[2]));
    double a2b = 0.5 * (amag(a2, m1[0], m1[1], m1[2]) + amag(a2, c[0], c[1], c[2]));
    ga = a1b * a2b / vb;
    int ce[3] = {ci, cj, ck};
    ce[e] += 1;
    double p0[3], p1[3];
    node(ci, cj, ck, p0);
    node(ce[0], ce[1], ce[2], p1);
    dl = std::sqrt((p1[0] - p0[0]) * (p1[0] - p0[0]) + (p1[1] - p0[1]) * (p1[1] - p0[1]) +
                   (p1[2] - p0[2]) * (p1[2] - p0[2]));
  }

  // conserved update with fluxes already multiplied by areas: / V
  void advance_corrector_metric(int which) {
    A3* F = flux[0]; A3* Gf = flux[1]; A3* H = flux[2];
    const int G = ng;
    FOR3(nx0, ny0, nz0) {
      double V = vol(G + i, G + j, G + k);
      auto d = [&](int q) {
        return ((F[q](i + 1, j, k) - F[q](i, j, k)) + (Gf[q](i, j + 1, k) - Gf[q](i, j, k)) +
                (H[q](i, j, k + 1) - H[q](i, j, k))) / V;
      };
      if (which == 1) {
        rho(G + i, G + j, G + k) = rho0(G + i, G + j, G + k) - tau * d(0);
        eng(G + i, G + j, G + k) = eng0(G + i, G + j, G + k) - tau * d(4);
        rhovx(G + i, G + j, G + k) = rhovx0(G + i, G + j, G + k) - tau * d(1);
        rhovy(G + i, G + j, G + k) = rhovy0(G + i, G + j, G + k) - tau * d(2);
        rhovz(G + i, G + j, G + k) = rhovz0(G + i, G + j, G + k) - tau * d(3);
      } else {
        rhovx(G + i, G + j, G + k) = rhovx(G + i, G + j, G + k) - tau * d(5);
        rhovy(G + i, G + j, G + k) = rhovy(G + i, G + j, G + k) - tau * d(6);
        rhovz(G + i, G + j, G + k) = rhovz(G + i, G + j, G + k) - tau * d(7);
      }
    }
  }

  // face fluxes: Phi -= tau * circulation of E.dl
  void advance_bijk_metric() {
    const int G = ng;
    FOR3(nx0 + 1, ny0, nz0) {
      bi(G + i, G + j, G + k) = bi(G + i, G + j, G + k) -
          tau * ((ek(i, j + 1, k) - ek(i, j, k)) - (ej(i, j, k + 1) - ej(i, j, k)));
    }
    FOR3(nx0, ny0 + 1, nz0) {
      bj(G + i, G + j, G + k) = bj(G + i, G + j, G + k) -
          tau * ((ei(i, j, k + 1) - ei(i, j, k)) - (ek(i + 1, j, k) - ek(i, j, k)));
    }
    FOR3(nx0, ny0, nz0 + 1) {
      bk(G + i, G + j, G + k) = bk(G + i, G + j, G + k) -
          tau * ((ej(i + 1, j, k) - ej(i, j, k)) - (ei(i, j + 1, k) - ei(i, j, k)));
    }
  }

  void check_status(double dtc) {
    // diag_rho_neg / diag_overflow (mhd3d3.f90:3143-3160) as status bits
    bool nan = false, negr = false, negp = false;
    for (size_t n = 0; n < rho.v.size(); ++n) {
      double r = rho.v[n], q = p.v[n];
      if (std::isnan(r) || std::isnan(q) || std::isnan(vx.v[n]) || std::isnan(vy.v[n]) || std::isnan(vz.v[n])) nan = true;
      if (r < 0.0) negr = true;
      if (q < 0.0) negp = true;
    }
    if (nan) status |= MHD_ST_NAN;
    if (negr) status |= MHD_ST_NEG_RHO;
    if (negp) status |= MHD_ST_NEG_P;
    (void)dtc;
  }

  // step (mhd3d3.f90:3585-3600) and step_ab/rk2/rk3
  void step() {
    double dtc = get_dt();  // get_dt at the top of every step_*
    check_status(dtc);
    if (stepop == 1) {  // step_ab (mhd3d3.f90:3602-3644)
      tau = dtc;
      get_conserve();
      advance_predictor_ab();
      tau0 = tau;
      edge_emf(rhoh, vxh, vyh, vzh, ph, bxh, byh, bzh, bih, bjh, bkh);
      get_flux_stress(rhoh, vxh, vyh, vzh, ph, bxh, byh, bzh);
      advance_corrector1();
      advance_corrector2();
      advance_bijk();
      fill_hydro();
      fill_mag();
      get_bxyz();
    } else {  // step_rk2 (3648-3711) / step_rk3 (3715-3792)
      if (dt_mode == MHD_DT_CFL) {
        tau = dtc;
        tau0 = dtc;
      } else {
        if (dtc < tau0) status |= MHD_ST_CFL;  // 'Attention! tau_cfl<' print
        tau = tau0;
      }
      advance_previous();
      int nst = (stepop == 2) ? 2 : 3;
      for (int s = 1; s <= nst; ++s) rk_stage(s, nst);
    }
  }

  // compensated (Neumaier) sums of mass and energy, max |div B|
  void diagnostics(double* out) {
    double ms = 0, mc = 0, es = 0, ec = 0, dmax = 0, rmin = INFINITY;
    auto add = [](double& s, double& c, double x) {
      double t = s + x;
      if (std::fabs(s) >= std::fabs(x)) c += (s - t) + x;
      else c += (x - t) + s;
      s = t;
    };
    const int G = ng;
    for (int k = 1; k <= nz0; ++k)
      for (int j = 1; j <= ny0; ++j)
        for (int i = 1; i <= nx0; ++i) {
          int I = G + i, J = G + j, K = G + k;
          double dv = metric ? vol(I, J, K) : dxv[I - 1] * dyv[J - 1] * dzv[K - 1];
          double r = rho(I, J, K), u = vx(I, J, K), v = vy(I, J, K), w = vz(I, J, K);
          double a = bx(I, J, K), b = by(I, J, K), c = bz(I, J, K);
          add(ms, mc, r * dv);
          double e = 0.5 * r * (u * u + v * v + w * w) + p(I, J, K) / (gam - 1.0) + 0.5 * (a * a + b * b + c * c);
          add(es, ec, e * dv);
          double db = metric ? ((bi(I + 1, J, K) - bi(I, J, K)) + (bj(I, J + 1, K) - bj(I, J, K)) +
                                (bk(I, J, K + 1) - bk(I, J, K))) / vol(I, J, K)
                             : (bi(I + 1, J, K) - bi(I, J, K)) / dxv[I - 1] + (bj(I, J + 1, K) - bj(I, J, K)) / dyv[J - 1] +
                                   (bk(I, J, K + 1) - bk(I, J, K)) / dzv[K - 1];
          dmax = std::max(dmax, std::fabs(db));
        }
    for (double r : rho.v) rmin = std::min(rmin, r);
    out[0] = ms + mc;
    out[1] = es + ec;
    out[2] = dmax;
    out[3] = rmin;
    out[4] = get_dt();
  }
};

void copy_in(A3& a, const double* src) { std::memcpy(a.v.data(), src, a.v.size() * sizeof(double)); }
void copy_out(const A3& a, double* dst) {
  if (dst) std::memcpy(dst, a.v.data(), a.v.size() * sizeof(double));
}

}  // namespace

extern "C" {

// Shared by oracle_init and oracle_init_mapped: dx/dy/dz are null in
// metric mode, xn/yn/zn null in Cartesian mode.
static void* init_common(const mhd_params* prm, const double* rho, const double* vx, const double* vy,
                         const double* vz, const double* p, const double* bi, const double* bj,
                         const double* bk, const double* dx, const double* dy, const double* dz,
                         const double* xn, const double* yn, const double* zn) {
  Oracle* o = new Oracle();
  o->nx0 = prm->nx0; o->ny0 = prm->ny0; o->nz0 = prm->nz0;
  o->nord = prm->nord; o->ng = prm->nord / 2;
  o->nx = o->nx0 + o->nord; o->ny = o->ny0 + o->nord; o->nz = o->nz0 + o->nord;
  o->reconop = prm->reconop; o->stepop = prm->stepop;
  for (int a = 0; a < 3; ++a) o->bc[a] = prm->bc[a];
  o->dt_mode = prm->dt_mode; o->tvd_shift = prm->tvd_shift; o->emf = prm->emf;
  o->gam = prm->gam; o->cfl = prm->cfl; o->pdmb = prm->pdmb; o->eps = prm->eps;
  o->alpha = prm->alpha; o->beta = prm->beta;
  o->pi = 4.0 * std::atan(1.0);
  o->tau = prm->tau; o->tau0 = prm->tau;  // read_input: tau0=tau (mhd3d3.f90:196)
  int nx = o->nx, ny = o->ny, nz = o->nz;
  if (xn) {
    o->metric = true;
    o->dxv.assign(nx, 1.0); o->dyv.assign(ny, 1.0); o->dzv.assign(nz, 1.0);
    for (int c = 0; c < 3; ++c) o->X[c].alloc(nx + 1, ny + 1, nz + 1);
    copy_in(o->X[0], xn); copy_in(o->X[1], yn); copy_in(o->X[2], zn);
    o->metric_geometry();
  } else {
    o->dxv.assign(dx, dx + nx); o->dyv.assign(dy, dy + ny); o->dzv.assign(dz, dz + nz);
  }
  A3* cells[] = {&o->rho, &o->vx, &o->vy, &o->vz, &o->p, &o->bx, &o->by, &o->bz, &o->rhovx, &o->rhovy,
                 &o->rhovz, &o->eng, &o->rho0, &o->rhovx0, &o->rhovy0, &o->rhovz0, &o->eng0, &o->rhop,
                 &o->vxp, &o->vyp, &o->vzp, &o->pp, &o->bxp, &o->byp, &o->bzp, &o->rhovxp, &o->rhovyp,
                 &o->rhovzp, &o->rhovxh, &o->rhovyh, &o->rhovzh, &o->engp};
  for (A3* a : cells) a->alloc(nx, ny, nz);
  o->bi.alloc(nx + 1, ny, nz); o->bj.alloc(nx, ny + 1, nz); o->bk.alloc(nx, ny, nz + 1);
  copy_in(o->rho, rho); copy_in(o->vx, vx); copy_in(o->vy, vy); copy_in(o->vz, vz); copy_in(o->p, p);
  copy_in(o->bi, bi); copy_in(o->bj, bj); copy_in(o->bk, bk);
  // initialization (mhd3d3.f90:3349-3351): fills then get_bxyz
  o->fill_hydro();
  o->fill_mag();
  o->get_bxyz();
  if (o->stepop == 1) {  // AB priming (mhd3d3.f90:3357-3373; mhd3d2.f90:3200-3216)
    double dtc = o->get_dt();
    if (!(prm->tau > 0.0)) o->tau = dtc;
    o->tau0 = o->tau;
    o->rhop = o->rho; o->vxp = o->vx; o->vyp = o->vy; o->vzp = o->vz; o->pp = o->p;
    o->bxp = o->bx; o->byp = o->by; o->bzp = o->bz; o->bip = o->bi; o->bjp = o->bj; o->bkp = o->bk;
  }
  return o;
}

void* oracle_init(const mhd_params* prm, const double* rho, const double* vx, const double* vy,
                  const double* vz, const double* p, const double* bi, const double* bj,
                  const double* bk, const double* dx, const double* dy, const double* dz) {
  return init_common(prm, rho, vx, vy, vz, p, bi, bj, bk, dx, dy, dz, nullptr, nullptr, nullptr);
}

// Metric mode: bi/bj/bk are face fluxes Phi = B.A; xn/yn/zn are the
// ghost-inclusive node coordinates, (nx+1)(ny+1)(nz+1) each, Fortran order.
void* oracle_init_mapped(const mhd_params* prm, const double* rho, const double* vx, const double* vy,
                         const double* vz, const double* p, const double* phi_i, const double* phi_j,
                         const double* phi_k, const double* xn, const double* yn, const double* zn) {
  return init_common(prm, rho, vx, vy, vz, p, phi_i, phi_j, phi_k, nullptr, nullptr, nullptr, xn, yn, zn);
}

// Cell volumes (nx, ny, nz) of a metric-mode oracle.
int oracle_volumes(void* h, double* out) {
  Oracle* o = (Oracle*)h;
  if (!o->metric) return -1;
  copy_out(o->vol, out);
  return 0;
}

int oracle_step(void* h, int nsteps, double* tau_out, uint32_t* status) {
  Oracle* o = (Oracle*)h;
  o->status = 0;
  for (int n = 0; n < nsteps; ++n) o->step();
  if (tau_out) *tau_out = o->tau;
  if (status) *status = o->status;
  return 0;
}

int oracle_fetch(void* h, double* rho, double* vx, double* vy, double* vz, double* p, double* bx,
                 double* by, double* bz, double* bi, double* bj, double* bk) {
  Oracle* o = (Oracle*)h;
  copy_out(o->rho, rho); copy_out(o->vx, vx); copy_out(o->vy, vy); copy_out(o->vz, vz);
  copy_out(o->p, p); copy_out(o->bx, bx); copy_out(o->by, by); copy_out(o->bz, bz);
  copy_out(o->bi, bi); copy_out(o->bj, bj); copy_out(o->bk, bk);
  return 0;
}

// Fluxes of the current state (get_flux_stress) in the reference's interior
// extents, dir-major then quantity-major.
int oracle_fluxes(void* h, double* out) {
  Oracle* o = (Oracle*)h;
  o->get_flux_stress(o->rho, o->vx, o->vy, o->vz, o->p, o->bx, o->by, o->bz);
  size_t off = 0;
  for (int d = 0; d < 3; ++d)
    for (int q = 0; q < 8; ++q) {
      const A3& a = o->flux[d][q];
      std::memcpy(out + off, a.v.data(), a.v.size() * sizeof(double));
      off += a.v.size();
    }
  return 0;
}

int oracle_emf(void* h, double* ei, double* ej, double* ek) {
  Oracle* o = (Oracle*)h;
  o->edge_emf(o->rho, o->vx, o->vy, o->vz, o->p, o->bx, o->by, o->bz, o->bi, o->bj, o->bk);
  copy_out(o->ei, ei); copy_out(o->ej, ej); copy_out(o->ek, ek);
  return 0;
}

int oracle_diagnostics(void* h, double* out) {
  ((Oracle*)h)->diagnostics(out);
  return 0;
}

// 1-D reconstruction of one line (unit tests): f has n values, faces
// m = 4..n-4 (1-based left cell m-1, right cell m); writes fl, fr of size n.
int oracle_recon_line(const mhd_params* prm, int n, const double* f, double* fl, double* fr) {
  Oracle o;
  o.ng = 4; o.nord = 8; o.reconop = prm->reconop; o.pdmb = prm->pdmb; o.eps = prm->eps;
  o.alpha = prm->alpha; o.beta = prm->beta; o.tvd_shift = 1;
  A3 F(n, 1, 1);
  for (int i = 0; i < n; ++i) F.v[i] = f[i];
  int lnx = n - 8;  // faces ng+1 .. ng+lnx: i in 1..lnx => face between cells ng+i-1, ng+i
  A3 L, R;
  // dir 4 keeps y,z extents (1,1) and shifts x by ng
  o.reconstruct_3d(L, R, F, lnx, 1, 1, 4);
  for (int i = 0; i < n; ++i) { fl[i] = 0.0; fr[i] = 0.0; }
  for (int i = 1; i <= lnx; ++i) { fl[o.ng + i - 1] = L(i, 1, 1); fr[o.ng + i - 1] = R(i, 1, 1); }
  return 0;
}

void oracle_free(void* h) { delete (Oracle*)h; }

// Fused mode of the following steps of handle h: one pass per face / edge
// family with no intermediate arrays; identical results to the array passes.
int oracle_set_fused(void* h, int on) {
  if (!h) return MHD_E_ARG;
  ((Oracle*)h)->fused = (on != 0);
  return 0;
}

int oracle_threads(void) { return omp_get_max_threads(); }

// Thread count of the following oracle calls (n <= 0: leave it unchanged).
void oracle_set_threads(int n) {
  if (n > 0) omp_set_num_threads(n);
}

}  // extern "C"
