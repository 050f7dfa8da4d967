// Device kernels of the per-timestep MHD update.  Included by exactly one
// translation unit per precision: mhd_fp64.cu (built with -fmad=false so that
// every FP64 expression is rounded exactly as the reference writes it) and
// mhd_fp32.cu (FMA contraction on, the performance path).
//
// Kernel map (reference routine -> kernel):
//   get_bxyz (mhd3d3.f90:2118-2128) + vf of get_eijk_LFM (1766)  -> k_bxyz_vf
//   get_dt   (1608-1639) + diag_rho_neg/diag_overflow (3143-3160) -> k_cfl, k_cfl_final
//   advance_previous (3794-3819)                                  -> k_save_prev
//   advance_predictor_ab (3821-3840)                              -> k_predictor_ab
//   get_flux_stress + get_v_face + reconstruct_3d (2385-2615, 833-1596)
//     -> k_flux (x faces), k_flux_t<D=1> (y faces, x+y divergence),
//        k_flux_t<D=2> (z faces + the conserved update below)
//   get_eijk_LFM + get_vav_center2corner + interp2_* (1754-2116, 926-1067) -> k_emf
//   get_conserve + advance_corrector1/2 + RK combines (1641-1650, 3842-3907,
//     3670-3697, 3741-3783)                                       -> k_flux_t<D=2>
//   advance_bijk + B combines (3909-3933, 3698-3702, 3784-3788)   -> k_update_b
//   fill_hydro_mpi / fill_mag_mpi (781-819, 346-616)              -> k_fill
#pragma once
#include <cuda_runtime.h>
#include <type_traits>
#include <atomic>
#include <math.h>
#include <stdint.h>
#include "mhd_state.h"

namespace mhd {

enum { R_PDM = 1, R_TVD = 2, R_WENO = 3, R_MPWENO = 4, R_TVDMC = 5 };
enum { BC_PERIODIC = 0, BC_EVEN = 1, BC_REFLECT = 2, BC_OUTFLOW = 3 };
enum { EMF_LFM = 0, EMF_YEE = 1 };

// Kernels with more than 48 KB of dynamic shared memory must be enabled per
// device: a launcher sets its attributes the first time it runs on the
// current device (idempotent if two host threads race; the bit is set only
// after the attributes are).
struct PerDevice {
  std::atomic<unsigned long long> done{0};
  bool need(unsigned long long& bit) {
    int dev = 0;
    cudaGetDevice(&dev);
    bit = 1ull << (dev & 63);
    return !(done.load(std::memory_order_acquire) & bit);
  }
  void mark(unsigned long long bit) { done.fetch_or(bit, std::memory_order_release); }
};

// Preferred shared-memory carveout (percent of the SM's maximum) of a kernel,
// set once per device.  The L1-reliant step passes ask for the shared memory
// they need and no more, so that the configuration a preceding
// shared-memory-heavy launch (the EMF slice rings) leaves behind does not
// shrink their L1.
#ifndef MHD_L1_PREF
#define MHD_L1_PREF 0
#endif
template <typename K>
inline void prefer_carveout(K kernel, int pct, PerDevice& attr) {
  if (!MHD_L1_PREF) return;
  unsigned long long bit = 0;
  if (attr.need(bit)) {
    cudaFuncSetAttribute(kernel, cudaFuncAttributePreferredSharedMemoryCarveout, pct);
    attr.mark(bit);
  }
}

inline dim3 grid3(int ni, int nj, int nk, dim3 b) {
  return dim3((ni + b.x - 1) / b.x, (nj + b.y - 1) / b.y, nk);
}
enum { ST_NAN = 1u, ST_NEG_RHO = 2u, ST_NEG_P = 4u, ST_CFL = 8u };

// ---------------------------------------------------------------- scalar ops
// Fortran sign(1,x) with ifort's default: +1 for x >= 0, including -0.0.
template <typename T> __device__ __forceinline__ T sgn1(T x) { return x >= T(0) ? T(1) : T(-1); }
template <typename T> __device__ __forceinline__ T mx(T a, T b) { return a > b ? a : b; }
template <typename T> __device__ __forceinline__ T mn(T a, T b) { return a < b ? a : b; }
__device__ __forceinline__ double fab(double x) { return fabs(x); }
__device__ __forceinline__ float fab(float x) { return fabsf(x); }
__device__ __forceinline__ double sq(double x) { return sqrt(x); }
__device__ __forceinline__ float sq(float x) { return sqrtf(x); }
__device__ __forceinline__ double ex(double x) { return exp(x); }
__device__ __forceinline__ float ex(float x) { return expf(x); }
__device__ __forceinline__ double erc(double x) { return erfc(x); }
__device__ __forceinline__ float erc(float x) { return erfcf(x); }

// Division by a constant: exact in FP64 (reference rounding), reciprocal
// multiply in FP32.
template <typename T> struct Div;
template <> struct Div<double> {
  static __device__ __forceinline__ double by(double a, double b) { return a / b; }
};
template <> struct Div<float> {
  static __device__ __forceinline__ float by(float a, float b) { return a * (1.0f / b); }
};

// Divisions on the hot path: FP64 divides exactly as the reference writes
// it; FP32 multiplies by a reciprocal (precomputed for the cell widths).
template <typename T> struct Ops;
template <> struct Ops<double> {
  static __device__ __forceinline__ double dw(double a, double w, double) { return a / w; }  // a / width
  static __device__ __forceinline__ double dv(double a, double b) { return a / b; }
  static __device__ __forceinline__ double rcp(double b) { return b; }  // used with dvr below
  static __device__ __forceinline__ double dvr(double a, double b, double) { return a / b; }
};
template <> struct Ops<float> {
  static __device__ __forceinline__ float dw(float a, float, float rw) { return a * rw; }
  static __device__ __forceinline__ float dv(float a, float b) { return __fdividef(a, b); }
  static __device__ __forceinline__ float rcp(float b) { return __frcp_rn(b); }
  static __device__ __forceinline__ float dvr(float a, float, float rb) { return a * rb; }
};

// 8-point centred interpolant (interp_pdm, mhd3d3.f90:866-872), operand order kept.
template <typename T>
__device__ __forceinline__ T tap8(T a0, T a1, T a2, T a3, T a4, T a5, T a6, T a7) {
  T s = T(-3) * a0;
  s = s + T(29) * a1;
  s = s - T(139) * a2;
  s = s + T(533) * a3;
  s = s + T(533) * a4;
  s = s - T(139) * a5;
  s = s + T(29) * a6;
  s = s - T(3) * a7;
  return Div<T>::by(s, T(840));
}

// PDM2 (mhd3d3.f90:1069-1172): clamp of the interpolant and partial-donor limiter.
template <typename T>
__device__ __forceinline__ void pdm2(T fm2, T fm1, T f0, T fp1, T fi, T pdmb, T& fl, T& fr) {
  T maxf = mx(fm1, f0), minf = mn(fm1, f0);
  T fii = mx(minf, mn(fi, maxf));
  T dfm = pdmb * (fm1 - fm2);
  T df0 = pdmb * (f0 - fm1);
  T dfp = pdmb * (fp1 - f0);
  T sm = sgn1(dfm), s0 = sgn1(df0), sp = sgn1(dfp);
  dfm = fab(dfm);
  dfp = fab(dfp);
  T qm = fab(sm + s0), qp = fab(s0 + sp);
  T dfl = fii - fm1, dfr = f0 - fii;
  fl = fii - s0 * mx(T(0), fab(dfl) - qm * dfm);
  fr = fii + s0 * mx(T(0), fab(dfr) - qp * dfp);
}

// TVD (mhd3d3.f90:1238-1248): van Leer b = (a+|a|)/(1+|a|); MC variant
// b = max(0, min(2a, (1+a)/2, 2)) (fi is the centred value, so b is phi(a)).
// Quotients: Ops<T>::dv divides exactly in FP64 (the reference's rounding)
// and multiplies by the hardware reciprocal in FP32.
template <typename T, bool MC>
__device__ __forceinline__ T tvdb(T a) {
  if (MC) return mx(T(0), mn(mn(T(2) * a, T(0.5) * (T(1) + a)), T(2)));
  return Ops<T>::dv(a + fab(a), T(1) + fab(a));
}
template <typename T, bool MC>
__device__ __forceinline__ void tvd(T fm2, T fm1, T f0, T fp1, T fi, T eps, T& fl, T& fr) {
  T a = Ops<T>::dv(fm1 - fm2, f0 - fm1 + eps);
  T b = tvdb<T, MC>(a);
  fl = fm1 - b * (fm1 - fi);
  a = Ops<T>::dv(f0 - fp1, fm1 - f0 + eps);
  b = tvdb<T, MC>(a);
  fr = f0 - b * (f0 - fi);
}

// WENO5 (mhd3d3.f90:1329-1375), one face.  The right state is the left-state
// formula on the mirrored stencil (fp2, fp1, f0, fm1, fm2), term for term, so
// both come from weno5_left.
template <typename T>
__device__ __forceinline__ T weno5_left(T fm3, T fm2, T fm1, T f0, T fp1, T eps) {
  const T c13 = T(13.0) / T(12.0);
  T h0 = Div<T>::by(T(2) * fm3 - T(7) * fm2 + T(11) * fm1, T(6));
  T h1 = Div<T>::by(-fm2 + T(5) * fm1 + T(2) * f0, T(6));
  T h2 = Div<T>::by(T(2) * fm1 + T(5) * f0 - fp1, T(6));
  T t = fm3 - T(2) * fm2 + fm1, u = fm3 - T(4) * fm2 + T(3) * fm1;
  T s0 = c13 * (t * t) + T(0.25) * (u * u);
  t = fm2 - T(2) * fm1 + f0; u = fm2 - f0;
  T s1 = c13 * (t * t) + T(0.25) * (u * u);
  t = fm1 - T(2) * f0 + fp1; u = T(3) * fm1 - T(4) * f0 + fp1;
  T s2 = c13 * (t * t) + T(0.25) * (u * u);
  s0 = Ops<T>::dv(T(0.1), (eps + s0) * (eps + s0));
  s1 = Ops<T>::dv(T(0.6), (eps + s1) * (eps + s1));
  s2 = Ops<T>::dv(T(0.3), (eps + s2) * (eps + s2));
  T sum = s0 + s1 + s2;
  return Ops<T>::dv(s0, sum) * h0 + Ops<T>::dv(s1, sum) * h1 + Ops<T>::dv(s2, sum) * h2;
}
template <typename T>
__device__ __forceinline__ void weno5(T fm3, T fm2, T fm1, T f0, T fp1, T fp2, T eps, T& fl, T& fr) {
  fl = weno5_left(fm3, fm2, fm1, f0, fp1, eps);
  fr = weno5_left(fp2, fp1, f0, fm1, fm2, eps);
}

// minmod (mhd3d3.f90:1380-1403): 0.5 (sign(1,a) + sign(1,b)) min(|a|, |b|).
// The factor is exactly 1, -1 or 0, so one comparison of the two signs and a
// select give the same value for every finite m = min(|a|, |b|) (NaN operands
// included: sign(1, NaN) counts as -1 on both forms).
template <typename T> __device__ __forceinline__ T minmod(T a, T b) {
  const T m = mn(fab(a), fab(b));
  const bool pa = a >= T(0), pb = b >= T(0);
  return (pa == pb) ? (pa ? m : -m) : T(0);
}
// Monotonicity-preserving bound of MPWENO5 (mhd3d3.f90:1530-1591) for one
// side; left state: (a3,a2,a1,b0,b1) = (fm3,fm2,fm1,f0,fp1), right state:
// (fp2,fp1,f0,fm1,fm2).
template <typename T>
__device__ __forceinline__ T mp_side(T w, T a3, T a2, T a1, T b0, T b1, T alpha, T beta) {
  T h0 = a3 - T(2) * a2 + a1;
  T h1 = a2 - T(2) * a1 + b0;
  T h2 = a1 - T(2) * b0 + b1;
  T s1 = minmod(T(4) * h1 - h2, T(4) * h2 - h1);
  T s2 = minmod(h1, h2);
  T s0 = minmod(s1, s2);
  T w1 = minmod(T(4) * h0 - h1, T(4) * h1 - h0);
  T w2 = minmod(h0, h1);
  T w0 = minmod(w1, w2);
  s1 = a1 + alpha * (a1 - a2);
  s2 = T(0.5) * (a1 + b0 - s0);
  s0 = T(0.5) * (T(3) * a1 - a2) + Div<T>::by(beta * w0, T(3));
  T lo = mx(mn(mn(a1, b0), s2), mn(mn(a1, s1), s0));
  T hi = mn(mx(mx(a1, b0), s2), mx(mx(a1, s1), s0));
  return w + minmod(lo - w, hi - w);
}

template <typename T>
struct Prm {
  T pdmb, eps, alpha, beta;
  int tvd_shift;
};

// One-sided face states of f at the low face of element c along stride s
// (reconstruct_3d for dirs 1-3, mhd3d3.f90:833-860).
// PDM face states from the 8 taps a0..a7 (cells c-4 .. c+3 along the
// reconstruction axis; the face at the low side of c).
template <typename T>
__device__ __forceinline__ void recon_pdm8(T a0, T a1, T a2, T a3, T a4, T a5, T a6, T a7, T pdmb, T& fl, T& fr) {
  const T fi = tap8(a0, a1, a2, a3, a4, a5, a6, a7);
  pdm2(a2, a3, a4, a5, fi, pdmb, fl, fr);
}

template <typename T, int RECON, typename I>
__device__ __forceinline__ void recon_face(const T* __restrict__ f, I c, I s, const Prm<T>& P, T& fl, T& fr) {
  if (RECON == R_PDM) {
    recon_pdm8(f[c - 4 * s], f[c - 3 * s], f[c - 2 * s], f[c - s], f[c], f[c + s], f[c + 2 * s], f[c + 3 * s], P.pdmb,
               fl, fr);
  } else if (RECON == R_TVD || RECON == R_TVDMC) {
    T fm2 = f[c - 2 * s], fm1 = f[c - s], f0 = f[c], fp1 = f[c + s];
    T fi = (fm1 + f0) / T(2);
    tvd<T, RECON == R_TVDMC>(fm2, fm1, f0, fp1, fi, P.eps, fl, fr);
  } else {
    T fm3 = f[c - 3 * s], fm2 = f[c - 2 * s], fm1 = f[c - s], f0 = f[c], fp1 = f[c + s], fp2 = f[c + 2 * s];
    weno5(fm3, fm2, fm1, f0, fp1, fp2, P.eps, fl, fr);
    if (RECON == R_MPWENO) {
      fl = mp_side(fl, fm3, fm2, fm1, f0, fp1, P.alpha, P.beta);
      fr = mp_side(fr, fp2, fp1, f0, fm1, fm2, P.alpha, P.beta);
    }
  }
}

// One side of weno_vals: the left state of the stencil (x0..x4) = (fm3..fp1);
// the right state is this on the mirrored stencil (fp2, fp1, f0, fm1, fm2).
template <typename T, int RECON>
__device__ __forceinline__ T weno_one(T x0, T x1, T x2, T x3, T x4, const Prm<T>& P) {
  T f = weno5_left(x0, x1, x2, x3, x4, P.eps);
  if (RECON == R_MPWENO) f = mp_side(f, x0, x1, x2, x3, x4, P.alpha, P.beta);
  return f;
}

// WENO5/MPWENO5 pair on six values held in registers.
template <typename T, int RECON>
__device__ __forceinline__ void weno_vals(const T* a, const Prm<T>& P, T& fl, T& fr) {
  weno5(a[0], a[1], a[2], a[3], a[4], a[5], P.eps, fl, fr);
  if (RECON == R_MPWENO) {
    fl = mp_side(fl, a[0], a[1], a[2], a[3], a[4], P.alpha, P.beta);
    fr = mp_side(fr, a[5], a[4], a[3], a[2], a[1], P.alpha, P.beta);
  }
}

// One half of pdm2 in a single form: the clamp pair (lo, hi) = (fm1, f0), the
// cell `outer` beyond the near end and the side (left: near = fm1, outer =
// fm2, result fii - s0*X; right: near = f0, outer = fp1, result fii + s0*X).
// The difference is formed in pdm2's own operand order for each side, so the
// result has pdm2's bits; the side is data, not control flow, so lanes that
// pick different sides do not diverge.
template <typename T>
__device__ __forceinline__ T pdm_half(T lo, T hi, T outer, bool left, T fi, T pdmb) {
  const T fii = mx(mn(lo, hi), mn(fi, mx(lo, hi)));
  const T near = left ? lo : hi;
  const T dn = pdmb * (left ? (lo - outer) : (outer - hi));  // pdm2's dfm / dfp
  const T s0 = sgn1(pdmb * (hi - lo));
  const T q = fab(sgn1(dn) + s0);
  const T x = s0 * mx(T(0), fab(near - fii) - q * fab(dn));
  return left ? fii - x : fii + x;
}

// PDM part of get_vav_center2corner (mhd3d3.f90:1901-1905, 2056-2108) for
// an edge with upper cell c and transverse strides s1 (d1), s2 (d2), given
// the corner interpolant vi: the four shifted PDM2 limiters, the quadrant
// choice by the sign of dif and the 4-quadrant mean.  Each quadrant keeps one
// of its two one-sided estimates, so the dif signs pick the stencil and the
// side first and only that half-limiter is evaluated (pdm_half: same bits as
// evaluating all four pdm2 and selecting).  v may point to global or shared
// memory.
// The same on the 12 cells it reads, named by (offset along d1, offset along
// d2) from the upper cell: mAB = (-A, -B), pAB = (+A, -B) etc.
template <typename T>
__device__ __forceinline__ T corner_pdm_vals(T m11, T m21, T m12, T m01, T p11, T m02, T m10, T m20, T m1p, T c0,
                                             T p10, T p01, T vi, T pd) {
  // quadrant cells q00 = (-1,-1), q10 = (0,-1), q01 = (-1,0), q11 = (0,0)
  const T d00 = fab(m21 - m11) - fab(m12 - m11);
  const T d10 = fab(p11 - m01) - fab(m02 - m01);
  const T d01 = fab(m20 - m10) - fab(m1p - m10);
  const T d11 = fab(p10 - c0) - fab(p01 - c0);
  // pdm2 #1 on (c-s2-2s1, c-s2-s1, c-s2, c-s2+s1) -> (v00_0, v10_0)
  // pdm2 #2 on (c-s1-2s2, c-s1-s2, c-s1, c-s1+s2) -> (v00_1, v01_1)
  // pdm2 #3 on (c-2s2, c-s2, c, c+s2)             -> (v10_1, v11_1)
  // pdm2 #4 on (c-2s1, c-s1, c, c+s1)             -> (v01_0, v11_0)
  const bool b00 = d00 >= T(0), b10 = d10 >= T(0), b01 = d01 >= T(0), b11 = d11 >= T(0);
  const T v00 = pdm_half(m11, b00 ? m01 : m10, b00 ? m21 : m12, true, vi, pd);
  const T v10 = pdm_half(b10 ? m11 : m01, b10 ? m01 : c0, b10 ? p11 : m02, !b10, vi, pd);
  const T v01 = pdm_half(b01 ? m10 : m11, b01 ? c0 : m10, b01 ? m20 : m1p, b01, vi, pd);
  const T v11 = pdm_half(b11 ? m10 : m01, c0, b11 ? p10 : p01, false, vi, pd);
  return T(0.25) * (v00 + v01 + v10 + v11);
}

template <typename T, typename I>
__device__ __forceinline__ T corner_pdm(const T* __restrict__ v, I c, I s1, I s2, T vi, T pd) {
  return corner_pdm_vals(v[c - s1 - s2], v[c - 2 * s1 - s2], v[c - s1 - 2 * s2], v[c - s2], v[c + s1 - s2],
                         v[c - 2 * s2], v[c - s1], v[c - 2 * s1], v[c - s1 + s2], v[c], v[c + s1], v[c + s2], vi, pd);
}

// Two values carried together (the v_a1 and v_a2 components of an edge): one
// 8-byte (FP32) or 16-byte (FP64) shared-memory access per pair, and FP32
// pair arithmetic on the packed FMA / MUL pipes (each lane rounds as the
// scalar fma / mul does); FP64 stays scalar, with separate mul and add as
// the reference writes them.
template <typename T> struct Pr;
template <> struct Pr<float> {
  typedef float2 V;
  static __device__ __forceinline__ V mk(float a, float b) { return make_float2(a, b); }
  static __device__ __forceinline__ V mul(float k, V a) { return __fmul2_rn(make_float2(k, k), a); }
  static __device__ __forceinline__ V mad(float k, V a, V c) { return __ffma2_rn(make_float2(k, k), a, c); }  // c + k a
  static __device__ __forceinline__ V by(V a, float b) { return mul(1.0f / b, a); }  // Div<float>::by
};
template <> struct Pr<double> {
  typedef double2 V;
  static __device__ __forceinline__ V mk(double a, double b) { return make_double2(a, b); }
  static __device__ __forceinline__ V mul(double k, V a) { return make_double2(k * a.x, k * a.y); }
  static __device__ __forceinline__ V mad(double k, V a, V c) { return make_double2(c.x + k * a.x, c.y + k * a.y); }
  static __device__ __forceinline__ V by(V a, double b) { return make_double2(a.x / b, a.y / b); }
};

// tap8 on pairs (same operand order: s = -3 a0, s + 29 a1, s - 139 a2, ...)
template <typename T>
__device__ __forceinline__ typename Pr<T>::V tap8p(typename Pr<T>::V a0, typename Pr<T>::V a1, typename Pr<T>::V a2,
                                                    typename Pr<T>::V a3, typename Pr<T>::V a4, typename Pr<T>::V a5,
                                                    typename Pr<T>::V a6, typename Pr<T>::V a7) {
  typedef Pr<T> Q;
  typename Q::V s = Q::mul(T(-3), a0);
  s = Q::mad(T(29), a1, s);
  s = Q::mad(T(-139), a2, s);
  s = Q::mad(T(533), a3, s);
  s = Q::mad(T(533), a4, s);
  s = Q::mad(T(-139), a5, s);
  s = Q::mad(T(29), a6, s);
  s = Q::mad(T(-3), a7, s);
  return Q::by(s, T(840));
}

// Compile-time knobs: MHD_FLUX_PACKED = 0 keeps the FP32 flux scalar (two
// independent left / right chains), MHD_RECON_PACKED = 0 the reconstruction.
#ifndef MHD_FLUX_PACKED
#define MHD_FLUX_PACKED 1
#endif
#ifndef MHD_RECON_PACKED
#define MHD_RECON_PACKED 1
#endif
namespace p2 {
__device__ __forceinline__ float2 K(float c) { return make_float2(c, c); }
__device__ __forceinline__ float2 add(float2 a, float2 b) { return __fadd2_rn(a, b); }
__device__ __forceinline__ float2 sub(float2 a, float2 b) { return __ffma2_rn(b, K(-1.0f), a); }  // a - b, one rounding
__device__ __forceinline__ float2 mul(float2 a, float2 b) { return __fmul2_rn(a, b); }
__device__ __forceinline__ float2 fma(float2 a, float2 b, float2 c) { return __ffma2_rn(a, b, c); }
__device__ __forceinline__ float2 rcp(float2 a) { return make_float2(__fdividef(1.0f, a.x), __fdividef(1.0f, a.y)); }
__device__ __forceinline__ float2 rsq(float2 a) { return make_float2(rsqrtf(a.x), rsqrtf(a.y)); }
}  // namespace p2

// corner_pdm of both components from pair-interleaved shared memory.
template <typename T>
__device__ __forceinline__ void corner_pdm_pair(const typename Pr<T>::V* __restrict__ v, int c, int s1, int s2,
                                                typename Pr<T>::V vi, T pd, T& r0, T& r1) {
  typedef typename Pr<T>::V V;
  const V m11 = v[c - s1 - s2], m21 = v[c - 2 * s1 - s2], m12 = v[c - s1 - 2 * s2], m01 = v[c - s2];
  const V p11 = v[c + s1 - s2], m02 = v[c - 2 * s2], m10 = v[c - s1], m20 = v[c - 2 * s1];
  const V m1p = v[c - s1 + s2], c0 = v[c], p10 = v[c + s1], p01 = v[c + s2];
  r0 = corner_pdm_vals(m11.x, m21.x, m12.x, m01.x, p11.x, m02.x, m10.x, m20.x, m1p.x, c0.x, p10.x, p01.x, vi.x, pd);
  r1 = corner_pdm_vals(m11.y, m21.y, m12.y, m01.y, p11.y, m02.y, m10.y, m20.y, m1p.y, c0.y, p10.y, p01.y, vi.y, pd);
}

// Limited corner value of v at the edge whose two transverse axes have
// strides s1 (d1) and s2 (d2) and whose upper cell is c
// (get_vav_center2corner, mhd3d3.f90:1858-2116).  Quadrant cell q_ab =
// c - (1-a) s1 - (1-b) s2; v_ab_0 / v_ab_1 are the two one-sided estimates.
template <typename T, int RECON>
__device__ __forceinline__ T corner_vel(const T* __restrict__ v, long long c, long long s1, long long s2,
                                        const Prm<T>& P) {
  T v00_0, v00_1, v10_0, v10_1, v01_0, v01_1, v11_0, v11_1;
  if (RECON == R_PDM) {
    // interp2_pdm (926-989): 8-tap along d1 at the 8 d2-rows, then along d2
    T g[8];
#pragma unroll
    for (int m = 0; m < 8; ++m) {
      const T* r = v + c + (long long)(m - 4) * s2;
      g[m] = tap8(r[-4 * s1], r[-3 * s1], r[-2 * s1], r[-s1], r[0], r[s1], r[2 * s1], r[3 * s1]);
    }
    T vi = tap8(g[0], g[1], g[2], g[3], g[4], g[5], g[6], g[7]);
    return corner_pdm(v, c, s1, s2, vi, P.pdmb);
  } else if (RECON == R_TVD || RECON == R_TVDMC) {
    // interp2_tvd (1037-1067) and TVD with (mhd3d2) or without (mhd3d3) shifts
    constexpr bool MC = (RECON == R_TVDMC);
    T vi = (v[c - s1 - s2] + v[c - s2] + v[c] + v[c - s1]) / T(4);
    long long a = P.tvd_shift ? c - s2 : c;
    long long b = P.tvd_shift ? c - s1 : c;
    tvd<T, MC>(v[a - 2 * s1], v[a - s1], v[a], v[a + s1], vi, P.eps, v00_0, v10_0);
    tvd<T, MC>(v[b - 2 * s2], v[b - s2], v[b], v[b + s2], vi, P.eps, v00_1, v01_1);
    tvd<T, MC>(v[c - 2 * s2], v[c - s2], v[c], v[c + s2], vi, P.eps, v10_1, v11_1);
    tvd<T, MC>(v[c - 2 * s1], v[c - s1], v[c], v[c + s1], vi, P.eps, v01_0, v11_0);
  } else {
    // WENO5 / MPWENO5 two-level reconstruction (1925-2049): "_1" = along d1
    // then d2, "_0" = along d2 then d1, with the reference's output naming.
    T L[6], R[6], a[6];
#pragma unroll
    for (int m = 0; m < 6; ++m) {
      const T* r = v + c + (long long)(m - 3) * s2;
#pragma unroll
      for (int t = 0; t < 6; ++t) a[t] = r[(long long)(t - 3) * s1];
      weno_vals<T, RECON>(a, P, L[m], R[m]);
    }
    weno_vals<T, RECON>(L, P, v00_1, v01_1);
    weno_vals<T, RECON>(R, P, v10_1, v11_1);
#pragma unroll
    for (int m = 0; m < 6; ++m) {
      const T* r = v + c + (long long)(m - 3) * s1;
#pragma unroll
      for (int t = 0; t < 6; ++t) a[t] = r[(long long)(t - 3) * s2];
      weno_vals<T, RECON>(a, P, L[m], R[m]);
    }
    weno_vals<T, RECON>(L, P, v00_0, v01_0);
    weno_vals<T, RECON>(R, P, v10_0, v11_0);
  }
  // dif signs pick the smoother one-sided estimate per quadrant (2056-2106)
  const long long q00 = c - s1 - s2, q10 = c - s2, q01 = c - s1, q11 = c;
  T d00 = fab(v[q00 - s1] - v[q00]) - fab(v[q00 - s2] - v[q00]);
  T d10 = fab(v[q10 + s1] - v[q10]) - fab(v[q10 - s2] - v[q10]);
  T d01 = fab(v[q01 - s1] - v[q01]) - fab(v[q01 + s2] - v[q01]);
  T d11 = fab(v[q11 + s1] - v[q11]) - fab(v[q11 + s2] - v[q11]);
  T v00 = d00 >= T(0) ? v00_0 : v00_1;
  T v10 = d10 >= T(0) ? v10_0 : v10_1;
  T v01 = d01 >= T(0) ? v01_0 : v01_1;
  T v11 = d11 >= T(0) ? v11_0 : v11_1;
  return T(0.25) * (v00 + v01 + v10 + v11);
}

// The current state as a stage input (RK stages of a batch read their own grid's state).
template <typename T>
__device__ __forceinline__ Inp<T> state_view(const Dev<T>& d) {
  return Inp<T>{d.rho, d.vx, d.vy, d.vz, d.p, d.bx, d.by, d.bz, d.bi, d.bj, d.bk};
}

// ------------------------------------------------------------ kernel args
// Argument of the step kernels that also run batched over an ensemble.
// B = false: one grid, its Dev by value, block index from blockIdx.
// B = true: many grids in one flattened 1-D launch; block b takes its grid
// and block coordinates from map[b] = {grid, bx, by, bz} and its Dev from
// tab[grid] (by value: a snapshot the compiler keeps in registers).
template <typename T, bool B> struct KArg;
template <typename T> struct KArg<T, false> {
  Dev<T> d;
  __device__ __forceinline__ int4 blk() const {
    return make_int4(0, (int)blockIdx.x, (int)blockIdx.y, (int)blockIdx.z);
  }
  __device__ __forceinline__ const Dev<T>& dev(const int4&) const { return d; }
};
template <typename T> struct KArg<T, true> {
  const Dev<T>* __restrict__ tab;
  const int4* __restrict__ map;
  __device__ __forceinline__ int4 blk() const { return map[blockIdx.x]; }
  __device__ __forceinline__ Dev<T> dev(const int4& b) const { return tab[b.x]; }
};
template <typename T>
inline KArg<T, false> one(const Dev<T>& d) { return KArg<T, false>{d}; }

// Resident 256-thread blocks per SM requested for the cell passes (CFL, CT +
// bxyz, fill).  Single grid: none (0; they take 32 registers).  Batched: each
// thread holds its grid's array pointers in registers (from the grid table,
// not the constant bank), about 75 registers unbounded, which would leave 3
// blocks per SM for these latency-bound passes; a budget keeps more resident.
#ifndef MHD_BATCH_MINB
#define MHD_BATCH_MINB 6
#endif
constexpr int pass_min_blocks(bool B) { return B ? MHD_BATCH_MINB : 0; }

// ------------------------------------------------------------- small kernels
template <typename T>
__device__ __forceinline__ long long idx3(const Geom& g, int i, int j, int k) {
  return (long long)i + (long long)g.px * ((long long)j + (long long)g.py * (long long)k);
}

// Metric-mode cell B from the face fluxes of cell c (low / high faces):
// B = sum_a (Phi_a averaged over the two a-faces / V) e_a, e_a the cell's
// edge vector along a (the oracle's get_bxyz_metric, in its operand order).
template <typename T>
__device__ __forceinline__ void cell_b_metric(const Metric& m, long long c, T lo0, T hi0, T lo1, T hi1, T lo2,
                                              T hi2, T& bx, T& by, T& bz) {
  const T V = (T)m.vol[c], rV = (T)m.rvol[c];
  const T p0 = Ops<T>::dw(T(0.5) * (hi0 + lo0), V, rV);
  const T p1 = Ops<T>::dw(T(0.5) * (hi1 + lo1), V, rV);
  const T p2 = Ops<T>::dw(T(0.5) * (hi2 + lo2), V, rV);
  bx = p0 * (T)m.eb[0][0][c] + p1 * (T)m.eb[1][0][c] + p2 * (T)m.eb[2][0][c];
  by = p0 * (T)m.eb[0][1][c] + p1 * (T)m.eb[1][1][c] + p2 * (T)m.eb[2][1][c];
  bz = p0 * (T)m.eb[0][2][c] + p1 * (T)m.eb[1][2][c] + p2 * (T)m.eb[2][2][c];
}

// get_bxyz over all cells (incl. ghosts) and vf = |v| + |B|/sqrt(rho).
template <typename T, bool M>
__global__ void k_bxyz_vf(Dev<T> d, int want_vf) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  int j = blockIdx.y * blockDim.y + threadIdx.y;
  int k = blockIdx.z;
  const Geom& g = d.g;
  if (i >= g.nx || j >= g.ny || k >= g.nz) return;
  long long c = idx3<T>(g, i, j, k);
  T bx, by, bz;
  if (M) {
    cell_b_metric<T>(d.m, c, d.bi[c], d.bi[c + 1], d.bj[c], d.bj[c + g.px], d.bk[c], d.bk[c + g.plane], bx, by, bz);
  } else {
    bx = T(0.5) * (d.bi[c + 1] + d.bi[c]);
    by = T(0.5) * (d.bj[c + g.px] + d.bj[c]);
    bz = T(0.5) * (d.bk[c + g.plane] + d.bk[c]);
  }
  d.bx[c] = bx;
  d.by[c] = by;
  d.bz[c] = bz;
  if (want_vf) {
    T u = d.vx[c], v = d.vy[c], w = d.vz[c];
    d.vf[c] = sq(u * u + v * v + w * w) + sq((bx * bx + by * by + bz * bz) / d.rho[c]);
  }
}

// get_dt over all cells incl. ghosts: per-block min, then atomicMin on the
// bit pattern (positive doubles order like their bits).  Status bits mirror
// diag_rho_neg / diag_overflow.
// Fast square root for the FP32 CFL estimate; exact in FP64.
__device__ __forceinline__ double cfl_sqrt(double x) { return sqrt(x); }
__device__ __forceinline__ float cfl_sqrt(float x) { return x > 0.0f ? x * rsqrtf(x) : 0.0f; }

// get_dt of one cell (mhd3d3.f90:1608-1639) from its primitives and cell B,
// with the status bits of its values.
template <typename T, bool M>
__device__ __forceinline__ T cell_dt(const Dev<T>& d, int c, int i, int j, int k, T r0, T p0, T u, T v, T w, T a,
                                     T b, T cc, unsigned& st) {
  typedef Ops<T> O;
  T vv = cfl_sqrt(u * u + v * v + w * w);
  T btot = cfl_sqrt(a * a + b * b + cc * cc);
  T valf = O::dv(btot, cfl_sqrt(r0));
  T vs = cfl_sqrt(O::dv(d.gam * p0, r0));
  T vcfl = vv + cfl_sqrt(valf * valf + vs * vs);
  T dt;
  if (M)  // metric mode: 1/dx_a -> |mean area vector of the a-faces| / V
    dt = O::dv(d.cfl, O::dw(vcfl * (T)d.m.sa[c], (T)d.m.vol[c], (T)d.m.rvol[c]));
  else
    dt = O::dv(d.cfl, O::dw(vcfl, d.wx[i], d.rwx[i]) + O::dw(vcfl, d.wy[j], d.rwy[j]) +
                          O::dw(vcfl, d.wz[k], d.rwz[k]));
  if (isnan(r0) || isnan(p0) || isnan(u) || isnan(v) || isnan(w)) st |= ST_NAN;
  if (r0 < T(0)) st |= ST_NEG_RHO;
  if (p0 < T(0)) st |= ST_NEG_P;
  if (isnan(dt)) st |= ST_NAN;
  return dt;
}

// Fold a thread's (dt, status) into the accumulators of the next step's
// state: block minimum (warp shuffles, then shared memory), then one atomic
// per block that lowers the running minimum (a plain read first skips the
// rest).  Every thread of the 256-thread block calls it.
template <typename T>
__device__ __forceinline__ void dt_next_accumulate(Scal* sc, T m, unsigned st) {
  for (int o = 16; o > 0; o >>= 1) {
    T y = __shfl_xor_sync(0xffffffffu, m, o);
    m = (y < m) ? y : m;
    st |= __shfl_xor_sync(0xffffffffu, st, o);
  }
  __shared__ T bm[8];
  __shared__ unsigned bs[8];
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  if (lane == 0) { bm[wid] = m; bs[wid] = st; }
  __syncthreads();
  if (threadIdx.x == 0) {
    for (int w = 1; w < 8; ++w) {
      m = (bm[w] < m) ? bm[w] : m;
      st |= bs[w];
    }
    const double md = (double)m;
    if (md >= 0.0) {
      const unsigned long long bits = (unsigned long long)__double_as_longlong(md);
      if (bits < *(volatile unsigned long long*)&sc->dtnext_bits) atomicMin(&sc->dtnext_bits, bits);
    }
    if (st) atomicOr(&sc->pend_status, st);
  }
}

// save != 0 also stores U^n of the RK stage combines (advance_previous,
// 3794-3819) at interior cells and faces, the only places they are read.
// next != 0: the dt and status go to the next-step accumulators.
// The minimum is reduced in T and converted to FP64 once per block.
template <typename T, bool M, bool B>
__global__ void __launch_bounds__(256, pass_min_blocks(B)) k_cfl(KArg<T, B> ka, int save, int next) {
  const int4 bb = ka.blk();
  const auto& d = ka.dev(bb);
  const Geom& g = d.g;
  T m = T(INFINITY);
  unsigned st = 0;
  const T gm1 = d.gam - T(1);
  typedef Ops<T> O;
  const int i = bb.y * 32 + (threadIdx.x & 31);
  const int j = bb.z * 8 + (threadIdx.x >> 5);
  const int k1 = min(g.nz, (bb.w + 1) * 8);
  for (int k = bb.w * 8; k < k1; ++k) {
    if (i >= g.nx || j >= g.ny) break;
    const int c = i + g.px * (j + g.py * k);
    T r0 = d.rho[c], p0 = d.p[c], u = d.vx[c], v = d.vy[c], w = d.vz[c];
    if (save) {
      const bool ix = i >= g.ng && i < g.ng + g.nx0, iy = j >= g.ng && j < g.ng + g.ny0,
                 iz = k >= g.ng && k < g.ng + g.nz0;
      if (ix && iy && iz) {
        d.q[0][c] = r0;
        d.q[1][c] = r0 * u;
        d.q[2][c] = r0 * v;
        d.q[3][c] = r0 * w;
        d.q[4][c] = T(0.5) * r0 * (u * u + v * v + w * w) + O::dv(p0, gm1);
      }
      const bool fx = i >= g.ng && i <= g.ng + g.nx0, fy = j >= g.ng && j <= g.ng + g.ny0,
                 fz = k >= g.ng && k <= g.ng + g.nz0;
      if (fx && iy && iz) d.q[5][c] = d.bi[c];
      if (ix && fy && iz) d.q[6][c] = d.bj[c];
      if (ix && iy && fz) d.q[7][c] = d.bk[c];
    }
    const T dt = cell_dt<T, M>(d, c, i, j, k, r0, p0, u, v, w, d.bx[c], d.by[c], d.bz[c], st);
    m = (dt < m) ? dt : m;
  }
  for (int o = 16; o > 0; o >>= 1) {
    T y = __shfl_xor_sync(0xffffffffu, m, o);
    m = (y < m) ? y : m;
    st |= __shfl_xor_sync(0xffffffffu, st, o);
  }
  __shared__ T sm[8];
  __shared__ unsigned ss[8];
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  if (lane == 0) { sm[wid] = m; ss[wid] = st; }
  __syncthreads();
  if (threadIdx.x == 0) {
    for (int w2 = 1; w2 < 8; ++w2) {
      m = (sm[w2] < m) ? sm[w2] : m;
      st |= ss[w2];
    }
    const double md = (double)m;
    if (md >= 0.0) atomicMin(next ? &d.sc->dtnext_bits : &d.sc->dtmin_bits, (unsigned long long)__double_as_longlong(md));
    if (st) atomicOr(next ? &d.sc->pend_status : &d.sc->status, st);
  }
}

// Empties the next-step accumulators before a dt pass refills them.
__global__ inline void k_next_reset(Scal* sc) {
  sc->dtnext_bits = (unsigned long long)__double_as_longlong(INFINITY);
  sc->pend_status = 0;
}

// tau selection of step_ab (3609) / step_rk2,3 (3656-3661, 3723-3728).
// mode 0: RK with fixed deck dt; 1: CFL dt every step; 2: AB (CFL dt and the
// predictor coefficient tau/tau0/2, then tau0=tau).
// mode | 4: take the dt and status accumulated for this state by the
// previous step (dtnext_bits, pend_status) and empty them.
template <typename T>
__global__ void k_cfl_final(Dev<T> d, int mode) {
  Scal* s = d.sc;
  double dt;
  if (mode & 4) {
    dt = __longlong_as_double((long long)s->dtnext_bits);
    s->dtnext_bits = (unsigned long long)__double_as_longlong(INFINITY);
    s->status |= s->pend_status;
    s->pend_status = 0;
    mode &= 3;
  } else {
    dt = __longlong_as_double((long long)s->dtmin_bits);
    s->dtmin_bits = (unsigned long long)__double_as_longlong(INFINITY);
  }
  s->dt_cfl = dt;
  if (mode == 0) {
    if (dt < s->tau0) s->status |= ST_CFL;
    s->tau = s->tau0;
  } else if (mode == 1) {
    s->tau = dt;
    s->tau0 = dt;
  } else if (mode == 2) {
    s->tau = dt;
    s->ab_coef = dt / s->tau0 / 2.0;
    s->tau0 = dt;
  }
  // mode 3: read-only (diagnostics); tau untouched
}

// k_cfl_final of every grid of a batch (one thread per grid; RK modes 0, 1).
template <typename T>
__global__ void k_cfl_final_batch(const Dev<T>* __restrict__ tab, int ngrids, int mode) {
  const int gi = blockIdx.x * blockDim.x + threadIdx.x;
  if (gi >= ngrids) return;
  Scal* s = tab[gi].sc;
  double dt = __longlong_as_double((long long)s->dtmin_bits);
  s->dtmin_bits = (unsigned long long)__double_as_longlong(INFINITY);
  s->dt_cfl = dt;
  if (mode == 0) {
    if (dt < s->tau0) s->status |= ST_CFL;
    s->tau = s->tau0;
  } else if (mode == 1) {
    s->tau = dt;
    s->tau0 = dt;
  }
}

// advance_previous for RK (3794-3819): U^n of the stage combines.
template <typename T>
__global__ void k_save_prev(Dev<T> d) {
  long long n = d.g.vol;
  T gm1 = d.gam - T(1);
  for (long long c = blockIdx.x * (long long)blockDim.x + threadIdx.x; c < n;
       c += (long long)gridDim.x * blockDim.x) {
    T r = d.rho[c], u = d.vx[c], v = d.vy[c], w = d.vz[c];
    d.q[0][c] = r;
    d.q[1][c] = r * u;
    d.q[2][c] = r * v;
    d.q[3][c] = r * w;
    d.q[4][c] = T(0.5) * r * (u * u + v * v + w * w) + d.p[c] / gm1;
    d.q[5][c] = d.bi[c];
    d.q[6][c] = d.bj[c];
    d.q[7][c] = d.bk[c];
  }
}

// advance_predictor_ab (3821-3840): Xh = X + tau/tau0/2*(X-Xp), then Xp = X;
// also vf of the predicted state.
template <typename T>
__global__ void k_predictor_ab(Dev<T> d) {
  long long n = d.g.vol;
  T cf = (T)d.sc->ab_coef;
  T* x[11] = {d.rho, d.vx, d.vy, d.vz, d.p, d.bi, d.bj, d.bk, d.bx, d.by, d.bz};
  for (long long c = blockIdx.x * (long long)blockDim.x + threadIdx.x; c < n;
       c += (long long)gridDim.x * blockDim.x) {
    T hv[11];
#pragma unroll
    for (int a = 0; a < 11; ++a) {
      T xv = x[a][c], xp = d.q[a][c];
      hv[a] = xv + cf * (xv - xp);
      d.h[a][c] = hv[a];
      d.q[a][c] = xv;
    }
    T rr = hv[0];
    d.vf[c] = (rr > T(0)) ? sq(hv[1] * hv[1] + hv[2] * hv[2] + hv[3] * hv[3]) +
                                sq((hv[8] * hv[8] + hv[9] * hv[9] + hv[10] * hv[10]) / rr)
                          : T(0);
  }
}

// ------------------------------------------------------------------ fluxes
// Gaussian velocity moments of get_v_face (mhd3d3.f90:2594-2615):
//   a = sqrt(lam), b = .5 exp(-lam v^2)/a/sqrt(pi), v0+- = .5 erfc(-+a v),
//   v1+- = v v0+- +- b.
// FP64: CUDA's sqrt/exp/erfc in the reference's operand order (parity mode).
// FP32: erfc from the Chebyshev fit "erfcc" of Numerical Recipes (Press et
// al., 2nd ed., sec. 6.2; fractional error < 1.2e-7 for all arguments),
// rsqrt and exp2-based exp (the performance path).
template <typename T> struct Moments;
template <> struct Moments<double> {
  static __device__ __forceinline__ void hydro(double lam, double vn, bool left, double& v0, double& v1) {
    const double rspi = sqrt(3.14159265358979323846);
    double a = sqrt(lam);
    double b = 0.5 * exp(-lam * (vn * vn)) / a / rspi;
    if (left) {
      v0 = 0.5 * erfc(-a * vn);
      v1 = vn * v0 + b;
    } else {
      v0 = 0.5 * erfc(a * vn);
      v1 = vn * v0 - b;
    }
  }
  static __device__ __forceinline__ double mag(double lam, double vn, bool left) {
    double a = sqrt(lam);
    return left ? 0.5 * erfc(-a * vn) : 0.5 * erfc(a * vn);
  }
  static __device__ __forceinline__ double div(double a, double b) { return a / b; }
};
template <> struct Moments<float> {
  // erfc(z) for z >= 0 (Numerical Recipes erfcc)
  static __device__ __forceinline__ float erfc_pos(float z) {
    float t = __fdividef(1.0f, fmaf(0.5f, z, 1.0f));
    float q = fmaf(t, 0.17087277f, -0.82215223f);
    q = fmaf(t, q, 1.48851587f);
    q = fmaf(t, q, -1.13520398f);
    q = fmaf(t, q, 0.27886807f);
    q = fmaf(t, q, -0.18628806f);
    q = fmaf(t, q, 0.09678418f);
    q = fmaf(t, q, 0.37409196f);
    q = fmaf(t, q, 1.00002368f);
    q = fmaf(t, q, -1.26551223f);
    return t * __expf(fmaf(-z, z, q));
  }
  // 0.5 erfc(-s x) for the left (s=+1) or 0.5 erfc(x) for the right state
  static __device__ __forceinline__ float half_erfc(float x, bool left) {
    float h = 0.5f * erfc_pos(fabsf(x));
    bool direct = left ? (x <= 0.0f) : (x >= 0.0f);
    return direct ? h : 1.0f - h;
  }
  static __device__ __forceinline__ void hydro(float lam, float vn, bool left, float& v0, float& v1) {
    float ra = rsqrtf(lam);
    float a = lam * ra;
    v0 = half_erfc(a * vn, left);
    float b = (0.5f * 0.56418958354775628f) * ra * __expf(-lam * vn * vn);
    v1 = left ? fmaf(vn, v0, b) : fmaf(vn, v0, -b);
  }
  static __device__ __forceinline__ float mag(float lam, float vn, bool left) {
    float a = lam * rsqrtf(lam);
    return half_erfc(a * vn, left);
  }
  static __device__ __forceinline__ float div(float a, float b) { return __fdividef(a, b); }
};

// ------------------------------------------------ FP32 packed-pair arithmetic
// Blackwell's packed FP32 instructions (FFMA2 / FMUL2 / FADD2) issue once for
// two lanes, each rounded as the scalar fma / mul / add.  The FP32 path
// evaluates the PDM face reconstruction on pairs of fields and the
// Gaussian-split flux on the (left, right) pair of a face with them; absolute
// values, min / max, signs and selects stay per lane, where the absolute
// values fold into the scalar instructions that use them.  Every FP32 face
// kernel (x faces, y / z face tiles and column sweeps, batched or not) goes
// through these functions, so they agree bit for bit.

// The limiter of pdm2 for one stencil, given the clamped interpolant fii, the
// one-sided differences dfl = fii - fm1, dfr = f0 - fii and the scaled cell
// differences dfm, df0, dfp: (left, right) face states.
__device__ __forceinline__ float2 pdm_lim(float fii, float dfl, float dfr, float dfm, float df0, float dfp) {
  const float sm = sgn1(dfm), s0 = sgn1(df0), sp = sgn1(dfp);
  const float qm = fabsf(sm + s0), qp = fabsf(s0 + sp);
  return make_float2(fii - s0 * mx(0.0f, fabsf(dfl) - qm * fabsf(dfm)),
                     fii + s0 * mx(0.0f, fabsf(dfr) - qp * fabsf(dfp)));
}

// PDM2 (mhd3d3.f90:1069-1172) of two stencils at once (lanes .x and .y, e.g.
// two fields at one face) from the interpolant pair fi: the differences on
// the packed pipe, the clamp and the limiter per lane.  lr0 / lr1 are the
// (left, right) states of lane x / lane y.
__device__ __forceinline__ void pdm2x2(float2 fm2, float2 fm1, float2 f0, float2 fp1, float2 fi, float pdmb,
                                       float2& lr0, float2& lr1) {
  const float2 kp = p2::K(pdmb);
  const float2 dfm = p2::mul(kp, p2::sub(fm1, fm2));
  const float2 df0 = p2::mul(kp, p2::sub(f0, fm1));
  const float2 dfp = p2::mul(kp, p2::sub(fp1, f0));
  float2 fii;
  fii.x = mx(mn(fm1.x, f0.x), mn(fi.x, mx(fm1.x, f0.x)));
  fii.y = mx(mn(fm1.y, f0.y), mn(fi.y, mx(fm1.y, f0.y)));
  const float2 dfl = p2::sub(fii, fm1), dfr = p2::sub(f0, fii);
  lr0 = pdm_lim(fii.x, dfl.x, dfr.x, dfm.x, df0.x, dfp.x);
  lr1 = pdm_lim(fii.y, dfl.y, dfr.y, dfm.y, df0.y, dfp.y);
}

// PDM face states of two fields from their 8-tap windows (tap m = cell
// c+m-4 for the face at the low side of cell c), packed as field pairs.
__device__ __forceinline__ void pdm_pair_states(const float2* a, float pdmb, float2& lr0, float2& lr1) {
  const float2 fi = tap8p<float>(a[0], a[1], a[2], a[3], a[4], a[5], a[6], a[7]);
  pdm2x2(a[2], a[3], a[4], a[5], fi, pdmb, lr0, lr1);
}

// 0.5 erfc(-x.x) (left state, + moment) and 0.5 erfc(x.y) (right state, -
// moment) with the erfcc fit of Moments<float>::erfc_pos: its polynomial is
// evaluated with negated coefficients, so exp(z^2 - (-q)) takes the same
// argument as erfc_pos's exp(-z^2 + q).
__device__ __forceinline__ float2 half_erfc_lr(float2 x) {
  const float2 z = make_float2(fabsf(x.x), fabsf(x.y));
  const float2 t = p2::rcp(p2::fma(p2::K(0.5f), z, p2::K(1.0f)));
  float2 nq = p2::fma(t, p2::K(-0.17087277f), p2::K(0.82215223f));
  nq = p2::fma(t, nq, p2::K(-1.48851587f));
  nq = p2::fma(t, nq, p2::K(1.13520398f));
  nq = p2::fma(t, nq, p2::K(-0.27886807f));
  nq = p2::fma(t, nq, p2::K(0.18628806f));
  nq = p2::fma(t, nq, p2::K(-0.09678418f));
  nq = p2::fma(t, nq, p2::K(-0.37409196f));
  nq = p2::fma(t, nq, p2::K(-1.00002368f));
  nq = p2::fma(t, nq, p2::K(1.26551223f));
  const float2 y = p2::fma(z, z, nq);  // z^2 - q
  const float2 e = make_float2(__expf(-y.x), __expf(-y.y));
  const float2 h = p2::mul(p2::K(0.5f), p2::mul(t, e));
  const float2 g = p2::sub(p2::K(1.0f), h);
  return make_float2(x.x <= 0.0f ? h.x : g.x, x.y >= 0.0f ? h.y : g.y);
}

// Fluxes and magnetic stress through one face normal to axis D (the
// formulas of face_flux) with the left state in lane x and the right state
// in lane y of X[q] = (l[q], r[q]); out = left + right.
template <int D>
__device__ __forceinline__ void face_flux_lr(const float2* X, float gam, float* out) {
  using namespace p2;
  const float rg = __frcp_rn(gam - 1.0f);
  const float2 r = X[0], u = X[1], v = X[2], w = X[3], pr = X[4], bx = X[5], by = X[6], bz = X[7];
  const float2 vn = X[1 + D], bn = X[5 + D];
  float2 ke = mul(u, u);
  ke = fma(v, v, ke);
  ke = fma(w, w, ke);
  const float2 leng = fma(pr, K(rg), mul(mul(K(0.5f), r), ke));
  // hydro moments, lam = rho / (2 p)
  const float2 lam = mul(r, rcp(mul(K(2.0f), pr)));
  const float2 ra = rsq(lam);
  const float2 v0 = half_erfc_lr(mul(mul(lam, ra), vn));
  const float2 lv = mul(mul(lam, vn), vn);
  const float2 b = mul(mul(K(0.5f * 0.56418958354775628f), ra), make_float2(__expf(-lv.x), __expf(-lv.y)));
  const float2 v1 = fma(vn, v0, make_float2(b.x, -b.y));
  float2 f[8];
  f[0] = mul(r, v1);
  f[1] = mul(mul(r, u), v1);
  f[2] = mul(mul(r, v), v1);
  f[3] = mul(mul(r, w), v1);
  f[4] = mul(fma(K(0.5f), pr, leng), v1);
  f[1 + D] = fma(pr, v0, f[1 + D]);
  f[4] = fma(mul(mul(K(0.5f), pr), vn), v0, f[4]);
  // magnetic stress, lam = rho / (2 p + B^2)
  float2 lb = mul(bx, bx);
  lb = fma(by, by, lb);
  lb = fma(bz, bz, lb);
  const float2 lm = mul(r, rcp(fma(K(2.0f), pr, lb)));
  const float2 m0 = half_erfc_lr(mul(mul(lm, rsq(lm)), vn));
  const float2 nm0 = mul(K(-1.0f), m0);
  const float2 hb = mul(K(0.5f), lb);
  f[5] = (D == 0) ? mul(sub(hb, mul(bx, bx)), m0) : mul(mul(bx, bn), nm0);
  f[6] = (D == 1) ? mul(sub(hb, mul(by, by)), m0) : mul(mul(by, bn), nm0);
  f[7] = (D == 2) ? mul(sub(hb, mul(bz, bz)), m0) : mul(mul(bz, bn), nm0);
#pragma unroll
  for (int q = 0; q < 8; ++q) out[q] = f[q].x + f[q].y;
}

// Fluxes and magnetic stress through one face normal to axis D from the
// reconstructed left (l) and right (r) states {rho, vx, vy, vz, p, bx, by, bz}
// (get_flux_stress, mhd3d3.f90:2385-2560): out = {rho, rvx, rvy, rvz, eng,
// s_x, s_y, s_z}.  Left state with the + moments, right with the - moments.
// FP32: on the packed pipe (face_flux_lr).
template <typename T, int D>
__device__ __forceinline__ void face_flux(const T* l, const T* r, T gam, T* out) {
  if constexpr (std::is_same<T, float>::value && MHD_FLUX_PACKED) {
    float2 X[8];
#pragma unroll
    for (int q = 0; q < 8; ++q) X[q] = make_float2(l[q], r[q]);
    face_flux_lr<D>(X, gam, out);
    return;
  }
  typedef Moments<T> M;
  const T gm1 = gam - T(1);
  {
    T rl = l[0], ul = l[1], vl = l[2], wl = l[3], pl = l[4], xl = l[5], yl = l[6], zl = l[7];
    T vn = l[1 + D];
    T bn = l[5 + D];
    T leng = T(0.5) * rl * (ul * ul + vl * vl + wl * wl) + Ops<T>::dv(pl, gm1);
    T lam = M::div(rl, T(2) * pl);
    T v0, v1;
    M::hydro(lam, vn, true, v0, v1);
    out[0] = rl * v1;
    out[1] = rl * ul * v1;
    out[2] = rl * vl * v1;
    out[3] = rl * wl * v1;
    out[4] = (leng + T(0.5) * pl) * v1;
    out[1 + D] = out[1 + D] + pl * v0;
    out[4] = out[4] + T(0.5) * pl * vn * v0;
    T lbsq = xl * xl + yl * yl + zl * zl;
    lam = M::div(rl, T(2) * pl + lbsq);
    v0 = M::mag(lam, vn, true);
    out[5] = ((D == 0) ? (T(0.5) * lbsq - xl * xl) : (-xl * bn)) * v0;
    out[6] = ((D == 1) ? (T(0.5) * lbsq - yl * yl) : (-yl * bn)) * v0;
    out[7] = ((D == 2) ? (T(0.5) * lbsq - zl * zl) : (-zl * bn)) * v0;
  }
  {
    T rr = r[0], ur = r[1], vr = r[2], wr = r[3], pr = r[4], xr = r[5], yr = r[6], zr = r[7];
    T vn = r[1 + D];
    T bn = r[5 + D];
    T leng = T(0.5) * rr * (ur * ur + vr * vr + wr * wr) + Ops<T>::dv(pr, gm1);
    T lam = M::div(rr, T(2) * pr);
    T v0, v1;
    M::hydro(lam, vn, false, v0, v1);
    T f[8];
    f[0] = rr * v1;
    f[1] = rr * ur * v1;
    f[2] = rr * vr * v1;
    f[3] = rr * wr * v1;
    f[4] = (leng + T(0.5) * pr) * v1;
    f[1 + D] = f[1 + D] + pr * v0;
    f[4] = f[4] + T(0.5) * pr * vn * v0;
    T lbsq = xr * xr + yr * yr + zr * zr;
    lam = M::div(rr, T(2) * pr + lbsq);
    v0 = M::mag(lam, vn, false);
    f[5] = ((D == 0) ? (T(0.5) * lbsq - xr * xr) : (-xr * bn)) * v0;
    f[6] = ((D == 1) ? (T(0.5) * lbsq - yr * yr) : (-yr * bn)) * v0;
    f[7] = ((D == 2) ? (T(0.5) * lbsq - zr * zr) : (-zr * bn)) * v0;
#pragma unroll
    for (int q = 0; q < 8; ++q) out[q] = out[q] + f[q];
  }
}

// Metric-mode flux through a face of unit normal n and area am: the
// Gaussian-split formulas of face_flux with n in place of the axis (vector
// momentum and magnetic stress), left with the + moments and right with the
// - moments, the sum multiplied by am (the oracle's get_flux_stress_metric).
template <typename T>
__device__ __forceinline__ void face_flux_n(const T* l, const T* r, T gam, const T* n, T am, T* out) {
  typedef Moments<T> Mo;
  const T gm1 = gam - T(1);
  T tot[8];
#pragma unroll
  for (int side = 0; side < 2; ++side) {
    const T* s = side ? r : l;
    const T rr = s[0], u0 = s[1], u1 = s[2], u2 = s[3], pr = s[4], b0 = s[5], b1 = s[6], b2 = s[7];
    const T vn = u0 * n[0] + u1 * n[1] + u2 * n[2];
    const T bn = b0 * n[0] + b1 * n[1] + b2 * n[2];
    const T leng = T(0.5) * rr * (u0 * u0 + u1 * u1 + u2 * u2) + Ops<T>::dv(pr, gm1);
    T lam = Mo::div(rr, T(2) * pr);
    T v0, v1;
    Mo::hydro(lam, vn, side == 0, v0, v1);
    T f[8];
    f[0] = rr * v1;
    f[1] = rr * u0 * v1 + pr * n[0] * v0;
    f[2] = rr * u1 * v1 + pr * n[1] * v0;
    f[3] = rr * u2 * v1 + pr * n[2] * v0;
    f[4] = (leng + T(0.5) * pr) * v1 + T(0.5) * pr * vn * v0;
    const T lbsq = b0 * b0 + b1 * b1 + b2 * b2;
    lam = Mo::div(rr, T(2) * pr + lbsq);
    v0 = Mo::mag(lam, vn, side == 0);
    f[5] = (T(0.5) * lbsq * n[0] - b0 * bn) * v0;
    f[6] = (T(0.5) * lbsq * n[1] - b1 * bn) * v0;
    f[7] = (T(0.5) * lbsq * n[2] - b2 * bn) * v0;
#pragma unroll
    for (int q = 0; q < 8; ++q) tot[q] = side ? tot[q] + f[q] : f[q];
  }
#pragma unroll
  for (int q = 0; q < 8; ++q) out[q] = tot[q] * am;
}

// Face flux of axis D at face c, Cartesian or metric.
template <typename T, int D, bool M>
__device__ __forceinline__ void any_face_flux(const Dev<T>& d, long long c, const T* L, const T* R, T* out) {
  if (M) {
    const T n[3] = {(T)d.m.nrm[D][0][c], (T)d.m.nrm[D][1][c], (T)d.m.nrm[D][2][c]};
    face_flux_n<T>(L, R, d.gam, n, (T)d.m.am[D][c], out);
  } else {
    face_flux<T, D>(L, R, d.gam, out);
  }
}

// One-sided states from an 8-tap register window (tap m = cell c+m-4 for the
// face at the low side of cell c): slot of tap m is (m + PH) & 7.
template <typename T, int RECON, int PH>
__device__ __forceinline__ void recon_win(const T* w, const Prm<T>& P, T& fl, T& fr) {
#define TAP(m) w[((m) + PH) & 7]
  if (RECON == R_PDM) {
    T fi = tap8(TAP(0), TAP(1), TAP(2), TAP(3), TAP(4), TAP(5), TAP(6), TAP(7));
    pdm2(TAP(2), TAP(3), TAP(4), TAP(5), fi, P.pdmb, fl, fr);
  } else if (RECON == R_TVD || RECON == R_TVDMC) {
    T fi = (TAP(3) + TAP(4)) / T(2);
    tvd<T, RECON == R_TVDMC>(TAP(2), TAP(3), TAP(4), TAP(5), fi, P.eps, fl, fr);
  } else {
    weno5(TAP(1), TAP(2), TAP(3), TAP(4), TAP(5), TAP(6), P.eps, fl, fr);
    if (RECON == R_MPWENO) {
      fl = mp_side(fl, TAP(1), TAP(2), TAP(3), TAP(4), TAP(5), P.alpha, P.beta);
      fr = mp_side(fr, TAP(6), TAP(5), TAP(4), TAP(3), TAP(2), P.alpha, P.beta);
    }
  }
#undef TAP
}

// One-sided states of the 8 cell fields src[0..7] at the low face of element
// c along stride s (recon_face per field); FP32 PDM on field pairs.
template <typename T, int RECON, typename I>
__device__ __forceinline__ void face_states(const T* const* src, I c, I s, const Prm<T>& P, T* L, T* R) {
  if constexpr (std::is_same<T, float>::value && RECON == R_PDM && MHD_RECON_PACKED) {
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      const float *fa = src[2 * q], *fb = src[2 * q + 1];
      float2 a[8];
#pragma unroll
      for (int m = 0; m < 8; ++m) a[m] = make_float2(fa[c + (m - 4) * s], fb[c + (m - 4) * s]);
      float2 lr0, lr1;
      pdm_pair_states(a, P.pdmb, lr0, lr1);
      L[2 * q] = lr0.x; R[2 * q] = lr0.y;
      L[2 * q + 1] = lr1.x; R[2 * q + 1] = lr1.y;
    }
  } else {
#pragma unroll
    for (int v = 0; v < 8; ++v) recon_face<T, RECON>(src[v], c, s, P, L[v], R[v]);
  }
}

// Face fluxes through the low face of cell c along axis D by direct (cached)
// loads; one face per thread.  Used for the x faces of every stage and, for
// all three axes, by the kernel-level debug entry point.
template <typename T, int RECON, int D, bool M, bool B>
__global__ void k_flux(KArg<T, B> ka, Inp<T> in0, Prm<T> P) {
  const int4 bb = ka.blk();
  const auto& d = ka.dev(bb);
  const Inp<T> in = B ? state_view(d) : in0;
  const Geom& g = d.g;
  const int ni = g.nx0 + (D == 0), nj = g.ny0 + (D == 1), nk = g.nz0 + (D == 2);
  const int t = bb.y * blockDim.x + threadIdx.x;
  if (t >= ni * nj * nk) return;
  const int i = t % ni + g.ng;
  const int r = t / ni;
  const int j = r % nj + g.ng;
  const int k = r / nj + g.ng;
  const int c = i + g.px * (j + g.py * k);
  const int s = (D == 0) ? 1 : (D == 1) ? g.px : (int)g.plane;
  const T* src[8] = {in.rho, in.vx, in.vy, in.vz, in.p, in.bx, in.by, in.bz};
  T L[8], R[8], out[8];
  face_states<T, RECON>(src, c, s, P, L, R);
  any_face_flux<T, D, M>(d, c, L, R, out);
#pragma unroll
  for (int q = 0; q < 8; ++q) d.F[D][q][c] = out[q];
}

// Stage combine of the RK steps (mhd3d3.f90:3674-3702, 3745-3788):
// form 0: (Xp+X)/den, 1: (c*Xp+X)/den, 2: (Xp+c*X)/den.
template <typename T>
__device__ __forceinline__ T comb(int form, T c, T xp, T x, T den) {
  if (form == 0) return Ops<T>::dv(xp + x, den);
  if (form == 1) return Ops<T>::dv(c * xp + x, den);
  return Ops<T>::dv(xp + c * x, den);
}

// One-sided states from a column of taps in shared memory: tap m (cell
// c+m-4 for the face at the low side of cell c) at col[m * RS].
template <typename T, int RECON, int RS>
__device__ __forceinline__ void recon_col(const T* col, const Prm<T>& P, T& fl, T& fr) {
  if (RECON == R_PDM) {
    T fi = tap8(col[0], col[RS], col[2 * RS], col[3 * RS], col[4 * RS], col[5 * RS], col[6 * RS], col[7 * RS]);
    pdm2(col[2 * RS], col[3 * RS], col[4 * RS], col[5 * RS], fi, P.pdmb, fl, fr);
  } else if (RECON == R_TVD || RECON == R_TVDMC) {
    T fi = (col[3 * RS] + col[4 * RS]) / T(2);
    tvd<T, RECON == R_TVDMC>(col[2 * RS], col[3 * RS], col[4 * RS], col[5 * RS], fi, P.eps, fl, fr);
  } else {
    T a1 = col[RS], a2 = col[2 * RS], a3 = col[3 * RS], a4 = col[4 * RS], a5 = col[5 * RS], a6 = col[6 * RS];
    weno5(a1, a2, a3, a4, a5, a6, P.eps, fl, fr);
    if (RECON == R_MPWENO) {
      fl = mp_side(fl, a1, a2, a3, a4, a5, P.alpha, P.beta);
      fr = mp_side(fr, a6, a5, a4, a3, a2, P.alpha, P.beta);
    }
  }
}

// y / z faces with the flux divergence fused through shared memory.  A block
// covers 32 cells along x and TD cells along the sweep axis D (1: y, 2: z) at
// one value of the remaining axis.  It stages the 8 reconstructed cell fields
// of TD+8 rows (4-cell halo each side) with independent coalesced loads, its
// TD+1 thread rows compute the TD+1 faces bounding those cells from shared
// memory, and the first TD rows combine the face pair of their cell:
//   D == 1: dU_q = (Fx_q(i+1)-Fx_q(i))/dx + (Fy_q(j+1)-Fy_q(j))/dy, the first
//     two terms of advance_corrector1/2 (mhd3d3.f90:3850-3906) in their order;
//   D == 2: the z term completes advance_corrector1 + stage combine + p +
//     advance_corrector2 + combine + v (RK: 3666-3697 / 3736-3783; AB:
//     3626-3627, 3876, 3901-3905), written to the other half of the
//     double-buffered primitives.
// Tuning knobs (compile time): cells per block along the sweep axis, whether
// the cell tile is staged in shared memory (1) or read through L1 (0), and
// the minimum resident blocks per SM requested from the register allocator.
#ifndef MHD_FLUX_TD
#define MHD_FLUX_TD 8
#endif
#ifndef MHD_FLUX_STAGED
#define MHD_FLUX_STAGED 0
#endif
#ifndef MHD_FLUX_MINB
#define MHD_FLUX_MINB 6
#endif
constexpr int TD = MHD_FLUX_TD;  // default tile length; FP32 PDM also has 4 and 16 (autotuner)
constexpr bool FLUX_STAGED = MHD_FLUX_STAGED != 0;

// Resident blocks per SM requested for the flux tiles: FP32 trades registers
// for occupancy (latency-bound); FP64 needs about twice the registers and
// would spill at the FP32 setting.
template <typename T> struct FluxMinB { static constexpr int value = MHD_FLUX_MINB; };
template <> struct FluxMinB<double> { static constexpr int value = 2; };

template <typename T, int TDV = TD>
__host__ __device__ constexpr size_t flux_t_smem() {
  // [+ staged cells] + face fluxes of the sweep + the x-face fluxes the y kernel reads (8 x TD x 33)
  return sizeof(T) * ((FLUX_STAGED ? 8 * (TDV + 8) * 32 : 0) + 8 * (TDV + 1) * 32 + 8 * TDV * 33);
}

// The conserved update of one cell from its z-face flux difference dF and the
// x+y divergence in dU (advance_corrector1 + stage combine + p +
// advance_corrector2 + combine + v, mhd3d3.f90:3666-3697 / 3736-3783; AB:
// 3626-3627, 3876, 3901-3905), written to the other half of the
// double-buffered primitives.  cd is the cell's z index.
// du: the x+y divergence dU of the cell; pv: its rho, vx, vy, vz, p; qv: its
// U^n (q[0..4], read only when form >= 0).
template <typename T, bool M>
__device__ __forceinline__ void cell_update_vals(const Dev<T>& d, int c, int cd, const T* dF, const T* du,
                                                 const T* pv, const T* qv, int form, T cw, T den) {
  const T tau = (T)d.sc->tau;
  const T gm1 = d.gam - T(1);
  T dv[8];
  if (M) {
    const T V = (T)d.m.vol[c], rV = (T)d.m.rvol[c];
#pragma unroll
    for (int q = 0; q < 8; ++q) dv[q] = Ops<T>::dw(du[q] + dF[q], V, rV);
  } else {
    const T dz = d.wz[cd], rdz = d.rwz[cd];
#pragma unroll
    for (int q = 0; q < 8; ++q) dv[q] = du[q] + Ops<T>::dw(dF[q], dz, rdz);
  }
  // get_conserve of the current state (AB: the state, not the prediction)
  T rr = pv[0], u = pv[1], v = pv[2], ww = pv[3], pr = pv[4];
  T rvx0 = rr * u, rvy0 = rr * v, rvz0 = rr * ww;
  T eng0 = T(0.5) * rr * (u * u + v * v + ww * ww) + Ops<T>::dv(pr, gm1);
  if (form == FORM_SAVE) {  // U^n of the step (this first stage's input), read by the later stages' combines
    d.q[0][c] = rr;
    d.q[1][c] = rvx0;
    d.q[2][c] = rvy0;
    d.q[3][c] = rvz0;
    d.q[4][c] = eng0;
  }
  T rho1 = rr - tau * dv[0];
  T eng1 = eng0 - tau * dv[4];
  T rx = rvx0 - tau * dv[1], ry = rvy0 - tau * dv[2], rz = rvz0 - tau * dv[3];
  T hx = rx, hy = ry, hz = rz;
  if (form >= 0) {
    rho1 = comb(form, cw, qv[0], rho1, den);
    hx = comb(form, cw, qv[1], rx, den);
    hy = comb(form, cw, qv[2], ry, den);
    hz = comb(form, cw, qv[3], rz, den);
    eng1 = comb(form, cw, qv[4], eng1, den);
  }
  const T rrho = Ops<T>::rcp(rho1);
  T pn = gm1 * (eng1 - Ops<T>::dvr(T(0.5) * (hx * hx + hy * hy + hz * hz), rho1, rrho));
  rx = rx - tau * dv[5];
  ry = ry - tau * dv[6];
  rz = rz - tau * dv[7];
  if (form >= 0) {
    rx = comb(form, cw, qv[1], rx, den);
    ry = comb(form, cw, qv[2], ry, den);
    rz = comb(form, cw, qv[3], rz, den);
  }
  d.orho[c] = rho1;
  d.op[c] = pn;
  d.ovx[c] = Ops<T>::dvr(rx, rho1, rrho);
  d.ovy[c] = Ops<T>::dvr(ry, rho1, rrho);
  d.ovz[c] = Ops<T>::dvr(rz, rho1, rrho);
}

template <typename T, bool M>
__device__ __forceinline__ void cell_update(const Dev<T>& d, int c, int cd, const T* dF, int form, T cw, T den) {
  T du[8], pv[5], qv[5];
#pragma unroll
  for (int q = 0; q < 8; ++q) du[q] = d.dU[q][c];
  pv[0] = d.rho[c]; pv[1] = d.vx[c]; pv[2] = d.vy[c]; pv[3] = d.vz[c]; pv[4] = d.p[c];
#pragma unroll
  for (int q = 0; q < 5; ++q) qv[q] = (form >= 0) ? d.q[q][c] : T(0);
  cell_update_vals<T, M>(d, c, cd, dF, du, pv, qv, form, cw, den);
}

template <typename T, int RECON, int D, bool M, bool B, int TDV = TD>
__global__ void __launch_bounds__(32 * (TDV + 1), FluxMinB<T>::value)
    k_flux_t(KArg<T, B> ka, Inp<T> in0, Prm<T> P, int form, T cw, T den, int ab) {
  constexpr int TD = TDV;
  constexpr int TROWS = TDV + 8;
  const int4 bb = ka.blk();
  const auto& d = ka.dev(bb);
  const Inp<T> in = B ? state_view(d) : in0;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  T* sv = reinterpret_cast<T*>(smem_raw);                      // [8][TROWS][32] cell fields
  T* sF = sv + (FLUX_STAGED ? 8 * TROWS * 32 : 0);             // [8][TD+1][32] face fluxes
  T* sX = sF + 8 * (TD + 1) * 32;                              // [8][TD][33] x-face fluxes (D == 1)
  const Geom& g = d.g;
  const int tx = threadIdx.x, r = threadIdx.y;
  const int i0 = bb.y * 32 + g.ng;
  const int i = i0 + tx;
  const int n0 = (D == 1) ? g.ny0 : g.nz0;
  const int nD = (D == 1) ? g.ny : g.nz;
  const int cd0 = bb.z * TD + g.ng;  // first cell of the tile along D
  const int o = bb.w + g.ng;         // remaining transverse index
  const int s = (D == 1) ? g.px : (int)g.plane;
  const int rowbase = (D == 1) ? i0 + g.px * g.py * o : i0 + g.px * o;  // + cd * s
  const T* src[8] = {in.rho, in.vx, in.vy, in.vz, in.p, in.bx, in.by, in.bz};
  if (D == 1) {
    // The x-face fluxes of the tile's cells (faces i0 .. i0+32 of rows cd0 ..
    // cd0+TD-1) are only needed in the epilogue: copy them asynchronously now
    // so their latency hides behind the reconstructions.
    const int nthr = 32 * (TD + 1);
#pragma unroll
    for (int q = 0; q < 8; ++q) {  // static q: the flux pointers stay in registers
      const T* fq = d.F[0][q];
      for (int t = r * 32 + tx; t < TD * 33; t += nthr) {
        const int rr = t / 33, col = t - rr * 33;
        if (cd0 + rr < g.ng + n0 && i0 + col <= g.ng + g.nx0) {
          const T* gp = fq + rowbase + col + (cd0 + rr) * s;
          const uint32_t sp = (uint32_t)__cvta_generic_to_shared(sX + q * TD * 33 + t);
          if (sizeof(T) == 4)
            asm volatile("cp.async.ca.shared.global [%0], [%1], 4;" ::"r"(sp), "l"(gp) : "memory");
          else
            asm volatile("cp.async.ca.shared.global [%0], [%1], 8;" ::"r"(sp), "l"(gp) : "memory");
        }
      }
    }
    asm volatile("cp.async.commit_group;" ::: "memory");
  }
  if (FLUX_STAGED) {
    const int nthr = 32 * (TD + 1);
    const bool xok = i0 + tx < g.nx;
#pragma unroll
    for (int v = 0; v < 8; ++v) {
      const T* sp = src[v] + rowbase + tx;
      for (int t = r * 32 + tx; t < TROWS * 32; t += nthr) {
        const int cd = cd0 - 4 + (t >> 5);
        sv[v * TROWS * 32 + t] = (xok && cd < nD) ? sp[cd * s] : T(0);
      }
    }
    __syncthreads();
  }
  const int cd = cd0 + r;  // cell whose low face this thread computes
  const bool xin = i < g.ng + g.nx0;
  if (xin && cd <= g.ng + n0) {
    T L[8], R[8], F[8];
    if (FLUX_STAGED) {
#pragma unroll
      for (int v = 0; v < 8; ++v) recon_col<T, RECON, 32>(sv + (v * TROWS + r) * 32 + tx, P, L[v], R[v]);
    } else {
      const int cf = rowbase + tx + cd * s;
      face_states<T, RECON>(src, cf, s, P, L, R);
    }
    any_face_flux<T, D, M>(d, rowbase + tx + cd * s, L, R, F);
#pragma unroll
    for (int q = 0; q < 8; ++q) sF[(q * (TD + 1) + r) * 32 + tx] = F[q];
  }
  if (D == 1) asm volatile("cp.async.wait_all;" ::: "memory");
  __syncthreads();
  if (r >= TD || !xin || cd >= g.ng + n0) return;
  const int c = rowbase + tx + cd * s;
  T dF[8];
#pragma unroll
  for (int q = 0; q < 8; ++q) dF[q] = sF[(q * (TD + 1) + r + 1) * 32 + tx] - sF[(q * (TD + 1) + r) * 32 + tx];
  if (D == 1) {
    if (M) {  // area-weighted fluxes: the sum is divided by V after the z term
#pragma unroll
      for (int q = 0; q < 8; ++q) {
        const T* x = sX + (q * TD + r) * 33 + tx;
        d.dU[q][c] = (x[1] - x[0]) + dF[q];
      }
      return;
    }
    const T dx = d.wx[i], dy = d.wy[cd], rdx = d.rwx[i], rdy = d.rwy[cd];
#pragma unroll
    for (int q = 0; q < 8; ++q) {
      const T* x = sX + (q * TD + r) * 33 + tx;
      d.dU[q][c] = Ops<T>::dw(x[1] - x[0], dx, rdx) + Ops<T>::dw(dF[q], dy, rdy);
    }
    return;
  }
  cell_update<T, M>(d, c, cd, dF, form, cw, den);
  (void)ab;
}

// y / z faces by column sweeps: the FP32 Cartesian PDM alternative to the face
// tiles, one more launch shape for the autotuner.  A thread owns one column of
// cells along D (x from the lane, the remaining axis from the warp) over a
// segment of SWEEP_SEG cells and keeps the 8 reconstructed fields of the 8
// cells around its current face in registers: one new cell is loaded per face
// (issued a face ahead, before that face's arithmetic), every face flux is
// computed once, and a cell's face-pair difference is the current minus the
// previous face's flux.  Face arithmetic and epilogues are those of k_flux_t,
// so the two give the same bits.
#ifndef MHD_SWEEP_SEG
#define MHD_SWEEP_SEG 32
#endif
constexpr int SWEEP_SEG = MHD_SWEEP_SEG;  // cells per column segment (compile-time knob)
#ifndef MHD_SWEEP_UNROLL
#define MHD_SWEEP_UNROLL 1
#endif
constexpr int kSweepUnroll = MHD_SWEEP_UNROLL;  // face-loop unroll (compile-time knob)
#ifndef MHD_SWEEP_MINB
#define MHD_SWEEP_MINB 4
#endif
constexpr int kSweepMinB = MHD_SWEEP_MINB;  // resident 128-thread blocks per SM (register budget)

template <typename T, int D, bool B, int RECON = R_PDM>
__global__ void __launch_bounds__(128, kSweepMinB)
    k_flux_sweep(KArg<T, B> ka, Inp<T> in0, Prm<T> P, int form, T cw, T den) {
  const int4 bb = ka.blk();
  const auto& d = ka.dev(bb);
  const Inp<T> in = B ? state_view(d) : in0;
  const Geom& g = d.g;
  const int n0 = (D == 1) ? g.ny0 : g.nz0;
  const int no = (D == 1) ? g.nz0 : g.ny0;
  const int o = bb.w * 4 + threadIdx.y + g.ng;  // remaining axis (one per warp): z for y faces, y for z faces
  if (o >= g.ng + no) return;
  const int tx = threadIdx.x;
  // lanes past the last column work on a copy of it and store nothing, so the
  // whole warp stays in the loop (warp-synchronous copies below)
  const int i0 = bb.y * 32 + tx + g.ng;
  const bool xin = i0 < g.ng + g.nx0;
  const int i = xin ? i0 : g.ng + g.nx0 - 1;
  const int c0 = g.ng + bb.z * SWEEP_SEG;
  const int c1 = min(c0 + SWEEP_SEG, g.ng + n0);
  const int s = (D == 1) ? g.px : (int)g.plane;
  const int col = (D == 1) ? i + (int)g.plane * o : i + g.px * o;  // + cd * s
  const T* src[8] = {in.rho, in.vx, in.vy, in.vz, in.p, in.bx, in.by, in.bz};
  // y faces: the x-face fluxes of the next cell are copied asynchronously into
  // a per-warp double buffer one face ahead of the epilogue that reads them
  __shared__ __align__(16) T sxf[4][2][8][33];
  T (*xs)[8][33] = sxf[threadIdx.y];
  // z faces: dU, the state (rho, v, p) and U^n of the next cell, likewise
  // (each lane reads back only what it copied)
  __shared__ __align__(16) T szf[4][2][18][32];
  T (*zs)[18][32] = szf[threadIdx.y];
  // the window holds the 8 fields as pairs (rho, vx), (vy, vz), (p, bx),
  // (by, bz), the operands of the packed FP32 reconstruction
  typedef typename Pr<T>::V V2;
  V2 w[4][8], nx[4];
  T Fp[8];
  // window of the first face (cell c0): cells c0-4 .. c0+3; the loop shifts
  // one cell in per face, so w[q][1..7] start as cells c0-4 .. c0+2.  Window
  // cells are clamped to the ghost-inclusive range [0, nD-1]: with fewer than
  // 4 ghost layers (nord 4 or 6: TVD, WENO) the outermost taps lie outside
  // it, and those taps are exactly the ones such a stencil never reads.
  const int nD = (D == 1) ? g.ny : g.nz;
#pragma unroll
  for (int q = 0; q < 4; ++q) {
#pragma unroll
    for (int m = 1; m < 8; ++m) {
      const int x = col + max(c0 - 5 + m, 0) * s;
      w[q][m] = Pr<T>::mk(src[2 * q][x], src[2 * q + 1][x]);
    }
    const int x = col + min(c0 + 3, nD - 1) * s;
    nx[q] = Pr<T>::mk(src[2 * q][x], src[2 * q + 1][x]);
  }
  T dx = T(0), rdx = T(0);
  if (D == 1) {
    dx = d.wx[i];
    rdx = d.rwx[i];
  }
#pragma unroll kSweepUnroll
  for (int cd = c0; cd <= c1; ++cd) {  // the face at the low side of cell cd
#pragma unroll
    for (int q = 0; q < 4; ++q) {
#pragma unroll
      for (int m = 0; m < 7; ++m) w[q][m] = w[q][m + 1];
      w[q][7] = nx[q];
    }
    if (cd < c1) {
      const int x = col + min(cd + 4, nD - 1) * s;
#pragma unroll
      for (int q = 0; q < 4; ++q) nx[q] = Pr<T>::mk(src[2 * q][x], src[2 * q + 1][x]);
    }
    if (D == 1) {
      __syncwarp();  // every lane is done reading the slot refilled here
      if (cd < c1) {
        // x faces i0 (this lane) and, on lane 31, i0 + 32, clamped to the last
        // face (a lane past the last column supplies its left neighbour's high face)
        const int fo = ((D == 1) ? (int)g.plane * o : g.px * o) + cd * s;
        const int fl = fo + min(i0, g.ng + g.nx0), fh = fo + min(i0 + 1, g.ng + g.nx0);
#pragma unroll
        for (int q = 0; q < 8; ++q) {
          const T* fx = d.F[0][q] + fl;
          const uint32_t sp = (uint32_t)__cvta_generic_to_shared(&xs[cd & 1][q][tx]);
          if (sizeof(T) == 4)
            asm volatile("cp.async.ca.shared.global [%0], [%1], 4;" ::"r"(sp), "l"(fx) : "memory");
          else
            asm volatile("cp.async.ca.shared.global [%0], [%1], 8;" ::"r"(sp), "l"(fx) : "memory");
          if (tx == 31) {
            const uint32_t sq = (uint32_t)__cvta_generic_to_shared(&xs[cd & 1][q][32]);
            const T* fy = d.F[0][q] + fh;
            if (sizeof(T) == 4)
              asm volatile("cp.async.ca.shared.global [%0], [%1], 4;" ::"r"(sq), "l"(fy) : "memory");
            else
              asm volatile("cp.async.ca.shared.global [%0], [%1], 8;" ::"r"(sq), "l"(fy) : "memory");
          }
        }
      }
      asm volatile("cp.async.commit_group;" ::: "memory");  // one group per face, empty on the last
    } else {
      if (cd < c1) {
        const int c = col + cd * s;
        const T* gsrc[18] = {d.dU[0] + c, d.dU[1] + c, d.dU[2] + c, d.dU[3] + c, d.dU[4] + c, d.dU[5] + c,
                             d.dU[6] + c, d.dU[7] + c, d.rho + c,   d.vx + c,    d.vy + c,    d.vz + c,
                             d.p + c,     d.q[0] + c, d.q[1] + c, d.q[2] + c, d.q[3] + c, d.q[4] + c};
        const int nz = (form >= 0) ? 18 : 13;
#pragma unroll
        for (int a = 0; a < 18; ++a) {
          if (a < nz) {
            const uint32_t sp = (uint32_t)__cvta_generic_to_shared(&zs[cd & 1][a][tx]);
            if (sizeof(T) == 4)
              asm volatile("cp.async.ca.shared.global [%0], [%1], 4;" ::"r"(sp), "l"(gsrc[a]) : "memory");
            else
              asm volatile("cp.async.ca.shared.global [%0], [%1], 8;" ::"r"(sp), "l"(gsrc[a]) : "memory");
          }
        }
      }
      asm volatile("cp.async.commit_group;" ::: "memory");
    }
    T L[8], R[8], F[8];
    if constexpr (std::is_same<T, float>::value && RECON == R_PDM && MHD_RECON_PACKED) {
#pragma unroll
      for (int q = 0; q < 4; ++q) {
        float2 lr0, lr1;
        pdm_pair_states(w[q], P.pdmb, lr0, lr1);
        L[2 * q] = lr0.x; R[2 * q] = lr0.y;
        L[2 * q + 1] = lr1.x; R[2 * q + 1] = lr1.y;
      }
    } else {
#pragma unroll
      for (int v = 0; v < 8; ++v) {
        T wv[8];
#pragma unroll
        for (int m = 0; m < 8; ++m) wv[m] = (v & 1) ? w[v >> 1][m].y : w[v >> 1][m].x;
        recon_win<T, RECON, 0>(wv, P, L[v], R[v]);
      }
    }
    face_flux<T, D>(L, R, d.gam, F);
    if (cd > c0) {
      const int cc = cd - 1;
      const int c = col + cc * s;
      T dF[8];
#pragma unroll
      for (int q = 0; q < 8; ++q) dF[q] = F[q] - Fp[q];
      if (D == 1) {
        asm volatile("cp.async.wait_group 1;" ::: "memory");  // the group of cell cc (one face old)
        __syncwarp();
        const T dy = d.wy[cc], rdy = d.rwy[cc];
        if (xin) {
#pragma unroll
          for (int q = 0; q < 8; ++q) {
            const T* x = &xs[cc & 1][q][tx];
            d.dU[q][c] = Ops<T>::dw(x[1] - x[0], dx, rdx) + Ops<T>::dw(dF[q], dy, rdy);
          }
        }
      } else {
        asm volatile("cp.async.wait_group 1;" ::: "memory");  // this lane's copies of cell cc
        if (xin) {
          const T* zv = &zs[cc & 1][0][tx];
          T du[8], pv[5], qv[5];
#pragma unroll
          for (int q = 0; q < 8; ++q) du[q] = zv[q * 32];
#pragma unroll
          for (int q = 0; q < 5; ++q) pv[q] = zv[(8 + q) * 32];
#pragma unroll
          for (int q = 0; q < 5; ++q) qv[q] = (form >= 0) ? zv[(13 + q) * 32] : T(0);
          cell_update_vals<T, false>(d, c, cc, dF, du, pv, qv, form, cw, den);
        }
      }
    }
#pragma unroll
    for (int q = 0; q < 8; ++q) Fp[q] = F[q];
  }
  asm volatile("cp.async.wait_all;" ::: "memory");
}

// -------------------------------------------------------------------- EMF
// Edge EMF of family E (0: ei along x, 1: ej along y, 2: ek along z) at the
// edge whose upper cell is c (get_eijk_LFM, 1754-1856).  a1 = E+1, a2 = E+2
// (cyclic): v1 = v_a1, v2 = v_a2; b1 = B_a1 reconstructed along a2 and
// upwinded by sign(v2); b2 = B_a2 reconstructed along a1, upwinded by sign(v1).
// E of an edge from its corner velocities, the one-sided face states of b1
// and b2 and eta = 0.25 (vf[c-s1-s2] + vf[c-s2] + vf[c] + vf[c-s1]): the
// upwinded convective term plus the resistive term (metric: g_e and |dl_e|).
template <typename T>
__device__ __forceinline__ T eta4(T a, T b, T c, T e) {
  return T(0.25) * (a + b + c + e);
}
template <typename T, int E, bool M, typename I>
__device__ __forceinline__ T emf_value(const Dev<T>& d, I c, T v1av, T v2av, T b1l, T b1r, T b2l, T b2r, T eta) {
  const T b1u = (v2av >= T(0)) ? b1l : b1r;
  const T b2u = (v1av >= T(0)) ? b2l : b2r;
  const T e = -v1av * b2u + v2av * b1u;
  if (M)  // E.dl: g_e * (convective term) + eta |dl_e| * (resistive term)
    return (T)d.m.ge[E][c] * e + eta * (T)d.m.dl[E][c] * (b1l + b2r - b1r - b2l);
  return e + eta * (b1l + b2r - b1r - b2l);
}

// One edge of family E from global memory (upper cell index c).
template <typename T, int RECON, int E, bool M>
__device__ __forceinline__ void emf_edge(const Dev<T>& d, const Inp<T>& in, const Prm<T>& P, long long c) {
  const long long st[3] = {1, (long long)d.g.px, d.g.plane};
  constexpr int A1 = (E + 1) % 3, A2 = (E + 2) % 3;
  const long long s1 = st[A1], s2 = st[A2];
  const T* vel[3] = {in.vx, in.vy, in.vz};
  const T* fb[3] = {in.bi, in.bj, in.bk};
  const T v1av = corner_vel<T, RECON>(vel[A1], c, s1, s2, P);
  const T v2av = corner_vel<T, RECON>(vel[A2], c, s1, s2, P);
  T b1l, b1r, b2l, b2r;
  recon_face<T, RECON>(fb[A1], c, s2, P, b1l, b1r);
  recon_face<T, RECON>(fb[A2], c, s1, P, b2l, b2r);
  const T* vf = d.vf;
  const T eta = eta4(vf[c - s1 - s2], vf[c - s2], vf[c], vf[c - s1]);
  d.E[E][c] = emf_value<T, E, M>(d, c, v1av, v2av, b1l, b1r, b2l, b2r, eta);
}

template <typename T, int RECON, int E, bool M>
__global__ void k_emf(Dev<T> d, Inp<T> in, Prm<T> P) {
  const Geom& g = d.g;
  int i = blockIdx.x * blockDim.x + threadIdx.x + g.ng;
  int j = blockIdx.y * blockDim.y + threadIdx.y + g.ng;
  int k = blockIdx.z + g.ng;
  int ni = g.nx0 + (E != 0), nj = g.ny0 + (E != 1), nk = g.nz0 + (E != 2);
  if (i >= g.ng + ni || j >= g.ng + nj || k >= g.ng + nk) return;
  emf_edge<T, RECON, E, M>(d, in, P, idx3<T>(g, i, j, k));
}

// Shared-memory tiled EMF of family E for PDM (the default deck's
// reconstruction).  A block stages v_a1 and v_a2 of its tile of edges plus a
// 4-cell halo in the transverse (a1, a2) plane, computes the first pass of
// interp2_pdm (8-tap along a1, mhd3d3.f90:926-989) once per (a1 face, a2 row)
// into shared memory, and each edge then takes the second pass along a2, the
// limiters (corner_pdm), the upwinded face-B reconstructions and the Alfven
// resistivity term exactly as k_emf does.  Tile (TX, TY, TZ) in edges.
//
// A transverse axis of an edge family holds n0 + 1 edges.  For ej and ek,
// when that count is one more than a multiple of the tile (n0 a multiple of
// 32 along x, of 8 along the other transverse axis), the last tile of the
// axis is one edge wider instead of a block of its own holding a single edge
// row: emf_edge_tiles() counts the tiles, and k_emf_pdm runs the widened
// variant of emf_pdm_tile in those blocks.  ei keeps the plain count (its
// halo-padded tile is large, so a wider variant would cost shared memory and
// occupancy in every block).
// Depth of the ej / ek plane tiles along their second transverse axis
// (32 x kPT edges, 32 kPT threads); compile-time knob.
#ifndef MHD_EMF_PLANE
#define MHD_EMF_PLANE 8
#endif
constexpr int kPT = MHD_EMF_PLANE;
constexpr bool emf_merges(int E, int axis) { return E != 0 && axis != E; }

__host__ __device__ constexpr int emf_edge_tiles(int ext, int t, bool merge) {
  return (merge && t > 1 && ext > t && ext % t == 1) ? ext / t : (ext + t - 1) / t;
}

// dynamic shared memory of k_emf_pdm: enough for the widest tile it runs
template <typename T, int E, int TX, int TY, int TZ>
constexpr size_t emf_pdm_smem() {
  constexpr int WX = TX + emf_merges(E, 0), WY = TY + emf_merges(E, 1), WZ = TZ + emf_merges(E, 2);
  constexpr int A1 = (E + 1) % 3, A2 = (E + 2) % 3;
  constexpr int HX = (E == 0) ? 0 : 4, HY = (E == 1) ? 0 : 4, HZ = (E == 2) ? 0 : 4;
  constexpr int NV = (WX + 2 * HX) * (WY + 2 * HY) * (WZ + 2 * HZ);
  constexpr int TE = (E == 0) ? WX : (E == 1) ? WY : WZ;
  constexpr int T1 = (A1 == 0) ? WX : (A1 == 1) ? WY : WZ;
  constexpr int T2 = (A2 == 0) ? WX : (A2 == 1) ? WY : WZ;
  return sizeof(T) * (2 * NV + 2 * TE * T1 * (T2 + 8));
}

inline dim3 emf_grid(int E, const Geom& g, int tx, int ty, int tz) {
  const int ex = g.nx0 + (E != 0), ey = g.ny0 + (E != 1), ez = g.nz0 + (E != 2);
  return dim3(emf_edge_tiles(ex, tx, emf_merges(E, 0)), emf_edge_tiles(ey, ty, emf_merges(E, 1)),
              emf_edge_tiles(ez, tz, emf_merges(E, 2)));
}

template <typename T, int E, int TX, int TY, int TZ, bool M>
__device__ __forceinline__ void emf_pdm_tile(const Dev<T>& d, const Inp<T>& in, const Prm<T>& P, int ox, int oy,
                                             int oz) {
  constexpr int A1 = (E + 1) % 3, A2 = (E + 2) % 3;
  constexpr int HX = (E == 0) ? 0 : 4, HY = (E == 1) ? 0 : 4, HZ = (E == 2) ? 0 : 4;
  constexpr int SX = TX + 2 * HX, SY = TY + 2 * HY, SZ = TZ + 2 * HZ;
  constexpr int NV = SX * SY * SZ;
  constexpr int SE = (E == 0) ? 1 : (E == 1) ? SX : SX * SY;
  constexpr int S1 = (A1 == 0) ? 1 : (A1 == 1) ? SX : SX * SY;
  constexpr int S2 = (A2 == 0) ? 1 : (A2 == 1) ? SX : SX * SY;
  constexpr int TE = (E == 0) ? TX : (E == 1) ? TY : TZ;
  constexpr int T1 = (A1 == 0) ? TX : (A1 == 1) ? TY : TZ;
  constexpr int T2 = (A2 == 0) ? TX : (A2 == 1) ? TY : TZ;
  constexpr int NG = TE * T1 * (T2 + 8);
  // first-pass layout with the x-mapped index contiguous (conflict-free banks)
  constexpr int R2 = T2 + 8;
  constexpr int GE = (E == 0) ? 1 : (A1 == 0) ? T1 : R2;
  constexpr int G1 = (E == 0) ? TE : (A1 == 0) ? 1 : R2 * TE;
  constexpr int G2 = (E == 0) ? TE * T1 : (A1 == 0) ? T1 * TE : 1;
  typedef Pr<T> Q;
  typedef typename Q::V V;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  V* sv = reinterpret_cast<V*>(smem_raw);  // [NV] (v_a1, v_a2) pairs
  V* sg = sv + NV;                         // [NG] first-pass interpolant pairs
  const Geom& g = d.g;
  const T* vel[3] = {in.vx, in.vy, in.vz};
  const T* v1 = vel[A1];
  const T* v2 = vel[A2];
  // stage v_a1, v_a2: one flat pass over the (x, y, z) tile, x fastest, so
  // every lane has an element even when a row is not a multiple of 32 wide
  for (int t = threadIdx.x; t < NV; t += blockDim.x) {
    const int lx = t % SX, row = t / SX;
    const int ly = row % SY, lz = row / SY;
    const int gx = ox - HX + lx, gy = oy - HY + ly, gz = oz - HZ + lz;
    T a = T(0), b = T(0);
    if (gx < g.nx && gy < g.ny && gz < g.nz) {
      const int gi = gx + g.px * (gy + g.py * gz);
      a = v1[gi];
      b = v2[gi];
    }
    sv[t] = Q::mk(a, b);
  }
  __syncthreads();
  // first pass of interp2_pdm over (e, f1, r2), flat with the x-mapped index fastest
  constexpr int NX = (E == 0) ? TE : (A1 == 0) ? T1 : R2;   // x-mapped extent
  for (int t = threadIdx.x; t < NG; t += blockDim.x) {
    const int ix = t % NX, row = t / NX;
    int e, f1, r2;
    if (E == 0) {
      e = ix; f1 = row % T1; r2 = row / T1;
    } else if (A1 == 0) {
      f1 = ix; e = row % TE; r2 = row / TE;
    } else {
      r2 = ix; e = row % TE; f1 = row / TE;
    }
    const int b0 = e * SE + f1 * S1 + r2 * S2;
    const int gi = e * GE + f1 * G1 + r2 * G2;
    const V* a = sv + b0;
    sg[gi] = tap8p<T>(a[0], a[S1], a[2 * S1], a[3 * S1], a[4 * S1], a[5 * S1], a[6 * S1], a[7 * S1]);
  }
  __syncthreads();
  const int n0[3] = {g.nx0, g.ny0, g.nz0};
  const int lim[3] = {g.ng + n0[0] + (E != 0), g.ng + n0[1] + (E != 1), g.ng + n0[2] + (E != 2)};
  const int st[3] = {1, g.px, (int)g.plane};
  const T* fb[3] = {in.bi, in.bj, in.bk};
  for (int t = threadIdx.x; t < TX * TY * TZ; t += blockDim.x) {
    const int lx = t % TX, r = t / TX, ly = r % TY, lz = r / TY;
    const int gx = ox + lx, gy = oy + ly, gz = oz + lz;
    if (gx >= lim[0] || gy >= lim[1] || gz >= lim[2]) continue;
    const int e = (E == 0) ? lx : (E == 1) ? ly : lz;
    const int f1 = (A1 == 0) ? lx : (A1 == 1) ? ly : lz;
    const int f2 = (A2 == 0) ? lx : (A2 == 1) ? ly : lz;
    const int cv = e * SE + (f1 + 4) * S1 + (f2 + 4) * S2;
    const V* gg = sg + e * GE + f1 * G1 + f2 * G2;
    constexpr int GS = G2;
    const V vi = tap8p<T>(gg[0], gg[GS], gg[2 * GS], gg[3 * GS], gg[4 * GS], gg[5 * GS], gg[6 * GS], gg[7 * GS]);
    T v1av, v2av;
    corner_pdm_pair<T>(sv, cv, S1, S2, vi, P.pdmb, v1av, v2av);
    const int c = gx + g.px * (gy + g.py * gz);
    const int s1 = st[A1], s2 = st[A2];
    T b1l, b1r, b2l, b2r;
    recon_face<T, R_PDM>(fb[A1], c, s2, P, b1l, b1r);
    recon_face<T, R_PDM>(fb[A2], c, s1, P, b2l, b2r);
    const T* vf = d.vf;
    const T eta = eta4(vf[c - s1 - s2], vf[c - s2], vf[c], vf[c - s1]);
    d.E[E][c] = emf_value<T, E, M>(d, c, v1av, v2av, b1l, b1r, b2l, b2r, eta);
  }
}

// Register budgets of the EMF tiles (resident threads per SM the allocator
// must allow): single grid 2048 (full occupancy); batched 1536 for the plane
// tiles and 1024 for ei, whose shared memory allows 2 blocks anyway (the
// batched kernels carry a grid-table lookup and spill at 32 registers).
// MHD_EMF_FULL_OCC=0 leaves every budget to the compiler.
#ifndef MHD_EMF_FULL_OCC
#define MHD_EMF_FULL_OCC 1
#endif
constexpr int emf_min_blocks(int E, int NT, bool B) {
  return !MHD_EMF_FULL_OCC ? 1 : !B ? 2048 / NT : (E == 0 ? 1024 / NT : 1536 / NT);
}
template <typename T, int E, int TX, int TY, int TZ, int NT, bool M, bool B>
__global__ void __launch_bounds__(NT, emf_min_blocks(E, NT, B))
    k_emf_pdm(KArg<T, B> ka, Inp<T> in0, Prm<T> P) {
  const int4 bb = ka.blk();
  const auto& d = ka.dev(bb);
  const Inp<T> in = B ? state_view(d) : in0;
  const Geom& g = d.g;
  const int ox = g.ng + bb.y * TX, oy = g.ng + bb.z * TY, oz = g.ng + bb.w * TZ;
  if constexpr (E == 0) {
    emf_pdm_tile<T, E, TX, TY, TZ, M>(d, in, P, ox, oy, oz);
  } else {
    // transverse axes a1, a2: is this block the widened last tile of the axis?
    constexpr int A1 = (E + 1) % 3, A2 = (E + 2) % 3;
    const int n0[3] = {g.nx0, g.ny0, g.nz0};
    const int org[3] = {ox - g.ng, oy - g.ng, oz - g.ng};
    constexpr int tl[3] = {TX, TY, TZ};
    const bool w1 = tl[A1] > 1 && n0[A1] - org[A1] == tl[A1];
    const bool w2 = tl[A2] > 1 && n0[A2] - org[A2] == tl[A2];
    constexpr int X1 = A1 == 0, Y1 = A1 == 1, Z1 = A1 == 2, X2 = A2 == 0, Y2 = A2 == 1, Z2 = A2 == 2;
    if (w1 && w2)
      emf_pdm_tile<T, E, TX + X1 + X2, TY + Y1 + Y2, TZ + Z1 + Z2, M>(d, in, P, ox, oy, oz);
    else if (w1)
      emf_pdm_tile<T, E, TX + X1, TY + Y1, TZ + Z1, M>(d, in, P, ox, oy, oz);
    else if (w2)
      emf_pdm_tile<T, E, TX + X2, TY + Y2, TZ + Z2, M>(d, in, P, ox, oy, oz);
    else
      emf_pdm_tile<T, E, TX, TY, TZ, M>(d, in, P, ox, oy, oz);
  }
}

template <typename T, int E, int TX, int TY, int TZ, int NT, bool M>
void launch_emf_pdm(const Dev<T>& d, const Inp<T>& in, const Prm<T>& P, cudaStream_t st) {
  constexpr size_t bytes = emf_pdm_smem<T, E, TX, TY, TZ>();
  static PerDevice attr;
  unsigned long long bit = 0;
  if (attr.need(bit)) {
    cudaFuncSetAttribute(k_emf_pdm<T, E, TX, TY, TZ, NT, M, false>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                         (int)bytes);
    attr.mark(bit);
  }
  k_emf_pdm<T, E, TX, TY, TZ, NT, M, false><<<emf_grid(E, d.g, TX, TY, TZ), NT, bytes, st>>>(one(d), in, P);
}

// ------------------------------------------------------ streamed PDM EMF
// The PDM EMF of one family as slice streams.  A block owns a patch of edges
// across the stream axis S (32 lanes along x times NW warps) and walks S over
// a segment of edge positions.  Each step copies one new cell slice of
// (v_a1, v_a2), of the face-B component that is reconstructed across the
// slice and of vf into shared-memory rings, asynchronously and a step ahead,
// and each thread computes the edge of its column at the current position:
// every cell is staged once per segment (no halo re-reads along S, no
// per-tap index arithmetic), and the taps along S come from a register window
// or the ring.
//   ei (E = 0): lanes along x (the edge axis), warps along y = a1, S = z = a2.
//   ek (E = 2): lanes along x = a1, warps along z (the edge axis), S = y = a2.
//   ej (E = 1): lanes along x = a2, warps along y (the edge axis), S = z = a1.
// With S = a2 the first pass of interp2_pdm (8 taps along a1) runs inside
// the new slice and the second pass (along S) on a register window of eight
// first-pass values; with S = a1 the first pass runs across eight ring slices
// into a per-warp row (32 columns plus the 8-column halo) and the second pass
// along x reads that row.  The face-B component reconstructed along S is a
// register window of eight values of the thread's own column.  The
// arithmetic per edge is emf_pdm_tile's and k_emf's (same operands, same
// order), so all three give the same bits.  The in-slice transverse axis
// holds n0 + 1 edges; the tiles cover the first n0 and k_emf_rows the last.
template <typename T, int E, int NW>
struct EmfStream {
  static constexpr bool SA2 = (E != 1);             // S = a2 (ei, ek) or S = a1 (ej)
  static constexpr int NT = 32 * NW;
  static constexpr int C = (E == 0) ? 32 : 40;      // slice columns (x), with the x halo for ek / ej
  static constexpr int R = (E == 0) ? NW + 8 : NW;  // slice rows, with the y halo for ei
  static constexpr int NS = R * C;                  // cells per slice
  static constexpr int NE = (NS + NT - 1) / NT;     // slice cells each thread copies
  static constexpr int TS = (E == 0) ? C : 1;       // in-slice stride of the transverse axis
  static constexpr int DV = SA2 ? 8 : 16;           // (v_a1, v_a2) ring depth
  static constexpr size_t smem =
      sizeof(typename Pr<T>::V) * (DV * NS + (SA2 ? 0 : NW * C)) + sizeof(T) * (2 * NS + 4 * NS);
};

template <typename T>
__device__ __forceinline__ void cp_async_zfill(uint32_t dst, const T* src, bool ok) {
  const int n = ok ? (int)sizeof(T) : 0;  // 0: nothing is read, the element is zeroed
  if (sizeof(T) == 4)
    asm volatile("cp.async.ca.shared.global [%0], [%1], 4, %2;" ::"r"(dst), "l"(src), "r"(n) : "memory");
  else
    asm volatile("cp.async.ca.shared.global [%0], [%1], 8, %2;" ::"r"(dst), "l"(src), "r"(n) : "memory");
}

#ifndef MHD_EMF_STREAM_MINB
#define MHD_EMF_STREAM_MINB 3
#endif
template <typename T, int E, int NW, bool M, bool B>
__global__ void __launch_bounds__(32 * NW, MHD_EMF_STREAM_MINB)
    k_emf_stream(KArg<T, B> ka, Inp<T> in0, Prm<T> P) {
  const int4 bb = ka.blk();
  const auto& d = ka.dev(bb);
  const Inp<T> in = B ? state_view(d) : in0;
  typedef EmfStream<T, E, NW> K;
  typedef Pr<T> Q;
  typedef typename Q::V V;
  constexpr int A1 = (E + 1) % 3, A2 = (E + 2) % 3;
  constexpr int C = K::C, NS = K::NS, TS = K::TS, DV = K::DV, NT = K::NT, NE = K::NE;
  constexpr bool SA2 = K::SA2;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  V* vr = reinterpret_cast<V*>(smem_raw);              // [DV][NS] (v_a1, v_a2)
  V* gr = vr + DV * NS;                                // ej: [NW][C] first-pass rows
  T* br = reinterpret_cast<T*>(gr + (SA2 ? 0 : NW * C));  // [2][NS] face B across the slice
  T* fr = br + 2 * NS;                                 // [4][NS] vf
  const Geom& g = d.g;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int x0 = g.ng + 32 * bb.y;   // first x of the tile (edge or cell index)
  const int w0 = g.ng + NW * bb.z;   // first index along the warp axis (y, z, y)
  const int nS0 = (E == 2) ? g.ny0 : g.nz0;     // interior cells along S
  const int nSg = (E == 2) ? g.ny : g.nz;
  const int nW0 = (E == 2) ? g.nz0 : g.ny0;
  const int seg = emf_stream_seg(g.nx0, nW0, nS0);
  const int s_lo = g.ng + seg * bb.w;
  const int s_hi = (bb.w == emf_stream_segs(nS0, seg) - 1) ? g.ng + nS0 : s_lo + seg - 1;
  const int SS = (E == 2) ? g.px : (int)g.plane;  // global stride along S
  const int ox = x0 + lane, ow = w0 + warp;
  const bool own = ox < g.ng + g.nx0 && ow < g.ng + nW0;
  const int obase = ox + ((E == 2) ? (int)g.plane * ow : g.px * ow);  // own column at S = 0
  const int oi = (E == 0) ? (warp + 4) * C + lane : warp * C + lane + 4;  // own cell in a slice
  // the slice cells this thread copies: global offset at S = 0 and bounds
  int go[NE];
  bool gok[NE];
#pragma unroll
  for (int k = 0; k < NE; ++k) {
    const int idx = tid + k * NT, r = idx / C, q = idx - r * C;
    int x, w;
    if (E == 0) { x = x0 + q; w = w0 - 4 + r; }
    else { x = x0 - 4 + q; w = w0 + r; }
    const int nw = (E == 2) ? g.nz : g.ny;
    gok[k] = idx < NS && (unsigned)x < (unsigned)g.nx && (unsigned)w < (unsigned)nw;
    go[k] = x + ((E == 2) ? (int)g.plane * w : g.px * w);
  }
  const T* vel[3] = {in.vx, in.vy, in.vz};
  const T* fb[3] = {in.bi, in.bj, in.bk};
  const T* v1 = vel[A1];
  const T* v2 = vel[A2];
  const T* bst = SA2 ? fb[A2] : fb[A1];  // reconstructed across the slice (staged)
  const T* bwn = SA2 ? fb[A1] : fb[A2];  // reconstructed along S (own-column window)
  const T* vf = d.vf;
  const uint32_t vr_s = (uint32_t)__cvta_generic_to_shared(vr);
  const uint32_t br_s = (uint32_t)__cvta_generic_to_shared(br);
  const uint32_t fr_s = (uint32_t)__cvta_generic_to_shared(fr);
  auto vslot = [&](int s) { return (s - s_lo + 4) & (DV - 1); };
  // copy slice s of the selected arrays into their ring slots
  auto stage = [&](int s, bool with_v, bool with_bf) {
    const bool sok = (unsigned)s < (unsigned)nSg;
#pragma unroll
    for (int k = 0; k < NE; ++k) {
      if (k * NT + tid < NS) {
        const int idx = tid + k * NT;
        const bool ok = gok[k] && sok;
        const int o = ok ? go[k] + s * SS : 0;
        if (with_v) {
          const uint32_t a = vr_s + (uint32_t)((vslot(s) * NS + idx) * sizeof(V));
          cp_async_zfill<T>(a, v1 + o, ok);
          cp_async_zfill<T>(a + sizeof(T), v2 + o, ok);
        }
        if (with_bf) {
          cp_async_zfill<T>(br_s + (uint32_t)(((s & 1) * NS + idx) * sizeof(T)), bst + o, ok);
          cp_async_zfill<T>(fr_s + (uint32_t)(((s & 3) * NS + idx) * sizeof(T)), vf + o, ok);
        }
      }
    }
  };
  // prologue: v slices s_lo-4 .. s_lo+3, face B at s_lo, vf at s_lo-1 and s_lo
#pragma unroll 1
  for (int m = 0; m < 8; ++m) stage(s_lo - 4 + m, true, m == 3 || m == 4);
  asm volatile("cp.async.commit_group;" ::: "memory");
  T bw[8];
#pragma unroll
  for (int m = 0; m < 8; ++m) bw[m] = own ? bwn[obase + (s_lo - 4 + m) * SS] : T(0);
  asm volatile("cp.async.wait_all;" ::: "memory");
  __syncthreads();
  // first pass along a1 inside slice s (S = a2)
  auto first_a1 = [&](int s) {
    const V* a = vr + vslot(s) * NS + oi;
    return tap8p<T>(a[-4 * TS], a[-3 * TS], a[-2 * TS], a[-TS], a[0], a[TS], a[2 * TS], a[3 * TS]);
  };
  V gw[8];
  if constexpr (SA2) {
#pragma unroll
    for (int m = 0; m < 8; ++m) gw[m] = first_a1(s_lo - 4 + m);
    __syncthreads();  // the first step refills the slot of slice s_lo - 4
  }
#pragma unroll 1
  for (int s = s_lo; s <= s_hi; ++s) {
    const bool more = s < s_hi;
    T bnext = T(0);
    if (more) {  // inputs of the next step
      stage(s + 4, true, false);
      stage(s + 1, false, true);
      if (own) bnext = bwn[obase + (s + 4) * SS];
    }
    asm volatile("cp.async.commit_group;" ::: "memory");
    V vi;
    if constexpr (SA2) {
      vi = tap8p<T>(gw[0], gw[1], gw[2], gw[3], gw[4], gw[5], gw[6], gw[7]);
    } else {
      // first pass along a1 = S across the ring into this warp's row
#pragma unroll
      for (int h = 0; h < 2; ++h) {
        const int r2 = lane + 32 * h;
        if (r2 < C) {
          const int col = warp * C + r2;
          gr[col] = tap8p<T>(vr[vslot(s - 4) * NS + col], vr[vslot(s - 3) * NS + col], vr[vslot(s - 2) * NS + col],
                             vr[vslot(s - 1) * NS + col], vr[vslot(s) * NS + col], vr[vslot(s + 1) * NS + col],
                             vr[vslot(s + 2) * NS + col], vr[vslot(s + 3) * NS + col]);
        }
      }
      __syncwarp();
      const V* gg = gr + warp * C + lane;
      vi = tap8p<T>(gg[0], gg[1], gg[2], gg[3], gg[4], gg[5], gg[6], gg[7]);
    }
    // the 12 corner cells, (d1, d2) from the upper cell
    const V* sm2 = vr + vslot(s - 2) * NS + oi;
    const V* sm1 = vr + vslot(s - 1) * NS + oi;
    const V* s00 = vr + vslot(s) * NS + oi;
    const V* sp1 = vr + vslot(s + 1) * NS + oi;
    V m11, m21, m12, m01, p11, m02, m10, m20, m1p, c0, p10, p01;
    if constexpr (SA2) {  // d1 in the slice (stride TS), d2 across slices
      m11 = sm1[-TS]; m21 = sm1[-2 * TS]; m12 = sm2[-TS]; m01 = sm1[0]; p11 = sm1[TS]; m02 = sm2[0];
      m10 = s00[-TS]; m20 = s00[-2 * TS]; m1p = sp1[-TS]; c0 = s00[0]; p10 = s00[TS]; p01 = sp1[0];
    } else {  // d1 across slices, d2 in the slice (stride 1)
      m11 = sm1[-1]; m21 = sm2[-1]; m12 = sm1[-2]; m01 = s00[-1]; p11 = sp1[-1]; m02 = s00[-2];
      m10 = sm1[0]; m20 = sm2[0]; m1p = sm1[1]; c0 = s00[0]; p10 = sp1[0]; p01 = s00[1];
    }
    const T v1av = corner_pdm_vals(m11.x, m21.x, m12.x, m01.x, p11.x, m02.x, m10.x, m20.x, m1p.x, c0.x, p10.x, p01.x,
                                   vi.x, P.pdmb);
    const T v2av = corner_pdm_vals(m11.y, m21.y, m12.y, m01.y, p11.y, m02.y, m10.y, m20.y, m1p.y, c0.y, p10.y, p01.y,
                                   vi.y, P.pdmb);
    // face B: across the slice from the staged slice, along S from the window
    constexpr int BS = SA2 ? TS : 1;
    const T* bb = br + (s & 1) * NS + oi;
    T sl, sr, wl, wr;
    recon_pdm8(bb[-4 * BS], bb[-3 * BS], bb[-2 * BS], bb[-BS], bb[0], bb[BS], bb[2 * BS], bb[3 * BS], P.pdmb, sl, sr);
    recon_pdm8(bw[0], bw[1], bw[2], bw[3], bw[4], bw[5], bw[6], bw[7], P.pdmb, wl, wr);
    const T* f0 = fr + (s & 3) * NS + oi;
    const T* fm = fr + ((s - 1) & 3) * NS + oi;
    T eta;
    if constexpr (SA2) eta = eta4(fm[-TS], fm[0], f0[0], f0[-TS]);  // s1 in the slice, s2 = S
    else eta = eta4(fm[-1], f0[-1], f0[0], fm[0]);                  // s1 = S, s2 in the slice
    if (own) {
      const int c = obase + s * SS;
      // b1 = B_a1 along a2, b2 = B_a2 along a1
      d.E[E][c] = SA2 ? emf_value<T, E, M>(d, c, v1av, v2av, wl, wr, sl, sr, eta)
                      : emf_value<T, E, M>(d, c, v1av, v2av, sl, sr, wl, wr, eta);
    }
    asm volatile("cp.async.wait_all;" ::: "memory");
    __syncthreads();
    if (more) {
#pragma unroll
      for (int m = 0; m < 7; ++m) bw[m] = bw[m + 1];
      bw[7] = bnext;
      if constexpr (SA2) {
#pragma unroll
        for (int m = 0; m < 7; ++m) gw[m] = gw[m + 1];
        gw[7] = first_a1(s + 4);
      }
    }
  }
}

// The (n0+1)-th edge row of the in-slice transverse axis of each streamed
// family, as thin shared-memory tiles of emf_pdm_tile in one launch of
// 256-thread blocks: ei at y = ny0 in 32 x 1 x 8 tiles (x, y, z edges), ek
// at x = nx0 in 1 x 32 x 8 tiles, ej at x = nx0 in 1 x 8 x 32 tiles.
struct EmfRows {
  int bi, bk, bj;  // blocks of the three planes
  __host__ __device__ explicit EmfRows(const Geom& g)
      : bi(((g.nx0 + 31) / 32) * ((g.nz0 + 8) / 8)), bk(((g.ny0 + 32) / 32) * ((g.nz0 + 7) / 8)),
        bj(((g.ny0 + 7) / 8) * ((g.nz0 + 32) / 32)) {}
  __host__ __device__ int blocks() const { return bi + bk + bj; }
};
template <typename T>
constexpr size_t emf_rows_smem() {
  constexpr size_t a = emf_pdm_smem<T, 0, 32, 1, 8>(), b = emf_pdm_smem<T, 2, 1, 32, 8>(),
                   c = emf_pdm_smem<T, 1, 1, 8, 32>();
  return a > b ? (a > c ? a : c) : (b > c ? b : c);
}
template <typename T, bool M, bool B>
__global__ void __launch_bounds__(256) k_emf_rows(KArg<T, B> ka, Inp<T> in0, Prm<T> P) {
  const int4 bb = ka.blk();
  const auto& d = ka.dev(bb);
  const Inp<T> in = B ? state_view(d) : in0;
  const Geom& g = d.g;
  const EmfRows r(g);
  int b = bb.y;
  if (b < r.bi) {
    const int nbx = (g.nx0 + 31) / 32, bx = b % nbx, bz = b / nbx;
    emf_pdm_tile<T, 0, 32, 1, 8, M>(d, in, P, g.ng + 32 * bx, g.ng + g.ny0, g.ng + 8 * bz);
    return;
  }
  b -= r.bi;
  if (b < r.bk) {
    const int nby = (g.ny0 + 32) / 32, by = b % nby, bz = b / nby;
    emf_pdm_tile<T, 2, 1, 32, 8, M>(d, in, P, g.ng + g.nx0, g.ng + 32 * by, g.ng + 8 * bz);
    return;
  }
  b -= r.bk;
  const int nby = (g.ny0 + 7) / 8, by = b % nby, bz = b / nby;
  emf_pdm_tile<T, 1, 1, 8, 32, M>(d, in, P, g.ng + g.nx0, g.ng + 8 * by, g.ng + 32 * bz);
}

// blocks of streamed family E on one grid (x tiles, warp-axis tiles, segments)
inline dim3 emf_stream_grid(int E, const Geom& g) {
  const int nS0 = (E == 2) ? g.ny0 : g.nz0, nW0 = (E == 2) ? g.nz0 : g.ny0;
  return dim3((g.nx0 + 31) / 32, (nW0 + MHD_EMF_NW - 1) / MHD_EMF_NW,
              emf_stream_segs(nS0, emf_stream_seg(g.nx0, nW0, nS0)));
}
template <typename T, int E, bool M, bool B>
void stream_attr() {
  static PerDevice attr;
  unsigned long long bit = 0;
  if (attr.need(bit)) {
    cudaFuncSetAttribute(k_emf_stream<T, E, MHD_EMF_NW, M, B>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                         (int)EmfStream<T, E, MHD_EMF_NW>::smem);
    attr.mark(bit);
  }
}
template <typename T, int E, bool M>
void launch_emf_stream(const Dev<T>& d, const Inp<T>& in, const Prm<T>& P, cudaStream_t st) {
  typedef EmfStream<T, E, MHD_EMF_NW> K;
  stream_attr<T, E, M, false>();
  k_emf_stream<T, E, MHD_EMF_NW, M, false><<<emf_stream_grid(E, d.g), K::NT, K::smem, st>>>(one(d), in, P);
}

template <typename T, bool M>
void emf_pdm_stream(const Dev<T>& d, const Inp<T>& in, const Prm<T>& P, cudaStream_t st) {
  launch_emf_stream<T, 0, M>(d, in, P, st);
  launch_emf_stream<T, 1, M>(d, in, P, st);
  launch_emf_stream<T, 2, M>(d, in, P, st);
  static_assert(emf_rows_smem<T>() <= 48 * 1024, "k_emf_rows fits the default shared-memory limit");
  k_emf_rows<T, M, false><<<EmfRows(d.g).blocks(), 256, emf_rows_smem<T>(), st>>>(one(d), in, P);
}

// ------------------------------------------------------------- WENO EMF
// Shared-memory tiled EMF of family E for WENO5 / MP-WENO5.  The corner
// velocity of get_vav_center2corner (mhd3d3.f90:1925-2049) reconstructs six
// rows of cells along d1 and then the six row results along d2 ("_1"), and
// six columns along d2 and then along d1 ("_0").  Neighbouring edges share
// five of the six rows, so a block stages v_a1 and v_a2 of its tile of edges
// with the stencil halo (3 cells below and 2 above on each transverse axis),
// computes every row and column reconstruction of the tile once into shared
// memory (first pass), and each edge then takes its four second-pass
// reconstructions, the dif-sign quadrant choice and the 4-quadrant mean of
// corner_vel, the upwinded face-B reconstructions and the resistivity term
// of k_emf, with the same operands in the same order.

// An (e, a1, a2) array of edge family E with the x-mapped index fastest, so
// that lanes of a warp touch consecutive words.
template <int E, int DE, int D1, int D2>
struct EdgeLay {
  static constexpr int A1 = (E + 1) % 3;
  static constexpr int N = DE * D1 * D2;
  static constexpr int NX = (E == 0) ? DE : (A1 == 0) ? D1 : D2;
  static constexpr int GE = (E == 0) ? 1 : (A1 == 0) ? D1 : D2;
  static constexpr int G1 = (E == 0) ? DE : (A1 == 0) ? 1 : D2 * DE;
  static constexpr int G2 = (E == 0) ? DE * D1 : (A1 == 0) ? D1 * DE : 1;
  // coordinates of flat index t (t == e * GE + f1 * G1 + f2 * G2)
  __device__ static __forceinline__ void coords(int t, int& e, int& f1, int& f2) {
    const int ix = t % NX, row = t / NX;
    if (E == 0) {
      e = ix; f1 = row % D1; f2 = row / D1;
    } else if (A1 == 0) {
      f1 = ix; e = row % DE; f2 = row / DE;
    } else {
      f2 = ix; e = row % DE; f1 = row / DE;
    }
  }
};

template <typename T, int E, int TX, int TY, int TZ>
struct EmfWeno {
  static constexpr int A1 = (E + 1) % 3, A2 = (E + 2) % 3;
  // staged cells: the edge axis without halo, each transverse axis [-3, T+2)
  static constexpr int LX = (E == 0) ? 0 : 3, LY = (E == 1) ? 0 : 3, LZ = (E == 2) ? 0 : 3;
  static constexpr int SX = TX + ((E == 0) ? 0 : 5), SY = TY + ((E == 1) ? 0 : 5), SZ = TZ + ((E == 2) ? 0 : 5);
  static constexpr int NV = SX * SY * SZ;
  static constexpr int SE = (E == 0) ? 1 : (E == 1) ? SX : SX * SY;
  static constexpr int S1 = (A1 == 0) ? 1 : (A1 == 1) ? SX : SX * SY;
  static constexpr int S2 = (A2 == 0) ? 1 : (A2 == 1) ? SX : SX * SY;
  static constexpr int TE = (E == 0) ? TX : (E == 1) ? TY : TZ;
  static constexpr int T1 = (A1 == 0) ? TX : (A1 == 1) ? TY : TZ;
  static constexpr int T2 = (A2 == 0) ? TX : (A2 == 1) ? TY : TZ;
  typedef EdgeLay<E, TE, T1, T2 + 5> L1;  // "_1": rows [-3, T2+2) reconstructed along a1 at the a1 faces
  typedef EdgeLay<E, TE, T1 + 5, T2> L0;  // "_0": columns [-3, T1+2) reconstructed along a2 at the a2 faces
  static constexpr int NP = L1::N + L0::N;
  // sv[2][NV] (v_a1, v_a2), then per component: L1, R1 [L1::N], L0, R0 [L0::N]
  static constexpr size_t smem = sizeof(T) * (2 * NV + 4 * NP);
};

template <typename T, int RECON, int E, int TX, int TY, int TZ, int NT, bool M>
__global__ void __launch_bounds__(NT) k_emf_weno(Dev<T> d, Inp<T> in, Prm<T> P) {
  typedef EmfWeno<T, E, TX, TY, TZ> K;
  typedef typename K::L1 L1;
  typedef typename K::L0 L0;
  constexpr int A1 = K::A1, A2 = K::A2, NV = K::NV, NP = K::NP, N1 = L1::N, N0 = L0::N;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  T* sv = reinterpret_cast<T*>(smem_raw);
  T* sp = sv + 2 * NV;
  const Geom& g = d.g;
  const int ox = g.ng + blockIdx.x * TX, oy = g.ng + blockIdx.y * TY, oz = g.ng + blockIdx.z * TZ;
  const T* vel[3] = {in.vx, in.vy, in.vz};
  const T* v1 = vel[A1];
  const T* v2 = vel[A2];
  for (int t = threadIdx.x; t < NV; t += blockDim.x) {
    const int lx = t % K::SX, row = t / K::SX;
    const int ly = row % K::SY, lz = row / K::SY;
    const int gx = ox - K::LX + lx, gy = oy - K::LY + ly, gz = oz - K::LZ + lz;
    T a = T(0), b = T(0);
    if (gx < g.nx && gy < g.ny && gz < g.nz) {
      const int gi = gx + g.px * (gy + g.py * gz);
      a = v1[gi];
      b = v2[gi];
    }
    sv[t] = a;
    sv[NV + t] = b;
  }
  __syncthreads();
  // first pass: every row ("_1") and column ("_0") reconstruction of the
  // tile for both components; tap q of an entry is the cell at offset q - 3
  for (int t = threadIdx.x; t < 2 * NP; t += blockDim.x) {
    const int w = t >= NP;
    const int u = t - w * NP;
    const T* src = sv + w * NV;
    T* dst = sp + w * 2 * NP;
    int e, f1, f2, base, step, o1, o2;
    if (u < N1) {  // row f2 - 3 along a2, reconstructed along a1 at the face of cell f1
      L1::coords(u, e, f1, f2);
      base = e * K::SE + f1 * K::S1 + f2 * K::S2;
      step = K::S1;
      o1 = u;
      o2 = N1 + u;
    } else {  // column f1 - 3 along a1, reconstructed along a2 at the face of cell f2
      L0::coords(u - N1, e, f1, f2);
      base = e * K::SE + f1 * K::S1 + f2 * K::S2;
      step = K::S2;
      o1 = 2 * N1 + (u - N1);
      o2 = 2 * N1 + N0 + (u - N1);
    }
    T a[6];
#pragma unroll
    for (int q = 0; q < 6; ++q) a[q] = src[base + q * step];
    T fl, fr;
    weno_vals<T, RECON>(a, P, fl, fr);
    dst[o1] = fl;
    dst[o2] = fr;
  }
  __syncthreads();
  const int lim[3] = {g.ng + g.nx0 + (E != 0), g.ng + g.ny0 + (E != 1), g.ng + g.nz0 + (E != 2)};
  const int st[3] = {1, g.px, (int)g.plane};
  const T* fb[3] = {in.bi, in.bj, in.bk};
  for (int t = threadIdx.x; t < TX * TY * TZ; t += blockDim.x) {
    const int lx = t % TX, r = t / TX, ly = r % TY, lz = r / TY;
    const int gx = ox + lx, gy = oy + ly, gz = oz + lz;
    if (gx >= lim[0] || gy >= lim[1] || gz >= lim[2]) continue;
    const int e = (E == 0) ? lx : (E == 1) ? ly : lz;
    const int f1 = (A1 == 0) ? lx : (A1 == 1) ? ly : lz;
    const int f2 = (A2 == 0) ? lx : (A2 == 1) ? ly : lz;
    T v1av = T(0), v2av = T(0);
#pragma unroll 1
    for (int w = 0; w < 2; ++w) {
      const T* s = sp + w * 2 * NP;
      // dif signs pick the smoother one-sided estimate per quadrant (2056-2106):
      // "_0" (columns, second pass along d1) if d >= 0, else "_1" (rows)
      const T* v = sv + w * NV;
      const int c = e * K::SE + (f1 + 3) * K::S1 + (f2 + 3) * K::S2;
      constexpr int s1 = K::S1, s2 = K::S2;
      const int q00 = c - s1 - s2, q10 = c - s2, q01 = c - s1, q11 = c;
      const T d00 = fab(v[q00 - s1] - v[q00]) - fab(v[q00 - s2] - v[q00]);
      const T d10 = fab(v[q10 + s1] - v[q10]) - fab(v[q10 - s2] - v[q10]);
      const T d01 = fab(v[q01 - s1] - v[q01]) - fab(v[q01 + s2] - v[q01]);
      const T d11 = fab(v[q11 + s1] - v[q11]) - fab(v[q11 + s2] - v[q11]);
      // left (L) and right (R) first-pass arrays of the rows ("_1") and columns ("_0")
      const T* l1 = s + e * L1::GE + f1 * L1::G1 + f2 * L1::G2;           // rows f2 - 3 + m at m * G2
      const T* l0 = s + 2 * N1 + e * L0::GE + f1 * L0::G1 + f2 * L0::G2;  // columns f1 - 3 + m
      // only the chosen estimate of each quadrant is evaluated: v_00 / v_10 are
      // the left states of the L / R stencils, v_01 / v_11 the right states
      // (the left-state formula on the mirrored stencil)
      auto pick = [&](bool col, int off) -> const T* { return col ? l0 + off : l1 + off; };
      const T* a00 = pick(d00 >= T(0), 0);
      const T* a10 = pick(d10 >= T(0), d10 >= T(0) ? N0 : N1);
      const T* a01 = pick(d01 >= T(0), 0);
      const T* a11 = pick(d11 >= T(0), d11 >= T(0) ? N0 : N1);
      const int g00 = d00 >= T(0) ? L0::G1 : L1::G2, g10 = d10 >= T(0) ? L0::G1 : L1::G2;
      const int g01 = d01 >= T(0) ? L0::G1 : L1::G2, g11 = d11 >= T(0) ? L0::G1 : L1::G2;
      const T v00 = weno_one<T, RECON>(a00[0], a00[g00], a00[2 * g00], a00[3 * g00], a00[4 * g00], P);
      const T v10 = weno_one<T, RECON>(a10[0], a10[g10], a10[2 * g10], a10[3 * g10], a10[4 * g10], P);
      const T v01 = weno_one<T, RECON>(a01[5 * g01], a01[4 * g01], a01[3 * g01], a01[2 * g01], a01[g01], P);
      const T v11 = weno_one<T, RECON>(a11[5 * g11], a11[4 * g11], a11[3 * g11], a11[2 * g11], a11[g11], P);
      const T vc = T(0.25) * (v00 + v01 + v10 + v11);
      if (w == 0)
        v1av = vc;
      else
        v2av = vc;
    }
    const int c = gx + g.px * (gy + g.py * gz);
    const int s1 = st[A1], s2 = st[A2];
    T b1l, b1r, b2l, b2r;
    recon_face<T, RECON>(fb[A1], c, s2, P, b1l, b1r);
    recon_face<T, RECON>(fb[A2], c, s1, P, b2l, b2r);
    T b1u = (v2av >= T(0)) ? b1l : b1r;
    T b2u = (v1av >= T(0)) ? b2l : b2r;
    T ee = -v1av * b2u + v2av * b1u;
    const T* vf = d.vf;
    T eta = T(0.25) * (vf[c - s1 - s2] + vf[c - s2] + vf[c] + vf[c - s1]);
    if (M)
      ee = (T)d.m.ge[E][c] * ee + eta * (T)d.m.dl[E][c] * (b1l + b2r - b1r - b2l);
    else
      ee = ee + eta * (b1l + b2r - b1r - b2l);
    d.E[E][c] = ee;
  }
}

template <typename T, int RECON, int E, int TX, int TY, int TZ, int NT, bool M>
void launch_emf_weno(const Dev<T>& d, const Inp<T>& in, const Prm<T>& P, cudaStream_t st) {
  constexpr size_t bytes = EmfWeno<T, E, TX, TY, TZ>::smem;
  static PerDevice attr;
  unsigned long long bit = 0;
  if (attr.need(bit)) {
    cudaFuncSetAttribute(k_emf_weno<T, RECON, E, TX, TY, TZ, NT, M>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                         (int)bytes);
    attr.mark(bit);
  }
  const Geom& g = d.g;
  const int ex = g.nx0 + (E != 0), ey = g.ny0 + (E != 1), ez = g.nz0 + (E != 2);
  const dim3 grid((ex + TX - 1) / TX, (ey + TY - 1) / TY, (ez + TZ - 1) / TZ);
  k_emf_weno<T, RECON, E, TX, TY, TZ, NT, M><<<grid, NT, bytes, st>>>(d, in, P);
}


// Metric-mode EMF inputs of a stage: w^a = v . nbar_a at every cell and the
// face-normal field b_a = Phi_a / |A_a| at every face (ghosts included),
// which the EMF kernels then treat as the reference treats v and bi/bj/bk.
template <typename T>
__global__ void k_metric_prep(Dev<T> d, Inp<T> in) {
  const Geom& g = d.g;
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const int j = blockIdx.y * blockDim.y + threadIdx.y;
  const int k = blockIdx.z;
  if (i > g.nx || j > g.ny || k > g.nz) return;
  const long long c = idx3<T>(g, i, j, k);
  const Metric& m = d.m;
  if (i < g.nx && j < g.ny && k < g.nz) {
    const T u = in.vx[c], v = in.vy[c], w = in.vz[c];
#pragma unroll
    for (int a = 0; a < 3; ++a) d.mw[a][c] = u * (T)m.nb[a][0][c] + v * (T)m.nb[a][1][c] + w * (T)m.nb[a][2][c];
  }
  if (j < g.ny && k < g.nz) d.mbn[0][c] = Ops<T>::dv(in.bi[c], (T)m.am[0][c]);
  if (i < g.nx && k < g.nz) d.mbn[1][c] = Ops<T>::dv(in.bj[c], (T)m.am[1][c]);
  if (i < g.nx && j < g.ny) d.mbn[2][c] = Ops<T>::dv(in.bk[c], (T)m.am[2][c]);
}

// ------------------------------------------------------------------ update
// advance_bijk (3909-3933) + B combine, interior faces of all three arrays,
// read from the stage's half of the face B and written to the other half.
template <typename T, bool M, bool B>
__global__ void k_update_b(KArg<T, B> ka, int form, T cw, T den) {
  const int4 bb = ka.blk();
  const auto& d = ka.dev(bb);
  const Geom& g = d.g;
  int i = bb.y * blockDim.x + threadIdx.x + g.ng;
  int j = bb.z * blockDim.y + threadIdx.y + g.ng;
  int k = bb.w + g.ng;
  if (i > g.ng + g.nx0 || j > g.ng + g.ny0 || k > g.ng + g.nz0) return;
  bool in_x = i < g.ng + g.nx0, in_y = j < g.ng + g.ny0, in_z = k < g.ng + g.nz0;
  long long c = idx3<T>(g, i, j, k);
  const long long sy = g.px, sz = g.plane;
  const T tau = (T)d.sc->tau;
  const T dx = d.wx[i], dy = d.wy[j], dz = d.wz[k];
  const T rx = d.rwx[i], ry = d.rwy[j], rz = d.rwz[k];
  const T *ei = d.E[0], *ej = d.E[1], *ek = d.E[2];
  typedef Ops<T> O;
  if (M) {  // face fluxes minus tau times the circulation of E.dl
    if (in_y && in_z) {
      T b = d.bi[c] - tau * ((ek[c + sy] - ek[c]) - (ej[c + sz] - ej[c]));
      if (form >= 0) b = comb(form, cw, d.q[5][c], b, den);
      d.obi[c] = b;
    }
    if (in_x && in_z) {
      T b = d.bj[c] - tau * ((ei[c + sz] - ei[c]) - (ek[c + 1] - ek[c]));
      if (form >= 0) b = comb(form, cw, d.q[6][c], b, den);
      d.obj[c] = b;
    }
    if (in_x && in_y) {
      T b = d.bk[c] - tau * ((ej[c + 1] - ej[c]) - (ei[c + sy] - ei[c]));
      if (form >= 0) b = comb(form, cw, d.q[7][c], b, den);
      d.obk[c] = b;
    }
    return;
  }
  if (in_y && in_z) {
    T b = d.bi[c] - tau * (O::dw(ek[c + sy] - ek[c], dy, ry) - O::dw(ej[c + sz] - ej[c], dz, rz));
    if (form >= 0) b = comb(form, cw, d.q[5][c], b, den);
    d.obi[c] = b;
  }
  if (in_x && in_z) {
    T b = d.bj[c] - tau * (O::dw(ei[c + sz] - ei[c], dz, rz) - O::dw(ek[c + 1] - ek[c], dx, rx));
    if (form >= 0) b = comb(form, cw, d.q[6][c], b, den);
    d.obj[c] = b;
  }
  if (in_x && in_y) {
    T b = d.bk[c] - tau * (O::dw(ej[c + 1] - ej[c], dx, rx) - O::dw(ei[c + sy] - ei[c], dy, ry));
    if (form >= 0) b = comb(form, cw, d.q[7][c], b, den);
    d.obk[c] = b;
  }
}

// ------------------------------------------------------------------- fill
// Single-device replacement of fill_hydro_mpi / fill_mag_mpi (781-819): every
// ghost element takes the value of its per-axis image (the x, y, z passes of
// the reference compose to exactly this, since each pass reads only interior
// values along its own axis).  Cell axes: interior [ng, ng+n0); the face
// array's own axis: interior [ng, ng+n0].
__device__ __forceinline__ int ghost_src(int x, int ng, int n0, bool face, int kind, bool& flip) {
  flip = false;
  int hi = face ? ng + n0 : ng + n0 - 1;  // last interior index
  if (x >= ng && x <= hi) return x;
  bool lo = x < ng;
  if (kind == BC_PERIODIC) return lo ? x + n0 : x - n0;
  if (kind == BC_OUTFLOW) return lo ? ng : hi;
  flip = true;  // mirror: even (flip ignored) or odd
  if (!face) return lo ? 2 * ng - 1 - x : 2 * n0 + 2 * ng - 1 - x;
  return lo ? 2 * ng - x : 2 * n0 + 2 * ng - x;
}

template <typename T>
__global__ void k_fill(Dev<T> d) {
  const Geom& g = d.g;
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  int j = blockIdx.y * blockDim.y + threadIdx.y;
  int k = blockIdx.z;
  if (i > g.nx || j > g.ny || k > g.nz) return;
  T* arr[8] = {d.rho, d.vx, d.vy, d.vz, d.p, d.bi, d.bj, d.bk};
  const int n0[3] = {g.nx0, g.ny0, g.nz0};
  const int x3[3] = {i, j, k};
#pragma unroll
  for (int a = 0; a < 8; ++a) {
    int fa = a - 5;  // own staggering axis of bi/bj/bk
    bool ghost = false, inside = true;
    int s3[3];
    T sgn = T(1);
#pragma unroll
    for (int ax = 0; ax < 3; ++ax) {
      bool face = (fa == ax);
      int ext = (ax == 0 ? g.nx : ax == 1 ? g.ny : g.nz) + (face ? 1 : 0);
      if (x3[ax] >= ext) inside = false;
      bool flip;
      s3[ax] = ghost_src(x3[ax], g.ng, n0[ax], face, d.bc[ax], flip);
      if (s3[ax] != x3[ax]) ghost = true;
      // reflecting wall: the normal velocity is odd (a = 1,2,3 -> vx,vy,vz)
      if (flip && d.bc[ax] == BC_REFLECT && a == 1 + ax) sgn = -sgn;
    }
    if (!inside || !ghost) continue;
    long long c = idx3<T>(g, i, j, k);
    long long s = idx3<T>(g, s3[0], s3[1], s3[2]);
    T val = arr[a][s];
    arr[a][c] = (sgn > T(0)) ? val : -val;
  }
}

// Ghost fill fused with get_bxyz (mhd3d3.f90:2118-2128) and vf: every thread
// fills the ghost elements it owns (as k_fill) and computes the cell-centred
// B and vf of its cell from the ghost images of the faces and cells it needs,
// so no thread reads an element another thread is filling.  Face B is even
// under every boundary kind and vf uses only squares, so the images give
// exactly the values the separate fill followed by get_bxyz produces.  The
// per-axis image of every index comes from d.gmap (ghost_src tabulated at
// set-up): cell maps of x, y, z then face maps of x, y, z, each padded to n+2.
//
// Launch layout (256 threads per block, block index bb.y): first the interior
// tiles, 32 x 8 cells of one z plane each, which take the fast path with no
// divergence; then the shell, every (i <= nx, j <= ny, k <= nz) outside the
// interior box, 256 elements per block in a flattened order (the z slabs,
// then the y slabs, then the x slabs of the remaining rows).
struct FillShape {
  int nbx, nby, nint, nshell;
  __host__ __device__ FillShape(const Geom& g)
      : nbx((g.nx0 + 31) / 32), nby((g.ny0 + 7) / 8), nint(nbx * nby * g.nz0),
        nshell((g.nz + 1 - g.nz0) * (g.ny + 1) * (g.nx + 1) + g.nz0 * (g.ny + 1 - g.ny0) * (g.nx + 1) +
               g.nz0 * g.ny0 * (g.nx + 1 - g.nx0)) {}
  __host__ __device__ int blocks() const { return nint + (nshell + 255) / 256; }
};

// (i, j, k) of shell element u (0 <= u < nshell)
__device__ __forceinline__ void fill_shell_ijk(const Geom& g, int u, int& i, int& j, int& k) {
  const int X = g.nx + 1, Y = g.ny + 1, Z = g.nz + 1;
  const int a = (Z - g.nz0) * Y * X;
  if (u < a) {  // k outside the interior
    const int kk = u / (Y * X), r = u - kk * (Y * X);
    k = kk < g.ng ? kk : kk + g.nz0;
    j = r / X;
    i = r - j * X;
    return;
  }
  u -= a;
  const int yb = (Y - g.ny0) * X, b = g.nz0 * yb;
  if (u < b) {  // k inside, j outside
    const int kk = u / yb, r = u - kk * yb;
    k = g.ng + kk;
    const int jj = r / X;
    j = jj < g.ng ? jj : jj + g.ny0;
    i = r - jj * X;
    return;
  }
  u -= b;  // k, j inside, i outside
  const int xs = X - g.nx0, xb = g.ny0 * xs;
  const int kk = u / xb, r = u - kk * xb;
  k = g.ng + kk;
  const int jj = r / xs;
  j = g.ng + jj;
  const int ii = r - jj * xs;
  i = ii < g.ng ? ii : ii + g.nx0;
}

// One element of k_fill_bxyz; returns the CFL dt of its cell when want_dt
// (its values and widths, as get_dt sees them after the fill), else +inf.
template <typename T, bool M>
__device__ __forceinline__ T fill_bxyz_elem(const Dev<T>& d, int4 bb, int want_vf, int shell_only, int want_dt,
                                            unsigned& st) {
  const Geom& g = d.g;
  const FillShape fs(g);
  const int blk = shell_only ? bb.y + fs.nint : bb.y;
  int i, j, k;
  bool inner;
  if (blk < fs.nint) {
    const int bx = blk % fs.nbx, r = blk / fs.nbx, by = r % fs.nby, kz = r / fs.nby;
    i = g.ng + bx * 32 + (threadIdx.x & 31);
    j = g.ng + by * 8 + (threadIdx.x >> 5);
    k = g.ng + kz;
    if (i >= g.ng + g.nx0 || j >= g.ng + g.ny0) return T(INFINITY);  // those cells belong to no block here
    inner = true;
  } else {
    const int u = (blk - fs.nint) * 256 + threadIdx.x;
    if (u >= fs.nshell) return T(INFINITY);
    fill_shell_ijk(g, u, i, j, k);
    inner = false;
  }
  const int px = g.px, pl = (int)g.plane;
  const int c = i + px * j + pl * k;
  // interior fast path (no ghost element owned, all images are the identity)
  if (inner) {
    T bx, by, bz;
    if (M) {
      cell_b_metric<T>(d.m, c, d.bi[c], d.bi[c + 1], d.bj[c], d.bj[c + px], d.bk[c], d.bk[c + pl], bx, by, bz);
    } else {
      bx = T(0.5) * (d.bi[c + 1] + d.bi[c]);
      by = T(0.5) * (d.bj[c + px] + d.bj[c]);
      bz = T(0.5) * (d.bk[c + pl] + d.bk[c]);
    }
    d.bx[c] = bx;
    d.by[c] = by;
    d.bz[c] = bz;
    if (want_vf || want_dt) {
      const T u = d.vx[c], v = d.vy[c], w = d.vz[c], r0 = d.rho[c];
      if (want_vf) d.vf[c] = sq(u * u + v * v + w * w) + sq((bx * bx + by * by + bz * bz) / r0);
      if (want_dt) return cell_dt<T, M>(d, c, i, j, k, r0, d.p[c], u, v, w, bx, by, bz, st);
    }
    return T(INFINITY);
  }
  const int* cx = d.gmap;
  const int* cy = cx + g.nx + 2;
  const int* cz = cy + g.ny + 2;
  const int* fx = cz + g.nz + 2;
  const int* fy = fx + g.nx + 2;
  const int* fz = fy + g.ny + 2;
  // every image index first, then every load, then every store: the loads of
  // one thread are in flight together (no store sits between them)
  const int sci = cx[i], scj = cy[j], sck = cz[k];  // cell images (entries n, n+1 unused)
  const int sfi = fx[i], sfj = fy[j], sfk = fz[k];  // face images
  const int sfi1 = fx[i + 1], sfj1 = fy[j + 1], sfk1 = fz[k + 1];
  const bool cin = i < g.nx && j < g.ny && k < g.nz;
  const bool gx = sci != i, gy = scj != j, gz = sck != k;
  const bool cell_copy = cin && (gx || gy || gz);
  const bool bi_copy = j < g.ny && k < g.nz && (sfi != i || gy || gz);
  const bool bj_copy = i < g.nx && k < g.nz && (gx || sfj != j || gz);
  const bool bk_copy = i < g.nx && j < g.ny && (gx || gy || sfk != k);
  const bool need_cell = cell_copy || (cin && (want_vf || want_dt));
  const int sc = sci + px * scj + pl * sck;
  const int fi0 = sfi + px * scj + pl * sck, fi1 = sfi1 + px * scj + pl * sck;  // faces of the image cell
  const int fj0 = sci + px * sfj + pl * sck, fj1 = sci + px * sfj1 + pl * sck;
  const int fk0 = sci + px * scj + pl * sfk, fk1 = sci + px * scj + pl * sfk1;
  T r0 = T(0), p0 = T(0), ux = T(0), uy = T(0), uz = T(0);
  if (need_cell) {
    r0 = d.rho[sc]; p0 = d.p[sc]; ux = d.vx[sc]; uy = d.vy[sc]; uz = d.vz[sc];
  }
  T bi0 = T(0), bi1 = T(0), bj0 = T(0), bj1 = T(0), bk0 = T(0), bk1 = T(0);
  if (bi_copy || cin) bi0 = d.bi[fi0];
  if (bj_copy || cin) bj0 = d.bj[fj0];
  if (bk_copy || cin) bk0 = d.bk[fk0];
  if (cin) {
    bi1 = d.bi[fi1];
    bj1 = d.bj[fj1];
    bk1 = d.bk[fk1];
  }
  // ghost copies: cell arrays (rho, vx, vy, vz, p), then bi, bj, bk
  if (cell_copy) {
    d.rho[c] = r0;
    d.p[c] = p0;
    d.vx[c] = (gx && d.bc[0] == BC_REFLECT) ? -ux : ux;
    d.vy[c] = (gy && d.bc[1] == BC_REFLECT) ? -uy : uy;
    d.vz[c] = (gz && d.bc[2] == BC_REFLECT) ? -uz : uz;
  }
  if (bi_copy) d.bi[c] = bi0;
  if (bj_copy) d.bj[c] = bj0;
  if (bk_copy) d.bk[c] = bk0;
  if (!cin) return T(INFINITY);
  T bx, by, bz;
  if (M) {  // face fluxes of the images, geometry of this cell (as fill then get_bxyz)
    cell_b_metric<T>(d.m, c, bi0, bi1, bj0, bj1, bk0, bk1, bx, by, bz);
  } else {
    bx = T(0.5) * (bi1 + bi0);
    by = T(0.5) * (bj1 + bj0);
    bz = T(0.5) * (bk1 + bk0);
  }
  d.bx[c] = bx;
  d.by[c] = by;
  d.bz[c] = bz;
  if (want_vf) d.vf[c] = sq(ux * ux + uy * uy + uz * uz) + sq((bx * bx + by * by + bz * bz) / r0);
  return want_dt ? cell_dt<T, M>(d, c, i, j, k, r0, p0, ux, uy, uz, bx, by, bz, st) : T(INFINITY);
}

// shell_only != 0: the launch covers only the shell blocks (block b is shell
// block b), after k_ct_fill has done the interior.  dt_next != 0: the CFL dt
// and status of the cells the launch covers go to the next-step accumulators.
template <typename T, bool M, bool B>
__global__ void __launch_bounds__(256, pass_min_blocks(B))
    k_fill_bxyz(KArg<T, B> ka, int want_vf, int shell_only, int dt_next) {
  const int4 bb = ka.blk();
  const auto& d = ka.dev(bb);
  unsigned st = 0;
  const bool want_dt = !B && dt_next;  // single grids only (a batch runs its own CFL pass)
  const T m = fill_bxyz_elem<T, M>(d, bb, want_vf, shell_only, want_dt, st);
  if (want_dt) dt_next_accumulate(d.sc, m, st);
}

// CT fused with get_bxyz and vf on Cartesian meshes (advance_bijk + combine,
// mhd3d3.f90:3909-3933, 3698-3702, 3784-3788; get_bxyz 2118-2128; vf of
// get_eijk_LFM 1766): one thread per interior cell, blocks of 32 x 8 cells of
// one z plane (the fill's interior tiles).  The thread advances its cell's
// three low faces into the new half of the face B with k_update_b's
// expressions and recomputes the new values of its three high faces from the
// same inputs (the cell that owns such a face writes it; the last cell of an
// axis writes the boundary face), then forms the cell-centred B from the six
// new faces and vf from the new primitives, which the z sweep wrote into the
// new half.  Every input here is read-only (old half of the face B, EMFs,
// U^n, new primitives), so a recomputed face equals what its owner writes,
// bit for bit, and the result equals k_update_b followed by the fill's
// interior tiles.  The ghost shell of the new half follows in k_fill_bxyz
// (shell_only).  An RK first stage (form FORM_SAVE) also stores its input
// face B as U^n of the later combines; dt_next (the last stage) accumulates
// the CFL dt and status of the new cells for the next step, as k_cfl would
// compute them at its start.
template <typename T, bool B>
__global__ void __launch_bounds__(256, pass_min_blocks(B))
    k_ct_fill(KArg<T, B> ka, int form, T cw, T den, int want_vf, int dt_next) {
  const int4 bb = ka.blk();
  const auto& d = ka.dev(bb);
  const Geom& g = d.g;
  const int i = g.ng + bb.y * 32 + (threadIdx.x & 31);
  const int j = g.ng + bb.z * 8 + (threadIdx.x >> 5);
  const int k = g.ng + bb.w;
  // batched stages neither store U^n nor accumulate the next dt (their CFL pass does both)
  const bool save = !B && form == FORM_SAVE, want_dt = !B && dt_next;
  T m = T(INFINITY);
  unsigned st = 0;
  if (i < g.ng + g.nx0 && j < g.ng + g.ny0) {
    const int px = g.px, pl = (int)g.plane;
    const int c = i + px * j + pl * k;
    const T tau = (T)d.sc->tau;
    const T dx = d.wx[i], dy = d.wy[j], dz = d.wz[k];
    const T rx = d.rwx[i], ry = d.rwy[j], rz = d.rwz[k];
    const T *ei = d.E[0], *ej = d.E[1], *ek = d.E[2];
    typedef Ops<T> O;
    auto new_bi = [&](int f) {
      T b = d.bi[f] - tau * (O::dw(ek[f + px] - ek[f], dy, ry) - O::dw(ej[f + pl] - ej[f], dz, rz));
      return form >= 0 ? comb(form, cw, d.q[5][f], b, den) : b;
    };
    auto new_bj = [&](int f) {
      T b = d.bj[f] - tau * (O::dw(ei[f + pl] - ei[f], dz, rz) - O::dw(ek[f + 1] - ek[f], dx, rx));
      return form >= 0 ? comb(form, cw, d.q[6][f], b, den) : b;
    };
    auto new_bk = [&](int f) {
      T b = d.bk[f] - tau * (O::dw(ej[f + 1] - ej[f], dx, rx) - O::dw(ei[f + px] - ei[f], dy, ry));
      return form >= 0 ? comb(form, cw, d.q[7][f], b, den) : b;
    };
    const bool lx = i == g.ng + g.nx0 - 1, ly = j == g.ng + g.ny0 - 1, lz = k == g.ng + g.nz0 - 1;
    if (save) {  // face B^n of the step (this first stage's input) for the later combines
      d.q[5][c] = d.bi[c];
      d.q[6][c] = d.bj[c];
      d.q[7][c] = d.bk[c];
      if (lx) d.q[5][c + 1] = d.bi[c + 1];
      if (ly) d.q[6][c + px] = d.bj[c + px];
      if (lz) d.q[7][c + pl] = d.bk[c + pl];
    }
    const T bil = new_bi(c), bih = new_bi(c + 1);
    const T bjl = new_bj(c), bjh = new_bj(c + px);
    const T bkl = new_bk(c), bkh = new_bk(c + pl);
    d.obi[c] = bil;
    d.obj[c] = bjl;
    d.obk[c] = bkl;
    if (lx) d.obi[c + 1] = bih;
    if (ly) d.obj[c + px] = bjh;
    if (lz) d.obk[c + pl] = bkh;
    const T bx = T(0.5) * (bih + bil);
    const T by = T(0.5) * (bjh + bjl);
    const T bz = T(0.5) * (bkh + bkl);
    d.bx[c] = bx;
    d.by[c] = by;
    d.bz[c] = bz;
    if (want_vf || want_dt) {
      const T u = d.ovx[c], v = d.ovy[c], w = d.ovz[c], r0 = d.orho[c];
      if (want_vf) d.vf[c] = sq(u * u + v * v + w * w) + sq((bx * bx + by * by + bz * bz) / r0);
      if (want_dt) m = cell_dt<T, false>(d, c, i, j, k, r0, d.op[c], u, v, w, bx, by, bz, st);
    }
  }
  if (want_dt) dt_next_accumulate(d.sc, m, st);
}

// ------------------------------------------------------------ diagnostics
// Double-double (Neumaier/TwoSum) accumulation of mass and energy, max |div B|
// (FP64), min rho incl. ghosts.  Deterministic: fixed per-thread order,
// fixed tree; partial results per block reduced by one block in order.
__device__ __forceinline__ void two_sum(double a, double b, double& s, double& e) {
  s = a + b;
  double bb = s - a;
  e = (a - (s - bb)) + (b - bb);
}
struct DD { double s, c; };
__device__ __forceinline__ DD dd_add(DD x, DD y) {
  double s, e;
  two_sum(x.s, y.s, s, e);
  e += x.c + y.c;
  double s2, e2;
  two_sum(s, e, s2, e2);
  return DD{s2, e2};
}

template <typename T, bool M>
__global__ void k_diag_partial(Dev<T> d, double* part) {
  const Geom& g = d.g;
  long long n = (long long)g.nx0 * g.ny0 * g.nz0;
  DD ms{0, 0}, es{0, 0};
  double dmax = 0.0;
  const double gm1 = (double)d.gam - 1.0;
  for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < n;
       t += (long long)gridDim.x * blockDim.x) {
    int i = (int)(t % g.nx0) + g.ng;
    long long r = t / g.nx0;
    int j = (int)(r % g.ny0) + g.ng;
    int k = (int)(r / g.ny0) + g.ng;
    long long c = idx3<T>(g, i, j, k);
    double dv = M ? d.m.vol[c] : d.dx[i] * d.dy[j] * d.dz[k];
    double rr = d.rho[c], u = d.vx[c], v = d.vy[c], w = d.vz[c], pp = d.p[c];
    double a = d.bx[c], b = d.by[c], cc = d.bz[c];
    ms = dd_add(ms, DD{rr * dv, 0.0});
    double e = 0.5 * rr * (u * u + v * v + w * w) + pp / gm1 + 0.5 * (a * a + b * b + cc * cc);
    es = dd_add(es, DD{e * dv, 0.0});
    double db;
    if (M)  // net face flux out of the cell / V
      db = (((double)d.bi[c + 1] - (double)d.bi[c]) + ((double)d.bj[c + g.px] - (double)d.bj[c]) +
            ((double)d.bk[c + g.plane] - (double)d.bk[c])) / dv;
    else
      db = ((double)d.bi[c + 1] - (double)d.bi[c]) / d.dx[i] +
           ((double)d.bj[c + g.px] - (double)d.bj[c]) / d.dy[j] +
           ((double)d.bk[c + g.plane] - (double)d.bk[c]) / d.dz[k];
    db = fabs(db);
    dmax = db > dmax ? db : dmax;
  }
  __shared__ double sh[5][256];
  int tid = threadIdx.x;
  sh[0][tid] = ms.s; sh[1][tid] = ms.c; sh[2][tid] = es.s; sh[3][tid] = es.c; sh[4][tid] = dmax;
  __syncthreads();
  for (int w = blockDim.x / 2; w > 0; w >>= 1) {
    if (tid < w) {
      DD a = dd_add(DD{sh[0][tid], sh[1][tid]}, DD{sh[0][tid + w], sh[1][tid + w]});
      DD b = dd_add(DD{sh[2][tid], sh[3][tid]}, DD{sh[2][tid + w], sh[3][tid + w]});
      sh[0][tid] = a.s; sh[1][tid] = a.c; sh[2][tid] = b.s; sh[3][tid] = b.c;
      sh[4][tid] = sh[4][tid] > sh[4][tid + w] ? sh[4][tid] : sh[4][tid + w];
    }
    __syncthreads();
  }
  if (tid == 0) {
    double* o = part + 5 * blockIdx.x;
    o[0] = sh[0][0]; o[1] = sh[1][0]; o[2] = sh[2][0]; o[3] = sh[3][0]; o[4] = sh[4][0];
  }
}

template <typename T>
__global__ void k_diag_final(Dev<T> d, const double* part, int nb, double* out) {
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  DD m{0, 0}, e{0, 0};
  double dm = 0;
  for (int b = 0; b < nb; ++b) {
    const double* o = part + 5 * b;
    m = dd_add(m, DD{o[0], o[1]});
    e = dd_add(e, DD{o[2], o[3]});
    dm = o[4] > dm ? o[4] : dm;
  }
  out[0] = m.s + m.c;
  out[1] = e.s + e.c;
  out[2] = dm;
}

template <typename T>
__global__ void k_min_rho(Dev<T> d, double* out) {
  const Geom& g = d.g;
  long long n = (long long)g.nx * g.ny * g.nz;
  double m = INFINITY;
  for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < n;
       t += (long long)gridDim.x * blockDim.x) {
    int i = (int)(t % g.nx);
    long long r = t / g.nx;
    int j = (int)(r % g.ny);
    int k = (int)(r / g.ny);
    double v = d.rho[idx3<T>(g, i, j, k)];
    m = v < m ? v : m;
  }
  for (int o = 16; o > 0; o >>= 1) {
    double y = __shfl_xor_sync(0xffffffffu, m, o);
    m = y < m ? y : m;
  }
  __shared__ double sm[32];
  int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  if (lane == 0) sm[wid] = m;
  __syncthreads();
  if (threadIdx.x == 0) {
    for (int w = 1; w < (int)(blockDim.x >> 5); ++w) m = sm[w] < m ? sm[w] : m;
    m = sm[0] < m ? sm[0] : m;
    // single block launch: plain store
    out[3] = m;
  }
}

// ---------------------------------------------------------------- launchers

template <typename T>
Prm<T> prm_of(const Dev<T>& d) {
  Prm<T> P;
  P.pdmb = d.pdmb; P.eps = d.eps; P.alpha = d.alpha; P.beta = d.beta; P.tvd_shift = d.tvd_shift;
  return P;
}

template <typename T, bool M>
void Launch<T, M>::bxyz_vf(const Dev<T>& d, bool want_vf, cudaStream_t st) {
  dim3 b(64, 4, 1);
  k_bxyz_vf<T, M><<<grid3(d.g.nx, d.g.ny, d.g.nz, b), b, 0, st>>>(d, want_vf ? 1 : 0);
}

template <typename T, bool M>
void Launch<T, M>::fill_bxyz(const Dev<T>& d, bool want_vf, cudaStream_t st, bool dt_next) {
  const bool dt = dt_next && !M;
  if (dt) k_next_reset<<<1, 1, 0, st>>>(d.sc);
  k_fill_bxyz<T, M, false><<<FillShape(d.g).blocks(), 256, 0, st>>>(one(d), want_vf ? 1 : 0, 0, dt ? 1 : 0);
}

template <typename T, bool M>
void Launch<T, M>::ct_fill(const Dev<T>& d, int form, double c, double den, bool want_vf, cudaStream_t st,
                           bool dt_next) {
  if constexpr (M) {  // metric mode: CT, then the fill + bxyz pass of the new half
    ct(d, form, c, den, st);
    fill_bxyz(other_half(d), want_vf, st);
  } else {
    const FillShape fs(d.g);
    static PerDevice pref_ct, pref_fill;
    prefer_carveout(k_ct_fill<T, false>, 0, pref_ct);
    prefer_carveout(k_fill_bxyz<T, false, false>, 0, pref_fill);
    k_ct_fill<T, false><<<dim3(fs.nbx, fs.nby, d.g.nz0), 256, 0, st>>>(one(d), form, (T)c, (T)den,
                                                                        want_vf ? 1 : 0, dt_next ? 1 : 0);
    k_fill_bxyz<T, false, false><<<(fs.nshell + 255) / 256, 256, 0, st>>>(one(other_half(d)), want_vf ? 1 : 0, 1,
                                                                         dt_next ? 1 : 0);
  }
}

template <typename T, bool M>
void Launch<T, M>::cfl(const Dev<T>& d, int mode, cudaStream_t st, bool save) {
  dim3 grid((d.g.nx + 31) / 32, (d.g.ny + 7) / 8, (d.g.nz + 7) / 8);
  static PerDevice pref;
  prefer_carveout(k_cfl<T, M, false>, 0, pref);
  k_cfl<T, M, false><<<grid, 256, 0, st>>>(one(d), save ? 1 : 0, 0);
  k_cfl_final<T><<<1, 1, 0, st>>>(d, mode);
}

template <typename T, bool M>
void Launch<T, M>::cfl_folded(const Dev<T>& d, int mode, bool recompute, cudaStream_t st) {
  if (recompute) {
    k_next_reset<<<1, 1, 0, st>>>(d.sc);
    dim3 grid((d.g.nx + 31) / 32, (d.g.ny + 7) / 8, (d.g.nz + 7) / 8);
    k_cfl<T, M, false><<<grid, 256, 0, st>>>(one(d), 0, 1);
  }
  k_cfl_final<T><<<1, 1, 0, st>>>(d, mode | 4);
}

template <typename T, bool M>
void Launch<T, M>::save_prev(const Dev<T>& d, cudaStream_t st) {
  k_save_prev<T><<<152 * 8, 256, 0, st>>>(d);
}

template <typename T, bool M>
void Launch<T, M>::predictor_ab(const Dev<T>& d, cudaStream_t st) {
  k_predictor_ab<T><<<152 * 8, 256, 0, st>>>(d);
}

template <typename T, int RECON, bool M>
void flux_r(const Dev<T>& d, const Inp<T>& in, cudaStream_t st) {
  Prm<T> P = prm_of(d);
  const Geom& g = d.g;
  const int n0 = (g.nx0 + 1) * g.ny0 * g.nz0, n1 = g.nx0 * (g.ny0 + 1) * g.nz0, n2 = g.nx0 * g.ny0 * (g.nz0 + 1);
  k_flux<T, RECON, 0, M, false><<<(n0 + 127) / 128, 128, 0, st>>>(one(d), in, P);
  k_flux<T, RECON, 1, M, false><<<(n1 + 127) / 128, 128, 0, st>>>(one(d), in, P);
  k_flux<T, RECON, 2, M, false><<<(n2 + 127) / 128, 128, 0, st>>>(one(d), in, P);
}

template <typename T, bool M>
void Launch<T, M>::fluxes(const Dev<T>& d, const Inp<T>& in, cudaStream_t st) {
  switch (d.recon) {
    case R_PDM: flux_r<T, R_PDM, M>(d, in, st); break;
    case R_TVD: flux_r<T, R_TVD, M>(d, in, st); break;
    case R_WENO: flux_r<T, R_WENO, M>(d, in, st); break;
    case R_MPWENO: flux_r<T, R_MPWENO, M>(d, in, st); break;
    default: flux_r<T, R_TVDMC, M>(d, in, st); break;
  }
}

// Face tiles of axis D (1: y, 2: z) with tile length TDV along the sweep.
template <typename T, int RECON, int D, bool M, int TDV>
void launch_flux_t(const Dev<T>& d, const Inp<T>& in, const Prm<T>& P, int form, T c, T den, int ab,
                   cudaStream_t st) {
  constexpr size_t sm = flux_t_smem<T, TDV>();
  static PerDevice attr;
  unsigned long long bit = 0;
  if (attr.need(bit)) {
    cudaFuncSetAttribute(k_flux_t<T, RECON, D, M, false, TDV>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
    attr.mark(bit);
  }
  const Geom& g = d.g;
  const dim3 grid = (D == 1) ? dim3((g.nx0 + 31) / 32, (g.ny0 + TDV - 1) / TDV, g.nz0)
                             : dim3((g.nx0 + 31) / 32, (g.nz0 + TDV - 1) / TDV, g.ny0);
  k_flux_t<T, RECON, D, M, false, TDV><<<grid, dim3(32, TDV + 1), sm, st>>>(one(d), in, P, form, c, den, ab);
}

// Tile lengths compiled for a (precision, reconstruction, mode): 4, 8 and 16
// for the FP32 Cartesian PDM path (chosen by the autotuner), 8 elsewhere.
template <typename T, int RECON, bool M>
constexpr bool tunable() {
  return std::is_same<T, float>::value && RECON == R_PDM && !M;
}

inline dim3 sweep_grid(int D, const Geom& g) {
  const int n0 = (D == 1) ? g.ny0 : g.nz0, no = (D == 1) ? g.nz0 : g.ny0;
  return dim3((g.nx0 + 31) / 32, (n0 + SWEEP_SEG - 1) / SWEEP_SEG, (no + 3) / 4);
}

template <typename T, int RECON, int D, bool M>
void flux_t_any(const Dev<T>& d, const Inp<T>& in, const Prm<T>& P, int form, T c, T den, int ab, cudaStream_t st) {
  if constexpr (std::is_same<T, float>::value && !M) {
    if (d.tile_td == kSweepTile) {  // column sweeps (every FP32 Cartesian reconstruction with a register window)
      static PerDevice pref;  // 4 blocks of 27 KB static shared memory
      prefer_carveout(k_flux_sweep<T, D, false, RECON>, 50, pref);
      k_flux_sweep<T, D, false, RECON><<<sweep_grid(D, d.g), dim3(32, 4), 0, st>>>(one(d), in, P, form, c, den);
      return;
    }
  }
  if constexpr (tunable<T, RECON, M>()) {
    if (d.tile_td == 4) return launch_flux_t<T, RECON, D, M, 4>(d, in, P, form, c, den, ab, st);
    if (d.tile_td == 16) return launch_flux_t<T, RECON, D, M, 16>(d, in, P, form, c, den, ab, st);
  }
  launch_flux_t<T, RECON, D, M, TD>(d, in, P, form, c, den, ab, st);
}

template <typename T, int RECON, bool M>
void hydro_r(const Dev<T>& d, const Inp<T>& in, int part, int form, double c, double den, bool ab,
             cudaStream_t st) {
  Prm<T> P = prm_of(d);
  const Geom& g = d.g;
  if (part == 0) {
    const int n0 = (g.nx0 + 1) * g.ny0 * g.nz0;
    static PerDevice pref;
    prefer_carveout(k_flux<T, RECON, 0, M, false>, 0, pref);
    k_flux<T, RECON, 0, M, false><<<(n0 + 127) / 128, 128, 0, st>>>(one(d), in, P);
  } else if (part == 1) {
    flux_t_any<T, RECON, 1, M>(d, in, P, -1, T(0), T(1), 0, st);
  } else {
    flux_t_any<T, RECON, 2, M>(d, in, P, form, (T)c, (T)den, ab ? 1 : 0, st);
  }
}

template <typename T, bool M>
void Launch<T, M>::hydro(const Dev<T>& d, const Inp<T>& in, int part, int form, double c, double den, bool ab,
                         cudaStream_t st) {
  switch (d.recon) {
    case R_PDM: hydro_r<T, R_PDM, M>(d, in, part, form, c, den, ab, st); break;
    case R_TVD: hydro_r<T, R_TVD, M>(d, in, part, form, c, den, ab, st); break;
    case R_WENO: hydro_r<T, R_WENO, M>(d, in, part, form, c, den, ab, st); break;
    case R_MPWENO: hydro_r<T, R_MPWENO, M>(d, in, part, form, c, den, ab, st); break;
    default: hydro_r<T, R_TVDMC, M>(d, in, part, form, c, den, ab, st); break;
  }
}

// ------------------------------------------------------------- Yee EMF
// get_eijk_Yee (mhd3d3.f90:1654-1752).  First the 12 split electric fields
// of every cell, ghosts included, from the Gaussian moments of get_v_center
// (2562-2592, the get_v_face element formula):
//   ez_ab = bx vx0a vy1b - by vx1a vy0b, ex_ab = by vy0a vz1b - bz vy1a vz0b,
//   ey_ab = bz vz0a vx1b - bx vz1a vx0b   (a, b = + / - moments),
// stored as ye[f * 4 + s], f = x, y, z edges, s = pp, np, pn, nn.
template <typename T>
__global__ void k_yee_split(Dev<T> d, Inp<T> in) {
  const Geom& g = d.g;
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const int j = blockIdx.y * blockDim.y + threadIdx.y;
  const int k = blockIdx.z;
  if (i >= g.nx || j >= g.ny || k >= g.nz) return;
  const int c = i + g.px * (j + g.py * k);
  const T bxc = in.bx[c], byc = in.by[c], bzc = in.bz[c];
  const T bsq = bxc * bxc + byc * byc + bzc * bzc;
  const T lam = Ops<T>::dv(in.rho[c], T(2) * in.p[c] + bsq);
  T x0p, x0n, x1p, x1n, y0p, y0n, y1p, y1n, z0p, z0n, z1p, z1n;
  Moments<T>::hydro(lam, in.vx[c], true, x0p, x1p);
  Moments<T>::hydro(lam, in.vx[c], false, x0n, x1n);
  Moments<T>::hydro(lam, in.vy[c], true, y0p, y1p);
  Moments<T>::hydro(lam, in.vy[c], false, y0n, y1n);
  Moments<T>::hydro(lam, in.vz[c], true, z0p, z1p);
  Moments<T>::hydro(lam, in.vz[c], false, z0n, z1n);
  d.ye[0][c] = byc * y0p * z1p - bzc * y1p * z0p;
  d.ye[1][c] = byc * y0n * z1p - bzc * y1n * z0p;
  d.ye[2][c] = byc * y0p * z1n - bzc * y1p * z0n;
  d.ye[3][c] = byc * y0n * z1n - bzc * y1n * z0n;
  d.ye[4][c] = bzc * z0p * x1p - bxc * z1p * x0p;
  d.ye[5][c] = bzc * z0n * x1p - bxc * z1n * x0p;
  d.ye[6][c] = bzc * z0p * x1n - bxc * z1p * x0n;
  d.ye[7][c] = bzc * z0n * x1n - bxc * z1n * x0n;
  d.ye[8][c] = bxc * x0p * y1p - byc * x1p * y0p;
  d.ye[9][c] = bxc * x0n * y1p - byc * x1n * y0p;
  d.ye[10][c] = bxc * x0p * y1n - byc * x1p * y0n;
  d.ye[11][c] = bxc * x0n * y1n - byc * x1n * y0n;
}

// Then, per edge of family E, each split field is reconstructed to the edge
// in two passes -- along axis DA to the edge's DA face (first index of the
// field), at the rows of the DB stencil, then along DB to its DB face (second
// index) -- taking the left state for a + moment and the right one for a -
// moment; the edge EMF is epp + enp + epn + enn.  ei: y then z, ej: z then x,
// ek: x then y (reconstruct_3d dirs 5/6, 6/4, 4/5).  Only the rows the
// second pass reads are reconstructed in the first.
template <typename T, int RECON, int E>
__global__ void k_emf_yee(Dev<T> d, Prm<T> P) {
  const Geom& g = d.g;
  const int i = blockIdx.x * blockDim.x + threadIdx.x + g.ng;
  const int j = blockIdx.y * blockDim.y + threadIdx.y + g.ng;
  const int k = blockIdx.z + g.ng;
  const int ni = g.nx0 + (E != 0), nj = g.ny0 + (E != 1), nk = g.nz0 + (E != 2);
  if (i >= g.ng + ni || j >= g.ng + nj || k >= g.ng + nk) return;
  const int c = i + g.px * (j + g.py * k);
  const int st[3] = {1, g.px, (int)g.plane};
  constexpr int DA = (E == 0) ? 1 : (E == 1) ? 2 : 0;
  constexpr int DB = (E == 0) ? 2 : (E == 1) ? 0 : 1;
  const int sA = st[DA], sB = st[DB];
  constexpr bool TV = (RECON == R_TVD || RECON == R_TVDMC);
  constexpr int M0 = (RECON == R_PDM) ? 0 : TV ? 2 : 1;
  constexpr int M1 = (RECON == R_PDM) ? 7 : TV ? 5 : 6;
  T part[4];
#pragma unroll
  for (int s = 0; s < 4; ++s) {  // pp, np, pn, nn
    const T* f = d.ye[E * 4 + s];
    const bool left1 = (s == 0 || s == 2), left2 = (s < 2);
    T q[8];
#pragma unroll
    for (int m = 0; m < 8; ++m) {
      q[m] = T(0);
      if (m >= M0 && m <= M1) {
        T l, r;
        recon_face<T, RECON>(f, c + (m - 4) * sB, sA, P, l, r);
        q[m] = left1 ? l : r;
      }
    }
    T l, r;
    recon_win<T, RECON, 0>(q, P, l, r);
    part[s] = left2 ? l : r;
  }
  d.E[E][c] = part[0] + part[1] + part[2] + part[3];
}

template <typename T, int RECON>
void emf_yee_r(const Dev<T>& d, const Inp<T>& in, cudaStream_t st) {
  const Prm<T> P = prm_of(d);
  const Geom& g = d.g;
  const dim3 b(32, 4, 1);
  k_yee_split<T><<<grid3(g.nx, g.ny, g.nz, b), b, 0, st>>>(d, in);
  k_emf_yee<T, RECON, 0><<<grid3(g.nx0, g.ny0 + 1, g.nz0 + 1, b), b, 0, st>>>(d, P);
  k_emf_yee<T, RECON, 1><<<grid3(g.nx0 + 1, g.ny0, g.nz0 + 1, b), b, 0, st>>>(d, P);
  k_emf_yee<T, RECON, 2><<<grid3(g.nx0 + 1, g.ny0 + 1, g.nz0, b), b, 0, st>>>(d, P);
}

template <typename T>
void emf_yee(const Dev<T>& d, const Inp<T>& in, cudaStream_t st) {
  switch (d.recon) {
    case R_PDM: emf_yee_r<T, R_PDM>(d, in, st); break;
    case R_TVD: emf_yee_r<T, R_TVD>(d, in, st); break;
    case R_WENO: emf_yee_r<T, R_WENO>(d, in, st); break;
    case R_MPWENO: emf_yee_r<T, R_MPWENO>(d, in, st); break;
    default: emf_yee_r<T, R_TVDMC>(d, in, st); break;
  }
}

// ei tiles of 32 (FP32) or 16 (FP64) edges x 4 x 4; ej, ek plane tiles of 32 x 8.
template <typename T, int RECON, bool M>
void emf_weno(const Dev<T>& d, const Inp<T>& in, cudaStream_t st) {
  const Prm<T> P = prm_of(d);
  constexpr int EX = std::is_same<T, float>::value ? 32 : 16;
  launch_emf_weno<T, RECON, 0, EX, 4, 4, EX * 16, M>(d, in, P, st);
  launch_emf_weno<T, RECON, 1, 32, 1, 8, 256, M>(d, in, P, st);
  launch_emf_weno<T, RECON, 2, 32, 8, 1, 256, M>(d, in, P, st);
}

template <typename T, int RECON, bool M>
void emf_r(const Dev<T>& d, const Inp<T>& in, cudaStream_t st) {
  Prm<T> P = prm_of(d);
  dim3 b(32, 4, 1);
  const Geom& g = d.g;
  k_emf<T, RECON, 0, M><<<grid3(g.nx0, g.ny0 + 1, g.nz0 + 1, b), b, 0, st>>>(d, in, P);
  k_emf<T, RECON, 1, M><<<grid3(g.nx0 + 1, g.ny0, g.nz0 + 1, b), b, 0, st>>>(d, in, P);
  k_emf<T, RECON, 2, M><<<grid3(g.nx0 + 1, g.ny0 + 1, g.nz0, b), b, 0, st>>>(d, in, P);
}

// ei tile cross-section: 8 x 8 edges in FP32, 4 x 4 in FP64; its length along
// the edge axis is ei_x() below.
#ifndef MHD_EI_TILE
#define MHD_EI_TILE 8
#endif
template <typename T> struct EiTile { static constexpr int Y = MHD_EI_TILE; };
// Edge-axis length of the 8 x 8 ei tile (the 4 x 4 tile stays 32 long): 16
// halves its 96 KB of shared memory, so 4 blocks (full occupancy) fit an SM;
// measured 2 % faster for the EMF family than 32 at 256^3.
#ifndef MHD_EI_X
#define MHD_EI_X 16
#endif
constexpr int ei_x(int y) { return y == 8 ? MHD_EI_X : 32; }
template <> struct EiTile<double> { static constexpr int Y = 4; };

template <typename T, bool M>
void Launch<T, M>::emf(const Dev<T>& d, const Inp<T>& in0, cudaStream_t st) {
  if constexpr (!M) {  // Yee: Cartesian only (checked at mhd_init)
    if (d.emf == EMF_YEE) {
      emf_yee<T>(d, in0, st);
      return;
    }
  }
  Inp<T> in = in0;
  if (M) {
    // normal velocities and face-normal field of the stage input, in the
    // places of v and bi/bj/bk
    dim3 b(64, 4, 1);
    k_metric_prep<T><<<grid3(d.g.nx + 1, d.g.ny + 1, d.g.nz + 1, b), b, 0, st>>>(d, in0);
    in.vx = d.mw[0]; in.vy = d.mw[1]; in.vz = d.mw[2];
    in.bi = d.mbn[0]; in.bj = d.mbn[1]; in.bk = d.mbn[2];
  }
  if (d.recon == R_PDM) {
    Prm<T> P = prm_of(d);
    if constexpr (std::is_same<T, float>::value && !M) {
      if (d.tile_ey == kEmfStream) {
        emf_pdm_stream<T, M>(d, in, P, st);
        return;
      }
    }
    if (std::is_same<T, float>::value && !M && d.tile_ey == 4)
      launch_emf_pdm<T, 0, 32, 4, 4, 512, M>(d, in, P, st);
    else
      launch_emf_pdm<T, 0, ei_x(EiTile<T>::Y), EiTile<T>::Y, EiTile<T>::Y, 512, M>(d, in, P, st);
    launch_emf_pdm<T, 1, 32, 1, kPT, 32 * kPT, M>(d, in, P, st);
    launch_emf_pdm<T, 2, 32, kPT, 1, 32 * kPT, M>(d, in, P, st);
    return;
  }
  switch (d.recon) {
    case R_TVD: emf_r<T, R_TVD, M>(d, in, st); break;
    case R_WENO: emf_weno<T, R_WENO, M>(d, in, st); break;
    case R_MPWENO: emf_weno<T, R_MPWENO, M>(d, in, st); break;
    default: emf_r<T, R_TVDMC, M>(d, in, st); break;
  }
}

template <typename T, bool M>
void Launch<T, M>::ct(const Dev<T>& d, int form, double c, double den, cudaStream_t st) {
  dim3 b(32, 4, 1);
  const Geom& g = d.g;
  k_update_b<T, M, false><<<grid3(g.nx0 + 1, g.ny0 + 1, g.nz0 + 1, b), b, 0, st>>>(one(d), form, (T)c, (T)den);
}

template <typename T, bool M>
void Launch<T, M>::fill(const Dev<T>& d, cudaStream_t st) {
  dim3 b(64, 4, 1);
  k_fill<T><<<grid3(d.g.nx + 1, d.g.ny + 1, d.g.nz + 1, b), b, 0, st>>>(d);
}

// ------------------------------------------------------------ batched ensemble
template <typename T>
dim3 Batch<T>::dims(int fam, const Geom& g, int td, int ey) {
  const bool stream = std::is_same<T, float>::value && ey == kEmfStream;
  const int Y = std::is_same<T, float>::value && !stream ? ey : EiTile<T>::Y;
  if (!std::is_same<T, float>::value) td = TD;
  switch (fam) {
    case BF_CFL: return dim3((g.nx + 31) / 32, (g.ny + 7) / 8, (g.nz + 7) / 8);
    case BF_FLUX_X: return dim3(((g.nx0 + 1) * g.ny0 * g.nz0 + 127) / 128, 1, 1);
    case BF_FLUX_Y: return td == kSweepTile ? sweep_grid(1, g) : dim3((g.nx0 + 31) / 32, (g.ny0 + td - 1) / td, g.nz0);
    case BF_FLUX_Z: return td == kSweepTile ? sweep_grid(2, g) : dim3((g.nx0 + 31) / 32, (g.nz0 + td - 1) / td, g.ny0);
    case BF_EMF_I: return stream ? emf_stream_grid(0, g) : emf_grid(0, g, ei_x(Y), Y, Y);
    case BF_EMF_J: return stream ? emf_stream_grid(1, g) : emf_grid(1, g, 32, 1, kPT);
    case BF_EMF_K: return stream ? emf_stream_grid(2, g) : emf_grid(2, g, 32, kPT, 1);
    case BF_EMF_R: return stream ? dim3(EmfRows(g).blocks(), 1, 1) : dim3(0, 0, 0);
    case BF_CT: {  // k_ct_fill: the fill's interior tiles
      const FillShape fs(g);
      return dim3(fs.nbx, fs.nby, g.nz0);
    }
    default: return dim3((FillShape(g).nshell + 255) / 256, 1, 1);  // BF_FILL: the shell of the new half
  }
}

template <typename T>
void Batch<T>::cfl(const BatchView& v, int sel, int mode, cudaStream_t st) {
  KArg<T, true> a{(const Dev<T>*)v.tab[sel], v.map[BF_CFL]};
  k_cfl<T, false, true><<<v.nblk[BF_CFL], 256, 0, st>>>(a, 1, 0);
  k_cfl_final_batch<T><<<(v.ngrids + 127) / 128, 128, 0, st>>>((const Dev<T>*)v.tab[sel], v.ngrids, mode);
}

template <typename K>
void set_smem(K kernel, size_t bytes) {
  cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes);
}

// Batched EMF families with ei tile Y (edges along y and z per block).
template <typename T, int Y>
void batch_emf(const BatchView& v, const Dev<T>* tab, const Prm<T>& P, cudaStream_t st) {
  constexpr int X = ei_x(Y);
  constexpr size_t si = emf_pdm_smem<T, 0, X, Y, Y>();
  constexpr size_t sj = emf_pdm_smem<T, 1, 32, 1, kPT>();
  constexpr size_t sk = emf_pdm_smem<T, 2, 32, kPT, 1>();
  static PerDevice attr;
  unsigned long long bit = 0;
  if (attr.need(bit)) {
    set_smem(k_emf_pdm<T, 0, X, Y, Y, 512, false, true>, si);
    set_smem(k_emf_pdm<T, 1, 32, 1, kPT, 32 * kPT, false, true>, sj);
    set_smem(k_emf_pdm<T, 2, 32, kPT, 1, 32 * kPT, false, true>, sk);
    attr.mark(bit);
  }
  const Inp<T> none{};
  k_emf_pdm<T, 0, X, Y, Y, 512, false, true><<<v.nblk[BF_EMF_I], 512, si, st>>>(
      KArg<T, true>{tab, v.map[BF_EMF_I]}, none, P);
  k_emf_pdm<T, 1, 32, 1, kPT, 32 * kPT, false, true><<<v.nblk[BF_EMF_J], 32 * kPT, sj, st>>>(
      KArg<T, true>{tab, v.map[BF_EMF_J]}, none, P);
  k_emf_pdm<T, 2, 32, kPT, 1, 32 * kPT, false, true><<<v.nblk[BF_EMF_K], 32 * kPT, sk, st>>>(
      KArg<T, true>{tab, v.map[BF_EMF_K]}, none, P);
}

// Batched slice-streamed EMF families and their boundary rows.
template <typename T>
void batch_emf_stream(const BatchView& v, const Dev<T>* tab, const Prm<T>& P, cudaStream_t st) {
  stream_attr<T, 0, false, true>();
  stream_attr<T, 1, false, true>();
  stream_attr<T, 2, false, true>();
  const Inp<T> none{};
  constexpr int NT = 32 * MHD_EMF_NW;
  k_emf_stream<T, 0, MHD_EMF_NW, false, true><<<v.nblk[BF_EMF_I], NT, EmfStream<T, 0, MHD_EMF_NW>::smem, st>>>(
      KArg<T, true>{tab, v.map[BF_EMF_I]}, none, P);
  k_emf_stream<T, 1, MHD_EMF_NW, false, true><<<v.nblk[BF_EMF_J], NT, EmfStream<T, 1, MHD_EMF_NW>::smem, st>>>(
      KArg<T, true>{tab, v.map[BF_EMF_J]}, none, P);
  k_emf_stream<T, 2, MHD_EMF_NW, false, true><<<v.nblk[BF_EMF_K], NT, EmfStream<T, 2, MHD_EMF_NW>::smem, st>>>(
      KArg<T, true>{tab, v.map[BF_EMF_K]}, none, P);
  k_emf_rows<T, false, true><<<v.nblk[BF_EMF_R], 256, emf_rows_smem<T>(), st>>>(
      KArg<T, true>{tab, v.map[BF_EMF_R]}, none, P);
}

// Batched y / z face tiles of length TDV.
template <typename T, int TDV>
void batch_flux_t(const BatchView& v, const Dev<T>* tab, const Prm<T>& P, int form, T c, T den, cudaStream_t st) {
  constexpr size_t sf = flux_t_smem<T, TDV>();
  static PerDevice attr;
  unsigned long long bit = 0;
  if (attr.need(bit)) {
    set_smem(k_flux_t<T, R_PDM, 1, false, true, TDV>, sf);
    set_smem(k_flux_t<T, R_PDM, 2, false, true, TDV>, sf);
    attr.mark(bit);
  }
  const Inp<T> none{};
  k_flux_t<T, R_PDM, 1, false, true, TDV><<<v.nblk[BF_FLUX_Y], dim3(32, TDV + 1), sf, st>>>(
      KArg<T, true>{tab, v.map[BF_FLUX_Y]}, none, P, -1, T(0), T(1), 0);
  k_flux_t<T, R_PDM, 2, false, true, TDV><<<v.nblk[BF_FLUX_Z], dim3(32, TDV + 1), sf, st>>>(
      KArg<T, true>{tab, v.map[BF_FLUX_Z]}, none, P, form, c, den, 0);
}

template <typename T>
void Batch<T>::parts(const BatchView& v, int sel, int which, int form, double c, double den, cudaStream_t st) {
  const Dev<T>* tab = (const Dev<T>*)v.tab[sel];
  // the batch shares the deck's limiter constants (checked when it is built)
  Prm<T> P;
  P.pdmb = (T)v.pdmb; P.eps = (T)v.eps; P.alpha = (T)v.alpha; P.beta = (T)v.beta; P.tvd_shift = v.tvd_shift;
  constexpr bool F32 = std::is_same<T, float>::value;
  if (which & 1) {  // EMF families
    if constexpr (F32) {
      if (v.tile_ey == kEmfStream) {
        batch_emf_stream<T>(v, tab, P, st);
        return parts(v, sel, which & ~1, form, c, den, st);
      }
    }
    if (F32 && v.tile_ey == 4) batch_emf<T, 4>(v, tab, P, st);
    else batch_emf<T, EiTile<T>::Y>(v, tab, P, st);
  }
  if (which & 2) {  // face fluxes and the conserved update
    const Inp<T> none{};
    k_flux<T, R_PDM, 0, false, true><<<v.nblk[BF_FLUX_X], 128, 0, st>>>(KArg<T, true>{tab, v.map[BF_FLUX_X]}, none,
                                                                       P);
    if (F32 && v.tile_td == kSweepTile) {
      k_flux_sweep<T, 1, true><<<v.nblk[BF_FLUX_Y], dim3(32, 4), 0, st>>>(KArg<T, true>{tab, v.map[BF_FLUX_Y]}, none,
                                                                           P, -1, T(0), T(1));
      k_flux_sweep<T, 2, true><<<v.nblk[BF_FLUX_Z], dim3(32, 4), 0, st>>>(KArg<T, true>{tab, v.map[BF_FLUX_Z]}, none,
                                                                           P, form, (T)c, (T)den);
    } else if (F32 && v.tile_td == 4) batch_flux_t<T, F32 ? 4 : TD>(v, tab, P, form, (T)c, (T)den, st);
    else if (F32 && v.tile_td == 16) batch_flux_t<T, F32 ? 16 : TD>(v, tab, P, form, (T)c, (T)den, st);
    else batch_flux_t<T, TD>(v, tab, P, form, (T)c, (T)den, st);
  }
  if (which & 4) {  // face-B update + bxyz + vf (interior), then the ghost shell of the half the stage wrote
    k_ct_fill<T, true><<<v.nblk[BF_CT], 256, 0, st>>>(KArg<T, true>{tab, v.map[BF_CT]}, form, (T)c, (T)den, 1, 0);
    KArg<T, true> fa{(const Dev<T>*)v.tab[sel ^ 1], v.map[BF_FILL]};
    k_fill_bxyz<T, false, true><<<v.nblk[BF_FILL], 256, 0, st>>>(fa, 1, 1, 0);
  }
}

template <typename T>
void Batch<T>::stage(const BatchView& v, int sel, int form, double c, double den, cudaStream_t st) {
  parts(v, sel, 7, form, c, den, st);
}

template <typename T, bool M>
void Launch<T, M>::diagnostics(const Dev<T>& d, double* out, cudaStream_t st) {
  // out: device buffer of 5 + 5*nb doubles; out[4] (CFL dt) is filled by the caller
  const int nb = 152 * 2;
  double* part = out + 8;
  k_diag_partial<T, M><<<nb, 256, 0, st>>>(d, part);
  k_diag_final<T><<<1, 1, 0, st>>>(d, part, nb, out);
  k_min_rho<T><<<1, 1024, 0, st>>>(d, out);
}

}  // namespace mhd
