// BF16 tensor-core (tcgen05) kernels of the learned coarse-grid correction:
// a per-cell MLP 256 -> 64 -> 64 -> 16 (GELU), of which 216 inputs (a 3x3x3
// stencil of the 8 conserved variables, normalised) and 8 outputs are used.
// Training (forward, backward, weight gradients) and inference run on the
// 5th-generation tensor cores with FP32 accumulators in TMEM; the optimiser
// (Adam) and the bias gradients run on the CUDA cores.
#include <cuda_runtime.h>
#include <cuda_bf16.h>
#include <math.h>
#include <stdint.h>
#include <string>

#include "../../include/mhd_gpu.h"
#include "mhd_state.h"
#include "tc_sm100.cuh"

namespace mhd {
namespace {

// ------------------------------------------------------- GEMM primitive
// C[M x N] = A[M x K] B[N x K]^T, BF16 operands (row-major, K contiguous),
// FP32 result.  One CTA of 128 threads per 128-row tile; the whole K extent
// is staged in shared memory.  N multiple of 16 (<= 256), K multiple of 16
// (<= 256).  err[0] is set when a bounded wait gave up.
__global__ void __launch_bounds__(128) k_tc_gemm(const __nv_bfloat16* __restrict__ A,
                                                 const __nv_bfloat16* __restrict__ B, float* __restrict__ C, int M,
                                                 int N, int K, int ncols, int* err) {
  extern __shared__ __align__(1024) unsigned char smem[];
  __shared__ __align__(8) uint64_t bar;
  __shared__ uint32_t tslot;
  unsigned char* sa = smem;                // 128 x K
  unsigned char* sb = smem + 128 * K * 2;  // N x K
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int row0 = blockIdx.x * 128;
  if (warp == 0) tc::tmem_alloc(&tslot, (uint32_t)ncols);
  if (tid == 0) tc::bar_init(&bar, 1);
  // stage A (zero rows past M) and B, 8 elements (one core-matrix row) per copy
  const int ka = K / 8;
  for (int t = tid; t < 128 * ka; t += 128) {
    const int r = t / ka, k8 = (t % ka) * 8;
    uint4 v = make_uint4(0, 0, 0, 0);
    if (row0 + r < M) v = *reinterpret_cast<const uint4*>(A + (size_t)(row0 + r) * K + k8);
    *reinterpret_cast<uint4*>(sa + tc::kmaj(r, k8, K)) = v;
  }
  for (int t = tid; t < N * ka; t += 128) {
    const int r = t / ka, k8 = (t % ka) * 8;
    *reinterpret_cast<uint4*>(sb + tc::kmaj(r, k8, K)) = *reinterpret_cast<const uint4*>(B + (size_t)r * K + k8);
  }
  tc::fence_smem();
  tc::fence_before();
  __syncthreads();
  tc::fence_after();
  const uint32_t tbase = tslot;
  if (tid == 0) {
    const uint32_t a0 = tc::smem_u32(sa), b0 = tc::smem_u32(sb);
    const uint32_t id = tc::idesc_bf16(128, N);
    for (int kk = 0; kk < K / 16; ++kk) tc::mma(tbase, tc::tile_desc(a0, K, kk), tc::tile_desc(b0, K, kk), id, kk > 0);
    tc::commit(&bar);
  }
  __syncwarp();
  const bool ok = tc::bar_wait(&bar, 0);
  tc::fence_after();
  if (!ok) {
    if (lane == 0) atomicExch(err, 1);
    tc::bar_wait(&bar, 0);  // a second bounded wait for MMAs still in flight
  } else {
    const int r = row0 + warp * 32 + lane;
    for (int c0 = 0; c0 < N; c0 += 16) {
      float v[16];
      tc::tmem_ld16(tc::tmem_at(tbase, warp, c0), v);
      if (r < M)
        for (int i = 0; i < 16; ++i) C[(size_t)r * N + c0 + i] = v[i];
    }
  }
  tc::fence_before();
  __syncthreads();
  if (warp == 0) tc::tmem_free(tbase, (uint32_t)ncols);
}

// ------------------------------------------------------------------ MLP
constexpr int FIN = 256, NH = 64, NO = 16, NOUT = 8;
// flat FP32 parameter vector: W1[64][256] b1[64] W2[64][64] b2[64] W3[16][64] b3[16]
constexpr int OW1 = 0, OB1 = OW1 + NH * FIN, OW2 = OB1 + NH, OB2 = OW2 + NH * NH, OW3 = OB2 + NH,
              OB3 = OW3 + NO * NH, NPARAM = OB3 + NO;

// shared-memory map of the training kernel (bytes)
constexpr int S_W1 = 0, S_W2 = S_W1 + NH * FIN * 2, S_W2T = S_W2 + NH * NH * 2, S_W3 = S_W2T + NH * NH * 2,
              S_W3T = S_W3 + NO * NH * 2, S_R1 = S_W3T + NH * NO * 2, S_XT = S_R1 + 128 * FIN * 2,
              S_H1 = S_XT + FIN * 128 * 2, S_H2 = S_H1 + 128 * NH * 2, S_TOTAL = S_H2 + 128 * NH * 2;
// backward buffers inside R1 (the X tile is consumed by the first MMA):
// H^T stacks H1^T (rows 0..63) over H2^T (rows 64..127)
constexpr int R_HT = 0, R_DY = R_HT + 128 * 128 * 2, R_DYT = R_DY + 128 * NO * 2, R_DZ2 = R_DYT + NO * 128 * 2;
static_assert(R_DZ2 + 128 * NH * 2 <= 128 * FIN * 2, "backward buffers exceed the X tile");
// TMEM columns
constexpr uint32_t T_D1 = 0, T_D2 = 64, T_D3 = 128, T_DH2 = 160, T_DH1 = 224, T_G1A = 288, T_G1B = 352, T_G2 = 416,
                   T_G3 = 480, T_COLS = 512;

struct MlpW {
  const __nv_bfloat16 *w1, *w2, *w2t, *w3, *w3t;  // BF16 copies (row-major)
  const float* p;                                 // FP32 parameters (biases read from here)
};

// Division by a grid extent d >= 1 with a multiplier and shift computed on
// the host (the round-up method of Granlund & Montgomery, 1994): q =
// (umulhi(n, m) + n) >> l with l = ceil(log2 d) and m = 2^32 (2^l - d) / d + 1,
// exact for 0 <= n < 2^31 (the sum then stays below 2^32).
struct FastDiv {
  uint32_t m = 0;
  int l = 0;
  FastDiv() = default;
  explicit FastDiv(int d) {
    while ((1ull << l) < (unsigned long long)d) ++l;
    m = (uint32_t)(((1ull << 32) * ((1ull << l) - (unsigned long long)d)) / (unsigned long long)d + 1ull);
  }
  __device__ __forceinline__ uint32_t div(uint32_t n) const { return (__umulhi(n, m) + n) >> l; }
};
// interior cell index t -> (i, j, k) of an nx0 x ny0 x nz0 grid
struct CellMap {
  FastDiv by_nx, by_ny;
};
inline CellMap cell_map(const Geom& g) { return CellMap{FastDiv(g.nx0), FastDiv(g.ny0)}; }

// tanh on the SFU (PTX tanh.approx.f32, sm_75+; maximum relative error about
// 2^-11, below the BF16 rounding the activations take next).
__device__ __forceinline__ float tanh_sfu(float x) {
  float y;
  asm("tanh.approx.f32 %0, %1;" : "=f"(y) : "f"(x));
  return y;
}

// GELU, tanh form (Hendrycks & Gimpel), and its derivative in dg.
__device__ __forceinline__ float gelu_t(float z, float& dg) {
  const float c = 0.7978845608028654f, a = 0.044715f;
  const float u = c * (z + a * z * z * z);
  const float t = tanh_sfu(u);
  dg = 0.5f * (1.0f + t) + 0.5f * z * (1.0f - t * t) * c * (1.0f + 3.0f * a * z * z);
  return 0.5f * z * (1.0f + t);
}

// GELU of the 16 accumulators z[0..16) of row r, columns c0.. (+ bias),
// rounded to BF16 and stored as two 16-byte core-matrix rows of the K-major
// [128 x NH] activation tile.
__device__ __forceinline__ void gelu16_store(unsigned char* tile, int r, int c0, const float* z,
                                             const float* __restrict__ bias) {
#pragma unroll
  for (int h = 0; h < 2; ++h) {
    uint32_t pk[4];
#pragma unroll
    for (int a = 0; a < 4; ++a) {
      float d0, d1;
      const int i = 8 * h + 2 * a;
      const __nv_bfloat162 v = __floats2bfloat162_rn(gelu_t(z[i] + bias[c0 + i], d0),
                                                     gelu_t(z[i + 1] + bias[c0 + i + 1], d1));
      pk[a] = *reinterpret_cast<const uint32_t*>(&v);
    }
    *reinterpret_cast<uint4*>(tile + tc::kmaj(r, c0 + 8 * h, NH)) = make_uint4(pk[0], pk[1], pk[2], pk[3]);
  }
}

// The inference epilogue of gelu16_store on the packed FP32 pipe: GELU (tanh
// form) of two accumulators plus their biases (bias pairs from shared memory),
// rounded to BF16 as one pair.  gelu_t's value with its constants folded:
// u = c z + (c a) z^3 = z (c + (c a) z^2), GELU = h z + h z t (h = 1/2).
__device__ __forceinline__ uint32_t gelu2_bf16(float2 z, float2 b) {
  const float2 c = make_float2(0.7978845608028654f, 0.7978845608028654f);
  const float2 ca = make_float2(0.7978845608028654f * 0.044715f, 0.7978845608028654f * 0.044715f);
  const float2 h = make_float2(0.5f, 0.5f);
  z = __fadd2_rn(z, b);
  const float2 u = __fmul2_rn(z, __ffma2_rn(ca, __fmul2_rn(z, z), c));
  const float2 t = make_float2(tanh_sfu(u.x), tanh_sfu(u.y));
  const float2 hz = __fmul2_rn(h, z);
  const float2 g = __ffma2_rn(hz, t, hz);
  const __nv_bfloat162 v = __floats2bfloat162_rn(g.x, g.y);
  return *reinterpret_cast<const uint32_t*>(&v);
}
__device__ __forceinline__ void gelu16_store_sm(unsigned char* tile, int r, int c0, const float* z,
                                                const float* sbias) {
#pragma unroll
  for (int h = 0; h < 2; ++h) {
    const float4 b0 = *reinterpret_cast<const float4*>(sbias + c0 + 8 * h);
    const float4 b1 = *reinterpret_cast<const float4*>(sbias + c0 + 8 * h + 4);
    const float* zz = z + 8 * h;
    const uint32_t p0 = gelu2_bf16(make_float2(zz[0], zz[1]), make_float2(b0.x, b0.y));
    const uint32_t p1 = gelu2_bf16(make_float2(zz[2], zz[3]), make_float2(b0.z, b0.w));
    const uint32_t p2 = gelu2_bf16(make_float2(zz[4], zz[5]), make_float2(b1.x, b1.y));
    const uint32_t p3 = gelu2_bf16(make_float2(zz[6], zz[7]), make_float2(b1.z, b1.w));
    *reinterpret_cast<uint4*>(tile + tc::kmaj(r, c0 + 8 * h, NH)) = make_uint4(p0, p1, p2, p3);
  }
}

// Copy a row-major [R x K] BF16 matrix into a K-major canonical tile.
__device__ __forceinline__ void stage_w(unsigned char* dst, const __nv_bfloat16* src, int R, int K) {
  const int k8n = K / 8;
  for (int t = threadIdx.x; t < R * k8n; t += blockDim.x) {
    const int r = t / k8n, k8 = (t % k8n) * 8;
    *reinterpret_cast<uint4*>(dst + tc::kmaj(r, k8, K)) = *reinterpret_cast<const uint4*>(src + (size_t)r * K + k8);
  }
}

// All threads: make generic smem writes visible to the MMA, then sync.
__device__ __forceinline__ void publish() {
  tc::fence_smem();
  tc::fence_before();
  __syncthreads();
  tc::fence_after();
}

// thread 0: D[128 x N] (+)= A[128 x K] B[N x K]^T from canonical tiles
__device__ __forceinline__ void gemm(uint32_t d, uint32_t a, uint32_t b, int N, int K, bool acc) {
  const uint32_t id = tc::idesc_bf16(128, N);
  for (int kk = 0; kk < K / 16; ++kk)
    tc::mma(d, tc::tile_desc(a, K, kk), tc::tile_desc(b, K, kk), id, (acc || kk > 0) ? 1u : 0u);
}

// One training pass over `count` samples idx[0..count): accumulates the
// gradient of loss = mean over samples and outputs of (y - t)^2 into grad
// (FP32, parameter layout) and the loss sum into *loss.  Persistent CTAs of
// 128 threads, one 128-sample tile at a time; thread r owns sample row r and
// reads TMEM lane r.
__global__ void __launch_bounds__(128, 1)
    k_mlp_train(const __nv_bfloat16* __restrict__ X, const float* __restrict__ T, const int* __restrict__ idx,
                int count, float gscale, MlpW w, float* __restrict__ grad, float* __restrict__ loss, int* err) {
  extern __shared__ __align__(1024) unsigned char sm[];
  __shared__ __align__(8) uint64_t bar;
  __shared__ uint32_t tslot;
  __shared__ float red[4][NH], red1[4][NH];  // per-warp bias-gradient sums (dZ2, dZ1 phases)
  const int tid = threadIdx.x, q = tid >> 5, lane = tid & 31;
  if (q == 0) tc::tmem_alloc(&tslot, T_COLS);
  if (tid == 0) tc::bar_init(&bar, 1);
  stage_w(sm + S_W1, w.w1, NH, FIN);
  stage_w(sm + S_W2, w.w2, NH, NH);
  stage_w(sm + S_W2T, w.w2t, NH, NH);
  stage_w(sm + S_W3, w.w3, NO, NH);
  stage_w(sm + S_W3T, w.w3t, NH, NO);
  publish();
  const uint32_t tb = tslot;
  const uint32_t s0 = tc::smem_u32(sm);
  unsigned char* R1 = sm + S_R1;
  unsigned char* XT = sm + S_XT;
  const float* b1 = w.p + OB1;
  const float* b2 = w.p + OB2;
  const float* b3 = w.p + OB3;
  uint32_t ph = 0;
  bool ok = true, any = false;
  float lsum = 0.0f;
  auto sync_mma = [&]() {  // every thread calls it; `ok` ends up the same in all of them
    if (tid == 0) tc::commit(&bar);
    __syncwarp();
    if (ok) ok = tc::bar_wait(&bar, ph);
    ok = __syncthreads_and(ok) != 0;
    ph ^= 1u;
    tc::fence_after();
  };
  const int ntiles = (count + 127) / 128;
  for (int tile = blockIdx.x; tile < ntiles && ok; tile += gridDim.x) {
    // ---- stage the sample tile: X (sample-major) into R1, X^T into XT
    for (int t = tid; t < 128 * (FIN / 8); t += 128) {
      const int r = t >> 5, c8 = (t & 31) * 8;
      const int g = tile * 128 + r;
      uint4 v = make_uint4(0, 0, 0, 0);
      if (g < count) v = *reinterpret_cast<const uint4*>(X + (size_t)idx[g] * FIN + c8);
      *reinterpret_cast<uint4*>(R1 + tc::kmaj(r, c8, FIN)) = v;
      const uint16_t* e = reinterpret_cast<const uint16_t*>(&v);
#pragma unroll
      for (int i = 0; i < 8; ++i) *reinterpret_cast<uint16_t*>(XT + tc::kmaj(c8 + i, r, 128)) = e[i];
    }
    const int gr = tile * 128 + tid;
    const bool valid = gr < count;
    float tgt[NOUT];
#pragma unroll
    for (int o = 0; o < NOUT; ++o) tgt[o] = valid ? T[(size_t)idx[gr] * NOUT + o] : 0.0f;
    publish();
    // ---- layer 1
    if (tid == 0) gemm(tb + T_D1, s0 + S_R1, s0 + S_W1, NH, FIN, false);
    sync_mma();
    if (!ok) break;
    for (int c0 = 0; c0 < NH; c0 += 16) {
      float z[16];
      tc::tmem_ld16(tc::tmem_at(tb + T_D1, q, c0), z);
#pragma unroll
      for (int i = 0; i < 16; ++i) {
        float dg;
        const float h = gelu_t(z[i] + b1[c0 + i], dg);
        tc::st_bf16(sm + S_H1, tc::kmaj(tid, c0 + i, NH), h);
        tc::st_bf16(R1 + R_HT, tc::kmaj(c0 + i, tid, 128), h);
      }
    }
    publish();
    // ---- layer 2
    if (tid == 0) gemm(tb + T_D2, s0 + S_H1, s0 + S_W2, NH, NH, false);
    sync_mma();
    if (!ok) break;
    for (int c0 = 0; c0 < NH; c0 += 16) {
      float z[16];
      tc::tmem_ld16(tc::tmem_at(tb + T_D2, q, c0), z);
#pragma unroll
      for (int i = 0; i < 16; ++i) {
        float dg;
        const float h = gelu_t(z[i] + b2[c0 + i], dg);
        tc::st_bf16(sm + S_H2, tc::kmaj(tid, c0 + i, NH), h);
        tc::st_bf16(R1 + R_HT, tc::kmaj(NH + c0 + i, tid, 128), h);
      }
    }
    publish();
    // ---- layer 3 and the loss
    if (tid == 0) gemm(tb + T_D3, s0 + S_H2, s0 + S_W3, NO, NH, false);
    sync_mma();
    if (!ok) break;
    {
      float y[16];
      tc::tmem_ld16(tc::tmem_at(tb + T_D3, q, 0), y);
#pragma unroll
      for (int o = 0; o < NO; ++o) {
        float dy = 0.0f;
        if (o < NOUT && valid) {
          const float e = y[o] + b3[o] - tgt[o];
          lsum += e * e;
          dy = gscale * e;
        }
        tc::st_bf16(R1 + R_DY, tc::kmaj(tid, o, NO), dy);
        tc::st_bf16(R1 + R_DYT, tc::kmaj(o, tid, 128), dy);
        float sdy = dy;
        for (int m = 16; m > 0; m >>= 1) sdy += __shfl_xor_sync(0xffffffffu, sdy, m);
        if (lane == 0 && o < NOUT) atomicAdd(grad + OB3 + o, sdy);
      }
    }
    publish();
    // ---- dH2 = dY W3 ; dW3^T += H2^T dY (rows 64..127 of the stacked H^T)
    if (tid == 0) {
      gemm(tb + T_DH2, s0 + S_R1 + R_DY, s0 + S_W3T, NH, NO, false);
      gemm(tb + T_G3, s0 + S_R1 + R_HT, s0 + S_R1 + R_DYT, NO, 128, any);
    }
    sync_mma();
    if (!ok) break;
    for (int c0 = 0; c0 < NH; c0 += 16) {
      float dh[16], z[16];
      tc::tmem_ld16(tc::tmem_at(tb + T_DH2, q, c0), dh);
      tc::tmem_ld16(tc::tmem_at(tb + T_D2, q, c0), z);
#pragma unroll
      for (int i = 0; i < 16; ++i) {
        float dg;
        gelu_t(z[i] + b2[c0 + i], dg);
        const float dz = valid ? dh[i] * dg : 0.0f;
        tc::st_bf16(R1 + R_DZ2, tc::kmaj(tid, c0 + i, NH), dz);
        tc::st_bf16(sm + S_H1, tc::kmaj(c0 + i, tid, 128), dz);  // dZ2^T (the H1 tile is free)
        float sd = dz;
        for (int m = 16; m > 0; m >>= 1) sd += __shfl_xor_sync(0xffffffffu, sd, m);
        if (lane == 0) red[q][c0 + i] = sd;
      }
    }
    publish();
    if (tid < NH) atomicAdd(grad + OB2 + tid, red[0][tid] + red[1][tid] + red[2][tid] + red[3][tid]);
    // ---- dH1 = dZ2 W2 ; dW2^T += H1^T dZ2 (rows 0..63 of the stacked H^T)
    if (tid == 0) {
      gemm(tb + T_DH1, s0 + S_R1 + R_DZ2, s0 + S_W2T, NH, NH, false);
      gemm(tb + T_G2, s0 + S_R1 + R_HT, s0 + S_H1, NH, 128, any);
    }
    sync_mma();
    if (!ok) break;
    for (int c0 = 0; c0 < NH; c0 += 16) {
      float dh[16], z[16];
      tc::tmem_ld16(tc::tmem_at(tb + T_DH1, q, c0), dh);
      tc::tmem_ld16(tc::tmem_at(tb + T_D1, q, c0), z);
#pragma unroll
      for (int i = 0; i < 16; ++i) {
        float dg;
        gelu_t(z[i] + b1[c0 + i], dg);
        const float dz = valid ? dh[i] * dg : 0.0f;
        tc::st_bf16(sm + S_H2, tc::kmaj(c0 + i, tid, 128), dz);  // dZ1^T (the H2 tile is free)
        float sd = dz;
        for (int m = 16; m > 0; m >>= 1) sd += __shfl_xor_sync(0xffffffffu, sd, m);
        if (lane == 0) red1[q][c0 + i] = sd;
      }
    }
    publish();
    if (tid < NH) atomicAdd(grad + OB1 + tid, red1[0][tid] + red1[1][tid] + red1[2][tid] + red1[3][tid]);
    // ---- dW1^T += X^T dZ1, features 0..127 and 128..255
    if (tid == 0) {
      gemm(tb + T_G1A, s0 + S_XT, s0 + S_H2, NH, 128, any);
      gemm(tb + T_G1B, s0 + S_XT + tc::kmaj(128, 0, 128), s0 + S_H2, NH, 128, any);
    }
    sync_mma();
    any = true;
    __syncthreads();  // the next tile overwrites R1, XT and the reductions
  }
  if (!ok) {
    if (tid == 0) atomicExch(err, 1);
    tc::bar_wait(&bar, ph ^ 1u);  // a second bounded wait for MMAs still in flight
  } else if (any) {
    // ---- weight gradients from TMEM: lane = input index, column = output index
    for (int c0 = 0; c0 < NH; c0 += 16) {
      float ga[16], gb[16], g2[16];
      tc::tmem_ld16(tc::tmem_at(tb + T_G1A, q, c0), ga);
      tc::tmem_ld16(tc::tmem_at(tb + T_G1B, q, c0), gb);
      tc::tmem_ld16(tc::tmem_at(tb + T_G2, q, c0), g2);
#pragma unroll
      for (int i = 0; i < 16; ++i) {
        atomicAdd(grad + OW1 + (c0 + i) * FIN + tid, ga[i]);
        atomicAdd(grad + OW1 + (c0 + i) * FIN + 128 + tid, gb[i]);
        if (tid < NH) atomicAdd(grad + OW2 + (c0 + i) * NH + tid, g2[i]);
      }
    }
    float g3[16];
    tc::tmem_ld16(tc::tmem_at(tb + T_G3, q, 0), g3);
    if (tid >= NH)
      for (int o = 0; o < NOUT; ++o) atomicAdd(grad + OW3 + o * NH + (tid - NH), g3[o]);
    for (int m = 16; m > 0; m >>= 1) lsum += __shfl_xor_sync(0xffffffffu, lsum, m);
    if (lane == 0) atomicAdd(loss, lsum);
  }
  tc::fence_before();
  __syncthreads();
  if (q == 0) tc::tmem_free(tb, T_COLS);
}

// shared-memory map of the inference kernel: weights, then one 128 x 256 input
// tile that the hidden activations reuse once the MMA reading it has finished,
// so two CTAs fit on an SM and hide each other's MMA / TMEM latency
constexpr int I_W1 = 0, I_W2 = I_W1 + NH * FIN * 2, I_W3 = I_W2 + NH * NH * 2, I_X = 43008,
              I_TOTAL = I_X + 128 * FIN * 2;
static_assert(I_W3 + NO * NH * 2 <= I_X && I_X % 1024 == 0, "inference smem map");

// The 8 normalised conserved variables (rho, rho v, hydro energy, cell B)
// of every cell, ghosts included, as BF16 into one 16-byte record per cell
// (the cell's padded index): the inference gathers a stencil row as 27 such
// records instead of recomputing each cell's variables for the 27 rows that
// use it.
__global__ void k_mlp_features(Dev<float> d, MlpNorm nm, uint4* __restrict__ field) {
  const Geom& g = d.g;
  const long long n = (long long)g.nx * g.ny * g.nz;
  const long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (t >= n) return;
  const int i = (int)(t % g.nx);
  const long long q = t / g.nx;
  const int j = (int)(q % g.ny), k = (int)(q / g.ny);
  const long long c = (long long)i + (long long)g.px * ((long long)j + (long long)g.py * k);
  const float gm1 = d.gam - 1.0f;
  const float rho = d.rho[c], u = d.vx[c], v = d.vy[c], w = d.vz[c];
  const float U[8] = {rho, rho * u, rho * v, rho * w, 0.5f * rho * (u * u + v * v + w * w) + d.p[c] / gm1,
                      d.bx[c], d.by[c], d.bz[c]};
  uint32_t pk[4];
#pragma unroll
  for (int a = 0; a < 4; ++a) {
    const __nv_bfloat162 h = __floats2bfloat162_rn((U[2 * a] - nm.mean[2 * a]) / nm.std[2 * a],
                                                   (U[2 * a + 1] - nm.mean[2 * a + 1]) / nm.std[2 * a + 1]);
    pk[a] = *reinterpret_cast<const uint32_t*>(&h);
  }
  field[c] = make_uint4(pk[0], pk[1], pk[2], pk[3]);
}

// Features of interior cell t of an FP32 Cartesian grid into row r of an
// input tile: the 3x3x3 stencil of the feature records, feature
// ((dz+1)*9 + (dy+1)*3 + (dx+1))*8 + var; 216..255 zero.  Eight features are
// one 16-byte core-matrix row of the K-major tile; this thread writes the
// 16 of the row's 32 such chunks that start at chunk H*16 (t < 0: zeros).
// H is a template argument, so every chunk's stencil offset is a constant.
template <int H>
__device__ __forceinline__ void gather_half_row(const Dev<float>& d, const CellMap& cm,
                                                const uint4* __restrict__ field, long long t, unsigned char* tile,
                                                int r) {
  const Geom& g = d.g;
  long long c0 = 0;
  if (t >= 0) {
    const uint32_t q = cm.by_nx.div((uint32_t)t), k = cm.by_ny.div(q);
    const int i = (int)((uint32_t)t - q * (uint32_t)g.nx0) + g.ng;
    const int j = (int)(q - k * (uint32_t)g.ny0) + g.ng;
    c0 = (long long)i + (long long)g.px * ((long long)j + (long long)g.py * ((int)k + g.ng));
  }
  const long long px = g.px, pl = g.plane;
#pragma unroll
  for (int u = 0; u < 16; ++u) {
    constexpr int base = 16 * H;
    const int ch = base + u;  // chunk = stencil point ((dz+1)*9 + (dy+1)*3 + (dx+1)), 27..31 padding
    uint4 v = make_uint4(0, 0, 0, 0);
    if (t >= 0 && ch < 27) {
      const int dz = ch / 9 - 1, dy = (ch / 3) % 3 - 1, dx = ch % 3 - 1;
      v = field[c0 + dx + px * dy + pl * dz];
    }
    *reinterpret_cast<uint4*>(tile + tc::kmaj(r, 8 * ch, FIN)) = v;
  }
}

// Inference: Y[n][8] = raw network outputs.  GRID = false: rows of the BF16
// feature matrix X; GRID = true: the features of the n interior cells of the
// grid d, gathered straight into the input tile.
// 256 threads: thread (row r, half h) = (tid % 128, tid / 128) gathers half
// of row r's input chunks and takes the activation columns [32 h, 32 h + 32)
// of row r in the epilogues (TMEM lane quarter r / 32 = warp % 4), so two
// warps share each TMEM lane quarter and the GELU work.
template <bool GRID>
__global__ void __launch_bounds__(256, 2)
    k_mlp_infer(const __nv_bfloat16* __restrict__ X, Dev<float> d, CellMap cm, const uint4* __restrict__ field, int n,
                MlpW w, float* __restrict__ Y, int* err) {
  extern __shared__ __align__(1024) unsigned char sm[];
  __shared__ __align__(8) uint64_t bar;
  __shared__ uint32_t tslot;
  __shared__ __align__(16) float sbias[2 * NH + NOUT];  // biases b1, b2 and the used outputs of b3
  const int tid = threadIdx.x, warp = tid >> 5, q = warp & 3, row = tid & 127, half = tid >> 7;
  if (warp == 0) tc::tmem_alloc(&tslot, 256);
  if (tid == 0) tc::bar_init(&bar, 1);
  if (tid < 2 * NH + NOUT)
    sbias[tid] = tid < NH ? w.p[OB1 + tid] : tid < 2 * NH ? w.p[OB2 + tid - NH] : w.p[OB3 + tid - 2 * NH];
  stage_w(sm + I_W1, w.w1, NH, FIN);
  stage_w(sm + I_W2, w.w2, NH, NH);
  stage_w(sm + I_W3, w.w3, NO, NH);
  publish();
  const uint32_t tb = tslot, s0 = tc::smem_u32(sm);
  unsigned char* XS = sm + I_X;
  uint32_t ph = 0;
  bool ok = true;
  auto sync_mma = [&]() {  // every thread calls it; `ok` ends up the same in all of them
    if (tid == 0) tc::commit(&bar);
    __syncwarp();
    if (ok) ok = tc::bar_wait(&bar, ph);
    ok = __syncthreads_and(ok) != 0;
    ph ^= 1u;
    tc::fence_after();
  };
  const int ntiles = (n + 127) / 128;
  for (int tile = blockIdx.x; tile < ntiles && ok; tile += gridDim.x) {
    if (GRID) {
      const long long g = (long long)tile * 128 + row;
      if (half == 0) gather_half_row<0>(d, cm, field, g < n ? g : -1, XS, row);
      else gather_half_row<1>(d, cm, field, g < n ? g : -1, XS, row);
    } else {
      for (int t = tid; t < 128 * (FIN / 8); t += blockDim.x) {
        const int r = t >> 5, c8 = (t & 31) * 8;
        const int g = tile * 128 + r;
        uint4 v = make_uint4(0, 0, 0, 0);
        if (g < n) v = *reinterpret_cast<const uint4*>(X + (size_t)g * FIN + c8);
        *reinterpret_cast<uint4*>(XS + tc::kmaj(r, c8, FIN)) = v;
      }
    }
    publish();
    if (tid == 0) gemm(tb + T_D1, s0 + I_X, s0 + I_W1, NH, FIN, false);
    sync_mma();
    if (!ok) break;
    for (int c0 = 32 * half; c0 < 32 * half + 32; c0 += 16) {  // H1 over the consumed input tile
      float z[16];
      tc::tmem_ld16(tc::tmem_at(tb + T_D1, q, c0), z);
      gelu16_store_sm(XS, row, c0, z, sbias);
    }
    publish();
    if (tid == 0) gemm(tb + T_D2, s0 + I_X, s0 + I_W2, NH, NH, false);
    sync_mma();
    if (!ok) break;
    for (int c0 = 32 * half; c0 < 32 * half + 32; c0 += 16) {  // H2 over H1 (consumed)
      float z[16];
      tc::tmem_ld16(tc::tmem_at(tb + T_D2, q, c0), z);
      gelu16_store_sm(XS, row, c0, z, sbias + NH);
    }
    publish();
    if (tid == 0) gemm(tb + T_D3, s0 + I_X, s0 + I_W3, NO, NH, false);
    sync_mma();
    if (!ok) break;
    if (half == 0) {
      float y[16];
      tc::tmem_ld16(tc::tmem_at(tb + T_D3, q, 0), y);
      const long long g = (long long)tile * 128 + row;
      if (g < n) {
        const float* b3 = sbias + 2 * NH;
        float4* yo = reinterpret_cast<float4*>(Y + g * NOUT);
        yo[0] = make_float4(y[0] + b3[0], y[1] + b3[1], y[2] + b3[2], y[3] + b3[3]);
        yo[1] = make_float4(y[4] + b3[4], y[5] + b3[5], y[6] + b3[6], y[7] + b3[7]);
      }
    }
    tc::fence_before();
    __syncthreads();
    tc::fence_after();
  }
  if (!ok) {
    if (tid == 0) atomicExch(err, 1);
    tc::bar_wait(&bar, ph ^ 1u);
  }
  tc::fence_before();
  __syncthreads();
  if (warp == 0) tc::tmem_free(tb, 256);
}

// Adam (Kingma & Ba, 2015) on the FP32 parameters.
__global__ void k_adam(float* p, const float* g, float* m, float* v, float lr, float b1, float b2, float eps,
                       float c1, float c2) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= NPARAM) return;
  const float gi = g[i];
  const float mi = b1 * m[i] + (1.0f - b1) * gi;
  const float vi = b2 * v[i] + (1.0f - b2) * gi * gi;
  m[i] = mi;
  v[i] = vi;
  p[i] -= lr * (mi / c1) / (sqrtf(vi / c2) + eps);
}

// BF16 operand copies of the weights, and the transposes the backward pass uses.
__global__ void k_bf16_weights(const float* p, __nv_bfloat16* w1, __nv_bfloat16* w2, __nv_bfloat16* w2t,
                               __nv_bfloat16* w3, __nv_bfloat16* w3t) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < NH * FIN) w1[i] = __float2bfloat16_rn(p[OW1 + i]);
  if (i < NH * NH) {
    const int r = i / NH, c = i % NH;
    w2[i] = __float2bfloat16_rn(p[OW2 + i]);
    w2t[c * NH + r] = __float2bfloat16_rn(p[OW2 + i]);
  }
  if (i < NO * NH) {
    const int o = i / NH, c = i % NH;
    w3[i] = __float2bfloat16_rn(p[OW3 + i]);
    w3t[c * NO + o] = __float2bfloat16_rn(p[OW3 + i]);
  }
}

// Random minibatch indices: a 64-bit mixing hash of (seed, position) mod n.
__global__ void k_batch_idx(int* idx, int count, long long n, unsigned long long seed) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= count) return;
  unsigned long long x = seed * 0x9E3779B97F4A7C15ull + (unsigned long long)i * 0xBF58476D1CE4E5B9ull;
  x ^= x >> 31;
  x *= 0x94D049BB133111EBull;
  x ^= x >> 29;
  idx[i] = (int)(x % (unsigned long long)n);
}

__global__ void k_iota(int* idx, int count, long long off) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < count) idx[i] = (int)(off + i);
}

// ------------------------------------------------------- solver coupling
// Domain sums of the hydro increments y[0..4] (for a conservative correction):
// FP64 per thread, then per warp and per block (256 threads), one atomic per
// block and variable.
__global__ void __launch_bounds__(256) k_mlp_sums(const float* __restrict__ Y, long long n, double* sums) {
  __shared__ double part[8][5];
  // a thread's own few rows in FP32 with compensation (Neumaier), then FP64
  float s[5] = {0, 0, 0, 0, 0}, e[5] = {0, 0, 0, 0, 0};
  for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < n; t += (long long)gridDim.x * blockDim.x) {
    const float4 y0 = *reinterpret_cast<const float4*>(Y + t * NOUT);
    const float y[5] = {y0.x, y0.y, y0.z, y0.w, Y[t * NOUT + 4]};
#pragma unroll
    for (int q = 0; q < 5; ++q) {
      const float u = s[q] + y[q];
      e[q] += fabsf(s[q]) >= fabsf(y[q]) ? (s[q] - u) + y[q] : (y[q] - u) + s[q];
      s[q] = u;
    }
  }
  double a[5];
#pragma unroll
  for (int q = 0; q < 5; ++q) a[q] = (double)s[q] + (double)e[q];
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
#pragma unroll
  for (int q = 0; q < 5; ++q) {
    for (int m = 16; m > 0; m >>= 1) a[q] += __shfl_xor_sync(0xffffffffu, a[q], m);
    if (lane == 0) part[wid][q] = a[q];
  }
  __syncthreads();
  if (threadIdx.x < 5) {
    double b = 0.0;
    for (int w2 = 0; w2 < 8; ++w2) b += part[w2][threadIdx.x];
    atomicAdd(sums + threadIdx.x, b);
  }
}

// Hydro part of the correction: U += (y[0..4] - domain mean) * scale (rho,
// rho v, energy), so mass, momentum and energy are conserved; a cell whose
// corrected rho or p would not be positive keeps its state.  The vector-
// potential part y[5..7] * scale goes to d.dU[5..7] for the face update.
__global__ void k_mlp_apply_hydro(Dev<float> d, MlpNorm nm, const float* __restrict__ Y, const double* sums) {
  const Geom& g = d.g;
  const long long n = (long long)g.nx0 * g.ny0 * g.nz0;
  __shared__ float mean[5];  // domain means of the increments, divided once per block
  if (threadIdx.x < 5) mean[threadIdx.x] = (float)(sums[threadIdx.x] / (double)n);
  __syncthreads();
  const long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (t >= n) return;
  const int i = (int)(t % g.nx0) + g.ng;
  const long long r = t / g.nx0;
  const int j = (int)(r % g.ny0) + g.ng, k = (int)(r / g.ny0) + g.ng;
  const long long c = (long long)i + (long long)g.px * ((long long)j + (long long)g.py * k);
  const float* y = Y + t * NOUT;
  const float gm1 = d.gam - 1.0f;
  const float rho = d.rho[c], u = d.vx[c], v = d.vy[c], w = d.vz[c];
  float U[5] = {rho, rho * u, rho * v, rho * w, 0.5f * rho * (u * u + v * v + w * w) + d.p[c] / gm1};
#pragma unroll
  for (int a = 0; a < 5; ++a) U[a] += (y[a] - mean[a]) * nm.scale[a];
  const float rn = U[0];
  const float pn = gm1 * (U[4] - 0.5f * (U[1] * U[1] + U[2] * U[2] + U[3] * U[3]) / rn);
  if (rn > 0.0f && pn > 0.0f) {
    d.rho[c] = rn;
    d.vx[c] = U[1] / rn;
    d.vy[c] = U[2] / rn;
    d.vz[c] = U[3] / rn;
    d.p[c] = pn;
  }
#pragma unroll
  for (int a = 0; a < 3; ++a) d.dU[5 + a][c] = y[5 + a] * nm.scale[5 + a];
}

// Magnetic part: face B += curl of the edge vector potential, each edge value
// the mean of the cell-centred potentials of its 4 cells (periodic wrap), so
// the face update is divergence-free and div B stays at round-off.  Covers all
// n0+1 faces per axis (the top face is the periodic image of the bottom one
// and gets the same increment).
__global__ void k_mlp_apply_b(Dev<float> d) {
  const Geom& g = d.g;
  const long long n = (long long)(g.nx0 + 1) * (g.ny0 + 1) * (g.nz0 + 1);
  const long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (t >= n) return;
  const int i0 = (int)(t % (g.nx0 + 1));
  const long long r = t / (g.nx0 + 1);
  const int j0 = (int)(r % (g.ny0 + 1)), k0 = (int)(r / (g.ny0 + 1));
  // interior-periodic cell value of d.dU[5+a]; every index here lies in
  // [-1, n0], so one conditional wrap per axis is the periodic image
  auto wrap = [](int x, int n) { return x < 0 ? x + n : (x >= n ? x - n : x); };
  const int iw = i0 % g.nx0, jw = j0 % g.ny0, kw = k0 % g.nz0;  // the periodic face this one images
  // padded offsets of the wrapped indices iw-1, iw, iw+1 (and likewise j, k):
  // the edges below read cells at offsets -1 .. +1 of (iw, jw, kw) only
  int ox[3], oy[3], oz[3];
#pragma unroll
  for (int m = 0; m < 3; ++m) {
    ox[m] = wrap(iw + m - 1, g.nx0) + g.ng;
    oy[m] = g.px * (wrap(jw + m - 1, g.ny0) + g.ng);
    oz[m] = (int)g.plane * (wrap(kw + m - 1, g.nz0) + g.ng);
  }
  // cell value of d.dU[5+a] at (iw + di, jw + dj, kw + dk), di, dj, dk in -1..1
  auto at = [&](int a, int di, int dj, int dk) -> float { return d.dU[5 + a][ox[di + 1] + oy[dj + 1] + oz[dk + 1]]; };
  auto ex = [&](int i, int j, int k) {
    return 0.25f * (at(0, i, j, k) + at(0, i, j - 1, k) + at(0, i, j, k - 1) + at(0, i, j - 1, k - 1));
  };
  auto ey = [&](int i, int j, int k) {
    return 0.25f * (at(1, i, j, k) + at(1, i - 1, j, k) + at(1, i, j, k - 1) + at(1, i - 1, j, k - 1));
  };
  auto ez = [&](int i, int j, int k) {
    return 0.25f * (at(2, i, j, k) + at(2, i - 1, j, k) + at(2, i, j - 1, k) + at(2, i - 1, j - 1, k));
  };
  const int i = i0 + g.ng, j = j0 + g.ng, k = k0 + g.ng;
  const long long c = (long long)i + (long long)g.px * ((long long)j + (long long)g.py * k);
  const float rdx = d.rwx[g.ng + iw], rdy = d.rwy[g.ng + jw], rdz = d.rwz[g.ng + kw];
  const bool in_x = i0 < g.nx0, in_y = j0 < g.ny0, in_z = k0 < g.nz0;
  // the nine edge potentials (every cell load ahead of the stores, so loads
  // shared between edges are issued once), then the three face increments
  const float ex0 = ex(0, 0, 0), ex_z = ex(0, 0, 1), ex_y = ex(0, 1, 0);
  const float ey0 = ey(0, 0, 0), ey_z = ey(0, 0, 1), ey_x = ey(1, 0, 0);
  const float ez0 = ez(0, 0, 0), ez_y = ez(0, 1, 0), ez_x = ez(1, 0, 0);
  const float dbi = (ez_y - ez0) * rdy - (ey_z - ey0) * rdz;
  const float dbj = (ex_z - ex0) * rdz - (ez_x - ez0) * rdx;
  const float dbk = (ey_x - ey0) * rdx - (ex_y - ex0) * rdy;
  if (in_y && in_z) d.bi[c] += dbi;
  if (in_x && in_z) d.bj[c] += dbj;
  if (in_x && in_y) d.bk[c] += dbk;
}

int mfail(int code, const std::string& m) {
  set_last_error(m);
  return code;
}

}  // namespace

struct Mlp {
  float *p = nullptr, *g = nullptr, *m = nullptr, *v = nullptr;
  __nv_bfloat16 *w1 = nullptr, *w2 = nullptr, *w2t = nullptr, *w3 = nullptr, *w3t = nullptr;
  __nv_bfloat16* X = nullptr;  // training features [n][256]
  float* T = nullptr;          // training targets [n][8]
  long long n = 0;
  int* idx = nullptr;
  int idx_cap = 0;
  float* loss = nullptr;
  int* err = nullptr;
  int step = 0;
  MlpNorm norm{};
  float* ys = nullptr;          // correction of a grid: the network outputs
  double* sums = nullptr;       // domain sums of the hydro increments
  size_t cap = 0;
  int sms = 148;
};

}  // namespace mhd

using namespace mhd;

#define MCK(call)                                                                                          \
  do {                                                                                                     \
    cudaError_t e_ = (call);                                                                               \
    if (e_ != cudaSuccess) return mfail(MHD_E_CUDA, std::string(#call) + ": " + cudaGetErrorString(e_)); \
  } while (0)

namespace {
MlpW wview(const Mlp* m) { return MlpW{m->w1, m->w2, m->w2t, m->w3, m->w3t, m->p}; }

int refresh_bf16(Mlp* m) {
  k_bf16_weights<<<(NH * FIN + 255) / 256, 256>>>(m->p, m->w1, m->w2, m->w2t, m->w3, m->w3t);
  MCK(cudaGetLastError());
  return MHD_OK;
}

int ensure_idx(Mlp* m, int count) {
  if (count <= m->idx_cap) return MHD_OK;
  cudaFree(m->idx);
  m->idx = nullptr;
  m->idx_cap = 0;
  MCK(cudaMalloc(&m->idx, sizeof(int) * (size_t)count));
  m->idx_cap = count;
  return MHD_OK;
}

int set_smem_once() {
  static bool done = false;
  if (done) return MHD_OK;
  MCK(cudaFuncSetAttribute(k_mlp_train, cudaFuncAttributeMaxDynamicSharedMemorySize, S_TOTAL));
  MCK(cudaFuncSetAttribute(k_mlp_infer<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, I_TOTAL));
  MCK(cudaFuncSetAttribute(k_mlp_infer<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, I_TOTAL));
  done = true;
  return MHD_OK;
}

// gradient of the mean loss over idx[0..count) into m->g, loss sum into m->loss
int grad_pass(Mlp* m, int count) {
  int rc = set_smem_once();
  if (rc) return rc;
  MCK(cudaMemset(m->g, 0, sizeof(float) * NPARAM));
  MCK(cudaMemset(m->loss, 0, sizeof(float)));
  const int tiles = (count + 127) / 128;
  const int grid = tiles < m->sms ? tiles : m->sms;
  k_mlp_train<<<grid, 128, S_TOTAL>>>(m->X, m->T, m->idx, count, 2.0f / ((float)count * NOUT), wview(m), m->g,
                                       m->loss, m->err);
  MCK(cudaGetLastError());
  return MHD_OK;
}

int check_err(Mlp* m) {
  int e = 0;
  MCK(cudaMemcpy(&e, m->err, sizeof(int), cudaMemcpyDeviceToHost));
  if (e) return mfail(MHD_E_TIMEOUT, "MLP kernel: a tensor-core completion wait gave up");
  return MHD_OK;
}
}  // namespace

int mhd_tc_gemm_test(const uint16_t* a, const uint16_t* b, float* c, int32_t M, int32_t N, int32_t K) {
  if (!a || !b || !c || M <= 0 || N < 16 || N > 256 || (N % 16) || K < 16 || K > 256 || (K % 16))
    return mfail(MHD_E_ARG, "tc gemm test: M > 0, N and K multiples of 16 in [16, 256]");
  __nv_bfloat16 *da = nullptr, *db = nullptr;
  float* dc = nullptr;
  int* derr = nullptr;
  int rc = MHD_OK;
  const size_t sm = (size_t)(128 + N) * K * 2;
  int ncols = 32;
  while (ncols < N) ncols *= 2;
  if (cudaMalloc(&da, (size_t)M * K * 2) != cudaSuccess || cudaMalloc(&db, (size_t)N * K * 2) != cudaSuccess ||
      cudaMalloc(&dc, (size_t)M * N * 4) != cudaSuccess || cudaMalloc(&derr, 4) != cudaSuccess) {
    rc = mfail(MHD_E_NOMEM, "tc gemm test: device allocation failed");
  } else {
    cudaMemcpy(da, a, (size_t)M * K * 2, cudaMemcpyHostToDevice);
    cudaMemcpy(db, b, (size_t)N * K * 2, cudaMemcpyHostToDevice);
    cudaMemset(derr, 0, 4);
    cudaFuncSetAttribute(k_tc_gemm, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
    k_tc_gemm<<<(M + 127) / 128, 128, sm>>>(da, db, dc, M, N, K, ncols, derr);
    cudaError_t e = cudaDeviceSynchronize();
    int herr = 0;
    if (e == cudaSuccess) e = cudaMemcpy(&herr, derr, 4, cudaMemcpyDeviceToHost);
    if (e == cudaSuccess) e = cudaMemcpy(c, dc, (size_t)M * N * 4, cudaMemcpyDeviceToHost);
    if (e != cudaSuccess) rc = mfail(MHD_E_CUDA, std::string("tc gemm test: ") + cudaGetErrorString(e));
    else if (herr) rc = mfail(MHD_E_TIMEOUT, "tc gemm test: MMA completion wait gave up");
  }
  cudaFree(da);
  cudaFree(db);
  cudaFree(dc);
  cudaFree(derr);
  return rc;
}

int mhd_mlp_create(const float* params, void** out) {
  if (!params || !out) return mfail(MHD_E_ARG, "null argument");
  *out = nullptr;
  Mlp* m = new Mlp();
  int dev = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&m->sms, cudaDevAttrMultiProcessorCount, dev);
  bool ok = cudaMalloc(&m->p, sizeof(float) * NPARAM) == cudaSuccess &&
            cudaMalloc(&m->g, sizeof(float) * NPARAM) == cudaSuccess &&
            cudaMalloc(&m->m, sizeof(float) * NPARAM) == cudaSuccess &&
            cudaMalloc(&m->v, sizeof(float) * NPARAM) == cudaSuccess &&
            cudaMalloc(&m->w1, 2 * NH * FIN) == cudaSuccess && cudaMalloc(&m->w2, 2 * NH * NH) == cudaSuccess &&
            cudaMalloc(&m->w2t, 2 * NH * NH) == cudaSuccess && cudaMalloc(&m->w3, 2 * NO * NH) == cudaSuccess &&
            cudaMalloc(&m->w3t, 2 * NO * NH) == cudaSuccess && cudaMalloc(&m->loss, sizeof(float)) == cudaSuccess &&
            cudaMalloc(&m->err, sizeof(int)) == cudaSuccess;
  if (!ok) {
    mhd_mlp_free(m);
    return mfail(MHD_E_NOMEM, "MLP device allocation failed");
  }
  cudaMemcpy(m->p, params, sizeof(float) * NPARAM, cudaMemcpyHostToDevice);
  cudaMemset(m->m, 0, sizeof(float) * NPARAM);
  cudaMemset(m->v, 0, sizeof(float) * NPARAM);
  cudaMemset(m->err, 0, sizeof(int));
  for (int a = 0; a < 8; ++a) {
    m->norm.mean[a] = 0.0f;
    m->norm.std[a] = 1.0f;
    m->norm.scale[a] = 1.0f;
  }
  int rc = refresh_bf16(m);
  if (rc) {
    mhd_mlp_free(m);
    return rc;
  }
  *out = m;
  return MHD_OK;
}

int mhd_mlp_params(void* h, float* params_out, const float* params_in) {
  Mlp* m = (Mlp*)h;
  if (!m) return mfail(MHD_E_ARG, "null MLP handle");
  if (params_in) {
    MCK(cudaMemcpy(m->p, params_in, sizeof(float) * NPARAM, cudaMemcpyHostToDevice));
    int rc = refresh_bf16(m);
    if (rc) return rc;
  }
  if (params_out) MCK(cudaMemcpy(params_out, m->p, sizeof(float) * NPARAM, cudaMemcpyDeviceToHost));
  return MHD_OK;
}

int mhd_mlp_set_norm(void* h, const float* mean8, const float* std8, const float* scale8) {
  Mlp* m = (Mlp*)h;
  if (!m || !mean8 || !std8 || !scale8) return mfail(MHD_E_ARG, "null argument");
  for (int a = 0; a < 8; ++a)
    if (!(std8[a] > 0.0f)) return mfail(MHD_E_ARG, "feature std must be positive");
  for (int a = 0; a < 8; ++a) {
    m->norm.mean[a] = mean8[a];
    m->norm.std[a] = std8[a];
    m->norm.scale[a] = scale8[a];
  }
  return MHD_OK;
}

int mhd_mlp_set_data(void* h, const uint16_t* x, const float* t, int64_t n) {
  Mlp* m = (Mlp*)h;
  if (!m || !x || !t || n <= 0 || n >= (1LL << 31)) return mfail(MHD_E_ARG, "bad training data");
  cudaFree(m->X);
  cudaFree(m->T);
  m->X = nullptr;
  m->T = nullptr;
  m->n = 0;
  MCK(cudaMalloc(&m->X, (size_t)n * FIN * 2));
  MCK(cudaMalloc(&m->T, (size_t)n * NOUT * 4));
  MCK(cudaMemcpy(m->X, x, (size_t)n * FIN * 2, cudaMemcpyHostToDevice));
  MCK(cudaMemcpy(m->T, t, (size_t)n * NOUT * 4, cudaMemcpyHostToDevice));
  m->n = n;
  return MHD_OK;
}

int mhd_mlp_grad(void* h, int64_t offset, int32_t count, float* grad_out, float* loss_out) {
  Mlp* m = (Mlp*)h;
  if (!m || !grad_out || count <= 0 || offset < 0 || offset + count > m->n)
    return mfail(MHD_E_ARG, "bad gradient range");
  int rc = ensure_idx(m, count);
  if (rc) return rc;
  k_iota<<<(count + 255) / 256, 256>>>(m->idx, count, offset);
  rc = grad_pass(m, count);
  if (rc) return rc;
  MCK(cudaDeviceSynchronize());
  rc = check_err(m);
  if (rc) return rc;
  MCK(cudaMemcpy(grad_out, m->g, sizeof(float) * NPARAM, cudaMemcpyDeviceToHost));
  if (loss_out) {
    float l = 0;
    MCK(cudaMemcpy(&l, m->loss, sizeof(float), cudaMemcpyDeviceToHost));
    *loss_out = l / ((float)count * NOUT);
  }
  return MHD_OK;
}

int mhd_mlp_train(void* h, int32_t iters, int32_t batch, float lr, uint64_t seed, float* loss_out) {
  Mlp* m = (Mlp*)h;
  if (!m || iters <= 0 || batch <= 0 || !(lr > 0.0f) || m->n <= 0) return mfail(MHD_E_ARG, "bad training arguments");
  int rc = ensure_idx(m, batch);
  if (rc) return rc;
  double lacc = 0.0;
  int lcnt = 0;
  for (int it = 0; it < iters; ++it) {
    k_batch_idx<<<(batch + 255) / 256, 256>>>(m->idx, batch, m->n, seed + (uint64_t)m->step);
    rc = grad_pass(m, batch);
    if (rc) return rc;
    m->step += 1;
    const float b1 = 0.9f, b2 = 0.999f;
    const float c1 = 1.0f - powf(b1, (float)m->step), c2 = 1.0f - powf(b2, (float)m->step);
    k_adam<<<(NPARAM + 255) / 256, 256>>>(m->p, m->g, m->m, m->v, lr, b1, b2, 1e-8f, c1, c2);
    rc = refresh_bf16(m);
    if (rc) return rc;
    if (it >= iters - 8 || it % 64 == 63) {  // host sync only here: loss of the last iterations, error word
      float l = 0;
      MCK(cudaMemcpy(&l, m->loss, sizeof(float), cudaMemcpyDeviceToHost));
      if (it >= iters - 8) {
        lacc += l / ((double)batch * NOUT);
        ++lcnt;
      }
      rc = check_err(m);
      if (rc) return rc;
    }
  }
  MCK(cudaDeviceSynchronize());
  rc = check_err(m);
  if (rc) return rc;
  if (loss_out) *loss_out = (float)(lacc / (lcnt ? lcnt : 1));
  return MHD_OK;
}

int mhd_mlp_forward(void* h, const uint16_t* x, int64_t n, float* y) {
  Mlp* m = (Mlp*)h;
  if (!m || !x || !y || n <= 0 || n >= (1LL << 31)) return mfail(MHD_E_ARG, "bad forward arguments");
  int rc = set_smem_once();
  if (rc) return rc;
  __nv_bfloat16* dx = nullptr;
  float* dy = nullptr;
  MCK(cudaMalloc(&dx, (size_t)n * FIN * 2));
  if (cudaMalloc(&dy, (size_t)n * NOUT * 4) != cudaSuccess) {
    cudaFree(dx);
    return mfail(MHD_E_NOMEM, "MLP forward buffers");
  }
  cudaMemcpy(dx, x, (size_t)n * FIN * 2, cudaMemcpyHostToDevice);
  const int tiles = (int)((n + 127) / 128);
  k_mlp_infer<false><<<tiles < 2 * m->sms ? tiles : 2 * m->sms, 256, I_TOTAL>>>(dx, Dev<float>{}, CellMap{}, nullptr,
                                                                                 (int)n, wview(m), dy, m->err);
  cudaError_t e = cudaDeviceSynchronize();
  if (e == cudaSuccess) e = cudaMemcpy(y, dy, (size_t)n * NOUT * 4, cudaMemcpyDeviceToHost);
  cudaFree(dx);
  cudaFree(dy);
  if (e != cudaSuccess) return mfail(MHD_E_CUDA, std::string("MLP forward: ") + cudaGetErrorString(e));
  return check_err(m);
}

int mhd_mlp_free(void* h) {
  Mlp* m = (Mlp*)h;
  if (!m) return MHD_OK;
  cudaDeviceSynchronize();
  void* ptrs[] = {m->p, m->g, m->m, m->v, m->w1, m->w2, m->w2t, m->w3, m->w3t, m->X, m->T, m->idx, m->loss, m->err,
                  m->ys, m->sums};
  for (void* q : ptrs)
    if (q) cudaFree(q);
  delete m;
  return MHD_OK;
}

// Correction of one FP32 grid (called by mhd_mlp_apply in mhd_api.cu).
int mhd::mlp_correct(void* h, Dev<float>& d, cudaStream_t st) {
  Mlp* m = (Mlp*)h;
  const size_t n = (size_t)d.g.nx0 * d.g.ny0 * d.g.nz0;
  if (n > m->cap) {
    cudaFree(m->ys);
    m->ys = nullptr;
    m->cap = 0;
    MCK(cudaMalloc(&m->ys, n * NOUT * 4));
    m->cap = n;
  }
  int rc = set_smem_once();
  if (rc) return rc;
  const int nb = (int)((n + 255) / 256);
  const int tiles = (int)((n + 127) / 128);
  // the feature records go to the x-face flux arrays, scratch outside a step
  // (4 consecutive FP32 arrays = one 16-byte record per padded cell index)
  uint4* field = reinterpret_cast<uint4*>(d.F[0][0]);
  const long long ncell = (long long)d.g.nx * d.g.ny * d.g.nz;
  k_mlp_features<<<(int)((ncell + 255) / 256), 256, 0, st>>>(d, m->norm, field);
  k_mlp_infer<true><<<tiles < 2 * m->sms ? tiles : 2 * m->sms, 256, I_TOTAL, st>>>(nullptr, d, cell_map(d.g), field,
                                                                                   (int)n, wview(m), m->ys, m->err);
  if (!m->sums) MCK(cudaMalloc(&m->sums, 8 * sizeof(double)));
  MCK(cudaMemsetAsync(m->sums, 0, 8 * sizeof(double), st));
  k_mlp_sums<<<m->sms * 4, 256, 0, st>>>(m->ys, (long long)n, m->sums);
  k_mlp_apply_hydro<<<nb, 256, 0, st>>>(d, m->norm, m->ys, m->sums);
  const long long nf = (long long)(d.g.nx0 + 1) * (d.g.ny0 + 1) * (d.g.nz0 + 1);
  k_mlp_apply_b<<<(int)((nf + 255) / 256), 256, 0, st>>>(d);
  MCK(cudaGetLastError());
  return MHD_OK;
}

int mhd::mlp_status(void* h) { return check_err((Mlp*)h); }
