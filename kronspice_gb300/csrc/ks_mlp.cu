// ks_mlp.cu — the learned Newton start: a BF16 MLP trained and run on the GB300's
// tensor cores by hand-written kernels.
//
// Network: in -> H -> H -> H -> out, ReLU on the hidden layers, linear output,
// on standardized features and targets.  Weights are FP32 masters (Adam) with
// BF16 copies W[out][in] and W^T[in][out] for the GEMMs; activations are BF16,
// accumulation FP32.  One GEMM kernel serves every product through layout
// flags: ldmatrix (.trans where an operand is stored the other way round)
// feeds mma.sync m16n8k16 BF16 with FP32 accumulators; the epilogue fuses bias,
// ReLU, the ReLU-backward mask, or split-K atomic accumulation of weight
// gradients.  Dimensions are padded: batch to 64, feature and output widths to
// 64, so every tile is full and every 16-byte access aligned.
#include <cuda.h>  // CUtensorMap and its encoder's signature (the encoder is fetched at run time)
#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <string>
#include <vector>
#include "ks_internal.h"
#include "ks_tc.cuh"

using ksh::set_error;

namespace {

constexpr int BM = 64, BN = 64, BK = 32, PAD = 8;

enum Epi { EPI_RELU_BF16 = 0, EPI_LINEAR_F32 = 1, EPI_MASK_BF16 = 2, EPI_ATOMIC_F32 = 3 };

__device__ __forceinline__ void ldsm_x4(uint32_t* r, const void* p) {
  uint32_t a = (uint32_t)__cvta_generic_to_shared(p);
  asm volatile("ldmatrix.sync.aligned.m8n8.x4.shared.b16 {%0,%1,%2,%3}, [%4];\n"
               : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]) : "r"(a));
}
__device__ __forceinline__ void ldsm_x4_t(uint32_t* r, const void* p) {
  uint32_t a = (uint32_t)__cvta_generic_to_shared(p);
  asm volatile("ldmatrix.sync.aligned.m8n8.x4.trans.shared.b16 {%0,%1,%2,%3}, [%4];\n"
               : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]) : "r"(a));
}
__device__ __forceinline__ void mma_bf16(float* c, const uint32_t* a, uint32_t b0, uint32_t b1) {
  asm volatile("mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
               "{%0,%1,%2,%3};\n"
               : "+f"(c[0]), "+f"(c[1]), "+f"(c[2]), "+f"(c[3])
               : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b0), "r"(b1));
}

// C[M][N] = A * B over K.
//   A_T = false: A stored [M][K] (lda = row stride);  A_T = true: A stored [K][M]
//   B_T = false: B stored [N][K] (the weight layout); B_T = true: B stored [K][N]
// Grid: (N/BN, M/BM, splits); blockIdx.z takes K range [z*kchunk, (z+1)*kchunk).
template <bool A_T, bool B_T, int EPI>
__global__ void __launch_bounds__(128) k_gemm(const __nv_bfloat16* __restrict__ A, const __nv_bfloat16* __restrict__ Bm,
                                              void* C, const float* __restrict__ bias,
                                              const __nv_bfloat16* __restrict__ mask, int M, int N, int K, int lda,
                                              int ldb, int ldc, int kchunk) {
  constexpr int AR = A_T ? BK : BM, AC = A_T ? BM : BK;  // smem tile rows x cols as stored
  constexpr int BR = B_T ? BK : BN, BC = B_T ? BN : BK;
  __shared__ __align__(16) __nv_bfloat16 As[AR][AC + PAD];
  __shared__ __align__(16) __nv_bfloat16 Bs[BR][BC + PAD];
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int wm = (warp >> 1) * 32, wn = (warp & 1) * 32;
  const int m0 = blockIdx.y * BM, n0 = blockIdx.x * BN;
  const int kbeg = blockIdx.z * kchunk, kend = min(K, kbeg + kchunk);
  float acc[2][4][4];
#pragma unroll
  for (int i = 0; i < 2; i++)
#pragma unroll
    for (int j = 0; j < 4; j++)
#pragma unroll
      for (int e = 0; e < 4; e++) acc[i][j][e] = 0.f;

  for (int k0 = kbeg; k0 < kend; k0 += BK) {
    // global -> shared, 16-byte vectors (AR*AC/8 = 256 vectors per tile)
#pragma unroll
    for (int v = tid; v < AR * AC / 8; v += 128) {
      int r = v / (AC / 8), cc = (v % (AC / 8)) * 8;
      const __nv_bfloat16* src = A_T ? A + (size_t)(k0 + r) * lda + m0 + cc : A + (size_t)(m0 + r) * lda + k0 + cc;
      *reinterpret_cast<uint4*>(&As[r][cc]) = *reinterpret_cast<const uint4*>(src);
    }
#pragma unroll
    for (int v = tid; v < BR * BC / 8; v += 128) {
      int r = v / (BC / 8), cc = (v % (BC / 8)) * 8;
      const __nv_bfloat16* src = B_T ? Bm + (size_t)(k0 + r) * ldb + n0 + cc : Bm + (size_t)(n0 + r) * ldb + k0 + cc;
      *reinterpret_cast<uint4*>(&Bs[r][cc]) = *reinterpret_cast<const uint4*>(src);
    }
    __syncthreads();
#pragma unroll
    for (int kk = 0; kk < BK; kk += 16) {
      uint32_t af[2][4], bf[2][4];
      const int j = lane >> 3, r = lane & 7;
#pragma unroll
      for (int i = 0; i < 2; i++) {
        int mb = wm + i * 16;
        if (!A_T) ldsm_x4(af[i], &As[mb + (lane & 15)][kk + (lane >> 4) * 8]);
        else ldsm_x4_t(af[i], &As[kk + (j >> 1) * 8 + r][mb + (j & 1) * 8]);
      }
#pragma unroll
      for (int i = 0; i < 2; i++) {  // two n16 groups -> b fragments of 4 n8 blocks
        int nb = wn + i * 16;
        if (!B_T) ldsm_x4(bf[i], &Bs[nb + (j >> 1) * 8 + r][kk + (j & 1) * 8]);
        else ldsm_x4_t(bf[i], &Bs[kk + (j & 1) * 8 + r][nb + (j >> 1) * 8]);
      }
#pragma unroll
      for (int i = 0; i < 2; i++)
#pragma unroll
        for (int jn = 0; jn < 4; jn++) mma_bf16(acc[i][jn], af[i], bf[jn >> 1][(jn & 1) * 2], bf[jn >> 1][(jn & 1) * 2 + 1]);
    }
    __syncthreads();
  }
  const int g = lane >> 2, t4 = lane & 3;
#pragma unroll
  for (int i = 0; i < 2; i++)
#pragma unroll
    for (int jn = 0; jn < 4; jn++)
#pragma unroll
      for (int h = 0; h < 2; h++) {
        int row = m0 + wm + i * 16 + g + h * 8;
        int col = n0 + wn + jn * 8 + t4 * 2;
        float v0 = acc[i][jn][h * 2], v1 = acc[i][jn][h * 2 + 1];
        if (row >= M || col >= N) continue;  // N even except for the atomic (unpadded) case below
        if (EPI == EPI_RELU_BF16) {
          v0 = fmaxf(v0 + bias[col], 0.f); v1 = fmaxf(v1 + bias[col + 1], 0.f);
          *reinterpret_cast<__nv_bfloat162*>((__nv_bfloat16*)C + (size_t)row * ldc + col) = __floats2bfloat162_rn(v0, v1);
        } else if (EPI == EPI_LINEAR_F32) {
          float* o = (float*)C + (size_t)row * ldc + col;
          o[0] = v0 + bias[col]; o[1] = v1 + bias[col + 1];
        } else if (EPI == EPI_MASK_BF16) {  // dX of a ReLU layer: zero where the forward activation was 0
          const __nv_bfloat16* mk = mask + (size_t)row * ldc + col;
          if (!(__bfloat162float(mk[0]) > 0.f)) v0 = 0.f;
          if (!(__bfloat162float(mk[1]) > 0.f)) v1 = 0.f;
          *reinterpret_cast<__nv_bfloat162*>((__nv_bfloat16*)C + (size_t)row * ldc + col) = __floats2bfloat162_rn(v0, v1);
        } else {
          float* o = (float*)C + (size_t)row * ldc + col;
          atomicAdd(o, v0);
          if (col + 1 < N) atomicAdd(o + 1, v1);
        }
      }
}

inline int pad64(int x) { return (x + 63) / 64 * 64; }

// Gather standardized features: X[r][j] = bf16((f(values[col_j][idx[r]]) - mean_j) / std_j),
// f = log when logmask bit j is set; rows beyond rows_valid and columns beyond d are 0.
__global__ void k_features(const double* __restrict__ vals_soa, int64_t B, const int32_t* __restrict__ idx,
                           const int32_t* __restrict__ cols, uint64_t logmask, const float* __restrict__ mean,
                           const float* __restrict__ stdv, int d, int dp, int rows_valid, __nv_bfloat16* X, int rows) {
  int r = blockIdx.x * blockDim.y + threadIdx.y;
  int j = threadIdx.x;
  if (r >= rows) return;
  for (int jj = j; jj < dp; jj += blockDim.x) {
    float v = 0.f;
    if (r < rows_valid && jj < d) {
      int64_t c = idx ? idx[r] : r;
      float x = (float)vals_soa[(int64_t)cols[jj] * B + c];  // the network reads BF16: FP32 is ample here
      if ((logmask >> jj) & 1) x = logf(x);
      v = (x - mean[jj]) / stdv[jj];
    }
    X[(size_t)r * dp + jj] = __float2bfloat16(v);
  }
}

// Standardized targets T[r][j] (FP32) from solutions x [B][n] (node voltages).
__global__ void k_targets(const double* __restrict__ x, int n, const int32_t* __restrict__ idx, const float* __restrict__ mean,
                          const float* __restrict__ stdv, int dout, int dop, int rows_valid, float* T, int rows,
                          const double* __restrict__ vals_soa, int64_t B, int scale_col) {
  int r = blockIdx.x * blockDim.y + threadIdx.y;
  if (r >= rows) return;
  double sc = 1.0;
  if (scale_col >= 0 && r < rows_valid) sc = vals_soa[(int64_t)scale_col * B + idx[r]];
  for (int j = threadIdx.x; j < dop; j += blockDim.x) {
    float v = 0.f;
    if (r < rows_valid && j < dout) v = (float)((x[(int64_t)idx[r] * n + j] / sc - mean[j]) / stdv[j]);
    T[(size_t)r * dop + j] = v;
  }
}

// MSE gradient dY = 2 (Y - T) / rows_valid on the valid block, bf16; loss partials.
__global__ void k_loss_grad(const float* __restrict__ Y, const float* __restrict__ T, int dout, int dop, int rows_valid,
                            __nv_bfloat16* dY, int rows, float* loss) {
  const int r = blockIdx.x * blockDim.y + threadIdx.y;
  float l = 0.f;
  if (r < rows) {
    for (int j = threadIdx.x; j < dop; j += blockDim.x) {
      float g = 0.f;
      if (r < rows_valid && j < dout) {
        float e = Y[(size_t)r * dop + j] - T[(size_t)r * dop + j];
        l += e * e;
        g = 2.f * e / rows_valid;
      }
      dY[(size_t)r * dop + j] = __float2bfloat16(g);
    }
  }
  // one atomic per block: the squared errors summed over the block's warps
  // (one per thread serialized on the single loss word)
  __shared__ float part[32];
  const int tid = threadIdx.y * blockDim.x + threadIdx.x, nthr = blockDim.x * blockDim.y;
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) l += __shfl_down_sync(0xffffffffu, l, o);
  if ((tid & 31) == 0) part[tid >> 5] = l;
  __syncthreads();
  if (tid == 0 && loss) {
    float sum = 0.f;
    for (int w = 0; w < (nthr + 31) / 32; w++) sum += part[w];
    atomicAdd(loss, sum / (rows_valid * (float)dout));
  }
}

// Column sums of dY (bias gradients): db[j] += sum_r dY[r][j], each block a
// stripe of KS_COLSUM_ROWS rows (independent loads, one atomic per column).
constexpr int KS_COLSUM_ROWS = 32;
__global__ void k_colsum(const __nv_bfloat16* __restrict__ dY, int rows, int cols, int ld, float* db) {
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= cols) return;
  const int r0 = blockIdx.y * KS_COLSUM_ROWS, r1 = min(rows, r0 + KS_COLSUM_ROWS);
  float s = 0.f;
#pragma unroll 8
  for (int r = r0; r < r1; r++) s += __bfloat162float(dY[(size_t)r * ld + j]);
  atomicAdd(&db[j], s);
}

// Adam step on FP32 masters, then BF16 copies W[o][i] (ld ip) and W^T[i][o] (ld op).
__global__ void k_adam(float* w, const float* __restrict__ g, float* m, float* v, int nparam, float lr, float b1, float b2,
                       float eps, float c1, float c2) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nparam) return;
  float gi = g[i];
  float mi = b1 * m[i] + (1 - b1) * gi, vi = b2 * v[i] + (1 - b2) * gi * gi;
  m[i] = mi; v[i] = vi;
  w[i] -= lr * (mi / c1) / (sqrtf(vi / c2) + eps);
}

__global__ void k_quantize(const float* __restrict__ w, int out, int in, __nv_bfloat16* W, int ldw, __nv_bfloat16* WT,
                           int ldt) {
  int o = blockIdx.y, i = blockIdx.x * blockDim.x + threadIdx.x;
  if (o >= out || i >= in) return;
  __nv_bfloat16 q = __float2bfloat16(w[(size_t)o * in + i]);
  W[(size_t)o * ldw + i] = q;
  WT[(size_t)i * ldt + o] = q;
}

// Decode standardized outputs into Newton starting points x0[c][0..dout) (doubles).
__global__ void k_decode(const float* __restrict__ Y, int dop, int dout, const float* __restrict__ mean,
                         const float* __restrict__ stdv, double* x0, int n, int rows, const double* __restrict__ vals_soa,
                         int64_t B, int scale_col) {
  int r = blockIdx.x * blockDim.y + threadIdx.y;
  if (r >= rows) return;
  double sc = scale_col >= 0 ? vals_soa[(int64_t)scale_col * B + r] : 1.0;
  for (int j = threadIdx.x; j < n; j += blockDim.x)
    x0[(size_t)r * n + j] = j < dout ? ((double)Y[(size_t)r * dop + j] * stdv[j] + mean[j]) * sc : 0.0;
}


// Inference in one kernel: each block takes 128 circuits through the whole
// network with the activations in shared memory.  Features are read in place
// from the batch's SoA values; each layer's BF16 weights [N][K] are staged in
// shared memory (read from L2, which holds them for every block); eight warps
// each own a quarter of the layer's output columns for 64 of the rows (mma.sync
// m16n8k16, FP32 accumulators); the bias + ReLU epilogue writes the next
// activations over the previous ones; the output layer is decoded straight
// into the Newton starting points (doubles).
constexpr int IR = 128;  // rows per block: 8 warps, each 64 rows x a quarter of the columns

template <int NT>  // n8 tiles per warp: 8 for 256-wide layers, 2 for the 64-wide output layer
__device__ __forceinline__ void infer_layer(const __nv_bfloat16* As, int lda, const __nv_bfloat16* Ws, int ldw, int K,
                                            float (&acc)[4][NT][4]) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int j = lane >> 3, r = lane & 7;
  const int n0 = (warp & 3) * NT * 8;
  As += (size_t)(warp >> 2) * 64 * lda;
#pragma unroll
  for (int i = 0; i < 4; i++)
#pragma unroll
    for (int t = 0; t < NT; t++)
#pragma unroll
      for (int e = 0; e < 4; e++) acc[i][t][e] = 0.f;
  for (int kk = 0; kk < K; kk += 16) {
    uint32_t af[4][4];
#pragma unroll
    for (int i = 0; i < 4; i++) ldsm_x4(af[i], As + (size_t)(i * 16 + (lane & 15)) * lda + kk + (lane >> 4) * 8);
#pragma unroll
    for (int g = 0; g < NT / 2; g++) {
      uint32_t bf[4];
      ldsm_x4(bf, Ws + (size_t)(n0 + g * 16 + (j >> 1) * 8 + r) * ldw + kk + (j & 1) * 8);
#pragma unroll
      for (int i = 0; i < 4; i++) {
        mma_bf16(acc[i][2 * g], af[i], bf[0], bf[1]);
        mma_bf16(acc[i][2 * g + 1], af[i], bf[2], bf[3]);
      }
    }
  }
}

// Copy a [rows][cols] BF16 matrix (global row stride ldg) into shared memory (row
// stride lds) with asynchronous 16-byte copies, all in flight at once; the
// caller waits (cp_async_wait_all) and synchronises the block.
__device__ __forceinline__ void stage(__nv_bfloat16* dst, int lds, const __nv_bfloat16* __restrict__ src, int ldg,
                                      int rows, int cols) {
  const int vpr = cols / 8;
  for (int v = threadIdx.x; v < rows * vpr; v += blockDim.x) {
    int rr = v / vpr, cc = (v % vpr) * 8;
    uint32_t d = (uint32_t)__cvta_generic_to_shared(dst + (size_t)rr * lds + cc);
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(d), "l"(src + (size_t)rr * ldg + cc));
  }
  asm volatile("cp.async.commit_group;\n" ::);
}
__device__ __forceinline__ void cp_async_wait_all() { asm volatile("cp.async.wait_group 0;\n" ::: "memory"); }

struct InferArgs {
  const double* vals; int64_t B; int n;
  const int32_t* cols; uint64_t logmask; const float *fmean, *fstd;
  int din, dip, h, dout, dop;
  const __nv_bfloat16* W[4]; const float* bias[4];
  const float *tmean, *tstd; int scale_col;
  double* x0;
};

__global__ void __launch_bounds__(256) k_mlp_infer(InferArgs a) {
  extern __shared__ __align__(16) unsigned char sm[];
  const int ldh = a.h + PAD, ldx = a.dip + PAD;
  __nv_bfloat16* Hs = reinterpret_cast<__nv_bfloat16*>(sm);              // [IR][h + PAD]
  __nv_bfloat16* Xs = Hs + (size_t)IR * ldh;                              // [IR][dip + PAD]
  __nv_bfloat16* Ws = Xs + (size_t)IR * ldx;                              // [h][h + PAD] (largest layer)
  const int64_t r0 = (int64_t)blockIdx.x * IR;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, g = lane >> 2, t4 = lane & 3;
  const int wrow = (warp >> 2) * 64, wcol = warp & 3;
  // features
  for (int v = threadIdx.x; v < IR * a.dip; v += blockDim.x) {
    int rr = v / a.dip, jj = v % a.dip;
    int64_t c = r0 + rr;
    float f = 0.f;
    if (c < a.B && jj < a.din) {
      float x = (float)a.vals[(int64_t)a.cols[jj] * a.B + c];
      if ((a.logmask >> jj) & 1) x = logf(x);
      f = (x - a.fmean[jj]) / a.fstd[jj];
    }
    Xs[(size_t)rr * ldx + jj] = __float2bfloat16(f);
  }
  // hidden layers
  float acc[4][8][4];
  for (int l = 0; l < 3; l++) {
    const int K = l == 0 ? a.dip : a.h, ldw = K + PAD;
    stage(Ws, ldw, a.W[l], K, a.h, K);
    cp_async_wait_all();
    __syncthreads();
    infer_layer<8>(l == 0 ? Xs : Hs, l == 0 ? ldx : ldh, Ws, ldw, K, acc);
    __syncthreads();  // every warp is done reading Hs and Ws
#pragma unroll
    for (int i = 0; i < 4; i++)
#pragma unroll
      for (int t = 0; t < 8; t++)
#pragma unroll
        for (int hh = 0; hh < 2; hh++) {
          int row = wrow + i * 16 + g + hh * 8, col = wcol * 64 + t * 8 + t4 * 2;
          float v0 = fmaxf(acc[i][t][hh * 2] + a.bias[l][col], 0.f);
          float v1 = fmaxf(acc[i][t][hh * 2 + 1] + a.bias[l][col + 1], 0.f);
          *reinterpret_cast<__nv_bfloat162*>(Hs + (size_t)row * ldh + col) = __floats2bfloat162_rn(v0, v1);
        }
  }
  // output layer (dop = 64 columns, 16 per warp) and decode
  stage(Ws, ldh, a.W[3], a.h, a.dop, a.h);
  cp_async_wait_all();
  __syncthreads();
  float out[4][2][4];
  infer_layer<2>(Hs, ldh, Ws, ldh, a.h, out);
#pragma unroll
  for (int i = 0; i < 4; i++)
#pragma unroll
    for (int t = 0; t < 2; t++)
#pragma unroll
      for (int hh = 0; hh < 2; hh++)
#pragma unroll
        for (int e = 0; e < 2; e++) {
          int row = wrow + i * 16 + g + hh * 8, col = wcol * 16 + t * 8 + t4 * 2 + e;
          int64_t c = r0 + row;
          if (c >= a.B || col >= a.n) continue;
          double sc = a.scale_col >= 0 ? a.vals[(int64_t)a.scale_col * a.B + c] : 1.0;
          double y = out[i][t][hh * 2 + e] + a.bias[3][col];
          a.x0[(size_t)c * a.n + col] = col < a.dout ? (y * a.tstd[col] + a.tmean[col]) * sc : 0.0;
        }
}

// ---------------------------------------------------------------- inference on tcgen05
// The learned start's whole inference in one kernel on the 5th-generation tensor
// cores: a CTA of 128 threads takes 128 circuits (the MMA's M).  Thread r
// computes circuit r's standardized features from the SoA values and writes them
// as BF16 into shared memory in the 128-byte-swizzled K-major layout; TMA
// (cp.async.bulk.tensor, 128-byte swizzle) brings each layer's BF16 weights
// W[out][in] into shared memory in the same layout, the next layer's while the
// current one computes where the buffers allow; one thread issues the layer's
// tcgen05.mma (M = 128, N = the layer's width, K = 16 per instruction, FP32
// accumulation in tensor memory) and commits it to an mbarrier; each warp then
// reads its 32 rows of the accumulator back with tcgen05.ld, adds the bias,
// applies ReLU and writes the next layer's BF16 operand over the previous one.
// The output layer is decoded straight into the Newton starting points.
// Shared memory: activations 64 KB (hidden width <= 256), the hidden layers'
// weights 128 KB, the first / last layer's weights 32 KB; 256 TMEM columns.
// Every wait is bounded: a wait that gives up sets *err, writes zero starts for
// the CTA's circuits, and the CTA still frees its tensor memory.
constexpr int TC_M = 128;
constexpr size_t TC_ACT = 65536, TC_WBIG = 131072, TC_WSM = 32768;
constexpr size_t TC_SMEM = TC_ACT + TC_WBIG + TC_WSM + 64 + 1024;  // + barriers, + alignment slack

struct TcArgs {
  const double* vals; int64_t B; int n;
  const int32_t* cols; uint64_t logmask; const float *fmean, *fstd;
  int din, h, dout;
  const float* bias[4];
  const float *tmean, *tstd; int scale_col;
  double* x0;
  int* err;
};

__global__ void __launch_bounds__(128, 1)
k_mlp_infer_tc(TcArgs a, const __grid_constant__ CUtensorMap tw0, const __grid_constant__ CUtensorMap tw1,
               const __grid_constant__ CUtensorMap tw2, const __grid_constant__ CUtensorMap tw3) {
  extern __shared__ __align__(1024) unsigned char sm_raw[];
  unsigned char* sm = sm_raw + ((1024 - (ktc::smem_u32(sm_raw) & 1023)) & 1023);
  unsigned char* act = sm;
  unsigned char* wbig = sm + TC_ACT;
  unsigned char* wsm = wbig + TC_WBIG;
  uint64_t* bars = reinterpret_cast<uint64_t*>(wsm + TC_WSM);  // [0] small weights, [1] big weights, [2] MMA
  uint32_t* tslot = reinterpret_cast<uint32_t*>(bars + 3);
  int* abort_flag = reinterpret_cast<int*>(tslot + 1);
  const int tid = threadIdx.x, warp = tid >> 5, H = a.h, NC = a.h >> 6;
  const int64_t c = (int64_t)blockIdx.x * TC_M + tid;  // this thread's circuit (its accumulator row)
  if (tid == 0) {
    ktc::mbar_init(&bars[0], 1);
    ktc::mbar_init(&bars[1], 1);
    ktc::mbar_init(&bars[2], 1);
    *abort_flag = 0;
    ktc::mbar_fence_init();
  }
  if (warp == 0) ktc::tmem_alloc(tslot, 256);
  ktc::tc_fence_before();
  __syncthreads();
  ktc::tc_fence_after();
  const uint32_t tmem = *tslot;
  if (tid == 0) {  // first layer's weights [H][64] and the first hidden layer's [H][H]
    ktc::tma_prefetch(&tw0); ktc::tma_prefetch(&tw1); ktc::tma_prefetch(&tw2); ktc::tma_prefetch(&tw3);
    ktc::mbar_expect_tx(&bars[0], (uint32_t)H * 128u);
    ktc::tma_load_2d(wsm, &tw0, 0, 0, &bars[0]);
    ktc::mbar_expect_tx(&bars[1], (uint32_t)NC * H * 128u);
    for (int k = 0; k < NC; k++) ktc::tma_load_2d(wbig + (size_t)k * H * 128, &tw1, 64 * k, 0, &bars[1]);
  }
  // features: 64 K-elements (the inputs, then zeros), 8 units of 8 BF16
#pragma unroll 1
  for (int u = 0; u < 8; u++) {
    uint32_t w[4];
#pragma unroll
    for (int e = 0; e < 4; e++) {
      float f[2];
#pragma unroll
      for (int h2 = 0; h2 < 2; h2++) {
        const int j = u * 8 + e * 2 + h2;
        f[h2] = 0.f;
        if (c < a.B && j < a.din) {
          float x = (float)a.vals[(int64_t)a.cols[j] * a.B + c];
          if ((a.logmask >> j) & 1) x = logf(x);
          f[h2] = (x - a.fmean[j]) / a.fstd[j];
        }
      }
      __nv_bfloat162 b2 = __floats2bfloat162_rn(f[0], f[1]);
      w[e] = *reinterpret_cast<uint32_t*>(&b2);
    }
    *reinterpret_cast<uint4*>(act + ktc::sw128_offset(tid, u * 8, TC_M)) = make_uint4(w[0], w[1], w[2], w[3]);
  }
  ktc::fence_proxy_async();
  __syncthreads();
  const uint32_t wait_parity[4][2] = {{0, 0}, {1, 0}, {1, 1}, {0, 1}};  // (weights barrier, its parity) per layer
  bool bad = false;
#pragma unroll 1
  for (int l = 0; l < 4; l++) {
    const int N = l == 3 ? 64 : H, KC = l == 0 ? 1 : NC, brows = l == 0 ? H : N;
    unsigned char* Bs = (l == 1 || l == 2) ? wbig : wsm;
    if (tid == 0) {
      if (!ktc::mbar_wait(&bars[wait_parity[l][0]], wait_parity[l][1])) {
        *abort_flag = 1;
      } else {
        ktc::tc_fence_after();
        const uint32_t idesc = ktc::bf16_idesc(TC_M, N);
        for (int kc = 0; kc < KC; kc++)
          for (int ks = 0; ks < 4; ks++) {
            const uint64_t ad = ktc::sw128_desc(ktc::smem_u32(act) + kc * TC_M * 128 + ks * 32);
            const uint64_t bd = ktc::sw128_desc(ktc::smem_u32(Bs) + kc * brows * 128 + ks * 32);
            ktc::mma_bf16(tmem, ad, bd, idesc, (kc | ks) != 0);
          }
        ktc::mma_commit(&bars[2]);
      }
    }
    __syncthreads();
    if (*abort_flag) { bad = true; break; }
    if (!ktc::mbar_wait(&bars[2], (uint32_t)(l & 1))) bad = true;
    if (__syncthreads_or(bad)) { bad = true; break; }
    ktc::tc_fence_after();
    if (tid == 0 && l == 0) {  // the first layer's weights are consumed: the output layer's [64][H] into their place
      ktc::mbar_expect_tx(&bars[0], (uint32_t)NC * 64u * 128u);
      for (int k = 0; k < NC; k++) ktc::tma_load_2d(wsm + (size_t)k * 64 * 128, &tw3, 64 * k, 0, &bars[0]);
    }
    if (tid == 0 && l == 1) {  // the first hidden layer's weights are consumed: the second's into their place
      ktc::mbar_expect_tx(&bars[1], (uint32_t)NC * H * 128u);
      for (int k = 0; k < NC; k++) ktc::tma_load_2d(wbig + (size_t)k * H * 128, &tw2, 64 * k, 0, &bars[1]);
    }
    const uint32_t row_addr = tmem + ((uint32_t)(warp * 32) << 16);
    const float* bias = a.bias[l];
    if (l < 3) {  // bias + ReLU, BF16, over the activations this layer consumed
#pragma unroll 1
      for (int cb = 0; cb < (H >> 5); cb++) {
        float v[32];
        ktc::tmem_ld32(row_addr + cb * 32, v);
#pragma unroll
        for (int u = 0; u < 4; u++) {
          uint32_t w[4];
#pragma unroll
          for (int e = 0; e < 4; e++) {
            const int k0 = cb * 32 + u * 8 + e * 2;
            __nv_bfloat162 b2 = __floats2bfloat162_rn(fmaxf(v[u * 8 + e * 2] + bias[k0], 0.f),
                                                      fmaxf(v[u * 8 + e * 2 + 1] + bias[k0 + 1], 0.f));
            w[e] = *reinterpret_cast<uint32_t*>(&b2);
          }
          *reinterpret_cast<uint4*>(act + ktc::sw128_offset(tid, cb * 32 + u * 8, TC_M)) =
              make_uint4(w[0], w[1], w[2], w[3]);
        }
      }
      ktc::fence_proxy_async();
      ktc::tc_fence_before();
      __syncthreads();
    } else {  // decode the output layer into the Newton start (every lane loads: warp-collective)
      float v[64];
      ktc::tmem_ld32(row_addr, v);
      ktc::tmem_ld32(row_addr + 32, v + 32);
      if (c < a.B) {
        const double sc = a.scale_col >= 0 ? a.vals[(int64_t)a.scale_col * a.B + c] : 1.0;
        for (int col = 0; col < a.n && col < 64; col++) {
          const double y = (double)v[col] + bias[col];
          a.x0[(size_t)c * a.n + col] = col < a.dout ? (y * a.tstd[col] + a.tmean[col]) * sc : 0.0;
        }
      }
    }
  }
  if (bad) {  // a wait gave up: report it, leave defined (zero) starts, wait briefly for copies in flight
    if (tid == 0) {
      atomicExch(a.err, 1);
      ktc::mbar_wait(&bars[0], 1, 100000000ull);
      ktc::mbar_wait(&bars[1], 1, 100000000ull);
    }
    if (c < a.B)
      for (int col = 0; col < a.n; col++) a.x0[(size_t)c * a.n + col] = 0.0;
  }
  ktc::tc_fence_before();
  __syncthreads();
  if (warp == 0) ktc::tmem_dealloc(tmem, 256);
}

}  // namespace

struct ks_mlp {
  int din, h, dout, dip, dop;  // dims and padded dims
  int nlayers = 4;
  int in_[4], out_[4], ldi[4], ldo[4];   // per layer fan-in/out (unpadded) and padded
  std::vector<size_t> woff, boff;        // offsets in the flat parameter vector
  size_t nparam = 0;
  float *w = nullptr, *g = nullptr, *m = nullptr, *v = nullptr;  // FP32 masters, grads, Adam moments
  __nv_bfloat16* Wq[4] = {};  // [out_pad][in_pad]
  __nv_bfloat16* WTq[4] = {}; // [in_pad][out_pad]
  float* bias_pad[4] = {};    // padded bias views (copies)
  // normalization
  float *fmean = nullptr, *fstd = nullptr, *tmean = nullptr, *tstd = nullptr;
  int32_t* fcols = nullptr;
  uint64_t logmask = 0;
  int scale_col = -1;  // targets are unknowns divided by this value column (-1: none)
  int adam_t = 0;
  // activations for a batch of up to cap rows
  int cap = 0;
  __nv_bfloat16 *X = nullptr, *H[3] = {}, *dH[3] = {}, *dYb = nullptr;
  float *Y = nullptr, *T = nullptr, *loss = nullptr;
  int32_t* idx = nullptr;
  // tcgen05 inference: TMA descriptors of the four BF16 weight matrices (encoded
  // once: the matrices stay where they are) and the kernel's error word
  CUtensorMap tmap[4];
  int tc_state = 0;  // 0: not tried, 1: ready, -1: descriptors not available
  int* tc_err = nullptr;
};

// TMA descriptor of a BF16 [rows][cols] row-major matrix, boxes of 64 columns x
// box_rows rows with 128-byte swizzle (the tcgen05 K-major operand layout).
typedef CUresult (*EncodeTiledFn)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*, const cuuint64_t*,
                                  const cuuint64_t*, const cuuint32_t*, const cuuint32_t*, CUtensorMapInterleave,
                                  CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

static int tc_prepare(ks_mlp* p) {
  if (p->tc_state) return p->tc_state;
  p->tc_state = -1;
  void* fn = nullptr;
  cudaDriverEntryPointQueryResult q;
  if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &fn, 12000, cudaEnableDefault, &q) != cudaSuccess ||
      q != cudaDriverEntryPointSuccess || !fn)
    return p->tc_state;
  EncodeTiledFn enc = reinterpret_cast<EncodeTiledFn>(fn);
  for (int l = 0; l < 4; l++) {
    cuuint64_t dims[2] = {(cuuint64_t)p->ldi[l], (cuuint64_t)p->ldo[l]};
    cuuint64_t strides[1] = {(cuuint64_t)p->ldi[l] * 2};
    cuuint32_t box[2] = {64, (cuuint32_t)p->ldo[l]};
    cuuint32_t estr[2] = {1, 1};
    if (enc(&p->tmap[l], CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, p->Wq[l], dims, strides, box, estr,
            CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
            CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) != CUDA_SUCCESS)
      return p->tc_state;
  }
  if (!p->tc_err && cudaMalloc(&p->tc_err, sizeof(int)) != cudaSuccess) return p->tc_state;
  if (cudaMemset(p->tc_err, 0, sizeof(int)) != cudaSuccess) return p->tc_state;
  if (cudaFuncSetAttribute(k_mlp_infer_tc, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)TC_SMEM) != cudaSuccess)
    return p->tc_state;
  p->tc_state = 1;
  return p->tc_state;
}

static int mlp_alloc_batch(ks_mlp* p, int rows) {
  int R = pad64(rows);
  if (R <= p->cap) return KS_OK;
  cudaFree(p->X); cudaFree(p->Y); cudaFree(p->T); cudaFree(p->dYb); cudaFree(p->idx);
  for (int i = 0; i < 3; i++) { cudaFree(p->H[i]); cudaFree(p->dH[i]); }
  bool ok = cudaMalloc(&p->X, (size_t)R * p->dip * 2) == cudaSuccess &&
            cudaMalloc(&p->Y, (size_t)R * p->dop * 4) == cudaSuccess &&
            cudaMalloc(&p->T, (size_t)R * p->dop * 4) == cudaSuccess &&
            cudaMalloc(&p->dYb, (size_t)R * p->dop * 2) == cudaSuccess &&
            cudaMalloc(&p->idx, (size_t)R * 4) == cudaSuccess;
  for (int i = 0; i < 3 && ok; i++)
    ok = cudaMalloc(&p->H[i], (size_t)R * p->h * 2) == cudaSuccess && cudaMalloc(&p->dH[i], (size_t)R * p->h * 2) == cudaSuccess;
  if (!ok) { set_error("ks_mlp: device allocation failed"); p->cap = 0; return KS_ENOMEM; }
  p->cap = R;
  return KS_OK;
}

template <bool AT, bool BT, int EPI>
static void gemm(const __nv_bfloat16* A, const __nv_bfloat16* B, void* C, const float* bias, const __nv_bfloat16* mask,
                 int M, int N, int K, int lda, int ldb, int ldc, int splits, cudaStream_t st) {
  int kchunk = (K + splits - 1) / splits;
  kchunk = (kchunk + BK - 1) / BK * BK;
  splits = (K + kchunk - 1) / kchunk;
  dim3 grid((N + BN - 1) / BN, (M + BM - 1) / BM, splits);  // M, N: logical bounds; tiles read padded storage
  k_gemm<AT, BT, EPI><<<grid, 128, 0, st>>>(A, B, C, bias, mask, M, N, K, lda, ldb, ldc, kchunk);
}

static void sync_weights(ks_mlp* p, cudaStream_t st) {
  for (int l = 0; l < p->nlayers; l++) {
    dim3 grid((p->in_[l] + 127) / 128, p->out_[l]);
    k_quantize<<<grid, 128, 0, st>>>(p->w + p->woff[l], p->out_[l], p->in_[l], p->Wq[l], p->ldi[l], p->WTq[l], p->ldo[l]);
    cudaMemcpyAsync(p->bias_pad[l], p->w + p->boff[l], sizeof(float) * p->out_[l], cudaMemcpyDeviceToDevice, st);
  }
}

// forward on p->X (rows R) -> p->H[*], p->Y
static void mlp_forward(ks_mlp* p, int R, cudaStream_t st) {
  gemm<false, false, EPI_RELU_BF16>(p->X, p->Wq[0], p->H[0], p->bias_pad[0], nullptr, R, p->ldo[0], p->ldi[0], p->dip,
                                    p->ldi[0], p->h, 1, st);
  gemm<false, false, EPI_RELU_BF16>(p->H[0], p->Wq[1], p->H[1], p->bias_pad[1], nullptr, R, p->h, p->h, p->h, p->h, p->h, 1, st);
  gemm<false, false, EPI_RELU_BF16>(p->H[1], p->Wq[2], p->H[2], p->bias_pad[2], nullptr, R, p->h, p->h, p->h, p->h, p->h, 1, st);
  gemm<false, false, EPI_LINEAR_F32>(p->H[2], p->Wq[3], p->Y, p->bias_pad[3], nullptr, R, p->dop, p->h, p->h, p->h, p->dop, 1, st);
}

// backward from p->dYb; accumulates into p->g (zeroed by the caller)
static void mlp_backward(ks_mlp* p, int R, cudaStream_t st) {
  int splits = R / 256 > 1 ? R / 256 : 1;  // K = rows: 256-row chunks fill the SMs at the minibatch sizes
  const __nv_bfloat16* acts[4] = {p->X, p->H[0], p->H[1], p->H[2]};
  const __nv_bfloat16* dout = p->dYb;
  int ldd = p->dop;
  for (int l = 3; l >= 0; l--) {
    // dW_l[o][i] += sum_r dout[r][o] * act[r][i]:  A = dout^T (stored [R][o]), B = act (stored [R][i])
    gemm<true, true, EPI_ATOMIC_F32>(dout, acts[l], p->g + p->woff[l], nullptr, nullptr, p->out_[l], p->in_[l], R, ldd,
                                     p->ldi[l], p->in_[l], splits, st);
    dim3 cg((p->out_[l] + 127) / 128, (R + KS_COLSUM_ROWS - 1) / KS_COLSUM_ROWS);
    k_colsum<<<cg, 128, 0, st>>>(dout, R, p->out_[l], ldd, p->g + p->boff[l]);
    if (l == 0) break;
    // dact[r][i] = sum_o dout[r][o] W[o][i], masked by the ReLU of layer l-1
    gemm<false, false, EPI_MASK_BF16>(dout, p->WTq[l], p->dH[l - 1], nullptr, acts[l], R, p->ldi[l], p->ldo[l], ldd,
                                      p->ldo[l], p->ldi[l], 1, st);
    dout = p->dH[l - 1];
    ldd = p->h;
  }
}

extern "C" int ks_mlp_create(int32_t in_dim, int32_t hidden, int32_t out_dim, uint64_t seed, ks_mlp** out) {
  if (in_dim <= 0 || in_dim > 64 || out_dim <= 0 || out_dim > 64 || hidden <= 0 || hidden % 64 || !out) {
    set_error("ks_mlp_create: dimensions (in <= 64, out <= 64, hidden a multiple of 64)");
    return KS_EINVAL;
  }
  ks_mlp* p = new ks_mlp();
  p->din = in_dim; p->h = hidden; p->dout = out_dim; p->dip = pad64(in_dim); p->dop = pad64(out_dim);
  int ins[4] = {in_dim, hidden, hidden, hidden}, outs[4] = {hidden, hidden, hidden, out_dim};
  int insp[4] = {p->dip, hidden, hidden, hidden}, outsp[4] = {hidden, hidden, hidden, p->dop};
  size_t off = 0;
  for (int l = 0; l < 4; l++) {
    p->in_[l] = ins[l]; p->out_[l] = outs[l]; p->ldi[l] = insp[l]; p->ldo[l] = outsp[l];
    p->woff.push_back(off); off += (size_t)outs[l] * ins[l];
    p->boff.push_back(off); off += outs[l];
  }
  p->nparam = off;
  // He-uniform initial weights from a fixed-seed generator, zero biases
  std::vector<float> w(off, 0.f);
  uint64_t s = seed * 6364136223846793005ULL + 1442695040888963407ULL;
  auto rnd = [&]() { s = s * 6364136223846793005ULL + 1442695040888963407ULL; return ((s >> 11) * (1.0 / 9007199254740992.0)) * 2 - 1; };
  for (int l = 0; l < 4; l++) {
    float a = sqrtf(6.f / ins[l]) * (l == 3 ? 0.5f : 1.f);
    for (size_t i = 0; i < (size_t)outs[l] * ins[l]; i++) w[p->woff[l] + i] = (float)(a * rnd());
  }
  bool ok = cudaMalloc(&p->w, off * 4) == cudaSuccess && cudaMalloc(&p->g, off * 4) == cudaSuccess &&
            cudaMalloc(&p->m, off * 4) == cudaSuccess && cudaMalloc(&p->v, off * 4) == cudaSuccess &&
            cudaMalloc(&p->fmean, 64 * 4) == cudaSuccess && cudaMalloc(&p->fstd, 64 * 4) == cudaSuccess &&
            cudaMalloc(&p->tmean, 64 * 4) == cudaSuccess && cudaMalloc(&p->tstd, 64 * 4) == cudaSuccess &&
            cudaMalloc(&p->fcols, 64 * 4) == cudaSuccess;
  for (int l = 0; l < 4 && ok; l++)
    ok = cudaMalloc(&p->Wq[l], (size_t)p->ldo[l] * p->ldi[l] * 2) == cudaSuccess &&
         cudaMalloc(&p->WTq[l], (size_t)p->ldo[l] * p->ldi[l] * 2) == cudaSuccess &&
         cudaMalloc(&p->bias_pad[l], (size_t)p->ldo[l] * 4) == cudaSuccess;
  if (!ok) { set_error("ks_mlp_create: device allocation failed"); return KS_ENOMEM; }
  for (int l = 0; l < 4; l++) {
    cudaMemset(p->Wq[l], 0, (size_t)p->ldo[l] * p->ldi[l] * 2);
    cudaMemset(p->WTq[l], 0, (size_t)p->ldo[l] * p->ldi[l] * 2);
    cudaMemset(p->bias_pad[l], 0, (size_t)p->ldo[l] * 4);
  }
  cudaMemcpy(p->w, w.data(), off * 4, cudaMemcpyHostToDevice);
  cudaMemset(p->m, 0, off * 4);
  cudaMemset(p->v, 0, off * 4);
  std::vector<float> one(64, 1.f), zero(64, 0.f);
  cudaMemcpy(p->fmean, zero.data(), 256, cudaMemcpyHostToDevice);
  cudaMemcpy(p->tmean, zero.data(), 256, cudaMemcpyHostToDevice);
  cudaMemcpy(p->fstd, one.data(), 256, cudaMemcpyHostToDevice);
  cudaMemcpy(p->tstd, one.data(), 256, cudaMemcpyHostToDevice);
  sync_weights(p, nullptr);
  if (cudaDeviceSynchronize() != cudaSuccess) { set_error("ks_mlp_create: CUDA error"); return KS_ECUDA; }
  *out = p;
  return KS_OK;
}

extern "C" void ks_mlp_destroy(ks_mlp* p) {
  if (!p) return;
  cudaFree(p->w); cudaFree(p->g); cudaFree(p->m); cudaFree(p->v);
  cudaFree(p->fmean); cudaFree(p->fstd); cudaFree(p->tmean); cudaFree(p->tstd); cudaFree(p->fcols);
  for (int l = 0; l < 4; l++) { cudaFree(p->Wq[l]); cudaFree(p->WTq[l]); cudaFree(p->bias_pad[l]); }
  cudaFree(p->X); cudaFree(p->Y); cudaFree(p->T); cudaFree(p->dYb); cudaFree(p->idx); cudaFree(p->loss);
  for (int i = 0; i < 3; i++) { cudaFree(p->H[i]); cudaFree(p->dH[i]); }
  cudaFree(p->tc_err);
  delete p;
}

extern "C" int ks_mlp_num_params(const ks_mlp* p, int64_t* n) {
  if (!p || !n) return KS_EINVAL;
  *n = (int64_t)p->nparam;
  return KS_OK;
}

extern "C" int ks_mlp_get_params(const ks_mlp* p, float* host) {
  if (!p || !host) return KS_EINVAL;
  return cudaMemcpy(host, p->w, p->nparam * 4, cudaMemcpyDeviceToHost) == cudaSuccess ? KS_OK : KS_ECUDA;
}

extern "C" int ks_mlp_set_params(ks_mlp* p, const float* host) {
  if (!p || !host) return KS_EINVAL;
  if (cudaMemcpy(p->w, host, p->nparam * 4, cudaMemcpyHostToDevice) != cudaSuccess) return KS_ECUDA;
  sync_weights(p, nullptr);
  return cudaDeviceSynchronize() == cudaSuccess ? KS_OK : KS_ECUDA;
}

// Features: value columns `cols` (log-transformed where logmask has the bit),
// standardized by fmean/fstd; targets: the first out_dim unknowns, by tmean/tstd.
extern "C" int ks_mlp_set_io(ks_mlp* p, const int32_t* cols, uint64_t logmask, const float* fmean, const float* fstd,
                             const float* tmean, const float* tstd, int32_t scale_col) {
  if (!p || !cols || !fmean || !fstd || !tmean || !tstd) return KS_EINVAL;
  p->scale_col = scale_col;
  cudaMemcpy(p->fcols, cols, p->din * 4, cudaMemcpyHostToDevice);
  cudaMemcpy(p->fmean, fmean, p->din * 4, cudaMemcpyHostToDevice);
  cudaMemcpy(p->fstd, fstd, p->din * 4, cudaMemcpyHostToDevice);
  cudaMemcpy(p->tmean, tmean, p->dout * 4, cudaMemcpyHostToDevice);
  cudaMemcpy(p->tstd, tstd, p->dout * 4, cudaMemcpyHostToDevice);
  p->logmask = logmask;
  return cudaDeviceSynchronize() == cudaSuccess ? KS_OK : KS_ECUDA;
}

// One forward + backward on host data (standardized X [rows][in], T [rows][out]);
// grads (FP32, parameter layout) and the loss come back to the host.  For the
// gradient check against the CPU oracle network.
extern "C" int ks_mlp_grad(ks_mlp* p, const float* X, const float* T, int32_t rows, float* grads, float* loss) {
  if (!p || !X || !T || rows <= 0) return KS_EINVAL;
  int rc = mlp_alloc_batch(p, rows);
  if (rc) return rc;
  int R = pad64(rows);
  std::vector<__nv_bfloat16> xb((size_t)R * p->dip, __float2bfloat16(0.f));
  std::vector<float> tb((size_t)R * p->dop, 0.f);
  for (int r = 0; r < rows; r++) {
    for (int j = 0; j < p->din; j++) xb[(size_t)r * p->dip + j] = __float2bfloat16(X[(size_t)r * p->din + j]);
    for (int j = 0; j < p->dout; j++) tb[(size_t)r * p->dop + j] = T[(size_t)r * p->dout + j];
  }
  cudaMemcpy(p->X, xb.data(), xb.size() * 2, cudaMemcpyHostToDevice);
  cudaMemcpy(p->T, tb.data(), tb.size() * 4, cudaMemcpyHostToDevice);
  if (!p->loss && cudaMalloc(&p->loss, 4) != cudaSuccess) return KS_ENOMEM;
  cudaMemset(p->loss, 0, 4);
  cudaMemset(p->g, 0, p->nparam * 4);
  mlp_forward(p, R, nullptr);
  dim3 blk(64, 4);
  k_loss_grad<<<(R + 3) / 4, blk>>>(p->Y, p->T, p->dout, p->dop, rows, p->dYb, R, p->loss);
  mlp_backward(p, R, nullptr);
  if (cudaDeviceSynchronize() != cudaSuccess) { set_error("ks_mlp_grad: CUDA error"); return KS_ECUDA; }
  if (grads) cudaMemcpy(grads, p->g, p->nparam * 4, cudaMemcpyDeviceToHost);
  if (loss) cudaMemcpy(loss, p->loss, 4, cudaMemcpyDeviceToHost);
  return KS_OK;
}

// Train on the circuits of a batch: features from the batch's values, targets from
// solutions x_dev [B][n] (device), rows with status_dev != 0 skipped by the caller's
// index list idx_dev (device, n_train entries).  `epochs` passes of minibatches of
// `mb` rows in the order of idx (the caller shuffles).  Returns the last epoch's mean loss.
extern "C" int ks_mlp_train(ks_mlp* p, ks_batch* b, const double* x_dev, const int32_t* idx_dev, int32_t n_train,
                            int32_t epochs, int32_t mb, float lr, float* last_loss, void* stream);

// Predict Newton starting points x0_dev [B][n] for every circuit of a batch.
extern "C" int ks_mlp_predict(ks_mlp* p, ks_batch* b, double* x0_dev, void* stream);

// The batch's SoA value array and shape (for the two calls above).
int ks_batch_values_view(ks_batch* b, const double** vals, int64_t* B, int* n);

extern "C" int ks_mlp_train(ks_mlp* p, ks_batch* b, const double* x_dev, const int32_t* idx_dev, int32_t n_train,
                            int32_t epochs, int32_t mb, float lr, float* last_loss, void* stream) {
  if (!p || !b || !x_dev || !idx_dev || n_train <= 0 || epochs <= 0 || mb <= 0 || mb % 64) return KS_EINVAL;
  cudaStream_t st = (cudaStream_t)stream;
  const double* vals;
  int64_t B;
  int n;
  ks_batch_values_view(b, &vals, &B, &n);
  if (p->dout > n) { set_error("ks_mlp_train: more outputs than unknowns"); return KS_EINVAL; }
  int rc = mlp_alloc_batch(p, mb);
  if (rc) return rc;
  if (!p->loss && cudaMalloc(&p->loss, 4) != cudaSuccess) return KS_ENOMEM;
  const float b1 = 0.9f, b2 = 0.999f, eps = 1e-8f;
  float lsum = 0.f;
  int nb = 0;
  for (int ep = 0; ep < epochs; ep++) {
    lsum = 0.f; nb = 0;
    for (int r0 = 0; r0 + mb <= n_train; r0 += mb) {
      cudaMemcpyAsync(p->idx, idx_dev + r0, mb * 4, cudaMemcpyDeviceToDevice, st);
      dim3 blk(64, 4);
      k_features<<<(mb + 3) / 4, blk, 0, st>>>(vals, B, p->idx, p->fcols, p->logmask, p->fmean, p->fstd, p->din, p->dip,
                                               mb, p->X, mb);
      k_targets<<<(mb + 3) / 4, blk, 0, st>>>(x_dev, n, p->idx, p->tmean, p->tstd, p->dout, p->dop, mb, p->T, mb, vals,
                                              B, p->scale_col);
      cudaMemsetAsync(p->loss, 0, 4, st);
      cudaMemsetAsync(p->g, 0, p->nparam * 4, st);
      mlp_forward(p, mb, st);
      k_loss_grad<<<(mb + 3) / 4, blk, 0, st>>>(p->Y, p->T, p->dout, p->dop, mb, p->dYb, mb, p->loss);
      mlp_backward(p, mb, st);
      p->adam_t++;
      float c1 = 1.f - powf(b1, (float)p->adam_t), c2 = 1.f - powf(b2, (float)p->adam_t);
      k_adam<<<(unsigned)((p->nparam + 255) / 256), 256, 0, st>>>(p->w, p->g, p->m, p->v, (int)p->nparam, lr, b1, b2, eps, c1, c2);
      sync_weights(p, st);
      if (ep == epochs - 1) {
        float l = 0.f;
        cudaMemcpyAsync(&l, p->loss, 4, cudaMemcpyDeviceToHost, st);
        cudaStreamSynchronize(st);
        lsum += l; nb++;
      }
    }
  }
  if (cudaStreamSynchronize(st) != cudaSuccess) { set_error("ks_mlp_train: CUDA error"); return KS_ECUDA; }
  if (last_loss) *last_loss = nb ? lsum / nb : 0.f;
  return KS_OK;
}

extern "C" int ks_mlp_predict(ks_mlp* p, ks_batch* b, double* x0_dev, void* stream) {
  if (!p || !b || !x0_dev) return KS_EINVAL;
  cudaStream_t st = (cudaStream_t)stream;
  const double* vals;
  int64_t B;
  int n;
  ks_batch_values_view(b, &vals, &B, &n);
  int rc = mlp_alloc_batch(p, (int)B);
  if (rc) return rc;
  int R = pad64((int)B);
  if (p->h % 64 == 0 && p->h <= 256 && p->dip == 64 && p->dop == 64 && n <= 64 && tc_prepare(p) == 1) {
    TcArgs a;  // the tcgen05 kernel
    a.vals = vals; a.B = B; a.n = n; a.cols = p->fcols; a.logmask = p->logmask; a.fmean = p->fmean; a.fstd = p->fstd;
    a.din = p->din; a.h = p->h; a.dout = p->dout;
    for (int l = 0; l < 4; l++) a.bias[l] = p->bias_pad[l];
    a.tmean = p->tmean; a.tstd = p->tstd; a.scale_col = p->scale_col; a.x0 = x0_dev; a.err = p->tc_err;
    k_mlp_infer_tc<<<(unsigned)((B + TC_M - 1) / TC_M), TC_M, TC_SMEM, st>>>(a, p->tmap[0], p->tmap[1], p->tmap[2],
                                                                             p->tmap[3]);
    return cudaGetLastError() == cudaSuccess ? KS_OK : KS_ECUDA;
  }
  if (p->h % 64 == 0 && p->h <= 256 && p->dip <= p->h && p->dop == 64 && n <= 64) {  // the fused kernel's shapes
    InferArgs a;
    a.vals = vals; a.B = B; a.n = n; a.cols = p->fcols; a.logmask = p->logmask; a.fmean = p->fmean; a.fstd = p->fstd;
    a.din = p->din; a.dip = p->dip; a.h = p->h; a.dout = p->dout; a.dop = p->dop;
    for (int l = 0; l < 4; l++) { a.W[l] = p->Wq[l]; a.bias[l] = p->bias_pad[l]; }
    a.tmean = p->tmean; a.tstd = p->tstd; a.scale_col = p->scale_col; a.x0 = x0_dev;
    size_t smem = sizeof(__nv_bfloat16) * ((size_t)IR * (p->h + PAD) + (size_t)IR * (p->dip + PAD) +
                                           (size_t)p->h * (p->h + PAD));
    cudaFuncSetAttribute(k_mlp_infer, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    k_mlp_infer<<<(unsigned)((B + IR - 1) / IR), 256, smem, st>>>(a);
    return cudaGetLastError() == cudaSuccess ? KS_OK : KS_ECUDA;
  }
  dim3 blk(64, 4);
  k_features<<<(R + 3) / 4, blk, 0, st>>>(vals, B, nullptr, p->fcols, p->logmask, p->fmean, p->fstd, p->din, p->dip,
                                          (int)B, p->X, R);
  mlp_forward(p, R, st);
  dim3 blk2(32, 8);
  k_decode<<<(unsigned)((B + 7) / 8), blk2, 0, st>>>(p->Y, p->dop, p->dout, p->tmean, p->tstd, x0_dev, n, (int)B, vals,
                                                     B, p->scale_col);
  return cudaGetLastError() == cudaSuccess ? KS_OK : KS_ECUDA;
}
