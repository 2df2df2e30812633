// Proposal network: a small CNN that maps a reference/target subset pair to the six
// first-order warp parameters, so IC-GN starts close to the answer.  No counterpart in the
// reference; the architecture is the one the learned-seed workload names:
//
//   x0  [2, 31, 31]  reference and target windows at the POI, each zero-mean, unit-variance
//   c1  3x3 stride 2 pad 1, 2 -> 32, ReLU      -> [32, 16, 16]
//   c2  3x3 stride 2 pad 1, 32 -> 32, ReLU     -> [32, 8, 8]
//   c3  3x3 stride 2 pad 1, 32 -> 32, ReLU     -> [32, 4, 4]
//   c4  3x3 stride 2 pad 1, 32 -> 32, ReLU     -> [32, 2, 2]
//   f1  128 -> 256, ReLU
//   f2  256 -> 6: (u, v, 100 ux, 100 uy, 100 vx, 100 vy)
//
// Activations are BF16 in NHWC order (channels fastest), weights are kept in FP32 (master)
// with BF16 working copies, and every product runs on the tensor cores with FP32
// accumulation.  Training: one GEMM kernel (mma.sync.m16n8k16 bf16) serves all layers and
// passes; an operand functor gathers its A and B tiles (implicit im2col for the
// convolutions) and an epilogue functor stores the result.  Inference (k_proposal_fused)
// runs conv2, its largest layer, as tcgen05.mma from shared-memory descriptors into TMEM.
#pragma once

#include <cuda_bf16.h>
#include <cstdint>

#include "dic_kernels.cuh"   // mbarrier helpers

namespace dic
{
namespace cnn
{

constexpr int kWin = 31;          // input window side
constexpr int kCh = 32;           // conv channels
constexpr int kHidden = 256;
constexpr int kOut = 6;
constexpr int kOutPad = 8;
constexpr int kC1K = 32;          // conv1 K = 3*3*2 = 18, padded to 32

// Spatial sides: input 31, then 16, 8, 4, 2.
__host__ __device__ constexpr int side_of(int layer) { return layer == 0 ? 31 : (32 >> layer); }

// FP32 master parameter layout (offsets in floats).  Conv weights are [co][ky][kx][ci].
struct ParamLayout
{
  static constexpr int w1 = 0, b1 = w1 + 32 * 9 * 2;
  static constexpr int w2 = b1 + 32, b2 = w2 + 32 * 9 * 32;
  static constexpr int w3 = b2 + 32, b3 = w3 + 32 * 9 * 32;
  static constexpr int w4 = b3 + 32, b4 = w4 + 32 * 9 * 32;
  static constexpr int w5 = b4 + 32, b5 = w5 + kHidden * 128;   // [256][128], k = (y, x, c)
  static constexpr int w6 = b5 + kHidden, b6 = w6 + kOut * kHidden;  // [6][256]
  static constexpr int count = b6 + kOut;
};
static_assert(ParamLayout::count == 62918, "parameter count");

// BF16 working copies, B operands stored [n][k] with k contiguous and K padded:
//   c1: [32][32], c2..c4: [32][288], f1: [256][128], f2: [8][256] (rows 6, 7 zero).
struct WeightLayout
{
  static constexpr int c1 = 0, c2 = c1 + 32 * kC1K, c3 = c2 + 32 * 288, c4 = c3 + 32 * 288;
  static constexpr int f1 = c4 + 32 * 288, f2 = f1 + kHidden * 128;
  static constexpr int count = f2 + kOutPad * kHidden;
};

__device__ __forceinline__ uint32_t pack_bf16(__nv_bfloat16 lo, __nv_bfloat16 hi)
{
  return (uint32_t)__bfloat16_as_ushort(lo) | ((uint32_t)__bfloat16_as_ushort(hi) << 16);
}

__device__ __forceinline__ void mma_bf16_16816(float (&c)[4], const uint32_t (&a)[4], const uint32_t (&b)[2])
{
  asm volatile(
      "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
      "{%0,%1,%2,%3};\n"
      : "+f"(c[0]), "+f"(c[1]), "+f"(c[2]), "+f"(c[3])
      : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b[0]), "r"(b[1]));
}

// --------------------------------------------------------------------------------------
// Generic GEMM: C[M x N] = A[M x K] * B[K x N] over k in [k_lo, k_hi) of this split.
// CTA tile 64 x 32 x 32, 4 warps, each warp 16 rows x 32 columns (four m16n8k16 per
// k16 step).  Op supplies M, N, K, splits, a(m, k), b(k, n) (BF16, 0 outside), and
// store(split, m, n, value) for the FP32 accumulator.
// --------------------------------------------------------------------------------------
constexpr int BM = 64, BN = 32, BK = 32;

template <class Op>
__global__ void __launch_bounds__(128) k_gemm(Op op)
{
  __shared__ __nv_bfloat16 As[BM][BK + 8];
  __shared__ __nv_bfloat16 Bs[BN][BK + 8];
  const int m0 = blockIdx.x * BM, n0 = blockIdx.y * BN;
  const int split = blockIdx.z;
  const int64_t kper = ((op.K + BK - 1) / BK + op.splits - 1) / op.splits * BK;
  const int64_t k_lo = (int64_t)split * kper;
  const int64_t k_hi = k_lo + kper < op.K ? k_lo + kper : op.K;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, g = lane >> 2, t4 = lane & 3;
  float acc[4][4];
#pragma unroll
  for (int j = 0; j < 4; ++j)
#pragma unroll
    for (int q = 0; q < 4; ++q) acc[j][q] = 0.f;
  for (int64_t k0 = k_lo; k0 < k_hi; k0 += BK)
  {
    for (int e = threadIdx.x; e < BM * BK; e += blockDim.x)
    {
      const int r = e / BK, c = e % BK;
      const int64_t k = k0 + c;
      As[r][c] = (k < k_hi) ? op.a(m0 + r, k) : __float2bfloat16(0.f);
    }
    for (int e = threadIdx.x; e < BN * BK; e += blockDim.x)
    {
      const int r = e / BK, c = e % BK;
      const int64_t k = k0 + c;
      Bs[r][c] = (k < k_hi) ? op.b(k, n0 + r) : __float2bfloat16(0.f);
    }
    __syncthreads();
#pragma unroll
    for (int kk = 0; kk < BK; kk += 16)
    {
      const int r = warp * 16 + g, c = kk + t4 * 2;
      uint32_t a[4];
      a[0] = pack_bf16(As[r][c], As[r][c + 1]);
      a[1] = pack_bf16(As[r + 8][c], As[r + 8][c + 1]);
      a[2] = pack_bf16(As[r][c + 8], As[r][c + 9]);
      a[3] = pack_bf16(As[r + 8][c + 8], As[r + 8][c + 9]);
#pragma unroll
      for (int j = 0; j < 4; ++j)
      {
        const int nn = j * 8 + g;
        uint32_t b[2];
        b[0] = pack_bf16(Bs[nn][c], Bs[nn][c + 1]);
        b[1] = pack_bf16(Bs[nn][c + 8], Bs[nn][c + 9]);
        mma_bf16_16816(acc[j], a, b);
      }
    }
    __syncthreads();
  }
  const int r0 = m0 + warp * 16 + g;
#pragma unroll
  for (int j = 0; j < 4; ++j)
  {
    const int c = n0 + j * 8 + t4 * 2;
    op.store(split, r0, c, acc[j][0]);
    op.store(split, r0, c + 1, acc[j][1]);
    op.store(split, r0 + 8, c, acc[j][2]);
    op.store(split, r0 + 8, c + 1, acc[j][3]);
  }
}

__device__ __forceinline__ __nv_bfloat16 bz() { return __float2bfloat16(0.f); }

// Convolution geometry: input side si, channels ci; output side so = si / 2 rounded up
// (3x3, stride 2, pad 1).  Activations NHWC: act[((n * s + y) * s + x) * c + ch].
struct ConvGeom
{
  int si, so, ci, co;
  int kdim() const { return 9 * ci; }
};

// Forward: A[m = (n, oy, ox)][k = (ky, kx, ci)] = in[n, 2oy+ky-1, 2ox+kx-1, ci],
// B[k][n = co] = W[co][k]; store z + bias, ReLU, BF16.
struct ConvFwdOp
{
  const __nv_bfloat16* in;
  const __nv_bfloat16* w;   // [co][kpad]
  const float* bias;
  __nv_bfloat16* out;
  int64_t M;
  int N, splits;
  int64_t K;                // padded K
  int si, so, ci, kreal, kpad;
  __device__ __nv_bfloat16 a(int64_t m, int64_t k) const
  {
    if (m >= M || k >= kreal) return bz();
    const int64_t n = m / (so * so);
    const int p = (int)(m % (so * so)), oy = p / so, ox = p % so;
    const int c = (int)(k % ci), kk = (int)(k / ci), ky = kk / 3, kx = kk % 3;
    const int iy = 2 * oy + ky - 1, ix = 2 * ox + kx - 1;
    if (iy < 0 || ix < 0 || iy >= si || ix >= si) return bz();
    return in[((n * si + iy) * si + ix) * ci + c];
  }
  __device__ __nv_bfloat16 b(int64_t k, int n) const { return n < N ? w[(int64_t)n * kpad + k] : bz(); }
  __device__ void store(int, int64_t m, int n, float v) const
  {
    if (m >= M || n >= N) return;
    out[m * N + n] = __float2bfloat16(fmaxf(v + bias[n], 0.f));
  }
};

// Backward data: dIn[m = (n, iy, ix)][c] = sum over (ky, kx, co) of
// dZ[n, oy, ox, co] W[co][ky][kx][c] with iy = 2oy+ky-1; then the ReLU mask of the input
// activation (act > 0), stored BF16 as the previous layer's dZ.
struct ConvBwdDataOp
{
  const __nv_bfloat16* dz;    // [N][so][so][co]
  const __nv_bfloat16* w;     // [co][kpad], k = (ky, kx, ci)
  const __nv_bfloat16* act;   // input activation [N][si][si][ci] (ReLU output)
  __nv_bfloat16* dzin;        // [N][si][si][ci]
  int64_t M;
  int N, splits;
  int64_t K;                  // 9 * co
  int si, so, ci, co, kpad;
  __device__ __nv_bfloat16 a(int64_t m, int64_t k) const
  {
    if (m >= M || k >= K) return bz();
    const int64_t n = m / (si * si);
    const int p = (int)(m % (si * si)), iy = p / si, ix = p % si;
    const int o = (int)(k % co), kk = (int)(k / co), ky = kk / 3, kx = kk % 3;
    const int ty = iy + 1 - ky, tx = ix + 1 - kx;
    if (ty < 0 || tx < 0 || (ty & 1) || (tx & 1)) return bz();
    const int oy = ty >> 1, ox = tx >> 1;
    if (oy >= so || ox >= so) return bz();
    return dz[((n * so + oy) * so + ox) * co + o];
  }
  __device__ __nv_bfloat16 b(int64_t k, int c) const
  {
    if (c >= N || k >= K) return bz();
    const int o = (int)(k % co), kk = (int)(k / co);
    return w[(int64_t)o * kpad + kk * ci + c];
  }
  __device__ void store(int, int64_t m, int c, float v) const
  {
    if (m >= M || c >= N) return;
    const int64_t i = m * N + c;
    dzin[i] = __float2bfloat16(__bfloat162float(act[i]) > 0.f ? v : 0.f);
  }
};

// Backward weights: dW[co][k = (ky, kx, ci)] = sum over (n, oy, ox) of dZ[n, oy, ox, co] *
// in[n, 2oy+ky-1, 2ox+kx-1, ci]; split-K partials go to part[split][co][kpad] (FP32) and
// k_reduce_splits sums them in a fixed order.
struct ConvBwdWeightOp
{
  const __nv_bfloat16* dz;    // [Nb][so][so][co]
  const __nv_bfloat16* in;    // [Nb][si][si][ci]
  float* part;
  int64_t M;                  // co
  int N, splits;              // N = kpad columns
  int64_t K;                  // Nb * so * so
  int si, so, ci, co, kreal, kpad;
  __device__ __nv_bfloat16 a(int64_t m, int64_t k) const
  {
    if (m >= M || k >= K) return bz();
    return dz[k * co + m];
  }
  __device__ __nv_bfloat16 b(int64_t k, int col) const
  {
    if (col >= kreal || k >= K) return bz();
    const int64_t n = k / (so * so);
    const int p = (int)(k % (so * so)), oy = p / so, ox = p % so;
    const int c = col % ci, kk = col / ci, ky = kk / 3, kx = kk % 3;
    const int iy = 2 * oy + ky - 1, ix = 2 * ox + kx - 1;
    if (iy < 0 || ix < 0 || iy >= si || ix >= si) return bz();
    return in[((n * si + iy) * si + ix) * ci + c];
  }
  __device__ void store(int split, int64_t m, int col, float v) const
  {
    if (m >= M || col >= N) return;
    part[((int64_t)split * M + m) * N + col] = v;
  }
};

// Dense forward: out[m][n] = act(sum_k in[m][k] W[n][k] + bias[n]).
struct LinearFwdOp
{
  const __nv_bfloat16* in;    // [M][K]
  const __nv_bfloat16* w;     // [Npad][K]
  const float* bias;
  __nv_bfloat16* out_bf;      // ReLU layer output (nullable)
  float* out_f;               // linear output (nullable), [M][ld]
  int64_t M;
  int N, splits;
  int64_t K;
  int ld;
  __device__ __nv_bfloat16 a(int64_t m, int64_t k) const { return m < M ? in[m * K + k] : bz(); }
  __device__ __nv_bfloat16 b(int64_t k, int n) const { return n < N ? w[(int64_t)n * K + k] : bz(); }
  __device__ void store(int, int64_t m, int n, float v) const
  {
    if (m >= M || n >= N) return;
    const float z = v + bias[n];
    if (out_bf) out_bf[m * N + n] = __float2bfloat16(fmaxf(z, 0.f));
    if (out_f) out_f[m * ld + n] = z;
  }
};

// Dense backward data: dIn[m][k] = sum_n dZ[m][n] W[n][k], masked by act[m][k] > 0.
struct LinearBwdDataOp
{
  const __nv_bfloat16* dz;    // [M][Nout]
  const __nv_bfloat16* w;     // [Npad][Kin]
  const __nv_bfloat16* act;   // [M][Kin]
  __nv_bfloat16* dzin;        // [M][Kin]
  int64_t M;
  int N, splits;              // N = Kin
  int64_t K;                  // Nout
  int nout_pad;
  __device__ __nv_bfloat16 a(int64_t m, int64_t k) const { return (m < M && k < K) ? dz[m * nout_pad + k] : bz(); }
  __device__ __nv_bfloat16 b(int64_t k, int c) const { return (c < N && k < K) ? w[k * N + c] : bz(); }
  __device__ void store(int, int64_t m, int c, float v) const
  {
    if (m >= M || c >= N) return;
    const int64_t i = m * N + c;
    dzin[i] = __float2bfloat16(__bfloat162float(act[i]) > 0.f ? v : 0.f);
  }
};

// Dense backward weights: dW[n][k] = sum_m dZ[m][n] in[m][k]; split-K partials.
struct LinearBwdWeightOp
{
  const __nv_bfloat16* dz;    // [Mb][ldz]
  const __nv_bfloat16* in;    // [Mb][Kin]
  float* part;                // [split][Nout][Kin]
  int64_t M;                  // Nout
  int N, splits;              // Kin
  int64_t K;                  // batch
  int ldz;
  __device__ __nv_bfloat16 a(int64_t m, int64_t k) const { return (m < M && k < K) ? dz[k * ldz + m] : bz(); }
  __device__ __nv_bfloat16 b(int64_t k, int c) const { return (c < N && k < K) ? in[k * N + c] : bz(); }
  __device__ void store(int split, int64_t m, int c, float v) const
  {
    if (m >= M || c >= N) return;
    part[((int64_t)split * M + m) * N + c] = v;
  }
};

// --------------------------------------------------------------------------------------
// Element kernels
// --------------------------------------------------------------------------------------

// Network input of one POI: the 31x31 reference and target windows centred on the POI's
// integer position (the target window is NOT shifted by any guess), each normalised to
// zero mean and unit variance.  Window pixels outside the image repeat the edge.  One warp
// per POI; x0 is NHWC [n][31][31][2].
__global__ void k_extract_input(const float* __restrict__ ref, const float* __restrict__ tar, int w, int h,
                                const dic_poi* __restrict__ pois, int64_t n, __nv_bfloat16* __restrict__ x0)
{
  const int lane = threadIdx.x & 31;
  const int64_t i = (int64_t)blockIdx.x * (blockDim.x / 32) + (threadIdx.x >> 5);
  if (i >= n) return;
  const int cx = (int)pois[i].x, cy = (int)pois[i].y;
  constexpr int R = kWin / 2, NPIX = kWin * kWin;
  float sr = 0.f, st = 0.f;
  for (int k = lane; k < NPIX; k += 32)
  {
    const int x = min(max(cx + k % kWin - R, 0), w - 1), y = min(max(cy + k / kWin - R, 0), h - 1);
    sr += ref[(size_t)y * w + x];
    st += tar[(size_t)y * w + x];
  }
  for (int o = 16; o > 0; o >>= 1)
  {
    sr += __shfl_xor_sync(0xffffffffu, sr, o);
    st += __shfl_xor_sync(0xffffffffu, st, o);
  }
  const float mr = sr / NPIX, mt = st / NPIX;
  float vr = 0.f, vt = 0.f;
  for (int k = lane; k < NPIX; k += 32)
  {
    const int x = min(max(cx + k % kWin - R, 0), w - 1), y = min(max(cy + k / kWin - R, 0), h - 1);
    const float a = ref[(size_t)y * w + x] - mr, b = tar[(size_t)y * w + x] - mt;
    vr += a * a;
    vt += b * b;
  }
  for (int o = 16; o > 0; o >>= 1)
  {
    vr += __shfl_xor_sync(0xffffffffu, vr, o);
    vt += __shfl_xor_sync(0xffffffffu, vt, o);
  }
  const float ir = vr > 0.f ? rsqrtf(vr / NPIX) : 1.f, it = vt > 0.f ? rsqrtf(vt / NPIX) : 1.f;
  __nv_bfloat16* out = x0 + i * NPIX * 2;
  for (int k = lane; k < NPIX; k += 32)
  {
    const int x = min(max(cx + k % kWin - R, 0), w - 1), y = min(max(cy + k / kWin - R, 0), h - 1);
    out[2 * k] = __float2bfloat16((ref[(size_t)y * w + x] - mr) * ir);
    out[2 * k + 1] = __float2bfloat16((tar[(size_t)y * w + x] - mt) * it);
  }
}

// FP32 master parameters -> BF16 working weights (padded GEMM layouts).
__global__ void k_pack_weights(const float* __restrict__ p, __nv_bfloat16* __restrict__ wb)
{
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  using P = ParamLayout;
  using L = WeightLayout;
  if (i < 32 * kC1K)
  {
    const int co = i / kC1K, k = i % kC1K;
    wb[L::c1 + i] = __float2bfloat16(k < 18 ? p[P::w1 + co * 18 + k] : 0.f);
  }
  if (i < 32 * 288)
  {
    wb[L::c2 + i] = __float2bfloat16(p[P::w2 + i]);
    wb[L::c3 + i] = __float2bfloat16(p[P::w3 + i]);
    wb[L::c4 + i] = __float2bfloat16(p[P::w4 + i]);
  }
  if (i < kHidden * 128) wb[L::f1 + i] = __float2bfloat16(p[P::w5 + i]);
  if (i < kOutPad * kHidden)
  {
    const int r = i / kHidden;
    wb[L::f2 + i] = __float2bfloat16(r < kOut ? p[P::w6 + i] : 0.f);
  }
}

// Output scaling: the network predicts (u, v, 100 ux, 100 uy, 100 vx, 100 vy).
__host__ __device__ constexpr float out_scale(int j) { return j < 2 ? 1.f : 100.f; }

// MSE over the six scaled outputs, mean over batch and outputs.  dout = dL/dout (BF16),
// per-row loss partial into row_loss (summed on the host side in a fixed order).
__global__ void k_loss_grad(const float* __restrict__ out, const float* __restrict__ target, int64_t n,
                            __nv_bfloat16* __restrict__ dout, float* __restrict__ row_loss)
{
  const int64_t m = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (m >= n) return;
  float l = 0.f;
  const float scale = 2.f / (float)(n * kOut);
#pragma unroll
  for (int j = 0; j < kOutPad; ++j)
  {
    float g = 0.f;
    if (j < kOut)
    {
      const float d = out[m * kOutPad + j] - target[m * kOut + j] * out_scale(j);
      l += d * d;
      g = d * scale;
    }
    dout[m * kOutPad + j] = __float2bfloat16(g);
  }
  row_loss[m] = l;
}

// Bias gradient: db[c] = sum over rows of dz[row][c] (BF16 rows of width ld), fixed order.
__global__ void k_bias_grad(const __nv_bfloat16* __restrict__ dz, int64_t rows, int ld, int ncol, float* __restrict__ db)
{
  const int c = blockIdx.x;
  if (c >= ncol) return;
  float s = 0.f;
  for (int64_t r = threadIdx.x; r < rows; r += blockDim.x) s += __bfloat162float(dz[r * ld + c]);
  __shared__ float red[256];
  red[threadIdx.x] = s;
  __syncthreads();
  for (int o = blockDim.x / 2; o > 0; o >>= 1)
  {
    if ((int)threadIdx.x < o) red[threadIdx.x] += red[threadIdx.x + o];
    __syncthreads();
  }
  if (threadIdx.x == 0) db[c] = red[0];
}

// Sum split-K partials part[s][rows][cols] in split order into out[r * out_ld + c] for
// c < keep (the unpadded columns).
__global__ void k_reduce_splits(const float* __restrict__ part, int splits, int rows, int cols, int keep,
                                float* __restrict__ out, int out_ld)
{
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= rows * keep) return;
  const int r = i / keep, c = i % keep;
  float s = 0.f;
  for (int k = 0; k < splits; ++k) s += part[((int64_t)k * rows + r) * cols + c];
  out[(int64_t)r * out_ld + c] = s;
}

// Adam (Kingma & Ba 2015) on the FP32 master parameters.
__global__ void k_adam(float* __restrict__ p, const float* __restrict__ g, float* __restrict__ m, float* __restrict__ v,
                       int n, float lr, float b1, float b2, float eps, float c1, float c2)
{
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const float gi = g[i];
  const float mi = b1 * m[i] + (1.f - b1) * gi;
  const float vi = b2 * v[i] + (1.f - b2) * gi * gi;
  m[i] = mi;
  v[i] = vi;
  p[i] -= lr * (mi / c1) / (sqrtf(vi / c2) + eps);
}

// Network output -> queue seed (u, ux, uy, v, vx, vy); result fields cleared.
__global__ void k_write_seeds(const float* __restrict__ out, dic_poi* __restrict__ pois, int64_t n)
{
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const float* o = out + i * kOutPad;
  dic_poi q = pois[i];
  q.u = o[0];
  q.v = o[1];
  q.ux = o[2] / out_scale(2);
  q.uy = o[3] / out_scale(3);
  q.vx = o[4] / out_scale(4);
  q.vy = o[5] / out_scale(5);
  q.u0 = 0.f; q.v0 = 0.f; q.zncc = 0.f; q.iteration = 0.f; q.convergence = 0.f; q.feature = 0.f;
  pois[i] = q;
}

// --------------------------------------------------------------------------------------
// Fused inference: the whole network, activations resident in shared memory, seeds written
// straight into the POI queue.  conv2 (62 % of the network's products) runs on tcgen05: a
// tile's two POIs are one M = 128 (2 POIs x 8 x 8 output pixels), N = 32, K = 288 product,
// 18 tcgen05.mma.kind::f16 issued by one thread from shared-memory descriptors, accumulated
// in 32 TMEM columns per warp group and read back with tcgen05.ld for the epilogue; the
// other layers use mma.sync.  One 512-thread CTA per SM holds two independent warp groups
// of 8 warps; each group runs tiles of kT = 2 POIs (tiles strided over groups and CTAs) and
// syncs on its own named barrier, so one group's serial phases (window staging, conv3/conv4,
// the MLP) overlap the other's conv1/conv2.  Same arithmetic as the GEMM path (BF16
// operands, FP32 accumulation, BF16 ReLU outputs), so both give the same seeds up to
// accumulation order.
//
// Shared memory (bytes), weights shared by the groups: W1 [32][40] 2.5 KB (rows padded to
// 80 B: the B-fragment loads of 8 rows x 4 lanes hit 32 distinct banks); W2..W4 [32][296]
// 57 KB (row padded to 37 16-byte chunks: conflict-free ldmatrix).  Per group: x0p
// [2][33][48][2] 12.4 KB (zero border; a 48-pixel row puts tap (ky, kx) at word
// 16 ky + kx mod 32, and conv1's K slots are grouped so that each A-fragment load reads taps
// {0, 16, 1, 17} or {2, 18, 1} words apart: 32 distinct banks for the 8 stride-2 rows x 4
// taps of a load); a1p [2][18][18][40] 50.6 KB and a2p [2][10][10][40] 15.6 KB (zero border,
// pixel stride 80 B); a4 [16][136] (conv4 outputs of 8 tiles, for the batched MLP).
// conv1's output a1c is conv2's A operand in the canonical no-swizzle K-major layout
// (core matrices of 8 rows x 16 B): four planes of 8 channels; in a plane, the padded rows
// of the two POIs interleaved as slots (row Y of POI p in slot (Y >> 1) * 2 + p, the even
// rows 0..16 first, then the odd rows 1..15), each slot 18 parity-split padded columns of
// 16 B.  For tap (ky, kx) and M row m = (2 oy + p) * 8 + ox the pixel (2 oy + ky, 2 ox + kx)
// then sits at a fixed base + (m >> 3) * 288 B + (m & 7) * 16 B: one descriptor per
// (tap, channel half) with SBO = 288 B (row slot) and LBO = one plane (next 8 channels).
// W2 is stored as B core matrices too: 8 output channels x 8 k per 128 B, LBO 512 B.
// The padded activation rows are stored parity-split: padded column X sits at
// (X & 1) * (width / 2) + (X >> 1), so the stride-2 im2col rows of an ldmatrix (8 output
// pixels, input columns 2 ox + kx) are 8 consecutive 80 B pixels, which cover all 32 banks.
// a3p [2][6][6][40] has its own region, so x0p takes the next tile's windows while conv2's
// products run; the split-K partials and a5 overlay the start of a1c once those products
// have completed.
// --------------------------------------------------------------------------------------
constexpr int kT = 2;                           // POIs per tile of a warp group
constexpr int kGroups = 2;                      // independent warp groups per CTA
constexpr int kGW = 8;                          // warps per group
constexpr int kGThreads = kGW * 32;             // 256
constexpr int kFusedThreads = kGroups * kGThreads;
constexpr int kPix = 40;                        // padded channel stride (80 B) of a1p/a2p/a3p
constexpr int kWRow = 296;                      // padded row of W2..W4 (288 + 8)
constexpr int kX0Row = 48;                      // x0p row stride in pixels (33 used)
constexpr int kSmX0 = kT * 33 * kX0Row * 2 * 2; // 12672
constexpr int kA1Slot = 18 * 16;                 // one padded row of one POI, 8 channels
constexpr int kA1Even = 9 * kT * kA1Slot;        // padded rows 0, 2, .., 16 of the tile's POIs
constexpr int kA1Plane = kA1Even + 8 * kT * kA1Slot;   // + rows 1, 3, .., 15: 9792 B
constexpr int kSmA1 = 4 * kA1Plane;              // 39168
static_assert(kT == 2, "conv2's M = 128 rows are the two POIs of a tile");
constexpr int kSmA2 = kT * 10 * 10 * kPix * 2;  // 16000
constexpr int kW1Row = 40;                      // padded row of W1 (32 + 8)
constexpr int kSmW1 = 32 * kW1Row * 2;          // 2560
constexpr int kSmW = 3 * 32 * kWRow * 2;        // 56832
// The MLP runs once per kMlpTiles tiles (16 POIs: one full m-tile), so its 64 KB of f1
// weights stream from L2 once per 16 POIs instead of once per tile.
constexpr int kMlpTiles = 8;
constexpr int kMlpRows = kMlpTiles * kT;         // 16
constexpr int kA4Row = 128 + 8, kA5Row = 256 + 8;   // rows padded by 16 B: distinct banks per fragment
constexpr int kSmA4 = kMlpRows * kA4Row * 2;     // 4352, persists across the batched tiles
constexpr int kSmOut = kMlpRows * 8 * 4;         // 512
constexpr int kSmPoi = kMlpTiles * 8;            // first POI of each batched tile
constexpr int kSmA3 = kT * 6 * 6 * kPix * 2;    // 5760
constexpr int kSmGroup = kSmX0 + kSmA1 + kSmA2 + kSmA3 + kSmA4 + kSmOut + kSmPoi;   // 78528
constexpr int kSmTotal = kSmW1 + kSmW + kGroups * kSmGroup;
// In a1p, free after conv2: conv4 split-K partials [4][16][32], f2 partials [8][16][8], a5
constexpr int kSmPart4 = 4 * 16 * 32 * 4, kSmPart2 = kGW * 16 * 8 * 4;
constexpr int kSmA5Off = kSmPart4 + kSmPart2;
constexpr int kSmScratch = kSmA5Off + kMlpRows * kA5Row * 2;
static_assert(kSmScratch <= kSmA1 && kSmA5Off % 16 == 0, "partials and a5 fit in a1c");
static_assert(kSmGroup % 16 == 0, "group regions stay 16-byte aligned");
static_assert(kSmTotal <= 227 * 1024, "shared memory");

// barrier of one warp group (ids 1.., 0 is __syncthreads)
__device__ __forceinline__ void group_sync(int grp)
{
  asm volatile("bar.sync %0, %1;\n" ::"r"(1 + grp), "r"(kGThreads) : "memory");
}

__device__ __forceinline__ uint32_t smem_u32(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

// conv1 K slot -> tap (ky * 3 + kx), or -1 for a zero slot; k = 2 slot + channel.  Each
// group of four slots is read by one A-fragment load (see the x0p row stride).
__device__ __forceinline__ int conv1_slot_tap(int slot)
{
  // {0, 3, 1, 4, 2, 5, 7, -, 6, -, -, -, 8, -, -, -}, four bits per slot, 15 = zero slot
  constexpr unsigned long long kTaps = 0xFFF8FFF6F7524130ull;
  const int t = (int)((kTaps >> (4 * slot)) & 15ull);
  return t == 15 ? -1 : t;
}

// storage column of padded column X in a parity-split row of WIDTH (even) padded columns
template <int WIDTH>
__device__ __forceinline__ int pcol(int X)
{
  return (X & 1) * (WIDTH / 2) + (X >> 1);
}

__device__ __forceinline__ void ldsm_x4(uint32_t (&r)[4], uint32_t addr)
{
  asm volatile("ldmatrix.sync.aligned.m8n8.x4.shared.b16 {%0,%1,%2,%3}, [%4];\n"
               : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3])
               : "r"(addr));
}

// byte offset of channel co of padded pixel (Y, X) of POI p in a1c
__device__ __forceinline__ int a1c_offset(int p, int Y, int X, int co)
{
  return (co >> 3) * kA1Plane + (Y & 1) * kA1Even + ((Y >> 1) * kT + p) * kA1Slot + pcol<18>(X) * 16 + (co & 7) * 2;
}

// tcgen05 shared-memory matrix descriptor, no swizzle: start, LBO (next core matrix along
// K), SBO (next 8 rows along M or N), descriptor version 1
__device__ __forceinline__ uint64_t umma_desc(uint32_t addr, uint32_t lbo, uint32_t sbo)
{
  return (uint64_t)((addr & 0x3FFFFu) >> 4) | ((uint64_t)((lbo & 0x3FFFFu) >> 4) << 16) |
         ((uint64_t)((sbo & 0x3FFFFu) >> 4) << 32) | (1ull << 46);
}
// kind::f16 instruction descriptor: D f32, A and B bf16, both K-major, N = 32, M = 128
constexpr uint32_t kConv2Idesc = (1u << 4) | (1u << 7) | (1u << 10) | ((32u >> 3) << 17) | ((128u >> 4) << 24);

__device__ __forceinline__ void umma_bf16(uint32_t tmem_d, uint64_t a, uint64_t b, uint32_t idesc, bool accumulate)
{
  asm volatile(
      "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
      " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(tmem_d),
      "l"(a), "l"(b), "r"(idesc), "r"((uint32_t)accumulate));
}
// the mbarrier arrives when every tcgen05.mma this thread issued has completed
__device__ __forceinline__ void umma_commit(uint32_t bar)
{
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(bar) : "memory");
}
__device__ __forceinline__ void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }
// 32 TMEM lanes (the warp's quarter) x 16 columns of 32 bits
__device__ __forceinline__ void tmem_ld16(uint32_t taddr, uint32_t (&r)[16])
{
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, %15}, "
      "[%16];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]), "=r"(r[8]),
        "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
      : "r"(taddr));
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
}
// true on every thread of the warp group when v holds on all of them
__device__ __forceinline__ bool group_all(int grp, bool v)
{
  uint32_t r;
  asm volatile(
      "{\n .reg .pred p, q;\n setp.ne.u32 p, %1, 0;\n bar.red.and.pred q, %2, %3, p;\n selp.u32 %0, 1, 0, q;\n}\n"
      : "=r"(r)
      : "r"((uint32_t)v), "r"(1 + grp), "r"(kGThreads)
      : "memory");
  return r != 0;
}
constexpr int kProposalTmemCols = 32 * kGroups;   // one 128 x 32 f32 accumulator per warp group

// Input windows of the tile starting at POI p0 into x0p's interior: warp 2p + c of the group
// stages channel c (0 ref, 1 tar) of POI p.  Lane l holds column l of the 31x31 window in
// registers (coalesced row loads, one pass), the warp reduces mean and variance, and writes
// the normalised values.  POIs past n leave x0p as it was (their rows are never written out).
__device__ __forceinline__ void stage_windows(__nv_bfloat16* x0p, const float* __restrict__ ref,
                                              const float* __restrict__ tar, int w, int h,
                                              const dic_poi* __restrict__ pois, int64_t n, int64_t p0, int warp,
                                              int lane)
{
  if (warp >= 2 * kT) return;
  const int p = warp >> 1, ch = warp & 1;
  const int64_t i = p0 + p;
  if (i >= n) return;
  const float* img = ch ? tar : ref;
  const int cx = (int)pois[i].x, cy = (int)pois[i].y;
  constexpr int R = kWin / 2, NPIX = kWin * kWin;
  const int x = min(max(cx + lane - R, 0), w - 1);
  float v[kWin];
  float s = 0.f;
  if (lane < kWin)
  {
#pragma unroll
    for (int r = 0; r < kWin; ++r)
    {
      const int y = min(max(cy + r - R, 0), h - 1);
      v[r] = __ldg(img + (size_t)y * w + x);
    }
#pragma unroll
    for (int r = 0; r < kWin; ++r) s += v[r];
  }
  for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
  const float mean = s / NPIX;
  float q = 0.f;
  if (lane < kWin)
  {
#pragma unroll
    for (int r = 0; r < kWin; ++r) q += (v[r] - mean) * (v[r] - mean);
  }
  for (int o = 16; o > 0; o >>= 1) q += __shfl_xor_sync(0xffffffffu, q, o);
  const float inv = q > 0.f ? rsqrtf(q / NPIX) : 1.f;
  if (lane < kWin)
  {
    __nv_bfloat16* dst = x0p + ((p * 33 + 1) * kX0Row + lane + 1) * 2 + ch;
#pragma unroll
    for (int r = 0; r < kWin; ++r) dst[r * kX0Row * 2] = __float2bfloat16((v[r] - mean) * inv);
  }
}

// One 3x3 stride-2 conv layer from padded NHWC smem (pixel stride kPix) to the interior of
// the next padded buffer, K = 288 (ci = 32).  Tasks = (MPAIR m-tiles MT/MPAIR apart, pair
// of n-tiles): with MPAIR = 2 a warp loads each B fragment once for two m-tiles.
template <int SIP, int SO, int SOP, int MPAIR>
__device__ __forceinline__ void fused_conv32(const __nv_bfloat16* in, __nv_bfloat16* out, const __nv_bfloat16* W,
                                             const float* __restrict__ bias, int warp, int lane)   // warp: within the group
{
  constexpr int M = kT * SO * SO;
  constexpr int MT = (M + 15) / 16;
  static_assert(MT % MPAIR == 0, "m-tiles split evenly");
  constexpr int MSTEP = MT / MPAIR;
  const int g = lane >> 2, t4 = lane & 3;
  const int q = lane >> 3;
  for (int task = warp; task < MSTEP * 2; task += kGW)
  {
    const int mt0 = task >> 1, nh = task & 1;
    // ldmatrix A addresses: lane -> row (q & 1) * 8 + (lane & 7), k offset (q >> 1) * 8;
    // input pixel (2 oy + ky, 2 ox + kx): storage column ox + (kx >> 1) + (kx & 1) * SIP / 2
    const __nv_bfloat16* abase[MPAIR];
#pragma unroll
    for (int m = 0; m < MPAIR; ++m)
    {
      const int arow = (mt0 + m * MSTEP) * 16 + (q & 1) * 8 + (lane & 7);
      const int rr = arow < M ? arow : M - 1;
      const int p = rr / (SO * SO), oy = (rr % (SO * SO)) / SO, ox = rr % SO;
      abase[m] = in + ((p * SIP + 2 * oy) * SIP + ox) * kPix + (q >> 1) * 8;
    }
    // ldmatrix B addresses: lane -> n row (q >> 1) * 8 + (lane & 7), k offset (q & 1) * 8
    const __nv_bfloat16* bbase = W + (nh * 16 + (q >> 1) * 8 + (lane & 7)) * kWRow + (q & 1) * 8;
    float acc[MPAIR][2][4];
#pragma unroll
    for (int m = 0; m < MPAIR; ++m)
#pragma unroll
      for (int j = 0; j < 2; ++j)
#pragma unroll
        for (int e = 0; e < 4; ++e) acc[m][j][e] = 0.f;
#pragma unroll
    for (int kk = 0; kk < 9; ++kk)
    {
      const int ky = kk / 3, kx = kk % 3;
      const int aoff = (ky * SIP + (kx >> 1) + (kx & 1) * (SIP / 2)) * kPix;
#pragma unroll
      for (int half = 0; half < 2; ++half)
      {
        uint32_t b[4];
        ldsm_x4(b, smem_u32(bbase + kk * 32 + half * 16));
        const uint32_t b0[2] = {b[0], b[1]}, b1[2] = {b[2], b[3]};
#pragma unroll
        for (int m = 0; m < MPAIR; ++m)
        {
          uint32_t a[4];
          ldsm_x4(a, smem_u32(abase[m] + aoff + half * 16));
          mma_bf16_16816(acc[m][0], a, b0);
          mma_bf16_16816(acc[m][1], a, b1);
        }
      }
    }
#pragma unroll
    for (int m = 0; m < MPAIR; ++m)
#pragma unroll
      for (int j = 0; j < 2; ++j)
      {
        const int co = nh * 16 + j * 8 + t4 * 2;
        const float bb0 = bias[co], bb1 = bias[co + 1];
#pragma unroll
        for (int h2 = 0; h2 < 2; ++h2)
        {
          const int row = (mt0 + m * MSTEP) * 16 + g + h2 * 8;
          if (row >= M) continue;
          const int pp = row / (SO * SO), y = (row % (SO * SO)) / SO, x = row % SO;
          __nv_bfloat16* dst = out + ((pp * SOP + y + 1) * SOP + pcol<SOP>(x + 1)) * kPix + co;
          *reinterpret_cast<uint32_t*>(dst) = pack_bf16(__float2bfloat16(fmaxf(acc[m][j][h2 * 2] + bb0, 0.f)),
                                                        __float2bfloat16(fmaxf(acc[m][j][h2 * 2 + 1] + bb1, 0.f)));
        }
      }
  }
}

__global__ void __launch_bounds__(kFusedThreads, 1)
    k_proposal_fused(const float* __restrict__ ref, const float* __restrict__ tar, int w, int h,
                     dic_poi* __restrict__ pois, int64_t n, const __nv_bfloat16* __restrict__ wb,
                     const float* __restrict__ params, int* __restrict__ err, uint32_t wait_polls = kWaitPolls,
                     int wait_test = 0)   // wait_test: never issue conv2's products (timeout-path test)
{
  extern __shared__ __align__(16) unsigned char sm[];
  __shared__ __align__(8) unsigned long long mma_bar[kGroups];
  __shared__ uint32_t tmem_base;
  __nv_bfloat16* W1s = reinterpret_cast<__nv_bfloat16*>(sm);
  __nv_bfloat16* W2s = reinterpret_cast<__nv_bfloat16*>(sm + kSmW1);
  __nv_bfloat16* W3s = W2s + 32 * kWRow;
  __nv_bfloat16* W4s = W3s + 32 * kWRow;
  using L = WeightLayout;
  using P = ParamLayout;
  const int tid = threadIdx.x, lane = tid & 31, g = lane >> 2, t4 = lane & 3;
  const int grp = tid / kGThreads, gt = tid % kGThreads, warp = gt >> 5;   // warp within the group
  unsigned char* gs = sm + kSmW1 + kSmW + grp * kSmGroup;
  __nv_bfloat16* x0p = reinterpret_cast<__nv_bfloat16*>(gs);
  unsigned char* a1c = gs + kSmX0;
  __nv_bfloat16* a1p = reinterpret_cast<__nv_bfloat16*>(a1c);   // its start, for the overlays
  __nv_bfloat16* a2p = reinterpret_cast<__nv_bfloat16*>(gs + kSmX0 + kSmA1);
  __nv_bfloat16* a3p = reinterpret_cast<__nv_bfloat16*>(gs + kSmX0 + kSmA1 + kSmA2);          // [2][6][6][kPix]
  __nv_bfloat16* a4 = reinterpret_cast<__nv_bfloat16*>(gs + kSmX0 + kSmA1 + kSmA2 + kSmA3);   // [16][136]
  float* outs = reinterpret_cast<float*>(gs + kSmX0 + kSmA1 + kSmA2 + kSmA3 + kSmA4);         // [16][8]
  int64_t* tile_p0 = reinterpret_cast<int64_t*>(gs + kSmX0 + kSmA1 + kSmA2 + kSmA3 + kSmA4 + kSmOut);
  float* part4 = reinterpret_cast<float*>(a1p);                                              // [4][16][32]
  float* part2 = reinterpret_cast<float*>(reinterpret_cast<unsigned char*>(a1p) + kSmPart4); // [8][16][8]
  __nv_bfloat16* a5 = reinterpret_cast<__nv_bfloat16*>(reinterpret_cast<unsigned char*>(a1p) + kSmA5Off);   // [16][264]
  // weights and zero borders, once per CTA (both groups)
  for (int i = tid; i < 32 * kW1Row; i += kFusedThreads)
  {
    const int r = i / kW1Row, c = i % kW1Row;
    const int tap = c < 32 ? conv1_slot_tap(c >> 1) : -1;
    W1s[i] = tap >= 0 ? wb[L::c1 + r * 32 + 2 * tap + (c & 1)] : bz();
  }
  // W2 as B core matrices for tcgen05: (k >> 3, co >> 3) at 512 B x 128 B, rows of 16 B
  for (int i = tid; i < 32 * 288; i += kFusedThreads)
  {
    const int co = i / 288, k = i % 288;
    W2s[(k >> 3) * 256 + (co >> 3) * 64 + (co & 7) * 8 + (k & 7)] = wb[L::c2 + i];
  }
  for (int i = tid; i < 2 * 32 * kWRow; i += kFusedThreads)
  {
    const int l = 1 + i / (32 * kWRow), r = (i / kWRow) % 32, c = i % kWRow;
    W3s[i] = c < 288 ? wb[L::c2 + l * 32 * 288 + r * 288 + c] : bz();
  }
  for (int i = tid; i < kGroups * kSmGroup / 4; i += kFusedThreads)
    reinterpret_cast<uint32_t*>(sm + kSmW1 + kSmW)[i] = 0u;
  if (tid == 0)
    for (int g2 = 0; g2 < kGroups; ++g2) mbar_init(smem_addr(&mma_bar[g2]), 1);
  if (tid < 32)
  {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_addr(&tmem_base)),
                 "n"(kProposalTmemCols)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  fence_proxy_async_smem();   // W2 (generic writes) before the tensor core reads it
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem_d = tmem_base + 32u * (uint32_t)grp;   // lanes 0..127, this group's 32 columns
  const uint32_t bar = smem_addr(&mma_bar[grp]);
  uint32_t mma_phase = 0;
  // From here on the two groups run independently: group grp takes tiles 2 b + grp, stepping
  // by 2 * gridDim.x, and meets only its own barrier.
  const int64_t tiles = (n + kT - 1) / kT;
  const int64_t tstep = (int64_t)gridDim.x * kGroups;
  int nsub = 0;   // tiles whose conv4 output waits in a4 (uniform over the group)
  // Borders of x0p, a1c, a2p and a3p stay zero: their interiors are all that is written,
  // except for the overlays at the start of a1c, which each tile clears.  A tile's windows
  // are staged while the previous tile's conv2 products run (the first tile's here).
  if ((int64_t)blockIdx.x * kGroups + grp < tiles)
    stage_windows(x0p, ref, tar, w, h, pois, n, ((int64_t)blockIdx.x * kGroups + grp) * kT, warp, lane);
  for (int64_t tile = (int64_t)blockIdx.x * kGroups + grp; tile < tiles; tile += tstep)
  {
    const int64_t p0 = tile * kT;
    // the split-K partials and a5 of the previous tile overlay the start of a1c: clear them
    // so a1c's borders read as padding again
    for (int i = gt; i < kSmScratch / 4; i += kGThreads) reinterpret_cast<uint32_t*>(a1p)[i] = 0u;
    group_sync(grp);
    // ---- conv1: M = kT * 256 rows, K = 18 (padded 32), A gathered as (ci0, ci1) pairs
    {
      constexpr int M = kT * 256;
      for (int mt = warp; mt < M / 16; mt += kGW)
      {
        int rbase[2];
#pragma unroll
        for (int h2 = 0; h2 < 2; ++h2)
        {
          const int row = mt * 16 + g + h2 * 8;
          const int p = row >> 8, oy = (row >> 4) & 15, ox = row & 15;
          rbase[h2] = ((p * 33 + 2 * oy) * kX0Row + 2 * ox) * 2;
        }
        float acc[4][4];
#pragma unroll
        for (int j = 0; j < 4; ++j)
#pragma unroll
          for (int e = 0; e < 4; ++e) acc[j][e] = 0.f;
#pragma unroll
        for (int ks = 0; ks < 2; ++ks)
        {
          uint32_t a[4];
#pragma unroll
          for (int r = 0; r < 4; ++r)
          {
            const int tap = conv1_slot_tap(ks * 8 + (r >> 1) * 4 + t4);   // k = ks*16 + (r>>1)*8 + 2 t4
            const int h2 = r & 1;
            a[r] = tap >= 0 ? *reinterpret_cast<const uint32_t*>(x0p + rbase[h2] + ((tap / 3) * kX0Row + tap % 3) * 2)
                            : 0u;
          }
#pragma unroll
          for (int j = 0; j < 4; ++j)
          {
            const __nv_bfloat16* wr = W1s + (j * 8 + g) * kW1Row + ks * 16 + t4 * 2;
            const uint32_t b[2] = {*reinterpret_cast<const uint32_t*>(wr), *reinterpret_cast<const uint32_t*>(wr + 8)};
            mma_bf16_16816(acc[j], a, b);
          }
        }
#pragma unroll
        for (int j = 0; j < 4; ++j)
        {
          const int co = j * 8 + t4 * 2;
          const float bb0 = params[P::b1 + co], bb1 = params[P::b1 + co + 1];
#pragma unroll
          for (int h2 = 0; h2 < 2; ++h2)
          {
            const int row = mt * 16 + g + h2 * 8;
            const int p = row >> 8, y = (row >> 4) & 15, x = row & 15;
            *reinterpret_cast<uint32_t*>(a1c + a1c_offset(p, y + 1, x + 1, co)) =
                pack_bf16(__float2bfloat16(fmaxf(acc[j][h2 * 2] + bb0, 0.f)),
                          __float2bfloat16(fmaxf(acc[j][h2 * 2 + 1] + bb1, 0.f)));
          }
        }
      }
    }
    fence_proxy_async_smem();   // this thread's a1c writes before the tensor core reads them
    group_sync(grp);
    // ---- conv2 on tcgen05: step s = (tap, channel half) reads a1c through one descriptor
    if (gt == 0 && !wait_test)
    {
      tc_fence_after();
      const uint32_t a0 = smem_addr(a1c), b0 = smem_addr(W2s);
#pragma unroll
      for (int st = 0; st < 18; ++st)
      {
        const int tap = st >> 1, half = st & 1, ky = tap / 3, kx = tap % 3;
        const uint32_t aoff = 2 * half * kA1Plane + (ky & 1) * kA1Even + (ky >> 1) * kT * kA1Slot +
                              ((kx & 1) * 9 + (kx >> 1)) * 16;
        umma_bf16(tmem_d, umma_desc(a0 + aoff, kA1Plane, kA1Slot), umma_desc(b0 + 2 * st * 512, 512, 128), kConv2Idesc,
                  st > 0);
      }
      umma_commit(bar);
    }
    // conv1 has consumed x0p: stage the next tile's windows while the products run
    if (tile + tstep < tiles) stage_windows(x0p, ref, tar, w, h, pois, n, (tile + tstep) * kT, warp, lane);
    if (!group_all(grp, mbar_wait_bounded(bar, mma_phase, wait_polls)))
    {
      // the products did not complete in time: flag it, give them one more bounded wait
      // (TMEM and a1c stay in use until they finish) and leave the tile loop
      if (gt == 0) atomicOr(err, 2);
      mbar_wait_bounded(bar, mma_phase, wait_polls);
      break;
    }
    mma_phase ^= 1u;
    tc_fence_after();
    {
      // warp w reads TMEM lanes 32 (w & 3) .. + 31 (rows m), columns 16 (w >> 2) .. + 15
      const int quarter = warp & 3, chalf = warp >> 2;
      uint32_t r[16];
      tmem_ld16(tmem_d + ((uint32_t)(32 * quarter) << 16) + 16u * (uint32_t)chalf, r);
      const int m = 32 * quarter + lane, g2 = m >> 3, ox = m & 7, oy = g2 >> 1, p = g2 & 1;
      const int co0 = 16 * chalf;
      uint32_t packed[8];
#pragma unroll
      for (int k = 0; k < 8; ++k)
        packed[k] = pack_bf16(__float2bfloat16(fmaxf(__uint_as_float(r[2 * k]) + params[P::b2 + co0 + 2 * k], 0.f)),
                              __float2bfloat16(fmaxf(__uint_as_float(r[2 * k + 1]) + params[P::b2 + co0 + 2 * k + 1], 0.f)));
      uint4* dst = reinterpret_cast<uint4*>(a2p + ((p * 10 + oy + 1) * 10 + pcol<10>(ox + 1)) * kPix + co0);
      dst[0] = make_uint4(packed[0], packed[1], packed[2], packed[3]);
      dst[1] = make_uint4(packed[4], packed[5], packed[6], packed[7]);
    }
    tc_fence_before();
    group_sync(grp);
    fused_conv32<10, 4, 6, 1>(a2p, a3p, W3s, params + P::b3, warp, lane);
    group_sync(grp);
    // ---- conv4: 4x4 -> 2x2, M = kT*4 = 8 rows (half an m-tile), N = 32, K = 288, split over
    // the group's 8 warps: warp = (n-tile pair, one of 4 K slices of the 18 k16 steps).
    // Partial sums go to a1p (free after conv2) and are added in slice order
    // (deterministic), then bias + ReLU into this tile's rows of a4 [p][y][x][c].
    {
      constexpr int SIP = 6, M = kT * 4;
      const int nh = warp & 1, slice = warp >> 1, q = lane >> 3;
      const int s0 = slice * 18 / 4, s1 = (slice + 1) * 18 / 4;
      const int arow = min((q & 1) * 8 + (lane & 7), M - 1);
      const int p = arow / 4, oy = (arow % 4) / 2, ox = arow % 2;
      const __nv_bfloat16* abase = a3p + ((p * SIP + 2 * oy) * SIP + ox) * kPix + (q >> 1) * 8;
      const __nv_bfloat16* bbase = W4s + (nh * 16 + (q >> 1) * 8 + (lane & 7)) * kWRow + (q & 1) * 8;
      float acc[2][4] = {{0.f, 0.f, 0.f, 0.f}, {0.f, 0.f, 0.f, 0.f}};
      for (int st = s0; st < s1; ++st)
      {
        const int kk = st >> 1, half = st & 1;
        uint32_t a[4], b[4];
        ldsm_x4(a, smem_u32(abase + ((kk / 3) * SIP + ((kk % 3) >> 1) + ((kk % 3) & 1) * (SIP / 2)) * kPix +
                                half * 16));
        ldsm_x4(b, smem_u32(bbase + kk * 32 + half * 16));
        const uint32_t b0[2] = {b[0], b[1]}, b1[2] = {b[2], b[3]};
        mma_bf16_16816(acc[0], a, b0);
        mma_bf16_16816(acc[1], a, b1);
      }
#pragma unroll
      for (int j = 0; j < 2; ++j)
      {
        const int co = nh * 16 + j * 8 + t4 * 2;
        float* dst = part4 + (slice * 16 + g) * 32 + co;   // rows g < 8 = the M rows
        dst[0] = acc[j][0];
        dst[1] = acc[j][1];
      }
      group_sync(grp);
      {
        const int row = gt >> 5, col = gt & 31;    // 256 threads = 8 rows x 32 channels
        float sum = 0.f;
#pragma unroll
        for (int sl = 0; sl < 4; ++sl) sum += part4[(sl * 16 + row) * 32 + col];
        a4[(nsub * kT + (row >> 2)) * kA4Row + (row & 3) * 32 + col] =
            __float2bfloat16(fmaxf(sum + params[P::b4 + col], 0.f));
        if (gt == 0) tile_p0[nsub] = p0;
      }
    }
    ++nsub;
    if (nsub < kMlpTiles && tile + tstep < tiles)
    {
      group_sync(grp);
      continue;   // the MLP waits for a full m-tile of POIs
    }
    group_sync(grp);
    // ---- f1: [16 x 128] x W5^T -> [16 x 256] for the batched tiles (rows past nsub * kT
    // hold stale values and are never written out); B fragments from global (L2).  A warp
    // takes n-tiles warp + 8 h, h < 4, and loads each A fragment once for the four.
    {
      constexpr int NT = kHidden / 8 / kGW;   // 4
      static_assert(kHidden / 8 == NT * kGW, "f1 n-tiles split evenly over the group");
      float acc[NT][4];
#pragma unroll
      for (int hh = 0; hh < NT; ++hh)
#pragma unroll
        for (int e = 0; e < 4; ++e) acc[hh][e] = 0.f;
#pragma unroll
      for (int ks = 0; ks < 8; ++ks)
      {
        const int c = ks * 16 + t4 * 2;
        uint32_t a[4];
        a[0] = *reinterpret_cast<const uint32_t*>(a4 + g * kA4Row + c);
        a[1] = *reinterpret_cast<const uint32_t*>(a4 + (g + 8) * kA4Row + c);
        a[2] = *reinterpret_cast<const uint32_t*>(a4 + g * kA4Row + c + 8);
        a[3] = *reinterpret_cast<const uint32_t*>(a4 + (g + 8) * kA4Row + c + 8);
#pragma unroll
        for (int hh = 0; hh < NT; ++hh)
        {
          const int nt = warp + hh * kGW;
          const __nv_bfloat16* wr = wb + L::f1 + (nt * 8 + g) * 128 + c;
          const uint32_t b[2] = {__ldg(reinterpret_cast<const unsigned int*>(wr)),
                                 __ldg(reinterpret_cast<const unsigned int*>(wr + 8))};
          mma_bf16_16816(acc[hh], a, b);
        }
      }
#pragma unroll
      for (int hh = 0; hh < NT; ++hh)
      {
        const int co = (warp + hh * kGW) * 8 + t4 * 2;
        const float bb0 = params[P::b5 + co], bb1 = params[P::b5 + co + 1];
#pragma unroll
        for (int h2 = 0; h2 < 2; ++h2)
          *reinterpret_cast<uint32_t*>(a5 + (g + h2 * 8) * kA5Row + co) =
              pack_bf16(__float2bfloat16(fmaxf(acc[hh][h2 * 2] + bb0, 0.f)),
                        __float2bfloat16(fmaxf(acc[hh][h2 * 2 + 1] + bb1, 0.f)));
      }
    }
    group_sync(grp);
    // ---- f2: [16 x 256] x W6^T -> [16 x 6] (n padded to 8): warp w takes k16 steps 2w and
    // 2w + 1, partials [8][16][8] summed in warp order
    {
      float acc[4] = {0.f, 0.f, 0.f, 0.f};
#pragma unroll
      for (int kk = 0; kk < 2; ++kk)
      {
        const int c = (warp * 2 + kk) * 16 + t4 * 2;
        uint32_t a[4];
        a[0] = *reinterpret_cast<const uint32_t*>(a5 + g * kA5Row + c);
        a[1] = *reinterpret_cast<const uint32_t*>(a5 + (g + 8) * kA5Row + c);
        a[2] = *reinterpret_cast<const uint32_t*>(a5 + g * kA5Row + c + 8);
        a[3] = *reinterpret_cast<const uint32_t*>(a5 + (g + 8) * kA5Row + c + 8);
        const __nv_bfloat16* wr = wb + L::f2 + g * 256 + c;
        const uint32_t b[2] = {__ldg(reinterpret_cast<const unsigned int*>(wr)),
                               __ldg(reinterpret_cast<const unsigned int*>(wr + 8))};
        mma_bf16_16816(acc, a, b);
      }
#pragma unroll
      for (int h2 = 0; h2 < 2; ++h2)
      {
        part2[(warp * kMlpRows + g + h2 * 8) * 8 + t4 * 2] = acc[h2 * 2];
        part2[(warp * kMlpRows + g + h2 * 8) * 8 + t4 * 2 + 1] = acc[h2 * 2 + 1];
      }
      group_sync(grp);
      if (gt < kMlpRows * 8)
      {
        const int row = gt >> 3, co = gt & 7;
        float sum = 0.f;
#pragma unroll
        for (int k = 0; k < kGW; ++k) sum += part2[(k * kMlpRows + row) * 8 + co];
        outs[row * 8 + co] = sum + (co < kOut ? params[P::b6 + co] : 0.f);
      }
    }
    group_sync(grp);
    if (gt < nsub * kT && tile_p0[gt / kT] + gt % kT < n)
    {
      const float* o = outs + gt * 8;
      dic_poi* dst = pois + tile_p0[gt / kT] + gt % kT;
      dst->u = o[0];
      dst->v = o[1];
      dst->ux = o[2] / out_scale(2);
      dst->uy = o[3] / out_scale(3);
      dst->vx = o[4] / out_scale(4);
      dst->vy = o[5] / out_scale(5);
      dst->u0 = 0.f; dst->v0 = 0.f; dst->zncc = 0.f; dst->iteration = 0.f; dst->convergence = 0.f; dst->feature = 0.f;
    }
    nsub = 0;
    group_sync(grp);
  }
  tc_fence_before();
  __syncthreads();
  if (tid < 32)
  {
    tc_fence_after();
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem_base), "n"(kProposalTmemCols)
                 : "memory");
  }
}

}  // namespace cnn
}  // namespace dic
