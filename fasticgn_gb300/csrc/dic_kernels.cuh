// GB300 (sm_103a) kernels of the FFTCC -> first-order IC-GN path.
//
// Data layout in HBM (one engine):
//   raw_ref, raw_tar   W*H input pixels as uploaded (u8 / u16 / f32)
//   ref_f32, tar_f32   W*H float grey levels (FFTCC subsets read these)
//   ref_pack           W*H float4 {ref, gx, gy, 0}: one 16-byte load per IC-GN sample
//   tar_coef           BicubicBspline table: 2 planes of W*H texels x 32 B (coefficient rows
//                      0-1, rows 2-3): one 256-bit load per plane and IC-GN sample
//   poi_ref            per prepared POI: PoiRef (224 B), resident across frames
//   queue              dic_poi records (56 B)
#pragma once

#include <climits>
#include <cstdint>
#include <cuda.h>            // CUtensorMap (the type only; maps are encoded through the runtime's driver entry point)
#include <cuda_runtime.h>

#include "../../include/dic.h"

namespace dic
{

constexpr int kWarp = 32;
constexpr unsigned kFull = 0xffffffffu;
// Widest subset (columns) of the pair walk: two column classes of at most 32 each.
#ifndef DIC_PAIR_MAX_WIDTH
#define DIC_PAIR_MAX_WIDTH 64
#endif
constexpr int kPairMaxWidth = DIC_PAIR_MAX_WIDTH;
// Column of lane l in class k of the pair walk: halves (32 k + l; the default) or interleaved
// (2 l + k).  Halves keep a warp's texel loads on consecutive columns, one contiguous run per
// coefficient plane; interleaved classes balance the two classes' lanes but stride the loads
// by two texels.  Measured on the uneven batch's r 20 / 30 jobs: halves 16.7 ms, interleaved
// 19.1 ms, the flat walk 17.7 ms; those pairs one at a time 48.6 / 57.9 / 47.5 ms.
#ifndef DIC_PAIR_HALVES
#define DIC_PAIR_HALVES 1
#endif
__host__ __device__ constexpr int pair_column(int lane, int k) { return DIC_PAIR_HALVES ? 32 * k + lane : 2 * lane + k; }

// --------------------------------------------------------------------------------------
// Per-POI reference record, built once per (reference, layout) by k_poi_prepare.
// The IC-GN kernel evaluates the ZNSSD terms in a single pass over the warped samples:
// with tau = t - t0 (t0 = reference subset mean), rc = reference zero-mean value and
// sd = [gx, gx*lx, gx*ly, gy, gy*lx, gy*ly] it accumulates
//   A0 = sum tau, A1 = sum tau^2, A2 = sum tau*rc, B_i = sum sd_i * tau
// and recovers the two-pass quantities of src/oc_icgn.cpp:303-322 exactly in algebra:
//   |t_c|^2 = A1 - A0*m_t, sum t_c rc = A2 - m_t*sum(rc)      (m_t = A0/N),
//   num_i   = s*(B_i - m_t*S_i) - G_i      with s = |rc| / |t_c|,
//   S_i = sum sd_i, G_i = sum sd_i*rc  (per-POI constants kept here).
// The reference-side constants are formed with the same expressions and the same
// accumulation order as the target-side sums (rn_sq = sum rc^2 - sum(rc)*m_r with
// m_r = sum(rc)/N, G_i likewise centred), so a target subset equal to the reference subset
// reproduces s = 1, ZNSSD = 0 and num = 0 bit for bit, as the CPU's two-pass form does.
// --------------------------------------------------------------------------------------
struct __align__(16) PoiRef
{
  float t0;          // reference subset mean
  float ref_norm;    // sqrt(rn_sq)
  float ref_norm_sq; // rn_sq = sum rc^2 - sum(rc) * m_r
  float sum_rc;      // sum rc (0 up to rounding)
  float S[6];
  float G[6];        // sum sd_i*rc - m_r * S_i
  float inv_h[36];   // row-major inverse Hessian
  float valid;       // 1 when the reference subset lies inside the image
  float pad[3];
};
static_assert(sizeof(PoiRef) == 224, "PoiRef layout");

// BicubicBspline BC matrix (src/oc_cubic_bspline.h:52-58)
#define DIC_BC_MATRIX                                                              \
  {{-144.0f / 336.0f, 384.0f / 336.0f, -384.0f / 336.0f, 144.0f / 336.0f},        \
   {342.0f / 336.0f, -702.0f / 336.0f, 450.0f / 336.0f, -90.0f / 336.0f},         \
   {-198.0f / 336.0f, -18.0f / 336.0f, 270.0f / 336.0f, -54.0f / 336.0f},         \
   {0.0f, 1.0f, 0.0f, 0.0f}}

// Products BC[l][m] * BC[k][n] rounded to float, indexed [k][l][m][n]; filled by the host.
// (This header is compiled in exactly one translation unit, dic_engine.cu.)
__constant__ float c_bc2[256];
// FFT twiddles: W_N^k = exp(-2 pi i k / N) for N in [2, kMaxTwiddleN], at tw_offset(N).
constexpr int kMaxTwiddleN = 64;
__host__ __device__ constexpr int tw_offset(int n) { return n * (n - 1) / 2 - 1; }
constexpr int kTwiddleCount = tw_offset(kMaxTwiddleN + 1);
__constant__ float2 c_tw[kTwiddleCount];

template <typename T>
__device__ __forceinline__ float load_px(const T* p, size_t i, float scale);
template <>
__device__ __forceinline__ float load_px<uint8_t>(const uint8_t* p, size_t i, float scale)
{ return scale == 1.0f ? (float)p[i] : (float)p[i] * scale; }
template <>
__device__ __forceinline__ float load_px<uint16_t>(const uint16_t* p, size_t i, float scale)
{ return scale == 1.0f ? (float)p[i] : (float)p[i] * scale; }
template <>
__device__ __forceinline__ float load_px<float>(const float* p, size_t i, float scale)
{ return scale == 1.0f ? p[i] : p[i] * scale; }

// --------------------------------------------------------------------------------------
// Reference prep: raw -> float plane, Gradient2D4 (src/oc_gradient.cpp:37-79), packed
// {ref, gx, gy, 0}.  16x16 output tile per 256-thread block, 2-px halo staged in smem.
// Stencil term order follows the CPU: -f(c+2)/12 + 2f(c+1)/3 - 2f(c-1)/3 + f(c-2)/12,
// each product rounded separately (no contraction), so planes are bit-identical.
// --------------------------------------------------------------------------------------
constexpr int kPrepTile = 16;

template <typename T>
__global__ void __launch_bounds__(256) k_prepare_ref(const T* __restrict__ raw, int w, int h, float scale,
                                                     float* __restrict__ ref_f32,
                                                     float4* __restrict__ ref_pack)
{
  __shared__ float tile[kPrepTile + 4][kPrepTile + 4 + 1];
  const int bx = blockIdx.x * kPrepTile, by = blockIdx.y * kPrepTile;
  for (int i = threadIdx.x; i < (kPrepTile + 4) * (kPrepTile + 4); i += blockDim.x)
  {
    int ty = i / (kPrepTile + 4), tx = i % (kPrepTile + 4);
    int gx = bx + tx - 2, gy = by + ty - 2;
    float v = 0.f;
    if (gx >= 0 && gx < w && gy >= 0 && gy < h) v = load_px<T>(raw, (size_t)gy * w + gx, scale);
    tile[ty][tx] = v;
  }
  __syncthreads();
  const int tx = threadIdx.x % kPrepTile, ty = threadIdx.x / kPrepTile;
  const int x = bx + tx, y = by + ty;
  if (x >= w || y >= h) return;
  const float c = tile[ty + 2][tx + 2];
  const float f1 = 1.f / 12.f, f2 = 2.f / 3.f;
  float gxv = 0.f, gyv = 0.f;
  if (x >= 2 && x < w - 2)
  {
    float r = 0.f;
    r = __fsub_rn(r, __fmul_rn(tile[ty + 2][tx + 4], f1));
    r = __fadd_rn(r, __fmul_rn(tile[ty + 2][tx + 3], f2));
    r = __fsub_rn(r, __fmul_rn(tile[ty + 2][tx + 1], f2));
    r = __fadd_rn(r, __fmul_rn(tile[ty + 2][tx + 0], f1));
    gxv = r;
  }
  if (y >= 2 && y < h - 2)
  {
    float r = 0.f;
    r = __fsub_rn(r, __fmul_rn(tile[ty + 4][tx + 2], f1));
    r = __fadd_rn(r, __fmul_rn(tile[ty + 3][tx + 2], f2));
    r = __fsub_rn(r, __fmul_rn(tile[ty + 1][tx + 2], f2));
    r = __fadd_rn(r, __fmul_rn(tile[ty + 0][tx + 2], f1));
    gyv = r;
  }
  const size_t o = (size_t)y * w + x;
  ref_f32[o] = c;
  ref_pack[o] = make_float4(c, gxv, gyv, 0.f);
}

// --------------------------------------------------------------------------------------
// Target prep: raw -> float plane + BicubicBspline table (src/oc_cubic_bspline.cpp:84-132).
// Texel (r, c) for 1 <= c < w-2, 1 <= r < h-2 holds coef[k][l] = P[3-k][3-l] with
// P[k][l] = sum_m sum_n BC[l][m] BC[k][n] q[n][m], accumulated in the CPU's m, n order with
// separate roundings, so the table is bit-identical to the CPU's; other texels are 0.
// Layout: two planes of W*H texels x 8 floats, plane j holding coefficient rows 2j and 2j+1
// of every texel, so a warp reading one plane for 32 neighbouring texels (one 256-bit load
// per lane) touches one contiguous 1 KB run.  Against four 16 B row planes this is two
// loads per sample instead of four and fewer partly-used cache lines per warp: 3 % less
// IC-GN time on GB300, same values (the texel-major 64 B layout spreads a warp load over
// 16 cache lines).
// --------------------------------------------------------------------------------------
// tar_px (nullable): the float plane again with rows of `pitch` floats (a multiple of 4), for
// the pixel-sampled IC-GN's TMA windows when W itself is not a multiple of 4.
template <typename T>
__global__ void __launch_bounds__(256) k_prepare_tar(const T* __restrict__ raw, int w, int h, float scale,
                                                     float* __restrict__ tar_f32,
                                                     float4* __restrict__ coef, float* __restrict__ lattice = nullptr,
                                                     float* __restrict__ tar_px = nullptr, int pitch = 0)
{
  __shared__ float tile[kPrepTile + 3][kPrepTile + 3 + 1];
  const int bx = blockIdx.x * kPrepTile, by = blockIdx.y * kPrepTile;
  for (int i = threadIdx.x; i < (kPrepTile + 3) * (kPrepTile + 3); i += blockDim.x)
  {
    int ty = i / (kPrepTile + 3), tx = i % (kPrepTile + 3);
    int gx = bx + tx - 1, gy = by + ty - 1;
    float v = 0.f;
    if (gx >= 0 && gx < w && gy >= 0 && gy < h) v = load_px<T>(raw, (size_t)gy * w + gx, scale);
    tile[ty][tx] = v;
  }
  __syncthreads();
  const int tx = threadIdx.x % kPrepTile, ty = threadIdx.x / kPrepTile;
  const int x = bx + tx, y = by + ty;
  if (x >= w || y >= h) return;
  const size_t o = (size_t)y * w + x;
  tar_f32[o] = tile[ty + 1][tx + 1];
  if (tar_px) tar_px[(size_t)y * pitch + x] = tile[ty + 1][tx + 1];
  if (!coef) return;   // pixel sampling: no table
  const size_t plane = (size_t)w * h;
  float4* dst = coef + 2 * o;   // row k at dst[(k >> 1) * 2 * plane + (k & 1)]
  if (x < 1 || y < 1 || x >= w - 2 || y >= h - 2)
  {
    const float4 z = make_float4(0.f, 0.f, 0.f, 0.f);
    dst[0] = z; dst[1] = z; dst[2 * plane] = z; dst[2 * plane + 1] = z;
    if (lattice) lattice[o] = 0.f;
    return;
  }
  float q[4][4];
#pragma unroll
  for (int i = 0; i < 4; ++i)
#pragma unroll
    for (int j = 0; j < 4; ++j) q[i][j] = tile[ty + i][tx + j];
  float p[4][4];
#pragma unroll
  for (int k = 0; k < 4; ++k)
#pragma unroll
    for (int l = 0; l < 4; ++l)
    {
      float acc = 0.f;
#pragma unroll
      for (int m = 0; m < 4; ++m)
#pragma unroll
        for (int n = 0; n < 4; ++n)
          acc = __fadd_rn(acc, __fmul_rn(c_bc2[((k * 4 + l) * 4 + m) * 4 + n], q[n][m]));
      p[k][l] = acc;
    }
#pragma unroll
  for (int k = 0; k < 4; ++k)
    dst[(k >> 1) * 2 * plane + (k & 1)] = make_float4(p[3 - k][3], p[3 - k][2], p[3 - k][1], p[3 - k][0]);
  // the interpolant at the texel's own integer position (dx = dy = 0): coefficient [0][0]
  if (lattice) lattice[o] = p[3][3];
}

// --------------------------------------------------------------------------------------
// Warp helpers
// --------------------------------------------------------------------------------------
__device__ __forceinline__ float warp_sum(float v)
{
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(kFull, v, o);
  return v;
}

// 6x6 inverse by partial-pivot LU in float (restates Eigen's Matrix6f::inverse, which
// src/oc_icgn.cpp:234 calls).  Fully unrolled with static indices, so the matrix lives in
// registers; row swaps are predicated.  lu6 factorises in place, solve6_column produces one
// column of the inverse; the column solves are independent, so k_poi_prepare runs them on
// six lanes at once.
__device__ __forceinline__ void lu6(float (&a)[6][6], int (&perm)[6])
{
#pragma unroll
  for (int i = 0; i < 6; ++i) perm[i] = i;
#pragma unroll
  for (int k = 0; k < 6; ++k)
  {
    int piv = k;
    float best = fabsf(a[k][k]);
#pragma unroll
    for (int i = k + 1; i < 6; ++i)
      if (fabsf(a[i][k]) > best) { best = fabsf(a[i][k]); piv = i; }
#pragma unroll
    for (int i = k + 1; i < 6; ++i)
    {
      const bool sw = (piv == i);
#pragma unroll
      for (int j = 0; j < 6; ++j)
      {
        const float ak = a[k][j], ai = a[i][j];
        a[k][j] = sw ? ai : ak;
        a[i][j] = sw ? ak : ai;
      }
      const int pk = perm[k], pi = perm[i];
      perm[k] = sw ? pi : pk;
      perm[i] = sw ? pk : pi;
    }
#pragma unroll
    for (int i = k + 1; i < 6; ++i)
    {
      a[i][k] = a[i][k] / a[k][k];
#pragma unroll
      for (int j = k + 1; j < 6; ++j) a[i][j] -= a[i][k] * a[k][j];
    }
  }
}

__device__ __forceinline__ void solve6_column(const float (&a)[6][6], const int (&perm)[6], int col, float (&x)[6])
{
  float y[6];
#pragma unroll
  for (int i = 0; i < 6; ++i)
  {
    float s = (perm[i] == col) ? 1.f : 0.f;
#pragma unroll
    for (int j = 0; j < i; ++j) s -= a[i][j] * y[j];
    y[i] = s;
  }
#pragma unroll
  for (int i = 5; i >= 0; --i)
  {
    float s = y[i];
#pragma unroll
    for (int j = i + 1; j < 6; ++j) s -= a[i][j] * x[j];
    x[i] = s / a[i][i];
  }
}

// --------------------------------------------------------------------------------------
// Subset walk shared by the per-POI prep and the IC-GN kernel, so both visit the samples
// of a subset in the same lane and the same per-lane order (the exact self-match property
// of PoiRef depends on it).  For subsets at most 32 columns wide lane l owns column
// lx = l - rx and walks the rows, so every warp-wide load reads one row of neighbouring
// texels; wider subsets use the flat order k = l + 32 j.
// --------------------------------------------------------------------------------------
#define DIC_FOR_EACH_SAMPLE(LANE, RX, RY, ...)                                   \
  {                                                                              \
    const int sw_ = 2 * (RX) + 1;                                                \
    if (sw_ <= 32)                                                               \
    {                                                                            \
      if ((LANE) < sw_)                                                          \
      {                                                                          \
        const int lx = (LANE) - (RX);                                            \
        for (int ly = -(RY); ly <= (RY); ++ly) { __VA_ARGS__ }                   \
      }                                                                          \
    }                                                                            \
    else                                                                         \
    {                                                                            \
      const int size_ = sw_ * (2 * (RY) + 1);                                    \
      int lx_ = (LANE) % sw_ - (RX), ly_ = (LANE) / sw_ - (RY);                  \
      for (int k_ = (LANE); k_ < size_; k_ += 32)                                \
      {                                                                          \
        {                                                                        \
          const int lx = lx_, ly = ly_;                                          \
          __VA_ARGS__                                                            \
        }                                                                        \
        lx_ += 32;                                                               \
        if (lx_ > (RX)) { lx_ -= sw_; ly_ += 1; }                                \
      }                                                                          \
    }                                                                            \
  }

// --------------------------------------------------------------------------------------
// Per-POI reference prep (src/oc_icgn.cpp:197-234): one warp per POI.  Reads the packed
// {ref, gx, gy} plane, forms mean, zero-mean norm, S, G, the float Hessian and its
// inverse, and stores a PoiRef.  POIs whose reference subset leaves the image get
// valid = 0 (the IC-GN entry test rejects them before any of this is read).
//
// Column walk (subset at most 32 wide): lane l owns column lx = l - rx, so every factor
// lx is constant within a lane and comes out of the row loop.  The lane accumulates
// row moments sum g*g'*ly^k (k = 0, 1, 2; g, g' in {gx, gy}) and forms its share of the
// 21 Hessian entries from them once; S and G likewise (S_1 = lx * sum gx, ...).  The
// target-side sums of k_icgn use the same forms, which keeps the exact self-match.
// --------------------------------------------------------------------------------------
// Sums of one POI's reference subset, butterfly-reduced so every lane holds them.
struct PoiSums
{
  float nsq, src, S[6], G[6], H[21];
};

// The sums of one subset column that do not depend on the subset's mean, over the rows
// ly = -ry..ry in order: the grey sum t, the gradient products' row moments
// q = {xx, yy, xy} x ly^{0,1,2} (Qxx0 Qxx1 Qxx2 Qyy0 ... Qxy2) and S's terms s = {gx, gx ly,
// gy, gy ly}.  Neighbouring POIs on one grid row share most of their columns, so
// k_poi_prepare32 forms each image column's sums once per CTA (kColSums floats, in shared
// memory) and every POI reads its columns from there; the per-POI path forms the same sums
// with the same function, so both give the same bits.
constexpr int kColSums = 14;
struct ColSums
{
  float t, q[9], s[4];
};
__device__ __forceinline__ void col_sums_add(ColSums& c, const float4 v, float fly)
{
  c.t += v.x;
  const float xx = __fmul_rn(v.y, v.y), yy = __fmul_rn(v.z, v.z), xy = __fmul_rn(v.y, v.z);
  const float xxl = __fmul_rn(xx, fly), yyl = __fmul_rn(yy, fly), xyl = __fmul_rn(xy, fly);
  c.q[0] = __fadd_rn(c.q[0], xx); c.q[1] = __fadd_rn(c.q[1], xxl); c.q[2] = __fmaf_rn(xxl, fly, c.q[2]);
  c.q[3] = __fadd_rn(c.q[3], yy); c.q[4] = __fadd_rn(c.q[4], yyl); c.q[5] = __fmaf_rn(yyl, fly, c.q[5]);
  c.q[6] = __fadd_rn(c.q[6], xy); c.q[7] = __fadd_rn(c.q[7], xyl); c.q[8] = __fmaf_rn(xyl, fly, c.q[8]);
  c.s[0] = __fadd_rn(c.s[0], v.y); c.s[1] = __fmaf_rn(v.y, fly, c.s[1]);
  c.s[2] = __fadd_rn(c.s[2], v.z); c.s[3] = __fmaf_rn(v.z, fly, c.s[3]);
}
// col: the column's texel in the subset's first row
__device__ __forceinline__ ColSums col_sums(const float4* __restrict__ col, int w, int ry)
{
  ColSums c;
  c.t = 0.f;
#pragma unroll
  for (int k = 0; k < 9; ++k) c.q[k] = 0.f;
#pragma unroll
  for (int k = 0; k < 4; ++k) c.s[k] = 0.f;
  for (int r = 0; r < 2 * ry + 1; ++r) col_sums_add(c, __ldg(col + (size_t)r * w), (float)(r - ry));
  return c;
}
// Column sums staged in shared memory, value-major: v[k * stride + j] is value k of column j.
struct ColSumsShared
{
  const float* v;   // column 0 of the calling POI's subset
  int stride;
};

// Entry test, mean (written to rec->t0), and the warp-reduced sums of one POI.  Returns false
// (after writing valid = 0) when the reference subset leaves the image.  `shared`: the POI's
// column sums as k_poi_prepare32 staged them (column and pair walks); otherwise col_sums forms
// them here, and a second pass over the subset forms the sums that depend on the mean.
// (Before the column sums were shared, the mean pass read ref_pack, whose lines the second
// pass then found in L1; reading the grey levels from the float plane instead, 4 B per
// sample, took 0.64 against 0.60 ms on the 2048x2048 pair.  Forming the means from
// precomputed horizontal window sums saved 0.01 ms and cost 0.03 ms to build them: dropped.)
__device__ __forceinline__ bool poi_sums(const float4* __restrict__ ref_pack, int w, int h, float px, float py,
                                         int rx, int ry, int lane, PoiRef* __restrict__ rec, PoiSums& out_sums,
                                         ColSumsShared shared = ColSumsShared{nullptr, 0})
{
  // Entry-test geometry of src/oc_icgn.cpp:184-185.
  if (!(py - ry >= 0 && px - rx >= 0 && py + ry <= h - 1 && px + rx <= w - 1))
  {
    if (lane == 0) rec->valid = 0.f;
    return false;
  }
  const int sw = 2 * rx + 1, size = sw * (2 * ry + 1);
  const int cx = (int)px, cy = (int)py;
  float sum = 0.f;
  float nsq = 0.f, src = 0.f, S[6] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f}, G[6] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
  float H[21];
#pragma unroll
  for (int t = 0; t < 21; ++t) H[t] = 0.f;
  if (sw <= 32)
  {
    const float4* col = ref_pack + (size_t)(cy - ry) * w + cx + (lane - rx);
    ColSums cs;
    cs.t = 0.f;
#pragma unroll
    for (int k = 0; k < 9; ++k) cs.q[k] = 0.f;
#pragma unroll
    for (int k = 0; k < 4; ++k) cs.s[k] = 0.f;
    if (lane < sw)
    {
      if (shared.v)
      {
        cs.t = shared.v[lane];
#pragma unroll
        for (int k = 0; k < 9; ++k) cs.q[k] = shared.v[(1 + k) * shared.stride + lane];
#pragma unroll
        for (int k = 0; k < 4; ++k) cs.s[k] = shared.v[(10 + k) * shared.stride + lane];
      }
      else
        cs = col_sums(col, w, ry);
    }
    sum = warp_sum(cs.t);
    const float t0 = sum / (float)size;
    const float Qxx[3] = {cs.q[0], cs.q[1], cs.q[2]}, Qyy[3] = {cs.q[3], cs.q[4], cs.q[5]},
                Qxy[3] = {cs.q[6], cs.q[7], cs.q[8]};
    S[0] = cs.s[0];
    S[2] = cs.s[1];
    S[3] = cs.s[2];
    S[5] = cs.s[3];
    if (lane < sw)
    {
      // the sums that depend on the mean, per sample in the IC-GN walk's order
      for (int r = 0; r < 2 * ry + 1; ++r)
      {
        const float fly = (float)(r - ry);
        const float4 v = __ldg(&col[(size_t)r * w]);
        const float rc = v.x - t0;
        nsq = fmaf(rc, rc, nsq);
        src += rc;
        const float grc = __fmul_rn(v.y, rc), hrc = __fmul_rn(v.z, rc);
        G[0] = __fadd_rn(G[0], grc);
        G[2] = fmaf(grc, fly, G[2]);
        G[3] = __fadd_rn(G[3], hrc);
        G[5] = fmaf(hrc, fly, G[5]);
      }
    }
    const float lx = (float)(lane - rx), lx2 = lx * lx;
    G[1] = lx * G[0];
    G[4] = lx * G[3];
    S[1] = lx * S[0];
    S[4] = lx * S[3];
    // sd = [gx, gx lx, gx ly, gy, gy lx, gy ly]; H lower triangle, row-major (a >= b).
    // Factor of sd_a sd_b by (f_a, f_b) with f in {1, lx, ly}:
    //   (1,1) Q0, (lx,1) lx Q0, (lx,lx) lx^2 Q0, (ly,1) Q1, (ly,lx) lx Q1, (ly,ly) Q2.
    H[0] = Qxx[0];                                   // (0,0)
    H[1] = lx * Qxx[0];  H[2] = lx2 * Qxx[0];        // (1,0) (1,1)
    H[3] = Qxx[1];  H[4] = lx * Qxx[1];  H[5] = Qxx[2];   // (2,0) (2,1) (2,2)
    H[6] = Qxy[0];  H[7] = lx * Qxy[0];  H[8] = Qxy[1];  H[9] = Qyy[0];                 // (3,*)
    H[10] = lx * Qxy[0];  H[11] = lx2 * Qxy[0];  H[12] = lx * Qxy[1];                   // (4,0..2)
    H[13] = lx * Qyy[0];  H[14] = lx2 * Qyy[0];                                          // (4,3) (4,4)
    H[15] = Qxy[1];  H[16] = lx * Qxy[1];  H[17] = Qxy[2];                               // (5,0..2)
    H[18] = Qyy[1];  H[19] = lx * Qyy[1];  H[20] = Qyy[2];                               // (5,3..5)
    if (lane >= sw)
    {
#pragma unroll
      for (int t = 0; t < 21; ++t) H[t] = 0.f;
#pragma unroll
      for (int a = 0; a < 6; ++a) { S[a] = 0.f; G[a] = 0.f; }
    }
    if (lane == 0) rec->t0 = t0;
  }
  else if (sw <= kPairMaxWidth)
  {
    // Pair walk (33 to 64 columns): column classes c = pair_column(lane, k), each walked like
    // the column walk and butterfly-reduced on its own, class totals added in class order --
    // the order in which the IC-GN pair walk forms its target-side sums.  The lane's two
    // column grey sums are added in class order before the reduction.
    const float4* base = ref_pack + (size_t)(cy - ry) * w + cx - rx;
    float tl = 0.f;
#pragma unroll
    for (int k = 0; k < 2; ++k)
    {
      const int c = pair_column(lane, k);
      if (c < sw)
      {
        float t = 0.f;
        if (shared.v)
          t = shared.v[c];
        else
          for (int r = 0; r < 2 * ry + 1; ++r) t += __ldg(&base[(size_t)r * w + c].x);
        tl += t;
      }
    }
    sum = warp_sum(tl);
    const float t0 = sum / (float)size;
#pragma unroll 1
    for (int k = 0; k < 2; ++k)
    {
      const int c = pair_column(lane, k);
      float pn = 0.f, ps = 0.f, pS[6] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f}, pG[6] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
      ColSums cs;
      cs.t = 0.f;
#pragma unroll
      for (int v = 0; v < 9; ++v) cs.q[v] = 0.f;
#pragma unroll
      for (int v = 0; v < 4; ++v) cs.s[v] = 0.f;
      if (c < sw)
      {
        const float4* col = base + c;
        const auto mean_sums = [&](const float4 v, float fly) {
          const float rc = v.x - t0;
          pn = fmaf(rc, rc, pn);
          ps += rc;
          const float grc = __fmul_rn(v.y, rc), hrc = __fmul_rn(v.z, rc);
          pG[0] = __fadd_rn(pG[0], grc);
          pG[2] = fmaf(grc, fly, pG[2]);
          pG[3] = __fadd_rn(pG[3], hrc);
          pG[5] = fmaf(hrc, fly, pG[5]);
        };
        if (shared.v)
        {
#pragma unroll
          for (int v = 0; v < 9; ++v) cs.q[v] = shared.v[(1 + v) * shared.stride + c];
#pragma unroll
          for (int v = 0; v < 4; ++v) cs.s[v] = shared.v[(10 + v) * shared.stride + c];
          for (int r = 0; r < 2 * ry + 1; ++r) mean_sums(__ldg(&col[(size_t)r * w]), (float)(r - ry));
        }
        else
          for (int r = 0; r < 2 * ry + 1; ++r)
          {
            const float fly = (float)(r - ry);
            const float4 v = __ldg(&col[(size_t)r * w]);
            mean_sums(v, fly);
            col_sums_add(cs, v, fly);
          }
      }
      pS[0] = cs.s[0];
      pS[2] = cs.s[1];
      pS[3] = cs.s[2];
      pS[5] = cs.s[3];
      const float Qxx[3] = {cs.q[0], cs.q[1], cs.q[2]}, Qyy[3] = {cs.q[3], cs.q[4], cs.q[5]},
                  Qxy[3] = {cs.q[6], cs.q[7], cs.q[8]};
      const float lx = (float)(c - rx), lx2 = lx * lx;
      pG[1] = lx * pG[0];
      pG[4] = lx * pG[3];
      pS[1] = lx * pS[0];
      pS[4] = lx * pS[3];
      float pH[21] = {Qxx[0], lx * Qxx[0], lx2 * Qxx[0], Qxx[1], lx * Qxx[1], Qxx[2],
                      Qxy[0], lx * Qxy[0], Qxy[1], Qyy[0],
                      lx * Qxy[0], lx2 * Qxy[0], lx * Qxy[1], lx * Qyy[0], lx2 * Qyy[0],
                      Qxy[1], lx * Qxy[1], Qxy[2], Qyy[1], lx * Qyy[1], Qyy[2]};
      pn = warp_sum(pn);
      ps = warp_sum(ps);
#pragma unroll
      for (int a = 0; a < 6; ++a) { pS[a] = warp_sum(pS[a]); pG[a] = warp_sum(pG[a]); }
#pragma unroll
      for (int t = 0; t < 21; ++t) pH[t] = warp_sum(pH[t]);
      if (k == 0)
      {
        nsq = pn;
        src = ps;
#pragma unroll
        for (int a = 0; a < 6; ++a) { S[a] = pS[a]; G[a] = pG[a]; }
#pragma unroll
        for (int t = 0; t < 21; ++t) H[t] = pH[t];
      }
      else
      {
        nsq = __fadd_rn(nsq, pn);
        src = __fadd_rn(src, ps);
#pragma unroll
        for (int a = 0; a < 6; ++a) { S[a] = __fadd_rn(S[a], pS[a]); G[a] = __fadd_rn(G[a], pG[a]); }
#pragma unroll
        for (int t = 0; t < 21; ++t) H[t] = __fadd_rn(H[t], pH[t]);
      }
    }
    if (lane == 0) rec->t0 = t0;
#pragma unroll
    for (int a = 0; a < 6; ++a) { out_sums.S[a] = S[a]; out_sums.G[a] = G[a]; }
#pragma unroll
    for (int t = 0; t < 21; ++t) out_sums.H[t] = H[t];
    out_sums.nsq = nsq;
    out_sums.src = src;
    return true;   // already reduced
  }
  else
  {
    DIC_FOR_EACH_SAMPLE(lane, rx, ry, sum += __ldg(&ref_pack[(size_t)(cy + ly) * w + cx + lx].x);)
    sum = warp_sum(sum);
    const float t0 = sum / (float)size;
    DIC_FOR_EACH_SAMPLE(lane, rx, ry,
      const float4 v = __ldg(&ref_pack[(size_t)(cy + ly) * w + cx + lx]);
      const float rc = v.x - t0;
      const float flx = (float)lx, fly = (float)ly;
      const float sd[6] = {v.y, v.y * flx, v.y * fly, v.z, v.z * flx, v.z * fly};
      nsq = fmaf(rc, rc, nsq);
      src += rc;
      int t = 0;
      _Pragma("unroll")
      for (int a = 0; a < 6; ++a)
      {
        S[a] += sd[a];
        G[a] = fmaf(sd[a], rc, G[a]);
        _Pragma("unroll")
        for (int b = 0; b <= a; ++b) H[t++] += sd[a] * sd[b];
      }
    )
    if (lane == 0) rec->t0 = t0;
  }
  nsq = warp_sum(nsq);
  src = warp_sum(src);
#pragma unroll
  for (int a = 0; a < 6; ++a) { S[a] = warp_sum(S[a]); G[a] = warp_sum(G[a]); }
#pragma unroll
  for (int t = 0; t < 21; ++t) H[t] = warp_sum(H[t]);
#pragma unroll
  for (int a = 0; a < 6; ++a) { out_sums.S[a] = S[a]; out_sums.G[a] = G[a]; }
#pragma unroll
  for (int t = 0; t < 21; ++t) out_sums.H[t] = H[t];
  out_sums.nsq = nsq;
  out_sums.src = src;
  return true;
}

// S and G (lane c < 6 writes entry c, G centred), the norms and valid (lane 0).
__device__ __forceinline__ void poi_write_sums(const PoiSums& q, int size, int lane, PoiRef* __restrict__ rec)
{
  const float m_r = q.src * (1.f / (float)size);
  if (lane < 6)
  {
    float S_l = q.S[0], G_l = q.G[0];
#pragma unroll
    for (int a = 1; a < 6; ++a)
      if (lane == a) { S_l = q.S[a]; G_l = q.G[a]; }
    rec->S[lane] = S_l;
    rec->G[lane] = fmaf(-m_r, S_l, G_l);
  }
  if (lane == 0)
  {
    const float rn_sq = fmaf(-q.src, m_r, q.nsq);
    rec->ref_norm = sqrtf(rn_sq);
    rec->ref_norm_sq = rn_sq;
    rec->sum_rc = q.src;
    rec->valid = 1.f;
  }
}

__global__ void __launch_bounds__(128) k_poi_prepare(const float4* __restrict__ ref_pack, int w, int h,
                                                     const dic_poi* __restrict__ pois, int64_t n,
                                                     int rx, int ry, PoiRef* __restrict__ out)
{
  const int lane = threadIdx.x & 31;
  const int64_t i = (int64_t)blockIdx.x * (blockDim.x / 32) + (threadIdx.x >> 5);
  if (i >= n) return;
  PoiRef* rec = out + i;
  PoiSums q;
  if (!poi_sums(ref_pack, w, h, pois[i].x, pois[i].y, rx, ry, lane, rec, q)) return;
  // Every lane holds the same sums (butterfly reductions), so the LU runs uniformly and
  // lane c < 6 solves and writes column c of the inverse.
  float hf[6][6];
  int t = 0;
#pragma unroll
  for (int a = 0; a < 6; ++a)
#pragma unroll
    for (int b = 0; b <= a; ++b) { hf[a][b] = q.H[t]; hf[b][a] = q.H[t]; ++t; }
  int perm[6];
  lu6(hf, perm);
  if (lane < 6)
  {
    float x[6];
    solve6_column(hf, perm, lane, x);
#pragma unroll
    for (int a = 0; a < 6; ++a) rec->inv_h[a * 6 + lane] = x[a];
  }
  poi_write_sums(q, (2 * rx + 1) * (2 * ry + 1), lane, rec);
}

// --------------------------------------------------------------------------------------
// The same record for 32 POIs per CTA with the inverse batched: four warps form the sums
// of eight POIs each (poi_sums, as above), the 21 Hessian entries go to shared memory, and
// warp 0 factorises and inverts all 32 Hessians at once, one POI per lane (the same lu6 /
// solve6_column code), instead of every warp running one uniform LU per POI.  The inverse
// leaves through shared memory as one 144 B run per POI.
//
// Column sums shared across the CTA (column and pair walks): when the CTA's POIs lie on at most two
// grid rows (one integer y each) and each row's subsets span at most kPrepCols image columns,
// the CTA first forms every such column's ColSums once (one thread per column, the rows in
// order) and the POIs read them from shared memory; only the sums that depend on a POI's mean
// (norm, G) are formed per POI.  Any other set of POIs takes the per-POI path.  Same bits
// either way.
// --------------------------------------------------------------------------------------
constexpr int kPrepPois = 32, kPrepWarps = 4;   // (8 warps per 32 POIs: 0.72 against 0.60 ms at 2048^2)
constexpr int kPrepCols = 256;   // shared columns per grid row (32 POIs at step <= 7 for r 15, <= 6 for r 30)
#ifndef DIC_PREP_SHARED_COLUMNS
#define DIC_PREP_SHARED_COLUMNS 1
#endif
__global__ void __launch_bounds__(kPrepWarps * 32) k_poi_prepare32(const float4* __restrict__ ref_pack, int w,
                                                                  int h, const dic_poi* __restrict__ pois,
                                                                  int64_t n, int rx, int ry,
                                                                  PoiRef* __restrict__ out)
{
  __shared__ float sh_h[kPrepPois * 21];       // odd stride: lane p reads row p conflict-free
  __shared__ float sh_inv[kPrepPois * 37];
  __shared__ int sh_live[kPrepPois];
  __shared__ float sh_col[2][kColSums][kPrepCols];
  __shared__ int sh_row[2][3];                 // per grid row: cy, first column, columns
  __shared__ int sh_shared;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int64_t base = (int64_t)blockIdx.x * kPrepPois;
  const int size = (2 * rx + 1) * (2 * ry + 1);
  if (warp == 0)
  {
    // the POIs' rows and column spans (POIs whose subset leaves the image take no part)
    const int64_t i = base + lane;
    bool valid = false;
    int pcx = 0, pcy = 0;
    if (i < n)
    {
      const float px = pois[i].x, py = pois[i].y;
      valid = py - ry >= 0 && px - rx >= 0 && py + ry <= h - 1 && px + rx <= w - 1;
      pcx = (int)px;
      pcy = (int)py;
    }
    const unsigned vm = __ballot_sync(kFull, valid);
    const int cy0 = vm ? __shfl_sync(kFull, pcy, __ffs(vm) - 1) : 0;
    const bool in0 = valid && pcy == cy0;
    const unsigned rest = vm & ~__ballot_sync(kFull, in0);
    const int cy1 = rest ? __shfl_sync(kFull, pcy, __ffs(rest) - 1) : 0;
    const bool in1 = valid && !in0 && pcy == cy1;
    const bool other = __any_sync(kFull, valid && !in0 && !in1);
    const int lo0 = __reduce_min_sync(kFull, in0 ? pcx : INT_MAX), hi0 = __reduce_max_sync(kFull, in0 ? pcx : INT_MIN);
    const int lo1 = __reduce_min_sync(kFull, in1 ? pcx : INT_MAX), hi1 = __reduce_max_sync(kFull, in1 ? pcx : INT_MIN);
    const int n0 = vm ? hi0 - lo0 + 2 * rx + 1 : 0, n1 = rest ? hi1 - lo1 + 2 * rx + 1 : 0;
    if (lane == 0)
    {
      sh_shared =
          (DIC_PREP_SHARED_COLUMNS && 2 * rx + 1 <= kPairMaxWidth && vm && !other && n0 <= kPrepCols && n1 <= kPrepCols)
              ? 1 : 0;
      sh_row[0][0] = cy0;
      sh_row[0][1] = lo0 - rx;
      sh_row[0][2] = n0;
      sh_row[1][0] = cy1;
      sh_row[1][1] = lo1 - rx;
      sh_row[1][2] = n1;
    }
  }
  __syncthreads();
  const bool shared = sh_shared != 0;
  if (shared)
  {
    const int n0 = sh_row[0][2], total = n0 + sh_row[1][2];
    for (int k = threadIdx.x; k < total; k += kPrepWarps * 32)
    {
      const int g = k < n0 ? 0 : 1, j = k < n0 ? k : k - n0;
      const ColSums c = col_sums(ref_pack + (size_t)(sh_row[g][0] - ry) * w + sh_row[g][1] + j, w, ry);
      sh_col[g][0][j] = c.t;
#pragma unroll
      for (int v = 0; v < 9; ++v) sh_col[g][1 + v][j] = c.q[v];
#pragma unroll
      for (int v = 0; v < 4; ++v) sh_col[g][10 + v][j] = c.s[v];
    }
    __syncthreads();
  }
  for (int k = 0; k < kPrepPois / kPrepWarps; ++k)
  {
    const int p = warp + kPrepWarps * k;
    const int64_t i = base + p;
    bool live = false;
    if (i < n)
    {
      PoiSums q;
      const float px = pois[i].x, py = pois[i].y;
      ColSumsShared cols{nullptr, 0};
      if (shared && py - ry >= 0 && px - rx >= 0 && py + ry <= h - 1 && px + rx <= w - 1)
      {
        const int g = (int)py == sh_row[0][0] ? 0 : 1;
        cols = ColSumsShared{&sh_col[g][0][0] + ((int)px - rx - sh_row[g][1]), kPrepCols};
      }
      live = poi_sums(ref_pack, w, h, px, py, rx, ry, lane, out + i, q, cols);
      if (live)
      {
        poi_write_sums(q, size, lane, out + i);
        if (lane == 0)
        {
#pragma unroll
          for (int t = 0; t < 21; ++t) sh_h[p * 21 + t] = q.H[t];
        }
      }
    }
    if (lane == 0) sh_live[p] = live ? 1 : 0;
  }
  __syncthreads();
  if (warp == 0 && sh_live[lane])
  {
    float hf[6][6];
    int t = 0;
#pragma unroll
    for (int a = 0; a < 6; ++a)
#pragma unroll
      for (int b = 0; b <= a; ++b)
      {
        const float v = sh_h[lane * 21 + t];
        hf[a][b] = v;
        hf[b][a] = v;
        ++t;
      }
    int perm[6];
    lu6(hf, perm);
    for (int c = 0; c < 6; ++c)
    {
      float x[6];
      solve6_column(hf, perm, c, x);
#pragma unroll
      for (int a = 0; a < 6; ++a) sh_inv[lane * 37 + a * 6 + c] = x[a];
    }
  }
  __syncthreads();
  for (int idx = threadIdx.x; idx < kPrepPois * 36; idx += kPrepWarps * 32)
  {
    const int p = idx / 36, e = idx - p * 36;
    if (sh_live[p]) out[base + p].inv_h[e] = sh_inv[p * 37 + e];
  }
}

// --------------------------------------------------------------------------------------
// IC-GN iteration (src/oc_icgn.cpp:168-387): one warp per POI.  Per iteration one pass
// over the (2rx+1)(2ry+1) warped samples: warp the local coordinate, test the
// interpolatable range, gather the texel's 16 B-spline coefficients (one 256-bit load from
// each of the two coefficient planes), evaluate the bicubic polynomial, and accumulate the nine
// single-pass sums (PoiRef).  The warp then reduces the sums with an xor butterfly, solves
// dp = invH * num on lanes 0-5, and every lane applies the same inverse-compositional
// update W <- W * W(dp)^-1.  Control flow is warp-uniform; results do not depend on other
// POIs or on scheduling.
//
// The per-sample test is one combined range test (a NaN coordinate fails it too); only
// when some sample fails does the warp re-walk the subset to apply the CPU's order, out of
// range (-3) before NaN (-5).
// --------------------------------------------------------------------------------------
// Polls of a bounded mbarrier wait before a kernel gives up and reports (a few ms at most).
constexpr uint32_t kWaitPolls = 1u << 22;

struct IcgnParams
{
  const float4* coef;      // tar B-spline table: 2 planes of W*H texels x 2 float4
  const float* lattice = nullptr;   // coefficient [0][0] of every texel (nullable, see on_lattice)
  const float* tar = nullptr;       // target plane (pixel sampling, k_icgn_px): rows of px_pitch(w) floats
  const float4* ref_pack;  // {ref, gx, gy, 0}
  const PoiRef* poi_ref;   // per layout slot
  const int64_t* slot;     // queue index -> layout slot (nullptr: identity)
  dic_poi* pois;
  int64_t n;
  int w, h, rx, ry;
  float conv;
  float max_iter;
  unsigned long long* iter_sum;  // sum of iterations (nullable)
  const int64_t* n_dev = nullptr;   // device-side queue length (overrides n when set)
  const int* enable = nullptr;      // device-side switch: the launch does nothing when 0
  uint32_t wait_polls = kWaitPolls; // k_icgn_tile: bound of its copy wait
  int wait_test = 0;                // k_icgn_tile: 1 = arm the wait but never issue the copy (timeout-path test)
};

// Queue-slot guard shared by the solver kernels: launches sized for the largest possible
// queue take their real length and an on/off switch from device memory, so a frame's
// whole launch sequence can be enqueued (or captured in a graph) before its data-dependent
// branches are known.
template <class Params>
__device__ __forceinline__ bool queue_slot_active(const Params& P, int64_t i)
{
  if (P.enable && *P.enable == 0) return false;
  return i < (P.n_dev ? *P.n_dev : P.n);
}

__device__ __forceinline__ void compose_update(float (&W)[6], const float (&dp)[6])
{
  // W(dp) = [[1+dux, duy, du], [dvx, 1+dvy, dv], [0, 0, 1]]; inverse by cofactors
  // (Eigen compute_inverse_size3 restated), then W <- W * inv.
  const float m0 = 1.f + dp[1], m1 = dp[2], m2 = dp[0];
  const float m3 = dp[4], m4 = 1.f + dp[5], m5 = dp[3];
  const float c00 = m4 * 1.f - m5 * 0.f;
  const float c10 = m5 * 0.f - m3 * 1.f;
  const float c20 = m3 * 0.f - m4 * 0.f;
  const float det = m0 * c00 + m1 * c10 + m2 * c20;
  const float id = 1.f / det;
  const float i0 = c00 * id, i1 = (m2 * 0.f - m1 * 1.f) * id, i2 = (m1 * m5 - m2 * m4) * id;
  const float i3 = c10 * id, i4 = (m0 * 1.f - m2 * 0.f) * id, i5 = (m2 * m3 - m0 * m5) * id;
  const float i6 = c20 * id, i7 = (m1 * 0.f - m0 * 0.f) * id, i8 = (m0 * m4 - m1 * m3) * id;
  const float a0 = W[0], a1 = W[1], a2 = W[2], a3 = W[3], a4 = W[4], a5 = W[5];
  W[0] = a0 * i0 + a1 * i3 + a2 * i6;
  W[1] = a0 * i1 + a1 * i4 + a2 * i7;
  W[2] = a0 * i2 + a1 * i5 + a2 * i8;
  W[3] = a3 * i0 + a4 * i3 + a5 * i6;
  W[4] = a3 * i1 + a4 * i4 + a5 * i7;
  W[5] = a3 * i2 + a4 * i5 + a5 * i8;
}

// Lattice samples.  A warp that is a pure integer translation (ux = uy = vx = vy = 0, u, v
// and the POI's x, y integers: every FFTCC seed) puts every sample on a texel's own
// integer position, where dx = dy = 0 and the bicubic polynomial reduces to its constant
// coefficient [0][0] -- fmaf(c, 0, r) = r, so the full evaluation returns exactly that
// float.  Those iterations read it from the one-float-per-texel lattice plane (4 B per
// sample instead of two 32 B coefficient rows) with the same result.
__device__ __forceinline__ bool on_lattice(const float (&W)[6], float px, float py)
{
  return W[0] == 1.f && W[1] == 0.f && W[3] == 0.f && W[4] == 1.f && W[2] == rintf(W[2]) && W[5] == rintf(W[5]) &&
         px == rintf(px) && py == rintf(py);
}

// 32 bytes of read-only global memory in one 256-bit load (p 32-byte aligned)
__device__ __forceinline__ void ldg_256(const float4* p, float4& a, float4& b)
{
  asm("ld.global.nc.v8.f32 {%0, %1, %2, %3, %4, %5, %6, %7}, [%8];"
      : "=f"(a.x), "=f"(a.y), "=f"(a.z), "=f"(a.w), "=f"(b.x), "=f"(b.y), "=f"(b.z), "=f"(b.w)
      : "l"(p));
}

// The texel's four coefficient rows from the global table (plane = W*H texels).
__device__ __forceinline__ void load_texel(const float4* __restrict__ coef, size_t plane, size_t texel, float4& c0,
                                           float4& c1, float4& c2, float4& c3)
{
  const float4* c = coef + 2 * texel;
  ldg_256(c, c0, c1);
  ldg_256(c + 2 * plane, c2, c3);
}

// Bicubic value at a warped sample from the coefficient planes (texel floor(x, y)).
__device__ __forceinline__ float sample_bspline(const float4* __restrict__ coef, size_t plane, int w,
                                                float gxp, float gyp)
{
  const float fx = floorf(gxp), fy = floorf(gyp);
  const float dx = gxp - fx, dy = gyp - fy;
  float4 c0, c1, c2, c3;
  load_texel(coef, plane, (size_t)((int)fy * w + (int)fx), c0, c1, c2, c3);   // images < 2^31 pixels
  const float r0 = fmaf(fmaf(fmaf(c0.w, dx, c0.z), dx, c0.y), dx, c0.x);
  const float r1 = fmaf(fmaf(fmaf(c1.w, dx, c1.z), dx, c1.y), dx, c1.x);
  const float r2 = fmaf(fmaf(fmaf(c2.w, dx, c2.z), dx, c2.y), dx, c2.x);
  const float r3 = fmaf(fmaf(fmaf(c3.w, dx, c3.z), dx, c3.y), dx, c3.x);
  return fmaf(fmaf(fmaf(r3, dy, r2), dy, r1), dy, r0);
}

// A block of the coefficient table staged in shared memory (k_icgn_tile): texels
// [ox, ox + bx) x [oy, oy + by) of both coefficient planes, plane-major, rows of bx texels
// of 2 float4 (the global layout).  Samples whose texel lies outside it are read from the global table; either way
// the same 16 values enter the same polynomial, so results are bit-identical to
// sample_bspline.
struct CoefTile
{
  const float4* s = nullptr;
  int ox = 0, oy = 0, bx = 0, by = 0;
};

__device__ __forceinline__ float sample_bspline_tile(const CoefTile& T, const float4* __restrict__ coef, size_t plane,
                                                     int w, float gxp, float gyp)
{
  const float fx = floorf(gxp), fy = floorf(gyp);
  const int ix = (int)fx, iy = (int)fy;
  const float dx = gxp - fx, dy = gyp - fy;
  const int tx = ix - T.ox, ty = iy - T.oy;
  float4 c0, c1, c2, c3;
  if ((unsigned)tx < (unsigned)T.bx && (unsigned)ty < (unsigned)T.by)
  {
    const int pl = T.bx * T.by;
    const float4* t = T.s + 2 * (ty * T.bx + tx);
    c0 = t[0];
    c1 = t[1];
    c2 = t[2 * pl];
    c3 = t[2 * pl + 1];
  }
  else
    load_texel(coef, plane, (size_t)(iy * w + ix), c0, c1, c2, c3);
  const float r0 = fmaf(fmaf(fmaf(c0.w, dx, c0.z), dx, c0.y), dx, c0.x);
  const float r1 = fmaf(fmaf(fmaf(c1.w, dx, c1.z), dx, c1.y), dx, c1.x);
  const float r2 = fmaf(fmaf(fmaf(c2.w, dx, c2.z), dx, c2.y), dx, c2.x);
  const float r3 = fmaf(fmaf(fmaf(c3.w, dx, c3.z), dx, c3.y), dx, c3.x);
  return fmaf(fmaf(fmaf(r3, dy, r2), dy, r1), dy, r0);
}

// --------------------------------------------------------------------------------------
// Pixel sampling.  The bicubic value at (ix + dx, iy + dy) is the texel's polynomial
// sum_{a,b} P[3-a][3-b] dy^a dx^b with P = BC q BC^T over the 4 x 4 pixels q[n][m] =
// I(iy - 1 + n, ix - 1 + m) (k_prepare_tar).  Regrouped by pixel it is
//   sum_n wy[n] sum_m wx[m] q[n][m],   w[m](d) = sum_b BC[3-b][m] d^b,
// the B-spline weights of the BC matrix.  Evaluated that way a sample reads 16 pixels (4 B
// each) instead of the texel's 16 coefficients (64 B), so a warp's whole warped subset fits
// in a few KB of shared memory (k_icgn_px) and the coefficient table is not needed.  The
// polynomial is the same, the rounding is not: results agree with the table forms to float
// rounding, not bit for bit.  At d = 0 the weights are exactly (0, 1, 0, 0) (BC's last row),
// so a sample on the lattice returns the pixel itself, as the table does.
// --------------------------------------------------------------------------------------
// Row pitch (floats) of the target plane the pixel-sampled IC-GN reads: W rounded up to a
// multiple of 4, so every row starts on the 16-byte boundary TMA needs (the plane itself where
// W is a multiple of 4, a padded copy otherwise).
__host__ __device__ constexpr int px_pitch(int w) { return (w + 3) & ~3; }

// The weights of both axes at once, d = (dx, dy): w[m] = (wx[m], wy[m]).  Packed FP32 pairs
// (fma.rn.f32x2, sm_100 and later) round each half like the scalar operation, so the
// values are the scalar Horner forms' bit for bit, in half the instructions.
__device__ __forceinline__ float2 k2(float v) { return make_float2(v, v); }
__device__ __forceinline__ void bspline_weights2(float2 d, float2 (&w)[4])
{
  w[0] = __fmul2_rn(__ffma2_rn(__ffma2_rn(k2(-144.0f / 336.0f), d, k2(342.0f / 336.0f)), d, k2(-198.0f / 336.0f)), d);
  w[1] = __ffma2_rn(__ffma2_rn(__ffma2_rn(k2(384.0f / 336.0f), d, k2(-702.0f / 336.0f)), d, k2(-18.0f / 336.0f)), d,
                    k2(1.0f));
  w[2] = __fmul2_rn(__ffma2_rn(__ffma2_rn(k2(-384.0f / 336.0f), d, k2(450.0f / 336.0f)), d, k2(270.0f / 336.0f)), d);
  w[3] = __fmul2_rn(__ffma2_rn(__ffma2_rn(k2(144.0f / 336.0f), d, k2(-90.0f / 336.0f)), d, k2(-54.0f / 336.0f)), d);
}

// The dynamic shared memory of the pixel-window kernels (k_icgn_px, k_icgn_batch_px) as
// floats: indexing it with 32-bit offsets keeps the window loads in the shared window's own
// 32-bit addressing, and as ordinary loads the compiler keeps them after the copy's mbarrier
// wait.
extern __shared__ __align__(128) float px_smem[];

// A warp's block of the target plane in shared memory: pixels [ox, ox + bx) x [oy, oy + by),
// rows of bx floats, from px_smem[s].  bx = 0: nothing staged.  (A compile-time row pitch,
// which turns the 16 loads of a sample into one base plus immediate offsets, was measured
// slower: 3.06 against 2.77 ms of IC-GN on the 2048x2048 pair.)
struct PixelTile
{
  int s = 0;
  int ox = 0, oy = 0, bx = 0, by = 0;
};

// sum_n wy[n] sum_m wx[m] q[n][m] with w[m] = (wx[m], wy[m]), pixels from a load functor
// ld(n, m).  (Packing the row sums as FP32 pairs needs the x weights broadcast into pairs,
// which costs the moves it saves: 2.96 against 2.94 ms of IC-GN on the 2048x2048 pair.)
template <class Ld>
__device__ __forceinline__ float eval_pixels(const float2 (&w)[4], Ld ld)
{
  float h[4];
#pragma unroll
  for (int n = 0; n < 4; ++n)
    h[n] = fmaf(w[3].x, ld(n, 3), fmaf(w[2].x, ld(n, 2), fmaf(w[1].x, ld(n, 1), w[0].x * ld(n, 0))));
  return fmaf(w[3].y, h[3], fmaf(w[2].y, h[2], fmaf(w[1].y, h[1], w[0].y * h[0])));
}

// The weights of a sample and the window address of its 4 x 4 support's first pixel.
__device__ __forceinline__ void pixel_setup(float gxp, float gyp, float2 (&w)[4], int& ix, int& iy)
{
  const float fx = floorf(gxp), fy = floorf(gyp);
  ix = (int)fx;
  iy = (int)fy;
  bspline_weights2(make_float2(gxp - fx, gyp - fy), w);
}

__device__ __forceinline__ float sample_pixels(const PixelTile& T, const float* __restrict__ tar, int pitch, float gxp,
                                               float gyp)
{
  float2 wt[4];
  int ix, iy;
  pixel_setup(gxp, gyp, wt, ix, iy);
  const int tx = ix - 1 - T.ox, ty = iy - 1 - T.oy;
  if (tx >= 0 && ty >= 0 && tx <= T.bx - 4 && ty <= T.by - 4)
  {
    const int a = T.s + (ty * T.bx + tx);
    const int row = T.bx;
    return eval_pixels(wt, [&](int n, int m) { return px_smem[a + n * row + m]; });
  }
  const float* g = tar + ((size_t)(iy - 1) * pitch + (ix - 1));   // images < 2^31 pixels
  return eval_pixels(wt, [&](int n, int m) { return __ldg(g + (size_t)n * pitch + m); });
}

// A sample whose support lies in the window (the caller has checked): no tests.
__device__ __forceinline__ float sample_window(const PixelTile& T, int row, float gxp, float gyp)
{
  float2 wt[4];
  int ix, iy;
  pixel_setup(gxp, gyp, wt, ix, iy);
  const int a = T.s + ((iy - 1 - T.oy) * T.bx + (ix - 1 - T.ox));
  return eval_pixels(wt, [&](int n, int m) { return px_smem[a + n * row + m]; });
}

// Column walk under pixel sampling: whether every sample of the current warp lies in the
// interpolation range and has its support inside the window.  Sample coordinates are
// px + fmaf(W1, ly, fmaf(W0, lx, W2)) (y likewise), rounded monotone functions of lx and of
// ly, so their extremes are the subset's corners, computed here with the same expression;
// lanes 0-3 take one corner each.  Warp-uniform.
__device__ __forceinline__ bool window_covers(const float (&W)[6], float px, float py, int rx, int ry, float xmax,
                                              float ymax, const PixelTile& T, int lane)
{
  bool ok = true;
  if (lane < 4)
  {
    const float flx = (lane & 1) ? (float)rx : (float)-rx, fly = (lane & 2) ? (float)ry : (float)-ry;
    const float gxp = px + fmaf(W[1], fly, fmaf(W[0], flx, W[2]));
    const float gyp = py + fmaf(W[4], fly, fmaf(W[3], flx, W[5]));
    ok = gxp >= 1.f && gyp >= 1.f && gxp < xmax && gyp < ymax;
    if (ok)
    {
      const int tx = (int)floorf(gxp) - 1 - T.ox, ty = (int)floorf(gyp) - 1 - T.oy;
      ok = tx >= 0 && ty >= 0 && tx <= T.bx - 4 && ty <= T.by - 4;
    }
  }
  return __all_sync(kFull, ok);
}

// the pixel at an integer sample (the lattice case of sample_pixels)
__device__ __forceinline__ float pixel_at(const PixelTile& T, const float* __restrict__ tar, int pitch, float gxp,
                                          float gyp)
{
  const int ix = (int)gxp, iy = (int)gyp;
  const int tx = ix - T.ox, ty = iy - T.oy;
  if (tx >= 0 && ty >= 0 && tx < T.bx && ty < T.by) return px_smem[T.s + ty * T.bx + tx];
  return __ldg(tar + ((size_t)iy * pitch + ix));
}

// The column walk's checked row loop under pixel sampling, for iterations whose samples are
// not all inside the range and the window: per-sample range tests, window or global-plane
// reads, the same sums in the same order as the fast loop.  Returns the sums (A0, A1, A2, B0,
// B2, B3, B5) and whether a sample left the range.  (The fast loop's code generation is
// sensitive to this rare path: written as this function and inlined, k_icgn_px runs 2.80 ms
// on the 2048x2048 pair; as a call, 2.84 ms; as the same loop written inside icgn_solve with
// the padded pitch, 3.00 ms.)
struct ColumnSums
{
  float A0, A1, A2, B0, B2, B3, B5;
  int bad;
};
__device__ __forceinline__ ColumnSums px_column_checked(const float* __restrict__ tar, int w, int h, PixelTile T,
                                                     const float4* __restrict__ ref_col, float px, float py, float W0,
                                                     float W1, float W2, float W3, float W4, float W5, float flx_col,
                                                     float t0, int ry, int lat)
{
  ColumnSums c{0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0};
  const float xmax = (float)(w - 2), ymax = (float)(h - 2);
  const int pitch = px_pitch(w);
  const float ax = fmaf(W0, flx_col, W2), ay = fmaf(W3, flx_col, W5);
  for (int r = 0; r < 2 * ry + 1; ++r)
  {
    const float fly = (float)(r - ry);
    const float gxp = px + fmaf(W1, fly, ax);
    const float gyp = py + fmaf(W4, fly, ay);
    if (!(gxp >= 1.f && gyp >= 1.f && gxp < xmax && gyp < ymax))
    {
      c.bad = 1;
      continue;
    }
    const float t = lat ? pixel_at(T, tar, pitch, gxp, gyp) : sample_pixels(T, tar, pitch, gxp, gyp);
    const float4 rv = __ldg(ref_col + (size_t)r * w);
    const float tau = t - t0;
    const float rc = rv.x - t0;
    c.A0 += tau;
    c.A1 = fmaf(tau, tau, c.A1);
    c.A2 = fmaf(tau, rc, c.A2);
    const float gt = __fmul_rn(rv.y, tau), ht = __fmul_rn(rv.z, tau);
    c.B0 = __fadd_rn(c.B0, gt);
    c.B2 = fmaf(gt, fly, c.B2);
    c.B3 = __fadd_rn(c.B3, ht);
    c.B5 = fmaf(ht, fly, c.B5);
  }
  return c;
}

// Sample sources of icgn_solve: the global coefficient table, a coefficient block staged
// in shared memory (k_icgn_tile), or the target pixels (k_icgn_px).
constexpr int kSrcTable = 0, kSrcCoefTile = 1, kSrcPixels = 2;

// Rows of the column walk unrolled together (their gathers in flight at once), and the
// warps per SM the IC-GN launch bounds keep resident (which sets the register budget).
// The 256-bit coefficient gathers are served from L2 and their latency is what the kernel
// waits on; more resident warps (the persistent form's 32 at 64 registers) hide it better
// than more rows per warp (two rows at 28 warps: 3.44 ms; one row at 32 warps: 3.33 ms on
// the 2048x2048 pair; 3 or 4 rows, or 24 warps with more registers, were slower).
#ifndef DIC_ICGN_ROW_UNROLL
#define DIC_ICGN_ROW_UNROLL 1
#endif
#ifndef DIC_ICGN_RESIDENT_WARPS
#define DIC_ICGN_RESIDENT_WARPS 28
#endif
constexpr int kIcgnRowUnroll = DIC_ICGN_ROW_UNROLL;

// One POI (queue index i) on the calling warp; shared by the per-queue launch (k_icgn) and
// the persistent multi-job launch (k_icgn_batch, which keeps one row in flight: its job
// lookup leaves no registers for two without spilling).
template <bool kColumn, int kSrc = kSrcTable, int kRowUnroll = kIcgnRowUnroll, class Tile = CoefTile>
__device__ __forceinline__ void icgn_solve(const IcgnParams& P, int64_t i, int lane, const Tile& T = Tile{})
{
  dic_poi* poi = P.pois + i;
  const float px = poi->x, py = poi->y;
  const float u_in = poi->u, ux_in = poi->ux, uy_in = poi->uy;
  const float v_in = poi->v, vx_in = poi->vx, vy_in = poi->vy;
  const float zncc_in = poi->zncc;
  const int w = P.w, h = P.h, rx = P.rx, ry = P.ry;
  // Entry test (src/oc_icgn.cpp:184-191).
  if (py - ry < 0 || px - rx < 0 || py + ry > h - 1 || px + rx > w - 1 || fabsf(u_in) >= w ||
      fabsf(v_in) >= h || zncc_in < 0 || isnan(u_in) || isnan(v_in))
  {
    if (lane == 0) poi->zncc = zncc_in >= 0 ? -3.f : zncc_in;
    return;
  }
  // Only t0 stays live across the sample loop; the other per-POI constants are re-read
  // (L1-resident) after each reduction, which keeps the loop within 64 registers.
  const PoiRef* R = P.poi_ref + (P.slot ? P.slot[i] : i);
  const float t0 = R->t0;
  const int sw = 2 * rx + 1, size = sw * (2 * ry + 1);
  const float inv_size = 1.f / (float)size;
  const int cx = (int)px, cy = (int)py;
  const size_t plane = (size_t)w * h;
  const float4* __restrict__ coef = P.coef;
  const float4* __restrict__ ref_pack = P.ref_pack;
  // warp matrix rows (Deformation2D1::setWarp, src/oc_deformation.cpp:116-128)
  float W[6] = {1.f + ux_in, uy_in, u_in, vx_in, 1.f + vy_in, v_in};
  const float rx2 = (float)(rx * rx), ry2 = (float)(ry * ry);
  const float xmax = (float)(w - 2), ymax = (float)(h - 2);
  constexpr bool column_walk = kColumn;   // the host picks kColumn = (2 rx + 1 <= 32)
  const bool col_active = lane < sw;
  const float flx_col = (float)(lane - rx);
  const float4* ref_col = ref_pack + (size_t)(cy - ry) * w + cx + (lane - rx);
  int it = 0;
  float conv = 0.f, znssd = 0.f;
  int status = 0;  // 0 ok, -3 out of range, -5 NaN coordinate
  do
  {
    ++it;
    float A0 = 0.f, A1 = 0.f, A2 = 0.f, B[6] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
    bool bad = false;
    const bool lat = kSrc != kSrcCoefTile && (kSrc == kSrcPixels || P.lattice) && on_lattice(W, px, py);   // warp-uniform
    if constexpr (column_walk)
    {
      bool fast = false;
      if constexpr (kSrc == kSrcPixels)
        fast = !lat && window_covers(W, px, py, rx, ry, xmax, ymax, T, lane);
      if (fast)
      {
        if constexpr (kSrc == kSrcPixels)
          if (col_active)
          {
            // every sample in range and in the window: no per-sample tests
            const float ax = fmaf(W[0], flx_col, W[2]), ay = fmaf(W[3], flx_col, W[5]);
            const int row = T.bx;
            // (Loading the reference texel a row ahead of its use shortens the L2 waits but
            // costs the registers that keep 32 warps resident: 3.27 against 2.94 ms.)
            const float4* rp = ref_col;
#pragma unroll kRowUnroll
            for (int r = 0; r < 2 * ry + 1; ++r)
            {
              const float4 cur = __ldg(rp);
              rp += w;
              const float fly = (float)(r - ry);
              const float gxp = px + fmaf(W[1], fly, ax);
              const float gyp = py + fmaf(W[4], fly, ay);
              const float t = sample_window(T, row, gxp, gyp);
              const float tau = t - t0;
              const float rc = cur.x - t0;
              A0 += tau;
              A1 = fmaf(tau, tau, A1);
              A2 = fmaf(tau, rc, A2);
              const float gt = __fmul_rn(cur.y, tau), ht = __fmul_rn(cur.z, tau);
              B[0] = __fadd_rn(B[0], gt);
              B[2] = fmaf(gt, fly, B[2]);
              B[3] = __fadd_rn(B[3], ht);
              B[5] = fmaf(ht, fly, B[5]);
            }
          }
      }
      else if (kSrc == kSrcPixels && col_active)
      {
        if constexpr (kSrc == kSrcPixels)
        {
          const ColumnSums c = px_column_checked(P.tar, w, h, T, ref_col, px, py, W[0], W[1], W[2], W[3], W[4], W[5],
                                                 flx_col, t0, ry, lat ? 1 : 0);
          A0 = c.A0;
          A1 = c.A1;
          A2 = c.A2;
          B[0] = c.B0;
          B[2] = c.B2;
          B[3] = c.B3;
          B[5] = c.B5;
          bad = c.bad != 0;
        }
      }
      else if (col_active)
      {
        const float ax = fmaf(W[0], flx_col, W[2]), ay = fmaf(W[3], flx_col, W[5]);
#pragma unroll kRowUnroll
        for (int r = 0; r < 2 * ry + 1; ++r)
        {
          const float fly = (float)(r - ry);
          const float gxp = px + fmaf(W[1], fly, ax);
          const float gyp = py + fmaf(W[4], fly, ay);
          if (!(gxp >= 1.f && gyp >= 1.f && gxp < xmax && gyp < ymax))
          {
            bad = true;
            continue;
          }
          float t;
          if constexpr (kSrc == kSrcCoefTile)
            t = sample_bspline_tile(T, coef, plane, w, gxp, gyp);
          else if (lat)
            t = __ldg(P.lattice + ((size_t)(int)gyp * w + (int)gxp));
          else
            t = sample_bspline(coef, plane, w, gxp, gyp);
          const float4 rv = __ldg(ref_col + (size_t)r * w);
          const float tau = t - t0;
          const float rc = rv.x - t0;
          A0 += tau;
          A1 = fmaf(tau, tau, A1);
          A2 = fmaf(tau, rc, A2);
          // __fmul_rn / __fadd_rn: never contracted, so these match k_poi_prepare's G bit for bit
          const float gt = __fmul_rn(rv.y, tau), ht = __fmul_rn(rv.z, tau);
          B[0] = __fadd_rn(B[0], gt);
          B[2] = fmaf(gt, fly, B[2]);
          B[3] = __fadd_rn(B[3], ht);
          B[5] = fmaf(ht, fly, B[5]);
        }
      }
      B[1] = flx_col * B[0];
      B[4] = flx_col * B[3];
    }
    else
    {
      DIC_FOR_EACH_SAMPLE(lane, rx, ry,
        const float flx = (float)lx, fly = (float)ly;
        const float gxp = px + (W[0] * flx + W[1] * fly + W[2]);
        const float gyp = py + (W[3] * flx + W[4] * fly + W[5]);
        if (!(gxp >= 1.f && gyp >= 1.f && gxp < xmax && gyp < ymax))
          bad = true;
        else
        {
          float t;
          if constexpr (kSrc == kSrcPixels)
            t = lat ? pixel_at(T, P.tar, px_pitch(w), gxp, gyp) : sample_pixels(T, P.tar, px_pitch(w), gxp, gyp);
          else
            t = lat ? __ldg(P.lattice + ((size_t)(int)gyp * w + (int)gxp)) : sample_bspline(coef, plane, w, gxp, gyp);
          const float4 rv = __ldg(ref_pack + (size_t)(cy + ly) * w + (cx + lx));
          const float tau = t - t0;
          const float rc = rv.x - t0;
          A0 += tau;
          A1 = fmaf(tau, tau, A1);
          A2 = fmaf(tau, rc, A2);
          B[0] = fmaf(rv.y, tau, B[0]);
          B[1] = fmaf(rv.y * flx, tau, B[1]);
          B[2] = fmaf(rv.y * fly, tau, B[2]);
          B[3] = fmaf(rv.z, tau, B[3]);
          B[4] = fmaf(rv.z * flx, tau, B[4]);
          B[5] = fmaf(rv.z * fly, tau, B[5]);
        }
      )
    }
    if (__any_sync(kFull, bad))
    {
      // Rare path: classify with the CPU's order (src/oc_icgn.cpp:266-301).
      bool oob = false;
      if constexpr (column_walk)
      {
        if (col_active)
        {
          const float ax = fmaf(W[0], flx_col, W[2]), ay = fmaf(W[3], flx_col, W[5]);
          for (int r = 0; r < 2 * ry + 1; ++r)
          {
            const float fly = (float)(r - ry);
            const float gxp = px + fmaf(W[1], fly, ax), gyp = py + fmaf(W[4], fly, ay);
            if (gxp < 1.f || gyp < 1.f || gxp >= xmax || gyp >= ymax) oob = true;
          }
        }
      }
      else
      {
        DIC_FOR_EACH_SAMPLE(lane, rx, ry,
          const float gxp = px + (W[0] * (float)lx + W[1] * (float)ly + W[2]);
          const float gyp = py + (W[3] * (float)lx + W[4] * (float)ly + W[5]);
          if (gxp < 1.f || gyp < 1.f || gxp >= xmax || gyp >= ymax) oob = true;
        )
      }
      status = __any_sync(kFull, oob) ? -3 : -5;
      break;
    }
    A0 = warp_sum(A0);
    A1 = warp_sum(A1);
    A2 = warp_sum(A2);
#pragma unroll
    for (int a = 0; a < 6; ++a) B[a] = warp_sum(B[a]);
    const float ref_norm = R->ref_norm, ref_norm_sq = R->ref_norm_sq, sum_rc = R->sum_rc;
    const float mean_tau = A0 * inv_size;
    const float tnorm_sq = fmaf(-A0, mean_tau, A1);
    // A flat target subset has zero norm; the CPU then divides by zero and the POI ends
    // as NaN (-5).  Rounding can leave a tiny residue here, so force the same outcome.
    const float tar_norm = tnorm_sq > 0.f ? sqrtf(tnorm_sq) : __int_as_float(0x7fc00000);
    const float s = ref_norm / tar_norm;
    const float tc_rc = fmaf(-mean_tau, sum_rc, A2);
    const float esq = s * s * tnorm_sq - 2.f * s * tc_rc + ref_norm_sq;
    znssd = esq / (ref_norm * ref_norm);
    // lane a < 6: num_a, then dp_a = invH row a . num
    const int row = lane < 6 ? lane : 0;
    const float S_l = R->S[row], G_l = R->G[row];
    float num_l = 0.f;
#pragma unroll
    for (int a = 0; a < 6; ++a)
      if (lane == a) num_l = s * fmaf(-mean_tau, S_l, B[a]) - G_l;
    float dp_l = 0.f;
#pragma unroll
    for (int c = 0; c < 6; ++c)
    {
      const float nc = __shfl_sync(kFull, num_l, c);
      dp_l += R->inv_h[row * 6 + c] * nc;
    }
    float dp[6];
#pragma unroll
    for (int a = 0; a < 6; ++a) dp[a] = __shfl_sync(kFull, dp_l, a);
    compose_update(W, dp);
    conv = sqrtf(dp[0] * dp[0] + dp[1] * dp[1] * rx2 + dp[2] * dp[2] * ry2 + dp[3] * dp[3] +
                 dp[4] * dp[4] * rx2 + dp[5] * dp[5] * ry2);
  } while ((float)it < P.max_iter && conv >= P.conv);

  if (lane != 0) return;
  if (P.iter_sum) atomicAdd(P.iter_sum, (unsigned long long)it);
  if (status == -3) { poi->zncc = -3.f; return; }   // src/oc_icgn.cpp:285-289
  if (status == -5) { poi->zncc = -5.f; return; }   // :297-301
  float u = W[2], ux = W[0] - 1.f, uy = W[1], v = W[5], vx = W[3], vy = W[4] - 1.f;
  float zncc = 0.5f * (2.f - znssd);
  if (conv >= P.conv && (float)it >= P.max_iter) zncc = -4.f;
  // The incoming guess is re-read here (the record is still unmodified) rather than kept
  // live across the iteration loop.
  const float u_init = poi->u, v_init = poi->v;
  if (isnan(zncc) || isnan(u) || isnan(v))
  {
    u = u_init;
    v = v_init;
    zncc = -5.f;
  }
  poi->u = u; poi->ux = ux; poi->uy = uy;
  poi->v = v; poi->vx = vx; poi->vy = vy;
  poi->u0 = u_init;
  poi->v0 = v_init;
  poi->zncc = zncc;
  poi->iteration = (float)it;
  poi->convergence = conv;
}

// Launch shape: kWarps POIs per CTA (one warp each); the occupancy hint keeps
// DIC_ICGN_RESIDENT_WARPS (28: 72 registers per thread) warps per SM resident for every shape.
constexpr int icgn_min_blocks(int warps) { return DIC_ICGN_RESIDENT_WARPS / warps; }
// The persistent single-queue form keeps 32 warps per SM (64 registers) with one row in
// flight per lane: its gathers wait on L2, and more warps hide that better than a second
// row does (3.43 -> 3.33 ms on the 2048x2048 pair; the grid and batch forms spill at 64).
#ifndef DIC_ICGN_PERSISTENT_RESIDENT_WARPS
#define DIC_ICGN_PERSISTENT_RESIDENT_WARPS 32
#endif
constexpr int icgn_persistent_min_blocks(int warps) { return DIC_ICGN_PERSISTENT_RESIDENT_WARPS / warps; }

template <bool kColumn, int kWarps = 4>
__global__ void __launch_bounds__(kWarps * 32, icgn_min_blocks(kWarps)) k_icgn(IcgnParams P)
{
  const int lane = threadIdx.x & 31;
  const int64_t i = (int64_t)blockIdx.x * (blockDim.x / 32) + (threadIdx.x >> 5);
  if (!queue_slot_active(P, i)) return;
  icgn_solve<kColumn>(P, i, lane);
}

// Persistent single-queue form: CTAs stay resident and each warp takes the next POI from an
// atomic counter (reset to 0 before the launch), so POIs that need many iterations do not
// hold a whole CTA back.  Same solver and guards as k_icgn.
template <bool kColumn, int kWarps = 4>
__global__ void __launch_bounds__(kWarps * 32, icgn_persistent_min_blocks(kWarps))
    k_icgn_persistent(IcgnParams P, unsigned long long* next)
{
  const int lane = threadIdx.x & 31;
  if (P.enable && *P.enable == 0) return;
  for (;;)
  {
    unsigned long long t = 0;
    if (lane == 0) t = atomicAdd(next, 1ull);
    const int64_t i = (int64_t)__shfl_sync(kFull, t, 0);
    if (!queue_slot_active(P, i)) return;
    icgn_solve<kColumn, kSrcTable, 1>(P, i, lane);
  }
}

// --------------------------------------------------------------------------------------
// Pair walk: IC-GN for subsets of 33 to 64 columns (subset radius 16 to 31), one or two
// warps per POI.  The columns form two classes, c = pair_column(l, k) for lane l and class k
// (the halves 32 k + l); each class is walked like the column walk (the lane's lx is constant, so the
// lx-weighted sums factor out of the row loop) and butterfly-reduced on its own, and the
// two class totals are added in class order.  With one warp per POI the warp walks both
// classes in turn; with two, warp k of the pair walks class k and the pair exchanges its
// class totals through shared memory (double-buffered by iteration parity, one named
// barrier per iteration).  The sums are the same bits either way, so results do not depend
// on the warps per POI; k_poi_prepare forms the per-POI constants in the same class order,
// which keeps the exact self-match.
// --------------------------------------------------------------------------------------
// barrier of the two warps of a pair (ids 1..4, 0 is __syncthreads).  The id is an immediate
// in every branch, so the kernel reserves only the barriers it names (a register id makes
// ptxas reserve all 16 per CTA).
__device__ __forceinline__ void pair_sync(int id)
{
  switch (id)
  {
    case 1: asm volatile("bar.sync 1, 64;" ::: "memory"); break;
    case 2: asm volatile("bar.sync 2, 64;" ::: "memory"); break;
    case 3: asm volatile("bar.sync 3, 64;" ::: "memory"); break;
    default: asm volatile("bar.sync 4, 64;" ::: "memory"); break;
  }
}

// The nine single-pass sums of column class k under warp W, butterfly-reduced (s: A0, A1,
// A2, B0..B5).  Returns (warp-uniformly) whether a sample of the class failed the range test.
__device__ __forceinline__ bool pair_class_sums(const IcgnParams& P, int k, int lane, float px, float py, int cx,
                                                int cy, float t0, const float (&W)[6], float (&s)[9])
{
  const int rx = P.rx, ry = P.ry, w = P.w;
  const int c = pair_column(lane, k);
  const float flx = (float)(c - rx);
  const float xmax = (float)(P.w - 2), ymax = (float)(P.h - 2);
  const size_t plane = (size_t)P.w * P.h;
  float A0 = 0.f, A1 = 0.f, A2 = 0.f, B[6] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
  bool bad = false;
  const bool lat = P.lattice && on_lattice(W, px, py);
  if (c < 2 * rx + 1)
  {
    const float4* __restrict__ ref_col = P.ref_pack + (size_t)(cy - ry) * w + cx + (c - rx);
    const float ax = fmaf(W[0], flx, W[2]), ay = fmaf(W[3], flx, W[5]);
    for (int r = 0; r < 2 * ry + 1; ++r)
    {
      const float fly = (float)(r - ry);
      const float gxp = px + fmaf(W[1], fly, ax);
      const float gyp = py + fmaf(W[4], fly, ay);
      if (!(gxp >= 1.f && gyp >= 1.f && gxp < xmax && gyp < ymax))
      {
        bad = true;
        continue;
      }
      const float t = lat ? __ldg(P.lattice + ((size_t)(int)gyp * w + (int)gxp)) : sample_bspline(P.coef, plane, w, gxp, gyp);
      const float4 rv = __ldg(ref_col + (size_t)r * w);
      const float tau = t - t0;
      const float rc = rv.x - t0;
      A0 += tau;
      A1 = fmaf(tau, tau, A1);
      A2 = fmaf(tau, rc, A2);
      const float gt = __fmul_rn(rv.y, tau), ht = __fmul_rn(rv.z, tau);
      B[0] = __fadd_rn(B[0], gt);
      B[2] = fmaf(gt, fly, B[2]);
      B[3] = __fadd_rn(B[3], ht);
      B[5] = fmaf(ht, fly, B[5]);
    }
  }
  B[1] = flx * B[0];
  B[4] = flx * B[3];
  const bool any_bad = __any_sync(kFull, bad);
  s[0] = warp_sum(A0);
  s[1] = warp_sum(A1);
  s[2] = warp_sum(A2);
#pragma unroll
  for (int a = 0; a < 6; ++a) s[3 + a] = warp_sum(B[a]);
  return any_bad;
}

// The same nine sums under pixel sampling (T: the POI's staged window).  `fast`: every sample of
// the subset lies in the interpolation range and has its support in the window (window_covers,
// once per iteration), so the rows run without tests; otherwise the checked loop of the column
// walk (px_column_checked: range tests, window or global plane; `lat` on the pixel lattice).
// Same sums in the same order as pair_class_sums, same bits in either loop.
__device__ __forceinline__ bool pair_class_sums_px(const IcgnParams& P, const PixelTile& T, int k, int lane, float px,
                                                   float py, int cx, int cy, float t0, const float (&W)[6], bool fast,
                                                   bool lat, float (&s)[9])
{
  const int rx = P.rx, ry = P.ry, w = P.w;
  const int c = pair_column(lane, k);
  const float flx = (float)(c - rx);
  float A0 = 0.f, A1 = 0.f, A2 = 0.f, B[6] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
  bool bad = false;
  if (c < 2 * rx + 1)
  {
    const float4* __restrict__ ref_col = P.ref_pack + (size_t)(cy - ry) * w + cx + (c - rx);
    if (fast)
    {
      const float ax = fmaf(W[0], flx, W[2]), ay = fmaf(W[3], flx, W[5]);
      const int row = T.bx;
      const float4* rp = ref_col;
      const auto accumulate = [&](float t, const float4& cur, float fly) {
        const float tau = t - t0;
        const float rc = cur.x - t0;
        A0 += tau;
        A1 = fmaf(tau, tau, A1);
        A2 = fmaf(tau, rc, A2);
        const float gt = __fmul_rn(cur.y, tau), ht = __fmul_rn(cur.z, tau);
        B[0] = __fadd_rn(B[0], gt);
        B[2] = fmaf(gt, fly, B[2]);
        B[3] = __fadd_rn(B[3], ht);
        B[5] = fmaf(ht, fly, B[5]);
      };
      for (int r = 0; r < 2 * ry + 1; ++r)
      {
        const float4 cur = __ldg(rp);
        rp += w;
        const float fly = (float)(r - ry);
        accumulate(sample_window(T, row, px + fmaf(W[1], fly, ax), py + fmaf(W[4], fly, ay)), cur, fly);
      }
    }
    else
    {
      const ColumnSums cs = px_column_checked(P.tar, w, P.h, T, ref_col, px, py, W[0], W[1], W[2], W[3], W[4], W[5],
                                              flx, t0, ry, lat ? 1 : 0);
      A0 = cs.A0;
      A1 = cs.A1;
      A2 = cs.A2;
      B[0] = cs.B0;
      B[2] = cs.B2;
      B[3] = cs.B3;
      B[5] = cs.B5;
      bad = cs.bad != 0;
    }
  }
  B[1] = flx * B[0];
  B[4] = flx * B[3];
  const bool any_bad = __any_sync(kFull, bad);
  s[0] = warp_sum(A0);
  s[1] = warp_sum(A1);
  s[2] = warp_sum(A2);
#pragma unroll
  for (int a = 0; a < 6; ++a) s[3 + a] = warp_sum(B[a]);
  return any_bad;
}

// Whether a sample of column class k lies outside the interpolatable range (warp-uniform).
__device__ __forceinline__ bool pair_class_oob(const IcgnParams& P, int k, int lane, float px, float py,
                                               const float (&W)[6])
{
  const int c = pair_column(lane, k), ry = P.ry;
  const float flx = (float)(c - P.rx);
  const float xmax = (float)(P.w - 2), ymax = (float)(P.h - 2);
  bool oob = false;
  if (c < 2 * P.rx + 1)
  {
    const float ax = fmaf(W[0], flx, W[2]), ay = fmaf(W[3], flx, W[5]);
    for (int r = 0; r < 2 * ry + 1; ++r)
    {
      const float fly = (float)(r - ry);
      const float gxp = px + fmaf(W[1], fly, ax), gyp = py + fmaf(W[4], fly, ay);
      if (gxp < 1.f || gyp < 1.f || gxp >= xmax || gyp >= ymax) oob = true;
    }
  }
  return __any_sync(kFull, oob);
}

// Shared exchange area of one POI pair: [iteration parity][class][9 sums + bad flag], and
// the two classes' out-of-range flags.
struct PairExchange
{
  float sums[2][2][10];
  int oob[2];
};

// One POI (queue index i) on one warp (kPoiWarps 1) or on the two warps of a pair
// (kPoiWarps 2: this warp walks class `cls`, barrier `bar` joins the pair).  Same rules,
// status codes and outputs as icgn_solve; class 0's lane 0 writes the record.
template <int kPoiWarps, int kSrc = kSrcTable>
__device__ __forceinline__ void icgn_solve_pair(const IcgnParams& P, int64_t i, int lane, int cls,
                                                PairExchange* xch, int bar, const PixelTile& T = PixelTile{})
{
  dic_poi* poi = P.pois + i;
  const float px = poi->x, py = poi->y;
  const float u_in = poi->u, ux_in = poi->ux, uy_in = poi->uy;
  const float v_in = poi->v, vx_in = poi->vx, vy_in = poi->vy;
  const float zncc_in = poi->zncc;
  const int w = P.w, h = P.h, rx = P.rx, ry = P.ry;
  // Entry test (src/oc_icgn.cpp:184-191); both warps of a pair take the same branch.
  if (py - ry < 0 || px - rx < 0 || py + ry > h - 1 || px + rx > w - 1 || fabsf(u_in) >= w ||
      fabsf(v_in) >= h || zncc_in < 0 || isnan(u_in) || isnan(v_in))
  {
    if (cls == 0 && lane == 0) poi->zncc = zncc_in >= 0 ? -3.f : zncc_in;
    return;
  }
  const PoiRef* R = P.poi_ref + (P.slot ? P.slot[i] : i);
  const float t0 = R->t0;
  const int size = (2 * rx + 1) * (2 * ry + 1);
  const float inv_size = 1.f / (float)size;
  const int cx = (int)px, cy = (int)py;
  float W[6] = {1.f + ux_in, uy_in, u_in, vx_in, 1.f + vy_in, v_in};
  const float rx2 = (float)(rx * rx), ry2 = (float)(ry * ry);
  int it = 0;
  float conv = 0.f, znssd = 0.f;
  int status = 0;
  do
  {
    ++it;
    float s[9];
    bool bad;
    // pixel sampling: on the lattice, or every sample inside the window (warp-uniform)
    bool fast = false, lat = false;
    if constexpr (kSrc == kSrcPixels)
    {
      lat = on_lattice(W, px, py);
      fast = !lat && window_covers(W, px, py, rx, ry, (float)(w - 2), (float)(h - 2), T, lane);
    }
    const auto class_sums = [&](int k, float(&out)[9]) {
      if constexpr (kSrc == kSrcPixels)
        return pair_class_sums_px(P, T, k, lane, px, py, cx, cy, t0, W, fast, lat, out);
      else
        return pair_class_sums(P, k, lane, px, py, cx, cy, t0, W, out);
    };
    if constexpr (kPoiWarps == 1)
    {
      float s1[9];
      bad = class_sums(0, s);
      bad = class_sums(1, s1) || bad;
#pragma unroll
      for (int j = 0; j < 9; ++j) s[j] = __fadd_rn(s[j], s1[j]);
    }
    else
    {
      float mine[9];
      const bool b = class_sums(cls, mine);
      float* slot = xch->sums[it & 1][cls];
      if (lane == 0)
      {
#pragma unroll
        for (int j = 0; j < 9; ++j) slot[j] = mine[j];
        slot[9] = b ? 1.f : 0.f;
      }
      pair_sync(bar);
      const float* s0 = xch->sums[it & 1][0];
      const float* s1 = xch->sums[it & 1][1];
#pragma unroll
      for (int j = 0; j < 9; ++j) s[j] = __fadd_rn(s0[j], s1[j]);
      bad = s0[9] != 0.f || s1[9] != 0.f;
    }
    if (bad)
    {
      // Rare path: the CPU's order (src/oc_icgn.cpp:266-301), out of range before NaN.
      bool oob;
      if constexpr (kPoiWarps == 1)
        oob = pair_class_oob(P, 0, lane, px, py, W) || pair_class_oob(P, 1, lane, px, py, W);
      else
      {
        const bool mo = pair_class_oob(P, cls, lane, px, py, W);
        if (lane == 0) xch->oob[cls] = mo ? 1 : 0;
        pair_sync(bar);
        oob = xch->oob[0] != 0 || xch->oob[1] != 0;
      }
      status = oob ? -3 : -5;
      break;
    }
    const float A0 = s[0], A1 = s[1], A2 = s[2];
    const float ref_norm = R->ref_norm, ref_norm_sq = R->ref_norm_sq, sum_rc = R->sum_rc;
    const float mean_tau = A0 * inv_size;
    const float tnorm_sq = fmaf(-A0, mean_tau, A1);
    const float tar_norm = tnorm_sq > 0.f ? sqrtf(tnorm_sq) : __int_as_float(0x7fc00000);
    const float sc = ref_norm / tar_norm;
    const float tc_rc = fmaf(-mean_tau, sum_rc, A2);
    const float esq = sc * sc * tnorm_sq - 2.f * sc * tc_rc + ref_norm_sq;
    znssd = esq / (ref_norm * ref_norm);
    const int row = lane < 6 ? lane : 0;
    const float S_l = R->S[row], G_l = R->G[row];
    float num_l = 0.f;
#pragma unroll
    for (int a = 0; a < 6; ++a)
      if (lane == a) num_l = sc * fmaf(-mean_tau, S_l, s[3 + a]) - G_l;
    float dp_l = 0.f;
#pragma unroll
    for (int c = 0; c < 6; ++c)
    {
      const float nc = __shfl_sync(kFull, num_l, c);
      dp_l += R->inv_h[row * 6 + c] * nc;
    }
    float dp[6];
#pragma unroll
    for (int a = 0; a < 6; ++a) dp[a] = __shfl_sync(kFull, dp_l, a);
    compose_update(W, dp);
    conv = sqrtf(dp[0] * dp[0] + dp[1] * dp[1] * rx2 + dp[2] * dp[2] * ry2 + dp[3] * dp[3] +
                 dp[4] * dp[4] * rx2 + dp[5] * dp[5] * ry2);
  } while ((float)it < P.max_iter && conv >= P.conv);

  if (cls != 0 || lane != 0) return;
  if (P.iter_sum) atomicAdd(P.iter_sum, (unsigned long long)it);
  if (status == -3) { poi->zncc = -3.f; return; }
  if (status == -5) { poi->zncc = -5.f; return; }
  float u = W[2], ux = W[0] - 1.f, uy = W[1], v = W[5], vx = W[3], vy = W[4] - 1.f;
  float zncc = 0.5f * (2.f - znssd);
  if (conv >= P.conv && (float)it >= P.max_iter) zncc = -4.f;
  const float u_init = poi->u, v_init = poi->v;
  if (isnan(zncc) || isnan(u) || isnan(v))
  {
    u = u_init;
    v = v_init;
    zncc = -5.f;
  }
  poi->u = u; poi->ux = ux; poi->uy = uy;
  poi->v = v; poi->vx = vx; poi->vy = vy;
  poi->u0 = u_init;
  poi->v0 = v_init;
  poi->zncc = zncc;
  poi->iteration = (float)it;
  poi->convergence = conv;
}

// Launch shapes of the pair walk: kWarps warps per CTA, kPoiWarps (1 or 2) per POI, 28
// resident warps per SM (72 registers: one warp walking both classes keeps the first
// class's nine totals live through the second).  The grid form takes POIs
// blockIdx.x * (kWarps / kPoiWarps) + slot; the persistent form
// draws them from an atomic counter (the pair's class-0 warp fetches, double-buffered by
// fetch parity, a named barrier per fetch).
template <int kPoiWarps, int kWarps>
__global__ void __launch_bounds__(kWarps * 32, icgn_min_blocks(kWarps)) k_icgn_pair(IcgnParams P)
{
  constexpr int kSlots = kWarps / kPoiWarps;
  __shared__ PairExchange xch[kSlots];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int slot = warp / kPoiWarps, cls = warp % kPoiWarps;
  const int64_t i = (int64_t)blockIdx.x * kSlots + slot;
  if (!queue_slot_active(P, i)) return;   // uniform over a pair
  icgn_solve_pair<kPoiWarps>(P, i, lane, cls, &xch[slot], 1 + slot);
}

template <int kPoiWarps, int kWarps>
__global__ void __launch_bounds__(kWarps * 32, icgn_min_blocks(kWarps))
    k_icgn_pair_persistent(IcgnParams P, unsigned long long* next)
{
  constexpr int kSlots = kWarps / kPoiWarps;
  __shared__ PairExchange xch[kSlots];
  __shared__ long long fetched[kSlots][2];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int slot = warp / kPoiWarps, cls = warp % kPoiWarps;
  if (P.enable && *P.enable == 0) return;
  for (unsigned f = 0;; ++f)
  {
    int64_t i;
    if constexpr (kPoiWarps == 1)
    {
      unsigned long long t = 0;
      if (lane == 0) t = atomicAdd(next, 1ull);
      i = (int64_t)__shfl_sync(kFull, t, 0);
    }
    else
    {
      if (cls == 0 && lane == 0) fetched[slot][f & 1] = (long long)atomicAdd(next, 1ull);
      pair_sync(1 + slot);
      i = (int64_t)fetched[slot][f & 1];
    }
    if (!queue_slot_active(P, i)) return;
    icgn_solve_pair<kPoiWarps>(P, i, lane, cls, &xch[slot], 1 + slot);
  }
}

// --------------------------------------------------------------------------------------
// mbarrier and TMA (cp.async.bulk.tensor) in inline PTX, sm_90 and later.
// --------------------------------------------------------------------------------------
__device__ __forceinline__ uint32_t smem_addr(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }
__device__ __forceinline__ void mbar_init(uint32_t bar, uint32_t count)
{
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(bar), "r"(count) : "memory");
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}
__device__ __forceinline__ void mbar_arrive_expect_tx(uint32_t bar, uint32_t bytes)
{
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar), "r"(bytes) : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(uint32_t bar, uint32_t parity)
{
  uint32_t done;
  asm volatile(
      "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}"
      : "=r"(done)
      : "r"(bar), "r"(parity)
      : "memory");
  return done != 0;
}
// a bounded wait: false when the phase did not complete within `limit` polls
__device__ __forceinline__ bool mbar_wait_bounded(uint32_t bar, uint32_t parity, uint32_t limit)
{
  for (uint32_t k = 0; k < limit; ++k)
    if (mbar_try_wait(bar, parity)) return true;
  return false;
}
// generic-proxy reads of shared memory ordered before a following async-proxy (TMA) write
__device__ __forceinline__ void fence_proxy_async_smem() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }
__device__ __forceinline__ void tma_load_4d(uint32_t dst, const CUtensorMap* map, int c0, int c1, int c2, int c3,
                                            uint32_t bar)
{
  asm volatile(
      "cp.async.bulk.tensor.4d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4, %5}], [%6];"
      ::"r"(dst), "l"(reinterpret_cast<uint64_t>(map)), "r"(c0), "r"(c1), "r"(c2), "r"(c3), "r"(bar)
      : "memory");
}

// --------------------------------------------------------------------------------------
// IC-GN with the target coefficient tile staged in shared memory by TMA (column walk).
// Persistent CTAs of kWarps warps take chunks of kWarps consecutive queue POIs (for a grid
// queue: neighbours along a row, whose warped subsets overlap by most of their width).  Per
// chunk, every warp bounds its POI's warped subset at the incoming warp (corners, plus
// kTileMargin texels for the updates to come), the CTA takes the union, and one thread
// loads that BX x BY texel block of both coefficient planes with one
// cp.async.bulk.tensor (4-D map {component 8, x, y, plane 2}; the innermost coordinate is always
// 0, other coordinates may be negative: out-of-range texels read as zero and are never
// sampled, the range test rejects them first).  Warps then solve their POIs reading texels
// from shared memory (global table outside the block, or for the whole chunk when the union
// does not fit).  The mbarrier wait is bounded; a timeout is decided for the whole CTA,
// flagged in `err`, and the CTA waits (bounded) for its copy before it leaves.
// --------------------------------------------------------------------------------------
constexpr int kTileMargin = 2;

// dynamic shared memory of one k_icgn_tile CTA: the block plus room to align it to 128 B
template <int BX, int BY>
constexpr size_t tile_smem_bytes() { return (size_t)4 * BX * BY * sizeof(float4) + 128; }

template <int kWarps, int BX, int BY>
__global__ void __launch_bounds__(kWarps * 32) k_icgn_tile(IcgnParams P, const __grid_constant__ CUtensorMap map,
                                                           unsigned long long* next, int* err)
{
  extern __shared__ unsigned char tile_raw[];
  // the TMA destination on a 128 B boundary
  unsigned char* tile_smem = tile_raw + ((128u - (smem_addr(tile_raw) & 127u)) & 127u);
  __shared__ __align__(8) unsigned long long bar;
  __shared__ int box[kWarps][4];
  __shared__ int org[3];
  __shared__ unsigned long long chunk;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  if (P.enable && *P.enable == 0) return;
  const uint32_t bar_a = smem_addr(&bar);
  if (threadIdx.x == 0) mbar_init(bar_a, 1);
  __syncthreads();
  uint32_t parity = 0;
  const int rx = P.rx, ry = P.ry;
  for (;;)
  {
    if (threadIdx.x == 0) chunk = atomicAdd(next, 1ull);
    __syncthreads();
    const int64_t first = (int64_t)chunk * kWarps;
    if (!queue_slot_active(P, first)) break;   // uniform: every thread read the same chunk
    const int64_t i = first + warp;
    const bool active = queue_slot_active(P, i);
    if (lane == 0)
    {
      int b[4] = {INT_MAX, INT_MAX, INT_MIN, INT_MIN};
      if (active)
      {
        const dic_poi* poi = P.pois + i;
        const float px = poi->x, py = poi->y, u = poi->u, v = poi->v;
        const float W0 = 1.f + poi->ux, W1 = poi->uy, W3 = poi->vx, W4 = 1.f + poi->vy;
        // only POIs the solver will sample (its entry test passes a non-negative incoming zncc)
        if (poi->zncc >= 0.f && isfinite(u) && isfinite(v) && isfinite(W0) && isfinite(W1) && isfinite(W3) &&
            isfinite(W4) && fabsf(u) < P.w && fabsf(v) < P.h)
        {
          float x0 = 3.4e38f, x1 = -3.4e38f, y0 = 3.4e38f, y1 = -3.4e38f;
#pragma unroll
          for (int k = 0; k < 4; ++k)
          {
            const float lx = (k & 1) ? (float)rx : (float)-rx, ly = (k & 2) ? (float)ry : (float)-ry;
            const float gx = px + (W0 * lx + W1 * ly + u), gy = py + (W3 * lx + W4 * ly + v);
            x0 = fminf(x0, gx); x1 = fmaxf(x1, gx);
            y0 = fminf(y0, gy); y1 = fmaxf(y1, gy);
          }
          b[0] = (int)floorf(x0) - kTileMargin;
          b[1] = (int)floorf(y0) - kTileMargin;
          b[2] = (int)floorf(x1) + kTileMargin;
          b[3] = (int)floorf(y1) + kTileMargin;
        }
      }
#pragma unroll
      for (int k = 0; k < 4; ++k) box[warp][k] = b[k];
    }
    __syncthreads();
    if (threadIdx.x == 0)
    {
      int u0 = INT_MAX, v0 = INT_MAX, u1 = INT_MIN, v1 = INT_MIN;
      for (int k = 0; k < kWarps; ++k)
      {
        u0 = min(u0, box[k][0]); v0 = min(v0, box[k][1]);
        u1 = max(u1, box[k][2]); v1 = max(v1, box[k][3]);
      }
      const bool fits = u0 <= u1 && (int64_t)u1 - u0 < BX && (int64_t)v1 - v0 < BY;
      org[0] = fits ? u0 : 0;
      org[1] = fits ? v0 : 0;
      org[2] = fits ? 1 : 0;
      if (fits)
      {
        fence_proxy_async_smem();   // the previous chunk's shared-memory reads come first
        mbar_arrive_expect_tx(bar_a, (uint32_t)(4 * BX * BY * sizeof(float4)));
        if (!P.wait_test) tma_load_4d(smem_addr(tile_smem), &map, 0, u0, v0, 0, bar_a);
      }
    }
    __syncthreads();
    CoefTile T;
    T.s = reinterpret_cast<const float4*>(tile_smem);
    T.bx = BX;
    T.by = BY;
    T.ox = org[0];
    T.oy = org[1];
    if (org[2])
    {
      const bool done = mbar_wait_bounded(bar_a, parity, P.wait_polls);
      parity ^= 1u;
      if (!__syncthreads_and(done))
      {
        if (threadIdx.x == 0) atomicOr(err, 1);
        mbar_wait_bounded(bar_a, parity ^ 1u, P.wait_polls);   // the copy in flight, once more
        return;
      }
    }
    else
      T.bx = 0;   // nothing staged: every texel from the global table
    if (active) icgn_solve<true, kSrcCoefTile>(P, i, lane, T);
    __syncthreads();   // every read of this block before the next copy overwrites it
  }
}

__device__ __forceinline__ void tma_load_2d(uint32_t dst, const CUtensorMap* map, int c0, int c1, uint32_t bar)
{
  asm volatile(
      "cp.async.bulk.tensor.2d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], [%4];"
      ::"r"(dst), "l"(reinterpret_cast<uint64_t>(map)), "r"(c0), "r"(c1), "r"(bar)
      : "memory");
}

// --------------------------------------------------------------------------------------
// IC-GN from target pixels staged per warp (column walk, pixel sampling).  Persistent CTAs;
// every warp takes the next POI from the atomic counter and works alone: it bounds the
// POI's warped subset at the incoming warp (corners, the 4 x 4 pixel support -1..+2, and
// kPxMargin pixels for the updates to come), and when that block fits its bx x by window
// it stages the block in its own shared memory -- one cp.async.bulk.tensor.2d issued by
// lane 0 (map {x, y} over the f32 target plane, box {bx, by}; the x origin is rounded
// down to a multiple of 4 pixels, TMA's 16-byte rule; pixels outside the image read as
// zero and are never sampled: the range test rejects their samples first), or, where the
// plane's row pitch is not a multiple of 16 bytes, a warp-wide copy.  The POI then
// iterates on shared memory: 16 pixel loads per sample, 4 B each, against the table's
// two 32-byte coefficient gathers from L2.  Samples whose support leaves the block (an
// update that walked further than the margin) read the global plane; both give the same
// bits.  A POI's window is ~6.7 KB at subset radius 15 and stays for all its iterations.
// The wait on the copy is bounded: a warp that times out sets bit 0 of `err`, waits
// (bounded) for the copy still in flight, and leaves.
// --------------------------------------------------------------------------------------
constexpr int kPxMargin = 1;
#ifndef DIC_PX_ROW_UNROLL
#define DIC_PX_ROW_UNROLL 1
#endif
constexpr int kPxRowUnroll = DIC_PX_ROW_UNROLL;   // rows of the pixel walk unrolled together

// window of one warp for a subset radius: the support of the subset with the margin and
// the x alignment slack, x rounded up to a multiple of 4 pixels
__host__ __device__ constexpr int px_window_x(int rx) { return ((2 * rx + 1 + 3 + 2 * kPxMargin + 1 + 3) + 3) & ~3; }
__host__ __device__ constexpr int px_window_y(int ry) { return 2 * ry + 1 + 3 + 2 * kPxMargin + 1; }
__host__ __device__ constexpr size_t px_window_bytes(int rx, int ry)
{
  return ((size_t)px_window_x(rx) * px_window_y(ry) * sizeof(float) + 127) & ~(size_t)127;
}

// Stages POI i's window for the calling warp (px_smem[win_f...], shared address win) and fills T.
// kMode 2: one TMA copy (map, the warp's mbarrier bar and its phase parity); 1: warp copies;
// 0: nothing staged (T.bx = 0, every sample from the global plane).  A compile-time mode keeps
// each kernel form to its own staging code (the copy loop's registers slowed the TMA form by
// 7 % when both were compiled into one kernel).  Returns false when the TMA copy did not
// arrive within P.wait_polls polls: bit 0 of err is set, lane 0 waits once more (bounded) for
// the copy in flight, and the caller leaves.
//
// kPoiWarps 2 (the two-warp pair walk): both warps of the POI bound the same window (from the
// same record) and share it; warp cls 0 issues the copy, both wait for it and agree through
// verdict[2] and the pair's barrier pair_bar whether it arrived; warp copies split the columns.
template <int kMode, int kPoiWarps = 1>
__device__ __forceinline__ bool px_stage(const IcgnParams& P, int64_t i, int lane, int win_f, uint32_t win,
                                         const CUtensorMap* map, uint32_t bar, uint32_t& parity, int* err,
                                         PixelTile& T, int cls = 0, int* verdict = nullptr, int pair_bar = 0)
{
  constexpr int mode = kMode;
  const int rx = P.rx, ry = P.ry, w = P.w, h = P.h;
  const int bx = px_window_x(rx), by = px_window_y(ry);
  int ox = 0, oy = 0, fits = 0;
  if (lane == 0 && mode != 0)
  {
    const dic_poi* poi = P.pois + i;
    const float px = poi->x, py = poi->y, u = poi->u, v = poi->v;
    const float W0 = 1.f + poi->ux, W1 = poi->uy, W3 = poi->vx, W4 = 1.f + poi->vy;
    // only POIs the solver will sample (the entry test passes a non-negative incoming zncc)
    if (poi->zncc >= 0.f && isfinite(u) && isfinite(v) && isfinite(W0) && isfinite(W1) && isfinite(W3) &&
        isfinite(W4) && fabsf(u) < w && fabsf(v) < h)
    {
      float x0 = 3.4e38f, x1 = -3.4e38f, y0 = 3.4e38f, y1 = -3.4e38f;
#pragma unroll
      for (int k = 0; k < 4; ++k)
      {
        const float lx = (k & 1) ? (float)rx : (float)-rx, ly = (k & 2) ? (float)ry : (float)-ry;
        const float gx = px + (W0 * lx + W1 * ly + u), gy = py + (W3 * lx + W4 * ly + v);
        x0 = fminf(x0, gx); x1 = fmaxf(x1, gx);
        y0 = fminf(y0, gy); y1 = fmaxf(y1, gy);
      }
      if (x0 > -1e6f && x1 < 1e6f && y0 > -1e6f && y1 < 1e6f)
      {
        const int ax = (int)floorf(x0) - 1 - kPxMargin, ay = (int)floorf(y0) - 1 - kPxMargin;
        const int ex = (int)floorf(x1) + 2 + kPxMargin, ey = (int)floorf(y1) + 2 + kPxMargin;
        ox = ax & ~3;   // floor to a multiple of 4 (two's complement)
        oy = ay;
        fits = ex - ox < bx && ey - oy < by;
      }
    }
    if (fits)
    {
      fence_proxy_async_smem();   // this warp's reads of the previous window come first
      if (mode == 2 && cls == 0)
      {
        mbar_arrive_expect_tx(bar, (uint32_t)(bx * by * sizeof(float)));
        if (!P.wait_test) tma_load_2d(win, map, ox, oy, bar);
      }
    }
  }
  ox = __shfl_sync(kFull, ox, 0);
  oy = __shfl_sync(kFull, oy, 0);
  fits = __shfl_sync(kFull, fits, 0);
  T.s = win_f;
  T.ox = ox;
  T.oy = oy;
  T.bx = 0;
  T.by = 0;
  if (!fits) return true;
  if (mode == 2)
  {
    const bool done = mbar_wait_bounded(bar, parity, P.wait_polls);
    parity ^= 1u;
    bool arrived = __all_sync(kFull, done);
    if constexpr (kPoiWarps == 2)
    {
      if (lane == 0) verdict[cls] = arrived ? 1 : 0;
      pair_sync(pair_bar);
      arrived = verdict[0] != 0 && verdict[1] != 0;
    }
    if (!arrived)
    {
      if (lane == 0 && cls == 0)
      {
        atomicOr(err, 1);
        mbar_wait_bounded(bar, parity ^ 1u, P.wait_polls);   // the copy in flight, once more
      }
      return false;
    }
  }
  else
  {
    // rows of the window by the whole warp, eight rows' loads in flight before their stores;
    // pixels outside the image as zero
    for (int c = lane + 32 * cls; c < bx; c += 32 * kPoiWarps)
    {
      const int gx = ox + c;
      const bool xin = gx >= 0 && gx < w;
      for (int r0 = 0; r0 < by; r0 += 8)
      {
        float v[8];
#pragma unroll
        for (int j = 0; j < 8; ++j)
        {
          const int gy = oy + r0 + j;
          v[j] = (xin && r0 + j < by && gy >= 0 && gy < h) ? __ldg(P.tar + ((size_t)gy * px_pitch(w) + gx)) : 0.f;
        }
#pragma unroll
        for (int j = 0; j < 8; ++j)
          if (r0 + j < by) px_smem[win_f + (r0 + j) * bx + c] = v[j];
      }
    }
    if constexpr (kPoiWarps == 2)
      pair_sync(pair_bar);
    else
      __syncwarp();
  }
  T.bx = bx;
  T.by = by;
  return true;
}

// the calling warp's window in the dynamic shared memory (128-byte aligned slots of win_bytes),
// as a float offset into px_smem and as a shared-window address
__device__ __forceinline__ int px_window(int warp, size_t win_bytes, uint32_t& addr)
{
  const uint32_t base = smem_addr(px_smem);
  const uint32_t off = ((128u - (base & 127u)) & 127u) + (uint32_t)(warp * win_bytes);
  addr = base + off;
  return (int)(off / sizeof(float));
}

// kMode: 2 windows staged by TMA, 1 staged by warp copies, 0 no windows (every sample from
// the global plane)
template <int kWarps, int kMode>
__global__ void __launch_bounds__(kWarps * 32, icgn_persistent_min_blocks(kWarps))
    k_icgn_px(IcgnParams P, const __grid_constant__ CUtensorMap map, unsigned long long* next, int* err)
{
  __shared__ __align__(8) unsigned long long bars[kWarps];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  if (P.enable && *P.enable == 0) return;
  uint32_t win = 0;
  const int win_f = px_window(warp, px_window_bytes(P.rx, P.ry), win);
  const uint32_t bar = smem_addr(&bars[warp]);
  if (lane == 0) mbar_init(bar, 1);
  __syncwarp();
  uint32_t parity = 0;
  for (;;)
  {
    unsigned long long t = 0;
    if (lane == 0) t = atomicAdd(next, 1ull);
    const int64_t i = (int64_t)__shfl_sync(kFull, t, 0);
    if (!queue_slot_active(P, i)) return;
    PixelTile T;
    if (!px_stage<kMode>(P, i, lane, win_f, win, &map, bar, parity, err, T)) return;
    icgn_solve<true, kSrcPixels, kPxRowUnroll, PixelTile>(P, i, lane, T);
    __syncwarp();   // every lane's reads of this window before the next copy overwrites it
  }
}

// The POI fetch of the persistent pair-walk kernels: with two warps per POI the pair's class-0
// warp takes the next index and shares it through `fetched` (double-buffered by fetch parity f,
// the pair's barrier bar), which also orders both warps' reads of the previous POI's window
// before the next copy.
template <int kPoiWarps>
__device__ __forceinline__ int64_t pair_fetch(unsigned long long* next, long long (&fetched)[2], unsigned f, int lane,
                                              int cls, int bar)
{
  if constexpr (kPoiWarps == 1)
  {
    unsigned long long t = 0;
    if (lane == 0) t = atomicAdd(next, 1ull);
    return (int64_t)__shfl_sync(kFull, t, 0);
  }
  else
  {
    if (cls == 0 && lane == 0) fetched[f & 1] = (long long)atomicAdd(next, 1ull);
    pair_sync(bar);
    return (int64_t)fetched[f & 1];
  }
}

// Pair walk (33 to 64 columns) under pixel sampling: k_icgn_pair_persistent's drain with
// k_icgn_px's staged windows, one window per POI (shared by the two warps of a two-warp POI).
// kMode as in k_icgn_px (2 TMA, 1 warp copies, 0 no windows).  Same bits for every kPoiWarps,
// kWarps and kMode.
template <int kPoiWarps, int kWarps, int kMode>
__global__ void __launch_bounds__(kWarps * 32, icgn_min_blocks(kWarps))
    k_icgn_pair_px(IcgnParams P, const __grid_constant__ CUtensorMap map, unsigned long long* next, int* err)
{
  constexpr int kSlots = kWarps / kPoiWarps;
  __shared__ PairExchange xch[kSlots];
  __shared__ long long fetched[kSlots][2];
  __shared__ __align__(8) unsigned long long bars[kSlots];
  __shared__ int verdict[kSlots][2];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int slot = warp / kPoiWarps, cls = warp % kPoiWarps;
  if (P.enable && *P.enable == 0) return;
  uint32_t win = 0, parity = 0;
  const int win_f = px_window(slot, px_window_bytes(P.rx, P.ry), win);
  const uint32_t bar = smem_addr(&bars[slot]);
  if (cls == 0 && lane == 0) mbar_init(bar, 1);
  __syncthreads();   // the barrier's initialisation before the pair's other warp waits on it
  for (unsigned f = 0;; ++f)
  {
    const int64_t i = pair_fetch<kPoiWarps>(next, fetched[slot], f, lane, cls, 1 + slot);
    if (!queue_slot_active(P, i)) return;   // uniform over a pair
    PixelTile T;
    if (!px_stage<kMode, kPoiWarps>(P, i, lane, win_f, win, &map, bar, parity, err, T, cls, verdict[slot], 1 + slot))
      return;
    icgn_solve_pair<kPoiWarps, kSrcPixels>(P, i, lane, cls, &xch[slot], 1 + slot, T);
    __syncwarp();
  }
}

// --------------------------------------------------------------------------------------
// Persistent multi-job IC-GN (uneven batches): every warp takes the next POI of the
// concatenated queue from an atomic counter, looks up its job (image pair, planes, subset
// radius) and solves it, so pairs of different sizes, radii and iteration counts share one
// launch and no warp idles on a short job.  Jobs are sorted by first POI; PoiRef records are
// concatenated in queue order.  Per-POI results do not depend on which warp takes the POI.
// --------------------------------------------------------------------------------------
struct BatchJob
{
  const float4* coef;
  const float* lattice;
  const float4* ref_pack;
  int64_t first;   // first queue index of the job
  int w, h, rx, ry;
  const float* tar = nullptr;          // target plane (pixel sampling), rows of px_pitch(w) floats
  const CUtensorMap* map = nullptr;    // its 2-D map in device memory for the window copies (null: warp copies)
};

template <bool kColumn, int kWarps = 4>
__global__ void __launch_bounds__(kWarps * 32, icgn_min_blocks(kWarps)) k_icgn_batch(const BatchJob* __restrict__ jobs, int njobs, dic_poi* pois,
                                                       const PoiRef* poi_ref, int64_t begin, int64_t end,
                                                       unsigned long long* next, float conv, float max_iter,
                                                       unsigned long long* iter_sum)
{
  const int lane = threadIdx.x & 31;
  for (;;)
  {
    unsigned long long t = 0;
    if (lane == 0) t = atomicAdd(next, 1ull);
    const int64_t k = begin + (int64_t)__shfl_sync(kFull, t, 0);
    if (k >= end) return;
    int j = 0, hi = njobs - 1;   // last job whose first index is <= k
    while (j < hi)
    {
      const int mid = (j + hi + 1) >> 1;
      if (jobs[mid].first <= k) j = mid;
      else hi = mid - 1;
    }
    const BatchJob& J = jobs[j];
    IcgnParams P;
    P.coef = J.coef;
    P.lattice = J.lattice;
    P.ref_pack = J.ref_pack;
    P.poi_ref = poi_ref;
    P.slot = nullptr;
    P.pois = pois;
    P.n = end;
    P.w = J.w;
    P.h = J.h;
    P.rx = J.rx;
    P.ry = J.ry;
    P.conv = conv;
    P.max_iter = max_iter;
    P.iter_sum = iter_sum;
    icgn_solve<kColumn, kSrcTable, 1>(P, k, lane);
  }
}

// Job lookup of the batch kernels: the last job whose first queue index is <= k.
__device__ __forceinline__ int batch_job_of(const BatchJob* __restrict__ jobs, int njobs, int64_t k)
{
  int j = 0, hi = njobs - 1;
  while (j < hi)
  {
    const int mid = (j + hi + 1) >> 1;
    if (jobs[mid].first <= k) j = mid;
    else hi = mid - 1;
  }
  return j;
}

// Uneven batches under pixel sampling (column-walk jobs): the persistent multi-job drain of
// k_icgn_batch with k_icgn_px's per-warp windows.  Each job's plane has its own tensor map in
// device memory (BatchJob::map, encoded by the host before the launch), so the windows are
// TMA copies as in k_icgn_px; a job without one (row pitch not a multiple of 16 bytes) is
// staged by warp copies.  win_bytes is the window slot of the largest radius in the launch.
// Same bits as each job's single-pair pixel solve.  The copy wait is bounded as in k_icgn_px.
// kMode 2: every job has a map (TMA windows); 1: warp copies for all.  32 resident warps per
// SM (64 registers, no spills), as k_icgn_px.
template <int kWarps, int kMode>
__global__ void __launch_bounds__(kWarps * 32, icgn_persistent_min_blocks(kWarps))
    k_icgn_batch_px(const BatchJob* __restrict__ jobs, int njobs, dic_poi* pois, const PoiRef* poi_ref, int64_t begin,
                    int64_t end, unsigned long long* next, float conv, float max_iter, unsigned long long* iter_sum,
                    uint32_t win_bytes, uint32_t wait_polls, int* err)
{
  __shared__ __align__(8) unsigned long long bars[kWarps];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  uint32_t win = 0, parity = 0;
  const int win_f = px_window(warp, win_bytes, win);
  const uint32_t bar = smem_addr(&bars[warp]);
  if (lane == 0) mbar_init(bar, 1);
  __syncwarp();
  for (;;)
  {
    unsigned long long t = 0;
    if (lane == 0) t = atomicAdd(next, 1ull);
    const int64_t k = begin + (int64_t)__shfl_sync(kFull, t, 0);
    if (k >= end) return;
    const BatchJob& J = jobs[batch_job_of(jobs, njobs, k)];
    IcgnParams P;
    P.coef = nullptr;
    P.tar = J.tar;
    P.ref_pack = J.ref_pack;
    P.poi_ref = poi_ref;
    P.slot = nullptr;
    P.pois = pois;
    P.n = end;
    P.w = J.w;
    P.h = J.h;
    P.rx = J.rx;
    P.ry = J.ry;
    P.conv = conv;
    P.max_iter = max_iter;
    P.iter_sum = iter_sum;
    P.wait_polls = wait_polls;
    PixelTile T;
    if (!px_stage<kMode>(P, k, lane, win_f, win, J.map, bar, parity, err, T)) return;
    icgn_solve<true, kSrcPixels, 1, PixelTile>(P, k, lane, T);
    __syncwarp();
  }
}

// The persistent multi-job launch for the jobs whose subsets take the pair walk (33 to 64
// columns), one or two warps per POI (see k_icgn_pair_persistent).
template <int kPoiWarps, int kWarps>
__global__ void __launch_bounds__(kWarps * 32, icgn_min_blocks(kWarps))
    k_icgn_batch_pair(const BatchJob* __restrict__ jobs, int njobs, dic_poi* pois, const PoiRef* poi_ref,
                      int64_t begin, int64_t end, unsigned long long* next, float conv, float max_iter,
                      unsigned long long* iter_sum)
{
  constexpr int kSlots = kWarps / kPoiWarps;
  __shared__ PairExchange xch[kSlots];
  __shared__ long long fetched[kSlots][2];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int slot = warp / kPoiWarps, cls = warp % kPoiWarps;
  for (unsigned f = 0;; ++f)
  {
    int64_t k;
    if constexpr (kPoiWarps == 1)
    {
      unsigned long long t = 0;
      if (lane == 0) t = atomicAdd(next, 1ull);
      k = begin + (int64_t)__shfl_sync(kFull, t, 0);
    }
    else
    {
      if (cls == 0 && lane == 0) fetched[slot][f & 1] = (long long)atomicAdd(next, 1ull);
      pair_sync(1 + slot);
      k = begin + (int64_t)fetched[slot][f & 1];
    }
    if (k >= end) return;
    const BatchJob& J = jobs[batch_job_of(jobs, njobs, k)];
    IcgnParams P;
    P.coef = J.coef;
    P.lattice = J.lattice;
    P.ref_pack = J.ref_pack;
    P.poi_ref = poi_ref;
    P.slot = nullptr;
    P.pois = pois;
    P.n = end;
    P.w = J.w;
    P.h = J.h;
    P.rx = J.rx;
    P.ry = J.ry;
    P.conv = conv;
    P.max_iter = max_iter;
    P.iter_sum = iter_sum;
    icgn_solve_pair<kPoiWarps>(P, k, lane, cls, &xch[slot], 1 + slot);
  }
}

// The batch's pair-walk jobs under pixel sampling: k_icgn_batch_pair's drain with
// k_icgn_pair_px's windows (each job's map in device memory, win_bytes the window of the
// launch's largest radius).  kMode 2: TMA windows (every job has a map), 0: no windows.
template <int kPoiWarps, int kWarps, int kMode>
__global__ void __launch_bounds__(kWarps * 32, icgn_min_blocks(kWarps))
    k_icgn_batch_pair_px(const BatchJob* __restrict__ jobs, int njobs, dic_poi* pois, const PoiRef* poi_ref,
                         int64_t begin, int64_t end, unsigned long long* next, float conv, float max_iter,
                         unsigned long long* iter_sum, uint32_t win_bytes, uint32_t wait_polls, int* err)
{
  constexpr int kSlots = kWarps / kPoiWarps;
  __shared__ PairExchange xch[kSlots];
  __shared__ long long fetched[kSlots][2];
  __shared__ __align__(8) unsigned long long bars[kSlots];
  __shared__ int verdict[kSlots][2];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int slot = warp / kPoiWarps, cls = warp % kPoiWarps;
  uint32_t win = 0, parity = 0;
  const int win_f = px_window(slot, win_bytes, win);
  const uint32_t bar = smem_addr(&bars[slot]);
  if (cls == 0 && lane == 0) mbar_init(bar, 1);
  __syncthreads();
  for (unsigned f = 0;; ++f)
  {
    const int64_t k = begin + pair_fetch<kPoiWarps>(next, fetched[slot], f, lane, cls, 1 + slot);
    if (k >= end) return;
    const BatchJob& J = jobs[batch_job_of(jobs, njobs, k)];
    IcgnParams P;
    P.coef = nullptr;
    P.tar = J.tar;
    P.ref_pack = J.ref_pack;
    P.poi_ref = poi_ref;
    P.slot = nullptr;
    P.pois = pois;
    P.n = end;
    P.w = J.w;
    P.h = J.h;
    P.rx = J.rx;
    P.ry = J.ry;
    P.conv = conv;
    P.max_iter = max_iter;
    P.iter_sum = iter_sum;
    P.wait_polls = wait_polls;
    PixelTile T;
    if (!px_stage<kMode, kPoiWarps>(P, k, lane, win_f, win, J.map, bar, parity, err, T, cls, verdict[slot], 1 + slot))
      return;
    icgn_solve_pair<kPoiWarps, kSrcPixels>(P, k, lane, cls, &xch[slot], 1 + slot, T);
    __syncwarp();
  }
}

// --------------------------------------------------------------------------------------
// Register FFT of compile-time length N (mixed radix 2/3/4/5 + generic primes), one
// transform per thread.  Four-step decomposition N = N1*N2 with n = N2*n1 + n2,
// k = k1 + N1*k2.  After full unrolling every twiddle index is a constant, so twiddles are
// read straight from the constant bank.
// --------------------------------------------------------------------------------------
// Complex add / subtract / real scale as packed FP32 pairs (add/sub/mul.rn.f32x2, sm_100 and
// later; each half rounded as the scalar operation): the FFTCC line transforms issue half the
// instructions for their butterflies (k_fftcc2<30> 0.756 -> 0.674 ms on the 2048x2048 pair).
__device__ __forceinline__ float2 cadd(float2 a, float2 b) { return __fadd2_rn(a, b); }
__device__ __forceinline__ float2 csub(float2 a, float2 b)
{
  unsigned long long ra, rb, rd;
  memcpy(&ra, &a, 8);
  memcpy(&rb, &b, 8);
  asm("sub.rn.f32x2 %0, %1, %2;" : "=l"(rd) : "l"(ra), "l"(rb));
  float2 d;
  memcpy(&d, &rd, 8);
  return d;
}
__device__ __forceinline__ float2 cscale(float2 a, float s) { return __fmul2_rn(a, make_float2(s, s)); }
__device__ __forceinline__ float2 cmul(float2 a, float2 b)
{ return make_float2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x); }
__device__ __forceinline__ float2 mul_mi(float2 a) { return make_float2(a.y, -a.x); }  // -i * a

__host__ __device__ constexpr bool is_prime(int n)
{
  if (n < 2) return false;
  for (int d = 2; d * d <= n; ++d)
    if (n % d == 0) return false;
  return true;
}
__host__ __device__ constexpr int first_factor(int n)
{
  if (n <= 5 || is_prime(n)) return n;
  if (n % 4 == 0) return 4;
  if (n % 2 == 0) return 2;
  if (n % 3 == 0) return 3;
  if (n % 5 == 0) return 5;
  for (int d = 7; d <= n; d += 2)
    if (n % d == 0) return d;
  return n;
}

template <int N>
__device__ __forceinline__ float2 twiddle_mul(float2 v, int e)
{
  const int r = e % N;
  if (r == 0) return v;
  return cmul(v, c_tw[tw_offset(N) + r]);
}

template <int N>
struct Dft
{
  // generic prime length: direct DFT with table twiddles
  __device__ __forceinline__ static void run(const float2 (&in)[N], float2 (&out)[N])
  {
#pragma unroll
    for (int k = 0; k < N; ++k)
    {
      float2 acc = in[0];
#pragma unroll
      for (int j = 1; j < N; ++j) acc = cadd(acc, twiddle_mul<N>(in[j], j * k));
      out[k] = acc;
    }
  }
};
template <>
struct Dft<1>
{
  __device__ __forceinline__ static void run(const float2 (&in)[1], float2 (&out)[1]) { out[0] = in[0]; }
};
template <>
struct Dft<2>
{
  __device__ __forceinline__ static void run(const float2 (&in)[2], float2 (&out)[2])
  {
    out[0] = cadd(in[0], in[1]);
    out[1] = csub(in[0], in[1]);
  }
};
template <>
struct Dft<3>
{
  __device__ __forceinline__ static void run(const float2 (&in)[3], float2 (&out)[3])
  {
    const float k = 0.86602540378443864676f;  // sin(2 pi / 3)
    const float2 s = cadd(in[1], in[2]), d = csub(in[1], in[2]);
    const float2 m = make_float2(in[0].x - 0.5f * s.x, in[0].y - 0.5f * s.y);
    const float2 rot = mul_mi(cscale(d, k));
    out[0] = cadd(in[0], s);
    out[1] = cadd(m, rot);
    out[2] = csub(m, rot);
  }
};
template <>
struct Dft<4>
{
  __device__ __forceinline__ static void run(const float2 (&in)[4], float2 (&out)[4])
  {
    const float2 a = cadd(in[0], in[2]), b = csub(in[0], in[2]);
    const float2 c = cadd(in[1], in[3]), d = mul_mi(csub(in[1], in[3]));
    out[0] = cadd(a, c);
    out[2] = csub(a, c);
    out[1] = cadd(b, d);
    out[3] = csub(b, d);
  }
};
template <>
struct Dft<5>
{
  __device__ __forceinline__ static void run(const float2 (&in)[5], float2 (&out)[5])
  {
    const float c1 = 0.30901699437494742410f;   // cos(2 pi / 5)
    const float c2 = -0.80901699437494742410f;  // cos(4 pi / 5)
    const float s1 = 0.95105651629515357212f;   // sin(2 pi / 5)
    const float s2 = 0.58778525229247312917f;   // sin(4 pi / 5)
    const float2 a1 = cadd(in[1], in[4]), b1 = csub(in[1], in[4]);
    const float2 a2 = cadd(in[2], in[3]), b2 = csub(in[2], in[3]);
    out[0] = cadd(in[0], cadd(a1, a2));
    const float2 m1 = make_float2(in[0].x + c1 * a1.x + c2 * a2.x, in[0].y + c1 * a1.y + c2 * a2.y);
    const float2 m2 = make_float2(in[0].x + c2 * a1.x + c1 * a2.x, in[0].y + c2 * a1.y + c1 * a2.y);
    const float2 r1 = mul_mi(make_float2(s1 * b1.x + s2 * b2.x, s1 * b1.y + s2 * b2.y));
    const float2 r2 = mul_mi(make_float2(s2 * b1.x - s1 * b2.x, s2 * b1.y - s1 * b2.y));
    out[1] = cadd(m1, r1);
    out[4] = csub(m1, r1);
    out[2] = cadd(m2, r2);
    out[3] = csub(m2, r2);
  }
};

template <int N, int N1 = first_factor(N)>
struct Fft
{
  static constexpr int N2 = N / N1;
  __device__ __forceinline__ static void run(const float2 (&in)[N], float2 (&out)[N])
  {
    float2 y[N];
#pragma unroll
    for (int n2 = 0; n2 < N2; ++n2)
    {
      float2 a[N1], b[N1];
#pragma unroll
      for (int n1 = 0; n1 < N1; ++n1) a[n1] = in[N2 * n1 + n2];
      Fft<N1>::run(a, b);
#pragma unroll
      for (int k1 = 0; k1 < N1; ++k1) y[k1 * N2 + n2] = twiddle_mul<N>(b[k1], n2 * k1);
    }
#pragma unroll
    for (int k1 = 0; k1 < N1; ++k1)
    {
      float2 a[N2], b[N2];
#pragma unroll
      for (int n2 = 0; n2 < N2; ++n2) a[n2] = y[k1 * N2 + n2];
      Fft<N2>::run(a, b);
#pragma unroll
      for (int k2 = 0; k2 < N2; ++k2) out[k1 + N1 * k2] = b[k2];
    }
  }
};
template <int N>
struct Fft<N, N>
{
  __device__ __forceinline__ static void run(const float2 (&in)[N], float2 (&out)[N]) { Dft<N>::run(in, out); }
};

// Prime-factor (Good-Thomas) transform: N = N1 * N2 with gcd(N1, N2) = 1, N1 the full power
// of N's smallest prime.  Input n = (N2 n1 + N1 n2) mod N and output k with k = k1 (mod N1),
// k = k2 (mod N2) make W_N^(nk) = W_N1^(n1 k1) W_N2^(n2 k2), so the N-point DFT is an
// N1 x N2 two-dimensional DFT with no twiddle multiplications between the stages (30 =
// 2 x 3 x 5: none at all, against 30 complex products for the Cooley-Tukey split).
// Prime powers fall back to Fft (Cooley-Tukey).
__host__ __device__ constexpr int prime_power_part(int n)
{
  const int p = first_factor(n) == 4 ? 2 : first_factor(n);
  int q = 1;
  while (n % p == 0)
  {
    n /= p;
    q *= p;
  }
  return q;
}
__host__ __device__ constexpr int inverse_mod(int a, int m)
{
  for (int x = 1; x < m; ++x)
    if ((a * x) % m == 1) return x;
  return 1;
}

template <int N, int N1 = prime_power_part(N)>
struct FftPfa
{
  static constexpr int N2 = N / N1;
  static constexpr int E1 = N2 * inverse_mod(N2 % N1, N1);   // = 1 mod N1, 0 mod N2
  static constexpr int E2 = N1 * inverse_mod(N1 % N2, N2);   // = 0 mod N1, 1 mod N2
  __device__ __forceinline__ static void run(const float2 (&in)[N], float2 (&out)[N])
  {
    float2 y[N];
#pragma unroll
    for (int n2 = 0; n2 < N2; ++n2)
    {
      float2 a[N1], b[N1];
#pragma unroll
      for (int n1 = 0; n1 < N1; ++n1) a[n1] = in[(N2 * n1 + N1 * n2) % N];
      Fft<N1>::run(a, b);
#pragma unroll
      for (int k1 = 0; k1 < N1; ++k1) y[k1 * N2 + n2] = b[k1];
    }
#pragma unroll
    for (int k1 = 0; k1 < N1; ++k1)
    {
      float2 a[N2], b[N2];
#pragma unroll
      for (int n2 = 0; n2 < N2; ++n2) a[n2] = y[k1 * N2 + n2];
      FftPfa<N2>::run(a, b);
#pragma unroll
      for (int k2 = 0; k2 < N2; ++k2) out[(k1 * E1 + k2 * E2) % N] = b[k2];
    }
  }
};
template <int N>
struct FftPfa<N, N>
{
  __device__ __forceinline__ static void run(const float2 (&in)[N], float2 (&out)[N]) { Fft<N>::run(in, out); }
};

// --------------------------------------------------------------------------------------
// FFTCC (src/oc_fftcc.cpp:396-496), one warp per POI, M = 2r <= 32.
// The zero-mean reference and target subsets are packed as z = ref + i*tar and
// transformed once (rows then columns, one lane per line).  With Z[-k] read back from
// shared memory, R = (Z[k] + conj Z[-k]) / 2 and T = (Z[k] - conj Z[-k]) / 2i are the two
// real-input spectra, X = conj(R) * T is the cross-power spectrum FFTW's r2c/c2r pair
// produces, and the inverse transform (columns then rows) gives the unnormalised
// correlation map.  Argmax: strict '>' from index 0, i.e. the largest value and, among
// equal values, the lowest row-major index, reduced as (value, index) pairs.
// --------------------------------------------------------------------------------------
struct FftccParams
{
  const float* ref;
  const float* tar;
  dic_poi* pois;
  int64_t n;
  int w, h;
  const int64_t* n_dev = nullptr;   // device-side queue length (overrides n when set)
  const int* enable = nullptr;      // device-side switch: the launch does nothing when 0
};

template <int M>
__global__ void __launch_bounds__(128) k_fftcc(FftccParams P)
{
  constexpr int R = M / 2;
  constexpr int S = (M % 2 == 0) ? M + 1 : M;  // odd row stride: conflict-free float2 rows
  constexpr int kWarpsPerBlock = 4;
  __shared__ float2 smem[kWarpsPerBlock][M * S];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int64_t i = (int64_t)blockIdx.x * kWarpsPerBlock + warp;
  if (!queue_slot_active(P, i)) return;
  float2* z = smem[warp];
  dic_poi* poi = P.pois + i;
  const float px = poi->x, py = poi->y, u_init = poi->u, v_init = poi->v;
  const int w = P.w, h = P.h;
  if ((int)px < R || (int)px >= w - R || (int)py < R || (int)py >= h - R ||
      int(px + u_init) < R || int(px + u_init) >= w - R || int(py + v_init) < R ||
      int(py + v_init) >= h - R)
    return;  // untouched, as the CPU leaves it
  // subsets: lane c < M reads column c of every row (coordinates as the CPU forms them)
  float rv[M], tv[M];
  float rsum = 0.f, tsum = 0.f;
  if (lane < M)
  {
    const float fxr = __fsub_rn(__fadd_rn(px, (float)lane), (float)R);
    const int xr = (int)fxr, xt = (int)__fadd_rn(fxr, u_init);
#pragma unroll
    for (int r = 0; r < M; ++r)
    {
      const float fyr = __fsub_rn(__fadd_rn(py, (float)r), (float)R);
      const int yr = (int)fyr, yt = (int)__fadd_rn(fyr, v_init);
      rv[r] = P.ref[(size_t)yr * w + xr];
      tv[r] = P.tar[(size_t)yt * w + xt];
      rsum += rv[r];
      tsum += tv[r];
    }
  }
  rsum = warp_sum(rsum);
  tsum = warp_sum(tsum);
  const float rmean = rsum / (float)(M * M), tmean = tsum / (float)(M * M);
  float rn = 0.f, tn = 0.f;
  if (lane < M)
  {
#pragma unroll
    for (int r = 0; r < M; ++r)
    {
      rv[r] -= rmean;
      tv[r] -= tmean;
      rn += rv[r] * rv[r];
      tn += tv[r] * tv[r];
      z[r * S + lane] = make_float2(rv[r], tv[r]);
    }
  }
  rn = warp_sum(rn);
  tn = warp_sum(tn);
  __syncwarp();
  float2 a[M], b[M];
  // forward rows
  if (lane < M)
  {
#pragma unroll
    for (int k = 0; k < M; ++k) a[k] = z[lane * S + k];
    Fft<M>::run(a, b);
#pragma unroll
    for (int k = 0; k < M; ++k) z[lane * S + k] = b[k];
  }
  __syncwarp();
  // forward columns; keep column `lane` of Z in b[]
  if (lane < M)
  {
#pragma unroll
    for (int k = 0; k < M; ++k) a[k] = z[k * S + lane];
    Fft<M>::run(a, b);
  }
  __syncwarp();
  if (lane < M)
  {
#pragma unroll
    for (int k = 0; k < M; ++k) z[k * S + lane] = b[k];
  }
  __syncwarp();
  // cross-power spectrum, conjugated for the inverse transform: conj(X)
  if (lane < M)
  {
    const int cm = (M - lane) % M;
#pragma unroll
    for (int k = 0; k < M; ++k)
    {
      const float2 A = b[k];
      const float2 zm = z[((M - k) % M) * S + cm];
      const float2 B = make_float2(zm.x, -zm.y);
      const float2 Rk = make_float2(0.5f * (A.x + B.x), 0.5f * (A.y + B.y));
      const float2 D = csub(A, B);
      const float2 Tk = make_float2(0.5f * D.y, -0.5f * D.x);  // D / (2i)
      const float2 X = make_float2(Rk.x * Tk.x + Rk.y * Tk.y, Rk.x * Tk.y - Rk.y * Tk.x);
      a[k] = make_float2(X.x, -X.y);  // inverse via conj(FFT(conj(X)))
    }
    Fft<M>::run(a, b);
  }
  __syncwarp();
  if (lane < M)
  {
#pragma unroll
    for (int k = 0; k < M; ++k) z[k * S + lane] = b[k];
  }
  __syncwarp();
  float best = -2.f;
  int best_idx = 0;
  if (lane < M)
  {
#pragma unroll
    for (int k = 0; k < M; ++k) a[k] = z[lane * S + k];
    Fft<M>::run(a, b);
    // real part of conj(FFT(conj(.))) is the real part of the FFT output
#pragma unroll
    for (int k = 0; k < M; ++k)
      if (b[k].x > best) { best = b[k].x; best_idx = lane * M + k; }
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1)
  {
    const float ov = __shfl_xor_sync(kFull, best, o);
    const int oi = __shfl_xor_sync(kFull, best_idx, o);
    if (ov > best || (ov == best && oi < best_idx)) { best = ov; best_idx = oi; }
  }
  if (lane == 0)
  {
    int lu = best_idx % M, lv = best_idx / M;
    if (lu > R) lu -= M;
    if (lv > R) lv -= M;
    poi->u = (float)lu + u_init;
    poi->v = (float)lv + v_init;
    poi->u0 = u_init;
    poi->v0 = v_init;
    poi->zncc = best / (sqrtf(rn * tn) * (float)(M * M));
  }
}

// --------------------------------------------------------------------------------------
// FFTCC for M <= 30 with two POIs per warp and the Hermitian half of the inverse.
// The correlation is real, so its spectrum X is Hermitian: after the forward transform only
// the columns 0..M/2 of conj(X) need the inverse column pass (the others are conjugate
// mirrors), and the inverse row pass pairs rows (ra, rb) into one complex transform whose
// real and imaginary parts are the two real output rows.  A warp owns two POIs: the
// forward passes run once per POI (lane = line; the column transform straight from the
// loaded registers, so the raw subset never goes through shared memory), the inverse
// passes once for both (lanes 0-15 POI 0, 16-31 POI 1), i.e. 3 line passes per POI instead
// of 4; each line transform is the prime-factor form (FftPfa).  Same packing, algebra, tie
// rule and outputs as k_fftcc (the results differ only in float rounding: columns are
// transformed before rows, and without twiddles between coprime stages).
// --------------------------------------------------------------------------------------
#ifndef DIC_FFTCC_INT_ROWS
#define DIC_FFTCC_INT_ROWS 1
#endif
constexpr bool kFftccIntRows = DIC_FFTCC_INT_ROWS != 0;
template <int M>
// (Register caps for 7 or 8 CTAs per SM spill: 0.93 against 0.67 ms at 2048^2.)
__global__ void __launch_bounds__(64) k_fftcc2(FftccParams P)
{
  static_assert(M % 2 == 0 && M / 2 + 1 <= 16, "16 inverse lanes per POI");
  constexpr int R = M / 2, S = M + 1;
  constexpr int kWarps = 2;
  __shared__ float2 smem[kWarps * 2][M * S];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int64_t i0 = ((int64_t)blockIdx.x * kWarps + warp) * 2;
  const int w = P.w, h = P.h;
  // per-POI scalars of the two POIs, kept as named registers (the POI loop is not unrolled,
  // which keeps one copy of the forward transforms in the instruction stream)
  bool live0 = false, live1 = false;
  float rn0 = 0.f, rn1 = 0.f, tn0 = 0.f, tn1 = 0.f, uq0 = 0.f, uq1 = 0.f, vq0 = 0.f, vq1 = 0.f;
  float2 a[M], b[M];
  // per POI: load (lane = subset column), zero-mean, forward column transform from the
  // registers, store; then the forward row transform (lane = row) in place
#pragma unroll 1
  for (int q = 0; q < 2; ++q)
  {
    const int64_t i = i0 + q;
    bool lv = queue_slot_active(P, i);
    float ui = 0.f, vi = 0.f, px = 0.f, py = 0.f;
    if (lv)
    {
      const dic_poi* poi = P.pois + i;
      px = poi->x;
      py = poi->y;
      ui = poi->u;
      vi = poi->v;
      // out-of-range POIs are left untouched, as the CPU leaves them
      lv = !((int)px < R || (int)px >= w - R || (int)py < R || (int)py >= h - R || int(px + ui) < R ||
             int(px + ui) >= w - R || int(py + vi) < R || int(py + vi) >= h - R);
    }
    if (q == 0) { live0 = lv; uq0 = ui; vq0 = vi; }
    else { live1 = lv; uq1 = ui; vq1 = vi; }
    if (!lv) continue;
    float2* z = smem[warp * 2 + q];
    float rv[M], tv[M];
    float rsum = 0.f, tsum = 0.f;
    if (lane < M)
    {
      const float fxr = __fsub_rn(__fadd_rn(px, (float)lane), (float)R);
      const int xr = (int)fxr, xt = (int)__fadd_rn(fxr, ui);
      if (kFftccIntRows && py == rintf(py) && vi == rintf(vi))
      {
        // whole-pixel row coordinate and seed (every grid queue): the CPU's float row
        // coordinates py + r - R and + v are exact, so the rows are consecutive pointers
        const float* rp = P.ref + (size_t)((int)py - R) * w + xr;
        const float* tp = P.tar + (size_t)((int)py - R + (int)vi) * w + xt;
#pragma unroll
        for (int r = 0; r < M; ++r)
        {
          rv[r] = rp[(size_t)r * w];
          tv[r] = tp[(size_t)r * w];
          rsum += rv[r];
          tsum += tv[r];
        }
      }
      else
#pragma unroll
        for (int r = 0; r < M; ++r)
        {
          const float fyr = __fsub_rn(__fadd_rn(py, (float)r), (float)R);
          const int yr = (int)fyr, yt = (int)__fadd_rn(fyr, vi);
          rv[r] = P.ref[(size_t)yr * w + xr];
          tv[r] = P.tar[(size_t)yt * w + xt];
          rsum += rv[r];
          tsum += tv[r];
        }
    }
    rsum = warp_sum(rsum);
    tsum = warp_sum(tsum);
    const float rmean = rsum / (float)(M * M), tmean = tsum / (float)(M * M);
    float rnl = 0.f, tnl = 0.f;
    if (lane < M)
    {
#pragma unroll
      for (int r = 0; r < M; ++r)
      {
        rv[r] -= rmean;
        tv[r] -= tmean;
        rnl += rv[r] * rv[r];
        tnl += tv[r] * tv[r];
        a[r] = make_float2(rv[r], tv[r]);
      }
      FftPfa<M>::run(a, b);
#pragma unroll
      for (int k = 0; k < M; ++k) z[k * S + lane] = b[k];
    }
    const float rnq = warp_sum(rnl), tnq = warp_sum(tnl);
    if (q == 0) { rn0 = rnq; tn0 = tnq; }
    else { rn1 = rnq; tn1 = tnq; }
    __syncwarp();
    if (lane < M)
    {
#pragma unroll
      for (int k = 0; k < M; ++k) a[k] = z[lane * S + k];
      FftPfa<M>::run(a, b);
#pragma unroll
      for (int k = 0; k < M; ++k) z[lane * S + k] = b[k];
    }
    __syncwarp();
  }
  // inverse columns c = 0..R of conj(X), X = conj(R) T, both POIs at once: lane -> (POI, c)
  const int q = lane >> 4, c = lane & 15;
  float2* zq = smem[warp * 2 + q];
  const bool live_q = q ? live1 : live0;
  const bool col_live = live_q && c <= R;
  if (col_live)
  {
    const int cm = (M - c) % M;
#pragma unroll
    for (int k = 0; k < M; ++k)
    {
      const float2 A = zq[k * S + c];
      const float2 zm = zq[((M - k) % M) * S + cm];
      const float2 B = make_float2(zm.x, -zm.y);
      const float2 Rk = make_float2(0.5f * (A.x + B.x), 0.5f * (A.y + B.y));
      const float2 D = csub(A, B);
      const float2 Tk = make_float2(0.5f * D.y, -0.5f * D.x);  // D / (2i)
      const float2 X = make_float2(Rk.x * Tk.x + Rk.y * Tk.y, Rk.x * Tk.y - Rk.y * Tk.x);
      a[k] = make_float2(X.x, -X.y);
    }
    FftPfa<M>::run(a, b);
  }
  __syncwarp();   // every partner column is read before any column is overwritten
  if (col_live)
  {
#pragma unroll
    for (int k = 0; k < M; ++k) zq[k * S + c] = b[k];
  }
  __syncwarp();
  // inverse rows, rows j and j + R of POI q in one transform (with the odd stride S the 16
  // lanes' rows fall in distinct banks); columns past R are the conjugate mirrors of 1..R-1
  const int j = c;
  const bool row_live = live_q && j < R;
  float best = -2.f;
  int best_idx = 0;
  if (row_live)
  {
    const int ra = j, rb = j + R;
#pragma unroll
    for (int col = 0; col < M; ++col)
    {
      float2 va, vb;
      if (col <= R)
      {
        va = zq[ra * S + col];
        vb = zq[rb * S + col];
      }
      else
      {
        const float2 ma = zq[ra * S + (M - col)], mb = zq[rb * S + (M - col)];
        va = make_float2(ma.x, -ma.y);
        vb = make_float2(mb.x, -mb.y);
      }
      a[col] = make_float2(va.x - vb.y, va.y + vb.x);   // va + i vb
    }
    FftPfa<M>::run(a, b);
    // real part: row ra, imaginary part: row rb (ra first: lower row-major indices)
#pragma unroll
    for (int k = 0; k < M; ++k)
      if (b[k].x > best) { best = b[k].x; best_idx = ra * M + k; }
#pragma unroll
    for (int k = 0; k < M; ++k)
      if (b[k].y > best) { best = b[k].y; best_idx = rb * M + k; }
  }
  // argmax over the 16 lanes of each POI (largest value, then lowest index)
#pragma unroll
  for (int o = 8; o > 0; o >>= 1)
  {
    const float ov = __shfl_xor_sync(kFull, best, o);
    const int oi = __shfl_xor_sync(kFull, best_idx, o);
    if (ov > best || (ov == best && oi < best_idx)) { best = ov; best_idx = oi; }
  }
  if (c == 0 && live_q)
  {
    const float uq = q ? uq1 : uq0, vq = q ? vq1 : vq0;
    const float nq = q ? rn1 * tn1 : rn0 * tn0;
    dic_poi* poi = P.pois + i0 + q;
    int lu = best_idx % M, lv = best_idx / M;
    if (lu > R) lu -= M;
    if (lv > R) lv -= M;
    poi->u = (float)lu + uq;
    poi->v = (float)lv + vq;
    poi->u0 = uq;
    poi->v0 = vq;
    poi->zncc = best / (sqrtf(nq) * (float)(M * M));
  }
}

// --------------------------------------------------------------------------------------
// FFTCC for 32 < M <= 64 (subset radius 17..32): one 256-thread CTA per POI.  Same packing
// and cross-power algebra as k_fftcc; each 1-D transform is a direct DFT over one line,
// with (line, bin) outputs spread over the CTA and twiddles from the constant table.
// --------------------------------------------------------------------------------------
__device__ __forceinline__ void block_argmax(float& v, int& idx, float* sv, int* si)
{
#pragma unroll
  for (int o = 16; o > 0; o >>= 1)
  {
    const float ov = __shfl_xor_sync(kFull, v, o);
    const int oi = __shfl_xor_sync(kFull, idx, o);
    if (ov > v || (ov == v && oi < idx)) { v = ov; idx = oi; }
  }
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  if (lane == 0) { sv[warp] = v; si[warp] = idx; }
  __syncthreads();
  if (warp == 0)
  {
    v = lane < (int)(blockDim.x >> 5) ? sv[lane] : -2.f;
    idx = lane < (int)(blockDim.x >> 5) ? si[lane] : 0;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1)
    {
      const float ov = __shfl_xor_sync(kFull, v, o);
      const int oi = __shfl_xor_sync(kFull, idx, o);
      if (ov > v || (ov == v && oi < idx)) { v = ov; idx = oi; }
    }
  }
}

__device__ __forceinline__ float block_sum(float v, float* sbuf)
{
  v = warp_sum(v);
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  __syncthreads();
  if (lane == 0) sbuf[warp] = v;
  __syncthreads();
  float t = lane < (int)(blockDim.x >> 5) ? sbuf[lane] : 0.f;
  return warp_sum(t);
}

// out[line][k] = sum_j in[line][j] W^(j k) along rows (by_rows) or columns; conj twiddles
// when inverse.  in/out are m x s float2 arrays (row stride s, odd), m even.  A warp takes
// one bin pair (k, k + m/2) for all lines, lane = line: the twiddle index j k mod m is the
// same in every lane (one constant-cache broadcast per term), the line reads are
// conflict-free, and the pair shares its even- and odd-j sums,
// out[k] = E + O, out[k + m/2] = E - O, since W^(j m/2) = (-1)^j.
__device__ void dft_lines(const float2* in, float2* out, int m, int s, bool by_rows, bool inverse)
{
  const float2* tw = c_tw + tw_offset(m);
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
  const int half = m >> 1;
  const float sgn = inverse ? -1.f : 1.f;
  const int step_in = by_rows ? 1 : s;      // along the line
  const int line_in = by_rows ? s : 1;      // between lines
  for (int k = warp; k < half; k += nw)
  {
    for (int line = lane; line < m; line += 32)
    {
      const float2* src = in + line * line_in;
      float2 E = make_float2(0.f, 0.f), O = make_float2(0.f, 0.f);
      int e = 0;
      for (int j = 0; j < m; j += 2)
      {
        const float2 a = src[j * step_in];
        const float2 wa = tw[e];
        e += k;
        if (e >= m) e -= m;
        const float2 b = src[(j + 1) * step_in];
        const float2 wb = tw[e];
        e += k;
        if (e >= m) e -= m;
        const float wai = sgn * wa.y, wbi = sgn * wb.y;
        E.x += a.x * wa.x - a.y * wai;
        E.y += a.x * wai + a.y * wa.x;
        O.x += b.x * wb.x - b.y * wbi;
        O.y += b.x * wbi + b.y * wb.x;
      }
      const float2 lo = make_float2(E.x + O.x, E.y + O.y), hi = make_float2(E.x - O.x, E.y - O.y);
      if (by_rows)
      {
        out[line * s + k] = lo;
        out[line * s + k + half] = hi;
      }
      else
      {
        out[k * s + line] = lo;
        out[(k + half) * s + line] = hi;
      }
    }
  }
  __syncthreads();
}

__global__ void __launch_bounds__(256) k_fftcc_large(FftccParams P, int m)
{
  extern __shared__ float2 dyn[];
  __shared__ float s_red[32];
  __shared__ int s_idx[32];
  const int s = m + 1;
  float2* za = dyn;
  float2* zb = dyn + m * s;
  const int64_t i = blockIdx.x;
  if (!queue_slot_active(P, i)) return;
  dic_poi* poi = P.pois + i;
  const float px = poi->x, py = poi->y, u_init = poi->u, v_init = poi->v;
  const int w = P.w, h = P.h, R = m / 2;
  if ((int)px < R || (int)px >= w - R || (int)py < R || (int)py >= h - R ||
      int(px + u_init) < R || int(px + u_init) >= w - R || int(py + v_init) < R ||
      int(py + v_init) >= h - R)
    return;
  float rsum = 0.f, tsum = 0.f;
  for (int t = threadIdx.x; t < m * m; t += blockDim.x)
  {
    const int r = t / m, c = t % m;
    const float fxr = __fsub_rn(__fadd_rn(px, (float)c), (float)R);
    const float fyr = __fsub_rn(__fadd_rn(py, (float)r), (float)R);
    const float rv = P.ref[(size_t)(int)fyr * w + (int)fxr];
    const float tv = P.tar[(size_t)(int)__fadd_rn(fyr, v_init) * w + (int)__fadd_rn(fxr, u_init)];
    za[r * s + c] = make_float2(rv, tv);
    rsum += rv;
    tsum += tv;
  }
  rsum = block_sum(rsum, s_red);
  tsum = block_sum(tsum, s_red);
  const float rmean = rsum / (float)(m * m), tmean = tsum / (float)(m * m);
  float rn = 0.f, tn = 0.f;
  for (int t = threadIdx.x; t < m * m; t += blockDim.x)
  {
    const int r = t / m, c = t % m;
    float2 v = za[r * s + c];
    v.x -= rmean;
    v.y -= tmean;
    rn += v.x * v.x;
    tn += v.y * v.y;
    za[r * s + c] = v;
  }
  rn = block_sum(rn, s_red);
  tn = block_sum(tn, s_red);
  __syncthreads();
  dft_lines(za, zb, m, s, true, false);    // rows
  dft_lines(zb, za, m, s, false, false);   // columns -> Z in za
  for (int t = threadIdx.x; t < m * m; t += blockDim.x)
  {
    const int k1 = t / m, k2 = t % m;
    const float2 A = za[k1 * s + k2];
    const float2 zm = za[((m - k1) % m) * s + (m - k2) % m];
    const float2 B = make_float2(zm.x, -zm.y);
    const float2 Rk = make_float2(0.5f * (A.x + B.x), 0.5f * (A.y + B.y));
    const float2 D = csub(A, B);
    const float2 Tk = make_float2(0.5f * D.y, -0.5f * D.x);
    zb[k1 * s + k2] = make_float2(Rk.x * Tk.x + Rk.y * Tk.y, Rk.x * Tk.y - Rk.y * Tk.x);
  }
  __syncthreads();
  dft_lines(zb, za, m, s, false, true);    // inverse columns
  dft_lines(za, zb, m, s, true, true);     // inverse rows -> correlation in zb (real part)
  float best = -2.f;
  int best_idx = 0;
  for (int t = threadIdx.x; t < m * m; t += blockDim.x)
  {
    const float v = zb[(t / m) * s + t % m].x;
    if (v > best) { best = v; best_idx = t; }
  }
  block_argmax(best, best_idx, s_red, s_idx);
  if (threadIdx.x == 0)
  {
    int lu = best_idx % m, lv = best_idx / m;
    if (lu > R) lu -= m;
    if (lv > R) lv -= m;
    poi->u = (float)lu + u_init;
    poi->v = (float)lv + v_init;
    poi->u0 = u_init;
    poi->v0 = v_init;
    poi->zncc = best / (sqrtf(rn * tn) * (float)(m * m));
  }
}

// --------------------------------------------------------------------------------------
// FFTCC for 32 < M <= 64 (subset radius 17..32) as a real FFT: one 128-thread CTA per POI,
// the packed window z = ref + i tar in shared memory ([M][M + 1] float2; consecutive lanes
// take consecutive lines, whose odd float2 stride keeps a warp's accesses conflict-free in
// both directions), every line transform a four-step FFT M = N1 * N2 done in place by
// small register FFTs:
//   forward, natural input -> output X[k1 + N1 k2] stored at N2 k1 + k2 (permuted);
//   inverse of a permuted input -> natural output, so no transpose pass is needed.
// Rows, then columns, the cross-power conj(R) T paired with its mirror frequency (in place),
// inverse columns, inverse rows, argmax with the CPU's tie rule.  Same packing and algebra
// as k_fftcc.
// --------------------------------------------------------------------------------------
__host__ __device__ constexpr int big_n1(int m)
{
  int best = 1;
  for (int d = 2; d * d <= m; ++d)
    if (m % d == 0) best = d;
  return best;
}

template <int M, bool kRows>
__device__ __forceinline__ int line_at(int line, int j)
{
  return kRows ? line * (M + 1) + j : j * (M + 1) + line;
}

// Work mapping of k_fftcc_big: thread -> line (or column) `line` = tid % M and part
// `part` = tid / M of `parts` = kBigThreads / M; a thread walks its line's sub-transforms (or
// rows) part, part + parts, ...  (A flat index per item, divided by M in every loop, made
// integer arithmetic 61 % of the ALU pipe and the kernel instruction-bound.)  Threads past
// parts * M only join the barriers and reductions.
constexpr int kBigThreads = 128;

// forward line transforms over all M lines: natural -> permuted
template <int M, bool kRows>
__device__ __forceinline__ void big_forward(float2* z, int line, int part, bool on)
{
  constexpr int N1 = big_n1(M), N2 = M / N1, kParts = kBigThreads / M;
  const float2* tw = c_tw + tw_offset(M);
  if (on)
    for (int n2 = part; n2 < N2; n2 += kParts)
    {
      float2 a[N1], b[N1];
#pragma unroll
      for (int n1 = 0; n1 < N1; ++n1) a[n1] = z[line_at<M, kRows>(line, N2 * n1 + n2)];
      Fft<N1>::run(a, b);
#pragma unroll
      for (int k1 = 0; k1 < N1; ++k1) z[line_at<M, kRows>(line, N2 * k1 + n2)] = k1 ? cmul(b[k1], tw[n2 * k1]) : b[k1];
    }
  __syncthreads();
  if (on)
    for (int k1 = part; k1 < N1; k1 += kParts)
    {
      float2 a[N2], b[N2];
#pragma unroll
      for (int n2 = 0; n2 < N2; ++n2) a[n2] = z[line_at<M, kRows>(line, N2 * k1 + n2)];
      Fft<N2>::run(a, b);
#pragma unroll
      for (int k2 = 0; k2 < N2; ++k2) z[line_at<M, kRows>(line, N2 * k1 + k2)] = b[k2];
    }
  __syncthreads();
}

// forward-kernel transforms of permuted input over all M lines: permuted -> natural
template <int M, bool kRows>
__device__ __forceinline__ void big_from_permuted(float2* z, int line, int part, bool on)
{
  constexpr int N1 = big_n1(M), N2 = M / N1, kParts = kBigThreads / M;
  const float2* tw = c_tw + tw_offset(M);
  if (on)
    for (int k1 = part; k1 < N1; k1 += kParts)
    {
      float2 a[N2], b[N2];
#pragma unroll
      for (int k2 = 0; k2 < N2; ++k2) a[k2] = z[line_at<M, kRows>(line, N2 * k1 + k2)];
      Fft<N2>::run(a, b);
#pragma unroll
      for (int j = 0; j < N2; ++j) z[line_at<M, kRows>(line, N2 * k1 + j)] = k1 ? cmul(b[j], tw[j * k1]) : b[j];
    }
  __syncthreads();
  if (on)
    for (int j = part; j < N2; j += kParts)
    {
      float2 a[N1], b[N1];
#pragma unroll
      for (int k1 = 0; k1 < N1; ++k1) a[k1] = z[line_at<M, kRows>(line, N2 * k1 + j)];
      Fft<N1>::run(a, b);
#pragma unroll
      for (int i = 0; i < N1; ++i) z[line_at<M, kRows>(line, N2 * i + j)] = b[i];
    }
  __syncthreads();
}

template <int M>
__global__ void __launch_bounds__(kBigThreads) k_fftcc_big(FftccParams P)
{
  constexpr int N1 = big_n1(M), N2 = M / N1, S = M + 1, R = M / 2, kParts = kBigThreads / M;
  static_assert(kParts >= 1, "one thread per line at least");
  extern __shared__ float2 zbig[];
  __shared__ float s_red[32];
  __shared__ int s_idx[32];
  const int64_t i = blockIdx.x;
  if (!queue_slot_active(P, i)) return;
  dic_poi* poi = P.pois + i;
  const float px = poi->x, py = poi->y, u_init = poi->u, v_init = poi->v;
  const int w = P.w, h = P.h;
  if ((int)px < R || (int)px >= w - R || (int)py < R || (int)py >= h - R ||
      int(px + u_init) < R || int(px + u_init) >= w - R || int(py + v_init) < R ||
      int(py + v_init) >= h - R)
    return;
  const int c = (int)threadIdx.x % M, part = (int)threadIdx.x / M;
  const bool on = part < kParts;
  // window columns: thread column c, rows part, part + kParts, ...
  float rsum = 0.f, tsum = 0.f;
  if (on)
  {
    const float fxr = __fsub_rn(__fadd_rn(px, (float)c), (float)R);
    const int xr = (int)fxr, xt = (int)__fadd_rn(fxr, u_init);
    for (int r = part; r < M; r += kParts)
    {
      const float fyr = __fsub_rn(__fadd_rn(py, (float)r), (float)R);
      const float rv = P.ref[(size_t)(int)fyr * w + xr];
      const float tv = P.tar[(size_t)(int)__fadd_rn(fyr, v_init) * w + xt];
      zbig[r * S + c] = make_float2(rv, tv);
      rsum += rv;
      tsum += tv;
    }
  }
  rsum = block_sum(rsum, s_red);
  tsum = block_sum(tsum, s_red);
  const float rmean = rsum / (float)(M * M), tmean = tsum / (float)(M * M);
  float rn = 0.f, tn = 0.f;
  if (on)
    for (int r = part; r < M; r += kParts)
    {
      float2 v = zbig[r * S + c];
      v.x -= rmean;
      v.y -= tmean;
      rn += v.x * v.x;
      tn += v.y * v.y;
      zbig[r * S + c] = v;
    }
  rn = block_sum(rn, s_red);
  tn = block_sum(tn, s_red);
  __syncthreads();
  big_forward<M, true>(zbig, c, part, on);    // rows (thread = row c)
  big_forward<M, false>(zbig, c, part, on);   // columns (thread = column c): Z[kr][kc] at (pos kr, pos kc)
  // cross-power, conjugated for the inverse (conj(FFT(conj(.))) keeps the real part):
  // X(k) = conj(R(k)) T(k) with R, T recovered from Z[k] and Z[-k]; X(-k) = conj(X(k)).
  if (on)
  {
    const int pc = c, kc = pc / N2 + N1 * (pc % N2), mc = (M - kc) % M, qc = N2 * (mc % N1) + mc / N1;
    for (int pr = part; pr < M; pr += kParts)
    {
      const int kr = pr / N2 + N1 * (pr % N2);
      const int mr = (M - kr) % M;
      const int qr = N2 * (mr % N1) + mr / N1;
      const int p = pr * M + pc, q = qr * M + qc;
      if (p > q) continue;
      const float2 A = zbig[pr * S + pc];
      const float2 zm = zbig[qr * S + qc];
      const float2 B = make_float2(zm.x, -zm.y);
      const float2 Rk = make_float2(0.5f * (A.x + B.x), 0.5f * (A.y + B.y));
      const float2 D = csub(A, B);
      const float2 Tk = make_float2(0.5f * D.y, -0.5f * D.x);
      const float2 X = make_float2(Rk.x * Tk.x + Rk.y * Tk.y, Rk.x * Tk.y - Rk.y * Tk.x);
      zbig[pr * S + pc] = make_float2(X.x, -X.y);
      if (q != p) zbig[qr * S + qc] = X;
    }
  }
  __syncthreads();
  big_from_permuted<M, false>(zbig, c, part, on);   // columns back to natural rows
  big_from_permuted<M, true>(zbig, c, part, on);    // rows back to natural columns: correlation in .x
  float best = -2.f;
  int best_idx = 0;
  if (on)
    for (int r = part; r < M; r += kParts)   // increasing index: strict '>' keeps the lowest
    {
      const float v = zbig[r * S + c].x;
      if (v > best) { best = v; best_idx = r * M + c; }
    }
  block_argmax(best, best_idx, s_red, s_idx);
  if (threadIdx.x == 0)
  {
    int lu = best_idx % M, lv = best_idx / M;
    if (lu > R) lu -= M;
    if (lv > R) lv -= M;
    poi->u = (float)lu + u_init;
    poi->v = (float)lv + v_init;
    poi->u0 = u_init;
    poi->v0 = v_init;
    poi->zncc = best / (sqrtf(rn * tn) * (float)(M * M));
  }
}

// --------------------------------------------------------------------------------------
// Frame policy (processFrame, opencorr_cli_cuda_mvp.cpp:3024-3210) on the device.
// A frame is one fixed launch sequence: seed from the previous frame, IC-GN, scan for bad
// POIs, decide, then either the whole-frame FFTCC + IC-GN pass with a per-POI merge or
// the POI-level repair (FFTCC + IC-GN on the candidates only, through the layout slots),
// each gated by a device-side switch.  The per-POI rules are the reference's own:
//   bad        isBadPoiForFallback            (:490-494)
//   candidate  isPoiLevelFallbackCandidate    (:541-558)
//   replace    shouldReplacePoiWithFallback   (:503-515)
//   take       shouldTakeFrameFallbackResult  (:524-539)
// --------------------------------------------------------------------------------------
struct FrameCounters
{
  unsigned long long bad;         // bad POIs after the skip attempt
  unsigned long long candidates;  // POI-level repair candidates
  unsigned long long recovered;   // repaired POIs that are no longer bad
  unsigned long long bad_after;   // bad POIs in the final result
  int64_t candidate_count;        // = candidates, as a queue length for the repair launches
  int frame_fallback;             // 1: whole-frame pass runs
  int poi_repair;                 // 1: POI-level repair runs
  unsigned long long temporal;    // POIs seeded by temporal extrapolation
};

__device__ __forceinline__ bool is_bad_poi(float z, float thr) { return z != -3.f && (!isfinite(z) || z < thr); }

__device__ __forceinline__ bool replace_with_fallback(float cur_z, float fb_z)
{
  if (!isfinite(fb_z) || fb_z == -3.f) return false;
  if (!isfinite(cur_z)) return true;
  return fb_z >= cur_z;
}

// isEligibleTemporalSeedHistory (:499-504)
__device__ __forceinline__ bool temporal_history_ok(const dic_poi& p, float thr)
{
  return isfinite(p.u) && isfinite(p.v) && isfinite(p.zncc) && p.zncc >= thr;
}

// seedPoiQueueFromPrevious (:560-624): the template record, with the previous frame's six
// first-order parameters where that result is valid and its result fields cleared.  With
// `prev2` (the frame before; for sequences only once *hist_frames >= 2) and both results
// eligible at the same location, u and v become prev + (prev - prev2) when that step is at
// least 0.05 px and neither component's step exceeds max_delta (the subset radius); float
// arithmetic with separate roundings, as the CPU's expressions read.
__global__ void k_seed_from_previous(const dic_poi* __restrict__ tmpl, const dic_poi* __restrict__ prev,
                                     const dic_poi* __restrict__ prev2, const int* __restrict__ hist_frames,
                                     float thr, float max_delta, dic_poi* __restrict__ cur, int64_t n,
                                     FrameCounters* __restrict__ counters)
{
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  dic_poi q = tmpl[i];
  const dic_poi p = prev[i];
  if (isfinite(p.zncc) && p.zncc >= 0.f)
  {
    q.u = p.u; q.ux = p.ux; q.uy = p.uy;
    q.v = p.v; q.vx = p.vx; q.vy = p.vy;
    q.u0 = 0.f; q.v0 = 0.f; q.zncc = 0.f; q.iteration = 0.f; q.convergence = 0.f; q.feature = 0.f;
    if (prev2 && (!hist_frames || *hist_frames >= 2))
    {
      const dic_poi pp = prev2[i];
      if (p.x == pp.x && p.y == pp.y && p.x == q.x && p.y == q.y && temporal_history_ok(p, thr) &&
          temporal_history_ok(pp, thr))
      {
        constexpr float kMinStep = 0.05f;   // kTemporalSeedMinStepPx (:481)
        const float du = __fsub_rn(p.u, pp.u), dv = __fsub_rn(p.v, pp.v);
        const float pu = __fadd_rn(p.u, du), pv = __fadd_rn(p.v, dv);
        const float step_sq = __fadd_rn(__fmul_rn(du, du), __fmul_rn(dv, dv));
        if (isfinite(pu) && isfinite(pv) && step_sq >= __fmul_rn(kMinStep, kMinStep) && fabsf(du) <= max_delta &&
            fabsf(dv) <= max_delta)
        {
          q.u = pu;
          q.v = pv;
          atomicAdd(&counters->temporal, 1ull);
        }
      }
    }
  }
  cur[i] = q;
}

// the sequence's history depth (frames whose results are in prev / prev2), saturating at 2
__global__ void k_bump_history(int* hist_frames)
{
  if (threadIdx.x == 0 && *hist_frames < 2) ++*hist_frames;
}

__global__ void k_scan_bad(const dic_poi* __restrict__ cur, const dic_poi* __restrict__ prev, float thr,
                           int poi_fallback, FrameCounters* __restrict__ c, int64_t* __restrict__ cand, int64_t n)
{
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  bool bad = false, candidate = false;
  if (i < n)
  {
    const float z = cur[i].zncc;
    bad = is_bad_poi(z, thr);
    if (bad && poi_fallback)
    {
      if (!isfinite(z) || z < 0.f)
        candidate = true;
      else if (!prev || prev[i].x != cur[i].x || prev[i].y != cur[i].y || !isfinite(prev[i].zncc))
        candidate = true;
      else
        candidate = prev[i].zncc >= thr;
    }
  }
  const unsigned bad_mask = __ballot_sync(kFull, bad);
  if ((threadIdx.x & 31) == 0 && bad_mask) atomicAdd(&c->bad, (unsigned long long)__popc(bad_mask));
  if (candidate)
  {
    // Slot order depends on scheduling; every candidate is solved and merged on its own,
    // so the frame's result does not.
    const unsigned long long k = atomicAdd(&c->candidates, 1ull);
    cand[k] = i;
  }
}

__global__ void k_decide(FrameCounters* c, int64_t n, float frame_threshold, int poi_fallback)
{
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  // computeBadZnccRatioFromCount (:626-634), then the > test of :3115
  const float ratio = n > 0 ? (float)c->bad / (float)n : 0.f;
  c->frame_fallback = ratio > frame_threshold ? 1 : 0;
  c->poi_repair = (!c->frame_fallback && poi_fallback && c->candidates > 0) ? 1 : 0;
  c->candidate_count = (int64_t)c->candidates;
}

// The same with the threshold in device memory (fixed-reference sequences).
__global__ void k_decide_dev(FrameCounters* c, int64_t n, const float* frame_threshold, int poi_fallback)
{
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  const float ratio = n > 0 ? (float)c->bad / (float)n : 0.f;
  c->frame_fallback = ratio > *frame_threshold ? 1 : 0;
  c->poi_repair = (!c->frame_fallback && poi_fallback && c->candidates > 0) ? 1 : 0;
  c->candidate_count = (int64_t)c->candidates;
}

// First frame of a sequence: fallback threshold = its bad ratio + margin (:4275-4279).
__global__ void k_set_baseline(const FrameCounters* c, int64_t n, float margin, float* threshold)
{
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  const float ratio = n > 0 ? (float)c->bad / (float)n : 0.f;
  *threshold = ratio + margin;
}

__global__ void k_copy_queue(const dic_poi* __restrict__ src, dic_poi* __restrict__ dst, const int* enable, int64_t n)
{
  if (enable && *enable == 0) return;
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) dst[i] = src[i];
}

__global__ void k_gather_candidates(const dic_poi* __restrict__ tmpl, const int64_t* __restrict__ cand,
                                    const FrameCounters* c, dic_poi* __restrict__ fq, int64_t n_max)
{
  if (c->poi_repair == 0) return;
  const int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (k < c->candidate_count && k < n_max) fq[k] = tmpl[cand[k]];
}

// runPoiLevelFallback merge (:3003-3017)
__global__ void k_merge_repair(dic_poi* __restrict__ cur, const dic_poi* __restrict__ fq,
                               const int64_t* __restrict__ cand, FrameCounters* c, float thr, int64_t n_max)
{
  if (c->poi_repair == 0) return;
  const int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= c->candidate_count || k >= n_max) return;
  const int64_t idx = cand[k];
  const dic_poi f = fq[k];
  if (replace_with_fallback(cur[idx].zncc, f.zncc))
  {
    if (!is_bad_poi(f.zncc, thr)) atomicAdd(&c->recovered, 1ull);
    cur[idx] = f;
  }
}

// Whole-frame merge (:3141-3149, shouldTakeFrameFallbackResult)
__global__ void k_merge_frame(dic_poi* __restrict__ cur, const dic_poi* __restrict__ scratch,
                              const FrameCounters* c, float thr, int64_t n)
{
  if (c->frame_fallback == 0) return;
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const float sk = cur[i].zncc, sc = scratch[i].zncc;
  bool take;
  if (sk == -3.f)
    take = isfinite(sc) && sc != -3.f && sc >= thr;
  else if (is_bad_poi(sk, thr))
    take = replace_with_fallback(sk, sc);
  else
    take = false;
  if (take) cur[i] = scratch[i];
}

// Learned-seed fallback: a POI whose IC-GN from the proposal did not converge within the
// capped iteration budget (-4), was rejected (-3, -5), or ended with ZNCC below the
// acceptance threshold goes to FFTCC + IC-GN.  Slots are compacted as in k_scan_bad.
__global__ void k_scan_learned(const dic_poi* __restrict__ cur, float accept, FrameCounters* __restrict__ c,
                               int64_t* __restrict__ cand, int64_t n)
{
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const float z = cur[i].zncc;
  if (!(z >= accept))
  {
    const unsigned long long k = atomicAdd(&c->candidates, 1ull);
    cand[k] = i;
  }
}

__global__ void k_enable_candidates(FrameCounters* c)
{
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  c->candidate_count = (int64_t)c->candidates;
  c->poi_repair = c->candidates > 0 ? 1 : 0;
  c->frame_fallback = 0;
}

// The fallback result replaces the learned attempt for every candidate; `recovered` counts
// the candidates whose fallback result is not bad (zncc >= thr, or -3).
__global__ void k_merge_fallback(dic_poi* __restrict__ cur, const dic_poi* __restrict__ fq,
                                 const int64_t* __restrict__ cand, FrameCounters* c, float thr, int64_t n_max)
{
  if (c->poi_repair == 0) return;
  const int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= c->candidate_count || k >= n_max) return;
  const dic_poi f = fq[k];
  if (!is_bad_poi(f.zncc, thr)) atomicAdd(&c->recovered, 1ull);
  cur[cand[k]] = f;
}

__global__ void k_count_bad(const dic_poi* __restrict__ cur, float thr, unsigned long long* out, int64_t n)
{
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const bool bad = i < n && is_bad_poi(cur[i].zncc, thr);
  const unsigned m = __ballot_sync(kFull, bad);
  if ((threadIdx.x & 31) == 0 && m) atomicAdd(out, (unsigned long long)__popc(m));
}

}  // namespace dic
