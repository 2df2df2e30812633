// TEST INFRASTRUCTURE -- the oracle, not the product.
//
// CPU restatement of OpenCorr's FFTCC-seeded first-order IC-GN path as vendored by
// FastICGN.  Only tests/, __graft_entry__.smoke() and bench.py's CPU legs (cpu_baseline
// and the reference arm) load this library, and only as the checker or the timed CPU
// baseline.  The GPU product never links or calls it.
//
// Parity status: the reference's own CPU path (oc_icgn.cpp, oc_fftcc.cpp ...) needs
// Eigen, OpenCV and FFTW, none of which exists in this build environment, so it cannot
// be compiled.  This restatement follows those files line by line (citations below) and
// restates the three third-party pieces it calls:
//   * Eigen 3 (unpinned system package): Matrix6f::inverse() -> partial-pivot LU in
//     float (Eigen's PartialPivLU for fixed sizes > 4); Matrix3f::inverse() -> cofactor
//     formula; mean()/squaredNorm() -> serial float sums.
//   * FFTW3f 3.3 (unpinned): fftwf_plan_dft_r2c_2d / c2r_2d -> a mixed-radix complex
//     FFT of our own in float with the same unnormalised round-trip convention.
//   * OpenCV imread/convertTo -> callers pass float planes.
// It is pinned against analytic truth (the reference's sub-pixel accuracy gate cases
// and whole-pixel shift sequences) by tests/test_oracle.py.
//
// Build: g++ -O2 -fopenmp -ffp-contract=off -shared -fPIC (oracle/build.py).  FP
// contraction is off so x86_64 and aarch64 produce the same bits.

#include <omp.h>

#include <cmath>
#include <cstdint>
#include <cstring>
#include <vector>
#include <algorithm>
#include <chrono>

extern "C" {

// Memory layout of opencorr::POI2D (src/oc_poi.h:102-136): Point2D x, y, then
// DeformationVector2D p[12] (u ux uy uxx uxy uyy v vx vy vxx vxy vyy, :25-33),
// Result2D r[6] (u0 v0 zncc iteration convergence feature, :44-51),
// StrainVector2D e[3], Point2D subset_radius.
typedef struct oc_poi2d
{
  float x, y;
  float p[12];
  float r[6];
  float e[3];
  float subset_radius[2];
} oc_poi2d;

}  // extern "C"

namespace
{

enum { U = 0, UX = 1, UY = 2, V = 6, VX = 7, VY = 8 };
enum { U0 = 0, V0 = 1, ZNCC = 2, ITER = 3, CONV = 4 };

// ---------------------------------------------------------------------------
// Gradient2D4 (src/oc_gradient.cpp:21-22 factors, :37-79 loops)
// ---------------------------------------------------------------------------
const float kFirstFactor = 1.f / 12.f;
const float kSecondFactor = 2.f / 3.f;

// ---------------------------------------------------------------------------
// BicubicBspline (src/oc_cubic_bspline.h:52-58 BC matrix, .cpp:84-181)
// ---------------------------------------------------------------------------
const float kBC[4][4] = {
    {-144.0f / 336.0f, 384.0f / 336.0f, -384.0f / 336.0f, 144.0f / 336.0f},
    {342.0f / 336.0f, -702.0f / 336.0f, 450.0f / 336.0f, -90.0f / 336.0f},
    {-198.0f / 336.0f, -18.0f / 336.0f, 270.0f / 336.0f, -54.0f / 336.0f},
    {0.0f, 1.0f, 0.0f, 0.0f}};

inline float bspline_value(const float* coef, int w, int h, float x, float y)
{
  // BicubicBspline::compute (src/oc_cubic_bspline.cpp:134-181)
  if (x < 1 || y < 1 || x >= w - 2 || y >= h - 2 || std::isnan(x) || std::isnan(y))
    return -1.f;
  int xi = (int)std::floor(x);
  int yi = (int)std::floor(y);
  float xd = x - xi, yd = y - yi;
  float x2 = xd * xd, y2 = yd * yd;
  float x3 = x2 * xd, y3 = y2 * yd;
  const float* c = coef + ((size_t)yi * w + xi) * 16;
  return c[0] + c[1] * xd + c[2] * x2 + c[3] * x3
       + c[4] * yd + c[5] * yd * xd + c[6] * yd * x2 + c[7] * yd * x3
       + c[8] * y2 + c[9] * y2 * xd + c[10] * y2 * x2 + c[11] * y2 * x3
       + c[12] * y3 + c[13] * y3 * xd + c[14] * y3 * x2 + c[15] * y3 * x3;
}

// ---------------------------------------------------------------------------
// 6x6 inverse: restates Eigen's PartialPivLU-based inverse in float.
// ---------------------------------------------------------------------------
void inverse6(const float a_in[6][6], float inv[6][6])
{
  float a[6][6];
  int perm[6];
  std::memcpy(a, a_in, sizeof(a));
  for (int i = 0; i < 6; ++i) perm[i] = i;
  for (int k = 0; k < 6; ++k)
  {
    int piv = k;
    float best = std::fabs(a[k][k]);
    for (int i = k + 1; i < 6; ++i)
      if (std::fabs(a[i][k]) > best) { best = std::fabs(a[i][k]); piv = i; }
    if (piv != k)
    {
      for (int j = 0; j < 6; ++j) std::swap(a[k][j], a[piv][j]);
      std::swap(perm[k], perm[piv]);
    }
    for (int i = k + 1; i < 6; ++i)
    {
      a[i][k] = a[i][k] / a[k][k];
      for (int j = k + 1; j < 6; ++j) a[i][j] -= a[i][k] * a[k][j];
    }
  }
  // Solve L U x = P e_col for each column.
  for (int col = 0; col < 6; ++col)
  {
    float y[6];
    for (int i = 0; i < 6; ++i)
    {
      float s = (perm[i] == col) ? 1.f : 0.f;
      for (int j = 0; j < i; ++j) s -= a[i][j] * y[j];
      y[i] = s;
    }
    for (int i = 5; i >= 0; --i)
    {
      float s = y[i];
      for (int j = i + 1; j < 6; ++j) s -= a[i][j] * inv[j][col];
      inv[i][col] = s / a[i][i];
    }
  }
}

// 3x3 inverse by cofactors (Eigen compute_inverse_size3), row-major.
void inverse3(const float m[9], float out[9])
{
  float c00 = m[4] * m[8] - m[5] * m[7];
  float c10 = m[5] * m[6] - m[3] * m[8];
  float c20 = m[3] * m[7] - m[4] * m[6];
  float det = m[0] * c00 + m[1] * c10 + m[2] * c20;
  float inv_det = 1.f / det;
  out[0] = c00 * inv_det;
  out[1] = (m[2] * m[7] - m[1] * m[8]) * inv_det;
  out[2] = (m[1] * m[5] - m[2] * m[4]) * inv_det;
  out[3] = c10 * inv_det;
  out[4] = (m[0] * m[8] - m[2] * m[6]) * inv_det;
  out[5] = (m[2] * m[3] - m[0] * m[5]) * inv_det;
  out[6] = c20 * inv_det;
  out[7] = (m[1] * m[6] - m[0] * m[7]) * inv_det;
  out[8] = (m[0] * m[4] - m[1] * m[3]) * inv_det;
}

void mul3(const float a[9], const float b[9], float out[9])
{
  for (int r = 0; r < 3; ++r)
    for (int c = 0; c < 3; ++c)
      out[r * 3 + c] = a[r * 3 + 0] * b[0 * 3 + c] + a[r * 3 + 1] * b[1 * 3 + c] + a[r * 3 + 2] * b[2 * 3 + c];
}

// Deformation2D1::setWarp (src/oc_deformation.cpp:116-128)
void set_warp(float u, float ux, float uy, float v, float vx, float vy, float w[9])
{
  w[0] = 1.f + ux; w[1] = uy; w[2] = u;
  w[3] = vx; w[4] = 1.f + vy; w[5] = v;
  w[6] = 0.f; w[7] = 0.f; w[8] = 1.f;
}

// ---------------------------------------------------------------------------
// FFT (restates FFTW's unnormalised DFT; mixed-radix decimation in time)
// ---------------------------------------------------------------------------
struct cf { float re, im; };

struct Fft1d
{
  int n = 0;
  std::vector<int> factors;
  std::vector<cf> tw_fwd, tw_inv;  // exp(-+2 pi i k / n), k in [0, n)

  explicit Fft1d(int n_in) : n(n_in)
  {
    int m = n;
    for (int p : {4, 2, 3, 5})
      while (m % p == 0) { factors.push_back(p); m /= p; }
    for (int p = 7; m > 1; p += 2)
      while (m % p == 0) { factors.push_back(p); m /= p; }
    tw_fwd.resize(n);
    tw_inv.resize(n);
    for (int k = 0; k < n; ++k)
    {
      double a = -2.0 * M_PI * k / n;
      tw_fwd[k] = {(float)std::cos(a), (float)std::sin(a)};
      tw_inv[k] = {(float)std::cos(a), (float)-std::sin(a)};
    }
  }

  // out[k] = sum_j in[j * stride] * W^(j k), length len = n / (product of factors used so far)
  void rec(const cf* in, int stride, cf* out, int len, int fi, const cf* tw, int tw_step) const
  {
    if (len == 1) { out[0] = in[0]; return; }
    int p = factors[fi];
    int m = len / p;
    for (int q = 0; q < p; ++q)
      rec(in + q * stride, stride * p, out + q * m, m, fi + 1, tw, tw_step * p);
    // combine: X[k + s m] = sum_q W_len^{q (k + s m)} Y_q[k]
    cf tmp_stack[64];
    std::vector<cf> tmp_heap;
    cf* tmp = tmp_stack;
    if (p > 64) { tmp_heap.resize(p); tmp = tmp_heap.data(); }
    for (int k = 0; k < m; ++k)
    {
      for (int q = 0; q < p; ++q) tmp[q] = out[q * m + k];
      for (int s = 0; s < p; ++s)
      {
        int kk = k + s * m;
        float re = 0.f, im = 0.f;
        for (int q = 0; q < p; ++q)
        {
          int e = (int)(((long long)q * kk) % len) * tw_step;
          cf w = tw[e];
          re += tmp[q].re * w.re - tmp[q].im * w.im;
          im += tmp[q].re * w.im + tmp[q].im * w.re;
        }
        out[kk] = {re, im};
      }
    }
  }

  void run(const cf* in, int stride, cf* out, bool inverse) const
  {
    rec(in, stride, out, n, 0, inverse ? tw_inv.data() : tw_fwd.data(), 1);
  }
};

// In-place 2D transform of an n x n row-major complex array.
void fft2d(const Fft1d& f, cf* a, bool inverse, std::vector<cf>& line_in, std::vector<cf>& line_out)
{
  int n = f.n;
  for (int r = 0; r < n; ++r)
  {
    f.run(a + r * n, 1, line_out.data(), inverse);
    std::memcpy(a + r * n, line_out.data(), n * sizeof(cf));
  }
  for (int c = 0; c < n; ++c)
  {
    for (int r = 0; r < n; ++r) line_in[r] = a[r * n + c];
    f.run(line_in.data(), 1, line_out.data(), inverse);
    for (int r = 0; r < n; ++r) a[r * n + c] = line_out[r];
  }
}

struct FftccScratch
{
  std::vector<cf> ref, tar, line_in, line_out;
  std::vector<float> zncc;
  explicit FftccScratch(int m) : ref(m * m), tar(m * m), line_in(m), line_out(m), zncc(m * m) {}
};

}  // namespace

extern "C" {

int oc_oracle_version(void) { return 1; }

// Gradient2D4::getGradientX / getGradientY (src/oc_gradient.cpp:37-79).
void oc_gradient(const float* img, int w, int h, float* gx, float* gy, int threads)
{
  std::memset(gx, 0, sizeof(float) * (size_t)w * h);
  std::memset(gy, 0, sizeof(float) * (size_t)w * h);
#pragma omp parallel for num_threads(threads)
  for (int r = 0; r < h; r++)
  {
    for (int c = 2; c < w - 2; c++)
    {
      float result = 0.0f;
      result -= img[(size_t)r * w + c + 2] * kFirstFactor;
      result += img[(size_t)r * w + c + 1] * kSecondFactor;
      result -= img[(size_t)r * w + c - 1] * kSecondFactor;
      result += img[(size_t)r * w + c - 2] * kFirstFactor;
      gx[(size_t)r * w + c] = result;
    }
  }
#pragma omp parallel for num_threads(threads)
  for (int r = 2; r < h - 2; r++)
  {
    for (int c = 0; c < w; c++)
    {
      float result = 0.0f;
      result -= img[(size_t)(r + 2) * w + c] * kFirstFactor;
      result += img[(size_t)(r + 1) * w + c] * kSecondFactor;
      result -= img[(size_t)(r - 1) * w + c] * kSecondFactor;
      result += img[(size_t)(r - 2) * w + c] * kFirstFactor;
      gy[(size_t)r * w + c] = result;
    }
  }
}

// BicubicBspline::prepare (src/oc_cubic_bspline.cpp:84-132).  coef holds h*w*16 floats,
// texel (r, c) at [(r*w + c)*16 + k*4 + l]; texels outside 1 <= c < w-2, 1 <= r < h-2 are 0.
void oc_bspline_prepare(const float* img, int w, int h, float* coef, int threads)
{
  std::memset(coef, 0, sizeof(float) * (size_t)w * h * 16);
#pragma omp parallel for num_threads(threads)
  for (int r = 1; r < h - 2; r++)
  {
    for (int c = 1; c < w - 2; c++)
    {
      float q[4][4];
      for (int i = 0; i < 4; i++)
        for (int j = 0; j < 4; j++)
          q[i][j] = img[(size_t)(r - 1 + i) * w + (c - 1 + j)];
      float p[4][4] = {{0.f}};
      for (int k = 0; k < 4; k++)
        for (int l = 0; l < 4; l++)
          for (int m = 0; m < 4; m++)
            for (int n = 0; n < 4; n++)
              p[k][l] += kBC[l][m] * kBC[k][n] * q[n][m];
      float* dst = coef + ((size_t)r * w + c) * 16;
      for (int k = 0; k < 4; k++)
        for (int l = 0; l < 4; l++)
          dst[k * 4 + l] = p[3 - k][3 - l];
    }
  }
}

float oc_bspline_value(const float* coef, int w, int h, float x, float y)
{
  return bspline_value(coef, w, h, x, y);
}

// ICGN2D1::compute(POI2D*) (src/oc_icgn.cpp:168-387) over a queue with an OpenMP
// parallel for (:389-397).  ref/gx/gy are the reference plane and its Gradient2D4
// planes, coef the target's BicubicBspline table; all w x h.
void oc_icgn2d1(const float* ref, const float* gx, const float* gy, const float* coef, int w, int h,
                int rx, int ry, float conv_criterion, float stop_condition,
                oc_poi2d* pois, long long n, int threads)
{
  const int sw = 2 * rx + 1, sh = 2 * ry + 1, size = sw * sh;
#pragma omp parallel num_threads(threads)
  {
    std::vector<float> ref_sub(size), tar_sub(size), err(size), sd((size_t)size * 6);
#pragma omp for schedule(dynamic, 64)
    for (long long i = 0; i < n; ++i)
    {
      oc_poi2d* poi = &pois[i];
      // entry test (:184-191)
      if (poi->y - ry < 0 || poi->x - rx < 0 || poi->y + ry > h - 1 || poi->x + rx > w - 1
          || std::fabs(poi->p[U]) >= w || std::fabs(poi->p[V]) >= h
          || poi->r[ZNCC] < 0 || std::isnan(poi->p[U]) || std::isnan(poi->p[V]))
      {
        poi->r[ZNCC] = poi->r[ZNCC] >= 0 ? -3.f : poi->r[ZNCC];
        continue;
      }
      // reference subset: Subset2D::fill + zeroMeanNorm (src/oc_subset.cpp:39-53)
      const int ul_x = (int)poi->x - rx, ul_y = (int)poi->y - ry;
      float sum = 0.f;
      for (int r = 0; r < sh; ++r)
        for (int c = 0; c < sw; ++c)
        {
          float v = ref[(size_t)(ul_y + r) * w + ul_x + c];
          ref_sub[r * sw + c] = v;
          sum += v;
        }
      float mean = sum / size;
      float sq = 0.f;
      for (int k = 0; k < size; ++k)
      {
        ref_sub[k] -= mean;
        sq += ref_sub[k] * ref_sub[k];
      }
      const float ref_norm = std::sqrt(sq);

      // Hessian (:203-231), float, lower triangle mirrored
      float hess[6][6] = {{0.f}};
      for (int r = 0; r < sh; r++)
        for (int c = 0; c < sw; c++)
        {
          int xl = c - rx, yl = r - ry;
          int xg = (int)poi->x + xl, yg = (int)poi->y + yl;
          float gxv = gx[(size_t)yg * w + xg], gyv = gy[(size_t)yg * w + xg];
          float* s = &sd[((size_t)r * sw + c) * 6];
          s[0] = gxv; s[1] = gxv * xl; s[2] = gxv * yl;
          s[3] = gyv; s[4] = gyv * xl; s[5] = gyv * yl;
          for (int a = 0; a < 6; a++)
            for (int b = 0; b < a + 1; b++)
            {
              hess[a][b] += s[a] * s[b];
              hess[b][a] = hess[a][b];
            }
        }
      float inv_h[6][6];
      inverse6(hess, inv_h);

      const float p_init[6] = {poi->p[U], poi->p[UX], poi->p[UY], poi->p[V], poi->p[VX], poi->p[VY]};
      float warp[9];
      set_warp(p_init[0], p_init[1], p_init[2], p_init[3], p_init[4], p_init[5], warp);
      float pc[6] = {p_init[0], p_init[1], p_init[2], p_init[3], p_init[4], p_init[5]};
      int it = 0;
      float dp_norm_max = 0.f, znssd = 0.f;
      bool rejected = false;
      do
      {
        it++;
        bool oob = false, nan = false;
        for (int r = 0; r < sh; r++)
          for (int c = 0; c < sw; c++)
          {
            float xl = (float)(c - rx), yl = (float)(r - ry);
            // Deformation2D1::warp (src/oc_deformation.cpp:94-106): warp_matrix * (x, y, 1)
            float wx = warp[0] * xl + warp[1] * yl + warp[2] * 1.f;
            float wy = warp[3] * xl + warp[4] * yl + warp[5] * 1.f;
            float gxp = poi->x + wx, gyp = poi->y + wy;
            // outOfInterpolatableRange (src/oc_icgn.cpp:39-43), then NaN (:266-273)
            if (gxp < 1 || gyp < 1 || gxp >= w - 2 || gyp >= h - 2) oob = true;
            else if (std::isnan(gxp) || std::isnan(gyp)) nan = true;
            tar_sub[r * sw + c] = bspline_value(coef, w, h, gxp, gyp);
          }
        if (oob) { poi->r[ZNCC] = -3.f; rejected = true; break; }   // :285-289
        if (nan) { poi->r[ZNCC] = -5.f; rejected = true; break; }   // :297-301
        float tsum = 0.f;
        for (int k = 0; k < size; ++k) tsum += tar_sub[k];
        float tmean = tsum / size;
        float tsq = 0.f;
        for (int k = 0; k < size; ++k)
        {
          tar_sub[k] -= tmean;
          tsq += tar_sub[k] * tar_sub[k];
        }
        float tar_norm = std::sqrt(tsq);
        // error image and ZNSSD (:306-309)
        float scale = ref_norm / tar_norm;
        float esq = 0.f;
        for (int k = 0; k < size; ++k)
        {
          err[k] = tar_sub[k] * scale - ref_sub[k];
          esq += err[k] * err[k];
        }
        znssd = esq / (ref_norm * ref_norm);
        // numerator (:312-322)
        float num[6] = {0.f};
        for (int k = 0; k < size; ++k)
        {
          const float* s = &sd[(size_t)k * 6];
          for (int a = 0; a < 6; a++) num[a] += s[a] * err[k];
        }
        float dp[6] = {0.f};
        for (int a = 0; a < 6; a++)
          for (int b = 0; b < 6; b++) dp[a] += inv_h[a][b] * num[b];
        // warp update W <- W * W(dp)^-1 (:333-339)
        float inc[9], inc_inv[9], next[9];
        set_warp(dp[0], dp[1], dp[2], dp[3], dp[4], dp[5], inc);
        inverse3(inc, inc_inv);
        mul3(warp, inc_inv, next);
        std::memcpy(warp, next, sizeof(warp));
        pc[0] = warp[2]; pc[1] = warp[0] - 1.f; pc[2] = warp[1];
        pc[3] = warp[5]; pc[4] = warp[3]; pc[5] = warp[4] - 1.f;
        // convergence (:342-352)
        int rx2 = rx * rx, ry2 = ry * ry;
        dp_norm_max = dp[0] * dp[0] + dp[1] * dp[1] * rx2 + dp[2] * dp[2] * ry2
                    + dp[3] * dp[3] + dp[4] * dp[4] * rx2 + dp[5] * dp[5] * ry2;
        dp_norm_max = std::sqrt(dp_norm_max);
      } while (it < stop_condition && dp_norm_max >= conv_criterion);
      if (rejected) continue;

      // outputs (:355-386)
      poi->p[U] = pc[0]; poi->p[UX] = pc[1]; poi->p[UY] = pc[2];
      poi->p[V] = pc[3]; poi->p[VX] = pc[4]; poi->p[VY] = pc[5];
      poi->r[U0] = p_init[0];
      poi->r[V0] = p_init[3];
      poi->r[ZNCC] = 0.5f * (2 - znssd);
      poi->r[ITER] = (float)it;
      poi->r[CONV] = dp_norm_max;
      poi->subset_radius[0] = (float)rx;
      poi->subset_radius[1] = (float)ry;
      if (poi->r[CONV] >= conv_criterion && poi->r[ITER] >= stop_condition) poi->r[ZNCC] = -4.f;
      if (std::isnan(poi->r[ZNCC]) || std::isnan(poi->p[U]) || std::isnan(poi->p[V]))
      {
        poi->p[U] = poi->r[U0];
        poi->p[V] = poi->r[V0];
        poi->r[ZNCC] = -5.f;
      }
    }
  }
}

// FFTCC2D::compute(POI2D*) (src/oc_fftcc.cpp:396-496) over a queue (:529-557).  Square
// radius r only, as the FFTCC2D constructor enforces (:162-164).  The prepared-reference
// path (:246-394) computes the same reference spectrum, so it gives the same results.
void oc_fftcc2d(const float* ref, const float* tar, int w, int h, int r,
                oc_poi2d* pois, long long n, int threads)
{
  const int m = 2 * r, size = m * m;
#pragma omp parallel num_threads(threads)
  {
    Fft1d fft(m);
    FftccScratch s(m);
#pragma omp for schedule(dynamic, 64)
    for (long long i = 0; i < n; ++i)
    {
      oc_poi2d* poi = &pois[i];
      const float u_init = poi->p[U], v_init = poi->p[V];
      if ((int)poi->x < r || (int)poi->x >= w - r || (int)poi->y < r || (int)poi->y >= h - r
          || int(poi->x + u_init) < r || int(poi->x + u_init) >= w - r
          || int(poi->y + v_init) < r || int(poi->y + v_init) >= h - r)
        continue;
      float ref_mean = 0.f, tar_mean = 0.f, ref_norm = 0.f, tar_norm = 0.f;
      std::vector<float> rs(size), ts(size);
      for (int rr = 0; rr < m; rr++)
        for (int c = 0; c < m; c++)
        {
          float rxp = poi->x + c - r, ryp = poi->y + rr - r;
          float v = ref[(size_t)(int)ryp * w + (int)rxp];
          rs[rr * m + c] = v;
          ref_mean += v;
          float txp = rxp + u_init, typ = ryp + v_init;
          v = tar[(size_t)(int)typ * w + (int)txp];
          ts[rr * m + c] = v;
          tar_mean += v;
        }
      ref_mean /= size;
      tar_mean /= size;
      for (int k = 0; k < size; k++)
      {
        rs[k] -= ref_mean;
        ts[k] -= tar_mean;
        ref_norm += rs[k] * rs[k];
        tar_norm += ts[k] * ts[k];
      }
      for (int k = 0; k < size; k++)
      {
        s.ref[k] = {rs[k], 0.f};
        s.tar[k] = {ts[k], 0.f};
      }
      fft2d(fft, s.ref.data(), false, s.line_in, s.line_out);
      fft2d(fft, s.tar.data(), false, s.line_in, s.line_out);
      // zncc_freq = conj(ref) * tar (:450-455)
      for (int k = 0; k < size; k++)
      {
        cf a = s.ref[k], b = s.tar[k];
        s.ref[k] = {a.re * b.re + a.im * b.im, a.re * b.im - a.im * b.re};
      }
      fft2d(fft, s.ref.data(), true, s.line_in, s.line_out);
      // argmax, strict '>' from index 0 (:466-475)
      float max_zncc = -2.f;
      int max_idx = 0;
      for (int k = 0; k < size; k++)
      {
        float z = s.ref[k].re;
        s.zncc[k] = z;
        if (z > max_zncc) { max_zncc = z; max_idx = k; }
      }
      int lu = max_idx % m, lv = max_idx / m;
      if (lu > r) lu -= m;
      if (lv > r) lv -= m;
      poi->p[U] = (float)lu + u_init;
      poi->p[V] = (float)lv + v_init;
      poi->r[U0] = u_init;
      poi->r[V0] = v_init;
      poi->r[ZNCC] = max_zncc / (std::sqrt(ref_norm * tar_norm) * size);
    }
  }
}

// The full correlation map of one POI (for tie analysis in tests): writes m*m floats
// (unnormalised, as FFTW's c2r returns them) and returns 1, or 0 when the POI is out of
// bounds and FFTCC would leave it untouched.
int oc_fftcc2d_map(const float* ref, const float* tar, int w, int h, int r, float x, float y,
                   float u_init, float v_init, float* out_map)
{
  oc_poi2d poi;
  std::memset(&poi, 0, sizeof(poi));
  poi.x = x; poi.y = y; poi.p[U] = u_init; poi.p[V] = v_init;
  const int m = 2 * r, size = m * m;
  if ((int)x < r || (int)x >= w - r || (int)y < r || (int)y >= h - r
      || int(x + u_init) < r || int(x + u_init) >= w - r
      || int(y + v_init) < r || int(y + v_init) >= h - r)
    return 0;
  Fft1d fft(m);
  FftccScratch s(m);
  std::vector<float> rs(size), ts(size);
  float ref_mean = 0.f, tar_mean = 0.f;
  for (int rr = 0; rr < m; rr++)
    for (int c = 0; c < m; c++)
    {
      float rxp = x + c - r, ryp = y + rr - r;
      rs[rr * m + c] = ref[(size_t)(int)ryp * w + (int)rxp];
      ts[rr * m + c] = tar[(size_t)(int)(ryp + v_init) * w + (int)(rxp + u_init)];
      ref_mean += rs[rr * m + c];
      tar_mean += ts[rr * m + c];
    }
  ref_mean /= size;
  tar_mean /= size;
  for (int k = 0; k < size; k++)
  {
    s.ref[k] = {rs[k] - ref_mean, 0.f};
    s.tar[k] = {ts[k] - tar_mean, 0.f};
  }
  fft2d(fft, s.ref.data(), false, s.line_in, s.line_out);
  fft2d(fft, s.tar.data(), false, s.line_in, s.line_out);
  for (int k = 0; k < size; k++)
  {
    cf a = s.ref[k], b = s.tar[k];
    s.ref[k] = {a.re * b.re + a.im * b.im, a.re * b.im - a.im * b.re};
  }
  fft2d(fft, s.ref.data(), true, s.line_in, s.line_out);
  for (int k = 0; k < size; k++) out_map[k] = s.ref[k].re;
  return 1;
}

// One image pair through the CPU path as opencorr_cli.cpp:120-135 runs it (FFTCC seed,
// then ICGN2D1 prepare + compute), with each phase timed (seconds) into t[4]:
// gradient, B-spline table, FFTCC, IC-GN.
void oc_run_pair(const float* ref, const float* tar, int w, int h, int r, float conv_criterion,
                 float stop_condition, oc_poi2d* pois, long long n, int threads, double* t)
{
  using clk = std::chrono::steady_clock;
  std::vector<float> gx((size_t)w * h), gy((size_t)w * h), coef((size_t)w * h * 16);
  auto t0 = clk::now();
  oc_gradient(ref, w, h, gx.data(), gy.data(), threads);
  auto t1 = clk::now();
  oc_bspline_prepare(tar, w, h, coef.data(), threads);
  auto t2 = clk::now();
  oc_fftcc2d(ref, tar, w, h, r, pois, n, threads);
  auto t3 = clk::now();
  oc_icgn2d1(ref, gx.data(), gy.data(), coef.data(), w, h, r, r, conv_criterion, stop_condition,
             pois, n, threads);
  auto t4 = clk::now();
  if (t)
  {
    t[0] = std::chrono::duration<double>(t1 - t0).count();
    t[1] = std::chrono::duration<double>(t2 - t1).count();
    t[2] = std::chrono::duration<double>(t3 - t2).count();
    t[3] = std::chrono::duration<double>(t4 - t3).count();
  }
}

}  // extern "C"
