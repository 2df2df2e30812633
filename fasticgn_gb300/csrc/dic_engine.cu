// Host engine behind the C ABI of include/dic.h.
//
// One dic_engine owns a CUDA stream and the device state of one reference/target pair
// (see dic_kernels.cuh for the HBM layout).  Calls are synchronous from the caller's
// point of view except dic_run_device, which only enqueues work on the engine stream.
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <functional>
#include <mutex>
#include <set>
#include <string>
#include <thread>
#include <vector>
#include <algorithm>

#include "dic_kernels.cuh"
#include "dic_cnn.cuh"

using namespace dic;

namespace
{

const char* kVersion = "gb300-dic 0.1.0 (sm_103a)";

struct DicError
{
  int code;
  std::string msg;
};

#define DIC_CUDA(call)                                                                         \
  do                                                                                           \
  {                                                                                            \
    cudaError_t e_ = (call);                                                                   \
    if (e_ != cudaSuccess)                                                                     \
      throw DicError{DIC_ERR_CUDA, std::string(#call) + ": " + cudaGetErrorString(e_)};         \
  } while (0)

int dtype_size(int dtype)
{
  switch (dtype)
  {
    case DIC_U8: return 1;
    case DIC_U16: return 2;
    case DIC_F32: return 4;
    default: return 0;
  }
}

template <typename T>
struct DevBuf
{
  T* ptr = nullptr;
  size_t cap = 0;  // elements
  void ensure(size_t n)
  {
    if (n <= cap) return;
    if (ptr) cudaFree(ptr);
    ptr = nullptr;
    cap = 0;
    cudaError_t e = cudaMalloc(&ptr, std::max<size_t>(n, 1) * sizeof(T));
    if (e != cudaSuccess)
    {
      ptr = nullptr;
      throw DicError{DIC_ERR_MEMORY, std::string("cudaMalloc: ") + cudaGetErrorString(e)};
    }
    cap = n;
  }
  void release()
  {
    if (ptr) cudaFree(ptr);
    ptr = nullptr;
    cap = 0;
  }
};

std::mutex g_init_mutex;
std::set<int> g_initialized_devices;

void init_constants(int device)
{
  std::lock_guard<std::mutex> lock(g_init_mutex);
  if (g_initialized_devices.count(device)) return;
  const float bc[4][4] = DIC_BC_MATRIX;
  float bc2[256];
  for (int k = 0; k < 4; ++k)
    for (int l = 0; l < 4; ++l)
      for (int m = 0; m < 4; ++m)
        for (int n = 0; n < 4; ++n) bc2[((k * 4 + l) * 4 + m) * 4 + n] = bc[l][m] * bc[k][n];
  std::vector<float2> tw(kTwiddleCount);
  for (int N = 2; N <= kMaxTwiddleN; ++N)
    for (int k = 0; k < N; ++k)
    {
      const double a = -2.0 * M_PI * (double)k / (double)N;
      tw[tw_offset(N) + k] = make_float2((float)std::cos(a), (float)std::sin(a));
    }
  DIC_CUDA(cudaMemcpyToSymbol(c_bc2, bc2, sizeof(bc2)));
  DIC_CUDA(cudaMemcpyToSymbol(c_tw, tw.data(), sizeof(float2) * tw.size()));
  g_initialized_devices.insert(device);
}

enum Phase { kPhRef = 0, kPhPoi, kPhTar, kPhFftcc, kPhIcgn, kPhFrame, kPhProposal, kPhCount };

}  // namespace


// ======================================================================================
// Proposal network host side (see dic_cnn.cuh for the architecture and the kernels).
// ======================================================================================
struct dic_cnn
{
  int device = 0;
  cudaStream_t stream = nullptr;   // own stream; an engine borrows the network on its stream
  std::string last_error;
  DevBuf<float> params, grads, adam_m, adam_v, out, part, row_loss;
  DevBuf<__nv_bfloat16> wb, x0, a1, a2, a3, a4, a5, d1, d2, d3, d4, d5, dout;
  DevBuf<int> wait_err;   // k_proposal_fused's bounded tensor-core wait (bit 1)
  int64_t cap = 0;
  long long adam_t = 0;
  long long launches = 0;

  void check(const char* what)
  {
    ++launches;
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) throw DicError{DIC_ERR_CUDA, std::string(what) + ": " + cudaGetErrorString(e)};
  }

  void ensure_batch(int64_t n)
  {
    if (n <= cap) return;
    x0.ensure((size_t)n * 31 * 31 * 2);
    a1.ensure((size_t)n * 256 * 32); d1.ensure((size_t)n * 256 * 32);
    a2.ensure((size_t)n * 64 * 32);  d2.ensure((size_t)n * 64 * 32);
    a3.ensure((size_t)n * 16 * 32);  d3.ensure((size_t)n * 16 * 32);
    a4.ensure((size_t)n * 128);      d4.ensure((size_t)n * 128);
    a5.ensure((size_t)n * 256);      d5.ensure((size_t)n * 256);
    out.ensure((size_t)n * cnn::kOutPad);
    dout.ensure((size_t)n * cnn::kOutPad);
    row_loss.ensure((size_t)n);
    DIC_CUDA(cudaMemsetAsync(out.ptr, 0, sizeof(float) * n * cnn::kOutPad, stream));
    cap = n;
  }

  void pack()
  {
    const int n = cnn::kHidden * 128;
    cnn::k_pack_weights<<<(n + 255) / 256, 256, 0, stream>>>(params.ptr, wb.ptr);
    check("k_pack_weights");
  }

  template <class Op>
  void gemm(const Op& op, int64_t m_rows, int n_cols)
  {
    dim3 grid((unsigned)((m_rows + cnn::BM - 1) / cnn::BM), (unsigned)((n_cols + cnn::BN - 1) / cnn::BN),
              (unsigned)op.splits);
    cnn::k_gemm<Op><<<grid, 128, 0, stream>>>(op);
    check("k_gemm");
  }

  static int splits_for(int64_t k) { return (int)std::min<int64_t>(128, std::max<int64_t>(1, k / 2048)); }

  // Forward on x0 (already in this->x0 or given), batch n; logits into out [n][8].
  void forward(const __nv_bfloat16* in, int64_t n)
  {
    using L = cnn::WeightLayout;
    using P = cnn::ParamLayout;
    const __nv_bfloat16* acts_in[4] = {in, a1.ptr, a2.ptr, a3.ptr};
    __nv_bfloat16* acts_out[4] = {a1.ptr, a2.ptr, a3.ptr, a4.ptr};
    const int woff[4] = {L::c1, L::c2, L::c3, L::c4};
    const int boff[4] = {P::b1, P::b2, P::b3, P::b4};
    for (int l = 0; l < 4; ++l)
    {
      const int si = cnn::side_of(l), so = cnn::side_of(l + 1), ci = l == 0 ? 2 : 32;
      cnn::ConvFwdOp op;
      op.in = acts_in[l];
      op.w = wb.ptr + woff[l];
      op.bias = params.ptr + boff[l];
      op.out = acts_out[l];
      op.M = n * so * so;
      op.N = 32;
      op.splits = 1;
      op.kreal = 9 * ci;
      op.kpad = l == 0 ? cnn::kC1K : 288;
      op.K = op.kpad;
      op.si = si;
      op.so = so;
      op.ci = ci;
      gemm(op, op.M, 32);
    }
    cnn::LinearFwdOp f1{a4.ptr, wb.ptr + L::f1, params.ptr + P::b5, a5.ptr, nullptr, n, cnn::kHidden, 1, 128, 0};
    gemm(f1, n, cnn::kHidden);
    cnn::LinearFwdOp f2{a5.ptr, wb.ptr + L::f2, params.ptr + P::b6, nullptr, out.ptr, n, cnn::kOut, 1, cnn::kHidden,
                        cnn::kOutPad};
    gemm(f2, n, cnn::kOutPad);
  }

  void reduce_into(int splits, int rows, int cols, int keep, float* dst, int ld)
  {
    const int total = rows * keep;
    cnn::k_reduce_splits<<<(total + 255) / 256, 256, 0, stream>>>(part.ptr, splits, rows, cols, keep, dst, ld);
    check("k_reduce_splits");
  }

  void bias_grad(const __nv_bfloat16* dz, int64_t rows, int ld, int ncol, float* db)
  {
    cnn::k_bias_grad<<<ncol, 256, 0, stream>>>(dz, rows, ld, ncol, db);
    check("k_bias_grad");
  }

  // Backward after forward(in, n) with targets [n][6]; gradients into grads (param layout).
  void backward(const __nv_bfloat16* in, const float* target, int64_t n)
  {
    using L = cnn::WeightLayout;
    using P = cnn::ParamLayout;
    cnn::k_loss_grad<<<(unsigned)((n + 255) / 256), 256, 0, stream>>>(out.ptr, target, n, dout.ptr, row_loss.ptr);
    check("k_loss_grad");
    // f2
    {
      const int S = splits_for(n);
      cnn::LinearBwdWeightOp op{dout.ptr, a5.ptr, part.ptr, cnn::kOut, cnn::kHidden, S, n, cnn::kOutPad};
      gemm(op, cnn::kOut, cnn::kHidden);
      reduce_into(S, cnn::kOut, cnn::kHidden, cnn::kHidden, grads.ptr + P::w6, cnn::kHidden);
      bias_grad(dout.ptr, n, cnn::kOutPad, cnn::kOut, grads.ptr + P::b6);
      cnn::LinearBwdDataOp dop{dout.ptr, wb.ptr + L::f2, a5.ptr, d5.ptr, n, cnn::kHidden, 1, cnn::kOut, cnn::kOutPad};
      gemm(dop, n, cnn::kHidden);
    }
    // f1
    {
      const int S = splits_for(n);
      cnn::LinearBwdWeightOp op{d5.ptr, a4.ptr, part.ptr, cnn::kHidden, 128, S, n, cnn::kHidden};
      gemm(op, cnn::kHidden, 128);
      reduce_into(S, cnn::kHidden, 128, 128, grads.ptr + P::w5, 128);
      bias_grad(d5.ptr, n, cnn::kHidden, cnn::kHidden, grads.ptr + P::b5);
      cnn::LinearBwdDataOp dop{d5.ptr, wb.ptr + L::f1, a4.ptr, d4.ptr, n, 128, 1, cnn::kHidden, cnn::kHidden};
      gemm(dop, n, 128);
    }
    // conv4 .. conv1
    const __nv_bfloat16* acts_in[4] = {in, a1.ptr, a2.ptr, a3.ptr};
    __nv_bfloat16* dz_out[4] = {d1.ptr, d2.ptr, d3.ptr, d4.ptr};
    const int woff[4] = {L::c1, L::c2, L::c3, L::c4};
    const int wpo[4] = {P::w1, P::w2, P::w3, P::w4};
    const int bpo[4] = {P::b1, P::b2, P::b3, P::b4};
    for (int l = 3; l >= 0; --l)
    {
      const int si = cnn::side_of(l), so = cnn::side_of(l + 1), ci = l == 0 ? 2 : 32;
      const int kreal = 9 * ci, kpad = l == 0 ? cnn::kC1K : 288;
      const int64_t K = n * so * so;
      const int S = splits_for(K);
      cnn::ConvBwdWeightOp wop{dz_out[l], acts_in[l], part.ptr, 32, kpad, S, K, si, so, ci, 32, kreal, kpad};
      gemm(wop, 32, kpad);
      reduce_into(S, 32, kpad, kreal, grads.ptr + wpo[l], kreal);
      bias_grad(dz_out[l], K, 32, 32, grads.ptr + bpo[l]);
      if (l > 0)
      {
        cnn::ConvBwdDataOp dop{dz_out[l], wb.ptr + woff[l], acts_in[l], dz_out[l - 1], n * si * si, ci, 1, 9 * 32,
                               si, so, ci, 32, kpad};
        gemm(dop, n * si * si, ci);
      }
    }
  }

  float loss(int64_t n)
  {
    std::vector<float> h((size_t)n);
    DIC_CUDA(cudaMemcpyAsync(h.data(), row_loss.ptr, sizeof(float) * n, cudaMemcpyDeviceToHost, stream));
    DIC_CUDA(cudaStreamSynchronize(stream));
    double s = 0.0;
    for (float v : h) s += v;
    return (float)(s / ((double)n * cnn::kOut));
  }
};

struct dic_engine
{
  dic_config cfg{};
  cudaStream_t stream = nullptr;
  std::string last_error;

  int w = 0, h = 0;
  int ref_dtype = 0, tar_dtype = 0;
  bool ref_set = false, tar_set = false;
  bool ref_dirty = true, tar_dirty = true;
  DevBuf<unsigned char> raw_ref, raw_tar;
  DevBuf<float> ref_f32, tar_f32;
  DevBuf<float4> ref_pack, coef;
  DevBuf<float> lattice;   // coefficient [0][0] of every texel (the integer-translation fast path)

  // prepared layout
  std::vector<int> layout_x, layout_y;   // host copy of a host-defined layout
  bool layout_ready = false;
  int64_t layout_count = 0;
  DevBuf<PoiRef> poi_ref;
  DevBuf<dic_poi> queue;
  DevBuf<int64_t> slots;
  DevBuf<unsigned long long> counters;

  // Per-phase CUDA events; a phase launched several times in one call (the learned path's
  // two IC-GN passes) reports the sum of its launches.
  static constexpr int kMarks = 8;
  bool timing = true;
  cudaEvent_t ev[kPhCount][kMarks][2] = {};
  int ev_used[kPhCount] = {};
  bool ev_pending[kPhCount] = {};
  double ms[kPhCount] = {};
  long long launches = 0;
  long long icgn_pois = 0;
  bool iter_pending = false;
  unsigned long long iter_sum = 0;

  void check_launch(const char* what)
  {
    ++launches;
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) throw DicError{DIC_ERR_CUDA, std::string(what) + ": " + cudaGetErrorString(e)};
  }
  void mark(int ph, int which)
  {
    if (!timing || ev_used[ph] >= kMarks) return;
    DIC_CUDA(cudaEventRecord(ev[ph][ev_used[ph]][which], stream));
    if (which == 1)
    {
      ++ev_used[ph];
      ev_pending[ph] = true;
    }
  }
  // A new API call starts a new measurement (pending events of the previous call are dropped).
  void begin_call()
  {
    for (int p = 0; p < kPhCount; ++p) ev_used[p] = 0;
  }
  void harvest()
  {
    for (int p = 0; p < kPhCount; ++p)
      if (ev_pending[p])
      {
        double tot = 0.0;
        for (int k = 0; k < ev_used[p]; ++k)
        {
          float t = 0.f;
          DIC_CUDA(cudaEventSynchronize(ev[p][k][1]));
          DIC_CUDA(cudaEventElapsedTime(&t, ev[p][k][0], ev[p][k][1]));
          tot += t;
        }
        ms[p] = tot;
        ev_pending[p] = false;
      }
    if (iter_pending)
    {
      DIC_CUDA(cudaMemcpyAsync(&iter_sum, counters.ptr, sizeof(unsigned long long), cudaMemcpyDeviceToHost, stream));
      DIC_CUDA(cudaStreamSynchronize(stream));
      iter_pending = false;
      check_wait_error();
    }
  }

  // ---------------------------------------------------------------- images
  // The solvers index texels with 32-bit products (y * w + x): images stay below 2^31 pixels
  // (the B-spline table alone would then be 128 GiB).
  static void check_pixel_count(int width, int height)
  {
    if ((int64_t)width * height >= ((int64_t)1 << 31))
      throw DicError{DIC_ERR_ARGUMENT, "image: 2^31 pixels or more (texel indices are 32-bit)"};
  }
  void set_image(bool is_ref, const void* px, int width, int height, int64_t stride, int dtype, bool device)
  {
    const int es = dtype_size(dtype);
    if (!px || es == 0 || width < 5 || height < 5)
      throw DicError{DIC_ERR_ARGUMENT, "image: null pixels, unknown dtype or size below 5x5"};
    if (stride < (int64_t)width * es) throw DicError{DIC_ERR_ARGUMENT, "image: row stride smaller than a row"};
    check_pixel_count(width, height);
    const bool other_set = is_ref ? tar_set : ref_set;
    if (other_set && (width != w || height != h))
    {
      // A new size invalidates the other image; the caller must set it again.
      if (is_ref) tar_set = false; else ref_set = false;
    }
    if (w != width || h != height) layout_ready = false;
    w = width;
    h = height;
    auto& raw = is_ref ? raw_ref : raw_tar;
    raw.ensure((size_t)width * height * es);
    DIC_CUDA(cudaMemcpy2DAsync(raw.ptr, (size_t)width * es, px, (size_t)stride, (size_t)width * es, height,
                               device ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice, stream));
    if (is_ref)
    {
      ref_dtype = dtype;
      ref_set = true;
      ref_dirty = true;
      layout_ready = false;   // setRefImage invalidates the prepared layout's data
    }
    else
    {
      tar_dtype = dtype;
      tar_set = true;
      tar_dirty = true;
    }
  }

  float scale() const { return cfg.input_scale == 0.f ? 1.f : cfg.input_scale; }

  template <typename T>
  void launch_prepare_ref()
  {
    dim3 grid((w + kPrepTile - 1) / kPrepTile, (h + kPrepTile - 1) / kPrepTile);
    k_prepare_ref<T><<<grid, 256, 0, stream>>>(reinterpret_cast<const T*>(raw_ref.ptr), w, h, scale(),
                                               ref_f32.ptr, ref_pack.ptr);
    check_launch("k_prepare_ref");
  }
  template <typename T>
  void launch_prepare_tar(bool table, bool pitched)
  {
    dim3 grid((w + kPrepTile - 1) / kPrepTile, (h + kPrepTile - 1) / kPrepTile);
    k_prepare_tar<T><<<grid, 256, 0, stream>>>(reinterpret_cast<const T*>(raw_tar.ptr), w, h, scale(),
                                               tar_f32.ptr, table ? coef.ptr : nullptr, lattice.ptr,
                                               pitched ? tar_px.ptr : nullptr, px_pitch(w));
    check_launch("k_prepare_tar");
  }

  void ensure_ref()
  {
    if (!ref_set) throw DicError{DIC_ERR_STATE, "reference image must be set first"};
    if (!ref_dirty) return;
    const size_t px = (size_t)w * h;
    ref_f32.ensure(px);
    ref_pack.ensure(px);
    mark(kPhRef, 0);
    switch (ref_dtype)
    {
      case DIC_U8: launch_prepare_ref<uint8_t>(); break;
      case DIC_U16: launch_prepare_ref<uint16_t>(); break;
      default: launch_prepare_ref<float>(); break;
    }
    mark(kPhRef, 1);
    ref_dirty = false;
  }
  // Sampling of the target in IC-GN (DIC_SAMPLE_*): the B-spline coefficient table, or the
  // pixels themselves (column and pair walks; the flat walk keeps the table).
  int sampling = DIC_SAMPLE_PIXELS;
  bool pixel_radius(int rx) const { return sampling == DIC_SAMPLE_PIXELS && walk_of(rx) != kWalkFlat; }
  bool pixel_walk() const { return pixel_radius(cfg.subset_radius_x); }
  // the launch kind (shape slot) of a radius's IC-GN under the current sampling
  int icgn_walk(int rx) const
  {
    const int wk = walk_of(rx);
    if (!pixel_radius(rx)) return wk;
    return wk == kWalkColumn ? kWalkColumnPx : kWalkPairPx;
  }
  bool table_ready = false;   // coef / lattice hold the current target's table
  // Pixel sampling stages windows by TMA, whose rows must start on 16-byte boundaries: where W
  // is not a multiple of 4 floats the target is also written with a padded pitch (tar_px).
  DevBuf<float> tar_px;
  bool px_ready = false;       // tar_px holds the current target
  bool pitched_target() const { return pixel_walk() && (w & 3) != 0; }
  const float* px_plane() const { return pitched_target() ? tar_px.ptr : tar_f32.ptr; }
  // The target's float plane, plus its coefficient table when IC-GN samples the table (or
  // `table` asks for it), plus the padded-pitch plane pixel sampling needs for odd widths.
  void ensure_tar(bool table = false)
  {
    if (!tar_set) throw DicError{DIC_ERR_STATE, "target image must be set first"};
    if (!ref_set) throw DicError{DIC_ERR_STATE, "reference image must be set first"};
    table = table || !pixel_walk();
    const bool pitched = pitched_target();
    if (!tar_dirty && (table_ready || !table) && (px_ready || !pitched)) return;
    const size_t px = (size_t)w * h;
    tar_f32.ensure(px);
    if (table)
    {
      coef.ensure(px * 4);
      lattice.ensure(px);
    }
    if (pitched) tar_px.ensure((size_t)px_pitch(w) * h);
    mark(kPhTar, 0);
    switch (tar_dtype)
    {
      case DIC_U8: launch_prepare_tar<uint8_t>(table, pitched); break;
      case DIC_U16: launch_prepare_tar<uint16_t>(table, pitched); break;
      default: launch_prepare_tar<float>(table, pitched); break;
    }
    mark(kPhTar, 1);
    tar_dirty = false;
    table_ready = table;
    px_ready = pitched;
  }

  // ---------------------------------------------------------------- layout
  void upload_queue(const dic_poi* pois, int64_t n)
  {
    queue.ensure((size_t)n);
    DIC_CUDA(cudaMemcpyAsync(queue.ptr, pois, sizeof(dic_poi) * n, cudaMemcpyHostToDevice, stream));
  }
  // The pair path's queue upload on a side stream, so that it overlaps the reference and
  // target preparation kernels enqueued after it: the side stream first waits for all
  // earlier engine-stream work (nothing still reading the queue is overtaken), and
  // join_queue_upload makes the engine stream wait for the copy before the solvers.
  cudaStream_t qup_stream = nullptr;
  cudaEvent_t qup_before = nullptr, qup_done = nullptr;
  void upload_queue_beside(const dic_poi* pois, int64_t n)
  {
    queue.ensure((size_t)n);
    if (!qup_stream)
    {
      DIC_CUDA(cudaStreamCreateWithFlags(&qup_stream, cudaStreamNonBlocking));
      DIC_CUDA(cudaEventCreateWithFlags(&qup_before, cudaEventDisableTiming));
      DIC_CUDA(cudaEventCreateWithFlags(&qup_done, cudaEventDisableTiming));
    }
    DIC_CUDA(cudaEventRecord(qup_before, stream));
    DIC_CUDA(cudaStreamWaitEvent(qup_stream, qup_before, 0));
    DIC_CUDA(cudaMemcpyAsync(queue.ptr, pois, sizeof(dic_poi) * n, cudaMemcpyHostToDevice, qup_stream));
    DIC_CUDA(cudaEventRecord(qup_done, qup_stream));
  }
  void join_queue_upload() { DIC_CUDA(cudaStreamWaitEvent(stream, qup_done, 0)); }
  void release_queue_upload()
  {
    if (qup_stream)
    {
      cudaStreamSynchronize(qup_stream);
      cudaStreamDestroy(qup_stream);
    }
    if (qup_before) cudaEventDestroy(qup_before);
    if (qup_done) cudaEventDestroy(qup_done);
    qup_stream = nullptr;
    qup_before = qup_done = nullptr;
  }
  void download_queue(dic_poi* pois, int64_t n)
  {
    DIC_CUDA(cudaMemcpyAsync(pois, queue.ptr, sizeof(dic_poi) * n, cudaMemcpyDeviceToHost, stream));
    DIC_CUDA(cudaStreamSynchronize(stream));
    check_wait_error();
  }
  bool layout_matches(const dic_poi* pois, int64_t n) const
  {
    if (!layout_ready || (int64_t)layout_x.size() != n) return false;
    for (int64_t i = 0; i < n; ++i)
      if (layout_x[i] != (int)pois[i].x || layout_y[i] != (int)pois[i].y) return false;
    return true;
  }
  void record_layout(const dic_poi* pois, int64_t n)
  {
    layout_x.resize(n);
    layout_y.resize(n);
    for (int64_t i = 0; i < n; ++i)
    {
      layout_x[i] = (int)pois[i].x;
      layout_y[i] = (int)pois[i].y;
    }
  }
  // Per-POI reference data for the POIs currently in `src` (device records).
  void prepare_layout_device(const dic_poi* src, int64_t n)
  {
    ensure_ref();
    poi_ref.ensure((size_t)std::max<int64_t>(n, 1));
    if (n > 0)
    {
      mark(kPhPoi, 0);
      const unsigned blocks = (unsigned)((n + kPrepPois - 1) / kPrepPois);
      k_poi_prepare32<<<blocks, kPrepWarps * 32, 0, stream>>>(ref_pack.ptr, w, h, src, n, cfg.subset_radius_x,
                                                              cfg.subset_radius_y, poi_ref.ptr);
      check_launch("k_poi_prepare32");
      mark(kPhPoi, 1);
    }
    layout_ready = true;
    layout_count = n;
  }

  // ---------------------------------------------------------------- launch shapes
  // What can be tuned: how many warps a CTA holds (2, 4 or 8), one CTA per group of POIs or
  // a persistent launch (and, for the batch kernel, how many CTAs per SM), the staging tile
  // (column walk) and the warps per POI (pair walk: 1 or 2).  Per-POI results depend on
  // none of them.  shape[batch][walk]: batch 0 single queues, 1 batches; walk kWalkFlat,
  // kWalkColumn, kWalkPair.
  struct IcgnShape
  {
    int warps = 4;
    int ctas_per_sm = 7;     // persistent launches: resident CTAs per SM (0: one CTA per kWarps POIs)
    float ms = 0.f;
    int tile = 0;            // column walk: 0 gathers from the table; 1, 2: k_icgn_tile (kTileKinds)
    int poi_warps = 1;       // pair walk: warps per POI
  };
  static constexpr int kWalkFlat = 0, kWalkColumn = 1, kWalkPair = 2;
  // the column and pair walks' launches under pixel sampling (k_icgn_px, k_icgn_pair_px and
  // their batch forms), tuned separately
  static constexpr int kWalkColumnPx = 3, kWalkPairPx = 4, kWalks = 5;
  // the subset walk of a radius: column walk up to 32 columns, pair walk up to 64, else flat
  static int walk_of(int rx)
  {
    const int sw = 2 * rx + 1;
    return sw <= 32 ? kWalkColumn : sw <= kPairMaxWidth ? kWalkPair : kWalkFlat;
  }
  // TMA-staged tile forms: POIs (warps) per CTA, block width and height in texels, CTAs per SM
  // (shared memory: 2 planes x 32 B per texel, 110.7 KB and 163.9 KB)
  struct TileKind
  {
    int warps, bx, by, ctas;
  };
  static constexpr TileKind kTileKinds[3] = {{0, 0, 0, 0}, {4, 48, 36, 2}, {8, 64, 40, 1}};
  // cuTensorMapEncodeTiled through the runtime's driver entry point (no link against libcuda)
  using EncodeTiledFn = CUresult (*)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*, const cuuint64_t*,
                                     const cuuint64_t*, const cuuint32_t*, const cuuint32_t*, CUtensorMapInterleave,
                                     CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);
  static EncodeTiledFn encode_tiled()
  {
    static EncodeTiledFn fn = nullptr;
    static std::once_flag once;
    std::call_once(once, [] {
      void* f = nullptr;
      cudaDriverEntryPointQueryResult q{};
      if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &f, 12000, cudaEnableDefault, &q) == cudaSuccess &&
          q == cudaDriverEntryPointSuccess)
        fn = reinterpret_cast<EncodeTiledFn>(f);
      else
        cudaGetLastError();
    });
    return fn;
  }
  struct TileMap
  {
    alignas(128) CUtensorMap map;
    const void* base = nullptr;
    int w = 0, h = 0, bx = 0, by = 0, pitch = 0;
  };
  TileMap tile_maps[3];
  // Bounded waits inside kernels report here instead of hanging: bit 0, a k_icgn_tile CTA
  // whose TMA copy did not arrive in time; bit 1, a k_proposal_fused warp group whose
  // tensor-core products did not complete in time.
  DevBuf<int> wait_err;
  bool wait_pending = false;   // a launch that can set wait_err since the last check
  // Timeout-path test hook, read once at engine creation from DIC_TEST_WAIT_FAULT: bit 0,
  // k_icgn_tile arms its copy wait but never issues the copy; bit 1, k_proposal_fused never
  // issues conv2's products.  Either wait then runs out after kTestWaitPolls polls, the
  // kernel reports through wait_err, and the call fails with DIC_ERR_CUDA.  Nothing faults:
  // no copy or product is left in flight.
  static constexpr uint32_t kTestWaitPolls = 1u << 12;
  int wait_test = 0;
  uint32_t wait_polls = kWaitPolls;
  int* wait_flag()
  {
    if (!wait_err.ptr)
    {
      wait_err.ensure(1);
      DIC_CUDA(cudaMemsetAsync(wait_err.ptr, 0, sizeof(int), stream));
    }
    wait_pending = true;
    return wait_err.ptr;
  }
  // the 4-D map {component, x, y, plane} of a coefficient table (8 floats per texel and
  // plane, 2 planes), box {8, bx, by, 2}
  const CUtensorMap& coef_map(int kind, const float4* table, int tw, int th)
  {
    TileMap& m = tile_maps[kind];
    if (m.base == table && m.w == tw && m.h == th) return m.map;
    EncodeTiledFn fn = encode_tiled();
    if (!fn) throw DicError{DIC_ERR_CUDA, "cuTensorMapEncodeTiled is not available from the driver"};
    const TileKind& k = kTileKinds[kind];
    constexpr cuuint64_t texel = 2 * sizeof(float4);
    const cuuint64_t dims[4] = {8, (cuuint64_t)tw, (cuuint64_t)th, 2};
    const cuuint64_t strides[3] = {texel, texel * (cuuint64_t)tw, texel * (cuuint64_t)tw * (cuuint64_t)th};
    const cuuint32_t box[4] = {8, (cuuint32_t)k.bx, (cuuint32_t)k.by, 2};
    const cuuint32_t estr[4] = {1, 1, 1, 1};
    const CUresult r = fn(&m.map, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 4, const_cast<float4*>(table), dims, strides, box, estr,
                          CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                          CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (r != CUDA_SUCCESS)
    {
      m.base = nullptr;
      throw DicError{DIC_ERR_CUDA, "cuTensorMapEncodeTiled failed (" + std::to_string((int)r) + ")"};
    }
    m.base = table;
    m.w = tw;
    m.h = th;
    return m.map;
  }
  static std::string wait_error_text(int flag)
  {
    std::string t = (flag & 1) ? "k_icgn_tile / k_icgn_px: a TMA tile copy did not complete in time" : "";
    if (flag & 2) t += std::string(t.empty() ? "" : "; ") + "k_proposal_fused: a tensor-core product did not complete in time";
    return t + "; results are invalid";
  }
  // after a synchronisation: a launch whose bounded wait ran out makes its results invalid
  void check_wait_error()
  {
    if (!wait_pending) return;
    wait_pending = false;
    int flag = 0;
    DIC_CUDA(cudaMemcpyAsync(&flag, wait_err.ptr, sizeof(int), cudaMemcpyDeviceToHost, stream));
    DIC_CUDA(cudaStreamSynchronize(stream));
    if (flag)
    {
      DIC_CUDA(cudaMemsetAsync(wait_err.ptr, 0, sizeof(int), stream));
      throw DicError{DIC_ERR_CUDA, wait_error_text(flag)};
    }
  }
  static constexpr int64_t kTuneMinPois = 2048;
  bool autotune = false;
  // Untuned default: the persistent form for single queues too (8 CTAs of 4 warps: its
  // 32-warp residency).  The grid form of the column walk (k_icgn<1, 4>) spills a register
  // inside its row loop under the 7-CTA register cap (a local store and load per row: 14 %
  // of its L1 wavefronts on the 2048² pair, 3.73 ms against 3.59 ms persistent with the
  // four-plane table); the autotuner still times both forms.  shape[0]: single queues,
  // shape[1]: batches.
  // The pixel pair walk's default (2 warps per CTA, 2 per POI, TMA windows) is its fastest
  // measured form on the 2048² pair at r 20 and 30 (5.84 and 8.05 ms; 4 warps per CTA 7.15 and
  // 11.8, 8 warps 7.16 and 12.6, one warp per POI 6.9 and 17.1).
  IcgnShape shape[2][kWalks] = {{{4, 8, 0.f}, {4, 8, 0.f}, {4, 8, 0.f}, {4, 0, 0.f, 1}, {2, 0, 0.f, 1, 2}},
                                {{4, 7, 0.f}, {4, 7, 0.f}, {4, 7, 0.f}, {4, 7, 0.f}, {2, 0, 0.f, 0, 2}}};
  bool tuned[2][kWalks] = {};
  DevBuf<dic_poi> tune_q;
  cudaEvent_t tune_ev[2] = {};

  bool capturing()
  {
    cudaStreamCaptureStatus st = cudaStreamCaptureStatusNone;
    DIC_CUDA(cudaStreamIsCapturing(stream, &st));
    return st != cudaStreamCaptureStatusNone;
  }
  template <bool C, int W>
  static int max_ctas(bool persistent)
  {
    int b = 0;
    if (persistent)
      DIC_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, k_icgn_batch<C, W>, W * 32, 0));
    else
      DIC_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, k_icgn<C, W>, W * 32, 0));
    return std::max(b, 1);
  }
  template <bool C, int W>
  static int max_ctas_single()
  {
    int b = 0;
    DIC_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, k_icgn_persistent<C, W>, W * 32, 0));
    return std::max(b, 1);
  }
  static int occupancy_single(bool column, int warps)
  {
    if (column) return warps == 2 ? max_ctas_single<true, 2>() : warps == 8 ? max_ctas_single<true, 8>()
                                                                             : max_ctas_single<true, 4>();
    return warps == 2 ? max_ctas_single<false, 2>() : warps == 8 ? max_ctas_single<false, 8>()
                                                                  : max_ctas_single<false, 4>();
  }
  template <int PW, int W>
  static int max_ctas_pair(bool batch)
  {
    int b = 0;
    if (batch)
      DIC_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, k_icgn_batch_pair<PW, W>, W * 32, 0));
    else
      DIC_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, k_icgn_pair_persistent<PW, W>, W * 32, 0));
    return std::max(b, 1);
  }
  static int occupancy_pair(bool batch, int poi_warps, int warps)
  {
    if (poi_warps == 2)
      return warps == 2 ? max_ctas_pair<2, 2>(batch) : warps == 8 ? max_ctas_pair<2, 8>(batch) : max_ctas_pair<2, 4>(batch);
    return warps == 2 ? max_ctas_pair<1, 2>(batch) : warps == 8 ? max_ctas_pair<1, 8>(batch) : max_ctas_pair<1, 4>(batch);
  }
  static int occupancy(bool persistent, bool column, int warps)
  {
    if (column) return warps == 2 ? max_ctas<true, 2>(persistent) : warps == 8 ? max_ctas<true, 8>(persistent)
                                                                                : max_ctas<true, 4>(persistent);
    return warps == 2 ? max_ctas<false, 2>(persistent) : warps == 8 ? max_ctas<false, 8>(persistent)
                                                                     : max_ctas<false, 4>(persistent);
  }
  DevBuf<unsigned long long> icgn_next;   // work counter of the persistent single-queue launch

  // k_icgn_px: dynamic shared memory of one CTA (the warps' windows plus alignment room)
  static size_t px_smem(int warps, int rx, int ry) { return 128 + (size_t)warps * px_window_bytes(rx, ry); }
  // the shared-memory opt-in of the three k_icgn_px widths (per engine, so per device): the
  // device's per-block maximum, set once outside any capture
  bool px_attr_set = false;
  void px_attributes()
  {
    if (px_attr_set) return;
    int optin = 0;
    DIC_CUDA(cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, cfg.device));
    auto opt_in = [optin](const void* k) {
      cudaFuncAttributes fa{};
      DIC_CUDA(cudaFuncGetAttributes(&fa, k));   // the dynamic maximum leaves room for the static part
      DIC_CUDA(cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, optin - (int)fa.sharedSizeBytes));
    };
    opt_in((const void*)k_icgn_px<2, 2>);
    opt_in((const void*)k_icgn_px<4, 2>);
    opt_in((const void*)k_icgn_px<8, 2>);
    opt_in((const void*)k_icgn_px<2, 1>);
    opt_in((const void*)k_icgn_px<4, 1>);
    opt_in((const void*)k_icgn_px<8, 1>);
    opt_in((const void*)k_icgn_batch_px<2, 2>);
    opt_in((const void*)k_icgn_batch_px<4, 2>);
    opt_in((const void*)k_icgn_batch_px<8, 2>);
    opt_in((const void*)k_icgn_batch_px<2, 1>);
    opt_in((const void*)k_icgn_batch_px<4, 1>);
    opt_in((const void*)k_icgn_batch_px<8, 1>);
#define DIC_PAIR_PX_OPT(PW, W)                                \
  opt_in((const void*)k_icgn_pair_px<PW, W, 2>);              \
  opt_in((const void*)k_icgn_pair_px<PW, W, 1>);              \
  opt_in((const void*)k_icgn_batch_pair_px<PW, W, 2>)
    DIC_PAIR_PX_OPT(1, 2);
    DIC_PAIR_PX_OPT(1, 4);
    DIC_PAIR_PX_OPT(1, 8);
    DIC_PAIR_PX_OPT(2, 2);
    DIC_PAIR_PX_OPT(2, 4);
    DIC_PAIR_PX_OPT(2, 8);
#undef DIC_PAIR_PX_OPT
    px_attr_set = true;
  }
  template <int W>
  static int max_ctas_px(size_t smem)
  {
    int b = 0;
    if (smem)
      DIC_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, k_icgn_px<W, 2>, W * 32, smem));
    else
      DIC_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, k_icgn_px<W, 0>, W * 32, smem));
    return b;
  }
  int occupancy_batch_px(int warps, size_t smem)
  {
    px_attributes();
    int b = 0;
    if (warps == 2) DIC_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, k_icgn_batch_px<2, 2>, 64, smem));
    else if (warps == 8) DIC_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, k_icgn_batch_px<8, 2>, 256, smem));
    else DIC_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, k_icgn_batch_px<4, 2>, 128, smem));
    if (b < 1) throw DicError{DIC_ERR_ARGUMENT, "IC-GN pixel windows of this subset radius do not fit in shared memory"};
    return b;
  }
  // resident CTAs per SM of a k_icgn_px width, cached per (warps, staged, radius)
  struct PxOcc
  {
    int warps = 0, staged = 0, rx = -1, ry = -1, ctas = 0;
  };
  PxOcc px_occ[6];
  int occupancy_px(int warps, bool staged, int rx, int ry)
  {
    const int slot = (warps == 2 ? 0 : warps == 4 ? 1 : 2) * 2 + (staged ? 1 : 0);
    PxOcc& o = px_occ[slot];
    if (o.warps == warps && o.rx == rx && o.ry == ry) return o.ctas;
    px_attributes();
    const size_t smem = staged ? px_smem(warps, rx, ry) : 0;
    const int b = warps == 2 ? max_ctas_px<2>(smem) : warps == 8 ? max_ctas_px<8>(smem) : max_ctas_px<4>(smem);
    if (b < 1) throw DicError{DIC_ERR_ARGUMENT, "IC-GN pixel windows of this subset radius do not fit in shared memory"};
    o = PxOcc{warps, staged ? 1 : 0, rx, ry, b};
    return b;
  }
  // the 2-D map {x, y} of the target plane, box {bx, by} (only for rows of a multiple of 16 bytes)
  TileMap px_map;
  const CUtensorMap* tar_map(const float* plane, int tw, int th, int pitch, int bx, int by)
  {
    if ((pitch * sizeof(float)) % 16 != 0) return nullptr;
    EncodeTiledFn fn = encode_tiled();
    if (!fn) return nullptr;
    TileMap& m = px_map;
    if (m.base == plane && m.w == tw && m.h == th && m.pitch == pitch && m.bx == bx && m.by == by) return &m.map;
    const cuuint64_t dims[2] = {(cuuint64_t)tw, (cuuint64_t)th};
    const cuuint64_t strides[1] = {(cuuint64_t)pitch * sizeof(float)};
    const cuuint32_t box[2] = {(cuuint32_t)bx, (cuuint32_t)by};
    const cuuint32_t estr[2] = {1, 1};
    const CUresult r = fn(&m.map, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 2, const_cast<float*>(plane), dims, strides, box, estr,
                          CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
                          CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (r != CUDA_SUCCESS)
    {
      m.base = nullptr;
      throw DicError{DIC_ERR_CUDA, "cuTensorMapEncodeTiled failed (" + std::to_string((int)r) + ")"};
    }
    m.base = plane;
    m.w = tw;
    m.h = th;
    m.pitch = pitch;
    m.bx = bx;
    m.by = by;
    return &m.map;
  }
  // shape.tile: 1 stages each POI's pixel window in shared memory by TMA (by warp copies where
  // the plane's row pitch is not a multiple of 16 bytes), 2 by warp copies, 0 reads the global plane
  void launch_px(const IcgnParams& p, const IcgnShape& sh)
  {
    icgn_next.ensure(1);
    DIC_CUDA(cudaMemsetAsync(icgn_next.ptr, 0, sizeof(unsigned long long), stream));
    int sms = 0;
    DIC_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, cfg.device));
    const int warps = sh.warps;
    px_attributes();
    const size_t smem = sh.tile ? px_smem(warps, p.rx, p.ry) : 0;
    const int ctas = sh.ctas_per_sm > 0 ? sh.ctas_per_sm : occupancy_px(warps, sh.tile != 0, p.rx, p.ry);
    const unsigned grid = (unsigned)std::max<int64_t>(1, std::min<int64_t>((int64_t)sms * ctas, (p.n + warps - 1) / warps));
    const CUtensorMap* m =
        sh.tile == 1 ? tar_map(p.tar, p.w, p.h, px_pitch(p.w), px_window_x(p.rx), px_window_y(p.ry)) : nullptr;
    CUtensorMap none{};
    IcgnParams q = p;
    q.wait_polls = wait_polls;
    q.wait_test = wait_test & 1;
    const int mode = sh.tile ? (m ? 2 : 1) : 0;   // 2: TMA, 1: warp copies, 0: no window
#define DIC_PX_LAUNCH(W, M) k_icgn_px<W, M><<<grid, W * 32, smem, stream>>>(q, m ? *m : none, icgn_next.ptr, wait_flag())
#define DIC_PX_MODES(W)                       \
  do                                          \
  {                                           \
    if (mode == 2) DIC_PX_LAUNCH(W, 2);      \
    else if (mode == 1) DIC_PX_LAUNCH(W, 1); \
    else DIC_PX_LAUNCH(W, 0);                 \
  } while (0)
    if (warps == 2) DIC_PX_MODES(2);
    else if (warps == 8) DIC_PX_MODES(8);
    else DIC_PX_MODES(4);
#undef DIC_PX_MODES
#undef DIC_PX_LAUNCH
  }
  // Pair walk under pixel sampling: the dynamic shared memory of one CTA (a window per POI slot)
  // and its resident CTAs per SM (cached per form, width and size).
  static size_t pair_px_smem(int warps, int poi_warps, size_t win) { return 128 + (size_t)(warps / poi_warps) * win; }
  template <int PW, int W>
  static int max_ctas_pair_px(bool batch, size_t smem)
  {
    int b = 0;
    if (batch)
      DIC_CUDA(smem ? cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, k_icgn_batch_pair_px<PW, W, 2>, W * 32, smem)
                    : cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, k_icgn_batch_pair_px<PW, W, 0>, W * 32, 0));
    else
      DIC_CUDA(smem ? cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, k_icgn_pair_px<PW, W, 2>, W * 32, smem)
                    : cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, k_icgn_pair_px<PW, W, 0>, W * 32, 0));
    return b;
  }
  struct PairPxOcc
  {
    int batch, poi_warps, warps;
    size_t smem;
    int ctas;
  };
  std::vector<PairPxOcc> pair_px_occ;
  int occupancy_pair_px(bool batch, int poi_warps, int warps, size_t smem)
  {
    for (const PairPxOcc& o : pair_px_occ)
      if (o.batch == (batch ? 1 : 0) && o.poi_warps == poi_warps && o.warps == warps && o.smem == smem) return o.ctas;
    px_attributes();
    int b;
    if (poi_warps == 2)
      b = warps == 2 ? max_ctas_pair_px<2, 2>(batch, smem) : warps == 8 ? max_ctas_pair_px<2, 8>(batch, smem)
                                                                           : max_ctas_pair_px<2, 4>(batch, smem);
    else
      b = warps == 2 ? max_ctas_pair_px<1, 2>(batch, smem) : warps == 8 ? max_ctas_pair_px<1, 8>(batch, smem)
                                                                           : max_ctas_pair_px<1, 4>(batch, smem);
    if (b < 1) throw DicError{DIC_ERR_ARGUMENT, "IC-GN pixel windows of this subset radius do not fit in shared memory"};
    pair_px_occ.push_back(PairPxOcc{batch ? 1 : 0, poi_warps, warps, smem, b});
    return b;
  }
  // shape.tile as in launch_px: 1 TMA windows (warp copies where no map), 2 warp copies, 0 none;
  // shape.poi_warps 1 or 2
  void launch_pair_px(const IcgnParams& p, const IcgnShape& sh)
  {
    icgn_next.ensure(1);
    DIC_CUDA(cudaMemsetAsync(icgn_next.ptr, 0, sizeof(unsigned long long), stream));
    int sms = 0;
    DIC_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, cfg.device));
    const int warps = sh.warps, pw = sh.poi_warps == 2 ? 2 : 1, slots = warps / pw;
    px_attributes();
    const size_t smem = sh.tile ? pair_px_smem(warps, pw, px_window_bytes(p.rx, p.ry)) : 0;
    const int ctas = sh.ctas_per_sm > 0 ? sh.ctas_per_sm : occupancy_pair_px(false, pw, warps, smem);
    const unsigned grid = (unsigned)std::max<int64_t>(1, std::min<int64_t>((int64_t)sms * ctas, (p.n + slots - 1) / slots));
    const CUtensorMap* m =
        sh.tile == 1 ? tar_map(p.tar, p.w, p.h, px_pitch(p.w), px_window_x(p.rx), px_window_y(p.ry)) : nullptr;
    CUtensorMap none{};
    IcgnParams q = p;
    q.wait_polls = wait_polls;
    q.wait_test = wait_test & 1;
    const int mode = sh.tile ? (m ? 2 : 1) : 0;
#define DIC_PAIR_PX_LAUNCH(PW, W, M) \
  k_icgn_pair_px<PW, W, M><<<grid, W * 32, smem, stream>>>(q, m ? *m : none, icgn_next.ptr, wait_flag())
#define DIC_PAIR_PX_MODES(PW, W)                     \
  do                                                 \
  {                                                  \
    if (mode == 2) DIC_PAIR_PX_LAUNCH(PW, W, 2);     \
    else if (mode == 1) DIC_PAIR_PX_LAUNCH(PW, W, 1); \
    else DIC_PAIR_PX_LAUNCH(PW, W, 0);               \
  } while (0)
    if (pw == 2)
    {
      if (warps == 2) DIC_PAIR_PX_MODES(2, 2);
      else if (warps == 8) DIC_PAIR_PX_MODES(2, 8);
      else DIC_PAIR_PX_MODES(2, 4);
    }
    else
    {
      if (warps == 2) DIC_PAIR_PX_MODES(1, 2);
      else if (warps == 8) DIC_PAIR_PX_MODES(1, 8);
      else DIC_PAIR_PX_MODES(1, 4);
    }
#undef DIC_PAIR_PX_MODES
#undef DIC_PAIR_PX_LAUNCH
  }
  bool tile_attr_set[3] = {};   // per engine, so per device: the shared-memory opt-in of each tile form
  template <int W, int BX, int BY>
  void launch_tile(const IcgnParams& p, int kind, int sms)
  {
    if (!tile_attr_set[kind])
    {
      DIC_CUDA(cudaFuncSetAttribute(k_icgn_tile<W, BX, BY>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                    (int)tile_smem_bytes<BX, BY>()));
      tile_attr_set[kind] = true;
    }
    const CUtensorMap& m = coef_map(kind, p.coef, p.w, p.h);
    IcgnParams q = p;
    q.wait_polls = wait_polls;
    q.wait_test = wait_test & 1;
    const unsigned grid =
        (unsigned)std::min<int64_t>((int64_t)sms * kTileKinds[kind].ctas, (p.n + W - 1) / W);
    k_icgn_tile<W, BX, BY><<<grid, W * 32, tile_smem_bytes<BX, BY>(), stream>>>(q, m, icgn_next.ptr, wait_flag());
  }
  void launch_icgn_pair(const IcgnParams& p, const IcgnShape& sh)
  {
    const int warps = sh.warps, pw = sh.poi_warps == 2 ? 2 : 1;
    const int slots = warps / pw;
    if (sh.ctas_per_sm > 0)
    {
      icgn_next.ensure(1);
      DIC_CUDA(cudaMemsetAsync(icgn_next.ptr, 0, sizeof(unsigned long long), stream));
      int sms = 0;
      DIC_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, cfg.device));
      const unsigned grid = (unsigned)std::min<int64_t>((int64_t)sms * sh.ctas_per_sm, (p.n + slots - 1) / slots);
#define DIC_PAIR_PERSIST(PW, W) k_icgn_pair_persistent<PW, W><<<grid, W * 32, 0, stream>>>(p, icgn_next.ptr)
      if (pw == 2)
      {
        if (warps == 2) DIC_PAIR_PERSIST(2, 2);
        else if (warps == 8) DIC_PAIR_PERSIST(2, 8);
        else DIC_PAIR_PERSIST(2, 4);
      }
      else
      {
        if (warps == 2) DIC_PAIR_PERSIST(1, 2);
        else if (warps == 8) DIC_PAIR_PERSIST(1, 8);
        else DIC_PAIR_PERSIST(1, 4);
      }
#undef DIC_PAIR_PERSIST
      return;
    }
    const unsigned blocks = (unsigned)((p.n + slots - 1) / slots);
#define DIC_PAIR_GRID(PW, W) k_icgn_pair<PW, W><<<blocks, W * 32, 0, stream>>>(p)
    if (pw == 2)
    {
      if (warps == 2) DIC_PAIR_GRID(2, 2);
      else if (warps == 8) DIC_PAIR_GRID(2, 8);
      else DIC_PAIR_GRID(2, 4);
    }
    else
    {
      if (warps == 2) DIC_PAIR_GRID(1, 2);
      else if (warps == 8) DIC_PAIR_GRID(1, 8);
      else DIC_PAIR_GRID(1, 4);
    }
#undef DIC_PAIR_GRID
  }
  void launch_icgn(const IcgnParams& p, int walk, const IcgnShape& sh)
  {
    if (walk == kWalkColumnPx)
    {
      launch_px(p, sh);
      return;
    }
    if (walk == kWalkPairPx)
    {
      launch_pair_px(p, sh);
      return;
    }
    if (walk == kWalkPair)
    {
      launch_icgn_pair(p, sh);
      return;
    }
    const bool column = walk == kWalkColumn;
    const int warps = sh.warps;
    if (sh.tile && column)
    {
      icgn_next.ensure(1);
      DIC_CUDA(cudaMemsetAsync(icgn_next.ptr, 0, sizeof(unsigned long long), stream));
      int sms = 0;
      DIC_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, cfg.device));
      if (sh.tile == 1) launch_tile<4, 48, 36>(p, 1, sms);
      else launch_tile<8, 64, 40>(p, 2, sms);
      return;
    }
    if (sh.ctas_per_sm > 0)
    {
      icgn_next.ensure(1);
      DIC_CUDA(cudaMemsetAsync(icgn_next.ptr, 0, sizeof(unsigned long long), stream));
      int sms = 0;
      DIC_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, cfg.device));
      const unsigned grid = (unsigned)std::min<int64_t>((int64_t)sms * sh.ctas_per_sm, (p.n + warps - 1) / warps);
#define DIC_ICGN_PERSIST(C, W) k_icgn_persistent<C, W><<<grid, W * 32, 0, stream>>>(p, icgn_next.ptr)
      if (column)
      {
        if (warps == 2) DIC_ICGN_PERSIST(true, 2);
        else if (warps == 8) DIC_ICGN_PERSIST(true, 8);
        else DIC_ICGN_PERSIST(true, 4);
      }
      else
      {
        if (warps == 2) DIC_ICGN_PERSIST(false, 2);
        else if (warps == 8) DIC_ICGN_PERSIST(false, 8);
        else DIC_ICGN_PERSIST(false, 4);
      }
#undef DIC_ICGN_PERSIST
      return;
    }
    const unsigned blocks = (unsigned)((p.n + warps - 1) / warps);
#define DIC_ICGN_LAUNCH(C, W) k_icgn<C, W><<<blocks, W * 32, 0, stream>>>(p)
    if (column)
    {
      if (warps == 2) DIC_ICGN_LAUNCH(true, 2);
      else if (warps == 8) DIC_ICGN_LAUNCH(true, 8);
      else DIC_ICGN_LAUNCH(true, 4);
    }
    else
    {
      if (warps == 2) DIC_ICGN_LAUNCH(false, 2);
      else if (warps == 8) DIC_ICGN_LAUNCH(false, 8);
      else DIC_ICGN_LAUNCH(false, 4);
    }
#undef DIC_ICGN_LAUNCH
  }
  struct BatchLaunch
  {
    const BatchJob* jobs;
    int njobs;
    dic_poi* pois;
    const PoiRef* poi_ref;
    int64_t begin, end;
    unsigned long long* next;
    unsigned long long* iter_sum;
    int rmax = 0;   // pixel sampling: the largest subset radius of the range (window size)
  };
  void launch_batch(const BatchLaunch& b, int walk, const IcgnShape& sh)
  {
    int sms = 0;
    DIC_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, cfg.device));
    const float mi = (float)cfg.max_iteration;
    if (walk == kWalkColumnPx)
    {
      // windows sized for the largest radius of the launch's jobs
      px_attributes();
      const uint32_t win = (uint32_t)px_window_bytes(b.rmax, b.rmax);
      const size_t smem = 128 + (size_t)sh.warps * win;
      const int ctas = sh.ctas_per_sm > 0 ? sh.ctas_per_sm : occupancy_batch_px(sh.warps, smem);
      const unsigned grid = (unsigned)(sms * ctas);
#define DIC_BATCH_PX(W, M)                                                                                         \
  k_icgn_batch_px<W, M><<<grid, W * 32, smem, stream>>>(b.jobs, b.njobs, b.pois, b.poi_ref, b.begin, b.end, b.next,     \
                                                        cfg.conv_criterion, mi, b.iter_sum, win, wait_polls, wait_flag())
      if (b_px_maps)
      {
        if (sh.warps == 2) DIC_BATCH_PX(2, 2);
        else if (sh.warps == 8) DIC_BATCH_PX(8, 2);
        else DIC_BATCH_PX(4, 2);
      }
      else
      {
        if (sh.warps == 2) DIC_BATCH_PX(2, 1);
        else if (sh.warps == 8) DIC_BATCH_PX(8, 1);
        else DIC_BATCH_PX(4, 1);
      }
#undef DIC_BATCH_PX
      check_launch("k_icgn_batch_px");
      return;
    }
    if (walk == kWalkPairPx)
    {
      // windows sized for the largest radius of the launch's jobs
      px_attributes();
      const int pw = sh.poi_warps == 2 ? 2 : 1;
      const uint32_t win = (uint32_t)px_window_bytes(b.rmax, b.rmax);
      const size_t smem = b_px_maps ? pair_px_smem(sh.warps, pw, win) : 0;
      const int ctas = sh.ctas_per_sm > 0 ? sh.ctas_per_sm : occupancy_pair_px(true, pw, sh.warps, smem);
      const unsigned grid = (unsigned)(sms * ctas);
#define DIC_BATCH_PAIR_PX(PW, W, M)                                                                                  \
  k_icgn_batch_pair_px<PW, W, M><<<grid, W * 32, smem, stream>>>(b.jobs, b.njobs, b.pois, b.poi_ref, b.begin, b.end,    \
                                                                 b.next, cfg.conv_criterion, mi, b.iter_sum, win,     \
                                                                 wait_polls, wait_flag())
#define DIC_BATCH_PAIR_PX_W(PW)                                \
  do                                                           \
  {                                                            \
    if (b_px_maps)                                            \
    {                                                          \
      if (sh.warps == 2) DIC_BATCH_PAIR_PX(PW, 2, 2);          \
      else if (sh.warps == 8) DIC_BATCH_PAIR_PX(PW, 8, 2);     \
      else DIC_BATCH_PAIR_PX(PW, 4, 2);                        \
    }                                                          \
    else                                                       \
    {                                                          \
      if (sh.warps == 2) DIC_BATCH_PAIR_PX(PW, 2, 0);          \
      else if (sh.warps == 8) DIC_BATCH_PAIR_PX(PW, 8, 0);     \
      else DIC_BATCH_PAIR_PX(PW, 4, 0);                        \
    }                                                          \
  } while (0)
      if (pw == 2) DIC_BATCH_PAIR_PX_W(2);
      else DIC_BATCH_PAIR_PX_W(1);
#undef DIC_BATCH_PAIR_PX_W
#undef DIC_BATCH_PAIR_PX
      check_launch("k_icgn_batch_pair_px");
      return;
    }
    const unsigned grid = (unsigned)(sms * sh.ctas_per_sm);
    if (walk == kWalkPair)
    {
#define DIC_BATCH_PAIR(PW, W)                                                                                      \
  k_icgn_batch_pair<PW, W><<<grid, W * 32, 0, stream>>>(b.jobs, b.njobs, b.pois, b.poi_ref, b.begin, b.end, b.next,    \
                                                       cfg.conv_criterion, mi, b.iter_sum)
      if (sh.poi_warps == 2)
      {
        if (sh.warps == 2) DIC_BATCH_PAIR(2, 2);
        else if (sh.warps == 8) DIC_BATCH_PAIR(2, 8);
        else DIC_BATCH_PAIR(2, 4);
      }
      else
      {
        if (sh.warps == 2) DIC_BATCH_PAIR(1, 2);
        else if (sh.warps == 8) DIC_BATCH_PAIR(1, 8);
        else DIC_BATCH_PAIR(1, 4);
      }
#undef DIC_BATCH_PAIR
      check_launch("k_icgn_batch_pair");
      return;
    }
    const bool column = walk == kWalkColumn;
#define DIC_BATCH_LAUNCH(C, W)                                                                                     \
  k_icgn_batch<C, W><<<grid, W * 32, 0, stream>>>(b.jobs, b.njobs, b.pois, b.poi_ref, b.begin, b.end, b.next,          \
                                                  cfg.conv_criterion, mi, b.iter_sum)
    if (column)
    {
      if (sh.warps == 2) DIC_BATCH_LAUNCH(true, 2);
      else if (sh.warps == 8) DIC_BATCH_LAUNCH(true, 8);
      else DIC_BATCH_LAUNCH(true, 4);
    }
    else
    {
      if (sh.warps == 2) DIC_BATCH_LAUNCH(false, 2);
      else if (sh.warps == 8) DIC_BATCH_LAUNCH(false, 8);
      else DIC_BATCH_LAUNCH(false, 4);
    }
#undef DIC_BATCH_LAUNCH
    check_launch("k_icgn_batch");
  }
  float time_once(const std::function<void()>& f)
  {
    if (!tune_ev[0])
      for (auto& ev : tune_ev) DIC_CUDA(cudaEventCreate(&ev));
    DIC_CUDA(cudaEventRecord(tune_ev[0], stream));
    f();
    DIC_CUDA(cudaEventRecord(tune_ev[1], stream));
    DIC_CUDA(cudaEventSynchronize(tune_ev[1]));
    float ms = 0.f;
    DIC_CUDA(cudaEventElapsedTime(&ms, tune_ev[0], tune_ev[1]));
    return ms;
  }
  // Times every candidate shape on a copy of the seeded queue (best of two runs) and keeps
  // the fastest.  The queue itself is not touched.
  void tune_icgn(const IcgnParams& p0, int walk)
  {
    const bool column = walk == kWalkColumn;
    tune_q.ensure((size_t)p0.n);
    IcgnParams p = p0;
    p.pois = tune_q.ptr;
    p.iter_sum = nullptr;
    IcgnShape best;
    best.ms = INFINITY;
    std::vector<IcgnShape> cand;
    for (int warps : {2, 4, 8})
      for (int persistent = 0; persistent < 2; ++persistent)
        if (walk == kWalkColumnPx)
        {
          // windows staged by TMA, or not staged; and staged by warp copies
          cand.push_back(IcgnShape{warps, 0, 0.f, persistent});
          if (persistent) cand.push_back(IcgnShape{warps, 0, 0.f, 2});
        }
        else if (walk == kWalkPair)
          for (int pw : {1, 2})
            cand.push_back(IcgnShape{warps, persistent ? occupancy_pair(false, pw, warps) : 0, 0.f, 0, pw});
        else if (walk == kWalkPairPx)
        {
          // windows staged by TMA or not staged, one or two warps per POI (always persistent)
          if (persistent)
            for (int pw : {1, 2})
              for (int tile : {1, 0}) cand.push_back(IcgnShape{warps, 0, 0.f, tile, pw});
        }
        else
          cand.push_back(IcgnShape{warps, persistent ? occupancy_single(column, warps) : 0, 0.f, 0});
    // the TMA-staged tile forms (column walk, where the driver provides tensor maps)
    if (column && encode_tiled())
      for (int kind = 1; kind <= 2; ++kind)
        cand.push_back(IcgnShape{kTileKinds[kind].warps, kTileKinds[kind].ctas, 0.f, kind});
    for (const IcgnShape& sh : cand)
    {
      float t = INFINITY;
      for (int rep = 0; rep < 2; ++rep)
      {
        DIC_CUDA(cudaMemcpyAsync(tune_q.ptr, p0.pois, sizeof(dic_poi) * p0.n, cudaMemcpyDeviceToDevice, stream));
        t = std::min(t, time_once([&] { launch_icgn(p, walk, sh); }));
      }
      if (t < best.ms) best = IcgnShape{sh.warps, sh.ctas_per_sm, t, sh.tile, sh.poi_warps};
    }
    check_wait_error();
    shape[0][walk] = best;
    tuned[0][walk] = true;
  }
  void tune_batch(const BatchLaunch& b0, int walk, int64_t total)
  {
    tune_q.ensure((size_t)total);
    BatchLaunch b = b0;
    b.pois = tune_q.ptr;
    b.iter_sum = nullptr;
    IcgnShape best;
    best.ms = INFINITY;
    for (int warps : {2, 4, 8})
      for (int pw : {1, 2})
      {
        if (walk != kWalkPair && walk != kWalkPairPx && pw == 2) continue;
        // the pixel pair walk's drains run per window size, each at its own full occupancy
        // (ctas_per_sm 0); the other drains try full and 3/4 occupancy
        int cands[2] = {0, -1};
        if (walk != kWalkPairPx)
        {
          const int full = walk == kWalkColumnPx
                               ? occupancy_batch_px(warps, 128 + (size_t)warps * px_window_bytes(b.rmax, b.rmax))
                           : walk == kWalkPair ? occupancy_pair(true, pw, warps)
                                               : occupancy(true, walk == kWalkColumn, warps);
          cands[0] = full;
          cands[1] = std::max(1, (3 * full) / 4);
        }
        for (int ctas : cands)
        {
          if (ctas < 0) continue;
          const IcgnShape sh{warps, ctas, 0.f, 0, pw};
          float t = INFINITY;
          for (int rep = 0; rep < 2; ++rep)
          {
            DIC_CUDA(cudaMemcpyAsync(tune_q.ptr + b.begin, b0.pois + b.begin, sizeof(dic_poi) * (b.end - b.begin),
                                     cudaMemcpyDeviceToDevice, stream));
            DIC_CUDA(cudaMemsetAsync(b.next, 0, sizeof(unsigned long long), stream));
            t = std::min(t, time_once([&] { launch_batch(b, walk, sh); }));
          }
          if (t < best.ms) best = IcgnShape{warps, ctas, t, 0, pw};
        }
      }
    shape[1][walk] = best;
    tuned[1][walk] = true;
    DIC_CUDA(cudaMemsetAsync(b0.next, 0, sizeof(unsigned long long), stream));
  }

  // ---------------------------------------------------------------- solvers
  // FFTCC launch for an explicit plane pair and (square) radius.
  void fftcc_launch(const FftccParams& p, int r, cudaStream_t on = nullptr)
  {
    cudaStream_t st = on ? on : stream;
    const unsigned blocks = (unsigned)((p.n + 3) / 4);
    switch (2 * r)
    {
#define DIC_FFTCC_CASE2(M) \
  case M: k_fftcc2<M><<<(unsigned)((p.n + 3) / 4), 64, 0, st>>>(p); break;
      DIC_FFTCC_CASE2(8) DIC_FFTCC_CASE2(10) DIC_FFTCC_CASE2(12) DIC_FFTCC_CASE2(14) DIC_FFTCC_CASE2(16)
      DIC_FFTCC_CASE2(18) DIC_FFTCC_CASE2(20) DIC_FFTCC_CASE2(22) DIC_FFTCC_CASE2(24) DIC_FFTCC_CASE2(26)
      DIC_FFTCC_CASE2(28) DIC_FFTCC_CASE2(30)
#undef DIC_FFTCC_CASE2
      case 32: k_fftcc<32><<<blocks, 128, 0, st>>>(p); break;
#define DIC_FFTCC_BIG(M) \
  case M: k_fftcc_big<M><<<(unsigned)p.n, 128, (size_t)M * (M + 1) * sizeof(float2), st>>>(p); break;
      // 2r = 2 x prime (34, 38, 46, 58, 62) stays on the line-DFT kernel below
      DIC_FFTCC_BIG(36) DIC_FFTCC_BIG(40) DIC_FFTCC_BIG(42) DIC_FFTCC_BIG(44) DIC_FFTCC_BIG(48)
      DIC_FFTCC_BIG(50) DIC_FFTCC_BIG(52) DIC_FFTCC_BIG(54) DIC_FFTCC_BIG(56) DIC_FFTCC_BIG(60) DIC_FFTCC_BIG(64)
#undef DIC_FFTCC_BIG
      default:
        if (r < 1 || 2 * r > kMaxTwiddleN)
          throw DicError{DIC_ERR_ARGUMENT, "FFTCC supports subset radius 1..32 on this engine"};
        k_fftcc_large<<<(unsigned)p.n, 256, (size_t)2 * (2 * r) * (2 * r + 1) * sizeof(float2), st>>>(p, 2 * r);
    }
    check_launch("k_fftcc");
  }

  void run_fftcc(dic_poi* d_pois, int64_t n, const int64_t* n_dev = nullptr, const int* enable = nullptr)
  {
    if (n == 0) return;
    ensure_ref();
    ensure_tar();
    FftccParams p{ref_f32.ptr, tar_f32.ptr, d_pois, n, w, h};
    p.n_dev = n_dev;
    p.enable = enable;
    mark(kPhFftcc, 0);
    fftcc_launch(p, cfg.subset_radius_x);
    mark(kPhFftcc, 1);
  }

  void run_icgn(dic_poi* d_pois, int64_t n, const int64_t* d_slots, const int64_t* n_dev = nullptr,
                const int* enable = nullptr, bool reset_iterations = true, int max_iter_override = 0)
  {
    if (n == 0) return;
    ensure_ref();
    ensure_tar();
    counters.ensure(1);
    if (reset_iterations) DIC_CUDA(cudaMemsetAsync(counters.ptr, 0, sizeof(unsigned long long), stream));
    IcgnParams p;
    p.n_dev = n_dev;
    p.enable = enable;
    p.coef = coef.ptr;
    p.lattice = lattice.ptr;
    p.tar = px_plane();
    p.ref_pack = ref_pack.ptr;
    p.poi_ref = poi_ref.ptr;
    p.slot = d_slots;
    p.pois = d_pois;
    p.n = n;
    p.w = w;
    p.h = h;
    p.rx = cfg.subset_radius_x;
    p.ry = cfg.subset_radius_y;
    p.conv = cfg.conv_criterion;
    p.max_iter = (float)(max_iter_override > 0 ? max_iter_override : cfg.max_iteration);
    p.iter_sum = counters.ptr;
    const int walk = icgn_walk(p.rx);
    if (autotune && !tuned[0][walk] && n >= kTuneMinPois && !capturing()) tune_icgn(p, walk);
    mark(kPhIcgn, 0);
    launch_icgn(p, walk, shape[0][walk]);
    check_launch("k_icgn");
    mark(kPhIcgn, 1);
    icgn_pois = n;
    iter_pending = true;
  }

  // ---------------------------------------------------------------- frames
  // Device queues of the frame policy: tmpl (layout template), prev (previous frame's
  // results), queue (current frame), scratch (whole-frame pass), fq (repair candidates).
  DevBuf<dic_poi> tmpl, prev, scratch, fq;
  DevBuf<dic_poi> prev2;          // the frame before prev (temporal extrapolation)
  DevBuf<int> hist;               // sequence: frames of history in prev / prev2 (0, 1, 2)
  DevBuf<int64_t> cand;
  DevBuf<FrameCounters> fcount;
  DevBuf<float> baseline;         // sequence: first frame's bad ratio + margin
  dic_frame_policy seq_policy{};
  int64_t seq_n = 0;
  long long seq_frame = 0;
  bool seq_last_skip = false;     // the most recent frame's kind
  // The last two frames' results and counters (slot = frame & 1), for dic_sequence_fetch: a
  // frame's slot is read on down_stream while the next frame already runs on the engine stream.
  DevBuf<dic_poi> seq_out[2];
  DevBuf<FrameCounters> seq_cnt[2];
  long long seq_out_frame[2] = {-1, -1};
  bool seq_out_skip[2] = {false, false};
  cudaEvent_t seq_done[2] = {};
  cudaStream_t down_stream = nullptr;
  void save_frame_output(int64_t n, bool use_skip)
  {
    const int slot = (int)(seq_frame & 1);
    if (!down_stream)
    {
      DIC_CUDA(cudaStreamCreateWithFlags(&down_stream, cudaStreamNonBlocking));
      for (auto& ev : seq_done) DIC_CUDA(cudaEventCreateWithFlags(&ev, cudaEventDisableTiming));
    }
    seq_out[slot].ensure((size_t)n);
    seq_cnt[slot].ensure(1);
    DIC_CUDA(cudaMemcpyAsync(seq_out[slot].ptr, queue.ptr, sizeof(dic_poi) * n, cudaMemcpyDeviceToDevice, stream));
    DIC_CUDA(cudaMemcpyAsync(seq_cnt[slot].ptr, fcount.ptr, sizeof(FrameCounters), cudaMemcpyDeviceToDevice, stream));
    DIC_CUDA(cudaEventRecord(seq_done[slot], stream));
    seq_out_frame[slot] = seq_frame;
    seq_out_skip[slot] = use_skip;
  }
  void release_frame_outputs()
  {
    if (down_stream) cudaStreamSynchronize(down_stream);
    for (int k = 0; k < 2; ++k)
    {
      seq_out[k].release();
      seq_cnt[k].release();
      if (seq_done[k]) cudaEventDestroy(seq_done[k]);
      seq_done[k] = nullptr;
    }
    if (down_stream) cudaStreamDestroy(down_stream);
    down_stream = nullptr;
  }
  bool use_graphs = true;
  cudaGraphExec_t seq_graph = nullptr;
  int seq_graph_kernels = 0;

  void ensure_frame_buffers(int64_t n)
  {
    tmpl.ensure((size_t)n);
    prev.ensure((size_t)n);
    prev2.ensure((size_t)n);
    hist.ensure(1);
    scratch.ensure((size_t)n);
    fq.ensure((size_t)n);
    cand.ensure((size_t)n);
    queue.ensure((size_t)n);
    fcount.ensure(1);
    baseline.ensure(1);
  }

  // Enqueue one frame on the device queues (no host synchronisation).  The layout must be
  // tmpl's.  use_skip: seed from prev and run the policy; otherwise FFTCC + IC-GN from the
  // template.  frame_threshold: device pointer (sequence) or host value.
  void enqueue_frame(int64_t n, bool use_skip, const dic_frame_policy& pol, const float* threshold_dev,
                     float threshold_host, const dic_poi* prev2_dev = nullptr, const int* hist_dev = nullptr)
  {
    const unsigned tb = 256, nb = (unsigned)((n + tb - 1) / tb);
    const float thr = pol.zncc_threshold;
    DIC_CUDA(cudaMemsetAsync(fcount.ptr, 0, sizeof(FrameCounters), stream));
    DIC_CUDA(cudaMemsetAsync(counters.ptr, 0, sizeof(unsigned long long), stream));
    if (!use_skip)
    {
      DIC_CUDA(cudaMemcpyAsync(queue.ptr, tmpl.ptr, sizeof(dic_poi) * n, cudaMemcpyDeviceToDevice, stream));
      run_fftcc(queue.ptr, n);
      run_icgn(queue.ptr, n, nullptr, nullptr, nullptr, false);
      k_count_bad<<<nb, tb, 0, stream>>>(queue.ptr, thr, &fcount.ptr->bad, n);
      check_launch("k_count_bad");
      k_count_bad<<<nb, tb, 0, stream>>>(queue.ptr, thr, &fcount.ptr->bad_after, n);
      check_launch("k_count_bad");
      return;
    }
    k_seed_from_previous<<<nb, tb, 0, stream>>>(tmpl.ptr, prev.ptr, pol.temporal_extrapolation ? prev2_dev : nullptr,
                                                hist_dev, thr, (float)cfg.subset_radius_x, queue.ptr, n, fcount.ptr);
    check_launch("k_seed_from_previous");
    run_icgn(queue.ptr, n, nullptr, nullptr, nullptr, false);
    k_scan_bad<<<nb, tb, 0, stream>>>(queue.ptr, prev.ptr, thr, pol.poi_fallback, fcount.ptr, cand.ptr, n);
    check_launch("k_scan_bad");
    if (threshold_dev)
      k_decide_dev<<<1, 32, 0, stream>>>(fcount.ptr, n, threshold_dev, pol.poi_fallback);
    else
      k_decide<<<1, 32, 0, stream>>>(fcount.ptr, n, threshold_host, pol.poi_fallback);
    check_launch("k_decide");
    // whole-frame pass: FFTCC + IC-GN from the template, merged per POI
    const int* ff = &fcount.ptr->frame_fallback;
    k_copy_queue<<<nb, tb, 0, stream>>>(tmpl.ptr, scratch.ptr, ff, n);
    check_launch("k_copy_queue");
    run_fftcc(scratch.ptr, n, nullptr, ff);
    run_icgn(scratch.ptr, n, nullptr, nullptr, ff, false);
    k_merge_frame<<<nb, tb, 0, stream>>>(queue.ptr, scratch.ptr, fcount.ptr, thr, n);
    check_launch("k_merge_frame");
    // POI-level repair of the candidates (layout slots = template indices)
    const int* pr = &fcount.ptr->poi_repair;
    const int64_t* cn = &fcount.ptr->candidate_count;
    k_gather_candidates<<<nb, tb, 0, stream>>>(tmpl.ptr, cand.ptr, fcount.ptr, fq.ptr, n);
    check_launch("k_gather_candidates");
    run_fftcc(fq.ptr, n, cn, pr);
    run_icgn(fq.ptr, n, cand.ptr, cn, pr, false);
    k_merge_repair<<<nb, tb, 0, stream>>>(queue.ptr, fq.ptr, cand.ptr, fcount.ptr, thr, n);
    check_launch("k_merge_repair");
    k_count_bad<<<nb, tb, 0, stream>>>(queue.ptr, thr, &fcount.ptr->bad_after, n);
    check_launch("k_count_bad");
  }

  // ---------------------------------------------------------------- learned seed
  dic_cnn* proposal = nullptr;
  static constexpr int kLearnedMaxIter = 6;      // IC-GN budget from the proposal's seed
  static constexpr float kLearnedAccept = 0.9f;  // ZNCC the proposal's result must reach
  static constexpr int64_t kProposalBatch = 32768;

  // Proposal seeds, IC-GN capped at kLearnedMaxIter, then FFTCC + IC-GN (full budget) for
  // the POIs that fail; the layout is the template's.  from_template: the sequence form
  // (tmpl holds the template, copied into queue); otherwise `queue` holds it (pair form).
  // `bad_thr` counts the final bad POIs for the frame report.
  void enqueue_learned(int64_t n, bool from_template = false, float bad_thr = 0.8f)
  {
    if (!proposal) throw DicError{DIC_ERR_STATE, "no proposal network attached (dic_set_proposal)"};
    ensure_ref();
    ensure_tar();
    ensure_frame_buffers(n);
    const unsigned tb = 256, nb = (unsigned)((n + tb - 1) / tb);
    DIC_CUDA(cudaMemsetAsync(fcount.ptr, 0, sizeof(FrameCounters), stream));
    DIC_CUDA(cudaMemsetAsync(counters.ptr, 0, sizeof(unsigned long long), stream));
    if (from_template)
      DIC_CUDA(cudaMemcpyAsync(queue.ptr, tmpl.ptr, sizeof(dic_poi) * n, cudaMemcpyDeviceToDevice, stream));
    else
      DIC_CUDA(cudaMemcpyAsync(tmpl.ptr, queue.ptr, sizeof(dic_poi) * n, cudaMemcpyDeviceToDevice, stream));
    mark(kPhProposal, 0);
    {
      // fused inference: one persistent CTA per SM (two warp groups of kT POIs per tile), seeds into the queue
      int sms = 0;
      DIC_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, cfg.device));
      const int64_t tiles = (n + cnn::kT - 1) / cnn::kT;
      const unsigned grid = (unsigned)std::min<int64_t>((tiles + cnn::kGroups - 1) / cnn::kGroups, sms);
      cnn::k_proposal_fused<<<grid, cnn::kFusedThreads, cnn::kSmTotal, stream>>>(
          ref_f32.ptr, tar_f32.ptr, w, h, queue.ptr, n, proposal->wb.ptr, proposal->params.ptr, wait_flag(), wait_polls,
          (wait_test >> 1) & 1);
      check_launch("k_proposal_fused");
    }
    mark(kPhProposal, 1);
    run_icgn(queue.ptr, n, nullptr, nullptr, nullptr, false, std::min(kLearnedMaxIter, cfg.max_iteration));
    k_scan_learned<<<nb, tb, 0, stream>>>(queue.ptr, kLearnedAccept, fcount.ptr, cand.ptr, n);
    check_launch("k_scan_learned");
    k_enable_candidates<<<1, 32, 0, stream>>>(fcount.ptr);
    check_launch("k_enable_candidates");
    const int* pr = &fcount.ptr->poi_repair;
    const int64_t* cn = &fcount.ptr->candidate_count;
    k_gather_candidates<<<nb, tb, 0, stream>>>(tmpl.ptr, cand.ptr, fcount.ptr, fq.ptr, n);
    check_launch("k_gather_candidates");
    run_fftcc(fq.ptr, n, cn, pr);
    run_icgn(fq.ptr, n, cand.ptr, cn, pr, false);
    k_merge_fallback<<<nb, tb, 0, stream>>>(queue.ptr, fq.ptr, cand.ptr, fcount.ptr, bad_thr, n);
    check_launch("k_merge_fallback");
    k_count_bad<<<nb, tb, 0, stream>>>(queue.ptr, bad_thr, &fcount.ptr->bad_after, n);
    check_launch("k_count_bad");
  }

  // ---------------------------------------------------------------- staged uploads
  cudaStream_t up_stream = nullptr;
  unsigned char* stage_host[2] = {nullptr, nullptr};
  size_t stage_host_cap[2] = {0, 0};
  DevBuf<unsigned char> stage_dev[2];
  cudaEvent_t stage_uploaded[2] = {nullptr, nullptr}, stage_consumed[2] = {nullptr, nullptr};
  int stage_w[2] = {0, 0}, stage_h[2] = {0, 0}, stage_dtype[2] = {0, 0};
  bool stage_full[2] = {false, false};
  int stage_next = 0, stage_take = 0;

  void stage_frame(const void* px, int width, int height, int64_t stride, int dtype)
  {
    const int es = dtype_size(dtype);
    if (!px || es == 0 || width < 5 || height < 5 || stride < (int64_t)width * es)
      throw DicError{DIC_ERR_ARGUMENT, "stage_frame: null pixels, unknown dtype, bad size or stride"};
    const int s = stage_next;
    if (stage_full[s]) throw DicError{DIC_ERR_STATE, "stage_frame: two frames are already staged"};
    if (!up_stream)
    {
      DIC_CUDA(cudaStreamCreateWithFlags(&up_stream, cudaStreamNonBlocking));
      for (int k = 0; k < 2; ++k)
      {
        DIC_CUDA(cudaEventCreateWithFlags(&stage_uploaded[k], cudaEventDisableTiming));
        DIC_CUDA(cudaEventCreateWithFlags(&stage_consumed[k], cudaEventDisableTiming));
      }
    }
    const size_t row = (size_t)width * es, bytes = row * height;
    // A page-locked source is uploaded straight from the caller's buffer, and the call waits
    // for that copy (~40 us for 8 MB) so that the buffer is free on return; a pageable one
    // goes through a host copy into the pinned double buffer and uploads asynchronously.
    cudaPointerAttributes attr{};
    const bool pinned = cudaPointerGetAttributes(&attr, px) == cudaSuccess && attr.type == cudaMemoryTypeHost;
    if (!pinned) cudaGetLastError();
    if (pinned)
    {
      if (stage_dev[s].cap < bytes)
      {
        DIC_CUDA(cudaEventSynchronize(stage_consumed[s]));
        stage_dev[s].ensure(bytes);
      }
      DIC_CUDA(cudaStreamWaitEvent(up_stream, stage_consumed[s], 0));   // the device copy was taken
      DIC_CUDA(cudaMemcpy2DAsync(stage_dev[s].ptr, row, px, (size_t)stride, row, height, cudaMemcpyHostToDevice,
                                 up_stream));
      DIC_CUDA(cudaEventRecord(stage_uploaded[s], up_stream));
      DIC_CUDA(cudaEventSynchronize(stage_uploaded[s]));
      stage_w[s] = width;
      stage_h[s] = height;
      stage_dtype[s] = dtype;
      stage_full[s] = true;
      stage_next ^= 1;
      return;
    }
    DIC_CUDA(cudaEventSynchronize(stage_uploaded[s]));   // the pinned buffer's last copy is done
    if (stage_host_cap[s] < bytes)
    {
      if (stage_host[s]) DIC_CUDA(cudaFreeHost(stage_host[s]));
      stage_host[s] = nullptr;
      stage_host_cap[s] = 0;
      if (cudaMallocHost((void**)&stage_host[s], bytes) != cudaSuccess)
      {
        stage_host[s] = nullptr;
        throw DicError{DIC_ERR_MEMORY, "stage_frame: pinned allocation failed"};
      }
      stage_host_cap[s] = bytes;
    }
    const unsigned char* src = static_cast<const unsigned char*>(px);
    if ((size_t)stride == row) std::memcpy(stage_host[s], src, bytes);
    else
      for (int y = 0; y < height; ++y) std::memcpy(stage_host[s] + (size_t)y * row, src + (size_t)y * stride, row);
    if (stage_dev[s].cap < bytes)
    {
      DIC_CUDA(cudaEventSynchronize(stage_consumed[s]));
      stage_dev[s].ensure(bytes);
    }
    DIC_CUDA(cudaStreamWaitEvent(up_stream, stage_consumed[s], 0));   // the device copy was taken
    DIC_CUDA(cudaMemcpyAsync(stage_dev[s].ptr, stage_host[s], bytes, cudaMemcpyHostToDevice, up_stream));
    DIC_CUDA(cudaEventRecord(stage_uploaded[s], up_stream));
    stage_w[s] = width;
    stage_h[s] = height;
    stage_dtype[s] = dtype;
    stage_full[s] = true;
    stage_next ^= 1;
  }

  // The oldest staged frame becomes the target (engine stream waits for its copy only).
  void take_staged(int width, int height, int dtype)
  {
    const int s = stage_take;
    if (!stage_full[s]) throw DicError{DIC_ERR_STATE, "no staged frame (dic_stage_frame)"};
    if (stage_w[s] != width || stage_h[s] != height || stage_dtype[s] != dtype)
      throw DicError{DIC_ERR_ARGUMENT, "the staged frame's size or type differs from the call's"};
    DIC_CUDA(cudaStreamWaitEvent(stream, stage_uploaded[s], 0));
    set_image(false, stage_dev[s].ptr, width, height, (int64_t)width * dtype_size(dtype), dtype, true);
    DIC_CUDA(cudaEventRecord(stage_consumed[s], stream));
    stage_full[s] = false;
    stage_take ^= 1;
  }

  void release_staging()
  {
    if (up_stream) cudaStreamSynchronize(up_stream);
    for (int k = 0; k < 2; ++k)
    {
      if (stage_host[k]) cudaFreeHost(stage_host[k]);
      stage_host[k] = nullptr;
      stage_dev[k].release();
      if (stage_uploaded[k]) cudaEventDestroy(stage_uploaded[k]);
      if (stage_consumed[k]) cudaEventDestroy(stage_consumed[k]);
      stage_uploaded[k] = stage_consumed[k] = nullptr;
    }
    if (up_stream) cudaStreamDestroy(up_stream);
    up_stream = nullptr;
  }

  // ---------------------------------------------------------------- uneven batches
  struct JobBufs
  {
    DevBuf<unsigned char> raw_ref, raw_tar;
    DevBuf<float> ref_f32, tar_f32;
    DevBuf<float4> ref_pack, coef;
    DevBuf<float> lattice, tar_px;
    void release()
    {
      raw_ref.release(); raw_tar.release(); ref_f32.release(); tar_f32.release(); ref_pack.release(); coef.release();
      lattice.release(); tar_px.release();
    }
  };
  std::vector<JobBufs> jobs_mem;
  DevBuf<dic_poi> bq;
  DevBuf<PoiRef> bpoi;
  DevBuf<BatchJob> bjobs;
  DevBuf<unsigned long long> bnext;

  template <typename T>
  void prep_planes(const unsigned char* raw_r, const unsigned char* raw_t, int bw, int bh, JobBufs& J, bool table,
                   bool pitched, cudaStream_t st)
  {
    dim3 grid((bw + kPrepTile - 1) / kPrepTile, (bh + kPrepTile - 1) / kPrepTile);
    k_prepare_ref<T><<<grid, 256, 0, st>>>(reinterpret_cast<const T*>(raw_r), bw, bh, scale(), J.ref_f32.ptr,
                                               J.ref_pack.ptr);
    check_launch("k_prepare_ref");
    k_prepare_tar<T><<<grid, 256, 0, st>>>(reinterpret_cast<const T*>(raw_t), bw, bh, scale(), J.tar_f32.ptr,
                                           table ? J.coef.ptr : nullptr, J.lattice.ptr,
                                           pitched ? J.tar_px.ptr : nullptr, px_pitch(bw));
    check_launch("k_prepare_tar");
  }

  // Batch plan: column-walk jobs (2r + 1 <= 32) first, then the pair walk's (33 to 64
  // columns), then wider subsets, stable otherwise.
  std::vector<int> b_order;
  std::vector<int64_t> b_first;
  int64_t b_total = 0, b_col_end = 0, b_pair_end = 0;
  int b_col_rmax = 0;                   // largest subset radius among the column-walk jobs
  // The pair-walk jobs' drains: one per subset radius under pixel sampling (queue range and
  // radius), one for all of them under table sampling.
  struct PairGroup
  {
    int64_t begin, end;
    int rmax;
  };
  std::vector<PairGroup> b_pair_groups;
#ifndef DIC_BATCH_PAIR_BY_RADIUS
#define DIC_BATCH_PAIR_BY_RADIUS 1
#endif
  static constexpr bool kBatchPairByRadius = DIC_BATCH_PAIR_BY_RADIUS != 0;
  static constexpr int kMaxPairGroups = kPairMaxWidth / 2 - 15;   // radii 16 .. (width - 1) / 2
  DevBuf<CUtensorMap> bmaps;            // the jobs' target-plane tensor maps (pixel sampling)
  bool b_px_maps = false;              // every pixel-sampled job has one (TMA windows), else warp copies / none
  std::vector<CUtensorMap> b_maps_host; // their host copy (kept alive for the asynchronous upload)
  // pixel sampling covers the batch's column- and pair-walk jobs; the flat walk's sample the table
  bool job_table(int radius) const { return !pixel_radius(radius); }
  // a pixel-sampled job whose width is not a multiple of 4 floats gets a padded-pitch plane
  bool job_pitched(int radius, int width) const { return !job_table(radius) && (width & 3) != 0; }
  std::vector<dic_job> b_key;           // jobs of the captured batch graph (device pointers)
  bool b_key_seen = false;
  cudaGraphExec_t batch_graph = nullptr;
  int batch_graph_kernels = 0;

  void plan_batch(const dic_job* jobs, int nj)
  {
    b_order.resize(nj);
    for (int j = 0; j < nj; ++j) b_order[j] = j;
    // walk rank: column 0, pair 1, flat 2; pair-walk jobs by subset radius under pixel
    // sampling, whose windows, and so the drain's residency, depend on it
    const auto rank = [&](int j) {
      const int wk = walk_of(jobs[j].subset_radius);
      return wk == kWalkColumn ? 0 : wk == kWalkPair ? 1 : 2;
    };
    const bool px_pairs = kBatchPairByRadius && sampling == DIC_SAMPLE_PIXELS;
    std::stable_sort(b_order.begin(), b_order.end(), [&](int a, int b) {
      if (rank(a) != rank(b)) return rank(a) < rank(b);
      return px_pairs && rank(a) == 1 && jobs[a].subset_radius < jobs[b].subset_radius;
    });
    b_first.assign(nj, 0);
    b_total = 0;
    b_col_end = 0;
    b_pair_end = 0;
    b_col_rmax = 0;
    b_pair_groups.clear();
    for (int k = 0; k < nj; ++k)
    {
      const dic_job& J = jobs[b_order[k]];
      b_first[k] = b_total;
      b_total += J.count;
      const int r = rank(b_order[k]);
      if (r == 0) b_col_end = b_total;
      if (r == 0) b_col_rmax = std::max(b_col_rmax, J.subset_radius);
      if (r == 1)
      {
        if (b_pair_groups.empty() || (px_pairs && b_pair_groups.back().rmax != J.subset_radius))
          b_pair_groups.push_back(PairGroup{b_first[k], b_total, J.subset_radius});
        b_pair_groups.back().end = b_total;
        b_pair_groups.back().rmax = std::max(b_pair_groups.back().rmax, J.subset_radius);
      }
      if (r <= 1) b_pair_end = b_total;
    }
    if ((int)jobs_mem.size() < nj) jobs_mem.resize(nj);
    bq.ensure((size_t)std::max<int64_t>(b_total, 1));
    bpoi.ensure((size_t)std::max<int64_t>(b_total, 1));
    bjobs.ensure((size_t)nj);
    bnext.ensure(2 + kMaxPairGroups);
    counters.ensure(1);
    std::vector<BatchJob> table(nj);
    for (int k = 0; k < nj; ++k)
    {
      const dic_job& J = jobs[b_order[k]];
      JobBufs& M = jobs_mem[k];
      const int es = dtype_size(J.dtype);
      const size_t px = (size_t)J.width * J.height;
      M.raw_ref.ensure(px * es);
      M.raw_tar.ensure(px * es);
      M.ref_f32.ensure(px);
      M.tar_f32.ensure(px);
      M.ref_pack.ensure(px);
      if (job_table(J.subset_radius))
      {
        M.coef.ensure(px * 4);
        M.lattice.ensure(px);
      }
      const bool pitched = job_pitched(J.subset_radius, J.width);
      if (pitched) M.tar_px.ensure((size_t)px_pitch(J.width) * J.height);
      table[k] = BatchJob{M.coef.ptr, M.lattice.ptr, M.ref_pack.ptr, b_first[k], J.width, J.height, J.subset_radius,
                          J.subset_radius, pitched ? M.tar_px.ptr : M.tar_f32.ptr};
    }
    // tensor maps of the pixel-sampled jobs' target planes (window copies by TMA), in device
    // memory beside the job table
    bmaps.ensure((size_t)nj);
    std::vector<TileMap> maps(nj);
    bool any_map = false;
    b_px_maps = encode_tiled() != nullptr;
    for (int k = 0; k < nj; ++k)
    {
      const dic_job& J = jobs[b_order[k]];
      const int r = J.subset_radius;
      if (job_table(r) || !encode_tiled()) continue;
      const cuuint64_t dims[2] = {(cuuint64_t)J.width, (cuuint64_t)J.height};
      const cuuint64_t strides[1] = {(cuuint64_t)px_pitch(J.width) * sizeof(float)};
      const cuuint32_t box[2] = {(cuuint32_t)px_window_x(r), (cuuint32_t)px_window_y(r)};
      const cuuint32_t estr[2] = {1, 1};
      const CUresult res = encode_tiled()(&maps[k].map, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 2, const_cast<float*>(table[k].tar), dims,
                                          strides, box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
                                          CU_TENSOR_MAP_L2_PROMOTION_L2_128B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
      if (res != CUDA_SUCCESS)
        throw DicError{DIC_ERR_CUDA, "cuTensorMapEncodeTiled failed (" + std::to_string((int)res) + ")"};
      table[k].map = bmaps.ptr + k;
      any_map = true;
    }
    if (any_map)
    {
      b_maps_host.resize(nj);
      for (int k = 0; k < nj; ++k) b_maps_host[k] = maps[k].map;
      DIC_CUDA(cudaMemcpyAsync(bmaps.ptr, b_maps_host.data(), sizeof(CUtensorMap) * nj, cudaMemcpyHostToDevice, stream));
    }
    DIC_CUDA(cudaMemcpyAsync(bjobs.ptr, table.data(), sizeof(BatchJob) * nj, cudaMemcpyHostToDevice, stream));
  }

  // Everything from pixel upload to results, on the engine stream (capturable when the
  // pixels and queues are device memory).
  // Side streams of the batch's per-job preparation: each job's chain (uploads, planes,
  // per-POI prep, FFTCC) touches only that job's buffers and queue slice, so the chains run
  // side by side (in a captured batch they become parallel graph branches) and small jobs'
  // kernels share the GPU instead of running one after another.
  static constexpr int kBatchLanes = 4;
  cudaStream_t b_lane[kBatchLanes] = {};
  cudaEvent_t b_fork = nullptr, b_join[kBatchLanes] = {};
  void batch_lanes()
  {
    if (b_fork) return;
    for (int l = 0; l < kBatchLanes; ++l)
    {
      DIC_CUDA(cudaStreamCreateWithFlags(&b_lane[l], cudaStreamNonBlocking));
      DIC_CUDA(cudaEventCreateWithFlags(&b_join[l], cudaEventDisableTiming));
    }
    DIC_CUDA(cudaEventCreateWithFlags(&b_fork, cudaEventDisableTiming));
  }
  void release_batch_lanes()
  {
    for (int l = 0; l < kBatchLanes; ++l)
    {
      if (b_lane[l]) cudaStreamDestroy(b_lane[l]);
      if (b_join[l]) cudaEventDestroy(b_join[l]);
      b_lane[l] = nullptr;
      b_join[l] = nullptr;
    }
    if (b_fork) cudaEventDestroy(b_fork);
    b_fork = nullptr;
  }
  void enqueue_batch(const dic_job* jobs, int nj, bool on_device)
  {
    const cudaMemcpyKind in_kind = on_device ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice;
    mark(kPhFrame, 0);
    DIC_CUDA(cudaMemsetAsync(counters.ptr, 0, sizeof(unsigned long long), stream));
    DIC_CUDA(cudaMemsetAsync(bnext.ptr, 0, (2 + kMaxPairGroups) * sizeof(unsigned long long), stream));
    batch_lanes();
    DIC_CUDA(cudaEventRecord(b_fork, stream));
    for (int l = 0; l < kBatchLanes; ++l) DIC_CUDA(cudaStreamWaitEvent(b_lane[l], b_fork, 0));
    for (int k = 0; k < nj; ++k)
    {
      const dic_job& J = jobs[b_order[k]];
      JobBufs& M = jobs_mem[k];
      cudaStream_t st = b_lane[k % kBatchLanes];
      const int es = dtype_size(J.dtype);
      DIC_CUDA(cudaMemcpy2DAsync(M.raw_ref.ptr, (size_t)J.width * es, J.ref, (size_t)J.row_stride_bytes,
                                 (size_t)J.width * es, J.height, in_kind, st));
      DIC_CUDA(cudaMemcpy2DAsync(M.raw_tar.ptr, (size_t)J.width * es, J.tar, (size_t)J.row_stride_bytes,
                                 (size_t)J.width * es, J.height, in_kind, st));
      const bool table = job_table(J.subset_radius), pitched = job_pitched(J.subset_radius, J.width);
      switch (J.dtype)
      {
        case DIC_U8: prep_planes<uint8_t>(M.raw_ref.ptr, M.raw_tar.ptr, J.width, J.height, M, table, pitched, st); break;
        case DIC_U16: prep_planes<uint16_t>(M.raw_ref.ptr, M.raw_tar.ptr, J.width, J.height, M, table, pitched, st); break;
        default: prep_planes<float>(M.raw_ref.ptr, M.raw_tar.ptr, J.width, J.height, M, table, pitched, st); break;
      }
      if (J.count == 0) continue;
      const int r = J.subset_radius;
      dic_poi* q = bq.ptr + b_first[k];
      DIC_CUDA(cudaMemcpyAsync(q, J.pois, sizeof(dic_poi) * J.count, in_kind, st));
      k_poi_prepare32<<<(unsigned)((J.count + kPrepPois - 1) / kPrepPois), kPrepWarps * 32, 0, st>>>(
          M.ref_pack.ptr, J.width, J.height, q, J.count, r, r, bpoi.ptr + b_first[k]);
      check_launch("k_poi_prepare32");
      FftccParams fp{M.ref_f32.ptr, M.tar_f32.ptr, q, J.count, J.width, J.height};
      fftcc_launch(fp, r, st);
    }
    BatchLaunch col{bjobs.ptr, nj, bq.ptr, bpoi.ptr, 0, b_col_end, bnext.ptr, counters.ptr, b_col_rmax};
    BatchLaunch flat{bjobs.ptr, nj, bq.ptr, bpoi.ptr, b_pair_end, b_total, bnext.ptr + 1, counters.ptr};
    std::vector<BatchLaunch> pairs;
    for (size_t g = 0; g < b_pair_groups.size(); ++g)
      pairs.push_back(BatchLaunch{bjobs.ptr, nj, bq.ptr, bpoi.ptr, b_pair_groups[g].begin, b_pair_groups[g].end,
                                  bnext.ptr + 2 + g, counters.ptr, b_pair_groups[g].rmax});
    // the pair walk is tuned on its largest drain
    size_t pair_big = 0;
    for (size_t g = 1; g < pairs.size(); ++g)
      if (pairs[g].end - pairs[g].begin > pairs[pair_big].end - pairs[pair_big].begin) pair_big = g;
    for (int l = 0; l < kBatchLanes; ++l)
    {
      DIC_CUDA(cudaEventRecord(b_join[l], b_lane[l]));
      DIC_CUDA(cudaStreamWaitEvent(stream, b_join[l], 0));
    }
    const bool cap = capturing();
    const int col_walk = sampling == DIC_SAMPLE_PIXELS ? kWalkColumnPx : kWalkColumn;
    const int pair_walk = sampling == DIC_SAMPLE_PIXELS ? kWalkPairPx : kWalkPair;
    if (autotune && !cap)
    {
      if (b_col_end >= kTuneMinPois && !tuned[1][col_walk]) tune_batch(col, col_walk, b_total);
      if (!pairs.empty() && pairs[pair_big].end - pairs[pair_big].begin >= kTuneMinPois && !tuned[1][pair_walk])
        tune_batch(pairs[pair_big], pair_walk, b_total);
      if (b_total - b_pair_end >= kTuneMinPois && !tuned[1][kWalkFlat]) tune_batch(flat, kWalkFlat, b_total);
    }
    mark(kPhIcgn, 0);
    if (b_col_end > 0) launch_batch(col, col_walk, shape[1][col_walk]);
    for (const BatchLaunch& pl : pairs)
      if (pl.end > pl.begin) launch_batch(pl, pair_walk, shape[1][pair_walk]);
    if (b_total > b_pair_end) launch_batch(flat, kWalkFlat, shape[1][kWalkFlat]);
    mark(kPhIcgn, 1);
    for (int k = 0; k < nj; ++k)
    {
      const dic_job& J = jobs[b_order[k]];
      if (J.count == 0) continue;
      DIC_CUDA(cudaMemcpyAsync(J.pois, bq.ptr + b_first[k], sizeof(dic_poi) * J.count,
                               on_device ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost, stream));
    }
    mark(kPhFrame, 1);
  }

  static bool same_jobs(const std::vector<dic_job>& a, const dic_job* b, int nb)
  {
    if ((int)a.size() != nb) return false;
    for (int j = 0; j < nb; ++j)
      if (a[j].ref != b[j].ref || a[j].tar != b[j].tar || a[j].width != b[j].width || a[j].height != b[j].height ||
          a[j].row_stride_bytes != b[j].row_stride_bytes || a[j].dtype != b[j].dtype ||
          a[j].subset_radius != b[j].subset_radius || a[j].pois != b[j].pois || a[j].count != b[j].count)
        return false;
    return true;
  }
  void drop_batch_graph()
  {
    if (batch_graph) cudaGraphExecDestroy(batch_graph);
    batch_graph = nullptr;
  }

  // With device-resident pixels and queues and graphs enabled, a batch whose jobs repeat
  // (same pointers, sizes, radii and counts) is captured on its second call and replayed
  // from the third on; host-memory batches always run eagerly.
  void run_batch(const dic_job* jobs, int nj, bool on_device, dic_batch_report* rep)
  {
    const bool repeat = on_device && use_graphs && b_key_seen && same_jobs(b_key, jobs, nj);
    if (!repeat)
    {
      drop_batch_graph();
      b_key.assign(jobs, jobs + nj);
      b_key_seen = on_device && use_graphs;
      plan_batch(jobs, nj);
      enqueue_batch(jobs, nj, on_device);
    }
    else
    {
      if (!batch_graph)
      {
        plan_batch(jobs, nj);   // buffers already have their sizes: no allocation below
        const bool t = timing;
        timing = false;
        const long long l0 = launches;
        cudaGraph_t g = nullptr;
        DIC_CUDA(cudaStreamBeginCapture(stream, cudaStreamCaptureModeThreadLocal));
        try
        {
          enqueue_batch(jobs, nj, on_device);
        }
        catch (...)
        {
          cudaStreamEndCapture(stream, &g);
          if (g) cudaGraphDestroy(g);
          timing = t;
          throw;
        }
        DIC_CUDA(cudaStreamEndCapture(stream, &g));
        timing = t;
        batch_graph_kernels = (int)(launches - l0);
        launches = l0;
        cudaError_t ie = cudaGraphInstantiate(&batch_graph, g, 0);
        cudaGraphDestroy(g);
        if (ie != cudaSuccess)
        {
          batch_graph = nullptr;
          throw DicError{DIC_ERR_CUDA, std::string("cudaGraphInstantiate: ") + cudaGetErrorString(ie)};
        }
      }
      mark(kPhFrame, 0);
      DIC_CUDA(cudaGraphLaunch(batch_graph, stream));
      mark(kPhFrame, 1);
      launches += batch_graph_kernels;
    }
    DIC_CUDA(cudaStreamSynchronize(stream));
    iter_pending = true;
    icgn_pois = b_total;
    if (rep)
    {
      rep->pois = b_total;
      rep->jobs = nj;
      rep->graph = repeat ? 1 : 0;
      int64_t valid = 0;
      if (!on_device)
        for (int j = 0; j < nj; ++j)
          for (int64_t i = 0; i < jobs[j].count; ++i) valid += jobs[j].pois[i].zncc >= 0.f;
      rep->valid = on_device ? -1 : valid;
    }
  }

  void fill_report(dic_frame_report* r, int64_t n, bool use_skip, const dic_poi* host_results, bool learned = false)
  {
    if (!r) return;
    FrameCounters c{};
    DIC_CUDA(cudaMemcpyAsync(&c, fcount.ptr, sizeof(c), cudaMemcpyDeviceToHost, stream));
    DIC_CUDA(cudaStreamSynchronize(stream));
    check_wait_error();
    report_from(r, c, n, use_skip, host_results, learned);
  }
  void report_from(dic_frame_report* r, const FrameCounters& c, int64_t n, bool use_skip, const dic_poi* host_results,
                   bool learned)
  {
    if (!r) return;
    if (learned)
    {
      // learned seed: "before repair" = POIs the proposal's IC-GN did not bring to ZNCC 0.9
      r->pois = n;
      r->bad_before_repair = (int64_t)c.candidates;
      r->bad_after_repair = (int64_t)c.bad_after;
      r->repaired_candidates = (int64_t)c.candidates;
      r->repaired_recovered = (int64_t)c.recovered;
      r->frame_fallback_used = 0;
      r->fftcc_used = c.candidates > 0 ? 1 : 0;
      double it = 0.0;
      int64_t valid = 0;
      if (host_results)
        for (int64_t i = 0; i < n; ++i)
          if (host_results[i].zncc >= 0.f) { it += host_results[i].iteration; ++valid; }
      r->iteration_mean = valid ? it / (double)valid : 0.0;
      return;
    }
    r->pois = n;
    r->bad_before_repair = (int64_t)c.bad;
    r->bad_after_repair = (int64_t)c.bad_after;
    r->repaired_candidates = use_skip && c.poi_repair ? (int64_t)c.candidates : 0;
    r->repaired_recovered = use_skip && c.poi_repair ? (int64_t)c.recovered : 0;
    r->temporal_seed_count = use_skip ? (int64_t)c.temporal : 0;
    r->frame_fallback_used = use_skip ? c.frame_fallback : 0;
    r->fftcc_used = (!use_skip || c.frame_fallback || c.poi_repair) ? 1 : 0;
    double it = 0.0;
    int64_t valid = 0;
    if (host_results)
      for (int64_t i = 0; i < n; ++i)
        if (host_results[i].zncc >= 0.f) { it += host_results[i].iteration; ++valid; }
    r->iteration_mean = valid ? it / (double)valid : 0.0;
  }

  // IC-GN on the device queue `queue` whose host copy is `pois`.
  void icgn_queue(const dic_poi* host_pois, int64_t n)
  {
    if (!layout_matches(host_pois, n))
    {
      record_layout(host_pois, n);
      prepare_layout_device(queue.ptr, n);
    }
    run_icgn(queue.ptr, n, nullptr);
  }
};

namespace
{

template <typename F>
int guarded(dic_engine* e, F&& f, bool new_call = true)
{
  if (!e) return DIC_ERR_ARGUMENT;
  try
  {
    int dev = 0;
    cudaGetDevice(&dev);
    if (dev != e->cfg.device) DIC_CUDA(cudaSetDevice(e->cfg.device));
    if (new_call) e->begin_call();
    f();
    e->last_error.clear();
    return DIC_OK;
  }
  catch (const DicError& err)
  {
    e->last_error = err.msg;
    return err.code;
  }
  catch (const std::exception& ex)
  {
    e->last_error = ex.what();
    return DIC_ERR_MEMORY;
  }
}

bool finite_xy(const dic_poi& p) { return std::isfinite(p.x) && std::isfinite(p.y); }

}  // namespace

extern "C" {

const char* dic_version(void) { return kVersion; }

int dic_host_alloc(size_t bytes, void** ptr)
{
  if (!ptr) return DIC_ERR_ARGUMENT;
  *ptr = nullptr;
  if (cudaMallocHost(ptr, bytes ? bytes : 1) != cudaSuccess)
  {
    cudaGetLastError();
    *ptr = nullptr;
    return DIC_ERR_MEMORY;
  }
  return DIC_OK;
}

void dic_host_free(void* ptr)
{
  if (ptr) cudaFreeHost(ptr);
}
int32_t dic_abi_version(void) { return DIC_ABI_VERSION; }

int dic_engine_create(const dic_config* config, dic_engine** out)
{
  if (!config || !out) return DIC_ERR_ARGUMENT;
  *out = nullptr;
  if (config->subset_radius_x < 1 || config->subset_radius_y < 1 || config->max_iteration < 1 ||
      !(config->conv_criterion >= 0.f))
    return DIC_ERR_ARGUMENT;
  dic_engine* e = new (std::nothrow) dic_engine();
  if (!e) return DIC_ERR_MEMORY;
  e->cfg = *config;
  try
  {
    DIC_CUDA(cudaSetDevice(config->device));
    init_constants(config->device);
    DIC_CUDA(cudaStreamCreateWithFlags(&e->stream, cudaStreamNonBlocking));
    if (const char* t = std::getenv("DIC_TEST_WAIT_FAULT"))
    {
      e->wait_test = std::atoi(t) & 3;
      if (e->wait_test) e->wait_polls = dic_engine::kTestWaitPolls;
    }
    DIC_CUDA(cudaFuncSetAttribute(k_fftcc_large, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                  (int)(2 * kMaxTwiddleN * (kMaxTwiddleN + 1) * sizeof(float2))));
    DIC_CUDA(cudaFuncSetAttribute(cnn::k_proposal_fused, cudaFuncAttributeMaxDynamicSharedMemorySize, cnn::kSmTotal));
    for (int p = 0; p < kPhCount; ++p)
      for (int m = 0; m < dic_engine::kMarks; ++m)
        for (int k = 0; k < 2; ++k) DIC_CUDA(cudaEventCreate(&e->ev[p][m][k]));
  }
  catch (const DicError& err)
  {
    std::fprintf(stderr, "dic_engine_create: %s\n", err.msg.c_str());
    delete e;
    return err.code;
  }
  *out = e;
  return DIC_OK;
}

int dic_device_info(int32_t device, char* name, int32_t name_capacity, int32_t* cc_major, int32_t* cc_minor,
                    int32_t* driver_version, int32_t* runtime_version)
{
  cudaDeviceProp prop{};
  if (cudaGetDeviceProperties(&prop, device) != cudaSuccess) return DIC_ERR_CUDA;
  if (name && name_capacity > 0)
  {
    std::strncpy(name, prop.name, (size_t)name_capacity - 1);
    name[name_capacity - 1] = 0;
  }
  if (cc_major) *cc_major = prop.major;
  if (cc_minor) *cc_minor = prop.minor;
  int d = 0, r = 0;
  if (driver_version) *driver_version = cudaDriverGetVersion(&d) == cudaSuccess ? d : 0;
  if (runtime_version) *runtime_version = cudaRuntimeGetVersion(&r) == cudaSuccess ? r : 0;
  return DIC_OK;
}

void dic_engine_destroy(dic_engine* e)
{
  if (!e) return;
  cudaSetDevice(e->cfg.device);
  if (e->stream) cudaStreamSynchronize(e->stream);
  e->raw_ref.release();
  e->raw_tar.release();
  e->ref_f32.release();
  e->tar_f32.release();
  e->tar_px.release();
  e->ref_pack.release();
  e->coef.release();
  e->lattice.release();
  e->poi_ref.release();
  e->queue.release();
  e->slots.release();
  e->counters.release();
  if (e->seq_graph) cudaGraphExecDestroy(e->seq_graph);
  e->drop_batch_graph();
  for (auto& ev : e->tune_ev)
    if (ev) cudaEventDestroy(ev);
  e->tmpl.release();
  e->prev.release();
  e->scratch.release();
  e->fq.release();
  e->cand.release();
  e->fcount.release();
  e->baseline.release();
  for (auto& J : e->jobs_mem) J.release();
  e->bq.release();
  e->bpoi.release();
  e->bjobs.release();
  e->bmaps.release();
  e->bnext.release();
  e->icgn_next.release();
  e->wait_err.release();
  e->tune_q.release();
  e->release_staging();
  e->release_batch_lanes();
  e->release_frame_outputs();
  e->release_queue_upload();
  for (int p = 0; p < kPhCount; ++p)
    for (int m = 0; m < dic_engine::kMarks; ++m)
      for (int k = 0; k < 2; ++k)
        if (e->ev[p][m][k]) cudaEventDestroy(e->ev[p][m][k]);
  if (e->stream) cudaStreamDestroy(e->stream);
  delete e;
}

const char* dic_last_error(const dic_engine* e) { return e ? e->last_error.c_str() : "null engine"; }
void* dic_stream(dic_engine* e) { return e ? (void*)e->stream : nullptr; }

int dic_set_ref(dic_engine* e, const void* px, int32_t w, int32_t h, int64_t stride, int32_t dtype)
{
  return guarded(e, [&] { e->set_image(true, px, w, h, stride, dtype, false); });
}
int dic_set_tar(dic_engine* e, const void* px, int32_t w, int32_t h, int64_t stride, int32_t dtype)
{
  return guarded(e, [&] {
    if (e->ref_set && (w != e->w || h != e->h))
      throw DicError{DIC_ERR_ARGUMENT, "reference and target image sizes must match"};
    e->set_image(false, px, w, h, stride, dtype, false);
  });
}
int dic_set_ref_device(dic_engine* e, const void* px, int32_t w, int32_t h, int64_t stride, int32_t dtype)
{
  return guarded(e, [&] { e->set_image(true, px, w, h, stride, dtype, true); });
}
int dic_set_tar_device(dic_engine* e, const void* px, int32_t w, int32_t h, int64_t stride, int32_t dtype)
{
  return guarded(e, [&] {
    if (e->ref_set && (w != e->w || h != e->h))
      throw DicError{DIC_ERR_ARGUMENT, "reference and target image sizes must match"};
    e->set_image(false, px, w, h, stride, dtype, true);
  });
}

int dic_prepare_ref(dic_engine* e, const dic_poi* pois, int64_t n)
{
  return guarded(e, [&] {
    if (n < 0 || (n > 0 && !pois)) throw DicError{DIC_ERR_ARGUMENT, "prepare_ref: bad queue"};
    for (int64_t i = 0; i < n; ++i)
      if (!finite_xy(pois[i])) throw DicError{DIC_ERR_ARGUMENT, "prepare_ref: non-finite POI coordinate"};
    e->ensure_ref();
    e->record_layout(pois, n);
    e->upload_queue(pois, n);
    e->prepare_layout_device(e->queue.ptr, n);
    DIC_CUDA(cudaStreamSynchronize(e->stream));
  });
}

int dic_prepare_tar(dic_engine* e)
{
  return guarded(e, [&] {
    e->ensure_tar();
    DIC_CUDA(cudaStreamSynchronize(e->stream));
  });
}

int dic_fftcc(dic_engine* e, dic_poi* pois, int64_t n, const int64_t* cache_idx)
{
  return guarded(e, [&] {
    if (n < 0 || (n > 0 && !pois)) throw DicError{DIC_ERR_ARGUMENT, "fftcc: bad queue"};
    if (e->cfg.subset_radius_x != e->cfg.subset_radius_y)
      throw DicError{DIC_ERR_ARGUMENT, "FFTCC2D supports positive square radii only"};
    if (!e->ref_set || !e->tar_set) throw DicError{DIC_ERR_STATE, "FFTCC2D images must be set before compute"};
    if (cache_idx)
    {
      // FFTCC2D::compute(queue, cache_indices) checks (src/oc_fftcc.cpp:498-527).
      if (n == 0) return;
      if (!e->layout_ready || e->layout_x.empty())
        throw DicError{DIC_ERR_STATE, "FFTCC2D indexed compute requires a prepared reference layout"};
      for (int64_t i = 0; i < n; ++i)
      {
        const int64_t k = cache_idx[i];
        if (k < 0 || k >= (int64_t)e->layout_x.size())
          throw DicError{DIC_ERR_RANGE, "FFTCC2D reference cache index out of range"};
        if (!finite_xy(pois[i]) || e->layout_x[k] != (int)pois[i].x || e->layout_y[k] != (int)pois[i].y)
          throw DicError{DIC_ERR_ARGUMENT, "FFTCC2D reference cache index does not match POI coordinates"};
      }
    }
    if (n == 0) return;
    e->upload_queue(pois, n);
    e->run_fftcc(e->queue.ptr, n);
    e->download_queue(pois, n);
  });
}

int dic_icgn(dic_engine* e, dic_poi* pois, int64_t n)
{
  return guarded(e, [&] {
    if (n < 0 || (n > 0 && !pois)) throw DicError{DIC_ERR_ARGUMENT, "icgn: bad queue"};
    if (!e->ref_set || !e->tar_set) throw DicError{DIC_ERR_STATE, "ICGN images must be set before compute"};
    if (n == 0) return;
    e->upload_queue(pois, n);
    e->icgn_queue(pois, n);
    e->download_queue(pois, n);
  });
}

int dic_process_pair(dic_engine* e, dic_poi* pois, int64_t n)
{
  return guarded(e, [&] {
    if (n < 0 || (n > 0 && !pois)) throw DicError{DIC_ERR_ARGUMENT, "process_pair: bad queue"};
    if (!e->ref_set || !e->tar_set) throw DicError{DIC_ERR_STATE, "images must be set before compute"};
    if (e->cfg.subset_radius_x != e->cfg.subset_radius_y)
      throw DicError{DIC_ERR_ARGUMENT, "FFTCC2D supports positive square radii only"};
    if (n == 0) return;
    // the queue's upload overlaps the reference and target preparation, which do not read it
    e->upload_queue_beside(pois, n);
    // If the preparation throws (an allocation or a launch fails), the copy is still joined
    // to the engine stream and waited for before the error returns: later engine work on
    // the queue buffer stays ordered after it, and the caller may free its source at once.
    struct JoinOnError
    {
      dic_engine* e;
      ~JoinOnError()
      {
        if (!e) return;
        cudaStreamWaitEvent(e->stream, e->qup_done, 0);
        cudaEventSynchronize(e->qup_done);
      }
    } join_on_error{e};
    e->ensure_ref();
    e->ensure_tar();
    join_on_error.e = nullptr;
    e->join_queue_upload();
    // FFTCC reads only (x, y, u, v) and writes the seed; the per-POI reference data reads
    // only (x, y).  Launching FFTCC first lets the host's layout check and record (a pass
    // over the queue) run while the GPU works.
    e->run_fftcc(e->queue.ptr, n);
    if (!e->layout_matches(pois, n))
    {
      e->record_layout(pois, n);
      e->prepare_layout_device(e->queue.ptr, n);
    }
    e->run_icgn(e->queue.ptr, n, nullptr);
    e->download_queue(pois, n);
  });
}

int dic_split_rows(const dic_poi* pois, int64_t n, int32_t parts, int64_t* starts)
{
  if (parts < 1 || n < 0 || (n > 0 && !pois) || !starts) return DIC_ERR_ARGUMENT;
  // Cut k at the first row start at or after k * n / parts, so that no row of POIs (equal y,
  // contiguous in buildPoiQueue order) is split between two parts.
  starts[0] = 0;
  for (int32_t k = 1; k < parts; ++k)
  {
    int64_t c = std::max<int64_t>(starts[k - 1], (int64_t)((__int128)n * k / parts));
    while (c > 0 && c < n && pois[c].y == pois[c - 1].y) ++c;
    starts[k] = c;
  }
  starts[parts] = n;
  return DIC_OK;
}

int dic_process_pair_multi(dic_engine* const* engines, int32_t count, dic_poi* pois, int64_t n, int64_t* band_starts)
{
  if (!engines || count < 1 || n < 0 || (n > 0 && !pois)) return DIC_ERR_ARGUMENT;
  for (int32_t k = 0; k < count; ++k)
    if (!engines[k]) return DIC_ERR_ARGUMENT;
  std::vector<int64_t> starts(count + 1);
  const int rc = dic_split_rows(pois, n, count, starts.data());
  if (rc != DIC_OK) return rc;
  if (band_starts) std::copy(starts.begin(), starts.end(), band_starts);
  // one host thread per engine (each engine keeps its one-thread-per-handle rule); the bands
  // are disjoint ranges of the caller's queue, so the results land in queue order
  std::vector<int> status(count, DIC_OK);
  std::vector<std::thread> workers;
  workers.reserve(count);
  for (int32_t k = 0; k < count; ++k)
    workers.emplace_back([&, k] {
      status[k] = dic_process_pair(engines[k], pois + starts[k], starts[k + 1] - starts[k]);
    });
  for (auto& w : workers) w.join();
  for (int32_t k = 0; k < count; ++k)
    if (status[k] != DIC_OK) return status[k];
  return DIC_OK;
}

int dic_run_device(dic_engine* e, dic_poi* d_pois, int64_t n, int32_t flags)
{
  return guarded(e, [&] {
    if (n < 0 || (n > 0 && !d_pois)) throw DicError{DIC_ERR_ARGUMENT, "run_device: bad queue"};
    if (!e->ref_set || !e->tar_set) throw DicError{DIC_ERR_STATE, "images must be set before compute"};
    if (n == 0) return;
    // The device queue defines the layout when asked to (DIC_RUN_PREPARE), when no layout of
    // this size is resident, or when the reference changed; otherwise it is trusted to hold
    // the resident layout's integer (x, y).  A device-defined layout has no host copy, so
    // the next host-queue call prepares its own.
    if ((flags & DIC_RUN_PREPARE) || !e->layout_ready || e->layout_count != n || e->ref_dirty)
    {
      e->layout_x.clear();
      e->layout_y.clear();
      e->prepare_layout_device(d_pois, n);
    }
    if (flags & DIC_RUN_LEARNED)
    {
      // the learned path works on the engine queue; device records are copied in and out
      e->queue.ensure((size_t)n);
      DIC_CUDA(cudaMemcpyAsync(e->queue.ptr, d_pois, sizeof(dic_poi) * n, cudaMemcpyDeviceToDevice, e->stream));
      e->enqueue_learned(n);
      DIC_CUDA(cudaMemcpyAsync(d_pois, e->queue.ptr, sizeof(dic_poi) * n, cudaMemcpyDeviceToDevice, e->stream));
      e->iter_pending = true;
      return;
    }
    if (flags & DIC_RUN_FFTCC) e->run_fftcc(d_pois, n);
    if (flags & DIC_RUN_ICGN) e->run_icgn(d_pois, n, nullptr);
  });
}

int dic_process_frame(dic_engine* e, dic_poi* pois, int64_t n, const dic_poi* prev,
                      const dic_frame_policy* policy, dic_frame_report* report)
{
  return dic_process_frame_history(e, pois, n, prev, nullptr, policy, report);
}

int dic_process_frame_history(dic_engine* e, dic_poi* pois, int64_t n, const dic_poi* prev, const dic_poi* prev_prev,
                              const dic_frame_policy* policy, dic_frame_report* report)
{
  return guarded(e, [&] {
    if (n < 0 || (n > 0 && !pois) || !policy) throw DicError{DIC_ERR_ARGUMENT, "process_frame: bad arguments"};
    if (!e->ref_set || !e->tar_set) throw DicError{DIC_ERR_STATE, "images must be set before compute"};
    if (e->cfg.subset_radius_x != e->cfg.subset_radius_y)
      throw DicError{DIC_ERR_ARGUMENT, "FFTCC2D supports positive square radii only"};
    if (report) *report = dic_frame_report{};
    if (n == 0) return;
    e->ensure_frame_buffers(n);
    e->counters.ensure(1);
    DIC_CUDA(cudaMemcpyAsync(e->tmpl.ptr, pois, sizeof(dic_poi) * n, cudaMemcpyHostToDevice, e->stream));
    const bool use_skip = policy->skip_fftcc && prev != nullptr;
    if (use_skip)
      DIC_CUDA(cudaMemcpyAsync(e->prev.ptr, prev, sizeof(dic_poi) * n, cudaMemcpyHostToDevice, e->stream));
    const bool with_prev2 = use_skip && prev_prev != nullptr && policy->temporal_extrapolation;
    if (with_prev2)
      DIC_CUDA(cudaMemcpyAsync(e->prev2.ptr, prev_prev, sizeof(dic_poi) * n, cudaMemcpyHostToDevice, e->stream));
    if (!e->layout_matches(pois, n))
    {
      e->record_layout(pois, n);
      e->prepare_layout_device(e->tmpl.ptr, n);
    }
    e->enqueue_frame(n, use_skip, *policy, nullptr, policy->frame_fallback_ratio, with_prev2 ? e->prev2.ptr : nullptr,
                     nullptr);
    e->iter_pending = true;
    e->download_queue(pois, n);
    e->fill_report(report, n, use_skip, pois);
  });
}

int dic_sequence_begin(dic_engine* e, const dic_poi* pois, int64_t n, const dic_frame_policy* policy)
{
  return guarded(e, [&] {
    if (n <= 0 || !pois || !policy) throw DicError{DIC_ERR_ARGUMENT, "sequence_begin: bad arguments"};
    if (!e->ref_set) throw DicError{DIC_ERR_STATE, "reference image must be set before a sequence"};
    if (e->cfg.subset_radius_x != e->cfg.subset_radius_y)
      throw DicError{DIC_ERR_ARGUMENT, "FFTCC2D supports positive square radii only"};
    for (int64_t i = 0; i < n; ++i)
      if (!finite_xy(pois[i])) throw DicError{DIC_ERR_ARGUMENT, "sequence_begin: non-finite POI coordinate"};
    if (e->seq_graph)
    {
      cudaGraphExecDestroy(e->seq_graph);
      e->seq_graph = nullptr;
    }
    e->ensure_frame_buffers(n);
    e->counters.ensure(1);
    DIC_CUDA(cudaMemcpyAsync(e->tmpl.ptr, pois, sizeof(dic_poi) * n, cudaMemcpyHostToDevice, e->stream));
    e->record_layout(pois, n);
    e->prepare_layout_device(e->tmpl.ptr, n);
    const float inf = INFINITY;
    DIC_CUDA(cudaMemcpyAsync(e->baseline.ptr, &inf, sizeof(float), cudaMemcpyHostToDevice, e->stream));
    DIC_CUDA(cudaMemsetAsync(e->hist.ptr, 0, sizeof(int), e->stream));
    DIC_CUDA(cudaStreamSynchronize(e->stream));
    e->seq_policy = *policy;
    e->seq_n = n;
    e->seq_frame = 0;
    e->seq_out_frame[0] = e->seq_out_frame[1] = -1;
  });
}

int dic_sequence_frame(dic_engine* e, const void* px, int32_t w, int32_t h, int64_t stride, int32_t dtype,
                       int32_t pixels_on_device, dic_poi* results, dic_frame_report* report)
{
  return guarded(e, [&] {
    if (e->seq_n <= 0) throw DicError{DIC_ERR_STATE, "dic_sequence_begin must come first"};
    if (w != e->w || h != e->h) throw DicError{DIC_ERR_ARGUMENT, "reference and target image sizes must match"};
    if (report) *report = dic_frame_report{};
    const int64_t n = e->seq_n;
    if (e->ref_dirty || !e->layout_ready || e->layout_count != n)
      throw DicError{DIC_ERR_STATE, "the reference or the POI layout changed; call dic_sequence_begin again"};
    const dic_frame_policy& pol = e->seq_policy;
    const bool learned = pol.learned_seed != 0;
    if (learned && !e->proposal) throw DicError{DIC_ERR_STATE, "learned-seed sequence without a proposal network"};
    if (pixels_on_device == DIC_PIXELS_STAGED)
      e->take_staged(w, h, dtype);
    else
      e->set_image(false, px, w, h, stride, dtype, pixels_on_device != 0);
    const bool use_skip = !learned && pol.skip_fftcc && e->seq_frame > 0;
    // the steady-state frame (learned: every frame after the first; skip-FFTCC: every seeded
    // frame): target table, seeds, IC-GN, repair paths behind device switches, merge, count,
    // results -> prev
    const bool temporal = !learned && pol.temporal_extrapolation != 0;
    // results -> prev (and, for temporal extrapolation, prev -> prev2 first and one more frame
    // of history; the seed kernel reads the depth on the device, so a captured frame stays valid)
    auto shift_history = [&] {
      if (temporal)
        DIC_CUDA(cudaMemcpyAsync(e->prev2.ptr, e->prev.ptr, sizeof(dic_poi) * n, cudaMemcpyDeviceToDevice, e->stream));
      DIC_CUDA(cudaMemcpyAsync(e->prev.ptr, e->queue.ptr, sizeof(dic_poi) * n, cudaMemcpyDeviceToDevice, e->stream));
      if (temporal)
      {
        k_bump_history<<<1, 32, 0, e->stream>>>(e->hist.ptr);
        e->check_launch("k_bump_history");
      }
    };
    auto steady = [&] {
      e->ensure_tar();
      if (learned)
        e->enqueue_learned(n, true, pol.zncc_threshold);
      else
        e->enqueue_frame(n, true, pol, e->baseline.ptr, 0.f, e->prev2.ptr, e->hist.ptr);
      shift_history();
    };
    e->mark(kPhFrame, 0);
    if (!use_skip && !(learned && e->seq_frame > 0))
    {
      e->ensure_tar();
      if (learned)
        e->enqueue_learned(n, true, pol.zncc_threshold);
      else
      {
        e->enqueue_frame(n, false, pol, nullptr, INFINITY);
        if (pol.skip_fftcc && e->seq_frame == 0)
        {
          k_set_baseline<<<1, 32, 0, e->stream>>>(e->fcount.ptr, n, pol.frame_fallback_ratio, e->baseline.ptr);
          e->check_launch("k_set_baseline");
        }
      }
      shift_history();
    }
    else if (e->use_graphs)
    {
      if (!e->seq_graph)
      {
        // Capture the steady-state frame once (all buffers exist after the first frame).
        const bool timing = e->timing;
        e->timing = false;
        e->tar_dirty = true;
        const int64_t l0 = e->launches;
        cudaGraph_t g = nullptr;
        DIC_CUDA(cudaStreamBeginCapture(e->stream, cudaStreamCaptureModeThreadLocal));
        try
        {
          steady();
        }
        catch (...)
        {
          cudaStreamEndCapture(e->stream, &g);
          if (g) cudaGraphDestroy(g);
          e->timing = timing;
          throw;
        }
        DIC_CUDA(cudaStreamEndCapture(e->stream, &g));
        e->timing = timing;
        e->seq_graph_kernels = (int)(e->launches - l0);
        e->launches = l0;
        cudaError_t ie = cudaGraphInstantiate(&e->seq_graph, g, 0);
        cudaGraphDestroy(g);
        if (ie != cudaSuccess)
        {
          e->seq_graph = nullptr;
          throw DicError{DIC_ERR_CUDA, std::string("cudaGraphInstantiate: ") + cudaGetErrorString(ie)};
        }
      }
      DIC_CUDA(cudaGraphLaunch(e->seq_graph, e->stream));
      e->launches += e->seq_graph_kernels;
      e->tar_dirty = false;
    }
    else
      steady();
    e->mark(kPhFrame, 1);
    e->iter_pending = true;
    e->icgn_pois = n;
    e->save_frame_output(n, use_skip);
    if (results)
      DIC_CUDA(cudaMemcpyAsync(results, e->queue.ptr, sizeof(dic_poi) * n, cudaMemcpyDeviceToHost, e->stream));
    if (results || report)
    {
      DIC_CUDA(cudaStreamSynchronize(e->stream));
      e->check_wait_error();
    }
    e->fill_report(report, n, use_skip, results, learned);
    e->seq_last_skip = use_skip;
    ++e->seq_frame;
  });
}

int dic_sequence_fetch(dic_engine* e, int32_t frames_back, dic_poi* results, dic_frame_report* report)
{
  return guarded(e, [&] {
    if (frames_back != 0 && frames_back != 1) throw DicError{DIC_ERR_ARGUMENT, "sequence_fetch: frames_back must be 0 or 1"};
    const long long frame = e->seq_frame - 1 - frames_back;
    const int slot = (int)(frame & 1);
    if (frame < 0 || e->seq_out_frame[slot] != frame)
      throw DicError{DIC_ERR_STATE, "sequence_fetch: that frame of this sequence has not been solved"};
    const int64_t n = e->seq_n;
    if (report) *report = dic_frame_report{};
    // on the download stream: the engine stream may already be solving the next frame
    FrameCounters c{};
    DIC_CUDA(cudaStreamWaitEvent(e->down_stream, e->seq_done[slot], 0));
    if (results)
      DIC_CUDA(cudaMemcpyAsync(results, e->seq_out[slot].ptr, sizeof(dic_poi) * n, cudaMemcpyDeviceToHost,
                               e->down_stream));
    DIC_CUDA(cudaMemcpyAsync(&c, e->seq_cnt[slot].ptr, sizeof(c), cudaMemcpyDeviceToHost, e->down_stream));
    int wait_flag = 0;   // a bounded wait of this frame's kernels that ran out
    if (e->wait_err.ptr)
      DIC_CUDA(cudaMemcpyAsync(&wait_flag, e->wait_err.ptr, sizeof(int), cudaMemcpyDeviceToHost, e->down_stream));
    DIC_CUDA(cudaStreamSynchronize(e->down_stream));
    if (wait_flag) throw DicError{DIC_ERR_CUDA, dic_engine::wait_error_text(wait_flag)};
    e->report_from(report, c, n, e->seq_out_skip[slot], results, e->seq_policy.learned_seed != 0);
  });
}

int dic_set_proposal(dic_engine* e, dic_cnn* net)
{
  return guarded(e, [&] {
    if (net && net->device != e->cfg.device)
      throw DicError{DIC_ERR_ARGUMENT, "the proposal network lives on another device"};
    e->proposal = net;
    if (e->seq_graph)
    {
      cudaGraphExecDestroy(e->seq_graph);   // it holds the previous network's weight pointers
      e->seq_graph = nullptr;
    }
  });
}

int dic_stage_frame(dic_engine* e, const void* pixels, int32_t width, int32_t height, int64_t row_stride_bytes,
                    int32_t dtype)
{
  return guarded(e, [&] { e->stage_frame(pixels, width, height, row_stride_bytes, dtype); });
}

int dic_process_pair_learned(dic_engine* e, dic_poi* pois, int64_t n, dic_frame_report* report)
{
  return guarded(e, [&] {
    if (n < 0 || (n > 0 && !pois)) throw DicError{DIC_ERR_ARGUMENT, "process_pair_learned: bad queue"};
    if (!e->ref_set || !e->tar_set) throw DicError{DIC_ERR_STATE, "images must be set before compute"};
    if (e->cfg.subset_radius_x != e->cfg.subset_radius_y)
      throw DicError{DIC_ERR_ARGUMENT, "FFTCC2D supports positive square radii only"};
    if (report) *report = dic_frame_report{};
    if (n == 0) return;
    e->counters.ensure(1);
    e->upload_queue(pois, n);
    if (!e->layout_matches(pois, n))
    {
      e->record_layout(pois, n);
      e->prepare_layout_device(e->queue.ptr, n);
    }
    e->enqueue_learned(n);
    e->iter_pending = true;
    e->icgn_pois = n;
    e->download_queue(pois, n);
    e->fill_report(report, n, true, pois, true);
  });
}

int dic_batch_process(dic_engine* e, const dic_job* jobs, int32_t njobs, int32_t pixels_on_device,
                      dic_batch_report* report)
{
  return guarded(e, [&] {
    if (njobs <= 0 || !jobs) throw DicError{DIC_ERR_ARGUMENT, "batch: no jobs"};
    if (report) *report = dic_batch_report{};
    for (int j = 0; j < njobs; ++j)
    {
      const dic_job& J = jobs[j];
      const int es = dtype_size(J.dtype);
      if (!J.ref || !J.tar || es == 0 || J.width < 5 || J.height < 5 || J.row_stride_bytes < (int64_t)J.width * es ||
          J.count < 0 || (J.count > 0 && !J.pois) || J.subset_radius < 1 || 2 * J.subset_radius > kMaxTwiddleN)
        throw DicError{DIC_ERR_ARGUMENT, "batch job " + std::to_string(j) +
                                             ": bad image, queue or subset radius (square, 1..32)"};
      dic_engine::check_pixel_count(J.width, J.height);
    }
    e->run_batch(jobs, njobs, pixels_on_device != 0, report);
  });
}

int dic_set_autotune(dic_engine* e, int32_t enabled)
{
  return guarded(e, [&] {
    e->autotune = enabled != 0;
    for (auto& row : e->tuned)
      for (bool& t : row) t = false;
  });
}

int dic_get_tuning(dic_engine* e, dic_tuning* out)
{
  return guarded(e, [&] {
    if (!out) throw DicError{DIC_ERR_ARGUMENT, "get_tuning: null output"};
    for (int pers = 0; pers < 2; ++pers)
      for (int walk = 0; walk < dic_engine::kWalks; ++walk)
      {
        dic_launch_shape& d = pers ? out->batch[walk] : out->icgn[walk];
        const auto& s = e->shape[pers][walk];
        d.warps_per_cta = s.warps;
        d.ctas_per_sm = s.ctas_per_sm;
        d.tuned = e->tuned[pers][walk] ? 1 : 0;
        d.ms = s.ms;
        d.tile = s.tile;
        d.warps_per_poi = walk == dic_engine::kWalkPair || walk == dic_engine::kWalkPairPx ? s.poi_warps : 1;
      }
  }, false);
}

int dic_set_launch_shape(dic_engine* e, int32_t walk, const dic_launch_shape* shape)
{
  return guarded(e, [&] {
    if (!shape) throw DicError{DIC_ERR_ARGUMENT, "set_launch_shape: null shape"};
    if (walk < 0 || walk >= dic_engine::kWalks)
      throw DicError{DIC_ERR_ARGUMENT, "set_launch_shape: walk must be 0 (flat), 1 (column), 2 (pair), 3 (column, "
                                       "pixel sampling) or 4 (pair, pixel sampling)"};
    dic_engine::IcgnShape sh;
    if (walk == dic_engine::kWalkColumnPx || walk == dic_engine::kWalkPairPx)
    {
      if (shape->warps_per_cta != 2 && shape->warps_per_cta != 4 && shape->warps_per_cta != 8)
        throw DicError{DIC_ERR_ARGUMENT, "set_launch_shape: warps_per_cta must be 2, 4 or 8"};
      if (shape->ctas_per_sm < 0) throw DicError{DIC_ERR_ARGUMENT, "set_launch_shape: ctas_per_sm must be >= 0"};
      if (shape->tile < 0 || shape->tile > 2)
        throw DicError{DIC_ERR_ARGUMENT, "set_launch_shape: tile must be 0, 1 or 2 with walks 3 and 4"};
      const int pw = shape->warps_per_poi == 0 ? 1 : shape->warps_per_poi;
      if (pw != 1 && !(pw == 2 && walk == dic_engine::kWalkPairPx))
        throw DicError{DIC_ERR_ARGUMENT, "set_launch_shape: warps_per_poi must be 1, or 2 with the pair walks"};
      sh = dic_engine::IcgnShape{shape->warps_per_cta, shape->ctas_per_sm, 0.f, shape->tile, pw};
    }
    else if (shape->tile != 0)
    {
      if (shape->tile < 0 || shape->tile > 2 || walk != dic_engine::kWalkColumn)
        throw DicError{DIC_ERR_ARGUMENT, "set_launch_shape: tile must be 0, or 1 or 2 with the column walk"};
      const auto& k = dic_engine::kTileKinds[shape->tile];
      sh = dic_engine::IcgnShape{k.warps, k.ctas, 0.f, shape->tile};
    }
    else
    {
      if (shape->warps_per_cta != 2 && shape->warps_per_cta != 4 && shape->warps_per_cta != 8)
        throw DicError{DIC_ERR_ARGUMENT, "set_launch_shape: warps_per_cta must be 2, 4 or 8"};
      if (shape->ctas_per_sm < 0) throw DicError{DIC_ERR_ARGUMENT, "set_launch_shape: ctas_per_sm must be >= 0"};
      const int pw = shape->warps_per_poi == 0 ? 1 : shape->warps_per_poi;
      if (pw != 1 && !(pw == 2 && walk == dic_engine::kWalkPair))
        throw DicError{DIC_ERR_ARGUMENT, "set_launch_shape: warps_per_poi must be 1, or 2 with the pair walk"};
      sh = dic_engine::IcgnShape{shape->warps_per_cta, shape->ctas_per_sm, 0.f, 0, pw};
    }
    e->shape[0][walk] = sh;
    e->tuned[0][walk] = false;
    if (e->seq_graph)
    {
      // a captured sequence frame holds the previous launch
      cudaGraphExecDestroy(e->seq_graph);
      e->seq_graph = nullptr;
    }
  });
}

int dic_set_sampling(dic_engine* e, int32_t mode)
{
  return guarded(e, [&] {
    if (mode != DIC_SAMPLE_TABLE && mode != DIC_SAMPLE_PIXELS)
      throw DicError{DIC_ERR_ARGUMENT, "set_sampling: mode must be DIC_SAMPLE_TABLE or DIC_SAMPLE_PIXELS"};
    if (mode == e->sampling) return;
    e->sampling = mode;
    e->drop_batch_graph();   // a captured batch holds the previous kernels
    if (e->seq_graph)
    {
      // a captured sequence frame holds the previous solver
      cudaGraphExecDestroy(e->seq_graph);
      e->seq_graph = nullptr;
    }
  });
}

int dic_set_graphs(dic_engine* e, int32_t enabled)
{
  return guarded(e, [&] {
    e->use_graphs = enabled != 0;
    if (!e->use_graphs && e->seq_graph)
    {
      cudaGraphExecDestroy(e->seq_graph);
      e->seq_graph = nullptr;
    }
    if (!e->use_graphs)
    {
      e->drop_batch_graph();
      e->b_key_seen = false;
    }
  });
}

int dic_read_plane(dic_engine* e, int32_t plane, void* dst, int64_t bytes)
{
  return guarded(e, [&] {
    if (!dst) throw DicError{DIC_ERR_ARGUMENT, "read_plane: null destination"};
    const void* src = nullptr;
    size_t size = 0;
    const size_t px = (size_t)e->w * e->h;
    switch (plane)
    {
      case DIC_PLANE_REF: e->ensure_ref(); src = e->ref_f32.ptr; size = px * sizeof(float); break;
      case DIC_PLANE_REF_PACK: e->ensure_ref(); src = e->ref_pack.ptr; size = px * sizeof(float4); break;
      case DIC_PLANE_TAR: e->ensure_tar(); src = e->tar_f32.ptr; size = px * sizeof(float); break;
      case DIC_PLANE_TAR_COEF: e->ensure_tar(true); src = e->coef.ptr; size = px * 4 * sizeof(float4); break;
      default: throw DicError{DIC_ERR_ARGUMENT, "read_plane: unknown plane"};
    }
    if ((size_t)bytes != size) throw DicError{DIC_ERR_ARGUMENT, "read_plane: size mismatch"};
    DIC_CUDA(cudaMemcpyAsync(dst, src, size, cudaMemcpyDeviceToHost, e->stream));
    DIC_CUDA(cudaStreamSynchronize(e->stream));
  });
}

int dic_get_stats(const dic_engine* ce, dic_stats* out)
{
  dic_engine* e = const_cast<dic_engine*>(ce);
  if (!out) return DIC_ERR_ARGUMENT;
  return guarded(e, [&] {
    e->harvest();
    out->ms_prepare_ref = e->ms[kPhRef];
    out->ms_poi_prepare = e->ms[kPhPoi];
    out->ms_prepare_tar = e->ms[kPhTar];
    out->ms_fftcc = e->ms[kPhFftcc];
    out->ms_icgn = e->ms[kPhIcgn];
    out->ms_frame = e->ms[kPhFrame];
    out->ms_proposal = e->ms[kPhProposal];
    out->kernel_launches = e->launches;
    out->icgn_pois = e->icgn_pois;
    out->icgn_iterations = (int64_t)e->iter_sum;
  }, false);
}

int dic_set_timing(dic_engine* e, int32_t enabled)
{
  return guarded(e, [&] {
    e->harvest();
    e->timing = enabled != 0;
  }, false);
}

}  // extern "C"

// ---------------------------------------------------------------- read-bandwidth probe
// The denominator of the IC-GN gather roofline.  The gathers read 32-byte halves of
// coefficient texels with 256-bit non-coherent loads and are served by L2 (the table's
// working set of a few thousand POIs in flight fits there; DRAM carries only the
// compulsory bytes), so their bound is the L2-to-SM read bandwidth, measured here with
// the same load instruction: every thread streams 32-byte chunks of a buffer that L2 holds,
// four loads in flight, `repeats` passes per launch.
namespace
{
__global__ void __launch_bounds__(256) k_read_probe(const float4* __restrict__ buf, int64_t chunks, int repeats,
                                                    float* __restrict__ sink)
{
  const int64_t T = (int64_t)gridDim.x * blockDim.x;
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  float acc = 0.f;
  for (int rep = 0; rep < repeats; ++rep)
  {
    int64_t j = t;
    for (; j + 3 * T < chunks; j += 4 * T)
    {
      float4 a0, b0, a1, b1, a2, b2, a3, b3;
      ldg_256(buf + 2 * j, a0, b0);
      ldg_256(buf + 2 * (j + T), a1, b1);
      ldg_256(buf + 2 * (j + 2 * T), a2, b2);
      ldg_256(buf + 2 * (j + 3 * T), a3, b3);
      acc += (a0.x + b0.w) + (a1.x + b1.w) + (a2.x + b2.w) + (a3.x + b3.w);
    }
    for (; j < chunks; j += T)
    {
      float4 a, b;
      ldg_256(buf + 2 * j, a, b);
      acc += a.x + b.w;
    }
  }
  if (acc == 1.2345678e-30f) *sink = acc;   // keeps the loads; never true for finite data of sane size
}

// FP32 FMA issue rate (the FFTCC kernels' bound): eight independent FMA chains per thread,
// 8 CTAs of 256 threads per SM, `iterations` rounds of eight FMAs (16 FLOP each round-lane).
__global__ void __launch_bounds__(256) k_fma_probe(int iterations, float seed, float* __restrict__ sink)
{
  float a[8];
#pragma unroll
  for (int k = 0; k < 8; ++k) a[k] = seed + (float)(threadIdx.x + k);
  const float m = 0.999999f, c = 1e-7f;
  for (int it = 0; it < iterations; ++it)
  {
#pragma unroll
    for (int k = 0; k < 8; ++k) a[k] = fmaf(a[k], m, c);
  }
  float acc = 0.f;
#pragma unroll
  for (int k = 0; k < 8; ++k) acc += a[k];
  if (acc == 1.2345678e-30f) *sink = acc;
}

// Shared-memory load bandwidth (the pixel-sampled IC-GN's sample path): every warp reads
// 32 consecutive floats per load (one wavefront, no bank conflicts) from a 16 KB block,
// 16 loads per pass, `repeats` passes; 8 CTAs of 256 threads per SM.
__global__ void __launch_bounds__(256) k_smem_probe(int repeats, float* __restrict__ sink)
{
  __shared__ float buf[4096 + 32];
  for (int i = threadIdx.x; i < 4096 + 32; i += 256) buf[i] = (float)i;
  __syncthreads();
  float acc[8] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
  for (int rep = 0; rep < repeats; ++rep)
  {
    // the pass's offset (0 or 32 floats) keeps the loads from being hoisted out of the loop
    const volatile float* a = buf + threadIdx.x + ((rep & 1) << 5);
#pragma unroll
    for (int k = 0; k < 16; ++k) acc[k & 7] += a[256 * k];
  }
  float t = 0.f;
#pragma unroll
  for (int k = 0; k < 8; ++k) t += acc[k];
  if (t == 1.2345678e-30f) *sink = t;
}
}  // namespace

extern "C" int dic_smem_probe(int32_t device, int32_t repeats, float* device_sink, void* stream, int64_t* bytes_out)
{
  if (!device_sink || repeats < 1 || !bytes_out) return DIC_ERR_ARGUMENT;
  int sms = 0;
  if (cudaSetDevice(device) != cudaSuccess ||
      cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device) != cudaSuccess)
    return DIC_ERR_CUDA;
  const unsigned blocks = (unsigned)(sms * 8);
  k_smem_probe<<<blocks, 256, 0, static_cast<cudaStream_t>(stream)>>>(repeats, device_sink);
  *bytes_out = (int64_t)blocks * 256 * 16 * 4 * repeats;
  return cudaGetLastError() == cudaSuccess ? DIC_OK : DIC_ERR_CUDA;
}

extern "C" int dic_fma_probe(int32_t device, int32_t iterations, float* device_sink, void* stream,
                             int64_t* flop_out)
{
  if (!device_sink || iterations < 1 || !flop_out) return DIC_ERR_ARGUMENT;
  int sms = 0;
  if (cudaSetDevice(device) != cudaSuccess ||
      cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device) != cudaSuccess)
    return DIC_ERR_CUDA;
  const unsigned blocks = (unsigned)(sms * 8);
  k_fma_probe<<<blocks, 256, 0, static_cast<cudaStream_t>(stream)>>>(iterations, 1.f, device_sink);
  *flop_out = (int64_t)blocks * 256 * iterations * 8 * 2;
  return cudaGetLastError() == cudaSuccess ? DIC_OK : DIC_ERR_CUDA;
}

extern "C" int dic_read_probe(int32_t device, const void* device_buf, int64_t bytes, int32_t repeats,
                              float* device_sink, void* stream)
{
  if (!device_buf || !device_sink || bytes < 32 || repeats < 1 || (reinterpret_cast<uintptr_t>(device_buf) & 31))
    return DIC_ERR_ARGUMENT;
  int sms = 0;
  if (cudaSetDevice(device) != cudaSuccess ||
      cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device) != cudaSuccess)
    return DIC_ERR_CUDA;
  // 8 resident CTAs of 256 threads per SM: 64 warps, the SM's limit
  k_read_probe<<<(unsigned)(sms * 8), 256, 0, static_cast<cudaStream_t>(stream)>>>(
      static_cast<const float4*>(device_buf), bytes / 32, repeats, device_sink);
  return cudaGetLastError() == cudaSuccess ? DIC_OK : DIC_ERR_CUDA;
}

// ---------------------------------------------------------------- proposal network ABI
namespace
{
template <typename F>
int cnn_guarded(dic_cnn* c, F&& f)
{
  if (!c) return DIC_ERR_ARGUMENT;
  try
  {
    int dev = 0;
    cudaGetDevice(&dev);
    if (dev != c->device) DIC_CUDA(cudaSetDevice(c->device));
    f();
    c->last_error.clear();
    return DIC_OK;
  }
  catch (const DicError& err)
  {
    c->last_error = err.msg;
    return err.code;
  }
  catch (const std::exception& ex)
  {
    c->last_error = ex.what();
    return DIC_ERR_MEMORY;
  }
}
}  // namespace

extern "C" {

int64_t dic_cnn_param_count(void) { return cnn::ParamLayout::count; }

int dic_cnn_create(int32_t device, dic_cnn** out)
{
  if (!out) return DIC_ERR_ARGUMENT;
  *out = nullptr;
  dic_cnn* c = new (std::nothrow) dic_cnn();
  if (!c) return DIC_ERR_MEMORY;
  c->device = device;
  try
  {
    DIC_CUDA(cudaSetDevice(device));
    DIC_CUDA(cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking));
    const size_t np = cnn::ParamLayout::count;
    c->params.ensure(np);
    c->grads.ensure(np);
    c->adam_m.ensure(np);
    c->adam_v.ensure(np);
    c->wb.ensure(cnn::WeightLayout::count);
    c->part.ensure((size_t)128 * cnn::kHidden * 128);
    DIC_CUDA(cudaMemsetAsync(c->params.ptr, 0, sizeof(float) * np, c->stream));
    DIC_CUDA(cudaMemsetAsync(c->grads.ptr, 0, sizeof(float) * np, c->stream));
    DIC_CUDA(cudaMemsetAsync(c->adam_m.ptr, 0, sizeof(float) * np, c->stream));
    DIC_CUDA(cudaMemsetAsync(c->adam_v.ptr, 0, sizeof(float) * np, c->stream));
    c->pack();
    DIC_CUDA(cudaStreamSynchronize(c->stream));
  }
  catch (const DicError& err)
  {
    std::fprintf(stderr, "dic_cnn_create: %s\n", err.msg.c_str());
    if (c->stream) cudaStreamDestroy(c->stream);
    delete c;
    return err.code;
  }
  *out = c;
  return DIC_OK;
}

void dic_cnn_destroy(dic_cnn* c)
{
  if (!c) return;
  cudaSetDevice(c->device);
  if (c->stream) cudaStreamSynchronize(c->stream);
  for (auto* b : {&c->params, &c->grads, &c->adam_m, &c->adam_v, &c->out, &c->part, &c->row_loss}) b->release();
  for (auto* b : {&c->wb, &c->x0, &c->a1, &c->a2, &c->a3, &c->a4, &c->a5, &c->d1, &c->d2, &c->d3, &c->d4, &c->d5,
                  &c->dout})
    b->release();
  c->wait_err.release();
  if (c->stream) cudaStreamDestroy(c->stream);
  delete c;
}

const char* dic_cnn_last_error(const dic_cnn* c) { return c ? c->last_error.c_str() : "null network"; }

int dic_cnn_set_params(dic_cnn* c, const float* host, int64_t n)
{
  return cnn_guarded(c, [&] {
    if (!host || n != cnn::ParamLayout::count) throw DicError{DIC_ERR_ARGUMENT, "set_params: wrong parameter count"};
    DIC_CUDA(cudaMemcpyAsync(c->params.ptr, host, sizeof(float) * n, cudaMemcpyHostToDevice, c->stream));
    DIC_CUDA(cudaMemsetAsync(c->adam_m.ptr, 0, sizeof(float) * n, c->stream));
    DIC_CUDA(cudaMemsetAsync(c->adam_v.ptr, 0, sizeof(float) * n, c->stream));
    c->adam_t = 0;
    c->pack();
    DIC_CUDA(cudaStreamSynchronize(c->stream));
  });
}

int dic_cnn_get_params(dic_cnn* c, float* host, int64_t n)
{
  return cnn_guarded(c, [&] {
    if (!host || n != cnn::ParamLayout::count) throw DicError{DIC_ERR_ARGUMENT, "get_params: wrong parameter count"};
    DIC_CUDA(cudaMemcpyAsync(host, c->params.ptr, sizeof(float) * n, cudaMemcpyDeviceToHost, c->stream));
    DIC_CUDA(cudaStreamSynchronize(c->stream));
  });
}

int dic_cnn_input(dic_cnn* c, const float* d_ref, const float* d_tar, int32_t w, int32_t h, const dic_poi* d_pois,
                  int64_t n, void* d_x0)
{
  return cnn_guarded(c, [&] {
    if (!d_ref || !d_tar || !d_x0 || (n > 0 && !d_pois) || w < 1 || h < 1)
      throw DicError{DIC_ERR_ARGUMENT, "cnn_input: bad arguments"};
    if (n == 0) return;
    cnn::k_extract_input<<<(unsigned)((n + 3) / 4), 128, 0, c->stream>>>(d_ref, d_tar, w, h, d_pois, n,
                                                                        static_cast<__nv_bfloat16*>(d_x0));
    c->check("k_extract_input");
    DIC_CUDA(cudaStreamSynchronize(c->stream));
  });
}

int dic_cnn_seed(dic_cnn* c, const float* d_ref, const float* d_tar, int32_t w, int32_t h, dic_poi* d_pois, int64_t n)
{
  return cnn_guarded(c, [&] {
    if (!d_ref || !d_tar || (n > 0 && !d_pois) || w < 1 || h < 1) throw DicError{DIC_ERR_ARGUMENT, "cnn_seed: bad arguments"};
    if (n == 0) return;
    int sms = 0;
    DIC_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, c->device));
    DIC_CUDA(cudaFuncSetAttribute(cnn::k_proposal_fused, cudaFuncAttributeMaxDynamicSharedMemorySize, cnn::kSmTotal));
    const int64_t tiles = (n + cnn::kT - 1) / cnn::kT;
    c->wait_err.ensure(1);
    DIC_CUDA(cudaMemsetAsync(c->wait_err.ptr, 0, sizeof(int), c->stream));
    cnn::k_proposal_fused<<<(unsigned)std::min<int64_t>((tiles + cnn::kGroups - 1) / cnn::kGroups, sms),
                            cnn::kFusedThreads, cnn::kSmTotal, c->stream>>>(
        d_ref, d_tar, w, h, d_pois, n, c->wb.ptr, c->params.ptr, c->wait_err.ptr);
    c->check("k_proposal_fused");
    int flag = 0;
    DIC_CUDA(cudaMemcpyAsync(&flag, c->wait_err.ptr, sizeof(int), cudaMemcpyDeviceToHost, c->stream));
    DIC_CUDA(cudaStreamSynchronize(c->stream));
    if (flag) throw DicError{DIC_ERR_CUDA, "k_proposal_fused: a tensor-core product did not complete in time"};
  });
}

int dic_cnn_forward(dic_cnn* c, const void* d_x0, int64_t n, float* d_out)
{
  return cnn_guarded(c, [&] {
    if (!d_x0 || !d_out || n < 0) throw DicError{DIC_ERR_ARGUMENT, "cnn_forward: bad arguments"};
    if (n == 0) return;
    c->ensure_batch(n);
    c->forward(static_cast<const __nv_bfloat16*>(d_x0), n);
    DIC_CUDA(cudaMemcpyAsync(d_out, c->out.ptr, sizeof(float) * n * cnn::kOutPad, cudaMemcpyDeviceToDevice, c->stream));
    DIC_CUDA(cudaStreamSynchronize(c->stream));
  });
}

int dic_cnn_gradient(dic_cnn* c, const void* d_x0, const float* d_target, int64_t n, float* d_grad, float* loss)
{
  return cnn_guarded(c, [&] {
    if (!d_x0 || !d_target || !d_grad || n <= 0) throw DicError{DIC_ERR_ARGUMENT, "cnn_gradient: bad arguments"};
    c->ensure_batch(n);
    const __nv_bfloat16* in = static_cast<const __nv_bfloat16*>(d_x0);
    c->forward(in, n);
    c->backward(in, d_target, n);
    DIC_CUDA(cudaMemcpyAsync(d_grad, c->grads.ptr, sizeof(float) * cnn::ParamLayout::count,
                             cudaMemcpyDeviceToDevice, c->stream));
    const float l = c->loss(n);
    if (loss) *loss = l;
  });
}

int dic_cnn_train_step(dic_cnn* c, const void* d_x0, const float* d_target, int64_t n, float lr, float* loss)
{
  return cnn_guarded(c, [&] {
    if (!d_x0 || !d_target || n <= 0 || !(lr > 0.f)) throw DicError{DIC_ERR_ARGUMENT, "cnn_train_step: bad arguments"};
    c->ensure_batch(n);
    const __nv_bfloat16* in = static_cast<const __nv_bfloat16*>(d_x0);
    c->forward(in, n);
    c->backward(in, d_target, n);
    ++c->adam_t;
    const float b1 = 0.9f, b2 = 0.999f;
    const float c1 = 1.f - std::pow(b1, (float)c->adam_t), c2 = 1.f - std::pow(b2, (float)c->adam_t);
    const int np = cnn::ParamLayout::count;
    cnn::k_adam<<<(np + 255) / 256, 256, 0, c->stream>>>(c->params.ptr, c->grads.ptr, c->adam_m.ptr, c->adam_v.ptr,
                                                         np, lr, b1, b2, 1e-8f, c1, c2);
    c->check("k_adam");
    c->pack();
    if (loss) *loss = c->loss(n);
    else DIC_CUDA(cudaStreamSynchronize(c->stream));
  });
}

}  // extern "C"

// --------------------------------------------------------------------------------------
// Allocation-free pair solve.
//
// Some callers cannot call cudaMalloc: a host application that reserves the device memory
// up front and hands its plug-ins only buffers it owns, or an acquisition loop in which
// the implicit device synchronisation of an allocation would stall the camera's stream.
// dic_process_pair_noalloc serves them.  The caller passes the two images and the POI queue
// in device memory; everything else the pair needs (float planes, Gradient2D4 planes,
// B-spline table, per-POI reference records) is carved from the fixed array below, which
// every GPU that loads this library holds until the process exits.
// --------------------------------------------------------------------------------------
namespace
{
constexpr size_t kNoAllocScratchBytes = size_t(32) << 20;   // 32 MiB
static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocScratchBytes];

std::mutex g_noalloc_mutex;
std::vector<void*> g_noalloc_base;   // per device: device address of g_noalloc_scratch

size_t align256(size_t b) { return (b + 255) & ~size_t(255); }

void noalloc_error(char* text, int64_t cap, const std::string& msg)
{
  if (text && cap > 0)
  {
    const size_t n = std::min<size_t>(msg.size(), (size_t)cap - 1);
    std::memcpy(text, msg.data(), n);
    text[n] = '\0';
  }
}

template <typename T>
void noalloc_prepare(const void* ref, const void* tar, int w, int h, float scale, float* ref_f32,
                     float4* ref_pack, float* tar_f32, float4* coef, cudaStream_t s)
{
  dim3 grid((w + kPrepTile - 1) / kPrepTile, (h + kPrepTile - 1) / kPrepTile);
  k_prepare_ref<T><<<grid, 256, 0, s>>>(static_cast<const T*>(ref), w, h, scale, ref_f32, ref_pack);
  k_prepare_tar<T><<<grid, 256, 0, s>>>(static_cast<const T*>(tar), w, h, scale, tar_f32, coef);
}
}  // namespace

extern "C" int dic_process_pair_noalloc(const dic_config* cfg, const void* d_ref, const void* d_tar,
                                        int32_t w, int32_t h, int32_t dtype, dic_poi* d_pois, int64_t n,
                                        void* stream, char* error_text, int64_t error_capacity)
{
  if (!cfg || !d_ref || !d_tar || (n > 0 && !d_pois) || n < 0)
  {
    noalloc_error(error_text, error_capacity, "dic_process_pair_noalloc: null pointer or negative count");
    return DIC_ERR_ARGUMENT;
  }
  const int r = cfg->subset_radius_x;
  if (r < 1 || cfg->subset_radius_y != r || 2 * r > kMaxTwiddleN || cfg->max_iteration < 1 || w < 5 || h < 5 ||
      dtype_size(dtype) == 0)
  {
    noalloc_error(error_text, error_capacity,
                  "dic_process_pair_noalloc: needs a square subset radius 1..32, max_iteration >= 1, "
                  "an image of at least 5x5 and dtype u8, u16 or f32");
    return DIC_ERR_ARGUMENT;
  }
  const size_t px = (size_t)w * h;
  // Bound each term before the sum, so that no product or sum of huge sizes can wrap and
  // pass the capacity check (88 bytes of planes per pixel, one PoiRef per POI).
  if (px > kNoAllocScratchBytes / 88 || (uint64_t)n > kNoAllocScratchBytes / sizeof(PoiRef))
  {
    noalloc_error(error_text, error_capacity,
                  "dic_process_pair_noalloc: " + std::to_string(w) + "x" + std::to_string(h) + " with " +
                      std::to_string(n) + " POIs exceeds the fixed scratch of " +
                      std::to_string(kNoAllocScratchBytes) +
                      " bytes (88 bytes per pixel + 224 bytes per POI, each plane rounded up to 256 bytes)");
    return DIC_ERR_ARGUMENT;
  }
  const size_t off_ref = 0, off_pack = off_ref + align256(px * sizeof(float));
  const size_t off_tar = off_pack + align256(px * sizeof(float4));
  const size_t off_coef = off_tar + align256(px * sizeof(float));
  const size_t off_poi = off_coef + align256(px * 4 * sizeof(float4));
  const size_t need = off_poi + align256((size_t)n * sizeof(PoiRef));
  if (need > kNoAllocScratchBytes)
  {
    noalloc_error(error_text, error_capacity,
                  "dic_process_pair_noalloc: " + std::to_string(w) + "x" + std::to_string(h) + " with " +
                      std::to_string(n) + " POIs needs " + std::to_string(need) +
                      " bytes of scratch; the fixed scratch holds " + std::to_string(kNoAllocScratchBytes) +
                      " (88 bytes per pixel + 224 bytes per POI, each plane rounded up to 256 bytes)");
    return DIC_ERR_ARGUMENT;
  }
  try
  {
    int dev = 0;
    DIC_CUDA(cudaGetDevice(&dev));
    unsigned char* base = nullptr;
    {
      std::lock_guard<std::mutex> lock(g_noalloc_mutex);
      if ((int)g_noalloc_base.size() <= dev) g_noalloc_base.resize(dev + 1, nullptr);
      if (!g_noalloc_base[dev])
      {
        // One-time set-up on this device (the current one): the array's device address,
        // the constant tables, and the large-FFTCC shared-memory opt-in.
        void* addr = nullptr;
        DIC_CUDA(cudaGetSymbolAddress(&addr, g_noalloc_scratch));
        init_constants(dev);
        DIC_CUDA(cudaFuncSetAttribute(k_fftcc_large, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                      (int)(2 * kMaxTwiddleN * (kMaxTwiddleN + 1) * sizeof(float2))));
        g_noalloc_base[dev] = addr;
      }
      base = static_cast<unsigned char*>(g_noalloc_base[dev]);
    }
    if (n == 0) return DIC_OK;
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    float* ref_f32 = reinterpret_cast<float*>(base + off_ref);
    float4* ref_pack = reinterpret_cast<float4*>(base + off_pack);
    float* tar_f32 = reinterpret_cast<float*>(base + off_tar);
    float4* coef = reinterpret_cast<float4*>(base + off_coef);
    PoiRef* poi_ref = reinterpret_cast<PoiRef*>(base + off_poi);
    const float scale = cfg->input_scale == 0.f ? 1.f : cfg->input_scale;
    switch (dtype)
    {
      case DIC_U8: noalloc_prepare<uint8_t>(d_ref, d_tar, w, h, scale, ref_f32, ref_pack, tar_f32, coef, s); break;
      case DIC_U16: noalloc_prepare<uint16_t>(d_ref, d_tar, w, h, scale, ref_f32, ref_pack, tar_f32, coef, s); break;
      default: noalloc_prepare<float>(d_ref, d_tar, w, h, scale, ref_f32, ref_pack, tar_f32, coef, s); break;
    }
    constexpr int wpb = 4;
    const unsigned blocks = (unsigned)((n + wpb - 1) / wpb);
    k_poi_prepare<<<blocks, wpb * 32, 0, s>>>(ref_pack, w, h, d_pois, n, r, r, poi_ref);
    FftccParams fp{ref_f32, tar_f32, d_pois, n, w, h};
    switch (2 * r)
    {
#define DIC_NOALLOC_FFTCC(M) \
  case M: k_fftcc<M><<<(unsigned)((n + 3) / 4), 128, 0, s>>>(fp); break;
      DIC_NOALLOC_FFTCC(8) DIC_NOALLOC_FFTCC(10) DIC_NOALLOC_FFTCC(12) DIC_NOALLOC_FFTCC(14) DIC_NOALLOC_FFTCC(16)
      DIC_NOALLOC_FFTCC(18) DIC_NOALLOC_FFTCC(20) DIC_NOALLOC_FFTCC(22) DIC_NOALLOC_FFTCC(24)
      DIC_NOALLOC_FFTCC(26) DIC_NOALLOC_FFTCC(28) DIC_NOALLOC_FFTCC(30) DIC_NOALLOC_FFTCC(32)
#undef DIC_NOALLOC_FFTCC
      default:
        k_fftcc_large<<<(unsigned)n, 256, (size_t)2 * (2 * r) * (2 * r + 1) * sizeof(float2), s>>>(fp, 2 * r);
    }
    IcgnParams ip;
    ip.coef = coef;
    ip.ref_pack = ref_pack;
    ip.poi_ref = poi_ref;
    ip.slot = nullptr;
    ip.pois = d_pois;
    ip.n = n;
    ip.w = w;
    ip.h = h;
    ip.rx = r;
    ip.ry = r;
    ip.conv = cfg->conv_criterion;
    ip.max_iter = (float)cfg->max_iteration;
    ip.iter_sum = nullptr;
    if (2 * r + 1 <= 32)
      k_icgn<true><<<blocks, wpb * 32, 0, s>>>(ip);
    else if (2 * r + 1 <= kPairMaxWidth)
      k_icgn_pair<1, wpb><<<blocks, wpb * 32, 0, s>>>(ip);
    else
      k_icgn<false><<<blocks, wpb * 32, 0, s>>>(ip);
    DIC_CUDA(cudaGetLastError());
  }
  catch (const DicError& err)
  {
    noalloc_error(error_text, error_capacity, err.msg);
    return err.code;
  }
  return DIC_OK;
}
