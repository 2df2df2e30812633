// Command line of the GB300 DIC engine: the process surface of opencorr_cli_cuda_mvp that
// the Python pipeline drives (pipeline/dic_pipeline.py:910-1016 builds the argv; it reads
// the raw records and manifest through pipeline/fasticgn_io.py:132-316).
//
//   opencorr_cli_gb300 <ref> <tar> <subset_radius> <grid_space> <output_path> [options]
//   opencorr_cli_gb300 --multi-frame --ref <ref> --tar-list <list> --output-dir <dir>
//                      <subset_radius> <grid_space> [options]
//   opencorr_cli_gb300 --version | --help
//
// Kept from the reference (opencorr_cli_cuda_mvp.cpp): the argv and its strict parsing
// (:2021-2110, :3212-3480), the tar list "<tar_path> <output_name>" split on the last
// whitespace run (:3482-3540), the POI grid of buildPoiQueue (:2439-2472), the frame
// policy of runMultiFrame / processFrame (:3834-4516, :3024-3210; here run on the device
// through dic_sequence_*), the 36-byte opencorr-gpu-raw-v1 records (:2498-2536), the CSV
// rows (:1091-1160), the raw manifest with its engine block and per-frame QA
// (:2544-2731, :654-723), the diagnostics CSV and its manifest (:2734-2800), one JSON status
// line (schema fasticgn.run-status/1) on stdout at the end of every computing run, and the
// output ledger (ledger.h): multi-frame runs publish through .opencorr-state/, a rerun of
// the same command verifies or resumes (replay from frame 1), --repair quarantines damaged
// files, --durability picks rename or fsync, and --verify-only <dir> audits a directory
// without computing (:3785-4060, :4613-4760).
//
// Not provided: --dual-gpu (one GPU) and --fftcc cpu.  Asking for them is an error with a
// message saying so.  --kernel legacy selects the IC-GN grid launch form (one CTA per POI
// group) instead of the persistent work queue; the results are the same bytes.
//
// Host threads and streams: a decode thread reads ahead (--preload, the default); while frame
// k is solved, frame k+1 is staged (copied to pinned memory, uploaded on the engine's upload
// stream, dic_stage_frame) and enqueued behind it, then frame k's results are read one frame
// back (dic_sequence_fetch) while frame k+1 runs; a writer thread formats and publishes frame
// k's payload.  Payload bytes do not depend on any of this.
#include "dic.h"
#include "image_io.h"
#include "json.h"
#include "ledger.h"

#include <algorithm>
#include <atomic>
#include <charconv>
#include <chrono>
#include <cmath>
#include <condition_variable>
#include <cerrno>
#include <cstdio>
#include <cstring>
#include <deque>
#include <exception>
#include <filesystem>
#include <fstream>
#include <functional>
#include <iostream>
#include <limits>
#include <cstdlib>
#include <map>
#include <mutex>
#include <optional>
#include <set>
#include <sstream>
#include <system_error>
#include <stdexcept>
#include <string>
#include <thread>
#include <vector>

#include <fcntl.h>
#include <unistd.h>

#ifndef DIC_CLI_GIT_HASH
#define DIC_CLI_GIT_HASH "unknown"
#endif
#ifndef DIC_CLI_BUILD_DATE
#define DIC_CLI_BUILD_DATE "unknown"
#endif
#ifndef DIC_CLI_GIT_DIRTY
#define DIC_CLI_GIT_DIRTY ""
#endif

namespace fs = std::filesystem;
using namespace dic_cli;

namespace
{

const char* kTool = "opencorr_cli_gb300";
const char* kVersion = "0.2.0";
constexpr float kSkipFftccZnccThreshold = 0.8f;   // :479
constexpr float kSkipFftccBadRatioMargin = 0.03f; // :480
constexpr size_t kRecordBytes = 36;

// ------------------------------------------------------------------ run report
struct Report
{
  std::string mode;   // "" = rejected before a mode was chosen
  long long frames_total = 0, frames_processed = 0;
  std::string output_dir, output_path, output_format = "csv";
  std::string error;
  std::vector<std::string> warnings;
  long long skip_fftcc_frames = 0, fallback_frames = 0, poi_fallback_frames = 0, poi_fallback_pois = 0,
            poi_fallback_recovered = 0;
  long long frames_skipped = 0, resumed_files = 0;
  long long temporal_seed_frames = 0, temporal_seed_pois = 0;
  bool multi = false;
};
Report g_report;

std::string json_escape(const std::string& s)
{
  std::string o;
  for (unsigned char c : s)
  {
    switch (c)
    {
      case '"': o += "\\\""; break;
      case '\\': o += "\\\\"; break;
      case '\n': o += "\\n"; break;
      case '\r': o += "\\r"; break;
      case '\t': o += "\\t"; break;
      default:
        if (c < 0x20)
        {
          char b[8];
          std::snprintf(b, sizeof b, "\\u%04x", c);
          o += b;
        }
        else
          o += (char)c;
    }
  }
  return o;
}
std::string jstr(const std::string& s) { return "\"" + json_escape(s) + "\""; }

std::string json_float(double v)
{
  if (!std::isfinite(v)) return "null";
  char b[64];
  std::snprintf(b, sizeof b, "%.9g", v);
  return b;
}

void error_line(const std::string& msg)
{
  std::cerr << "Error: " << msg << std::endl;
  if (g_report.error.empty()) g_report.error = msg;
}
void warning_line(const std::string& msg)
{
  std::cerr << "Warning: " << msg << std::endl;
  g_report.warnings.push_back(msg);
}

const char* git_dirty_json()
{
  const std::string d = DIC_CLI_GIT_DIRTY;
  return d == "1" ? "true" : d == "0" ? "false" : "null";
}

void print_status(int exit_code, double elapsed)
{
  std::ostringstream o;
  o << "{\"schema\":\"fasticgn.run-status/1\",\"status\":" << (exit_code == 0 ? "\"ok\"" : "\"error\"")
    << ",\"exit_code\":" << exit_code << ",\"error\":" << (g_report.error.empty() ? "null" : jstr(g_report.error))
    << ",\"mode\":" << (g_report.mode.empty() ? "null" : jstr(g_report.mode))
    << ",\"frames_total\":" << g_report.frames_total << ",\"frames_processed\":" << g_report.frames_processed
    << ",\"frames_skipped\":" << g_report.frames_skipped;
  if (g_report.multi) o << ",\"output_dir\":" << jstr(g_report.output_dir);
  else o << ",\"output_path\":" << jstr(g_report.output_path);
  o << ",\"output_format\":" << jstr(g_report.output_format) << ",\"elapsed_sec\":" << std::round(elapsed * 1000.0) / 1000.0
    << ",\"tool\":" << jstr(kTool) << ",\"version\":" << jstr(kVersion) << ",\"git_hash\":" << jstr(DIC_CLI_GIT_HASH)
    << ",\"git_dirty\":" << git_dirty_json() << ",\"build_date\":" << jstr(DIC_CLI_BUILD_DATE)
    << ",\"backend\":\"cuda\"";
  if (g_report.multi && exit_code == 0)
    o << ",\"totals\":{\"skip_fftcc_frames\":" << g_report.skip_fftcc_frames
      << ",\"fallback_frames\":" << g_report.fallback_frames
      << ",\"poi_fallback_frames\":" << g_report.poi_fallback_frames
      << ",\"poi_fallback_pois\":" << g_report.poi_fallback_pois
      << ",\"poi_fallback_recovered\":" << g_report.poi_fallback_recovered
      << ",\"temporal_seed_frames\":" << g_report.temporal_seed_frames
      << ",\"temporal_seed_pois\":" << g_report.temporal_seed_pois
      << ",\"resumed_from_existing_files\":" << g_report.resumed_files
      << "}";
  o << ",\"warning_count\":" << g_report.warnings.size() << ",\"warnings\":[";
  for (size_t i = 0; i < g_report.warnings.size() && i < 20; ++i) o << (i ? "," : "") << jstr(g_report.warnings[i]);
  o << "]}";
  std::cout << o.str() << std::endl;
}

// ------------------------------------------------------------------ options
struct Options
{
  int subset_size = -1;
  int device = 0;
  int max_iter = 10;
  float conv = 0.001f;
  std::vector<int> lines;
  int threads = 1;
  bool raw = false;
  bool roi = false;
  int roi_x1 = 0, roi_y1 = 0, roi_x2 = 0, roi_y2 = 0;
  int out_step = 1;
  bool diagnostics = false;
  std::string diagnostics_dir;
  InputOptions input;
  bool fsync = false;
  bool repair = false;
  bool quiet = false;
  bool skip_fftcc = true, poi_fallback = true, preload = true;
  bool temporal = false;   // --temporal-extrapolation
  int decode_threads = 1;
  bool legacy_kernel = false;   // --kernel legacy: the grid launch form (one CTA per POI group)
  bool keep(int x, int y) const
  {
    if (roi && (x < roi_x1 || x > roi_x2 || y < roi_y1 || y > roi_y2)) return false;
    return out_step <= 1 || (x % out_step == 0 && y % out_step == 0);
  }
};

bool parse_int(const std::string& t, const std::string& name, int lo, int hi, int& out, std::string& err)
{
  if (t.empty())
  {
    err = name + " must not be empty";
    return false;
  }
  int v = 0;
  auto r = std::from_chars(t.data(), t.data() + t.size(), v);
  if (r.ec != std::errc() || r.ptr != t.data() + t.size())
  {
    err = name + " must be an integer, got '" + t + "'";
    return false;
  }
  if (v < lo || v > hi)
  {
    err = name + " out of range: " + t;
    return false;
  }
  out = v;
  return true;
}

bool parse_positive_float(const std::string& t, const std::string& name, float& out, std::string& err)
{
  char* end = nullptr;
  errno = 0;
  const float v = t.empty() ? 0.f : std::strtof(t.c_str(), &end);
  if (t.empty() || end != t.c_str() + t.size() || !std::isfinite(v) || v <= 0.f)
  {
    err = name + " must be a finite positive number, got '" + t + "'";
    return false;
  }
  out = v;
  return true;
}

std::vector<std::string> split_commas(const std::string& t)
{
  std::vector<std::string> out;
  size_t a = 0;
  for (;;)
  {
    const size_t b = t.find(',', a);
    out.push_back(t.substr(a, b == std::string::npos ? std::string::npos : b - a));
    if (b == std::string::npos) break;
    a = b + 1;
  }
  return out;
}

// Returns true when args[i] was an option (i advanced past its value); false with err set
// on a malformed option; false with err empty for a positional.
bool parse_common(const std::vector<std::string>& a, size_t& i, Options& o, std::string& err)
{
  const std::string& arg = a[i];
  auto value = [&](const char* name) -> const std::string* {
    if (i + 1 >= a.size())
    {
      err = std::string("missing value for ") + name;
      return nullptr;
    }
    return &a[++i];
  };
  auto unsupported = [&](const std::string& what) {
    err = what + " is not available in this build (one GB300, hand-written CUDA path)";
    return false;
  };
  if (arg == "--gpu-device")
  {
    auto v = value("--gpu-device");
    return v && parse_int(*v, arg, 0, std::numeric_limits<int>::max(), o.device, err);
  }
  if (arg == "--max-iter")
  {
    auto v = value("--max-iter");
    return v && parse_int(*v, arg, 1, std::numeric_limits<int>::max(), o.max_iter, err);
  }
  if (arg == "--subset-size")
  {
    auto v = value("--subset-size");
    int size = 0;
    if (!v || !parse_int(*v, arg, 3, std::numeric_limits<int>::max(), size, err)) return false;
    if (size % 2 == 0)
    {
      err = "--subset-size must be an odd subset SIZE in pixels; radius = (size - 1) / 2";
      return false;
    }
    o.subset_size = size;
    return true;
  }
  if (arg == "--conv-threshold")
  {
    auto v = value("--conv-threshold");
    return v && parse_positive_float(*v, arg, o.conv, err);
  }
  if (arg == "--kernel")
  {
    auto v = value("--kernel");
    if (!v) return false;
    if (*v == "warp")
    {
      o.legacy_kernel = false;
      return true;
    }
    if (*v == "legacy")
    {
      o.legacy_kernel = true;
      return true;
    }
    err = "--kernel must be legacy or warp, got '" + *v + "'";
    return false;
  }
  if (arg == "--fftcc")
  {
    auto v = value("--fftcc");
    if (!v) return false;
    if (*v == "gpu") return true;
    if (*v == "cpu") return unsupported("--fftcc cpu");
    err = "--fftcc must be cpu or gpu, got '" + *v + "'";
    return false;
  }
  if (arg == "--threads")
  {
    auto v = value("--threads");
    return v && parse_int(*v, arg, 1, std::numeric_limits<int>::max(), o.threads, err);
  }
  if (arg == "--line")
  {
    auto v = value("--line");
    if (!v) return false;
    if (v->empty())
    {
      err = "--line must not be empty";
      return false;
    }
    for (const auto& part : split_commas(*v))
    {
      int y = 0;
      if (!parse_int(part, "--line", 0, std::numeric_limits<int>::max(), y, err)) return false;
      o.lines.push_back(y);
    }
    return true;
  }
  if (arg == "--durability")
  {
    auto v = value("--durability");
    if (!v) return false;
    if (*v != "rename" && *v != "fsync")
    {
      err = "--durability must be rename or fsync, got '" + *v + "'";
      return false;
    }
    o.fsync = *v == "fsync";
    return true;
  }
  if (arg == "--repair") return o.repair = true, true;
  if (arg == "--no-repair") return o.repair = false, true;
  if (arg == "--temporal-extrapolation") return o.temporal = true, true;
  if (arg == "--no-temporal-extrapolation") return o.temporal = false, true;
  if (arg == "--quiet") return o.quiet = true, true;
  if (arg == "--dual-gpu") return unsupported("--dual-gpu");
  if (arg == "--skip-fftcc") return o.skip_fftcc = true, true;
  if (arg == "--no-skip-fftcc") return o.skip_fftcc = false, true;
  if (arg == "--poi-fallback") return o.poi_fallback = true, true;
  if (arg == "--no-poi-fallback") return o.poi_fallback = false, true;
  if (arg == "--output-format")
  {
    auto v = value("--output-format");
    if (!v) return false;
    if (*v == "csv") o.raw = false;
    else if (*v == "raw" || *v == "binary") o.raw = true;
    else
    {
      err = "--output-format must be csv or raw, got '" + *v + "'";
      return false;
    }
    return true;
  }
  if (arg == "--binary-output") return o.raw = true, true;
  if (arg == "--input-depth")
  {
    auto v = value("--input-depth");
    if (!v) return false;
    if (*v == "8") o.input.depth = Depth::k8;
    else if (*v == "12") o.input.depth = Depth::k12;
    else if (*v == "16") o.input.depth = Depth::k16;
    else if (*v == "auto") o.input.depth = Depth::kAuto;
    else
    {
      err = "--input-depth must be 8, 12, 16 or auto, got '" + *v + "'";
      return false;
    }
    return true;
  }
  if (arg == "--input-align")
  {
    auto v = value("--input-align");
    if (!v) return false;
    if (*v == "right") o.input.align = Align::kRight;
    else if (*v == "left") o.input.align = Align::kLeft;
    else if (*v == "auto") o.input.align = Align::kAuto;
    else
    {
      err = "--input-align must be right, left or auto, got '" + *v + "'";
      return false;
    }
    return true;
  }
  if (arg == "--input-normalize")
  {
    auto v = value("--input-normalize");
    if (!v) return false;
    if (*v == "none") o.input.normalize = Normalize::kNone;
    else if (*v == "to-8") o.input.normalize = Normalize::kTo8;
    else if (*v == "to-16") o.input.normalize = Normalize::kTo16;
    else if (*v == "unit") o.input.normalize = Normalize::kUnit;
    else
    {
      err = "--input-normalize must be none, to-8, to-16 or unit, got '" + *v + "'";
      return false;
    }
    return true;
  }
  if (arg == "--diagnostics") return o.diagnostics = true, true;
  if (arg == "--diagnostics-dir")
  {
    auto v = value("--diagnostics-dir");
    if (!v) return false;
    if (v->empty())
    {
      err = "--diagnostics-dir must not be empty";
      return false;
    }
    o.diagnostics = true;
    o.diagnostics_dir = *v;
    return true;
  }
  if (arg == "--preload") return o.preload = true, true;
  if (arg == "--no-preload") return o.preload = false, true;
  if (arg == "--decode-threads")
  {
    auto v = value("--decode-threads");
    return v && parse_int(*v, arg, 1, std::numeric_limits<int>::max(), o.decode_threads, err);
  }
  if (arg == "--output-roi")
  {
    auto v = value("--output-roi");
    if (!v) return false;
    const auto parts = split_commas(*v);
    int vals[4];
    if (parts.size() != 4)
    {
      err = "--output-roi needs x1,y1,x2,y2";
      return false;
    }
    for (int k = 0; k < 4; ++k)
      if (!parse_int(parts[k], "--output-roi", 0, std::numeric_limits<int>::max(), vals[k], err)) return false;
    if (vals[2] < vals[0] || vals[3] < vals[1])
    {
      err = "--output-roi needs x1 <= x2 and y1 <= y2";
      return false;
    }
    o.roi = true;
    o.roi_x1 = vals[0];
    o.roi_y1 = vals[1];
    o.roi_x2 = vals[2];
    o.roi_y2 = vals[3];
    return true;
  }
  if (arg == "--output-step")
  {
    auto v = value("--output-step");
    return v && parse_int(*v, arg, 1, std::numeric_limits<int>::max(), o.out_step, err);
  }
  if (!arg.empty() && arg[0] == '-' && arg.size() > 1 && !(arg[1] >= '0' && arg[1] <= '9'))
    err = "unknown option: " + arg;
  return false;
}

bool validate(const Options& o, std::string& err)
{
  if (o.input.depth != Depth::k12 && o.input.align != Align::kAuto)
  {
    err = "--input-align is only meaningful with --input-depth 12; use --input-depth 12 for left/right 12-bit storage";
    return false;
  }
  return true;
}

void print_usage(std::ostream& out, bool full)
{
  out << "GB300 DIC engine command line (" << kTool << ")\n"
      << "Usage: " << kTool << " <ref_image> <tar_image> <subset_radius> <grid_space> <output_path>\n"
      << "       [--subset-size N] [--gpu-device N] [--max-iter M] [--conv-threshold T] [--line y1,y2] [--threads N]\n"
      << "       [--output-format csv|raw] [--diagnostics|--diagnostics-dir DIR] [--kernel warp|legacy] [--fftcc gpu]\n"
      << "       [--input-depth 8|12|16|auto] [--input-align right|left|auto] [--input-normalize none|to-8|to-16|unit]\n"
      << "       [--output-roi x1,y1,x2,y2] [--output-step N] [--durability rename|fsync] [--quiet]\n"
      << "   or: " << kTool << " --multi-frame --ref <ref_image> --tar-list <tar_list.txt> --output-dir <output_dir>\n"
      << "       <subset_radius> <grid_space> [the options above] [--skip-fftcc|--no-skip-fftcc]\n"
      << "       [--poi-fallback|--no-poi-fallback] [--temporal-extrapolation] [--preload|--no-preload]\n"
      << "       [--decode-threads N] [--repair]\n"
      << "   or: " << kTool << " --verify-only <output_dir>\n"
      << "   or: " << kTool << " --version\n"
      << "   or: " << kTool << " --help\n"
      << "<subset_radius> is the subset RADIUS in pixels; --subset-size N gives the odd full SIZE instead.\n"
      << "Images: PGM (P5/P2, 8 or 16 bit) and uncompressed grey TIFF.\n"
      << "stdout: one JSON status line (schema fasticgn.run-status/1) at the end of every computing run;\n"
      << "  --verify-only prints its own verdict (schema fasticgn.verify-only/1) instead.\n"
      << "Multi-frame output carries a .opencorr-state/ ledger: rerunning the same command verifies a complete\n"
      << "  directory without computing, or replays from frame 1 and publishes what is missing; --repair moves\n"
      << "  damaged files to .opencorr-state/quarantine/ and regenerates them; --verify-only audits a directory.\n";
  if (full)
    out << "Defaults: --max-iter 10, --conv-threshold 0.001, --gpu-device 0, --output-format csv, --input-depth 8,\n"
        << "  --input-normalize none, --skip-fftcc on, --poi-fallback on, --temporal-extrapolation off, --preload on,\n"
        << "  --durability rename.\n"
        << "Not available here: --dual-gpu, --fftcc cpu (one GPU).  --kernel legacy runs the IC-GN grid launch\n"
        << "  form instead of the persistent work queue (same results).\n"
        << "Exit status: 0 success (--verify-only: the directory is complete and verified); 1 any usage, input,\n"
        << "  compute or output error (--verify-only: the directory is not complete, or could not be read).\n";
}

void print_version()
{
  std::cout << "GB300 DIC engine (" << kTool << ")\n"
            << "name=" << kTool << "\n"
            << "git_hash=" << DIC_CLI_GIT_HASH << "\n"
            << "build_date=" << DIC_CLI_BUILD_DATE << "\n"
            << "version=" << kVersion << "\n"
            << "git_dirty=" << DIC_CLI_GIT_DIRTY << "\n"
            << "backend=cuda\n"
            << "fftw=0\n"
            << "engine=" << dic_version() << "\n";
}

// ------------------------------------------------------------------ POIs and output
std::vector<dic_poi> build_queue(int w, int h, int r, int step, const std::vector<int>& lines)
{
  // buildPoiQueue (:2439-2472): margin r + 2, y outer, x inner; --line rows in the given
  // order (repeats kept), rows outside the margin skipped
  const int margin = r + 2;
  std::vector<int> rows;
  if (!lines.empty())
  {
    for (int y : lines)
      if (y >= margin && y < h - margin) rows.push_back(y);
  }
  else
    for (int y = margin; y < h - margin; y += step) rows.push_back(y);
  std::vector<dic_poi> q;
  for (int y : rows)
    for (int x = margin; x < w - margin; x += step)
    {
      dic_poi p{};
      p.x = (float)x;
      p.y = (float)y;
      q.push_back(p);
    }
  return q;
}

// A read-only view of POI records: a std::vector or a page-locked result buffer.
struct PoiSpan
{
  const dic_poi* p = nullptr;
  size_t n = 0;
  PoiSpan(const dic_poi* ptr, size_t count) : p(ptr), n(count) {}
  PoiSpan(const std::vector<dic_poi>& v) : p(v.data()), n(v.size()) {}
  const dic_poi* begin() const { return p; }
  const dic_poi* end() const { return p + n; }
  size_t size() const { return n; }
  bool empty() const { return n == 0; }
  const dic_poi& operator[](size_t i) const { return p[i]; }
};

// Page-locked POI records (dic_host_alloc): frame results are read into these by DMA.
class PinnedPois
{
 public:
  explicit PinnedPois(size_t count) : n_(count)
  {
    void* ptr = nullptr;
    if (dic_host_alloc(sizeof(dic_poi) * std::max<size_t>(count, 1), &ptr) != DIC_OK)
      throw std::runtime_error("cannot allocate page-locked result buffers");
    p_ = static_cast<dic_poi*>(ptr);
  }
  PinnedPois(PinnedPois&& o) noexcept : p_(o.p_), n_(o.n_) { o.p_ = nullptr; }
  PinnedPois(const PinnedPois&) = delete;
  PinnedPois& operator=(const PinnedPois&) = delete;
  ~PinnedPois() { dic_host_free(p_); }
  dic_poi* data() { return p_; }
  size_t size() const { return n_; }
  operator PoiSpan() const { return PoiSpan(p_, n_); }

 private:
  dic_poi* p_ = nullptr;
  size_t n_ = 0;
};

struct Payload
{
  std::vector<char> bytes;
  size_t rows = 0;
};

// into `p`, whose buffer keeps its capacity across frames
void format_raw_into(PoiSpan q, const Options& o, Payload& p)
{
  p.rows = 0;
  p.bytes.resize(q.size() * kRecordBytes);
  char* c = p.bytes.data();
  for (const auto& poi : q)
  {
    const int32_t x = (int32_t)poi.x, y = (int32_t)poi.y;
    if (!o.keep(x, y)) continue;
    const float f[7] = {poi.u, poi.v, poi.ux, poi.uy, poi.vx, poi.vy, poi.zncc};
    std::memcpy(c, &x, 4);
    std::memcpy(c + 4, &y, 4);
    std::memcpy(c + 8, f, 28);   // little-endian on every target of this build
    c += kRecordBytes;
    ++p.rows;
  }
  p.bytes.resize((size_t)(c - p.bytes.data()));
}

Payload format_raw(PoiSpan q, const Options& o)
{
  Payload p;
  format_raw_into(q, o, p);
  return p;
}

void append_g6(std::string& s, float v)
{
  char b[48];
  auto r = std::to_chars(b, b + sizeof b, v, std::chars_format::general, 6);
  s.append(b, r.ptr);
}

Payload format_csv(PoiSpan q, const Options& o)
{
  std::string s = "x,y,u,v,zncc,uy,vy,ux,vx\n";
  s.reserve(q.size() * 80 + 32);
  Payload p;
  for (const auto& poi : q)
  {
    const int x = (int)poi.x, y = (int)poi.y;
    if (!o.keep(x, y)) continue;
    s += std::to_string(x);
    s += ',';
    s += std::to_string(y);
    for (float v : {poi.u, poi.v, poi.zncc, poi.uy, poi.vy, poi.ux, poi.vx})
    {
      s += ',';
      append_g6(s, v);
    }
    s += '\n';
    ++p.rows;
  }
  p.bytes.assign(s.begin(), s.end());
  return p;
}

std::string format_diagnostics(PoiSpan q)
{
  std::ostringstream o;
  o.precision(9);
  o << "x,y,iteration,convergence,status,zncc\n";
  for (const auto& poi : q)
  {
    const float status = !std::isfinite(poi.zncc) ? -5.f : (poi.zncc >= 0.f ? 1.f : poi.zncc);   // :725-732
    o << (int)poi.x << "," << (int)poi.y << "," << poi.iteration << "," << poi.convergence << "," << status << ","
      << poi.zncc << "\n";
  }
  return o.str();
}

// a uniquely named temporary in the destination directory, then rename (replaces);
// with fsync also the file and the directory
void publish(const fs::path& dst, const char* data, size_t n, bool do_fsync)
{
  publish_file(dst, data, n, true, do_fsync);
}

// per-frame QA of computeFrameQa (:654-723)
struct FrameQa
{
  float bad_ratio = 0.f;
  bool has_baseline = false;
  float baseline_bad_ratio = 0.f;
  bool has_threshold = false;
  float fallback_threshold = 0.f;
  bool fallback_used = false, skip_fftcc_used = false;
  float valid_ratio = 0.f, iteration_mean = 0.f;
  int iteration_max = 0;
  long long poi_fallback_count = 0, poi_fallback_recovered = 0;
  long long temporal_seed_count = 0;
};

void fill_qa_stats(PoiSpan q, FrameQa& qa)
{
  if (q.empty()) return;
  long long valid = 0, finite_it = 0, it_sum = 0;
  int it_max = 0;
  for (const auto& p : q)
  {
    if (std::isfinite(p.zncc) && p.zncc >= 0.f) ++valid;
    if (std::isfinite(p.iteration))
    {
      ++finite_it;
      it_sum += (long long)p.iteration;
      it_max = std::max(it_max, (int)(p.iteration + 0.5f));
    }
  }
  qa.valid_ratio = (float)valid / (float)q.size();
  qa.iteration_mean = finite_it == 0 ? 0.f : (float)(it_sum / (double)finite_it);
  qa.iteration_max = it_max;
}

struct FrameRecord
{
  std::string tar_path, output_name, file;
  size_t rows = 0, bytes = 0;
  double format_sec = 0, write_sec = 0;
  FrameQa qa;
};

std::string nf(bool has, float v) { return has ? json_float(v) : "null"; }
std::string nb(bool has, bool v) { return has ? (v ? "true" : "false") : "null"; }

std::string engine_block(const Options& o, int device)
{
  int driver = 0, runtime = 0;
  std::ostringstream s;
  s << "  \"engine\": {\n"
    << "    \"implementation\": \"FastICGN-GB300\",\n"
    << "    \"git_hash\": " << jstr(DIC_CLI_GIT_HASH) << ",\n"
    << "    \"build_date\": " << jstr(DIC_CLI_BUILD_DATE) << ",\n"
    << "    \"version\": " << jstr(kVersion) << ",\n"
    << "    \"git_dirty\": " << git_dirty_json() << ",\n"
    << "    \"icgn_backend\": \"cuda\",\n"
    << "    \"icgn_kernel\": " << (o.legacy_kernel ? "\"legacy\"" : "\"warp\"") << ",\n"
    << "    \"oob_policy\": \"geometric-v1\",\n"
    << "    \"fftcc_backend\": \"gpu\",\n"
    << "    \"skip_fftcc\": " << (o.skip_fftcc ? "true" : "false") << ",\n"
    << "    \"poi_fallback\": " << (o.poi_fallback ? "true" : "false") << ",\n"
    << "    \"temporal_extrapolation\": " << (o.temporal ? "true" : "false") << ",\n"
    << "    \"frame_fallback_policy\": \"per-poi-merge-v1\",\n"
    << "    \"preload\": " << (o.preload ? "true" : "false") << ",\n"
    << "    \"durability\": " << (o.fsync ? "\"fsync\"" : "\"rename\"") << ",\n"
    << "    \"threads\": " << o.threads << ",\n"
    << "    \"decode_threads\": " << o.decode_threads << ",\n"
    << "    \"dual_gpu\": false,\n"
    << "    \"gpu_device\": " << device << ",\n"
    << "    \"cuda\": ";
  char name[256] = {0};
  int major = 0, minor = 0;
  if (dic_device_info(device, name, (int32_t)sizeof name, &major, &minor, &driver, &runtime) == DIC_OK)
    s << "{\"device_name\": " << jstr(name) << ", \"compute_capability\": \"" << major << "." << minor
      << "\", \"driver_version\": " << driver << ", \"runtime_version\": " << runtime << ", \"engine\": "
      << jstr(dic_version()) << "}\n";
  else
    s << "{\"device_name\": null, \"compute_capability\": null, \"driver_version\": null, "
         "\"runtime_version\": null, \"engine\": "
      << jstr(dic_version()) << "}\n";
  s
    << "  },\n";
  return s.str();
}

std::string manifest_json(const std::string& ref_path, const std::string& tar_list, const std::string& out_dir, int r,
                          int grid, const Options& o, const Samples& ref, const std::vector<FrameRecord>& frames,
                          long long depth_mismatches)
{
  std::ostringstream s;
  s << "{\n"
    << "  \"format\": \"opencorr-gpu-raw-v1\",\n"
    << "  \"endianness\": \"little\",\n"
    << "  \"record_bytes\": 36,\n"
    << "  \"ref_path\": " << jstr(ref_path) << ",\n"
    << "  \"tar_list_path\": " << jstr(tar_list) << ",\n"
    << "  \"output_dir\": " << jstr(out_dir) << ",\n"
    << "  \"subset_radius\": " << r << ",\n"
    << "  \"grid_space\": " << grid << ",\n"
    << "  \"conv_threshold\": " << json_float(o.conv) << ",\n"
    << "  \"max_iteration\": " << o.max_iter << ",\n"
    << "  \"durability\": " << (o.fsync ? "\"fsync\"" : "\"rename\"") << ",\n"
    << engine_block(o, o.device);
  if (o.roi || o.out_step > 1)
  {
    s << "  \"output_filter\": {\n    \"roi_enabled\": " << (o.roi ? "true" : "false");
    if (o.roi) s << ",\n    \"roi\": [" << o.roi_x1 << ", " << o.roi_y1 << ", " << o.roi_x2 << ", " << o.roi_y2 << "]";
    s << ",\n    \"step\": " << o.out_step << "\n  },\n";
  }
  s << "  \"input_image\": {\n"
    << "    \"depth\": \"" << depth_name(o.input.depth) << "\",\n"
    << "    \"align\": \"" << align_name(o.input.align) << "\",\n"
    << "    \"normalize\": \"" << normalize_name(o.input.normalize) << "\",\n"
    << "    \"imread_flags\": \"" << (o.input.depth == Depth::k8 ? "IMREAD_GRAYSCALE" : "IMREAD_ANYDEPTH|IMREAD_GRAYSCALE")
    << "\",\n"
    << "    \"reference_source_depth\": \"" << (ref.source_bits == 8 ? "CV_8U" : "CV_16U") << "\",\n"
    << "    \"reference_source_range\": [" << json_float(ref.source_min) << ", " << json_float(ref.source_max) << "],\n"
    << "    \"target_source_depth_mismatches\": " << depth_mismatches << ",\n"
    << "    \"gray_conversion\": \"grey files only (PGM, grey TIFF); colour input is rejected\"\n"
    << "  },\n"
    << "  \"fields\": [\n"
    << "    {\"name\":\"x\",\"dtype\":\"int32\",\"offset\":0},\n"
    << "    {\"name\":\"y\",\"dtype\":\"int32\",\"offset\":4},\n"
    << "    {\"name\":\"u\",\"dtype\":\"float32\",\"offset\":8},\n"
    << "    {\"name\":\"v\",\"dtype\":\"float32\",\"offset\":12},\n"
    << "    {\"name\":\"ux\",\"dtype\":\"float32\",\"offset\":16},\n"
    << "    {\"name\":\"uy\",\"dtype\":\"float32\",\"offset\":20},\n"
    << "    {\"name\":\"vx\",\"dtype\":\"float32\",\"offset\":24},\n"
    << "    {\"name\":\"vy\",\"dtype\":\"float32\",\"offset\":28},\n"
    << "    {\"name\":\"zncc\",\"dtype\":\"float32\",\"offset\":32}\n"
    << "  ],\n"
    << "  \"csv_field_order\": [\"x\",\"y\",\"u\",\"v\",\"zncc\",\"uy\",\"vy\",\"ux\",\"vx\"],\n"
    << "  \"frames\": [\n";
  for (size_t i = 0; i < frames.size(); ++i)
  {
    const auto& f = frames[i];
    const auto& q = f.qa;
    s << "    {\"tar_path\":" << jstr(f.tar_path) << ",\"output_name\":" << jstr(f.output_name)
      << ",\"file\":" << jstr(f.file) << ",\"rows\":" << f.rows << ",\"bytes\":" << f.bytes
      << ",\"format_sec\":" << json_float(f.format_sec) << ",\"write_sec\":" << json_float(f.write_sec)
      << ",\"bad_ratio\":" << json_float(q.bad_ratio) << ",\"baseline_bad_ratio\":" << nf(q.has_baseline, q.baseline_bad_ratio)
      << ",\"fallback_threshold\":" << nf(q.has_threshold, q.fallback_threshold)
      << ",\"fallback_used\":" << nb(true, q.fallback_used) << ",\"skip_fftcc_used\":" << nb(true, q.skip_fftcc_used)
      << ",\"valid_ratio\":" << json_float(q.valid_ratio) << ",\"iteration_mean\":" << json_float(q.iteration_mean)
      << ",\"iteration_max\":" << q.iteration_max << ",\"poi_fallback_count\":" << q.poi_fallback_count
      << ",\"poi_fallback_recovered\":" << q.poi_fallback_recovered
      << ",\"temporal_seed_used\":" << (q.temporal_seed_count > 0 ? "true" : "false")
      << ",\"temporal_seed_count\":" << q.temporal_seed_count << "}" << (i + 1 < frames.size() ? "," : "") << "\n";
  }
  s << "  ]\n}\n";
  return s.str();
}

// diagnosticsPathForFrame (:2802-2807): <output stem>.diagnostics.csv
fs::path diagnostics_file(const fs::path& dir, const std::string& output_file)
{
  return dir / (fs::path(output_file).stem().string() + ".diagnostics.csv");
}

struct DiagRecord
{
  std::string tar_path, output_name, file;
  size_t rows = 0;
};

// writeDiagnosticsManifest (:2758-2792)
std::string diagnostics_manifest_json(const std::string& ref_path, const std::string& tar_list, const Options& o,
                                      const std::vector<DiagRecord>& frames)
{
  std::ostringstream s;
  s << "{\n"
    << "  \"format\": \"opencorr-gpu-diagnostics-csv-v1\",\n"
    << "  \"ref_path\": " << jstr(ref_path) << ",\n"
    << "  \"tar_list_path\": " << jstr(tar_list) << ",\n"
    << "  \"status_semantics\": \"1 means zncc>=0 success; negative values mirror failure/status codes carried by "
       "zncc; non-finite zncc maps to -5\",\n"
    << "  \"durability\": " << (o.fsync ? "\"fsync\"" : "\"rename\"") << ",\n"
    << engine_block(o, o.device)
    << "  \"columns\": [\"x\",\"y\",\"iteration\",\"convergence\",\"status\",\"zncc\"],\n"
    << "  \"frames\": [\n";
  for (size_t i = 0; i < frames.size(); ++i)
    s << "    {\"tar_path\":" << jstr(frames[i].tar_path) << ",\"output_name\":" << jstr(frames[i].output_name)
      << ",\"file\":" << jstr(frames[i].file) << ",\"rows\":" << frames[i].rows << "}" << (i + 1 < frames.size() ? "," : "")
      << "\n";
  s << "  ]\n}\n";
  return s.str();
}

std::string raw_name(const std::string& name)
{
  const std::string ext = ".csv";
  if (name.size() >= ext.size() && name.compare(name.size() - ext.size(), ext.size(), ext) == 0)
    return name.substr(0, name.size() - ext.size()) + ".bin";
  if (name.size() >= 4 && name.compare(name.size() - 4, 4, ".bin") == 0) return name;
  return name + ".bin";
}

// ------------------------------------------------------------------ engine
struct Engine
{
  dic_engine* e = nullptr;
  Engine(int r, const Options& o, float scale)
  {
    dic_config c{};
    c.subset_radius_x = r;
    c.subset_radius_y = r;
    c.conv_criterion = o.conv;
    c.max_iteration = o.max_iter;
    c.device = o.device;
    c.input_scale = scale;
    const int rc = dic_engine_create(&c, &e);
    if (rc != DIC_OK)
      throw std::runtime_error("cannot create the DIC engine on CUDA device " + std::to_string(o.device) +
                               " (status " + std::to_string(rc) + ")");
    if (o.legacy_kernel)
    {
      // --kernel legacy: every walk in the grid form, one CTA of 4 warps per POI group, each
      // POI solved to completion by its own CTA slot (the reference's legacy kernel is
      // block-per-POI); the default is the persistent work-queue form.  Same results.
      for (int walk = 0; walk < 3; ++walk)
      {
        dic_launch_shape sh{};
        sh.warps_per_cta = 4;
        sh.ctas_per_sm = 0;
        sh.warps_per_poi = 1;
        if (dic_set_launch_shape(e, walk, &sh) != DIC_OK)
          throw std::runtime_error(std::string("--kernel legacy: ") + dic_last_error(e));
      }
    }
  }
  ~Engine()
  {
    if (e) dic_engine_destroy(e);
  }
  void check(int rc, const char* what)
  {
    if (rc != DIC_OK) throw std::runtime_error(std::string(what) + ": " + dic_last_error(e));
  }
};

// ------------------------------------------------------------------ background workers
// Decodes the targets with `workers` threads (--decode-threads; worker w takes frames
// w, w + workers, ...), at most workers + 1 frames ahead of the consumer, and hands them
// out in list order, so results do not depend on the count.  Each worker reads files into
// its own buffer, and decodes into the sample vectors the consumer returns (recycle), so
// a steady frame loop allocates and first-touches no memory.
class Preloader
{
 public:
  Preloader(std::vector<std::string> paths, InputOptions opt, bool enabled, int workers)
      : paths_(std::move(paths)), opt_(opt), enabled_(enabled),
        workers_(std::max(1, std::min<int>(workers, (int)std::max<size_t>(paths_.size(), 1))))
  {
    if (enabled_)
      for (int w = 0; w < workers_; ++w) threads_.emplace_back([this, w] { run(w); });
  }
  ~Preloader()
  {
    {
      std::lock_guard<std::mutex> l(m_);
      stop_ = true;
    }
    cv_.notify_all();
    for (auto& t : threads_)
      if (t.joinable()) t.join();
  }
  // frame k, in order; rethrows a decode error of that frame
  Samples get(size_t k)
  {
    if (!enabled_) return configure(read_image(paths_[k], inline_buf_, take_spare()), opt_, paths_[k]);
    std::unique_lock<std::mutex> l(m_);
    cv_.wait(l, [&] { return ready_.count(k) != 0 || stop_; });
    Item it = std::move(ready_[k]);
    ready_.erase(k);
    next_ = k + 1;
    cv_.notify_all();
    l.unlock();
    if (!it.error.empty()) throw std::runtime_error(it.error);
    return std::move(it.s);
  }
  // a consumed frame's sample vectors, for a later decode
  void recycle(Samples&& s)
  {
    Image spare;
    spare.u8 = std::move(s.u8);
    spare.u16 = std::move(s.u16);
    std::lock_guard<std::mutex> l(m_);
    if (spares_.size() < (size_t)workers_ + 2) spares_.push_back(std::move(spare));
  }

 private:
  struct Item
  {
    Samples s;
    std::string error;
  };
  Image take_spare()
  {
    std::lock_guard<std::mutex> l(m_);
    if (spares_.empty()) return Image{};
    Image im = std::move(spares_.back());
    spares_.pop_back();
    return im;
  }
  void run(int w)
  {
    std::vector<uint8_t> buf;
    for (size_t k = (size_t)w; k < paths_.size(); k += (size_t)workers_)
    {
      {
        std::unique_lock<std::mutex> l(m_);
        cv_.wait(l, [&] { return k < next_ + (size_t)workers_ + 1 || stop_; });
        if (stop_) return;
      }
      Item it;
      try
      {
        it.s = configure(read_image(paths_[k], buf, take_spare()), opt_, paths_[k]);
      }
      catch (const std::exception& ex)
      {
        it.error = ex.what();
      }
      std::lock_guard<std::mutex> l(m_);
      if (stop_) return;
      ready_[k] = std::move(it);
      cv_.notify_all();
    }
  }
  std::vector<std::string> paths_;
  InputOptions opt_;
  bool enabled_;
  int workers_;
  std::vector<std::thread> threads_;
  std::mutex m_;
  std::condition_variable cv_;
  std::map<size_t, Item> ready_;
  std::vector<Image> spares_;
  std::vector<uint8_t> inline_buf_;   // the file buffer without preloading
  size_t next_ = 0;                   // the next frame the consumer takes
  bool stop_ = false;
};

// Runs jobs on `threads` threads, taken in submission order (a job gets the index of the
// thread that runs it, for per-thread buffers); the first failure is kept and rethrown, and
// no job starts after it.
class Writer
{
 public:
  explicit Writer(int threads = 1)
  {
    for (int t = 0; t < std::max(1, threads); ++t) t_.emplace_back([this, t] { run(t); });
  }
  ~Writer()
  {
    {
      std::lock_guard<std::mutex> l(m_);
      done_ = true;
    }
    cv_.notify_all();
    for (auto& t : t_)
      if (t.joinable()) t.join();
  }
  int threads() const { return (int)t_.size(); }
  void submit(std::function<void(int)> job)
  {
    std::lock_guard<std::mutex> l(m_);
    q_.push_back(std::move(job));
    cv_.notify_all();
  }
  void finish()
  {
    {
      std::lock_guard<std::mutex> l(m_);
      if (done_) return;
      done_ = true;
    }
    cv_.notify_all();
    for (auto& t : t_)
      if (t.joinable()) t.join();
    if (!error_.empty()) throw std::runtime_error(error_);
  }
  void check()
  {
    std::lock_guard<std::mutex> l(m_);
    if (!error_.empty()) throw std::runtime_error(error_);
  }

 private:
  void run(int me)
  {
    for (;;)
    {
      std::function<void(int)> job;
      {
        std::unique_lock<std::mutex> l(m_);
        cv_.wait(l, [&] { return !q_.empty() || done_; });
        if (q_.empty()) return;
        job = std::move(q_.front());
        q_.pop_front();
        if (!error_.empty()) continue;
      }
      try
      {
        job(me);
      }
      catch (const std::exception& ex)
      {
        std::lock_guard<std::mutex> l(m_);
        if (error_.empty()) error_ = ex.what();
      }
    }
  }
  std::vector<std::thread> t_;
  std::mutex m_;
  std::condition_variable cv_;
  std::deque<std::function<void(int)>> q_;
  bool done_ = false;
  std::string error_;
};


double now_sec()
{
  return std::chrono::duration<double>(std::chrono::steady_clock::now().time_since_epoch()).count();
}

// ------------------------------------------------------------------ modes
struct Positionals
{
  int radius = 0, grid = 0;
};

bool parse_geometry(const Options& o, const std::vector<std::string>& pos, size_t first, Positionals& g)
{
  std::string err;
  size_t k = first;
  bool ok = true;
  if (o.subset_size > 0) g.radius = (o.subset_size - 1) / 2;
  else ok = parse_int(pos[k++], "subset_radius", 1, std::numeric_limits<int>::max(), g.radius, err);
  if (ok) ok = parse_int(pos[k], "grid_space", 1, std::numeric_limits<int>::max(), g.grid, err);
  if (!ok)
  {
    error_line(err);
    print_usage(std::cerr, false);
  }
  return ok;
}

int run_single(const std::vector<std::string>& args)
{
  g_report.mode = "single-frame";
  Options o;
  std::vector<std::string> pos;
  for (size_t i = 0; i < args.size(); ++i)
  {
    std::string err;
    if (parse_common(args, i, o, err)) continue;
    if (!err.empty())
    {
      error_line(err);
      print_usage(std::cerr, false);
      return 1;
    }
    pos.push_back(args[i]);
  }
  g_report.output_format = o.raw ? "raw" : "csv";
  g_report.frames_total = 1;
  const size_t want = o.subset_size > 0 ? 4 : 5;
  if (pos.size() != want)
  {
    error_line(o.subset_size > 0 && pos.size() == 5 ? "--subset-size conflicts with the positional subset_radius; pass exactly one"
                                                    : "wrong number of positional arguments");
    print_usage(std::cerr, false);
    return 1;
  }
  std::string err;
  if (!validate(o, err))
  {
    error_line(err);
    return 1;
  }
  const std::string ref_path = pos[0], tar_path = pos[1];
  const std::string out_arg = pos[want - 1];
  Positionals g;
  if (!parse_geometry(o, pos, 2, g)) return 1;
  const fs::path out_path = o.raw ? fs::path(raw_name(out_arg)) : fs::path(out_arg);
  g_report.output_path = fs::absolute(out_path).string();

  Samples ref = configure(read_image(ref_path), o.input, ref_path);
  Samples tar = configure(read_image(tar_path), o.input, tar_path);
  std::cerr << summary_line("Reference input", ref) << std::endl;
  if (ref.reduced_to_8)
    warning_line("the reference image is stored as CV_16U but is read with --input-depth 8; pass --input-depth 12 or 16 to keep its precision");
  if (tar.width != ref.width || tar.height != ref.height)
    throw std::runtime_error("reference and target image sizes differ");
  if (tar.dtype != ref.dtype || tar.scale != ref.scale)
    throw std::runtime_error("reference and target are stored at different depths");
  std::vector<dic_poi> q = build_queue(ref.width, ref.height, g.radius, g.grid, o.lines);
  if (q.empty()) throw std::runtime_error("no POIs generated");
  Engine eng(g.radius, o, ref.scale);
  eng.check(dic_set_ref(eng.e, ref.data(), ref.width, ref.height, ref.row_bytes(), ref.dtype), "set reference");
  eng.check(dic_set_tar(eng.e, tar.data(), tar.width, tar.height, tar.row_bytes(), tar.dtype), "set target");
  eng.check(dic_process_pair(eng.e, q.data(), (int64_t)q.size()), "FFTCC + IC-GN");
  if (!out_path.parent_path().empty()) fs::create_directories(out_path.parent_path());
  const double t0 = now_sec();
  Payload p = o.raw ? format_raw(q, o) : format_csv(q, o);
  const double t1 = now_sec();
  publish(out_path, p.bytes.data(), p.bytes.size(), o.fsync);
  const double t2 = now_sec();
  if (o.raw)
  {
    FrameRecord f;
    f.tar_path = tar_path;
    f.output_name = out_path.filename().string();
    f.file = out_path.filename().string();
    f.rows = p.rows;
    f.bytes = p.bytes.size();
    f.format_sec = t1 - t0;
    f.write_sec = t2 - t1;
    float bad = 0.f;
    for (const auto& poi : q) bad += (poi.zncc != -3.f && (!std::isfinite(poi.zncc) || poi.zncc < kSkipFftccZnccThreshold));
    f.qa.bad_ratio = bad / (float)q.size();
    fill_qa_stats(q, f.qa);
    const std::string m = manifest_json(ref_path, "", fs::absolute(out_path).parent_path().string(), g.radius, g.grid, o,
                                        ref, {f}, 0);
    publish(fs::path(out_path.string() + ".manifest.json"), m.data(), m.size(), o.fsync);
  }
  if (o.diagnostics)
  {
    // defaultDiagnosticsDirForSingleFrame (:2794-2800): <output stem>.diagnostics beside the output
    const fs::path parent = out_path.parent_path();
    const fs::path dflt = parent.empty() ? fs::path(out_path.stem().string() + ".diagnostics")
                                         : parent / (out_path.stem().string() + ".diagnostics");
    const fs::path d = o.diagnostics_dir.empty() ? dflt : fs::path(o.diagnostics_dir);
    fs::create_directories(d);
    const std::string text = format_diagnostics(q);
    const fs::path file = diagnostics_file(d, out_path.filename().string());
    publish(file, text.data(), text.size(), o.fsync);
    const std::string m = diagnostics_manifest_json(
        ref_path, "", o, {DiagRecord{tar_path, out_path.filename().string(), file.filename().string(), q.size()}});
    publish(d / "manifest.opencorr-diagnostics.json", m.data(), m.size(), o.fsync);
  }
  g_report.frames_processed = 1;
  return 0;
}

struct ListEntry
{
  std::string tar_path, output_name;
};

std::vector<ListEntry> load_tar_list(const std::string& path)
{
  std::ifstream f(path);
  if (!f) throw std::runtime_error("cannot open tar list " + path);
  std::vector<ListEntry> out;
  std::string line;
  while (std::getline(f, line))
  {
    while (!line.empty() && (line.back() == '\r' || line.back() == ' ' || line.back() == '\t')) line.pop_back();
    if (line.empty()) continue;
    // "<tar_path> <output_name>", split on the last whitespace run; a tab wins (:3504-3512)
    size_t sep = line.rfind('\t');
    if (sep == std::string::npos) sep = line.find_last_of(" \t");
    if (sep == std::string::npos)
      throw std::runtime_error("invalid tar list line (need '<tar_path> <output_name>'): " + line);
    ListEntry e;
    e.tar_path = line.substr(0, sep);
    e.output_name = line.substr(sep + 1);
    while (!e.tar_path.empty() && (e.tar_path.back() == ' ' || e.tar_path.back() == '\t')) e.tar_path.pop_back();
    const size_t ns = e.output_name.find_first_not_of(" \t");
    e.output_name = ns == std::string::npos ? std::string() : e.output_name.substr(ns);
    if (e.tar_path.empty() || e.output_name.empty())
      throw std::runtime_error("invalid tar list line (need '<tar_path> <output_name>'): " + line);
    out.push_back(e);
  }
  return out;
}

void require_utf8(const std::string& what, const std::string& text)
{
  if (!valid_utf8(text)) throw std::runtime_error("non-UTF-8 " + what + ": " + text);
}

// inputIdentity (:3777-3782): canonical path and content fingerprint
Json input_identity(const std::string& path)
{
  const std::string c = fs::canonical(path).string();
  require_utf8("input path", c);
  Json j = Json::object();
  j["path"] = c;
  j["content"] = file_fingerprint(c);
  return j;
}

// validateOutputName (:3784-3792): a unique plain file name, not in the reserved namespace
void check_output_name(const std::string& name)
{
  const fs::path p(name);
  if (name.empty() || p.filename() != p || name == "." || name == ".." || name.rfind(".opencorr-", 0) == 0 ||
      std::any_of(name.begin(), name.end(), [](unsigned char c) { return c < 32 || c == 127; }))
    throw std::runtime_error("output names must be unique plain filenames: " + name);
  require_utf8("output name", name);
}

std::string diagnostics_dir_text(const Options& o)
{
  return o.diagnostics_dir.empty() ? std::string("default") : fs::weakly_canonical(fs::absolute(o.diagnostics_dir)).string();
}

// runContract (:3794-3833): everything that decides the output bytes.  Scheduling options
// (--gpu-device, --threads, --preload, --decode-threads), --durability, --repair and
// --quiet are not part of it.
Json run_contract(const std::string& ref_path, const std::vector<ListEntry>& entries, const Positionals& g,
                  const Options& o, std::vector<std::string>& files)
{
  Json c = Json::object();
  c["schema_version"] = 1;
  c["git_hash"] = DIC_CLI_GIT_HASH;
  c["build_date"] = DIC_CLI_BUILD_DATE;
  c["binary"] = file_fingerprint("/proc/self/exe");
  c["reference"] = input_identity(ref_path);
  Json op = Json::object();
  op["radius"] = g.radius;
  op["step"] = g.grid;
  op["dual_gpu"] = false;
  op["kernel"] = o.legacy_kernel ? "legacy" : "warp";
  op["fftcc"] = "gpu";
  op["max_iteration"] = o.max_iter;
  op["convergence"] = (double)o.conv;
  op["skip_fftcc"] = o.skip_fftcc;
  op["poi_fallback"] = o.poi_fallback;
  op["temporal_extrapolation"] = o.temporal;
  op["format"] = o.raw ? "raw" : "csv";
  Json lines = Json::array();
  for (int y : o.lines) lines.push(y);
  op["line_ys"] = lines;
  op["input_depth"] = depth_name(o.input.depth);
  op["input_align"] = align_name(o.input.align);
  op["input_normalize"] = normalize_name(o.input.normalize);
  op["output_roi_enabled"] = o.roi;
  Json roi = Json::array();
  for (int v : {o.roi_x1, o.roi_y1, o.roi_x2, o.roi_y2}) roi.push(v);
  op["output_roi"] = roi;
  op["output_step"] = o.out_step;
  op["diagnostics"] = o.diagnostics;
  op["diagnostics_dir"] = diagnostics_dir_text(o);
  c["options"] = op;
  Json targets = Json::array();
  std::map<std::string, Json> seen;
  std::set<std::string> names;
  files.clear();
  // The distinct inputs' fingerprints (a full XXH3-128 of every file) on up to 8 threads: the
  // digests do not depend on the order, and the contract is assembled in list order below.
  // Names and paths are checked in list order first, as before, so the first bad entry is
  // still the one reported.
  std::vector<std::string> uniq, canon;
  for (const auto& e : entries)
  {
    check_output_name(e.output_name);
    const std::string file = o.raw ? raw_name(e.output_name) : e.output_name;
    if (!names.insert(file).second) throw std::runtime_error("duplicate output filename: " + file);
    canon.push_back(fs::canonical(e.tar_path).string());
    if (seen.emplace(canon.back(), Json()).second) uniq.push_back(canon.back());
  }
  {
    std::vector<Json> ids(uniq.size());
    std::vector<std::exception_ptr> errs(uniq.size());   // the first failing input in list order is reported
    std::atomic<size_t> next{0};
    const size_t nt = std::min<size_t>({uniq.size(), 8, std::max(1u, std::thread::hardware_concurrency())});
    std::vector<std::thread> pool;
    for (size_t t = 0; t < nt; ++t)
      pool.emplace_back([&] {
        for (size_t i = next++; i < uniq.size(); i = next++)
        {
          try
          {
            ids[i] = input_identity(uniq[i]);
          }
          catch (...)
          {
            errs[i] = std::current_exception();
          }
        }
      });
    for (auto& t : pool) t.join();
    for (const auto& e : errs)
      if (e) std::rethrow_exception(e);
    for (size_t i = 0; i < uniq.size(); ++i) seen[uniq[i]] = std::move(ids[i]);
  }
  for (size_t k = 0; k < entries.size(); ++k)
  {
    const auto& e = entries[k];
    const std::string file = o.raw ? raw_name(e.output_name) : e.output_name;
    auto it = seen.find(canon[k]);
    Json t = Json::object();
    t["input"] = it->second;
    t["output_name"] = e.output_name;
    t["file"] = file;
    targets.push(t);
    files.push_back(file);
  }
  c["targets"] = targets;
  return c;
}

// An existing manifest must describe a prefix of the requested frames (:4000-4030): a
// reader takes the frame list from it.
void check_existing_manifests(const fs::path& root, const fs::path& diag_dir, const std::vector<ListEntry>& entries,
                              const std::vector<std::string>& files, uint64_t rows, uint64_t diag_rows, const Options& o)
{
  const auto same_input = [](const std::string& a, const std::string& b) {
    std::error_code e1, e2;
    const fs::path x = fs::weakly_canonical(a, e1), y = fs::weakly_canonical(b, e2);
    return !e1 && !e2 && x == y;
  };
  const fs::path raw_m = root / "manifest.opencorr-raw.json";
  if (o.raw && fs::exists(raw_m))
  {
    const Json m = read_json_file(raw_m);
    if (!m.is_object() || m.str_or("format", "") != "opencorr-gpu-raw-v1" || !m.has("frames") || !m.at("frames").is_array())
      throw std::runtime_error("invalid existing raw manifest: unexpected layout");
    const Json& fr = m.at("frames");
    if (fr.size() > entries.size()) throw std::runtime_error("existing manifest is not a prefix of this run");
    for (size_t i = 0; i < fr.size(); ++i)
    {
      const Json& f = fr.at(i);
      if (!f.is_object() || f.str_or("output_name", "") != entries[i].output_name || f.str_or("file", "") != files[i] ||
          !same_input(f.str_or("tar_path", ""), entries[i].tar_path) || f.u64_or("rows", ~0ull) != rows)
        throw std::runtime_error("existing raw manifest does not describe the requested frames");
    }
  }
  const fs::path diag_m = diag_dir / "manifest.opencorr-diagnostics.json";
  if (o.diagnostics && fs::exists(diag_m))
  {
    const Json m = read_json_file(diag_m);
    Json cols = Json::array();
    for (const char* c : {"x", "y", "iteration", "convergence", "status", "zncc"}) cols.push(c);
    if (!m.is_object() || m.str_or("format", "") != "opencorr-gpu-diagnostics-csv-v1" || !m.has("columns") ||
        m.at("columns") != cols || !m.has("frames") || !m.at("frames").is_array() || m.at("frames").size() > entries.size())
      throw std::runtime_error("invalid diagnostics manifest schema");
    for (size_t i = 0; i < m.at("frames").size(); ++i)
    {
      const Json& f = m.at("frames").at(i);
      if (!f.is_object() || f.str_or("output_name", "") != entries[i].output_name ||
          f.str_or("file", "") != diagnostics_file(diag_dir, files[i]).filename().string() ||
          f.u64_or("rows", ~0ull) != diag_rows)
        throw std::runtime_error("diagnostics manifest does not describe the requested frames");
    }
  }
}

int run_multi(const std::vector<std::string>& args)
{
  g_report.mode = "multi-frame";
  g_report.multi = true;
  Options o;
  std::string ref_path, list_path, out_dir;
  std::vector<std::string> pos;
  for (size_t i = 0; i < args.size(); ++i)
  {
    const std::string& a = args[i];
    if (a == "--multi-frame") continue;
    if ((a == "--ref" || a == "--tar-list" || a == "--output-dir") && i + 1 < args.size())
    {
      (a == "--ref" ? ref_path : a == "--tar-list" ? list_path : out_dir) = args[++i];
      continue;
    }
    if (a == "--ref" || a == "--tar-list" || a == "--output-dir")
    {
      error_line("missing value for " + a);
      print_usage(std::cerr, false);
      return 1;
    }
    std::string err;
    if (parse_common(args, i, o, err)) continue;
    if (!err.empty())
    {
      error_line(err);
      print_usage(std::cerr, false);
      return 1;
    }
    pos.push_back(a);
  }
  g_report.output_format = o.raw ? "raw" : "csv";
  if (ref_path.empty() || list_path.empty() || out_dir.empty())
  {
    error_line("--multi-frame needs --ref, --tar-list and --output-dir");
    print_usage(std::cerr, false);
    return 1;
  }
  g_report.output_dir = fs::absolute(out_dir).lexically_normal().string();
  if (o.subset_size > 0 && pos.size() == 2)
  {
    error_line("--subset-size conflicts with the positional subset_radius; pass exactly one");
    return 1;
  }
  if (pos.size() != (o.subset_size > 0 ? 1u : 2u))
  {
    error_line("wrong number of positional arguments (expected <subset_radius> <grid_space>; positional arguments given: " +
               std::to_string(pos.size()) + ")");
    print_usage(std::cerr, false);
    return 1;
  }
  std::string err;
  if (!validate(o, err))
  {
    error_line(err);
    return 1;
  }
  Positionals g;
  if (!parse_geometry(o, pos, 0, g)) return 1;
  const std::vector<ListEntry> entries = load_tar_list(list_path);
  if (entries.empty()) throw std::runtime_error("tar list is empty");
  g_report.frames_total = (long long)entries.size();
  // the ledger is JSON: paths and names must be UTF-8, refused before any file exists
  require_utf8("reference path", ref_path);
  require_utf8("output directory", fs::absolute(out_dir).string());
  if (!o.diagnostics_dir.empty()) require_utf8("diagnostics directory", fs::absolute(o.diagnostics_dir).string());
  for (const auto& e : entries)
  {
    require_utf8("target path", e.tar_path);
    require_utf8("output name", e.output_name);
  }
  fs::create_directories(out_dir);

  Samples ref = configure(read_image(ref_path), o.input, ref_path);
  std::cerr << summary_line("Reference input", ref) << std::endl;
  if (ref.reduced_to_8)
    warning_line("the reference image is stored as CV_16U but is read with --input-depth 8; pass --input-depth 12 or 16 to keep its precision");
  std::vector<dic_poi> tmpl = build_queue(ref.width, ref.height, g.radius, g.grid, o.lines);
  if (tmpl.empty()) throw std::runtime_error("no POIs generated");
  const int64_t n = (int64_t)tmpl.size();
  uint64_t out_rows = 0;   // rows of every frame payload after --output-roi / --output-step
  for (const auto& poi : tmpl) out_rows += o.keep((int)poi.x, (int)poi.y) ? 1 : 0;

  // the run record: a rerun of the same command verifies or resumes, anything else is refused
  const fs::path root(out_dir);
  const fs::path diag_dir = o.diagnostics ? (o.diagnostics_dir.empty() ? root / "diagnostics" : fs::path(o.diagnostics_dir))
                                          : fs::path();
  std::vector<std::string> files;
  Json contract = run_contract(ref_path, entries, g, o, files);
  std::vector<LedgerOutput> outs;
  for (size_t k = 0; k < entries.size(); ++k)
  {
    outs.push_back(LedgerOutput{"frame/" + files[k], root / files[k], out_rows, o.raw ? (uint64_t)kRecordBytes : 0});
    if (o.diagnostics)
    {
      const fs::path d = diagnostics_file(diag_dir, files[k]);
      outs.push_back(LedgerOutput{"diagnostics/" + d.filename().string(), d, (uint64_t)n, 0});
    }
  }
  std::vector<fs::path> manifests;
  if (o.raw) manifests.push_back(root / "manifest.opencorr-raw.json");
  if (o.diagnostics) manifests.push_back(diag_dir / "manifest.opencorr-diagnostics.json");
  RunLedger ledger(root, std::move(contract), std::move(outs), manifests, list_path,
                   o.fsync ? Durability::Fsync : Durability::Rename, o.repair);
  if (ledger.quarantined())
    std::cerr << "Repair: quarantined " << ledger.quarantined() << " damaged file(s) in " << ledger.quarantine_dir().string()
              << "; they are regenerated by replay" << std::endl;
  check_existing_manifests(root, diag_dir, entries, files, out_rows, (uint64_t)n, o);
  ledger.archive_residue();
  if (ledger.complete())
  {
    std::ostringstream mib;
    mib.setf(std::ios::fixed);
    mib.precision(1);
    mib << (double)ledger.verified_bytes() / (1024.0 * 1024.0);
    std::cerr << "Verified complete run; no computation or output rewrite required (" << ledger.verified_files()
              << " output files re-read and checked, " << mib.str() << " MiB, plus a full fingerprint of every input)"
              << std::endl;
    std::cerr << "Processed frames: 0, skipped: " << entries.size() << std::endl;
    g_report.frames_skipped = (long long)entries.size();
    return 0;
  }
  ledger.begin();
  g_report.resumed_files = (long long)ledger.existing_files();
  if (ledger.existing_files())
    std::cerr << "Resume: " << ledger.existing_files()
              << " verified files; replay from frame 1 to restore temporal state (no overwrite)" << std::endl;
  std::cerr << "Durability: " << (o.fsync ? "fsync" : "rename") << (o.repair ? ", repair: enabled" : "") << std::endl;
  if (!o.quiet)
    std::cerr << "Multi-frame: " << entries.size() << " targets, image " << ref.width << "x" << ref.height << ", radius "
              << g.radius << ", grid " << g.grid << ", " << n << " POIs, skip_fftcc=" << (o.skip_fftcc ? "on" : "off")
              << ", poi_fallback=" << (o.poi_fallback ? "on" : "off") << std::endl;

  Engine eng(g.radius, o, ref.scale);
  eng.check(dic_set_ref(eng.e, ref.data(), ref.width, ref.height, ref.row_bytes(), ref.dtype), "set reference");
  const dic_frame_policy pol{o.skip_fftcc ? 1 : 0, o.poi_fallback ? 1 : 0, kSkipFftccZnccThreshold,
                             kSkipFftccBadRatioMargin, /*learned_seed=*/0, o.temporal ? 1 : 0};
  eng.check(dic_sequence_begin(eng.e, tmpl.data(), n, &pol), "sequence begin");

  std::vector<std::string> paths;
  for (const auto& e : entries) paths.push_back(e.tar_path);
  // everything the writer's jobs reference is declared before the writer, so that it
  // outlives the writer thread on every exit path
  std::vector<FrameRecord> frames(entries.size());
  std::mutex frames_m;
  // Two writer threads format and publish frames while the next ones are solved; a frame's
  // results stay in their page-locked ring slot until its writer is done (the loop keeps at
  // most kWriters frames unwritten, the ring has two more slots).
  constexpr int kWriters = 2;
  std::vector<PinnedPois> bufs;
  for (int b = 0; b < kWriters + 2; ++b) bufs.emplace_back((size_t)n);
  if (o.diagnostics) fs::create_directories(diag_dir);
  Preloader pre(paths, o.input, o.preload, o.decode_threads);
  std::vector<Payload> payloads(kWriters);   // one output buffer per writer thread
  // DIC_CLI_PROFILE set: per-stage time totals on stderr at the end (diagnostics only; the
  // writer jobs add to t_format / t_publish, so these too are declared before the writer)
  const bool profile = std::getenv("DIC_CLI_PROFILE") != nullptr;
  double t_get = 0, t_stage = 0, t_enqueue = 0, t_fetch = 0, t_throttle = 0, t_format = 0, t_publish = 0;
  std::mutex prof_m;
  Writer writer(kWriters);
  bool baseline_ready = false;
  float baseline = 0.f;
  long long depth_mismatches = 0;
  // Frame k + 1 is decoded (preload thread) and staged (its upload started on the engine's
  // upload stream) before frame k is solved, so decode, upload and solve overlap.
  auto check_frame = [&](const Samples& t, size_t k) {
    if (t.width != ref.width || t.height != ref.height)
      throw std::runtime_error("target " + entries[k].tar_path + " is " + std::to_string(t.width) + "x" +
                               std::to_string(t.height) + ", the reference " + std::to_string(ref.width) + "x" +
                               std::to_string(ref.height));
    if (t.dtype != ref.dtype || t.scale != ref.scale)
    {
      ++depth_mismatches;
      throw std::runtime_error("target " + entries[k].tar_path + " is not on the reference's grey scale");
    }
  };
  auto stage = [&](size_t k) {
    const double a = now_sec();
    Samples t = pre.get(k);
    const double b = now_sec();
    check_frame(t, k);
    eng.check(dic_stage_frame(eng.e, t.data(), t.width, t.height, t.row_bytes(), t.dtype), "stage frame");
    pre.recycle(std::move(t));   // dic_stage_frame has copied it
    t_get += b - a;
    t_stage += now_sec() - b;
  };
  auto enqueue = [&] {
    const double a = now_sec();
    eng.check(dic_sequence_frame(eng.e, nullptr, ref.width, ref.height, ref.row_bytes(), ref.dtype, DIC_PIXELS_STAGED,
                                 nullptr, nullptr),
              "frame");
    t_enqueue += now_sec() - a;
  };
  stage(0);
  enqueue();
  std::exception_ptr next_failed;   // a bad next frame fails the run after this frame is written
  for (size_t k = 0; k < entries.size(); ++k)
  {
    writer.check();
    if (next_failed) std::rethrow_exception(next_failed);
    // frame k is running: decode-wait and stage frame k + 1, enqueue it behind frame k, then
    // read frame k's results (one frame back) while frame k + 1 runs
    bool next_enqueued = false;
    if (k + 1 < entries.size())
    {
      try
      {
        stage(k + 1);
        enqueue();
        next_enqueued = true;
      }
      catch (...)
      {
        next_failed = std::current_exception();
      }
    }
    PinnedPois& res = bufs[k % bufs.size()];
    dic_frame_report rep{};
    const bool attempted_skip = o.skip_fftcc && k > 0;
    const double tf = now_sec();
    eng.check(dic_sequence_fetch(eng.e, next_enqueued ? 1 : 0, res.data(), &rep), "frame results");
    t_fetch += now_sec() - tf;
    FrameRecord f;
    f.tar_path = entries[k].tar_path;
    f.output_name = entries[k].output_name;
    f.file = o.raw ? raw_name(entries[k].output_name) : entries[k].output_name;
    FrameQa& qa = f.qa;
    qa.bad_ratio = (float)rep.bad_after_repair / (float)n;
    if (o.skip_fftcc && !baseline_ready && !attempted_skip)
    {
      baseline = qa.bad_ratio;
      baseline_ready = true;
      if (!o.quiet)
        std::cerr << "  [BASELINE] skip-FFTCC guard baseline_bad_ratio=" << baseline
                  << ", margin=" << kSkipFftccBadRatioMargin << ", fallback_threshold=" << baseline + kSkipFftccBadRatioMargin
                  << ", source=" << f.output_name << std::endl;
    }
    qa.has_baseline = baseline_ready;
    qa.baseline_bad_ratio = baseline;
    qa.has_threshold = o.skip_fftcc && baseline_ready;
    qa.fallback_threshold = baseline + kSkipFftccBadRatioMargin;
    qa.fallback_used = rep.frame_fallback_used != 0;
    qa.skip_fftcc_used = attempted_skip;
    qa.poi_fallback_count = rep.repaired_candidates;
    qa.poi_fallback_recovered = rep.repaired_recovered;
    qa.temporal_seed_count = rep.temporal_seed_count;
    if (rep.temporal_seed_count > 0)
    {
      ++g_report.temporal_seed_frames;
      g_report.temporal_seed_pois += rep.temporal_seed_count;
    }
    if (attempted_skip) ++g_report.skip_fftcc_frames;
    if (qa.fallback_used)
    {
      ++g_report.fallback_frames;
      if (!o.quiet)
        std::cerr << "  [FALLBACK] " << f.output_name << " reason=bad_ratio > baseline + margin"
                  << " bad_ratio=" << (float)rep.bad_before_repair / (float)n << ", baseline_bad_ratio=" << baseline
                  << ", margin=" << kSkipFftccBadRatioMargin << ", fallback_threshold=" << qa.fallback_threshold
                  << ", post_fallback_bad_ratio=" << qa.bad_ratio << ", re-ran FFTCC + ICGN" << std::endl;
    }
    if (rep.repaired_candidates > 0)
    {
      ++g_report.poi_fallback_frames;
      g_report.poi_fallback_pois += rep.repaired_candidates;
      g_report.poi_fallback_recovered += rep.repaired_recovered;
      if (!o.quiet)
        std::cerr << "  [POI-FALLBACK] " << f.output_name << " count=" << rep.repaired_candidates
                  << ", recovered=" << rep.repaired_recovered << ", post_bad_ratio=" << qa.bad_ratio << std::endl;
    }
    // format + publish on a writer thread; the ring slot is reused kWriters + 2 frames later,
    // after its writer is done with it (the loop below)
    const size_t idx = k;
    const PoiSpan resp = res;
    writer.submit([&, idx, resp, f](int me) mutable {
      fill_qa_stats(resp, f.qa);
      const double t0 = now_sec();
      Payload& p = payloads[(size_t)me];   // this thread's buffer, reused frame after frame
      if (o.raw) format_raw_into(resp, o, p);
      else p = format_csv(resp, o);
      const double t1 = now_sec();
      ledger.publish(root / f.file, p.bytes.data(), p.bytes.size());
      f.rows = p.rows;
      f.bytes = p.bytes.size();
      f.format_sec = t1 - t0;
      f.write_sec = now_sec() - t1;
      {
        std::lock_guard<std::mutex> pl(prof_m);
        t_format += f.format_sec;
        t_publish += f.write_sec;
      }
      if (o.diagnostics)
      {
        const std::string text = format_diagnostics(resp);
        ledger.publish(diagnostics_file(diag_dir, f.file), text.data(), text.size());
      }
      std::lock_guard<std::mutex> l(frames_m);
      frames[idx] = f;
    });
    if (!o.quiet)
      std::cerr << "[" << (k + 1) << "/" << entries.size() << "] " << entries[k].tar_path << " -> " << f.file
                << " (bad_ratio " << qa.bad_ratio << (attempted_skip ? ", skip-FFTCC" : ", FFTCC") << ")" << std::endl;
    ++g_report.frames_processed;
    // keep at most kWriters frames unwritten (frames finish out of order; every earlier
    // frame was waited for in an earlier iteration), so that no ring slot is refilled under
    // its writer
    const double tt = now_sec();
    if (k >= (size_t)kWriters)
      for (;;)
      {
        {
          std::lock_guard<std::mutex> l(frames_m);
          if (!frames[k - kWriters].file.empty()) break;
        }
        writer.check();
        std::this_thread::sleep_for(std::chrono::microseconds(200));
      }
    t_throttle += now_sec() - tt;
  }
  writer.finish();
  if (profile)
    std::fprintf(stderr,
                 "[profile] frames=%zu decode-wait=%.3f stage=%.3f enqueue=%.3f fetch=%.3f writer-throttle=%.3f "
                 "format=%.3f publish=%.3f (s; format/publish summed over %d writer threads)\n",
                 entries.size(), t_get, t_stage, t_enqueue, t_fetch, t_throttle, t_format, t_publish, kWriters);
  if (o.raw)
  {
    const std::string m = manifest_json(ref_path, list_path, out_dir, g.radius, g.grid, o, ref, frames, depth_mismatches);
    publish(root / "manifest.opencorr-raw.json", m.data(), m.size(), o.fsync);
  }
  if (o.diagnostics)
  {
    std::vector<DiagRecord> dr;
    for (size_t k = 0; k < entries.size(); ++k)
      dr.push_back(DiagRecord{entries[k].tar_path, entries[k].output_name,
                              diagnostics_file(diag_dir, files[k]).filename().string(), (size_t)n});
    const std::string m = diagnostics_manifest_json(ref_path, list_path, o, dr);
    publish(diag_dir / "manifest.opencorr-diagnostics.json", m.data(), m.size(), o.fsync);
  }
  ledger.finish();
  try
  {
    ledger.archive_residue();   // after the completion record: a failure here is only a warning
  }
  catch (const std::exception& ex)
  {
    warning_line(std::string("post-run housekeeping: ") + ex.what());
  }
  if (!o.quiet)
    std::cerr << "Done: " << entries.size() << " frames, skip-FFTCC frames " << g_report.skip_fftcc_frames
              << ", frames with fallback FFTCC " << g_report.fallback_frames << ", POI-level fallback POIs "
              << g_report.poi_fallback_pois << " (recovered " << g_report.poi_fallback_recovered << ")" << std::endl;
  return 0;
}

// ------------------------------------------------------------------ --verify-only
// auditLayoutFromContract (:4571-4611): the files a contract promises, by the run's naming
AuditLayout layout_from_contract(const Json& contract, const fs::path& root)
{
  AuditLayout l;
  const Json& op = contract.at("options");
  const std::string format = op.at("format").as_string();
  if (format != "csv" && format != "raw") throw std::runtime_error("unknown output format in contract: " + format);
  const bool raw = format == "raw";
  const bool diag = op.has("diagnostics") && op.at("diagnostics").is_bool() && op.at("diagnostics").as_bool();
  fs::path dd;
  if (diag)
  {
    const std::string rec = op.str_or("diagnostics_dir", "default");
    dd = rec == "default" ? root / "diagnostics" : fs::path(rec);
  }
  for (const auto& t : contract.at("targets").items())
  {
    const std::string file = t.at("file").as_string();
    check_output_name(file);
    l.outputs.push_back(AuditOutput{"frame/" + file, root / file, raw ? (uint64_t)kRecordBytes : 0, true});
    if (diag)
    {
      const fs::path d = diagnostics_file(dd, file);
      l.outputs.push_back(AuditOutput{"diagnostics/" + d.filename().string(), d, 0, false});
    }
  }
  if (raw) l.manifests.push_back(root / "manifest.opencorr-raw.json");
  if (diag) l.manifests.push_back(dd / "manifest.opencorr-diagnostics.json");
  return l;
}

// runVerifyOnly (:4613-4760): one JSON verdict on stdout, a summary on stderr; computes,
// creates and moves nothing and opens no GPU.  Exit 0 only for "complete".
int run_verify(const std::vector<std::string>& args)
{
  Json report = Json::object();
  Json contract;
  if (args.size() != 2 || args[1].empty())
  {
    const std::string msg = "--verify-only takes exactly one argument, the multi-frame output directory (got " +
                            std::to_string(args.size() - 1) + (args.size() == 2 ? ", empty)" : ")");
    std::cerr << "Error: " << msg << std::endl;
    report["status"] = "error";
    report["complete"] = false;
    report["output_dir"] = nullptr;
    report["problems"] = Json::array();
    report["problems"].push(msg);
  }
  else
    try
    {
      report = audit_run_directory(args[1], [&](const Json& found, const fs::path& root) {
        if (contract.is_null()) contract = found;   // the recorded contract comes first
        return layout_from_contract(found, root);
      });
      // a reader takes the frame list from the raw manifest: it must list exactly the
      // contract's frames, with the sizes on disk
      const std::string status = report.at("status").as_string();
      if ((status == "complete" || status == "inputs_changed") && contract.at("options").at("format").as_string() == "raw")
      {
        const fs::path root(report.at("output_dir").as_string());
        std::string problem;
        try
        {
          const Json m = read_json_file(root / "manifest.opencorr-raw.json");
          const Json& fr = m.at("frames");
          const Json& tg = contract.at("targets");
          if (!fr.is_array())
            problem = "raw manifest layout is invalid: frames is not an array";
          else if (fr.size() != tg.size())
            problem = "raw manifest lists " + std::to_string(fr.size()) + " frames, the contract " + std::to_string(tg.size());
          else
            for (size_t i = 0; i < fr.size() && problem.empty(); ++i)
            {
              const std::string file = tg.at(i).at("file").as_string();
              std::error_code ec;
              const auto size = fs::file_size(root / fr.at(i).str_or("file", ""), ec);
              if (fr.at(i).str_or("file", "") != file || fr.at(i).str_or("output_name", "") != tg.at(i).at("output_name").as_string() ||
                  ec || size != fr.at(i).u64_or("bytes", ~0ull))
                problem = "raw manifest entry " + std::to_string(i + 1) + " does not describe frame file " + file;
            }
        }
        catch (const std::system_error&)
        {
          throw;
        }
        catch (const std::exception& ex)
        {
          problem = std::string("raw manifest layout is invalid: ") + ex.what();
        }
        if (!problem.empty())
        {
          report["problems"].push(problem);
          report["status"] = "damaged";
          report["complete"] = false;
        }
      }
    }
    catch (const std::system_error& ex)
    {
      report["status"] = "error";
      report["complete"] = false;
      report["problems"] = Json::array();
      report["problems"].push(std::string(ex.what()) + " (errno=" + std::to_string(ex.code().value()) + ")");
    }
    catch (const std::exception& ex)
    {
      report["status"] = "error";
      report["complete"] = false;
      report["problems"] = Json::array();
      report["problems"].push(std::string(ex.what()));
    }
  const bool complete = report.has("complete") && report.at("complete").is_bool() && report.at("complete").as_bool();
  if (!report.has("output_dir")) report["output_dir"] = args.size() > 1 ? Json(args[1]) : Json();
  // the verdict first, then the counts, then the detail
  std::string line = "{\"schema\":\"fasticgn.verify-only/1\"";
  std::set<std::string> done;
  const auto put = [&](const std::string& k, const Json& v) {
    line += "," + json_quote(k) + ":" + v.dump();
    done.insert(k);
  };
  for (const char* k : {"status", "complete"})
    if (report.has(k)) put(k, report.at(k));
  put("exit_code", Json(complete ? 0 : 1));
  for (const char* k : {"output_dir", "frames_expected", "frames_verified", "files_expected", "files_verified",
                        "bytes_verified", "rows_per_frame", "problems", "warnings", "completion", "manifests", "inputs",
                        "contract"})
    if (report.has(k)) put(k, report.at(k));
  for (const auto& m : report.members())
    if (!done.count(m.first)) put(m.first, m.second);
  // the binary that checked; the one that wrote the directory is under "contract"
  put("tool", Json(kTool));
  put("version", Json(kVersion));
  put("git_hash", Json(DIC_CLI_GIT_HASH));
  line += "}";
  std::cerr << "Verify-only: " << report.str_or("status", "error");
  if (report.has("frames_expected"))
    std::cerr << ", " << report.u64_or("frames_verified", 0) << "/" << report.u64_or("frames_expected", 0)
              << " frames match the ledger";
  std::cerr << "; nothing was computed or written" << std::endl;
  if (report.has("problems"))
    for (const auto& pr : report.at("problems").items()) std::cerr << "  problem: " << pr.as_string() << std::endl;
  if (report.has("warnings"))
    for (const auto& w : report.at("warnings").items()) std::cerr << "  note: " << w.as_string() << std::endl;
  std::cout << line << std::endl;
  return complete ? 0 : 1;
}

void collect_warning(const std::string& text) { g_report.warnings.push_back(text); }

}  // namespace

int main(int argc, char** argv)
{
  const double start = now_sec();
  std::vector<std::string> args(argv + 1, argv + argc);
  // its one argument may be any directory name (even -h)
  if (!args.empty() && args[0] == "--verify-only") return run_verify(args);
  set_warning_sink(collect_warning);
  for (const auto& a : args)
    if (a == "--help" || a == "-h")
    {
      print_usage(std::cout, true);
      return 0;
    }
  if (args.size() == 1 && args[0] == "--version")
  {
    print_version();
    return 0;
  }
  int rc = 1;
  try
  {
    if (std::find(args.begin(), args.end(), "--multi-frame") != args.end())
      rc = run_multi(args);
    else if (args.empty())
    {
      print_usage(std::cerr, false);
      error_line("no arguments");
    }
    else
      rc = run_single(args);
  }
  catch (const std::exception& ex)
  {
    error_line(ex.what());
    rc = 1;
  }
  print_status(rc, now_sec() - start);
  return rc;
}
