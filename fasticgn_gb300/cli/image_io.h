// Image decode and grey-level handling for the command line (host code, no CUDA).
//
// Decoders: Netpbm PGM (P5 binary and P2 text, 8 or 16 bit, maxval <= 65535) and baseline
// TIFF (uncompressed, one grey sample of 8 or 16 bit per pixel, strips or tiles not needed:
// strips only).  The reference reads images through OpenCV imread; its own tests write PGM.
//
// Depth handling restates opencorr::Image2D's configured load (src/oc_image.cpp:130-200):
// --input-depth 8 hands 8-bit samples to the solver (a 16-bit file is reduced, value / 256
// rounded half to even, as a 16 -> 8 bit convertTo does); 12, 16 and auto hand the stored
// samples over with a float scale: 1/16 for left-aligned 12-bit data, times 255, 65535 or 1
// over the depth's logical maximum for --input-normalize to-8, to-16 and unit.
#pragma once

#include <cstdint>
#include <string>
#include <vector>

namespace dic_cli
{

struct Image
{
  int width = 0, height = 0;
  int bits = 8;                    // 8 or 16 as stored
  std::vector<uint8_t> u8;         // bits == 8
  std::vector<uint16_t> u16;       // bits == 16
  double min_value = 0.0, max_value = 0.0;
};

// Throws std::runtime_error with the file name on any decode error.
Image read_image(const std::string& path);
// The same, reading the file into `file_buf` and decoding into the vectors of `reuse` (a
// previous frame's, returned by the caller): a frame loop then allocates nothing.
Image read_image(const std::string& path, std::vector<uint8_t>& file_buf, Image&& reuse);
Image read_image(const std::string& path, std::vector<uint8_t>&& file_buf, Image&& reuse);

enum class Depth { k8, k12, k16, kAuto };
enum class Align { kRight, kLeft, kAuto };
enum class Normalize { kNone, kTo8, kTo16, kUnit };

struct InputOptions
{
  Depth depth = Depth::k8;
  Align align = Align::kAuto;
  Normalize normalize = Normalize::kNone;
};

// What the solver is handed: samples (u8 or u16) and the scale applied on upload.
struct Samples
{
  int width = 0, height = 0;
  int dtype = 0;                   // dic_dtype
  std::vector<uint8_t> u8;
  std::vector<uint16_t> u16;
  float scale = 1.f;
  // the "Reference input" summary of the reference CLI
  Depth effective_depth = Depth::k8;
  Align effective_align = Align::kAuto;
  double source_min = 0, source_max = 0, output_min = 0, output_max = 0;
  int source_bits = 8;
  bool reduced_to_8 = false;       // a 16-bit file read with depth 8
  const void* data() const { return dtype == 1 ? (const void*)u8.data() : (const void*)u16.data(); }
  int64_t row_bytes() const { return (int64_t)width * (dtype == 1 ? 1 : 2); }
};

Samples configure(Image&& img, const InputOptions& opt, const std::string& path);

const char* depth_name(Depth d);
const char* align_name(Align a);
const char* normalize_name(Normalize n);
std::string summary_line(const char* label, const Samples& s);

}  // namespace dic_cli
