// Image decode and grey-level handling for the command line.  See image_io.h.
#include "image_io.h"

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <fstream>
#include <sstream>
#include <stdexcept>

namespace dic_cli
{
namespace
{

// The whole file into `buf`, sized from the file and filled with large reads.  `buf` keeps
// its capacity across calls, so a frame loop touches no fresh pages (a character-by-character
// stream copy into a new vector cost ~45 ms per 8 MB frame; this costs a few ms).
void slurp(const std::string& path, std::vector<uint8_t>& buf)
{
  std::FILE* f = std::fopen(path.c_str(), "rb");
  if (!f) throw std::runtime_error("cannot open image " + path);
  size_t size = 0;
  if (std::fseek(f, 0, SEEK_END) == 0)
  {
    const long n = std::ftell(f);
    size = n > 0 ? (size_t)n : 0;
    std::rewind(f);
  }
  buf.resize(size);
  size_t got = size ? std::fread(buf.data(), 1, size, f) : 0;
  buf.resize(got);
  // a file that grew since it was sized (or whose size was unknown): read to its end
  constexpr size_t kChunk = size_t(1) << 20;
  while (got == size && !std::ferror(f))
  {
    const size_t old = buf.size();
    buf.resize(old + kChunk);
    const size_t more = std::fread(buf.data() + old, 1, kChunk, f);
    buf.resize(old + more);
    if (more < kChunk) break;
  }
  const bool failed = std::ferror(f) != 0;
  std::fclose(f);
  if (failed) throw std::runtime_error("cannot read image " + path);
}

// ------------------------------------------------------------------ PGM (Netpbm)
struct PnmCursor
{
  const std::vector<uint8_t>& d;
  size_t p = 2;
  void skip_space_and_comments()
  {
    for (;;)
    {
      while (p < d.size() && (d[p] == ' ' || d[p] == '\t' || d[p] == '\n' || d[p] == '\r' || d[p] == '\v' ||
                              d[p] == '\f'))
        ++p;
      if (p < d.size() && d[p] == '#')
      {
        while (p < d.size() && d[p] != '\n' && d[p] != '\r') ++p;
        continue;
      }
      return;
    }
  }
  long number(const std::string& path)
  {
    skip_space_and_comments();
    if (p >= d.size() || d[p] < '0' || d[p] > '9') throw std::runtime_error("malformed PGM header: " + path);
    long v = 0;
    while (p < d.size() && d[p] >= '0' && d[p] <= '9')
    {
      v = v * 10 + (d[p++] - '0');
      if (v > (1L << 30)) throw std::runtime_error("PGM header value too large: " + path);
    }
    return v;
  }
};

Image read_pgm(const std::vector<uint8_t>& d, const std::string& path, Image&& img)
{
  const bool binary = d[1] == '5';
  PnmCursor c{d};
  img.width = (int)c.number(path);
  img.height = (int)c.number(path);
  const long maxval = c.number(path);
  if (img.width <= 0 || img.height <= 0 || maxval <= 0 || maxval > 65535)
    throw std::runtime_error("unsupported PGM geometry or maxval: " + path);
  img.bits = maxval > 255 ? 16 : 8;
  const size_t n = (size_t)img.width * img.height;
  if (binary)
  {
    ++c.p;  // the single whitespace byte after maxval
    const size_t bytes = n * (img.bits / 8);
    if (c.p + bytes > d.size()) throw std::runtime_error("truncated PGM: " + path);
    if (img.bits == 8)
      img.u8.assign(d.begin() + c.p, d.begin() + c.p + n);
    else
    {
      img.u16.resize(n);
      for (size_t i = 0; i < n; ++i) img.u16[i] = (uint16_t)((d[c.p + 2 * i] << 8) | d[c.p + 2 * i + 1]);
    }
  }
  else
  {
    if (img.bits == 8) img.u8.resize(n);
    else img.u16.resize(n);
    for (size_t i = 0; i < n; ++i)
    {
      const long v = c.number(path);
      if (v > maxval) throw std::runtime_error("PGM sample above maxval: " + path);
      if (img.bits == 8) img.u8[i] = (uint8_t)v;
      else img.u16[i] = (uint16_t)v;
    }
  }
  return img;
}

// ------------------------------------------------------------------ TIFF (baseline)
struct TiffReader
{
  const std::vector<uint8_t>& d;
  bool le;
  const std::string& path;
  uint32_t u16at(size_t o) const
  {
    if (o + 2 > d.size()) throw std::runtime_error("truncated TIFF: " + path);
    return le ? (uint32_t)(d[o] | d[o + 1] << 8) : (uint32_t)(d[o] << 8 | d[o + 1]);
  }
  uint32_t u32at(size_t o) const
  {
    if (o + 4 > d.size()) throw std::runtime_error("truncated TIFF: " + path);
    return le ? (uint32_t)d[o] | (uint32_t)d[o + 1] << 8 | (uint32_t)d[o + 2] << 16 | (uint32_t)d[o + 3] << 24
              : (uint32_t)d[o] << 24 | (uint32_t)d[o + 1] << 16 | (uint32_t)d[o + 2] << 8 | (uint32_t)d[o + 3];
  }
  // values of a SHORT or LONG tag (count entries)
  std::vector<uint32_t> values(size_t entry) const
  {
    const uint32_t type = u16at(entry + 2), count = u32at(entry + 4);
    if (type != 3 && type != 4) throw std::runtime_error("unsupported TIFF tag type: " + path);
    if (count > (1u << 24)) throw std::runtime_error("TIFF tag count too large: " + path);
    const size_t size = type == 3 ? 2 : 4;
    const size_t base = size * count <= 4 ? entry + 8 : u32at(entry + 8);
    std::vector<uint32_t> out(count);
    for (uint32_t k = 0; k < count; ++k) out[k] = type == 3 ? u16at(base + 2 * k) : u32at(base + 4 * k);
    return out;
  }
};

Image read_tiff(const std::vector<uint8_t>& d, const std::string& path, Image&& img)
{
  TiffReader t{d, d[0] == 'I', path};
  if (t.u16at(2) != 42) throw std::runtime_error("not a classic TIFF: " + path);
  const size_t ifd = t.u32at(4);
  const uint32_t entries = t.u16at(ifd);
  if (entries > 4096) throw std::runtime_error("TIFF directory too large: " + path);
  uint32_t width = 0, height = 0, bits = 1, compression = 1, spp = 1, photometric = 1, rows_per_strip = 0,
           sample_format = 1, planar = 1;
  std::vector<uint32_t> offsets, counts;
  for (uint32_t k = 0; k < entries; ++k)
  {
    const size_t e = ifd + 2 + 12 * (size_t)k;
    const uint32_t tag = t.u16at(e);
    switch (tag)
    {
      case 256: width = t.values(e)[0]; break;
      case 257: height = t.values(e)[0]; break;
      case 258: bits = t.values(e)[0]; break;
      case 259: compression = t.values(e)[0]; break;
      case 262: photometric = t.values(e)[0]; break;
      case 273: offsets = t.values(e); break;
      case 277: spp = t.values(e)[0]; break;
      case 278: rows_per_strip = t.values(e)[0]; break;
      case 279: counts = t.values(e); break;
      case 284: planar = t.values(e)[0]; break;
      case 339: sample_format = t.values(e)[0]; break;
      default: break;
    }
  }
  if (compression != 1) throw std::runtime_error("compressed TIFF is not supported: " + path);
  if (spp != 1 || planar != 1) throw std::runtime_error("only single-channel grey TIFF is supported: " + path);
  if ((bits != 8 && bits != 16) || sample_format != 1)
    throw std::runtime_error("only 8- or 16-bit unsigned TIFF samples are supported: " + path);
  if (photometric > 1) throw std::runtime_error("only grey TIFF (photometric 0/1) is supported: " + path);
  if (width == 0 || height == 0 || offsets.empty() || offsets.size() != counts.size())
    throw std::runtime_error("malformed TIFF strips: " + path);
  if (rows_per_strip == 0 || rows_per_strip > height) rows_per_strip = height;
  img.width = (int)width;
  img.height = (int)height;
  img.bits = (int)bits;
  const size_t bpp = bits / 8, row = (size_t)width * bpp, total = row * height;
  std::vector<uint8_t> raw;
  raw.reserve(total);
  for (size_t s = 0; s < offsets.size() && raw.size() < total; ++s)
  {
    const size_t n = std::min<size_t>(counts[s], total - raw.size());
    if ((size_t)offsets[s] + n > d.size()) throw std::runtime_error("truncated TIFF strip: " + path);
    raw.insert(raw.end(), d.begin() + offsets[s], d.begin() + offsets[s] + n);
  }
  if (raw.size() < total) throw std::runtime_error("TIFF strips hold fewer bytes than the image: " + path);
  const size_t n = (size_t)width * height;
  const uint32_t maxv = bits == 8 ? 255u : 65535u;
  if (bits == 8)
  {
    img.u8.assign(raw.begin(), raw.begin() + n);
    if (photometric == 0)
      for (auto& v : img.u8) v = (uint8_t)(maxv - v);
  }
  else
  {
    img.u16.resize(n);
    for (size_t i = 0; i < n; ++i)
      img.u16[i] = t.le ? (uint16_t)(raw[2 * i] | raw[2 * i + 1] << 8) : (uint16_t)(raw[2 * i] << 8 | raw[2 * i + 1]);
    if (photometric == 0)
      for (auto& v : img.u16) v = (uint16_t)(maxv - v);
  }
  return img;
}

double logical_max(Depth d)
{
  return d == Depth::k8 ? 255.0 : d == Depth::k12 ? 4095.0 : 65535.0;
}

}  // namespace

Image read_image(const std::string& path) { return read_image(path, std::vector<uint8_t>{}, Image{}); }

Image read_image(const std::string& path, std::vector<uint8_t>&& file_buf, Image&& reuse)
{
  std::vector<uint8_t> d = std::move(file_buf);
  return read_image(path, d, std::move(reuse));
}

Image read_image(const std::string& path, std::vector<uint8_t>& d, Image&& reuse)
{
  slurp(path, d);
  Image img;
  // the vectors of a previous frame: same size, so no reallocation and no fresh pages
  img.u8 = std::move(reuse.u8);
  img.u16 = std::move(reuse.u16);
  if (d.size() >= 2 && d[0] == 'P' && (d[1] == '5' || d[1] == '2')) img = read_pgm(d, path, std::move(img));
  else if (d.size() >= 8 && ((d[0] == 'I' && d[1] == 'I') || (d[0] == 'M' && d[1] == 'M')))
    img = read_tiff(d, path, std::move(img));
  else throw std::runtime_error("unsupported image format (PGM P5/P2 and uncompressed grey TIFF are read): " + path);
  // range in the stored integer type (vectorises; a double per sample does not)
  unsigned lo = 65535, hi = 0;
  if (img.bits == 8)
  {
    uint8_t l8 = 255, h8 = 0;
    for (uint8_t v : img.u8) { l8 = v < l8 ? v : l8; h8 = v > h8 ? v : h8; }
    lo = l8;
    hi = h8;
  }
  else
  {
    uint16_t l16 = 65535, h16 = 0;
    for (uint16_t v : img.u16) { l16 = v < l16 ? v : l16; h16 = v > h16 ? v : h16; }
    lo = l16;
    hi = h16;
  }
  const bool empty = img.bits == 8 ? img.u8.empty() : img.u16.empty();
  img.min_value = empty ? 1e300 : (double)lo;
  img.max_value = empty ? -1e300 : (double)hi;
  return img;
}

Samples configure(Image&& img, const InputOptions& opt, const std::string& path)
{
  Samples s;
  s.width = img.width;
  s.height = img.height;
  s.source_min = img.min_value;
  s.source_max = img.max_value;
  s.source_bits = img.bits;
  if (opt.depth == Depth::k8)
  {
    s.effective_depth = Depth::k8;
    s.dtype = 1;
    if (img.bits == 8)
      s.u8 = std::move(img.u8);
    else
    {
      // 16 -> 8 bit: value / 256, rounded half to even
      s.u8.resize(img.u16.size());
      for (size_t i = 0; i < img.u16.size(); ++i)
      {
        const uint32_t v = img.u16[i], q = v >> 8, r = v & 255u;
        const uint32_t out = q + ((r > 128u || (r == 128u && (q & 1u))) ? 1u : 0u);
        s.u8[i] = (uint8_t)std::min<uint32_t>(out, 255u);
      }
      s.reduced_to_8 = true;
    }
    double scale = 1.0;
    switch (opt.normalize)
    {
      case Normalize::kNone: break;
      case Normalize::kTo8: break;
      case Normalize::kTo16: scale = 65535.0 / 255.0; break;
      case Normalize::kUnit: scale = 1.0 / 255.0; break;
    }
    s.scale = (float)scale;
  }
  else
  {
    Depth eff = opt.depth;
    if (eff == Depth::kAuto) eff = img.bits == 8 ? Depth::k8 : (img.max_value <= 4095.0 ? Depth::k12 : Depth::k16);
    s.effective_depth = eff;
    double scale = 1.0;
    if (eff == Depth::k12)
    {
      Align a = opt.align == Align::kAuto ? (img.max_value > 4095.0 ? Align::kLeft : Align::kRight) : opt.align;
      s.effective_align = a;
      if (a == Align::kRight && img.max_value > 4095.0)
        throw std::runtime_error("12-bit right-aligned input has values above 4095: " + path);
      if (a == Align::kLeft) scale *= 1.0 / 16.0;
    }
    switch (opt.normalize)
    {
      case Normalize::kNone: break;
      case Normalize::kTo8: scale *= 255.0 / logical_max(eff); break;
      case Normalize::kTo16: scale *= 65535.0 / logical_max(eff); break;
      case Normalize::kUnit: scale *= 1.0 / logical_max(eff); break;
    }
    s.scale = (float)scale;
    if (img.bits == 8)
    {
      s.dtype = 1;
      s.u8 = std::move(img.u8);
    }
    else
    {
      s.dtype = 2;
      s.u16 = std::move(img.u16);
    }
  }
  // stored range after conversion: the source range when the samples passed through
  // unchanged, else one integer pass over the reduced 8-bit samples
  double lo = img.min_value, hi = img.max_value;
  if (s.reduced_to_8)
  {
    uint8_t l8 = 255, h8 = 0;
    for (uint8_t v : s.u8) { l8 = v < l8 ? v : l8; h8 = v > h8 ? v : h8; }
    lo = s.u8.empty() ? 1e300 : l8;
    hi = s.u8.empty() ? -1e300 : h8;
  }
  s.output_min = lo * s.scale;
  s.output_max = hi * s.scale;
  return s;
}

const char* depth_name(Depth d)
{
  switch (d)
  {
    case Depth::k8: return "8";
    case Depth::k12: return "12";
    case Depth::k16: return "16";
    default: return "auto";
  }
}
const char* align_name(Align a)
{
  switch (a)
  {
    case Align::kRight: return "right";
    case Align::kLeft: return "left";
    default: return "auto";
  }
}
const char* normalize_name(Normalize n)
{
  switch (n)
  {
    case Normalize::kNone: return "none";
    case Normalize::kTo8: return "to-8";
    case Normalize::kTo16: return "to-16";
    default: return "unit";
  }
}

std::string summary_line(const char* label, const Samples& s)
{
  // the grey levels the solver sees: u8/u16 samples times the upload scale (float)
  const bool as_float = !(s.effective_depth == Depth::k8 && s.scale == 1.f && s.dtype == 1);
  std::ostringstream o;
  o << label << ": source_depth=" << (s.source_bits == 8 ? "CV_8U" : "CV_16U") << ", source_range=[" << s.source_min
    << "," << s.source_max << "], effective_depth=" << depth_name(s.effective_depth)
    << ", effective_align=" << align_name(s.effective_align) << ", output_depth=" << (as_float ? "CV_32F" : "CV_8U")
    << ", output_range=[" << s.output_min << "," << s.output_max << "], scale=" << s.scale;
  return o.str();
}

}  // namespace dic_cli
