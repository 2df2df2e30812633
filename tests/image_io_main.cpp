// Test driver for the command line's image decoder (fasticgn_gb300/cli/image_io.*): decodes
// the files named on the command line in order, once with fresh buffers and once reusing the
// previous frame's buffers (the frame loop's path), and prints per file the geometry, the
// stored depth, the range and a checksum of the samples for both; the test compares them.
#include "image_io.h"

#include <cstdio>
#include <string>
#include <vector>

namespace
{
unsigned long long checksum(const dic_cli::Image& im)
{
  unsigned long long h = 1469598103934665603ull;
  const size_t n = (size_t)im.width * im.height;
  for (size_t i = 0; i < n; ++i)
  {
    const unsigned v = im.bits == 8 ? im.u8[i] : im.u16[i];
    h = (h ^ v) * 1099511628211ull;
  }
  return h;
}

void line(const char* kind, const std::string& path, const dic_cli::Image& im)
{
  std::printf("%s %s %d %d %d %.0f %.0f %llu\n", kind, path.c_str(), im.width, im.height, im.bits, im.min_value,
              im.max_value, checksum(im));
}
}  // namespace

int main(int argc, char** argv)
{
  std::vector<uint8_t> buf;
  dic_cli::Image prev;
  for (int a = 1; a < argc; ++a)
  {
    const std::string path = argv[a];
    const dic_cli::Image fresh = dic_cli::read_image(path);
    line("fresh", path, fresh);
    dic_cli::Image reused = dic_cli::read_image(path, buf, std::move(prev));
    line("reused", path, reused);
    prev = std::move(reused);   // its vectors (and buf) carry over to the next file
  }
  return 0;
}
