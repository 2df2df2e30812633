// Test harness for the command line's XXH3-128 (fasticgn_gb300/cli/xxh3.cpp): the same
// xorshift32 byte stream as oracle/xxh3_check.c, hashed in one call and, to check the
// incremental form, in chunks of several sizes; prints "<length> <hex>" or a mismatch.
#include "xxh3.h"

#include <cstdio>
#include <cstdlib>
#include <vector>

int main(int argc, char** argv)
{
  for (int a = 1; a < argc; ++a)
  {
    const size_t n = (size_t)std::strtoull(argv[a], nullptr, 10);
    std::vector<unsigned char> p(n);
    unsigned int x = 0x12345678u;
    for (size_t i = 0; i < n; ++i)
    {
      x ^= x << 13;
      x ^= x >> 17;
      x ^= x << 5;
      p[i] = (unsigned char)(x & 0xffu);
    }
    const dic_cli::Hash128 whole = dic_cli::xxh3_128(p.data(), n);
    for (size_t chunk : {1, 7, 64, 100, 256, 257, 1000, 4096})
    {
      dic_cli::Xxh3Stream s;
      for (size_t o = 0; o < n; o += chunk) s.update(p.data() + o, o + chunk < n ? chunk : n - o);
      if (!(s.digest() == whole))
      {
        std::printf("%zu chunked-%zu-differs\n", n, chunk);
        return 1;
      }
    }
    std::printf("%zu %s\n", n, dic_cli::hex128(whole).c_str());
  }
  return 0;
}
