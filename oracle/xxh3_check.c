/* Checker for the ledger's XXH3-128 (test infrastructure, not the product).
 *
 * Built against the xxHash header the reference vendors (third_party/xxhash/xxhash.h,
 * header-only) by oracle/build.py into oracle/_ref/xxh3_ref, only where the reference
 * tree is present.  For each length given on the command line it hashes that many bytes
 * of a fixed xorshift32 stream (seed 0x12345678, low byte of each step) and prints
 * "<length> <32 hex digits>" in XXH128's canonical order. */
#define XXH_INLINE_ALL
#include "xxhash.h"

#include <stdio.h>
#include <stdlib.h>

static void fill(unsigned char* p, size_t n)
{
  unsigned int x = 0x12345678u;
  for (size_t i = 0; i < n; ++i)
  {
    x ^= x << 13;
    x ^= x >> 17;
    x ^= x << 5;
    p[i] = (unsigned char)(x & 0xffu);
  }
}

int main(int argc, char** argv)
{
  for (int a = 1; a < argc; ++a)
  {
    const size_t n = (size_t)strtoull(argv[a], NULL, 10);
    unsigned char* p = (unsigned char*)malloc(n ? n : 1);
    if (!p) return 2;
    fill(p, n);
    XXH128_canonical_t c;
    XXH128_canonicalFromHash(&c, XXH3_128bits(p, n));
    printf("%zu ", n);
    for (int i = 0; i < 16; ++i) printf("%02x", c.digest[i]);
    printf("\n");
    free(p);
  }
  return 0;
}
