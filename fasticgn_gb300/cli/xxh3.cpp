// XXH3-128, restated from the published xxHash algorithm description (XXH3, 128-bit
// variant, seed 0, the 192-byte default secret).  Constants below are the algorithm's own:
// the five 64-bit and three 32-bit primes, the two avalanche multipliers and the default
// secret.  Checked against the reference's vendored xxhash.h (third_party/xxhash, compiled
// as a separate checker) on inputs of every length class.
#include "xxh3.h"

#include <cstdio>
#include <cstring>

namespace dic_cli
{
namespace
{

constexpr uint64_t kP32_1 = 0x9E3779B1ULL, kP32_2 = 0x85EBCA77ULL, kP32_3 = 0xC2B2AE3DULL;
constexpr uint64_t kP64_1 = 0x9E3779B185EBCA87ULL, kP64_2 = 0xC2B2AE3D27D4EB4FULL, kP64_3 = 0x165667B19E3779F9ULL,
                   kP64_4 = 0x85EBCA77C2B2AE63ULL, kP64_5 = 0x27D4EB2F165667C5ULL;
constexpr uint64_t kMx1 = 0x165667919E3779F9ULL, kMx2 = 0x9FB21C651E98DF25ULL;
constexpr size_t kSecretSize = 192;

const unsigned char kSecret[kSecretSize] = {
    0xb8, 0xfe, 0x6c, 0x39, 0x23, 0xa4, 0x4b, 0xbe, 0x7c, 0x01, 0x81, 0x2c, 0xf7, 0x21, 0xad, 0x1c,
    0xde, 0xd4, 0x6d, 0xe9, 0x83, 0x90, 0x97, 0xdb, 0x72, 0x40, 0xa4, 0xa4, 0xb7, 0xb3, 0x67, 0x1f,
    0xcb, 0x79, 0xe6, 0x4e, 0xcc, 0xc0, 0xe5, 0x78, 0x82, 0x5a, 0xd0, 0x7d, 0xcc, 0xff, 0x72, 0x21,
    0xb8, 0x08, 0x46, 0x74, 0xf7, 0x43, 0x24, 0x8e, 0xe0, 0x35, 0x90, 0xe6, 0x81, 0x3a, 0x26, 0x4c,
    0x3c, 0x28, 0x52, 0xbb, 0x91, 0xc3, 0x00, 0xcb, 0x88, 0xd0, 0x65, 0x8b, 0x1b, 0x53, 0x2e, 0xa3,
    0x71, 0x64, 0x48, 0x97, 0xa2, 0x0d, 0xf9, 0x4e, 0x38, 0x19, 0xef, 0x46, 0xa9, 0xde, 0xac, 0xd8,
    0xa8, 0xfa, 0x76, 0x3f, 0xe3, 0x9c, 0x34, 0x3f, 0xf9, 0xdc, 0xbb, 0xc7, 0xc7, 0x0b, 0x4f, 0x1d,
    0x8a, 0x51, 0xe0, 0x4b, 0xcd, 0xb4, 0x59, 0x31, 0xc8, 0x9f, 0x7e, 0xc9, 0xd9, 0x78, 0x73, 0x64,
    0xea, 0xc5, 0xac, 0x83, 0x34, 0xd3, 0xeb, 0xc3, 0xc5, 0x81, 0xa0, 0xff, 0xfa, 0x13, 0x63, 0xeb,
    0x17, 0x0d, 0xdd, 0x51, 0xb7, 0xf0, 0xda, 0x49, 0xd3, 0x16, 0x55, 0x26, 0x29, 0xd4, 0x68, 0x9e,
    0x2b, 0x16, 0xbe, 0x58, 0x7d, 0x47, 0xa1, 0xfc, 0x8f, 0xf8, 0xb8, 0xd1, 0x7a, 0xd0, 0x31, 0xce,
    0x45, 0xcb, 0x3a, 0x8f, 0x95, 0x16, 0x04, 0x28, 0xaf, 0xd7, 0xfb, 0xca, 0xbb, 0x4b, 0x40, 0x7e,
};

// little-endian loads assembled byte by byte: the same on x86_64 and aarch64
inline uint32_t le32(const unsigned char* p)
{
  return (uint32_t)p[0] | ((uint32_t)p[1] << 8) | ((uint32_t)p[2] << 16) | ((uint32_t)p[3] << 24);
}
inline uint64_t le64(const unsigned char* p) { return (uint64_t)le32(p) | ((uint64_t)le32(p + 4) << 32); }
inline uint32_t rotl32(uint32_t v, int r) { return (v << r) | (v >> (32 - r)); }
inline uint32_t swap32(uint32_t v)
{
  return ((v & 0xffu) << 24) | ((v & 0xff00u) << 8) | ((v >> 8) & 0xff00u) | (v >> 24);
}
inline uint64_t swap64(uint64_t v) { return ((uint64_t)swap32((uint32_t)v) << 32) | swap32((uint32_t)(v >> 32)); }
inline uint64_t shift_xor(uint64_t v, int s) { return v ^ (v >> s); }

inline Hash128 wide_mul(uint64_t a, uint64_t b)
{
  const unsigned __int128 p = (unsigned __int128)a * b;
  return Hash128{(uint64_t)p, (uint64_t)(p >> 64)};
}
inline uint64_t folded_mul(uint64_t a, uint64_t b)
{
  const Hash128 p = wide_mul(a, b);
  return p.low ^ p.high;
}
// the 64-bit finaliser of the XXH3 family
inline uint64_t mix_final(uint64_t h) { return shift_xor(shift_xor(h, 37) * kMx1, 32); }
// XXH64's finaliser, used by the 0..3-byte inputs
inline uint64_t mix_final64(uint64_t h)
{
  h = shift_xor(h, 33) * kP64_2;
  h = shift_xor(h, 29) * kP64_3;
  return shift_xor(h, 32);
}

Hash128 hash_upto3(const unsigned char* in, size_t n, const unsigned char* s)
{
  if (n == 0)
    return Hash128{mix_final64(le64(s + 64) ^ le64(s + 72)), mix_final64(le64(s + 80) ^ le64(s + 88))};
  const uint32_t lo = ((uint32_t)in[0] << 16) | ((uint32_t)in[n >> 1] << 24) | (uint32_t)in[n - 1] | ((uint32_t)n << 8);
  const uint32_t hi = rotl32(swap32(lo), 13);
  const uint64_t flip_lo = (uint64_t)(le32(s) ^ le32(s + 4));
  const uint64_t flip_hi = (uint64_t)(le32(s + 8) ^ le32(s + 12));
  return Hash128{mix_final64((uint64_t)lo ^ flip_lo), mix_final64((uint64_t)hi ^ flip_hi)};
}

Hash128 hash_4to8(const unsigned char* in, size_t n, const unsigned char* s)
{
  const uint64_t word = (uint64_t)le32(in) + ((uint64_t)le32(in + n - 4) << 32);
  Hash128 m = wide_mul(word ^ (le64(s + 16) ^ le64(s + 24)), kP64_1 + ((uint64_t)n << 2));
  m.high += m.low << 1;
  m.low ^= m.high >> 3;
  m.low = shift_xor(shift_xor(m.low, 35) * kMx2, 28);
  m.high = mix_final(m.high);
  return m;
}

Hash128 hash_9to16(const unsigned char* in, size_t n, const unsigned char* s)
{
  const uint64_t flip_lo = le64(s + 32) ^ le64(s + 40);
  const uint64_t flip_hi = le64(s + 48) ^ le64(s + 56);
  const uint64_t first = le64(in);
  uint64_t last = le64(in + n - 8);
  Hash128 m = wide_mul(first ^ last ^ flip_lo, kP64_1);
  m.low += (uint64_t)(n - 1) << 54;
  last ^= flip_hi;
  m.high += last + (uint64_t)(uint32_t)last * (kP32_2 - 1);
  m.low ^= swap64(m.high);
  Hash128 h = wide_mul(m.low, kP64_2);
  h.high += m.high * kP64_2;
  return Hash128{mix_final(h.low), mix_final(h.high)};
}

inline uint64_t mix16(const unsigned char* in, const unsigned char* s)
{
  return folded_mul(le64(in) ^ le64(s), le64(in + 8) ^ le64(s + 8));
}

inline void mix32(Hash128& acc, const unsigned char* a, const unsigned char* b, const unsigned char* s)
{
  acc.low += mix16(a, s);
  acc.low ^= le64(b) + le64(b + 8);
  acc.high += mix16(b, s + 16);
  acc.high ^= le64(a) + le64(a + 8);
}

Hash128 finish_mid(const Hash128& acc, size_t n)
{
  const uint64_t lo = acc.low + acc.high;
  const uint64_t hi = acc.low * kP64_1 + acc.high * kP64_4 + (uint64_t)n * kP64_2;
  return Hash128{mix_final(lo), (uint64_t)0 - mix_final(hi)};
}

Hash128 hash_17to128(const unsigned char* in, size_t n, const unsigned char* s)
{
  Hash128 acc{(uint64_t)n * kP64_1, 0};
  // outermost pair first, working inwards, as many 32-byte pairs as the length needs
  const int pairs = n > 96 ? 4 : n > 64 ? 3 : n > 32 ? 2 : 1;
  for (int k = pairs - 1; k >= 0; --k) mix32(acc, in + 16 * k, in + n - 16 * (k + 1), s + 32 * k);
  return finish_mid(acc, n);
}

Hash128 hash_129to240(const unsigned char* in, size_t n, const unsigned char* s)
{
  Hash128 acc{(uint64_t)n * kP64_1, 0};
  const size_t rounds = n / 32;
  for (size_t k = 0; k < 4; ++k) mix32(acc, in + 32 * k, in + 32 * k + 16, s + 32 * k);
  acc.low = mix_final(acc.low);
  acc.high = mix_final(acc.high);
  for (size_t k = 4; k < rounds; ++k) mix32(acc, in + 32 * k, in + 32 * k + 16, s + 3 + 32 * (k - 4));
  mix32(acc, in + n - 16, in + n - 32, s + 136 - 17 - 16);
  return finish_mid(acc, n);
}

// one 64-byte stripe into the eight accumulators
inline void stripe(uint64_t* acc, const unsigned char* in, const unsigned char* s)
{
  for (int i = 0; i < 8; ++i)
  {
    const uint64_t v = le64(in + 8 * i);
    const uint64_t k = v ^ le64(s + 8 * i);
    acc[i ^ 1] += v;
    acc[i] += (k & 0xffffffffULL) * (k >> 32);
  }
}

inline void scramble(uint64_t* acc, const unsigned char* s)
{
  for (int i = 0; i < 8; ++i) acc[i] = (shift_xor(acc[i], 47) ^ le64(s + 8 * i)) * kP32_1;
}

// stripes in order; a block is 16 stripes and ends with a scramble
void run_stripes(uint64_t* acc, size_t& in_block, const unsigned char* p, size_t n)
{
  for (size_t i = 0; i < n; ++i)
  {
    stripe(acc, p + 64 * i, kSecret + 8 * in_block);
    if (++in_block == 16)
    {
      scramble(acc, kSecret + kSecretSize - 64);
      in_block = 0;
    }
  }
}

uint64_t merge(const uint64_t* acc, const unsigned char* s, uint64_t start)
{
  uint64_t r = start;
  for (int i = 0; i < 4; ++i) r += folded_mul(acc[2 * i] ^ le64(s + 16 * i), acc[2 * i + 1] ^ le64(s + 16 * i + 8));
  return mix_final(r);
}

}  // namespace

Xxh3Stream::Xxh3Stream()
{
  const uint64_t init[8] = {kP32_3, kP64_1, kP64_2, kP64_3, kP64_4, kP32_2, kP64_5, kP32_1};
  std::memcpy(acc_, init, sizeof acc_);
  std::memset(last_stripe_, 0, sizeof last_stripe_);
}

void Xxh3Stream::update(const void* data, size_t size)
{
  const unsigned char* p = static_cast<const unsigned char*>(data);
  total_ += size;
  while (size > 0)
  {
    // the buffer is emptied only when more input follows, so the last byte is always
    // still buffered when the digest is taken (the tail rules need the final stripe)
    if (buffered_ == kBuffer)
    {
      run_stripes(acc_, stripes_in_block_, buf_, kBuffer / kStripe);
      std::memcpy(last_stripe_, buf_ + kBuffer - kStripe, kStripe);
      buffered_ = 0;
      long_ = true;
    }
    const size_t take = size < kBuffer - buffered_ ? size : kBuffer - buffered_;
    std::memcpy(buf_ + buffered_, p, take);
    buffered_ += take;
    p += take;
    size -= take;
  }
}

Hash128 Xxh3Stream::digest() const
{
  if (total_ <= 240)
  {
    const size_t n = (size_t)total_;
    if (n <= 3) return hash_upto3(buf_, n, kSecret);
    if (n <= 8) return hash_4to8(buf_, n, kSecret);
    if (n <= 16) return hash_9to16(buf_, n, kSecret);
    if (n <= 128) return hash_17to128(buf_, n, kSecret);
    return hash_129to240(buf_, n, kSecret);
  }
  uint64_t acc[8];
  std::memcpy(acc, acc_, sizeof acc);
  size_t in_block = stripes_in_block_;
  unsigned char tail[kStripe];
  const unsigned char* last;
  if (buffered_ >= kStripe)
  {
    // every whole stripe but the one holding the final byte, then the last 64 bytes
    run_stripes(acc, in_block, buf_, (buffered_ - 1) / kStripe);
    last = buf_ + buffered_ - kStripe;
  }
  else
  {
    // fewer than 64 new bytes: the final stripe reaches back into consumed input
    std::memcpy(tail, last_stripe_ + buffered_, kStripe - buffered_);
    std::memcpy(tail + kStripe - buffered_, buf_, buffered_);
    last = tail;
  }
  stripe(acc, last, kSecret + kSecretSize - kStripe - 7);
  Hash128 h;
  h.low = merge(acc, kSecret + 11, total_ * kP64_1);
  h.high = merge(acc, kSecret + kSecretSize - 64 - 11, ~(total_ * kP64_2));
  return h;
}

Hash128 xxh3_128(const void* data, size_t size)
{
  Xxh3Stream s;
  s.update(data, size);
  return s.digest();
}

std::string hex128(const Hash128& h)
{
  char b[33];
  std::snprintf(b, sizeof b, "%016llx%016llx", (unsigned long long)h.high, (unsigned long long)h.low);
  return b;
}

}  // namespace dic_cli
