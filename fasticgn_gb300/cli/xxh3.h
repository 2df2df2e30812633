// XXH3-128 (xxHash 0.8 family, seed 0, default secret): the content fingerprint of the
// output ledger.  The reference's ledger (src/cli_output_integrity.cpp:35, :363-382) names
// its digests "xxh3-128" and writes them as 32 lowercase hex digits of the canonical
// (big-endian high half, then low half) form, so ledgers written by either binary can be
// audited by the other.  This is a restatement of the published algorithm, not a fast
// vectorised variant: one scalar pass, about 2-4 GB/s, which is far above the rate the
// command line produces output.
#pragma once

#include <cstddef>
#include <cstdint>
#include <string>

namespace dic_cli
{

struct Hash128
{
  uint64_t low = 0, high = 0;
  bool operator==(const Hash128& o) const { return low == o.low && high == o.high; }
};

Hash128 xxh3_128(const void* data, size_t size);

// incremental form for files: the whole input is never held in memory
class Xxh3Stream
{
 public:
  Xxh3Stream();
  void update(const void* data, size_t size);
  Hash128 digest() const;

 private:
  static constexpr size_t kStripe = 64, kBlockStripes = 16, kBuffer = 256;
  uint64_t acc_[8];
  unsigned char buf_[kBuffer];
  size_t buffered_ = 0;
  size_t stripes_in_block_ = 0;   // stripes of the current 1024-byte block already consumed
  uint64_t total_ = 0;
  unsigned char last_stripe_[kStripe];   // the 64 bytes before the buffer, for short tails
  bool long_ = false;                    // at least one stripe consumed
  void consume_stripes(const unsigned char* p, size_t n);
};

// 32 lowercase hex digits, high half first (XXH128's canonical byte order)
std::string hex128(const Hash128& h);

}  // namespace dic_cli
