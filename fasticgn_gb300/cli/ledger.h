// Output ledger of the multi-frame command line: crash-consistent publication, the
// .opencorr-state/ run record, contract-checked resume, --repair and --verify-only.
// Behaviour and on-disk layout follow the reference's output integrity layer
// (src/cli_output_integrity.h:20-138, src/cli_output_integrity.cpp; docs/output-integrity.md):
//   .opencorr-state/contract.json          what decides the output bytes (binary, reference,
//                                          options, targets); a resume must match it, the
//                                          target list may only grow by appending
//   .opencorr-state/<xxh3(key)>.json       one intent per output file (key, rows, bytes,
//                                          digest), published before the file itself
//   .opencorr-state/complete.json          the contract digest and the manifests' digests,
//                                          published last
//   .opencorr-state/contract.pending.json  a longer contract until its first new output
//   .opencorr-state/quarantine/<UTC>-<pid>/ files moved aside (never deleted)
// Files appear through a uniquely named temporary (.opencorr-tmp-<pid>-<n>, O_EXCL) in
// the destination directory and a link (payloads: never replaces) or rename (metadata).
// Digests are XXH3-128 (xxh3.h) over the bytes, or over the compact serialisation of a
// parsed JSON document.
#pragma once

#include "json.h"

#include <cstdint>
#include <filesystem>
#include <functional>
#include <memory>
#include <string>
#include <vector>

namespace dic_cli
{
namespace fs = std::filesystem;

enum class Durability { Rename, Fsync };
const char* durability_name(Durability d);

// hex XXH3-128 of a byte range
std::string content_digest(const void* data, size_t size);
// {"algorithm": "xxh3-128", "bytes": n, "digest": hex} of a file's content
Json file_fingerprint(const fs::path& path);
// strict read of a metadata file: a regular, non-symlink file of at most 256 MiB; a file
// that cannot be opened or read raises std::system_error, one that does not parse JsonError
Json read_json_file(const fs::path& path);
// temporary + link (replace = false) or rename (replace = true); sync adds the fsyncs
void publish_file(const fs::path& path, const char* data, size_t size, bool replace, bool sync);
// 2-space indented JSON plus a newline, replacing the destination
void publish_json(const fs::path& path, const Json& value, bool sync);
// "a.b: old -> new; ..." for up to `limit` differing leaves, then a count of the rest
std::string describe_differences(const Json& recorded, const Json& requested, size_t limit = 8);
// warnings printed on stderr are also handed here (the status line repeats them)
void set_warning_sink(void (*sink)(const std::string&));

struct LedgerOutput
{
  std::string key;           // "frame/<file>" or "diagnostics/<file>"
  fs::path path;
  uint64_t rows = 0;
  uint64_t record_bytes = 0; // 0: CSV, one header line plus `rows` lines
};

class RunLedger
{
 public:
  RunLedger(const fs::path& root, Json contract, std::vector<LedgerOutput> outputs, std::vector<fs::path> manifests,
            const fs::path& tar_list, Durability durability, bool repair);
  ~RunLedger();
  RunLedger(const RunLedger&) = delete;
  RunLedger& operator=(const RunLedger&) = delete;

  bool complete() const;           // every output and manifest verified under this contract
  void begin();                    // records the contract; call before the first publish
  void archive_residue();          // moves crash temporaries and a stale pending contract aside
  size_t existing_files() const;   // outputs verified at start
  size_t verified_files() const;   // outputs and manifests re-read at start
  uint64_t verified_bytes() const;
  size_t quarantined() const;
  fs::path quarantine_dir() const; // empty unless something was moved aside
  // one promised output; thread-safe.  A replayed output that is already on disk is kept
  // as it is after its bytes are shown equal to the recorded intent.
  void publish(const fs::path& path, const char* data, size_t size);
  void finish();                   // completion record; every output must be committed

 private:
  struct State;
  std::unique_ptr<State> st_;
};

// --verify-only
struct AuditOutput
{
  std::string key;
  fs::path path;
  uint64_t record_bytes = 0;
  bool frame = true;
};
struct AuditLayout
{
  std::vector<AuditOutput> outputs;
  std::vector<fs::path> manifests;
};
using AuditLayoutFn = std::function<AuditLayout(const Json& contract, const fs::path& root)>;
// the verdict object; "status": complete, incomplete, damaged, inputs_changed, locked,
// not_a_run or not_found.  Changes nothing on disk.
Json audit_run_directory(const fs::path& root, const AuditLayoutFn& layout);

}  // namespace dic_cli
