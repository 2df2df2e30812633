// Output ledger of the multi-frame command line (declared in ledger.h).
//
// The on-disk names, record keys, report keys and messages are the interface the
// reference's tools and the Python pipeline read (docs/output-integrity.md of the
// reference; pipeline/fasticgn_io.py:321-520 reads contract.json, complete.json, the
// intents and contract.pending.json).  The implementation is organised around one
// judgement table:
//
//   1. every promised output is judged once, from its intent record and its file, into one
//      of six states (Judged below);
//   2. a resume looks each state up in kResumeRules (keep, replay, set aside with --repair,
//      refuse), and the --verify-only audit files each state under the report list that
//      audit_list() names;
//   3. the entries of the directories the run owns are classified in one scan
//      (scan_owned), which both the resume's "dedicated directory" rule and the audit's
//      untracked / residue lists read.
#include "ledger.h"

#include "xxh3.h"

#include <algorithm>
#include <atomic>
#include <cerrno>
#include <cstdio>
#include <cstring>
#include <ctime>
#include <iostream>
#include <map>
#include <mutex>
#include <optional>
#include <set>
#include <system_error>

#include <fcntl.h>
#include <sys/file.h>
#include <unistd.h>

namespace dic_cli
{
namespace
{

const std::string kDigestName = "xxh3-128";
const std::string kRepairHint = " (use --repair to quarantine and regenerate it)";
const std::string kTmpPrefix = ".opencorr-tmp-";
// scheduling options that contracts of older builds carry; they never decide an output byte,
// so a resume ignores them and the audit lists them
const std::vector<std::string> kSchedulingOptions = {"gpu_device", "threads", "preload", "decode_threads"};

std::atomic<void (*)(const std::string&)> g_sink{nullptr};
std::atomic<unsigned long long> g_tmp_counter{0};

void note(const std::string& text)
{
  std::cerr << "Warning: " << text << std::endl;
  if (auto s = g_sink.load()) s(text);
}

[[noreturn]] void fail_io(const std::string& what, const fs::path& p)
{
  throw std::system_error(errno ? errno : EIO, std::generic_category(), what + ": " + p.string());
}

// an owned file descriptor
class Handle
{
 public:
  Handle() = default;
  explicit Handle(int fd) : fd_(fd) {}
  ~Handle() { reset(); }
  Handle(const Handle&) = delete;
  Handle& operator=(const Handle&) = delete;
  Handle(Handle&& o) noexcept : fd_(o.fd_) { o.fd_ = -1; }
  Handle& operator=(Handle&& o) noexcept
  {
    if (this != &o)
    {
      reset();
      fd_ = o.release();
    }
    return *this;
  }
  int get() const { return fd_; }
  bool ok() const { return fd_ >= 0; }
  int release()
  {
    const int f = fd_;
    fd_ = -1;
    return f;
  }
  void reset()
  {
    if (fd_ >= 0) ::close(fd_);
    fd_ = -1;
  }

 private:
  int fd_ = -1;
};

Handle open_dir(const fs::path& d, const char* what)
{
  Handle h(::open(d.c_str(), O_RDONLY | O_DIRECTORY | O_CLOEXEC));
  if (!h.ok()) fail_io(what, d);
  return h;
}

void fsync_dir(const fs::path& d)
{
  Handle h = open_dir(d, "open output directory");
  if (::fsync(h.get()) != 0) fail_io("sync output directory", d);
}

void fsync_file(const fs::path& p)
{
  Handle h(::open(p.c_str(), O_WRONLY | O_CLOEXEC | O_NOFOLLOW));
  if (!h.ok()) fail_io("open published output", p);
  if (::fsync(h.get()) != 0) fail_io("sync published output", p);
}

// lstat-style queries: a symlink is never followed
bool present(const fs::path& p) { return fs::exists(fs::symlink_status(p)); }
bool plain_file(const fs::path& p)
{
  const auto st = fs::symlink_status(p);
  return st.type() == fs::file_type::regular;
}
void need_plain_file(const fs::path& p)
{
  if (!plain_file(p)) throw std::runtime_error("expected a regular, non-symlink output file: " + p.string());
}

fs::path absolute_clean(const fs::path& p) { return fs::weakly_canonical(fs::absolute(p)); }
// the directory part resolved, the final component kept (so a symlinked output is seen)
fs::path resolve_parent(const fs::path& p) { return absolute_clean(p.parent_path()) / p.filename(); }

std::string relative_name(const fs::path& p, const fs::path& root)
{
  const fs::path r = p.lexically_relative(root);
  return (!r.empty() && *r.begin() != "..") ? r.string() : p.string();
}

bool is_hex32(const std::string& s)
{
  return s.size() == 32 && s.find_first_not_of("0123456789abcdef") == std::string::npos;
}

// ------------------------------------------------------------------ reserved temporaries
// ".opencorr-tmp-<pid>-<n>" names our own crash temporaries.
enum class Temp
{
  None,        // not in the reserved namespace
  Crash,       // ours, a regular file: archived by the next run
  Malformed,   // reserved prefix, other suffix: left in place with a warning
  Special      // ours by name but not a regular file: left in place with a warning
};

Temp temp_kind(const fs::path& p)
{
  const std::string n = p.filename().string();
  if (n.compare(0, kTmpPrefix.size(), kTmpPrefix) != 0) return Temp::None;
  const std::string rest = n.substr(kTmpPrefix.size());
  const size_t dash = rest.find('-');
  const auto all_digits = [](const std::string& s) {
    return !s.empty() && std::all_of(s.begin(), s.end(), [](char c) { return c >= '0' && c <= '9'; });
  };
  if (dash == std::string::npos || !all_digits(rest.substr(0, dash)) || !all_digits(rest.substr(dash + 1)))
    return Temp::Malformed;
  return plain_file(p) ? Temp::Crash : Temp::Special;
}

// ------------------------------------------------------------------ contract comparison
// A resume compares contracts without the target list (checked as a prefix) and without
// the scheduling options.
Json resume_view(Json c)
{
  if (!c.is_object()) return c;
  c.erase("targets");
  if (c.has("options") && c.at("options").is_object())
    for (const auto& k : kSchedulingOptions) c["options"].erase(k);
  return c;
}

std::string render_leaf(const Json& v)
{
  if (v.kind() == Json::Kind::Float)
  {
    char b[40];
    std::snprintf(b, sizeof b, "%.7g", v.as_double());   // the contract's floats were single precision
    return b;
  }
  try
  {
    return v.dump();
  }
  catch (const JsonError&)
  {
    return "\"<not UTF-8>\"";
  }
}

// dotted path -> rendered leaf
std::map<std::string, std::string> leaves(const Json& v)
{
  std::map<std::string, std::string> out;
  std::vector<std::pair<std::string, const Json*>> todo{{"", &v}};
  while (!todo.empty())
  {
    auto [path, node] = todo.back();
    todo.pop_back();
    if (node->is_object() && node->size() > 0)
      for (const auto& m : node->members()) todo.push_back({path.empty() ? m.first : path + "." + m.first, &m.second});
    else
      out[path] = render_leaf(*node);
  }
  return out;
}

struct Change
{
  std::string path, before, after;
};
std::vector<Change> changes(const Json& a, const Json& b)
{
  const auto la = leaves(a), lb = leaves(b);
  std::set<std::string> keys;
  for (const auto& l : la) keys.insert(l.first);
  for (const auto& l : lb) keys.insert(l.first);
  std::vector<Change> out;
  for (const auto& k : keys)
  {
    const auto x = la.find(k), y = lb.find(k);
    const std::string before = x == la.end() ? "(absent)" : x->second;
    const std::string after = y == lb.end() ? "(absent)" : y->second;
    if (x == la.end() || y == lb.end() || before != after) out.push_back({k, before, after});
  }
  return out;
}

std::string why_contract_differs(const Json& recorded, const Json& requested)
{
  bool binary = false, reference = false, options = false;
  const auto starts = [](const std::string& s, const char* p) { return s.compare(0, std::strlen(p), p) == 0; };
  for (const auto& c : changes(recorded, requested))
  {
    binary |= starts(c.path, "binary.") || c.path == "git_hash" || c.path == "build_date";
    reference |= starts(c.path, "reference.");
    options |= starts(c.path, "options.");
  }
  std::string s = " (recorded -> requested): " + describe_differences(recorded, requested);
  if (options) s += "; an option that decides the output differs from the recorded run";
  if (reference) s += "; the reference image path or content differs";
  if (binary) s += "; another build of the executable wrote this directory (resume needs the byte-identical binary)";
  return s + "; use a new output directory for a different run";
}

// the recorded target list is a prefix of the requested one
bool is_prefix(const Json& recorded, const Json& requested)
{
  if (!recorded.is_array() || !requested.is_array() || recorded.size() > requested.size()) return false;
  return std::equal(recorded.items().begin(), recorded.items().end(), requested.items().begin());
}

std::string why_targets_differ(const Json& recorded, const Json& requested)
{
  if (!recorded.is_array() || !requested.is_array()) return std::string();
  const auto& a = recorded.items();
  const auto& b = requested.items();
  const auto miss = std::mismatch(a.begin(), a.begin() + std::min(a.size(), b.size()), b.begin());
  if (miss.first != a.begin() + std::min(a.size(), b.size()))
  {
    const size_t i = (size_t)(miss.first - a.begin());
    return ": target " + std::to_string(i + 1) + " of the recorded " + std::to_string(a.size()) +
           " differs (recorded -> requested): " + describe_differences(a[i], b[i], 4);
  }
  if (b.size() < a.size())
    return ": the recorded run lists " + std::to_string(a.size()) + " targets, this command only " +
           std::to_string(b.size()) + " (a shorter list is not a resume)";
  return std::string();
}

std::string digest_of(const Json& doc)
{
  const std::string s = doc.dump();
  return content_digest(s.data(), s.size());
}

bool contract_shape(const Json& c)
{
  return c.is_object() && c.has("targets") && c.at("targets").is_array() && c.has("options") &&
         c.at("options").is_object();
}

// ------------------------------------------------------------------ the judgement table
enum class Judged
{
  Verified,       // intent valid, file present, bytes and digest as recorded
  Missing,        // no file (a resume replays it)
  NotRegular,     // a symlink, directory or device where the file should be
  NoIntent,       // a file with no intent record
  InvalidIntent,  // an intent record that does not parse or does not describe its file
  Mismatched      // a file whose size or digest differs from its intent
};

struct Judgement
{
  Judged state = Judged::Missing;
  bool intent_on_disk = false;
  fs::path intent_path;
  std::string intent_error;     // InvalidIntent: why
  Json intent;                  // the valid intent record, when there is one
  uint64_t bytes = 0, rows = 0; // Verified: the file's bytes and the intent's rows
};

fs::path intent_path_for(const fs::path& state_dir, const std::string& key)
{
  return state_dir / (content_digest(key.data(), key.size()) + ".json");
}

// The intent: schema 1, its key, unsigned rows (equal to `rows` when the caller knows them)
// and an xxh3-128 {bytes, digest} record; raw outputs also bytes == rows * record size.
std::string intent_problem(const Json& in, const std::string& key, std::optional<uint64_t> rows, uint64_t record_bytes,
                           const fs::path& ip, const fs::path& file)
{
  if (!in.is_object() || in.str_or("algorithm", "") != kDigestName || !in.has("bytes") || !in.at("bytes").is_unsigned() ||
      !in.has("digest") || !in.at("digest").is_string())
    return "invalid integrity record schema";
  if (!is_hex32(in.at("digest").as_string())) return "invalid integrity digest";
  if (in.u64_or("schema_version", 0) != 1 || in.str_or("key", "") != key || !in.has("rows") ||
      !in.at("rows").is_unsigned() || (rows && in.at("rows").as_u64() != *rows))
    return "invalid output intent: " + ip.string();
  if (record_bytes && in.at("bytes").as_u64() != in.at("rows").as_u64() * record_bytes)
    return "raw record size mismatch in intent: " + file.string();
  return std::string();
}

// Judges one output: the record first, then the file, then its bytes.  I/O faults propagate
// (std::system_error): they say nothing about the run.
Judgement judge(const fs::path& state_dir, const std::string& key, const fs::path& file, uint64_t record_bytes,
                std::optional<uint64_t> rows)
{
  Judgement j;
  j.intent_path = intent_path_for(state_dir, key);
  j.intent_on_disk = present(j.intent_path);
  Json& intent = j.intent;
  if (j.intent_on_disk)
  {
    try
    {
      intent = read_json_file(j.intent_path);
      j.intent_error = intent_problem(intent, key, rows, record_bytes, j.intent_path, file);
    }
    catch (const std::system_error&)
    {
      throw;
    }
    catch (const std::exception& ex)
    {
      j.intent_error = ex.what();
    }
    if (!j.intent_error.empty())
    {
      j.state = Judged::InvalidIntent;
      return j;
    }
  }
  if (!present(file)) j.state = Judged::Missing;
  else if (!plain_file(file)) j.state = Judged::NotRegular;
  else if (!j.intent_on_disk) j.state = Judged::NoIntent;
  else
  {
    const Json seen = file_fingerprint(file);
    const bool same = seen.at("bytes") == intent.at("bytes") && seen.at("digest") == intent.at("digest");
    j.state = same ? Judged::Verified : Judged::Mismatched;
    if (same)
    {
      j.bytes = seen.at("bytes").as_u64();
      j.rows = intent.at("rows").as_u64();
    }
  }
  return j;
}

// What a resume does with each state, without and with --repair.
enum class Step { Keep, Replay, SetAsideFile, SetAsideIntent, Refuse };
struct ResumeRule
{
  Judged state;
  Step plain, repair;
  const char* refusal;   // message prefix (the path follows); nullptr: the judgement's own
  bool hint;             // append the --repair hint
};
constexpr ResumeRule kResumeRules[] = {
    {Judged::Verified, Step::Keep, Step::Keep, nullptr, false},
    {Judged::Missing, Step::Replay, Step::Replay, nullptr, false},
    {Judged::NotRegular, Step::Refuse, Step::Refuse, "expected a regular, non-symlink output file: ", false},
    {Judged::NoIntent, Step::Refuse, Step::SetAsideFile, "existing output has no commit intent: ", true},
    {Judged::Mismatched, Step::Refuse, Step::SetAsideFile, "corrupt/truncated output; resume refused: ", true},
    {Judged::InvalidIntent, Step::Refuse, Step::SetAsideIntent, nullptr, true},
};
const ResumeRule& rule_for(Judged s)
{
  for (const auto& r : kResumeRules)
    if (r.state == s) return r;
  throw std::logic_error("no resume rule");
}

// Under which report list the audit files each damaged or missing state.
const char* audit_list(Judged s)
{
  switch (s)
  {
    case Judged::Missing: return "missing";
    case Judged::NoIntent: return "no_intent";
    case Judged::InvalidIntent: return "invalid_intent";
    case Judged::NotRegular:
    case Judged::Mismatched: return "mismatched";
    default: return nullptr;
  }
}

// ------------------------------------------------------------------ directory scan
enum class Entry
{
  Owned,        // the state directory, a promised output or manifest, or the target list
  Crash,        // our crash temporary (archived by the next run)
  OddReserved,  // reserved name we will not touch
  Foreign       // anything else
};
struct Scanned
{
  fs::path path, dir;
  Entry kind;
};

// One pass over the directories a run owns.  `owned` holds full paths and, for outputs in
// subdirectories of the root, the subdirectory itself.
std::vector<Scanned> scan_owned(const std::vector<fs::path>& dirs, const std::set<fs::path>& owned)
{
  std::vector<Scanned> out;
  for (const auto& d : dirs)
  {
    if (!fs::is_directory(d)) continue;
    for (const auto& e : fs::directory_iterator(d))
    {
      const Temp t = temp_kind(e.path());
      Entry k = Entry::Foreign;
      if (t == Temp::Crash) k = Entry::Crash;
      else if (t != Temp::None) k = Entry::OddReserved;
      else if (owned.count(e.path())) k = Entry::Owned;
      out.push_back({e.path(), d, k});
    }
  }
  return out;
}

// Adds a promised path (and its first component under root) to `owned`; returns the
// directory it lives in when that is not the root.
std::optional<fs::path> own(std::set<fs::path>& owned, const fs::path& p, const fs::path& root)
{
  owned.insert(p);
  const fs::path r = p.lexically_relative(root);
  if (!r.empty() && *r.begin() != "..") owned.insert(root / *r.begin());
  if (p.parent_path() != root) return p.parent_path();
  return std::nullopt;
}

// ------------------------------------------------------------------ completion record
struct Completion
{
  bool present = false, valid = false, current = false;
  std::string error;
  Json record;
};

Completion read_completion(const fs::path& state_dir, const std::string& contract_digest)
{
  Completion c;
  const fs::path p = state_dir / "complete.json";
  c.present = present(p);
  if (!c.present) return c;
  try
  {
    need_plain_file(p);
    c.record = read_json_file(p);
    const Json& r = c.record;
    if (!r.is_object() || r.u64_or("schema_version", 0) != 1 || !r.has("contract_digest") ||
        !r.at("contract_digest").is_string() || !r.has("metadata") || !r.at("metadata").is_object())
      throw std::runtime_error("invalid run completion record");
    c.valid = true;
    c.current = r.at("contract_digest").as_string() == contract_digest;
  }
  catch (const std::system_error&)
  {
    throw;
  }
  catch (const std::exception& ex)
  {
    c.error = ex.what();
  }
  return c;
}

// Up to 20 names per report list, with the exact count beside them.
class ReportLists
{
 public:
  void add(const std::string& list, const std::string& name)
  {
    auto& l = lists_[list];
    if (l.count++ < 20) l.names.push(name);
  }
  size_t count(const std::string& list) const
  {
    const auto it = lists_.find(list);
    return it == lists_.end() ? 0 : it->second.count;
  }
  void store(Json& report, const std::string& list) const
  {
    const auto it = lists_.find(list);
    report[list] = it == lists_.end() ? Json::array() : it->second.names;
    report[list + "_count"] = (unsigned long long)count(list);
  }

 private:
  struct L
  {
    size_t count = 0;
    Json names = Json::array();
  };
  std::map<std::string, L> lists_;
};

}  // namespace

// ------------------------------------------------------------------ public primitives
const char* durability_name(Durability d) { return d == Durability::Fsync ? "fsync" : "rename"; }

void set_warning_sink(void (*sink)(const std::string&)) { g_sink.store(sink); }

std::string content_digest(const void* data, size_t size) { return hex128(xxh3_128(data, size)); }

Json file_fingerprint(const fs::path& path)
{
  Handle h(::open(path.c_str(), O_RDONLY | O_CLOEXEC));
  if (!h.ok()) fail_io("cannot read fingerprint input", path);
  Xxh3Stream digest;
  std::vector<unsigned char> chunk(size_t(1) << 20);
  unsigned long long total = 0;
  for (;;)
  {
    const ssize_t n = ::read(h.get(), chunk.data(), chunk.size());
    if (n == 0) break;
    if (n < 0)
    {
      if (errno == EINTR) continue;
      fail_io("fingerprint read failed", path);
    }
    digest.update(chunk.data(), (size_t)n);
    total += (unsigned long long)n;
  }
  Json j = Json::object();
  j["algorithm"] = kDigestName;
  j["bytes"] = total;
  j["digest"] = hex128(digest.digest());
  return j;
}

Json read_json_file(const fs::path& path)
{
  if (!present(path))
  {
    errno = ENOENT;
    fail_io("open JSON metadata", path);
  }
  need_plain_file(path);
  if (fs::file_size(path) > (uint64_t(256) << 20)) throw std::runtime_error("JSON metadata exceeds 256 MiB: " + path.string());
  Handle h(::open(path.c_str(), O_RDONLY | O_CLOEXEC | O_NOFOLLOW));
  if (!h.ok()) fail_io("open JSON metadata", path);
  std::string text;
  std::vector<char> chunk(65536);
  for (;;)
  {
    const ssize_t n = ::read(h.get(), chunk.data(), chunk.size());
    if (n == 0) break;
    if (n < 0)
    {
      if (errno == EINTR) continue;
      fail_io("read JSON metadata", path);
    }
    text.append(chunk.data(), (size_t)n);
  }
  return Json::parse(text, path.string());
}

void publish_file(const fs::path& path, const char* data, size_t size, bool replace, bool sync)
{
  if (fs::is_symlink(fs::symlink_status(path))) throw std::runtime_error("refusing symlink output: " + path.string());
  const fs::path dir = path.has_parent_path() ? path.parent_path() : fs::path(".");
  // a fresh temporary beside the destination (O_EXCL: never an existing file)
  Handle out;
  fs::path tmp;
  for (int tries = 0; !out.ok(); ++tries)
  {
    if (tries == 1024) fail_io("allocate temporary output", path);
    tmp = dir / (kTmpPrefix + std::to_string(::getpid()) + "-" + std::to_string(g_tmp_counter.fetch_add(1)));
    out = Handle(::open(tmp.c_str(), O_WRONLY | O_CREAT | O_EXCL | O_CLOEXEC, 0666));
    if (!out.ok() && errno != EEXIST) fail_io("create temporary output", tmp);
  }
  try
  {
    for (size_t done = 0; done < size;)
    {
      const ssize_t n = ::write(out.get(), data + done, std::min(size - done, size_t(1) << 30));
      if (n < 0 && errno == EINTR) continue;
      if (n <= 0)
      {
        if (n == 0) errno = EIO;
        fail_io("write temporary output", tmp);
      }
      done += (size_t)n;
    }
    if (sync && ::fsync(out.get()) != 0) fail_io("sync temporary output", tmp);
    if (::close(out.release()) != 0) fail_io("close temporary output", tmp);
    if (replace)
    {
      if (::rename(tmp.c_str(), path.c_str()) != 0) fail_io("publish output", path);
    }
    else
    {
      // link() publishes the finished inode and fails if the name exists: never replaces
      if (::link(tmp.c_str(), path.c_str()) != 0) fail_io("publish new output", path);
      ::unlink(tmp.c_str());
    }
    if (sync) fsync_dir(dir);
  }
  catch (...)
  {
    std::error_code ignored;
    fs::remove(tmp, ignored);
    throw;
  }
}

void publish_json(const fs::path& path, const Json& value, bool sync)
{
  const std::string text = value.dump_indented(2) + "\n";
  publish_file(path, text.data(), text.size(), true, sync);
}

std::string describe_differences(const Json& recorded, const Json& requested, size_t limit)
{
  const auto diff = changes(recorded, requested);
  std::string out;
  for (size_t i = 0; i < diff.size() && i < limit; ++i)
    out += (i ? "; " : "") + (diff[i].path.empty() ? std::string("(value)") : diff[i].path) + ": " + diff[i].before +
           " -> " + diff[i].after;
  if (diff.size() > limit) out += "; and " + std::to_string(diff.size() - limit) + " more";
  return out;
}

// ------------------------------------------------------------------ the run session
struct RunLedger::State
{
  // set up once
  fs::path root, state_dir, list_path;
  Json contract;
  std::string digest;
  bool sync = false, repair = false, had_contract = false, contract_changed = false;
  std::map<fs::path, LedgerOutput> outputs;   // by resolved path
  std::vector<fs::path> manifests;
  std::vector<fs::path> side_dirs;            // output directories other than the root
  std::set<fs::path> owned;
  Handle root_lock;
  std::vector<Handle> side_locks;
  // progress
  std::mutex m;
  std::map<std::string, Json> recorded_intents;   // by key, valid intents found at start
  std::set<std::string> committed;
  size_t existing = 0, verified = 0, set_aside_count = 0;
  uint64_t verified_bytes = 0;
  bool complete = false, begun = false, pending_contract = false;
  fs::path quarantine;

  fs::path contract_file() const { return state_dir / "contract.json"; }
  fs::path pending_file() const { return state_dir / "contract.pending.json"; }

  fs::path quarantine_dir()
  {
    if (quarantine.empty())
    {
      const std::time_t now = std::time(nullptr);
      std::tm utc{};
      ::gmtime_r(&now, &utc);
      char stamp[32];
      std::strftime(stamp, sizeof stamp, "%Y%m%dT%H%M%SZ", &utc);
      quarantine = state_dir / "quarantine" / (std::string(stamp) + "-" + std::to_string(::getpid()));
      fs::create_directories(quarantine);
    }
    return quarantine;
  }

  // moves a file into the quarantine directory (never deletes)
  void set_aside(const fs::path& p)
  {
    const fs::path q = quarantine_dir();
    fs::path dst = q / p.filename();
    for (int k = 1; present(dst); ++k) dst = q / (p.filename().string() + "." + std::to_string(k));
    std::error_code ec;
    fs::rename(p, dst, ec);
    if (ec)
    {
      fs::copy_file(p, dst, fs::copy_options::overwrite_existing);   // another file system
      fs::remove(p);
    }
    ++set_aside_count;
  }

  // the longer contract of an append becomes the recorded one with its first new output
  void promote_pending()
  {
    if (!pending_contract) return;
    publish_json(contract_file(), contract, sync);
    std::error_code ignored;
    fs::remove(pending_file(), ignored);
    pending_contract = false;
  }

  void take_paths(std::vector<LedgerOutput>& outs, std::vector<fs::path>& mans, const fs::path& tar_list);
  void check_recorded_contract();
  void lock_side_dirs();
  void refuse_foreign_entries();
  void check_fresh_directory();
  void resume_outputs();
  void resume_manifests();
  void resume_completion();
};

void RunLedger::State::take_paths(std::vector<LedgerOutput>& outs, std::vector<fs::path>& mans, const fs::path& tar_list)
{
  owned = {state_dir, absolute_clean(tar_list)};
  std::set<fs::path> side;
  for (auto& o : outs)
  {
    o.path = resolve_parent(o.path);
    if (o.path == state_dir || o.path.filename().string().rfind(".opencorr-", 0) == 0)
      throw std::runtime_error("reserved output filename: " + o.path.string());
    if (!outputs.emplace(o.path, o).second) throw std::runtime_error("duplicate output destination: " + o.path.string());
    if (auto d = own(owned, o.path, root)) side.insert(*d);
  }
  for (auto& p : mans)
  {
    p = resolve_parent(p);
    if (outputs.count(p)) throw std::runtime_error("data output collides with manifest: " + p.string());
    if (auto d = own(owned, p, root)) side.insert(*d);
    manifests.push_back(p);
  }
  side_dirs.assign(side.begin(), side.end());
}

void RunLedger::State::check_recorded_contract()
{
  had_contract = present(contract_file());
  if (!had_contract)
  {
    contract_changed = true;
    return;
  }
  const Json recorded = read_json_file(contract_file());
  const Json a = resume_view(recorded), b = resume_view(contract);
  if (a != b)
    throw std::runtime_error("resume rejected: run configuration/reference/binary changed" + why_contract_differs(a, b));
  const Json old_targets = recorded.has("targets") ? recorded.at("targets") : Json();
  if (!is_prefix(old_targets, contract.at("targets")))
    throw std::runtime_error("resume rejected: targets changed/reordered; only an identical prefix plus append is allowed" +
                             why_targets_differ(old_targets, contract.at("targets")));
  contract_changed = recorded != contract;
}

void RunLedger::State::lock_side_dirs()
{
  for (const auto& d : side_dirs)
  {
    fs::create_directories(d);
    Handle h = open_dir(d, "open diagnostics directory");
    if (::flock(h.get(), LOCK_EX | LOCK_NB) != 0) fail_io("diagnostics directory already locked", d);
    side_locks.push_back(std::move(h));
  }
}

// a dedicated directory: anything the run does not own is refused (crash temporaries are
// recognised and archived later)
void RunLedger::State::refuse_foreign_entries()
{
  std::vector<fs::path> dirs{root};
  dirs.insert(dirs.end(), side_dirs.begin(), side_dirs.end());
  for (const auto& e : scan_owned(dirs, owned))
    if (e.kind == Entry::Foreign) throw std::runtime_error("untracked entry in output directory: " + e.path.string());
}

// without a recorded contract nothing the run would write may exist yet
void RunLedger::State::check_fresh_directory()
{
  for (const auto& o : outputs)
    if (present(o.first)) throw std::runtime_error("existing output has no verified run record: " + o.first.string());
  for (const auto& p : manifests)
    if (present(p)) throw std::runtime_error("existing manifest has no verified run record: " + p.string());
  if (fs::exists(state_dir))
    for (const auto& e : fs::directory_iterator(state_dir))
      if (temp_kind(e.path()) == Temp::None) throw std::runtime_error("run state has no valid contract: " + state_dir.string());
}

void RunLedger::State::resume_outputs()
{
  for (const auto& item : outputs)
  {
    const LedgerOutput& o = item.second;
    Judgement j = judge(state_dir, o.key, o.path, o.record_bytes, o.rows);
    for (;;)
    {
      const ResumeRule& r = rule_for(j.state);
      const Step step = repair ? r.repair : r.plain;
      if (step == Step::Refuse)
      {
        const std::string what = r.refusal ? std::string(r.refusal) + o.path.string() : j.intent_error;
        throw std::runtime_error(what + (r.hint ? kRepairHint : std::string()));
      }
      if (step == Step::SetAsideIntent)
      {
        set_aside(j.intent_path);   // then judge the file again, now without a record
        j = judge(state_dir, o.key, o.path, o.record_bytes, o.rows);
        continue;
      }
      if (step == Step::SetAsideFile) set_aside(o.path);
      if (step == Step::Keep)
      {
        committed.insert(o.key);
        verified_bytes += j.bytes;
        ++verified;
        ++existing;
      }
      // a valid record that stays on disk binds the replay: it must reproduce those bytes
      if (j.intent_on_disk) recorded_intents.emplace(o.key, j.intent);
      break;
    }
  }
}

void RunLedger::State::resume_manifests()
{
  for (const auto& p : manifests)
  {
    if (!fs::exists(p)) continue;
    need_plain_file(p);
    try
    {
      (void)read_json_file(p);
      verified_bytes += fs::file_size(p);
      ++verified;
    }
    catch (const std::system_error&)
    {
      throw;
    }
    catch (const std::exception&)
    {
      if (!repair) throw;
      set_aside(p);
    }
  }
}

void RunLedger::State::resume_completion()
{
  Completion c = read_completion(state_dir, digest);
  if (!c.present) return;
  fs::path changed_manifest;
  std::string reason = c.error;
  if (c.valid && c.current)
  {
    // the completion of this very contract vouches for the manifests it digested
    const Json& md = c.record.at("metadata");
    if (md.size() != manifests.size()) reason = "invalid metadata completion record";
    for (const auto& p : manifests)
    {
      if (!reason.empty()) break;
      const std::string name = p.filename().string();
      if (!md.has(name) || !md.at(name).is_string()) reason = "missing metadata completion digest";
      else if (fs::exists(p))
      {
        std::string got;
        try
        {
          got = digest_of(read_json_file(p));
        }
        catch (const std::system_error&)
        {
          throw;
        }
        catch (const std::exception& ex)
        {
          reason = ex.what();
          changed_manifest = p;
          break;
        }
        if (got != md.at(name).as_string())
        {
          reason = "completed manifest changed: " + p.string();
          changed_manifest = p;
        }
      }
    }
  }
  if (!reason.empty())
  {
    if (!repair) throw std::runtime_error(reason + kRepairHint);
    std::cerr << "Repair: run completion record rejected (" << reason << ")" << std::endl;
    set_aside(state_dir / "complete.json");
    if (!changed_manifest.empty() && fs::exists(changed_manifest)) set_aside(changed_manifest);
    complete = false;
    return;
  }
  // a completion of another contract (an append or a resume that did not finish) says
  // nothing about this one: the run continues as an ordinary resume
  complete = c.current && committed.size() == outputs.size() &&
             std::all_of(manifests.begin(), manifests.end(), [](const fs::path& p) { return fs::is_regular_file(p); });
}

RunLedger::RunLedger(const fs::path& root_in, Json contract, std::vector<LedgerOutput> outputs,
                     std::vector<fs::path> manifests, const fs::path& tar_list, Durability durability, bool repair)
    : st_(std::make_unique<State>())
{
  State& s = *st_;
  s.sync = durability == Durability::Fsync;
  s.repair = repair;
  s.root = absolute_clean(root_in);
  s.state_dir = s.root / ".opencorr-state";
  s.contract = std::move(contract);
  s.digest = digest_of(s.contract);
  s.root_lock = open_dir(s.root, "open run directory");
  if (::flock(s.root_lock.get(), LOCK_EX | LOCK_NB) != 0) fail_io("run directory already locked", s.root);
  if (fs::is_symlink(fs::symlink_status(s.state_dir))) throw std::runtime_error("run state must not be a symlink");
  s.take_paths(outputs, manifests, tar_list);
  s.check_recorded_contract();
  s.lock_side_dirs();
  s.refuse_foreign_entries();
  if (!s.had_contract) s.check_fresh_directory();
  s.repair = repair && s.had_contract;   // nothing to repair in a fresh directory
  s.resume_outputs();
  s.resume_manifests();
  if (s.had_contract) s.resume_completion();
}

RunLedger::~RunLedger() = default;

bool RunLedger::complete() const { return st_->complete; }
size_t RunLedger::existing_files() const { return st_->existing; }
size_t RunLedger::verified_files() const { return st_->verified; }
uint64_t RunLedger::verified_bytes() const { return st_->verified_bytes; }
size_t RunLedger::quarantined() const { return st_->set_aside_count; }
fs::path RunLedger::quarantine_dir() const { return st_->quarantine; }

void RunLedger::begin()
{
  State& s = *st_;
  fs::create_directories(s.state_dir);
  if (s.sync) fsync_dir(s.root);
  if (!s.contract_changed)
  {
    std::error_code ignored;
    fs::remove(s.pending_file(), ignored);   // an append that was abandoned
  }
  else if (s.had_contract)
  {
    // an append: the shorter recorded contract stays authoritative until a new output exists
    publish_json(s.pending_file(), s.contract, s.sync);
    s.pending_contract = true;
  }
  else
    publish_json(s.contract_file(), s.contract, s.sync);
  s.begun = true;
}

void RunLedger::archive_residue()
{
  State& s = *st_;
  if (!s.had_contract && !s.begun) return;
  std::vector<fs::path> dirs{s.root};
  if (fs::exists(s.state_dir)) dirs.push_back(s.state_dir);
  dirs.insert(dirs.end(), s.side_dirs.begin(), s.side_dirs.end());
  std::vector<fs::path> crash;
  for (const auto& e : scan_owned(dirs, s.owned))
  {
    if (e.kind == Entry::Crash) crash.push_back(e.path);
    else if (e.kind == Entry::OddReserved)
      note(temp_kind(e.path) == Temp::Special ? "leaving reserved name in place, not a regular file: " + e.path.string()
                                              : "leaving unrecognized reserved name in place: " + e.path.string());
  }
  if (!s.pending_contract && present(s.pending_file()))
  {
    if (plain_file(s.pending_file())) crash.push_back(s.pending_file());
    else note("leaving reserved name in place, not a regular file: " + s.pending_file().string());
  }
  for (const auto& p : crash) s.set_aside(p);
  if (crash.empty()) return;
  std::cerr << "Archived " << crash.size() << " abandoned private file(s) to " << s.quarantine.string()
            << "; nothing was deleted" << std::endl;
  if (s.sync)
  {
    fsync_dir(s.quarantine);
    for (const auto& d : dirs) fsync_dir(d);
  }
}

void RunLedger::publish(const fs::path& path, const char* data, size_t size)
{
  State& s = *st_;
  if (!s.begun) throw std::logic_error("output ledger has not begun");
  const fs::path full = resolve_parent(path);
  const auto it = s.outputs.find(full);
  if (it == s.outputs.end()) throw std::runtime_error("not an output of this run: " + full.string());
  const LedgerOutput& o = it->second;
  const bool rows_ok = o.record_bytes ? size == o.rows * o.record_bytes
                                      : (uint64_t)std::count(data, data + size, '\n') == o.rows + 1;
  if (!rows_ok)
    throw std::runtime_error(o.record_bytes ? "serialized raw row count mismatch" : "serialized CSV row count mismatch");
  Json intent = Json::object();
  intent["schema_version"] = 1;
  intent["key"] = o.key;
  intent["rows"] = (unsigned long long)o.rows;
  intent["algorithm"] = kDigestName;
  intent["bytes"] = (unsigned long long)size;
  intent["digest"] = content_digest(data, size);
  // recorded_intents is read-only after construction
  const auto known = s.recorded_intents.find(o.key);
  if (known != s.recorded_intents.end())
  {
    if (known->second != intent) throw std::runtime_error("replayed bytes differ from recorded output: " + full.string());
    std::lock_guard<std::mutex> g(s.m);
    if (s.committed.count(o.key)) return;   // already on disk as recorded: left untouched
  }
  if (present(full)) throw std::runtime_error("output appeared while run was active: " + full.string());
  // the intent first: a crash between the two leaves a replayable record
  publish_json(intent_path_for(s.state_dir, o.key), intent, s.sync);
  publish_file(full, data, size, false, s.sync);
  std::lock_guard<std::mutex> g(s.m);
  s.promote_pending();
  s.committed.insert(o.key);
}

void RunLedger::finish()
{
  State& s = *st_;
  std::lock_guard<std::mutex> g(s.m);
  if (s.committed.size() != s.outputs.size()) throw std::runtime_error("run has uncommitted output files");
  s.promote_pending();
  Json metadata = Json::object();
  for (const auto& p : s.manifests) metadata[p.filename().string()] = digest_of(read_json_file(p));
  if (!s.sync)
  {
    // one durability barrier per finished run: the ledger and the manifests reach the disk,
    // payloads are covered by their digests
    for (const auto& p : s.manifests) fsync_file(p);
    fsync_file(s.contract_file());
    fsync_dir(s.root);
    for (const auto& d : s.side_dirs) fsync_dir(d);
  }
  Json rec = Json::object();
  rec["schema_version"] = 1;
  rec["contract_digest"] = s.digest;
  rec["durability"] = durability_name(s.sync ? Durability::Fsync : Durability::Rename);
  rec["metadata"] = metadata;
  publish_json(s.state_dir / "complete.json", rec, true);   // always durable
  s.complete = true;
}

// ------------------------------------------------------------------ --verify-only
namespace
{

// The report's summary of the recorded contract.
Json contract_summary(const Json& contract, const std::string& digest)
{
  Json sum = Json::object();
  sum["digest"] = digest;
  sum["options"] = contract.at("options");
  for (const char* k : {"schema_version", "git_hash", "build_date"})
    if (contract.has(k)) sum[k] = contract.at(k);
  if (contract.has("binary") && contract.at("binary").is_object() && contract.at("binary").has("digest"))
    sum["binary_digest"] = contract.at("binary").at("digest");
  if (contract.has("reference") && contract.at("reference").is_object() && contract.at("reference").has("path"))
    sum["reference"] = contract.at("reference").at("path");
  Json legacy = Json::array();
  for (const auto& k : kSchedulingOptions)
    if (contract.at("options").has(k)) legacy.push(k);
  sum["legacy_scheduling_options"] = legacy;
  return sum;
}

// Input images named in the contract against their recorded fingerprints.
Json audit_inputs(const Json& contract, ReportLists& lists)
{
  std::map<std::string, Json> inputs;
  const auto collect = [&](const Json& d) {
    if (d.is_object() && d.has("path") && d.at("path").is_string() && d.has("content") && d.at("content").is_object())
      inputs.emplace(d.at("path").as_string(), d.at("content"));
  };
  if (contract.has("reference")) collect(contract.at("reference"));
  for (const auto& t : contract.at("targets").items())
    if (t.is_object() && t.has("input")) collect(t.at("input"));
  size_t checked = 0;
  for (const auto& [path, want] : inputs)
  {
    std::error_code ec;
    if (!fs::is_regular_file(fs::path(path), ec))
    {
      lists.add("in_missing", path);
      continue;
    }
    ++checked;
    const Json seen = file_fingerprint(path);
    if (!want.has("bytes") || !want.has("digest") || seen.at("bytes") != want.at("bytes") ||
        seen.at("digest") != want.at("digest"))
      lists.add("in_changed", path);
  }
  Json r = Json::object();
  r["checked"] = (unsigned long long)checked;
  r["status"] = lists.count("in_changed") ? "changed" : lists.count("in_missing") ? "missing" : "match";
  Json tmp = Json::object();
  lists.store(tmp, "in_changed");
  lists.store(tmp, "in_missing");
  r["changed"] = tmp.at("in_changed");
  r["changed_count"] = tmp.at("in_changed_count");
  r["missing"] = tmp.at("in_missing");
  r["missing_count"] = tmp.at("in_missing_count");
  return r;
}

}  // namespace

Json audit_run_directory(const fs::path& requested, const AuditLayoutFn& layout_fn)
{
  Json report = Json::object();
  Json problems = Json::array(), warnings = Json::array();
  const fs::path root = absolute_clean(requested);
  report["output_dir"] = root.string();
  const auto verdict = [&](const char* status) {
    report["status"] = status;
    report["complete"] = std::string(status) == "complete";
    report["problems"] = problems;
    report["warnings"] = warnings;
    return report;
  };
  if (!fs::exists(root))
  {
    problems.push("the output directory does not exist");
    return verdict("not_found");
  }
  if (!fs::is_directory(root))
  {
    problems.push("the path is not a directory");
    return verdict("not_a_run");
  }
  // a shared lock: audits run together; a run (exclusive) is either seen whole or refused
  Handle lock = open_dir(root, "open run directory");
  if (::flock(lock.get(), LOCK_SH | LOCK_NB) != 0)
  {
    if (errno != EWOULDBLOCK) fail_io("lock run directory", root);
    problems.push("a run holds this directory's lock right now; verify again when it has finished");
    return verdict("locked");
  }
  const fs::path state = root / ".opencorr-state";
  if (fs::is_symlink(fs::symlink_status(state)))
  {
    problems.push("the run state .opencorr-state is a symlink");
    return verdict("damaged");
  }
  if (!present(state / "contract.json"))
  {
    problems.push("no .opencorr-state/contract.json: not a ledgered multi-frame output directory "
                  "(single-frame output and binaries older than the output ledger write none)");
    return verdict("not_a_run");
  }
  Json contract;
  AuditLayout layout;
  try
  {
    contract = read_json_file(state / "contract.json");
    if (!contract_shape(contract)) throw std::runtime_error("unexpected contract layout");
    layout = layout_fn(contract, root);
  }
  catch (const std::system_error&)
  {
    throw;
  }
  catch (const std::exception& ex)
  {
    problems.push(std::string("contract.json is not a usable run contract: ") + ex.what());
    return verdict("damaged");
  }
  const std::string digest = digest_of(contract);
  report["contract"] = contract_summary(contract, digest);

  // ---- the judgement table over the promised outputs
  ReportLists lists;
  bool damaged = false, incomplete = false;
  size_t frames_expected = 0, frames_verified = 0, files_verified = 0;
  uint64_t bytes_verified = 0;
  std::set<uint64_t> rows_seen;
  std::set<fs::path> owned{state}, dirs{root}, promised;
  std::map<fs::path, std::set<std::string>> extensions;   // per directory, its outputs' extensions
  const auto adopt = [&](const fs::path& p) {
    if (auto d = own(owned, p, root)) dirs.insert(*d);
  };
  const auto file_under = [&](Judged s, const std::string& name) {
    lists.add(audit_list(s), name);
    if (s == Judged::Missing) incomplete = true;   // the next run replays it
    else damaged = true;
  };
  for (const auto& o : layout.outputs)
  {
    adopt(o.path);
    promised.insert(o.path);
    extensions[o.path.parent_path()].insert(o.path.extension().string());
    frames_expected += o.frame;
    const Judgement j = judge(state, o.key, o.path, o.record_bytes, std::nullopt);
    if (j.state != Judged::Verified)
    {
      file_under(j.state, relative_name(o.path, root));
      continue;
    }
    ++files_verified;
    bytes_verified += j.bytes;
    if (o.frame)
    {
      ++frames_verified;
      rows_seen.insert(j.rows);
    }
  }

  // ---- an append in progress: its outputs count when the longer list would accept them
  const fs::path pending_path = state / "contract.pending.json";
  const bool pending = present(pending_path);
  std::string pending_state = "none";
  size_t appended_damaged = 0;
  if (pending)
  {
    try
    {
      const Json longer = read_json_file(pending_path);
      if (!contract_shape(longer)) throw std::runtime_error("unexpected contract layout");
      if (resume_view(longer) != resume_view(contract) || !is_prefix(contract.at("targets"), longer.at("targets")))
        pending_state = "unrelated";
      else if (contract.at("targets").size() == longer.at("targets").size())
        pending_state = "promoted";
      else
      {
        pending_state = "append";
        for (const auto& o : layout_fn(longer, root).outputs)
        {
          if (promised.count(o.path)) continue;
          const Judgement j = judge(state, o.key, o.path, o.record_bytes, std::nullopt);
          if (j.state == Judged::Missing) continue;
          adopt(o.path);
          const std::string name = relative_name(o.path, root);
          if (j.state != Judged::Verified)
          {
            file_under(j.state, name);
            ++appended_damaged;
            continue;
          }
          lists.add("appended_published", name);
          if (o.frame) rows_seen.insert(j.rows);
        }
      }
    }
    catch (const std::system_error&)
    {
      throw;
    }
    catch (const std::exception&)
    {
      pending_state = "unreadable";
    }
  }
  if (lists.count("appended_published"))
  {
    problems.push("an append was interrupted after it published its first new output and before its longer target "
                  "list replaced the recorded one: rerun the append command (the longer --tar-list) unchanged to "
                  "continue, no --repair needed; the shorter list is no longer accepted, because it does not account "
                  "for the appended output");
    incomplete = true;
  }
  if (appended_damaged)
    problems.push("an interrupted append left an output that contradicts its ledger record; rerunning the append "
                  "command (the longer --tar-list) with --repair regenerates it");
  if (rows_seen.size() > 1)
  {
    problems.push("frames record different row counts; one run writes the same rows for every frame");
    damaged = true;
  }

  // ---- completion record
  const Completion c = read_completion(state, digest);
  Json completion = Json::object();
  completion["present"] = c.present;
  completion["state"] = !c.present ? "missing" : !c.valid ? "invalid" : c.current ? "current" : "other_contract";
  if (c.valid && c.record.has("durability")) completion["durability"] = c.record.at("durability");
  if (!c.present)
  {
    problems.push("no complete.json: the run has not finished");
    incomplete = true;
  }
  else if (!c.valid)
  {
    problems.push("complete.json is damaged: " + c.error);
    damaged = true;
  }
  else if (!c.current)
  {
    problems.push("complete.json belongs to another target list or contract (an append or resume was started and did "
                  "not finish)");
    incomplete = true;
  }
  report["completion"] = completion;

  // ---- manifests
  Json manifest_rows = Json::array();
  for (const auto& p : layout.manifests)
  {
    adopt(p);
    const std::string name = relative_name(p, root);
    Json row = Json::object();
    row["file"] = name;
    std::string st = "ok";
    if (!present(p))
    {
      st = "missing";
      incomplete = true;
      if (c.current) problems.push("manifest missing: " + name);
    }
    else
      try
      {
        need_plain_file(p);
        const std::string d = digest_of(read_json_file(p));
        ++files_verified;
        bytes_verified += fs::file_size(p);
        if (c.current)
        {
          const Json& md = c.record.at("metadata");
          const std::string key = p.filename().string();
          if (!md.has(key) || !md.at(key).is_string() || md.at(key).as_string() != d)
          {
            st = "changed";
            problems.push("manifest differs from the one the completion record digested: " + name);
            damaged = true;
          }
        }
      }
      catch (const std::system_error&)
      {
        throw;
      }
      catch (const std::exception& ex)
      {
        st = "invalid";
        problems.push("manifest does not parse: " + name + ": " + ex.what());
        damaged = true;
      }
    row["state"] = st;
    manifest_rows.push(row);
  }
  report["manifests"] = manifest_rows;

  // ---- one scan of the directories the run owns
  std::vector<fs::path> scan_dirs(dirs.begin(), dirs.end());
  for (const auto& e : scan_owned(scan_dirs, owned))
  {
    const std::string name = relative_name(e.path, root);
    if (e.kind == Entry::Crash || e.kind == Entry::OddReserved) lists.add("residue", name);
    else if (e.kind == Entry::Foreign)
    {
      // named like this directory's outputs: a reader globbing for frames would take it
      const auto ext = extensions.find(e.dir);
      const bool output_like = ext != extensions.end() && ext->second.count(e.path.extension().string());
      lists.add(output_like ? "untracked_outputs" : "untracked", name);
    }
  }
  if (fs::is_directory(state))
    for (const auto& e : fs::directory_iterator(state))
      if (temp_kind(e.path()) != Temp::None) lists.add("residue", relative_name(e.path(), root));
  if (lists.count("untracked_outputs"))
  {
    problems.push("entries named like this run's outputs (same directory, same extension) that the ledger does not list");
    damaged = true;
  }
  if (lists.count("residue"))
    warnings.push("temporary files of an interrupted run; the next run archives them under .opencorr-state/quarantine/");
  static const std::map<std::string, const char*> kPendingNotes = {
      {"promoted", "contract.pending.json repeats the recorded contract: an append was promoted and only this file is "
                   "left over; the next run archives it"},
      {"unrelated", "contract.pending.json does not extend the recorded contract (other binary, reference, options or "
                    "target prefix), so it says nothing about this directory; the next run archives it"},
      {"unreadable", "contract.pending.json cannot be read as a contract, so it says nothing about an interrupted append; "
                     "the next run archives it"}};
  if (pending_state == "append" && !lists.count("appended_published") && !appended_damaged)
    warnings.push("contract.pending.json: an append was started and stopped before any appended output was published; "
                  "the recorded target list is still the valid one");
  else if (kPendingNotes.count(pending_state))
    warnings.push(kPendingNotes.at(pending_state));
  static const std::pair<const char*, const char*> kListProblems[] = {
      {"missing", "frames or diagnostics files the contract promises are missing"},
      {"mismatched", "files whose bytes do not match their ledger record (or that are not regular files)"},
      {"no_intent", "files with no ledger record"},
      {"invalid_intent", "ledger records that do not parse or do not describe their file"}};
  for (const auto& [list, text] : kListProblems)
    if (lists.count(list)) problems.push(text);

  // ---- inputs
  report["inputs"] = audit_inputs(contract, lists);
  if (lists.count("in_changed"))
    problems.push("input images no longer match the fingerprints in the contract; the outputs still match their ledger, "
                  "but they describe images that are no longer at those paths");
  if (lists.count("in_missing"))
    warnings.push("input images are not at the recorded paths, so they were not compared; rerunning the command needs "
                  "them there");

  report["frames_expected"] = (unsigned long long)frames_expected;
  report["frames_verified"] = (unsigned long long)frames_verified;
  report["files_expected"] = (unsigned long long)(layout.outputs.size() + layout.manifests.size());
  report["files_verified"] = (unsigned long long)files_verified;
  report["bytes_verified"] = (unsigned long long)bytes_verified;
  if (rows_seen.size() == 1) report["rows_per_frame"] = (unsigned long long)*rows_seen.begin();
  for (const char* l : {"missing", "mismatched", "no_intent", "invalid_intent", "untracked_outputs", "untracked", "residue"})
    lists.store(report, l);
  report["pending_append"] = pending;
  report["pending_append_state"] = pending_state;
  lists.store(report, "appended_published");
  if (damaged) return verdict("damaged");
  if (incomplete) return verdict("incomplete");
  if (lists.count("in_changed")) return verdict("inputs_changed");
  return verdict("complete");
}

}  // namespace dic_cli
