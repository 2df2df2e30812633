// Output ledger (see ledger.h).  Reference behaviour: src/cli_output_integrity.cpp
// (publication :293-313, fingerprints :363-382, metadata reads :384-410, the session
// :434-835, the audit :855-1266) and docs/output-integrity.md.
#include "ledger.h"

#include "xxh3.h"

#include <algorithm>
#include <atomic>
#include <cerrno>
#include <cstdio>
#include <cstring>
#include <ctime>
#include <fstream>
#include <iostream>
#include <map>
#include <mutex>
#include <set>
#include <sstream>
#include <system_error>

#include <fcntl.h>
#include <sys/file.h>
#include <unistd.h>

namespace dic_cli
{
namespace
{

constexpr const char* kAlgorithm = "xxh3-128";
constexpr const char* kRepairHint = " (use --repair to quarantine and regenerate it)";
constexpr const char* kTmpPrefix = ".opencorr-tmp-";
// scheduling options older contracts listed; they never decide an output byte
const char* const kLegacyScheduling[4] = {"gpu_device", "threads", "preload", "decode_threads"};

std::atomic<void (*)(const std::string&)> g_warning_sink{nullptr};
std::atomic<unsigned long long> g_tmp_sequence{0};

void warn(const std::string& text)
{
  std::cerr << "Warning: " << text << std::endl;
  if (auto sink = g_warning_sink.load()) sink(text);
}

[[noreturn]] void io_fail(const std::string& what, const fs::path& path)
{
  const int e = errno ? errno : EIO;
  throw std::system_error(e, std::generic_category(), what + ": " + path.string());
}

struct Fd
{
  int fd = -1;
  ~Fd()
  {
    if (fd >= 0) ::close(fd);
  }
};

fs::path canonical_path(const fs::path& p) { return fs::weakly_canonical(fs::absolute(p)); }

bool regular_not_link(const fs::path& p)
{
  return !fs::is_symlink(fs::symlink_status(p)) && fs::is_regular_file(p);
}
void require_regular(const fs::path& p)
{
  if (!regular_not_link(p)) throw std::runtime_error("expected a regular, non-symlink output file: " + p.string());
}
bool exists_no_follow(const fs::path& p) { return fs::exists(fs::symlink_status(p)); }

void sync_directory(const fs::path& dir)
{
  Fd d;
  d.fd = ::open(dir.c_str(), O_RDONLY | O_DIRECTORY | O_CLOEXEC);
  if (d.fd < 0) io_fail("open output directory", dir);
  if (::fsync(d.fd) != 0) io_fail("sync output directory", dir);
}
void sync_file(const fs::path& p)
{
  Fd f;
  f.fd = ::open(p.c_str(), O_WRONLY | O_CLOEXEC | O_NOFOLLOW);
  if (f.fd < 0) io_fail("open published output", p);
  if (::fsync(f.fd) != 0) io_fail("sync published output", p);
}

// What the reserved temporary namespace holds: not ours (foreign), ours but malformed,
// ours but not a regular file, or a crash temporary that may be archived.
enum class Residue { Foreign, Unrecognized, NotRegular, Reclaimable };
Residue classify(const fs::path& p)
{
  const std::string name = p.filename().string();
  if (name.rfind(kTmpPrefix, 0) != 0) return Residue::Foreign;
  const std::string rest = name.substr(std::strlen(kTmpPrefix));
  const size_t dash = rest.find('-');
  const auto digits = [](const std::string& s) { return !s.empty() && s.find_first_not_of("0123456789") == std::string::npos; };
  if (dash == std::string::npos || !digits(rest.substr(0, dash)) || !digits(rest.substr(dash + 1)))
    return Residue::Unrecognized;
  return regular_not_link(p) ? Residue::Reclaimable : Residue::NotRegular;
}
void report_skipped(Residue r, const fs::path& p)
{
  if (r == Residue::NotRegular) warn("leaving reserved name in place, not a regular file: " + p.string());
  else if (r == Residue::Unrecognized) warn("leaving unrecognized reserved name in place: " + p.string());
}

// an integrity record: {"algorithm": "xxh3-128", "bytes": unsigned, "digest": 32 hex}
void require_record(const Json& r)
{
  if (!r.is_object() || r.str_or("algorithm", "") != kAlgorithm || !r.has("bytes") || !r.at("bytes").is_unsigned() ||
      !r.has("digest") || !r.at("digest").is_string())
    throw std::runtime_error("invalid integrity record schema");
  const std::string& d = r.at("digest").as_string();
  if (d.size() != 32 || d.find_first_not_of("0123456789abcdef") != std::string::npos)
    throw std::runtime_error("invalid integrity digest");
}
bool is_hex32(const std::string& d)
{
  return d.size() == 32 && d.find_first_not_of("0123456789abcdef") == std::string::npos;
}

// the contract as a resume compares it: without the target list (compared as a prefix)
// and without the old scheduling options
Json comparable(Json c)
{
  if (!c.is_object()) return c;
  c.erase("targets");
  if (c.has("options") && c.at("options").is_object())
    for (const char* k : kLegacyScheduling) c["options"].erase(k);
  return c;
}

// one JSON leaf for a message; floats at seven significant digits (the contract's floats
// were single precision when typed)
std::string leaf_text(const Json& v)
{
  if (v.kind() == Json::Kind::Float)
  {
    char b[32];
    std::snprintf(b, sizeof b, "%.7g", v.as_double());
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
void flatten(const Json& v, const std::string& prefix, std::map<std::string, std::string>& out)
{
  if (v.is_object() && v.size() > 0)
  {
    for (const auto& m : v.members()) flatten(m.second, prefix.empty() ? m.first : prefix + "." + m.first, out);
  }
  else
    out[prefix] = leaf_text(v);
}
std::vector<std::string> changed_keys(const Json& a, const Json& b)
{
  std::map<std::string, std::string> la, lb;
  flatten(a, "", la);
  flatten(b, "", lb);
  std::set<std::string> keys;
  for (const auto& l : la) keys.insert(l.first);
  for (const auto& l : lb) keys.insert(l.first);
  std::vector<std::string> out;
  for (const auto& k : keys)
  {
    const auto x = la.find(k), y = lb.find(k);
    if (x == la.end() || y == lb.end() || x->second != y->second) out.push_back(k);
  }
  return out;
}

std::string contract_change(const Json& recorded, const Json& requested)
{
  bool binary = false, reference = false, options = false;
  for (const auto& k : changed_keys(recorded, requested))
  {
    if (k.rfind("binary.", 0) == 0 || k == "git_hash" || k == "build_date") binary = true;
    else if (k.rfind("reference.", 0) == 0) reference = true;
    else if (k.rfind("options.", 0) == 0) options = true;
  }
  std::string hint;
  if (options) hint += "; an option that decides the output differs from the recorded run";
  if (reference) hint += "; the reference image path or content differs";
  if (binary) hint += "; another build of the executable wrote this directory (resume needs the byte-identical binary)";
  return " (recorded -> requested): " + describe_differences(recorded, requested) + hint +
         "; use a new output directory for a different run";
}

std::string target_change(const Json& recorded, const Json& requested)
{
  if (!recorded.is_array() || !requested.is_array()) return std::string();
  const size_t common = std::min(recorded.size(), requested.size());
  for (size_t i = 0; i < common; ++i)
    if (recorded.at(i) != requested.at(i))
      return ": target " + std::to_string(i + 1) + " of the recorded " + std::to_string(recorded.size()) +
             " differs (recorded -> requested): " + describe_differences(recorded.at(i), requested.at(i), 4);
  if (requested.size() < recorded.size())
    return ": the recorded run lists " + std::to_string(recorded.size()) + " targets, this command only " +
           std::to_string(requested.size()) + " (a shorter list is not a resume)";
  return std::string();
}

bool targets_extend(const Json& recorded, const Json& requested)
{
  if (!recorded.is_array() || !requested.is_array() || recorded.size() > requested.size()) return false;
  for (size_t i = 0; i < recorded.size(); ++i)
    if (recorded.at(i) != requested.at(i)) return false;
  return true;
}

std::string doc_digest(const Json& doc)
{
  const std::string s = doc.dump();
  return content_digest(s.data(), s.size());
}

// up to 20 names with the exact total, for the audit report
struct NameList
{
  size_t count = 0;
  Json names = Json::array();
  void add(const std::string& n)
  {
    if (count++ < 20) names.push(n);
  }
  void store(Json& report, const std::string& key) const
  {
    report[key] = names;
    report[key + "_count"] = (unsigned long long)count;
  }
};

std::string rel_name(const fs::path& p, const fs::path& root)
{
  const fs::path r = p.lexically_relative(root);
  return (!r.empty() && *r.begin() != "..") ? r.string() : p.string();
}

}  // namespace

// ------------------------------------------------------------------ primitives
const char* durability_name(Durability d) { return d == Durability::Fsync ? "fsync" : "rename"; }

void set_warning_sink(void (*sink)(const std::string&)) { g_warning_sink.store(sink); }

std::string content_digest(const void* data, size_t size) { return hex128(xxh3_128(data, size)); }

Json file_fingerprint(const fs::path& path)
{
  Fd f;
  f.fd = ::open(path.c_str(), O_RDONLY | O_CLOEXEC);
  if (f.fd < 0) io_fail("cannot read fingerprint input", path);
  Xxh3Stream h;
  std::vector<unsigned char> buf(1 << 20);
  unsigned long long bytes = 0;
  for (;;)
  {
    const ssize_t r = ::read(f.fd, buf.data(), buf.size());
    if (r < 0)
    {
      if (errno == EINTR) continue;
      io_fail("fingerprint read failed", path);
    }
    if (r == 0) break;
    h.update(buf.data(), (size_t)r);
    bytes += (unsigned long long)r;
  }
  Json j = Json::object();
  j["algorithm"] = kAlgorithm;
  j["bytes"] = bytes;
  j["digest"] = hex128(h.digest());
  return j;
}

Json read_json_file(const fs::path& path)
{
  if (!exists_no_follow(path))
  {
    errno = ENOENT;
    io_fail("open JSON metadata", path);
  }
  require_regular(path);
  if (fs::file_size(path) > 256ull * 1024 * 1024) throw std::runtime_error("JSON metadata exceeds 256 MiB: " + path.string());
  Fd f;
  f.fd = ::open(path.c_str(), O_RDONLY | O_CLOEXEC | O_NOFOLLOW);
  if (f.fd < 0) io_fail("open JSON metadata", path);
  std::string text;
  char buf[65536];
  for (;;)
  {
    const ssize_t r = ::read(f.fd, buf, sizeof buf);
    if (r < 0)
    {
      if (errno == EINTR) continue;
      io_fail("read JSON metadata", path);
    }
    if (r == 0) break;
    text.append(buf, (size_t)r);
  }
  return Json::parse(text, path.string());
}

void publish_file(const fs::path& path, const char* data, size_t size, bool replace, bool sync)
{
  if (fs::is_symlink(fs::symlink_status(path))) throw std::runtime_error("refusing symlink output: " + path.string());
  const fs::path dir = path.parent_path().empty() ? fs::path(".") : path.parent_path();
  Fd f;
  fs::path tmp;
  for (int attempt = 0; attempt < 1024 && f.fd < 0; ++attempt)
  {
    tmp = dir / (std::string(kTmpPrefix) + std::to_string(::getpid()) + "-" + std::to_string(g_tmp_sequence++));
    f.fd = ::open(tmp.c_str(), O_WRONLY | O_CREAT | O_EXCL | O_CLOEXEC, 0666);
    if (f.fd < 0 && errno != EEXIST) io_fail("create temporary output", tmp);
  }
  if (f.fd < 0) io_fail("allocate temporary output", path);
  try
  {
    size_t off = 0;
    while (off < size)
    {
      const ssize_t w = ::write(f.fd, data + off, std::min(size - off, (size_t)1 << 30));
      if (w < 0 && errno == EINTR) continue;
      if (w <= 0)
      {
        if (w == 0) errno = EIO;
        io_fail("write temporary output", tmp);
      }
      off += (size_t)w;
    }
    if (sync && ::fsync(f.fd) != 0) io_fail("sync temporary output", tmp);
    const int fd = f.fd;
    f.fd = -1;
    if (::close(fd) != 0) io_fail("close temporary output", tmp);
    if (replace)
    {
      if (::rename(tmp.c_str(), path.c_str()) != 0) io_fail("publish output", path);
    }
    else
    {
      // a hard link publishes the finished inode without replacing anything that appeared
      if (::link(tmp.c_str(), path.c_str()) != 0) io_fail("publish new output", path);
      ::unlink(tmp.c_str());
    }
    if (sync) sync_directory(dir);
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
  const std::string bytes = value.dump_indented(2) + "\n";
  publish_file(path, bytes.data(), bytes.size(), true, sync);
}

std::string describe_differences(const Json& recorded, const Json& requested, size_t limit)
{
  std::map<std::string, std::string> a, b;
  flatten(recorded, "", a);
  flatten(requested, "", b);
  const auto keys = changed_keys(recorded, requested);
  std::string out;
  for (size_t i = 0; i < keys.size() && i < limit; ++i)
  {
    const auto x = a.find(keys[i]), y = b.find(keys[i]);
    if (i) out += "; ";
    out += (keys[i].empty() ? std::string("(value)") : keys[i]) + ": " + (x == a.end() ? "(absent)" : x->second) +
           " -> " + (y == b.end() ? "(absent)" : y->second);
  }
  if (keys.size() > limit) out += "; and " + std::to_string(keys.size() - limit) + " more";
  return out;
}

// ------------------------------------------------------------------ the run record
struct RunLedger::State
{
  Fd lock;
  std::vector<std::unique_ptr<Fd>> extra_locks;
  fs::path root, state, quarantine;
  std::vector<fs::path> extra_dirs;
  Json contract;
  std::string contract_digest;
  std::map<fs::path, LedgerOutput> outputs;
  std::map<std::string, Json> intents;
  std::set<std::string> committed;
  std::vector<fs::path> manifests;
  std::mutex m;
  size_t existing = 0, verified = 0, moved = 0;
  uint64_t verified_bytes = 0;
  bool done = false, begun = false, dirty = false, prior = false, pending = false, sync = false, repair = false;

  fs::path intent_path(const std::string& key) const { return state / (content_digest(key.data(), key.size()) + ".json"); }
  fs::path contract_path() const { return state / "contract.json"; }
  fs::path pending_path() const { return state / "contract.pending.json"; }
  fs::path quarantine_dir()
  {
    if (!quarantine.empty()) return quarantine;
    const std::time_t now = std::time(nullptr);
    std::tm t{};
    ::gmtime_r(&now, &t);
    char stamp[32];
    std::strftime(stamp, sizeof stamp, "%Y%m%dT%H%M%SZ", &t);
    quarantine = state / "quarantine" / (std::string(stamp) + "-" + std::to_string(::getpid()));
    fs::create_directories(quarantine);
    return quarantine;
  }
  // moved aside, never deleted
  void set_aside(const fs::path& p)
  {
    const fs::path dir = quarantine_dir();
    fs::path dst = dir / p.filename();
    for (int k = 1; exists_no_follow(dst); ++k) dst = dir / (p.filename().string() + "." + std::to_string(k));
    std::error_code ec;
    fs::rename(p, dst, ec);
    if (ec)
    {
      // another file system (a diagnostics directory elsewhere)
      fs::copy_file(p, dst, fs::copy_options::overwrite_existing);
      fs::remove(p);
    }
    ++moved;
  }
  void promote()
  {
    if (!pending) return;
    publish_json(contract_path(), contract, sync);
    std::error_code ignored;
    fs::remove(pending_path(), ignored);
    pending = false;
  }
};

RunLedger::RunLedger(const fs::path& root_in, Json contract, std::vector<LedgerOutput> outputs,
                     std::vector<fs::path> manifests, const fs::path& tar_list, Durability durability, bool repair)
    : st_(std::make_unique<State>())
{
  State& s = *st_;
  s.sync = durability == Durability::Fsync;
  s.repair = repair;
  s.root = canonical_path(root_in);
  s.state = s.root / ".opencorr-state";
  s.contract = std::move(contract);
  s.contract_digest = doc_digest(s.contract);
  s.lock.fd = ::open(s.root.c_str(), O_RDONLY | O_DIRECTORY | O_CLOEXEC);
  if (s.lock.fd < 0) io_fail("open run directory", s.root);
  if (::flock(s.lock.fd, LOCK_EX | LOCK_NB) != 0) io_fail("run directory already locked", s.root);
  if (fs::is_symlink(fs::symlink_status(s.state))) throw std::runtime_error("run state must not be a symlink");

  std::set<fs::path> allowed{s.state, canonical_path(tar_list)};
  std::set<fs::path> extra;
  const auto allow = [&](const fs::path& p) {
    allowed.insert(p);
    const fs::path r = p.lexically_relative(s.root);
    if (!r.empty() && *r.begin() != "..") allowed.insert(s.root / *r.begin());
    if (p.parent_path() != s.root) extra.insert(p.parent_path());
  };
  for (auto& o : outputs)
  {
    // the final component is kept as given, so a symlinked output is rejected, not followed
    o.path = canonical_path(o.path.parent_path()) / o.path.filename();
    if (o.path == s.state || o.path.filename().string().rfind(".opencorr-", 0) == 0)
      throw std::runtime_error("reserved output filename: " + o.path.string());
    if (!s.outputs.emplace(o.path, o).second) throw std::runtime_error("duplicate output destination: " + o.path.string());
    allow(o.path);
  }
  for (auto& p : manifests)
  {
    p = canonical_path(p.parent_path()) / p.filename();
    if (s.outputs.count(p)) throw std::runtime_error("data output collides with manifest: " + p.string());
    allow(p);
    s.manifests.push_back(p);
  }

  const bool prior = exists_no_follow(s.contract_path());
  Json recorded;
  if (prior)
  {
    recorded = read_json_file(s.contract_path());
    const Json before = comparable(recorded), after = comparable(s.contract);
    if (before != after)
      throw std::runtime_error("resume rejected: run configuration/reference/binary changed" + contract_change(before, after));
    const Json& old_t = recorded.has("targets") ? recorded.at("targets") : Json();
    if (!targets_extend(old_t, s.contract.at("targets")))
      throw std::runtime_error("resume rejected: targets changed/reordered; only an identical prefix plus append is allowed" +
                               target_change(old_t, s.contract.at("targets")));
  }
  const bool repairing = s.repair && prior;
  for (const auto& dir : extra)
  {
    fs::create_directories(dir);
    auto l = std::make_unique<Fd>();
    l->fd = ::open(dir.c_str(), O_RDONLY | O_DIRECTORY | O_CLOEXEC);
    if (l->fd < 0) io_fail("open diagnostics directory", dir);
    if (::flock(l->fd, LOCK_EX | LOCK_NB) != 0) io_fail("diagnostics directory already locked", dir);
    s.extra_locks.push_back(std::move(l));
    s.extra_dirs.push_back(dir);
  }
  // a dedicated directory: anything the run does not own is refused (crash temporaries
  // are recognised here and archived later by archive_residue)
  const auto check_dir = [&](const fs::path& dir) {
    for (const auto& e : fs::directory_iterator(dir))
      if (classify(e.path()) == Residue::Foreign && !allowed.count(e.path()))
        throw std::runtime_error("untracked entry in output directory: " + e.path().string());
  };
  check_dir(s.root);
  for (const auto& d : s.extra_dirs) check_dir(d);
  if (!prior)
  {
    for (const auto& o : s.outputs)
      if (exists_no_follow(o.first)) throw std::runtime_error("existing output has no verified run record: " + o.first.string());
    for (const auto& p : s.manifests)
      if (exists_no_follow(p)) throw std::runtime_error("existing manifest has no verified run record: " + p.string());
    if (fs::exists(s.state))
      for (const auto& e : fs::directory_iterator(s.state))
        if (classify(e.path()) == Residue::Foreign) throw std::runtime_error("run state has no valid contract: " + s.state.string());
  }

  for (const auto& item : s.outputs)
  {
    const LedgerOutput& o = item.second;
    const fs::path ip = s.intent_path(o.key);
    bool has_intent = fs::exists(ip);
    if (has_intent)
    {
      try
      {
        const Json intent = read_json_file(ip);
        require_record(intent);
        if (intent.u64_or("schema_version", 0) != 1 || intent.str_or("key", "") != o.key || !intent.has("rows") ||
            !intent.at("rows").is_unsigned() || intent.at("rows").as_u64() != o.rows)
          throw std::runtime_error("invalid output intent: " + ip.string());
        if (o.record_bytes && intent.at("bytes").as_u64() != o.rows * o.record_bytes)
          throw std::runtime_error("raw record size mismatch in intent: " + o.path.string());
        s.intents.emplace(o.key, intent);
      }
      catch (const std::system_error&)
      {
        throw;   // an I/O fault is not a damaged record
      }
      catch (const std::exception& ex)
      {
        if (!repairing) throw std::runtime_error(std::string(ex.what()) + kRepairHint);
        s.set_aside(ip);
        has_intent = false;
      }
    }
    if (exists_no_follow(o.path))
    {
      require_regular(o.path);   // a symlinked output stays a hard rejection, with --repair too
      bool intact = has_intent;
      Json seen;
      if (intact)
      {
        seen = file_fingerprint(o.path);
        const Json& want = s.intents.at(o.key);
        intact = seen.at("bytes") == want.at("bytes") && seen.at("digest") == want.at("digest");
      }
      if (!intact)
      {
        if (!repairing)
          throw std::runtime_error(std::string(has_intent ? "corrupt/truncated output; resume refused: "
                                                          : "existing output has no commit intent: ") +
                                   o.path.string() + kRepairHint);
        s.set_aside(o.path);
      }
      else
      {
        s.committed.insert(o.key);
        s.verified_bytes += seen.at("bytes").as_u64();
        ++s.verified;
        ++s.existing;
      }
    }
  }
  for (const auto& p : s.manifests)
  {
    if (!fs::exists(p)) continue;
    require_regular(p);
    try
    {
      (void)read_json_file(p);
      s.verified_bytes += fs::file_size(p);
      ++s.verified;
    }
    catch (const std::system_error&)
    {
      throw;
    }
    catch (const std::exception&)
    {
      if (!repairing) throw;
      s.set_aside(p);
    }
  }
  const fs::path cp = s.state / "complete.json";
  if (prior && fs::exists(cp))
  {
    require_regular(cp);
    std::string reason;
    fs::path bad_manifest;
    try
    {
      const Json c = read_json_file(cp);
      if (!c.is_object() || c.u64_or("schema_version", 0) != 1 || !c.has("contract_digest") ||
          !c.at("contract_digest").is_string() || !c.has("metadata") || !c.at("metadata").is_object())
        throw std::runtime_error("invalid run completion record");
      if (!is_hex32(c.at("contract_digest").as_string())) throw std::runtime_error("invalid completion contract digest");
      const bool ours = c.at("contract_digest").as_string() == s.contract_digest;
      if (ours)
      {
        const Json& md = c.at("metadata");
        if (md.size() != s.manifests.size()) throw std::runtime_error("invalid metadata completion record");
        for (const auto& p : s.manifests)
        {
          const std::string key = p.filename().string();
          if (!md.has(key) || !md.at(key).is_string()) throw std::runtime_error("missing metadata completion digest");
          if (fs::exists(p))
          {
            bad_manifest = p;
            if (md.at(key).as_string() != doc_digest(read_json_file(p)))
              throw std::runtime_error("completed manifest changed: " + p.string());
            bad_manifest.clear();
          }
        }
      }
      // a completion of another contract (an append, a resume that did not finish) says
      // nothing about this one: the run continues as an ordinary resume
      s.done = ours && s.committed.size() == s.outputs.size() &&
               std::all_of(s.manifests.begin(), s.manifests.end(), [](const fs::path& p) { return fs::is_regular_file(p); });
    }
    catch (const std::system_error&)
    {
      throw;
    }
    catch (const std::exception& ex)
    {
      reason = ex.what();
    }
    if (!reason.empty())
    {
      if (!repairing) throw std::runtime_error(reason + kRepairHint);
      std::cerr << "Repair: run completion record rejected (" << reason << ")" << std::endl;
      s.set_aside(cp);
      if (!bad_manifest.empty() && fs::exists(bad_manifest)) s.set_aside(bad_manifest);
      s.done = false;
    }
  }
  s.prior = prior;
  s.dirty = !prior || recorded != s.contract;
}

RunLedger::~RunLedger() = default;

bool RunLedger::complete() const { return st_->done; }
size_t RunLedger::existing_files() const { return st_->existing; }
size_t RunLedger::verified_files() const { return st_->verified; }
uint64_t RunLedger::verified_bytes() const { return st_->verified_bytes; }
size_t RunLedger::quarantined() const { return st_->moved; }
fs::path RunLedger::quarantine_dir() const { return st_->quarantine; }

void RunLedger::begin()
{
  State& s = *st_;
  fs::create_directories(s.state);
  if (s.sync) sync_directory(s.root);
  if (s.dirty && s.prior)
  {
    // an append: the shorter contract stays authoritative until a new output exists
    publish_json(s.pending_path(), s.contract, s.sync);
    s.pending = true;
  }
  else if (s.dirty)
    publish_json(s.contract_path(), s.contract, s.sync);
  else
  {
    std::error_code ignored;
    fs::remove(s.pending_path(), ignored);   // an abandoned append
  }
  s.begun = true;
}

void RunLedger::archive_residue()
{
  State& s = *st_;
  if (!s.prior && !s.begun) return;
  std::vector<fs::path> dirs{s.root};
  if (fs::exists(s.state)) dirs.push_back(s.state);
  dirs.insert(dirs.end(), s.extra_dirs.begin(), s.extra_dirs.end());
  std::vector<fs::path> found;
  for (const auto& d : dirs)
    for (const auto& e : fs::directory_iterator(d))
    {
      const Residue r = classify(e.path());
      if (r == Residue::Reclaimable) found.push_back(e.path());
      else report_skipped(r, e.path());
    }
  if (!s.pending && exists_no_follow(s.pending_path()))
  {
    if (regular_not_link(s.pending_path())) found.push_back(s.pending_path());
    else report_skipped(Residue::NotRegular, s.pending_path());
  }
  for (const auto& p : found) s.set_aside(p);
  if (!found.empty())
  {
    std::cerr << "Archived " << found.size() << " abandoned private file(s) to " << s.quarantine.string()
              << "; nothing was deleted" << std::endl;
    if (s.sync)
    {
      sync_directory(s.quarantine);
      for (const auto& d : dirs) sync_directory(d);
    }
  }
}

void RunLedger::publish(const fs::path& path, const char* data, size_t size)
{
  State& s = *st_;
  if (!s.begun) throw std::logic_error("output ledger has not begun");
  const fs::path full = canonical_path(path.parent_path()) / path.filename();
  const auto it = s.outputs.find(full);
  if (it == s.outputs.end()) throw std::runtime_error("not an output of this run: " + full.string());
  const LedgerOutput& o = it->second;
  if (o.record_bytes)
  {
    if (size != o.rows * o.record_bytes) throw std::runtime_error("serialized raw row count mismatch");
  }
  else if ((uint64_t)std::count(data, data + size, '\n') != o.rows + 1)
    throw std::runtime_error("serialized CSV row count mismatch");
  Json intent = Json::object();
  intent["schema_version"] = 1;
  intent["key"] = o.key;
  intent["rows"] = (unsigned long long)o.rows;
  intent["algorithm"] = kAlgorithm;
  intent["bytes"] = (unsigned long long)size;
  intent["digest"] = content_digest(data, size);
  const auto known = s.intents.find(o.key);   // not modified after construction
  if (known != s.intents.end())
  {
    if (known->second != intent) throw std::runtime_error("replayed bytes differ from recorded output: " + full.string());
    std::lock_guard<std::mutex> g(s.m);
    if (s.committed.count(o.key)) return;   // the file on disk stays as it is (inode, mtime)
  }
  if (exists_no_follow(full)) throw std::runtime_error("output appeared while run was active: " + full.string());
  publish_json(s.intent_path(o.key), intent, s.sync);   // the intent first: a crash between is replayable
  publish_file(full, data, size, false, s.sync);
  std::lock_guard<std::mutex> g(s.m);
  s.promote();
  s.committed.insert(o.key);
}

void RunLedger::finish()
{
  State& s = *st_;
  std::lock_guard<std::mutex> g(s.m);
  if (s.committed.size() != s.outputs.size()) throw std::runtime_error("run has uncommitted output files");
  s.promote();
  Json md = Json::object();
  for (const auto& p : s.manifests) md[p.filename().string()] = doc_digest(read_json_file(p));
  if (!s.sync)
  {
    // one barrier per finished job: ledger and manifests durable, payloads verified by digest
    for (const auto& p : s.manifests) sync_file(p);
    sync_file(s.contract_path());
    sync_directory(s.root);
    for (const auto& d : s.extra_dirs) sync_directory(d);
  }
  Json c = Json::object();
  c["schema_version"] = 1;
  c["contract_digest"] = s.contract_digest;
  c["durability"] = durability_name(s.sync ? Durability::Fsync : Durability::Rename);
  c["metadata"] = md;
  publish_json(s.state / "complete.json", c, true);   // always durable
  s.done = true;
}

// ------------------------------------------------------------------ --verify-only
Json audit_run_directory(const fs::path& requested, const AuditLayoutFn& layout_fn)
{
  Json report = Json::object();
  Json problems = Json::array(), warnings = Json::array();
  const fs::path root = canonical_path(requested);
  report["output_dir"] = root.string();
  const auto conclude = [&](const char* status) {
    report["status"] = status;
    report["complete"] = std::string(status) == "complete";
    report["problems"] = problems;
    report["warnings"] = warnings;
    return report;
  };
  if (!fs::exists(root))
  {
    problems.push("the output directory does not exist");
    return conclude("not_found");
  }
  if (!fs::is_directory(root))
  {
    problems.push("the path is not a directory");
    return conclude("not_a_run");
  }
  Fd lock;
  lock.fd = ::open(root.c_str(), O_RDONLY | O_DIRECTORY | O_CLOEXEC);
  if (lock.fd < 0) io_fail("open run directory", root);
  // shared: audits run together; a run (exclusive) is either seen here or refused meanwhile
  if (::flock(lock.fd, LOCK_SH | LOCK_NB) != 0)
  {
    if (errno != EWOULDBLOCK) io_fail("lock run directory", root);
    problems.push("a run holds this directory's lock right now; verify again when it has finished");
    return conclude("locked");
  }
  const fs::path state = root / ".opencorr-state";
  if (fs::is_symlink(fs::symlink_status(state)))
  {
    problems.push("the run state .opencorr-state is a symlink");
    return conclude("damaged");
  }
  if (!exists_no_follow(state / "contract.json"))
  {
    problems.push("no .opencorr-state/contract.json: not a ledgered multi-frame output directory "
                  "(single-frame output and binaries older than the output ledger write none)");
    return conclude("not_a_run");
  }
  Json contract;
  AuditLayout layout;
  try
  {
    contract = read_json_file(state / "contract.json");
    if (!contract.is_object() || !contract.has("targets") || !contract.at("targets").is_array() ||
        !contract.has("options") || !contract.at("options").is_object())
      throw std::runtime_error("unexpected contract layout");
    layout = layout_fn(contract, root);
  }
  catch (const std::system_error&)
  {
    throw;
  }
  catch (const std::exception& ex)
  {
    problems.push(std::string("contract.json is not a usable run contract: ") + ex.what());
    return conclude("damaged");
  }
  const std::string cdigest = doc_digest(contract);
  {
    Json sum = Json::object();
    sum["digest"] = cdigest;
    sum["options"] = contract.at("options");
    for (const char* k : {"schema_version", "git_hash", "build_date"})
      if (contract.has(k)) sum[k] = contract.at(k);
    if (contract.has("binary") && contract.at("binary").is_object() && contract.at("binary").has("digest"))
      sum["binary_digest"] = contract.at("binary").at("digest");
    if (contract.has("reference") && contract.at("reference").is_object() && contract.at("reference").has("path"))
      sum["reference"] = contract.at("reference").at("path");
    Json legacy = Json::array();
    for (const char* k : kLegacyScheduling)
      if (contract.at("options").has(k)) legacy.push(k);
    sum["legacy_scheduling_options"] = legacy;
    report["contract"] = sum;
  }

  bool damaged = false, incomplete = false;
  NameList missing, mismatched, no_intent, invalid_intent;
  size_t frames_expected = 0, frames_verified = 0, files_verified = 0;
  uint64_t bytes_verified = 0;
  std::set<uint64_t> frame_rows;
  std::set<fs::path> tracked{state}, dirs{root};
  const auto track = [&](const fs::path& p) {
    tracked.insert(p);
    const fs::path r = p.lexically_relative(root);
    if (!r.empty() && *r.begin() != "..") tracked.insert(root / *r.begin());
    if (p.parent_path() != root) dirs.insert(p.parent_path());
  };
  enum class Verdict { Verified, Missing, NotRegular, NoIntent, InvalidIntent, Mismatched };
  struct Seen
  {
    Verdict v;
    uint64_t bytes = 0, rows = 0;
  };
  // the record, then the file, then its bytes: the order a resume checks them
  const auto check = [&](const AuditOutput& o) -> Seen {
    const fs::path ip = state / (content_digest(o.key.data(), o.key.size()) + ".json");
    Json intent;
    const bool has_intent = exists_no_follow(ip);
    if (has_intent)
    {
      try
      {
        intent = read_json_file(ip);
        require_record(intent);
        if (intent.u64_or("schema_version", 0) != 1 || intent.str_or("key", "") != o.key || !intent.has("rows") ||
            !intent.at("rows").is_unsigned())
          throw std::runtime_error("invalid output intent");
        if (o.record_bytes && intent.at("bytes").as_u64() != intent.at("rows").as_u64() * o.record_bytes)
          throw std::runtime_error("raw record size mismatch in intent");
      }
      catch (const std::system_error&)
      {
        throw;
      }
      catch (const std::exception&)
      {
        return {Verdict::InvalidIntent};
      }
    }
    if (!exists_no_follow(o.path)) return {Verdict::Missing};
    if (!regular_not_link(o.path)) return {Verdict::NotRegular};
    if (!has_intent) return {Verdict::NoIntent};
    const Json seen = file_fingerprint(o.path);
    if (seen.at("bytes") != intent.at("bytes") || seen.at("digest") != intent.at("digest")) return {Verdict::Mismatched};
    return {Verdict::Verified, seen.at("bytes").as_u64(), intent.at("rows").as_u64()};
  };
  const auto file_damage = [&](Verdict v, const std::string& name) {
    if (v == Verdict::InvalidIntent) invalid_intent.add(name);
    else if (v == Verdict::NoIntent) no_intent.add(name);
    else mismatched.add(name);
    damaged = true;
  };
  std::map<fs::path, std::set<std::string>> suffixes;   // per directory, its outputs' extensions
  std::set<fs::path> promised;
  for (const auto& o : layout.outputs)
  {
    track(o.path);
    promised.insert(o.path);
    suffixes[o.path.parent_path()].insert(o.path.extension().string());
    if (o.frame) ++frames_expected;
    const std::string name = rel_name(o.path, root);
    const Seen r = check(o);
    if (r.v == Verdict::Missing)
    {
      missing.add(name);   // the next run publishes it by replay
      incomplete = true;
    }
    else if (r.v != Verdict::Verified)
      file_damage(r.v, name);
    else
    {
      ++files_verified;
      bytes_verified += r.bytes;
      if (o.frame)
      {
        ++frames_verified;
        frame_rows.insert(r.rows);
      }
    }
  }

  // an append in progress: its outputs count when a resume with the longer list would
  // accept them
  const fs::path pending_p = state / "contract.pending.json";
  const bool pending = exists_no_follow(pending_p);
  std::string pending_state = "none";
  NameList appended;
  bool appended_damage = false;
  if (pending)
  {
    pending_state = "unreadable";
    try
    {
      const Json pc = read_json_file(pending_p);
      if (!pc.is_object() || !pc.has("targets") || !pc.at("targets").is_array() || !pc.has("options") ||
          !pc.at("options").is_object())
        throw std::runtime_error("unexpected contract layout");
      if (comparable(pc) != comparable(contract) || !targets_extend(contract.at("targets"), pc.at("targets")))
        pending_state = "unrelated";
      else if (contract.at("targets").size() == pc.at("targets").size())
        pending_state = "promoted";
      else
      {
        pending_state = "append";
        const AuditLayout longer = layout_fn(pc, root);
        for (const auto& o : longer.outputs)
        {
          if (promised.count(o.path)) continue;
          const Seen r = check(o);
          if (r.v == Verdict::Missing) continue;
          const std::string name = rel_name(o.path, root);
          track(o.path);
          if (r.v != Verdict::Verified)
          {
            file_damage(r.v, name);
            appended_damage = true;
          }
          else
          {
            appended.add(name);
            if (o.frame) frame_rows.insert(r.rows);
          }
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
  if (appended.count)
  {
    problems.push("an append was interrupted after it published its first new output and before its longer target "
                  "list replaced the recorded one: rerun the append command (the longer --tar-list) unchanged to "
                  "continue, no --repair needed; the shorter list is no longer accepted, because it does not account "
                  "for the appended output");
    incomplete = true;
  }
  if (appended_damage)
    problems.push("an interrupted append left an output that contradicts its ledger record; rerunning the append "
                  "command (the longer --tar-list) with --repair regenerates it");
  if (frame_rows.size() > 1)
  {
    problems.push("frames record different row counts; one run writes the same rows for every frame");
    damaged = true;
  }

  Json completion = Json::object();
  completion["present"] = false;
  completion["state"] = "missing";
  Json crec;
  bool current = false;
  const fs::path cp = state / "complete.json";
  if (exists_no_follow(cp))
  {
    completion["present"] = true;
    try
    {
      require_regular(cp);
      crec = read_json_file(cp);
      if (!crec.is_object() || crec.u64_or("schema_version", 0) != 1 || !crec.has("contract_digest") ||
          !crec.at("contract_digest").is_string() || !crec.has("metadata") || !crec.at("metadata").is_object())
        throw std::runtime_error("invalid run completion record");
      current = crec.at("contract_digest").as_string() == cdigest;
      completion["state"] = current ? "current" : "other_contract";
      if (crec.has("durability")) completion["durability"] = crec.at("durability");
      if (!current)
      {
        problems.push("complete.json belongs to another target list or contract (an append or resume was started and "
                      "did not finish)");
        incomplete = true;
      }
    }
    catch (const std::system_error&)
    {
      throw;
    }
    catch (const std::exception& ex)
    {
      completion["state"] = "invalid";
      problems.push(std::string("complete.json is damaged: ") + ex.what());
      damaged = true;
    }
  }
  else
  {
    problems.push("no complete.json: the run has not finished");
    incomplete = true;
  }
  report["completion"] = completion;

  Json mans = Json::array();
  for (const auto& p : layout.manifests)
  {
    track(p);
    Json entry = Json::object();
    entry["file"] = rel_name(p, root);
    entry["state"] = "ok";
    if (!exists_no_follow(p))
    {
      entry["state"] = "missing";
      incomplete = true;
      if (current) problems.push("manifest missing: " + rel_name(p, root));
    }
    else
    {
      try
      {
        require_regular(p);
        const std::string d = doc_digest(read_json_file(p));
        ++files_verified;
        bytes_verified += fs::file_size(p);
        if (current)
        {
          const Json& md = crec.at("metadata");
          const std::string key = p.filename().string();
          if (!md.has(key) || !md.at(key).is_string() || md.at(key).as_string() != d)
          {
            entry["state"] = "changed";
            problems.push("manifest differs from the one the completion record digested: " + rel_name(p, root));
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
        entry["state"] = "invalid";
        problems.push("manifest does not parse: " + rel_name(p, root) + ": " + ex.what());
        damaged = true;
      }
    }
    mans.push(entry);
  }
  report["manifests"] = mans;

  NameList untracked, untracked_outputs, residue;
  for (const auto& d : dirs)
  {
    if (!fs::is_directory(d)) continue;
    for (const auto& e : fs::directory_iterator(d))
    {
      if (classify(e.path()) != Residue::Foreign)
      {
        residue.add(rel_name(e.path(), root));
        continue;
      }
      if (tracked.count(e.path())) continue;
      // named like this directory's outputs: a reader globbing frames would take it
      const auto sfx = suffixes.find(d);
      if (sfx != suffixes.end() && sfx->second.count(e.path().extension().string()))
        untracked_outputs.add(rel_name(e.path(), root));
      else
        untracked.add(rel_name(e.path(), root));
    }
  }
  if (fs::is_directory(state))
    for (const auto& e : fs::directory_iterator(state))
      if (classify(e.path()) != Residue::Foreign) residue.add(rel_name(e.path(), root));
  if (untracked_outputs.count)
  {
    problems.push("entries named like this run's outputs (same directory, same extension) that the ledger does not list");
    damaged = true;
  }
  if (residue.count)
    warnings.push("temporary files of an interrupted run; the next run archives them under .opencorr-state/quarantine/");
  if (pending_state == "append" && !appended.count && !appended_damage)
    warnings.push("contract.pending.json: an append was started and stopped before any appended output was published; "
                  "the recorded target list is still the valid one");
  else if (pending_state == "promoted")
    warnings.push("contract.pending.json repeats the recorded contract: an append was promoted and only this file is "
                  "left over; the next run archives it");
  else if (pending_state == "unrelated")
    warnings.push("contract.pending.json does not extend the recorded contract (other binary, reference, options or "
                  "target prefix), so it says nothing about this directory; the next run archives it");
  else if (pending_state == "unreadable")
    warnings.push("contract.pending.json cannot be read as a contract, so it says nothing about an interrupted append; "
                  "the next run archives it");
  if (missing.count) problems.push("frames or diagnostics files the contract promises are missing");
  if (mismatched.count) problems.push("files whose bytes do not match their ledger record (or that are not regular files)");
  if (no_intent.count) problems.push("files with no ledger record");
  if (invalid_intent.count) problems.push("ledger records that do not parse or do not describe their file");

  NameList in_changed, in_missing;
  size_t checked = 0;
  {
    std::map<std::string, Json> inputs;
    const auto collect = [&](const Json& id) {
      if (id.is_object() && id.has("path") && id.at("path").is_string() && id.has("content") && id.at("content").is_object())
        inputs.emplace(id.at("path").as_string(), id.at("content"));
    };
    if (contract.has("reference")) collect(contract.at("reference"));
    for (const auto& t : contract.at("targets").items())
      if (t.is_object() && t.has("input")) collect(t.at("input"));
    for (const auto& in : inputs)
    {
      std::error_code ec;
      if (!fs::is_regular_file(fs::path(in.first), ec))
      {
        in_missing.add(in.first);
        continue;
      }
      ++checked;
      const Json seen = file_fingerprint(in.first);
      if (!in.second.has("bytes") || !in.second.has("digest") || seen.at("bytes") != in.second.at("bytes") ||
          seen.at("digest") != in.second.at("digest"))
        in_changed.add(in.first);
    }
  }
  Json ir = Json::object();
  ir["checked"] = (unsigned long long)checked;
  ir["status"] = in_changed.count ? "changed" : in_missing.count ? "missing" : "match";
  in_changed.store(ir, "changed");
  in_missing.store(ir, "missing");
  report["inputs"] = ir;
  if (in_changed.count)
    problems.push("input images no longer match the fingerprints in the contract; the outputs still match their ledger, "
                  "but they describe images that are no longer at those paths");
  if (in_missing.count)
    warnings.push("input images are not at the recorded paths, so they were not compared; rerunning the command needs "
                  "them there");

  report["frames_expected"] = (unsigned long long)frames_expected;
  report["frames_verified"] = (unsigned long long)frames_verified;
  report["files_expected"] = (unsigned long long)(layout.outputs.size() + layout.manifests.size());
  report["files_verified"] = (unsigned long long)files_verified;
  report["bytes_verified"] = (unsigned long long)bytes_verified;
  if (frame_rows.size() == 1) report["rows_per_frame"] = (unsigned long long)*frame_rows.begin();
  missing.store(report, "missing");
  mismatched.store(report, "mismatched");
  no_intent.store(report, "no_intent");
  invalid_intent.store(report, "invalid_intent");
  untracked_outputs.store(report, "untracked_outputs");
  untracked.store(report, "untracked");
  residue.store(report, "residue");
  report["pending_append"] = pending;
  report["pending_append_state"] = pending_state;
  appended.store(report, "appended_published");
  if (damaged) return conclude("damaged");
  if (incomplete) return conclude("incomplete");
  if (in_changed.count) return conclude("inputs_changed");
  return conclude("complete");
}

}  // namespace dic_cli
