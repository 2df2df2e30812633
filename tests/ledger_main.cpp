// Test harness for the output ledger (fasticgn_gb300/cli/ledger.cpp) without a GPU: a
// synthetic multi-frame "run" publishes raw frame payloads (rows x 36 bytes whose content
// depends only on the frame index) and a manifest through RunLedger, exactly as the
// command line does, and `verify` runs the --verify-only audit.
//
//   ledger_main run <root> <tar_list> <frames> <rows> [--repair] [--fsync] [--option V]
//                   [--stop-after K] [--corrupt-replay K] [--input PATH]
//   ledger_main verify <root>
//
// `run` prints one JSON line: complete_at_start, existing, quarantined, published; an
// error prints {"error": "..."} and exits 1.
#include "json.h"
#include "ledger.h"

#include <cstdio>
#include <cstring>
#include <iostream>
#include <string>
#include <vector>

using namespace dic_cli;

namespace
{

std::string frame_name(int k)
{
  char b[32];
  std::snprintf(b, sizeof b, "frame_%06d.bin", k);
  return b;
}

std::vector<char> payload(int k, uint64_t rows)
{
  std::vector<char> p(rows * 36);
  unsigned x = 0x9e3779b9u ^ (unsigned)(k * 2654435761u);
  for (auto& c : p)
  {
    x ^= x << 13;
    x ^= x >> 17;
    x ^= x << 5;
    c = (char)(x & 0xff);
  }
  return p;
}

Json contract_for(int frames, const std::string& option, const std::string& input)
{
  Json c = Json::object();
  c["schema_version"] = 1;
  c["git_hash"] = "harness";
  c["build_date"] = "harness";
  Json op = Json::object();
  op["format"] = "raw";
  op["option"] = option;
  op["diagnostics"] = false;
  c["options"] = op;
  if (!input.empty())
  {
    Json ref = Json::object();
    ref["path"] = fs::canonical(input).string();
    ref["content"] = file_fingerprint(input);
    c["reference"] = ref;
  }
  Json t = Json::array();
  for (int k = 0; k < frames; ++k)
  {
    Json e = Json::object();
    e["file"] = frame_name(k);
    e["output_name"] = frame_name(k);
    t.push(e);
  }
  c["targets"] = t;
  return c;
}

AuditLayout layout(const Json& contract, const fs::path& root)
{
  AuditLayout l;
  for (const auto& t : contract.at("targets").items())
  {
    const std::string f = t.at("file").as_string();
    l.outputs.push_back(AuditOutput{"frame/" + f, root / f, 36, true});
  }
  l.manifests.push_back(root / "manifest.opencorr-raw.json");
  return l;
}

}  // namespace

int main(int argc, char** argv)
{
  std::vector<std::string> a(argv + 1, argv + argc);
  try
  {
    if (a.size() >= 2 && a[0] == "verify")
    {
      const Json r = audit_run_directory(a[1], layout);
      std::cout << r.dump() << std::endl;
      return r.at("status").as_string() == "complete" ? 0 : 1;
    }
    if (a.size() < 5 || a[0] != "run") return 2;
    const fs::path root = a[1];
    const fs::path list = a[2];
    const int frames = std::stoi(a[3]);
    const uint64_t rows = std::stoull(a[4]);
    bool repair = false, fsync = false;
    std::string option = "1", input;
    int stop_after = -1, corrupt_replay = -1;
    for (size_t i = 5; i < a.size(); ++i)
    {
      if (a[i] == "--repair") repair = true;
      else if (a[i] == "--fsync") fsync = true;
      else if (a[i] == "--option") option = a[++i];
      else if (a[i] == "--stop-after") stop_after = std::stoi(a[++i]);
      else if (a[i] == "--corrupt-replay") corrupt_replay = std::stoi(a[++i]);
      else if (a[i] == "--input") input = a[++i];
    }
    fs::create_directories(root);
    std::vector<LedgerOutput> outs;
    for (int k = 0; k < frames; ++k) outs.push_back(LedgerOutput{"frame/" + frame_name(k), root / frame_name(k), rows, 36});
    RunLedger ledger(root, contract_for(frames, option, input), outs, {root / "manifest.opencorr-raw.json"}, list,
                     fsync ? Durability::Fsync : Durability::Rename, repair);
    ledger.archive_residue();
    Json out = Json::object();
    out["complete_at_start"] = ledger.complete();
    out["existing"] = (unsigned long long)ledger.existing_files();
    out["quarantined"] = (unsigned long long)ledger.quarantined();
    out["verified_bytes"] = (unsigned long long)ledger.verified_bytes();
    unsigned long long published = 0;
    if (!ledger.complete())
    {
      ledger.begin();
      Json manifest = Json::object();
      manifest["format"] = "opencorr-gpu-raw-v1";
      Json mf = Json::array();
      for (int k = 0; k < frames; ++k)
      {
        std::vector<char> p = payload(k, rows);
        if (k == corrupt_replay) p[0] ^= 1;   // a replay that does not reproduce its bytes
        const bool existed = fs::exists(root / frame_name(k));
        ledger.publish(root / frame_name(k), p.data(), p.size());
        published += existed ? 0 : 1;
        Json e = Json::object();
        e["file"] = frame_name(k);
        e["output_name"] = frame_name(k);
        e["rows"] = (unsigned long long)rows;
        e["bytes"] = (unsigned long long)p.size();
        mf.push(e);
        if (k + 1 == stop_after)
        {
          out["published"] = published;
          out["stopped"] = true;
          std::cout << out.dump() << std::endl;
          return 0;
        }
      }
      manifest["frames"] = mf;
      publish_json(root / "manifest.opencorr-raw.json", manifest, fsync);
      ledger.finish();
      ledger.archive_residue();
    }
    out["published"] = published;
    out["quarantine_dir"] = ledger.quarantine_dir().string();
    std::cout << out.dump() << std::endl;
    return 0;
  }
  catch (const std::exception& ex)
  {
    Json e = Json::object();
    e["error"] = std::string(ex.what());
    std::cout << e.dump() << std::endl;
    return 1;
  }
}
