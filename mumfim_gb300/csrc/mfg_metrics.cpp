// Structured metrics sink: one JSON object per line, appended to a file, for
// a service loop to log what each call of the C ABI did (the reference's
// only record is its MUMFIM_V1 timing prints, MultiscaleRVEAnalysis.cc:241,283-286).
// Off unless mfg_set_metrics_log() names a file or the MFG_METRICS_LOG
// environment variable does; a record is written by one locked append, so
// several threads and batches may share the file.
#include <chrono>
#include <cstdio>
#include <cstdlib>
#include <mutex>
#include <string>

#include "mfg_metrics.h"
#include "mumfim_gpu.h"

namespace mfg {
namespace {

std::mutex g_mu;
std::string g_path;
bool g_init = false;

void init_locked() {
  if (g_init) return;
  g_init = true;
  const char* env = std::getenv("MFG_METRICS_LOG");
  if (env && *env) g_path = env;
}

}  // namespace

bool metrics_enabled() {
  std::lock_guard<std::mutex> lock(g_mu);
  init_locked();
  return !g_path.empty();
}

double wall_seconds() {
  using namespace std::chrono;
  return duration<double>(system_clock::now().time_since_epoch()).count();
}

void metrics_write(const std::string& fields) {
  std::lock_guard<std::mutex> lock(g_mu);
  init_locked();
  if (g_path.empty()) return;
  FILE* f = std::fopen(g_path.c_str(), "a");
  if (!f) return;
  std::fprintf(f, "{\"t\": %.6f, %s}\n", wall_seconds(), fields.c_str());
  std::fclose(f);
}

std::string json_escape(const char* s) {
  std::string o;
  for (; s && *s; ++s) {
    const char c = *s;
    if (c == '"' || c == '\\') {
      o += '\\';
      o += c;
    } else if (static_cast<unsigned char>(c) < 0x20) {
      o += ' ';
    } else {
      o += c;
    }
  }
  return o;
}

}  // namespace mfg

extern "C" mfg_status mfg_set_metrics_log(const char* path) {
  std::lock_guard<std::mutex> lock(mfg::g_mu);
  mfg::g_init = true;
  mfg::g_path = path ? path : "";
  return MFG_OK;
}
