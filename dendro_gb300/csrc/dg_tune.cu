// Disk cache of the autotuner's decisions (dg_runtime.cuh): one line per
// (device, key width, size class), tab-separated:
//   device-key  width  log2-size  keys-per-thread  blocks-per-SM  histogram-blocks-per-SM
// The device key is "<name>|<SMs>|cc<major>.<minor>|v<library version>", so
// decisions never travel between GPU models or library versions.  The file
// is read once per process and rewritten (to a temporary file, then
// renamed) after every new decision.
#include <cuda_runtime.h>

#include <cstdio>
#include <cstdlib>
#include <fstream>
#include <map>
#include <mutex>
#include <sstream>
#include <string>
#include <sys/stat.h>
#include <tuple>
#include <unistd.h>

#include "dendro_gb300.h"
#include "dg_runtime.cuh"

namespace dg {
namespace {

std::mutex g_tune_mu;
bool g_tune_loaded = false;
std::map<std::tuple<std::string, int, int>, Context::Tune> g_tune;
std::map<int, std::string> g_dev_key;

std::string device_key(int device) {
  auto it = g_dev_key.find(device);
  if (it != g_dev_key.end()) return it->second;
  cudaDeviceProp p;
  std::string key;
  if (cudaGetDeviceProperties(&p, device) == cudaSuccess) {
    std::ostringstream o;
    o << p.name << "|" << p.multiProcessorCount << "|cc" << p.major << "." << p.minor << "|v" << dg_version();
    key = o.str();
    for (char &c : key)
      if (c == '\t' || c == '\n') c = ' ';
  } else {
    cudaGetLastError();
  }
  g_dev_key[device] = key;
  return key;
}

void mkdirs(const std::string &dir) {
  for (size_t i = 1; i <= dir.size(); i++)
    if (i == dir.size() || dir[i] == '/') mkdir(dir.substr(0, i).c_str(), 0755);
}

void load_locked() {
  if (g_tune_loaded) return;
  g_tune_loaded = true;
  const std::string path = tune_cache_path();
  if (path.empty()) return;
  std::ifstream f(path);
  std::string line;
  while (std::getline(f, line)) {
    std::istringstream in(line);
    std::string key, w, b, it, mb, hm;
    if (!std::getline(in, key, '\t') || !std::getline(in, w, '\t') || !std::getline(in, b, '\t') ||
        !std::getline(in, it, '\t') || !std::getline(in, mb, '\t') || !std::getline(in, hm))
      continue;
    Context::Tune t;
    t.items = std::atoi(it.c_str());
    t.minb = std::atoi(mb.c_str());
    t.hist_mul = std::atoi(hm.c_str());
    const int wi = std::atoi(w.c_str()), bi = std::atoi(b.c_str());
    // only shapes the library compiles: 16 or 8 keys per thread for 8-byte
    // keys, 8 or 4 for 16-byte keys; 3 to 5 blocks per SM
    const int big = wi == 0 ? 16 : 8;
    const bool valid = (wi == 0 || wi == 1) && bi >= 0 && bi < 64 && (t.items == big || t.items == big / 2) &&
                       t.minb >= 3 && t.minb <= 5 && (t.hist_mul == 2 || t.hist_mul == 4 || t.hist_mul == 8);
    if (valid) g_tune[std::make_tuple(key, wi, bi)] = t;
  }
}

void save_locked() {
  const std::string path = tune_cache_path();
  if (path.empty()) return;
  const size_t slash = path.rfind('/');
  if (slash != std::string::npos) mkdirs(path.substr(0, slash));
  const std::string tmp = path + ".tmp" + std::to_string((long)getpid());
  {
    std::ofstream f(tmp);
    if (!f) return;
    for (auto &kv : g_tune)
      f << std::get<0>(kv.first) << '\t' << std::get<1>(kv.first) << '\t' << std::get<2>(kv.first) << '\t'
        << kv.second.items << '\t' << kv.second.minb << '\t' << kv.second.hist_mul << '\n';
    if (!f) return;
  }
  std::rename(tmp.c_str(), path.c_str());
}

}  // namespace

std::string tune_cache_path() {
  if (const char *e = std::getenv("DENDRO_GB300_TUNE_CACHE")) return e;  // "" turns the cache off
  if (const char *x = std::getenv("XDG_CACHE_HOME"))
    if (*x) return std::string(x) + "/dendro_gb300/autotune.tsv";
  if (const char *h = std::getenv("HOME"))
    if (*h) return std::string(h) + "/.cache/dendro_gb300/autotune.tsv";
  return "";
}

bool tune_cache_get(int device, int width, int bucket, Context::Tune *out) {
  std::lock_guard<std::mutex> lk(g_tune_mu);
  load_locked();
  const std::string key = device_key(device);
  if (key.empty()) return false;
  auto it = g_tune.find(std::make_tuple(key, width, bucket));
  if (it == g_tune.end()) return false;
  *out = it->second;
  return true;
}

void tune_cache_put(int device, int width, int bucket, const Context::Tune &t) {
  std::lock_guard<std::mutex> lk(g_tune_mu);
  load_locked();
  const std::string key = device_key(device);
  if (key.empty()) return;
  g_tune[std::make_tuple(key, width, bucket)] = t;
  save_locked();
}

}  // namespace dg
