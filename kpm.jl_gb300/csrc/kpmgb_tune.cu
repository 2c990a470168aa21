// Persistent autotuning cache.
//
// The autotuners (the per-step kernel choice of kernel_variant 4 and the
// ensemble kernel's launch shape) time their candidates once per problem
// shape.  Their choices are kept in a text file, one "key value" line per
// shape, so a later process on the same kind of GPU reuses them without
// timing again.  Keys carry the device name, SM count and compute capability.
// The file is KPMGB_TUNE_CACHE if set (an empty value disables the cache),
// else $XDG_CACHE_HOME/kpmgb/tune.txt or $HOME/.cache/kpmgb/tune.txt.
// Writes go to a temporary file renamed over the cache, so a reader never sees
// a partial file; concurrent writers may drop each other's newest line, which
// only costs a re-tune.
#include <cuda_runtime.h>

#include <sys/stat.h>
#include <unistd.h>

#include <cstdio>
#include <cstdlib>
#include <fstream>
#include <map>
#include <mutex>
#include <sstream>
#include <string>

#include "kpmgb_internal.h"

namespace kpmgb {
namespace {

std::mutex g_tune_mtx;

void make_dirs(const std::string& path) {
  for (size_t i = 1; i < path.size(); ++i)
    if (path[i] == '/') mkdir(path.substr(0, i).c_str(), 0755);
}

std::map<std::string, std::string> read_all(const std::string& path) {
  std::map<std::string, std::string> m;
  std::ifstream f(path);
  std::string line;
  while (std::getline(f, line)) {
    const size_t sp = line.rfind(' ');
    if (sp == std::string::npos || sp == 0) continue;
    m[line.substr(0, sp)] = line.substr(sp + 1);
  }
  return m;
}

}  // namespace

std::string tune_cache_path() {
  if (const char* e = std::getenv("KPMGB_TUNE_CACHE")) return e;
  if (const char* x = std::getenv("XDG_CACHE_HOME"); x && *x) return std::string(x) + "/kpmgb/tune.txt";
  if (const char* h = std::getenv("HOME"); h && *h) return std::string(h) + "/.cache/kpmgb/tune.txt";
  return "";
}

std::string device_tag() {
  int dev = 0;
  cudaDeviceProp p{};
  if (cudaGetDevice(&dev) != cudaSuccess || cudaGetDeviceProperties(&p, dev) != cudaSuccess) {
    cudaGetLastError();
    return "unknown";
  }
  std::string name(p.name);
  for (char& c : name)
    if (c == ' ') c = '_';
  std::ostringstream o;
  o << name << "/sm" << p.major << p.minor << "/" << p.multiProcessorCount;
  return o.str();
}

bool tune_cache_get(const std::string& key, std::string* value) {
  const std::string path = tune_cache_path();
  if (path.empty()) return false;
  std::lock_guard<std::mutex> lk(g_tune_mtx);
  const auto m = read_all(path);
  auto it = m.find(key);
  if (it == m.end()) return false;
  *value = it->second;
  return true;
}

void tune_cache_put(const std::string& key, const std::string& value) {
  const std::string path = tune_cache_path();
  if (path.empty() || key.find('\n') != std::string::npos || value.find(' ') != std::string::npos)
    return;
  std::lock_guard<std::mutex> lk(g_tune_mtx);
  auto m = read_all(path);
  m[key] = value;
  make_dirs(path);
  const std::string tmp = path + ".tmp" + std::to_string((long)getpid());
  bool ok = false;
  {
    std::ofstream f(tmp, std::ios::trunc);
    if (!f) return;
    for (const auto& kv : m) f << kv.first << ' ' << kv.second << '\n';
    f.flush();
    ok = f.good();
  }
  // a short write (full disk) must not replace a good cache
  if (!ok || std::rename(tmp.c_str(), path.c_str()) != 0) std::remove(tmp.c_str());
}

}  // namespace kpmgb
