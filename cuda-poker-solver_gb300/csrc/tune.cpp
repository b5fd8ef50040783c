// Launch-shape cache of the autotuner (see tune.h).
#include "tune.h"

#include <cuda_runtime.h>

#include <cstdio>
#include <cstdlib>
#include <map>
#include <mutex>
#include <sys/stat.h>
#include <unistd.h>

namespace pps {
namespace gb {

namespace {

struct Entry {
  LaunchShape shape;
  double ms = 0.0;
};

std::mutex gMutex;
bool gLoaded = false;
std::map<std::pair<int, int>, Entry> gCache;

std::string cachePath() {
  const char* f = std::getenv("PPS_GB_TUNE_FILE");
  if (f && *f) return std::string(f) == "off" ? std::string() : std::string(f);
  std::string dir;
  if (const char* x = std::getenv("XDG_CACHE_HOME"); x && *x) dir = x;
  else if (const char* h = std::getenv("HOME"); h && *h) dir = std::string(h) + "/.cache";
  else return std::string();
  return dir + "/pps_gb/launch_shapes";
}

// One line per class: width size plan fwd bwd sd fd ms.
void loadLocked() {
  if (gLoaded) return;
  gLoaded = true;
  const std::string path = cachePath();
  if (path.empty()) return;
  FILE* f = std::fopen(path.c_str(), "r");
  if (!f) return;
  int w, z;
  Entry e;
  while (std::fscanf(f, "%d %d %d %d %d %d %d %lf", &w, &z, &e.shape.plan, &e.shape.fwdCap,
                     &e.shape.bwdCap, &e.shape.sdCap, &e.shape.fdCap, &e.ms) == 8) {
    if (e.shape.plan != 0 && e.shape.plan != 2) continue;
    gCache[{w, z}] = e;
  }
  std::fclose(f);
}

void mkdirs(const std::string& path) {
  for (size_t i = 1; i < path.size(); ++i)
    if (path[i] == '/') ::mkdir(path.substr(0, i).c_str(), 0755);
}

// Rewrites the file (temporary file, then rename): the last writer wins, a
// reader never sees a half-written file. Failures are ignored (the cache is
// an optimization).
void saveLocked() {
  const std::string path = cachePath();
  if (path.empty()) return;
  mkdirs(path);
  const std::string tmp = path + ".tmp" + std::to_string((long)::getpid());
  FILE* f = std::fopen(tmp.c_str(), "w");
  if (!f) return;
  for (const auto& kv : gCache) {
    const LaunchShape& s = kv.second.shape;
    std::fprintf(f, "%d %d %d %d %d %d %d %.6f\n", kv.first.first, kv.first.second, s.plan,
                 s.fwdCap, s.bwdCap, s.sdCap, s.fdCap, kv.second.ms);
  }
  if (std::fclose(f) == 0) std::rename(tmp.c_str(), path.c_str());
  else std::remove(tmp.c_str());
}

}  // namespace

TuneKey tuneKeyOf(int maxN, int64_t rowBytes) {
  TuneKey k;
  k.widthClass = maxN <= 511 ? 0 : maxN <= 1023 ? 1 : 2;
  int z = 0;
  while (z < 62 && ((int64_t)1 << (z + 1)) <= rowBytes) ++z;
  k.sizeClass = z;
  return k;
}

bool lookupShape(const TuneKey& k, LaunchShape* out) {
  std::lock_guard<std::mutex> lock(gMutex);
  loadLocked();
  const auto it = gCache.find({k.widthClass, k.sizeClass});
  if (it == gCache.end()) return false;
  *out = it->second.shape;
  return true;
}

void storeShape(const TuneKey& k, const LaunchShape& s, double msPerIteration) {
  std::lock_guard<std::mutex> lock(gMutex);
  loadLocked();
  gCache[{k.widthClass, k.sizeClass}] = Entry{s, msPerIteration};
  saveLocked();
}

std::string shapeText(const LaunchShape& s) {
  return std::string(s.plan == 2 ? "fused" : "staged") + " fwd" + std::to_string(s.fwdCap) +
         " bwd" + std::to_string(s.bwdCap) + " sd" + std::to_string(s.sdCap) + " fd" +
         std::to_string(s.fdCap);
}

unsigned cappedGrid(unsigned grid, int capSms) {
  if (capSms <= 0) return grid;
  int dev = 0, sms = 0;
  if (cudaGetDevice(&dev) != cudaSuccess ||
      cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || sms <= 0)
    return grid;
  const unsigned cap = (unsigned)capSms * (unsigned)sms;
  return grid > cap ? cap : grid;
}

}  // namespace gb
}  // namespace pps
