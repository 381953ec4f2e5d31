// Optional per-kernel timing with CUDA events recorded on the launching stream,
// and optional NVTX ranges per public entry point and per kernel launch (both
// off by default; rc_profile_enable picks them).  Each launch site brackets its
// kernel with prof_begin / prof_end; rc_profile_report sums the event intervals
// per kernel name.  The NVTX ranges are host-side markers for a timeline tool
// (they cost nothing when no tool is attached) and are also emitted for launches
// recorded into a CUDA graph.
#include <nvtx3/nvToolsExt.h>

#include <atomic>
#include <cstdio>
#include <map>
#include <mutex>
#include <string>
#include <vector>

#include "context.hpp"

namespace rc {

namespace {
struct Rec {
  const char* name;
  cudaEvent_t a, b;
};
std::mutex g_mu;
bool g_on = false;
std::vector<Rec> g_recs;
std::vector<cudaEvent_t> g_pool;
struct Open {
  const char* name;
  cudaEvent_t a;
};
std::map<cudaStream_t, std::vector<Open>> g_open;

cudaEvent_t take_event() {
  if (!g_pool.empty()) {
    cudaEvent_t e = g_pool.back();
    g_pool.pop_back();
    return e;
  }
  cudaEvent_t e;
  cudaEventCreate(&e);
  return e;
}
}  // namespace

std::atomic<bool> g_nvtx{false};

bool prof_enabled() { return g_on; }
bool nvtx_enabled() { return g_nvtx.load(std::memory_order_relaxed); }
void nvtx_push(const char* name) { nvtxRangePushA(name); }
void nvtx_pop() { nvtxRangePop(); }

// launches recorded into a CUDA graph are not timed (an event record would become a graph node)
static bool capturing(cudaStream_t s) {
  cudaStreamCaptureStatus st = cudaStreamCaptureStatusNone;
  return cudaStreamIsCapturing(s, &st) == cudaSuccess && st != cudaStreamCaptureStatusNone;
}

void prof_begin(const char* name, cudaStream_t s) {
  if (nvtx_enabled()) nvtx_push(name);
  if (!g_on || capturing(s)) return;
  std::lock_guard<std::mutex> lk(g_mu);
  cudaEvent_t e = take_event();
  cudaEventRecord(e, s);
  g_open[s].push_back(Open{name, e});
}

void prof_end(const char* name, cudaStream_t s) {
  if (nvtx_enabled()) nvtx_pop();
  if (!g_on || capturing(s)) return;
  std::lock_guard<std::mutex> lk(g_mu);
  auto& v = g_open[s];
  if (v.empty()) return;
  Open o = v.back();
  v.pop_back();
  cudaEvent_t e = take_event();
  cudaEventRecord(e, s);
  g_recs.push_back(Rec{name ? name : o.name, o.a, e});
}

}  // namespace rc

using namespace rc;

extern "C" int rc_profile_enable(int flags) {
  std::lock_guard<std::mutex> lk(g_mu);
  g_on = (flags & RC_PROFILE_EVENTS) != 0;
  g_nvtx.store((flags & RC_PROFILE_NVTX) != 0, std::memory_order_relaxed);
  return RC_OK;
}

extern "C" int rc_profile_report(char* buf, size_t len) {
  std::lock_guard<std::mutex> lk(g_mu);
  cudaDeviceSynchronize();
  std::map<std::string, std::pair<long, double>> agg;
  for (auto& r : g_recs) {
    float ms = 0.f;
    if (cudaEventElapsedTime(&ms, r.a, r.b) == cudaSuccess) {
      auto& x = agg[r.name];
      x.first += 1;
      x.second += ms;
    }
    g_pool.push_back(r.a);
    g_pool.push_back(r.b);
  }
  g_recs.clear();
  std::string out = "{";
  bool first = true;
  for (auto& kv : agg) {
    char tmp[256];
    snprintf(tmp, sizeof(tmp), "%s\"%s\": {\"launches\": %ld, \"ms\": %.6f}", first ? "" : ", ", kv.first.c_str(),
             kv.second.first, kv.second.second);
    out += tmp;
    first = false;
  }
  out += "}";
  if (buf && len) {
    size_t n = out.size() < len - 1 ? out.size() : len - 1;
    memcpy(buf, out.data(), n);
    buf[n] = 0;
  }
  return out.size() < len ? RC_OK : RC_ERR_INVALID_ARGUMENT;
}
