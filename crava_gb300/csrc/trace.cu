// Launch tracing: per-kernel CUDA-event timing and algorithmic byte counts,
// the GPU counterpart of the reference's Timings phase timers
// (src/timings.h:11-30).  Off by default; when on, every library launch
// records a start/stop event pair on the stream it was launched on.
#include <map>
#include <mutex>
#include <string>
#include <vector>

#include "common.cuh"
#include "trace.cuh"

namespace cg {

namespace {
struct Rec {
  std::string name;
  cudaEvent_t a, b;
  double bytes;
};
std::mutex g_mu;
bool g_on = false;
std::vector<Rec> g_recs;
std::vector<cudaEvent_t> g_pool;

cudaEvent_t get_event()
{
  if (!g_pool.empty()) {
    cudaEvent_t e = g_pool.back();
    g_pool.pop_back();
    return e;
  }
  cudaEvent_t e = nullptr;
  cudaEventCreate(&e);
  return e;
}

struct Agg {
  long launches = 0;
  double ms = 0, bytes = 0;
};
std::vector<std::pair<std::string, Agg>> g_report;
}  // namespace

thread_local bool t_suppress = false;

bool trace_on() { return g_on; }

TraceSuppress::TraceSuppress() : prev_(t_suppress) { t_suppress = true; }
TraceSuppress::~TraceSuppress() { t_suppress = prev_; }

TraceScope::TraceScope(const char *name, cudaStream_t st, double bytes) : name_(name), st_(st), bytes_(bytes)
{
  if (!g_on || t_suppress) return;
  std::lock_guard<std::mutex> lk(g_mu);
  a_ = get_event();
  b_ = get_event();
  if (a_ && b_) cudaEventRecord((cudaEvent_t)a_, st_);
}

TraceScope::~TraceScope()
{
  if (!a_ || !b_) return;
  std::lock_guard<std::mutex> lk(g_mu);
  cudaEventRecord((cudaEvent_t)b_, st_);
  g_recs.push_back({name_, (cudaEvent_t)a_, (cudaEvent_t)b_, bytes_});
}

}  // namespace cg

using namespace cg;

extern "C" int cg_trace_enable(int on)
{
  std::lock_guard<std::mutex> lk(g_mu);
  g_on = on != 0;
  for (auto &r : g_recs) { g_pool.push_back(r.a); g_pool.push_back(r.b); }
  g_recs.clear();
  g_report.clear();
  return CG_OK;
}

/* Synchronise, aggregate the recorded launches by kernel name and return how
 * many distinct kernels were seen. */
extern "C" int cg_trace_collect(void)
{
  CG_CUDA(cudaDeviceSynchronize());
  std::lock_guard<std::mutex> lk(g_mu);
  std::map<std::string, Agg> m;
  for (auto &r : g_recs) {
    float ms = 0;
    CG_CUDA(cudaEventElapsedTime(&ms, r.a, r.b));
    Agg &a = m[r.name];
    a.launches++;
    a.ms += ms;
    a.bytes += r.bytes;
    g_pool.push_back(r.a);
    g_pool.push_back(r.b);
  }
  g_recs.clear();
  g_report.assign(m.begin(), m.end());
  return (int)g_report.size();
}

extern "C" int cg_trace_entry(int i, char *name, int name_len, long *launches, double *ms, double *bytes)
{
  std::lock_guard<std::mutex> lk(g_mu);
  if (i < 0 || i >= (int)g_report.size()) { set_error("trace entry %d out of range", i); return CG_ERR_ARG; }
  const auto &e = g_report[i];
  if (name && name_len > 0) {
    snprintf(name, name_len, "%s", e.first.c_str());
  }
  if (launches) *launches = e.second.launches;
  if (ms) *ms = e.second.ms;
  if (bytes) *bytes = e.second.bytes;
  return CG_OK;
}
