// Live per-kernel timing: when enabled (ctm_profile_begin), selected kernel
// launches are bracketed by CUDA events on their own stream; ctm_profile_end
// synchronizes the recorded events and sums duration and algorithmic work
// per kernel class.  Disabled, the timer costs one branch.
#include "ctm_common.cuh"

#include <mutex>

namespace ctm {

namespace {

struct Record {
  cudaEvent_t a, b;
  int tag;  // -1: named
  const char* name;
  int unit;
  double work;
};

struct NamedClass {
  std::string name;
  int unit;
  double ms, work;
  long long count;
};

std::mutex g_mu;
bool g_on = false;
std::vector<Record> g_records;
std::vector<cudaEvent_t> g_pool;
double g_ms[kProfileTags];
double g_work[kProfileTags];
long long g_count[kProfileTags];
std::vector<NamedClass> g_named;

cudaEvent_t take_event() {
  if (!g_pool.empty()) {
    cudaEvent_t e = g_pool.back();
    g_pool.pop_back();
    return e;
  }
  cudaEvent_t e;
  CTM_CUDA(cudaEventCreate(&e));
  return e;
}

}  // namespace

KernelTimer::KernelTimer(cudaStream_t s, int tag, double work) : stream_(s) {
  start(tag, nullptr, kUnitFlop, work);
}

KernelTimer::KernelTimer(cudaStream_t s, const char* name, int unit, double work) : stream_(s) {
  start(-1, name, unit, work);
}

void KernelTimer::start(int tag, const char* name, int unit, double work) {
  std::lock_guard<std::mutex> lk(g_mu);
  if (!g_on || work < 0.0) return;  // negative work: a disabled timer
  active_ = true;
  idx_ = g_records.size();
  Record r{take_event(), take_event(), tag, name, unit, work};
  CTM_CUDA(cudaEventRecord(r.a, stream_));
  g_records.push_back(r);
}

KernelTimer::~KernelTimer() {
  if (!active_) return;
  std::lock_guard<std::mutex> lk(g_mu);
  if (idx_ < g_records.size()) cudaEventRecord(g_records[idx_].b, stream_);
}

}  // namespace ctm

using namespace ctm;

extern "C" {

void ctm_profile_begin(void) {
  std::lock_guard<std::mutex> lk(g_mu);
  for (auto& r : g_records) {
    g_pool.push_back(r.a);
    g_pool.push_back(r.b);
  }
  g_records.clear();
  for (int i = 0; i < kProfileTags; ++i) g_ms[i] = g_work[i] = 0.0, g_count[i] = 0;
  g_named.clear();
  g_on = true;
}

int ctm_profile_end(void) {
  return guarded([&] {
    std::lock_guard<std::mutex> lk(g_mu);
    g_on = false;
    for (auto& r : g_records) {
      CTM_CUDA(cudaEventSynchronize(r.b));
      float ms = 0.f;
      CTM_CUDA(cudaEventElapsedTime(&ms, r.a, r.b));
      if (r.tag >= 0 && r.tag < kProfileTags) {
        g_ms[r.tag] += ms;
        g_work[r.tag] += r.work;
        g_count[r.tag] += 1;
      } else if (r.tag < 0 && r.name != nullptr) {
        NamedClass* nc = nullptr;
        for (auto& x : g_named)
          if (x.name == r.name && x.unit == r.unit) nc = &x;
        if (nc == nullptr) {
          g_named.push_back(NamedClass{r.name, r.unit, 0.0, 0.0, 0});
          nc = &g_named.back();
        }
        nc->ms += ms;
        nc->work += r.work;
        nc->count += 1;
      }
    }
  });
}

int ctm_profile_kernel_count(int* count) {
  return guarded([&] {
    CTM_REQUIRE(count != nullptr, CTM_ERR_INVALID, "count is NULL");
    std::lock_guard<std::mutex> lk(g_mu);
    *count = static_cast<int>(g_named.size());
  });
}

int ctm_profile_kernel(int i, const char** name, int* unit, double* total_ms, double* total_work,
                       long long* launches) {
  return guarded([&] {
    std::lock_guard<std::mutex> lk(g_mu);
    CTM_REQUIRE(i >= 0 && i < static_cast<int>(g_named.size()), CTM_ERR_INVALID,
                "bad kernel-class index");
    const NamedClass& x = g_named[static_cast<size_t>(i)];
    if (name) *name = x.name.c_str();
    if (unit) *unit = x.unit;
    if (total_ms) *total_ms = x.ms;
    if (total_work) *total_work = x.work;
    if (launches) *launches = x.count;
  });
}

int ctm_profile_query(int tag, double* total_ms, double* total_work, long long* launches) {
  return guarded([&] {
    CTM_REQUIRE(tag >= 0 && tag < kProfileTags, CTM_ERR_INVALID, "bad profile tag");
    std::lock_guard<std::mutex> lk(g_mu);
    if (total_ms) *total_ms = g_ms[tag];
    if (total_work) *total_work = g_work[tag];
    if (launches) *launches = g_count[tag];
  });
}

}  // extern "C"
