// Stage profiler: CUDA events around each pipeline launch, on the launch
// stream, read back on request.  Off by default; costs nothing when off.
#include <mutex>
#include <vector>

#include "fgb_internal.h"
#include "fgb_profile.h"

namespace fgb {
namespace {

const char *kNames[kNumStages] = {
    "neighbors",      "b2_forward",     "species_perm",  "kernel_gemm",
    "row_energy",     "adjoint_gemm",   "variance_gemm", "variance_final",
    "b2_adjoint",     "forces",         "struct_reduce", "mapped_gemm",
    "plain_dervs",    "plain_envs_struc", "other",       "row_slice"};

struct Pending {
  int stage;
  int launches;
  cudaEvent_t a, b;
};

struct Prof {
  bool on = false;
  std::mutex mu;
  std::vector<Pending> pending;
  std::vector<cudaEvent_t> pool;
  double ms[kNumStages] = {0};
  long long n[kNumStages] = {0};
};

Prof &prof() {
  static Prof p;
  return p;
}

cudaEvent_t get_event(Prof &p) {
  if (!p.pool.empty()) {
    cudaEvent_t e = p.pool.back();
    p.pool.pop_back();
    return e;
  }
  cudaEvent_t e = nullptr;
  cudaEventCreate(&e);
  return e;
}

void drain(Prof &p) {
  for (auto &q : p.pending) {
    cudaEventSynchronize(q.b);
    float t = 0.f;
    cudaEventElapsedTime(&t, q.a, q.b);
    p.ms[q.stage] += t;
    p.n[q.stage] += q.launches;
    p.pool.push_back(q.a);
    p.pool.push_back(q.b);
  }
  p.pending.clear();
}

}  // namespace

StageTimer::StageTimer(int stage, cudaStream_t st, int launches)
    : stage_(stage), launches_(launches), st_(st) {
  Prof &p = prof();
  if (!p.on) return;
  // launches captured into a graph are not timed (their events would be
  // graph dependencies, not timestamps)
  cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
  if (cudaStreamIsCapturing(st_, &cs) != cudaSuccess ||
      cs != cudaStreamCaptureStatusNone)
    return;
  std::lock_guard<std::mutex> g(p.mu);
  a_ = get_event(p);
  cudaEventRecord((cudaEvent_t)a_, st_);
  active_ = true;
}

StageTimer::~StageTimer() {
  if (!active_) return;
  Prof &p = prof();
  std::lock_guard<std::mutex> g(p.mu);
  cudaEvent_t b = get_event(p);
  cudaEventRecord(b, st_);
  p.pending.push_back({stage_, launches_, (cudaEvent_t)a_, b});
  if (p.pending.size() > 4096) drain(p);
}

}  // namespace fgb

using namespace fgb;

extern "C" int fgb_profile_enable(int on) {
  Prof &p = prof();
  std::lock_guard<std::mutex> g(p.mu);
  p.on = on != 0;
  return FGB_OK;
}

extern "C" int fgb_profile_reset(void) {
  Prof &p = prof();
  std::lock_guard<std::mutex> g(p.mu);
  drain(p);
  for (int i = 0; i < kNumStages; i++) { p.ms[i] = 0; p.n[i] = 0; }
  return FGB_OK;
}

extern "C" int fgb_profile_n_stages(void) { return kNumStages; }

extern "C" const char *fgb_profile_stage_name(int stage) {
  if (stage < 0 || stage >= kNumStages) return "";
  return kNames[stage];
}

extern "C" int fgb_profile_read(double *ms, long long *launches, int n) {
  Prof &p = prof();
  std::lock_guard<std::mutex> g(p.mu);
  drain(p);
  for (int i = 0; i < n && i < kNumStages; i++) {
    if (ms) ms[i] = p.ms[i];
    if (launches) launches[i] = p.n[i];
  }
  return FGB_OK;
}
