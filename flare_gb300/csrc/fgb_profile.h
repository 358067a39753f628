// Stage timer used around pipeline launches (see profile.cu).
#pragma once
#include <cuda_runtime.h>

namespace fgb {

enum Stage {
  kStNeighbors = 0,
  kStB2Forward,
  kStSpeciesPerm,
  kStKernelGemm,
  kStRowEnergy,
  kStAdjointGemm,
  kStVarianceGemm,
  kStVarianceFinal,
  kStB2Adjoint,
  kStForces,
  kStStructReduce,
  kStMappedGemm,
  kStPlainDervs,
  kStPlainEnvsStruc,
  kStOther,
  kStRowSlice,
  kNumStages
};

// RAII: records an event on `st` at construction and at destruction when
// the profiler is on.
class StageTimer {
 public:
  StageTimer(int stage, cudaStream_t st, int launches = 1);
  ~StageTimer();
  StageTimer(const StageTimer &) = delete;
  StageTimer &operator=(const StageTimer &) = delete;
  // the stage's kernel count when it is known only after its launches
  void set_launches(int n) { launches_ = n; }

 private:
  int stage_;
  int launches_;
  cudaStream_t st_;
  void *a_ = nullptr;
  bool active_ = false;
};

}  // namespace fgb
