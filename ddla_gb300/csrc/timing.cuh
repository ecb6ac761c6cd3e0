// Kernel-class timing hooks (see timing.cu).
#pragma once
#include <cuda_runtime.h>

namespace ddla {

enum TimingClass { TC_UPDATE = 0, TC_PANEL = 1, TC_TRSM = 2, TC_LASWP = 3, TC_REFINE = 4, TC_BATCHED = 5,
                   TC_CONTRACT = 6, TC_QR_T = 7, TC_SOLVE = 8, TC_BD_BAND = 9, TC_BD_CHASE = 10,
                   TC_BD_BACK = 11, TC_COUNT = 12 };

bool timing_on();

// Brackets the launches issued during its lifetime with CUDA events.
class Timed {
  public:
    Timed(cudaStream_t s, int cls, double flops, double bytes);
    ~Timed();

  private:
    cudaStream_t s_;
    int idx_;
};

}  // namespace ddla
