// mixed.cuh -- mixed-precision (split-BF16 tensor-core + FP64 refinement) state.
#pragma once
#include "common.cuh"

namespace sqbem {

struct MixedLU {
    int n = 0;
};

struct MixedSwimmer {
    int built = 0;
};

}  // namespace sqbem
