// sqbem_cxx.hpp -- small C++ helpers shared by the drop-in headers: error
// translation from the C ABI status codes and the precision selection.
#pragma once
#include <cstdlib>
#include <cstring>
#include <memory>
#include <stdexcept>
#include <string>
#include "sqbem.h"

namespace bem {

// Precision used by the drop-in classes when none is given explicitly:
// SQBEM_PRECISION=mixed selects the split-BF16 tensor-core path with FP64
// refinement, anything else the FP64 path (the reference's results to 1e-10).
inline int default_precision() {
    const char* p = std::getenv("SQBEM_PRECISION");
    return (p && std::strcmp(p, "mixed") == 0) ? SQBEM_MIXED : SQBEM_FP64;
}

// Throw the library's message (e.g. "dgetrf failed") as the reference does.
inline void check(int status) {
    if (status != SQBEM_OK) throw std::runtime_error(sqbem_last_error());
}

}  // namespace bem
