// CUDA runtime status -> ath::Error.
#pragma once

#include <cuda_runtime.h>

#include <string>

#include "errors.hpp"

namespace ath {

inline void Check(cudaError_t e, const char *what) {
  if (e != cudaSuccess)
    throw Error(ATH_ERR_CUDA, std::string(what) + ": " + cudaGetErrorString(e));
}

}  // namespace ath
