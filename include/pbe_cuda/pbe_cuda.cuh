// pbe_cuda/pbe_cuda.cuh -- umbrella header of the C++ drop-in API
// (mirrors acuoci/pbe-fixed-pivot-cuda include/pbe_cuda/pbe_cuda.cuh:17-18).
#pragma once

#include "pbe_cuda/aggregation.cuh"
#include "pbe_cuda/breakage.cuh"
