// Comparisons of FP64 values on the integer pipe, with the selection semantics
// of the FP comparison they replace (GB300 issues FP64 compares on its FP64
// pipe, at 1/64 of the FP32 rate).  Valid for all non-NaN operands; -0 and +0
// compare equal, as in IEEE arithmetic.
#pragma once

#include <cuda_runtime.h>

namespace mom5 {
namespace sel {

// order-preserving integer image of a double, with -0 mapped onto +0
__device__ __forceinline__ long long ord0(double x) {
  long long b = __double_as_longlong(x);
  b = b == (long long)0x8000000000000000ULL ? 0 : b;
  return b ^ ((b >> 63) & 0x7fffffffffffffffLL);
}
// a < b ? a : b  and  a > b ? a : b
__device__ __forceinline__ double lt_min(double a, double b) { return ord0(a) < ord0(b) ? a : b; }
__device__ __forceinline__ double gt_max(double a, double b) { return ord0(a) > ord0(b) ? a : b; }
// x > 0, x < 0, x >= 0
__device__ __forceinline__ bool gt0(double x) { return __double_as_longlong(x) > 0; }
__device__ __forceinline__ bool lt0(double x) { return ord0(x) < 0; }
__device__ __forceinline__ bool ge0(double x) { return ord0(x) >= 0; }

}  // namespace sel
}  // namespace mom5
