// Precision-typed math for templated device code. Each helper is overloaded
// for float and double and calls the function of that precision explicitly,
// so FP32 code never promotes to double (a promoted call such as round(float)
// would run on the FP64 pipe, which is narrow on GB300).
#pragma once

namespace smpc {

__device__ __forceinline__ float r_round(float x) { return roundf(x); }
__device__ __forceinline__ double r_round(double x) { return ::round(x); }
__device__ __forceinline__ float r_sqrt(float x) { return sqrtf(x); }
__device__ __forceinline__ double r_sqrt(double x) { return ::sqrt(x); }
__device__ __forceinline__ float r_log(float x) { return logf(x); }
__device__ __forceinline__ double r_log(double x) { return ::log(x); }
__device__ __forceinline__ float r_cos(float x) { return cosf(x); }
__device__ __forceinline__ double r_cos(double x) { return ::cos(x); }
__device__ __forceinline__ void r_sincos(float x, float* s, float* c) { sincosf(x, s, c); }
__device__ __forceinline__ void r_sincos(double x, double* s, double* c) { ::sincos(x, s, c); }
__device__ __forceinline__ float r_fabs(float x) { return fabsf(x); }
__device__ __forceinline__ double r_fabs(double x) { return ::fabs(x); }
__device__ __forceinline__ bool r_isfinite(float x) { return isfinite(x); }
__device__ __forceinline__ bool r_isfinite(double x) { return isfinite(x); }

}  // namespace smpc
