// cplx.h -- device complex helpers for double2 (FP64 path) and float2 (mixed path).
#pragma once

#include <cuda_runtime.h>

namespace cqpi {

template <class C> struct real_of;
template <> struct real_of<double2> { using type = double; };
template <> struct real_of<float2> { using type = float; };

template <class C> __device__ __forceinline__ C cmake(double re, double im);
template <> __device__ __forceinline__ double2 cmake<double2>(double re, double im) { return make_double2(re, im); }
template <> __device__ __forceinline__ float2 cmake<float2>(double re, double im) { return make_float2((float)re, (float)im); }

__device__ __forceinline__ double2 cmul(double2 a, double2 b) { return make_double2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x); }
__device__ __forceinline__ float2 cmul(float2 a, float2 b) { return make_float2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x); }
__device__ __forceinline__ double2 cadd(double2 a, double2 b) { return make_double2(a.x + b.x, a.y + b.y); }
__device__ __forceinline__ float2 cadd(float2 a, float2 b) { return make_float2(a.x + b.x, a.y + b.y); }
__device__ __forceinline__ double2 csub(double2 a, double2 b) { return make_double2(a.x - b.x, a.y - b.y); }
__device__ __forceinline__ float2 csub(float2 a, float2 b) { return make_float2(a.x - b.x, a.y - b.y); }
__device__ __forceinline__ double2 cscale(double2 a, double s) { return make_double2(a.x * s, a.y * s); }
__device__ __forceinline__ float2 cscale(float2 a, float s) { return make_float2(a.x * s, a.y * s); }
__device__ __forceinline__ double2 to_d2(double2 a) { return a; }
__device__ __forceinline__ double2 to_d2(float2 a) { return make_double2((double)a.x, (double)a.y); }

}  // namespace cqpi
