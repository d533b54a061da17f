// Minimal complex arithmetic for the FFT kernels (FP32 or FP64 scalars).
#pragma once
#include <cuda_runtime.h>

template <typename T>
struct __align__(2 * sizeof(T)) cplx {
  T x, y;
};

template <typename T>
__device__ __forceinline__ cplx<T> operator+(cplx<T> a, cplx<T> b) {
  return cplx<T>{a.x + b.x, a.y + b.y};
}
template <typename T>
__device__ __forceinline__ cplx<T> operator-(cplx<T> a, cplx<T> b) {
  return cplx<T>{a.x - b.x, a.y - b.y};
}
template <typename T>
__device__ __forceinline__ cplx<T> cmul(cplx<T> a, cplx<T> b) {
  return cplx<T>{a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x};
}
// a * conj(b)
template <typename T>
__device__ __forceinline__ cplx<T> cmulc(cplx<T> a, cplx<T> b) {
  return cplx<T>{a.x * b.x + a.y * b.y, a.y * b.x - a.x * b.y};
}
template <typename T>
__device__ __forceinline__ cplx<T> cconj(cplx<T> a) {
  return cplx<T>{a.x, -a.y};
}
template <typename T>
__device__ __forceinline__ cplx<T> cscale(cplx<T> a, T s) {
  return cplx<T>{a.x * s, a.y * s};
}
