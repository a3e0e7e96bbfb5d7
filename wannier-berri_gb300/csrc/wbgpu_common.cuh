// Common helpers for the wbgpu kernels (sm_103a).
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#define WBG_HD __host__ __device__ __forceinline__
#define WBG_D __device__ __forceinline__

// Status codes shared with include/wbgpu.h
#define WBG_OK 0
#define WBG_ERR_ARG 1
#define WBG_ERR_SIZE 2
#define WBG_ERR_CUDA 3
#define WBG_ERR_NOCONV 4
#define WBG_ERR_WORKSPACE 5

// Device-side error flags (bitmask) written by kernels into a caller-provided int.
#define WBG_FLAG_QL_NOCONV 1
#define WBG_FLAG_BOUNDS 2
#define WBG_FLAG_REFINE_WIDE 4  // refined eigensolver: a cluster wider than its Rayleigh-Ritz block

template <typename T> struct C2;
template <> struct C2<double> { typedef double2 t; };
template <> struct C2<float> { typedef float2 t; };

template <typename T> WBG_HD typename C2<T>::t mkc(T re, T im) {
  typename C2<T>::t r; r.x = re; r.y = im; return r;
}
template <typename V> WBG_HD V cadd(V a, V b) { a.x += b.x; a.y += b.y; return a; }
template <typename V> WBG_HD V csub(V a, V b) { a.x -= b.x; a.y -= b.y; return a; }
template <typename V> WBG_HD V cmul(V a, V b) {
  V r; r.x = a.x * b.x - a.y * b.y; r.y = a.x * b.y + a.y * b.x; return r;
}
// conj(a) * b
template <typename V> WBG_HD V cmulc(V a, V b) {
  V r; r.x = a.x * b.x + a.y * b.y; r.y = a.x * b.y - a.y * b.x; return r;
}
// acc += a * b
template <typename V> WBG_HD void cfma(V& acc, V a, V b) {
  acc.x = fma(a.x, b.x, acc.x); acc.x = fma(-a.y, b.y, acc.x);
  acc.y = fma(a.x, b.y, acc.y); acc.y = fma(a.y, b.x, acc.y);
}
// acc += conj(a) * b
template <typename V> WBG_HD void cfmac(V& acc, V a, V b) {
  acc.x = fma(a.x, b.x, acc.x); acc.x = fma(a.y, b.y, acc.x);
  acc.y = fma(a.x, b.y, acc.y); acc.y = fma(-a.y, b.x, acc.y);
}
template <typename V, typename S> WBG_HD V cscale(V a, S s) { a.x *= s; a.y *= s; return a; }
// i * a
template <typename V> WBG_HD V cmuli(V a) { V r; r.x = -a.y; r.y = a.x; return r; }
template <typename V> WBG_HD V cconj(V a) { a.y = -a.y; return a; }

template <typename T> struct CvtC;
WBG_HD float2 to_c32(double2 a) { return make_float2((float)a.x, (float)a.y); }
WBG_HD float2 to_c32(float2 a) { return a; }
WBG_HD double2 to_c64(float2 a) { return make_double2(a.x, a.y); }
WBG_HD double2 to_c64(double2 a) { return a; }

template <typename V> WBG_HD V czero() { V r; r.x = 0; r.y = 0; return r; }

// Records e as the library's last CUDA error (wbg_last_cuda_error_string) and returns WBG_ERR_CUDA.
int wbg_note_cuda_error(cudaError_t e);
static inline int wbg_cuda_status(cudaError_t e) { return e == cudaSuccess ? WBG_OK : wbg_note_cuda_error(e); }
