// geom_math.cuh — small vector helpers templated on the real type, usable
// from host and device code.
#pragma once
#include <cuda_runtime.h>
#include <math.h>

namespace hc {

template <class R>
struct V3 {
  R x, y, z;
};

template <class R>
__host__ __device__ __forceinline__ V3<R> mk(R x, R y, R z) {
  V3<R> v;
  v.x = x; v.y = y; v.z = z;
  return v;
}
template <class R>
__host__ __device__ __forceinline__ V3<R> operator+(V3<R> a, V3<R> b) { return mk(a.x + b.x, a.y + b.y, a.z + b.z); }
template <class R>
__host__ __device__ __forceinline__ V3<R> operator-(V3<R> a, V3<R> b) { return mk(a.x - b.x, a.y - b.y, a.z - b.z); }
template <class R>
__host__ __device__ __forceinline__ V3<R> operator*(V3<R> a, R s) { return mk(a.x * s, a.y * s, a.z * s); }
template <class R>
__host__ __device__ __forceinline__ R dot(V3<R> a, V3<R> b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
template <class R>
__host__ __device__ __forceinline__ V3<R> cross(V3<R> a, V3<R> b) {
  return mk(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x);
}
template <class R>
__host__ __device__ __forceinline__ R amax(V3<R> a) {
  R x = a.x < 0 ? -a.x : a.x, y = a.y < 0 ? -a.y : a.y, z = a.z < 0 ? -a.z : a.z;
  return x > y ? (x > z ? x : z) : (y > z ? y : z);
}
__host__ __device__ __forceinline__ float rsqrt_r(float x) { return 1.0f / sqrtf(x); }
__host__ __device__ __forceinline__ double rsqrt_r(double x) { return 1.0 / sqrt(x); }
__host__ __device__ __forceinline__ float sqrt_r(float x) { return sqrtf(x); }
__host__ __device__ __forceinline__ double sqrt_r(double x) { return sqrt(x); }
__host__ __device__ __forceinline__ float abs_r(float x) { return fabsf(x); }
__host__ __device__ __forceinline__ double abs_r(double x) { return fabs(x); }

template <class R>
__host__ __device__ __forceinline__ R norm(V3<R> a) { return sqrt_r(dot(a, a)); }

// y = R x for a row-major 3x3.
template <class R, class M>
__host__ __device__ __forceinline__ V3<R> mat_mul(const M* m, V3<R> a) {
  return mk<R>((R)m[0] * a.x + (R)m[1] * a.y + (R)m[2] * a.z, (R)m[3] * a.x + (R)m[4] * a.y + (R)m[5] * a.z,
               (R)m[6] * a.x + (R)m[7] * a.y + (R)m[8] * a.z);
}
// y = R^T x.
template <class R, class M>
__host__ __device__ __forceinline__ V3<R> mat_tmul(const M* m, V3<R> a) {
  return mk<R>((R)m[0] * a.x + (R)m[3] * a.y + (R)m[6] * a.z, (R)m[1] * a.x + (R)m[4] * a.y + (R)m[7] * a.z,
               (R)m[2] * a.x + (R)m[5] * a.y + (R)m[8] * a.z);
}

}  // namespace hc
