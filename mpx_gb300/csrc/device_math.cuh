// Device scalar helpers: a forward-mode dual number (value + one tangent) so
// that one warp lane evaluates one directional derivative of a model, i.e.
// one column of its Jacobian, and the SRBD models written once over the
// scalar type S (float or DF).
#pragma once
#include <cuda_runtime.h>

namespace mpxg {

struct DF {
  float v, d;
};

__device__ __forceinline__ DF mkd(float v, float d) { DF r; r.v = v; r.d = d; return r; }
__device__ __forceinline__ DF operator+(DF a, DF b) { return mkd(a.v + b.v, a.d + b.d); }
__device__ __forceinline__ DF operator-(DF a, DF b) { return mkd(a.v - b.v, a.d - b.d); }
__device__ __forceinline__ DF operator-(DF a) { return mkd(-a.v, -a.d); }
__device__ __forceinline__ DF operator*(DF a, DF b) { return mkd(a.v * b.v, a.d * b.v + a.v * b.d); }
__device__ __forceinline__ DF operator/(DF a, DF b) {
  float q = a.v / b.v;
  return mkd(q, (a.d - q * b.d) / b.v);
}
__device__ __forceinline__ DF operator+(DF a, float b) { return mkd(a.v + b, a.d); }
__device__ __forceinline__ DF operator+(float b, DF a) { return mkd(a.v + b, a.d); }
__device__ __forceinline__ DF operator-(DF a, float b) { return mkd(a.v - b, a.d); }
__device__ __forceinline__ DF operator-(float b, DF a) { return mkd(b - a.v, -a.d); }
__device__ __forceinline__ DF operator*(DF a, float b) { return mkd(a.v * b, a.d * b); }
__device__ __forceinline__ DF operator*(float b, DF a) { return mkd(a.v * b, a.d * b); }
__device__ __forceinline__ DF operator/(DF a, float b) { return mkd(a.v / b, a.d / b); }
__device__ __forceinline__ DF operator/(float b, DF a) {
  float q = b / a.v;
  return mkd(q, -q * a.d / a.v);
}

__device__ __forceinline__ float sval(float x) { return x; }
__device__ __forceinline__ float sval(DF x) { return x.v; }
__device__ __forceinline__ float sder(float) { return 0.0f; }
__device__ __forceinline__ float sder(DF x) { return x.d; }

__device__ __forceinline__ float s_sqrt(float x) { return sqrtf(x); }
__device__ __forceinline__ DF s_sqrt(DF x) {
  float s = sqrtf(x.v);
  return mkd(s, x.d * (0.5f / s));
}
__device__ __forceinline__ void s_sincos(float x, float* s, float* c) { sincosf(x, s, c); }
__device__ __forceinline__ void s_sincos(DF x, DF* s, DF* c) {
  float sv, cv;
  sincosf(x.v, &sv, &cv);
  *s = mkd(sv, cv * x.d);
  *c = mkd(cv, -sv * x.d);
}
__device__ __forceinline__ float s_tan(float x) { return tanf(x); }
__device__ __forceinline__ DF s_tan(DF x) {
  float t = tanf(x.v);
  return mkd(t, x.d * (1.0f + t * t));
}
__device__ __forceinline__ float s_atan2(float y, float x) { return atan2f(y, x); }
__device__ __forceinline__ DF s_atan2(DF y, DF x) {
  float den = x.v * x.v + y.v * y.v;
  return mkd(atan2f(y.v, x.v), (x.v * y.d - y.v * x.d) / den);
}
__device__ __forceinline__ float s_log(float x) { return logf(x); }
__device__ __forceinline__ DF s_log(DF x) { return mkd(logf(x.v), x.d / x.v); }

template <class S> __device__ __forceinline__ S s_const(float v);
template <> __device__ __forceinline__ float s_const<float>(float v) { return v; }
template <> __device__ __forceinline__ DF s_const<DF>(float v) { return mkd(v, 0.0f); }

template <class S> __device__ __forceinline__ S seed(float v, bool on);
template <> __device__ __forceinline__ float seed<float>(float v, bool) { return v; }
template <> __device__ __forceinline__ DF seed<DF>(float v, bool on) { return mkd(v, on ? 1.0f : 0.0f); }

// ------------------------------------------------------------ warp helpers
__device__ __forceinline__ float warp_sum(float v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}
__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}
__device__ __forceinline__ float warp_max(float v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v = fmaxf(v, __shfl_xor_sync(0xffffffffu, v, o));
  return v;
}
__device__ __forceinline__ int warp_or(int v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v |= __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

}  // namespace mpxg

namespace mpxg {

// Forward-mode dual number with K tangents: one lane propagates K directional
// derivatives at once (K columns of a Jacobian per model evaluation).
template <int K>
struct DK {
  float v;
  float d[K];
};
template <int K> __device__ __forceinline__ DK<K> dk_const(float v) {
  DK<K> r; r.v = v;
#pragma unroll
  for (int k = 0; k < K; ++k) r.d[k] = 0.0f;
  return r;
}
template <int K> __device__ __forceinline__ DK<K> operator+(const DK<K>& a, const DK<K>& b) {
  DK<K> r; r.v = a.v + b.v;
#pragma unroll
  for (int k = 0; k < K; ++k) r.d[k] = a.d[k] + b.d[k];
  return r;
}
template <int K> __device__ __forceinline__ DK<K> operator-(const DK<K>& a, const DK<K>& b) {
  DK<K> r; r.v = a.v - b.v;
#pragma unroll
  for (int k = 0; k < K; ++k) r.d[k] = a.d[k] - b.d[k];
  return r;
}
template <int K> __device__ __forceinline__ DK<K> operator-(const DK<K>& a) {
  DK<K> r; r.v = -a.v;
#pragma unroll
  for (int k = 0; k < K; ++k) r.d[k] = -a.d[k];
  return r;
}
template <int K> __device__ __forceinline__ DK<K> operator*(const DK<K>& a, const DK<K>& b) {
  DK<K> r; r.v = a.v * b.v;
#pragma unroll
  for (int k = 0; k < K; ++k) r.d[k] = a.d[k] * b.v + a.v * b.d[k];
  return r;
}
template <int K> __device__ __forceinline__ DK<K> operator/(const DK<K>& a, const DK<K>& b) {
  DK<K> r;
  const float ib = 1.0f / b.v;
  r.v = a.v * ib;
#pragma unroll
  for (int k = 0; k < K; ++k) r.d[k] = (a.d[k] - r.v * b.d[k]) * ib;
  return r;
}
template <int K> __device__ __forceinline__ DK<K> operator+(const DK<K>& a, float b) { DK<K> r = a; r.v += b; return r; }
template <int K> __device__ __forceinline__ DK<K> operator+(float b, const DK<K>& a) { DK<K> r = a; r.v += b; return r; }
template <int K> __device__ __forceinline__ DK<K> operator-(const DK<K>& a, float b) { DK<K> r = a; r.v -= b; return r; }
template <int K> __device__ __forceinline__ DK<K> operator-(float b, const DK<K>& a) {
  DK<K> r; r.v = b - a.v;
#pragma unroll
  for (int k = 0; k < K; ++k) r.d[k] = -a.d[k];
  return r;
}
template <int K> __device__ __forceinline__ DK<K> operator*(const DK<K>& a, float b) {
  DK<K> r; r.v = a.v * b;
#pragma unroll
  for (int k = 0; k < K; ++k) r.d[k] = a.d[k] * b;
  return r;
}
template <int K> __device__ __forceinline__ DK<K> operator*(float b, const DK<K>& a) { return a * b; }
template <int K> __device__ __forceinline__ DK<K> operator/(const DK<K>& a, float b) { return a * (1.0f / b); }
template <int K> __device__ __forceinline__ DK<K> operator/(float b, const DK<K>& a) {
  DK<K> r; r.v = b / a.v;
  const float s = -r.v / a.v;
#pragma unroll
  for (int k = 0; k < K; ++k) r.d[k] = s * a.d[k];
  return r;
}
template <int K> __device__ __forceinline__ float sval(const DK<K>& x) { return x.v; }
template <int K> __device__ __forceinline__ DK<K> s_sqrt(const DK<K>& x) {
  DK<K> r; r.v = sqrtf(x.v);
  const float s = 0.5f / r.v;
#pragma unroll
  for (int k = 0; k < K; ++k) r.d[k] = x.d[k] * s;
  return r;
}
template <int K> __device__ __forceinline__ void s_sincos(const DK<K>& x, DK<K>* s, DK<K>* c) {
  float sv, cv;
  sincosf(x.v, &sv, &cv);
  s->v = sv; c->v = cv;
#pragma unroll
  for (int k = 0; k < K; ++k) { s->d[k] = cv * x.d[k]; c->d[k] = -sv * x.d[k]; }
}
template <int K> __device__ __forceinline__ DK<K> s_atan2(const DK<K>& y, const DK<K>& x) {
  DK<K> r; r.v = atan2f(y.v, x.v);
  const float den = 1.0f / (x.v * x.v + y.v * y.v);
#pragma unroll
  for (int k = 0; k < K; ++k) r.d[k] = (x.v * y.d[k] - y.v * x.d[k]) * den;
  return r;
}
template <int K> __device__ __forceinline__ DK<K> s_log(const DK<K>& x) {
  DK<K> r; r.v = logf(x.v);
  const float s = 1.0f / x.v;
#pragma unroll
  for (int k = 0; k < K; ++k) r.d[k] = x.d[k] * s;
  return r;
}
template <> __device__ __forceinline__ DK<1> s_const<DK<1>>(float v) { return dk_const<1>(v); }
template <> __device__ __forceinline__ DK<2> s_const<DK<2>>(float v) { return dk_const<2>(v); }
template <> __device__ __forceinline__ DK<3> s_const<DK<3>>(float v) { return dk_const<3>(v); }
template <> __device__ __forceinline__ DK<4> s_const<DK<4>>(float v) { return dk_const<4>(v); }

}  // namespace mpxg
