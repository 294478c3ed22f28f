// aloha_owl_shim.h -- host stand-ins for the parts of OWL, OptiX and the CUDA
// runtime that the reference's device code (deviceCode.cpp / deviceCode.h)
// and its chopSuey tool (chopSuey.cpp, volume.h, mesh.h) use, so that those
// reference sources compile unchanged as CPU code.
//
// TEST INFRASTRUCTURE ONLY.  The reference's own CPU build (ALOHA_CPU) gets
// the same pieces from OWL and fakeOwl, which are git submodules that are not
// vendored with the reference; this file is a small restatement of the
// interfaces those sources call, written for this project:
//   * vector / box / interval math with the member names and operators the
//     reference uses (owl::common::vec_t, box_t, interval);
//   * OptiX device calls (launch index, payload, program data, intersection
//     reporting, traversal) answered by the harness (oracle/ref_harness.cpp),
//     which emulates closest-hit traversal over a rank's bricks;
//   * CUDA texture fetches tex3D / tex1D with the semantics the reference
//     configures (waikikiRenderer.cpp:715-775 volume: normalized coordinates,
//     linear filter, clamp; 964-1008 transfer function: normalized
//     coordinates, linear filter, border colour 0), evaluated with exact fp32
//     weights in the harness;
//   * owl::common::LCG<4> (the jitter source, deviceCode.cpp:12,354,386):
//     its draws come from the harness, which hands out the jitter the run is
//     configured with (none, a constant, or this project's documented hash of
//     pixel, accumID and draw index), because owl's generator is not vendored;
//   * make_rgba (deviceCode.cpp:416): round to nearest of clamp(x,0,1)*255,
//     this project's documented choice (owl's is not vendored).
#pragma once

#include <algorithm>
#include <cfloat>
#include <climits>
#include <cmath>
#include <cstdint>
#include <cstdlib>
#include <iostream>
#include <memory>
#include <numeric>
#include <string>
#include <vector>

// ---------------------------------------------------------------- CUDA
#define __device__
#define __host__
#define __global__
#define __constant__
#define __forceinline__ inline
#define __both__

struct float2 { float x, y; };
struct float3 { float x, y, z; };
struct float4 { float x, y, z, w; };
struct uint3 { unsigned x, y, z; };
inline float4 make_float4(float x, float y, float z, float w) { return float4{x, y, z, w}; }

typedef unsigned long long cudaTextureObject_t;
typedef unsigned long long OptixTraversableHandle;

// Answered by the harness.
float aloha_ref_tex3D(cudaTextureObject_t tex, float x, float y, float z);
float4 aloha_ref_tex1D(cudaTextureObject_t tex, float x);
long long aloha_ref_clock();

template <class T> T tex3D(cudaTextureObject_t tex, float x, float y, float z);
template <> inline float tex3D<float>(cudaTextureObject_t tex, float x, float y, float z) {
  return aloha_ref_tex3D(tex, x, y, z);
}
template <class T> T tex1D(cudaTextureObject_t tex, float x);
template <> inline float4 tex1D<float4>(cudaTextureObject_t tex, float x) { return aloha_ref_tex1D(tex, x); }
inline long long clock64() { return aloha_ref_clock(); }

// ---------------------------------------------------------------- OptiX
#define OPTIX_RAYGEN_PROGRAM(name) void optix_raygen_##name
#define OPTIX_INTERSECT_PROGRAM(name) void optix_isect_##name
#define OPTIX_CLOSEST_HIT_PROGRAM(name) void optix_ch_##name
#define OPTIX_BOUNDS_PROGRAM(name) void optix_bounds_##name
#define OPTIX_RAY_FLAG_DISABLE_ANYHIT 1u

unsigned optixGetPrimitiveIndex();
float3 optixGetObjectRayOrigin();
float3 optixGetObjectRayDirection();
float optixGetRayTmin();
float optixGetRayTmax();
bool optixReportIntersection(float t, unsigned kind);
uint3 optixGetLaunchDimensions();

#define OWL_TERMINAL_RED "\033[1;31m"
#define OWL_TERMINAL_DEFAULT "\033[0m"

namespace owl {
namespace common {

// ------------------------------------------------------------ vectors
template <class T> struct vec4;

template <class T> struct vec2 {
  union { T x; T u; };
  union { T y; T v; };
  vec2() {}
  vec2(T s) : x(s), y(s) {}
  vec2(T a, T b) : x(a), y(b) {}
  template <class O> explicit vec2(const vec2<O>& o) : x((T)o.x), y((T)o.y) {}
  T& operator[](int i) { return i == 0 ? x : y; }
  const T& operator[](int i) const { return i == 0 ? x : y; }
};

template <class T> struct vec3 {
  T x, y, z;
  vec3() {}
  vec3(T s) : x(s), y(s), z(s) {}
  vec3(T a, T b, T c) : x(a), y(b), z(c) {}
  template <class O> explicit vec3(const vec3<O>& o) : x((T)o.x), y((T)o.y), z((T)o.z) {}
  explicit vec3(const vec4<T>& o);
  vec3(const float3& f) : x((T)f.x), y((T)f.y), z((T)f.z) {}
  T& operator[](int i) { return i == 0 ? x : (i == 1 ? y : z); }
  const T& operator[](int i) const { return i == 0 ? x : (i == 1 ? y : z); }
};

template <class T> struct vec4 {
  T x, y, z, w;
  vec4() {}
  vec4(T s) : x(s), y(s), z(s), w(s) {}
  vec4(T a, T b, T c, T d) : x(a), y(b), z(c), w(d) {}
  vec4(const vec3<T>& v, T d) : x(v.x), y(v.y), z(v.z), w(d) {}
  vec4(const float4& f) : x((T)f.x), y((T)f.y), z((T)f.z), w((T)f.w) {}
  operator float4() const { return float4{(float)x, (float)y, (float)z, (float)w}; }
  T& operator[](int i) { return i == 0 ? x : (i == 1 ? y : (i == 2 ? z : w)); }
  const T& operator[](int i) const { return i == 0 ? x : (i == 1 ? y : (i == 2 ? z : w)); }
};

template <class T> vec3<T>::vec3(const vec4<T>& o) : x(o.x), y(o.y), z(o.z) {}

typedef vec2<int> vec2i;
typedef vec2<float> vec2f;
typedef vec3<int> vec3i;
typedef vec3<float> vec3f;
typedef vec4<float> vec4f;

// Component-wise arithmetic: vector-vector (the right operand converted to
// the left one's element type, as `vec3f -= vec3i` needs), vector-scalar and
// scalar-vector.
#define ALOHA_SHIM_VEC_OPS(OP, OPEQ)                                                                   \
  template <class T> vec2<T> operator OP(const vec2<T>& a, const vec2<T>& b) {                        \
    return vec2<T>(a.x OP b.x, a.y OP b.y);                                                            \
  }                                                                                                    \
  template <class T> vec3<T> operator OP(const vec3<T>& a, const vec3<T>& b) {                        \
    return vec3<T>(a.x OP b.x, a.y OP b.y, a.z OP b.z);                                                \
  }                                                                                                    \
  template <class T> vec4<T> operator OP(const vec4<T>& a, const vec4<T>& b) {                        \
    return vec4<T>(a.x OP b.x, a.y OP b.y, a.z OP b.z, a.w OP b.w);                                    \
  }                                                                                                    \
  template <class T> vec2<T> operator OP(const vec2<T>& a, T s) { return vec2<T>(a.x OP s, a.y OP s); } \
  template <class T> vec3<T> operator OP(const vec3<T>& a, T s) {                                     \
    return vec3<T>(a.x OP s, a.y OP s, a.z OP s);                                                      \
  }                                                                                                    \
  template <class T> vec4<T> operator OP(const vec4<T>& a, T s) {                                     \
    return vec4<T>(a.x OP s, a.y OP s, a.z OP s, a.w OP s);                                            \
  }                                                                                                    \
  template <class T> vec2<T> operator OP(T s, const vec2<T>& a) { return vec2<T>(s OP a.x, s OP a.y); } \
  template <class T> vec3<T> operator OP(T s, const vec3<T>& a) {                                     \
    return vec3<T>(s OP a.x, s OP a.y, s OP a.z);                                                      \
  }                                                                                                    \
  template <class T> vec4<T> operator OP(T s, const vec4<T>& a) {                                     \
    return vec4<T>(s OP a.x, s OP a.y, s OP a.z, s OP a.w);                                            \
  }                                                                                                    \
  template <class T, class O> vec3<T>& operator OPEQ(vec3<T>& a, const vec3<O>& b) {                  \
    a.x = a.x OP (T)b.x;                                                                               \
    a.y = a.y OP (T)b.y;                                                                               \
    a.z = a.z OP (T)b.z;                                                                               \
    return a;                                                                                          \
  }                                                                                                    \
  template <class T, class O> vec4<T>& operator OPEQ(vec4<T>& a, const vec4<O>& b) {                  \
    a.x = a.x OP (T)b.x;                                                                               \
    a.y = a.y OP (T)b.y;                                                                               \
    a.z = a.z OP (T)b.z;                                                                               \
    a.w = a.w OP (T)b.w;                                                                               \
    return a;                                                                                          \
  }                                                                                                    \
  template <class T> vec3<T>& operator OPEQ(vec3<T>& a, T s) {                                        \
    a.x = a.x OP s;                                                                                    \
    a.y = a.y OP s;                                                                                    \
    a.z = a.z OP s;                                                                                    \
    return a;                                                                                          \
  }                                                                                                    \
  template <class T> vec4<T>& operator OPEQ(vec4<T>& a, T s) {                                        \
    a.x = a.x OP s;                                                                                    \
    a.y = a.y OP s;                                                                                    \
    a.z = a.z OP s;                                                                                    \
    a.w = a.w OP s;                                                                                    \
    return a;                                                                                          \
  }

ALOHA_SHIM_VEC_OPS(+, +=)
ALOHA_SHIM_VEC_OPS(-, -=)
ALOHA_SHIM_VEC_OPS(*, *=)
ALOHA_SHIM_VEC_OPS(/, /=)
#undef ALOHA_SHIM_VEC_OPS

template <class T> vec3<T> operator-(const vec3<T>& a) { return vec3<T>(-a.x, -a.y, -a.z); }
template <class T> bool operator==(const vec2<T>& a, const vec2<T>& b) { return a.x == b.x && a.y == b.y; }
template <class T> bool operator!=(const vec2<T>& a, const vec2<T>& b) { return !(a == b); }
template <class T> bool operator==(const vec3<T>& a, const vec3<T>& b) {
  return a.x == b.x && a.y == b.y && a.z == b.z;
}
template <class T> bool operator!=(const vec3<T>& a, const vec3<T>& b) { return !(a == b); }

inline float min(float a, float b) { return a < b ? a : b; }
inline float max(float a, float b) { return a > b ? a : b; }
inline int min(int a, int b) { return a < b ? a : b; }
inline int max(int a, int b) { return a > b ? a : b; }
template <class T> vec3<T> min(const vec3<T>& a, const vec3<T>& b) {
  return vec3<T>(a.x < b.x ? a.x : b.x, a.y < b.y ? a.y : b.y, a.z < b.z ? a.z : b.z);
}
template <class T> vec3<T> max(const vec3<T>& a, const vec3<T>& b) {
  return vec3<T>(a.x > b.x ? a.x : b.x, a.y > b.y ? a.y : b.y, a.z > b.z ? a.z : b.z);
}
template <class T> T reduce_min(const vec3<T>& a) { return min(min(a.x, a.y), a.z); }
template <class T> T reduce_max(const vec3<T>& a) { return max(max(a.x, a.y), a.z); }
template <class T> T dot(const vec3<T>& a, const vec3<T>& b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
template <class T> vec3<T> cross(const vec3<T>& a, const vec3<T>& b) {
  return vec3<T>(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x);
}
inline float length(const vec3f& a) { return std::sqrt(dot(a, a)); }
inline vec3f normalize(const vec3f& a) { return a * (1.f / std::sqrt(dot(a, a))); }
inline float saturate(float f) { return std::fmin(std::fmax(f, 0.f), 1.f); }

template <class T> std::ostream& operator<<(std::ostream& o, const vec3<T>& v) {
  return o << '(' << v.x << ',' << v.y << ',' << v.z << ')';
}

// --------------------------------------------------------- boxes, intervals
template <class T> struct box3 {
  vec3<T> lower, upper;
  vec3<T> size() const { return upper - lower; }
  vec3<T> center() const { return (lower + upper) / (T)2; }
  T volume() const {
    const vec3<T> s = size();
    return s.x * s.y * s.z;
  }
  box3& extend(const vec3<T>& p) {
    lower = min(lower, p);
    upper = max(upper, p);
    return *this;
  }
  box3& extend(const box3& b) {
    lower = min(lower, b.lower);
    upper = max(upper, b.upper);
    return *this;
  }
};
typedef box3<int> box3i;
typedef box3<float> box3f;

template <class T> std::ostream& operator<<(std::ostream& o, const box3<T>& b) {
  return o << '{' << b.lower << ',' << b.upper << '}';
}

template <class T> struct interval {
  T lower, upper;
  interval() {}
  interval(T lo, T hi) : lower(lo), upper(hi) {}
  interval& extend(T v) {
    lower = v < lower ? v : lower;
    upper = v > upper ? v : upper;
    return *this;
  }
  interval& extend(const interval& o) {
    lower = o.lower < lower ? o.lower : lower;
    upper = o.upper > upper ? o.upper : upper;
    return *this;
  }
};
template <class T> std::ostream& operator<<(std::ostream& o, const interval<T>& i) {
  return o << '[' << i.lower << ',' << i.upper << ']';
}

inline std::string prettyNumber(size_t n) { return std::to_string(n); }

// ------------------------------------------------------------ jitter
// Answered by the harness: the configured jitter for (pixel, accumID, draw).
float aloha_ref_jitter(unsigned pixel, unsigned accum_id, unsigned draw);

template <unsigned N> struct LCG {
  unsigned pixel = 0, accum = 0, draw = 0;
  LCG() {}
  LCG(unsigned p, unsigned a) : pixel(p), accum(a), draw(0) {}
  float operator()() { return aloha_ref_jitter(pixel, accum, draw++); }
};

}  // namespace common

using namespace common;

// ----------------------------------------------------- OptiX / OWL device
struct Ray {
  vec3f origin, direction;
  float tmin = 0.f, tmax = 1e30f;
  Ray() {}
  Ray(const vec3f& o, const vec3f& d, float t0, float t1) : origin(o), direction(d), tmin(t0), tmax(t1) {}
};

vec2i getLaunchIndex();
vec2i getLaunchDims();
void* aloha_ref_prd();
const void* aloha_ref_program_data();
void aloha_ref_trace(OptixTraversableHandle group, const Ray& ray, void* prd);

template <class T> T& getPRD() { return *static_cast<T*>(aloha_ref_prd()); }
template <class T> const T& getProgramData() { return *static_cast<const T*>(aloha_ref_program_data()); }
template <class PRD> void traceRay(OptixTraversableHandle group, const Ray& ray, PRD& prd, unsigned = 0) {
  aloha_ref_trace(group, ray, &prd);
}

// make_rgba (deviceCode.cpp:416): round to nearest of clamp(x, 0, 1) * 255.
inline uint32_t shim_make_8bit(float f) { return (uint32_t)(std::fmin(std::fmax(f, 0.f), 1.f) * 255.f + .5f); }
inline uint32_t make_rgba(const vec4f& c) {
  return shim_make_8bit(c.x) | (shim_make_8bit(c.y) << 8) | (shim_make_8bit(c.z) << 16) |
         (shim_make_8bit(c.w) << 24);
}

}  // namespace owl
