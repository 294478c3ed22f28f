// steps.h -- the march's t sequence: first sample, iteration cap and exact
// runs of steps (host and device).
//
// The march advances t by the rounded sequence t, t+dt, (t+dt)+dt, ...
// (integrateBrick, deviceCode.cpp:271-296).  If t and dt are both multiples
// of 2^q and every t the march reaches stays below 2^(24+q) in magnitude,
// every t + dt is a float (a multiple of 2^q with at most 24 significant
// bits), so the rounded sequence equals the exact one, and fmaf(k, dt, t)
// (exact for the same reason) lands on the k-th step directly.  A run of k
// skipped samples then costs a few instructions instead of k loop trips.
//
// Host-compilable so that the CPU tests can compare the jump with the loop.
#pragma once

#include <math.h>
#include <stdint.h>
#include <string.h>

#ifdef __CUDACC__
#define ALOHA_HD __host__ __device__ __forceinline__
#else
#define ALOHA_HD inline
#endif

namespace aloha {

// firstSampleT (deviceCode.cpp:245-254).
ALOHA_HD float first_sample_t(float lower, float dt, float ils) {
  const float n = floorf((lower - dt * ils) / dt);
  float t = dt * (ils + n);
  if (t < lower) t = t + dt;
  return t;
}

// Iteration cap of one brick march: twice the lattice points in [t0, t1) plus
// 16.  It never binds while t advances by about dt; it ends the loop when
// t + dt rounds back to t (ray parameters beyond ~2^24 dt).
ALOHA_HD uint32_t march_cap(float t0, float t1, float dt) {
  const float span = (t1 - t0) / dt;
  return span < 1e8f ? (uint32_t)(span * 2.0f) + 16u : 200000016u;
}

ALOHA_HD uint32_t float_bits(float x) {
  uint32_t b;
  memcpy(&b, &x, sizeof b);
  return b;
}

// Largest q with x a multiple of 2^q (x finite; 1000 for 0).
ALOHA_HD int low_bit_exp(float x) {
  const uint32_t b = float_bits(x) & 0x7fffffffu;
  if (b == 0u) return 1000;
  const int e = (int)(b >> 23);
  const uint32_t m = (b & 0x7fffffu) | (e ? 0x800000u : 0u);
#ifdef __CUDA_ARCH__
  const int tz = __ffs((int)m) - 1;
#else
  const int tz = __builtin_ctz(m);
#endif
  return (e ? e : 1) - 150 + tz;
}

// True when the steps from t_first (>= 0) up to t1 + dt are exact, with at
// most 2^22 of them (so step counts convert to float exactly).
ALOHA_HD bool exact_steps(float t_first, float t1, float dt) {
  if (!(dt > 0.0f) || !(t_first >= 0.0f) || !((t1 - t_first) < 4194304.0f * dt)) return false;
  const int qt = low_bit_exp(t_first), qd = low_bit_exp(dt);
  const int q = qt < qd ? qt : qd;
  const float hi = t1 + 2.0f * dt;  // above every t reached (the last is below t1 + dt)
  if (!(hi < 3.0e38f)) return false;
  const int e = (int)((float_bits(hi) >> 23) & 0xffu) - 127;  // hi < 2^(e+1)
  return e + 1 <= 24 + q;
}

// Smallest k in [lo, lim] with t + k dt >= tb (lim if there is none), for
// exact steps: an estimate from the division, corrected with exact compares.
ALOHA_HD uint32_t run_steps(float t, float tb, float dt, float inv_dt, uint32_t lo, uint32_t lim) {
  if (lim <= lo) return lim;
  const float kf = fminf(fmaxf(ceilf((tb - t) * inv_dt), (float)lo), 4194304.0f);
  uint32_t k = (uint32_t)kf < lim ? (uint32_t)kf : lim;
  while (k > lo && !(fmaf((float)(k - 1u), dt, t) < tb)) --k;
  while (k < lim && fmaf((float)k, dt, t) < tb) ++k;
  return k;
}

}  // namespace aloha
