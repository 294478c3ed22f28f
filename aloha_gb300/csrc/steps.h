// steps.h -- the march's t sequence: first sample, iteration cap and exact
// runs of steps (host and device).
//
// The march advances t by the rounded sequence t, t+dt, (t+dt)+dt, ...
// (integrateBrick, deviceCode.cpp:271-296).  Every float in a binade
// [2^e, 2^(e+1)) is a multiple of its spacing 2^(e-23); if dt is a multiple
// of it too, t + dt is exact while it stays in the binade (or lands on
// 2^(e+1)), and fmaf(j, dt, t) -- exact for the same reason -- lands on the
// j-th step directly.  Only the step that crosses a power of two can round.
// A run of k skipped samples then costs a few instructions per binade it
// crosses instead of k loop trips.
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

ALOHA_HD float bits_float(uint32_t b) {
  float x;
  memcpy(&x, &b, sizeof x);
  return x;
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

// True when dt is a multiple of the float spacing of every t the march of a
// brick reaches (all below t1 + dt, above t_first >= 0): then t + dt is exact
// for every t in a binade [2^e, 2^(e+1)) as long as it stays at or below
// 2^(e+1), whatever the low bits of t.  Also bounds the brick to 2^22 steps,
// so step counts convert to float exactly.
ALOHA_HD bool exact_steps(float t_first, float t1, float dt) {
  if (!(dt > 0.0f) || !(t_first >= 0.0f) || !((t1 - t_first) < 4194304.0f * dt)) return false;
  const float hi = t1 + 2.0f * dt;  // above every t reached
  if (!(hi < 3.0e38f)) return false;
  const int e = (int)((float_bits(hi) >> 23) & 0xffu) - 127;  // every t reached is below 2^(e+1)
  return e - 23 <= low_bit_exp(dt);
}

// Advances (t, n) like the loop
//   while (k < max_steps && t < tb && n < cap) { ++n; t = t + dt; ++k; }
// and returns k, for t > 0 on a brick with exact_steps.  Within t's binade,
// up to its upper end B = 2^(e+1), the steps are exact, so fmaf(j, dt, t)
// lands on the j-th one; the step that crosses B may round and is taken as
// the loop takes it.  A run that ends inside the binade (the common case)
// costs one estimate and one check; one that crosses B, a pass per binade.
ALOHA_HD uint32_t run_steps(float& t, uint32_t& n, float tb, uint32_t cap, float dt, float inv_dt,
                            uint32_t max_steps) {
  uint32_t k = 0;
  while (k < max_steps && t < tb && n < cap) {
    const uint32_t lim = (max_steps - k) < (cap - n) ? (max_steps - k) : (cap - n);
    const float d = t - bits_float((float_bits(t) & 0x7f800000u) + 0x00800000u);  // t - B, exact, < 0
    // j: the first step at or past tb (lim if none), an estimate from the
    // division corrected with compares; they are exact wherever
    // t + j dt <= B, which the check below establishes for the final j
    const float kf = fminf(fmaxf(ceilf((tb - t) * inv_dt), 1.0f), 4194304.0f);
    uint32_t j = (uint32_t)kf < lim ? (uint32_t)kf : lim;
    while (j > 1u && !(fmaf((float)(j - 1u), dt, t) < tb)) --j;
    while (j < lim && fmaf((float)j, dt, t) < tb) ++j;
    if (fmaf((float)j, dt, d) <= 0.0f) {  // sign of t + j dt - B, exact
      t = fmaf((float)j, dt, t);
      n += j;
      return k + j;
    }
    // the run leaves the binade first: the most steps that stay at or below B
    const float jf = fminf(fmaxf(floorf(-d * inv_dt), 0.0f), 4194304.0f);
    uint32_t jb = (uint32_t)jf < lim ? (uint32_t)jf : lim;
    while (jb > 0u && fmaf((float)jb, dt, d) > 0.0f) --jb;
    while (jb < lim && fmaf((float)(jb + 1u), dt, d) <= 0.0f) ++jb;
    t = fmaf((float)jb, dt, t);
    n += jb;
    k += jb;
    if (jb == lim) break;
    // the crossing step (t < tb, n < cap, k < max_steps still hold)
    t = t + dt;
    ++n;
    ++k;
  }
  return k;
}

}  // namespace aloha
