// Compares the march's jump over a run of skipped samples (steps.h) with the
// sample-by-sample loop it replaces, on random bricks: first samples with no,
// constant and hashed jitter, step sizes that are and are not powers of two,
// runs that cross powers of two, ray parameters near the limit of exactness,
// runs clipped by the iteration cap, and step budgets (a checkpoint hook
// stops a run every K samples).
//
// Build: g++ -O2 -std=c++17 -ffp-contract=off -I <csrc> exact_steps_check.cpp
// Prints one summary line; exit status 1 on any mismatch.
#include <cstdint>
#include <cstdio>
#include <random>

#include "steps.h"

using namespace aloha;

namespace {

struct Stats {
  long bricks = 0, exact_bricks = 0, runs = 0, jumped = 0, crossings = 0, mismatches = 0;
};

bool same(float a, float b) { return float_bits(a) == float_bits(b); }

// The loop run_steps replaces.
uint32_t loop_steps(float& t, uint32_t& n, float tb, uint32_t cap, float dt, uint32_t max_steps) {
  uint32_t k = 0;
  while (k < max_steps && t < tb && n < cap) {
    ++n;
    t = t + dt;
    ++k;
  }
  return k;
}

void check_brick(std::mt19937_64& rng, float dt, float t0, float t1, float ils, Stats& st, bool small_cap) {
  std::uniform_real_distribution<float> u01(0.0f, 1.0f);
  ++st.bricks;
  const float t_first = first_sample_t(t0, dt, ils);
  uint32_t cap = march_cap(t0, t1, dt);
  if (small_cap) cap = 1u + (uint32_t)(u01(rng) * 40.0f);
  const bool exact = exact_steps(t_first, t1, dt);
  st.exact_bricks += exact;
  const float inv_dt = 1.0f / dt;
  float t = t_first;
  uint32_t n = 0;
  while (t < t1 && n < cap) {
    const float r = u01(rng);
    if (r < 0.3f) {  // a full sample
      ++n;
      t = t + dt;
      continue;
    }
    // a skipped run: the first sample always, then up to tb (sometimes at or
    // before t; never past t1, as in the march, where tb is a macrocell exit
    // clamped to the brick's exit), within a step budget now and then
    const float tb = fminf(t + (u01(rng) * 48.0f - 4.0f) * dt, t1);
    const uint32_t budget = r < 0.5f ? (uint32_t)(u01(rng) * 12.0f) : 0xffffffffu;
    ++n;
    t = t + dt;
    float tr = t;
    uint32_t nr = n;
    const uint32_t kr = loop_steps(tr, nr, tb, cap, dt, budget);
    ++st.runs;
    if (exact) {
      ++st.jumped;
      const float before = t;
      float tj = t;
      uint32_t nj = n;
      const uint32_t kj = run_steps(tj, nj, tb, cap, dt, inv_dt, budget);
      if (kj != kr || nj != nr || !same(tj, tr)) {
        if (st.mismatches++ < 5)
          std::printf("run: dt %a t %a tb %a n %u cap %u budget %u: loop %u %u %a, jump %u %u %a\n", dt, before, tb,
                      n, cap, budget, kr, nr, tr, kj, nj, tj);
      }
      if ((float_bits(before) >> 23) != (float_bits(tr) >> 23)) ++st.crossings;
    }
    t = tr;
    n = nr;
  }
}

}  // namespace

int main() {
  std::mt19937_64 rng(20240611u);
  std::uniform_real_distribution<float> u01(0.0f, 1.0f);
  const float dts[] = {0.5f, 0.25f, 1.0f, 2.0f, 0.125f, 0.3f, 0.1f, 0.7f, 1.0f / 3.0f, 0.0009765625f, 0.75f, 1.5f};
  Stats st;
  for (int i = 0; i < 60000; ++i) {
    const int which = i % 16;
    const float dt = which < 12 ? dts[which] : 0.05f + 1.95f * u01(rng);
    float t0;
    switch (i % 6) {
      case 0: t0 = 16.0f * u01(rng); break;
      case 1: t0 = 4096.0f * u01(rng); break;
      case 2: t0 = 2097152.0f + 6291456.0f * u01(rng); break;  // up to 2^23: near the limit for dt 0.5
      case 3: t0 = 8388608.0f * dt * (0.97f + 0.06f * u01(rng)); break;  // around 2^23 dt
      case 4: t0 = ldexpf(1.0f, 1 + (int)(u01(rng) * 12.0f)) - 40.0f * dt * u01(rng); break;  // just below 2^k
      default: t0 = 0.0f; break;
    }
    if (t0 < 0.0f) t0 = 0.0f;
    const float t1 = t0 + (i % 7 == 0 ? 4.0f : 1200.0f) * u01(rng) * (dt < 0.01f ? 0.05f : 1.0f);
    float ils = 0.0f;
    if (i % 3 == 1) ils = u01(rng);
    if (i % 3 == 2) ils = (float)(uint32_t)(u01(rng) * 16777215.0f) * (1.0f / 16777216.0f);
    check_brick(rng, dt, t0, t1, ils, st, i % 11 == 0);
  }
  std::printf("bricks %ld exact %ld runs %ld jumped %ld crossings %ld mismatches %ld\n", st.bricks, st.exact_bricks,
              st.runs, st.jumped, st.crossings, st.mismatches);
  return st.mismatches == 0 && st.exact_bricks > st.bricks / 4 && st.crossings > 1000 ? 0 : 1;
}
