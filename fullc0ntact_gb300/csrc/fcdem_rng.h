// fcdem_rng.h -- the seeded generator of the scene set-up (host code):
// splitmix64 and uniform floats/doubles drawn from it, the same on every
// platform.
#pragma once

namespace fcdem_rng {

// splitmix64: a small, platform-independent generator.
typedef unsigned long long u64;
inline u64 nextU64(u64 &s) {
  u64 z = (s += 0x9e3779b97f4a7c15ull);
  z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ull;
  z = (z ^ (z >> 27)) * 0x94d049bb133111ebull;
  return z ^ (z >> 31);
}
// Uniform in [0, 1) with 24 random bits (exact in float).
inline float uniformF(u64 &s) { return (float)(nextU64(s) >> 40) * (1.0f / 16777216.0f); }
inline double uniformD(u64 &s) { return (double)(nextU64(s) >> 11) * (1.0 / 9007199254740992.0); }

}  // namespace fcdem_rng
