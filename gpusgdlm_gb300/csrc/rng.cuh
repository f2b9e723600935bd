// Counter-based random streams for the SGDLM samplers.
//
// The reference draws its uniforms and normals from a cuRAND host generator
// (rSGDLM/src/curand_manager.cuh:28-56) into HBM caches of n*m*max_p doubles and
// then compacts accepted Marsaglia-Tsang draws with shared-memory atomics
// (rSGDLM/src/kernel_functions.cuh:569-634), so its sample order is not
// reproducible.  Here every (draw i, series j, purpose, sub-index, epoch) tuple
// owns one Philox4x32-10 block (Salmon, Moraes, Dror, Shaw, SC'11), generated in
// registers by the kernel that consumes it: nothing is cached in HBM and any
// kernel (or the CPU oracle) can regenerate a draw bit-exactly from its indices.
//
// Counter layout: ctr = (i, j, (tag << 24) | sub, epoch), key = (seed_lo, seed_hi).
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

namespace sgdlm {

enum : uint32_t {
  TAG_GAMMA = 1u,   // lambda ~ Gamma(n/2, rate n s/2); sub = attempt
  TAG_THETA = 2u,   // standard normals for theta; sub = group of 4
  TAG_NU = 3u,      // observation noise of a forecast draw
  TAG_BETA_A = 4u,  // first gamma of the Beta discount draw; sub = attempt
  TAG_BETA_B = 5u,  // second gamma of the Beta discount draw; sub = attempt
  TAG_OMEGA = 6u,   // standard normals of the state evolution; sub = group of 4
};

// Attempts per gamma draw before the sampler gives up and flags the draw.
constexpr int kGammaMaxAttempts = 32;

struct U4 {
  uint32_t x, y, z, w;
};

__host__ __device__ __forceinline__ uint32_t mulhi32(uint32_t a, uint32_t b) {
#ifdef __CUDA_ARCH__
  return __umulhi(a, b);
#else
  return (uint32_t)(((uint64_t)a * (uint64_t)b) >> 32);
#endif
}

// Philox4x32 with 10 rounds: multipliers and Weyl key increments as published.
__host__ __device__ __forceinline__ U4 philox(uint32_t i, uint32_t j,
                                               uint32_t tag_sub, uint32_t epoch,
                                               uint32_t k0, uint32_t k1) {
  U4 c{i, j, tag_sub, epoch};
#pragma unroll
  for (int r = 0; r < 10; ++r) {
    const uint32_t hi0 = mulhi32(0xD2511F53u, c.x);
    const uint32_t lo0 = 0xD2511F53u * c.x;
    const uint32_t hi1 = mulhi32(0xCD9E8D57u, c.z);
    const uint32_t lo1 = 0xCD9E8D57u * c.z;
    c = U4{hi1 ^ c.y ^ k0, lo1, hi0 ^ c.w ^ k1, lo0};
    k0 += 0x9E3779B9u;
    k1 += 0xBB67AE85u;
  }
  return c;
}

template <typename Key> __device__ __forceinline__ uint32_t key_epoch(const Key &k) {
  return k.dev_epoch ? (*k.dev_epoch + k.epoch) : k.epoch;
}

__host__ __device__ __forceinline__ uint32_t tag_sub(uint32_t tag, uint32_t sub) {
  return (tag << 24) | (sub & 0x00FFFFFFu);
}

// Uniform on the open interval (0, 1).
//   double: (x + 1/2) 2^-32, exact.
//   float : the same value rounded to float (within 2^-23 relative of it), so the
//           lower tail keeps its resolution: Box-Muller's log(u) and the gamma
//           boost's u^(1/a) then follow the FP64 stream draw by draw even for the
//           smallest u (a grid of 2^-23 absolute would move those tails by
//           percents).  Values that round up to 1 become the largest float below 1.
template <typename T> struct Uniform;
template <> struct Uniform<double> {
  __host__ __device__ static __forceinline__ double of(uint32_t x) {
    return ((double)x + 0.5) * 2.3283064365386963e-10;  // 2^-32
  }
};
template <> struct Uniform<float> {
  __host__ __device__ static __forceinline__ float of(uint32_t x) {
    const float u = ((float)x + 0.5f) * 2.3283064365386963e-10f;  // 2^-32
    return u < 1.0f ? u : 0.99999994f;
  }
};

// Box-Muller (1958): two uniforms -> two independent standard normals.
template <typename T>
__device__ __forceinline__ void box_muller(uint32_t a, uint32_t b, T &z0, T &z1);

template <>
__device__ __forceinline__ void box_muller<double>(uint32_t a, uint32_t b,
                                                   double &z0, double &z1) {
  const double u1 = Uniform<double>::of(a);
  const double u2 = Uniform<double>::of(b);
  const double r = sqrt(-2.0 * log(u1));
  double s, c;
  sincospi(2.0 * u2, &s, &c);
  z0 = r * c;
  z1 = r * s;
}

template <>
__device__ __forceinline__ void box_muller<float>(uint32_t a, uint32_t b, float &z0,
                                                  float &z1) {
  const float u1 = Uniform<float>::of(a);
  const float u2 = Uniform<float>::of(b);
  const float r = sqrtf(-2.0f * logf(u1));
  float s, c;
  sincospif(2.0f * u2, &s, &c);
  z0 = r * c;
  z1 = r * s;
}

__device__ __forceinline__ double dev_log(double x) { return log(x); }
__device__ __forceinline__ float dev_log(float x) { return logf(x); }
__device__ __forceinline__ double dev_sqrt(double x) { return sqrt(x); }
__device__ __forceinline__ float dev_sqrt(float x) { return sqrtf(x); }
__device__ __forceinline__ double dev_pow(double x, double y) { return pow(x, y); }
__device__ __forceinline__ float dev_pow(float x, float y) { return powf(x, y); }

// Marsaglia & Tsang (2000), "A simple method for generating gamma variables",
// with the U^(1/alpha) boost for alpha < 1 from the same paper.
//
// Attempt t of draw (i, j) uses Philox block (i, j, tag<<24 | t, epoch):
// x, y -> one Box-Muller normal, z -> the acceptance uniform, and attempt 0's
// w -> the boost uniform.  Returns a Gamma(alpha, 1) variate; *failed is set if
// kGammaMaxAttempts attempts were all rejected (the mean alpha is returned).
//
// no_boost reproduces the reference's Beta sampler, which applies the
// Marsaglia-Tsang recurrence to shapes below one without the boost
// (rSGDLM/src/kernel_functions.cuh:725-798).
template <typename T>
__device__ __forceinline__ T gamma_mt(T alpha, uint32_t i, uint32_t j, uint32_t tag,
                                      uint32_t epoch, uint32_t k0, uint32_t k1,
                                      bool no_boost, bool *failed) {
  const bool boost = (alpha < T(1)) && !no_boost;
  const T a = boost ? alpha + T(1) : alpha;
  const T d = a - T(1) / T(3);
  const T c = T(1) / dev_sqrt(T(9) * d);
  T result = alpha;
  T boost_u = T(1);
  bool ok = false;
  for (int t = 0; t < kGammaMaxAttempts; ++t) {
    const U4 r = philox(i, j, tag_sub(tag, (uint32_t)t), epoch, k0, k1);
    if (t == 0) boost_u = Uniform<T>::of(r.w);
    T x, unused;
    box_muller<T>(r.x, r.y, x, unused);
    const T cx = T(1) + c * x;
    const T v = cx * cx * cx;
    if (v <= T(0)) continue;
    const T u = Uniform<T>::of(r.z);
    const T x2 = x * x;
    if (u < T(1) - T(0.0331) * x2 * x2 ||
        dev_log(u) < T(0.5) * x2 + d * (T(1) - v + dev_log(v))) {
      result = d * v;
      ok = true;
      break;
    }
  }
  if (!ok) *failed = true;
  if (boost && ok) result *= dev_pow(boost_u, T(1) / alpha);
  return result;
}

}  // namespace sgdlm
