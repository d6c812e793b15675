// Small vector math and the counter-based RNG shared by all device code.
//
// The vector helpers keep MCell4's operation order (glm's dot is
// (x*x' + y*y') + z*z', cross as in glm::cross); the fp64 translation unit is
// compiled with -fmad=false so that every result matches the reference's
// CPU arithmetic bit for bit.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

namespace mcg {

template <typename T>
struct V3 {
  T x, y, z;
};

template <typename T>
__host__ __device__ __forceinline__ V3<T> v3(T x, T y, T z) {
  V3<T> r;
  r.x = x;
  r.y = y;
  r.z = z;
  return r;
}
template <typename T>
__host__ __device__ __forceinline__ V3<T> operator+(V3<T> a, V3<T> b) {
  return v3<T>(a.x + b.x, a.y + b.y, a.z + b.z);
}
template <typename T>
__host__ __device__ __forceinline__ V3<T> operator-(V3<T> a, V3<T> b) {
  return v3<T>(a.x - b.x, a.y - b.y, a.z - b.z);
}
// component-wise product (glm vec * vec)
template <typename T>
__host__ __device__ __forceinline__ V3<T> cmul(V3<T> a, V3<T> b) {
  return v3<T>(a.x * b.x, a.y * b.y, a.z * b.z);
}
template <typename T>
__host__ __device__ __forceinline__ V3<T> cdiv(V3<T> a, V3<T> b) {
  return v3<T>(a.x / b.x, a.y / b.y, a.z / b.z);
}
template <typename T>
__host__ __device__ __forceinline__ V3<T> scale(V3<T> a, T s) {
  return v3<T>(a.x * s, a.y * s, a.z * s);
}
template <typename T>
__host__ __device__ __forceinline__ T dot(V3<T> a, V3<T> b) {
  return a.x * b.x + a.y * b.y + a.z * b.z;
}
template <typename T>
__host__ __device__ __forceinline__ V3<T> cross(V3<T> a, V3<T> b) {
  return v3<T>(a.y * b.z - b.y * a.z, a.z * b.x - b.z * a.x, a.x * b.y - b.x * a.y);
}
// Round-to-nearest products and sums that the compiler may not fuse or reassociate on
// its own. The fp32 translation unit allows fused multiply-adds; the partner geometry
// (walk crossings, neighbour tests, octant bounds, the closest-approach test) is
// written with these, so that every code path that builds a segment's candidates —
// the fast mask, the list, the refilled pages of the exact fallbacks — rounds alike.
// In fp32 the dot product and the closest-approach test fuse explicitly (fewer
// instructions, one rounding per fused step); in fp64 (the unit built without fused
// multiply-adds) every operation rounds on its own, as the reference's do.
__device__ __forceinline__ float mul_rn(float a, float b) { return __fmul_rn(a, b); }
__device__ __forceinline__ double mul_rn(double a, double b) { return __dmul_rn(a, b); }
__device__ __forceinline__ float add_rn(float a, float b) { return __fadd_rn(a, b); }
__device__ __forceinline__ double add_rn(double a, double b) { return __dadd_rn(a, b); }
__device__ __forceinline__ float sub_rn(float a, float b) { return __fsub_rn(a, b); }
__device__ __forceinline__ double sub_rn(double a, double b) { return __dsub_rn(a, b); }
__device__ __forceinline__ float dot_rn(V3<float> a, V3<float> b) {
  return __fmaf_rn(a.z, b.z, __fmaf_rn(a.y, b.y, __fmul_rn(a.x, b.x)));
}
__device__ __forceinline__ double dot_rn(V3<double> a, V3<double> b) {
  return __dadd_rn(__dadd_rn(__dmul_rn(a.x, b.x), __dmul_rn(a.y, b.y)), __dmul_rn(a.z, b.z));
}
// collide_mol's miss test movelen2 * dirlen2 - d * d > movelen2 * sigma2
__device__ __forceinline__ bool misses_disk(float movelen2, float dirlen2, float d, float sigma2) {
  return __fmaf_rn(movelen2, dirlen2, -__fmul_rn(d, d)) > __fmul_rn(movelen2, sigma2);
}
__device__ __forceinline__ bool misses_disk(double movelen2, double dirlen2, double d, double sigma2) {
  return __dsub_rn(__dmul_rn(movelen2, dirlen2), __dmul_rn(d, d)) > __dmul_rn(movelen2, sigma2);
}

template <typename T>
__host__ __device__ __forceinline__ T tmax(T a, T b) {
  return a > b ? a : b;
}
template <typename T>
__host__ __device__ __forceinline__ T tabs(T a) {
  return a < T(0) ? -a : a;
}

// --------------------------------------------------------------------------
// Philox4x32-10 (Salmon, Moraes, Dror, Shaw, "Parallel random numbers: as easy
// as 1, 2, 3", SC 2011): a counter-based generator, so every molecule-step owns
// an independent stream addressed by (molecule id, iteration, phase, block) and
// any draw can be replayed without storing generator state.
// One block of the generator: four 32-bit words for key (k0, k1) and counter
// (c0, c1, c2, c3).
__device__ __forceinline__ uint4 philox_block(uint32_t k0, uint32_t k1, uint32_t c0, uint32_t c1, uint32_t c2,
                                              uint32_t c3) {
  uint32_t x0 = c0, x1 = c1, x2 = c2, x3 = c3;
  uint32_t a = k0, b = k1;
#pragma unroll
  for (int r = 0; r < 10; r++) {
    uint32_t hi0 = __umulhi(0xD2511F53u, x0), lo0 = 0xD2511F53u * x0;
    uint32_t hi1 = __umulhi(0xCD9E8D57u, x2), lo1 = 0xCD9E8D57u * x2;
    uint32_t y0 = hi1 ^ x1 ^ a, y1 = lo1, y2 = hi0 ^ x3 ^ b, y3 = lo0;
    x0 = y0;
    x1 = y1;
    x2 = y2;
    x3 = y3;
    a += 0x9E3779B9u;
    b += 0xBB67AE85u;
  }
  return make_uint4(x0, x1, x2, x3);
}
// the same out of line, for the rare draws after the first block
__device__ __noinline__ static uint4 philox_block_rare(uint32_t k0, uint32_t k1, uint32_t c0, uint32_t c1,
                                                       uint32_t c2, uint32_t c3) {
  return philox_block(k0, k1, c0, c1, c2, c3);
}

// The stream of one molecule-step: key = seed, counter = (id low, id high, iteration,
// phase << 24 | block). It holds no buffer, only the index of the next draw: a draw
// computes its block (the first four, the displacement's, are taken together by
// first4), so the state is six registers and the stream is the same as a buffered one.
struct Philox {
  uint32_t k0, k1;      // key = seed
  uint32_t c0, c1, c2;  // counter words: id low, id high, iteration
  uint32_t n;           // phase << 24 | index of the next draw

  __device__ __forceinline__ void init(uint64_t seed, uint64_t id, uint32_t iteration, uint32_t phase) {
    k0 = (uint32_t)seed;
    k1 = (uint32_t)(seed >> 32);
    c0 = (uint32_t)id;
    c1 = (uint32_t)(id >> 32);
    c2 = iteration;
    n = phase << 24;
  }
  // the next four draws (the displacement's): one block, or two when a draw was taken
  // before them (a newborn molecule's unimolecular time)
  __device__ __forceinline__ uint4 next4() {
    const uint32_t idx = n & 0xFFFFFFu, ph = n & 0xFF000000u;
    n += 4;
    const uint4 w0 = philox_block(k0, k1, c0, c1, c2, ph | (idx >> 2));
    const uint32_t off = idx & 3u;
    if (off == 0) return w0;
    const uint4 w1 = philox_block_rare(k0, k1, c0, c1, c2, ph | ((idx >> 2) + 1));
    if (off == 1) return make_uint4(w0.y, w0.z, w0.w, w1.x);
    if (off == 2) return make_uint4(w0.z, w0.w, w1.x, w1.y);
    return make_uint4(w0.w, w1.x, w1.y, w1.z);
  }
  __device__ __forceinline__ uint32_t next_u32() {
    const uint32_t idx = n & 0xFFFFFFu;
    const uint4 w = philox_block_rare(k0, k1, c0, c1, c2, (n & 0xFF000000u) | (idx >> 2));
    n++;
    const uint32_t q = idx & 3u;
    return q == 0 ? w.x : (q == 1 ? w.y : (q == 2 ? w.z : w.w));
  }
};

}  // namespace mcg
