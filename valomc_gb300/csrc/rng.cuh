// rng.cuh -- uniform sources of the photon kernels.
//
// PhiloxRng: Philox4x32-10 (Salmon, Moraes, Dror, Shaw, "Parallel random numbers: as easy
// as 1, 2, 3", SC'11), one counter stream per photon: key = seed, counter = (photon lo,
// photon hi, block, stream).  Words are consumed in order x, y, z, w of each block.
// TapeRng: a caller-supplied word sequence (trajectory replay).
// The double mappings are the reference's (cpp/3d/mt_rng.hpp:187-204); the float mappings
// keep 24 (closed, half-open) or 23 (open) bits so every value is exact in FP32.
#pragma once
#include <stdint.h>

namespace vmc {

struct PhiloxRng {
  uint32_t k0, k1, c0, c1, c2, c3;
  uint4 buf;
  int32_t n;

  __device__ __forceinline__ void start(uint64_t seed, uint32_t stream, uint64_t photon) {
    k0 = (uint32_t)seed; k1 = (uint32_t)(seed >> 32);
    c0 = (uint32_t)photon; c1 = (uint32_t)(photon >> 32);
    c2 = 0; c3 = stream; n = 0;
  }
  __device__ __forceinline__ void block() {
    uint32_t x0 = c0, x1 = c1, x2 = c2, x3 = c3, a = k0, b = k1;
#pragma unroll
    for (int r = 0; r < 10; r++) {
      if (r) { a += 0x9E3779B9u; b += 0xBB67AE85u; }
      uint32_t hi0 = __umulhi(0xD2511F53u, x0), lo0 = 0xD2511F53u * x0;
      uint32_t hi1 = __umulhi(0xCD9E8D57u, x2), lo1 = 0xCD9E8D57u * x2;
      uint32_t y0 = hi1 ^ x1 ^ a, y2 = hi0 ^ x3 ^ b;
      x0 = y0; x1 = lo1; x2 = y2; x3 = lo0;
    }
    buf = make_uint4(x0, x1, x2, x3);
    c2++;
    n = 4;
  }
  __device__ __forceinline__ uint32_t next() {
    if (n == 0) block();
    uint32_t r = buf.x;
    buf.x = buf.y; buf.y = buf.z; buf.z = buf.w;
    n--;
    return r;
  }
  __device__ __forceinline__ bool exhausted() const { return false; }
};

struct TapeRng {
  const uint32_t *p, *end;
  bool out;
  __device__ __forceinline__ void start_tape(const uint32_t *b, const uint32_t *e) { p = b; end = e; out = false; }
  __device__ __forceinline__ uint32_t next() {
    if (p < end) return *p++;
    out = true;
    return 0x80000000u;
  }
  __device__ __forceinline__ bool exhausted() const { return out; }
};

// reference mappings (double)
template <class R> __device__ __forceinline__ double unif_closed(R &r) { return (double)r.next() * (1.0 / 4294967295.0); }
template <class R> __device__ __forceinline__ double unif_open(R &r) { return ((double)r.next() + 0.5) * (1.0 / 4294967296.0); }
template <class R> __device__ __forceinline__ double unif_halfup(R &r) { return (double)r.next() * (1.0 / 4294967296.0); }

// float mappings
template <class R> __device__ __forceinline__ float unif_closed_f(R &r) { return (float)(r.next() >> 8) * (1.0f / 16777215.0f); }
template <class R> __device__ __forceinline__ float unif_open_f(R &r) { return ((float)(r.next() >> 9) + 0.5f) * (1.0f / 8388608.0f); }
template <class R> __device__ __forceinline__ float unif_halfup_f(R &r) { return (float)(r.next() >> 8) * (1.0f / 16777216.0f); }

}  // namespace vmc
