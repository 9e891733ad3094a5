// rng.cuh -- uniform sources of the photon kernels.
//
// PhiloxRng: Philox4x32-10 (Salmon, Moraes, Dror, Shaw, "Parallel random numbers: as easy
// as 1, 2, 3", SC'11), one counter stream per photon: key = seed, counter = (photon lo,
// photon hi, block, stream).  Words are consumed in order x, y, z, w of each block, except
// that each scatter event (the end of a free path) starts a new block (align()).
// TapeRng: a caller-supplied word sequence (trajectory replay).
// The double mappings are the reference's (cpp/3d/mt_rng.hpp:187-204); the float mappings
// keep 24 (closed, half-open) or 23 (open) bits so every value is exact in FP32.
#pragma once
#include <stdint.h>

namespace vmc {

// The per-photon constants of the counter (key, photon index high word, stream) wait in a
// shared-memory slot of the lane, read once per block, so that only the words that change
// occupy registers.  A pool kernel runs at most 256 threads per CTA.  A one-job launch
// takes its round keys from the kernel parameters, so its slot holds the photon's high
// word and the stream only: an 8-byte read per block instead of 16 (half the shared-memory
// wavefronts) and 2 KB per CTA instead of 4 (+0.8% on the 648k-tet phantom).
__device__ __forceinline__ uint4 *philox_slot() {
  __shared__ uint4 slots[256];
  return slots + threadIdx.x;
}
__device__ __forceinline__ uint2 *philox_slot_hi_stream() {
  __shared__ uint2 slots_hs[256];
  return slots_hs + threadIdx.x;
}

// kLaunchKey: every photon of the launch has the same key (a launch of one job), and the
// ten round keys are kernel parameters (rk, set by the kernel): the rounds read them from
// the constant bank instead of running the key schedule per lane.  The stream is the same.
template <bool kLaunchKey>
struct PhiloxT {
  static constexpr bool kOneJob = kLaunchKey;
  static constexpr bool kReplay = false;
  uint32_t c0, c2;  // photon index low word, block counter
  uint4 buf;
  int32_t n;
  const uint32_t *rk;  // kLaunchKey: round keys k_r = key + r (W0, W1), r = 0..9

  __device__ __forceinline__ void start(uint64_t seed, uint32_t stream, uint64_t photon) {
    if constexpr (kLaunchKey) *philox_slot_hi_stream() = make_uint2((uint32_t)(photon >> 32), stream);
    else *philox_slot() = make_uint4((uint32_t)seed, (uint32_t)(seed >> 32), (uint32_t)(photon >> 32), stream);
    c0 = (uint32_t)photon;
    c2 = 0; n = 0;
  }
  __device__ __forceinline__ void block() {
    uint4 k;  // (key lo, key hi, photon hi, stream); the one-job form's key is in rk
    if constexpr (kLaunchKey) {
      const uint2 hs = *philox_slot_hi_stream();
      k = make_uint4(0u, 0u, hs.x, hs.y);
    } else {
      k = *philox_slot();
    }
    uint32_t x0 = c0, x1 = k.z, x2 = c2, x3 = k.w, a = k.x, b = k.y;
#pragma unroll
    for (int r = 0; r < 10; r++) {
      if constexpr (kLaunchKey) {
        a = rk[2 * r]; b = rk[2 * r + 1];
      } else if (r) {
        a += 0x9E3779B9u; b += 0xBB67AE85u;
      }
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
  // A scatter event starts a fresh block: its draws (direction, then the next free path;
  // at most 3 words) come from one block that every scattering lane of a warp computes
  // together, instead of each lane computing blocks at a different draw.  Words left in
  // the previous block are dropped.
  __device__ __forceinline__ void align() { n = 0; }
};
using PhiloxRng = PhiloxT<false>;  // per-photon key (batched launches)
using PhiloxOne = PhiloxT<true>;   // launch-wide key (one job)

struct TapeRng {
  static constexpr bool kOneJob = false;
  static constexpr bool kReplay = true;
  const uint32_t *p, *end;
  bool out;
  __device__ __forceinline__ void start_tape(const uint32_t *b, const uint32_t *e) { p = b; end = e; out = false; }
  __device__ __forceinline__ uint32_t next() {
    if (p < end) return *p++;
    out = true;
    return 0x80000000u;
  }
  __device__ __forceinline__ bool exhausted() const { return out; }
  __device__ __forceinline__ void align() {}  // a tape is consumed word by word
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
