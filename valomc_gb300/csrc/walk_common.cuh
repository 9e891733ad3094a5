// walk_common.cuh -- pieces shared by the 2D and 3D photon walkers: job access, tracing,
// photon launch from a precomputed emitting face, and counters.
#pragma once
#include <cuda_runtime.h>
#include <math.h>
#include <stdint.h>

#include "rng.cuh"
#include "vmc_types.hpp"

namespace vmc {

constexpr unsigned kFull = 0xffffffffu;
constexpr int kMaxRejections = 4096;   // bound on launch-direction rejection loops

// ---- replay trace (tape variant only) ----
struct NoTrace {
  __device__ __forceinline__ void begin(const JobDev &, int64_t) {}
  __device__ __forceinline__ void put(int64_t) {}
  __device__ __forceinline__ void end() {}
};

struct Trace {
  int64_t *p, *len;
  int64_t n, cap;
  bool on;
  __device__ __forceinline__ void begin(const JobDev &J, int64_t q) {
    on = J.trace_on && q < J.trace_photons;
    if (on) { p = J.trace + q * J.trace_stride; len = J.trace_len + q; cap = J.trace_stride; n = 0; }
  }
  __device__ __forceinline__ void put(int64_t ev) {
    if (on) { if (n < cap) p[n] = ev; n++; }
  }
  __device__ __forceinline__ void end() {
    if (on) {
      if (n > cap) { p[cap - 1] = INT64_MIN + 5; n = cap; }
      *len = n;
      on = false;
    }
  }
};

constexpr int64_t kEvRoulette = INT64_MIN + 1;
constexpr int64_t kEvLost = INT64_MIN + 2;
constexpr int64_t kEvCapped = INT64_MIN + 3;
constexpr int64_t kEvTapeEnd = INT64_MIN + 4;

template <class R> struct TraceFor { using type = NoTrace; };
template <> struct TraceFor<TapeRng> { using type = Trace; };

__device__ __forceinline__ void job_count_add(const JobDev &J, int which, unsigned long long n) {
  atomicAdd(J.jc + (blockIdx.x & (kSlots - 1)) * kJcN + which, n);
}
__device__ __forceinline__ void job_count(const JobDev &J, int which) {
  atomicAdd(J.jc + (blockIdx.x & (kSlots - 1)) * kJcN + which, 1ull);
}
__device__ __forceinline__ void job_ledger(const JobDev &J, int which, double v) {
  atomicAdd(J.ledger + (blockIdx.x & (kSlots - 1)) * kLgN + which, v);
}

// first source with xi < CDF (cpp/3d/MC3D.hpp:1068-1070), clamped to the last source
// (cpp/2d/MC2D.hpp:969; in 3D the reference would read one past the end at xi == 1)
__device__ __forceinline__ int pick_source(const JobDev &J, double xi) {
  int lo = 0, hi = J.Ns;  // first index with cdf > xi in [lo, hi]
  while (lo < hi) {
    int mid = (lo + hi) >> 1;
    if (xi < __ldg(J.cdf + mid)) hi = mid;
    else lo = mid + 1;
  }
  return lo < J.Ns ? lo : J.Ns - 1;
}

// ---- 3D CreatePhoton (cpp/3d/MC3D.hpp:1060-1294) in double, from the face record ----
template <class R>
__device__ __forceinline__ void create_photon_3d(const JobDev &J, R &rng, double pos[3], double dir[3], int &curel, int &curface) {
  double xi = unif_closed(rng);
  const SourceRec &S = J.src[pick_source(J, xi)];
  curel = S.mother;
  curface = S.curface;
  double r1 = unif_open(rng), r2 = unif_open(rng);
  double sr = sqrt(r1);
#pragma unroll
  for (int c = 0; c < 3; c++) pos[c] = (1.0 - sr) * S.v0[c] + sr * (1.0 - r2) * S.v1[c] + sr * r2 * S.v2[c];
  const double n0 = S.n[0], n1 = S.n[1], n2 = S.n[2];
  dir[0] = n0; dir[1] = n1; dir[2] = n2;  // 'l', and the combinations the reference leaves undefined
  const char bt = S.type, dt = S.dirtype;
  if (dt != 'n' && (bt == 'l' || bt == 'L')) {
    dir[0] = S.L[0]; dir[1] = S.L[1]; dir[2] = S.L[2];
  } else if (dt != 'n' && bt == 'p') {
    pos[0] = S.L[0]; pos[1] = S.L[1]; pos[2] = S.L[2];
  } else if ((dt == 'n' && bt == 'i') || (dt != 'n' && (bt == 'i' || bt == 'I'))) {
    // rejection on the sphere, Mathworld sphere point picking (MC3D.hpp:1124-1141)
    double rr0 = n0, rr1 = n1, rr2 = n2;
    for (int it = 0; it < kMaxRejections; it++) {
      double th = 2.0 * kPi * unif_halfup(rng);
      double u = 2.0 * unif_closed(rng) - 1.0;
      double st, ct;
      sincos(th, &st, &ct);
      double sq = sqrt(1.0 - u * u);
      rr0 = sq * ct; rr1 = sq * st; rr2 = u;
      if (n0 * rr0 + n1 * rr1 + n2 * rr2 > 0.0 || rng.exhausted()) break;
    }
    dir[0] = rr0; dir[1] = rr1; dir[2] = rr2;
  } else if (bt == 'c' || bt == 'C') {
    // cosinic: phi = asin(2U - 1), theta = 2 pi U, mapped onto the face frame (MC3D.hpp:1142-1191)
    double phi = asin(2.0 * unif_open(rng) - 1.0);
    double th = 2.0 * kPi * unif_closed(rng);
    double sp, cp, st, ct;
    sincos(phi, &sp, &cp);
    sincos(th, &st, &ct);
    double f0 = cp, f1 = ct * sp, f2 = st * sp;
#pragma unroll
    for (int c = 0; c < 3; c++) dir[c] = f0 * S.n[c] + f1 * S.e1[c] + f2 * S.e2[c];
  }
}

// ---- 2D CreatePhoton (cpp/2d/MC2D.hpp:958-1132) ----
template <class R>
__device__ double gauss_angle(R &rng, double sigma, double h) {
  double xi = unif_open(rng);
  double a = -kPi / 2, b = kPi / 2, phi = 0.0;
  const double isq2 = sqrt(2.0);
  for (int it = 0; it < 16; it++) {
    phi = (a + b) / 2.0;
    double cdf = (0.5 + 0.5 * erf(phi / sigma / isq2) - h) / (1 - 2.0 * h);
    if (cdf - xi < 0.0) a = phi;
    else b = phi;
  }
  return phi;
}

template <class R>
__device__ __forceinline__ void create_photon_2d(const JobDev &J, R &rng, double pos[2], double dir[2], int &curel, int &curface) {
  double xi = unif_closed(rng);
  const SourceRec &S = J.src[pick_source(J, xi)];
  curel = S.mother;
  curface = S.curface;
  double wv = unif_open(rng);
  pos[0] = S.v0[0] + wv * (S.v1[0] - S.v0[0]);
  pos[1] = S.v0[1] + wv * (S.v1[1] - S.v0[1]);
  const double n0 = S.n[0], n1 = S.n[1];
  dir[0] = n0; dir[1] = n1;
  const char bt = S.type, dt = S.dirtype;
  if (bt == 'l') {
    if (dt != 'n') { dir[0] = S.L[0]; dir[1] = S.L[1]; }
  } else if (bt == 'i') {
    double phi = kPi * (unif_open(rng) - 0.5);
    sincos(S.phi0 + phi, &dir[1], &dir[0]);
  } else if (bt == 'c' || bt == 'g') {
    // direction type 'n': one draw; otherwise redraw until the direction points inward
    // (MC2D.hpp:1085-1124)
    for (int it = 0; it < kMaxRejections; it++) {
      double phi = (bt == 'c') ? asin(2.0 * unif_open(rng) - 1.0) : gauss_angle(rng, S.sigma, S.gauss_h);
      sincos(S.phi0 + phi, &dir[1], &dir[0]);
      if (dt == 'n' || n0 * dir[0] + n1 * dir[1] > 0.0 || rng.exhausted()) break;
    }
  }
}

// A reduction into a global FP64 accumulator.  The accumulators are plain device buffers,
// so the address is converted to the global window once and the add is issued as a
// fire-and-forget global reduction (no generic-address resolution, no returned value).
__device__ __forceinline__ void red_global(double *p, double v) {
  asm volatile("red.global.add.f64 [%0], %1;" :: "l"(__cvta_generic_to_global(p)), "d"(v));
}

// The pool kernel's dynamic shared memory (every extern __shared__ array names this base).
extern __shared__ __align__(16) unsigned char vmc_smem[];

__device__ __forceinline__ void red_shared(double *p, double v) {
  asm volatile("red.shared.add.f64 [%0], %1;" :: "r"((uint32_t)__cvta_generic_to_shared(p)), "d"(v));
}

// Addition into one of the job's FP64 accumulators (ER, EI, EBR, EBI, DEBR, DEBI, back to
// back from ER).  When the launch stages the whole set in each CTA's shared memory
// (J.dense > 0: one job on a small mesh, FP32 walks, whose descriptor is a kernel
// parameter: kStage) the addition stays in the CTA and the kernel adds the CTA's copy to
// global memory once at its end; otherwise it is a global reduction.  On a mesh of a few
// hundred elements the global reductions all land in a handful of L2 lines, whose slice's
// atomic unit then limits the whole launch.
template <bool kStage>
__device__ __forceinline__ void acc_add(const JobDev &J, double *p, double v) {
  if constexpr (kStage) {
    if (J.dense) {
      red_shared(reinterpret_cast<double *>(vmc_smem) + (p - J.ER), v);
      return;
    }
  }
  red_global(p, v);
}

__device__ __forceinline__ void add_d(const JobDev &J, double *p, double v) {
  if (v != 0.0) acc_add<false>(J, p, v);
}

// float -> double by bit manipulation on the integer pipe (exact for normal floats; zero
// and subnormal inputs give 0).  GB300's FP64 pipe is 1/64 of FP32, so the tracking form
// keeps conversions off it.
__device__ __forceinline__ double f2d_int(float x) {
  const uint32_t b = __float_as_uint(x);
  const uint32_t e = (b >> 23) & 0xffu;
  if (e == 0u) return 0.0;
  const uint64_t bits = ((uint64_t)(b >> 31) << 63) | ((uint64_t)(e + (1023u - 127u)) << 52) |
                        ((uint64_t)(b & 0x7fffffu) << 29);
  return __longlong_as_double((long long)bits);
}

// double -> float, rounded to nearest even, on the integer pipe for zeros and doubles in
// float's normal range (anything else through the FP64 pipe's conversion)
__device__ __forceinline__ float d2f_int(double x) {
  const uint64_t b = (uint64_t)__double_as_longlong(x);
  if ((b << 1) == 0u) return __uint_as_float((uint32_t)(b >> 32));
  const int e = (int)((b >> 52) & 0x7ffu) - 1023 + 127;
  if (e <= 0 || e >= 255) return (float)x;
  const uint32_t m = (uint32_t)(b >> 29) & 0x7fffffu;
  const uint32_t rest = (uint32_t)b & 0x1fffffffu;
  uint32_t r = ((uint32_t)(b >> 63) << 31) | ((uint32_t)e << 23) | m;
  if (rest > 0x10000000u || (rest == 0x10000000u && (m & 1u))) r += 1u;  // a carry moves into the exponent
  return __uint_as_float(r);
}

template <bool kStage>
__device__ __forceinline__ void add_f(const JobDev &J, double *p, float v) {
  if (v != 0.0f) acc_add<kStage>(J, p, f2d_int(v));
}

// element deposit through the CTA's shared-memory stage when it holds (or can claim) the
// element's slot, else straight to the global accumulator
template <bool kStage>
__device__ __forceinline__ void add_staged(const Stage &S, const JobDev &J, int el, float v) {
  if (v == 0.0f) return;
  const double d = f2d_int(v);
  if (S.mask) {
    const uint32_t h = (((uint32_t)el * 2654435761u) >> 16) & S.mask;  // Fibonacci hash, high bits
    int32_t t = S.tag[h];
    if (t < 0) t = atomicCAS(S.tag + h, -1, el), t = (t < 0) ? el : t;
    if (t == el) {
      atomicAdd(S.val + h, d);
      return;
    }
  }
  acc_add<kStage>(J, J.ER + el, d);
}

// ---- FP32 launch for the tracking form: same draws and sampling laws as CreatePhoton,
// evaluated in float from the FP32 face records (cos(asin(s)) = sqrt(1 - s^2)) ----
__device__ __forceinline__ int pick_source_f(const JobDev &J, float xi) {
  int lo = 0, hi = J.Ns;
  while (lo < hi) {
    int mid = (lo + hi) >> 1;
    if (xi < __ldg(J.cdf_f + mid)) hi = mid;
    else lo = mid + 1;
  }
  return lo < J.Ns ? lo : J.Ns - 1;
}

template <class R>
__device__ __forceinline__ void create_photon_3d_f(const JobDev &J, R &rng, float pos[3], float dir[3], int &curel,
                                                   int &curface) {
  const SourceRecF &S = J.src_f[pick_source_f(J, unif_closed_f(rng))];
  curel = S.mother;
  curface = S.curface;
  const float r1 = unif_open_f(rng), r2 = unif_open_f(rng);
  const float sr = sqrtf(r1);
#pragma unroll
  for (int c = 0; c < 3; c++) pos[c] = (1.0f - sr) * S.v0[c] + sr * (1.0f - r2) * S.v1[c] + sr * r2 * S.v2[c];
  const float n0 = S.n[0], n1 = S.n[1], n2 = S.n[2];
  dir[0] = n0; dir[1] = n1; dir[2] = n2;
  const char bt = S.type, dt = S.dirtype;
  if (dt != 'n' && (bt == 'l' || bt == 'L')) {
    dir[0] = S.L[0]; dir[1] = S.L[1]; dir[2] = S.L[2];
  } else if (dt != 'n' && bt == 'p') {
    pos[0] = S.L[0]; pos[1] = S.L[1]; pos[2] = S.L[2];
  } else if ((dt == 'n' && bt == 'i') || (dt != 'n' && (bt == 'i' || bt == 'I'))) {
    float rr0 = n0, rr1 = n1, rr2 = n2;
    for (int it = 0; it < kMaxRejections; it++) {
      const float th2 = 2.0f * unif_halfup_f(rng);  // theta / pi
      const float u = 2.0f * unif_closed_f(rng) - 1.0f;
      float st, ct;
      sincospif(th2, &st, &ct);
      const float sq = sqrtf(fmaxf(0.0f, 1.0f - u * u));
      rr0 = sq * ct; rr1 = sq * st; rr2 = u;
      if (n0 * rr0 + n1 * rr1 + n2 * rr2 > 0.0f || rng.exhausted()) break;
    }
    dir[0] = rr0; dir[1] = rr1; dir[2] = rr2;
  } else if (bt == 'c' || bt == 'C') {
    const float s = 2.0f * unif_open_f(rng) - 1.0f;  // sin(phi), phi = asin(2U - 1)
    const float cphi = sqrtf(fmaxf(0.0f, 1.0f - s * s));
    float st, ct;
    sincospif(2.0f * unif_closed_f(rng), &st, &ct);
    const float f0 = cphi, f1 = ct * s, f2 = st * s;
#pragma unroll
    for (int c = 0; c < 3; c++) dir[c] = f0 * S.n[c] + f1 * S.e1[c] + f2 * S.e2[c];
  }
}

template <class R>
__device__ __forceinline__ float gauss_angle_f(R &rng, float sigma, float h) {
  const float xi = unif_open_f(rng);
  float a = -0.5f * (float)kPi, b = 0.5f * (float)kPi, phi = 0.0f;
  for (int it = 0; it < 16; it++) {
    phi = 0.5f * (a + b);
    const float cdf = (0.5f + 0.5f * erff(phi / sigma * 0.70710678118654752f) - h) / (1.0f - 2.0f * h);
    if (cdf - xi < 0.0f) a = phi;
    else b = phi;
  }
  return phi;
}

template <class R>
__device__ __forceinline__ void create_photon_2d_f(const JobDev &J, R &rng, float pos[2], float dir[2], int &curel,
                                                   int &curface) {
  const SourceRecF &S = J.src_f[pick_source_f(J, unif_closed_f(rng))];
  curel = S.mother;
  curface = S.curface;
  const float wv = unif_open_f(rng);
  pos[0] = S.v0[0] + wv * (S.v1[0] - S.v0[0]);
  pos[1] = S.v0[1] + wv * (S.v1[1] - S.v0[1]);
  const float n0 = S.n[0], n1 = S.n[1];
  dir[0] = n0; dir[1] = n1;
  const char bt = S.type, dt = S.dirtype;
  if (bt == 'l') {
    if (dt != 'n') { dir[0] = S.L[0]; dir[1] = S.L[1]; }
  } else if (bt == 'i') {
    // the direction at phi0 + phi, as (cos phi0, sin phi0) turned by phi
    float sp, cp;
    sincospif(unif_open_f(rng) - 0.5f, &sp, &cp);
    dir[0] = S.cphi0 * cp - S.sphi0 * sp;
    dir[1] = S.sphi0 * cp + S.cphi0 * sp;
  } else if (bt == 'c' || bt == 'g') {
    for (int it = 0; it < kMaxRejections; it++) {
      float sp, cp;
      if (bt == 'c') {  // phi = asin(s): sin phi = s, cos phi = sqrt(1 - s^2)
        sp = 2.0f * unif_open_f(rng) - 1.0f;
        cp = sqrtf(fmaxf(0.0f, 1.0f - sp * sp));
      } else {
        sincosf(gauss_angle_f(rng, S.sigma, S.gauss_h), &sp, &cp);
      }
      dir[0] = S.cphi0 * cp - S.sphi0 * sp;
      dir[1] = S.sphi0 * cp + S.cphi0 * sp;
      if (dt == 'n' || n0 * dir[0] + n1 * dir[1] > 0.0f || rng.exhausted()) break;
    }
  }
}

}  // namespace vmc
