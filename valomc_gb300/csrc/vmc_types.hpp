// vmc_types.hpp -- records shared by the host setup and the sm_103a kernels.
//
// Device layout (all arrays element-indexed, 16-byte aligned, one record per element so a
// step's gather is a few 128-bit loads from consecutive sectors):
//   Tet64 (112 B)  plain FP64 form: the four vertices of the tetrahedron (the reference's
//                  r(H(el, v), c), cpp/3d/MC3D.hpp:1015-1018) + its HN row.
//   Tet32 (80 B)   FP32 tracking form: four outward face planes (unit normal, offset) + HN.
//   Tri64 (64 B)   plain FP64 triangles: three vertices + HN row.
//   Tri32 (64 B)   FP32 triangles: three outward edge lines + HN row.
// HN entries: neighbour element >= 0, boundary -1 - ib, or kOpenFace for a 3D face the
// reference leaves at INT_FAST64_MAX (cpp/3d/MC3D.hpp:863).
// Optics are per job: (mua, mus, g, n) per element, or one row for a homogeneous job.
#pragma once
#include <stdint.h>

#if defined(__CUDACC__)
#define VMC_HD __host__ __device__
#else
#define VMC_HD
#endif

namespace vmc {

constexpr int32_t kOpenFace = 0x7fffffff;
constexpr double kWeight0 = 0.001;        // roulette threshold, cpp/3d/MC3D.hpp:182
constexpr double kChance = 0.1;           // roulette survival, cpp/3d/MC3D.hpp:183
constexpr double kC0 = 2.99792458e11;     // mm/s, cpp/3d/MC3D.hpp:178
constexpr double kPi = 3.14159265358979323846;
constexpr double kDblEps = 2.220446049250313080847e-16;  // cpp/3d/MC3D.hpp:36

struct alignas(16) Tet64 {
  double v[4][3];
  int32_t nbr[4];
};
static_assert(sizeof(Tet64) == 112, "Tet64 layout");

struct alignas(16) Tet32 {
  float pl[4][4];  // (nx, ny, nz, d): n . x = d on the face, n points out of the element
  int32_t nbr[4];
};
static_assert(sizeof(Tet32) == 80, "Tet32 layout");

struct alignas(16) Tri64 {
  double v[3][2];
  int32_t nbr[4];  // 3 used
};
static_assert(sizeof(Tri64) == 64, "Tri64 layout");

struct alignas(16) Tri32 {
  float ln[3][4];  // (nx, ny, d, 0) per edge, outward
  int32_t nbr[4];
};
static_assert(sizeof(Tri32) == 64, "Tri32 layout");

// One emitting boundary face, derived on the host in double with the reference's
// arithmetic (CreatePhoton's per-face quantities, cpp/3d/MC3D.hpp:1072-1107,1148-1183,
// 1243-1278; cpp/2d/MC2D.hpp:971-1002).
struct alignas(16) SourceRec {
  double v0[3], v1[3], v2[3];  // face vertices (2D: segment v0-v1)
  double n[3];                 // inward unit normal
  double e1[3], e2[3];         // cosinic frame (3D, both direction types)
  double L[3];                 // BCLNormal row after Init's normalisation / relative mapping
  double phi0;                 // 2D: atan2 of the mean direction (normal or BCLNormal)
  double sigma;                // 2D Gaussian sigma
  double gauss_h;              // 2D: 0.5 - 0.5 erf(pi / sigma / 2 / sqrt 2)
  int32_t mother;              // LightSourcesMother
  int32_t curface;             // face of the mother element on the boundary (-1 if none)
  int32_t ib;
  int8_t type;                 // BCType
  int8_t dirtype;              // BCLightDirectionType
  int8_t pad[2];
};

// The same face record in FP32 for the tracking form's launch (no FP64 on its hot path).
struct alignas(16) SourceRecF {
  float v0[3], v1[3], v2[3];
  float n[3];
  float e1[3], e2[3];
  float L[3];
  float phi0, sigma, gauss_h;
  float cphi0, sphi0;  // cos, sin of phi0: 2D launch directions by rotation
  int32_t mother, curface, ib;
  int8_t type, dirtype;
  int8_t pad[2];
};

// Per-job counters written by the kernel (rare events only; steps are global).
// Rare-event counters are spread over kSlots copies (slot = block index mod kSlots) so that
// concurrent warps do not serialise on one address; the host sums the slots.
// kJcSteps: element steps of the job's finished walks (one addition per walk)
enum JobCounter { kJcLoss = 0, kJcCapped = 1, kJcRoulette = 2, kJcTapeEnd = 3, kJcSteps = 4, kJcN = 8 };
enum LedgerSlot { kLgLaunched = 0, kLgAbsorbed = 1, kLgExited = 2, kLgRouletteKill = 3, kLgRouletteGain = 4, kLgLost = 5, kLgN = 8 };
constexpr int kSlots = 64;
// idle lanes a warp waits for before relaunching them (at most 7 iterations): on the 2D
// square (32 steps per photon) launching four together is 9% faster than one at a time;
// on the 648k-tet phantom (1420 steps per photon) it makes no difference
constexpr int kDefaultRefill = 4;
// largest accumulator set (2 Ne + 4 Nb doubles) a launch stages whole in each CTA's shared memory
constexpr int64_t kDenseStageBytes = 32 * 1024;
// largest job table a multi-job launch copies into each CTA's shared memory
constexpr int kSmemJobs = 64;

struct JobDev {
  const void *geom;            // Tet64 / Tet32 / Tri64 / Tri32 [Ne]
  const void *optics;          // double4 or float4 rows
  int32_t opt_mask;            // -1: per element, 0: one homogeneous row
  int32_t Ns;                  // emitting faces
  int32_t Ne, Nb;
  const double *cdf;           // [Ns]
  const SourceRec *src;        // [Ns]
  const float *cdf_f;          // [Ns] FP32 copies for the tracking form
  const SourceRecF *src_f;     // [Ns]
  const uint8_t *bctype;       // [Nb]
  const double *bcn;           // [Nb]
  const double *bnorm;         // [Nb x 4] Normal(ib) for MirrorPhoton (FP64 forms)
  double omega;                // 2 pi f
  double k_scale;              // omega / c0: k = k_scale * n  (cpp/3d/MC3D.hpp:662)
  float k_scale_f;             // the same in FP32, for the tracking form
  int32_t dense;               // > 0: the launch stages the 2 Ne + 4 Nb accumulators per CTA in shared memory
  double phase0;
  uint64_t seed;
  uint32_t stream;
  int32_t trace_on;
  int64_t pbegin, pcount;      // global photon index range of this job
  int64_t poffset;             // offset inside the seed's photon stream
  double *ER, *EI, *EBR, *EBI, *DEBR, *DEBI;
  const uint32_t *tape;        // replay
  const int64_t *tape_off;
  int64_t *trace, *trace_len;
  int64_t trace_stride, trace_photons;
  unsigned long long *jc;      // [kSlots x kJcN]
  double *ledger;              // [kSlots x kLgN]
};
static_assert(sizeof(JobDev) % sizeof(uint64_t) == 0, "JobDev is copied as 8-byte words");

// Launch-wide control block in device memory.
struct Ctl {
  unsigned long long next_photon;  // global fetch counter
  unsigned long long done_photons; // completed walks (for cancelled runs)
  unsigned long long steps, scatters;
  int32_t cancel;                  // host sets 1 to stop
  int32_t error_flags;
  int32_t pad[2];
};
enum ErrorFlag { kErrTapeEnd = 1, kErrBadIndex = 2 };

struct LaunchParams {
  const JobDev *jobs;
  const int64_t *job_begin;   // [njobs + 1] prefix of photon counts
  int32_t njobs;
  int32_t chunk;              // photons per warp reservation
  int64_t total;              // sum of photon counts
  int64_t max_steps;
  Ctl *ctl;
  int32_t stage_slots;        // > 0: per-CTA shared-memory staging of ER deposits (power of 2)
  int32_t dense;              // > 0: doubles of the single job's accumulators staged per CTA (as JobDev::dense)
  int32_t refill_min;         // a warp relaunches idle lanes once this many are idle (or every 8th iteration)
  int32_t pad;
  // launches of one job (the kernels whose RNG has kOneJob): the job's descriptor and the
  // ten Philox round keys of its seed, (lo, hi) per round
  JobDev job0;
  uint32_t rk[20];
};

// Shared-memory staging of element deposits: a direct-mapped table of stage_slots entries
// per CTA (element tag, FP64 sum).  A flush into an element whose slot this CTA holds is a
// shared-memory add; a free slot is claimed by the first element hashed to it; anything else
// goes to the global atomic.  The table is added to global memory once, when the CTA ends.
struct Stage {
  int32_t *tag;
  double *val;
  uint32_t mask;  // slots - 1; 0 disables staging
};

}  // namespace vmc
