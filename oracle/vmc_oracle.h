/*
 * vmc_oracle.h -- CPU restatement of ValoMC's photon-packet propagation loop.
 *
 * TEST INFRASTRUCTURE ONLY.  This is the checker: tests/, __graft_entry__.smoke()
 * and bench.py's cpu_baseline / reference legs load it; the product library
 * (valomc_gb300/csrc) never links or calls it.
 *
 * It restates, in plain C99 (+OpenMP), the functions of the reference engines
 *   cpp/3d/MC3D.hpp  (ErrorChecks :460-571, Init :576-738, BuildNeighbourhoods :835-871,
 *                     BuildLightSource :941-1002, WhichFace :1006-1057, CreatePhoton :1060-1294,
 *                     ScatterPhoton :1297-1340, MirrorPhoton :1343-1351, FresnelPhoton :1365-1447,
 *                     PropagatePhoton :1450-1638, MonteCarlo :1641-1822,
 *                     RayTriangleIntersects :1825-1869)
 *   cpp/2d/MC2D.hpp  (the same functions at :390-1722)
 *   cpp/3d/mt_rng.hpp (MT19937 and its four uniform mappings :155-204)
 * with the same arithmetic (compiled with -ffp-contract=off so that x86 and Arm
 * give identical bits), so that in MT19937 mode it reproduces the reference
 * executable's output bit for bit.  Two more uniform sources exist for parity
 * with the GPU: a per-photon Philox4x32-10 stream (the GPU's generator) and a
 * caller-supplied tape of 32-bit words (trajectory replay).
 *
 * Arrays follow the reference's Array<T> layout (cpp/3d/Array.hpp:58-69):
 * column-major, element (row) index fastest: H(el, c) = H[el + Ne * c].
 */
#ifndef VMC_ORACLE_H
#define VMC_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* uniform sources */
enum { VO_RNG_MT = 0, VO_RNG_PHILOX = 1, VO_RNG_TAPE = 2 };

/* status codes: 0 ok, 1 + mcerror (cpp/Errors.hpp:4-21) for engine errors */
enum {
  VO_OK = 0,
  VO_ERR_MC_BASE = 1,          /* 1 + NO_LIGHTSOURCE ... 1 + MISSING_BOUNDARY */
  VO_ERR_BAD_ARG = 64,
  VO_ERR_NOMEM = 65
};

/* terminal trace codes (deposits are element indices >= 0, exits are -1 - ib) */
#define VO_EV_ROULETTE (INT64_MIN + 1)
#define VO_EV_LOST (INT64_MIN + 2)
#define VO_EV_CAPPED (INT64_MIN + 3)
#define VO_EV_TAPE_END (INT64_MIN + 4)
#define VO_EV_TRUNCATED (INT64_MIN + 5)

/* ledger slots (weights, summed over photons) */
enum {
  VO_LG_LAUNCHED = 0,      /* photons launched (weight 1 each) */
  VO_LG_ABSORBED = 1,      /* sum of (1 - exp(-mua ds)) w over steps with mua > 0 */
  VO_LG_EXITED = 2,        /* weight leaving through the boundary */
  VO_LG_ROULETTE_KILL = 3, /* weight removed by roulette */
  VO_LG_ROULETTE_GAIN = 4, /* weight added by roulette survivors (w/chance - w) */
  VO_LG_LOST = 5,          /* weight of lost / capped photons */
  VO_LG_N = 8
};

typedef struct vo_problem {
  int32_t dim;          /* 2 or 3 */
  int32_t rng_kind;     /* VO_RNG_* */
  int32_t nthreads;     /* OpenMP team size; the photon split follows MC3D.hpp:1654-1668 */
  int32_t hn_given;     /* 1: HN holds a caller neighbourhood (MEX arg), 0: build it */
  int64_t Ne, Nb, Nr;   /* rows of H, BH, r */
  const int64_t *H;     /* [Ne x (dim+1)] */
  int64_t *HN;          /* [Ne x (dim+1)] in/out */
  const int64_t *BH;    /* [Nb x dim] */
  const double *r;      /* [Nr x dim] */
  const double *mua, *mus, *g, *n;
  int64_t n_mua, n_mus, n_g, n_n;
  const char *BCType;           int64_t n_BCType;
  const double *BCn;            int64_t n_BCn;
  double *BCLNormal;            int64_t n_BCLNormal;   /* [Nb x dim], modified by init */
  char *BCLightDirectionType;   int64_t n_BCLDT;       /* [Nb], filled with 'n' when n_BCLDT == 0 */
  const double *BCIntensity;    int64_t n_BCIntensity; /* [Nb] or none (=1) */
  const double *GaussianSigma;  int64_t n_GaussianSigma;
  double f, phase0;
  int64_t Nphoton;
  uint64_t seed;
  uint32_t stream;      /* Philox stream id (counter word 3) */
  int64_t max_steps;    /* 0: unlimited (reference behaviour) */
  /* tape mode: photon p consumes tape[tape_off[p] .. tape_off[p+1]) */
  const uint32_t *tape;
  const int64_t *tape_off;
  /* outputs, caller-allocated: ER/EI [Ne], EBR/EBI/DEBR/DEBI [Nb] */
  double *ER, *EI, *EBR, *EBI, *DEBR, *DEBI;
  int32_t normalize;    /* 1: apply MonteCarlo's normalisation (MC3D.hpp:1792-1818) */
  int32_t pad0;
  /* counters */
  int64_t loss, steps, scatters, photons_done, capped;
  double ledger[VO_LG_N];
  /* optional trace: photon p writes trace[p*trace_stride ...], length trace_len[p] */
  int64_t *trace;
  int64_t *trace_len;
  int64_t trace_stride;
  int64_t trace_photons;   /* photons [0, trace_photons) are traced */
  double seconds;          /* wall time of the photon loop */
  int64_t photon_offset;   /* Philox mode: simulate photons [offset, offset + Nphoton) */
} vo_problem;

/* ErrorChecks + Init + MonteCarlo; returns VO_OK or 1 + mcerror */
int vo_run(vo_problem *P);

/* setup pieces, exposed for tests */
int vo_error_checks(const vo_problem *P);
int vo_build_neighbours(vo_problem *P);            /* fills P->HN */

/* light sources in BuildLightSource order; returns count or -1 */
int64_t vo_light_sources(vo_problem *P, int64_t *ls, int64_t *mother, double *cdf, int64_t cap);

/* generators, exposed for known-answer tests */
void vo_mt_words(uint64_t seed, uint32_t *out, int64_t n);
void vo_philox4x32_10(const uint32_t ctr[4], const uint32_t key[2], uint32_t out[4]);
void vo_philox4x64_10(const uint64_t ctr[4], const uint64_t key[2], uint64_t out[4]);
void vo_philox_words(uint64_t seed, uint32_t stream, uint64_t photon, uint32_t *out, int64_t n);

int vo_max_threads(void);

#ifdef __cplusplus
}
#endif
#endif
