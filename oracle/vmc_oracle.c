/*
 * vmc_oracle.c -- CPU restatement of ValoMC's photon loop (test infrastructure only;
 * see vmc_oracle.h for scope).  Each function cites the reference lines it follows.
 * Build with -O3 -ffp-contract=off -fopenmp so its arithmetic is IEEE-exact on any host.
 */
#define _GNU_SOURCE
#include "vmc_oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>
#include <time.h>
#ifdef _OPENMP
#include <omp.h>
#endif

/* mcerror values, cpp/Errors.hpp:4-21 */
enum {
  E_NO_LIGHTSOURCE = 0, E_SIZE_MISMATCH_G, E_SIZE_MISMATCH_MUA, E_SIZE_MISMATCH_MUS,
  E_SIZE_MISMATCH_N, E_SIZE_MISMATCH_BCN, E_MISSING_BCN, E_SIZE_MISMATCH_BCTYPE,
  E_SIZE_MISMATCH_LIGHT_DIRECTION, E_SIZE_MISMATCH_LIGHT_DIRECTION_TYPE, E_INCONSISTENT_H,
  E_INCONSISTENT_BH, E_INCONSISTENT_MESH, E_INCONSISTENT_MESH_DUPLICATE_NEIGHBORS,
  E_NO_GAUSSIAN_SIGMA, E_MISSING_BOUNDARY
};
#define MCERR(e) (VO_ERR_MC_BASE + (e))

static const double kEps = 2.220446049250313080847e-16; /* DBL_EPSILON, MC3D.hpp:36 */
static const double kPi = 3.14159265358979323846;         /* M_PI */
static const double kWeight0 = 0.001, kChance = 0.1;      /* MC3D.hpp:182-183 */
static const double kC0 = 2.99792458e11;                  /* MC3D.hpp:178 */
#define HN_UNSET INT64_MAX                                /* INT_FAST64_MAX, MC3D.hpp:863 */

/* ------------------------------------------------------------------------- */
/* uniform sources                                                            */
/* ------------------------------------------------------------------------- */

/* MT19937 (Matsumoto & Nishimura, mt19937ar), as used by cpp/3d/mt_rng.hpp:119-179 */
typedef struct { uint32_t mt[624]; int mti; } mt_state;

static void mt_seed(mt_state *s, uint64_t seed) {
  s->mt[0] = (uint32_t)(seed & 0xffffffffu);
  for (int i = 1; i < 624; i++)
    s->mt[i] = (uint32_t)(1812433253u * (s->mt[i - 1] ^ (s->mt[i - 1] >> 30)) + (uint32_t)i);
  s->mti = 624;
}

static uint32_t mt_next(mt_state *s) {
  static const uint32_t mag[2] = {0u, 0x9908b0dfu};
  uint32_t y;
  if (s->mti >= 624) {
    int k;
    for (k = 0; k < 624 - 397; k++) {
      y = (s->mt[k] & 0x80000000u) | (s->mt[k + 1] & 0x7fffffffu);
      s->mt[k] = s->mt[k + 397] ^ (y >> 1) ^ mag[y & 1u];
    }
    for (; k < 623; k++) {
      y = (s->mt[k] & 0x80000000u) | (s->mt[k + 1] & 0x7fffffffu);
      s->mt[k] = s->mt[k + 397 - 624] ^ (y >> 1) ^ mag[y & 1u];
    }
    y = (s->mt[623] & 0x80000000u) | (s->mt[0] & 0x7fffffffu);
    s->mt[623] = s->mt[396] ^ (y >> 1) ^ mag[y & 1u];
    s->mti = 0;
  }
  y = s->mt[s->mti++];
  y ^= (y >> 11);
  y ^= (y << 7) & 0x9d2c5680u;
  y ^= (y << 15) & 0xefc60000u;
  y ^= (y >> 18);
  return y;
}

/* Philox4x32-10 (Salmon, Moraes, Dror, Shaw, SC'11): 10 rounds of two 32x32->64
 * multiplies with a Weyl key schedule. */
static inline void philox32_round(uint32_t c[4], const uint32_t k[2]) {
  uint64_t p0 = (uint64_t)0xD2511F53u * c[0];
  uint64_t p1 = (uint64_t)0xCD9E8D57u * c[2];
  uint32_t hi0 = (uint32_t)(p0 >> 32), lo0 = (uint32_t)p0;
  uint32_t hi1 = (uint32_t)(p1 >> 32), lo1 = (uint32_t)p1;
  uint32_t n0 = hi1 ^ c[1] ^ k[0];
  uint32_t n2 = hi0 ^ c[3] ^ k[1];
  c[0] = n0; c[1] = lo1; c[2] = n2; c[3] = lo0;
}

void vo_philox4x32_10(const uint32_t ctr[4], const uint32_t key[2], uint32_t out[4]) {
  uint32_t c[4] = {ctr[0], ctr[1], ctr[2], ctr[3]};
  uint32_t k[2] = {key[0], key[1]};
  for (int r = 0; r < 10; r++) {
    if (r) { k[0] += 0x9E3779B9u; k[1] += 0xBB67AE85u; }
    philox32_round(c, k);
  }
  memcpy(out, c, sizeof(c));
}

/* the 64-bit-word variant shares the round structure; numpy.random.Philox implements it,
 * which gives a known-answer check of the construction */
static inline void mulhilo64(uint64_t a, uint64_t b, uint64_t *hi, uint64_t *lo) {
  unsigned __int128 p = (unsigned __int128)a * b;
  *hi = (uint64_t)(p >> 64); *lo = (uint64_t)p;
}

void vo_philox4x64_10(const uint64_t ctr[4], const uint64_t key[2], uint64_t out[4]) {
  uint64_t c[4] = {ctr[0], ctr[1], ctr[2], ctr[3]};
  uint64_t k[2] = {key[0], key[1]};
  for (int r = 0; r < 10; r++) {
    if (r) { k[0] += 0x9E3779B97F4A7C15ull; k[1] += 0xBB67AE8584CAA73Bull; }
    uint64_t hi0, lo0, hi1, lo1;
    mulhilo64(0xD2E7470EE14C6C93ull, c[0], &hi0, &lo0);
    mulhilo64(0xCA5A826395121157ull, c[2], &hi1, &lo1);
    uint64_t n0 = hi1 ^ c[1] ^ k[0], n2 = hi0 ^ c[3] ^ k[1];
    c[0] = n0; c[1] = lo1; c[2] = n2; c[3] = lo0;
  }
  memcpy(out, c, sizeof(c));
}

/* one photon's Philox stream: key = seed, counter = (photon lo, photon hi, block, stream) */
typedef struct { uint32_t key[2]; uint32_t ctr[4]; uint32_t buf[4]; int nbuf; } philox_stream;

static void philox_start(philox_stream *s, uint64_t seed, uint32_t stream, uint64_t photon) {
  s->key[0] = (uint32_t)seed; s->key[1] = (uint32_t)(seed >> 32);
  s->ctr[0] = (uint32_t)photon; s->ctr[1] = (uint32_t)(photon >> 32);
  s->ctr[2] = 0; s->ctr[3] = stream; s->nbuf = 0;
}

static uint32_t philox_next(philox_stream *s) {
  if (s->nbuf == 0) {
    vo_philox4x32_10(s->ctr, s->key, s->buf);
    s->ctr[2]++;
    s->nbuf = 4;
  }
  return s->buf[4 - s->nbuf--];
}

void vo_philox_words(uint64_t seed, uint32_t stream, uint64_t photon, uint32_t *out, int64_t n) {
  philox_stream s;
  philox_start(&s, seed, stream, photon);
  for (int64_t i = 0; i < n; i++) out[i] = philox_next(&s);
}

void vo_mt_words(uint64_t seed, uint32_t *out, int64_t n) {
  mt_state s;
  mt_seed(&s, seed);
  for (int64_t i = 0; i < n; i++) out[i] = mt_next(&s);
}

typedef struct {
  int kind;
  mt_state mt;
  philox_stream ph;
  const uint32_t *tape; int64_t tpos, tend; int tape_out;
} urng;

static uint32_t u_word(urng *u) {
  switch (u->kind) {
    case VO_RNG_MT: return mt_next(&u->mt);
    case VO_RNG_PHILOX: return philox_next(&u->ph);
    default:
      if (u->tpos < u->tend) return u->tape[u->tpos++];
      u->tape_out = 1;
      return 0x80000000u;
  }
}

/* Philox streams only: the end of a free path (a scatter event) starts a new counter
   block and drops the words left in the current one, so that the draws of one event come
   from one block (the GPU kernels compute that block for all scattering lanes at once).
   The reference's MT19937 stream and a tape are consumed word by word. */
static void u_align(urng *u) {
  if (u->kind == VO_RNG_PHILOX) u->ph.nbuf = 0;
}

/* the four mappings of cpp/3d/mt_rng.hpp:187-204 */
static double UnifClosed(urng *u) { return (double)u_word(u) * (1.0 / 4294967295.0); }
static double UnifOpen(urng *u) { return ((double)u_word(u) + 0.5) * (1.0 / 4294967296.0); }
static double UnifHalfUp(urng *u) { return (double)u_word(u) * (1.0 / 4294967296.0); }

/* ------------------------------------------------------------------------- */
/* engine state                                                               */
/* ------------------------------------------------------------------------- */

typedef struct {
  double pos[3], dir[3];
  int64_t curel, nextel, curface, nextface;
  double weight, phase;
} photon;

typedef struct {
  const vo_problem *P;
  int D;                 /* dim */
  int NF;                /* faces per element: dim + 1 */
  double omega;
  double *k, *g2;        /* MC3D.hpp:660-666 */
  int64_t Ns;
  int64_t *ls, *lsm;     /* LightSources, LightSourcesMother */
  double *cdf;
  const double *BCI;     /* BCIntensity or NULL (=1) */
  const double *BCLN;    /* working BCLNormal */
  const char *BCLDT;
} engine;

typedef struct {
  double *ER, *EI, *EBR, *EBI, *DEBR, *DEBI;
  int64_t loss, steps, scatters, capped;
  double ledger[VO_LG_N];
  urng u;
  int64_t *tr; int64_t trn, trcap; int tracing;
} worker;

#define Hx(P, el, c) ((P)->H[(el) + (P)->Ne * (c)])
#define HNx(P, el, c) ((P)->HN[(el) + (P)->Ne * (c)])
#define BHx(P, ib, c) ((P)->BH[(ib) + (P)->Nb * (c)])
#define Rx(P, i, c) ((P)->r[(i) + (P)->Nr * (c)])

static inline void trace_ev(worker *w, int64_t ev) {
  if (!w->tracing) return;
  if (w->trn < w->trcap) w->tr[w->trn] = ev;
  w->trn++;
}

/* ------------------------------------------------------------------------- */
/* geometry helpers                                                           */
/* ------------------------------------------------------------------------- */

/* ElementVolume, MC3D.hpp:306-332 */
static double volume3(const vo_problem *P, int64_t el) {
  double ax = Rx(P, Hx(P, el, 0), 0), ay = Rx(P, Hx(P, el, 0), 1), az = Rx(P, Hx(P, el, 0), 2);
  double bx = Rx(P, Hx(P, el, 1), 0), by = Rx(P, Hx(P, el, 1), 1), bz = Rx(P, Hx(P, el, 1), 2);
  double cx = Rx(P, Hx(P, el, 2), 0), cy = Rx(P, Hx(P, el, 2), 1), cz = Rx(P, Hx(P, el, 2), 2);
  double dx = Rx(P, Hx(P, el, 3), 0), dy = Rx(P, Hx(P, el, 3), 1), dz = Rx(P, Hx(P, el, 3), 2);
  double vol = (ax - dx) * ((by - dy) * (cz - dz) - (bz - dz) * (cy - dy)) -
               (ay - dy) * ((bx - dx) * (cz - dz) - (bz - dz) * (cx - dx)) +
               (az - dz) * ((bx - dx) * (cy - dy) - (by - dy) * (cx - dx));
  return fabs(vol) / 6.0;
}

static inline double sq(double x) { return x * x; } /* pow(x, 2) */

/* ElementArea(ib), MC3D.hpp:335-343 (Heron) */
static double area3(const vo_problem *P, int64_t ib) {
  int64_t i0 = BHx(P, ib, 0), i1 = BHx(P, ib, 1), i2 = BHx(P, ib, 2);
  double a = sqrt(sq(Rx(P, i1, 0) - Rx(P, i0, 0)) + sq(Rx(P, i1, 1) - Rx(P, i0, 1)) + sq(Rx(P, i1, 2) - Rx(P, i0, 2)));
  double b = sqrt(sq(Rx(P, i2, 0) - Rx(P, i0, 0)) + sq(Rx(P, i2, 1) - Rx(P, i0, 1)) + sq(Rx(P, i2, 2) - Rx(P, i0, 2)));
  double c = sqrt(sq(Rx(P, i1, 0) - Rx(P, i2, 0)) + sq(Rx(P, i1, 1) - Rx(P, i2, 1)) + sq(Rx(P, i1, 2) - Rx(P, i2, 2)));
  return sqrt((a + b + c) * (b + c - a) * (c + a - b) * (a + b - c)) / 4.0;
}

/* Normal(ib), MC3D.hpp:386-405: normalised cross product of the two edges */
static void normal_b3(const vo_problem *P, int64_t ib, double *nrm) {
  int64_t i0 = BHx(P, ib, 0), i1 = BHx(P, ib, 1), i2 = BHx(P, ib, 2);
  double x1 = Rx(P, i1, 0) - Rx(P, i0, 0), y1 = Rx(P, i1, 1) - Rx(P, i0, 1), z1 = Rx(P, i1, 2) - Rx(P, i0, 2);
  double x2 = Rx(P, i2, 0) - Rx(P, i0, 0), y2 = Rx(P, i2, 1) - Rx(P, i0, 1), z2 = Rx(P, i2, 2) - Rx(P, i0, 2);
  double nx = y1 * z2 - z1 * y2, ny = z1 * x2 - x1 * z2, nz = x1 * y2 - y1 * x2;
  double norm = sqrt(nx * nx + ny * ny + nz * nz);
  nrm[0] = nx / norm; nrm[1] = ny / norm; nrm[2] = nz / norm;
}

/* face f of a tetrahedron: (0,1,2), (0,1,3), (0,2,3), (1,2,3), MC3D.hpp:1013 */
static const int kFace3[4][3] = {{0, 1, 2}, {0, 1, 3}, {0, 2, 3}, {1, 2, 3}};

/* Normal(el, f), MC3D.hpp:408-457 */
static void normal_f3(const vo_problem *P, int64_t el, int64_t f, double *nrm) {
  if (f < 0 || f > 3) { nrm[0] = nrm[1] = nrm[2] = 0.0; return; }
  int64_t i0 = Hx(P, el, kFace3[f][0]), i1 = Hx(P, el, kFace3[f][1]), i2 = Hx(P, el, kFace3[f][2]);
  double x1 = Rx(P, i1, 0) - Rx(P, i0, 0), y1 = Rx(P, i1, 1) - Rx(P, i0, 1), z1 = Rx(P, i1, 2) - Rx(P, i0, 2);
  double x2 = Rx(P, i2, 0) - Rx(P, i0, 0), y2 = Rx(P, i2, 1) - Rx(P, i0, 1), z2 = Rx(P, i2, 2) - Rx(P, i0, 2);
  double nx = y1 * z2 - z1 * y2, ny = z1 * x2 - x1 * z2, nz = x1 * y2 - y1 * x2;
  double norm = sqrt(nx * nx + ny * ny + nz * nz);
  nrm[0] = nx / norm; nrm[1] = ny / norm; nrm[2] = nz / norm;
}

/* ElementArea(el) of a triangle, MC2D.hpp:303-310 */
static double area2(const vo_problem *P, int64_t el) {
  double ax = Rx(P, Hx(P, el, 1), 0) - Rx(P, Hx(P, el, 0), 0);
  double ay = Rx(P, Hx(P, el, 1), 1) - Rx(P, Hx(P, el, 0), 1);
  double bx = Rx(P, Hx(P, el, 2), 0) - Rx(P, Hx(P, el, 0), 0);
  double by = Rx(P, Hx(P, el, 2), 1) - Rx(P, Hx(P, el, 0), 1);
  double c = ax * by - ay * bx;
  return 0.5 * (c >= 0.0 ? c : -c);
}

/* ElementLength(ib), MC2D.hpp:313-318 */
static double length2(const vo_problem *P, int64_t ib) {
  return sqrt(sq(Rx(P, BHx(P, ib, 1), 0) - Rx(P, BHx(P, ib, 0), 0)) + sq(Rx(P, BHx(P, ib, 1), 1) - Rx(P, BHx(P, ib, 0), 1)));
}

/* Normal(ib), MC2D.hpp:347-355 */
static void normal_b2(const vo_problem *P, int64_t ib, double *nrm) {
  double dx = Rx(P, BHx(P, ib, 1), 0) - Rx(P, BHx(P, ib, 0), 0);
  double dy = Rx(P, BHx(P, ib, 1), 1) - Rx(P, BHx(P, ib, 0), 1);
  double norm = sqrt(dx * dx + dy * dy);
  nrm[0] = dy / norm; nrm[1] = -dx / norm;
}

/* edge f of a triangle: (0,1), (1,2), (2,0), MC2D.hpp:921 */
static const int kEdge2[3][2] = {{0, 1}, {1, 2}, {2, 0}};

/* Normal(el, f), MC2D.hpp:358-387 */
static void normal_f2(const vo_problem *P, int64_t el, int64_t f, double *nrm) {
  if (f < 0 || f > 2) { nrm[0] = nrm[1] = 0.0; return; }
  int64_t i0 = Hx(P, el, kEdge2[f][0]), i1 = Hx(P, el, kEdge2[f][1]);
  double dx = Rx(P, i1, 0) - Rx(P, i0, 0), dy = Rx(P, i1, 1) - Rx(P, i0, 1);
  double norm = sqrt(dx * dx + dy * dy);
  nrm[0] = dy / norm; nrm[1] = -dx / norm;
}

/* RayTriangleIntersects (Moller-Trumbore), MC3D.hpp:1825-1869 */
static int ray_tri(const double *O, const double *D, const double *V0, const double *V1,
                   const double *V2, double *t) {
  double e1[3] = {V1[0] - V0[0], V1[1] - V0[1], V1[2] - V0[2]};
  double e2[3] = {V2[0] - V0[0], V2[1] - V0[1], V2[2] - V0[2]};
  double pv[3] = {D[1] * e2[2] - D[2] * e2[1], D[2] * e2[0] - D[0] * e2[2], D[0] * e2[1] - D[1] * e2[0]};
  double det = e1[0] * pv[0] + e1[1] * pv[1] + e1[2] * pv[2];
  if ((-kEps < det) && (det < kEps)) return 0;
  double inv_det = 1.0 / det;
  double tv[3] = {O[0] - V0[0], O[1] - V0[1], O[2] - V0[2]};
  double u = (tv[0] * pv[0] + tv[1] * pv[1] + tv[2] * pv[2]) * inv_det;
  if ((u < 0.0) || (u > 1.0)) return 0;
  double qv[3] = {tv[1] * e1[2] - tv[2] * e1[1], tv[2] * e1[0] - tv[0] * e1[2], tv[0] * e1[1] - tv[1] * e1[0]};
  double v = (D[0] * qv[0] + D[1] * qv[1] + D[2] * qv[2]) * inv_det;
  if ((v < 0.0) || (u + v > 1.0)) return 0;
  *t = (e2[0] * qv[0] + e2[1] * qv[1] + e2[2] * qv[2]) * inv_det;
  return 1;
}

/* RayRayIntersects, MC2D.hpp:1710-1722 */
static int ray_seg(const double *R, const double *D, const double *U, const double *V, double *t) {
  double det = D[0] * (U[1] - V[1]) - D[1] * (U[0] - V[0]);
  if ((-kEps < det) && (det < kEps)) return 0;
  double s = (D[1] * (R[0] - U[0]) - D[0] * (R[1] - U[1])) / det;
  if ((s < 0.0) || (s > 1.0)) return 0;
  *t = ((R[1] - U[1]) * (U[0] - V[0]) - (R[0] - U[0]) * (U[1] - V[1])) / det;
  return 1;
}

/* ------------------------------------------------------------------------- */
/* setup                                                                      */
/* ------------------------------------------------------------------------- */

/* ErrorChecks, MC3D.hpp:460-571 and MC2D.hpp:390-513 (same order of checks) */
int vo_error_checks(const vo_problem *P) {
  if (P->n_g != P->Ne) return MCERR(E_SIZE_MISMATCH_G);
  if (P->n_mua != P->Ne) return MCERR(E_SIZE_MISMATCH_MUA);
  if (P->n_mus != P->Ne) return MCERR(E_SIZE_MISMATCH_MUS);
  if (P->n_n != P->Ne) return MCERR(E_SIZE_MISMATCH_N);
  if (P->n_BCn == 0) return MCERR(E_MISSING_BCN);
  if (P->n_BCn != P->Nb) return MCERR(E_SIZE_MISMATCH_BCN);
  if (P->n_BCType != P->Nb) return MCERR(E_SIZE_MISMATCH_BCTYPE);
  int has_ls = 0, has_g = 0;
  for (int64_t i = 0; i < P->n_BCType; i++) {
    if (P->BCType[i] != 'a') has_ls = 1;
    if (P->BCType[i] == 'g') has_g = 1;
  }
  if (!has_ls) return MCERR(E_NO_LIGHTSOURCE);
  if (P->dim == 2 && has_g && P->n_GaussianSigma != P->Nb) return MCERR(E_NO_GAUSSIAN_SIGMA);
  if (P->n_BCLNormal && P->n_BCLNormal != P->Nb) return MCERR(E_SIZE_MISMATCH_LIGHT_DIRECTION);
  if (P->n_BCLDT && P->n_BCLDT != P->Nb) return MCERR(E_SIZE_MISMATCH_LIGHT_DIRECTION_TYPE);
  int64_t nh = P->Ne * (P->dim + 1), nb = P->Nb * P->dim;
  for (int64_t i = 0; i < nh; i++)
    if (P->H[i] < 0 || P->H[i] >= P->Nr) return MCERR(E_INCONSISTENT_H);
  for (int64_t i = 0; i < nb; i++)
    if (P->BH[i] < 0 || P->BH[i] >= P->Nr) return MCERR(E_INCONSISTENT_BH);
  return VO_OK;
}

/* BuildNeighbourhoods (NEW_NHOOD branch), MC3D.hpp:835-871 with search_neighbor :740-832,
 * and MC2D.hpp:724-773 with :645-721.  Vertex -> incident (element | -1-boundary) lists,
 * filled in the reference's push order. */
int vo_build_neighbours(vo_problem *P) {
  const int D = P->dim, NF = D + 1;
  const int64_t Ne = P->Ne, Nb = P->Nb, Nr = P->Nr;
  int64_t *cnt = (int64_t *)calloc((size_t)Nr + 1, sizeof(int64_t));
  if (!cnt) return VO_ERR_NOMEM;
  for (int64_t i = 0; i < Ne; i++)
    for (int c = 0; c < NF; c++) cnt[Hx(P, i, c) + 1]++;
  for (int64_t i = 0; i < Nb; i++)
    for (int c = 0; c < D; c++) cnt[BHx(P, i, c) + 1]++;
  for (int64_t v = 0; v < Nr; v++) cnt[v + 1] += cnt[v];
  int64_t *fill = (int64_t *)malloc(sizeof(int64_t) * (size_t)(Nr + 1));
  int64_t *lst = (int64_t *)malloc(sizeof(int64_t) * (size_t)(cnt[Nr] + 1));
  if (!fill || !lst) { free(cnt); free(fill); free(lst); return VO_ERR_NOMEM; }
  memcpy(fill, cnt, sizeof(int64_t) * (size_t)(Nr + 1));
  for (int64_t i = 0; i < Ne; i++)
    for (int c = 0; c < NF; c++) lst[fill[Hx(P, i, c)]++] = i;
  for (int64_t i = 0; i < Nb; i++)
    for (int c = 0; c < D; c++) lst[fill[BHx(P, i, c)]++] = -1 - i;

  int status = VO_OK;
  const int dup_err = (D == 3) ? MCERR(E_INCONSISTENT_MESH_DUPLICATE_NEIGHBORS) : MCERR(E_INCONSISTENT_MESH);
  for (int64_t el = 0; el < Ne && status == VO_OK; el++) {
    for (int f = 0; f < NF; f++) HNx(P, el, f) = HN_UNSET;
    for (int cv = 0; cv < NF && status == VO_OK; cv++) {
      int64_t v = Hx(P, el, cv);
      for (int64_t q = cnt[v]; q < cnt[v + 1]; q++) {
        int64_t nb = lst[q];
        if (nb == el) continue;
        /* part[a]: vertex a of el belongs to the candidate */
        int part[4] = {0, 0, 0, 0};
        for (int a = 0; a < NF; a++) {
          int hit = 0;
          if (nb >= 0) {
            for (int b = 0; b < NF; b++) hit |= (Hx(P, el, a) == Hx(P, nb, b));
          } else {
            int64_t ib = -(nb + 1);
            for (int b = 0; b < D; b++) hit |= (Hx(P, el, a) == BHx(P, ib, b));
          }
          part[a] = hit;
        }
        for (int f = 0; f < NF; f++) {
          int ok;
          if (D == 3) ok = part[kFace3[f][0]] && part[kFace3[f][1]] && part[kFace3[f][2]];
          else ok = part[kEdge2[f][0]] && part[kEdge2[f][1]];
          if (!ok) continue;
          if (HNx(P, el, f) != HN_UNSET && HNx(P, el, f) != nb) { status = dup_err; break; }
          HNx(P, el, f) = nb;
        }
        if (status != VO_OK) break;
      }
    }
    if (status == VO_OK && D == 2) {
      for (int f = 0; f < 3; f++)
        if (HNx(P, el, f) == HN_UNSET) status = MCERR(E_MISSING_BOUNDARY);  /* MC2D.hpp:768-771 */
    }
  }
  free(cnt); free(fill); free(lst);
  return status;
}

static int is_source(int D, char t) {
  if (D == 3)  /* MC3D.hpp:957-959 */
    return t == 'l' || t == 'L' || t == 'i' || t == 'I' || t == 'c' || t == 'C' || t == 'p';
  return t == 'l' || t == 'i' || t == 'c' || t == 'g';  /* MC2D.hpp:865-868 */
}

/* BuildLightSource, MC3D.hpp:941-1002 / MC2D.hpp:851-911 */
int64_t vo_light_sources(vo_problem *P, int64_t *ls, int64_t *mother, double *cdf, int64_t cap) {
  const int D = P->dim, NF = D + 1;
  int64_t k = 0;
  for (int64_t i = 0; i < P->Ne; i++)
    for (int f = 0; f < NF; f++) {
      int64_t h = HNx(P, i, f);
      if (h <= -1) {
        int64_t ib = -1 - h;
        if (is_source(D, P->BCType[ib])) {
          if (k < cap) {
            ls[k] = ib; mother[k] = i;
            cdf[k] = (D == 3) ? area3(P, ib) : length2(P, ib);
          }
          k++;
        }
      }
    }
  if (k > cap) return k;
  for (int64_t i = 0; i < k; i++) cdf[i] *= P->n_BCIntensity ? P->BCIntensity[ls[i]] : 1.0;
  for (int64_t i = 1; i < k; i++) cdf[i] += cdf[i - 1];
  for (int64_t i = 0; i < k; i++) cdf[i] /= cdf[k - 1];
  return k;
}

/* Init's derived arrays and BCLNormal handling: MC3D.hpp:611-735, MC2D.hpp:553-640 */
static int engine_init(vo_problem *P, engine *E) {
  const int D = P->dim;
  memset(E, 0, sizeof(*E));
  E->P = P; E->D = D; E->NF = D + 1;
  E->omega = 2.0 * kPi * P->f;
  if (!P->hn_given) {
    int s = vo_build_neighbours(P);
    if (s) return s;
  }
  if (P->n_BCLDT == 0) {
    for (int64_t i = 0; i < P->Nb; i++) P->BCLightDirectionType[i] = 'n';
    P->n_BCLDT = P->Nb;
  }
  int64_t ns = vo_light_sources(P, NULL, NULL, NULL, 0);
  E->Ns = ns;
  E->ls = (int64_t *)malloc(sizeof(int64_t) * (size_t)(ns + 1));
  E->lsm = (int64_t *)malloc(sizeof(int64_t) * (size_t)(ns + 1));
  E->cdf = (double *)malloc(sizeof(double) * (size_t)(ns + 1));
  E->k = (double *)malloc(sizeof(double) * (size_t)(P->Ne + 1));
  E->g2 = (double *)malloc(sizeof(double) * (size_t)(P->Ne + 1));
  if (!E->ls || !E->lsm || !E->cdf || !E->k || !E->g2) return VO_ERR_NOMEM;
  vo_light_sources(P, E->ls, E->lsm, E->cdf, ns);
  /* the reference divides by CDF[Ns-1] and later indexes past the end when there is no
   * emitting face with positive weight (e.g. only 'm' or 3D 'g' faces); report it as such */
  if (ns == 0 || !(E->cdf[ns - 1] == E->cdf[ns - 1])) return MCERR(E_NO_LIGHTSOURCE);
  for (int64_t i = 0; i < P->Ne; i++) E->k[i] = E->omega / kC0 * P->n[i];
  for (int64_t i = 0; i < P->Ne; i++) E->g2[i] = sq(P->g[i]);
  E->BCI = P->n_BCIntensity ? P->BCIntensity : NULL;
  E->BCLDT = P->BCLightDirectionType;
  double *L = P->BCLNormal;
  const int64_t Nb = P->Nb;
  if (P->n_BCLNormal) {
    for (int64_t i = 0; i < Nb; i++) {
      if (D == 3) {
        double norm = sqrt(sq(L[i]) + sq(L[i + Nb]) + sq(L[i + 2 * Nb]));
        if (P->BCLightDirectionType[i] != 'n') continue;  /* MC3D.hpp:679-683 */
        L[i] /= norm; L[i + Nb] /= norm; L[i + 2 * Nb] /= norm;
      } else {
        double norm = sqrt(sq(L[i]) + sq(L[i + Nb]));
        L[i] /= norm; L[i + Nb] /= norm;
      }
    }
  }
  for (int64_t i = 0; i < Nb; i++) {
    if (P->BCLightDirectionType[i] != 'r' || !P->n_BCLNormal) continue;
    if (D == 3) {  /* MC3D.hpp:693-735 */
      double n[3], e1[3], e2[3];
      normal_b3(P, i, n);
      for (int c = 0; c < 3; c++) {
        e1[c] = Rx(P, BHx(P, i, 1), c) - Rx(P, BHx(P, i, 0), c);
        e2[c] = Rx(P, BHx(P, i, 2), c) - Rx(P, BHx(P, i, 0), c);
      }
      double dpn = n[0] * e1[0] + n[1] * e1[1] + n[2] * e1[2];
      for (int c = 0; c < 3; c++) e1[c] -= dpn * n[c];
      double norm = sqrt(e1[0] * e1[0] + e1[1] * e1[1] + e1[2] * e1[2]);
      for (int c = 0; c < 3; c++) e1[c] /= norm;
      dpn = n[0] * e2[0] + n[1] * e2[1] + n[2] * e2[2];
      double dp1 = e1[0] * e2[0] + e1[1] * e2[1] + e1[2] * e2[2];
      for (int c = 0; c < 3; c++) e2[c] -= dpn * n[c] + dp1 * e1[c];
      norm = sqrt(e2[0] * e2[0] + e2[1] * e2[1] + e2[2] * e2[2]);
      for (int c = 0; c < 3; c++) e2[c] /= norm;
      double ox = L[i], oy = L[i + Nb], oz = L[i + 2 * Nb];
      for (int c = 0; c < 3; c++) L[i + c * Nb] = ox * e1[c] + oy * e2[c] + oz * n[c];
    } else {  /* MC2D.hpp:625-640 */
      double n[2], t[2];
      normal_b2(P, i, n);
      t[0] = Rx(P, BHx(P, i, 1), 0) - Rx(P, BHx(P, i, 0), 0);
      t[1] = Rx(P, BHx(P, i, 1), 1) - Rx(P, BHx(P, i, 0), 1);
      double norm = sqrt(t[0] * t[0] + t[1] * t[1]);
      t[0] /= norm; t[1] /= norm;
      double ox = L[i], oy = L[i + Nb];
      L[i] = ox * t[0] + oy * n[0];
      L[i + Nb] = ox * t[1] + oy * n[1];
    }
  }
  E->BCLN = L;
  return VO_OK;
}

static void engine_free(engine *E) {
  free(E->ls); free(E->lsm); free(E->cdf); free(E->k); free(E->g2);
}

/* source face pick: first ib with xi < CDF[ib] (MC3D.hpp:1068-1070); the 2D clamp
 * (MC2D.hpp:969) is applied in 3D too, where the reference would read past the end */
static int64_t pick_source(const engine *E, double xi) {
  int64_t ib;
  for (ib = 0; ib < E->Ns; ib++)
    if (xi < E->cdf[ib]) break;
  if (ib > E->Ns - 1) ib = E->Ns - 1;
  return ib;
}

/* ------------------------------------------------------------------------- */
/* 3D photon functions                                                        */
/* ------------------------------------------------------------------------- */

/* CreatePhoton, MC3D.hpp:1060-1294 */
static void create3(const engine *E, worker *w, photon *ph) {
  const vo_problem *P = E->P;
  const int64_t Nb = P->Nb;
  double xi = UnifClosed(&w->u);
  double n[3], t[3], norm;
  int64_t s = pick_source(E, xi);
  ph->curel = E->lsm[s];
  int64_t ib = E->ls[s];
  ph->curface = -1;
  for (int f = 0; f < 4; f++)
    if (-1 - HNx(P, ph->curel, f) == ib) { ph->curface = f; break; }
  double r1 = UnifOpen(&w->u), r2 = UnifOpen(&w->u);
  for (int c = 0; c < 3; c++)
    ph->pos[c] = (1.0 - sqrt(r1)) * Rx(P, BHx(P, ib, 0), c) + sqrt(r1) * (1.0 - r2) * Rx(P, BHx(P, ib, 1), c) +
                 sqrt(r1) * r2 * Rx(P, BHx(P, ib, 2), c);
  normal_b3(P, ib, n);
  for (int c = 0; c < 3; c++)
    t[c] = (Rx(P, Hx(P, ph->curel, 0), c) + Rx(P, Hx(P, ph->curel, 1), c) + Rx(P, Hx(P, ph->curel, 2), c) +
            Rx(P, Hx(P, ph->curel, 3), c)) / 4.0 - ph->pos[c];
  norm = sqrt(t[0] * t[0] + t[1] * t[1] + t[2] * t[2]);
  t[0] /= norm; t[1] /= norm; t[2] /= norm;
  if (n[0] * t[0] + n[1] * t[1] + n[2] * t[2] < 0.0) { n[0] = -n[0]; n[1] = -n[1]; n[2] = -n[2]; }

  const char bt = P->BCType[ib];
  const char dt = E->BCLDT[ib];
  const double *L = E->BCLN;
  /* combinations the reference leaves undefined ('L'/'I' or 'p' with direction type 'n')
   * start along the inward normal here */
  ph->dir[0] = n[0]; ph->dir[1] = n[1]; ph->dir[2] = n[2];
  if (dt == 'n') {
    if (bt == 'l') {
      ph->dir[0] = n[0]; ph->dir[1] = n[1]; ph->dir[2] = n[2];
    } else if (bt == 'i') {
      double dot, rr[3], th, u;
      do {
        th = 2.0 * kPi * UnifHalfUp(&w->u);
        u = 2.0 * UnifClosed(&w->u) - 1.0;
        rr[0] = sqrt(1.0 - sq(u)) * cos(th);
        rr[1] = sqrt(1.0 - sq(u)) * sin(th);
        rr[2] = u;
        dot = n[0] * rr[0] + n[1] * rr[1] + n[2] * rr[2];
      } while (dot <= 0.0 && !w->u.tape_out);
      ph->dir[0] = rr[0]; ph->dir[1] = rr[1]; ph->dir[2] = rr[2];
    } else if (bt == 'c' || bt == 'C') {
      double phi, th, dpn, dp1, fv[3], e1[3], e2[3];
      for (int c = 0; c < 3; c++) {
        e1[c] = Rx(P, BHx(P, ib, 1), c) - Rx(P, BHx(P, ib, 0), c);
        e2[c] = Rx(P, BHx(P, ib, 2), c) - Rx(P, BHx(P, ib, 0), c);
      }
      phi = asin(2.0 * UnifOpen(&w->u) - 1.0);
      th = 2.0 * kPi * UnifClosed(&w->u);
      fv[0] = cos(phi); fv[1] = cos(th) * sin(phi); fv[2] = sin(th) * sin(phi);
      norm = sqrt(e1[0] * e1[0] + e1[1] * e1[1] + e1[2] * e1[2]);
      e1[0] /= norm; e1[1] /= norm; e1[2] /= norm;
      dpn = n[0] * e2[0] + n[1] * e2[1] + n[2] * e2[2];
      dp1 = e1[0] * e2[0] + e1[1] * e2[1] + e1[2] * e2[2];
      for (int c = 0; c < 3; c++) e2[c] -= dpn * n[c] + dp1 * e1[c];
      norm = sqrt(e2[0] * e2[0] + e2[1] * e2[1] + e2[2] * e2[2]);
      e2[0] /= norm; e2[1] /= norm; e2[2] /= norm;
      for (int c = 0; c < 3; c++) ph->dir[c] = fv[0] * n[c] + fv[1] * e1[c] + fv[2] * e2[c];
    }
  } else {
    if (bt == 'l' || bt == 'L') {
      ph->dir[0] = L[ib]; ph->dir[1] = L[ib + Nb]; ph->dir[2] = L[ib + 2 * Nb];
    } else if (bt == 'p') {  /* MC3D.hpp:1204-1218: pencil at the BCLNormal point */
      ph->dir[0] = n[0]; ph->dir[1] = n[1]; ph->dir[2] = n[2];
      ph->pos[0] = L[ib]; ph->pos[1] = L[ib + Nb]; ph->pos[2] = L[ib + 2 * Nb];
    } else if (bt == 'i' || bt == 'I') {
      double dot, rr[3], th, u;
      do {
        th = 2.0 * kPi * UnifHalfUp(&w->u);
        u = 2.0 * UnifClosed(&w->u) - 1.0;
        rr[0] = sqrt(1.0 - sq(u)) * cos(th);
        rr[1] = sqrt(1.0 - sq(u)) * sin(th);
        rr[2] = u;
        dot = n[0] * rr[0] + n[1] * rr[1] + n[2] * rr[2];
      } while (dot <= 0.0 && !w->u.tape_out);
      ph->dir[0] = rr[0]; ph->dir[1] = rr[1]; ph->dir[2] = rr[2];
    } else if (bt == 'c' || bt == 'C') {  /* MC3D.hpp:1237-1286 */
      double phi, th, dpn, dp1, fv[3], e1[3], e2[3], Ln[3] = {L[ib], L[ib + Nb], L[ib + 2 * Nb]};
      for (int c = 0; c < 3; c++) {
        e1[c] = Rx(P, BHx(P, ib, 1), c) - Rx(P, BHx(P, ib, 0), c);
        e2[c] = Rx(P, BHx(P, ib, 2), c) - Rx(P, BHx(P, ib, 0), c);
      }
      phi = asin(2.0 * UnifOpen(&w->u) - 1.0);
      th = 2.0 * kPi * UnifClosed(&w->u);
      fv[0] = cos(phi); fv[1] = cos(th) * sin(phi); fv[2] = sin(th) * sin(phi);
      dpn = Ln[0] * e1[0] + Ln[1] * e1[1] + Ln[2] * e1[2];
      for (int c = 0; c < 3; c++) e1[c] -= dpn * Ln[c];
      norm = sqrt(e1[0] * e1[0] + e1[1] * e1[1] + e1[2] * e1[2]);
      e1[0] /= norm; e1[1] /= norm; e1[2] /= norm;
      dpn = Ln[0] * e2[0] + Ln[1] * e2[1] + Ln[2] * e2[2];
      dp1 = e1[0] * e2[0] + e1[1] * e2[1] + e1[2] * e2[2];
      for (int c = 0; c < 3; c++) e2[c] -= dpn * Ln[c] + dp1 * e1[c];
      norm = sqrt(e2[0] * e2[0] + e2[1] * e2[1] + e2[2] * e2[2]);
      e2[0] /= norm; e2[1] /= norm; e2[2] /= norm;
      /* the reference maps the mean direction onto the face normal n, not BCLNormal */
      for (int c = 0; c < 3; c++) ph->dir[c] = fv[0] * n[c] + fv[1] * e1[c] + fv[2] * e2[c];
    }
  }
  ph->nextel = -1; ph->nextface = -1;
  ph->weight = 1.0;
  ph->phase = P->phase0;
}

/* WhichFace, MC3D.hpp:1006-1057 */
static int which_face3(const vo_problem *P, photon *ph, double *dist) {
  double V[4][3];
  for (int v = 0; v < 4; v++)
    for (int c = 0; c < 3; c++) V[v][c] = Rx(P, Hx(P, ph->curel, v), c);
  for (int f = 0; f < 4; f++) {
    if (ph->curface == f) continue;
    if (ray_tri(ph->pos, ph->dir, V[kFace3[f][0]], V[kFace3[f][1]], V[kFace3[f][2]], dist) && *dist > 0.0) {
      ph->nextface = f;
      ph->nextel = HNx(P, ph->curel, f);
      return f;
    }
  }
  return -1;
}

/* ScatterPhoton, MC3D.hpp:1297-1340 */
static void scatter3(const engine *E, worker *w, photon *ph) {
  const vo_problem *P = E->P;
  double xi, theta, phi, dxn, dyn, dzn;
  const int64_t el = ph->curel;
  if (P->g[el] != 0.0) {
    xi = UnifClosed(&w->u);
    if ((0.0 < xi) && (xi < 1.0))
      theta = acos((1.0 + E->g2[el] - sq((1.0 - E->g2[el]) / (1.0 - P->g[el] * (1.0 - 2.0 * xi)))) / (2.0 * P->g[el]));
    else
      theta = (1.0 - xi) * kPi;
  } else {
    theta = acos(2.0 * UnifClosed(&w->u) - 1.0);
  }
  phi = 2.0 * kPi * UnifClosed(&w->u);
  double *d = ph->dir;
  if (fabs(d[2]) > 0.999) {
    dxn = sin(theta) * cos(phi);
    dyn = sin(theta) * sin(phi);
    dzn = d[2] * cos(theta) / fabs(d[2]);
  } else {
    dxn = sin(theta) * (d[0] * d[2] * cos(phi) - d[1] * sin(phi)) / sqrt(1.0 - d[2] * d[2]) + d[0] * cos(theta);
    dyn = sin(theta) * (d[1] * d[2] * cos(phi) + d[0] * sin(phi)) / sqrt(1.0 - d[2] * d[2]) + d[1] * cos(theta);
    dzn = -sin(theta) * cos(phi) * sqrt(1.0 - d[2] * d[2]) + d[2] * cos(theta);
  }
  double norm = sqrt(dxn * dxn + dyn * dyn + dzn * dzn);
  dxn /= norm; dyn /= norm; dzn /= norm;
  d[0] = dxn; d[1] = dyn; d[2] = dzn;
  ph->curface = -1;
}

/* MirrorPhoton(ib), MC3D.hpp:1343-1351 */
static void mirror3(const vo_problem *P, photon *ph, int64_t ib) {
  double n[3];
  normal_b3(P, ib, n);
  double cdot = n[0] * ph->dir[0] + n[1] * ph->dir[1] + n[2] * ph->dir[2];
  for (int c = 0; c < 3; c++) ph->dir[c] -= 2.0 * cdot * n[c];
}

/* Fresnel R and the reflect/refract decision shared by 2D and 3D (MC3D.hpp:1397-1430) */
static int fresnel_core(urng *u, double nipnt, double costhi, double *costht_out, int *tir) {
  double s = 1.0 - sq(nipnt) * (1.0 - sq(costhi));
  if (s <= 0.0) { *tir = 1; return 1; }
  *tir = 0;
  double costht = sqrt(s);
  *costht_out = costht;
  double thi = (costhi > 0.0) ? acos(costhi) : acos(-costhi);
  double tht = acos(costht);
  double R;
  if (!(sin(thi + tht) > kEps))
    R = sq((nipnt - 1.0) / (nipnt + 1.0));
  else
    R = 0.5 * (sq(sin(thi - tht) / sin(thi + tht)) + sq(tan(thi - tht) / tan(thi + tht)));
  double xi = UnifClosed(u);
  return xi <= R;
}

/* FresnelPhoton, MC3D.hpp:1365-1447 */
static int fresnel3(const engine *E, worker *w, photon *ph) {
  const vo_problem *P = E->P;
  double nor[3];
  normal_f3(P, ph->curel, ph->nextface, nor);
  double nipnt = (ph->nextel < 0) ? P->n[ph->curel] / P->BCn[-1 - ph->nextel] : P->n[ph->curel] / P->n[ph->nextel];
  double costhi = -(ph->dir[0] * nor[0] + ph->dir[1] * nor[1] + ph->dir[2] * nor[2]);
  double costht = 0.0;
  int tir;
  if (fresnel_core(&w->u, nipnt, costhi, &costht, &tir)) {
    for (int c = 0; c < 3; c++) ph->dir[c] += 2.0 * costhi * nor[c];
    ph->curface = ph->nextface;
    return 1;
  }
  if (costhi > 0.0) {
    for (int c = 0; c < 3; c++) ph->dir[c] = nipnt * ph->dir[c] + (nipnt * costhi - costht) * nor[c];
  } else {
    for (int c = 0; c < 3; c++) ph->dir[c] = nipnt * ph->dir[c] + (nipnt * costhi + costht) * nor[c];
  }
  return 0;
}

/* roulette at an element crossing, MC3D.hpp:1578-1585 / :1597-1604; returns 1 if killed */
static int roulette(worker *w, photon *ph) {
  if (ph->weight < kWeight0) {
    if (UnifClosed(&w->u) > kChance) {
      w->ledger[VO_LG_ROULETTE_KILL] += ph->weight;
      return 1;
    }
    w->ledger[VO_LG_ROULETTE_GAIN] += ph->weight / kChance - ph->weight;
    ph->weight /= kChance;
  }
  return 0;
}

/* one element step's scoring and weight update, MC3D.hpp:1479-1526 (same in 2D) */
static void score_step(const engine *E, worker *w, photon *ph, double ds) {
  const vo_problem *P = E->P;
  const int64_t el = ph->curel;
  trace_ev(w, el);
  double att = exp(-P->mua[el] * ds);
  if (E->omega <= 0.0) {
    if (P->mua[el] > 0.0) {
      double dep = (1.0 - att) * ph->weight;
      w->ER[el] += dep;
      w->ledger[VO_LG_ABSORBED] += dep;
    } else {
      w->ER[el] += ph->weight * ds;
    }
  } else {
    double kds = E->k[el] * ds;
    w->ER[el] += ph->weight * (cos(ph->phase) - cos(-ph->phase - kds) * att);
    w->EI[el] += ph->weight * (-sin(ph->phase) + sin(ph->phase + kds) * att);
    ph->phase += kds;
    if (P->mua[el] > 0.0) w->ledger[VO_LG_ABSORBED] += (1.0 - att) * ph->weight;
  }
  ph->weight *= att;
}

/* PropagatePhoton, MC3D.hpp:1450-1638 */
static void propagate3(const engine *E, worker *w, photon *ph, int64_t max_steps) {
  const vo_problem *P = E->P;
  double prop, dist, ds;
  int64_t ib, nsteps = 0;
  for (;;) {
    prop = -log(UnifOpen(&w->u)) / P->mus[ph->curel];
    for (;;) {
      if (w->u.tape_out) { trace_ev(w, VO_EV_TAPE_END); return; }
      if (max_steps && nsteps >= max_steps) {
        w->capped++; w->ledger[VO_LG_LOST] += ph->weight; trace_ev(w, VO_EV_CAPPED); return;
      }
      if (which_face3(P, ph, &dist) == -1) {
        w->loss++; w->ledger[VO_LG_LOST] += ph->weight; trace_ev(w, VO_EV_LOST); return;
      }
      nsteps++; w->steps++;
      ds = fmin(prop, dist);
      for (int c = 0; c < 3; c++) ph->pos[c] += ph->dir[c] * ds;
      score_step(E, w, ph, ds);
      prop -= ds;
      if (prop <= 0.0) { u_align(&w->u); break; }
      if (ph->nextel < 0) {
        ib = -1 - ph->nextel;
        char bt = P->BCType[ib];
        if (bt == 'm' || bt == 'L' || bt == 'I' || bt == 'C') {
          mirror3(P, ph, ib);
          ph->curface = ph->nextface;
          continue;
        }
        if (P->BCn[ib] > 0.0)
          if (fresnel3(E, w, ph)) continue;
        if (E->omega <= 0.0) {
          w->EBR[ib] += ph->weight;
        } else {
          w->EBR[ib] += ph->weight * cos(ph->phase);
          w->EBI[ib] -= ph->weight * sin(ph->phase);
        }
        w->ledger[VO_LG_EXITED] += ph->weight;
        trace_ev(w, -1 - ib);
        return;
      }
      if (ph->nextel == HN_UNSET) {  /* open face left by the 3D builder (MC3D.hpp:863) */
        w->loss++; w->ledger[VO_LG_LOST] += ph->weight; trace_ev(w, VO_EV_LOST); return;
      }
      if ((P->mus[ph->curel] <= 0.0) && (P->mus[ph->nextel] > 0.0)) {
        prop = -log(UnifOpen(&w->u)) / P->mus[ph->nextel];
        if (roulette(w, ph)) { trace_ev(w, VO_EV_ROULETTE); return; }
        if (P->n[ph->curel] != P->n[ph->nextel])
          if (fresnel3(E, w, ph)) continue;
      } else {
        if (roulette(w, ph)) { trace_ev(w, VO_EV_ROULETTE); return; }
        if (P->n[ph->curel] != P->n[ph->nextel])
          if (fresnel3(E, w, ph)) continue;
        prop *= P->mus[ph->curel] / P->mus[ph->nextel];
      }
      int f;
      for (f = 0; f < 4; f++)
        if (HNx(P, ph->nextel, f) == ph->curel) break;
      if (f == 4) { w->loss++; w->ledger[VO_LG_LOST] += ph->weight; trace_ev(w, VO_EV_LOST); return; }
      ph->curface = f;
      ph->curel = ph->nextel;
    }
    if (P->mus[ph->curel] > 0.0) {
      scatter3(E, w, ph);
      w->scatters++;
    }
  }
}

/* ------------------------------------------------------------------------- */
/* 2D photon functions                                                        */
/* ------------------------------------------------------------------------- */

/* inverse of the truncated-Gaussian angular CDF by 16 bisection steps, MC2D.hpp:1044-1056 */
static double gauss_angle(double sigma, double xi) {
  double h = 0.5 - 0.5 * erf(kPi / sigma / 2.0 / sqrt(2.0));
  double a = -kPi / 2, b = kPi / 2, phi = 0.0, cdf;
  for (int it = 0; it < 16; it++) {
    phi = (a + b) / 2.0;
    cdf = (0.5 + 0.5 * erf(phi / sigma / sqrt(2.0)) - h) / (1 - 2.0 * h);
    if (cdf - xi < 0.0) a = phi;
    else b = phi;
  }
  return phi;
}

/* CreatePhoton, MC2D.hpp:958-1132 */
static void create2(const engine *E, worker *w, photon *ph) {
  const vo_problem *P = E->P;
  const int64_t Nb = P->Nb;
  double xi = UnifClosed(&w->u);
  double n[2], t[2], norm;
  int64_t s = pick_source(E, xi);
  ph->curel = E->lsm[s];
  int64_t ib = E->ls[s];
  ph->curface = -1;
  for (int f = 0; f < 3; f++)
    if (-1 - HNx(P, ph->curel, f) == ib) { ph->curface = f; break; }
  double wv = UnifOpen(&w->u);
  ph->pos[0] = Rx(P, BHx(P, ib, 0), 0) + wv * (Rx(P, BHx(P, ib, 1), 0) - Rx(P, BHx(P, ib, 0), 0));
  ph->pos[1] = Rx(P, BHx(P, ib, 0), 1) + wv * (Rx(P, BHx(P, ib, 1), 1) - Rx(P, BHx(P, ib, 0), 1));
  ph->pos[2] = 0.0;
  normal_b2(P, ib, n);
  t[0] = (Rx(P, Hx(P, ph->curel, 0), 0) + Rx(P, Hx(P, ph->curel, 1), 0) + Rx(P, Hx(P, ph->curel, 2), 0)) / 3.0 - ph->pos[0];
  t[1] = (Rx(P, Hx(P, ph->curel, 0), 1) + Rx(P, Hx(P, ph->curel, 1), 1) + Rx(P, Hx(P, ph->curel, 2), 1)) / 3.0 - ph->pos[1];
  norm = sqrt(t[0] * t[0] + t[1] * t[1]);
  t[0] /= norm; t[1] /= norm;
  if (n[0] * t[0] + n[1] * t[1] < 0.0) { n[0] = -n[0]; n[1] = -n[1]; }
  const char bt = P->BCType[ib];
  const char dt = E->BCLDT[ib];
  const double *L = E->BCLN;
  ph->dir[0] = n[0]; ph->dir[1] = n[1]; ph->dir[2] = 0.0;
  if (dt == 'n') {
    if (bt == 'l') {
      ph->dir[0] = n[0]; ph->dir[1] = n[1];
    } else if (bt == 'i') {
      double phi0 = atan2(n[1], n[0]);
      double phi = kPi * (UnifOpen(&w->u) - 0.5);
      ph->dir[0] = cos(phi0 + phi); ph->dir[1] = sin(phi0 + phi);
    } else if (bt == 'c') {
      double phi0 = atan2(n[1], n[0]);
      double phi = asin(2.0 * UnifOpen(&w->u) - 1.0);
      ph->dir[0] = cos(phi0 + phi); ph->dir[1] = sin(phi0 + phi);
    } else if (bt == 'g') {
      double phi0 = atan2(n[1], n[0]);
      double phi = gauss_angle(P->GaussianSigma[ib], UnifOpen(&w->u));
      ph->dir[0] = cos(phi0 + phi); ph->dir[1] = sin(phi0 + phi);
    }
  } else {
    if (bt == 'l') {
      ph->dir[0] = L[ib]; ph->dir[1] = L[ib + Nb];
    } else if (bt == 'i') {
      double phi0 = atan2(L[ib + Nb], L[ib]);
      double phi = kPi * (UnifOpen(&w->u) - 0.5);
      ph->dir[0] = cos(phi0 + phi); ph->dir[1] = sin(phi0 + phi);
    } else if (bt == 'c') {
      do {
        double phi0 = atan2(L[ib + Nb], L[ib]);
        double phi = asin(2.0 * UnifOpen(&w->u) - 1.0);
        ph->dir[0] = cos(phi0 + phi); ph->dir[1] = sin(phi0 + phi);
      } while (n[0] * ph->dir[0] + n[1] * ph->dir[1] <= 0.0 && !w->u.tape_out);
    } else if (bt == 'g') {
      do {
        double phi0 = atan2(L[ib + Nb], L[ib]);
        double phi = gauss_angle(P->GaussianSigma[ib], UnifOpen(&w->u));
        ph->dir[0] = cos(phi0 + phi); ph->dir[1] = sin(phi0 + phi);
      } while (n[0] * ph->dir[0] + n[1] * ph->dir[1] <= 0.0 && !w->u.tape_out);
    }
  }
  ph->nextel = -1; ph->nextface = -1;
  ph->weight = 1.0;
  ph->phase = P->phase0;
}

/* WhichFace, MC2D.hpp:914-955 */
static int which_face2(const vo_problem *P, photon *ph, double *dist) {
  double V[3][2];
  for (int v = 0; v < 3; v++)
    for (int c = 0; c < 2; c++) V[v][c] = Rx(P, Hx(P, ph->curel, v), c);
  for (int f = 0; f < 3; f++) {
    if (ph->curface == f) continue;
    if (ray_seg(ph->pos, ph->dir, V[kEdge2[f][0]], V[kEdge2[f][1]], dist) && *dist > 0.0) {
      ph->nextface = f;
      ph->nextel = HNx(P, ph->curel, f);
      return f;
    }
  }
  return -1;
}

/* ScatterPhoton, MC2D.hpp:1135-1155 */
static void scatter2(const engine *E, worker *w, photon *ph) {
  const vo_problem *P = E->P;
  const int64_t el = ph->curel;
  if (P->g[el] != 0.0) {
    double xi = UnifHalfUp(&w->u);
    double g = P->g[el], g2 = E->g2[el];
    double t = sqrt(sq(g2 + 1.0) - 4.0 * g2);
    double th = 2.0 * atan(tan(-xi * t * kPi / (g2 - 1.0)) * (g2 - 2 * g + 1.0) / t);
    double th0 = atan2(ph->dir[1], ph->dir[0]);
    ph->dir[0] = cos(th0 + th); ph->dir[1] = sin(th0 + th);
  } else {
    double th = 2.0 * kPi * UnifHalfUp(&w->u);
    ph->dir[0] = cos(th); ph->dir[1] = sin(th);
  }
  ph->curface = -1;
}

/* MirrorPhoton(ib), MC2D.hpp:1158-1165 */
static void mirror2(const vo_problem *P, photon *ph, int64_t ib) {
  double n[2];
  normal_b2(P, ib, n);
  double cdot = n[0] * ph->dir[0] + n[1] * ph->dir[1];
  ph->dir[0] -= 2.0 * cdot * n[0];
  ph->dir[1] -= 2.0 * cdot * n[1];
}

/* FresnelPhoton, MC2D.hpp:1178-1304: at the outer boundary a transmitted photon keeps
 * its direction */
static int fresnel2(const engine *E, worker *w, photon *ph) {
  const vo_problem *P = E->P;
  double nor[2];
  normal_f2(P, ph->curel, ph->nextface, nor);
  int boundary = ph->nextel < 0;
  double nipnt = boundary ? P->n[ph->curel] / P->BCn[-1 - ph->nextel] : P->n[ph->curel] / P->n[ph->nextel];
  double costhi = -(ph->dir[0] * nor[0] + ph->dir[1] * nor[1]);
  double costht = 0.0;
  int tir;
  if (fresnel_core(&w->u, nipnt, costhi, &costht, &tir)) {
    ph->dir[0] += 2.0 * costhi * nor[0];
    ph->dir[1] += 2.0 * costhi * nor[1];
    ph->curface = ph->nextface;
    return 1;
  }
  if (boundary) return 0;
  if (costhi > 0.0) {
    for (int c = 0; c < 2; c++) ph->dir[c] = nipnt * ph->dir[c] + (nipnt * costhi - costht) * nor[c];
  } else {
    for (int c = 0; c < 2; c++) ph->dir[c] = nipnt * ph->dir[c] + (nipnt * costhi + costht) * nor[c];
  }
  return 0;
}

/* PropagatePhoton, MC2D.hpp:1307-1511 */
static void propagate2(const engine *E, worker *w, photon *ph, int64_t max_steps) {
  const vo_problem *P = E->P;
  double prop, dist, ds;
  int64_t ib, nsteps = 0;
  for (;;) {
    prop = -log(UnifOpen(&w->u)) / P->mus[ph->curel];
    for (;;) {
      if (w->u.tape_out) { trace_ev(w, VO_EV_TAPE_END); return; }
      if (max_steps && nsteps >= max_steps) {
        w->capped++; w->ledger[VO_LG_LOST] += ph->weight; trace_ev(w, VO_EV_CAPPED); return;
      }
      if (which_face2(P, ph, &dist) == -1) {
        w->loss++; w->ledger[VO_LG_LOST] += ph->weight; trace_ev(w, VO_EV_LOST); return;
      }
      nsteps++; w->steps++;
      ds = fmin(prop, dist);
      ph->pos[0] += ph->dir[0] * ds;
      ph->pos[1] += ph->dir[1] * ds;
      score_step(E, w, ph, ds);
      prop -= ds;
      if (prop <= 0.0) { u_align(&w->u); break; }
      if (ph->nextel < 0) {
        ib = -1 - ph->nextel;
        char bt = P->BCType[ib];
        if (bt == 'm' || bt == 'L' || bt == 'I' || bt == 'C') {
          mirror2(P, ph, ib);
          ph->curface = ph->nextface;
          continue;
        }
        if (P->BCn[ib] > 0.0)
          if (fresnel2(E, w, ph)) continue;
        /* outward edge normal for the DEBR weighting, MC2D.hpp:1410-1423 */
        double n[2], t[2];
        normal_f2(P, ph->curel, ph->nextface, n);
        t[0] = (Rx(P, Hx(P, ph->curel, 0), 0) + Rx(P, Hx(P, ph->curel, 1), 0) + Rx(P, Hx(P, ph->curel, 2), 0)) / 3.0 - ph->pos[0];
        t[1] = (Rx(P, Hx(P, ph->curel, 0), 1) + Rx(P, Hx(P, ph->curel, 1), 1) + Rx(P, Hx(P, ph->curel, 2), 1)) / 3.0 - ph->pos[1];
        if (n[0] * t[0] + n[1] * t[1] > 0.0) { n[0] = -n[0]; n[1] = -n[1]; }
        double dn = ph->dir[0] * n[0] + ph->dir[1] * n[1];
        if (E->omega <= 0.0) {
          w->EBR[ib] += ph->weight;
          w->DEBR[ib] += ph->weight / dn;
        } else {
          w->EBR[ib] += ph->weight * cos(ph->phase);
          w->EBI[ib] -= ph->weight * sin(ph->phase);
          w->DEBR[ib] += ph->weight * cos(ph->phase) / dn;
          w->DEBI[ib] -= ph->weight * sin(ph->phase) / dn;
        }
        w->ledger[VO_LG_EXITED] += ph->weight;
        trace_ev(w, -1 - ib);
        return;
      }
      if ((P->mus[ph->curel] <= 0.0) && (P->mus[ph->nextel] > 0.0)) {
        prop = -log(UnifOpen(&w->u)) / P->mus[ph->nextel];
        if (roulette(w, ph)) { trace_ev(w, VO_EV_ROULETTE); return; }
        if (P->n[ph->curel] != P->n[ph->nextel])
          if (fresnel2(E, w, ph)) continue;
      } else {
        if (roulette(w, ph)) { trace_ev(w, VO_EV_ROULETTE); return; }
        if (P->n[ph->curel] != P->n[ph->nextel])
          if (fresnel2(E, w, ph)) continue;
        prop *= P->mus[ph->curel] / P->mus[ph->nextel];
      }
      int f;
      for (f = 0; f < 3; f++)
        if (HNx(P, ph->nextel, f) == ph->curel) break;
      if (f == 3) { w->loss++; w->ledger[VO_LG_LOST] += ph->weight; trace_ev(w, VO_EV_LOST); return; }
      ph->curface = f;
      ph->curel = ph->nextel;
    }
    if (P->mus[ph->curel] > 0.0) {
      scatter2(E, w, ph);
      w->scatters++;
    }
  }
}

/* ------------------------------------------------------------------------- */
/* MonteCarlo driver, MC3D.hpp:1641-1822 / MC2D.hpp:1514-1707                 */
/* ------------------------------------------------------------------------- */

int vo_max_threads(void) {
#ifdef _OPENMP
  return omp_get_max_threads();
#else
  return 1;
#endif
}

static double now_s(void) {
  struct timespec ts;
  clock_gettime(CLOCK_MONOTONIC, &ts);
  return (double)ts.tv_sec + 1e-9 * (double)ts.tv_nsec;
}

int vo_run(vo_problem *P) {
  if (P->dim != 2 && P->dim != 3) return VO_ERR_BAD_ARG;
  int s = vo_error_checks(P);
  if (s) return s;
  engine E;
  s = engine_init(P, &E);
  if (s) { engine_free(&E); return s; }
  const int D = P->dim;
  const int64_t Ne = P->Ne, Nb = P->Nb, N = P->Nphoton;
  int nthread = P->nthreads > 0 ? P->nthreads : 1;
  if (P->rng_kind == VO_RNG_TAPE || P->trace) nthread = 1;
  worker *W = (worker *)calloc((size_t)nthread, sizeof(worker));
  if (!W) { engine_free(&E); return VO_ERR_NOMEM; }
  int64_t *cnt = (int64_t *)calloc((size_t)nthread, sizeof(int64_t));
  int64_t *first = (int64_t *)calloc((size_t)nthread, sizeof(int64_t));
  int alloc_ok = cnt && first;
  for (int t = 0; t < nthread && alloc_ok; t++) {
    W[t].ER = (double *)calloc((size_t)Ne + 1, sizeof(double));
    W[t].EI = (double *)calloc((size_t)Ne + 1, sizeof(double));
    W[t].EBR = (double *)calloc((size_t)Nb + 1, sizeof(double));
    W[t].EBI = (double *)calloc((size_t)Nb + 1, sizeof(double));
    W[t].DEBR = (double *)calloc((size_t)Nb + 1, sizeof(double));
    W[t].DEBI = (double *)calloc((size_t)Nb + 1, sizeof(double));
    alloc_ok = W[t].ER && W[t].EI && W[t].EBR && W[t].EBI && W[t].DEBR && W[t].DEBI;
    W[t].u.kind = P->rng_kind;
    /* thread seed = seed * totalthreads + thread, MC3D.hpp:1658 (totalthreads = 1) */
    if (P->rng_kind == VO_RNG_MT) mt_seed(&W[t].u.mt, P->seed + (uint64_t)t);
    cnt[t] = N / nthread;
  }
  if (!alloc_ok) {
    for (int t = 0; t < nthread; t++) {
      free(W[t].ER); free(W[t].EI); free(W[t].EBR); free(W[t].EBI); free(W[t].DEBR); free(W[t].DEBI);
    }
    free(W); free(cnt); free(first); engine_free(&E);
    return VO_ERR_NOMEM;
  }
  cnt[nthread - 1] += N - (N / nthread) * nthread;  /* remainder to the last thread, :1663-1668 */
  for (int t = 1; t < nthread; t++) first[t] = first[t - 1] + cnt[t - 1];

  double t0 = now_s();
#pragma omp parallel for num_threads(nthread) schedule(static, 1)
  for (int t = 0; t < nthread; t++) {
    worker *w = &W[t];
    photon ph;
    memset(&ph, 0, sizeof(ph));
    for (int64_t i = 0; i < cnt[t]; i++) {
      int64_t p = first[t] + i;
      if (P->rng_kind == VO_RNG_PHILOX) philox_start(&w->u.ph, P->seed, P->stream, (uint64_t)(p + P->photon_offset));
      if (P->rng_kind == VO_RNG_TAPE) {
        w->u.tape = P->tape; w->u.tpos = P->tape_off[p]; w->u.tend = P->tape_off[p + 1]; w->u.tape_out = 0;
      }
      w->tracing = (P->trace && p < P->trace_photons);
      if (w->tracing) { w->tr = P->trace + p * P->trace_stride; w->trcap = P->trace_stride; w->trn = 0; }
      w->ledger[VO_LG_LAUNCHED] += 1.0;
      if (D == 3) { create3(&E, w, &ph); propagate3(&E, w, &ph, P->max_steps); }
      else { create2(&E, w, &ph); propagate2(&E, w, &ph, P->max_steps); }
      if (w->tracing) {
        if (w->trn > w->trcap) { w->tr[w->trcap - 1] = VO_EV_TRUNCATED; w->trn = w->trcap; }
        P->trace_len[p] = w->trn;
      }
    }
  }
  P->seconds = now_s() - t0;

  /* reduction in thread order, :1713-1748 */
  P->loss = P->steps = P->scatters = P->capped = 0;
  for (int k = 0; k < VO_LG_N; k++) P->ledger[k] = 0.0;
  for (int t = 0; t < nthread; t++) {
    P->loss += W[t].loss; P->steps += W[t].steps; P->scatters += W[t].scatters; P->capped += W[t].capped;
    for (int k = 0; k < VO_LG_N; k++) P->ledger[k] += W[t].ledger[k];
  }
  P->photons_done = N;
  for (int64_t i = 0; i < Ne; i++) {
    double a = 0.0, b = 0.0;
    for (int t = 0; t < nthread; t++) { a += W[t].ER[i]; b += W[t].EI[i]; }
    P->ER[i] = a; P->EI[i] = b;
  }
  for (int64_t i = 0; i < Nb; i++) {
    double a = 0.0, b = 0.0, c = 0.0, d = 0.0;
    for (int t = 0; t < nthread; t++) { a += W[t].EBR[i]; b += W[t].EBI[i]; c += W[t].DEBR[i]; d += W[t].DEBI[i]; }
    P->EBR[i] = a; P->EBI[i] = b;
    if (P->DEBR) P->DEBR[i] = c;
    if (P->DEBI) P->DEBI[i] = d;
  }
  /* normalisation, MC3D.hpp:1792-1818 / MC2D.hpp:1672-1703 */
  if (P->normalize) {
    const double Nd = (double)N;
    if (E.omega <= 0.0) {
      for (int64_t i = 0; i < Ne; i++) {
        double V = (D == 3) ? volume3(P, i) : area2(P, i);
        if (P->mua[i] > 0.0) P->ER[i] /= P->mua[i] * V * Nd;
        else P->ER[i] /= V * Nd;
      }
      for (int64_t i = 0; i < Nb; i++) {
        double A = (D == 3) ? area3(P, i) : length2(P, i);
        P->EBR[i] /= Nd * A;
        if (D == 2 && P->DEBR) P->DEBR[i] /= Nd * A;
      }
    } else {
      for (int64_t i = 0; i < Ne; i++) {
        double V = (D == 3) ? volume3(P, i) : area2(P, i);
        double a = P->ER[i], b = P->EI[i], k = E.k[i], mu = P->mua[i];
        P->ER[i] = (b * k + a * mu) / (sq(k) + sq(mu)) / Nd / V;
        P->EI[i] = -(a * k - b * mu) / (sq(k) + sq(mu)) / Nd / V;
      }
      for (int64_t i = 0; i < Nb; i++) {
        double A = (D == 3) ? area3(P, i) : length2(P, i);
        P->EBR[i] /= Nd * A;
        P->EBI[i] /= Nd * A;
        if (D == 2) {
          if (P->DEBR) P->DEBR[i] /= Nd * A;
          if (P->DEBI) P->DEBI[i] /= Nd * A;
        }
      }
    }
  }
  for (int t = 0; t < nthread; t++) {
    free(W[t].ER); free(W[t].EI); free(W[t].EBR); free(W[t].EBI); free(W[t].DEBR); free(W[t].DEBI);
  }
  free(W); free(cnt); free(first);
  engine_free(&E);
  return VO_OK;
}
