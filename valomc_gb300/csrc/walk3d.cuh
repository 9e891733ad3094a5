// walk3d.cuh -- the tetrahedral photon walk, one element step per call.
//
// Walk3D64: plain form.  Follows PropagatePhoton (cpp/3d/MC3D.hpp:1450-1638) with the
//   reference's FP64 arithmetic: Moller-Trumbore exit test over the faces in order,
//   skipping the entry face (WhichFace :1006-1057), Henyey-Greenstein ScatterPhoton
//   (:1297-1340; the polar cosine used as drawn, without acos / cos), FresnelPhoton with
//   the face normal from the vertices (:1365-1447),
//   MirrorPhoton (:1343-1351), roulette and the reverse-face lookup (:1573-1631).  Draw
//   order is the reference's, so a tape replay visits the same elements.
// Walk3D32: tracking form.  Position, direction and weight in FP32; the exit face is the
//   nearest of the faces the direction points out of, from precomputed outward planes
//   (the barycentric coordinate of the opposite vertex reaching zero), with the distance
//   clamped at 0 -- a photon cannot be lost to rounding.  Fluence is still accumulated
//   into FP64 arrays.
// Both merge consecutive deposits in one element in a register and flush them with one
// FP64 atomic when the photon leaves the element or dies.
#pragma once
#include "walk_common.cuh"

namespace vmc {

enum StepResult { kAlive = 0, kDied = 1, kScattered = 2, kDiedEarly = 3 };

// Moller-Trumbore (RayTriangleIntersects, cpp/3d/MC3D.hpp:1825-1869)
__device__ __forceinline__ bool ray_tri(const double O[3], const double D[3], const double *V0, const double *V1,
                                        const double *V2, double &t) {
  double e1[3] = {V1[0] - V0[0], V1[1] - V0[1], V1[2] - V0[2]};
  double e2[3] = {V2[0] - V0[0], V2[1] - V0[1], V2[2] - V0[2]};
  double pv[3] = {D[1] * e2[2] - D[2] * e2[1], D[2] * e2[0] - D[0] * e2[2], D[0] * e2[1] - D[1] * e2[0]};
  double det = e1[0] * pv[0] + e1[1] * pv[1] + e1[2] * pv[2];
  if ((-kDblEps < det) && (det < kDblEps)) return false;
  double tv[3] = {O[0] - V0[0], O[1] - V0[1], O[2] - V0[2]};
  double inv = 1.0 / det;
  double u = (tv[0] * pv[0] + tv[1] * pv[1] + tv[2] * pv[2]) * inv;
  if ((u < 0.0) || (u > 1.0)) return false;
  double qv[3] = {tv[1] * e1[2] - tv[2] * e1[1], tv[2] * e1[0] - tv[0] * e1[2], tv[0] * e1[1] - tv[1] * e1[0]};
  double v = (D[0] * qv[0] + D[1] * qv[1] + D[2] * qv[2]) * inv;
  if ((v < 0.0) || (u + v > 1.0)) return false;
  t = (e2[0] * qv[0] + e2[1] * qv[1] + e2[2] * qv[2]) * inv;
  return true;
}

// Fresnel reflect-or-transmit decision in FP64 (cpp/3d/MC3D.hpp:1397-1430).  Returns true
// when reflected.  costht is the transmitted cosine when false is returned.
template <class R>
__device__ __forceinline__ bool fresnel_reflects_d(R &rng, double nipnt, double costhi, double &costht) {
  double s = 1.0 - nipnt * nipnt * (1.0 - costhi * costhi);
  if (s <= 0.0) return true;
  costht = sqrt(s);
  double thi = acos(costhi > 0.0 ? costhi : -costhi);
  double tht = acos(costht);
  double refl;
  double sp = sin(thi + tht);
  if (!(sp > kDblEps)) {
    double q = (nipnt - 1.0) / (nipnt + 1.0);
    refl = q * q;
  } else {
    double a = sin(thi - tht) / sp, b = tan(thi - tht) / tan(thi + tht);
    refl = 0.5 * (a * a + b * b);
  }
  return unif_closed(rng) <= refl;
}

// Fresnel in FP32 from the closed forms rs = (eta ci - ct)/(eta ci + ct),
// rp = (ci - eta ct)/(ci + eta ct), R = (rs^2 + rp^2)/2 (same R as the reference's angle form).
template <class R>
__device__ __forceinline__ bool fresnel_reflects_f(R &rng, float eta, float ci, float &ct) {
  float s = 1.0f - eta * eta * (1.0f - ci * ci);
  if (s <= 0.0f) return true;
  ct = sqrtf(s);
  // a launch direction that is not unit length (3D BCLNormal of direction type 'a'/'r' is
  // not normalised, MC3D.hpp:679-683) can give |cos| > 1: acos is then NaN in the
  // reference, R is NaN and the photon is transmitted
  if (!(ci <= 1.0f)) return false;
  float rs = (eta * ci - ct) / (eta * ci + ct);
  float rp = (ci - eta * ct) / (ci + eta * ct);
  float Rf = 0.5f * (rs * rs + rp * rp);
  return unif_closed_f(rng) <= Rf;
}

__device__ __forceinline__ bool is_mirror(uint8_t bt) { return bt == 'm' || bt == 'L' || bt == 'I' || bt == 'C'; }

// 1 - exp(-x) for x >= 0 in FP32 without cancellation: below 0.1 the series to x^5
// (truncation x^6/720, relative x^5/720 < 1.4e-8); above, 1 - exp(-x) from the fast
// exponential (relative error < 2^-22 / (1 - e^-0.1) ~ 1.3e-6 at the cut, falling beyond).
__device__ __forceinline__ float one_minus_exp_neg(float x) {
  const float s = x * (1.0f + x * (-0.5f + x * (1.0f / 6.0f + x * (-1.0f / 24.0f + x * (1.0f / 120.0f)))));
  const float e = 1.0f - __expf(-x);
  return x < 0.1f ? s : e;  // a select, not a branch
}

// sin(t) for the per-step phase increments of the frequency-domain walk (|t| ~ 1e-3): the
// series to t^5 below 0.1 (relative error < t^6 / 5040 < 2e-10), the fast sine above.
__device__ __forceinline__ float sin_small(float t) {
  if (fabsf(t) < 0.1f) {
    const float t2 = t * t;
    return t * (1.0f + t2 * (-1.0f / 6.0f + t2 * (1.0f / 120.0f)));
  }
  return __sinf(t);
}

// The FP32 walks carry the phase reduced to [0, 2 pi) so that the fast sine and cosine
// keep their absolute accuracy (cos and sin of the reduced angle are those of the phase).
constexpr float kTwoPiF = 6.28318530717958647692f;
__device__ __forceinline__ float wrap_phase(float p) { return p >= kTwoPiF ? p - kTwoPiF : p; }

// distance to the next interaction, -log(U) / mus, with U in (0, 1).  The fast logarithm's
// absolute error (~1e-7) can make -log(U) of a U within 1e-7 of 1 come out at or just
// below zero; such a draw is an interaction at once, as it nearly is exactly.  The floor is
// 1e-30 rather than 0 so that a vacuum element (mus = 0) still gets an infinite path, as
// the reference's -log(U) / 0 does, and never 0 / 0.
__device__ __forceinline__ float free_path_f(float u, float mus) {
  return __fdividef(fmaxf(-__logf(u), 1e-30f), mus);
}

// =====================================================================================
// plain FP64 form
// =====================================================================================
template <bool FD, class R>
struct Walk3D64 {
  static constexpr int kMinBlocks = 1;  // ~125 registers: 2 CTAs of 256 per SM
  static constexpr bool kStaged = false;
  static constexpr bool kLaunchLoss = false;
  Stage stage;
  using Tr = typename TraceFor<R>::type;
  double pos[3], dir[3];
  double w, prop, phase, cph, sph;
  double mua, mus, g, nidx;
  double acc, accI;
  int el, curface;
  int64_t nsteps;
  Tr tr;

  __device__ __forceinline__ void optics(const JobDev &J, int e, double &a, double &s, double &gg, double &nn) const {
    const double2 *o = reinterpret_cast<const double2 *>(J.optics) + 2 * (int64_t)(e & J.opt_mask);
    const double2 o0 = __ldg(o), o1 = __ldg(o + 1);
    a = o0.x; s = o0.y; gg = o1.x; nn = o1.y;
  }

  __device__ void launch(const JobDev &J, R &rng, int64_t q) {
    tr.begin(J, q);
    create_photon_3d(J, rng, pos, dir, el, curface);
    w = 1.0;
    phase = J.phase0;
    if (FD) sincos(phase, &sph, &cph);
    optics(J, el, mua, mus, g, nidx);
    prop = -log(unif_open(rng)) / mus;  // the outer loop's first draw, MC3D.hpp:1458
    acc = accI = 0.0;
    nsteps = 0;
  }

  __device__ __forceinline__ void flush(const JobDev &J) {
    add_d(J, J.ER + el, acc);
    if (FD) add_d(J, J.EI + el, accI);
    acc = accI = 0.0;
  }

  __device__ __forceinline__ int die(const JobDev &J, int64_t ev) {
    flush(J);
    tr.put(ev);
    tr.end();
    return kDied;
  }

  __device__ void scatter(const JobDev &J, R &rng) {
    // ScatterPhoton, MC3D.hpp:1297-1340, without the round trip through the angle: the
    // reference draws theta = acos(c) from the HG inverse CDF c and takes sin and cos of it;
    // here cos theta is c itself and sin theta = sqrt(1 - c^2) (the same values to a few
    // ulps; |c| > 1 from rounding at the CDF's ends gives a NaN sine, as acos gives a NaN
    // angle), and the azimuth's sine and cosine come from sincospi(2 U).  The replays still
    // visit the reference's elements bit for bit; the FP64 pipe that bounds this form does
    // 10% less work.
    double ct;
    if (g != 0.0) {
      double xi = unif_closed(rng);
      if ((0.0 < xi) && (xi < 1.0)) {
        double g2 = g * g;
        double q = (1.0 - g2) / (1.0 - g * (1.0 - 2.0 * xi));
        ct = (1.0 + g2 - q * q) / (2.0 * g);
      } else {
        ct = xi > 0.5 ? 1.0 : -1.0;
      }
    } else {
      ct = 2.0 * unif_closed(rng) - 1.0;
    }
    const double st = sqrt(1.0 - ct * ct);
    double sp, cp;
    sincospi(2.0 * unif_closed(rng), &sp, &cp);
    double dxn, dyn, dzn;
    if (fabs(dir[2]) > 0.999) {
      dxn = st * cp;
      dyn = st * sp;
      dzn = dir[2] * ct / fabs(dir[2]);
    } else {
      double sq = sqrt(1.0 - dir[2] * dir[2]);
      const double isq = 1.0 / sq;
      dxn = st * (dir[0] * dir[2] * cp - dir[1] * sp) * isq + dir[0] * ct;
      dyn = st * (dir[1] * dir[2] * cp + dir[0] * sp) * isq + dir[1] * ct;
      dzn = -st * cp * sq + dir[2] * ct;
    }
    // one reciprocal for the three components (and one for the two 1 / sq above) instead of
    // a division each: the same direction to an ulp, 4.5% less FP64 work per photon
    const double inorm = 1.0 / sqrt(dxn * dxn + dyn * dyn + dzn * dzn);
    dir[0] = dxn * inorm; dir[1] = dyn * inorm; dir[2] = dzn * inorm;
    curface = -1;
  }

  // FresnelPhoton with the unoriented face normal nor (MC3D.hpp:1365-1447); true if reflected
  __device__ bool fresnel(R &rng, const double nor[3], double nipnt, int nf) {
    double costhi = -(dir[0] * nor[0] + dir[1] * nor[1] + dir[2] * nor[2]);
    double costht = 0.0;
    if (fresnel_reflects_d(rng, nipnt, costhi, costht)) {
#pragma unroll
      for (int c = 0; c < 3; c++) dir[c] += 2.0 * costhi * nor[c];
      curface = nf;
      return true;
    }
    double m = (costhi > 0.0) ? (nipnt * costhi - costht) : (nipnt * costhi + costht);
#pragma unroll
    for (int c = 0; c < 3; c++) dir[c] = nipnt * dir[c] + m * nor[c];
    return false;
  }

  __device__ int step(const JobDev &J, R &rng, int64_t max_steps) {
    if (rng.exhausted()) { job_count(J, kJcTapeEnd); die(J, kEvTapeEnd); return kDiedEarly; }
    if (nsteps >= max_steps) {
      job_count(J, kJcCapped); job_ledger(J, kLgLost, w);
      die(J, kEvCapped);
      return kDiedEarly;
    }
    const Tet64 *T = reinterpret_cast<const Tet64 *>(J.geom) + el;
    double V[4][3];
    {
      const double2 *src = reinterpret_cast<const double2 *>(T->v);
#pragma unroll
      for (int i = 0; i < 6; i++) {
        double2 d2 = __ldg(src + i);
        reinterpret_cast<double *>(V)[2 * i] = d2.x;
        reinterpret_cast<double *>(V)[2 * i + 1] = d2.y;
      }
    }
    const int4 nb = __ldg(reinterpret_cast<const int4 *>(T->nbr));
    // WhichFace: faces (0,1,2), (0,1,3), (0,2,3), (1,2,3) in order, skipping curface
    double dist = 0.0;
    int nf = -1;
    if (curface != 0 && ray_tri(pos, dir, V[0], V[1], V[2], dist) && dist > 0.0) nf = 0;
    else if (curface != 1 && ray_tri(pos, dir, V[0], V[1], V[3], dist) && dist > 0.0) nf = 1;
    else if (curface != 2 && ray_tri(pos, dir, V[0], V[2], V[3], dist) && dist > 0.0) nf = 2;
    else if (curface != 3 && ray_tri(pos, dir, V[1], V[2], V[3], dist) && dist > 0.0) nf = 3;
    if (nf < 0) {
      job_count(J, kJcLoss); job_ledger(J, kLgLost, w);
      die(J, kEvLost);
      return kDiedEarly;
    }
    const int nextel = nf == 0 ? nb.x : nf == 1 ? nb.y : nf == 2 ? nb.z : nb.w;
    nsteps++;
    const double ds = fmin(prop, dist);
#pragma unroll
    for (int c = 0; c < 3; c++) pos[c] += dir[c] * ds;
    tr.put(el);
    // element fluence, MC3D.hpp:1479-1526
    const double att = exp(-mua * ds);
    if (!FD) {
      if (mua > 0.0) acc += (1.0 - att) * w;
      else acc += w * ds;
    } else {
      const double kds = J.k_scale * nidx * ds;
      double sn, cn;
      sincos(phase + kds, &sn, &cn);
      acc += w * (cph - cn * att);
      accI += w * (-sph + sn * att);
      phase += kds;
      cph = cn; sph = sn;
    }
    w *= att;
    prop -= ds;
    if (prop <= 0.0) {
      int res = kAlive;
      rng.align();
      if (mus > 0.0) { scatter(J, rng); res = kScattered; }
      prop = -log(unif_open(rng)) / mus;
      return res;
    }
    if (nextel < 0) {
      const int ib = -1 - nextel;
      const uint8_t bt = __ldg(J.bctype + ib);
      if (is_mirror(bt)) {  // MirrorPhoton(ib) with Normal(ib)
        const double *bn = J.bnorm + 4 * (int64_t)ib;
        double cdot = bn[0] * dir[0] + bn[1] * dir[1] + bn[2] * dir[2];
#pragma unroll
        for (int c = 0; c < 3; c++) dir[c] -= 2.0 * cdot * bn[c];
        curface = nf;
        return kAlive;
      }
      const double bcn = __ldg(J.bcn + ib);
      if (bcn > 0.0) {
        double nor[3];
        face_normal(V, nf, nor);
        if (fresnel(rng, nor, nidx / bcn, nf)) return kAlive;
      }
      flush(J);
      if (!FD) add_d(J, J.EBR + ib, w);
      else { add_d(J, J.EBR + ib, w * cph); add_d(J, J.EBI + ib, -(w * sph)); }
      tr.put(-1 - (int64_t)ib);
      tr.end();
      return kDied;
    }
    if (nextel >= J.Ne) {  // open face: the reference would index past its arrays here
      job_count(J, kJcLoss); job_ledger(J, kLgLost, w);
      return die(J, kEvLost);
    }
    double mua2, mus2, g2, n2;
    optics(J, nextel, mua2, mus2, g2, n2);
    if ((mus <= 0.0) && (mus2 > 0.0)) {
      prop = -log(unif_open(rng)) / mus2;
      if (w < kWeight0) {
        if (unif_closed(rng) > kChance) {
          job_count(J, kJcRoulette); job_ledger(J, kLgRouletteKill, w);
          return die(J, kEvRoulette);
        }
        job_ledger(J, kLgRouletteGain, w / kChance - w);
        w /= kChance;
      }
      if (nidx != n2) {
        double nor[3];
        face_normal(V, nf, nor);
        if (fresnel(rng, nor, nidx / n2, nf)) return kAlive;
      }
    } else {
      if (w < kWeight0) {
        if (unif_closed(rng) > kChance) {
          job_count(J, kJcRoulette); job_ledger(J, kLgRouletteKill, w);
          return die(J, kEvRoulette);
        }
        job_ledger(J, kLgRouletteGain, w / kChance - w);
        w /= kChance;
      }
      if (nidx != n2) {
        double nor[3];
        face_normal(V, nf, nor);
        if (fresnel(rng, nor, nidx / n2, nf)) return kAlive;
      }
      if (mus2 != mus) prop *= mus / mus2;  // x (mus / mus) == x: skip the division
    }
    // reverse-face lookup, MC3D.hpp:1616-1628
    const int4 nb2 = __ldg(reinterpret_cast<const int4 *>((reinterpret_cast<const Tet64 *>(J.geom) + nextel)->nbr));
    int f2 = nb2.x == el ? 0 : nb2.y == el ? 1 : nb2.z == el ? 2 : nb2.w == el ? 3 : -1;
    if (f2 < 0) {
      job_count(J, kJcLoss); job_ledger(J, kLgLost, w);
      return die(J, kEvLost);
    }
    flush(J);
    curface = f2;
    el = nextel;
    mua = mua2; mus = mus2; g = g2; nidx = n2;
    return kAlive;
  }

  // Normal(el, f), MC3D.hpp:408-457: the unit normal of the face through vertices a, b, c
  __device__ __forceinline__ static void normal_of(const double a[3], const double b[3], const double c[3],
                                                   double nor[3]) {
    double x1 = b[0] - a[0], y1 = b[1] - a[1], z1 = b[2] - a[2];
    double x2 = c[0] - a[0], y2 = c[1] - a[1], z2 = c[2] - a[2];
    double nx = y1 * z2 - z1 * y2, ny = z1 * x2 - x1 * z2, nz = x1 * y2 - y1 * x2;
    double norm = sqrt(nx * nx + ny * ny + nz * nz);
    nor[0] = nx / norm; nor[1] = ny / norm; nor[2] = nz / norm;
  }
  // Face f of the tetrahedron is (0,1,2), (0,1,3), (0,2,3) or (1,2,3).  The index computed
  // from f puts the step's vertex array in local memory (an L1-resident store of 96 B per
  // step); keeping it in registers to the end of the step (constant indices per case), or
  // reading the vertices again on the Fresnel paths, takes more registers, halves the
  // resident CTAs and measured 5-15 % slower on the phantom, whose FP64 pipe is the bound.
  __device__ __forceinline__ static void face_normal(const double V[4][3], int f, double nor[3]) {
    const int i0 = f == 3 ? 1 : 0;
    const int i1 = f == 0 ? 1 : f == 1 ? 1 : 2;
    const int i2 = f == 0 ? 2 : 3;
    normal_of(V[i0], V[i1], V[i2], nor);
  }
};

// =====================================================================================
// FP32 tracking form
// =====================================================================================
template <bool FD, class R>
struct Walk3D32 {
  // 4 CTAs of 256 per SM (64 registers): the walk is latency bound and 32 resident warps
  // per SM beat 24 (+7% on the 648k-tet phantom); 5 CTAs (48 registers) spill and lose
  static constexpr int kMinBlocks = 4;
  static constexpr bool kStaged = !FD;
  using Tr = typename TraceFor<R>::type;
  float px, py, pz, dx, dy, dz;
  float w, prop, phase;
  float mua, mus, g, nidx;
  float acc, accI;
  int el;
  int32_t nsteps;
  bool outward;  // launched out through its own entry face
  Stage stage;   // shared-memory staging of ER deposits (continuous wave, single job)
  Tr tr;
  // Per-job forms (batched and served launches): the job's geometry and optics pointers,
  // optics index mask and element count, copied into registers at launch.  The one-job form
  // reads them as kernel-parameter operands; the per-job form would otherwise read them
  // from the job table on every step, the geometry pointer ahead of the record load on the
  // step's latency chain (2.7% on a two-job launch of the phantom; 56 -> 64 registers).
  const Tet32 *hg;
  const float4 *ho;
  int32_t hm, hne;

  __device__ __forceinline__ const Tet32 *geomp(const JobDev &J) const {
    if constexpr (R::kOneJob) return reinterpret_cast<const Tet32 *>(J.geom);
    else return hg;
  }
  __device__ __forceinline__ int32_t ne(const JobDev &J) const {
    if constexpr (R::kOneJob) return J.Ne;
    else return hne;
  }
  __device__ __forceinline__ float4 optics(const JobDev &J, int e) const {
    if constexpr (R::kOneJob) return __ldg(reinterpret_cast<const float4 *>(J.optics) + (e & J.opt_mask));
    else return __ldg(ho + (e & hm));
  }

  __device__ void launch(const JobDev &J, R &rng, int64_t q) {
    tr.begin(J, q);
    if constexpr (!R::kOneJob) {
      hg = reinterpret_cast<const Tet32 *>(J.geom);
      ho = reinterpret_cast<const float4 *>(J.optics);
      hm = J.opt_mask;
      hne = J.Ne;
    }
    float p[3], d[3];
    int cf;
    create_photon_3d_f(J, rng, p, d, el, cf);
    px = p[0]; py = p[1]; pz = p[2];
    dx = d[0]; dy = d[1]; dz = d[2];
    // The reference's WhichFace never tests the face a photon starts on, so a photon
    // launched pointing out of that face finds no exit and is lost (MC3D.hpp:1020-1056,
    // :1464-1468).  Keep that rule: the outward plane of the entry face decides.
    outward = false;
    if (cf >= 0) {
      const float4 pl = __ldg(reinterpret_cast<const float4 *>((reinterpret_cast<const Tet32 *>(J.geom) + el)->pl) + cf);
      outward = pl.x * dx + pl.y * dy + pl.z * dz > 0.0f;
    }
    w = 1.0f;
    phase = fmodf(d2f_int(J.phase0), kTwoPiF);
    float4 o = optics(J, el);
    mua = o.x; mus = o.y; g = o.z; nidx = o.w;
    prop = free_path_f(unif_open_f(rng), mus);
    acc = accI = 0.0f;
    nsteps = 0;
  }

  __device__ __forceinline__ void flush(const JobDev &J) {
    if (!FD) add_staged<R::kOneJob>(stage, J, el, acc);
    else add_f<R::kOneJob>(J, J.ER + el, acc);
    if (FD) add_f<R::kOneJob>(J, J.EI + el, accI);
    acc = accI = 0.0f;
  }

  __device__ __forceinline__ int die(const JobDev &J, int64_t ev) {
    flush(J);
    tr.put(ev);
    tr.end();
    return kDied;
  }

  // Philox streams: a photon launched out through its own entry face is lost before its
  // first step (as the step would find it), so the step needs no test for it
  static constexpr bool kLaunchLoss = !R::kReplay;
  __device__ __forceinline__ bool lost_at_launch(const JobDev &J) {
    if (!outward) return false;
    job_count(J, kJcLoss); job_ledger(J, kLgLost, f2d_int(w));
    die(J, kEvLost);
    return true;
  }

  __device__ __forceinline__ void scatter(R &rng) {
    // Henyey-Greenstein: cos(theta) from the inverse CDF, phi uniform; same rotation as
    // ScatterPhoton (MC3D.hpp:1316-1332)
    float xi = unif_closed_f(rng);
    float ct;
    if (g != 0.0f) {
      if (xi > 0.0f && xi < 1.0f) {
        // (1 + g^2 - q^2) / (2 g) with q = (1 - g^2) / D, D = 1 - g + 2 g xi, over one
        // division: ((1 + g^2) D^2 - (1 - g^2)^2) / (2 g D^2)
        const float D = 1.0f - g + 2.0f * g * xi;
        const float a = 1.0f - g * g;
        const float D2 = D * D;
        ct = __fdividef((1.0f + g * g) * D2 - a * a, 2.0f * g * D2);
      } else {
        ct = xi > 0.5f ? 1.0f : -1.0f;  // theta = (1 - xi) pi at xi in {0, 1}
      }
    } else {
      ct = 2.0f * xi - 1.0f;
    }
    ct = fminf(1.0f, fmaxf(-1.0f, ct));
    const float s2 = fmaxf(0.0f, 1.0f - ct * ct);
    const float st = s2 > 0.0f ? s2 * rsqrtf(s2) : 0.0f;
    float sp, cp;
    // phi uniform on [-pi, pi] (the reference's [0, 2 pi] shifted; same distribution)
    __sincosf((float)kPi * (2.0f * unif_closed_f(rng) - 1.0f), &sp, &cp);
    float nx, ny, nz;
    {
      // the general rotation and the near-pole case (|dz| > 0.999) as selects, no branch
      const bool pole = fabsf(dz) > 0.999f;
      const float s2z = pole ? 1.0f : 1.0f - dz * dz;
      const float isq = rsqrtf(s2z);
      const float sq = s2z * isq;
      const float rx = st * (dx * dz * cp - dy * sp) * isq + dx * ct;
      const float ry = st * (dy * dz * cp + dx * sp) * isq + dy * ct;
      const float rz = -st * cp * sq + dz * ct;
      nx = pole ? st * cp : rx;
      ny = pole ? st * sp : ry;
      nz = pole ? (dz > 0.0f ? ct : -ct) : rz;  // cos(theta) times the sign of dz (not |cos| with that sign)
    }
    float in = rsqrtf(nx * nx + ny * ny + nz * nz);
    dx = nx * in; dy = ny * in; dz = nz * in;
  }

  // true if reflected; N is the outward unit normal of the face being crossed
  __device__ __forceinline__ bool fresnel(R &rng, float nx, float ny, float nz, float eta) {
    float dn = dx * nx + dy * ny + dz * nz;  // > 0: leaving through the face
    float ci = fabsf(dn);
    float ct = 0.0f;
    if (fresnel_reflects_f(rng, eta, ci, ct)) {
      dx -= 2.0f * dn * nx; dy -= 2.0f * dn * ny; dz -= 2.0f * dn * nz;
      return true;
    }
    // refraction: d' = eta d + (ct - eta ci) s N with s the side the photon moves to
    float m = copysignf(ct, dn) - eta * dn;
    dx = eta * dx + m * nx; dy = eta * dy + m * ny; dz = eta * dz + m * nz;
    return false;
  }

  __device__ __forceinline__ bool roulette(const JobDev &J, R &rng) {
    if (w < (float)kWeight0) {
      if (unif_closed_f(rng) > (float)kChance) {
        job_count(J, kJcRoulette); job_ledger(J, kLgRouletteKill, f2d_int(w));
        return true;
      }
      float nw = w * 10.0f;
      job_ledger(J, kLgRouletteGain, f2d_int(nw) - f2d_int(w));
      w = nw;
    }
    return false;
  }

  __device__ int step(const JobDev &J, R &rng, int64_t max_steps) {
    if (rng.exhausted()) { job_count(J, kJcTapeEnd); die(J, kEvTapeEnd); return kDiedEarly; }
    if (nsteps >= (int32_t)min(max_steps, (int64_t)INT32_MAX)) {  // a 32-bit compare (loop invariant bound)
      job_count(J, kJcCapped); job_ledger(J, kLgLost, f2d_int(w));
      die(J, kEvCapped);
      return kDiedEarly;
    }
    if (R::kReplay && outward) {  // with Philox streams this is settled at launch
      job_count(J, kJcLoss); job_ledger(J, kLgLost, f2d_int(w));
      die(J, kEvLost);
      return kDiedEarly;
    }
    const Tet32 *T = geomp(J) + el;
    const float4 *P4 = reinterpret_cast<const float4 *>(T->pl);
    const float4 p0 = __ldg(P4 + 0), p1 = __ldg(P4 + 1), p2 = __ldg(P4 + 2), p3 = __ldg(P4 + 3);
    const int4 nb = __ldg(reinterpret_cast<const int4 *>(T->nbr));
    // exit: nearest face the direction points out of, as selects over all four faces (no
    // branch per face: fewer divergent regions and 6 fewer registers).  The distances
    // num / nd (nd > 0) are compared as num_f bnd < bnum nd_f, so that only the winning
    // face's quotient is computed: one reciprocal per step instead of four (bnd = 0 stands
    // for "none yet")
    float bnum = 1.0f, bnd = 0.0f;
    int nf = -1;
    {
      const float4 pl[4] = {p0, p1, p2, p3};
#pragma unroll
      for (int f = 0; f < 4; f++) {
        const float nd = pl[f].x * dx + pl[f].y * dy + pl[f].z * dz;
        const float num = pl[f].w - (pl[f].x * px + pl[f].y * py + pl[f].z * pz);
        const bool better = nd > 0.0f && num * bnd < bnum * nd;
        bnum = better ? num : bnum;
        bnd = better ? nd : bnd;
        nf = better ? f : nf;
      }
    }
    const float best = __fdividef(bnum, bnd);
    if (nf < 0) {
      job_count(J, kJcLoss); job_ledger(J, kLgLost, f2d_int(w));
      die(J, kEvLost);
      return kDiedEarly;
    }
    nsteps++;
    const float dist = fmaxf(best, 0.0f);
    const float ds = fminf(prop, dist);
    // a photon that leaves the element: fetch the next element's optics now, so that the
    // load runs under the deposit arithmetic
    const int nextel = nf == 0 ? nb.x : nf == 1 ? nb.y : nf == 2 ? nb.z : nb.w;
    float4 o2 = make_float4(0.f, 0.f, 0.f, 0.f);
    if (prop > dist && (unsigned)nextel < (unsigned)ne(J)) o2 = optics(J, nextel);
    px += dx * ds; py += dy * ds; pz += dz * ds;
    tr.put(el);
    const float x = mua * ds;
    if (!FD) {
      if (mua > 0.0f) {
        float dep = w * one_minus_exp_neg(x);
        acc += dep;
        w -= dep;
      } else {
        acc += w * ds;
      }
    } else {
      // w (cos phi - cos(phi + k ds) a) and w (-sin phi + sin(phi + k ds) a), a = exp(-mua ds),
      // written so that neither difference cancels: 1 - a cos(th) = (1 - a) + 2 a sin^2(th/2)
      const float th = J.k_scale_f * nidx * ds;
      const float om = one_minus_exp_neg(x);
      const float a = 1.0f - om;
      const float sh = sin_small(0.5f * th);
      const float c1 = om + 2.0f * a * sh * sh;
      const float s1 = a * sin_small(th);
      float sp, cp;
      __sincosf(phase, &sp, &cp);
      acc += w * (cp * c1 + sp * s1);
      accI += w * (cp * s1 - sp * c1);
      phase = wrap_phase(phase + th);
      w *= a;
    }
    prop -= ds;
    if (prop <= 0.0f) {
      int res = kAlive;
      rng.align();
      if (mus > 0.0f) { scatter(rng); res = kScattered; }
      prop = free_path_f(unif_open_f(rng), mus);
      return res;
    }
    // the crossed face's plane, only on the (rare) mirror and Fresnel paths
    auto face = [&]() { return nf == 0 ? p0 : nf == 1 ? p1 : nf == 2 ? p2 : p3; };
    if (nextel < 0) {
      const int ib = -1 - nextel;
      const uint8_t bt = __ldg(J.bctype + ib);
      if (is_mirror(bt)) {
        const float4 pf = face();
        float dn = dx * pf.x + dy * pf.y + dz * pf.z;
        dx -= 2.0f * dn * pf.x; dy -= 2.0f * dn * pf.y; dz -= 2.0f * dn * pf.z;
        return kAlive;
      }
      const float bcn = d2f_int(__ldg(J.bcn + ib));
      if (bcn > 0.0f) {
        const float4 pf = face();
        if (fresnel(rng, pf.x, pf.y, pf.z, nidx / bcn)) return kAlive;
      }
      flush(J);
      if (!FD) add_f<R::kOneJob>(J, J.EBR + ib, w);
      else {
        float sp, cp;
        sincosf(phase, &sp, &cp);
        add_f<R::kOneJob>(J, J.EBR + ib, w * cp);
        add_f<R::kOneJob>(J, J.EBI + ib, -(w * sp));
      }
      tr.put(-1 - (int64_t)ib);
      tr.end();
      return kDied;
    }
    // the common crossing (interior, scattering medium, weight above the roulette
    // threshold, no index jump) tested at once
    if (nextel < ne(J) && mus > 0.0f && w >= (float)kWeight0 && nidx == o2.w) {
      if (o2.y != mus) prop *= mus / o2.y;
      flush(J);
      el = nextel;
      mua = o2.x; mus = o2.y; g = o2.z; nidx = o2.w;
      return kAlive;
    }
    if (nextel >= J.Ne) {
      job_count(J, kJcLoss); job_ledger(J, kLgLost, f2d_int(w));
      return die(J, kEvLost);
    }
    if (mus <= 0.0f && o2.y > 0.0f) {
      prop = free_path_f(unif_open_f(rng), o2.y);
      if (roulette(J, rng)) return die(J, kEvRoulette);
      if (nidx != o2.w) {
        const float4 pf = face();
        if (fresnel(rng, pf.x, pf.y, pf.z, nidx / o2.w)) return kAlive;
      }
    } else {
      if (roulette(J, rng)) return die(J, kEvRoulette);
      if (nidx != o2.w) {
        const float4 pf = face();
        if (fresnel(rng, pf.x, pf.y, pf.z, nidx / o2.w)) return kAlive;
      }
      if (o2.y != mus) prop *= mus / o2.y;
    }
    flush(J);
    el = nextel;
    mua = o2.x; mus = o2.y; g = o2.z; nidx = o2.w;
    return kAlive;
  }
};

}  // namespace vmc
