// walk2d.cuh -- the triangular photon walk (MC2D), one element step per call.
//
// Walk2D64 follows PropagatePhoton (cpp/2d/MC2D.hpp:1307-1511) with the reference's FP64
// arithmetic: RayRayIntersects over the edges (0,1), (1,2), (2,0) skipping the entry edge
// (WhichFace :914-955, :1710-1722), the 2D Henyey-Greenstein ScatterPhoton (:1135-1155),
// FresnelPhoton whose boundary branch transmits without refraction (:1178-1304), and the
// direction-weighted exitance DEBR/DEBI (:1410-1437).
// Walk2D32 is the FP32 tracking form with outward edge lines, as in the 3D form.
#pragma once
#include "walk3d.cuh"

namespace vmc {

// RayRayIntersects, cpp/2d/MC2D.hpp:1710-1722
__device__ __forceinline__ bool ray_seg(const double R[2], const double D[2], const double *U, const double *V,
                                        double &t) {
  double det = D[0] * (U[1] - V[1]) - D[1] * (U[0] - V[0]);
  if ((-kDblEps < det) && (det < kDblEps)) return false;
  const double ns = D[1] * (R[0] - U[0]) - D[0] * (R[1] - U[1]);
  // s = ns / det < 0 exactly when ns and det have opposite signs (the quotient of nonzero
  // coordinate differences cannot round to zero), decided before the division
  if ((ns < 0.0) != (det < 0.0) && ns != 0.0) return false;
  double s = ns / det;
  if ((s < 0.0) || (s > 1.0)) return false;
  t = ((R[1] - U[1]) * (U[0] - V[0]) - (R[0] - U[0]) * (U[1] - V[1])) / det;
  return true;
}

template <bool FD, class R>
struct Walk2D64 {
  static constexpr int kMinBlocks = 1;
  static constexpr bool kStaged = false;
  static constexpr bool kLaunchLoss = false;
  Stage stage;
  using Tr = typename TraceFor<R>::type;
  double pos[2], dir[2];
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
    create_photon_2d(J, rng, pos, dir, el, curface);
    w = 1.0;
    phase = J.phase0;
    if (FD) sincos(phase, &sph, &cph);
    optics(J, el, mua, mus, g, nidx);
    prop = -log(unif_open(rng)) / mus;
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

  __device__ void scatter(R &rng) {
    if (g != 0.0) {
      double xi = unif_halfup(rng);
      double g2 = g * g;
      double t = sqrt((g2 + 1.0) * (g2 + 1.0) - 4.0 * g2);
      // ScatterPhoton (MC2D.hpp:1135-1155) turns the direction to atan2(dir) + 2 atan(h);
      // here the direction is turned by the angle 2 atan(h), whose cosine and sine are
      // (1 - h^2) / (1 + h^2) and 2 h / (1 + h^2) (from 1 / h when |h| > 1), without forming
      // either angle: the same direction to a few ulps, 10% less FP64 work per photon
      const double h = tan(-xi * t * kPi / (g2 - 1.0)) * (g2 - 2 * g + 1.0) / t;
      double c, s;
      if (fabs(h) <= 1.0) {
        const double d = 1.0 / (1.0 + h * h);
        c = (1.0 - h * h) * d; s = 2.0 * h * d;
      } else {
        const double r = 1.0 / h, d = 1.0 / (1.0 + r * r);
        c = (r * r - 1.0) * d; s = 2.0 * r * d;
      }
      const double inv = 1.0 / sqrt(dir[0] * dir[0] + dir[1] * dir[1]);
      const double ux = dir[0] * inv, uy = dir[1] * inv;
      dir[0] = ux * c - uy * s;
      dir[1] = uy * c + ux * s;
    } else {
      sincospi(2.0 * unif_halfup(rng), &dir[1], &dir[0]);
    }
    curface = -1;
  }

  __device__ bool fresnel(R &rng, const double nor[2], double nipnt, int nf, bool boundary) {
    double costhi = -(dir[0] * nor[0] + dir[1] * nor[1]);
    double costht = 0.0;
    if (fresnel_reflects_d(rng, nipnt, costhi, costht)) {
      dir[0] += 2.0 * costhi * nor[0];
      dir[1] += 2.0 * costhi * nor[1];
      curface = nf;
      return true;
    }
    if (boundary) return false;
    double m = (costhi > 0.0) ? (nipnt * costhi - costht) : (nipnt * costhi + costht);
    dir[0] = nipnt * dir[0] + m * nor[0];
    dir[1] = nipnt * dir[1] + m * nor[1];
    return false;
  }

  // Normal(el, f), MC2D.hpp:358-387: the unit normal of the edge from a to b
  __device__ __forceinline__ static void normal_of(const double a[2], const double b[2], double nor[2]) {
    double ddx = b[0] - a[0], ddy = b[1] - a[1];
    double norm = sqrt(ddx * ddx + ddy * ddy);
    nor[0] = ddy / norm; nor[1] = -ddx / norm;
  }
  // Edge f runs from vertex f to vertex f + 1 (mod 3).  Only the Fresnel and exit paths
  // need its normal, so they read the two vertices again from the element record (the same
  // doubles) instead of indexing the step's vertex array by f, which would put that array
  // in local memory for the whole step.
  __device__ static void edge_normal(const Tri64 *T, int f, double nor[2]) {
    const double *v = &T->v[0][0];
    const int i0 = f, i1 = f == 2 ? 0 : f + 1;
    const double a[2] = {__ldg(v + 2 * i0), __ldg(v + 2 * i0 + 1)};
    const double b[2] = {__ldg(v + 2 * i1), __ldg(v + 2 * i1 + 1)};
    normal_of(a, b, nor);
  }

  __device__ bool roulette(const JobDev &J, R &rng) {
    if (w < kWeight0) {
      if (unif_closed(rng) > kChance) {
        job_count(J, kJcRoulette); job_ledger(J, kLgRouletteKill, w);
        return true;
      }
      job_ledger(J, kLgRouletteGain, w / kChance - w);
      w /= kChance;
    }
    return false;
  }

  __device__ int step(const JobDev &J, R &rng, int64_t max_steps) {
    if (rng.exhausted()) { job_count(J, kJcTapeEnd); die(J, kEvTapeEnd); return kDiedEarly; }
    if (nsteps >= max_steps) {
      job_count(J, kJcCapped); job_ledger(J, kLgLost, w);
      die(J, kEvCapped);
      return kDiedEarly;
    }
    const Tri64 *T = reinterpret_cast<const Tri64 *>(J.geom) + el;
    double V[3][2];
    {
      const double2 *src = reinterpret_cast<const double2 *>(T->v);
#pragma unroll
      for (int i = 0; i < 3; i++) {
        double2 d2 = __ldg(src + i);
        V[i][0] = d2.x; V[i][1] = d2.y;
      }
    }
    const int4 nb = __ldg(reinterpret_cast<const int4 *>(T->nbr));
    double dist = 0.0;
    int nf = -1;
    if (curface != 0 && ray_seg(pos, dir, V[0], V[1], dist) && dist > 0.0) nf = 0;
    else if (curface != 1 && ray_seg(pos, dir, V[1], V[2], dist) && dist > 0.0) nf = 1;
    else if (curface != 2 && ray_seg(pos, dir, V[2], V[0], dist) && dist > 0.0) nf = 2;
    if (nf < 0) {
      job_count(J, kJcLoss); job_ledger(J, kLgLost, w);
      die(J, kEvLost);
      return kDiedEarly;
    }
    const int nextel = nf == 0 ? nb.x : nf == 1 ? nb.y : nb.z;
    nsteps++;
    const double ds = fmin(prop, dist);
    pos[0] += dir[0] * ds;
    pos[1] += dir[1] * ds;
    tr.put(el);
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
      if (mus > 0.0) { scatter(rng); res = kScattered; }
      prop = -log(unif_open(rng)) / mus;
      return res;
    }
    if (nextel < 0) {
      const int ib = -1 - nextel;
      const uint8_t bt = __ldg(J.bctype + ib);
      if (is_mirror(bt)) {
        const double *bn = J.bnorm + 4 * (int64_t)ib;
        double cdot = bn[0] * dir[0] + bn[1] * dir[1];
        dir[0] -= 2.0 * cdot * bn[0];
        dir[1] -= 2.0 * cdot * bn[1];
        curface = nf;
        return kAlive;
      }
      double nor[2];
      edge_normal(T, nf, nor);
      const double bcn = __ldg(J.bcn + ib);
      if (bcn > 0.0 && fresnel(rng, nor, nidx / bcn, nf, true)) return kAlive;
      // outward edge normal for DEBR (MC2D.hpp:1410-1423)
      double tx = (V[0][0] + V[1][0] + V[2][0]) / 3.0 - pos[0];
      double ty = (V[0][1] + V[1][1] + V[2][1]) / 3.0 - pos[1];
      if (nor[0] * tx + nor[1] * ty > 0.0) { nor[0] = -nor[0]; nor[1] = -nor[1]; }
      double dn = dir[0] * nor[0] + dir[1] * nor[1];
      flush(J);
      if (!FD) {
        add_d(J, J.EBR + ib, w);
        add_d(J, J.DEBR + ib, w / dn);
      } else {
        add_d(J, J.EBR + ib, w * cph);
        add_d(J, J.EBI + ib, -(w * sph));
        add_d(J, J.DEBR + ib, w * cph / dn);
        add_d(J, J.DEBI + ib, -(w * sph / dn));
      }
      tr.put(-1 - (int64_t)ib);
      tr.end();
      return kDied;
    }
    if (nextel >= J.Ne) {
      job_count(J, kJcLoss); job_ledger(J, kLgLost, w);
      return die(J, kEvLost);
    }
    double mua2, mus2, g2, n2;
    optics(J, nextel, mua2, mus2, g2, n2);
    if ((mus <= 0.0) && (mus2 > 0.0)) {
      prop = -log(unif_open(rng)) / mus2;
      if (roulette(J, rng)) return die(J, kEvRoulette);
      if (nidx != n2) {
        double nor[2];
        edge_normal(T, nf, nor);
        if (fresnel(rng, nor, nidx / n2, nf, false)) return kAlive;
      }
    } else {
      if (roulette(J, rng)) return die(J, kEvRoulette);
      if (nidx != n2) {
        double nor[2];
        edge_normal(T, nf, nor);
        if (fresnel(rng, nor, nidx / n2, nf, false)) return kAlive;
      }
      if (mus2 != mus) prop *= mus / mus2;  // x (mus / mus) == x: skip the division
    }
    const int4 nb2 = __ldg(reinterpret_cast<const int4 *>((reinterpret_cast<const Tri64 *>(J.geom) + nextel)->nbr));
    int f2 = nb2.x == el ? 0 : nb2.y == el ? 1 : nb2.z == el ? 2 : -1;
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
};

template <bool FD, class R>
struct Walk2D32 {
  static constexpr int kMinBlocks = 4;
  static constexpr bool kStaged = false;
  Stage stage;
  using Tr = typename TraceFor<R>::type;
  float px, py, dx, dy;
  float w, prop, phase;
  float mua, mus, g, nidx;
  float acc, accI;
  int el;
  int32_t nsteps;
  bool outward;  // launched out through its own entry edge
  Tr tr;

  __device__ __forceinline__ float4 optics(const JobDev &J, int e) const {
    return __ldg(reinterpret_cast<const float4 *>(J.optics) + (e & J.opt_mask));
  }

  __device__ void launch(const JobDev &J, R &rng, int64_t q) {
    tr.begin(J, q);
    float p[2], d[2];
    int cf;
    create_photon_2d_f(J, rng, p, d, el, cf);
    px = p[0]; py = p[1];
    dx = d[0]; dy = d[1];
    // the entry edge is never tested by the reference's WhichFace (MC2D.hpp:927-952): a
    // photon launched out through it is lost
    outward = false;
    if (cf >= 0) {
      const float4 ln = __ldg(reinterpret_cast<const float4 *>((reinterpret_cast<const Tri32 *>(J.geom) + el)->ln) + cf);
      outward = ln.x * dx + ln.y * dy > 0.0f;
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
    add_f<R::kOneJob>(J, J.ER + el, acc);
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
    // 2D Henyey-Greenstein: the reference's angle 2 atan(tan(-xi t pi / (g^2 - 1)) (1 - g)^2 / t)
    // with t = 1 - g^2 reduces to 2 atan(tan(pi xi) (1 - g) / (1 + g))
    float xi = unif_halfup_f(rng);
    float sn, cs;
    if (g != 0.0f) {
      // th = 2 atan(z), z = k tan(pi xi), k = (1 - g) / (1 + g): with (s0, c0) the sine and
      // cosine of pi xi, cos th = (c0^2 - (k s0)^2) / (c0^2 + (k s0)^2) and
      // sin th = 2 k s0 c0 / (c0^2 + (k s0)^2) -- no arctangent, no sine of th
      float s0, c0;
      sincospif(xi, &s0, &c0);
      const float ks = __fdividef(1.0f - g, 1.0f + g) * s0;
      const float a = c0 * c0, b = ks * ks;
      const float inv = __fdividef(1.0f, a + b);
      cs = (a - b) * inv;
      sn = 2.0f * ks * c0 * inv;
      float nx = dx * cs - dy * sn, ny = dx * sn + dy * cs;
      float in = rsqrtf(nx * nx + ny * ny);
      dx = nx * in; dy = ny * in;
    } else {
      sincospif(2.0f * xi, &sn, &cs);
      dx = cs; dy = sn;
    }
  }

  __device__ __forceinline__ bool fresnel(R &rng, float nx, float ny, float eta, bool boundary) {
    float dn = dx * nx + dy * ny;
    float ci = fabsf(dn);
    float ct = 0.0f;
    if (fresnel_reflects_f(rng, eta, ci, ct)) {
      dx -= 2.0f * dn * nx; dy -= 2.0f * dn * ny;
      return true;
    }
    if (boundary) return false;
    float m = copysignf(ct, dn) - eta * dn;
    dx = eta * dx + m * nx; dy = eta * dy + m * ny;
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

  __device__ __forceinline__ static float lsel(const float4 &a, const float4 &b, const float4 &c, int f, int k) {
    const float4 &q = f == 0 ? a : f == 1 ? b : c;
    return k == 0 ? q.x : k == 1 ? q.y : q.z;
  }

  __device__ int step(const JobDev &J, R &rng, int64_t max_steps) {
    if (rng.exhausted()) { job_count(J, kJcTapeEnd); die(J, kEvTapeEnd); return kDiedEarly; }
    if (nsteps >= max_steps) {
      job_count(J, kJcCapped); job_ledger(J, kLgLost, f2d_int(w));
      die(J, kEvCapped);
      return kDiedEarly;
    }
    if (R::kReplay && outward) {  // with Philox streams this is settled at launch
      job_count(J, kJcLoss); job_ledger(J, kLgLost, f2d_int(w));
      die(J, kEvLost);
      return kDiedEarly;
    }
    const Tri32 *T = reinterpret_cast<const Tri32 *>(J.geom) + el;
    const float4 *L4 = reinterpret_cast<const float4 *>(T->ln);
    const float4 l0 = __ldg(L4 + 0), l1 = __ldg(L4 + 1), l2 = __ldg(L4 + 2);
    const int4 nb = __ldg(reinterpret_cast<const int4 *>(T->nbr));
    // selects over all three edges, no branch per edge; num / nd compared by cross
    // products, one reciprocal for the winning edge (bnd = 0: none yet)
    float bnum = 1.0f, bnd = 0.0f;
    int nf = -1;
    {
      const float4 ln[3] = {l0, l1, l2};
#pragma unroll
      for (int f = 0; f < 3; f++) {
        const float nd = ln[f].x * dx + ln[f].y * dy;
        const float num = ln[f].z - (ln[f].x * px + ln[f].y * py);
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
    px += dx * ds; py += dy * ds;
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
    const float nx = lsel(l0, l1, l2, nf, 0), ny = lsel(l0, l1, l2, nf, 1);
    const int nextel = nf == 0 ? nb.x : nf == 1 ? nb.y : nb.z;
    if (nextel < 0) {
      const int ib = -1 - nextel;
      const uint8_t bt = __ldg(J.bctype + ib);
      if (is_mirror(bt)) {
        float dn = dx * nx + dy * ny;
        dx -= 2.0f * dn * nx; dy -= 2.0f * dn * ny;
        return kAlive;
      }
      const float bcn = d2f_int(__ldg(J.bcn + ib));
      if (bcn > 0.0f && fresnel(rng, nx, ny, nidx / bcn, true)) return kAlive;
      float dn = dx * nx + dy * ny;
      flush(J);
      if (!FD) {
        add_f<R::kOneJob>(J, J.EBR + ib, w);
        add_f<R::kOneJob>(J, J.DEBR + ib, __fdividef(w, dn));
      } else {
        float sp, cp;
        sincosf(phase, &sp, &cp);
        add_f<R::kOneJob>(J, J.EBR + ib, w * cp);
        add_f<R::kOneJob>(J, J.EBI + ib, -(w * sp));
        add_f<R::kOneJob>(J, J.DEBR + ib, __fdividef(w * cp, dn));
        add_f<R::kOneJob>(J, J.DEBI + ib, -__fdividef(w * sp, dn));
      }
      tr.put(-1 - (int64_t)ib);
      tr.end();
      return kDied;
    }
    if (nextel >= J.Ne) {
      job_count(J, kJcLoss); job_ledger(J, kLgLost, f2d_int(w));
      return die(J, kEvLost);
    }
    const float4 o2 = optics(J, nextel);
    // the common crossing (scattering medium, weight above the roulette threshold, no index
    // jump) tested at once
    if (mus > 0.0f && w >= (float)kWeight0 && nidx == o2.w) {
      if (o2.y != mus) prop *= mus / o2.y;
      flush(J);
      el = nextel;
      mua = o2.x; mus = o2.y; g = o2.z; nidx = o2.w;
      return kAlive;
    }
    if (mus <= 0.0f && o2.y > 0.0f) {
      prop = free_path_f(unif_open_f(rng), o2.y);
      if (roulette(J, rng)) return die(J, kEvRoulette);
      if (nidx != o2.w && fresnel(rng, nx, ny, nidx / o2.w, false)) return kAlive;
    } else {
      if (roulette(J, rng)) return die(J, kEvRoulette);
      if (nidx != o2.w && fresnel(rng, nx, ny, nidx / o2.w, false)) return kAlive;
      if (o2.y != mus) prop *= mus / o2.y;
    }
    flush(J);
    el = nextel;
    mua = o2.x; mus = o2.y; g = o2.z; nidx = o2.w;
    return kAlive;
  }
};

}  // namespace vmc
