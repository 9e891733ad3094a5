// host_setup.cpp -- ErrorChecks / Init / normalisation of the reference engines, restated
// for the GPU path.  Each function cites the reference lines it follows.
#include "host_setup.hpp"

#include <math.h>
#include <string.h>

#include <algorithm>
#include <limits>

#ifdef _OPENMP
#include <omp.h>
#endif

namespace vmc {

namespace {

// mcerror, cpp/Errors.hpp:4-21 (status = 1 + value)
enum {
  E_NO_LIGHTSOURCE = 1, E_SIZE_MISMATCH_G, E_SIZE_MISMATCH_MUA, E_SIZE_MISMATCH_MUS, E_SIZE_MISMATCH_N,
  E_SIZE_MISMATCH_BCN, E_MISSING_BCN, E_SIZE_MISMATCH_BCTYPE, E_SIZE_MISMATCH_LIGHT_DIRECTION,
  E_SIZE_MISMATCH_LIGHT_DIRECTION_TYPE, E_INCONSISTENT_H, E_INCONSISTENT_BH, E_INCONSISTENT_MESH,
  E_INCONSISTENT_MESH_DUPLICATE_NEIGHBORS, E_NO_GAUSSIAN_SIGMA, E_MISSING_BOUNDARY
};

inline double sq(double x) { return x * x; }  // pow(x, 2)

const int kFace3[4][3] = {{0, 1, 2}, {0, 1, 3}, {0, 2, 3}, {1, 2, 3}};  // MC3D.hpp:1013
const int kOpp3[4] = {3, 2, 1, 0};
const int kEdge2[3][2] = {{0, 1}, {1, 2}, {2, 0}};  // MC2D.hpp:921
const int kOpp2[3] = {2, 0, 1};

struct Geo {
  const int64_t *H, *BH;
  const double *r;
  int64_t Ne, Nb, Nr;
  int64_t h(int64_t el, int c) const { return H[el + Ne * c]; }
  int64_t bh(int64_t ib, int c) const { return BH[ib + Nb * c]; }
  double x(int64_t i, int c) const { return r[i + Nr * c]; }
};

// ElementVolume, MC3D.hpp:306-332
double volume3(const Geo &G, int64_t el) {
  double ax = G.x(G.h(el, 0), 0), ay = G.x(G.h(el, 0), 1), az = G.x(G.h(el, 0), 2);
  double bx = G.x(G.h(el, 1), 0), by = G.x(G.h(el, 1), 1), bz = G.x(G.h(el, 1), 2);
  double cx = G.x(G.h(el, 2), 0), cy = G.x(G.h(el, 2), 1), cz = G.x(G.h(el, 2), 2);
  double dx = G.x(G.h(el, 3), 0), dy = G.x(G.h(el, 3), 1), dz = G.x(G.h(el, 3), 2);
  double vol = (ax - dx) * ((by - dy) * (cz - dz) - (bz - dz) * (cy - dy)) -
               (ay - dy) * ((bx - dx) * (cz - dz) - (bz - dz) * (cx - dx)) +
               (az - dz) * ((bx - dx) * (cy - dy) - (by - dy) * (cx - dx));
  return fabs(vol) / 6.0;
}

// ElementArea(ib), MC3D.hpp:335-343
double area3(const Geo &G, int64_t ib) {
  int64_t i0 = G.bh(ib, 0), i1 = G.bh(ib, 1), i2 = G.bh(ib, 2);
  double a = sqrt(sq(G.x(i1, 0) - G.x(i0, 0)) + sq(G.x(i1, 1) - G.x(i0, 1)) + sq(G.x(i1, 2) - G.x(i0, 2)));
  double b = sqrt(sq(G.x(i2, 0) - G.x(i0, 0)) + sq(G.x(i2, 1) - G.x(i0, 1)) + sq(G.x(i2, 2) - G.x(i0, 2)));
  double c = sqrt(sq(G.x(i1, 0) - G.x(i2, 0)) + sq(G.x(i1, 1) - G.x(i2, 1)) + sq(G.x(i1, 2) - G.x(i2, 2)));
  return sqrt((a + b + c) * (b + c - a) * (c + a - b) * (a + b - c)) / 4.0;
}

// Normal(ib), MC3D.hpp:386-405
void normal_b3(const Geo &G, int64_t ib, double *n) {
  int64_t i0 = G.bh(ib, 0), i1 = G.bh(ib, 1), i2 = G.bh(ib, 2);
  double x1 = G.x(i1, 0) - G.x(i0, 0), y1 = G.x(i1, 1) - G.x(i0, 1), z1 = G.x(i1, 2) - G.x(i0, 2);
  double x2 = G.x(i2, 0) - G.x(i0, 0), y2 = G.x(i2, 1) - G.x(i0, 1), z2 = G.x(i2, 2) - G.x(i0, 2);
  double nx = y1 * z2 - z1 * y2, ny = z1 * x2 - x1 * z2, nz = x1 * y2 - y1 * x2;
  double norm = sqrt(nx * nx + ny * ny + nz * nz);
  n[0] = nx / norm; n[1] = ny / norm; n[2] = nz / norm;
}

// ElementArea(el), MC2D.hpp:303-310
double area2(const Geo &G, int64_t el) {
  double ax = G.x(G.h(el, 1), 0) - G.x(G.h(el, 0), 0);
  double ay = G.x(G.h(el, 1), 1) - G.x(G.h(el, 0), 1);
  double bx = G.x(G.h(el, 2), 0) - G.x(G.h(el, 0), 0);
  double by = G.x(G.h(el, 2), 1) - G.x(G.h(el, 0), 1);
  double c = ax * by - ay * bx;
  return 0.5 * (c >= 0.0 ? c : -c);
}

// ElementLength(ib), MC2D.hpp:313-318
double length2(const Geo &G, int64_t ib) {
  return sqrt(sq(G.x(G.bh(ib, 1), 0) - G.x(G.bh(ib, 0), 0)) + sq(G.x(G.bh(ib, 1), 1) - G.x(G.bh(ib, 0), 1)));
}

// Normal(ib), MC2D.hpp:347-355
void normal_b2(const Geo &G, int64_t ib, double *n) {
  double dx = G.x(G.bh(ib, 1), 0) - G.x(G.bh(ib, 0), 0);
  double dy = G.x(G.bh(ib, 1), 1) - G.x(G.bh(ib, 0), 1);
  double norm = sqrt(dx * dx + dy * dy);
  n[0] = dy / norm; n[1] = -dx / norm;
}

bool is_source(int dim, char t) {
  if (dim == 3)  // MC3D.hpp:957-959
    return t == 'l' || t == 'L' || t == 'i' || t == 'I' || t == 'c' || t == 'C' || t == 'p';
  return t == 'l' || t == 'i' || t == 'c' || t == 'g';  // MC2D.hpp:865-868
}

}  // namespace

const char *mcerror_string(int s) {
  switch (s) {  // cpp/Errors.hpp:24-58
    case VMC_NO_LIGHTSOURCE: return "No lightsource";
    case VMC_SIZE_MISMATCH_G: return "Scattering anisotropy array is not equal in size to the number of elements";
    case VMC_SIZE_MISMATCH_MUA: return "Absorption array is not equal in size to the number of elements";
    case VMC_SIZE_MISMATCH_MUS: return "Undefined error";  // the reference has no text for it (:25-56)
    case VMC_SIZE_MISMATCH_N: return "Refractive index array is not equal in size to the number of elements";
    case VMC_SIZE_MISMATCH_BCN:
      return "External refractive index array is not equal in size to the number of boundary elements";
    case VMC_MISSING_BCN: return "No external refractive index array given";
    case VMC_SIZE_MISMATCH_BCTYPE:
      return "The boundary condition array is not equal in size to the number of boundary elements";
    case VMC_SIZE_MISMATCH_LIGHT_DIRECTION:
      return "The light direction array is not equal in size to the number of boundary elements";
    case VMC_SIZE_MISMATCH_LIGHT_DIRECTION_TYPE:
      return "The light direction type array is not equal in size to the number of boundary elements";
    case VMC_INCONSISTENT_H: return "H matrix contain indices that are not in the coordinate matrix";
    case VMC_INCONSISTENT_BH: return "BH matrix contain indices that are not in the coordinate matrix";
    case VMC_INCONSISTENT_MESH: return "Ill defined mesh - cannot find nodes. Check Mesh.";
    case VMC_INCONSISTENT_MESH_DUPLICATE_NEIGHBORS:
      return "Ill defined mesh - some boundary elements are trapped between two elements. A boundary element must "
             "belong to a single element. Check Mesh.";
    case VMC_NO_GAUSSIAN_SIGMA: return "A gaussian light source exists but no sigma parameter was provided";
    case VMC_MISSING_BOUNDARY: return "Ill defined mesh - a complete boundary cannot be constructed. Check Mesh.";
    default: return nullptr;
  }
}

// ErrorChecks, MC3D.hpp:460-571 / MC2D.hpp:390-513
int check_input(const vmc_input *in) {
  if (!in || (in->dim != 2 && in->dim != 3)) return VMC_ERR_INVALID_ARGUMENT;
  if (in->Ne < 0 || in->Nb < 0 || in->Nr < 0) return VMC_ERR_INVALID_ARGUMENT;
  if (in->n_g != in->Ne) return E_SIZE_MISMATCH_G;
  if (in->n_mua != in->Ne) return E_SIZE_MISMATCH_MUA;
  if (in->n_mus != in->Ne) return E_SIZE_MISMATCH_MUS;
  if (in->n_n != in->Ne) return E_SIZE_MISMATCH_N;
  if (in->n_BCn == 0) return E_MISSING_BCN;
  if (in->n_BCn != in->Nb) return E_SIZE_MISMATCH_BCN;
  if (in->n_BCType != in->Nb) return E_SIZE_MISMATCH_BCTYPE;
  bool has_ls = false, has_g = false;
  for (int64_t i = 0; i < in->n_BCType; i++) {
    if (in->BCType[i] != 'a') has_ls = true;
    if (in->BCType[i] == 'g') has_g = true;
  }
  if (!has_ls) return E_NO_LIGHTSOURCE;
  if (in->dim == 2 && has_g && in->n_GaussianSigma != in->Nb) return E_NO_GAUSSIAN_SIGMA;
  if (in->n_BCLNormal && in->n_BCLNormal != in->Nb) return E_SIZE_MISMATCH_LIGHT_DIRECTION;
  if (in->n_BCLightDirectionType && in->n_BCLightDirectionType != in->Nb) return E_SIZE_MISMATCH_LIGHT_DIRECTION_TYPE;
  if ((in->Ne && !in->H) || (in->Nb && !in->BH) || (in->Nr && !in->r)) return VMC_ERR_INVALID_ARGUMENT;
  const int64_t nh = in->Ne * (in->dim + 1), nb = in->Nb * in->dim;
  for (int64_t i = 0; i < nh; i++)
    if (in->H[i] < 0 || in->H[i] >= in->Nr) return E_INCONSISTENT_H;
  for (int64_t i = 0; i < nb; i++)
    if (in->BH[i] < 0 || in->BH[i] >= in->Nr) return E_INCONSISTENT_BH;
  return VMC_OK;
}

// BuildNeighbourhoods, MC3D.hpp:835-871 + search_neighbor :740-832 (3D) and
// MC2D.hpp:724-773 + :645-721 (2D).  The candidates of a face are the elements and
// boundary elements that contain all of its vertices; they all appear in the incidence
// list of any one face vertex, so only the shortest such list is scanned (the reference
// scans the lists of every vertex of the element).  Elements are independent, so the
// loop runs in parallel; the error reported is the one of the lowest element, as in the
// reference's sequential loop.
int build_neighbours(int dim, int64_t Ne, int64_t Nb, int64_t Nr, const int64_t *H, const int64_t *BH, int64_t *HN) {
  const int NF = dim + 1;
  std::vector<int64_t> off((size_t)Nr + 1, 0);
  for (int64_t i = 0; i < Ne; i++)
    for (int c = 0; c < NF; c++) off[(size_t)H[i + Ne * c] + 1]++;
  for (int64_t i = 0; i < Nb; i++)
    for (int c = 0; c < dim; c++) off[(size_t)BH[i + Nb * c] + 1]++;
  for (int64_t v = 0; v < Nr; v++) off[(size_t)v + 1] += off[(size_t)v];
  std::vector<int64_t> fill(off.begin(), off.end() - 1), lst((size_t)off[(size_t)Nr]);
  for (int64_t i = 0; i < Ne; i++)
    for (int c = 0; c < NF; c++) lst[(size_t)fill[(size_t)H[i + Ne * c]]++] = i;
  for (int64_t i = 0; i < Nb; i++)
    for (int c = 0; c < dim; c++) lst[(size_t)fill[(size_t)BH[i + Nb * c]]++] = -1 - i;

  const int dup_err = dim == 3 ? E_INCONSISTENT_MESH_DUPLICATE_NEIGHBORS : E_INCONSISTENT_MESH;
  int64_t worst_el = std::numeric_limits<int64_t>::max();
  int worst_code = 0;
#pragma omp parallel
  {
    int64_t my_el = std::numeric_limits<int64_t>::max();
    int my_code = 0;
#pragma omp for schedule(static)
    for (int64_t el = 0; el < Ne; el++) {
      if (el > my_el) continue;
      int code = 0;
      for (int f = 0; f < NF && !code; f++) {
        int64_t fv[3];
        const int nv = dim;  // vertices per face
        for (int k = 0; k < nv; k++) fv[k] = H[el + Ne * (dim == 3 ? kFace3[f][k] : kEdge2[f][k])];
        int64_t best = fv[0];
        for (int k = 1; k < nv; k++)
          if (off[(size_t)fv[k] + 1] - off[(size_t)fv[k]] < off[(size_t)best + 1] - off[(size_t)best]) best = fv[k];
        int64_t found = std::numeric_limits<int64_t>::max();
        for (int64_t q = off[(size_t)best]; q < off[(size_t)best + 1]; q++) {
          const int64_t cand = lst[(size_t)q];
          if (cand == el) continue;
          bool all = true;
          for (int k = 0; k < nv && all; k++) {
            bool hit = false;
            if (cand >= 0) {
              for (int b = 0; b < NF; b++) hit |= (H[cand + Ne * b] == fv[k]);
            } else {
              const int64_t ib = -(cand + 1);
              for (int b = 0; b < dim; b++) hit |= (BH[ib + Nb * b] == fv[k]);
            }
            all = hit;
          }
          if (!all) continue;
          if (found != std::numeric_limits<int64_t>::max() && found != cand) { code = dup_err; break; }
          found = cand;
        }
        HN[el + Ne * f] = found;
      }
      if (!code && dim == 2)  // MC2D.hpp:768-771
        for (int f = 0; f < 3; f++)
          if (HN[el + Ne * f] == std::numeric_limits<int64_t>::max()) code = E_MISSING_BOUNDARY;
      if (code && el < my_el) { my_el = el; my_code = code; }
    }
#pragma omp critical
    {
      if (my_el < worst_el) { worst_el = my_el; worst_code = my_code; }
    }
  }
  return worst_code;
}

int build_mesh(const vmc_input *in, int precision_mask, HostMesh &m) {
  const int D = in->dim, NF = D + 1;
  m.dim = D; m.Ne = in->Ne; m.Nb = in->Nb; m.Nr = in->Nr;
  if (m.Ne >= (int64_t)kOpenFace || m.Nb >= (int64_t)kOpenFace) return VMC_ERR_SIZE_LIMIT;
  m.H.assign(in->H, in->H + m.Ne * NF);
  m.BH.assign(in->BH, in->BH + m.Nb * D);
  m.r.assign(in->r, in->r + m.Nr * D);
  m.HN.assign((size_t)(m.Ne * NF), 0);
  if (in->HN && in->n_HN == in->Ne) {  // MC3D.hpp:839: a neighbourhood of the right size is used as given
    m.HN.assign(in->HN, in->HN + m.Ne * NF);
  } else {
    int s = build_neighbours(D, m.Ne, m.Nb, m.Nr, m.H.data(), m.BH.data(), m.HN.data());
    if (s) return s;
  }
  Geo G{m.H.data(), m.BH.data(), m.r.data(), m.Ne, m.Nb, m.Nr};
  m.volume.resize((size_t)m.Ne);
  m.area.resize((size_t)m.Nb);
  m.bnorm.assign((size_t)m.Nb * 4, 0.0);
#pragma omp parallel for schedule(static)
  for (int64_t i = 0; i < m.Ne; i++) m.volume[(size_t)i] = D == 3 ? volume3(G, i) : area2(G, i);
  for (int64_t i = 0; i < m.Nb; i++) {
    m.area[(size_t)i] = D == 3 ? area3(G, i) : length2(G, i);
    if (D == 3) normal_b3(G, i, &m.bnorm[(size_t)i * 4]);
    else normal_b2(G, i, &m.bnorm[(size_t)i * 4]);
  }
  auto nbr32 = [&](int64_t el, int f) -> int32_t {
    int64_t h = m.HN[(size_t)(el + m.Ne * f)];
    if (h >= m.Ne || h < -m.Nb) return kOpenFace;  // INT64_MAX open face, or an invalid given HN
    return (int32_t)h;
  };
  if (D == 3) {
    if (precision_mask & 1) {
      m.tet64.resize((size_t)m.Ne);
#pragma omp parallel for schedule(static)
      for (int64_t el = 0; el < m.Ne; el++) {
        Tet64 &T = m.tet64[(size_t)el];
        for (int v = 0; v < 4; v++)
          for (int c = 0; c < 3; c++) T.v[v][c] = G.x(G.h(el, v), c);
        for (int f = 0; f < 4; f++) T.nbr[f] = nbr32(el, f);
      }
    }
    if (precision_mask & 2) {
      m.tet32.resize((size_t)m.Ne);
#pragma omp parallel for schedule(static)
      for (int64_t el = 0; el < m.Ne; el++) {
        Tet32 &T = m.tet32[(size_t)el];
        for (int f = 0; f < 4; f++) {
          // plane from the face's vertices in ascending id order, so the two elements
          // sharing a face store exactly opposite planes (no gaps, no overlaps)
          int64_t ids[3] = {G.h(el, kFace3[f][0]), G.h(el, kFace3[f][1]), G.h(el, kFace3[f][2])};
          std::sort(ids, ids + 3);
          double P[3][3];
          for (int k = 0; k < 3; k++)
            for (int c = 0; c < 3; c++) P[k][c] = G.x(ids[k], c);
          double a[3] = {P[1][0] - P[0][0], P[1][1] - P[0][1], P[1][2] - P[0][2]};
          double b[3] = {P[2][0] - P[0][0], P[2][1] - P[0][1], P[2][2] - P[0][2]};
          double n[3] = {a[1] * b[2] - a[2] * b[1], a[2] * b[0] - a[0] * b[2], a[0] * b[1] - a[1] * b[0]};
          double nn = sqrt(n[0] * n[0] + n[1] * n[1] + n[2] * n[2]);
          for (int c = 0; c < 3; c++) n[c] /= nn;
          double d = n[0] * P[0][0] + n[1] * P[0][1] + n[2] * P[0][2];
          int64_t o = G.h(el, kOpp3[f]);
          double side = n[0] * (G.x(o, 0) - P[0][0]) + n[1] * (G.x(o, 1) - P[0][1]) + n[2] * (G.x(o, 2) - P[0][2]);
          float s = side > 0.0 ? -1.0f : 1.0f;  // outward: away from the opposite vertex
          T.pl[f][0] = s * (float)n[0];
          T.pl[f][1] = s * (float)n[1];
          T.pl[f][2] = s * (float)n[2];
          T.pl[f][3] = s * (float)d;
          T.nbr[f] = nbr32(el, f);
        }
      }
    }
  } else {
    if (precision_mask & 1) {
      m.tri64.resize((size_t)m.Ne);
      for (int64_t el = 0; el < m.Ne; el++) {
        Tri64 &T = m.tri64[(size_t)el];
        for (int v = 0; v < 3; v++)
          for (int c = 0; c < 2; c++) T.v[v][c] = G.x(G.h(el, v), c);
        for (int f = 0; f < 3; f++) T.nbr[f] = nbr32(el, f);
        T.nbr[3] = kOpenFace;
      }
    }
    if (precision_mask & 2) {
      m.tri32.resize((size_t)m.Ne);
      for (int64_t el = 0; el < m.Ne; el++) {
        Tri32 &T = m.tri32[(size_t)el];
        for (int f = 0; f < 3; f++) {
          int64_t ids[2] = {G.h(el, kEdge2[f][0]), G.h(el, kEdge2[f][1])};
          if (ids[0] > ids[1]) std::swap(ids[0], ids[1]);
          double tx = G.x(ids[1], 0) - G.x(ids[0], 0), ty = G.x(ids[1], 1) - G.x(ids[0], 1);
          double nn = sqrt(tx * tx + ty * ty);
          double n0 = ty / nn, n1 = -tx / nn;
          double d = n0 * G.x(ids[0], 0) + n1 * G.x(ids[0], 1);
          int64_t o = G.h(el, kOpp2[f]);
          double side = n0 * (G.x(o, 0) - G.x(ids[0], 0)) + n1 * (G.x(o, 1) - G.x(ids[0], 1));
          float s = side > 0.0 ? -1.0f : 1.0f;
          T.ln[f][0] = s * (float)n0;
          T.ln[f][1] = s * (float)n1;
          T.ln[f][2] = s * (float)d;
          T.ln[f][3] = 0.0f;
          T.nbr[f] = nbr32(el, f);
        }
        T.nbr[3] = kOpenFace;
      }
    }
  }
  return VMC_OK;
}

// Init's light sources and BCLNormal handling (MC3D.hpp:611-735, :941-1002;
// MC2D.hpp:553-640, :851-911) and the per-face launch quantities of CreatePhoton.
int build_job(const vmc_input *in, const HostMesh &m, HostJob &j) {
  const int D = m.dim, NF = D + 1;
  const int64_t Ne = m.Ne, Nb = m.Nb;
  if (in->dim != D || in->Ne != Ne || in->Nb != Nb) return VMC_ERR_INVALID_ARGUMENT;
  Geo G{m.H.data(), m.BH.data(), m.r.data(), m.Ne, m.Nb, m.Nr};
  j.dim = D; j.Ne = Ne; j.Nb = Nb;
  j.f = in->f;
  j.omega = 2.0 * kPi * in->f;
  j.k_scale = j.omega / kC0;
  double ph0 = in->phase0;
  if (ph0 < 0) ph0 += 2 * kPi * ceil(-ph0 / (2 * kPi));  // MC3D.cpp:141-143, MC3Dmex.cpp:158-160
  j.phase0 = ph0;
  j.Nphoton = in->Nphoton;
  // optics rows; a job whose elements all share one row keeps a single row
  bool hom = Ne > 0;
  for (int64_t i = 1; i < Ne && hom; i++)
    hom = in->mua[i] == in->mua[0] && in->mus[i] == in->mus[0] && in->g[i] == in->g[0] && in->n[i] == in->n[0];
  j.homogeneous = hom;
  const int64_t rows = hom ? 1 : Ne;
  j.optics.resize((size_t)rows * 4);
  for (int64_t i = 0; i < rows; i++) {
    j.optics[(size_t)i * 4 + 0] = in->mua[i];
    j.optics[(size_t)i * 4 + 1] = in->mus[i];
    j.optics[(size_t)i * 4 + 2] = in->g[i];
    j.optics[(size_t)i * 4 + 3] = in->n[i];
  }
  j.mua.assign(in->mua, in->mua + Ne);
  j.k.resize((size_t)Ne);
  for (int64_t i = 0; i < Ne; i++) j.k[(size_t)i] = j.omega / kC0 * in->n[i];  // MC3D.hpp:660-662
  j.bctype.assign(reinterpret_cast<const uint8_t *>(in->BCType), reinterpret_cast<const uint8_t *>(in->BCType) + Nb);
  j.bcn.assign(in->BCn, in->BCn + Nb);
  // BCLightDirectionType defaults to 'n' (MC3D.hpp:646-654), BCLNormal is normalised
  // (3D: only rows of type 'n', MC3D.hpp:671-688; 2D: every row, MC2D.hpp:612-622) and
  // relative rows are mapped to absolute ones (MC3D.hpp:693-735, MC2D.hpp:625-640)
  std::vector<char> dtype((size_t)Nb, 'n');
  if (in->n_BCLightDirectionType) dtype.assign(in->BCLightDirectionType, in->BCLightDirectionType + Nb);
  std::vector<double> L;
  if (in->n_BCLNormal) L.assign(in->BCLNormal, in->BCLNormal + Nb * D);
  if (in->n_BCLNormal) {
    for (int64_t i = 0; i < Nb; i++) {
      if (D == 3) {
        double norm = sqrt(sq(L[i]) + sq(L[i + Nb]) + sq(L[i + 2 * Nb]));
        if (dtype[(size_t)i] != 'n') continue;
        L[i] /= norm; L[i + Nb] /= norm; L[i + 2 * Nb] /= norm;
      } else {
        double norm = sqrt(sq(L[i]) + sq(L[i + Nb]));
        L[i] /= norm; L[i + Nb] /= norm;
      }
    }
    for (int64_t i = 0; i < Nb; i++) {
      if (dtype[(size_t)i] != 'r') continue;
      if (D == 3) {
        double n[3], e1[3], e2[3];
        normal_b3(G, i, n);
        for (int c = 0; c < 3; c++) {
          e1[c] = G.x(G.bh(i, 1), c) - G.x(G.bh(i, 0), c);
          e2[c] = G.x(G.bh(i, 2), c) - G.x(G.bh(i, 0), c);
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
      } else {
        double n[2], t[2];
        normal_b2(G, i, n);
        t[0] = G.x(G.bh(i, 1), 0) - G.x(G.bh(i, 0), 0);
        t[1] = G.x(G.bh(i, 1), 1) - G.x(G.bh(i, 0), 1);
        double norm = sqrt(t[0] * t[0] + t[1] * t[1]);
        t[0] /= norm; t[1] /= norm;
        double ox = L[i], oy = L[i + Nb];
        L[i] = ox * t[0] + oy * n[0];
        L[i + Nb] = ox * t[1] + oy * n[1];
      }
    }
  }
  // BuildLightSource: emitting faces in (element, face) order; CDF of area x intensity
  j.src.clear();
  std::vector<double> w;
  for (int64_t el = 0; el < Ne; el++) {
    for (int f = 0; f < NF; f++) {
      const int64_t h = m.HN[(size_t)(el + Ne * f)];
      if (h > -1) continue;
      const int64_t ib = -1 - h;
      const char bt = in->BCType[ib];
      if (!is_source(D, bt)) continue;
      SourceRec S;
      memset(&S, 0, sizeof(S));
      S.mother = (int32_t)el;
      S.ib = (int32_t)ib;
      S.type = bt;
      S.dirtype = dtype[(size_t)ib];
      S.curface = -1;
      for (int ff = 0; ff < NF; ff++)
        if (-1 - m.HN[(size_t)(el + Ne * ff)] == ib) { S.curface = ff; break; }
      if (D == 3) {
        for (int c = 0; c < 3; c++) {
          S.v0[c] = G.x(G.bh(ib, 0), c);
          S.v1[c] = G.x(G.bh(ib, 1), c);
          S.v2[c] = G.x(G.bh(ib, 2), c);
        }
        double n[3], t[3];
        normal_b3(G, ib, n);
        // inward orientation, CreatePhoton :1094-1107 (the sign does not depend on where
        // on the face the photon starts, so the face centroid stands in for it)
        for (int c = 0; c < 3; c++)
          t[c] = (G.x(G.h(el, 0), c) + G.x(G.h(el, 1), c) + G.x(G.h(el, 2), c) + G.x(G.h(el, 3), c)) / 4.0 -
                 (S.v0[c] + S.v1[c] + S.v2[c]) / 3.0;
        if (n[0] * t[0] + n[1] * t[1] + n[2] * t[2] < 0.0) { n[0] = -n[0]; n[1] = -n[1]; n[2] = -n[2]; }
        for (int c = 0; c < 3; c++) S.n[c] = n[c];
        if (in->n_BCLNormal)
          for (int c = 0; c < 3; c++) S.L[c] = L[ib + c * Nb];
        if (bt == 'c' || bt == 'C') {
          double e1[3], e2[3], norm, dpn, dp1;
          for (int c = 0; c < 3; c++) { e1[c] = S.v1[c] - S.v0[c]; e2[c] = S.v2[c] - S.v0[c]; }
          if (S.dirtype == 'n') {  // CreatePhoton :1148-1183
            norm = sqrt(e1[0] * e1[0] + e1[1] * e1[1] + e1[2] * e1[2]);
            for (int c = 0; c < 3; c++) e1[c] /= norm;
            dpn = n[0] * e2[0] + n[1] * e2[1] + n[2] * e2[2];
            dp1 = e1[0] * e2[0] + e1[1] * e2[1] + e1[2] * e2[2];
            for (int c = 0; c < 3; c++) e2[c] -= dpn * n[c] + dp1 * e1[c];
          } else {  // :1243-1278, frame around BCLNormal
            const double *Ln = S.L;
            dpn = Ln[0] * e1[0] + Ln[1] * e1[1] + Ln[2] * e1[2];
            for (int c = 0; c < 3; c++) e1[c] -= dpn * Ln[c];
            norm = sqrt(e1[0] * e1[0] + e1[1] * e1[1] + e1[2] * e1[2]);
            for (int c = 0; c < 3; c++) e1[c] /= norm;
            dpn = Ln[0] * e2[0] + Ln[1] * e2[1] + Ln[2] * e2[2];
            dp1 = e1[0] * e2[0] + e1[1] * e2[1] + e1[2] * e2[2];
            for (int c = 0; c < 3; c++) e2[c] -= dpn * Ln[c] + dp1 * e1[c];
          }
          norm = sqrt(e2[0] * e2[0] + e2[1] * e2[1] + e2[2] * e2[2]);
          for (int c = 0; c < 3; c++) e2[c] /= norm;
          for (int c = 0; c < 3; c++) { S.e1[c] = e1[c]; S.e2[c] = e2[c]; }
        }
        w.push_back(m.area[(size_t)ib]);
      } else {
        for (int c = 0; c < 2; c++) {
          S.v0[c] = G.x(G.bh(ib, 0), c);
          S.v1[c] = G.x(G.bh(ib, 1), c);
        }
        double n[2], t[2];
        normal_b2(G, ib, n);
        for (int c = 0; c < 2; c++)
          t[c] = (G.x(G.h(el, 0), c) + G.x(G.h(el, 1), c) + G.x(G.h(el, 2), c)) / 3.0 - (S.v0[c] + S.v1[c]) / 2.0;
        if (n[0] * t[0] + n[1] * t[1] < 0.0) { n[0] = -n[0]; n[1] = -n[1]; }
        S.n[0] = n[0]; S.n[1] = n[1];
        if (in->n_BCLNormal) { S.L[0] = L[ib]; S.L[1] = L[ib + Nb]; }
        S.phi0 = S.dirtype == 'n' ? atan2(n[1], n[0]) : atan2(S.L[1], S.L[0]);
        if (bt == 'g') {  // MC2D.hpp:1044
          S.sigma = in->GaussianSigma[ib];
          S.gauss_h = 0.5 - 0.5 * erf(kPi / S.sigma / 2.0 / sqrt(2.0));
        }
        w.push_back(m.area[(size_t)ib]);
      }
      j.src.push_back(S);
    }
  }
  const size_t ns = j.src.size();
  if (ns == 0 || ns >= (size_t)kOpenFace) return E_NO_LIGHTSOURCE;
  j.cdf.resize(ns);
  for (size_t i = 0; i < ns; i++) j.cdf[i] = w[i] * (in->n_BCIntensity ? in->BCIntensity[j.src[i].ib] : 1.0);
  for (size_t i = 1; i < ns; i++) j.cdf[i] += j.cdf[i - 1];
  const double tot = j.cdf[ns - 1];
  for (size_t i = 0; i < ns; i++) j.cdf[i] /= tot;
  if (!(j.cdf[ns - 1] == j.cdf[ns - 1])) return E_NO_LIGHTSOURCE;  // zero total weight
  j.src_f.resize(ns);
  j.cdf_f.resize(ns);
  for (size_t i = 0; i < ns; i++) {
    const SourceRec &S = j.src[i];
    SourceRecF &F = j.src_f[i];
    memset(&F, 0, sizeof(F));
    for (int c = 0; c < 3; c++) {
      F.v0[c] = (float)S.v0[c]; F.v1[c] = (float)S.v1[c]; F.v2[c] = (float)S.v2[c];
      F.n[c] = (float)S.n[c]; F.e1[c] = (float)S.e1[c]; F.e2[c] = (float)S.e2[c]; F.L[c] = (float)S.L[c];
    }
    F.phi0 = (float)S.phi0; F.sigma = (float)S.sigma; F.gauss_h = (float)S.gauss_h;
    F.cphi0 = (float)cos(S.phi0); F.sphi0 = (float)sin(S.phi0);
    F.mother = S.mother; F.curface = S.curface; F.ib = S.ib; F.type = S.type; F.dirtype = S.dirtype;
    j.cdf_f[i] = (float)j.cdf[i];
  }
  j.cdf_f[ns - 1] = 1.0f;
  return VMC_OK;
}

// MonteCarlo's normalisation, MC3D.hpp:1792-1818 / MC2D.hpp:1672-1703
void normalise(const HostMesh &m, const HostJob &j, int64_t nphoton, const double *ER, const double *EI,
               const double *EBR, const double *EBI, const double *DEBR, const double *DEBI, vmc_output *out,
               bool apply) {
  const int64_t Ne = m.Ne, Nb = m.Nb;
  const double Nd = (double)nphoton;
  const bool cw = j.omega <= 0.0;
#pragma omp parallel for schedule(static) if (Ne > 100000)
  for (int64_t i = 0; i < Ne; i++) {
    double a = ER[i], b = EI[i], er, ei;
    if (!apply) { er = a; ei = b; }
    else if (cw) {
      const double mu = j.mua[(size_t)i], V = m.volume[(size_t)i];
      er = mu > 0.0 ? a / (mu * V * Nd) : a / (V * Nd);
      ei = b;
    } else {
      const double k = j.k[(size_t)i], mu = j.mua[(size_t)i], V = m.volume[(size_t)i];
      er = (b * k + a * mu) / (sq(k) + sq(mu)) / Nd / V;
      ei = -(a * k - b * mu) / (sq(k) + sq(mu)) / Nd / V;
    }
    if (out->ER) out->ER[i] = er;
    if (out->EI) out->EI[i] = ei;
  }
  for (int64_t i = 0; i < Nb; i++) {
    const double A = m.area[(size_t)i];
    double ebr = EBR[i], ebi = EBI[i], dbr = DEBR[i], dbi = DEBI[i];
    if (apply) {
      ebr /= Nd * A;
      if (!cw) ebi /= Nd * A;
      if (m.dim == 2) {
        dbr /= Nd * A;
        if (!cw) dbi /= Nd * A;
      }
    }
    if (out->EBR) out->EBR[i] = ebr;
    if (out->EBI) out->EBI[i] = ebi;
    if (out->DEBR) out->DEBR[i] = dbr;
    if (out->DEBI) out->DEBI[i] = dbi;
  }
}

}  // namespace vmc
