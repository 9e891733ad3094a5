// host_setup.hpp -- host half of the drop-in: ErrorChecks, Init and the normalisation of
// MC3D/MC2D (cpp/3d/MC3D.hpp:460-738, :1792-1818; cpp/2d/MC2D.hpp:390-643, :1672-1703),
// producing the device records of vmc_types.hpp.  Compiled with -ffp-contract=off so the
// per-face launch quantities are the reference's doubles bit for bit.
#pragma once
#include <stdint.h>

#include <string>
#include <vector>

#include "../../include/valomc_gb300.h"
#include "vmc_types.hpp"

namespace vmc {

// Geometry shared by every job on a mesh.
struct HostMesh {
  int dim = 3;
  int64_t Ne = 0, Nb = 0, Nr = 0;
  std::vector<int64_t> H, BH;   // column-major copies
  std::vector<double> r;
  std::vector<int64_t> HN;      // column-major [Ne x (dim+1)]
  std::vector<double> volume;   // ElementVolume / ElementArea(el)
  std::vector<double> area;     // ElementArea(ib) / ElementLength(ib)
  std::vector<double> bnorm;    // [Nb x 4] Normal(ib)
  // device records
  std::vector<Tet64> tet64;
  std::vector<Tet32> tet32;
  std::vector<Tri64> tri64;
  std::vector<Tri32> tri32;
};

// One problem on a mesh: optics, boundary conditions, sources, scalars.
struct HostJob {
  int dim = 3;
  int64_t Ne = 0, Nb = 0;
  bool homogeneous = false;
  std::vector<double> optics;   // rows of (mua, mus, g, n); one row when homogeneous
  std::vector<double> mua;      // for the normalisation
  std::vector<uint8_t> bctype;
  std::vector<double> bcn;
  std::vector<SourceRec> src;
  std::vector<double> cdf;
  std::vector<SourceRecF> src_f;  // FP32 copies for the tracking form
  std::vector<float> cdf_f;
  double f = 0, omega = 0, k_scale = 0, phase0 = 0;
  int64_t Nphoton = 0;
  uint64_t seed = 0;
  std::vector<double> k;        // omega / c0 * n per element (FD normalisation)
};

// ErrorChecks (same checks, same order, same codes).  Returns VMC_OK or 1 + mcerror.
int check_input(const vmc_input *in);

// BuildNeighbourhoods: HN [Ne x (dim+1)] column-major with the reference's semantics
// (boundary -1 - ib, 3D open faces INT64_MAX, 2D open edges -> MISSING_BOUNDARY,
// two different candidates for one face -> INCONSISTENT_MESH[_DUPLICATE_NEIGHBORS]).
int build_neighbours(int dim, int64_t Ne, int64_t Nb, int64_t Nr, const int64_t *H, const int64_t *BH, int64_t *HN);

// Mesh from the geometry arrays of an input (HN built unless given).  precision_mask:
// bit 0 builds the FP64 records, bit 1 the FP32 records.
int build_mesh(const vmc_input *in, int precision_mask, HostMesh &m);

// Job from the problem arrays of an input on mesh m (Init's light sources, BCLNormal
// processing and wave numbers).
int build_job(const vmc_input *in, const HostMesh &m, HostJob &j);

// MonteCarlo's normalisation of raw accumulators into the caller's output arrays.
void normalise(const HostMesh &m, const HostJob &j, int64_t nphoton, const double *ER, const double *EI,
               const double *EBR, const double *EBI, const double *DEBR, const double *DEBI, vmc_output *out,
               bool apply);

const char *mcerror_string(int status);

}  // namespace vmc
