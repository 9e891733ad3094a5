// mc_mex.hpp -- MATLAB gateways MC3Dmex / MC2Dmex on the GB300 engine.
//
// Same call contract as the reference gateways (cpp/3d/MC3Dmex.cpp:98-253,
// cpp/2d/MC2Dmex.cpp:98-252), as marshalled by ValoMC.m:128-157,338:
//   [vsol, bsol, ebsol, simulationtime, rnseed, [HN]] = MC3Dmex(H, HN, BH, r, BCType,
//       BCIntensity, BCLightDirectionType, BCLNormal, BCn, mua, mus, g, n, f, phase0,
//       Nphoton, disablepbar, rnseed)
//   MC2Dmex takes GaussianSigma after Nphoton (19 inputs).
// Inputs are borrowed zero-copy (the ABI takes the column-major arrays as they are);
// outputs are created complex [N x 1] arrays, the run time, the seed used and optionally
// the neighbourhood.  Progress and cancellation keep the reference's waitbar protocol
// (abort_photonMC in the base workspace, cpp/3d/MC3Dmex.cpp:47-90).
// Optional environment: VALOMC_PRECISION=fp64 selects the plain FP64 form.
#pragma once
#include <math.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <time.h>

#include <string>
#include <vector>

#include "mex.h"
#include "valomc_gb300.h"

namespace vmcmex {

inline void type_error() { mexErrMsgTxt("mxArray type error! Incorrect type received!\n"); }

// zero-copy view of a 2-D numeric array of the expected class (Convert_mxArray,
// cpp/3d/ArrayMEX.hpp:11-42)
template <class T>
const T *view(const mxArray *a, mxClassID want, int64_t *rows, int64_t *cols = nullptr) {
  if (mxGetClassID(a) != want) type_error();
  if (mxGetNumberOfDimensions(a) != 2) mexErrMsgTxt("Only 2D-mxArrays are supported!\n");
  *rows = (int64_t)mxGetM(a);
  if (cols) *cols = (int64_t)mxGetN(a);
  return reinterpret_cast<const T *>(mxGetData(a));
}

// BCType / BCLightDirectionType arrive as int8 (ValoMC.m:412-442); MATLAB char arrays
// (16-bit) are narrowed
inline const char *chars(const mxArray *a, int64_t *rows, std::vector<char> &tmp) {
  if (mxGetNumberOfDimensions(a) != 2) mexErrMsgTxt("Only 2D-mxArrays are supported!\n");
  *rows = (int64_t)mxGetM(a);
  mxClassID id = mxGetClassID(a);
  if (id == mxINT8_CLASS || id == mxUINT8_CLASS) return reinterpret_cast<const char *>(mxGetData(a));
  if (id == mxCHAR_CLASS) {
    const uint16_t *c = reinterpret_cast<const uint16_t *>(mxGetData(a));
    size_t n = (size_t)mxGetM(a) * (size_t)mxGetN(a);
    tmp.resize(n);
    for (size_t i = 0; i < n; i++) tmp[i] = (char)c[i];
    return tmp.data();
  }
  type_error();
  return nullptr;
}

static time_t g_start;
static bool g_use_bar = false;

// Progress_with_bar (cpp/3d/MC3Dmex.cpp:47-90): abort when abort_photonMC is true
static int progress_bar(double perc, void *) {
  if (!g_use_bar) {
    mexPrintf("  %f %%\r", perc);
    return 1;
  }
  mxArray *res = mexGetVariable("base", "abort_photonMC");
  if (res) {
    bool stop = mxIsLogicalScalarTrue(res);
    mxDestroyArray(res);
    if (stop) return 0;
  }
  time_t now = time(NULL);
  double dt = difftime(now, g_start);
  char cmd[512];
  if (dt > 0 && perc > 0) {
    double rem = (100.0 - perc) / (perc / dt);
    double h = floor(rem / 3600), m = floor((rem - h * 3600) / 60), s = rem - h * 3600 - m * 60;
    snprintf(cmd, sizeof cmd, "waitbar(%f,mcwaitbar,'%i hours %i minutes and %i seconds left');\n", perc / 100.0,
             (int)h, (int)m, (int)ceil(s));
  } else {
    snprintf(cmd, sizeof cmd, "waitbar(0, mcwaitbar,'Estimating the time left');\n");
  }
  mexEvalString(cmd);
  return 1;
}

inline void gateway(int nlhs, mxArray **plhs, int nrhs, const mxArray **prhs, int dim) {
  mexPrintf("                 ValoMC-%dD\n", dim);
  mexPrintf("  GB300 sm_103a photon engine\n");
  const int want = dim == 3 ? 18 : 19;
  if (nrhs != want || (nlhs != 5 && nlhs != 6)) {
    mexPrintf("nrhs %i nlhs %i", nrhs, nlhs);
    if (dim == 3)
      mexErrMsgTxt("Syntax:\n [vsol, bsol, ebsol, simulationtime, rnseed, [HN]] = MC3Dmex(H, HN, BH, r, BCType, "
                   "BCIntensity, BCLightDirectionType, BCLNormal, BCn, mua, mus, g, n, f, phase0, Nphoton, "
                   "disablepbar, rnseed)\n");
    else
      mexErrMsgTxt("Syntax:\n [vsol, bsol, ebsol, simulationtime, seed, [HN]] = MC2Dmex(H, HN, BH, r, BCType, "
                   "BCIntensity, BCLightDirectionType, BCLNormal, BCn, mua, mus, g, n, f, phase0, Nphoton, "
                   "GaussianSigma, disablepbar, rndseed)\n");
  }
  mexPrintf("Initializing MC%dD...\n", dim);
  vmc_input in;
  memset(&in, 0, sizeof(in));
  in.dim = dim;
  int64_t rows, cols, tmp;
  std::vector<char> bct_tmp, dt_tmp;
  in.H = view<int64_t>(prhs[0], mxINT64_CLASS, &in.Ne);
  in.HN = view<int64_t>(prhs[1], mxINT64_CLASS, &in.n_HN);
  in.BH = view<int64_t>(prhs[2], mxINT64_CLASS, &in.Nb);
  in.r = view<double>(prhs[3], mxDOUBLE_CLASS, &in.Nr);
  in.BCType = chars(prhs[4], &in.n_BCType, bct_tmp);
  in.BCIntensity = view<double>(prhs[5], mxDOUBLE_CLASS, &in.n_BCIntensity);
  in.BCLightDirectionType = chars(prhs[6], &in.n_BCLightDirectionType, dt_tmp);
  in.BCLNormal = view<double>(prhs[7], mxDOUBLE_CLASS, &in.n_BCLNormal);
  in.BCn = view<double>(prhs[8], mxDOUBLE_CLASS, &in.n_BCn);
  in.mua = view<double>(prhs[9], mxDOUBLE_CLASS, &in.n_mua);
  in.mus = view<double>(prhs[10], mxDOUBLE_CLASS, &in.n_mus);
  in.g = view<double>(prhs[11], mxDOUBLE_CLASS, &in.n_g);
  in.n = view<double>(prhs[12], mxDOUBLE_CLASS, &in.n_n);
  const double *f = view<double>(prhs[13], mxDOUBLE_CLASS, &tmp);
  const double *phase0 = view<double>(prhs[14], mxDOUBLE_CLASS, &tmp);
  const int64_t *nphoton = view<int64_t>(prhs[15], mxINT64_CLASS, &tmp);
  int k = 16;
  if (dim == 2) in.GaussianSigma = view<double>(prhs[k++], mxDOUBLE_CLASS, &in.n_GaussianSigma);
  const int64_t *disable_pbar = view<int64_t>(prhs[k++], mxINT64_CLASS, &tmp);
  const uint64_t *rndseed = view<uint64_t>(prhs[k++], mxUINT64_CLASS, &rows, &cols);
  (void)cols;
  in.f = f[0];
  in.phase0 = phase0[0];  // negative values are wrapped inside vmc_run
  in.Nphoton = nphoton[0];
  in.seed_given = rndseed[1] ? 1 : 0;
  in.seed = rndseed[0];
  if (in.n_HN == 0) in.HN = nullptr;

  const int64_t NF = dim + 1;
  std::vector<double> ER((size_t)in.Ne), EI((size_t)in.Ne), EBR((size_t)in.Nb), EBI((size_t)in.Nb),
      DEBR((size_t)in.Nb), DEBI((size_t)in.Nb);
  std::vector<int64_t> HN(nlhs == 6 ? (size_t)(in.Ne * NF) : 0);
  vmc_output out;
  memset(&out, 0, sizeof(out));
  out.ER = ER.data(); out.EI = EI.data(); out.EBR = EBR.data(); out.EBI = EBI.data();
  out.DEBR = DEBR.data(); out.DEBI = DEBI.data();
  if (nlhs == 6) out.HN = HN.data();
  vmc_options opt;
  vmc_default_options(&opt);
  const char *prec = getenv("VALOMC_PRECISION");
  if (prec && !strcmp(prec, "fp64")) opt.precision = VMC_FP64;
  opt.progress = progress_bar;
  g_use_bar = disable_pbar[0] == 0;
  g_start = time(NULL);
  mexPrintf("Computing... \n");
  if (g_use_bar) {
    mexEvalString("assignin('base','abort_photonMC', false);");
    mexEvalString("mcwaitbar = waitbar(0,'Please wait..', 'name', 'Running simulation', "
                  "'CreateCancelBtn','abort_photonMC=true;');");
  }
  vmc_stats st;
  int s = vmc_run(&in, &opt, &out, &st);
  if (g_use_bar) mexEvalString("delete(mcwaitbar);");
  if (s >= VMC_NO_LIGHTSOURCE && s <= VMC_MISSING_BOUNDARY) {
    std::string msg = std::string("Error in initializing MC") + (dim == 3 ? "3D: " : "2D: ") +
                      vmc_status_string(s) + "\n";
    mexErrMsgTxt(msg.c_str());
    return;
  }
  if (s == VMC_ERR_CANCELLED)  // finalchecks, cpp/3d/MC3Dmex.cpp:33-40
    mexPrintf("WARNING: RUN WAS ABORTED OR PARALLEL COMPUTING ENVIRONMENT IS NOT WORKING CORRECTLY. \n");
  else if (s != VMC_OK) {
    std::string msg = std::string("GPU photon engine failed: ") + vmc_status_string(s) + " " + vmc_last_error() + "\n";
    mexErrMsgTxt(msg.c_str());
    return;
  }
  mexPrintf("...done\n");
  if (st.loss) mexPrintf(" %lld photons lost during computation!\n", (long long)st.loss);
  // outputs (cpp/3d/MC3Dmex.cpp:214-246)
  auto complex_col = [](mxArray **dst, const std::vector<double> &re, const std::vector<double> &im) {
    mwSize dims[2] = {(mwSize)re.size(), 1};
    *dst = mxCreateNumericArray(2, dims, mxDOUBLE_CLASS, mxCOMPLEX);
    if (!re.empty()) {
      memcpy(mxGetData(*dst), re.data(), re.size() * sizeof(double));
      memcpy(mxGetImagData(*dst), im.data(), im.size() * sizeof(double));
    }
  };
  complex_col(&plhs[0], ER, EI);
  complex_col(&plhs[1], EBR, EBI);
  complex_col(&plhs[2], DEBR, DEBI);
  plhs[3] = mxCreateDoubleMatrix(1, 1, mxREAL);
  *mxGetPr(plhs[3]) = difftime(time(NULL), g_start);
  plhs[4] = mxCreateNumericMatrix(1, 1, mxUINT64_CLASS, mxREAL);
  *reinterpret_cast<uint64_t *>(mxGetData(plhs[4])) = st.seed_used;
  if (nlhs == 6) {
    mwSize dims[2] = {(mwSize)in.Ne, (mwSize)NF};
    plhs[5] = mxCreateNumericArray(2, dims, mxINT64_CLASS, mxREAL);
    if (!HN.empty()) memcpy(mxGetData(plhs[5]), HN.data(), HN.size() * sizeof(int64_t));
  }
  mexPrintf("Done\n");
}

}  // namespace vmcmex
