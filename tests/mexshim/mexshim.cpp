// mexshim.cpp -- test stand-in for the MATLAB MEX runtime (see mex.h).  mexErrMsgTxt
// unwinds with an exception that shim_invoke turns into an error return; mexEvalString
// records the commands; abort_photonMC in the "base" workspace is settable from the test.
#include <stdarg.h>
#include <stdio.h>
#include <string.h>

#include <stdexcept>
#include <string>
#include <vector>

#include "mex.h"

struct mxArray_tag {
  mxClassID id = mxDOUBLE_CLASS;
  size_t m = 0, n = 0, elem = 8;
  std::vector<char> re, im;
  bool complex = false;
};

static size_t elem_size(mxClassID id) {
  switch (id) {
    case mxDOUBLE_CLASS: case mxINT64_CLASS: case mxUINT64_CLASS: return 8;
    case mxSINGLE_CLASS: case mxINT32_CLASS: case mxUINT32_CLASS: return 4;
    case mxINT16_CLASS: case mxUINT16_CLASS: case mxCHAR_CLASS: return 2;
    default: return 1;
  }
}

static std::string g_err, g_log;
static std::vector<std::string> g_eval;
static int g_abort = 0;
static int g_abort_after = -1;  // set abort_photonMC true after this many progress polls

extern "C" {
mxClassID mxGetClassID(const mxArray *a) { return a->id; }
mwSize mxGetNumberOfDimensions(const mxArray *) { return 2; }
void *mxGetData(const mxArray *a) { return a->re.empty() ? nullptr : (void *)a->re.data(); }
void *mxGetImagData(const mxArray *a) { return a->im.empty() ? nullptr : (void *)a->im.data(); }
double *mxGetPr(const mxArray *a) { return (double *)mxGetData(a); }
size_t mxGetM(const mxArray *a) { return a->m; }
size_t mxGetN(const mxArray *a) { return a->n; }
mxArray *mxCreateNumericArray(mwSize ndim, const mwSize *dims, mxClassID id, mxComplexity c) {
  mxArray *a = new mxArray_tag;
  a->id = id;
  a->m = dims[0];
  a->n = ndim > 1 ? dims[1] : 1;
  a->elem = elem_size(id);
  a->re.assign(a->m * a->n * a->elem, 0);
  a->complex = c == mxCOMPLEX;
  if (a->complex) a->im.assign(a->m * a->n * a->elem, 0);
  return a;
}
mxArray *mxCreateNumericMatrix(mwSize m, mwSize n, mxClassID id, mxComplexity c) {
  mwSize d[2] = {m, n};
  return mxCreateNumericArray(2, d, id, c);
}
mxArray *mxCreateDoubleMatrix(mwSize m, mwSize n, mxComplexity c) { return mxCreateNumericMatrix(m, n, mxDOUBLE_CLASS, c); }
void mxDestroyArray(mxArray *a) { delete a; }
bool mxIsLogicalScalarTrue(const mxArray *a) { return a && a->id == mxLOGICAL_CLASS && !a->re.empty() && a->re[0]; }
int mexPrintf(const char *fmt, ...) {
  char buf[4096];
  va_list ap;
  va_start(ap, fmt);
  int n = vsnprintf(buf, sizeof buf, fmt, ap);
  va_end(ap);
  g_log += buf;
  return n;
}
void mexErrMsgTxt(const char *msg) { throw std::runtime_error(msg); }
int mexEvalString(const char *cmd) {
  g_eval.push_back(cmd);
  return 0;
}
mxArray *mexGetVariable(const char *, const char *name) {
  if (strcmp(name, "abort_photonMC")) return nullptr;
  if (g_abort_after >= 0 && --g_abort_after < 0) g_abort = 1;
  mxArray *a = mxCreateNumericMatrix(1, 1, mxLOGICAL_CLASS, mxREAL);
  a->re[0] = (char)g_abort;
  return a;
}

// ---- test driver interface ----


mxArray *shim_create(int id, size_t m, size_t n, int complex, const void *re, const void *im) {
  mxArray *a = mxCreateNumericMatrix(m, n, (mxClassID)id, complex ? mxCOMPLEX : mxREAL);
  if (re && m * n) memcpy(a->re.data(), re, m * n * a->elem);
  if (im && complex && m * n) memcpy(a->im.data(), im, m * n * a->elem);
  return a;
}
int shim_invoke(int nlhs, mxArray **plhs, int nrhs, const mxArray **prhs) {
  g_err.clear();
  try {
    mexFunction(nlhs, plhs, nrhs, prhs);
  } catch (const std::exception &e) {
    g_err = e.what();
    return 1;
  }
  return 0;
}
const char *shim_error() { return g_err.c_str(); }
const char *shim_log() { return g_log.c_str(); }
int shim_eval_count() { return (int)g_eval.size(); }
void shim_set_abort_after(int polls) { g_abort = 0; g_abort_after = polls; }
int shim_class(const mxArray *a) { return a->id; }
size_t shim_m(const mxArray *a) { return a->m; }
size_t shim_n(const mxArray *a) { return a->n; }
int shim_is_complex(const mxArray *a) { return a->complex; }
}
