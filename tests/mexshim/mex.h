/* Minimal stand-in for MATLAB's mex.h / matrix.h, for testing the MEX gateways without
 * MATLAB.  Test infrastructure only: declares the handful of mx / mex functions the
 * gateways call, implemented by mexshim.cpp over plain heap arrays. */
#ifndef VMC_MEXSHIM_H
#define VMC_MEXSHIM_H
#include <stddef.h>
#include <stdbool.h>

typedef size_t mwSize;
typedef enum {
  mxUNKNOWN_CLASS = 0, mxCELL_CLASS, mxSTRUCT_CLASS, mxLOGICAL_CLASS, mxCHAR_CLASS, mxVOID_CLASS, mxDOUBLE_CLASS,
  mxSINGLE_CLASS, mxINT8_CLASS, mxUINT8_CLASS, mxINT16_CLASS, mxUINT16_CLASS, mxINT32_CLASS, mxUINT32_CLASS,
  mxINT64_CLASS, mxUINT64_CLASS, mxFUNCTION_CLASS
} mxClassID;
typedef enum { mxREAL = 0, mxCOMPLEX = 1 } mxComplexity;
typedef struct mxArray_tag mxArray;

#ifdef __cplusplus
extern "C" {
#endif
mxClassID mxGetClassID(const mxArray *a);
mwSize mxGetNumberOfDimensions(const mxArray *a);
void *mxGetData(const mxArray *a);
void *mxGetImagData(const mxArray *a);
double *mxGetPr(const mxArray *a);
size_t mxGetM(const mxArray *a);
size_t mxGetN(const mxArray *a);
mxArray *mxCreateNumericArray(mwSize ndim, const mwSize *dims, mxClassID id, mxComplexity c);
mxArray *mxCreateNumericMatrix(mwSize m, mwSize n, mxClassID id, mxComplexity c);
mxArray *mxCreateDoubleMatrix(mwSize m, mwSize n, mxComplexity c);
void mxDestroyArray(mxArray *a);
bool mxIsLogicalScalarTrue(const mxArray *a);
int mexPrintf(const char *fmt, ...);
void mexErrMsgTxt(const char *msg);
int mexEvalString(const char *cmd);
mxArray *mexGetVariable(const char *ws, const char *name);
/* the gateway every MEX file defines (C linkage, as MATLAB's header declares it) */
void mexFunction(int nlhs, mxArray *plhs[], int nrhs, const mxArray *prhs[]);
#ifdef __cplusplus
}
#endif
#endif
