// MC3Dmex -- MATLAB gateway on the GB300 engine; drop-in for cpp/3d/MC3Dmex.cpp:98-253.
// Build in MATLAB: mex -I<repo>/include MC3Dmex.cpp -L<repo>/valomc_gb300/_build -lvalomc_gb300
#include "mc_mex.hpp"

void mexFunction(int nlhs, mxArray **plhs, int nrhs, const mxArray **prhs) {
  vmcmex::gateway(nlhs, plhs, nrhs, prhs, 3);
}
