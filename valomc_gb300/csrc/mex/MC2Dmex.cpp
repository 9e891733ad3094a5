// MC2Dmex -- MATLAB gateway on the GB300 engine; drop-in for cpp/2d/MC2Dmex.cpp:98-252.
// Build in MATLAB: mex -I<repo>/include MC2Dmex.cpp -L<repo>/valomc_gb300/_build -lvalomc_gb300
#include "mc_mex.hpp"

void mexFunction(int nlhs, mxArray **plhs, int nrhs, const mxArray **prhs) {
  vmcmex::gateway(nlhs, plhs, nrhs, prhs, 2);
}
