// MC3D -- drop-in for the reference MC3D executable (cpp/3d/MC3D.cpp:34-94).
#include "mc_main.hpp"

int main(int argc, char **argv) { return vmcapp::mc_main(argc, argv, 3); }
