// MC2D -- drop-in for the reference MC2D executable (cpp/2d/MC2D.cpp:38-122).
#include "mc_main.hpp"

int main(int argc, char **argv) { return vmcapp::mc_main(argc, argv, 2); }
