// mc_main.hpp -- the drop-in MC3D / MC2D executables (cpp/3d/MC3D.cpp:34-94,
// cpp/2d/MC2D.cpp:38-122): same command line, messages, exit codes and files; the
// ErrorChecks / Init / MonteCarlo sequence is one vmc_run call on the GPU.
//
//   MC3D inputfile outputfile [--fp64|--fp32] [--device=N]
//   MC2D inputfile outputfile [-s] [--fp64|--fp32] [--device=N]
// The default arithmetic form is FP32 tracking; --fp64 selects the plain FP64 form.
#pragma once
#include <stdio.h>
#include <string.h>
#include <time.h>

#include "textio.hpp"

namespace vmcapp {

static bool g_quiet = false;

static int progress_print(double perc, void *) {
  if (!g_quiet) {
    printf("  %f %%\r", perc);
    fflush(stdout);
  }
  return 1;
}

inline int mc_main(int argc, char **argv, int dim) {
  banner(dim == 3 ? "ValoMC-3D" : "ValoMC-2D");
  if (argc < 3) {
    printf("Use syntax:\n");
    printf(" MC%dD inputfile outputfile\n", dim);
    if (dim == 2) {
      printf(" or \n");
      printf(" MC2D inputfile outputfile -s\n");
      printf(" to suppress progress bar.\n");
    }
    printf("\n");
    return 0;
  }
  vmc_options opt;
  vmc_default_options(&opt);
  for (int i = 3; i < argc; i++) {
    if (!strcmp(argv[i], "-s") && dim == 2) g_quiet = true;
    else if (!strcmp(argv[i], "--fp64")) opt.precision = VMC_FP64;
    else if (!strcmp(argv[i], "--fp32")) opt.precision = VMC_FP32;
    else if (!strncmp(argv[i], "--device=", 9)) opt.device = atoi(argv[i] + 9);
  }
  opt.progress = progress_print;
  const char *fin = argv[1], *fout = argv[2];
  if (dim == 3) printf("Loading problem %s\n", fin);
  Problem P;
  if (load(fin, dim, P)) {
    printf("Error while loading!\n");
    return 1;
  }
  vmc_input in = to_input(P);
  printf("Initializing MC%dD\n", dim);
  std::vector<double> ER((size_t)in.Ne), EI((size_t)in.Ne), EBR((size_t)in.Nb), EBI((size_t)in.Nb),
      DEBR((size_t)in.Nb), DEBI((size_t)in.Nb);
  vmc_output out;
  memset(&out, 0, sizeof(out));
  out.ER = ER.data(); out.EI = EI.data(); out.EBR = EBR.data(); out.EBI = EBI.data();
  out.DEBR = DEBR.data(); out.DEBI = DEBI.data();
  vmc_stats st;
  printf("Computing...\n");
  time_t t0 = time(NULL);
  int s = vmc_run(&in, &opt, &out, &st);
  time_t t1 = time(NULL);
  if (s >= VMC_NO_LIGHTSOURCE && s <= VMC_MISSING_BOUNDARY) {
    printf("MC Initialization failed!: Reason %s\n", vmc_status_string(s));
    return 1;
  }
  if (s != VMC_OK) {
    printf("MC computation failed!: %s %s\n", vmc_status_string(s), vmc_last_error());
    return 1;
  }
  if (dim == 3) printf("Initialization took %i seconds\n", (int)st.seconds_setup);
  printf("seed %llu\n", (unsigned long long)st.seed_used);
  printf("Saving problem\n");
  if (save(fout, (int)(t1 - t0), ER, EI, EBR, EBI, dim == 3 ? "%18.10e %18.10e\n" : "%e %e\n")) {
    printf("Error while saving!\n");
    return 1;
  }
  if (st.loss) printf(" %lld photons lost during computation!\n", (long long)st.loss);
  printf("Computation took %i seconds\n", (int)(t1 - t0));
  return 0;
}

}  // namespace vmcapp
