// textdump.cpp -- vmc_textdump <2|3> <input file> <dump file>
//
// Reads an input file as MC2D / MC3D read it and writes every array they took from it,
// one value per line (doubles as %.17g, integers and characters as integers), after a
// line with the constants.  It shows how a file is read without running a simulation.
#include <stdio.h>
#include <stdlib.h>

#include "textio.hpp"

template <class T>
static void dump(FILE *f, const char *name, const std::vector<T> &v, int64_t rows) {
  fprintf(f, "%s %lld %zu\n", name, (long long)rows, v.size());
  for (const T &x : v) {
    if constexpr (std::is_same<T, double>::value) fprintf(f, "%.17g\n", x);
    else fprintf(f, "%lld\n", (long long)x);
  }
}

int main(int argc, char **argv) {
  if (argc != 4 || (argv[1][0] != '2' && argv[1][0] != '3')) {
    printf("Use syntax:\n vmc_textdump 2|3 inputfile dumpfile\n");
    return 2;
  }
  const int dim = argv[1][0] - '0';
  vmcapp::Problem P;
  if (vmcapp::load(argv[2], dim, P)) {
    printf("Error while loading!\n");
    return 1;
  }
  FILE *f = fopen(argv[3], "w");
  if (!f) return 1;
  fprintf(f, "Ne %lld Nb %lld Nr %lld Nphoton %lld f %.17g phase0 %.17g seed %lld %lld\n", (long long)P.Ne,
          (long long)P.Nb, (long long)P.Nr, (long long)P.Nphoton, P.f, P.phase0, (long long)P.sd1, (long long)P.sd2);
  dump(f, "H", P.H, P.rows_H);
  dump(f, "BH", P.BH, P.rows_BH);
  dump(f, "r", P.r, P.rows_r);
  dump(f, "mua", P.mua, P.rows_opt);
  dump(f, "mus", P.mus, P.rows_opt);
  dump(f, "g", P.g, P.rows_opt);
  dump(f, "n", P.n, P.rows_opt);
  dump(f, "BCType", P.BCType, P.rows_BCType);
  dump(f, "BCn", P.BCn, P.rows_BCn);
  dump(f, "BCLightDirection", P.BCLNormal, P.rows_BCLN);
  dump(f, "BCLightDirectionType", P.BCLightDirectionType, P.rows_BCLDT);
  dump(f, "BCIntensity", P.BCIntensity, P.rows_BCI);
  if (dim == 2) dump(f, "GaussianSigma", P.GaussianSigma, P.rows_GS);
  fclose(f);
  return 0;
}
