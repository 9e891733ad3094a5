/*
 * ref_textio.cpp -- the reference executables' text reader, for the checker.  TEST
 * INFRASTRUCTURE ONLY; built by oracle/Makefile into oracle/_ref/ when the reference tree
 * is present.
 *
 * The reference's own reader (cpp/fileio.hpp, over cpp/3d/Array.hpp) is included
 * unmodified and called in the order of the reference loaders (LoadProblem_TXT,
 * cpp/3d/MC3D.cpp:116-171 and cpp/2d/MC2D.cpp:148-203): the header lines by fscanf, one
 * skipped line, then the tagged blocks.  Every array it read is written in the format of
 * the package's vmc_textdump, so the two readers can be compared value by value.
 *
 * The reference allocates arrays with new[] and leaves entries that a failed stream did
 * not write uninitialised; this harness makes new[] return zeroed memory so that those
 * entries read as 0, as the package's reader leaves them.
 *
 *   ref_textio <2|3> input.txt dump.txt
 */
#include <cinttypes>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <iomanip>
#include <iostream>
#include <new>
#include <string>
#include <type_traits>
#include <vector>

void *operator new[](std::size_t n) {
  void *p = std::calloc(1, n ? n : 1);
  if (!p) throw std::bad_alloc();
  return p;
}
void operator delete[](void *p) noexcept { std::free(p); }
void operator delete[](void *p, std::size_t) noexcept { std::free(p); }

#include "Array.hpp"
#include "../fileio.hpp"

template <class T>
static void dump(FILE *f, const char *name, Array<T> &a) {
  fprintf(f, "%s %lld %lld\n", name, (long long)a.Nx, (long long)a.N);
  // column-major, as the package stores its arrays
  for (int_fast64_t i = 0; i < a.N; i++) {
    if (std::is_same<T, double>::value) fprintf(f, "%.17g\n", (double)a[i]);
    else fprintf(f, "%lld\n", (long long)a[i]);
  }
}

int main(int argc, char **argv) {
  if (argc != 4) return 2;
  const int dim = argv[1][0] - '0';
  FILE *fp = fopen(argv[2], "r");
  if (!fp) return 1;
  int_fast64_t Ne = 0, Nb = 0, Nr = 0, Nphoton = 0, sd1 = 0, sd2 = 0;
  double f = 0, phase0 = 0;
  int fsr = fscanf(fp, "%li %li %li %li\n", &Ne, &Nb, &Nr, &Nphoton);
  fsr = fscanf(fp, "%lf %lf %li %li\n", &f, &phase0, &sd1, &sd2);
  (void)fsr;
  char line[5012];
  char *tmp = fgets(line, 5011, fp);
  (void)tmp;
  if (phase0 < 0) phase0 += 2 * M_PI * ceil(-phase0 / (2 * M_PI));
  Array<int_fast64_t> H, BH;
  Array<double> r, mua, mus, g, n, BCn, BCLNormal, BCIntensity, GaussianSigma;
  Array<char> BCType, BCLightDirectionType;
  if (dim == 3) {
    readAndResize(fp, (int)Ne, 4, true, &H, "H");
    readAndResize(fp, (int)Nb, 3, true, &BH, "BH");
    readAndResize(fp, (int)Nr, 3, true, &r, "r");
  } else {
    readAndResize(fp, Ne, 3, true, &H, "H");
    readAndResize(fp, Nb, 2, true, &BH, "BH");
    readAndResize(fp, Nr, 2, true, &r, "r");
  }
  readAndResize(fp, (int)Ne, 1, true, &mua, &mus, &g, &n, "mua", "mus", "g", "n");
  readAndResize(fp, (int)Nb, 1, true, &BCType, "BCType");
  readAndResize(fp, (int)Nb, 1, false, &BCn, "BCn");
  readAndResize(fp, (int)Nb, dim, false, &BCLNormal, "BCLightDirection");
  readAndResize(fp, (int)Nb, 1, false, &BCLightDirectionType, dim == 3 ? "BCLDirType" : "BCLightDirectionType");
  readAndResize(fp, (int)Nb, 1, false, &BCIntensity, "BCIntensity");
  if (dim == 2) readAndResize(fp, (int)Nb, 1, false, &GaussianSigma, "GaussianSigma");
  fclose(fp);
  FILE *o = fopen(argv[3], "w");
  if (!o) return 1;
  fprintf(o, "Ne %lld Nb %lld Nr %lld Nphoton %lld f %.17g phase0 %.17g seed %lld %lld\n", (long long)Ne,
          (long long)Nb, (long long)Nr, (long long)Nphoton, f, phase0, (long long)sd1, (long long)sd2);
  dump(o, "H", H);
  dump(o, "BH", BH);
  dump(o, "r", r);
  dump(o, "mua", mua);
  dump(o, "mus", mus);
  dump(o, "g", g);
  dump(o, "n", n);
  dump(o, "BCType", BCType);
  dump(o, "BCn", BCn);
  dump(o, "BCLightDirection", BCLNormal);
  dump(o, "BCLightDirectionType", BCLightDirectionType);
  dump(o, "BCIntensity", BCIntensity);
  if (dim == 2) dump(o, "GaussianSigma", GaussianSigma);
  fclose(o);
  return 0;
}
