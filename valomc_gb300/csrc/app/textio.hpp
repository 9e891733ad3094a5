// textio.hpp -- the external executables' text input/output (cpp/fileio.hpp,
// cpp/3d/MC3D.cpp:97-201, cpp/2d/MC2D.cpp:125-226), for the drop-in MC3D / MC2D.
//
// Input: "Ne Nb Nr Nphoton", "f phase0 seed seedflag", one skipped line, then tagged
// blocks in a fixed order.  A block is read when its tag line holds exactly the expected
// names; otherwise the stream is rewound to the tag and the block is left empty (an
// optional block that is absent -- or misnamed -- is skipped, and so is everything the
// reference would skip).  Rows are read column by column into the column-major arrays
// the C ABI takes.  A short or unreadable block of a required array ends the program with
// "Reading error!" and exit code 1, as the reference does.
#pragma once
#include <inttypes.h>
#include <math.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include <chrono>
#include <sstream>
#include <string>
#include <vector>

#include "valomc_gb300.h"

namespace vmcapp {

struct Problem {
  int dim = 3;
  int64_t Ne = 0, Nb = 0, Nr = 0, Nphoton = 0;
  double f = 0, phase0 = 0;
  int64_t sd1 = 0, sd2 = 0;
  std::vector<int64_t> H, BH;
  std::vector<double> r, mua, mus, g, n, BCn, BCLNormal, BCIntensity, GaussianSigma;
  std::vector<char> BCType, BCLightDirectionType;
  int64_t rows_H = 0, rows_BH = 0, rows_r = 0, rows_opt = 0, rows_BCType = 0, rows_BCn = 0, rows_BCLN = 0,
          rows_BCLDT = 0, rows_BCI = 0, rows_GS = 0;
};

inline bool parse_value(std::stringstream &ss, int64_t &v) {
  long long x = 0;
  if (!(ss >> x)) { v = 0; return false; }
  v = (int64_t)x;
  return true;
}
inline bool parse_value(std::stringstream &ss, double &v) {
  std::string w;
  if (!(ss >> w)) { v = 0; return false; }
  char *end = nullptr;
  v = strtod(w.c_str(), &end);
  return true;
}
inline bool parse_value(std::stringstream &ss, char &v) {
  if (!(ss >> v)) { v = 0; return false; }
  return true;
}

// Reads one block of `height` rows into each of `arrays` (each `width` columns).
// Returns the number of rows read (height), 0 when the tag is absent, -1 on a read error.
template <class T>
int64_t read_block(FILE *fp, int64_t height, int width, const std::vector<std::string> &names,
                   const std::vector<std::vector<T> *> &arrays, bool halt) {
  char line[5012];
  fpos_t pos;
  fgetpos(fp, &pos);
  if (!fgets(line, 5011, fp)) return 0;
  std::stringstream tag(line);
  std::vector<std::string> words;
  std::string w;
  while (tag >> w) words.push_back(w);
  bool match = words.size() == names.size();
  for (size_t i = 0; match && i < names.size(); i++) match = words[i] == names[i];
  if (!match) {
    fsetpos(fp, &pos);
    return 0;
  }
  for (auto *a : arrays) a->assign((size_t)(height * width), T());
  bool ok = true;
  for (int64_t i = 0; i < height && ok; i++) {
    if (feof(fp) || !fgets(line, 5011, fp)) { ok = false; break; }
    std::stringstream ls(line);
    for (auto *a : arrays)
      for (int k = 0; k < width; k++) parse_value(ls, (*a)[(size_t)(i + height * k)]);
  }
  if (!ok) {
    for (auto *a : arrays) a->clear();
    if (halt) {
      printf("Reading error!\n");
      exit(1);
    }
    return -1;
  }
  for (size_t j = 0; j < arrays.size(); j++) printf("%12s   (%" PRId64 "x%d)\n", names[j].c_str(), height, width);
  return height;
}

template <class T>
int64_t read_one(FILE *fp, int64_t height, int width, const char *name, std::vector<T> &a, bool halt) {
  int64_t r = read_block<T>(fp, height, width, {name}, {&a}, halt);
  return r > 0 ? r : 0;
}

inline int load(const char *fin, int dim, Problem &P) {
  P.dim = dim;
  FILE *fp = fopen(fin, "r");
  if (!fp) return 1;
  long long ne = 0, nb = 0, nr = 0, nph = 0, s1 = 0, s2 = 0;
  if (fscanf(fp, "%lld %lld %lld %lld\n", &ne, &nb, &nr, &nph) != 4) { fclose(fp); return 1; }
  if (fscanf(fp, "%lf %lf %lld %lld\n", &P.f, &P.phase0, &s1, &s2) != 4) { fclose(fp); return 1; }
  P.Ne = ne; P.Nb = nb; P.Nr = nr; P.Nphoton = nph; P.sd1 = s1; P.sd2 = s2;
  char line[5012];
  if (!fgets(line, 5011, fp)) { fclose(fp); return 1; }
  // a negative phase0 is made positive by a multiple of 2 pi (cpp/3d/MC3D.cpp:141-143)
  if (P.phase0 < 0) P.phase0 += 2 * M_PI * ceil(-P.phase0 / (2 * M_PI));
  printf("Constants:\n");
  printf("  %10s   (%e)\n", "f", P.f);
  printf("  %10s   (%e)\n", "phase0", P.phase0);
  printf("  %10s   (%lld)\n", "Ne", ne);
  printf("  %10s   (%lld)\n", "Nb", nb);
  printf("  %10s   (%lld)\n", "Nr", nr);
  printf("  %10s   (%lld)\n", "Nphoton", nph);
  printf("Arrays:\n");
  P.rows_H = read_one(fp, P.Ne, dim + 1, "H", P.H, true);
  P.rows_BH = read_one(fp, P.Nb, dim, "BH", P.BH, true);
  P.rows_r = read_one(fp, P.Nr, dim, "r", P.r, true);
  int64_t ro = read_block<double>(fp, P.Ne, 1, {"mua", "mus", "g", "n"}, {&P.mua, &P.mus, &P.g, &P.n}, true);
  P.rows_opt = ro > 0 ? ro : 0;
  P.rows_BCType = read_one(fp, P.Nb, 1, "BCType", P.BCType, true);
  P.rows_BCn = read_one(fp, P.Nb, 1, "BCn", P.BCn, false);
  P.rows_BCLN = read_one(fp, P.Nb, dim, "BCLightDirection", P.BCLNormal, false);
  P.rows_BCLDT = read_one(fp, P.Nb, 1, dim == 3 ? "BCLDirType" : "BCLightDirectionType", P.BCLightDirectionType, false);
  P.rows_BCI = read_one(fp, P.Nb, 1, "BCIntensity", P.BCIntensity, false);
  if (dim == 2) P.rows_GS = read_one(fp, P.Nb, 1, "GaussianSigma", P.GaussianSigma, false);
  fclose(fp);
  return 0;
}

inline vmc_input to_input(const Problem &P) {
  vmc_input in;
  memset(&in, 0, sizeof(in));
  in.dim = P.dim;
  in.Ne = P.rows_H;
  in.Nb = P.rows_BH;
  in.Nr = P.rows_r;
  in.H = P.H.data();
  in.BH = P.BH.data();
  in.r = P.r.data();
  in.BCType = P.BCType.data(); in.n_BCType = P.rows_BCType;
  in.BCn = P.BCn.data(); in.n_BCn = P.rows_BCn;
  in.BCLNormal = P.BCLNormal.data(); in.n_BCLNormal = P.rows_BCLN;
  in.BCLightDirectionType = P.BCLightDirectionType.data(); in.n_BCLightDirectionType = P.rows_BCLDT;
  in.BCIntensity = P.BCIntensity.data(); in.n_BCIntensity = P.rows_BCI;
  in.GaussianSigma = P.GaussianSigma.data(); in.n_GaussianSigma = P.rows_GS;
  in.mua = P.mua.data(); in.n_mua = P.rows_opt;
  in.mus = P.mus.data(); in.n_mus = P.rows_opt;
  in.g = P.g.data(); in.n_g = P.rows_opt;
  in.n = P.n.data(); in.n_n = P.rows_opt;
  in.f = P.f;
  in.phase0 = P.phase0;
  in.Nphoton = P.Nphoton;
  in.seed_given = P.sd2 ? 1 : 0;
  in.seed = (uint64_t)P.sd1;
  return in;
}

// "%i 0" then Ne rows "ER EI" and Nb rows "EBR EBI" (cpp/3d/MC3D.cpp:186-201: %18.10e;
// cpp/2d/MC2D.cpp:210-226: %e)
inline int save(const char *fout, int seconds, const std::vector<double> &ER, const std::vector<double> &EI,
                const std::vector<double> &EBR, const std::vector<double> &EBI, const char *fmt) {
  FILE *fp = fopen(fout, "w");
  if (!fp) return 1;
  fprintf(fp, "%i 0\n", seconds);
  for (size_t i = 0; i < ER.size(); i++) fprintf(fp, fmt, ER[i], EI[i]);
  for (size_t i = 0; i < EBR.size(); i++) fprintf(fp, fmt, EBR[i], EBI[i]);
  fclose(fp);
  return 0;
}

inline void banner(const char *name) {
  printf("                 %s\n", name);
  printf("--------------------------------------------\n");
  printf("  Version:  v1.0rc (GB300 sm_103a photon engine)\n");
  printf("  Revision: 1\n");
  printf("  CUDA enabled: persistent photon pool\n");
  printf("--------------------------------------------\n");
}

}  // namespace vmcapp
