// textio.hpp -- the external executables' text input/output (cpp/fileio.hpp,
// cpp/3d/MC3D.cpp:97-201, cpp/2d/MC2D.cpp:125-226), for the drop-in MC3D / MC2D.
//
// Input: "Ne Nb Nr Nphoton", "f phase0 seed seedflag", one skipped line, then tagged
// blocks in a fixed order (the reference's readers take about 2 s for the 648k-tet
// phantom; this one reads the file once and parses the rows of a block in parallel).  A block is read when its tag line holds exactly the expected
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

#include <float.h>
#include <limits.h>

#include <algorithm>
#include <chrono>
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

// The whole file is read into memory once.  Lines are cut as fgets(line, 5011, fp) cuts
// them (at a newline, or after 5010 characters), so a file reads exactly as the reference
// reads it; the rows of a block are then parsed in parallel.
struct Text {
  std::vector<char> buf;  // file contents + a terminating NUL
  size_t pos = 0;
  size_t size() const { return buf.size() - 1; }
};

constexpr size_t kLineMax = 5010;

// the next fgets line [b, e) from pos; false at the end of the data
inline bool next_line(const Text &t, size_t &pos, size_t &b, size_t &e) {
  const size_t n = t.size();
  if (pos >= n) return false;
  b = pos;
  const size_t lim = std::min(n, pos + kLineMax);
  const void *nl = memchr(t.buf.data() + pos, '\n', lim - pos);
  e = nl ? (size_t)(static_cast<const char *>(nl) - t.buf.data()) + 1 : lim;
  pos = e;
  return true;
}

inline bool is_ws(char c) { return c == ' ' || c == '\t' || c == '\n' || c == '\v' || c == '\f' || c == '\r'; }

// Token readers with the semantics of the reference's `linestream >> entry` (the GNU C++
// library's num_get in the "C" locale), one line at a time:
//  - white space is skipped first; at the end of the line the read fails and the entry
//    keeps its initial value (0 here; the reference's entry is uninitialised memory);
//  - an integer is [+-]digits in base 10; no digits give 0, out of range gives the
//    saturated value; both fail the stream;
//  - a double is the longest prefix [+-]digits[.digits][(e|E)[+-]digits] (no inf, nan or
//    hex), converted by strtod; a prefix strtod does not take whole ("1e", ".") gives 0,
//    an overflow gives +-DBL_MAX; both fail the stream;
//  - a char is the next non-blank character;
//  - once the stream has failed, every later read of the line leaves its entry as is.
struct LineCursor {
  const char *p, *e;
  bool failed = false;
  void skip() {
    while (p < e && is_ws(*p)) p++;
  }
  void get(int64_t &v) {
    if (failed) return;
    skip();
    if (p >= e) { failed = true; return; }
    bool neg = false;
    if (*p == '+' || *p == '-') { neg = *p == '-'; p++; }
    if (p >= e || *p < '0' || *p > '9') { v = 0; failed = true; return; }
    unsigned long long x = 0;
    bool over = false;
    while (p < e && *p >= '0' && *p <= '9') {
      const unsigned d = (unsigned)(*p - '0');
      if (x > (ULLONG_MAX - d) / 10) over = true;
      else x = x * 10 + d;
      p++;
    }
    const unsigned long long lim = neg ? (unsigned long long)LLONG_MAX + 1ull : (unsigned long long)LLONG_MAX;
    if (over || x > lim) {
      v = neg ? LLONG_MIN : LLONG_MAX;
      failed = true;
      return;
    }
    v = neg ? (int64_t)(0ull - x) : (int64_t)x;
  }
  void get(double &v) {
    if (failed) return;
    skip();
    if (p >= e) { failed = true; return; }
    char buf[kLineMax + 2];
    size_t n = 0;
    if (*p == '+' || *p == '-') buf[n++] = *p++;
    bool mant = false, dec = false, sci = false;
    while (p < e) {
      const char c = *p;
      if (c >= '0' && c <= '9') {
        buf[n++] = c;
        mant = true;
      } else if (c == '.' && !dec && !sci) {
        buf[n++] = c;
        dec = true;
      } else if ((c == 'e' || c == 'E') && mant && !sci) {
        buf[n++] = c;
        sci = true;
        if (p + 1 < e && (p[1] == '+' || p[1] == '-')) buf[n++] = *++p;
      } else {
        break;
      }
      p++;
    }
    buf[n] = 0;
    char *end = nullptr;
    const double x = strtod(buf, &end);
    if (n == 0 || end == buf || *end != 0) { v = 0; failed = true; return; }
    if (x == HUGE_VAL) { v = DBL_MAX; failed = true; return; }
    if (x == -HUGE_VAL) { v = -DBL_MAX; failed = true; return; }
    v = x;
  }
  void get(char &v) {
    if (failed) return;
    skip();
    if (p >= e) { failed = true; return; }
    v = *p++;
  }
};

// Reads one block of `height` rows into each of `arrays` (each `width` columns).
// Returns the number of rows read (height), 0 when the tag is absent, -1 on a read error.
template <class T>
int64_t read_block(Text &t, int64_t height, int width, const std::vector<std::string> &names,
                   const std::vector<std::vector<T> *> &arrays, bool halt) {
  size_t pos = t.pos, b = 0, e = 0;
  if (!next_line(t, pos, b, e)) return 0;
  std::vector<std::string> words;
  {
    size_t i = b;
    while (i < e) {
      while (i < e && is_ws(t.buf[i])) i++;
      size_t j = i;
      while (j < e && !is_ws(t.buf[j])) j++;
      if (j > i) words.emplace_back(t.buf.data() + i, j - i);
      i = j;
    }
  }
  bool match = words.size() == names.size();
  for (size_t i = 0; match && i < names.size(); i++) match = words[i] == names[i];
  if (!match) return 0;  // the tag is left for the next reader
  std::vector<size_t> lb((size_t)std::max<int64_t>(height, 0)), le(lb.size());
  bool ok = true;
  for (int64_t i = 0; i < height; i++)
    if (!next_line(t, pos, lb[(size_t)i], le[(size_t)i])) { ok = false; break; }
  if (!ok) {
    t.pos = pos;
    for (auto *a : arrays) a->clear();
    if (halt) {
      printf("Reading error!\n");
      exit(1);
    }
    return -1;
  }
  t.pos = pos;
  for (auto *a : arrays) a->assign((size_t)(height * width), T());
#pragma omp parallel for schedule(static, 4096)
  for (int64_t i = 0; i < height; i++) {
    LineCursor c{t.buf.data() + lb[(size_t)i], t.buf.data() + le[(size_t)i]};
    for (auto *a : arrays)
      for (int k = 0; k < width; k++) c.get((*a)[(size_t)(i + height * k)]);
  }
  for (size_t j = 0; j < arrays.size(); j++) printf("%12s   (%" PRId64 "x%d)\n", names[j].c_str(), height, width);
  return height;
}

template <class T>
int64_t read_one(Text &t, int64_t height, int width, const char *name, std::vector<T> &a, bool halt) {
  int64_t r = read_block<T>(t, height, width, {name}, {&a}, halt);
  return r > 0 ? r : 0;
}

// the header's fscanf("... \n"): the values, then any run of white space
inline bool scan_header(Text &t, const char *fmt, int nval, void *a, void *b, void *c, void *d) {
  char f2[64];
  snprintf(f2, sizeof f2, "%s%%n", fmt);
  int used = 0;
  if (sscanf(t.buf.data() + t.pos, f2, a, b, c, d, &used) != nval) return false;
  t.pos += (size_t)used;
  while (t.pos < t.size() && is_ws(t.buf[t.pos])) t.pos++;
  return true;
}

inline int load(const char *fin, int dim, Problem &P) {
  P.dim = dim;
  Text t;
  {
    FILE *fp = fopen(fin, "rb");
    if (!fp) return 1;
    fseek(fp, 0, SEEK_END);
    long sz = ftell(fp);
    fseek(fp, 0, SEEK_SET);
    if (sz < 0) { fclose(fp); return 1; }
    t.buf.resize((size_t)sz + 1);
    size_t got = fread(t.buf.data(), 1, (size_t)sz, fp);
    fclose(fp);
    t.buf.resize(got + 1);
    t.buf[got] = 0;
  }
  long long ne = 0, nb = 0, nr = 0, nph = 0, s1 = 0, s2 = 0;
  if (!scan_header(t, "%lld %lld %lld %lld", 4, &ne, &nb, &nr, &nph)) return 1;
  if (!scan_header(t, "%lf %lf %lld %lld", 4, &P.f, &P.phase0, &s1, &s2)) return 1;
  P.Ne = ne; P.Nb = nb; P.Nr = nr; P.Nphoton = nph; P.sd1 = s1; P.sd2 = s2;
  {
    size_t b = 0, e = 0;
    if (!next_line(t, t.pos, b, e)) return 1;  // the skipped grid-size line
  }
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
  P.rows_H = read_one(t, P.Ne, dim + 1, "H", P.H, true);
  P.rows_BH = read_one(t, P.Nb, dim, "BH", P.BH, true);
  P.rows_r = read_one(t, P.Nr, dim, "r", P.r, true);
  int64_t ro = read_block<double>(t, P.Ne, 1, {"mua", "mus", "g", "n"}, {&P.mua, &P.mus, &P.g, &P.n}, true);
  P.rows_opt = ro > 0 ? ro : 0;
  P.rows_BCType = read_one(t, P.Nb, 1, "BCType", P.BCType, true);
  P.rows_BCn = read_one(t, P.Nb, 1, "BCn", P.BCn, false);
  P.rows_BCLN = read_one(t, P.Nb, dim, "BCLightDirection", P.BCLNormal, false);
  P.rows_BCLDT = read_one(t, P.Nb, 1, dim == 3 ? "BCLDirType" : "BCLightDirectionType", P.BCLightDirectionType, false);
  P.rows_BCI = read_one(t, P.Nb, 1, "BCIntensity", P.BCIntensity, false);
  if (dim == 2) P.rows_GS = read_one(t, P.Nb, 1, "GaussianSigma", P.GaussianSigma, false);
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
  // rows formatted in parallel into chunk buffers, written in order
  const int64_t n1 = (int64_t)ER.size(), n = n1 + (int64_t)EBR.size();
  const int64_t rows_per_chunk = 16384;
  const int64_t nchunk = (n + rows_per_chunk - 1) / rows_per_chunk;
  std::vector<std::string> out((size_t)nchunk);
#pragma omp parallel for schedule(dynamic, 1)
  for (int64_t c = 0; c < nchunk; c++) {
    std::string &o = out[(size_t)c];
    char line[128];
    for (int64_t i = c * rows_per_chunk; i < std::min(n, (c + 1) * rows_per_chunk); i++) {
      const double a = i < n1 ? ER[(size_t)i] : EBR[(size_t)(i - n1)];
      const double b = i < n1 ? EI[(size_t)i] : EBI[(size_t)(i - n1)];
      int k = snprintf(line, sizeof line, fmt, a, b);
      if (k > 0) o.append(line, (size_t)std::min(k, (int)sizeof line - 1));
    }
  }
  for (auto &o : out) fwrite(o.data(), 1, o.size(), fp);
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
