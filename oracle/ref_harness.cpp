/*
 * ref_harness.cpp -- drives the reference engine (cpp/3d/MC3D.hpp or cpp/2d/MC2D.hpp,
 * included unmodified from the reference tree) for the checker.  TEST INFRASTRUCTURE
 * ONLY; built by oracle/Makefile into oracle/_ref/ when the reference tree is present.
 *
 *   -DVMC_DIM=3|2    which engine
 *   -DVMC_TRACE      replay mode: the engine's uniforms come from a caller tape (the
 *                    injection seam is the mt_rng include guard, cpp/3d/mt_rng.hpp:1-2),
 *                    and every ER/EBR update is logged (through the Array include guard,
 *                    cpp/3d/Array.hpp:1-2), i.e. the element visited at each step.
 *   (default)        timed mode: the stock engine (MT19937, OpenMP), MonteCarlo() timed
 *                    with std::chrono, accumulators printed at full precision.
 *
 * Input files use the reference executable's text format (cpp/3d/MC3D.cpp:97-179,
 * cpp/2d/MC2D.cpp:125-203) and are read with the reference's own reader (cpp/fileio.hpp).
 *
 *   timed:  <bin> input.txt output.txt nthreads   (output "-": only the statistics line, on stdout)
 *   trace:  <bin> input.txt tape.bin output.txt
 * tape.bin: int64 nphot, int64 off[nphot+1], uint32 words[off[nphot]].
 */
#include <cinttypes>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <chrono>
#include <iomanip>
#include <iostream>
#include <string>
#include <vector>

#ifdef VMC_TRACE
/* ---- logging array: same public interface as the reference Array<T> ---- */
#define __ARRAY_HPP__
struct TraceSink {
  const void *er = nullptr, *ebr = nullptr;
  std::vector<long long> *out = nullptr;
  bool on = false;
};
static TraceSink g_sink;

template <class T>
class Array {
 public:
  Array() : IsRef(0), rank(0), Nx(0), Ny(0), Nz(0), Nxy(0), N(0), data(nullptr) {}
  Array(Array<T> &o) : IsRef(1), rank(o.rank), Nx(o.Nx), Ny(o.Ny), Nz(o.Nz), Nxy(o.Nxy), N(o.N), data(o.data) {}
  Array &operator=(const Array &o) {
    if (this != &o) {
      IsRef = 1; rank = o.rank; Nx = o.Nx; Ny = o.Ny; Nz = o.Nz; Nxy = o.Nxy; N = o.N; data = o.data;
    }
    return *this;
  }
  T *alloc(int_fast64_t a, int_fast64_t b, int_fast64_t c, int rk) {
    rank = rk; Nx = a; Ny = b; Nz = c; N = a * b * c; Nxy = a * b;
    data = new T[N > 0 ? N : 1];
    IsRef = 0;
    return data;
  }
  T *resize(int_fast64_t a, int_fast64_t b, int_fast64_t c) { return alloc(a, b, c, 3); }
  T *resize(int_fast64_t a, int_fast64_t b) { return alloc(a, b, 1, 2); }
  T *resize(int_fast64_t a) { return alloc(a, 1, 1, 1); }
  T &operator()(int_fast64_t x, int_fast64_t y, int_fast64_t z) { return data[x + Nx * y + Nxy * z]; }
  T &operator()(int_fast64_t x, int_fast64_t y) { return data[x + Nx * y]; }
  T &operator()(int_fast64_t x) { return data[x]; }
  T &operator[](int_fast64_t i) {
    if (g_sink.on) {
      if ((const void *)this == g_sink.er) g_sink.out->push_back((long long)i);
      else if ((const void *)this == g_sink.ebr) g_sink.out->push_back(-1 - (long long)i);
    }
    return data[i];
  }
  void destroy() {
    if (!IsRef && data) delete[] data;
    data = nullptr; rank = Nx = Ny = Nz = Nxy = N = 0;
  }
  ~Array() { destroy(); }
  int IsRef;
  int_fast64_t rank, Nx, Ny, Nz, Nxy, N;
  T *data;
};

/* ---- tape-fed uniform source with the four mappings of cpp/3d/mt_rng.hpp:187-204 ---- */
#define __MT_RNG_HPP__
struct TapeState {
  const uint32_t *w = nullptr;
  long long pos = 0, end = 0;
  bool out = false;
};
static TapeState g_tape;
class mt_rng {
 public:
  mt_rng(unsigned long = 5489UL) {}
  void Seed(unsigned long) {}
  unsigned long ulrand() {
    if (g_tape.pos < g_tape.end) return g_tape.w[g_tape.pos++];
    g_tape.out = true;
    return 0x80000000UL;
  }
  double drand_closed() { return (double)ulrand() * (1.0 / 4294967295.0); }
  double drand_open() { return ((double)ulrand() + 0.5) * (1.0 / 4294967296.0); }
  double drand_open_up() { return (double)ulrand() * (1.0 / 4294967296.0); }
  double drand_open_down() { return ((double)ulrand() + 1.0) * (1.0 / 4294967296.0); }
};
#endif /* VMC_TRACE */

#if VMC_DIM == 3
#include "MC3D.hpp"
typedef MC3D Engine;
#define VMC_NV 4
#define VMC_NB 3
#define VMC_ND 3
#else
#include "MC2D.hpp"
typedef MC2D Engine;
#define VMC_NV 3
#define VMC_NB 2
#define VMC_ND 2
#endif
#include "../fileio.hpp"

static Engine MC;

static bool progress_cb(double) { return true; }
static void finalchecks_cb(int, int) {}

/* the executable's text loader, cpp/3d/MC3D.cpp:97-179 and cpp/2d/MC2D.cpp:125-203 */
static int load(const char *fin) {
  int_fast64_t Ne, Nb, Nr, sd1, sd2;
  FILE *fp = fopen(fin, "r");
  if (!fp) return 1;
  if (fscanf(fp, "%" SCNdFAST64 " %" SCNdFAST64 " %" SCNdFAST64 " %" SCNdFAST64 "\n", &Ne, &Nb, &Nr, &MC.Nphoton) != 4) return 1;
  if (fscanf(fp, "%lf %lf %" SCNdFAST64 " %" SCNdFAST64 "\n", &MC.f, &MC.phase0, &sd1, &sd2) != 4) return 1;
  MC.seed = sd2 ? (unsigned long)sd1 : 5489UL;
  char line[5012];
  if (!fgets(line, 5011, fp)) return 1;
  if (MC.phase0 < 0) MC.phase0 += 2 * M_PI * ceil(-MC.phase0 / (2 * M_PI));
  readAndResize(fp, (int)Ne, VMC_NV, true, &MC.H, "H");
  readAndResize(fp, (int)Nb, VMC_NB, true, &MC.BH, "BH");
  readAndResize(fp, (int)Nr, VMC_ND, true, &MC.r, "r");
  readAndResize(fp, (int)Ne, 1, true, &MC.mua, &MC.mus, &MC.g, &MC.n, "mua", "mus", "g", "n");
  readAndResize(fp, (int)Nb, 1, true, &MC.BCType, "BCType");
  readAndResize(fp, (int)Nb, 1, false, &MC.BCn, "BCn");
  readAndResize(fp, (int)Nb, VMC_ND, false, &MC.BCLNormal, "BCLightDirection");
#if VMC_DIM == 3
  readAndResize(fp, (int)Nb, 1, false, &MC.BCLightDirectionType, "BCLDirType");
  readAndResize(fp, (int)Nb, 1, false, &MC.BCIntensity, "BCIntensity");
  if (MC.BCLightDirectionType.N == 0) {
    MC.BCLightDirectionType.resize(Nb, 1);
    for (int i = 0; i < Nb; i++) MC.BCLightDirectionType[i] = 'n';
  }
#else
  readAndResize(fp, (int)Nb, 1, false, &MC.BCLightDirectionType, "BCLightDirectionType");
  readAndResize(fp, (int)Nb, 1, false, &MC.BCIntensity, "BCIntensity");
  readAndResize(fp, (int)Nb, 1, false, &MC.GaussianSigma, "GaussianSigma");
#endif
  fclose(fp);
  return 0;
}

static void dump_arrays(FILE *fo) {
  fprintf(fo, "ER_EI %ld\n", (long)MC.ER.N);
  for (long i = 0; i < (long)MC.ER.N; i++) fprintf(fo, "%.17e %.17e\n", MC.ER.data[i], MC.EI.data[i]);
  fprintf(fo, "EBR_EBI_DEBR_DEBI %ld\n", (long)MC.EBR.N);
  for (long i = 0; i < (long)MC.EBR.N; i++)
    fprintf(fo, "%.17e %.17e %.17e %.17e\n", MC.EBR.data[i], MC.EBI.data[i], MC.DEBR.data[i], MC.DEBI.data[i]);
}

int main(int argc, char **argv) {
  if (argc < 4) {
    fprintf(stderr, "usage: %s input.txt (output.txt nthreads | tape.bin output.txt)\n", argv[0]);
    return 2;
  }
  if (load(argv[1])) { fprintf(stderr, "load failed\n"); return 1; }
  try {
    MC.ErrorChecks();
    MC.Init();
  } catch (mcerror e) {
    printf("MCERROR %d %s\n", (int)e, errorstring(e));
    return 3;
  }
#ifndef VMC_TRACE
  int nthreads = atoi(argv[3]);
#ifdef USE_OMP
  if (nthreads > 0) omp_set_num_threads(nthreads);
#endif
  auto t0 = std::chrono::steady_clock::now();
  MC.MonteCarlo(progress_cb, finalchecks_cb);
  auto t1 = std::chrono::steady_clock::now();
  double secs = std::chrono::duration<double>(t1 - t0).count();
#ifdef USE_OMP
  int used = omp_get_max_threads();
#else
  int used = 1;
#endif
  if (strcmp(argv[2], "-") == 0) {  /* timing only: the statistics line on stdout, no arrays */
    printf("STATS seconds %.9f loss %ld threads %d nphoton %ld\n", secs, (long)MC.loss, used, (long)MC.Nphoton);
    return 0;
  }
  FILE *fo = fopen(argv[2], "w");
  if (!fo) return 1;
  fprintf(fo, "STATS seconds %.9f loss %ld threads %d nphoton %ld\n", secs, (long)MC.loss, used, (long)MC.Nphoton);
  dump_arrays(fo);
  fclose(fo);
#else
  FILE *ft = fopen(argv[2], "rb");
  if (!ft) return 1;
  int64_t nphot = 0;
  if (fread(&nphot, 8, 1, ft) != 1) return 1;
  std::vector<int64_t> off((size_t)nphot + 1);
  if (fread(off.data(), 8, off.size(), ft) != off.size()) return 1;
  std::vector<uint32_t> words((size_t)off[(size_t)nphot]);
  if (!words.empty() && fread(words.data(), 4, words.size(), ft) != words.size()) return 1;
  fclose(ft);
  FILE *fo = fopen(argv[3], "w");
  if (!fo) return 1;
  std::vector<long long> ev;
  g_sink.er = &MC.ER; g_sink.ebr = &MC.EBR; g_sink.out = &ev;
  Photon ph;
  memset(&ph, 0, sizeof(ph));
  for (int64_t p = 0; p < nphot; p++) {
    g_tape.w = words.data(); g_tape.pos = off[(size_t)p]; g_tape.end = off[(size_t)p + 1]; g_tape.out = false;
    ev.clear();
    long loss0 = MC.loss;
    g_sink.on = true;
    MC.CreatePhoton(&ph);
    MC.PropagatePhoton(&ph);
    g_sink.on = false;
    /* terminal code in the oracle's encoding: exit events are already logged (-1-ib) */
    const char *term = "";
    if (g_tape.out) term = "TAPE_END";
    else if (MC.loss != loss0) term = "LOST";
    else if (ev.empty() || ev.back() >= 0) term = "ROULETTE";
    fprintf(fo, "P %ld used %lld n %zu %s :", (long)p, (long long)(g_tape.pos - off[(size_t)p]), ev.size(), term);
    for (long long e : ev) fprintf(fo, " %lld", e);
    fprintf(fo, "\n");
  }
  dump_arrays(fo);
  fclose(fo);
#endif
  return 0;
}
