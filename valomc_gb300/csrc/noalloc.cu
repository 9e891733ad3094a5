// noalloc.cu -- vmc_run_noalloc: the photon-pool launch with no device allocation.
//
// Who needs it: callers whose device memory belongs to their own allocator (a framework's
// caching allocator, a pool reserved up front by a serving process) cannot have a library
// call cudaMalloc / cudaFree: those calls synchronise the device and take memory outside
// the caller's accounting.  Here the job's device arrays are buffers the caller owns, and
// the pool kernel's scratch -- the launch control block, the one-entry job table, the
// rare-event counter slots and the emitting-face records -- is one file-scope device
// array of a fixed size, held by every GPU that loads the library until the process
// exits.  The kernel is the per-job form of the photon-pool kernel, the one multi-job
// batches launch: it reads the job descriptor from the job table in global memory (here in
// the scratch array).  vmc_run launches a single FP32 job in the one-job form, whose
// descriptor and Philox round keys are kernel parameters.  Both walk the same photons to
// the same results; the per-job form runs a few percent slower.
//
// In host code `g_scratch` names a host-side stand-in, not a device address, so the
// address is looked up once per device (with that device current) by
// cudaGetSymbolAddress and passed to the kernel.  The cached address belongs to the
// device's primary context: it does not survive cudaDeviceReset, so a process that resets
// a device must not call vmc_run_noalloc on it again.  Every call reuses the array: the
// counters that must start at zero are cleared at each call, and calls that overlap on the
// GPU race on it.  Each call runs on a non-blocking stream of its own, like the other entry
// points, and waits for it before returning.
#include <cuda_runtime.h>
#include <string.h>

#include <algorithm>
#include <chrono>
#include <mutex>
#include <string>
#include <vector>

#include "engine.hpp"

namespace vmc {
DeviceMesh *mesh_impl(vmc_mesh *m);
int mesh_precision_mask(const vmc_mesh *m);
}  // namespace vmc

using namespace vmc;

namespace {

constexpr size_t kScratchBytes = VMC_NOALLOC_SCRATCH_BYTES;
constexpr int kMaxSources = VMC_NOALLOC_MAX_SOURCES;

static __device__ __align__(256) unsigned char g_scratch[kScratchBytes];

constexpr size_t align256(size_t x) { return (x + 255) & ~size_t(255); }

// byte offsets inside the scratch array
constexpr size_t kOffCtl = 0;
constexpr size_t kOffJob = align256(kOffCtl + sizeof(Ctl));
constexpr size_t kOffBegin = align256(kOffJob + sizeof(JobDev));
constexpr size_t kOffJc = align256(kOffBegin + 2 * sizeof(int64_t));
constexpr size_t kOffLedger = align256(kOffJc + sizeof(unsigned long long) * kSlots * kJcN);
constexpr size_t kOffCdf = align256(kOffLedger + sizeof(double) * kSlots * kLgN);
constexpr size_t kOffCdfF = align256(kOffCdf + sizeof(double) * kMaxSources);
constexpr size_t kOffSrc = align256(kOffCdfF + sizeof(float) * kMaxSources);
constexpr size_t kOffSrcF = align256(kOffSrc + sizeof(SourceRec) * kMaxSources);
constexpr size_t kEnd = align256(kOffSrcF + sizeof(SourceRecF) * kMaxSources);
static_assert(kEnd <= kScratchBytes, "scratch layout exceeds VMC_NOALLOC_SCRATCH_BYTES");

// device address of g_scratch per device, looked up on the first call on that device
std::mutex g_addr_mu;
unsigned char *g_addr[128] = {nullptr};

int scratch_address(int device, unsigned char **out) {
  if (device < 0 || device >= 128) return VMC_ERR_INVALID_ARGUMENT;
  std::lock_guard<std::mutex> lk(g_addr_mu);
  if (!g_addr[device]) {
    void *p = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&p, g_scratch);  // the device is current here
    if (e != cudaSuccess) return cuda_status(e, "cudaGetSymbolAddress(g_scratch)");
    g_addr[device] = static_cast<unsigned char *>(p);
  }
  *out = g_addr[device];
  return VMC_OK;
}

// a caller buffer must be device memory of the launch device (a host pointer, or another
// GPU's memory, would fault in the kernel)
int check_device_buffer(const void *p, int device, const char *name) {
  cudaPointerAttributes a;
  cudaError_t e = cudaPointerGetAttributes(&a, p);
  if (e != cudaSuccess) {
    cudaGetLastError();
    set_error(std::string("vmc_run_noalloc: ") + name + " is not a device pointer");
    return VMC_ERR_INVALID_ARGUMENT;
  }
  if ((a.type != cudaMemoryTypeDevice && a.type != cudaMemoryTypeManaged) || a.device != device) {
    set_error(std::string("vmc_run_noalloc: ") + name + " must be device memory of device " + std::to_string(device));
    return VMC_ERR_INVALID_ARGUMENT;
  }
  return VMC_OK;
}

struct OwnStream {
  cudaStream_t s = nullptr;
  ~OwnStream() {
    if (s) cudaStreamDestroy(s);
  }
};

template <class T>
int put(unsigned char *base, size_t off, const T *src, size_t count, cudaStream_t st) {
  if (!count) return VMC_OK;
  VMC_CK(cudaMemcpyAsync(base + off, src, count * sizeof(T), cudaMemcpyHostToDevice, st));
  return VMC_OK;
}

}  // namespace

extern "C" int vmc_run_noalloc(vmc_mesh *mesh, const vmc_input *job, const vmc_options *opt_in,
                               const vmc_noalloc_buffers *dev, vmc_output *out, vmc_stats *stats) {
  auto t0 = std::chrono::steady_clock::now();
  if (!mesh || !job || !dev || !out || !dev->optics || !dev->bctype || !dev->bcn || !dev->acc)
    return VMC_ERR_INVALID_ARGUMENT;
  vmc_options o;
  if (opt_in) o = *opt_in;
  else vmc_default_options(&o);
  if (o.precision != VMC_FP32 && o.precision != VMC_FP64) return VMC_ERR_INVALID_ARGUMENT;
  if (o.rng != VMC_RNG_PHILOX || o.trace_photons) {
    set_error("vmc_run_noalloc runs Philox streams only (no tape, no trace)");
    return VMC_ERR_INVALID_ARGUMENT;
  }
  if (o.progress || o.cancel || o.timeout_s > 0) {
    set_error("vmc_run_noalloc does not poll a progress callback, a cancel flag or a timeout");
    return VMC_ERR_INVALID_ARGUMENT;
  }
  DeviceMesh *m = mesh_impl(mesh);
  if (m->device != o.device) {
    set_error("vmc_run_noalloc: the mesh lives on device " + std::to_string(m->device) + ", options.device is " +
              std::to_string(o.device));
    return VMC_ERR_INVALID_ARGUMENT;
  }
  if (!(mesh_precision_mask(mesh) & (o.precision == VMC_FP64 ? 1 : 2))) return VMC_ERR_INVALID_ARGUMENT;
  // host half: ErrorChecks + Init on the mesh's geometry
  vmc_input in = *job;
  in.dim = m->host.dim; in.Ne = m->host.Ne; in.Nb = m->host.Nb; in.Nr = m->host.Nr;
  in.H = m->host.H.data(); in.BH = m->host.BH.data(); in.r = m->host.r.data();
  in.HN = nullptr; in.n_HN = 0;
  int s = check_input(&in);
  if (s) return s;
  HostJob hj;
  s = build_job(&in, m->host, hj);
  if (s) return s;
  hj.seed = in.seed_given ? in.seed : clock_seed();
  const size_t ns = hj.src.size();
  if (ns > (size_t)kMaxSources) {
    set_error("vmc_run_noalloc: " + std::to_string(ns) + " emitting faces; the static scratch holds at most " +
              std::to_string(kMaxSources));
    return VMC_ERR_SIZE_LIMIT;
  }
  s = select_device(o.device);
  if (s) return s;
  if ((s = check_device_buffer(dev->optics, o.device, "optics")) || (s = check_device_buffer(dev->bctype, o.device, "bctype")) ||
      (s = check_device_buffer(dev->bcn, o.device, "bcn")) || (s = check_device_buffer(dev->acc, o.device, "acc")))
    return s;
  unsigned char *base = nullptr;
  s = scratch_address(o.device, &base);
  if (s) return s;
  const int64_t Ne = m->host.Ne, Nb = m->host.Nb;
  const size_t rows = hj.homogeneous ? 1 : (size_t)Ne;
  OwnStream own;
  VMC_CK(cudaStreamCreateWithFlags(&own.s, cudaStreamNonBlocking));
  cudaStream_t st = own.s;
  // the job's arrays into the caller's buffers
  std::vector<float> optf;
  if (o.precision == VMC_FP64) {
    VMC_CK(cudaMemcpyAsync(dev->optics, hj.optics.data(), rows * 4 * sizeof(double), cudaMemcpyHostToDevice, st));
  } else {
    optf.resize(rows * 4);
    for (size_t i = 0; i < rows * 4; i++) optf[i] = (float)hj.optics[i];
    VMC_CK(cudaMemcpyAsync(dev->optics, optf.data(), rows * 4 * sizeof(float), cudaMemcpyHostToDevice, st));
  }
  VMC_CK(cudaMemcpyAsync(dev->bctype, hj.bctype.data(), (size_t)Nb, cudaMemcpyHostToDevice, st));
  VMC_CK(cudaMemcpyAsync(dev->bcn, hj.bcn.data(), (size_t)Nb * sizeof(double), cudaMemcpyHostToDevice, st));
  VMC_CK(cudaMemsetAsync(dev->acc, 0, sizeof(double) * (size_t)(2 * Ne + 4 * Nb), st));
  // scratch: clear the control block and counters, then the face records and job table
  VMC_CK(cudaMemsetAsync(base + kOffCtl, 0, sizeof(Ctl), st));
  VMC_CK(cudaMemsetAsync(base + kOffJc, 0, sizeof(unsigned long long) * kSlots * kJcN, st));
  VMC_CK(cudaMemsetAsync(base + kOffLedger, 0, sizeof(double) * kSlots * kLgN, st));
  s = put(base, kOffCdf, hj.cdf.data(), ns, st);
  if (!s) s = put(base, kOffCdfF, hj.cdf_f.data(), ns, st);
  if (!s) s = put(base, kOffSrc, hj.src.data(), ns, st);
  if (!s) s = put(base, kOffSrcF, hj.src_f.data(), ns, st);
  if (s) return s;
  JobDev d;
  memset(&d, 0, sizeof(d));
  double *acc = dev->acc;
  d.geom = m->geom(o.precision);
  d.optics = dev->optics;
  d.opt_mask = hj.homogeneous ? 0 : -1;
  d.Ns = (int32_t)ns;
  d.Ne = (int32_t)Ne;
  d.Nb = (int32_t)Nb;
  d.cdf = reinterpret_cast<const double *>(base + kOffCdf);
  d.src = reinterpret_cast<const SourceRec *>(base + kOffSrc);
  d.cdf_f = reinterpret_cast<const float *>(base + kOffCdfF);
  d.src_f = reinterpret_cast<const SourceRecF *>(base + kOffSrcF);
  d.bctype = dev->bctype;
  d.bcn = dev->bcn;
  d.bnorm = m->d_bnorm;
  d.omega = hj.omega;
  d.k_scale = hj.k_scale;
  d.k_scale_f = (float)hj.k_scale;
  d.phase0 = hj.phase0;
  d.seed = hj.seed;
  d.stream = o.stream_id;
  d.pbegin = 0;
  d.pcount = in.Nphoton;
  d.poffset = o.photon_offset;
  d.ER = acc;
  d.EI = acc + Ne;
  d.EBR = acc + 2 * Ne;
  d.EBI = acc + 2 * Ne + Nb;
  d.DEBR = acc + 2 * Ne + 2 * Nb;
  d.DEBI = acc + 2 * Ne + 3 * Nb;
  d.jc = reinterpret_cast<unsigned long long *>(base + kOffJc);
  d.ledger = reinterpret_cast<double *>(base + kOffLedger);
  const int64_t begin[2] = {0, in.Nphoton};
  s = put(base, kOffJob, &d, 1, st);
  if (!s) s = put(base, kOffBegin, begin, 2, st);
  if (s) return s;
  // launch the pool kernel of this form with its scratch in g_scratch
  LaunchSpec spec;
  spec.dim = m->host.dim;
  spec.precision = o.precision;
  spec.fd = hj.omega > 0.0;
  spec.tape = false;
  const void *fn = select_kernel(spec);
  int sms = 0;
  VMC_CK(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, o.device));
  const int block = o.block_size > 0 ? o.block_size : 256;
  if (block % 32 || block > 256) return VMC_ERR_INVALID_ARGUMENT;  // the pool kernels run <= 256 threads
  int per_sm = 0;
  reset_carveout(fn);
  VMC_CK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, fn, block, 0));
  if (o.blocks_per_sm > 0) per_sm = std::min(per_sm, (int)o.blocks_per_sm);
  if (per_sm < 1) return VMC_ERR_INVALID_ARGUMENT;
  fit_carveout(fn, o.device, per_sm, 0);
  LaunchParams lp{};
  lp.jobs = reinterpret_cast<const JobDev *>(base + kOffJob);
  lp.job_begin = reinterpret_cast<const int64_t *>(base + kOffBegin);
  lp.njobs = 1;
  lp.chunk = o.fetch_chunk > 0 ? o.fetch_chunk : 32;
  lp.total = in.Nphoton;
  lp.max_steps = o.max_steps > 0 ? o.max_steps : 10000000;
  lp.ctl = reinterpret_cast<Ctl *>(base + kOffCtl);
  lp.stage_slots = 0;
  lp.dense = 0;
  lp.refill_min = o.refill_lanes > 0 ? o.refill_lanes : kDefaultRefill;
  auto t1 = std::chrono::steady_clock::now();
  if (in.Nphoton > 0) {
    void *args[] = {&lp};
    VMC_CK(cudaLaunchKernel(fn, dim3(per_sm * sms), dim3(block), args, 0, st));
  }
  VMC_CK(cudaStreamSynchronize(st));
  VMC_CK(cudaGetLastError());
  auto t2 = std::chrono::steady_clock::now();
  // results back to the host, normalised as MonteCarlo does
  Ctl hc;
  std::vector<double> h((size_t)(2 * Ne + 4 * Nb));
  std::vector<unsigned long long> jc((size_t)kSlots * kJcN);
  std::vector<double> lg((size_t)kSlots * kLgN);
  VMC_CK(cudaMemcpyAsync(&hc, base + kOffCtl, sizeof(Ctl), cudaMemcpyDeviceToHost, st));
  VMC_CK(cudaMemcpyAsync(h.data(), acc, h.size() * sizeof(double), cudaMemcpyDeviceToHost, st));
  VMC_CK(cudaMemcpyAsync(jc.data(), base + kOffJc, jc.size() * sizeof(unsigned long long), cudaMemcpyDeviceToHost, st));
  VMC_CK(cudaMemcpyAsync(lg.data(), base + kOffLedger, lg.size() * sizeof(double), cudaMemcpyDeviceToHost, st));
  VMC_CK(cudaStreamSynchronize(st));
  const double *ER = h.data(), *EI = ER + Ne, *EBR = EI + Ne, *EBI = EBR + Nb, *DEBR = EBI + Nb, *DEBI = DEBR + Nb;
  normalise(m->host, hj, in.Nphoton, ER, EI, EBR, EBI, DEBR, DEBI, out, o.normalize != 0 || !opt_in);
  if (out->HN) memcpy(out->HN, m->host.HN.data(), m->host.HN.size() * sizeof(int64_t));
  if (stats) {
    memset(stats, 0, sizeof(*stats));
    unsigned long long c[kJcN] = {0};
    double L[kLgN] = {0};
    for (int sl = 0; sl < kSlots; sl++) {
      for (int k = 0; k < kJcN; k++) c[k] += jc[(size_t)sl * kJcN + k];
      for (int k = 0; k < kLgN; k++) L[k] += lg[(size_t)sl * kLgN + k];
    }
    stats->photons_requested = in.Nphoton;
    stats->photons_done = (int64_t)hc.done_photons;
    stats->steps = (int64_t)hc.steps;
    stats->scatters = (int64_t)hc.scatters;
    stats->loss = (int64_t)c[kJcLoss];
    stats->capped = (int64_t)c[kJcCapped];
    stats->roulette_kills = (int64_t)c[kJcRoulette];
    stats->seed_used = hj.seed;
    stats->ledger[kLgLaunched] = (double)hc.done_photons;
    stats->ledger[kLgRouletteKill] = L[kLgRouletteKill];
    stats->ledger[kLgRouletteGain] = L[kLgRouletteGain];
    stats->ledger[kLgLost] = L[kLgLost];
    stats->seconds_setup = std::chrono::duration<double>(t1 - t0).count();
    stats->seconds_kernel = std::chrono::duration<double>(t2 - t1).count();
    stats->seconds_total = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    stats->grid_blocks = per_sm * sms;
    stats->block_size = block;
  }
  return VMC_OK;
}
