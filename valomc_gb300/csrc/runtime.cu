// runtime.cu -- the C ABI of include/valomc_gb300.h: device selection, uploads, the
// persistent launch with host-side progress / cancel / timeout polling, read-back and
// normalisation, resident meshes, batched launches, autotuning and the roofline
// micro-benchmarks.  No CPU fallback: without an sm_103 device every call fails with
// VMC_ERR_NO_DEVICE.
#include <cuda_runtime.h>
#include <stdio.h>
#include <string.h>

#include <algorithm>
#include <chrono>
#include <cmath>
#include <memory>
#include <string>
#include <thread>
#include <vector>

#include "engine.hpp"

namespace vmc {

static thread_local std::string g_last_error;
// bytes copied between host and device by the calling thread (reported in vmc_stats)
thread_local int64_t g_h2d_bytes = 0, g_d2h_bytes = 0;

void set_error(const std::string &msg) { g_last_error = msg; }

int cuda_status(cudaError_t e, const char *what) {
  set_error(std::string(what) + ": " + cudaGetErrorString(e));
  cudaGetLastError();  // clear a sticky launch error from this thread's view
  if (e == cudaErrorMemoryAllocation) return VMC_ERR_OUT_OF_MEMORY;
  if (e == cudaErrorNoDevice || e == cudaErrorInsufficientDriver || e == cudaErrorNoKernelImageForDevice)
    return VMC_ERR_NO_DEVICE;
  return VMC_ERR_CUDA;
}

int select_device(int device, int *num_sms) {
  int n = 0;
  cudaError_t e = cudaGetDeviceCount(&n);
  if (e != cudaSuccess || n == 0) {
    set_error("no CUDA device visible");
    cudaGetLastError();
    return VMC_ERR_NO_DEVICE;
  }
  if (device < 0 || device >= n) {
    set_error("device ordinal out of range");
    return VMC_ERR_INVALID_ARGUMENT;
  }
  VMC_CK(cudaSetDevice(device));
  int major = 0, minor = 0, sms = 0;
  VMC_CK(cudaDeviceGetAttribute(&major, cudaDevAttrComputeCapabilityMajor, device));
  VMC_CK(cudaDeviceGetAttribute(&minor, cudaDevAttrComputeCapabilityMinor, device));
  VMC_CK(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device));
  if (major != 10 || minor != 3) {
    char buf[128];
    snprintf(buf, sizeof buf, "device %d is sm_%d%d; this library is built for sm_103a only", device, major, minor);
    set_error(buf);
    return VMC_ERR_NO_DEVICE;
  }
  if (num_sms) *num_sms = sms;
  return VMC_OK;
}

uint64_t clock_seed() {
  // the reference seeds from the high-resolution clock when no seed is given
  // (cpp/3d/MC3Dmex.cpp:170-175)
  return (uint64_t)std::chrono::high_resolution_clock::now().time_since_epoch().count();
}

template <class T>
static int dalloc(T **p, size_t count, int64_t &bytes) {
  *p = nullptr;
  if (count == 0) count = 1;
  VMC_CK(cudaMalloc(reinterpret_cast<void **>(p), count * sizeof(T)));
  bytes += (int64_t)(count * sizeof(T));
  return VMC_OK;
}

// from a memory pool, ordered on stream st (pool == nullptr: plain cudaMalloc)
template <class T>
static int dalloc(T **p, size_t count, int64_t &bytes, cudaMemPool_t pool, cudaStream_t st) {
  if (!pool) return dalloc(p, count, bytes);
  *p = nullptr;
  if (count == 0) count = 1;
  VMC_CK(cudaMallocFromPoolAsync(reinterpret_cast<void **>(p), count * sizeof(T), pool, st));
  bytes += (int64_t)(count * sizeof(T));
  return VMC_OK;
}

template <class T>
static int h2d(T *d, const T *h, size_t count, cudaStream_t st) {
  if (count) VMC_CK(cudaMemcpyAsync(d, h, count * sizeof(T), cudaMemcpyHostToDevice, st));
  g_h2d_bytes += (int64_t)(count * sizeof(T));
  return VMC_OK;
}

#define VMC_TRY(x)            \
  do {                        \
    int _s = (x);             \
    if (_s != VMC_OK) return _s; \
  } while (0)

// ---------------------------------------------------------------------------------------
// meshes and jobs
// ---------------------------------------------------------------------------------------

DeviceMesh::~DeviceMesh() {
  void *ps[] = {d_geom[0], d_geom[1], d_bnorm};
  for (void *p : ps)
    if (p) {
      if (pool) cudaFreeAsync(p, st);
      else cudaFree(p);
    }
}

int upload_mesh(DeviceMesh &m, int precision_mask) {
  const HostMesh &h = m.host;
  m.dim = h.dim;
  cudaStream_t st = m.st;
  if ((precision_mask & 1) && !m.d_geom[VMC_FP64]) {
    if (h.dim == 3) {
      Tet64 *d;
      VMC_TRY(dalloc(&d, h.tet64.size(), m.bytes, m.pool, st));
      m.d_geom[VMC_FP64] = d;
      VMC_TRY(h2d(d, h.tet64.data(), h.tet64.size(), st));
    } else {
      Tri64 *d;
      VMC_TRY(dalloc(&d, h.tri64.size(), m.bytes, m.pool, st));
      m.d_geom[VMC_FP64] = d;
      VMC_TRY(h2d(d, h.tri64.data(), h.tri64.size(), st));
    }
  }
  if ((precision_mask & 2) && !m.d_geom[VMC_FP32]) {
    if (h.dim == 3) {
      Tet32 *d;
      VMC_TRY(dalloc(&d, h.tet32.size(), m.bytes, m.pool, st));
      m.d_geom[VMC_FP32] = d;
      VMC_TRY(h2d(d, h.tet32.data(), h.tet32.size(), st));
    } else {
      Tri32 *d;
      VMC_TRY(dalloc(&d, h.tri32.size(), m.bytes, m.pool, st));
      m.d_geom[VMC_FP32] = d;
      VMC_TRY(h2d(d, h.tri32.data(), h.tri32.size(), st));
    }
  }
  if (!m.d_bnorm) {
    VMC_TRY(dalloc(&m.d_bnorm, h.bnorm.size(), m.bytes, m.pool, st));
    VMC_TRY(h2d(m.d_bnorm, h.bnorm.data(), h.bnorm.size(), st));
  }
  VMC_CK(cudaStreamSynchronize(st));
  return VMC_OK;
}

JobBuffers::~JobBuffers() { release(); }

void JobBuffers::release() {
  void *ps[] = {d_optics, d_bctype, d_bcn, d_cdf, d_src, d_cdf_f, d_src_f, d_acc, d_jc, d_ledger,
                d_tape, d_tape_off, d_trace, d_trace_len};
  for (void *p : ps)
    if (p) {
      if (pool) cudaFreeAsync(p, free_stream);
      else cudaFree(p);
    }
  d_optics = nullptr; d_bctype = nullptr; d_bcn = d_cdf = nullptr; d_src = nullptr; d_acc = nullptr;
  d_cdf_f = nullptr; d_src_f = nullptr;
  d_jc = nullptr; d_ledger = nullptr; d_tape = nullptr; d_tape_off = d_trace = d_trace_len = nullptr;
  bytes = 0;
}

int64_t job_footprint(const HostJob &j, const HostMesh &m) {
  const int64_t rows = j.homogeneous ? 1 : m.Ne;
  return rows * 32 + m.Nb * 9 + (int64_t)j.src.size() * (int64_t)(sizeof(SourceRec) + sizeof(SourceRecF) + 12) +
         (2 * m.Ne + 4 * m.Nb) * 8 + kSlots * (kJcN + kLgN) * 8;
}

int upload_job(const HostJob &j, const DeviceMesh &m, int precision, JobBuffers &b, cudaStream_t st) {
  const int64_t Ne = m.host.Ne, Nb = m.host.Nb;
  b.Ne = Ne; b.Nb = Nb;
  const size_t rows = j.homogeneous ? 1 : (size_t)Ne;
  if (precision == VMC_FP64) {
    double *d;
    VMC_TRY(dalloc(&d, rows * 4, b.bytes, b.pool, st));
    b.d_optics = d;
    VMC_TRY(h2d(d, j.optics.data(), rows * 4, st));
  } else {
    std::vector<float> f(rows * 4);
    for (size_t i = 0; i < rows * 4; i++) f[i] = (float)j.optics[i];
    float *d;
    VMC_TRY(dalloc(&d, rows * 4, b.bytes, b.pool, st));
    b.d_optics = d;
    VMC_TRY(h2d(d, f.data(), rows * 4, st));
    VMC_CK(cudaStreamSynchronize(st));  // f is a temporary
  }
  VMC_TRY(dalloc(&b.d_bctype, (size_t)Nb, b.bytes, b.pool, st));
  VMC_TRY(h2d(b.d_bctype, j.bctype.data(), (size_t)Nb, st));
  VMC_TRY(dalloc(&b.d_bcn, (size_t)Nb, b.bytes, b.pool, st));
  VMC_TRY(h2d(b.d_bcn, j.bcn.data(), (size_t)Nb, st));
  VMC_TRY(dalloc(&b.d_cdf, j.cdf.size(), b.bytes, b.pool, st));
  VMC_TRY(h2d(b.d_cdf, j.cdf.data(), j.cdf.size(), st));
  VMC_TRY(dalloc(&b.d_src, j.src.size(), b.bytes, b.pool, st));
  VMC_TRY(h2d(b.d_src, j.src.data(), j.src.size(), st));
  VMC_TRY(dalloc(&b.d_cdf_f, j.cdf_f.size(), b.bytes, b.pool, st));
  VMC_TRY(h2d(b.d_cdf_f, j.cdf_f.data(), j.cdf_f.size(), st));
  VMC_TRY(dalloc(&b.d_src_f, j.src_f.size(), b.bytes, b.pool, st));
  VMC_TRY(h2d(b.d_src_f, j.src_f.data(), j.src_f.size(), st));
  VMC_TRY(dalloc(&b.d_acc, (size_t)(2 * Ne + 4 * Nb), b.bytes, b.pool, st));
  VMC_TRY(dalloc(&b.d_jc, (size_t)kSlots * kJcN, b.bytes, b.pool, st));
  VMC_TRY(dalloc(&b.d_ledger, (size_t)kSlots * kLgN, b.bytes, b.pool, st));
  return zero_job(b, st);
}

int zero_job(JobBuffers &b, cudaStream_t st) {
  VMC_CK(cudaMemsetAsync(b.d_acc, 0, sizeof(double) * (size_t)(2 * b.Ne + 4 * b.Nb), st));
  VMC_CK(cudaMemsetAsync(b.d_jc, 0, sizeof(unsigned long long) * kSlots * kJcN, st));
  VMC_CK(cudaMemsetAsync(b.d_ledger, 0, sizeof(double) * kSlots * kLgN, st));
  return VMC_OK;
}

JobDev describe_job(const HostJob &j, const DeviceMesh &m, int precision, const JobBuffers &b) {
  JobDev d;
  memset(&d, 0, sizeof(d));
  const int64_t Ne = m.host.Ne, Nb = m.host.Nb;
  d.geom = m.geom(precision);
  d.optics = b.d_optics;
  d.opt_mask = j.homogeneous ? 0 : -1;
  d.Ns = (int32_t)j.src.size();
  d.Ne = (int32_t)Ne;
  d.Nb = (int32_t)Nb;
  d.cdf = b.d_cdf;
  d.src = b.d_src;
  d.cdf_f = b.d_cdf_f;
  d.src_f = b.d_src_f;
  d.bctype = b.d_bctype;
  d.bcn = b.d_bcn;
  d.bnorm = m.d_bnorm;
  d.omega = j.omega;
  d.k_scale = j.k_scale;
  d.k_scale_f = (float)j.k_scale;
  d.phase0 = j.phase0;
  d.seed = j.seed;
  d.ER = b.d_acc;
  d.EI = b.d_acc + Ne;
  d.EBR = b.d_acc + 2 * Ne;
  d.EBI = b.d_acc + 2 * Ne + Nb;
  d.DEBR = b.d_acc + 2 * Ne + 2 * Nb;
  d.DEBI = b.d_acc + 2 * Ne + 3 * Nb;
  d.jc = b.d_jc;
  d.ledger = b.d_ledger;
  return d;
}

const void *select_kernel(const LaunchSpec &s, bool one, bool tab) {
  // The one-job form is used for the FP32 walks only: for the FP64 walks it measured 2.3x
  // slower per element step than the per-job form on the 648k-tet phantom (same
  // trajectories, same registers), so they keep the descriptor and keys in global memory.
  one = one && !s.tape && s.precision == VMC_FP32;
  tab = tab && !one;
  if (s.dim == 3)
    return s.precision == VMC_FP64 ? kernel_3d64(s.fd, s.tape, one, tab) : kernel_3d32(s.fd, s.tape, one, tab);
  return s.precision == VMC_FP64 ? kernel_2d64(s.fd, s.tape, one, tab) : kernel_2d32(s.fd, s.tape, one, tab);
}

// The SM's unified L1 / shared-memory array is split per launch.  Left to itself the driver
// gave the pool kernels more shared memory than they use, at the cost of L1, where each
// step's element record is re-read after a scatter; preferring the smallest split that
// still holds every resident CTA's static and dynamic shared memory (plus the 1 KiB the
// hardware reserves per CTA) was 2.3% faster on the 648k-tet phantom and 1.8% on the
// serving mix, and changed nothing on meshes staged whole in shared memory.  The occupancy
// is taken at the driver's default split (reset_carveout) and the split fitted after it.
void reset_carveout(const void *fn) {
  cudaFuncSetAttribute(fn, cudaFuncAttributePreferredSharedMemoryCarveout, -1);
  cudaGetLastError();  // a hint: a refusal leaves the default split
}

void fit_carveout(const void *fn, int device, int per_sm, size_t dyn_smem) {
  cudaFuncAttributes fa;
  int smem_sm = 0;
  if (cudaFuncGetAttributes(&fa, fn) == cudaSuccess &&
      cudaDeviceGetAttribute(&smem_sm, cudaDevAttrMaxSharedMemoryPerMultiprocessor, device) == cudaSuccess &&
      smem_sm > 0) {
    const double need = (double)per_sm * (double)(fa.sharedSizeBytes + dyn_smem + 1024);
    const int pct = std::min(100, (int)std::ceil(100.0 * need / smem_sm) + 1);
    cudaFuncSetAttribute(fn, cudaFuncAttributePreferredSharedMemoryCarveout, pct);
  }
  cudaGetLastError();
}

void set_single_job(LaunchParams &lp, const JobDev &job) {
  lp.job0 = job;
  // Philox4x32-10 key schedule: round r uses key + r * (0x9E3779B9, 0xBB67AE85) mod 2^32
  uint32_t a = (uint32_t)job.seed, b = (uint32_t)(job.seed >> 32);
  for (int r = 0; r < 10; r++) {
    lp.rk[2 * r] = a;
    lp.rk[2 * r + 1] = b;
    a += 0x9E3779B9u;
    b += 0xBB67AE85u;
  }
}

// ---------------------------------------------------------------------------------------
// launch
// ---------------------------------------------------------------------------------------

namespace {
struct StreamGuard {
  cudaStream_t s = nullptr;
  ~StreamGuard() {
    if (s) cudaStreamDestroy(s);
  }
};
struct EventGuard {
  cudaEvent_t e = nullptr;
  ~EventGuard() {
    if (e) cudaEventDestroy(e);
  }
};
// device scratch of one launch: allocated and freed in order on the launch's stream
template <class T>
struct DevGuard {
  T *p = nullptr;
  cudaStream_t st = nullptr;
  int alloc(size_t count, cudaStream_t s) {
    st = s;
    VMC_CK(cudaMallocAsync(reinterpret_cast<void **>(&p), (count ? count : 1) * sizeof(T), s));
    return VMC_OK;
  }
  ~DevGuard() {
    if (p) cudaFreeAsync(p, st);
  }
};
struct PinnedGuard {
  void *p = nullptr;
  ~PinnedGuard() {
    if (p) cudaFreeHost(p);
  }
};

// instantiated launch graphs of this thread, by kernel and launch shape
struct GraphSlot {
  const void *fn = nullptr;
  int grid = 0, block = 0;
  cudaGraphExec_t exec = nullptr;
};
GraphSlot &graph_slot(const void *fn, int grid, int block) {
  static thread_local GraphSlot slots[16];
  static thread_local int next_evict = 0;
  for (auto &s : slots)
    if (s.fn == fn && s.grid == grid && s.block == block) return s;
  for (auto &s : slots)
    if (!s.fn) {
      s.fn = fn; s.grid = grid; s.block = block;
      return s;
    }
  GraphSlot &s = slots[next_evict];
  next_evict = (next_evict + 1) % 16;
  if (s.exec) cudaGraphExecDestroy(s.exec);
  s = GraphSlot{fn, grid, block, nullptr};
  return s;
}
}  // namespace

namespace {
// What one launch needs before any buffer exists: the kernel, the grid, the job table with
// its photon prefix.
struct LaunchPlan {
  const void *fn = nullptr;
  bool one = false, tab = false;
  int grid = 0, block = 0, stage_slots = 0, dense = 0;
  size_t smem = 0;
  int64_t total = 0;
  std::vector<JobDev> jobs;
  std::vector<int64_t> begin;
};

int plan_launch(int device, const LaunchSpec &spec, const std::vector<JobDev> &jobs_in, LaunchPlan &p,
                LaunchResult &res) {
  int sms = 0;
  VMC_TRY(select_device(device, &sms));
  // the one-job kernels: FP32 walks on Philox streams (descriptor and keys as parameters);
  // the others copy a job table of up to kSmemJobs entries into each CTA's shared memory,
  // unless the launch stages deposits in a hashed shared-memory table (a single job on the
  // replay tape), which starts at the same place
  p.one = jobs_in.size() == 1 && !spec.tape && spec.precision == VMC_FP32;
  const bool staged = spec.stage_slots > 0 && spec.dim == 3 && spec.precision == VMC_FP32 && !spec.fd &&
                      jobs_in.size() == 1;
  p.tab = !p.one && !staged && jobs_in.size() <= (size_t)kSmemJobs;
  p.fn = select_kernel(spec, p.one, p.tab);
  if (!p.fn) { set_error("no kernel for this configuration"); return VMC_ERR_INVALID_ARGUMENT; }
  reset_carveout(p.fn);
  p.jobs = jobs_in;
  p.begin.assign(p.jobs.size() + 1, 0);
  for (size_t i = 0; i < p.jobs.size(); i++) {
    p.jobs[i].pbegin = p.begin[i];
    p.begin[i + 1] = p.begin[i] + p.jobs[i].pcount;
  }
  p.total = p.begin.back();
  res = LaunchResult();
  p.block = spec.block > 0 ? spec.block : 256;
  if (p.block % 32 || p.block > 256) { set_error("block size must be a multiple of 32, at most 256"); return VMC_ERR_INVALID_ARGUMENT; }
  int per_sm = 0;
  // shared-memory staging of deposits: FP32 tetrahedral walk, continuous wave, one job
  p.stage_slots = 0;
  if (staged) {
    p.stage_slots = 1;
    while (p.stage_slots < spec.stage_slots && p.stage_slots < 4096) p.stage_slots <<= 1;
  }
  p.smem = (size_t)p.stage_slots * (sizeof(double) + sizeof(int32_t));
  if (p.tab) p.smem = p.jobs.size() * sizeof(JobDev) + (p.jobs.size() + 1) * sizeof(int64_t);
  VMC_CK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, p.fn, p.block, p.smem));
  if (per_sm < 1) { set_error("kernel does not fit on an SM at this block size"); return VMC_ERR_INVALID_ARGUMENT; }
  // A one-job launch on a small mesh, without the hashed stage: every CTA keeps the whole
  // accumulator set (2 Ne + 4 Nb doubles) in shared memory, when that costs no resident
  // CTA, and adds it to the job's accumulators once at its end (stage_slots < 0: off).
  p.dense = 0;
  if (spec.stage_slots >= 0 && p.stage_slots == 0 && p.one) {
    JobDev &j = p.jobs[0];
    const int64_t Ne = j.Ne, Nb = j.Nb, n = 2 * Ne + 4 * Nb;
    const bool packed = j.EI == j.ER + Ne && j.EBR == j.ER + 2 * Ne && j.EBI == j.EBR + Nb &&
                        j.DEBR == j.EBR + 2 * Nb && j.DEBI == j.EBR + 3 * Nb;
    if (packed && n > 0 && n * (int64_t)sizeof(double) <= kDenseStageBytes) {
      int per_sm_dense = 0;
      VMC_CK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm_dense, p.fn, p.block, (size_t)n * sizeof(double)));
      const int want = spec.blocks_per_sm > 0 ? std::min(per_sm, spec.blocks_per_sm) : per_sm;
      if (per_sm_dense >= want) {
        p.dense = (int)n;
        j.dense = (int32_t)n;
        p.smem = (size_t)n * sizeof(double);
        per_sm = per_sm_dense;
      }
    }
  }
  if (spec.blocks_per_sm > 0) per_sm = std::min(per_sm, spec.blocks_per_sm);
  p.grid = per_sm * sms;
  fit_carveout(p.fn, device, per_sm, p.smem);
  res.grid = p.grid;
  res.block = p.block;
  return VMC_OK;
}

LaunchParams make_params(const LaunchSpec &spec, const LaunchPlan &p, const JobDev *djobs, const int64_t *dbegin,
                         Ctl *dctl) {
  LaunchParams lp{};
  lp.jobs = djobs;
  if (p.one) set_single_job(lp, p.jobs[0]);
  lp.job_begin = dbegin;
  lp.njobs = (int32_t)p.jobs.size();
  lp.chunk = spec.chunk > 0 ? spec.chunk : 32;
  lp.total = p.total;
  lp.max_steps = spec.max_steps > 0 ? spec.max_steps : 10000000;
  lp.ctl = dctl;
  lp.stage_slots = p.stage_slots;
  lp.dense = p.dense;
  lp.refill_min = spec.refill > 0 ? spec.refill : kDefaultRefill;
  return lp;
}

// Records the control-block reset and the kernel as a graph on `cap` and updates `exec` in
// place when it holds a graph of the same shape (else instantiates it anew).
int capture_launch(cudaStream_t cap, const LaunchPlan &p, void **args, Ctl *dctl, cudaGraphExec_t &exec) {
  VMC_CK(cudaStreamBeginCapture(cap, cudaStreamCaptureModeThreadLocal));
  cudaError_t ce = cudaMemsetAsync(dctl, 0, sizeof(Ctl), cap);
  if (ce == cudaSuccess) ce = cudaLaunchKernel(p.fn, dim3(p.grid), dim3(p.block), args, p.smem, cap);
  cudaGraph_t graph = nullptr;
  cudaError_t ee = cudaStreamEndCapture(cap, &graph);
  if (ce != cudaSuccess) { if (graph) cudaGraphDestroy(graph); return cuda_status(ce, "graph capture"); }
  if (ee != cudaSuccess) return cuda_status(ee, "cudaStreamEndCapture");
  bool updated = false;
  if (exec) {
    cudaGraphExecUpdateResultInfo info;
    updated = cudaGraphExecUpdate(exec, graph, &info) == cudaSuccess;
    if (!updated) {
      cudaGetLastError();
      cudaGraphExecDestroy(exec);
      exec = nullptr;
    }
  }
  if (!updated) {
    cudaError_t ie = cudaGraphInstantiate(&exec, graph, 0);
    if (ie != cudaSuccess) { cudaGraphDestroy(graph); exec = nullptr; return cuda_status(ie, "cudaGraphInstantiate"); }
  }
  cudaGraphDestroy(graph);
  return VMC_OK;
}
}  // namespace

int launch_jobs(int device, const LaunchSpec &spec, const std::vector<JobDev> &jobs_in, const vmc_options *opt,
                cudaStream_t st, LaunchResult &res) {
  LaunchPlan plan;
  VMC_TRY(plan_launch(device, spec, jobs_in, plan, res));
  const std::vector<JobDev> &jobs = plan.jobs;
  const std::vector<int64_t> &begin = plan.begin;
  const int64_t total = plan.total;
  const void *fn = plan.fn;
  const int grid = plan.grid, block = plan.block;
  const size_t smem = plan.smem;
  if (total == 0) return VMC_OK;

  DevGuard<JobDev> djobs;
  DevGuard<int64_t> dbegin;
  DevGuard<Ctl> dctl;
  VMC_TRY(djobs.alloc(jobs.size(), st));
  VMC_TRY(dbegin.alloc(begin.size(), st));
  VMC_TRY(dctl.alloc(1, st));
  VMC_TRY(h2d(djobs.p, jobs.data(), jobs.size(), st));
  VMC_TRY(h2d(dbegin.p, begin.data(), begin.size(), st));
  VMC_CK(cudaMemsetAsync(dctl.p, 0, sizeof(Ctl), st));
  LaunchParams lp = make_params(spec, plan, djobs.p, dbegin.p, dctl.p);
  EventGuard e0, e1;
  VMC_CK(cudaEventCreate(&e0.e));
  VMC_CK(cudaEventCreate(&e1.e));
  void *args[] = {&lp};
  StreamGuard gstream;
  if (!spec.graph) {
    VMC_CK(cudaEventRecord(e0.e, st));
    VMC_CK(cudaLaunchKernel(fn, dim3(grid), dim3(block), args, smem, st));
    VMC_CK(cudaEventRecord(e1.e, st));
  } else {
    // The control-block reset and the persistent kernel are recorded as a CUDA graph on a
    // capture stream ordered after `st`; a graph of the same shape launched before on this
    // thread is updated in place (cudaGraphExecUpdate) instead of instantiated again.
    VMC_CK(cudaStreamCreateWithFlags(&gstream.s, cudaStreamNonBlocking));
    VMC_CK(cudaEventRecord(e0.e, st));
    VMC_CK(cudaStreamWaitEvent(gstream.s, e0.e, 0));
    GraphSlot &slot = graph_slot(fn, grid, block);
    VMC_TRY(capture_launch(gstream.s, plan, args, dctl.p, slot.exec));
    VMC_CK(cudaEventRecord(e0.e, gstream.s));
    VMC_CK(cudaGraphLaunch(slot.exec, gstream.s));
    VMC_CK(cudaEventRecord(e1.e, gstream.s));
    VMC_CK(cudaStreamWaitEvent(st, e1.e, 0));
  }

  const bool poll = opt && (opt->progress || opt->cancel || opt->timeout_s > 0);
  int status = VMC_OK;
  if (poll) {
    // The host thread watches the run: progress from the fetch counter, cancellation and
    // the timeout set the device cancel flag, which the kernel reads every 1024 steps.
    StreamGuard side;
    VMC_CK(cudaStreamCreateWithFlags(&side.s, cudaStreamNonBlocking));
    PinnedGuard pin;
    VMC_CK(cudaMallocHost(&pin.p, 64));
    unsigned long long *h_next = reinterpret_cast<unsigned long long *>(pin.p);
    int32_t *h_one = reinterpret_cast<int32_t *>(reinterpret_cast<char *>(pin.p) + 32);
    *h_one = 1;
    auto t0 = std::chrono::steady_clock::now();
    auto last = t0;
    bool cancel_sent = false;
    for (;;) {
      cudaError_t q = cudaEventQuery(e1.e);
      if (q == cudaSuccess) break;
      if (q != cudaErrorNotReady) return cuda_status(q, "cudaEventQuery");
      std::this_thread::sleep_for(std::chrono::microseconds(200));
      auto now = std::chrono::steady_clock::now();
      double el = std::chrono::duration<double>(now - t0).count();
      bool stop = false;
      if (opt->cancel && *opt->cancel) { stop = true; if (status == VMC_OK) status = VMC_ERR_CANCELLED; }
      if (opt->timeout_s > 0 && el > opt->timeout_s) { stop = true; if (status == VMC_OK) status = VMC_ERR_TIMEOUT; }
      if (opt->progress && std::chrono::duration<double>(now - last).count() > 0.1 && !cancel_sent) {
        last = now;
        VMC_CK(cudaMemcpyAsync(h_next, &dctl.p->next_photon, 8, cudaMemcpyDeviceToHost, side.s));
        VMC_CK(cudaStreamSynchronize(side.s));
        double pct = 100.0 * (double)std::min<unsigned long long>(*h_next, (unsigned long long)total) / (double)total;
        if (!opt->progress(pct, opt->progress_user)) { stop = true; if (status == VMC_OK) status = VMC_ERR_CANCELLED; }
      }
      if (stop && !cancel_sent) {
        VMC_CK(cudaMemcpyAsync(&dctl.p->cancel, h_one, 4, cudaMemcpyHostToDevice, side.s));
        VMC_CK(cudaStreamSynchronize(side.s));
        cancel_sent = true;
      }
    }
  }
  VMC_CK(cudaEventSynchronize(e1.e));
  VMC_CK(cudaGetLastError());
  float ms = 0;
  VMC_CK(cudaEventElapsedTime(&ms, e0.e, e1.e));
  Ctl h;
  VMC_CK(cudaMemcpyAsync(&h, dctl.p, sizeof(Ctl), cudaMemcpyDeviceToHost, st));
  VMC_CK(cudaStreamSynchronize(st));
  g_d2h_bytes += (int64_t)sizeof(Ctl);
  res.steps = h.steps;
  res.scatters = h.scatters;
  res.done = h.done_photons;
  res.kernel_ms = ms;
  if (opt && opt->progress && status == VMC_OK) opt->progress(100.0, opt->progress_user);
  return status;
}

LaunchArena::~LaunchArena() {
  if (djobs) cudaFree(djobs);
  if (dbegin) cudaFree(dbegin);
  if (dctl) cudaFree(dctl);
  if (hjobs) cudaFreeHost(hjobs);
  if (hbegin) cudaFreeHost(hbegin);
  if (hctl) cudaFreeHost(hctl);
  if (e0) cudaEventDestroy(e0);
  if (e1) cudaEventDestroy(e1);
  if (exec) cudaGraphExecDestroy(exec);
  if (cap_stream) cudaStreamDestroy(cap_stream);
}

int launch_start(int device, const LaunchSpec &spec, const std::vector<JobDev> &jobs_in, LaunchArena &a,
                 cudaStream_t st, LaunchResult &res) {
  if (a.pending) { set_error("arena has a launch in flight"); return VMC_ERR_INVALID_ARGUMENT; }
  LaunchPlan plan;
  VMC_TRY(plan_launch(device, spec, jobs_in, plan, res));
  a.total = plan.total;
  if (plan.total == 0) return VMC_OK;
  const size_t nj = plan.jobs.size();
  if (nj > a.cap_jobs) {
    // grow the job table (device and pinned staging) to the next power of two
    size_t cap = 16;
    while (cap < nj) cap <<= 1;
    if (a.djobs) { cudaFree(a.djobs); a.djobs = nullptr; }
    if (a.dbegin) { cudaFree(a.dbegin); a.dbegin = nullptr; }
    if (a.hjobs) { cudaFreeHost(a.hjobs); a.hjobs = nullptr; }
    if (a.hbegin) { cudaFreeHost(a.hbegin); a.hbegin = nullptr; }
    a.cap_jobs = 0;
    int64_t bytes = 0;
    VMC_TRY(dalloc(&a.djobs, cap, bytes));
    VMC_TRY(dalloc(&a.dbegin, cap + 1, bytes));
    VMC_CK(cudaMallocHost(reinterpret_cast<void **>(&a.hjobs), cap * sizeof(JobDev)));
    VMC_CK(cudaMallocHost(reinterpret_cast<void **>(&a.hbegin), (cap + 1) * sizeof(int64_t)));
    a.cap_jobs = cap;
  }
  if (!a.dctl) {
    int64_t bytes = 0;
    VMC_TRY(dalloc(&a.dctl, 1, bytes));
    VMC_CK(cudaMallocHost(reinterpret_cast<void **>(&a.hctl), sizeof(Ctl)));
    VMC_CK(cudaEventCreate(&a.e0));
    VMC_CK(cudaEventCreate(&a.e1));
  }
  // the pinned staging is free: the previous launch of this arena has finished
  memcpy(a.hjobs, plan.jobs.data(), nj * sizeof(JobDev));
  memcpy(a.hbegin, plan.begin.data(), (nj + 1) * sizeof(int64_t));
  VMC_TRY(h2d(a.djobs, a.hjobs, nj, st));
  VMC_TRY(h2d(a.dbegin, a.hbegin, nj + 1, st));
  LaunchParams lp = make_params(spec, plan, a.djobs, a.dbegin, a.dctl);
  void *args[] = {&lp};
  if (!spec.graph) {
    VMC_CK(cudaMemsetAsync(a.dctl, 0, sizeof(Ctl), st));
    VMC_CK(cudaEventRecord(a.e0, st));
    VMC_CK(cudaLaunchKernel(plan.fn, dim3(plan.grid), dim3(plan.block), args, plan.smem, st));
    VMC_CK(cudaEventRecord(a.e1, st));
  } else {
    // the arena's own graph: it is never updated while one of its launches is in flight
    if (!a.cap_stream) VMC_CK(cudaStreamCreateWithFlags(&a.cap_stream, cudaStreamNonBlocking));
    VMC_TRY(capture_launch(a.cap_stream, plan, args, a.dctl, a.exec));
    VMC_CK(cudaEventRecord(a.e0, st));
    VMC_CK(cudaGraphLaunch(a.exec, st));
    VMC_CK(cudaEventRecord(a.e1, st));
  }
  a.pending = true;
  return VMC_OK;
}

int launch_finish(LaunchArena &a, cudaStream_t st, LaunchResult &res) {
  if (!a.pending) return VMC_OK;
  a.pending = false;
  VMC_CK(cudaEventSynchronize(a.e1));
  VMC_CK(cudaGetLastError());
  float ms = 0;
  VMC_CK(cudaEventElapsedTime(&ms, a.e0, a.e1));
  VMC_CK(cudaMemcpyAsync(a.hctl, a.dctl, sizeof(Ctl), cudaMemcpyDeviceToHost, st));
  VMC_CK(cudaStreamSynchronize(st));
  g_d2h_bytes += (int64_t)sizeof(Ctl);
  res.steps = a.hctl->steps;
  res.scatters = a.hctl->scatters;
  res.done = a.hctl->done_photons;
  res.kernel_ms = ms;
  return VMC_OK;
}

int collect_job(const HostJob &j, const DeviceMesh &m, const JobBuffers &b, int64_t nphoton, bool normalize,
                vmc_output *out, vmc_stats *st, cudaStream_t stream) {
  const int64_t Ne = m.host.Ne, Nb = m.host.Nb;
  std::vector<double> acc((size_t)(2 * Ne + 4 * Nb));
  std::vector<unsigned long long> jc((size_t)kSlots * kJcN);
  std::vector<double> lg((size_t)kSlots * kLgN);
  VMC_CK(cudaMemcpyAsync(acc.data(), b.d_acc, acc.size() * 8, cudaMemcpyDeviceToHost, stream));
  VMC_CK(cudaMemcpyAsync(jc.data(), b.d_jc, jc.size() * 8, cudaMemcpyDeviceToHost, stream));
  VMC_CK(cudaMemcpyAsync(lg.data(), b.d_ledger, lg.size() * 8, cudaMemcpyDeviceToHost, stream));
  VMC_CK(cudaStreamSynchronize(stream));
  g_d2h_bytes += (int64_t)(acc.size() + jc.size() + lg.size()) * 8;
  const double *ER = acc.data(), *EI = ER + Ne, *EBR = EI + Ne, *EBI = EBR + Nb, *DEBR = EBI + Nb, *DEBI = DEBR + Nb;
  if (out) normalise(m.host, j, nphoton, ER, EI, EBR, EBI, DEBR, DEBI, out, normalize);
  if (st) {
    unsigned long long c[kJcN] = {0};
    double L[kLgN] = {0};
    for (int s = 0; s < kSlots; s++) {
      for (int k = 0; k < kJcN; k++) c[k] += jc[(size_t)s * kJcN + k];
      for (int k = 0; k < kLgN; k++) L[k] += lg[(size_t)s * kLgN + k];
    }
    if (st->steps == 0) st->steps = (int64_t)c[kJcSteps];  // batched and served jobs
    st->loss = (int64_t)c[kJcLoss];
    st->capped = (int64_t)c[kJcCapped];
    st->roulette_kills = (int64_t)c[kJcRoulette];
    if (c[kJcTapeEnd]) st->status_detail |= kErrTapeEnd;
    double absorbed = 0, exited = 0;
    if (j.omega <= 0.0) {
      for (int64_t i = 0; i < Ne; i++)
        if (j.mua[(size_t)i] > 0.0) absorbed += ER[i];
      for (int64_t i = 0; i < Nb; i++) exited += EBR[i];
    } else {
      absorbed = exited = NAN;
    }
    st->ledger[kLgLaunched] = (double)st->photons_done;
    st->ledger[kLgAbsorbed] = absorbed;
    st->ledger[kLgExited] = exited;
    st->ledger[kLgRouletteKill] = L[kLgRouletteKill];
    st->ledger[kLgRouletteGain] = L[kLgRouletteGain];
    st->ledger[kLgLost] = L[kLgLost];
  }
  if (out && out->HN) memcpy(out->HN, m.host.HN.data(), m.host.HN.size() * sizeof(int64_t));
  return VMC_OK;
}

}  // namespace vmc

using namespace vmc;

// =========================================================================================
// C ABI
// =========================================================================================

struct vmc_mesh {
  DeviceMesh m;
  int precision_mask = 0;
};

extern "C" {

int vmc_abi_version(void) { return VMC_ABI_VERSION; }

const char *vmc_status_string(int s) {
  if (const char *m = mcerror_string(s)) return m;
  switch (s) {
    case VMC_OK: return "ok";
    case VMC_ERR_INVALID_ARGUMENT: return "invalid argument";
    case VMC_ERR_CUDA: return "CUDA error";
    case VMC_ERR_NO_DEVICE: return "no sm_103 CUDA device";
    case VMC_ERR_OUT_OF_MEMORY: return "out of device memory";
    case VMC_ERR_CANCELLED: return "cancelled";
    case VMC_ERR_TIMEOUT: return "timeout";
    case VMC_ERR_TAPE: return "replay tape exhausted";
    case VMC_ERR_ADMISSION: return "request exceeds the memory budget";
    case VMC_ERR_NOT_FOUND: return "unknown id";
    case VMC_ERR_SIZE_LIMIT: return "size beyond the supported maximum";
    default: return "Undefined error";
  }
}

const char *vmc_last_error(void) { return g_last_error.c_str(); }

void vmc_default_options(vmc_options *opt) {
  memset(opt, 0, sizeof(*opt));
  opt->precision = VMC_FP32;
  opt->rng = VMC_RNG_PHILOX;
  opt->normalize = 1;
}

int vmc_build_neighbourhood(const vmc_input *in, int64_t *HN_out) {
  if (!in || !HN_out || (in->dim != 2 && in->dim != 3)) return VMC_ERR_INVALID_ARGUMENT;
  return build_neighbours(in->dim, in->Ne, in->Nb, in->Nr, in->H, in->BH, HN_out);
}

static int prepare_options(const vmc_options *in, vmc_options &o) {
  if (in) o = *in;
  else vmc_default_options(&o);
  if (o.precision != VMC_FP64 && o.precision != VMC_FP32) return VMC_ERR_INVALID_ARGUMENT;
  if (o.rng != VMC_RNG_PHILOX && o.rng != VMC_RNG_TAPE) return VMC_ERR_INVALID_ARGUMENT;
  if (o.rng == VMC_RNG_TAPE && (!o.tape || !o.tape_off)) return VMC_ERR_INVALID_ARGUMENT;
  if (o.trace_photons && (!o.trace || !o.trace_len || o.trace_stride <= 0)) return VMC_ERR_INVALID_ARGUMENT;
  return VMC_OK;
}

int vmc_run(const vmc_input *in, const vmc_options *opt_in, vmc_output *out, vmc_stats *stats) {
  auto t0 = std::chrono::steady_clock::now();
  g_h2d_bytes = g_d2h_bytes = 0;
  vmc_options o;
  int s = prepare_options(opt_in, o);
  if (s) return s;
  if (!in || !out) return VMC_ERR_INVALID_ARGUMENT;
  s = check_input(in);
  if (s) return s;
  vmc_stats local;
  vmc_stats *st = stats ? stats : &local;
  memset(st, 0, sizeof(*st));
  // one stream per call, so calls from several host threads overlap on the device; the
  // call's device memory is allocated and freed in order on it (it outlives both holders)
  StreamGuard call_stream;
  DeviceMesh dm;
  dm.device = o.device;
  const int mask = o.precision == VMC_FP64 ? 1 : 2;
  s = build_mesh(in, mask, dm.host);
  if (s) return s;
  HostJob hj;
  s = build_job(in, dm.host, hj);
  if (s) return s;
  hj.seed = in->seed_given ? in->seed : clock_seed();
  // photons simulated: a negative count runs none, as MonteCarlo's loop does, and is still
  // the divisor of the normalisation (the reference's -0.0 results)
  const int64_t nph = std::max<int64_t>(0, in->Nphoton);
  if (o.rng == VMC_RNG_TAPE && o.tape_photons < nph) return VMC_ERR_INVALID_ARGUMENT;
  // every host-side check of ErrorChecks / Init has passed: now the device
  s = select_device(o.device);
  if (s) return s;
  VMC_CK(cudaStreamCreateWithFlags(&call_stream.s, cudaStreamNonBlocking));
  cudaStream_t stream = call_stream.s;
  cudaMemPool_t call_pool = nullptr;
  VMC_CK(cudaDeviceGetDefaultMemPool(&call_pool, o.device));
  dm.pool = call_pool;
  dm.st = stream;
  s = upload_mesh(dm, mask);
  if (s) return s;
  JobBuffers jb;
  jb.pool = call_pool;
  jb.free_stream = stream;
  s = upload_job(hj, dm, o.precision, jb, stream);
  if (s) return s;
  JobDev d = describe_job(hj, dm, o.precision, jb);
  d.pcount = nph;
  d.poffset = o.photon_offset;
  d.stream = o.stream_id;
  if (o.rng == VMC_RNG_TAPE) {
    const int64_t nw = o.tape_off[nph];
    VMC_TRY(dalloc(&jb.d_tape, (size_t)nw, jb.bytes, jb.pool, stream));
    VMC_TRY(h2d(jb.d_tape, o.tape, (size_t)nw, stream));
    VMC_TRY(dalloc(&jb.d_tape_off, (size_t)nph + 1, jb.bytes, jb.pool, stream));
    VMC_TRY(h2d(jb.d_tape_off, o.tape_off, (size_t)nph + 1, stream));
    d.tape = jb.d_tape;
    d.tape_off = jb.d_tape_off;
  }
  const int64_t ntr = std::min<int64_t>(o.trace_photons, nph);
  if (ntr > 0) {
    VMC_TRY(dalloc(&jb.d_trace, (size_t)(ntr * o.trace_stride), jb.bytes, jb.pool, stream));
    VMC_TRY(dalloc(&jb.d_trace_len, (size_t)ntr, jb.bytes, jb.pool, stream));
    VMC_CK(cudaMemsetAsync(jb.d_trace_len, 0, sizeof(int64_t) * (size_t)ntr, stream));
    d.trace = jb.d_trace;
    d.trace_len = jb.d_trace_len;
    d.trace_stride = o.trace_stride;
    d.trace_photons = ntr;
    d.trace_on = 1;
  }
  auto t1 = std::chrono::steady_clock::now();
  LaunchSpec spec;
  spec.dim = in->dim;
  spec.precision = o.precision;
  spec.fd = hj.omega > 0.0;
  spec.tape = o.rng == VMC_RNG_TAPE;
  spec.block = o.block_size;
  spec.blocks_per_sm = o.blocks_per_sm;
  spec.chunk = o.fetch_chunk;
  spec.max_steps = o.max_steps;
  spec.graph = o.use_graph != 0;
  spec.stage_slots = o.stage_slots;
  spec.refill = o.refill_lanes;
  LaunchResult lr;
  int ls = launch_jobs(o.device, spec, std::vector<JobDev>{d}, &o, stream, lr);
  if (ls != VMC_OK && ls != VMC_ERR_CANCELLED && ls != VMC_ERR_TIMEOUT) return ls;
  st->photons_requested = in->Nphoton;
  st->photons_done = (int64_t)lr.done;
  st->steps = (int64_t)lr.steps;
  st->scatters = (int64_t)lr.scatters;
  st->seed_used = hj.seed;
  st->seconds_kernel = lr.kernel_ms * 1e-3;
  st->grid_blocks = lr.grid;
  st->block_size = lr.block;
  s = collect_job(hj, dm, jb, in->Nphoton, o.normalize != 0 || !opt_in, out, st, stream);
  if (s) return s;
  if (ntr > 0) {
    VMC_CK(cudaMemcpyAsync(o.trace, jb.d_trace, sizeof(int64_t) * (size_t)(ntr * o.trace_stride),
                           cudaMemcpyDeviceToHost, stream));
    VMC_CK(cudaMemcpyAsync(o.trace_len, jb.d_trace_len, sizeof(int64_t) * (size_t)ntr, cudaMemcpyDeviceToHost, stream));
    VMC_CK(cudaStreamSynchronize(stream));
  }
  auto t2 = std::chrono::steady_clock::now();
  st->seconds_setup = std::chrono::duration<double>(t1 - t0).count();
  st->seconds_total = std::chrono::duration<double>(t2 - t0).count();
  st->bytes_h2d = g_h2d_bytes;
  st->bytes_d2h = g_d2h_bytes + (ntr > 0 ? (int64_t)sizeof(int64_t) * ntr * (o.trace_stride + 1) : 0);
  if (ls != VMC_OK) return ls;
  if (st->status_detail & kErrTapeEnd) return VMC_ERR_TAPE;
  return VMC_OK;
}

// ---------------------------------------------------------------------------------------
// resident meshes and batches
// ---------------------------------------------------------------------------------------

int vmc_mesh_create(const vmc_input *geometry, int32_t precision, int32_t device, vmc_mesh **out) {
  if (!geometry || !out || (precision != VMC_FP64 && precision != VMC_FP32)) return VMC_ERR_INVALID_ARGUMENT;
  *out = nullptr;
  if ((geometry->Ne && !geometry->H) || (geometry->Nb && !geometry->BH) || (geometry->Nr && !geometry->r))
    return VMC_ERR_INVALID_ARGUMENT;
  const int64_t nh = geometry->Ne * (geometry->dim + 1), nb = geometry->Nb * geometry->dim;
  for (int64_t i = 0; i < nh; i++)
    if (geometry->H[i] < 0 || geometry->H[i] >= geometry->Nr) return VMC_INCONSISTENT_H;
  for (int64_t i = 0; i < nb; i++)
    if (geometry->BH[i] < 0 || geometry->BH[i] >= geometry->Nr) return VMC_INCONSISTENT_BH;
  int s = select_device(device);
  if (s) return s;
  std::unique_ptr<vmc_mesh> m(new vmc_mesh);
  m->m.device = device;
  const int mask = precision == VMC_FP64 ? 1 : 2;
  s = build_mesh(geometry, mask, m->m.host);
  if (s) return s;
  s = upload_mesh(m->m, mask);
  if (s) return s;
  m->precision_mask = mask;
  *out = m.release();
  return VMC_OK;
}

int vmc_mesh_destroy(vmc_mesh *mesh) {
  delete mesh;
  return VMC_OK;
}

int64_t vmc_mesh_device_bytes(const vmc_mesh *mesh) { return mesh ? mesh->m.bytes : 0; }

extern "C++" {
namespace vmc {
DeviceMesh *mesh_impl(vmc_mesh *m) { return m ? &m->m : nullptr; }
int mesh_precision_mask(const vmc_mesh *m) { return m ? m->precision_mask : 0; }
}  // namespace vmc
}

// jobs of one (dim, frequency-domain) class share a launch
int vmc_run_batch(vmc_mesh *const *meshes, const vmc_input *jobs, int32_t njobs, const vmc_options *opt_in,
                  vmc_output *outs, vmc_stats *stats, vmc_stats *job_stats) {
  auto t0 = std::chrono::steady_clock::now();
  g_h2d_bytes = g_d2h_bytes = 0;
  vmc_options o;
  int s = prepare_options(opt_in, o);
  if (s) return s;
  if (o.rng != VMC_RNG_PHILOX) return VMC_ERR_INVALID_ARGUMENT;
  if (!meshes || !jobs || njobs <= 0 || !outs) return VMC_ERR_INVALID_ARGUMENT;
  const int mask = o.precision == VMC_FP64 ? 1 : 2;
  // one stream per call; the jobs' buffers are allocated and freed in order on it, so it
  // is declared before them and outlives them
  StreamGuard call_stream;
  std::vector<HostJob> hj((size_t)njobs);
  std::vector<std::unique_ptr<JobBuffers>> jb((size_t)njobs);
  for (int i = 0; i < njobs; i++) {
    vmc_mesh *mm = meshes[i];
    if (!mm || !(mm->precision_mask & mask)) return VMC_ERR_INVALID_ARGUMENT;
    vmc_input in = jobs[i];
    // geometry comes from the mesh
    in.dim = mm->m.host.dim; in.Ne = mm->m.host.Ne; in.Nb = mm->m.host.Nb; in.Nr = mm->m.host.Nr;
    in.H = mm->m.host.H.data(); in.BH = mm->m.host.BH.data(); in.r = mm->m.host.r.data();
    in.HN = nullptr; in.n_HN = 0;
    s = check_input(&in);
    if (s) return s;
    s = build_job(&in, mm->m.host, hj[(size_t)i]);
    if (s) return s;
    hj[(size_t)i].seed = in.seed_given ? in.seed : clock_seed() + (uint64_t)i;
  }
  s = select_device(o.device);
  if (s) return s;
  VMC_CK(cudaStreamCreateWithFlags(&call_stream.s, cudaStreamNonBlocking));
  cudaStream_t stream = call_stream.s;
  cudaMemPool_t call_pool = nullptr;
  VMC_CK(cudaDeviceGetDefaultMemPool(&call_pool, o.device));
  // group by launch class
  struct Group { LaunchSpec spec; std::vector<int> idx; };
  std::vector<Group> groups;
  for (int i = 0; i < njobs; i++) {
    LaunchSpec sp;
    sp.dim = meshes[i]->m.host.dim;
    sp.precision = o.precision;
    sp.fd = hj[(size_t)i].omega > 0.0;
    sp.block = o.block_size;
    sp.blocks_per_sm = o.blocks_per_sm;
    sp.chunk = o.fetch_chunk;
    sp.max_steps = o.max_steps;
    sp.graph = o.use_graph != 0;
    sp.stage_slots = o.stage_slots;
    sp.refill = o.refill_lanes;
    auto it = std::find_if(groups.begin(), groups.end(), [&](const Group &g) { return g.spec.dim == sp.dim && g.spec.fd == sp.fd; });
    if (it == groups.end()) { groups.push_back(Group{sp, {}}); it = groups.end() - 1; }
    it->idx.push_back(i);
  }
  vmc_stats tot;
  memset(&tot, 0, sizeof(tot));
  auto t1 = std::chrono::steady_clock::now();
  double kernel_s = 0;
  for (auto &g : groups) {
    std::vector<JobDev> descs;
    for (int i : g.idx) {
      jb[(size_t)i].reset(new JobBuffers);
      jb[(size_t)i]->pool = call_pool;
      jb[(size_t)i]->free_stream = stream;
      s = upload_job(hj[(size_t)i], meshes[i]->m, o.precision, *jb[(size_t)i], stream);
      if (s) return s;
      JobDev d = describe_job(hj[(size_t)i], meshes[i]->m, o.precision, *jb[(size_t)i]);
      d.pcount = std::max<int64_t>(0, jobs[i].Nphoton);  // a negative count runs none
      d.poffset = o.photon_offset;
      d.stream = o.stream_id;
      descs.push_back(d);
    }
    LaunchResult lr;
    int ls = launch_jobs(o.device, g.spec, descs, &o, stream, lr);
    if (ls != VMC_OK) return ls;
    kernel_s += lr.kernel_ms * 1e-3;
    tot.steps += (int64_t)lr.steps;
    tot.scatters += (int64_t)lr.scatters;
    tot.photons_done += (int64_t)lr.done;
    tot.grid_blocks = lr.grid;
    tot.block_size = lr.block;
    for (int i : g.idx) {
      vmc_stats js;
      memset(&js, 0, sizeof(js));
      js.photons_requested = jobs[i].Nphoton;
      js.photons_done = std::max<int64_t>(0, jobs[i].Nphoton);
      js.seed_used = hj[(size_t)i].seed;
      s = collect_job(hj[(size_t)i], meshes[i]->m, *jb[(size_t)i], jobs[i].Nphoton, o.normalize != 0 || !opt_in,
                      &outs[i], &js, stream);
      if (s) return s;
      tot.photons_requested += jobs[i].Nphoton;
      tot.loss += js.loss;
      tot.capped += js.capped;
      tot.roulette_kills += js.roulette_kills;
      if (job_stats) job_stats[i] = js;
      jb[(size_t)i].reset();
    }
  }
  auto t2 = std::chrono::steady_clock::now();
  tot.seconds_kernel = kernel_s;
  tot.seconds_setup = std::chrono::duration<double>(t1 - t0).count();
  tot.seconds_total = std::chrono::duration<double>(t2 - t0).count();
  tot.bytes_h2d = g_h2d_bytes;
  tot.bytes_d2h = g_d2h_bytes;
  if (stats) *stats = tot;
  return VMC_OK;
}

}  // extern "C"
