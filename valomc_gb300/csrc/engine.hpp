// engine.hpp -- internal interface between the C ABI, the batch path and the serving loop.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include <string>
#include <vector>

#include "host_setup.hpp"

namespace vmc {

void set_error(const std::string &msg);
int cuda_status(cudaError_t e, const char *what);
#define VMC_CK(call)                                      \
  do {                                                    \
    cudaError_t _e = (call);                              \
    if (_e != cudaSuccess) return cuda_status(_e, #call); \
  } while (0)

int select_device(int device, int *num_sms = nullptr);
uint64_t clock_seed();

// Resident geometry (the opaque vmc_mesh).
struct DeviceMesh {
  int device = 0;
  int dim = 3;
  HostMesh host;
  void *d_geom[2] = {nullptr, nullptr};  // [precision]
  double *d_bnorm = nullptr;
  int64_t bytes = 0;
  // a mesh that lives for one call: allocated from `pool` and copied, then freed, in order
  // on `st` (no device-wide synchronisation); resident meshes keep plain allocations
  cudaMemPool_t pool = nullptr;
  cudaStream_t st = nullptr;
  ~DeviceMesh();
  const void *geom(int precision) const { return d_geom[precision]; }
};
int upload_mesh(DeviceMesh &m, int precision_mask);

// Device state of one job.
struct JobBuffers {
  void *d_optics = nullptr;
  uint8_t *d_bctype = nullptr;
  double *d_bcn = nullptr, *d_cdf = nullptr;
  SourceRec *d_src = nullptr;
  float *d_cdf_f = nullptr;
  SourceRecF *d_src_f = nullptr;
  double *d_acc = nullptr;  // ER, EI [Ne]; EBR, EBI, DEBR, DEBI [Nb]
  unsigned long long *d_jc = nullptr;
  double *d_ledger = nullptr;
  uint32_t *d_tape = nullptr;
  int64_t *d_tape_off = nullptr, *d_trace = nullptr, *d_trace_len = nullptr;
  int64_t bytes = 0;
  int64_t Ne = 0, Nb = 0;
  // Stream-ordered allocation (the serving loop): buffers come from `pool` on the upload
  // stream and go back with cudaFreeAsync on `free_stream`, so that freeing a finished
  // request never waits for the device (cudaFree would, and stall the launches in flight).
  cudaMemPool_t pool = nullptr;
  cudaStream_t free_stream = nullptr;
  ~JobBuffers();
  void release();
};
// bytes of device state a job on mesh m needs (admission control)
int64_t job_footprint(const HostJob &j, const HostMesh &m);
int upload_job(const HostJob &j, const DeviceMesh &m, int precision, JobBuffers &b, cudaStream_t st);
JobDev describe_job(const HostJob &j, const DeviceMesh &m, int precision, const JobBuffers &b);
int zero_job(JobBuffers &b, cudaStream_t st);

struct LaunchSpec {
  int dim = 3, precision = VMC_FP32;
  bool fd = false, tape = false;
  bool graph = false;  // launch through a (reused) CUDA graph
  int stage_slots = 0; // shared-memory staging slots per CTA (0: off)
  int block = 0, blocks_per_sm = 0, chunk = 0;
  int refill = 0;      // idle lanes a warp waits for before relaunching (0: default)
  int64_t max_steps = 0;
};
struct LaunchResult {
  uint64_t steps = 0, scatters = 0, done = 0;
  double kernel_ms = 0;
  int grid = 0, block = 0;
};
// Runs the pool kernel over jobs (device descriptors are uploaded here) and waits,
// polling progress / cancel / timeout from opt (may be null).  Stream-ordered.
int launch_jobs(int device, const LaunchSpec &spec, const std::vector<JobDev> &jobs, const vmc_options *opt,
                cudaStream_t st, LaunchResult &res);

// Device and pinned buffers of one launch at a time, reused across launches: the job
// table, its photon prefix, the control block, the timing events and a graph.  Lets a
// caller keep a launch in flight while it prepares the next on another arena and stream.
struct LaunchArena {
  JobDev *djobs = nullptr, *hjobs = nullptr;
  int64_t *dbegin = nullptr, *hbegin = nullptr;
  Ctl *dctl = nullptr, *hctl = nullptr;
  size_t cap_jobs = 0;
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  cudaStream_t cap_stream = nullptr;  // graph capture
  cudaGraphExec_t exec = nullptr;
  int64_t total = 0;
  bool pending = false;
  LaunchArena() = default;
  LaunchArena(const LaunchArena &) = delete;
  LaunchArena &operator=(const LaunchArena &) = delete;
  ~LaunchArena();
};
// Enqueues the pool kernel over jobs on `st` without waiting (no progress polling).
int launch_start(int device, const LaunchSpec &spec, const std::vector<JobDev> &jobs, LaunchArena &a,
                 cudaStream_t st, LaunchResult &res);
// Waits for the arena's launch and reads its counters (no-op when nothing is in flight).
int launch_finish(LaunchArena &a, cudaStream_t st, LaunchResult &res);

// Copies a job's accumulators and counters back and fills out/stats.
int collect_job(const HostJob &j, const DeviceMesh &m, const JobBuffers &b, int64_t nphoton, bool normalize,
                vmc_output *out, vmc_stats *st, cudaStream_t stream);

const void *kernel_3d64(bool fd, bool tape, bool one, bool tab);
const void *kernel_3d32(bool fd, bool tape, bool one, bool tab);
const void *kernel_2d64(bool fd, bool tape, bool one, bool tab);
const void *kernel_2d32(bool fd, bool tape, bool one, bool tab);
// one: the single-job form (descriptor and round keys in LaunchParams::job0 / rk);
// tab: the per-job form with the job table copied into each CTA's shared memory
const void *select_kernel(const LaunchSpec &s, bool one = false, bool tab = false);
void set_single_job(LaunchParams &lp, const JobDev &job);
// the L1 / shared-memory split of a pool kernel: reset to the driver's default before the
// occupancy query, then the smallest split holding per_sm CTAs' shared memory
void reset_carveout(const void *fn);
void fit_carveout(const void *fn, int device, int per_sm, size_t dyn_smem);

}  // namespace vmc
