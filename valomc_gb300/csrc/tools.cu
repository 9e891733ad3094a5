// tools.cu -- autotuner over launch shapes and the micro-benchmarks that give the roofline
// denominators the photon kernels are measured against:
//   vmc_bench_gather: random 32-byte-sector gathers whose next address depends on the data
//     just loaded (the shape of the element walk: load element, compute, load neighbour),
//     over a buffer of the mesh's size, at full occupancy.  For meshes that fit in L2 this
//     is the L2 random-gather ceiling; for larger buffers it approaches HBM.
//   vmc_bench_fp64: independent FP64 FMA chains (the plain form's arithmetic ceiling).
#include <cuda_runtime.h>
#include <string.h>

#include <algorithm>
#include <chrono>
#include <memory>
#include <vector>

#include "engine.hpp"

namespace vmc {
DeviceMesh *mesh_impl(vmc_mesh *m);
int mesh_precision_mask(const vmc_mesh *m);
}  // namespace vmc

using namespace vmc;

namespace {

__global__ void __launch_bounds__(256) gather_kernel(const uint4 *__restrict__ buf, unsigned long long nsec, int iters,
                                                    unsigned long long *sink) {
  unsigned long long x = (blockIdx.x * (unsigned long long)blockDim.x + threadIdx.x) * 0x9E3779B97F4A7C15ull + 1;
  unsigned acc = 0;
  for (int i = 0; i < iters; i++) {
    x ^= x >> 33;
    x *= 0xff51afd7ed558ccdull;
    x ^= x >> 29;
    const unsigned long long s = x % nsec;
    const uint4 a = __ldg(buf + 2 * s);
    const uint4 b = __ldg(buf + 2 * s + 1);
    const unsigned v = a.x ^ a.y ^ a.z ^ a.w ^ b.x ^ b.y ^ b.z ^ b.w;
    x += v;  // the next address depends on the loaded data
    acc += v;
  }
  if (acc == 0x12345678u) atomicAdd(sink, 1ull);
}

__global__ void __launch_bounds__(256) fp64_kernel(int iters, double *sink) {
  double a0 = threadIdx.x * 1e-3, a1 = a0 + 1, a2 = a0 + 2, a3 = a0 + 3, a4 = a0 + 4, a5 = a0 + 5, a6 = a0 + 6, a7 = a0 + 7;
  const double m = 0.999999, c = 1e-7;
  for (int i = 0; i < iters; i++) {
    a0 = fma(a0, m, c); a1 = fma(a1, m, c); a2 = fma(a2, m, c); a3 = fma(a3, m, c);
    a4 = fma(a4, m, c); a5 = fma(a5, m, c); a6 = fma(a6, m, c); a7 = fma(a7, m, c);
  }
  double s = a0 + a1 + a2 + a3 + a4 + a5 + a6 + a7;
  if (s == 12345.678) sink[0] = s;
}

}  // namespace

extern "C" {

int vmc_bench_gather(int32_t device, int64_t bytes, double seconds, double *gbs_out) {
  int sms = 0;
  int s = select_device(device, &sms);
  if (s) return s;
  if (bytes < 4096 || !gbs_out) return VMC_ERR_INVALID_ARGUMENT;
  const unsigned long long nsec = (unsigned long long)(bytes / 32);
  uint4 *buf = nullptr;
  unsigned long long *sink = nullptr;
  VMC_CK(cudaMalloc(&buf, nsec * 32));
  VMC_CK(cudaMalloc(&sink, 8));
  VMC_CK(cudaMemset(buf, 0x5a, nsec * 32));
  int per_sm = 0;
  VMC_CK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, gather_kernel, 256, 0));
  const int grid = per_sm * sms;
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  int iters = 64;
  float ms = 0;
  for (int round = 0; round < 12; round++) {
    cudaEventRecord(e0);
    gather_kernel<<<grid, 256>>>(buf, nsec, iters, sink);
    cudaEventRecord(e1);
    cudaEventSynchronize(e1);
    cudaEventElapsedTime(&ms, e0, e1);
    if (ms > 1000.0 * seconds || iters > (1 << 24)) break;
    iters *= 2;
  }
  cudaError_t e = cudaGetLastError();
  *gbs_out = (double)grid * 256.0 * iters * 32.0 / (ms * 1e-3) / 1e9;
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaFree(buf);
  cudaFree(sink);
  if (e != cudaSuccess) return cuda_status(e, "gather_kernel");
  return VMC_OK;
}

int vmc_bench_fp64(int32_t device, double seconds, double *tflops_out) {
  int sms = 0;
  int s = select_device(device, &sms);
  if (s) return s;
  if (!tflops_out) return VMC_ERR_INVALID_ARGUMENT;
  double *sink = nullptr;
  VMC_CK(cudaMalloc(&sink, 8));
  int per_sm = 0;
  VMC_CK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, fp64_kernel, 256, 0));
  const int grid = per_sm * sms;
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  int iters = 256;
  float ms = 0;
  for (int round = 0; round < 16; round++) {
    cudaEventRecord(e0);
    fp64_kernel<<<grid, 256>>>(iters, sink);
    cudaEventRecord(e1);
    cudaEventSynchronize(e1);
    cudaEventElapsedTime(&ms, e0, e1);
    if (ms > 1000.0 * seconds || iters > (1 << 26)) break;
    iters *= 2;
  }
  cudaError_t e = cudaGetLastError();
  *tflops_out = (double)grid * 256.0 * iters * 8.0 * 2.0 / (ms * 1e-3) / 1e12;
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaFree(sink);
  if (e != cudaSuccess) return cuda_status(e, "fp64_kernel");
  return VMC_OK;
}

// Times each launch shape on a bounded share of the jobs' photons (all jobs scaled by the
// same factor so the mix is kept) and keeps the fastest in photons per second.  A trial
// must keep every lane of the pool busy for many photon lifetimes: on a short trial the
// drain at the end of the launch (the longest walks) dominates the time and favours small
// grids, which lose at full size.  The default shape (256 threads, chunk 32, full
// occupancy) is kept unless another beats it by more than 2%.
int vmc_autotune(vmc_mesh *const *meshes, const vmc_input *jobs, int32_t njobs, vmc_options *opt, double budget_s) {
  if (!meshes || !jobs || njobs <= 0 || !opt) return VMC_ERR_INVALID_ARGUMENT;
  const int prec = opt->precision;
  const int mask = prec == VMC_FP64 ? 1 : 2;
  int s = select_device(opt->device);
  if (s) return s;
  std::vector<HostJob> hj((size_t)njobs);
  std::vector<std::unique_ptr<JobBuffers>> jb((size_t)njobs);
  std::vector<JobDev> descs;
  int64_t total = 0;
  bool fd = false;
  int dim = 0;
  for (int i = 0; i < njobs; i++) {
    DeviceMesh *m = mesh_impl(meshes[i]);
    if (!m || !(mesh_precision_mask(meshes[i]) & mask)) return VMC_ERR_INVALID_ARGUMENT;
    vmc_input in = jobs[i];
    in.dim = m->host.dim; in.Ne = m->host.Ne; in.Nb = m->host.Nb; in.Nr = m->host.Nr;
    in.H = m->host.H.data(); in.BH = m->host.BH.data(); in.r = m->host.r.data();
    in.HN = nullptr; in.n_HN = 0;
    s = check_input(&in);
    if (s) return s;
    s = build_job(&in, m->host, hj[(size_t)i]);
    if (s) return s;
    hj[(size_t)i].seed = 1234567 + (uint64_t)i;
    if (i == 0) { fd = hj[0].omega > 0; dim = m->host.dim; }
    if ((hj[(size_t)i].omega > 0) != fd || m->host.dim != dim) return VMC_ERR_INVALID_ARGUMENT;
    jb[(size_t)i].reset(new JobBuffers);
    s = upload_job(hj[(size_t)i], *m, prec, *jb[(size_t)i], 0);
    if (s) return s;
    descs.push_back(describe_job(hj[(size_t)i], *m, prec, *jb[(size_t)i]));
    total += jobs[i].Nphoton;
  }
  if (total <= 0) return VMC_ERR_INVALID_ARGUMENT;
  // a first short run calibrates the photon rate so each trial lasts about budget / trials
  const int blocks[] = {128, 256, 64};
  const int chunks[] = {32, 64, 128};
  const int refills[] = {1, 2, 8, 16};  // besides the default kDefaultRefill
  const int nshape = 3 * 3 * 2 + 4;
  LaunchSpec base;
  base.dim = dim; base.precision = prec; base.fd = fd; base.max_steps = opt->max_steps;
  auto run = [&](const LaunchSpec &sp, double frac, double &rate) -> int {
    std::vector<JobDev> d = descs;
    int64_t n = 0;
    for (int i = 0; i < njobs; i++) {
      d[(size_t)i].pcount = std::max<int64_t>(1, (int64_t)(frac * (double)jobs[i].Nphoton));
      n += d[(size_t)i].pcount;
      int z = zero_job(*jb[(size_t)i], 0);
      if (z) return z;
    }
    LaunchResult lr;
    int r = launch_jobs(opt->device, sp, d, nullptr, 0, lr);
    if (r) return r;
    rate = (double)n / std::max(1e-9, lr.kernel_ms * 1e-3);
    return VMC_OK;
  };
  int sms = 0;
  s = select_device(opt->device, &sms);
  if (s) return s;
  const double min_photons = 16.0 * 2048.0 * (double)sms;  // 16 fills of a full SM's lanes
  double rate0 = 0;
  double frac = std::min(1.0, min_photons / (double)total);
  s = run(base, frac, rate0);
  if (s) return s;
  const double per_trial = std::max(0.02, budget_s / nshape);
  frac = std::min(1.0, std::max(min_photons, rate0 * per_trial) / (double)total);
  double best = -1, dflt = -1;
  LaunchSpec bsp = base;
  for (int b : blocks)
    for (int c : chunks)
      for (int half = 0; half < 2; half++) {
        LaunchSpec sp = base;
        sp.block = b;
        sp.chunk = c;
        if (half) {
          int per_sm = 0;
          reset_carveout(select_kernel(sp));  // occupancy at the default split, as the launch plans it
          cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, select_kernel(sp), b, 0);
          if (per_sm < 2) continue;
          sp.blocks_per_sm = per_sm / 2;
        }
        double rate = 0;
        s = run(sp, frac, rate);
        if (s) return s;
        if (b == 256 && c == 32 && !half) dflt = rate;
        if (rate > best) { best = rate; bsp = sp; }
      }
  if (dflt > 0 && best < 1.04 * dflt) {
    bsp = base;
    bsp.block = 256;
    bsp.chunk = 32;
    bsp.blocks_per_sm = 0;
    best = dflt;
  }
  // second stage, on the chosen shape: the idle lanes a warp waits for before relaunching
  // them (short walks gain from launching several photons together), kept at the default
  // unless another count is 4% faster
  const double at_default = best;
  int best_refill = 0;
  for (int rf : refills) {
    LaunchSpec sp = bsp;
    sp.refill = rf;
    double rate = 0;
    s = run(sp, frac, rate);
    if (s) return s;
    if (rate > 1.04 * at_default && rate > best) { best = rate; best_refill = rf; }
  }
  opt->block_size = bsp.block;
  opt->fetch_chunk = bsp.chunk;
  opt->blocks_per_sm = bsp.blocks_per_sm;
  opt->refill_lanes = best_refill;
  return VMC_OK;
}

}  // extern "C"
