// pool.cuh -- the persistent photon-pool kernel.
//
// One CTA per SM slot stays resident for the whole run (the replacement of the reference's
// OpenMP team, cpp/3d/MC3D.hpp:1670-1700).  Every lane carries one photon; when photons
// end, the warp ballots its dead lanes and hands them the next indices from a warp-owned
// chunk of the global photon counter (one atomic per chunk), once refill_min lanes are
// idle or on every 8th iteration, so a warp never runs half-empty for long while photons
// remain.  A one-job launch on a small mesh stages the job's accumulators in shared memory
// (LaunchParams::dense) and adds them to the job's arrays when the CTA ends.  A photon index selects its job (batched launches),
// its Philox stream (key = job seed, counter = photon index) or its tape segment, and the
// walk advances one element step per loop iteration.  Each loop iteration polls nothing
// but registers; the host cancel flag is read every 1024 iterations.
#pragma once
#include "walk2d.cuh"

namespace vmc {

template <bool K> __device__ __forceinline__ void start_rng(PhiloxT<K> &rng, const JobDev &J, int64_t q) {
  rng.start(J.seed, J.stream, (uint64_t)(q + J.poffset));
}
__device__ __forceinline__ void start_rng(TapeRng &rng, const JobDev &J, int64_t q) {
  rng.start_tape(J.tape + J.tape_off[q], J.tape + J.tape_off[q + 1]);
}

// the job whose photon range [begin[j], begin[j + 1]) holds photon p
__device__ __forceinline__ int find_job(const int64_t *begin, int njobs, int64_t p) {
  int lo = 0, hi = njobs - 1;
  while (lo < hi) {
    int mid = (lo + hi + 1) >> 1;
    if (begin[mid] <= p) lo = mid;
    else hi = mid - 1;
  }
  return lo;
}

// R::kOneJob: a launch of one job, whose descriptor (lp.job0) and Philox round keys are read
// from the kernel parameters (constant bank) rather than from global memory and registers.
// kTab: a launch of at most kSmemJobs jobs whose CTAs first copy the job table and its
// photon prefix into shared memory, so that the walk reads the descriptor of each lane's
// job there instead of from global memory (the table follows the dynamic shared memory's
// start; multi-job launches stage no accumulators).
template <class W, class R, bool kTab>
__global__ void __launch_bounds__(256, W::kMinBlocks) pool_kernel(const __grid_constant__ LaunchParams lp) {
  constexpr bool kOne = R::kOneJob;
  static_assert(!(kOne && kTab), "a one-job launch has no job table");
  W s;
  R rng;
  if constexpr (kOne) rng.rk = lp.rk;
  const JobDev *jobs = lp.jobs;
  const int64_t *job_begin = lp.job_begin;
  if constexpr (kTab) {
    JobDev *tab = reinterpret_cast<JobDev *>(vmc_smem);
    int64_t *tbeg = reinterpret_cast<int64_t *>(vmc_smem + sizeof(JobDev) * (size_t)lp.njobs);
    const int nw = lp.njobs * (int)(sizeof(JobDev) / sizeof(uint64_t));
    const uint64_t *src = reinterpret_cast<const uint64_t *>(lp.jobs);
    uint64_t *dst = reinterpret_cast<uint64_t *>(tab);
    for (int i = threadIdx.x; i < nw; i += blockDim.x) dst[i] = __ldg(src + i);
    for (int i = threadIdx.x; i <= lp.njobs; i += blockDim.x) tbeg[i] = __ldg(lp.job_begin + i);
    __syncthreads();
    jobs = tab;
    job_begin = tbeg;
  }
  const JobDev *J = kOne ? &lp.job0 : jobs;
  Stage stg{nullptr, nullptr, 0u};
  if constexpr (W::kStaged) {
    if (lp.stage_slots > 0) {
      stg.val = reinterpret_cast<double *>(vmc_smem);
      stg.tag = reinterpret_cast<int32_t *>(vmc_smem + sizeof(double) * lp.stage_slots);
      stg.mask = (uint32_t)lp.stage_slots - 1u;
      for (int i = threadIdx.x; i < lp.stage_slots; i += blockDim.x) {
        stg.tag[i] = -1;
        stg.val[i] = 0.0;
      }
      __syncthreads();
    }
  }
  s.stage = stg;
  if (lp.dense > 0) {  // the CTA's copy of the single job's accumulators starts at zero
    double *sm = reinterpret_cast<double *>(vmc_smem);
    for (int i = threadIdx.x; i < lp.dense; i += blockDim.x) sm[i] = 0.0;
    __syncthreads();
  }
  bool alive = false, done = false;
  uint32_t n_steps = 0, n_scat = 0, n_done = 0;
  long long chunk_next = 0, chunk_end = 0;
  const unsigned lane = threadIdx.x & 31u;
  const unsigned lt_mask = (1u << lane) - 1u;
  const long long total = lp.total;
  for (unsigned it = 0;; ++it) {
    if ((it & 1023u) == 0u) {  // the host's cancel flag (an L2 round trip), every 1024 steps
      if (*reinterpret_cast<volatile const int32_t *>(&lp.ctl->cancel)) { done = true; alive = false; }
    }
    // refill and the exit test only when some lane is idle (one vote in the common case)
    if (__any_sync(kFull, !alive)) {
    unsigned need = __ballot_sync(kFull, !alive && !done);
    // short walks: wait (at most 7 iterations) until enough lanes are idle to launch together
    if (__popc(need) < lp.refill_min && (it & 7u) != 0u) need = 0u;
    while (need) {
      if (chunk_next >= chunk_end) {
        unsigned long long base = 0;
        if (lane == 0) base = atomicAdd(&lp.ctl->next_photon, (unsigned long long)lp.chunk);
        base = __shfl_sync(kFull, base, 0);
        if ((long long)base >= total) {
          if (!alive) done = true;
          break;
        }
        chunk_next = (long long)base;
        chunk_end = min(chunk_next + (long long)lp.chunk, total);
      }
      const long long avail = chunk_end - chunk_next;
      const int rank = __popc(need & lt_mask);
      if (((need >> lane) & 1u) && rank < avail) {
        const long long p = chunk_next + rank;
        if constexpr (!kOne) J = jobs + (lp.njobs > 1 ? find_job(job_begin, lp.njobs, p) : 0);
        const long long q = p - J->pbegin;
        start_rng(rng, *J, q);
        s.launch(*J, rng, q);
        alive = true;
        if constexpr (W::kLaunchLoss) {
          if (s.lost_at_launch(*J)) { alive = false; n_done++; }
        }
      }
      chunk_next += min((long long)__popc(need), avail);
      need = __ballot_sync(kFull, !alive && !done);
    }
    if (__all_sync(kFull, done)) break;
    }
    if (alive) {
      const int r = s.step(*J, rng, lp.max_steps);
      if (r == kScattered) { n_steps++; n_scat++; }
      else if (r == kAlive) { n_steps++; }
      else {
        if (r == kDied) n_steps++;
        alive = false;
        n_done++;
        job_count_add(*J, kJcSteps, (unsigned long long)s.nsteps);
      }
    }
  }
  if constexpr (W::kStaged) {
    // every warp of the CTA has left the loop: add the staged sums to the accumulator
    if (lp.stage_slots > 0) {
      __syncthreads();
      double *ER = lp.jobs[0].ER;
      for (int i = threadIdx.x; i < lp.stage_slots; i += blockDim.x) {
        const int32_t t = stg.tag[i];
        if (t >= 0 && stg.val[i] != 0.0) atomicAdd(ER + t, stg.val[i]);
      }
    }
  }
  if (lp.dense > 0) {
    // every warp of the CTA has left the loop: add the CTA's accumulators to the job's
    __syncthreads();
    const double *sm = reinterpret_cast<const double *>(vmc_smem);
    double *acc = kOne ? lp.job0.ER : lp.jobs[0].ER;
    for (int i = threadIdx.x; i < lp.dense; i += blockDim.x) {
      const double v = sm[i];
      if (v != 0.0) red_global(acc + i, v);
    }
  }
  unsigned long long a = n_steps, b = n_scat, c = n_done;
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    a += __shfl_xor_sync(kFull, a, o);
    b += __shfl_xor_sync(kFull, b, o);
    c += __shfl_xor_sync(kFull, c, o);
  }
  if (lane == 0) {
    atomicAdd(&lp.ctl->steps, a);
    atomicAdd(&lp.ctl->scatters, b);
    atomicAdd(&lp.ctl->done_photons, c);
  }
}

}  // namespace vmc
