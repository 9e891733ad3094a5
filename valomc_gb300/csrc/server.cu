// server.cu -- serving loop: resident meshes, requests admitted into slots by their
// device-memory footprint, continuous batching of all admitted requests into persistent
// launches ("epochs") sized by the backlog (50 ms of work when it is small, up to a cap,
// 0.5 s by default).
//
// Epochs alternate between two streams ("lanes"): the next epoch is built and queued once
// the running one has handed out most of its photons, so that it takes the SMs as the
// running launch drains and still carries the requests that arrived during that launch.
//
// A request's photons are issued in slices across epochs; slice k of a request simulates
// photon indices [issued, issued + quota) of the request's own Philox stream (key = the
// request seed, counter = photon index), so the photons and their draws do not depend on
// what else shares the launch or how the request was sliced -- a result alone and in a
// mix differs only by the order of the FP64 atomic additions.  New requests join at the
// next epoch boundary while older ones are still in flight, so their work overlaps on the
// device.
#include <cuda_runtime.h>
#include <string.h>

#include <algorithm>
#include <chrono>
#include <condition_variable>
#include <deque>
#include <map>
#include <memory>
#include <mutex>
#include <thread>
#include <vector>

#include "engine.hpp"
#include "epoch_plan.hpp"

namespace vmc {
DeviceMesh *mesh_impl(vmc_mesh *m);
int mesh_precision_mask(const vmc_mesh *m);
}  // namespace vmc

using namespace vmc;
using Clock = std::chrono::steady_clock;

namespace {

enum ReqState { kQueued = 0, kActive = 1, kFinished = 2, kFailed = 3 };

struct Request {
  int64_t id = 0;
  int mesh_id = 0;
  HostJob job;
  int64_t nphoton = 0, issued = 0;
  int64_t footprint = 0;
  std::unique_ptr<JobBuffers> buf;
  int state = kQueued;
  int status = VMC_OK;
  int inflight = 0;  // launches holding a slice of this request
  int64_t slice = 0; // photons of this request in the epoch being built
  bool retiring = false;
  Clock::time_point t_submit, t_admit, t_finish;
  double kernel_s = 0;
  std::vector<double> ER, EI, EBR, EBI, DEBR, DEBI;
  vmc_stats stats;
};

}  // namespace

struct vmc_server {
  vmc_server_config cfg;
  std::vector<vmc_mesh *> meshes;
  std::mutex mu;
  std::condition_variable cv_work, cv_done;
  std::deque<Request *> queue;
  std::vector<Request *> active;
  std::map<int64_t, std::unique_ptr<Request>> all;
  int64_t next_id = 1;
  int64_t mem_in_use = 0;
  double rate = 0;  // photons per second seen in recent epochs
  bool stop = false;
  std::thread worker;
  // Finished requests wait here for their results to be copied back and normalised by the
  // collector thread, so that the launch loop never stops for a read-back.
  std::deque<Request *> to_collect;
  std::condition_variable cv_collect;
  bool collector_stop = false;
  std::thread collector;
  // request buffers: a memory pool of the device, allocated on the upload stream and
  // returned on free_stream (no device-wide wait when a request finishes)
  cudaMemPool_t pool = nullptr;
  cudaStream_t free_stream = nullptr;
  void loop();
  void collect_loop();
  void finalize(Request *r);
};

namespace {
// One of the two launch pipelines of the serving loop: a stream, an arena per launch class
// (dimension x CW/FD) and the requests whose slices ride in its current epoch.
struct Lane {
  cudaStream_t st = nullptr;
  std::vector<std::unique_ptr<LaunchArena>> arenas;
  std::vector<std::vector<Request *>> members;  // per arena: the requests of its launch
  std::vector<std::vector<int64_t>> quotas;
  bool pending = false;
  double photons = 0;
};

// Returns when the epoch running on lane R has handed out 85% of its photons (its launch's
// fetch counter, read with an 8-byte copy on the probe stream every 0.5 ms; the last 15%
// keep the SMs busy while the next epoch is built and queued), when it has ended, after
// 1.2 x its duration expected at the measured rate, or when the server stops.  The counter
// is read only from 1 ms after the launch has started, when the launch's reset of its
// control block has run.
void wait_until_drain_nears(vmc_server &s, Lane &R, cudaStream_t probe, unsigned long long *hnext) {
  if (!R.pending) return;
  LaunchArena *a = nullptr;  // the epoch's largest launch
  for (size_t k = 0; k < R.members.size(); k++)
    if (!R.members[k].empty() && (!a || R.arenas[k]->total > a->total)) a = R.arenas[k].get();
  const double expect_s = s.rate > 0 ? R.photons / s.rate : 0.0;
  if (!a || a->total <= 0 || expect_s <= 0.01) return;
  const auto t0 = Clock::now();
  bool started = false;
  Clock::time_point ts;
  for (;;) {
    if (cudaEventQuery(a->e1) == cudaSuccess) break;
    const auto now = Clock::now();
    if (std::chrono::duration<double>(now - t0).count() > 1.2 * expect_s + 0.005) break;
    if (!started) {
      if (cudaEventQuery(a->e0) == cudaSuccess) { started = true; ts = now; }
    } else if (std::chrono::duration<double>(now - ts).count() > 0.001) {
      if (cudaMemcpyAsync(hnext, &a->dctl->next_photon, sizeof(unsigned long long), cudaMemcpyDeviceToHost, probe) !=
              cudaSuccess ||
          cudaStreamSynchronize(probe) != cudaSuccess)
        break;
      if ((double)*hnext >= 0.85 * (double)a->total) break;
    }
    {
      std::lock_guard<std::mutex> lk(s.mu);
      if (s.stop) break;
    }
    std::this_thread::sleep_for(std::chrono::microseconds(500));
  }
  cudaGetLastError();  // a query that found its event pending is not an error
}

}  // namespace

void vmc_server::loop() {
  cudaSetDevice(cfg.device);
  // Two lanes: while an epoch runs on one, the next is prepared and queued on the other,
  // so its CTAs take the SMs as the running launch drains (no idle tail between epochs).
  Lane lanes[2];
  for (auto &l : lanes) cudaStreamCreateWithFlags(&l.st, cudaStreamNonBlocking);
  // progress reads of the running epoch (late binding, below): a stream of their own and a
  // pinned word
  cudaStream_t probe = nullptr;
  cudaStreamCreateWithFlags(&probe, cudaStreamNonBlocking);
  unsigned long long *hnext = nullptr;
  if (cudaMallocHost(reinterpret_cast<void **>(&hnext), sizeof(unsigned long long)) != cudaSuccess) hnext = nullptr;
  cudaGetLastError();
  Clock::time_point last_finish = Clock::now();
  int cur = 0;
  for (;;) {
    // Late binding: the next epoch is built when most of the running one's photons have
    // been handed out, not as soon as it starts, so that requests arriving meanwhile ride
    // in it: a request waits for about one epoch instead of up to two (at 50 req/s on the serving
    // mix, median latency 0.14 s against 0.17 s, no change in capacity).
    if (probe && hnext) wait_until_drain_nears(*this, lanes[cur ^ 1], probe, hnext);
    std::vector<Request *> admitted;
    std::vector<Request *> batch;
    int64_t backlog = 0;  // photons not yet issued, active and queued
    {
      std::unique_lock<std::mutex> lk(mu);
      auto has_work = [&] {
        // a queued request that can be admitted now (or refused: larger than the budget)
        if (!queue.empty() && (int)active.size() < cfg.max_slots &&
            (queue.front()->footprint > cfg.memory_budget ||
             mem_in_use + queue.front()->footprint <= cfg.memory_budget))
          return true;
        for (Request *r : active)
          if (r->status == VMC_OK && r->issued < r->nphoton) return true;
        return false;
      };
      if (!lanes[0].pending && !lanes[1].pending) cv_work.wait(lk, [&] { return stop || has_work(); });
      if (stop) break;
      // admission: FIFO while a slot is free and the footprint fits the budget
      while (!queue.empty() && (int)active.size() < cfg.max_slots) {
        Request *r = queue.front();
        if (r->footprint > cfg.memory_budget) {
          queue.pop_front();
          r->state = kFailed;
          r->status = VMC_ERR_ADMISSION;
          r->t_finish = Clock::now();
          cv_done.notify_all();
          continue;
        }
        if (mem_in_use + r->footprint > cfg.memory_budget) break;
        queue.pop_front();
        mem_in_use += r->footprint;
        r->state = kActive;
        r->t_admit = Clock::now();
        active.push_back(r);
        admitted.push_back(r);
      }
      batch = active;
      for (Request *r : active)
        if (r->status == VMC_OK) backlog += std::max<int64_t>(0, r->nphoton - r->issued);
      for (Request *r : queue) backlog += std::max<int64_t>(0, r->nphoton);
    }
    Lane &L = lanes[cur];
    // L's previous epoch has finished (it was the other lane one iteration ago), so its
    // stream is idle: upload the new requests there and wait for the copies, which orders
    // them before any launch on either lane.
    for (Request *r : admitted) {
      r->buf.reset(new JobBuffers);
      r->buf->pool = pool;
      r->buf->free_stream = free_stream;
      DeviceMesh *m = mesh_impl(meshes[(size_t)r->mesh_id]);
      r->status = upload_job(r->job, *m, cfg.precision, *r->buf, L.st);
    }
    if (!admitted.empty()) cudaStreamSynchronize(L.st);
    // epoch: a slice of every active request with photons left, one launch per class.  Its
    // size follows the load (epoch_photons): 50 ms of work while the backlog is small
    // (latency), up to the backlog and at most epoch_max_ms (0.5 s) of work as it grows.
    // Every launch ends in a drain (CTAs keep their SM slot until their slowest walk ends);
    // larger epochs pay it less often, so the loop's capacity rises with the load that needs
    // it, while a request that arrives waits for about one epoch (late binding, above).
    const int64_t epoch = epoch_photons(cfg.epoch_photons, rate, cfg.epoch_max_ms, backlog);
    std::vector<Request *> open;
    for (Request *r : batch)
      if (r->status == VMC_OK && r->issued < r->nphoton) open.push_back(r);
    // slices: shortest remaining first with a floor share (default), or water-filling
    // (epoch_plan.hpp)
    {
      std::vector<int64_t> left;
      for (Request *r : open) left.push_back(r->nphoton - r->issued);
      const std::vector<int64_t> sl = epoch_slices(left, epoch, cfg.slicing != VMC_SLICE_EQUAL);
      for (size_t i = 0; i < open.size(); i++) open[i]->slice = sl[i];
    }
    struct Cls { int dim; bool fd; std::vector<Request *> rs; };
    std::vector<Cls> classes;
    for (Request *r : open) {
      DeviceMesh *m = mesh_impl(meshes[(size_t)r->mesh_id]);
      bool fd = r->job.omega > 0;
      Cls *c = nullptr;
      for (auto &x : classes)
        if (x.dim == m->host.dim && x.fd == fd) c = &x;
      if (!c) { classes.push_back(Cls{m->host.dim, fd, {}}); c = &classes.back(); }
      c->rs.push_back(r);
    }
    L.members.assign(classes.size(), {});
    L.quotas.assign(classes.size(), {});
    while (L.arenas.size() < classes.size()) L.arenas.emplace_back(new LaunchArena);
    L.photons = 0;
    for (size_t k = 0; k < classes.size(); k++) {
      Cls &c = classes[k];
      std::vector<JobDev> descs;
      std::vector<int64_t> quota;
      for (Request *r : c.rs) {
        DeviceMesh *m = mesh_impl(meshes[(size_t)r->mesh_id]);
        JobDev d = describe_job(r->job, *m, cfg.precision, *r->buf);
        int64_t qn = r->slice;
        d.pcount = qn;
        d.poffset = r->issued;
        descs.push_back(d);
        quota.push_back(qn);
      }
      LaunchSpec sp;
      sp.dim = c.dim;
      sp.precision = cfg.precision;
      sp.fd = c.fd;
      sp.block = cfg.block_size;
      sp.blocks_per_sm = cfg.blocks_per_sm;
      sp.graph = cfg.use_graph != 0;
      LaunchResult lr;
      int st = launch_start(cfg.device, sp, descs, *L.arenas[k], L.st, lr);
      for (size_t i = 0; i < c.rs.size(); i++) {
        Request *r = c.rs[i];
        if (st != VMC_OK) { r->status = st; continue; }
        r->issued += quota[i];
        r->inflight++;
        L.photons += (double)quota[i];
      }
      if (st == VMC_OK) {
        L.members[k] = c.rs;
        L.quotas[k] = quota;
        L.pending = true;
      }
    }
    // finish the other lane's epoch (queued ahead of this one) and retire what it completed
    Lane &O = lanes[cur ^ 1];
    if (O.pending) {
      O.pending = false;
      std::vector<int> ok(O.members.size(), VMC_OK);
      for (size_t k = 0; k < O.members.size(); k++) {
        if (O.members[k].empty()) continue;
        LaunchResult lr;
        ok[k] = launch_finish(*O.arenas[k], O.st, lr);
      }
      auto now = Clock::now();
      // Epochs overlap, so a request's device time is counted as the disjoint intervals
      // between successive epoch ends, from its submission on.
      for (size_t k = 0; k < O.members.size(); k++)
        for (Request *r : O.members[k]) {
          r->inflight--;
          if (ok[k] != VMC_OK) r->status = ok[k];
          r->kernel_s += std::chrono::duration<double>(now - std::max(last_finish, r->t_submit)).count();
        }
      const double dt = std::chrono::duration<double>(now - last_finish).count();
      if (dt > 0 && O.photons > 0) rate = O.photons / dt;
      last_finish = now;
      O.members.clear();
    } else {
      last_finish = Clock::now();  // the device was idle: the rate clock starts now
    }
    // retire finished (or failed) requests that have no slice in flight: the results of
    // finished ones go to the collector thread
    std::vector<Request *> fin;
    for (Request *r : batch)
      if (r->inflight == 0 && !r->retiring && (r->status != VMC_OK || r->issued >= r->nphoton)) fin.push_back(r);
    for (Request *r : fin) {
      r->retiring = true;
      if (r->status == VMC_OK) {
        std::lock_guard<std::mutex> lk(mu);
        to_collect.push_back(r);
        cv_collect.notify_one();
      } else {
        finalize(r);
      }
    }
    cur ^= 1;
  }
  if (probe) cudaStreamDestroy(probe);
  if (hnext) cudaFreeHost(hnext);
  // stopping: let launches in flight end before their buffers go
  for (auto &l : lanes) {
    if (l.st) cudaStreamSynchronize(l.st);
    l.arenas.clear();
    if (l.st) cudaStreamDestroy(l.st);
  }
}

void vmc_server::finalize(Request *r) {
  r->buf.reset();
  std::lock_guard<std::mutex> lk(mu);
  mem_in_use -= r->footprint;
  r->t_finish = Clock::now();
  r->state = r->status == VMC_OK ? kFinished : kFailed;
  r->stats.seconds_kernel = r->kernel_s;
  r->stats.seconds_setup = std::chrono::duration<double>(r->t_admit - r->t_submit).count();
  r->stats.seconds_total = std::chrono::duration<double>(r->t_finish - r->t_submit).count();
  active.erase(std::find(active.begin(), active.end(), r));
  cv_done.notify_all();
  cv_work.notify_all();  // memory and a slot were freed
}

void vmc_server::collect_loop() {
  cudaSetDevice(cfg.device);
  cudaStream_t st = nullptr;
  cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking);
  for (;;) {
    Request *r = nullptr;
    {
      std::unique_lock<std::mutex> lk(mu);
      cv_collect.wait(lk, [&] { return collector_stop || !to_collect.empty(); });
      if (to_collect.empty()) break;  // stopping and nothing left
      r = to_collect.front();
      to_collect.pop_front();
    }
    // the request's last launch has completed (the loop saw its event), so its
    // accumulators are final
    DeviceMesh *m = mesh_impl(meshes[(size_t)r->mesh_id]);
    const int64_t Ne = m->host.Ne, Nb = m->host.Nb;
    r->ER.resize((size_t)Ne); r->EI.resize((size_t)Ne);
    r->EBR.resize((size_t)Nb); r->EBI.resize((size_t)Nb); r->DEBR.resize((size_t)Nb); r->DEBI.resize((size_t)Nb);
    vmc_output o;
    memset(&o, 0, sizeof(o));
    o.ER = r->ER.data(); o.EI = r->EI.data(); o.EBR = r->EBR.data(); o.EBI = r->EBI.data();
    o.DEBR = r->DEBR.data(); o.DEBI = r->DEBI.data();
    r->stats.photons_requested = r->nphoton;
    r->stats.photons_done = r->issued;
    r->stats.seed_used = r->job.seed;
    r->status = collect_job(r->job, *m, *r->buf, r->nphoton, true, &o, &r->stats, st);
    finalize(r);
  }
  cudaStreamDestroy(st);
}

extern "C" {

int vmc_server_create(const vmc_server_config *cfg, vmc_server **out) {
  if (!cfg || !out || cfg->max_slots <= 0 || cfg->memory_budget <= 0) return VMC_ERR_INVALID_ARGUMENT;
  if (cfg->precision != VMC_FP32 && cfg->precision != VMC_FP64) return VMC_ERR_INVALID_ARGUMENT;
  if (cfg->slicing < VMC_SLICE_DEFAULT || cfg->slicing > VMC_SLICE_SHORTEST_FIRST) return VMC_ERR_INVALID_ARGUMENT;
  if (cfg->epoch_max_ms < 0 || (cfg->epoch_max_ms > 0 && cfg->epoch_max_ms < 50)) return VMC_ERR_INVALID_ARGUMENT;
  int s = select_device(cfg->device);
  if (s) return s;
  vmc_server *sv = new vmc_server;
  sv->cfg = *cfg;
  {
    // admission cannot promise more device memory than the device has free: the budget is
    // clamped to the free bytes at creation, less a margin for the launch tables and the
    // stream-ordered pool's own granularity
    size_t free_b = 0, total_b = 0;
    if (cudaMemGetInfo(&free_b, &total_b) == cudaSuccess) {
      const int64_t margin = 256ll << 20;
      const int64_t usable = std::max<int64_t>(0, (int64_t)free_b - margin);
      if (sv->cfg.memory_budget > usable) sv->cfg.memory_budget = usable;
    }
  }
  {
    cudaMemPoolProps props;
    memset(&props, 0, sizeof(props));
    props.allocType = cudaMemAllocationTypePinned;
    props.location.type = cudaMemLocationTypeDevice;
    props.location.id = cfg->device;
    cudaError_t e = cudaMemPoolCreate(&sv->pool, &props);
    if (e == cudaSuccess) {
      uint64_t keep = UINT64_MAX;  // keep freed blocks for the next requests
      e = cudaMemPoolSetAttribute(sv->pool, cudaMemPoolAttrReleaseThreshold, &keep);
    }
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&sv->free_stream, cudaStreamNonBlocking);
    if (e != cudaSuccess) {
      if (sv->pool) cudaMemPoolDestroy(sv->pool);
      delete sv;
      return cuda_status(e, "server memory pool");
    }
  }
  sv->worker = std::thread([sv] { sv->loop(); });
  sv->collector = std::thread([sv] { sv->collect_loop(); });
  *out = sv;
  return VMC_OK;
}

int vmc_server_add_mesh(vmc_server *s, vmc_mesh *mesh, int32_t *mesh_id) {
  if (!s || !mesh || !mesh_id) return VMC_ERR_INVALID_ARGUMENT;
  const int mask = s->cfg.precision == VMC_FP64 ? 1 : 2;
  if (!(mesh_precision_mask(mesh) & mask)) return VMC_ERR_INVALID_ARGUMENT;
  std::lock_guard<std::mutex> lk(s->mu);
  s->meshes.push_back(mesh);
  *mesh_id = (int32_t)s->meshes.size() - 1;
  return VMC_OK;
}

int vmc_server_submit(vmc_server *s, int32_t mesh_id, const vmc_input *job, int64_t *req_id) {
  if (!s || !job || !req_id) return VMC_ERR_INVALID_ARGUMENT;
  vmc_mesh *mm;
  {
    std::lock_guard<std::mutex> lk(s->mu);
    if (mesh_id < 0 || mesh_id >= (int32_t)s->meshes.size()) return VMC_ERR_NOT_FOUND;
    mm = s->meshes[(size_t)mesh_id];
  }
  DeviceMesh *m = mesh_impl(mm);
  std::unique_ptr<Request> r(new Request);
  memset(&r->stats, 0, sizeof(r->stats));
  vmc_input in = *job;
  in.dim = m->host.dim; in.Ne = m->host.Ne; in.Nb = m->host.Nb; in.Nr = m->host.Nr;
  in.H = m->host.H.data(); in.BH = m->host.BH.data(); in.r = m->host.r.data();
  in.HN = nullptr; in.n_HN = 0;
  int st = check_input(&in);
  if (st) return st;
  st = build_job(&in, m->host, r->job);
  if (st) return st;
  r->job.seed = in.seed_given ? in.seed : clock_seed();
  r->mesh_id = mesh_id;
  r->nphoton = in.Nphoton;
  r->footprint = job_footprint(r->job, m->host);
  r->t_submit = Clock::now();
  std::lock_guard<std::mutex> lk(s->mu);
  r->id = s->next_id++;
  *req_id = r->id;
  s->queue.push_back(r.get());
  s->all[r->id] = std::move(r);
  s->cv_work.notify_all();
  return VMC_OK;
}

static int take_result(Request *r, vmc_output *out, vmc_stats *stats) {
  if (r->state == kFailed) return -r->status;
  if (out) {
    auto cp = [](double *dst, const std::vector<double> &v) {
      if (dst && !v.empty()) memcpy(dst, v.data(), v.size() * sizeof(double));
    };
    cp(out->ER, r->ER); cp(out->EI, r->EI); cp(out->EBR, r->EBR); cp(out->EBI, r->EBI);
    cp(out->DEBR, r->DEBR); cp(out->DEBI, r->DEBI);
  }
  if (stats) *stats = r->stats;
  return 1;
}

int vmc_server_poll(vmc_server *s, int64_t req_id, vmc_output *out, vmc_stats *stats) {
  if (!s) return -VMC_ERR_INVALID_ARGUMENT;
  std::lock_guard<std::mutex> lk(s->mu);
  auto it = s->all.find(req_id);
  if (it == s->all.end()) return -VMC_ERR_NOT_FOUND;
  Request *r = it->second.get();
  if (r->state == kQueued || r->state == kActive) return 0;
  return take_result(r, out, stats);
}

int vmc_server_wait(vmc_server *s, int64_t req_id, vmc_output *out, vmc_stats *stats, double timeout_s) {
  if (!s) return -VMC_ERR_INVALID_ARGUMENT;
  std::unique_lock<std::mutex> lk(s->mu);
  auto it = s->all.find(req_id);
  if (it == s->all.end()) return -VMC_ERR_NOT_FOUND;
  Request *r = it->second.get();
  auto done = [&] { return r->state == kFinished || r->state == kFailed; };
  if (timeout_s > 0) {
    if (!s->cv_done.wait_for(lk, std::chrono::duration<double>(timeout_s), done)) return 0;
  } else {
    s->cv_done.wait(lk, done);
  }
  return take_result(r, out, stats);
}

int vmc_server_destroy(vmc_server *s) {
  if (!s) return VMC_ERR_INVALID_ARGUMENT;
  {
    std::lock_guard<std::mutex> lk(s->mu);
    s->stop = true;
    s->cv_work.notify_all();
  }
  if (s->worker.joinable()) s->worker.join();
  {
    std::lock_guard<std::mutex> lk(s->mu);
    s->collector_stop = true;
    s->cv_collect.notify_all();
  }
  if (s->collector.joinable()) s->collector.join();
  for (auto &kv : s->all) kv.second->buf.reset();
  if (s->free_stream) {
    cudaStreamSynchronize(s->free_stream);
    cudaStreamDestroy(s->free_stream);
  }
  if (s->pool) cudaMemPoolDestroy(s->pool);
  delete s;
  return VMC_OK;
}

}  // extern "C"
