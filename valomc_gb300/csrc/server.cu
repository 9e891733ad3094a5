// server.cu -- serving loop: resident meshes, requests admitted into slots by their
// device-memory footprint, continuous batching of all admitted requests into short
// persistent launches ("epochs").
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
  void loop();
};

void vmc_server::loop() {
  cudaSetDevice(cfg.device);
  cudaStream_t st = 0;
  for (;;) {
    std::vector<Request *> admitted;
    std::vector<Request *> batch;
    {
      std::unique_lock<std::mutex> lk(mu);
      cv_work.wait(lk, [&] { return stop || !queue.empty() || !active.empty(); });
      if (stop) return;
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
    }
    for (Request *r : admitted) {
      r->buf.reset(new JobBuffers);
      DeviceMesh *m = mesh_impl(meshes[(size_t)r->mesh_id]);
      r->status = upload_job(r->job, *m, cfg.precision, *r->buf, st);
    }
    // epoch: a slice of every active request, in as many launches as there are classes
    int64_t epoch = cfg.epoch_photons > 0 ? cfg.epoch_photons
                                          : std::max<int64_t>(200000, (int64_t)(rate * 0.05));
    const int64_t share = std::max<int64_t>(1, epoch / (int64_t)std::max<size_t>(1, batch.size()));
    struct Cls { int dim; bool fd; std::vector<Request *> rs; };
    std::vector<Cls> classes;
    for (Request *r : batch) {
      if (r->status != VMC_OK) continue;
      DeviceMesh *m = mesh_impl(meshes[(size_t)r->mesh_id]);
      bool fd = r->job.omega > 0;
      Cls *c = nullptr;
      for (auto &x : classes)
        if (x.dim == m->host.dim && x.fd == fd) c = &x;
      if (!c) { classes.push_back(Cls{m->host.dim, fd, {}}); c = &classes.back(); }
      c->rs.push_back(r);
    }
    double epoch_ph = 0, epoch_s = 0;
    for (auto &c : classes) {
      std::vector<JobDev> descs;
      std::vector<int64_t> quota;
      for (Request *r : c.rs) {
        DeviceMesh *m = mesh_impl(meshes[(size_t)r->mesh_id]);
        JobDev d = describe_job(r->job, *m, cfg.precision, *r->buf);
        int64_t qn = std::min(share, r->nphoton - r->issued);
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
      int s = launch_jobs(cfg.device, sp, descs, nullptr, st, lr);
      for (size_t i = 0; i < c.rs.size(); i++) {
        Request *r = c.rs[i];
        if (s != VMC_OK) { r->status = s; continue; }
        r->issued += quota[i];
        r->kernel_s += lr.kernel_ms * 1e-3;
      }
      if (s == VMC_OK) {
        for (int64_t q : quota) epoch_ph += (double)q;
        epoch_s += lr.kernel_ms * 1e-3;
      }
    }
    if (epoch_s > 0) rate = epoch_ph / epoch_s;
    // retire finished (or failed) requests
    std::vector<Request *> fin;
    for (Request *r : batch)
      if (r->status != VMC_OK || r->issued >= r->nphoton) fin.push_back(r);
    for (Request *r : fin) {
      if (r->status == VMC_OK) {
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
      }
      r->buf.reset();
      std::lock_guard<std::mutex> lk(mu);
      mem_in_use -= r->footprint;
      r->t_finish = Clock::now();
      r->state = r->status == VMC_OK ? kFinished : kFailed;
      r->stats.seconds_kernel = r->kernel_s;
      r->stats.seconds_setup = std::chrono::duration<double>(r->t_admit - r->t_submit).count();
      r->stats.seconds_total = std::chrono::duration<double>(r->t_finish - r->t_submit).count();
      active.erase(std::find(active.begin(), active.end(), r));
    }
    if (!fin.empty()) cv_done.notify_all();
  }
}

extern "C" {

int vmc_server_create(const vmc_server_config *cfg, vmc_server **out) {
  if (!cfg || !out || cfg->max_slots <= 0 || cfg->memory_budget <= 0) return VMC_ERR_INVALID_ARGUMENT;
  if (cfg->precision != VMC_FP32 && cfg->precision != VMC_FP64) return VMC_ERR_INVALID_ARGUMENT;
  int s = select_device(cfg->device);
  if (s) return s;
  vmc_server *sv = new vmc_server;
  sv->cfg = *cfg;
  sv->worker = std::thread([sv] { sv->loop(); });
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
  for (auto &kv : s->all) kv.second->buf.reset();
  delete s;
  return VMC_OK;
}

}  // extern "C"
