// server.cpp -- continuous-batching service of RVE solve requests on one GPU.
//
// No counterpart in the reference (one DAMASK_grid process solves one RVE).  Requests
// (grid, microstructure, material, numerics, load case) are queued by any thread;
// one worker thread owns the device and a dgx_batch:
//   * admission: a queued request is admitted, in arrival order, when a batch slot is
//     free and its device footprint (dgx_rve_footprint: fields, constitutive state,
//     NGMRES history, spectra) fits the HBM budget next to the requests already
//     resident;
//   * an admitted request's RVE is created, initialised and added to the batch
//     between two rounds, so its work overlaps with everything already running;
//   * after every round finished members leave the batch, their RVE is freed and
//     their records are handed to the request; the freed memory and slot admit the
//     next requests.
// A request's state stays on the device from admission to completion.  Results do
// not depend on what else is in the batch (a batch member computes what it computes
// alone), so a request gives the same answer at any load.
#include <algorithm>
#include <atomic>
#include <chrono>
#include <condition_variable>
#include <cstdio>
#include <cstring>
#include <deque>
#include <map>
#include <memory>
#include <mutex>
#include <string>
#include <thread>
#include <vector>

#include <cuda_runtime.h>

#include "../../include/dgx.h"

namespace {

struct Req {
  int64_t id = 0;
  int32_t cells[3] = {0, 0, 0};
  double size[3] = {0, 0, 0};
  std::vector<int32_t> material_at;
  std::vector<double> orientations;
  int32_t n_materials = 0;
  dgx_material mat{};
  dgx_numerics num{};
  std::vector<dgx_loadstep> steps;
  std::vector<dgx_inc_record> records;
  int64_t bytes = 0, points = 0;
  // progress
  int32_t state = 0;             // 0 queued, 1 running, 2 done, 3 failed
  int32_t status = 0;
  int32_t n_records = 0;
  double t_submit = 0, t_admit = 0, t_done = 0;
  std::string error;
  dgx_rve* rve = nullptr;
  int32_t slot = -1;
};

}  // namespace

struct dgx_server {
  std::mutex mu;
  std::condition_variable cv_work, cv_done;
  std::deque<std::shared_ptr<Req>> queue;
  std::map<int64_t, std::shared_ptr<Req>> all;
  std::vector<std::shared_ptr<Req>> running;
  int64_t next_id = 1;
  int64_t budget = 0, used = 0;
  int32_t max_active = 0, cons_block = 128;
  std::atomic<bool> stop{false};
  std::thread worker;
  dgx_batch* batch = nullptr;
  std::chrono::steady_clock::time_point t0;
  int device = 0;
  // statistics
  std::atomic<int64_t> rounds{0};
  int64_t completed = 0, failed = 0;
  dgx_status fatal = DGX_OK;
  std::string fatal_msg;

  double now() const { return std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count(); }
  void run();
};

void dgx_server::run() {
  cudaSetDevice(device);
  for (;;) {
    std::vector<std::shared_ptr<Req>> admit;
    {
      std::unique_lock<std::mutex> lk(mu);
      if (running.empty() && !stop.load())
        cv_work.wait(lk, [&] { return stop.load() || !queue.empty(); });
      if (stop.load()) {
        double t = now();
        for (auto& q : queue) { q->state = 3; q->status = DGX_ERR_STATE; q->error = "server stopped"; q->t_done = t; }
        for (auto& q : running) { q->state = 3; q->status = DGX_ERR_STATE; q->error = "server stopped"; q->t_done = t; }
        queue.clear();
        cv_done.notify_all();
        break;                                 // running RVEs are released by dgx_server_destroy
      }
      // admission in arrival order while a slot and memory are free
      int64_t free_b = budget - used;
      int slots = max_active - (int)running.size();
      while (!queue.empty() && slots > 0 && queue.front()->bytes <= free_b) {
        auto r = queue.front();
        queue.pop_front();
        free_b -= r->bytes; used += r->bytes; slots--;
        r->state = 1; r->t_admit = now();
        running.push_back(r);
        admit.push_back(r);
      }
    }
    for (auto& r : admit) {
      dgx_rve* rve = nullptr;
      int32_t slot = -1;
      dgx_status s = dgx_rve_create(r->cells, r->size, r->material_at.data(), r->n_materials, r->orientations.data(),
                                    &r->mat, &r->num, &rve);
      if (s == DGX_OK)
        s = dgx_batch_add(batch, rve, (int32_t)r->steps.size(), r->steps.data(), r->records.data(),
                          (int32_t)r->records.size(), &slot);
      std::lock_guard<std::mutex> lk(mu);
      if (s != DGX_OK) {
        r->state = 3; r->status = s; r->error = dgx_last_error(); r->t_done = now();
        if (rve) dgx_rve_destroy(rve);
        used -= r->bytes;
        running.erase(std::find(running.begin(), running.end(), r));
        failed++;
        cv_done.notify_all();
      } else {
        r->rve = rve; r->slot = slot;
      }
    }
    if (running.empty()) continue;             // only this thread changes `running`
    int32_t n_active = 0;
    dgx_status s = dgx_batch_step(batch, &n_active);
    rounds++;
    if (s != DGX_OK) {                          // a device error ends the service
      std::lock_guard<std::mutex> lk(mu);
      fatal = s; fatal_msg = dgx_last_error();
      double t = now();
      for (auto& r : running) { r->state = 3; r->status = s; r->error = fatal_msg; r->t_done = t; }
      for (auto& r : queue) { r->state = 3; r->status = s; r->error = fatal_msg; r->t_done = t; }
      queue.clear();
      cv_done.notify_all();
      break;
    }
    // retire finished members: free their slot and memory
    struct Fin { std::shared_ptr<Req> r; int32_t nrec, st; };
    std::vector<Fin> fin;
    for (auto& r : running) {
      int32_t done = 0, nrec = 0, st = 0;
      if (dgx_batch_member(batch, r->slot, &done, &nrec, &st) == DGX_OK && done) {
        dgx_batch_remove(batch, r->slot);
        dgx_rve_destroy(r->rve);
        fin.push_back({r, nrec, st});
      }
    }
    if (!fin.empty()) {
      std::lock_guard<std::mutex> lk(mu);
      double t = now();
      for (auto& f : fin) {
        Req& r = *f.r;
        r.rve = nullptr;
        r.n_records = f.nrec; r.status = f.st;
        r.state = f.st == DGX_OK ? 2 : 3;
        if (f.st != DGX_OK) r.error = "solve failed";
        r.t_done = t;
        used -= r.bytes;
        running.erase(std::find(running.begin(), running.end(), f.r));
        if (r.state == 2) completed++; else failed++;
      }
      cv_done.notify_all();
    }
  }
}

extern "C" dgx_status dgx_server_create(int64_t hbm_budget_bytes, int32_t max_active, int32_t cons_block,
                                        dgx_server** out) {
  if (!out || max_active < 1) return DGX_ERR_ARG;
  dgx_server* s = new dgx_server();
  cudaGetDevice(&s->device);
  if (hbm_budget_bytes <= 0) {
    size_t fr = 0, tot = 0;
    if (cudaMemGetInfo(&fr, &tot) != cudaSuccess) { delete s; return DGX_ERR_CUDA; }
    hbm_budget_bytes = (int64_t)(0.85 * (double)fr);
  }
  s->budget = hbm_budget_bytes;
  s->max_active = max_active;
  s->cons_block = cons_block;
  dgx_status st = dgx_batch_create(max_active, cons_block, &s->batch);
  if (st != DGX_OK) { delete s; return st; }
  dgx_batch_set_round_points(s->batch, 1 << 20);
  s->t0 = std::chrono::steady_clock::now();
  s->worker = std::thread([s] { s->run(); });
  *out = s;
  return DGX_OK;
}

extern "C" void dgx_server_destroy(dgx_server* s) {
  if (!s) return;
  {
    std::lock_guard<std::mutex> lk(s->mu);
    s->stop = true;
  }
  s->cv_work.notify_all();
  if (s->worker.joinable()) s->worker.join();
  dgx_batch_destroy(s->batch);                 // detaches members still in it
  for (auto& r : s->running)
    if (r->rve) { dgx_rve_destroy(r->rve); r->rve = nullptr; }
  delete s;
}

extern "C" dgx_status dgx_server_submit(dgx_server* s, const dgx_request* q, int64_t* id) {
  if (!s || !q || !id || !q->material_at || !q->orientations || !q->steps || q->nsteps < 1 || q->n_materials < 1)
    return DGX_ERR_ARG;
  auto r = std::make_shared<Req>();
  for (int i = 0; i < 3; ++i) { r->cells[i] = q->cells[i]; r->size[i] = q->size[i]; }
  int64_t N = (int64_t)q->cells[0] * q->cells[1] * q->cells[2];
  if (N < 1) return DGX_ERR_ARG;
  r->points = N;
  r->material_at.assign(q->material_at, q->material_at + N);
  r->orientations.assign(q->orientations, q->orientations + 4 * (size_t)q->n_materials);
  r->n_materials = q->n_materials;
  r->mat = q->material; r->num = q->numerics;
  r->steps.assign(q->steps, q->steps + q->nsteps);
  int64_t nrec = 0;
  for (auto& st : r->steps) nrec += st.N;
  r->records.resize((size_t)std::max<int64_t>(1, nrec));
  dgx_status st = dgx_rve_footprint(r->cells, &r->num, r->n_materials, &r->bytes);
  if (st != DGX_OK) return st;
  std::lock_guard<std::mutex> lk(s->mu);
  if (s->fatal != DGX_OK) return s->fatal;
  if (r->bytes > s->budget) return DGX_ERR_NOMEM;         // could never be admitted
  r->id = s->next_id++;
  r->t_submit = s->now();
  s->queue.push_back(r);
  s->all[r->id] = r;
  *id = r->id;
  s->cv_work.notify_all();
  return DGX_OK;
}

static void fill_status(const Req& r, dgx_request_status* st) {
  st->state = r.state; st->status = r.status; st->n_records = r.n_records;
  st->t_submit = r.t_submit; st->t_admit = r.t_admit; st->t_done = r.t_done;
  st->device_bytes = r.bytes; st->points = r.points;
  snprintf(st->error, sizeof(st->error), "%s", r.error.c_str());
}

extern "C" dgx_status dgx_server_poll(dgx_server* s, int64_t id, double wait_s, dgx_request_status* st,
                                      dgx_inc_record* records, int32_t max_records) {
  if (!s || !st) return DGX_ERR_ARG;
  std::unique_lock<std::mutex> lk(s->mu);
  auto it = s->all.find(id);
  if (it == s->all.end()) return DGX_ERR_ARG;
  auto r = it->second;
  if (wait_s > 0.0 && r->state < 2)
    s->cv_done.wait_for(lk, std::chrono::duration<double>(wait_s), [&] { return r->state >= 2; });
  fill_status(*r, st);
  if (records && r->state == 2) {
    int n = std::min<int>(r->n_records, max_records);
    std::copy(r->records.begin(), r->records.begin() + n, records);
  }
  return DGX_OK;
}

extern "C" dgx_status dgx_server_release(dgx_server* s, int64_t id) {
  if (!s) return DGX_ERR_ARG;
  std::lock_guard<std::mutex> lk(s->mu);
  auto it = s->all.find(id);
  if (it == s->all.end()) return DGX_ERR_ARG;
  if (it->second->state < 2) return DGX_ERR_STATE;
  s->all.erase(it);
  return DGX_OK;
}

extern "C" dgx_status dgx_server_set_round_points(dgx_server* s, int64_t points) {
  if (!s || points < 0) return DGX_ERR_ARG;
  std::lock_guard<std::mutex> lk(s->mu);         // the worker reads it between rounds
  return dgx_batch_set_round_points(s->batch, points);
}

extern "C" dgx_status dgx_server_stats(dgx_server* s, dgx_server_info* info) {
  if (!s || !info) return DGX_ERR_ARG;
  std::lock_guard<std::mutex> lk(s->mu);
  info->queued = (int32_t)s->queue.size();
  info->running = (int32_t)s->running.size();
  info->completed = s->completed;
  info->failed = s->failed;
  info->rounds = s->rounds.load();
  info->budget_bytes = s->budget;
  info->used_bytes = s->used;
  info->now = s->now();
  info->status = s->fatal;
  return DGX_OK;
}
