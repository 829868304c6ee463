// Serving loop: continuous batching of simulation jobs on one GPU.
//
// One worker thread owns a context. Each turn it
//   1. admits pending jobs in arrival order while the context's resident
//      bytes plus the job's footprint fit the HBM budget (a job that does not
//      fit waits; nothing behind it overtakes it);
//   2. creates, uploads and initialises the admitted jobs' scenes (their state
//      stays resident until they finish);
//   3. picks the admitted jobs that step in this chunk (all of them, or --
//      with a particle cap -- the first ones in arrival order or by least
//      remaining work, SRPT) and advances them together with snow_batch_step
//      by k = min(chunk, fewest remaining steps) steps -- one launch per
//      phase for all of them, CUDA graphs per batch composition; jobs left
//      out keep their state resident and wait;
//   4. retires finished jobs (bulk statistics, optional final state), which
//      frees their memory for the next admissions.
// Jobs that arrive while others run join at the next chunk boundary, so their
// work overlaps on the device with the jobs already running.
#include <algorithm>
#include <chrono>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <map>
#include <mutex>
#include <thread>
#include <vector>

#include "../../include/snow_mpm.h"

namespace {

double now_s() {
  using namespace std::chrono;
  return duration<double>(steady_clock::now().time_since_epoch()).count();
}

struct Job {
  uint64_t id = 0;
  snow_params p{};
  std::vector<snow_collider> coll;
  std::vector<float> x, v, m;
  size_t n = 0;
  int steps = 0, left = 0;
  double dt = 1e-3;
  bool keep = false;
  size_t footprint = 0;
  double t_arrive = 0, t_admit = 0, t_done = 0;
  snow_scene* scene = nullptr;
  snow_job_result result{};
  std::vector<float> out_x, out_v, out_fe, out_jp;
};

}  // namespace

struct snow_server {
  snow_server_config cfg{};
  std::mutex mu;
  std::condition_variable cv;
  std::deque<Job*> pending;
  std::deque<Job*> done;
  std::map<uint64_t, Job*> kept;
  std::thread worker;
  bool stop = false;
  uint64_t next_id = 1;
  snow_server_report st{};
  double t_start = 0;
  snow_status init_status = SNOW_OK;
  bool ready = false;
};

namespace {

void finish(snow_server* srv, Job* j, snow_status status) {
  j->t_done = now_s();
  j->result.id = j->id;
  j->result.status = status;
  j->result.n = j->n;
  j->result.steps = j->steps;
  j->result.queue_s = j->t_admit > 0 ? j->t_admit - j->t_arrive : j->t_done - j->t_arrive;
  j->result.service_s = j->t_admit > 0 ? j->t_done - j->t_admit : 0.0;
  j->result.latency_s = j->t_done - j->t_arrive;
  std::lock_guard<std::mutex> lock(srv->mu);
  if (status == SNOW_OK) {
    srv->st.completed++;
    srv->st.particle_steps += (double)j->n * (double)j->steps;
  } else {
    srv->st.failed++;
  }
  srv->done.push_back(j);
  srv->cv.notify_all();
}

void run(snow_server* srv) {
  snow_ctx* ctx = nullptr;
  snow_status s0 = snow_ctx_create(srv->cfg.device, srv->cfg.hbm_budget_bytes, &ctx);
  {
    std::lock_guard<std::mutex> lock(srv->mu);
    srv->init_status = s0;
    srv->ready = true;
  }
  srv->cv.notify_all();
  if (s0 != SNOW_OK) return;
  const int max_resident = srv->cfg.max_active > 0 ? srv->cfg.max_active : 256;
  const int chunk = srv->cfg.chunk_steps > 0 ? srv->cfg.chunk_steps : 16;
  const size_t budget = srv->cfg.hbm_budget_bytes;
  const size_t cap = srv->cfg.max_active_particles;
  const bool srpt = srv->cfg.policy == SNOW_SERVE_SRPT;
  std::vector<Job*> resident;  // admitted, state on the device
  std::vector<Job*> running;   // the members of `batch`
  snow_batch* batch = nullptr;
  double busy_since = -1.0;
  for (;;) {
    // ---- admission (arrival order, HBM budget) ---------------------------
    std::vector<Job*> admit;
    {
      std::unique_lock<std::mutex> lock(srv->mu);
      if (resident.empty() && srv->pending.empty()) {
        if (srv->stop) break;
        srv->cv.wait_for(lock, std::chrono::milliseconds(2));
        continue;
      }
      size_t used = snow_ctx_bytes_in_use(ctx);
      while (!srv->pending.empty() && (int)(resident.size() + admit.size()) < max_resident) {
        Job* j = srv->pending.front();
        if (budget && used + j->footprint > budget) {
          if (!resident.empty() || !admit.empty()) break;  // wait for memory to free up
          if (j->footprint > budget) {                      // can never fit
            srv->pending.pop_front();
            srv->st.pending = srv->pending.size();
            lock.unlock();
            finish(srv, j, SNOW_EBUDGET);
            lock.lock();
            continue;
          }
        }
        srv->pending.pop_front();
        used += j->footprint;
        admit.push_back(j);
      }
      srv->st.pending = srv->pending.size();
    }
    for (Job* j : admit) {
      j->t_admit = now_s();
      snow_status s = snow_scene_create(ctx, &j->p, j->coll.data(), (int)j->coll.size(), j->n, &j->scene);
      if (s == SNOW_OK) s = snow_scene_upload(j->scene, j->x.data(), j->v.data(), j->m.data(), nullptr, nullptr, j->n);
      if (s == SNOW_OK) s = snow_scene_init(j->scene);
      if (s != SNOW_OK) {
        if (j->scene) snow_scene_destroy(j->scene);
        j->scene = nullptr;
        finish(srv, j, s);
        continue;
      }
      std::vector<float>().swap(j->x);  // the device holds the state now
      std::vector<float>().swap(j->v);
      std::vector<float>().swap(j->m);
      resident.push_back(j);
      std::lock_guard<std::mutex> lock(srv->mu);
      srv->st.admitted++;
    }
    {
      std::lock_guard<std::mutex> lock(srv->mu);
      srv->st.active = resident.size();
      srv->st.resident_bytes = snow_ctx_bytes_in_use(ctx);
    }
    if (resident.empty()) continue;
    if (busy_since < 0) busy_since = now_s();
    // ---- which resident jobs step in this chunk --------------------------
    // FIFO: arrival order; SRPT: least remaining particle-steps first. Jobs
    // are added until the particle cap is reached (at least one job).
    std::vector<Job*> order = resident;
    if (srpt)
      std::stable_sort(order.begin(), order.end(), [](const Job* a, const Job* b) {
        return (double)a->left * a->n < (double)b->left * b->n;
      });
    std::vector<Job*> pick;
    size_t parts = 0;
    for (Job* j : order) {
      if (cap && !pick.empty() && parts + j->n > cap) continue;
      pick.push_back(j);
      parts += j->n;
    }
    if (pick != running || !batch) {
      if (batch) snow_batch_destroy(batch);
      batch = nullptr;
      std::vector<snow_scene*> sc;
      for (Job* j : pick) sc.push_back(j->scene);
      snow_status s = snow_batch_create(ctx, sc.data(), (int)sc.size(), &batch);
      if (s != SNOW_OK) {
        for (Job* j : pick) {
          snow_scene_destroy(j->scene);
          j->scene = nullptr;
          finish(srv, j, s);
        }
        std::vector<Job*> keep;
        for (Job* j : resident)
          if (j->scene) keep.push_back(j);
        resident.swap(keep);
        running.clear();
        continue;
      }
      running = pick;
    }
    // ---- one chunk of batched steps -------------------------------------
    int k = chunk;
    std::vector<double> dts;
    for (Job* j : running) {
      k = std::min(k, j->left);
      dts.push_back(j->dt);
    }
    snow_status s = snow_batch_step(batch, dts.data(), k);
    if (s == SNOW_OK) s = snow_ctx_synchronize(ctx);
    bool retired = false;
    for (Job* j : running) {
      j->left -= (s == SNOW_OK) ? k : j->left;
      if (j->left > 0) continue;
      snow_status js = s;
      if (js == SNOW_OK) js = snow_scene_stats(j->scene, &j->result.stats);
      if (js == SNOW_OK && j->result.stats.nonfinite) js = SNOW_ENUMERIC;
      if (js == SNOW_OK && j->keep) {
        j->out_x.resize(3 * j->n);
        j->out_v.resize(3 * j->n);
        j->out_fe.resize(9 * j->n);
        j->out_jp.resize(j->n);
        js = snow_scene_download(j->scene, j->out_x.data(), j->out_v.data(), j->out_fe.data(), nullptr,
                                 j->out_jp.data(), nullptr);
      }
      if (batch) {  // the batch holds the scene: release it first
        snow_batch_destroy(batch);
        batch = nullptr;
      }
      snow_scene_destroy(j->scene);
      j->scene = nullptr;
      retired = true;
      finish(srv, j, js);
    }
    if (retired) {
      std::vector<Job*> keep;
      for (Job* j : resident)
        if (j->scene) keep.push_back(j);
      resident.swap(keep);
      running.clear();
    }
    if (resident.empty() && busy_since >= 0) {
      std::lock_guard<std::mutex> lock(srv->mu);
      srv->st.busy_s += now_s() - busy_since;
      busy_since = -1.0;
    }
  }
  if (batch) snow_batch_destroy(batch);
  snow_ctx_destroy(ctx);
}

// The scene's bound plus its entries in the batch tables (a scene descriptor
// and four prefix words), rounded up.
size_t footprint_of(const snow_params& p, size_t n) {
  const size_t f = snow_scene_footprint(&p, n);
  return f ? f + 4096 : 0;
}

}  // namespace

extern "C" {

snow_status snow_server_create(const snow_server_config* cfg, snow_server** out) {
  if (!cfg || !out) return SNOW_EINVAL;
  *out = nullptr;
  snow_server* srv = new snow_server();
  srv->cfg = *cfg;
  srv->t_start = now_s();
  srv->worker = std::thread(run, srv);
  std::unique_lock<std::mutex> lock(srv->mu);
  srv->cv.wait(lock, [&] { return srv->ready; });
  const snow_status s = srv->init_status;
  lock.unlock();
  if (s != SNOW_OK) {
    srv->worker.join();
    delete srv;
    return s;
  }
  *out = srv;
  return SNOW_OK;
}

void snow_server_destroy(snow_server* srv) {
  if (!srv) return;
  {
    std::lock_guard<std::mutex> lock(srv->mu);
    srv->stop = true;
    for (Job* j : srv->pending) delete j;
    srv->pending.clear();
  }
  srv->cv.notify_all();
  if (srv->worker.joinable()) srv->worker.join();
  for (Job* j : srv->done) delete j;
  for (auto& kv : srv->kept) delete kv.second;
  delete srv;
}

snow_status snow_server_submit(snow_server* srv, const snow_job_desc* d, uint64_t* id) {
  if (!srv || !d || !d->params || !d->x || !d->v || !d->m || d->n == 0 || d->steps <= 0 || !(d->dt > 0.0) ||
      d->n_colliders < 0 || (d->n_colliders > 0 && !d->colliders))
    return SNOW_EINVAL;
  Job* j = new Job();
  j->p = *d->params;
  j->p.mode = SNOW_MODE_FAST;
  j->coll.assign(d->colliders, d->colliders + d->n_colliders);
  j->x.assign(d->x, d->x + 3 * d->n);
  j->v.assign(d->v, d->v + 3 * d->n);
  j->m.assign(d->m, d->m + d->n);
  j->n = d->n;
  j->steps = j->left = d->steps;
  j->dt = d->dt;
  j->keep = d->keep_state != 0;
  j->footprint = footprint_of(j->p, j->n);
  if (j->footprint == 0) {
    delete j;
    return SNOW_EINVAL;
  }
  {
    std::lock_guard<std::mutex> lock(srv->mu);
    j->id = srv->next_id++;
    j->t_arrive = now_s();
    srv->pending.push_back(j);
    srv->st.submitted++;
    srv->st.pending = srv->pending.size();
  }
  srv->cv.notify_all();
  if (id) *id = j->id;
  return SNOW_OK;
}

snow_status snow_server_poll(snow_server* srv, snow_job_result* out, int max, int* n_out) {
  if (!srv || (!out && max > 0) || !n_out) return SNOW_EINVAL;
  std::lock_guard<std::mutex> lock(srv->mu);
  int k = 0;
  while (k < max && !srv->done.empty()) {
    Job* j = srv->done.front();
    srv->done.pop_front();
    out[k++] = j->result;
    if (j->keep && j->result.status == SNOW_OK)
      srv->kept[j->id] = j;
    else
      delete j;
  }
  *n_out = k;
  return SNOW_OK;
}

snow_status snow_server_fetch(snow_server* srv, uint64_t id, float* x, float* v, float* FE, float* Jp) {
  if (!srv) return SNOW_EINVAL;
  Job* j = nullptr;
  {
    std::lock_guard<std::mutex> lock(srv->mu);
    auto it = srv->kept.find(id);
    if (it == srv->kept.end()) return SNOW_EINVAL;
    j = it->second;
    srv->kept.erase(it);
  }
  if (x) std::memcpy(x, j->out_x.data(), j->out_x.size() * sizeof(float));
  if (v) std::memcpy(v, j->out_v.data(), j->out_v.size() * sizeof(float));
  if (FE) std::memcpy(FE, j->out_fe.data(), j->out_fe.size() * sizeof(float));
  if (Jp) std::memcpy(Jp, j->out_jp.data(), j->out_jp.size() * sizeof(float));
  delete j;
  return SNOW_OK;
}

snow_status snow_server_stats(snow_server* srv, snow_server_report* out) {
  if (!srv || !out) return SNOW_EINVAL;
  std::lock_guard<std::mutex> lock(srv->mu);
  *out = srv->st;
  out->uptime_s = now_s() - srv->t_start;
  return SNOW_OK;
}

snow_status snow_server_drain(snow_server* srv, double timeout_s) {
  if (!srv) return SNOW_EINVAL;
  const double until = now_s() + timeout_s;
  std::unique_lock<std::mutex> lock(srv->mu);
  while (srv->st.completed + srv->st.failed < srv->st.submitted) {
    if (now_s() >= until) return SNOW_ETIMEDOUT;
    srv->cv.wait_for(lock, std::chrono::milliseconds(5));
  }
  return SNOW_OK;
}

}  // extern "C"
