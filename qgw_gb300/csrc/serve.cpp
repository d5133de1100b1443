// serve.cpp -- continuous batching of qgw runs on one GPU.
//
// Requests (a parameter set, an initial q, a precision and a step count)
// are queued by any host thread.  One worker thread owns the GPU work:
//   1. admission: queued requests are admitted in arrival order while their
//      device footprint fits the HBM budget; an admitted request becomes a
//      resident run (its state stays on the device until it finishes);
//   2. a tick: every resident run advances by up to `steps_per_tick` steps,
//      FP64 runs in one batch and FP32-compensated runs in another, each
//      batch one launch per step stage, the two batches on separate streams
//      so that their work overlaps on the device;
//   3. retirement: runs that reached their step count are copied out, their
//      device memory released, and the next admission pass sees the freed
//      budget -- requests that arrive while others run join at the next tick.
// A run's arithmetic does not depend on its batch (see ensemble.cu), so a
// request gives bitwise the same result alone and in the mix.
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <map>
#include <memory>
#include <mutex>
#include <thread>
#include <vector>

#include "../../include/qgw_gpu.h"
#include "ensemble_core.h"
#include "run.h"

namespace {

using Clock = std::chrono::steady_clock;

struct Request {
  long long id = 0;
  qgw_params p{};
  int precision = 0;
  int nsteps = 0;
  std::vector<double> q0;
  size_t footprint = 0;
  Clock::time_point t_submit, t_admit, t_done;
  // while resident
  qgw_run* run = nullptr;
  int remaining = 0;
  // result
  int status = QGW_ERR_NOT_READY;
  std::vector<double> psi, q;
  qgw_time time{};
};

}  // namespace

struct qgw_pool {
  int device = 0;
  size_t budget = 0, used = 0;
  int steps_per_tick = 32;
  std::mutex mu;
  std::condition_variable cv, done_cv;
  std::deque<std::shared_ptr<Request>> queue;
  std::map<long long, std::shared_ptr<Request>> all;
  std::vector<std::shared_ptr<Request>> resident;
  long long next_id = 1;
  bool stop = false;
  std::thread worker;
  // batch b: precision b % 2 (0 FP64, 1 FP32c), boundary b / 2 (0 closed, 1 periodic)
  qgw::EnsembleCore batch[4];
  // statistics
  long long completed = 0, admitted = 0, ticks = 0;
  double lgp_steps = 0;
  int max_resident = 0;
};

namespace {

size_t lgp_of(const qgw_params& p) {
  const size_t cut = p.bc_fac == -1 ? 0 : 1;  // a closed basin has NX-1 interior points
  return (p.NX - cut) * (p.NY - cut) * (size_t)p.nl;
}

int batch_of(const qgw_params& p, int precision) { return (precision == QGW_FP64 ? 0 : 1) + (p.bc_fac == -1 ? 2 : 0); }

int admit_one(qgw_pool* pl, const std::shared_ptr<Request>& r) {
  qgw_run* run = nullptr;
  int rc = qgw_create(&r->p, nullptr, nullptr, nullptr, nullptr, r->precision, &run);
  if (rc) return rc;
  // the pool batches runs through the ensemble kernels, which hold the
  // half-length transforms only (odd or prime-sized grids run alone)
  const bool blue = r->precision == QGW_FP64 ? (run->a64.gx.blue || run->a64.gy.blue)
                                             : (run->a32.gx.blue || run->a32.gy.blue);
  if (blue) {
    qgw_destroy(run);
    return QGW_ERR_UNSUPPORTED;
  }
  if ((rc = qgw_set_q(run, r->q0.data()))) {
    qgw_destroy(run);
    return rc;
  }
  r->q0.clear();
  r->q0.shrink_to_fit();
  r->run = run;
  r->remaining = r->nsteps;
  r->t_admit = Clock::now();
  return QGW_OK;
}

void rebuild(qgw_pool* pl) {
  for (int b = 0; b < 4; ++b) {
    qgw::EnsembleCore& e = pl->batch[b];
    e.members.clear();
    for (auto& r : pl->resident)
      if (batch_of(r->p, r->precision) == b) e.members.push_back(r->run);
    qgw::ens_core_build(&e);
  }
}

void retire(qgw_pool* pl, const std::shared_ptr<Request>& r, int status) {
  const size_t ring = r->p.bc_fac == -1 ? 2 : 1;  // interior + ghost ring
  const size_t n3 = (size_t)r->p.nl * (r->p.NY + ring) * (r->p.NX + ring);
  if (status == QGW_OK) {
    r->psi.resize(n3);
    r->q.resize(n3);
    status = qgw_get(r->run, r->psi.data(), r->q.data());
    qgw_get_time(r->run, &r->time);
  }
  qgw_destroy(r->run);
  r->run = nullptr;
  r->t_done = Clock::now();
  std::lock_guard<std::mutex> lk(pl->mu);
  r->status = status;
  pl->used -= r->footprint;
  pl->completed += 1;
  pl->done_cv.notify_all();
}

void worker_loop(qgw_pool* pl) {
  cudaSetDevice(pl->device);
  for (int b = 0; b < 4; ++b) {
    cudaStreamCreateWithFlags(&pl->batch[b].stream, cudaStreamNonBlocking);
    cudaDeviceGetAttribute(&pl->batch[b].nsm, cudaDevAttrMultiProcessorCount, pl->device);
    pl->batch[b].precision = b % 2 == 0 ? QGW_FP64 : QGW_FP32C;
    pl->batch[b].periodic = b / 2;
  }
  for (;;) {
    // admission, in arrival order, by footprint
    std::vector<std::shared_ptr<Request>> admit;
    {
      std::unique_lock<std::mutex> lk(pl->mu);
      pl->cv.wait(lk, [&] { return pl->stop || !pl->queue.empty() || !pl->resident.empty(); });
      if (pl->stop && pl->resident.empty()) break;
      while (!pl->queue.empty() && pl->used + pl->queue.front()->footprint <= pl->budget) {
        pl->used += pl->queue.front()->footprint;
        admit.push_back(pl->queue.front());
        pl->queue.pop_front();
      }
      // a request larger than the whole budget can never run
      if (pl->resident.empty() && admit.empty() && !pl->queue.empty() &&
          pl->queue.front()->footprint > pl->budget) {
        auto r = pl->queue.front();
        pl->queue.pop_front();
        r->status = QGW_ERR_ADMISSION;
        r->t_done = Clock::now();
        pl->completed += 1;
        pl->done_cv.notify_all();
        continue;
      }
    }
    bool changed = false;
    for (auto& r : admit) {
      const int rc = admit_one(pl, r);
      if (rc) {
        std::lock_guard<std::mutex> lk(pl->mu);
        r->status = rc;
        r->t_done = Clock::now();
        pl->used -= r->footprint;
        pl->completed += 1;
        pl->done_cv.notify_all();
        continue;
      }
      pl->resident.push_back(r);
      pl->admitted += 1;
      changed = true;
    }
    if (changed) rebuild(pl);
    if (pl->resident.empty()) continue;
    pl->max_resident = std::max(pl->max_resident, (int)pl->resident.size());
    // one tick: every batch enqueued (own stream) before any is waited on
    std::vector<int> caps[4];
    for (int b = 0; b < 4; ++b) {
      qgw::EnsembleCore& e = pl->batch[b];
      if (e.members.empty()) continue;
      for (qgw_run* run : e.members)
        for (auto& r : pl->resident)
          if (r->run == run) caps[b].push_back(std::min(r->remaining, pl->steps_per_tick));
      qgw::ens_core_step(&e, pl->steps_per_tick, caps[b].data(), false);
    }
    std::vector<std::shared_ptr<Request>> finished;
    for (int b = 0; b < 4; ++b) {
      qgw::EnsembleCore& e = pl->batch[b];
      if (e.members.empty()) continue;
      qgw::ens_core_finish(&e);
      for (size_t i = 0; i < e.members.size(); ++i)
        for (auto& r : pl->resident)
          if (r->run == e.members[i]) {
            const qgw::DevState& st = e.h_states[i];
            r->remaining -= st.steps_taken;
            pl->lgp_steps += (double)lgp_of(r->p) * st.steps_taken;
            if (st.nonfinite) r->remaining = -1;
            if (st.dev_error) r->remaining = -2;  // a bounded device wait ran out
            if (r->remaining <= 0) finished.push_back(r);
          }
    }
    pl->ticks += 1;
    if (!finished.empty()) {
      for (auto& r : finished) {
        retire(pl, r, r->remaining == -2 ? QGW_ERR_TIMEOUT : (r->remaining < 0 ? QGW_ERR_NAN : QGW_OK));
        pl->resident.erase(std::find(pl->resident.begin(), pl->resident.end(), r));
      }
      rebuild(pl);
    }
  }
  for (int b = 0; b < 4; ++b) {
    qgw::ens_core_free_tables(&pl->batch[b]);
    if (pl->batch[b].stream) cudaStreamDestroy(pl->batch[b].stream);
  }
}

}  // namespace

extern "C" {

int qgw_pool_create(size_t hbm_budget_bytes, int steps_per_tick, qgw_pool** out) {
  if (!out || steps_per_tick < 1) return QGW_ERR_PARAM;
  qgw_pool* pl = new qgw_pool();
  if (cudaGetDevice(&pl->device) != cudaSuccess) {
    delete pl;
    return QGW_ERR_CUDA;
  }
  if (hbm_budget_bytes == 0) {
    size_t freeb = 0, total = 0;
    cudaMemGetInfo(&freeb, &total);
    hbm_budget_bytes = freeb / 10 * 8;
  }
  pl->budget = hbm_budget_bytes;
  pl->steps_per_tick = steps_per_tick;
  pl->worker = std::thread(worker_loop, pl);
  *out = pl;
  return QGW_OK;
}

int qgw_pool_submit(qgw_pool* pl, const qgw_params* p, const double* q0, int precision, int nsteps,
                    long long* id) {
  if (!pl || !p || !q0 || !id || nsteps < 1) return QGW_ERR_PARAM;
  auto r = std::make_shared<Request>();
  r->p = *p;
  r->precision = precision;
  r->nsteps = nsteps;
  const size_t ring = p->bc_fac == -1 ? 2 : 1;  // interior + ghost ring
  const size_t n3 = (size_t)p->nl * (p->NY + ring) * (p->NX + ring);
  r->q0.assign(q0, q0 + n3);
  int rc = qgw_footprint(p, precision, &r->footprint);
  if (rc) return rc;
  r->t_submit = Clock::now();
  std::lock_guard<std::mutex> lk(pl->mu);
  r->id = pl->next_id++;
  pl->all[r->id] = r;
  pl->queue.push_back(r);
  *id = r->id;
  pl->cv.notify_all();
  return QGW_OK;
}

// QGW_OK when done (the request's own status is in *status), or
// QGW_ERR_NOT_READY; wait_ms > 0 blocks up to that long.
int qgw_pool_poll(qgw_pool* pl, long long id, int wait_ms, int* status) {
  if (!pl) return QGW_ERR_PARAM;
  std::unique_lock<std::mutex> lk(pl->mu);
  auto it = pl->all.find(id);
  if (it == pl->all.end()) return QGW_ERR_PARAM;
  auto r = it->second;
  if (r->status == QGW_ERR_NOT_READY && wait_ms > 0)
    pl->done_cv.wait_for(lk, std::chrono::milliseconds(wait_ms), [&] { return r->status != QGW_ERR_NOT_READY; });
  if (r->status == QGW_ERR_NOT_READY) return QGW_ERR_NOT_READY;
  if (status) *status = r->status;
  return QGW_OK;
}

// Copy a finished request out (reference layout) and forget it.  latency
// [3]: seconds from submit to admission, from admission to completion, and
// from submit to completion.
int qgw_pool_fetch(qgw_pool* pl, long long id, double* psi, double* q, qgw_time* tm, double* latency) {
  if (!pl) return QGW_ERR_PARAM;
  std::shared_ptr<Request> r;
  {
    std::lock_guard<std::mutex> lk(pl->mu);
    auto it = pl->all.find(id);
    if (it == pl->all.end()) return QGW_ERR_PARAM;
    r = it->second;
    if (r->status == QGW_ERR_NOT_READY) return QGW_ERR_NOT_READY;
    pl->all.erase(it);
  }
  if (r->status != QGW_OK) return r->status;
  if (psi) std::memcpy(psi, r->psi.data(), sizeof(double) * r->psi.size());
  if (q) std::memcpy(q, r->q.data(), sizeof(double) * r->q.size());
  if (tm) *tm = r->time;
  if (latency) {
    using S = std::chrono::duration<double>;
    latency[0] = S(r->t_admit - r->t_submit).count();
    latency[1] = S(r->t_done - r->t_admit).count();
    latency[2] = S(r->t_done - r->t_submit).count();
  }
  return QGW_OK;
}

// stats[6]: completed, admitted, ticks, max resident, lgp-steps done,
// bytes in use
int qgw_pool_stats(qgw_pool* pl, double* stats) {
  if (!pl || !stats) return QGW_ERR_PARAM;
  std::lock_guard<std::mutex> lk(pl->mu);
  stats[0] = (double)pl->completed;
  stats[1] = (double)pl->admitted;
  stats[2] = (double)pl->ticks;
  stats[3] = (double)pl->max_resident;
  stats[4] = pl->lgp_steps;
  stats[5] = (double)pl->used;
  return QGW_OK;
}

void qgw_pool_destroy(qgw_pool* pl) {
  if (!pl) return;
  {
    std::lock_guard<std::mutex> lk(pl->mu);
    pl->stop = true;
    pl->queue.clear();
    pl->cv.notify_all();
  }
  // resident runs finish their remaining steps before the worker exits
  if (pl->worker.joinable()) pl->worker.join();
  delete pl;
}

}  // extern "C"
