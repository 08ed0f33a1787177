// api_server.cu -- EPSGB300Server: a request loop that serves eigenproblems as they arrive (continuous batching).
//
// Clients submit configured EPS objects from any thread.  The loop thread admits queued requests while their byte
// footprint fits the HBM budget, sets them up and loads them into free engine slots while the GPU runs the current
// restart cycle, adds them to the live set between cycles, and retires every solve whose restart loop ended, so a
// request that arrives while others are on the GPU joins them at the next cycle.  Each solve's basis, projected
// matrix and restart state stay in HBM from admission to retirement.  An instance's arithmetic depends only on its
// own problem and the engine's tuning table, so its result is the same alone and in any mix.
#include <chrono>
#include <condition_variable>
#include <deque>
#include <mutex>
#include <thread>
#include <unordered_map>

#include "batch_engine.h"
#include "internal.h"

using namespace ksg;

namespace {

using Clock = std::chrono::steady_clock;

struct Request {
  int state = 0;  // 0 queued, 1 admitted, 2 done
  int err = 0;
  int slot = -1;
  double bytes = 0.0;
  Clock::time_point t_submit, t_admit, t_done;
};

}  // namespace

struct _p_EPSGB300Server {
  BatchEngine B;
  int device = 0;
  double budget = 0.0, in_use = 0.0, peak = 0.0;
  std::mutex m;
  std::condition_variable cv_work, cv_done;
  std::deque<EPS> queue;
  std::unordered_map<EPS, Request> req;
  bool stopping = false;
  bool canceling = false;
  int loop_err = 0;
  long long submitted = 0, completed = 0, failed = 0, max_live = 0;
  long long live_now = 0, cycles_now = 0;  // copies of the engine's counters, under m
  std::thread th;
};

// bytes a request holds while admitted: basis n (ncv+1) 8 plus the operator nnz 12 (CSR values and column indices)
static double request_bytes(EPS e) {
  const double n = e->A ? e->A->m : 0.0, nnz = e->A ? (double)e->A->nnz : 0.0;
  int ncv = e->ncv;
  if (ncv == PETSC_DETERMINE || ncv <= 0) ncv = std::max(2 * e->nev, e->nev + 15);
  return n * (ncv + 1) * 8.0 + nnz * 12.0;
}

static void server_loop(EPSGB300Server S) {
  cudaSetDevice(S->device);
  std::vector<std::pair<int, int>> retired;
  auto fail_all = [&](int err) {
    std::lock_guard<std::mutex> lk(S->m);
    S->loop_err = err;
    for (auto &kv : S->req)
      if (kv.second.state != 2) {
        kv.second.state = 2;
        kv.second.err = err;
        kv.second.t_done = Clock::now();
      }
    S->queue.clear();
    S->cv_done.notify_all();
  };
  for (;;) {
    // 0. cancellation: every queued and live request ends now (the stream is idle between cycles)
    {
      std::unique_lock<std::mutex> lk(S->m);
      if (S->canceling) {
        const auto now = Clock::now();
        for (auto &kv : S->req)
          if (kv.second.state != 2) {
            kv.second.state = 2;
            kv.second.err = PETSC_ERR_ARG_WRONGSTATE;
            kv.second.t_done = now;
            S->failed++;
          }
        S->queue.clear();
        S->in_use = 0.0;
        for (int i : S->B.live) {
          S->B.eps[i] = nullptr;
          S->B.free_slots.push_back(i);
        }
        S->B.live.clear();
        S->B.maps_dirty = true;
        S->canceling = false;
        S->cv_done.notify_all();
      }
    }
    // 1. admission: move queued requests whose footprint fits into free slots
    std::vector<EPS> take;
    {
      std::unique_lock<std::mutex> lk(S->m);
      if (S->B.live.empty() && S->queue.empty()) {
        if (S->stopping) break;
        S->cv_work.wait_for(lk, std::chrono::milliseconds(20));
        continue;
      }
      const size_t slots_free = S->B.free_slots.size();  // engine state: this thread only
      while (!S->queue.empty() && take.size() < slots_free) {
        EPS e = S->queue.front();
        Request &r = S->req[e];
        const bool fits = S->in_use + r.bytes <= S->budget;
        const bool alone = S->B.live.empty() && take.empty();  // a request larger than the budget runs alone
        if (!fits && !alone) break;
        S->queue.pop_front();
        S->in_use += r.bytes;
        S->peak = std::max(S->peak, S->in_use);
        r.state = 1;
        r.t_admit = Clock::now();
        take.push_back(e);
      }
    }
    // 2. the GPU runs the current cycle while the admitted requests are set up on their own streams
    const bool running = !S->B.live.empty();
    if (running) {
      PetscErrorCode ierr = ksg_engine_launch(S->B);
      if (ierr) {
        fail_all(ierr);
        return;
      }
    }
    std::vector<int> new_slots;
    for (EPS e : take) {
      PetscErrorCode ierr = EPSSetUp(e);
      if (!ierr) ierr = ksg_engine_check(e, S->B.max_ld - 1, false);
      int slot = -1;
      if (!ierr) ierr = ksg_engine_admit(S->B, e, &slot);
      std::lock_guard<std::mutex> lk(S->m);
      Request &r = S->req[e];
      if (ierr) {
        r.state = 2;
        r.err = ierr;
        r.t_done = Clock::now();
        S->in_use -= r.bytes;
        S->failed++;
        S->cv_done.notify_all();
      } else {
        r.slot = slot;
        new_slots.push_back(slot);
      }
    }
    // 3. end of the cycle: retire finished solves, then the new requests join the live set
    if (running) {
      retired.clear();
      PetscErrorCode ierr = ksg_engine_finish(S->B, &retired);
      if (ierr) {
        fail_all(ierr);
        return;
      }
      if (!retired.empty()) {
        std::lock_guard<std::mutex> lk(S->m);
        const auto now = Clock::now();
        for (auto &rt : retired) {
          for (auto &kv : S->req) {
            Request &r = kv.second;
            if (r.state == 1 && r.slot == rt.first) {
              r.state = 2;
              r.err = rt.second;
              r.t_done = now;
              kv.first->stats.solve_seconds = std::chrono::duration<double>(now - r.t_submit).count();
              S->in_use -= r.bytes;
              if (rt.second) S->failed++;
              else S->completed++;
              break;
            }
          }
        }
        S->cv_done.notify_all();
      }
    }
    if (!new_slots.empty()) ksg_engine_activate(S->B, new_slots);
    {
      std::lock_guard<std::mutex> lk(S->m);
      S->live_now = (long long)S->B.live.size();
      S->cycles_now = S->B.cycles;
      S->max_live = std::max(S->max_live, S->live_now);
    }
  }
}

extern "C" PetscErrorCode EPSGB300ServerCreate(double hbm_budget_bytes, PetscInt max_requests, PetscInt max_ncv,
                                               EPSGB300Server *server) {
  KSG_CHECK(server, PETSC_ERR_ARG_NULL, "Null argument");
  KSG_CHECK(hbm_budget_bytes > 0.0, PETSC_ERR_ARG_OUTOFRANGE, "The HBM budget must be positive");
  KSG_CHECK(max_requests >= 1, PETSC_ERR_ARG_OUTOFRANGE, "max_requests must be at least 1");
  EPSGB300Server S = new _p_EPSGB300Server();
  KSG_CUDA(cudaGetDevice(&S->device));
  S->budget = hbm_budget_bytes;
  PetscErrorCode ierr = ksg_engine_init(S->B, S->device, (int)max_requests, (int)max_ncv);
  if (ierr) {
    delete S;
    return ierr;
  }
  S->th = std::thread(server_loop, S);
  *server = S;
  return 0;
}

extern "C" PetscErrorCode EPSGB300ServerSubmit(EPSGB300Server S, EPS eps) {
  KSG_CHECK(S && eps, PETSC_ERR_ARG_NULL, "Null argument");
  KSG_CHECK(eps->A, PETSC_ERR_ORDER, "EPSSetOperators must be called before submitting");
  std::lock_guard<std::mutex> lk(S->m);
  KSG_CHECK(!S->stopping, PETSC_ERR_ORDER, "The server is shutting down");
  KSG_CHECK(!S->loop_err, S->loop_err, "The server stopped after an error");
  auto it = S->req.find(eps);
  KSG_CHECK(it == S->req.end() || it->second.state == 2, PETSC_ERR_ARG_WRONGSTATE, "This EPS is already in flight");
  Request r;
  r.bytes = request_bytes(eps);
  r.t_submit = Clock::now();
  S->req[eps] = r;
  S->queue.push_back(eps);
  S->submitted++;
  S->cv_work.notify_one();
  return 0;
}

extern "C" PetscErrorCode EPSGB300ServerWait(EPSGB300Server S, EPS eps, double timeout_seconds, PetscBool *done) {
  KSG_CHECK(S && eps, PETSC_ERR_ARG_NULL, "Null argument");
  std::unique_lock<std::mutex> lk(S->m);
  auto it = S->req.find(eps);
  KSG_CHECK(it != S->req.end(), PETSC_ERR_ARG_WRONG, "This EPS was not submitted to this server");
  auto pred = [&] { return S->req[eps].state == 2; };
  if (timeout_seconds < 0) S->cv_done.wait(lk, pred);
  else S->cv_done.wait_for(lk, std::chrono::duration<double>(timeout_seconds), pred);
  const Request r = S->req[eps];
  if (done) *done = r.state == 2 ? PETSC_TRUE : PETSC_FALSE;
  if (r.state == 2) {
    S->req.erase(eps);
    KSG_CHECK(!r.err, r.err, "The served solve failed (error %d)", r.err);
  }
  return 0;
}

extern "C" PetscErrorCode EPSGB300ServerGetStats(EPSGB300Server S, EPSGB300ServerStats *st) {
  KSG_CHECK(S && st, PETSC_ERR_ARG_NULL, "Null argument");
  std::lock_guard<std::mutex> lk(S->m);
  st->submitted = S->submitted;
  st->completed = S->completed;
  st->failed = S->failed;
  st->queued = (long long)S->queue.size();
  st->live = S->live_now;
  st->max_live = S->max_live;
  st->cycles = S->cycles_now;
  st->bytes_in_use = S->in_use;
  st->peak_bytes = S->peak;
  return 0;
}

extern "C" PetscErrorCode EPSGB300ServerCancel(EPSGB300Server S) {
  KSG_CHECK(S, PETSC_ERR_ARG_NULL, "Null argument");
  std::lock_guard<std::mutex> lk(S->m);
  S->canceling = true;
  S->cv_work.notify_all();
  return 0;
}

extern "C" PetscErrorCode EPSGB300ServerDestroy(EPSGB300Server *server) {
  if (!server || !*server) return 0;
  EPSGB300Server S = *server;
  {
    std::lock_guard<std::mutex> lk(S->m);
    S->stopping = true;
    S->cv_work.notify_all();
  }
  if (S->th.joinable()) S->th.join();  // the loop drains every submitted request first
  const int err = S->loop_err;
  delete S;
  *server = nullptr;
  KSG_CHECK(!err, err, "The server loop stopped after an error");
  return 0;
}
