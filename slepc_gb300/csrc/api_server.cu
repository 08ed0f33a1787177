// api_server.cu -- EPSGB300Server: a request loop that serves eigenproblems as they arrive (continuous batching).
//
// Clients submit configured EPS objects from any thread.  Requests are routed by footprint to one of two lanes,
// small and large problems, each with its own batched engine, CUDA graph, stream and loop thread: a restart cycle
// lasts as long as its longest Krylov segment, so small solves that shared a cycle with large ones would wait for
// them at every restart.  The lanes share the GPU and one HBM budget.  A lane's loop admits its queued requests while
// their byte footprint fits the budget, sets them up and loads them into free engine slots while the GPU runs the
// lane's current restart cycle, adds them to the live set between cycles, and retires every solve whose restart loop
// ended, so a request that arrives while others are on the GPU joins them at the next cycle.  Each solve's basis,
// projected matrix and restart state stay in HBM from admission to retirement.  An instance's arithmetic depends
// only on its own problem and the engine's tuning table, so its result is the same alone, in either lane and in
// any mix.
#include <chrono>
#include <climits>
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
  int lane = 0;
  double bytes = 0.0;
  Clock::time_point t_submit, t_admit, t_done;
};

// requests whose footprint (basis and operator bytes) is at most this go to the small-problem lane
constexpr double SMALL_LANE_BYTES = 64.0 * 1024 * 1024;
constexpr int LANES = 2;

struct Lane {
  BatchEngine B;
  std::deque<EPS> queue;
  std::thread th;
  bool canceling = false;
  double reserve = 0.0;                    // footprint of the queue head while the budget holds it back
  long long reserve_seq = 0;               // order in which the reservations were made
  long long live_now = 0, cycles_now = 0;  // copies of the engine's counters, under the server mutex
};

}  // namespace

struct _p_EPSGB300Server {
  Lane lane[LANES];
  int device = 0;
  double budget = 0.0, in_use = 0.0, peak = 0.0;
  std::mutex m;
  std::condition_variable cv_work, cv_done;
  std::unordered_map<EPS, Request> req;
  bool stopping = false;
  int loop_err = 0;
  long long reserve_seq = 0;
  long long submitted = 0, completed = 0, failed = 0, max_live = 0;
};

// bytes a request holds while admitted: basis n (ncv+1) 8 plus the operator nnz 12 (CSR values and column indices)
static double request_bytes(EPS e) {
  const double n = e->A ? e->A->m : 0.0, nnz = e->A ? (double)e->A->nnz : 0.0;
  int ncv = e->ncv;
  if (ncv == PETSC_DETERMINE || ncv <= 0) ncv = std::max(2 * e->nev, e->nev + 15);
  return n * (ncv + 1) * 8.0 + nnz * 12.0;
}

// One lane's loop.  The engine (slots, live set, graph, stream) belongs to this thread; the queue, the request
// table and the budget are shared and read or written under the server mutex.
static void server_loop(EPSGB300Server S, int li) {
  cudaSetDevice(S->device);
  Lane &L = S->lane[li];
  BatchEngine &B = L.B;
  std::vector<std::pair<int, int>> retired;
  auto fail_all = [&](int err) {
    std::lock_guard<std::mutex> lk(S->m);
    S->loop_err = err;
    for (auto &kv : S->req)
      if (kv.second.state != 2 && kv.second.lane == li) {
        kv.second.state = 2;
        kv.second.err = err;
        kv.second.t_done = Clock::now();
      }
    L.queue.clear();
    L.reserve = 0.0;
    S->cv_done.notify_all();
  };
  for (;;) {
    // 0. cancellation: every queued and live request of the lane ends now (the stream is idle between cycles)
    {
      std::unique_lock<std::mutex> lk(S->m);
      if (L.canceling) {
        const auto now = Clock::now();
        for (auto &kv : S->req) {
          Request &r = kv.second;
          if (r.state == 2 || r.lane != li) continue;
          if (r.state == 1) S->in_use -= r.bytes;
          r.state = 2;
          r.err = PETSC_ERR_ARG_WRONGSTATE;
          r.t_done = now;
          S->failed++;
        }
        L.queue.clear();
        L.reserve = 0.0;
        for (int i : B.live) {
          B.eps[i] = nullptr;
          B.free_slots.push_back(i);
        }
        B.live.clear();
        B.maps_dirty = true;
        L.canceling = false;
        S->cv_done.notify_all();
      }
    }
    // 1. admission: move queued requests whose footprint fits into free slots.  A queue head that the budget holds
    // back reserves its footprint; a lane leaves out of its budget the reservations older than its own, so a large
    // request is not starved by a stream of small ones, and the oldest reservation (a request larger than the whole
    // budget included) is admitted once enough of the admitted work has retired.
    std::vector<EPS> take;
    {
      std::unique_lock<std::mutex> lk(S->m);
      if (B.live.empty() && L.queue.empty()) {
        if (S->stopping) break;
        S->cv_work.wait_for(lk, std::chrono::milliseconds(20));
        continue;
      }
      const size_t slots_free = B.free_slots.size();
      bool held = false;
      while (!L.queue.empty() && take.size() < slots_free) {
        EPS e = L.queue.front();
        Request &r = S->req[e];
        const long long mine = L.reserve > 0.0 ? L.reserve_seq : LLONG_MAX;
        double reserved = 0.0;
        for (int q = 0; q < LANES; ++q)
          if (q != li && S->lane[q].reserve > 0.0 && S->lane[q].reserve_seq < mine) reserved += S->lane[q].reserve;
        const bool fits = S->in_use + reserved + r.bytes <= S->budget;
        const bool alone = S->in_use == 0.0 && reserved == 0.0;  // larger than the budget: runs with nothing else
        if (!fits && !alone) {
          held = true;
          if (L.reserve == 0.0) L.reserve_seq = ++S->reserve_seq;
          L.reserve = r.bytes;
          break;
        }
        L.queue.pop_front();
        L.reserve = 0.0;
        S->in_use += r.bytes;
        S->peak = std::max(S->peak, S->in_use);
        r.state = 1;
        r.t_admit = Clock::now();
        take.push_back(e);
      }
      if (!held) L.reserve = 0.0;
      if (take.empty() && B.live.empty()) {  // nothing to run: wait for a retirement in another lane
        S->cv_work.wait_for(lk, std::chrono::milliseconds(5));
        continue;
      }
    }
    // 2. the GPU runs the lane's current cycle while the admitted requests are set up on their own streams
    const bool running = !B.live.empty();
    if (running) {
      PetscErrorCode ierr = ksg_engine_launch(B);
      if (ierr) {
        fail_all(ierr);
        return;
      }
    }
    std::vector<int> new_slots;
    for (EPS e : take) {
      PetscErrorCode ierr = EPSSetUp(e);
      if (!ierr) ierr = ksg_engine_check(e, B.max_ld - 1, false);
      int slot = -1;
      if (!ierr) ierr = ksg_engine_admit(B, e, &slot);
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
      std::vector<EPS> owner(B.cap, nullptr);
      for (int i : B.live) owner[i] = B.eps[i];
      PetscErrorCode ierr = ksg_engine_finish(B, &retired);
      if (ierr) {
        fail_all(ierr);
        return;
      }
      if (!retired.empty()) {
        std::lock_guard<std::mutex> lk(S->m);
        const auto now = Clock::now();
        for (auto &rt : retired) {
          EPS e = owner[rt.first];
          auto it = e ? S->req.find(e) : S->req.end();
          if (it == S->req.end() || it->second.state != 1) continue;
          Request &r = it->second;
          r.state = 2;
          r.err = rt.second;
          r.t_done = now;
          e->stats.solve_seconds = std::chrono::duration<double>(now - r.t_submit).count();
          S->in_use -= r.bytes;
          if (rt.second) S->failed++;
          else S->completed++;
        }
        S->cv_done.notify_all();
        S->cv_work.notify_all();
      }
    }
    if (!new_slots.empty()) ksg_engine_activate(B, new_slots);
    {
      std::lock_guard<std::mutex> lk(S->m);
      L.live_now = (long long)B.live.size();
      L.cycles_now = B.cycles;
      long long live = 0;
      for (int q = 0; q < LANES; ++q) live += S->lane[q].live_now;
      S->max_live = std::max(S->max_live, live);
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
  for (int q = 0; q < LANES; ++q) {
    PetscErrorCode ierr = ksg_engine_init(S->lane[q].B, S->device, (int)max_requests, (int)max_ncv);
    if (ierr) {
      delete S;
      return ierr;
    }
  }
  for (int q = 0; q < LANES; ++q) S->lane[q].th = std::thread(server_loop, S, q);
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
  r.lane = r.bytes <= SMALL_LANE_BYTES ? 0 : 1;
  r.t_submit = Clock::now();
  S->req[eps] = r;
  S->lane[r.lane].queue.push_back(eps);
  S->submitted++;
  S->cv_work.notify_all();
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
  st->queued = st->live = st->cycles = 0;
  for (int q = 0; q < LANES; ++q) {
    st->queued += (long long)S->lane[q].queue.size();
    st->live += S->lane[q].live_now;
    st->cycles += S->lane[q].cycles_now;
  }
  st->max_live = S->max_live;
  st->bytes_in_use = S->in_use;
  st->peak_bytes = S->peak;
  return 0;
}

extern "C" PetscErrorCode EPSGB300ServerCancel(EPSGB300Server S) {
  KSG_CHECK(S, PETSC_ERR_ARG_NULL, "Null argument");
  std::lock_guard<std::mutex> lk(S->m);
  for (int q = 0; q < LANES; ++q) S->lane[q].canceling = true;
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
  for (int q = 0; q < LANES; ++q)
    if (S->lane[q].th.joinable()) S->lane[q].th.join();  // each loop drains its lane's requests first
  const int err = S->loop_err;
  delete S;
  *server = nullptr;
  KSG_CHECK(!err, err, "The server loop stopped after an error");
  return 0;
}
