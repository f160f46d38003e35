// server.cpp — continuous-batching request loop for world-solve requests.
//
// A request is a world (a copy of a solver's contents) plus a number of
// Solver::update calls.  A worker thread repeats one tick:
//   1. take queued requests, first come first served, while the device bytes
//      of the resident worlds plus the candidate stay within the budget;
//   2. launch one Solver::update for every resident world, all in one launch
//      sequence of a shared Engine (the same batched kernels as
//      b2d_batch_update), and while it runs plan the requests taken in
//      step 1 on the host and install them (their uploads go to the engine's
//      install stream, so the device keeps stepping);
//   3. wait, then retire requests that reached their step count: copy the
//      state back, free the world's device block, record the latency.
// Requests that arrive while a tick runs wait in the queue and join the
// tick after next at the latest, so work overlaps on the device as memory
// frees up.  On an idle device a request is planned and installed at once.
// World state
// stays device-resident across ticks.  Every world is computed independently
// (per-world grids, order-independent sums), so a result is bit-identical
// whether the request ran alone or in a mix.
//
// Cancellation: a queued request is dropped at once; one taken for planning
// or resident on the device is dropped by the worker at its next install or
// retire phase, so no kernel of the tick in flight loses its world.
#include <algorithm>
#include <chrono>
#include <condition_variable>
#include <deque>
#include <memory>
#include <mutex>
#include <thread>
#include <unordered_map>

#include "engine.hpp"
#include "server.hpp"

namespace b2d {

using Clock = std::chrono::steady_clock;

struct Server::Req {
  uint64_t id;
  WorldHost world;
  uint32_t steps = 0, done = 0;
  float dt = 0.0f;
  int state = SERVE_QUEUED;
  bool cancel = false;  // cancellation asked after the worker took it
  uint32_t slot = 0;
  size_t bytes = 0;
  uint64_t np = 0;      // solver particles (the residency limit counts these)
  Clock::time_point t_submit, t_admit, t_done;
  std::string error;
};

Server::Server(uint64_t budget) : budget_(budget) {}

Server::~Server() { stop(); }

int Server::start() {
  std::lock_guard<std::mutex> lk(mu_);
  if (running_) return OK;
  running_ = true;
  worker_ = std::thread([this] { loop(); });
  return OK;
}

int Server::stop() {
  {
    std::lock_guard<std::mutex> lk(mu_);
    if (!running_) return OK;
    running_ = false;
  }
  cv_.notify_all();
  if (worker_.joinable()) worker_.join();
  return OK;
}

// Upper bound of the device bytes a world holds while resident: its block
// (every array at its largest: one body per particle) plus its share of the
// collision grid.
size_t Server::estimate_bytes(const WorldHost& w) {
  const size_t np = w.particles.size(), nl = w.particle_links.size(), nc = w.circles.size(),
               ng = w.polygons.size();
  size_t nv = 0, npl = 0;
  for (const Polygon& g : w.polygons) {
    nv += g.particles.size();
    npl += g.particle_links.size();
  }
  size_t b = 24 * np + 4 * np + sizeof(DBody) * np + 16 * nl;
  b += 36 * nc + 12 * w.circle_links.size();
  b += 24 * nv + (sizeof(DPoly) + 24) * ng + 12 * npl + 4 * (ng * ng + 1);
  if (w.collide) b += 48 * np + 64;
  return b + 32 * 16;
}

int Server::submit(const WorldHost& w, uint32_t steps, float dt, uint64_t* id, std::string* why) {
  int st = validate_world(w, why);
  if (st != OK) return st;
  const size_t bytes = estimate_bytes(w);
  if (bytes > budget_) {
    if (why) *why = "world needs " + std::to_string(bytes) + " device bytes, budget is " +
                    std::to_string(budget_);
    return ERR_BUDGET;
  }
  auto r = std::make_unique<Req>();
  r->world = w;
  r->steps = steps;
  r->dt = dt;
  r->bytes = bytes;
  r->np = w.particles.size();
  r->t_submit = Clock::now();
  {
    std::lock_guard<std::mutex> lk(mu_);
    r->id = next_id_++;
    *id = r->id;
    queue_.push_back(r.get());
    reqs_.emplace(r->id, std::move(r));
    ++stats_.submitted;
  }
  cv_.notify_all();
  return OK;
}

int Server::poll(uint64_t id, int* state) {
  std::lock_guard<std::mutex> lk(mu_);
  auto it = reqs_.find(id);
  if (it == reqs_.end()) return ERR_INDEX;
  *state = it->second->state;
  return OK;
}

int Server::cancel(uint64_t id) {
  std::lock_guard<std::mutex> lk(mu_);
  auto it = reqs_.find(id);
  if (it == reqs_.end()) return ERR_INDEX;
  Req& r = *it->second;
  if (r.state != SERVE_QUEUED && r.state != SERVE_RUNNING) return ERR_STATE;
  auto q = std::find(queue_.begin(), queue_.end(), &r);
  if (q != queue_.end()) {  // not yet taken by the worker
    queue_.erase(q);
    r.state = SERVE_CANCELLED;
    r.t_admit = r.t_done = Clock::now();
    ++stats_.cancelled;
    finished_.push_back(r.id);
    return OK;
  }
  r.cancel = true;  // the worker drops it at its next install or retire
  return OK;
}

void Server::set_max_resident_particles(uint64_t n) {
  {
    std::lock_guard<std::mutex> lk(mu_);
    max_resident_np_ = n;
  }
  cv_.notify_all();
}

void Server::set_fault(int kind, uint64_t value) {
  std::lock_guard<std::mutex> lk(mu_);
  faults_.emplace_back(kind, value);
}

int Server::take(uint64_t id, WorldHost* out, double* latency_s, double* queue_s,
                 std::string* why) {
  std::lock_guard<std::mutex> lk(mu_);
  auto it = reqs_.find(id);
  if (it == reqs_.end()) return ERR_INDEX;
  Req& r = *it->second;
  if (r.state == SERVE_FAILED || r.state == SERVE_CANCELLED) {
    if (why) *why = r.state == SERVE_CANCELLED ? std::string("request cancelled") : r.error;
    reqs_.erase(it);
    return ERR_STATE;
  }
  if (r.state != SERVE_DONE) {
    if (why) *why = "request not finished";
    return ERR_STATE;
  }
  if (out) *out = std::move(r.world);
  if (latency_s) *latency_s = std::chrono::duration<double>(r.t_done - r.t_submit).count();
  if (queue_s) *queue_s = std::chrono::duration<double>(r.t_admit - r.t_submit).count();
  reqs_.erase(it);
  return OK;
}

std::vector<uint64_t> Server::finished() {
  std::lock_guard<std::mutex> lk(mu_);
  std::vector<uint64_t> out;
  out.swap(finished_);
  return out;
}

ServerStats Server::stats() {
  std::lock_guard<std::mutex> lk(mu_);
  ServerStats s = stats_;
  s.queued = queue_.size();
  s.active = active_.size();
  s.resident_bytes = resident_;
  s.resident_particles = resident_np_;
  return s;
}

void Server::loop() {
  std::unique_ptr<Engine> eng;
  // requests taken from the queue and planned during the last tick, waiting
  // to be installed after it
  std::vector<std::pair<Req*, WorldImage>> planned;
  // a request taken from the queue leaves before it reached the device:
  // failed (planning or install) or cancelled
  auto drop = [&](Req* r, int state, const std::string& why) {
    std::lock_guard<std::mutex> lk(mu_);
    r->t_admit = r->t_done = Clock::now();
    r->state = state;
    r->error = why;
    resident_ -= r->bytes;
    resident_np_ -= r->np;
    ++(state == SERVE_CANCELLED ? stats_.cancelled : stats_.failed);
    finished_.push_back(r->id);
  };
  auto fail = [&](Req* r, const std::string& why) { drop(r, SERVE_FAILED, why); };
  auto plan = [&](Req* r) {
    WorldImage img;
    std::string why;
    const int st = eng->plan(r->world, &img, &why);
    if (st != OK) fail(r, why.empty() ? eng->last_error : why);
    else planned.emplace_back(r, std::move(img));
  };
  // install the planned requests: they join the next tick
  auto install = [&]() {
    for (auto& pr : planned) {
      Req* r = pr.first;
      bool cancelled;
      {
        std::lock_guard<std::mutex> lk(mu_);
        cancelled = r->cancel;
      }
      if (cancelled) {
        drop(r, SERVE_CANCELLED, "request cancelled");
        continue;
      }
      uint32_t slot = 0;
      int st = eng->add_planned(&r->world, std::move(pr.second), &slot);
      if (st == OK) st = eng->set_dt(slot, r->dt);
      if (st != OK) {
        fail(r, eng->last_error);
        continue;
      }
      std::lock_guard<std::mutex> lk(mu_);
      r->slot = slot;
      r->t_admit = Clock::now();
      r->state = SERVE_RUNNING;
      active_.push_back(r);
      ++stats_.admitted;
    }
    planned.clear();
  };
  for (;;) {
    std::vector<Req*> taken;
    std::vector<std::pair<int, uint64_t>> faults;
    {
      std::unique_lock<std::mutex> lk(mu_);
      cv_.wait(lk, [&] {
        return !running_ || !queue_.empty() || !active_.empty() || !planned.empty();
      });
      if (!running_) break;
      // first come, first served while the memory budget and the residency
      // limit hold (one request is always taken onto an idle device)
      while (!queue_.empty() && resident_ + queue_.front()->bytes <= budget_ &&
             (max_resident_np_ == 0 || resident_np_ == 0 ||
              resident_np_ + queue_.front()->np <= max_resident_np_)) {
        Req* r = queue_.front();
        queue_.pop_front();
        resident_ += r->bytes;
        resident_np_ += r->np;
        taken.push_back(r);
      }
      faults.swap(faults_);
    }
    if (!eng) eng = std::make_unique<Engine>(nullptr);
    for (const auto& f : faults) eng->set_fault(f.first, f.second);
    const Clock::time_point ta = Clock::now();
    // with nothing on the device there is no tick to plan under: plan now
    bool idle;
    {
      std::lock_guard<std::mutex> lk(mu_);
      idle = active_.empty();
    }
    if (idle) {  // nothing on the device: plan and install now
      for (Req* r : taken) plan(r);
      taken.clear();
      install();
    }
    std::vector<Req*> act;
    const Clock::time_point ts = Clock::now();
    {
      std::lock_guard<std::mutex> lk(mu_);
      act = active_;
      stats_.admit_ns += (uint64_t)std::chrono::duration_cast<std::chrono::nanoseconds>(ts - ta).count();
    }
    if (act.empty()) {
      for (Req* r : taken) plan(r);
      continue;
    }
    // requests that asked for zero steps finish without a tick
    int st = OK;
    bool any_steps = false;
    for (Req* r : act) any_steps |= r->done < r->steps;
    if (any_steps) st = eng->step();
    // the requests taken this tick are planned and installed while it
    // runs (their uploads on the engine's install stream)
    const Clock::time_point tp = Clock::now();
    for (Req* r : taken) plan(r);
    if (any_steps && st == OK) {
      eng->install_beside(true);
      install();
      eng->install_beside(false);
    }
    const Clock::time_point tq = Clock::now();
    if (any_steps && st == OK) st = eng->sync();
    const Clock::time_point tr = Clock::now();
    uint64_t units = 0;
    std::vector<Req*> finished;
    std::vector<char> cancelled;
    {
      std::lock_guard<std::mutex> lk(mu_);
      for (Req* r : act) cancelled.push_back(r->cancel ? 1 : 0);
    }
    for (size_t k = 0; k < act.size(); ++k) {
      Req* r = act[k];
      if (r->done < r->steps) {
        ++r->done;
        units += (uint64_t)r->world.particles.size() * r->world.sub_steps;
      }
      if (r->done >= r->steps || st != OK || cancelled[k]) finished.push_back(r);
    }
    for (Req* r : finished) {
      const bool cancel_it = cancelled[std::find(act.begin(), act.end(), r) - act.begin()] != 0;
      int ds = st != OK ? st : (cancel_it ? OK : eng->download(r->slot));
      const std::string err = ds != OK ? eng->last_error : std::string();
      eng->remove(r->slot);
      std::lock_guard<std::mutex> lk(mu_);
      r->t_done = Clock::now();
      resident_ -= r->bytes;
      resident_np_ -= r->np;
      if (ds != OK) {
        r->state = SERVE_FAILED;
        r->error = err;
        ++stats_.failed;
      } else if (cancel_it) {
        r->state = SERVE_CANCELLED;
        ++stats_.cancelled;
      } else {
        r->state = SERVE_DONE;
        ++stats_.completed;
      }
      active_.erase(std::find(active_.begin(), active_.end(), r));
      finished_.push_back(r->id);
    }
    const Clock::time_point te = Clock::now();
    std::lock_guard<std::mutex> lk(mu_);
    ++stats_.ticks;
    stats_.particle_substeps += units;
    // planning under the tick counts as admission, the rest of the tick as
    // stepping
    stats_.admit_ns += (uint64_t)std::chrono::duration_cast<std::chrono::nanoseconds>(tq - tp).count();
    stats_.step_ns += (uint64_t)std::chrono::duration_cast<std::chrono::nanoseconds>((tr - ts) - (tq - tp)).count();
    stats_.retire_ns += (uint64_t)std::chrono::duration_cast<std::chrono::nanoseconds>(te - tr).count();
  }
  // requests planned but never installed are released
  for (auto& pr : planned) fail(pr.first, "server stopped");
  eng.reset();
}

}  // namespace b2d
