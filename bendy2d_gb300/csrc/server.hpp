// server.hpp — continuous-batching request loop (see server.cpp).
#pragma once
#include <condition_variable>
#include <cstdint>
#include <deque>
#include <memory>
#include <mutex>
#include <string>
#include <thread>
#include <unordered_map>
#include <vector>

#include "host.hpp"

namespace b2d {

enum : int {
  SERVE_QUEUED = 0,
  SERVE_RUNNING = 1,
  SERVE_DONE = 2,
  SERVE_FAILED = 3,
  SERVE_CANCELLED = 4
};

struct ServerStats {
  uint64_t submitted = 0, admitted = 0, completed = 0, failed = 0, cancelled = 0;
  uint64_t queued = 0, active = 0;
  uint64_t ticks = 0, particle_substeps = 0;
  uint64_t resident_bytes = 0, resident_particles = 0;
  uint64_t admit_ns = 0, step_ns = 0, retire_ns = 0;  // worker wall time per phase
};

class Server {
 public:
  explicit Server(uint64_t budget_bytes);
  ~Server();
  int start();
  int stop();
  int submit(const WorldHost& w, uint32_t steps, float dt, uint64_t* id, std::string* why);
  int poll(uint64_t id, int* state);
  // a queued request is dropped at once; a running one leaves the device at
  // the end of the tick in flight; ERR_STATE once it has finished
  int cancel(uint64_t id);
  // admission also keeps the resident solver particles at or below n (0: no
  // limit), except that one request is always admitted onto an idle device
  void set_max_resident_particles(uint64_t n);
  // fault injection for tests of failure handling (FAULT_* of engine.hpp);
  // applied by the worker before its next tick
  void set_fault(int kind, uint64_t value);
  // hands over a finished request's world and releases the request
  int take(uint64_t id, WorldHost* out, double* latency_s, double* queue_s, std::string* why);
  ServerStats stats();
  static size_t estimate_bytes(const WorldHost& w);
  // ids of requests finished (done or failed) since the last call
  std::vector<uint64_t> finished();

 private:
  struct Req;
  void loop();
  uint64_t budget_;
  std::mutex mu_;
  std::condition_variable cv_;
  bool running_ = false;
  std::thread worker_;
  uint64_t next_id_ = 1;
  std::unordered_map<uint64_t, std::unique_ptr<Req>> reqs_;
  std::deque<Req*> queue_;
  std::vector<Req*> active_;
  uint64_t resident_ = 0;
  uint64_t resident_np_ = 0;
  uint64_t max_resident_np_ = 0;
  std::vector<std::pair<int, uint64_t>> faults_;  // to hand to the engine
  ServerStats stats_;
  std::vector<uint64_t> finished_;
};

}  // namespace b2d
