// serve.h -- continuous-batching request server (see serve.cpp).
#pragma once
#include <condition_variable>
#include <deque>
#include <memory>
#include <mutex>
#include <string>
#include <thread>
#include <unordered_map>
#include <vector>

#include "engine.h"
#include "voss/voss_gb300.h"

namespace vg {

constexpr uint32_t kOpCount = VOSS_OP_COUNT;
constexpr uint32_t kOpTwins = VOSS_OP_TWINS;
constexpr uint32_t kOpGapHist = VOSS_OP_GAP_HIST;
constexpr uint32_t kOpChebyshev = VOSS_OP_CHEBYSHEV;

struct ServerConfig {
  uint32_t slots = 4;            // batches in flight at once
  uint32_t max_batch = 1024;     // requests per batch
  uint64_t max_segs = 1u << 16;  // segments per batch
  uint64_t mem_budget = 1ull << 30;   // device bytes over all batches in flight
  uint32_t use_graphs = 1;
  uint64_t bucket_bytes = 256ull << 20;   // bucket-list arena per slot
  uint32_t share = 1;            // batches sieve shared atoms of their ranges once
};

class Server {
 public:
  Server(Engine& e, const ServerConfig& c);
  ~Server();
  uint64_t submit(uint64_t a, uint64_t b, uint32_t op);
  // true when the result is ready (copied to *out and the ticket released)
  bool result(uint64_t id, bool wait, voss_range_stats_t* out, double* latency_us);
  void drain();
  void metrics(voss_gb300_server_metrics_t* m);
  void reset_metrics();
  static uint64_t request_bytes(uint64_t segs);

 private:
  struct Ticket {
    uint64_t a = 0, b = 0;
    uint32_t op = 0;
    uint64_t segs = 0, bytes = 0;
    double t_submit = 0, t_done = 0;
    bool done = false, error = false;
    std::string message;
    voss_range_stats_t res{};
    // A request wider than half a batch runs as consecutive pieces, each an
    // internal ticket (parent = the request's id, index = its place); the
    // request collects their results and is done with the last one.
    uint64_t parent = 0;
    uint32_t index = 0;
    uint32_t npieces = 0, pieces_done = 0;
    std::vector<ReqResult> parts;
  };
  struct Slot {
    Plan plan;
    cudaStream_t stream = nullptr;
    cudaEvent_t done = nullptr;
    std::vector<uint64_t> ids;
    std::vector<uint64_t> a, b;     // the batch, kept for a rerun without bucket lists
    std::vector<uint32_t> rf;
    uint64_t bytes = 0;
    bool busy = false;
  };
  void loop();
  void retire(Slot& s);
  bool admit(Slot& s);
  void finish_ticket(uint64_t id, Ticket& tk, const ReqResult* r, const std::string& err, double t);

  Engine& E;
  ServerConfig cfg;
  std::vector<std::unique_ptr<Slot>> slots;
  std::mutex mu;
  std::condition_variable cv_work, cv_done;
  std::thread worker;
  bool stop = false;
  std::deque<uint64_t> pending;
  std::unordered_map<uint64_t, Ticket> tickets;
  uint64_t next_id = 1;
  uint64_t inflight = 0, inflight_requests = 0, inflight_bytes = 0;
  uint64_t submitted = 0, completed = 0, batches = 0, batched_requests = 0;
  uint64_t max_inflight = 0, peak_bytes = 0;
  double first_submit = 0, last_done = 0;
  std::vector<double> lat;
};

}  // namespace vg
