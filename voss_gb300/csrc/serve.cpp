// serve.cpp -- continuous-batching request server on the GB300 sieve.
//
// The reference serves one query per Context: it allocates, sieves the whole
// range host-serially segment by segment and frees, one call at a time
// (library/src/primes/context.cu:212-559, 608-635).  Here requests arrive at
// any time and are batched continuously:
//   * K slots, each a stream with a fixed-capacity launch plan whose device
//     part (memsets, the persistent sieve over a work queue, finalize) is a
//     CUDA graph captured once and replayed for every batch;
//   * a scheduler thread retires finished slots (event polling, results
//     copied back asynchronously) and admits pending requests into free
//     slots, FIFO, bounded by requests and segments per batch and by a
//     device-memory budget over all batches in flight;
//   * batches in different slots overlap on the device: CTAs of the next
//     batch start as SMs free up from the previous one;
//   * the sieving-prime table and tiles stay resident; count and Chebyshev
//     requests skip the ordered gap scan;
//   * requests of one batch share work: their ranges are cut at every
//     endpoint into disjoint atoms, each atom is sieved once, and a combine
//     kernel rebuilds every request from its run of atoms (gaps stitched
//     where atoms meet), so overlapping requests do not sieve the same
//     integers twice.
// A result is the same whether the request ran alone or in a batch.
#include "serve.h"

#include <algorithm>
#include <chrono>
#include <cstring>

#include "voss/voss.h"

namespace vg {

static double now_us() {
  using namespace std::chrono;
  return duration<double, std::micro>(steady_clock::now().time_since_epoch()).count();
}

uint64_t Server::request_bytes(uint64_t segs) {
  return segs * sizeof(SegRec) + sizeof(ReqAccum) + sizeof(ReqResult) + sizeof(ReqDesc);
}

Server::Server(Engine& e, const ServerConfig& c) : E(e), cfg(c) {
  if (cfg.slots == 0 || cfg.slots > 64) throw Error(VOSS_ERR_INVALID_ARG, "slots must be in [1, 64]");
  if (cfg.max_batch == 0) throw Error(VOSS_ERR_INVALID_ARG, "max_batch must be > 0");
  if (cfg.max_segs == 0) throw Error(VOSS_ERR_INVALID_ARG, "max_segs must be > 0");
  {
    std::lock_guard<std::mutex> g(E.mu);
    E.ensure_table(isqrt_u64(kMaxB - 1));     // graphs keep the table's pointers
  }
  slots.resize(cfg.slots);
  for (auto& sp : slots) {
    sp.reset(new Slot());
    Slot& s = *sp;
    s.plan.eng = &E;
    s.plan.device = E.device;
    s.plan.batch_mode = true;
    s.plan.share = cfg.share != 0;
    s.plan.reserve_capacity(cfg.max_batch, cfg.max_segs, cfg.bucket_bytes / 4);
    check_cuda(cudaStreamCreateWithFlags(&s.stream, cudaStreamNonBlocking), "server stream");
    check_cuda(cudaEventCreateWithFlags(&s.done, cudaEventDisableTiming), "server event");
  }
  worker = std::thread([this] { loop(); });
  std::lock_guard<std::mutex> g(E.mu);
  ++E.servers;
}

Server::~Server() {
  {
    std::lock_guard<std::mutex> g(mu);
    stop = true;
  }
  cv_work.notify_all();
  if (worker.joinable()) worker.join();
  {
    std::lock_guard<std::mutex> g(E.mu);
    --E.servers;
  }
  for (auto& sp : slots) {
    if (sp->stream) {
      cudaStreamSynchronize(sp->stream);
      cudaStreamDestroy(sp->stream);
    }
    if (sp->done) cudaEventDestroy(sp->done);
  }
}

uint64_t Server::submit(uint64_t a, uint64_t b, uint32_t op) {
  if (b > kMaxB) throw Error(VOSS_ERR_OUT_OF_RANGE, "range end exceeds 10^14 + 10^10 + 1");
  if (op > kOpChebyshev) throw Error(VOSS_ERR_INVALID_ARG, "unknown request op");
  const Plan& plan = slots[0]->plan;
  // A request wider than half a batch runs as consecutive pieces of at most
  // half a batch each (batches sieve with the largest segment S, and a piece
  // of (half S - 2) wheel bytes spans at most half segments), so that other
  // requests' batches interleave with them.
  const uint64_t half = std::max<uint64_t>(cfg.max_segs / 2, 1);
  std::vector<std::pair<uint64_t, uint64_t>> pieces;
  if (b > a && plan.segments_for(a, b) > half) {
    const uint64_t S = E.cfg.seg_bytes;
    const uint64_t w = 30ull * std::max<uint64_t>(half * S, 3) - 60ull;   // integers per piece
    for (uint64_t x = a; x < b; x += std::min(w, b - x)) pieces.emplace_back(x, std::min(b, x + w));
  } else {
    pieces.emplace_back(a, b);
  }
  std::vector<Ticket> parts(pieces.size());
  for (size_t i = 0; i < pieces.size(); ++i) {
    Ticket& t = parts[i];
    t.a = pieces[i].first;
    t.b = pieces[i].second;
    t.op = op;
    t.segs = plan.segments_for(t.a, t.b);
    if (t.segs > cfg.max_segs)
      throw Error(VOSS_ERR_INTERNAL, "a request piece needs more segments than a server batch holds");
    // bucket lists that do not fit a slot's arena are not used (the plan skips them)
    uint64_t bb = plan.list_bytes_for(t.a, t.b);
    if (bb > cfg.bucket_bytes) bb = 0;
    t.bytes = request_bytes(t.segs) + bb;
  }
  const double now = now_us();
  uint64_t id;
  {
    std::lock_guard<std::mutex> g(mu);
    if (stop) throw Error(VOSS_ERR_INVALID_ARG, "server is shutting down");
    id = next_id++;
    if (parts.size() == 1) {
      parts[0].t_submit = now;
      tickets.emplace(id, parts[0]);
      pending.push_back(id);
    } else {
      Ticket t;
      t.a = a;
      t.b = b;
      t.op = op;
      t.t_submit = now;
      t.npieces = (uint32_t)parts.size();
      t.parts.resize(parts.size());
      tickets.emplace(id, std::move(t));
      for (size_t i = 0; i < parts.size(); ++i) {
        const uint64_t cid = next_id++;
        parts[i].parent = id;
        parts[i].index = (uint32_t)i;
        parts[i].t_submit = now;
        tickets.emplace(cid, parts[i]);
        pending.push_back(cid);
      }
    }
    ++submitted;
    if (!first_submit) first_submit = now;
  }
  cv_work.notify_one();
  return id;
}

bool Server::result(uint64_t id, bool wait, voss_range_stats_t* out, double* latency_us) {
  std::unique_lock<std::mutex> g(mu);
  auto it = tickets.find(id);
  if (it == tickets.end()) throw Error(VOSS_ERR_INVALID_ARG, "unknown or already collected ticket");
  if (!it->second.done) {
    if (!wait) return false;
    cv_done.wait(g, [&] { return tickets.at(id).done; });
    it = tickets.find(id);
  }
  const Ticket& t = it->second;
  if (t.error) {
    const std::string msg = t.message;
    tickets.erase(it);
    throw Error(VOSS_ERR_CUDA, msg);
  }
  if (out) *out = t.res;
  if (latency_us) *latency_us = t.t_done - t.t_submit;
  tickets.erase(it);
  return true;
}

void Server::drain() {
  std::unique_lock<std::mutex> g(mu);
  cv_done.wait(g, [&] { return pending.empty() && inflight == 0; });
}

void Server::metrics(voss_gb300_server_metrics_t* m) {
  std::lock_guard<std::mutex> g(mu);
  std::memset(m, 0, sizeof(*m));
  m->submitted = submitted;
  m->completed = completed;
  m->batches = batches;
  m->max_inflight_batches = max_inflight;
  m->peak_admitted_bytes = peak_bytes;
  m->pending = pending.size();
  if (!lat.empty()) {
    std::vector<double> v(lat);
    std::sort(v.begin(), v.end());
    auto q = [&](double f) { return v[std::min<size_t>(v.size() - 1, (size_t)(f * (v.size() - 1) + 0.5))]; };
    m->p50_us = q(0.50);
    m->p99_us = q(0.99);
    double s = 0;
    for (double x : v) s += x;
    m->mean_us = s / v.size();
  }
  if (completed && last_done > first_submit)
    m->req_per_s = completed / ((last_done - first_submit) * 1e-6);
  m->mean_batch = batches ? (double)batched_requests / batches : 0.0;
}

void Server::reset_metrics() {
  std::lock_guard<std::mutex> g(mu);
  lat.clear();
  completed = batches = batched_requests = 0;
  submitted = 0;                          // requests not yet done (a split one counts once)
  for (const auto& kv : tickets)
    if (!kv.second.parent && !kv.second.done) ++submitted;
  first_submit = last_done = 0;
  max_inflight = 0;
  peak_bytes = 0;
}

// Called with mu held: a batch entry is done (r = its result, or null with
// err).  A piece hands its result to its request, which completes with its
// last piece; the piece's own ticket goes.
void Server::finish_ticket(uint64_t id, Ticket& tk, const ReqResult* r, const std::string& err, double t) {
  if (!tk.parent) {
    if (r) to_public(*r, tk.a, tk.b, &tk.res);
    else { tk.error = true; tk.message = err; }
    tk.done = true;
    tk.t_done = t;
    lat.push_back(t - tk.t_submit);
    ++completed;
    return;
  }
  const uint64_t pid = tk.parent;
  const uint32_t idx = tk.index;
  Ticket& par = tickets.at(pid);
  if (r) par.parts[idx] = *r;
  else if (!par.error) { par.error = true; par.message = err; }
  ++par.pieces_done;
  tickets.erase(id);                     // tk is gone from here on
  if (par.pieces_done < par.npieces) return;
  if (!par.error) {
    const bool gaps = par.op == kOpTwins || par.op == kOpGapHist;
    const ReqResult m = merge_ordered(par.parts.data(), par.parts.size(), gaps);
    to_public(m, par.a, par.b, &par.res);
  }
  std::vector<ReqResult>().swap(par.parts);
  par.done = true;
  par.t_done = t;
  lat.push_back(t - par.t_submit);
  ++completed;
}

void Server::retire(Slot& s) {
  const cudaError_t q = cudaEventQuery(s.done);
  if (q == cudaErrorNotReady) return;
  std::string err;
  const ReqResult* r = nullptr;
  if (q != cudaSuccess) {
    err = std::string("batch failed: ") + cudaGetErrorString(q);
  } else {
    try {
      if (s.plan.overflowed()) {              // a bucket list ran out of room: redo without lists
        s.plan.allow_buckets = false;
        s.plan.load((uint32_t)s.a.size(), s.a.data(), s.b.data(), 0, s.rf.data());
        s.plan.upload(s.stream);
        s.plan.run_device(s.stream);
        s.plan.fetch(s.stream);
        s.plan.allow_buckets = true;
      }
      r = s.plan.finish();
    } catch (const std::exception& e) {
      err = e.what();
      s.plan.allow_buckets = true;
    }
  }
  const double t = now_us();
  std::lock_guard<std::mutex> g(mu);
  for (size_t i = 0; i < s.ids.size(); ++i)
    finish_ticket(s.ids[i], tickets.at(s.ids[i]), r ? r + i : nullptr, err, t);
  inflight_requests -= s.ids.size();
  last_done = t;
  inflight_bytes -= s.bytes;
  --inflight;
  s.busy = false;
  s.ids.clear();
  cv_done.notify_all();
}

bool Server::admit(Slot& s) {
  std::vector<uint64_t>& a = s.a;
  std::vector<uint64_t>& b = s.b;
  std::vector<uint32_t>& rf = s.rf;
  a.clear();
  b.clear();
  rf.clear();
  uint64_t segs = 0, bytes = 0;
  {
    std::lock_guard<std::mutex> g(mu);
    while (!pending.empty() && s.ids.size() < cfg.max_batch) {
      const uint64_t id = pending.front();
      const Ticket& t = tickets.at(id);
      const bool first = s.ids.empty();
      if (!first && segs + t.segs > cfg.max_segs) break;
      // memory admission: what the request's segment records, accumulators
      // and results occupy, against the budget over every batch in flight
      if (inflight_bytes + bytes + t.bytes > cfg.mem_budget && !(first && inflight == 0)) break;
      pending.pop_front();
      s.ids.push_back(id);
      a.push_back(t.a);
      b.push_back(t.b);
      rf.push_back(t.op == kOpTwins || t.op == kOpGapHist ? kReqGaps : 0u);
      segs += t.segs;
      bytes += t.bytes;
    }
    if (s.ids.empty()) return false;
    inflight_bytes += bytes;
    peak_bytes = std::max(peak_bytes, inflight_bytes);
    ++inflight;
    inflight_requests += s.ids.size();
    max_inflight = std::max<uint64_t>(max_inflight, inflight);
    ++batches;
    batched_requests += s.ids.size();
  }
  s.bytes = bytes;
  try {
    s.plan.load((uint32_t)a.size(), a.data(), b.data(), 0, rf.data());
    s.plan.upload(s.stream);
    if (cfg.use_graphs) s.plan.launch_graph(s.stream);
    else s.plan.run_device(s.stream);
    s.plan.fetch_async(s.stream);
    check_cuda(cudaEventRecord(s.done, s.stream), "server event");
  } catch (const std::exception& e) {
    std::lock_guard<std::mutex> g(mu);
    const double t = now_us();
    for (uint64_t id : s.ids) finish_ticket(id, tickets.at(id), nullptr, e.what(), t);
    inflight_requests -= s.ids.size();
    inflight_bytes -= bytes;
    --inflight;
    s.ids.clear();
    cv_done.notify_all();
    return false;
  }
  s.busy = true;
  return true;
}

void Server::loop() {
  int dev = E.device;
  cudaSetDevice(dev);
  for (;;) {
    bool progressed = false;
    for (auto& sp : slots)
      if (sp->busy) {
        const bool was = sp->busy;
        retire(*sp);
        progressed |= was && !sp->busy;
      }
    for (auto& sp : slots)
      if (!sp->busy) {
        if (!admit(*sp)) break;
        progressed = true;
      }
    if (progressed) continue;
    std::unique_lock<std::mutex> g(mu);
    if (stop && pending.empty() && inflight == 0) break;
    if (inflight == 0) {
      cv_work.wait_for(g, std::chrono::milliseconds(5));     // idle: wait for submissions
    } else {
      g.unlock();
      std::this_thread::sleep_for(std::chrono::microseconds(20));   // batches in flight: poll
    }
  }
}

}  // namespace vg
