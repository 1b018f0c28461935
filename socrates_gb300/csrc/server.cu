// server.cu -- continuous-batching request server (socgpu_server_*).
//
// Requests are radiance_calc calls with host arrays.  Every request's inputs
// and outputs live in one device arena, sized at creation, while the request
// is in flight.  One scheduler thread runs this loop:
//   * it retires finished requests one by one (each has its own event,
//     recorded after its outputs are copied back): they are marked done and
//     their arena blocks freed; a stream slot is free again when all of its
//     wave's requests are;
//   * when a stream slot is free, it admits queued requests in arrival order
//     for as long as their blocks fit the arena (admission by free device
//     memory), up to max_wave_requests, and launches them as one wave.
// Requests are of two size classes.  Small ones (at most
// small_column_gpoints column x g-points) are waved on high-priority streams
// and large ones on low-priority streams (a low-priority slot takes small
// requests only when no large one waits or runs), so that a small request
// never shares a wave, or a stream priority, with a large one.  Every kernel
// is loaded onto the device when the server is created: a first launch that
// loaded its module could wait for the kernels already running.  Each kernel class of a wave (precision,
// mode, tile) is one launch of the batched kernel with one CTA per column: as
// the CTAs of a large wave retire, the block scheduler gives the SMs to the
// pending CTAs of high-priority streams first, so a small request that
// arrives during a large one waits for a few columns' worth of work, not for
// the whole wave.  Up to `streams` waves are in flight at once, so requests
// that arrive while others run are admitted as soon as a slot and memory
// free up, and their work overlaps on the device.  The spectra stay device
// resident in the library's registry.  Requests whose host arrays are
// page-locked are copied asynchronously on the wave's stream; pageable ones
// synchronously, in before the wave's kernels and out when the request is
// retired.
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <map>
#include <memory>
#include <mutex>
#include <string>
#include <thread>
#include <tuple>
#include <unordered_map>
#include <vector>

#include "host_internal.h"

using namespace socgpu;
using Clock = std::chrono::steady_clock;

namespace {

size_t align256(size_t n) { return (n + 255) & ~(size_t)255; }

// First-fit allocator over one device allocation; blocks are 256-byte
// aligned and merged with their neighbours when freed.  Used by the
// scheduler thread only.
class Arena {
 public:
  void init(size_t bytes) {
    size_ = bytes;
    free_.clear();
    free_[0] = bytes;
    used_ = peak_ = 0;
  }
  bool alloc(size_t bytes, size_t *off) {
    bytes = align256(bytes);
    for (auto it = free_.begin(); it != free_.end(); ++it) {
      if (it->second < bytes) continue;
      *off = it->first;
      const size_t rest = it->second - bytes, start = it->first + bytes;
      free_.erase(it);
      if (rest) free_[start] = rest;
      used_ += bytes;
      peak_ = std::max(peak_, used_);
      return true;
    }
    return false;
  }
  void release(size_t off, size_t bytes) {
    bytes = align256(bytes);
    used_ -= bytes;
    auto it = free_.emplace(off, bytes).first;
    auto nx = std::next(it);
    if (nx != free_.end() && it->first + it->second == nx->first) {
      it->second += nx->second;
      free_.erase(nx);
    }
    if (it != free_.begin()) {
      auto pv = std::prev(it);
      if (pv->first + pv->second == it->first) {
        pv->second += it->second;
        free_.erase(it);
      }
    }
  }
  size_t size() const { return size_; }
  size_t peak() const { return peak_; }

 private:
  size_t size_ = 0, used_ = 0, peak_ = 0;
  std::map<size_t, size_t> free_;
};

struct Request {
  long long ticket = 0;
  socgpu_control control{};
  socgpu_dimen dimen{};
  socgpu_atm atm{};
  socgpu_cld cld{};
  socgpu_aer aer{};
  socgpu_bound bound{};
  socgpu_radout radout{};
  bool has_cld = false, has_aer = false;
  StagedCall call;
  bool pinned = false;   // every host array page-locked: asynchronous copies on the wave's stream
  size_t bytes = 0, off = 0;
  long long colg = 0;
  Clock::time_point t_submit, t_start, t_done;
  int status = SOCGPU_I_NORMAL;
  bool done = false;
  std::string msg;
};

struct StreamSlot {
  cudaStream_t stream = nullptr;
  bool high = false;                  // high priority: waves of small requests
  bool small_wave = false;            // the wave in flight is of small requests
  std::vector<cudaEvent_t> done;      // one per request of the wave, in wave order
  FluxParams *d_items = nullptr, *h_items = nullptr;     // per-wave kernel tables
  long long *d_start = nullptr, *h_start = nullptr;
  bool busy = false;
  size_t n_retired = 0;               // requests of the wave already retired (in order)
  std::vector<Request *> reqs;
};

}  // namespace

struct socgpu_server_s {
  socgpu_server_config cfg{};
  int device = 0;
  char *dmem = nullptr;
  Arena arena;
  std::vector<StreamSlot> slots;
  std::mutex mu;
  std::condition_variable cv_work, cv_done;
  std::deque<Request *> pending;
  long long small_colg = 0;
  std::unordered_map<long long, std::unique_ptr<Request>> requests;
  long long next_ticket = 1;
  bool stop = false;
  std::thread worker;
  socgpu_server_stats stats{};
};

namespace {

// Synchronous copies of a request whose host arrays are pageable: the
// copy engines never read or write pageable memory asynchronously.
int copy_sync(const Request &r, char *base, bool out, char *msg, size_t msg_len) {
  const auto &slots = r.call.plan.slots;
  for (size_t k = out ? r.call.n_inputs : 0; k < (out ? slots.size() : r.call.n_inputs); ++k) {
    const Slot &sl = slots[k];
    if (sl.row_bytes == 0) continue;
    if (out)
      CUDA_TRY(cudaMemcpy2D(sl.out_host, sl.host_pitch, base + sl.off, sl.dev_pitch, sl.row_bytes, sl.rows,
                            cudaMemcpyDeviceToHost));
    else
      CUDA_TRY(cudaMemcpy2D(base + sl.off, sl.dev_pitch, sl.host, sl.host_pitch, sl.row_bytes, sl.rows,
                            cudaMemcpyHostToDevice));
  }
  return SOCGPU_I_NORMAL;
}

// Retire one finished request of a wave (called with the server mutex held).
void finish(socgpu_server_s &S, Request *r, cudaError_t e) {
  if (e == cudaSuccess && r->status == SOCGPU_I_NORMAL && !r->pinned) {
    char m[256] = "";
    if (copy_sync(*r, S.dmem + r->off, true, m, sizeof(m)) != SOCGPU_I_NORMAL) {
      r->status = SOCGPU_I_ABORT_CALCULATION;
      r->msg = m;
    }
  }
  r->t_done = Clock::now();
  if (e != cudaSuccess && r->status == SOCGPU_I_NORMAL) {
    r->status = SOCGPU_I_ABORT_CALCULATION;
    r->msg = std::string("wave failed on the device: ") + cudaGetErrorString(e);
  }
  r->done = true;
  S.arena.release(r->off, r->bytes);
  S.stats.completed += 1;
  if (r->status == SOCGPU_I_NORMAL) S.stats.column_gpoints += r->colg;
}

// Retire the requests of a wave whose events have fired, in wave order;
// the slot is free once all are retired.  Returns whether any was retired.
bool retire(socgpu_server_s &S, StreamSlot &sl) {
  bool any = false;
  while (sl.n_retired < sl.reqs.size()) {
    cudaError_t e = cudaEventQuery(sl.done[sl.n_retired]);
    if (e == cudaErrorNotReady) break;
    finish(S, sl.reqs[sl.n_retired], e);
    ++sl.n_retired;
    any = true;
  }
  if (sl.n_retired == sl.reqs.size()) {
    sl.reqs.clear();
    sl.n_retired = 0;
    sl.busy = false;
  }
  return any;
}

// Every request's event of a wave that stops early (on the slot's stream,
// after whatever was enqueued).
void record_all(StreamSlot &sl) {
  for (size_t i = 0; i < sl.reqs.size(); ++i) cudaEventRecord(sl.done[i], sl.stream);
}

void fail_all(std::vector<Request *> &wave, int status, const char *msg) {
  for (Request *r : wave) {
    if (r->status == SOCGPU_I_NORMAL) {
      r->status = status;
      r->msg = msg;
    }
  }
}

// Enqueue one wave on its slot's stream (called without the mutex; the
// slot is already marked busy and owns the requests).
void launch_wave(socgpu_server_s &S, StreamSlot &sl) {
  std::vector<Request *> &wave = sl.reqs;
  cudaStream_t st = sl.stream;
  char msg[512] = "";
  const size_t msg_len = sizeof(msg);
  const Clock::time_point now = Clock::now();
  for (Request *r : wave) r->t_start = now;
  // inputs
  for (Request *r : wave)
    if ((r->pinned ? r->call.copy_in(S.dmem + r->off, st, msg, msg_len)
                   : copy_sync(*r, S.dmem + r->off, false, msg, msg_len)) != SOCGPU_I_NORMAL) {
      fail_all(wave, SOCGPU_I_ABORT_CALCULATION, msg);
      record_all(sl);
      return;
    }
  // kernel classes of the wave
  std::map<std::tuple<int, int, int, int, int, int>, std::vector<int>> classes;
  std::vector<FluxParams> params(wave.size());
  for (size_t i = 0; i < wave.size(); ++i) {
    Request *r = wave[i];
    r->call.params(S.dmem + r->off, params[i]);
    const int mode = mode_index(&r->control);
    TileConfig t = choose_tile(r->control.precision, mode, r->atm.n_layer);
    if (t.lanes_per_solve == 1) t = scan_tile(r->control.precision, r->atm.n_layer);
    classes[std::make_tuple(r->control.precision, mode, t.lanes_per_solve, t.chunk, t.warps_per_cta,
                            r->control.isolir)].push_back((int)i);
  }
  size_t n_item = 0, n_start = 0;
  std::vector<BatchGroup> groups;
  std::vector<std::pair<size_t, size_t>> table_off;
  for (auto &kv : classes) {
    BatchGroup g{};
    g.precision = std::get<0>(kv.first);
    g.mode = std::get<1>(kv.first);
    g.tile = TileConfig{std::get<2>(kv.first), std::get<4>(kv.first), std::get<3>(kv.first)};
    FluxParams *items = sl.h_items + n_item;
    long long *start = sl.h_start + n_start;
    start[0] = 0;
    int k = 0;
    for (int i : kv.second) {
      items[k] = params[i];
      start[k + 1] = start[k] + params[i].n_profile;
      ++k;
    }
    g.items = items;
    g.col_start = start;
    g.n_items = k;
    g.total = start[k];
    const FluxVariant *v = find_variant(g.precision, g.mode, g.tile.lanes_per_solve);
    if (!v || v->prepare(g, msg, msg_len) != SOCGPU_I_NORMAL) {
      if (!v) snprintf(msg, msg_len, "no kernel built for %d lanes per solve", g.tile.lanes_per_solve);
      fail_all(wave, SOCGPU_I_ERR_RANGE, msg);
      record_all(sl);
      return;
    }
    // one CTA per column (not the persistent grid): CTAs retire column by
    // column, so higher-priority streams get SMs as they do
    g.grid = (int)std::min<long long>(g.total, 0x7fffffffLL);
    groups.push_back(g);
    table_off.emplace_back(n_item, n_start);
    n_item += k;
    n_start += k + 1;
  }
  cudaError_t e = cudaMemcpyAsync(sl.d_items, sl.h_items, sizeof(FluxParams) * n_item, cudaMemcpyHostToDevice, st);
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(sl.d_start, sl.h_start, sizeof(long long) * n_start, cudaMemcpyHostToDevice, st);
  for (size_t gi = 0; gi < groups.size() && e == cudaSuccess; ++gi) {
    const BatchGroup &g = groups[gi];
    if (g.total <= 0) continue;
    FluxParams *di = sl.d_items + table_off[gi].first;
    long long *ds = sl.d_start + table_off[gi].second;
    int n = g.n_items;
    long long total = g.total;
    void *args[] = {&di, &ds, &n, &total};
    e = cudaLaunchKernel(g.kernel, dim3(g.grid), dim3(g.threads), args, g.smem, st);
    count_launch();
  }
  if (e != cudaSuccess) {
    cudaGetLastError();
    fail_all(wave, SOCGPU_I_ABORT_CALCULATION, cudaGetErrorString(e));
    record_all(sl);
    return;
  }
  // each request's outputs, then its own event
  for (size_t i = 0; i < wave.size(); ++i) {
    Request *r = wave[i];
    if (r->pinned && r->status == SOCGPU_I_NORMAL &&
        r->call.copy_out(S.dmem + r->off, st, msg, msg_len) != SOCGPU_I_NORMAL) {
      r->status = SOCGPU_I_ABORT_CALCULATION;
      r->msg = msg;
    }
    cudaEventRecord(sl.done[i], st);
  }
}

void worker_main(socgpu_server_s *Sp) {
  socgpu_server_s &S = *Sp;
  cudaSetDevice(S.device);
  std::unique_lock<std::mutex> lk(S.mu);
  // Take queued requests of one size class for a wave, in arrival order,
  // while their blocks fit the arena.
  auto take = [&](bool small, std::vector<Request *> &wave) {
    for (auto it = S.pending.begin(); it != S.pending.end() && (int)wave.size() < S.cfg.max_wave_requests;) {
      Request *r = *it;
      if ((r->colg <= S.small_colg) != small) { ++it; continue; }
      size_t off = 0;
      if (!S.arena.alloc(r->bytes, &off)) break;
      r->off = off;
      wave.push_back(r);
      it = S.pending.erase(it);
    }
  };
  for (;;) {
    bool progressed = false;
    for (StreamSlot &sl : S.slots)
      if (sl.busy) progressed |= retire(S, sl);
    if (progressed) S.cv_done.notify_all();
    for (StreamSlot &sl : S.slots) {
      if (sl.busy || S.pending.empty()) continue;
      std::vector<Request *> wave;
      // high-priority slots take small requests; the others large ones
      // first, and small ones when no large request waits or runs (a small
      // wave on a low-priority stream would queue behind a large wave's CTAs)
      bool small = sl.high;
      take(small, wave);
      if (wave.empty() && !sl.high) {
        bool large_running = false;
        for (const StreamSlot &x : S.slots) large_running |= x.busy && !x.small_wave;
        if (!large_running) { small = true; take(true, wave); }
      }
      if (wave.empty()) continue;
      sl.busy = true;
      sl.small_wave = small;
      sl.n_retired = 0;
      sl.reqs = std::move(wave);
      S.stats.waves += 1;
      if (small) S.stats.small_waves += 1;
      S.stats.max_wave_requests = std::max<long long>(S.stats.max_wave_requests, (long long)sl.reqs.size());
      S.stats.peak_bytes = S.arena.peak();
      long long in_flight = 0;
      for (const StreamSlot &x : S.slots) in_flight += x.busy;
      S.stats.max_waves_in_flight = std::max(S.stats.max_waves_in_flight, in_flight);
      lk.unlock();
      launch_wave(S, sl);
      lk.lock();
      progressed = true;
    }
    bool any_busy = false;
    for (StreamSlot &sl : S.slots) any_busy |= sl.busy;
    if (S.stop && S.pending.empty() && !any_busy) break;
    if (!progressed) {
      if (any_busy) {
        lk.unlock();
        std::this_thread::sleep_for(std::chrono::microseconds(20));
        lk.lock();
      } else {
        S.cv_work.wait(lk, [&] { return S.stop || !S.pending.empty(); });
      }
    }
  }
}

void destroy_server(socgpu_server_s *S) {
  for (StreamSlot &sl : S->slots) {
    if (sl.stream) cudaStreamSynchronize(sl.stream);
    for (cudaEvent_t e : sl.done)
      if (e) cudaEventDestroy(e);
    if (sl.stream) cudaStreamDestroy(sl.stream);
    if (sl.d_items) cudaFree(sl.d_items);
    if (sl.d_start) cudaFree(sl.d_start);
    if (sl.h_items) cudaFreeHost(sl.h_items);
    if (sl.h_start) cudaFreeHost(sl.h_start);
  }
  if (S->dmem) cudaFree(S->dmem);
  delete S;
}

}  // namespace

extern "C" {

int socgpu_server_create(const socgpu_server_config *config, socgpu_server *server, char *msg, size_t msg_len) {
  if (!server) { set_msg(msg, msg_len, "null argument"); return SOCGPU_I_ERR_FATAL; }
  socgpu_server_config cfg{};
  if (config) cfg = *config;
  if (cfg.streams <= 0) cfg.streams = 4;
  if (cfg.max_wave_requests <= 0) cfg.max_wave_requests = 256;
  if (cfg.streams > 64 || cfg.max_wave_requests > 65536) {
    set_msg(msg, msg_len, "streams (1..64) or max_wave_requests (1..65536) out of range");
    return SOCGPU_I_ERR_RANGE;
  }
  std::unique_ptr<socgpu_server_s> S(new socgpu_server_s);
  CUDA_TRY(cudaGetDevice(&S->device));
  // every kernel loaded before the first wave, so that no launch waits on a
  // module load behind a long-running kernel of another wave
  if (preload_kernels() != SOCGPU_I_NORMAL) {
    set_msg(msg, msg_len, "the flux kernels could not be loaded onto the device");
    return SOCGPU_I_ABORT_CALCULATION;
  }
  int prio_low = 0, prio_high = 0;
  CUDA_TRY(cudaDeviceGetStreamPriorityRange(&prio_low, &prio_high));
  if (cfg.device_bytes == 0) {
    size_t free_b = 0, total_b = 0;
    CUDA_TRY(cudaMemGetInfo(&free_b, &total_b));
    cfg.device_bytes = free_b / 2;
  }
  cfg.device_bytes = align256(cfg.device_bytes);
  S->cfg = cfg;
  S->arena.init(cfg.device_bytes);
  cudaError_t e = cudaMalloc(&S->dmem, cfg.device_bytes);
  if (e != cudaSuccess) {
    cudaGetLastError();
    set_msg(msg, msg_len, "device arena of %zu bytes not available: %s", cfg.device_bytes, cudaGetErrorString(e));
    return SOCGPU_I_ERR_RANGE;
  }
  S->small_colg = cfg.small_column_gpoints > 0 ? cfg.small_column_gpoints : (1LL << 17);
  S->slots.resize(cfg.streams);
  const size_t n_items = cfg.max_wave_requests;
  // a wave has at most one kernel class per request, so n_items + 1 starts per class fit in 2 n_items + 1
  const size_t n_start = 2 * n_items + 1;
  const int n_high = cfg.streams >= 2 ? cfg.streams / 2 : 0;
  for (size_t q = 0; q < S->slots.size(); ++q) {
    StreamSlot &sl = S->slots[q];
    sl.high = (int)q < n_high;
    sl.done.assign(n_items, nullptr);
    bool ok = true;
    for (cudaEvent_t &e : sl.done) ok = ok && cudaEventCreateWithFlags(&e, cudaEventDisableTiming) == cudaSuccess;
    if (!ok ||
        cudaStreamCreateWithPriority(&sl.stream, cudaStreamNonBlocking, sl.high ? prio_high : prio_low) !=
            cudaSuccess ||
        cudaMalloc(&sl.d_items, sizeof(FluxParams) * n_items) != cudaSuccess ||
        cudaMalloc(&sl.d_start, sizeof(long long) * n_start) != cudaSuccess ||
        cudaMallocHost(&sl.h_items, sizeof(FluxParams) * n_items) != cudaSuccess ||
        cudaMallocHost(&sl.h_start, sizeof(long long) * n_start) != cudaSuccess) {
      cudaGetLastError();
      set_msg(msg, msg_len, "stream slot resources not available");
      destroy_server(S.release());
      return SOCGPU_I_ABORT_CALCULATION;
    }
  }
  S->stats.device_bytes = cfg.device_bytes;
  socgpu_server_s *raw = S.release();
  raw->worker = std::thread(worker_main, raw);
  *server = raw;
  return SOCGPU_I_NORMAL;
}

int socgpu_server_submit(socgpu_server server, const socgpu_request *q, long long *ticket, char *msg,
                         size_t msg_len) {
  if (!server || !q || !ticket) { set_msg(msg, msg_len, "null argument"); return SOCGPU_I_ERR_FATAL; }
  SpectrumEntry *sp = find_spectrum(q->spectrum);
  int st = validate(q->control, q->dimen, sp, q->atm, q->cld, q->aer, q->bound, q->radout, msg, msg_len);
  if (st != SOCGPU_I_NORMAL) return st;
  std::unique_ptr<Request> r(new Request);
  r->control = *q->control;
  r->dimen = *q->dimen;
  r->atm = *q->atm;
  r->bound = *q->bound;
  r->radout = *q->radout;
  if (q->cld) { r->cld = *q->cld; r->has_cld = true; }
  if (q->aer) { r->aer = *q->aer; r->has_aer = true; }
  r->call.stage(&r->control, &r->dimen, sp, &r->atm, r->has_cld ? &r->cld : nullptr,
                r->has_aer ? &r->aer : nullptr, &r->bound, &r->radout);
  if (r->call.prsc) {
    set_msg(msg, msg_len, "prescribed aerosol properties run through socgpu_radiance_calc and "
                          "socgpu_radiance_calc_device, not the server");
    return SOCGPU_I_ERR_FATAL;
  }
  r->bytes = align256(r->call.plan.bytes);
  r->pinned = true;
  for (const Slot &sl : r->call.plan.slots) {
    cudaPointerAttributes at{};
    const void *hp = sl.output ? sl.out_host : sl.host;
    if (cudaPointerGetAttributes(&at, hp) != cudaSuccess) { cudaGetLastError(); r->pinned = false; break; }
    if (at.type != cudaMemoryTypeHost) { r->pinned = false; break; }
  }
  r->colg = r->call.column_gpoints();
  if (r->bytes > server->arena.size()) {
    set_msg(msg, msg_len, "request needs %zu bytes of device memory, more than the server's %zu", r->bytes,
            server->arena.size());
    return SOCGPU_I_ERR_RANGE;
  }
  {
    std::lock_guard<std::mutex> lk(server->mu);
    if (server->stop) { set_msg(msg, msg_len, "server is shutting down"); return SOCGPU_I_ERR_FATAL; }
    r->ticket = server->next_ticket++;
    r->t_submit = Clock::now();
    *ticket = r->ticket;
    server->pending.push_back(r.get());
    server->stats.submitted += 1;
    server->requests[r->ticket] = std::move(r);
  }
  server->cv_work.notify_one();
  return SOCGPU_I_NORMAL;
}

int socgpu_server_wait(socgpu_server server, long long ticket, double timeout_s, int *status, double *queue_ms,
                       double *latency_ms, char *msg, size_t msg_len) {
  if (!server) { set_msg(msg, msg_len, "null argument"); return SOCGPU_I_ERR_FATAL; }
  std::unique_lock<std::mutex> lk(server->mu);
  auto it = server->requests.find(ticket);
  if (it == server->requests.end()) { set_msg(msg, msg_len, "unknown ticket %lld", ticket); return SOCGPU_I_ERR_EXIST; }
  Request *r = it->second.get();
  auto ready = [&] { return r->done; };
  if (timeout_s < 0) {
    server->cv_done.wait(lk, ready);
  } else if (!server->cv_done.wait_for(lk, std::chrono::duration<double>(timeout_s), ready)) {
    set_msg(msg, msg_len, "request %lld not finished", ticket);
    return SOCGPU_SERVER_PENDING;
  }
  if (status) *status = r->status;
  if (queue_ms) *queue_ms = std::chrono::duration<double, std::milli>(r->t_start - r->t_submit).count();
  if (latency_ms) *latency_ms = std::chrono::duration<double, std::milli>(r->t_done - r->t_submit).count();
  if (r->status != SOCGPU_I_NORMAL) set_msg(msg, msg_len, "%s", r->msg.c_str());
  server->requests.erase(it);
  return SOCGPU_I_NORMAL;
}

int socgpu_server_stats_get(socgpu_server server, socgpu_server_stats *stats) {
  if (!server || !stats) return SOCGPU_I_ERR_FATAL;
  std::lock_guard<std::mutex> lk(server->mu);
  *stats = server->stats;
  stats->peak_bytes = server->arena.peak();
  stats->queued = (long long)server->pending.size();
  return SOCGPU_I_NORMAL;
}

int socgpu_server_destroy(socgpu_server server) {
  if (!server) return SOCGPU_I_NORMAL;
  {
    std::lock_guard<std::mutex> lk(server->mu);
    server->stop = true;
  }
  server->cv_work.notify_all();
  if (server->worker.joinable()) server->worker.join();
  destroy_server(server);
  return SOCGPU_I_NORMAL;
}

}  // extern "C"
