// The serving loop (include/sgx.h, "Serving"): a worker thread that admits
// PTE closure requests into CUDA-stream slots under a device-memory budget
// and overlaps their copies and solves on the device.
//
// Memory: one cudaMalloc of hbm_budget_bytes at creation, carved per request
// by a first-fit free list (256-byte granules, neighbours coalesced on
// free). A request's block holds its arrays and, for the mixed solver, the
// scratch that sgx_pte_solve would otherwise take from the stream-ordered
// pool (launch_pte_mixed_with), so nothing is allocated per request.
//
// Scheduling: strict arrival order. The head of the queue is admitted when a
// slot is idle and its block fits; a request that does not fit waits for
// blocks to be freed (no overtaking, so no starvation of large requests).
// An admitted request's host->device copies, solve and device->host copies
// are issued on its slot's stream, followed by an event; the worker polls
// the events, releases the block and the slot of each finished request and
// wakes its waiters. The GPU runs the slots' work concurrently.
#include <chrono>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <map>
#include <memory>
#include <mutex>
#include <string>
#include <thread>
#include <unordered_map>
#include <vector>

#include <cuda_runtime.h>

#include "sgx_internal.h"

namespace sgx {
namespace {

using Clock = std::chrono::steady_clock;
constexpr size_t GRAIN = 256;

size_t up(size_t b) { return (b + GRAIN - 1) / GRAIN * GRAIN; }

class Arena {
 public:
  bool init(size_t bytes, std::string &msg) {
    cap_ = bytes / GRAIN * GRAIN;
    const cudaError_t e = cudaMalloc(reinterpret_cast<void **>(&base_), cap_);
    if (e != cudaSuccess) {
      msg = std::string("sgx_server_create: cudaMalloc of the arena: ") + cudaGetErrorString(e);
      base_ = nullptr;
      return false;
    }
    free_[0] = cap_;
    return true;
  }
  void release() {
    if (base_) cudaFree(base_);
    base_ = nullptr;
  }
  // First fit; returns SIZE_MAX when no free block is large enough.
  size_t alloc(size_t bytes) {
    bytes = up(bytes);
    for (auto it = free_.begin(); it != free_.end(); ++it) {
      if (it->second < bytes) continue;
      const size_t off = it->first, rest = it->second - bytes;
      free_.erase(it);
      if (rest) free_[off + bytes] = rest;
      used_ += bytes;
      if (used_ > peak_) peak_ = used_;
      return off;
    }
    return SIZE_MAX;
  }
  void free(size_t off, size_t bytes) {
    bytes = up(bytes);
    used_ -= bytes;
    auto it = free_.emplace(off, bytes).first;
    auto next = std::next(it);
    if (next != free_.end() && it->first + it->second == next->first) {
      it->second += next->second;
      free_.erase(next);
    }
    if (it != free_.begin()) {
      auto prev = std::prev(it);
      if (prev->first + prev->second == it->first) {
        prev->second += it->second;
        free_.erase(it);
      }
    }
  }
  char *base() const { return base_; }
  size_t cap() const { return cap_; }
  size_t used() const { return used_; }
  size_t peak() const { return peak_; }

 private:
  char *base_ = nullptr;
  size_t cap_ = 0, used_ = 0, peak_ = 0;
  std::map<size_t, size_t> free_;
};

// Offsets of one request's arrays inside its arena block.
struct Layout {
  size_t idx, vt, st, mat[5], status, bins, retry, perm, total;
  Layout(const sgx_pte_request &r, const bool mixed) {
    const size_t n = static_cast<size_t>(r.ncell), m = static_cast<size_t>(r.nmat);
    size_t o = 0;
    idx = o;
    o += r.eos_idx ? up(4 * n * m) : 0;
    vt = o;
    o += up(8 * n);
    st = o;
    o += up(8 * n);
    for (int k = 0; k < 5; ++k) {
      mat[k] = o;
      o += up(8 * n * m);
    }
    status = o;
    o += up(sizeof(sgx_pte_status) * n);
    bins = retry = perm = o;
    if (mixed || r.eos_idx) {
      o += up(PTE_BINS_BYTES); // counters and the signature histogram
      retry = o;
      o += mixed ? up(4 * n) : 0;
      perm = o;
      o += r.eos_idx ? up(4 * n) : 0;
    }
    total = o;
  }
};

struct Request {
  uint64_t ticket = 0;
  sgx_pte_request r{};
  size_t bytes = 0, off = 0;
  int slot = -1;
  int state = 0; // 0 queued, 3 being issued, 1 running, 2 finished
  int err = SGX_OK;
  std::string msg;
  Clock::time_point t_submit, t_done;
};

struct Slot {
  cudaStream_t stream = nullptr;
  cudaEvent_t done = nullptr;
  Request *req = nullptr;
};

} // namespace

struct Server {
  int device = 0;
  int solver = SGX_PTE_RHOT, precision = SGX_PREC_FP64;
  int neos = 0;
  sgx_eos eos[MAX_EOS];
  sgx_mix_params params{};
  Arena arena;
  std::vector<Slot> slots;
  std::mutex mu;
  std::condition_variable cv_work, cv_done;
  std::deque<Request *> queue;
  std::unordered_map<uint64_t, std::unique_ptr<Request>> requests;
  uint64_t next_ticket = 1;
  bool stop = false;
  uint64_t submitted = 0, completed = 0, failed = 0, cells_completed = 0;
  std::thread worker;

  bool mixed() const { return precision == SGX_PREC_MIXED; }

  // Issues the copies, the solve and the copies back of q on slot k, then
  // records the slot's event. Called by the worker without the lock (with
  // pageable host arrays the device-to-host copies block); returns the first
  // CUDA error, after which nothing reliable is in flight on the stream.
  cudaError_t issue(Request *q, const int k) {
    Slot &sl = slots[k];
    const sgx_pte_request &r = q->r;
    const Layout L(r, mixed());
    char *b = arena.base() + q->off;
    const size_t n = static_cast<size_t>(r.ncell), nm = n * static_cast<size_t>(r.nmat);
    cudaStream_t s = sl.stream;
    cudaError_t e = cudaSuccess;
    auto h2d = [&](size_t off, const void *src, size_t bytes) {
      if (e == cudaSuccess) e = cudaMemcpyAsync(b + off, src, bytes, cudaMemcpyHostToDevice, s);
    };
    auto d2h = [&](void *dst, size_t off, size_t bytes) {
      if (e == cudaSuccess && dst)
        e = cudaMemcpyAsync(dst, b + off, bytes, cudaMemcpyDeviceToHost, s);
    };
    if (r.eos_idx) h2d(L.idx, r.eos_idx, 4 * nm);
    h2d(L.vt, r.vfrac_tot, 8 * n);
    h2d(L.st, r.sie_tot, 8 * n);
    const double *in[5] = {r.rho_in, r.vfrac_in, r.sie_in, r.temp_in, r.press_in};
    for (int m = 0; m < 5; ++m)
      h2d(L.mat[m], in[m], 8 * nm);
    PteArgs a;
    std::memset(&a, 0, sizeof(a));
    a.solver = solver;
    a.nmat = r.nmat;
    a.ncell = r.ncell;
    a.neos = neos;
    for (int i = 0; i < neos; ++i)
      a.eos[i] = eos[i];
    a.eos_idx = r.eos_idx ? reinterpret_cast<const int32_t *>(b + L.idx) : nullptr;
    a.vfrac_tot = reinterpret_cast<const double *>(b + L.vt);
    a.sie_tot = reinterpret_cast<const double *>(b + L.st);
    double *mat[5];
    for (int m = 0; m < 5; ++m)
      mat[m] = reinterpret_cast<double *>(b + L.mat[m]);
    a.rho = mat[0];
    a.vfrac = mat[1];
    a.sie = mat[2];
    a.temp = mat[3];
    a.press = mat[4];
    a.lambda = nullptr;
    a.status = reinterpret_cast<sgx_pte_status *>(b + L.status);
    a.params = params;
    if (e == cudaSuccess) {
      if (mixed()) {
        a.bins = reinterpret_cast<unsigned *>(b + L.bins);
        a.retry_idx = reinterpret_cast<int *>(b + L.retry);
        e = launch_pte_mixed_with(a, r.eos_idx ? reinterpret_cast<int *>(b + L.perm) : nullptr,
                                  s);
      } else {
        e = launch_pte_fp64_with(a, reinterpret_cast<unsigned *>(b + L.bins),
                                 r.eos_idx ? reinterpret_cast<int *>(b + L.perm) : nullptr, s);
      }
    }
    double *out[5] = {r.rho_out, r.vfrac_out, r.sie_out, r.temp_out, r.press_out};
    for (int m = 0; m < 5; ++m)
      d2h(out[m], L.mat[m], 8 * nm);
    d2h(r.status, L.status, sizeof(sgx_pte_status) * n);
    if (e == cudaSuccess) e = cudaEventRecord(sl.done, s);
    if (e != cudaSuccess) cudaStreamSynchronize(s);
    return e;
  }

  void finish(const int k, const int err, const std::string &msg) {
    Slot &sl = slots[k];
    Request *q = sl.req;
    sl.req = nullptr;
    arena.free(q->off, q->bytes);
    q->err = err;
    q->msg = msg;
    q->state = 2;
    q->t_done = Clock::now();
    if (err == SGX_OK) {
      ++completed;
      cells_completed += static_cast<uint64_t>(q->r.ncell);
    } else {
      ++failed;
    }
    cv_done.notify_all();
  }

  void run() {
    cudaSetDevice(device);
    for (;;) {
      std::vector<std::pair<Request *, int>> admitted;
      bool progress = false;
      {
        std::unique_lock<std::mutex> lk(mu);
        int inflight = 0;
        for (int k = 0; k < static_cast<int>(slots.size()); ++k) {
          if (!slots[k].req || slots[k].req->state != 1) continue;
          const cudaError_t e = cudaEventQuery(slots[k].done);
          if (e == cudaSuccess) {
            finish(k, SGX_OK, "");
            progress = true;
          } else if (e != cudaErrorNotReady) {
            finish(k, SGX_ERR_CUDA, std::string("sgx_server: ") + cudaGetErrorString(e));
            progress = true;
          } else {
            ++inflight;
          }
        }
        for (int k = 0; k < static_cast<int>(slots.size()) && !queue.empty(); ++k) {
          if (slots[k].req) continue;
          Request *q = queue.front();
          const size_t off = arena.alloc(q->bytes);
          if (off == SIZE_MAX) break; // the head waits for memory
          queue.pop_front();
          q->off = off;
          q->slot = k;
          q->state = 3; // being issued
          slots[k].req = q;
          admitted.emplace_back(q, k);
          ++inflight;
        }
        if (stop && queue.empty() && inflight == 0) break;
        if (admitted.empty() && !progress)
          cv_work.wait_for(lk, std::chrono::microseconds(inflight ? 20 : 2000));
      }
      for (auto &qk : admitted) {
        const cudaError_t e = issue(qk.first, qk.second);
        std::lock_guard<std::mutex> lk(mu);
        if (e == cudaSuccess)
          qk.first->state = 1;
        else
          finish(qk.second, SGX_ERR_CUDA, std::string("sgx_server: ") + cudaGetErrorString(e));
      }
    }
  }
};

} // namespace sgx

using sgx::Server;

struct sgx_server {
  Server impl;
};

extern "C" {

int sgx_server_create(const sgx_server_config *cfg, sgx_server **out) {
  using sgx::set_error;
  if (!cfg || !out) return set_error(SGX_ERR_INVALID, "sgx_server_create: null");
  *out = nullptr;
  if (cfg->max_inflight < 1 || cfg->max_inflight > 64)
    return set_error(SGX_ERR_INVALID, "sgx_server_create: max_inflight must be in 1..64");
  if (cfg->neos < 1 || cfg->neos > sgx::MAX_EOS || !cfg->eos_list)
    return set_error(SGX_ERR_INVALID, "sgx_server_create: neos must be in 1..16");
  if (cfg->solver != SGX_PTE_RHOT && cfg->solver != SGX_PTE_PT)
    return set_error(SGX_ERR_INVALID, "sgx_server_create: bad solver");
  if (cfg->precision != SGX_PREC_FP64 && cfg->precision != SGX_PREC_MIXED)
    return set_error(SGX_ERR_INVALID, "sgx_server_create: bad precision");
  if (cfg->precision == SGX_PREC_MIXED && cfg->solver != SGX_PTE_RHOT)
    return set_error(SGX_ERR_UNSUPPORTED, "sgx_server_create: mixed precision is RhoT only");
  for (int k = 0; k < cfg->neos; ++k)
    if (cfg->eos_list[k].type < SGX_IDEAL_GAS || cfg->eos_list[k].type > SGX_SPINER_RHOT)
      return set_error(SGX_ERR_UNSUPPORTED, "sgx_server_create: EOS not available in PTE");
    else if (const int rc = sgx::check_eos_mods(cfg->eos_list[k],
                                                cfg->precision == SGX_PREC_MIXED,
                                                "sgx_server_create"))
      return rc;
  if (cfg->hbm_budget_bytes < (1u << 20))
    return set_error(SGX_ERR_INVALID, "sgx_server_create: hbm_budget_bytes below 1 MiB");
  auto *h = new sgx_server;
  Server &s = h->impl;
  cudaGetDevice(&s.device);
  s.solver = cfg->solver;
  s.precision = cfg->precision;
  s.neos = cfg->neos;
  for (int k = 0; k < cfg->neos; ++k)
    s.eos[k] = cfg->eos_list[k];
  if (cfg->params)
    s.params = *cfg->params;
  else
    sgx_mix_params_default(&s.params);
  std::string msg;
  if (!s.arena.init(cfg->hbm_budget_bytes, msg)) {
    delete h;
    return set_error(SGX_ERR_CUDA, msg);
  }
  s.slots.resize(cfg->max_inflight);
  for (auto &sl : s.slots) {
    cudaError_t e = cudaStreamCreateWithFlags(&sl.stream, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&sl.done, cudaEventDisableTiming);
    if (e != cudaSuccess) {
      for (auto &t : s.slots) {
        if (t.stream) cudaStreamDestroy(t.stream);
        if (t.done) cudaEventDestroy(t.done);
      }
      s.arena.release();
      delete h;
      return set_error(SGX_ERR_CUDA, std::string("sgx_server_create: ") + cudaGetErrorString(e));
    }
  }
  s.worker = std::thread([&s] { s.run(); });
  *out = h;
  return SGX_OK;
}

int sgx_server_submit(sgx_server *h, const sgx_pte_request *req, uint64_t *ticket) {
  using sgx::set_error;
  if (!h || !req || !ticket) return set_error(SGX_ERR_INVALID, "sgx_server_submit: null");
  const sgx_pte_request &r = *req;
  if (r.nmat < 1 || r.nmat > sgx::PTE_MAX_N)
    return set_error(SGX_ERR_UNSUPPORTED, "sgx_server_submit: nmat must be in 1..6");
  if (r.ncell < 1 || r.ncell > 0x7fffffffLL)
    return set_error(SGX_ERR_INVALID, "sgx_server_submit: ncell must be in 1..2^31-1");
  if (!r.vfrac_tot || !r.sie_tot || !r.rho_in || !r.vfrac_in || !r.sie_in || !r.temp_in ||
      !r.press_in || !r.rho_out || !r.vfrac_out || !r.sie_out || !r.temp_out || !r.press_out)
    return set_error(SGX_ERR_INVALID, "sgx_server_submit: null array");
  Server &s = h->impl;
  if (!r.eos_idx && s.neos < r.nmat)
    return set_error(SGX_ERR_INVALID, "sgx_server_submit: eos_idx NULL needs neos >= nmat");
  auto q = std::make_unique<sgx::Request>();
  q->r = r;
  q->bytes = sgx::Layout(r, s.mixed()).total;
  if (q->bytes > s.arena.cap())
    return set_error(SGX_ERR_INVALID, "sgx_server_submit: request needs " +
                                          std::to_string(q->bytes) +
                                          " bytes, more than the whole arena");
  q->t_submit = sgx::Clock::now();
  {
    std::lock_guard<std::mutex> lk(s.mu);
    if (s.stop) return set_error(SGX_ERR_INVALID, "sgx_server_submit: server is stopping");
    q->ticket = s.next_ticket++;
    *ticket = q->ticket;
    s.queue.push_back(q.get());
    s.requests.emplace(q->ticket, std::move(q));
    ++s.submitted;
  }
  s.cv_work.notify_one();
  return SGX_OK;
}

int sgx_server_wait(sgx_server *h, uint64_t ticket, double timeout_s, double *latency_s) {
  using sgx::set_error;
  if (!h) return set_error(SGX_ERR_INVALID, "sgx_server_wait: null");
  Server &s = h->impl;
  std::unique_lock<std::mutex> lk(s.mu);
  auto it = s.requests.find(ticket);
  if (it == s.requests.end())
    return set_error(SGX_ERR_INVALID, "sgx_server_wait: unknown ticket (already waited on?)");
  sgx::Request *q = it->second.get();
  auto done = [&] { return q->state == 2; };
  if (timeout_s < 0)
    s.cv_done.wait(lk, done);
  else if (!s.cv_done.wait_for(lk, std::chrono::duration<double>(timeout_s), done))
    return set_error(SGX_ERR_TIMEOUT, "sgx_server_wait: still pending");
  if (latency_s) latency_s[0] = std::chrono::duration<double>(q->t_done - q->t_submit).count();
  const int err = q->err;
  const std::string msg = q->msg;
  s.requests.erase(it);
  return err == SGX_OK ? SGX_OK : set_error(err, msg);
}

int sgx_server_stats_get(sgx_server *h, sgx_server_stats *out) {
  if (!h || !out) return sgx::set_error(SGX_ERR_INVALID, "sgx_server_stats_get: null");
  Server &s = h->impl;
  std::lock_guard<std::mutex> lk(s.mu);
  out->submitted = s.submitted;
  out->completed = s.completed;
  out->failed = s.failed;
  out->cells_completed = s.cells_completed;
  int inflight = 0;
  for (auto &sl : s.slots)
    inflight += sl.req ? 1 : 0;
  out->inflight = inflight;
  out->queued = static_cast<int>(s.queue.size());
  out->arena_used = s.arena.used();
  out->arena_peak = s.arena.peak();
  return SGX_OK;
}

int sgx_server_destroy(sgx_server *h) {
  if (!h) return SGX_OK;
  Server &s = h->impl;
  {
    std::lock_guard<std::mutex> lk(s.mu);
    s.stop = true;
  }
  s.cv_work.notify_all();
  if (s.worker.joinable()) s.worker.join();
  for (auto &sl : s.slots) {
    cudaStreamDestroy(sl.stream);
    cudaEventDestroy(sl.done);
  }
  s.arena.release();
  delete h;
  return SGX_OK;
}

void *sgx_host_alloc(size_t bytes) {
  void *p = nullptr;
  if (cudaHostAlloc(&p, bytes, cudaHostAllocDefault) != cudaSuccess) {
    sgx::set_error(SGX_ERR_CUDA, "sgx_host_alloc: cudaHostAlloc failed");
    return nullptr;
  }
  return p;
}

void sgx_host_free(void *p) {
  if (p) cudaFreeHost(p);
}

} // extern "C"
