// The serving loop (include/sgx.h, "Serving"): a worker thread that folds
// the PTE closure requests waiting at each admission tick into one merged
// solve on the device, under a device-memory budget, with several merged
// batches in flight.
//
// Memory: one cudaMalloc of hbm_budget_bytes at creation, carved per batch
// by a first-fit free list (256-byte granules, neighbours coalesced on
// free). A batch's block holds the merged arrays of its requests and the
// solver's scratch (what sgx_pte_solve would take from the stream-ordered
// pool), so nothing is allocated per request or per batch.
//
// Folding: when a batch slot is free, the worker takes queued requests in
// arrival order while their merged layout still fits the largest free block
// (and stays under SERVE_BATCH_CELLS cells), lays them out one after the
// other along the cell axis ([nmax][sum of cells], each request's cells
// contiguous; material slots a request does not use are marked absent),
// copies every request's inputs into place, runs ONE binned solve over the
// whole batch, and copies each request's rows back to its own output arrays.
// Every cell is solved independently of the others, so each result is the
// one a solve of that request alone gives, bit for bit. A request that does
// not fit waits at the head of the queue (no overtaking, so no starvation of
// large requests). Batches in flight overlap: the next batch's copies and
// solve run while the previous one is still on the device.
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
  // The largest block alloc() can return now.
  size_t largest() const {
    size_t m = 0;
    for (const auto &f : free_)
      m = f.second > m ? f.second : m;
    return m;
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

// Offsets of a batch's merged arrays inside its arena block: nmat material
// slots by ncell cells (the cells of every request of the batch).
struct Layout {
  size_t idx, vt, st, mat[5], status, bins, retry, perm, total;
  Layout(const int nmat, const int64_t ncell, const bool mixed) {
    const size_t n = static_cast<size_t>(ncell), m = static_cast<size_t>(nmat);
    size_t o = 0;
    idx = o;
    o += up(4 * n * m);
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
    bins = o;
    o += up(PTE_BINS_BYTES); // counters and the signature histogram
    retry = o;
    o += mixed ? up(4 * n) : 0;
    perm = o;
    o += up(4 * n);
    total = o;
  }
};

// Cells per merged batch at most (bounds the time a request waits behind the
// batch it lands in).
constexpr int64_t SERVE_BATCH_CELLS = int64_t(1) << 22;

// The material-slot rows of one request inside a merged batch: eos_idx
// rows [0, nmat_r) take the request's own indices (or, with none, the slot
// number), rows [nmat_r, nmat) are absent (-1).
__global__ void serve_fill_idx(int32_t *idx, const int64_t N, const int64_t off,
                               const int64_t n, const int nmat_r, const int nmat,
                               const bool own) {
  const int64_t i = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x;
  if (i >= n) return;
  for (int m = own ? nmat_r : 0; m < nmat; ++m)
    idx[m * N + off + i] = m < nmat_r ? m : -1;
}

struct Request {
  uint64_t ticket = 0;
  sgx_pte_request r{};
  size_t bytes = 0; // the request's layout alone (admission check at submit)
  int64_t cell_off = 0; // first cell inside its batch
  int state = 0; // 0 queued, 3 being issued, 1 running, 2 finished
  int err = SGX_OK;
  std::string msg;
  Clock::time_point t_submit, t_done;
};

// One merged batch in flight.
struct Slot {
  cudaStream_t stream = nullptr;
  cudaEvent_t done = nullptr;
  std::vector<Request *> reqs; // empty: the slot is free
  int nmat = 0;
  int64_t ncell = 0;
  size_t off = 0, bytes = 0;
  int state = 0; // 3 being issued, 1 running
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
  uint64_t submitted = 0, completed = 0, failed = 0, cells_completed = 0, batches = 0;
  std::thread worker;

  bool mixed() const { return precision == SGX_PREC_MIXED; }

  // Issues the batch of slot k: the requests' inputs copied into their
  // places in the merged arrays, one solve of the whole batch, each
  // request's results copied back, then the slot's event. Called by the
  // worker without the lock (with pageable host arrays the device-to-host
  // copies block); returns the first CUDA error, after which nothing
  // reliable is in flight on the stream.
  cudaError_t issue(const int k) {
    Slot &sl = slots[k];
    const Layout L(sl.nmat, sl.ncell, mixed());
    char *b = arena.base() + sl.off;
    const size_t N = static_cast<size_t>(sl.ncell);
    cudaStream_t s = sl.stream;
    cudaError_t e = cudaSuccess;
    int32_t *idx = reinterpret_cast<int32_t *>(b + L.idx);
    double *mat[5];
    for (int m = 0; m < 5; ++m)
      mat[m] = reinterpret_cast<double *>(b + L.mat[m]);
    sgx_pte_status *status = reinterpret_cast<sgx_pte_status *>(b + L.status);
    for (Request *q : sl.reqs) {
      const sgx_pte_request &r = q->r;
      const size_t n = static_cast<size_t>(r.ncell), o = static_cast<size_t>(q->cell_off);
      auto h2d = [&](void *dst, const void *src, size_t bytes) {
        if (e == cudaSuccess) e = cudaMemcpyAsync(dst, src, bytes, cudaMemcpyHostToDevice, s);
      };
      for (int m = 0; m < r.nmat; ++m) {
        if (r.eos_idx) h2d(idx + m * N + o, r.eos_idx + m * n, 4 * n);
        const double *in[5] = {r.rho_in, r.vfrac_in, r.sie_in, r.temp_in, r.press_in};
        for (int a = 0; a < 5; ++a)
          h2d(mat[a] + m * N + o, in[a] + m * n, 8 * n);
      }
      h2d(reinterpret_cast<double *>(b + L.vt) + o, r.vfrac_tot, 8 * n);
      h2d(reinterpret_cast<double *>(b + L.st) + o, r.sie_tot, 8 * n);
      if (e == cudaSuccess && (!r.eos_idx || r.nmat < sl.nmat)) {
        serve_fill_idx<<<static_cast<unsigned>((n + 255) / 256), 256, 0, s>>>(
            idx, sl.ncell, q->cell_off, r.ncell, r.nmat, sl.nmat, r.eos_idx != nullptr);
        e = cudaGetLastError();
      }
    }
    PteArgs a;
    std::memset(&a, 0, sizeof(a));
    a.solver = solver;
    a.nmat = sl.nmat;
    a.ncell = sl.ncell;
    a.neos = neos;
    for (int i = 0; i < neos; ++i)
      a.eos[i] = eos[i];
    a.eos_idx = idx;
    a.vfrac_tot = reinterpret_cast<const double *>(b + L.vt);
    a.sie_tot = reinterpret_cast<const double *>(b + L.st);
    a.rho = mat[0];
    a.vfrac = mat[1];
    a.sie = mat[2];
    a.temp = mat[3];
    a.press = mat[4];
    a.lambda = nullptr;
    a.status = status;
    a.params = params;
    int *perm = reinterpret_cast<int *>(b + L.perm);
    if (e == cudaSuccess) {
      if (mixed()) {
        a.bins = reinterpret_cast<unsigned *>(b + L.bins);
        a.retry_idx = reinterpret_cast<int *>(b + L.retry);
        e = launch_pte_mixed_with(a, perm, s);
      } else {
        e = launch_pte_fp64_with(a, reinterpret_cast<unsigned *>(b + L.bins), perm, s);
      }
    }
    for (Request *q : sl.reqs) {
      const sgx_pte_request &r = q->r;
      const size_t n = static_cast<size_t>(r.ncell), o = static_cast<size_t>(q->cell_off);
      auto d2h = [&](void *dst, const void *src, size_t bytes) {
        if (e == cudaSuccess && dst)
          e = cudaMemcpyAsync(dst, src, bytes, cudaMemcpyDeviceToHost, s);
      };
      double *out[5] = {r.rho_out, r.vfrac_out, r.sie_out, r.temp_out, r.press_out};
      for (int m = 0; m < r.nmat; ++m)
        for (int a2 = 0; a2 < 5; ++a2)
          d2h(out[a2] + m * n, mat[a2] + m * N + o, 8 * n);
      d2h(r.status, status + o, sizeof(sgx_pte_status) * n);
    }
    if (e == cudaSuccess) e = cudaEventRecord(sl.done, s);
    if (e != cudaSuccess) cudaStreamSynchronize(s);
    return e;
  }

  // Releases slot k's block and completes its requests.
  void finish(const int k, const int err, const std::string &msg) {
    Slot &sl = slots[k];
    arena.free(sl.off, sl.bytes);
    const auto now = Clock::now();
    for (Request *q : sl.reqs) {
      q->err = err;
      q->msg = msg;
      q->state = 2;
      q->t_done = now;
      if (err == SGX_OK) {
        ++completed;
        cells_completed += static_cast<uint64_t>(q->r.ncell);
      } else {
        ++failed;
      }
    }
    sl.reqs.clear();
    sl.state = 0;
    cv_done.notify_all();
  }

  // Folds the head of the queue into a batch for slot k (with the lock
  // held): requests in arrival order while the merged layout fits the
  // largest free block and the cell cap. False when not even the head fits.
  bool form_batch(const int k) {
    Slot &sl = slots[k];
    const size_t room = arena.largest();
    int nmat = 0;
    int64_t ncell = 0;
    size_t bytes = 0;
    size_t take = 0;
    for (Request *q : queue) {
      const int nm = nmat > q->r.nmat ? nmat : q->r.nmat;
      const int64_t nc = ncell + q->r.ncell;
      const size_t by = Layout(nm, nc, mixed()).total;
      if (by > room || (take > 0 && nc > SERVE_BATCH_CELLS)) break;
      nmat = nm;
      ncell = nc;
      bytes = by;
      ++take;
    }
    if (take == 0) return false;
    sl.off = arena.alloc(bytes);
    if (sl.off == SIZE_MAX) return false;
    sl.bytes = bytes;
    sl.nmat = nmat;
    sl.ncell = ncell;
    int64_t off = 0;
    for (size_t i = 0; i < take; ++i) {
      Request *q = queue.front();
      queue.pop_front();
      q->cell_off = off;
      off += q->r.ncell;
      q->state = 3;
      sl.reqs.push_back(q);
    }
    sl.state = 3; // being issued
    ++batches;
    return true;
  }

  void run() {
    cudaSetDevice(device);
    for (;;) {
      std::vector<int> admitted;
      bool progress = false;
      {
        std::unique_lock<std::mutex> lk(mu);
        int inflight = 0;
        for (int k = 0; k < static_cast<int>(slots.size()); ++k) {
          if (slots[k].reqs.empty() || slots[k].state != 1) continue;
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
          if (!slots[k].reqs.empty()) continue;
          if (!form_batch(k)) break; // the head waits for memory
          admitted.push_back(k);
          ++inflight;
        }
        if (stop && queue.empty() && inflight == 0) break;
        if (admitted.empty() && !progress)
          cv_work.wait_for(lk, std::chrono::microseconds(inflight ? 20 : 2000));
      }
      for (const int k : admitted) {
        const cudaError_t e = issue(k);
        std::lock_guard<std::mutex> lk(mu);
        if (e == cudaSuccess)
          slots[k].state = 1;
        else
          finish(k, SGX_ERR_CUDA, std::string("sgx_server: ") + cudaGetErrorString(e));
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
    if (!sgx::pte_model(cfg->eos_list[k].type))
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
  q->bytes = sgx::Layout(r.nmat, r.ncell, s.mixed()).total;
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
    inflight += static_cast<int>(sl.reqs.size());
  out->inflight = inflight;
  out->batches = s.batches;
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
