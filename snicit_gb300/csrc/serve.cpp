// Serving loop: continuous batching of inference requests.
//
// The reference's beyond driver runs fixed rounds of `batch_size` samples
// (src/beyond/SNICIT/SNICIT.hpp:494-641); here requests of any size (1 to the
// slot capacity) arrive at any time:
//
//  * sdnn_submit copies the request's rows into the server and queues it;
//  * a dispatcher thread hands queued requests, in arrival order, to the first
//    free slot while they fit: a slot holds the rows its buffers already have
//    room for, plus what the device's free memory, read at that moment
//    (cudaMemGetInfo, less what other slots are about to take), allows it to
//    grow by ("admitted by free HBM"); the slot's worker grows its buffers
//    before the pass;
//  * each slot owns an engine (its stream and row buffers; the weights are
//    the model engine's, one device copy for all slots) and a
//    worker thread that runs one pass: the slot's requests gathered back to
//    back, one inference over all their rows (in SNICIT mode the clustering
//    spans every co-resident request), the dense head, results copied out;
//    slots run concurrently, so requests that arrive while a pass is on the
//    GPU start in the next free slot and their work overlaps on the device;
//  * every row is computed independently of the other rows of its pass, so a
//    request's result does not depend on what it was batched with (bitwise in
//    the plain modes; in SNICIT mode within the FP32 rounding of the residue
//    form, the category set exactly).
#include <atomic>
#include <chrono>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <memory>
#include <mutex>
#include <string>
#include <thread>
#include <unordered_map>
#include <vector>

#include <cuda_runtime.h>

#include "sdnn_internal.h"
#include "snicit_gb300.h"

namespace sdnn {
int engine_prepare(sdnn_engine* e, int64_t rows);
int engine_share_weights(sdnn_engine* dst, sdnn_engine* src);
sdnn_config engine_config(const sdnn_engine* e);
cudaStream_t engine_stream(const sdnn_engine* e);
float* engine_input(sdnn_engine* e);
int32_t* engine_flags(sdnn_engine* e);
int engine_run(sdnn_engine* e, int64_t rows);
int engine_check(sdnn_engine* e);
std::vector<int32_t> engine_final_positions(const sdnn_engine* e);
bool engine_head(sdnn_engine* e, const float* Hp, const float* hb, int32_t H, int64_t rows,
                 float* logits, int32_t* argmax);
std::string engine_error(const sdnn_engine* e);
void engine_set_error(sdnn_engine* e, const std::string& msg);
}  // namespace sdnn

namespace {

using Clock = std::chrono::steady_clock;

struct Request {
  uint64_t id = 0;
  int64_t rows = 0;
  std::vector<float> in;
  std::vector<int32_t> flags, argmax;
  std::vector<float> logits;
  Clock::time_point t_submit, t_start, t_done;
  int status = SDNN_OK;
  bool done = false;
};

struct Slot {
  sdnn_engine* eng = nullptr;
  int64_t cap = 0;        // rows the buffers below hold
  int64_t grow_to = 0;    // set at admission: rows to grow to before the pass
  int64_t reserved = 0;   // device bytes set aside for that growth
  float* h_in = nullptr;  // pinned staging: rows x N
  float* h_logits = nullptr;
  int32_t* h_argmax = nullptr;
  int32_t* h_flags = nullptr;
  float* d_logits = nullptr;
  int32_t* d_argmax = nullptr;
  std::vector<std::shared_ptr<Request>> work;
  bool busy = false;
  std::thread worker;
};

}  // namespace

struct sdnn_server {
  sdnn_server_config cfg{};
  int N = 0, H = 0;
  int64_t cap = 0;           // largest admissible request (rows)
  int64_t per_row = 0;       // device bytes per row of a slot
  int64_t reserved = 0;      // device bytes admitted but not yet allocated
  sdnn_engine* model = nullptr;
  std::vector<std::unique_ptr<Slot>> slots;
  float* d_head = nullptr;  // head by final position, N x H
  float* d_hb = nullptr;
  std::mutex mu;
  std::condition_variable cv_dispatch, cv_slot, cv_done;
  std::deque<std::shared_ptr<Request>> queue;
  int64_t queued_rows = 0;
  std::unordered_map<uint64_t, std::shared_ptr<Request>> table;
  uint64_t next_id = 1;
  bool stop = false;
  std::thread dispatcher;
  std::string err;
  // counters
  int64_t passes = 0, rows_done = 0, requests_done = 0, max_rows_in_pass = 0;
};

namespace {

// Grows a slot's row buffers (engine, pinned staging, head outputs) to `rows`.
int grow_slot(sdnn_server* sv, Slot& slot, int64_t rows) {
  if (rows <= slot.cap) return SDNN_OK;
  const size_t N = (size_t)sv->N, H = (size_t)sv->H;
  int rc = sdnn::engine_prepare(slot.eng, rows);
  if (rc) return rc;
  if (slot.h_in) cudaFreeHost(slot.h_in);
  if (slot.h_flags) cudaFreeHost(slot.h_flags);
  if (slot.h_logits) cudaFreeHost(slot.h_logits);
  if (slot.h_argmax) cudaFreeHost(slot.h_argmax);
  if (slot.d_logits) cudaFree(slot.d_logits);
  if (slot.d_argmax) cudaFree(slot.d_argmax);
  slot.h_in = slot.h_logits = nullptr;
  slot.h_flags = slot.h_argmax = slot.d_argmax = nullptr;
  slot.d_logits = nullptr;
  slot.cap = 0;
  bool ok = cudaMallocHost((void**)&slot.h_in, sizeof(float) * (size_t)rows * N) == cudaSuccess;
  ok = ok && cudaMallocHost((void**)&slot.h_flags, sizeof(int32_t) * (size_t)rows) == cudaSuccess;
  if (H > 0) {
    ok = ok && cudaMallocHost((void**)&slot.h_logits, sizeof(float) * (size_t)rows * H) == cudaSuccess;
    ok = ok && cudaMallocHost((void**)&slot.h_argmax, sizeof(int32_t) * (size_t)rows) == cudaSuccess;
    ok = ok && cudaMalloc((void**)&slot.d_logits, sizeof(float) * (size_t)rows * H) == cudaSuccess;
    ok = ok && cudaMalloc((void**)&slot.d_argmax, sizeof(int32_t) * (size_t)rows) == cudaSuccess;
  }
  if (!ok) {
    cudaGetLastError();
    return SDNN_ERR_OOM;
  }
  slot.cap = rows;
  return SDNN_OK;
}

void run_pass(sdnn_server* sv, Slot& slot) {
  const int N = sv->N, H = sv->H;
  int64_t total = 0;
  for (auto& r : slot.work) total += r->rows;
  int grc = grow_slot(sv, slot, std::max(total, slot.grow_to));
  {
    std::lock_guard<std::mutex> lock(sv->mu);
    sv->reserved -= slot.reserved;
    slot.reserved = 0;
    slot.grow_to = 0;
  }
  if (grc != SDNN_OK) {
    const auto t = Clock::now();
    std::lock_guard<std::mutex> lock(sv->mu);
    for (auto& r : slot.work) {
      r->status = grc;
      r->t_start = r->t_done = t;
      std::vector<float>().swap(r->in);
      r->done = true;
    }
    slot.work.clear();
    slot.busy = false;
    return;
  }
  total = 0;
  for (auto& r : slot.work) {
    std::memcpy(slot.h_in + total * N, r->in.data(), sizeof(float) * (size_t)r->rows * N);
    total += r->rows;
  }
  const auto t0 = Clock::now();
  for (auto& r : slot.work) r->t_start = t0;
  sdnn_engine* e = slot.eng;
  cudaStream_t s = sdnn::engine_stream(e);
  int rc = SDNN_OK;
  if (cudaMemcpyAsync(sdnn::engine_input(e), slot.h_in, sizeof(float) * (size_t)total * N,
                      cudaMemcpyHostToDevice, s) != cudaSuccess)
    rc = SDNN_ERR_CUDA;
  if (rc == SDNN_OK) rc = sdnn::engine_run(e, total);
  if (rc == SDNN_OK && H > 0 &&
      !sdnn::engine_head(e, sv->d_head, sv->d_hb, H, total, slot.d_logits, slot.d_argmax))
    rc = SDNN_ERR_UNSUPPORTED;
  if (rc == SDNN_OK) {
    bool ok = cudaMemcpyAsync(slot.h_flags, sdnn::engine_flags(e), sizeof(int32_t) * total,
                              cudaMemcpyDeviceToHost, s) == cudaSuccess;
    if (H > 0) {
      ok = ok && cudaMemcpyAsync(slot.h_logits, slot.d_logits, sizeof(float) * total * H,
                                 cudaMemcpyDeviceToHost, s) == cudaSuccess;
      ok = ok && cudaMemcpyAsync(slot.h_argmax, slot.d_argmax, sizeof(int32_t) * total,
                                 cudaMemcpyDeviceToHost, s) == cudaSuccess;
    }
    if (!ok) rc = SDNN_ERR_CUDA;
  }
  if (rc == SDNN_OK) rc = sdnn::engine_check(e);  // synchronizes the slot's stream
  const auto t1 = Clock::now();
  int64_t off = 0;
  for (auto& r : slot.work) {
    r->status = rc;
    if (rc == SDNN_OK) {
      r->flags.assign(slot.h_flags + off, slot.h_flags + off + r->rows);
      if (H > 0) {
        r->logits.assign(slot.h_logits + off * H, slot.h_logits + (off + r->rows) * H);
        r->argmax.assign(slot.h_argmax + off, slot.h_argmax + off + r->rows);
      }
    }
    std::vector<float>().swap(r->in);
    r->t_done = t1;
    off += r->rows;
  }
  std::lock_guard<std::mutex> lock(sv->mu);
  for (auto& r : slot.work) r->done = true;
  sv->passes++;
  sv->rows_done += total;
  sv->requests_done += (int64_t)slot.work.size();
  sv->max_rows_in_pass = std::max(sv->max_rows_in_pass, total);
  slot.work.clear();
  slot.busy = false;
}

void worker_main(sdnn_server* sv, Slot* slot) {
  cudaSetDevice(sdnn::engine_config(slot->eng).device);
  for (;;) {
    {
      std::unique_lock<std::mutex> lock(sv->mu);
      sv->cv_slot.wait(lock, [&] { return sv->stop || (slot->busy && !slot->work.empty()); });
      if (sv->stop && !(slot->busy && !slot->work.empty())) return;
    }
    run_pass(sv, *slot);
    sv->cv_done.notify_all();
    sv->cv_dispatch.notify_all();
  }
}

void dispatcher_main(sdnn_server* sv) {
  const auto delay = std::chrono::microseconds(sv->cfg.max_delay_us);
  std::unique_lock<std::mutex> lock(sv->mu);
  for (;;) {
    if (sv->stop) return;
    bool free_slot = false;
    for (auto& s : sv->slots) free_slot |= !s->busy;
    if (sv->queue.empty() || !free_slot) {
      sv->cv_dispatch.wait(lock);
      continue;
    }
    // batching window: an under-full pass waits for more requests until the
    // oldest queued one has waited max_delay_us
    if (delay.count() > 0 && sv->queued_rows < sv->cap) {
      const auto deadline = sv->queue.front()->t_submit + delay;
      if (Clock::now() < deadline) {
        sv->cv_dispatch.wait_until(lock, deadline);
        continue;
      }
    }
    bool admitted = false, any_busy = false;
    for (auto& s : sv->slots) any_busy |= s->busy;
    for (auto& s : sv->slots) {
      if (s->busy || sv->queue.empty()) continue;
      // rows this slot may take now: its buffers, plus what the free device
      // memory (read now, less the growth other slots were granted) allows
      int64_t allow = s->cap;
      if (allow < sv->cap) {
        size_t free_b = 0, total_b = 0;
        if (cudaMemGetInfo(&free_b, &total_b) == cudaSuccess) {
          const double frac =
              sv->cfg.memory_fraction > 0 ? std::min(sv->cfg.memory_fraction, 0.95) : 0.5;
          const double avail = (double)free_b * frac - (double)sv->reserved;
          if (avail > 0) allow += (int64_t)(avail / (double)sv->per_row);
        }
        allow = std::min(allow, sv->cap);
      }
      int64_t rows = 0;
      const size_t max_req = sv->cfg.max_requests_per_pass > 0
                                 ? (size_t)sv->cfg.max_requests_per_pass
                                 : sv->queue.size();
      while (!sv->queue.empty() && s->work.size() < max_req &&
             rows + sv->queue.front()->rows <= allow) {
        rows += sv->queue.front()->rows;
        s->work.push_back(sv->queue.front());
        sv->queue.pop_front();
      }
      if (s->work.empty() && !any_busy && !admitted) {
        // nothing fits and nothing runs that could free memory: the request
        // is not admissible now (SDNN_ERR_OOM), rather than waiting forever
        auto r = sv->queue.front();
        sv->queue.pop_front();
        sv->queued_rows -= r->rows;
        r->status = SDNN_ERR_OOM;
        r->t_start = r->t_done = Clock::now();
        std::vector<float>().swap(r->in);
        r->done = true;
        sv->cv_done.notify_all();
        continue;
      }
      sv->queued_rows -= rows;
      if (!s->work.empty()) {
        if (rows > s->cap) {
          // grow a little ahead (up to twice the pass) while memory allows
          s->grow_to = std::min(allow, std::max(rows, std::min(sv->cap, 2 * rows)));
          s->reserved = (s->grow_to - s->cap) * sv->per_row;
          sv->reserved += s->reserved;
        }
        s->busy = true;
        admitted = any_busy = true;
        sv->cv_slot.notify_all();
      }
    }
    if (!admitted && !sv->queue.empty()) sv->cv_dispatch.wait(lock);
  }
}

void destroy_server(sdnn_server* sv) {
  {
    std::lock_guard<std::mutex> lock(sv->mu);
    sv->stop = true;
  }
  sv->cv_dispatch.notify_all();
  sv->cv_slot.notify_all();
  if (sv->dispatcher.joinable()) sv->dispatcher.join();
  for (auto& s : sv->slots) {
    if (s->worker.joinable()) s->worker.join();
    if (s->h_in) cudaFreeHost(s->h_in);
    if (s->h_logits) cudaFreeHost(s->h_logits);
    if (s->h_argmax) cudaFreeHost(s->h_argmax);
    if (s->h_flags) cudaFreeHost(s->h_flags);
    if (s->d_logits) cudaFree(s->d_logits);
    if (s->d_argmax) cudaFree(s->d_argmax);
    if (s->eng) sdnn_destroy(s->eng);
  }
  if (sv->d_head) cudaFree(sv->d_head);
  if (sv->d_hb) cudaFree(sv->d_hb);
  delete sv;
}

}  // namespace

extern "C" {

int sdnn_server_config_default(sdnn_server_config* c) {
  if (!c) return SDNN_ERR_INVALID;
  std::memset(c, 0, sizeof(*c));
  c->slots = 2;
  c->head_outputs = 0;
  c->max_rows = 16384;
  c->memory_fraction = 0.25;
  c->max_pending = 1 << 16;
  return SDNN_OK;
}

int sdnn_server_create(sdnn_engine* model, const sdnn_server_config* cfg, const float* head_w,
                       const float* head_b, sdnn_server** out) {
  if (!model || !cfg || !out || cfg->slots < 1 || cfg->slots > 16 || cfg->head_outputs < 0 ||
      (cfg->head_outputs > 0 && (!head_w || !head_b)))
    return SDNN_ERR_INVALID;
  *out = nullptr;
  auto* sv = new (std::nothrow) sdnn_server();
  if (!sv) return SDNN_ERR_OOM;
  sv->cfg = *cfg;
  const sdnn_config mc = sdnn::engine_config(model);
  sv->N = mc.num_neurons;
  sv->H = cfg->head_outputs;
  if (cudaSetDevice(mc.device) != cudaSuccess) {
    delete sv;
    return SDNN_ERR_CUDA;
  }
  // device bytes per row of a slot: input, two layer buffers (the
  // materialise scratch is one of them), row lists/state (~64 B), logits
  sv->per_row = (int64_t)sv->N * 4 * 3 + 64 + (int64_t)sv->H * 4;
  sv->cap = cfg->max_rows > 0 ? std::min<int64_t>(cfg->max_rows, 1 << 20) : (1 << 20);
  sv->model = model;
  sdnn_config ec = mc;
  // slots start small and grow at admission, as free device memory allows
  const int64_t initial = std::min<int64_t>(sv->cap, 4096);
  ec.batch = initial;
  int rc = SDNN_OK;
  for (int i = 0; i < cfg->slots && rc == SDNN_OK; ++i) {
    auto slot = std::make_unique<Slot>();
    rc = sdnn_create(&ec, &slot->eng);
    if (rc == SDNN_OK) {
      rc = sdnn::engine_share_weights(slot->eng, model);
      if (rc) sv->err = sdnn::engine_error(slot->eng);
    }
    if (rc == SDNN_OK) {
      rc = grow_slot(sv, *slot, initial);
      if (rc) sv->err = sdnn::engine_error(slot->eng);
    }
    sv->slots.push_back(std::move(slot));
  }
  if (rc == SDNN_OK && sv->H > 0) {
    // the head by final neuron position (every slot packs the same placement)
    const std::vector<int32_t> pos = sdnn::engine_final_positions(sv->slots[0]->eng);
    std::vector<float> hp((size_t)sv->N * sv->H);
    for (int j = 0; j < sv->N; ++j) {
      const int p = pos.empty() ? j : pos[j];
      for (int k = 0; k < sv->H; ++k) hp[(size_t)p * sv->H + k] = head_w[(size_t)j * sv->H + k];
    }
    bool ok = cudaMalloc((void**)&sv->d_head, sizeof(float) * hp.size()) == cudaSuccess;
    ok = ok && cudaMalloc((void**)&sv->d_hb, sizeof(float) * sv->H) == cudaSuccess;
    ok = ok && cudaMemcpy(sv->d_head, hp.data(), sizeof(float) * hp.size(), cudaMemcpyHostToDevice) == cudaSuccess;
    ok = ok && cudaMemcpy(sv->d_hb, head_b, sizeof(float) * sv->H, cudaMemcpyHostToDevice) == cudaSuccess;
    if (!ok) {
      cudaGetLastError();
      rc = SDNN_ERR_OOM;
    }
  }
  if (rc != SDNN_OK) {
    sdnn::engine_set_error(model, "server: " + (sv->err.empty() ? std::string(sdnn_status_string(rc)) : sv->err));
    destroy_server(sv);
    return rc;
  }
  for (auto& s : sv->slots) s->worker = std::thread(worker_main, sv, s.get());
  sv->dispatcher = std::thread(dispatcher_main, sv);
  *out = sv;
  return SDNN_OK;
}

int sdnn_server_destroy(sdnn_server* sv) {
  if (!sv) return SDNN_OK;
  destroy_server(sv);
  return SDNN_OK;
}

int64_t sdnn_server_capacity(const sdnn_server* sv) { return sv ? sv->cap : 0; }

int sdnn_submit(sdnn_server* sv, const float* rows_host, int64_t rows, uint64_t* request_id) {
  if (!sv || !rows_host || rows <= 0 || !request_id) return SDNN_ERR_INVALID;
  if (rows > sv->cap) return SDNN_ERR_INVALID;  // larger than any slot: never admissible
  auto r = std::make_shared<Request>();
  r->rows = rows;
  r->in.assign(rows_host, rows_host + (size_t)rows * sv->N);
  r->t_submit = Clock::now();
  {
    std::lock_guard<std::mutex> lock(sv->mu);
    if ((int64_t)sv->queue.size() >= sv->cfg.max_pending) return SDNN_ERR_BUSY;
    r->id = sv->next_id++;
    sv->table[r->id] = r;
    sv->queue.push_back(r);
    sv->queued_rows += rows;
    *request_id = r->id;
  }
  sv->cv_dispatch.notify_all();
  return SDNN_OK;
}

static int take_result(sdnn_server* sv, const std::shared_ptr<Request>& r, int32_t* flags,
                       float* logits, int32_t* argmax, double* latency_s) {
  if (flags) std::memcpy(flags, r->flags.data(), sizeof(int32_t) * r->flags.size());
  if (logits && !r->logits.empty()) std::memcpy(logits, r->logits.data(), sizeof(float) * r->logits.size());
  if (argmax && !r->argmax.empty()) std::memcpy(argmax, r->argmax.data(), sizeof(int32_t) * r->argmax.size());
  if (latency_s) latency_s[0] = std::chrono::duration<double>(r->t_done - r->t_submit).count();
  sv->table.erase(r->id);
  return r->status;
}

int sdnn_poll(sdnn_server* sv, uint64_t id, int32_t* done, int32_t* flags, float* logits,
              int32_t* argmax, double* latency_s) {
  if (!sv || !done) return SDNN_ERR_INVALID;
  std::lock_guard<std::mutex> lock(sv->mu);
  auto it = sv->table.find(id);
  if (it == sv->table.end()) return SDNN_ERR_INVALID;
  *done = it->second->done ? 1 : 0;
  if (!*done) return SDNN_OK;
  return take_result(sv, it->second, flags, logits, argmax, latency_s);
}

int sdnn_wait(sdnn_server* sv, uint64_t id, int32_t* flags, float* logits, int32_t* argmax,
              double* latency_s) {
  if (!sv) return SDNN_ERR_INVALID;
  std::unique_lock<std::mutex> lock(sv->mu);
  auto it = sv->table.find(id);
  if (it == sv->table.end()) return SDNN_ERR_INVALID;
  auto r = it->second;
  sv->cv_done.wait(lock, [&] { return r->done; });
  return take_result(sv, r, flags, logits, argmax, latency_s);
}

int sdnn_server_get_stats(sdnn_server* sv, sdnn_server_stats* out) {
  if (!sv || !out) return SDNN_ERR_INVALID;
  std::lock_guard<std::mutex> lock(sv->mu);
  std::memset(out, 0, sizeof(*out));
  out->passes = sv->passes;
  out->rows = sv->rows_done;
  out->requests = sv->requests_done;
  out->max_rows_in_pass = sv->max_rows_in_pass;
  out->queued = (int64_t)sv->queue.size();
  for (auto& sl : sv->slots) out->slot_rows = std::max(out->slot_rows, sl->cap);
  out->slots = (int32_t)sv->slots.size();
  return SDNN_OK;
}

}  // extern "C"
