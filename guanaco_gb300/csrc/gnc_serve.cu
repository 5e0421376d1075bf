// Request server: continuous batching of whole-series FBP requests on one GPU.
//
// A scheduler thread admits requests.  Callers queue requests
// (gnc_server_submit); the scheduler admits a request when a slot (a CUDA
// stream) is free and its plan fits in the device-memory budget, and enqueues
// on that slot: the parameter upload, the input copy, the device work and the
// volume copy, followed by a host callback that marks the slot finished.
// Requests on different slots overlap on the device.
//
// Plans are cached by shape (plan_key).  A request with no idle plan of its
// shape gets its slot, memory and cache entry from the scheduler and is handed
// to a builder thread, which creates the plan, runs the request as direct
// launches (creating the FFT tables and kernel attributes they need) and then
// captures the same launch sequence once as a CUDA graph; meanwhile the
// scheduler keeps admitting requests of known shapes.  Later requests of that
// shape replay the graph after uploading their own parameter block (the
// kernels read per-request values from device memory).  Only the builder
// captures, on its own stream.
//
// Admission takes the oldest queued request that can run now; when it cannot
// (no idle plan of its shape and not enough memory even after releasing idle
// plans), up to kLookAhead younger requests may pass it, at most kMaxSkips
// times in a row, after which the scheduler waits for memory to free up.
//
// Memory: plans and request buffers come from a CUDA memory pool of the
// server (stream-ordered cudaMallocFromPoolAsync / cudaFreeAsync on the
// builder's stream, the pool keeping up to the budget reserved), and the
// page-locked parameter blocks of released plans are kept for reuse, so
// creating and releasing plans while requests run neither synchronises the
// device (as cudaMalloc, cudaFree and cudaFreeHost do) nor copies
// synchronously.
//
// Locking: gn_server::mu guards the queue, the request table, the slots'
// state, the cache bookkeeping and the statistics.  No CUDA call is made while
// it is held (a host callback waiting for it would otherwise hold up a device
// synchronisation inside the CUDA call).
#include <algorithm>
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

#include "gnc_common.cuh"
#include "gnc_plan_hooks.h"

namespace {

constexpr int kLookAhead = 16;
constexpr int kMaxSkips = 32;

struct Cached {
  std::string key;
  gnc_fbp_plan *plan = nullptr;
  float *d_in = nullptr, *d_out = nullptr;
  unsigned char *h_params = nullptr;  // page-locked parameter block
  size_t h_bytes = 0;                  // its size
  cudaGraphExec_t exec = nullptr;
  size_t bytes = 0;
  bool busy = false;
  bool ready = false;  // created (and its memory held)
  uint64_t last_use = 0;
};

struct Request {
  uint64_t id = 0;
  gnc_fbp_desc desc{};
  std::vector<float> angles, centre;
  std::vector<double> slabs, weights;
  const float *h_in = nullptr;
  float *h_out = nullptr;
  size_t in_bytes = 0, out_bytes = 0, bytes = 0;
  std::string key;
  int status = GNC_OK;
  bool done = false;
  int graph = 0, device_error = 0;
  double t_submit = 0, t_start = 0, t_done = 0;
  std::string error;
};

struct Slot {
  cudaStream_t s = nullptr;
  Request *req = nullptr;
  Cached *plan = nullptr;
  int *h_err = nullptr;  // page-locked copy of the plan's device error word
  bool finished = false;
  double t_done = 0;
  gnc_server *srv = nullptr;
};

}  // namespace

struct gnc_server {
  int device = 0;
  size_t budget = 0, used = 0;
  std::vector<Slot> slots;
  std::deque<Request *> queue;
  std::unordered_map<uint64_t, std::unique_ptr<Request>> reqs;
  // ids of finished requests in the order they finished, for
  // gnc_server_wait_any (ids already collected by gnc_server_wait are skipped)
  std::deque<uint64_t> finished;
  std::vector<std::unique_ptr<Cached>> cache;
  std::mutex mu;
  std::condition_variable cv_sched, cv_done, cv_build;
  std::thread th, th_build;
  bool stop = false, wake = false, stop_build = false;
  struct Build {  // a request whose new plan the builder creates
    Slot *sl;
    Request *r;
    Cached *c;
    std::vector<std::unique_ptr<Cached>> victims;  // idle plans released for its memory
  };
  std::deque<Build> builds;
  uint64_t next_id = 1, tick = 0;
  int head_skips = 0;
  std::chrono::steady_clock::time_point t0 = std::chrono::steady_clock::now();
  cudaStream_t s_cap = nullptr;  // the builder's stream: captures, pool allocations and frees
  cudaMemPool_t pool = nullptr;
  std::mutex host_mu;  // page-locked parameter blocks for reuse: (bytes, pointer)
  std::vector<std::pair<size_t, unsigned char *>> host_blocks;
  gnc_server_stats st{};

  double now() const {
    return std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
  }
};

namespace {

void CUDART_CB on_done(void *arg) {
  Slot *sl = static_cast<Slot *>(arg);
  gnc_server *S = sl->srv;
  std::lock_guard<std::mutex> lk(S->mu);
  sl->finished = true;
  sl->t_done = S->now();
  S->wake = true;
  S->cv_sched.notify_one();
}

// Without the lock, on the builder thread (or at destruction): the plan's
// memory goes back to the pool on the builder's stream (its last use on a
// slot has finished: only idle plans are released), its page-locked block to
// the reuse list.
void release(gnc_server *S, Cached *c) {
  if (c->exec) cudaGraphExecDestroy(c->exec);
  if (c->plan) gnc_fbp_plan_destroy(c->plan);
  if (c->d_in) cudaFreeAsync(c->d_in, S->s_cap);
  if (c->d_out) cudaFreeAsync(c->d_out, S->s_cap);
  if (c->h_params) {
    std::lock_guard<std::mutex> lk(S->host_mu);
    S->host_blocks.emplace_back(c->h_bytes, c->h_params);
  }
  c->exec = nullptr;
  c->plan = nullptr;
  c->d_in = c->d_out = nullptr;
  c->h_params = nullptr;
}

// A page-locked block of at least `bytes` (a released one of up to twice the
// size when there is one); its size in *got.
unsigned char *host_block(gnc_server *S, size_t bytes, size_t *got) {
  {
    std::lock_guard<std::mutex> lk(S->host_mu);
    for (size_t i = 0; i < S->host_blocks.size(); ++i)
      if (S->host_blocks[i].first >= bytes && S->host_blocks[i].first <= 2 * bytes + 4096) {
        unsigned char *p = S->host_blocks[i].second;
        *got = S->host_blocks[i].first;
        S->host_blocks.erase(S->host_blocks.begin() + i);
        return p;
      }
  }
  unsigned char *p = nullptr;
  const size_t rounded = (bytes + 4095) & ~(size_t)4095;
  if (cudaHostAlloc((void **)&p, rounded, cudaHostAllocDefault) != cudaSuccess) return nullptr;
  *got = rounded;
  return p;
}

Cached *find_idle(gnc_server *S, const std::string &key) {
  for (auto &c : S->cache)
    if (c->ready && !c->busy && c->key == key) return c.get();
  return nullptr;
}

// Whether the shape has a plan (running a request, or being built).
bool has_plan(gnc_server *S, const std::string &key) {
  for (auto &c : S->cache)
    if (c->key == key) return true;
  return false;
}

size_t idle_bytes(gnc_server *S) {
  size_t b = 0;
  for (auto &c : S->cache)
    if (c->ready && !c->busy) b += c->bytes;
  return b;
}

// Under the lock: r has finished; gnc_server_wait_any reports it in this order.
void mark_done(gnc_server *S, Request *r) {
  r->done = true;
  S->finished.push_back(r->id);
  if (S->finished.size() > 2 * S->reqs.size() + 64) {  // drop ids collected by id
    std::deque<uint64_t> keep;
    for (uint64_t id : S->finished)
      if (S->reqs.count(id)) keep.push_back(id);
    S->finished.swap(keep);
  }
}

// Under the lock: finish the requests whose slots reported back, in the
// order they finished.
void reap(gnc_server *S) {
  std::vector<Slot *> fin;
  for (Slot &sl : S->slots)
    if (sl.req && sl.finished) fin.push_back(&sl);
  std::sort(fin.begin(), fin.end(), [](const Slot *a, const Slot *b) { return a->t_done < b->t_done; });
  for (Slot *slp : fin) {
    Slot &sl = *slp;
    Request *r = sl.req;
    r->t_done = sl.t_done;
    r->device_error = *sl.h_err != 0;
    if (r->device_error) {
      r->status = GNC_ERR_CUDA;
      r->error = "a bounded wait in a kernel gave up (device error word set)";
    }
    mark_done(S, r);
    sl.plan->busy = false;
    sl.plan->last_use = ++S->tick;
    sl.req = nullptr;
    sl.plan = nullptr;
    sl.finished = false;
    S->st.in_flight--;
    if (r->status == GNC_OK)
      S->st.completed++;
    else
      S->st.failed++;
  }
  S->cv_done.notify_all();
}

void fail(gnc_server *S, Request *r, int status, const std::string &msg) {
  r->status = status;
  r->error = msg;
  r->t_done = S->now();
  mark_done(S, r);
  S->st.failed++;
}

// Without the lock, on the builder thread: plan, buffers and parameter block
// of a new cache entry, from the pool on the builder's stream; ready for use
// on any stream when this returns.
int create_entry(gnc_server *S, Cached *c, const Request *r) {
  int st = gnc::plan_create_pooled(&r->desc, S->pool, S->s_cap, &c->plan);
  if (st != GNC_OK) return st;
  cudaError_t e = cudaMallocFromPoolAsync((void **)&c->d_in, r->in_bytes, S->pool, S->s_cap);
  if (e == cudaSuccess)
    e = cudaMallocFromPoolAsync((void **)&c->d_out, r->out_bytes, S->pool, S->s_cap);
  if (e == cudaSuccess) {
    c->h_params = host_block(S, gnc::plan_param_bytes(c->plan), &c->h_bytes);
    if (!c->h_params) e = cudaErrorMemoryAllocation;
  }
  // the allocations and the plan's parameter upload are ordered on the
  // builder's stream; the slots' streams use them after this
  if (e == cudaSuccess) e = cudaStreamSynchronize(S->s_cap);
  if (e != cudaSuccess) {
    gnc::set_error(std::string("gnc_server: ") + cudaGetErrorString(e));
    return e == cudaErrorMemoryAllocation ? GNC_ERR_OUT_OF_MEMORY : GNC_ERR_CUDA;
  }
  return GNC_OK;
}

// Without the lock: the launch sequence of c, captured for replay.
void capture(gnc_server *S, Cached *c) {
  if (cudaStreamBeginCapture(S->s_cap, cudaStreamCaptureModeRelaxed) != cudaSuccess) return;
  const int st = gnc_fbp_execute(c->plan, c->d_in, c->d_out, S->s_cap);
  cudaGraph_t g = nullptr;
  const cudaError_t e = cudaStreamEndCapture(S->s_cap, &g);
  if (st == GNC_OK && e == cudaSuccess && g) {
    cudaGraphExec_t x = nullptr;
    if (cudaGraphInstantiate(&x, g, 0) == cudaSuccess) c->exec = x;
  }
  if (g) cudaGraphDestroy(g);
  cudaGetLastError();  // a failed capture leaves direct launches in use
}

// Without the lock: everything one request puts on its slot's stream; with
// may_capture (the builder), a plan without a graph captures one afterwards.
// On failure, whatever was already queued for the request has finished when
// this returns, so the caller may hand the slot, the plan and the caller's
// host buffers back.
int enqueue(gnc_server *S, Slot *sl, Request *r, Cached *c, bool may_capture) {
  cudaStream_t s = sl->s;
  auto drained = [s](int status) {
    cudaStreamSynchronize(s);
    return status;
  };
  int st = gnc::plan_set_request(c->plan, &r->desc, c->h_params, s);
  if (st != GNC_OK) return drained(st);
  cudaError_t e = cudaMemcpyAsync(c->d_in, r->h_in, r->in_bytes, cudaMemcpyHostToDevice, s);
  if (e == cudaSuccess) {
    if (c->exec) {
      e = cudaGraphLaunch(c->exec, s);
      r->graph = 1;
    } else {
      st = gnc_fbp_execute(c->plan, c->d_in, c->d_out, s);
      if (st != GNC_OK) return drained(st);
    }
  }
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(r->h_out, c->d_out, r->out_bytes, cudaMemcpyDeviceToHost, s);
  int *derr = gnc::plan_error_word(c->plan);
  if (e == cudaSuccess) e = cudaMemcpyAsync(sl->h_err, derr, sizeof(int), cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess) e = cudaMemsetAsync(derr, 0, sizeof(int), s);
  if (e == cudaSuccess) e = cudaLaunchHostFunc(s, on_done, sl);
  if (e != cudaSuccess) {
    gnc::set_error(std::string("gnc_server: ") + cudaGetErrorString(e));
    return drained(GNC_ERR_CUDA);
  }
  if (may_capture && !c->exec) capture(S, c);
  return GNC_OK;
}

// Under the lock on entry and exit; drops it around the CUDA work.
void admit(gnc_server *S, std::unique_lock<std::mutex> &lk) {
  while (!S->stop && !S->queue.empty()) {
    Slot *sl = nullptr;
    for (Slot &x : S->slots)
      if (!x.req) {
        sl = &x;
        break;
      }
    if (!sl) return;
    Request *r = nullptr;
    Cached *c = nullptr;
    size_t qi = 0;
    const size_t idle = idle_bytes(S);
    for (; qi < S->queue.size() && qi < (size_t)kLookAhead; ++qi) {
      if (qi > 0 && S->head_skips >= kMaxSkips) break;
      Request *q = S->queue[qi];
      c = find_idle(S, q->key);
      // a shape whose plan is busy or being built waits for it rather than
      // building a second copy: under load a copy per overlapping request
      // multiplied the builds (each a direct run and a capture on the same
      // GPU), which slowed service and so made more requests overlap
      if (!c && has_plan(S, q->key)) continue;
      if (c || S->used - idle + q->bytes <= S->budget) {
        r = q;
        break;
      }
    }
    if (!r) return;
    S->head_skips = qi == 0 ? 0 : S->head_skips + 1;
    S->queue.erase(S->queue.begin() + qi);
    // reserve: an idle plan of the shape, or new memory after releasing idle plans
    std::vector<std::unique_ptr<Cached>> victims;
    bool fresh = false;
    if (!c) {
      fresh = true;
      while (S->used + r->bytes > S->budget) {
        auto lru = S->cache.end();
        for (auto it = S->cache.begin(); it != S->cache.end(); ++it)
          if ((*it)->ready && !(*it)->busy &&
              (lru == S->cache.end() || (*it)->last_use < (*lru)->last_use))
            lru = it;
        if (lru == S->cache.end()) break;  // cannot happen: checked above
        S->used -= (*lru)->bytes;
        victims.push_back(std::move(*lru));
        S->cache.erase(lru);
        S->st.plans_evicted++;
      }
      auto nc = std::make_unique<Cached>();
      nc->key = r->key;
      nc->bytes = r->bytes;
      c = nc.get();
      S->cache.push_back(std::move(nc));
      S->used += r->bytes;
    }
    c->busy = true;
    sl->req = r;
    sl->plan = c;
    sl->finished = false;
    r->t_start = S->now();
    S->st.in_flight++;
    S->st.peak_in_flight = std::max(S->st.peak_in_flight, S->st.in_flight);
    if (fresh) {  // the builder creates the plan and runs the request
      S->builds.push_back(gnc_server::Build{sl, r, c, std::move(victims)});
      S->cv_build.notify_one();
      continue;
    }
    lk.unlock();
    std::string msg;
    const bool replay = c->exec != nullptr;
    int st = enqueue(S, sl, r, c, false);
    if (st != GNC_OK) msg = gnc::last_error();
    lk.lock();
    if (st != GNC_OK) {
      c->busy = false;
      sl->req = nullptr;
      sl->plan = nullptr;
      S->st.in_flight--;
      fail(S, r, st, msg);
      S->cv_done.notify_all();
      continue;
    }
    if (replay)
      S->st.graph_launches++;
    else
      S->st.direct_launches++;
  }
}

// The builder thread: new plans, their first (direct) run and their capture.
void build_loop(gnc_server *S) {
  cudaSetDevice(S->device);
  std::unique_lock<std::mutex> lk(S->mu);
  for (;;) {
    S->cv_build.wait(lk, [S] { return S->stop_build || !S->builds.empty(); });
    if (S->builds.empty()) break;  // stop_build and nothing left
    gnc_server::Build b = std::move(S->builds.front());
    S->builds.pop_front();
    lk.unlock();
    for (auto &v : b.victims) release(S, v.get());
    b.victims.clear();
    std::string msg;
    int st = create_entry(S, b.c, b.r);
    if (st != GNC_OK) msg = gnc::last_error();
    if (st == GNC_OK) {
      st = enqueue(S, b.sl, b.r, b.c, true);
      if (st != GNC_OK) msg = gnc::last_error();
    }
    if (st != GNC_OK) release(S, b.c);
    lk.lock();
    if (st != GNC_OK) {
      S->used -= b.c->bytes;
      Cached *c = b.c;
      S->cache.erase(std::find_if(S->cache.begin(), S->cache.end(),
                                  [c](const std::unique_ptr<Cached> &p) { return p.get() == c; }));
      b.sl->req = nullptr;
      b.sl->plan = nullptr;
      S->st.in_flight--;
      fail(S, b.r, st, msg);
      S->cv_done.notify_all();
      S->wake = true;  // the slot and the memory are free again
      S->cv_sched.notify_one();
      continue;
    }
    b.c->ready = true;
    S->st.plans_created++;
    S->st.direct_launches++;
    S->wake = true;  // requests that waited for this shape can be admitted
    S->cv_sched.notify_one();
  }
}

void run(gnc_server *S) {
  cudaSetDevice(S->device);
  std::unique_lock<std::mutex> lk(S->mu);
  for (;;) {
    S->cv_sched.wait(lk, [S] { return S->stop || S->wake; });
    S->wake = false;
    reap(S);
    if (S->stop) {
      bool busy = false;
      for (Slot &sl : S->slots) busy = busy || sl.req != nullptr;
      if (!busy) break;
      continue;
    }
    admit(S, lk);
  }
}

}  // namespace

using gnc::set_error;

namespace {
// Under the lock: a finished request's outcome into info, then forgotten.
int collect(gnc_server *S, std::unordered_map<uint64_t, std::unique_ptr<Request>>::iterator it,
            gnc_request_info *info) {
  Request *r = it->second.get();
  if (info) {
    info->status = r->status;
    info->graph = r->graph;
    info->device_error = r->device_error;
    info->t_submit = r->t_submit;
    info->t_start = r->t_start;
    info->t_done = r->t_done;
  }
  const int status = r->status;
  if (status != GNC_OK) gnc::set_error(r->error);
  S->reqs.erase(it);
  return status;
}
}  // namespace

extern "C" {

int gnc_server_create(size_t budget_bytes, int slots, gnc_server **server) {
  if (!server || slots < 1 || slots > 64 || budget_bytes == 0) {
    set_error("gnc_server_create: ASSERT (server != nullptr && 1 <= slots <= 64 && budget > 0) failed");
    return GNC_ERR_INVALID_ARGUMENT;
  }
  *server = nullptr;
  int n = 0;
  if (cudaGetDeviceCount(&n) != cudaSuccess || n == 0) {
    cudaGetLastError();
    set_error("gnc_server_create: no CUDA device");
    return GNC_ERR_DEVICE;
  }
  auto S = std::make_unique<gnc_server>();
  cudaGetDevice(&S->device);
  S->budget = budget_bytes;
  S->slots.resize(slots);
  cudaError_t e = cudaStreamCreateWithFlags(&S->s_cap, cudaStreamNonBlocking);
  if (e == cudaSuccess) {
    // the plans' pool: keeps what is freed (up to the budget) instead of
    // returning it to the driver, so later plans are carved from it
    cudaMemPoolProps props{};
    props.allocType = cudaMemAllocationTypePinned;
    props.location.type = cudaMemLocationTypeDevice;
    props.location.id = S->device;
    e = cudaMemPoolCreate(&S->pool, &props);
    if (e == cudaSuccess) {
      unsigned long long keep = (unsigned long long)budget_bytes;
      e = cudaMemPoolSetAttribute(S->pool, cudaMemPoolAttrReleaseThreshold, &keep);
    }
  }
  for (Slot &sl : S->slots) {
    sl.srv = S.get();
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&sl.s, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaHostAlloc((void **)&sl.h_err, sizeof(int), cudaHostAllocDefault);
  }
  if (e != cudaSuccess) {
    set_error(std::string("gnc_server_create: ") + cudaGetErrorString(e));
    for (Slot &sl : S->slots) {
      if (sl.s) cudaStreamDestroy(sl.s);
      if (sl.h_err) cudaFreeHost(sl.h_err);
    }
    if (S->s_cap) cudaStreamDestroy(S->s_cap);
    if (S->pool) cudaMemPoolDestroy(S->pool);
    return GNC_ERR_CUDA;
  }
  S->st.budget_bytes = budget_bytes;
  S->st.slots = slots;
  gnc_server *raw = S.release();
  raw->th = std::thread(run, raw);
  raw->th_build = std::thread(build_loop, raw);
  *server = raw;
  return GNC_OK;
}

int gnc_server_destroy(gnc_server *S) {
  if (!S) return GNC_OK;
  {
    std::lock_guard<std::mutex> lk(S->mu);
    S->stop = true;
    S->wake = true;
    for (Request *r : S->queue) fail(S, r, GNC_ERR_INVALID_ARGUMENT, "gnc_server: destroyed");
    S->queue.clear();
    S->cv_sched.notify_one();
    S->cv_done.notify_all();
  }
  S->th.join();  // returns once every slot, those being built included, is done
  {
    std::lock_guard<std::mutex> lk(S->mu);
    S->stop_build = true;
    S->cv_build.notify_one();
  }
  S->th_build.join();
  cudaSetDevice(S->device);
  for (Slot &sl : S->slots) cudaStreamSynchronize(sl.s);
  for (auto &c : S->cache) release(S, c.get());
  cudaStreamSynchronize(S->s_cap);  // the pool's frees
  for (auto &hb : S->host_blocks) cudaFreeHost(hb.second);
  if (S->pool) cudaMemPoolDestroy(S->pool);
  for (Slot &sl : S->slots) {
    cudaStreamDestroy(sl.s);
    cudaFreeHost(sl.h_err);
  }
  cudaStreamDestroy(S->s_cap);
  delete S;
  return GNC_OK;
}

int gnc_server_submit(gnc_server *S, const gnc_fbp_desc *desc, const float *h_input,
                      float *h_volume, uint64_t *id) {
  if (!S || !desc || !h_input || !h_volume || !id) {
    set_error("gnc_server_submit: ASSERT (server && desc && h_input && h_volume && id) failed");
    return GNC_ERR_INVALID_ARGUMENT;
  }
  const int st = gnc::desc_check(desc);
  if (st != GNC_OK) return st;
  auto r = std::make_unique<Request>();
  r->desc = *desc;
  const size_t T = desc->num_angles, H = desc->height, D = desc->num_defocus;
  r->angles.assign(desc->angles, desc->angles + T);
  r->desc.angles = r->angles.data();
  if (desc->centre) {
    r->centre.assign(desc->centre, desc->centre + H);
    r->desc.centre = r->centre.data();
  }
  if (desc->slab_defocus) {
    r->slabs.assign(desc->slab_defocus, desc->slab_defocus + D);
    r->desc.slab_defocus = r->slabs.data();
  }
  if (desc->weights) {
    r->weights.assign(desc->weights, desc->weights + T);
    r->desc.weights = r->weights.data();
  }
  r->h_in = h_input;
  r->h_out = h_volume;
  r->in_bytes = T * (desc->input == GNC_INPUT_CORRECTED ? D : 1) * H * desc->width * sizeof(float);
  r->out_bytes = H * desc->grid_height * desc->grid_width * sizeof(float);
  r->bytes = gnc::plan_bytes(desc);
  r->key = gnc::plan_key(desc);
  if (r->bytes > S->budget) {
    set_error("gnc_server_submit: the request needs " + std::to_string(r->bytes) +
              " device bytes, more than the server's budget of " + std::to_string(S->budget));
    return GNC_ERR_OUT_OF_MEMORY;
  }
  std::lock_guard<std::mutex> lk(S->mu);
  if (S->stop) {
    set_error("gnc_server_submit: the server is being destroyed");
    return GNC_ERR_INVALID_ARGUMENT;
  }
  r->id = S->next_id++;
  r->t_submit = S->now();
  *id = r->id;
  S->queue.push_back(r.get());
  S->reqs.emplace(r->id, std::move(r));
  S->st.submitted++;
  S->wake = true;
  S->cv_sched.notify_one();
  return GNC_OK;
}

int gnc_server_wait(gnc_server *S, uint64_t id, double timeout_s, gnc_request_info *info) {
  if (!S) {
    set_error("gnc_server_wait: ASSERT (server != nullptr) failed");
    return GNC_ERR_INVALID_ARGUMENT;
  }
  std::unique_lock<std::mutex> lk(S->mu);
  auto it = S->reqs.find(id);
  if (it == S->reqs.end()) {
    set_error("gnc_server_wait: unknown request id " + std::to_string(id));
    return GNC_ERR_INVALID_ARGUMENT;
  }
  Request *r = it->second.get();
  auto pred = [r] { return r->done; };
  if (timeout_s < 0)
    S->cv_done.wait(lk, pred);
  else
    S->cv_done.wait_for(lk, std::chrono::duration<double>(timeout_s), pred);
  if (!r->done) return GNC_ERR_PENDING;
  return collect(S, it, info);
}

int gnc_server_wait_any(gnc_server *S, double timeout_s, uint64_t *id, gnc_request_info *info) {
  if (!S || !id) {
    set_error("gnc_server_wait_any: ASSERT (server != nullptr && id != nullptr) failed");
    return GNC_ERR_INVALID_ARGUMENT;
  }
  std::unique_lock<std::mutex> lk(S->mu);
  auto ready = [S] {
    while (!S->finished.empty() && !S->reqs.count(S->finished.front())) S->finished.pop_front();
    return !S->finished.empty();
  };
  // nothing submitted and uncollected: nothing to wait for
  auto pred = [S, &ready] { return ready() || S->reqs.empty(); };
  if (timeout_s < 0)
    S->cv_done.wait(lk, pred);
  else
    S->cv_done.wait_for(lk, std::chrono::duration<double>(timeout_s), pred);
  if (!ready()) return GNC_ERR_PENDING;
  *id = S->finished.front();
  S->finished.pop_front();
  return collect(S, S->reqs.find(*id), info);
}

double gnc_server_now(const gnc_server *S) { return S ? S->now() : 0.0; }

int gnc_server_get_stats(gnc_server *S, gnc_server_stats *out) {
  if (!S || !out) {
    set_error("gnc_server_get_stats: ASSERT (server && stats) failed");
    return GNC_ERR_INVALID_ARGUMENT;
  }
  std::lock_guard<std::mutex> lk(S->mu);
  *out = S->st;
  out->bytes_in_use = S->used;
  out->cached_plans = (int)S->cache.size();
  out->queued = (int)S->queue.size();
  return GNC_OK;
}

}  // extern "C"
