// Served form: the GB300 counterpart of ReconstructionRunner
// (LM/ReconstructionRunner.java:140-593, 599-748, 753-829).
//
// * Admission: a stack is admitted into a slot (pinned host staging + device raw/output
//   buffers) of its channel's size class, so that a 512^2 stack does not hold a 1024^2
//   slot. At open the slots are sized from the free HBM (cudaMemGetInfo, less a headroom
//   for other users of the device) and hbm_budget_bytes, at most max_inflight per class;
//   the classes take the memory in equal shares of bytes (a class of small stacks gets
//   more slots than one of large stacks). After every refit the free HBM is read again and
//   classes below max_inflight grow. A class without a free slot returns FSIM_EBUSY
//   instead of dropping frames silently (the reference counts misses when its queue is
//   full, :140-150), while other classes still admit.
// * Continuous batching: a worker thread takes every pending stack (up to max_batch) and
//   launches one fused batch (H2D, reconstruction, D2H) on the next of `streams` CUDA
//   streams; stacks arriving while batches run are taken by the next launch, so batches
//   overlap on the device. Completion is signalled by a host callback on the stream.
// * Refit: every refit_every stacks of a channel, ParameterRefitThread.doRefit runs on the
//   device (estimate_core, live mode) on a side stream and thread, then the channel's
//   inactive plan is rebuilt and swapped in (double-buffered filters, so batches in
//   flight keep reading the tables they were launched with).
#include <algorithm>
#include <chrono>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <string>
#include <map>
#include <memory>
#include <mutex>
#include <thread>
#include <vector>

#include "common.cuh"
#include "estimate.cuh"
#include "recon.cuh"
#include "runtime.cuh"
#include "sim_host.h"


using namespace fsim;
using clk = std::chrono::steady_clock;

// Host copies of whole stacks and images (megabytes each) split over a few threads: with
// one thread, memcpy bandwidth of a single core bounds the served throughput.
class CopyPool {
 public:
  explicit CopyPool(int n) {
    for (int i = 0; i < n; i++) th_.emplace_back([this] { loop(); });
  }
  ~CopyPool() {
    {
      std::lock_guard<std::mutex> g(mu_);
      stop_ = true;
    }
    cv_.notify_all();
    for (auto& t : th_) t.join();
  }
  void copy(void* dst, const void* src, size_t bytes) {
    constexpr size_t kMin = (size_t)1 << 20;
    const size_t parts = std::min(th_.size() + 1, (bytes + kMin - 1) / kMin);
    if (parts <= 1) {
      std::memcpy(dst, src, bytes);
      return;
    }
    const size_t per = ((bytes / parts) + 63) & ~(size_t)63;
    Latch latch;
    latch.left = (int)parts - 1;
    {
      std::lock_guard<std::mutex> g(mu_);
      for (size_t k = 1; k < parts; k++) {
        const size_t off = k * per;
        if (off >= bytes) {
          latch.left--;
          continue;
        }
        q_.push_back(Task{(char*)dst + off, (const char*)src + off, std::min(per, bytes - off), &latch});
      }
    }
    cv_.notify_all();
    std::memcpy(dst, src, std::min(per, bytes));
    std::unique_lock<std::mutex> lk(latch.mu);
    latch.cv.wait(lk, [&] { return latch.left == 0; });
  }

 private:
  struct Latch {
    std::mutex mu;
    std::condition_variable cv;
    int left = 0;
  };
  struct Task {
    char* dst;
    const char* src;
    size_t n;
    Latch* latch;
  };
  void loop() {
    for (;;) {
      Task t;
      {
        std::unique_lock<std::mutex> lk(mu_);
        cv_.wait(lk, [&] { return stop_ || !q_.empty(); });
        if (q_.empty()) return;
        t = q_.front();
        q_.pop_front();
      }
      std::memcpy(t.dst, t.src, t.n);
      std::lock_guard<std::mutex> g(t.latch->mu);
      if (--t.latch->left == 0) t.latch->cv.notify_all();
    }
  }
  std::vector<std::thread> th_;
  std::deque<Task> q_;
  std::mutex mu_;
  std::condition_variable cv_;
  bool stop_ = false;
};

static double now_ms() {
  return std::chrono::duration<double, std::milli>(clk::now().time_since_epoch()).count();
}

struct fsim_server {
  struct Channel {
    fsim_sim_param prm{};
    Plan* plans[2] = {nullptr, nullptr};
    int active = 0;
    cudaEvent_t last_use[2] = {nullptr, nullptr};
    uint64_t count = 0;
    bool refit_busy = false;
    void* d_refit_raw = nullptr;
    size_t raw_bytes = 0;
    int cls = 0;  // slot class (stack and image size)
  };
  struct SlotClass {
    size_t raw_bytes = 0, out_bytes = 0;
    int n_channels = 0;
    int total = 0;  // slots allocated (at most max_inflight)
    std::vector<int> free;
  };
  enum { FREE = 0, FILLING, PENDING, RUNNING, DONE, COLLECTING };
  struct Slot {
    void* h_raw = nullptr;
    void* d_raw = nullptr;
    float* h_out = nullptr;
    float* d_out = nullptr;
    int state = FREE;
    bool cancelled = false;  // the client gave the ticket up; the slot frees itself when done
    uint64_t ticket = 0;
    int channel = 0;
    int cls = 0;
    double t_submit = 0, t_done = 0;
  };
  struct Done {
    fsim_server* s;
    std::vector<int> slots;
  };

  fsim_serve_config cfg{};
  std::vector<Channel> ch;
  std::vector<Slot> slots;  // capacity max_inflight, reserved at open: slots never move
  std::vector<SlotClass> cls;
  std::deque<int> pending;
  std::map<uint64_t, int> by_ticket;
  uint64_t next_ticket = 1;
  std::vector<cudaStream_t> streams;
  std::vector<void*> ws;
  size_t ws_bytes = 0;
  int rr = 0;
  cudaStream_t refit_stream = nullptr;
  std::mutex mu;
  std::condition_variable cv_work, cv_done, cv_refit;
  std::thread worker, refitter;
  std::unique_ptr<CopyPool> copier;
  std::deque<int> refit_queue;
  bool stop = false;
  // stats
  std::vector<double> lat;
  uint64_t submitted = 0, completed = 0, rejected = 0, refits = 0, cancelled = 0;
  double t_first = 0, t_last = 0;
};

static void CUDART_CB on_batch_done(void* arg) {
  auto* d = static_cast<fsim_server::Done*>(arg);
  fsim_server* s = d->s;
  {
    std::lock_guard<std::mutex> g(s->mu);
    double t = now_ms();
    for (int i : d->slots) {
      auto& sl = s->slots[i];
      sl.state = fsim_server::DONE;
      sl.t_done = t;
      s->lat.push_back(t - sl.t_submit);
      s->completed++;
      s->t_last = t;
      if (sl.cancelled) {
        sl.state = fsim_server::FREE;
        sl.cancelled = false;
        s->by_ticket.erase(sl.ticket);
        sl.ticket = 0;
        s->cls[sl.cls].free.push_back(i);
      }
    }
  }
  s->cv_done.notify_all();
  delete d;
}

static void worker_loop(fsim_server* s) {
  cudaSetDevice(ctx().device);
  for (;;) {
    std::vector<int> batch;
    int si;
    {
      std::unique_lock<std::mutex> lk(s->mu);
      s->cv_work.wait(lk, [&] { return s->stop || !s->pending.empty(); });
      if (s->stop && s->pending.empty()) return;
      while (!s->pending.empty() && (int)batch.size() < s->cfg.max_batch) {
        int i = s->pending.front();
        s->pending.pop_front();
        s->slots[i].state = fsim_server::RUNNING;
        batch.push_back(i);
      }
      si = s->rr;
      s->rr = (s->rr + 1) % (int)s->streams.size();
    }
    cudaStream_t st = s->streams[si];
    std::vector<fsim_job> jobs(batch.size());
    std::vector<int> used_plan(batch.size());
    std::vector<int> refit_now;
    {
      std::lock_guard<std::mutex> g(s->mu);
      for (size_t k = 0; k < batch.size(); k++) {
        auto& sl = s->slots[batch[k]];
        auto& c = s->ch[sl.channel];
        used_plan[k] = c.active;
        jobs[k] = fsim_job{reinterpret_cast<const fsim_plan*>(c.plans[c.active]), sl.d_raw, sl.d_out, nullptr};
        c.count++;
        if (s->cfg.refit_every > 0 && c.count % s->cfg.refit_every == 0 && !c.refit_busy) {
          c.refit_busy = true;
          refit_now.push_back(batch[k]);
        }
      }
    }
    for (int i : batch) {
      auto& sl = s->slots[i];
      cudaMemcpyAsync(sl.d_raw, sl.h_raw, s->ch[sl.channel].raw_bytes, cudaMemcpyHostToDevice, st);
    }
    // the job table goes to the device as launch parameters (no copy engine, so the passes
    // never wait behind another stream's uploads)
    std::vector<JobDesc> table(batch.size());
    int rc = recon_batch(jobs.data(), (int)jobs.size(), s->ws[si], s->ws_bytes, st, table.data(), true);
    for (size_t k = 0; k < batch.size(); k++) {
      auto& sl = s->slots[batch[k]];
      auto& c = s->ch[sl.channel];
      const size_t W = 2 * (size_t)c.prm.w;
      cudaMemcpyAsync(sl.h_out, sl.d_out, W * W * sizeof(float), cudaMemcpyDeviceToHost, st);
      cudaEventRecord(c.last_use[used_plan[k]], st);
    }
    // the newest stack of a channel due for a refit is copied for the refit thread
    for (int i : refit_now) {
      auto& sl = s->slots[i];
      auto& c = s->ch[sl.channel];
      cudaMemcpyAsync(c.d_refit_raw, sl.d_raw, c.raw_bytes, cudaMemcpyDeviceToDevice, st);
    }
    if (!refit_now.empty()) {
      cudaStreamSynchronize(st);
      std::lock_guard<std::mutex> g(s->mu);
      for (int i : refit_now) s->refit_queue.push_back(s->slots[i].channel);
      s->cv_refit.notify_all();
    }
    if (rc != FSIM_OK) {
      std::lock_guard<std::mutex> g(s->mu);
      for (int i : batch) s->slots[i].state = fsim_server::DONE;  // waiter sees the error
      s->cv_done.notify_all();
      continue;
    }
    auto* d = new fsim_server::Done{s, batch};
    cudaLaunchHostFunc(st, on_batch_done, d);
  }
}

static void grow_slots(fsim_server* s);

static void refit_loop(fsim_server* s) {
  cudaSetDevice(ctx().device);
  for (;;) {
    int c;
    {
      std::unique_lock<std::mutex> lk(s->mu);
      s->cv_refit.wait(lk, [&] { return s->stop || !s->refit_queue.empty(); });
      if (s->stop) return;
      c = s->refit_queue.front();
      s->refit_queue.pop_front();
    }
    auto& chn = s->ch[c];
    fsim_sim_param p = chn.prm;
    const int N = p.w, frames = p.nr_dirs * p.nr_phases;
    const size_t n = (size_t)N * N;
    cudaStream_t st = s->refit_stream;
    int rc = FSIM_OK;
    // ParameterRefitThread.doRefit on the device: damp, FFT, estimate (live mode)
    float2* spec = nullptr;
    if (fsim::dev_alloc_async(&spec, sizeof(float2) * n * frames, st) != cudaSuccess) rc = FSIM_EOOM;
    if (!rc) {
      extern int refit_spectra(const fsim_sim_param* p, const void* raw, int input_u16, int fade, float2* spec,
                               cudaStream_t st);
      rc = refit_spectra(&p, chn.d_refit_raw, s->cfg.input_type == FSIM_INPUT_U16, s->cfg.fade_px, spec, st);
    }
    if (!rc) {
      std::vector<const float2*> ptrs(frames);
      for (int i = 0; i < frames; i++) ptrs[i] = spec + i * n;
      rc = estimate_core(&p, ptrs.data(), 1, .8, true, nullptr, st);
    }
    if (spec) cudaFreeAsync(spec, st);
    if (!rc) {
      const int spare = 1 - chn.active;
      cudaEventSynchronize(chn.last_use[spare]);  // no batch in flight reads the spare tables
      chn.plans[spare]->prm = p;
      rc = chn.plans[spare]->build_live(st);
      if (!rc) {
        std::lock_guard<std::mutex> g(s->mu);
        chn.prm = p;
        chn.active = spare;
        s->refits++;
      }
    }
    {
      std::lock_guard<std::mutex> g(s->mu);
      chn.refit_busy = false;
    }
    grow_slots(s);  // the free HBM may have changed since open
  }
}

// damp + forward FFT of a raw stack on the device (shared with the estimation entry points)
namespace fsim {
std::vector<float> fade_vector(int w, int h, int px);
int fft2d_device(float2* data, int w, int h, bool inverse, cudaStream_t stream, int batch);
int raw_to_cplx_device(float2* y, const void* raw, int input_u16, const float* damp, size_t n, size_t frames,
                       cudaStream_t st);
}  // namespace fsim
int refit_spectra(const fsim_sim_param* p, const void* raw, int input_u16, int fade, float2* spec, cudaStream_t st) {
  const int N = p->w, frames = p->nr_dirs * p->nr_phases;
  const size_t n = (size_t)N * N;
  float* damp = nullptr;
  if (fade > 0) {
    std::vector<float> h = fade_vector(N, N, fade);
    FSIM_CUDA(fsim::dev_alloc_async(&damp, sizeof(float) * n, st));
    FSIM_CUDA(cudaMemcpyAsync(damp, h.data(), sizeof(float) * n, cudaMemcpyHostToDevice, st));
    FSIM_CUDA(cudaStreamSynchronize(st));
  }
  int rc = raw_to_cplx_device(spec, raw, input_u16, damp, n, frames, st);
  if (!rc) rc = fft2d_device(spec, N, N, false, st, frames);
  if (damp) cudaFreeAsync(damp, st);
  return rc;
}

extern "C" {

static int serve_setup(fsim_server* s, const fsim_serve_config* cfg, const fsim_sim_param* channels,
                       int n_channels);

int fsim_serve_open(fsim_server** out, const fsim_serve_config* cfg, const fsim_sim_param* channels, int n_channels) {
  FSIM_REQUIRE(out && cfg && channels && n_channels > 0, FSIM_EINVAL, "serve_open: bad arguments");
  *out = nullptr;
  FSIM_REQUIRE(cfg->max_batch > 0 && cfg->max_inflight > 0 && cfg->streams > 0, FSIM_EINVAL,
               "serve_open: max_batch, max_inflight and streams must be positive");
  FSIM_REQUIRE(cfg->input_type == FSIM_INPUT_U16 || cfg->input_type == FSIM_INPUT_F32, FSIM_EINVAL,
               "serve_open: unknown input type %d", cfg->input_type);
  for (int c = 0; c < n_channels; c++) {
    int rc = validate_param(&channels[c]);
    if (rc) return rc;
    FSIM_REQUIRE(live_size_supported(channels[c].w), FSIM_EINVAL, "serve_open: channel %d: unsupported size %d", c,
                 channels[c].w);
  }
  int rc = ensure_init();
  if (rc) return rc;
  auto* s = new fsim_server();
  rc = serve_setup(s, cfg, channels, n_channels);
  if (rc) {
    const std::string msg = last_error();
    fsim_serve_close(s);  // releases whatever was set up
    set_error("%s", msg.c_str());
    return rc;
  }
  s->worker = std::thread(worker_loop, s);
  s->refitter = std::thread(refit_loop, s);
  *out = s;
  return FSIM_OK;
}

}  // extern "C"

// Device memory left to other users of the GPU when slots are sized from its free HBM.
static size_t hbm_headroom(size_t total) { return std::max(total / 16, (size_t)1 << 30); }

// One slot of class c: pinned host staging and device buffers; false when an allocation fails
// (whatever was allocated is released).
static bool alloc_slot(const fsim_server::SlotClass& c, fsim_server::Slot* sl) {
  if (cudaMallocHost(&sl->h_raw, c.raw_bytes) != cudaSuccess) sl->h_raw = nullptr;
  if (sl->h_raw && cudaMallocHost(&sl->h_out, c.out_bytes) != cudaSuccess) sl->h_out = nullptr;
  if (sl->h_out && fsim::dev_alloc(&sl->d_raw, c.raw_bytes) != cudaSuccess) sl->d_raw = nullptr;
  if (sl->d_raw && fsim::dev_alloc(&sl->d_out, c.out_bytes) != cudaSuccess) sl->d_out = nullptr;
  if (sl->d_out) return true;
  if (sl->d_raw) cudaFree(sl->d_raw);
  if (sl->h_out) cudaFreeHost(sl->h_out);
  if (sl->h_raw) cudaFreeHost(sl->h_raw);
  sl->h_raw = sl->d_raw = nullptr;
  sl->h_out = sl->d_out = nullptr;
  cudaGetLastError();  // a failed allocation is not a sticky error
  return false;
}

// Bytes of device memory slots may still take: the free HBM less the headroom, and within
// hbm_budget_bytes (which also covers the batch workspaces) when that is set.
static size_t slot_room(fsim_server* s, size_t slot_bytes_now) {
  size_t free_b = 0, total_b = 0;
  if (cudaMemGetInfo(&free_b, &total_b) != cudaSuccess) return 0;
  const size_t head = hbm_headroom(total_b);
  size_t room = free_b > head ? free_b - head : 0;
  if (s->cfg.hbm_budget_bytes > 0) {
    const size_t used = s->ws_bytes * s->streams.size() + slot_bytes_now;
    room = std::min(room, s->cfg.hbm_budget_bytes > used ? s->cfg.hbm_budget_bytes - used : (size_t)0);
  }
  return room;
}

// Adds slots, one at a time to the class with the fewest bytes of slots among those below
// max_inflight, while the room allows.
// Called at open (no other thread yet) and after refits (slots only grow up to the reserved
// capacity, so the indices and references of existing slots stay valid).
static void grow_slots(fsim_server* s) {
  for (;;) {
    int c = -1;
    size_t slot_bytes_now = 0;
    {
      std::lock_guard<std::mutex> g(s->mu);
      if (s->slots.size() >= s->slots.capacity()) return;
      int best = -1;
      size_t best_bytes = 0;
      for (size_t k = 0; k < s->cls.size(); k++) {
        const auto& sc = s->cls[k];
        const size_t bytes = (sc.raw_bytes + sc.out_bytes) * sc.total;
        slot_bytes_now += bytes;
        if (sc.total < s->cfg.max_inflight && (best < 0 || bytes < best_bytes)) {
          best = (int)k;
          best_bytes = bytes;
        }
      }
      c = best;
    }
    if (c < 0) return;
    const auto& sc = s->cls[c];  // the class list is fixed after open
    if (slot_room(s, slot_bytes_now) < sc.raw_bytes + sc.out_bytes) return;
    fsim_server::Slot sl;
    if (!alloc_slot(sc, &sl)) return;
    sl.cls = c;
    std::lock_guard<std::mutex> g(s->mu);
    s->slots.push_back(sl);
    s->cls[c].total++;
    s->cls[c].free.push_back((int)s->slots.size() - 1);
  }
}

extern "C" {

static int serve_setup(fsim_server* s, const fsim_serve_config* cfg, const fsim_sim_param* channels,
                       int n_channels) {
  int rc = FSIM_OK;
  s->cfg = *cfg;
  s->ch.resize(n_channels);
  size_t max_ws = 0;
  const int in_sz = cfg->input_type == FSIM_INPUT_U16 ? 2 : 4;
  for (int c = 0; c < n_channels; c++) {
    auto& chn = s->ch[c];
    chn.prm = channels[c];
    for (int k = 0; k < 2; k++) {
      fsim_plan* pl = nullptr;
      rc = fsim_plan_create(&pl, &channels[c], FSIM_PATH_LIVE, cfg->input_type, cfg->fade_px, 0.0);
      if (rc) return rc;
      chn.plans[k] = reinterpret_cast<Plan*>(pl);
      cudaEventCreateWithFlags(&chn.last_use[k], cudaEventDisableTiming);
    }
    const size_t N = channels[c].w;
    chn.raw_bytes = N * N * channels[c].nr_dirs * channels[c].nr_phases * in_sz;
    FSIM_CUDA(fsim::dev_alloc(&chn.d_refit_raw, chn.raw_bytes));
    const size_t out_bytes = 4 * N * N * sizeof(float);
    // size classes: channels with the same stack and image size share slots
    int k = 0;
    while (k < (int)s->cls.size() && !(s->cls[k].raw_bytes == chn.raw_bytes && s->cls[k].out_bytes == out_bytes)) k++;
    if (k == (int)s->cls.size()) {
      s->cls.emplace_back();
      s->cls[k].raw_bytes = chn.raw_bytes;
      s->cls[k].out_bytes = out_bytes;
    }
    s->cls[k].n_channels++;
    chn.cls = k;
    max_ws = std::max(max_ws, (plan_ws(chn.plans[0]) + 255) & ~(size_t)255);
  }
  s->ws_bytes = ((sizeof(JobDesc) * cfg->max_batch + 255) & ~(size_t)255) + max_ws * cfg->max_batch;
  if (cfg->hbm_budget_bytes > 0)
    FSIM_REQUIRE(cfg->hbm_budget_bytes > s->ws_bytes * cfg->streams, FSIM_EOOM,
                 "serve_open: HBM budget %zu below the batch workspaces %zu", cfg->hbm_budget_bytes,
                 s->ws_bytes * cfg->streams);
  s->streams.resize(cfg->streams);
  s->ws.resize(cfg->streams);
  for (int k = 0; k < cfg->streams; k++) {
    FSIM_CUDA(cudaStreamCreateWithFlags(&s->streams[k], cudaStreamNonBlocking));
    FSIM_CUDA(fsim::dev_alloc(&s->ws[k], s->ws_bytes));
  }
  FSIM_CUDA(cudaStreamCreateWithFlags(&s->refit_stream, cudaStreamNonBlocking));
  s->slots.reserve((size_t)cfg->max_inflight * s->cls.size());
  grow_slots(s);
  for (size_t k = 0; k < s->cls.size(); k++)
    FSIM_REQUIRE(s->cls[k].total > 0, FSIM_EOOM,
                 "serve_open: no device memory for a slot of %zu + %zu bytes (class %zu) within the free HBM "
                 "and the budget", s->cls[k].raw_bytes, s->cls[k].out_bytes, k);
  FSIM_CUDA(cudaDeviceSynchronize());
  const unsigned hw = std::max(1u, std::thread::hardware_concurrency());
  s->copier.reset(new CopyPool((int)std::min(7u, std::max(1u, hw / 4))));
  return FSIM_OK;
}

int fsim_serve_submit(fsim_server* s, int channel, const void* raw_host, size_t raw_bytes, uint64_t* ticket) {
  FSIM_REQUIRE(s && raw_host && ticket, FSIM_EINVAL, "serve_submit: bad arguments");
  FSIM_REQUIRE(channel >= 0 && channel < (int)s->ch.size(), FSIM_EINVAL, "serve_submit: no channel %d", channel);
  FSIM_REQUIRE(raw_bytes == s->ch[channel].raw_bytes, FSIM_EINVAL,
               "serve_submit: stack of %zu bytes for channel %d, which takes %zu (%d frames of %d x %d)", raw_bytes,
               channel, s->ch[channel].raw_bytes, s->ch[channel].prm.nr_dirs * s->ch[channel].prm.nr_phases,
               s->ch[channel].prm.w, s->ch[channel].prm.w);
  int i;
  {
    std::lock_guard<std::mutex> g(s->mu);
    auto& fl = s->cls[s->ch[channel].cls].free;
    if (fl.empty()) {
      s->rejected++;
      set_error("serve_submit: no free slot for channel %d (all %d slots of its %d x %d class in flight)", channel,
                s->cls[s->ch[channel].cls].total, s->ch[channel].prm.w, s->ch[channel].prm.w);
      return FSIM_EBUSY;
    }
    i = fl.back();
    fl.pop_back();
    auto& sl = s->slots[i];
    sl.state = fsim_server::FILLING;
    sl.channel = channel;
    sl.ticket = s->next_ticket++;
    sl.t_submit = now_ms();
    if (s->submitted == 0) s->t_first = sl.t_submit;
    s->submitted++;
    s->by_ticket[sl.ticket] = i;
    *ticket = sl.ticket;
  }
  s->copier->copy(s->slots[i].h_raw, raw_host, s->ch[channel].raw_bytes);
  {
    std::lock_guard<std::mutex> g(s->mu);
    s->slots[i].state = fsim_server::PENDING;
    s->pending.push_back(i);
  }
  s->cv_work.notify_one();
  return FSIM_OK;
}

int fsim_serve_wait(fsim_server* s, uint64_t ticket, float* out_host, int timeout_ms, double* latency_ms) {
  FSIM_REQUIRE(s && out_host, FSIM_EINVAL, "serve_wait: bad arguments");
  std::unique_lock<std::mutex> lk(s->mu);
  auto it = s->by_ticket.find(ticket);
  FSIM_REQUIRE(it != s->by_ticket.end(), FSIM_ENOTFOUND, "serve_wait: unknown ticket %llu", (unsigned long long)ticket);
  const int i = it->second;
  auto& sl = s->slots[i];
  FSIM_REQUIRE(!sl.cancelled, FSIM_ENOTFOUND, "serve_wait: ticket %llu was cancelled", (unsigned long long)ticket);
  // the slot may be cancelled by another thread (and reused) while this one waits
  auto mine = [&] { return sl.ticket == ticket && !sl.cancelled; };
  if (!s->cv_done.wait_for(lk, std::chrono::milliseconds(timeout_ms),
                           [&] { return !mine() || sl.state == fsim_server::DONE; })) {
    set_error("serve_wait: ticket %llu not done after %d ms", (unsigned long long)ticket, timeout_ms);
    return FSIM_ETIMEOUT;
  }
  FSIM_REQUIRE(mine(), FSIM_ENOTFOUND, "serve_wait: ticket %llu was cancelled while waiting",
               (unsigned long long)ticket);
  // copy out without the server lock: the ticket is retired first, so no other call
  // (wait, cancel) can reach this slot until it is back on the free list
  const size_t W = 2 * (size_t)s->ch[sl.channel].prm.w;
  if (latency_ms) *latency_ms = sl.t_done - sl.t_submit;
  sl.state = fsim_server::COLLECTING;
  s->by_ticket.erase(ticket);
  lk.unlock();
  s->copier->copy(out_host, sl.h_out, W * W * sizeof(float));
  lk.lock();
  sl.state = fsim_server::FREE;
  sl.ticket = 0;
  s->cls[sl.cls].free.push_back(i);
  return FSIM_OK;
}

int fsim_serve_cancel(fsim_server* s, uint64_t ticket) {
  FSIM_REQUIRE(s, FSIM_EINVAL, "serve_cancel: null server");
  std::lock_guard<std::mutex> g(s->mu);
  auto it = s->by_ticket.find(ticket);
  FSIM_REQUIRE(it != s->by_ticket.end(), FSIM_ENOTFOUND, "serve_cancel: unknown ticket %llu",
               (unsigned long long)ticket);
  const int i = it->second;
  auto& sl = s->slots[i];
  FSIM_REQUIRE(!sl.cancelled, FSIM_ENOTFOUND, "serve_cancel: ticket %llu already cancelled", (unsigned long long)ticket);
  s->cancelled++;
  if (sl.state == fsim_server::PENDING) {
    // not started: drop it from the queue and free the slot now
    s->pending.erase(std::find(s->pending.begin(), s->pending.end(), i));
    sl.state = fsim_server::FREE;
    sl.ticket = 0;
    s->by_ticket.erase(it);
    s->cls[sl.cls].free.push_back(i);
  } else if (sl.state == fsim_server::DONE) {
    sl.state = fsim_server::FREE;
    sl.ticket = 0;
    s->by_ticket.erase(it);
    s->cls[sl.cls].free.push_back(i);
  } else {
    sl.cancelled = true;  // on the GPU: the completion callback frees the slot
  }
  s->cv_done.notify_all();
  return FSIM_OK;
}

int fsim_serve_stats_get(fsim_server* s, fsim_serve_stats* out) {
  FSIM_REQUIRE(s && out, FSIM_EINVAL, "serve_stats: bad arguments");
  std::lock_guard<std::mutex> g(s->mu);
  std::memset(out, 0, sizeof(*out));
  out->submitted = s->submitted;
  out->completed = s->completed;
  out->rejected = s->rejected;
  out->refits = s->refits;
  out->cancelled = s->cancelled;
  if (!s->lat.empty()) {
    std::vector<double> v = s->lat;
    std::sort(v.begin(), v.end());
    auto pct = [&](double q) { return v[std::min(v.size() - 1, (size_t)(q * (v.size() - 1) + 0.5))]; };
    out->p50_ms = pct(0.50);
    out->p99_ms = pct(0.99);
    double sum = 0;
    for (double x : v) sum += x;
    out->mean_ms = sum / v.size();
    out->max_ms = v.back();
  }
  out->wall_s = (s->t_last - s->t_first) / 1000.0;
  out->recon_per_s = out->wall_s > 0 ? s->completed / out->wall_s : 0;
  return FSIM_OK;
}

int fsim_serve_capacity(fsim_server* s, int channel, int* slots, int* free_slots) {
  FSIM_REQUIRE(s && channel >= 0 && channel < (int)s->ch.size(), FSIM_EINVAL, "serve_capacity: bad arguments");
  std::lock_guard<std::mutex> g(s->mu);
  const auto& sc = s->cls[s->ch[channel].cls];
  if (slots) *slots = sc.total;
  if (free_slots) *free_slots = (int)sc.free.size();
  return FSIM_OK;
}

int fsim_serve_params(fsim_server* s, int channel, fsim_sim_param* out) {
  FSIM_REQUIRE(s && out && channel >= 0 && channel < (int)s->ch.size(), FSIM_EINVAL, "serve_params: bad arguments");
  std::lock_guard<std::mutex> g(s->mu);
  *out = s->ch[channel].prm;
  return FSIM_OK;
}

int fsim_serve_close(fsim_server* s) {
  if (!s) return FSIM_OK;
  {
    std::lock_guard<std::mutex> g(s->mu);
    s->stop = true;
  }
  s->cv_work.notify_all();
  s->cv_refit.notify_all();
  if (s->worker.joinable()) s->worker.join();
  if (s->refitter.joinable()) s->refitter.join();
  cudaDeviceSynchronize();
  for (auto& sl : s->slots) {
    if (sl.h_raw) cudaFreeHost(sl.h_raw);
    if (sl.h_out) cudaFreeHost(sl.h_out);
    if (sl.d_raw) cudaFree(sl.d_raw);
    if (sl.d_out) cudaFree(sl.d_out);
  }
  for (size_t k = 0; k < s->streams.size(); k++) {
    if (s->ws[k]) cudaFree(s->ws[k]);
    if (s->streams[k]) cudaStreamDestroy(s->streams[k]);
  }
  for (auto& c : s->ch) {
    for (int k = 0; k < 2; k++) {
      if (c.plans[k]) fsim_plan_destroy(reinterpret_cast<fsim_plan*>(c.plans[k]));
      if (c.last_use[k]) cudaEventDestroy(c.last_use[k]);
    }
    if (c.d_refit_raw) cudaFree(c.d_refit_raw);
  }
  if (s->refit_stream) cudaStreamDestroy(s->refit_stream);
  delete s;
  return FSIM_OK;
}

}  // extern "C"
