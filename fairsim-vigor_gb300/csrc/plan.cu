// C ABI of the fused reconstruction plans and batches.
#include <algorithm>
#include <cstring>
#include <mutex>
#include <vector>

#include "common.cuh"
#include "recon.cuh"
#include "runtime.cuh"
#include "sim_host.h"

struct fsim_plan : fsim::Plan {};

namespace fsim {

static size_t align256(size_t b) { return (b + 255) & ~(size_t)255; }

size_t plan_ws(const Plan* p) {
  return p->path == FSIM_PATH_LIVE ? p->workspace_bytes_live() : p->workspace_bytes();
}

// pinned staging blocks for the per-batch job tables, reused once their copy completed
struct Staging {
  void* ptr = nullptr;
  size_t bytes = 0;
  cudaEvent_t done = nullptr;
};
static std::mutex g_stage_mu;
static std::vector<Staging> g_stage;

static int get_staging(size_t bytes, Staging** out) {
  std::lock_guard<std::mutex> g(g_stage_mu);
  for (auto& s : g_stage) {
    if (s.bytes >= bytes && cudaEventQuery(s.done) == cudaSuccess) {
      *out = &s;
      return FSIM_OK;
    }
  }
  g_stage.emplace_back();
  Staging& s = g_stage.back();
  s.bytes = std::max<size_t>(bytes, 64 * 1024);
  FSIM_CUDA(cudaMallocHost(&s.ptr, s.bytes));
  FSIM_CUDA(cudaEventCreateWithFlags(&s.done, cudaEventDisableTiming));
  *out = &s;
  return FSIM_OK;
}

// Fill job tables and launch: jobs are grouped by (path, size) with one set of passes each.
int recon_batch(const fsim_job* jobs, int n, void* ws, size_t ws_bytes, cudaStream_t st, JobDesc* host_table,
                bool upload_table) {
  FSIM_REQUIRE(jobs && n > 0, FSIM_EINVAL, "recon_batch: no jobs");
  std::vector<int> order(n);
  for (int i = 0; i < n; i++) {
    FSIM_REQUIRE(jobs[i].plan && jobs[i].raw && jobs[i].out, FSIM_EINVAL, "job %d: null plan/raw/out", i);
    order[i] = i;
  }
  auto key = [&](int i) {
    const Plan* p = static_cast<const Plan*>(jobs[i].plan);
    return std::make_pair(p->path, p->prm.w);
  };
  std::stable_sort(order.begin(), order.end(), [&](int a, int b) { return key(a) < key(b); });
  size_t need = align256(sizeof(JobDesc) * n);
  for (int i = 0; i < n; i++) need += align256(plan_ws(static_cast<const Plan*>(jobs[i].plan)));
  FSIM_REQUIRE(ws && ws_bytes >= need, FSIM_EINVAL, "recon_batch: workspace %zu < required %zu", ws_bytes, need);
  char* base = (char*)ws;
  JobDesc* d_table = (JobDesc*)base;
  char* cur = base + align256(sizeof(JobDesc) * n);
  for (int k = 0; k < n; k++) {
    const fsim_job& jb = jobs[order[k]];
    const Plan* p = static_cast<const Plan*>(jb.plan);
    if (p->path == FSIM_PATH_LIVE)
      p->fill_job_live(host_table[k], jb.raw, jb.out, jb.widefield, cur);
    else
      p->fill_job(host_table[k], jb.raw, jb.out, jb.widefield, cur);
    cur += align256(plan_ws(p));
  }
  if (upload_table) FSIM_CUDA(cudaMemcpyAsync(d_table, host_table, sizeof(JobDesc) * n, cudaMemcpyHostToDevice, st));
  int k = 0;
  while (k < n) {
    const Plan* p0 = static_cast<const Plan*>(jobs[order[k]].plan);
    int e = k, maxA = 0, maxP = 0;
    while (e < n && key(order[e]) == key(order[k])) {
      maxA = std::max(maxA, static_cast<const Plan*>(jobs[order[e]].plan)->prm.nr_dirs);
      maxP = std::max(maxP, static_cast<const Plan*>(jobs[order[e]].plan)->prm.nr_phases);
      e++;
    }
    int rc = (p0->path == FSIM_PATH_LIVE) ? launch_live_size(p0->prm.w, d_table + k, e - k, maxA, st)
                                          : launch_offline_size(p0->prm.w, d_table + k, e - k, maxA, maxP, st);
    if (rc) return rc;
    k = e;
  }
  return FSIM_OK;
}

static bool g_prof_on = false;
static cudaEvent_t g_prof_ev[8];
static int g_prof_n = 0;
cudaEvent_t* profile_events() { return g_prof_on ? g_prof_ev : nullptr; }
void profile_mark(int n_passes) { g_prof_n = n_passes; }

size_t batch_workspace_bytes(const Plan* const* plans, int n) {
  size_t need = align256(sizeof(JobDesc) * n);
  for (int i = 0; i < n; i++) need += align256(plan_ws(plans[i]));
  return need;
}

}  // namespace fsim

using namespace fsim;

#define NEED_INIT()          \
  do {                       \
    int rc_ = ensure_init(); \
    if (rc_) return rc_;     \
  } while (0)

extern "C" {

int fsim_plan_create(fsim_plan** out, const fsim_sim_param* p, int path, int input_type, int fade_px, double bgr) {
  NEED_INIT();
  FSIM_REQUIRE(out, FSIM_EINVAL, "null output pointer");
  int rc = validate_param(p);
  if (rc) return rc;
  FSIM_REQUIRE(path == FSIM_PATH_OFFLINE || path == FSIM_PATH_LIVE, FSIM_EINVAL, "unknown path %d", path);
  FSIM_REQUIRE(input_type == FSIM_INPUT_F32 || input_type == FSIM_INPUT_U16, FSIM_EINVAL, "unknown input type");
  if (path == FSIM_PATH_OFFLINE)
    FSIM_REQUIRE(offline_size_supported(p->w), FSIM_EINVAL, "fused reconstruction: unsupported image size %d", p->w);
  else
    FSIM_REQUIRE(live_size_supported(p->w), FSIM_EINVAL, "live reconstruction: unsupported image size %d", p->w);
  FSIM_REQUIRE(p->nr_phases <= FSIM_MAX_PHASES && 2 * p->nr_bands - 1 <= 7, FSIM_EINVAL, "too many phases/bands");
  fsim_plan* pl = new fsim_plan();
  pl->prm = *p;
  pl->path = path;
  pl->input_type = input_type;
  pl->fade_px = fade_px;
  pl->bgr = bgr;
  rc = (path == FSIM_PATH_LIVE) ? pl->build_live(ctx().stream) : pl->build(ctx().stream);
  if (rc) {
    if (pl->dev) cudaFree(pl->dev);
    delete pl;
    return rc;
  }
  *out = pl;
  return FSIM_OK;
}

int fsim_plan_update(fsim_plan* plan, const fsim_sim_param* p) {
  NEED_INIT();
  FSIM_REQUIRE(plan, FSIM_EINVAL, "null plan");
  int rc = validate_param(p);
  if (rc) return rc;
  FSIM_REQUIRE(p->w == plan->prm.w && p->nr_dirs == plan->prm.nr_dirs && p->nr_bands == plan->prm.nr_bands &&
                   p->nr_phases == plan->prm.nr_phases,
               FSIM_EINVAL, "plan_update: geometry (size, dirs, bands, phases) must not change");
  // callers may have work in flight that reads the old tables
  FSIM_CUDA(cudaDeviceSynchronize());
  plan->prm = *p;
  return plan->path == FSIM_PATH_LIVE ? plan->build_live(ctx().stream) : plan->build(ctx().stream);
}

int fsim_plan_destroy(fsim_plan* plan) {
  if (!plan) return FSIM_OK;
  cudaDeviceSynchronize();
  if (plan->dev) cudaFree(plan->dev);
  if (plan->h_ws) cudaFree(plan->h_ws);
  if (plan->h_io) cudaFree(plan->h_io);
  if (plan->h_job) cudaFreeHost(plan->h_job);
  delete plan;
  return FSIM_OK;
}

size_t fsim_plan_workspace_bytes(const fsim_plan* plan) { return plan ? align256(plan_ws(plan)) : 0; }

size_t fsim_plan_filter_bytes(const fsim_plan* plan) { return plan ? plan->filter_bytes : 0; }

int fsim_plan_info(const fsim_plan* plan, int* w, int* path, int* input_type) {
  FSIM_REQUIRE(plan, FSIM_EINVAL, "null plan");
  if (w) *w = plan->prm.w;
  if (path) *path = plan->path;
  if (input_type) *input_type = plan->input_type;
  return FSIM_OK;
}

int fsim_recon_batch(const fsim_job* jobs, int n_jobs, void* workspace, size_t workspace_bytes, void* stream) {
  NEED_INIT();
  cudaStream_t st = stream ? (cudaStream_t)stream : ctx().stream;
  Staging* s = nullptr;
  int rc = get_staging(sizeof(JobDesc) * std::max(1, n_jobs), &s);
  if (rc) return rc;
  rc = recon_batch(jobs, n_jobs, workspace, workspace_bytes, st, (JobDesc*)s->ptr, true);
  if (rc) return rc;
  FSIM_CUDA(cudaEventRecord(s->done, st));
  return FSIM_OK;
}

int fsim_tune_set(int n, int path, int pass, int variant) {
  FSIM_REQUIRE(path == FSIM_PATH_OFFLINE, FSIM_EINVAL, "tune: only the offline passes have variants");
  return offline_tune_set(n, pass, variant);
}

int fsim_tune_get(int n, int path, int pass, int* variant, int* n_variants) {
  FSIM_REQUIRE(variant && n_variants, FSIM_EINVAL, "tune_get: bad arguments");
  FSIM_REQUIRE(path == FSIM_PATH_OFFLINE && pass >= 0 && pass <= 1, FSIM_EINVAL, "tune_get: bad path/pass");
  *variant = offline_tune_get(n, pass);
  *n_variants = offline_variants(pass);
  FSIM_REQUIRE(*variant >= 0, FSIM_EINVAL, "tune_get: unsupported size %d", n);
  return FSIM_OK;
}

int fsim_profile_enable(int on) {
  NEED_INIT();
  if (on && !g_prof_ev[0])
    for (int i = 0; i < 8; i++) FSIM_CUDA(cudaEventCreate(&g_prof_ev[i]));
  g_prof_on = on != 0;
  g_prof_n = 0;
  return FSIM_OK;
}

int fsim_profile_read(float* ms, int max_passes, int* n_passes) {
  FSIM_REQUIRE(ms && n_passes, FSIM_EINVAL, "profile_read: bad arguments");
  *n_passes = 0;
  if (!g_prof_on || g_prof_n == 0) return FSIM_OK;
  FSIM_CUDA(cudaEventSynchronize(g_prof_ev[g_prof_n]));
  int n = std::min(g_prof_n, max_passes);
  for (int i = 0; i < n; i++) FSIM_CUDA(cudaEventElapsedTime(&ms[i], g_prof_ev[i], g_prof_ev[i + 1]));
  *n_passes = n;
  return FSIM_OK;
}

int fsim_recon_host(fsim_plan* plan, const void* raw_host, float* out_host) {
  NEED_INIT();
  FSIM_REQUIRE(plan && raw_host && out_host, FSIM_EINVAL, "recon_host: null argument");
  cudaStream_t st = ctx().stream;
  const int N = plan->prm.w, W = 2 * N;
  const size_t raw_bytes = (size_t)N * N * plan->prm.nr_dirs * plan->prm.nr_phases *
                           (plan->input_type == FSIM_INPUT_U16 ? 2 : 4);
  const size_t out_bytes = (size_t)W * W * sizeof(float);
  const size_t ws = align256(sizeof(JobDesc)) + align256(plan_ws(plan));
  if (plan->h_ws_bytes < ws) {
    if (plan->h_ws) cudaFree(plan->h_ws);
    FSIM_CUDA(cudaMalloc(&plan->h_ws, ws));
    plan->h_ws_bytes = ws;
  }
  if (plan->h_io_bytes < align256(raw_bytes) + out_bytes) {
    if (plan->h_io) cudaFree(plan->h_io);
    FSIM_CUDA(cudaMalloc(&plan->h_io, align256(raw_bytes) + out_bytes));
    plan->h_io_bytes = align256(raw_bytes) + out_bytes;
  }
  if (!plan->h_job) FSIM_CUDA(cudaMallocHost(&plan->h_job, sizeof(JobDesc)));
  char* io = (char*)plan->h_io;
  float* d_out = (float*)(io + align256(raw_bytes));
  FSIM_CUDA(cudaMemcpyAsync(io, raw_host, raw_bytes, cudaMemcpyHostToDevice, st));
  fsim_job j{plan, io, d_out, nullptr};
  int rc = recon_batch(&j, 1, plan->h_ws, plan->h_ws_bytes, st, plan->h_job, true);
  if (rc) return rc;
  FSIM_CUDA(cudaMemcpyAsync(out_host, d_out, out_bytes, cudaMemcpyDeviceToHost, st));
  FSIM_CUDA(cudaStreamSynchronize(st));
  return FSIM_OK;
}

}  // extern "C"
