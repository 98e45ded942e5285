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

// A fixed batch recorded as a CUDA graph (fsim_batch_graph_*).
struct fsim_batch_graph {
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
  cudaStream_t aux[3] = {};
  int n_jobs = 0;
  int kernels = 0;
};

namespace fsim {

static size_t align256(size_t b) { return (b + 255) & ~(size_t)255; }

size_t plan_ws(const Plan* p) {
  return p->path == FSIM_PATH_LIVE ? p->workspace_bytes_live() : p->workspace_bytes();
}

// Job tables reach the device as kernel parameters, not by a copy-engine upload: an upload
// on the compute stream queues behind the raw-frame uploads that other streams have in
// flight (one engine serves the host-to-device direction), and the passes would wait for
// them (measured on GB300: a 4-stack batch beside a 38 MB upload took 0.37 ms instead of
// 0.20 ms). The parameter block is captured at launch, so a graph replays its own table.
template <int WORDS>
struct TableBlob {
  uint4* dst;
  int words;
  int pad;
  uint4 data[WORDS];
};
constexpr int kBlobSmall = 254, kBlobLarge = 2046;  // 4 080- and 32 752-byte parameter blocks

template <int WORDS>
__global__ void k_put_table(const __grid_constant__ TableBlob<WORDS> b) {
  for (int i = threadIdx.x; i < b.words; i += blockDim.x) b.dst[i] = b.data[i];
}

template <int WORDS>
static int put_table_blob(char* dst, const char* src, size_t bytes, cudaStream_t st) {
  TableBlob<WORDS> b;
  b.dst = reinterpret_cast<uint4*>(dst);
  b.words = (int)((bytes + 15) / 16);
  b.pad = 0;
  b.data[b.words - 1] = make_uint4(0, 0, 0, 0);
  std::memcpy(b.data, src, bytes);
  k_put_table<WORDS><<<1, 256, 0, st>>>(b);
  FSIM_CUDA(cudaGetLastError());
  return FSIM_OK;
}

// bytes of host memory to dst (16-byte aligned, room for bytes rounded up to 16)
static int put_table(void* dst, const void* src, size_t bytes, cudaStream_t st) {
  const char* s = static_cast<const char*>(src);
  char* d = static_cast<char*>(dst);
  if (bytes <= (size_t)16 * kBlobSmall) return put_table_blob<kBlobSmall>(d, s, bytes, st);
  for (size_t off = 0; off < bytes; off += (size_t)16 * kBlobLarge) {
    int rc = put_table_blob<kBlobLarge>(d + off, s + off, std::min(bytes - off, (size_t)16 * kBlobLarge), st);
    if (rc) return rc;
  }
  return FSIM_OK;
}

// Fill job tables and launch: jobs are grouped by (path, size) with one set of passes each.
int recon_batch(const fsim_job* jobs, int n, void* ws, size_t ws_bytes, cudaStream_t st, JobDesc* host_table,
                bool upload_table, const cudaStream_t* aux, int naux) {
  FSIM_REQUIRE(jobs && n > 0, FSIM_EINVAL, "recon_batch: no jobs");
  std::vector<int> order(n);
  for (int i = 0; i < n; i++) {
    FSIM_REQUIRE(jobs[i].plan && jobs[i].raw && jobs[i].out, FSIM_EINVAL, "job %d: null plan/raw/out", i);
    FSIM_REQUIRE(!jobs[i].filtered_widefield || static_cast<const Plan*>(jobs[i].plan)->path == FSIM_PATH_OFFLINE,
                 FSIM_EINVAL, "job %d: the filtered widefield needs an offline-path plan", i);
    FSIM_REQUIRE(((uintptr_t)jobs[i].widefield & 7) == 0 && ((uintptr_t)jobs[i].filtered_widefield & 7) == 0,
                 FSIM_EINVAL, "job %d: widefield outputs must be 8-byte aligned", i);
    FSIM_REQUIRE(((uintptr_t)jobs[i].out & 7) == 0, FSIM_EINVAL, "job %d: the output must be 8-byte aligned", i);
    FSIM_REQUIRE(!jobs[i].filtered_widefield || !otf_measured(&static_cast<const Plan*>(jobs[i].plan)->prm), FSIM_EINVAL,
                 "job %d: the filtered widefield needs an estimated OTF (its filter is real)", i);
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
  FSIM_REQUIRE(((uintptr_t)ws & 255) == 0, FSIM_EINVAL, "recon_batch: workspace must be 256-byte aligned");
  char* base = (char*)ws;
  JobDesc* d_table = (JobDesc*)base;
  char* cur = base + align256(sizeof(JobDesc) * n);
  for (int k = 0; k < n; k++) {
    const fsim_job& jb = jobs[order[k]];
    const Plan* p = static_cast<const Plan*>(jb.plan);
    if (p->path == FSIM_PATH_LIVE)
      p->fill_job_live(host_table[k], jb.raw, jb.out, jb.widefield, cur);
    else
      p->fill_job(host_table[k], jb.raw, jb.out, jb.widefield, jb.filtered_widefield, cur);
    cur += align256(plan_ws(p));
  }
  if (upload_table) {
    int prc = put_table(d_table, host_table, sizeof(JobDesc) * n, st);
    if (prc) return prc;
  }
  // size classes: [start, end) ranges of the sorted table
  std::vector<std::pair<int, int>> groups;
  for (int k = 0; k < n;) {
    int e = k;
    while (e < n && key(order[e]) == key(order[k])) e++;
    groups.emplace_back(k, e);
    k = e;
  }
  // per-pass profiling times one stream's passes: no fork while it is on
  const int nfork = (profile_events() || !aux) ? 0 : std::min<int>(naux, (int)groups.size() - 1);
  cudaEvent_t fork_ev = nullptr, join_ev[8] = {};
  if (nfork > 0) {
    FSIM_REQUIRE(nfork <= 8, FSIM_EINVAL, "recon_batch: at most 8 auxiliary streams");
    FSIM_CUDA(cudaEventCreateWithFlags(&fork_ev, cudaEventDisableTiming));
    FSIM_CUDA(cudaEventRecord(fork_ev, st));
    for (int i = 0; i < nfork; i++) {
      FSIM_CUDA(cudaEventCreateWithFlags(&join_ev[i], cudaEventDisableTiming));
      FSIM_CUDA(cudaStreamWaitEvent(aux[i], fork_ev, 0));
    }
  }
  int rc = FSIM_OK;
  for (size_t g = 0; g < groups.size() && rc == FSIM_OK; g++) {
    const int k = groups[g].first, e = groups[g].second;
    const Plan* p0 = static_cast<const Plan*>(jobs[order[k]].plan);
    int maxA = 0, maxPair = 0, maxWin = 0;
    for (int i = k; i < e; i++) {
      const Plan* pi = static_cast<const Plan*>(jobs[order[i]].plan);
      maxA = std::max(maxA, pi->prm.nr_dirs);
      maxPair = std::max(maxPair, pi->prm.nr_bands - 1);
      maxWin = std::max(maxWin, pi->nwin);
    }
    // largest classes sort last; the first class stays on st, the rest spread over aux
    cudaStream_t s = (nfork > 0 && g > 0) ? aux[(g - 1) % nfork] : st;
    bool scale_clip = false;
    int masks = 0;
    for (int i = k; i < e; i++) {
      const Plan* pi = static_cast<const Plan*>(jobs[order[i]].plan);
      scale_clip = scale_clip || pi->clip_scale == 2;
      masks |= otf_measured(&pi->prm) ? 2 : 1;
    }
    rc = (p0->path == FSIM_PATH_LIVE)
             ? launch_live_size(p0->prm.w, d_table + k, e - k, maxA, s)
             : launch_offline_size(p0->prm.w, d_table + k, e - k, maxA, maxPair, maxWin, scale_clip, masks, s);
    if (rc == FSIM_OK && p0->path == FSIM_PATH_OFFLINE) {
      bool wf = false;
      for (int i = k; i < e; i++) wf = wf || jobs[order[i]].widefield || jobs[order[i]].filtered_widefield;
      if (wf) rc = launch_widefield_size(p0->prm.w, d_table + k, e - k, s);
    }
  }
  if (nfork > 0) {
    // join even after a failed launch, so that a capture in progress can still end
    for (int i = 0; i < nfork; i++) {
      cudaEventRecord(join_ev[i], aux[i]);
      cudaStreamWaitEvent(st, join_ev[i], 0);
      cudaEventDestroy(join_ev[i]);
    }
    cudaEventDestroy(fork_ev);
  }
  return rc;
}

// auxiliary streams of fsim_recon_batch: the size classes of one batch run side by side
constexpr int FSIM_AUX_STREAMS = 3;
static std::mutex g_aux_mu;
static cudaStream_t g_aux[FSIM_AUX_STREAMS] = {};

static int aux_streams(cudaStream_t** out) {
  if (!g_aux[0])
    for (auto& a : g_aux) FSIM_CUDA(cudaStreamCreateWithFlags(&a, cudaStreamNonBlocking));
  *out = g_aux;
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
  FSIM_REQUIRE(out, FSIM_EINVAL, "null output pointer");
  *out = nullptr;
  int rc = validate_param(p);
  if (rc) return rc;
  FSIM_REQUIRE(fade_px >= 0 && 2 * fade_px <= p->w, FSIM_EINVAL, "fade of %d pixels on a %d-pixel image", fade_px,
               p->w);
  FSIM_REQUIRE(path == FSIM_PATH_OFFLINE || path == FSIM_PATH_LIVE, FSIM_EINVAL, "unknown path %d", path);
  FSIM_REQUIRE(input_type == FSIM_INPUT_F32 || input_type == FSIM_INPUT_U16, FSIM_EINVAL, "unknown input type");
  if (path == FSIM_PATH_OFFLINE)
    FSIM_REQUIRE(offline_size_supported(p->w), FSIM_EINVAL, "fused reconstruction: unsupported image size %d", p->w);
  else
    FSIM_REQUIRE(live_size_supported(p->w), FSIM_EINVAL, "live reconstruction: unsupported image size %d", p->w);
  FSIM_REQUIRE(p->nr_phases <= FSIM_MAX_PHASES && 2 * p->nr_bands - 1 <= 7, FSIM_EINVAL, "too many phases/bands");
  FSIM_REQUIRE(p->filter_style == FSIM_FILTER_WIENER, FSIM_EINVAL,
               "fused plans apply the Wiener filter; RL filter styles run through fsim_run_reconstruction");
  FSIM_REQUIRE(path == FSIM_PATH_OFFLINE || !otf_measured(p), FSIM_EINVAL,
               "live plans take estimated OTFs; measured OTFs run through offline plans or fsim_run_reconstruction");
  NEED_INIT();
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
  FSIM_REQUIRE(p->filter_style == FSIM_FILTER_WIENER && (plan->path == FSIM_PATH_OFFLINE || !otf_measured(p)),
               FSIM_EINVAL, "fused plans apply the Wiener filter; live plans take estimated OTFs");
  FSIM_REQUIRE(otf_measured(p) == otf_measured(&plan->prm), FSIM_EINVAL,
               "plan_update: an estimated OTF cannot become a measured one (or back) in place");
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

int fsim_plan_set_clip_scale(fsim_plan* plan, int clip_scale) {
  FSIM_REQUIRE(plan, FSIM_EINVAL, "null plan");
  FSIM_REQUIRE(clip_scale >= 0 && clip_scale <= 2, FSIM_EINVAL, "clip_scale %d: 0 (NONE), 1 (CLIP) or 2 (BOTH)",
               clip_scale);
  FSIM_REQUIRE(plan->path == FSIM_PATH_OFFLINE || clip_scale == 0, FSIM_EINVAL,
               "clip_scale: live plans return the reference's unclipped live image");
  plan->clip_scale = clip_scale;
  return FSIM_OK;
}

int fsim_plan_filter_table(const fsim_plan* plan, float* host_out, size_t n_floats, int* ncols) {
  FSIM_REQUIRE(plan && host_out, FSIM_EINVAL, "filter_table: null plan or output");
  const int N = plan->prm.w, W = 2 * N, nc = plan->path == FSIM_PATH_LIVE ? W : N + 1;
  FSIM_REQUIRE(n_floats >= (size_t)W * nc, FSIM_EINVAL, "filter_table: %zu floats given, %zu needed", n_floats,
               (size_t)W * nc);
  NEED_INIT();
  FSIM_CUDA(cudaDeviceSynchronize());
  if (plan->path == FSIM_PATH_LIVE) {
    FSIM_CUDA(cudaMemcpy(host_out, plan->d_wa, (size_t)W * W * sizeof(float), cudaMemcpyDeviceToHost));
  } else {
    // quad layout [X/4][Y][X%4] over the columns X < N + 4
    std::vector<float> q((size_t)(N + 4) * W);
    FSIM_CUDA(cudaMemcpy(q.data(), plan->d_wa, q.size() * sizeof(float), cudaMemcpyDeviceToHost));
    for (int Y = 0; Y < W; Y++)
      for (int X = 0; X < nc; X++) host_out[(size_t)Y * nc + X] = q[((size_t)(X >> 2) * W + Y) * 4 + (X & 3)];
  }
  if (ncols) *ncols = nc;
  return FSIM_OK;
}

int fsim_plan_info(const fsim_plan* plan, int* w, int* path, int* input_type) {
  FSIM_REQUIRE(plan, FSIM_EINVAL, "null plan");
  if (w) *w = plan->prm.w;
  if (path) *path = plan->path;
  if (input_type) *input_type = plan->input_type;
  return FSIM_OK;
}

int fsim_recon_batch(const fsim_job* jobs, int n_jobs, void* workspace, size_t workspace_bytes, void* stream) {
  FSIM_REQUIRE(jobs && n_jobs > 0, FSIM_EINVAL, "recon_batch: no jobs");
  NEED_INIT();
  cudaStream_t st = stream ? (cudaStream_t)stream : ctx().stream;
  // the table is consumed at launch (kernel parameters): plain host memory, reused per thread
  thread_local std::vector<JobDesc> table;
  table.resize(n_jobs);
  int rc = FSIM_OK;
  {
    // the shared auxiliary streams carry one caller's fork/join at a time
    std::lock_guard<std::mutex> g(g_aux_mu);
    cudaStream_t* aux = nullptr;
    rc = aux_streams(&aux);
    if (rc) return rc;
    rc = recon_batch(jobs, n_jobs, workspace, workspace_bytes, st, table.data(), true, aux, FSIM_AUX_STREAMS);
  }
  return rc;
}

int fsim_batch_graph_create(fsim_batch_graph** out, const fsim_job* jobs, int n_jobs, void* workspace,
                            size_t workspace_bytes, void* stream) {
  FSIM_REQUIRE(out && jobs && n_jobs > 0, FSIM_EINVAL, "batch_graph_create: bad arguments");
  *out = nullptr;
  NEED_INIT();
  cudaStream_t st = stream ? (cudaStream_t)stream : ctx().stream;
  cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
  FSIM_CUDA(cudaStreamIsCapturing(st, &cs));
  FSIM_REQUIRE(cs == cudaStreamCaptureStatusNone, FSIM_EINVAL, "batch_graph_create: stream is already capturing");
  fsim_batch_graph* g = new fsim_batch_graph();
  g->n_jobs = n_jobs;
  auto fail = [&](int rc) {
    for (auto a : g->aux)
      if (a) cudaStreamDestroy(a);
    delete g;
    return rc;
  };
  // the job table is a kernel parameter of the captured put launch: every replay writes it
  // to the workspace head before the passes, so the graph does not depend on what else used
  // the workspace in between
  std::vector<JobDesc> table(n_jobs);
  for (auto& a : g->aux)
    if (cudaStreamCreateWithFlags(&a, cudaStreamNonBlocking) != cudaSuccess) {
      set_error("batch_graph_create: stream creation failed");
      return fail(FSIM_ECUDA);
    }
  const bool prof = g_prof_on;
  g_prof_on = false;  // profiling events are not recorded inside a graph
  cudaError_t e = cudaStreamBeginCapture(st, cudaStreamCaptureModeRelaxed);
  int rc = FSIM_OK;
  if (e != cudaSuccess) {
    set_error("batch_graph_create: begin capture: %s", cudaGetErrorString(e));
    rc = FSIM_ECUDA;
  } else {
    rc = recon_batch(jobs, n_jobs, workspace, workspace_bytes, st, table.data(), true, g->aux,
                     FSIM_AUX_STREAMS);
    cudaGraph_t graph = nullptr;
    e = cudaStreamEndCapture(st, &graph);
    if (rc == FSIM_OK && e != cudaSuccess) {
      set_error("batch_graph_create: end capture: %s", cudaGetErrorString(e));
      rc = FSIM_ECUDA;
    }
    g->graph = graph;
  }
  g_prof_on = prof;
  if (rc == FSIM_OK) {
    e = cudaGraphInstantiate(&g->exec, g->graph, 0);
    if (e != cudaSuccess) {
      set_error("batch_graph_create: instantiate: %s", cudaGetErrorString(e));
      rc = FSIM_ECUDA;
    }
  }
  if (rc == FSIM_OK) {
    size_t nn = 0;
    cudaGraphGetNodes(g->graph, nullptr, &nn);
    std::vector<cudaGraphNode_t> nodes(nn);
    if (nn) cudaGraphGetNodes(g->graph, nodes.data(), &nn);
    for (auto nd : nodes) {
      cudaGraphNodeType t;
      if (cudaGraphNodeGetType(nd, &t) == cudaSuccess && t == cudaGraphNodeTypeKernel) g->kernels++;
    }
  }
  if (rc != FSIM_OK) {
    if (g->exec) cudaGraphExecDestroy(g->exec);
    if (g->graph) cudaGraphDestroy(g->graph);
    cudaGetLastError();
    return fail(rc);
  }
  *out = g;
  return FSIM_OK;
}

int fsim_batch_graph_launch(fsim_batch_graph* g, void* stream) {
  FSIM_REQUIRE(g && g->exec, FSIM_EINVAL, "batch_graph_launch: null graph");
  cudaStream_t st = stream ? (cudaStream_t)stream : ctx().stream;
  FSIM_CUDA(cudaGraphLaunch(g->exec, st));
  return FSIM_OK;
}

int fsim_batch_graph_info(const fsim_batch_graph* g, int* n_jobs, int* n_kernels) {
  FSIM_REQUIRE(g, FSIM_EINVAL, "batch_graph_info: null graph");
  if (n_jobs) *n_jobs = g->n_jobs;
  if (n_kernels) *n_kernels = g->kernels;
  return FSIM_OK;
}

int fsim_batch_graph_destroy(fsim_batch_graph* g) {
  if (!g) return FSIM_OK;
  cudaDeviceSynchronize();
  if (g->exec) cudaGraphExecDestroy(g->exec);
  if (g->graph) cudaGraphDestroy(g->graph);
  for (auto a : g->aux)
    if (a) cudaStreamDestroy(a);
  delete g;
  return FSIM_OK;
}

int fsim_tune_set(int n, int path, int pass, int variant) {
  FSIM_REQUIRE(path == FSIM_PATH_OFFLINE, FSIM_EINVAL, "tune: only the offline passes have variants");
  return offline_tune_set(n, pass, variant);
}

int fsim_tune_get(int n, int path, int pass, int* variant, int* n_variants) {
  FSIM_REQUIRE(variant && n_variants, FSIM_EINVAL, "tune_get: bad arguments");
  FSIM_REQUIRE(path == FSIM_PATH_OFFLINE && pass >= 0 && pass <= 2, FSIM_EINVAL, "tune_get: bad path/pass");
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
    FSIM_CUDA(fsim::dev_alloc(&plan->h_ws, ws));
    plan->h_ws_bytes = ws;
  }
  if (plan->h_io_bytes < align256(raw_bytes) + out_bytes) {
    if (plan->h_io) cudaFree(plan->h_io);
    FSIM_CUDA(fsim::dev_alloc(&plan->h_io, align256(raw_bytes) + out_bytes));
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
