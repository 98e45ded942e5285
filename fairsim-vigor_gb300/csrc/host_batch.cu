// fsim_recon_batch_host: batched reconstruction from host buffers with the copies overlapped.
//
// The reference hands every stack over from Java arrays (AccelVectorReal.setFrom*,
// org/fairsim/accel/AccelVectorReal.java:218-247, then one JNI op per step). Here a whole
// batch of host stacks is reconstructed in chunks that flow through three library-owned
// streams: the upload of chunk i+1, the passes of chunk i and the download of chunk i-1 run
// at the same time. A ring of FSIM_HOST_SLOTS slots of device buffers (raw frames, outputs,
// workspace) serves the chunks in turn; events order each slot's reuse (K = slots):
//   upload(i)   waits for passes(i-K)    (raw slot free)
//   passes(i)   waits for upload(i), download(i-K) (out slot free)
//   download(i) waits for passes(i)
// The host carves chunk i's slot only after passes(i-K) finished with it, so the host runs
// at most K chunks ahead. The job tables travel as kernel parameters: a table upload on the
// compute stream would queue behind the raw-frame uploads on the one host-to-device copy
// engine and serialize the passes with them. The call returns when every output is in host
// memory.
// Host buffers that are page-locked (cudaHostAlloc / cudaHostRegister) are copied by DMA
// directly; pageable ones make each copy synchronous on the host.
#include <algorithm>
#include <mutex>
#include <vector>

#include "common.cuh"
#include "recon.cuh"
#include "runtime.cuh"

// three slots: 17.1k against 16.7k reconstructions/s with two (512^2 3x3, chunks of 4, GB300)
#ifndef FSIM_HOST_SLOTS
#define FSIM_HOST_SLOTS 3
#endif
static_assert(FSIM_HOST_SLOTS >= 2 && FSIM_HOST_SLOTS <= 8, "host pipeline: 2..8 slots");

namespace fsim {
namespace {

struct Slot {
  char* dev = nullptr;  // raw | out | widefields | workspace
  size_t bytes = 0;
  cudaEvent_t up = nullptr, done = nullptr, down = nullptr;
  bool used = false;
};

struct HostPipe {
  std::mutex mu;
  bool ready = false;
  cudaStream_t s_up = nullptr, s_comp = nullptr, s_down = nullptr;
  Slot slot[FSIM_HOST_SLOTS];
};
HostPipe g_pipe;

size_t a256(size_t b) { return (b + 255) & ~(size_t)255; }

// Copies of one direction, queued so that a copy which continues the previous one on both
// sides (the next job's host buffer right after this one's, and its device buffer too)
// extends it: a chunk of jobs whose host buffers are one array moves as one copy per
// direction and kind of buffer (measured on GB300: 206 GB/s host to device in 32 MB copies
// against 198 in 8 MB ones, 320 against 284 GB/s with both directions at once). Host buffers
// that are adjacent but belong to different page-locked allocations cannot be one copy (the
// runtime refuses it with cudaErrorInvalidValue before queueing anything): such a run is
// copied piece by piece.
struct CopyRun {
  struct Piece {
    char* dst;
    const char* src;
    size_t n;
  };
  cudaMemcpyKind kind;
  cudaStream_t st;
  std::vector<Piece> pieces;
  size_t n = 0;  // bytes of the run
  CopyRun(cudaMemcpyKind k, cudaStream_t s) : kind(k), st(s) {}
  int flush() {
    if (pieces.empty()) return FSIM_OK;
    cudaError_t e = cudaMemcpyAsync(pieces[0].dst, pieces[0].src, n, kind, st);
    if (e == cudaErrorInvalidValue && pieces.size() > 1) {
      (void)cudaGetLastError();  // nothing was queued: copy the pieces one by one
      for (const Piece& q : pieces) FSIM_CUDA(cudaMemcpyAsync(q.dst, q.src, q.n, kind, st));
    } else {
      FSIM_CUDA(e);
    }
    pieces.clear();
    n = 0;
    return FSIM_OK;
  }
  int add(void* d, const void* s, size_t bytes) {
    if (!pieces.empty() && (char*)d == pieces[0].dst + n && (const char*)s == pieces[0].src + n) {
      pieces.push_back({(char*)d, (const char*)s, bytes});
      n += bytes;
      return FSIM_OK;
    }
    int rc = flush();
    pieces.push_back({(char*)d, (const char*)s, bytes});
    n = bytes;
    return rc;
  }
};

size_t raw_bytes(const Plan* p) {
  return (size_t)p->prm.w * p->prm.w * p->prm.nr_dirs * p->prm.nr_phases * (p->input_type == FSIM_INPUT_U16 ? 2 : 4);
}
size_t out_bytes(const Plan* p) { return (size_t)4 * p->prm.w * p->prm.w * sizeof(float); }
// widefield: w x w on the live path, 2w x 2w (as the output) on the offline path
size_t wf_bytes(const Plan* p) {
  return p->path == FSIM_PATH_LIVE ? (size_t)p->prm.w * p->prm.w * sizeof(float) : out_bytes(p);
}

// device bytes of one chunk: per job raw + out (+ widefields) + workspace, plus the table
size_t chunk_bytes(const fsim_host_job* jobs, int k0, int k1) {
  size_t b = a256(sizeof(JobDesc) * (k1 - k0));
  for (int k = k0; k < k1; k++) {
    const Plan* p = reinterpret_cast<const Plan*>(jobs[k].plan);
    b += a256(raw_bytes(p)) + a256(out_bytes(p)) + (jobs[k].widefield_host ? a256(wf_bytes(p)) : 0) +
         (jobs[k].filtered_widefield_host ? a256(out_bytes(p)) : 0) + a256(plan_ws(p));
  }
  return b;
}

int init_pipe(HostPipe& P) {
  if (P.ready) return FSIM_OK;
  FSIM_CUDA(cudaStreamCreateWithFlags(&P.s_up, cudaStreamNonBlocking));
  FSIM_CUDA(cudaStreamCreateWithFlags(&P.s_comp, cudaStreamNonBlocking));
  FSIM_CUDA(cudaStreamCreateWithFlags(&P.s_down, cudaStreamNonBlocking));
  for (auto& s : P.slot) {
    FSIM_CUDA(cudaEventCreateWithFlags(&s.up, cudaEventDisableTiming));
    FSIM_CUDA(cudaEventCreateWithFlags(&s.done, cudaEventDisableTiming));
    FSIM_CUDA(cudaEventCreateWithFlags(&s.down, cudaEventDisableTiming));
  }
  P.ready = true;
  return FSIM_OK;
}

}  // namespace
}  // namespace fsim

using namespace fsim;

extern "C" int fsim_recon_batch_host(const fsim_host_job* jobs, int n_jobs, int chunk) {
  FSIM_REQUIRE(jobs && n_jobs > 0, FSIM_EINVAL, "recon_batch_host: no jobs");
  for (int k = 0; k < n_jobs; k++) {
    const Plan* p = reinterpret_cast<const Plan*>(jobs[k].plan);
    FSIM_REQUIRE(p && jobs[k].raw_host && jobs[k].out_host, FSIM_EINVAL, "host job %d: null plan/raw/out", k);
    FSIM_REQUIRE(!jobs[k].filtered_widefield_host || p->path == FSIM_PATH_OFFLINE, FSIM_EINVAL,
                 "host job %d: the filtered widefield needs an offline-path plan", k);
  }
  int rc = ensure_init();
  if (rc) return rc;
  if (chunk <= 0) {
    // about 60 MiB of raw frames per chunk (six 512^2 3x3 f32 stacks): the host link, not
    // the passes, bounds a host-buffer batch, and short chunks keep both copy directions
    // busy from the start (measured on GB300, 64 stacks from one array, merged copies:
    // chunks of 3 18.1k/s, 4 18.0k/s, 6 18.3k/s, 8 17.6k/s, 12 17.5k/s, 16 16.4k/s)
    const size_t rb = raw_bytes(reinterpret_cast<const Plan*>(jobs[0].plan));
    chunk = (int)std::max<size_t>(1, ((size_t)60 << 20) / std::max<size_t>(rb, 1));
  }
  chunk = std::min(chunk, n_jobs);
  std::lock_guard<std::mutex> lock(g_pipe.mu);
  HostPipe& P = g_pipe;
  rc = init_pipe(P);
  if (rc) return rc;
  // size every slot for the largest chunk of this batch (the previous call has finished)
  size_t need = 0;
  for (int k0 = 0; k0 < n_jobs; k0 += chunk) need = std::max(need, chunk_bytes(jobs, k0, std::min(n_jobs, k0 + chunk)));
  for (auto& s : P.slot) {
    if (s.bytes < need) {
      if (s.dev) cudaFree(s.dev);
      s.dev = nullptr;
      s.bytes = 0;
      FSIM_CUDA(fsim::dev_alloc(&s.dev, need));
      s.bytes = need;
    }
    s.used = false;
  }
  std::vector<fsim_job> dj(chunk);
  std::vector<JobDesc> table(chunk);  // consumed at launch (kernel parameters)
  int c = 0;
  for (int k0 = 0; k0 < n_jobs; k0 += chunk, c++) {
    const int k1 = std::min(n_jobs, k0 + chunk), m = k1 - k0;
    Slot& S = P.slot[c % FSIM_HOST_SLOTS];
    if (S.used) {
      // the raw buffers of chunk c-K must be consumed, and its outputs downloaded
      FSIM_CUDA(cudaEventSynchronize(S.done));
      FSIM_CUDA(cudaStreamWaitEvent(P.s_up, S.done, 0));
      FSIM_CUDA(cudaStreamWaitEvent(P.s_comp, S.down, 0));
    }
    // carve the slot: the raw buffers of all jobs, then the outputs, then the widefields |
    // job table and workspaces (recon_batch lays out [table | ws_0 | ws_1 ...] from the
    // pointer it is given); buffers of one kind are adjacent, so copies can merge
    char* cur = S.dev;
    CopyRun up(cudaMemcpyHostToDevice, P.s_up);
    for (int i = 0; i < m; i++) {
      const fsim_host_job& h = jobs[k0 + i];
      const Plan* p = reinterpret_cast<const Plan*>(h.plan);
      dj[i].plan = h.plan;
      dj[i].raw = cur;
      if ((rc = up.add(cur, h.raw_host, raw_bytes(p)))) return rc;
      cur += a256(raw_bytes(p));
    }
    if ((rc = up.flush())) return rc;
    for (int i = 0; i < m; i++) {
      dj[i].out = reinterpret_cast<float*>(cur);
      cur += a256(out_bytes(reinterpret_cast<const Plan*>(jobs[k0 + i].plan)));
    }
    for (int i = 0; i < m; i++) {
      const fsim_host_job& h = jobs[k0 + i];
      const Plan* p = reinterpret_cast<const Plan*>(h.plan);
      dj[i].widefield = nullptr;
      if (h.widefield_host) {
        dj[i].widefield = reinterpret_cast<float*>(cur);
        cur += a256(wf_bytes(p));
      }
    }
    for (int i = 0; i < m; i++) {
      const fsim_host_job& h = jobs[k0 + i];
      const Plan* p = reinterpret_cast<const Plan*>(h.plan);
      dj[i].filtered_widefield = nullptr;
      if (h.filtered_widefield_host) {
        dj[i].filtered_widefield = reinterpret_cast<float*>(cur);
        cur += a256(out_bytes(p));
      }
    }
    FSIM_CUDA(cudaEventRecord(S.up, P.s_up));
    FSIM_CUDA(cudaStreamWaitEvent(P.s_comp, S.up, 0));
    rc = recon_batch(dj.data(), m, cur, S.bytes - (size_t)(cur - S.dev), P.s_comp, table.data(), true);
    if (rc) {
      cudaStreamSynchronize(P.s_up);
      cudaStreamSynchronize(P.s_comp);
      cudaStreamSynchronize(P.s_down);
      return rc;
    }
    FSIM_CUDA(cudaEventRecord(S.done, P.s_comp));
    FSIM_CUDA(cudaStreamWaitEvent(P.s_down, S.done, 0));
    CopyRun down(cudaMemcpyDeviceToHost, P.s_down);
    for (int i = 0; i < m; i++) {
      const Plan* p = reinterpret_cast<const Plan*>(jobs[k0 + i].plan);
      if ((rc = down.add(jobs[k0 + i].out_host, dj[i].out, out_bytes(p)))) return rc;
    }
    for (int i = 0; i < m; i++) {
      const fsim_host_job& h = jobs[k0 + i];
      if (h.widefield_host &&
          (rc = down.add(h.widefield_host, dj[i].widefield, wf_bytes(reinterpret_cast<const Plan*>(h.plan)))))
        return rc;
    }
    for (int i = 0; i < m; i++) {
      const fsim_host_job& h = jobs[k0 + i];
      if (h.filtered_widefield_host &&
          (rc = down.add(h.filtered_widefield_host, dj[i].filtered_widefield,
                         out_bytes(reinterpret_cast<const Plan*>(h.plan)))))
        return rc;
    }
    if ((rc = down.flush())) return rc;
    FSIM_CUDA(cudaEventRecord(S.down, P.s_down));
    S.used = true;
  }
  FSIM_CUDA(cudaStreamSynchronize(P.s_down));
  FSIM_CUDA(cudaStreamSynchronize(P.s_comp));
  return FSIM_OK;
}
