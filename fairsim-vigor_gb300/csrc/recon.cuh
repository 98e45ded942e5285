// Internal interface of the fused reconstruction (recon.cu, live.cu, plan.cu).
#pragma once

#include "common.cuh"
#include "otf.cuh"

namespace fsim {

// One dataset in a batched launch (device-resident table, read by every pass).
struct JobDesc {
  const void* raw;    // nA*nP frames of N*N (f32 or u16)
  float* out;         // W*W reconstruction
  float* widefield;   // N*N (live path), nullable
  int input_u16, nA, nP, nC, nWin;
  int clip;   // offline output: 0 CLIPSCALE.NONE, 1 CLIP, 2 BOTH
  int cmask;  // offline: masks are complex (float2; measured OTFs), else real
  float bgr;
  const float* damp;    // N*N border fade, nullable
  const float2* coef;   // [a][c][p] separation coefficients
  const float2* ramps;  // [a][c] {x ramp[W], y ramp[W]}  (offline) / {x ramp[N], y ramp[N]} (live)
  const int* win;       // [a][c] {Xs, Ys} window origins (offline) / {xInt, yInt} paste offsets (live)
  const float* masks;   // [a][c] OTF masks (offline; float2 when cmask) / N*N conj-OTF vector (live)
  const float* wa;      // Wiener x apodization, quad layout [X/4][Y][X%4]
  const float2* nyq;    // offline: [a][b-1][x, y][N] FFT_N((-1)^n ro_pos[n]) of the pos component's x and y
                        // odd-sample ramps (the Nyquist response, see pass A)
  float2* I;            // workspace: row-transformed windows [band 0, neg of (a, b)][nWin/4][N][4] (offline);
                        // live: [a][c] N*N row transforms
  float2* D;            // workspace: [a][b-1][N] Nyquist term d of every row's neg component (pass A)
  float2* G;            // workspace: [a][b-1][nWin] column transform of D with the pos y shift (pass G)
  float2* Tw;           // workspace: column-transformed windows [band 0, neg of (a, b)][nWin/4][nWin][4] (pass B1)
  float2* Dy;           // workspace: [a][b-1][nWin] Nyquist term d' of every neg window column (pass B1)
  float2* O;            // workspace: offline: W x N, columns 0..N-1 of the Hermitian half after pass B2
                        // (row-major, stride N); live: W*W after the column pass
  float2* On;           // workspace (offline): column N of the Hermitian half, W entries
  float* clip_max;      // workspace (offline): the image maximum for CLIPSCALE.BOTH
  // widefield side outputs of the offline path (widefield.cu), run after the passes above
  float* fwf;              // W*W filtered widefield, nullable (widefield: W*W offline, N*N live)
  const float* wff;        // N*N filter of the filtered widefield (resident, k_build_wff)
  float2* Wf;              // workspace (reused after pass C): N*N band-0 rows, then 2 x [W][N] columns
  int* status;             // the context's device status word (bounded waits that expired)
};

struct Plan {
  fsim_sim_param prm{};
  int path = FSIM_PATH_OFFLINE;
  int input_type = FSIM_INPUT_F32;
  int fade_px = 0;
  double bgr = 0;
  int clip_scale = 0;  // offline output: SimParam.CLIPSCALE ordinal (0 NONE, 1 CLIP, 2 BOTH)
  int nwin = 0;
  void* dev = nullptr;
  size_t dev_bytes = 0;
  size_t filter_bytes = 0;
  float2* d_coef = nullptr;
  float2* d_ramps = nullptr;
  int* d_win = nullptr;
  OtfTable* d_otf = nullptr;
  float* d_damp = nullptr;
  float* d_masks = nullptr;
  float* d_wa = nullptr;
  float2* d_nyq = nullptr;
  float* d_wff = nullptr;  // filtered-widefield filter, N*N
  // host-call convenience buffers (fsim_recon_host)
  void* h_ws = nullptr;
  size_t h_ws_bytes = 0;
  void* h_io = nullptr;
  size_t h_io_bytes = 0;
  JobDesc* h_job = nullptr;
  JobDesc* d_job = nullptr;

  int build(cudaStream_t st);       // offline tables
  int build_live(cudaStream_t st);  // live tables
  size_t workspace_bytes() const;
  size_t workspace_bytes_live() const;
  void fill_job(JobDesc& j, const void* raw, float* out, float* wf, float* fwf, char* ws) const;
  void fill_job_live(JobDesc& j, const void* raw, float* out, float* wf, char* ws) const;
};

// Optional per-pass CUDA-event timing of the next batches (fsim_profile_*): returns the
// event array to record into, or nullptr when profiling is off.
cudaEvent_t* profile_events();
void profile_mark(int n_passes);

bool offline_size_supported(int n);
int offline_variants(int pass);
int offline_tune_set(int n, int pass, int v);
int offline_tune_get(int n, int pass);
bool live_size_supported(int n);
// maxA, maxPair, maxWin: the largest angle count, band-pair count and OTF-support window
// of the batch's datasets of size n (they bound the grids; extra blocks exit at once)
// scale_clip: some job of the class asks for CLIPSCALE.BOTH (one more pass scales its image)
// masks: bit 0 some job of the class has real OTF masks, bit 1 some has complex ones
int launch_offline_size(int n, const JobDesc* d_jobs, int njobs, int maxA, int maxPair, int maxWin, bool scale_clip,
                        int masks, cudaStream_t st);
int launch_live_size(int n, const JobDesc* d_jobs, int njobs, int maxA, cudaStream_t st);
// widefield and filtered widefield of the offline jobs that ask for them (widefield.cu);
// launched after launch_offline_size on the same stream (it reuses the job workspaces)
int launch_widefield_size(int n, const JobDesc* d_jobs, int njobs, cudaStream_t st);
// workspace bytes the widefield kernels need per job of size n
size_t widefield_ws_bytes(int n);
// the plan's filtered-widefield filter (n*n floats), from its device OTF table
int build_widefield_filter(float* d_wff, int n, const OtfTable* d_otf, float wp, cudaStream_t st);

// Fill the job table of a batch (sorted by path and size) into host_table, optionally copy it
// to the head of the workspace, and launch every size class's passes. With aux streams, the
// size classes after the first run on them, forked from and joined back into st by events.
int recon_batch(const fsim_job* jobs, int n, void* ws, size_t ws_bytes, cudaStream_t st, JobDesc* host_table,
                bool upload_table, const cudaStream_t* aux = nullptr, int naux = 0);
size_t plan_ws(const Plan* p);

}  // namespace fsim
