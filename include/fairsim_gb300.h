/*
 * fairsim_gb300.h — C ABI of the GB300-native (sm_103a) fairSIM 2D SIM reconstruction path.
 *
 * This is the drop-in boundary. It replaces, one for one, the JNI natives that the
 * reference's accel backend binds, and it adds the fused entry points the reference
 * lacks. Reference paths are relative to the fairSIM project root.
 *
 *   accel vector natives  org/fairsim/accel/AccelVectorReal.java:218-247,330-333
 *                         org/fairsim/accel/AccelVectorCplx.java:296-331,483-492
 *   FFT plan native       org/fairsim/accel/FFTProvider.java:105
 *   factory natives       org/fairsim/accel/AccelVectorFactory.java:139-146
 *   SIM algorithm         org/fairsim/sim_algorithm/SimAlgorithm.java:37 (estimateParameters),
 *                         :268 (runReconstruction); WienerFilter.java:115; OtfProvider.java:331-559
 *   live serving loop     org/fairsim/livemode/ReconstructionRunner.java:415-593
 *
 * Conventions: every function returns an int32 status (FSIM_OK == 0, negative on error;
 * fsim_last_error() gives a message for the calling thread). Vectors are row-major
 * (x + w*y); complex vectors are interleaved float32 (re, im), as in
 * org/fairsim/linalg/Vec2d.java:23-24. Frequency coordinates follow
 * org/fairsim/sim_algorithm/OtfProvider.java:345-346 (y flipped).
 * "stream" arguments are cudaStream_t values passed as void* (NULL = the library stream).
 */
#ifndef FAIRSIM_GB300_H
#define FAIRSIM_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes (the JNI shim maps them to the reference's exception types) ---- */
#define FSIM_OK 0
#define FSIM_EINVAL (-1)   /* bad argument: RuntimeException / IndexOutOfBounds in Java */
#define FSIM_EOOM (-2)     /* allocation failed: OutOfMemoryError (AccelVectorCplx.java:51-54) */
#define FSIM_ECUDA (-3)    /* CUDA runtime error: cudaRE's RuntimeException (accel/cuda_common.h:33-63) */
#define FSIM_ETIMEOUT (-4) /* a bounded wait expired */
#define FSIM_EBUSY (-5)    /* admission refused: no slot / HBM budget, retry later */
#define FSIM_ENOTFOUND (-6)
#define FSIM_ENODEV (-7)   /* no CUDA device / library not initialised */

#define FSIM_MAX_DIRS 8
#define FSIM_MAX_BANDS 4
#define FSIM_MAX_PHASES 16

/* ---- library ------------------------------------------------------------------- */
const char* fsim_last_error(void);
int fsim_init(int device);               /* select device, upload FFT twiddle tables */
int fsim_sync(void);                     /* AccelVectorFactory.nativeSync (cudaDeviceSynchronize) */
int fsim_version(void);
int fsim_set_stream(void* stream);       /* stream used by the vector API (NULL = own stream) */

/* AccelVectorFactory.nativeAllocMemory / nativeAllocMemoryHost (AccelVectorFactory.java:140-141):
 * raw device (host == 0) or page-locked host (host != 0) buffers, and their release. */
int fsim_buffer_alloc(size_t bytes, int host, void** out);
int fsim_buffer_free(void* p, int host);
/* AccelVectorFactory.startProfiler / stopProfiler (AccelVectorFactory.java:143-146). */
int fsim_profiler(int start);
/* FFTProvider.nativeCreatePlan2d (FFTProvider.java:105): checks that w x h has line FFTs and
 * returns a handle carrying the shape (no plan object is built; nothing to free). */
int fsim_fft_plan_2d(int w, int h, int64_t* plan);

/* ---- SimParam (+ OtfProvider.fromEstimate) as a flat record ------------------------
 * org/fairsim/sim_algorithm/SimParam.java:31-615, OtfProvider.java:96-127.
 * px/py: Dir.pX/pY (band-1 shift; setPxPy divides the highest-band shift by nBands-1),
 * modulation[d][b]: raw Dir.modul (clamped to [0.3,1.1] where the reference clamps). */
typedef struct fsim_sim_param {
  int32_t w; /* raw image width == height */
  int32_t nr_dirs, nr_bands, nr_phases;
  double microns_per_pixel;
  double na, em_wavelength, otf_a;
  int32_t use_attenuation;
  double att_strength, att_fwhm;
  double wiener, apo_cutoff, apo_bend;
  double px[FSIM_MAX_DIRS], py[FSIM_MAX_DIRS], pha_off[FSIM_MAX_DIRS];
  double modulation[FSIM_MAX_DIRS][FSIM_MAX_BANDS];
  int32_t has_phases;
  double phases[FSIM_MAX_DIRS][FSIM_MAX_PHASES];
  /* SimParam.FilterStyle ordinal (SimParam.java:33-43): FSIM_FILTER_WIENER (the fused plans
   * and the live path), or an RL style (fsim_run_reconstruction); rl_iterations as
   * SimParam.getRLiterations (the reference's default is 5) */
  int32_t filter_style;
  int32_t rl_iterations;
  /* Measured OTF (OtfProvider.loadFromConfig with band data, OtfProvider.java:588-621):
   * otf_bands x otf_samples complex values (re, im) in host memory, otf_cycles cycles/micron
   * per sample; read when the call is made. NULL / 0 samples: OtfProvider.fromEstimate
   * (na, em_wavelength, otf_a). The op-by-op path and the parameter fit take both; the fused
   * plans take estimates only. */
  const float* otf_data;
  int32_t otf_bands, otf_samples; /* otf_samples <= 1024 */
  double otf_cycles;
} fsim_sim_param;
#define FSIM_FILTER_WIENER 0
#define FSIM_FILTER_RL_IN 1
#define FSIM_FILTER_RL_OUT 2
#define FSIM_FILTER_RL_BOTH 3

/* ---- Vector API: device vectors (AccelVectorReal/Cplx[2d]) ---------------------------- */
typedef struct fsim_vec fsim_vec;
/* AccelVector*.alloc / dealloc (AccelVectorCplx.java:305,308; AccelVectorReal.java:226,229) */
int fsim_vec_create(fsim_vec** out, int w, int h, int is_complex);
int fsim_vec_destroy(fsim_vec* v);
int fsim_vec_info(const fsim_vec* v, int* w, int* h, int* is_complex, void** device_ptr);
/* copyBuffer (AccelVectorCplx.java:311): host <-> device, n floats of the vector */
int fsim_vec_upload(fsim_vec* v, const float* host);
int fsim_vec_download(const fsim_vec* v, float* host);
/* The accel vectors are allocated by element count (AccelVectorCplx.java:305) and learn
 * their 2D shape from the call that needs it (FFT plan, nativeFourierShift's N,
 * nativePasteFreq's wo/ho): reshape sets w x h with w*h equal to the element count. */
int fsim_vec_reshape(fsim_vec* v, int w, int h);
/* nativeSet / nativeGet (AccelVectorCplx.java:486-487, AccelVectorReal.java:332-333):
 * element index = x + y*width; im is ignored (set) or not written (get) for real vectors. */
int fsim_vec_set_elem(fsim_vec* v, size_t index, float re, float im);
int fsim_vec_get_elem(const fsim_vec* v, size_t index, float* re, float* im);
/* nativeCOPYSHORT (AccelVectorCplx.java:483, AccelVectorReal.java:330): unsigned 16-bit pixels */
int fsim_vec_upload_u16(fsim_vec* v, const uint16_t* host);
/* elementwise ops (AccelVectorCplx.java:314-331, AccelVectorReal.java:235-247) */
int fsim_vec_zero(fsim_vec* y);
int fsim_vec_add(fsim_vec* y, const fsim_vec* x);
int fsim_vec_addconst(fsim_vec* y, float re, float im);
int fsim_vec_axpy(fsim_vec* y, float re, float im, const fsim_vec* x); /* y += a*x */
int fsim_vec_times(fsim_vec* y, const fsim_vec* x, int conj);         /* y = x .* y (x real or complex) */
int fsim_vec_scal(fsim_vec* y, float re, float im);
int fsim_vec_copy(fsim_vec* y, const fsim_vec* x); /* real->cplx (im 0), cplx->real (real part), same */
int fsim_vec_reciproc(fsim_vec* y);
int fsim_vec_norm2(const fsim_vec* x, double* out);                     /* nativeREDUCE(sqr=true) */
int fsim_vec_sum(const fsim_vec* x, double* re, double* im);            /* sumElements */
int fsim_vec_dot(const fsim_vec* x, const fsim_vec* y, double* re, double* im); /* <conj(x), y> */
/* nativeFFT (AccelVectorCplx.java:489): 2D C2C in place; inverse scaled 1/(w*h) */
int fsim_vec_fft2d(fsim_vec* v, int inverse);
/* The same 2D FFT on `batch` contiguous w x h complex float32 planes in device memory
 * (row-major, interleaved), on `stream`; inverse scaled 1/(w*h). No reference counterpart
 * (the reference transforms one vector per JNI call). */
int fsim_fft2d_batch(void* data, int w, int h, int batch, int inverse, void* stream);
/* nativeFourierShift (AccelVectorCplx.java:490): v *= exp(i 2pi (kx x + ky y)/N), square N */
int fsim_vec_fourier_shift(fsim_vec* v, double kx, double ky);
/* nativePasteFreq (AccelVectorCplx.java:491): zero out, place in's spectrum with offset */
int fsim_vec_paste_freq(fsim_vec* out, const fsim_vec* in, int x_off, int y_off);

/* ---- SIM building blocks on device vectors --------------------------------------- */
/* OtfProvider.otfToVector (OtfProvider.java:331-373): write != 0 writes OTF, else v *= conj(OTF) */
int fsim_otf_to_vector(fsim_vec* v, const fsim_sim_param* p, int band, double kx, double ky,
                       int use_att, int write);
int fsim_apo_vector(fsim_vec* v, const fsim_sim_param* p, double bend, double cutoff);        /* :437-492 */
int fsim_attenuation_vector(fsim_vec* v, const fsim_sim_param* p, double str, double fwhm,
                            double kx, double ky);                                            /* :503-529 */
int fsim_mask_otf(fsim_vec* v, const fsim_sim_param* p, double kx, double ky);                /* :538-559 */
/* WienerFilter.getDenominator (WienerFilter.java:88-122): out is real 2w x 2w */
int fsim_wiener_denominator(fsim_vec* out, const fsim_sim_param* p, double wiener);
/* BandSeparation.createSeparationMatrix (BandSeparation.java:40-114) for the phases of band 1
 * (band b at b times them), fac (bands entries) nullable: the inverse or, with more phases
 * than components, the pseudo-inverse, out = (2*bands-1) x n_phases complex doubles
 * (re, im interleaved, component-major). Host-only: needs no device. */
int fsim_separation_matrix(const double* phases, int n_phases, int bands, const double* fac, double* out);
/* BandSeparation.separateBands (BandSeparation.java:131-165), phases of band 1, fac nullable */
int fsim_separate_bands(fsim_vec* const* in, int n_in, fsim_vec* const* out, int n_out,
                        const double* phases, int bands, const double* fac);
/* Correlation (Correlation.java:43-288) */
int fsim_common_region(fsim_vec* b0, fsim_vec* b1, const fsim_sim_param* p, double kx, double ky,
                       double dist, double weight_limit, int divide);
int fsim_locate_peak(const fsim_vec* v, double k_min, double out4[4]);
int fsim_fit_peak(const fsim_vec* band0, const fsim_vec* band1, const fsim_sim_param* p, double kx,
                  double ky, double weight_limit, double search, double out4[4], double* grid_out);
int fsim_get_peak(const fsim_vec* band0, const fsim_vec* band1, const fsim_sim_param* p, double kx,
                  double ky, double weight_limit, double out2[2]);
/* Correlation.autoCorrelation (Correlation.java:294-325): Wicker's non-iterative phase
 * estimate; band (complex, square) pasted to 2w, one copy shifted by (kx, ky), sum of
 * a*conj(b) in double over norm2(a). */
int fsim_auto_correlation(const fsim_vec* band, double kx, double ky, double* re, double* im);
/* RLDeconvolution.deconvolve (RLDeconvolution.java:45-103): `steps` Richardson-Lucy
 * iterations on img with the complex OTF vector otf (same shape); input_in_freq_space:
 * img holds a spectrum (transformed to real space and back). */
int fsim_rl_deconvolve(fsim_vec* img, const fsim_vec* otf, int steps, int input_in_freq_space);

/* ---- SimAlgorithm-compatible entries (SimAlgorithm.java:37, :268) -------------------
 * in_fft: nr_dirs*nr_phases complex w x w spectra (angle-major). The op-by-op variant
 * chains the vector kernels exactly like the reference's Java on an accel factory
 * (the "plain GPU form"); it runs every filter style (p->filter_style: Wiener, RL on the
 * input, the output, or both, SimAlgorithm.java:318-361,587-641). */
int fsim_run_reconstruction(const fsim_sim_param* p, fsim_vec* const* in_fft, fsim_vec* out_real,
                            int otf_before_shift, int clip_scale);
int fsim_estimate_parameters(fsim_sim_param* p, fsim_vec* const* in_fft, int fit_band,
                             double fit_exclude, double* peaks_out /* nr_dirs*4, nullable */);

/* ---- fused batched reconstruction (new; no reference counterpart) --------------------- */
#define FSIM_PATH_OFFLINE 0 /* runReconstruction: OTF after a 2w-grid shift, apo bend p->apo_bend */
#define FSIM_PATH_LIVE 1    /* ReconstructionThread: damp, OTF before a w-grid fast shift, apo bend 1 */
#define FSIM_INPUT_F32 0
#define FSIM_INPUT_U16 1
typedef struct fsim_plan fsim_plan;
/* Builds the resident per-channel filters (OTF masks, Wiener x apodization, damping,
 * separation coefficients, shift tables) for one parameter set. fade_px: border fade
 * (SimUtils.fadeBorderCos) applied to raw frames, 0 = off; bgr: background subtracted and
 * clipped at 0 (SimUtils.subtractBackground) when != 0 (offline path). */
int fsim_plan_create(fsim_plan** out, const fsim_sim_param* p, int path, int input_type, int fade_px,
                     double bgr);
int fsim_plan_update(fsim_plan* plan, const fsim_sim_param* p); /* new shifts/phases/modulation */
int fsim_plan_destroy(fsim_plan* plan);
size_t fsim_plan_workspace_bytes(const fsim_plan* plan);      /* per dataset */
size_t fsim_plan_filter_bytes(const fsim_plan* plan);         /* resident filters */
int fsim_plan_info(const fsim_plan* plan, int* w, int* path, int* input_type);
/* The plan's resident Wiener x apodization table, 1/(sum |OTF|^2 + wiener^2) * apo
 * (WienerFilter.getDenominator times OtfProvider.writeApoVector, S/SimAlgorithm.java:506-518;
 * the live path's setupFilters, LM/ReconstructionRunner.java:773-828), copied to host memory
 * as rows Y = 0..2w-1 of columns X = 0..ncols-1 in the reference's vector layout:
 * ncols = w + 1 for offline plans (the Hermitian half their column pass reads), 2w for live
 * plans. n_floats must hold 2w * ncols values; *ncols receives ncols. Synchronises the device. */
/* Bits set on the device since the last clear by kernels that detected a failure instead of
 * hanging or faulting (FSIM_STATUS_*; 0 when none): read after the work has finished.
 * detail (nullable, 3 ints) receives a description of the first event (kernel-specific:
 * pass B2 records (block x) | (stage << 12) | (stages << 18) | (depth << 24), then the two
 * 32-bit halves of the barrier word it waited on). Synchronises the device; clear != 0
 * resets the words. */
#define FSIM_STATUS_BULK_WAIT 1    /* pass B2: a staged bulk copy was not seen complete in time */
#define FSIM_STATUS_STAGE_LAYOUT 2 /* pass B2: a stage would span more than two column quads */
int fsim_device_status(int* bits, int* detail, int clear);
int fsim_plan_filter_table(const fsim_plan* plan, float* host_out, size_t n_floats, int* ncols);
/* Output scaling of an offline plan's reconstruction, SimParam.CLIPSCALE
 * (SimParam.java:61-62, applied by SimUtils.spatial / clipAndScale, SimUtils.java:146-153,
 * 244-264): 0 NONE (the default here), 1 CLIP (negative values set to 0), 2 BOTH (scaled to
 * 255 at the image maximum, then clipped; the reference's default). Live plans: NONE only. */
int fsim_plan_set_clip_scale(fsim_plan* plan, int clip_scale);

typedef struct fsim_job {
  const fsim_plan* plan;
  const void* raw;  /* device: nr_dirs*nr_phases frames, w*w each, f32 or u16 (plan input type) */
  float* out;       /* device, 8-byte aligned: 2w x 2w float32 reconstruction (real part, scaled
                       as fsim_plan_set_clip_scale chose; CLIPSCALE.NONE by default) */
  float* widefield; /* device, nullable. Live plans: w x w mean of the damped raw frames
                       (ReconstructionRunner.java:449-496). Offline plans: the 2w x 2w
                       "Widefield" image of runReconstruction (SimAlgorithm.java:533-560) */
  float* filtered_widefield; /* device, nullable; offline plans only: the 2w x 2w "filtered
                                Widefield" (OTF band 0, widefield Wiener denominator and OTF
                                support mask, SimAlgorithm.java:562-576). Both widefield
                                outputs must be 8-byte aligned. */
} fsim_job;
/* Reconstruct n_jobs datasets (mixed sizes and plans allowed) with one set of launches per
 * size class; the size classes run side by side on library-owned streams forked from and
 * joined back into `stream`. workspace: 256-byte aligned device memory of at least the sum
 * of fsim_plan_workspace_bytes plus 256 bytes per job. The job table travels as a kernel
 * parameter (no copy engine: the passes never wait behind other streams' uploads). Not for
 * use inside a caller's stream capture (the fork onto library streams is not capturable
 * there): record a batch with fsim_batch_graph_create instead. */
int fsim_recon_batch(const fsim_job* jobs, int n_jobs, void* workspace, size_t workspace_bytes,
                     void* stream);
/* Host-buffer batch (replaces the per-op Java-array copies of the accel vectors,
 * AccelVectorReal.java:218-247 / AccelVectorCplx.java:296-331, for whole stacks): uploads,
 * passes and downloads of successive chunks of `chunk` jobs
 * overlap on three library-owned streams (chunk 0 = about 60 MiB of raw frames); returns
 * when every output is in host memory.
 * Page-locked host buffers are copied by DMA; pageable ones copy synchronously. Jobs whose
 * host buffers follow one another in one allocation (one array of stacks, one of images)
 * move as one copy per chunk and direction. One call runs at a time per process (others
 * wait). */
typedef struct fsim_host_job {
  const fsim_plan* plan;
  const void* raw_host;  /* nr_dirs*nr_phases frames, w*w each, f32 or u16 */
  float* out_host;       /* 2w x 2w float32 */
  float* widefield_host; /* nullable; w x w (live plans) or 2w x 2w (offline plans), as fsim_job */
  float* filtered_widefield_host; /* nullable; offline plans only: 2w x 2w */
} fsim_host_job;
int fsim_recon_batch_host(const fsim_host_job* jobs, int n_jobs, int chunk);
/* A fixed batch recorded once as a CUDA graph (no reference counterpart): the job-table
 * write (the table is a parameter of the recorded launch) and every size class's passes,
 * with the classes on parallel branches. Replays
 * (fsim_batch_graph_launch) reconstruct the same jobs' current raw buffers into the same
 * outputs. Plans, raw/out buffers and the workspace must stay allocated while the graph
 * exists; fsim_plan_update keeps a plan's table addresses, so replays pick up new
 * parameters. n_kernels: kernel launches per replay. */
typedef struct fsim_batch_graph fsim_batch_graph;
int fsim_batch_graph_create(fsim_batch_graph** out, const fsim_job* jobs, int n_jobs, void* workspace,
                            size_t workspace_bytes, void* stream);
int fsim_batch_graph_launch(fsim_batch_graph* g, void* stream);
int fsim_batch_graph_info(const fsim_batch_graph* g, int* n_jobs, int* n_kernels);
int fsim_batch_graph_destroy(fsim_batch_graph* g);
/* Kernel variant per image size (no reference counterpart), chosen by the project's
 * autotuner (fairsim-vigor_gb300/autotune.py, results in tuning.json): pass 0 = row pass
 * (elements per thread), pass 1 = column transforms, pass 2 = masked column sum and inverse
 * (elements per thread x interleaved columns).
 * Variants only change launch shapes; results are identical to float rounding. */
int fsim_tune_set(int n, int path, int pass, int variant);
int fsim_tune_get(int n, int path, int pass, int* variant, int* n_variants);
/* Per-pass CUDA-event timing of fused batches (no reference counterpart): while enabled,
 * every batch records events between its passes on its stream; fsim_profile_read waits
 * for the last batch and returns the duration of each pass of its last size class
 * (offline: A, G+B1, B2, C; live: LA, LB, LC, LD). */
int fsim_profile_enable(int on);
int fsim_profile_read(float* ms, int max_passes, int* n_passes);
/* Host-buffer convenience: H2D copy of raw, reconstruction, D2H copy of out. */
int fsim_recon_host(fsim_plan* plan, const void* raw_host, float* out_host);
/* Parameter fit on device raw frames (fade + FFT + SimAlgorithm.estimateParameters). */
int fsim_estimate_raw(fsim_sim_param* p, const void* raw_device, int input_type, int fade_px,
                      int fit_band, double fit_exclude, double* peaks_out);
/* ParameterRefitThread.doRefit (ReconstructionRunner.java:642-746) on u16 device frames. */
int fsim_live_refit(fsim_sim_param* p, const uint16_t* raw_device, double* peaks_out);

/* ---- allocation-free correlation sweep (no counterpart in the reference) ---------------
 * For callers that cannot allocate device memory at this point: a real-time acquisition
 * thread (no room in its latency budget for the allocator) or a process whose device
 * memory was partitioned up front (an allocation mid-run could fail or take memory another
 * component counts on). The fit's 10 x 10 correlation grid of Correlation.fitPeak's inner
 * loop, evaluated on caller-provided real-space bands b0, b1 (n x n complex float, device)
 * for shifts kx[nx], ky[ny] (host arrays), scaled by scal; out (host, nx*ny*2 doubles,
 * [yi][xi] re/im), equal bit for bit to the allocating fit's grid. Scratch is one static
 * device array per GPU (n <= 2048, nx, ny <= 10; ~0.66 MB kept until exit); the call
 * allocates nothing and returns once out is written. Overlapping calls race on that
 * scratch. The first call on a device resolves the array's address; make it before any
 * stream capture. stream: cudaStream_t (NULL = legacy default stream). */
int fsim_corr_grid_noalloc(const void* b0, const void* b1, int n, const double* kx, int nx, const double* ky,
                           int ny, double scal, double* out, void* stream);

/* ---- test hook (no reference counterpart) ------------------------------------------------
 * The nth next device allocation made by the library (nth >= 1) fails as out of memory;
 * 0 disarms. Lets tests drive every FSIM_EOOM path without exhausting a shared GPU. */
int fsim_debug_fail_alloc(int nth);
/* Pass B2 of the fused offline path stages its inputs into shared memory with bulk copies
 * where they fit (on = 1, the default) or reads them with plain loads (on = 0); both give the
 * same bits. *prev (nullable) receives the previous setting. Lets tests and benchmarks compare
 * the two. */
int fsim_debug_b2_staging(int on, int* prev);

/* ---- served form: continuous batching over channels (replaces ReconstructionRunner) --- */
typedef struct fsim_server fsim_server;
typedef struct fsim_serve_config {
  int32_t max_batch;        /* stacks per launch */
  int32_t max_inflight;     /* admitted stacks not yet returned, per size class (slots) */
  int32_t streams;          /* concurrent batch streams */
  int32_t refit_every;      /* re-fit a channel's parameters every N stacks (0 = never) */
  int32_t input_type;       /* FSIM_INPUT_U16 or FSIM_INPUT_F32 */
  int32_t fade_px;
  size_t hbm_budget_bytes;  /* 0, or a bound on the device memory of the batch workspaces and
                               the slots together */
} fsim_serve_config;
typedef struct fsim_serve_stats {
  uint64_t submitted, completed, rejected, refits;
  double p50_ms, p99_ms, mean_ms, max_ms;
  double recon_per_s;
  double wall_s;
  uint64_t cancelled;
} fsim_serve_stats;
/* Admission by free HBM: channels of one stack and image size share a class of slots
 * (pinned staging + device buffers of that size). At open, slots are allocated, one at a
 * time to the class with the fewest bytes of slots, up to max_inflight per class, while the
 * free device memory (cudaMemGetInfo, less a headroom of max(1/16 of the device, 1 GiB) for
 * other users) and hbm_budget_bytes allow; after every refit the free memory is read again
 * and classes below max_inflight grow. FSIM_EOOM when some class gets no slot at all. */
int fsim_serve_open(fsim_server** out, const fsim_serve_config* cfg, const fsim_sim_param* channels,
                    int n_channels);
/* Copies the raw stack (host, raw_bytes long) into a staging slot of the channel's class.
 * FSIM_EBUSY when that class has no free slot (the reference's live queue drops and counts
 * the frame instead, ReconstructionRunner.java:140-150); other classes keep admitting.
 * FSIM_EINVAL when raw_bytes is not the channel's nr_dirs*nr_phases*w*w*sample size (the
 * reference throws from Vec.failSize). */
int fsim_serve_submit(fsim_server* s, int channel, const void* raw_host, size_t raw_bytes, uint64_t* ticket);
/* Gives a ticket up: a queued stack is dropped, a finished one released, and one on the GPU
 * releases its slot when its batch completes. Waiting on it afterwards gives
 * FSIM_ENOTFOUND. */
int fsim_serve_cancel(fsim_server* s, uint64_t ticket);
/* Waits up to timeout_ms for the ticket; copies the 2w x 2w result to out_host. */
int fsim_serve_wait(fsim_server* s, uint64_t ticket, float* out_host, int timeout_ms, double* latency_ms);
int fsim_serve_stats_get(fsim_server* s, fsim_serve_stats* out);
int fsim_serve_params(fsim_server* s, int channel, fsim_sim_param* out);
/* Slots of the channel's size class: allocated so far, and free now (no reference
 * counterpart). */
int fsim_serve_capacity(fsim_server* s, int channel, int* slots, int* free_slots);
int fsim_serve_close(fsim_server* s);

/* ---- live stream ingest (host only, no device work) -------------------------------------
 * The camera-stream side of the live path: the 128-byte LIVESIM frame header
 * (transport/header-definition.md, as transport/ImageWrapper.java:418-478 writes and
 * checks it), the TCP byte stream split into frames (transport/ImageReceiver.java:122-164)
 * and the per-channel SIM sequence detection (livemode/SimSequenceExtractor.java:152-518)
 * that hands complete stacks to the reconstruction. */
#define FSIM_LIVESIM_HEADER_BYTES 128
typedef struct fsim_livesim_header {
  int64_t seq_nr;          /* byte 0 */
  int32_t payload_offset;  /* byte 8 (0) */
  int32_t payload_len;     /* byte 12: width*height (pixels, as ImageWrapper writes it) */
  int32_t version;         /* byte 16 (1) */
  int32_t bytes_per_pixel; /* byte 17: 1 or 2 */
  int32_t width, height;   /* bytes 32, 34 */
  int32_t pos_a, pos_b;    /* bytes 36, 38: angle, phase */
  int32_t pos0, pos1;      /* bytes 40, 42: z plane, channel (excitation wavelength) */
  int32_t pos2;            /* byte 44: time point */
  int64_t time_camera, time_capture, time_record; /* bytes 48, 56, 64: microseconds */
} fsim_livesim_header;
/* ImageWrapper.parseHeader: FSIM_EINVAL for a frame larger than max_width x max_height,
 * payload_len != width*height, bytes per pixel not 1 or 2, or version != 1. */
int fsim_livesim_parse(const void* header_bytes, int max_width, int max_height, fsim_livesim_header* out);
/* ImageWrapper.writeHeader: zero-filled 128 bytes, version 1, payload_len = width*height. */
int fsim_livesim_write(const fsim_livesim_header* h, void* header_bytes);

#define FSIM_MAX_CHANNELS 8
typedef struct fsim_seqx fsim_seqx;
typedef struct fsim_seqx_config {
  int32_t n_channels;
  int32_t channel_numbers[FSIM_MAX_CHANNELS]; /* header pos1 of each channel ("ChannelNumber") */
  int32_t raws_per_recon;   /* nr_dirs * nr_phases (at most 20, the sort buffer's size) */
  int32_t width, height;    /* frame size (larger frames are broken headers) */
  int32_t sync_mode;        /* "SyncMode" 0: time gap > delay; 1: gap = delay +- 50 or bright frame */
  int32_t sync_frame_freq;  /* "SyncFrameFreq": SIM sequences per sync frame */
  int32_t sync_frame_avr;   /* "SyncFrameAvr": mean pixel value of a bright sync frame */
  int64_t sync_frame_delay; /* "SyncFrameDelay": microseconds */
  int32_t raw_queue;        /* raw frames buffered per channel (0: raws_per_recon^2 * 10) */
  int32_t sim_queue;        /* finished sequences buffered per channel (0: the same) */
} fsim_seqx_config;
typedef struct fsim_seqx_stats {
  uint64_t frames, bytes;          /* accepted frames and stream bytes */
  uint64_t unknown_channel;        /* frames whose pos1 is no configured channel (dropped) */
  uint64_t missed_raw[FSIM_MAX_CHANNELS];  /* raw queue full (PerChannelBuffer.pushImg) */
  uint64_t missed_sim[FSIM_MAX_CHANNELS];  /* sequence queue full */
  uint64_t sync_frames[FSIM_MAX_CHANNELS];
  uint64_t resyncs[FSIM_MAX_CHANNELS];     /* sort-buffer overflows (a frame lost, re-sorted) */
  uint64_t duplicates[FSIM_MAX_CHANNELS];  /* frames with a sequence number already buffered */
  uint64_t sequences;              /* joined multi-channel stacks handed out */
} fsim_seqx_stats;
int fsim_seqx_create(fsim_seqx** out, const fsim_seqx_config* cfg);
/* One frame: 128-byte header followed by its payload (u8 or u16 little endian). Pixels of
 * 8-bit frames are widened as the reference's getPixels does (Java's signed byte, so values
 * >= 128 become 0xFF80..0xFFFF). FSIM_EINVAL for a broken header or a short frame,
 * FSIM_ENOTFOUND for an unknown channel (counted, dropped). */
int fsim_seqx_push(fsim_seqx* s, const void* frame, size_t bytes);
/* Raw TCP bytes in arbitrary pieces: split into frames and pushed. A broken header closes
 * the stream (FSIM_EINVAL now and for every later call until fsim_seqx_reset), as the
 * reference's receiving thread ends on one. */
int fsim_seqx_feed(fsim_seqx* s, const void* bytes, size_t n);
/* The next stack with one SIM sequence of every channel (JoinedChannelBuffer): out is
 * n_channels x raws_per_recon x height x width u16; first_seq (nullable, n_channels) gets
 * the sequence number of each channel's first frame. FSIM_ENOTFOUND when none is ready. */
int fsim_seqx_pop(fsim_seqx* s, uint16_t* out, int64_t* first_seq);
int fsim_seqx_stats_get(const fsim_seqx* s, fsim_seqx_stats* out);
/* Clears every buffer and restarts the sequence search (resetChannelBufferThreads and
 * clearBuffers); reopens a stream closed by a broken header. */
int fsim_seqx_reset(fsim_seqx* s);
int fsim_seqx_destroy(fsim_seqx* s);

#ifdef __cplusplus
}
#endif
#endif /* FAIRSIM_GB300_H */
