// Fused, batched 2D SIM reconstruction: SimAlgorithm.runReconstruction
// (S/SimAlgorithm.java:268-582; Wiener filter style, OTF applied after a Fourier shift on
// the 2w x 2w grid) in three passes over HBM instead of ~40 vector ops.
//
// The reference's per-component chain, with W = 2N,
//   sep_c = sum_p M[c][p] FFT_N(raw_p);  V_c = FFT_W(ramp_c * iFFT_W(paste(sep_c)));
//   T = sum_{a,c} conj(OTF(r - k_c)) V_c;  out = Re iFFT_W(T * wiener * apo)
// is separable along x and y except for the OTF/Wiener/apo multiplications, which act
// where both axes are in frequency space. The passes are therefore:
//   A  (rows,    per dataset x angle x raw row): band mix of the raw rows in real space
//      (FFT is linear, so mixing before the transform is the same separation), FFT_N along
//      x, paste, and for shifted components the x half of the shift
//      (iFFT_W, ramp_x, FFT_W) -> only the columns inside each component's OTF support
//      window are written (the OTF zeroes everything else);
//   B  (columns, per dataset x 4-column quad): FFT_N along y, paste, y half of the shift,
//      times the exact conj(OTF) mask, accumulate all components, times wiener*apo,
//      iFFT_W along y;
//   C  (rows,    per output row): iFFT_W along x, real part, 1/W^2.
// Shift phases use exact per-axis ramp tables; OTF masks and the Wiener*apo filter are
// resident per plan, built with the reference's floor-indexed OTF lookup (table positions in
// float-float arithmetic, the reference's double-precision radius at their boundaries) and
// its double-precision apodization (one evaluation per octant point).
#include <algorithm>
#include <cmath>
#include <complex>
#include <cstring>
#include <mutex>
#include <vector>

#include "common.cuh"
#include "fft_line.cuh"
#include "filters.cuh"
#include "otf.cuh"
#include "recon.cuh"
#include "recon_kernels.cuh"
#include "runtime.cuh"
#include "sim_host.h"

namespace fsim {

std::vector<float> fade_vector(int w, int h, int px);

// ---- plan build kernels -------------------------------------------------------------------------
// conj(OTF(r - k)) mask of one component over its window, quad layout [xl/4][yl][xl%4]:
// real values for estimated OTFs; complex values (float2) of OTF band `band` for measured
// ones (OtfProvider.applyOtf(vec, band, kx, ky), S/SimAlgorithm.java:397-403). Table
// positions in float-float, the reference's double-precision lookup at their boundaries.
__global__ void k_build_mask(float* __restrict__ mask, int W, int nWin, int Xs, int Ys, double kx, double ky, FShift kf,
                             const OtfTable* __restrict__ t, int att, int band) {
  const int xl = blockIdx.x * blockDim.x + threadIdx.x, yl = blockIdx.y;
  if (xl >= nWin) return;
  int X = (Xs + xl) % W, Y = (Ys + yl) % W;
  const size_t i = ((size_t)(xl >> 2) * nWin + yl) * 4 + (xl & 3);
  float2 c = make_float2(0.f, 0.f);
  if (!otf_at_fast(*t, band, freq_x(X, W), freq_y(Y, W), kf, kx, ky, att != 0, &c)) c = make_float2(0.f, 0.f);
  if (t->measured) reinterpret_cast<float2*>(mask)[i] = make_float2(c.x, -c.y);
  else mask[i] = c.x;
}

// 1/(sum |OTF|^2 + w^2) * apo, quad layout [X/4][Y][X%4], for the columns X < ncols; the
// apodization from its octant table apo (W/2 + 1 entries per row)
__global__ void k_build_wa(float* __restrict__ wa, int ncols, int W, const OtfTable* __restrict__ t, ShiftSet shifts,
                           FShiftSet fsh, int use_att, float wp, const float* __restrict__ apo) {
  const int X = blockIdx.x * blockDim.x + threadIdx.x, Y = blockIdx.y;
  if (X >= ncols) return;
  const int xh = freq_x(X, W), yh = freq_y(Y, W);
  float acc = 0.f;
  for (int d = 0; d < shifts.n_dirs; d++)
    for (int b = 0; b < shifts.n_bands; b++) {
      const double kx = shifts.px[d] * b, ky = shifts.py[d] * b;
      const FShift k = fsh.k[d][b];
      const float v1 = wiener_term(*t, b, xh, yh, k, kx, ky, use_att != 0);
      const float v2 = wiener_term(*t, b, xh, yh, fshift_neg(k), -kx, -ky, use_att != 0);
      acc = __fadd_rn(__fadd_rn(acc, v1), v2);
    }
  const float den = __fdiv_rn(1.f, __fadd_rn(acc, wp));
  const int ax = abs(xh), ay = abs(yh);
  const float ap = __ldg(apo + (size_t)max(ax, ay) * (W / 2 + 1) + min(ax, ay));
  wa[((size_t)(X >> 2) * W + Y) * 4 + (X & 3)] = __fmul_rn(den, ap);
}

// ---- plan --------------------------------------------------------------------------------------
static int floor4(int v) { return (v >= 0) ? (v / 4) * 4 : -(((-v) + 3) / 4) * 4; }

int plan_window(const fsim_sim_param* p, double R, int* nwin) {
  const int W = 2 * p->w;
  int n = ((2 * (int)std::ceil(R) + 3 + 3) / 4) * 4 + 4;
  if (n >= W) n = W;
  *nwin = n;
  return FSIM_OK;
}

static void comp_shift(const fsim_sim_param* p, int a, int c, double* kx, double* ky) {
  if (c == 0) {
    *kx = 0;
    *ky = 0;
    return;
  }
  const int b = (c + 1) / 2;
  const double s = (c % 2 == 0) ? 1.0 : -1.0;  // pos = 2b, neg = 2b-1 (SimAlgorithm.java:385-391)
  *kx = s * band_px(p, a, b);
  *ky = s * band_py(p, a, b);
}

int Plan::build(cudaStream_t st) {
  const int N = prm.w, W = 2 * N, nA = prm.nr_dirs, nP = prm.nr_phases, nC = 2 * prm.nr_bands - 1;
  OtfTable ht;
  build_otf_table(&prm, &ht);
  const double R = ht.cutoff / ht.vec_cpm;  // OTF support radius in frequency pixels
  plan_window(&prm, R, &nwin);
  // host-side tables
  std::vector<float2> coef((size_t)nA * nC * nP);
  for (int a = 0; a < nA; a++) {
    auto m = separation_coeffs(&prm, a, false);
    for (int c = 0; c < nC; c++)
      for (int q = 0; q < nP; q++) coef[(a * nC + c) * nP + q] = make_float2(m[c * nP + q].real(), m[c * nP + q].imag());
  }
  std::vector<float2> ramps((size_t)nA * nC * 2 * W);
  std::vector<int> win((size_t)nA * nC * 2);
  for (int a = 0; a < nA; a++)
    for (int c = 0; c < nC; c++) {
      double kx, ky;
      comp_shift(&prm, a, c, &kx, &ky);
      // even/odd samples of the shift ramps on the W grid, the upsampling factors folded in:
      // x: 0.5 exp(+2 pi i kx 2n/W), exp(+2 pi i kx (2n+1)/W)/W; y likewise with -ky
      // (SimUtils.fourierShift multiplies exp(i 2 pi (kx x - ky y)/W), S/SimUtils.java:43-50)
      float2* r = &ramps[(size_t)(a * nC + c) * 2 * W];
      auto ph = [&](double k, int n) {
        double f = k * n / W;
        f -= std::floor(f);
        return 2 * M_PI * f;
      };
      for (int n = 0; n < N; n++) {
        const double e = ph(kx, 2 * n), o = ph(kx, 2 * n + 1), ey = ph(-ky, 2 * n), oy = ph(-ky, 2 * n + 1);
        r[n] = make_float2((float)(0.5 * std::cos(e)), (float)(0.5 * std::sin(e)));
        r[N + n] = make_float2((float)(std::cos(o) / W), (float)(std::sin(o) / W));
        r[W + n] = make_float2((float)(0.5 * std::cos(ey)), (float)(0.5 * std::sin(ey)));
        r[W + N + n] = make_float2((float)(std::cos(oy) / W), (float)(std::sin(oy) / W));
      }
      int xs, ys;
      if (nwin >= W) {
        xs = 0;
        ys = 0;
      } else {
        int xlo = (int)std::floor(kx - R) - 1;
        int ylo = (int)std::floor(-ky - R) - 1;  // index-space row of display y: Y = -yh mod W
        xs = ((floor4(xlo) % W) + W) % W;
        ys = ((ylo % W) + W) % W;
      }
      win[2 * (a * nC + c)] = xs;
      win[2 * (a * nC + c) + 1] = ys;
    }
  // The neg component of each pair uses the mirror image of its pos window (columns and
  // rows), so that pos values can be formed from the neg transforms at (-X, -Y). The pos
  // window has slack on both sides of the OTF support, so the mirror covers the neg support.
  const int nPair = prm.nr_bands - 1;
  for (int a = 0; a < nA; a++)
    for (int b = 1; b <= nPair; b++) {
      const int cp = 2 * b, cn = 2 * b - 1;
      win[2 * (a * nC + cn)] = ((W - win[2 * (a * nC + cp)] - nwin + 1) % W + W) % W;
      win[2 * (a * nC + cn) + 1] = ((W - win[2 * (a * nC + cp) + 1] - nwin + 1) % W + W) % W;
    }
  // Nyquist response of each pair's pos component along x and along y:
  // FFT_N((-1)^n ro[n]) with ro[n] = exp(+2 pi i k (2n+1)/W)/W (k = kx, resp. -ky), i.e.
  // exp(i phi0)/W * sum_n exp(i theta n), theta = 4 pi k/W + pi - 2 pi m/N, in closed form
  std::vector<float2> nyq((size_t)nA * nPair * 2 * N);
  for (int a = 0; a < nA; a++)
    for (int b = 1; b <= nPair; b++) {
      double kx, ky;
      comp_shift(&prm, a, 2 * b, &kx, &ky);
      for (int dim = 0; dim < 2; dim++) {
        const double k = dim == 0 ? kx : -ky;
        const double f0 = k / W - std::floor(k / W), f1 = 2 * k / W - std::floor(2 * k / W);
        const std::complex<double> e0 = std::polar(1.0 / W, 2 * M_PI * f0);
        for (int m = 0; m < N; m++) {
          double th = 2 * M_PI * f1 + M_PI - 2 * M_PI * (double)m / N;
          th -= 2 * M_PI * std::floor(th / (2 * M_PI) + 0.5);  // (-pi, pi]
          std::complex<double> S;
          if (std::fabs(th) < 1e-14) {
            S = (double)N;
          } else {
            double fn = (double)N * th / (2 * M_PI);
            fn -= std::floor(fn);
            S = (1.0 - std::polar(1.0, 2 * M_PI * fn)) / (1.0 - std::polar(1.0, th));
          }
          const std::complex<double> q = e0 * S;
          nyq[(((size_t)a * nPair + (b - 1)) * 2 + dim) * N + m] = make_float2((float)q.real(), (float)q.imag());
        }
      }
    }
  // device layout: one allocation
  auto al = [](size_t b) { return (b + 255) & ~(size_t)255; };
  size_t off_coef = 0, off_ramp = off_coef + al(coef.size() * sizeof(float2));
  size_t off_win = off_ramp + al(ramps.size() * sizeof(float2));
  size_t off_otf = off_win + al(win.size() * sizeof(int));
  size_t off_damp = off_otf + al(sizeof(OtfTable));
  size_t off_mask = off_damp + al((size_t)N * N * sizeof(float));
  const size_t mask_elem = otf_measured(&prm) ? sizeof(float2) : sizeof(float);
  size_t off_wa = off_mask + al((size_t)nA * nC * nwin * nwin * mask_elem);
  // Wiener x apo over the Hermitian half read by pass B2 (columns X <= N in whole quads),
  // then the apodization's octant table ((N + 1)^2 floats, plan build only)
  const size_t wa_elems = (size_t)(N + 4) * W, apo_elems = (size_t)(N + 1) * (N + 1);
  size_t off_nyq = off_wa + al((wa_elems + apo_elems) * sizeof(float));
  size_t off_wff = off_nyq + al(nyq.size() * sizeof(float2));
  size_t total = off_wff + al((size_t)N * N * sizeof(float));
  if (total > dev_bytes) {
    if (dev) cudaFree(dev);
    dev = nullptr;
    FSIM_CUDA(fsim::dev_alloc(&dev, total));
    dev_bytes = total;
  }
  char* b = (char*)dev;
  d_nyq = (float2*)(b + off_nyq);
  d_wff = (float*)(b + off_wff);
  d_coef = (float2*)(b + off_coef);
  d_ramps = (float2*)(b + off_ramp);
  d_win = (int*)(b + off_win);
  d_otf = (OtfTable*)(b + off_otf);
  d_damp = fade_px > 0 ? (float*)(b + off_damp) : nullptr;
  d_masks = (float*)(b + off_mask);
  d_wa = (float*)(b + off_wa);
  // uploads are synchronous (pageable sources on this stack frame)
  FSIM_CUDA(cudaMemcpyAsync(d_coef, coef.data(), coef.size() * sizeof(float2), cudaMemcpyHostToDevice, st));
  FSIM_CUDA(cudaMemcpyAsync(d_ramps, ramps.data(), ramps.size() * sizeof(float2), cudaMemcpyHostToDevice, st));
  FSIM_CUDA(cudaMemcpyAsync(d_win, win.data(), win.size() * sizeof(int), cudaMemcpyHostToDevice, st));
  FSIM_CUDA(cudaMemcpyAsync(d_otf, &ht, sizeof(OtfTable), cudaMemcpyHostToDevice, st));
  FSIM_CUDA(cudaMemcpyAsync(d_nyq, nyq.data(), nyq.size() * sizeof(float2), cudaMemcpyHostToDevice, st));
  if (d_damp) {
    std::vector<float> dv = fade_vector(N, N, fade_px);
    FSIM_CUDA(cudaMemcpyAsync(d_damp, dv.data(), dv.size() * sizeof(float), cudaMemcpyHostToDevice, st));
    FSIM_CUDA(cudaStreamSynchronize(st));
  }
  FSIM_CUDA(cudaStreamSynchronize(st));
  // masks (exact double-precision OTF lookups), Wiener x apo
  for (int a = 0; a < nA; a++)
    for (int c = 0; c < nC; c++) {
      double kx, ky;
      comp_shift(&prm, a, c, &kx, &ky);
      dim3 g(div_up(nwin, 128), nwin);
      k_build_mask<<<g, 128, 0, st>>>(d_masks + (size_t)(a * nC + c) * nwin * nwin * (mask_elem / sizeof(float)), W,
                                      nwin, win[2 * (a * nC + c)], win[2 * (a * nC + c) + 1], kx, ky,
                                      fshift_host(kx, ky), d_otf, prm.use_attenuation, (c + 1) / 2);
    }
  {
    float* d_apo = d_wa + wa_elems;
    int rc = apo_octant_device(d_apo, N, ht.vec_cpm, ht.cutoff * prm.apo_cutoff, prm.apo_bend, st);
    if (rc) return rc;
    const ShiftSet sh = shift_set(&prm);
    dim3 g(div_up(N + 4, 128), W);
    k_build_wa<<<g, 128, 0, st>>>(d_wa, N + 4, W, d_otf, sh, fshift_set(sh), prm.use_attenuation,
                                  (float)(prm.wiener * prm.wiener), d_apo);
  }
  FSIM_CHECK_LAUNCH();
  {
    int rc = build_widefield_filter(d_wff, N, d_otf, (float)(prm.wiener * prm.wiener), st);
    if (rc) return rc;
  }
  FSIM_CUDA(cudaStreamSynchronize(st));
  filter_bytes = total;
  return FSIM_OK;
}

// workspace of one dataset: I | D | G | Tw | Dy | O | On | clip max (each 256-byte aligned).
// I holds the band-0 slot (all angles summed) and one slot per angle and band pair.
static void ws_parts(const fsim_sim_param& p, int nwin, size_t part[8]) {
  const int N = p.w, W = 2 * N, nPair = p.nr_bands - 1;
  auto al = [](size_t b) { return (b + 255) & ~(size_t)255; };
  part[0] = al((size_t)(1 + p.nr_dirs * nPair) * nwin * N * sizeof(float2));
  part[1] = al((size_t)p.nr_dirs * nPair * N * sizeof(float2));
  part[2] = al((size_t)p.nr_dirs * nPair * nwin * sizeof(float2));
  part[3] = al((size_t)(1 + p.nr_dirs * nPair) * nwin * nwin * sizeof(float2));
  part[4] = al((size_t)p.nr_dirs * nPair * nwin * sizeof(float2));
  part[5] = al((size_t)W * N * sizeof(float2));
  part[6] = al((size_t)W * sizeof(float2));
  part[7] = 256;
}

size_t Plan::workspace_bytes() const {
  size_t part[8];
  ws_parts(prm, nwin, part);
  size_t sum = 0;
  for (size_t v : part) sum += v;
  return std::max(sum, widefield_ws_bytes(prm.w));
}

void Plan::fill_job(JobDesc& j, const void* raw, float* out, float* wf, float* fwf, char* ws) const {
  const int nC = 2 * prm.nr_bands - 1;
  j.raw = raw;
  j.out = out;
  j.widefield = wf;
  j.fwf = fwf;
  j.wff = d_wff;
  j.Wf = (float2*)ws;
  j.input_u16 = input_type == FSIM_INPUT_U16;
  j.nA = prm.nr_dirs;
  j.nP = prm.nr_phases;
  j.nC = nC;
  j.nWin = nwin;
  j.status = ctx().status;
  j.cmask = otf_measured(&prm) ? 1 : 0;
  j.clip = clip_scale;
  j.bgr = (float)bgr;
  j.damp = d_damp;
  j.coef = d_coef;
  j.ramps = d_ramps;
  j.win = d_win;
  j.masks = d_masks;
  j.wa = d_wa;
  j.nyq = d_nyq;
  size_t part[8];
  ws_parts(prm, nwin, part);
  char* w = ws;
  j.I = (float2*)w;
  j.D = (float2*)(w += part[0]);
  j.G = (float2*)(w += part[1]);
  j.Tw = (float2*)(w += part[2]);
  j.Dy = (float2*)(w += part[3]);
  j.O = (float2*)(w += part[4]);
  j.On = (float2*)(w += part[5]);
  j.clip_max = (float*)(w += part[6]);
}

// ---- autotuned variants ------------------------------------------------------------------------
int g_var_a[16] = {0}, g_var_b[16] = {0}, g_var_b2[16] = {0};
// variant lists: pass 0 = A (and G) elements/thread {default, alternative}; passes 1 = B1 and
// 2 = B2 (elements, columns per block), four each (recon_kernels.cuh, launch_offline)
int offline_variants(int pass) { return pass == 0 ? 2 : 4; }
static int* var_table(int pass) { return pass == 0 ? g_var_a : (pass == 1 ? g_var_b : g_var_b2); }
int offline_tune_set(int n, int pass, int v) {
  int k = size_slot(n);
  FSIM_REQUIRE(k >= 0 && pass >= 0 && pass <= 2 && v >= 0 && v < offline_variants(pass), FSIM_EINVAL,
               "tune: bad size/pass/variant %d/%d/%d", n, pass, v);
  var_table(pass)[k] = v;
  return FSIM_OK;
}
int offline_tune_get(int n, int pass) {
  int k = size_slot(n);
  return (k < 0 || pass < 0 || pass > 2) ? -1 : var_table(pass)[k];
}

extern template int launch_offline<64>(const JobDesc*, int, int, int, int, bool, int, cudaStream_t);
extern template int launch_offline<128>(const JobDesc*, int, int, int, int, bool, int, cudaStream_t);
extern template int launch_offline<192>(const JobDesc*, int, int, int, int, bool, int, cudaStream_t);
extern template int launch_offline<256>(const JobDesc*, int, int, int, int, bool, int, cudaStream_t);
extern template int launch_offline<384>(const JobDesc*, int, int, int, int, bool, int, cudaStream_t);
extern template int launch_offline<512>(const JobDesc*, int, int, int, int, bool, int, cudaStream_t);
extern template int launch_offline<768>(const JobDesc*, int, int, int, int, bool, int, cudaStream_t);
extern template int launch_offline<1024>(const JobDesc*, int, int, int, int, bool, int, cudaStream_t);
extern template int launch_offline<2048>(const JobDesc*, int, int, int, int, bool, int, cudaStream_t);

#define FSIM_RECON_SIZES(X) X(64) X(128) X(192) X(256) X(384) X(512) X(768) X(1024) X(2048)

bool offline_size_supported(int n) {
  switch (n) {
#define CASE(v) case v:
    FSIM_RECON_SIZES(CASE)
#undef CASE
    return true;
    default:
      return false;
  }
}

int launch_offline_size(int n, const JobDesc* d_jobs, int njobs, int maxA, int maxPair, int maxWin, bool scale_clip,
                        int masks, cudaStream_t st) {
  switch (n) {
#define CASE(v) \
  case v:       \
    return launch_offline<v>(d_jobs, njobs, maxA, maxPair, maxWin, scale_clip, masks, st);
    FSIM_RECON_SIZES(CASE)
#undef CASE
  }
  set_error("fused reconstruction: unsupported image size %d", n);
  return FSIM_EINVAL;
}

}  // namespace fsim
