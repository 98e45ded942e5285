// JNI shim: exports the symbols the reference's accel Java classes bind
// (org/fairsim/accel/AccelVectorReal.java:218-247,330-333, AccelVectorCplx.java:296-331,
// 483-492, FFTProvider.java:105, AccelVectorFactory.java:139-146) and the natives of
// org.fairsim.gb300.FusedSim (jni/org/fairsim/gb300/FusedSim.java), each forwarding to the C
// ABI in include/fairsim_gb300.h. With this library on java.library.path in place of the
// reference's libcudaimpl, the existing Java classes run unchanged on the GB300 kernels.
//
// Failures become the Java exceptions the reference raises: FSIM_EOOM -> OutOfMemoryError
// (alloc returns 0 instead, which AccelVectorCplx.java:51-54 turns into one),
// FSIM_EINVAL -> IllegalArgumentException, anything else -> RuntimeException, all with
// fsim_last_error()'s message. Nothing is called back from CUDA threads: buffers the Java
// factory hands in are returned before the native returns.
//
// Built by fairsim-vigor_gb300/build.py only when a JDK's jni.h is found (JAVA_HOME).
#include <jni.h>

#include <cstdint>
#include <vector>

#include "../../include/fairsim_gb300.h"

namespace {

struct JVec {  // what a Java vector's natData points to
  fsim_vec* v = nullptr;
  jobject factory = nullptr;  // global ref: buffers go back to its pools
  jmethodID ret_host = nullptr, ret_dev = nullptr;
};

JVec* jv(jlong h) { return reinterpret_cast<JVec*>(h); }

void throw_status(JNIEnv* env, int rc) {
  if (rc == FSIM_OK || env->ExceptionCheck()) return;
  const char* cls = rc == FSIM_EOOM     ? "java/lang/OutOfMemoryError"
                    : rc == FSIM_EINVAL ? "java/lang/IllegalArgumentException"
                                        : "java/lang/RuntimeException";
  env->ThrowNew(env->FindClass(cls), fsim_last_error());
}

jlong alloc_vec(JNIEnv* env, jobject factory, jint n, int cplx) {
  JVec* h = new JVec();
  if (fsim_vec_create(&h->v, n, 1, cplx) != FSIM_OK) {
    delete h;
    return 0;  // the Java side raises OutOfMemoryError
  }
  if (factory) {
    h->factory = env->NewGlobalRef(factory);
    jclass fc = env->GetObjectClass(factory);
    h->ret_host = env->GetMethodID(fc, "returnNativeHostBuffer", "(J)V");
    h->ret_dev = env->GetMethodID(fc, "returnNativeDeviceBuffer", "(J)V");
  }
  return reinterpret_cast<jlong>(h);
}

void dealloc_vec(JNIEnv* env, jlong addr) {
  JVec* h = jv(addr);
  if (!h) return;
  fsim_vec_destroy(h->v);
  if (h->factory) env->DeleteGlobalRef(h->factory);
  delete h;
}

void give_back(JNIEnv* env, JVec* h, jlong host_buf, jlong dev_buf) {
  if (!h->factory) return;
  if (host_buf && h->ret_host) env->CallVoidMethod(h->factory, h->ret_host, host_buf);
  if (dev_buf && h->ret_dev) env->CallVoidMethod(h->factory, h->ret_dev, dev_buf);
}

// copyBuffer: every copy mode is synchronous here (the library stages through its own
// pinned memory); the Java pool's host buffer (mode 2) is returned at once
void copy_buffer(JNIEnv* env, jlong addr, jfloatArray arr, jlong buffer, jboolean to_java) {
  JVec* h = jv(addr);
  float* p = static_cast<float*>(env->GetPrimitiveArrayCritical(arr, nullptr));
  if (!p) {
    env->ThrowNew(env->FindClass("java/lang/OutOfMemoryError"), "JNI buffer copy");
    return;
  }
  const int rc = to_java ? fsim_vec_download(h->v, p) : fsim_vec_upload(h->v, p);
  env->ReleasePrimitiveArrayCritical(arr, p, to_java ? 0 : JNI_ABORT);
  give_back(env, h, buffer, 0);
  throw_status(env, rc);
}

void copy_short(JNIEnv* env, jlong addr, jlong host_buf, jlong dev_buf, jshortArray arr) {
  JVec* h = jv(addr);
  void* p = env->GetPrimitiveArrayCritical(arr, nullptr);
  if (!p) {
    env->ThrowNew(env->FindClass("java/lang/OutOfMemoryError"), "JNI buffer copy");
    return;
  }
  const int rc = fsim_vec_upload_u16(h->v, static_cast<const uint16_t*>(p));
  env->ReleasePrimitiveArrayCritical(arr, p, JNI_ABORT);
  give_back(env, h, host_buf, dev_buf);
  throw_status(env, rc);
}

jdouble reduce(JNIEnv* env, jlong addr, jboolean sqr) {
  double re = 0, im = 0;
  const int rc = sqr ? fsim_vec_norm2(jv(addr)->v, &re) : fsim_vec_sum(jv(addr)->v, &re, &im);
  throw_status(env, rc);
  return re;
}

}  // namespace

#define JFN(ret, cls, name) JNIEXPORT ret JNICALL Java_org_fairsim_accel_##cls##_##name

extern "C" {

// ---- AccelVectorReal / AccelVectorReal2d ----
JFN(jlong, AccelVectorReal, alloc)(JNIEnv* env, jobject, jobject vf, jint n) { return alloc_vec(env, vf, n, 0); }
JFN(void, AccelVectorReal, dealloc)(JNIEnv* env, jobject, jlong a) { dealloc_vec(env, a); }
JFN(void, AccelVectorReal, copyBuffer)(JNIEnv* env, jobject, jlong a, jfloatArray arr, jlong buf, jboolean to_java,
                                      jint) {
  copy_buffer(env, a, arr, buf, to_java);
}
JFN(void, AccelVectorReal, nativeAdd)(JNIEnv* env, jobject, jlong a, jlong b, jint) {
  throw_status(env, fsim_vec_add(jv(a)->v, jv(b)->v));
}
JFN(void, AccelVectorReal, nativeADDCONST)(JNIEnv* env, jobject, jlong a, jint, jfloat c) {
  throw_status(env, fsim_vec_addconst(jv(a)->v, c, 0.f));
}
JFN(void, AccelVectorReal, nativeAXPY)(JNIEnv* env, jobject, jfloat c, jlong a, jlong b, jint) {
  throw_status(env, fsim_vec_axpy(jv(a)->v, c, 0.f, jv(b)->v));
}
JFN(void, AccelVectorReal, nativeTIMES)(JNIEnv* env, jobject, jlong a, jlong b, jint) {
  throw_status(env, fsim_vec_times(jv(a)->v, jv(b)->v, 0));
}
JFN(jdouble, AccelVectorReal, nativeREDUCE)(JNIEnv* env, jobject, jlong a, jint, jboolean sqr) {
  return reduce(env, a, sqr);
}
JFN(void, AccelVectorReal, nativeZero)(JNIEnv* env, jobject, jlong a, jint) { throw_status(env, fsim_vec_zero(jv(a)->v)); }
JFN(void, AccelVectorReal, nativeScal)(JNIEnv* env, jobject, jlong a, jint, jfloat c) {
  throw_status(env, fsim_vec_scal(jv(a)->v, c, 0.f));
}
JFN(void, AccelVectorReal2d, nativeCOPYSHORT)(JNIEnv* env, jobject, jlong a, jlong hb, jlong db, jshortArray arr, jint) {
  copy_short(env, a, hb, db, arr);
}
JFN(void, AccelVectorReal2d, nativeSet)(JNIEnv* env, jobject, jlong a, jint x, jint y, jint w, jfloat v) {
  throw_status(env, fsim_vec_set_elem(jv(a)->v, (size_t)x + (size_t)y * w, v, 0.f));
}
JFN(jfloat, AccelVectorReal2d, nativeGet)(JNIEnv* env, jobject, jlong a, jint x, jint y, jint w) {
  float re = 0;
  throw_status(env, fsim_vec_get_elem(jv(a)->v, (size_t)x + (size_t)y * w, &re, nullptr));
  return re;
}

// ---- AccelVectorCplx / AccelVectorCplx2d ----
JFN(jlong, AccelVectorCplx, alloc)(JNIEnv* env, jobject, jobject vf, jint n) { return alloc_vec(env, vf, n, 1); }
JFN(void, AccelVectorCplx, dealloc)(JNIEnv* env, jobject, jlong a) { dealloc_vec(env, a); }
JFN(void, AccelVectorCplx, copyBuffer)(JNIEnv* env, jobject, jlong a, jfloatArray arr, jlong buf, jboolean to_java,
                                      jint) {
  copy_buffer(env, a, arr, buf, to_java);
}
JFN(void, AccelVectorCplx, nativeCOPYREAL)(JNIEnv* env, jobject, jlong out, jlong in, jint) {
  throw_status(env, fsim_vec_copy(jv(out)->v, jv(in)->v));
}
JFN(void, AccelVectorCplx, nativeCOPYCPLX)(JNIEnv* env, jobject, jlong out, jlong in, jint) {
  throw_status(env, fsim_vec_copy(jv(out)->v, jv(in)->v));
}
JFN(void, AccelVectorCplx, nativeAdd)(JNIEnv* env, jobject, jlong a, jlong b, jint) {
  throw_status(env, fsim_vec_add(jv(a)->v, jv(b)->v));
}
JFN(void, AccelVectorCplx, nativeADDCONST)(JNIEnv* env, jobject, jlong a, jint, jfloat re, jfloat im) {
  throw_status(env, fsim_vec_addconst(jv(a)->v, re, im));
}
JFN(void, AccelVectorCplx, nativeAXPY)(JNIEnv* env, jobject, jfloat re, jfloat im, jlong a, jlong b, jint) {
  throw_status(env, fsim_vec_axpy(jv(a)->v, re, im, jv(b)->v));
}
JFN(void, AccelVectorCplx, nativeTIMES)(JNIEnv* env, jobject, jlong a, jlong b, jint, jboolean conj) {
  throw_status(env, fsim_vec_times(jv(a)->v, jv(b)->v, conj ? 1 : 0));
}
JFN(void, AccelVectorCplx, nativeTIMESREAL)(JNIEnv* env, jobject, jlong a, jlong b, jint) {
  throw_status(env, fsim_vec_times(jv(a)->v, jv(b)->v, 0));
}
JFN(jdouble, AccelVectorCplx, nativeREDUCE)(JNIEnv* env, jobject, jlong a, jint, jboolean sqr) {
  return reduce(env, a, sqr);
}
JFN(void, AccelVectorCplx, nativeZero)(JNIEnv* env, jobject, jlong a, jint) { throw_status(env, fsim_vec_zero(jv(a)->v)); }
JFN(void, AccelVectorCplx, nativeScal)(JNIEnv* env, jobject, jlong a, jint, jfloat re, jfloat im) {
  throw_status(env, fsim_vec_scal(jv(a)->v, re, im));
}
JFN(void, AccelVectorCplx2d, nativeCOPYSHORT)(JNIEnv* env, jobject, jlong a, jlong hb, jlong db, jshortArray arr, jint,
                                              jint) {
  copy_short(env, a, hb, db, arr);
}
JFN(void, AccelVectorCplx2d, nativeSet)(JNIEnv* env, jobject, jlong a, jint x, jint y, jint w, jfloat re, jfloat im) {
  throw_status(env, fsim_vec_set_elem(jv(a)->v, (size_t)x + (size_t)y * w, re, im));
}
JFN(jfloatArray, AccelVectorCplx2d, nativeGet)(JNIEnv* env, jobject, jlong a, jint x, jint y, jint w) {
  float v[2] = {0.f, 0.f};
  throw_status(env, fsim_vec_get_elem(jv(a)->v, (size_t)x + (size_t)y * w, &v[0], &v[1]));
  jfloatArray r = env->NewFloatArray(2);
  if (r) env->SetFloatArrayRegion(r, 0, 2, v);
  return r;
}
JFN(void, AccelVectorCplx2d, nativeFFT)(JNIEnv* env, jobject, jlong plan, jlong a, jboolean inverse) {
  const int w = (int)(plan >> 32), h = (int)(plan & 0xffffffff);
  int rc = fsim_vec_reshape(jv(a)->v, w, h);
  if (rc == FSIM_OK) rc = fsim_vec_fft2d(jv(a)->v, inverse ? 1 : 0);
  throw_status(env, rc);
}
JFN(void, AccelVectorCplx2d, nativeFourierShift)(JNIEnv* env, jobject, jlong a, jint n, jdouble kx, jdouble ky) {
  int rc = fsim_vec_reshape(jv(a)->v, n, n);
  if (rc == FSIM_OK) rc = fsim_vec_fourier_shift(jv(a)->v, kx, ky);
  throw_status(env, rc);
}
JFN(void, AccelVectorCplx2d, nativePasteFreq)(JNIEnv* env, jobject, jlong out, jint wo, jint ho, jlong in, jint wi,
                                              jint hi, jint xoff, jint yoff) {
  int rc = fsim_vec_reshape(jv(out)->v, wo, ho);
  if (rc == FSIM_OK) rc = fsim_vec_reshape(jv(in)->v, wi, hi);
  if (rc == FSIM_OK) rc = fsim_vec_paste_freq(jv(out)->v, jv(in)->v, xoff, yoff);
  throw_status(env, rc);
}

// ---- FFTProvider / AccelVectorFactory ----
JFN(jlong, FFTProvider, nativeCreatePlan2d)(JNIEnv* env, jclass, jint w, jint h) {
  int64_t plan = 0;
  throw_status(env, fsim_fft_plan_2d(w, h, &plan));
  return (jlong)plan;
}
JFN(void, AccelVectorFactory, nativeSync)(JNIEnv* env, jclass) { throw_status(env, fsim_sync()); }
JFN(jlong, AccelVectorFactory, nativeAllocMemory)(JNIEnv* env, jobject, jint size) {
  void* p = nullptr;
  throw_status(env, fsim_buffer_alloc((size_t)size, 0, &p));
  return reinterpret_cast<jlong>(p);
}
JFN(jlong, AccelVectorFactory, nativeAllocMemoryHost)(JNIEnv* env, jobject, jint size) {
  void* p = nullptr;
  throw_status(env, fsim_buffer_alloc((size_t)size, 1, &p));
  return reinterpret_cast<jlong>(p);
}
JFN(void, AccelVectorFactory, startProfiler)(JNIEnv* env, jclass) { throw_status(env, fsim_profiler(1)); }
JFN(void, AccelVectorFactory, stopProfiler)(JNIEnv* env, jclass) { throw_status(env, fsim_profiler(0)); }

// ---- org.fairsim.gb300.FusedSim: fused plans, batches, fit ----
static int fill_param(JNIEnv* env, fsim_sim_param* p, jintArray geom, jdoubleArray optics, jdoubleArray dirs) {
  // geom: w, nDirs, nBands, nPhases, useAttenuation
  // optics: micronsPerPixel, na, emWavelength, otfA, attStrength, attFWHM, wiener, apoCutoff, apoBend
  // dirs: per direction px, py, phaOff, then modulations of bands 0..nBands-1
  *p = fsim_sim_param{};
  jint g[5];
  jdouble o[9];
  env->GetIntArrayRegion(geom, 0, 5, g);
  env->GetDoubleArrayRegion(optics, 0, 9, o);
  if (env->ExceptionCheck()) return FSIM_EINVAL;
  p->w = g[0];
  p->nr_dirs = g[1];
  p->nr_bands = g[2];
  p->nr_phases = g[3];
  p->use_attenuation = g[4];
  p->microns_per_pixel = o[0];
  p->na = o[1];
  p->em_wavelength = o[2];
  p->otf_a = o[3];
  p->att_strength = o[4];
  p->att_fwhm = o[5];
  p->wiener = o[6];
  p->apo_cutoff = o[7];
  p->apo_bend = o[8];
  if (p->nr_dirs < 1 || p->nr_dirs > FSIM_MAX_DIRS || p->nr_bands < 1 || p->nr_bands > FSIM_MAX_BANDS) return FSIM_EINVAL;
  const int per = 3 + p->nr_bands;
  std::vector<jdouble> d((size_t)per * p->nr_dirs);
  env->GetDoubleArrayRegion(dirs, 0, (jsize)d.size(), d.data());
  if (env->ExceptionCheck()) return FSIM_EINVAL;
  for (int i = 0; i < p->nr_dirs; i++) {
    p->px[i] = d[i * per + 0];
    p->py[i] = d[i * per + 1];
    p->pha_off[i] = d[i * per + 2];
    for (int b = 0; b < p->nr_bands; b++) p->modulation[i][b] = d[i * per + 3 + b];
  }
  return FSIM_OK;
}

}  // extern "C"

#define GFN(ret, name) JNIEXPORT ret JNICALL Java_org_fairsim_gb300_FusedSim_##name

extern "C" {

GFN(jlong, planCreate)(JNIEnv* env, jclass, jintArray geom, jdoubleArray optics, jdoubleArray dirs, jint path,
                      jint input_type, jint fade_px, jdouble bgr) {
  fsim_sim_param p;
  int rc = fill_param(env, &p, geom, optics, dirs);
  fsim_plan* plan = nullptr;
  if (rc == FSIM_OK) rc = fsim_plan_create(&plan, &p, path, input_type, fade_px, bgr);
  throw_status(env, rc);
  return reinterpret_cast<jlong>(plan);
}
GFN(void, planUpdate)(JNIEnv* env, jclass, jlong plan, jintArray geom, jdoubleArray optics, jdoubleArray dirs) {
  fsim_sim_param p;
  int rc = fill_param(env, &p, geom, optics, dirs);
  if (rc == FSIM_OK) rc = fsim_plan_update(reinterpret_cast<fsim_plan*>(plan), &p);
  throw_status(env, rc);
}
GFN(void, planDestroy)(JNIEnv* env, jclass, jlong plan) {
  throw_status(env, fsim_plan_destroy(reinterpret_cast<fsim_plan*>(plan)));
}
// raw: float[] (f32 plans) or short[] (u16 plans), nDirs*nPhases*w*w; out: float[] 2w*2w
GFN(void, reconstruct)(JNIEnv* env, jclass, jlong plan, jarray raw, jfloatArray out) {
  void* r = env->GetPrimitiveArrayCritical(raw, nullptr);
  float* o = r ? static_cast<float*>(env->GetPrimitiveArrayCritical(out, nullptr)) : nullptr;
  int rc = (r && o) ? fsim_recon_host(reinterpret_cast<fsim_plan*>(plan), r, o) : FSIM_EOOM;
  if (o) env->ReleasePrimitiveArrayCritical(out, o, 0);
  if (r) env->ReleasePrimitiveArrayCritical(raw, r, JNI_ABORT);
  throw_status(env, rc);
}
// the reconstruction with runReconstruction's "Widefield" and "filtered Widefield" images
// (SimAlgorithm.java:533-576): offline plans, each output float[] 2w*2w; wf or fwf may be null
GFN(void, reconstructWidefield)(JNIEnv* env, jclass, jlong plan, jarray raw, jfloatArray out, jfloatArray wf,
                                jfloatArray fwf) {
  fsim_host_job j{};
  j.plan = reinterpret_cast<const fsim_plan*>(plan);
  j.raw_host = env->GetPrimitiveArrayCritical(raw, nullptr);
  int rc = j.raw_host ? FSIM_OK : FSIM_EOOM;
  if (rc == FSIM_OK) j.out_host = static_cast<float*>(env->GetPrimitiveArrayCritical(out, nullptr));
  if (rc == FSIM_OK && !j.out_host) rc = FSIM_EOOM;
  if (rc == FSIM_OK && wf) {
    j.widefield_host = static_cast<float*>(env->GetPrimitiveArrayCritical(wf, nullptr));
    if (!j.widefield_host) rc = FSIM_EOOM;
  }
  if (rc == FSIM_OK && fwf) {
    j.filtered_widefield_host = static_cast<float*>(env->GetPrimitiveArrayCritical(fwf, nullptr));
    if (!j.filtered_widefield_host) rc = FSIM_EOOM;
  }
  if (rc == FSIM_OK) rc = fsim_recon_batch_host(&j, 1, 1);
  if (j.filtered_widefield_host) env->ReleasePrimitiveArrayCritical(fwf, j.filtered_widefield_host, 0);
  if (j.widefield_host) env->ReleasePrimitiveArrayCritical(wf, j.widefield_host, 0);
  if (j.out_host) env->ReleasePrimitiveArrayCritical(out, j.out_host, 0);
  if (j.raw_host) env->ReleasePrimitiveArrayCritical(raw, const_cast<void*>(j.raw_host), JNI_ABORT);
  throw_status(env, rc);
}
// many stacks at once: overlapped uploads, passes and downloads (fsim_recon_batch_host)
GFN(void, reconstructBatch)(JNIEnv* env, jclass, jlongArray plans, jobjectArray raws, jobjectArray outs) {
  const jsize n = env->GetArrayLength(plans);
  std::vector<jlong> ph(n);
  env->GetLongArrayRegion(plans, 0, n, ph.data());
  std::vector<fsim_host_job> jobs(n);
  std::vector<jarray> ra(n), oa(n);
  int rc = FSIM_OK;
  jsize got = 0;
  for (; got < n; got++) {  // critical sections may nest; no JNI calls in between
    ra[got] = (jarray)env->GetObjectArrayElement(raws, got);
    oa[got] = (jarray)env->GetObjectArrayElement(outs, got);
  }
  for (jsize i = 0; i < n; i++) {
    jobs[i].plan = reinterpret_cast<const fsim_plan*>(ph[i]);
    jobs[i].raw_host = env->GetPrimitiveArrayCritical(ra[i], nullptr);
    jobs[i].out_host = static_cast<float*>(env->GetPrimitiveArrayCritical(oa[i], nullptr));
    jobs[i].widefield_host = nullptr;
    jobs[i].filtered_widefield_host = nullptr;
    if (!jobs[i].raw_host || !jobs[i].out_host) rc = FSIM_EOOM;
  }
  if (rc == FSIM_OK) rc = fsim_recon_batch_host(jobs.data(), n, 0);
  for (jsize i = n; i-- > 0;) {
    if (jobs[i].out_host) env->ReleasePrimitiveArrayCritical(oa[i], jobs[i].out_host, 0);
    if (jobs[i].raw_host) env->ReleasePrimitiveArrayCritical(ra[i], const_cast<void*>(jobs[i].raw_host), JNI_ABORT);
  }
  throw_status(env, rc);
}
// SimAlgorithm.estimateParameters on a raw stack; writes the fitted px, py, phaOff and
// modulations back into dirs (same layout as planCreate's)
GFN(void, estimate)(JNIEnv* env, jclass, jintArray geom, jdoubleArray optics, jdoubleArray dirs, jfloatArray raw,
                   jint fade_px, jint fit_band, jdouble fit_exclude) {
  fsim_sim_param p;
  int rc = fill_param(env, &p, geom, optics, dirs);
  const size_t n = (size_t)p.w * p.w * p.nr_dirs * p.nr_phases;
  if (rc == FSIM_OK) {
    std::vector<float> h(n);
    env->GetFloatArrayRegion(raw, 0, (jsize)n, h.data());
    fsim_vec* tmp = nullptr;  // the stack goes to the device as one real vector
    rc = fsim_vec_create(&tmp, (int)n, 1, 0);
    if (rc == FSIM_OK) rc = fsim_vec_upload(tmp, h.data());
    void* src = nullptr;
    if (rc == FSIM_OK) rc = fsim_vec_info(tmp, nullptr, nullptr, nullptr, &src);
    if (rc == FSIM_OK) rc = fsim_estimate_raw(&p, src, FSIM_INPUT_F32, fade_px, fit_band, fit_exclude, nullptr);
    fsim_vec_destroy(tmp);
  }
  if (rc == FSIM_OK) {
    const int per = 3 + p.nr_bands;
    std::vector<jdouble> d((size_t)per * p.nr_dirs);
    for (int i = 0; i < p.nr_dirs; i++) {
      d[i * per + 0] = p.px[i];
      d[i * per + 1] = p.py[i];
      d[i * per + 2] = p.pha_off[i];
      for (int b = 0; b < p.nr_bands; b++) d[i * per + 3 + b] = p.modulation[i][b];
    }
    env->SetDoubleArrayRegion(dirs, 0, (jsize)d.size(), d.data());
  }
  throw_status(env, rc);
}

JNIEXPORT jint JNICALL JNI_OnLoad(JavaVM*, void*) { return JNI_VERSION_1_6; }

}  // extern "C"
