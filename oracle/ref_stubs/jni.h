/* Minimal C declarations of the Java Native Interface, written from the public JNI
 * specification: the types and linkage macros, and the JNIEnv functions that the
 * reference's standard-C vector backend (accel/stdC_*.c) names. Test infrastructure for
 * the oracle only: the harness calls the compute natives with env == NULL, and none of
 * those touch env (the array-copy natives that do are never called). */
#ifndef FSIM_REF_STUB_JNI_H
#define FSIM_REF_STUB_JNI_H
#include <stdarg.h>
#include <stdint.h>

#define JNIEXPORT __attribute__((visibility("default")))
#define JNICALL
#define JNI_FALSE 0
#define JNI_TRUE 1

typedef int32_t jint;
typedef int64_t jlong;
typedef int8_t jbyte;
typedef uint8_t jboolean;
typedef uint16_t jchar;
typedef int16_t jshort;
typedef float jfloat;
typedef double jdouble;
typedef jint jsize;
typedef void* jobject;
typedef jobject jclass;
typedef jobject jarray;
typedef jarray jfloatArray;
typedef jarray jshortArray;

struct JNINativeInterface_;
typedef const struct JNINativeInterface_* JNIEnv;
struct JNINativeInterface_ {
  jclass (*FindClass)(JNIEnv*, const char*);
  jint (*ThrowNew)(JNIEnv*, jclass, const char*);
  jfloatArray (*NewFloatArray)(JNIEnv*, jsize);
  void (*SetFloatArrayRegion)(JNIEnv*, jfloatArray, jsize, jsize, const jfloat*);
  void* (*GetPrimitiveArrayCritical)(JNIEnv*, jarray, jboolean*);
  void (*ReleasePrimitiveArrayCritical)(JNIEnv*, jarray, void*, jint);
};
#endif
