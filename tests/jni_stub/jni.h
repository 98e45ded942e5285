/* Minimal declarations of the Java Native Interface, written from the public JNI
 * specification (types, linkage macros and the JNIEnv functions the fsim JNI shim calls),
 * so that tests/test_jni_shim.py can type-check the shim on a machine without a JDK.
 * Declarations only: nothing here is linked or run. */
#ifndef FSIM_TEST_JNI_STUB_H
#define FSIM_TEST_JNI_STUB_H
#include <cstdarg>
#include <cstdint>

#define JNIEXPORT __attribute__((visibility("default")))
#define JNICALL
#define JNI_FALSE 0
#define JNI_TRUE 1
#define JNI_COMMIT 1
#define JNI_ABORT 2

typedef int32_t jint;
typedef int64_t jlong;
typedef int8_t jbyte;
typedef uint8_t jboolean;
typedef uint16_t jchar;
typedef int16_t jshort;
typedef float jfloat;
typedef double jdouble;
typedef jint jsize;

class _jobject {};
class _jclass : public _jobject {};
class _jthrowable : public _jobject {};
class _jstring : public _jobject {};
class _jarray : public _jobject {};
class _jbooleanArray : public _jarray {};
class _jbyteArray : public _jarray {};
class _jcharArray : public _jarray {};
class _jshortArray : public _jarray {};
class _jintArray : public _jarray {};
class _jlongArray : public _jarray {};
class _jfloatArray : public _jarray {};
class _jdoubleArray : public _jarray {};
class _jobjectArray : public _jarray {};
typedef _jobject* jobject;
typedef _jclass* jclass;
typedef _jthrowable* jthrowable;
typedef _jstring* jstring;
typedef _jarray* jarray;
typedef _jbooleanArray* jbooleanArray;
typedef _jbyteArray* jbyteArray;
typedef _jcharArray* jcharArray;
typedef _jshortArray* jshortArray;
typedef _jintArray* jintArray;
typedef _jlongArray* jlongArray;
typedef _jfloatArray* jfloatArray;
typedef _jdoubleArray* jdoubleArray;
typedef _jobjectArray* jobjectArray;
struct _jmethodID;
typedef struct _jmethodID* jmethodID;
struct _jfieldID;
typedef struct _jfieldID* jfieldID;

struct JNIEnv_ {
  jclass FindClass(const char* name);
  jint ThrowNew(jclass clazz, const char* msg);
  jboolean ExceptionCheck();
  jobject NewGlobalRef(jobject obj);
  void DeleteGlobalRef(jobject obj);
  jclass GetObjectClass(jobject obj);
  jmethodID GetMethodID(jclass clazz, const char* name, const char* sig);
  void CallVoidMethod(jobject obj, jmethodID methodID, ...);
  jsize GetArrayLength(jarray array);
  jobject GetObjectArrayElement(jobjectArray array, jsize index);
  jfloatArray NewFloatArray(jsize len);
  void GetIntArrayRegion(jintArray array, jsize start, jsize len, jint* buf);
  void GetLongArrayRegion(jlongArray array, jsize start, jsize len, jlong* buf);
  void GetFloatArrayRegion(jfloatArray array, jsize start, jsize len, jfloat* buf);
  void GetDoubleArrayRegion(jdoubleArray array, jsize start, jsize len, jdouble* buf);
  void SetFloatArrayRegion(jfloatArray array, jsize start, jsize len, const jfloat* buf);
  void SetDoubleArrayRegion(jdoubleArray array, jsize start, jsize len, const jdouble* buf);
  void* GetPrimitiveArrayCritical(jarray array, jboolean* isCopy);
  void ReleasePrimitiveArrayCritical(jarray array, void* carray, jint mode);
};
typedef JNIEnv_ JNIEnv;
struct JavaVM_ {};
typedef JavaVM_ JavaVM;
#define JNI_VERSION_1_6 0x00010006

#endif
