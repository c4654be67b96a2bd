// crm_device.cuh -- device helpers of the column kernel: precision policy,
// saturation functions (crm/sat.F90) and the slab accessors.
#pragma once
#include <cuda_runtime.h>
#include "crm_layout.h"
#include "../../include/crm_detmath.h"

namespace crm {

// Fortran default-REAL literal (the reference is built without -r8):
// the value is the float nearest the decimal, widened to double.
#define R4(x) ((double)(x##f))

// ------------------------------------------------------------ precision
// T is the bulk arithmetic type: double for the plain form, float for the
// FP32-mixed form.  Math wrappers pick the deterministic double functions
// (bit-identical to the CPU restatement) or the float intrinsics.
__device__ __forceinline__ double tsqrt(double x) { return sqrt(x); }
__device__ __forceinline__ float tsqrt(float x) { return sqrtf(x); }
__device__ __forceinline__ double tabs_(double x) { return fabs(x); }
__device__ __forceinline__ float tabs_(float x) { return fabsf(x); }
__device__ __forceinline__ double tpow(double x, double y) { return crm_detmath::det_pow(x, y); }
__device__ __forceinline__ float tpow(float x, float y) { return (x == 0.f) ? 0.f : __expf(y * __logf(x)); }
__device__ __forceinline__ double texp(double x) { return crm_detmath::det_exp(x); }
__device__ __forceinline__ float texp(float x) { return __expf(x); }
__device__ __forceinline__ double tlog(double x) { return crm_detmath::det_log(x); }
__device__ __forceinline__ float tlog(float x) { return __logf(x); }

// max/min with a fixed choice on ties and signed zeros, the same on the
// CPU restatement: returns b only if it compares greater (smaller).
template <typename T> __device__ __forceinline__ T mx2(T a, T b) { return (b > a) ? b : a; }
template <typename T> __device__ __forceinline__ T mn2(T a, T b) { return (b < a) ? b : a; }
// FP32-mixed form: the hardware min/max, one instruction; it differs from
// the rule above only for NaN operands and the sign of a zero result.
template <> __device__ __forceinline__ float mx2<float>(float a, float b) { return fmaxf(a, b); }
template <> __device__ __forceinline__ float mn2<float>(float a, float b) { return fminf(a, b); }
template <typename T> __device__ __forceinline__ T mx3(T a, T b, T c) { return mx2(mx2(a, b), c); }
template <typename T> __device__ __forceinline__ T mn3(T a, T b, T c) { return mn2(mn2(a, b), c); }

// ------------------------------------------------------------ sat.F90
// Flatau et al. (JAM 1992) 8th-order polynomials above -80 C, Murphy and
// Koop (2005) below (sat.F90:12-139).  Coefficients are REAL*4 values.
template <typename T> __device__ __forceinline__ T poly8(T dt, const double *a) {
  return (T)a[0] + dt * ((T)a[1] + dt * ((T)a[2] + dt * ((T)a[3] + dt * ((T)a[4] + dt * ((T)a[5] + dt * ((T)a[6] + dt * ((T)a[7] + (T)a[8] * dt)))))));
}
__device__ __constant__ double c_esatw[9] = {R4(6.105851), R4(0.4440316), R4(0.1430341e-1), R4(0.2641412e-3),
                                             R4(0.2995057e-5), R4(0.2031998e-7), R4(0.6936113e-10),
                                             R4(0.2564861e-13), R4(-0.3704404e-15)};
__device__ __constant__ double c_dtesatw[9] = {R4(0.443956472), R4(0.285976452e-1), R4(0.794747212e-3),
                                               R4(0.121167162e-4), R4(0.103167413e-6), R4(0.385208005e-9),
                                               R4(-0.604119582e-12), R4(-0.792933209e-14), R4(-0.599634321e-17)};
__device__ __constant__ double c_esati[9] = {R4(6.11147274), R4(0.503160820), R4(0.188439774e-1),
                                             R4(0.420895665e-3), R4(0.615021634e-5), R4(0.602588177e-7),
                                             R4(0.385852041e-9), R4(0.146898966e-11), R4(0.252751365e-14)};
__device__ __constant__ double c_dtesati[9] = {R4(0.503223089), R4(0.377174432e-1), R4(0.126710138e-2),
                                               R4(0.249065913e-4), R4(0.312668753e-6), R4(0.255653718e-8),
                                               R4(0.132073448e-10), R4(0.390204672e-13), R4(0.497275778e-16)};

template <typename T> __device__ __forceinline__ T mk_low(T t) {
  return texp((((T)R4(9.550426) - (T)R4(5723.265) / t) + (T)R4(3.53068) * tlog(t)) - (T)R4(0.00728332) * t);
}
template <typename T> __device__ T esatw(T t) {
  T dt = t - (T)R4(273.16);
  if (dt > (T)-80.) return poly8(dt, c_esatw);
  return (T)(double)(2.0f * 0.01f) * mk_low(t);
}
template <typename T> __device__ T esati(T t) {
  T dt = t - (T)R4(273.16);
  if (dt > (T)-80.) return poly8(dt, c_esati);
  return (T)R4(0.01) * mk_low(t);
}
template <typename T> __device__ T dtesatw(T t) {
  T dt = t - (T)R4(273.16);
  if (dt > (T)-80.) return poly8(dt, c_dtesatw);
  return esatw(t + (T)1.0) - esatw(t);
}
template <typename T> __device__ T dtesati(T t) {
  T dt = t - (T)R4(273.16);
  if (dt > (T)-80.) return poly8(dt, c_dtesati);
  return esati(t + (T)1.0) - esati(t);
}
template <typename T> __device__ __forceinline__ T qsatw(T t, T p) {
  T es = esatw(t);
  return ((T)R4(0.622) * es) / mx2(es, p - es);
}
template <typename T> __device__ __forceinline__ T qsati(T t, T p) {
  T es = esati(t);
  return ((T)R4(0.622) * es) / mx2(es, p - es);
}
template <typename T> __device__ __forceinline__ T dtqsatw(T t, T p) { return ((T)R4(0.622) * dtesatw(t)) / p; }
template <typename T> __device__ __forceinline__ T dtqsati(T t, T p) { return ((T)R4(0.622) * dtesati(t)) / p; }

// ------------------------------------------------------------ accessors
// (i, k) view of a slab field of the 2D CRM (Y3 = false); a 3D CRM field
// (Y3 = true) is stored level by level, each level nya rows of nxa, and is
// addressed either as (i, j, k) or, by the phases that never look at a
// horizontal neighbour, as (h, k) with h = i + nx (j - 1) the interior cell
// index 1..nx*ny (nx a power of two: lnx = log2 nx).
template <typename T, bool Y3 = false> struct F2 {
  T *p;
  int x1, nxa, z1;
  int y1, plane, lnx;                 // 3D only
  __device__ __forceinline__ T &operator()(int h, int k) const {
    if constexpr (!Y3) {
      return p[(k - z1) * nxa + (h - x1)];
    } else {
      const int hh = h - 1, i = (hh & ((1 << lnx) - 1)) + 1, j = (hh >> lnx) + 1;
      return p[(size_t)(k - z1) * plane + (j - y1) * nxa + (i - x1)];
    }
  }
  __device__ __forceinline__ T &operator()(int i, int j, int k) const {
    return p[(size_t)(k - z1) * plane + (j - y1) * nxa + (i - x1)];
  }
};

}  // namespace crm
