// crm_oracle.cpp -- CPU FP64 restatement of the reference crm() (2D and 3D,
// sam1mom, SGS_TKE, MPDATA), used as the parity oracle of the GB300 library.
//
// TEST INFRASTRUCTURE ONLY: loaded by tests/, __graft_entry__.smoke() and the
// CPU-baseline leg of bench.py.  The product never links or calls this file.
//
// PARITY UNPINNED for the whole call: the reference ships no golden vectors
// or fixtures for crm(), and its Fortran cannot be compiled here, so the
// call's outputs are not checked against outputs of the reference itself;
// they are held to the reference's conservation identities and to
// mathematical properties (tests/test_oracle*.py, tests/test_gcm_coupling.py).
// Two routines are pinned against values computed from the reference's own
// source text: the sat.F90 saturation functions and the RNG_MT.F90 draws
// (tests/golden/kat.json, tests/test_oracle_kat.py).
//
// Every routine follows the reference source named in its comment line by
// line, including the Fortran numerics contract of the reference build:
//  * unsuffixed real literals are default REAL (FP32) and are rounded to float
//    before being widened (R4() below);
//  * crm/fft.F90 has no `implicit none`: its trig tables, twiddle factors and
//    scale are REAL*4 (float) values;
//  * x**2, x**3, x**4 with integer exponents are products, real exponents are
//    pow(), evaluated with the deterministic exp/log/pow of crm_detmath.h.
// The FP64 device form of the library evaluates the same operations in the
// same order, so the two agree bit for bit (tests/test_gpu_parity.py).
#include "oracle_core.h"
#include "../include/crm_gb300.h"
#include "../include/crm_detmath.h"

#include <algorithm>
#include <cmath>
#include <cstring>
#include <cstdint>
#include <vector>
#ifdef _OPENMP
#include <omp.h>
#endif

using namespace crm_detmath;

namespace oracle {

// ---------------------------------------------------------------- constants
// crm/params.F90:49-64 with the CRM branch (shr_const_mod.F90:17-55)
static const double cp = 1.00464e3;
static const double ggr = 9.80616;
static const double lcond = 2.501e6;
static const double lfus = 3.337e5;
static const double lsub = lcond + lfus;
static const double rgas_univ = 6.02214e26 * 1.38065e-23;
static const double rgas = rgas_univ / 28.966;
static const double rv = rgas_univ / 18.016;
static const double diffelq = R4(2.21e-05);
static const double therco = R4(2.40e-02);
static const double muelq = R4(1.717e-05);
static const double fac_cond = lcond / cp;
static const double fac_fus = lfus / cp;
static const double fac_sub = lsub / cp;
static const double pi = R4(3.141592653589793);
static const double epsv = R4(0.61);          // setparm.F90:87
// MICRO_SAM1MOM/micro_params.F90
static const double rhor = 1000., rhos = 100., rhog = 400.;
static const double tbgmin = R4(253.16), tbgmax = R4(273.16);
static const double tprmin = R4(268.16), tprmax = R4(283.16);
static const double tgrmin = R4(223.16), tgrmax = R4(283.16);
static const double a_rain = 842., b_rain = R4(0.8);
static const double a_snow = R4(4.84), b_snow = 0.25;
static const double a_grau = 94.5, b_grau = 0.5;
static const double qcw0 = R4(1.e-3), qci0 = R4(1.e-4);
static const double alphaelq = R4(1.e-3), betaelq = R4(1.e-3);
static const double erccoef = 1.0, esccoef = 1.0, esicoef = R4(0.1);
static const double egccoef = 1.0, egicoef = R4(0.1);
static const double nzeror = 8.e6, nzeros = 3.e6, nzerog = 4.e6;
static const double qp_threshold = R4(1.e-8);

static inline double fmax2(double a, double b) { return (b > a) ? b : a; }
static inline double fmin2(double a, double b) { return (b < a) ? b : a; }
static inline double fmax3(double a, double b, double c) { return fmax2(fmax2(a, b), c); }
static inline double fmin3(double a, double b, double c) { return fmin2(fmin2(a, b), c); }
// gammafff.c (crm/gammafff.c:12): the REAL*4 gamma function of the sam1mom
// set-up, exp of the C library's lgamma rounded to float
static float gammafff_r4(float x) { return (float)exp(lgamma((double)x)); }

// ---------------------------------------------------------------- sat.F90
// Flatau et al. (1992) polynomials; Murphy & Koop (2005) below -80 C.
static double esatw(double t) {            // sat.F90:12-31
  const double a0 = R4(6.105851), a1 = R4(0.4440316), a2 = R4(0.1430341e-1),
               a3 = R4(0.2641412e-3), a4 = R4(0.2995057e-5), a5 = R4(0.2031998e-7),
               a6 = R4(0.6936113e-10), a7 = R4(0.2564861e-13), a8 = R4(-0.3704404e-15);
  double dt = t - R4(273.16);
  if (dt > -80.)
    return a0 + dt * (a1 + dt * (a2 + dt * (a3 + dt * (a4 + dt * (a5 + dt * (a6 + dt * (a7 + a8 * dt)))))));
  return (double)(2.0f * 0.01f) *
         det_exp(((R4(9.550426) - R4(5723.265) / t) + R4(3.53068) * det_log(t)) - R4(0.00728332) * t);
}
static double qsatw(double t, double p) {  // sat.F90:35-45
  double es = esatw(t);
  return (R4(0.622) * es) / fmax2(es, p - es);
}
static double dtesatw(double t) {          // sat.F90:48-66
  const double a0 = R4(0.443956472), a1 = R4(0.285976452e-1), a2 = R4(0.794747212e-3),
               a3 = R4(0.121167162e-4), a4 = R4(0.103167413e-6), a5 = R4(0.385208005e-9),
               a6 = R4(-0.604119582e-12), a7 = R4(-0.792933209e-14), a8 = R4(-0.599634321e-17);
  double dt = t - R4(273.16);
  if (dt > -80.)
    return a0 + dt * (a1 + dt * (a2 + dt * (a3 + dt * (a4 + dt * (a5 + dt * (a6 + dt * (a7 + a8 * dt)))))));
  return esatw(t + 1.0) - esatw(t);
}
static double dtqsatw(double t, double p) { return (R4(0.622) * dtesatw(t)) / p; }
static double esati(double t) {            // sat.F90:79-97
  const double a0 = R4(6.11147274), a1 = R4(0.503160820), a2 = R4(0.188439774e-1),
               a3 = R4(0.420895665e-3), a4 = R4(0.615021634e-5), a5 = R4(0.602588177e-7),
               a6 = R4(0.385852041e-9), a7 = R4(0.146898966e-11), a8 = R4(0.252751365e-14);
  double dt = t - R4(273.16);
  if (dt > -80.)
    return a0 + dt * (a1 + dt * (a2 + dt * (a3 + dt * (a4 + dt * (a5 + dt * (a6 + dt * (a7 + a8 * dt)))))));
  return R4(0.01) *
         det_exp(((R4(9.550426) - R4(5723.265) / t) + R4(3.53068) * det_log(t)) - R4(0.00728332) * t);
}
static double qsati(double t, double p) {
  double es = esati(t);
  return (R4(0.622) * es) / fmax2(es, p - es);
}
static double dtesati(double t) {          // sat.F90:112-130
  const double a0 = R4(0.503223089), a1 = R4(0.377174432e-1), a2 = R4(0.126710138e-2),
               a3 = R4(0.249065913e-4), a4 = R4(0.312668753e-6), a5 = R4(0.255653718e-8),
               a6 = R4(0.132073448e-10), a7 = R4(0.390204672e-13), a8 = R4(0.497275778e-16);
  double dt = t - R4(273.16);
  if (dt > -80.)
    return a0 + dt * (a1 + dt * (a2 + dt * (a3 + dt * (a4 + dt * (a5 + dt * (a6 + dt * (a7 + a8 * dt)))))));
  return esati(t + 1.) - esati(t);
}
static double dtqsati(double t, double p) { return (R4(0.622) * dtesati(t)) / p; }

// ---------------------------------------------------------------- fft.F90
// fax_crm (fft.F90:181-246): factors of n/2 (mode 3), ascending.
static void fax(int *ifax, int n) {
  int nn = n / 2;
  if (nn + nn != n) { ifax[0] = -99; return; }
  int k = 0;
  while (nn % 4 == 0) { ifax[++k] = 4; nn /= 4; if (nn == 1) goto done; }
  if (nn % 2 == 0) { ifax[++k] = 2; nn /= 2; if (nn == 1) goto done; }
  while (nn % 3 == 0) { ifax[++k] = 3; nn /= 3; if (nn == 1) goto done; }
  {
    int l = 5, inc = 2;
    for (;;) {
      while (nn % l == 0) { ifax[++k] = l; nn /= l; if (nn == 1) goto done; }
      l += inc; inc = 6 - inc;
    }
  }
done:
  ifax[0] = k;
  for (int ii = 2; ii <= k; ++ii)
    for (int i = 1; i <= k + 1 - ii; ++i)
      if (ifax[i + 1] < ifax[i]) std::swap(ifax[i], ifax[i + 1]);
}
// fftrig_crm (fft.F90:247-300), mode 3.  pi, del and angle are REAL*4.
static void fftrig(std::vector<double> &trigs, int n) {
  trigs.assign(3 * n / 2 + 2 + n, 0.0);
  float pi_f = (float)(2.0f * asinf(1.0f));
  int nn = n / 2;
  float del = (float)((double)(pi_f + pi_f) / (double)nn);
  for (int i = 1; i <= nn + nn; i += 2) {
    float angle = (float)(0.5 * (double)(i - 1) * (double)del);
    trigs[i - 1] = (double)cosf(angle);
    trigs[i] = (double)sinf(angle);
  }
  del = 0.5f * del;
  int nh = (nn + 1) / 2, l = nh + nh, la = nn + nn;
  for (int i = 1; i <= l; i += 2) {
    float angle = (float)(0.5 * (double)(i - 1) * (double)del);
    trigs[la + i - 1] = (double)cosf(angle);
    trigs[la + i] = (double)sinf(angle);
  }
}

// One pass of the complex transform (vpassm_crm, fft.F90:466-806) with
// lot = 1.  A and C hold nh interleaved complex numbers.  The twiddles
// c1..s4 and the radix constants are REAL*4 values.
static void vpass(const double *A, double *C, const double *trigs, int nh, int ifac, int la) {
  const double sin36 = (double)(float)0.587785252292473, cos36 = (double)(float)0.809016994374947;
  const double sin72 = (double)(float)0.951056516295154, cos72 = (double)(float)0.309016994374947;
  const double sin60 = (double)(float)0.866025403784437;
  int m = nh / ifac;
  int ngroups = m / la;
  for (int g = 0; g < ngroups; ++g) {
    double c1 = 1, s1 = 0, c2 = 1, s2 = 0, c3 = 1, s3 = 0, c4 = 1, s4 = 0;
    int kb = 2 * g * la;
    if (g > 0) {
      c1 = trigs[kb]; s1 = trigs[kb + 1];
      c2 = trigs[2 * kb]; s2 = trigs[2 * kb + 1];
      if (ifac >= 4) { c3 = trigs[3 * kb]; s3 = trigs[3 * kb + 1]; }
      if (ifac >= 5) { c4 = trigs[4 * kb]; s4 = trigs[4 * kb + 1]; }
    }
    for (int l = 0; l < la; ++l) {
      int p = g * la + l, q = g * ifac * la + l;
#define AR(r) A[2 * (p + (r) * m)]
#define AI(r) A[2 * (p + (r) * m) + 1]
#define CR(r) C[2 * (q + (r) * la)]
#define CI(r) C[2 * (q + (r) * la) + 1]
      double a0 = AR(0), b0 = AI(0), a1 = AR(1), b1 = AI(1);
      if (ifac == 2) {
        CR(0) = a0 + a1; CI(0) = b0 + b1;
        if (g == 0) { CR(1) = a0 - a1; CI(1) = b0 - b1; }
        else {
          CR(1) = c1 * (a0 - a1) - s1 * (b0 - b1);
          CI(1) = s1 * (a0 - a1) + c1 * (b0 - b1);
        }
      } else if (ifac == 3) {
        double a2 = AR(2), b2 = AI(2);
        CR(0) = a0 + (a1 + a2); CI(0) = b0 + (b1 + b2);
        double xr = a0 - 0.5 * (a1 + a2), xi = b0 - 0.5 * (b1 + b2);
        double yr = sin60 * (b1 - b2), yi = sin60 * (a1 - a2);
        if (g == 0) {
          CR(1) = xr - yr; CR(2) = xr + yr; CI(1) = xi + yi; CI(2) = xi - yi;
        } else {
          CR(1) = c1 * (xr - yr) - s1 * (xi + yi);
          CI(1) = s1 * (xr - yr) + c1 * (xi + yi);
          CR(2) = c2 * (xr + yr) - s2 * (xi - yi);
          CI(2) = s2 * (xr + yr) + c2 * (xi - yi);
        }
      } else if (ifac == 4) {
        double a2 = AR(2), b2 = AI(2), a3 = AR(3), b3 = AI(3);
        if (g == 0) {
          CR(0) = (a0 + a2) + (a1 + a3); CR(2) = (a0 + a2) - (a1 + a3);
          CI(0) = (b0 + b2) + (b1 + b3); CI(2) = (b0 + b2) - (b1 + b3);
          CR(1) = (a0 - a2) - (b1 - b3); CR(3) = (a0 - a2) + (b1 - b3);
          CI(1) = (b0 - b2) + (a1 - a3); CI(3) = (b0 - b2) - (a1 - a3);
        } else {
          CR(0) = (a0 + a2) + (a1 + a3); CI(0) = (b0 + b2) + (b1 + b3);
          CR(2) = c2 * ((a0 + a2) - (a1 + a3)) - s2 * ((b0 + b2) - (b1 + b3));
          CI(2) = s2 * ((a0 + a2) - (a1 + a3)) + c2 * ((b0 + b2) - (b1 + b3));
          CR(1) = c1 * ((a0 - a2) - (b1 - b3)) - s1 * ((b0 - b2) + (a1 - a3));
          CI(1) = s1 * ((a0 - a2) - (b1 - b3)) + c1 * ((b0 - b2) + (a1 - a3));
          CR(3) = c3 * ((a0 - a2) + (b1 - b3)) - s3 * ((b0 - b2) - (a1 - a3));
          CI(3) = s3 * ((a0 - a2) + (b1 - b3)) + c3 * ((b0 - b2) - (a1 - a3));
        }
      } else {  // 5
        double a2 = AR(2), b2 = AI(2), a3 = AR(3), b3 = AI(3), a4 = AR(4), b4 = AI(4);
        CR(0) = (a0 + (a1 + a4)) + (a2 + a3);
        CI(0) = (b0 + (b1 + b4)) + (b2 + b3);
        double p1r = (a0 + cos72 * (a1 + a4)) - cos36 * (a2 + a3);
        double q1r = sin72 * (b1 - b4) + sin36 * (b2 - b3);
        double p1i = (b0 + cos72 * (b1 + b4)) - cos36 * (b2 + b3);
        double q1i = sin72 * (a1 - a4) + sin36 * (a2 - a3);
        double p2r = (a0 - cos36 * (a1 + a4)) + cos72 * (a2 + a3);
        double q2r = sin36 * (b1 - b4) - sin72 * (b2 - b3);
        double p2i = (b0 - cos36 * (b1 + b4)) + cos72 * (b2 + b3);
        double q2i = sin36 * (a1 - a4) - sin72 * (a2 - a3);
        if (g == 0) {
          CR(1) = p1r - q1r; CR(4) = p1r + q1r; CI(1) = p1i + q1i; CI(4) = p1i - q1i;
          CR(2) = p2r - q2r; CR(3) = p2r + q2r; CI(2) = p2i + q2i; CI(3) = p2i - q2i;
        } else {
          CR(1) = c1 * (p1r - q1r) - s1 * (p1i + q1i);
          CI(1) = s1 * (p1r - q1r) + c1 * (p1i + q1i);
          CR(4) = c4 * (p1r + q1r) - s4 * (p1i - q1i);
          CI(4) = s4 * (p1r + q1r) + c4 * (p1i - q1i);
          CR(2) = c2 * (p2r - q2r) - s2 * (p2i + q2i);
          CI(2) = s2 * (p2r - q2r) + c2 * (p2i + q2i);
          CR(3) = c3 * (p2r + q2r) - s3 * (p2i - q2i);
          CI(3) = s3 * (p2r + q2r) + c3 * (p2i - q2i);
        }
      }
#undef AR
#undef AI
#undef CR
#undef CI
    }
  }
}

// fft991_crm (fft.F90:5-154) for one vector a[0..n+1] (lot = 1, inc = 1).
// isign = -1: grid point -> spectral; +1: spectral -> grid point.
static void fft991(double *a, double *work, const double *trigs, const int *ifax, int n, int isign) {
  int nfax = ifax[0], nh = n / 2;
  bool in_work;          // where the current data lives
  if (isign == -1) {
    if (nfax % 2 == 1) in_work = false;
    else { for (int m = 0; m < n; ++m) work[m] = a[m]; in_work = true; }
  } else {
    // fft99a_crm (fft.F90:301-381): a -> work
    work[0] = a[0] + a[n];
    work[1] = a[0] - a[n];
    int ia = 2, ib = n - 2;
    for (int k = 3; k <= nh; k += 2) {
      double c = trigs[n + k - 1], s = trigs[n + k];
      double ap = a[ia] + a[ib], am = a[ia] - a[ib];
      double bp = a[ia + 1] + a[ib + 1], bm = a[ia + 1] - a[ib + 1];
      work[ia] = ap - (s * am + c * bp);
      work[ib] = ap + (s * am + c * bp);
      work[ia + 1] = (c * am - s * bp) + bm;
      work[ib + 1] = (c * am - s * bp) - bm;
      ia += 2; ib -= 2;
    }
    if (ia == ib) { work[ia] = 2.0 * a[ia]; work[ia + 1] = -2.0 * a[ia + 1]; }
    in_work = true;
  }
  int la = 1;
  for (int k = 1; k <= nfax; ++k) {
    if (in_work) vpass(work, a, trigs, nh, ifax[k], la);
    else vpass(a, work, trigs, nh, ifax[k], la);
    in_work = !in_work;
    la *= ifax[k];
  }
  if (isign == -1) {
    // fft99b_crm (fft.F90:382-465): work -> a
    float scale = (float)(1.0 / (double)n);
    a[0] = (double)scale * (work[0] + work[1]);
    a[n] = (double)scale * (work[0] - work[1]);
    a[1] = 0.0;
    a[n + 1] = 0.0;
    scale = 0.5f * scale;
    double sc = (double)scale;
    int ia = 2, ib = n - 2;
    for (int k = 3; k <= nh; k += 2) {
      double c = trigs[n + k - 1], s = trigs[n + k];
      double wp = work[ia] + work[ib], wm = work[ia] - work[ib];
      double vp = work[ia + 1] + work[ib + 1], vm = work[ib + 1] - work[ia + 1];
      a[ia] = sc * (wp + (c * vp + s * wm));
      a[ib] = sc * (wp - (c * vp + s * wm));
      a[ia + 1] = sc * ((c * wm - s * vp) + vm);
      a[ib + 1] = sc * ((c * wm - s * vp) - vm);
      ia += 2; ib -= 2;
    }
    if (ia == ib) {
      scale = 2.0f * scale;
      a[ia] = (double)scale * work[ia];
      a[ia + 1] = -(double)scale * work[ia + 1];
    }
  } else {
    if (in_work) for (int m = 0; m < n; ++m) a[m] = work[m];
    a[n] = 0.0;
    a[n + 1] = 0.0;
  }
}

// ---------------------------------------------------------------- model
// ---------------------------------------------------------------- RNG_MT.F90
// cam/RNG_MT.F90:52-142: a Mersenne-Twister variant.  The seeding is the old
// 69069 linear congruential fill (RNG_MT_set_seed :52-63), the upper mask is
// -1147483648 (0xBB9ACA00, not 0x80000000; :13), and the draw maps a
// negative (signed) tempered word y to (y + 2^32) / 2^32 and a non-negative
// one to (y + 0.5) / 2^32 (:133-137).
struct RngMT {
  int32_t mt[624];
  int mti;
  explicit RngMT(int seed) {
    mt[0] = (int32_t)seed;
    for (mti = 1; mti < 624; ++mti) mt[mti] = (int32_t)((uint32_t)69069 * (uint32_t)mt[mti - 1]);
  }
  double gen() {
    const int32_t UMASK = -1147483648, LMASK = 2147483647;
    const int32_t MATA = -1727483681, TMASKB = -1658038656, TMASKC = -272236544;
    int32_t y;
    if (mti >= 624) {
      int kk;
      for (kk = 0; kk < 624 - 397; ++kk) {
        y = (mt[kk] & UMASK) | (mt[kk + 1] & LMASK);
        mt[kk] = mt[kk + 397] ^ (int32_t)((uint32_t)y >> 1) ^ ((y & 1) ? MATA : 0);
      }
      for (; kk < 623; ++kk) {
        y = (mt[kk] & UMASK) | (mt[kk + 1] & LMASK);
        mt[kk] = mt[kk + (397 - 624)] ^ (int32_t)((uint32_t)y >> 1) ^ ((y & 1) ? MATA : 0);
      }
      y = (mt[623] & UMASK) | (mt[0] & LMASK);
      mt[623] = mt[396] ^ (int32_t)((uint32_t)y >> 1) ^ ((y & 1) ? MATA : 0);
      mti = 0;
    }
    y = mt[mti++];
    y ^= (int32_t)((uint32_t)y >> 11);
    y ^= (int32_t)(((uint32_t)y << 7) & (uint32_t)TMASKB);
    y ^= (int32_t)(((uint32_t)y << 15) & (uint32_t)TMASKC);
    y ^= (int32_t)((uint32_t)y >> 18);
    if (y < 0) return ((double)y + 4294967296.0) / 4294967296.0;
    return ((double)y + 0.5) / 4294967296.0;
  }
};

struct Model {
  Grid g;
  std::vector<Column> cols;
  const crm_call_desc *desc;
  const crm_input_c *in;
  int ld;
  std::vector<int> col_status_saved;

  double IN(const double *a, int icrm, int l) const {  // (ld, *) array, l 1-based
    return a[(size_t)icrm + (size_t)ld * (l - 1)];
  }

  // ---- allocation (vars.F90:200-574, grid.F90:170-203, sgs.F90:50-80,
  //      microphysics.F90:52-88, micro_params.F90:90-125): everything zero
  void alloc_column(Column &c) {
    const int nx = g.nx, ny = g.ny, nzm = g.nzm, nz = g.nz, Y = g.YES3D;
    c.u.init(-1, nx + 3, 1 - 2 * Y, ny + 2 * Y, 1, nzm);
    c.v.init(-1, nx + 2, 1 - 2 * Y, ny + 3 * Y, 1, nzm);
    c.w.init(-1, nx + 2, 1 - 2 * Y, ny + 2 * Y, 1, nz);
    c.t.init(-2, nx + 3, 1 - 3 * Y, ny + 3 * Y, 1, nzm);
    c.qt.init(-2, nx + 3, 1 - 3 * Y, ny + 3 * Y, 1, nzm);
    c.qp.init(-2, nx + 3, 1 - 3 * Y, ny + 3 * Y, 1, nzm);
    c.tke.init(-2, nx + 3, 1 - 3 * Y, ny + 3 * Y, 1, nzm);
    c.p.init(0, nx, 1 - Y, ny, 1, nzm);
    for (A3 *a : {&c.tabs, &c.qv, &c.qcl, &c.qpl, &c.qci, &c.qpi, &c.qn}) a->init(1, nx, 1, ny, 1, nzm);
    c.tk.init(0, nx + 1, 1 - Y, ny + Y, 1, nzm);
    c.tkh.init(0, nx + 1, 1 - Y, ny + Y, 1, nzm);
    for (int l = 0; l < 3; ++l) {
      c.dudt[l].init(1, nx + 1, 1, ny, 1, nzm);
      c.dvdt[l].init(1, nx, 1, ny + Y, 1, nzm);
      c.dwdt[l].init(1, nx, 1, ny, 1, nz);
    }
    c.precsfc.init(1, nx, 1, ny, 1, 1);
    c.precssfc.init(1, nx, 1, ny, 1, 1);
    for (A1 *a : {&c.z, &c.zi, &c.presi, &c.adzw, &c.rhow}) a->init(1, nz);
    for (A1 *a : {&c.pres, &c.adz, &c.prespot, &c.rho, &c.bet, &c.gamaz, &c.t0, &c.q0, &c.qv0,
                  &c.tabs0, &c.u0, &c.v0, &c.tke0, &c.qp0, &c.qn0, &c.t00, &c.ttend, &c.qtend,
                  &c.utend, &c.vtend, &c.ug0, &c.vg0, &c.tg0, &c.qg0, &c.grdf_x, &c.grdf_y,
                  &c.grdf_z, &c.accrsc, &c.accrsi, &c.accrrc, &c.coefice, &c.accrgc, &c.accrgi,
                  &c.evaps1, &c.evaps2, &c.evapr1, &c.evapr2, &c.evapg1, &c.evapg2})
      a->init(1, nzm);
    for (A1 *a : {&c.uwle, &c.vwle, &c.uwsb, &c.vwsb, &c.precflux, &c.qpfall, &c.tlat, &c.tlatqi,
                  &c.qifall, &c.mkwle[0], &c.mkwle[1], &c.mkwsb[0], &c.mkwsb[1], &c.mkadv[0],
                  &c.mkadv[1], &c.mkdiff[0], &c.mkdiff[1], &c.qpsrc, &c.qpevp})
      a->init(1, nz);
    for (A1 *a : {&c.o_cld, &c.o_cldtop, &c.o_gicewp, &c.o_gliqwp, &c.o_mcup, &c.o_mcdn,
                  &c.o_mcuup, &c.o_mcudn})
      a->init(1, g.plev);
    c.mui.init(1, g.plev + 1);
    c.mdi.init(1, g.plev + 1);
    for (A3 *a : {&c.rad_t, &c.rad_qv, &c.rad_qc, &c.rad_qi, &c.rad_cld, &c.qrad})
      a->init(1, g.nx_rad, 1, g.ny_rad, 1, nzm);
    for (std::vector<double> *a : {&c.st_cwp, &c.st_cwph, &c.st_cwpm, &c.st_cwpl, &c.st_ct,
                                   &c.st_ch, &c.st_cm, &c.st_cl})
      a->assign((size_t)nx * ny, 0.0);
    c.cltot = c.clhgh = c.clmed = c.cllow = 0;
    c.na = 1; c.nb = 2; c.nc = 3;      // grid.F90:191-193
    c.dt3[0] = c.dt3[1] = c.dt3[2] = 0.0;
    c.at = c.bt = c.ct = 0;
    c.status = CRM_OK;
    c.z0 = R4(0.035);                  // params.F90:160
  }
  A3 &DU(Column &c, int l) { return c.dudt[l - 1]; }
  A3 &DV(Column &c, int l) { return c.dvdt[l - 1]; }
  A3 &DW(Column &c, int l) { return c.dwdt[l - 1]; }

  // ---- bound_exchange.F90:14-239 / periodic.F90: periodic halos.  Every
  // halo value is copied from the interior (x first, then y with the x
  // halos and corners in 3D), so the result is the periodic wrap of the
  // interior onto i in [1-i_1, nx+i_2], j in [1-j_1, ny+j_2] (3D only).
  void exch(A3 &f, int dimz, int i_1, int i_2, int j_1 = 1, int j_2 = 1) {
    const int nx = g.nx, ny = g.ny;
    int i1 = i_1 - 1, i2 = i_2 - 1;
    if (!g.YES3D) {
      for (int k = 1; k <= dimz; ++k) {
        for (int i = -i1; i <= 0; ++i) f(i, 1, k) = f(i + nx, 1, k);
        for (int i = nx + 1; i <= nx + 1 + i2; ++i) f(i, 1, k) = f(i - nx, 1, k);
      }
      return;
    }
    int j1 = j_1 - 1, j2 = j_2 - 1;
    auto wrap = [](int a, int n) { return a < 1 ? a + n : (a > n ? a - n : a); };
    for (int k = 1; k <= dimz; ++k)
      for (int j = -j1; j <= ny + 1 + j2; ++j)
        for (int i = -i1; i <= nx + 1 + i2; ++i) {
          if (i >= 1 && i <= nx && j >= 1 && j <= ny) continue;
          f(i, j, k) = f(wrap(i, nx), wrap(j, ny), k);
        }
  }
  void boundaries(Column &c, int flag) {   // periodic.F90:8-136
    const int nzm = g.nzm, nz = g.nz;
    if (flag == 0) {
      exch(c.u, nzm, 1, 1, 1, 1);
      exch(c.v, nzm, 1, 1, 1, 1);
      // w(:,:,nz) carries the (zero) sstxy through the exchange, then is zeroed
      for (int j = 1; j <= g.ny; ++j)
        for (int i = 1; i <= g.nx; ++i) c.w(i, j, nz) = 0.0;
      exch(c.w, nz, 1, 1, 1, 1);
      for (int j = 1 - g.YES3D; j <= g.ny + g.YES3D; ++j)
        for (int i = 0; i <= g.nx + 1; ++i) c.w(i, j, nz) = 0.0;
    } else if (flag == 2) {
      exch(c.u, nzm, 2, 3, 2, 2);
      exch(c.v, nzm, 2, 2, 2, 3);
      exch(c.w, nz, 2, 2, 2, 2);
      exch(c.t, nzm, 3, 3, 3, 3);
      exch(c.qt, nzm, 3, 3, 3, 3);
      exch(c.qp, nzm, 3, 3, 3, 3);
    } else if (flag == 3) {
      exch(c.t, nzm, 1, 1, 1, 1);
      exch(c.qt, nzm, 1, 1, 1, 1);
      exch(c.qp, nzm, 1, 1, 1, 1);
    } else if (flag == 4) {
      exch(c.tk, nzm, 1, 1, 1, 1);
      exch(c.tkh, nzm, 1, 1, 1, 1);
    }
  }

  // ---- grid setup from crm_input (crm_module.F90:320-375)
  void setup_grid(Column &c, int icrm) {
    const int nzm = g.nzm, nz = g.nz, plev = g.plev;
    for (int k = 1; k <= nzm; ++k) {
      c.z(k) = IN(in->zmid, icrm, plev - k + 1) - IN(in->zint, icrm, plev + 1);
      c.zi(k) = IN(in->zint, icrm, plev - k + 2) - IN(in->zint, icrm, plev + 1);
      c.pres(k) = IN(in->pmid, icrm, plev - k + 1) / 100.;
      c.presi(k) = IN(in->pint, icrm, plev - k + 2) / 100.;
      c.prespot(k) = det_pow(1000. / c.pres(k), rgas / cp);
      c.bet(k) = ggr / IN(in->tl, icrm, plev - k + 1);
      c.gamaz(k) = ggr / cp * c.z(k);
    }
    c.zi(nz) = IN(in->zint, icrm, plev - nz + 2) - IN(in->zint, icrm, plev + 1);
    c.presi(nz) = IN(in->pint, icrm, plev - nz + 2) / 100.;
    c.dz = 0.5 * (c.z(1) + c.z(2));
    for (int k = 2; k <= nzm; ++k) c.adzw(k) = (c.z(k) - c.z(k - 1)) / c.dz;
    c.adzw(1) = 1.;
    c.adzw(nz) = c.adzw(nzm);
    for (int k = 1; k <= nzm; ++k) c.adz(k) = (c.zi(k + 1) - c.zi(k)) / c.dz;
    for (int k = 1; k <= nzm; ++k) c.rho(k) = IN(in->pdel, icrm, plev - k + 1) / ggr / (c.adz(k) * c.dz);
    for (int k = 2; k <= nzm; ++k)
      c.rhow(k) = (IN(in->pmid, icrm, plev - k + 2) - IN(in->pmid, icrm, plev - k + 1)) / ggr / (c.adzw(k) * c.dz);
    c.rhow(1) = 2. * c.rhow(2) - c.rhow(3);
    c.rhow(nz) = 2. * c.rhow(nzm) - c.rhow(nzm - 1);
  }

  // ---- micro_diagnose (MICRO_SAM1MOM/microphysics.F90:334-357)
  void micro_diagnose(Column &c) {
    for (int k = 1; k <= g.nzm; ++k)
      for (int j = 1; j <= g.ny; ++j)
        for (int i = 1; i <= g.nx; ++i) {
          c.qv(i, j, k) = c.qt(i, j, k) - c.qn(i, j, k);
          double omn = fmax2(0., fmin2(1., (c.tabs(i, j, k) - tbgmin) * g.a_bg));
          c.qcl(i, j, k) = c.qn(i, j, k) * omn;
          c.qci(i, j, k) = c.qn(i, j, k) * (1. - omn);
          double omp = fmax2(0., fmin2(1., (c.tabs(i, j, k) - tprmin) * g.a_pr));
          c.qpl(i, j, k) = c.qp(i, j, k) * omp;
          c.qpi(i, j, k) = c.qp(i, j, k) * (1. - omp);
        }
  }

  // ---- precip_init (MICRO_SAM1MOM/precip_init.F90:8-94)
  void precip_init(Column &c) {
    for (int k = 1; k <= g.nzm; ++k) {
      double rho = c.rho(k), t0 = c.tabs0(k);
      double pratio = sqrt(R4(1.29) / rho);
      double rrr1 = 393. / (t0 + 120.) * det_pow(t0 / 273., 1.5);
      double rrr2 = det_pow(t0 / 273., R4(1.94)) * (1000. / c.pres(k));
      double estw = 100. * esatw(t0);
      double esti = 100. * esati(t0);
      double coef1 = 0.25 * pi * nzeros * a_snow * g.gams1 * pratio /
                     det_pow(pi * rhos * nzeros / rho, (3 + b_snow) / 4.);
      double coef2 = det_exp(R4(0.025) * (t0 - R4(273.15)));
      c.accrsi(k) = coef1 * coef2 * esicoef;
      c.accrsc(k) = coef1 * esccoef;
      c.coefice(k) = coef2;
      coef1 = (lsub / (t0 * rv) - 1.) * lsub / (therco * rrr1 * t0);
      coef2 = rv * t0 / (diffelq * rrr2 * esti);
      c.evaps1(k) = (double)(0.65f * 4.f) * nzeros / sqrt(pi * rhos * nzeros) / (coef1 + coef2) / sqrt(rho);
      c.evaps2(k) = (double)(0.49f * 4.f) * nzeros * g.gams2 * sqrt(a_snow / (muelq * rrr1)) /
                    det_pow(pi * rhos * nzeros, (5 + b_snow) / 8.) / (coef1 + coef2) *
                    det_pow(rho, (1 + b_snow) / 8.) * sqrt(pratio);
      coef1 = 0.25 * pi * nzerog * a_grau * g.gamg1 * pratio /
              det_pow(pi * rhog * nzerog / rho, (3 + b_grau) / 4.);
      coef2 = det_exp(R4(0.025) * (t0 - R4(273.15)));
      c.accrgi(k) = coef1 * coef2 * egicoef;
      c.accrgc(k) = coef1 * egccoef;
      coef1 = (lsub / (t0 * rv) - 1.) * lsub / (therco * rrr1 * t0);
      coef2 = rv * t0 / (diffelq * rrr2 * esti);
      c.evapg1(k) = (double)(0.65f * 4.f) * nzerog / sqrt(pi * rhog * nzerog) / (coef1 + coef2) / sqrt(rho);
      c.evapg2(k) = (double)(0.49f * 4.f) * nzerog * g.gamg2 * sqrt(a_grau / (muelq * rrr1)) /
                    det_pow(pi * rhog * nzerog, (5 + b_grau) / 8.) / (coef1 + coef2) *
                    det_pow(rho, (1 + b_grau) / 8.) * sqrt(pratio);
      c.accrrc(k) = 0.25 * pi * nzeror * a_rain * g.gamr1 * pratio /
                    det_pow(pi * rhor * nzeror / rho, (3 + b_rain) / 4.) * erccoef;
      coef1 = (lcond / (t0 * rv) - 1.) * lcond / (therco * rrr1 * t0);
      coef2 = rv * t0 / (diffelq * rrr2 * estw);
      c.evapr1(k) = (double)(0.78f * 2.f) * pi * nzeror / sqrt(pi * rhor * nzeror) / (coef1 + coef2) / sqrt(rho);
      c.evapr2(k) = (double)(0.31f * 2.f) * pi * nzeror * g.gamr2 * R4(0.89) * sqrt(a_rain / (muelq * rrr1)) /
                    det_pow(pi * rhor * nzeror, (5 + b_rain) / 8.) / (coef1 + coef2) *
                    det_pow(rho, (1 + b_rain) / 8.) * sqrt(pratio);
    }
  }

  // ---- crm_module.F90:380-681: state in, initial means, nudging, setperturb
  void init_column(Column &c, int icrm, const crm_state_c *st, const crm_rad_c *rad, bool clamp) {
    const int nx = g.nx, ny = g.ny, nzm = g.nzm, Y = g.YES3D;
    auto S = [&](const double *a, int i, int j, int k) {
      return a[(size_t)icrm + (size_t)ld * ((i - 1) + (size_t)nx * ((j - 1) + (size_t)ny * (k - 1)))];
    };
    setup_grid(c, icrm);
    c.nstop = g.nstop;
    c.nstep = 0;
    c.ceaseflag = false;
    c.bflx = in->bflxls[icrm];
    c.wnd = in->wndls[icrm];
    for (int k = 1; k <= nzm; ++k)
      for (int j = 1; j <= ny; ++j)
        for (int i = 1; i <= nx; ++i) {
          c.u(i, j, k) = S(st->u_wind, i, j, k);
          c.v(i, j, k) = S(st->v_wind, i, j, k) * (double)Y;
          c.w(i, j, k) = S(st->w_wind, i, j, k);
          c.tabs(i, j, k) = S(st->temperature, i, j, k);
        }
    for (int k = 1; k <= nzm; ++k)
      for (int j = 1; j <= g.ny_rad; ++j)
        for (int i = 1; i <= g.nx_rad; ++i)
          c.qrad(i, j, k) = rad->qrad[(size_t)icrm + (size_t)ld * ((i - 1) + (size_t)g.nx_rad * ((j - 1) + (size_t)g.ny_rad * (k - 1)))];
    const double umax = (double)(0.5f * (float)g.dx / (float)g.dt);
    if (clamp) {
      for (int k = 1; k <= nzm; ++k)
        for (int j = 1; j <= ny; ++j)
          for (int i = 1; i <= nx; ++i) {
            c.u(i, j, k) = fmin2(umax, fmax2(-umax, c.u(i, j, k)));
            c.v(i, j, k) = fmin2(umax, fmax2(-umax, c.v(i, j, k))) * (double)Y;
          }
    }
    for (int k = 1; k <= nzm; ++k)
      for (int j = 1; j <= ny; ++j)
        for (int i = 1; i <= nx; ++i) {
          c.qt(i, j, k) = S(st->qt, i, j, k);
          c.qp(i, j, k) = S(st->qp, i, j, k);
          c.qn(i, j, k) = S(st->qn, i, j, k);
        }
    // micro_init (microphysics.F90:140-200): diagnose only
    micro_diagnose(c);
    // sgs_init (sgs.F90:174-230): LES = .false.
    for (int k = 1; k <= nzm; ++k) {
      double adzdz = c.adz(k) * c.dz;
      c.grdf_x(k) = fmin2(16., g.dx * g.dx / (adzdz * adzdz));
      c.grdf_y(k) = fmin2(16., g.dy * g.dy / (adzdz * adzdz));
      c.grdf_z(k) = 1.;
    }
    c.colprec = 0; c.colprecs = 0;
    for (int k = 1; k <= nzm; ++k) {
      c.u0(k) = c.v0(k) = c.t0(k) = c.t00(k) = c.tabs0(k) = c.q0(k) = c.qv0(k) = 0;
      c.qn0(k) = c.qp0(k) = c.tke0(k) = 0;
    }
    for (int k = 1; k <= nzm; ++k) {
      double pdel = IN(in->pdel, icrm, g.plev - k + 1);
      for (int j = 1; j <= ny; ++j)
        for (int i = 1; i <= nx; ++i) {
          c.t(i, j, k) = c.tabs(i, j, k) + c.gamaz(k) - fac_cond * c.qcl(i, j, k) - fac_sub * c.qci(i, j, k) -
                         fac_cond * c.qpl(i, j, k) - fac_sub * c.qpi(i, j, k);
          c.colprec = c.colprec + (c.qpl(i, j, k) + c.qpi(i, j, k)) * pdel;
          c.colprecs = c.colprecs + c.qpi(i, j, k) * pdel;
          c.u0(k) += c.u(i, j, k);
          c.v0(k) += c.v(i, j, k);
          c.t0(k) += c.t(i, j, k);
          c.t00(k) += c.t(i, j, k) + fac_cond * c.qpl(i, j, k) + fac_sub * c.qpi(i, j, k);
          c.tabs0(k) += c.tabs(i, j, k);
          c.q0(k) += c.qv(i, j, k) + c.qcl(i, j, k) + c.qci(i, j, k);
          c.qv0(k) += c.qv(i, j, k);
          c.qn0(k) += c.qcl(i, j, k) + c.qci(i, j, k);
          c.qp0(k) += c.qpl(i, j, k) + c.qpi(i, j, k);
          c.tke0(k) += c.tke(i, j, k);
        }
    }
    const double factor_xy = 1.0 / (double)(nx * ny);
    const double idt_gl = 1.0 / desc->dt_gl;
    for (int k = 1; k <= nzm; ++k) {
      c.u0(k) *= factor_xy; c.v0(k) *= factor_xy; c.t0(k) *= factor_xy; c.t00(k) *= factor_xy;
      c.tabs0(k) *= factor_xy; c.q0(k) *= factor_xy; c.qv0(k) *= factor_xy; c.qn0(k) *= factor_xy;
      c.qp0(k) *= factor_xy; c.tke0(k) *= factor_xy;
      int l = g.plev - k + 1;
      double uln = fmin2(umax, fmax2(-umax, IN(in->ul, icrm, l)));
      double vln = fmin2(umax, fmax2(-umax, IN(in->vl, icrm, l))) * (double)Y;
      double tl = IN(in->tl, icrm, l), qccl = IN(in->qccl, icrm, l), qiil = IN(in->qiil, icrm, l);
      double ql = IN(in->ql, icrm, l);
      c.ttend(k) = (tl + c.gamaz(k) - fac_cond * (qccl + qiil) - fac_fus * qiil - c.t00(k)) * idt_gl;
      c.qtend(k) = (ql + qccl + qiil - c.q0(k)) * idt_gl;
      c.utend(k) = (uln - c.u0(k)) * idt_gl;
      c.vtend(k) = (vln - c.v0(k)) * idt_gl;
      c.ug0(k) = uln;
      c.vg0(k) = vln;
      c.tg0(k) = tl + c.gamaz(k) - fac_cond * qccl - fac_sub * qiil;
      c.qg0(k) = ql + qccl + qiil;
    }
    // roughness length (crm_module.F90:583-594, crmsurface.F90:104-133)
    c.ustar = sqrt(in->tau00[icrm] / c.rho(1));
    {
      const double vonk = R4(0.4), am = R4(4.8), bm = R4(19.3), eps = R4(1.e-10);
      double z = c.z(1), bflx = c.bflx, wnd = c.wnd, ustar = c.ustar;
      double c1 = (double)(3.14159f / 2.f - 3.f * logf(2.f));
      double rlmo = -bflx * vonk / (ustar * ustar * ustar + eps);
      double zeta = fmin2(1., z * rlmo);
      double psi1;
      if (zeta >= 0.) psi1 = -am * zeta;
      else {
        double x = sqrt(sqrt(1.0 - bm * zeta));
        psi1 = 2. * det_log(1.0 + x) + det_log(1.0 + x * x) - 2. * det_atan(x) + c1;
      }
      double lnz = fmax2(0., vonk * wnd / (ustar + eps) + psi1);
      c.z0 = z * det_exp(-lnz);
      c.z0 = fmax2(R4(0.00001), fmin2(1., c.z0));
    }
    precip_init(c);
  }

  // setperturb (crm/setperturb.F90:7-84) with RNG_MT (cam/RNG_MT.F90:52-142)
  void setperturb(Column &c, int iseed) {
    const int nx = g.nx, ny = g.ny;
    RngMT rng(iseed);
    auto gen = [&]() -> double { return rng.gen(); };
    const double factor_xy = 1. / (double)(nx * ny);
    for (int k = 1; k <= 5; ++k) {
      double perturb_k_scaling = (double)(5 + 1 - k) / (double)5;
      double t02 = 0.0;
      for (int j = 1; j <= ny; ++j)
        for (int i = 1; i <= nx; ++i) {
          double r = gen();
          r = 1. - 2. * r;
          c.t(i, j, k) = c.t(i, j, k) + 1.0 * r * perturb_k_scaling;
          t02 = t02 + c.t(i, j, k) * factor_xy;
        }
      for (int j = 1; j <= ny; ++j)
        for (int i = 1; i <= nx; ++i) c.t(i, j, k) = c.t(i, j, k) * c.t0(k) / t02;
    }
  }

  // ---- kurant (kurant.F90:9-83) + kurant_sgs (sgs.F90:329-372)
  void kurant(Column &c) {
    const int nx = g.nx, ny = g.ny, nzm = g.nzm, Y = g.YES3D;
    std::vector<double> wm(nzm + 2, 0.0), uhm(nzm + 2, 0.0);
    bool bad = false;     // no counterpart in the reference (it has no finiteness check)
    for (int k = 1; k <= nzm; ++k)
      for (int j = 1; j <= ny; ++j)
        for (int i = 1; i <= nx; ++i) {
          bad = bad || !std::isfinite(c.w(i, j, k)) || !std::isfinite(c.u(i, j, k)) ||
                !std::isfinite(c.tkh(i, j, k)) || (Y && !std::isfinite(c.v(i, j, k)));
          wm[k] = fmax2(wm[k], fabs(c.w(i, j, k)));
          double uu = c.u(i, j, k), vv = c.v(i, j, k);
          uhm[k] = fmax2(uhm[k], sqrt(uu * uu + (double)Y * (vv * vv)));
        }
    double cfl = 0.;
    const double rdx = 1. / g.dx, rdy = 1. / g.dy;
    for (int k = 1; k <= nzm; ++k) {
      double tmp = fmax2(uhm[k] * g.dt * sqrt(rdx * rdx + (double)Y * (rdy * rdy)),
                         fmax2(wm[k], wm[k + 1]) * g.dt / (c.dz * c.adzw(k)));
      cfl = fmax2(cfl, tmp);
    }
    for (int k = 1; k <= nzm; ++k) {
      double tkhmax = 0.;
      for (int j = 1; j <= ny; ++j)
        for (int i = 1; i <= nx; ++i) tkhmax = fmax2(tkhmax, c.tkh(i, j, k));
      double dza = c.dz * c.adzw(k);
      double tmp = fmax3(0.5 * tkhmax * c.grdf_z(k) * g.dt / (dza * dza),
                         0.5 * tkhmax * c.grdf_x(k) * g.dt / (g.dx * g.dx),
                         (double)((float)Y * 0.5f) * tkhmax * c.grdf_y(k) * g.dt / (g.dy * g.dy));
      cfl = fmax2(cfl, tmp);
    }
    // a column whose state is not finite stops here with CRM_ERR_NONFINITE;
    // its CFL is unbounded, so a reference batch stops with it
    c.nonfinite = bad;
    c.cfl = bad ? 1.0e300 : cfl;
  }
  static int ncycle_of(double cfl) {
    double n = std::ceil(cfl / R4(0.7));
    if (!(n < 1.0e6)) return 1000000;
    return std::max(1, (int)n);
  }

  // ---- abcoefs.F90:7-31
  void abcoefs(Column &c, int nstep) {
    if (nstep >= 3) {
      double alpha = c.dt3[c.nb - 1] / c.dt3[c.na - 1];
      double beta = c.dt3[c.nc - 1] / c.dt3[c.na - 1];
      c.ct = (2. + 3. * alpha) / (6. * (alpha + beta) * beta);
      c.bt = -(1. + 2. * (alpha + beta) * c.ct) / (2. * alpha);
      c.at = 1. - c.bt - c.ct;
    } else if (nstep >= 2) {
      c.at = 3. / 2.; c.bt = -1. / 2.; c.ct = 0.;
    } else {
      c.at = 1.; c.bt = 0.; c.ct = 0.;
    }
  }

  // ---- zero.F90:17-29
  void zero(Column &c) {
    DU(c, c.na).zero(); DV(c, c.na).zero(); DW(c, c.na).zero();
  }

  // ---- buoyancy.F90:15-37
  void buoyancy(Column &c) {
    A3 &dwdt = DW(c, c.na);
    for (int k = 2; k <= g.nzm; ++k)
      for (int j = 1; j <= g.ny; ++j)
        for (int i = 1; i <= g.nx; ++i) {
          int kb = k - 1;
          double betu = c.adz(kb) / (c.adz(k) + c.adz(kb));
          double betd = c.adz(k) / (c.adz(k) + c.adz(kb));
          dwdt(i, j, k) = dwdt(i, j, k) +
              c.bet(k) * betu *
                  (c.tabs0(k) * (epsv * (c.qv(i, j, k) - c.qv0(k)) -
                                 (c.qcl(i, j, k) + c.qci(i, j, k) - c.qn0(k) + c.qpl(i, j, k) + c.qpi(i, j, k) - c.qp0(k))) +
                   (c.tabs(i, j, k) - c.tabs0(k)) * (1. + epsv * c.qv0(k) - c.qn0(k) - c.qp0(k))) +
              c.bet(kb) * betd *
                  (c.tabs0(kb) * (epsv * (c.qv(i, j, kb) - c.qv0(kb)) -
                                  (c.qcl(i, j, kb) + c.qci(i, j, kb) - c.qn0(kb) + c.qpl(i, j, kb) + c.qpi(i, j, kb) - c.qp0(kb))) +
                   (c.tabs(i, j, kb) - c.tabs0(kb)) * (1. + epsv * c.qv0(kb) - c.qn0(kb) - c.qp0(kb)));
        }
  }

  // ---- forcing.F90:7-79
  void forcing(Column &c) {
    const int nzm = g.nzm;
    std::vector<double> qneg(nzm + 1, 0.), qpoz(nzm + 1, 0.);
    std::vector<int> nneg(nzm + 1, 0);
    A3 &dudt = DU(c, c.na), &dvdt = DV(c, c.na);
    for (int k = 1; k <= nzm; ++k)
      for (int j = 1; j <= g.ny; ++j)
        for (int i = 1; i <= g.nx; ++i) {
          c.t(i, j, k) = c.t(i, j, k) + c.ttend(k) * c.dtn;
          c.qt(i, j, k) = c.qt(i, j, k) + c.qtend(k) * c.dtn;
          if (c.qt(i, j, k) < 0.) { nneg[k] += 1; qneg[k] = qneg[k] + c.qt(i, j, k); }
          else qpoz[k] = qpoz[k] + c.qt(i, j, k);
          dudt(i, j, k) = dudt(i, j, k) + c.utend(k);
          dvdt(i, j, k) = dvdt(i, j, k) + c.vtend(k);
        }
    for (int k = 1; k <= nzm; ++k)
      for (int j = 1; j <= g.ny; ++j)
        for (int i = 1; i <= g.nx; ++i)
          if (nneg[k] > 0 && qpoz[k] + qneg[k] > 0.) {
            double factor = 1. + qneg[k] / qpoz[k];
            c.qt(i, j, k) = fmax2(0., c.qt(i, j, k) * factor);
          }
  }

  // ---- radiative heating (crm_module.F90:766-777)
  void radiation(Column &c) {
    for (int k = 1; k <= g.nzm; ++k)
      for (int j = 1; j <= g.ny; ++j)
        for (int i = 1; i <= g.nx; ++i) {
          int i_rad = (i - 1) / (g.nx / g.nx_rad) + 1;
          int j_rad = (j - 1) / (g.ny / g.ny_rad) + 1;
          c.t(i, j, k) = c.t(i, j, k) + c.qrad(i_rad, j_rad, k) * c.dtn;
        }
  }

  // ---- damping.F90:9-117
  void damping(Column &c) {
    const int nzm = g.nzm, nx = g.nx, ny = g.ny;
    const double tau_min = 60., tau_max = 450., damp_depth = R4(0.4);
    int n_damp = 0;
    for (int k = nzm; k >= 1; --k)
      if (c.z(nzm) - c.z(k) < damp_depth * c.z(nzm)) n_damp = nzm - k + 1;
    std::vector<double> tau(nzm + 1, 0.), u0l(nzm + 1, 0.), v0l(nzm + 1, 0.), t0l(nzm + 1, 0.);
    for (int k = 1; k <= nzm; ++k)
      if (k >= nzm - n_damp) {
        tau[k] = tau_min * det_pow(tau_max / tau_min, (c.z(nzm) - c.z(k)) / (c.z(nzm) - c.z(nzm - n_damp)));
        tau[k] = 1. / tau[k];
      }
    const double nxy = (double)(nx * ny);
    for (int k = 1; k <= nzm; ++k)
      for (int j = 1; j <= ny; ++j)
        for (int i = 1; i <= nx; ++i) {
          u0l[k] = u0l[k] + c.u(i, j, k) / nxy;
          v0l[k] = v0l[k] + c.v(i, j, k) / nxy;
          t0l[k] = t0l[k] + c.t(i, j, k) / nxy;
        }
    A3 &dudt = DU(c, c.na), &dvdt = DV(c, c.na), &dwdt = DW(c, c.na);
    for (int k = 1; k <= nzm; ++k)
      for (int j = 1; j <= ny; ++j)
        for (int i = 1; i <= nx; ++i)
          if (k >= nzm - n_damp) {
            dudt(i, j, k) = dudt(i, j, k) - (c.u(i, j, k) - u0l[k]) * tau[k];
            dvdt(i, j, k) = dvdt(i, j, k) - (c.v(i, j, k) - v0l[k]) * tau[k];
            dwdt(i, j, k) = dwdt(i, j, k) - c.w(i, j, k) * tau[k];
            c.t(i, j, k) = c.t(i, j, k) - c.dtn * (c.t(i, j, k) - t0l[k]) * tau[k];
            c.qt(i, j, k) = c.qt(i, j, k) - c.dtn * (c.qv(i, j, k) - c.qv0(k)) * tau[k];
          }
  }

  // ---- ice_fall.F90:6-173
  void ice_fall(Column &c) {
    const int nx = g.nx, ny = g.ny, nzm = g.nzm, nz = g.nz;
    int kmax = 0, kmin = nzm + 1;
    for (int j = 1; j <= ny; ++j)
      for (int i = 1; i <= nx; ++i)
        for (int k = 1; k <= nzm; ++k)
          if (c.qcl(i, j, k) + c.qci(i, j, k) > 0. && c.tabs(i, j, k) < R4(273.15)) {
            kmin = std::min(kmin, k);
            kmax = std::max(kmax, k);
          }
    for (int k = 1; k <= nzm; ++k) { c.qifall(k) = 0.; c.tlatqi(k) = 0.; }
    A3 fz;
    fz.init(1, nx, 1, ny, 1, nz);
    for (int k = 1; k <= nz; ++k)
      for (int j = 1; j <= ny; ++j)
        for (int i = 1; i <= nx; ++i)
          if (k >= std::max(1, kmin - 1) && k <= kmax) {
            int kc = std::min(nzm, k + 1), kb = std::max(1, k - 1);
            double coef = c.dtn / (0.5 * (c.adz(kb) + c.adz(k)) * c.dz);
            double qiu = c.rho(kc) * c.qci(i, j, kc);
            double qic = c.rho(k) * c.qci(i, j, k);
            double qid = c.rho(kb) * c.qci(i, j, kb);
            double vt_ice = fmin2(R4(0.4), R4(8.66) * det_pow(fmax2(0., qic) + R4(1.e-10), R4(0.24)));
            double tmp_phi;
            if (fabs(qic - qid) < R4(1.0e-25)) tmp_phi = 0.;
            else {
              double tmp_theta = (qiu - qic) / (qic - qid);
              tmp_phi = fmax2(0., fmin3(0.5 * (1. + tmp_theta), 2., 2. * tmp_theta));
            }
            fz(i, j, k) = -vt_ice * (qic - 0.5 * (1. - coef * vt_ice) * tmp_phi * (qic - qid));
          }
    for (int j = 1; j <= ny; ++j)
      for (int i = 1; i <= nx; ++i) fz(i, j, nz) = 0.;
    for (int k = 1; k <= nz; ++k)
      for (int j = 1; j <= ny; ++j)
        for (int i = 1; i <= nx; ++i)
          if (k >= std::max(1, kmin - 2) && k <= kmax) {
            double coef = c.dtn / (c.dz * c.adz(k) * c.rho(k));
            double dqi = coef * (fz(i, j, k) - fz(i, j, k + 1));
            c.qt(i, j, k) = c.qt(i, j, k) + dqi;
            c.qifall(k) = c.qifall(k) + dqi;
            double lat_heat = (fac_cond + fac_fus) * dqi;
            c.t(i, j, k) = c.t(i, j, k) - lat_heat;
            c.tlatqi(k) = c.tlatqi(k) - lat_heat;
          }
    for (int j = 1; j <= ny; ++j)
      for (int i = 1; i <= nx; ++i) {
        double coef = c.dtn / c.dz;
        double dqi = -coef * fz(i, j, 1);
        c.precsfc(i, j, 1) = c.precsfc(i, j, 1) + dqi;
        c.precssfc(i, j, 1) = c.precssfc(i, j, 1) + dqi;
      }
  }

  // ---- shear_prod2D.F90:7-96
  // SGS_TKE/shear_prod3D.F90:7-140
  void shear_prod3D(Column &c, A3 &def2) {
    const double rdx0 = 1. / g.dx, rdy0 = 1. / g.dy, dx = g.dx, dy = g.dy;
    const int nzm = g.nzm;
    A3 &u = c.u, &v = c.v, &w = c.w;
    A1 &u0 = c.u0, &v0 = c.v0;
    auto sq = [](double x) { return x * x; };
    for (int k = 1; k <= nzm; ++k)
      for (int j = 1; j <= g.ny; ++j)
        for (int i = 1; i <= g.nx; ++i) {
          int jb = j - 1, jc = j + 1, ib = i - 1, ic = i + 1;
          if (k >= 2 && k <= nzm - 1) {
            int kb = k - 1, kc = k + 1;
            double rdz = 1. / (c.dz * c.adz(k));
            double rdzw_up = 1. / (c.dz * c.adzw(kc));
            double rdzw_dn = 1. / (c.dz * c.adzw(k));
            double rdx = rdx0 * sqrt(dx * rdz), rdy = rdy0 * sqrt(dy * rdz);
            double rdx_up = rdx0 * sqrt(dx * rdzw_up), rdy_up = rdy0 * sqrt(dy * rdzw_up);
            double rdx_dn = rdx0 * sqrt(dx * rdzw_dn), rdy_dn = rdy0 * sqrt(dy * rdzw_dn);
            double d = 2. * (sq((u(ic, j, k) - u(i, j, k)) * rdx) + sq((v(i, jc, k) - v(i, j, k)) * rdy) +
                             sq((w(i, j, kc) - w(i, j, k)) * rdz)) +
                       0.25 * (sq((u(ic, jc, k) - u(ic, j, k)) * rdy + (v(ic, jc, k) - v(i, jc, k)) * rdx) +
                               sq((u(i, jc, k) - u(i, j, k)) * rdy + (v(i, jc, k) - v(ib, jc, k)) * rdx) +
                               sq((u(ic, j, k) - u(ic, jb, k)) * rdy + (v(ic, j, k) - v(i, j, k)) * rdx) +
                               sq((u(i, j, k) - u(i, jb, k)) * rdy + (v(i, j, k) - v(ib, j, k)) * rdx));
            d = d + 0.25 * (sq((u(ic, j, kc) - u0(kc) - u(ic, j, k) + u0(k)) * rdzw_up + (w(ic, j, kc) - w(i, j, kc)) * rdx_up) +
                            sq((u(i, j, kc) - u0(kc) - u(i, j, k) + u0(k)) * rdzw_up + (w(i, j, kc) - w(ib, j, kc)) * rdx_up) +
                            sq((u(ic, j, k) - u0(k) - u(ic, j, kb) + u0(kb)) * rdzw_dn + (w(ic, j, k) - w(i, j, k)) * rdx_dn) +
                            sq((u(i, j, k) - u0(k) - u(i, j, kb) + u0(kb)) * rdzw_dn + (w(i, j, k) - w(ib, j, k)) * rdx_dn));
            d = d + 0.25 * (sq((v(i, jc, kc) - v0(kc) - v(i, jc, k) + v0(k)) * rdzw_up + (w(i, jc, kc) - w(i, j, kc)) * rdy_up) +
                            sq((v(i, j, kc) - v0(kc) - v(i, j, k) + v0(k)) * rdzw_up + (w(i, j, kc) - w(i, jb, kc)) * rdy_up) +
                            sq((v(i, jc, k) - v0(k) - v(i, jc, kb) + v0(kb)) * rdzw_dn + (w(i, jc, k) - w(i, j, k)) * rdy_dn) +
                            sq((v(i, j, k) - v0(k) - v(i, j, kb) + v0(kb)) * rdzw_dn + (w(i, j, k) - w(i, jb, k)) * rdy_dn));
            def2(i, j, k) = d;
          } else if (k == 1) {
            int kc = k + 1;
            double rdz = 1. / (c.dz * c.adz(k));
            double rdzw_up = 1. / (c.dz * c.adzw(kc));
            double rdx = rdx0 * sqrt(dx * rdz), rdy = rdy0 * sqrt(dy * rdz);
            double rdx_up = rdx0 * sqrt(dx * rdzw_up), rdy_up = rdy0 * sqrt(dy * rdzw_up);
            def2(i, j, k) =
                2. * (sq((u(ic, j, k) - u(i, j, k)) * rdx) + sq((v(i, jc, k) - v(i, j, k)) * rdy) +
                      sq((w(i, j, kc) - w(i, j, k)) * rdz)) +
                0.25 * (sq((u(ic, jc, k) - u(ic, j, k)) * rdy + (v(ic, jc, k) - v(i, jc, k)) * rdx) +
                        sq((u(i, jc, k) - u(i, j, k)) * rdy + (v(i, jc, k) - v(ib, jc, k)) * rdx) +
                        sq((u(ic, j, k) - u(ic, jb, k)) * rdy + (v(ic, j, k) - v(i, j, k)) * rdx) +
                        sq((u(i, j, k) - u(i, jb, k)) * rdy + (v(i, j, k) - v(ib, j, k)) * rdx)) +
                0.5 * (sq((v(i, jc, kc) - v0(kc) - v(i, jc, k) + v0(k)) * rdzw_up + (w(i, jc, kc) - w(i, j, kc)) * rdy_up) +
                       sq((v(i, j, kc) - v0(kc) - v(i, j, k) + v0(k)) * rdzw_up + (w(i, j, kc) - w(i, jb, kc)) * rdy_up)) +
                0.5 * (sq((u(ic, j, kc) - u0(kc) - u(ic, j, k) + u0(k)) * rdzw_up + (w(ic, j, kc) - w(i, j, kc)) * rdx_up) +
                       sq((u(i, j, kc) - u0(kc) - u(i, j, k) + u0(k)) * rdzw_up + (w(i, j, kc) - w(ib, j, kc)) * rdx_up));
          } else {  // k == nzm
            int kc = k + 1, kb = k - 1;
            double rdz = 1. / (c.dz * c.adz(k));
            double rdzw_dn = 1. / (c.dz * c.adzw(k));
            double rdx = rdx0 * sqrt(dx * rdz), rdy = rdy0 * sqrt(dy * rdz);
            double rdx_dn = rdx0 * sqrt(dx * rdzw_dn), rdy_dn = rdy0 * sqrt(dy * rdzw_dn);
            def2(i, j, k) =
                2. * (sq((u(ic, j, k) - u(i, j, k)) * rdx) + sq((v(i, jc, k) - v(i, j, k)) * rdy) +
                      sq((w(i, j, kc) - w(i, j, k)) * rdz)) +
                0.25 * (sq((u(ic, jc, k) - u(ic, j, k)) * rdy + (v(ic, jc, k) - v(i, jc, k)) * rdx) +
                        sq((u(i, jc, k) - u(i, j, k)) * rdy + (v(i, jc, k) - v(ib, jc, k)) * rdx) +
                        sq((u(ic, j, k) - u(ic, jb, k)) * rdy + (v(ic, j, k) - v(i, j, k)) * rdx) +
                        sq((u(i, j, k) - u(i, jb, k)) * rdy + (v(i, j, k) - v(ib, j, k)) * rdx)) +
                0.5 * (sq((v(i, jc, k) - v0(k) - v(i, jc, kb) + v0(kb)) * rdzw_dn + (w(i, jc, k) - w(i, j, k)) * rdy_dn) +
                       sq((v(i, j, k) - v0(k) - v(i, j, kb) + v0(kb)) * rdzw_dn + (w(i, j, k) - w(i, jb, k)) * rdy_dn)) +
                0.5 * (sq((u(ic, j, k) - u0(k) - u(ic, j, kb) + u0(kb)) * rdzw_dn + (w(ic, j, k) - w(i, j, k)) * rdx_dn) +
                       sq((u(i, j, k) - u0(k) - u(i, j, kb) + u0(kb)) * rdzw_dn + (w(i, j, k) - w(ib, j, k)) * rdx_dn));
          }
        }
  }
  void shear_prod2D(Column &c, A3 &def2) {
    const double rdx0 = 1. / g.dx, dx = g.dx;
    const int j = 1, nzm = g.nzm;
    for (int k = 1; k <= nzm; ++k)
      for (int i = 1; i <= g.nx; ++i) {
        int ib = i - 1, ic = i + 1;
        A3 &u = c.u, &v = c.v, &w = c.w;
        A1 &u0 = c.u0, &v0 = c.v0;
        auto sq = [](double x) { return x * x; };
        if (k >= 2 && k <= nzm - 1) {
          int kb = k - 1, kc = k + 1;
          double rdz = 1. / (c.dz * c.adz(k));
          double rdzw_up = 1. / (c.dz * c.adzw(kc));
          double rdzw_dn = 1. / (c.dz * c.adzw(k));
          double rdx = rdx0 * sqrt(dx * rdz);
          double rdx_up = rdx0 * sqrt(dx * rdzw_up);
          double rdx_dn = rdx0 * sqrt(dx * rdzw_dn);
          def2(i, j, k) = 2. * (sq((u(ic, j, k) - u(i, j, k)) * rdx) + sq((w(i, j, kc) - w(i, j, k)) * rdz)) +
              0.5 * (sq((v(ic, j, k) - v(i, j, k)) * rdx) + sq((v(i, j, k) - v(ib, j, k)) * rdx) +
                     sq((u(ic, j, kc) - u0(kc) - u(ic, j, k) + u0(k)) * rdzw_up + (w(ic, j, kc) - w(i, j, kc)) * rdx_up) +
                     sq((u(i, j, kc) - u0(kc) - u(i, j, k) + u0(k)) * rdzw_up + (w(i, j, kc) - w(ib, j, kc)) * rdx_up) +
                     sq((u(ic, j, k) - u0(k) - u(ic, j, kb) + u0(kb)) * rdzw_dn + (w(ic, j, k) - w(i, j, k)) * rdx_dn) +
                     sq((u(i, j, k) - u0(k) - u(i, j, kb) + u0(kb)) * rdzw_dn + (w(i, j, k) - w(ib, j, k)) * rdx_dn) +
                     sq((v(i, j, kc) - v0(kc) - v(i, j, k) + v0(k)) * rdzw_up) +
                     sq((v(i, j, k) - v0(k) - v(i, j, kb) + v0(kb)) * rdzw_dn));
        } else if (k == 1) {
          int kc = k + 1;
          double rdz = 1. / (c.dz * c.adz(k));
          double rdzw_up = 1. / (c.dz * c.adzw(kc));
          double rdx = rdx0 * sqrt(dx * rdz);
          double rdx_up = rdx0 * sqrt(dx * rdzw_up);
          def2(i, j, k) = 2. * (sq((u(ic, j, k) - u(i, j, k)) * rdx) + sq((w(i, j, kc) - w(i, j, k)) * rdz)) +
              0.5 * (sq((v(ic, j, k) - v(i, j, k)) * rdx) + sq((v(i, j, k) - v(ib, j, k)) * rdx)) +
              sq((v(i, j, kc) - v0(kc) - v(i, j, k) + v0(k)) * rdzw_up) +
              0.5 * (sq((u(ic, j, kc) - u0(kc) - u(ic, j, k) + u0(k)) * rdzw_up + (w(ic, j, kc) - w(i, j, kc)) * rdx_up) +
                     sq((u(i, j, kc) - u0(kc) - u(i, j, k) + u0(k)) * rdzw_up + (w(i, j, kc) - w(ib, j, kc)) * rdx_up));
        } else {  // k == nzm
          int kc = k + 1, kb = k - 1;
          double rdz = 1. / (c.dz * c.adz(k));
          double rdzw_dn = 1. / (c.dz * c.adzw(k));
          double rdx = rdx0 * sqrt(dx * rdz);
          double rdx_dn = rdx0 * sqrt(dx * rdzw_dn);
          def2(i, j, k) = 2. * (sq((u(ic, j, k) - u(i, j, k)) * rdx) + sq((w(i, j, kc) - w(i, j, k)) * rdz)) +
              0.5 * (sq((v(ic, j, k) - v(i, j, k)) * rdx) + sq((v(i, j, k) - v(ib, j, k)) * rdx)) +
              sq((v(i, j, k) - v0(k) - v(i, j, kb) + v0(kb)) * rdzw_dn) +
              0.5 * (sq((u(ic, j, k) - u0(k) - u(ic, j, kb) + u0(kb)) * rdzw_dn + (w(ic, j, k) - w(i, j, k)) * rdx_dn) +
                     sq((u(i, j, k) - u0(k) - u(i, j, kb) + u0(kb)) * rdzw_dn + (w(i, j, k) - w(ib, j, k)) * rdx_dn));
        }
      }
  }

  // ---- tke_full.F90:11-317 (dosmagor = .true.)
  void tke_full(Column &c) {
    const int nx = g.nx, ny = g.ny, nzm = g.nzm;
    A3 def2;
    def2.init(1, nx, 1, ny, 1, nzm);
    if (g.YES3D) shear_prod3D(c, def2);    // tke_full.F90:109-113
    else shear_prod2D(c, def2);
    A3 buoy_v, aprod_v;
    buoy_v.init(1, nx, 1, ny, 0, nzm);
    aprod_v.init(1, nx, 1, ny, 0, nzm);
    const double Cs = R4(0.15), Ck = R4(0.1);
    const double Ce = Ck * Ck * Ck / ((Cs * Cs) * (Cs * Cs));
    const double Pr = 1.;
    for (int k = 1; k <= nzm - 1; ++k)
      for (int j = 1; j <= ny; ++j)
        for (int i = 1; i <= nx; ++i) {
          int kc = k + 1, kb = k;
          double betdz = 0.5 * (c.bet(kc) + c.bet(kb)) / c.dz / c.adzw(k + 1);
          double tabs_if = 0.5 * (c.tabs(i, j, kc) + fac_cond * c.qcl(i, j, kc) + fac_sub * c.qci(i, j, kc) +
                                  c.tabs(i, j, kb) + fac_cond * c.qcl(i, j, kb) + fac_sub * c.qci(i, j, kb));
          double qtot_if = 0.5 * (c.qv(i, j, kc) + c.qcl(i, j, kc) + c.qci(i, j, kc) + c.qv(i, j, kb) +
                                  c.qcl(i, j, kb) + c.qci(i, j, kb));
          double qp_if = 0.5 * (c.qpl(i, j, kc) + c.qpi(i, j, kc) + c.qpl(i, j, kb) + c.qpi(i, j, kb));
          double bbb = 1. + epsv * qtot_if - qp_if;
          double dqtot = c.qv(i, j, kc) + c.qcl(i, j, kc) + c.qci(i, j, kc) - c.qv(i, j, kb) - c.qcl(i, j, kb) - c.qci(i, j, kb);
          double buoy_sgs = betdz * (bbb * (c.t(i, j, kc) - c.t(i, j, kb)) + epsv * tabs_if * dqtot +
                                     (bbb * fac_cond - tabs_if) * (c.qpl(i, j, kc) - c.qpl(i, j, kb)) +
                                     (bbb * fac_sub - tabs_if) * (c.qpi(i, j, kc) - c.qpi(i, j, kb)));
          buoy_v(i, j, k) = buoy_sgs;
          aprod_v(i, j, k) = -0.5 * (c.tkh(i, j, kc) + c.tkh(i, j, kb) + R4(0.002)) * buoy_sgs;
          double qctot = c.qcl(i, j, kc) + c.qci(i, j, kc) + c.qcl(i, j, kb) + c.qci(i, j, kb);
          if (qctot > 0.) {
            double omn = (c.qcl(i, j, kc) + c.qcl(i, j, kb)) / (qctot + R4(1.e-20));
            tabs_if = 0.5 * (c.tabs(i, j, kc) + fac_cond * c.qcl(i, j, kc) + fac_sub * c.qci(i, j, kc) +
                             c.tabs(i, j, kb) + fac_cond * c.qcl(i, j, kb) + fac_sub * c.qci(i, j, kb));
            qtot_if = 0.5 * (c.qv(i, j, kc) + c.qcl(i, j, kc) + c.qci(i, j, kc) + c.qv(i, j, kb) +
                             c.qcl(i, j, kb) + c.qci(i, j, kb));
            double qsat_check = omn * qsatw(tabs_if, c.presi(k + 1)) + (1. - omn) * qsati(tabs_if, c.presi(k + 1));
            if (qtot_if > qsat_check) {
              double lstarn = fac_cond + (1. - omn) * fac_fus;
              tabs_if = 0.5 * (c.tabs(i, j, kc) + c.tabs(i, j, kb));
              qp_if = 0.5 * (c.qpl(i, j, kc) + c.qpi(i, j, kc) + c.qpl(i, j, kb) + c.qpi(i, j, kb));
              double dqsat = omn * dtqsatw(tabs_if, c.presi(k + 1)) + (1. - omn) * dtqsati(tabs_if, c.presi(k + 1));
              double qsatt = omn * qsatw(tabs_if, c.presi(k + 1)) + (1. - omn) * qsati(tabs_if, c.presi(k + 1));
              bbb = 1. + epsv * qsatt + qsatt - qtot_if - qp_if + R4(1.61) * tabs_if * dqsat;
              bbb = bbb / (1. + lstarn * dqsat);
              buoy_sgs = betdz * (bbb * (c.t(i, j, kc) - c.t(i, j, kb)) +
                                  (bbb * lstarn - (1. + lstarn * dqsat) * tabs_if) * dqtot +
                                  (bbb * fac_cond - (1. + fac_cond * dqsat) * c.tabs(i, j, k)) * (c.qpl(i, j, kc) - c.qpl(i, j, kb)) +
                                  (bbb * fac_sub - (1. + fac_sub * dqsat) * c.tabs(i, j, k)) * (c.qpi(i, j, kc) - c.qpi(i, j, kb)));
              buoy_v(i, j, k) = buoy_sgs;
              aprod_v(i, j, k) = -0.5 * (c.tkh(i, j, kc) + c.tkh(i, j, kb) + R4(0.002)) * buoy_sgs;
            }
          }
        }
    for (int k = 1; k <= nzm - 1; ++k)
      for (int j = 1; j <= ny; ++j)
        for (int i = 1; i <= nx; ++i) {
          double grd = c.dz * c.adz(k);
          double Ce1 = Ce / R4(0.7) * R4(0.19);
          double Ce2 = Ce / R4(0.7) * R4(0.51);
          double cx = g.dx * g.dx / g.dt / c.grdf_x(k);
          double cy = g.dy * g.dy / g.dt / c.grdf_y(k);
          double dzm = c.dz * fmin2(c.adzw(k), c.adzw(k + 1));
          double cz = dzm * dzm / g.dt / c.grdf_z(k);
          double tkmax = R4(0.09) / (1. / cx + 1. / cy + 1. / cz);
          double buoy_sgs = 0.5 * (buoy_v(i, j, k - 1) + buoy_v(i, j, k));
          double smix;
          if (buoy_sgs <= 0.) smix = grd;
          else smix = fmin2(grd, fmax2(R4(0.1) * grd, sqrt(R4(0.76) * c.tk(i, j, k) / Ck / sqrt(buoy_sgs + R4(1.e-10)))));
          double ratio = smix / grd;
          double Cee = Ce1 + Ce2 * ratio;
          c.tk(i, j, k) = sqrt(Ck * Ck * Ck / Cee * fmax2(0., def2(i, j, k) - Pr * buoy_sgs)) * (smix * smix);
          double tq = c.tk(i, j, k) / (Ck * smix);
          c.tke(i, j, k) = tq * tq;
          c.tk(i, j, k) = fmin2(c.tk(i, j, k), tkmax);
          c.tkh(i, j, k) = Pr * c.tk(i, j, k);
        }
  }

  // ---- advect2_mom_xy.F90:7-86 (2D) and advect2_mom_z.F90:7-128
  // advect2_mom_xy.F90:7-86 and advect2_mom_z.F90:7-128 (2D and 3D)
  void advect_mom(Column &c) {
    const int nx = g.nx, ny = g.ny, nzm = g.nzm, nz = g.nz;
    A3 &dudt = DU(c, c.na), &dvdt = DV(c, c.na), &dwdt = DW(c, c.na);
    A3 &u = c.u, &v = c.v, &w = c.w;
    const double dx25 = 0.25 / g.dx;
    const double dy25 = 0.25 / g.dy;
    for (int k = 1; k <= nzm; ++k)
      for (int j = 1; j <= ny; ++j)
        for (int i = 1; i <= nx; ++i) {
          int kc = k + 1, kcu = std::min(kc, nzm);
          double irho = 1. / (c.rhow(kc) * c.adzw(kc));
          int ic = i + 1;
          double fu1 = dx25 * (u(ic - 1, j, k) + u(i - 1, j, k)) * (u(i - 1, j, k) + u(ic - 1, j, k));
          double fu2 = dx25 * (u(ic, j, k) + u(i, j, k)) * (u(i, j, k) + u(ic, j, k));
          dudt(i, j, k) = dudt(i, j, k) - (fu2 - fu1);
          double fv1, fv2;
          if (g.YES3D) {
            int jb = j - 1;
            fv1 = dx25 * (u(ic - 1, j, k) + u(ic - 1, jb, k)) * (v(i - 1, j, k) + v(ic - 1, j, k));
            fv2 = dx25 * (u(ic, j, k) + u(ic, jb, k)) * (v(i, j, k) + v(ic, j, k));
          } else {
            fv1 = dx25 * (u(ic - 1, j, k) + u(i - 1, j, k)) * (v(i - 1, j, k) + v(ic - 1, j, k));
            fv2 = dx25 * (u(ic, j, k) + u(i, j, k)) * (v(i, j, k) + v(ic, j, k));
          }
          dvdt(i, j, k) = dvdt(i, j, k) - (fv2 - fv1);
          double fw1 = dx25 * (u(ic - 1, j, k) * c.rho(k) * c.adz(k) + u(ic - 1, j, kcu) * c.rho(kcu) * c.adz(kcu)) *
                       (w(i - 1, j, kc) + w(ic - 1, j, kc));
          double fw2 = dx25 * (u(ic, j, k) * c.rho(k) * c.adz(k) + u(ic, j, kcu) * c.rho(kcu) * c.adz(kcu)) *
                       (w(i, j, kc) + w(ic, j, kc));
          dwdt(i, j, kc) = dwdt(i, j, kc) - irho * (fw2 - fw1);
          if (g.YES3D) {                       // the y terms (advect2_mom_xy.F90:46-60)
            int jc = j + 1, ib = i - 1;
            fu1 = dy25 * (v(i, jc - 1, k) + v(ib, jc - 1, k)) * (u(i, j - 1, k) + u(i, jc - 1, k));
            fu2 = dy25 * (v(i, jc, k) + v(ib, jc, k)) * (u(i, j, k) + u(i, jc, k));
            dudt(i, j, k) = dudt(i, j, k) - (fu2 - fu1);
            fv1 = dy25 * (v(i, jc - 1, k) + v(i, j - 1, k)) * (v(i, j - 1, k) + v(i, jc - 1, k));
            fv2 = dy25 * (v(i, jc, k) + v(i, j, k)) * (v(i, j, k) + v(i, jc, k));
            dvdt(i, j, k) = dvdt(i, j, k) - (fv2 - fv1);
            fw1 = dy25 * (v(i, jc - 1, k) * c.rho(k) * c.adz(k) + v(i, jc - 1, kcu) * c.rho(kcu) * c.adz(kcu)) *
                  (w(i, j - 1, kc) + w(i, jc - 1, kc));
            fw2 = dy25 * (v(i, jc, k) * c.rho(k) * c.adz(k) + v(i, jc, kcu) * c.rho(kcu) * c.adz(kcu)) *
                  (w(i, j, kc) + w(i, jc, kc));
            dwdt(i, j, kc) = dwdt(i, j, kc) - irho * (fw2 - fw1);
          }
        }
    // vertical
    A3 fuz, fvz, fwz;
    fuz.init(1, nx, 1, ny, 1, nz); fvz.init(1, nx, 1, ny, 1, nz); fwz.init(1, nx, 1, ny, 1, nzm);
    for (int k = 1; k <= nz; ++k) { c.uwle(k) = 0.; c.vwle(k) = 0.; }
    for (int k = 2; k <= nzm; ++k)
      for (int j = 1; j <= ny; ++j)
        for (int i = 1; i <= nx; ++i) {
          double dz25 = 1. / (4. * c.dz);
          int kb = k - 1;
          double rhoi = dz25 * c.rhow(k);
          double www = rhoi * (w(i, j, k) + w(i - 1, j, k));
          fuz(i, j, k) = www * (u(i, j, k) + u(i, j, kb));
          if (g.YES3D) fvz(i, j, k) = rhoi * (w(i, j, k) + w(i, j - 1, k)) * (v(i, j, k) + v(i, j, kb));
          else fvz(i, j, k) = www * (v(i, j, k) + v(i, j, kb));
          c.uwle(k) = c.uwle(k) + fuz(i, j, k);
          c.vwle(k) = c.vwle(k) + fvz(i, j, k);
        }
    for (int k = 1; k <= nzm; ++k)
      for (int j = 1; j <= ny; ++j)
        for (int i = 1; i <= nx; ++i) {
          double dz25 = 1. / (4. * c.dz);
          int kc = k + 1;
          double rhoi = 1. / (c.rho(k) * c.adz(k));
          dudt(i, j, k) = dudt(i, j, k) - (fuz(i, j, kc) - fuz(i, j, k)) * rhoi;
          dvdt(i, j, k) = dvdt(i, j, k) - (fvz(i, j, kc) - fvz(i, j, k)) * rhoi;
          fwz(i, j, k) = dz25 * (w(i, j, kc) * c.rhow(kc) + w(i, j, k) * c.rhow(k)) * (w(i, j, kc) + w(i, j, k));
        }
    for (int k = 2; k <= nzm; ++k)
      for (int j = 1; j <= ny; ++j)
        for (int i = 1; i <= nx; ++i) {
          int kb = k - 1;
          double rhoi = 1. / (c.rhow(k) * c.adzw(k));
          dwdt(i, j, k) = dwdt(i, j, k) - (fwz(i, j, k) - fwz(i, j, kb)) * rhoi;
        }
  }
  // SGS_TKE/diffuse_mom3D.F90:7-207 (fluxbu, fluxbv, fluxtu, fluxtv are 0)
  void diffuse_mom3D(Column &c) {
    const int nx = g.nx, ny = g.ny, nzm = g.nzm, nz = g.nz;
    A3 &dudt = DU(c, c.na), &dvdt = DV(c, c.na), &dwdt = DW(c, c.na);
    A3 &u = c.u, &v = c.v, &w = c.w, &tk = c.tk;
    A3 fu, fv, fw;
    fu.init(0, nx, 0, ny, 1, nz); fv.init(0, nx, 0, ny, 1, nz); fw.init(0, nx, 0, ny, 1, nz);
    const double rdx2 = 1. / (g.dx * g.dx), rdy2 = 1. / (g.dy * g.dy);
    const double rdx25 = 0.25 * rdx2, rdy25 = 0.25 * rdy2;
    const double dxy = g.dx / g.dy, dyx = g.dy / g.dx;
    for (int k = 1; k <= nzm; ++k)
      for (int j = 1; j <= ny; ++j)
        for (int i = 0; i <= nx; ++i) {
          int jb = j - 1, kc = k + 1, kcu = std::min(kc, nzm), ic = i + 1;
          double dxz = g.dx / (c.dz * c.adzw(kc));
          double rdx21 = rdx2 * c.grdf_x(k);
          double rdx251 = rdx25 * c.grdf_x(k);
          double tkx = rdx21 * tk(i, j, k);
          fu(i, j, k) = -2. * tkx * (u(ic, j, k) - u(i, j, k));
          tkx = rdx251 * (tk(i, j, k) + tk(i, jb, k) + tk(ic, j, k) + tk(ic, jb, k));
          fv(i, j, k) = -tkx * (v(ic, j, k) - v(i, j, k) + (u(ic, j, k) - u(ic, jb, k)) * dxy);
          tkx = rdx251 * (tk(i, j, k) + tk(ic, j, k) + tk(i, j, kcu) + tk(ic, j, kcu));
          fw(i, j, k) = -tkx * (w(ic, j, kc) - w(i, j, kc) + (u(ic, j, kcu) - u(ic, j, k)) * dxz);
        }
    for (int k = 1; k <= nzm; ++k)
      for (int j = 1; j <= ny; ++j)
        for (int i = 1; i <= nx; ++i) {
          int kc = k + 1, ib = i - 1;
          dudt(i, j, k) = dudt(i, j, k) - (fu(i, j, k) - fu(ib, j, k));
          dvdt(i, j, k) = dvdt(i, j, k) - (fv(i, j, k) - fv(ib, j, k));
          dwdt(i, j, kc) = dwdt(i, j, kc) - (fw(i, j, k) - fw(ib, j, k));
        }
    for (int k = 1; k <= nzm; ++k)
      for (int j = 0; j <= ny; ++j)
        for (int i = 1; i <= nx; ++i) {
          int jc = j + 1, kc = k + 1, kcu = std::min(kc, nzm), ib = i - 1;
          double dyz = g.dy / (c.dz * c.adzw(kc));
          double rdy21 = rdy2 * c.grdf_y(k);
          double rdy251 = rdy25 * c.grdf_y(k);
          double tky = rdy21 * tk(i, j, k);
          fv(i, j, k) = -2. * tky * (v(i, jc, k) - v(i, j, k));
          tky = rdy251 * (tk(i, j, k) + tk(ib, j, k) + tk(i, jc, k) + tk(ib, jc, k));
          fu(i, j, k) = -tky * (u(i, jc, k) - u(i, j, k) + (v(i, jc, k) - v(ib, jc, k)) * dyx);
          tky = rdy251 * (tk(i, j, k) + tk(i, jc, k) + tk(i, j, kcu) + tk(i, jc, kcu));
          fw(i, j, k) = -tky * (w(i, jc, kc) - w(i, j, kc) + (v(i, jc, kcu) - v(i, jc, k)) * dyz);
        }
    for (int k = 1; k <= nzm; ++k)
      for (int j = 1; j <= ny; ++j)
        for (int i = 1; i <= nx; ++i) {
          int jb = j - 1, kc = k + 1;
          dudt(i, j, k) = dudt(i, j, k) - (fu(i, j, k) - fu(i, jb, k));
          dvdt(i, j, k) = dvdt(i, j, k) - (fv(i, j, k) - fv(i, jb, k));
          dwdt(i, j, kc) = dwdt(i, j, kc) - (fw(i, j, k) - fw(i, jb, k));
        }
    for (int k = 1; k <= nzm; ++k) { c.uwsb(k) = 0.; c.vwsb(k) = 0.; }
    for (int k = 1; k <= nzm - 1; ++k)
      for (int j = 1; j <= ny; ++j)
        for (int i = 1; i <= nx; ++i) {
          int jb = j - 1, kc = k + 1, ib = i - 1;
          double rdz = 1. / c.dz;
          double rdz2 = rdz * rdz * c.grdf_z(k);
          double rdz25 = 0.25 * rdz2;
          double iadz = 1. / c.adz(k);
          double iadzw = 1. / c.adzw(kc);
          double dzx = c.dz / g.dx, dzy = c.dz / g.dy;
          double tkz = rdz2 * tk(i, j, k);
          fw(i, j, kc) = -2. * tkz * (w(i, j, kc) - w(i, j, k)) * c.rho(k) * iadz;
          tkz = rdz25 * (tk(i, j, k) + tk(ib, j, k) + tk(i, j, kc) + tk(ib, j, kc));
          fu(i, j, kc) = -tkz * ((u(i, j, kc) - u(i, j, k)) * iadzw + (w(i, j, kc) - w(ib, j, kc)) * dzx) * c.rhow(kc);
          tkz = rdz25 * (tk(i, j, k) + tk(i, jb, k) + tk(i, j, kc) + tk(i, jb, kc));
          fv(i, j, kc) = -tkz * ((v(i, j, kc) - v(i, j, k)) * iadzw + (w(i, j, kc) - w(i, jb, kc)) * dzy) * c.rhow(kc);
          c.uwsb(kc) = c.uwsb(kc) + fu(i, j, kc);
          c.vwsb(kc) = c.vwsb(kc) + fv(i, j, kc);
        }
    for (int j = 1; j <= ny; ++j)
      for (int i = 1; i <= nx; ++i) {
        double rdz = 1. / c.dz;
        double rdz2 = rdz * rdz * c.grdf_z(nzm - 1);
        double tkz = rdz2 * c.grdf_z(nzm) * tk(i, j, nzm);
        fw(i, j, nz) = -2. * tkz * (w(i, j, nz) - w(i, j, nzm)) / c.adz(nzm) * c.rho(nzm);
        fu(i, j, 1) = 0.0 * rdz * c.rhow(1);
        fv(i, j, 1) = 0.0 * rdz * c.rhow(1);
        fu(i, j, nz) = 0.0 * rdz * c.rhow(nz);
        fv(i, j, nz) = 0.0 * rdz * c.rhow(nz);
        c.uwsb(1) = c.uwsb(1) + fu(i, j, 1);
        c.vwsb(1) = c.vwsb(1) + fv(i, j, 1);
      }
    for (int k = 1; k <= nzm; ++k)
      for (int j = 1; j <= ny; ++j)
        for (int i = 1; i <= nx; ++i) {
          int kc = k + 1;
          double rhoi = 1. / (c.rho(k) * c.adz(k));
          dudt(i, j, k) = dudt(i, j, k) - (fu(i, j, kc) - fu(i, j, k)) * rhoi;
          dvdt(i, j, k) = dvdt(i, j, k) - (fv(i, j, kc) - fv(i, j, k)) * rhoi;
        }
    for (int k = 2; k <= nzm; ++k)
      for (int j = 1; j <= ny; ++j)
        for (int i = 1; i <= nx; ++i) {
          double rhoi = 1. / (c.rhow(k) * c.adzw(k));
          dwdt(i, j, k) = dwdt(i, j, k) - (fw(i, j, k + 1) - fw(i, j, k)) * rhoi;
        }
  }
  void diffuse_mom2D(Column &c) {
    const int nx = g.nx, nzm = g.nzm, nz = g.nz, j = 1;
    A3 &dudt = DU(c, c.na), &dvdt = DV(c, c.na), &dwdt = DW(c, c.na);
    A3 &u = c.u, &v = c.v, &w = c.w, &tk = c.tk;
    A3 fu, fv, fw;
    fu.init(0, nx, 1, 1, 1, nz); fv.init(0, nx, 1, 1, 1, nz); fw.init(0, nx, 1, 1, 1, nz);
    const double rdx2 = 1. / g.dx / g.dx;
    const double rdx25 = 0.25 * rdx2;
    for (int k = 1; k <= nzm; ++k)
      for (int i = 0; i <= nx; ++i) {
        int kc = k + 1, kcu = std::min(kc, nzm);
        double dxz = g.dx / (c.dz * c.adzw(kc));
        double rdx21 = rdx2 * c.grdf_x(k);
        double rdx251 = rdx25 * c.grdf_x(k);
        int ic = i + 1;
        double tkx = rdx21 * tk(i, j, k);
        fu(i, j, k) = -2. * tkx * (u(ic, j, k) - u(i, j, k));
        fv(i, j, k) = -tkx * (v(ic, j, k) - v(i, j, k));
        tkx = rdx251 * (tk(i, j, k) + tk(ic, j, k) + tk(i, j, kcu) + tk(ic, j, kcu));
        fw(i, j, k) = -tkx * (w(ic, j, kc) - w(i, j, kc) + (u(ic, j, kcu) - u(ic, j, k)) * dxz);
      }
    for (int k = 1; k <= nzm; ++k)
      for (int i = 1; i <= nx; ++i) {
        int kc = k + 1, ib = i - 1;
        dudt(i, j, k) = dudt(i, j, k) - (fu(i, j, k) - fu(ib, j, k));
        dvdt(i, j, k) = dvdt(i, j, k) - (fv(i, j, k) - fv(ib, j, k));
        dwdt(i, j, kc) = dwdt(i, j, kc) - (fw(i, j, k) - fw(ib, j, k));
      }
    for (int k = 1; k <= nzm; ++k) { c.uwsb(k) = 0.; c.vwsb(k) = 0.; }
    for (int k = 1; k <= nzm - 1; ++k)
      for (int i = 1; i <= nx; ++i) {
        int kc = k + 1;
        double rdz = 1. / c.dz;
        double rdz2 = rdz * rdz * c.grdf_z(k);
        double rdz25 = 0.25 * rdz2;
        double dzx = c.dz / g.dx;
        double iadz = 1. / c.adz(k);
        double iadzw = 1. / c.adzw(kc);
        int ib = i - 1;
        double tkz = rdz2 * tk(i, j, k);
        fw(i, j, kc) = -2. * tkz * (w(i, j, kc) - w(i, j, k)) * c.rho(k) * iadz;
        tkz = rdz25 * (tk(i, j, k) + tk(ib, j, k) + tk(i, j, kc) + tk(ib, j, kc));
        fu(i, j, kc) = -tkz * ((u(i, j, kc) - u(i, j, k)) * iadzw + (w(i, j, kc) - w(ib, j, kc)) * dzx) * c.rhow(kc);
        fv(i, j, kc) = -tkz * (v(i, j, kc) - v(i, j, k)) * iadzw * c.rhow(kc);
        c.uwsb(kc) = c.uwsb(kc) + fu(i, j, kc);
        c.vwsb(kc) = c.vwsb(kc) + fv(i, j, kc);
      }
    for (int i = 1; i <= nx; ++i) {
      double rdz = 1. / c.dz;
      double rdz2 = rdz * rdz * c.grdf_z(nzm - 1);
      double tkz = rdz2 * c.grdf_z(nzm) * tk(i, j, nzm);
      fw(i, j, nz) = -2. * tkz * (w(i, j, nz) - w(i, j, nzm)) / c.adz(nzm) * c.rho(nzm);
      fu(i, j, 1) = 0.0 * rdz * c.rhow(1);      // fluxbu = 0
      fv(i, j, 1) = 0.0 * rdz * c.rhow(1);      // fluxbv = 0
      fu(i, j, nz) = 0.0 * rdz * c.rhow(nz);    // fluxtu = 0
      fv(i, j, nz) = 0.0 * rdz * c.rhow(nz);    // fluxtv = 0
      c.uwsb(1) = c.uwsb(1) + fu(i, j, 1);
      c.vwsb(1) = c.vwsb(1) + fv(i, j, 1);
    }
    for (int k = 1; k <= nzm; ++k)
      for (int i = 1; i <= nx; ++i) {
        int kc = k + 1;
        double rhoi = 1. / (c.rho(k) * c.adz(k));
        dudt(i, j, k) = dudt(i, j, k) - (fu(i, j, kc) - fu(i, j, k)) * rhoi;
        dvdt(i, j, k) = dvdt(i, j, k) - (fv(i, j, kc) - fv(i, j, k)) * rhoi;
      }
    for (int k = 2; k <= nzm; ++k)
      for (int i = 1; i <= nx; ++i) {
        double rhoi = 1. / (c.rhow(k) * c.adzw(k));
        dwdt(i, j, k) = dwdt(i, j, k) - (fw(i, j, k + 1) - fw(i, j, k)) * rhoi;
      }
  }

  // ---- pressure.F90:8-323 + press_rhs.F90 + press_grad.F90 (2D)
  // pressure.F90:8-323 with press_rhs.F90:8-106 and press_grad.F90:8-76, 3D:
  // real transform in x of every row, then in y of every x coefficient
  // (i = 1..nx+1), a tridiagonal solve per (i, j) coefficient with the
  // eigenvalue eign(i, j), and the inverse transforms in the reverse order.
  void pressure3D(Column &c) {
    const int nx = g.nx, ny = g.ny, nzm = g.nzm;
    A3 &u = c.u, &v = c.v, &w = c.w;
    A3 &dua = DU(c, c.na), &dub = DU(c, c.nb), &duc = DU(c, c.nc);
    A3 &dva = DV(c, c.na), &dvb = DV(c, c.nb), &dvc = DV(c, c.nc);
    A3 &dwa = DW(c, c.na), &dwb = DW(c, c.nb), &dwc = DW(c, c.nc);
    auto bound_duvdt = [&]() {        // bound_duvdt.F90:14-31
      for (int k = 1; k <= nzm; ++k)
        for (int j = 1; j <= ny; ++j) dua(nx + 1, j, k) = dua(1, j, k);
      for (int k = 1; k <= nzm; ++k)
        for (int i = 1; i <= nx; ++i) dva(i, ny + 1, k) = dva(i, 1, k);
    };
    bound_duvdt();
    const double rdx = 1. / g.dx, rdy = 1. / g.dy;
    const double btat = c.bt / c.at, ctat = c.ct / c.at;
    for (int k = 1; k <= nzm; ++k)
      for (int j = 1; j <= ny; ++j)
        for (int i = 1; i <= nx; ++i) {
          int kc = k + 1, jc = j + 1, ic = i + 1;
          double rdz = 1. / (c.adz(k) * c.dz);
          double rup = c.rhow(kc) / c.rho(k) * rdz;
          double rdn = c.rhow(k) / c.rho(k) * rdz;
          double dta = 1. / c.dt3[c.na - 1] / c.at;
          c.p(i, j, k) = (rdx * (u(ic, j, k) - u(i, j, k)) + rdy * (v(i, jc, k) - v(i, j, k)) +
                          (w(i, j, kc) * rup - w(i, j, k) * rdn)) * dta +
                         (rdx * (dua(ic, j, k) - dua(i, j, k)) + rdy * (dva(i, jc, k) - dva(i, j, k)) +
                          (dwa(i, j, kc) * rup - dwa(i, j, k) * rdn)) +
                         btat * (rdx * (dub(ic, j, k) - dub(i, j, k)) + rdy * (dvb(i, jc, k) - dvb(i, j, k)) +
                                 (dwb(i, j, kc) * rup - dwb(i, j, k) * rdn)) +
                         ctat * (rdx * (duc(ic, j, k) - duc(i, j, k)) + rdy * (dvc(i, jc, k) - dvc(i, j, k)) +
                                 (dwc(i, j, kc) * rup - dwc(i, j, k) * rdn));
          c.p(i, j, k) = c.p(i, j, k) * c.rho(k);
        }
    const int nx2 = nx + 2, ny2 = ny + 2;
    // f(i, j, k), i = 1..nx2, j = 1..ny2 (1-based), level k = 1..nzm
    std::vector<double> f((size_t)nx2 * ny2 * (nzm + 1), 0.0), work((size_t)std::max(nx2, ny2) + 2, 0.0);
    std::vector<double> col((size_t)ny2, 0.0);
    auto F = [&](int i, int j, int k) -> double & { return f[((size_t)k * ny2 + (j - 1)) * nx2 + (i - 1)]; };
    for (int k = 1; k <= nzm; ++k) {
      for (int j = 1; j <= ny; ++j) {
        for (int i = 1; i <= nx; ++i) F(i, j, k) = c.p(i, j, k);
        fft991(&F(1, j, k), work.data(), g.trigxi.data(), g.ifaxi, nx, -1);
      }
      for (int i = 1; i <= nx + 1; ++i) {
        for (int j = 1; j <= ny2; ++j) col[j - 1] = F(i, j, k);
        fft991(col.data(), work.data(), g.trigxj.data(), g.ifaxj, ny, -1);
        for (int j = 1; j <= ny2; ++j) F(i, j, k) = col[j - 1];
      }
    }
    std::vector<double> a(nzm + 1), cc(nzm + 1), alfa(nzm + 1), beta(nzm + 1);
    for (int k = 1; k <= nzm; ++k) {
      a[k] = c.rhow(k) / (c.adz(k) * c.adzw(k) * c.dz * c.dz);
      cc[k] = c.rhow(k + 1) / (c.adz(k) * c.adzw(k + 1) * c.dz * c.dz);
    }
    for (int j = 1; j <= ny2; ++j)
      for (int i = 1; i <= nx + 1; ++i) {
        int jd = (int)(((float)j - 0.1f) / 2.0f);
        int id = (int)(((float)i - 0.1f) / 2.0f);
        double eign = g.eign[(size_t)(j - 1) * g.eign_ni + (i - 1)];
        double b;
        if (id + jd == 0) b = 1. / (eign * c.rho(1) - a[1] - cc[1]);
        else b = 1. / (eign * c.rho(1) - cc[1]);
        alfa[1] = -cc[1] * b;
        beta[1] = F(i, j, 1) * b;
        for (int k = 2; k <= nzm - 1; ++k) {
          double e = 1. / (eign * c.rho(k) - a[k] - cc[k] + a[k] * alfa[k - 1]);
          alfa[k] = -cc[k] * e;
          beta[k] = (F(i, j, k) - a[k] * beta[k - 1]) * e;
        }
        F(i, j, nzm) = (F(i, j, nzm) - a[nzm] * beta[nzm - 1]) / (eign * c.rho(nzm) - a[nzm] + a[nzm] * alfa[nzm - 1]);
        for (int k = nzm - 1; k >= 1; --k) F(i, j, k) = alfa[k] * F(i, j, k + 1) + beta[k];
      }
    for (int k = 1; k <= nzm; ++k) {
      for (int i = 1; i <= nx + 1; ++i) {
        for (int j = 1; j <= ny2; ++j) col[j - 1] = F(i, j, k);
        fft991(col.data(), work.data(), g.trigxj.data(), g.ifaxj, ny, +1);
        for (int j = 1; j <= ny2; ++j) F(i, j, k) = col[j - 1];
      }
      for (int j = 1; j <= ny; ++j) fft991(&F(1, j, k), work.data(), g.trigxi.data(), g.ifaxi, nx, +1);
      for (int j = 0; j <= ny; ++j)
        for (int i = 0; i <= nx; ++i) c.p(i, j, k) = F(i == 0 ? nx : i, j == 0 ? ny : j, k);
    }
    for (int k = 1; k <= nzm; ++k)
      for (int j = 1; j <= ny; ++j)
        for (int i = 1; i <= nx; ++i) {
          int kb = std::max(1, k - 1), jb = j - 1, ib = i - 1;
          double rdz = 1. / (c.dz * c.adzw(k));
          dua(i, j, k) = dua(i, j, k) - (c.p(i, j, k) - c.p(ib, j, k)) * rdx;
          dva(i, j, k) = dva(i, j, k) - (c.p(i, j, k) - c.p(i, jb, k)) * rdy;
          dwa(i, j, k) = dwa(i, j, k) - (c.p(i, j, k) - c.p(i, j, kb)) * rdz;
        }
    for (int k = 1; k <= nzm; ++k)
      for (int j = 0; j <= ny; ++j)
        for (int i = 0; i <= nx; ++i) c.p(i, j, k) = c.p(i, j, k) * c.rho(k);
    bound_duvdt();
  }
  void pressure(Column &c) {
    if (g.YES3D) { pressure3D(c); return; }
    const int nx = g.nx, nzm = g.nzm, j = 1;
    A3 &u = c.u, &w = c.w;
    // bound_duvdt (bound_duvdt.F90): periodic copy of dudt(nxp1, na)
    {
      A3 &du = DU(c, c.na);
      for (int k = 1; k <= nzm; ++k) du(nx + 1, j, k) = du(1, j, k);
    }
    // press_rhs (press_rhs.F90:61-101)
    const double rdx = 1. / g.dx;
    const double btat = c.bt / c.at, ctat = c.ct / c.at;
    A3 &dua = DU(c, c.na), &dub = DU(c, c.nb), &duc = DU(c, c.nc);
    A3 &dwa = DW(c, c.na), &dwb = DW(c, c.nb), &dwc = DW(c, c.nc);
    for (int k = 1; k <= nzm; ++k)
      for (int i = 1; i <= nx; ++i) {
        int kc = k + 1;
        double rdz = 1. / (c.adz(k) * c.dz);
        double rup = c.rhow(kc) / c.rho(k) * rdz;
        double rdn = c.rhow(k) / c.rho(k) * rdz;
        int ic = i + 1;
        double dta = 1. / c.dt3[c.na - 1] / c.at;
        c.p(i, j, k) = (rdx * (u(ic, j, k) - u(i, j, k)) + (w(i, j, kc) * rup - w(i, j, k) * rdn)) * dta +
                       (rdx * (dua(ic, j, k) - dua(i, j, k)) + (dwa(i, j, kc) * rup - dwa(i, j, k) * rdn)) +
                       btat * (rdx * (dub(ic, j, k) - dub(i, j, k)) + (dwb(i, j, kc) * rup - dwb(i, j, k) * rdn)) +
                       ctat * (rdx * (duc(ic, j, k) - duc(i, j, k)) + (dwc(i, j, kc) * rup - dwc(i, j, k) * rdn));
        c.p(i, j, k) = c.p(i, j, k) * c.rho(k);
      }
    // forward FFT of every level, tridiagonal solve per wavenumber, inverse
    const int nx2 = nx + 2;
    std::vector<double> f((size_t)nx2 * (nzm + 1), 0.0), work(nx2 + 2, 0.0);
    for (int k = 1; k <= nzm; ++k) {
      double *fk = &f[(size_t)nx2 * k];
      for (int i = 1; i <= nx; ++i) fk[i - 1] = c.p(i, j, k);
      fft991(fk, work.data(), g.trigxi.data(), g.ifaxi, nx, -1);
    }
    std::vector<double> a(nzm + 1), cc(nzm + 1), alfa(nzm + 1), beta(nzm + 1);
    for (int k = 1; k <= nzm; ++k) {
      a[k] = c.rhow(k) / (c.adz(k) * c.adzw(k) * c.dz * c.dz);
      cc[k] = c.rhow(k + 1) / (c.adz(k) * c.adzw(k + 1) * c.dz * c.dz);
    }
    for (int i = 1; i <= nx + 1; ++i) {
      int id = (int)(((float)i - 0.1f) / 2.0f);
      int jd = 0;
      double eign = g.eign[(size_t)(i - 1)];
      auto FF = [&](int k) -> double & { return f[(size_t)nx2 * k + (i - 1)]; };
      double b;
      if (id + jd == 0) b = 1. / (eign * c.rho(1) - a[1] - cc[1]);
      else b = 1. / (eign * c.rho(1) - cc[1]);
      alfa[1] = -cc[1] * b;
      beta[1] = FF(1) * b;
      for (int k = 2; k <= nzm - 1; ++k) {
        double e = 1. / (eign * c.rho(k) - a[k] - cc[k] + a[k] * alfa[k - 1]);
        alfa[k] = -cc[k] * e;
        beta[k] = (FF(k) - a[k] * beta[k - 1]) * e;
      }
      FF(nzm) = (FF(nzm) - a[nzm] * beta[nzm - 1]) / (eign * c.rho(nzm) - a[nzm] + a[nzm] * alfa[nzm - 1]);
      for (int k = nzm - 1; k >= 1; --k) FF(k) = alfa[k] * FF(k + 1) + beta[k];
    }
    for (int k = 1; k <= nzm; ++k) {
      double *fk = &f[(size_t)nx2 * k];
      fft991(fk, work.data(), g.trigxi.data(), g.ifaxi, nx, +1);
      for (int i = 0; i <= nx; ++i) c.p(i, j, k) = fk[(i == 0 ? nx : i) - 1];
    }
    // press_grad (press_grad.F90:18-72)
    for (int k = 1; k <= nzm; ++k)
      for (int i = 1; i <= nx; ++i) {
        int kb = std::max(1, k - 1);
        double rdz = 1. / (c.dz * c.adzw(k));
        int ib = i - 1;
        dua(i, j, k) = dua(i, j, k) - (c.p(i, j, k) - c.p(ib, j, k)) * rdx;
        DV(c, c.na)(i, j, k) = DV(c, c.na)(i, j, k) - (c.p(i, j, k) - c.p(i, j, k)) * (1. / g.dy);
        dwa(i, j, k) = dwa(i, j, k) - (c.p(i, j, k) - c.p(i, j, kb)) * rdz;
      }
    for (int k = 1; k <= nzm; ++k)
      for (int i = 0; i <= nx; ++i) c.p(i, j, k) = c.p(i, j, k) * c.rho(k);
    for (int k = 1; k <= nzm; ++k) dua(nx + 1, j, k) = dua(1, j, k);
  }

  // ---- adams.F90:17-38
  void adams(Column &c) {
    const double dtdx = c.dtn / g.dx;
    const double dtdy = c.dtn / g.dy;
    A3 &dua = DU(c, c.na), &dub = DU(c, c.nb), &duc = DU(c, c.nc);
    A3 &dva = DV(c, c.na), &dvb = DV(c, c.nb), &dvc = DV(c, c.nc);
    A3 &dwa = DW(c, c.na), &dwb = DW(c, c.nb), &dwc = DW(c, c.nc);
    const double d3 = c.dt3[c.na - 1];
    for (int k = 1; k <= g.nzm; ++k)
      for (int j = 1; j <= g.ny; ++j)
        for (int i = 1; i <= g.nx; ++i) {
          double dtdz = c.dtn / c.dz;
          double rhox = c.rho(k) * dtdx;
          double rhoy = c.rho(k) * dtdy;
          double rhoz = c.rhow(k) * dtdz;
          duc(i, j, k) = c.u(i, j, k) + d3 * (c.at * dua(i, j, k) + c.bt * dub(i, j, k) + c.ct * duc(i, j, k));
          dvc(i, j, k) = c.v(i, j, k) + d3 * (c.at * dva(i, j, k) + c.bt * dvb(i, j, k) + c.ct * dvc(i, j, k));
          dwc(i, j, k) = c.w(i, j, k) + d3 * (c.at * dwa(i, j, k) + c.bt * dwb(i, j, k) + c.ct * dwc(i, j, k));
          c.u(i, j, k) = 0.5 * (c.u(i, j, k) + duc(i, j, k)) * rhox;
          c.v(i, j, k) = 0.5 * (c.v(i, j, k) + dvc(i, j, k)) * rhoy;
          c.w(i, j, k) = 0.5 * (c.w(i, j, k) + dwc(i, j, k)) * rhoz;
        }
  }
  // ---- uvw.F90
  void uvw(Column &c) {
    A3 &duc = DU(c, c.nc), &dvc = DV(c, c.nc), &dwc = DW(c, c.nc);
    for (int k = 1; k <= g.nzm; ++k)
      for (int j = 1; j <= g.ny; ++j)
        for (int i = 1; i <= g.nx; ++i) {
          c.u(i, j, k) = duc(i, j, k);
          c.v(i, j, k) = dvc(i, j, k);
          c.w(i, j, k) = dwc(i, j, k);
        }
  }

  // ---- advect_scalar.F90:9-76 + ADV_MPDATA/advect_scalar2D.F90:8-244
  // ADV_MPDATA/advect_scalar3D.F90:8-349 (nonos, no walls), with the
  // advect_scalar.F90 wrapper's fadv (horizontal sum of the change)
  void advect_scalar3D(Column &c, A3 &f, A1 *fadv, A1 *flux) {
    const int nx = g.nx, ny = g.ny, nzm = g.nzm, nz = g.nz;
    A3 &u = c.u, &v = c.v, &w = c.w;
    std::vector<double> f0;
    if (fadv) {
      f0.resize((size_t)(nx + 1) * (ny + 1) * (nzm + 1));
      for (int k = 1; k <= nzm; ++k)
        for (int j = 1; j <= ny; ++j)
          for (int i = 1; i <= nx; ++i) f0[((size_t)k * (ny + 1) + j) * (nx + 1) + i] = f(i, j, k);
    }
    A3 mx, mn, uuu, vvv, www;
    mx.init(0, nx + 1, 0, ny + 1, 1, nzm);
    mn.init(0, nx + 1, 0, ny + 1, 1, nzm);
    uuu.init(-1, nx + 3, -1, ny + 2, 1, nzm);
    vvv.init(-1, nx + 2, -1, ny + 3, 1, nzm);
    www.init(-1, nx + 2, -1, ny + 2, 1, nz);
    std::vector<double> iadz(nzm + 1), irho(nzm + 1), irhow(nzm + 1), fl(nz + 1, 0.0);
    const double eps = R4(1.e-10);
    auto andiff = [](double x1, double x2, double a, double b) { return (fabs(a) - a * a * b) * 0.5 * (x2 - x1); };
    auto across = [](double x1, double a1, double a2) { return 0.03125 * a1 * a2 * x1; };
    auto pp = [](double y) { return fmax2(0., y); };
    auto pn = [](double y) { return -fmin2(0., y); };
    auto max7 = [](double a, double b, double c_, double d, double e, double f_, double g_) {
      return fmax2(fmax2(fmax2(fmax2(fmax2(fmax2(a, b), c_), d), e), f_), g_);
    };
    auto min7 = [](double a, double b, double c_, double d, double e, double f_, double g_) {
      return fmin2(fmin2(fmin2(fmin2(fmin2(fmin2(a, b), c_), d), e), f_), g_);
    };
    for (int j = -1; j <= ny + 2; ++j)
      for (int i = -1; i <= nx + 2; ++i) www(i, j, nz) = 0.;
    for (int k = 1; k <= nzm; ++k)
      for (int j = 0; j <= ny + 1; ++j)
        for (int i = 0; i <= nx + 1; ++i) {
          int kc = std::min(nzm, k + 1), kb = std::max(1, k - 1);
          mx(i, j, k) = max7(f(i - 1, j, k), f(i + 1, j, k), f(i, j - 1, k), f(i, j + 1, k), f(i, j, kb), f(i, j, kc), f(i, j, k));
          mn(i, j, k) = min7(f(i - 1, j, k), f(i + 1, j, k), f(i, j - 1, k), f(i, j + 1, k), f(i, j, kb), f(i, j, kc), f(i, j, k));
        }
    for (int k = 1; k <= nzm; ++k)
      for (int j = -1; j <= ny + 3; ++j)
        for (int i = -1; i <= nx + 3; ++i) {
          int kb = std::max(1, k - 1);
          if (j <= ny + 2) uuu(i, j, k) = fmax2(0., u(i, j, k)) * f(i - 1, j, k) + fmin2(0., u(i, j, k)) * f(i, j, k);
          if (i <= nx + 2) vvv(i, j, k) = fmax2(0., v(i, j, k)) * f(i, j - 1, k) + fmin2(0., v(i, j, k)) * f(i, j, k);
          if (i <= nx + 2 && j <= ny + 2)
            www(i, j, k) = fmax2(0., w(i, j, k)) * f(i, j, kb) + fmin2(0., w(i, j, k)) * f(i, j, k);
          if (i == -1 && j == -1) fl[k] = 0.;
        }
    for (int k = 1; k <= nzm; ++k) {
      irho[k] = 1. / c.rho(k);
      iadz[k] = 1. / c.adz(k);
      irhow[k] = 1. / (c.rhow(k) * c.adz(k));
    }
    for (int k = 1; k <= nzm; ++k)
      for (int j = -1; j <= ny + 2; ++j)
        for (int i = -1; i <= nx + 2; ++i) {
          if (i >= 1 && i <= nx && j >= 1 && j <= ny) fl[k] = fl[k] + www(i, j, k);
          f(i, j, k) = f(i, j, k) - (uuu(i + 1, j, k) - uuu(i, j, k) + vvv(i, j + 1, k) - vvv(i, j, k) +
                                     (www(i, j, k + 1) - www(i, j, k)) * iadz[k]) * irho[k];
        }
    for (int k = 1; k <= nzm; ++k)
      for (int j = 0; j <= ny + 2; ++j)
        for (int i = 0; i <= nx + 2; ++i) {
          int kc = std::min(nzm, k + 1), kb = std::max(1, k - 1);
          double dd = (double)(2.f / (float)(kc - kb)) / c.adz(k);
          int jb = j - 1, jc = j + 1, ib = i - 1, ic = i + 1;
          if (j <= ny + 1)
            uuu(i, j, k) = andiff(f(ib, j, k), f(i, j, k), u(i, j, k), irho[k]) -
                           (across(f(ib, jc, k) + f(i, jc, k) - f(ib, jb, k) - f(i, jb, k), u(i, j, k),
                                   v(ib, j, k) + v(ib, jc, k) + v(i, jc, k) + v(i, j, k)) +
                            across(dd * (f(ib, j, kc) + f(i, j, kc) - f(ib, j, kb) - f(i, j, kb)), u(i, j, k),
                                   w(ib, j, k) + w(ib, j, kc) + w(i, j, k) + w(i, j, kc))) * irho[k];
          if (i <= nx + 1)
            vvv(i, j, k) = andiff(f(i, jb, k), f(i, j, k), v(i, j, k), irho[k]) -
                           (across(f(ic, jb, k) + f(ic, j, k) - f(ib, jb, k) - f(ib, j, k), v(i, j, k),
                                   u(i, jb, k) + u(i, j, k) + u(ic, j, k) + u(ic, jb, k)) +
                            across(dd * (f(i, jb, kc) + f(i, j, kc) - f(i, jb, kb) - f(i, j, kb)), v(i, j, k),
                                   w(i, jb, k) + w(i, j, k) + w(i, j, kc) + w(i, jb, kc))) * irho[k];
          if (i <= nx + 1 && j <= ny + 1)
            www(i, j, k) = andiff(f(i, j, kb), f(i, j, k), w(i, j, k), irhow[k]) -
                           (across(f(ic, j, kb) + f(ic, j, k) - f(ib, j, kb) - f(ib, j, k), w(i, j, k),
                                   u(i, j, kb) + u(i, j, k) + u(ic, j, k) + u(ic, j, kb)) +
                            across(f(i, jc, k) + f(i, jc, kb) - f(i, jb, k) - f(i, jb, kb), w(i, j, k),
                                   v(i, j, kb) + v(i, jc, kb) + v(i, jc, k) + v(i, j, k))) * irho[k];
        }
    for (int j = -1; j <= ny + 2; ++j)
      for (int i = -1; i <= nx + 2; ++i) www(i, j, 1) = 0.;
    for (int k = 1; k <= nzm; ++k)
      for (int j = 0; j <= ny + 1; ++j)
        for (int i = 0; i <= nx + 1; ++i) {
          int kc = std::min(nzm, k + 1), kb = std::max(1, k - 1);
          mx(i, j, k) = fmax2(max7(f(i - 1, j, k), f(i + 1, j, k), f(i, j - 1, k), f(i, j + 1, k), f(i, j, kb), f(i, j, kc), f(i, j, k)), mx(i, j, k));
          mn(i, j, k) = fmin2(min7(f(i - 1, j, k), f(i + 1, j, k), f(i, j - 1, k), f(i, j + 1, k), f(i, j, kb), f(i, j, kc), f(i, j, k)), mn(i, j, k));
        }
    for (int k = 1; k <= nzm; ++k)
      for (int j = 0; j <= ny + 1; ++j)
        for (int i = 0; i <= nx + 1; ++i) {
          int kc = std::min(nzm, k + 1), jc = j + 1, ic = i + 1;
          mx(i, j, k) = c.rho(k) * (mx(i, j, k) - f(i, j, k)) /
                        (pn(uuu(ic, j, k)) + pp(uuu(i, j, k)) + pn(vvv(i, jc, k)) + pp(vvv(i, j, k)) +
                         (pn(www(i, j, kc)) + pp(www(i, j, k))) * iadz[k] + eps);
          mn(i, j, k) = c.rho(k) * (f(i, j, k) - mn(i, j, k)) /
                        (pp(uuu(ic, j, k)) + pn(uuu(i, j, k)) + pp(vvv(i, jc, k)) + pn(vvv(i, j, k)) +
                         (pp(www(i, j, kc)) + pn(www(i, j, k))) * iadz[k] + eps);
        }
    for (int k = 1; k <= nzm; ++k)
      for (int j = 1; j <= ny + 1; ++j)
        for (int i = 1; i <= nx + 1; ++i) {
          if (j <= ny) {
            int ib = i - 1;
            uuu(i, j, k) = pp(uuu(i, j, k)) * fmin3(1., mx(i, j, k), mn(ib, j, k)) -
                           pn(uuu(i, j, k)) * fmin3(1., mx(ib, j, k), mn(i, j, k));
          }
          if (i <= nx) {
            int jb = j - 1;
            vvv(i, j, k) = pp(vvv(i, j, k)) * fmin3(1., mx(i, j, k), mn(i, jb, k)) -
                           pn(vvv(i, j, k)) * fmin3(1., mx(i, jb, k), mn(i, j, k));
          }
          if (i <= nx && j <= ny) {
            int kb = std::max(1, k - 1);
            www(i, j, k) = pp(www(i, j, k)) * fmin3(1., mx(i, j, k), mn(i, j, kb)) -
                           pn(www(i, j, k)) * fmin3(1., mx(i, j, kb), mn(i, j, k));
            fl[k] = fl[k] + www(i, j, k);
          }
        }
    for (int k = 1; k <= nzm; ++k)
      for (int j = 1; j <= ny; ++j)
        for (int i = 1; i <= nx; ++i)
          f(i, j, k) = fmax2(0., f(i, j, k) - (uuu(i + 1, j, k) - uuu(i, j, k) + vvv(i, j + 1, k) - vvv(i, j, k) +
                                               (www(i, j, k + 1) - www(i, j, k)) * iadz[k]) * irho[k]);
    if (flux)
      for (int k = 1; k <= nzm; ++k) (*flux)(k) = fl[k];
    if (fadv)
      for (int k = 1; k <= nzm; ++k) {
        double s_ = 0.;
        for (int j = 1; j <= ny; ++j)
          for (int i = 1; i <= nx; ++i) s_ = s_ + (f(i, j, k) - f0[((size_t)k * (ny + 1) + j) * (nx + 1) + i]);
        (*fadv)(k) = s_;
      }
  }
  void advect_scalar2D(Column &c, A3 &f, A1 *fadv, A1 *flux) {
    const int nx = g.nx, nzm = g.nzm, nz = g.nz, j = 1;
    A3 &u = c.u, &w = c.w;
    std::vector<double> f0;
    if (fadv) {
      f0.resize((size_t)(nx + 1) * (nzm + 1));
      for (int k = 1; k <= nzm; ++k)
        for (int i = 1; i <= nx; ++i) f0[(size_t)k * (nx + 1) + i] = f(i, j, k);
    }
    A3 mx, mn, uuu, www;
    mx.init(0, nx + 1, 1, 1, 1, nzm);
    mn.init(0, nx + 1, 1, 1, 1, nzm);
    uuu.init(-1, nx + 3, 1, 1, 1, nzm);
    www.init(-1, nx + 2, 1, 1, 1, nz);
    std::vector<double> iadz(nzm + 1), irho(nzm + 1), irhow(nzm + 1), fl(nz + 1, 0.0);
    const double eps = R4(1.e-10);
    auto andiff = [](double x1, double x2, double a, double b) { return (fabs(a) - a * a * b) * 0.5 * (x2 - x1); };
    auto across = [](double x1, double a1, double a2) { return 0.03125 * a1 * a2 * x1; };
    auto pp = [](double y) { return fmax2(0., y); };
    auto pn = [](double y) { return -fmin2(0., y); };
    for (int i = -1; i <= nx + 2; ++i) www(i, j, nz) = 0.;
    for (int k = 1; k <= nzm; ++k)
      for (int i = 0; i <= nx + 1; ++i) {
        int kc = std::min(nzm, k + 1), kb = std::max(1, k - 1), ib = i - 1, ic = i + 1;
        mx(i, j, k) = fmax2(fmax2(fmax2(fmax2(f(ib, j, k), f(ic, j, k)), f(i, j, kb)), f(i, j, kc)), f(i, j, k));
        mn(i, j, k) = fmin2(fmin2(fmin2(fmin2(f(ib, j, k), f(ic, j, k)), f(i, j, kb)), f(i, j, kc)), f(i, j, k));
      }
    for (int k = 1; k <= nzm; ++k)
      for (int i = -1; i <= nx + 3; ++i) {
        int kb = std::max(1, k - 1);
        uuu(i, j, k) = fmax2(0., u(i, j, k)) * f(i - 1, j, k) + fmin2(0., u(i, j, k)) * f(i, j, k);
        if (i <= nx + 2) www(i, j, k) = fmax2(0., w(i, j, k)) * f(i, j, kb) + fmin2(0., w(i, j, k)) * f(i, j, k);
        if (i == 0) fl[k] = 0.;
      }
    for (int k = 1; k <= nzm; ++k) {
      irho[k] = 1. / c.rho(k);
      iadz[k] = 1. / c.adz(k);
      irhow[k] = 1. / (c.rhow(k) * c.adz(k));
    }
    for (int k = 1; k <= nzm; ++k)
      for (int i = -1; i <= nx + 2; ++i) {
        if (i >= 1 && i <= nx) fl[k] = fl[k] + www(i, j, k);
        f(i, j, k) = f(i, j, k) - (uuu(i + 1, j, k) - uuu(i, j, k) + (www(i, j, k + 1) - www(i, j, k)) * iadz[k]) * irho[k];
      }
    for (int k = 1; k <= nzm; ++k)
      for (int i = 0; i <= nx + 2; ++i) {
        int kc = std::min(nzm, k + 1), kb = std::max(1, k - 1);
        double dd = (double)(2.f / (float)(kc - kb)) / c.adz(k);
        int ib = i - 1;
        uuu(i, j, k) = andiff(f(ib, j, k), f(i, j, k), u(i, j, k), irho[k]) -
                       across(dd * (f(ib, j, kc) + f(i, j, kc) - f(ib, j, kb) - f(i, j, kb)), u(i, j, k),
                              w(ib, j, k) + w(ib, j, kc) + w(i, j, k) + w(i, j, kc)) * irho[k];
        if (i <= nx + 1) {
          int ic = i + 1;
          www(i, j, k) = andiff(f(i, j, kb), f(i, j, k), w(i, j, k), irhow[k]) -
                         across(f(ic, j, kb) + f(ic, j, k) - f(ib, j, kb) - f(ib, j, k), w(i, j, k),
                                u(i, j, kb) + u(i, j, k) + u(ic, j, k) + u(ic, j, kb)) * irho[k];
        }
      }
    for (int i = -1; i <= nx + 2; ++i) www(i, j, 1) = 0.;
    for (int k = 1; k <= nzm; ++k)
      for (int i = 0; i <= nx + 1; ++i) {
        int kc = std::min(nzm, k + 1), kb = std::max(1, k - 1), ib = i - 1, ic = i + 1;
        mx(i, j, k) = fmax2(fmax2(fmax2(fmax2(fmax2(f(ib, j, k), f(ic, j, k)), f(i, j, kb)), f(i, j, kc)), f(i, j, k)), mx(i, j, k));
        mn(i, j, k) = fmin2(fmin2(fmin2(fmin2(fmin2(f(ib, j, k), f(ic, j, k)), f(i, j, kb)), f(i, j, kc)), f(i, j, k)), mn(i, j, k));
      }
    for (int k = 1; k <= nzm; ++k)
      for (int i = 0; i <= nx + 1; ++i) {
        int kc = std::min(nzm, k + 1), ic = i + 1;
        mx(i, j, k) = c.rho(k) * (mx(i, j, k) - f(i, j, k)) /
                      (pn(uuu(ic, j, k)) + pp(uuu(i, j, k)) + iadz[k] * (pn(www(i, j, kc)) + pp(www(i, j, k))) + eps);
        mn(i, j, k) = c.rho(k) * (f(i, j, k) - mn(i, j, k)) /
                      (pp(uuu(ic, j, k)) + pn(uuu(i, j, k)) + iadz[k] * (pp(www(i, j, kc)) + pn(www(i, j, k))) + eps);
      }
    for (int k = 1; k <= nzm; ++k)
      for (int i = 1; i <= nx + 1; ++i) {
        int ib = i - 1;
        uuu(i, j, k) = pp(uuu(i, j, k)) * fmin3(1., mx(i, j, k), mn(ib, j, k)) -
                       pn(uuu(i, j, k)) * fmin3(1., mx(ib, j, k), mn(i, j, k));
        if (i <= nx) {
          int kb = std::max(1, k - 1);
          www(i, j, k) = pp(www(i, j, k)) * fmin3(1., mx(i, j, k), mn(i, j, kb)) -
                         pn(www(i, j, k)) * fmin3(1., mx(i, j, kb), mn(i, j, k));
          fl[k] = fl[k] + www(i, j, k);
        }
      }
    for (int k = 1; k <= nzm; ++k)
      for (int i = 1; i <= nx; ++i)
        f(i, j, k) = fmax2(0., f(i, j, k) - (uuu(i + 1, j, k) - uuu(i, j, k) + (www(i, j, k + 1) - www(i, j, k)) * iadz[k]) * irho[k]);
    if (flux)
      for (int k = 1; k <= nzm; ++k) (*flux)(k) = fl[k];
    if (fadv) {
      for (int k = 1; k <= nzm; ++k) {
        double s = 0.;
        for (int i = 1; i <= nx; ++i) s = s + (f(i, j, k) - f0[(size_t)k * (nx + 1) + i]);
        (*fadv)(k) = s;
      }
    }
  }

  // ---- term_vel_qp (MICRO_SAM1MOM/microphysics.F90:453-486)
  double term_vel(Column &c, int i, int j, int k, double qploc) {
    double term_vel = 0.;
    if (qploc > qp_threshold) {
      double omp = fmax2(0., fmin2(1., (c.tabs(i, j, k) - tprmin) * g.a_pr));
      if (omp == 1.) {
        term_vel = g.vrain * det_pow(c.rho(k) * qploc, g.crain);
      } else if (omp == 0.) {
        double omg = fmax2(0., fmin2(1., (c.tabs(i, j, k) - tgrmin) * g.a_gr));
        double qgg = omg * qploc;
        double qss = qploc - qgg;
        term_vel = omg * g.vgrau * det_pow(c.rho(k) * qgg, g.cgrau) + (1. - omg) * g.vsnow * det_pow(c.rho(k) * qss, g.csnow);
      } else {
        double omg = fmax2(0., fmin2(1., (c.tabs(i, j, k) - tgrmin) * g.a_gr));
        double qrr = omp * qploc;
        double qss = qploc - qrr;
        double qgg = omg * qss;
        qss = qss - qgg;
        term_vel = omp * g.vrain * det_pow(c.rho(k) * qrr, g.crain) +
                   (1. - omp) * (omg * g.vgrau * det_pow(c.rho(k) * qgg, g.cgrau) +
                                 (1. - omg) * g.vsnow * det_pow(c.rho(k) * qss, g.csnow));
      }
    }
    return term_vel;
  }

  // ---- micro_precip_fall / precip_fall (microphysics.F90:491-833)
  // Part 1: terminal velocities and the column CFL; part 2 (after nprec is
  // known, per column or as a batch maximum) the sedimentation sub-steps.
  struct FallScratch {
    A3 mx, mn, lfac, www, fz, wp, tmp_qp, omega;
    std::vector<double> irhoadz, iwmax, rhofac;
  };
  void precip_fall_part1(Column &c, FallScratch &s) {
    const int nx = g.nx, ny = g.ny, nzm = g.nzm, nz = g.nz;
    s.omega.init(1, nx, 1, ny, 1, nzm);
    s.mx.init(1, nx, 1, ny, 1, nzm); s.mn.init(1, nx, 1, ny, 1, nzm);
    s.lfac.init(1, nx, 1, ny, 1, nz); s.www.init(1, nx, 1, ny, 1, nz);
    s.fz.init(1, nx, 1, ny, 1, nz); s.wp.init(1, nx, 1, ny, 1, nzm);
    s.tmp_qp.init(1, nx, 1, ny, 1, nzm);
    s.irhoadz.assign(nzm + 1, 0.); s.iwmax.assign(nzm + 1, 0.); s.rhofac.assign(nzm + 1, 0.);
    for (int k = 1; k <= nzm; ++k)
      for (int j = 1; j <= ny; ++j)
        for (int i = 1; i <= nx; ++i)
          s.omega(i, j, k) = fmax2(0., fmin2(1., (c.tabs(i, j, k) - tprmin) * g.a_pr));
    for (int k = 1; k <= nzm; ++k) {
      s.rhofac[k] = sqrt(R4(1.29) / c.rho(k));
      s.irhoadz[k] = 1. / (c.rho(k) * c.adz(k));
      int kb = std::max(1, k - 1);
      double wmax = c.dz * c.adz(kb) / c.dtn;
      s.iwmax[k] = 1. / wmax;
    }
    double prec_cfl = 0.;
    for (int k = 1; k <= nzm; ++k)
      for (int j = 1; j <= ny; ++j)
        for (int i = 1; i <= nx; ++i) {
          s.lfac(i, j, k) = fac_cond + (1 - s.omega(i, j, k)) * fac_fus;
          double tmp = term_vel(c, i, j, k, c.qp(i, j, k));
          s.wp(i, j, k) = s.rhofac[k] * tmp;
          tmp = s.wp(i, j, k) * s.iwmax[k];
          prec_cfl = fmax2(prec_cfl, tmp);
          s.wp(i, j, k) = -s.wp(i, j, k) * c.rhow(k) * c.dtn / c.dz;
          if (k == 1) { s.fz(i, j, nz) = 0.; s.www(i, j, nz) = 0.; s.lfac(i, j, nz) = 0; }
        }
    c.prec_cfl = prec_cfl;
  }
  // nprec = ceil(cfl / 0.9) (microphysics.F90:602-661), saturated at 10^4
  // sub-steps so that garbage fall speeds cannot make the loop unbounded
  static int nprec_of(double prec_cfl) {
    if (!(prec_cfl > R4(0.9))) return 1;
    double n = std::ceil(prec_cfl / R4(0.9));
    return n < 1.0e4 ? (int)n : 10000;
  }
  void precip_fall_part2(Column &c, FallScratch &s, int nprec) {
    const int nx = g.nx, ny = g.ny, nzm = g.nzm, nz = g.nz;
    const double eps = R4(1.e-10);
    const double flagstat = 1.;
    auto pp = [](double y) { return fmax2(0., y); };
    auto pn = [](double y) { return -fmin2(0., y); };
    if (nprec > 1)
      for (int k = 1; k <= nzm; ++k)
        for (int j = 1; j <= ny; ++j)
          for (int i = 1; i <= nx; ++i) s.wp(i, j, k) = s.wp(i, j, k) / (double)nprec;
    for (int iprec = 1; iprec <= nprec; ++iprec) {
      for (int k = 1; k <= nzm; ++k)
        for (int j = 1; j <= ny; ++j)
          for (int i = 1; i <= nx; ++i) s.tmp_qp(i, j, k) = c.qp(i, j, k);
      for (int k = 1; k <= nzm; ++k)
        for (int j = 1; j <= ny; ++j)
          for (int i = 1; i <= nx; ++i) {
            int kc = std::min(nzm, k + 1), kb = std::max(1, k - 1);
            s.mx(i, j, k) = fmax3(s.tmp_qp(i, j, kb), s.tmp_qp(i, j, kc), s.tmp_qp(i, j, k));
            s.mn(i, j, k) = fmin3(s.tmp_qp(i, j, kb), s.tmp_qp(i, j, kc), s.tmp_qp(i, j, k));
            s.fz(i, j, k) = s.tmp_qp(i, j, k) * s.wp(i, j, k);
          }
      for (int k = 1; k <= nzm; ++k)
        for (int j = 1; j <= ny; ++j)
          for (int i = 1; i <= nx; ++i)
            s.tmp_qp(i, j, k) = s.tmp_qp(i, j, k) - (s.fz(i, j, k + 1) - s.fz(i, j, k)) * s.irhoadz[k];
      for (int k = 1; k <= nzm; ++k)
        for (int j = 1; j <= ny; ++j)
          for (int i = 1; i <= nx; ++i) {
            int kb = std::max(1, k - 1);
            s.www(i, j, k) = 0.5 * (1. + s.wp(i, j, k) * s.irhoadz[k]) *
                             (s.tmp_qp(i, j, kb) * s.wp(i, j, kb) - s.tmp_qp(i, j, k) * s.wp(i, j, k));
          }
      for (int k = 1; k <= nzm; ++k)
        for (int j = 1; j <= ny; ++j)
          for (int i = 1; i <= nx; ++i) {
            int kc = std::min(nzm, k + 1), kb = std::max(1, k - 1);
            s.mx(i, j, k) = fmax2(fmax3(s.tmp_qp(i, j, kb), s.tmp_qp(i, j, kc), s.tmp_qp(i, j, k)), s.mx(i, j, k));
            s.mn(i, j, k) = fmin2(fmin3(s.tmp_qp(i, j, kb), s.tmp_qp(i, j, kc), s.tmp_qp(i, j, k)), s.mn(i, j, k));
            s.mx(i, j, k) = c.rho(k) * c.adz(k) * (s.mx(i, j, k) - s.tmp_qp(i, j, k)) /
                            (pn(s.www(i, j, kc)) + pp(s.www(i, j, k)) + eps);
            s.mn(i, j, k) = c.rho(k) * c.adz(k) * (s.tmp_qp(i, j, k) - s.mn(i, j, k)) /
                            (pp(s.www(i, j, kc)) + pn(s.www(i, j, k)) + eps);
          }
      for (int k = 1; k <= nzm; ++k)
        for (int j = 1; j <= ny; ++j)
          for (int i = 1; i <= nx; ++i) {
            int kb = std::max(1, k - 1);
            s.fz(i, j, k) = s.fz(i, j, k) + pp(s.www(i, j, k)) * fmin3(1., s.mx(i, j, k), s.mn(i, j, kb)) -
                            pn(s.www(i, j, k)) * fmin3(1., s.mx(i, j, kb), s.mn(i, j, k));
          }
      for (int j = 1; j <= ny; ++j)
        for (int i = 1; i <= nx; ++i)
          for (int k = 1; k <= nzm; ++k) {
            int kc = k + 1;
            c.qp(i, j, k) = c.qp(i, j, k) - (s.fz(i, j, kc) - s.fz(i, j, k)) * s.irhoadz[k];
            double tmp = -(s.fz(i, j, kc) - s.fz(i, j, k)) * s.irhoadz[k] * flagstat;
            c.qpfall(k) = c.qpfall(k) + tmp;
            double lat_heat = -(s.lfac(i, j, kc) * s.fz(i, j, kc) - s.lfac(i, j, k) * s.fz(i, j, k)) * s.irhoadz[k];
            c.t(i, j, k) = c.t(i, j, k) - lat_heat;
            c.tlat(k) = c.tlat(k) - lat_heat;
            tmp = s.fz(i, j, k) * flagstat;
            c.precflux(k) = c.precflux(k) - tmp;
            if (k == 1) {
              c.precsfc(i, j, 1) = c.precsfc(i, j, 1) - s.fz(i, j, 1) * flagstat;
              c.precssfc(i, j, 1) = c.precssfc(i, j, 1) - s.fz(i, j, 1) * (1. - s.omega(i, j, 1)) * flagstat;
            }
          }
      if (iprec < nprec)
        for (int j = 1; j <= ny; ++j)
          for (int i = 1; i <= nx; ++i)
            for (int k = 1; k <= nzm; ++k) {
              double tmp = term_vel(c, i, j, k, c.qp(i, j, k));
              s.wp(i, j, k) = s.rhofac[k] * tmp;
              s.wp(i, j, k) = -s.wp(i, j, k) * c.rhow(k) * c.dtn / c.dz / (double)nprec;
              if (k == 1) { s.fz(i, j, nz) = 0.; s.www(i, j, nz) = 0.; s.lfac(i, j, nz) = 0.; }
            }
    }
  }

  // ---- diffuse_scalar.F90:6-72 + diffuse_scalar2D.F90:6-140
  // SGS_TKE/diffuse_scalar3D.F90:6-218 (fluxb = fluxt = 0, no walls), with
  // the sgs_scalars wrapper's fdiff (horizontal sum of the change)
  void diffuse_scalar3D(Column &c, A3 &f, A1 *fdiff, A1 *flux) {
    const int nx = g.nx, ny = g.ny, nzm = g.nzm, nz = g.nz;
    std::vector<double> df;
    if (fdiff) {
      df.resize((size_t)(nx + 1) * (ny + 1) * (nzm + 1));
      for (int k = 1; k <= nzm; ++k)
        for (int j = 1; j <= ny; ++j)
          for (int i = 1; i <= nx; ++i) df[((size_t)k * (ny + 1) + j) * (nx + 1) + i] = f(i, j, k);
    }
    const double rdx2 = 1. / (g.dx * g.dx), rdy2 = 1. / (g.dy * g.dy);
    A3 flx_x, flx_y, flx_z, dfdt;
    flx_x.init(0, nx, 0, ny, 1, nzm);
    flx_y.init(0, nx, 0, ny, 1, nzm);
    flx_z.init(1, nx, 1, ny, 0, nzm);
    dfdt.init(1, nx, 1, ny, 1, nzm);
    A3 &tkh = c.tkh;
    for (int k = 1; k <= nzm; ++k)
      for (int j = 0; j <= ny; ++j)
        for (int i = 0; i <= nx; ++i) {
          if (j >= 1) {
            int ic = i + 1;
            double rdx5 = 0.5 * rdx2 * c.grdf_x(k);
            double tkx = rdx5 * (tkh(i, j, k) + tkh(ic, j, k));
            flx_x(i, j, k) = -tkx * (f(ic, j, k) - f(i, j, k));
          }
          if (i >= 1) {
            int jc = j + 1;
            double rdy5 = 0.5 * rdy2 * c.grdf_y(k);
            double tky = rdy5 * (tkh(i, j, k) + tkh(i, jc, k));
            flx_y(i, j, k) = -tky * (f(i, jc, k) - f(i, j, k));
          }
        }
    for (int k = 1; k <= nzm; ++k)
      for (int j = 1; j <= ny; ++j)
        for (int i = 1; i <= nx; ++i) {
          dfdt(i, j, k) = dfdt(i, j, k) - (flx_x(i, j, k) - flx_x(i - 1, j, k));
          dfdt(i, j, k) = dfdt(i, j, k) - (flx_y(i, j, k) - flx_y(i, j - 1, k));
        }
    std::vector<double> fl(nz + 1, 0.0);
    for (int k = 1; k <= nzm; ++k)
      for (int j = 1; j <= ny; ++j)
        for (int i = 1; i <= nx; ++i) {
          if (k <= nzm - 1) {
            int kc = k + 1;
            double rhoi = c.rhow(kc) / c.adzw(kc);
            double rdz2 = 1. / (c.dz * c.dz);
            double rdz5 = 0.5 * rdz2 * c.grdf_z(k);
            double tkz = rdz5 * (tkh(i, j, k) + tkh(i, j, kc));
            flx_z(i, j, k) = -tkz * (f(i, j, kc) - f(i, j, k)) * rhoi;
            fl[kc] = fl[kc] + flx_z(i, j, k);
          } else {
            double tmp = 1. / c.adzw(nz);
            double rdz = 1. / c.dz;
            flx_z(i, j, 0) = 0.0 * rdz * c.rhow(1);
            flx_z(i, j, nzm) = 0.0 * rdz * tmp * c.rhow(nz);
            fl[1] = fl[1] + flx_z(i, j, 0);
          }
        }
    for (int k = 1; k <= nzm; ++k)
      for (int j = 1; j <= ny; ++j)
        for (int i = 1; i <= nx; ++i) {
          int kb = k - 1;
          double rhoi = 1. / (c.adz(k) * c.rho(k));
          dfdt(i, j, k) = c.dtn * (dfdt(i, j, k) - (flx_z(i, j, k) - flx_z(i, j, kb)) * rhoi);
          f(i, j, k) = f(i, j, k) + dfdt(i, j, k);
        }
    if (flux)
      for (int k = 1; k <= nzm; ++k) (*flux)(k) = fl[k];
    if (fdiff)
      for (int k = 1; k <= nzm; ++k) {
        double s_ = 0.;
        for (int j = 1; j <= ny; ++j)
          for (int i = 1; i <= nx; ++i) s_ = s_ + (f(i, j, k) - df[((size_t)k * (ny + 1) + j) * (nx + 1) + i]);
        (*fdiff)(k) = s_;
      }
  }
  void diffuse_scalar2D(Column &c, A3 &f, A1 *fdiff, A1 *flux) {
    const int nx = g.nx, nzm = g.nzm, nz = g.nz, j = 1;
    std::vector<double> df;
    if (fdiff) {
      df.resize((size_t)(nx + 1) * (nzm + 1));
      for (int k = 1; k <= nzm; ++k)
        for (int i = 1; i <= nx; ++i) df[(size_t)k * (nx + 1) + i] = f(i, j, k);
    }
    const double rdx2 = 1. / (g.dx * g.dx);
    A3 flx, dfdt;
    flx.init(0, nx, 1, 1, 0, nzm);
    dfdt.init(1, nx, 1, 1, 1, nzm);
    A3 &tkh = c.tkh;
    for (int k = 1; k <= nzm; ++k)
      for (int i = 0; i <= nx; ++i) {
        double rdx5 = 0.5 * rdx2 * c.grdf_x(k);
        int ic = i + 1;
        double tkx = rdx5 * (tkh(i, j, k) + tkh(ic, j, k));
        flx(i, j, k) = -tkx * (f(ic, j, k) - f(i, j, k));
      }
    for (int k = 1; k <= nzm; ++k)
      for (int i = 1; i <= nx; ++i) dfdt(i, j, k) = dfdt(i, j, k) - (flx(i, j, k) - flx(i - 1, j, k));
    std::vector<double> fl(nz + 1, 0.0);
    for (int k = 1; k <= nzm; ++k)
      for (int i = 1; i <= nx; ++i) {
        if (k <= nzm - 1) {
          int kc = k + 1;
          double rhoi = c.rhow(kc) / c.adzw(kc);
          double rdz2 = 1. / (c.dz * c.dz);
          double rdz5 = 0.5 * rdz2 * c.grdf_z(k);
          double tkz = rdz5 * (tkh(i, j, k) + tkh(i, j, kc));
          flx(i, j, k) = -tkz * (f(i, j, kc) - f(i, j, k)) * rhoi;
          fl[kc] = fl[kc] + flx(i, j, k);
        } else {
          double tmp = 1. / c.adzw(nz);
          double rdz = 1. / c.dz;
          flx(i, j, 0) = 0.0 * rdz * c.rhow(1);             // fluxb = 0
          flx(i, j, nzm) = 0.0 * rdz * tmp * c.rhow(nz);    // fluxt = 0
          fl[1] = fl[1] + flx(i, j, 0);
        }
      }
    for (int k = 1; k <= nzm; ++k)
      for (int i = 1; i <= nx; ++i) {
        int kb = k - 1;
        double rhoi = 1. / (c.adz(k) * c.rho(k));
        dfdt(i, j, k) = c.dtn * (dfdt(i, j, k) - (flx(i, j, k) - flx(i, j, kb)) * rhoi);
        f(i, j, k) = f(i, j, k) + dfdt(i, j, k);
      }
    if (flux)
      for (int k = 1; k <= nzm; ++k) (*flux)(k) = fl[k];
    if (fdiff)
      for (int k = 1; k <= nzm; ++k) {
        double s = 0.;
        for (int i = 1; i <= nx; ++i) s = s + (f(i, j, k) - df[(size_t)k * (nx + 1) + i]);
        (*fdiff)(k) = s;
      }
  }

  // ---- cloud.F90:7-114 (saturation adjustment)
  void cloud(Column &c) {
    const double an = 1. / (tbgmax - tbgmin), bn = tbgmin * an;
    const double ap = 1. / (tprmax - tprmin), bp = tprmin * ap;
    const double fac1 = fac_cond + (1 + bp) * fac_fus;
    const double fac2 = fac_fus * ap;
    for (int k = 1; k <= g.nzm; ++k)
      for (int j = 1; j <= g.ny; ++j)
        for (int i = 1; i <= g.nx; ++i) {
          double &q = c.qt(i, j, k), &qp = c.qp(i, j, k);
          double pres = c.pres(k);
          q = fmax2(0., q);
          c.tabs(i, j, k) = c.t(i, j, k) - c.gamaz(k);
          double tabs = c.tabs(i, j, k);
          double tabs1 = (tabs + fac1 * qp) / (1. + fac2 * qp);
          double qsatt;
          if (tabs1 >= tbgmax) {
            tabs1 = tabs + fac_cond * qp;
            qsatt = qsatw(tabs1, pres);
          } else if (tabs1 <= tbgmin) {
            tabs1 = tabs + fac_sub * qp;
            qsatt = qsati(tabs1, pres);
          } else {
            double om = an * tabs1 - bn;
            qsatt = om * qsatw(tabs1, pres) + (1. - om) * qsati(tabs1, pres);
          }
          if (q > qsatt) {
            int niter = 0;
            double dtabs = 100.;
            double dqsat = 0.;
            while (fabs(dtabs) > R4(0.01) && niter < 10) {
              double lstarn, dlstarn, lstarp, dlstarp;
              if (tabs1 >= tbgmax) {
                lstarn = fac_cond; dlstarn = 0.;
                qsatt = qsatw(tabs1, pres); dqsat = dtqsatw(tabs1, pres);
              } else if (tabs1 <= tbgmin) {
                lstarn = fac_sub; dlstarn = 0.;
                qsatt = qsati(tabs1, pres); dqsat = dtqsati(tabs1, pres);
              } else {
                double om = an * tabs1 - bn;
                lstarn = fac_cond + (1. - om) * fac_fus;
                dlstarn = an * fac_fus;
                qsatt = om * qsatw(tabs1, pres) + (1. - om) * qsati(tabs1, pres);
                dqsat = om * dtqsatw(tabs1, pres) + (1. - om) * dtqsati(tabs1, pres);
              }
              if (tabs1 >= tprmax) { lstarp = fac_cond; dlstarp = 0.; }
              else if (tabs1 <= tprmin) { lstarp = fac_sub; dlstarp = 0.; }
              else {
                double omp = ap * tabs1 - bp;
                lstarp = fac_cond + (1. - omp) * fac_fus;
                dlstarp = ap * fac_fus;
              }
              double fff = tabs - tabs1 + lstarn * (q - qsatt) + lstarp * qp;
              double dfff = dlstarn * (q - qsatt) + dlstarp * qp - lstarn * dqsat - 1.;
              dtabs = -fff / dfff;
              niter = niter + 1;
              tabs1 = tabs1 + dtabs;
            }
            qsatt = qsatt + dqsat * dtabs;
            c.qn(i, j, k) = fmax2(0., q - qsatt);
          } else {
            c.qn(i, j, k) = 0.;
          }
          c.tabs(i, j, k) = tabs1;
          qp = fmax2(0., qp);
        }
  }

  // ---- precip_proc.F90:7-151
  void precip_proc(Column &c) {
    const double powr1 = (3 + b_rain) / 4., powr2 = (5 + b_rain) / 8.;
    const double pows1 = (3 + b_snow) / 4., pows2 = (5 + b_snow) / 8.;
    const double powg1 = (3 + b_grau) / 4., powg2 = (5 + b_grau) / 8.;
    for (int k = 1; k <= g.nzm; ++k) { c.qpsrc(k) = 0.; c.qpevp(k) = 0.; }
    for (int k = 1; k <= g.nzm; ++k)
      for (int j = 1; j <= g.ny; ++j)
        for (int i = 1; i <= g.nx; ++i) {
          double &q = c.qt(i, j, k), &qp = c.qp(i, j, k), &qn = c.qn(i, j, k);
          double tabs = c.tabs(i, j, k);
          if (qn + qp > 0.) {
            double omn = fmax2(0., fmin2(1., (tabs - tbgmin) * g.a_bg));
            double omp = fmax2(0., fmin2(1., (tabs - tprmin) * g.a_pr));
            double omg = fmax2(0., fmin2(1., (tabs - tgrmin) * g.a_gr));
            if (qn > 0.) {
              double qcc = qn * omn;
              double qii = qn * (1. - omn);
              double autor = (qcc > qcw0) ? alphaelq : 0.;
              double autos = (qii > qci0) ? betaelq * c.coefice(k) : 0.;
              double accrr = 0.;
              if (omp > R4(0.001)) {
                double qrr = qp * omp;
                accrr = c.accrrc(k) * det_pow(qrr, powr1);
              }
              double accrcs = 0., accris = 0.;
              if (omp < R4(0.999) && omg < R4(0.999)) {
                double qss = qp * (1. - omp) * (1. - omg);
                double tmp = det_pow(qss, pows1);
                accrcs = c.accrsc(k) * tmp;
                accris = c.accrsi(k) * tmp;
              }
              double accrcg = 0., accrig = 0.;
              if (omp < R4(0.999) && omg > R4(0.001)) {
                double qgg = qp * (1. - omp) * omg;
                double tmp = det_pow(qgg, powg1);
                accrcg = c.accrgc(k) * tmp;
                accrig = c.accrgi(k) * tmp;
              }
              qcc = (qcc + c.dtn * autor * qcw0) / (1. + c.dtn * (accrr + accrcs + accrcg + autor));
              qii = (qii + c.dtn * autos * qci0) / (1. + c.dtn * (accris + accrig + autos));
              double dq = c.dtn * (accrr * qcc + autor * (qcc - qcw0) + (accris + accrig) * qii +
                                   (accrcs + accrcg) * qcc + autos * (qii - qci0));
              dq = fmin2(dq, qn);
              qp = qp + dq;
              q = q - dq;
              qn = qn - dq;
              c.qpsrc(k) = c.qpsrc(k) + dq;
            } else if (qp > qp_threshold && qn == 0.) {
              double qsatt = 0.;
              if (omn > R4(0.001)) qsatt = qsatt + omn * qsatw(tabs, c.pres(k));
              if (omn < R4(0.999)) qsatt = qsatt + (1. - omn) * qsati(tabs, c.pres(k));
              double dq = 0.;
              if (omp > R4(0.001)) {
                double qrr = qp * omp;
                dq = dq + c.evapr1(k) * sqrt(qrr) + c.evapr2(k) * det_pow(qrr, powr2);
              }
              if (omp < R4(0.999) && omg < R4(0.999)) {
                double qss = qp * (1. - omp) * (1. - omg);
                dq = dq + c.evaps1(k) * sqrt(qss) + c.evaps2(k) * det_pow(qss, pows2);
              }
              if (omp < R4(0.999) && omg > R4(0.001)) {
                double qgg = qp * (1. - omp) * omg;
                dq = dq + c.evapg1(k) * sqrt(qgg) + c.evapg2(k) * det_pow(qgg, powg2);
              }
              dq = dq * c.dtn * (q / qsatt - 1.);
              dq = fmax2(-0.5 * qp, dq);
              qp = qp + dq;
              q = q - dq;
              c.qpevp(k) = c.qpevp(k) + dq;
            } else {
              q = q + qp;
              c.qpevp(k) = c.qpevp(k) - qp;
              qp = 0.;
            }
          }
          double dq = qp;
          qp = fmax2(0., qp);
          q = q + (dq - qp);
        }
  }

  // ---- diagnose.F90:8-177 (the fields that feed the model and outputs)
  void diagnose(Column &c) {
    const int nx = g.nx, ny = g.ny, nzm = g.nzm;
    const double coef = 1. / (double)(nx * ny);
    for (int k = 1; k <= nzm; ++k) {
      c.u0(k) = 0.; c.v0(k) = 0.; c.t0(k) = 0.; c.tabs0(k) = 0.; c.q0(k) = 0.; c.qn0(k) = 0.; c.qp0(k) = 0.;
    }
    for (int k = 1; k <= nzm; ++k)
      for (int j = 1; j <= ny; ++j)
        for (int i = 1; i <= nx; ++i) {
          c.tabs(i, j, k) = c.t(i, j, k) - c.gamaz(k) + fac_cond * (c.qcl(i, j, k) + c.qpl(i, j, k)) +
                            fac_sub * (c.qci(i, j, k) + c.qpi(i, j, k));
          c.u0(k) = c.u0(k) + c.u(i, j, k);
          c.v0(k) = c.v0(k) + c.v(i, j, k);
          c.t0(k) = c.t0(k) + c.t(i, j, k);
          c.tabs0(k) = c.tabs0(k) + c.tabs(i, j, k);
          c.q0(k) = c.q0(k) + (c.qv(i, j, k) + c.qcl(i, j, k) + c.qci(i, j, k));
          c.qn0(k) = c.qn0(k) + (c.qcl(i, j, k) + c.qci(i, j, k));
          c.qp0(k) = c.qp0(k) + (c.qpl(i, j, k) + c.qpi(i, j, k));
        }
    for (int k = 1; k <= nzm; ++k) {
      c.u0(k) = c.u0(k) * coef; c.v0(k) = c.v0(k) * coef; c.t0(k) = c.t0(k) * coef;
      c.tabs0(k) = c.tabs0(k) * coef; c.q0(k) = c.q0(k) * coef; c.qn0(k) = c.qn0(k) * coef;
      c.qp0(k) = c.qp0(k) * coef;
    }
    for (int k = 1; k <= nzm; ++k) c.qv0(k) = c.q0(k) - c.qn0(k);
  }

  // ---- one substep (crm_module.F90:743-887), split at precip_fall's nprec
  void substep_a(Column &c, int nstep, int icyc, FallScratch &s) {
    c.icycle = icyc;
    c.dtn = g.dt / c.ncycle;
    c.dt3[c.na - 1] = c.dtn;
    c.dtfactor = c.dtn / g.dt;
    abcoefs(c, nstep);
    zero(c);
    buoyancy(c);
    forcing(c);
    radiation(c);
    damping(c);
    ice_fall(c);
    boundaries(c, 3);
    boundaries(c, 0);
    tke_full(c);
    boundaries(c, 4);
    advect_mom(c);
    if (g.YES3D) diffuse_mom3D(c);       // diffuse_mom.F90:15-31
    else diffuse_mom2D(c);
    pressure(c);
    adams(c);
    boundaries(c, 2);
    if (g.YES3D) {                       // advect_scalar.F90:52-56
      advect_scalar3D(c, c.t, nullptr, nullptr);
      advect_scalar3D(c, c.qt, &c.mkadv[0], &c.mkwle[0]);
      advect_scalar3D(c, c.qp, &c.mkadv[1], &c.mkwle[1]);
    } else {
      advect_scalar2D(c, c.t, nullptr, nullptr);
      advect_scalar2D(c, c.qt, &c.mkadv[0], &c.mkwle[0]);
      advect_scalar2D(c, c.qp, &c.mkadv[1], &c.mkwle[1]);
    }
    precip_fall_part1(c, s);
  }
  // ---- mean-state acceleration (accelerate_crm.F90:109-366), split so the
  // batch mode can take its cease decision across all columns.
  struct AccelTend {
    std::vector<double> t, q, u, v;
  };
  // horizontal means minus the previous diagnose means; true when some
  // |ttend| exceeds 5 K (accelerate_crm.F90:181-236)
  bool accel_tend(Column &c, AccelTend &a) {
    const int nx = g.nx, ny = g.ny, nzm = g.nzm;
    const double coef = 1.0 / (double)(nx * ny);
    a.t.assign(nzm + 1, 0.); a.q.assign(nzm + 1, 0.); a.u.assign(nzm + 1, 0.); a.v.assign(nzm + 1, 0.);
    bool cease = false;
    for (int k = 1; k <= nzm; ++k) {
      double tb = 0, qb = 0, ub = 0, vb = 0;
      for (int j = 1; j <= ny; ++j)
        for (int i = 1; i <= nx; ++i) {
          tb = tb + c.t(i, j, k) * coef;
          qb = qb + (c.qcl(i, j, k) + c.qci(i, j, k) + c.qv(i, j, k)) * coef;
          if (g.accel_uv) {
            ub = ub + c.u(i, j, k) * coef;
            vb = vb + c.v(i, j, k) * coef;
          }
        }
      a.t[k] = tb - c.t0(k);
      a.q[k] = qb - c.q0(k);
      if (g.accel_uv) { a.u[k] = ub - c.u0(k); a.v[k] = vb - c.v0(k); }
      if (fabs(a.t[k]) > 5.) cease = true;
    }
    return cease;
  }
  // accelerate_crm.F90:238-262: no acceleration now or later; nstop grows
  // so the integration still covers dt_gl
  void accel_cease(Column &c) {
    c.ceaseflag = true;
    c.nstop = (int)((double)c.nstop + (double)(c.nstop - c.nstep + 1) * g.accel_factor);
  }
  // accelerate_crm.F90:264-352: apply, then clip negative qt per level and
  // repartition qv, qcl, qci
  void accel_apply(Column &c, const AccelTend &a) {
    const int nx = g.nx, ny = g.ny, nzm = g.nzm;
    const double f = g.accel_factor, tmin = 50.;
    for (int k = 1; k <= nzm; ++k)
      for (int j = 1; j <= ny; ++j)
        for (int i = 1; i <= nx; ++i) {
          c.t(i, j, k) = fmax2(tmin, c.t(i, j, k) + f * a.t[k]);
          if (g.accel_uv) {
            c.u(i, j, k) = c.u(i, j, k) + f * a.u[k];
            c.v(i, j, k) = c.v(i, j, k) + f * a.v[k];
          }
          c.qt(i, j, k) = c.qt(i, j, k) + f * a.q[k];
        }
    for (int k = 1; k <= nzm; ++k) {
      double qpoz = 0., qneg = 0.;
      for (int j = 1; j <= ny; ++j)
        for (int i = 1; i <= nx; ++i) {
          if (c.qt(i, j, k) < 0.) qneg = qneg + c.qt(i, j, k);
          else qpoz = qpoz + c.qt(i, j, k);
        }
      for (int j = 1; j <= ny; ++j)
        for (int i = 1; i <= nx; ++i) {
          if (qpoz + qneg <= 0.) {
            c.qt(i, j, k) = 0.; c.qv(i, j, k) = 0.; c.qcl(i, j, k) = 0.; c.qci(i, j, k) = 0.;
          } else {
            double factor = 1. + qneg / qpoz;
            c.qt(i, j, k) = fmax2(0., c.qt(i, j, k) * factor);
            if (c.qt(i, j, k) <= 0.) {
              c.qv(i, j, k) = 0.; c.qcl(i, j, k) = 0.; c.qci(i, j, k) = 0.;
            } else {
              double qt_res = c.qt(i, j, k) - c.qcl(i, j, k) - c.qci(i, j, k);
              c.qv(i, j, k) = fmax2(0., qt_res);
              if (qt_res < 0.) {
                double fr = 1. + qt_res / (c.qcl(i, j, k) + c.qci(i, j, k));
                c.qcl(i, j, k) = c.qcl(i, j, k) * fr;
                c.qci(i, j, k) = c.qci(i, j, k) * fr;
              }
            }
          }
        }
    }
  }

  // substep_b up to the microphysics (crm_module.F90:800-869)
  void substep_b_micro(Column &c, FallScratch &s, int nprec) {
    precip_fall_part2(c, s, nprec);
    uvw(c);
    boundaries(c, 3);
    if (g.YES3D) {                       // diffuse_scalar.F90:30-36
      diffuse_scalar3D(c, c.t, nullptr, nullptr);
      diffuse_scalar3D(c, c.qt, &c.mkdiff[0], &c.mkwsb[0]);
      diffuse_scalar3D(c, c.qp, &c.mkdiff[1], &c.mkwsb[1]);
    } else {
      diffuse_scalar2D(c, c.t, nullptr, nullptr);
      diffuse_scalar2D(c, c.qt, &c.mkdiff[0], &c.mkwsb[0]);
      diffuse_scalar2D(c, c.qp, &c.mkdiff[1], &c.mkwsb[1]);
    }
    if (c.icycle == 1) precip_init(c);
    cloud(c);
    precip_proc(c);
    micro_diagnose(c);
  }
  // after the (optional) acceleration: diagnose and rotate the AB levels
  void substep_b_end(Column &c) {
    diagnose(c);
    int nn = c.na; c.na = c.nc; c.nc = c.nb; c.nb = nn;
  }
  void substep_b(Column &c, FallScratch &s, int nprec) {
    substep_b_micro(c, s, nprec);
    if (g.use_accel && !c.ceaseflag) {   // crm_module.F90:871-876
      AccelTend a;
      if (accel_tend(c, a)) accel_cease(c);
      else accel_apply(c, a);
    }
    substep_b_end(c);
  }

  // ---- per-step statistics (crm_module.F90:896-1073)
  void step_stats(Column &c) {
    const int nx = g.nx, ny = g.ny, nzm = g.nzm, nz = g.nz, plev = g.plev;
    const double cwp_threshold = R4(0.001), wmin = 2.;
    for (int j = 1; j <= ny; ++j)
      for (int i = 1; i <= nx; ++i) {
        double cwp = 0, cwph = 0, cwpm = 0, cwpl = 0;
        bool flag_top = true;
        double cltemp = 0, cmtemp = 0, chtemp = 0, cttemp = 0;
        for (int k = 1; k <= nzm; ++k) {
          int l = plev - k + 1;
          int kk = nz - k;
          double tmp1 = c.rho(kk) * c.adz(kk) * c.dz * (c.qcl(i, j, kk) + c.qci(i, j, kk));
          cwp = cwp + tmp1;
          cttemp = fmax2(1.0, cttemp);     // cf3d = 1
          if (cwp > cwp_threshold && flag_top) {
            c.o_cldtop(l) = c.o_cldtop(l) + 1;
            flag_top = false;
          }
          if (c.pres(kk) >= 700.) { cwpl = cwpl + tmp1; cltemp = fmax2(1.0, cltemp); }
          else if (c.pres(kk) < 400.) { cwph = cwph + tmp1; chtemp = fmax2(1.0, chtemp); }
          else { cwpm = cwpm + tmp1; cmtemp = fmax2(1.0, cmtemp); }
          tmp1 = c.rho(k) * c.adz(k) * c.dz;
          double ws = c.w(i, j, k + 1) + c.w(i, j, k);
          if (tmp1 * (c.qcl(i, j, k) + c.qci(i, j, k)) > cwp_threshold) {
            c.o_cld(l) = c.o_cld(l) + 1.0;
            if (ws > 2 * wmin) {
              c.o_mcup(l) = c.o_mcup(l) + c.rho(k) * 0.5 * ws * 1.0;
              c.o_mcuup(l) = c.o_mcuup(l) + c.rho(k) * 0.5 * ws * (1.0 - 1.0);
            }
            if (ws < -2 * wmin) {
              c.o_mcdn(l) = c.o_mcdn(l) + c.rho(k) * 0.5 * ws * 1.0;
              c.o_mcudn(l) = c.o_mcudn(l) + c.rho(k) * 0.5 * ws * (1. - 1.0);
            }
          } else {
            if (ws > 2 * wmin) c.o_mcuup(l) = c.o_mcuup(l) + c.rho(k) * 0.5 * ws;
            if (ws < -2 * wmin) c.o_mcudn(l) = c.o_mcudn(l) + c.rho(k) * 0.5 * ws;
          }
          c.o_gliqwp(l) = c.o_gliqwp(l) + c.qcl(i, j, k);
          c.o_gicewp(l) = c.o_gicewp(l) + c.qci(i, j, k);
        }
        // cloud-fraction totals (crm_module.F90:1053-1072)
        c.st_cwp[(j - 1) * nx + (i - 1)] = cwp;
        c.st_ct[(j - 1) * nx + (i - 1)] = cttemp;
        c.st_cwph[(j - 1) * nx + (i - 1)] = cwph; c.st_ch[(j - 1) * nx + (i - 1)] = chtemp;
        c.st_cwpm[(j - 1) * nx + (i - 1)] = cwpm; c.st_cm[(j - 1) * nx + (i - 1)] = cmtemp;
        c.st_cwpl[(j - 1) * nx + (i - 1)] = cwpl; c.st_cl[(j - 1) * nx + (i - 1)] = cltemp;
      }
    for (int k = 1; k <= nzm; ++k)
      for (int j = 1; j <= ny; ++j)
        for (int i = 1; i <= nx; ++i) {
          int i_rad = (i - 1) / (nx / g.nx_rad) + 1;
          int j_rad = (j - 1) / (ny / g.ny_rad) + 1;
          c.rad_t(i_rad, j_rad, k) = c.rad_t(i_rad, j_rad, k) + c.tabs(i, j, k);
          c.rad_qv(i_rad, j_rad, k) = c.rad_qv(i_rad, j_rad, k) + fmax2(0., c.qv(i, j, k));
          c.rad_qc(i_rad, j_rad, k) = c.rad_qc(i_rad, j_rad, k) + c.qcl(i, j, k);
          c.rad_qi(i_rad, j_rad, k) = c.rad_qi(i_rad, j_rad, k) + c.qci(i, j, k);
          if (c.qcl(i, j, k) + c.qci(i, j, k) > 0) c.rad_cld(i_rad, j_rad, k) = c.rad_cld(i_rad, j_rad, k) + 1.0;
        }
    for (int j = 1; j <= ny; ++j)
      for (int i = 1; i <= nx; ++i)
        for (int k = 1; k <= nzm + 1; ++k) {
          int l = plev + 1 - k + 1;
          double wv = c.w(i, j, k);
          if (wv > 0.) {
            int kx = std::max(1, k - 1);
            double qsat = qsatw(c.tabs(i, j, kx), c.pres(kx));
            if (c.qcl(i, j, kx) + c.qci(i, j, kx) > fmin2(R4(1.e-5), R4(0.01) * qsat))
              c.mui(l) = c.mui(l) + c.rhow(k) * wv;
          } else if (wv < 0.) {
            int kx = std::min(k + 1, nzm);
            double qsat = qsatw(c.tabs(i, j, kx), c.pres(kx));
            if (c.qcl(i, j, kx) + c.qci(i, j, kx) > fmin2(R4(1.e-5), R4(0.01) * qsat))
              c.mdi(l) = c.mdi(l) + c.rhow(k) * wv;
            else if (c.qpl(i, j, kx) + c.qpi(i, j, kx) > R4(1.0e-4))
              c.mdi(l) = c.mdi(l) + c.rhow(k) * wv;
          }
        }
    for (int j = 1; j <= ny; ++j)
      for (int i = 1; i <= nx; ++i) {
        int ij = (j - 1) * nx + (i - 1);
        if (c.st_cwp[ij] > cwp_threshold) c.cltot = c.cltot + c.st_ct[ij];
        if (c.st_cwph[ij] > cwp_threshold) c.clhgh = c.clhgh + c.st_ch[ij];
        if (c.st_cwpm[ij] > cwp_threshold) c.clmed = c.clmed + c.st_cm[ij];
        if (c.st_cwpl[ij] > cwp_threshold) c.cllow = c.cllow + c.st_cl[ij];
      }
  }
};

}  // namespace oracle

namespace oracle {

// ---- per-call constants (crm_module.F90:301-318, pressure.F90:118-198,
//      precip_init.F90:25-49, microphysics.F90:500-507)
static int setup_grid_constants(Grid &g, const crm_config *cfg, const crm_call_desc *desc) {
  g.nx = cfg->crm_nx; g.ny = cfg->crm_ny; g.nzm = cfg->crm_nz; g.nz = g.nzm + 1;
  g.YES3D = g.ny > 1 ? 1 : 0;
  g.plev = cfg->plev;
  g.nx_rad = cfg->crm_nx_rad; g.ny_rad = cfg->crm_ny_rad;
  g.dx = cfg->crm_dx;
  g.dy = (g.ny == 1) ? g.dx : cfg->crm_dy;    // setparm.F90:56,70
  g.batch_mode = cfg->batch_mode;
  if (g.nx < 4 || g.nx % 2 || g.nzm < 4 || g.plev < g.nzm + 1) return CRM_ERR_ARG;
  if (g.YES3D && (g.ny < 4 || g.ny % 2 || !(g.dy > 0))) return CRM_ERR_ARG;
  if (g.nx % g.nx_rad || g.ny % g.ny_rad) return CRM_ERR_ARG;
  if (cfg->microphysics != CRM_MICRO_SAM1MOM) return CRM_ERR_UNSUPPORTED;
  g.nstop = (int)(desc->dt_gl / cfg->crm_dt);   // crm_module.F90:712-713
  if (g.nstop < 1) return CRM_ERR_ARG;
  g.dt = desc->dt_gl / g.nstop;
  // crm_accel_nstop (accelerate_crm.F90:84-106)
  g.use_accel = cfg->use_crm_accel != 0;
  g.accel_factor = cfg->crm_accel_factor;
  g.accel_uv = cfg->crm_accel_uv != 0;
  if (g.use_accel) {
    if (!(g.accel_factor >= 0.) || g.nstop % (int)(1 + g.accel_factor) != 0) return CRM_ERR_ARG;
    g.nstop = (int)((double)g.nstop / (1 + g.accel_factor));
  }
  if (60. < 2 * g.dt) return CRM_ERR_ARG;       // damping.F90:39-42
  fax(g.ifaxi, g.nx);
  for (int k = 1; k <= g.ifaxi[0]; ++k)
    if (g.ifaxi[k] > 5) return CRM_ERR_ARG;
  fftrig(g.trigxi, g.nx);
  if (g.YES3D) {
    fax(g.ifaxj, g.ny);
    for (int k = 1; k <= g.ifaxj[0]; ++k)
      if (g.ifaxj[k] > 5) return CRM_ERR_ARG;
    fftrig(g.trigxj, g.ny);
  }
  // eigenvalues (pressure.F90:172-198) for i = 1..nx+1 and j = 1..ny+2
  // (2D: j = 1 only), periodic in both directions (no walls)
  g.eign_ni = g.nx + 1; g.eign_nj = g.YES3D ? g.ny + 2 : 1;
  g.eign.assign((size_t)g.eign_ni * g.eign_nj, 0.0);
  {
    double ddx2 = 1.0 / (g.dx * g.dx), ddy2 = 1.0 / (g.dy * g.dy);
    double pii = 3.14159265358979323846;
    double xnx = pii / g.nx, xny = pii / g.ny;
    for (int j = 1; j <= g.eign_nj; ++j) {
      int jd = (int)(((float)j - 0.1f) / 2.f);
      double xj = jd, facty = 2.0;
      for (int i = 1; i <= g.nx + 1; ++i) {
        int id = (int)(((float)i - 0.1f) / 2.f);
        double xi = id, factx = 2.0;
        g.eign[(size_t)(j - 1) * g.eign_ni + (i - 1)] =
            (2.0 * cos(factx * xnx * xi) - 2.0) * ddx2 + (2.0 * cos(facty * xny * xj) - 2.0) * ddy2;
      }
    }
  }
  // gamma functions: gammafff.c returns (float)exp(lgamma(x)) for float x
  auto gammafff = [](float x) { return gammafff_r4(x); };
  g.gam3 = gammafff(3.f);
  g.gamr1 = gammafff((float)(3. + b_rain));
  g.gamr2 = gammafff((float)((5. + b_rain) / 2.));
  g.gamr3 = gammafff((float)(4. + b_rain));
  g.gams1 = gammafff((float)(3. + b_snow));
  g.gams2 = gammafff((float)((5. + b_snow) / 2.));
  g.gams3 = gammafff((float)(4. + b_snow));
  g.gamg1 = gammafff((float)(3. + b_grau));
  g.gamg2 = gammafff((float)((5. + b_grau) / 2.));
  g.gamg3 = gammafff((float)(4. + b_grau));
  g.crain = b_rain / 4.; g.csnow = b_snow / 4.; g.cgrau = b_grau / 4.;
  g.vrain = a_rain * g.gamr3 / 6. / det_pow(pi * rhor * nzeror, g.crain);
  g.vsnow = a_snow * g.gams3 / 6. / det_pow(pi * rhos * nzeros, g.csnow);
  g.vgrau = a_grau * g.gamg3 / 6. / det_pow(pi * rhog * nzerog, g.cgrau);
  g.a_bg = 1. / (tbgmax - tbgmin);
  g.a_pr = 1. / (tprmax - tprmin);
  g.a_gr = 1. / (tgrmax - tgrmin);
  return CRM_OK;
}

// ---- end of call: crm_module.F90:1086-1594
static void finalize_column(Model &M, Column &c, int icrm, crm_state_c *st, crm_rad_c *rad, crm_output_c *out) {
  Grid &g = M.g;
  const int nx = g.nx, ny = g.ny, nzm = g.nzm, plev = g.plev, ld = M.ld, Y = g.YES3D;
  const double factor_xy = 1.0 / (double)(nx * ny);
  const double icrm_run_time = 1.0 / M.desc->dt_gl;
  const double factor_xyt = factor_xy / (double)c.nstop;
  const int ptop = plev - nzm + 1;
  auto O1 = [&](int f) -> double & { return out->field[f][icrm]; };
  auto O2 = [&](int f, int l) -> double & { return out->field[f][(size_t)icrm + (size_t)ld * (l - 1)]; };
  auto O4 = [&](double *a, int i, int j, int k) -> double & {
    return a[(size_t)icrm + (size_t)ld * ((i - 1) + (size_t)nx * ((j - 1) + (size_t)ny * (k - 1)))];
  };
  auto IN = [&](const double *a, int l) { return M.IN(a, icrm, l); };
  // radiation means
  {
    double fx = (double)g.nx_rad / (double)nx, fy = (double)g.ny_rad / (double)ny;
    double tmp1 = fx * fy / (double)c.nstop;
    for (int k = 1; k <= nzm; ++k)
      for (int j = 1; j <= g.ny_rad; ++j)
        for (int i = 1; i <= g.nx_rad; ++i) {
          size_t o = (size_t)icrm + (size_t)ld * ((i - 1) + (size_t)g.nx_rad * ((j - 1) + (size_t)g.ny_rad * (k - 1)));
          rad->temperature[o] = c.rad_t(i, j, k) * tmp1;
          rad->qv[o] = c.rad_qv(i, j, k) * tmp1;
          rad->qc[o] = c.rad_qc(i, j, k) * tmp1;
          rad->qi[o] = c.rad_qi(i, j, k) * tmp1;
          rad->cld[o] = c.rad_cld(i, j, k) * tmp1;
        }
  }
  std::vector<double> tln(plev + 1), qln(plev + 1), qccln(plev + 1), qiiln(plev + 1), uln(plev + 1), vln(plev + 1);
  for (int k = 1; k <= ptop - 1; ++k) {
    tln[k] = IN(M.in->tl, k); qln[k] = IN(M.in->ql, k); qccln[k] = IN(M.in->qccl, k);
    qiiln[k] = IN(M.in->qiil, k); uln[k] = IN(M.in->ul, k); vln[k] = IN(M.in->vl, k);
  }
  for (int k = ptop; k <= plev; ++k) tln[k] = qln[k] = qccln[k] = qiiln[k] = uln[k] = vln[k] = 0.;
  double prectend0 = c.colprec, precstend0 = c.colprecs;
  double colprec = 0, colprecs = 0;
  for (int k = 1; k <= nzm; ++k)
    for (int i = 1; i <= nx; ++i)
      for (int j = 1; j <= ny; ++j) {
        int l = plev - k + 1;
        double pdel = IN(M.in->pdel, plev - k + 1);
        colprec = colprec + (c.qpl(i, j, k) + c.qpi(i, j, k)) * pdel;
        colprecs = colprecs + c.qpi(i, j, k) * pdel;
        tln[l] = tln[l] + c.tabs(i, j, k);
        qln[l] = qln[l] + c.qv(i, j, k);
        qccln[l] = qccln[l] + c.qcl(i, j, k);
        qiiln[l] = qiiln[l] + c.qci(i, j, k);
        uln[l] = uln[l] + c.u(i, j, k);
        vln[l] = vln[l] + c.v(i, j, k);
      }
  for (int k = ptop; k <= plev; ++k) {
    tln[k] *= factor_xy; qln[k] *= factor_xy; qccln[k] *= factor_xy; qiiln[k] *= factor_xy;
    uln[k] *= factor_xy; vln[k] *= factor_xy;
  }
  for (int k = 1; k <= plev; ++k) {
    O2(CRM_OUT_SLTEND, k) = cp * (tln[k] - IN(M.in->tl, k)) * icrm_run_time;
    O2(CRM_OUT_QLTEND, k) = (qln[k] - IN(M.in->ql, k)) * icrm_run_time;
    O2(CRM_OUT_QCLTEND, k) = (qccln[k] - IN(M.in->qccl, k)) * icrm_run_time;
    O2(CRM_OUT_QILTEND, k) = (qiiln[k] - IN(M.in->qiil, k)) * icrm_run_time;
  }
  O1(CRM_OUT_PRECTEND) = (colprec - prectend0) / ggr * factor_xy * icrm_run_time;
  O1(CRM_OUT_PRECSTEND) = (colprecs - precstend0) / ggr * factor_xy * icrm_run_time;
  for (int k = ptop; k <= ptop + 1; ++k) {
    O2(CRM_OUT_SLTEND, k) = 0.; O2(CRM_OUT_QLTEND, k) = 0.;
    O2(CRM_OUT_QCLTEND, k) = 0.; O2(CRM_OUT_QILTEND, k) = 0.;
  }
  for (int k = 1; k <= nzm; ++k)
    for (int j = 1; j <= ny; ++j)
      for (int i = 1; i <= nx; ++i) {
        O4(st->u_wind, i, j, k) = c.u(i, j, k);
        O4(st->v_wind, i, j, k) = c.v(i, j, k);
        O4(st->w_wind, i, j, k) = c.w(i, j, k);
        O4(st->temperature, i, j, k) = c.tabs(i, j, k);
        O4(st->qt, i, j, k) = c.qt(i, j, k);
        O4(st->qp, i, j, k) = c.qp(i, j, k);
        O4(st->qn, i, j, k) = c.qn(i, j, k);
        O4(out->field[CRM_OUT_TK], i, j, k) = c.tk(i, j, k);
        O4(out->field[CRM_OUT_TKH], i, j, k) = c.tkh(i, j, k);
        O4(out->field[CRM_OUT_QCL], i, j, k) = c.qcl(i, j, k);
        O4(out->field[CRM_OUT_QCI], i, j, k) = c.qci(i, j, k);
        O4(out->field[CRM_OUT_QPL], i, j, k) = c.qpl(i, j, k);
        O4(out->field[CRM_OUT_QPI], i, j, k) = c.qpi(i, j, k);
      }
  O1(CRM_OUT_Z0M) = c.z0;
  O1(CRM_OUT_TAUX) = 0.0 / (double)c.nstop;
  O1(CRM_OUT_TAUY) = 0.0 / (double)c.nstop;
  // domain means of condensate at the end of the call
  std::vector<double> qcm(plev + 1, 0.), qim(plev + 1, 0.), qrm(plev + 1, 0.), qgm(plev + 1, 0.), qsm(plev + 1, 0.);
  for (int k = 1; k <= nzm; ++k)
    for (int j = 1; j <= ny; ++j)
      for (int i = 1; i <= nx; ++i) {
        int l = plev - k + 1;
        qcm[l] = qcm[l] + c.qcl(i, j, k);
        qim[l] = qim[l] + c.qci(i, j, k);
        qrm[l] = qrm[l] + c.qpl(i, j, k);
        double omg = fmax2(0., fmin2(1., (c.tabs(i, j, k) - tgrmin) * g.a_gr));
        qgm[l] = qgm[l] + c.qpi(i, j, k) * omg;
        qsm[l] = qsm[l] + c.qpi(i, j, k) * (1. - omg);
      }
  for (int k = 1; k <= plev; ++k) {
    double pdel = IN(M.in->pdel, k);
    O2(CRM_OUT_CLD, k) = fmin2(1.0, c.o_cld(k) * factor_xyt);
    O2(CRM_OUT_CLDTOP, k) = fmin2(1.0, c.o_cldtop(k) * factor_xyt);
    O2(CRM_OUT_GICEWP, k) = c.o_gicewp(k) * pdel * 1000. / ggr * factor_xyt;
    O2(CRM_OUT_GLIQWP, k) = c.o_gliqwp(k) * pdel * 1000. / ggr * factor_xyt;
    double mcup = c.o_mcup(k) * factor_xyt, mcdn = c.o_mcdn(k) * factor_xyt;
    double mcuup = c.o_mcuup(k) * factor_xyt, mcudn = c.o_mcudn(k) * factor_xyt;
    O2(CRM_OUT_MCUP, k) = mcup; O2(CRM_OUT_MCDN, k) = mcdn;
    O2(CRM_OUT_MCUUP, k) = mcuup; O2(CRM_OUT_MCUDN, k) = mcudn;
    O2(CRM_OUT_MCTOT, k) = mcup + mcdn + mcuup + mcudn;
    O2(CRM_OUT_QC_MEAN, k) = qcm[k] * factor_xy;
    O2(CRM_OUT_QI_MEAN, k) = qim[k] * factor_xy;
    O2(CRM_OUT_QS_MEAN, k) = qsm[k] * factor_xy;
    O2(CRM_OUT_QG_MEAN, k) = qgm[k] * factor_xy;
    O2(CRM_OUT_QR_MEAN, k) = qrm[k] * factor_xy;
  }
  double precc = 0, precl = 0, precsc = 0, precsl = 0;
  const double thr = (double)(10.f / 86400.f);
  for (int j = 1; j <= ny; ++j)
    for (int i = 1; i <= nx; ++i) {
      double ps = c.precsfc(i, j, 1) * c.dz / g.dt / (double)c.nstop;
      double pss = c.precssfc(i, j, 1) * c.dz / g.dt / (double)c.nstop;
      if (ps > thr) { precc = precc + ps; precsc = precsc + pss; }
      else { precl = precl + ps; precsl = precsl + pss; }
      out->field[CRM_OUT_PREC_CRM][(size_t)icrm + (size_t)ld * ((i - 1) + (size_t)nx * (j - 1))] = ps / 1000.;
    }
  O1(CRM_OUT_PRECC) = precc * factor_xy / 1000.;
  O1(CRM_OUT_PRECL) = precl * factor_xy / 1000.;
  O1(CRM_OUT_PRECSC) = precsc * factor_xy / 1000.;
  O1(CRM_OUT_PRECSL) = precsl * factor_xy / 1000.;
  O1(CRM_OUT_CLTOT) = c.cltot * factor_xyt;
  O1(CRM_OUT_CLHGH) = c.clhgh * factor_xyt;
  O1(CRM_OUT_CLMED) = c.clmed * factor_xyt;
  O1(CRM_OUT_CLLOW) = c.cllow * factor_xyt;
  double jt = plev * 1.0, mx = 1.0;
  for (int k = 1; k <= plev; ++k) {
    double mu = 0.5 * (c.mui(k) + c.mui(k + 1));
    double md = 0.5 * (c.mdi(k) + c.mdi(k + 1));
    mu = mu * ggr / 100.;
    md = md * ggr / 100.;
    O2(CRM_OUT_MU_CRM, k) = mu;
    O2(CRM_OUT_MD_CRM, k) = md;
    double pdel = IN(M.in->pdel, k);
    O2(CRM_OUT_EU_CRM, k) = 0.;
    O2(CRM_OUT_DU_CRM, k) = 0.;
    O2(CRM_OUT_ED_CRM, k) = 0.;
    if (c.mui(k) - c.mui(k + 1) > 0) O2(CRM_OUT_EU_CRM, k) = (c.mui(k) - c.mui(k + 1)) * ggr / pdel;
    else O2(CRM_OUT_DU_CRM, k) = -1.0 * (c.mui(k) - c.mui(k + 1)) * ggr / pdel;
    if (c.mdi(k + 1) - c.mdi(k) < 0) O2(CRM_OUT_ED_CRM, k) = (c.mdi(k) - c.mdi(k + 1)) * ggr / pdel;
    if (fabs(mu) > R4(1.0e-15) || fabs(md) > R4(1.0e-15)) {
      jt = fmin2((double)k, jt);
      mx = fmax2((double)k, mx);
    }
  }
  O1(CRM_OUT_JT_CRM) = jt;
  O1(CRM_OUT_MX_CRM) = mx;
  for (int k = 1; k <= nzm; ++k) {
    double u2z = 0., v2z = 0., w2z = 0.;
    for (int j = 1; j <= ny; ++j)
      for (int i = 1; i <= nx; ++i) {
        double du = c.u(i, j, k) - c.u0(k), dv = c.v(i, j, k) - c.v0(k);
        u2z = u2z + du * du;
        v2z = v2z + dv * dv;
        double w1 = c.w(i, j, k + 1), w0 = c.w(i, j, k);
        w2z = w2z + 0.5 * (w1 * w1 + w0 * w0);
      }
    double tmp1 = c.dz / c.rhow(k);
    double tmp2 = tmp1 / c.dtn;
    double mkwsb[2], mkwle[2], mkadv[2], mkdiff[2];
    for (int m = 0; m < 2; ++m) {
      mkwsb[m] = c.mkwsb[m](k) * tmp1 * c.rhow(k) * factor_xy / (double)c.nstop;
      mkwle[m] = c.mkwle[m](k) * tmp2 * c.rhow(k) * factor_xy / (double)c.nstop;
      mkadv[m] = c.mkadv[m](k) * factor_xy * icrm_run_time;
      mkdiff[m] = c.mkdiff[m](k) * factor_xy * icrm_run_time;
    }
    double qpsrc = c.qpsrc(k) * factor_xy * icrm_run_time;
    double qpevp = c.qpevp(k) * factor_xy * icrm_run_time;
    double qpfall = c.qpfall(k) * factor_xy * icrm_run_time;
    double precflux = c.precflux(k) * factor_xy * c.dz / g.dt / (double)c.nstop;
    int l = plev - k + 1;
    O2(CRM_OUT_FLUX_U, l) = (c.uwle(k) + c.uwsb(k)) * tmp1 * factor_xy / (double)c.nstop;
    O2(CRM_OUT_FLUX_V, l) = (c.vwle(k) + c.vwsb(k)) * tmp1 * factor_xy / (double)c.nstop;
    O2(CRM_OUT_FLUX_QT, l) = mkwle[0] + mkwsb[0];
    O2(CRM_OUT_FLUXSGS_QT, l) = mkwsb[0];
    O2(CRM_OUT_FLUX_QP, l) = mkwle[1] + mkwsb[1];
    O2(CRM_OUT_QT_TRANS, l) = mkadv[0] + mkdiff[0];
    O2(CRM_OUT_QP_TRANS, l) = mkadv[1] + mkdiff[1];
    double tmp = 0;
    for (int j = 1; j <= ny; ++j)
      for (int i = 1; i <= nx; ++i) tmp = tmp + c.tke(i, j, k);
    double tkesgsz = c.rho(k) * tmp * factor_xy;
    O2(CRM_OUT_TKESGSZ, l) = tkesgsz;
    O2(CRM_OUT_TKEZ, l) = c.rho(k) * 0.5 * (u2z + v2z * (double)Y + w2z) * factor_xy + tkesgsz;
    tmp = 0;
    for (int j = 1; j <= ny; ++j)
      for (int i = 1; i <= nx; ++i) tmp = tmp + c.tk(i, j, k);
    O2(CRM_OUT_TKZ, l) = tmp * factor_xy;
    O2(CRM_OUT_PRECFLUX, l) = precflux / 1000.;
    O2(CRM_OUT_QP_FALL, l) = qpfall;
    O2(CRM_OUT_QP_EVP, l) = qpevp;
    O2(CRM_OUT_QP_SRC, l) = qpsrc;
    O2(CRM_OUT_QT_LS, l) = c.qtend(k);
    O2(CRM_OUT_T_LS, l) = c.ttend(k);
  }
  O1(CRM_OUT_TIMING_FACTOR) = (double)c.nstop / (double)c.nstop;
}

}  // namespace oracle

namespace oracle {

static void zero_outputs(const Grid &g, int icrm, int ld, crm_output_c *out) {
  for (int f = 0; f < CRM_NOUT; ++f) {
    size_t n;
    if (f < CRM_OUT_FIRST_3D) n = (size_t)g.nx * g.ny * g.nzm;
    else if (f < CRM_OUT_FIRST_1D) n = (size_t)g.nx * g.ny;
    else if (f < CRM_OUT_FIRST_2D) n = 1;
    else n = (size_t)g.plev;
    for (size_t e = 0; e < n; ++e) out->field[f][(size_t)icrm + (size_t)ld * e] = 0.0;
  }
}

// first-step velocity clamp test (crm_module.F90:400): equal neighbours
static bool clamp_test(const Grid &g, const crm_state_c *st, int icrm, int ld) {
  auto U = [&](int i, int k) { return st->u_wind[(size_t)icrm + (size_t)ld * ((i - 1) + (size_t)g.nx * g.ny * (k - 1))]; };
  return U(1, 1) == U(2, 1) && U(3, 2) == U(4, 2);
}

// icrm: the column's slot in the (ld, ...) arrays; pos: its position in the
// call (gcol and status index); the two differ only under a col_map.
static void run_column_full(Model &M, Column &c, int icrm, int pos, crm_state_c *st, crm_rad_c *rad,
                            crm_output_c *out) {
  Grid &g = M.g;
  M.alloc_column(c);
  zero_outputs(g, icrm, M.ld, out);
  M.init_column(c, icrm, st, rad, clamp_test(g, st, icrm, M.ld));
  if (M.desc->igstep <= 1) M.setperturb(c, M.desc->gcol[pos] * 1000);
  Model::FallScratch s;
  for (int nstep = 1; nstep <= c.nstop && c.status == CRM_OK; ++nstep) {
    c.nstep = nstep;
    M.kurant(c);
    if (c.nonfinite) { c.status = CRM_ERR_NONFINITE; break; }
    c.ncycle = Model::ncycle_of(c.cfl);
    if (c.ncycle > 16) { c.status = CRM_ERR_CFL; break; }
    for (int icyc = 1; icyc <= c.ncycle; ++icyc) {
      M.substep_a(c, nstep, icyc, s);
      c.nprec = Model::nprec_of(c.prec_cfl);
      M.substep_b(c, s, c.nprec);
    }
    M.step_stats(c);
  }
  finalize_column(M, c, icrm, st, rad, out);
}

}  // namespace oracle

using namespace oracle;

extern "C" {

// Test hook: fft991 on one vector a[0..n+1] with the pressure solver's trig
// table and factors (isign -1: grid point -> spectral, +1: back).  Returns
// CRM_ERR_ARG for a length the transform does not factor (radix 2..5).
int oracle_fft991(double *a, int n, int isign) {
  if (!a || n < 4 || n % 2) return CRM_ERR_ARG;
  int ifax[20] = {0};
  fax(ifax, n);
  for (int k = 1; k <= ifax[0]; ++k)
    if (ifax[k] > 5) return CRM_ERR_ARG;
  std::vector<double> trigs, work((size_t)n + 2);
  fftrig(trigs, n);
  fft991(a, work.data(), trigs.data(), ifax, n, isign);
  return CRM_OK;
}

// Run the restatement of crm() on the host.  Same arguments and array
// conventions as crm_run() in include/crm_gb300.h; nthreads <= 0 uses the
// OpenMP default.  Returns a crm_status.
int oracle_crm_run(const crm_config *cfg, const crm_call_desc *desc, const crm_input_c *in,
                   crm_state_c *st, crm_rad_c *rad, crm_output_c *out, int *col_status, int nthreads) {
  if (!cfg || !desc || !in || !st || !rad || !out) return CRM_ERR_ARG;
  if (desc->ncrms < 1 || desc->ld < desc->ncrms) return CRM_ERR_ARG;
  Model M;
  int rc = setup_grid_constants(M.g, cfg, desc);
  if (rc != CRM_OK) return rc;
  M.desc = desc;
  M.in = in;
  M.ld = desc->ld;
  const int ncrms = desc->ncrms;
  M.cols.resize(ncrms);
  M.col_status_saved.assign(ncrms, CRM_OK);
#ifdef _OPENMP
  if (nthreads > 0) omp_set_num_threads(nthreads);
#else
  (void)nthreads;
#endif
  auto slot_of = [&](int pos) { return desc->col_map ? desc->col_map[pos] : pos; };
  for (int pos = 0; pos < ncrms; ++pos)
    if (slot_of(pos) < 0 || slot_of(pos) >= desc->ld) return CRM_ERR_ARG;
  if (cfg->batch_mode == CRM_PER_COLUMN) {
#pragma omp parallel for schedule(dynamic, 1)
    for (int pos = 0; pos < ncrms; ++pos) {
      run_column_full(M, M.cols[pos], slot_of(pos), pos, st, rad, out);
      M.col_status_saved[pos] = M.cols[pos].status;
      M.cols[pos] = Column();        // release memory early
    }
  } else {
    if (desc->col_map) return CRM_ERR_UNSUPPORTED;
    Grid &g = M.g;
    bool clamp = clamp_test(g, st, 0, M.ld);
    std::vector<Model::FallScratch> scr(ncrms);
#pragma omp parallel for schedule(dynamic, 1)
    for (int icrm = 0; icrm < ncrms; ++icrm) {
      Column &c = M.cols[icrm];
      M.alloc_column(c);
      zero_outputs(g, icrm, M.ld, out);
      M.init_column(c, icrm, st, rad, clamp);
      if (desc->igstep <= 1) M.setperturb(c, desc->gcol[icrm] * 1000);
    }
    int status = CRM_OK;
    int nstop = g.nstop;          // batch-wide, like the reference's
    bool cease = false;
    std::vector<Model::AccelTend> acc(ncrms);
    for (int nstep = 1; nstep <= nstop && status == CRM_OK; ++nstep) {
      for (int icrm = 0; icrm < ncrms; ++icrm) M.cols[icrm].nstep = nstep;
      int ncycle = 1;
      for (int icrm = 0; icrm < ncrms; ++icrm) {
        M.kurant(M.cols[icrm]);
        ncycle = std::max(ncycle, Model::ncycle_of(M.cols[icrm].cfl));
      }
      if (ncycle > 16) { status = CRM_ERR_CFL; break; }
      for (int icyc = 1; icyc <= ncycle; ++icyc) {
#pragma omp parallel for schedule(dynamic, 1)
        for (int icrm = 0; icrm < ncrms; ++icrm) {
          M.cols[icrm].ncycle = ncycle;
          M.substep_a(M.cols[icrm], nstep, icyc, scr[icrm]);
        }
        int nprec = 1;
        for (int icrm = 0; icrm < ncrms; ++icrm) nprec = std::max(nprec, Model::nprec_of(M.cols[icrm].prec_cfl));
#pragma omp parallel for schedule(dynamic, 1)
        for (int icrm = 0; icrm < ncrms; ++icrm) M.substep_b_micro(M.cols[icrm], scr[icrm], nprec);
        if (g.use_accel && !cease) {   // one cease decision for the batch
          bool any = false;
          for (int icrm = 0; icrm < ncrms; ++icrm) any = M.accel_tend(M.cols[icrm], acc[icrm]) || any;
          if (any) {
            cease = true;
            nstop = (int)((double)nstop + (double)(nstop - nstep + 1) * g.accel_factor);
            for (int icrm = 0; icrm < ncrms; ++icrm) { M.cols[icrm].ceaseflag = true; M.cols[icrm].nstop = nstop; }
          } else {
#pragma omp parallel for schedule(dynamic, 1)
            for (int icrm = 0; icrm < ncrms; ++icrm) M.accel_apply(M.cols[icrm], acc[icrm]);
          }
        }
#pragma omp parallel for schedule(dynamic, 1)
        for (int icrm = 0; icrm < ncrms; ++icrm) M.substep_b_end(M.cols[icrm]);
      }
#pragma omp parallel for schedule(dynamic, 1)
      for (int icrm = 0; icrm < ncrms; ++icrm) M.step_stats(M.cols[icrm]);
    }
    for (int icrm = 0; icrm < ncrms; ++icrm)
      M.col_status_saved[icrm] = M.cols[icrm].nonfinite ? CRM_ERR_NONFINITE : status;
#pragma omp parallel for schedule(dynamic, 1)
    for (int icrm = 0; icrm < ncrms; ++icrm) finalize_column(M, M.cols[icrm], icrm, st, rad, out);
  }
  int worst = CRM_OK;
  for (int icrm = 0; icrm < ncrms; ++icrm) {
    int s = M.col_status_saved[icrm];
    if (col_status) col_status[icrm] = s;
    if (s != CRM_OK) worst = s;
  }
  return worst;
}

// Test hooks for known-answer checks of single routines.
// RNG_MT: n draws after RNG_MT_set_seed(seed).
float oracle_gammafff(float x) { return gammafff_r4(x); }

int oracle_rng_mt(int seed, int n, double *out) {
  if (!out || n < 0) return CRM_ERR_ARG;
  RngMT r(seed);
  for (int i = 0; i < n; ++i) out[i] = r.gen();
  return CRM_OK;
}
// sat.F90: which = 0 esatw, 1 esati, 2 dtesatw, 3 dtesati, 4 qsatw, 5 qsati,
// 6 dtqsatw, 7 dtqsati at temperatures t [K] (and pressures p [mb] for 4-7).
int oracle_sat(int which, const double *t, const double *p, int n, double *out) {
  if (!t || !out || n < 0 || which < 0 || which > 7 || (which >= 4 && !p)) return CRM_ERR_ARG;
  for (int i = 0; i < n; ++i) {
    switch (which) {
      case 0: out[i] = esatw(t[i]); break;
      case 1: out[i] = esati(t[i]); break;
      case 2: out[i] = dtesatw(t[i]); break;
      case 3: out[i] = dtesati(t[i]); break;
      case 4: out[i] = qsatw(t[i], p[i]); break;
      case 5: out[i] = qsati(t[i], p[i]); break;
      case 6: out[i] = dtqsatw(t[i], p[i]); break;
      default: out[i] = dtqsati(t[i], p[i]); break;
    }
  }
  return CRM_OK;
}

int oracle_version(void) { return 1; }

}  // extern "C"
