// crm_kernel.cuh -- the persistent column kernel: one CTA integrates one CRM
// column through a whole GCM step (crm/crm_module.F90:380-1594), then takes
// the next column.  T is the bulk arithmetic type (double: plain form;
// float: FP32-mixed form, with FP64 kept for the pressure tridiagonal solve,
// all domain-mean / column sums and the saturation-adjustment Newton solve).
//
// Every phase follows the reference routine named in its comment.  Cell-wise
// loops are spread over the CTA's threads with a barrier between phases;
// every sum over the horizontal runs sequentially in the reference's loop
// order (one thread per level), so the FP64 form reproduces the CPU
// restatement bit for bit.  The FP32-mixed form adds what only it needs:
// warp-parallel sums, per-cell residues carried by the t and qt updates
// (add_carry), FP64 means where a mean feeds a relaxation or a returned
// tendency.  Both forms skip work that provably changes no bit (the
// sedimentation of a column with no falling precipitation, qp transport of a
// column whose qp is +0 everywhere).
#pragma once
#include "crm_device.cuh"
#include "crm_kernel.h"
#include "crm_tc.cuh"

namespace crm {

// physical constants (crm/params.F90:49-64, shr_const_mod.F90)
#define C_CP 1.00464e3
#define C_GGR 9.80616
#define C_LCOND 2.501e6
#define C_LFUS 3.337e5
#define C_LSUB (C_LCOND + C_LFUS)
#define C_RGASU (6.02214e26 * 1.38065e-23)
#define C_RV (C_RGASU / 18.016)
#define C_FAC_COND (C_LCOND / C_CP)
#define C_FAC_FUS (C_LFUS / C_CP)
#define C_FAC_SUB (C_LSUB / C_CP)
#define C_PI R4(3.141592653589793)
#define C_EPSV R4(0.61)
// MICRO_SAM1MOM/micro_params.F90
#define C_TBGMIN R4(253.16)
#define C_TBGMAX R4(273.16)
#define C_TPRMIN R4(268.16)
#define C_TPRMAX R4(283.16)
#define C_TGRMIN R4(223.16)
#define C_TGRMAX R4(283.16)
#define C_A_RAIN 842.
#define C_B_RAIN R4(0.8)
#define C_A_SNOW R4(4.84)
#define C_B_SNOW 0.25
#define C_A_GRAU 94.5
#define C_B_GRAU 0.5
#define C_QCW0 R4(1.e-3)
#define C_QCI0 R4(1.e-4)
#define C_ALPHAELQ R4(1.e-3)
#define C_BETAELQ R4(1.e-3)
#define C_ESICOEF R4(0.1)
#define C_EGICOEF R4(0.1)
#define C_NZEROR 8.e6
#define C_NZEROS 3.e6
#define C_NZEROG 4.e6
#define C_RHOR 1000.
#define C_RHOS 100.
#define C_RHOG 400.
#define C_QP_THRESHOLD R4(1.e-8)
#define C_DIFFELQ R4(2.21e-05)
#define C_THERCO R4(2.40e-02)
#define C_MUELQ R4(1.717e-05)

#ifdef CRM_PHASE_TIMERS
#define PHASE_MARK(id)                                                          \
  do {                                                                          \
    if (threadIdx.x == 0) {                                                     \
      unsigned long long t_ = clock64();                                        \
      p.phase_cycles[(size_t)blockIdx.x * 64 + (id)] += t_ - S.t_last;          \
      S.t_last = t_;                                                            \
    }                                                                           \
  } while (0)
#else
#define PHASE_MARK(id) \
  do {                 \
  } while (0)
#endif

#define TID ((int)threadIdx.x)
#define NT ((int)blockDim.x)
#define SYNC __syncthreads()

// CFL of a column whose state is not finite (enters the batch maximum)
constexpr double kCflNonfinite = 1.0e300;

// ncycle = max(1, ceil(cfl / 0.7)) (kurant.F90:54-64), saturated at 10^6 so
// that an unbounded CFL converts to an int safely; anything above 16 stops
// the column
__device__ __forceinline__ int ncycle_of(double cfl) {
  double n = ceil(cfl / R4(0.7));
  if (!(n < 1.0e6)) return 1000000;
  return n > 1. ? (int)n : 1;
}

// per-CTA scalars of the column being integrated
struct ColShared {
  int na, nb, nc, ncycle, icycle, nprec, prec_any, status, kmin, kmax, n_damp, col;
  double dt3[3], at, bt, ct, dtn, dtfactor, dz, cfl, prec_cfl, z0;
  double colprec0, colprecs0;
  double cltot, clhgh, clmed, cllow;
  int jt_min, mx_max;
  int nstop, ceaseflag, acc_flag;   // per-column step count (acceleration)
  int gbar;                         // grid barriers passed (batch mode)
  unsigned long long t_last;
  double red_d[32];
  int red_i[64];
  // tensor-core transforms of the 3D pressure solve (crm_tc.cuh)
  unsigned long long tc_mbar;
  unsigned tc_tmem, tc_phase;
  int tc_fail;
  float t_off;                      // FP32-mixed form: t's offset in the upwind fluxes
};

// The CRM's horizontal size: a compile-time constant for the sizes built
// into the library (the reference fixes it at build time too, CRM_NX in
// crmdims.F90), so strides and the (i, k) index arithmetic of every cell loop
// fold to constants; NX = 0 reads it from the layout at run time.
template <int NX> struct NxDim {
  static constexpr int nx = NX;
  __device__ explicit NxDim(int) {}
};
template <> struct NxDim<0> {
  const int nx;
  __device__ explicit NxDim(int n) : nx(n) {}
};

// The CRM's y size: 1 for the 2D CRM (compile-time, so the 2D kernel is the
// same code as without a y dimension), a compile-time size or 0 (run time)
// for the 3D CRM.
template <int NY> struct NyDim {
  static constexpr int ny = NY;
  __device__ explicit NyDim(int) {}
};
template <> struct NyDim<0> {
  const int ny;
  __device__ explicit NyDim(int n) : ny(n) {}
};

// TC = 1: the 3D FP32-mixed form with the pressure solve's transforms on
// the tensor cores (crm_tc.cuh); a kernel that contains tcgen05 code runs
// one CTA per SM on GB300, so it is a separate instance
template <typename T, int NX, int NY = 1, int TC = 0>
struct ColumnKernel : NxDim<NX>, NyDim<NY> {
  using NxDim<NX>::nx;
  using NyDim<NY>::ny;
  static constexpr bool Y3 = NY != 1;
  using FT = F2<T, Y3>;
  // horizontal cells of the column: phases that never look at a horizontal
  // neighbour run over h = 1..NH() (the (h, k) accessor decodes h in 3D)
  __device__ __forceinline__ int NH() const {
    if constexpr (Y3) return nx * ny;
    else return nx;
  }
  // radiation columns (crm_nx_rad x crm_ny_rad; the 3D form has one per CRM
  // column, so the group of cell h is h there)
  __device__ __forceinline__ int NR() const {
    if constexpr (Y3) return p.L.nx_rad * p.L.ny_rad;
    else return p.L.nx_rad;
  }
  // the end-of-call sums of crm_module.F90:1034-1060 run i outer, j inner:
  // the n-th cell (n = 1..NH()) of that order as a cell h = i + nx (j - 1)
  __device__ __forceinline__ int h_ij(int n) const {
    if constexpr (Y3) return (n - 1) / ny + 1 + nx * ((n - 1) % ny);
    else return n;
  }
  const KParams &p;
  ColShared &S;
  T *base;
  int nzm, nz, plev;
  int icrm;   // slot of the column in the (ld, ...) arrays
  int cpos;   // position of the column in the call (status index)
  T *spl;     // scratch planes A, B in shared memory, or null (slab planes)
  int fdir = 0;  // direction of the transform in progress (3D: 1 is y)

  __device__ ColumnKernel(const KParams &p_, ColShared &s_, T *b, int col, T *planes = nullptr)
      : NxDim<NX>(p_.L.nx), NyDim<NY>(p_.L.ny), p(p_), S(s_), base(b), nzm(p_.L.nzm), nz(p_.L.nz), plev(p_.L.plev),
        icrm(p_.col_map ? p_.col_map[col] : col), cpos(col), spl(planes) {}

  // ---------------------------------------------------------- accessors
  // x extents of the field classes (first index, row length = nx + extra):
  // the halo widths of crm/grid.F90:31-46 with NADV = NADVS = 0, as laid
  // out by make_layout (crm_layout.h)
  // y extents come from the layout (3D) and are {1, 1} in 2D
  __device__ __forceinline__ FT fld(size_t off, int x1, int extra, XRange y, int z1 = 1) const {
    if constexpr (Y3) return FT{base + off, x1, nx + extra, z1, y.x1, (nx + extra) * y.nxa, p.L.lnx};
    else return FT{base + off, x1, nx + extra, z1, 1, nx + extra, 0};
  }
  __device__ __forceinline__ FT U() const { return fld(p.L.u, -1, 5, p.L.yu); }
  __device__ __forceinline__ FT V() const { return fld(p.L.v, -1, 4, p.L.yv); }
  __device__ __forceinline__ FT W() const { return fld(p.L.w, -1, 4, p.L.yw); }
  __device__ __forceinline__ FT TT() const { return fld(p.L.t, -2, 6, p.L.ys); }
  __device__ __forceinline__ FT QT() const { return fld(p.L.qt, -2, 6, p.L.ys); }
  __device__ __forceinline__ FT QP() const { return fld(p.L.qp, -2, 6, p.L.ys); }
  __device__ __forceinline__ FT TKE() const { return fld(p.L.tke, 1, 0, p.L.yi); }
  __device__ __forceinline__ FT TK() const { return fld(p.L.tk, 0, 2, p.L.yd); }
  __device__ __forceinline__ FT TKH() const { return fld(p.L.tkh, 0, 2, p.L.yd); }
  __device__ __forceinline__ FT PP() const { return fld(p.L.p, 0, 1, p.L.yp); }
  __device__ __forceinline__ FT TABS() const { return fld(p.L.tabs, 1, 0, p.L.yi); }
  __device__ __forceinline__ FT QV() const { return fld(p.L.qv, 1, 0, p.L.yi); }
  __device__ __forceinline__ FT QCL() const { return fld(p.L.qcl, 1, 0, p.L.yi); }
  __device__ __forceinline__ FT QCI() const { return fld(p.L.qci, 1, 0, p.L.yi); }
  __device__ __forceinline__ FT QPL() const { return fld(p.L.qpl, 1, 0, p.L.yi); }
  __device__ __forceinline__ FT QPI() const { return fld(p.L.qpi, 1, 0, p.L.yi); }
  __device__ __forceinline__ FT QN() const { return fld(p.L.qn, 1, 0, p.L.yi); }
  __device__ __forceinline__ FT DU(int l) const { return fld(p.L.du[l - 1], 1, 1, p.L.yi); }
  __device__ __forceinline__ FT DV(int l) const { return fld(p.L.dv[l - 1], 1, 0, p.L.ydv); }
  __device__ __forceinline__ FT DW(int l) const { return fld(p.L.dw[l - 1], 1, 0, p.L.yi); }
  // scratch planes (x from -2, k from 0; 3D: y from -2); A and B
  // (contiguous: A may be used as one double-length area) live in shared
  // memory when the launch shape provides them (2D only)
  __device__ __forceinline__ FT SCR(size_t off) const { return fld(off, -2, 6, p.L.ysc, 0); }
  __device__ __forceinline__ T *sa() const { return spl ? spl : base + p.L.s_a; }
  __device__ __forceinline__ T *sb() const { return spl ? spl + (p.L.s_b - p.L.s_a) : base + p.L.s_b; }
  __device__ __forceinline__ FT SA() const {
    if constexpr (Y3) return SCR(p.L.s_a);
    else return FT{sa(), -2, nx + 6, 0, 1, nx + 6, 0};
  }
  __device__ __forceinline__ FT SB() const {
    if constexpr (Y3) return SCR(p.L.s_b);
    else return FT{sb(), -2, nx + 6, 0, 1, nx + 6, 0};
  }
  __device__ __forceinline__ T *PR(int id) const { return base + p.L.prof + (size_t)id * (nz + 2); }
  __device__ __forceinline__ T *OP(int id) const { return base + p.L.o_plev + (size_t)id * (plev + 2); }
  __device__ __forceinline__ T &PS(int i) const { return base[p.L.precsfc + (i - 1)]; }
  __device__ __forceinline__ T &PSS(int i) const { return base[p.L.precssfc + (i - 1)]; }

  __device__ __forceinline__ double IN(const double *a, int l) const { return a[(size_t)icrm + (size_t)p.ld * (l - 1)]; }
  __device__ __forceinline__ size_t S4(int i, int k) const {
    return (size_t)icrm + (size_t)p.ld * ((i - 1) + (size_t)NH() * (k - 1));
  }

  // ---------------------------------------------------------- reductions
  // Horizontal sums for every level k in [k0, k1] and quantity q < nq:
  // out(q, k, s) receives s = init(q, k) + sum over the horizontal cells
  // i = 1..NH() (3D: h in the reference's (j, i) loop order) of term(q, i, k).
  // FP64 form: one thread per (q, k) adding in the reference's loop order,
  // so the result is bit-identical to a sequential CPU evaluation.
  // FP32-mixed form: one warp per (q, k); each lane adds its (at most four)
  // cells in FP32, groups of four lanes combine in FP32, and the FP64 tree
  // across the eight groups accumulates into the FP64 result.
  // Must be called by the whole CTA; results are visible after a barrier.
  template <typename Term, typename Init, typename Out>
  __device__ void level_sums(int nq, int k0, int k1, Term term, Init init, Out out) {
    const int nk = k1 - k0 + 1, npairs = nq * nk;
    if constexpr (sizeof(T) == 8) {
      for (int e = TID; e < npairs; e += NT) {
        int q = e / nk, k = k0 + e % nk;
        double s = init(q, k);
        for (int i = 1; i <= NH(); ++i) s = s + (double)term(q, i, k);
        out(q, k, s);
      }
    } else {
      const int lane = TID & 31, warp = TID >> 5, nw = NT >> 5;
      for (int e = warp; e < npairs; e += nw) {
        int q = e / nk, k = k0 + e % nk;
        T part = (T)0;
        for (int i = 1 + lane; i <= NH(); i += 32) part = part + term(q, i, k);
        part = part + __shfl_xor_sync(0xffffffffu, part, 1);
        part = part + __shfl_xor_sync(0xffffffffu, part, 2);
        double sd = (double)part;
        sd = sd + __shfl_xor_sync(0xffffffffu, sd, 4);
        sd = sd + __shfl_xor_sync(0xffffffffu, sd, 8);
        sd = sd + __shfl_xor_sync(0xffffffffu, sd, 16);
        if (lane == 0) out(q, k, init(q, k) + sd);
      }
    }
  }
  // Horizontal sums that only feed statistics and diagnostics (no
  // conservation fixer): the FP64 form is level_sums itself; the FP32-mixed
  // form reduces the warp entirely in FP32 (pairwise, error ~log2(NH()) ulp),
  // sparing the slow FP64 pipe.
  template <typename Term, typename Init, typename Out>
  __device__ void level_sums_lo(int nq, int k0, int k1, Term term, Init init, Out out) {
    if constexpr (sizeof(T) == 8) {
      level_sums(nq, k0, k1, term, init, out);
    } else {
      const int nk = k1 - k0 + 1;
      const int lane = TID & 31, warp = TID >> 5, nw = NT >> 5;
      if (nq <= 4) {
        // a warp per level takes all nq quantities from one pass over the
        // level's cells (each quantity summed in the same order as below)
        for (int kk = warp; kk < nk; kk += nw) {
          const int k = k0 + kk;
          T part[4] = {(T)0, (T)0, (T)0, (T)0};
          for (int i = 1 + lane; i <= NH(); i += 32) {
#pragma unroll
            for (int q = 0; q < 4; ++q)
              if (q < nq) part[q] = part[q] + term(q, i, k);
          }
#pragma unroll
          for (int q = 0; q < 4; ++q) {
            if (q < nq) {
              T x = part[q];
              for (int o = 1; o < 32; o <<= 1) x = x + __shfl_xor_sync(0xffffffffu, x, o);
              if (lane == 0) out(q, k, (double)((T)init(q, k) + x));
            }
          }
        }
        return;
      }
      const int npairs = nq * nk;
      for (int e = warp; e < npairs; e += nw) {
        int q = e / nk, k = k0 + e % nk;
        T part = (T)0;
        for (int i = 1 + lane; i <= NH(); i += 32) part = part + term(q, i, k);
        for (int o = 1; o < 32; o <<= 1) part = part + __shfl_xor_sync(0xffffffffu, part, o);
        if (lane == 0) out(q, k, (double)((T)init(q, k) + part));
      }
    }
  }

  // level_sums_lo for NQ quantities that share their loads: the FP64 form
  // is level_sums with termq(q, i, k) (the reference's order, bit-exact);
  // the FP32-mixed form gives one warp a whole level, termv(i, k, v) fills
  // all NQ terms of a cell from one set of loads, and each quantity is
  // reduced in FP32 (pairwise warp tree).
  template <int NQ, typename TermQ, typename TermV, typename Init, typename Out>
  __device__ void level_sums_lo_multi(int k0, int k1, TermQ termq, TermV termv, Init init, Out out) {
    if constexpr (sizeof(T) == 8) {
      level_sums(NQ, k0, k1, termq, init, out);
    } else {
      const int lane = TID & 31, warp = TID >> 5, nw = NT >> 5;
      for (int k = k0 + warp; k <= k1; k += nw) {
        T part[NQ];
#pragma unroll
        for (int q = 0; q < NQ; ++q) part[q] = (T)0;
        for (int i = 1 + lane; i <= NH(); i += 32) {
          T v[NQ];
          termv(i, k, v);
#pragma unroll
          for (int q = 0; q < NQ; ++q) part[q] = part[q] + v[q];
        }
#pragma unroll
        for (int q = 0; q < NQ; ++q) {
          T x = part[q];
          for (int o = 1; o < 32; o <<= 1) x = x + __shfl_xor_sync(0xffffffffu, x, o);
          part[q] = x;
        }
        if (lane == 0) {
#pragma unroll
          for (int q = 0; q < NQ; ++q) out(q, k, (double)((T)init(q, k) + part[q]));
        }
      }
    }
  }

  // level_sums for NQ quantities that share their loads, FP64-accumulated:
  // the FP64 form is level_sums with termq (bit-exact); the FP32-mixed form
  // gives one warp a level, termv fills all NQ terms of a cell, and each
  // quantity is reduced like level_sums (FP32 within groups of four lanes,
  // FP64 across the groups).
  template <int NQ, typename TermQ, typename TermV, typename Init, typename Out>
  __device__ void level_sums_multi(int k0, int k1, TermQ termq, TermV termv, Init init, Out out) {
    if constexpr (sizeof(T) == 8) {
      level_sums(NQ, k0, k1, termq, init, out);
    } else {
      const int lane = TID & 31, warp = TID >> 5, nw = NT >> 5;
      for (int k = k0 + warp; k <= k1; k += nw) {
        T part[NQ];
#pragma unroll
        for (int q = 0; q < NQ; ++q) part[q] = (T)0;
        for (int i = 1 + lane; i <= NH(); i += 32) {
          T v[NQ];
          termv(i, k, v);
#pragma unroll
          for (int q = 0; q < NQ; ++q) part[q] = part[q] + v[q];
        }
#pragma unroll
        for (int q = 0; q < NQ; ++q) {
          T x = part[q];
          x = x + __shfl_xor_sync(0xffffffffu, x, 1);
          x = x + __shfl_xor_sync(0xffffffffu, x, 2);
          double sd = (double)x;
          sd = sd + __shfl_xor_sync(0xffffffffu, sd, 4);
          sd = sd + __shfl_xor_sync(0xffffffffu, sd, 8);
          sd = sd + __shfl_xor_sync(0xffffffffu, sd, 16);
          if (lane == 0) out(q, k, init(q, k) + sd);
        }
      }
    }
  }

  // FP32-mixed form: t and qt each carry a per-cell residue plane, the part
  // of past increments that the FP32 value could not hold (t ~ 300 K lies on
  // a 2^-15 K grid, and steady increments of a few grid steps would be
  // rounded the same way every step; carrying the same residues for u, v, w
  // was measured to change no output).  add_carry returns x + d with the
  // residue r folded into the increment and leaves in r the rounding error
  // of the result (TwoSum: exact at any magnitudes; it has no product, so no
  // contraction applies).  The FP64 form has no residues (rct/rcq null).
  __device__ __forceinline__ static T add_carry(T x, T d, T &r) {
    const T y = d + r, s = x + y, yb = s - x;
    r = (x - (s - yb)) + (y - yb);
    return s;
  }
  __device__ __forceinline__ T *rct() const {
    if constexpr (sizeof(T) == 4) return base + p.L.fcomp;
    return nullptr;
  }
  __device__ __forceinline__ T *rcq() const {
    if constexpr (sizeof(T) == 4) return base + p.L.fcomp + (size_t)NH() * nzm;
    return nullptr;
  }

  // ---------------------------------------------------------- batch coupling
  // Reference-batch mode (crm_batch_mode CRM_REFERENCE_BATCH): the column
  // kernel is a cooperative launch with one co-resident CTA per column, and
  // the reference's batch-wide decisions (ncycle from the largest CFL,
  // kurant.F90:54-64; nprec, microphysics.F90:602-661; the acceleration
  // cease flag) take the maximum over all CTAs through a grid barrier.
  // Sense-reversing barrier by thread 0; every wait is bounded (~4 s): on
  // timeout the column records CRM_ERR_TIMEOUT and stops.
  __device__ bool grid_barrier() {
    unsigned int *count = reinterpret_cast<unsigned int *>(p.gsync);
    volatile unsigned int *gen = count + 1;
    if (cpos == p.barrier_withhold && S.gbar == 0) return false;   // test hook: never arrives
    __threadfence();
    const unsigned int g = *gen;
    if (atomicAdd(count, 1u) == gridDim.x - 1) {
      atomicExch(count, 0u);
      __threadfence();
      atomicAdd(const_cast<unsigned int *>(gen), 1u);
      return true;
    }
    for (long long it = 0; it < p.barrier_spins; ++it) {
      if (*gen != g) {
        __threadfence();
        return true;
      }
      __nanosleep(256);
    }
    return false;
  }
  // max over the columns of the call of v >= 0 (per-column mode: v itself);
  // called by the whole CTA with the same v
  __device__ double batch_max(double v) {
    if (p.batch_mode != CRM_REFERENCE_BATCH) return v;
    SYNC;
    if (TID == 0 && S.status == CRM_ERR_TIMEOUT) {
      // a column whose earlier wait ran out does not arrive again: the
      // others' waits run out too, and the call ends with CRM_ERR_TIMEOUT
      S.red_d[0] = v;
    } else if (TID == 0) {
      unsigned long long *slot = p.gsync + 2 + (S.gbar & 3);
      atomicMax(slot, (unsigned long long)__double_as_longlong(v));
      bool ok = grid_barrier();
      double m = __longlong_as_double((long long)atomicAdd(slot, 0ull));
      if (blockIdx.x == 0) atomicExch(p.gsync + 2 + ((S.gbar + 2) & 3), 0ull);
      S.gbar = S.gbar + 1;
      if (!ok) S.status = CRM_ERR_TIMEOUT;
      S.red_d[0] = ok ? m : v;
    }
    SYNC;
    double r = S.red_d[0];
    SYNC;
    return r;
  }

  __device__ double block_max(double v) {
    for (int o = 16; o > 0; o >>= 1) v = mx2(v, __shfl_xor_sync(0xffffffffu, v, o));
    SYNC;
    if ((TID & 31) == 0) S.red_d[TID >> 5] = v;
    SYNC;
    if (TID == 0) {
      double m = S.red_d[0];
      for (int w = 1; w < NT / 32; ++w) m = mx2(m, S.red_d[w]);
      S.red_d[0] = m;
    }
    SYNC;
    double r = S.red_d[0];
    SYNC;
    return r;
  }

  // ---------------------------------------------------------- halos
  // bound_exchange.F90:188-236 (2D): periodic copies in x only
  __device__ void exch(FT f, int k1, int k2, int i_1, int i_2) {
    int i1 = i_1 - 1, i2 = i_2 - 1;
    int nl = i1 + 1, nr = i2 + 1, per = nl + nr;
    int n = (k2 - k1 + 1) * per;
    for (int e = TID; e < n; e += NT) {
      int k = k1 + e / per, r = e % per;
      if (r < nl) { int i = -i1 + r; f(i, k) = f(i + nx, k); }
      else { int i = nx + 1 + (r - nl); f(i, k) = f(i - nx, k); }
    }
  }
  // bound_exchange.F90:14-239 in 3D: every halo cell of the rectangle
  // [1 - i_1, nx + i_2] x [1 - j_1, ny + j_2] takes the interior value it
  // wraps to (the reference copies x halos, y halos and corners from the
  // interior only, so the order of the copies does not matter)
  __device__ void exch3(FT f, int k1, int k2, int i_1, int i_2, int j_1, int j_2) {
    const int x0 = 1 - i_1, xw = nx + i_1 + i_2, y0 = 1 - j_1, ni = i_1 + i_2;
    const int nrow = (j_1 + j_2) * xw, per = nrow + ny * ni;
    const int n = (k2 - k1 + 1) * per;
    for (int e = TID; e < n; e += NT) {
      const int k = k1 + e / per, r = e % per;
      int i, j;
      if (r < nrow) {
        const int jj = r / xw;
        i = x0 + r % xw;
        j = jj < j_1 ? y0 + jj : ny + 1 + (jj - j_1);
      } else {
        const int r2 = r - nrow, ii = r2 % ni;
        j = 1 + r2 / ni;
        i = ii < i_1 ? x0 + ii : nx + 1 + (ii - i_1);
      }
      const int si = i < 1 ? i + nx : (i > nx ? i - nx : i);
      const int sj = j < 1 ? j + ny : (j > ny ? j - ny : j);
      f(i, j, k) = f(si, sj, k);
    }
  }
  __device__ void boundaries3(int flag) {     // periodic.F90:8-136, 3D
    if (flag == 0) {
      exch3(U(), 1, nzm, 1, 1, 1, 1);
      exch3(V(), 1, nzm, 1, 1, 1, 1);
      FT w = W();
      for (int h = TID + 1; h <= NH(); h += NT) w(h, nz) = (T)0.;
      SYNC;
      exch3(w, 1, nz, 1, 1, 1, 1);
      SYNC;
      for (int e = TID; e < (nx + 2) * (ny + 2); e += NT) w(e % (nx + 2), e / (nx + 2), nz) = (T)0.;
    } else if (flag == 2) {
      exch3(U(), 1, nzm, 2, 3, 2, 2);
      exch3(V(), 1, nzm, 2, 2, 2, 3);
      exch3(W(), 1, nz, 2, 2, 2, 2);
      exch3(TT(), 1, nzm, 3, 3, 3, 3);
      exch3(QT(), 1, nzm, 3, 3, 3, 3);
      exch3(QP(), 1, nzm, 3, 3, 3, 3);
    } else if (flag == 3) {
      exch3(TT(), 1, nzm, 1, 1, 1, 1);
      exch3(QT(), 1, nzm, 1, 1, 1, 1);
      exch3(QP(), 1, nzm, 1, 1, 1, 1);
    } else if (flag == 4) {
      exch3(TK(), 1, nzm, 1, 1, 1, 1);
      exch3(TKH(), 1, nzm, 1, 1, 1, 1);
    }
    SYNC;
  }
  __device__ void boundaries(int flag) {      // periodic.F90:8-136
    if constexpr (Y3) {
      boundaries3(flag);
      return;
    }
    if (flag == 0) {
      exch(U(), 1, nzm, 1, 1);
      exch(V(), 1, nzm, 1, 1);
      FT w = W();
      for (int i = TID + 1; i <= nx; i += NT) w(i, nz) = (T)0.;
      SYNC;
      exch(w, 1, nz, 1, 1);
      SYNC;
      for (int i = TID; i <= nx + 1; i += NT) w(i, nz) = (T)0.;
    } else if (flag == 2) {
      exch(U(), 1, nzm, 2, 3);
      exch(V(), 1, nzm, 2, 2);
      exch(W(), 1, nz, 2, 2);
      exch(TT(), 1, nzm, 3, 3);
      exch(QT(), 1, nzm, 3, 3);
      exch(QP(), 1, nzm, 3, 3);
    } else if (flag == 3) {
      exch(TT(), 1, nzm, 1, 1);
      exch(QT(), 1, nzm, 1, 1);
      exch(QP(), 1, nzm, 1, 1);
    } else if (flag == 4) {
      exch(TK(), 1, nzm, 1, 1);
      exch(TKH(), 1, nzm, 1, 1);
    }
    SYNC;
  }

  // ---------------------------------------------------------- micro_diagnose
  __device__ void micro_diagnose() {          // MICRO_SAM1MOM/microphysics.F90:334-357
    FT qv = QV(), qt = QT(), qn = QN(), tabs = TABS(), qcl = QCL(), qci = QCI(), qpl = QPL(), qpi = QPI(), qp = QP();
    const T a_bg = (T)p.a_bg, a_pr = (T)p.a_pr;
    for (int e = TID; e < NH() * nzm; e += NT) {
      int i = 1 + e % NH(), k = 1 + e / NH();
      qv(i, k) = qt(i, k) - qn(i, k);
      T omn = mx2((T)0., mn2((T)1., (tabs(i, k) - (T)C_TBGMIN) * a_bg));
      qcl(i, k) = qn(i, k) * omn;
      qci(i, k) = qn(i, k) * ((T)1. - omn);
      T omp = mx2((T)0., mn2((T)1., (tabs(i, k) - (T)C_TPRMIN) * a_pr));
      qpl(i, k) = qp(i, k) * omp;
      qpi(i, k) = qp(i, k) * ((T)1. - omp);
    }
    SYNC;
  }

  // ---------------------------------------------------------- precip_init
  __device__ void precip_init() {             // MICRO_SAM1MOM/precip_init.F90:54-91
    const T pi = (T)C_PI;
    for (int k = TID + 1; k <= nzm; k += NT) {
      T rho = PR(P_RHO)[k], t0 = PR(P_TABS0)[k];
      T pratio = tsqrt((T)R4(1.29) / rho);
      T rrr1 = (T)393. / (t0 + (T)120.) * tpow(t0 / (T)273., (T)1.5);
      T rrr2 = tpow(t0 / (T)273., (T)R4(1.94)) * ((T)1000. / PR(P_PRES)[k]);
      T estw = (T)100. * esatw(t0);
      T esti = (T)100. * esati(t0);
      T coef1 = (T)0.25 * pi * (T)C_NZEROS * (T)C_A_SNOW * (T)p.gams1 * pratio /
                tpow(pi * (T)C_RHOS * (T)C_NZEROS / rho, (T)((3 + C_B_SNOW) / 4.));
      T coef2 = texp((T)R4(0.025) * (t0 - (T)R4(273.15)));
      PR(P_ACCRSI)[k] = coef1 * coef2 * (T)C_ESICOEF;
      PR(P_ACCRSC)[k] = coef1 * (T)1.0;
      PR(P_COEFICE)[k] = coef2;
      coef1 = ((T)C_LSUB / (t0 * (T)C_RV) - (T)1.) * (T)C_LSUB / ((T)C_THERCO * rrr1 * t0);
      coef2 = (T)C_RV * t0 / ((T)C_DIFFELQ * rrr2 * esti);
      PR(P_EVAPS1)[k] = (T)(double)(0.65f * 4.f) * (T)C_NZEROS / tsqrt(pi * (T)C_RHOS * (T)C_NZEROS) / (coef1 + coef2) / tsqrt(rho);
      PR(P_EVAPS2)[k] = (T)(double)(0.49f * 4.f) * (T)C_NZEROS * (T)p.gams2 * tsqrt((T)C_A_SNOW / ((T)C_MUELQ * rrr1)) /
                        tpow(pi * (T)C_RHOS * (T)C_NZEROS, (T)((5 + C_B_SNOW) / 8.)) / (coef1 + coef2) *
                        tpow(rho, (T)((1 + C_B_SNOW) / 8.)) * tsqrt(pratio);
      coef1 = (T)0.25 * pi * (T)C_NZEROG * (T)C_A_GRAU * (T)p.gamg1 * pratio /
              tpow(pi * (T)C_RHOG * (T)C_NZEROG / rho, (T)((3 + C_B_GRAU) / 4.));
      coef2 = texp((T)R4(0.025) * (t0 - (T)R4(273.15)));
      PR(P_ACCRGI)[k] = coef1 * coef2 * (T)C_EGICOEF;
      PR(P_ACCRGC)[k] = coef1 * (T)1.0;
      coef1 = ((T)C_LSUB / (t0 * (T)C_RV) - (T)1.) * (T)C_LSUB / ((T)C_THERCO * rrr1 * t0);
      coef2 = (T)C_RV * t0 / ((T)C_DIFFELQ * rrr2 * esti);
      PR(P_EVAPG1)[k] = (T)(double)(0.65f * 4.f) * (T)C_NZEROG / tsqrt(pi * (T)C_RHOG * (T)C_NZEROG) / (coef1 + coef2) / tsqrt(rho);
      PR(P_EVAPG2)[k] = (T)(double)(0.49f * 4.f) * (T)C_NZEROG * (T)p.gamg2 * tsqrt((T)C_A_GRAU / ((T)C_MUELQ * rrr1)) /
                        tpow(pi * (T)C_RHOG * (T)C_NZEROG, (T)((5 + C_B_GRAU) / 8.)) / (coef1 + coef2) *
                        tpow(rho, (T)((1 + C_B_GRAU) / 8.)) * tsqrt(pratio);
      PR(P_ACCRRC)[k] = (T)0.25 * pi * (T)C_NZEROR * (T)C_A_RAIN * (T)p.gamr1 * pratio /
                        tpow(pi * (T)C_RHOR * (T)C_NZEROR / rho, (T)((3 + C_B_RAIN) / 4.)) * (T)1.0;
      coef1 = ((T)C_LCOND / (t0 * (T)C_RV) - (T)1.) * (T)C_LCOND / ((T)C_THERCO * rrr1 * t0);
      coef2 = (T)C_RV * t0 / ((T)C_DIFFELQ * rrr2 * estw);
      PR(P_EVAPR1)[k] = (T)(double)(0.78f * 2.f) * pi * (T)C_NZEROR / tsqrt(pi * (T)C_RHOR * (T)C_NZEROR) / (coef1 + coef2) / tsqrt(rho);
      PR(P_EVAPR2)[k] = (T)(double)(0.31f * 2.f) * pi * (T)C_NZEROR * (T)p.gamr2 * (T)R4(0.89) *
                        tsqrt((T)C_A_RAIN / ((T)C_MUELQ * rrr1)) /
                        tpow(pi * (T)C_RHOR * (T)C_NZEROR, (T)((5 + C_B_RAIN) / 8.)) / (coef1 + coef2) *
                        tpow(rho, (T)((1 + C_B_RAIN) / 8.)) * tsqrt(pratio);
    }
    SYNC;
  }

  // profile id of the q-th initial mean (the order of init_column's sums)
  __device__ __forceinline__ static int ids9(int q) {
    switch (q) {
      case 0: return P_U0;
      case 1: return P_V0;
      case 2: return P_T0;
      case 3: return P_T00;
      case 4: return P_TABS0;
      case 5: return P_Q0;
      case 6: return P_QV0;
      case 7: return P_QN0;
      default: return P_QP0;
    }
  }

  // ---------------------------------------------------------- init
  // crm_module.F90:320-681
  __device__ void init_column() {
    const int plev_ = plev;
    // zero the slab (allocate_* zero every module array)
    {
      size_t n = p.L.slab;
      for (size_t e = TID; e < n; e += NT) base[e] = (T)0.;
      if (spl) {                                  // shared-memory planes A, B
        size_t m = 2 * (p.L.s_b - p.L.s_a);
        for (size_t e = TID; e < m; e += NT) spl[e] = (T)0.;
      }
    }
    if (TID == 0) {
      S.na = 1; S.nb = 2; S.nc = 3;
      S.dt3[0] = S.dt3[1] = S.dt3[2] = 0.;
      S.status = CRM_OK;
      S.z0 = p.z0[icrm];
      S.nstop = p.nstop;
      S.ceaseflag = 0;
    }
    SYNC;
    {
      // crm_rad%qrad of this column, cached in the slab's sixth radiation
      // plane (the GCM array is strided by ld; the heating is read every step)
      const int nxr = NR();
      T *qr = base + p.L.rad + (size_t)5 * nxr * nzm;
      for (int e = TID; e < nxr * nzm; e += NT) {
        int ir = e % nxr, k = e / nxr;
        qr[e] = (T)p.qrad[(size_t)icrm + (size_t)p.ld * (ir + (size_t)nxr * k)];
      }
    }
    // vertical grid (crm_module.F90:341-375)
    for (int k = TID + 1; k <= nzm; k += NT) {
      double z = IN(p.zmid, plev_ - k + 1) - IN(p.zint, plev_ + 1);
      PR(P_Z)[k] = (T)z;
      PR(P_ZI)[k] = (T)(IN(p.zint, plev_ - k + 2) - IN(p.zint, plev_ + 1));
      PR(P_PRES)[k] = (T)(IN(p.pmid, plev_ - k + 1) / 100.);
      PR(P_PRESI)[k] = (T)(IN(p.pint, plev_ - k + 2) / 100.);
      PR(P_BET)[k] = (T)(C_GGR / IN(p.tl, plev_ - k + 1));
      PR(P_GAMAZ)[k] = (T)(C_GGR / C_CP * z);
    }
    if (TID == 0) {
      PR(P_ZI)[nz] = (T)(IN(p.zint, plev_ - nz + 2) - IN(p.zint, plev_ + 1));
      PR(P_PRESI)[nz] = (T)(IN(p.pint, plev_ - nz + 2) / 100.);
    }
    SYNC;
    // the grid metrics are computed in double from the double inputs
    if (TID == 0) {
      double z1 = IN(p.zmid, plev_) - IN(p.zint, plev_ + 1);
      double z2 = IN(p.zmid, plev_ - 1) - IN(p.zint, plev_ + 1);
      S.dz = 0.5 * (z1 + z2);
    }
    SYNC;
    const double dz = S.dz;
    for (int k = TID + 1; k <= nzm; k += NT) {
      double zk = IN(p.zmid, plev_ - k + 1) - IN(p.zint, plev_ + 1);
      double adzw = 1.;
      if (k >= 2) {
        double zkm = IN(p.zmid, plev_ - k + 2) - IN(p.zint, plev_ + 1);
        adzw = (zk - zkm) / dz;
      }
      PR(P_ADZW)[k] = (T)adzw;
      double zi1 = IN(p.zint, plev_ - k + 1) - IN(p.zint, plev_ + 1);
      double zi0 = IN(p.zint, plev_ - k + 2) - IN(p.zint, plev_ + 1);
      double adz = (zi1 - zi0) / dz;
      PR(P_ADZ)[k] = (T)adz;
      PR(P_RHO)[k] = (T)(IN(p.pdel, plev_ - k + 1) / C_GGR / (adz * dz));
      if (k >= 2) PR(P_RHOW)[k] = (T)((IN(p.pmid, plev_ - k + 2) - IN(p.pmid, plev_ - k + 1)) / C_GGR / (adzw * dz));
      if (k == nzm) {
        // adzw(nz) = adzw(nzm)
        PR(P_ADZW)[nz] = (T)adzw;
      }
    }
    SYNC;
    if (TID == 0) {
      // rhow(1), rhow(nz) by linear extrapolation in double
      double zk2 = IN(p.zmid, plev_ - 1) - IN(p.zint, plev_ + 1), zk1 = IN(p.zmid, plev_) - IN(p.zint, plev_ + 1);
      double zk3 = IN(p.zmid, plev_ - 2) - IN(p.zint, plev_ + 1);
      double adzw2 = (zk2 - zk1) / dz, adzw3 = (zk3 - zk2) / dz;
      double rhow2 = (IN(p.pmid, plev_ - 2 + 2) - IN(p.pmid, plev_ - 2 + 1)) / C_GGR / (adzw2 * dz);
      double rhow3 = (IN(p.pmid, plev_ - 3 + 2) - IN(p.pmid, plev_ - 3 + 1)) / C_GGR / (adzw3 * dz);
      PR(P_RHOW)[1] = (T)(2. * rhow2 - rhow3);
      double zn = IN(p.zmid, plev_ - nzm + 1) - IN(p.zint, plev_ + 1), zn1 = IN(p.zmid, plev_ - nzm + 2) - IN(p.zint, plev_ + 1);
      double zn2 = IN(p.zmid, plev_ - nzm + 3) - IN(p.zint, plev_ + 1);
      double adzwn = (zn - zn1) / dz, adzwn1 = (zn1 - zn2) / dz;
      double rhown = (IN(p.pmid, plev_ - nzm + 2) - IN(p.pmid, plev_ - nzm + 1)) / C_GGR / (adzwn * dz);
      double rhown1 = (IN(p.pmid, plev_ - (nzm - 1) + 2) - IN(p.pmid, plev_ - (nzm - 1) + 1)) / C_GGR / (adzwn1 * dz);
      PR(P_RHOW)[nz] = (T)(2. * rhown - rhown1);
    }
    SYNC;
    // per-level reciprocals used by the cell loops, evaluated exactly as the
    // cell loops would (same operands and order), once per column
    {
      const T dzT = (T)S.dz;
      T *adz = PR(P_ADZ), *adzw = PR(P_ADZW), *rho = PR(P_RHO), *rhow = PR(P_RHOW);
      for (int k = TID + 1; k <= nz; k += NT) {
        if (k <= nzm) {
          const int kc = min(nzm, k + 1), kb = max(1, k - 1);
          PR(P_IADZ)[k] = (T)1. / adz[k];
          PR(P_IRHO)[k] = (T)1. / rho[k];
          PR(P_IRHOADZ)[k] = (T)1. / (rho[k] * adz[k]);
          PR(P_IRHOWADZ)[k] = (T)1. / (rhow[k] * adz[k]);
          PR(P_RDZ)[k] = (T)1. / (dzT * adz[k]);
          PR(P_MPDD)[k] = (T)(double)(2.f / (float)(kc - kb)) / adz[k];
          if (k >= 2) {
            PR(P_BETU)[k] = adz[k - 1] / (adz[k] + adz[k - 1]);
            PR(P_BETD)[k] = adz[k] / (adz[k] + adz[k - 1]);
          }
          PR(P_RUP)[k] = rhow[k + 1] / rho[k] * PR(P_RDZ)[k];
          PR(P_RDN)[k] = rhow[k] / rho[k] * PR(P_RDZ)[k];
        }
        PR(P_RHOWDADZW)[k] = rhow[k] / adzw[k];
        PR(P_IADZW)[k] = (T)1. / adzw[k];
        PR(P_IRHOWADZW)[k] = (T)1. / (rhow[k] * adzw[k]);
        PR(P_RDZW)[k] = (T)1. / (dzT * adzw[k]);
      }
    }
    SYNC;
    // state in (crm_module.F90:380-397) and the first-step clamp (:400-417)
    FT u = U(), v = V(), w = W(), tabs = TABS(), qt = QT(), qp = QP(), qn = QN();
    bool clamp;
    if (p.batch_mode == CRM_REFERENCE_BATCH) {
      // the reference tests the first column of the batch only: its input
      // state is untouched until every column has passed the first barrier
      auto U0 = [&](int i, int k) { return p.st[0][(size_t)p.ld * ((i - 1) + (size_t)NH() * (k - 1))]; };
      clamp = (U0(1, 1) == U0(2, 1)) && (U0(3, 2) == U0(4, 2));
    } else {
      clamp = (p.st[0][S4(1, 1)] == p.st[0][S4(2, 1)]) && (p.st[0][S4(3, 2)] == p.st[0][S4(4, 2)]);
    }
    const double umax = (double)(0.5f * (float)p.dx / (float)p.dt);
    for (int e = TID; e < NH() * nzm; e += NT) {
      int i = 1 + e % NH(), k = 1 + e / NH();
      size_t o = S4(i, k);
      constexpr double YD = Y3 ? 1. : 0.;      // v is zero in the 2D CRM
      double uu = p.st[0][o], vv = p.st[1][o] * YD;
      if (clamp) {
        uu = mn2(umax, mx2(-umax, uu));
        vv = mn2(umax, mx2(-umax, vv)) * YD;
      }
      u(i, k) = (T)uu;
      v(i, k) = (T)vv;
      w(i, k) = (T)p.st[2][o];
      tabs(i, k) = (T)p.st[3][o];
      qt(i, k) = (T)p.st[4][o];
      qp(i, k) = (T)p.st[5][o];
      qn(i, k) = (T)p.st[6][o];
    }
    SYNC;
    micro_diagnose();
    // sgs_init grid factors (SGS_TKE/sgs.F90:213-220)
    for (int k = TID + 1; k <= nzm; k += NT) {
      T adzdz = PR(P_ADZ)[k] * (T)dz;
      PR(P_GRDFX)[k] = mn2((T)16., (T)p.dx * (T)p.dx / (adzdz * adzdz));
      PR(P_GRDFY)[k] = mn2((T)16., (T)p.dy * (T)p.dy / (adzdz * adzdz));
      PR(P_GRDFZ)[k] = (T)1.;
    }
    SYNC;
    // per-level factors of the SGS closure (tke_full), evaluated exactly as
    // its cell loops would, once per column
    {
      const T dzT = (T)S.dz, dxT = (T)p.dx, rdx0 = (T)1. / dxT, dtT = (T)p.dt;
      T *adzw = PR(P_ADZW), *bet = PR(P_BET);
      for (int k = TID + 1; k <= nz; k += NT) {
        if (k <= nzm) PR(P_RDXZ)[k] = rdx0 * tsqrt(dxT * PR(P_RDZ)[k]);
        PR(P_RDXW)[k] = rdx0 * tsqrt(dxT * PR(P_RDZW)[k]);
        if constexpr (Y3) {
          const T dyT = (T)p.dy, rdy0 = (T)1. / dyT;
          if (k <= nzm) PR(P_RDYZ)[k] = rdy0 * tsqrt(dyT * PR(P_RDZ)[k]);
          PR(P_RDYW)[k] = rdy0 * tsqrt(dyT * PR(P_RDZW)[k]);
        }
        if (k <= nzm - 1) {
          PR(P_BETDZ)[k] = (T)0.5 * (bet[k + 1] + bet[k]) / dzT / adzw[k + 1];
          T cx = dxT * dxT / dtT / PR(P_GRDFX)[k];
          T cy = (T)p.dy * (T)p.dy / dtT / PR(P_GRDFY)[k];
          T dzm = dzT * mn2(adzw[k], adzw[k + 1]);
          T cz = dzm * dzm / dtT / PR(P_GRDFZ)[k];
          PR(P_TKMAX)[k] = (T)R4(0.09) / ((T)1. / cx + (T)1. / cy + (T)1. / cz);
        }
      }
    }
    SYNC;
    tridiag_factor();
    // t from tabs (crm_module.F90:508-509)
    FT t = TT(), qcl = QCL(), qci = QCI(), qpl = QPL(), qpi = QPI(), qv = QV();
    for (int e = TID; e < NH() * nzm; e += NT) {
      int i = 1 + e % NH(), k = 1 + e / NH();
      if constexpr (sizeof(T) == 8) {
        t(i, k) = tabs(i, k) + PR(P_GAMAZ)[k] - (T)C_FAC_COND * qcl(i, k) - (T)C_FAC_SUB * qci(i, k) -
                  (T)C_FAC_COND * qpl(i, k) - (T)C_FAC_SUB * qpi(i, k);
      } else {
        // FP32-mixed form: t and qt start from the FP64 state with the
        // rounding of their FP32 values in the residue planes, so the
        // carried (value + residue) pairs hold the input state to ~1e-12
        const size_t o = S4(i, k);
        const double td = p.st[3][o] + (double)PR(P_GAMAZ)[k] - C_FAC_COND * (double)qcl(i, k) -
                          C_FAC_SUB * (double)qci(i, k) - C_FAC_COND * (double)qpl(i, k) -
                          C_FAC_SUB * (double)qpi(i, k);
        const T tf = (T)td;
        t(i, k) = tf;
        rct()[e] = (T)(td - (double)tf);
        rcq()[e] = (T)(p.st[4][o] - (double)qt(i, k));
      }
    }
    SYNC;
    // initial domain means (crm_module.F90:500-546)
    const double factor_xy = 1.0 / (double)NH();
    const double idt_gl = 1.0 / p.dt_gl;
    double *md = reinterpret_cast<double *>(sa());   // FP64 copies of the means
    {
      const int ids[9] = {P_U0, P_V0, P_T0, P_T00, P_TABS0, P_Q0, P_QV0, P_QN0, P_QP0};
      level_sums(9, 1, nzm,
                 [&](int q, int i, int k) -> T {
                   switch (q) {
                     case 0: return u(i, k);
                     case 1: return v(i, k);
                     case 2: return t(i, k);
                     case 3: return t(i, k) + (T)C_FAC_COND * qpl(i, k) + (T)C_FAC_SUB * qpi(i, k);
                     case 4: return tabs(i, k);
                     case 5: return qv(i, k) + qcl(i, k) + qci(i, k);
                     case 6: return qv(i, k);
                     case 7: return qcl(i, k) + qci(i, k);
                     default: return qpl(i, k) + qpi(i, k);
                   }
                 },
                 [&](int, int) { return 0.; },
                 [&](int q, int k, double sv) {
                   PR(ids[q])[k] = (T)(sv * factor_xy);
                   md[(size_t)q * (nz + 2) + k] = sv * factor_xy;
                 });
    }
    SYNC;
    if constexpr (sizeof(T) == 4) {
      // FP32-mixed form: the means of t (t0, t00) and of the total water (q0,
      // qv0) from the values plus their residues, in FP64: the nudging
      // tendencies below and setperturb's rescaling aim at these means, and
      // an FP32 mean would shift every cell of a level by its rounding
      const int lane = TID & 31, warp = TID >> 5, nw = NT >> 5;
      for (int k = 1 + warp; k <= nzm; k += nw) {
        double st = 0., st0 = 0., sq = 0., sv = 0.;
        for (int i = 1 + lane; i <= NH(); i += 32) {
          const size_t e = (size_t)(i - 1) + (size_t)NH() * (k - 1);
          const double tt = (double)t(i, k) + (double)rct()[e];
          const double rq = (double)rcq()[e];
          st = st + tt;
          st0 = st0 + (tt + (C_FAC_COND * (double)qpl(i, k) + C_FAC_SUB * (double)qpi(i, k)));
          sq = sq + (((double)qv(i, k) + rq) + ((double)qcl(i, k) + (double)qci(i, k)));
          sv = sv + ((double)qv(i, k) + rq);
        }
        for (int o = 16; o > 0; o >>= 1) {
          st = st + __shfl_xor_sync(0xffffffffu, st, o);
          st0 = st0 + __shfl_xor_sync(0xffffffffu, st0, o);
          sq = sq + __shfl_xor_sync(0xffffffffu, sq, o);
          sv = sv + __shfl_xor_sync(0xffffffffu, sv, o);
        }
        if (lane == 0) {
          const double m[4] = {st * factor_xy, st0 * factor_xy, sq * factor_xy, sv * factor_xy};
          const int q[4] = {2, 3, 5, 6};
          for (int a = 0; a < 4; ++a) {
            md[(size_t)q[a] * (nz + 2) + k] = m[a];
            PR(ids9(q[a]))[k] = (T)m[a];
          }
          if (k == 1) S.t_off = rintf((float)m[0]);
        }
      }
      SYNC;
    }
    for (int k = TID + 1; k <= nzm; k += NT) {
      double u0 = md[k], v0 = md[(nz + 2) + k], t00 = md[3 * (nz + 2) + k];
      double q0 = md[5 * (nz + 2) + k];
      int l = plev_ - k + 1;
      double uln = mn2(umax, mx2(-umax, IN(p.ul, l)));
      double vln = mn2(umax, mx2(-umax, IN(p.vl, l))) * (Y3 ? 1. : 0.);
      double tl = IN(p.tl, l), qccl = IN(p.qccl, l), qiil = IN(p.qiil, l), ql = IN(p.ql, l);
      double gamaz = (double)PR(P_GAMAZ)[k];
      PR(P_TTEND)[k] = (T)((tl + gamaz - C_FAC_COND * (qccl + qiil) - C_FAC_FUS * qiil - t00) * idt_gl);
      PR(P_QTEND)[k] = (T)((ql + qccl + qiil - q0) * idt_gl);
      PR(P_UTEND)[k] = (T)((uln - u0) * idt_gl);
      PR(P_VTEND)[k] = (T)((vln - v0) * idt_gl);
    }
    // column precipitation at the start (prectend, precstend)
    if (TID == 0) {
      double cp = 0, cps = 0;
      for (int k = 1; k <= nzm; ++k) {
        double pdel = IN(p.pdel, plev_ - k + 1);
        for (int i = 1; i <= NH(); ++i) {
          cp = cp + (double)(qpl(i, k) + qpi(i, k)) * pdel;
          cps = cps + (double)qpi(i, k) * pdel;
        }
      }
      S.colprec0 = cp;
      S.colprecs0 = cps;
      S.cltot = S.clhgh = S.clmed = S.cllow = 0.;
    }
    SYNC;
    precip_init();
    // setperturb (setperturb.F90:33-80) with draws precomputed on the host
    if (p.igstep <= 1) {
      const double fxy = 1. / (double)NH();
      for (int k = TID + 1; k <= 5; k += NT) {
        double scaling = (double)(5 + 1 - k) / (double)5;
        double t02 = 0.0;
        const double *r = p.rnd + ((size_t)icrm * 5 + (k - 1)) * NH();
        if constexpr (sizeof(T) == 8) {
          for (int i = 1; i <= NH(); ++i) {
            t(i, k) = t(i, k) + (T)(1.0 * r[i - 1] * scaling);
            t02 = t02 + (double)t(i, k) * fxy;
          }
          T t0k = PR(P_T0)[k];
          for (int i = 1; i <= NH(); ++i) t(i, k) = (T)((double)(t(i, k) * t0k) / t02);
        } else {
          // FP32-mixed form: the perturbed t and its rescaling to the level
          // mean t0 in FP64 on the (value + residue) pairs
          T *rt = rct() + (size_t)NH() * (k - 1);
          for (int i = 1; i <= NH(); ++i) {
            const double tt = ((double)t(i, k) + (double)rt[i - 1]) + 1.0 * r[i - 1] * scaling;
            t02 = t02 + tt * fxy;
          }
          const double t0k = md[2 * (nz + 2) + k];
          for (int i = 1; i <= NH(); ++i) {
            const double tt = (((double)t(i, k) + (double)rt[i - 1]) + 1.0 * r[i - 1] * scaling) * t0k / t02;
            const T tf = (T)tt;
            t(i, k) = tf;
            rt[i - 1] = (T)(tt - (double)tf);
          }
        }
      }
      SYNC;
    }
  }

  // ---------------------------------------------------------- kurant
  // kurant.F90:31-64 and kurant_sgs (SGS_TKE/sgs.F90:342-367); per column
  __device__ void kurant() {
    FT u = U(), w = W(), tkh = TKH();
    T *wm = PR(P_TMP0), *uhm = PR(P_TMP1), *tkhm = PR(P_TMP2);
    // the horizontal speed of the 2D reference is sqrt(u*u + 0*(v*v)); for
    // a finite v the second term is +0 and the sum is u*u exactly, so v is
    // not read.  The same pass screens u, w and tkh for NaN/Inf: every
    // prognostic field feeds w (buoyancy) or u and tkh within a step, so a
    // column whose state stops being finite is caught at the next step.
    bool bad = false;
    FT v = V();
    // one warp per level takes the three maxima from one pass over the
    // level's cells (maxima are order-independent, hence exact)
    {
      const int lane = TID & 31, warp = TID >> 5, nw = NT >> 5;
      for (int k = 1 + warp; k <= nzm; k += nw) {
        T mw = (T)0, mu = (T)0, mt = (T)0;
        for (int i = 1 + lane; i <= NH(); i += 32) {
          const T ww = w(i, k), uu = u(i, k), th = tkh(i, k);
          bad |= !isfinite(ww) || !isfinite(uu) || !isfinite(th);
          mw = mx2(mw, tabs_(ww));
          if constexpr (Y3) {
            const T vv = v(i, k);
            bad |= !isfinite(vv);
            mu = mx2(mu, tsqrt(uu * uu + (T)1. * (vv * vv)));
          } else {
            mu = mx2(mu, tsqrt(uu * uu));
          }
          mt = mx2(mt, th);
        }
        for (int o = 16; o > 0; o >>= 1) {
          mw = mx2(mw, __shfl_xor_sync(0xffffffffu, mw, o));
          mu = mx2(mu, __shfl_xor_sync(0xffffffffu, mu, o));
          mt = mx2(mt, __shfl_xor_sync(0xffffffffu, mt, o));
        }
        if (lane == 0) { wm[k] = mw; uhm[k] = mu; tkhm[k] = mt; }
      }
    }
    if (TID == 0) wm[nz] = (T)0.;
    const int nonfinite = __syncthreads_or(bad);
    double cfl = 0.;
    const double rdx = 1. / p.dx;
    for (int k = TID + 1; k <= nzm; k += NT) {
      double dza = S.dz * (double)PR(P_ADZW)[k];
      constexpr double YD = Y3 ? 1. : 0.;
      constexpr float YF = Y3 ? 1.f : 0.f;
      double t1 = mx2((double)uhm[k] * p.dt * sqrt(rdx * rdx + YD * ((1. / p.dy) * (1. / p.dy))),
                      mx2((double)wm[k], (double)wm[k + 1]) * p.dt / dza);
      double tk = (double)tkhm[k];
      double t2 = mx3(0.5 * tk * (double)PR(P_GRDFZ)[k] * p.dt / (dza * dza),
                      0.5 * tk * (double)PR(P_GRDFX)[k] * p.dt / (p.dx * p.dx),
                      (double)(YF * 0.5f) * tk * (double)PR(P_GRDFY)[k] * p.dt / (p.dy * p.dy));
      cfl = mx2(cfl, mx2(t1, t2));
    }
    cfl = block_max(cfl);
    // a non-finite column enters the batch maximum as an unbounded CFL, so
    // in reference-batch mode every column of the call stops at this step
    // (the reference would have aborted the model) instead of waiting at a
    // grid barrier the stopped column never reaches
    if (nonfinite) cfl = kCflNonfinite;
    const double cfl_b = batch_max(cfl);
    if (TID == 0) {
      S.cfl = cfl;
      if (nonfinite && S.status == CRM_OK) S.status = CRM_ERR_NONFINITE;
      S.ncycle = ncycle_of(cfl_b);
    }
    SYNC;
  }

  // ---------------------------------------------------------- abcoefs
  __device__ void abcoefs(int nstep) {        // abcoefs.F90:7-31 (thread 0)
    if (nstep >= 3) {
      double alpha = S.dt3[S.nb - 1] / S.dt3[S.na - 1];
      double beta = S.dt3[S.nc - 1] / S.dt3[S.na - 1];
      S.ct = (2. + 3. * alpha) / (6. * (alpha + beta) * beta);
      S.bt = -(1. + 2. * (alpha + beta) * S.ct) / (2. * alpha);
      S.at = 1. - S.bt - S.ct;
    } else if (nstep >= 2) {
      S.at = 3. / 2.; S.bt = -1. / 2.; S.ct = 0.;
    } else {
      S.at = 1.; S.bt = 0.; S.ct = 0.;
    }
  }

  // ---------------------------------------------------------- zero, buoyancy
  __device__ void zero_and_buoyancy() {       // zero.F90:17-29, buoyancy.F90:15-37
    FT du = DU(S.na), dv = DV(S.na), dw = DW(S.na);
    if constexpr (Y3) {                  // the whole arrays, x and y halos included
      const size_t nu = (size_t)(nx + 1) * p.L.yi.nxa * nzm, nv = (size_t)nx * p.L.ydv.nxa * nzm;
      for (size_t e = TID; e < nu; e += NT) du.p[e] = (T)0.;
      for (size_t e = TID; e < nv; e += NT) dv.p[e] = (T)0.;
    } else {
      for (int e = TID; e < (nx + 1) * nzm; e += NT) { int i = 1 + e % (nx + 1), k = 1 + e / (nx + 1); du(i, k) = (T)0.; }
      for (int e = TID; e < nx * nzm; e += NT) { int i = 1 + e % nx, k = 1 + e / nx; dv(i, k) = (T)0.; }
    }
    FT tabs = TABS(), qv = QV(), qcl = QCL(), qci = QCI(), qpl = QPL(), qpi = QPI();
    const T epsv = (T)C_EPSV;
    T *adz = PR(P_ADZ), *bet = PR(P_BET), *tabs0 = PR(P_TABS0), *qv0 = PR(P_QV0), *qn0 = PR(P_QN0), *qp0 = PR(P_QP0);
    for (int e = TID; e < NH() * nz; e += NT) {
      int i = 1 + e % NH(), k = 1 + e / NH();
      if (k >= 2 && k <= nzm) {
        int kb = k - 1;
        T betu = PR(P_BETU)[k];
        T betd = PR(P_BETD)[k];
        dw(i, k) = (T)0. +
            bet[k] * betu *
                (tabs0[k] * (epsv * (qv(i, k) - qv0[k]) - (qcl(i, k) + qci(i, k) - qn0[k] + qpl(i, k) + qpi(i, k) - qp0[k])) +
                 (tabs(i, k) - tabs0[k]) * ((T)1. + epsv * qv0[k] - qn0[k] - qp0[k])) +
            bet[kb] * betd *
                (tabs0[kb] * (epsv * (qv(i, kb) - qv0[kb]) - (qcl(i, kb) + qci(i, kb) - qn0[kb] + qpl(i, kb) + qpi(i, kb) - qp0[kb])) +
                 (tabs(i, kb) - tabs0[kb]) * ((T)1. + epsv * qv0[kb] - qn0[kb] - qp0[kb]));
      } else {
        dw(i, k) = (T)0.;
      }
    }
    SYNC;
  }

  // ---------------------------------------------------------- forcing + radiation
  __device__ void forcing_radiation() {       // forcing.F90:31-74, crm_module.F90:766-777
    FT t = TT(), qt = QT(), du = DU(S.na), dv = DV(S.na);
    const T dtn = (T)S.dtn;
    T *ttend = PR(P_TTEND), *qtend = PR(P_QTEND), *utend = PR(P_UTEND), *vtend = PR(P_VTEND);
    // The FP32-mixed form adds the steady forcing through the carried
    // residues (add_carry): rounded the same way every step, -1.5 K/day at
    // dt 10 s would be biased by up to ~5 %.  Its t forcing is added after
    // the fixer below, which does not read t.
    T *rc_t = rct(), *rc_q = rcq();
    int neg_any = 0;
    for (int e = TID; e < NH() * nzm; e += NT) {
      int i = 1 + e % NH(), k = 1 + e / NH();
      if constexpr (sizeof(T) == 8) {
        t(i, k) = t(i, k) + ttend[k] * dtn;
        qt(i, k) = qt(i, k) + qtend[k] * dtn;
      } else {
        qt(i, k) = add_carry(qt(i, k), qtend[k] * dtn, rc_q[e]);
      }
      neg_any |= qt(i, k) < (T)0.;
      du(i, k) = du(i, k) + utend[k];
      dv(i, k) = dv(i, k) + vtend[k];
    }
    const int qrad_base = 5;
    const int gx = NH() / NR(), nxr = NR();
    const T *qrad = base + p.L.rad + (size_t)qrad_base * nxr * nzm;    // (nx_rad, nzm), cached at init
    if (!__syncthreads_or(neg_any)) {
      // no negative qt in the column: every level's count is zero and the
      // fixer below changes nothing (its sums are skipped)
      for (int e = TID; e < NH() * nzm; e += NT) {
        int i = 1 + e % NH(), k = 1 + e / NH();
        int i_rad = (i - 1) / gx + 1;
        T qr = qrad[(size_t)(k - 1) * nxr + (i_rad - 1)];
        if constexpr (sizeof(T) == 8) t(i, k) = t(i, k) + qr * dtn;
        else t(i, k) = add_carry(t(i, k), ttend[k] * dtn + qr * dtn, rc_t[e]);
      }
      SYNC;
      return;
    }
    // negative-vapour fixer: per-level sums (a cell outside a sum adds an
    // exact zero, which leaves a sum that starts at +0 unchanged)
    T *qneg = PR(P_TMP0), *qpoz = PR(P_TMP1), *nneg = PR(P_TMP2);
    level_sums_multi<3>(1, nzm,
               [&](int q, int i, int k) -> T {
                 T v = qt(i, k);
                 bool neg = v < (T)0.;
                 if (q == 0) return neg ? v : (T)0.;
                 if (q == 1) return neg ? (T)0. : v;
                 return neg ? (T)1. : (T)0.;
               },
               [&](int i, int k, T *r) {
                 const T v = qt(i, k);
                 const bool neg = v < (T)0.;
                 r[0] = neg ? v : (T)0.;
                 r[1] = neg ? (T)0. : v;
                 r[2] = neg ? (T)1. : (T)0.;
               },
               [&](int, int) { return 0.; },
               [&](int q, int k, double sv) { (q == 0 ? qneg : q == 1 ? qpoz : nneg)[k] = (T)sv; });
    SYNC;
    for (int e = TID; e < NH() * nzm; e += NT) {
      int i = 1 + e % NH(), k = 1 + e / NH();
      if (nneg[k] > (T)0. && qpoz[k] + qneg[k] > (T)0.) {
        T factor = (T)1. + qneg[k] / qpoz[k];
        qt(i, k) = mx2((T)0., qt(i, k) * factor);
      }
      int i_rad = (i - 1) / gx + 1;
      T qr = qrad[(size_t)(k - 1) * nxr + (i_rad - 1)];
      if constexpr (sizeof(T) == 8) {
        t(i, k) = t(i, k) + qr * dtn;
      } else {
        t(i, k) = add_carry(t(i, k), ttend[k] * dtn + qr * dtn, rc_t[e]);
      }
    }
    SYNC;
  }

  // ---------------------------------------------------------- damping
  __device__ void damping() {                  // damping.F90:44-107
    T *z = PR(P_Z);
    if (TID == 0) {
      int n_damp = 0;
      for (int k = nzm; k >= 1; --k)
        if (z[nzm] - z[k] < (T)R4(0.4) * z[nzm]) n_damp = nzm - k + 1;
      S.n_damp = n_damp;
    }
    SYNC;
    const int n_damp = S.n_damp;
    FT u = U(), v = V(), t = TT();
    T *tau = PR(P_TMP0), *u0l = PR(P_TMP1), *v0l = PR(P_TMP2), *t0l = PR(P_TMP3);
    const T nxy = (T)(double)NH();
    for (int k = TID + 1; k <= nzm; k += NT) {
      if (k >= nzm - n_damp) {
        T tk = (T)60. * tpow((T)450. / (T)60., (z[nzm] - z[k]) / (z[nzm] - z[nzm - n_damp]));
        tau[k] = (T)1. / tk;
      }
    }
    // the level means only where the sponge acts (each level's sum is
    // independent of the others); the FP32-mixed form takes t's in FP64 below
    level_sums_lo(sizeof(T) == 8 ? 3 : 2, max(1, nzm - n_damp), nzm,
               [&](int q, int i, int k) -> T { return (q == 0 ? u(i, k) : q == 1 ? v(i, k) : t(i, k)) / nxy; },
               [&](int, int) { return 0.; },
               [&](int q, int k, double sv) { (q == 0 ? u0l : q == 1 ? v0l : t0l)[k] = (T)sv; });
    // FP32-mixed form: the sponge relaxes t towards its level mean strongly
    // (up to dtn/60 s per step), so an FP32 mean, off by up to half a unit
    // in the last place, would pull the whole sponge layer by that much; the
    // mean of t plus its residue is taken in FP64 instead
    double *t0d = reinterpret_cast<double *>(sa());
    if constexpr (sizeof(T) == 4) {
      const int lane = TID & 31, warp = TID >> 5, nw = NT >> 5;
      for (int k = nzm - n_damp + warp; k <= nzm; k += nw) {
        if (k < 1) continue;
        double s = 0.;
        for (int i = 1 + lane; i <= NH(); i += 32) s = s + ((double)t(i, k) + (double)rct()[(size_t)(i - 1) + (size_t)NH() * (k - 1)]);
        for (int o = 16; o > 0; o >>= 1) s = s + __shfl_xor_sync(0xffffffffu, s, o);
        if (lane == 0) t0d[k] = s / (double)NH();
      }
    }
    SYNC;
    FT w = W(), qt = QT(), qv = QV(), du = DU(S.na), dv = DV(S.na), dw = DW(S.na);
    const T dtn = (T)S.dtn;
    T *qv0 = PR(P_QV0);
    for (int e = TID; e < NH() * nzm; e += NT) {
      int i = 1 + e % NH(), k = 1 + e / NH();
      if (k >= nzm - n_damp) {
        du(i, k) = du(i, k) - (u(i, k) - u0l[k]) * tau[k];
        dv(i, k) = dv(i, k) - (v(i, k) - v0l[k]) * tau[k];
        dw(i, k) = dw(i, k) - w(i, k) * tau[k];
        if constexpr (sizeof(T) == 8) {
          t(i, k) = t(i, k) - dtn * (t(i, k) - t0l[k]) * tau[k];
          qt(i, k) = qt(i, k) - dtn * (qv(i, k) - qv0[k]) * tau[k];
        } else {
          const size_t o = (size_t)(i - 1) + (size_t)NH() * (k - 1);
          const T anom = (T)(((double)t(i, k) + (double)rct()[o]) - t0d[k]);
          t(i, k) = add_carry(t(i, k), -(dtn * anom * tau[k]), rct()[o]);
          qt(i, k) = add_carry(qt(i, k), -(dtn * (qv(i, k) - qv0[k]) * tau[k]), rcq()[o]);
        }
      }
    }
    SYNC;
  }

  // ---------------------------------------------------------- ice_fall
  __device__ void ice_fall() {                 // ice_fall.F90:26-167
    FT qcl = QCL(), qci = QCI(), tabs = TABS();
    int kmin = nzm + 1, kmax = 0;
    for (int e = TID; e < NH() * nzm; e += NT) {
      int i = 1 + e % NH(), k = 1 + e / NH();
      if (qcl(i, k) + qci(i, k) > (T)0. && tabs(i, k) < (T)R4(273.15)) {
        kmin = min(kmin, k);
        kmax = max(kmax, k);
      }
    }
    for (int o = 16; o > 0; o >>= 1) {
      kmin = min(kmin, __shfl_xor_sync(0xffffffffu, kmin, o));
      kmax = max(kmax, __shfl_xor_sync(0xffffffffu, kmax, o));
    }
    if ((TID & 31) == 0) { S.red_i[TID >> 5] = kmin; S.red_i[32 + (TID >> 5)] = kmax; }
    SYNC;
    if (TID == 0) {
      int a = nzm + 1, b = 0;
      for (int w = 0; w < NT / 32; ++w) { a = min(a, S.red_i[w]); b = max(b, S.red_i[32 + w]); }
      S.kmin = a; S.kmax = b;
    }
    SYNC;
    kmin = S.kmin; kmax = S.kmax;
    if (kmax == 0) return;                     // no ice cloud: nothing falls
    FT fz = SA();
    T *adz = PR(P_ADZ), *rho = PR(P_RHO);
    const T dtn = (T)S.dtn, dz = (T)S.dz;
    for (int e = TID; e < NH() * nz; e += NT) {
      int i = 1 + e % NH(), k = 1 + e / NH();
      T f = (T)0.;
      if (k >= max(1, kmin - 1) && k <= kmax) {
        int kc = min(nzm, k + 1), kb = max(1, k - 1);
        T coef = dtn / ((T)0.5 * (adz[kb] + adz[k]) * dz);
        T qiu = rho[kc] * qci(i, kc);
        T qic = rho[k] * qci(i, k);
        T qid = rho[kb] * qci(i, kb);
        T vt_ice = mn2((T)R4(0.4), (T)R4(8.66) * tpow(mx2((T)0., qic) + (T)R4(1.e-10), (T)R4(0.24)));
        T tmp_phi;
        if (tabs_(qic - qid) < (T)R4(1.0e-25)) tmp_phi = (T)0.;
        else {
          T tmp_theta = (qiu - qic) / (qic - qid);
          tmp_phi = mx2((T)0., mn3((T)0.5 * ((T)1. + tmp_theta), (T)2., (T)2. * tmp_theta));
        }
        f = -vt_ice * (qic - (T)0.5 * ((T)1. - coef * vt_ice) * tmp_phi * (qic - qid));
      }
      if (k == nz) f = (T)0.;
      fz(i, k) = f;
    }
    SYNC;
    FT qt = QT(), t = TT();
    for (int e = TID; e < NH() * nzm; e += NT) {
      int i = 1 + e % NH(), k = 1 + e / NH();
      if (k >= max(1, kmin - 2) && k <= kmax) {
        T coef = dtn / (dz * adz[k] * rho[k]);
        T dqi = coef * (fz(i, k) - fz(i, k + 1));
        T lat_heat = (T)(C_FAC_COND + C_FAC_FUS) * dqi;
        if constexpr (sizeof(T) == 8) {
          qt(i, k) = qt(i, k) + dqi;
          t(i, k) = t(i, k) - lat_heat;
        } else {
          // FP32-mixed form: through the carried residues
          qt(i, k) = add_carry(qt(i, k), dqi, rcq()[e]);
          t(i, k) = add_carry(t(i, k), -lat_heat, rct()[e]);
        }
      }
    }
    for (int i = TID + 1; i <= NH(); i += NT) {
      T coef = dtn / dz;
      T dqi = -coef * fz(i, 1);
      PS(i) = PS(i) + dqi;
      PSS(i) = PSS(i) + dqi;
    }
    SYNC;
  }

  // ---------------------------------------------------------- SGS TKE, 3D
#define SQ(x) ((x) * (x))
  // SGS_TKE/shear_prod3D.F90:14-138 into def2(i, j, k); the per-level
  // factors rdx, rdy (grid anisotropy) come from the column's tables
  __device__ void shear_prod3(FT def2) {
    FT u = U(), v = V(), w = W();
    T *u0 = PR(P_U0), *v0 = PR(P_V0);
    const int nxy = nx * ny;
    for (int e = TID; e < nxy * nzm; e += NT) {
      const int i = 1 + e % nx, j = 1 + (e / nx) % ny, k = 1 + e / nxy;
      const int ib = i - 1, ic = i + 1, jb = j - 1, jc = j + 1;
      const T rdz = PR(P_RDZ)[k], rdx = PR(P_RDXZ)[k], rdy = PR(P_RDYZ)[k];
      // horizontal shear, shared by every level branch
      T r = (T)2. * (SQ((u(ic, j, k) - u(i, j, k)) * rdx) + SQ((v(i, jc, k) - v(i, j, k)) * rdy) +
                     SQ((w(i, j, k + 1) - w(i, j, k)) * rdz)) +
            (T)0.25 * (SQ((u(ic, jc, k) - u(ic, j, k)) * rdy + (v(ic, jc, k) - v(i, jc, k)) * rdx) +
                       SQ((u(i, jc, k) - u(i, j, k)) * rdy + (v(i, jc, k) - v(ib, jc, k)) * rdx) +
                       SQ((u(ic, j, k) - u(ic, jb, k)) * rdy + (v(ic, j, k) - v(i, j, k)) * rdx) +
                       SQ((u(i, j, k) - u(i, jb, k)) * rdy + (v(i, j, k) - v(ib, j, k)) * rdx));
      if (k >= 2 && k <= nzm - 1) {
        const int kb = k - 1, kc = k + 1;
        const T rzu = PR(P_RDZW)[kc], rzd = PR(P_RDZW)[k];
        const T rxu = PR(P_RDXW)[kc], rxd = PR(P_RDXW)[k], ryu = PR(P_RDYW)[kc], ryd = PR(P_RDYW)[k];
        r = r + (T)0.25 * (SQ((u(ic, j, kc) - u0[kc] - u(ic, j, k) + u0[k]) * rzu + (w(ic, j, kc) - w(i, j, kc)) * rxu) +
                           SQ((u(i, j, kc) - u0[kc] - u(i, j, k) + u0[k]) * rzu + (w(i, j, kc) - w(ib, j, kc)) * rxu) +
                           SQ((u(ic, j, k) - u0[k] - u(ic, j, kb) + u0[kb]) * rzd + (w(ic, j, k) - w(i, j, k)) * rxd) +
                           SQ((u(i, j, k) - u0[k] - u(i, j, kb) + u0[kb]) * rzd + (w(i, j, k) - w(ib, j, k)) * rxd));
        r = r + (T)0.25 * (SQ((v(i, jc, kc) - v0[kc] - v(i, jc, k) + v0[k]) * rzu + (w(i, jc, kc) - w(i, j, kc)) * ryu) +
                           SQ((v(i, j, kc) - v0[kc] - v(i, j, k) + v0[k]) * rzu + (w(i, j, kc) - w(i, jb, kc)) * ryu) +
                           SQ((v(i, jc, k) - v0[k] - v(i, jc, kb) + v0[kb]) * rzd + (w(i, jc, k) - w(i, j, k)) * ryd) +
                           SQ((v(i, j, k) - v0[k] - v(i, j, kb) + v0[kb]) * rzd + (w(i, j, k) - w(i, jb, k)) * ryd));
      } else if (k == 1) {
        const int kc = k + 1;
        const T rzu = PR(P_RDZW)[kc], rxu = PR(P_RDXW)[kc], ryu = PR(P_RDYW)[kc];
        r = r + (T)0.5 * (SQ((v(i, jc, kc) - v0[kc] - v(i, jc, k) + v0[k]) * rzu + (w(i, jc, kc) - w(i, j, kc)) * ryu) +
                          SQ((v(i, j, kc) - v0[kc] - v(i, j, k) + v0[k]) * rzu + (w(i, j, kc) - w(i, jb, kc)) * ryu));
        r = r + (T)0.5 * (SQ((u(ic, j, kc) - u0[kc] - u(ic, j, k) + u0[k]) * rzu + (w(ic, j, kc) - w(i, j, kc)) * rxu) +
                          SQ((u(i, j, kc) - u0[kc] - u(i, j, k) + u0[k]) * rzu + (w(i, j, kc) - w(ib, j, kc)) * rxu));
      } else {
        const int kb = k - 1;
        const T rzd = PR(P_RDZW)[k], rxd = PR(P_RDXW)[k], ryd = PR(P_RDYW)[k];
        r = r + (T)0.5 * (SQ((v(i, jc, k) - v0[k] - v(i, jc, kb) + v0[kb]) * rzd + (w(i, jc, k) - w(i, j, k)) * ryd) +
                          SQ((v(i, j, k) - v0[k] - v(i, j, kb) + v0[kb]) * rzd + (w(i, j, k) - w(i, jb, k)) * ryd));
        r = r + (T)0.5 * (SQ((u(ic, j, k) - u0[k] - u(ic, j, kb) + u0[kb]) * rzd + (w(ic, j, k) - w(i, j, k)) * rxd) +
                          SQ((u(i, j, k) - u0[k] - u(i, j, kb) + u0[kb]) * rzd + (w(i, j, k) - w(ib, j, k)) * rxd));
      }
      def2(i, j, k) = r;
    }
  }

  // ---------------------------------------------------------- SGS TKE
  // shear_prod2D.F90:14-95 + tke_full.F90:108-312 (dosmagor = .true.)
  __device__ void tke_full() {
    FT u = U(), v = V(), w = W(), def2 = SA(), buoy = SB(), aprod = SCR(p.L.s_c);
    T *u0 = PR(P_U0), *v0 = PR(P_V0), *adz = PR(P_ADZ), *adzw = PR(P_ADZW);
    const T dz = (T)S.dz, dx = (T)p.dx;
    const T rdx0 = (T)1. / dx;
    if constexpr (Y3) shear_prod3(def2);
    else
    for (int e = TID; e < nx * nzm; e += NT) {
      int i = 1 + e % nx, k = 1 + e / nx;
      int ib = i - 1, ic = i + 1;
      T r;
      if (k >= 2 && k <= nzm - 1) {
        int kb = k - 1, kc = k + 1;
        T rdz = PR(P_RDZ)[k];
        T rdzw_up = PR(P_RDZW)[kc];
        T rdzw_dn = PR(P_RDZW)[k];
        T rdx = PR(P_RDXZ)[k];
        T rdx_up = PR(P_RDXW)[kc];
        T rdx_dn = PR(P_RDXW)[k];
        r = (T)2. * (SQ((u(ic, k) - u(i, k)) * rdx) + SQ((w(i, kc) - w(i, k)) * rdz)) +
            (T)0.5 * (SQ((v(ic, k) - v(i, k)) * rdx) + SQ((v(i, k) - v(ib, k)) * rdx) +
                      SQ((u(ic, kc) - u0[kc] - u(ic, k) + u0[k]) * rdzw_up + (w(ic, kc) - w(i, kc)) * rdx_up) +
                      SQ((u(i, kc) - u0[kc] - u(i, k) + u0[k]) * rdzw_up + (w(i, kc) - w(ib, kc)) * rdx_up) +
                      SQ((u(ic, k) - u0[k] - u(ic, kb) + u0[kb]) * rdzw_dn + (w(ic, k) - w(i, k)) * rdx_dn) +
                      SQ((u(i, k) - u0[k] - u(i, kb) + u0[kb]) * rdzw_dn + (w(i, k) - w(ib, k)) * rdx_dn) +
                      SQ((v(i, kc) - v0[kc] - v(i, k) + v0[k]) * rdzw_up) +
                      SQ((v(i, k) - v0[k] - v(i, kb) + v0[kb]) * rdzw_dn));
      } else if (k == 1) {
        int kc = k + 1;
        T rdz = PR(P_RDZ)[k];
        T rdzw_up = PR(P_RDZW)[kc];
        T rdx = PR(P_RDXZ)[k];
        T rdx_up = PR(P_RDXW)[kc];
        r = (T)2. * (SQ((u(ic, k) - u(i, k)) * rdx) + SQ((w(i, kc) - w(i, k)) * rdz)) +
            (T)0.5 * (SQ((v(ic, k) - v(i, k)) * rdx) + SQ((v(i, k) - v(ib, k)) * rdx)) +
            SQ((v(i, kc) - v0[kc] - v(i, k) + v0[k]) * rdzw_up) +
            (T)0.5 * (SQ((u(ic, kc) - u0[kc] - u(ic, k) + u0[k]) * rdzw_up + (w(ic, kc) - w(i, kc)) * rdx_up) +
                      SQ((u(i, kc) - u0[kc] - u(i, k) + u0[k]) * rdzw_up + (w(i, kc) - w(ib, kc)) * rdx_up));
      } else {
        int kc = k + 1, kb = k - 1;
        T rdz = PR(P_RDZ)[k];
        T rdzw_dn = PR(P_RDZW)[k];
        T rdx = PR(P_RDXZ)[k];
        T rdx_dn = PR(P_RDXW)[k];
        r = (T)2. * (SQ((u(ic, k) - u(i, k)) * rdx) + SQ((w(i, kc) - w(i, k)) * rdz)) +
            (T)0.5 * (SQ((v(ic, k) - v(i, k)) * rdx) + SQ((v(i, k) - v(ib, k)) * rdx)) +
            SQ((v(i, k) - v0[k] - v(i, kb) + v0[kb]) * rdzw_dn) +
            (T)0.5 * (SQ((u(ic, k) - u0[k] - u(ic, kb) + u0[kb]) * rdzw_dn + (w(ic, k) - w(i, k)) * rdx_dn) +
                      SQ((u(i, k) - u0[k] - u(i, kb) + u0[kb]) * rdzw_dn + (w(i, k) - w(ib, k)) * rdx_dn));
      }
      def2(i, k) = r;
    }
    // SGS buoyancy flux at the interfaces k+1/2, k = 1..nzm-1
    FT tabs = TABS(), qv = QV(), qcl = QCL(), qci = QCI(), qpl = QPL(), qpi = QPI(), t = TT(), tkh = TKH();
    T *bet = PR(P_BET), *presi = PR(P_PRESI);
    const T epsv = (T)C_EPSV, fc = (T)C_FAC_COND, fs = (T)C_FAC_SUB, ff = (T)C_FAC_FUS;
    for (int e = TID; e < NH() * (nzm + 1); e += NT) {
      int i = 1 + e % NH(), k = e / NH();     // k = 0..nzm
      if (k == 0 || k == nzm) { buoy(i, k) = (T)0.; aprod(i, k) = (T)0.; continue; }
      int kc = k + 1, kb = k;
      T betdz = PR(P_BETDZ)[k];
      T tabs_if = (T)0.5 * (tabs(i, kc) + fc * qcl(i, kc) + fs * qci(i, kc) + tabs(i, kb) + fc * qcl(i, kb) + fs * qci(i, kb));
      T qtot_if = (T)0.5 * (qv(i, kc) + qcl(i, kc) + qci(i, kc) + qv(i, kb) + qcl(i, kb) + qci(i, kb));
      T qp_if = (T)0.5 * (qpl(i, kc) + qpi(i, kc) + qpl(i, kb) + qpi(i, kb));
      T bbb = (T)1. + epsv * qtot_if - qp_if;
      T dqtot = qv(i, kc) + qcl(i, kc) + qci(i, kc) - qv(i, kb) - qcl(i, kb) - qci(i, kb);
      T dtk = t(i, kc) - t(i, kb);
      if constexpr (sizeof(T) == 4) {
        // FP32-mixed form: the vertical differences of t and of the total
        // water with their carried residues.  In a well-mixed layer the
        // difference of t is a few FP32 units of ~300 K, and the residues
        // (up to half a unit each) changed the stability, hence tk and tkh,
        // by ~1e-3 and the boundary layer's heat flux with them.
        const size_t oc = (size_t)(i - 1) + (size_t)NH() * (kc - 1), ob = (size_t)(i - 1) + (size_t)NH() * (kb - 1);
        dtk = dtk + (rct()[oc] - rct()[ob]);
        dqtot = dqtot + (rcq()[oc] - rcq()[ob]);
      }
      T bs = betdz * (bbb * dtk + epsv * tabs_if * dqtot +
                      (bbb * fc - tabs_if) * (qpl(i, kc) - qpl(i, kb)) + (bbb * fs - tabs_if) * (qpi(i, kc) - qpi(i, kb)));
      T ap = (T)-0.5 * (tkh(i, kc) + tkh(i, kb) + (T)R4(0.002)) * bs;
      T qctot = qcl(i, kc) + qci(i, kc) + qcl(i, kb) + qci(i, kb);
      if (qctot > (T)0.) {
        T omn = (qcl(i, kc) + qcl(i, kb)) / (qctot + (T)R4(1.e-20));
        T qsat_check = omn * qsatw(tabs_if, presi[k + 1]) + ((T)1. - omn) * qsati(tabs_if, presi[k + 1]);
        if (qtot_if > qsat_check) {
          T lstarn = fc + ((T)1. - omn) * ff;
          T tif = (T)0.5 * (tabs(i, kc) + tabs(i, kb));
          T qpif = (T)0.5 * (qpl(i, kc) + qpi(i, kc) + qpl(i, kb) + qpi(i, kb));
          T dqsat = omn * dtqsatw(tif, presi[k + 1]) + ((T)1. - omn) * dtqsati(tif, presi[k + 1]);
          T qsatt = omn * qsatw(tif, presi[k + 1]) + ((T)1. - omn) * qsati(tif, presi[k + 1]);
          T b2 = (T)1. + epsv * qsatt + qsatt - qtot_if - qpif + (T)R4(1.61) * tif * dqsat;
          b2 = b2 / ((T)1. + lstarn * dqsat);
          bs = betdz * (b2 * dtk + (b2 * lstarn - ((T)1. + lstarn * dqsat) * tif) * dqtot +
                        (b2 * fc - ((T)1. + fc * dqsat) * tabs(i, k)) * (qpl(i, kc) - qpl(i, kb)) +
                        (b2 * fs - ((T)1. + fs * dqsat) * tabs(i, k)) * (qpi(i, kc) - qpi(i, kb)));
          ap = (T)-0.5 * (tkh(i, kc) + tkh(i, kb) + (T)R4(0.002)) * bs;
        }
      }
      buoy(i, k) = bs;
      aprod(i, k) = ap;
    }
    SYNC;
    // eddy viscosity / conductivity (Smagorinsky), levels 1..nzm-1
    FT tk = TK(), tke = TKE();
    const T Cs = (T)R4(0.15), Ck = (T)R4(0.1);
    const T Ce = Ck * Ck * Ck / ((Cs * Cs) * (Cs * Cs));
    const T Pr = (T)1.;
    const T dt = (T)p.dt;
    T *grdfx = PR(P_GRDFX), *grdfy = PR(P_GRDFY), *grdfz = PR(P_GRDFZ);
    for (int e = TID; e < NH() * (nzm - 1); e += NT) {
      int i = 1 + e % NH(), k = 1 + e / NH();
      T grd = dz * adz[k];
      T Ce1 = Ce / (T)R4(0.7) * (T)R4(0.19);
      T Ce2 = Ce / (T)R4(0.7) * (T)R4(0.51);
      T tkmax = PR(P_TKMAX)[k];
      T bs = (T)0.5 * (buoy(i, k - 1) + buoy(i, k));
      T smix;
      if (bs <= (T)0.) smix = grd;
      else smix = mn2(grd, mx2((T)R4(0.1) * grd, tsqrt((T)R4(0.76) * tk(i, k) / Ck / tsqrt(bs + (T)R4(1.e-10)))));
      T ratio = smix / grd;
      T Cee = Ce1 + Ce2 * ratio;
      T tkv = tsqrt(Ck * Ck * Ck / Cee * mx2((T)0., def2(i, k) - Pr * bs)) * (smix * smix);
      T tq = tkv / (Ck * smix);
      tke(i, k) = tq * tq;
      tkv = mn2(tkv, tkmax);
      tk(i, k) = tkv;
      tkh(i, k) = Pr * tkv;
    }
    SYNC;
#undef SQ
  }

  // ---------------------------------------------------------- advect_mom, 3D
  // advect2_mom_xy.F90:23-57 (RUN3D) and advect2_mom_z.F90:30-122
  __device__ void advect_mom3() {
    FT u = U(), v = V(), w = W(), du = DU(S.na), dv = DV(S.na), dw = DW(S.na);
    FT fuz = SA(), fvz = SB(), fwz = SCR(p.L.s_c);
    T *rho = PR(P_RHO), *adz = PR(P_ADZ), *rhow = PR(P_RHOW);
    const T dx25 = (T)0.25 / (T)p.dx, dy25 = (T)0.25 / (T)p.dy;
    const T dz = (T)S.dz;
    const T dz25 = (T)1. / ((T)4. * dz);
    const int nxy = nx * ny;
    for (int e = TID; e < nxy * nzm; e += NT) {
      const int i = 1 + e % nx, j = 1 + (e / nx) % ny, k = 1 + e / nxy;
      const int kc = k + 1, kcu = min(kc, nzm), ic = i + 1, ib = i - 1, jb = j - 1, jc = j + 1;
      const T irho = PR(P_IRHOWADZW)[kc];
      T fu1 = dx25 * (u(ic - 1, j, k) + u(i - 1, j, k)) * (u(i - 1, j, k) + u(ic - 1, j, k));
      T fu2 = dx25 * (u(ic, j, k) + u(i, j, k)) * (u(i, j, k) + u(ic, j, k));
      T dun = du(i, j, k) - (fu2 - fu1);
      T fv1 = dx25 * (u(ic - 1, j, k) + u(ic - 1, jb, k)) * (v(i - 1, j, k) + v(ic - 1, j, k));
      T fv2 = dx25 * (u(ic, j, k) + u(ic, jb, k)) * (v(i, j, k) + v(ic, j, k));
      T dvn = dv(i, j, k) - (fv2 - fv1);
      T fw1 = dx25 * (u(ic - 1, j, k) * rho[k] * adz[k] + u(ic - 1, j, kcu) * rho[kcu] * adz[kcu]) *
              (w(i - 1, j, kc) + w(ic - 1, j, kc));
      T fw2 = dx25 * (u(ic, j, k) * rho[k] * adz[k] + u(ic, j, kcu) * rho[kcu] * adz[kcu]) * (w(i, j, kc) + w(ic, j, kc));
      T dwn = dw(i, j, kc) - irho * (fw2 - fw1);
      fu1 = dy25 * (v(i, jc - 1, k) + v(ib, jc - 1, k)) * (u(i, j - 1, k) + u(i, jc - 1, k));
      fu2 = dy25 * (v(i, jc, k) + v(ib, jc, k)) * (u(i, j, k) + u(i, jc, k));
      dun = dun - (fu2 - fu1);
      fv1 = dy25 * (v(i, jc - 1, k) + v(i, j - 1, k)) * (v(i, j - 1, k) + v(i, jc - 1, k));
      fv2 = dy25 * (v(i, jc, k) + v(i, j, k)) * (v(i, j, k) + v(i, jc, k));
      dvn = dvn - (fv2 - fv1);
      fw1 = dy25 * (v(i, jc - 1, k) * rho[k] * adz[k] + v(i, jc - 1, kcu) * rho[kcu] * adz[kcu]) *
            (w(i, j - 1, kc) + w(i, jc - 1, kc));
      fw2 = dy25 * (v(i, jc, k) * rho[k] * adz[k] + v(i, jc, kcu) * rho[kcu] * adz[kcu]) * (w(i, j, kc) + w(i, jc, kc));
      dwn = dwn - irho * (fw2 - fw1);
      T fzu = (T)0., fzv = (T)0.;
      if (k >= 2) {
        const int kb = k - 1;
        const T rhoi = dz25 * rhow[k];
        fzu = rhoi * (w(i, j, k) + w(i - 1, j, k)) * (u(i, j, k) + u(i, j, kb));
        fzv = rhoi * (w(i, j, k) + w(i, j - 1, k)) * (v(i, j, k) + v(i, j, kb));
      }
      du(i, j, k) = dun;
      dv(i, j, k) = dvn;
      dw(i, j, kc) = dwn;
      if (k >= 2) {
        fuz(i, j, k) = fzu;
        fvz(i, j, k) = fzv;
      } else {
        fuz(i, j, 1) = (T)0.; fvz(i, j, 1) = (T)0.;
        fuz(i, j, nz) = (T)0.; fvz(i, j, nz) = (T)0.;
      }
    }
    SYNC;
    T *uwle = PR(P_UWLE), *vwle = PR(P_VWLE);
    if (TID == 0) { uwle[1] = (T)0.; vwle[1] = (T)0.; uwle[nz] = (T)0.; vwle[nz] = (T)0.; }
    level_sums_lo(2, 2, nzm, [&](int q, int h, int k) -> T { return q == 0 ? fuz(h, k) : fvz(h, k); },
               [&](int, int) { return 0.; },
               [&](int q, int k, double sv) { (q == 0 ? uwle : vwle)[k] = (T)sv; });
    for (int e = TID; e < nxy * nzm; e += NT) {
      const int i = 1 + e % nx, j = 1 + (e / nx) % ny, k = 1 + e / nxy;
      const int kc = k + 1;
      const T rhoi = PR(P_IRHOADZ)[k];
      du(i, j, k) = du(i, j, k) - (fuz(i, j, kc) - fuz(i, j, k)) * rhoi;
      dv(i, j, k) = dv(i, j, k) - (fvz(i, j, kc) - fvz(i, j, k)) * rhoi;
      fwz(i, j, k) = dz25 * (w(i, j, kc) * rhow[kc] + w(i, j, k) * rhow[k]) * (w(i, j, kc) + w(i, j, k));
    }
    SYNC;
    for (int e = TID; e < nxy * (nzm - 1); e += NT) {
      const int i = 1 + e % nx, j = 1 + (e / nx) % ny, k = 2 + e / nxy;
      const T rhoi = PR(P_IRHOWADZW)[k];
      dw(i, j, k) = dw(i, j, k) - (fwz(i, j, k) - fwz(i, j, k - 1)) * rhoi;
    }
    SYNC;
  }

  // ---------------------------------------------------------- diffuse_mom3D
  // SGS_TKE/diffuse_mom3D.F90:40-204 (fluxbu, fluxbv, fluxtu, fluxtv are 0)
  __device__ void diffuse_mom3() {
    FT u = U(), v = V(), w = W(), tk = TK(), du = DU(S.na), dv = DV(S.na), dw = DW(S.na);
    FT fu = SA(), fv = SB(), fw = SCR(p.L.s_c);
    T *rho = PR(P_RHO), *adz = PR(P_ADZ), *rhow = PR(P_RHOW), *adzw = PR(P_ADZW);
    T *grdfx = PR(P_GRDFX), *grdfy = PR(P_GRDFY), *grdfz = PR(P_GRDFZ);
    const T dx = (T)p.dx, dy = (T)p.dy, dz = (T)S.dz;
    const T rdx2 = (T)1. / (dx * dx), rdy2 = (T)1. / (dy * dy);
    const T rdx25 = (T)0.25 * rdx2, rdy25 = (T)0.25 * rdy2;
    const T dxy = dx / dy, dyx = dy / dx;
    const int nxy = nx * ny;
    // x faces i = 0..nx
    for (int e = TID; e < (nx + 1) * ny * nzm; e += NT) {
      const int i = e % (nx + 1), j = 1 + (e / (nx + 1)) % ny, k = 1 + e / ((nx + 1) * ny);
      const int jb = j - 1, kc = k + 1, kcu = min(kc, nzm), ic = i + 1;
      const T dxz = dx / (dz * adzw[kc]);
      const T rdx21 = rdx2 * grdfx[k];
      const T rdx251 = rdx25 * grdfx[k];
      T tkx = rdx21 * tk(i, j, k);
      const T fuv = (T)-2. * tkx * (u(ic, j, k) - u(i, j, k));
      tkx = rdx251 * (tk(i, j, k) + tk(i, jb, k) + tk(ic, j, k) + tk(ic, jb, k));
      const T fvv = -tkx * (v(ic, j, k) - v(i, j, k) + (u(ic, j, k) - u(ic, jb, k)) * dxy);
      tkx = rdx251 * (tk(i, j, k) + tk(ic, j, k) + tk(i, j, kcu) + tk(ic, j, kcu));
      const T fwv = -tkx * (w(ic, j, kc) - w(i, j, kc) + (u(ic, j, kcu) - u(ic, j, k)) * dxz);
      fu(i, j, k) = fuv;
      fv(i, j, k) = fvv;
      fw(i, j, k) = fwv;
    }
    SYNC;
    for (int e = TID; e < nxy * nzm; e += NT) {
      const int i = 1 + e % nx, j = 1 + (e / nx) % ny, k = 1 + e / nxy;
      const int kc = k + 1, ib = i - 1;
      du(i, j, k) = du(i, j, k) - (fu(i, j, k) - fu(ib, j, k));
      dv(i, j, k) = dv(i, j, k) - (fv(i, j, k) - fv(ib, j, k));
      dw(i, j, kc) = dw(i, j, kc) - (fw(i, j, k) - fw(ib, j, k));
    }
    SYNC;
    // y faces j = 0..ny
    for (int e = TID; e < nx * (ny + 1) * nzm; e += NT) {
      const int i = 1 + e % nx, j = (e / nx) % (ny + 1), k = 1 + e / (nx * (ny + 1));
      const int jc = j + 1, kc = k + 1, kcu = min(kc, nzm), ib = i - 1;
      const T dyz = dy / (dz * adzw[kc]);
      const T rdy21 = rdy2 * grdfy[k];
      const T rdy251 = rdy25 * grdfy[k];
      T tky = rdy21 * tk(i, j, k);
      const T fvv = (T)-2. * tky * (v(i, jc, k) - v(i, j, k));
      tky = rdy251 * (tk(i, j, k) + tk(ib, j, k) + tk(i, jc, k) + tk(ib, jc, k));
      const T fuv = -tky * (u(i, jc, k) - u(i, j, k) + (v(i, jc, k) - v(ib, jc, k)) * dyx);
      tky = rdy251 * (tk(i, j, k) + tk(i, jc, k) + tk(i, j, kcu) + tk(i, jc, kcu));
      const T fwv = -tky * (w(i, jc, kc) - w(i, j, kc) + (v(i, jc, kcu) - v(i, jc, k)) * dyz);
      fv(i, j, k) = fvv;
      fu(i, j, k) = fuv;
      fw(i, j, k) = fwv;
    }
    SYNC;
    for (int e = TID; e < nxy * nzm; e += NT) {
      const int i = 1 + e % nx, j = 1 + (e / nx) % ny, k = 1 + e / nxy;
      const int kc = k + 1, jb = j - 1;
      du(i, j, k) = du(i, j, k) - (fu(i, j, k) - fu(i, jb, k));
      dv(i, j, k) = dv(i, j, k) - (fv(i, j, k) - fv(i, jb, k));
      dw(i, j, kc) = dw(i, j, kc) - (fw(i, j, k) - fw(i, jb, k));
    }
    SYNC;
    // vertical fluxes at w levels (reuse fu, fv, fw)
    for (int e = TID; e < nxy * nzm; e += NT) {
      const int i = 1 + e % nx, j = 1 + (e / nx) % ny, k = 1 + e / nxy;
      const T rdz = (T)1. / dz;
      if (k <= nzm - 1) {
        const int jb = j - 1, kc = k + 1, ib = i - 1;
        const T rdz2 = rdz * rdz * grdfz[k];
        const T rdz25 = (T)0.25 * rdz2;
        const T iadz = (T)1. / adz[k];
        const T iadzw = (T)1. / adzw[kc];
        const T dzx = dz / dx, dzy = dz / dy;
        T tkz = rdz2 * tk(i, j, k);
        const T fwv = (T)-2. * tkz * (w(i, j, kc) - w(i, j, k)) * rho[k] * iadz;
        tkz = rdz25 * (tk(i, j, k) + tk(ib, j, k) + tk(i, j, kc) + tk(ib, j, kc));
        const T fuv = -tkz * ((u(i, j, kc) - u(i, j, k)) * iadzw + (w(i, j, kc) - w(ib, j, kc)) * dzx) * rhow[kc];
        tkz = rdz25 * (tk(i, j, k) + tk(i, jb, k) + tk(i, j, kc) + tk(i, jb, kc));
        const T fvv = -tkz * ((v(i, j, kc) - v(i, j, k)) * iadzw + (w(i, j, kc) - w(i, jb, kc)) * dzy) * rhow[kc];
        fw(i, j, kc) = fwv;
        fu(i, j, kc) = fuv;
        fv(i, j, kc) = fvv;
      } else {
        const T rdz2 = rdz * rdz * grdfz[nzm - 1];
        const T tkz = rdz2 * grdfz[nzm] * tk(i, j, nzm);
        fw(i, j, nz) = (T)-2. * tkz * (w(i, j, nz) - w(i, j, nzm)) / adz[nzm] * rho[nzm];
        fu(i, j, 1) = (T)0.0 * rdz * rhow[1];
        fv(i, j, 1) = (T)0.0 * rdz * rhow[1];
        fu(i, j, nz) = (T)0.0 * rdz * rhow[nz];
        fv(i, j, nz) = (T)0.0 * rdz * rhow[nz];
      }
    }
    SYNC;
    T *uwsb = PR(P_UWSB), *vwsb = PR(P_VWSB);
    level_sums_lo(2, 1, nzm, [&](int q, int h, int k) -> T { return q == 0 ? fu(h, k) : fv(h, k); },
               [&](int, int) { return 0.; },
               [&](int q, int k, double sv) { (q == 0 ? uwsb : vwsb)[k] = (T)sv; });
    for (int e = TID; e < nxy * nzm; e += NT) {
      const int i = 1 + e % nx, j = 1 + (e / nx) % ny, k = 1 + e / nxy;
      const int kc = k + 1;
      const T rhoi = (T)1. / (rho[k] * adz[k]);
      du(i, j, k) = du(i, j, k) - (fu(i, j, kc) - fu(i, j, k)) * rhoi;
      dv(i, j, k) = dv(i, j, k) - (fv(i, j, kc) - fv(i, j, k)) * rhoi;
      if (k >= 2) {
        const T rhoiw = (T)1. / (rhow[k] * adzw[k]);
        dw(i, j, k) = dw(i, j, k) - (fw(i, j, k + 1) - fw(i, j, k)) * rhoiw;
      }
    }
    SYNC;
  }

  // ---------------------------------------------------------- advect_mom
  // advect2_mom_xy.F90:60-80 (2D) and advect2_mom_z.F90:30-122
  __device__ void advect_mom() {
    FT u = U(), v = V(), w = W(), du = DU(S.na), dv = DV(S.na), dw = DW(S.na);
    FT fuz = SA(), fvz = SB(), fwz = SCR(p.L.s_c);
    T *rho = PR(P_RHO), *adz = PR(P_ADZ), *rhow = PR(P_RHOW), *adzw = PR(P_ADZW);
    const T dx25 = (T)0.25 / (T)p.dx;
    const T dz = (T)S.dz;
    const T dz25 = (T)1. / ((T)4. * dz);
    for (int e = TID; e < nx * nzm; e += NT) {
      int i = 1 + e % nx, k = 1 + e / nx;
      int kc = k + 1, kcu = min(kc, nzm);
      T irho = PR(P_IRHOWADZW)[kc];
      int ic = i + 1;
      // all loads first (the stores below may alias them for the compiler);
      // u(ic - 1, .) is u(i, .)
      const T um = u(i - 1, k), ui = u(i, k), uc = u(ic, k), uiu = u(i, kcu), ucu = u(ic, kcu);
      const T vm = v(i - 1, k), vi = v(i, k), vc = v(ic, k);
      const T wmc = w(i - 1, kc), wic = w(i, kc), wcc = w(ic, kc);
      T fu1 = dx25 * (ui + um) * (um + ui);
      T fu2 = dx25 * (uc + ui) * (ui + uc);
      T fv1 = dx25 * (ui + um) * (vm + vi);
      T fv2 = dx25 * (uc + ui) * (vi + vc);
      T fw1 = dx25 * (ui * rho[k] * adz[k] + uiu * rho[kcu] * adz[kcu]) * (wmc + wic);
      T fw2 = dx25 * (uc * rho[k] * adz[k] + ucu * rho[kcu] * adz[kcu]) * (wic + wcc);
      T fzu = (T)0., fzv = (T)0.;
      if (k >= 2) {
        int kb = k - 1;
        T rhoi = dz25 * rhow[k];
        T www = rhoi * (w(i, k) + w(i - 1, k));
        fzu = www * (ui + u(i, kb));
        fzv = www * (vi + v(i, kb));
      }
      const T dun = du(i, k) - (fu2 - fu1);
      const T dvn = dv(i, k) - (fv2 - fv1);
      const T dwn = dw(i, kc) - irho * (fw2 - fw1);
      du(i, k) = dun;
      dv(i, k) = dvn;
      dw(i, kc) = dwn;
      // vertical fluxes of u, v at w level k (k = 2..nzm); 0 at 1 and nz
      if (k >= 2) {
        fuz(i, k) = fzu;
        fvz(i, k) = fzv;
      } else {
        fuz(i, 1) = (T)0.; fvz(i, 1) = (T)0.;
        fuz(i, nz) = (T)0.; fvz(i, nz) = (T)0.;
      }
    }
    SYNC;
    T *uwle = PR(P_UWLE), *vwle = PR(P_VWLE);
    if (TID == 0) { uwle[1] = (T)0.; vwle[1] = (T)0.; uwle[nz] = (T)0.; vwle[nz] = (T)0.; }
    level_sums_lo(2, 2, nzm, [&](int q, int i, int k) -> T { return q == 0 ? fuz(i, k) : fvz(i, k); },
               [&](int, int) { return 0.; },
               [&](int q, int k, double sv) { (q == 0 ? uwle : vwle)[k] = (T)sv; });
    for (int e = TID; e < nx * nzm; e += NT) {
      int i = 1 + e % nx, k = 1 + e / nx;
      int kc = k + 1;
      T rhoi = PR(P_IRHOADZ)[k];
      du(i, k) = du(i, k) - (fuz(i, kc) - fuz(i, k)) * rhoi;
      dv(i, k) = dv(i, k) - (fvz(i, kc) - fvz(i, k)) * rhoi;
      fwz(i, k) = dz25 * (w(i, kc) * rhow[kc] + w(i, k) * rhow[k]) * (w(i, kc) + w(i, k));
    }
    SYNC;
    for (int e = TID; e < nx * (nzm - 1); e += NT) {
      int i = 1 + e % nx, k = 2 + e / nx;
      int kb = k - 1;
      T rhoi = PR(P_IRHOWADZW)[k];
      dw(i, k) = dw(i, k) - (fwz(i, k) - fwz(i, kb)) * rhoi;
    }
    SYNC;
  }

  // ---------------------------------------------------------- diffuse_mom2D
  // SGS_TKE/diffuse_mom2D.F90:42-160
  __device__ void diffuse_mom() {
    FT u = U(), v = V(), w = W(), tk = TK(), du = DU(S.na), dv = DV(S.na), dw = DW(S.na);
    FT fu = SA(), fv = SB(), fw = SCR(p.L.s_c);
    T *rho = PR(P_RHO), *adz = PR(P_ADZ), *rhow = PR(P_RHOW), *adzw = PR(P_ADZW);
    T *grdfx = PR(P_GRDFX), *grdfz = PR(P_GRDFZ);
    const T dx = (T)p.dx, dz = (T)S.dz;
    const T rdx2 = (T)1. / dx / dx;
    const T rdx25 = (T)0.25 * rdx2;
    for (int e = TID; e < (nx + 1) * nzm; e += NT) {
      int i = e % (nx + 1), k = 1 + e / (nx + 1);
      int kc = k + 1, kcu = min(kc, nzm);
      T dxz = dx / (dz * adzw[kc]);
      T rdx21 = rdx2 * grdfx[k];
      T rdx251 = rdx25 * grdfx[k];
      int ic = i + 1;
      const T tki = tk(i, k), tkc = tk(ic, k), tkiu = tk(i, kcu), tkcu = tk(ic, kcu);
      const T uc = u(ic, k), ui = u(i, k), ucu = u(ic, kcu), vc = v(ic, k), vi = v(i, k);
      const T wcc = w(ic, kc), wic = w(i, kc);
      T tkx = rdx21 * tki;
      const T fuv = (T)-2. * tkx * (uc - ui);
      const T fvv = -tkx * (vc - vi);
      tkx = rdx251 * (tki + tkc + tkiu + tkcu);
      const T fwv = -tkx * (wcc - wic + (ucu - uc) * dxz);
      fu(i, k) = fuv;
      fv(i, k) = fvv;
      fw(i, k) = fwv;
    }
    SYNC;
    for (int e = TID; e < nx * nzm; e += NT) {
      int i = 1 + e % nx, k = 1 + e / nx;
      int kc = k + 1, ib = i - 1;
      du(i, k) = du(i, k) - (fu(i, k) - fu(ib, k));
      dv(i, k) = dv(i, k) - (fv(i, k) - fv(ib, k));
      dw(i, kc) = dw(i, kc) - (fw(i, k) - fw(ib, k));
    }
    SYNC;
    // vertical fluxes (reuse fu, fv, fw)
    for (int e = TID; e < nx * nzm; e += NT) {
      int i = 1 + e % nx, k = 1 + e / nx;
      if (k <= nzm - 1) {
        int kc = k + 1;
        T rdz = (T)1. / dz;
        T rdz2 = rdz * rdz * grdfz[k];
        T rdz25 = (T)0.25 * rdz2;
        T dzx = dz / dx;
        T iadz = PR(P_IADZ)[k];
        T iadzw = PR(P_IADZW)[kc];
        int ib = i - 1;
        const T tki = tk(i, k), tkb = tk(ib, k), tkic = tk(i, kc), tkbc = tk(ib, kc);
        const T wic = w(i, kc), wi = w(i, k), wbc = w(ib, kc);
        const T uic = u(i, kc), ui = u(i, k), vic = v(i, kc), vi = v(i, k), rk = rho[k], rwc = rhow[kc];
        T tkz = rdz2 * tki;
        const T fwv = (T)-2. * tkz * (wic - wi) * rk * iadz;
        tkz = rdz25 * (tki + tkb + tkic + tkbc);
        const T fuv = -tkz * ((uic - ui) * iadzw + (wic - wbc) * dzx) * rwc;
        const T fvv = -tkz * (vic - vi) * iadzw * rwc;
        fw(i, kc) = fwv;
        fu(i, kc) = fuv;
        fv(i, kc) = fvv;
      } else {
        T rdz = (T)1. / dz;
        T rdz2 = rdz * rdz * grdfz[nzm - 1];
        T tkz = rdz2 * grdfz[nzm] * tk(i, nzm);
        fw(i, nz) = (T)-2. * tkz * (w(i, nz) - w(i, nzm)) / adz[nzm] * rho[nzm];
        fu(i, 1) = (T)0.0 * rdz * rhow[1];
        fv(i, 1) = (T)0.0 * rdz * rhow[1];
        fu(i, nz) = (T)0.0 * rdz * rhow[nz];
        fv(i, nz) = (T)0.0 * rdz * rhow[nz];
      }
    }
    SYNC;
    T *uwsb = PR(P_UWSB), *vwsb = PR(P_VWSB);
    level_sums_lo(2, 1, nzm, [&](int q, int i, int k) -> T { return q == 0 ? fu(i, k) : fv(i, k); },
               [&](int, int) { return 0.; },
               [&](int q, int k, double sv) { (q == 0 ? uwsb : vwsb)[k] = (T)sv; });
    for (int e = TID; e < nx * nzm; e += NT) {
      int i = 1 + e % nx, k = 1 + e / nx;
      int kc = k + 1;
      T rhoi = PR(P_IRHOADZ)[k];
      const T fuc = fu(i, kc), fuk = fu(i, k), fvc = fv(i, kc), fvk = fv(i, k);
      const T fwc = k >= 2 ? fw(i, k + 1) : (T)0., fwk = k >= 2 ? fw(i, k) : (T)0.;
      const T dun = du(i, k) - (fuc - fuk) * rhoi;
      const T dvn = dv(i, k) - (fvc - fvk) * rhoi;
      du(i, k) = dun;
      dv(i, k) = dvn;
      if (k >= 2) {
        T rhoiw = PR(P_IRHOWADZW)[k];
        dw(i, k) = dw(i, k) - (fwc - fwk) * rhoiw;
      }
    }
    SYNC;
  }

  // ---------------------------------------------------------- FFT
  // Real/half-complex transform of crm/fft.F90 (fft991_crm :5-154 with
  // fft99a/b :301-465 and vpassm_crm :466-806, radix 2 and 4, lot = 1) for
  // one row held in shared memory, computed by one warp: within each pass
  // every butterfly is independent, so lanes take butterflies and the warp
  // synchronises between passes.  Each output keeps the reference's
  // expression, so results are identical to a sequential evaluation.
  // Twiddle factors are REAL*4 values (fft.F90 has no implicit none).
  // twiddle i of the trig table: the REAL*4 value, read as T without a
  // widening or narrowing conversion in either form
  __device__ __forceinline__ T tw(int i) const {
    if constexpr (Y3) {
      if (fdir) {
        if constexpr (sizeof(T) == 4) return p.trigs_y_f[i];
        else return p.trigs_y[i];
      }
    }
    if constexpr (sizeof(T) == 4) return p.trigs_f[i];
    else return p.trigs[i];
  }
  // transform factors of the current direction (3D: fdir 1 is y)
  __device__ __forceinline__ int nfax_() const {
    if constexpr (Y3) return fdir ? p.nfax_y : p.nfax;
    else return p.nfax;
  }
  __device__ __forceinline__ int ifax_(int k) const {
    if constexpr (Y3) return fdir ? p.ifax_y[k] : p.ifax[k];
    else return p.ifax[k];
  }
  __device__ void vpass_warp(const T *A, T *C, int nh, int ifac, int la, int lane) const {
    const int m = nh / ifac;
    for (int bf = lane; bf < m; bf += 32) {
      int g = bf / la, l = bf - g * la;
      int pp = g * la + l, q = g * ifac * la + l;
      int kb = 2 * g * la;
      T a0 = A[2 * pp], b0 = A[2 * pp + 1], a1 = A[2 * (pp + m)], b1 = A[2 * (pp + m) + 1];
      if (ifac == 2) {
        C[2 * q] = a0 + a1; C[2 * q + 1] = b0 + b1;
        if (g == 0) { C[2 * (q + la)] = a0 - a1; C[2 * (q + la) + 1] = b0 - b1; }
        else {
          T c1 = tw(kb), s1 = tw(kb + 1);
          C[2 * (q + la)] = c1 * (a0 - a1) - s1 * (b0 - b1);
          C[2 * (q + la) + 1] = s1 * (a0 - a1) + c1 * (b0 - b1);
        }
      } else if (ifac == 3) {
        // fft.F90 vpassm_crm, radix 3 (REAL*4 sin60)
        const T sin60 = (T)(double)(float)0.866025403784437;
        T a2 = A[2 * (pp + 2 * m)], b2 = A[2 * (pp + 2 * m) + 1];
        T *C0 = C + 2 * q, *C1 = C + 2 * (q + la), *C2 = C + 2 * (q + 2 * la);
        C0[0] = a0 + (a1 + a2);
        C0[1] = b0 + (b1 + b2);
        T xr = a0 - (T)0.5 * (a1 + a2), xi = b0 - (T)0.5 * (b1 + b2);
        T yr = sin60 * (b1 - b2), yi = sin60 * (a1 - a2);
        if (g == 0) {
          C1[0] = xr - yr; C2[0] = xr + yr; C1[1] = xi + yi; C2[1] = xi - yi;
        } else {
          T c1 = tw(kb), s1 = tw(kb + 1), c2 = tw(2 * kb), s2 = tw(2 * kb + 1);
          C1[0] = c1 * (xr - yr) - s1 * (xi + yi);
          C1[1] = s1 * (xr - yr) + c1 * (xi + yi);
          C2[0] = c2 * (xr + yr) - s2 * (xi - yi);
          C2[1] = s2 * (xr + yr) + c2 * (xi - yi);
        }
      } else if (ifac == 5) {
        // fft.F90 vpassm_crm, radix 5 (REAL*4 sin36, cos36, sin72, cos72)
        const T sin36 = (T)(double)(float)0.587785252292473, cos36 = (T)(double)(float)0.809016994374947;
        const T sin72 = (T)(double)(float)0.951056516295154, cos72 = (T)(double)(float)0.309016994374947;
        T a2 = A[2 * (pp + 2 * m)], b2 = A[2 * (pp + 2 * m) + 1];
        T a3 = A[2 * (pp + 3 * m)], b3 = A[2 * (pp + 3 * m) + 1];
        T a4 = A[2 * (pp + 4 * m)], b4 = A[2 * (pp + 4 * m) + 1];
        T *C0 = C + 2 * q, *C1 = C + 2 * (q + la), *C2 = C + 2 * (q + 2 * la), *C3 = C + 2 * (q + 3 * la),
          *C4 = C + 2 * (q + 4 * la);
        C0[0] = (a0 + (a1 + a4)) + (a2 + a3);
        C0[1] = (b0 + (b1 + b4)) + (b2 + b3);
        T p1r = (a0 + cos72 * (a1 + a4)) - cos36 * (a2 + a3);
        T q1r = sin72 * (b1 - b4) + sin36 * (b2 - b3);
        T p1i = (b0 + cos72 * (b1 + b4)) - cos36 * (b2 + b3);
        T q1i = sin72 * (a1 - a4) + sin36 * (a2 - a3);
        T p2r = (a0 - cos36 * (a1 + a4)) + cos72 * (a2 + a3);
        T q2r = sin36 * (b1 - b4) - sin72 * (b2 - b3);
        T p2i = (b0 - cos36 * (b1 + b4)) + cos72 * (b2 + b3);
        T q2i = sin36 * (a1 - a4) - sin72 * (a2 - a3);
        if (g == 0) {
          C1[0] = p1r - q1r; C4[0] = p1r + q1r; C1[1] = p1i + q1i; C4[1] = p1i - q1i;
          C2[0] = p2r - q2r; C3[0] = p2r + q2r; C2[1] = p2i + q2i; C3[1] = p2i - q2i;
        } else {
          T c1 = tw(kb), s1 = tw(kb + 1), c2 = tw(2 * kb), s2 = tw(2 * kb + 1);
          T c3 = tw(3 * kb), s3 = tw(3 * kb + 1), c4 = tw(4 * kb), s4 = tw(4 * kb + 1);
          C1[0] = c1 * (p1r - q1r) - s1 * (p1i + q1i);
          C1[1] = s1 * (p1r - q1r) + c1 * (p1i + q1i);
          C4[0] = c4 * (p1r + q1r) - s4 * (p1i - q1i);
          C4[1] = s4 * (p1r + q1r) + c4 * (p1i - q1i);
          C2[0] = c2 * (p2r - q2r) - s2 * (p2i + q2i);
          C2[1] = s2 * (p2r - q2r) + c2 * (p2i + q2i);
          C3[0] = c3 * (p2r + q2r) - s3 * (p2i - q2i);
          C3[1] = s3 * (p2r + q2r) + c3 * (p2i - q2i);
        }
      } else {  // 4
        T a2 = A[2 * (pp + 2 * m)], b2 = A[2 * (pp + 2 * m) + 1];
        T a3 = A[2 * (pp + 3 * m)], b3 = A[2 * (pp + 3 * m) + 1];
        T *C0 = C + 2 * q, *C1 = C + 2 * (q + la), *C2 = C + 2 * (q + 2 * la), *C3 = C + 2 * (q + 3 * la);
        if (g == 0) {
          C0[0] = (a0 + a2) + (a1 + a3); C2[0] = (a0 + a2) - (a1 + a3);
          C0[1] = (b0 + b2) + (b1 + b3); C2[1] = (b0 + b2) - (b1 + b3);
          C1[0] = (a0 - a2) - (b1 - b3); C3[0] = (a0 - a2) + (b1 - b3);
          C1[1] = (b0 - b2) + (a1 - a3); C3[1] = (b0 - b2) - (a1 - a3);
        } else {
          T c1 = tw(kb), s1 = tw(kb + 1);
          T c2 = tw(2 * kb), s2 = tw(2 * kb + 1);
          T c3 = tw(3 * kb), s3 = tw(3 * kb + 1);
          C0[0] = (a0 + a2) + (a1 + a3); C0[1] = (b0 + b2) + (b1 + b3);
          C2[0] = c2 * ((a0 + a2) - (a1 + a3)) - s2 * ((b0 + b2) - (b1 + b3));
          C2[1] = s2 * ((a0 + a2) - (a1 + a3)) + c2 * ((b0 + b2) - (b1 + b3));
          C1[0] = c1 * ((a0 - a2) - (b1 - b3)) - s1 * ((b0 - b2) + (a1 - a3));
          C1[1] = s1 * ((a0 - a2) - (b1 - b3)) + c1 * ((b0 - b2) + (a1 - a3));
          C3[0] = c3 * ((a0 - a2) + (b1 - b3)) - s3 * ((b0 - b2) - (a1 - a3));
          C3[1] = s3 * ((a0 - a2) + (b1 - b3)) + c3 * ((b0 - b2) - (a1 - a3));
        }
      }
    }
    __syncwarp();
  }
  // fft991_crm on a[0..n+1] (shared memory), work[0..n+1]; isign -1: grid
  // point -> spectral, +1: spectral -> grid point.  Called by a whole warp.
  __device__ void fft991_warp(T *a, T *work, int n, int isign, int lane) const {
    const int nfax = nfax_(), nh = n / 2, npair = (nh - 1) / 2;   // k = 3,5,..,nh
    bool in_work;
    if (isign == -1) {
      if (nfax % 2 == 1) in_work = false;
      else {
        for (int m = lane; m < n; m += 32) work[m] = a[m];
        in_work = true;
      }
    } else {
      // fft99a_crm: a -> work
      if (lane == 0) {
        work[0] = a[0] + a[n];
        work[1] = a[0] - a[n];
      }
      for (int t = lane; t < npair; t += 32) {
        int k = 3 + 2 * t, ia = 2 + 2 * t, ib = n - 2 - 2 * t;
        T c = tw(n + k - 1), s = tw(n + k);
        T ap = a[ia] + a[ib], am = a[ia] - a[ib];
        T bp = a[ia + 1] + a[ib + 1], bm = a[ia + 1] - a[ib + 1];
        work[ia] = ap - (s * am + c * bp);
        work[ib] = ap + (s * am + c * bp);
        work[ia + 1] = (c * am - s * bp) + bm;
        work[ib + 1] = (c * am - s * bp) - bm;
      }
      {
        int ia = 2 + 2 * npair, ib = n - 2 - 2 * npair;
        if (ia == ib && lane == 0) { work[ia] = (T)2.0 * a[ia]; work[ia + 1] = (T)-2.0 * a[ia + 1]; }
      }
      in_work = true;
    }
    __syncwarp();
    int la = 1;
    for (int k = 1; k <= nfax; ++k) {
      if (in_work) vpass_warp(work, a, nh, ifax_(k), la, lane);
      else vpass_warp(a, work, nh, ifax_(k), la, lane);
      in_work = !in_work;
      la *= ifax_(k);
    }
    if (isign == -1) {
      // fft99b_crm: work -> a
      float scale = (float)(1.0 / (double)n);
      const T sc0 = (T)(double)scale;
      const T sc = (T)(double)(0.5f * scale);
      const T sc2 = (T)(double)(2.0f * (0.5f * scale));
      if (lane == 0) {
        T w0 = work[0], w1 = work[1];
        a[0] = sc0 * (w0 + w1);
        a[n] = sc0 * (w0 - w1);
        a[1] = (T)0.0;
        a[n + 1] = (T)0.0;
      }
      for (int t = lane; t < npair; t += 32) {
        int k = 3 + 2 * t, ia = 2 + 2 * t, ib = n - 2 - 2 * t;
        T c = tw(n + k - 1), s = tw(n + k);
        T wp = work[ia] + work[ib], wm = work[ia] - work[ib];
        T vp = work[ia + 1] + work[ib + 1], vm = work[ib + 1] - work[ia + 1];
        a[ia] = sc * (wp + (c * vp + s * wm));
        a[ib] = sc * (wp - (c * vp + s * wm));
        a[ia + 1] = sc * ((c * wm - s * vp) + vm);
        a[ib + 1] = sc * ((c * wm - s * vp) - vm);
      }
      {
        int ia = 2 + 2 * npair, ib = n - 2 - 2 * npair;
        if (ia == ib && lane == 0) {
          a[ia] = sc2 * work[ia];
          a[ia + 1] = -sc2 * work[ia + 1];
        }
      }
    } else {
      if (in_work)
        for (int m = lane; m < n; m += 32) a[m] = work[m];
      if (lane == 0) { a[n] = (T)0.0; a[n + 1] = (T)0.0; }
    }
    __syncwarp();
  }

  // ---------------------------------------------------------- pressure
  // Tridiagonal factors of the vertical Poisson operator per Fourier
  // coefficient (pressure.F90:200-236).  They depend only on the column's
  // grid and the eigenvalues, so they are formed once per call: alfa(k) and
  // the reciprocal pivots e(k) exactly as the reference computes them every
  // substep, the last pivot kept as a divisor.
  __device__ double *TRI() const { return reinterpret_cast<double *>(base + p.L.tri); }
  __device__ void tridiag_factor() {
    // coefficients c = (i - 1) + (nx + 1) (j - 1): i = 1..nx+1, j = 1..ny+2 in
    // 3D, j = 1 in 2D
    const int np = (nx + 1) * (Y3 ? ny + 2 : 1), ls = nzm + 1;
    // [a(k)], then alfa(k, i) and e(k, i) with the Fourier index i fastest
    // (the solve runs one coefficient per thread, so its loads coalesce), then
    // the np last pivots
    double *tri = TRI();
    double *ak = tri;
    T *rho = PR(P_RHO), *rhow = PR(P_RHOW), *adz = PR(P_ADZ), *adzw = PR(P_ADZW);
    const double dz = S.dz;
    for (int k = TID + 1; k <= nzm; k += NT)
      ak[k] = (double)rhow[k] / ((double)adz[k] * (double)adzw[k] * dz * dz);
    SYNC;
    for (int i = TID + 1; i <= np; i += NT) {
      double *alb = tri + (size_t)ls + (i - 1), *eb = alb + (size_t)ls * np;
      auto al = [&](int k) -> double & { return alb[(size_t)k * np]; };
      auto e = [&](int k) -> double & { return eb[(size_t)k * np]; };
      const int ic = (i - 1) % (nx + 1) + 1, jc = (i - 1) / (nx + 1) + 1;
      int id = (int)(((float)ic - 0.1f) / 2.0f);
      int jd = (int)(((float)jc - 0.1f) / 2.0f);
      double eign = p.eign[i - 1];
      double a1 = ak[1];
      double c1 = (double)rhow[2] / ((double)adz[1] * (double)adzw[2] * dz * dz);
      double b;
      if (id + jd == 0) b = 1. / (eign * (double)rho[1] - a1 - c1);
      else b = 1. / (eign * (double)rho[1] - c1);
      al(1) = -c1 * b;
      e(1) = b;
      double alprev = -c1 * b;
      for (int k = 2; k <= nzm - 1; ++k) {
        double a = ak[k];
        double c = (double)rhow[k + 1] / ((double)adz[k] * (double)adzw[k + 1] * dz * dz);
        double ee = 1. / (eign * (double)rho[k] - a - c + a * alprev);
        alprev = -c * ee;
        al(k) = alprev;
        e(k) = ee;
      }
      double an = ak[nzm];
      tri[(size_t)ls + (size_t)np * 2 * ls + (i - 1)] = eign * (double)rho[nzm] - an + an * alprev;
    }
    SYNC;
  }

  // pressure.F90:97-310, press_rhs.F90:48-101, press_grad.F90:18-72 and
  // bound_duvdt.F90 in 3D: the coefficients live in the slab (fft_f,
  // (nx+2) x (ny+2) x nzm); each warp transforms rows in x (every j) and
  // then columns in y (every x coefficient i = 1..nx+1) through its own
  // shared-memory row and work buffers; one FP64 tridiagonal solve per
  // (i, j) coefficient; the inverse transforms in the reverse order
  __device__ void pressure3(T *wsh, float *tcsm) {
    FT u = U(), v = V(), w = W(), pp = PP();
    FT dua = DU(S.na), dub = DU(S.nb), duc = DU(S.nc);
    FT dva = DV(S.na), dvb = DV(S.nb), dvc = DV(S.nc);
    FT dwa = DW(S.na), dwb = DW(S.nb), dwc = DW(S.nc);
    T *rho = PR(P_RHO);
    const int nxy = nx * ny, nx2 = nx + 2, ny2 = ny + 2, np = (nx + 1) * ny2;
    T *F = base + p.L.fft_f;
    auto FF = [&](int i, int j, int k) -> T & { return F[((size_t)(k - 1) * ny2 + (j - 1)) * nx2 + (i - 1)]; };
    auto bound_duvdt = [&]() {
      for (int e = TID; e < ny * nzm; e += NT) {
        const int j = 1 + e % ny, k = 1 + e / ny;
        dua(nx + 1, j, k) = dua(1, j, k);
      }
      for (int e = TID; e < nx * nzm; e += NT) {
        const int i = 1 + e % nx, k = 1 + e / nx;
        dva(i, ny + 1, k) = dva(i, 1, k);
      }
    };
    bound_duvdt();
    SYNC;
    const T rdx = (T)1. / (T)p.dx, rdy = (T)1. / (T)p.dy;
    const T btat = (T)(S.bt / S.at), ctat = (T)(S.ct / S.at);
    const T dta = (T)(1. / S.dt3[S.na - 1] / S.at);
    for (int e = TID; e < nxy * nzm; e += NT) {
      const int i = 1 + e % nx, j = 1 + (e / nx) % ny, k = 1 + e / nxy;
      const int kc = k + 1, jc = j + 1, ic = i + 1;
      const T rup = PR(P_RUP)[k], rdn = PR(P_RDN)[k];
      const T r = (rdx * (u(ic, j, k) - u(i, j, k)) + rdy * (v(i, jc, k) - v(i, j, k)) +
                   (w(i, j, kc) * rup - w(i, j, k) * rdn)) * dta +
                  (rdx * (dua(ic, j, k) - dua(i, j, k)) + rdy * (dva(i, jc, k) - dva(i, j, k)) +
                   (dwa(i, j, kc) * rup - dwa(i, j, k) * rdn)) +
                  btat * (rdx * (dub(ic, j, k) - dub(i, j, k)) + rdy * (dvb(i, jc, k) - dvb(i, j, k)) +
                          (dwb(i, j, kc) * rup - dwb(i, j, k) * rdn)) +
                  ctat * (rdx * (duc(ic, j, k) - duc(i, j, k)) + rdy * (dvc(i, jc, k) - dvc(i, j, k)) +
                          (dwc(i, j, kc) * rup - dwc(i, j, k) * rdn));
      FF(i, j, k) = r * rho[k];
    }
    SYNC;
    PHASE_MARK(PH_PRESS_RHS);
    const int warp = TID >> 5, lane = TID & 31, nwarps = NT >> 5;
    const int nmax = nx > ny ? nx : ny;
    T *ra = wsh + (size_t)warp * (2 * nmax + 8), *wk = ra + nmax + 2;
    auto xrows = [&](int isign) {
      fdir = 0;
      for (int r = warp; r < ny * nzm; r += nwarps) {
        const int j = 1 + r % ny, k = 1 + r / ny;
        T *row = &FF(1, j, k);
        for (int m = lane; m < nx2; m += 32) ra[m] = row[m];
        __syncwarp();
        fft991_warp(ra, wk, nx, isign, lane);
        for (int m = lane; m < nx2; m += 32) row[m] = ra[m];
        __syncwarp();
      }
    };
    auto ycols = [&](int isign) {
      fdir = 1;
      for (int r = warp; r < (nx + 1) * nzm; r += nwarps) {
        const int i = 1 + r % (nx + 1), k = 1 + r / (nx + 1);
        for (int m = lane; m < ny2; m += 32) ra[m] = FF(i, 1 + m, k);
        __syncwarp();
        fft991_warp(ra, wk, ny, isign, lane);
        for (int m = lane; m < ny2; m += 32) FF(i, 1 + m, k) = ra[m];
        __syncwarp();
      }
      fdir = 0;
    };
    if constexpr (TC != 0) {
      if constexpr (sizeof(T) == 4) {
        tc::Engine E(p.tc_n, tcsm, S.tc_tmem, tc::smem_u32(&S.tc_mbar), &S.tc_phase, &S.tc_fail, TID, NT);
        for (int k0 = 1; k0 <= nzm; k0 += E.d.L) E.forward_tile(FF, k0, nzm);
      }
    } else {
      xrows(-1);
      SYNC;
      ycols(-1);
      SYNC;
    }
    PHASE_MARK(PH_FFT_FWD);
    // vertical tridiagonal solve per coefficient c = (i-1) + (nx+1)(j-1), in FP64
    {
      const int ls = nzm + 1;
      const size_t lstride = (size_t)nx2 * ny2;
      const double *tri = TRI();
      double *beta = reinterpret_cast<double *>(sa());   // (nzm+1) x np doubles, c fastest (planes A and B)
      for (int c = TID; c < np; c += NT) {
        const int i = 1 + c % (nx + 1), j = 1 + c / (nx + 1);
        const double *al = tri + (size_t)ls + c, *e = al + (size_t)ls * np;
        double *be = beta + c;
        T *ff = F + (size_t)(j - 1) * nx2 + (i - 1);
        double bprev = (double)ff[0] * e[np];
        be[np] = bprev;
        for (int k = 2; k <= nzm - 1; ++k) {
          bprev = ((double)ff[lstride * (k - 1)] - tri[k] * bprev) * e[(size_t)k * np];
          be[(size_t)k * np] = bprev;
        }
        double fk = ((double)ff[lstride * (nzm - 1)] - tri[nzm] * bprev) / tri[(size_t)ls + (size_t)np * 2 * ls + c];
        ff[lstride * (nzm - 1)] = (T)fk;
        for (int k = nzm - 1; k >= 1; --k) {
          fk = al[(size_t)k * np] * fk + be[(size_t)k * np];
          ff[lstride * (k - 1)] = (T)fk;
        }
      }
    }
    SYNC;
    PHASE_MARK(PH_TRIDIAG);
    if constexpr (TC != 0) {
      if constexpr (sizeof(T) == 4) {
        tc::Engine E(p.tc_n, tcsm, S.tc_tmem, tc::smem_u32(&S.tc_mbar), &S.tc_phase, &S.tc_fail, TID, NT);
        for (int k0 = 1; k0 <= nzm; k0 += E.d.L) E.inverse_tile(FF, k0, nzm);
        if (TID == 0 && S.tc_fail && S.status == CRM_OK) S.status = CRM_ERR_TIMEOUT;
      }
    } else {
      ycols(+1);
      SYNC;
      xrows(+1);
      SYNC;
    }
    PHASE_MARK(PH_FFT_INV);
    for (int e = TID; e < (nx + 1) * (ny + 1) * nzm; e += NT) {
      const int i = e % (nx + 1), j = (e / (nx + 1)) % (ny + 1), k = 1 + e / ((nx + 1) * (ny + 1));
      pp(i, j, k) = FF(i == 0 ? nx : i, j == 0 ? ny : j, k);
    }
    SYNC;
    for (int e = TID; e < nxy * nzm; e += NT) {
      const int i = 1 + e % nx, j = 1 + (e / nx) % ny, k = 1 + e / nxy;
      const int kb = max(1, k - 1);
      const T rdz = PR(P_RDZW)[k];
      dua(i, j, k) = dua(i, j, k) - (pp(i, j, k) - pp(i - 1, j, k)) * rdx;
      dva(i, j, k) = dva(i, j, k) - (pp(i, j, k) - pp(i, j - 1, k)) * rdy;
      dwa(i, j, k) = dwa(i, j, k) - (pp(i, j, k) - pp(i, j, kb)) * rdz;
    }
    SYNC;
    for (int e = TID; e < (nx + 1) * (ny + 1) * nzm; e += NT) {
      const int i = e % (nx + 1), j = (e / (nx + 1)) % (ny + 1), k = 1 + e / ((nx + 1) * (ny + 1));
      pp(i, j, k) = pp(i, j, k) * rho[k];
    }
    bound_duvdt();
    SYNC;
    PHASE_MARK(PH_PRESS_GRAD);
  }

  // pressure.F90:97-310, press_rhs.F90:48-101, press_grad.F90:18-72,
  // bound_duvdt.F90 (2D); the Fourier coefficients live in shared memory
  __device__ void pressure(T *fsh, T *wsh) {
    FT u = U(), w = W(), pp = PP();
    FT dua = DU(S.na), dub = DU(S.nb), duc = DU(S.nc);
    FT dwa = DW(S.na), dwb = DW(S.nb), dwc = DW(S.nc);
    T *rho = PR(P_RHO), *rhow = PR(P_RHOW), *adz = PR(P_ADZ), *adzw = PR(P_ADZW);
    const T dz = (T)S.dz;
    for (int k = TID + 1; k <= nzm; k += NT) dua(nx + 1, k) = dua(1, k);
    SYNC;
    const T rdx = (T)1. / (T)p.dx;
    const T btat = (T)(S.bt / S.at), ctat = (T)(S.ct / S.at);
    const T dta = (T)(1. / S.dt3[S.na - 1] / S.at);
    const int nx2 = nx + 2;
    for (int e = TID; e < nx * nzm; e += NT) {
      int i = 1 + e % nx, k = 1 + e / nx;
      int kc = k + 1, ic = i + 1;
      T rdz = PR(P_RDZ)[k];
      T rup = PR(P_RUP)[k];
      T rdn = PR(P_RDN)[k];
      T r = (rdx * (u(ic, k) - u(i, k)) + (w(i, kc) * rup - w(i, k) * rdn)) * dta +
            (rdx * (dua(ic, k) - dua(i, k)) + (dwa(i, kc) * rup - dwa(i, k) * rdn)) +
            btat * (rdx * (dub(ic, k) - dub(i, k)) + (dwb(i, kc) * rup - dwb(i, k) * rdn)) +
            ctat * (rdx * (duc(ic, k) - duc(i, k)) + (dwc(i, kc) * rup - dwc(i, k) * rdn));
      fsh[(size_t)nx2 * (k - 1) + (i - 1)] = r * rho[k];
    }
    SYNC;
    PHASE_MARK(PH_PRESS_RHS);
    const int warp = TID >> 5, lane = TID & 31, nwarps = NT >> 5;
    T *wk = wsh + (size_t)warp * (nx + 4);
    for (int k = 1 + warp; k <= nzm; k += nwarps) fft991_warp(fsh + (size_t)nx2 * (k - 1), wk, nx, -1, lane);
    SYNC;
    PHASE_MARK(PH_FFT_FWD);
    // vertical tridiagonal solve per Fourier coefficient, in FP64
    {
      const int np = nx + 1, ls = nzm + 1;
      const double *tri = TRI();
      double *beta = reinterpret_cast<double *>(sa());   // (nzm+1) x np doubles, i fastest
      for (int i = TID + 1; i <= np; i += NT) {
        const double *al = tri + (size_t)ls + (i - 1), *e = al + (size_t)ls * np;
        double *be = beta + (i - 1);
        T *ff = fsh + (i - 1);
        double bprev = (double)ff[0] * e[np];
        be[np] = bprev;
        // the recurrences are serial in k: the loads of each group of
        // levels are issued together, ahead of its arithmetic (the stores
        // to be/ff could alias them, so the compiler would not hoist them)
        constexpr int G = 4;
        for (int k0 = 2; k0 <= nzm - 1; k0 += G) {
          double ev[G], tv[G];
          T fv[G];
#pragma unroll
          for (int j = 0; j < G; ++j) {
            const int k = min(k0 + j, nzm - 1);
            ev[j] = e[(size_t)k * np];
            tv[j] = tri[k];
            fv[j] = ff[(size_t)nx2 * (k - 1)];
          }
#pragma unroll
          for (int j = 0; j < G; ++j) {
            if (k0 + j <= nzm - 1) {
              bprev = ((double)fv[j] - tv[j] * bprev) * ev[j];
              be[(size_t)(k0 + j) * np] = bprev;
            }
          }
        }
        double fk = ((double)ff[(size_t)nx2 * (nzm - 1)] - tri[nzm] * bprev) / tri[(size_t)ls + (size_t)np * 2 * ls + (i - 1)];
        ff[(size_t)nx2 * (nzm - 1)] = (T)fk;
        for (int k0 = nzm - 1; k0 >= 1; k0 -= G) {
          double av[G], bv[G];
#pragma unroll
          for (int j = 0; j < G; ++j) {
            const int k = max(k0 - j, 1);
            av[j] = al[(size_t)k * np];
            bv[j] = be[(size_t)k * np];
          }
#pragma unroll
          for (int j = 0; j < G; ++j) {
            if (k0 - j >= 1) {
              fk = av[j] * fk + bv[j];
              ff[(size_t)nx2 * (k0 - j - 1)] = (T)fk;
            }
          }
        }
      }
    }
    SYNC;
    PHASE_MARK(PH_TRIDIAG);
    for (int k = 1 + warp; k <= nzm; k += nwarps) fft991_warp(fsh + (size_t)nx2 * (k - 1), wk, nx, +1, lane);
    SYNC;
    PHASE_MARK(PH_FFT_INV);
    for (int e = TID; e < (nx + 1) * nzm; e += NT) {
      int i = e % (nx + 1), k = 1 + e / (nx + 1);
      pp(i, k) = fsh[(size_t)nx2 * (k - 1) + ((i == 0 ? nx : i) - 1)];
    }
    SYNC;
    FT dva = DV(S.na);
    const T rdy = (T)1. / (T)p.dy;
    for (int e = TID; e < nx * nzm; e += NT) {
      int i = 1 + e % nx, k = 1 + e / nx;
      int kb = max(1, k - 1);
      T rdz = PR(P_RDZW)[k];
      dua(i, k) = dua(i, k) - (pp(i, k) - pp(i - 1, k)) * rdx;
      dva(i, k) = dva(i, k) - (pp(i, k) - pp(i, k)) * rdy;
      dwa(i, k) = dwa(i, k) - (pp(i, k) - pp(i, kb)) * rdz;
    }
    SYNC;
    for (int e = TID; e < (nx + 1) * nzm; e += NT) {
      int i = e % (nx + 1), k = 1 + e / (nx + 1);
      pp(i, k) = pp(i, k) * rho[k];
    }
    for (int k = TID + 1; k <= nzm; k += NT) dua(nx + 1, k) = dua(1, k);
    SYNC;
    PHASE_MARK(PH_PRESS_GRAD);
  }

  // ---------------------------------------------------------- adams / uvw
  __device__ void adams() {                    // adams.F90:17-38
    FT u = U(), v = V(), w = W();
    FT dua = DU(S.na), dub = DU(S.nb), duc = DU(S.nc);
    FT dva = DV(S.na), dvb = DV(S.nb), dvc = DV(S.nc);
    FT dwa = DW(S.na), dwb = DW(S.nb), dwc = DW(S.nc);
    const T dtdx = (T)(S.dtn / p.dx), dtdz = (T)(S.dtn / S.dz), dtdy = (T)(S.dtn / p.dy);
    const T d3 = (T)S.dt3[S.na - 1], at = (T)S.at, bt = (T)S.bt, ct = (T)S.ct;
    T *rho = PR(P_RHO), *rhow = PR(P_RHOW);
    if constexpr (sizeof(T) == 8) {
      for (int e = TID; e < NH() * nzm; e += NT) {
        int i = 1 + e % NH(), k = 1 + e / NH();
        T rhox = rho[k] * dtdx, rhoy = rho[k] * dtdy, rhoz = rhow[k] * dtdz;
        T un = u(i, k) + d3 * (at * dua(i, k) + bt * dub(i, k) + ct * duc(i, k));
        T vn = v(i, k) + d3 * (at * dva(i, k) + bt * dvb(i, k) + ct * dvc(i, k));
        T wn = w(i, k) + d3 * (at * dwa(i, k) + bt * dwb(i, k) + ct * dwc(i, k));
        duc(i, k) = un; dvc(i, k) = vn; dwc(i, k) = wn;
        u(i, k) = (T)0.5 * (u(i, k) + un) * rhox;
        v(i, k) = (T)0.5 * (v(i, k) + vn) * rhoy;
        w(i, k) = (T)0.5 * (w(i, k) + wn) * rhoz;
      }
    } else {
      // FP32-mixed form: the projected new w has zero horizontal mean at
      // every level in exact arithmetic (anelastic continuity, periodic
      // sides, w = 0 at the surface; the FP64 form's means are ~1e-16 of the
      // level's rms w).  FP32 rounding in the momentum and pressure phases
      // leaves a mean of ~1e-6 of the rms, and the upwind scalar fluxes of
      // the next advection multiply it by the level's mean value (~300 K for
      // t), which moved the level means of t by ~1e-4 of their change over a
      // call.  The mean, summed in FP64, is taken out of the new w before it
      // forms the advecting flux (w = 0.5 (w_old + w_new) rho dt/dz).  A warp
      // per level: the level's sum is reduced by the warp that formed it and
      // applied by the same threads to the cells they wrote.
      const int lane = TID & 31, warp = TID >> 5, nw = NT >> 5;
      const double fxy = 1. / (double)NH();
      for (int k = 1 + warp; k <= nzm; k += nw) {
        const T rhox = rho[k] * dtdx, rhoy = rho[k] * dtdy, rhoz = rhow[k] * dtdz;
        double sm = 0.;
        for (int h = 1 + lane; h <= NH(); h += 32) {
          T un = u(h, k) + d3 * (at * dua(h, k) + bt * dub(h, k) + ct * duc(h, k));
          T vn = v(h, k) + d3 * (at * dva(h, k) + bt * dvb(h, k) + ct * dvc(h, k));
          T wn = w(h, k) + d3 * (at * dwa(h, k) + bt * dwb(h, k) + ct * dwc(h, k));
          duc(h, k) = un; dvc(h, k) = vn; dwc(h, k) = wn;
          u(h, k) = (T)0.5 * (u(h, k) + un) * rhox;
          v(h, k) = (T)0.5 * (v(h, k) + vn) * rhoy;
          sm = sm + (double)wn;
        }
        for (int o = 16; o > 0; o >>= 1) sm = sm + __shfl_xor_sync(0xffffffffu, sm, o);
        const T wm = k >= 2 ? (T)(sm * fxy) : (T)0.;
        for (int h = 1 + lane; h <= NH(); h += 32) {
          T wn = dwc(h, k);
          if (k >= 2) {
            wn = wn - wm;
            dwc(h, k) = wn;
          }
          w(h, k) = (T)0.5 * (w(h, k) + wn) * rhoz;
        }
      }
    }
    SYNC;
  }
  __device__ void uvw() {                      // uvw.F90
    FT u = U(), v = V(), w = W(), duc = DU(S.nc), dvc = DV(S.nc), dwc = DW(S.nc);
    for (int e = TID; e < NH() * nzm; e += NT) {
      int i = 1 + e % NH(), k = 1 + e / NH();
      u(i, k) = duc(i, k); v(i, k) = dvc(i, k); w(i, k) = dwc(i, k);
    }
    SYNC;
  }

  // ---------------------------------------------------------- MPDATA
  // ADV_MPDATA/advect_scalar.F90:39-72 + advect_scalar2D.F90:60-240.
  // f is advected in place; fadv/flux (may be null) receive the per-level
  // advective tendency sum and vertical flux sum.
  // Runs a pass over cells e = TID, TID + NT, ... < n two cells per thread at
  // a time: calc(e) only loads and computes, put(e, r) only stores, so both
  // cells' loads are in flight together (stores through the field pointers
  // would otherwise keep the compiler from hoisting the second cell's loads).
  template <typename Calc, typename Put>
  __device__ __forceinline__ void for_cells2(int n, Calc calc, Put put) {
    int e = TID;
    for (; e + NT < n; e += 2 * NT) {
      const auto r0 = calc(e);
      const auto r1 = calc(e + NT);
      put(e, r0);
      put(e + NT, r1);
    }
    if (e < n) put(e, calc(e));
  }

  // True when every stored value of a scalar field (x halos included) is +0
  // bit for bit.  Advection (MPDATA) and SGS diffusion of such a field leave
  // every bit of it unchanged and give +0 for their statistics (every flux is
  // a signed zero, every update adds or subtracts a zero to +0), so a column
  // without precipitating water skips both for qp.
  __device__ bool all_pos_zero(FT f) {
    int nonzero = 0;
    // 2D: the x row of every level 1..nzm; 3D: every stored cell of those
    // levels (x and y halos included), which lie contiguous
    const int n = Y3 ? f.plane * nzm : (nx + 6) * nzm;
    for (int e = TID; e < n; e += NT) {
      T v;
      if constexpr (Y3) v = f.p[e];
      else v = f(-2 + e % (nx + 6), 1 + e / (nx + 6));
      if constexpr (sizeof(T) == 8) nonzero |= (__double_as_longlong(v) != 0);
      else nonzero |= (__float_as_uint(v) != 0u);
    }
    return !__syncthreads_or(nonzero);
  }
  // the statistics a skipped advection or diffusion of a zero field gives
  __device__ void zero_stats(T *a, T *b) {
    for (int k = TID + 1; k <= nzm; k += NT) {
      if (a) a[k] = (T)0.;
      if (b) b[k] = (T)0.;
    }
    SYNC;
  }

  // FP32-mixed form: t is advected as its offset from a column constant c
  // (the call's initial level-1 mean of t, rounded to an integer).  The
  // upwind pass forms its fluxes u+ f(i-1) + u- f(i) (and the w terms) from
  // f - c, writes the intermediate field as f - c (with the bounds of the
  // limiter), and the final update adds c back through an exact two-sum into
  // the carried residue; the positive-definite clip sees the value itself.
  // The upwind update changes by c D, D the advecting velocity's discrete
  // divergence, which is zero in exact arithmetic when that velocity is the
  // mean of two projected fields: from the second substep of the call (the
  // first one's old velocity is the input state).  Every other MPDATA term
  // sees f only through differences.  In FP32 the lowest levels' fluxes and
  // intermediate values are then a few K instead of ~300 K, and their
  // rounding, which reached the level means of t and so sltend, drops with
  // them (64x58 dry columns over 1200 s: sltend 1.3e-4 -> 5.8e-5 relative
  // L2; over 100 s 7e-5 -> 2.9e-5).  The halos the upwind pass writes keep
  // the offset; the next exchange before any read of them rewrites them.
  __device__ __forceinline__ T t_offset(int nstep, int icyc) const {
    if constexpr (sizeof(T) == 4) return (nstep >= 2 || icyc >= 2) ? (T)S.t_off : (T)0.;
    return (T)0.;
  }
  __device__ void advect_scalar(FT f, T *fadv, T *flux, T *rc = nullptr, T toff = (T)0.) {
    FT u = U(), w = W();
    FT mx = SA(), mn = SB(), uuu = SCR(p.L.s_c), www = SCR(p.L.s_d), f0 = SCR(p.L.s_e);
    FT wfl1 = SCR(p.L.s_f);
    T *rho = PR(P_RHO), *adz = PR(P_ADZ), *rhow = PR(P_RHOW);
    const T eps = (T)R4(1.e-10);
    // Every pass gathers from other cells and writes only its own cell, so
    // each runs two cells per thread at a time (for_cells2: both cells'
    // loads are issued before either's stores).
    // f0, mx/mn from the initial field, upwind fluxes
    struct R1 { int i, k; T mx, mn, fk, uuu, www; };
    for_cells2((nx + 5) * nzm,
      [&](int e) -> R1 {
        R1 r;
        r.i = -1 + e % (nx + 5); r.k = 1 + e / (nx + 5);    // i = -1 .. nx+3
        const int i = r.i, k = r.k, kc = min(nzm, k + 1), kb = max(1, k - 1);
        const T fk = f(i, k), fb = f(i - 1, k), uk = u(i, k);
        const bool in_w = i <= nx + 2, in_m = i >= 0 && i <= nx + 1;
        const T fkb = in_w ? f(i, kb) : (T)0., wk = in_w ? w(i, k) : (T)0.;
        const T fc = in_m ? f(i + 1, k) : (T)0., fkc = in_m ? f(i, kc) : (T)0.;
        r.mx = mx2(mx2(mx2(mx2(fb, fc), fkb), fkc), fk);
        r.mn = mn2(mn2(mn2(mn2(fb, fc), fkb), fkc), fk);
        r.fk = fk;
        r.uuu = mx2((T)0., uk) * (fb - toff) + mn2((T)0., uk) * (fk - toff);
        r.www = mx2((T)0., wk) * (fkb - toff) + mn2((T)0., wk) * (fk - toff);
        return r;
      },
      [&](int, const R1 &r) {
        const int i = r.i, k = r.k;
        const bool in_w = i <= nx + 2, in_m = i >= 0 && i <= nx + 1;
        if (in_m) { mx(i, k) = r.mx - toff; mn(i, k) = r.mn - toff; }
        if (fadv && i >= 1 && i <= nx) f0(i, k) = r.fk;
        uuu(i, k) = r.uuu;
        if (in_w) {
          www(i, k) = r.www;
          if (k == 1) www(i, nz) = (T)0.;
        }
      });
    SYNC;
    // first-pass (upwind) vertical flux sum, then the upwind update; the
    // residue keeps the update's rounding error (the next update folds it in)
    if (flux)
      level_sums_lo(1, 1, nzm, [&](int, int i, int k) -> T { return www(i, k); },
                 [&](int, int) { return 0.; }, [&](int, int k, double sv) { wfl1(0, k) = (T)sv; });
    struct R2 { int i, k; T fn, err; };
    for_cells2((nx + 4) * nzm,
      [&](int e) -> R2 {
        R2 r;
        r.i = -1 + e % (nx + 4); r.k = 1 + e / (nx + 4);    // -1 .. nx+2
        const int i = r.i, k = r.k;
        const T iadz = PR(P_IADZ)[k], irho = PR(P_IRHO)[k];
        const T c1 = (uuu(i + 1, k) - uuu(i, k) + (www(i, k + 1) - www(i, k)) * iadz) * irho;
        r.err = (T)0.;
        if (sizeof(T) == 4 && rc && i >= 1 && i <= nx) r.fn = add_carry(f(i, k) - toff, -c1, r.err);
        else r.fn = (f(i, k) - toff) - c1;
        return r;
      },
      [&](int, const R2 &r) {
        f(r.i, r.k) = r.fn;
        if (sizeof(T) == 4 && rc && r.i >= 1 && r.i <= nx) rc[(r.i - 1) + nx * (r.k - 1)] += r.err;
      });
    SYNC;
    // antidiffusive velocities (andiff, across)
    struct R3 { int i, k; T uval, wval; };
    for_cells2((nx + 3) * nzm,
      [&](int e) -> R3 {
        R3 r;
        r.i = e % (nx + 3); r.k = 1 + e / (nx + 3);          // 0 .. nx+2
        const int i = r.i, k = r.k, kc = min(nzm, k + 1), kb = max(1, k - 1), ib = i - 1;
        const T irho = PR(P_IRHO)[k], irhow = PR(P_IRHOWADZ)[k], dd = PR(P_MPDD)[k];
        {
          T a = u(i, k), x1 = f(ib, k), x2 = f(i, k);
          T andiff = (tabs_(a) - a * a * irho) * (T)0.5 * (x2 - x1);
          T ax1 = dd * (f(ib, kc) + f(i, kc) - f(ib, kb) - f(i, kb));
          T a2 = w(ib, k) + w(ib, kc) + w(i, k) + w(i, kc);
          T across = (T)0.03125 * a * a2 * ax1;
          r.uval = andiff - across * irho;
        }
        r.wval = (T)0.;
        if (i <= nx + 1) {
          int ic = i + 1;
          T a = w(i, k), x1 = f(i, kb), x2 = f(i, k);
          T andiff = (tabs_(a) - a * a * irhow) * (T)0.5 * (x2 - x1);
          T ax1 = f(ic, kb) + f(ic, k) - f(ib, kb) - f(ib, k);
          T a2 = u(i, kb) + u(i, k) + u(ic, k) + u(ic, kb);
          T across = (T)0.03125 * a * a2 * ax1;
          r.wval = (k == 1) ? (T)0. : andiff - across * irho;
        }
        return r;
      },
      [&](int, const R3 &r) {
        uuu(r.i, r.k) = r.uval;
        if (r.i <= nx + 1) www(r.i, r.k) = r.wval;
      });
    SYNC;
    // non-oscillatory limiter
    struct R4 { int i, k; T mxv, mnv; };
    for_cells2((nx + 2) * nzm,
      [&](int e) -> R4 {
        R4 r;
        r.i = e % (nx + 2); r.k = 1 + e / (nx + 2);          // 0 .. nx+1
        const int i = r.i, k = r.k, kc = min(nzm, k + 1), kb = max(1, k - 1), ib = i - 1, ic = i + 1;
        const T iadz = PR(P_IADZ)[k];
        T m1 = mx2(mx2(mx2(mx2(mx2(f(ib, k), f(ic, k)), f(i, kb)), f(i, kc)), f(i, k)), mx(i, k));
        T m2 = mn2(mn2(mn2(mn2(mn2(f(ib, k), f(ic, k)), f(i, kb)), f(i, kc)), f(i, k)), mn(i, k));
        const T fk = f(i, k), uc = uuu(ic, k), ui = uuu(i, k), wc = www(i, kc), wi = www(i, k);
        T pu_c = -mn2((T)0., uc), pu_i = mx2((T)0., ui);
        T pw_c = -mn2((T)0., wc), pw_i = mx2((T)0., wi);
        r.mxv = rho[k] * (m1 - fk) / (pu_c + pu_i + iadz * (pw_c + pw_i) + eps);
        T qu_c = mx2((T)0., uc), qu_i = -mn2((T)0., ui);
        T qw_c = mx2((T)0., wc), qw_i = -mn2((T)0., wi);
        r.mnv = rho[k] * (fk - m2) / (qu_c + qu_i + iadz * (qw_c + qw_i) + eps);
        return r;
      },
      [&](int, const R4 &r) {
        mx(r.i, r.k) = r.mxv;
        mn(r.i, r.k) = r.mnv;
      });
    SYNC;
    struct R5 { int i, k; T uval, wval; };
    for_cells2((nx + 1) * nzm,
      [&](int e) -> R5 {
        R5 r;
        r.i = 1 + e % (nx + 1); r.k = 1 + e / (nx + 1);      // 1 .. nx+1
        const int i = r.i, k = r.k, ib = i - 1;
        const T uu = uuu(i, k), mxk = mx(i, k), mnk = mn(i, k);
        r.uval = mx2((T)0., uu) * mn3((T)1., mxk, mn(ib, k)) - (-mn2((T)0., uu)) * mn3((T)1., mx(ib, k), mnk);
        r.wval = (T)0.;
        if (i <= nx) {
          int kb = max(1, k - 1);
          const T ww = www(i, k);
          r.wval = mx2((T)0., ww) * mn3((T)1., mxk, mn(i, kb)) - (-mn2((T)0., ww)) * mn3((T)1., mx(i, kb), mnk);
        }
        return r;
      },
      [&](int, const R5 &r) {
        if (r.i <= nx) www(r.i, r.k) = r.wval;
        uuu(r.i, r.k) = r.uval;
      });
    SYNC;
    if (flux)
      level_sums_lo(1, 1, nzm, [&](int, int i, int k) -> T { return www(i, k); },
                 [&](int, int k) { return (double)wfl1(0, k); },
                 [&](int, int k, double sv) { flux[k] = (T)sv; });
    // final update with the positive-definite clip
    struct R6 { int i, k; T fn, r; };
    for_cells2(nx * nzm,
      [&](int e) -> R6 {
        R6 r;
        r.i = 1 + e % nx; r.k = 1 + e / nx;
        const int i = r.i, k = r.k;
        const T iadz = PR(P_IADZ)[k], irho = PR(P_IRHO)[k];
        const T c2 = (uuu(i + 1, k) - uuu(i, k) + (www(i, k + 1) - www(i, k)) * iadz) * irho;
        if (sizeof(T) == 4 && rc) {
          r.r = rc[e];
          r.fn = add_carry(f(i, k), -c2, r.r);
          if (toff != (T)0.) {
            T e2 = (T)0.;
            r.fn = add_carry(toff, r.fn, e2);
            r.r = r.r + e2;
          }
          if (!(r.fn > (T)0.)) { r.fn = (T)0.; r.r = (T)0.; }
        } else {
          r.r = (T)0.;
          r.fn = mx2((T)0., (f(i, k) - c2) + toff);
        }
        return r;
      },
      [&](int e, const R6 &r) {
        f(r.i, r.k) = r.fn;
        if (sizeof(T) == 4 && rc) rc[e] = r.r;
      });
    SYNC;
    if (fadv) {
      level_sums_lo(1, 1, nzm, [&](int, int i, int k) -> T { return f(i, k) - f0(i, k); },
                 [&](int, int) { return 0.; }, [&](int, int k, double sv) { fadv[k] = (T)sv; });
      SYNC;
    }
  }

  // ---------------------------------------------------------- MPDATA, 3D
  // ADV_MPDATA/advect_scalar3D.F90:8-349 (nonos, no walls) with the
  // advect_scalar.F90 wrapper's fadv; scratch planes: mx, mn in A, B, the
  // fluxes uuu, vvv, www in C, D, E, the initial field in F, the first-pass
  // vertical flux sum in G
  __device__ void advect_scalar3(FT f, T *fadv, T *flux, T *rc = nullptr, T toff = (T)0.) {
    FT u = U(), v = V(), w = W();
    FT mx = SA(), mn = SB(), uuu = SCR(p.L.s_c), vvv = SCR(p.L.s_d), www = SCR(p.L.s_e), f0 = SCR(p.L.s_f);
    FT wfl1 = SCR(p.L.s_g);
    T *rho = PR(P_RHO);
    const T eps = (T)R4(1.e-10);
    const int nxy = nx * ny;
    auto mx7 = [](T a, T b, T c, T d, T e, T f_, T g) { return mx2(mx2(mx2(mx2(mx2(mx2(a, b), c), d), e), f_), g); };
    auto mn7 = [](T a, T b, T c, T d, T e, T f_, T g) { return mn2(mn2(mn2(mn2(mn2(mn2(a, b), c), d), e), f_), g); };
    // bounds of the initial field, upwind fluxes (i = -1..nx+3, j = -1..ny+3)
    {
      const int wx = nx + 5, wy = ny + 5;
      for (int e = TID; e < wx * wy * nzm; e += NT) {
        const int i = -1 + e % wx, j = -1 + (e / wx) % wy, k = 1 + e / (wx * wy);
        const int kc = min(nzm, k + 1), kb = max(1, k - 1);
        if (i >= 0 && i <= nx + 1 && j >= 0 && j <= ny + 1) {
          const T a = f(i - 1, j, k), b = f(i + 1, j, k), c = f(i, j - 1, k), d = f(i, j + 1, k);
          const T fb = f(i, j, kb), fc = f(i, j, kc), fk = f(i, j, k);
          mx(i, j, k) = mx7(a, b, c, d, fb, fc, fk) - toff;
          mn(i, j, k) = mn7(a, b, c, d, fb, fc, fk) - toff;
        }
        if (j <= ny + 2) {
          const T uk = u(i, j, k);
          uuu(i, j, k) = mx2((T)0., uk) * (f(i - 1, j, k) - toff) + mn2((T)0., uk) * (f(i, j, k) - toff);
        }
        if (i <= nx + 2) {
          const T vk = v(i, j, k);
          vvv(i, j, k) = mx2((T)0., vk) * (f(i, j - 1, k) - toff) + mn2((T)0., vk) * (f(i, j, k) - toff);
        }
        if (i <= nx + 2 && j <= ny + 2) {
          const T wk = w(i, j, k);
          www(i, j, k) = mx2((T)0., wk) * (f(i, j, kb) - toff) + mn2((T)0., wk) * (f(i, j, k) - toff);
          if (k == 1) www(i, j, nz) = (T)0.;
        }
        if (fadv && i >= 1 && i <= nx && j >= 1 && j <= ny) f0(i, j, k) = f(i, j, k);
      }
    }
    SYNC;
    if (flux)
      level_sums_lo(1, 1, nzm, [&](int, int h, int k) -> T { return www(h, k); },
                    [&](int, int) { return 0.; }, [&](int, int k, double sv) { wfl1(0, 0, k) = (T)sv; });
    // upwind update (i = -1..nx+2, j = -1..ny+2); the residue keeps the
    // interior update's rounding error
    {
      const int wx = nx + 4, wy = ny + 4;
      for (int e = TID; e < wx * wy * nzm; e += NT) {
        const int i = -1 + e % wx, j = -1 + (e / wx) % wy, k = 1 + e / (wx * wy);
        const T iadz = PR(P_IADZ)[k], irho = PR(P_IRHO)[k];
        const T c1 = (uuu(i + 1, j, k) - uuu(i, j, k) + vvv(i, j + 1, k) - vvv(i, j, k) +
                      (www(i, j, k + 1) - www(i, j, k)) * iadz) * irho;
        if (sizeof(T) == 4 && rc && i >= 1 && i <= nx && j >= 1 && j <= ny) {
          T err = (T)0.;
          f(i, j, k) = add_carry(f(i, j, k) - toff, -c1, err);
          rc[(size_t)(i - 1) + (size_t)nx * (j - 1) + (size_t)nxy * (k - 1)] += err;
        } else {
          f(i, j, k) = (f(i, j, k) - toff) - c1;
        }
      }
    }
    SYNC;
    // antidiffusive velocities (i = 0..nx+2, j = 0..ny+2)
    {
      const int wx = nx + 3, wy = ny + 3;
      for (int e = TID; e < wx * wy * nzm; e += NT) {
        const int i = e % wx, j = (e / wx) % wy, k = 1 + e / (wx * wy);
        const int kc = min(nzm, k + 1), kb = max(1, k - 1), ib = i - 1, ic = i + 1, jb = j - 1, jc = j + 1;
        const T irho = PR(P_IRHO)[k], irhow = PR(P_IRHOWADZ)[k], dd = PR(P_MPDD)[k];
        T uval = (T)0., vval = (T)0., wval = (T)0.;
        if (j <= ny + 1) {
          const T a = u(i, j, k);
          const T andiff = (tabs_(a) - a * a * irho) * (T)0.5 * (f(i, j, k) - f(ib, j, k));
          const T ac1 = (T)0.03125 * a * (v(ib, j, k) + v(ib, jc, k) + v(i, jc, k) + v(i, j, k)) *
                        (f(ib, jc, k) + f(i, jc, k) - f(ib, jb, k) - f(i, jb, k));
          const T ac2 = (T)0.03125 * a * (w(ib, j, k) + w(ib, j, kc) + w(i, j, k) + w(i, j, kc)) *
                        (dd * (f(ib, j, kc) + f(i, j, kc) - f(ib, j, kb) - f(i, j, kb)));
          uval = andiff - (ac1 + ac2) * irho;
        }
        if (i <= nx + 1) {
          const T a = v(i, j, k);
          const T andiff = (tabs_(a) - a * a * irho) * (T)0.5 * (f(i, j, k) - f(i, jb, k));
          const T ac1 = (T)0.03125 * a * (u(i, jb, k) + u(i, j, k) + u(ic, j, k) + u(ic, jb, k)) *
                        (f(ic, jb, k) + f(ic, j, k) - f(ib, jb, k) - f(ib, j, k));
          const T ac2 = (T)0.03125 * a * (w(i, jb, k) + w(i, j, k) + w(i, j, kc) + w(i, jb, kc)) *
                        (dd * (f(i, jb, kc) + f(i, j, kc) - f(i, jb, kb) - f(i, j, kb)));
          vval = andiff - (ac1 + ac2) * irho;
        }
        if (i <= nx + 1 && j <= ny + 1 && k > 1) {
          const T a = w(i, j, k);
          const T andiff = (tabs_(a) - a * a * irhow) * (T)0.5 * (f(i, j, k) - f(i, j, kb));
          const T ac1 = (T)0.03125 * a * (u(i, j, kb) + u(i, j, k) + u(ic, j, k) + u(ic, j, kb)) *
                        (f(ic, j, kb) + f(ic, j, k) - f(ib, j, kb) - f(ib, j, k));
          const T ac2 = (T)0.03125 * a * (v(i, j, kb) + v(i, jc, kb) + v(i, jc, k) + v(i, j, k)) *
                        (f(i, jc, k) + f(i, jc, kb) - f(i, jb, k) - f(i, jb, kb));
          wval = andiff - (ac1 + ac2) * irho;
        }
        if (j <= ny + 1) uuu(i, j, k) = uval;
        if (i <= nx + 1) vvv(i, j, k) = vval;
        if (i <= nx + 1 && j <= ny + 1) www(i, j, k) = wval;
      }
    }
    SYNC;
    // non-oscillatory limiter (i = 0..nx+1, j = 0..ny+1)
    {
      const int wx = nx + 2, wy = ny + 2;
      for (int e = TID; e < wx * wy * nzm; e += NT) {
        const int i = e % wx, j = (e / wx) % wy, k = 1 + e / (wx * wy);
        const int kc = min(nzm, k + 1), kb = max(1, k - 1);
        const T iadz = PR(P_IADZ)[k];
        const T a = f(i - 1, j, k), b = f(i + 1, j, k), c = f(i, j - 1, k), d = f(i, j + 1, k);
        const T fb = f(i, j, kb), fc = f(i, j, kc), fk = f(i, j, k);
        const T m1 = mx2(mx7(a, b, c, d, fb, fc, fk), mx(i, j, k));
        const T m2 = mn2(mn7(a, b, c, d, fb, fc, fk), mn(i, j, k));
        const T uc = uuu(i + 1, j, k), ui = uuu(i, j, k), vc = vvv(i, j + 1, k), vi = vvv(i, j, k);
        const T wc = www(i, j, kc), wi = www(i, j, k);
        const T dmx = -mn2((T)0., uc) + mx2((T)0., ui) + -mn2((T)0., vc) + mx2((T)0., vi) +
                      (-mn2((T)0., wc) + mx2((T)0., wi)) * iadz + eps;
        const T dmn = mx2((T)0., uc) + -mn2((T)0., ui) + mx2((T)0., vc) + -mn2((T)0., vi) +
                      (mx2((T)0., wc) + -mn2((T)0., wi)) * iadz + eps;
        mx(i, j, k) = rho[k] * (m1 - fk) / dmx;
        mn(i, j, k) = rho[k] * (fk - m2) / dmn;
      }
    }
    SYNC;
    // limited antidiffusive fluxes (i = 1..nx+1, j = 1..ny+1)
    {
      const int wx = nx + 1, wy = ny + 1;
      for (int e = TID; e < wx * wy * nzm; e += NT) {
        const int i = 1 + e % wx, j = 1 + (e / wx) % wy, k = 1 + e / (wx * wy);
        const T mxk = mx(i, j, k), mnk = mn(i, j, k);
        if (j <= ny) {
          const T uu = uuu(i, j, k);
          uuu(i, j, k) = mx2((T)0., uu) * mn3((T)1., mxk, mn(i - 1, j, k)) -
                         (-mn2((T)0., uu)) * mn3((T)1., mx(i - 1, j, k), mnk);
        }
        if (i <= nx) {
          const T vv = vvv(i, j, k);
          vvv(i, j, k) = mx2((T)0., vv) * mn3((T)1., mxk, mn(i, j - 1, k)) -
                         (-mn2((T)0., vv)) * mn3((T)1., mx(i, j - 1, k), mnk);
        }
        if (i <= nx && j <= ny) {
          const int kb = max(1, k - 1);
          const T ww = www(i, j, k);
          www(i, j, k) = mx2((T)0., ww) * mn3((T)1., mxk, mn(i, j, kb)) -
                         (-mn2((T)0., ww)) * mn3((T)1., mx(i, j, kb), mnk);
        }
      }
    }
    SYNC;
    if (flux)
      level_sums_lo(1, 1, nzm, [&](int, int h, int k) -> T { return www(h, k); },
                    [&](int, int k) { return (double)wfl1(0, 0, k); },
                    [&](int, int k, double sv) { flux[k] = (T)sv; });
    // final update with the positive-definite clip
    for (int e = TID; e < nxy * nzm; e += NT) {
      const int i = 1 + e % nx, j = 1 + (e / nx) % ny, k = 1 + e / nxy;
      const T iadz = PR(P_IADZ)[k], irho = PR(P_IRHO)[k];
      const T c2 = (uuu(i + 1, j, k) - uuu(i, j, k) + vvv(i, j + 1, k) - vvv(i, j, k) +
                    (www(i, j, k + 1) - www(i, j, k)) * iadz) * irho;
      if (sizeof(T) == 4 && rc) {
        T r = rc[e];
        T fn = add_carry(f(i, j, k), -c2, r);
        if (toff != (T)0.) {
          T e2 = (T)0.;
          fn = add_carry(toff, fn, e2);
          r = r + e2;
        }
        if (!(fn > (T)0.)) { fn = (T)0.; r = (T)0.; }
        f(i, j, k) = fn;
        rc[e] = r;
      } else {
        f(i, j, k) = mx2((T)0., (f(i, j, k) - c2) + toff);
      }
    }
    SYNC;
    if (fadv) {
      level_sums_lo(1, 1, nzm, [&](int, int h, int k) -> T { return f(h, k) - f0(h, k); },
                    [&](int, int) { return 0.; }, [&](int, int k, double sv) { fadv[k] = (T)sv; });
      SYNC;
    }
  }

  // ---------------------------------------------------------- precip_fall
  // MICRO_SAM1MOM/microphysics.F90:453-486 (term_vel_qp) and :491-833
  __device__ T term_vel(T tabs, T rho, T qploc) const {
    T term = (T)0.;
    if (qploc > (T)C_QP_THRESHOLD) {
      T omp = mx2((T)0., mn2((T)1., (tabs - (T)C_TPRMIN) * (T)p.a_pr));
      if (omp == (T)1.) {
        term = (T)p.vrain * tpow(rho * qploc, (T)p.crain);
      } else if (omp == (T)0.) {
        T omg = mx2((T)0., mn2((T)1., (tabs - (T)C_TGRMIN) * (T)p.a_gr));
        T qgg = omg * qploc;
        T qss = qploc - qgg;
        term = omg * (T)p.vgrau * tpow(rho * qgg, (T)p.cgrau) + ((T)1. - omg) * (T)p.vsnow * tpow(rho * qss, (T)p.csnow);
      } else {
        T omg = mx2((T)0., mn2((T)1., (tabs - (T)C_TGRMIN) * (T)p.a_gr));
        T qrr = omp * qploc;
        T qss = qploc - qrr;
        T qgg = omg * qss;
        qss = qss - qgg;
        term = omp * (T)p.vrain * tpow(rho * qrr, (T)p.crain) +
               ((T)1. - omp) * (omg * (T)p.vgrau * tpow(rho * qgg, (T)p.cgrau) + ((T)1. - omg) * (T)p.vsnow * tpow(rho * qss, (T)p.csnow));
      }
    }
    return term;
  }
  // part 1: terminal velocities and the column precipitation CFL number
  __device__ void precip_fall_1(bool qp_zero) {
    if (qp_zero) {
      // qp is +0 in every cell: every fall speed is zero (term_vel below
      // returns 0 at or under the threshold), so the loops below would give
      // a CFL of 0, no moving cell and one sub-step, and write only planes
      // that precip_fall_2, then skipped, reads.  The batch maximum is still
      // taken, as every column of a reference batch must arrive.
      const double cfl_b = batch_max(0.);
      if (TID == 0) {
        S.prec_cfl = 0.;
        S.prec_any = 0;
        const double nf = ceil(cfl_b / R4(0.9));
        S.nprec = (cfl_b > R4(0.9)) ? (nf < 1.0e4 ? (int)nf : 10000) : 1;
      }
      SYNC;
      return;
    }
    FT tabs = TABS(), qp = QP();
    FT wp = SA(), omega = SB();
    T *rho = PR(P_RHO), *rhow = PR(P_RHOW), *adz = PR(P_ADZ);
    T *rhofac = PR(P_TMP4), *irhoadz = PR(P_TMP5), *iwmax = PR(P_TMP6);
    const T dtn = (T)S.dtn, dz = (T)S.dz;
    for (int k = TID + 1; k <= nzm; k += NT) {
      rhofac[k] = tsqrt((T)R4(1.29) / rho[k]);
      irhoadz[k] = (T)1. / (rho[k] * adz[k]);
      int kb = max(1, k - 1);
      T wmax = dz * adz[kb] / dtn;
      iwmax[k] = (T)1. / wmax;
    }
    SYNC;
    // the maximum is taken in T and widened once (widening is exact and
    // monotone, so the result equals a maximum of widened values)
    T cflt = (T)0.;
    int moving = 0;
    for (int e = TID; e < NH() * nzm; e += NT) {
      int i = 1 + e % NH(), k = 1 + e / NH();
      omega(i, k) = mx2((T)0., mn2((T)1., (tabs(i, k) - (T)C_TPRMIN) * (T)p.a_pr));
      T tmp = term_vel(tabs(i, k), rho[k], qp(i, k));
      T wv = rhofac[k] * tmp;
      cflt = mx2(cflt, wv * iwmax[k]);
      wp(i, k) = -wv * rhow[k] * dtn / dz;
      moving |= (wv != (T)0.);
    }
    // With every fall speed zero (wp = -0 everywhere) the sedimentation
    // sub-steps change no bit of qp, t, the surface precipitation or the
    // qpfall/precflux sums (every flux works out to +0 and every update adds
    // or subtracts a zero to a value it leaves unchanged, signs of zero
    // included), so precip_fall_2 is skipped for such a column.
    moving = __syncthreads_or(moving);
    double cfl = block_max((double)cflt);
    const double cfl_b = batch_max(cfl);
    if (TID == 0) {
      S.prec_cfl = cfl;
      S.prec_any = moving;
      // ceil(cfl / 0.9) sub-steps (microphysics.F90:602-661), saturated at
      // 10^4 so that garbage fall speeds cannot make the loop unbounded
      const double nf = ceil(cfl_b / R4(0.9));
      S.nprec = (cfl_b > R4(0.9)) ? (nf < 1.0e4 ? (int)nf : 10000) : 1;
    }
    SYNC;
  }
  // part 2: nprec monotone flux-limited sedimentation sub-steps
  __device__ void precip_fall_2(int nprec) {
    FT tabs = TABS(), qp = QP(), t = TT();
    FT wp = SA(), omega = SB(), tq = SCR(p.L.s_c), fz = SCR(p.L.s_d);
    FT mx = SCR(p.L.s_e), mn = SCR(p.L.s_f), www = SCR(p.L.s_g);
    T *rho = PR(P_RHO), *rhow = PR(P_RHOW), *adz = PR(P_ADZ);
    T *rhofac = PR(P_TMP4), *irhoadz = PR(P_TMP5);
    T *qpfall = PR(P_QPFALL), *precflux = PR(P_PRECFLUX);
    const T eps = (T)R4(1.e-10);
    const T dtn = (T)S.dtn, dz = (T)S.dz;
    const T fc = (T)C_FAC_COND, ffus = (T)C_FAC_FUS;
    if (nprec > 1) {
      for (int e = TID; e < NH() * nzm; e += NT) {
        int i = 1 + e % NH(), k = 1 + e / NH();
        wp(i, k) = wp(i, k) / (T)(double)nprec;
      }
      SYNC;
    }
    for (int iprec = 1; iprec <= nprec; ++iprec) {
      for (int e = TID; e < NH() * nzm; e += NT) {
        int i = 1 + e % NH(), k = 1 + e / NH();
        int kc = min(nzm, k + 1), kb = max(1, k - 1);
        T q0 = qp(i, k), qb = qp(i, kb), qc = qp(i, kc);
        mx(i, k) = mx3(qb, qc, q0);
        mn(i, k) = mn3(qb, qc, q0);
        fz(i, k) = q0 * wp(i, k);
        if (k == 1) { fz(i, nz) = (T)0.; www(i, nz) = (T)0.; }
      }
      SYNC;
      for (int e = TID; e < NH() * nzm; e += NT) {
        int i = 1 + e % NH(), k = 1 + e / NH();
        tq(i, k) = qp(i, k) - (fz(i, k + 1) - fz(i, k)) * irhoadz[k];
      }
      SYNC;
      for (int e = TID; e < NH() * nzm; e += NT) {
        int i = 1 + e % NH(), k = 1 + e / NH();
        int kb = max(1, k - 1);
        www(i, k) = (T)0.5 * ((T)1. + wp(i, k) * irhoadz[k]) * (tq(i, kb) * wp(i, kb) - tq(i, k) * wp(i, k));
      }
      SYNC;
      for (int e = TID; e < NH() * nzm; e += NT) {
        int i = 1 + e % NH(), k = 1 + e / NH();
        int kc = min(nzm, k + 1), kb = max(1, k - 1);
        const T tb = tq(i, kb), tc = tq(i, kc), tk0 = tq(i, k), wc = www(i, kc), wk = www(i, k);
        T a = mx2(mx3(tb, tc, tk0), mx(i, k));
        T b = mn2(mn3(tb, tc, tk0), mn(i, k));
        const T mxv = rho[k] * adz[k] * (a - tk0) / (-mn2((T)0., wc) + mx2((T)0., wk) + eps);
        const T mnv = rho[k] * adz[k] * (tk0 - b) / (mx2((T)0., wc) + -mn2((T)0., wk) + eps);
        mx(i, k) = mxv;
        mn(i, k) = mnv;
      }
      SYNC;
      for (int e = TID; e < NH() * nzm; e += NT) {
        int i = 1 + e % NH(), k = 1 + e / NH();
        int kb = max(1, k - 1);
        T ww = www(i, k);
        fz(i, k) = fz(i, k) + mx2((T)0., ww) * mn3((T)1., mx(i, k), mn(i, kb)) - (-mn2((T)0., ww)) * mn3((T)1., mx(i, kb), mn(i, k));
      }
      SYNC;
      // per-level budget sums in the reference's order, then the update
      level_sums_lo(2, 1, nzm,
                 [&](int q, int i, int k) -> T {
                   if (q == 0) return -(fz(i, k + 1) - fz(i, k)) * irhoadz[k] * (T)1.;
                   return -(fz(i, k) * (T)1.);
                 },
                 [&](int q, int k) { return (double)(q == 0 ? qpfall[k] : precflux[k]); },
                 [&](int q, int k, double sv) { (q == 0 ? qpfall : precflux)[k] = (T)sv; });
      for (int e = TID; e < NH() * nzm; e += NT) {
        int i = 1 + e % NH(), k = 1 + e / NH();
        int kc = k + 1;
        T lf_c = (kc == nz) ? (T)0. : fc + ((T)1. - omega(i, kc)) * ffus;
        const T omk = omega(i, k), fzc = fz(i, kc), fzk = fz(i, k), ia = irhoadz[k];
        T lf_k = fc + ((T)1. - omk) * ffus;
        const T qpn = qp(i, k) - (fzc - fzk) * ia;
        T lat_heat = -(lf_c * fzc - lf_k * fzk) * ia;
        qp(i, k) = qpn;
        if constexpr (sizeof(T) == 8) t(i, k) = t(i, k) - lat_heat;
        else t(i, k) = add_carry(t(i, k), -lat_heat, rct()[e]);   // FP32-mixed form: carried
        if (k == 1) {
          PS(i) = PS(i) - fzk * (T)1.;
          PSS(i) = PSS(i) - fzk * ((T)1. - omk) * (T)1.;
        }
      }
      SYNC;
      if (iprec < nprec) {
        for (int e = TID; e < NH() * nzm; e += NT) {
          int i = 1 + e % NH(), k = 1 + e / NH();
          T tmp = term_vel(tabs(i, k), rho[k], qp(i, k));
          T wv = rhofac[k] * tmp;
          wp(i, k) = -wv * rhow[k] * dtn / dz / (T)(double)nprec;
        }
        SYNC;
      }
    }
  }

  // ---------------------------------------------------------- SGS scalar diffusion
  // SGS_TKE/diffuse_scalar.F90:33-72 + diffuse_scalar2D.F90:44-140
  __device__ void diffuse_scalar(FT f, T *fdiff, T *flux, T *rc = nullptr) {
    FT tkh = TKH(), flx = SA(), dfdt = SB(), f0 = SCR(p.L.s_c);
    T *rho = PR(P_RHO), *rhow = PR(P_RHOW), *adz = PR(P_ADZ), *adzw = PR(P_ADZW);
    T *grdfx = PR(P_GRDFX), *grdfz = PR(P_GRDFZ);
    const T dx = (T)p.dx, dz = (T)S.dz, dtn = (T)S.dtn;
    const T rdx2 = (T)1. / (dx * dx);
    for (int e = TID; e < (nx + 1) * nzm; e += NT) {
      int i = e % (nx + 1), k = 1 + e / (nx + 1);        // 0 .. nx
      T rdx5 = (T)0.5 * rdx2 * grdfx[k];
      int ic = i + 1;
      T tkx = rdx5 * (tkh(i, k) + tkh(ic, k));
      const T fc = f(ic, k), fi = f(i, k);
      flx(i, k) = -tkx * (fc - fi);
      if (fdiff && i >= 1) f0(i, k) = fi;
    }
    SYNC;
    for (int e = TID; e < nx * nzm; e += NT) {
      int i = 1 + e % nx, k = 1 + e / nx;
      dfdt(i, k) = (T)0. - (flx(i, k) - flx(i - 1, k));
    }
    SYNC;
    // vertical fluxes (flx reused, levels 0..nzm)
    for (int e = TID; e < nx * nzm; e += NT) {
      int i = 1 + e % nx, k = 1 + e / nx;
      if (k <= nzm - 1) {
        int kc = k + 1;
        T rhoi = PR(P_RHOWDADZW)[kc];
        T rdz2 = (T)1. / (dz * dz);
        T rdz5 = (T)0.5 * rdz2 * grdfz[k];
        T tkz = rdz5 * (tkh(i, k) + tkh(i, kc));
        flx(i, k) = -tkz * (f(i, kc) - f(i, k)) * rhoi;
      } else {
        T tmp = (T)1. / adzw[nz];
        T rdz = (T)1. / dz;
        flx(i, 0) = (T)0.0 * rdz * rhow[1];
        flx(i, nzm) = (T)0.0 * rdz * tmp * rhow[nz];
      }
    }
    SYNC;
    if (flux)
      level_sums_lo(1, 1, nzm, [&](int, int i, int k) -> T { return flx(i, k == 1 ? 0 : k - 1); },
                 [&](int, int) { return 0.; }, [&](int, int k, double sv) { flux[k] = (T)sv; });
    for (int e = TID; e < nx * nzm; e += NT) {
      int i = 1 + e % nx, k = 1 + e / nx;
      int kb = k - 1;
      T rhoi = PR(P_IRHOADZ)[k];
      T d = dtn * (dfdt(i, k) - (flx(i, k) - flx(i, kb)) * rhoi);
      if (sizeof(T) == 4 && rc) f(i, k) = add_carry(f(i, k), d, rc[e]);
      else f(i, k) = f(i, k) + d;
    }
    SYNC;
    if (fdiff) {
      level_sums_lo(1, 1, nzm, [&](int, int i, int k) -> T { return f(i, k) - f0(i, k); },
                 [&](int, int) { return 0.; }, [&](int, int k, double sv) { fdiff[k] = (T)sv; });
      SYNC;
    }
  }

  // ---------------------------------------------------------- SGS scalar diffusion, 3D
  // SGS_TKE/diffuse_scalar3D.F90:6-218 (fluxb = fluxt = 0, no walls) with
  // the sgs_scalars wrapper's fdiff; scratch planes: x and y fluxes in A, B,
  // the tendency in C, vertical fluxes in D (levels 0..nzm), the initial
  // field in E
  __device__ void diffuse_scalar3(FT f, T *fdiff, T *flux, T *rc = nullptr) {
    FT tkh = TKH(), flx = SA(), fly = SB(), dfdt = SCR(p.L.s_c), flz = SCR(p.L.s_d), f0 = SCR(p.L.s_e);
    T *rhow = PR(P_RHOW), *adzw = PR(P_ADZW);
    T *grdfx = PR(P_GRDFX), *grdfy = PR(P_GRDFY), *grdfz = PR(P_GRDFZ);
    const T dx = (T)p.dx, dy = (T)p.dy, dz = (T)S.dz, dtn = (T)S.dtn;
    const T rdx2 = (T)1. / (dx * dx), rdy2 = (T)1. / (dy * dy);
    const int nxy = nx * ny;
    for (int e = TID; e < (nx + 1) * (ny + 1) * nzm; e += NT) {
      const int i = e % (nx + 1), j = (e / (nx + 1)) % (ny + 1), k = 1 + e / ((nx + 1) * (ny + 1));
      const T fk = f(i, j, k);
      if (j >= 1) {
        const T rdx5 = (T)0.5 * rdx2 * grdfx[k];
        const T tkx = rdx5 * (tkh(i, j, k) + tkh(i + 1, j, k));
        flx(i, j, k) = -tkx * (f(i + 1, j, k) - fk);
      }
      if (i >= 1) {
        const T rdy5 = (T)0.5 * rdy2 * grdfy[k];
        const T tky = rdy5 * (tkh(i, j, k) + tkh(i, j + 1, k));
        fly(i, j, k) = -tky * (f(i, j + 1, k) - fk);
      }
      if (fdiff && i >= 1 && j >= 1) f0(i, j, k) = fk;
    }
    SYNC;
    for (int e = TID; e < nxy * nzm; e += NT) {
      const int i = 1 + e % nx, j = 1 + (e / nx) % ny, k = 1 + e / nxy;
      dfdt(i, j, k) = ((T)0. - (flx(i, j, k) - flx(i - 1, j, k))) - (fly(i, j, k) - fly(i, j - 1, k));
      if (k <= nzm - 1) {
        const int kc = k + 1;
        const T rhoi = PR(P_RHOWDADZW)[kc];
        const T rdz2 = (T)1. / (dz * dz);
        const T rdz5 = (T)0.5 * rdz2 * grdfz[k];
        const T tkz = rdz5 * (tkh(i, j, k) + tkh(i, j, kc));
        flz(i, j, k) = -tkz * (f(i, j, kc) - f(i, j, k)) * rhoi;
      } else {
        const T tmp = (T)1. / adzw[nz];
        const T rdz = (T)1. / dz;
        flz(i, j, 0) = (T)0.0 * rdz * rhow[1];
        flz(i, j, nzm) = (T)0.0 * rdz * tmp * rhow[nz];
      }
    }
    SYNC;
    if (flux)
      level_sums_lo(1, 1, nzm, [&](int, int h, int k) -> T { return flz(h, k == 1 ? 0 : k - 1); },
                    [&](int, int) { return 0.; }, [&](int, int k, double sv) { flux[k] = (T)sv; });
    for (int e = TID; e < nxy * nzm; e += NT) {
      const int i = 1 + e % nx, j = 1 + (e / nx) % ny, k = 1 + e / nxy;
      const T rhoi = PR(P_IRHOADZ)[k];
      const T d = dtn * (dfdt(i, j, k) - (flz(i, j, k) - flz(i, j, k - 1)) * rhoi);
      if (sizeof(T) == 4 && rc) f(i, j, k) = add_carry(f(i, j, k), d, rc[e]);
      else f(i, j, k) = f(i, j, k) + d;
    }
    SYNC;
    if (fdiff) {
      level_sums_lo(1, 1, nzm, [&](int, int h, int k) -> T { return f(h, k) - f0(h, k); },
                    [&](int, int) { return 0.; }, [&](int, int k, double sv) { fdiff[k] = (T)sv; });
      SYNC;
    }
  }

  // ---------------------------------------------------------- cloud
  // MICRO_SAM1MOM/cloud.F90:26-111: saturation adjustment, Newton in FP64
  __device__ void cloud() {
    FT qt = QT(), qp = QP(), qn = QN(), tabs = TABS(), t = TT();
    T *gamaz = PR(P_GAMAZ), *pres = PR(P_PRES);
    const double an = 1. / (C_TBGMAX - C_TBGMIN), bn = C_TBGMIN * an;
    const double ap = 1. / (C_TPRMAX - C_TPRMIN), bp = C_TPRMIN * ap;
    const double fac1 = C_FAC_COND + (1 + bp) * C_FAC_FUS;
    const double fac2 = C_FAC_FUS * ap;
    for (int e = TID; e < NH() * nzm; e += NT) {
      int i = 1 + e % NH(), k = 1 + e / NH();
      if constexpr (sizeof(T) == 4) {
        // FP32-mixed form: a cell that is clearly unsaturated (total water
        // 0.1 % or more below saturation, far beyond FP32 rounding of qsat)
        // takes the no-condensate branch in FP32; the FP64 path, with the
        // Newton iteration, runs only near or above saturation.
        const float qf = mx2(0.f, (float)qt(i, k)), qpf = (float)qp(i, k);
        const float tabf = (float)(t(i, k) - gamaz[k]), prf = (float)pres[k];
        float t1 = (tabf + (float)fac1 * qpf) / (1.f + (float)fac2 * qpf);
        float qsf;
        if (t1 >= (float)C_TBGMAX) {
          t1 = tabf + (float)C_FAC_COND * qpf;
          qsf = qsatw(t1, prf);
        } else if (t1 <= (float)C_TBGMIN) {
          t1 = tabf + (float)C_FAC_SUB * qpf;
          qsf = qsati(t1, prf);
        } else {
          float om = (float)an * t1 - (float)bn;
          qsf = om * qsatw(t1, prf) + (1.f - om) * qsati(t1, prf);
        }
        if (qf < 0.999f * qsf) {
          qt(i, k) = (T)qf;
          qn(i, k) = (T)0.;
          tabs(i, k) = (T)t1;
          qp(i, k) = mx2((T)0., qp(i, k));
          continue;
        }
      }
      double pr = (double)pres[k];
      double q = mx2(0., (double)qt(i, k));
      double qpv = (double)qp(i, k);
      double tab = (double)(t(i, k) - gamaz[k]);
      double tabs1 = (tab + fac1 * qpv) / (1. + fac2 * qpv);
      double qsatt;
      if (tabs1 >= C_TBGMAX) {
        tabs1 = tab + C_FAC_COND * qpv;
        qsatt = qsatw(tabs1, pr);
      } else if (tabs1 <= C_TBGMIN) {
        tabs1 = tab + C_FAC_SUB * qpv;
        qsatt = qsati(tabs1, pr);
      } else {
        double om = an * tabs1 - bn;
        qsatt = om * qsatw(tabs1, pr) + (1. - om) * qsati(tabs1, pr);
      }
      double qnv;
      if (q > qsatt) {
        int niter = 0;
        double dtabs = 100.;
        double dqsat = 0.;
        while (fabs(dtabs) > R4(0.01) && niter < 10) {
          double lstarn, dlstarn, lstarp, dlstarp;
          if (tabs1 >= C_TBGMAX) {
            lstarn = C_FAC_COND; dlstarn = 0.;
            qsatt = qsatw(tabs1, pr); dqsat = dtqsatw(tabs1, pr);
          } else if (tabs1 <= C_TBGMIN) {
            lstarn = C_FAC_SUB; dlstarn = 0.;
            qsatt = qsati(tabs1, pr); dqsat = dtqsati(tabs1, pr);
          } else {
            double om = an * tabs1 - bn;
            lstarn = C_FAC_COND + (1. - om) * C_FAC_FUS;
            dlstarn = an * C_FAC_FUS;
            qsatt = om * qsatw(tabs1, pr) + (1. - om) * qsati(tabs1, pr);
            dqsat = om * dtqsatw(tabs1, pr) + (1. - om) * dtqsati(tabs1, pr);
          }
          if (tabs1 >= C_TPRMAX) { lstarp = C_FAC_COND; dlstarp = 0.; }
          else if (tabs1 <= C_TPRMIN) { lstarp = C_FAC_SUB; dlstarp = 0.; }
          else {
            double omp = ap * tabs1 - bp;
            lstarp = C_FAC_COND + (1. - omp) * C_FAC_FUS;
            dlstarp = ap * C_FAC_FUS;
          }
          double fff = tab - tabs1 + lstarn * (q - qsatt) + lstarp * qpv;
          double dfff = dlstarn * (q - qsatt) + dlstarp * qpv - lstarn * dqsat - 1.;
          dtabs = -fff / dfff;
          niter = niter + 1;
          tabs1 = tabs1 + dtabs;
        }
        qsatt = qsatt + dqsat * dtabs;
        qnv = mx2(0., q - qsatt);
      } else {
        qnv = 0.;
      }
      qt(i, k) = (T)q;
      qn(i, k) = (T)qnv;
      tabs(i, k) = (T)tabs1;
      qp(i, k) = mx2((T)0., qp(i, k));
    }
    SYNC;
  }

  // ---------------------------------------------------------- precip_proc
  // MICRO_SAM1MOM/precip_proc.F90:40-148; qpsrc/qpevp summed per level in
  // the reference's order from the per-cell contributions
  __device__ void precip_proc() {
    FT qt = QT(), qp = QP(), qn = QN(), tabs = TABS();
    FT csrc = SA(), cevp = SB();
    T *pres = PR(P_PRES);
    const T powr1 = (T)((3 + C_B_RAIN) / 4.), powr2 = (T)((5 + C_B_RAIN) / 8.);
    const T pows1 = (T)((3 + C_B_SNOW) / 4.), pows2 = (T)((5 + C_B_SNOW) / 8.);
    const T powg1 = (T)((3 + C_B_GRAU) / 4.), powg2 = (T)((5 + C_B_GRAU) / 8.);
    const T dtn = (T)S.dtn;
    const T a_bg = (T)p.a_bg, a_pr = (T)p.a_pr, a_gr = (T)p.a_gr;
    for (int e = TID; e < NH() * nzm; e += NT) {
      int i = 1 + e % NH(), k = 1 + e / NH();
      T q = qt(i, k), qpv = qp(i, k), qnv = qn(i, k), tb = tabs(i, k);
      T src = (T)0., evp = (T)0.;
      if (qnv + qpv > (T)0.) {
        T omn = mx2((T)0., mn2((T)1., (tb - (T)C_TBGMIN) * a_bg));
        T omp = mx2((T)0., mn2((T)1., (tb - (T)C_TPRMIN) * a_pr));
        T omg = mx2((T)0., mn2((T)1., (tb - (T)C_TGRMIN) * a_gr));
        if (qnv > (T)0.) {
          T qcc = qnv * omn;
          T qii = qnv * ((T)1. - omn);
          T autor = (qcc > (T)C_QCW0) ? (T)C_ALPHAELQ : (T)0.;
          T autos = (qii > (T)C_QCI0) ? (T)C_BETAELQ * PR(P_COEFICE)[k] : (T)0.;
          T accrr = (T)0.;
          if (omp > (T)R4(0.001)) {
            T qrr = qpv * omp;
            accrr = PR(P_ACCRRC)[k] * tpow(qrr, powr1);
          }
          T accrcs = (T)0., accris = (T)0.;
          if (omp < (T)R4(0.999) && omg < (T)R4(0.999)) {
            T qss = qpv * ((T)1. - omp) * ((T)1. - omg);
            T tmp = tpow(qss, pows1);
            accrcs = PR(P_ACCRSC)[k] * tmp;
            accris = PR(P_ACCRSI)[k] * tmp;
          }
          T accrcg = (T)0., accrig = (T)0.;
          if (omp < (T)R4(0.999) && omg > (T)R4(0.001)) {
            T qgg = qpv * ((T)1. - omp) * omg;
            T tmp = tpow(qgg, powg1);
            accrcg = PR(P_ACCRGC)[k] * tmp;
            accrig = PR(P_ACCRGI)[k] * tmp;
          }
          qcc = (qcc + dtn * autor * (T)C_QCW0) / ((T)1. + dtn * (accrr + accrcs + accrcg + autor));
          qii = (qii + dtn * autos * (T)C_QCI0) / ((T)1. + dtn * (accris + accrig + autos));
          T dq = dtn * (accrr * qcc + autor * (qcc - (T)C_QCW0) + (accris + accrig) * qii +
                        (accrcs + accrcg) * qcc + autos * (qii - (T)C_QCI0));
          dq = mn2(dq, qnv);
          qpv = qpv + dq;
          q = q - dq;
          qnv = qnv - dq;
          src = dq;
        } else if (qpv > (T)C_QP_THRESHOLD && qnv == (T)0.) {
          T qsatt = (T)0.;
          if (omn > (T)R4(0.001)) qsatt = qsatt + omn * qsatw(tb, pres[k]);
          if (omn < (T)R4(0.999)) qsatt = qsatt + ((T)1. - omn) * qsati(tb, pres[k]);
          T dq = (T)0.;
          if (omp > (T)R4(0.001)) {
            T qrr = qpv * omp;
            dq = dq + PR(P_EVAPR1)[k] * tsqrt(qrr) + PR(P_EVAPR2)[k] * tpow(qrr, powr2);
          }
          if (omp < (T)R4(0.999) && omg < (T)R4(0.999)) {
            T qss = qpv * ((T)1. - omp) * ((T)1. - omg);
            dq = dq + PR(P_EVAPS1)[k] * tsqrt(qss) + PR(P_EVAPS2)[k] * tpow(qss, pows2);
          }
          if (omp < (T)R4(0.999) && omg > (T)R4(0.001)) {
            T qgg = qpv * ((T)1. - omp) * omg;
            dq = dq + PR(P_EVAPG1)[k] * tsqrt(qgg) + PR(P_EVAPG2)[k] * tpow(qgg, powg2);
          }
          dq = dq * dtn * (q / qsatt - (T)1.);
          dq = mx2((T)-0.5 * qpv, dq);
          qpv = qpv + dq;
          q = q - dq;
          evp = dq;
        } else {
          q = q + qpv;
          evp = -qpv;                   // qpevp = qpevp - qp
          qpv = (T)0.;
        }
      }
      T dq = qpv;
      qpv = mx2((T)0., qpv);
      q = q + (dq - qpv);
      qt(i, k) = q; qp(i, k) = qpv; qn(i, k) = qnv;
      csrc(i, k) = src; cevp(i, k) = evp;
    }
    SYNC;
    T *qpsrc = PR(P_QPSRC), *qpevp = PR(P_QPEVP);
    level_sums_lo(2, 1, nzm, [&](int q, int i, int k) -> T { return q == 0 ? csrc(i, k) : cevp(i, k); },
               [&](int, int) { return 0.; },
               [&](int q, int k, double sv) { (q == 0 ? qpsrc : qpevp)[k] = (T)sv; });
    SYNC;
  }

  // ---------------------------------------------------------- diagnose
  // ---------------------------------------------------------- acceleration
  // Mean-state acceleration, accelerate_crm.F90:109-366 (per column): the
  // horizontal-mean change of t and qt (u, v) since the last diagnose is
  // applied accel_factor more times; a |dT| above 5 K stops acceleration for
  // the rest of the call and stretches nstop so the call still spans dt_gl.
  __device__ void accelerate(int nstep) {
    FT t = TT(), qt = QT(), qv = QV(), qcl = QCL(), qci = QCI(), u = U(), v = V();
    double *ta = reinterpret_cast<double *>(base + p.L.s_c);   // 4 x (nz + 2) FP64
    auto TA = [&](int q, int k) -> double & { return ta[(size_t)q * (nz + 2) + k]; };
    const double coef = 1.0 / (double)NH();
    const int nq = p.accel_uv ? 4 : 2;
    if (TID == 0) S.acc_flag = 0;
    SYNC;
    T *t0 = PR(P_T0), *q0 = PR(P_Q0), *u0 = PR(P_U0), *v0 = PR(P_V0);
    level_sums(nq, 1, nzm,
               [&](int q, int i, int k) -> T {
                 switch (q) {
                   case 0: return t(i, k) * (T)coef;
                   case 1: return (qcl(i, k) + qci(i, k) + qv(i, k)) * (T)coef;
                   case 2: return u(i, k) * (T)coef;
                   default: return v(i, k) * (T)coef;
                 }
               },
               [&](int, int) { return 0.; },
               [&](int q, int k, double sv) {
                 const T *m = q == 0 ? t0 : q == 1 ? q0 : q == 2 ? u0 : v0;
                 double d = sv - (double)m[k];
                 TA(q, k) = d;
                 if (q == 0 && fabs(d) > 5.) S.acc_flag = 1;
               });
    SYNC;
    const bool cease = batch_max(S.acc_flag ? 1.0 : 0.0) > 0.0;   // one flag per batch
    if (cease) {
      if (TID == 0) {
        S.ceaseflag = 1;
        S.nstop = (int)((double)S.nstop + (double)(S.nstop - nstep + 1) * p.accel_factor);
      }
      SYNC;
      return;
    }
    const T f = (T)p.accel_factor, tmin = (T)50.;
    for (int e = TID; e < NH() * nzm; e += NT) {
      int i = 1 + e % NH(), k = 1 + e / NH();
      t(i, k) = mx2(tmin, t(i, k) + f * (T)TA(0, k));
      if (p.accel_uv) {
        u(i, k) = u(i, k) + f * (T)TA(2, k);
        v(i, k) = v(i, k) + f * (T)TA(3, k);
      }
      qt(i, k) = qt(i, k) + f * (T)TA(1, k);
    }
    SYNC;
    // clip negative qt per level, rescaling the positive cells (FP64 sums)
    level_sums(2, 1, nzm,
               [&](int q, int i, int k) -> T {
                 T x = qt(i, k);
                 bool neg = x < (T)0.;
                 return q == 0 ? (neg ? x : (T)0.) : (neg ? (T)0. : x);
               },
               [&](int, int) { return 0.; }, [&](int q, int k, double sv) { TA(q, k) = sv; });
    SYNC;
    for (int e = TID; e < NH() * nzm; e += NT) {
      int i = 1 + e % NH(), k = 1 + e / NH();
      const double qneg = TA(0, k), qpoz = TA(1, k);
      if (qpoz + qneg <= 0.) {
        qt(i, k) = (T)0.; qv(i, k) = (T)0.; qcl(i, k) = (T)0.; qci(i, k) = (T)0.;
      } else {
        double factor = 1. + qneg / qpoz;
        T q = (T)mx2(0., (double)qt(i, k) * factor);
        qt(i, k) = q;
        if (q <= (T)0.) {
          qv(i, k) = (T)0.; qcl(i, k) = (T)0.; qci(i, k) = (T)0.;
        } else {
          T qt_res = q - qcl(i, k) - qci(i, k);
          qv(i, k) = mx2((T)0., qt_res);
          if (qt_res < (T)0.) {
            T fr = (T)1. + qt_res / (qcl(i, k) + qci(i, k));
            qcl(i, k) = qcl(i, k) * fr;
            qci(i, k) = qci(i, k) * fr;
          }
        }
      }
    }
    SYNC;
  }

  __device__ void diagnose() {                 // diagnose.F90:21-85
    FT t = TT(), tabs = TABS(), qcl = QCL(), qci = QCI(), qpl = QPL(), qpi = QPI(), qv = QV(), u = U(), v = V();
    T *gamaz = PR(P_GAMAZ);
    if constexpr (sizeof(T) == 4) {
      // FP32-mixed form: one pass, a warp per level: each lane forms tabs of
      // its cells (the same expression as below) and adds them to the level
      // sums, and the lane that writes the level's means forms qv0 from the
      // FP64 means of total and condensed water right after them
      const double coef = 1. / (double)NH();
      double q0k = 0.;
      level_sums_lo_multi<7>(1, nzm,
                 [&](int, int, int) -> T { return (T)0.; },   // (FP64 form: not used)
                 [&](int i, int k, T *r) {
                   const T ql = qcl(i, k), qi = qci(i, k);
                   const T tb = t(i, k) - gamaz[k] + (T)C_FAC_COND * (ql + qpl(i, k)) + (T)C_FAC_SUB * (qi + qpi(i, k));
                   tabs(i, k) = tb;
                   const T c = ql + qi;
                   r[0] = u(i, k); r[1] = v(i, k); r[2] = t(i, k); r[3] = tb;
                   r[4] = qv(i, k) + ql + qi; r[5] = c; r[6] = qpl(i, k) + qpi(i, k);
                 },
                 [&](int, int) { return 0.; },
                 [&](int q, int k, double sv) {
                   sv = sv * coef;
                   const int ids[7] = {P_U0, P_V0, P_T0, P_TABS0, P_Q0, P_QN0, P_QP0};
                   PR(ids[q])[k] = (T)sv;
                   if (q == 4) q0k = sv;
                   if (q == 5) PR(P_QV0)[k] = (T)(q0k - sv);
                 });
      SYNC;
    } else {
      diagnose_plain(t, tabs, qcl, qci, qpl, qpi, qv, u, v, gamaz);
    }
  }
  // the FP64 form: tabs, then the means with one thread per (quantity,
  // level) in the reference's order (level_sums_lo_multi), then qv0
  __device__ void diagnose_plain(FT t, FT tabs, FT qcl, FT qci, FT qpl, FT qpi, FT qv, FT u, FT v, T *gamaz) {
    for (int e = TID; e < NH() * nzm; e += NT) {
      int i = 1 + e % NH(), k = 1 + e / NH();
      tabs(i, k) = t(i, k) - gamaz[k] + (T)C_FAC_COND * (qcl(i, k) + qpl(i, k)) + (T)C_FAC_SUB * (qci(i, k) + qpi(i, k));
    }
    SYNC;
    const double coef = 1. / (double)NH();
    // domain means; q0 and qn0 are kept in FP64 in TMP0/TMP1 for qv0
    double *q0d = reinterpret_cast<double *>(sa());
    level_sums_lo_multi<7>(1, nzm,
               [&](int q, int i, int k) -> T {
                 switch (q) {
                   case 0: return u(i, k);
                   case 1: return v(i, k);
                   case 2: return t(i, k);
                   case 3: return tabs(i, k);
                   case 4: return qv(i, k) + qcl(i, k) + qci(i, k);
                   case 5: return qcl(i, k) + qci(i, k);
                   default: return qpl(i, k) + qpi(i, k);
                 }
               },
               [&](int i, int k, T *r) {
                 const T c = qcl(i, k) + qci(i, k);
                 r[0] = u(i, k); r[1] = v(i, k); r[2] = t(i, k); r[3] = tabs(i, k);
                 r[4] = qv(i, k) + qcl(i, k) + qci(i, k); r[5] = c; r[6] = qpl(i, k) + qpi(i, k);
               },
               [&](int, int) { return 0.; },
               [&](int q, int k, double sv) {
                 sv = sv * coef;
                 const int ids[7] = {P_U0, P_V0, P_T0, P_TABS0, P_Q0, P_QN0, P_QP0};
                 PR(ids[q])[k] = (T)sv;
                 if (q == 4) q0d[k] = sv;
                 if (q == 5) q0d[nz + 1 + k] = sv;
               });
    SYNC;
    for (int k = TID + 1; k <= nzm; k += NT) PR(P_QV0)[k] = (T)(q0d[k] - q0d[nz + 1 + k]);
    SYNC;
  }

  // ---------------------------------------------------------- step statistics
  // crm_module.F90:896-1073, accumulated every CRM step
  __device__ void step_stats() {
    FT qcl = QCL(), qci = QCI(), qpl = QPL(), qpi = QPI(), w = W(), tabs = TABS(), qv = QV();
    T *rho = PR(P_RHO), *adz = PR(P_ADZ), *pres = PR(P_PRES), *rhow = PR(P_RHOW);
    T *cs = base + p.L.colstat;     // 5 x NH(): cwp, cwph, cwpm, cwpl, top level
    const T dz = (T)S.dz;
    const T thr = (T)R4(0.001);
    // condensate paths from the top down, per CRM column (i)
    for (int i = TID + 1; i <= NH(); i += NT) {
      T cwp = (T)0., cwph = (T)0., cwpm = (T)0., cwpl = (T)0.;
      int top = 0;
      for (int k = 1; k <= nzm; ++k) {
        int kk = nz - k;
        T tmp1 = rho[kk] * adz[kk] * dz * (qcl(i, kk) + qci(i, kk));
        cwp = cwp + tmp1;
        if (cwp > thr && top == 0) top = k;
        if (pres[kk] >= (T)700.) cwpl = cwpl + tmp1;
        else if (pres[kk] < (T)400.) cwph = cwph + tmp1;
        else cwpm = cwpm + tmp1;
      }
      cs[(i - 1)] = cwp; cs[NH() + (i - 1)] = cwph; cs[2 * NH() + (i - 1)] = cwpm; cs[3 * NH() + (i - 1)] = cwpl;
      cs[4 * NH() + (i - 1)] = (T)top;
    }
    // cloudy mass flux of a cell at w level k (Xu et al. 2002): qsat > 0, so
    // a cell without condensate never passes the threshold and qsatw is
    // evaluated only where condensate exists (same result)
    auto mass_flux = [&](int i, int k, T &cu, T &cd) {
      const T wv = w(i, k);
      cu = (T)0.; cd = (T)0.;
      if (wv > (T)0.) {
        int kx = max(1, k - 1);
        T cond = qcl(i, kx) + qci(i, kx);
        if (cond > (T)0. && cond > mn2((T)R4(1.e-5), (T)R4(0.01) * qsatw(tabs(i, kx), pres[kx]))) cu = rhow[k] * wv;
      } else if (wv < (T)0.) {
        int kx = min(k + 1, nzm);
        T cond = qcl(i, kx) + qci(i, kx);
        if (cond > (T)0. && cond > mn2((T)R4(1.e-5), (T)R4(0.01) * qsatw(tabs(i, kx), pres[kx]))) cd = rhow[k] * wv;
        else if (qpl(i, kx) + qpi(i, kx) > (T)R4(1.0e-4)) cd = rhow[k] * wv;
      }
    };
    T *mui = OP(O_MUI), *mdi = OP(O_MDI);
    T *acc[8] = {OP(O_CLD), OP(O_CLDTOP), OP(O_MCUP), OP(O_MCDN), OP(O_MCUUP), OP(O_MCUDN), OP(O_GLIQWP), OP(O_GICEWP)};
    const int nxr = NR();
    T *rad = base + p.L.rad;
    if (sizeof(T) == 4 && nxr == NH()) {
      // FP32-mixed form, one radiation column per CRM column: the level
      // statistics, the mass fluxes at w levels 1..nzm and the radiation
      // sums in one pass (a warp per level, each cell visited once); the same
      // terms and FP32 warp reductions as the separate passes below
      SYNC;                                     // cloud tops (cs) complete
      const size_t pl = (size_t)NH() * nzm;
      level_sums_lo_multi<10>(1, nzm,
                 [&](int, int, int) -> T { return (T)0.; },   // (FP64 form: not used)
                 [&](int i, int k, T *r) {
                   const T ql = qcl(i, k), qi = qci(i, k);
                   const bool cloudy = rho[k] * adz[k] * dz * (ql + qi) > thr;
                   const T ws = w(i, k + 1) + w(i, k), m = rho[k] * (T)0.5 * ws;
                   r[0] = cloudy ? (T)1.0 : (T)0.;
                   r[1] = ((int)cs[4 * NH() + (i - 1)] == k) ? (T)1. : (T)0.;
                   r[2] = (cloudy && ws > (T)4.) ? m : (T)0.;
                   r[3] = (cloudy && ws < (T)-4.) ? m : (T)0.;
                   r[4] = (!cloudy && ws > (T)4.) ? m : (T)0.;
                   r[5] = (!cloudy && ws < (T)-4.) ? m : (T)0.;
                   r[6] = ql;
                   r[7] = qi;
                   mass_flux(i, k, r[8], r[9]);
                   const size_t o = (size_t)(k - 1) * NH() + (i - 1);
                   const T st = rad[o] + tabs(i, k), sq = rad[pl + o] + mx2((T)0., qv(i, k));
                   const T sc = rad[2 * pl + o] + ql, si = rad[3 * pl + o] + qi;
                   const T sl = (ql + qi > (T)0) ? rad[4 * pl + o] + (T)1.0 : rad[4 * pl + o];
                   rad[o] = st; rad[pl + o] = sq; rad[2 * pl + o] = sc; rad[3 * pl + o] = si; rad[4 * pl + o] = sl;
                 },
                 [&](int q, int k) {
                   return (double)(q < 8 ? acc[q][plev - k + 1] : (q == 8 ? mui : mdi)[plev + 2 - k]);
                 },
                 [&](int q, int k, double sv) {
                   (q < 8 ? acc[q][plev - k + 1] : (q == 8 ? mui : mdi)[plev + 2 - k]) = (T)sv;
                 });
      // w level nz (the rigid lid) for the mass fluxes
      level_sums_lo(2, nz, nz,
                 [&](int q, int i, int k) -> T { T cu, cd; mass_flux(i, k, cu, cd); return q == 0 ? cu : cd; },
                 [&](int q, int k) { return (double)(q == 0 ? mui : mdi)[plev + 2 - k]; },
                 [&](int q, int k, double sv) { (q == 0 ? mui : mdi)[plev + 2 - k] = (T)sv; });
      SYNC;
    } else {
      // interface mass fluxes (Xu et al. 2002): per-cell contributions at w
      // levels k = 1..nz, zero where a cell does not count
      FT cmu = SA(), cmd = SB();
      for (int e = TID; e < NH() * nz; e += NT) {
        int i = 1 + e % NH(), k = 1 + e / NH();
        T cu, cd;
        mass_flux(i, k, cu, cd);
        cmu(i, k) = cu;
        cmd(i, k) = cd;
      }
      SYNC;
      level_sums_lo(2, 1, nz, [&](int q, int i, int k) -> T { return q == 0 ? cmu(i, k) : cmd(i, k); },
                 [&](int q, int k) { return (double)(q == 0 ? mui : mdi)[plev + 2 - k]; },
                 [&](int q, int k, double sv) { (q == 0 ? mui : mdi)[plev + 2 - k] = (T)sv; });
      // cloud fraction, cloud top counts, cloudy mass fluxes, water paths
      level_sums_lo_multi<8>(1, nzm,
                 [&](int q, int i, int k) -> T {
                   if (q == 1) return ((int)cs[4 * NH() + (i - 1)] == k) ? (T)1. : (T)0.;
                   if (q == 6) return qcl(i, k);
                   if (q == 7) return qci(i, k);
                   T tmp1 = rho[k] * adz[k] * dz;
                   bool cloudy = tmp1 * (qcl(i, k) + qci(i, k)) > thr;
                   if (q == 0) return cloudy ? (T)1.0 : (T)0.;
                   T ws = w(i, k + 1) + w(i, k);
                   if (q == 2) return (cloudy && ws > (T)4.) ? rho[k] * (T)0.5 * ws * (T)1.0 : (T)0.;
                   if (q == 3) return (cloudy && ws < (T)-4.) ? rho[k] * (T)0.5 * ws * (T)1.0 : (T)0.;
                   if (q == 4) return (!cloudy && ws > (T)4.) ? rho[k] * (T)0.5 * ws : (T)0.;
                   return (!cloudy && ws < (T)-4.) ? rho[k] * (T)0.5 * ws : (T)0.;
                 },
                 [&](int i, int k, T *r) {
                   const T ql = qcl(i, k), qi = qci(i, k);
                   const bool cloudy = rho[k] * adz[k] * dz * (ql + qi) > thr;
                   const T ws = w(i, k + 1) + w(i, k), m = rho[k] * (T)0.5 * ws;
                   r[0] = cloudy ? (T)1.0 : (T)0.;
                   r[1] = ((int)cs[4 * NH() + (i - 1)] == k) ? (T)1. : (T)0.;
                   r[2] = (cloudy && ws > (T)4.) ? m : (T)0.;
                   r[3] = (cloudy && ws < (T)-4.) ? m : (T)0.;
                   r[4] = (!cloudy && ws > (T)4.) ? m : (T)0.;
                   r[5] = (!cloudy && ws < (T)-4.) ? m : (T)0.;
                   r[6] = ql;
                   r[7] = qi;
                 },
                 [&](int q, int k) { return (double)acc[q][plev - k + 1]; },
                 [&](int q, int k, double sv) { acc[q][plev - k + 1] = (T)sv; });
      // radiation-group sums (crm_module.F90:1000-1028)
      const int gx = NH() / nxr;
      for (int e = TID; e < nxr * nzm; e += NT) {
        int ir = 1 + e % nxr, k = 1 + e / nxr;
        size_t o = (size_t)(k - 1) * nxr + (ir - 1);
        T st = rad[o], sq = rad[(size_t)nxr * nzm + o], sc = rad[(size_t)2 * nxr * nzm + o];
        T si = rad[(size_t)3 * nxr * nzm + o], sl = rad[(size_t)4 * nxr * nzm + o];
        for (int i = (ir - 1) * gx + 1; i <= ir * gx; ++i) {
          st = st + tabs(i, k);
          sq = sq + mx2((T)0., qv(i, k));
          sc = sc + qcl(i, k);
          si = si + qci(i, k);
          if (qcl(i, k) + qci(i, k) > (T)0) sl = sl + (T)1.0;
        }
        rad[o] = (T)st; rad[(size_t)nxr * nzm + o] = (T)sq; rad[(size_t)2 * nxr * nzm + o] = (T)sc;
        rad[(size_t)3 * nxr * nzm + o] = (T)si; rad[(size_t)4 * nxr * nzm + o] = (T)sl;
      }
      SYNC;
    }
    if (TID < 32) {
      // shaded cloud fractions (counts, exact in any order): cf3d = 1, so a
      // column counts wherever its layer class exists (crm_module.F90:1053-1072)
      bool anyl = false, anyh = false, anym = false;
      for (int k = 1; k <= nzm; ++k) {
        if (pres[k] >= (T)700.) anyl = true;
        else if (pres[k] < (T)400.) anyh = true;
        else anym = true;
      }
      int ct = 0, ch = 0, cm = 0, cl = 0;
      for (int i = 1 + TID; i <= NH(); i += 32) {
        ct += cs[(i - 1)] > thr;
        ch += cs[NH() + (i - 1)] > thr;
        cm += cs[2 * NH() + (i - 1)] > thr;
        cl += cs[3 * NH() + (i - 1)] > thr;
      }
      for (int o = 16; o > 0; o >>= 1) {
        ct += __shfl_xor_sync(0xffffffffu, ct, o);
        ch += __shfl_xor_sync(0xffffffffu, ch, o);
        cm += __shfl_xor_sync(0xffffffffu, cm, o);
        cl += __shfl_xor_sync(0xffffffffu, cl, o);
      }
      if (TID == 0) {
        S.cltot = S.cltot + (double)ct;
        S.clhgh = S.clhgh + (anyh ? (double)ch : 0.0);
        S.clmed = S.clmed + (anym ? (double)cm : 0.0);
        S.cllow = S.cllow + (anyl ? (double)cl : 0.0);
      }
    }
    SYNC;
  }

  // ---------------------------------------------------------- finalize
  // crm_module.F90:1086-1594
  __device__ void finalize() {
    const int ld = p.ld;
    const double factor_xy = 1.0 / (double)NH();
    const double icrm_run_time = 1.0 / p.dt_gl;
    const double factor_xyt = factor_xy / (double)S.nstop;
    const int ptop = plev - nzm + 1;
    auto O1 = [&](int f) -> double & { return p.out[f][icrm]; };
    auto O2 = [&](int f, int l) -> double & { return p.out[f][(size_t)icrm + (size_t)ld * (l - 1)]; };
    // zero every GCM-level output of this column first
    for (int e = TID; e < (CRM_NOUT - CRM_OUT_FIRST_2D) * plev; e += NT) {
      int f = CRM_OUT_FIRST_2D + e / plev, l = 1 + e % plev;
      O2(f, l) = 0.;
    }
    FT tabs = TABS(), qv = QV(), qcl = QCL(), qci = QCI(), qpl = QPL(), qpi = QPI(), u = U(), v = V(), w = W();
    FT qt = QT(), qp = QP(), qn = QN(), tk = TK(), tkh = TKH(), tke = TKE();
    // radiation means
    {
      const int nxr = NR();
      // crm_nx_rad_fac * crm_ny_rad_fac / nstop (crm_module.F90:1080-1083)
      double tmp1 = ((double)p.L.nx_rad / (double)nx) * ((double)p.L.ny_rad / (double)ny) / (double)S.nstop;
      T *rad = base + p.L.rad;
      for (int e = TID; e < nxr * nzm; e += NT) {
        int ir = 1 + e % nxr, k = 1 + e / nxr;
        size_t o = (size_t)icrm + (size_t)ld * ((ir - 1) + (size_t)nxr * (k - 1));
        size_t s = (size_t)(k - 1) * nxr + (ir - 1);
        for (int f = 0; f < 5; ++f) p.radout[f][o] = (double)rad[(size_t)f * nxr * nzm + s] * tmp1;
      }
    }
    SYNC;
    // horizontal sums of the final state per CRM level (FP64 scratch)
    double *hs = reinterpret_cast<double *>(sa());    // 14 x (nz + 2)
    auto HS = [&](int q, int k) -> double & { return hs[(size_t)q * (nz + 2) + k]; };
    {
      T *u0p = PR(P_U0), *v0p = PR(P_V0);
      // 3D: tln, qln, qccln, qiiln sum i outer, j inner; the condensate
      // means (12, 13: qcl, qci) j outer like every other sum
      level_sums(Y3 ? 14 : 12, 1, nzm,
                 [&](int q, int i, int k) -> T {
                   if (q < 4) i = h_ij(i);
                   switch (q) {
                     case 0: return tabs(i, k);
                     case 1: return qv(i, k);
                     case 2: return qcl(i, k);
                     case 3: return qci(i, k);
                     case 4: return qpl(i, k);
                     case 5: {
                       T omg = mx2((T)0., mn2((T)1., (tabs(i, k) - (T)C_TGRMIN) * (T)p.a_gr));
                       return qpi(i, k) * omg;
                     }
                     case 6: {
                       T omg = mx2((T)0., mn2((T)1., (tabs(i, k) - (T)C_TGRMIN) * (T)p.a_gr));
                       return qpi(i, k) * ((T)1. - omg);
                     }
                     case 7: { T d = u(i, k) - u0p[k]; return d * d; }
                     case 8: { T d = v(i, k) - v0p[k]; return d * d; }
                     case 9: { T w1 = w(i, k + 1), w0 = w(i, k); return (T)0.5 * (w1 * w1 + w0 * w0); }
                     case 10: return tke(i, k);
                     case 11: return tk(i, k);
                     case 12: return qcl(i, k);
                     default: return qci(i, k);
                   }
                 },
                 [&](int, int) { return 0.; }, [&](int q, int k, double sv) { HS(q, k) = sv; });
    }
    SYNC;
    // FP32-mixed form: the means of tabs and qv behind sltend and qltend (and
    // the state's temperature and qt) from t and qt with their carried
    // residues, diagnosed in FP64.  FP32 tabs and qv are rounded to within
    // half a unit in the last place, which in a layer where nothing happens is
    // the same bias in every cell and does not average out.
    auto tabs_d = [&](int i, int k) -> double {
      const size_t e = (size_t)(i - 1) + (size_t)NH() * (k - 1);
      return ((double)TT()(i, k) + (double)rct()[e]) - (double)PR(P_GAMAZ)[k] +
             C_FAC_COND * ((double)qcl(i, k) + (double)qpl(i, k)) + C_FAC_SUB * ((double)qci(i, k) + (double)qpi(i, k));
    };
    auto qt_d = [&](int i, int k) -> double {
      return (double)qt(i, k) + (double)rcq()[(size_t)(i - 1) + (size_t)NH() * (k - 1)];
    };
    if constexpr (sizeof(T) == 4) {
      const int lane = TID & 31, warp = TID >> 5, nw = NT >> 5;
      for (int k = 1 + warp; k <= nzm; k += nw) {
        double st = 0., sq = 0.;
        for (int i = 1 + lane; i <= NH(); i += 32) {
          st = st + tabs_d(i, k);
          sq = sq + (qt_d(i, k) - (double)qn(i, k));
        }
        for (int o = 16; o > 0; o >>= 1) {
          st = st + __shfl_xor_sync(0xffffffffu, st, o);
          sq = sq + __shfl_xor_sync(0xffffffffu, sq, o);
        }
        if (lane == 0) { HS(0, k) = st; HS(1, k) = sq; }
      }
      SYNC;
    }
    // GCM-level tendencies and statistics
    for (int l = TID + 1; l <= plev; l += NT) {
      double tln, qln, qccln, qiiln;
      if (l < ptop) {
        tln = IN(p.tl, l); qln = IN(p.ql, l); qccln = IN(p.qccl, l); qiiln = IN(p.qiil, l);
      } else {
        int k = plev - l + 1;
        tln = HS(0, k) * factor_xy; qln = HS(1, k) * factor_xy; qccln = HS(2, k) * factor_xy; qiiln = HS(3, k) * factor_xy;
      }
      bool top2 = (l == ptop || l == ptop + 1);
      O2(CRM_OUT_SLTEND, l) = top2 ? 0. : C_CP * (tln - IN(p.tl, l)) * icrm_run_time;
      O2(CRM_OUT_QLTEND, l) = top2 ? 0. : (qln - IN(p.ql, l)) * icrm_run_time;
      O2(CRM_OUT_QCLTEND, l) = top2 ? 0. : (qccln - IN(p.qccl, l)) * icrm_run_time;
      O2(CRM_OUT_QILTEND, l) = top2 ? 0. : (qiiln - IN(p.qiil, l)) * icrm_run_time;
      double pdel = IN(p.pdel, l);
      O2(CRM_OUT_CLD, l) = mn2(1.0, (double)OP(O_CLD)[l] * factor_xyt);
      O2(CRM_OUT_CLDTOP, l) = mn2(1.0, (double)OP(O_CLDTOP)[l] * factor_xyt);
      O2(CRM_OUT_GICEWP, l) = (double)OP(O_GICEWP)[l] * pdel * 1000. / C_GGR * factor_xyt;
      O2(CRM_OUT_GLIQWP, l) = (double)OP(O_GLIQWP)[l] * pdel * 1000. / C_GGR * factor_xyt;
      double mcup = (double)OP(O_MCUP)[l] * factor_xyt, mcdn = (double)OP(O_MCDN)[l] * factor_xyt;
      double mcuup = (double)OP(O_MCUUP)[l] * factor_xyt, mcudn = (double)OP(O_MCUDN)[l] * factor_xyt;
      O2(CRM_OUT_MCUP, l) = mcup; O2(CRM_OUT_MCDN, l) = mcdn;
      O2(CRM_OUT_MCUUP, l) = mcuup; O2(CRM_OUT_MCUDN, l) = mcudn;
      O2(CRM_OUT_MCTOT, l) = mcup + mcdn + mcuup + mcudn;
      double mui0 = (double)OP(O_MUI)[l], mui1 = (double)OP(O_MUI)[l + 1];
      double mdi0 = (double)OP(O_MDI)[l], mdi1 = (double)OP(O_MDI)[l + 1];
      double mu = 0.5 * (mui0 + mui1), md = 0.5 * (mdi0 + mdi1);
      mu = mu * C_GGR / 100.;
      md = md * C_GGR / 100.;
      O2(CRM_OUT_MU_CRM, l) = mu;
      O2(CRM_OUT_MD_CRM, l) = md;
      if (mui0 - mui1 > 0) O2(CRM_OUT_EU_CRM, l) = (mui0 - mui1) * C_GGR / pdel;
      else O2(CRM_OUT_DU_CRM, l) = -1.0 * (mui0 - mui1) * C_GGR / pdel;
      if (mdi1 - mdi0 < 0) O2(CRM_OUT_ED_CRM, l) = (mdi0 - mdi1) * C_GGR / pdel;
      bool act = fabs(mu) > R4(1.0e-15) || fabs(md) > R4(1.0e-15);
      if (act) atomicMin(&S.jt_min, l);
      if (act) atomicMax(&S.mx_max, l);
    }
    // flux and condensate profiles at CRM levels
    for (int k = TID + 1; k <= nzm; k += NT) {
      int l = plev - k + 1;
      double qcm = HS(Y3 ? 12 : 2, k), qim = HS(Y3 ? 13 : 3, k), qrm = HS(4, k), qgm = HS(5, k), qsm = HS(6, k);
      double u2z = HS(7, k), v2z = HS(8, k), w2z = HS(9, k), stke = HS(10, k), stk = HS(11, k);
      O2(CRM_OUT_QC_MEAN, l) = qcm * factor_xy;
      O2(CRM_OUT_QI_MEAN, l) = qim * factor_xy;
      O2(CRM_OUT_QS_MEAN, l) = qsm * factor_xy;
      O2(CRM_OUT_QG_MEAN, l) = qgm * factor_xy;
      O2(CRM_OUT_QR_MEAN, l) = qrm * factor_xy;
      double rhow = (double)PR(P_RHOW)[k], rho = (double)PR(P_RHO)[k];
      double tmp1 = S.dz / rhow;
      double tmp2 = tmp1 / S.dtn;
      double ns = (double)S.nstop;
      double mkwsb0 = (double)PR(P_MKWSB0)[k] * tmp1 * rhow * factor_xy / ns;
      double mkwsb1 = (double)PR(P_MKWSB1)[k] * tmp1 * rhow * factor_xy / ns;
      double mkwle0 = (double)PR(P_MKWLE0)[k] * tmp2 * rhow * factor_xy / ns;
      double mkwle1 = (double)PR(P_MKWLE1)[k] * tmp2 * rhow * factor_xy / ns;
      double mkadv0 = (double)PR(P_MKADV0)[k] * factor_xy * icrm_run_time;
      double mkadv1 = (double)PR(P_MKADV1)[k] * factor_xy * icrm_run_time;
      double mkdiff0 = (double)PR(P_MKDIFF0)[k] * factor_xy * icrm_run_time;
      double mkdiff1 = (double)PR(P_MKDIFF1)[k] * factor_xy * icrm_run_time;
      O2(CRM_OUT_FLUX_U, l) = ((double)PR(P_UWLE)[k] + (double)PR(P_UWSB)[k]) * tmp1 * factor_xy / ns;
      O2(CRM_OUT_FLUX_V, l) = ((double)PR(P_VWLE)[k] + (double)PR(P_VWSB)[k]) * tmp1 * factor_xy / ns;
      O2(CRM_OUT_FLUX_QT, l) = mkwle0 + mkwsb0;
      O2(CRM_OUT_FLUXSGS_QT, l) = mkwsb0;
      O2(CRM_OUT_FLUX_QP, l) = mkwle1 + mkwsb1;
      O2(CRM_OUT_QT_TRANS, l) = mkadv0 + mkdiff0;
      O2(CRM_OUT_QP_TRANS, l) = mkadv1 + mkdiff1;
      double tkesgsz = rho * stke * factor_xy;
      O2(CRM_OUT_TKESGSZ, l) = tkesgsz;
      O2(CRM_OUT_TKEZ, l) = rho * 0.5 * (u2z + v2z * (Y3 ? 1.0 : 0.0) + w2z) * factor_xy + tkesgsz;
      O2(CRM_OUT_TKZ, l) = stk * factor_xy;
      O2(CRM_OUT_PRECFLUX, l) = ((double)PR(P_PRECFLUX)[k] * factor_xy * S.dz / p.dt / ns) / 1000.;
      O2(CRM_OUT_QP_FALL, l) = (double)PR(P_QPFALL)[k] * factor_xy * icrm_run_time;
      O2(CRM_OUT_QP_EVP, l) = (double)PR(P_QPEVP)[k] * factor_xy * icrm_run_time;
      O2(CRM_OUT_QP_SRC, l) = (double)PR(P_QPSRC)[k] * factor_xy * icrm_run_time;
      O2(CRM_OUT_QT_LS, l) = (double)PR(P_QTEND)[k];
      O2(CRM_OUT_T_LS, l) = (double)PR(P_TTEND)[k];
    }
    // state and 4D outputs
    for (int e = TID; e < NH() * nzm; e += NT) {
      int i = 1 + e % NH(), k = 1 + e / NH();
      size_t o = S4(i, k);
      p.st[0][o] = (double)u(i, k);
      p.st[1][o] = (double)v(i, k);
      p.st[2][o] = (double)w(i, k);
      if constexpr (sizeof(T) == 4) {
        p.st[3][o] = tabs_d(i, k);
        p.st[4][o] = qt_d(i, k);
      } else {
        p.st[3][o] = (double)tabs(i, k);
        p.st[4][o] = (double)qt(i, k);
      }
      p.st[5][o] = (double)qp(i, k);
      p.st[6][o] = (double)qn(i, k);
      p.out[CRM_OUT_TK][o] = (double)tk(i, k);
      p.out[CRM_OUT_TKH][o] = (double)tkh(i, k);
      p.out[CRM_OUT_QCL][o] = (double)qcl(i, k);
      p.out[CRM_OUT_QCI][o] = (double)qci(i, k);
      p.out[CRM_OUT_QPL][o] = (double)qpl(i, k);
      p.out[CRM_OUT_QPI][o] = (double)qpi(i, k);
    }
    // scalars (thread 0): column precipitation, surface precip, cloud cover
    if (TID == 0) {
      double cp = 0, cps = 0;
      for (int k = 1; k <= nzm; ++k) {
        double pdel = IN(p.pdel, plev - k + 1);
        for (int n = 1; n <= NH(); ++n) {
          const int i = h_ij(n);
          cp = cp + (double)(qpl(i, k) + qpi(i, k)) * pdel;
          cps = cps + (double)qpi(i, k) * pdel;
        }
      }
      O1(CRM_OUT_PRECTEND) = (cp - S.colprec0) / C_GGR * factor_xy * icrm_run_time;
      O1(CRM_OUT_PRECSTEND) = (cps - S.colprecs0) / C_GGR * factor_xy * icrm_run_time;
      O1(CRM_OUT_Z0M) = S.z0;
      O1(CRM_OUT_TAUX) = 0.0 / (double)S.nstop;
      O1(CRM_OUT_TAUY) = 0.0 / (double)S.nstop;
      double precc = 0, precl = 0, precsc = 0, precsl = 0;
      const double thr = (double)(10.f / 86400.f);
      for (int i = 1; i <= NH(); ++i) {
        double ps = (double)PS(i) * S.dz / p.dt / (double)S.nstop;
        double pss = (double)PSS(i) * S.dz / p.dt / (double)S.nstop;
        if (ps > thr) { precc = precc + ps; precsc = precsc + pss; }
        else { precl = precl + ps; precsl = precsl + pss; }
        p.out[CRM_OUT_PREC_CRM][(size_t)icrm + (size_t)ld * (i - 1)] = ps / 1000.;
      }
      O1(CRM_OUT_PRECC) = precc * factor_xy / 1000.;
      O1(CRM_OUT_PRECL) = precl * factor_xy / 1000.;
      O1(CRM_OUT_PRECSC) = precsc * factor_xy / 1000.;
      O1(CRM_OUT_PRECSL) = precsl * factor_xy / 1000.;
      O1(CRM_OUT_CLTOT) = S.cltot * factor_xyt;
      O1(CRM_OUT_CLHGH) = S.clhgh * factor_xyt;
      O1(CRM_OUT_CLMED) = S.clmed * factor_xyt;
      O1(CRM_OUT_CLLOW) = S.cllow * factor_xyt;
      int jt = S.jt_min, mx = S.mx_max;
      O1(CRM_OUT_JT_CRM) = (jt <= plev) ? mn2((double)plev, (double)jt) : (double)plev;
      O1(CRM_OUT_MX_CRM) = mx2(1.0, (double)mx);
      O1(CRM_OUT_TIMING_FACTOR) = (double)S.nstop / (double)S.nstop;
      p.col_status[cpos] = S.status;
    }
    SYNC;
  }

  // ---------------------------------------------------------- one column
  // Inlined into the kernel: as a separate function its register allocation
  // spilled around the call (12 % slower in the FP32-mixed form).
  __device__ __forceinline__ void run(T *fsh, T *wsh, float *tcsm = nullptr) {
    if (icrm < 0 || icrm >= p.ld) {            // bad slot in col_map: no access
      if (TID == 0) p.col_status[cpos] = CRM_ERR_ARG;
      return;
    }
    if (TID == 0) S.t_last = clock64();
    init_column();
    if (TID == 0) { S.jt_min = 1 << 30; S.mx_max = 0; }
    SYNC;
    PHASE_MARK(PH_INIT);
    for (int nstep = 1; nstep <= S.nstop; ++nstep) {
      kurant();
      PHASE_MARK(PH_KURANT);
      if (S.ncycle > 16 || S.status != CRM_OK) {
        if (TID == 0 && S.status == CRM_OK) S.status = CRM_ERR_CFL;
        SYNC;
        break;
      }
      const int ncycle = S.ncycle;
      for (int icyc = 1; icyc <= ncycle; ++icyc) {
        if (TID == 0) {
          S.icycle = icyc;
          S.dtn = p.dt / ncycle;
          S.dt3[S.na - 1] = S.dtn;
          S.dtfactor = S.dtn / p.dt;
          abcoefs(nstep);
        }
        SYNC;
        zero_and_buoyancy();
        PHASE_MARK(PH_BUOY);
        forcing_radiation();
        PHASE_MARK(PH_FORCING);
        damping();
        PHASE_MARK(PH_DAMPING);
        ice_fall();
        PHASE_MARK(PH_ICEFALL);
        boundaries(3);
        boundaries(0);
        PHASE_MARK(PH_BOUND);
        tke_full();
        PHASE_MARK(PH_TKE);
        boundaries(4);
        if constexpr (Y3) advect_mom3();
        else advect_mom();
        PHASE_MARK(PH_ADVMOM);
        if constexpr (Y3) diffuse_mom3();
        else diffuse_mom();
        PHASE_MARK(PH_DIFFMOM);
        if constexpr (Y3) pressure3(fsh, tcsm);
        else pressure(fsh, wsh);
        adams();
        boundaries(2);
        PHASE_MARK(PH_ADAMS);
        bool qp_zero;
        if constexpr (Y3) {
          advect_scalar3(TT(), nullptr, nullptr, rct(), t_offset(nstep, icyc));
          PHASE_MARK(PH_ADV_T);
          advect_scalar3(QT(), PR(P_MKADV0), PR(P_MKWLE0), rcq());
          PHASE_MARK(PH_ADV_QT);
          qp_zero = all_pos_zero(QP());
          if (qp_zero) zero_stats(PR(P_MKADV1), PR(P_MKWLE1));
          else advect_scalar3(QP(), PR(P_MKADV1), PR(P_MKWLE1));
        } else {
          advect_scalar(TT(), nullptr, nullptr, rct(), t_offset(nstep, icyc));
          PHASE_MARK(PH_ADV_T);
          advect_scalar(QT(), PR(P_MKADV0), PR(P_MKWLE0), rcq());
          PHASE_MARK(PH_ADV_QT);
          qp_zero = all_pos_zero(QP());
          if (qp_zero) zero_stats(PR(P_MKADV1), PR(P_MKWLE1));
          else advect_scalar(QP(), PR(P_MKADV1), PR(P_MKWLE1));
        }
        PHASE_MARK(PH_ADV_QP);
        precip_fall_1(qp_zero);
        PHASE_MARK(PH_FALL1);
        if (S.prec_any) precip_fall_2(S.nprec);
        PHASE_MARK(PH_FALL2);
        uvw();
        boundaries(3);
        PHASE_MARK(PH_UVW);
        if constexpr (Y3) {
          diffuse_scalar3(TT(), nullptr, nullptr, rct());
          PHASE_MARK(PH_DIFF_T);
          diffuse_scalar3(QT(), PR(P_MKDIFF0), PR(P_MKWSB0), rcq());
          if (qp_zero || all_pos_zero(QP())) zero_stats(PR(P_MKDIFF1), PR(P_MKWSB1));
          else diffuse_scalar3(QP(), PR(P_MKDIFF1), PR(P_MKWSB1));
        } else {
          diffuse_scalar(TT(), nullptr, nullptr, rct());
          PHASE_MARK(PH_DIFF_T);
          diffuse_scalar(QT(), PR(P_MKDIFF0), PR(P_MKWSB0), rcq());
          if (qp_zero || all_pos_zero(QP())) zero_stats(PR(P_MKDIFF1), PR(P_MKWSB1));
          else diffuse_scalar(QP(), PR(P_MKDIFF1), PR(P_MKWSB1));
        }
        PHASE_MARK(PH_DIFF_Q);
        if (S.icycle == 1) precip_init();
        PHASE_MARK(PH_PINIT);
        cloud();
        PHASE_MARK(PH_CLOUD);
        precip_proc();
        PHASE_MARK(PH_PPROC);
        micro_diagnose();
        PHASE_MARK(PH_MDIAG);
        if (p.use_accel && !S.ceaseflag) accelerate(nstep);
        diagnose();
        if (TID == 0) { int nn = S.na; S.na = S.nc; S.nc = S.nb; S.nb = nn; }
        SYNC;
        PHASE_MARK(PH_DIAG);
      }
      step_stats();
      PHASE_MARK(PH_STATS);
    }
    finalize();
    PHASE_MARK(PH_FINAL);
  }
};

// Dynamic shared memory: FFT rows (nx+2) x nzm, one FFT work row per warp,
// then (optionally) scratch planes A and B, each starting on 64 elements.
__host__ __device__ inline size_t crm_round64(size_t n) { return (n + 63) / 64 * 64; }
__host__ __device__ inline size_t crm_plane_elems(int nx, int nzm) { return crm_round64((size_t)(nx + 6) * (nzm + 2)); }
template <typename T>
__host__ __device__ inline size_t crm_smem_bytes(int nx, int nzm, int block, int planes = 0) {
  size_t e = (size_t)(nx + 2) * nzm + (size_t)(block / 32) * (nx + 4);
  if (planes) e = crm_round64(e) + (size_t)planes * crm_plane_elems(nx, nzm);
  return sizeof(T) * e;
}

// 3D: the Fourier coefficients live in the slab; shared memory holds one
// transform row and one work row (2 max(nx, ny) + 8) per warp
// (with the tensor-core transforms, tc_n != 0, their operands instead)
template <typename T>
__host__ __device__ inline size_t crm_smem_bytes3(int nx, int ny, int block, int tc_n = 0) {
  const int nmax = nx > ny ? nx : ny;
  const size_t fft = sizeof(T) * (size_t)(block / 32) * (size_t)(2 * nmax + 8);
  const size_t tcb = tc::smem_bytes(tc_n);
  return fft > tcb ? fft : tcb;
}

// VAR: kVarPlain, kVarTc (the tensor-core transforms) or kVarFma (the FP64
// form compiled with multiply-add contraction); a separate instance each
template <typename T, int NX, int NY, int NTH, int MINB, int SMP, int VAR>
__global__ void __launch_bounds__(NTH, MINB) crm_columns_kernel(const __grid_constant__ KParams p) {
  constexpr int TC = VAR == kVarTc ? 1 : 0;
  __shared__ ColShared S;
  extern __shared__ __align__(16) unsigned char crm_dsm[];
  T *fsh = reinterpret_cast<T *>(crm_dsm);
  T *wsh = fsh + (size_t)(p.L.nx + 2) * p.L.nzm;
  T *planes = nullptr;
  if constexpr (SMP && NY == 1)
    planes = fsh + crm_round64((size_t)(p.L.nx + 2) * p.L.nzm + (size_t)(NTH / 32) * (p.L.nx + 4));
  T *base = reinterpret_cast<T *>(p.slabs) + (size_t)blockIdx.x * p.L.slab;
  if (threadIdx.x == 0) S.gbar = 0;
  float *tcsm = nullptr;
  if constexpr (TC != 0 && NY != 1 && sizeof(T) == 4) {
    if (p.tc_n) {
      // tensor memory for the transforms' accumulator (warp 0), the
      // mbarrier their commits arrive on, the constant matrices split into
      // TF32 head and tail
      tcsm = reinterpret_cast<float *>((reinterpret_cast<uintptr_t>(crm_dsm) + 127) & ~(uintptr_t)127);
      if (threadIdx.x < 32) {
        tc::tmem_alloc(tc::smem_u32(&S.tc_tmem), tc::kTmemCols);
        tc::fence_before();
      }
      if (threadIdx.x == 0) {
        tc::mbar_init(tc::smem_u32(&S.tc_mbar));
        S.tc_phase = 0;
        S.tc_fail = 0;
      }
      tc::Engine(p.tc_n, tcsm, 0u, 0u, nullptr, nullptr, threadIdx.x, NTH).load_mats(p.dft_tc);
      __syncthreads();
      tc::fence_after();
    }
  }
  for (int col = blockIdx.x; col < p.ncrms; col += gridDim.x) {
    ColumnKernel<T, NX, NY, TC> K(p, S, base, col, planes);
    K.run(fsh, wsh, tcsm);
    __syncthreads();
  }
  if constexpr (TC != 0 && NY != 1 && sizeof(T) == 4) {
    if (p.tc_n) {
      // a commit that outlived its wait is awaited (bounded) before the
      // accumulator is released
      if (threadIdx.x == 0 && S.tc_fail) tc::mbar_wait(tc::smem_u32(&S.tc_mbar), S.tc_phase ^ 1u, tc::kWaitLimit);
      __syncthreads();
      if (threadIdx.x < 32) {
        tc::fence_after();
        tc::tmem_free(S.tc_tmem, tc::kTmemCols);
      }
    }
  }
}

template <typename T, int NX, int NY, int SHAPE, int VAR>
size_t crm_launch_smem(int nx, int ny, int nzm, int tc_n) {
  constexpr int nth = kShapes[SHAPE].threads, smp = kShapes[SHAPE].smem_planes;
  if constexpr (NY != 1) return crm_smem_bytes3<T>(nx, ny, nth, (VAR == kVarTc && sizeof(T) == 4) ? tc_n : 0);
  else return crm_smem_bytes<T>(nx, nzm, nth, smp);
}

template <typename T, int NX, int NY, int SHAPE, int VAR>
void launch_crm_columns(const KParams &p, int grid, cudaStream_t s, bool cooperative) {
  constexpr int nth = kShapes[SHAPE].threads, minb = kShapes[SHAPE].min_ctas, smp = kShapes[SHAPE].smem_planes;
  size_t smem = crm_launch_smem<T, NX, NY, SHAPE, VAR>(p.L.nx, p.L.ny, p.L.nzm, p.tc_n);
  auto kern = crm_columns_kernel<T, NX, NY, nth, minb, smp, VAR>;
  cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (cooperative) {
    // every CTA co-resident (the batch-mode grid barrier relies on it); the
    // launch fails rather than over-subscribe
    KParams q = p;
    void *args[] = {&q};
    cudaLaunchCooperativeKernel(reinterpret_cast<const void *>(kern), dim3(grid), dim3(nth), args, smem, s);
  } else {
    kern<<<grid, nth, smem, s>>>(p);
  }
}

// CTAs of the shape resident per SM (0: the shape does not fit); 3D runs
// without shared-memory scratch planes, so those shapes report 0 there
template <typename T, int NX, int NY, int SHAPE, int VAR>
int occupancy_crm_columns(int nx, int ny, int nzm, int tc_n) {
  constexpr int nth = kShapes[SHAPE].threads, minb = kShapes[SHAPE].min_ctas, smp = kShapes[SHAPE].smem_planes;
  if (NY != 1 && smp) return 0;
  int n = 0;
  size_t smem = crm_launch_smem<T, NX, NY, SHAPE, VAR>(nx, ny, nzm, tc_n);
  if (smem > 227 * 1024) return 0;
  auto kern = crm_columns_kernel<T, NX, NY, nth, minb, smp, VAR>;
  cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, kern, nth, smem) != cudaSuccess) return 0;
  return n;
}

}  // namespace crm
