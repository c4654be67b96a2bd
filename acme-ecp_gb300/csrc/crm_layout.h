// crm_layout.h -- per-column slab layout shared by host and device code.
//
// The device keeps each CRM column's fields in one contiguous slab (x fastest,
// then k), so the CTA that owns the column touches one compact block of
// memory that stays resident in L1/L2 across the whole GCM step.  Index
// ranges (halos included) are those of the reference's module arrays
// (crm/grid.F90:31-46 with NADV = NADVS = 0, crm/vars.F90:200-238,
// SGS_TKE/sgs.F90:50-60).  A 3D column (ny > 1) stores every field level
// by level, each level nya rows of nxa (the y halos of the same module
// arrays); ny = 1 gives the 2D layout, with no y halo.
#pragma once
#include <cstddef>

namespace crm {

// x extents (first index, length) of the field classes
struct XRange {
  int x1, nxa;
};

struct Layout {
  int nx, nzm, nz, plev, nx_rad;
  int ny, ny_rad, yes3d, lnx;      // ny = 1 and yes3d = 0: 2D; lnx = log2 nx (3D)
  // x ranges
  XRange xu, xv, xw, xs, xd, xp, xi, xdu;
  // y ranges (2D: {1, 1} each)
  XRange yu, yv, yw, ys, yd, yp, yi, ydv, ysc;
  // offsets (in elements) of every array inside one column slab
  size_t u, v, w, t, qt, qp, tke, tk, tkh, p, tabs, qv, qcl, qci, qpl, qpi, qn;
  size_t du[3], dv[3], dw[3];
  size_t precsfc, precssfc;
  // scratch (per phase)
  size_t s_a, s_b, s_c, s_d, s_e, s_f, s_g, s_h;   // nxs x (nz+1) each
  size_t fft_f, fft_w;                             // (nx+2) x nzm, work
  // profiles: each (nz + 2) long, indexed directly by k (0 .. nz+1)
  size_t prof;           // first profile
  int nprof;             // number of profiles
  size_t o_plev;         // GCM-level accumulators, (plev + 2) each
  int n_oplev;
  size_t rad;            // rad accumulators 5 x (nx_rad x nzm) + qrad
  size_t rnd;            // setperturb random numbers 5 x nx
  size_t colstat;        // per-column scratch for step statistics, 8 x nx
  size_t fcomp;          // FP32-mixed form only: carried residues of t, qt (2 x nx x nzm)
  size_t tri;            // FP64 tridiagonal factors (see tridiag_factor)
  size_t slab;           // total elements per column
};

// profile indices (each profile is (nz+2) long, indexed by k)
enum Prof {
  P_Z, P_ZI, P_PRES, P_PRESI, P_ADZ, P_ADZW, P_RHO, P_RHOW, P_BET, P_GAMAZ,
  P_T0, P_Q0, P_QV0, P_TABS0, P_U0, P_V0, P_QP0, P_QN0, P_T00,
  P_TTEND, P_QTEND, P_UTEND, P_VTEND,
  P_GRDFX, P_GRDFY, P_GRDFZ,
  P_ACCRSC, P_ACCRSI, P_ACCRRC, P_COEFICE, P_ACCRGC, P_ACCRGI,
  P_EVAPS1, P_EVAPS2, P_EVAPR1, P_EVAPR2, P_EVAPG1, P_EVAPG2,
  P_UWLE, P_VWLE, P_UWSB, P_VWSB, P_PRECFLUX, P_QPFALL, P_TLAT, P_TLATQI, P_QIFALL,
  P_MKWLE0, P_MKWLE1, P_MKWSB0, P_MKWSB1, P_MKADV0, P_MKADV1, P_MKDIFF0, P_MKDIFF1,
  P_QPSRC, P_QPEVP,
  // per-level reciprocals of the grid metrics, fixed for the call (the
  // reference divides per cell or keeps such arrays per routine)
  P_IADZ, P_IADZW, P_IRHO, P_IRHOADZ, P_IRHOWADZ, P_IRHOWADZW, P_RDZ, P_RDZW, P_MPDD,
  P_RDXZ, P_RDXW, P_BETDZ, P_TKMAX,   // SGS closure per-level factors
  P_RDYZ, P_RDYW,                      // the same in y (3D)
  P_BETU, P_BETD, P_RUP, P_RDN, P_RHOWDADZW,   // buoyancy, pressure RHS, diffusion
  P_TMP0, P_TMP1, P_TMP2, P_TMP3, P_TMP4, P_TMP5, P_TMP6, P_TMP7,
  P_COUNT
};

// GCM-level accumulators (plev + 2 each, indexed by l)
enum OPlev {
  O_CLD, O_CLDTOP, O_GICEWP, O_GLIQWP, O_MCUP, O_MCDN, O_MCUUP, O_MCUDN, O_MUI, O_MDI,
  O_COUNT
};

// esz: bytes per element of the bulk type (8: FP64 form, 4: FP32-mixed)
inline Layout make_layout(int nx, int nzm, int plev, int nx_rad, int esz, int ny = 1, int ny_rad = 1) {
  Layout L{};
  L.nx = nx; L.nzm = nzm; L.nz = nzm + 1; L.plev = plev; L.nx_rad = nx_rad;
  L.ny = ny; L.ny_rad = ny_rad;
  const int Y = ny > 1 ? 1 : 0;
  L.yes3d = Y;
  L.lnx = 0;
  while ((1 << L.lnx) < nx) ++L.lnx;
  L.xu = {-1, nx + 5};
  L.xv = {-1, nx + 4};
  L.xw = {-1, nx + 4};
  L.xs = {-2, nx + 6};
  L.xd = {0, nx + 2};
  L.xp = {0, nx + 1};
  L.xi = {1, nx};
  L.xdu = {1, nx + 1};
  // y extents of the same arrays (crm/grid.F90:31-46 with YES3D)
  L.yu = {1 - 2 * Y, ny + 4 * Y};
  L.yv = {1 - 2 * Y, ny + 5 * Y};
  L.yw = {1 - 2 * Y, ny + 4 * Y};
  L.ys = {1 - 3 * Y, ny + 6 * Y};
  L.yd = {1 - Y, ny + 2 * Y};
  L.yp = {1 - Y, ny + Y};
  L.yi = {1, ny};
  L.ydv = {1, ny + Y};
  L.ysc = {1 - 3 * Y, ny + 6 * Y};
  size_t o = 0;
  auto take = [&](size_t n) { size_t r = o; o += (n + 63) / 64 * 64; return r; };
  const int nz = L.nz;
  auto plane = [&](XRange x, XRange y) { return (size_t)x.nxa * y.nxa; };
  L.u = take(plane(L.xu, L.yu) * nzm);
  L.v = take(plane(L.xv, L.yv) * nzm);
  L.w = take(plane(L.xw, L.yw) * nz);
  L.t = take(plane(L.xs, L.ys) * nzm);
  L.qt = take(plane(L.xs, L.ys) * nzm);
  L.qp = take(plane(L.xs, L.ys) * nzm);
  L.tke = take(plane(L.xi, L.yi) * nzm);
  L.tk = take(plane(L.xd, L.yd) * nzm);
  L.tkh = take(plane(L.xd, L.yd) * nzm);
  L.p = take(plane(L.xp, L.yp) * nzm);
  const size_t nh = (size_t)nx * ny;
  L.tabs = take(nh * nzm);
  L.qv = take(nh * nzm);
  L.qcl = take(nh * nzm);
  L.qci = take(nh * nzm);
  L.qpl = take(nh * nzm);
  L.qpi = take(nh * nzm);
  L.qn = take(nh * nzm);
  for (int l = 0; l < 3; ++l) {
    L.du[l] = take(plane(L.xdu, L.yi) * nzm);
    L.dv[l] = take(plane(L.xi, L.ydv) * nzm);
    L.dw[l] = take(nh * nz);
  }
  L.precsfc = take(nh);
  L.precssfc = take(nh);
  const size_t sc = (size_t)(nx + 6) * L.ysc.nxa * (nz + 1);
  L.s_a = take(sc); L.s_b = take(sc); L.s_c = take(sc); L.s_d = take(sc);
  L.s_e = take(sc); L.s_f = take(sc); L.s_g = take(sc); L.s_h = take(sc);
  const size_t ny2 = Y ? (size_t)ny + 2 : 1;
  L.fft_f = take((size_t)(nx + 2) * ny2 * (nzm + 1));
  L.fft_w = take((size_t)(nx + 4) * (nzm + 1));
  L.nprof = P_COUNT;
  L.prof = take((size_t)(nz + 2) * P_COUNT);
  L.n_oplev = O_COUNT;
  L.o_plev = take((size_t)(plev + 2) * O_COUNT);
  L.rad = take((size_t)6 * nx_rad * ny_rad * nzm);
  L.rnd = take((size_t)5 * nh);
  L.colstat = take((size_t)8 * nh);
  L.fcomp = esz == 4 ? take((size_t)2 * nh * nzm) : 0;
  {
    const size_t np = (size_t)(nx + 1) * ny2;    // Fourier coefficients per level
    size_t nd = (size_t)(nzm + 1) + np * 2 * (nzm + 1) + np;
    L.tri = take(nd * 8 / esz + 2);
  }
  L.slab = o;
  return L;
}

}  // namespace crm
