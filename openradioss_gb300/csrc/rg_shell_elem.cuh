#pragma once
// Belytschko-Tsay 4-node shell element (CFORC3 chain): parameters, state
// layout and the per-element device function shared by the single-model
// kernel (rg_shell.cu) and the batched persistent kernel (rg_batch.cu).
//
// One thread per element, the NPT through-thickness points in registers.
// The arithmetic follows, step by step and in the same expression order,
// the reference routines (paths relative to the OpenRadioss source tree):
//   CCOOR3 gather            elements/shell/coque/ccoor3.F:31
//   CNVEC3 convected frame   elements/shell/coque/cnvec3.F:35 (ISHFRAM 0 or 2)
//   CDERI3 local geometry    elements/shell/coque/cderi3.F:30 (ISMSTR = 4)
//   CCOEF3 coefficients      elements/shell/coque/ccoef3.F:30 (ITHK 1 or 0)
//   CDLEN3 length for dt     elements/shell/coque/cdlen3.F:30
//   CDEFO3 membrane rates    elements/shell/coque/cdefo3.F:30 (IHBE <= 1)
//   CCURV3 curvature rates   elements/shell/coque/ccurv3.F:30
//   CSTRA3 increments, GSTR  elements/shell/coque/cstra3.F:30
//   MULAWC + SIGEPS02C + M2CPLR  materials/mat_share/mulawc.F90:185,
//                            materials/mat/mat002/sigeps02c.F:33, m2cplr.F:29
//   CHVIS3 hourglass         elements/shell/coque/chvis3.F:32
//   CDT3 element dt, STI     elements/shell/coque/cdt3.F:32
//   CFINT3 nodal forces      elements/shell/coque/cfint3.F:30
//   CUPDT3P slot writes      elements/shell/coque/cupdt3.F:967-1100
// Through-thickness positions / weights: the COQINI tables
// (elements/shell/coqini.F:46-123), default-real literals.
#include "rg_device.cuh"

#include <algorithm>
#include <cmath>
#include <cstring>
#include <type_traits>
#include <vector>


// Cooperative 16-byte staging of full warps (see shell_element).
#ifndef RG_SHELL_COOP_STAGE
#define RG_SHELL_COOP_STAGE 1
#endif

namespace rg {

struct ShellParams {
  int nft, nel, npt, ipla;
  int part_off;
  // launch layout: nblk blocks; wtasks = 0: one element per thread, else
  // the group's wtasks 32-element warp tasks, taken by the warps of one wave
  // of resident blocks from the counter qctr (zeroed before each launch)
  unsigned *qctr;
  int nblk, wtasks;
  int ishfram;  // local frame: 0 symmetric (default), 2 version-4 (/SHFRA/V4)
  double rho, young, nu, g, a11, ssp;
  double h1, h2, h3, srh1, srh2, srh3, dm, ish, fsh;
  double ca, cb, cn, ymax, cc, eps0, pm9;
  int icc, vp, israte;
  int ithk;     // 1: current thickness in CCOEF3, 0: initial thickness
  double dtfac;
  // group constants derived once on the host (they are the same for every
  // element of the group): plane-stress moduli, 1/(1-NU), 1/(1+NU),
  // 1/MAX(H1,H2), DTFAC/SSP and, when ISH = 0 (SHF = FSH), the hourglass
  // coefficients of CHVIS3
  double a1, a2, inv1mnu, inv1pnu, inv_hmax, dtfac_ssp;
  double shf0, hA1, hA3, hA5, hA7, hA8;
  int shf_const;
  int nodadt;   // nodal time step: STI / STIR for DTNODA, no element dt
  // kinematic / mixed hardening (FISOKIN, m2cplr.F:115-121, 289-363) and
  // Johnson-Cook thermal softening with adiabatic heating (T* from each
  // point's temperature, sigeps02c.F:125, 226-229; thermal = rho*Cp > 0)
  double fisokin, m_exp, tref, tmelt, rhocp;
  int thermal;
  // element time-step action (IDTMIN(3), DTMIN1(3), cdt3.F:77-141): 0 none,
  // 1 or 5 stop the run (RG_ST_DTMIN), 2 delete the element
  int idtmin;
  double dtmin;
  // FP32 copies for the mixed form (converted once on the host) and the
  // branch flags CC /= 0, DM /= 0 evaluated on the FP64 values
  struct {
    float rho, young, nu, g, a11, ssp, h1, h2, h3, dm, ish, fsh;
    float ca, cb, cn, ymax, cc, eps0, pm9, dtfac;
    float a1, a2, inv1mnu, inv1pnu, inv_hmax, dtfac_ssp;
    float shf0, hA1, hA3, hA5, hA7, hA8;
    float fisokin, m_exp, tref, tmelt, rhocp, dtmin;
    int cc_nz, dm_nz;
  } f;
};

inline void shell_params_mirror(ShellParams &P) {
  // derived group constants (same expressions as the per-element code)
  P.a1 = P.young / (1.0 - P.nu * P.nu);
  P.a2 = P.a1 * P.nu;
  P.inv1mnu = 1.0 / (1.0 - P.nu);
  P.inv1pnu = 1.0 / (1.0 + P.nu);
  P.inv_hmax = 1.0 / (P.h1 > P.h2 ? P.h1 : P.h2);
  P.dtfac_ssp = P.dtfac / P.ssp;
  P.shf_const = (P.npt == 1 || P.ish == 0.0) ? 1 : 0;
  P.shf0 = P.npt == 1 ? 0.0 : P.fsh;
  {
    const double shfpr3 = P.shf0 / (3.0 * (1.0 + P.nu));
    const double r1 = 0.25 * P.rho * 100.0;
    const double r0e = 0.25 * P.young * 0.5;
    P.hA1 = r1 * (0.5 * P.h1);
    P.hA3 = r1 * (0.5 * P.h2) * std::sqrt(shfpr3);
    P.hA5 = (0.5 * P.h3) * r1 * RG_ZEP072169;
    P.hA7 = P.h1 * r0e;
    P.hA8 = P.h2 * r0e * shfpr3;
  }
  P.f.dtmin = (float)P.dtmin;
  P.f.a1 = (float)P.a1;
  P.f.a2 = (float)P.a2;
  P.f.inv1mnu = (float)P.inv1mnu;
  P.f.inv1pnu = (float)P.inv1pnu;
  P.f.inv_hmax = (float)P.inv_hmax;
  P.f.dtfac_ssp = (float)P.dtfac_ssp;
  P.f.shf0 = (float)P.shf0;
  P.f.hA1 = (float)P.hA1;
  P.f.hA3 = (float)P.hA3;
  P.f.hA5 = (float)P.hA5;
  P.f.hA7 = (float)P.hA7;
  P.f.hA8 = (float)P.hA8;
  P.f.rho = (float)P.rho;
  P.f.young = (float)P.young;
  P.f.nu = (float)P.nu;
  P.f.g = (float)P.g;
  P.f.a11 = (float)P.a11;
  P.f.ssp = (float)P.ssp;
  P.f.h1 = (float)P.h1;
  P.f.h2 = (float)P.h2;
  P.f.h3 = (float)P.h3;
  P.f.dm = (float)P.dm;
  P.f.ish = (float)P.ish;
  P.f.fsh = (float)P.fsh;
  P.f.ca = (float)P.ca;
  P.f.cb = (float)P.cb;
  P.f.cn = (float)P.cn;
  P.f.ymax = (float)P.ymax;
  P.f.cc = (float)P.cc;
  P.f.eps0 = (float)P.eps0;
  P.f.pm9 = (float)P.pm9;
  P.f.dtfac = (float)P.dtfac;
  P.f.fisokin = (float)P.fisokin;
  P.f.m_exp = (float)P.m_exp;
  P.f.tref = (float)P.tref;
  P.f.tmelt = (float)P.tmelt;
  P.f.rhocp = (float)P.rhocp;
  P.f.cc_nz = P.cc != 0.0;
  P.f.dm_nz = P.dm != 0.0;
}


template <typename ER>
struct ShellArrays {
  int nc;                 // shell count (SoA stride)
  const int *ix;          // [4][nc] 0-based nodes
  const int *iadc;        // [4][nc] 0-based slots
  const int *degen;       // [nc] IXC(4) == IXC(5) (degenerate quad)
  ER *offg, *thke;
  double *thk;            // FP64 in both forms (slow accumulation)
  ER *forc, *mom, *hour, *gstr, *epsdg;  // [5|3|5|8|1][nc]
  double *eint;           // [2][nc]
  ER *sig, *pla, *epsd;   // [npt][5][nc], [npt][nc], [npt][nc]
  double *ehou;           // [nc]
  ER *sigbak;             // back stress [npt][3][nc] (FISOKIN > 0), else null
  ER *temp;               // temperature [npt][nc] (thermal groups), else null
};


// COQINI tables (NPT = 1..5), single-precision DATA literals.
static __constant__ float c_z0[5][5] = {{0.f, 0.f, 0.f, 0.f, 0.f},
                                 {-.5f, 0.5f, 0.f, 0.f, 0.f},
                                 {-.5f, 0.f, 0.5f, 0.f, 0.f},
                                 {-.5f, -.1666667f, 0.1666667f, 0.5f, 0.f},
                                 {-.5f, -.25f, 0.f, 0.25f, 0.5f}};
static __constant__ float c_wf[5][5] = {{1.f, 0.f, 0.f, 0.f, 0.f},
                                 {0.5f, 0.5f, 0.f, 0.f, 0.f},
                                 {0.25f, 0.5f, 0.25f, 0.f, 0.f},
                                 {0.1666667f, 0.3333333f, 0.3333333f, 0.1666667f, 0.f},
                                 {0.125f, 0.25f, 0.25f, 0.25f, 0.125f}};
static __constant__ float c_wm[5][5] = {{0.f, 0.f, 0.f, 0.f, 0.f},
                                 {-.0833333f, 0.0833333f, 0.f, 0.f, 0.f},
                                 {-.0833333f, 0.f, 0.0833333f, 0.f, 0.f},
                                 {-.0648148f, -.0555556f, 0.0555556f, 0.0648148f, 0.f},
                                 {-.0520833f, -.0625f, 0.f, 0.0625f, 0.0520833f}};

// The same tables widened to FP64 (exact conversions of the REAL*4 values):
// the FP64 form reads them without a per-use conversion.
#define RG_WIDEN5(a, b, c, d, e) {(double)(a), (double)(b), (double)(c), (double)(d), (double)(e)}
static __constant__ double c_z0d[5][5] = {RG_WIDEN5(0.f, 0.f, 0.f, 0.f, 0.f),
                                          RG_WIDEN5(-.5f, 0.5f, 0.f, 0.f, 0.f),
                                          RG_WIDEN5(-.5f, 0.f, 0.5f, 0.f, 0.f),
                                          RG_WIDEN5(-.5f, -.1666667f, 0.1666667f, 0.5f, 0.f),
                                          RG_WIDEN5(-.5f, -.25f, 0.f, 0.25f, 0.5f)};
static __constant__ double c_wfd[5][5] = {RG_WIDEN5(1.f, 0.f, 0.f, 0.f, 0.f),
                                          RG_WIDEN5(0.5f, 0.5f, 0.f, 0.f, 0.f),
                                          RG_WIDEN5(0.25f, 0.5f, 0.25f, 0.f, 0.f),
                                          RG_WIDEN5(0.1666667f, 0.3333333f, 0.3333333f, 0.1666667f, 0.f),
                                          RG_WIDEN5(0.125f, 0.25f, 0.25f, 0.25f, 0.125f)};
static __constant__ double c_wmd[5][5] = {RG_WIDEN5(0.f, 0.f, 0.f, 0.f, 0.f),
                                          RG_WIDEN5(-.0833333f, 0.0833333f, 0.f, 0.f, 0.f),
                                          RG_WIDEN5(-.0833333f, 0.f, 0.0833333f, 0.f, 0.f),
                                          RG_WIDEN5(-.0648148f, -.0555556f, 0.0555556f, 0.0648148f, 0.f),
                                          RG_WIDEN5(-.0520833f, -.0625f, 0.f, 0.0625f, 0.0520833f)};
#undef RG_WIDEN5

template <typename T>
__device__ __forceinline__ T smax(T a, T b) {
  return a > b ? a : b;
}
template <typename T>
__device__ __forceinline__ T smin(T a, T b) {
  return a < b ? a : b;
}

// 1 / MAX(SQRT(S), EM20) of CNVEC3's normalisations.  FP64 form: one
// reciprocal square root (a square root and a division each cost about ten
// instructions of the FP64 pipe, which bounds the FP64 kernel); below
// EM20^2 the value 1/EM20 as in the reference.  FP32 form: as written.
template <typename R>
__device__ __forceinline__ R inv_norm_em20(const R s) {
  if constexpr (std::is_same<R, double>::value)
    return s > RG_EM20 * RG_EM20 ? rsqrt(s) : RG_ONE / RG_EM20;
  else
    return (R)RG_ONE / smax(sqrt(s), (R)RG_EM20);
}

// SQRT(S1 / S2) (CNVEC3); FP64 form as S1 * RSQRT(S1 * S2).
template <typename R>
__device__ __forceinline__ R sqrt_ratio(const R s1, const R s2) {
  if constexpr (std::is_same<R, double>::value)
    return s1 > 0.0 ? s1 * rsqrt(s1 * s2) : sqrt(s1 / s2);
  else
    return sqrt(s1 / s2);
}

// Shared-memory staging of a block's element state (mixed form, single-model
// kernel): per thread of an SNT-thread block, the float components
// [forc 5 | mom 3 | hour 5 | gstr 8 | sig 5*NPT | pla NPT | epsd NPT] and the
// doubles [eint 2 | ehou], component-major (slot = component * NT + thread).
constexpr int SHELL_STG_NT = 128;
constexpr int SG_FORC = 0, SG_MOM = 5, SG_HOUR = 8, SG_GSTR = 13, SG_SIG = 21;
template <int NPT>
struct ShellStage {
  static constexpr int nfloat = 21 + 7 * NPT;
  static constexpr int pla = SG_SIG + 5 * NPT;
  static constexpr int epsd = SG_SIG + 6 * NPT;
  static constexpr int ndouble = 3;
};

// Material branches compiled into a kernel variant (MF bits): 1 kinematic /
// mixed hardening, 2 thermal softening, 4 IPLA = 2.  The lean variant (MF =
// 0) serves groups that use none of them; the full one (SHELL_MF_ALL) the
// others -- the extra live values of those branches would otherwise cost
// every group registers and time.
constexpr int SHELL_MF_ALL = 7;
inline int shell_mf(const ShellParams &P) {
  return (P.fisokin > 0.0 || P.thermal || P.ipla == 2) ? SHELL_MF_ALL : 0;
}

template <typename ER, int NPT, bool STAGE = false, int MF = 0, int SNT = SHELL_STG_NT>
__device__ __forceinline__ void shell_element(const ShellParams &P, const ShellArrays<ER> &S,
                                              const NodeView &N,
                                              typename SlotT<ER>::type *__restrict__ fsky,
                                              typename SlotT<ER>::type *__restrict__ fskyr,
                                              const Time *__restrict__ T, const int key0,
                                              const int nc_total, const int il, ER &dtmine,
                                              int &elmin, const double DT1in = -1.0,
                                              const ER dtinv_in = (ER)0,
                                              float *__restrict__ stg = nullptr,
                                              double *__restrict__ stgd = nullptr,
                                              int *__restrict__ status_dt = nullptr) {
  typedef ER R;
  constexpr bool F64 = std::is_same<ER, double>::value;
  static_assert(!(STAGE && F64), "shared-memory staging is the mixed form's");
  typedef ShellStage<NPT> SG;
  const int nc = S.nc;
  {
    const int e = P.nft + il;
    // DT1 and DT1/MAX(DT1^2, EM20) are the same for every element: a caller
    // looping over elements passes them (DT1in >= 0) to form them once
    const double DT1 = DT1in >= 0.0 ? DT1in : T->dt2;
    const R dt1 = (R)DT1;
    const int tid = threadIdx.x;
    // the connectivity first: its loads head the gather chain, and the
    // staging below (asm with a memory clobber) would keep them behind it
    int nn[4];
#pragma unroll
    for (int k = 0; k < 4; k++) nn[k] = __ldg(S.ix + k * nc + e);
    // staged form: the whole element state is requested now, into this
    // thread's shared-memory slots, and waited for at its first use (CSTRA3).
    // A full warp whose 32 elements start on a 16-byte boundary copies them
    // cooperatively: each component of its 32 elements is 128 contiguous
    // bytes (SoA), 8 lanes x 16 bytes, so one instruction moves 4 components
    // (15 + 2 copies per thread for NPT = 5 instead of 59 of 4 or 8 bytes).
    const int lane = tid & 31;
    const int e0 = e - lane;
    const bool coop = STAGE && RG_SHELL_COOP_STAGE && ((e0 & 3) == 0) && ((nc & 3) == 0) &&
                      il - lane + 32 <= P.nel;
    if constexpr (STAGE) {
      constexpr int NT = SNT;
      if (coop) {
        __syncwarp();  // the warp's slots are free: its previous task read them
        const int wb = tid - lane;
        const int sub = lane & 7, grp = lane >> 3;
#pragma unroll
        for (int k = 0; k < (SG::nfloat + 3) / 4; k++) {
          const int q = 4 * k + grp;
          if (q < SG::nfloat) {
            const ER *b;
            if (q < SG_MOM) b = S.forc + q * nc;
            else if (q < SG_HOUR) b = S.mom + (q - SG_MOM) * nc;
            else if (q < SG_GSTR) b = S.hour + (q - SG_HOUR) * nc;
            else if (q < SG_SIG) b = S.gstr + (q - SG_GSTR) * nc;
            else if (q < SG::pla) b = S.sig + (q - SG_SIG) * nc;
            else if (q < SG::epsd) b = S.pla + (q - SG::pla) * nc;
            else b = S.epsd + (q - SG::epsd) * nc;
            cp_async16(stg + q * NT + wb + 4 * sub, b + e0 + 4 * sub);
          }
        }
        const int sub2 = lane & 15, grp2 = lane >> 4;
#pragma unroll
        for (int k = 0; k < 2; k++) {
          const int q = 2 * k + grp2;
          if (q < SG::ndouble) {
            const double *b = q == 0 ? S.eint : (q == 1 ? S.eint + nc : S.ehou);
            cp_async16(stgd + q * NT + wb + 2 * sub2, b + e0 + 2 * sub2);
          }
        }
      } else {
#pragma unroll
      for (int c = 0; c < 5; c++) cp_async4(stg + (SG_FORC + c) * NT + tid, S.forc + c * nc + e);
#pragma unroll
      for (int c = 0; c < 3; c++) cp_async4(stg + (SG_MOM + c) * NT + tid, S.mom + c * nc + e);
#pragma unroll
      for (int c = 0; c < 5; c++) cp_async4(stg + (SG_HOUR + c) * NT + tid, S.hour + c * nc + e);
#pragma unroll
      for (int c = 0; c < 8; c++) cp_async4(stg + (SG_GSTR + c) * NT + tid, S.gstr + c * nc + e);
#pragma unroll
      for (int c = 0; c < 5 * NPT; c++) cp_async4(stg + (SG_SIG + c) * NT + tid, S.sig + c * nc + e);
#pragma unroll
      for (int it = 0; it < NPT; it++) {
        cp_async4(stg + (SG::pla + it) * NT + tid, S.pla + it * nc + e);
        cp_async4(stg + (SG::epsd + it) * NT + tid, S.epsd + it * nc + e);
      }
      cp_async8(stgd + 0 * NT + tid, S.eint + e);
      cp_async8(stgd + 1 * NT + tid, S.eint + nc + e);
      cp_async8(stgd + 2 * NT + tid, S.ehou + e);
      }
      cp_async_commit();
    }
    // ---- CCOOR3 ----
    R vl[4][3], vrl[4][3];
    const R offg = S.offg[e];
    const R off = smin((R)RG_ONE, fabs(offg));
    const bool z0 = offg < (R)0;
    // coordinates: absolute (FP64) or node-1-relative from the FP32 hi/lo
    // copies (mixed); every quantity below uses coordinate differences only.
    R xg[4], yg[4], zg[4];
    if constexpr (F64) {
#pragma unroll
      for (int k = 0; k < 4; k++) {
        const dbl4 x = ld4(N.X4 + nn[k]);
        const dbl4 v = ld4(N.V4 + nn[k]);
        const dbl4 w = ld4(N.VR4 + nn[k]);
        xg[k] = x.x;
        yg[k] = x.y;
        zg[k] = x.z;
        vl[k][0] = z0 ? (R)0 : v.x;
        vl[k][1] = z0 ? (R)0 : v.y;
        vl[k][2] = z0 ? (R)0 : v.z;
        vrl[k][0] = z0 ? (R)0 : w.x;
        vrl[k][1] = z0 ? (R)0 : w.y;
        vrl[k][2] = z0 ? (R)0 : w.z;
      }
    } else {
      F8 c[4];
#pragma unroll
      for (int k = 0; k < 4; k++) {
        c[k] = ldF8(N.XF + nn[k]);
        const float4 v = ldf4(N.VF + nn[k]);
        const float4 w = ldf4(N.VRF + nn[k]);
        vl[k][0] = z0 ? 0.f : v.x;
        vl[k][1] = z0 ? 0.f : v.y;
        vl[k][2] = z0 ? 0.f : v.z;
        vrl[k][0] = z0 ? 0.f : w.x;
        vrl[k][1] = z0 ? 0.f : w.y;
        vrl[k][2] = z0 ? 0.f : w.z;
      }
#pragma unroll
      for (int k = 0; k < 4; k++) {
        xg[k] = (c[k].hx - c[0].hx) + (c[k].lx - c[0].lx);
        yg[k] = (c[k].hy - c[0].hy) + (c[k].ly - c[0].ly);
        zg[k] = (c[k].hz - c[0].hz) + (c[k].lz - c[0].lz);
      }
    }
    R thk0 = S.thke[e];
    // Element state read up front, ahead of the first store (the compiler
    // must assume the state arrays may alias): the loads overlap the gathers.
    R st_forc[5], st_mom[3], st_hour[5];
    double st_eint0 = 0.0, st_eint1 = 0.0, st_ehou = 0.0;
    if constexpr (!STAGE) {
#pragma unroll
      for (int c = 0; c < 5; c++) st_forc[c] = S.forc[c * nc + e];
#pragma unroll
      for (int c = 0; c < 3; c++) st_mom[c] = S.mom[c * nc + e];
#pragma unroll
      for (int c = 0; c < 5; c++) st_hour[c] = S.hour[c * nc + e];
      st_eint0 = S.eint[e];
      st_eint1 = S.eint[nc + e];
      st_ehou = S.ehou[e];
    }
    // ---- CNVEC3 ----
    R e1x, e1y, e1z, e2x, e2y, e2z, e3x, e3y, e3z;
    {
      const R x21 = xg[1] - xg[0], x32 = xg[2] - xg[1], x34 = xg[2] - xg[3], x41 = xg[3] - xg[0];
      const R y21 = yg[1] - yg[0], y32 = yg[2] - yg[1], y34 = yg[2] - yg[3], y41 = yg[3] - yg[0];
      const R z21 = zg[1] - zg[0], z32 = zg[2] - zg[1], z34 = zg[2] - zg[3], z41 = zg[3] - zg[0];
      e1x = (x21 + x34);
      e1y = (y21 + y34);
      e1z = (z21 + z34);
      e2x = (x32 + x41);
      e2y = (y32 + y41);
      e2z = (z32 + z41);
      e3x = e1y * e2z - e1z * e2y;
      e3y = e1z * e2x - e1x * e2z;
      e3z = e1x * e2y - e1y * e2x;
      if (P.ishfram == 2) {
        // version-4 non-symmetric frame (cnvec3.F:143-170): e1 scaled by
        // |e2|^2 and tilted by e2 x e3 (unit e3 not yet formed), e2 = e3 x e1
        R suma = e2x * e2x + e2y * e2y + e2z * e2z;
        e1x = e1x * suma + e2y * e3z - e2z * e3y;
        e1y = e1y * suma + e2z * e3x - e2x * e3z;
        e1z = e1z * suma + e2x * e3y - e2y * e3x;
        suma = e1x * e1x + e1y * e1y + e1z * e1z;
        suma = inv_norm_em20(suma);
        e1x = e1x * suma;
        e1y = e1y * suma;
        e1z = e1z * suma;
        suma = e3x * e3x + e3y * e3y + e3z * e3z;
        suma = inv_norm_em20(suma);
        e3x = e3x * suma;
        e3y = e3y * suma;
        e3z = e3z * suma;
        e2x = e3y * e1z - e3z * e1y;
        e2y = e3z * e1x - e3x * e1z;
        e2z = e3x * e1y - e3y * e1x;
        suma = e2x * e2x + e2y * e2y + e2z * e2z;
        suma = inv_norm_em20(suma);
        e2x = e2x * suma;
        e2y = e2y * suma;
        e2z = e2z * suma;
      } else {
        // symmetric convected frame (cnvec3.F:117-141)
        R suma = e3x * e3x + e3y * e3y + e3z * e3z;
        suma = inv_norm_em20(suma);
        e3x = e3x * suma;
        e3y = e3y * suma;
        e3z = e3z * suma;
        const R s1 = e1x * e1x + e1y * e1y + e1z * e1z;
        const R s2 = e2x * e2x + e2y * e2y + e2z * e2z;
        suma = sqrt_ratio(s1, s2);
        e1x = e1x + (e2y * e3z - e2z * e3y) * suma;
        e1y = e1y + (e2z * e3x - e2x * e3z) * suma;
        e1z = e1z + (e2x * e3y - e2y * e3x) * suma;
        suma = e1x * e1x + e1y * e1y + e1z * e1z;
        suma = inv_norm_em20(suma);
        e1x = e1x * suma;
        e1y = e1y * suma;
        e1z = e1z * suma;
        e2x = e3y * e1z - e3z * e1y;
        e2y = e3z * e1x - e3x * e1z;
        e2z = e3x * e1y - e3y * e1x;
      }
    }
    // ---- CDERI3 ----
    R x2, y2, x3, y3, x4, y4, px1, px2, py1, py2, area, inv_area, vhx, vhy;
    R area2_m56 = (R)0;  // FP64 form: CDLEN3's AREA^2 / MAX(AL5, AL6, EM20)
    {
      const R x21 = xg[1] - xg[0], y21 = yg[1] - yg[0], z21 = zg[1] - zg[0];
      const R x31 = xg[2] - xg[0], y31 = yg[2] - yg[0], z31 = zg[2] - zg[0];
      const R x41 = xg[3] - xg[0], y41 = yg[3] - yg[0], z41 = zg[3] - zg[0];
      x2 = e1x * x21 + e1y * y21 + e1z * z21;
      y2 = e2x * x21 + e2y * y21 + e2z * z21;
      y3 = e2x * x31 + e2y * y31 + e2z * z31;
      x3 = e1x * x31 + e1y * y31 + e1z * z31;
      x4 = e1x * x41 + e1y * y41 + e1z * z41;
      y4 = e2x * x41 + e2y * y41 + e2z * z41;
      px1 = (R)RG_HALF * (y2 - y4);
      py1 = (R)RG_HALF * (x4 - x2);
      px2 = (R)RG_HALF * y3;
      py2 = -(R)RG_HALF * x3;
      area = smax((R)RG_TWO * (py2 * px1 - py1 * px2), (R)RG_EM20);
      if constexpr (F64) {
        // 1/AREA and CDLEN3's AREA^2 / MAX(AL5, AL6, EM20) from one
        // reciprocal (FP64-pipe work)
        const R al5c = (x4 - x2) * (x4 - x2) + (y4 - y2) * (y4 - y2);
        const R al6c = x3 * x3 + y3 * y3;
        const R m56 = smax(smax(al5c, al6c), (R)RG_EM20);
        const R r = (R)RG_ONE / (area * m56);
        inv_area = m56 * r;
        area2_m56 = area * area * (area * r);
      } else {
        inv_area = (R)RG_ONE / area;
      }
      vhx = (-x2 + x3 - x4) * inv_area;
      vhy = (-y2 + y3 - y4) * inv_area;
    }
    // ---- CCOEF3: ITHK > 0 works on the current thickness, ITHK = 0 on the
    // initial one (THKE, ccoor3.F:80) ----
    const double thk_cur = S.thk[e];
    if (P.ithk > 0) thk0 = (R)thk_cur;
    const R vol0 = thk0 * area;
    const R thk02 = thk0 * thk0;
    const R nu = PC(nu), ym = PC(young), gmod = PC(g), a11 = PC(a11), ssp = PC(ssp),
            rho = PC(rho);
    R shf;
    if (P.shf_const) {
      shf = PC(shf0);  // NPT = 1: 0; ISH = 0: FSH
    } else {
      const R fac1tmp = (R)2.0 * ((R)1.0 + nu) * thk02;
      const R ish = PC(ish), fsh = PC(fsh);
      shf = fsh * ((R)1.0 - ish + ish * fac1tmp / (fsh * area + fac1tmp));
    }
    const R gs = gmod * shf;
    // ---- CDLEN3 (IHBE /= 0) ----
    R aldt;
    {
      const R al1 = x2 * x2 + y2 * y2;
      const R al2 = (x3 - x2) * (x3 - x2) + (y3 - y2) * (y3 - y2);
      const R al6 = x3 * x3 + y3 * y3;
      const R al3 = (x4 - x3) * (x4 - x3) + (y4 - y3) * (y4 - y3);
      const R al4 = x4 * x4 + y4 * y4;
      const R al5 = (x4 - x2) * (x4 - x2) + (y4 - y2) * (y4 - y2);
      R almin = smin(smin(al1, al2), al4);
      const R alquad = smin(smin(al3, al5), al6);
      if (al3 != (R)0) almin = smin(almin, alquad);
      R dtdyn;
      if constexpr (F64)
        dtdyn = area2_m56;
      else
        dtdyn = area * area / smax(smax(al5, al6), (R)RG_EM20);
      aldt = smax(dtdyn, almin);
      const R dthour = (R)RG_HALF * (almin + aldt) * PC(inv_hmax);
      if (dthour < aldt) aldt = dthour;
      aldt = sqrt(aldt);
    }
    // ---- CDEFO3 (IHBE <= 1) ----
    R vx[4], vy[4], vz[4];
#pragma unroll
    for (int k = 0; k < 4; k++) {
      vx[k] = e1x * vl[k][0] + e1y * vl[k][1] + e1z * vl[k][2];
      vy[k] = e2x * vl[k][0] + e2y * vl[k][1] + e2z * vl[k][2];
      vz[k] = e3x * vl[k][0] + e3y * vl[k][1] + e3z * vl[k][2];
    }
    R exx, eyy, exy, exz, eyz;
    {
      const R vz13 = vz[0] - vz[2], vz24 = vz[1] - vz[3];
      eyz = py1 * vz13 + py2 * vz24;
      exz = px1 * vz13 + px2 * vz24;
      const R dt1v4 = (R)RG_FOURTH * dt1;
      const R tmp2a = py2 + py1;
      const R tmp3a = copysign(smax(fabs(tmp2a), (R)RG_EM20), tmp2a);
      const R tmp1b = px2 - px1;
      const R tmp3b = copysign(smax(fabs(tmp1b), (R)RG_EM20), tmp1b);
      // FP64 form: the two divisions share one reciprocal (FP64-pipe work)
      R tmp1a, tmp2b;
      if constexpr (F64) {
        const R rab = (R)RG_ONE / (tmp3a * tmp3b);
        tmp1a = dt1v4 * (vz13 - vz24) * (vz13 - vz24) * (tmp3b * rab);
        tmp2b = dt1v4 * (vz13 + vz24) * (vz13 + vz24) * (tmp3a * rab);
      } else {
        tmp1a = dt1v4 * (vz13 - vz24) * (vz13 - vz24) / tmp3a;
        tmp2b = dt1v4 * (vz13 + vz24) * (vz13 + vz24) / tmp3b;
      }
      R vx13 = vx[0] - vx[2], vx24 = vx[1] - vx[3];
      vx13 = vx13 - tmp1a;
      vx24 = vx24 + tmp1a;
      exx = px1 * vx13 + px2 * vx24;
      exy = py1 * vx13 + py2 * vx24;
      R vy13 = vy[0] - vy[2], vy24 = vy[1] - vy[3];
      vy13 = vy13 + tmp2b;
      vy24 = vy24 + tmp2b;
      exy = exy + px1 * vy13 + px2 * vy24;
      eyy = py1 * vy13 + py2 * vy24;
    }
    // ---- CCURV3 ----
    R rx[4], ry[4], kxx, kyy, kxy;
#pragma unroll
    for (int k = 0; k < 4; k++) {
      rx[k] = e1x * vrl[k][0] + e1y * vrl[k][1] + e1z * vrl[k][2];
      ry[k] = e2x * vrl[k][0] + e2y * vrl[k][1] + e2z * vrl[k][2];
    }
    {
      const R rx13 = rx[0] - rx[2], rxav = rx[0] + rx[1] + rx[2] + rx[3], rx24 = rx[1] - rx[3];
      kyy = -py1 * rx13 - py2 * rx24;
      kxy = px1 * rx13 + px2 * rx24;
      const R ry13 = ry[0] - ry[2], ryav = ry[0] + ry[1] + ry[2] + ry[3], ry24 = ry[1] - ry[3];
      kxx = px1 * ry13 + px2 * ry24;
      kxy = py1 * ry13 + py2 * ry24 - kxy;
      exz = exz + ryav * ((R)0.25 * area);
      eyz = eyz - rxav * ((R)0.25 * area);
    }
    // ---- CSTRA3 ----
    {
      const R fac1 = dt1 * inv_area;
      exx = exx * fac1;
      eyy = eyy * fac1;
      exy = exy * fac1;
      eyz = eyz * fac1;
      exz = exz * fac1;
      kxx = kxx * fac1;
      kyy = kyy * fac1;
      kxy = kxy * fac1;
      const R inc[8] = {exx, eyy, exy, eyz, exz, kxx, kyy, kxy};
      if constexpr (STAGE) {
        cp_async_wait_all();
        if (coop) __syncwarp();  // the lanes' copies are the warp's
#pragma unroll
        for (int c = 0; c < 8; c++)
          S.gstr[c * nc + e] = stg[(SG_GSTR + c) * SNT + tid] + inc[c];
      } else {
#pragma unroll
        for (int c = 0; c < 8; c++) S.gstr[c * nc + e] = S.gstr[c * nc + e] + inc[c];
      }
    }
    // element strain rate (ASRATE = 1)
    R epsd_pg;
    {
      const R dtinv = DT1in >= 0.0 ? dtinv_in : dt1 / smax(dt1 * dt1, (R)RG_EM20);
      const R th = (R)thk_cur;  // GBUF%THK: the current thickness
      const R eps_k2 = (kxx * kxx + kyy * kyy + kxx * kyy + (R)RG_FOURTH * kxy * kxy) *
                       (R)RG_ONE_OVER_9 * th * th;
      const R eps_m2 =
          (R)RG_FOUR_OVER_3 * (exx * exx + eyy * eyy + exx * eyy + (R)RG_FOURTH * exy * exy);
      epsd_pg = sqrt(eps_k2 + eps_m2) * dtinv;
      S.epsdg[e] = epsd_pg;
    }
    // ---- CHVIS3 (ISMSTR = 4, IHBE = 1) and CDT3: they read no result of
    // the material update.  The staged (mixed) kernel runs them ahead of
    // MULAWC, so that the local velocities and rotation rates are dead before
    // the through-thickness loop; the FP64 kernel, held by its FP64 pipe,
    // keeps the reference's order.  Same operations either way. ----
    R h11, h12, h13, h21, h22, h23, h31, h32, h33, hr4, hr5;
    R sti_noda = (R)0, stir_noda = (R)0;
    R inv_divm = (R)0;  // FP64 form: 1 / MAX(ALDT^2, EM20), formed with HH2
    R sti;
    bool kill = false;  // deleted by the element time-step action (CDT3)
    auto hourglass_and_dt = [&]() {
    if constexpr (STAGE) {
#pragma unroll
      for (int c = 0; c < 5; c++) st_hour[c] = stg[(SG_HOUR + c) * SNT + tid];
      st_ehou = stgd[2 * SNT + tid];
    }
    {
      const R px1v = px1 * vhx, px2v = px2 * vhx, py1v = py1 * vhy, py2v = py2 * vhy;
      const R gama1 = off * ((R)RG_ONE - px1v - py1v);
      const R gama3 = off * ((R)RG_ONE + px1v + py1v);
      const R gama2 = off * (-(R)RG_ONE - px2v - py2v);
      const R gama4 = off * (-(R)RG_ONE + px2v + py2v);
      // HVLIN = 0: the linear viscous terms vanish; HVISC = HELAS = 1/2
      R A1, A3, A5, A7, A8;
      if (P.shf_const) {
        A1 = PC(hA1);
        A3 = PC(hA3);
        A5 = PC(hA5);
        A7 = PC(hA7);
        A8 = PC(hA8);
      } else {
        const R shfpr3 = shf / ((R)RG_THREE * ((R)RG_ONE + nu));
        const R r1 = (R)RG_FOURTH * rho * (R)RG_HUNDRED;
        A1 = r1 * ((R)RG_HALF * PC(h1));
        A3 = r1 * ((R)RG_HALF * PC(h2)) * sqrt(shfpr3);
        A5 = ((R)RG_HALF * PC(h3)) * r1 * (R)RG_ZEP072169;
        const R r0e = (R)RG_FOURTH * ym * (R)RG_HALF;
        A7 = PC(h1) * r0e;
        A8 = PC(h2) * r0e * shfpr3;
      }
      const R t2a = thk02 * area;
      const R tsa = sqrt(t2a);
      R h1q = A1 * tsa;
      R h2q = A3 * thk02;
      R h3q = A5 * t2a;
      const R td = thk0 * dt1;
      R hh1 = A7 * td;
      const R b1 = px1 * px1 + py1 * py1, b2 = px2 * px2 + py2 * py2;
      R hh2;
      if constexpr (F64) {
        // FP64 form: HH2's division and CDT3's 1 / MAX(ALDT^2, EM20) share
        // one reciprocal (FP64-pipe work)
        const R divm = smax(aldt * aldt, (R)RG_EM20);
        const R rq = (R)RG_ONE / ((b1 + b2) * divm);
        hh2 = A8 * thk02 * td * (divm * rq);
        inv_divm = (b1 + b2) > (R)0 ? (b1 + b2) * rq : (R)RG_ONE / divm;
      } else {
        hh2 = A8 * thk02 * td / (b1 + b2);
      }
      if (S.degen[e]) h1q = h2q = h3q = hh1 = hh2 = (R)0;
      if (P.nodadt) {
        // nodal time step (chvis3.F:198-265, IGTYP=1): the element
        // stiffness STI with the elastic hourglass term SCALE, and STIR
        // (VISCMX = 1, ALPE = 1; the linear hourglass terms are 0)
        const R scale = smax(smax(gama1 * gama1, gama2 * gama2), smax(gama3 * gama3, gama4 * gama4)) *
                        dt1 * smax(smax(hh1, hh2), (R)0) / smax(dt1 * dt1, (R)RG_EM20);
        if (off != (R)0) {
          sti_noda = (R)0 + scale;
          sti_noda = sti_noda + smax(b1, b2) * thk0 * a11 / area;
          stir_noda = sti_noda * (thk02 * (R)RG_ONE_OVER_12 + area * (R)RG_ONE_OVER_9);
        }
      }
      R hg1 = vx[0] * gama1 + vx[1] * gama2 + vx[2] * gama3 + vx[3] * gama4;
      R hg2 = vy[0] * gama1 + vy[1] * gama2 + vy[2] * gama3 + vy[3] * gama4;
      R hou0 = st_hour[0] + hg1 * hh1;
      R hou1 = st_hour[1] + hg2 * hh1;
      const R hour1a = hou0 + hg1 * ((R)0 + h1q * fabs(hg1));
      h11 = hour1a * gama1;
      h12 = hour1a * gama2;
      h13 = hour1a * gama3;
      const R hour2a = hou1 + hg2 * ((R)0 + h1q * fabs(hg2));
      h21 = hour2a * gama1;
      h22 = hour2a * gama2;
      h23 = hour2a * gama3;
      R ehou = hour1a * hg1 + hour2a * hg2;
      hg1 = vz[0] * gama1 + vz[1] * gama2 + vz[2] * gama3 + vz[3] * gama4;
      const R hou2 = st_hour[2] + hg1 * hh2;
      const R hour3a = hou2 + hg1 * ((R)0 + h2q * fabs(hg1));
      h31 = hour3a * gama1;
      h32 = hour3a * gama2;
      h33 = hour3a * gama3;
      ehou = ehou + hour3a * hg1;
      hg1 = rx[0] - rx[1] + rx[2] - rx[3];
      hg2 = ry[0] - ry[1] + ry[2] - ry[3];
      hr4 = hg1 * ((R)0 + h3q * fabs(hg1));
      hr5 = hg2 * ((R)0 + h3q * fabs(hg2));
      ehou = ehou + hr4 * hg1 + hr5 * hg2;
      ehou = dt1 * ehou * off;
      S.hour[0 * nc + e] = hou0;
      S.hour[1 * nc + e] = hou1;
      S.hour[2 * nc + e] = hou2;
      S.hour[3 * nc + e] = hr4;
      S.hour[4 * nc + e] = hr5;
      S.ehou[e] = st_ehou + (double)ehou;
    }
    // ---- CDT3 (not called under the nodal time step, cforc3.F:668) ----
    sti = sti_noda;
    if (!P.nodadt) {
      const R dt = aldt * PC(dtfac_ssp);
      // IDTMIN(3) (cdt3.F:77-141), ahead of the step minimum: an element of
      // OFF = 1 whose step is at or below DTMIN1(3) stops the run (1, 5) or
      // is deleted (2): OFF = 0 from here on -- out of the minimum, STI = 0,
      // OFFG = 0 kept by CUPDT3P; its forces of this cycle are still
      // assembled (CFINT3 does not read OFF)
      R offd = off;
      if (P.idtmin && !(dt > PC(dtmin)) && off >= (R)RG_ONE && offg >= (R)0) {
        if (P.idtmin == 2) {
          offd = (R)0;
          kill = true;
        } else if (status_dt) {
          atomicOr(status_dt, RG_ST_DTMIN);
        }
      }
      if (offg > (R)0 && offd != (R)0) {
        // running minimum; reversed order key: the first element wins ties
        // (strict < in CDT3)
        dt_pair_min_t(dtmine, elmin, dt, key0 + (nc_total - 1 - e));
      }
      if constexpr (F64) {
        sti = (R)RG_HALF * vol0 * ym * inv_divm;
      } else {
        const R divm = smax(aldt * aldt, (R)RG_EM20);
        sti = (R)RG_HALF * vol0 * ym / divm;
      }
      sti = (R)RG_ZEP81 * sti * offd;
    }
    };
    if constexpr (STAGE) hourglass_and_dt();
    // ---- MULAWC: through-thickness loop (SIGEPS02C / M2CPLR) ----
    R forn[5] = {0, 0, 0, 0, 0}, momn[3] = {0, 0, 0};
    if constexpr (STAGE) {
#pragma unroll
      for (int c = 0; c < 5; c++) st_forc[c] = stg[(SG_FORC + c) * SNT + tid];
#pragma unroll
      for (int c = 0; c < 3; c++) st_mom[c] = stg[(SG_MOM + c) * SNT + tid];
    }
    R degmb = st_forc[0] * exx + st_forc[1] * eyy + st_forc[2] * exy + st_forc[3] * eyz +
              st_forc[4] * exz;
    R degfx = st_mom[0] * kxx + st_mom[1] * kyy + st_mom[2] * kxy;
    double thkn = thk_cur;
    R asrate = (R)RG_ONE;
    if (P.israte > 0) {
      if constexpr (F64)
        asrate = smin((R)RG_ONE, (R)(P.pm9 * DT1));
      else
        asrate = smin(1.f, P.f.pm9 * dt1);
    }
    const R a1 = PC(a1);
    const R a2 = PC(a2);
    const R epdr = smax(PC(eps0) * dt1, (R)RG_EM20);
    // LOG(EPSP/EPDR) of the previous point: the points usually share one
    // strain rate (ASRATE = 1), and an equal argument gives the same value
    R memo_epsp = (R)-1, memo_log = (R)0;
    R sigy_acc = (R)0;  // SIGY: YLD / NPT summed over the points so far
    // point state: point it+1 is loaded while point it is computed
    R nx_sig[5], nx_ep = (R)0, nx_pla = (R)0;
    if constexpr (!STAGE) {
#pragma unroll
      for (int c = 0; c < 5; c++) nx_sig[c] = S.sig[(c)*nc + e];
      nx_ep = S.epsd[e];
      nx_pla = S.pla[e];
    }
    // the FP64 form runs the points as a loop (fully unrolled it spilled at
    // 255 registers: 0.250 -> 0.244 ms on the crash box, same bits); the
    // FP32 form unrolled (a loop was slower, 36.8 -> 37.4 us)
#pragma unroll(F64 ? 1 : NPT)
    for (int it = 0; it < NPT; it++) {
      R sn[5];
      R ep, pla_in;
      if constexpr (STAGE) {
        // the staged point state (shared memory, this thread's slots)
#pragma unroll
        for (int c = 0; c < 5; c++) sn[c] = stg[(SG_SIG + it * 5 + c) * SNT + tid];
        ep = stg[(SG::epsd + it) * SNT + tid];
        pla_in = stg[(SG::pla + it) * SNT + tid];
      } else {
#pragma unroll
        for (int c = 0; c < 5; c++) sn[c] = nx_sig[c];
        ep = nx_ep;
        pla_in = nx_pla;
        if (it + 1 < NPT) {
          const int q5 = ((it + 1) * 5) * nc + e;
#pragma unroll
          for (int c = 0; c < 5; c++) nx_sig[c] = S.sig[q5 + c * nc];
          nx_ep = S.epsd[(it + 1) * nc + e];
          nx_pla = S.pla[(it + 1) * nc + e];
        }
      }
      const R thkly = pcoef<R>(c_wfd[NPT - 1][it], c_wf[NPT - 1][it]);
      const R thklyl = thkly * thk0;
      const R wmc = pcoef<R>(c_wmd[NPT - 1][it], c_wm[NPT - 1][it]);
      const R zt = pcoef<R>(c_z0d[NPT - 1][it], c_z0[NPT - 1][it]) * thk0;
      const R depsxx = exx + zt * kxx;
      const R depsyy = eyy + zt * kyy;
      const R depsxy = exy + zt * kxy;
      const int ip5 = (it * 5) * nc + e;
      R epsdot;
      if (P.vp == 2) {
        ep = asrate * epsd_pg + ((R)RG_ONE - asrate) * ep;
        S.epsd[it * nc + e] = ep;
        epsdot = ep * dt1;
      } else {
        epsdot = ep * dt1;
      }
      R ezz = (R)0;
      R ca = PC(ca), cb = PC(cb), ymax = PC(ymax);
      // T* of the point (sigeps02c.F:125), 0 without adiabatic heating
      R tstar = (R)0;
      if ((MF & 2) && P.thermal) tstar = smax((R)0, (S.temp[it * nc + e] - PC(tref)) / (PC(tmelt) - PC(tref)));
      // kinematic hardening: the predictor works on the shifted stress
      // (m2cplr.F:115-121)
      const bool kin = (MF & 1) && P.fisokin > 0.0;
      R sgb[3] = {(R)0, (R)0, (R)0};
      if (kin) {
#pragma unroll
        for (int c = 0; c < 3; c++) {
          sgb[c] = S.sigbak[(it * 3 + c) * nc + e];
          sn[c] = sn[c] - sgb[c];
        }
      }
      sn[0] = sn[0] + a1 * depsxx + a2 * depsyy;
      sn[1] = sn[1] + a2 * depsxx + a1 * depsyy;
      sn[2] = sn[2] + gmod * depsxy;
      sn[3] = sn[3] + gs * eyz;
      sn[4] = sn[4] + gs * exz;
      if (P.f.cc_nz) {
        R epsp = epsdot;
        if (P.israte == 0 && P.vp == 2)
          epsp = smax(smax(fabs(depsxx), fabs(depsyy)), (R)RG_HALF * fabs(depsxy));
        epsp = smax(epsp, epdr);
        R logep;
        if (epsp == memo_epsp) {
          logep = memo_log;
        } else {
          logep = log(epsp / epdr);
          memo_epsp = epsp;
          memo_log = logep;
        }
        R q = ((R)RG_ONE + PC(cc) * logep);
        if (tstar != (R)0) q = q * ((R)RG_ONE - exp(PC(m_exp) * log(tstar)));
        q = smax(q, (R)RG_EM20);
        ca = ca * q;
        cb = cb * q;
        if (P.icc == 1) ymax = ymax * q;
      } else if (tstar != (R)0) {
        // CC = 0: thermal softening alone (m2cplr.F:169-178)
        R q = (R)RG_ONE - exp(PC(m_exp) * log(tstar));
        q = smax(q, (R)RG_EM20);
        ca = ca * q;
        cb = cb * q;
      }
      R pla = pla_in;
      R yld;
      if (kin)
        yld = pla == (R)0 ? ca : ca + cb * ((R)RG_ONE - PC(fisokin)) * exp(PC(cn) * log(pla));
      else
        yld = pla == (R)0 ? ca : ca + cb * exp(PC(cn) * log(pla));
      yld = smin(yld, ymax);
      R h = (R)0, dpla_pt = (R)0;  // hardening modulus and DPLA of the point
      if (P.ipla == 0) {
        const R svm = sqrt(sn[0] * sn[0] + sn[1] * sn[1] - sn[0] * sn[1] + (R)RG_THREE * sn[2] * sn[2]);
        const R r = smin((R)RG_ONE, yld / (svm + (R)RG_EM15));
        if (r < (R)RG_ONE) {
          sn[0] = sn[0] * r;
          sn[1] = sn[1] * r;
          sn[2] = sn[2] * r;
          const R dpla = off * smax((R)0, (svm - yld) / ym);
          const R s1 = (R)RG_HALF * (sn[0] + sn[1]);
          ezz = dpla * s1 / yld;
          pla = pla + dpla;
          dpla_pt = dpla;
          if (kin && yld < ymax) h = PC(cn) * cb * exp((PC(cn) - (R)RG_ONE) * log(pla + (R)RG_EM07));
        }
      } else if ((MF & 4) && P.ipla == 2) {
        // m2cplr.F:380-445: projection along an approximate normal, then a
        // radial return to the yield stress advanced by H * DPLA
        const R svm2 = sn[0] * sn[0] + sn[1] * sn[1] - sn[0] * sn[1] + (R)RG_THREE * sn[2] * sn[2];
        const R yld2 = yld * yld;
        if (svm2 > yld2 && off == (R)RG_ONE) {
          const R svm = sqrt(svm2);
          h = yld >= ymax ? (R)0 : PC(cn) * cb * exp((PC(cn) - (R)RG_ONE) * log(pla + (R)RG_EM07));
          const R aa = (svm2 - yld2) /
                       ((R)RG_FIVE * svm2 + (R)RG_THREE * (-(sn[0] * sn[1]) + sn[2] * sn[2]));
          const R s1 = ((R)RG_ONE - (R)RG_TWO * aa) * sn[0] + aa * sn[1];
          const R s2 = aa * sn[0] + ((R)RG_ONE - (R)RG_TWO * aa) * sn[1];
          const R s3 = ((R)RG_ONE - (R)RG_THREE * aa) * sn[2];
          sn[0] = s1;
          sn[1] = s2;
          sn[2] = s3;
          const R dpla = off * (svm - yld) / ((R)RG_THREE * gmod + h);
          pla = pla + dpla;
          yld = yld + h * dpla;
          dpla_pt = dpla;
          const R svmn = sqrt(sn[0] * sn[0] + sn[1] * sn[1] - sn[0] * sn[1] + (R)RG_THREE * sn[2] * sn[2]);
          const R r = smin((R)RG_ONE, yld / smax((R)RG_EM20, svmn));
          sn[0] = sn[0] * r;
          sn[1] = sn[1] * r;
          sn[2] = sn[2] * r;
          ezz = dpla * (R)RG_HALF * (sn[0] + sn[1]) / yld;
        }
      } else {
        const R s1 = sn[0] + sn[1];
        const R s2 = sn[0] - sn[1];
        const R s3 = sn[2];
        const R A = (R)RG_FOURTH * s1 * s1;
        const R B = (R)RG_THREE_OVER_4 * s2 * s2 + (R)RG_THREE * s3 * s3;
        // SVM > YLD tested on the squares (YLD >= 0): the square root is
        // only taken at yielding points
        if (A + B > yld * yld && off == (R)RG_ONE) {
          const R svm = sqrt(A + B);
          const R nu1 = PC(inv1mnu);
          const R nu2 = PC(inv1pnu);
          h = yld >= ymax ? (R)0 : PC(cn) * cb * exp((PC(cn) - (R)RG_ONE) * log(pla + (R)RG_EM07));
          R dpla_j = (svm - yld) / ((R)RG_THREE * gmod + h);
          // isotropic Newton (FISOKIN = 0), or the kinematic / mixed one with
          // modified NU1, NU2 and the isotropic part of H (m2cplr.F:324-336)
          R anu1 = A * nu1;
          R bnu2 = (R)RG_THREE * B * nu2;
          R h2 = (R)RG_TWO * h;
          R nu11 = (R)0, nu21 = (R)0, beta = (R)RG_ONE;
          if (kin) {
            const R bh = h * PC(fisokin);
            const R hi = h - bh;
            const R hk = (R)RG_TWO_THIRD * bh;
            const R aaa = (R)RG_THREE * hk / ym;
            nu11 = nu1 + aaa;
            nu21 = (R)RG_THREE * nu2 + aaa;
            anu1 = A * nu11;
            bnu2 = B * nu21;
            h2 = (R)RG_TWO * hi;
            beta = (R)RG_ONE - PC(fisokin);
          }
          R dpla_i = 0, Pp = 1, Qq = 1, dr = 0;
#pragma unroll
          for (int n = 0; n < 3; n++) {
            dpla_i = dpla_j;
            const R pla_i = pla + dpla_i;
            R yld_i;
            if (pla_i == (R)0)
              yld_i = smin(ymax, ca);
            else if (kin)
              yld_i = smin(ymax, ca + beta * cb * exp(PC(cn) * log(pla_i)));
            else
              yld_i = smin(ymax, ca + cb * exp(PC(cn) * log(pla_i)));
            // FP64 form: the two divisions by YLD_I, and P and Q, each from
            // one reciprocal (FP64-pipe work of the plastic points)
            R inv_y = (R)0;
            if constexpr (F64) {
              inv_y = (R)RG_ONE / yld_i;
              dr = (R)RG_HALF * ym * dpla_i * inv_y;
              const R dp = (R)RG_ONE + dr * (kin ? nu11 : nu1);
              const R dq = kin ? (R)RG_ONE + dr * nu21 : (R)RG_ONE + (R)RG_THREE * dr * nu2;
              const R rpq = (R)RG_ONE / (dp * dq);
              Pp = dq * rpq;
              Qq = dp * rpq;
            } else {
              dr = (R)RG_HALF * ym * dpla_i / yld_i;
              Pp = (R)RG_ONE / ((R)RG_ONE + dr * (kin ? nu11 : nu1));
              Qq = kin ? (R)RG_ONE / ((R)RG_ONE + dr * nu21)
                       : (R)RG_ONE / ((R)RG_ONE + (R)RG_THREE * dr * nu2);
            }
            const R p2 = Pp * Pp, q2 = Qq * Qq;
            const R f = A * p2 + B * q2 - yld_i * yld_i;
            R df;
            if constexpr (F64)
              df = -(anu1 * p2 * Pp + bnu2 * q2 * Qq) * (ym - dr * h2) * inv_y - h2 * yld_i;
            else
              df = -(anu1 * p2 * Pp + bnu2 * q2 * Qq) * (ym - dr * h2) / yld_i - h2 * yld_i;
            dpla_j = dpla_i > (R)0 ? smax((R)0, dpla_i - f / df) : (R)0;
          }
          pla = pla + dpla_i;
          dpla_pt = dpla_i;
          const R t1 = (sn[0] + sn[1]) * Pp;
          const R t2 = (sn[0] - sn[1]) * Qq;
          sn[0] = (R)RG_HALF * (t1 + t2);
          sn[1] = (R)RG_HALF * (t1 - t2);
          sn[2] = sn[2] * Qq;
          ezz = dr * t1 / ym;
          // kinematic: YLD from the new PLA, H kept (m2cplr.F:465-476)
          if (kin) yld = pla == (R)0 ? ca : smin(ymax, ca + beta * cb * exp(PC(cn) * log(pla)));
        }
      }
      // kinematic / mixed hardening: back stress update, stress shifted back
      // (m2cplr.F:477-490)
      if (kin) {
        const R alpha = PC(fisokin) * h * dpla_pt / yld;
#pragma unroll
        for (int c = 0; c < 3; c++) {
          sgb[c] = sgb[c] + alpha * sn[c];
          sn[c] = sn[c] + sgb[c];
          S.sigbak[(it * 3 + c) * nc + e] = sgb[c];
        }
      }
      // SIGEPS02C: SIGY accumulates YLD / NPT over the points so far, and
      // this point's adiabatic heating uses that running sum
      // (sigeps02c.F:197-199, 226-229; SIGY zeroed per group, mulawc.F90:577)
      if ((MF & 2) && P.thermal) {
        sigy_acc = sigy_acc + yld / (R)NPT;
        S.temp[it * nc + e] = S.temp[it * nc + e] + sigy_acc * dpla_pt / PC(rhocp);
      }
      S.pla[it * nc + e] = pla;
      ezz = -(depsxx + depsyy) * nu - ((R)RG_ONE - (R)RG_TWO * nu) * ezz;
      ezz = ezz * PC(inv1mnu);
      thkn = thkn + (double)(ezz * thklyl * off);
#pragma unroll
      for (int c = 0; c < 5; c++) {
        S.sig[ip5 + c * nc] = sn[c];
        forn[c] = forn[c] + thkly * sn[c];
      }
      momn[0] = momn[0] + wmc * sn[0];
      momn[1] = momn[1] + wmc * sn[1];
      momn[2] = momn[2] + wmc * sn[2];
    }
    S.thk[e] = thkn > RG_EM30 ? thkn : RG_EM30;
    if (P.f.dm_nz) {
      const R dtinv = DT1in >= 0.0 ? dtinv_in : dt1 / smax(dt1 * dt1, (R)RG_EM20);
      const R visc = ((R)RG_ONEP414 * PC(dm)) * ssp * sqrt(area) * dtinv * rho;
      forn[0] = forn[0] + visc * (exx + (R)RG_HALF * eyy);
      forn[1] = forn[1] + visc * (eyy + (R)RG_HALF * exx);
      forn[2] = forn[2] + visc * exy * (R)RG_THIRD;
    }
#pragma unroll
    for (int c = 0; c < 5; c++) forn[c] = forn[c] * off;
#pragma unroll
    for (int c = 0; c < 3; c++) momn[c] = momn[c] * off;
    degmb = degmb + forn[0] * exx + forn[1] * eyy + forn[2] * exy + forn[3] * eyz + forn[4] * exz;
    degfx = degfx + momn[0] * kxx + momn[1] * kyy + momn[2] * kxy;
    if constexpr (STAGE) {
      st_eint0 = stgd[0 * SNT + tid];
      st_eint1 = stgd[1 * SNT + tid];
    }
    {
      const R vol2 = (R)RG_HALF * vol0;
      S.eint[e] = st_eint0 + (double)(degmb * vol2);
      S.eint[nc + e] = st_eint1 + (double)(degfx * thk0 * vol2);
    }
#pragma unroll
    for (int c = 0; c < 5; c++) S.forc[c * nc + e] = forn[c];
#pragma unroll
    for (int c = 0; c < 3; c++) S.mom[c * nc + e] = momn[c];
    if constexpr (!STAGE) hourglass_and_dt();
    // ---- CFINT3 ----
    R F[3][4], M[3][4];
    {
      const R f1a = forn[0] * thk0, f2a = forn[1] * thk0, f3a = forn[2] * thk0;
      const R f4a = forn[3] * thk0, f5a = forn[4] * thk0;
      R m4 = f4a * area, m5 = f5a * area;
      const R f12 = f1a * px2 + f3a * py2;
      const R f22 = f2a * py2 + f3a * px2;
      const R f32 = f5a * px2 + f4a * py2;
      const R f11 = f1a * px1 + f3a * py1;
      const R f21 = f2a * py1 + f3a * px1;
      const R f31 = f5a * px1 + f4a * py1;
      const R g11 = f11 + h11, g13 = h13 - f11;
      const R g21 = f21 + h21, g23 = h23 - f21;
      const R g31 = f31 + h31, g33 = h33 - f31;
      const R g12 = f12 + h12, g22 = f22 + h22, g32 = f32 + h32;
      F[0][0] = e1x * g11 + e2x * g21 + e3x * g31;
      F[0][1] = e1x * g12 + e2x * g22 + e3x * g32;
      F[0][2] = e1x * g13 + e2x * g23 + e3x * g33;
      F[1][0] = e1y * g11 + e2y * g21 + e3y * g31;
      F[1][1] = e1y * g12 + e2y * g22 + e3y * g32;
      F[1][2] = e1y * g13 + e2y * g23 + e3y * g33;
      F[2][0] = e1z * g11 + e2z * g21 + e3z * g31;
      F[2][1] = e1z * g12 + e2z * g22 + e3z * g32;
      F[2][2] = e1z * g13 + e2z * g23 + e3z * g33;
#pragma unroll
      for (int c = 0; c < 3; c++) F[c][3] = -F[c][0] - F[c][1] - F[c][2];
      const R m1a = momn[0] * thk02, m2a = momn[1] * thk02, m3a = momn[2] * thk02;
      m4 = m4 * (R)RG_FOURTH;
      m5 = m5 * (R)RG_FOURTH;
      const R m11 = -m2a * py1 - m3a * px1;
      const R m21 = m1a * px1 + m3a * py1;
      const R m12 = -m2a * py2 - m3a * px2;
      const R m22 = m1a * px2 + m3a * py2;
      const R b1x[4] = {hr4 * off, -hr4 * off, hr4 * off, -hr4 * off};
      const R b2x[4] = {hr5 * off, -hr5 * off, hr5 * off, -hr5 * off};
      const R gg1[4] = {m11 - m4 + b1x[0], m12 - m4 + b1x[1], -m11 - m4 + b1x[2], -m12 - m4 + b1x[3]};
      const R gg2[4] = {m21 + m5 + b2x[0], m22 + m5 + b2x[1], -m21 + m5 + b2x[2], -m22 + m5 + b2x[3]};
#pragma unroll
      for (int k = 0; k < 4; k++) {
        M[0][k] = e1x * gg1[k] + e2x * gg2[k];
        M[1][k] = e1y * gg1[k] + e2y * gg2[k];
        M[2][k] = e1z * gg1[k] + e2z * gg2[k];
      }
    }
    // ---- CUPDT3P ----
    R offg_new = offg;
    if (kill) {
      offg_new = (R)0;
      S.offg[e] = (R)0;
    } else if (off < (R)RG_ONE) {
      offg_new = off;
      S.offg[e] = off;
    }
    const bool zero = offg_new < (R)0;
#pragma unroll
    for (int k = 0; k < 4; k++) {
      const int K = __ldg(S.iadc + k * nc + e);
      typename SlotT<ER>::type a, b;
      a.x = zero ? (R)0 : -F[0][k];
      a.y = zero ? (R)0 : -F[1][k];
      a.z = zero ? (R)0 : -F[2][k];
      a.w = zero ? (R)0 : sti;
      b.x = zero ? (R)0 : -M[0][k];
      b.y = zero ? (R)0 : -M[1][k];
      b.z = zero ? (R)0 : -M[2][k];
      b.w = zero ? (R)0 : stir_noda;  // STIR: 0 under the element time step
      fsky[K] = a;
      fskyr[K] = b;
    }
  }
}

}  // namespace rg
