// One-point hexa element kernel of the explicit cycle (SFORC3 chain).
//
// One thread per element, SoA element state, 32-byte node records gathered
// through the read-only path.  The arithmetic follows, step by step and in
// the same expression order, the reference routines cited at each block
// (paths relative to the OpenRadioss source tree):
//   SCOOR3  gather                     elements/solid/solide/scoor3.F:38
//   SDERI3  Jacobian, volume, PX, PH   elements/solid/solide/sderi3.F:32-339
//   SDLEN3  characteristic length      elements/solid/solide/sdlen3.F:39-172
//   SDEFO3  strain rate, spin          elements/solid/solide/sdefo3.F:32-313
//   SRHO3   density, DVOL              elements/solid/solide/srho3.F:140-150
//   SROTA3  Jaumann rotation           elements/solid/solide/srota3.F:40
//   M1LAW / M2LAW + MQVISCB            materials/mat/mat001/m1law.F:35,
//                                      materials/mat/mat002/m2law.F:38,
//                                      materials/mat_share/mqviscb.F:44
//   SHVIS3  viscous hourglass          elements/solid/solide/shvis3.F:31
//   SFINT3  internal forces            elements/solid/solide/sfint3.F:257
//   SCUMU3P PARITH/ON slot writes      elements/solid/solide/scumu3p.F:37
//
// Two arithmetic forms come from one template:
//   ER = double : the plain form, everything in FP64, absolute coordinates;
//   ER = float  : strain, stress, hourglass and material in FP32 on
//                 coordinates taken relative to node 1 in FP64; the volume
//                 (Jacobian determinant), density, DVOL and the energy
//                 increments stay in FP64, like the reference's own
//                 double-precision volume shadow (VOLDP / IRESP=1,
//                 srho3.F:230-250).
#include "rg_device.cuh"
#include "rg_kernels.h"

#include <type_traits>

namespace rg {

template <typename T>
__device__ __forceinline__ T rmax(T a, T b) {
  return a > b ? a : (b != b ? b : a);
}
template <typename T>
__device__ __forceinline__ T rmin(T a, T b) {
  return a < b ? a : (b != b ? b : a);
}

// Fortran MAX/MIN with the argument order of the source: MAX(a,b) returns
// a if a>b, else b (NaN propagation is not relied on).
template <typename T>
__device__ __forceinline__ T fmax_(T a, T b) {
  return a > b ? a : b;
}
template <typename T>
__device__ __forceinline__ T fmin_(T a, T b) {
  return a < b ? a : b;
}

template <typename ER, int LAW, int NT>
__global__ void __launch_bounds__(NT)
hexa_kernel(const HexaParams P, const HexaArrays<ER> A, const NodeView N,
            typename SlotT<ER>::type *__restrict__ fsky, DtPartials dp,
            const Time *__restrict__ T, int *__restrict__ status) {
  typedef ER R;
  constexpr bool F64 = std::is_same<ER, double>::value;
  const int il = blockIdx.x * NT + threadIdx.x;
  const int ne = A.ne;
  double dtmine = RG_EP06;
  int elmin = -1;

  if (il < P.nel) {
    const int e = P.nft + il;
    const double DT1 = T->dt2;  // DT1 = DT2 of the previous cycle
    const R dt1 = (R)DT1;

    // ---- SCOOR3 gather ---------------------------------------------------
    int nc[8];
#pragma unroll
    for (int k = 0; k < 8; k++) nc[k] = __ldg(A.nc + k * ne + e);
    const R offg0 = A.off[e];
    R offg = offg0;
    R off = fabs(offg0);
    double xa[8], ya[8], za[8];
    R vx[8], vy[8], vz[8];
#pragma unroll
    for (int k = 0; k < 8; k++) {
      const dbl4 x = ld4(N.X4 + nc[k]);
      const dbl4 v = ld4(N.V4 + nc[k]);
      xa[k] = x.x;
      ya[k] = x.y;
      za[k] = x.z;
      if (offg0 < (R)0) {
        vx[k] = vy[k] = vz[k] = (R)0;
      } else {
        vx[k] = (R)v.x;
        vy[k] = (R)v.y;
        vz[k] = (R)v.z;
      }
    }
    // geometry in the element type: absolute (FP64) or relative to node 1
    R x[8], y[8], z[8];
#pragma unroll
    for (int k = 0; k < 8; k++) {
      if (F64) {
        x[k] = (R)xa[k];
        y[k] = (R)ya[k];
        z[k] = (R)za[k];
      } else {
        x[k] = (R)(xa[k] - xa[0]);
        y[k] = (R)(ya[k] - ya[0]);
        z[k] = (R)(za[k] - za[0]);
      }
    }

    // ---- SDERI3 ------------------------------------------------------------
    R px[4], py[4], pz[4], ph[4][3];
    double voln;  // VOLDP: FP64 in both forms
    {
      const R x17 = x[6] - x[0], x28 = x[7] - x[1], x35 = x[4] - x[2], x46 = x[5] - x[3];
      const R y17 = y[6] - y[0], y28 = y[7] - y[1], y35 = y[4] - y[2], y46 = y[5] - y[3];
      const R z17 = z[6] - z[0], z28 = z[7] - z[1], z35 = z[4] - z[2], z46 = z[5] - z[3];
      const R jac1 = x17 + x28 - x35 - x46;
      const R jac2 = y17 + y28 - y35 - y46;
      const R jac3 = z17 + z28 - z35 - z46;
      const R x_17_46 = x17 + x46, x_28_35 = x28 + x35;
      const R y_17_46 = y17 + y46, y_28_35 = y28 + y35;
      const R z_17_46 = z17 + z46, z_28_35 = z28 + z35;
      const R jac4 = x_17_46 + x_28_35, jac5 = y_17_46 + y_28_35, jac6 = z_17_46 + z_28_35;
      const R jac7 = x_17_46 - x_28_35, jac8 = y_17_46 - y_28_35, jac9 = z_17_46 - z_28_35;
      const R j5968 = jac5 * jac9 - jac6 * jac8;
      const R j6749 = jac6 * jac7 - jac4 * jac9;
      const R j4857 = jac4 * jac8 - jac5 * jac7;
      double det;
      if (F64) {
        det = RG_ONE_OVER_64 * ((double)jac1 * (double)j5968 + (double)jac2 * (double)j6749 +
                                (double)jac3 * (double)j4857);
      } else {
        // FP64 determinant from FP64 relative coordinates (VOLDP)
        const double X17 = xa[6] - xa[0], X28 = xa[7] - xa[1], X35 = xa[4] - xa[2], X46 = xa[5] - xa[3];
        const double Y17 = ya[6] - ya[0], Y28 = ya[7] - ya[1], Y35 = ya[4] - ya[2], Y46 = ya[5] - ya[3];
        const double Z17 = za[6] - za[0], Z28 = za[7] - za[1], Z35 = za[4] - za[2], Z46 = za[5] - za[3];
        const double J1 = X17 + X28 - X35 - X46, J2 = Y17 + Y28 - Y35 - Y46, J3 = Z17 + Z28 - Z35 - Z46;
        const double J4 = (X17 + X46) + (X28 + X35), J5 = (Y17 + Y46) + (Y28 + Y35),
                     J6 = (Z17 + Z46) + (Z28 + Z35);
        const double J7 = (X17 + X46) - (X28 + X35), J8 = (Y17 + Y46) - (Y28 + Y35),
                     J9 = (Z17 + Z46) - (Z28 + Z35);
        det = RG_ONE_OVER_64 * (J1 * (J5 * J9 - J6 * J8) + J2 * (J6 * J7 - J4 * J9) +
                                J3 * (J4 * J8 - J5 * J7));
      }
      // SCHKJABT3: a live element with a non-positive volume is switched
      // off and the run is flagged (INEG_V = 0 stops the run).
      if (off == (R)0) {
        det = RG_ONE;
      } else if (det <= RG_ZERO) {
        det = RG_ONE;
        off = (R)0;
        offg = (R)0;
        A.off[e] = (R)0;
        atomicOr(status, 1);
      }
      voln = det;
      const R dett = (R)(RG_ONE_OVER_64 / det);
      const R jaci1 = dett * j5968;
      const R jaci4 = dett * j6749;
      const R jaci7 = dett * j4857;
      const R jaci2 = dett * (jac3 * jac8 - jac2 * jac9);
      const R jaci5 = dett * (jac1 * jac9 - jac3 * jac7);
      const R jaci8 = dett * (jac2 * jac7 - jac1 * jac8);
      const R jaci3 = dett * (jac2 * jac6 - jac3 * jac5);
      const R jaci6 = dett * (jac3 * jac4 - jac1 * jac6);
      const R jaci9 = dett * (jac1 * jac5 - jac2 * jac4);
      R jac12 = jaci1 + jaci2, jac45 = jaci4 + jaci5, jac78 = jaci7 + jaci8;
      px[0] = -jac12 - jaci3;
      py[0] = -jac45 - jaci6;
      pz[0] = -jac78 - jaci9;
      px[1] = -jac12 + jaci3;
      py[1] = -jac45 + jaci6;
      pz[1] = -jac78 + jaci9;
      jac12 = jaci1 - jaci2;
      jac45 = jaci4 - jaci5;
      jac78 = jaci7 - jaci8;
      px[2] = jac12 + jaci3;
      py[2] = jac45 + jaci6;
      pz[2] = jac78 + jaci9;
      px[3] = jac12 - jaci3;
      py[3] = jac45 - jaci6;
      pz[3] = jac78 - jaci9;
      // hourglass projections (JHBE /= 0)
      R hx = (x[0] - x[1] + x[2] - x[3] + x[4] - x[5] + x[6] - x[7]);
      R hy = (y[0] - y[1] + y[2] - y[3] + y[4] - y[5] + y[6] - y[7]);
      R hz = (z[0] - z[1] + z[2] - z[3] + z[4] - z[5] + z[6] - z[7]);
#pragma unroll
      for (int k = 0; k < 4; k++) ph[k][0] = px[k] * hx + py[k] * hy + pz[k] * hz;
      hx = (x[0] + x[1] - x[2] - x[3] - x[4] - x[5] + x[6] + x[7]);
      hy = (y[0] + y[1] - y[2] - y[3] - y[4] - y[5] + y[6] + y[7]);
      hz = (z[0] + z[1] - z[2] - z[3] - z[4] - z[5] + z[6] + z[7]);
#pragma unroll
      for (int k = 0; k < 4; k++) ph[k][1] = px[k] * hx + py[k] * hy + pz[k] * hz;
      hx = (x[0] - x[1] - x[2] + x[3] - x[4] + x[5] + x[6] - x[7]);
      hy = (y[0] - y[1] - y[2] + y[3] - y[4] + y[5] + y[6] - y[7]);
      hz = (z[0] - z[1] - z[2] + z[3] - z[4] + z[5] + z[6] - z[7]);
#pragma unroll
      for (int k = 0; k < 4; k++) ph[k][2] = px[k] * hx + py[k] * hy + pz[k] * hz;
    }
    const R volr = (R)voln;

    // ---- SDLEN3 / SLEN -----------------------------------------------------
    R deltax;
    {
      R aream = (R)RG_EM20;
      const int fa[6][4] = {{0, 1, 2, 3}, {4, 5, 6, 7}, {0, 1, 5, 4},
                            {1, 2, 6, 5}, {2, 3, 7, 6}, {3, 0, 4, 7}};
#pragma unroll
      for (int j = 0; j < 6; j++) {
        const int a = fa[j][0], b = fa[j][1], c = fa[j][2], d = fa[j][3];
        const R x13 = x[c] - x[a], x24 = x[d] - x[b];
        const R y13 = y[c] - y[a], y24 = y[d] - y[b];
        const R z13 = z[c] - z[a], z24 = z[d] - z[b];
        const R fs1 = x13 - x24, ft1 = x13 + x24;
        const R fs2 = y13 - y24, ft2 = y13 + y24;
        const R fs3 = z13 - z24, ft3 = z13 + z24;
        const R ee = fs1 * fs1 + fs2 * fs2 + fs3 * fs3;
        const R ff = fs1 * ft1 + fs2 * ft2 + fs3 * ft3;
        const R gg = ft1 * ft1 + ft2 * ft2 + ft3 * ft3;
        const R area = ee * gg - ff * ff;
        aream = fmax_(area, aream);
      }
      deltax = (R)RG_FOUR * volr * (R)RG_ONE / sqrt(aream);
    }

    // ---- SDEFO3 (JHBE=1, JCVT=0) ---------------------------------------------
    R dxx, dyy, dzz, d4, d5, d6, wxx, wyy, wzz;
    {
      const R vx17 = vx[0] - vx[6], vx28 = vx[1] - vx[7], vx35 = vx[2] - vx[4], vx46 = vx[3] - vx[5];
      const R vy17 = vy[0] - vy[6], vy28 = vy[1] - vy[7], vy35 = vy[2] - vy[4], vy46 = vy[3] - vy[5];
      const R vz17 = vz[0] - vz[6], vz28 = vz[1] - vz[7], vz35 = vz[2] - vz[4], vz46 = vz[3] - vz[5];
      dxx = px[0] * vx17 + px[1] * vx28 + px[2] * vx35 + px[3] * vx46;
      dyy = py[0] * vy17 + py[1] * vy28 + py[2] * vy35 + py[3] * vy46;
      dzz = pz[0] * vz17 + pz[1] * vz28 + pz[2] * vz35 + pz[3] * vz46;
      const R dxy = py[0] * vx17 + py[1] * vx28 + py[2] * vx35 + py[3] * vx46;
      const R dxz = pz[0] * vx17 + pz[1] * vx28 + pz[2] * vx35 + pz[3] * vx46;
      const R dyx = px[0] * vy17 + px[1] * vy28 + px[2] * vy35 + px[3] * vy46;
      const R dyz = pz[0] * vy17 + pz[1] * vy28 + pz[2] * vy35 + pz[3] * vy46;
      const R dzx = px[0] * vz17 + px[1] * vz28 + px[2] * vz35 + px[3] * vz46;
      const R dzy = py[0] * vz17 + py[1] * vz28 + py[2] * vz35 + py[3] * vz46;
      d4 = dxy + dyx;
      d5 = dyz + dzy;
      d6 = dxz + dzx;
      const R dt1d2 = (R)RG_HALF * dt1;
      wzz = dt1d2 * (dyx - dxy);
      wyy = dt1d2 * (dxz - dzx);
      wxx = dt1d2 * (dzy - dyz);
    }

    // ---- SRHO3 (Lagrangian) -------------------------------------------------
    // FP64 form: RHO state, DVOL = VOLN - (RHO0/RHO)*VOL0, RHO = RHO0*VOL0/VOLN.
    // Mixed form: the FP64 state array holds the volume of the last cycle
    // instead of the density (same information, RHO = RHO0*VOL0/VOL), so
    // DVOL is one FP64 subtraction and no FP64 division is needed.
    const double vol0 = A.vol0[e];
    if (offg == (R)0 && voln == RG_ONE) voln = vol0;
    double dvol_d, rho_new;
    R rho_r, amu, dvol_r;
    if (F64) {
      const double rho_old = A.rho[e];
      dvol_d = voln - (P.rho0 / rho_old) * vol0;
      rho_new = P.rho0 * (vol0 / voln);
      A.rho[e] = rho_new;
      rho_r = (R)rho_new;
      amu = (R)(rho_new / P.rho0 - RG_ONE);
      dvol_r = (R)dvol_d;
    } else {
      const double vold = A.rho[e];
      dvol_d = voln - vold;
      A.rho[e] = voln;
      rho_new = 0.0;
      rho_r = (R)P.rho0 * ((R)vol0 / volr);
      amu = (R)(vol0 - voln) / volr;  // RHO/RHO0 - 1 = VOL0/VOLN - 1
      dvol_r = (R)dvol_d;
    }

    // ---- SROTA3 --------------------------------------------------------------
    R s[6], sg[6];
#pragma unroll
    for (int c = 0; c < 6; c++) s[c] = A.sig[c * ne + e];
    {
      const R q1 = (R)RG_TWO * s[3] * wzz;
      const R q2 = (R)RG_TWO * s[5] * wyy;
      const R q3 = (R)RG_TWO * s[4] * wxx;
      sg[0] = s[0] - q1 + q2;
      sg[1] = s[1] + q1 - q3;
      sg[2] = s[2] - q2 + q3;
      sg[3] = s[3] + wzz * (s[0] - s[1]) + wyy * s[4] - wxx * s[5];
      sg[4] = s[4] + wxx * (s[1] - s[2]) + wzz * s[5] - wyy * s[3];
      sg[5] = s[5] + wyy * (s[2] - s[0]) + wxx * s[3] - wzz * s[4];
    }

    // ---- MMAIN prologue: VOL_AVG, AMU (mmain.F90:676-700) --------------------
    const R vol_avg_r = volr - (R)RG_HALF * dvol_r;

    // ---- material law ----------------------------------------------------------
    const R gg = (R)P.g * off;
    // sound speed: per-group constant for live elements (OFF = 1)
    const R ssp = off == (R)RG_ONE ? (R)P.ssp1
                                   : sqrt(((R)RG_ONEP333 * gg + (R)P.c1) / (R)P.rho0);
    {
      const R g1 = dt1 * gg, g2 = (R)RG_TWO * g1;
      const R p = -(R)RG_THIRD * (sg[0] + sg[1] + sg[2]);
      const R dav = -(R)RG_THIRD * (dxx + dyy + dzz);
      sg[0] = sg[0] + p + g2 * (dxx + dav);
      sg[1] = sg[1] + p + g2 * (dyy + dav);
      sg[2] = sg[2] + p + g2 * (dzz + dav);
      sg[3] = sg[3] + g1 * d4;
      sg[4] = sg[4] + g1 * d5;
      sg[5] = sg[5] + g1 * d6;
    }
    if (LAW == 2) {
      // M2LAW Johnson-Cook radial return, isotropic hardening, no thermal.
      R aj2 = (R)RG_HALF * (sg[0] * sg[0] + sg[1] * sg[1] + sg[2] * sg[2]) +
              sg[3] * sg[3] + sg[4] * sg[4] + sg[5] * sg[5];
      aj2 = sqrt((R)RG_THREE * aj2);
      // MSTRAIN_RATE (materials/mat_share/mstrain_rate.F)
      R epsd = A.epsd[e];
      if (P.israte >= 0) {
        R epsdot;
        if (P.vp - 2 == 0) {
          const R e4 = (R)RG_HALF * d4, e5 = (R)RG_HALF * d5, e6 = (R)RG_HALF * d6;
          const R epsp = dxx * dxx + dyy * dyy + dzz * dzz + (R)RG_TWO * (e4 * e4 + e5 * e5 + e6 * e6);
          epsdot = sqrt(epsp);
        } else {
          const R dv = (dxx + dyy + dzz) * (R)RG_THIRD;
          const R e1 = dxx - dv, e2 = dyy - dv, e3 = dzz - dv;
          const R e4 = (R)RG_HALF * d4, e5 = (R)RG_HALF * d5, e6 = (R)RG_HALF * d6;
          const R epsp = (R)RG_HALF * (e1 * e1 + e2 * e2 + e3 * e3) + e4 * e4 + e5 * e5 + e6 * e6;
          epsdot = sqrt((R)RG_THREE * epsp) / (R)RG_THREE_HALF;
        }
        const R asrate = (R)fmin_(RG_ONE, P.asrate * DT1);
        if (P.israte == 0)
          epsd = epsdot;
        else
          epsd = asrate * epsdot + ((R)RG_ONE - asrate) * epsd;
        A.epsd[e] = epsd;
      }
      R epd = (R)RG_ONE, sigmx = (R)P.sigm0;
      if (P.cc != RG_ZERO) {
        if (P.vp == 1) {
          epd = fmax_(epsd, (R)P.epdr);
          epd = log(epd / (R)P.epdr);
        } else {
          epd = fmax_(epsd, (R)RG_EM15);
          epd = log(epd / (R)P.epdr);
        }
        epd = fmax_((R)RG_ZERO, epd);
        epd = ((R)RG_ONE + (R)P.cc * epd);  // (1 - T*^m) = 1 without heating
        if (P.icc == 1) sigmx = (R)P.sigm0 * epd;
      } else {
        epd = (R)RG_ONE;
        if (P.icc == 1) sigmx = (R)P.sigm0 * epd;
      }
      const R epxe = A.pla[e];
      R ak, qh;
      if (P.cn == RG_ONE) {
        ak = (R)P.ca + (R)P.cb * epxe;
        qh = (R)P.cb * epd;
      } else if (epxe > (R)0) {
        // EPXE**(N-1) = EPXE**N / EPXE: one power evaluation
        const R pn = pow(epxe, (R)P.cn);
        ak = (R)P.ca + (R)P.cb * pn;
        qh = ((R)P.cb * (R)P.cn * (pn / epxe)) * epd;
      } else {
        ak = (R)P.ca;
        qh = (R)0;
      }
      ak = ak * epd;
      if (sigmx < ak) {
        ak = sigmx;
        qh = (R)0;
      }
      if (epxe > (R)P.epmx) {
        ak = (R)0;
        qh = (R)0;
      }
      R scale = fmin_((R)RG_ONE, ak / fmax_(aj2, (R)RG_EM15));
      const R dpla = ((R)RG_ONE - scale) * aj2 / fmax_((R)RG_THREE * gg + qh, (R)RG_EM15);
      ak = ak + (R)RG_ONE * dpla * qh;
      scale = fmin_((R)RG_ONE, ak / fmax_(aj2, (R)RG_EM15));
#pragma unroll
      for (int c = 0; c < 6; c++) sg[c] = scale * sg[c];
      A.pla[e] = epxe + dpla;
    }

    // ---- MQVISCB (explicit, 3D, one point) -------------------------------------
    R qnew, sti;
    const R cbv = F64 ? (R)cbrt(voln) : cbrt(volr);  // VOL**(1/3)
    {
      const R dd = -dxx - dyy - dzz;
      R al = (R)0, ad = (R)0;
      if (off == (R)RG_ONE) {
        al = voln > RG_ZERO ? cbv : (R)0;
        ad = fmax_((R)0, dd);
      }
      const R rhoe = rho_r;
      const R qa = (R)P.qa, qb = (R)P.qb;
      const R qaa = qa * qa * ad;
      R qx = qb * ssp + al * qaa;
      if (P.has_cns) {
        const R nrho = sqrt(rhoe * (R)P.rho0);
        const R cns1 = (R)P.vns1 * al * nrho * ssp * off;
        const R cns2 = (R)P.vns2 * al * nrho * ssp * off;
        qx = qx + (cns1 + cns2) / fmax_((R)RG_EM20, rhoe * deltax);
      }
      qnew = rhoe * ad * al * (qaa * al + qb * ssp);
      const R ssp_eq = fmax_((R)RG_EM20, qx + sqrt(qx * qx + ssp * ssp));
      const R dtx = deltax / ssp_eq;
      sti = (R)0;
      if (!(off == (R)0 || offg < (R)0)) {
        const R tidt = (R)RG_ONE / dtx;
        sti = (rhoe * tidt) * (volr * tidt);
      }
      const double dtxd = F64 ? P.dtfac * (double)dtx : (double)((R)P.dtfac * dtx);
      if (voln > RG_ZERO && (off != (R)0 && offg >= (R)0)) {
        dtmine = dtxd;
        elmin = e;  // element order key; mapped to the user id by the dt kernel
      }
    }

    // ---- law epilogue: pressure, energy, QOLD ----------------------------------
    {
      const R pnew = (R)P.c1 * amu;
      sg[0] = (sg[0] - pnew) * off;
      sg[1] = (sg[1] - pnew) * off;
      sg[2] = (sg[2] - pnew) * off;
      sg[3] = sg[3] * off;
      sg[4] = sg[4] * off;
      sg[5] = sg[5] * off;
      const R qold = A.qvis[e];
      const R dta = (R)RG_HALF * dt1;
      R ework, qwork;
      if (LAW == 1) {
        const R p2 = -(s[0] + sg[0] + s[1] + sg[1] + s[2] + sg[2]) * (R)RG_THIRD;
        const R e1 = dxx * (s[0] + sg[0] + p2);
        const R e2 = dyy * (s[1] + sg[1] + p2);
        const R e3 = dzz * (s[2] + sg[2] + p2);
        const R e4 = d4 * (s[3] + sg[3]);
        const R e5 = d5 * (s[4] + sg[4]);
        const R e6 = d6 * (s[5] + sg[5]);
        ework = (e1 + e2 + e3 + e4 + e5 + e6);
        qwork = qold + qnew + p2;
      } else {
        const R e1 = dxx * (s[0] + sg[0]);
        const R e2 = dyy * (s[1] + sg[1]);
        const R e3 = dzz * (s[2] + sg[2]);
        const R e4 = d4 * (s[3] + sg[3]);
        const R e5 = d5 * (s[4] + sg[4]);
        const R e6 = d6 * (s[5] + sg[5]);
        ework = (e1 + e2 + e3 + e4 + e5 + e6);
        qwork = qold + qnew;
      }
      if (F64) {
        const double einc = (double)vol_avg_r * (double)ework * (double)dta -
                            RG_HALF * dvol_d * (double)qwork;
        const double eint = A.eint[e] * vol0;
        A.eint[e] = (eint + einc * (double)off) / fmax_(RG_ZERO + RG_EM15, vol0);
      } else {
        // EINT += EINC / VOL0: increment in FP32, accumulation in FP64
        const R einc = vol_avg_r * ework * dta - (R)RG_HALF * dvol_r * qwork;
        A.eint[e] = A.eint[e] + (double)(einc * off / (R)vol0);
      }
      A.qvis[e] = qnew;
#pragma unroll
      for (int c = 0; c < 6; c++) A.sig[c * ne + e] = sg[c];
      // SMALLB3
      if (off < (R)RG_ONE) {
        if (off == (R)0)
          A.off[e] = (R)0;
        else if (offg > (R)RG_ONE)
          A.off[e] = (R)RG_ONE + off;
        else
          A.off[e] = off;
      }
    }

    // ---- SHVIS3 (JHBE >= 1) ----------------------------------------------------
    R f[3][8];
    {
      const R caq = (R)RG_FOURTH * off * (R)P.qh;
      R fcl = caq * rho_r * (cbv * cbv);  // VOL**(2/3) = (VOL**(1/3))**2
      const R fcq = fcl * caq * (R)RG_HUNDRED;
      fcl = fcl * ssp;
      R g[8][3];
      g[0][0] = (R)1 - ph[0][0];
      g[1][0] = -(R)1 - ph[1][0];
      g[2][0] = (R)1 - ph[2][0];
      g[3][0] = -(R)1 - ph[3][0];
      g[4][0] = (R)1 + ph[2][0];
      g[5][0] = -(R)1 + ph[3][0];
      g[6][0] = (R)1 + ph[0][0];
      g[7][0] = -(R)1 + ph[1][0];
      g[0][1] = (R)1 - ph[0][1];
      g[1][1] = (R)1 - ph[1][1];
      g[2][1] = -(R)1 - ph[2][1];
      g[3][1] = -(R)1 - ph[3][1];
      g[4][1] = -(R)1 + ph[2][1];
      g[5][1] = -(R)1 + ph[3][1];
      g[6][1] = (R)1 + ph[0][1];
      g[7][1] = (R)1 + ph[1][1];
      g[0][2] = (R)1 - ph[0][2];
      g[1][2] = -(R)1 - ph[1][2];
      g[2][2] = -(R)1 - ph[2][2];
      g[3][2] = (R)1 - ph[3][2];
      g[4][2] = -(R)1 + ph[2][2];
      g[5][2] = (R)1 + ph[3][2];
      g[6][2] = (R)1 + ph[0][2];
      g[7][2] = -(R)1 + ph[1][2];
      R hgx[4], hgy[4], hgz[4];
#pragma unroll
      for (int m = 0; m < 3; m++) {
        hgx[m] = g[0][m] * vx[0] + g[1][m] * vx[1] + g[2][m] * vx[2] + g[3][m] * vx[3] +
                 g[4][m] * vx[4] + g[5][m] * vx[5] + g[6][m] * vx[6] + g[7][m] * vx[7];
        hgy[m] = g[0][m] * vy[0] + g[1][m] * vy[1] + g[2][m] * vy[2] + g[3][m] * vy[3] +
                 g[4][m] * vy[4] + g[5][m] * vy[5] + g[6][m] * vy[6] + g[7][m] * vy[7];
        hgz[m] = g[0][m] * vz[0] + g[1][m] * vz[1] + g[2][m] * vz[2] + g[3][m] * vz[3] +
                 g[4][m] * vz[4] + g[5][m] * vz[5] + g[6][m] * vz[6] + g[7][m] * vz[7];
      }
      hgx[3] = vx[0] - vx[1] + vx[2] - vx[3] - vx[4] + vx[5] - vx[6] + vx[7];
      hgy[3] = vy[0] - vy[1] + vy[2] - vy[3] - vy[4] + vy[5] - vy[6] + vy[7];
      hgz[3] = vz[0] - vz[1] + vz[2] - vz[3] - vz[4] + vz[5] - vz[6] + vz[7];
      R hx[4], hy[4], hz[4];
#pragma unroll
      for (int m = 0; m < 4; m++) {
        hx[m] = hgx[m] * (fcl + fabs(hgx[m]) * fcq);
        hy[m] = hgy[m] * (fcl + fabs(hgy[m]) * fcq);
        hz[m] = hgz[m] * (fcl + fabs(hgz[m]) * fcq);
      }
      const R s4[8] = {-1, 1, -1, 1, 1, -1, 1, -1};
#pragma unroll
      for (int k = 0; k < 8; k++) {
        f[0][k] = -g[k][0] * hx[0] - g[k][1] * hx[1] - g[k][2] * hx[2] + s4[k] * hx[3];
        f[1][k] = -g[k][0] * hy[0] - g[k][1] * hy[1] - g[k][2] * hy[2] + s4[k] * hy[3];
        f[2][k] = -g[k][0] * hz[0] - g[k][1] * hz[1] - g[k][2] * hz[2] + s4[k] * hz[3];
      }
      const R ehou = dt1 * (hz[0] * hgz[0] + hz[1] * hgz[1] + hz[2] * hgz[2] + hz[3] * hgz[3] +
                            hx[0] * hgx[0] + hx[1] * hgx[1] + hx[2] * hgx[2] + hx[3] * hgx[3] +
                            hy[0] * hgy[0] + hy[1] * hgy[1] + hy[2] * hgy[2] + hy[3] * hgy[3]);
      A.ehou[e] = A.ehou[e] + (double)ehou;
    }

    // ---- SFINT3 ------------------------------------------------------------------
    {
      const R s1 = (sg[0] - qnew) * volr;
      const R s2 = (sg[1] - qnew) * volr;
      const R s3 = (sg[2] - qnew) * volr;
      const R s4 = sg[3] * volr;
      const R s5 = sg[4] * volr;
      const R s6 = sg[5] * volr;
      const int pb[4] = {6, 7, 4, 5};
#pragma unroll
      for (int j = 0; j < 4; j++) {
        R fint = s1 * px[j] + s4 * py[j] + s6 * pz[j];
        f[0][j] = f[0][j] - fint;
        f[0][pb[j]] = f[0][pb[j]] + fint;
        fint = s2 * py[j] + s4 * px[j] + s5 * pz[j];
        f[1][j] = f[1][j] - fint;
        f[1][pb[j]] = f[1][pb[j]] + fint;
        fint = s3 * pz[j] + s6 * px[j] + s5 * py[j];
        f[2][j] = f[2][j] - fint;
        f[2][pb[j]] = f[2][pb[j]] + fint;
      }
    }

    // ---- SCUMU3P -------------------------------------------------------------------
    {
      const R offg_new = A.off[e];
      const bool zero = offg_new < (R)0;
      const R st = (R)RG_FOURTH * sti;
#pragma unroll
      for (int k = 0; k < 8; k++) {
        const int K = __ldg(A.iads + k * ne + e);
        typename SlotT<ER>::type w;
        w.x = zero ? (R)0 : f[0][k];
        w.y = zero ? (R)0 : f[1][k];
        w.z = zero ? (R)0 : f[2][k];
        w.w = st;
        fsky[K] = w;
      }
    }
  }

  // per-block time-step candidate
  block_dt_min<NT>(dtmine, elmin, dp.dt + P.part_off + blockIdx.x,
                   dp.el + P.part_off + blockIdx.x);
}

// ---------------------------------------------------------------------------
template <typename ER, int LAW>
static void launch_one(const HexaParams &P, const HexaArrays<ER> &A,
                       const NodeView &N, typename SlotT<ER>::type *fsky,
                       DtPartials dp, const Time *T, int *status,
                       cudaStream_t s) {
  constexpr int NT = 128;
  const int nb = (P.nel + NT - 1) / NT;
  hexa_kernel<ER, LAW, NT><<<nb, NT, 0, s>>>(P, A, N, fsky, dp, T, status);
}

int hexa_blocks(int nel) { return (nel + 127) / 128; }

void launch_hexa_f64(const HexaParams &P, const HexaArrays<double> &A,
                     const NodeView &N, dbl4 *fsky, DtPartials dp,
                     const Time *T, int *status, cudaStream_t s) {
  if (P.mtn == 1)
    launch_one<double, 1>(P, A, N, fsky, dp, T, status, s);
  else
    launch_one<double, 2>(P, A, N, fsky, dp, T, status, s);
}

void launch_hexa_f32(const HexaParams &P, const HexaArrays<float> &A,
                     const NodeView &N, float4 *fsky, DtPartials dp,
                     const Time *T, int *status, cudaStream_t s) {
  if (P.mtn == 1)
    launch_one<float, 1>(P, A, N, fsky, dp, T, status, s);
  else
    launch_one<float, 2>(P, A, N, fsky, dp, T, status, s);
}

}  // namespace rg
