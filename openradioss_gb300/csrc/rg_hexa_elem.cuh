#pragma once
// One-point hexa element of the explicit cycle (SFORC3 chain): the
// per-element device function shared by the single-model kernel
// (rg_hexa.cu) and the batched persistent kernel (rg_batch.cu).
//
// One thread per element, SoA element state, 32-byte node records gathered
// through the read-only path.  The arithmetic follows, step by step and in
// the same expression order, the reference routines cited at each block
// (paths relative to the OpenRadioss source tree):
//   SCOOR3  gather                     elements/solid/solide/scoor3.F:38
//   SRCOOR3 co-rotational frame (JCVT=1) elements/solid/solide/srcoor3.F:42,
//           SREPISO3 / SORTHO3         srepiso3.F, sortho3.F
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
//   SRROTA3 forces back (JCVT=1)       elements/solid/solide/srrota3.F,
//                                      sforc3.F:1634-1645
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

#include <type_traits>

namespace rg {


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

// Products and sums of the co-rotational frame and rotations: in the FP64
// form rounded one operation at a time in the reference's order (no
// contraction into multiply-adds), so that the frame -- a chain of
// normalisations whose round-off the rotated coordinates amplify -- is the
// same bits as a non-contracting CPU build; plain operators in FP32.
template <typename R>
__device__ __forceinline__ R mul_(R a, R b) {
  if constexpr (sizeof(R) == 8) return __dmul_rn(a, b);
  else return a * b;
}
template <typename R>
__device__ __forceinline__ R add_(R a, R b) {
  if constexpr (sizeof(R) == 8) return __dadd_rn(a, b);
  else return a + b;
}
template <typename R>
__device__ __forceinline__ R sub_(R a, R b) {
  if constexpr (sizeof(R) == 8) return __dsub_rn(a, b);
  else return a - b;
}
// a*x + b*y + c*z, left to right
template <typename R>
__device__ __forceinline__ R dot3_(R a, R x, R b, R y, R c, R z) {
  return add_(add_(mul_(a, x), mul_(b, y)), mul_(c, z));
}
// a*b - c*d + e
template <typename R>
__device__ __forceinline__ R cross_add_(R a, R b, R c, R d, R e) {
  return add_(sub_(mul_(a, b), mul_(c, d)), e);
}
template <typename R>
__device__ __forceinline__ R inv_norm_(R a, R b, R c) {
  R n = sqrt(dot3_(a, a, b, b, c, c));
  if (n != (R)0) n = (R)1 / n;
  return n;
}

// SREPISO3 + SORTHO3: the co-rotational frame of a hexa from its
// isoparametric directions r, s, t, orthogonalised by three symmetric
// iterations; R[3i+j] = Rij, column j = local axis j.  Only coordinate
// differences enter, so relative coordinates give the same frame.
template <typename R>
__device__ __forceinline__ void hexa_frame(const R *x, const R *y, const R *z, R *Rm) {
  const R x17 = x[6] - x[0], x28 = x[7] - x[1], x35 = x[4] - x[2], x46 = x[5] - x[3];
  const R y17 = y[6] - y[0], y28 = y[7] - y[1], y35 = y[4] - y[2], y46 = y[5] - y[3];
  const R z17 = z[6] - z[0], z28 = z[7] - z[1], z35 = z[4] - z[2], z46 = z[5] - z[3];
  const R a17 = x17 + x46, a28 = x28 + x35;
  const R b17 = y17 + y46, b28 = y28 + y35;
  const R c17 = z17 + z46, c28 = z28 + z35;
  const R rx = x17 + x28 - x35 - x46, ry = y17 + y28 - y35 - y46, rz = z17 + z28 - z35 - z46;
  const R sx = a17 + a28, sy = b17 + b28, sz = c17 + c28;
  const R tx = a17 - a28, ty = b17 - b28, tz = c17 - c28;
  R aa = inv_norm_(rx, ry, rz);
  R ux = mul_(rx, aa), uy = mul_(ry, aa), uz = mul_(rz, aa);
  aa = inv_norm_(sx, sy, sz);
  R vx = mul_(sx, aa), vy = mul_(sy, aa), vz = mul_(sz, aa);
  aa = inv_norm_(tx, ty, tz);
  R wx = mul_(tx, aa), wy = mul_(ty, aa), wz = mul_(tz, aa);
#pragma unroll
  for (int it = 0; it < 3; it++) {
    const R e1x = cross_add_(vy, wz, vz, wy, ux), e1y = cross_add_(vz, wx, vx, wz, uy),
            e1z = cross_add_(vx, wy, vy, wx, uz);
    const R e2x = cross_add_(wy, uz, wz, uy, vx), e2y = cross_add_(wz, ux, wx, uz, vy),
            e2z = cross_add_(wx, uy, wy, ux, vz);
    const R e3x = cross_add_(uy, vz, uz, vy, wx), e3y = cross_add_(uz, vx, ux, vz, wy),
            e3z = cross_add_(ux, vy, uy, vx, wz);
    R bb = inv_norm_(e1x, e1y, e1z);
    ux = mul_(e1x, bb);
    uy = mul_(e1y, bb);
    uz = mul_(e1z, bb);
    bb = inv_norm_(e2x, e2y, e2z);
    vx = mul_(e2x, bb);
    vy = mul_(e2y, bb);
    vz = mul_(e2z, bb);
    bb = inv_norm_(e3x, e3y, e3z);
    wx = mul_(e3x, bb);
    wy = mul_(e3y, bb);
    wz = mul_(e3z, bb);
  }
  R e3x = sub_(mul_(uy, vz), mul_(uz, vy)), e3y = sub_(mul_(uz, vx), mul_(ux, vz)),
    e3z = sub_(mul_(ux, vy), mul_(uy, vx));
  aa = inv_norm_(e3x, e3y, e3z);
  e3x = mul_(e3x, aa);
  e3y = mul_(e3y, aa);
  e3z = mul_(e3z, aa);
  Rm[0] = ux;
  Rm[3] = uy;
  Rm[6] = uz;
  Rm[1] = sub_(mul_(e3y, uz), mul_(e3z, uy));
  Rm[4] = sub_(mul_(e3z, ux), mul_(e3x, uz));
  Rm[7] = sub_(mul_(e3x, uy), mul_(e3y, ux));
  Rm[2] = e3x;
  Rm[5] = e3y;
  Rm[8] = e3z;
}

// JCVT = 0: Jaumann-rate formulation (Iframe=1); JCVT = 1: co-rotational
// frame (Iframe=2, the default of 8-node Lagrangian bricks): coordinates and
// velocities in the element frame, no spin, midpoint-corrected rates, the
// stress kept in the frame, forces rotated back.
template <typename ER, int LAW, int JCVT = 0>
__device__ __forceinline__ void hexa_element(const HexaParams &P, const HexaArrays<ER> &A,
                                             const NodeView &N,
                                             typename SlotT<ER>::type *__restrict__ fsky,
                                             const Time *__restrict__ T,
                                             int *__restrict__ status, const int il,
                                             ER &dtmine, int &elmin) {
  typedef ER R;
  constexpr bool F64 = std::is_same<ER, double>::value;
  const int ne = A.ne;
  {
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
    R off_stored = offg0;  // OFFG as last written by this element
    // The element state is read up front: as far as the compiler knows the
    // state arrays may alias, so a load placed after a store could not be
    // issued early; here all loads overlap the node gathers.
    const double st_rho = A.rho[e];
    const double st_vol0 = A.vol0[e];
    R st_sig[6];
#pragma unroll
    for (int c = 0; c < 6; c++) st_sig[c] = A.sig[c * ne + e];
    const R st_qvis = A.qvis[e];
    const double st_eint = A.eint[e];
    const double st_ehou = A.ehou[e];
    R st_epsd = (R)0, st_pla = (R)0;
    if (LAW == 2) {
      st_epsd = A.epsd[e];
      st_pla = A.pla[e];
    }
    R x[8], y[8], z[8];
    R vx[8], vy[8], vz[8];
    if constexpr (F64) {
      // FP64 form: absolute FP64 coordinates, as the reference
#pragma unroll
      for (int k = 0; k < 8; k++) {
        const dbl4 xk = ld4(N.X4 + nc[k]);
        const dbl4 vk = ld4(N.V4 + nc[k]);
        x[k] = xk.x;
        y[k] = xk.y;
        z[k] = xk.z;
        const bool z0 = offg0 < (R)0;
        vx[k] = z0 ? (R)0 : (R)vk.x;
        vy[k] = z0 ? (R)0 : (R)vk.y;
        vz[k] = z0 ? (R)0 : (R)vk.z;
      }
    } else {
      // mixed form: FP32 copies kept by the node kernel -- coordinates as a
      // hi + lo pair of floats, so that differences between the nodes of an
      // element keep FP32 relative precision at any distance from the origin
      F8 c[8];
#pragma unroll
      for (int k = 0; k < 8; k++) {
        c[k] = ldF8(N.XF + nc[k]);
        const float4 vk = ldf4(N.VF + nc[k]);
        const bool z0 = offg0 < (R)0;
        vx[k] = z0 ? 0.f : vk.x;
        vy[k] = z0 ? 0.f : vk.y;
        vz[k] = z0 ? 0.f : vk.z;
      }
#pragma unroll
      for (int k = 0; k < 8; k++) {
        x[k] = (c[k].hx - c[0].hx) + (c[k].lx - c[0].lx);
        y[k] = (c[k].hy - c[0].hy) + (c[k].ly - c[0].ly);
        z[k] = (c[k].hz - c[0].hz) + (c[k].lz - c[0].lz);
      }
    }

    // ---- SRCOOR3 (JCVT = 1): frame, local coordinates and velocities --------
    R Rm[9];
    if constexpr (JCVT != 0) {
      hexa_frame<R>(x, y, z, Rm);
#pragma unroll
      for (int k = 0; k < 8; k++) {
        const R X = x[k], Y = y[k], Z = z[k];
        x[k] = dot3_(Rm[0], X, Rm[3], Y, Rm[6], Z);
        y[k] = dot3_(Rm[1], X, Rm[4], Y, Rm[7], Z);
        z[k] = dot3_(Rm[2], X, Rm[5], Y, Rm[8], Z);
        const R U = vx[k], V = vy[k], W = vz[k];
        vx[k] = dot3_(Rm[0], U, Rm[3], V, Rm[6], W);
        vy[k] = dot3_(Rm[1], U, Rm[4], V, Rm[7], W);
        vz[k] = dot3_(Rm[2], U, Rm[5], V, Rm[8], W);
      }
    }

    // ---- SDERI3 ------------------------------------------------------------
    R px[4], py[4], pz[4], ph[4][3];
    double voln;  // element volume (VOLDP)
    double vold_mixed = 0.0;
    R dv_mixed = (R)0;  // mixed form: FP32 volume change of the cycle
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
      R det = (R)RG_ONE_OVER_64 * (jac1 * j5968 + jac2 * j6749 + jac3 * j4857);
      // SCHKJABT3: a live element with a non-positive volume is switched
      // off and the run is flagged (INEG_V = 0 stops the run).
      bool live = true;
      if (off == (R)0) {
        det = (R)RG_ONE;
        live = false;
      } else if (det <= (R)0) {
        det = (R)RG_ONE;
        off = (R)0;
        offg = (R)0;
        A.off[e] = (R)0;
        off_stored = (R)0;
        atomicOr(status, 1);
        live = false;
      }
      if constexpr (F64) {
        voln = det;
      } else {
        // Volume change over the last step, V(X) - V(X - DT1*V), as the
        // exact trilinear expansion of the determinant in the rows
        // a=(J1,J2,J3), b=(J4,J5,J6), c=(J7,J8,J9) and their velocity
        // increments: every term is computed in FP32 at its own scale (no
        // cancellation), and the volume is accumulated in FP64.
        vold_mixed = st_rho;
        if (live) {
          const R u17 = vx[6] - vx[0], u28 = vx[7] - vx[1], u35 = vx[4] - vx[2], u46 = vx[5] - vx[3];
          const R v17 = vy[6] - vy[0], v28 = vy[7] - vy[1], v35 = vy[4] - vy[2], v46 = vy[5] - vy[3];
          const R w17 = vz[6] - vz[0], w28 = vz[7] - vz[1], w35 = vz[4] - vz[2], w46 = vz[5] - vz[3];
          const R da1 = dt1 * (u17 + u28 - u35 - u46), da2 = dt1 * (v17 + v28 - v35 - v46),
                  da3 = dt1 * (w17 + w28 - w35 - w46);
          const R db1 = dt1 * ((u17 + u46) + (u28 + u35)), db2 = dt1 * ((v17 + v46) + (v28 + v35)),
                  db3 = dt1 * ((w17 + w46) + (w28 + w35));
          const R dc1 = dt1 * ((u17 + u46) - (u28 + u35)), dc2 = dt1 * ((v17 + v46) - (v28 + v35)),
                  dc3 = dt1 * ((w17 + w46) - (w28 + w35));
          // c x a, a x b
          const R ca1 = jac8 * jac3 - jac9 * jac2, ca2 = jac9 * jac1 - jac7 * jac3,
                  ca3 = jac7 * jac2 - jac8 * jac1;
          const R ab1 = jac2 * jac6 - jac3 * jac5, ab2 = jac3 * jac4 - jac1 * jac6,
                  ab3 = jac1 * jac5 - jac2 * jac4;
          const R t1 = (da1 * j5968 + da2 * j6749 + da3 * j4857) +
                       (db1 * ca1 + db2 * ca2 + db3 * ca3) + (dc1 * ab1 + dc2 * ab2 + dc3 * ab3);
          // db x c + b x dc, db x dc
          const R m1 = (db2 * jac9 - db3 * jac8) + (jac5 * dc3 - jac6 * dc2);
          const R m2 = (db3 * jac7 - db1 * jac9) + (jac6 * dc1 - jac4 * dc3);
          const R m3 = (db1 * jac8 - db2 * jac7) + (jac4 * dc2 - jac5 * dc1);
          const R q1 = db2 * dc3 - db3 * dc2, q2 = db3 * dc1 - db1 * dc3, q3 = db1 * dc2 - db2 * dc1;
          const R t2 = (da1 * m1 + da2 * m2 + da3 * m3) + (jac1 * q1 + jac2 * q2 + jac3 * q3);
          const R t3 = da1 * q1 + da2 * q2 + da3 * q3;
          const R dv = (R)RG_ONE_OVER_64 * ((t1 - t2) + t3);
          voln = vold_mixed + (double)dv;
          dv_mixed = dv;
        } else {
          voln = vold_mixed;
        }
      }
      const R dett = (R)RG_ONE_OVER_64 / det;
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
      // FP64 form: one reciprocal square root (the FP64 pipe bounds it)
      if constexpr (F64)
        deltax = (R)RG_FOUR * volr * rsqrt(aream);
      else
        deltax = (R)RG_FOUR * volr * (R)RG_ONE / sqrt(aream);
    }

    // ---- SDEFO3 (JHBE=1) -------------------------------------------------------
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
      const R dt1d2 = (R)RG_HALF * dt1;
      if constexpr (JCVT != 0) {
        // sdefo3.F:158-205 (explicit): no spin, midpoint correction
        const R exx = dxx, eyy = dyy, ezz = dzz;
        wxx = wyy = wzz = (R)0;
        dxx = dxx - dt1d2 * (exx * exx + dyx * dyx + dzx * dzx);
        dyy = dyy - dt1d2 * (eyy * eyy + dzy * dzy + dxy * dxy);
        dzz = dzz - dt1d2 * (ezz * ezz + dxz * dxz + dyz * dyz);
        R aaa = dt1d2 * (exx * dxy + dyx * eyy + dzx * dzy);
        d4 = (dxy - aaa) + (dyx - aaa);
        aaa = dt1d2 * (eyy * dyz + dzy * ezz + dxy * dxz);
        d5 = (dyz - aaa) + (dzy - aaa);
        aaa = dt1d2 * (ezz * dzx + dxz * exx + dyz * dyx);
        d6 = (dxz - aaa) + (dzx - aaa);
      } else {
        d4 = dxy + dyx;
        d5 = dyz + dzy;
        d6 = dxz + dzx;
        wzz = dt1d2 * (dyx - dxy);
        wyy = dt1d2 * (dxz - dzx);
        wxx = dt1d2 * (dzy - dyz);
      }
    }

    // ---- SRHO3 (Lagrangian) -------------------------------------------------
    // FP64 form: RHO state, DVOL = VOLN - (RHO0/RHO)*VOL0, RHO = RHO0*VOL0/VOLN.
    // Mixed form: the FP64 state array holds the element volume of the last
    // cycle instead of the density (RHO = RHO0*VOL0/VOL), DVOL is the
    // FP32 volume change computed above.
    const double vol0 = st_vol0;
    if constexpr (F64) {
      if (offg == (R)0 && voln == RG_ONE) voln = vol0;
    }
    R rho_r, amu, dvol_r;
    double dvol_d = 0.0;
    if constexpr (F64) {
      const double rho_old = st_rho;
      dvol_d = voln - (P.rho0 / rho_old) * vol0;
      const double rho_new = P.rho0 * (vol0 / voln);
      A.rho[e] = rho_new;
      rho_r = (R)rho_new;
      amu = (R)(rho_new * P.inv_rho0 - RG_ONE);
      dvol_r = (R)dvol_d;
    } else {
      A.rho[e] = voln;
      dvol_r = dv_mixed;
      rho_r = PC(rho0) * ((R)vol0 / volr);
      amu = (R)(vol0 - voln) / volr;  // RHO/RHO0 - 1 = VOL0/VOLN - 1
    }

    // ---- SROTA3 --------------------------------------------------------------
    R s[6], sg[6];
#pragma unroll
    for (int c = 0; c < 6; c++) s[c] = st_sig[c];
    if constexpr (JCVT != 0) {
      // SRMALLA3: the stress stays in the element frame
#pragma unroll
      for (int c = 0; c < 6; c++) sg[c] = s[c];
    } else {
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
    const R gg = PC(g) * off;
    // sound speed: per-group constant for live elements (OFF = 1)
    const R ssp = off == (R)RG_ONE ? PC(ssp1)
                                   : sqrt(((R)RG_ONEP333 * gg + PC(c1)) / PC(rho0));
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
      R epsd = st_epsd;
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
          epsdot = sqrt((R)RG_THREE * epsp) * (R)RG_TWO_THIRD;  // / THREE_HALF
        }
        R asrate;
        if constexpr (F64)
          asrate = fmin_(RG_ONE, P.asrate * DT1);
        else
          asrate = fmin_(1.f, P.f.asrate * dt1);
        if (P.israte == 0)
          epsd = epsdot;
        else
          epsd = asrate * epsdot + ((R)RG_ONE - asrate) * epsd;
        A.epsd[e] = epsd;
      }
      R epd = (R)RG_ONE, sigmx = PC(sigm0);
      if (P.f.cc_nz) {
        if (P.vp == 1) {
          epd = fmax_(epsd, PC(epdr));
          epd = log(epd / PC(epdr));
        } else {
          epd = fmax_(epsd, (R)RG_EM15);
          epd = log(epd / PC(epdr));
        }
        epd = fmax_((R)RG_ZERO, epd);
        epd = ((R)RG_ONE + PC(cc) * epd);  // (1 - T*^m) = 1 without heating
        if (P.icc == 1) sigmx = PC(sigm0) * epd;
      } else {
        epd = (R)RG_ONE;
        if (P.icc == 1) sigmx = PC(sigm0) * epd;
      }
      const R epxe = st_pla;
      R ak, qh;
      if (P.f.cn_one) {
        ak = PC(ca) + PC(cb) * epxe;
        qh = PC(cb) * epd;
      } else if (epxe > (R)0) {
        // EPXE**(N-1) = EPXE**N / EPXE: one power evaluation
        const R pn = pow(epxe, PC(cn));
        ak = PC(ca) + PC(cb) * pn;
        qh = (PC(cb) * PC(cn) * (pn / epxe)) * epd;
      } else {
        ak = PC(ca);
        qh = (R)0;
      }
      ak = ak * epd;
      if (sigmx < ak) {
        ak = sigmx;
        qh = (R)0;
      }
      if (epxe > PC(epmx)) {
        ak = (R)0;
        qh = (R)0;
      }
      const R inv_aj2 = (R)RG_ONE / fmax_(aj2, (R)RG_EM15);  // both scale factors
      R scale = fmin_((R)RG_ONE, ak * inv_aj2);
      const R dpla = ((R)RG_ONE - scale) * aj2 / fmax_((R)RG_THREE * gg + qh, (R)RG_EM15);
      ak = ak + (R)RG_ONE * dpla * qh;
      scale = fmin_((R)RG_ONE, ak * inv_aj2);
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
        al = (F64 ? voln > RG_ZERO : volr > (R)0) ? cbv : (R)0;
        ad = fmax_((R)0, dd);
      }
      const R rhoe = rho_r;
      const R qa = PC(qa), qb = PC(qb);
      const R qaa = qa * qa * ad;
      R qx = qb * ssp + al * qaa;
      if (P.has_cns) {
        const R nrho = sqrt(rhoe * PC(rho0));
        const R cns1 = PC(vns1) * al * nrho * ssp * off;
        const R cns2 = PC(vns2) * al * nrho * ssp * off;
        qx = qx + (cns1 + cns2) / fmax_((R)RG_EM20, rhoe * deltax);
      }
      qnew = rhoe * ad * al * (qaa * al + qb * ssp);
      const R ssp_eq = fmax_((R)RG_EM20, qx + sqrt(qx * qx + ssp * ssp));
      R dtx, tidt64 = (R)0;
      if constexpr (F64) {
        // DTX = DELTAX / SSP_EQ and 1/DTX from one reciprocal
        const R rd = (R)RG_ONE / (deltax * ssp_eq);
        dtx = deltax * deltax * rd;
        tidt64 = ssp_eq * ssp_eq * rd;
      } else {
        dtx = deltax / ssp_eq;
      }
      sti = (R)0;
      if (!(off == (R)0 || offg < (R)0)) {
        R tidt;
        if constexpr (F64)
          tidt = tidt64;
        else
          tidt = (R)RG_ONE / dtx;
        sti = (rhoe * tidt) * (volr * tidt);
      }
      const R dtxd = PC(dtfac) * dtx;
      // under the nodal time step the element only gives STI (mqviscb.F:351)
      if (!P.nodadt && (F64 ? voln > RG_ZERO : volr > (R)0) && (off != (R)0 && offg >= (R)0)) {
        // running minimum over the elements this thread handles; element
        // order key e, mapped to the user id by the time-step reduction
        dt_pair_min_t(dtmine, elmin, dtxd, e);
      }
    }

    // ---- law epilogue: pressure, energy, QOLD ----------------------------------
    {
      const R pnew = PC(c1) * amu;
      sg[0] = (sg[0] - pnew) * off;
      sg[1] = (sg[1] - pnew) * off;
      sg[2] = (sg[2] - pnew) * off;
      sg[3] = sg[3] * off;
      sg[4] = sg[4] * off;
      sg[5] = sg[5] * off;
      const R qold = st_qvis;
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
        const double eint = st_eint * vol0;
        A.eint[e] = (eint + einc * (double)off) / fmax_(RG_ZERO + RG_EM15, vol0);
      } else {
        // EINT += EINC / VOL0: increment in FP32, accumulation in FP64
        const R einc = vol_avg_r * ework * dta - (R)RG_HALF * dvol_r * qwork;
        A.eint[e] = st_eint + (double)(einc * off / (R)vol0);
      }
      A.qvis[e] = qnew;
#pragma unroll
      for (int c = 0; c < 6; c++) A.sig[c * ne + e] = sg[c];
      // SMALLB3
      if (off < (R)RG_ONE) {
        if (off == (R)0)
          off_stored = (R)0;
        else if (offg > (R)RG_ONE)
          off_stored = (R)RG_ONE + off;
        else
          off_stored = off;
        A.off[e] = off_stored;
      }
    }

    // ---- SHVIS3 (JHBE >= 1) ----------------------------------------------------
    // Mixed form: the node velocities are read again (the read-only FP32
    // copies, in L1/L2 since the gather) rather than held in registers
    // through the material update -- fewer live values, fewer spills.
    if constexpr (!F64 && JCVT == 0) {
#pragma unroll
      for (int k = 0; k < 8; k++) {
        const float4 vk = ldf4(N.VF + nc[k]);
        const bool z0 = offg0 < (R)0;
        vx[k] = z0 ? 0.f : vk.x;
        vy[k] = z0 ? 0.f : vk.y;
        vz[k] = z0 ? 0.f : vk.z;
      }
    }
    R f[3][8];
    {
      const R caq = (R)RG_FOURTH * off * PC(qh);
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
      A.ehou[e] = st_ehou + (double)ehou;
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

    // ---- SRROTA3 (JCVT = 1): forces back to the global frame, F = R F_loc ------
    if constexpr (JCVT != 0) {
#pragma unroll
      for (int k = 0; k < 8; k++) {
        const R fx = f[0][k], fy = f[1][k], fz = f[2][k];
        f[0][k] = dot3_(Rm[0], fx, Rm[1], fy, Rm[2], fz);
        f[1][k] = dot3_(Rm[3], fx, Rm[4], fy, Rm[5], fz);
        f[2][k] = dot3_(Rm[6], fx, Rm[7], fy, Rm[8], fz);
      }
    }

    // ---- SCUMU3P -------------------------------------------------------------------
    {
      const R offg_new = off_stored;
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
}

}  // namespace rg
