// CPU oracle for the OpenRadioss explicit hot path -- TEST INFRASTRUCTURE.
//
// A restatement, routine by routine and in the reference's own expression
// order, of the Fortran that one explicit cycle runs.  It checks the CUDA
// product (tests, smoke) and is the timed CPU baseline (bench.py); the
// product never links or calls it.  Compiled with -ffp-contract=off like the
// reference's gfortran build (engine/CMake_Compilers/cmake_linux64_gf.txt:163)
// so that no multiply-add is fused.
//
// Parity status: the reference engine cannot be built here (no Fortran
// compiler; the starter also needs an un-vendored binary library).  Both
// element paths are pinned against outputs the reference engine wrote for
// its own QA decks: the shell path by CRA2V44 (printed cycle table to every
// digit, time histories to ~1e-6 relative over 3375 cycles), the hexa path
// (LAW1, co-rotational frame, viscous hourglass) by H101 (six cantilevers
// with rigid-body tips under concentrated loads: printed table to every
// digit, energies and tip motions to ~1e-7 over 847 cycles).  Rigid bodies
// and concentrated loads are here to run that deck.
//
// Each block cites the reference file:line it follows (paths relative to the
// OpenRadioss source tree).
#include "rg_oracle.h"
#include "../openradioss_gb300/csrc/rg_constants.h"

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <numeric>
#include <vector>
#ifdef _OPENMP
#include <omp.h>
#endif

namespace {

constexpr int MVSIZ = 128;  // group length (engine/share/spe_inc/mvsiz_p.inc)

struct HexaGroup {
  int nft = 0, nel = 0, mtn = 1;
  int add = 0;  // index of the or_hexa_group_add call (the default part)
  int ismstr = 4, jhbe = 1, jcvt = 0;
  // material / property values used on the path
  double rho0 = 0, g = 0, c1 = 0;  // PM(1), PM(22), PM(32)
  double qh = 0, qa = 0, qb = 0, vns1 = 0, vns2 = 0;  // GEO(13..17)
  // LAW2 (mat_param%uparam / iparam)
  double ca = 0, cb = 0, cn = 1, epmx = 0, sigm0 = 0, cc = 0, epdr = 1;
  double fisokin = 0, asrate = 0, z3 = 1;
  int iform = 0, icc = 1, vp = 2, israte = 0;
};

struct ShellGroup;  // shells: rg_oracle_shell.cpp

struct Model {
  int numnod = 0;
  std::vector<double> X, V, D, A, AR, VR, DR, STIFN, STIFR, MS, IN;
  std::vector<double> FLAST, FRLAST;  // assembled forces of the last cycle
  std::vector<int> icodt;

  // hexa elements (global SoA over all hexa groups)
  int numels = 0;
  std::vector<int> ixs;  // 11 * numels, reference layout, 1-based nodes
  std::vector<HexaGroup> hg;
  std::vector<double> sig, eint, rho, vol, qvis, offg, pla, epsd, ehou;
  std::vector<int> iads;  // 8 * numels, 1-based slot numbers

  // skyline
  std::vector<int> adsky;      // numnod + 1 (1-based values)
  std::vector<double> fsky;    // 8 * lsky: {fx,fy,fz,mx,my,mz,sti,stir}
  int lsky = 0;

  // time (RESOL)
  double tt = 0, dt1 = 0, dt2 = 0, dt12 = 0, dt2old = 0, dtmx = RG_EP30;
  double dtfac_solid = RG_ZEP9, dtfac_shell = RG_ZEP9;
  int ncycle = 0, neltst = 0, nthreads = 1;
  int error = 0;
  bool finalized = false;
  double ehour_total = 0;

  // rigid links between nodes (engine /VEL/TRA, RLINK1)
  struct Link {
    std::vector<int> nodes;  // 0-based
    int ic = 0, icr = 0;     // direction codes: 4 = x, 2 = y, 1 = z
  };
  std::vector<Link> links;

  // nodal time step (/DT/NODA, DTNODA): DTFAC1(11), DTMIN1(11)
  int nodadt = 0;
  double dtfac_noda = RG_ZEP9, dtmin_noda = RG_ZERO;
  int idtmin_noda = 0;  // IDTMIN(11): 3 / 8 mass scaling, else flag

  // rigid bodies (/RBODY; starter INIRBY done by the caller: the main node
  // sits at the centre of mass with MS = body mass, IN = smallest principal
  // inertia)
  struct Body {
    int main = 0;            // 0-based
    std::vector<int> nodes;  // secondary nodes, 0-based
    double R[9] = {};        // principal axes, rows e1 e2 e3 (RBY(1:9))
    double I[3] = {};        // principal inertia (RBY(10:12))
  };
  std::vector<Body> bodies;
  std::vector<char> secondary;  // 1: secondary node of a rigid body, 2: main

  // concentrated loads (/CLOAD): node (0-based), direction 0..5 (x y z, then
  // rotations), abscissa / ordinate scales, load curve points
  struct Load {
    int node = 0, dir = 0;
    double fcx = 1, fcy = 1;
    std::vector<double> x, y;
  };
  std::vector<Load> loads;
  double wfext = 0;  // external work of the loads (OUTPUT%TH%WFEXT)

  // rigid-material bodies (/MAT/RIGID, LAW13): the starter's RIGID_MAT
  // record, set up by the caller (rigid_mat.F): mass RBYM(1), centre of mass
  // RBYM(2:4) (never moved by the engine), principal axes as rows
  // RBYM(5:13), principal inertia RBYM(14:16), smallest of them RBYM(17),
  // global inertia tensor RBYM(18:26); the codes CONDRMAT moved from the
  // secondary nodes, and the body's accelerations and velocities ARBYM,
  // VRBYM, ARRBYM, VRRBYM.
  struct RigidMat {
    std::vector<int> nodes;  // secondary nodes, 0-based
    double mass = 0, xg[3] = {}, R[9] = {}, I[3] = {}, in = 0, J[9] = {};
    int icod[2] = {0, 0};    // rotational, translational (Radioss codes: 4 x, 2 y, 1 z)
    double ar[3] = {}, vr[3] = {}, arr[3] = {}, vrr[3] = {};
  };
  std::vector<RigidMat> rmats;

  // imposed velocities (/IMPVEL, FIXVEL with IDIS = 1, global direction):
  // node (0-based), direction 0..2, 1/abscissa scale (FACX), ordinate scale,
  // start / stop times, load curve, and the power carried to the next
  // cycle's work (VEL(4))
  struct ImpVel {
    int node = 0, dir = 0;
    double facx = 1, fscale = 1, tstart = 0, tstop = 1e30;
    std::vector<double> x, y;
    double vel4 = 0;
  };
  std::vector<ImpVel> impvels;

  // forces supplied from outside for the next cycle (or_set_forces): the
  // cycle then skips its element groups and assembly
  bool ext = false;
  std::vector<double> ext_f, ext_fr, ext_stifn, ext_stifr;
  double ext_dt2t = 0;
  int ext_neltst = 0;

  // listing quantities of the last cycle, taken where ECRIT runs (after the
  // kinematic conditions, before VELOCITY)
  bool record = false;
  double out[11] = {};
  // per-part sums of the last recorded cycle (SBILAN / CBILAN): element ->
  // part maps (empty: one part per element group, hexa groups first)
  int npart = 0;
  int nhexa_adds = 0;  // or_hexa_group_add calls: the default parts of hexas
  std::vector<int> part_hexa, part_shell;
  std::vector<double> psum;  // [npart][7]
};

// ----------------------------------------------------------------------------
// SFORC3 one-point hexa, JCVT=0, Lagrangian, JHBE=1 (sforc3.F:60-1817).
// All arrays are local group SoA of length nel <= MVSIZ, as in the Fortran.
// ----------------------------------------------------------------------------
struct HexaLocal {
  int nc[8][MVSIZ];
  double x[8][MVSIZ], y[8][MVSIZ], z[8][MVSIZ];
  double vx[8][MVSIZ], vy[8][MVSIZ], vz[8][MVSIZ];
  double off[MVSIZ], voln[MVSIZ], deltax[MVSIZ];
  double px[4][MVSIZ], py[4][MVSIZ], pz[4][MVSIZ];
  double ph[4][3][MVSIZ];  // PXiHj
  double dxx[MVSIZ], dyy[MVSIZ], dzz[MVSIZ], dxy[MVSIZ], dyx[MVSIZ],
      dyz[MVSIZ], dzy[MVSIZ], dxz[MVSIZ], dzx[MVSIZ], d4[MVSIZ], d5[MVSIZ],
      d6[MVSIZ], wxx[MVSIZ], wyy[MVSIZ], wzz[MVSIZ];
  double dvol[MVSIZ], divde[MVSIZ], amu[MVSIZ], vol_avg[MVSIZ];
  double s[6][MVSIZ];  // stress before rotation (SOLD)
  double ssp[MVSIZ], qnew[MVSIZ], ssp_eq[MVSIZ], sti[MVSIZ];
  double f[3][8][MVSIZ];
  double r[9][MVSIZ];  // JCVT=1: element frame R11 R12 R13 R21 ... R33
};

// SREPISO3 + SORTHO3 (srepiso3.F, sortho3.F): the co-rotational frame of a
// hexa from its isoparametric directions r, s, t (the JAC1-9 combinations),
// orthogonalised by three symmetric iterations.  R(3i+j) holds Rij; column j
// is local axis j (SORTHO3's E1X = R11, E2X = R12, E3X = R13, ...).
static void hexa_frame(const double *x, const double *y, const double *z, double *R) {
  const double x17 = x[6] - x[0], x28 = x[7] - x[1], x35 = x[4] - x[2], x46 = x[5] - x[3];
  const double y17 = y[6] - y[0], y28 = y[7] - y[1], y35 = y[4] - y[2], y46 = y[5] - y[3];
  const double z17 = z[6] - z[0], z28 = z[7] - z[1], z35 = z[4] - z[2], z46 = z[5] - z[3];
  const double a17 = x17 + x46, a28 = x28 + x35;
  const double b17 = y17 + y46, b28 = y28 + y35;
  const double c17 = z17 + z46, c28 = z28 + z35;
  const double rx = x17 + x28 - x35 - x46, ry = y17 + y28 - y35 - y46, rz = z17 + z28 - z35 - z46;
  const double sx = a17 + a28, sy = b17 + b28, sz = c17 + c28;
  const double tx = a17 - a28, ty = b17 - b28, tz = c17 - c28;
  double aa = std::sqrt(rx * rx + ry * ry + rz * rz);
  if (aa != RG_ZERO) aa = RG_ONE / aa;
  double ux = rx * aa, uy = ry * aa, uz = rz * aa;
  aa = std::sqrt(sx * sx + sy * sy + sz * sz);
  if (aa != RG_ZERO) aa = RG_ONE / aa;
  double vx = sx * aa, vy = sy * aa, vz = sz * aa;
  aa = std::sqrt(tx * tx + ty * ty + tz * tz);
  if (aa != RG_ZERO) aa = RG_ONE / aa;
  double wx = tx * aa, wy = ty * aa, wz = tz * aa;
  for (int it = 0; it < 3; it++) {
    const double e1x = vy * wz - vz * wy + ux, e1y = vz * wx - vx * wz + uy,
                 e1z = vx * wy - vy * wx + uz;
    const double e2x = wy * uz - wz * uy + vx, e2y = wz * ux - wx * uz + vy,
                 e2z = wx * uy - wy * ux + vz;
    const double e3x = uy * vz - uz * vy + wx, e3y = uz * vx - ux * vz + wy,
                 e3z = ux * vy - uy * vx + wz;
    double bb = std::sqrt(e1x * e1x + e1y * e1y + e1z * e1z);
    if (bb != RG_ZERO) bb = RG_ONE / bb;
    ux = e1x * bb;
    uy = e1y * bb;
    uz = e1z * bb;
    bb = std::sqrt(e2x * e2x + e2y * e2y + e2z * e2z);
    if (bb != RG_ZERO) bb = RG_ONE / bb;
    vx = e2x * bb;
    vy = e2y * bb;
    vz = e2z * bb;
    bb = std::sqrt(e3x * e3x + e3y * e3y + e3z * e3z);
    if (bb != RG_ZERO) bb = RG_ONE / bb;
    wx = e3x * bb;
    wy = e3y * bb;
    wz = e3z * bb;
  }
  const double e1x = ux, e1y = uy, e1z = uz;
  double e3x = e1y * vz - e1z * vy, e3y = e1z * vx - e1x * vz, e3z = e1x * vy - e1y * vx;
  aa = std::sqrt(e3x * e3x + e3y * e3y + e3z * e3z);
  if (aa != RG_ZERO) aa = RG_ONE / aa;
  e3x = e3x * aa;
  e3y = e3y * aa;
  e3z = e3z * aa;
  const double e2x = e3y * e1z - e3z * e1y, e2y = e3z * e1x - e3x * e1z,
               e2z = e3x * e1y - e3y * e1x;
  R[0] = e1x; R[1] = e2x; R[2] = e3x;
  R[3] = e1y; R[4] = e2y; R[5] = e3y;
  R[6] = e1z; R[7] = e2z; R[8] = e3z;
}

void hexa_group(Model &M, const HexaGroup &G, double &dt2t, int &neltst) {
  HexaLocal L;
  const int nel = G.nel, nft = G.nft, NE = M.numels;
  double *SIG = M.sig.data();
  const double DT1 = M.dt1;

  // SCOOR3 gather (scoor3.F: NC, XD from X, OFF from OFFG, V)
  for (int i = 0; i < nel; i++) {
    const int e = nft + i;
    for (int k = 0; k < 8; k++) L.nc[k][i] = M.ixs[11 * e + 1 + k] - 1;
    const double og = M.offg[e];
    L.off[i] = std::fabs(og);
    for (int k = 0; k < 8; k++) {
      const int n = L.nc[k][i];
      L.x[k][i] = M.X[3 * n + 0];
      L.y[k][i] = M.X[3 * n + 1];
      L.z[k][i] = M.X[3 * n + 2];
      if (og < RG_ZERO) {
        L.vx[k][i] = L.vy[k][i] = L.vz[k][i] = RG_ZERO;
      } else {
        L.vx[k][i] = M.V[3 * n + 0];
        L.vy[k][i] = M.V[3 * n + 1];
        L.vz[k][i] = M.V[3 * n + 2];
      }
    }
  }

  // SRCOOR3 (srcoor3.F), JCVT=1: element frame, then coordinates and
  // velocities in it (X_loc = R^T X; SRROTA3 with the transposed frame)
  if (G.jcvt) {
    for (int i = 0; i < nel; i++) {
      double xs[8], ys[8], zs[8], R[9];
      for (int k = 0; k < 8; k++) {
        xs[k] = L.x[k][i];
        ys[k] = L.y[k][i];
        zs[k] = L.z[k][i];
      }
      hexa_frame(xs, ys, zs, R);
      for (int c = 0; c < 9; c++) L.r[c][i] = R[c];
      for (int k = 0; k < 8; k++) {
        const double X = L.x[k][i], Y = L.y[k][i], Z = L.z[k][i];
        L.x[k][i] = R[0] * X + R[3] * Y + R[6] * Z;
        L.y[k][i] = R[1] * X + R[4] * Y + R[7] * Z;
        L.z[k][i] = R[2] * X + R[5] * Y + R[8] * Z;
        const double U = L.vx[k][i], V = L.vy[k][i], W = L.vz[k][i];
        L.vx[k][i] = R[0] * U + R[3] * V + R[6] * W;
        L.vy[k][i] = R[1] * U + R[4] * V + R[7] * W;
        L.vz[k][i] = R[2] * U + R[5] * V + R[8] * W;
      }
    }
  }

  // SDERI3 (sderi3.F:32-339): Jacobian, volume, PX/PY/PZ, hourglass PH.
  for (int i = 0; i < nel; i++) {
    const double *X1 = &L.x[0][i];
    (void)X1;
    double x17 = L.x[6][i] - L.x[0][i], x28 = L.x[7][i] - L.x[1][i];
    double x35 = L.x[4][i] - L.x[2][i], x46 = L.x[5][i] - L.x[3][i];
    double y17 = L.y[6][i] - L.y[0][i], y28 = L.y[7][i] - L.y[1][i];
    double y35 = L.y[4][i] - L.y[2][i], y46 = L.y[5][i] - L.y[3][i];
    double z17 = L.z[6][i] - L.z[0][i], z28 = L.z[7][i] - L.z[1][i];
    double z35 = L.z[4][i] - L.z[2][i], z46 = L.z[5][i] - L.z[3][i];
    double jac1 = x17 + x28 - x35 - x46;
    double jac2 = y17 + y28 - y35 - y46;
    double jac3 = z17 + z28 - z35 - z46;
    double x_17_46 = x17 + x46, x_28_35 = x28 + x35;
    double y_17_46 = y17 + y46, y_28_35 = y28 + y35;
    double z_17_46 = z17 + z46, z_28_35 = z28 + z35;
    double jac4 = x_17_46 + x_28_35, jac5 = y_17_46 + y_28_35,
           jac6 = z_17_46 + z_28_35;
    double jac7 = x_17_46 - x_28_35, jac8 = y_17_46 - y_28_35,
           jac9 = z_17_46 - z_28_35;
    double j5968 = jac5 * jac9 - jac6 * jac8;
    double j6749 = jac6 * jac7 - jac4 * jac9;
    double j4857 = jac4 * jac8 - jac5 * jac7;
    double det = RG_ONE_OVER_64 * (jac1 * j5968 + jac2 * j6749 + jac3 * j4857);
    // SCHKJABT3 (solide4/schkjabt3.F), Lagrangian, ISMSTR=4: a non-positive
    // volume of a live element stops the run (INEG_V=0: element switched off,
    // MSTOP=1).  Here: the element is switched off and the error is flagged.
    if (L.off[i] == RG_ZERO) {
      det = RG_ONE;
    } else if (det <= RG_ZERO) {
      det = RG_ONE;
      L.off[i] = RG_ZERO;
      M.offg[nft + i] = RG_ZERO;
      M.error |= 1;
    }
    L.voln[i] = det;
    double dett = RG_ONE_OVER_64 / det;
    double jaci1 = dett * j5968;
    double jaci4 = dett * j6749;
    double jaci7 = dett * j4857;
    double jaci2 = dett * (jac3 * jac8 - jac2 * jac9);
    double jaci5 = dett * (jac1 * jac9 - jac3 * jac7);
    double jaci8 = dett * (jac2 * jac7 - jac1 * jac8);
    double jaci3 = dett * (jac2 * jac6 - jac3 * jac5);
    double jaci6 = dett * (jac3 * jac4 - jac1 * jac6);
    double jaci9 = dett * (jac1 * jac5 - jac2 * jac4);
    double jac12 = jaci1 + jaci2, jac45 = jaci4 + jaci5, jac78 = jaci7 + jaci8;
    L.px[0][i] = -jac12 - jaci3;
    L.py[0][i] = -jac45 - jaci6;
    L.pz[0][i] = -jac78 - jaci9;
    L.px[1][i] = -jac12 + jaci3;
    L.py[1][i] = -jac45 + jaci6;
    L.pz[1][i] = -jac78 + jaci9;
    jac12 = jaci1 - jaci2;
    jac45 = jaci4 - jaci5;
    jac78 = jaci7 - jaci8;
    L.px[2][i] = jac12 + jaci3;
    L.py[2][i] = jac45 + jaci6;
    L.pz[2][i] = jac78 + jaci9;
    L.px[3][i] = jac12 - jaci3;
    L.py[3][i] = jac45 - jaci6;
    L.pz[3][i] = jac78 - jaci9;
    // JHBE /= 0: hourglass projections (sderi3.F, three H vectors)
    const double *xx[8], *yy[8], *zz[8];
    for (int k = 0; k < 8; k++) {
      xx[k] = &L.x[k][i];
      yy[k] = &L.y[k][i];
      zz[k] = &L.z[k][i];
    }
#define XK(k) (*xx[(k)-1])
#define YK(k) (*yy[(k)-1])
#define ZK(k) (*zz[(k)-1])
    double hx, hy, hz;
    hx = (XK(1) - XK(2) + XK(3) - XK(4) + XK(5) - XK(6) + XK(7) - XK(8));
    hy = (YK(1) - YK(2) + YK(3) - YK(4) + YK(5) - YK(6) + YK(7) - YK(8));
    hz = (ZK(1) - ZK(2) + ZK(3) - ZK(4) + ZK(5) - ZK(6) + ZK(7) - ZK(8));
    for (int k = 0; k < 4; k++)
      L.ph[k][0][i] = L.px[k][i] * hx + L.py[k][i] * hy + L.pz[k][i] * hz;
    hx = (XK(1) + XK(2) - XK(3) - XK(4) - XK(5) - XK(6) + XK(7) + XK(8));
    hy = (YK(1) + YK(2) - YK(3) - YK(4) - YK(5) - YK(6) + YK(7) + YK(8));
    hz = (ZK(1) + ZK(2) - ZK(3) - ZK(4) - ZK(5) - ZK(6) + ZK(7) + ZK(8));
    for (int k = 0; k < 4; k++)
      L.ph[k][1][i] = L.px[k][i] * hx + L.py[k][i] * hy + L.pz[k][i] * hz;
    hx = (XK(1) - XK(2) - XK(3) + XK(4) - XK(5) + XK(6) + XK(7) - XK(8));
    hy = (YK(1) - YK(2) - YK(3) + YK(4) - YK(5) + YK(6) + YK(7) - YK(8));
    hz = (ZK(1) - ZK(2) - ZK(3) + ZK(4) - ZK(5) + ZK(6) + ZK(7) - ZK(8));
    for (int k = 0; k < 4; k++)
      L.ph[k][2][i] = L.px[k][i] * hx + L.py[k][i] * hy + L.pz[k][i] * hz;
#undef XK
#undef YK
#undef ZK
  }

  // SDLEN3 + SLEN (sdlen3.F:39-172, slen.F:30): DELTAX = 4 V / sqrt(max A^2)
  {
    static const int face[6][4] = {{0, 1, 2, 3}, {4, 5, 6, 7}, {0, 1, 5, 4},
                                   {1, 2, 6, 5}, {2, 3, 7, 6}, {3, 0, 4, 7}};
    for (int i = 0; i < nel; i++) {
      double aream = RG_EM20;
      for (int j = 0; j < 6; j++) {
        const int a = face[j][0], b = face[j][1], c = face[j][2], d = face[j][3];
        double x13 = L.x[c][i] - L.x[a][i], x24 = L.x[d][i] - L.x[b][i];
        double y13 = L.y[c][i] - L.y[a][i], y24 = L.y[d][i] - L.y[b][i];
        double z13 = L.z[c][i] - L.z[a][i], z24 = L.z[d][i] - L.z[b][i];
        double fs1 = x13 - x24, ft1 = x13 + x24;
        double fs2 = y13 - y24, ft2 = y13 + y24;
        double fs3 = z13 - z24, ft3 = z13 + z24;
        double e = fs1 * fs1 + fs2 * fs2 + fs3 * fs3;
        double f = fs1 * ft1 + fs2 * ft2 + fs3 * ft3;
        double g = ft1 * ft1 + ft2 * ft2 + ft3 * ft3;
        double area = e * g - f * f;
        aream = std::max(area, aream);
      }
      L.deltax[i] = RG_FOUR * L.voln[i] * RG_ONE / std::sqrt(aream);
    }
  }

  // SDEFO3 (sdefo3.F:32-313), JHBE=1, JCVT=0 branch.
  const double dt1d2 = RG_HALF * DT1;
  for (int i = 0; i < nel; i++) {
    double vx17 = L.vx[0][i] - L.vx[6][i], vx28 = L.vx[1][i] - L.vx[7][i];
    double vx35 = L.vx[2][i] - L.vx[4][i], vx46 = L.vx[3][i] - L.vx[5][i];
    double vy17 = L.vy[0][i] - L.vy[6][i], vy28 = L.vy[1][i] - L.vy[7][i];
    double vy35 = L.vy[2][i] - L.vy[4][i], vy46 = L.vy[3][i] - L.vy[5][i];
    double vz17 = L.vz[0][i] - L.vz[6][i], vz28 = L.vz[1][i] - L.vz[7][i];
    double vz35 = L.vz[2][i] - L.vz[4][i], vz46 = L.vz[3][i] - L.vz[5][i];
    const double *PX = nullptr;
    (void)PX;
#define P_(a, k) L.a[k][i]
    L.dxx[i] = P_(px, 0) * vx17 + P_(px, 1) * vx28 + P_(px, 2) * vx35 + P_(px, 3) * vx46;
    L.dyy[i] = P_(py, 0) * vy17 + P_(py, 1) * vy28 + P_(py, 2) * vy35 + P_(py, 3) * vy46;
    L.dzz[i] = P_(pz, 0) * vz17 + P_(pz, 1) * vz28 + P_(pz, 2) * vz35 + P_(pz, 3) * vz46;
    L.dxy[i] = P_(py, 0) * vx17 + P_(py, 1) * vx28 + P_(py, 2) * vx35 + P_(py, 3) * vx46;
    L.dxz[i] = P_(pz, 0) * vx17 + P_(pz, 1) * vx28 + P_(pz, 2) * vx35 + P_(pz, 3) * vx46;
    L.dyx[i] = P_(px, 0) * vy17 + P_(px, 1) * vy28 + P_(px, 2) * vy35 + P_(px, 3) * vy46;
    L.dyz[i] = P_(pz, 0) * vy17 + P_(pz, 1) * vy28 + P_(pz, 2) * vy35 + P_(pz, 3) * vy46;
    L.dzx[i] = P_(px, 0) * vz17 + P_(px, 1) * vz28 + P_(px, 2) * vz35 + P_(px, 3) * vz46;
    L.dzy[i] = P_(py, 0) * vz17 + P_(py, 1) * vz28 + P_(py, 2) * vz35 + P_(py, 3) * vz46;
#undef P_
    if (G.jcvt) {
      // JCVT /= 0, explicit (sdefo3.F:158-205): no spin; the midpoint
      // correction of the rates
      L.wxx[i] = L.wyy[i] = L.wzz[i] = RG_ZERO;
      const double exx = L.dxx[i], eyy = L.dyy[i], ezz = L.dzz[i];
      const double exy = L.dxy[i], eyx = L.dyx[i], exz = L.dxz[i];
      const double ezx = L.dzx[i], eyz = L.dyz[i], ezy = L.dzy[i];
      L.dxx[i] = L.dxx[i] - dt1d2 * (exx * exx + eyx * eyx + ezx * ezx);
      L.dyy[i] = L.dyy[i] - dt1d2 * (eyy * eyy + ezy * ezy + exy * exy);
      L.dzz[i] = L.dzz[i] - dt1d2 * (ezz * ezz + exz * exz + eyz * eyz);
      double aaa = dt1d2 * (exx * exy + eyx * eyy + ezx * ezy);
      L.dxy[i] = L.dxy[i] - aaa;
      L.dyx[i] = L.dyx[i] - aaa;
      L.d4[i] = L.dxy[i] + L.dyx[i];
      aaa = dt1d2 * (eyy * eyz + ezy * ezz + exy * exz);
      L.dyz[i] = L.dyz[i] - aaa;
      L.dzy[i] = L.dzy[i] - aaa;
      L.d5[i] = L.dyz[i] + L.dzy[i];
      aaa = dt1d2 * (ezz * ezx + exz * exx + eyz * eyx);
      L.dxz[i] = L.dxz[i] - aaa;
      L.dzx[i] = L.dzx[i] - aaa;
      L.d6[i] = L.dxz[i] + L.dzx[i];
    } else {
      L.d4[i] = L.dxy[i] + L.dyx[i];
      L.d5[i] = L.dyz[i] + L.dzy[i];
      L.d6[i] = L.dxz[i] + L.dzx[i];
      L.wzz[i] = dt1d2 * (L.dyx[i] - L.dxy[i]);
      L.wyy[i] = dt1d2 * (L.dxz[i] - L.dzx[i]);
      L.wxx[i] = dt1d2 * (L.dzy[i] - L.dyz[i]);
    }
  }

  // SRHO3 Lagrangian branch (srho3.F:140-150): VOLO = GBUF%VOL (initial)
  for (int i = 0; i < nel; i++) {
    const int e = nft + i;
    L.divde[i] = DT1 * (L.dxx[i] + L.dyy[i] + L.dzz[i]);
    if (M.offg[e] == RG_ZERO && L.voln[i] == RG_ONE) L.voln[i] = M.vol[e];
    L.dvol[i] = L.voln[i] - (G.rho0 / M.rho[e]) * M.vol[e];
    M.rho[e] = G.rho0 * (M.vol[e] / L.voln[i]);
    M.eint[e] = M.eint[e] * M.vol[e];
  }

  // SROTA3 (srota3.F:40-97): Jaumann rotation; S = stress before rotation.
  // JCVT=1: SRMALLA3 (srmall3.F) only copies the stress, kept in the
  // element frame.
  for (int i = 0; i < nel; i++) {
    const int e = nft + i;
    for (int c = 0; c < 6; c++) L.s[c][i] = SIG[c * NE + e];
    if (G.jcvt) continue;
    const double s1 = L.s[0][i], s2 = L.s[1][i], s3 = L.s[2][i],
                 s4 = L.s[3][i], s5 = L.s[4][i], s6 = L.s[5][i];
    const double q1 = RG_TWO * s4 * L.wzz[i];
    const double q2 = RG_TWO * s6 * L.wyy[i];
    const double q3 = RG_TWO * s5 * L.wxx[i];
    SIG[0 * NE + e] = s1 - q1 + q2;
    SIG[1 * NE + e] = s2 + q1 - q3;
    SIG[2 * NE + e] = s3 - q2 + q3;
    SIG[3 * NE + e] = s4 + L.wzz[i] * (s1 - s2) + L.wyy[i] * s5 - L.wxx[i] * s6;
    SIG[4 * NE + e] = s5 + L.wxx[i] * (s2 - s3) + L.wzz[i] * s6 - L.wyy[i] * s4;
    SIG[5 * NE + e] = s6 + L.wyy[i] * (s3 - s1) + L.wxx[i] * s4 - L.wzz[i] * s5;
  }

  // MMAIN prologue (mmain.F90:676-760): VOL_AVG, AMU (LAW1/2), RHOREF=RHO
  for (int i = 0; i < nel; i++) {
    const int e = nft + i;
    L.vol_avg[i] = L.voln[i] - RG_HALF * L.dvol[i];
    L.amu[i] = M.rho[e] / G.rho0 - RG_ONE;
  }

  // ---- material law: deviatoric update + radial return -------------------
  double dpla[MVSIZ];
  if (G.mtn == 1) {
    // M1LAW (m1law.F:35-190) first loop
    for (int i = 0; i < nel; i++) {
      const int e = nft + i;
      const double gg = G.g * L.off[i];
      const double g1 = DT1 * gg, g2 = RG_TWO * g1;
      L.ssp[i] = std::sqrt((RG_ONEP333 * gg + G.c1) / G.rho0);
      double *sg[6];
      for (int c = 0; c < 6; c++) sg[c] = &SIG[c * NE + e];
      const double p = -RG_THIRD * (*sg[0] + *sg[1] + *sg[2]);
      const double dav = -RG_THIRD * (L.dxx[i] + L.dyy[i] + L.dzz[i]);
      *sg[0] = *sg[0] + p + g2 * (L.dxx[i] + dav);
      *sg[1] = *sg[1] + p + g2 * (L.dyy[i] + dav);
      *sg[2] = *sg[2] + p + g2 * (L.dzz[i] + dav);
      *sg[3] = *sg[3] + g1 * L.d4[i];
      *sg[4] = *sg[4] + g1 * L.d5[i];
      *sg[5] = *sg[5] + g1 * L.d6[i];
    }
  } else {
    // M2LAW (m2law.F:38-580), Johnson-Cook, FISOKIN = 0, IFORM = 0, no
    // thermal (TSTAR = 0), explicit (IMPL_S = 0).
    const double asrate = std::min(RG_ONE, G.asrate * DT1);
    for (int i = 0; i < nel; i++) {
      const int e = nft + i;
      const double gg = G.g * L.off[i];
      double *sg[6];
      for (int c = 0; c < 6; c++) sg[c] = &SIG[c * NE + e];
      const double p = -RG_THIRD * (*sg[0] + *sg[1] + *sg[2]);
      const double dav = -RG_THIRD * (L.dxx[i] + L.dyy[i] + L.dzz[i]);
      const double g1 = DT1 * gg, g2 = RG_TWO * g1;
      L.ssp[i] = std::sqrt((RG_ONEP333 * gg + G.c1) / G.rho0);
      *sg[0] = *sg[0] + p + g2 * (L.dxx[i] + dav);
      *sg[1] = *sg[1] + p + g2 * (L.dyy[i] + dav);
      *sg[2] = *sg[2] + p + g2 * (L.dzz[i] + dav);
      *sg[3] = *sg[3] + g1 * L.d4[i];
      *sg[4] = *sg[4] + g1 * L.d5[i];
      *sg[5] = *sg[5] + g1 * L.d6[i];
      double aj2 = RG_HALF * (*sg[0] * *sg[0] + *sg[1] * *sg[1] + *sg[2] * *sg[2]) +
                   *sg[3] * *sg[3] + *sg[4] * *sg[4] + *sg[5] * *sg[5];
      aj2 = std::sqrt(RG_THREE * aj2);
      // MSTRAIN_RATE (mstrain_rate.F), IDEV = VP-2
      if (G.israte >= 0) {
        double epsdot;
        if (G.vp - 2 == 0) {
          const double e1 = L.dxx[i], e2 = L.dyy[i], e3 = L.dzz[i];
          const double e4 = RG_HALF * L.d4[i], e5 = RG_HALF * L.d5[i],
                       e6 = RG_HALF * L.d6[i];
          const double epsp = e1 * e1 + e2 * e2 + e3 * e3 +
                              RG_TWO * (e4 * e4 + e5 * e5 + e6 * e6);
          epsdot = std::sqrt(epsp);
        } else {
          const double dv = (L.dxx[i] + L.dyy[i] + L.dzz[i]) * RG_THIRD;
          const double e1 = L.dxx[i] - dv, e2 = L.dyy[i] - dv, e3 = L.dzz[i] - dv;
          const double e4 = RG_HALF * L.d4[i], e5 = RG_HALF * L.d5[i],
                       e6 = RG_HALF * L.d6[i];
          const double epsp = RG_HALF * (e1 * e1 + e2 * e2 + e3 * e3) +
                              e4 * e4 + e5 * e5 + e6 * e6;
          epsdot = std::sqrt(RG_THREE * epsp) / RG_THREE_HALF;
        }
        if (G.israte == 0)
          M.epsd[e] = epsdot;
        else
          M.epsd[e] = asrate * epsdot + (RG_ONE - asrate) * M.epsd[e];
      }
      double epd = RG_ONE, sigmx = G.sigm0;
      if (G.cc != RG_ZERO) {
        if (G.vp == 1) {
          epd = std::max(M.epsd[e], G.epdr);
          epd = std::log(epd / G.epdr);
        } else {
          epd = std::max(M.epsd[e], RG_EM15);
          epd = std::log(epd / G.epdr);
        }
        const double mt = std::max(RG_EM15, G.z3);
        epd = std::max(RG_ZERO, epd);
        epd = (RG_ONE + G.cc * epd) * (RG_ONE - std::pow(RG_ZERO, mt));
        if (G.icc == 1) sigmx = G.sigm0 * epd;
      } else {
        const double mt = std::max(RG_EM15, G.z3);
        epd = RG_ONE - std::pow(RG_ZERO, mt);
        if (G.icc == 1) sigmx = G.sigm0 * epd;
      }
      const double epxe = M.pla[e];
      double ak, qh;
      if (G.cn == RG_ONE) {
        ak = G.ca + G.cb * epxe;
        qh = G.cb * epd;
      } else if (epxe > RG_ZERO) {
        ak = G.ca + G.cb * std::pow(epxe, G.cn);
        if (G.cn > RG_ONE)
          qh = (G.cb * G.cn * std::pow(epxe, G.cn - RG_ONE)) * epd;
        else
          qh = (G.cb * G.cn / std::pow(epxe, RG_ONE - G.cn)) * epd;
      } else {
        ak = G.ca;
        qh = RG_ZERO;
      }
      ak = ak * epd;
      if (sigmx < ak) {
        ak = sigmx;
        qh = RG_ZERO;
      }
      if (epxe > G.epmx) {
        ak = RG_ZERO;
        qh = RG_ZERO;
      }
      double scale = std::min(RG_ONE, ak / std::max(aj2, RG_EM15));
      dpla[i] = (RG_ONE - scale) * aj2 / std::max(RG_THREE * gg + qh, RG_EM15);
      ak = ak + (RG_ONE - G.fisokin) * dpla[i] * qh;
      scale = std::min(RG_ONE, ak / std::max(aj2, RG_EM15));
      for (int c = 0; c < 6; c++) *sg[c] = scale * *sg[c];
      M.pla[e] = epxe + dpla[i];
    }
  }

  // MQVISCB (mqviscb.F:44-600): explicit, 3D, one point (FACPG = 1),
  // VISI = 1, FACQ = 1; VOL = VNEW, VOL0 = initial volume.
  for (int i = 0; i < nel; i++) {
    const int e = nft + i;
    const double dd = -L.dxx[i] - L.dyy[i] - L.dzz[i];
    double al = RG_ZERO, ad = RG_ZERO;
    const double cx = L.ssp[i] + std::sqrt(RG_ZERO);  // VD2 = 0 (Lagrange)
    if (L.off[i] == RG_ONE) {
      if (L.voln[i] > RG_ZERO)
        al = std::pow(L.voln[i], RG_ONE / RG_THREE);
      else
        al = RG_ZERO;
      ad = std::max(RG_ZERO, dd);
    }
    const double rhoe = M.rho[e];
    const double nrho = std::sqrt(rhoe * G.rho0);  // RHOREF = RHO (ISMSTR 4)
    const double qa = RG_ONE * G.qa, qb = RG_ONE * G.qb;
    const double cns1 = RG_ONE * G.vns1 * al * nrho * L.ssp[i] * L.off[i];
    const double cns2 = RG_ONE * G.vns2 * al * nrho * L.ssp[i] * L.off[i];
    const double qaa = qa * qa * ad;
    const double vis = RG_ZERO;
    const double qx = qb * L.ssp[i] + al * qaa +
                      RG_ONE * RG_TWO * vis / std::max(RG_EM20, rhoe * L.deltax[i]) +
                      (cns1 + RG_ONE * cns2) / std::max(RG_EM20, rhoe * L.deltax[i]);
    L.qnew[i] = rhoe * ad * al * (qaa * al + qb * L.ssp[i]);
    L.ssp_eq[i] = std::max(RG_EM20, qx + std::sqrt(qx * qx + cx * cx));
    double dtx = L.deltax[i] / L.ssp_eq[i];
    // STI (ISMSTR /= 1, 11): STI = (RHO/DTX) * (VOL/DTX)
    L.sti[i] = RG_ZERO;
    if (!(L.off[i] == RG_ZERO || M.offg[e] < RG_ZERO)) {
      const double tidt = RG_ONE / dtx;
      const double trho = rhoe * tidt;
      const double tvol = L.voln[i] * tidt;
      L.sti[i] = trho * tvol;
    }
    dtx = M.dtfac_solid * dtx;
    // NODADT = 0: DT2T = min over live elements (mqviscb.F:520-535); under
    // the nodal time step the elements only provide STI (mqviscb.F:351)
    if (!M.nodadt && L.voln[i] > RG_ZERO && (L.off[i] != RG_ZERO && M.offg[e] >= RG_ZERO)) {
      if (!(dtx > dt2t)) {
        dt2t = dtx;
        neltst = e;
      }
    }
  }

  // Law epilogue: pressure, energy, QOLD (m1law.F:170-190, m2law.F:430-460)
  const double dta = RG_HALF * DT1;
  for (int i = 0; i < nel; i++) {
    const int e = nft + i;
    double *sg[6];
    for (int c = 0; c < 6; c++) sg[c] = &SIG[c * NE + e];
    const double pnew = G.c1 * L.amu[i];
    *sg[0] = (*sg[0] - pnew) * L.off[i];
    *sg[1] = (*sg[1] - pnew) * L.off[i];
    *sg[2] = (*sg[2] - pnew) * L.off[i];
    *sg[3] = *sg[3] * L.off[i];
    *sg[4] = *sg[4] * L.off[i];
    *sg[5] = *sg[5] * L.off[i];
    double einc;
    if (G.mtn == 1) {
      const double p2 = -(L.s[0][i] + *sg[0] + L.s[1][i] + *sg[1] + L.s[2][i] + *sg[2]) *
                        RG_THIRD;
      const double e1 = L.dxx[i] * (L.s[0][i] + *sg[0] + p2);
      const double e2 = L.dyy[i] * (L.s[1][i] + *sg[1] + p2);
      const double e3 = L.dzz[i] * (L.s[2][i] + *sg[2] + p2);
      const double e4 = L.d4[i] * (L.s[3][i] + *sg[3]);
      const double e5 = L.d5[i] * (L.s[4][i] + *sg[4]);
      const double e6 = L.d6[i] * (L.s[5][i] + *sg[5]);
      einc = L.vol_avg[i] * (e1 + e2 + e3 + e4 + e5 + e6) * dta -
             RG_HALF * L.dvol[i] * (M.qvis[e] + L.qnew[i] + p2);
    } else {
      const double e1 = L.dxx[i] * (L.s[0][i] + *sg[0]);
      const double e2 = L.dyy[i] * (L.s[1][i] + *sg[1]);
      const double e3 = L.dzz[i] * (L.s[2][i] + *sg[2]);
      const double e4 = L.d4[i] * (L.s[3][i] + *sg[3]);
      const double e5 = L.d5[i] * (L.s[4][i] + *sg[4]);
      const double e6 = L.d6[i] * (L.s[5][i] + *sg[5]);
      einc = L.vol_avg[i] * (e1 + e2 + e3 + e4 + e5 + e6) * dta -
             RG_HALF * L.dvol[i] * (M.qvis[e] + L.qnew[i]);
    }
    M.eint[e] = (M.eint[e] + einc * L.off[i]) / std::max(RG_EM15, M.vol[e]);
    M.qvis[e] = L.qnew[i];
  }

  // SMALLB3 (smallb3.F:45): OFF < 1 propagates to OFFG
  for (int i = 0; i < nel; i++) {
    const int e = nft + i;
    if (L.off[i] < RG_ONE) {
      if (L.off[i] == RG_ZERO)
        M.offg[e] = RG_ZERO;
      else if (M.offg[e] > RG_ONE)
        M.offg[e] = RG_ONE + L.off[i];
      else
        M.offg[e] = L.off[i];
    }
  }

  // SHVIS3 (shvis3.F:31-473), IINT=1, JHBE>=1, ISMSTR=4 (not 1, 2).
  for (int i = 0; i < nel; i++) {
    const int e = nft + i;
    const double caq = RG_FOURTH * L.off[i] * G.qh;
    double fcl = caq * M.rho[e] * std::pow(L.voln[i], RG_TWO_THIRD);
    const double fcq = fcl * caq * RG_HUNDRED;
    fcl = fcl * L.ssp[i];
    const double *vx = &L.vx[0][0], *vy = &L.vy[0][0], *vz = &L.vz[0][0];
    (void)vx; (void)vy; (void)vz;
#define VX(k) L.vx[(k)-1][i]
#define VY(k) L.vy[(k)-1][i]
#define VZ(k) L.vz[(k)-1][i]
#define PH(k, j) L.ph[(k)-1][(j)-1][i]
    double g[8][3];
    g[0][0] = RG_ONE - PH(1, 1);
    g[1][0] = -RG_ONE - PH(2, 1);
    g[2][0] = RG_ONE - PH(3, 1);
    g[3][0] = -RG_ONE - PH(4, 1);
    g[4][0] = RG_ONE + PH(3, 1);
    g[5][0] = -RG_ONE + PH(4, 1);
    g[6][0] = RG_ONE + PH(1, 1);
    g[7][0] = -RG_ONE + PH(2, 1);
    g[0][1] = RG_ONE - PH(1, 2);
    g[1][1] = RG_ONE - PH(2, 2);
    g[2][1] = -RG_ONE - PH(3, 2);
    g[3][1] = -RG_ONE - PH(4, 2);
    g[4][1] = -RG_ONE + PH(3, 2);
    g[5][1] = -RG_ONE + PH(4, 2);
    g[6][1] = RG_ONE + PH(1, 2);
    g[7][1] = RG_ONE + PH(2, 2);
    g[0][2] = RG_ONE - PH(1, 3);
    g[1][2] = -RG_ONE - PH(2, 3);
    g[2][2] = -RG_ONE - PH(3, 3);
    g[3][2] = RG_ONE - PH(4, 3);
    g[4][2] = -RG_ONE + PH(3, 3);
    g[5][2] = RG_ONE + PH(4, 3);
    g[6][2] = RG_ONE + PH(1, 3);
    g[7][2] = -RG_ONE + PH(2, 3);
    double hgx[4], hgy[4], hgz[4];
    for (int m = 0; m < 3; m++) {
      hgx[m] = g[0][m] * VX(1) + g[1][m] * VX(2) + g[2][m] * VX(3) + g[3][m] * VX(4) +
               g[4][m] * VX(5) + g[5][m] * VX(6) + g[6][m] * VX(7) + g[7][m] * VX(8);
      hgy[m] = g[0][m] * VY(1) + g[1][m] * VY(2) + g[2][m] * VY(3) + g[3][m] * VY(4) +
               g[4][m] * VY(5) + g[5][m] * VY(6) + g[6][m] * VY(7) + g[7][m] * VY(8);
      hgz[m] = g[0][m] * VZ(1) + g[1][m] * VZ(2) + g[2][m] * VZ(3) + g[3][m] * VZ(4) +
               g[4][m] * VZ(5) + g[5][m] * VZ(6) + g[6][m] * VZ(7) + g[7][m] * VZ(8);
    }
    hgx[3] = VX(1) - VX(2) + VX(3) - VX(4) - VX(5) + VX(6) - VX(7) + VX(8);
    hgy[3] = VY(1) - VY(2) + VY(3) - VY(4) - VY(5) + VY(6) - VY(7) + VY(8);
    hgz[3] = VZ(1) - VZ(2) + VZ(3) - VZ(4) - VZ(5) + VZ(6) - VZ(7) + VZ(8);
    double hx[4], hy[4], hz[4];
    for (int m = 0; m < 4; m++) {
      hx[m] = hgx[m] * (fcl + std::fabs(hgx[m]) * fcq);
      hy[m] = hgy[m] * (fcl + std::fabs(hgy[m]) * fcq);
      hz[m] = hgz[m] * (fcl + std::fabs(hgz[m]) * fcq);
    }
    static const double s4[8] = {-1, 1, -1, 1, 1, -1, 1, -1};
    for (int k = 0; k < 8; k++) {
      // F1k = -G k1*HX1 - G k2*HX2 - G k3*HX3 +/- HX4
      const double *gk = g[k];
      if (s4[k] < 0) {
        L.f[0][k][i] = -gk[0] * hx[0] - gk[1] * hx[1] - gk[2] * hx[2] - hx[3];
        L.f[1][k][i] = -gk[0] * hy[0] - gk[1] * hy[1] - gk[2] * hy[2] - hy[3];
        L.f[2][k][i] = -gk[0] * hz[0] - gk[1] * hz[1] - gk[2] * hz[2] - hz[3];
      } else {
        L.f[0][k][i] = -gk[0] * hx[0] - gk[1] * hx[1] - gk[2] * hx[2] + hx[3];
        L.f[1][k][i] = -gk[0] * hy[0] - gk[1] * hy[1] - gk[2] * hy[2] + hy[3];
        L.f[2][k][i] = -gk[0] * hz[0] - gk[1] * hz[1] - gk[2] * hz[2] + hz[3];
      }
    }
    const double ehou =
        DT1 * (hz[0] * hgz[0] + hz[1] * hgz[1] + hz[2] * hgz[2] + hz[3] * hgz[3] +
               hx[0] * hgx[0] + hx[1] * hgx[1] + hx[2] * hgx[2] + hx[3] * hgx[3] +
               hy[0] * hgy[0] + hy[1] * hgy[1] + hy[2] * hgy[2] + hy[3] * hgy[3]);
    M.ehou[e] += ehou;
#undef VX
#undef VY
#undef VZ
#undef PH
  }

  // SFINT3 Lagrangian branch (sfint3.F:257-361): S = (SIG - QVIS) * VOLN
  for (int i = 0; i < nel; i++) {
    const int e = nft + i;
    const double q = L.qnew[i], v = L.voln[i];
    const double s1 = (SIG[0 * NE + e] + RG_ZERO - q) * v;
    const double s2 = (SIG[1 * NE + e] + RG_ZERO - q) * v;
    const double s3 = (SIG[2 * NE + e] + RG_ZERO - q) * v;
    const double s4 = (SIG[3 * NE + e] + RG_ZERO) * v;
    const double s5 = (SIG[4 * NE + e] + RG_ZERO) * v;
    const double s6 = (SIG[5 * NE + e] + RG_ZERO) * v;
    // nodes (1,7) (2,8) (3,5) (4,6) share P with opposite sign
    static const int pa[4] = {0, 1, 2, 3}, pb[4] = {6, 7, 4, 5};
    for (int j = 0; j < 4; j++) {
      const double px = L.px[j][i], py = L.py[j][i], pz = L.pz[j][i];
      double fint = s1 * px + s4 * py + s6 * pz;
      L.f[0][pa[j]][i] = L.f[0][pa[j]][i] - fint;
      L.f[0][pb[j]][i] = L.f[0][pb[j]][i] + fint;
      fint = s2 * py + s4 * px + s5 * pz;
      L.f[1][pa[j]][i] = L.f[1][pa[j]][i] - fint;
      L.f[1][pb[j]][i] = L.f[1][pb[j]][i] + fint;
      fint = s3 * pz + s6 * px + s5 * py;
      L.f[2][pa[j]][i] = L.f[2][pa[j]][i] - fint;
      L.f[2][pb[j]][i] = L.f[2][pb[j]][i] + fint;
    }
  }

  // SRROTA3 (srrota3.F, sforc3.F:1634-1645), JCVT=1: forces back to the
  // global frame, F = R F_loc
  if (G.jcvt) {
    for (int i = 0; i < nel; i++) {
      const double *R = nullptr;
      double Rl[9];
      for (int c = 0; c < 9; c++) Rl[c] = L.r[c][i];
      R = Rl;
      for (int k = 0; k < 8; k++) {
        const double fx = L.f[0][k][i], fy = L.f[1][k][i], fz = L.f[2][k][i];
        L.f[0][k][i] = R[0] * fx + R[1] * fy + R[2] * fz;
        L.f[1][k][i] = R[3] * fx + R[4] * fy + R[5] * fz;
        L.f[2][k][i] = R[6] * fx + R[7] * fy + R[8] * fz;
      }
    }
  }

  // SCUMU3P (scumu3p.F:37-664): zero deleted (OFFG<0) elements, STI/4,
  // write FSKY(1:3,K), FSKY(7,K) at K = IADS(k, e).
  for (int i = 0; i < nel; i++) {
    const int e = nft + i;
    if (M.offg[e] < RG_ZERO)
      for (int c = 0; c < 3; c++)
        for (int k = 0; k < 8; k++) L.f[c][k][i] = RG_ZERO;
    const double sti = RG_FOURTH * L.sti[i];
    for (int k = 0; k < 8; k++) {
      const int K = M.iads[8 * e + k] - 1;
      double *fs = &M.fsky[8 * K];
      fs[0] = L.f[0][k][i];
      fs[1] = L.f[1][k][i];
      fs[2] = L.f[2][k][i];
      fs[6] = sti;
    }
  }
}

}  // namespace

// shells (rg_oracle_shell.cpp)
namespace rg_oracle_shell {
struct Shells;
Shells *create();
void destroy(Shells *);
int group_add(Shells *, int nel, const int *ixc, int npt, const double *pm,
              const double *geo, const double *uparam, const int *iparam,
              const double *thk0, int ismstr, int ithk);
int numelc(const Shells *);
const int *ixc(const Shells *);
int *iadc(Shells *);
void step(Shells *, const double *X, const double *V, const double *VR,
          double *fsky, double dt1, double dtfac, double &dt2t, int &neltst,
          int &error, int nthreads);
void energy(const Shells *, double &eint, double &ehour);
int rwall_add(Shells *, const double *p0, const double *nrm, double dsearch);
void rwall_apply(Shells *, int numnod, const double *X, double *V,
                 const double *A, double dt12);
int get_state(const Shells *, int which, double *out);
int set_frame(Shells *, int ishfram);
void set_nodadt(Shells *, int on);
void set_dtmin(Shells *, int idtmin, double dtmin);
void part_sums(const Shells *, const double *X, const double *V, const int *part, int part0,
               double *out);
int group_count(const Shells *);
}  // namespace rg_oracle_shell

struct OrModelWrap {
  Model m;
  rg_oracle_shell::Shells *sh = nullptr;
  // planar rigid walls
  struct Wall {
    double p0[3], n[3], dsearch;
    std::vector<int> slaves;
  };
  std::vector<Wall> walls;
};

// SBILAN (elements/solid/solide/sbilan.F:118-160) + the hexas' accumulated
// hourglass energy: per element EI = EINT * VOL, XMAS = RHO * VNEW (= RHO0 *
// VOL0: SRHO3 keeps the element mass), the nodes' mean velocity <v> and mean
// square <v^2>, EK = XMAS <v^2> / 2, momentum XMAS <v>, mass if OFF >= 1;
// then the shells (CBILAN).  Sequential over elements into M.psum.
void part_sums(Model &M, rg_oracle_shell::Shells *sh) {
  const int nhg = (int)M.hg.size();
  const int npart = M.part_hexa.empty() && M.part_shell.empty()
                        ? M.nhexa_adds + rg_oracle_shell::group_count(sh)
                        : M.npart;
  M.psum.assign(7 * (size_t)npart, 0.0);
  for (int g = 0; g < nhg; g++) {
    const HexaGroup &G = M.hg[g];
    for (int i = 0; i < G.nel; i++) {
      const int e = G.nft + i;
      double vx[8], vy[8], vz[8];
      for (int k = 0; k < 8; k++) {
        const int n = M.ixs[11 * (size_t)e + 1 + k] - 1;
        vx[k] = M.V[3 * (size_t)n];
        vy[k] = M.V[3 * (size_t)n + 1];
        vz[k] = M.V[3 * (size_t)n + 2];
      }
      double sx = vx[0], sy = vy[0], sz = vz[0];
      for (int k = 1; k < 8; k++) {
        sx = sx + vx[k];
        sy = sy + vy[k];
        sz = sz + vz[k];
      }
      double va2 = vx[0] * vx[0];
      for (int k = 1; k < 8; k++) va2 = va2 + vx[k] * vx[k];
      for (int k = 0; k < 8; k++) va2 = va2 + vy[k] * vy[k];
      for (int k = 0; k < 8; k++) va2 = va2 + vz[k] * vz[k];
      sx = sx * RG_ONE_OVER_8;
      sy = sy * RG_ONE_OVER_8;
      sz = sz * RG_ONE_OVER_8;
      va2 = va2 * RG_ONE_OVER_8;
      const double xmas = G.rho0 * M.vol[e];
      double *o = &M.psum[7 * (size_t)(M.part_hexa.empty() ? G.add : M.part_hexa[e])];
      o[0] += M.eint[e] * M.vol[e];
      o[1] += xmas * va2 * RG_HALF;
      o[2] += xmas * sx;
      o[3] += xmas * sy;
      o[4] += xmas * sz;
      if (M.offg[e] >= RG_ONE) o[5] += xmas;
      o[6] += M.ehou[e];
    }
  }
  rg_oracle_shell::part_sums(sh, M.X.data(), M.V.data(),
                             M.part_shell.empty() ? nullptr : M.part_shell.data(),
                             M.nhexa_adds, M.psum.data());
}

extern "C" {

void *or_model_new(int numnod, const double *x, const double *v,
                   const double *ms, const int *icodt) {
  auto *w = new OrModelWrap();
  Model &M = w->m;
  M.numnod = numnod;
  M.X.assign(x, x + 3 * (size_t)numnod);
  M.V.assign(v, v + 3 * (size_t)numnod);
  M.D.assign(3 * (size_t)numnod, 0.0);
  M.A.assign(3 * (size_t)numnod, 0.0);
  M.AR.assign(3 * (size_t)numnod, 0.0);
  M.VR.assign(3 * (size_t)numnod, 0.0);
  M.DR.assign(3 * (size_t)numnod, 0.0);
  M.FLAST.assign(3 * (size_t)numnod, 0.0);
  M.FRLAST.assign(3 * (size_t)numnod, 0.0);
  M.STIFN.assign(numnod, 0.0);
  M.STIFR.assign(numnod, 0.0);
  M.MS.assign(ms, ms + numnod);
  M.IN.assign(numnod, 0.0);
  M.icodt.assign(numnod, 0);
  if (icodt) M.icodt.assign(icodt, icodt + numnod);
  w->sh = rg_oracle_shell::create();
  return w;
}

void or_model_free(void *m) {
  auto *w = (OrModelWrap *)m;
  if (!w) return;
  rg_oracle_shell::destroy(w->sh);
  delete w;
}

int or_set_inertia(void *m, const double *in) {
  Model &M = ((OrModelWrap *)m)->m;
  M.IN.assign(in, in + M.numnod);
  return 0;
}

int or_hexa_group_add(void *m, int nel, const int *ixs, int mtn,
                      const double *pm, const double *geo,
                      const double *uparam, const int *iparam, int ismstr,
                      int jhbe, int jcvt) {
  Model &M = ((OrModelWrap *)m)->m;
  if (M.finalized || nel <= 0) return -1;
  if (mtn != 1 && mtn != 2) return -2;
  if ((jcvt != 0 && jcvt != 1) || jhbe != 1 || ismstr != 4) return -3;
  // Split into MVSIZ-long groups like the starter (SGRTAILS).
  for (int s = 0; s < nel; s += MVSIZ) {
    HexaGroup G;
    G.add = M.nhexa_adds;
    G.nft = M.numels + s;
    G.nel = std::min(MVSIZ, nel - s);
    G.mtn = mtn;
    G.ismstr = ismstr;
    G.jhbe = jhbe;
    G.jcvt = jcvt;
    G.rho0 = pm[0];
    G.g = pm[21];
    G.c1 = pm[31];
    G.qh = geo[12];
    G.qa = geo[13];
    G.qb = geo[14];
    G.vns1 = geo[15];
    G.vns2 = geo[16];
    if (mtn == 2) {
      G.iform = iparam[0];
      G.icc = iparam[1];
      G.vp = iparam[2];
      G.israte = iparam[3];
      G.ca = uparam[0];
      G.cb = uparam[1];
      G.cn = uparam[2];
      G.epmx = uparam[3];
      G.sigm0 = uparam[4];
      G.cc = uparam[5];
      G.epdr = uparam[6];
      G.fisokin = uparam[7];
      G.asrate = uparam[8];
      G.z3 = uparam[9];
      if (G.iform != 0 || G.fisokin != 0.0) return -4;
      if (pm[68] > 0.0) return -4;  // adiabatic heating: no element temperature
    }
    M.hg.push_back(G);
  }
  const size_t old = M.numels;
  M.numels += nel;
  M.ixs.insert(M.ixs.end(), ixs, ixs + 11 * (size_t)nel);
  // element state: initial values (starter): SIG = 0, EINT = 0, RHO = RHO0,
  // OFF = 1, volume from the initial geometry (computed at finalize).
  M.eint.resize(M.numels, 0.0);
  M.rho.resize(M.numels, pm[0]);
  M.vol.resize(M.numels, 0.0);
  M.qvis.resize(M.numels, 0.0);
  M.offg.resize(M.numels, 1.0);
  M.pla.resize(M.numels, 0.0);
  M.epsd.resize(M.numels, 0.0);
  M.ehou.resize(M.numels, 0.0);
  (void)old;
  M.nhexa_adds += 1;
  return (int)M.hg.size() - 1;
}

int or_shell_group_add(void *m, int nel, const int *ixc, int npt,
                       const double *pm, const double *geo,
                       const double *uparam, const int *iparam,
                       const double *thk0, int ismstr, int ithk) {
  auto *w = (OrModelWrap *)m;
  if (w->m.finalized) return -1;
  return rg_oracle_shell::group_add(w->sh, nel, ixc, npt, pm, geo, uparam,
                                    iparam, thk0, ismstr, ithk);
}

int or_rwall_add(void *m, const double *p0, const double *nrm, double dsearch) {
  auto *w = (OrModelWrap *)m;
  OrModelWrap::Wall W;
  for (int c = 0; c < 3; c++) {
    W.p0[c] = p0[c];
    W.n[c] = nrm[c];
  }
  W.dsearch = dsearch;
  w->walls.push_back(W);
  return (int)w->walls.size() - 1;
}

// Initial hexa volume: the SDERI3 determinant of the initial geometry.
static double hexa_volume(const Model &M, int e) {
  double x[8], y[8], z[8];
  for (int k = 0; k < 8; k++) {
    const int n = M.ixs[11 * e + 1 + k] - 1;
    x[k] = M.X[3 * n];
    y[k] = M.X[3 * n + 1];
    z[k] = M.X[3 * n + 2];
  }
  double x17 = x[6] - x[0], x28 = x[7] - x[1], x35 = x[4] - x[2], x46 = x[5] - x[3];
  double y17 = y[6] - y[0], y28 = y[7] - y[1], y35 = y[4] - y[2], y46 = y[5] - y[3];
  double z17 = z[6] - z[0], z28 = z[7] - z[1], z35 = z[4] - z[2], z46 = z[5] - z[3];
  double jac1 = x17 + x28 - x35 - x46, jac2 = y17 + y28 - y35 - y46,
         jac3 = z17 + z28 - z35 - z46;
  double jac4 = (x17 + x46) + (x28 + x35), jac5 = (y17 + y46) + (y28 + y35),
         jac6 = (z17 + z46) + (z28 + z35);
  double jac7 = (x17 + x46) - (x28 + x35), jac8 = (y17 + y46) - (y28 + y35),
         jac9 = (z17 + z46) - (z28 + z35);
  return RG_ONE_OVER_64 * (jac1 * (jac5 * jac9 - jac6 * jac8) +
                           jac2 * (jac6 * jac7 - jac4 * jac9) +
                           jac3 * (jac4 * jac8 - jac5 * jac7));
}

int or_finalize(void *m, double dtfac_solid, double dtfac_shell, double dtmx,
                double dt2old_init, int nthreads) {
  auto *w = (OrModelWrap *)m;
  Model &M = w->m;
  if (M.finalized) return -1;
  M.dtfac_solid = dtfac_solid;
  M.dtfac_shell = dtfac_shell;
  M.dtmx = dtmx;
  M.dt2old = dt2old_init;
  M.nthreads = nthreads > 0 ? nthreads : 1;
  // sig 6 x numels SoA
  M.sig.assign(6 * (size_t)M.numels, 0.0);
  for (int e = 0; e < M.numels; e++) M.vol[e] = hexa_volume(M, e);

  // FILLCNE (starter/source/spmd/domdec2.F:2046-2250): per node, solids in
  // increasing user-id order (stable), then shells in increasing user-id
  // order.  W_PON (restart/ddsplit/w_pon.F:581-700) turns CNE positions
  // into IADS / IADC slot numbers.
  const int numelc = rg_oracle_shell::numelc(w->sh);
  const int *ixc = rg_oracle_shell::ixc(w->sh);
  std::vector<int> cnt(M.numnod + 2, 0);
  for (int e = 0; e < M.numels; e++)
    for (int k = 0; k < 8; k++) cnt[M.ixs[11 * e + 1 + k]]++;
  for (int e = 0; e < numelc; e++)
    for (int k = 0; k < 4; k++) cnt[ixc[7 * e + 1 + k]]++;
  M.adsky.assign(M.numnod + 1, 0);
  M.adsky[0] = 1;
  for (int n = 1; n <= M.numnod; n++) M.adsky[n] = M.adsky[n - 1] + cnt[n];
  M.lsky = M.adsky[M.numnod] - 1;
  std::vector<int> fill(M.adsky.begin(), M.adsky.end() - 1);  // next slot
  std::vector<int> ord(M.numels);
  std::iota(ord.begin(), ord.end(), 0);
  std::stable_sort(ord.begin(), ord.end(), [&](int a, int b) {
    return M.ixs[11 * a + 10] < M.ixs[11 * b + 10];
  });
  M.iads.assign(8 * (size_t)M.numels, 0);
  for (int e : ord)
    for (int k = 0; k < 8; k++) {
      const int n = M.ixs[11 * e + 1 + k];
      M.iads[8 * e + k] = fill[n - 1]++;
    }
  std::vector<int> ordc(numelc);
  std::iota(ordc.begin(), ordc.end(), 0);
  std::stable_sort(ordc.begin(), ordc.end(), [&](int a, int b) {
    return ixc[7 * a + 6] < ixc[7 * b + 6];
  });
  int *iadc = rg_oracle_shell::iadc(w->sh);
  for (int e : ordc)
    for (int k = 0; k < 4; k++) {
      const int n = ixc[7 * e + 1 + k];
      iadc[4 * e + k] = fill[n - 1]++;
    }
  M.fsky.assign(8 * (size_t)std::max(M.lsky, 1), 0.0);

  // rigid-wall slave nodes (all nodes within dsearch of the plane)
  for (auto &W : w->walls) {
    for (int n = 0; n < M.numnod; n++) {
      double d = (M.X[3 * n] - W.p0[0]) * W.n[0] + (M.X[3 * n + 1] - W.p0[1]) * W.n[1] +
                 (M.X[3 * n + 2] - W.p0[2]) * W.n[2];
      if (d <= W.dsearch) W.slaves.push_back(n);
    }
  }
  M.finalized = true;
  return 0;
}

int or_get_skyline(void *m, int *adsky, int *iads, int *iadc, int *lsky) {
  auto *w = (OrModelWrap *)m;
  Model &M = w->m;
  if (!M.finalized) return -1;
  if (adsky) std::copy(M.adsky.begin(), M.adsky.end(), adsky);
  if (iads) std::copy(M.iads.begin(), M.iads.end(), iads);
  if (iadc) {
    const int nc = rg_oracle_shell::numelc(w->sh);
    std::copy(rg_oracle_shell::iadc(w->sh), rg_oracle_shell::iadc(w->sh) + 4 * nc, iadc);
  }
  if (lsky) *lsky = M.lsky;
  return 0;
}

}  // extern "C"

namespace {

// FINTER (tools/curve/finter.F): piecewise-linear load curve; a one-point
// curve is constant; outside the abscissa range the end segments extend
// linearly.  The value is taken from the nearer end of the segment.
double finter(const std::vector<double> &x, const std::vector<double> &y, double t) {
  const size_t n = x.size();
  if (n == 1) return y[0];
  size_t i = 1;
  while (i < n - 1 && x[i] - t < RG_ZERO) i++;
  const double div0 = x[i] - x[i - 1];
  const double div = std::copysign(std::max(std::fabs(div0), 1e-16), div0);
  const double deri = (y[i] - y[i - 1]) / div;
  const double dx1 = t - x[i - 1], dx2 = x[i] - t;
  return dx1 <= dx2 ? y[i - 1] + dx1 * deri : y[i] - dx2 * deri;
}

// ROTBMR (tools/skew/rotbmr.F): turn the principal frame by the rotation
// vector dt*vi given in that frame (Rodrigues' formula, the matrix scaled by
// |r|^2 with |r|^2 >= 1e-10), renormalise e1, e2 and take e3 = e1 x e2.
void rotbmr(const double vi[3], double R[9], double dt) {
  const double rx = dt * vi[0], ry = dt * vi[1], rz = dt * vi[2];
  const double r2 = std::max(1e-10, rx * rx + ry * ry + rz * rz);
  const double r = std::sqrt(r2);
  const double cm1 = RG_ONE - std::cos(r);
  const double c = std::cos(r) * r2;
  const double s = std::sin(r) * r;
  const double e11 = rx * rx * cm1 + c, e22 = ry * ry * cm1 + c;
  const double e12 = rx * ry * cm1 + rz * s, e21 = rx * ry * cm1 - rz * s;
  const double e13 = rx * rz * cm1 - ry * s, e23 = ry * rz * cm1 + rx * s;
  double a[3], b[3];
  for (int k = 0; k < 3; k++) {
    a[k] = R[k] * e11 + R[3 + k] * e12 + R[6 + k] * e13;
    b[k] = R[k] * e21 + R[3 + k] * e22 + R[6 + k] * e23;
  }
  const double na = std::sqrt(a[0] * a[0] + a[1] * a[1] + a[2] * a[2]);
  const double nb = std::sqrt(b[0] * b[0] + b[1] * b[1] + b[2] * b[2]);
  for (int k = 0; k < 3; k++) {
    a[k] = a[k] / na;
    b[k] = b[k] / nb;
  }
  R[0] = a[0], R[1] = a[1], R[2] = a[2];
  R[3] = b[0], R[4] = b[1], R[5] = b[2];
  R[6] = a[1] * b[2] - a[2] * b[1];
  R[7] = a[2] * b[0] - a[0] * b[2];
  R[8] = a[0] * b[1] - a[1] * b[0];
}

// RBYFOR / RGBODFP (constraints/general/rbody/rbyfor.F, rgbodfp.F), after
// the slot assembly: the secondary nodes' forces, moments about the main
// node and stiffnesses go to the main node (summed in secondary order; the
// reference's PARITH/ON sum is order-independent, SUM_6_FLOAT); then, with
// no rotational condition on the main node (ICODR = 0) and a non-spherical
// body, the frame turns by VR*DT1 and the moment becomes the pseudo moment
// IN(M)/I_k (M_k + (I_l - I_m) w_l w_m) in the principal frame, so that
// ACCELE's AR = moment / IN(M) is the Euler angular acceleration.
void rbyfor(Model &M, Model::Body &B) {
  const int m = B.main;
  for (int k = 0; k < 3; k++) B.I[k] = std::max(B.I[k], M.IN[m]);
  double s[8] = {0, 0, 0, 0, 0, 0, 0, 0};
  const double xm = M.X[3 * m], ym = M.X[3 * m + 1], zm = M.X[3 * m + 2];
  for (int n : B.nodes) {
    const double rx = M.X[3 * n] - xm, ry = M.X[3 * n + 1] - ym, rz = M.X[3 * n + 2] - zm;
    const double dd = rx * rx + ry * ry + rz * rz;
    const double f0 = M.A[3 * n], f1 = M.A[3 * n + 1], f2 = M.A[3 * n + 2];
    s[0] = s[0] + M.STIFN[n];
    s[1] = s[1] + (M.STIFR[n] + dd * M.STIFN[n]);
    s[2] = s[2] + f0;
    s[3] = s[3] + f1;
    s[4] = s[4] + f2;
    s[5] = s[5] + (M.AR[3 * n] + ry * f2 - rz * f1);
    s[6] = s[6] + (M.AR[3 * n + 1] + rz * f0 - rx * f2);
    s[7] = s[7] + (M.AR[3 * n + 2] + rx * f1 - ry * f0);
  }
  M.STIFN[m] = M.STIFN[m] + s[0];
  M.STIFR[m] = M.STIFR[m] + s[1];
  for (int k = 0; k < 3; k++) {
    M.A[3 * m + k] = M.A[3 * m + k] + s[2 + k];
    M.AR[3 * m + k] = M.AR[3 * m + k] + s[5 + k];
  }
  double *R = B.R, *vr = &M.VR[3 * m], *am = &M.AR[3 * m];
  const double wa[3] = {am[0], am[1], am[2]};
  double vi[3];
  for (int k = 0; k < 3; k++) vi[k] = R[3 * k] * vr[0] + R[3 * k + 1] * vr[1] + R[3 * k + 2] * vr[2];
  rotbmr(vi, R, M.dt1);
  double ap[3];
  for (int k = 0; k < 3; k++) ap[k] = R[3 * k] * wa[0] + R[3 * k + 1] * wa[1] + R[3 * k + 2] * wa[2];
  ap[0] = ap[0] + (B.I[1] - B.I[2]) * vi[1] * vi[2];
  ap[1] = ap[1] + (B.I[2] - B.I[0]) * vi[2] * vi[0];
  ap[2] = ap[2] + (B.I[0] - B.I[1]) * vi[0] * vi[1];
  double w[3];
  for (int k = 0; k < 3; k++) w[k] = ap[k] * M.IN[m] / B.I[k];
  for (int k = 0; k < 3; k++) am[k] = R[k] * w[0] + R[3 + k] * w[1] + R[6 + k] * w[2];
  for (int n : B.nodes) {
    M.STIFN[n] = RG_EM20;
    M.STIFR[n] = RG_EM20;
  }
}

// RBYVIT / RGBODV (rbyvit.F, rgbodv.F), more than two secondary nodes: every
// secondary node gets the accelerations that make VELOCITY give it the rigid
// motion of the main node, V(M) + A(M)*DT12 + W x r + DT2/2 W x (W x r) and
// W, with W = VR(M) + AR(M)*DT12.  Returns 1 when DT2*|VR(M)| > 1.
int rgbodv(Model &M, const Model::Body &B) {
  const int m = B.main;
  const double *vrm = &M.VR[3 * m];
  int err = 0;
  if (M.dt2 * M.dt2 * (vrm[0] * vrm[0] + vrm[1] * vrm[1] + vrm[2] * vrm[2]) > RG_ONE) err = 1;
  const double vg0 = vrm[0] + M.AR[3 * m] * M.dt12;
  const double vg1 = vrm[1] + M.AR[3 * m + 1] * M.dt12;
  const double vg2 = vrm[2] + M.AR[3 * m + 2] * M.dt12;
  const double usdt = RG_ONE / M.dt12;
  const double am0 = M.A[3 * m], am1 = M.A[3 * m + 1], am2 = M.A[3 * m + 2];
  const double *vm = &M.V[3 * m];
  const double xm = M.X[3 * m], ym = M.X[3 * m + 1], zm = M.X[3 * m + 2];
  const double h = RG_HALF * M.dt2;
  for (int n : B.nodes) {
    M.AR[3 * n] = (vg0 - M.VR[3 * n]) * usdt;
    M.AR[3 * n + 1] = (vg1 - M.VR[3 * n + 1]) * usdt;
    M.AR[3 * n + 2] = (vg2 - M.VR[3 * n + 2]) * usdt;
    const double rx = M.X[3 * n] - xm, ry = M.X[3 * n + 1] - ym, rz = M.X[3 * n + 2] - zm;
    const double vx1 = vg1 * rz - vg2 * ry;
    const double vx2 = vg2 * rx - vg0 * rz;
    const double vx3 = vg0 * ry - vg1 * rx;
    M.A[3 * n] = am0 + (vm[0] + vx1 + h * (vg1 * vx3 - vg2 * vx2) - M.V[3 * n]) * usdt;
    M.A[3 * n + 1] = am1 + (vm[1] + vx2 + h * (vg2 * vx1 - vg0 * vx3) - M.V[3 * n + 1]) * usdt;
    M.A[3 * n + 2] = am2 + (vm[2] + vx3 + h * (vg0 * vx2 - vg1 * vx1) - M.V[3 * n + 2]) * usdt;
  }
  return err;
}

// RMATPON (materials/mat/mat013/rmatpon.F, IFLAG 1 then 2; called by
// RMATFORP at resol.F:5774, after the assembly): the secondary nodes'
// forces and their moments about the body's (initial) centre of mass are
// summed (the reference's SUM_6_FLOAT: order-independent, here in node
// order); without a rotational code the moment, taken to the principal
// frame, gains the gyroscopic term of the body's angular velocity turned by
// ROTBMR over DT1 (a local copy of the axes: RBYM(5:13) keeps its starter
// value) and comes back scaled by IN / I_k; the inertia tensor RBYM(18:26)
// is rebuilt from the turned axes.  Then ARBYM = F / mass, ARRBYM = M / IN,
// the translational code zeroes components, and the secondary nodes' forces,
// moments and stiffnesses are cleared.
void rmatpon(Model &M, Model::RigidMat &B, bool rot) {
  double s[6] = {0, 0, 0, 0, 0, 0};
  for (int n : B.nodes) {
    const double rx = M.X[3 * n] - B.xg[0], ry = M.X[3 * n + 1] - B.xg[1],
                 rz = M.X[3 * n + 2] - B.xg[2];
    const double f0 = M.A[3 * n], f1 = M.A[3 * n + 1], f2 = M.A[3 * n + 2];
    const double m0 = rot ? M.AR[3 * n] : RG_ZERO, m1 = rot ? M.AR[3 * n + 1] : RG_ZERO,
                 m2 = rot ? M.AR[3 * n + 2] : RG_ZERO;
    s[0] = s[0] + f0;
    s[1] = s[1] + f1;
    s[2] = s[2] + f2;
    s[3] = s[3] + (m0 + ry * f2 - rz * f1);
    s[4] = s[4] + (m1 + rz * f0 - rx * f2);
    s[5] = s[5] + (m2 + rx * f1 - ry * f0);
  }
  double *ar = B.ar, *arr = B.arr, *vrr = B.vrr, *J = B.J;
  for (int k = 0; k < 3; k++) {
    ar[k] = s[k];
    arr[k] = s[3 + k];
  }
  double RB[9];
  for (int k = 0; k < 9; k++) RB[k] = B.R[k];
  const double *I = B.I;
  auto rebuild_j = [&]() {
    const double ii1 = I[0] * RB[0], ii2 = I[0] * RB[1], ii3 = I[0] * RB[2];
    const double ii4 = I[1] * RB[3], ii5 = I[1] * RB[4], ii6 = I[1] * RB[5];
    const double ii7 = I[2] * RB[6], ii8 = I[2] * RB[7], ii9 = I[2] * RB[8];
    J[0] = RB[0] * ii1 + RB[3] * ii4 + RB[6] * ii7;
    J[1] = RB[0] * ii2 + RB[3] * ii5 + RB[6] * ii8;
    J[2] = RB[0] * ii3 + RB[3] * ii6 + RB[6] * ii9;
    J[3] = RB[1] * ii1 + RB[4] * ii4 + RB[7] * ii7;
    J[4] = RB[1] * ii2 + RB[4] * ii5 + RB[7] * ii8;
    J[5] = RB[1] * ii3 + RB[4] * ii6 + RB[7] * ii9;
    J[6] = RB[2] * ii1 + RB[5] * ii4 + RB[8] * ii7;
    J[7] = RB[2] * ii2 + RB[5] * ii5 + RB[8] * ii8;
    J[8] = RB[2] * ii3 + RB[5] * ii6 + RB[8] * ii9;
  };
  const int lcod = B.icod[0];
  if (lcod > 0) {
    double vi[3];
    for (int k = 0; k < 3; k++)
      vi[k] = RB[3 * k] * vrr[0] + RB[3 * k + 1] * vrr[1] + RB[3 * k + 2] * vrr[2];
    rotbmr(vi, RB, M.dt1);
    rebuild_j();
    const double wa1 = J[0] * vrr[0] + J[1] * vrr[1] + J[2] * vrr[2];
    const double wa2 = J[3] * vrr[0] + J[4] * vrr[1] + J[5] * vrr[2];
    const double wa3 = J[6] * vrr[0] + J[7] * vrr[1] + J[8] * vrr[2];
    arr[0] = arr[0] + (wa2 * vrr[2] - wa3 * vrr[1]);
    arr[1] = arr[1] + (wa3 * vrr[0] - wa1 * vrr[2]);
    arr[2] = arr[2] + (wa1 * vrr[1] - wa2 * vrr[0]);
    if (lcod == 1) {
      const double det = RG_ONE / (J[0] * J[4] - J[1] * J[3]);
      const double w1 = arr[0], w2 = arr[1];
      arr[0] = (J[4] * w1 - J[3] * w2) * det;
      arr[1] = (-J[1] * w1 + J[0] * w2) * det;
      arr[2] = RG_ZERO;
      vrr[2] = RG_ZERO;
    } else if (lcod == 2) {
      const double det = RG_ONE / (J[0] * J[8] - J[2] * J[6]);
      const double w1 = arr[0], w2 = arr[2];
      arr[0] = (J[8] * w1 - J[6] * w2) * det;
      arr[1] = RG_ZERO;
      arr[2] = (-J[2] * w1 + J[0] * w2) * det;
      vrr[1] = RG_ZERO;
    } else if (lcod == 3) {
      arr[0] = arr[0] / J[0];
      arr[1] = arr[2] = RG_ZERO;
      vrr[1] = vrr[2] = RG_ZERO;
    } else if (lcod == 4) {
      const double det = RG_ONE / (J[4] * J[8] - J[5] * J[7]);
      const double w1 = arr[1], w2 = arr[2];
      arr[0] = RG_ZERO;
      arr[1] = (J[8] * w1 - J[7] * w2) * det;
      arr[2] = (-J[5] * w1 + J[4] * w2) * det;
      vrr[0] = RG_ZERO;
    } else if (lcod == 5) {
      arr[0] = RG_ZERO;
      arr[1] = arr[1] / J[4];
      arr[2] = RG_ZERO;
      vrr[0] = vrr[2] = RG_ZERO;
    } else if (lcod == 6) {
      arr[0] = arr[1] = RG_ZERO;
      arr[2] = arr[2] / J[8];
      vrr[0] = vrr[1] = RG_ZERO;
    } else if (lcod == 7) {
      arr[0] = arr[1] = arr[2] = RG_ZERO;
      vrr[0] = vrr[1] = vrr[2] = RG_ZERO;
    }
  } else {
    const double wa[3] = {arr[0], arr[1], arr[2]};
    for (int k = 0; k < 3; k++)
      arr[k] = RB[3 * k] * wa[0] + RB[3 * k + 1] * wa[1] + RB[3 * k + 2] * wa[2];
    double vi[3];
    for (int k = 0; k < 3; k++)
      vi[k] = RB[3 * k] * vrr[0] + RB[3 * k + 1] * vrr[1] + RB[3 * k + 2] * vrr[2];
    rotbmr(vi, RB, M.dt1);
    arr[0] = arr[0] + ((I[1] - I[2]) * vi[1] * vi[2]);
    arr[1] = arr[1] + ((I[2] - I[0]) * vi[2] * vi[0]);
    arr[2] = arr[2] + ((I[0] - I[1]) * vi[0] * vi[1]);
    double w[3];
    for (int k = 0; k < 3; k++) w[k] = arr[k] * B.in / I[k];
    for (int k = 0; k < 3; k++) arr[k] = RB[k] * w[0] + RB[3 + k] * w[1] + RB[6 + k] * w[2];
    rebuild_j();
  }
  for (int k = 0; k < 3; k++) {
    ar[k] = B.mass > RG_ZERO ? ar[k] / B.mass : RG_ZERO;
    arr[k] = B.in > RG_ZERO ? arr[k] / B.in : RG_ZERO;
  }
  const int tcod = B.icod[1];
  if (tcod & 4) ar[0] = B.vr[0] = RG_ZERO;
  if (tcod & 2) ar[1] = B.vr[1] = RG_ZERO;
  if (tcod & 1) ar[2] = B.vr[2] = RG_ZERO;
  for (int n : B.nodes) {
    for (int k = 0; k < 3; k++) {
      M.A[3 * n + k] = RG_ZERO;
      if (rot) M.AR[3 * n + k] = RG_ZERO;
    }
    M.STIFN[n] = RG_EM20;
    if (rot) M.STIFR[n] = RG_EM20;
  }
}

// RMATACCE (materials/mat/mat013/rmatacce.F, resol.F:7879): the secondary
// nodes take the accelerations that make VELOCITY give them the body's
// motion about its (initial) centre of mass: VG = VRRBYM + ARRBYM*DT12,
// AR = (VG - VR)/DT12, A = ARBYM + (VRBYM + VG x r + DT2/2 VG x (VG x r) -
// V)/DT12; then VRBYM += ARBYM*DT12 and VRRBYM = VG.
void rmatacce(Model &M, Model::RigidMat &B, bool rot) {
  const double usdt = RG_ONE / M.dt12;
  double vg[3];
  for (int k = 0; k < 3; k++) vg[k] = B.vrr[k] + B.arr[k] * M.dt12;
  for (int n : B.nodes) {
    const double rx = M.X[3 * n] - B.xg[0], ry = M.X[3 * n + 1] - B.xg[1],
                 rz = M.X[3 * n + 2] - B.xg[2];
    if (rot)
      for (int k = 0; k < 3; k++) M.AR[3 * n + k] = (vg[k] - M.VR[3 * n + k]) * usdt;
    const double v1x2 = vg[0] * ry, v2x1 = vg[1] * rx, v2x3 = vg[1] * rz;
    const double v3x2 = vg[2] * ry, v3x1 = vg[2] * rx, v1x3 = vg[0] * rz;
    const double vx1 = v2x3 - v3x2, vx2 = v3x1 - v1x3, vx3 = v1x2 - v2x1;
    M.A[3 * n] = B.ar[0] + usdt * (B.vr[0] + vx1 + RG_HALF * M.dt2 * (vg[1] * vx3 - vg[2] * vx2) -
                                   M.V[3 * n]);
    M.A[3 * n + 1] = B.ar[1] + usdt * (B.vr[1] + vx2 +
                                       RG_HALF * M.dt2 * (vg[2] * vx1 - vg[0] * vx3) -
                                       M.V[3 * n + 1]);
    M.A[3 * n + 2] = B.ar[2] + usdt * (B.vr[2] + vx3 +
                                       RG_HALF * M.dt2 * (vg[0] * vx2 - vg[1] * vx1) -
                                       M.V[3 * n + 2]);
  }
  for (int k = 0; k < 3; k++) {
    B.vr[k] = B.vr[k] + B.ar[k] * M.dt12;
    B.vrr[k] = vg[k];
  }
}

// VINTERDP (tools/curve/vinterdp.F): linear interpolation on the segment
// holding t (the first one past the last abscissa below t), extended by the
// end segments.
double vinterdp(const std::vector<double> &x, const std::vector<double> &y, double t) {
  const size_t n = x.size();
  if (n == 1) return y[0];
  size_t j = 0;
  while (j + 2 < n && t > x[j + 1]) j++;
  const double dydx = (y[j + 1] - y[j]) / (x[j + 1] - x[j]);
  return y[j] + dydx * (t - x[j]);
}

// FIXVEL (constraints/general/impvel/fixvel.F:335-346, 367-379, 834-837),
// imposed velocity (IDIS = 1) along a global direction: the velocity
// F((TT + DT2/2) FACX) * FSCALE at mid-step is reached by the acceleration
// (VIMP - V)/DT12; the power DW = 1/4 MS (A DT12 + 2 V)(A - A_before) is
// counted DT1*DW now and DT2*DW at the next cycle.
void fixvel(Model &M) {
  for (auto &F : M.impvels) {
    if (M.tt < F.tstart || M.tt > F.tstop) continue;
    M.wfext = M.wfext + F.vel4;
    F.vel4 = RG_ZERO;
    const double tsc = (M.tt + RG_HALF * M.dt2) * F.facx;
    double yc = vinterdp(F.x, F.y, tsc) * F.fscale;
    const int i = F.node, j = F.dir;
    yc = (yc - M.V[3 * i + j]) / M.dt12;
    const double aold = M.A[3 * i + j];
    M.A[3 * i + j] = yc;
    const double dw = RG_FOURTH * M.MS[i] * (M.A[3 * i + j] * M.dt12 + RG_TWO * M.V[3 * i + j]) *
                      (M.A[3 * i + j] - aold);
    M.wfext = M.wfext + M.dt1 * dw;
    F.vel4 = F.vel4 + M.dt2 * dw;
  }
}

}  // namespace

extern "C" {

// One explicit cycle in RESOL order (engine/source/engine/resol.F).
int or_cycle(void *m, int ncycle) {
  auto *w = (OrModelWrap *)m;
  Model &M = w->m;
  if (!M.finalized) return -1;
  const int numnod = M.numnod;
  const bool shells = rg_oracle_shell::numelc(w->sh) > 0;
  const bool rot = shells || !M.bodies.empty();
  for (int c = 0; c < ncycle; c++) {
    RG_OPCOUNT_PHASE(0);
    // resol.F:2721-2722, 2826: DT1 = DT2, DT2 = 1e6, DT2T = DT2
    M.dt1 = M.dt2;
    M.dt2 = RG_EP06;
    double dt2t = M.dt2;
    int neltst = 0;
    // FORCE (loads/general/force.F90, PARITH/ON branch): a concentrated
    // load adds FCY * F(TT * FCX) to its node; the external work of the
    // cycle is 1/2 (F(TT - DT1) + F(TT)) * V, times the new DT2 once the
    // time step is known (resol.F:6508).  Here the load enters the node's
    // sum ahead of the element slots.
    double wfexc = RG_ZERO;
    for (auto &L : M.loads) {
      const double a0 = L.fcy * finter(L.x, L.y, (M.tt - M.dt1) * L.fcx);
      const double aa = L.fcy * finter(L.x, L.y, M.tt * L.fcx);
      double *acc = L.dir < 3 ? &M.A[3 * L.node + L.dir] : &M.AR[3 * L.node + L.dir - 3];
      const double vel = L.dir < 3 ? M.V[3 * L.node + L.dir] : M.VR[3 * L.node + L.dir - 3];
      *acc = *acc + aa;
      wfexc = wfexc + RG_HALF * (a0 + aa) * vel;
    }
    // FORINT: element groups (OpenMP over groups, forint.F:339).  Each
    // group reports the minimum of DTFAC1*DTX and the last element (group
    // order) attaining it; ties across groups resolve to the larger global
    // element index, i.e. the sequential-order result of MQVISCB.
    const int ng = M.ext ? 0 : (int)M.hg.size();
    std::vector<double> gdt(ng, RG_EP06);
    std::vector<int> gel(ng, -1);
    RG_OPCOUNT_PHASE(1);
#pragma omp parallel for schedule(dynamic, 1) num_threads(M.nthreads)
    for (int g = 0; g < ng; g++) {
      double d = RG_EP06;
      int el = -1;
      hexa_group(M, M.hg[g], d, el);
      gdt[g] = d;
      gel[g] = el;
    }
    RG_OPCOUNT_PHASE(0);
    int eidx = -1;
    for (int g = 0; g < ng; g++)
      if (gel[g] >= 0 && !(gdt[g] > dt2t)) {
        dt2t = gdt[g];
        eidx = gel[g];
      }
    if (eidx >= 0) neltst = M.ixs[11 * eidx + 10];
    if (M.ext && M.ext_dt2t < dt2t) {
      dt2t = M.ext_dt2t;
      neltst = M.ext_neltst;
    }
    if (shells && !M.ext) {
      int err = 0;
      double d = dt2t;
      int el = neltst;
      rg_oracle_shell::step(w->sh, M.X.data(), M.V.data(), M.VR.data(),
                            M.fsky.data(), M.dt1, M.dtfac_shell, d, el, err,
                            M.nthreads);
      M.error |= err;
      if (d < dt2t) {
        dt2t = d;
        neltst = el;
      }
    }
    // part sums of the element pass (SBILAN / CBILAN, taken in the cycles
    // that print): X(n), V(n-1/2), the cycle's element state
    if (M.record && !M.ext) part_sums(M, w->sh);
    // ASSPAR4 (asspar4.F:165-180): fixed-order slot sums
    RG_OPCOUNT_PHASE(3);
#pragma omp parallel for schedule(static) num_threads(M.nthreads)
    for (int n = 0; n < numnod; n++) {
      double a0 = M.A[3 * n], a1 = M.A[3 * n + 1], a2 = M.A[3 * n + 2];
      double r0 = M.AR[3 * n], r1 = M.AR[3 * n + 1], r2 = M.AR[3 * n + 2];
      double st = RG_ZERO, sr = RG_ZERO;
      if (M.ext) {
        a0 = a0 + M.ext_f[3 * n];
        a1 = a1 + M.ext_f[3 * n + 1];
        a2 = a2 + M.ext_f[3 * n + 2];
        st = M.ext_stifn[n];
        if (!M.ext_fr.empty()) {
          r0 = r0 + M.ext_fr[3 * n];
          r1 = r1 + M.ext_fr[3 * n + 1];
          r2 = r2 + M.ext_fr[3 * n + 2];
        }
        if (!M.ext_stifr.empty()) sr = M.ext_stifr[n];
      }
      for (int k = M.adsky[n] - 1; k < (M.ext ? M.adsky[n] - 1 : M.adsky[n + 1] - 1); k++) {
        const double *fs = &M.fsky[8 * k];
        a0 = a0 + fs[0];
        a1 = a1 + fs[1];
        a2 = a2 + fs[2];
        r0 = r0 + fs[3];
        r1 = r1 + fs[4];
        r2 = r2 + fs[5];
        st = st + fs[6];
        sr = sr + fs[7];
      }
      M.A[3 * n] = a0;
      M.A[3 * n + 1] = a1;
      M.A[3 * n + 2] = a2;
      M.AR[3 * n] = r0;
      M.AR[3 * n + 1] = r1;
      M.AR[3 * n + 2] = r2;
      M.STIFN[n] = st;
      M.STIFR[n] = sr;
      M.FLAST[3 * n] = a0;
      M.FLAST[3 * n + 1] = a1;
      M.FLAST[3 * n + 2] = a2;
      M.FRLAST[3 * n] = r0;
      M.FRLAST[3 * n + 1] = r1;
      M.FRLAST[3 * n + 2] = r2;
    }
    // RBYFOR (resol.F:5714), before the nodal time step
    for (auto &B : M.bodies) rbyfor(M, B);
    // RMATFORP (resol.F:5774): rigid-material bodies gather their nodes'
    // forces
    for (auto &B : M.rmats) rmatpon(M, B, rot);
    // DTNODA (time_step/dtnoda.F:213-345, 443-470), NODADT > 0: nodal time
    // step DTFAC1(11)*SQRT(2*MS/STIFN) over the nodes with mass, then the
    // rotational one DTFAC1(11)*SQRT(2*IN/STIFR); a node with non-positive
    // stiffness stops the run (flagged here).  Strict '<' scans: on ties the
    // first node of the translational pass, then of the rotational pass.
    // IDTMIN(11) = 3 / 8 (dtnoda.F:268-305, 466-500): a node below
    // DTMIN1(11) takes the mass (inertia) of a step DTMIN1(11),
    // 1/2 STIFN (DTMIN1/DTFAC1)^2 * ONEP00001 (inertia: the larger of that
    // and IN); the node's step of this cycle is the one computed before.
    if (M.nodadt) {
      const bool scale = M.idtmin_noda == 3 || M.idtmin_noda == 8;
      for (int n = 0; n < numnod; n++) {
        if (M.STIFN[n] <= RG_ZERO) {
          M.error |= 32;
        } else if (M.MS[n] > RG_ZERO) {
          const double d = M.dtfac_noda * std::sqrt(RG_TWO * M.MS[n] / M.STIFN[n]);
          if (d < M.dtmin_noda) {
            if (scale) {
              const double dt2p = M.dtmin_noda / M.dtfac_noda;
              M.MS[n] = RG_HALF * M.STIFN[n] * dt2p * dt2p * RG_ONEP00001;
            } else {
              M.error |= 8;
            }
          }
          if (d < dt2t) {
            dt2t = d;
            neltst = n + 1;
          }
        }
      }
      if (rot) {
        for (int n = 0; n < numnod; n++) {
          if (M.STIFR[n] <= RG_ZERO) {
            M.error |= 32;
          } else if (M.IN[n] > RG_ZERO) {
            const double d = M.dtfac_noda * std::sqrt(RG_TWO * M.IN[n] / M.STIFR[n]);
            if (d < M.dtmin_noda) {
              if (scale) {
                const double dt2p = M.dtmin_noda / M.dtfac_noda;
                const double iner = RG_HALF * M.STIFR[n] * dt2p * dt2p * RG_ONEP00001;
                M.IN[n] = std::max(iner, M.IN[n]);
              } else {
                M.error |= 8;
              }
            }
            if (d < dt2t) {
              dt2t = d;
              neltst = n + 1;
            }
          }
        }
      }
    }
    // resol.F:6123-6127, 6352, 6494-6497
    if (dt2t < M.dt2) {
      M.dt2 = dt2t;
      M.neltst = neltst;
    }
    M.dt2 = std::min(std::min(M.dt2, RG_SP_1P1 * M.dt2old), M.dtmx);
    M.dt2old = M.dt2;
    M.dt12 = RG_HALF * (M.dt1 + M.dt2);
    M.wfext = M.wfext + wfexc * M.dt2;
    // ACCELE (accele.F:66-78)
#pragma omp parallel for schedule(static) num_threads(M.nthreads)
    for (int n = 0; n < numnod; n++) {
      if (M.MS[n] > RG_ZERO) {
        const double rtmp = RG_ONE / M.MS[n];
        M.A[3 * n] = M.A[3 * n] * rtmp;
        M.A[3 * n + 1] = M.A[3 * n + 1] * rtmp;
        M.A[3 * n + 2] = M.A[3 * n + 2] * rtmp;
      } else {
        M.A[3 * n] = M.A[3 * n + 1] = M.A[3 * n + 2] = RG_ZERO;
      }
      if (rot) {
        if (M.IN[n] > RG_ZERO) {
          const double rtmp = RG_ONE / M.IN[n];
          M.AR[3 * n] = M.AR[3 * n] * rtmp;
          M.AR[3 * n + 1] = M.AR[3 * n + 1] * rtmp;
          M.AR[3 * n + 2] = M.AR[3 * n + 2] * rtmp;
        } else {
          M.AR[3 * n] = M.AR[3 * n + 1] = M.AR[3 * n + 2] = RG_ZERO;
        }
      }
      // BCS10 / BCS1V (bcs10.F:31): fixed translational DOFs; code bits
      // 1 = x, 2 = y, 4 = z; rotational bits 8, 16, 32.
      const int ic = M.icodt[n];
      if (ic) {
        if (ic & 1) M.A[3 * n] = RG_ZERO;
        if (ic & 2) M.A[3 * n + 1] = RG_ZERO;
        if (ic & 4) M.A[3 * n + 2] = RG_ZERO;
        if (ic & 8) M.AR[3 * n] = RG_ZERO;
        if (ic & 16) M.AR[3 * n + 1] = RG_ZERO;
        if (ic & 32) M.AR[3 * n + 2] = RG_ZERO;
      }
    }
    // RGWALL (constraints/general/rwall/rgwall.F:33), fixed infinite plane,
    // sliding: a slave node whose predicted position X + (V + A*DT12)*DT2 is
    // on or behind the plane and which does not move away from it loses the
    // normal components of its acceleration and velocity.
    // external work of the walls (rgwall.F:289-300, 515): TFXTN summed over
    // the corrected nodes, WFEXT += HALF*DT1*TFXTN
    double tfxtn = RG_ZERO;
    const double fact = M.dt12 != RG_ZERO ? RG_ONE / M.dt12 : RG_ZERO;
    for (auto &W : w->walls) {
      for (int n : W.slaves) {
        const int n1 = 3 * n, n2 = n1 + 1, n3 = n1 + 2;
        const double vx = M.V[n1] + M.A[n1] * M.dt12;
        const double vy = M.V[n2] + M.A[n2] * M.dt12;
        const double vz = M.V[n3] + M.A[n3] * M.dt12;
        const double ux = M.X[n1] + vx * M.dt2;
        const double uy = M.X[n2] + vy * M.dt2;
        const double uz = M.X[n3] + vz * M.dt2;
        const double xc = ux - W.p0[0], yc = uy - W.p0[1], zc = uz - W.p0[2];
        const double dp = xc * W.n[0] + yc * W.n[1] + zc * W.n[2];
        if (dp > RG_ZERO) continue;
        if ((vx - RG_ZERO) * W.n[0] + (vy - RG_ZERO) * W.n[1] + (vz - RG_ZERO) * W.n[2] > RG_ZERO)
          continue;
        const double dv = (M.V[n1] - RG_ZERO) * W.n[0] + (M.V[n2] - RG_ZERO) * W.n[1] +
                          (M.V[n3] - RG_ZERO) * W.n[2];
        const double da = M.A[n1] * W.n[0] + M.A[n2] * W.n[1] + M.A[n3] * W.n[2];
        {
          const double dvt = (dv + da * M.dt12) * M.MS[n];
          const double fnx = dvt * W.n[0], fny = dvt * W.n[1], fnz = dvt * W.n[2];
          tfxtn = tfxtn - fact * ((M.V[n1] - RG_ZERO) * fnx + (M.V[n2] - RG_ZERO) * fny +
                                  (M.V[n3] - RG_ZERO) * fnz);
        }
        M.A[n1] = M.A[n1] - da * W.n[0];
        M.A[n2] = M.A[n2] - da * W.n[1];
        M.A[n3] = M.A[n3] - da * W.n[2];
        M.V[n1] = M.V[n1] - dv * W.n[0];
        M.V[n2] = M.V[n2] - dv * W.n[1];
        M.V[n3] = M.V[n3] - dv * W.n[2];
      }
    }
    if (!w->walls.empty()) M.wfext = M.wfext + RG_HALF * M.dt1 * tfxtn;
    // RLINK1 (constraints/general/rlink/rlink1.F): every node of a link
    // takes the mass-weighted mean acceleration of the link in the linked
    // directions (IC bits 4 = x, 2 = y, 1 = z), after the boundary
    // conditions (resol.F:7322 BCS10, then :7355 RLINK10).
    for (auto &L : M.links) {
      if (L.ic != 0) {
        double mass = 0, ax = 0, ay = 0, az = 0;
        for (int n : L.nodes) {
          mass = mass + M.MS[n];
          ax = ax + M.MS[n] * M.A[3 * n];
          ay = ay + M.MS[n] * M.A[3 * n + 1];
          az = az + M.MS[n] * M.A[3 * n + 2];
        }
        if (mass != RG_ZERO) {
          ax = ax / mass;
          ay = ay / mass;
          az = az / mass;
          for (int n : L.nodes) {
            if (L.ic & 1) M.A[3 * n + 2] = az;
            if (L.ic & 2) M.A[3 * n + 1] = ay;
            if (L.ic & 4) M.A[3 * n] = ax;
          }
        }
      }
      if (L.icr != 0 && rot) {
        double iner = 0, ax = 0, ay = 0, az = 0;
        for (int n : L.nodes) {
          iner = iner + M.IN[n];
          ax = ax + M.IN[n] * M.AR[3 * n];
          ay = ay + M.IN[n] * M.AR[3 * n + 1];
          az = az + M.IN[n] * M.AR[3 * n + 2];
        }
        if (iner != RG_ZERO) {
          ax = ax / iner;
          ay = ay / iner;
          az = az / iner;
          for (int n : L.nodes) {
            if (L.icr & 1) M.AR[3 * n + 2] = az;
            if (L.icr & 2) M.AR[3 * n + 1] = ay;
            if (L.icr & 4) M.AR[3 * n] = ax;
          }
        }
      }
    }
    // FIXVEL (resol.F:7610): imposed velocities, after the boundary
    // conditions
    fixvel(M);
    // RBYVIT (resol.F:7849), after the boundary conditions
    for (auto &B : M.bodies)
      if (rgbodv(M, B)) M.error |= 64;
    // RMATACCE (resol.F:7879): rigid-material bodies drive their nodes
    for (auto &B : M.rmats) rmatacce(M, B, rot);
    // ECRIT (output/ecrit.F:193, 266-330): energies of the printout with the
    // velocities brought to the current time, V + DT1/2 * A.  RBYCOR /
    // RGBCOR (rbycor.F, rgbcor.F:213-380) take the secondary nodes of rigid
    // bodies out of the sums and count a body's rotation with its principal
    // inertia: 1/2 sum_k I_k (R W)_k^2, W = VR(M) + DT1/2 AR(M).
    if (M.record) {
      const double dt05 = RG_HALF * M.dt1;
      double ek = 0, ekr = 0, xm = 0, ym = 0, zm = 0, mass = 0;
      for (const auto &B : M.bodies) {
        const int n = B.main;
        const double *R = B.R;
        const double wx = M.VR[3 * n] + dt05 * M.AR[3 * n];
        const double wy = M.VR[3 * n + 1] + dt05 * M.AR[3 * n + 1];
        const double wz = M.VR[3 * n + 2] + dt05 * M.AR[3 * n + 2];
        for (int k = 0; k < 3; k++) {
          const double vi = R[3 * k] * wx + R[3 * k + 1] * wy + R[3 * k + 2] * wz;
          ekr = ekr + RG_HALF * B.I[k] * vi * vi;
        }
      }
      for (int n = 0; n < numnod; n++) {
        // role: 0 free node, 1 rigid-body secondary, 2 rigid-body main
        const int role = M.secondary.empty() ? 0 : M.secondary[n];
        if (role == 1) continue;
        const double vx = M.V[3 * n] + dt05 * M.A[3 * n];
        const double vy = M.V[3 * n + 1] + dt05 * M.A[3 * n + 1];
        const double vz = M.V[3 * n + 2] + dt05 * M.A[3 * n + 2];
        ek = ek + (vx * vx + vy * vy + vz * vz) * RG_HALF * M.MS[n];
        xm = xm + vx * M.MS[n];
        ym = ym + vy * M.MS[n];
        zm = zm + vz * M.MS[n];
        mass = mass + M.MS[n];
        if (rot && role == 0) {
          const double rx = M.VR[3 * n] + dt05 * M.AR[3 * n];
          const double ry = M.VR[3 * n + 1] + dt05 * M.AR[3 * n + 1];
          const double rz = M.VR[3 * n + 2] + dt05 * M.AR[3 * n + 2];
          ekr = ekr + (rx * rx + ry * ry + rz * rz) * RG_HALF * M.IN[n];
        }
      }
      double ei = 0, eh = 0;
      for (int e = 0; e < M.numels; e++) {
        ei += M.eint[e] * M.vol[e];
        eh += M.ehou[e];
      }
      double sei = 0, seh = 0;
      rg_oracle_shell::energy(w->sh, sei, seh);
      M.out[0] = M.tt;
      M.out[1] = M.dt2;
      M.out[2] = ei + sei;
      M.out[3] = ek;
      M.out[4] = ekr;
      M.out[5] = eh + seh;
      M.out[6] = xm;
      M.out[7] = ym;
      M.out[8] = zm;
      M.out[9] = mass;
      M.out[10] = M.wfext;
    }
    // VELOCITY (velocity.F:59-75), DEPLA (displacement.F:68-100)
#pragma omp parallel for schedule(static) num_threads(M.nthreads)
    for (int n = 0; n < numnod; n++) {
      for (int c = 0; c < 3; c++) {
        M.V[3 * n + c] = M.V[3 * n + c] + M.dt12 * M.A[3 * n + c];
        M.A[3 * n + c] = RG_ZERO;
      }
      if (rot)
        for (int c = 0; c < 3; c++) {
          M.VR[3 * n + c] = M.VR[3 * n + c] + M.dt12 * M.AR[3 * n + c];
          M.AR[3 * n + c] = RG_ZERO;
        }
      for (int c = 0; c < 3; c++) {
        const double vdt = M.dt2 * M.V[3 * n + c];
        M.D[3 * n + c] = M.D[3 * n + c] + vdt;
        M.X[3 * n + c] = M.X[3 * n + c] + vdt;
      }
    }
    // resol.F:8603-8611 (double accumulation), NCYCLE + 1
    M.tt = M.tt + M.dt2;
    M.ncycle++;
    M.ext = false;
  }
  return M.error;
}

int or_get_nodes(void *m, double *x, double *v, double *d, double *vr,
                 double *f, double *stifn, double *fr) {
  Model &M = ((OrModelWrap *)m)->m;
  const size_t n3 = 3 * (size_t)M.numnod;
  if (x) std::copy(M.X.begin(), M.X.begin() + n3, x);
  if (v) std::copy(M.V.begin(), M.V.begin() + n3, v);
  if (d) std::copy(M.D.begin(), M.D.begin() + n3, d);
  if (vr) std::copy(M.VR.begin(), M.VR.begin() + n3, vr);
  if (f) std::copy(M.FLAST.begin(), M.FLAST.begin() + n3, f);
  if (fr) std::copy(M.FRLAST.begin(), M.FRLAST.begin() + n3, fr);
  if (stifn) std::copy(M.STIFN.begin(), M.STIFN.end(), stifn);
  return 0;
}

int or_get_time(void *m, double *tt, double *dt1, double *dt2, int *ncycle,
                int *neltst) {
  Model &M = ((OrModelWrap *)m)->m;
  if (tt) *tt = M.tt;
  if (dt1) *dt1 = M.dt1;
  if (dt2) *dt2 = M.dt2;
  if (ncycle) *ncycle = M.ncycle;
  if (neltst) *neltst = M.neltst;
  return 0;
}

int or_get_hexa_state(void *m, int group, int which, double *out) {
  Model &M = ((OrModelWrap *)m)->m;
  (void)group;
  const int ne = M.numels;
  switch (which) {
    case 0:
      std::copy(M.sig.begin(), M.sig.end(), out);
      return 0;
    case 1: std::copy(M.eint.begin(), M.eint.end(), out); return 0;
    case 2: std::copy(M.rho.begin(), M.rho.end(), out); return 0;
    case 3: std::copy(M.qvis.begin(), M.qvis.end(), out); return 0;
    case 4: std::copy(M.offg.begin(), M.offg.end(), out); return 0;
    case 5: std::copy(M.pla.begin(), M.pla.end(), out); return 0;
    case 6: std::copy(M.epsd.begin(), M.epsd.end(), out); return 0;
    case 7: std::copy(M.vol.begin(), M.vol.end(), out); return 0;
    case 8: std::copy(M.ehou.begin(), M.ehou.end(), out); return 0;
  }
  (void)ne;
  return -1;
}

int or_energy(void *m, double *eint, double *ekin, double *ekinr,
              double *ehour) {
  auto *w = (OrModelWrap *)m;
  Model &M = w->m;
  double ei = 0, ek = 0, ekr = 0, eh = 0;
  for (int e = 0; e < M.numels; e++) {
    ei += M.eint[e] * M.vol[e];
    eh += M.ehou[e];
  }
  double sei = 0, seh = 0;
  rg_oracle_shell::energy(w->sh, sei, seh);
  ei += sei;
  eh += seh;
  for (int n = 0; n < M.numnod; n++) {
    const double v2 = M.V[3 * n] * M.V[3 * n] + M.V[3 * n + 1] * M.V[3 * n + 1] +
                      M.V[3 * n + 2] * M.V[3 * n + 2];
    ek += RG_HALF * M.MS[n] * v2;
    const double w2 = M.VR[3 * n] * M.VR[3 * n] + M.VR[3 * n + 1] * M.VR[3 * n + 1] +
                      M.VR[3 * n + 2] * M.VR[3 * n + 2];
    ekr += RG_HALF * M.IN[n] * w2;
  }
  if (eint) *eint = ei;
  if (ekin) *ekin = ek;
  if (ekinr) *ekinr = ekr;
  if (ehour) *ehour = eh;
  return 0;
}

int or_error(void *m) { return ((OrModelWrap *)m)->m.error; }

int or_set_dtmin(void *m, int kind, int idtmin, double dtmin) {
  auto *w = (OrModelWrap *)m;
  if (kind == 3) {
    rg_oracle_shell::set_dtmin(w->sh, idtmin, dtmin);
    return 0;
  }
  if (kind == 11) {
    w->m.idtmin_noda = idtmin;
    w->m.dtmin_noda = dtmin;
    return 0;
  }
  return -1;
}

int or_set_nodal_dt(void *m, double dtfac, double dtmin) {
  auto *w = (OrModelWrap *)m;
  if (w->m.finalized || !(dtfac > 0.0)) return -1;
  w->m.nodadt = 1;
  w->m.dtfac_noda = dtfac;
  w->m.dtmin_noda = dtmin;
  rg_oracle_shell::set_nodadt(w->sh, 1);
  return 0;
}

int or_shell_frame(void *m, int ishfram) {
  return rg_oracle_shell::set_frame(((OrModelWrap *)m)->sh, ishfram);
}

int or_rlink_add(void *m, int nsn, const int *nodes, int ic, int icr) {
  Model &M = ((OrModelWrap *)m)->m;
  if (nsn <= 0 || !nodes || ic < 0 || ic > 7 || icr < 0 || icr > 7) return -1;
  Model::Link L;
  for (int i = 0; i < nsn; i++) {
    if (nodes[i] < 1 || nodes[i] > M.numnod) return -2;
    L.nodes.push_back(nodes[i] - 1);
  }
  L.ic = ic;
  L.icr = icr;
  M.links.push_back(L);
  return (int)M.links.size() - 1;
}

int or_rbody_add(void *m, int main, int nsn, const int *nodes, const double *axes,
                 const double *inertia) {
  Model &M = ((OrModelWrap *)m)->m;
  if (M.finalized || nsn <= 2 || !nodes || !axes || !inertia || main < 1 || main > M.numnod)
    return -1;
  if (M.secondary.empty()) M.secondary.assign(M.numnod, 0);
  Model::Body B;
  B.main = main - 1;
  if (M.secondary[B.main]) return -2;
  for (int i = 0; i < nsn; i++) {
    const int n = nodes[i] - 1;
    if (n < 0 || n >= M.numnod || n == B.main || M.secondary[n]) return -2;
    B.nodes.push_back(n);
  }
  for (int k = 0; k < 9; k++) B.R[k] = axes[k];
  for (int k = 0; k < 3; k++) {
    if (!(inertia[k] > RG_ZERO)) return -1;
    B.I[k] = inertia[k];
  }
  if (!(M.IN[B.main] > RG_ZERO) || !(M.MS[B.main] > RG_ZERO)) return -3;
  for (int n : B.nodes) M.secondary[n] = 1;
  M.secondary[B.main] = 2;
  M.bodies.push_back(B);
  return (int)M.bodies.size() - 1;
}

int or_rmat_add(void *m, int nsl, const int *nodes, const double *xg, double mass,
                const double *axes, const double *inertia) {
  Model &M = ((OrModelWrap *)m)->m;
  if (M.finalized || nsl < 1 || !nodes || !xg || !axes || !inertia || !(mass > RG_ZERO))
    return -1;
  Model::RigidMat B;
  for (int i = 0; i < nsl; i++) {
    const int n = nodes[i] - 1;
    if (n < 0 || n >= M.numnod) return -1;
    B.nodes.push_back(n);
  }
  B.mass = mass;
  for (int k = 0; k < 3; k++) {
    B.xg[k] = xg[k];
    B.I[k] = inertia[k];
  }
  for (int k = 0; k < 9; k++) B.R[k] = axes[k];
  B.in = std::min(B.I[0], std::min(B.I[1], B.I[2]));
  {
    // RBYM(18:26) of rigid_mat.F
    const double *RB = B.R, *I = B.I;
    const double ii1 = I[0] * RB[0], ii2 = I[0] * RB[1], ii3 = I[0] * RB[2];
    const double ii4 = I[1] * RB[3], ii5 = I[1] * RB[4], ii6 = I[1] * RB[5];
    const double ii7 = I[2] * RB[6], ii8 = I[2] * RB[7], ii9 = I[2] * RB[8];
    B.J[0] = RB[0] * ii1 + RB[3] * ii4 + RB[6] * ii7;
    B.J[1] = RB[0] * ii2 + RB[3] * ii5 + RB[6] * ii8;
    B.J[2] = RB[0] * ii3 + RB[3] * ii6 + RB[6] * ii9;
    B.J[3] = RB[1] * ii1 + RB[4] * ii4 + RB[7] * ii7;
    B.J[4] = RB[1] * ii2 + RB[4] * ii5 + RB[7] * ii8;
    B.J[5] = RB[1] * ii3 + RB[4] * ii6 + RB[7] * ii9;
    B.J[6] = RB[2] * ii1 + RB[5] * ii4 + RB[8] * ii7;
    B.J[7] = RB[2] * ii2 + RB[5] * ii5 + RB[8] * ii8;
    B.J[8] = RB[2] * ii3 + RB[5] * ii6 + RB[8] * ii9;
  }
  // CONDRMAT (materials/mat/mat013/condrmat.F): the secondary nodes'
  // boundary codes move to the body (Radioss codes: 4 x, 2 y, 1 z)
  int it = 0, ir = 0;
  for (int n : B.nodes) {
    const int c = M.icodt[n];
    if (c & 1) it |= 4;
    if (c & 2) it |= 2;
    if (c & 4) it |= 1;
    if (c & 8) ir |= 4;
    if (c & 16) ir |= 2;
    if (c & 32) ir |= 1;
    M.icodt[n] = 0;
  }
  B.icod[0] = ir;
  B.icod[1] = it;
  M.rmats.push_back(B);
  return (int)M.rmats.size() - 1;
}

int or_impvel_add(void *m, int node, int dir, double facx, double fscale, double tstart,
                  double tstop, int npts, const double *x, const double *y) {
  Model &M = ((OrModelWrap *)m)->m;
  if (node < 1 || node > M.numnod || dir < 0 || dir > 2 || npts < 1 || !x || !y) return -1;
  for (int i = 1; i < npts; i++)
    if (!(x[i] > x[i - 1])) return -1;
  Model::ImpVel F;
  F.node = node - 1;
  F.dir = dir;
  F.facx = facx;
  F.fscale = fscale;
  F.tstart = tstart;
  F.tstop = tstop;
  F.x.assign(x, x + npts);
  F.y.assign(y, y + npts);
  M.impvels.push_back(F);
  return (int)M.impvels.size() - 1;
}

int or_cload_add(void *m, int node, int dir, double fcx, double fcy, int npts,
                 const double *x, const double *y) {
  Model &M = ((OrModelWrap *)m)->m;
  if (node < 1 || node > M.numnod || dir < 0 || dir > 5 || npts < 1 || !x || !y) return -1;
  for (int i = 1; i < npts; i++)
    if (!(x[i] > x[i - 1])) return -1;
  Model::Load L;
  L.node = node - 1;
  L.dir = dir;
  L.fcx = fcx;
  L.fcy = fcy;
  L.x.assign(x, x + npts);
  L.y.assign(y, y + npts);
  M.loads.push_back(L);
  return (int)M.loads.size() - 1;
}

int or_set_forces(void *m, const double *f, const double *stifn, const double *fr,
                  const double *stifr, double dt2t, int neltst) {
  Model &M = ((OrModelWrap *)m)->m;
  if (!M.finalized || !f || !stifn) return -1;
  const size_t n3 = 3 * (size_t)M.numnod;
  M.ext_f.assign(f, f + n3);
  M.ext_stifn.assign(stifn, stifn + M.numnod);
  if (fr) M.ext_fr.assign(fr, fr + n3); else M.ext_fr.clear();
  if (stifr) M.ext_stifr.assign(stifr, stifr + M.numnod); else M.ext_stifr.clear();
  M.ext_dt2t = dt2t;
  M.ext_neltst = neltst;
  M.ext = true;
  return 0;
}

int or_rlink_clear(void *m) {
  ((OrModelWrap *)m)->m.links.clear();
  return 0;
}

int or_set_record(void *m, int on) {
  ((OrModelWrap *)m)->m.record = on != 0;
  return 0;
}

// External work accumulated so far (loads and rigid walls).
int or_get_mass(void *m, double *ms, double *in) {
  const auto &M = ((OrModelWrap *)m)->m;
  for (size_t n = 0; n < M.MS.size(); n++) {
    ms[n] = M.MS[n];
    if (in) in[n] = n < M.IN.size() ? M.IN[n] : 0.0;
  }
  return 0;
}

int or_get_wfext(void *m, double *out) {
  *out = ((OrModelWrap *)m)->m.wfext;
  return 0;
}

int or_get_record(void *m, double *out, int *neltst) {
  Model &M = ((OrModelWrap *)m)->m;
  if (out) std::copy(M.out, M.out + 11, out);
  if (neltst) *neltst = M.neltst;
  return 0;
}

// Element -> part maps of the per-part sums (0-based parts < npart; null
// maps: one part per element group, hexa groups first).
int or_set_parts(void *m, int npart, const int *hexa_part, const int *shell_part) {
  auto *w = (OrModelWrap *)m;
  Model &M = w->m;
  const int nc = rg_oracle_shell::numelc(w->sh);
  if (npart <= 0) return -1;
  for (int e = 0; e < M.numels; e++)
    if (!hexa_part || hexa_part[e] < 0 || hexa_part[e] >= npart) return -1;
  for (int e = 0; e < nc; e++)
    if (!shell_part || shell_part[e] < 0 || shell_part[e] >= npart) return -1;
  M.npart = npart;
  M.part_hexa.assign(hexa_part, hexa_part + M.numels);
  M.part_shell.assign(shell_part, shell_part + nc);
  M.psum.clear();
  return 0;
}

// Per-part sums of the last recorded cycle: out[p * 7 + q] (IE, KE, XMOM,
// YMOM, ZMOM, MASS, HE); returns the part count (0 before any such cycle).
int or_get_part_sums(void *m, double *out, int npart) {
  const Model &M = ((OrModelWrap *)m)->m;
  const int n = (int)(M.psum.size() / 7);
  if (out) std::copy(M.psum.begin(), M.psum.begin() + 7 * (size_t)std::min(n, npart), out);
  return n;
}

int or_get_shell_state(void *m, int which, double *out) {
  return rg_oracle_shell::get_state(((OrModelWrap *)m)->sh, which, out);
}

}  // extern "C"
