// CPU oracle, Belytschko-Tsay 4-node shell with LAW2 -- TEST INFRASTRUCTURE.
//
// Restates, per element and in the reference's expression order, the CFORC3
// chain for the pinned formulation: Ishell=1 (IHBE=1, viscous/elastic
// hourglass CHVIS3), Ismstr=2/4 (no small-strain reference storage), Ithick=1
// (current thickness) or 0 (initial thickness), NPT through-thickness points
// with the COQINI tables, ISHFRAM=0 (symmetric CNVEC3 frame) or 2 (the
// version-4 non-symmetric frame of /SHFRA/V4), Johnson-Cook plane stress (SIGEPS02C + M2CPLR)
// with Iplas=1 (3 Newton iterations) or Iplas=0 (radial return), element
// time step (NODADT=0, IDTMIN(3)=2), PARITH/ON slot writes (CUPDT3P).
// Conventions: see rg_oracle.cpp.  Paths are relative to the OpenRadioss
// source tree.
#include <algorithm>
#include <atomic>
#include <cmath>
#include <vector>

#include "../openradioss_gb300/csrc/rg_constants.h"

// Phase marks of the op-counting build (rg_opcount.h); nothing elsewhere.
#ifndef RG_OPCOUNT_PHASE
#ifdef RG_OPCOUNT
#define RG_OPCOUNT_PHASE(p) (rg_count::phase = (p))
#else
#define RG_OPCOUNT_PHASE(p) ((void)0)
#endif
#endif
#ifdef _OPENMP
#include <omp.h>
#endif

namespace rg_oracle_shell {

// COQINI tables (engine/source/elements/shell/coqini.F:46-123): default-real
// (single precision) DATA literals assigned to double arrays; columns
// NPT = 1..5, rows the integration point.
static const float Z0T[5][5] = {{0.f, 0.f, 0.f, 0.f, 0.f},
                                {-.5f, 0.5f, 0.f, 0.f, 0.f},
                                {-.5f, 0.f, 0.5f, 0.f, 0.f},
                                {-.5f, -.1666667f, 0.1666667f, 0.5f, 0.f},
                                {-.5f, -.25f, 0.f, 0.25f, 0.5f}};
static const float WFT[5][5] = {{1.f, 0.f, 0.f, 0.f, 0.f},
                                {0.5f, 0.5f, 0.f, 0.f, 0.f},
                                {0.25f, 0.5f, 0.25f, 0.f, 0.f},
                                {0.1666667f, 0.3333333f, 0.3333333f, 0.1666667f, 0.f},
                                {0.125f, 0.25f, 0.25f, 0.25f, 0.125f}};
static const float WMT[5][5] = {{0.f, 0.f, 0.f, 0.f, 0.f},
                                {-.0833333f, 0.0833333f, 0.f, 0.f, 0.f},
                                {-.0833333f, 0.f, 0.0833333f, 0.f, 0.f},
                                {-.0648148f, -.0555556f, 0.0555556f, 0.0648148f, 0.f},
                                {-.0520833f, -.0625f, 0.f, 0.0625f, 0.0520833f}};

struct Group {
  int nft = 0, nel = 0, npt = 5, ipla = 1, ithk = 1, ismstr = 4, ihbe = 1;
  double rho = 0, young = 0, nu = 0, g = 0, a11 = 0, a12 = 0, ssp = 0;
  double h1 = 0, h2 = 0, h3 = 0, srh1 = 0, srh2 = 0, srh3 = 0, dm = 0;
  double ish = 0, fsh = 0;
  // LAW2
  double ca = 0, cb = 0, cn = 1, epmx = 0, ymax = 0, cc = 0, eps0 = 1, fisokin = 0;
  double pm9 = 0;
  int icc = 1, vp = 2, israte = 0;
  // Johnson-Cook thermal softening (mat_param%therm, uparam(10)): adiabatic
  // heating when RHOCP > 0, each point starting at TREF (allocbuf_auto.F:189)
  double m_exp = 1, tref = 300, tmelt = 1e20, rhocp = 0;
  int thermal = 0;
};

struct Shells {
  int numelc = 0;
  std::vector<int> ixc;  // 7 * numelc
  std::vector<int> iadc;
  std::vector<Group> groups;
  // state (element SoA)
  std::vector<double> offg, thk, thke, forc, mom, eint, hour, gstr, epsdg;
  std::vector<double> sig, pla, epsd;  // per IP: [npt][numelc] (max npt 5)
  std::vector<double> sigbak;          // back stress per IP: [npt][3][numelc]
  std::vector<double> temp;            // temperature per IP: [npt][numelc]
  bool temp_init = false;
  std::vector<double> ehou;            // accumulated hourglass energy
  int nptmax = 5;
  int ishfram = 0;                     // local frame (/SHFRA/V4: 2)
  int nodadt = 0;                      // nodal time step (/DT/NODA)
  int idtmin = 0;                      // IDTMIN(3): 1, 5 stop; 2 delete
  double dtmin = 0.0;                  // DTMIN1(3)
  std::atomic<int> stop{0};            // IDTMIN(3) = 1 / 5 reached
};

Shells *create() { return new Shells(); }
void set_nodadt(Shells *s, int on) { s->nodadt = on; }
void set_dtmin(Shells *s, int idtmin, double dtmin) {
  s->idtmin = idtmin;
  s->dtmin = dtmin;
}
int set_frame(Shells *s, int ishfram) {
  if (ishfram != 0 && ishfram != 2) return -1;
  s->ishfram = ishfram;
  return 0;
}
void destroy(Shells *s) { delete s; }
int numelc(const Shells *s) { return s->numelc; }
const int *ixc(const Shells *s) { return s->ixc.data(); }
int *iadc(Shells *s) {
  if ((int)s->iadc.size() < 4 * s->numelc) s->iadc.assign(4 * (size_t)s->numelc, 0);
  return s->iadc.data();
}

int group_add(Shells *S, int nel, const int *ixc, int npt, const double *pm,
              const double *geo, const double *uparam, const int *iparam,
              const double *thk0, int ismstr, int ithk) {
  if (nel <= 0 || npt < 1 || npt > 5) return -1;
  if (ismstr != 4 && ismstr != 2) return -3;
  Group G;
  G.nft = S->numelc;
  G.nel = nel;
  G.npt = npt;
  G.ithk = ithk;
  G.ismstr = 4;
  G.rho = pm[0];
  G.young = pm[19];
  G.nu = pm[20];
  G.g = pm[21];
  G.a11 = pm[23];
  G.a12 = pm[24];
  G.ssp = pm[26];
  G.h1 = geo[12];
  G.h2 = geo[13];
  G.h3 = geo[14];
  G.dm = geo[15];
  G.srh1 = geo[17];
  G.srh2 = geo[18];
  G.srh3 = geo[19];
  G.ish = geo[36];
  G.fsh = geo[37];
  G.ipla = (int)geo[38];
  if (iparam[0] != 0) return -4;  // Zerilli-Armstrong (IFORM = 1) not restated
  if (uparam[7] < 0.0 || uparam[7] > 1.0) return -4;
  // ductile rupture (SIGEPS02C EPMX test and MULAWC's layer failure) is not
  // restated: a finite EPMX is refused (the reader's default 1e20 is never
  // reached)
  if (uparam[3] < 1e20) return -4;
  G.icc = iparam[1];
  G.vp = iparam[2];
  G.israte = iparam[3];
  G.ca = uparam[0];
  G.cb = uparam[1];
  G.cn = uparam[2];
  G.epmx = uparam[3];
  G.ymax = uparam[4];
  G.cc = uparam[5];
  G.eps0 = uparam[6];
  G.pm9 = uparam[8];
  G.fisokin = uparam[7];
  G.m_exp = uparam[9] != 0.0 ? uparam[9] : 1.0;
  G.rhocp = pm[68];
  G.tref = pm[78];
  G.tmelt = pm[79];
  G.thermal = (G.rhocp > 0.0 && G.tmelt > G.tref) ? 1 : 0;
  S->groups.push_back(G);
  S->ixc.insert(S->ixc.end(), ixc, ixc + 7 * (size_t)nel);
  S->numelc += nel;
  const int n = S->numelc;
  S->offg.resize(n, 1.0);
  S->thke.insert(S->thke.end(), thk0, thk0 + nel);
  S->thk.insert(S->thk.end(), thk0, thk0 + nel);
  S->forc.resize(5 * (size_t)n, 0.0);
  S->mom.resize(3 * (size_t)n, 0.0);
  S->eint.resize(2 * (size_t)n, 0.0);
  S->hour.resize(5 * (size_t)n, 0.0);
  S->gstr.resize(8 * (size_t)n, 0.0);
  S->epsdg.resize(n, 0.0);
  S->sig.resize(5 * 5 * (size_t)n, 0.0);
  S->pla.resize(5 * (size_t)n, 0.0);
  S->epsd.resize(5 * (size_t)n, 0.0);
  S->ehou.resize(n, 0.0);
  S->sigbak.resize(5 * 3 * (size_t)n, 0.0);
  S->temp.resize(5 * (size_t)n, G.tref);
  return (int)S->groups.size() - 1;
}

// Element-major state accessors (component c of element e).
#define FOR_(c, e) S->forc[(size_t)(c) * S->numelc + (e)]
#define MOM_(c, e) S->mom[(size_t)(c) * S->numelc + (e)]
#define EIN_(c, e) S->eint[(size_t)(c) * S->numelc + (e)]
#define HOU_(c, e) S->hour[(size_t)(c) * S->numelc + (e)]
#define GST_(c, e) S->gstr[(size_t)(c) * S->numelc + (e)]
#define SIG_(c, p, e) S->sig[((size_t)(p) * 5 + (c)) * S->numelc + (e)]
#define PLA_(p, e) S->pla[(size_t)(p) * S->numelc + (e)]
#define EPS_(p, e) S->epsd[(size_t)(p) * S->numelc + (e)]
#define SGB_(c, p, e) S->sigbak[((size_t)(p) * 3 + (c)) * S->numelc + (e)]
#define TMP_(p, e) S->temp[(size_t)(p) * S->numelc + (e)]

static inline double dmax(double a, double b) { return a > b ? a : b; }
static inline double dmin(double a, double b) { return a < b ? a : b; }

static void element(Shells *S, const Group &G, int e, const double *X,
                    const double *V, const double *VR, double *fsky,
                    double DT1, double dtfac, double &dt2t, int &elmin) {
  const int *ix = &S->ixc[7 * (size_t)e];
  int nn[4];
  for (int k = 0; k < 4; k++) nn[k] = ix[1 + k] - 1;
  // ---- CCOOR3 (ccoor3.F:31) ----
  double xg[4], yg[4], zg[4], vl[4][3], vrl[4][3];
  for (int k = 0; k < 4; k++) {
    xg[k] = X[3 * nn[k]];
    yg[k] = X[3 * nn[k] + 1];
    zg[k] = X[3 * nn[k] + 2];
    for (int c = 0; c < 3; c++) {
      vl[k][c] = V[3 * nn[k] + c];
      vrl[k][c] = VR[3 * nn[k] + c];
    }
  }
  const double offg = S->offg[e];
  double off = dmin(RG_ONE, std::fabs(offg));
  if (offg < 0.0)
    for (int k = 0; k < 4; k++)
      for (int c = 0; c < 3; c++) vl[k][c] = vrl[k][c] = RG_ZERO;
  double thk0 = S->thke[e];
  // ---- CNVEC3 (cnvec3.F:35), ISHFRAM = 0 (cnvec3.F:117-141) or 2
  // (cnvec3.F:143-170) ----
  double e1x, e1y, e1z, e2x, e2y, e2z, e3x, e3y, e3z;
  {
    const double x21 = xg[1] - xg[0], x32 = xg[2] - xg[1], x34 = xg[2] - xg[3], x41 = xg[3] - xg[0];
    const double y21 = yg[1] - yg[0], y32 = yg[2] - yg[1], y34 = yg[2] - yg[3], y41 = yg[3] - yg[0];
    const double z21 = zg[1] - zg[0], z32 = zg[2] - zg[1], z34 = zg[2] - zg[3], z41 = zg[3] - zg[0];
    e1x = (x21 + x34);
    e1y = (y21 + y34);
    e1z = (z21 + z34);
    e2x = (x32 + x41);
    e2y = (y32 + y41);
    e2z = (z32 + z41);
    e3x = e1y * e2z - e1z * e2y;
    e3y = e1z * e2x - e1x * e2z;
    e3z = e1x * e2y - e1y * e2x;
    if (S->ishfram == 2) {
      // version-4 frame: e1 along the mean of the two x-sides, tilted by
      // e2 x e3, then normalised; e2 = e3 x e1
      double suma = e2x * e2x + e2y * e2y + e2z * e2z;
      e1x = e1x * suma + e2y * e3z - e2z * e3y;
      e1y = e1y * suma + e2z * e3x - e2x * e3z;
      e1z = e1z * suma + e2x * e3y - e2y * e3x;
      suma = e1x * e1x + e1y * e1y + e1z * e1z;
      suma = RG_ONE / dmax(std::sqrt(suma), RG_EM20);
      e1x = e1x * suma;
      e1y = e1y * suma;
      e1z = e1z * suma;
      suma = e3x * e3x + e3y * e3y + e3z * e3z;
      suma = RG_ONE / dmax(std::sqrt(suma), RG_EM20);
      e3x = e3x * suma;
      e3y = e3y * suma;
      e3z = e3z * suma;
      e2x = e3y * e1z - e3z * e1y;
      e2y = e3z * e1x - e3x * e1z;
      e2z = e3x * e1y - e3y * e1x;
      suma = e2x * e2x + e2y * e2y + e2z * e2z;
      suma = RG_ONE / dmax(std::sqrt(suma), RG_EM20);
      e2x = e2x * suma;
      e2y = e2y * suma;
      e2z = e2z * suma;
    } else {
    double suma = e3x * e3x + e3y * e3y + e3z * e3z;
    suma = RG_ONE / dmax(std::sqrt(suma), RG_EM20);
    e3x = e3x * suma;
    e3y = e3y * suma;
    e3z = e3z * suma;
    const double s1 = e1x * e1x + e1y * e1y + e1z * e1z;
    const double s2 = e2x * e2x + e2y * e2y + e2z * e2z;
    suma = std::sqrt(s1 / s2);
    e1x = e1x + (e2y * e3z - e2z * e3y) * suma;
    e1y = e1y + (e2z * e3x - e2x * e3z) * suma;
    e1z = e1z + (e2x * e3y - e2y * e3x) * suma;
    suma = e1x * e1x + e1y * e1y + e1z * e1z;
    suma = RG_ONE / dmax(std::sqrt(suma), RG_EM20);
    e1x = e1x * suma;
    e1y = e1y * suma;
    e1z = e1z * suma;
    e2x = e3y * e1z - e3z * e1y;
    e2y = e3z * e1x - e3x * e1z;
    e2z = e3x * e1y - e3y * e1x;
    }
  }
  // ---- CDERI3 (cderi3.F:30), ISMSTR = 4 ----
  double x2, y2, x3, y3, x4, y4, px1, px2, py1, py2, area, vhx, vhy;
  {
    const double x21 = xg[1] - xg[0], y21 = yg[1] - yg[0], z21 = zg[1] - zg[0];
    const double x31 = xg[2] - xg[0], y31 = yg[2] - yg[0], z31 = zg[2] - zg[0];
    const double x41 = xg[3] - xg[0], y41 = yg[3] - yg[0], z41 = zg[3] - zg[0];
    x2 = e1x * x21 + e1y * y21 + e1z * z21;
    y2 = e2x * x21 + e2y * y21 + e2z * z21;
    y3 = e2x * x31 + e2y * y31 + e2z * z31;
    x3 = e1x * x31 + e1y * y31 + e1z * z31;
    x4 = e1x * x41 + e1y * y41 + e1z * z41;
    y4 = e2x * x41 + e2y * y41 + e2z * z41;
    px1 = RG_HALF * (y2 - y4);
    py1 = RG_HALF * (x4 - x2);
    px2 = RG_HALF * y3;
    py2 = -RG_HALF * x3;
    area = dmax(RG_TWO * (py2 * px1 - py1 * px2), RG_EM20);
    vhx = (-x2 + x3 - x4) / area;
    vhy = (-y2 + y3 - y4) / area;
  }
  // ---- CCOEF3 (ccoef3.F:74-90): ITHK > 0 works on the current thickness,
  // ITHK = 0 on the initial one (THK0 = THKE from CCOOR3, ccoor3.F:80) ----
  const double vol00 = thk0 * area;
  if (G.ithk > 0) thk0 = S->thk[e];
  const double vol0 = thk0 * area;
  const double thk02 = thk0 * thk0;
  const double rho = G.rho, ym = G.young, nu = G.nu, gmod = G.g, a11 = G.a11;
  const double ssp = G.ssp;
  double shf;
  if (G.npt == 1) {
    shf = RG_ZERO;
  } else {
    const double fac1tmp = 2.0 * (1.0 + nu) * thk02;
    const double ish = std::nearbyint(G.ish);
    const double fsh = G.fsh;
    shf = fsh * (1.0 - ish + ish * fac1tmp / (fsh * area + fac1tmp));
  }
  const double gs = gmod * shf;
  (void)vol00;
  // ---- CDLEN3 (cdlen3.F:30), IHBE /= 0 ----
  double aldt;
  {
    const double al1 = x2 * x2 + y2 * y2;
    const double al2 = (x3 - x2) * (x3 - x2) + (y3 - y2) * (y3 - y2);
    const double al6 = x3 * x3 + y3 * y3;
    const double al3 = (x4 - x3) * (x4 - x3) + (y4 - y3) * (y4 - y3);
    const double al4 = x4 * x4 + y4 * y4;
    const double al5 = (x4 - x2) * (x4 - x2) + (y4 - y2) * (y4 - y2);
    double almin = dmin(dmin(al1, al2), al4);
    const double alquad = dmin(dmin(al3, al5), al6);
    if (al3 != RG_ZERO) almin = dmin(almin, alquad);
    const double dtdyn = area * area / dmax(dmax(al5, al6), RG_EM20);
    aldt = dmax(dtdyn, almin);
    const double dthour = RG_HALF * (almin + aldt) / dmax(G.h1, G.h2);
    if (dthour < aldt) aldt = dthour;
    aldt = std::sqrt(aldt);
  }
  // ---- CDEFO3 (cdefo3.F:30), IHBE <= 1 ----
  double vx[4], vy[4], vz[4];
  double exx, eyy, exy, exz, eyz;
  for (int k = 0; k < 4; k++) {
    vx[k] = e1x * vl[k][0] + e1y * vl[k][1] + e1z * vl[k][2];
    vy[k] = e2x * vl[k][0] + e2y * vl[k][1] + e2z * vl[k][2];
    vz[k] = e3x * vl[k][0] + e3y * vl[k][1] + e3z * vl[k][2];
  }
  {
    const double vz13 = vz[0] - vz[2], vz24 = vz[1] - vz[3];
    eyz = py1 * vz13 + py2 * vz24;
    exz = px1 * vz13 + px2 * vz24;
    const double dt1v4 = RG_FOURTH * DT1;
    const double tmp2a = py2 + py1;
    const double tmp3a = std::copysign(dmax(std::fabs(tmp2a), RG_EM20), tmp2a);
    const double tmp1a = dt1v4 * (vz13 - vz24) * (vz13 - vz24) / tmp3a;
    double vx13 = vx[0] - vx[2], vx24 = vx[1] - vx[3];
    vx13 = vx13 - tmp1a;
    vx24 = vx24 + tmp1a;
    exx = px1 * vx13 + px2 * vx24;
    exy = py1 * vx13 + py2 * vx24;
    const double tmp1b = px2 - px1;
    const double tmp3b = std::copysign(dmax(std::fabs(tmp1b), RG_EM20), tmp1b);
    const double tmp2b = dt1v4 * (vz13 + vz24) * (vz13 + vz24) / tmp3b;
    double vy13 = vy[0] - vy[2], vy24 = vy[1] - vy[3];
    vy13 = vy13 + tmp2b;
    vy24 = vy24 + tmp2b;
    exy = exy + px1 * vy13 + px2 * vy24;
    eyy = py1 * vy13 + py2 * vy24;
  }
  // ---- CCURV3 (ccurv3.F:30) ----
  double rx[4], ry[4], kxx, kyy, kxy;
  for (int k = 0; k < 4; k++) {
    rx[k] = e1x * vrl[k][0] + e1y * vrl[k][1] + e1z * vrl[k][2];
    ry[k] = e2x * vrl[k][0] + e2y * vrl[k][1] + e2z * vrl[k][2];
  }
  {
    const double rx13 = rx[0] - rx[2], rxav = rx[0] + rx[1] + rx[2] + rx[3], rx24 = rx[1] - rx[3];
    kyy = -py1 * rx13 - py2 * rx24;
    kxy = px1 * rx13 + px2 * rx24;
    const double ry13 = ry[0] - ry[2], ryav = ry[0] + ry[1] + ry[2] + ry[3], ry24 = ry[1] - ry[3];
    kxx = px1 * ry13 + px2 * ry24;
    kxy = py1 * ry13 + py2 * ry24 - kxy;
    exz = exz + ryav * (0.25 * area);
    eyz = eyz - rxav * (0.25 * area);
  }
  // ---- CSTRA3 (cstra3.F:30): increments, GSTR (ISTRAIN = 1) ----
  {
    const double fac1 = DT1 / area;
    exx = exx * fac1;
    eyy = eyy * fac1;
    exy = exy * fac1;
    eyz = eyz * fac1;
    exz = exz * fac1;
    kxx = kxx * fac1;
    kyy = kyy * fac1;
    kxy = kxy * fac1;
    GST_(0, e) += exx;
    GST_(1, e) += eyy;
    GST_(2, e) += exy;
    GST_(3, e) += eyz;
    GST_(4, e) += exz;
    GST_(5, e) += kxx;
    GST_(6, e) += kyy;
    GST_(7, e) += kxy;
  }
  // element strain rate (cforc3.F, before CMAIN3): ASRATE = 1
  double epsd_pg;
  {
    const double dtinv = DT1 / dmax(DT1 * DT1, RG_EM20);
    const double th = S->thk[e];
    const double eps_k2 = (kxx * kxx + kyy * kyy + kxx * kyy + RG_FOURTH * kxy * kxy) *
                          RG_ONE_OVER_9 * th * th;
    const double eps_m2 = RG_FOUR_OVER_3 * (exx * exx + eyy * eyy + exx * eyy + RG_FOURTH * exy * exy);
    epsd_pg = std::sqrt(eps_k2 + eps_m2) * dtinv;
    S->epsdg[e] = RG_ONE * epsd_pg + (RG_ONE - RG_ONE) * S->epsdg[e];
  }
  // ---- MULAWC (materials/mat_share/mulawc.F90:185) ----
  double degmb = FOR_(0, e) * exx + FOR_(1, e) * eyy + FOR_(2, e) * exy + FOR_(3, e) * eyz +
                 FOR_(4, e) * exz;
  double degfx = MOM_(0, e) * kxx + MOM_(1, e) * kyy + MOM_(2, e) * kxy;
  double thkn = S->thk[e];
  double forn[5] = {0, 0, 0, 0, 0}, momn[3] = {0, 0, 0};
  const double asrate = G.israte > 0 ? dmin(RG_ONE, G.pm9 * DT1) : RG_ONE;
  const int npt = G.npt;
  double sigy_acc = RG_ZERO;
  for (int it = 0; it < npt; it++) {
    const double thkly = (double)WFT[npt - 1][it];
    const double thklyl = thkly * thk0;
    const double wmc = (double)WMT[npt - 1][it];
    const double zt = (double)Z0T[npt - 1][it] * thk0;
    const double depsxx = exx + zt * kxx;
    const double depsyy = eyy + zt * kyy;
    const double depsxy = exy + zt * kxy;
    const double depsyz = eyz, depszx = exz;
    double so[5], sn[5];
    for (int c = 0; c < 5; c++) so[c] = SIG_(c, it, e);
    // SIGEPS02C (materials/mat/mat002/sigeps02c.F:33)
    const double young = G.young, gg = G.g, nuu = G.nu;
    const double a1 = young / (RG_ONE - nuu * nuu);
    const double a2 = a1 * nuu;
    const double epdr = dmax(G.eps0 * DT1, RG_EM20);
    double epsdot;
    {
      double &ep = EPS_(it, e);
      if (G.vp == 2) {
        ep = asrate * epsd_pg + (RG_ONE - asrate) * ep;
        epsdot = ep * DT1;
      } else {
        epsdot = ep * DT1;  // VP = 1: previous filtered plastic rate
      }
    }
    // SIGEPS02C: T* from the point's temperature (sigeps02c.F:125; JC, the
    // point buffer starts at TINI = TREF, allocbuf_auto.F:189)
    double tstar = RG_ZERO;
    if (G.thermal) tstar = dmax(RG_ZERO, (TMP_(it, e) - G.tref) / (G.tmelt - G.tref));
    // M2CPLR (materials/mat/mat002/m2cplr.F:29)
    double ezz = RG_ZERO;
    double ca = G.ca, cb = G.cb, ymax = G.ymax, h = RG_ZERO;
    double dpla = RG_ZERO;
    const double fisokin = G.fisokin;
    for (int c = 0; c < 5; c++) sn[c] = so[c];
    // kinematic hardening: the predictor works on the shifted stress
    // (m2cplr.F:115-121)
    if (fisokin > RG_ZERO) {
      sn[0] = sn[0] - SGB_(0, it, e);
      sn[1] = sn[1] - SGB_(1, it, e);
      sn[2] = sn[2] - SGB_(2, it, e);
    }
    sn[0] = sn[0] + a1 * depsxx + a2 * depsyy;
    sn[1] = sn[1] + a2 * depsxx + a1 * depsyy;
    sn[2] = sn[2] + gg * depsxy;
    sn[3] = sn[3] + gs * depsyz;
    sn[4] = sn[4] + gs * depszx;
    double logep = RG_ZERO;
    if (G.cc != RG_ZERO) {
      double epsp = epsdot;
      if (G.israte == 0 && G.vp == 2)
        epsp = dmax(dmax(std::fabs(depsxx), std::fabs(depsyy)), RG_HALF * std::fabs(depsxy));
      epsp = dmax(epsp, epdr);
      logep = std::log(epsp / epdr);
      double q;
      if (tstar == RG_ZERO)
        q = (RG_ONE + G.cc * logep);
      else
        q = (RG_ONE + G.cc * logep) * (RG_ONE - std::exp(G.m_exp * std::log(tstar)));
      q = dmax(q, RG_EM20);
      ca = ca * q;
      cb = cb * q;
      if (G.icc == 1) ymax = ymax * q;
    } else if (tstar != RG_ZERO) {
      // CC = 0: thermal softening alone (m2cplr.F:169-178)
      double q = RG_ONE - std::exp(G.m_exp * std::log(tstar));
      q = dmax(q, RG_EM20);
      ca = ca * q;
      cb = cb * q;
    }
    double &pla = PLA_(it, e);
    double yld;
    if (pla == RG_ZERO)
      yld = ca;
    else
      yld = ca + cb * (RG_ONE - fisokin) * std::exp(G.cn * std::log(pla));
    yld = dmin(yld, ymax);
    if (G.ipla == 0) {
      const double svm = std::sqrt(sn[0] * sn[0] + sn[1] * sn[1] - sn[0] * sn[1] + RG_THREE * sn[2] * sn[2]);
      const double r = dmin(RG_ONE, yld / (svm + RG_EM15));
      if (r < RG_ONE) {
        sn[0] = sn[0] * r;
        sn[1] = sn[1] * r;
        sn[2] = sn[2] * r;
        dpla = off * dmax(RG_ZERO, (svm - yld) / young);
        const double s1 = RG_HALF * (sn[0] + sn[1]);
        ezz = dpla * s1 / yld;
        pla = pla + dpla;
        if (yld >= ymax)
          h = RG_ZERO;
        else
          h = G.cn * cb * std::exp((G.cn - RG_ONE) * std::log(pla + RG_EM07));
      }
    } else if (G.ipla == 2) {
      // m2cplr.F:380-445: projection along an approximate normal, then a
      // radial return to the updated yield stress
      const double svm2 = sn[0] * sn[0] + sn[1] * sn[1] - sn[0] * sn[1] + RG_THREE * sn[2] * sn[2];
      const double svm = std::sqrt(svm2);
      const double yld2 = yld * yld;
      if (svm2 > yld2 && off == RG_ONE) {
        if (yld >= ymax)
          h = RG_ZERO;
        else
          h = G.cn * cb * std::exp((G.cn - RG_ONE) * std::log(pla + RG_EM07));
        const double aa = (svm2 - yld2) /
                          (RG_FIVE * svm2 + RG_THREE * (-(sn[0] * sn[1]) + sn[2] * sn[2]));
        const double s1 = (RG_ONE - RG_TWO * aa) * sn[0] + aa * sn[1];
        const double s2 = aa * sn[0] + (RG_ONE - RG_TWO * aa) * sn[1];
        const double s3 = (RG_ONE - RG_THREE * aa) * sn[2];
        sn[0] = s1;
        sn[1] = s2;
        sn[2] = s3;
        dpla = off * (svm - yld) / (RG_THREE * gg + h);
        pla = pla + dpla;
        yld = yld + h * dpla;
        const double svmn =
            std::sqrt(sn[0] * sn[0] + sn[1] * sn[1] - sn[0] * sn[1] + RG_THREE * sn[2] * sn[2]);
        const double r = dmin(RG_ONE, yld / dmax(RG_EM20, svmn));
        sn[0] = sn[0] * r;
        sn[1] = sn[1] * r;
        sn[2] = sn[2] * r;
        ezz = dpla * RG_HALF * (sn[0] + sn[1]) / yld;
      }
    } else {
      const double s1 = sn[0] + sn[1];
      const double s2 = sn[0] - sn[1];
      const double s3 = sn[2];
      const double A = RG_FOURTH * s1 * s1;
      const double B = RG_THREE_OVER_4 * s2 * s2 + RG_THREE * s3 * s3;
      const double svm = std::sqrt(A + B);
      if (svm > yld && off == RG_ONE) {
        const double nu1 = RG_ONE / (RG_ONE - nuu);
        const double nu2 = RG_ONE / (RG_ONE + nuu);
        if (yld >= ymax)
          h = RG_ZERO;
        else
          h = G.cn * cb * std::exp((G.cn - RG_ONE) * std::log(pla + RG_EM07));
        double dpla_j = (svm - yld) / (RG_THREE * gg + h);
        // isotropic Newton (FISOKIN = 0) or the kinematic / mixed one
        // (m2cplr.F:289-363): modified NU1, NU2 and the isotropic part of H
        double nu1k = nu1, nu2k = RG_THREE * nu2, h2 = RG_TWO * h, beta = RG_ONE;
        double anu1 = A * nu1, bnu2 = RG_THREE * B * nu2;
        if (fisokin > RG_ZERO) {
          const double bh = h * fisokin;
          const double hi = h - bh;
          const double hk = RG_TWO_THIRD * bh;
          const double aaa = RG_THREE * hk / young;
          nu1k = nu1 + aaa;
          nu2k = RG_THREE * nu2 + aaa;
          anu1 = A * nu1k;
          bnu2 = B * nu2k;
          h2 = RG_TWO * hi;
          beta = RG_ONE - fisokin;
        }
        double dpla_i = 0, P = 1, Q = 1, dr = 0;
        for (int n = 0; n < 3; n++) {
          dpla_i = dpla_j;
          const double pla_i = pla + dpla_i;
          double yld_i;
          if (pla_i == RG_ZERO)
            yld_i = dmin(ymax, ca);
          else if (fisokin > RG_ZERO)
            yld_i = dmin(ymax, ca + beta * cb * std::exp(G.cn * std::log(pla_i)));
          else
            yld_i = dmin(ymax, ca + cb * std::exp(G.cn * std::log(pla_i)));
          dr = RG_HALF * young * dpla_i / yld_i;
          if (fisokin > RG_ZERO) {
            P = RG_ONE / (RG_ONE + dr * nu1k);
            Q = RG_ONE / (RG_ONE + dr * nu2k);
          } else {
            P = RG_ONE / (RG_ONE + dr * nu1);
            Q = RG_ONE / (RG_ONE + RG_THREE * dr * nu2);
          }
          const double p2 = P * P, q2 = Q * Q;
          const double f = A * p2 + B * q2 - yld_i * yld_i;
          const double df = -(anu1 * p2 * P + bnu2 * q2 * Q) * (young - dr * h2) / yld_i - h2 * yld_i;
          if (dpla_i > RG_ZERO)
            dpla_j = dmax(RG_ZERO, dpla_i - f / df);
          else
            dpla_j = RG_ZERO;
        }
        dpla = dpla_i;
        pla = pla + dpla_i;
        const double t1 = (sn[0] + sn[1]) * P;
        const double t2 = (sn[0] - sn[1]) * Q;
        sn[0] = RG_HALF * (t1 + t2);
        sn[1] = RG_HALF * (t1 - t2);
        sn[2] = sn[2] * Q;
        ezz = dr * t1 / young;
        // kinematic: YLD from the new PLA, H kept (m2cplr.F:465-476)
        if (fisokin > RG_ZERO) {
          if (pla == RG_ZERO)
            yld = ca;
          else
            yld = dmin(ymax, ca + beta * cb * std::exp(G.cn * std::log(pla)));
        }
      }
    }
    // kinematic / mixed hardening: back stress update, stress shifted back
    // (m2cplr.F:477-490)
    if (fisokin > RG_ZERO) {
      const double hkin = fisokin * h;
      const double alpha = hkin * dpla / yld;
      for (int c = 0; c < 3; c++) {
        SGB_(c, it, e) = SGB_(c, it, e) + alpha * sn[c];
        sn[c] = sn[c] + SGB_(c, it, e);
      }
    }
    // SIGEPS02C: SIGY accumulates YLD / NPT over the points so far, and the
    // adiabatic heating of this point uses that running sum
    // (sigeps02c.F:197-199, 226-229; SIGY zeroed per group, mulawc.F90:577)
    sigy_acc = sigy_acc + yld / (double)npt;
    if (G.thermal) TMP_(it, e) = TMP_(it, e) + sigy_acc * dpla / G.rhocp;
    // SIGEPS02C epilogue: thickness strain, thickness (INLOC = 0)
    ezz = -(depsxx + depsyy) * nuu - (RG_ONE - RG_TWO * nuu) * ezz;
    ezz = ezz / (RG_ONE - nuu);
    thkn = thkn + ezz * thklyl * off;
    for (int c = 0; c < 5; c++) SIG_(c, it, e) = sn[c] * RG_ONE;
    forn[0] = forn[0] + thkly * sn[0];
    forn[1] = forn[1] + thkly * sn[1];
    forn[2] = forn[2] + thkly * sn[2];
    forn[3] = forn[3] + thkly * sn[3];
    forn[4] = forn[4] + thkly * sn[4];
    momn[0] = momn[0] + wmc * sn[0];
    momn[1] = momn[1] + wmc * sn[1];
    momn[2] = momn[2] + wmc * sn[2];
  }
  S->thk[e] = dmax(thkn, RG_EM30);
  if (G.dm != RG_ZERO) {
    const double dtinv = DT1 / dmax(DT1 * DT1, RG_EM20);
    const double visc = (RG_ONEP414 * G.dm) * ssp * std::sqrt(area) * dtinv * rho;
    forn[0] = forn[0] + visc * (exx + RG_HALF * eyy);
    forn[1] = forn[1] + visc * (eyy + RG_HALF * exx);
    forn[2] = forn[2] + visc * exy * RG_THIRD;
  }
  for (int c = 0; c < 5; c++) forn[c] = forn[c] * off * RG_ONE;
  for (int c = 0; c < 3; c++) momn[c] = momn[c] * off * RG_ONE;
  degmb = degmb + forn[0] * exx + forn[1] * eyy + forn[2] * exy + forn[3] * eyz + forn[4] * exz;
  degfx = degfx + momn[0] * kxx + momn[1] * kyy + momn[2] * kxy;
  {
    const double vol2 = RG_HALF * vol0;
    EIN_(0, e) = EIN_(0, e) + degmb * vol2;
    EIN_(1, e) = EIN_(1, e) + degfx * thk0 * vol2;
  }
  for (int c = 0; c < 5; c++) FOR_(c, e) = forn[c];
  for (int c = 0; c < 3; c++) MOM_(c, e) = momn[c];
  const double viscmx = std::sqrt(RG_ONE + RG_ZERO * RG_ZERO) - RG_ZERO;
  // ---- CHVIS3 (chvis3.F:32), ISMSTR = 4, IHBE = 1 ----
  double h11, h12, h13, h21, h22, h23, h31, h32, h33, b1x[4], b2x[4], ehou;
  double sti_noda = RG_ZERO, stir_noda = RG_ZERO;
  {
    const double px1v = px1 * vhx, px2v = px2 * vhx, py1v = py1 * vhy, py2v = py2 * vhy;
    const double gama1 = off * (RG_ONE - px1v - py1v);
    const double gama3 = off * (RG_ONE + px1v + py1v);
    const double gama2 = off * (-RG_ONE - px2v - py2v);
    const double gama4 = off * (-RG_ONE + px2v + py2v);
    const double sr2d2 = std::sqrt(RG_TWO) * RG_HALF;
    const double hvisc = RG_HALF, hvlin = RG_ZERO, helas = RG_HALF;
    const double zep072169 = RG_ZEP072169;
    const double shfpr3 = shf / (RG_THREE * (RG_ONE + nu));
    const double hvish1 = hvisc * G.h1, hvish2 = hvisc * G.h2;
    double r0 = RG_FOURTH * rho;
    const double r1 = r0 * RG_HUNDRED;
    r0 = r0 * hvlin;
    const double A1 = r1 * hvish1;
    const double A2 = r0 * sr2d2 * G.srh1;
    const double srshfpr3 = std::sqrt(shfpr3);
    const double A3 = r1 * hvish2 * srshfpr3;
    const double A4 = r0 * sr2d2 * G.srh2 * srshfpr3;
    double hh3 = helas * G.h3;
    const double A5 = hh3 * r1 * zep072169;
    hh3 = sr2d2 * G.srh3;
    const double A6 = hh3 * r0 * zep072169;
    const double r0e = RG_FOURTH * ym * helas;
    const double A7 = G.h1 * r0e;
    const double A8 = G.h2 * r0e * shfpr3;
    const double t2a = thk02 * area;
    const double tsa = std::sqrt(t2a);
    double h1q = A1 * tsa, h1l = A2 * ssp * tsa;
    double h2q = A3 * thk02, h2l = A4 * ssp * thk02;
    double h3q = A5 * t2a, h3l = A6 * ssp * t2a;
    const double td = thk0 * DT1;
    double hh1 = A7 * td;
    const double b1 = px1 * px1 + py1 * py1, b2 = px2 * px2 + py2 * py2;
    double hh2 = A8 * thk02 * td / (b1 + b2);
    if (ix[3] == ix[4]) h1q = h1l = h2q = h2l = h3q = h3l = hh1 = hh2 = RG_ZERO;
    if (S->nodadt) {
      // nodal time step (chvis3.F:198-265, IGTYP=1, no adaptive meshing):
      // element stiffness for DTNODA, with the hourglass stiffness SCALE
      const double scale =
          dmax(dmax(gama1 * gama1, gama2 * gama2), dmax(gama3 * gama3, gama4 * gama4)) * DT1 *
          dmax(dmax(hh1 + h1l, hh2 + h2l), h3l) / dmax(DT1 * DT1, RG_EM20);
      if (off == RG_ZERO) {
        sti_noda = stir_noda = RG_ZERO;
      } else {
        const double vv = viscmx * viscmx * RG_ONE;  // VISCMX^2 * ALPE
        sti_noda = RG_ZERO + scale;
        sti_noda = sti_noda + dmax(b1, b2) * thk0 * a11 / (area * vv);
        stir_noda = sti_noda * (thk02 * RG_ONE_OVER_12 + area * RG_ONE_OVER_9);
      }
    }
    double hg1 = vx[0] * gama1 + vx[1] * gama2 + vx[2] * gama3 + vx[3] * gama4;
    double hg2 = vy[0] * gama1 + vy[1] * gama2 + vy[2] * gama3 + vy[3] * gama4;
    HOU_(0, e) = HOU_(0, e) + hg1 * hh1;
    HOU_(1, e) = HOU_(1, e) + hg2 * hh1;
    const double hour1a = HOU_(0, e) + hg1 * (h1l + h1q * std::fabs(hg1));
    h11 = hour1a * gama1;
    h12 = hour1a * gama2;
    h13 = hour1a * gama3;
    const double hour2a = HOU_(1, e) + hg2 * (h1l + h1q * std::fabs(hg2));
    h21 = hour2a * gama1;
    h22 = hour2a * gama2;
    h23 = hour2a * gama3;
    ehou = hour1a * hg1 + hour2a * hg2;
    hg1 = vz[0] * gama1 + vz[1] * gama2 + vz[2] * gama3 + vz[3] * gama4;
    HOU_(2, e) = HOU_(2, e) + hg1 * hh2;
    const double hour3a = HOU_(2, e) + hg1 * (h2l + h2q * std::fabs(hg1));
    h31 = hour3a * gama1;
    h32 = hour3a * gama2;
    h33 = hour3a * gama3;
    ehou = ehou + hour3a * hg1;
    hg1 = rx[0] - rx[1] + rx[2] - rx[3];
    hg2 = ry[0] - ry[1] + ry[2] - ry[3];
    HOU_(3, e) = hg1 * (h3l + h3q * std::fabs(hg1));
    HOU_(4, e) = hg2 * (h3l + h3q * std::fabs(hg2));
    ehou = ehou + HOU_(3, e) * hg1 + HOU_(4, e) * hg2;
    ehou = DT1 * ehou * off;
    b1x[0] = HOU_(3, e) * off;
    b1x[1] = -HOU_(3, e) * off;
    b1x[2] = HOU_(3, e) * off;
    b1x[3] = -HOU_(3, e) * off;
    b2x[0] = HOU_(4, e) * off;
    b2x[1] = -HOU_(4, e) * off;
    b2x[2] = HOU_(4, e) * off;
    b2x[3] = -HOU_(4, e) * off;
  }
  // ---- CDT3 (cdt3.F:32): element time step, STI; not called under the
  // nodal time step (cforc3.F:668, IDTMIN(3) = 0) ----
  double sti = sti_noda, stir = stir_noda;
  if (!S->nodadt) {
    aldt = aldt * viscmx / std::sqrt(RG_ONE);
    const double dt = dtfac * aldt / ssp;
    // IDTMIN(3) (cdt3.F:77-141), ahead of the minimum loop (cdt3.F:143-155):
    // 1 / 5 flag the stop; 2 deletes the element (OFF = 0)
    if (S->idtmin && !(dt > S->dtmin) && !(off < RG_ONE) && !(S->offg[e] < RG_ZERO)) {
      if (S->idtmin == 2)
        off = RG_ZERO;
      else
        S->stop = 1;
    }
    if (S->offg[e] > RG_ZERO && off != RG_ZERO && dt < dt2t) {
      dt2t = dt;
      elmin = e;
    }
    const double divm = dmax(aldt * aldt, RG_EM20);
    sti = RG_HALF * vol0 * ym / divm;
    sti = RG_ZEP81 * sti * off;
    stir = RG_ZERO;
  }
  // ---- CFINT3 (cfint3.F:30), ISIGI /= 5 ----
  double F[3][4], M[3][4];
  {
    const double f1a = forn[0] * thk0, f2a = forn[1] * thk0, f3a = forn[2] * thk0;
    const double f4a = forn[3] * thk0, f5a = forn[4] * thk0;
    double m4 = f4a * area, m5 = f5a * area;
    double f12 = f1a * px2 + f3a * py2;
    double f22 = f2a * py2 + f3a * px2;
    double f32 = f5a * px2 + f4a * py2;
    double f11 = f1a * px1 + f3a * py1;
    double f21 = f2a * py1 + f3a * px1;
    double f31 = f5a * px1 + f4a * py1;
    const double g11 = f11 + h11, g13 = h13 - f11;
    const double g21 = f21 + h21, g23 = h23 - f21;
    const double g31 = f31 + h31, g33 = h33 - f31;
    const double g12 = f12 + h12, g22 = f22 + h22, g32 = f32 + h32;
    F[0][0] = e1x * g11 + e2x * g21 + e3x * g31;
    F[0][1] = e1x * g12 + e2x * g22 + e3x * g32;
    F[0][2] = e1x * g13 + e2x * g23 + e3x * g33;
    F[1][0] = e1y * g11 + e2y * g21 + e3y * g31;
    F[1][1] = e1y * g12 + e2y * g22 + e3y * g32;
    F[1][2] = e1y * g13 + e2y * g23 + e3y * g33;
    F[2][0] = e1z * g11 + e2z * g21 + e3z * g31;
    F[2][1] = e1z * g12 + e2z * g22 + e3z * g32;
    F[2][2] = e1z * g13 + e2z * g23 + e3z * g33;
    for (int c = 0; c < 3; c++) F[c][3] = -F[c][0] - F[c][1] - F[c][2];
    const double m1a = momn[0] * thk02, m2a = momn[1] * thk02, m3a = momn[2] * thk02;
    m4 = m4 * RG_FOURTH;
    m5 = m5 * RG_FOURTH;
    const double m11 = -m2a * py1 - m3a * px1;
    const double m21 = m1a * px1 + m3a * py1;
    const double m12 = -m2a * py2 - m3a * px2;
    const double m22 = m1a * px2 + m3a * py2;
    const double G11 = m11 - m4 + b1x[0];
    const double G13 = -m11 - m4 + b1x[2];
    const double G12 = m12 - m4 + b1x[1];
    const double G14 = -m12 - m4 + b1x[3];
    const double G21 = m21 + m5 + b2x[0];
    const double G23 = -m21 + m5 + b2x[2];
    const double G22 = m22 + m5 + b2x[1];
    const double G24 = -m22 + m5 + b2x[3];
    const double gg1[4] = {G11, G12, G13, G14}, gg2[4] = {G21, G22, G23, G24};
    for (int k = 0; k < 4; k++) {
      M[0][k] = e1x * gg1[k] + e2x * gg2[k];
      M[1][k] = e1y * gg1[k] + e2y * gg2[k];
      M[2][k] = e1z * gg1[k] + e2z * gg2[k];
    }
  }
  // ---- CUPDT3P (cupdt3.F:967-1100) ----
  if (off < RG_ONE) S->offg[e] = off;
  const bool zero = S->offg[e] < RG_ZERO;
  for (int k = 0; k < 4; k++) {
    const int K = S->iadc[4 * (size_t)e + k] - 1;
    double *fs = &fsky[8 * (size_t)K];
    fs[0] = zero ? RG_ZERO : -F[0][k];
    fs[1] = zero ? RG_ZERO : -F[1][k];
    fs[2] = zero ? RG_ZERO : -F[2][k];
    fs[3] = zero ? RG_ZERO : -M[0][k];
    fs[4] = zero ? RG_ZERO : -M[1][k];
    fs[5] = zero ? RG_ZERO : -M[2][k];
    fs[6] = zero ? RG_ZERO : sti;
    fs[7] = zero ? RG_ZERO : stir;
  }
  // accumulated hourglass energy (part sums, PARTSAV(8))
  S->ehou[e] += ehou;
}

void step(Shells *S, const double *X, const double *V, const double *VR,
          double *fsky, double dt1, double dtfac, double &dt2t, int &neltst,
          int &error, int nthreads) {
  const int ne = S->numelc;
  if (ne == 0) return;
  const int ng = (int)S->groups.size();
  if (!S->temp_init) {
    // each point's temperature starts at its material's TREF (TINI)
    for (const Group &G : S->groups)
      for (int p = 0; p < 5; p++)
        for (int i = 0; i < G.nel; i++) TMP_(p, G.nft + i) = G.tref;
    S->temp_init = true;
  }
  std::vector<double> gdt(ng, RG_EP06);
  std::vector<int> gel(ng, -1);
  RG_OPCOUNT_PHASE(2);
#pragma omp parallel for schedule(dynamic, 1) num_threads(nthreads)
  for (int g = 0; g < ng; g++) {
    const Group &G = S->groups[g];
    double d = RG_EP06;
    int el = -1;
    for (int i = 0; i < G.nel; i++)
      element(S, G, G.nft + i, X, V, VR, fsky, dt1, dtfac, d, el);
    gdt[g] = d;
    gel[g] = el;
  }
  RG_OPCOUNT_PHASE(0);
  // CDT3 keeps the first element attaining the minimum (strict <)
  int best = -1;
  double bd = dt2t;
  for (int g = 0; g < ng; g++)
    if (gel[g] >= 0 && gdt[g] < bd) {
      bd = gdt[g];
      best = gel[g];
    }
  if (best >= 0) {
    dt2t = bd;
    neltst = S->ixc[7 * (size_t)best + 6];
  }
  if (S->stop.exchange(0)) error |= 8;
}

// CBILAN (elements/shell/coque/cbilan.F:160-190) + CHVIS3's PARTSAV(8)
// (chvis3.F:355-395): per-part sums of the element pass just done, from the
// cycle's X(n) and V(n-1/2): IE = EINT(1) + EINT(2), KE = XMAS sum v^2 / 8,
// momentum XMAS / 4 sum v, mass of the elements not switched off, the
// accumulated hourglass energy.  XMAS = RHO * AREA * THK with the area of
// the cycle's coordinates (half the norm of the diagonals' cross product)
// and the thickness after the cycle's update.  part: the shell's part, or
// null for part0 + its group.  Adds into out[part][7].
void part_sums(const Shells *S, const double *X, const double *V, const int *part, int part0,
               double *out) {
  for (size_t g = 0; g < S->groups.size(); g++) {
    const Group &G = S->groups[g];
    for (int i = 0; i < G.nel; i++) {
      const int e = G.nft + i;
      const int *ix = &S->ixc[7 * (size_t)e];
      const double *x1 = &X[3 * (size_t)(ix[1] - 1)], *x2 = &X[3 * (size_t)(ix[2] - 1)];
      const double *x3 = &X[3 * (size_t)(ix[3] - 1)], *x4 = &X[3 * (size_t)(ix[4] - 1)];
      const double *v1 = &V[3 * (size_t)(ix[1] - 1)], *v2 = &V[3 * (size_t)(ix[2] - 1)];
      const double *v3 = &V[3 * (size_t)(ix[3] - 1)], *v4 = &V[3 * (size_t)(ix[4] - 1)];
      const double ax = x3[0] - x1[0], ay = x3[1] - x1[1], az = x3[2] - x1[2];
      const double bx = x4[0] - x2[0], by = x4[1] - x2[1], bz = x4[2] - x2[2];
      const double cx = ay * bz - az * by, cy = az * bx - ax * bz, cz = ax * by - ay * bx;
      const double area = RG_HALF * std::sqrt(cx * cx + cy * cy + cz * cz);
      const double xmas = G.rho * (area * S->thk[e]);
      const double vxa = v1[0] + v2[0] + v3[0] + v4[0];
      const double vya = v1[1] + v2[1] + v3[1] + v4[1];
      const double vza = v1[2] + v2[2] + v3[2] + v4[2];
      const double va2 = v1[0] * v1[0] + v2[0] * v2[0] + v3[0] * v3[0] + v4[0] * v4[0] +
                         v1[1] * v1[1] + v2[1] * v2[1] + v3[1] * v3[1] + v4[1] * v4[1] +
                         v1[2] * v1[2] + v2[2] * v2[2] + v3[2] * v3[2] + v4[2] * v4[2];
      const double xmas25 = xmas * RG_FOURTH;
      double *o = &out[7 * (size_t)(part ? part[e] : part0 + (int)g)];
      o[0] += S->eint[e] + S->eint[(size_t)S->numelc + e];
      o[1] += xmas * va2 * RG_ONE_OVER_8;
      o[2] += xmas25 * vxa;
      o[3] += xmas25 * vya;
      o[4] += xmas25 * vza;
      if (S->offg[e] != RG_ZERO) o[5] += xmas;
      o[6] += S->ehou[e];
    }
  }
}

int group_count(const Shells *S) { return (int)S->groups.size(); }

void energy(const Shells *S, double &eint, double &ehour) {
  eint = 0;
  ehour = 0;
  for (int e = 0; e < S->numelc; e++) {
    eint += S->eint[e] + S->eint[(size_t)S->numelc + e];
    ehour += S->ehou[e];
  }
}

int rwall_add(Shells *, const double *, const double *, double) { return -1; }
void rwall_apply(Shells *, int, const double *, double *, const double *, double) {}

// state download: which = 0 FOR (5 x ne), 1 MOM (3 x ne), 2 THK, 3 EINT
// (2 x ne), 4 OFF, 5 SIG (5 x npt x ne), 6 PLA (npt x ne), 7 HOUR (5 x ne)
int get_state(const Shells *S, int which, double *out) {
  const size_t n = S->numelc;
  switch (which) {
    case 0: std::copy(S->forc.begin(), S->forc.begin() + 5 * n, out); return 0;
    case 1: std::copy(S->mom.begin(), S->mom.begin() + 3 * n, out); return 0;
    case 2: std::copy(S->thk.begin(), S->thk.end(), out); return 0;
    case 3: std::copy(S->eint.begin(), S->eint.begin() + 2 * n, out); return 0;
    case 4: std::copy(S->offg.begin(), S->offg.end(), out); return 0;
    case 5: {
      const int npt = S->groups.empty() ? 0 : S->groups[0].npt;
      for (int p = 0; p < npt; p++)
        for (int c = 0; c < 5; c++)
          for (size_t e = 0; e < n; e++) out[((size_t)p * 5 + c) * n + e] = S->sig[((size_t)p * 5 + c) * n + e];
      return 0;
    }
    case 6: {
      const int npt = S->groups.empty() ? 0 : S->groups[0].npt;
      std::copy(S->pla.begin(), S->pla.begin() + npt * n, out);
      return 0;
    }
    case 7: std::copy(S->hour.begin(), S->hour.begin() + 5 * n, out); return 0;
    case 8: {  // back stress per IP: [npt][3][n]
      const int npt = S->groups.empty() ? 0 : S->groups[0].npt;
      std::copy(S->sigbak.begin(), S->sigbak.begin() + 3 * npt * n, out);
      return 0;
    }
    case 9: {  // temperature per IP: [npt][n]
      const int npt = S->groups.empty() ? 0 : S->groups[0].npt;
      std::copy(S->temp.begin(), S->temp.begin() + npt * n, out);
      return 0;
    }
  }
  return -1;
}

}  // namespace rg_oracle_shell
