// Belytschko-Tsay shell element kernel (single model) and the host-side
// bookkeeping of the shell groups; the element arithmetic is
// shell_element() in rg_shell_elem.cuh.
#include "../../include/rg_api.h"
#include "rg_shell.h"
#include "rg_shell_elem.cuh"
#include "rg_node.cuh"

#include <algorithm>
#include <cmath>
#include <cstring>
#include <type_traits>
#include <vector>

namespace rg {

struct ShellGroupHost {
  ShellParams P{};
};

struct ShellDev {
  ShellArrays<double> a64{};
  ShellArrays<float> a32{};
  int prec = 0;
  int *ix = nullptr, *iadc = nullptr, *degen = nullptr;
  double *epart = nullptr;  // energy partials
};

// Block size and resident blocks per SM of the mixed kernel (its register
// budget: 128 registers either way); the FP64 kernel runs 128-thread blocks,
// as many as its ~250 registers allow.  64-thread blocks, 8 per SM: a block
// ends -- and frees its place for the next -- when its two warps are done,
// not four (crash box 36.9 -> 36.7 us from a flushed L2, 38.9 -> 38.3 us per
// warm cycle, the same bits).
#ifndef RG_SHELL_MIXED_NT
#define RG_SHELL_MIXED_NT 64
#endif
#ifndef RG_SHELL_MIXED_MINB
#define RG_SHELL_MIXED_MINB 8
#endif
#ifndef RG_SHELL_F64_MINB
#define RG_SHELL_F64_MINB 1
#endif

// The mixed form stages each element's state in shared memory (cp.async at
// the start of the element, shell_element<..., STAGE>): the DRAM reads of the
// state overlap the node gathers and the geometry without holding registers.
template <typename ER, int NPT, int NT, int MF>
__global__ void __launch_bounds__(NT, sizeof(ER) == 4 ? RG_SHELL_MIXED_MINB : RG_SHELL_F64_MINB)
shell_kernel(const ShellParams P, const ShellArrays<ER> S, const NodeView N,
             typename SlotT<ER>::type *__restrict__ fsky,
             typename SlotT<ER>::type *__restrict__ fskyr, DtPartials dp,
             Time *__restrict__ T, int key0, int nc_total, int *__restrict__ status,
             const DtFinish F) {
  typedef ER R;
  constexpr bool STG = sizeof(ER) == 4;
  __shared__ __align__(16) float s_stg[STG ? ShellStage<NPT>::nfloat * NT : 1];
  __shared__ __align__(16) double s_stgd[STG ? ShellStage<NPT>::ndouble * NT : 1];
  R dtmine = (R)RG_EP06;
  int elmin = -1;
  // warp tasks of 32 consecutive elements.  wtasks = 0: each warp does the
  // one task of its own threads (element = block * NT + thread).  Otherwise
  // (FP64 groups of more than one wave) warps take tasks from a counter
  // until none is left: the FP64 kernel is bound by the FP64 pipe, and
  // dynamic tasks keep every SM's share equal even when plastic elements
  // cost more.  Results do not depend on which warp takes which task.
  const int lane = threadIdx.x & 31;
  int t = blockIdx.x * (NT / 32) + (int)(threadIdx.x >> 5);
  bool first = true;
  const double DT1 = T->dt2;
  const R dt1r = (R)DT1;
  const R dtinv = dt1r / smax(dt1r * dt1r, (R)RG_EM20);
  for (;;) {
    if (P.wtasks) {
      int g = 0;
      if (lane == 0) g = (int)atomicAdd(P.qctr, 1u);
      t = __shfl_sync(0xffffffffu, g, 0);
      if (t >= P.wtasks) break;
    } else {
      if (!first) break;
      first = false;
    }
    const int il = t * 32 + lane;
    if (il < P.nel)
      shell_element<ER, NPT, STG, MF, NT>(P, S, N, fsky, fskyr, T, key0, nc_total, il, dtmine,
                                          elmin, DT1, dtinv, s_stg, s_stgd, status);
  }
  block_dt_min<NT, R>(dtmine, elmin, dp.dt + P.part_off + blockIdx.x, dp.el + P.part_off + blockIdx.x);
  if (F.ctr) dt_finish_block<NT>(dp, F, P.part_off + blockIdx.x, T, status);
}

// Fixed-order shell energy sums, [0] internal (membrane + bending), [1]
// hourglass: SHE_BLOCKS block partials (thread t of block b takes elements
// b * 256 + t, then every SHE_BLOCKS * 256 further, in order; a fixed tree
// per block), then one block adds the partials the same way.
constexpr int SHE_BLOCKS = 152, SHE_NT = 256;
__global__ void __launch_bounds__(SHE_NT)
shell_energy_kernel(int nc, const double *__restrict__ eint, const double *__restrict__ ehou,
                    double *__restrict__ part) {
  __shared__ double sh[SHE_NT];
  double a = 0.0, b = 0.0;
  for (int i = blockIdx.x * SHE_NT + threadIdx.x; i < nc; i += SHE_BLOCKS * SHE_NT) {
    a += eint[i] + eint[nc + i];
    b += ehou[i];
  }
  a = block_sum_fixed<SHE_NT>(a, sh);
  b = block_sum_fixed<SHE_NT>(b, sh);
  if (threadIdx.x == 0) {
    part[blockIdx.x] = a;
    part[SHE_BLOCKS + blockIdx.x] = b;
  }
}

__global__ void __launch_bounds__(SHE_NT)
shell_energy_final(const double *__restrict__ part, double *__restrict__ out) {
  __shared__ double sh[SHE_NT];
  for (int j = 0; j < 2; j++) {
    const double v = (int)threadIdx.x < SHE_BLOCKS ? part[j * SHE_BLOCKS + threadIdx.x] : 0.0;
    const double s = block_sum_fixed<SHE_NT>(v, sh);
    if (threadIdx.x == 0) out[j] = s;
  }
}

constexpr int SHELL_NT = 128;
int shell_blocks(int nel) { return (nel + SHELL_NT - 1) / SHELL_NT; }
template <typename ER>
constexpr int shell_nt() { return sizeof(ER) == 4 ? RG_SHELL_MIXED_NT : SHELL_NT; }

template <typename ER>
static void launch_shell(const ShellParams &P, const ShellArrays<ER> &A, const NodeView &N,
                         void *fsky, void *fskyr, DtPartials dp, Time *T, int key0,
                         int nct, int *status, const DtFinish &F, cudaStream_t s) {
  typedef typename SlotT<ER>::type ST;
  const int nb = P.nblk;
  if (P.wtasks) cudaMemsetAsync(P.qctr, 0, sizeof(unsigned), s);
  ST *f = (ST *)fsky, *fr = (ST *)fskyr;
  constexpr int NTL = shell_nt<ER>();
  if (shell_mf(P) == 0) {
    switch (P.npt) {
      case 1: shell_kernel<ER, 1, NTL, 0><<<nb, NTL, 0, s>>>(P, A, N, f, fr, dp, T, key0, nct, status, F); break;
      case 2: shell_kernel<ER, 2, NTL, 0><<<nb, NTL, 0, s>>>(P, A, N, f, fr, dp, T, key0, nct, status, F); break;
      case 3: shell_kernel<ER, 3, NTL, 0><<<nb, NTL, 0, s>>>(P, A, N, f, fr, dp, T, key0, nct, status, F); break;
      case 4: shell_kernel<ER, 4, NTL, 0><<<nb, NTL, 0, s>>>(P, A, N, f, fr, dp, T, key0, nct, status, F); break;
      default: shell_kernel<ER, 5, NTL, 0><<<nb, NTL, 0, s>>>(P, A, N, f, fr, dp, T, key0, nct, status, F); break;
    }
  } else {
    constexpr int MF = SHELL_MF_ALL;
    switch (P.npt) {
      case 1: shell_kernel<ER, 1, NTL, MF><<<nb, NTL, 0, s>>>(P, A, N, f, fr, dp, T, key0, nct, status, F); break;
      case 2: shell_kernel<ER, 2, NTL, MF><<<nb, NTL, 0, s>>>(P, A, N, f, fr, dp, T, key0, nct, status, F); break;
      case 3: shell_kernel<ER, 3, NTL, MF><<<nb, NTL, 0, s>>>(P, A, N, f, fr, dp, T, key0, nct, status, F); break;
      case 4: shell_kernel<ER, 4, NTL, MF><<<nb, NTL, 0, s>>>(P, A, N, f, fr, dp, T, key0, nct, status, F); break;
      default: shell_kernel<ER, 5, NTL, MF><<<nb, NTL, 0, s>>>(P, A, N, f, fr, dp, T, key0, nct, status, F); break;
    }
  }
}

// ---------------------------------------------------------------------------
// host side
// ---------------------------------------------------------------------------
int shell_group_add(ShellModelHost &S, int numnod, int nel, const int *ixc, int npt,
                    const double *pm, const double *geo, const double *uparam,
                    const int *iparam, const double *thk0, int ismstr, int ithk,
                    std::string &why) {
  if (nel <= 0 || !ixc || !pm || !geo || !uparam || !iparam || !thk0) {
    why = "rg_shell_group_add: bad arguments";
    return RG_E_ARG;
  }
  if (npt < 1 || npt > 5) {
    why = "shell: NPT must be 1..5";
    return RG_E_UNSUP;
  }
  if (ismstr != 2 && ismstr != 4) {
    why = "shell: supported ISMSTR is 4 (2 accepted, run without the small-strain switch)";
    return RG_E_UNSUP;
  }
  if (ithk < 0) {
    why = "shell: ITHK must be 0 (initial thickness) or > 0 (current thickness)";
    return RG_E_UNSUP;
  }
  if (iparam[0] != 0) {
    why = "shell LAW2: Zerilli-Armstrong (IFORM = 1) not supported";
    return RG_E_UNSUP;
  }
  if (uparam[7] < 0.0 || uparam[7] > 1.0) {
    why = "shell LAW2: FISOKIN must be in [0, 1]";
    return RG_E_ARG;
  }
  // ductile rupture (SIGEPS02C: OFF = 4/5 once PLA >= EPMX, then the
  // layer-failure bookkeeping of MULAWC) is not built: a finite EPMX is
  // refused rather than ignored (the reader's default is 1e20, never reached)
  if (uparam[3] < 1e20) {
    why = "shell LAW2: ductile rupture (finite EPS_p_max) not supported";
    return RG_E_UNSUP;
  }
  for (int e = 0; e < nel; e++) {
    for (int k = 1; k <= 4; k++)
      if (ixc[7 * e + k] < 1 || ixc[7 * e + k] > numnod) {
        why = "IXC node number out of range";
        return RG_E_ARG;
      }
    if (!(thk0[e] > 0.0)) {
      why = "shell thickness must be > 0";
      return RG_E_ARG;
    }
  }
  auto *g = new ShellGroupHost();
  ShellParams &P = g->P;
  P.nft = S.numelc;
  P.nel = nel;
  P.npt = npt;
  P.ithk = ithk > 0 ? 1 : 0;
  P.ishfram = 0;  // set for every group at finalize (a model-wide option)
  P.ipla = (int)geo[38];
  if (P.ipla != 0 && P.ipla != 1 && P.ipla != 2) {
    delete g;
    why = "shell LAW2: Iplas 0, 1 or 2 supported";
    return RG_E_UNSUP;
  }
  P.rho = pm[0];
  P.young = pm[19];
  P.nu = pm[20];
  P.g = pm[21];
  P.a11 = pm[23];
  P.ssp = pm[26];
  P.h1 = geo[12];
  P.h2 = geo[13];
  P.h3 = geo[14];
  P.dm = geo[15];
  P.srh1 = geo[17];
  P.srh2 = geo[18];
  P.srh3 = geo[19];
  P.ish = std::nearbyint(geo[36]);
  P.fsh = geo[37];
  P.icc = iparam[1];
  P.vp = iparam[2];
  P.israte = iparam[3];
  P.ca = uparam[0];
  P.cb = uparam[1];
  P.cn = uparam[2];
  P.ymax = uparam[4];
  P.cc = uparam[5];
  P.eps0 = uparam[6];
  P.pm9 = uparam[8];
  P.fisokin = uparam[7];
  P.m_exp = uparam[9] != 0.0 ? uparam[9] : 1.0;
  // thermal parameters of the material (PM(69) rho*Cp, PM(79) T_r, PM(80)
  // T_melt; mat_param%therm): softening needs adiabatic heating
  P.rhocp = pm[68];
  P.tref = pm[78];
  P.tmelt = pm[79];
  P.thermal = (P.rhocp > 0.0 && P.tmelt > P.tref) ? 1 : 0;
  if (P.srh1 != 0.0 || P.srh2 != 0.0 || P.srh3 != 0.0) {
    delete g;
    why = "shell: linear hourglass viscosity (GEO(18..20)) not supported";
    return RG_E_UNSUP;
  }
  S.groups.push_back(g);
  S.ixc.insert(S.ixc.end(), ixc, ixc + 7 * (size_t)nel);
  S.thk0.insert(S.thk0.end(), thk0, thk0 + nel);
  S.numelc += nel;
  return (int)S.groups.size() - 1;
}

int shell_numelc(const ShellModelHost &S) { return S.numelc; }

const void *shell_device_arrays(const ShellModelHost &S, int prec) {
  if (!S.dev) return nullptr;
  const auto *D = (const ShellDev *)S.dev;
  return prec == RG_PREC_FP64 ? (const void *)&D->a64 : (const void *)&D->a32;
}
int shell_group_count(const ShellModelHost &S) { return (int)S.groups.size(); }
const ShellParams *shell_group_params(const ShellModelHost &S, int g) {
  return &S.groups[g]->P;
}
const int *shell_ixc(const ShellModelHost &S) { return S.ixc.data(); }
void shell_user_ids(const ShellModelHost &S, int *out) {
  // reversed: the dt kernel keeps the largest key on ties, CDT3 the first
  for (int e = 0; e < S.numelc; e++) out[S.numelc - 1 - e] = S.ixc[7 * e + 6];
}

template <typename ER>
static int alloc_arrays(ShellArrays<ER> &A, int nc, const DevAlloc &alloc, bool kin,
                        bool therm) {
  auto get = [&](void **p, size_t bytes) { return alloc(p, bytes); };
  int r = 0;
  A.nc = nc;
  A.sigbak = nullptr;
  A.temp = nullptr;
  if (kin && (r = get((void **)&A.sigbak, 15 * (size_t)nc * sizeof(ER)))) return r;
  if (therm && (r = get((void **)&A.temp, 5 * (size_t)nc * sizeof(ER)))) return r;
  if ((r = get((void **)&A.offg, nc * sizeof(ER)))) return r;
  if ((r = get((void **)&A.thke, nc * sizeof(ER)))) return r;
  if ((r = get((void **)&A.thk, nc * sizeof(double)))) return r;
  if ((r = get((void **)&A.forc, 5 * (size_t)nc * sizeof(ER)))) return r;
  if ((r = get((void **)&A.mom, 3 * (size_t)nc * sizeof(ER)))) return r;
  if ((r = get((void **)&A.hour, 5 * (size_t)nc * sizeof(ER)))) return r;
  if ((r = get((void **)&A.gstr, 8 * (size_t)nc * sizeof(ER)))) return r;
  if ((r = get((void **)&A.epsdg, nc * sizeof(ER)))) return r;
  if ((r = get((void **)&A.eint, 2 * (size_t)nc * sizeof(double)))) return r;
  if ((r = get((void **)&A.sig, 25 * (size_t)nc * sizeof(ER)))) return r;
  if ((r = get((void **)&A.pla, 5 * (size_t)nc * sizeof(ER)))) return r;
  if ((r = get((void **)&A.epsd, 5 * (size_t)nc * sizeof(ER)))) return r;
  if ((r = get((void **)&A.ehou, nc * sizeof(double)))) return r;
  return 0;
}

template <typename ER>
static int init_arrays(ShellModelHost &S, ShellArrays<ER> &A) {
  const int nc = S.numelc;
  std::vector<ER> one(nc, (ER)1), zero(25 * (size_t)nc, (ER)0), th(nc);
  std::vector<double> zd(2 * (size_t)nc, 0.0), thd(S.thk0.begin(), S.thk0.end());
  for (int e = 0; e < nc; e++) th[e] = (ER)S.thk0[e];
  auto cp = [](void *d, const void *h, size_t b) { return cudaMemcpy(d, h, b, cudaMemcpyHostToDevice); };
  if (cp(A.offg, one.data(), nc * sizeof(ER)) || cp(A.thke, th.data(), nc * sizeof(ER)) ||
      cp(A.thk, thd.data(), nc * sizeof(double)) ||
      cp(A.forc, zero.data(), 5 * (size_t)nc * sizeof(ER)) ||
      cp(A.mom, zero.data(), 3 * (size_t)nc * sizeof(ER)) ||
      cp(A.hour, zero.data(), 5 * (size_t)nc * sizeof(ER)) ||
      cp(A.gstr, zero.data(), 8 * (size_t)nc * sizeof(ER)) ||
      cp(A.epsdg, zero.data(), nc * sizeof(ER)) ||
      cp(A.eint, zd.data(), 2 * (size_t)nc * sizeof(double)) ||
      cp(A.sig, zero.data(), 25 * (size_t)nc * sizeof(ER)) ||
      cp(A.pla, zero.data(), 5 * (size_t)nc * sizeof(ER)) ||
      cp(A.epsd, zero.data(), 5 * (size_t)nc * sizeof(ER)) ||
      cp(A.ehou, zd.data(), nc * sizeof(double)))
    return RG_E_CUDA;
  if (A.sigbak) {
    std::vector<ER> z15(15 * (size_t)nc, (ER)0);
    if (cp(A.sigbak, z15.data(), z15.size() * sizeof(ER))) return RG_E_CUDA;
  }
  if (A.temp) {
    // each point starts at its material's T_r (the buffer's TINI)
    std::vector<ER> t(5 * (size_t)nc, (ER)0);
    for (auto *g : S.groups)
      for (int p = 0; p < 5; p++)
        for (int i = 0; i < g->P.nel; i++) t[(size_t)p * nc + g->P.nft + i] = (ER)g->P.tref;
    if (cp(A.temp, t.data(), t.size() * sizeof(ER))) return RG_E_CUDA;
  }
  return 0;
}

int shell_tile_count(const ShellModelHost &S) {
  int n = 0;
  for (auto *g : S.groups) n += shell_blocks(g->P.nel);
  return n;
}

// resident blocks per SM of the shell kernel for NPT points
template <typename ER>
static int shell_resident(int npt) {
  int r = 0;
  cudaError_t e;
  switch (npt) {
    case 1: e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&r, shell_kernel<ER, 1, SHELL_NT, 0>, SHELL_NT, 0); break;
    case 2: e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&r, shell_kernel<ER, 2, SHELL_NT, 0>, SHELL_NT, 0); break;
    case 3: e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&r, shell_kernel<ER, 3, SHELL_NT, 0>, SHELL_NT, 0); break;
    case 4: e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&r, shell_kernel<ER, 4, SHELL_NT, 0>, SHELL_NT, 0); break;
    default: e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&r, shell_kernel<ER, 5, SHELL_NT, 0>, SHELL_NT, 0); break;
  }
  return e == cudaSuccess && r > 0 ? r : 1;
}

int shell_finalize(ShellModelHost &S, int prec, const double *X, const int *iadc, int key0,
                   double dtfac, int &part_off, const DevAlloc &alloc, std::string &why) {
  (void)X;
  const int nc = S.numelc;
  if (nc == 0) return RG_OK;
  auto *D = new ShellDev();
  S.dev = D;
  D->prec = prec;
  std::vector<int> ix(4 * (size_t)nc), ia(4 * (size_t)nc), dg(nc);
  for (int e = 0; e < nc; e++) {
    for (int k = 0; k < 4; k++) {
      ix[(size_t)k * nc + e] = S.ixc[7 * e + 1 + k] - 1;
      ia[(size_t)k * nc + e] = iadc[4 * e + k] - 1;
    }
    dg[e] = S.ixc[7 * e + 3] == S.ixc[7 * e + 4] ? 1 : 0;
  }
  int r;
  if ((r = alloc((void **)&D->ix, ix.size() * sizeof(int)))) return r;
  if ((r = alloc((void **)&D->iadc, ia.size() * sizeof(int)))) return r;
  if ((r = alloc((void **)&D->degen, dg.size() * sizeof(int)))) return r;
  if ((r = alloc((void **)&D->epart, (2 * SHE_BLOCKS + 8) * sizeof(double)))) return r;
  if (cudaMemcpy(D->ix, ix.data(), ix.size() * sizeof(int), cudaMemcpyHostToDevice) ||
      cudaMemcpy(D->iadc, ia.data(), ia.size() * sizeof(int), cudaMemcpyHostToDevice) ||
      cudaMemcpy(D->degen, dg.data(), dg.size() * sizeof(int), cudaMemcpyHostToDevice)) {
    why = "copy of shell tables failed";
    return RG_E_CUDA;
  }
  bool kin = false, therm = false;
  for (auto *g : S.groups) {
    kin = kin || g->P.fisokin > 0.0;
    therm = therm || g->P.thermal;
  }
  if (prec == RG_PREC_FP64) {
    if ((r = alloc_arrays(D->a64, nc, alloc, kin, therm))) return r;
    D->a64.ix = D->ix;
    D->a64.iadc = D->iadc;
    D->a64.degen = D->degen;
    if ((r = init_arrays(S, D->a64))) return r;
  } else {
    if ((r = alloc_arrays(D->a32, nc, alloc, kin, therm))) return r;
    D->a32.ix = D->ix;
    D->a32.iadc = D->iadc;
    D->a32.degen = D->degen;
    if ((r = init_arrays(S, D->a32))) return r;
  }
  S.key0 = key0;
  for (auto *g : S.groups) {
    g->P.part_off = part_off;
    g->P.dtfac = dtfac;
    g->P.ishfram = S.ishfram;
    g->P.nodadt = S.nodadt;
    g->P.idtmin = S.idtmin;
    g->P.dtmin = S.dtmin;
    shell_params_mirror(g->P);
    // FP64 groups needing more than one wave of resident blocks: one wave
    // taking warp tasks from a counter (the mixed kernel, latency bound,
    // keeps one element per thread and the extra warps that hide latency)
    g->P.nblk = prec == RG_PREC_FP64 ? shell_blocks(g->P.nel)
                                     : (g->P.nel + RG_SHELL_MIXED_NT - 1) / RG_SHELL_MIXED_NT;
    g->P.wtasks = 0;
    if (prec == RG_PREC_FP64) {
      int dev = 0, nsm = 0;
      cudaGetDevice(&dev);
      cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
      const int wave = nsm * shell_resident<double>(g->P.npt);
      const int w = (g->P.nel + 31) / 32;
      if (nsm > 0 && w > wave * (SHELL_NT / 32)) {
        if ((r = alloc((void **)&g->P.qctr, sizeof(unsigned)))) return r;
        g->P.nblk = wave;
        g->P.wtasks = w;
      }
    }
    part_off += g->P.nblk;
  }
  return RG_OK;
}

void shell_enqueue(ShellModelHost &S, int prec, const NodeView &N, void *fsky, void *fskyr,
                   DtPartials dp, Time *T, int *status, const DtFinish &F, cudaStream_t s) {
  if (S.numelc == 0 || !S.dev) return;
  auto *D = (ShellDev *)S.dev;
  for (auto *g : S.groups) {
    if (prec == RG_PREC_FP64)
      launch_shell<double>(g->P, D->a64, N, fsky, fskyr, dp, T, S.key0, S.numelc, status, F, s);
    else
      launch_shell<float>(g->P, D->a32, N, fsky, fskyr, dp, T, S.key0, S.numelc, status, F, s);
  }
}

int shell_energy_enqueue(ShellModelHost &S, int prec, double *out2, cudaStream_t s) {
  if (S.numelc == 0 || !S.dev) return 0;
  auto *D = (ShellDev *)S.dev;
  const double *ei = prec == RG_PREC_FP64 ? D->a64.eint : D->a32.eint;
  const double *eh = prec == RG_PREC_FP64 ? D->a64.ehou : D->a32.ehou;
  shell_energy_kernel<<<SHE_BLOCKS, SHE_NT, 0, s>>>(S.numelc, ei, eh, D->epart);
  shell_energy_final<<<1, SHE_NT, 0, s>>>(D->epart, out2);
  return 2;
}

int shell_download(ShellModelHost &S, int prec, int which, double *out, std::string &why) {
  if (S.numelc == 0 || !S.dev) {
    why = "no shell groups";
    return RG_E_STATE;
  }
  auto *D = (ShellDev *)S.dev;
  const size_t n = S.numelc;
  const int npt = S.groups.empty() ? 0 : S.groups[0]->P.npt;
  auto fetch = [&](const void *src64, const void *src32, size_t cnt, bool isdouble) -> int {
    if (prec == RG_PREC_FP64 || isdouble) {
      return cudaMemcpy(out, prec == RG_PREC_FP64 ? src64 : src32, cnt * sizeof(double),
                        cudaMemcpyDeviceToHost) == cudaSuccess ? 0 : RG_E_CUDA;
    }
    std::vector<float> t(cnt);
    if (cudaMemcpy(t.data(), src32, cnt * sizeof(float), cudaMemcpyDeviceToHost) != cudaSuccess)
      return RG_E_CUDA;
    for (size_t i = 0; i < cnt; i++) out[i] = t[i];
    return 0;
  };
  const ShellArrays<double> &a = D->a64;
  const ShellArrays<float> &b = D->a32;
  switch (which) {
    case 0: return fetch(a.forc, b.forc, 5 * n, false);
    case 1: return fetch(a.mom, b.mom, 3 * n, false);
    case 2: return fetch(a.thk, b.thk, n, true);
    case 3: return fetch(a.eint, b.eint, 2 * n, true);
    case 4: return fetch(a.offg, b.offg, n, false);
    case 5: return fetch(a.sig, b.sig, 5 * (size_t)npt * n, false);
    case 6: return fetch(a.pla, b.pla, (size_t)npt * n, false);
    case 7: return fetch(a.hour, b.hour, 5 * n, false);
    case 8:  // back stress per point [npt][3][n] (zero without kinematic hardening)
      if (!(prec == RG_PREC_FP64 ? (const void *)a.sigbak : (const void *)b.sigbak)) {
        std::fill(out, out + 3 * (size_t)npt * n, 0.0);
        return 0;
      }
      return fetch(a.sigbak, b.sigbak, 3 * (size_t)npt * n, false);
    case 9:  // temperature per point [npt][n] (T_r without adiabatic heating)
      if (!(prec == RG_PREC_FP64 ? (const void *)a.temp : (const void *)b.temp)) {
        std::fill(out, out + (size_t)npt * n, S.groups[0]->P.tref);
        return 0;
      }
      return fetch(a.temp, b.temp, (size_t)npt * n, false);
  }
  why = "unknown shell state index";
  return RG_E_ARG;
}

void shell_free(ShellModelHost &S) {
  for (auto *g : S.groups) delete g;
  S.groups.clear();
  delete (ShellDev *)S.dev;
  S.dev = nullptr;
}

}  // namespace rg
