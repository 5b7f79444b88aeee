// Per-part element sums: the PARTSAV accumulation of SBILAN (one-point
// hexas, engine/source/elements/solid/solide/sbilan.F:118-160) and CBILAN
// (BT shells, engine/source/elements/shell/coque/cbilan.F:160-190), with the
// hourglass energy of CHVIS3 (chvis3.F:355-395) -- the quantities the
// engine writes per part to the time history (/TH/PART default variables,
// output/th/hist2.F:377-395):
//   0 IE    internal energy            hexa EINT * VOL, shell EINT(1) + EINT(2)
//   1 KE    element kinetic energy     hexa 1/2 XMAS <v^2>, shell XMAS sum v^2 / 8
//   2-4     momentum                   XMAS <v> (the nodes' mean velocity)
//   5 MASS  element mass               of the elements not switched off
//   6 HE    hourglass energy           accumulated since the start
// Element mass: hexa RHO * VNEW = RHO0 * VOL0 (SRHO3 conserves it); shell
// RHO * AREA * THK, with the element's area at the cycle's coordinates and
// its thickness after the cycle's update (the reference engine's part mass
// for the QA deck CRA2V44 follows exactly this, to its float32 digits).
//
// The sums are taken where the reference takes them: after the element pass
// of a cycle, before the nodal update -- coordinates X(n), velocities
// V(n-1/2), element energies and thickness of the cycle.  Each part's
// elements (in element order) are cut into chunks of PT_NT; one block sums a
// chunk with a fixed tree, one block per part then adds its chunks in order:
// the result depends on neither the launch nor the rest of the model.
#include "../../include/rg_api.h"
#include "rg_ctx.h"
#include "rg_shell_elem.cuh"

#include <algorithm>
#include <string>
#include <vector>

using namespace rg;

namespace {

constexpr int PT_NT = 256;
constexpr int NQ = RG_PART_NQ;

template <typename ER>
__global__ void __launch_bounds__(PT_NT)
hexa_parts_kernel(HexaArrays<ER> A, NodeView N, const int *__restrict__ perm,
                  const double *__restrict__ coef, const int4 *__restrict__ chunk,
                  double *__restrict__ partial) {
  __shared__ double sh[PT_NT];
  const int4 ch = chunk[blockIdx.x];
  double q[NQ] = {0, 0, 0, 0, 0, 0, 0};
  if ((int)threadIdx.x < ch.y) {
    const int j = ch.x + threadIdx.x;
    const int e = perm[j];
    double vx[8], vy[8], vz[8];
#pragma unroll
    for (int k = 0; k < 8; k++) {
      const dbl4 v = N.V4[A.nc[(size_t)k * A.ne + e]];
      vx[k] = v.x;
      vy[k] = v.y;
      vz[k] = v.z;
    }
    double sx = vx[0], sy = vy[0], sz = vz[0];
#pragma unroll
    for (int k = 1; k < 8; k++) {
      sx = sx + vx[k];
      sy = sy + vy[k];
      sz = sz + vz[k];
    }
    double va2 = vx[0] * vx[0];
#pragma unroll
    for (int k = 1; k < 8; k++) va2 = va2 + vx[k] * vx[k];
#pragma unroll
    for (int k = 0; k < 8; k++) va2 = va2 + vy[k] * vy[k];
#pragma unroll
    for (int k = 0; k < 8; k++) va2 = va2 + vz[k] * vz[k];
    sx = sx * RG_ONE_OVER_8;
    sy = sy * RG_ONE_OVER_8;
    sz = sz * RG_ONE_OVER_8;
    va2 = va2 * RG_ONE_OVER_8;
    const double vol = A.vol0[e];
    const double xmas = coef[j] * vol;
    q[0] = A.eint[e] * vol;
    q[1] = xmas * va2 * RG_HALF;
    q[2] = xmas * sx;
    q[3] = xmas * sy;
    q[4] = xmas * sz;
    q[5] = (double)A.off[e] >= RG_ONE ? xmas : 0.0;
    q[6] = A.ehou[e];
  }
#pragma unroll
  for (int k = 0; k < NQ; k++) {
    const double s = block_sum_fixed<PT_NT>(q[k], sh);
    if (threadIdx.x == 0) partial[(size_t)ch.z * NQ + k] = s;
  }
}

template <typename ER>
__global__ void __launch_bounds__(PT_NT)
shell_parts_kernel(ShellArrays<ER> S, NodeView N, const int *__restrict__ perm,
                   const double *__restrict__ coef, const int4 *__restrict__ chunk,
                   double *__restrict__ partial) {
  __shared__ double sh[PT_NT];
  const int4 ch = chunk[blockIdx.x];
  double q[NQ] = {0, 0, 0, 0, 0, 0, 0};
  if ((int)threadIdx.x < ch.y) {
    const int j = ch.x + threadIdx.x;
    const int e = perm[j];
    dbl4 x[4], v[4];
#pragma unroll
    for (int k = 0; k < 4; k++) {
      const int n = S.ix[(size_t)k * S.nc + e];
      x[k] = N.X4[n];
      v[k] = N.V4[n];
    }
    // area: half the norm of the diagonals' cross product
    const double ax = x[2].x - x[0].x, ay = x[2].y - x[0].y, az = x[2].z - x[0].z;
    const double bx = x[3].x - x[1].x, by = x[3].y - x[1].y, bz = x[3].z - x[1].z;
    const double cx = ay * bz - az * by, cy = az * bx - ax * bz, cz = ax * by - ay * bx;
    const double area = RG_HALF * sqrt(cx * cx + cy * cy + cz * cz);
    const double xmas = coef[j] * (area * S.thk[e]);
    const double vxa = v[0].x + v[1].x + v[2].x + v[3].x;
    const double vya = v[0].y + v[1].y + v[2].y + v[3].y;
    const double vza = v[0].z + v[1].z + v[2].z + v[3].z;
    const double va2 = v[0].x * v[0].x + v[1].x * v[1].x + v[2].x * v[2].x + v[3].x * v[3].x +
                       v[0].y * v[0].y + v[1].y * v[1].y + v[2].y * v[2].y + v[3].y * v[3].y +
                       v[0].z * v[0].z + v[1].z * v[1].z + v[2].z * v[2].z + v[3].z * v[3].z;
    const double xmas25 = xmas * RG_FOURTH;
    q[0] = S.eint[e] + S.eint[(size_t)S.nc + e];
    q[1] = xmas * va2 * RG_ONE_OVER_8;
    q[2] = xmas25 * vxa;
    q[3] = xmas25 * vya;
    q[4] = xmas25 * vza;
    q[5] = (double)S.offg[e] != 0.0 ? xmas : 0.0;
    q[6] = S.ehou[e];
  }
#pragma unroll
  for (int k = 0; k < NQ; k++) {
    const double s = block_sum_fixed<PT_NT>(q[k], sh);
    if (threadIdx.x == 0) partial[(size_t)ch.z * NQ + k] = s;
  }
}

// One block per part: its chunk partials in slot order (thread t takes
// slots t, t + PT_NT, ...), then a fixed tree.
__global__ void __launch_bounds__(PT_NT)
parts_final_kernel(const double *__restrict__ partial, const int *__restrict__ poff,
                   double *__restrict__ out) {
  __shared__ double sh[PT_NT];
  const int a = poff[blockIdx.x], b = poff[blockIdx.x + 1];
  for (int k = 0; k < NQ; k++) {
    double s = 0.0;
    for (int i = a + threadIdx.x; i < b; i += PT_NT) s += partial[(size_t)i * NQ + k];
    s = block_sum_fixed<PT_NT>(s, sh);
    if (threadIdx.x == 0) out[(size_t)blockIdx.x * NQ + k] = s;
  }
}

template <typename T>
int upload(T **d, const std::vector<T> &h) {
  const size_t bytes = std::max<size_t>(h.size(), 1) * sizeof(T);
  if (cudaMalloc((void **)d, bytes) != cudaSuccess) return RG_E_MEM;
  if (!h.empty() &&
      cudaMemcpy(*d, h.data(), h.size() * sizeof(T), cudaMemcpyHostToDevice) != cudaSuccess)
    return RG_E_CUDA;
  return RG_OK;
}

}  // namespace

namespace rg {

void parts_free(rg_ctx *c) {
  PartTables &t = c->pt;
  void *p[] = {t.hperm, t.sperm, t.hcoef, t.scoef, t.hchunk, t.schunk, t.poff, t.partial, t.out};
  for (void *q : p)
    if (q) cudaFree(q);
  t = PartTables{};
  c->parts_ready = false;
  c->parts_valid = false;
}

// Element -> part maps (given, or one part per element group: hexa groups
// first, then shell groups), chunk tables and buffers on the device.
int parts_prepare(rg_ctx *c) {
  if (c->parts_ready) return RG_OK;
  const int numels = c->numels, numelc = shell_numelc(c->shells);
  const int nsg = shell_group_count(c->shells);
  std::vector<int> ph = c->part_hexa, ps = c->part_shell;
  int npart = c->npart;
  std::vector<double> rho_h(numels), rho_s(numelc);
  for (size_t g = 0; g < c->hg.size(); g++)
    for (int i = 0; i < c->hg[g].nel; i++) rho_h[c->hg[g].P.nft + i] = c->hg[g].P.rho0;
  for (int g = 0; g < nsg; g++) {
    const ShellParams *P = shell_group_params(c->shells, g);
    for (int i = 0; i < P->nel; i++) rho_s[P->nft + i] = P->rho;
  }
  if (ph.empty() && ps.empty()) {
    npart = (int)c->hg.size() + nsg;
    ph.resize(numels);
    ps.resize(numelc);
    for (size_t g = 0; g < c->hg.size(); g++)
      for (int i = 0; i < c->hg[g].nel; i++) ph[c->hg[g].P.nft + i] = (int)g;
    for (int g = 0; g < nsg; g++) {
      const ShellParams *P = shell_group_params(c->shells, g);
      for (int i = 0; i < P->nel; i++) ps[P->nft + i] = (int)c->hg.size() + g;
    }
  }
  std::vector<std::vector<int>> lh(npart), ls(npart);
  for (int e = 0; e < numels; e++) lh[ph[e]].push_back(e);
  for (int e = 0; e < numelc; e++) ls[ps[e]].push_back(e);
  std::vector<int> hperm, sperm, poff(npart + 1, 0);
  std::vector<double> hcoef, scoef;
  std::vector<int4> hchunk, schunk;
  int slot = 0;
  for (int p = 0; p < npart; p++) {
    poff[p] = slot;
    for (size_t a = 0; a < lh[p].size(); a += PT_NT) {
      const int cnt = (int)std::min<size_t>(PT_NT, lh[p].size() - a);
      hchunk.push_back(make_int4((int)hperm.size(), cnt, slot++, p));
      for (int i = 0; i < cnt; i++) {
        hperm.push_back(lh[p][a + i]);
        hcoef.push_back(rho_h[lh[p][a + i]]);
      }
    }
    for (size_t a = 0; a < ls[p].size(); a += PT_NT) {
      const int cnt = (int)std::min<size_t>(PT_NT, ls[p].size() - a);
      schunk.push_back(make_int4((int)sperm.size(), cnt, slot++, p));
      for (int i = 0; i < cnt; i++) {
        sperm.push_back(ls[p][a + i]);
        scoef.push_back(rho_s[ls[p][a + i]]);
      }
    }
  }
  poff[npart] = slot;
  cudaSetDevice(c->device);
  PartTables &t = c->pt;
  int r;
  if ((r = upload(&t.hperm, hperm)) || (r = upload(&t.sperm, sperm)) ||
      (r = upload(&t.hcoef, hcoef)) || (r = upload(&t.scoef, scoef)) ||
      (r = upload(&t.hchunk, hchunk)) || (r = upload(&t.schunk, schunk)) ||
      (r = upload(&t.poff, poff))) {
    parts_free(c);
    c->err = "per-part tables: device allocation or copy failed";
    return r;
  }
  if (cudaMalloc((void **)&t.partial, std::max(slot, 1) * (size_t)NQ * sizeof(double)) !=
          cudaSuccess ||
      cudaMalloc((void **)&t.out, std::max(npart, 1) * (size_t)NQ * sizeof(double)) !=
          cudaSuccess) {
    parts_free(c);
    c->err = "per-part buffers: cudaMalloc failed";
    return RG_E_MEM;
  }
  cudaMemset(t.out, 0, std::max(npart, 1) * (size_t)NQ * sizeof(double));
  t.nh_chunks = (int)hchunk.size();
  t.ns_chunks = (int)schunk.size();
  t.nslots = slot;
  t.npart = npart;
  c->parts_ready = true;
  return RG_OK;
}

// The sums of the element pass just enqueued on the context stream.
void parts_enqueue(rg_ctx *c) {
  const PartTables &t = c->pt;
  cudaStream_t s = c->stream;
  if (t.nh_chunks) {
    if (c->prec == RG_PREC_FP64)
      hexa_parts_kernel<double><<<t.nh_chunks, PT_NT, 0, s>>>(c->h64, c->nv, t.hperm, t.hcoef,
                                                              t.hchunk, t.partial);
    else
      hexa_parts_kernel<float><<<t.nh_chunks, PT_NT, 0, s>>>(c->h32, c->nv, t.hperm, t.hcoef,
                                                             t.hchunk, t.partial);
  }
  if (t.ns_chunks) {
    const void *sa = shell_device_arrays(c->shells, c->prec);
    if (c->prec == RG_PREC_FP64)
      shell_parts_kernel<double><<<t.ns_chunks, PT_NT, 0, s>>>(
          *(const ShellArrays<double> *)sa, c->nv, t.sperm, t.scoef, t.schunk, t.partial);
    else
      shell_parts_kernel<float><<<t.ns_chunks, PT_NT, 0, s>>>(
          *(const ShellArrays<float> *)sa, c->nv, t.sperm, t.scoef, t.schunk, t.partial);
  }
  if (t.npart) parts_final_kernel<<<t.npart, PT_NT, 0, s>>>(t.partial, t.poff, t.out);
}

}  // namespace rg

extern "C" {

int rg_set_parts(rg_ctx *c, int npart, const int *hexa_part, const int *shell_part) {
  if (!c) return RG_E_ARG;
  if (!c->finalized) {
    c->err = "rg_set_parts: rg_finalize first (the element counts are final then)";
    return RG_E_STATE;
  }
  const int numels = c->numels, numelc = shell_numelc(c->shells);
  if (npart <= 0 || (numels && !hexa_part) || (numelc && !shell_part)) {
    c->err = "rg_set_parts: npart > 0 and a part for every element are required";
    return RG_E_ARG;
  }
  for (int e = 0; e < numels; e++)
    if (hexa_part[e] < 0 || hexa_part[e] >= npart) {
      c->err = "rg_set_parts: hexa part number out of range";
      return RG_E_ARG;
    }
  for (int e = 0; e < numelc; e++)
    if (shell_part[e] < 0 || shell_part[e] >= npart) {
      c->err = "rg_set_parts: shell part number out of range";
      return RG_E_ARG;
    }
  cudaSetDevice(c->device);
  cudaStreamSynchronize(c->stream);
  parts_free(c);
  c->npart = npart;
  c->part_hexa.assign(hexa_part, hexa_part + numels);
  c->part_shell.assign(shell_part, shell_part + numelc);
  if (c->parts_due) {
    // the captured graph holds the old tables: take it again on demand
    c->parts_due = false;
  }
  if (c->gexec_parts) cudaGraphExecDestroy(c->gexec_parts);
  if (c->graph_parts) cudaGraphDestroy(c->graph_parts);
  c->gexec_parts = nullptr;
  c->graph_parts = nullptr;
  return RG_OK;
}

int rg_part_count(rg_ctx *c, int *npart) {
  if (!c || !npart) return RG_E_ARG;
  if (!c->finalized) {
    c->err = "rg_part_count: rg_finalize first";
    return RG_E_STATE;
  }
  *npart = c->part_hexa.empty() && c->part_shell.empty()
               ? (int)c->hg.size() + shell_group_count(c->shells)
               : c->npart;
  return RG_OK;
}

int rg_part_sums(rg_ctx *c, double *out, int npart) {
  if (!c || !out) return RG_E_ARG;
  if (!c->parts_valid) {
    c->err = "rg_part_sums: no cycle has taken the part sums since rg_part_sums_due";
    return RG_E_STATE;
  }
  if (npart != c->pt.npart) {
    c->err = "rg_part_sums: npart differs from the context's part count";
    return RG_E_ARG;
  }
  cudaSetDevice(c->device);
  if (cudaMemcpyAsync(out, c->pt.out, (size_t)npart * NQ * sizeof(double),
                      cudaMemcpyDeviceToHost, c->stream) != cudaSuccess ||
      cudaStreamSynchronize(c->stream) != cudaSuccess) {
    c->err = "rg_part_sums: copy failed";
    return RG_E_CUDA;
  }
  return RG_OK;
}

}  // extern "C"
