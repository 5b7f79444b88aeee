// C-ABI implementation: context, device memory, PARITH/ON tables, the
// per-cycle launch sequence (captured in a CUDA graph), the node kernel
// (ASSPAR4 + ACCELE + BCS + rigid wall + VELOCITY + DEPLA), the time-step
// kernel (RESOL dt logic) and fixed-order energy reductions.
#include "../../include/rg_api.h"
#include "rg_device.cuh"
#include "rg_kernels.h"
#include "rg_node.cuh"
#include "rg_shell.h"
#include "rg_ctx.h"

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdint>
#include <cstring>
#include <numeric>
#include <string>
#include <type_traits>
#include <vector>

using namespace rg;

namespace {

// Node kernels: 64-thread blocks.  The node update is bound by the FP64
// pipe (FP64 form) or by conversions on it (mixed form), so its time per SM
// is the number of blocks placed there; a model of 120k nodes in 256-thread
// blocks put 4 blocks on some SMs and 3 on the rest (64: 0.0286 -> 0.0245 ms
// FP64, 0.0183 -> 0.0163 ms mixed).  At least DT_GROUP threads (nodal dt).
constexpr int NODE_NT = 64;
constexpr int LINK_NT = 128;
constexpr int DT_NT = 1024;
constexpr int EN_BLOCKS = 304;  // 2 x 152 SMs, fixed: reductions are order-fixed
constexpr int EN_NT = 256;

}  // namespace

namespace {

int fail(rg_ctx *c, int code, const std::string &msg) {
  if (c) c->err = msg;
  return code;
}

#define RG_CUDA(c, call)                                                      \
  do {                                                                        \
    cudaError_t _e = (call);                                                  \
    if (_e != cudaSuccess)                                                    \
      return fail((c), RG_E_CUDA,                                             \
                  std::string(#call) + ": " + cudaGetErrorString(_e));        \
  } while (0)

template <typename T>
int dalloc(rg_ctx *c, T **p, size_t n) {
  size_t bytes = std::max<size_t>(n, 1) * sizeof(T);
  cudaError_t e = cudaMalloc((void **)p, bytes);
  if (e != cudaSuccess)
    return fail(c, RG_E_MEM, std::string("cudaMalloc: ") + cudaGetErrorString(e));
  c->allocs.push_back((void *)*p);
  c->alloc_bytes.push_back(bytes);
  c->dev_bytes += bytes;
  return RG_OK;
}

// Node kernels: one thread per node (node_update in rg_node.cuh); LINK:
// the model has rigid links; the link-free variants are the hot path.
// RG_NODE_MINB: resident 64-thread blocks per SM the register budget is cut
// for.  14 (72 registers) puts a 120k-node model's 1882 blocks in one wave
// of 152 SMs (80 registers allowed 12 blocks per SM, two waves): mixed node
// kernel 15.4 -> 14.3 us on the crash box, FP64 and the 2.1M-node block
// unchanged or faster; 16 (64 registers, spills) is no better.
#ifndef RG_NODE_MINB
#define RG_NODE_MINB 14
#endif
template <bool F64, bool LINK>
__global__ void __launch_bounds__(NODE_NT, RG_NODE_MINB)
node_kernel(NodeView N, const int *__restrict__ adsky, const void *__restrict__ fsky_,
            const void *__restrict__ fskyr_, const Time *__restrict__ T,
            const int *__restrict__ wall, const double *__restrict__ walls,
            const dbl4 *__restrict__ lacc, int *__restrict__ status) {
  const int n = blockIdx.x * NODE_NT + threadIdx.x;
  if (n >= N.numnod) return;
  node_update<F64, false, false, LINK>(N, adsky, fsky_, fskyr_, T, wall, walls, lacc, status, n);
}

template <bool F64, bool LINK>
__global__ void __launch_bounds__(NODE_NT, RG_NODE_MINB)
node_kernel_rot(NodeView N, const int *__restrict__ adsky, const void *__restrict__ fsky_,
                const void *__restrict__ fskyr_, const Time *__restrict__ T,
                const int *__restrict__ wall, const double *__restrict__ walls,
                const dbl4 *__restrict__ lacc, int *__restrict__ status) {
  const int n = blockIdx.x * NODE_NT + threadIdx.x;
  if (n >= N.numnod) return;
  node_update<F64, true, false, LINK>(N, adsky, fsky_, fskyr_, T, wall, walls, lacc, status, n);
}

// Nodal time step, DTNODA (time_step/dtnoda.F:213-345, 443-470), NODADT > 0:
// node n's step DTFAC1(11)*SQRT(2*MS/STIFN) and, for shell models,
// DTFAC1(11)*SQRT(2*IN/STIFR), STIFN / STIFR the fixed-order sums of the
// element stiffness slots (ASSPAR4).  A node with non-positive stiffness
// raises RG_ST_NODSTIF (the reference stops).  Order keys: on ties the first
// node of the translational pass wins, then the first of the rotational
// pass (the strict '<' scans of DTNODA).  The block minima are reduced by
// the last block, which applies the RESOL dt logic.
template <bool F64, bool ROT>
__global__ void __launch_bounds__(NODE_NT)
nodal_dt_kernel(NodeView N, const int *__restrict__ adsky, const void *__restrict__ fsky_,
                const void *__restrict__ fskyr_, const double dtfac, const double dtmin,
                const int idtmin, DtPartials dp, Time *__restrict__ T,
                int *__restrict__ status, const DtFinish F) {
  const int n = blockIdx.x * NODE_NT + threadIdx.x;
  const int numnod = N.numnod;
  double d = RG_EP06;
  int k = -1;
  if (n < numnod) {
    double st = 0.0, sr = 0.0;
    const int k0 = adsky[n], k1 = adsky[n + 1];
    for (int q = k0; q < k1; q++) {
      if constexpr (F64) {
        st = __dadd_rn(st, ((const dbl4 *)fsky_)[q].w);
        if (ROT) sr = __dadd_rn(sr, ((const dbl4 *)fskyr_)[q].w);
      } else {
        st = __dadd_rn(st, (double)__ldg(&((const float4 *)fsky_)[q].w));
        if (ROT) sr = __dadd_rn(sr, (double)__ldg(&((const float4 *)fskyr_)[q].w));
      }
    }
    const double ms = N.D4[n].w;
    // IDTMIN(11) = 3 / 8 (dtnoda.F:268-305, 466-500): a node whose step is
    // below DTMIN1(11) takes the mass (inertia) of a step DTMIN1(11):
    // 1/2 STIFN (DTMIN1/DTFAC1)^2 * 1.00001, used by this cycle's ACCELE;
    // the step of this cycle stays the one computed before the scaling.
    // 0, 1, 5: the step below DTMIN1(11) raises RG_ST_DTMIN (1, 5: stop).
    const bool scale = idtmin == 3 || idtmin == 8;
    if (st <= 0.0) {
      atomicOr(status, RG_ST_NODSTIF);
    } else if (ms > 0.0) {
      const double dn = __dmul_rn(dtfac, sqrt(__dmul_rn(2.0, ms) / st));
      if (dn < dtmin) {
        if (scale) {
          const double dt2p = dtmin / dtfac;
          const double mas = __dmul_rn(__dmul_rn(__dmul_rn(__dmul_rn(RG_HALF, st), dt2p), dt2p),
                                       RG_ONEP00001);
          N.D4[n].w = mas;
          N.X4[n].w = 1.0 / mas;
          if (!F64) N.XF[n].pad0 = (float)(1.0 / mas);
        } else {
          atomicOr(status, RG_ST_DTMIN);
        }
      }
      dt_pair_min(d, k, dn, 2 * numnod - 1 - n);
    }
    if (ROT) {
      const double in = N.DR4[n].w;
      if (sr <= 0.0) {
        atomicOr(status, RG_ST_NODSTIF);
      } else if (in > 0.0) {
        const double dn = __dmul_rn(dtfac, sqrt(__dmul_rn(2.0, in) / sr));
        if (dn < dtmin) {
          if (scale) {
            const double dt2p = dtmin / dtfac;
            const double iner = __dmul_rn(
                __dmul_rn(__dmul_rn(__dmul_rn(RG_HALF, sr), dt2p), dt2p), RG_ONEP00001);
            const double in2 = fmax(iner, in);
            N.DR4[n].w = in2;
            N.VR4[n].w = 1.0 / in2;
            if (!F64) N.XF[n].pad1 = (float)(1.0 / in2);
          } else {
            atomicOr(status, RG_ST_DTMIN);
          }
        }
        dt_pair_min(d, k, dn, numnod - 1 - n);
      }
    }
  }
  block_dt_min<NODE_NT, double>(d, k, dp.dt + blockIdx.x, dp.el + blockIdx.x);
  dt_finish_block<NODE_NT>(dp, F, blockIdx.x, T, status);
}

// Rigid links, RLINK1 (constraints/general/rlink/rlink1.F) as called by
// RLINK10 after the boundary conditions: block l forms link l's mass (and
// inertia) and the mass- (inertia-) weighted sums of its nodes'
// accelerations -- each node's acceleration computed as the node kernel
// computes it (ASSPAR4 sums, ACCELE, BCS) -- in a fixed order (strided
// per-thread sums, then a fixed tree), and writes the common accelerations
// (AX/MASS ...) that the node kernel gives the linked directions.  An
// inactive link, or one of zero mass, writes direction bits 0 (no effect).
template <bool F64, bool ROT>
__global__ void __launch_bounds__(LINK_NT)
rlink_kernel(NodeView N, const int *__restrict__ adsky, const void *__restrict__ fsky_,
             const void *__restrict__ fskyr_, const int *__restrict__ lnodes,
             const int *__restrict__ loff, const int4 *__restrict__ lic,
             dbl4 *__restrict__ lacc, int *__restrict__ status) {
  const int l = blockIdx.x;
  double s[8] = {0, 0, 0, 0, 0, 0, 0, 0};
  for (int i = loff[l] + threadIdx.x; i < loff[l + 1]; i += LINK_NT) {
    const int n = lnodes[i];
    double a0, a1, a2, r0, r1, r2;
    node_assemble<F64, ROT, false>(adsky, fsky_, fskyr_, status, n, a0, a1, a2, r0, r1, r2);
    const dbl4 x = N.X4[n];
    const int code = (int)N.V4[n].w;
    const double ms = N.D4[n].w;
    a0 = __dmul_rn(a0, x.w);
    a1 = __dmul_rn(a1, x.w);
    a2 = __dmul_rn(a2, x.w);
    if (code & 1) a0 = 0.0;
    if (code & 2) a1 = 0.0;
    if (code & 4) a2 = 0.0;
    s[0] = __dadd_rn(s[0], ms);
    s[1] = __dadd_rn(s[1], __dmul_rn(ms, a0));
    s[2] = __dadd_rn(s[2], __dmul_rn(ms, a1));
    s[3] = __dadd_rn(s[3], __dmul_rn(ms, a2));
    if (ROT) {
      const double rin = N.VR4[n].w, in = N.DR4[n].w;
      r0 = __dmul_rn(r0, rin);
      r1 = __dmul_rn(r1, rin);
      r2 = __dmul_rn(r2, rin);
      if (code & 8) r0 = 0.0;
      if (code & 16) r1 = 0.0;
      if (code & 32) r2 = 0.0;
      s[4] = __dadd_rn(s[4], in);
      s[5] = __dadd_rn(s[5], __dmul_rn(in, r0));
      s[6] = __dadd_rn(s[6], __dmul_rn(in, r1));
      s[7] = __dadd_rn(s[7], __dmul_rn(in, r2));
    }
  }
  __shared__ double sh[8][LINK_NT];
  for (int j = 0; j < 8; j++) sh[j][threadIdx.x] = s[j];
  __syncthreads();
  for (int o = LINK_NT / 2; o > 0; o >>= 1) {
    if (threadIdx.x < o)
      for (int j = 0; j < 8; j++) sh[j][threadIdx.x] = __dadd_rn(sh[j][threadIdx.x], sh[j][threadIdx.x + o]);
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    const int4 c = lic[l];
    dbl4 t = mk4(0, 0, 0, 0), u = mk4(0, 0, 0, 0);
    const double mass = sh[0][0], iner = sh[4][0];
    if (c.z && c.x && mass != 0.0)
      t = mk4(sh[1][0] / mass, sh[2][0] / mass, sh[3][0] / mass, (double)c.x);
    if (ROT && c.z && c.y && iner != 0.0)
      u = mk4(sh[5][0] / iner, sh[6][0] / iner, sh[7][0] / iner, (double)c.y);
    lacc[2 * l] = t;
    lacc[2 * l + 1] = u;
  }
}

// Mixed form: refresh the FP32 copies from the FP64 node records (after a
// host upload).
__global__ void refresh_copies_kernel(NodeView N, int rot) {
  const int n = blockIdx.x * NODE_NT + threadIdx.x;
  if (n >= N.numnod) return;
  const dbl4 x = N.X4[n], v = N.V4[n];
  F8 c = split_hilo(x.x, x.y, x.z);
  c.pad0 = __double2float_rn(x.w);                       // 1/MS
  c.pad1 = rot ? __double2float_rn(N.VR4[n].w) : 0.f;    // 1/IN
  N.XF[n] = c;
  N.VF[n] = make_float4(__double2float_rn(v.x), __double2float_rn(v.y), __double2float_rn(v.z), 0.f);
  if (rot) {
    const dbl4 w = N.VR4[n];
    N.VRF[n] = make_float4(__double2float_rn(w.x), __double2float_rn(w.y), __double2float_rn(w.z), 0.f);
  }
}

// Assembled forces only (ASSPAR4 sums), written to F(3,n), STIFN(n),
// FR(3,n), STIFR(n) -- registered host memory or the staging buffer; any
// output may be null.
template <typename ST, bool ROT>
__global__ void assemble_kernel(int numnod, const int *__restrict__ adsky,
                                const ST *__restrict__ fsky,
                                const ST *__restrict__ fskyr, double *__restrict__ f,
                                double *__restrict__ stifn, double *__restrict__ fr,
                                double *__restrict__ stifr) {
  const int n = blockIdx.x * NODE_NT + threadIdx.x;
  if (n >= numnod) return;
  double a0 = 0.0, a1 = 0.0, a2 = 0.0, st = 0.0;
  double r0 = 0.0, r1 = 0.0, r2 = 0.0, sr = 0.0;
  for (int k = adsky[n]; k < adsky[n + 1]; k++) {
    const ST q = fsky[k];
    a0 = __dadd_rn(a0, (double)q.x);
    a1 = __dadd_rn(a1, (double)q.y);
    a2 = __dadd_rn(a2, (double)q.z);
    st = __dadd_rn(st, (double)q.w);
    if (ROT) {
      const ST g = fskyr[k];
      r0 = __dadd_rn(r0, (double)g.x);
      r1 = __dadd_rn(r1, (double)g.y);
      r2 = __dadd_rn(r2, (double)g.z);
      sr = __dadd_rn(sr, (double)g.w);
    }
  }
  if (f) {
    f[3 * n] = a0;
    f[3 * n + 1] = a1;
    f[3 * n + 2] = a2;
  }
  if (stifn) stifn[n] = st;
  if (ROT) {
    if (fr) {
      fr[3 * n] = r0;
      fr[3 * n + 1] = r1;
      fr[3 * n + 2] = r2;
    }
    if (stifr) stifr[n] = sr;
  }
}

// Time-step kernel: fixed-order reduction of the per-block element minima
// by one block, then the RESOL logic (dt_apply in rg_node.cuh).
__global__ void __launch_bounds__(DT_NT)
dt_kernel(DtPartials dp, int nparts, const int *__restrict__ ngl,
          Time *__restrict__ T, int *__restrict__ status, int advance) {
  double d = RG_EP06;
  int k = -1;
  for (int i = threadIdx.x; i < nparts; i += DT_NT) {
    const int ki = dp.el[i];
    if (ki >= 0) dt_pair_min(d, k, dp.dt[i], ki);
  }
  __shared__ double od;
  __shared__ int ok;
  block_dt_min<DT_NT>(d, k, &od, &ok);
  __syncthreads();
  if (threadIdx.x == 0) dt_apply(T, od, ok, ngl, status, advance);
}

// Fixed-order energy partials: [0] element internal (EINT * VOL0),
// [1] hourglass, [2] translational kinetic, [3] rotational kinetic.
template <typename ER>
__global__ void __launch_bounds__(EN_NT)
energy_kernel(int ne, const double *__restrict__ eint,
              const double *__restrict__ vol0, const double *__restrict__ ehou,
              NodeView N, int rot, double *__restrict__ part) {
  double s[4] = {0, 0, 0, 0};
  const int stride = EN_BLOCKS * EN_NT;
  for (int i = blockIdx.x * EN_NT + threadIdx.x; i < ne; i += stride) {
    s[0] += eint[i] * vol0[i];
    s[1] += ehou[i];
  }
  for (int i = blockIdx.x * EN_NT + threadIdx.x; i < N.numnod; i += stride) {
    const dbl4 m = N.D4[i], v = N.V4[i];
    s[2] += 0.5 * m.w * (v.x * v.x + v.y * v.y + v.z * v.z);
    if (rot) {
      const dbl4 w = N.VR4[i], in = N.DR4[i];
      s[3] += 0.5 * in.w * (w.x * w.x + w.y * w.y + w.z * w.z);
    }
  }
  __shared__ double sh[4][EN_NT];
  for (int j = 0; j < 4; j++) sh[j][threadIdx.x] = s[j];
  __syncthreads();
  for (int o = EN_NT / 2; o > 0; o >>= 1) {
    if (threadIdx.x < o)
      for (int j = 0; j < 4; j++) sh[j][threadIdx.x] += sh[j][threadIdx.x + o];
    __syncthreads();
  }
  if (threadIdx.x == 0)
    for (int j = 0; j < 4; j++) part[j * EN_BLOCKS + blockIdx.x] = sh[j][0];
}

// Fixed-order sum of the NJ rows of EN_BLOCKS partials: thread t takes
// partials t, t + EN_NT, ... in order, then a fixed tree (one block).
template <int NJ>
__device__ __forceinline__ void partials_final(const double *__restrict__ part,
                                               double *__restrict__ out) {
  __shared__ double sh[EN_NT];
  for (int j = 0; j < NJ; j++) {
    double s = 0.0;
    for (int b = threadIdx.x; b < EN_BLOCKS; b += EN_NT) s += part[j * EN_BLOCKS + b];
    s = block_sum_fixed<EN_NT>(s, sh);
    if (threadIdx.x == 0) out[j] = s;
  }
}

__global__ void __launch_bounds__(EN_NT)
energy_final(const double *__restrict__ part, int nextra, const double *__restrict__ extra,
             double *__restrict__ out) {
  partials_final<4>(part, out);
  if (threadIdx.x == 0)
    for (int j = 0; j < nextra; j++) out[j] += extra[j];
}

// Node sums of the energy balance, fixed order like energy_kernel: mass,
// momentum (x, y, z) and the rigid walls' external work.
__global__ void __launch_bounds__(EN_NT)
balance_kernel(NodeView N, double *__restrict__ part) {
  double s[5] = {0, 0, 0, 0, 0};
  const int stride = EN_BLOCKS * EN_NT;
  for (int i = blockIdx.x * EN_NT + threadIdx.x; i < N.numnod; i += stride) {
    const double m = N.D4[i].w;
    const dbl4 v = N.V4[i];
    s[0] += m;
    s[1] += m * v.x;
    s[2] += m * v.y;
    s[3] += m * v.z;
    if (N.wext) s[4] += N.wext[i];
  }
  __shared__ double sh[5][EN_NT];
  for (int j = 0; j < 5; j++) sh[j][threadIdx.x] = s[j];
  __syncthreads();
  for (int o = EN_NT / 2; o > 0; o >>= 1) {
    if (threadIdx.x < o)
      for (int j = 0; j < 5; j++) sh[j][threadIdx.x] += sh[j][threadIdx.x + o];
    __syncthreads();
  }
  if (threadIdx.x == 0)
    for (int j = 0; j < 5; j++) part[j * EN_BLOCKS + blockIdx.x] = sh[j][0];
}

__global__ void __launch_bounds__(EN_NT)
balance_final(const double *__restrict__ part, double *__restrict__ out) {
  partials_final<5>(part, out);
}

// AoS X(3,n) -> X4.xyz (keeps .w); same for V and VR.
// FORINT-level upload: X, V and (shell models) VR, xyz interleaved, read
// straight from registered host memory (or from the staging buffer) into the
// node records, and the mixed form's FP32 copies refreshed in the same pass.
__global__ void upload_nodes_kernel(NodeView N, const double *__restrict__ x,
                                    const double *__restrict__ v,
                                    const double *__restrict__ vr, int mixed,
                                    Time *__restrict__ T, double dt1) {
  const int i = blockIdx.x * NODE_NT + threadIdx.x;
  // DT1 of a FORINT-level call (the element kernels read Time::dt2); a
  // whole-cycle upload passes dt1 < 0 and keeps the device's time step
  if (i == 0 && dt1 >= 0.0) T->dt2 = dt1;
  if (i >= N.numnod) return;
  dbl4 a = N.X4[i], b = N.V4[i];
  a.x = x[3 * i];
  a.y = x[3 * i + 1];
  a.z = x[3 * i + 2];
  b.x = v[3 * i];
  b.y = v[3 * i + 1];
  b.z = v[3 * i + 2];
  N.X4[i] = a;
  N.V4[i] = b;
  if (mixed) {
    F8 c = split_hilo(a.x, a.y, a.z);
    c.pad0 = __double2float_rn(a.w);                             // 1/MS
    c.pad1 = N.VR4 ? __double2float_rn(N.VR4[i].w) : 0.f;        // 1/IN
    N.XF[i] = c;
    N.VF[i] = make_float4(__double2float_rn(b.x), __double2float_rn(b.y),
                          __double2float_rn(b.z), 0.f);
  }
  if (vr) {
    dbl4 w = N.VR4[i];
    w.x = vr[3 * i];
    w.y = vr[3 * i + 1];
    w.z = vr[3 * i + 2];
    N.VR4[i] = w;
    if (mixed)
      N.VRF[i] = make_float4(__double2float_rn(w.x), __double2float_rn(w.y),
                             __double2float_rn(w.z), 0.f);
  }
}

// Host-link writes with 16-byte stores: a block gathers XFER_NT nodes' xyz
// triples from their records into shared memory and writes them to the AoS
// array X(3, n) as contiguous double2 chunks (a warp writes 512 contiguous
// bytes per instruction; the per-node stores of unpack3_kernel touch each
// line three times).  The AoS pointers must be 16-byte aligned (the block's
// first triple then is too: 256 nodes are 6144 bytes).  Measured on the
// crash box's 120k nodes: the four outputs of rg_cycle_host 20 us faster than
// unpacking to the staging buffer and copying with the copy engine; the same
// transposition for the inputs was 7 us slower than upload_nodes_kernel.
constexpr int XFER_NT = 256;

__device__ __forceinline__ void aos_store(double *__restrict__ g, const double *__restrict__ s,
                                          int c3) {
  double2 *g2 = reinterpret_cast<double2 *>(g);
  for (int j = threadIdx.x; 2 * j < c3; j += XFER_NT) {
    if (2 * j + 1 < c3)
      g2[j] = make_double2(s[2 * j], s[2 * j + 1]);
    else
      g[2 * j] = s[2 * j];
  }
}

// Node records -> AoS outputs X, V, VR, D (any may be null) written straight
// into registered host memory with 16-byte stores; D = X - X0 in the mixed
// form (D4 holds X0), D4.xyz in the FP64 form; VR zero without rotations.
__global__ void __launch_bounds__(XFER_NT)
download_nodes_kernel(NodeView N, int mixed, double *__restrict__ x, double *__restrict__ v,
                          double *__restrict__ vr, double *__restrict__ d) {
  __shared__ double sh[3 * XFER_NT];
  const int n0 = blockIdx.x * XFER_NT;
  const int cnt = min(XFER_NT, N.numnod - n0);
  const int c3 = 3 * cnt;
  const int t = threadIdx.x;
  const int i = n0 + t;
  double *outs[4] = {x, v, vr, d};
  for (int k = 0; k < 4; k++) {
    if (!outs[k]) continue;  // uniform over the grid
    if (t < cnt) {
      dbl4 r;
      if (k == 0) {
        r = N.X4[i];
      } else if (k == 1) {
        r = N.V4[i];
      } else if (k == 2) {
        r = N.VR4 ? N.VR4[i] : mk4(0.0, 0.0, 0.0, 0.0);
      } else if (mixed) {
        const dbl4 p = N.X4[i], q = N.D4[i];
        r = mk4(p.x - q.x, p.y - q.y, p.z - q.z, 0.0);
      } else {
        r = N.D4[i];
      }
      sh[3 * t] = r.x;
      sh[3 * t + 1] = r.y;
      sh[3 * t + 2] = r.z;
    }
    __syncthreads();
    aos_store(outs[k] + 3 * (size_t)n0, sh, c3);
    __syncthreads();
  }
}

// assemble_kernel's sums (the same fixed-order adds) written straight into
// registered host memory: F and FR through shared memory with 16-byte
// stores, STIFN and STIFR with coalesced 8-byte stores.
template <typename ST, bool ROT>
__global__ void __launch_bounds__(XFER_NT)
assemble_host_kernel(int numnod, const int *__restrict__ adsky, const ST *__restrict__ fsky,
                     const ST *__restrict__ fskyr, double *__restrict__ f,
                     double *__restrict__ stifn, double *__restrict__ fr,
                     double *__restrict__ stifr) {
  __shared__ double sh[2][3 * XFER_NT];
  const int n0 = blockIdx.x * XFER_NT;
  const int cnt = min(XFER_NT, numnod - n0);
  const int t = threadIdx.x;
  const int n = n0 + t;
  if (t < cnt) {
    double a0 = 0.0, a1 = 0.0, a2 = 0.0, st = 0.0;
    double r0 = 0.0, r1 = 0.0, r2 = 0.0, sr = 0.0;
    for (int k = adsky[n]; k < adsky[n + 1]; k++) {
      const ST q = fsky[k];
      a0 = __dadd_rn(a0, (double)q.x);
      a1 = __dadd_rn(a1, (double)q.y);
      a2 = __dadd_rn(a2, (double)q.z);
      st = __dadd_rn(st, (double)q.w);
      if (ROT) {
        const ST g = fskyr[k];
        r0 = __dadd_rn(r0, (double)g.x);
        r1 = __dadd_rn(r1, (double)g.y);
        r2 = __dadd_rn(r2, (double)g.z);
        sr = __dadd_rn(sr, (double)g.w);
      }
    }
    sh[0][3 * t] = a0;
    sh[0][3 * t + 1] = a1;
    sh[0][3 * t + 2] = a2;
    sh[1][3 * t] = r0;
    sh[1][3 * t + 1] = r1;
    sh[1][3 * t + 2] = r2;
    if (stifn) stifn[n] = st;
    if (ROT && stifr) stifr[n] = sr;
  }
  __syncthreads();
  if (f) aos_store(f + 3 * (size_t)n0, sh[0], 3 * cnt);
  if (ROT && fr) aos_store(fr + 3 * (size_t)n0, sh[1], 3 * cnt);
}

// Mixed form: D = X - X0 (D4 holds the initial position).
__global__ void unpack_disp_kernel(int n, const dbl4 *__restrict__ x4,
                                   const dbl4 *__restrict__ x0, double *__restrict__ dst) {
  const int i = blockIdx.x * NODE_NT + threadIdx.x;
  if (i >= n) return;
  const dbl4 a = x4[i], b = x0[i];
  dst[3 * i] = a.x - b.x;
  dst[3 * i + 1] = a.y - b.y;
  dst[3 * i + 2] = a.z - b.z;
}

__global__ void unpack3_kernel(int n, const dbl4 *__restrict__ src,
                               double *__restrict__ dst) {
  const int i = blockIdx.x * NODE_NT + threadIdx.x;
  if (i >= n) return;
  const dbl4 t = src[i];
  dst[3 * i] = t.x;
  dst[3 * i + 1] = t.y;
  dst[3 * i + 2] = t.z;
}

template <typename T>
__global__ void widen_kernel(int n, const T *__restrict__ src,
                             double *__restrict__ dst) {
  const int i = blockIdx.x * NODE_NT + threadIdx.x;
  if (i < n) dst[i] = (double)src[i];
}

// ---------------------------------------------------------------------------
// FILLCNE order (starter/source/spmd/domdec2.F:2046-2250): for each node,
// hexas in increasing user id (stable), then shells in increasing user id;
// W_PON (starter/source/restart/ddsplit/w_pon.F:581-700) assigns each
// (element, corner) the position of that entry.
// ---------------------------------------------------------------------------
void build_skyline(int numnod, int numels, const int *ixs, int numelc,
                   const int *ixc, std::vector<int> &adsky,
                   std::vector<int> &iads, std::vector<int> &iadc) {
  std::vector<int> cnt(numnod + 1, 0);
  for (int e = 0; e < numels; e++)
    for (int k = 0; k < 8; k++) cnt[ixs[11 * e + 1 + k]]++;
  for (int e = 0; e < numelc; e++)
    for (int k = 0; k < 4; k++) cnt[ixc[7 * e + 1 + k]]++;
  adsky.assign(numnod + 1, 0);
  adsky[0] = 1;
  for (int n = 1; n <= numnod; n++) adsky[n] = adsky[n - 1] + cnt[n];
  std::vector<int> next(adsky.begin(), adsky.end() - 1);
  std::vector<int> ord(numels);
  std::iota(ord.begin(), ord.end(), 0);
  std::stable_sort(ord.begin(), ord.end(),
                   [&](int a, int b) { return ixs[11 * a + 10] < ixs[11 * b + 10]; });
  iads.assign(8 * (size_t)numels, 0);
  for (int e : ord)
    for (int k = 0; k < 8; k++) iads[8 * e + k] = next[ixs[11 * e + 1 + k] - 1]++;
  std::vector<int> ordc(numelc);
  std::iota(ordc.begin(), ordc.end(), 0);
  std::stable_sort(ordc.begin(), ordc.end(),
                   [&](int a, int b) { return ixc[7 * a + 6] < ixc[7 * b + 6]; });
  iadc.assign(4 * (size_t)numelc, 0);
  for (int e : ordc)
    for (int k = 0; k < 4; k++) iadc[4 * e + k] = next[ixc[7 * e + 1 + k] - 1]++;
}

// Host validation of engine-provided tables: monotone ADSKY and every slot
// referenced exactly once, so that no device write can leave the buffer.
bool check_skyline(int numnod, int numels, int numelc,
                   const std::vector<int> &adsky, const std::vector<int> &iads,
                   const std::vector<int> &iadc, int &lsky, std::string &why) {
  if ((int)adsky.size() != numnod + 1 || adsky[0] != 1) {
    why = "ADSKY(1) must be 1";
    return false;
  }
  for (int n = 0; n < numnod; n++)
    if (adsky[n + 1] < adsky[n]) {
      why = "ADSKY not monotone";
      return false;
    }
  lsky = adsky[numnod] - 1;
  if ((long long)lsky != 8LL * numels + 4LL * numelc) {
    why = "LSKY != 8*NUMELS + 4*NUMELC";
    return false;
  }
  std::vector<char> used(std::max(lsky, 1), 0);
  auto take = [&](int s) {
    if (s < 1 || s > lsky || used[s - 1]) return false;
    used[s - 1] = 1;
    return true;
  };
  for (int v : iads)
    if (!take(v)) {
      why = "IADS slot out of range or repeated";
      return false;
    }
  for (int v : iadc)
    if (!take(v)) {
      why = "IADC slot out of range or repeated";
      return false;
    }
  return true;
}

template <typename ER>
int alloc_hexa(rg_ctx *c, HexaArrays<ER> &A) {
  const int ne = c->numels;
  A.ne = ne;
  A.nc = c->d_nc;
  A.iads = c->d_iads;
  A.ngl = c->d_ngl_all;
  int r = RG_OK;
  if ((r = dalloc(c, &A.sig, 6 * (size_t)ne))) return r;
  if ((r = dalloc(c, &A.eint, ne))) return r;
  if ((r = dalloc(c, &A.rho, ne))) return r;
  if ((r = dalloc(c, &A.qvis, ne))) return r;
  if ((r = dalloc(c, &A.off, ne))) return r;
  if ((r = dalloc(c, &A.vol0, ne))) return r;
  if ((r = dalloc(c, &A.pla, ne))) return r;
  if ((r = dalloc(c, &A.epsd, ne))) return r;
  if ((r = dalloc(c, &A.ehou, ne))) return r;
  return RG_OK;
}

template <typename ER>
int init_hexa_state(rg_ctx *c, HexaArrays<ER> &A) {
  const int ne = c->numels;
  std::vector<double> vol(ne), rho(ne);
  std::vector<ER> one(ne, (ER)1), zero(6 * (size_t)ne, (ER)0);
  std::vector<double> zd(ne, 0.0);
  for (auto &g : c->hg)
    for (int i = 0; i < g.nel; i++) rho[g.P.nft + i] = g.P.rho0;
  const bool vol_history = !std::is_same<ER, double>::value;
  // initial volume: SDERI3 determinant of the initial geometry
  for (int e = 0; e < ne; e++) {
    double x[8], y[8], z[8];
    for (int k = 0; k < 8; k++) {
      const int n = c->ixs[11 * e + 1 + k] - 1;
      x[k] = c->X[3 * n];
      y[k] = c->X[3 * n + 1];
      z[k] = c->X[3 * n + 2];
    }
    double x17 = x[6] - x[0], x28 = x[7] - x[1], x35 = x[4] - x[2], x46 = x[5] - x[3];
    double y17 = y[6] - y[0], y28 = y[7] - y[1], y35 = y[4] - y[2], y46 = y[5] - y[3];
    double z17 = z[6] - z[0], z28 = z[7] - z[1], z35 = z[4] - z[2], z46 = z[5] - z[3];
    double j1 = x17 + x28 - x35 - x46, j2 = y17 + y28 - y35 - y46, j3 = z17 + z28 - z35 - z46;
    double j4 = (x17 + x46) + (x28 + x35), j5 = (y17 + y46) + (y28 + y35), j6 = (z17 + z46) + (z28 + z35);
    double j7 = (x17 + x46) - (x28 + x35), j8 = (y17 + y46) - (y28 + y35), j9 = (z17 + z46) - (z28 + z35);
    vol[e] = RG_ONE_OVER_64 *
             (j1 * (j5 * j9 - j6 * j8) + j2 * (j6 * j7 - j4 * j9) + j3 * (j4 * j8 - j5 * j7));
    if (!(vol[e] > 0.0)) return fail(c, RG_E_ARG, "hexa with non-positive initial volume");
  }
  RG_CUDA(c, cudaMemcpy(A.sig, zero.data(), 6 * (size_t)ne * sizeof(ER), cudaMemcpyHostToDevice));
  RG_CUDA(c, cudaMemcpy(A.eint, zd.data(), ne * sizeof(double), cudaMemcpyHostToDevice));
  RG_CUDA(c, cudaMemcpy(A.rho, vol_history ? vol.data() : rho.data(), ne * sizeof(double),
                        cudaMemcpyHostToDevice));
  RG_CUDA(c, cudaMemcpy(A.qvis, zero.data(), ne * sizeof(ER), cudaMemcpyHostToDevice));
  RG_CUDA(c, cudaMemcpy(A.off, one.data(), ne * sizeof(ER), cudaMemcpyHostToDevice));
  RG_CUDA(c, cudaMemcpy(A.vol0, vol.data(), ne * sizeof(double), cudaMemcpyHostToDevice));
  RG_CUDA(c, cudaMemcpy(A.pla, zero.data(), ne * sizeof(ER), cudaMemcpyHostToDevice));
  RG_CUDA(c, cudaMemcpy(A.epsd, zero.data(), ne * sizeof(ER), cudaMemcpyHostToDevice));
  RG_CUDA(c, cudaMemcpy(A.ehou, zd.data(), ne * sizeof(double), cudaMemcpyHostToDevice));
  return RG_OK;
}

// Enqueue the element phase (all groups) on the stream, with the time-step
// reduction fused into its last block (advance = 0: DT2T / NELTST only).  A
// model without elements gets the stand-alone time-step kernel.
int enqueue_elements(rg_ctx *c, int advance) {
  const DtPartials dp = c->dp;
  if (c->nparts == 0 && !c->nodadt) {
    dt_kernel<<<1, DT_NT, 0, c->stream>>>(dp, 0, c->d_ngl_all, c->d_time, c->d_status, advance);
    return RG_OK;
  }
  DtFinish F;
  // under the nodal time step the elements give no step: no fused finish
  // (the nodal dt kernel applies the cycle's step)
  F.ctr = c->nodadt ? nullptr : c->d_dtctr;
  F.gdt = c->d_gdt;
  F.gel = c->d_gel;
  F.nparts = c->nparts;
  F.advance = advance;
  F.ngl = c->d_ngl_all;
  for (auto &g : c->hg) {
    if (c->prec == RG_PREC_FP64)
      launch_hexa_f64(g.P, c->h64, c->nv, (dbl4 *)c->d_fsky, dp, c->d_time,
                      c->d_status, F, c->stream);
    else
      launch_hexa_f32(g.P, c->h32, c->nv, (float4 *)c->d_fsky, dp, c->d_time,
                      c->d_status, F, c->stream);
  }
  shell_enqueue(c->shells, c->prec, c->nv, c->d_fsky, c->d_fskyr, dp, c->d_time,
                c->d_status, F, c->stream);
  return RG_OK;
}

template <bool F64, bool ROT>
void launch_nodes(rg_ctx *c) {
  const int nb = (c->numnod + NODE_NT - 1) / NODE_NT;
  const void *fr = ROT ? c->d_fskyr : nullptr;
  if (c->nodadt) {
    DtFinish F;
    F.ctr = c->d_nctr;
    F.gdt = c->d_ngdt;
    F.gel = c->d_ngel;
    F.nparts = c->nnparts;
    F.advance = 1;
    F.ngl = c->d_ngl_nodes;
    nodal_dt_kernel<F64, ROT><<<nb, NODE_NT, 0, c->stream>>>(
        c->nv, c->d_adsky, c->d_fsky, fr, c->dtfac_noda, c->dtmin_noda, c->idtmin_noda, c->ndp,
        c->d_time, c->d_status, F);
  }
  if (c->nlinks)
    rlink_kernel<F64, ROT><<<c->nlinks, LINK_NT, 0, c->stream>>>(
        c->nv, c->d_adsky, c->d_fsky, fr, c->d_lnodes, c->d_loff, c->d_lic, c->d_lacc,
        c->d_status);
  const dbl4 *lacc = c->d_lacc;
  cudaStream_t s = c->stream;
  if (ROT) {
    if (c->nlinks)
      node_kernel_rot<F64, true><<<nb, NODE_NT, 0, s>>>(c->nv, c->d_adsky, c->d_fsky, fr, c->d_time,
                                                        c->d_wall, c->d_walls, lacc, c->d_status);
    else
      node_kernel_rot<F64, false><<<nb, NODE_NT, 0, s>>>(c->nv, c->d_adsky, c->d_fsky, fr, c->d_time,
                                                         c->d_wall, c->d_walls, nullptr, c->d_status);
  } else {
    if (c->nlinks)
      node_kernel<F64, true><<<nb, NODE_NT, 0, s>>>(c->nv, c->d_adsky, c->d_fsky, fr, c->d_time,
                                                    c->d_wall, c->d_walls, lacc, c->d_status);
    else
      node_kernel<F64, false><<<nb, NODE_NT, 0, s>>>(c->nv, c->d_adsky, c->d_fsky, fr, c->d_time,
                                                     c->d_wall, c->d_walls, nullptr, c->d_status);
  }
}

int enqueue_nodes(rg_ctx *c) {
  if (c->prec == RG_PREC_FP64) {
    if (c->rot)
      launch_nodes<true, true>(c);
    else
      launch_nodes<true, false>(c);
  } else {
    if (c->rot)
      launch_nodes<false, true>(c);
    else
      launch_nodes<false, false>(c);
  }
  return RG_OK;
}

int enqueue_assemble(rg_ctx *c, double *f, double *stifn, double *fr, double *stifr) {
  const int nb = (c->numnod + NODE_NT - 1) / NODE_NT;
  if (c->prec == RG_PREC_FP64) {
    if (c->rot)
      assemble_kernel<dbl4, true><<<nb, NODE_NT, 0, c->stream>>>(
          c->numnod, c->d_adsky, (const dbl4 *)c->d_fsky, (const dbl4 *)c->d_fskyr, f, stifn,
          fr, stifr);
    else
      assemble_kernel<dbl4, false><<<nb, NODE_NT, 0, c->stream>>>(
          c->numnod, c->d_adsky, (const dbl4 *)c->d_fsky, nullptr, f, stifn, fr, stifr);
  } else {
    if (c->rot)
      assemble_kernel<float4, true><<<nb, NODE_NT, 0, c->stream>>>(
          c->numnod, c->d_adsky, (const float4 *)c->d_fsky, (const float4 *)c->d_fskyr, f,
          stifn, fr, stifr);
    else
      assemble_kernel<float4, false><<<nb, NODE_NT, 0, c->stream>>>(
          c->numnod, c->d_adsky, (const float4 *)c->d_fsky, nullptr, f, stifn, fr, stifr);
  }
  return RG_OK;
}

int enqueue_cycle(rg_ctx *c, bool parts = false) {
  enqueue_elements(c, 1);
  if (parts) parts_enqueue(c);
  enqueue_nodes(c);
  return RG_OK;
}

// The graph of the next cycle: the one that also takes the per-part sums
// when they are due (rg_part_sums_due), else the plain one.
cudaGraphExec_t next_cycle_graph(rg_ctx *c) {
  if (!c->parts_due) return c->gexec;
  c->parts_due = false;
  c->parts_valid = true;
  return c->gexec_parts;
}

}  // namespace

// ===========================================================================
// C ABI
// ===========================================================================
extern "C" {

int rg_ctx_create(int device, rg_ctx **out) {
  if (!out) return RG_E_ARG;
  *out = nullptr;
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || device < 0 || device >= ndev)
    return RG_E_CUDA;
  rg_ctx *c = new rg_ctx();
  c->device = device;
  if (cudaSetDevice(device) != cudaSuccess ||
      cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking) != cudaSuccess) {
    delete c;
    return RG_E_CUDA;
  }
  for (auto &e : c->ev) cudaEventCreate(&e);
  *out = c;
  return RG_OK;
}

int rg_ctx_destroy(rg_ctx *c) {
  if (!c) return RG_E_ARG;
  cudaSetDevice(c->device);
  cudaStreamSynchronize(c->stream);
  if (c->gexec) cudaGraphExecDestroy(c->gexec);
  if (c->graph) cudaGraphDestroy(c->graph);
  if (c->gexec_parts) cudaGraphExecDestroy(c->gexec_parts);
  if (c->graph_parts) cudaGraphDestroy(c->graph_parts);
  parts_free(c);
  shell_free(c->shells);
  for (void *p : c->allocs) cudaFree(p);
  if (c->d_flush) cudaFree(c->d_flush);
  if (c->h_time) cudaFreeHost(c->h_time);
  for (auto &e : c->ev)
    if (e) cudaEventDestroy(e);
  cudaStreamDestroy(c->stream);
  delete c;
  return RG_OK;
}

const char *rg_last_error(rg_ctx *c) { return c ? c->err.c_str() : "null context"; }

int rg_set_precision(rg_ctx *c, int mode) {
  if (!c) return RG_E_ARG;
  if (c->finalized) return fail(c, RG_E_STATE, "rg_set_precision after rg_finalize");
  if (mode != RG_PREC_FP64 && mode != RG_PREC_MIXED) return fail(c, RG_E_ARG, "bad mode");
  c->prec = mode;
  return RG_OK;
}

int rg_mesh_upload(rg_ctx *c, int numnod, const double *x, const double *v,
                   const double *ms, const double *in, const int *icodt) {
  if (!c) return RG_E_ARG;
  if (c->finalized) return fail(c, RG_E_STATE, "mesh already finalized");
  if (numnod <= 0 || !x || !v || !ms) return fail(c, RG_E_ARG, "rg_mesh_upload: bad arguments");
  c->numnod = numnod;
  c->X.assign(x, x + 3 * (size_t)numnod);
  c->V.assign(v, v + 3 * (size_t)numnod);
  c->MS.assign(ms, ms + numnod);
  c->IN.assign(numnod, 0.0);
  if (in) c->IN.assign(in, in + numnod);
  c->icodt.assign(numnod, 0);
  if (icodt) c->icodt.assign(icodt, icodt + numnod);
  for (int n = 0; n < numnod; n++)
    if (c->icodt[n] < 0 || c->icodt[n] > 63) return fail(c, RG_E_ARG, "boundary code out of range");
  return RG_OK;
}

int rg_hexa_group_add(rg_ctx *c, int nel, const int *ixs, int mtn,
                      const double *pm, const double *geo,
                      const double *uparam, const int *iparam, int ismstr,
                      int jhbe, int jcvt) {
  if (!c) return RG_E_ARG;
  if (c->finalized) return fail(c, RG_E_STATE, "group added after rg_finalize");
  if (c->numnod <= 0) return fail(c, RG_E_STATE, "rg_mesh_upload first");
  if (nel <= 0 || !ixs || !pm || !geo) return fail(c, RG_E_ARG, "rg_hexa_group_add: bad arguments");
  if (mtn != 1 && mtn != 2) return fail(c, RG_E_UNSUP, "hexa: only LAW1 and LAW2");
  if (ismstr != 4 || jhbe != 1 || (jcvt != 0 && jcvt != 1))
    return fail(c, RG_E_UNSUP, "hexa: supported formulation is ISMSTR=4, JHBE=1, JCVT=0 or 1");
  if (mtn == 2 && (!uparam || !iparam)) return fail(c, RG_E_ARG, "LAW2 needs uparam/iparam");
  for (int e = 0; e < nel; e++)
    for (int k = 1; k <= 8; k++) {
      const int n = ixs[11 * e + k];
      if (n < 1 || n > c->numnod) return fail(c, RG_E_ARG, "IXS node number out of range");
    }
  HexaGroupHost g{};
  HexaParams &P = g.P;
  P.nft = c->numels;
  P.nel = nel;
  P.mtn = mtn;
  P.rho0 = pm[0];
  P.g = pm[21];
  P.c1 = pm[31];
  P.qh = geo[12];
  P.qa = geo[13];
  P.qb = geo[14];
  P.vns1 = geo[15];
  P.vns2 = geo[16];
  P.jcvt = jcvt;
  if (!(P.rho0 > 0.0)) return fail(c, RG_E_ARG, "PM(1) density must be > 0");
  // M1LAW / M2LAW: SSP = SQRT((ONEP333*G + C1)/RHO0), a group constant at OFF=1
  P.ssp1 = std::sqrt((RG_ONEP333 * (P.g * 1.0) + P.c1) / P.rho0);
  P.has_cns = (P.vns1 != 0.0 || P.vns2 != 0.0) ? 1 : 0;
  if (mtn == 2) {
    if (iparam[0] != 0 || uparam[7] != 0.0)
      return fail(c, RG_E_UNSUP, "LAW2: Zerilli or kinematic hardening not supported");
    // adiabatic heating needs a temperature per element (M2LAW's TSTAR):
    // not carried by the hexa path, refused rather than ignored
    if (pm[68] > 0.0)
      return fail(c, RG_E_UNSUP, "hexa LAW2: thermal softening (rho*Cp > 0) not supported");
    P.icc = iparam[1];
    P.vp = iparam[2];
    P.israte = iparam[3];
    P.ca = uparam[0];
    P.cb = uparam[1];
    P.cn = uparam[2];
    P.epmx = uparam[3];
    P.sigm0 = uparam[4];
    P.cc = uparam[5];
    P.epdr = uparam[6];
    P.asrate = uparam[8];
    P.z3 = uparam[9];
  }
  g.nel = nel;
  c->hg.push_back(g);
  c->ixs.insert(c->ixs.end(), ixs, ixs + 11 * (size_t)nel);
  c->numels += nel;
  return (int)c->hg.size() - 1;
}

int rg_shell_group_add(rg_ctx *c, int nel, const int *ixc, int npt,
                       const double *pm, const double *geo,
                       const double *uparam, const int *iparam,
                       const double *thk0, int ismstr, int ithk) {
  if (!c) return RG_E_ARG;
  if (c->finalized) return fail(c, RG_E_STATE, "group added after rg_finalize");
  if (c->numnod <= 0) return fail(c, RG_E_STATE, "rg_mesh_upload first");
  std::string why;
  const int r = shell_group_add(c->shells, c->numnod, nel, ixc, npt, pm, geo, uparam,
                                iparam, thk0, ismstr, ithk, why);
  if (r < 0) return fail(c, r, why);
  return r;
}

int rg_rwall_add(rg_ctx *c, const double *p0, const double *nrm, double dsearch) {
  if (!c || !p0 || !nrm) return RG_E_ARG;
  if (c->finalized) return fail(c, RG_E_STATE, "wall added after rg_finalize");
  WallHost w;
  const double nn = std::sqrt(nrm[0] * nrm[0] + nrm[1] * nrm[1] + nrm[2] * nrm[2]);
  if (!(nn > 0)) return fail(c, RG_E_ARG, "zero wall normal");
  for (int i = 0; i < 3; i++) {
    w.p0[i] = p0[i];
    w.n[i] = nrm[i] / nn;
  }
  w.dsearch = dsearch;
  c->walls.push_back(w);
  return (int)c->walls.size() - 1;
}

int rg_rlink_add(rg_ctx *c, int nsn, const int *nodes, int ic, int icr) {
  if (!c) return RG_E_ARG;
  if (c->finalized) return fail(c, RG_E_STATE, "rigid link added after rg_finalize");
  if (c->numnod <= 0) return fail(c, RG_E_STATE, "rg_mesh_upload first");
  if (nsn <= 0 || !nodes) return fail(c, RG_E_ARG, "rg_rlink_add: bad arguments");
  if (ic < 0 || ic > 7 || icr < 0 || icr > 7)
    return fail(c, RG_E_ARG, "rg_rlink_add: direction codes must be 0..7");
  LinkHost L;
  for (int i = 0; i < nsn; i++) {
    if (nodes[i] < 1 || nodes[i] > c->numnod) return fail(c, RG_E_ARG, "rigid link node out of range");
    L.nodes.push_back(nodes[i] - 1);
  }
  L.ic = ic;
  L.icr = icr;
  c->links.push_back(L);
  return (int)c->links.size() - 1;
}

int rg_rlink_set_active(rg_ctx *c, int link, int active) {
  if (!c) return RG_E_ARG;
  if (!c->finalized) return fail(c, RG_E_STATE, "rg_finalize first");
  if (link < 0 || link >= c->nlinks) return fail(c, RG_E_ARG, "no such rigid link");
  RG_CUDA(c, cudaSetDevice(c->device));
  // ordered after the cycles already queued on the context's stream
  const LinkHost &L = c->links[link];
  c->h_link = make_int4(L.ic, L.icr, active ? 1 : 0, 0);
  RG_CUDA(c, cudaMemcpyAsync(c->d_lic + link, &c->h_link, sizeof(int4), cudaMemcpyHostToDevice,
                             c->stream));
  RG_CUDA(c, cudaStreamSynchronize(c->stream));
  return RG_OK;
}

int rg_set_nodal_dt(rg_ctx *c, double dtfac, double dtmin) {
  if (!c) return RG_E_ARG;
  if (c->finalized) return fail(c, RG_E_STATE, "rg_set_nodal_dt after rg_finalize");
  if (!(dtfac > 0.0) || dtmin < 0.0) return fail(c, RG_E_ARG, "rg_set_nodal_dt: bad factors");
  c->nodadt = 1;
  c->shells.nodadt = 1;
  c->dtfac_noda = dtfac;
  c->dtmin_noda = dtmin;
  return RG_OK;
}

int rg_set_dtmin(rg_ctx *c, int kind, int idtmin, double dtmin) {
  if (!c) return RG_E_ARG;
  if (c->finalized) return fail(c, RG_E_STATE, "rg_set_dtmin after rg_finalize");
  if (!(dtmin >= 0.0)) return fail(c, RG_E_ARG, "rg_set_dtmin: DTMIN must be >= 0");
  if (kind == 3) {
    if (idtmin != 0 && idtmin != 1 && idtmin != 2 && idtmin != 5)
      return fail(c, RG_E_UNSUP, "shell IDTMIN must be 0, 1, 2 or 5 (3: small-strain switch not built)");
    c->shells.idtmin = idtmin;
    c->shells.dtmin = dtmin;
    return RG_OK;
  }
  if (kind == 11) {
    if (idtmin != 0 && idtmin != 1 && idtmin != 3 && idtmin != 5 && idtmin != 8)
      return fail(c, RG_E_UNSUP, "nodal IDTMIN must be 0, 1, 3, 5 or 8 (4: acceleration scaling not built)");
    c->idtmin_noda = idtmin;
    c->dtmin_noda = dtmin;
    return RG_OK;
  }
  return fail(c, RG_E_UNSUP, "rg_set_dtmin: kind must be 3 (shells) or 11 (nodal time step)");
}

int rg_set_shell_frame(rg_ctx *c, int ishfram) {
  if (!c) return RG_E_ARG;
  if (c->finalized) return fail(c, RG_E_STATE, "rg_set_shell_frame after rg_finalize");
  if (ishfram != 0 && ishfram != 2) return fail(c, RG_E_UNSUP, "ISHFRAM must be 0 or 2");
  c->shells.ishfram = ishfram;
  return RG_OK;
}

int rg_skyline_set(rg_ctx *c, const int *adsky, const int *iads, const int *iadc) {
  if (!c || !adsky) return RG_E_ARG;
  if (c->finalized) return fail(c, RG_E_STATE, "skyline set after rg_finalize");
  c->adsky.assign(adsky, adsky + c->numnod + 1);
  c->iads.assign(8 * (size_t)c->numels, 0);
  if (c->numels) {
    if (!iads) return fail(c, RG_E_ARG, "IADS missing");
    c->iads.assign(iads, iads + 8 * (size_t)c->numels);
  }
  const int nc = shell_numelc(c->shells);
  c->iadc.assign(4 * (size_t)nc, 0);
  if (nc) {
    if (!iadc) return fail(c, RG_E_ARG, "IADC missing");
    c->iadc.assign(iadc, iadc + 4 * (size_t)nc);
  }
  c->skyline_given = true;
  return RG_OK;
}

int rg_finalize(rg_ctx *c, double dtfac_solid, double dtfac_shell, double dtmx,
                double dt2old) {
  if (!c) return RG_E_ARG;
  if (c->finalized) return fail(c, RG_E_STATE, "already finalized");
  if (c->numnod <= 0) return fail(c, RG_E_STATE, "no mesh");
  RG_CUDA(c, cudaSetDevice(c->device));
  c->dtfac_solid = dtfac_solid;
  c->dtfac_shell = dtfac_shell;
  c->dtmx = dtmx;
  c->dt2old = dt2old;
  const int numnod = c->numnod, ne = c->numels;
  const int nc = shell_numelc(c->shells);
  c->rot = nc > 0;
  // PARITH/ON tables
  if (!c->skyline_given)
    build_skyline(numnod, ne, c->ixs.data(), nc, shell_ixc(c->shells), c->adsky, c->iads,
                  c->iadc);
  std::string why;
  if (!check_skyline(numnod, ne, nc, c->adsky, c->iads, c->iadc, c->lsky, why))
    return fail(c, RG_E_ARG, "skyline: " + why);
  int r;
  // rigid links: 1-based link index per node, carried in the node code
  c->nlinks = (int)c->links.size();
  std::vector<int> lnk(numnod, 0);
  for (int l = 0; l < c->nlinks; l++)
    for (int n : c->links[l].nodes) {
      if (lnk[n]) return fail(c, RG_E_ARG, "a node belongs to two rigid links");
      lnk[n] = l + 1;
    }
  // nodes
  // X4.w = 1/MS and VR4.w = 1/IN: ACCELE's RTMP = ONE/MS(N) evaluated once
  // (the same IEEE quotient), D4.w = MS and DR4.w = IN for the energies.
  std::vector<dbl4> x4(numnod), v4(numnod), z4(numnod, mk4(0, 0, 0, 0)),
      vr4(numnod, mk4(0, 0, 0, 0)), dr4(numnod, mk4(0, 0, 0, 0));
  for (int n = 0; n < numnod; n++) {
    const double ms = c->MS[n], in = c->IN[n];
    x4[n] = mk4(c->X[3 * n], c->X[3 * n + 1], c->X[3 * n + 2], ms > 0.0 ? 1.0 / ms : 0.0);
    v4[n] = mk4(c->V[3 * n], c->V[3 * n + 1], c->V[3 * n + 2],
                (double)(c->icodt[n] | (lnk[n] << RG_LINK_SHIFT)));
    // D4: displacement (FP64 form) or initial position (mixed form), MS
    z4[n] = c->prec == RG_PREC_MIXED
                ? mk4(c->X[3 * n], c->X[3 * n + 1], c->X[3 * n + 2], ms)
                : mk4(0, 0, 0, ms);
    vr4[n].w = in > 0.0 ? 1.0 / in : 0.0;
    dr4[n].w = in;
  }
  if ((r = dalloc(c, &c->nv.X4, numnod))) return r;
  if ((r = dalloc(c, &c->nv.V4, numnod))) return r;
  if ((r = dalloc(c, &c->nv.D4, numnod))) return r;
  c->nv.numnod = numnod;
  RG_CUDA(c, cudaMemcpy(c->nv.X4, x4.data(), numnod * sizeof(dbl4), cudaMemcpyHostToDevice));
  RG_CUDA(c, cudaMemcpy(c->nv.V4, v4.data(), numnod * sizeof(dbl4), cudaMemcpyHostToDevice));
  RG_CUDA(c, cudaMemcpy(c->nv.D4, z4.data(), numnod * sizeof(dbl4), cudaMemcpyHostToDevice));
  if (c->rot) {
    if ((r = dalloc(c, &c->nv.VR4, numnod))) return r;
    if ((r = dalloc(c, &c->nv.DR4, numnod))) return r;
    RG_CUDA(c, cudaMemcpy(c->nv.VR4, vr4.data(), numnod * sizeof(dbl4), cudaMemcpyHostToDevice));
    RG_CUDA(c, cudaMemcpy(c->nv.DR4, dr4.data(), numnod * sizeof(dbl4), cudaMemcpyHostToDevice));
  }
  if (c->prec == RG_PREC_MIXED) {
    if ((r = dalloc(c, &c->nv.XF, numnod))) return r;
    if ((r = dalloc(c, &c->nv.VF, numnod))) return r;
    if (c->rot && (r = dalloc(c, &c->nv.VRF, numnod))) return r;
    // the synchronous uploads above ran on the legacy stream, which the
    // context's non-blocking stream does not wait for: fence them first
    RG_CUDA(c, cudaStreamSynchronize(cudaStreamLegacy));
    refresh_copies_kernel<<<(numnod + NODE_NT - 1) / NODE_NT, NODE_NT, 0, c->stream>>>(
        c->nv, c->rot ? 1 : 0);
    RG_CUDA(c, cudaStreamSynchronize(c->stream));
  }
  // skyline (0-based on the device)
  std::vector<int> ad0(numnod + 1);
  for (int n = 0; n <= numnod; n++) ad0[n] = c->adsky[n] - 1;
  if ((r = dalloc(c, &c->d_adsky, numnod + 1))) return r;
  RG_CUDA(c, cudaMemcpy(c->d_adsky, ad0.data(), (numnod + 1) * sizeof(int), cudaMemcpyHostToDevice));
  const size_t slot_bytes = c->prec == RG_PREC_FP64 ? sizeof(dbl4) : sizeof(float4);
  {
    char *p = nullptr;
    if ((r = dalloc(c, &p, slot_bytes * std::max(c->lsky, 1)))) return r;
    RG_CUDA(c, cudaMemset(p, 0, slot_bytes * std::max(c->lsky, 1)));
    c->d_fsky = p;
    if (c->rot) {
      char *q = nullptr;
      if ((r = dalloc(c, &q, slot_bytes * std::max(c->lsky, 1)))) return r;
      RG_CUDA(c, cudaMemset(q, 0, slot_bytes * std::max(c->lsky, 1)));
      c->d_fskyr = q;
    }
  }
  // hexa connectivity / slots as SoA [8][ne], 0-based; user ids
  std::vector<int> nc8(8 * (size_t)std::max(ne, 1)), ia8(8 * (size_t)std::max(ne, 1));
  for (int e = 0; e < ne; e++)
    for (int k = 0; k < 8; k++) {
      nc8[(size_t)k * ne + e] = c->ixs[11 * e + 1 + k] - 1;
      ia8[(size_t)k * ne + e] = c->iads[8 * e + k] - 1;
    }
  std::vector<int> ngl_all(ne + nc + 1, 0);
  for (int e = 0; e < ne; e++) ngl_all[e] = c->ixs[11 * e + 10];
  shell_user_ids(c->shells, ngl_all.data() + ne);
  if ((r = dalloc(c, &c->d_nc, 8 * (size_t)std::max(ne, 1)))) return r;
  if ((r = dalloc(c, &c->d_iads, 8 * (size_t)std::max(ne, 1)))) return r;
  if ((r = dalloc(c, &c->d_ngl_all, ne + nc + 1))) return r;
  RG_CUDA(c, cudaMemcpy(c->d_nc, nc8.data(), nc8.size() * sizeof(int), cudaMemcpyHostToDevice));
  RG_CUDA(c, cudaMemcpy(c->d_iads, ia8.data(), ia8.size() * sizeof(int), cudaMemcpyHostToDevice));
  RG_CUDA(c, cudaMemcpy(c->d_ngl_all, ngl_all.data(), ngl_all.size() * sizeof(int),
                        cudaMemcpyHostToDevice));
  // hexa state
  if (ne > 0) {
    if (c->prec == RG_PREC_FP64) {
      if ((r = alloc_hexa(c, c->h64))) return r;
      if ((r = init_hexa_state(c, c->h64))) return r;
    } else {
      if ((r = alloc_hexa(c, c->h32))) return r;
      if ((r = init_hexa_state(c, c->h32))) return r;
    }
  }
  // dt partial slots: one per element block of every launch
  c->nparts = 0;
  for (auto &g : c->hg) {
    g.P.part_off = c->nparts;
    g.P.dtfac = dtfac_solid;
    g.P.nodadt = c->nodadt;
    hexa_params_mirror(g.P);
    c->nparts += hexa_blocks(g.nel);
  }
  {
    auto alloc_fn = [c](void **p, size_t bytes) -> int {
      cudaError_t e = cudaMalloc(p, std::max<size_t>(bytes, 16));
      if (e != cudaSuccess) return fail(c, RG_E_MEM, cudaGetErrorString(e));
      c->allocs.push_back(*p);
      c->alloc_bytes.push_back(std::max<size_t>(bytes, 16));
      c->dev_bytes += bytes;
      return RG_OK;
    };
    if ((r = shell_finalize(c->shells, c->prec, c->X.data(), c->iadc.data(), ne, dtfac_shell,
                            c->nparts, alloc_fn, why)))
      return fail(c, r, "shell set-up: " + why);
  }
  // the partial arrays also hold one slot per 128-element tile of every
  // group: the batched kernel writes a job's partials in that layout, which
  // has more slots than a balanced FP64 shell launch
  {
    int tiles = 0;
    for (auto &g : c->hg) tiles += hexa_blocks(g.nel);
    tiles += shell_tile_count(c->shells);
    c->nparts_cap = std::max(c->nparts, tiles);
  }
  if ((r = dalloc(c, &c->dp.dt, std::max(c->nparts_cap, 1)))) return r;
  if ((r = dalloc(c, &c->dp.el, std::max(c->nparts_cap, 1)))) return r;
  // time scalars
  Time t{};
  t.tt = 0;
  t.dt1 = 0;
  t.dt2 = 0;
  t.dt12 = 0;
  t.dt2old = dt2old;
  t.dtmx = dtmx;
  t.dt2t = 0;
  // the nodal kernel flags a node step below DTMIN1(11) itself; with mass
  // scaling (IDTMIN(11) = 3 / 8) the cycle of the scaling keeps its step
  // below DTMIN1(11) and the run goes on (no flag)
  t.dtmin = c->nodadt && c->idtmin_noda != 3 && c->idtmin_noda != 8 ? c->dtmin_noda : 0.0;
  if ((r = dalloc(c, &c->d_time, 1))) return r;
  RG_CUDA(c, cudaMemcpy(c->d_time, &t, sizeof(Time), cudaMemcpyHostToDevice));
  if ((r = dalloc(c, &c->d_status, 1))) return r;
  RG_CUDA(c, cudaMemset(c->d_status, 0, sizeof(int)));
  // rigid walls
  c->nwalls = (int)c->walls.size();
  if (c->nwalls) {
    std::vector<int> wn(numnod, -1);
    // device record: P0, N in FP64, then the same in FP32 (RG_WALL_STRIDE)
    std::vector<double> wd(RG_WALL_STRIDE * c->nwalls);
    for (int w = 0; w < c->nwalls; w++) {
      const WallHost &W = c->walls[w];
      double *rec = wd.data() + RG_WALL_STRIDE * w;
      float f32[6];
      for (int i = 0; i < 3; i++) {
        rec[i] = W.p0[i];
        rec[3 + i] = W.n[i];
        f32[i] = (float)W.p0[i];
        f32[3 + i] = (float)W.n[i];
      }
      memcpy(rec + 6, f32, sizeof f32);
      for (int n = 0; n < numnod; n++) {
        const double d = (c->X[3 * n] - W.p0[0]) * W.n[0] + (c->X[3 * n + 1] - W.p0[1]) * W.n[1] +
                         (c->X[3 * n + 2] - W.p0[2]) * W.n[2];
        if (d <= W.dsearch && wn[n] < 0) wn[n] = w;
      }
    }
    if ((r = dalloc(c, &c->d_wall, numnod))) return r;
    if ((r = dalloc(c, &c->d_walls, RG_WALL_STRIDE * c->nwalls))) return r;
    RG_CUDA(c, cudaMemcpy(c->d_wall, wn.data(), numnod * sizeof(int), cudaMemcpyHostToDevice));
    RG_CUDA(c, cudaMemcpy(c->d_walls, wd.data(), wd.size() * sizeof(double), cudaMemcpyHostToDevice));
    // external work of the walls, accumulated per node by the node kernel
    if ((r = dalloc(c, &c->nv.wext, numnod))) return r;
    RG_CUDA(c, cudaMemset(c->nv.wext, 0, numnod * sizeof(double)));
  }
  if (c->nlinks) {
    std::vector<int> ln, lo(1, 0);
    std::vector<int4> li;
    for (auto &L : c->links) {
      ln.insert(ln.end(), L.nodes.begin(), L.nodes.end());
      lo.push_back((int)ln.size());
      li.push_back(make_int4(L.ic, L.icr, 1, 0));
    }
    if ((r = dalloc(c, &c->d_lnodes, ln.size()))) return r;
    if ((r = dalloc(c, &c->d_loff, lo.size()))) return r;
    if ((r = dalloc(c, &c->d_lic, li.size()))) return r;
    if ((r = dalloc(c, &c->d_lacc, 2 * li.size()))) return r;
    RG_CUDA(c, cudaMemcpy(c->d_lnodes, ln.data(), ln.size() * sizeof(int), cudaMemcpyHostToDevice));
    RG_CUDA(c, cudaMemcpy(c->d_loff, lo.data(), lo.size() * sizeof(int), cudaMemcpyHostToDevice));
    RG_CUDA(c, cudaMemcpy(c->d_lic, li.data(), li.size() * sizeof(int4), cudaMemcpyHostToDevice));
  }
  {
    const int ng = (c->nparts + DT_GROUP - 1) / DT_GROUP;
    if ((r = dalloc(c, &c->d_dtctr, ng + 1))) return r;
    if ((r = dalloc(c, &c->d_gdt, std::max(ng, 1)))) return r;
    if ((r = dalloc(c, &c->d_gel, std::max(ng, 1)))) return r;
    RG_CUDA(c, cudaMemset(c->d_dtctr, 0, (ng + 1) * sizeof(unsigned)));
  }
  if (c->nodadt) {
    c->nnparts = (numnod + NODE_NT - 1) / NODE_NT;
    const int ng = (c->nnparts + DT_GROUP - 1) / DT_GROUP;
    if ((r = dalloc(c, &c->ndp.dt, c->nnparts))) return r;
    if ((r = dalloc(c, &c->ndp.el, c->nnparts))) return r;
    if ((r = dalloc(c, &c->d_nctr, ng + 1))) return r;
    if ((r = dalloc(c, &c->d_ngdt, ng))) return r;
    if ((r = dalloc(c, &c->d_ngel, ng))) return r;
    RG_CUDA(c, cudaMemset(c->d_nctr, 0, (ng + 1) * sizeof(unsigned)));
    // order key -> node number: translational keys 2*numnod-1-n, rotational
    // numnod-1-n
    std::vector<int> nn(2 * (size_t)numnod);
    for (int n = 0; n < numnod; n++) {
      nn[2 * (size_t)numnod - 1 - n] = n + 1;
      nn[numnod - 1 - n] = n + 1;
    }
    if ((r = dalloc(c, &c->d_ngl_nodes, nn.size()))) return r;
    RG_CUDA(c, cudaMemcpy(c->d_ngl_nodes, nn.data(), nn.size() * sizeof(int),
                          cudaMemcpyHostToDevice));
  }
  if ((r = dalloc(c, &c->d_stage, 12 * (size_t)numnod + 16))) return r;
  RG_CUDA(c, cudaMallocHost((void **)&c->h_time, sizeof(Time)));
  if ((r = dalloc(c, &c->d_epart, 9 * EN_BLOCKS + 8))) return r;
  RG_CUDA(c, cudaStreamSynchronize(cudaStreamLegacy));  // uploads complete
  RG_CUDA(c, cudaStreamSynchronize(c->stream));
  // capture one cycle as a graph
  RG_CUDA(c, cudaStreamBeginCapture(c->stream, cudaStreamCaptureModeThreadLocal));
  enqueue_cycle(c);
  cudaError_t ce = cudaStreamEndCapture(c->stream, &c->graph);
  if (ce != cudaSuccess) return fail(c, RG_E_CUDA, std::string("graph capture: ") + cudaGetErrorString(ce));
  RG_CUDA(c, cudaGraphInstantiate(&c->gexec, c->graph, 0));
  c->finalized = true;
  // cycle-0 totals of the energy balance (ECRIT's ENTOT0 and MASS0)
  {
    double b[13];
    if ((r = rg_energy_balance(c, b, 13))) return r;
    c->entot0 = b[6];
    c->mass0 = b[8];
  }
  return RG_OK;
}

int rg_skyline_get(rg_ctx *c, int *adsky, int *iads, int *iadc, int *lsky) {
  if (!c) return RG_E_ARG;
  if (!c->finalized) return fail(c, RG_E_STATE, "not finalized");
  if (adsky) std::copy(c->adsky.begin(), c->adsky.end(), adsky);
  if (iads) std::copy(c->iads.begin(), c->iads.end(), iads);
  if (iadc) std::copy(c->iadc.begin(), c->iadc.end(), iadc);
  if (lsky) *lsky = c->lsky;
  return RG_OK;
}

int rg_cycle(rg_ctx *c, int ncycle) {
  if (!c) return RG_E_ARG;
  if (!c->finalized) return fail(c, RG_E_STATE, "rg_finalize first");
  if (ncycle < 0) return fail(c, RG_E_ARG, "negative cycle count");
  RG_CUDA(c, cudaSetDevice(c->device));
  if (!c->timing) {
    for (int i = 0; i < ncycle; i++) RG_CUDA(c, cudaGraphLaunch(next_cycle_graph(c), c->stream));
    return RG_OK;
  }
  // timed path: the same launches, bracketed by events per kernel class
  double acc[4] = {0, 0, 0, 0};
  for (int i = 0; i < ncycle; i++) {
    // after rg_time_cycles_cold: each timed cycle starts from cold L2 too
    if (c->d_flush) cudaMemsetAsync(c->d_flush, i & 0xff, c->flush_bytes, c->stream);
    cudaEventRecord(c->ev[0], c->stream);
    const DtPartials dp = c->dp;
    DtFinish F;
    F.ctr = c->nodadt ? nullptr : c->d_dtctr;
    F.gdt = c->d_gdt;
    F.gel = c->d_gel;
    F.nparts = c->nparts;
    F.advance = 1;
    F.ngl = c->d_ngl_all;
    for (auto &g : c->hg) {
      if (c->prec == RG_PREC_FP64)
        launch_hexa_f64(g.P, c->h64, c->nv, (dbl4 *)c->d_fsky, dp, c->d_time, c->d_status, F,
                        c->stream);
      else
        launch_hexa_f32(g.P, c->h32, c->nv, (float4 *)c->d_fsky, dp, c->d_time, c->d_status, F,
                        c->stream);
    }
    cudaEventRecord(c->ev[1], c->stream);
    shell_enqueue(c->shells, c->prec, c->nv, c->d_fsky, c->d_fskyr, dp, c->d_time, c->d_status,
                  F, c->stream);
    cudaEventRecord(c->ev[2], c->stream);
    // the time-step reduction runs inside the last element block (or the
    // nodal dt kernel, launched with the node phase)
    if (c->nparts == 0 && !c->nodadt)
      dt_kernel<<<1, DT_NT, 0, c->stream>>>(dp, 0, c->d_ngl_all, c->d_time, c->d_status, 1);
    if (c->parts_due) {
      parts_enqueue(c);
      c->parts_due = false;
      c->parts_valid = true;
    }
    cudaEventRecord(c->ev[3], c->stream);
    enqueue_nodes(c);
    cudaEventRecord(c->ev[4], c->stream);
    RG_CUDA(c, cudaEventSynchronize(c->ev[4]));
    float ms;
    for (int k = 0; k < 4; k++) {
      cudaEventElapsedTime(&ms, c->ev[k], c->ev[k + 1]);
      acc[k] += ms;
    }
  }
  for (int k = 0; k < 4; k++) c->ktime[k] = ncycle ? acc[k] / ncycle : 0.0;
  return RG_OK;
}

int rg_synchronize(rg_ctx *c) {
  if (!c) return RG_E_ARG;
  RG_CUDA(c, cudaStreamSynchronize(c->stream));
  return RG_OK;
}

int rg_host_register(rg_ctx *c, void *ptr, unsigned long long bytes) {
  if (!c || !ptr) return RG_E_ARG;
  RG_CUDA(c, cudaHostRegister(ptr, bytes, cudaHostRegisterDefault));
  return RG_OK;
}
int rg_host_unregister(rg_ctx *c, void *ptr) {
  if (!c || !ptr) return RG_E_ARG;
  RG_CUDA(c, cudaHostUnregister(ptr));
  return RG_OK;
}

}  // extern "C"

namespace {
// Device address of a host buffer the kernels may access in place: memory
// registered with rg_host_register (or device / managed memory); null for
// ordinary pageable memory, which is staged instead.
// Device -> host copies of up to four staged arrays on the context's stream
// (spreading them over side streams, one copy engine each, measured no
// faster: the host link, not the engines, sets their pace).
int copy_out(rg_ctx *c, double *const dst[4], const double *const src[4],
             const size_t bytes[4]) {
  for (int k = 0; k < 4; k++)
    if (dst[k])
      RG_CUDA(c, cudaMemcpyAsync(dst[k], src[k], bytes[k], cudaMemcpyDeviceToHost, c->stream));
  return RG_OK;
}

bool al16(const void *p) { return p && ((uintptr_t)p & 15) == 0; }

// The node upload of a host-buffer call.
void launch_upload(rg_ctx *c, const double *dx, const double *dv, const double *dvr,
                   double dt1) {
  const int n = c->numnod;
  upload_nodes_kernel<<<(n + NODE_NT - 1) / NODE_NT, NODE_NT, 0, c->stream>>>(
      c->nv, dx, dv, dvr, c->prec == RG_PREC_MIXED ? 1 : 0, c->d_time, dt1);
}

const double *device_view(const void *p) {
  cudaPointerAttributes a;
  if (!p || cudaPointerGetAttributes(&a, p) != cudaSuccess) {
    cudaGetLastError();
    return nullptr;
  }
  if (a.type == cudaMemoryTypeHost) return (const double *)a.devicePointer;
  if (a.type == cudaMemoryTypeDevice || a.type == cudaMemoryTypeManaged) return (const double *)p;
  return nullptr;
}
}  // namespace

extern "C" {

int rg_forint_step(rg_ctx *c, const double *x, const double *v, const double *vr,
                   double dt1, double *f, double *stifn, double *fr, double *stifr,
                   double *dt2t, int *neltst) {
  if (!c || !x || !v) return RG_E_ARG;
  if (!c->finalized) return fail(c, RG_E_STATE, "rg_finalize first");
  RG_CUDA(c, cudaSetDevice(c->device));
  const int n = c->numnod;
  const size_t n3 = 3 * (size_t)n;
  double *st = c->d_stage;
  // Registered (pinned) host buffers are read and written by the kernels in
  // place over the host link; other buffers go through the staging buffer.
  const bool rot_in = vr && c->rot;
  const double *dx = device_view(x), *dv = device_view(v);
  const double *dvr = rot_in ? device_view(vr) : nullptr;
  if (!dx) {
    RG_CUDA(c, cudaMemcpyAsync(st, x, n3 * sizeof(double), cudaMemcpyHostToDevice, c->stream));
    dx = st;
  }
  if (!dv) {
    RG_CUDA(c, cudaMemcpyAsync(st + n3, v, n3 * sizeof(double), cudaMemcpyHostToDevice,
                               c->stream));
    dv = st + n3;
  }
  if (rot_in && !dvr) {
    RG_CUDA(c, cudaMemcpyAsync(st + 2 * n3, vr, n3 * sizeof(double), cudaMemcpyHostToDevice,
                               c->stream));
    dvr = st + 2 * n3;
  }
  launch_upload(c, dx, dv, dvr, dt1);
  if (c->prec == RG_PREC_MIXED && c->numels > 0)
    launch_hexa_prev_volume(c->h32, c->nv, c->d_time, c->stream);
  enqueue_elements(c, 0);
  if (c->parts_due) {
    parts_enqueue(c);
    c->parts_due = false;
    c->parts_valid = true;
  }
  // outputs: registered (or device) and F, FR 16-byte aligned -> written in
  // place by assemble_host_kernel (crash box: 0.375 -> 0.367 ms FP64, 0.172
  // -> 0.157 ms mixed per call); else assembled into the staging buffer and
  // returned by DMA copies
  {
    double *ho[4] = {f, stifn, fr, stifr};
    double *dvo[4] = {nullptr, nullptr, nullptr, nullptr};
    bool direct = true, any = false;
    for (int k = 0; k < 4 && direct; k++) {
      if (!ho[k]) continue;
      any = true;
      dvo[k] = const_cast<double *>(device_view(ho[k]));
      direct = dvo[k] && ((k & 1) ? ((uintptr_t)dvo[k] & 7) == 0 : al16(dvo[k]));
    }
    if (direct && any) {
      const int nbx = (n + XFER_NT - 1) / XFER_NT;
      if (c->prec == RG_PREC_FP64) {
        if (c->rot)
          assemble_host_kernel<dbl4, true><<<nbx, XFER_NT, 0, c->stream>>>(
              n, c->d_adsky, (const dbl4 *)c->d_fsky, (const dbl4 *)c->d_fskyr, dvo[0], dvo[1],
              dvo[2], dvo[3]);
        else
          assemble_host_kernel<dbl4, false><<<nbx, XFER_NT, 0, c->stream>>>(
              n, c->d_adsky, (const dbl4 *)c->d_fsky, nullptr, dvo[0], dvo[1], nullptr, nullptr);
      } else {
        if (c->rot)
          assemble_host_kernel<float4, true><<<nbx, XFER_NT, 0, c->stream>>>(
              n, c->d_adsky, (const float4 *)c->d_fsky, (const float4 *)c->d_fskyr, dvo[0],
              dvo[1], dvo[2], dvo[3]);
        else
          assemble_host_kernel<float4, false><<<nbx, XFER_NT, 0, c->stream>>>(
              n, c->d_adsky, (const float4 *)c->d_fsky, nullptr, dvo[0], dvo[1], nullptr,
              nullptr);
      }
      // without rotations FR and STIFR are zero, as enqueue_assemble leaves them
      if (!c->rot && dvo[2]) RG_CUDA(c, cudaMemsetAsync(dvo[2], 0, n3 * sizeof(double), c->stream));
      if (!c->rot && dvo[3]) RG_CUDA(c, cudaMemsetAsync(dvo[3], 0, n * sizeof(double), c->stream));
      RG_CUDA(c, cudaMemcpyAsync(c->h_time, c->d_time, sizeof(Time), cudaMemcpyDeviceToHost,
                                 c->stream));
      RG_CUDA(c, cudaStreamSynchronize(c->stream));
      if (dt2t) *dt2t = c->h_time->dt2t;
      if (neltst) *neltst = c->h_time->neltst;
      return RG_OK;
    }
  }
  double *of = st, *os = st + n3, *ofr = st + n3 + n, *osr = st + 2 * n3 + n;
  enqueue_assemble(c, f ? of : nullptr, stifn ? os : nullptr, fr ? ofr : nullptr,
                   stifr ? osr : nullptr);
  // a model without rotations has no moments: FR and STIFR come back zero
  if (!c->rot && fr) RG_CUDA(c, cudaMemsetAsync(ofr, 0, n3 * sizeof(double), c->stream));
  if (!c->rot && stifr) RG_CUDA(c, cudaMemsetAsync(osr, 0, n * sizeof(double), c->stream));
  {
    double *dst[4] = {f, stifn, fr, stifr};
    const double *src[4] = {of, os, ofr, osr};
    const size_t bytes[4] = {n3 * sizeof(double), n * sizeof(double), n3 * sizeof(double),
                             n * sizeof(double)};
    if (int r = copy_out(c, dst, src, bytes)) return r;
  }
  // the time-step record comes back through a pinned host copy
  RG_CUDA(c, cudaMemcpyAsync(c->h_time, c->d_time, sizeof(Time), cudaMemcpyDeviceToHost,
                             c->stream));
  RG_CUDA(c, cudaStreamSynchronize(c->stream));
  if (dt2t) *dt2t = c->h_time->dt2t;
  if (neltst) *neltst = c->h_time->neltst;
  return RG_OK;
}

// Whole device cycle with host node buffers: X, V (VR) uploaded as in
// rg_forint_step, one cycle of the captured graph (elements, PARITH/ON
// assembly, time step, nodal update), X, V (VR, D) and the cycle's step
// returned: written in place by download_nodes_kernel when every output is
// registered (or device) memory aligned to 16 bytes, else through the
// staging buffer by DMA copies.
int rg_cycle_host(rg_ctx *c, const double *x, const double *v, const double *vr,
                  double *x_out, double *v_out, double *vr_out, double *d_out, double *dt2) {
  if (!c) return RG_E_ARG;
  if (!c->finalized) return fail(c, RG_E_STATE, "rg_finalize first");
  if ((x == nullptr) != (v == nullptr))
    return fail(c, RG_E_ARG, "rg_cycle_host: give both X and V, or neither");
  if (c->timing) return fail(c, RG_E_STATE, "rg_cycle_host: event timing is on");
  RG_CUDA(c, cudaSetDevice(c->device));
  const int n = c->numnod;
  const int nb = (n + NODE_NT - 1) / NODE_NT;
  const size_t n3 = 3 * (size_t)n;
  double *st = c->d_stage;
  if (x) {
    const bool rot_in = vr && c->rot;
    const double *dx = device_view(x), *dv = device_view(v);
    const double *dvr = rot_in ? device_view(vr) : nullptr;
    if (!dx) {
      RG_CUDA(c, cudaMemcpyAsync(st, x, n3 * sizeof(double), cudaMemcpyHostToDevice, c->stream));
      dx = st;
    }
    if (!dv) {
      RG_CUDA(c, cudaMemcpyAsync(st + n3, v, n3 * sizeof(double), cudaMemcpyHostToDevice,
                                 c->stream));
      dv = st + n3;
    }
    if (rot_in && !dvr) {
      RG_CUDA(c, cudaMemcpyAsync(st + 2 * n3, vr, n3 * sizeof(double), cudaMemcpyHostToDevice,
                                 c->stream));
      dvr = st + 2 * n3;
    }
    launch_upload(c, dx, dv, dvr, -1.0);
    // the mixed form's FP64 element volumes follow the given coordinates
    if (c->prec == RG_PREC_MIXED && c->numels > 0)
      launch_hexa_prev_volume(c->h32, c->nv, c->d_time, c->stream);
  }
  RG_CUDA(c, cudaGraphLaunch(next_cycle_graph(c), c->stream));
  {
    // registered, 16-byte aligned outputs: one kernel writes them all in
    // place over the host link
    double *ho[4] = {x_out, v_out, vr_out, d_out};
    double *dvo[4] = {nullptr, nullptr, nullptr, nullptr};
    bool direct = true;
    bool any = false;
    for (int k = 0; k < 4 && direct; k++) {
      if (!ho[k]) continue;
      any = true;
      dvo[k] = const_cast<double *>(device_view(ho[k]));
      direct = dvo[k] && al16(dvo[k]);
    }
    if (direct && any) {
      download_nodes_kernel<<<(n + XFER_NT - 1) / XFER_NT, XFER_NT, 0, c->stream>>>(
          c->nv, c->prec == RG_PREC_MIXED ? 1 : 0, dvo[0], dvo[1], c->rot ? dvo[2] : nullptr,
          dvo[3]);
      if (vr_out && !c->rot) RG_CUDA(c, cudaMemsetAsync(dvo[2], 0, n3 * sizeof(double), c->stream));
      RG_CUDA(c, cudaMemcpyAsync(c->h_time, c->d_time, sizeof(Time), cudaMemcpyDeviceToHost,
                                 c->stream));
      RG_CUDA(c, cudaStreamSynchronize(c->stream));
      RG_CUDA(c, cudaGetLastError());
      if (dt2) *dt2 = c->h_time->dt2;
      return RG_OK;
    }
  }
  struct {
    double *dst;
    dbl4 *src;
  } items[4] = {{x_out, c->nv.X4}, {v_out, c->nv.V4}, {vr_out, c->rot ? c->nv.VR4 : nullptr},
                {d_out, c->nv.D4}};
  // other outputs go through staging slices and a DMA copy each (a copy
  // engine writes host memory faster than per-node kernel stores: 0.534 vs
  // 0.443 ms per crash-box cycle)
  double *dst[4] = {nullptr, nullptr, nullptr, nullptr};
  const double *src[4] = {nullptr, nullptr, nullptr, nullptr};
  size_t bytes[4] = {0, 0, 0, 0};
  for (int k = 0; k < 4; k++) {
    if (!items[k].dst) continue;
    double *sk = st + k * n3;  // 12 * numnod doubles of staging: one slice per array
    if (!items[k].src)
      RG_CUDA(c, cudaMemsetAsync(sk, 0, n3 * sizeof(double), c->stream));
    else if (items[k].src == c->nv.D4 && c->prec == RG_PREC_MIXED)
      unpack_disp_kernel<<<nb, NODE_NT, 0, c->stream>>>(n, c->nv.X4, c->nv.D4, sk);
    else
      unpack3_kernel<<<nb, NODE_NT, 0, c->stream>>>(n, items[k].src, sk);
    dst[k] = items[k].dst;
    src[k] = sk;
    bytes[k] = n3 * sizeof(double);
  }
  if (int r = copy_out(c, dst, src, bytes)) return r;
  RG_CUDA(c, cudaMemcpyAsync(c->h_time, c->d_time, sizeof(Time), cudaMemcpyDeviceToHost,
                             c->stream));
  RG_CUDA(c, cudaStreamSynchronize(c->stream));
  RG_CUDA(c, cudaGetLastError());
  if (dt2) *dt2 = c->h_time->dt2;
  return RG_OK;
}

int rg_download_nodes(rg_ctx *c, double *x, double *v, double *d, double *vr) {
  if (!c) return RG_E_ARG;
  if (!c->finalized) return fail(c, RG_E_STATE, "rg_finalize first");
  RG_CUDA(c, cudaSetDevice(c->device));
  const int n = c->numnod;
  const int nb = (n + NODE_NT - 1) / NODE_NT;
  double *st = c->d_stage;
  struct {
    double *dst;
    dbl4 *src;
  } items[4] = {{x, c->nv.X4}, {v, c->nv.V4}, {d, c->nv.D4}, {vr, c->nv.VR4}};
  for (auto &it : items) {
    if (!it.dst) continue;
    if (!it.src) {
      std::fill(it.dst, it.dst + 3 * (size_t)n, 0.0);
      continue;
    }
    if (it.src == c->nv.D4 && c->prec == RG_PREC_MIXED)
      unpack_disp_kernel<<<nb, NODE_NT, 0, c->stream>>>(n, c->nv.X4, c->nv.D4, st);
    else
      unpack3_kernel<<<nb, NODE_NT, 0, c->stream>>>(n, it.src, st);
    RG_CUDA(c, cudaMemcpyAsync(it.dst, st, 3 * (size_t)n * sizeof(double), cudaMemcpyDeviceToHost,
                               c->stream));
    RG_CUDA(c, cudaStreamSynchronize(c->stream));
  }
  return RG_OK;
}

int rg_download_forces(rg_ctx *c, double *f, double *stifn, double *fr) {
  if (!c) return RG_E_ARG;
  if (!c->finalized) return fail(c, RG_E_STATE, "rg_finalize first");
  RG_CUDA(c, cudaSetDevice(c->device));
  const int n = c->numnod;
  double *st = c->d_stage;
  enqueue_assemble(c, st, st + 3 * (size_t)n, st + 4 * (size_t)n, st + 7 * (size_t)n);
  if (f)
    RG_CUDA(c, cudaMemcpyAsync(f, st, 3 * (size_t)n * sizeof(double), cudaMemcpyDeviceToHost, c->stream));
  if (stifn)
    RG_CUDA(c, cudaMemcpyAsync(stifn, st + 3 * (size_t)n, (size_t)n * sizeof(double),
                               cudaMemcpyDeviceToHost, c->stream));
  if (fr)
    RG_CUDA(c, cudaMemcpyAsync(fr, st + 4 * (size_t)n, 3 * (size_t)n * sizeof(double),
                               cudaMemcpyDeviceToHost, c->stream));
  RG_CUDA(c, cudaStreamSynchronize(c->stream));
  return RG_OK;
}

int rg_download_hexa_state(rg_ctx *c, int which, double *out) {
  if (!c || !out) return RG_E_ARG;
  if (!c->finalized) return fail(c, RG_E_STATE, "rg_finalize first");
  RG_CUDA(c, cudaStreamSynchronize(c->stream));  // results of enqueued cycles
  const int ne = c->numels;
  if (ne == 0) return RG_OK;
  RG_CUDA(c, cudaSetDevice(c->device));
  RG_CUDA(c, cudaStreamSynchronize(c->stream));
  const bool f64 = c->prec == RG_PREC_FP64;
  const void *src = nullptr;
  bool isdouble = false;
  size_t cnt = ne;
  switch (which) {
    case 0: src = f64 ? (void *)c->h64.sig : (void *)c->h32.sig; cnt = 6 * (size_t)ne; break;
    case 1: src = f64 ? c->h64.eint : c->h32.eint; isdouble = true; break;
    case 2: src = f64 ? c->h64.rho : c->h32.rho; isdouble = true; break;
    case 3: src = f64 ? (void *)c->h64.qvis : (void *)c->h32.qvis; break;
    case 4: src = f64 ? (void *)c->h64.off : (void *)c->h32.off; break;
    case 5: src = f64 ? (void *)c->h64.pla : (void *)c->h32.pla; break;
    case 6: src = f64 ? (void *)c->h64.epsd : (void *)c->h32.epsd; break;
    case 7: src = f64 ? c->h64.vol0 : c->h32.vol0; isdouble = true; break;
    case 8: src = f64 ? c->h64.ehou : c->h32.ehou; isdouble = true; break;
    default: return fail(c, RG_E_ARG, "unknown hexa state index");
  }
  if (!f64 && which == 2) {
    // mixed form keeps the element volume: RHO = RHO0 * VOL0 / VOL
    std::vector<double> v(ne), v0(ne);
    RG_CUDA(c, cudaMemcpy(v.data(), c->h32.rho, ne * sizeof(double), cudaMemcpyDeviceToHost));
    RG_CUDA(c, cudaMemcpy(v0.data(), c->h32.vol0, ne * sizeof(double), cudaMemcpyDeviceToHost));
    for (auto &g : c->hg)
      for (int i = 0; i < g.nel; i++) {
        const int e = g.P.nft + i;
        out[e] = g.P.rho0 * (v0[e] / v[e]);
      }
  } else if (f64 || isdouble) {
    RG_CUDA(c, cudaMemcpy(out, src, cnt * sizeof(double), cudaMemcpyDeviceToHost));
  } else {
    std::vector<float> tmp(cnt);
    RG_CUDA(c, cudaMemcpy(tmp.data(), src, cnt * sizeof(float), cudaMemcpyDeviceToHost));
    for (size_t i = 0; i < cnt; i++) out[i] = tmp[i];
  }
  return RG_OK;
}

int rg_download_shell_state(rg_ctx *c, int which, double *out) {
  if (!c || !out) return RG_E_ARG;
  if (!c->finalized) return fail(c, RG_E_STATE, "rg_finalize first");
  RG_CUDA(c, cudaStreamSynchronize(c->stream));  // results of enqueued cycles
  RG_CUDA(c, cudaSetDevice(c->device));
  RG_CUDA(c, cudaStreamSynchronize(c->stream));
  std::string why;
  const int r = shell_download(c->shells, c->prec, which, out, why);
  if (r) return fail(c, r, why);
  return RG_OK;
}

int rg_get_time(rg_ctx *c, double *tt, double *dt1, double *dt2, int *ncycle, int *neltst) {
  if (!c) return RG_E_ARG;
  if (!c->finalized) return fail(c, RG_E_STATE, "rg_finalize first");
  RG_CUDA(c, cudaSetDevice(c->device));
  Time t;
  RG_CUDA(c, cudaMemcpyAsync(&t, c->d_time, sizeof(Time), cudaMemcpyDeviceToHost, c->stream));
  RG_CUDA(c, cudaStreamSynchronize(c->stream));
  if (tt) *tt = t.tt;
  if (dt1) *dt1 = t.dt1;
  if (dt2) *dt2 = t.dt2;
  if (ncycle) *ncycle = t.ncycle;
  if (neltst) *neltst = t.neltst;
  return RG_OK;
}

int rg_energy(rg_ctx *c, double *eint, double *ekin, double *ekinr, double *ehour) {
  if (!c) return RG_E_ARG;
  if (!c->finalized) return fail(c, RG_E_STATE, "rg_finalize first");
  RG_CUDA(c, cudaSetDevice(c->device));
  double *part = c->d_epart;
  double *out = c->d_stage;  // 4 doubles
  const bool f64 = c->prec == RG_PREC_FP64;
  const double *ei = f64 ? c->h64.eint : c->h32.eint;
  const double *v0 = f64 ? c->h64.vol0 : c->h32.vol0;
  const double *eh = f64 ? c->h64.ehou : c->h32.ehou;
  energy_kernel<double><<<EN_BLOCKS, EN_NT, 0, c->stream>>>(c->numels, ei, v0, eh, c->nv,
                                                           c->rot ? 1 : 0, part);
  // shell element energies (fixed order) go to out[4..5] via the shell module
  double *extra = c->d_stage + 8;
  int nextra = shell_energy_enqueue(c->shells, c->prec, extra, c->stream);
  energy_final<<<1, EN_NT, 0, c->stream>>>(part, nextra, extra, out);
  double h[4];
  RG_CUDA(c, cudaMemcpyAsync(h, out, 4 * sizeof(double), cudaMemcpyDeviceToHost, c->stream));
  RG_CUDA(c, cudaStreamSynchronize(c->stream));
  if (eint) *eint = h[0];
  if (ehour) *ehour = h[1];
  if (ekin) *ekin = h[2];
  if (ekinr) *ekinr = h[3];
  return RG_OK;
}

// Energy balance of the listing's cycle line (ECRIT, engine/source/output/
// ecrit.F:373-520): ENTOT = IE + KE + KE-R, ERROR = ENTOT / (ENTOT0 +
// WFEXT) - 1 (in %, clamped to +-99), mass error against the cycle-0 mass.
int rg_energy_balance(rg_ctx *c, double *out, int n) {
  if (!c || !out || n < 0) return RG_E_ARG;
  if (!c->finalized) return fail(c, RG_E_STATE, "rg_finalize first");
  double ei, ek, ekr, eh;
  int r = rg_energy(c, &ei, &ek, &ekr, &eh);
  if (r) return r;
  double *part = c->d_epart + 4 * EN_BLOCKS;
  double *dout = c->d_stage + 16;  // 5 doubles (staging holds >= 12 numnod + 16)
  balance_kernel<<<EN_BLOCKS, EN_NT, 0, c->stream>>>(c->nv, part);
  balance_final<<<1, EN_NT, 0, c->stream>>>(part, dout);
  double nb[5];
  RG_CUDA(c, cudaMemcpyAsync(nb, dout, 5 * sizeof(double), cudaMemcpyDeviceToHost, c->stream));
  RG_CUDA(c, cudaMemcpyAsync(c->h_time, c->d_time, sizeof(Time), cudaMemcpyDeviceToHost,
                             c->stream));
  RG_CUDA(c, cudaStreamSynchronize(c->stream));
  const double entot = ei + ek + ekr;
  const double den = c->entot0 + nb[4];
  double err = 0.0;
  if (std::fabs(den) > RG_EM20) err = std::fmax(-99.0, std::fmin(99.0, (entot / den - 1.0) * 100.0));
  const double mass0 = c->finalized && c->mass0 > 0.0 ? c->mass0 : nb[0];
  const double emass = (nb[0] - mass0) / std::fmax(mass0, RG_EM20);
  const double b[13] = {c->h_time->tt, ei, ek, ekr, eh, nb[4], entot, err, nb[0], emass,
                        nb[1], nb[2], nb[3]};
  for (int k = 0; k < n && k < 13; k++) out[k] = b[k];
  return RG_OK;
}

int rg_part_sums_due(rg_ctx *c) {
  if (!c) return RG_E_ARG;
  if (!c->finalized) return fail(c, RG_E_STATE, "rg_finalize first");
  RG_CUDA(c, cudaSetDevice(c->device));
  if (int r = parts_prepare(c)) return r;
  if (!c->gexec_parts) {
    // the cycle graph with the part sums between the element pass and the
    // nodal update, captured once
    RG_CUDA(c, cudaStreamSynchronize(c->stream));
    RG_CUDA(c, cudaStreamBeginCapture(c->stream, cudaStreamCaptureModeThreadLocal));
    enqueue_cycle(c, true);
    cudaError_t ce = cudaStreamEndCapture(c->stream, &c->graph_parts);
    if (ce != cudaSuccess)
      return fail(c, RG_E_CUDA, std::string("graph capture: ") + cudaGetErrorString(ce));
    RG_CUDA(c, cudaGraphInstantiate(&c->gexec_parts, c->graph_parts, 0));
  }
  c->parts_due = true;
  return RG_OK;
}

int rg_status(rg_ctx *c) {
  if (!c) return RG_E_ARG;
  if (!c->finalized) return 0;
  cudaSetDevice(c->device);
  int s = 0;
  if (cudaMemcpyAsync(&s, c->d_status, sizeof(int), cudaMemcpyDeviceToHost, c->stream) != cudaSuccess)
    return RG_E_CUDA;
  if (cudaMemsetAsync(c->d_status, 0, sizeof(int), c->stream) != cudaSuccess) return RG_E_CUDA;
  if (cudaStreamSynchronize(c->stream) != cudaSuccess) return RG_E_CUDA;
  return s;
}

// ---- checkpoint / restart ------------------------------------------------
// A snapshot is every device allocation of the context, in allocation order,
// behind a header that ties it to the model it came from (counts, precision,
// allocation sizes).  All of the model's state lives in those allocations
// (nodes, element and point state, skyline slots, the time-step record, link
// switches, status word), so restoring them resumes the run bit for bit.
namespace {
struct SnapHeader {
  char magic[8];
  unsigned long long nalloc, payload, layout;
  int numnod, numels, numelc, prec;
};
unsigned long long snap_layout(const rg_ctx *c) {
  // FNV-1a over the allocation sizes
  unsigned long long h = 1469598103934665603ull;
  for (size_t b : c->alloc_bytes) {
    h ^= (unsigned long long)b;
    h *= 1099511628211ull;
  }
  return h;
}
unsigned long long snap_payload(const rg_ctx *c) {
  unsigned long long t = 0;
  for (size_t b : c->alloc_bytes) t += b;
  return t;
}
void snap_header(const rg_ctx *c, SnapHeader &h) {
  std::memset(&h, 0, sizeof(h));
  std::memcpy(h.magic, "RGSNAP01", 8);
  h.nalloc = c->allocs.size();
  h.payload = snap_payload(c);
  h.layout = snap_layout(c);
  h.numnod = c->numnod;
  h.numels = c->numels;
  h.numelc = c->shells.numelc;
  h.prec = c->prec;
}
}  // namespace

int rg_snapshot_size(rg_ctx *c, unsigned long long *bytes) {
  if (!c || !bytes) return RG_E_ARG;
  if (!c->finalized) return fail(c, RG_E_STATE, "rg_finalize first");
  *bytes = sizeof(SnapHeader) + snap_payload(c);
  return RG_OK;
}

int rg_snapshot(rg_ctx *c, void *buf, unsigned long long bytes) {
  if (!c || !buf) return RG_E_ARG;
  if (!c->finalized) return fail(c, RG_E_STATE, "rg_finalize first");
  const unsigned long long need = sizeof(SnapHeader) + snap_payload(c);
  if (bytes < need) return fail(c, RG_E_ARG, "rg_snapshot: buffer smaller than rg_snapshot_size");
  RG_CUDA(c, cudaSetDevice(c->device));
  SnapHeader h;
  snap_header(c, h);
  std::memcpy(buf, &h, sizeof(h));
  char *q = (char *)buf + sizeof(h);
  for (size_t i = 0; i < c->allocs.size(); i++) {
    RG_CUDA(c, cudaMemcpyAsync(q, c->allocs[i], c->alloc_bytes[i], cudaMemcpyDeviceToHost,
                               c->stream));
    q += c->alloc_bytes[i];
  }
  RG_CUDA(c, cudaStreamSynchronize(c->stream));
  return RG_OK;
}

int rg_restore(rg_ctx *c, const void *buf, unsigned long long bytes) {
  if (!c || !buf) return RG_E_ARG;
  if (!c->finalized) return fail(c, RG_E_STATE, "rg_finalize first");
  if (bytes < sizeof(SnapHeader)) return fail(c, RG_E_ARG, "rg_restore: buffer too small");
  SnapHeader h, mine;
  std::memcpy(&h, buf, sizeof(h));
  snap_header(c, mine);
  if (std::memcmp(h.magic, mine.magic, 8) != 0)
    return fail(c, RG_E_ARG, "rg_restore: not a snapshot of this library");
  if (h.nalloc != mine.nalloc || h.payload != mine.payload || h.layout != mine.layout ||
      h.numnod != mine.numnod || h.numels != mine.numels || h.numelc != mine.numelc ||
      h.prec != mine.prec)
    return fail(c, RG_E_ARG, "rg_restore: snapshot of a different model or precision");
  if (bytes < sizeof(SnapHeader) + h.payload)
    return fail(c, RG_E_ARG, "rg_restore: truncated snapshot");
  RG_CUDA(c, cudaSetDevice(c->device));
  const char *q = (const char *)buf + sizeof(h);
  for (size_t i = 0; i < c->allocs.size(); i++) {
    RG_CUDA(c, cudaMemcpyAsync(c->allocs[i], q, c->alloc_bytes[i], cudaMemcpyHostToDevice,
                               c->stream));
    q += c->alloc_bytes[i];
  }
  RG_CUDA(c, cudaStreamSynchronize(c->stream));
  c->parts_valid = false;  // the part sums were of a cycle before the restore
  return RG_OK;
}

int rg_info(rg_ctx *c, int *numnod, int *numels, int *numelc, int *lsky,
            unsigned long long *device_bytes) {
  if (!c) return RG_E_ARG;
  if (numnod) *numnod = c->numnod;
  if (numels) *numels = c->numels;
  if (numelc) *numelc = shell_numelc(c->shells);
  if (lsky) *lsky = c->lsky;
  if (device_bytes) *device_bytes = c->dev_bytes;
  return RG_OK;
}

int rg_set_timing(rg_ctx *c, int on) {
  if (!c) return RG_E_ARG;
  c->timing = on != 0;
  return RG_OK;
}

int rg_time_cycles(rg_ctx *c, int ncycle, double *ms) {
  if (!c || !ms) return RG_E_ARG;
  if (!c->finalized) return fail(c, RG_E_STATE, "rg_finalize first");
  RG_CUDA(c, cudaSetDevice(c->device));
  RG_CUDA(c, cudaEventRecord(c->ev[5], c->stream));
  for (int i = 0; i < ncycle; i++) RG_CUDA(c, cudaGraphLaunch(c->gexec, c->stream));
  RG_CUDA(c, cudaEventRecord(c->ev[6], c->stream));
  RG_CUDA(c, cudaEventSynchronize(c->ev[6]));
  float f = 0;
  RG_CUDA(c, cudaEventElapsedTime(&f, c->ev[5], c->ev[6]));
  *ms = f;
  return RG_OK;
}

int rg_time_cycles_cold(rg_ctx *c, int ncycle, unsigned long long flush_bytes, double *ms) {
  if (!c || !ms || ncycle < 0) return RG_E_ARG;
  if (!c->finalized) return fail(c, RG_E_STATE, "rg_finalize first");
  RG_CUDA(c, cudaSetDevice(c->device));
  if (flush_bytes > c->flush_bytes) {
    if (c->d_flush) RG_CUDA(c, cudaFree(c->d_flush));
    c->d_flush = nullptr;
    c->flush_bytes = 0;
    RG_CUDA(c, cudaMalloc(&c->d_flush, flush_bytes));
    c->flush_bytes = flush_bytes;
  }
  double tot = 0.0;
  for (int i = 0; i < ncycle; i++) {
    // overwrite a buffer larger than L2 so the cycle starts from cold L2
    if (flush_bytes)
      RG_CUDA(c, cudaMemsetAsync(c->d_flush, i & 0xff, flush_bytes, c->stream));
    RG_CUDA(c, cudaEventRecord(c->ev[5], c->stream));
    RG_CUDA(c, cudaGraphLaunch(c->gexec, c->stream));
    RG_CUDA(c, cudaEventRecord(c->ev[6], c->stream));
    RG_CUDA(c, cudaEventSynchronize(c->ev[6]));
    float f = 0;
    RG_CUDA(c, cudaEventElapsedTime(&f, c->ev[5], c->ev[6]));
    tot += f;
  }
  *ms = tot;
  return RG_OK;
}

int rg_kernel_times(rg_ctx *c, double *ms4) {
  if (!c || !ms4) return RG_E_ARG;
  for (int k = 0; k < 4; k++) ms4[k] = c->ktime[k];
  return RG_OK;
}

}  // extern "C"
