// Device-side data structures shared by the kernels of the explicit cycle.
//
// Layout in HBM (structure of arrays, one context = one model):
//   nodes  : dbl4 X4[n] = {x, y, z, MS},  dbl4 V4[n] = {vx, vy, vz, code}
//            dbl4 D4[n] = {dx, dy, dz, 0}; shells add VR4 = {vrx, vry, vrz, IN}
//            -- one 32-byte sector per node record, read with two 16-byte loads.
//   hexa   : int32 NC[8][NE] and IADS[8][NE] (0-based), state arrays
//            SIG[6][NE], EINT, RHO, QVIS, OFF, VOL0, PLA, EPSD, EHOU.
//   slots  : FSKY[LSKY] = {fx, fy, fz, sti} (dbl4 in the FP64 form, float4
//            in the mixed form), FSKYR[LSKY] = {mx, my, mz, stir} for shells.
//   skyline: ADSKY[n+1] (0-based) -- node n sums slots ADSKY[n]..ADSKY[n+1]-1
//            in that order, the PARITH/ON order of ASSPAR4.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include "rg_constants.h"

namespace rg {

// 32-byte aligned node / slot records (one DRAM sector each).
typedef double4_32a dbl4;
__host__ __device__ __forceinline__ dbl4 mk4(double x, double y, double z,
                                             double w) {
  dbl4 t;
  t.x = x;
  t.y = y;
  t.z = z;
  t.w = w;
  return t;
}

// RESOL time-step scalars, resident on the device so that cycles chain
// without host round trips (engine/source/engine/resol.F:2721-2722, 6123,
// 6352, 6494-6497).
struct Time {
  double tt, dt1, dt2, dt12, dt2old, dtmx;
  double dt2t;       // element/nodal minimum of the current cycle
  double dtmin;      // error threshold (0 = none)
  int ncycle, neltst, status, pad;
};

// FP32 copy of a node position as an unevaluated sum hi + lo of two floats
// (mixed form): the difference of two nodes' copies keeps FP32 relative
// precision however far the nodes are from the origin.
struct __align__(32) F8 {
  float hx, hy, hz, pad0, lx, ly, lz, pad1;  // pad0 = 1/MS, pad1 = 1/IN (FP32)
};

struct NodeView {
  dbl4 *X4;   // x y z 1/MS      (1/MS = 0 when MS <= 0)
  dbl4 *V4;   // vx vy vz code(as double)
  dbl4 *D4;   // dx dy dz MS (mixed form: x0 y0 z0 MS, D = X - X0)
  dbl4 *VR4;  // vrx vry vrz 1/IN (shell models only)
  dbl4 *DR4;  // - - - IN          (shell models only)
  F8 *XF;     // mixed form: FP32 hi/lo position copies
  float4 *VF;   // mixed form: FP32 velocity copies
  float4 *VRF;  // mixed form: FP32 rotational velocity copies (shells)
  double *wext; // external work of the rigid walls per node (null without walls)
  int numnod;
};

// Per-block partial minimum of the element time step.
struct DtPartials {
  double *dt;
  int *el;  // user id of the element attaining it (-1 none)
};

// Time-step reduction fused into the element kernels, in two levels: the
// block completing the last partial of a group of DT_GROUP partials reduces
// that group; the block completing the last group (counted across all element
// launches of the cycle) reduces the group minima and applies the RESOL logic.
struct DtFinish {
  unsigned *ctr;     // [1 + ngroups]: groups done, blocks done per group
  double *gdt;       // [ngroups] group minima (64 partials per group)
  int *gel;
  int nparts;        // partials of the whole cycle
  int advance;       // 0: record DT2T / NELTST only (FORINT-level call)
  const int *ngl;    // element order key -> user id
};
constexpr int DT_GROUP = 64;  // partials per first-level group

__device__ __forceinline__ dbl4 ld4(const dbl4 *__restrict__ p) { return *p; }
__device__ __forceinline__ void st4(dbl4 *__restrict__ p, dbl4 v) { *p = v; }
__device__ __forceinline__ F8 ldF8(const F8 *__restrict__ p) { return *p; }
__device__ __forceinline__ float4 ldf4(const float4 *__restrict__ p) { return __ldg(p); }

// Sum of one double per thread over a block of NT threads (a power of two)
// in a fixed order: a shared-memory tree, the same additions every time.
// The result is valid in thread 0.
template <int NT>
__device__ __forceinline__ double block_sum_fixed(double v, double *sh) {
  sh[threadIdx.x] = v;
  __syncthreads();
  for (int o = NT / 2; o > 0; o >>= 1) {
    if ((int)threadIdx.x < o) sh[threadIdx.x] += sh[threadIdx.x + o];
    __syncthreads();
  }
  const double r = sh[0];
  __syncthreads();
  return r;
}

// Asynchronous global -> shared copies of one thread's own values (sm_80+
// cp.async): issued early, they fetch element state while the thread
// computes, without holding registers; cp_async_wait_all() makes them
// visible to the issuing thread.
__device__ __forceinline__ void cp_async4(void *smem, const void *gmem) {
  const unsigned s = (unsigned)__cvta_generic_to_shared(smem);
  asm volatile("cp.async.ca.shared.global [%0], [%1], 4;\n" ::"r"(s), "l"(gmem) : "memory");
}
__device__ __forceinline__ void cp_async8(void *smem, const void *gmem) {
  const unsigned s = (unsigned)__cvta_generic_to_shared(smem);
  asm volatile("cp.async.ca.shared.global [%0], [%1], 8;\n" ::"r"(s), "l"(gmem) : "memory");
}
// 16 bytes, both addresses 16-byte aligned (a lane's share of a warp's
// cooperative copy of contiguous data)
__device__ __forceinline__ void cp_async16(void *smem, const void *gmem) {
  const unsigned s = (unsigned)__cvta_generic_to_shared(smem);
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(s), "l"(gmem) : "memory");
}
__device__ __forceinline__ void cp_async_commit() {
  asm volatile("cp.async.commit_group;\n" ::: "memory");
}
__device__ __forceinline__ void cp_async_wait_all() {
  asm volatile("cp.async.wait_all;\n" ::: "memory");
}

// Block-level (min dt, element) reduction; ties keep the larger element
// order key (the last element attaining the minimum in sequential order).
__device__ __forceinline__ void dt_pair_min(double &d, int &k, double d2,
                                            int k2) {
  if (d2 < d || (d2 == d && k2 > k)) {
    d = d2;
    k = k2;
  }
}

template <typename T>
__device__ __forceinline__ void dt_pair_min_t(T &d, int &k, T d2, int k2) {
  if (d2 < d || (d2 == d && k2 > k)) {
    d = d2;
    k = k2;
  }
}

// Block minimum of (dt, key) in the element arithmetic type T; the block's
// result is stored as FP64.
template <int NT, typename T = double>
__device__ __forceinline__ void block_dt_min(T d, int k, double *out_d,
                                             int *out_k) {
  __shared__ T sd[NT / 32];
  __shared__ int sk[NT / 32];
  for (int o = 16; o > 0; o >>= 1) {
    T d2 = __shfl_down_sync(0xffffffffu, d, o);
    int k2 = __shfl_down_sync(0xffffffffu, k, o);
    dt_pair_min_t(d, k, d2, k2);
  }
  const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
  if (l == 0) {
    sd[w] = d;
    sk[w] = k;
  }
  __syncthreads();
  if (w == 0) {
    d = l < NT / 32 ? sd[l] : (T)RG_EP30;
    k = l < NT / 32 ? sk[l] : -1;
    for (int o = 16; o > 0; o >>= 1) {
      T d2 = __shfl_down_sync(0xffffffffu, d, o);
      int k2 = __shfl_down_sync(0xffffffffu, k, o);
      dt_pair_min_t(d, k, d2, k2);
    }
    if (l == 0) {
      *out_d = (double)d;
      *out_k = k;
    }
  }
}

// Hexa group parameters (one launch per group of identical material and
// property; values taken from PM / GEO / mat_param like the reference).
struct HexaParams {
  int nft, nel;            // element range in the hexa arrays
  int mtn;                 // 1 = LAW1, 2 = LAW2
  int part_off;            // first dt-partial slot of this launch
  double rho0, g, c1;      // PM(1), PM(22), PM(32)
  double qh, qa, qb, vns1, vns2;  // GEO(13..17)
  double dtfac;            // DTFAC1(1)
  double ssp1;             // sqrt((1.333 G + C1) / RHO0): sound speed at OFF = 1
  int has_cns;             // numerical damping GEO(16..17) set
  int jcvt;                // 0: Jaumann rate (Iframe=1), 1: co-rotational frame
  // LAW2 Johnson-Cook (mat_param%uparam / iparam)
  double ca, cb, cn, epmx, sigm0, cc, epdr, asrate, z3;
  int icc, vp, israte;
  int nodadt;              // nodal time step: the element gives STI only
  double inv_rho0;         // 1/RHO0 (group constant)
  // FP32 copies of the coefficients above (the same round-to-nearest
  // conversion, done once on the host) for the mixed form, and the two
  // branch flags CC /= 0, N == 1 evaluated on the FP64 values
  struct {
    float rho0, g, c1, qh, qa, qb, vns1, vns2, dtfac, ssp1;
    float ca, cb, cn, epmx, sigm0, cc, epdr, asrate;
    int cc_nz, cn_one;
  } f;
};

inline void hexa_params_mirror(HexaParams &P) {
  P.inv_rho0 = 1.0 / P.rho0;
  P.f.rho0 = (float)P.rho0;
  P.f.g = (float)P.g;
  P.f.c1 = (float)P.c1;
  P.f.qh = (float)P.qh;
  P.f.qa = (float)P.qa;
  P.f.qb = (float)P.qb;
  P.f.vns1 = (float)P.vns1;
  P.f.vns2 = (float)P.vns2;
  P.f.dtfac = (float)P.dtfac;
  P.f.ssp1 = (float)P.ssp1;
  P.f.ca = (float)P.ca;
  P.f.cb = (float)P.cb;
  P.f.cn = (float)P.cn;
  P.f.epmx = (float)P.epmx;
  P.f.sigm0 = (float)P.sigm0;
  P.f.cc = (float)P.cc;
  P.f.epdr = (float)P.epdr;
  P.f.asrate = (float)P.asrate;
  P.f.cc_nz = P.cc != 0.0;
  P.f.cn_one = P.cn == 1.0;
}

// coefficient in the element type: the FP64 value or its FP32 copy
template <typename R>
__device__ __forceinline__ R pcoef(double d, float f) {
  if constexpr (sizeof(R) == 8)
    return d;
  else
    return f;
}
#define PC(name) pcoef<R>(P.name, P.f.name)

template <typename ER>
struct HexaArrays {
  int ne;                  // total hexa count (SoA stride)
  const int *nc;           // [8][ne] 0-based node numbers
  const int *iads;         // [8][ne] 0-based slots
  const int *ngl;          // [ne] user ids
  ER *sig;                 // [6][ne]
  double *eint;            // [ne]   (FP64 in both forms: energy accumulator)
  double *rho;             // [ne]   (FP64 in both forms: volume history)
  ER *qvis;                // [ne]
  ER *off;                 // [ne]   OFFG
  double *vol0;            // [ne]
  ER *pla, *epsd;          // [ne]   LAW2
  double *ehou;            // [ne]   accumulated hourglass energy
};

template <typename ER>
struct SlotT;
template <>
struct SlotT<double> {
  typedef dbl4 type;
};
template <>
struct SlotT<float> {
  typedef float4 type;
};

}  // namespace rg
