#pragma once
// Nodal phase of the explicit cycle and the RESOL time-step logic as device
// functions, shared by the single-model kernels (rg_api.cu) and the batched
// persistent kernel (rg_batch.cu).
#include "../../include/rg_api.h"
#include "rg_bits.h"
#include "rg_device.cuh"

namespace rg {

// node code: bits below RG_LINK_SHIFT hold the boundary code, the bits above
// the 1-based rigid-link index
constexpr int RG_LINK_SHIFT = 8;

#ifndef RG_NODE_EARLY
#define RG_NODE_EARLY 1
#endif

// ---------------------------------------------------------------------------
// Node update: ASSPAR4 (asspar4.F:165-180) fixed-order slot sums, ACCELE
// (accele.F:66-78), BCS10/BCS1V (bcs10.F:31), planar rigid wall, VELOCITY
// (velocity.F:59-75), DEPLA (displacement.F:68-100).  The update arithmetic
// is written with explicit round-to-nearest multiply / add so that no
// multiply-add is fused and each node's result does not depend on the
// launch configuration.
// ---------------------------------------------------------------------------
// (pad0, pad1 = 1/MS, 1/IN in FP32 for the mixed node update: set by the
// callers)
__device__ __forceinline__ F8 split_hilo(double x, double y, double z) {
  F8 c;
  c.hx = __double2float_rn(x);
  c.hy = __double2float_rn(y);
  c.hz = __double2float_rn(z);
  c.lx = __double2float_rn(x - (double)c.hx);
  c.ly = __double2float_rn(y - (double)c.hy);
  c.lz = __double2float_rn(z - (double)c.hz);
  c.pad0 = c.pad1 = 0.f;
  return c;
}

// (hi, lo) += d in FP32, exact two-sum then renormalisation (Knuth's
// TwoSum, Dekker's fast renormalisation): hi + lo keeps about 48 bits.
__device__ __forceinline__ void ff_add(float &hi, float &lo, const float d) {
  const float s = __fadd_rn(hi, d);
  const float bb = __fsub_rn(s, hi);
  const float err = __fadd_rn(__fsub_rn(hi, __fsub_rn(s, bb)), __fsub_rn(d, bb));
  const float l = __fadd_rn(lo, err);
  const float h2 = __fadd_rn(s, l);
  lo = __fsub_rn(l, __fsub_rn(h2, s));
  hi = h2;
}

// Rigid wall record on the device: P0 (3), unit normal N (3) in FP64, then
// the same six values in FP32 (packed in the last three doubles) for the
// FP32 screen of the wall test.
constexpr int RG_WALL_STRIDE = 9;

// FP32 screen of the sliding-wall test: true when the predicted distance
// DP = (X - P0).N + DT2 (V + A DT12).N of the node is positive for certain,
// so that the FP64 test below would leave the node alone.  Every FP32 value
// here is within a few units of 2^-24 of the FP64 value it stands for, so
// the estimate is off by less than 2^-20 of MAG (the sum of the magnitudes
// it is formed from); the screen asks for a margin of 2^-14 MAG and sends
// every closer node (and any NaN or overflow) to the FP64 test.
__device__ __forceinline__ bool wall_clear(const double *__restrict__ W, const dbl4 &x,
                                           const dbl4 &v, const double a0, const double a1,
                                           const double a2, const double dt12,
                                           const double dt2) {
  const float *Wf = (const float *)(W + 6);
  const float d12 = narrow_f64(dt12), d2 = narrow_f64(dt2);
  const float nx = Wf[3], ny = Wf[4], nz = Wf[5];
  const float ax = narrow_f64(a0), ay = narrow_f64(a1), az = narrow_f64(a2);
  const float ux = narrow_f64(v.x), uy = narrow_f64(v.y), uz = narrow_f64(v.z);
  const float vx = fmaf(ax, d12, ux), vy = fmaf(ay, d12, uy), vz = fmaf(az, d12, uz);
  const float px = narrow_f64(x.x), py = narrow_f64(x.y), pz = narrow_f64(x.z);
  const float vn = fmaf(vz, nz, fmaf(vy, ny, vx * nx));
  const float dp0 = fmaf(pz - Wf[2], nz, fmaf(py - Wf[1], ny, (px - Wf[0]) * nx));
  const float dp = fmaf(d2, vn, dp0);
  const float mx = (fabsf(px) + fabsf(Wf[0]) + d2 * (fabsf(ux) + fabsf(ax) * d12)) * fabsf(nx);
  const float my = (fabsf(py) + fabsf(Wf[1]) + d2 * (fabsf(uy) + fabsf(ay) * d12)) * fabsf(ny);
  const float mz = (fabsf(pz) + fabsf(Wf[2]) + d2 * (fabsf(uz) + fabsf(az) * d12)) * fabsf(nz);
  return dp > 0x1p-14f * (mx + my + mz);
}

// L2-coherent loads (ld.global.cg): used where the data was written by other
// blocks earlier in the same launch (batched persistent kernel).
__device__ __forceinline__ dbl4 ldcg4(const dbl4 *p) {
  const double2 a = __ldcg((const double2 *)p), b = __ldcg((const double2 *)p + 1);
  return mk4(a.x, a.y, b.x, b.y);
}

// Mixed form, ASSPAR4 sums of node n: the FP32 slot forces summed in the
// fixed PARITH/ON order in FP32 (explicit round-to-nearest adds: no
// reassociation).  MLP: the first U slots of the node (all of them in a
// regular mesh: 4 per shell node, 8 per hexa node) are loaded together
// before the sums, so that their latencies overlap; further slots follow one
// by one.  COH = true: the slots were written earlier in the same launch by
// other blocks, so they are read through L2.

template <bool ROT, bool COH, bool MLP>
__device__ __forceinline__ void node_sums_f32(const int k0, const int k1,
                                              const float4 *__restrict__ fsky,
                                              const float4 *__restrict__ fskyr,
                                              int *__restrict__ status, float &b0, float &b1,
                                              float &b2, float &c0, float &c1, float &c2) {
  b0 = b1 = b2 = c0 = c1 = c2 = 0.f;
  constexpr int U = MLP ? (ROT ? 4 : 8) : 0;
  float4 fa[U > 0 ? U : 1], ga[ROT && U > 0 ? U : 1];
#pragma unroll
  for (int j = 0; j < U; j++) {
    if (k0 + j < k1) {
      fa[j] = COH ? __ldcg(fsky + k0 + j) : __ldg(fsky + k0 + j);
      if (ROT) ga[j] = COH ? __ldcg(fskyr + k0 + j) : __ldg(fskyr + k0 + j);
    }
  }
#pragma unroll
  for (int j = 0; j < U; j++) {
    if (k0 + j < k1) {
      b0 = __fadd_rn(b0, fa[j].x);
      b1 = __fadd_rn(b1, fa[j].y);
      b2 = __fadd_rn(b2, fa[j].z);
      if (ROT) {
        c0 = __fadd_rn(c0, ga[j].x);
        c1 = __fadd_rn(c1, ga[j].y);
        c2 = __fadd_rn(c2, ga[j].z);
      }
    }
  }
  for (int k = k0 + U; k < k1; k++) {
    const float4 f = COH ? __ldcg(fsky + k) : __ldg(fsky + k);
    b0 = __fadd_rn(b0, f.x);
    b1 = __fadd_rn(b1, f.y);
    b2 = __fadd_rn(b2, f.z);
    if (ROT) {
      const float4 g = COH ? __ldcg(fskyr + k) : __ldg(fskyr + k);
      c0 = __fadd_rn(c0, g.x);
      c1 = __fadd_rn(c1, g.y);
      c2 = __fadd_rn(c2, g.z);
    }
  }
  if (!(isfinite(b0) && isfinite(b1) && isfinite(b2))) atomicOr(status, RG_ST_NAN);
}

// ASSPAR4 sums of node n: A (and AR) = 0 + the node's slots in PARITH/ON
// order; FP64 slots summed in FP64, the mixed form's FP32 slots in FP32 and
// widened.  COH = true: the slots were written earlier in the same launch by
// other blocks, so they are read through L2.
template <bool F64, bool ROT, bool COH, bool MLP = true>
__device__ __forceinline__ void node_assemble(const int *__restrict__ adsky,
                                              const void *__restrict__ fsky_,
                                              const void *__restrict__ fskyr_,
                                              int *__restrict__ status, const int n,
                                              double &a0, double &a1, double &a2,
                                              double &r0, double &r1, double &r2) {
  const int k0 = __ldg(adsky + n), k1 = __ldg(adsky + n + 1);
  r0 = r1 = r2 = 0.0;
  if constexpr (F64) {
    const dbl4 *fsky = (const dbl4 *)fsky_;
    const dbl4 *fskyr = (const dbl4 *)fskyr_;
    a0 = a1 = a2 = 0.0;
    // unrolled by 4 (a node's slots: 4 for shells, 8 for hexas): crash-box
    // node kernel 22.4 -> 21.6 us, the same bits
#pragma unroll 4
    for (int k = k0; k < k1; k++) {
      const dbl4 f = COH ? ldcg4(fsky + k) : fsky[k];
      a0 = __dadd_rn(a0, f.x);
      a1 = __dadd_rn(a1, f.y);
      a2 = __dadd_rn(a2, f.z);
      if (ROT) {
        const dbl4 g = COH ? ldcg4(fskyr + k) : fskyr[k];
        r0 = __dadd_rn(r0, g.x);
        r1 = __dadd_rn(r1, g.y);
        r2 = __dadd_rn(r2, g.z);
      }
    }
    if (!(isfinite(a0) && isfinite(a1) && isfinite(a2))) atomicOr(status, RG_ST_NAN);
  } else {
    float b0, b1, b2, c0, c1, c2;
    node_sums_f32<ROT, COH, MLP>(k0, k1, (const float4 *)fsky_, (const float4 *)fskyr_, status,
                                 b0, b1, b2, c0, c1, c2);
    a0 = b0;
    a1 = b1;
    a2 = b2;
    r0 = c0;
    r1 = c1;
    r2 = c2;
  }
}

// COH = true: the slots and the time-step scalars were written earlier in
// the same launch by other blocks, so they are read through L2.  LINK: the
// model has rigid links; lacc holds their common accelerations (rlink
// kernel).  MLP: load a node's first slots together (more registers; off in
// the batched kernels, which are held to their register budgets).
template <bool F64, bool ROT, bool COH = false, bool LINK = false, bool MLP = true>
__device__ __forceinline__ void node_update(const NodeView &N, const int *__restrict__ adsky,
                                            const void *__restrict__ fsky_,
                                            const void *__restrict__ fskyr_,
                                            const Time *__restrict__ T,
                                            const int *__restrict__ wall,
                                            const double *__restrict__ walls,
                                            const dbl4 *__restrict__ lacc,
                                            int *__restrict__ status, const int n) {
  double a0, a1, a2, r0 = 0.0, r1 = 0.0, r2 = 0.0;
  F8 xf;  // mixed form: FP32 position copy; pad0 / pad1 = 1/MS, 1/IN in FP32
#if RG_NODE_EARLY
  // the node's own records are loaded ahead of the slot gathers (whose
  // status atomic would otherwise keep them behind), so that both latencies
  // overlap
  dbl4 x = ld4(N.X4 + n);
  dbl4 v = ld4(N.V4 + n);
  dbl4 d;
  if constexpr (F64) d = ld4(N.D4 + n);
  else xf = N.XF[n];
#endif
  if constexpr (F64) {
    node_assemble<F64, ROT, COH, MLP>(adsky, fsky_, fskyr_, status, n, a0, a1, a2, r0, r1, r2);
  } else {
    float b0, b1, b2, c0, c1, c2;
    node_sums_f32<ROT, COH, MLP>(__ldg(adsky + n), __ldg(adsky + n + 1),
                                 (const float4 *)fsky_, (const float4 *)fskyr_, status, b0, b1,
                                 b2, c0, c1, c2);
#if !RG_NODE_EARLY
    xf = N.XF[n];
#endif
    // ACCELE on the FP32 force sums: F * (1/MS) rounded once in FP32, then
    // widened (the forces carry FP32 precision already)
    a0 = widen_f32(__fmul_rn(b0, xf.pad0));
    a1 = widen_f32(__fmul_rn(b1, xf.pad0));
    a2 = widen_f32(__fmul_rn(b2, xf.pad0));
    if (ROT) {
      r0 = widen_f32(__fmul_rn(c0, xf.pad1));
      r1 = widen_f32(__fmul_rn(c1, xf.pad1));
      r2 = widen_f32(__fmul_rn(c2, xf.pad1));
    }
  }
  // FP64 form: D4 = displacement, MS.  Mixed form: D4 holds the initial
  // position and MS (D = X - X0 on download), so it is not touched here.
#if !RG_NODE_EARLY
  dbl4 x = ld4(N.X4 + n);
  dbl4 v = ld4(N.V4 + n);
  dbl4 d;
  if constexpr (F64) d = ld4(N.D4 + n);
#endif
  const double dt12 = COH ? __ldcg(&T->dt12) : T->dt12;
  const double dt2 = COH ? __ldcg(&T->dt2) : T->dt2;
  // ACCELE: A = A * (1/MS); X4.w holds 1/MS (0 when MS <= 0, giving A = 0)
  if constexpr (F64) {
    a0 = __dmul_rn(a0, x.w);
    a1 = __dmul_rn(a1, x.w);
    a2 = __dmul_rn(a2, x.w);
  }
  // node code: BCS bits 1/2/4 (x/y/z), 8/16/32 (rotations); above them the
  // 1-based index of the node's rigid link (0: none)
  const int code = small_int_f64(v.w);
  if (code) {
    if (code & 1) a0 = 0.0;
    if (code & 2) a1 = 0.0;
    if (code & 4) a2 = 0.0;
  }
  // RLINK1 (rlink1.F), after the boundary conditions (resol.F:7322, 7355):
  // the linked directions take the link's common acceleration
  const int lk = LINK ? code >> RG_LINK_SHIFT : 0;
  if (LINK && lk > 0) {
    const dbl4 L = lacc[2 * (lk - 1)];
    const int ic = (int)L.w;
    if (ic & 4) a0 = L.x;
    if (ic & 2) a1 = L.y;
    if (ic & 1) a2 = L.z;
  }
  // RGWALL (constraints/general/rwall/rgwall.F:33), fixed infinite plane,
  // sliding: a slave node whose predicted position X + (V + A*DT12)*DT2 is
  // on or behind the plane and which does not move away from it loses the
  // normal components of its acceleration and velocity.
  if (wall) {
    const int w = __ldg(wall + n);
    if (w >= 0 && !wall_clear(walls + RG_WALL_STRIDE * w, x, v, a0, a1, a2, dt12, dt2)) {
      const double *W = walls + RG_WALL_STRIDE * w;
      // predicted normal velocity VN = (V + A*DT12).n and distance
      // DP = (X + (V + A*DT12)*DT2 - P0).n = (X - P0).n + DT2*VN, in fused
      // multiply-adds written out (the same bits in every kernel)
      const double vx = fma(a0, dt12, v.x);
      const double vy = fma(a1, dt12, v.y);
      const double vz = fma(a2, dt12, v.z);
      const double vn = fma(vz, W[5], fma(vy, W[4], vx * W[3]));
      const double dp0 = fma(x.z - W[2], W[5], fma(x.y - W[1], W[4], (x.x - W[0]) * W[3]));
      const double dp = fma(dt2, vn, dp0);
      if (!(dp > 0.0) && !(vn > 0.0)) {
        const double dv = __dadd_rn(__dadd_rn(__dmul_rn(v.x, W[3]), __dmul_rn(v.y, W[4])),
                                    __dmul_rn(v.z, W[5]));
        const double da = __dadd_rn(__dadd_rn(__dmul_rn(a0, W[3]), __dmul_rn(a1, W[4])),
                                    __dmul_rn(a2, W[5]));
        if (N.wext) {
          // external work of the wall (rgwall.F:289-300, 515): the normal
          // impulse force FN = (DV + DA*DT12)*MS*n against the velocity
          // before the correction, TFXTN = -FACT*(V.FN), FACT = 1/DT12, and
          // WFEXT += HALF*DT1*TFXTN (accumulated per node; explicit rounding)
          const double ms = N.D4[n].w;
          const double dvt = __dmul_rn(__dadd_rn(dv, __dmul_rn(da, dt12)), ms);
          const double fact = dt12 != 0.0 ? __drcp_rn(dt12) : 0.0;
          const double vfn =
              __dadd_rn(__dadd_rn(__dmul_rn(v.x, __dmul_rn(dvt, W[3])),
                                  __dmul_rn(v.y, __dmul_rn(dvt, W[4]))),
                        __dmul_rn(v.z, __dmul_rn(dvt, W[5])));
          const double dt1 = COH ? __ldcg(&T->dt1) : T->dt1;
          N.wext[n] = __dadd_rn(N.wext[n], __dmul_rn(__dmul_rn(RG_HALF, dt1), -__dmul_rn(fact, vfn)));
        }
        a0 = __dadd_rn(a0, -__dmul_rn(da, W[3]));
        a1 = __dadd_rn(a1, -__dmul_rn(da, W[4]));
        a2 = __dadd_rn(a2, -__dmul_rn(da, W[5]));
        v.x = __dadd_rn(v.x, -__dmul_rn(dv, W[3]));
        v.y = __dadd_rn(v.y, -__dmul_rn(dv, W[4]));
        v.z = __dadd_rn(v.z, -__dmul_rn(dv, W[5]));
      }
    }
  }
  // VELOCITY + DEPLA (FP64 in both forms; FP64 form without fused
  // multiply-add, as the reference)
  if constexpr (F64) {
    v.x = __dadd_rn(v.x, __dmul_rn(dt12, a0));
    v.y = __dadd_rn(v.y, __dmul_rn(dt12, a1));
    v.z = __dadd_rn(v.z, __dmul_rn(dt12, a2));
    const double vdx = __dmul_rn(dt2, v.x), vdy = __dmul_rn(dt2, v.y), vdz = __dmul_rn(dt2, v.z);
    d.x = __dadd_rn(d.x, vdx);
    d.y = __dadd_rn(d.y, vdy);
    d.z = __dadd_rn(d.z, vdz);
    x.x = __dadd_rn(x.x, vdx);
    x.y = __dadd_rn(x.y, vdy);
    x.z = __dadd_rn(x.z, vdz);
  } else {
    v.x = fma(dt12, a0, v.x);
    v.y = fma(dt12, a1, v.y);
    v.z = fma(dt12, a2, v.z);
    x.x = fma(dt2, v.x, x.x);
    x.y = fma(dt2, v.y, x.y);
    x.z = fma(dt2, v.z, x.z);
    // the FP32 hi/lo copy advances by the FP32-rounded increment with an
    // exact two-sum (no FP64 split of the new position)
    // increment DT2 * V formed in FP32 from the FP32 velocity copy (one
    // rounding more than the FP64 product: below the copy's resolution)
    const float vfx = narrow_f64(v.x), vfy = narrow_f64(v.y), vfz = narrow_f64(v.z);
    const float dt2f = narrow_f64(dt2);
    ff_add(xf.hx, xf.lx, __fmul_rn(dt2f, vfx));
    ff_add(xf.hy, xf.ly, __fmul_rn(dt2f, vfy));
    ff_add(xf.hz, xf.lz, __fmul_rn(dt2f, vfz));
    N.XF[n] = xf;
    N.VF[n] = make_float4(vfx, vfy, vfz, 0.f);
  }
  st4(N.X4 + n, x);
  st4(N.V4 + n, v);
  if constexpr (F64) st4(N.D4 + n, d);
  if (ROT) {
    dbl4 vr = ld4(N.VR4 + n);
    if constexpr (F64) {
      r0 = __dmul_rn(r0, vr.w);
      r1 = __dmul_rn(r1, vr.w);
      r2 = __dmul_rn(r2, vr.w);
    }
    if (code) {
      if (code & 8) r0 = 0.0;
      if (code & 16) r1 = 0.0;
      if (code & 32) r2 = 0.0;
    }
    if (LINK && lk > 0) {
      const dbl4 L = lacc[2 * (lk - 1) + 1];
      const int icr = (int)L.w;
      if (icr & 4) r0 = L.x;
      if (icr & 2) r1 = L.y;
      if (icr & 1) r2 = L.z;
    }
    if constexpr (F64) {
      vr.x = __dadd_rn(vr.x, __dmul_rn(dt12, r0));
      vr.y = __dadd_rn(vr.y, __dmul_rn(dt12, r1));
      vr.z = __dadd_rn(vr.z, __dmul_rn(dt12, r2));
    } else {
      vr.x = fma(dt12, r0, vr.x);
      vr.y = fma(dt12, r1, vr.y);
      vr.z = fma(dt12, r2, vr.z);
    }
    st4(N.VR4 + n, vr);
    if constexpr (!F64)
      N.VRF[n] = make_float4(narrow_f64(vr.x), narrow_f64(vr.y), narrow_f64(vr.z), 0.f);
  }
}


// RESOL time-step logic (resol.F:2721-2722, 6123-6127, 6352, 6494-6497),
// applied by one thread to the reduced element minimum (dt2t, key ok):
// DT2 = min(DT2T, 1.1*DT2OLD, DTMX) (1.1 is a REAL*4 literal), DT12, TT.
// advance = 0 only records DT2T / NELTST (FORINT-level call).
__device__ __forceinline__ void dt_apply(Time *__restrict__ T, const double dt2t, const int ok,
                                         const int *__restrict__ ngl, int *__restrict__ status,
                                         const int advance) {
  T->dt2t = dt2t;
  if (!advance) {
    T->neltst = ok >= 0 ? ngl[ok] : 0;
    return;
  }
  const double dt1 = T->dt2;
  double dt2 = RG_EP06;
  if (dt2t < dt2) {
    dt2 = dt2t;
    T->neltst = ok >= 0 ? ngl[ok] : 0;
  }
  dt2 = fmin(fmin(dt2, __dmul_rn(RG_SP_1P1, T->dt2old)), T->dtmx);
  T->dt1 = dt1;
  T->dt2 = dt2;
  T->dt2old = dt2;
  T->dt12 = __dmul_rn(RG_HALF, __dadd_rn(dt1, dt2));
  T->tt = __dadd_rn(T->tt, dt2);
  T->ncycle += 1;
  if (T->dtmin > 0.0 && dt2 < T->dtmin) atomicOr(status, RG_ST_DTMIN);
}

// Last-block time-step reduction (DtFinish), called by every element block
// after thread 0 wrote its partial number p.  Thread 0 publishes (fence) and
// takes a ticket of the partial's group; the block with the group's last
// ticket reduces the group's partials through L2 and takes a ticket of the
// cycle; the block with the cycle's last ticket reduces the group minima,
// applies dt_apply and re-arms the counters.  No block waits on another.
template <int NT>
__device__ __forceinline__ void dt_finish_block(const DtPartials dp, const DtFinish F, int p,
                                                Time *__restrict__ T,
                                                int *__restrict__ status) {
  static_assert(NT >= DT_GROUP, "one thread per partial of a group");
  __shared__ int s_last;
  __shared__ double od;
  __shared__ int ok;
  const int g = p / DT_GROUP;
  const int ngroups = (F.nparts + DT_GROUP - 1) / DT_GROUP;
  const int gsize = min(DT_GROUP, F.nparts - g * DT_GROUP);
  if (threadIdx.x == 0) {
    __threadfence();
    s_last = atomicAdd(F.ctr + 1 + g, 1u) == (unsigned)(gsize - 1);
  }
  __syncthreads();
  if (!s_last) return;
  __threadfence();
  {
    double d = RG_EP06;
    int k = -1;
    if (threadIdx.x < gsize) {
      const int i = g * DT_GROUP + threadIdx.x;
      const int ki = __ldcg(dp.el + i);
      if (ki >= 0) {
        d = __ldcg(dp.dt + i);
        k = ki;
      }
    }
    block_dt_min<NT>(d, k, F.gdt + g, F.gel + g);
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    F.ctr[1 + g] = 0u;
    __threadfence();
    s_last = atomicAdd(F.ctr, 1u) == (unsigned)(ngroups - 1);
  }
  __syncthreads();
  if (!s_last) return;
  __threadfence();
  double d = RG_EP06;
  int k = -1;
  for (int i = threadIdx.x; i < ngroups; i += NT) {
    const int ki = __ldcg(F.gel + i);
    if (ki >= 0) dt_pair_min(d, k, __ldcg(F.gdt + i), ki);
  }
  block_dt_min<NT>(d, k, &od, &ok);
  __syncthreads();
  if (threadIdx.x == 0) {
    dt_apply(T, od, ok, F.ngl, status, F.advance);
    F.ctr[0] = 0u;
  }
}

}  // namespace rg
