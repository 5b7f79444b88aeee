// One-point hexa element kernel (single model) and its launch wrappers; the
// element arithmetic is hexa_element() in rg_hexa_elem.cuh.
#include "rg_hexa_elem.cuh"
#include "rg_kernels.h"
#include "rg_node.cuh"

#include <type_traits>

namespace rg {

// Resident 128-thread blocks per SM the FP32 hexa kernel's register budget
// is cut for: 6 (80 registers) -- 2.1M-hexa block 0.249 ms, against 0.251
// at 5 (96 registers) and 0.264 at 7 (72).
#ifndef RG_HEXA_MIXED_BLK128
#define RG_HEXA_MIXED_BLK128 6
#endif

template <typename ER, int LAW, int JCVT, int NT, int MINB>
__global__ void __launch_bounds__(NT, MINB)
hexa_kernel(const HexaParams P, const HexaArrays<ER> A, const NodeView N,
            typename SlotT<ER>::type *__restrict__ fsky, DtPartials dp,
            Time *__restrict__ T, int *__restrict__ status, const DtFinish F) {
  typedef ER R;
  const int il = blockIdx.x * NT + threadIdx.x;
  R dtmine = (R)RG_EP06;
  int elmin = -1;
  if (il < P.nel) hexa_element<ER, LAW, JCVT>(P, A, N, fsky, T, status, il, dtmine, elmin);
  // per-block time-step candidate
  block_dt_min<NT, R>(dtmine, elmin, dp.dt + P.part_off + blockIdx.x,
                      dp.el + P.part_off + blockIdx.x);
  if (F.ctr) dt_finish_block<NT>(dp, F, P.part_off + blockIdx.x, T, status);
}

// ---------------------------------------------------------------------------
// Block size of a group: 128 threads, or 64 for a group of fewer than two
// blocks of 128 per SM of a 152-SM GPU, whose 128-thread blocks would leave
// SMs idle (the 8,000-hexa bar: 63 blocks of 128 on 152 SMs, each SM's
// FP64 work then set by one block).
constexpr int HEXA_SMALL = 2 * 152 * 128;
static int hexa_nt(int nel) { return nel < HEXA_SMALL ? 64 : 128; }

template <typename ER, int LAW, int NT>
static void launch_nt(const HexaParams &P, const HexaArrays<ER> &A, const NodeView &N,
                      typename SlotT<ER>::type *fsky, DtPartials dp, Time *T, int *status,
                      const DtFinish &F, cudaStream_t s) {
  // mixed form: 6 resident 128-thread blocks per SM at 80 registers (about
  // 100 bytes per thread spill to L1: measured faster than 4, 5 or 7
  // blocks; 64-thread blocks keep the same register budget); the FP64 form
  // needs its ~250 registers
  constexpr int MINB = std::is_same<ER, float>::value ? RG_HEXA_MIXED_BLK128 * 128 / NT : 1;
  const int nb = (P.nel + NT - 1) / NT;
  if (P.jcvt)
    hexa_kernel<ER, LAW, 1, NT, MINB><<<nb, NT, 0, s>>>(P, A, N, fsky, dp, T, status, F);
  else
    hexa_kernel<ER, LAW, 0, NT, MINB><<<nb, NT, 0, s>>>(P, A, N, fsky, dp, T, status, F);
}

template <typename ER, int LAW>
static void launch_one(const HexaParams &P, const HexaArrays<ER> &A,
                       const NodeView &N, typename SlotT<ER>::type *fsky,
                       DtPartials dp, Time *T, int *status, const DtFinish &F,
                       cudaStream_t s) {
  if (hexa_nt(P.nel) == 64)
    launch_nt<ER, LAW, 64>(P, A, N, fsky, dp, T, status, F, s);
  else
    launch_nt<ER, LAW, 128>(P, A, N, fsky, dp, T, status, F, s);
}

// time-step partials of a group: one per block of its launch
int hexa_blocks(int nel) { return (nel + hexa_nt(nel) - 1) / hexa_nt(nel); }

// Mixed form, FORINT-level call: the host supplies X and V for the cycle, so
// the FP64 volume that the element kernel advances by its FP32 increment
// V(X) - V(X - DT1*V) is re-anchored to the previous configuration
// X - DT1*V, in FP64 with the SDERI3 determinant.
__global__ void hexa_prev_volume_kernel(const HexaArrays<float> A, const NodeView N,
                                        const Time *__restrict__ T) {
  const int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= A.ne) return;
  const double dt1 = T->dt2;
  double x[8], y[8], z[8];
#pragma unroll
  for (int k = 0; k < 8; k++) {
    const int n = __ldg(A.nc + k * A.ne + e);
    const dbl4 xk = ld4(N.X4 + n), vk = ld4(N.V4 + n);
    x[k] = xk.x - dt1 * vk.x;
    y[k] = xk.y - dt1 * vk.y;
    z[k] = xk.z - dt1 * vk.z;
  }
  const double x17 = x[6] - x[0], x28 = x[7] - x[1], x35 = x[4] - x[2], x46 = x[5] - x[3];
  const double y17 = y[6] - y[0], y28 = y[7] - y[1], y35 = y[4] - y[2], y46 = y[5] - y[3];
  const double z17 = z[6] - z[0], z28 = z[7] - z[1], z35 = z[4] - z[2], z46 = z[5] - z[3];
  const double jac1 = x17 + x28 - x35 - x46, jac2 = y17 + y28 - y35 - y46,
               jac3 = z17 + z28 - z35 - z46;
  const double jac4 = (x17 + x46) + (x28 + x35), jac5 = (y17 + y46) + (y28 + y35),
               jac6 = (z17 + z46) + (z28 + z35);
  const double jac7 = (x17 + x46) - (x28 + x35), jac8 = (y17 + y46) - (y28 + y35),
               jac9 = (z17 + z46) - (z28 + z35);
  const double det = RG_ONE_OVER_64 * (jac1 * (jac5 * jac9 - jac6 * jac8) +
                                       jac2 * (jac6 * jac7 - jac4 * jac9) +
                                       jac3 * (jac4 * jac8 - jac5 * jac7));
  if (A.off[e] != 0.f) A.rho[e] = det;
}

void launch_hexa_prev_volume(const HexaArrays<float> &A, const NodeView &N, const Time *T,
                             cudaStream_t s) {
  if (A.ne > 0) hexa_prev_volume_kernel<<<(A.ne + 255) / 256, 256, 0, s>>>(A, N, T);
}

void launch_hexa_f64(const HexaParams &P, const HexaArrays<double> &A,
                     const NodeView &N, dbl4 *fsky, DtPartials dp,
                     Time *T, int *status, const DtFinish &F, cudaStream_t s) {
  if (P.mtn == 1)
    launch_one<double, 1>(P, A, N, fsky, dp, T, status, F, s);
  else
    launch_one<double, 2>(P, A, N, fsky, dp, T, status, F, s);
}

void launch_hexa_f32(const HexaParams &P, const HexaArrays<float> &A,
                     const NodeView &N, float4 *fsky, DtPartials dp,
                     Time *T, int *status, const DtFinish &F, cudaStream_t s) {
  if (P.mtn == 1)
    launch_one<float, 1>(P, A, N, fsky, dp, T, status, F, s);
  else
    launch_one<float, 2>(P, A, N, fsky, dp, T, status, F, s);
}

}  // namespace rg
