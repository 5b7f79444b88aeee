// Kinetic energy of caller-owned device arrays without any device
// allocation: the variant of the energy reduction (energy_kernel /
// energy_final) whose per-block partial sums live in a fixed file-scope
// device array instead of memory allocated per context.
//
// Who needs it: a caller that must not allocate device memory at the moment
// it asks for the energy -- the serving loop once the HBM budget is fully
// reserved by admitted jobs (an allocation outside the budget could fail or
// push a job out), or an engine that accounts its own device memory and reads
// the energy of arrays it owns between two cycles.  It takes raw device
// pointers, so it also serves arrays that are not in an rg_ctx.
//
// Scratch: RG_NOALLOC_MAX_BLOCKS partial sums (one per block of 256 threads,
// each block summing RG_NOALLOC_NODES_PER_BLOCK nodes) + one result slot.
// Nothing in it has to start at zero: every call overwrites the partials it
// reads.  The scratch is shared by all callers on a device, so two calls that
// overlap in time on one device race: callers serialise them.
//
// The scratch is part of this library's device module.  With CUDA's lazy
// module loading (the default) the module -- and with it the 512 KB array --
// is loaded on the device when the first call looks the scratch address up,
// so that first call does take device memory.  A caller that must not
// allocate later makes one warm-up call per device while it still has room
// (at context creation, before it reserves its HBM budget); every later call
// allocates nothing.
//
// The kernels run on the legacy default stream.  Contexts of this library
// run on their own non-blocking streams, so the arrays of a context must be
// complete first: call rg_synchronize(ctx), or synchronise whatever stream
// produced the arrays, before this call.
#include "../../include/rg_api.h"

#include <cuda_runtime.h>

#include <mutex>

namespace {

constexpr int NA_NT = 256;
constexpr int NA_PER_BLOCK = RG_NOALLOC_NODES_PER_BLOCK;
constexpr int NA_MAX_BLOCKS = RG_NOALLOC_MAX_BLOCKS;
constexpr int NA_MAX_DEVICES = 64;

static __device__ __align__(256) double g_ke_scratch[NA_MAX_BLOCKS + 1];

// scratch address per device, looked up once with that device current
std::mutex g_setup_mu;
double *g_scratch_ptr[NA_MAX_DEVICES] = {};

// Pass 1: block b sums 0.5*MS*|V|^2 over its nodes [b*PER, (b+1)*PER) in a
// fixed order (per-thread strided sums, then a fixed tree).
__global__ void __launch_bounds__(NA_NT)
ke_partials(int numnod, const double *__restrict__ v, const double *__restrict__ ms,
            double *__restrict__ part) {
  const int n0 = blockIdx.x * NA_PER_BLOCK;
  const int n1 = min(numnod, n0 + NA_PER_BLOCK);
  double s = 0.0;
  for (int n = n0 + threadIdx.x; n < n1; n += NA_NT) {
    const double vx = v[3 * n], vy = v[3 * n + 1], vz = v[3 * n + 2];
    s += 0.5 * ms[n] * (vx * vx + vy * vy + vz * vz);
  }
  __shared__ double sh[NA_NT];
  sh[threadIdx.x] = s;
  __syncthreads();
  for (int o = NA_NT / 2; o > 0; o >>= 1) {
    if (threadIdx.x < o) sh[threadIdx.x] += sh[threadIdx.x + o];
    __syncthreads();
  }
  if (threadIdx.x == 0) part[blockIdx.x] = sh[0];
}

// Pass 2: one thread adds the partials in block order.
__global__ void ke_final(int nblocks, const double *__restrict__ part, double *__restrict__ out) {
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  double s = 0.0;
  for (int b = 0; b < nblocks; b++) s += part[b];
  *out = s;
}

// Address of the scratch on `device` (that device must be current).
int scratch_for(int device, double **out) {
  std::lock_guard<std::mutex> lk(g_setup_mu);
  if (!g_scratch_ptr[device]) {
    void *p = nullptr;
    if (cudaGetSymbolAddress(&p, g_ke_scratch) != cudaSuccess || !p) return RG_E_CUDA;
    g_scratch_ptr[device] = (double *)p;
  }
  *out = g_scratch_ptr[device];
  return RG_OK;
}

}  // namespace

extern "C" int rg_kinetic_energy_noalloc(int device, int numnod, const double *d_v,
                                         const double *d_ms, double *ekin) {
  if (!ekin || device < 0 || device >= NA_MAX_DEVICES || numnod < 0) return RG_E_ARG;
  const long long nb = ((long long)numnod + NA_PER_BLOCK - 1) / NA_PER_BLOCK;
  if (nb > NA_MAX_BLOCKS) return RG_E_SIZE;  // more nodes than the fixed scratch covers
  if (numnod > 0 && (!d_v || !d_ms)) return RG_E_ARG;
  int prev = -1;
  if (cudaGetDevice(&prev) != cudaSuccess) return RG_E_CUDA;
  if (prev != device && cudaSetDevice(device) != cudaSuccess) return RG_E_CUDA;
  double *scr = nullptr;
  int r = scratch_for(device, &scr);
  if (r == RG_OK) {
    if (nb > 0) ke_partials<<<(int)nb, NA_NT>>>(numnod, d_v, d_ms, scr);
    ke_final<<<1, 32>>>((int)nb, scr, scr + NA_MAX_BLOCKS);
    double h = 0.0;
    if (cudaGetLastError() != cudaSuccess ||
        cudaMemcpy(&h, scr + NA_MAX_BLOCKS, sizeof(double), cudaMemcpyDeviceToHost) !=
            cudaSuccess)
      r = RG_E_CUDA;
    else
      *ekin = h;
  }
  if (prev != device) cudaSetDevice(prev);
  return r;
}

// ---------------------------------------------------------------------------
// FP64 pipe ceiling of the device, measured: every thread runs 8 independent
// chains of dependent FP64 fused multiply-adds.  Used as the denominator of
// the FP64-pipe roofline of the plain form's kernels (bench).
namespace {
constexpr int PK_CHAINS = 8;
constexpr int PK_ITERS = 4096;

// sink of the FMA chains (never written in practice), apart from the
// kinetic-energy scratch
static __device__ double g_fp64_sink;

__global__ void __launch_bounds__(256) fp64_fma_kernel(double a, double b) {
  double c[PK_CHAINS];
#pragma unroll
  for (int k = 0; k < PK_CHAINS; k++) c[k] = threadIdx.x * 1e-3 + k;
  for (int i = 0; i < PK_ITERS; i++) {
#pragma unroll
    for (int k = 0; k < PK_CHAINS; k++) c[k] = fma(c[k], a, b);
  }
  double s = 0.0;
#pragma unroll
  for (int k = 0; k < PK_CHAINS; k++) s += c[k];
  if (s == 12345.678) g_fp64_sink = s;  // keeps the chains live
}
}  // namespace

extern "C" int rg_fp64_peak(int device, double *fma_per_s) {
  if (!fma_per_s || device < 0 || device >= NA_MAX_DEVICES) return RG_E_ARG;
  int prev = -1;
  if (cudaGetDevice(&prev) != cudaSuccess) return RG_E_CUDA;
  if (prev != device && cudaSetDevice(device) != cudaSuccess) return RG_E_CUDA;
  int nsm = 0;
  cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, device);
  const int blocks = nsm * 8;
  int r = RG_OK;
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  if (cudaEventCreate(&e0) != cudaSuccess || cudaEventCreate(&e1) != cudaSuccess) r = RG_E_CUDA;
  if (r == RG_OK) {
    fp64_fma_kernel<<<blocks, 256>>>(0.999999, 1e-9);  // warm-up
    cudaEventRecord(e0);
    fp64_fma_kernel<<<blocks, 256>>>(0.999999, 1e-9);
    cudaEventRecord(e1);
    float ms = 0.f;
    if (cudaEventSynchronize(e1) != cudaSuccess || cudaEventElapsedTime(&ms, e0, e1) != cudaSuccess)
      r = RG_E_CUDA;
    else
      *fma_per_s = (double)blocks * 256 * PK_CHAINS * PK_ITERS / (ms * 1e-3);
  }
  if (e0) cudaEventDestroy(e0);
  if (e1) cudaEventDestroy(e1);
  if (prev != device) cudaSetDevice(prev);
  return r;
}
