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
