// Batched explicit cycle: many independent models (jobs) advanced together,
// one persistent cooperative kernel per cycle.
//
// Each job is a finalized rg_ctx (its device arrays stay where rg_finalize
// put them); the batch adds descriptors over them:
//   element tiles   (group, tile) -> ktile x 128 consecutive elements of one
//                   hexa or shell group, taken by the blocks from an atomic
//                   work counter, each tile writing one dt partial;
//   per-job dt      one block reduces a job's partials and applies the RESOL
//                   time-step logic to that job's own Time record;
//   node tiles      (job, first node) -> knode x 128 nodes.
// With the persistent schedule the three phases run in one cooperative launch
// separated by two grid barriers (bounded waits, RG_ST_BARRIER on give-up);
// the three-launch schedule runs them as three ordinary launches.  Both are
// captured as a one-cycle CUDA graph.  Every element and node is computed by
// the same device functions as in the single-model kernels and the
// PARITH/ON sums keep their fixed order, so a job's results are bitwise the
// same alone and in any batch, under any tile / block / schedule choice.
//
// Each job carries its own cycle target: a job whose Time::ncycle has reached
// it is skipped by all three phases (jobs of different lengths share the
// batch; each advances with its own stable time step).
#include "../../include/rg_api.h"
#include "rg_ctx.h"
#include "rg_hexa_elem.cuh"
#include "rg_node.cuh"
#include "rg_shell_elem.cuh"

#include <algorithm>
#include <climits>
#include <cstring>
#include <string>
#include <vector>

namespace rg {

constexpr int BNT = 128;  // threads per block, elements / nodes per sub-tile
constexpr unsigned BAR_SPIN_LIMIT = 1u << 22;  // ~0.3-3 s of 64 ns naps

// tile kinds: hexa LAW1 / LAW2 (Jaumann rate), shells of 1..5 points,
// hexa LAW1 / LAW2 in the co-rotational frame (JCVT = 1); tiles run in
// decreasing kind order, the costliest first
enum { BK_HEXA1 = 0, BK_HEXA2 = 1, BK_SHELL = 2 /* + npt - 1 */, BK_HEXA1C = 7, BK_HEXA2C = 8 };
__host__ __device__ inline bool bk_hexa(int kind) { return kind < BK_SHELL || kind >= BK_HEXA1C; }

struct BatchTile {
  int kind, group, tile, part;
};
struct BatchNodeTile {
  int job, n0;
};

template <typename ER>
struct BatchJob {
  NodeView nv;
  const int *adsky;
  void *fsky, *fskyr;
  Time *T;
  int *status;
  const int *wall;
  const double *walls;
  const int *ngl;
  DtPartials dp;
  int nparts, rot, target, numelc;
  int key0, pad[3];
  HexaArrays<ER> ha;
  ShellArrays<ER> sa;
};

struct BatchHexaGroup {
  HexaParams P;
  int job, pad[3];
};
struct BatchShellGroup {
  ShellParams P;
  int job, pad[3];
};

struct GridBar {
  unsigned count, gen;
};

template <typename ER>
struct BatchDev {
  const BatchJob<ER> *jobs;
  const BatchHexaGroup *hg;
  const BatchShellGroup *sg;
  const BatchTile *tiles;
  const BatchNodeTile *ntl;
  int *ran;        // [njobs] job advanced in this cycle (phase 2 -> 3)
  int *ncyc;       // [njobs] Time::ncycle after the cycle (host progress)
  unsigned *ctr;   // [2] work counters: element tiles, node tiles
  GridBar *bar;
  int *bstatus;    // batch status word (RG_ST_BARRIER)
  int njobs, ntiles, nntiles, ktile, knode, pad;
  // barrier wait limit (64 ns naps) and the test hook: block late_block
  // (-1: none) arrives at every barrier after late_naps naps of 1 us
  unsigned spin_limit, late_naps;
  int late_block, pad2;
};

// Grid-wide barrier for a cooperative launch (all blocks co-resident).  The
// wait is bounded: on give-up the block records RG_ST_BARRIER and goes on.
// The counters of the barrier and of the work queues are re-armed before
// every cycle (batch_reset_counters), so a cycle whose barrier gave up leaves
// nothing behind for the next one.
__device__ __forceinline__ void grid_barrier(GridBar *bar, int *bstatus, unsigned spin_limit,
                                             int late_block, unsigned late_naps) {
  __syncthreads();
  if (threadIdx.x == 0) {
    if ((int)blockIdx.x == late_block)
      for (unsigned i = 0; i < late_naps; i++) __nanosleep(1000);  // bounded delay
    const unsigned g = atomicOr(&bar->gen, 0u);
    __threadfence();
    if (atomicAdd(&bar->count, 1u) == gridDim.x - 1) {
      atomicExch(&bar->count, 0u);
      __threadfence();
      atomicAdd(&bar->gen, 1u);
    } else {
      unsigned it = 0;
      while (atomicOr(&bar->gen, 0u) == g) {
        if (++it > spin_limit) {
          atomicOr(bstatus, RG_ST_BARRIER);
          break;
        }
        __nanosleep(64);
      }
    }
    __threadfence();
  }
  __syncthreads();
}

// Next work item of a phase: one atomic per block, broadcast through shared.
__device__ __forceinline__ int next_item(unsigned *ctr, int *s_item) {
  if (threadIdx.x == 0) *s_item = (int)atomicAdd(ctr, 1u);
  __syncthreads();
  const int t = *s_item;
  __syncthreads();
  return t;
}

template <typename T>
__device__ __forceinline__ void copy_to_shared(T *dst, const T *src) {
  static_assert(sizeof(T) % 4 == 0, "word copy");
  const int *s = (const int *)src;
  int *d = (int *)dst;
  for (int i = threadIdx.x; i < (int)(sizeof(T) / 4); i += BNT) d[i] = s[i];
  __syncthreads();
}

template <typename ER, int MINB>
__global__ void __launch_bounds__(BNT, MINB)
batch_kernel(const BatchDev<ER> B, const int phases) {
  typedef ER R;
  typedef typename SlotT<ER>::type ST;
  constexpr bool F64 = sizeof(ER) == 8;
  __shared__ BatchJob<ER> sJ;
  __shared__ union {
    HexaParams h;
    ShellParams s;
  } sP;
  __shared__ int s_item;

  // ---- phase 1: element tiles -------------------------------------------
  if (phases & 1) {
    for (;;) {
      const int t = next_item(B.ctr, &s_item);
      if (t >= B.ntiles) break;
      const BatchTile tl = B.tiles[t];
      const bool hexa = bk_hexa(tl.kind);
      const int j = hexa ? B.hg[tl.group].job : B.sg[tl.group].job;
      if (__ldcg(&B.jobs[j].T->ncycle) >= B.jobs[j].target) continue;  // block-uniform
      copy_to_shared(&sJ, B.jobs + j);
      if (hexa)
        copy_to_shared(&sP.h, &B.hg[tl.group].P);
      else
        copy_to_shared(&sP.s, &B.sg[tl.group].P);
      R dtmine = (R)RG_EP06;
      int elmin = -1;
      for (int k = 0; k < B.ktile; k++) {
        const int il = (tl.tile * B.ktile + k) * BNT + threadIdx.x;
        ST *fs = (ST *)sJ.fsky;
        ST *fr = (ST *)sJ.fskyr;
        switch (tl.kind) {
          case BK_HEXA1:
            if (il < sP.h.nel)
              hexa_element<ER, 1>(sP.h, sJ.ha, sJ.nv, fs, sJ.T, sJ.status, il, dtmine, elmin);
            break;
          case BK_HEXA2:
            if (il < sP.h.nel)
              hexa_element<ER, 2>(sP.h, sJ.ha, sJ.nv, fs, sJ.T, sJ.status, il, dtmine, elmin);
            break;
          case BK_HEXA1C:
            if (il < sP.h.nel)
              hexa_element<ER, 1, 1>(sP.h, sJ.ha, sJ.nv, fs, sJ.T, sJ.status, il, dtmine, elmin);
            break;
          case BK_HEXA2C:
            if (il < sP.h.nel)
              hexa_element<ER, 2, 1>(sP.h, sJ.ha, sJ.nv, fs, sJ.T, sJ.status, il, dtmine, elmin);
            break;
          case BK_SHELL + 0:
            if (il < sP.s.nel)
              shell_element<ER, 1>(sP.s, sJ.sa, sJ.nv, fs, fr, sJ.T, sJ.key0, sJ.numelc, il,
                                   dtmine, elmin);
            break;
          case BK_SHELL + 1:
            if (il < sP.s.nel)
              shell_element<ER, 2>(sP.s, sJ.sa, sJ.nv, fs, fr, sJ.T, sJ.key0, sJ.numelc, il,
                                   dtmine, elmin);
            break;
          case BK_SHELL + 2:
            if (il < sP.s.nel)
              shell_element<ER, 3>(sP.s, sJ.sa, sJ.nv, fs, fr, sJ.T, sJ.key0, sJ.numelc, il,
                                   dtmine, elmin);
            break;
          case BK_SHELL + 3:
            if (il < sP.s.nel)
              shell_element<ER, 4>(sP.s, sJ.sa, sJ.nv, fs, fr, sJ.T, sJ.key0, sJ.numelc, il,
                                   dtmine, elmin);
            break;
          default:
            if (il < sP.s.nel)
              shell_element<ER, 5>(sP.s, sJ.sa, sJ.nv, fs, fr, sJ.T, sJ.key0, sJ.numelc, il,
                                   dtmine, elmin);
            break;
        }
      }
      block_dt_min<BNT, R>(dtmine, elmin, sJ.dp.dt + tl.part, sJ.dp.el + tl.part);
      __syncthreads();
    }
  }
  if ((phases & 1) && (phases & 6))
    grid_barrier(B.bar, B.bstatus, B.spin_limit, B.late_block, B.late_naps);

  // ---- phase 2: time step of each job ----------------------------------------
  if (phases & 2) {
    __shared__ double od;
    __shared__ int ok;
    for (int j = blockIdx.x; j < B.njobs; j += gridDim.x) {
      const BatchJob<ER> &J = B.jobs[j];
      const int act = __ldcg(&J.T->ncycle) < J.target;
      if (act) {
        double d = RG_EP06;
        int k = -1;
        for (int i = threadIdx.x; i < J.nparts; i += BNT) {
          const int ki = __ldcg(J.dp.el + i);
          if (ki >= 0) dt_pair_min(d, k, __ldcg(J.dp.dt + i), ki);
        }
        block_dt_min<BNT>(d, k, &od, &ok);
        __syncthreads();
        if (threadIdx.x == 0) dt_apply(J.T, od, ok, J.ngl, J.status, 1);
      }
      if (threadIdx.x == 0) {
        B.ran[j] = act;
        B.ncyc[j] = J.T->ncycle;
      }
      __syncthreads();
    }
    // the element counter is free again (phase 1 ended before this phase)
    if (blockIdx.x == 0 && threadIdx.x == 0) B.ctr[0] = 0u;
  }
  if ((phases & 2) && (phases & 4))
    grid_barrier(B.bar, B.bstatus, B.spin_limit, B.late_block, B.late_naps);

  // ---- phase 3: node tiles -----------------------------------------------------
  if (phases & 4) {
    for (;;) {
      const int t = next_item(B.ctr + 1, &s_item);
      if (t >= B.nntiles) break;
      const BatchNodeTile nt = B.ntl[t];
      if (!__ldcg(B.ran + nt.job)) continue;
      const BatchJob<ER> &J = B.jobs[nt.job];
      const int nn = J.nv.numnod;
      for (int k = 0; k < B.knode; k++) {
        const int n = nt.n0 + k * BNT + threadIdx.x;
        if (n < nn) {
          if (J.rot)
            node_update<F64, true, true, false, false>(J.nv, J.adsky, J.fsky, J.fskyr, J.T, J.wall, J.walls, nullptr,
                                         J.status, n);
          else
            node_update<F64, false, true, false, false>(J.nv, J.adsky, J.fsky, J.fskyr, J.T, J.wall, J.walls, nullptr,
                                          J.status, n);
        }
      }
    }
  }
}

template <typename ER>
__global__ void batch_init_ncyc(const BatchJob<ER> *jobs, int n, int *ncyc) {
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j < n) ncyc[j] = jobs[j].T->ncycle;
}

// Node phase as its own kernel (three-launch schedule): the node update has
// few live values, so this kernel runs at full occupancy where the fused
// kernel is held to the element phase's register budget.  node_update's
// arithmetic is written with explicit rounding (no contraction), so the
// result is bitwise that of the fused kernel's node phase.
template <typename ER>
__global__ void __launch_bounds__(256)
batch_node_kernel(const BatchDev<ER> B) {
  constexpr bool F64 = sizeof(ER) == 8;
  const int t = blockIdx.x;  // one node tile per block row of 256 threads
  for (int tile = t; tile < B.nntiles; tile += gridDim.x) {
    const BatchNodeTile nt = B.ntl[tile];
    if (!__ldcg(B.ran + nt.job)) continue;
    const BatchJob<ER> &J = B.jobs[nt.job];
    const int nn = J.nv.numnod;
    const int span = B.knode * BNT;
    for (int i = threadIdx.x; i < span; i += 256) {
      const int n = nt.n0 + i;
      if (n < nn) {
        if (J.rot)
          node_update<F64, true, true, false, false>(J.nv, J.adsky, J.fsky, J.fskyr, J.T, J.wall, J.walls, nullptr,
                                       J.status, n);
        else
          node_update<F64, false, true, false, false>(J.nv, J.adsky, J.fsky, J.fskyr, J.T, J.wall, J.walls, nullptr,
                                        J.status, n);
      }
    }
  }
}

// The work counters and the barrier's arrival count are re-armed before each
// cycle's launch sequence by a separate one-thread kernel (stream order puts
// it after the previous cycle's last kernel): the rule is the same for both
// schedules, and a cycle whose barrier wait gave up cannot leave a stale count
// to the next one.  In a healthy run all three are zero already.
__global__ void batch_reset_counters(unsigned *ctr, GridBar *bar) {
  ctr[0] = 0u;
  ctr[1] = 0u;
  bar->count = 0u;
}

}  // namespace rg

using namespace rg;

struct rg_batch {
  int device = 0;
  int prec = -1;
  cudaStream_t stream = nullptr;
  std::string err;
  std::vector<rg_ctx *> jobs;   // slots; nullptr = free
  std::vector<int> target;      // per slot
  // launch configuration
  int ktile = 1, knode = 1, blocks_per_sm = 0, schedule = 0;  // 0 persistent, 1 three launches
  // grid barrier wait limit and its test hook (rg_batch_set_barrier_test)
  unsigned spin_limit = BAR_SPIN_LIMIT, late_naps = 0;
  int late_block = -1;
  int max_blocks_per_sm = 0, nsm = 0;
  // device descriptors
  void *d_jobs = nullptr;
  BatchHexaGroup *d_hg = nullptr;
  BatchShellGroup *d_sg = nullptr;
  BatchTile *d_tiles = nullptr;
  BatchNodeTile *d_ntl = nullptr;
  int *d_ran = nullptr, *d_ncyc = nullptr, *d_bstatus = nullptr;
  unsigned *d_ctr = nullptr;
  GridBar *d_bar = nullptr;
  size_t cap_jobs = 0, cap_hg = 0, cap_sg = 0, cap_tiles = 0, cap_ntl = 0;
  int njobs = 0, ntiles = 0, nntiles = 0;
  std::vector<int> slot_of_job;  // dense job index -> slot
  bool dirty = true;
  cudaGraphExec_t gexec = nullptr;
  cudaEvent_t ev[2] = {};
};

namespace {

int bfail(rg_batch *b, int code, const std::string &m) {
  if (b) b->err = m;
  return code;
}

#define RB_CUDA(b, call)                                                     \
  do {                                                                       \
    cudaError_t _e = (call);                                                 \
    if (_e != cudaSuccess)                                                   \
      return bfail((b), RG_E_CUDA, std::string(#call) + ": " + cudaGetErrorString(_e)); \
  } while (0)

template <typename T>
int grow(rg_batch *b, T **p, size_t &cap, size_t n) {
  if (n <= cap && *p) return RG_OK;
  if (*p) RB_CUDA(b, cudaFree(*p));
  *p = nullptr;
  const size_t c = std::max<size_t>(std::max<size_t>(n, 1), cap * 2);
  RB_CUDA(b, cudaMalloc((void **)p, c * sizeof(T)));
  cap = c;
  return RG_OK;
}

template <typename ER>
const HexaArrays<ER> &hexa_arrays(const rg_ctx *c);
template <>
const HexaArrays<double> &hexa_arrays<double>(const rg_ctx *c) {
  return c->h64;
}
template <>
const HexaArrays<float> &hexa_arrays<float>(const rg_ctx *c) {
  return c->h32;
}

// Rebuild descriptors and tiles from the occupied slots.
template <typename ER>
int rebuild(rg_batch *b) {
  std::vector<BatchJob<ER>> jobs;
  std::vector<BatchHexaGroup> hg;
  std::vector<BatchShellGroup> sg;
  std::vector<BatchTile> tiles;
  std::vector<BatchNodeTile> ntl;
  b->slot_of_job.clear();
  const int et = BNT * b->ktile, nt = BNT * b->knode;
  for (size_t s = 0; s < b->jobs.size(); s++) {
    rg_ctx *c = b->jobs[s];
    if (!c) continue;
    const int j = (int)jobs.size();
    b->slot_of_job.push_back((int)s);
    BatchJob<ER> J;
    std::memset(&J, 0, sizeof(J));
    J.nv = c->nv;
    J.adsky = c->d_adsky;
    J.fsky = c->d_fsky;
    J.fskyr = c->d_fskyr;
    J.T = c->d_time;
    J.status = c->d_status;
    J.wall = c->d_wall;
    J.walls = c->d_walls;
    J.ngl = c->d_ngl_all;
    J.dp = c->dp;
    J.rot = c->rot ? 1 : 0;
    J.target = b->target[s];
    J.ha = hexa_arrays<ER>(c);
    const void *sa = shell_device_arrays(c->shells, c->prec);
    if (sa) J.sa = *(const ShellArrays<ER> *)sa;
    J.key0 = c->numels;
    J.numelc = shell_numelc(c->shells);
    int part = 0;
    for (const auto &g : c->hg) {
      const int gi = (int)hg.size();
      BatchHexaGroup G;
      std::memset(&G, 0, sizeof(G));
      G.P = g.P;
      G.job = j;
      hg.push_back(G);
      const int ntl_g = (g.nel + et - 1) / et;
      for (int t = 0; t < ntl_g; t++)
        tiles.push_back({g.P.jcvt ? (g.P.mtn == 1 ? BK_HEXA1C : BK_HEXA2C)
                                  : (g.P.mtn == 1 ? BK_HEXA1 : BK_HEXA2),
                         gi, t, part + t});
      part += ntl_g;
    }
    const int nsg = shell_group_count(c->shells);
    for (int q = 0; q < nsg; q++) {
      const ShellParams *P = shell_group_params(c->shells, q);
      const int gi = (int)sg.size();
      BatchShellGroup G;
      std::memset(&G, 0, sizeof(G));
      G.P = *P;
      G.job = j;
      sg.push_back(G);
      const int ntl_g = (P->nel + et - 1) / et;
      for (int t = 0; t < ntl_g; t++) tiles.push_back({BK_SHELL + P->npt - 1, gi, t, part + t});
      part += ntl_g;
    }
    if (part > c->nparts_cap) return bfail(b, RG_E_STATE, "batch: dt partial count exceeds the job's");
    J.nparts = part;
    jobs.push_back(J);
    for (int n0 = 0; n0 < c->numnod; n0 += nt) ntl.push_back({j, n0});
  }
  // costlier tiles first (shell points, then hexa JC): better tail balance
  std::stable_sort(tiles.begin(), tiles.end(),
                   [](const BatchTile &a, const BatchTile &c) { return a.kind > c.kind; });
  int r;
  if ((r = grow(b, (BatchJob<ER> **)&b->d_jobs, b->cap_jobs, jobs.size()))) return r;
  if ((r = grow(b, &b->d_hg, b->cap_hg, hg.size()))) return r;
  if ((r = grow(b, &b->d_sg, b->cap_sg, sg.size()))) return r;
  if ((r = grow(b, &b->d_tiles, b->cap_tiles, tiles.size()))) return r;
  if ((r = grow(b, &b->d_ntl, b->cap_ntl, ntl.size()))) return r;
  if (b->cap_jobs > 0) {
    // ran / ncyc sized with the job capacity
    if (b->d_ran) RB_CUDA(b, cudaFree(b->d_ran));
    if (b->d_ncyc) RB_CUDA(b, cudaFree(b->d_ncyc));
    RB_CUDA(b, cudaMalloc(&b->d_ran, b->cap_jobs * sizeof(int)));
    RB_CUDA(b, cudaMalloc(&b->d_ncyc, b->cap_jobs * sizeof(int)));
    RB_CUDA(b, cudaMemsetAsync(b->d_ran, 0, b->cap_jobs * sizeof(int), b->stream));
    RB_CUDA(b, cudaMemsetAsync(b->d_ncyc, 0, b->cap_jobs * sizeof(int), b->stream));
  }
  if (!jobs.empty())
    RB_CUDA(b, cudaMemcpyAsync(b->d_jobs, jobs.data(), jobs.size() * sizeof(BatchJob<ER>),
                               cudaMemcpyHostToDevice, b->stream));
  if (!hg.empty())
    RB_CUDA(b, cudaMemcpyAsync(b->d_hg, hg.data(), hg.size() * sizeof(BatchHexaGroup),
                               cudaMemcpyHostToDevice, b->stream));
  if (!sg.empty())
    RB_CUDA(b, cudaMemcpyAsync(b->d_sg, sg.data(), sg.size() * sizeof(BatchShellGroup),
                               cudaMemcpyHostToDevice, b->stream));
  if (!tiles.empty())
    RB_CUDA(b, cudaMemcpyAsync(b->d_tiles, tiles.data(), tiles.size() * sizeof(BatchTile),
                               cudaMemcpyHostToDevice, b->stream));
  if (!ntl.empty())
    RB_CUDA(b, cudaMemcpyAsync(b->d_ntl, ntl.data(), ntl.size() * sizeof(BatchNodeTile),
                               cudaMemcpyHostToDevice, b->stream));
  if (!jobs.empty())
    batch_init_ncyc<ER><<<((int)jobs.size() + 127) / 128, 128, 0, b->stream>>>(
        (const BatchJob<ER> *)b->d_jobs, (int)jobs.size(), b->d_ncyc);
  RB_CUDA(b, cudaMemsetAsync(b->d_ctr, 0, 2 * sizeof(unsigned), b->stream));
  RB_CUDA(b, cudaMemsetAsync(b->d_bar, 0, sizeof(GridBar), b->stream));
  RB_CUDA(b, cudaStreamSynchronize(b->stream));
  b->njobs = (int)jobs.size();
  b->ntiles = (int)tiles.size();
  b->nntiles = (int)ntl.size();
  return RG_OK;
}

template <typename ER>
BatchDev<ER> dev_view(rg_batch *b) {
  BatchDev<ER> D;
  std::memset(&D, 0, sizeof(D));
  D.jobs = (const BatchJob<ER> *)b->d_jobs;
  D.hg = b->d_hg;
  D.sg = b->d_sg;
  D.tiles = b->d_tiles;
  D.ntl = b->d_ntl;
  D.ran = b->d_ran;
  D.ncyc = b->d_ncyc;
  D.ctr = b->d_ctr;
  D.bar = b->d_bar;
  D.bstatus = b->d_bstatus;
  D.njobs = b->njobs;
  D.ntiles = b->ntiles;
  D.nntiles = b->nntiles;
  D.ktile = b->ktile;
  D.knode = b->knode;
  D.spin_limit = b->spin_limit;
  D.late_block = b->late_block;
  D.late_naps = b->late_naps;
  return D;
}

// mixed form: 4 resident blocks of 128 threads (the NPT = 5 shell path needs
// 128 registers); FP64 form: 2
template <typename ER>
constexpr int batch_minb() {
  return sizeof(ER) == 4 ? 4 : 1;
}

template <typename ER>
int occupancy(rg_batch *b) {
  int n = 0;
  RB_CUDA(b, cudaOccupancyMaxActiveBlocksPerMultiprocessor(
                 &n, batch_kernel<ER, batch_minb<ER>()>, BNT, 0));
  b->max_blocks_per_sm = n;
  return RG_OK;
}

// Enqueue one batched cycle on the batch stream.
template <typename ER>
int enqueue(rg_batch *b) {
  if (b->njobs == 0) return RG_OK;
  const BatchDev<ER> D = dev_view<ER>(b);
  auto kern = batch_kernel<ER, batch_minb<ER>()>;
  const int bps = b->blocks_per_sm > 0 ? std::min(b->blocks_per_sm, b->max_blocks_per_sm)
                                       : b->max_blocks_per_sm;
  const int grid = std::max(1, bps * b->nsm);
  batch_reset_counters<<<1, 1, 0, b->stream>>>(b->d_ctr, b->d_bar);
  if (b->schedule == 0) {
    cudaLaunchConfig_t cfg;
    std::memset(&cfg, 0, sizeof(cfg));
    cfg.gridDim = dim3(grid);
    cfg.blockDim = dim3(BNT);
    cfg.stream = b->stream;
    cudaLaunchAttribute at[1];
    at[0].id = cudaLaunchAttributeCooperative;
    at[0].val.cooperative = 1;
    cfg.attrs = at;
    cfg.numAttrs = 1;
    RB_CUDA(b, cudaLaunchKernelEx(&cfg, kern, D, 7));
  } else {
    kern<<<std::min(grid, std::max(1, b->ntiles)), BNT, 0, b->stream>>>(D, 1);
    kern<<<std::min(grid, std::max(1, b->njobs)), BNT, 0, b->stream>>>(D, 2);
    batch_node_kernel<ER><<<std::max(1, b->nntiles), 256, 0, b->stream>>>(D);
  }
  RB_CUDA(b, cudaGetLastError());
  return RG_OK;
}

int enqueue_any(rg_batch *b) {
  return b->prec == RG_PREC_FP64 ? enqueue<double>(b) : enqueue<float>(b);
}

// Rebuild descriptors if membership or configuration changed, and capture
// the one-cycle graph.
int prepare(rg_batch *b) {
  if (!b->dirty) return RG_OK;
  int r;
  // launched cycles may still read the descriptors about to be replaced
  RB_CUDA(b, cudaStreamSynchronize(b->stream));
  if (b->gexec) {
    RB_CUDA(b, cudaGraphExecDestroy(b->gexec));
    b->gexec = nullptr;
  }
  if (b->prec < 0) {
    b->njobs = b->ntiles = b->nntiles = 0;
    b->dirty = false;
    return RG_OK;
  }
  r = b->prec == RG_PREC_FP64 ? rebuild<double>(b) : rebuild<float>(b);
  if (r) return r;
  r = b->prec == RG_PREC_FP64 ? occupancy<double>(b) : occupancy<float>(b);
  if (r) return r;
  if (b->njobs > 0) {
    cudaGraph_t g = nullptr;
    RB_CUDA(b, cudaStreamBeginCapture(b->stream, cudaStreamCaptureModeThreadLocal));
    r = enqueue_any(b);
    cudaError_t ce = cudaStreamEndCapture(b->stream, &g);
    if (r) return r;
    if (ce != cudaSuccess)
      return bfail(b, RG_E_CUDA, std::string("batch graph capture: ") + cudaGetErrorString(ce));
    cudaError_t ie = cudaGraphInstantiate(&b->gexec, g, 0);
    cudaGraphDestroy(g);
    if (ie != cudaSuccess)
      return bfail(b, RG_E_CUDA, std::string("batch graph: ") + cudaGetErrorString(ie));
  }
  b->dirty = false;
  return RG_OK;
}

}  // namespace

extern "C" {

int rg_batch_create(int device, rg_batch **out) {
  if (!out) return RG_E_ARG;
  *out = nullptr;
  rg_batch *b = new rg_batch();
  b->device = device;
  cudaError_t e = cudaSetDevice(device);
  if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking);
  if (e == cudaSuccess) e = cudaDeviceGetAttribute(&b->nsm, cudaDevAttrMultiProcessorCount, device);
  if (e == cudaSuccess) e = cudaMalloc(&b->d_ctr, 2 * sizeof(unsigned));
  if (e == cudaSuccess) e = cudaMalloc(&b->d_bar, sizeof(GridBar));
  if (e == cudaSuccess) e = cudaMalloc(&b->d_bstatus, sizeof(int));
  if (e == cudaSuccess) e = cudaMemset(b->d_bstatus, 0, sizeof(int));
  if (e == cudaSuccess) e = cudaEventCreate(&b->ev[0]);
  if (e == cudaSuccess) e = cudaEventCreate(&b->ev[1]);
  if (e != cudaSuccess) {
    delete b;
    return RG_E_CUDA;
  }
  *out = b;
  return RG_OK;
}

int rg_batch_destroy(rg_batch *b) {
  if (!b) return RG_E_ARG;
  cudaSetDevice(b->device);
  if (b->stream) cudaStreamSynchronize(b->stream);
  if (b->gexec) cudaGraphExecDestroy(b->gexec);
  void *ps[] = {b->d_jobs, b->d_hg, b->d_sg, b->d_tiles, b->d_ntl, b->d_ran,
                b->d_ncyc, b->d_bstatus, b->d_ctr, b->d_bar};
  for (void *p : ps)
    if (p) cudaFree(p);
  for (auto &e : b->ev)
    if (e) cudaEventDestroy(e);
  if (b->stream) cudaStreamDestroy(b->stream);
  delete b;
  return RG_OK;
}

const char *rg_batch_last_error(rg_batch *b) { return b ? b->err.c_str() : "null batch"; }

int rg_batch_add(rg_batch *b, rg_ctx *c, int target_ncycle) {
  if (!b || !c) return RG_E_ARG;
  if (!c->finalized) return bfail(b, RG_E_STATE, "batch: job context not finalized");
  if (c->device != b->device) return bfail(b, RG_E_ARG, "batch: job on another device");
  if (c->nlinks) return bfail(b, RG_E_UNSUP, "batch: jobs with rigid links run alone (rg_cycle)");
  if (c->nodadt) return bfail(b, RG_E_UNSUP, "batch: jobs with the nodal time step run alone (rg_cycle)");
  if (c->shells.idtmin)
    return bfail(b, RG_E_UNSUP, "batch: jobs with an element time-step action run alone (rg_cycle)");
  for (auto &g : c->hg)
  // the batched kernel carries the lean shell material (no kinematic
  // hardening, thermal softening or IPLA = 2: they run alone)
  for (int g = 0; g < shell_group_count(c->shells); g++)
    if (shell_mf(*shell_group_params(c->shells, g)) != 0)
      return bfail(b, RG_E_UNSUP,
                   "batch: shells with kinematic hardening, thermal softening or Iplas=2 run alone "
                   "(rg_cycle)");
  bool any = false;
  for (auto *q : b->jobs) any = any || q;
  if (any && c->prec != b->prec)
    return bfail(b, RG_E_ARG, "batch: all jobs must use the same arithmetic form");
  for (auto *q : b->jobs)
    if (q == c) return bfail(b, RG_E_ARG, "batch: context already in the batch");
  b->prec = c->prec;
  // the job's own stream may still hold work: order it before the batch's
  RB_CUDA(b, cudaSetDevice(b->device));
  RB_CUDA(b, cudaStreamSynchronize(c->stream));
  int slot = -1;
  for (size_t s = 0; s < b->jobs.size(); s++)
    if (!b->jobs[s]) {
      slot = (int)s;
      break;
    }
  if (slot < 0) {
    slot = (int)b->jobs.size();
    b->jobs.push_back(nullptr);
    b->target.push_back(INT_MAX);
  }
  b->jobs[slot] = c;
  b->target[slot] = target_ncycle < 0 ? INT_MAX : target_ncycle;
  b->dirty = true;
  return slot;
}

int rg_batch_remove(rg_batch *b, int slot) {
  if (!b || slot < 0 || slot >= (int)b->jobs.size() || !b->jobs[slot]) return RG_E_ARG;
  RB_CUDA(b, cudaSetDevice(b->device));
  RB_CUDA(b, cudaStreamSynchronize(b->stream));
  b->jobs[slot] = nullptr;
  b->dirty = true;
  return RG_OK;
}

int rg_batch_set_target(rg_batch *b, int slot, int target_ncycle) {
  if (!b || slot < 0 || slot >= (int)b->jobs.size() || !b->jobs[slot]) return RG_E_ARG;
  b->target[slot] = target_ncycle < 0 ? INT_MAX : target_ncycle;
  b->dirty = true;
  return RG_OK;
}

int rg_batch_set_config(rg_batch *b, int ktile, int knode, int blocks_per_sm, int schedule) {
  if (!b) return RG_E_ARG;
  if (ktile < 1 || ktile > 64 || knode < 1 || knode > 64 || blocks_per_sm < 0 ||
      (schedule != 0 && schedule != 1))
    return bfail(b, RG_E_ARG, "batch: bad configuration");
  b->ktile = ktile;
  b->knode = knode;
  b->blocks_per_sm = blocks_per_sm;
  b->schedule = schedule;
  b->dirty = true;
  return RG_OK;
}

int rg_batch_get_config(rg_batch *b, int *cfg5) {
  if (!b || !cfg5) return RG_E_ARG;
  int r = prepare(b);
  if (r) return r;
  cfg5[0] = b->ktile;
  cfg5[1] = b->knode;
  cfg5[2] = b->blocks_per_sm;
  cfg5[3] = b->schedule;
  cfg5[4] = b->max_blocks_per_sm;
  return RG_OK;
}

int rg_batch_cycle(rg_batch *b, int ncycle) {
  if (!b || ncycle < 0) return RG_E_ARG;
  RB_CUDA(b, cudaSetDevice(b->device));
  int r = prepare(b);
  if (r) return r;
  if (!b->gexec) return RG_OK;
  for (int i = 0; i < ncycle; i++) RB_CUDA(b, cudaGraphLaunch(b->gexec, b->stream));
  return RG_OK;
}

int rg_batch_synchronize(rg_batch *b) {
  if (!b) return RG_E_ARG;
  RB_CUDA(b, cudaStreamSynchronize(b->stream));
  return RG_OK;
}

int rg_batch_time_cycles(rg_batch *b, int ncycle, double *ms) {
  if (!b || !ms || ncycle < 0) return RG_E_ARG;
  RB_CUDA(b, cudaSetDevice(b->device));
  int r = prepare(b);
  if (r) return r;
  RB_CUDA(b, cudaEventRecord(b->ev[0], b->stream));
  if (b->gexec)
    for (int i = 0; i < ncycle; i++) RB_CUDA(b, cudaGraphLaunch(b->gexec, b->stream));
  RB_CUDA(b, cudaEventRecord(b->ev[1], b->stream));
  RB_CUDA(b, cudaEventSynchronize(b->ev[1]));
  float f = 0.f;
  RB_CUDA(b, cudaEventElapsedTime(&f, b->ev[0], b->ev[1]));
  *ms = f;
  return RG_OK;
}

// Cycle counts of the slots (Time::ncycle after the last batched cycle;
// -1 for a free slot) and the batch status word (cleared by the read).
int rg_batch_progress(rg_batch *b, int *ncycle, int nslots, int *bstatus) {
  if (!b) return RG_E_ARG;
  RB_CUDA(b, cudaSetDevice(b->device));
  int r = prepare(b);
  if (r) return r;
  std::vector<int> nc(std::max(b->njobs, 1), 0);
  if (b->njobs > 0)
    RB_CUDA(b, cudaMemcpyAsync(nc.data(), b->d_ncyc, b->njobs * sizeof(int),
                               cudaMemcpyDeviceToHost, b->stream));
  int st = 0;
  RB_CUDA(b, cudaMemcpyAsync(&st, b->d_bstatus, sizeof(int), cudaMemcpyDeviceToHost, b->stream));
  RB_CUDA(b, cudaMemsetAsync(b->d_bstatus, 0, sizeof(int), b->stream));
  RB_CUDA(b, cudaStreamSynchronize(b->stream));
  if (ncycle) {
    for (int s = 0; s < nslots; s++) ncycle[s] = -1;
    for (int j = 0; j < b->njobs; j++) {
      const int s = b->slot_of_job[j];
      if (s < nslots) ncycle[s] = nc[j];
    }
  }
  if (bstatus) *bstatus = st;
  return RG_OK;
}

// Status word of every job (RG_ST_* bits of its own context, 0 for a free
// slot), read after the batch's queued cycles and left set: the job's own
// rg_status still reads and clears it.  One small copy per job.
int rg_batch_job_status(rg_batch *b, int *status, int nslots) {
  if (!b || !status || nslots < 0) return RG_E_ARG;
  RB_CUDA(b, cudaSetDevice(b->device));
  for (int s = 0; s < nslots; s++) status[s] = 0;
  const int n = std::min(nslots, (int)b->jobs.size());
  for (int s = 0; s < n; s++)
    if (b->jobs[s])
      RB_CUDA(b, cudaMemcpyAsync(status + s, b->jobs[s]->d_status, sizeof(int),
                                 cudaMemcpyDeviceToHost, b->stream));
  RB_CUDA(b, cudaStreamSynchronize(b->stream));
  return RG_OK;
}

// Test hook of the bounded grid barrier: spin_limit naps of 64 ns before a
// block gives up (0 = the default), and block late_block (-1 = none) made to
// arrive at every barrier after late_us microseconds of sleep.  With a limit
// shorter than the delay the other blocks' waits run out, the kernel records
// RG_ST_BARRIER and returns; nothing hangs and nothing faults.
int rg_batch_set_barrier_test(rg_batch *b, unsigned spin_limit, int late_block,
                              unsigned late_us) {
  if (!b || late_us > 1000000u) return RG_E_ARG;
  b->spin_limit = spin_limit ? spin_limit : BAR_SPIN_LIMIT;
  b->late_block = late_block;
  b->late_naps = late_block >= 0 ? late_us : 0u;
  b->dirty = true;
  return RG_OK;
}

// Project autotuner: time every candidate launch configuration on the
// batch's own jobs and keep the fastest.  The jobs' device state is saved
// before the trials and restored after them, so tuning leaves the
// simulation exactly where it was.  cand = NULL uses the built-in candidate
// list; otherwise ncand rows of {ktile, knode, blocks_per_sm, schedule}.
// best5 receives {ktile, knode, blocks_per_sm, schedule, ms_per_cycle_x1000}.
int rg_batch_autotune(rg_batch *b, int trial_cycles, const int *cand, int ncand, int *best5) {
  if (!b || trial_cycles < 1) return RG_E_ARG;
  RB_CUDA(b, cudaSetDevice(b->device));
  int r = prepare(b);
  if (r) return r;
  if (b->njobs == 0) return bfail(b, RG_E_STATE, "batch: no jobs to tune on");
  std::vector<int> cl;
  if (cand && ncand > 0) {
    cl.assign(cand, cand + 4 * ncand);
  } else {
    const int mx = b->max_blocks_per_sm;
    const int kt[] = {1, 2, 4};
    const int kn[] = {1, 4};
    for (int sch = 0; sch < 2; sch++)
      for (int a : kt)
        for (int c : kn)
          for (int bps : {1, std::max(1, mx / 2), mx}) {
            cl.insert(cl.end(), {a, c, bps, sch});
            if (mx <= 2 && bps == 1) break;
          }
  }
  // save every allocation of every job
  std::vector<std::pair<void *, void *>> saved;
  std::vector<size_t> sizes;
  for (rg_ctx *c : b->jobs) {
    if (!c) continue;
    for (size_t i = 0; i < c->allocs.size(); i++) {
      void *p = nullptr;
      cudaError_t e = cudaMalloc(&p, c->alloc_bytes[i]);
      if (e != cudaSuccess) {
        for (auto &q : saved) cudaFree(q.second);
        return bfail(b, RG_E_MEM, "autotune: no room to save the job state");
      }
      cudaMemcpyAsync(p, c->allocs[i], c->alloc_bytes[i], cudaMemcpyDeviceToDevice, b->stream);
      saved.push_back({c->allocs[i], p});
      sizes.push_back(c->alloc_bytes[i]);
    }
  }
  const int k0 = b->ktile, n0 = b->knode, p0 = b->blocks_per_sm, s0 = b->schedule;
  double best = 1e30;
  int bi = -1;
  int err = RG_OK;
  for (size_t i = 0; i + 3 < cl.size() && !err; i += 4) {
    b->ktile = cl[i];
    b->knode = cl[i + 1];
    b->blocks_per_sm = cl[i + 2];
    b->schedule = cl[i + 3];
    b->dirty = true;
    if ((err = prepare(b))) break;
    double ms = 0.0;
    if ((err = rg_batch_cycle(b, 1))) break;  // warm-up
    if ((err = rg_batch_time_cycles(b, trial_cycles, &ms))) break;
    if (ms < best) {
      best = ms;
      bi = (int)i;
    }
  }
  for (size_t i = 0; i < saved.size(); i++)
    cudaMemcpyAsync(saved[i].first, saved[i].second, sizes[i], cudaMemcpyDeviceToDevice,
                    b->stream);
  cudaStreamSynchronize(b->stream);
  for (auto &q : saved) cudaFree(q.second);
  if (err) {
    b->ktile = k0;
    b->knode = n0;
    b->blocks_per_sm = p0;
    b->schedule = s0;
    b->dirty = true;
    return err;
  }
  b->ktile = cl[bi];
  b->knode = cl[bi + 1];
  b->blocks_per_sm = cl[bi + 2];
  b->schedule = cl[bi + 3];
  b->dirty = true;
  if ((r = prepare(b))) return r;
  RB_CUDA(b, cudaMemsetAsync(b->d_bstatus, 0, sizeof(int), b->stream));
  if (best5) {
    best5[0] = b->ktile;
    best5[1] = b->knode;
    best5[2] = b->blocks_per_sm;
    best5[3] = b->schedule;
    best5[4] = (int)(1000.0 * best / trial_cycles);
  }
  return RG_OK;
}

}  // extern "C"
