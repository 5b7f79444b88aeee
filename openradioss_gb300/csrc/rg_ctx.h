#pragma once
// Internal definition of the C-ABI context (rg_ctx): shared by the
// translation units of librg that work on a context's device arrays
// (rg_api.cu, rg_batch.cu).  Not part of the public interface.
#include <cuda_runtime.h>

#include <string>
#include <vector>

#include "../../include/rg_api.h"
#include "rg_device.cuh"
#include "rg_shell.h"

namespace rg {

struct HexaGroupHost {
  HexaParams P;
  int nel;
};

struct WallHost {
  double p0[3], n[3], dsearch;
};

struct LinkHost {
  std::vector<int> nodes;  // 0-based
  int ic = 0, icr = 0;     // direction bits 4 = x, 2 = y, 1 = z
};

// Device tables of the per-part sums (rg_parts.cu): each part's elements in
// element order, cut into chunks (start in perm, count, partial slot, part);
// the density per entry; the slot range of each part.  Outside the
// snapshot: derived from the model, not state.
struct PartTables {
  int npart = 0, nh_chunks = 0, ns_chunks = 0, nslots = 0;
  int *hperm = nullptr, *sperm = nullptr;
  double *hcoef = nullptr, *scoef = nullptr;
  int4 *hchunk = nullptr, *schunk = nullptr;
  int *poff = nullptr;        // [npart + 1]
  double *partial = nullptr;  // [nslots][RG_PART_NQ]
  double *out = nullptr;      // [npart][RG_PART_NQ]
};

}  // namespace rg

struct rg_ctx {
  typedef rg::HexaGroupHost HexaGroupHost;
  typedef rg::WallHost WallHost;
  typedef rg::LinkHost LinkHost;
  typedef rg::ShellModelHost ShellModelHost;
  typedef rg::NodeView NodeView;
  typedef rg::Time Time;
  typedef rg::DtPartials DtPartials;
  template <typename T>
  using HexaArrays = rg::HexaArrays<T>;
  int device = 0;
  cudaStream_t stream = nullptr;
  std::string err;
  int prec = RG_PREC_FP64;
  bool finalized = false;
  bool timing = false;
  double ktime[4] = {0, 0, 0, 0};

  // ---- host-side model (until finalize) ----
  int numnod = 0;
  std::vector<double> X, V, MS, IN;
  std::vector<int> icodt;
  int numels = 0;
  std::vector<int> ixs;  // 11 * numels
  std::vector<HexaGroupHost> hg;
  ShellModelHost shells;  // rg_shell.h
  std::vector<WallHost> walls;
  std::vector<LinkHost> links;
  std::vector<int> adsky, iads, iadc;  // 1-based as given / built
  bool skyline_given = false;
  int lsky = 0;
  double dtfac_solid = RG_ZEP9, dtfac_shell = RG_ZEP9, dtmx = RG_EP30,
         dt2old = RG_EP30;

  // ---- device ----
  NodeView nv{};
  int *d_adsky = nullptr;
  void *d_fsky = nullptr;   // dbl4 or float4 [lsky]
  void *d_fskyr = nullptr;  // rotational slots (shell models)
  HexaArrays<double> h64{};
  HexaArrays<float> h32{};
  int *d_nc = nullptr, *d_iads = nullptr, *d_ngl_all = nullptr;
  Time *d_time = nullptr;
  int *d_status = nullptr;
  DtPartials dp{};
  int nparts = 0;       // dt partials written by a cycle's element launches
  int nparts_cap = 0;   // slots allocated (also the batched kernel's tiles)
  unsigned *d_dtctr = nullptr;  // fused dt: [1 + groups] completion counters
  double *d_gdt = nullptr;      // fused dt: group minima
  int *d_gel = nullptr;
  int *d_wall = nullptr;       // per node: wall index or -1
  double *d_walls = nullptr;   // 6 doubles per wall (p0, n)
  int nwalls = 0;
  // rigid links: node lists (concatenated, 0-based), offsets, (ic, icr,
  // active, 0) per link, and the common accelerations (2 per link)
  int nlinks = 0;
  int *d_lnodes = nullptr, *d_loff = nullptr;
  int4 *d_lic = nullptr;
  rg::dbl4 *d_lacc = nullptr;
  int4 h_link = {0, 0, 0, 0};  // source of rg_rlink_set_active's copy
  // nodal time step (/DT/NODA): per-node-block partials, their fused
  // last-block reduction, and the key -> node number table
  int nodadt = 0;
  double dtfac_noda = 0.9, dtmin_noda = 0.0;
  int idtmin_noda = 0;  // IDTMIN(11): 0 flag only, 1/5 stop, 3/8 mass scaling
  int nnparts = 0;
  rg::DtPartials ndp{};
  unsigned *d_nctr = nullptr;
  double *d_ngdt = nullptr;
  int *d_ngel = nullptr;
  int *d_ngl_nodes = nullptr;
  bool rot = false;
  // staging for forint_step / downloads
  double *d_stage = nullptr;   // 12 * numnod doubles
  double *d_epart = nullptr;   // energy partials
  std::vector<void *> allocs;
  std::vector<size_t> alloc_bytes;  // size of each allocation (snapshots)
  unsigned long long dev_bytes = 0;
  cudaGraphExec_t gexec = nullptr;
  cudaGraph_t graph = nullptr;
  cudaEvent_t ev[8] = {};
  void *d_flush = nullptr;     // L2 flush buffer of rg_time_cycles_cold
  Time *h_time = nullptr;      // pinned host copy of the time-step record
  double entot0 = 0.0, mass0 = 0.0;  // cycle-0 totals of the energy balance
  size_t flush_bytes = 0;
  // per-part sums: element -> part maps (empty: one part per element
  // group), their tables, the request for the next cycle and the cycle
  // graph that takes them between the element pass and the nodal update
  int npart = 0;
  std::vector<int> part_hexa, part_shell;
  rg::PartTables pt{};
  bool parts_ready = false, parts_due = false, parts_valid = false;
  cudaGraphExec_t gexec_parts = nullptr;
  cudaGraph_t graph_parts = nullptr;
};

namespace rg {
// rg_parts.cu
int parts_prepare(rg_ctx *c);  // tables and buffers (after rg_finalize)
void parts_enqueue(rg_ctx *c); // the sums of the element pass just enqueued
void parts_free(rg_ctx *c);
}  // namespace rg

