// Host-side interface of the Belytschko-Tsay shell module (rg_shell.cu).
#pragma once
#include <functional>
#include <string>
#include <vector>

#include "rg_device.cuh"

namespace rg {

struct ShellGroupHost;

struct ShellModelHost {
  int numelc = 0;
  std::vector<int> ixc;                 // 7 * numelc (reference layout)
  std::vector<double> thk0;             // initial thickness per shell
  std::vector<ShellGroupHost *> groups;
  int key0 = 0;                         // dt-order key of the first shell
  int ishfram = 0;                      // local frame of every group (0 / 2)
  int nodadt = 0;                       // nodal time step (/DT/NODA)
  int idtmin = 0;                       // element time-step action IDTMIN(3)
  double dtmin = 0.0;                   // DTMIN1(3)
  void *dev = nullptr;                  // device arrays (rg_shell.cu)
};

typedef std::function<int(void **, size_t)> DevAlloc;

int shell_group_add(ShellModelHost &S, int numnod, int nel, const int *ixc,
                    int npt, const double *pm, const double *geo,
                    const double *uparam, const int *iparam,
                    const double *thk0, int ismstr, int ithk,
                    std::string &why);
int shell_numelc(const ShellModelHost &S);
const int *shell_ixc(const ShellModelHost &S);
void shell_user_ids(const ShellModelHost &S, int *out);
// Allocates and initialises the device state; part_off in/out: dt partial
// slots used by the shell launches are appended after the hexa ones; `key0`
// is the element-order key of the first shell (= number of hexas).
int shell_finalize(ShellModelHost &S, int prec, const double *X,
                   const int *iadc, int key0, double dtfac, int &part_off,
                   const DevAlloc &alloc, std::string &why);
void shell_enqueue(ShellModelHost &S, int prec, const NodeView &N, void *fsky,
                   void *fskyr, DtPartials dp, Time *T, int *status,
                   const DtFinish &F, cudaStream_t s);
int shell_energy_enqueue(ShellModelHost &S, int prec, double *out2,
                         cudaStream_t s);
int shell_download(ShellModelHost &S, int prec, int which, double *out,
                   std::string &why);
void shell_free(ShellModelHost &S);

// Views for the batched kernel (rg_batch.cu): the model's device arrays
// (a ShellArrays<double> or ShellArrays<float> by prec, nullptr before
// finalize) and the parameters of group g.
struct ShellParams;
const void *shell_device_arrays(const ShellModelHost &S, int prec);
int shell_group_count(const ShellModelHost &S);
// 128-element tiles over all shell groups (one dt partial each)
int shell_tile_count(const ShellModelHost &S);
const ShellParams *shell_group_params(const ShellModelHost &S, int g);

}  // namespace rg
