// Belytschko-Tsay 4-node shell module (CFORC3 chain): host bookkeeping and
// launches.  Filled in with the element kernel; until then a model without
// shells passes through these entry points unchanged.
#include "rg_shell.h"

#include "../../include/rg_api.h"

namespace rg {

struct ShellGroupHost {
  int nel = 0;
};

int shell_group_add(ShellModelHost &, int, int, const int *, int,
                    const double *, const double *, const double *,
                    const int *, const double *, int, int,
                    std::string &why) {
  why = "shell groups are not available in this build";
  return RG_E_UNSUP;
}
int shell_numelc(const ShellModelHost &S) { return S.numelc; }
const int *shell_ixc(const ShellModelHost &S) { return S.ixc.data(); }
void shell_user_ids(const ShellModelHost &S, int *out) {
  for (int e = 0; e < S.numelc; e++) out[e] = S.ixc[7 * e + 6];
}
int shell_finalize(ShellModelHost &, int, const double *, const int *, int,
                   double, int &, const DevAlloc &, std::string &) {
  return RG_OK;
}
void shell_enqueue(ShellModelHost &, int, const NodeView &, void *, void *,
                   DtPartials, const Time *, int *, cudaStream_t) {}
int shell_energy_enqueue(ShellModelHost &, int, double *, cudaStream_t) {
  return 0;
}
int shell_download(ShellModelHost &, int, int, double *, std::string &why) {
  why = "no shell groups";
  return RG_E_STATE;
}
void shell_free(ShellModelHost &) {}

}  // namespace rg
