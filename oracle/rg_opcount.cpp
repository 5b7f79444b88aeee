// Counters and C entry points of the op-counting build of the oracle --
// MEASUREMENT INFRASTRUCTURE ONLY (see rg_opcount.h).  Built into
// _build/librg_oracle_count.so together with the oracle's own sources, which
// the forced include rg_opcount_pre.h compiles with every `double` replaced
// by rg_count::Real.  Run single-threaded (the counters are plain globals).
#undef double
#include "rg_opcount.h"

namespace rg_count {
long long counts[NPHASE][NOPS];
int phase = 0;
}  // namespace rg_count

extern "C" {

// counts[NPHASE][NOPS] in phase-major order: phases 0 other, 1 hexa element
// groups, 2 shell element groups, 3 assembly and nodal update; operations
// add/sub, mul, div, sqrt, pow, log, exp, sin/cos, compare, min/max.
void or_opcount_get(long long *out) {
  for (int p = 0; p < rg_count::NPHASE; p++)
    for (int o = 0; o < rg_count::NOPS; o++) out[p * rg_count::NOPS + o] = rg_count::counts[p][o];
}

void or_opcount_reset() {
  for (int p = 0; p < rg_count::NPHASE; p++)
    for (int o = 0; o < rg_count::NOPS; o++) rg_count::counts[p][o] = 0;
}
}
