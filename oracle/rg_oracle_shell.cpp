// CPU oracle, Belytschko-Tsay shell part -- TEST INFRASTRUCTURE.
// (Filled in with the CFORC3 restatement; see rg_oracle.cpp for the
// conventions.)
#include <vector>

namespace rg_oracle_shell {

struct Shells {
  int numelc = 0;
  std::vector<int> ixc;
  std::vector<int> iadc;
};

Shells *create() { return new Shells(); }
void destroy(Shells *s) { delete s; }
int group_add(Shells *, int, const int *, int, const double *, const double *,
              const double *, const int *, const double *, int, int) {
  return -10;
}
int numelc(const Shells *s) { return s->numelc; }
const int *ixc(const Shells *s) { return s->ixc.data(); }
int *iadc(Shells *s) { return s->iadc.data(); }
void step(Shells *, const double *, const double *, const double *, double *,
          double, double, double &, int &, int &, int) {}
void energy(const Shells *, double &eint, double &ehour) {
  eint = 0;
  ehour = 0;
}
int rwall_add(Shells *, const double *, const double *, double) { return -1; }
void rwall_apply(Shells *, int, const double *, double *, const double *,
                 double) {}

}  // namespace rg_oracle_shell
