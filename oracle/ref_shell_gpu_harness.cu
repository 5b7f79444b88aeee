// Timing harness of the reference's own CUDA shell path -- a SPEED
// COMPARATOR, test / benchmark infrastructure only (never part of the
// product, never a parity oracle: the reference GPU path assembles with
// atomicAdd and uses its own through-thickness rule).
//
// It drives the reference's C entry points unchanged
// (engine/source/elements/shell/coque/shell_gpu_driver.h:302-477, built from
// the reference's own sources with -DMYREAL8 by the Makefile's ref_gpu
// target) the way its Fortran engine does (shell_gpu_mod.F90, resol.F:3670,
// 4295): one global node handle, one shell handle, Johnson-Cook and hourglass
// parameters, constants and point state uploaded once, then per step
//   kernels only:  shell_gpu_run_kernels (zeroing + geometry + strain and
//                  material + forces with atomic assembly), CUDA events on
//                  the handle's stream;
//   full step:     global upload of X, V, VR (pinned) -> the three kernels
//                  -> download of the 8*NUMNOD force record, synchronised;
//                  wall time.
// The node state is held fixed (the reference path leaves the nodal update
// to the host engine), as in a FORINT-level call.
//
// The reference's strain/material kernel is instantiated for ISMSTR 1, 2
// and 11 only; ISMSTR = 2 (large strain until a small-strain switch that a
// positive OFF never triggers) is the formulation timed here.
#include <cuda_runtime.h>

#include <chrono>
#include <cmath>
#include <vector>

#include "shell_gpu_driver.h"

extern "C" {
// Reference entry points defined in shell_gpu_driver.cu but not declared in
// its header.
ShellGPUData *shell_gpu_data_create();
void shell_gpu_data_destroy(ShellGPUData *g);
void shell_gpu_set_mat_params(ShellGPUData *g, Real E, Real nu, Real G, Real A11, Real A12,
                              Real CA, Real CB, Real CN, Real CC, Real EPDR, Real EPMX,
                              Real YMAX, Real M_EXP, Real FISOKIN, Real RHOCP, Real TREF,
                              Real TMELT, Real ASRATE, Real RHO, Real SSP, Real SHF_COEF,
                              int IPLA, int VP, int IFORM, int ICC, Real Z3, Real Z4);
void shell_gpu_set_hg_params(ShellGPUData *g, Real H1, Real H2, Real H3, Real SRH1, Real SRH2,
                             Real SRH3, Real HVISC, Real HELAS, Real HVLIN);

// numelc shells, numnod nodes; ixc4[4][numelc] 0-based nodes (< numnod);
// thk[numelc]; X, V, VR [3*numnod] (xyz interleaved); mat = {E, nu, rho, A,
// B, n, C, eps0}; hg = {h1, h2, h3} (membrane, flexural, rotational
// hourglass coefficients); dt the step.  nwarm untimed steps, then nsteps
// timed ones of each kind.  out[0] = device ms per step of the kernels,
// out[1] = wall ms per full step, out[2] = sum |F| of the last step (a
// check that work was done).  Returns 0 (the reference's own checks call
// exit() on a CUDA error).
int refgpu_shell_time(int numelc, int numnod, const int *ixc4, const double *thk,
                      double *X, double *V, double *VR, const double *mat, const double *hg,
                      double dt, int nwarm, int nsteps, double *out) {
  if (numelc <= 0 || numnod <= 0 || !ixc4 || !thk || !X || !V || !VR || !mat || !hg || !out)
    return -1;
  for (int i = 0; i < 4 * numelc; i++)
    if (ixc4[i] < 0 || ixc4[i] >= numnod) return -2;
  const int NE = numelc, NN = numnod, NPT = 5;
  const double E = mat[0], nu = mat[1], rho = mat[2];
  const double G = E / (2.0 * (1.0 + nu));
  const double A11 = E / (1.0 - nu * nu), A12 = nu * A11;
  const double ssp = std::sqrt(A11 / rho);
  const double shf = 5.0 / 6.0;

  ShellGPUGlobal *gh = shell_gpu_global_create(NN);
  ShellGPUData *g = shell_gpu_data_create();
  shell_gpu_allocate(g, NE, NN, NPT, /*ISMSTR*/ 2, /*ITHK*/ 1);
  shell_gpu_set_global(g, gh);
  shell_gpu_set_mat_params(g, E, nu, G, A11, A12, mat[3], mat[4], mat[5], mat[6], mat[7],
                           /*EPMX: no rupture*/ 0.0, /*YMAX: no cap*/ 1e30, /*M_EXP*/ 1.0,
                           /*FISOKIN*/ 0.0, /*RHOCP: no heating*/ 0.0, /*TREF*/ 0.0,
                           /*TMELT: no softening*/ 0.0, /*ASRATE*/ 1.0, rho, ssp, shf,
                           /*IPLA*/ 1, /*VP*/ 0, /*IFORM*/ 0, /*ICC*/ 1, 0.0, 0.0);
  shell_gpu_set_hg_params(g, hg[0], hg[1], hg[2], std::sqrt(hg[0]), std::sqrt(hg[1]),
                          std::sqrt(hg[2]), 0.5, 0.5, 0.0);
  shell_gpu_set_compute_sti(g, 1);
  shell_gpu_set_ihbe(g, 1);

  std::vector<double> one(NE, 1.0), vssp(NE, ssp), vrho(NE, rho), vym(NE, E), vnu(NE, nu),
      va11(NE, A11), vg(NE, G), vshf(NE, shf), zip((size_t)NPT * NE, 0.0);
  shell_gpu_upload_constant(g, ixc4, ixc4 + NE, ixc4 + 2 * NE, ixc4 + 3 * NE, thk, one.data(),
                            vssp.data(), vrho.data(), vym.data(), vnu.data(), va11.data(),
                            vg.data(), vshf.data());
  shell_gpu_upload_ip_state(g, zip.data(), zip.data(), zip.data(), zip.data(), zip.data(),
                            zip.data(), zip.data(), zip.data(), zip.data(), zip.data(),
                            zip.data());
  std::vector<double> f8((size_t)8 * NN, 0.0);
  shell_gpu_global_pin_host(X, V, VR, f8.data(), NN);

  // kernels only
  shell_gpu_global_upload_nodes(gh, X, V, VR);
  shell_gpu_global_synchronize(gh);
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  for (int i = 0; i < nwarm; i++) shell_gpu_run_kernels(g, dt);
  cudaStreamSynchronize(g->stream);
  cudaEventRecord(e0, g->stream);
  for (int i = 0; i < nsteps; i++) shell_gpu_run_kernels(g, dt);
  cudaEventRecord(e1, g->stream);
  cudaEventSynchronize(e1);
  float ms = 0.f;
  cudaEventElapsedTime(&ms, e0, e1);
  out[0] = ms / nsteps;

  // full step: upload -> kernels -> force download, synchronised
  auto step = [&]() {
    shell_gpu_global_upload_nodes(gh, X, V, VR);
    shell_gpu_full_step_async(g, dt, X, V, VR, f8.data());
    shell_gpu_global_wait_su(gh, g);
    shell_gpu_global_download_forces(gh, f8.data());
    shell_gpu_global_synchronize(gh);
  };
  for (int i = 0; i < nwarm; i++) step();
  const auto t0 = std::chrono::steady_clock::now();
  for (int i = 0; i < nsteps; i++) step();
  const auto t1 = std::chrono::steady_clock::now();
  out[1] = std::chrono::duration<double, std::milli>(t1 - t0).count() / nsteps;
  double s = 0.0;
  for (size_t i = 0; i < (size_t)3 * NN; i++) s += std::fabs(f8[i]);
  out[2] = s;

  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaHostUnregister(X);
  cudaHostUnregister(V);
  cudaHostUnregister(VR);
  cudaHostUnregister(f8.data());
  shell_gpu_deallocate(g);
  shell_gpu_data_destroy(g);
  shell_gpu_global_destroy(gh);
  return 0;
}
}
