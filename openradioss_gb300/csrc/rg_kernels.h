// Launch wrappers shared between the translation units of librg.
#pragma once
#include "rg_device.cuh"

namespace rg {

int hexa_blocks(int nel);
void launch_hexa_f64(const HexaParams &P, const HexaArrays<double> &A,
                     const NodeView &N, dbl4 *fsky, DtPartials dp,
                     Time *T, int *status, const DtFinish &F, cudaStream_t s);
void launch_hexa_f32(const HexaParams &P, const HexaArrays<float> &A,
                     const NodeView &N, float4 *fsky, DtPartials dp,
                     Time *T, int *status, const DtFinish &F, cudaStream_t s);
void launch_hexa_prev_volume(const HexaArrays<float> &A, const NodeView &N, const Time *T,
                             cudaStream_t s);

// Belytschko-Tsay shells (rg_shell.cu)
struct ShellParams;
template <typename ER>
struct ShellArrays;
int shell_blocks(int nel);

}  // namespace rg
