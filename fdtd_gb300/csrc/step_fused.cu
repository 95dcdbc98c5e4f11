// step_fused.cu -- single-pass step (H, D, sources, E) followed by Mur.
#include "native.cuh"

namespace fdtd {

// H (out of place), D, sources and E of one step.
int launch_h_de_fused(const NativeConsts &c, cudaStream_t s)
{
    int st = launch_h(c, s);
    if (st == FDTD_OK)
        st = launch_de(c, s);
    return st;
}

int launch_step(const NativeConsts &c, cudaStream_t s)
{
    int st = launch_h_de_fused(c, s);
    if (st == FDTD_OK)
        st = launch_mur(c, s);
    return st;
}

int step_kernels(int kernel_kind, StepKernel *out, int max)
{
    StepKernel single[] = {{"fused_step", launch_h_de_fused}, {"mur", launch_mur}};
    StepKernel two[] = {{"h", launch_h}, {"de", launch_de}, {"mur", launch_mur}};
    const StepKernel *src = kernel_kind == FDTD_KERNEL_SINGLE_PASS ? single : two;
    const int n = kernel_kind == FDTD_KERNEL_SINGLE_PASS ? 2 : 3;
    for (int k = 0; k < n && k < max; k++)
        out[k] = src[k];
    return n;
}

}  // namespace fdtd
