// Register-resident refined build, system sizes of the k = 20 stencils of the 2D and regrid
// workloads (single operator; the 40-row systems go to the split-row kernel,
// stencil_refined_c.cu).
#include "stencil_refined_reg.cuh"

#define RBF_LAUNCH_NO_VARIANT 1000

int rbf_launch_refined_reg_a(rbf_ctx *ctx, const StencilParams &P) {
    if (P.n == 26 && P.nops == 1) return launch_refined_reg<26, 1>(ctx, P);
    if (P.n == 24 && P.nops == 1) return launch_refined_reg<24, 1>(ctx, P);
    return RBF_LAUNCH_NO_VARIANT;
}
