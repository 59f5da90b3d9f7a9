// Register-resident refined build, system sizes of the fused gradient + Laplacian build (PHS5, degree 2, k = 40).
#include "stencil_refined_reg.cuh"

#define RBF_LAUNCH_NO_VARIANT 1000

int rbf_launch_refined_reg_b(rbf_ctx *ctx, const StencilParams &P) {
    if (P.n == 50 && P.nops == 4) return launch_refined_reg<50, 4>(ctx, P);
    return RBF_LAUNCH_NO_VARIANT;
}
