// Split-row register refined build, 40-row single-operator systems (k = 30 stencils with
// degree-2 polynomials in 3D: the 3D Laplacian and regrid workloads).
#include "stencil_refined_split.cuh"

#define RBF_LAUNCH_NO_VARIANT 1000

int rbf_launch_refined_split(rbf_ctx *ctx, const StencilParams &P) {
    if (P.n == 40 && P.nops == 1 && P.defer) return launch_refined_split<40>(ctx, P);
    return RBF_LAUNCH_NO_VARIANT;
}
