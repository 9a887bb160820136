// pt_mixed.cu -- mixed-precision stream-function solve (FP32 smoothing and transfers, FP64
// residual and defect correction, FP64 coarse LU).
#include "pt_consts.cuh"

namespace pt {

int upload_consts_mixed(const Engine& E) { return upload_tu_consts(E); }

int multigrid_mixed(Engine& E, pt_solve_info* info) {
    (void)E;
    (void)info;
    return fail(PT_ERR_CONFIG, "mixed precision solve not built yet");
}

}  // namespace pt
