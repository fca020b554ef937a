// Rcb with coupe's f32 key arithmetic (COUPE_GPU_REF32).
#include "runner.cuh"

namespace cg {
int run_rcb_ref32(DevCtx &C, const RunArgs &a, coupe_gpu_stats *st, std::string *err) {
    return run_mode<KeyF32>(C, a, st, err);
}
}  // namespace cg
