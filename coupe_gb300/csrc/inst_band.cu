// Rcb with f32 keys and f64 cuts, the keys' band re-decided in f64
// (COUPE_GPU_F32KEY_F64BAND): the decisions of COUPE_GPU_F64.
#include "runner.cuh"

namespace cg {
int run_rcb_band(DevCtx &C, const RunArgs &a, coupe_gpu_stats *st, std::string *err) {
    return run_mode<KeyBand>(C, a, st, err);
}
}  // namespace cg
