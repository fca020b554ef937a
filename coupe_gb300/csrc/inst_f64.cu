// Rcb with f64 keys, cuts and split positions (COUPE_GPU_F64).
#include "runner.cuh"

namespace cg {
int run_rcb_f64(DevCtx &C, const RunArgs &a, coupe_gpu_stats *st, std::string *err) {
    return run_mode<KeyF64>(C, a, st, err);
}
}  // namespace cg
