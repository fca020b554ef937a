// Internal interface of the allocation-free split (split_noalloc.cu).
#pragma once

#include <stdint.h>

#include "../../include/coupe.h"

namespace cg {

// Most points one call splits (positions and chunk geometry stay in range).
constexpr uint64_t SPLIT_MAX_POINTS = 0xffffffffull;

// Returns a coupe_err; on error *msg is a static message.
int split_noalloc(uint64_t n, uint64_t dimension, const double *d_points, int weight_type, const void *d_weights,
                  uint64_t coord, double cut, double *d_out_points, void *d_out_weights, uint64_t *n_left,
                  void *stream, const char **msg);

}  // namespace cg
