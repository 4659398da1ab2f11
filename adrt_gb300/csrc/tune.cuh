// Launch-configuration table of the autotuner (tune.cu).
#pragma once

#include "common.cuh"

namespace adrtg {

struct TuneConfig {
  int width = 0;      // forward tile width in offsets: 128 or 256 (0 = by size)
  int max_fused = 0;  // stages fused in shared memory per pass, 1..5 (0 = 5)
  int chunk_mb = 0;   // L2 budget of one chunk's intermediate in MB (0 = built-in)
  int use_fast = -1;  // float32 fast forward kernels: 1 on, 0 off, -1 = when eligible
};

TuneConfig tune_lookup(int op, int dtype, i64 n);

// Splits L stages into passes of at most max_fused stages, as even as
// possible; returns the number of passes.
int plan_stage_split(int L, int max_fused, int *sizes);

}  // namespace adrtg
