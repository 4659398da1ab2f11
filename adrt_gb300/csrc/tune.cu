// Launch-configuration table consulted by the forward and transposed
// (bdrt) dispatchers, filled by the autotuner (adrt_gb300/tune.py) through
// adrt_gb300_tune_set.  One entry per (op, dtype, log2 n); a zero field
// means "built-in choice".  The knobs change only how the work is tiled and
// staged, never which values are added in which order, so every setting
// gives bit-identical results.
#include <atomic>

#include "common.cuh"
#include "tune.cuh"

namespace adrtg {

namespace {
constexpr int kOps = 2, kTypes = 2, kLogs = 16;
struct Entry {
  std::atomic<int> width{0}, max_fused{0}, chunk_mb{0}, use_fast{-1};
};
Entry g_table[kOps][kTypes][kLogs];

Entry *entry(int op, int dtype, i64 n) {
  if (op < 0 || op >= kOps || dtype < 0 || dtype >= kTypes || !is_pow2(n)) return nullptr;
  const int lg = num_iters(n);
  return lg < kLogs ? &g_table[op][dtype][lg] : nullptr;
}
}  // namespace

TuneConfig tune_lookup(int op, int dtype, i64 n) {
  TuneConfig c;
  const Entry *e = entry(op, dtype, n);
  if (e) {
    c.width = e->width.load(std::memory_order_relaxed);
    c.max_fused = e->max_fused.load(std::memory_order_relaxed);
    c.chunk_mb = e->chunk_mb.load(std::memory_order_relaxed);
    c.use_fast = e->use_fast.load(std::memory_order_relaxed);
  }
  return c;
}

int plan_stage_split(int L, int max_fused, int *sizes) {
  if (max_fused < 1 || max_fused > 5) max_fused = 5;
  if (L == 0) {
    sizes[0] = 0;
    return 1;
  }
  const int P = (L + max_fused - 1) / max_fused;
  for (int p = 0; p < P; ++p) sizes[p] = L / P + (p < L % P ? 1 : 0);
  return P;
}

}  // namespace adrtg

using namespace adrtg;

extern "C" int adrt_gb300_tune_set(int op, int dtype, int64_t n, int width, int max_fused, int chunk_mb,
                                   int use_fast) {
  Entry *e = entry(op, dtype, n);
  if (!e) return ADRT_GB300_ERR_SHAPE;
  if (!(width == 0 || width == 128 || width == 256) || max_fused < 0 || max_fused > 5 || chunk_mb < 0 ||
      chunk_mb > 65536 || use_fast < -1 || use_fast > 1)
    return ADRT_GB300_ERR_SHAPE;
  e->width.store(width);
  e->max_fused.store(max_fused);
  e->chunk_mb.store(chunk_mb);
  e->use_fast.store(use_fast);
  return ADRT_GB300_OK;
}

extern "C" int adrt_gb300_tune_get(int op, int dtype, int64_t n, int *width, int *max_fused, int *chunk_mb,
                                   int *use_fast) {
  if (!width || !max_fused || !chunk_mb || !use_fast) return ADRT_GB300_ERR_NULL;
  if (!entry(op, dtype, n)) return ADRT_GB300_ERR_SHAPE;
  const TuneConfig c = tune_lookup(op, dtype, n);
  *width = c.width;
  *max_fused = c.max_fused;
  *chunk_mb = c.chunk_mb;
  *use_fast = c.use_fast;
  return ADRT_GB300_OK;
}

extern "C" void adrt_gb300_tune_reset(void) {
  for (auto &a : g_table)
    for (auto &b : a)
      for (auto &e : b) {
        e.width.store(0);
        e.max_fused.store(0);
        e.chunk_mb.store(0);
        e.use_fast.store(-1);
      }
}
