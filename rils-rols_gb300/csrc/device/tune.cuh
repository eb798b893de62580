// Launch-shape tuner (tune.cu): picks, per knob, column bucket and row class,
// the fastest of a knob's launch shapes by timing each on a real launch.  Only
// shapes that leave every result bit unchanged are knobs, so a choice changes
// speed only.
#pragma once
#include <cstdint>

namespace rrd {

enum TuneKnob {
  TK_EVAL_WAVES = 1,  // FP64 evaluator: blocks per level launch = waves x SMs (bucket 0)
  TK_FAC_GROUP = 2,   // double-float evaluator: factors per block (bucket 0); each factor's
                      // values and sums are computed alone, whatever its block-mates
  TK_PAIR_UNIT = 3,   // pair sums: partners per block at most (bucket 0); each pair's sum is
                      // formed alone, a long partner list only spreads over more blocks
  TK_FAC_STAGE = 4,   // double-float evaluator: 2 stages a chunk's X and y rows in shared memory by
                      // tensor copies, 1 reads them from global memory (bucket: feature count d)
  TK_COUNT = 5  // knob 0 is retired
};

// Values of a knob in a bucket, the default first; returns how many (<= 4).
int tune_variants(int knob, int bucket, int* out);
// Row class of a dataset: floor(log2(n)).
int tune_row_class(int64_t n);
// The value a launch uses: a pinned value, else the tuned one, else the
// default.  *trial is set when the tuner is on and has no choice for the key
// yet (the caller then times every variant, if the launch carries enough work,
// and reports through tune_store).
int tune_pick(int knob, int bucket, int64_t n, bool* trial);
void tune_store(int knob, int bucket, int64_t n, const int* vals, const float* ms, int cnt);
// Device work below which a launch is not timed for the tuner (row-candidates).
constexpr int64_t kTuneMinWork = int64_t(1) << 20;

}  // namespace rrd
