// Tile-shape variants of the evaluation kernels, selected at run time from a
// table that the autotuner (gempy_gb300/autotune.py) fills by timing every
// variant on the device and persisting the winners per GPU.
#pragma once

#include "gk_common.cuh"

namespace gk {

struct TuneVariant {
    int ppt;       // grid points per thread
    int stage_kb;  // bytes of one record stage in shared memory (two stages)
};

constexpr int kTuneVariants = 4;
constexpr TuneVariant kTuneTable[kTuneVariants] = {{4, 32}, {2, 32}, {4, 16}, {2, 16}};

TuneVariant tune_variant(int tunable);

}  // namespace gk
