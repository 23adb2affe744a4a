// Run-time selection of evaluation tile shapes (see gk_tune.h).
#include <atomic>

#include "gk_tune.h"

namespace gk {

namespace {
std::atomic<int> g_choice[GK_TUNE_COUNT] = {};
}

TuneVariant tune_variant(int tunable) {
    if (tunable < 0 || tunable >= GK_TUNE_COUNT) return kTuneTable[0];
    int v = g_choice[tunable].load(std::memory_order_relaxed);
    return kTuneTable[(v >= 0 && v < kTuneVariants) ? v : 0];
}

}  // namespace gk

using namespace gk;

extern "C" int32_t gk_tune_variants(void) { return kTuneVariants; }

extern "C" gk_status gk_tune_describe(int32_t variant, int32_t* ppt, int32_t* stage_kb) {
    if (variant < 0 || variant >= kTuneVariants || ppt == nullptr || stage_kb == nullptr) return GK_ERR_ARG;
    *ppt = kTuneTable[variant].ppt;
    *stage_kb = kTuneTable[variant].stage_kb;
    return GK_OK;
}

extern "C" gk_status gk_tune_set(int32_t tunable, int32_t variant) {
    if (tunable < 0 || tunable >= GK_TUNE_COUNT || variant < 0 || variant >= kTuneVariants) return GK_ERR_ARG;
    g_choice[tunable].store(variant, std::memory_order_relaxed);
    return GK_OK;
}

extern "C" int32_t gk_tune_get(int32_t tunable) {
    if (tunable < 0 || tunable >= GK_TUNE_COUNT) return -1;
    return g_choice[tunable].load(std::memory_order_relaxed);
}
