/*
 * mdrl_force_warp_fixed_exact.cu — the one-warp-per-item force-kernel instantiations for int64
 * fixed-point accumulation with the exact-difference rule (MDRL_FLAG_EXACT_DIFF): one instantiation set per translation unit so
 * that the sets compile in parallel.
 */
#include "mdrl_force_warp.cuh"

namespace mdrl {

template warp_fn pick_force_warp_set<0, kDiffExact>(int, bool, bool);

}  // namespace mdrl
