/*
 * mdrl_force_warp_fixed.cu — the one-warp-per-item force-kernel instantiations for int64
 * fixed-point accumulation with the per-unit shift of the reference's difference rule: one instantiation set per translation unit so
 * that the sets compile in parallel.
 */
#include "mdrl_force_warp.cuh"

namespace mdrl {

template warp_fn pick_force_warp_set<0, kDiffShift>(int, bool, bool);

}  // namespace mdrl
