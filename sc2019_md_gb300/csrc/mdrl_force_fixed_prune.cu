/*
 * mdrl_force_fixed_prune.cu — the force-kernel instantiations for int64 fixed-point accumulation, 4 warps per CTA, survivor-list pruning: one
 * instantiation set per translation unit so that the sets compile in parallel.
 */
#include "mdrl_force.cuh"

namespace mdrl {

template force_fn pick_force_set<0, 4, true, kDiffShift>(int, bool, bool);

}  // namespace mdrl
