/*
 * mdrl_force_fixed8.cu — the force-kernel instantiations for int64 fixed-point accumulation, 8 warps per CTA: one
 * instantiation set per translation unit so that the sets compile in parallel.
 */
#include "mdrl_force.cuh"

namespace mdrl {

template force_fn pick_force_set<0, 8, false, kDiffShift>(int, bool, bool);

}  // namespace mdrl
