/*
 * mdrl_force_atomic.cu — the force-kernel instantiations for FP32-atomic accumulation ("plain"): one
 * instantiation set per translation unit so that the sets compile in parallel.
 */
#include "mdrl_force.cuh"

namespace mdrl {

template force_fn pick_force_set<1, 4, false, kDiffShift>(int, bool, bool);

}  // namespace mdrl
