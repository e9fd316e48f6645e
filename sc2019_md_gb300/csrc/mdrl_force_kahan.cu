/*
 * mdrl_force_kahan.cu — the force-kernel instantiations for compensated (high + low plane) FP32 accumulation: one
 * instantiation set per translation unit so that the sets compile in parallel.
 */
#include "mdrl_force.cuh"

namespace mdrl {

template force_fn pick_force_set<2, 4, false, kDiffShift>(int, bool, bool);

}  // namespace mdrl
