/*
 * mdrl_force_batch.cu — the force-kernel instantiations for batched replicas (int64 fixed point, 4 warps, difference rule per work item): one
 * instantiation set per translation unit so that the sets compile in parallel.
 */
#include "mdrl_force.cuh"

namespace mdrl {

template force_fn pick_batch_set<false>(int, bool, bool);

}  // namespace mdrl
