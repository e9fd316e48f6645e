/*
 * mdrl_force_batch_prune.cu — the force-kernel instantiations for batched replicas with survivor-list pruning: one
 * instantiation set per translation unit so that the sets compile in parallel.
 */
#include "mdrl_force.cuh"

namespace mdrl {

template force_fn pick_batch_set<true>(int, bool, bool);

}  // namespace mdrl
