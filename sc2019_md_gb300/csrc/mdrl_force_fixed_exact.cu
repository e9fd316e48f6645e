/*
 * mdrl_force_fixed_exact.cu — the force-kernel instantiations for int64 fixed-point accumulation, 4 warps per CTA, with the exact-difference
 * rule (MDRL_FLAG_EXACT_DIFF): one instantiation set per translation unit so that the sets compile
 * in parallel.
 */
#include "mdrl_force.cuh"

namespace mdrl {

template force_fn pick_force_set<0, 4, false, kDiffExact>(int, bool, bool);

}  // namespace mdrl
