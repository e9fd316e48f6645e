/*
 * mdrl_force_batch.cu — the batched-replica instantiations of the force kernel (int64 fixed
 * point, 4 warps, difference rule chosen per work item), in their own translation unit so that
 * they compile in parallel with the single-system ones.
 */
#include "mdrl_force.cuh"

namespace mdrl {

template <int ORDER>
static force_fn pick_batch_order(bool sep, bool extra) {
    if (sep) return extra ? (force_fn)k_force<ORDER, true, true, 0, true, true, kBatchFT / 32>
                          : (force_fn)k_force<ORDER, true, false, 0, true, true, kBatchFT / 32>;
    return extra ? (force_fn)k_force<ORDER, false, true, 0, true, true, kBatchFT / 32>
                 : (force_fn)k_force<ORDER, false, false, 0, true, true, kBatchFT / 32>;
}

force_fn pick_force_batch(int order, bool sep, bool extra) {
    switch (order) {
        case 0: return pick_batch_order<0>(sep, extra);
        case 1: return pick_batch_order<1>(sep, extra);
        case 2: return pick_batch_order<2>(sep, extra);
        default: return pick_batch_order<3>(sep, extra);
    }
}

}  // namespace mdrl
