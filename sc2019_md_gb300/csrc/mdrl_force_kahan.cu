/*
 * mdrl_force_kahan.cu — instantiations of the half-shell force kernel with
 * compensated (high + low plane) FP32 accumulation (one translation unit per accumulation mode so
 * that they compile in parallel).
 */
#include "mdrl_force.cuh"

namespace mdrl {

template <int ORDER, bool SEP, bool EXTRA>
static force_fn pick_wrap_2(bool wrap) {
    return wrap ? (force_fn)k_force<ORDER, SEP, EXTRA, 2, true> : (force_fn)k_force<ORDER, SEP, EXTRA, 2, false>;
}

template <int ORDER>
static force_fn pick_order_2(bool sep, bool extra, bool wrap) {
    if (sep) return extra ? pick_wrap_2<ORDER, true, true>(wrap) : pick_wrap_2<ORDER, true, false>(wrap);
    return extra ? pick_wrap_2<ORDER, false, true>(wrap) : pick_wrap_2<ORDER, false, false>(wrap);
}

force_fn pick_force_acc2(int order, bool sep, bool extra, bool wrap) {
    switch (order) {
        case 0: return pick_order_2<0>(sep, extra, wrap);
        case 1: return pick_order_2<1>(sep, extra, wrap);
        case 2: return pick_order_2<2>(sep, extra, wrap);
        default: return pick_order_2<3>(sep, extra, wrap);
    }
}

}  // namespace mdrl
