/*
 * mdrl_force_fixed8.cu — the 8-warp-per-CTA instantiations of the half-shell force kernel with
 * int64 fixed-point accumulation (a tile the autotuner may pick), compiled apart from the 4-warp
 * ones so that the two translation units build in parallel.
 */
#include "mdrl_force.cuh"

namespace mdrl {

template <int ORDER, bool SEP, bool EXTRA, int FW>
static force_fn pick_wrap_0(bool wrap) {
    return wrap ? (force_fn)k_force<ORDER, SEP, EXTRA, 0, true, false, FW>
                : (force_fn)k_force<ORDER, SEP, EXTRA, 0, false, false, FW>;
}

template <int ORDER, int FW>
static force_fn pick_order_0(bool sep, bool extra, bool wrap) {
    if (sep) return extra ? pick_wrap_0<ORDER, true, true, FW>(wrap) : pick_wrap_0<ORDER, true, false, FW>(wrap);
    return extra ? pick_wrap_0<ORDER, false, true, FW>(wrap) : pick_wrap_0<ORDER, false, false, FW>(wrap);
}

template <int FW>
static force_fn pick_fw_0(int order, bool sep, bool extra, bool wrap) {
    switch (order) {
        case 0: return pick_order_0<0, FW>(sep, extra, wrap);
        case 1: return pick_order_0<1, FW>(sep, extra, wrap);
        case 2: return pick_order_0<2, FW>(sep, extra, wrap);
        default: return pick_order_0<3, FW>(sep, extra, wrap);
    }
}

force_fn pick_force_acc0_w8(int order, bool sep, bool extra, bool wrap) {
    return pick_fw_0<8>(order, sep, extra, wrap);
}

}  // namespace mdrl
