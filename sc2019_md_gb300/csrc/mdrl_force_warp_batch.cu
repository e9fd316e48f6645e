/*
 * mdrl_force_warp_batch.cu — the one-warp-per-item force-kernel instantiations for batches: the
 * half-shell units of the replicas that have at least 3 cells per axis (per-unit shift), and the
 * explicit cell pairs of the replicas whose edges all exceed 2 rc with fewer cells (per-pair
 * wrap); int64 fixed point; one translation unit so that the sets compile in parallel with the
 * others.
 */
#include "mdrl_force_warp.cuh"

namespace mdrl {

warp_fn pick_force_warp_batch(int order, bool sep, bool extra, bool cell_pairs) {
    auto w = [&](auto ord, auto sp, auto ex) -> warp_fn {
        constexpr int O = decltype(ord)::value;
        constexpr bool S = decltype(sp)::value, E = decltype(ex)::value;
        return cell_pairs ? (warp_fn)k_force_warp<O, S, E, 0, kDiffWrap, true>
                          : (warp_fn)k_force_warp<O, S, E, 0, kDiffShift, true>;
    };
    auto se = [&](auto ord) -> warp_fn {
        using T = std::true_type;
        using F = std::false_type;
        if (sep) return extra ? w(ord, T{}, T{}) : w(ord, T{}, F{});
        return extra ? w(ord, F{}, T{}) : w(ord, F{}, F{});
    };
    switch (order) {
        case 0: return se(std::integral_constant<int, 0>{});
        case 1: return se(std::integral_constant<int, 1>{});
        case 2: return se(std::integral_constant<int, 2>{});
        default: return se(std::integral_constant<int, 3>{});
    }
}

}  // namespace mdrl
