// step_policy.h -- which admitted requests a serving step renders.
#pragma once
#include <cstdint>
#include <vector>

namespace ptgpu {

// The requests of one step, as indices into `px` (the admitted requests'
// pixel counts, oldest first).  With a fill cap: oldest first while the
// pixels add up to at most fill_px, the oldest always, younger ones that fit
// after an older one did not (first fit); without it: every request.
inline std::vector<int> step_selection(const std::vector<int64_t> &px, bool fill_cap, int64_t fill_px) {
    std::vector<int> sel;
    int64_t sum = 0;
    for (int k = 0; k < (int)px.size(); ++k) {
        if (!fill_cap || sel.empty() || sum + px[k] <= fill_px) {
            sel.push_back(k);
            sum += px[k];
        }
    }
    return sel;
}

}  // namespace ptgpu
