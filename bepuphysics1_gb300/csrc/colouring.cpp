#include "colouring.h"

#include <algorithm>

namespace bepugpu {

bool ColourSolverList(const int32_t* a, const int32_t* b, int32_t n, const uint8_t* dynamic, int32_t bodies,
                      Colouring& out, const uint8_t* follows) {
    out.colour.assign(n, 0);
    out.order.assign(n, 0);
    out.colours = 0;
    // Per dynamic body, a bitset of the colours already used there.  Words grow
    // on demand, so no colour limit applies.
    std::vector<std::vector<uint64_t>> used(bodies);
    for (int32_t u = 0; u < n; u++) {
        int32_t ends[2] = {a[u], b[u]};
        for (int32_t e : ends)
            if (e < -1 || e >= bodies) return false;
        if (follows && follows[u] && u > 0) {
            out.colour[u] = out.colour[u - 1];
            continue;
        }
        const std::vector<uint64_t>* sets[2] = {nullptr, nullptr};
        int ns = 0;
        for (int32_t e : ends)
            if (e >= 0 && dynamic[e]) sets[ns++] = &used[e];
        int32_t c = 0;
        for (size_t w = 0;; w++) {
            uint64_t taken = 0;
            bool any = false;
            for (int k = 0; k < ns; k++)
                if (w < sets[k]->size()) { taken |= (*sets[k])[w]; any = true; }
            if (!any || taken != ~0ull) {
                c = (int32_t)(w * 64) + (any ? __builtin_ctzll(~taken) : 0);
                break;
            }
        }
        out.colour[u] = c;
        out.colours = std::max(out.colours, c + 1);
        for (int32_t e : ends)
            if (e >= 0 && dynamic[e]) {
                auto& v = used[e];
                size_t w = (size_t)c / 64;
                if (v.size() <= w) v.resize(w + 1, 0);
                v[w] |= 1ull << (c % 64);
            }
    }
    out.offsets.assign(out.colours + 1, 0);
    for (int32_t u = 0; u < n; u++) out.offsets[out.colour[u] + 1]++;
    for (int32_t c = 0; c < out.colours; c++) out.offsets[c + 1] += out.offsets[c];
    std::vector<int32_t> cursor(out.offsets.begin(), out.offsets.end() - 1);
    for (int32_t u = 0; u < n; u++) out.order[cursor[out.colour[u]]++] = u;
    return true;
}

}  // namespace bepugpu
