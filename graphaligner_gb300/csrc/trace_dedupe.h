// GraphAlignerBitvectorBanded::removeDuplicateTraces (GraphAlignerBitvectorBanded.h:144-169) on
// trace summaries: the multiseed DP's traces sorted by the X-score of their read span (std::sort,
// best first), then of two traces that start at the same cell the later one is swapped with the
// last and popped.  Sorting summaries makes the same comparisons and moves as sorting the traces,
// so the order is the reference's.  Used by the device path (on the summaries the kernels give)
// and by the host read flow (on packed traces).
#pragma once
#include <algorithm>
#include <cstddef>
#include <cstdint>
#include <vector>

namespace gahost
{

struct DedupeKey
{
    int32_t sortScore;
    uint32_t index;
    uint64_t start;      // the trace's last item (its start): cell and read position, packed
};

// the sort key, in the reference's 32-bit arithmetic: (span + 1) * 100 - score * cost
inline int32_t dedupeScore(size_t firstSeqPos, size_t lastSeqPos, int32_t score, int32_t cost)
{
    const uint32_t span = (uint32_t)((firstSeqPos - lastSeqPos + 1) * 100);
    return (int32_t)(span - (uint32_t)score * (uint32_t)cost);
}

// keys in the traces' order; returns the surviving traces' indices in their final order
inline std::vector<uint32_t> dedupeOrder(std::vector<DedupeKey>& keys)
{
    if (keys.empty()) return {};
    std::sort(keys.begin(), keys.end(), [](const DedupeKey& left, const DedupeKey& right) { return left.sortScore > right.sortScore; });
    for (size_t i = keys.size() - 1; i > 0; i--)
    {
        for (size_t j = 0; j < i; j++)
        {
            if (keys[i].start == keys[j].start)
            {
                std::swap(keys[i], keys.back());
                keys.pop_back();
                break;
            }
        }
    }
    std::vector<uint32_t> order(keys.size());
    for (size_t k = 0; k < keys.size(); k++) order[k] = keys[k].index;
    return order;
}

}
