// Minimizer index of the graph and per-read seed selection (host side of the
// seeding path; the k-mer lookups run in seed_kernel.cu).
//
// The index is MinimizerSeeder's with one bucket (the reference's layout for
// -t 1, MinimizerSeeder.cpp:299-491): minimizers of every bigraph node in
// AlignmentGraph::nodeLookup order, stored as (split node << 6) | offset and
// grouped per k-mer.  A k-mer's dense id is its rank among the distinct k-mers
// (the reference uses a minimal perfect hash there; the id only matters through
// initMaxCount, MinimizerSeeder.cpp:557-575, which skips the last id).
#include <algorithm>
#include <cmath>
#include <deque>
#include <limits>
#include <tuple>
#include <unordered_map>
#include "readalign.h"

namespace gahost
{

struct IndexFailure {};

static inline bool validChar(char c)
{
    return c == 'a' || c == 'A' || c == 'c' || c == 'C' || c == 'g' || c == 'G' || c == 't' || c == 'T';
}

static inline uint64_t charToInt(char c)
{
    switch (c)
    {
        case 'a': case 'A': return 0;
        case 'c': case 'C': return 1;
        case 'g': case 'G': return 2;
        case 't': case 'T': return 3;
    }
    return 0;
}

// MinimizerSeeder.cpp:45-54 (Thomas Wang's 64-bit integer hash, as cited there)
static inline uint64_t kmerHash(uint64_t key)
{
    key = (~key) + (key << 21);
    key = key ^ (key >> 24);
    key = (key + (key << 3)) + (key << 8);
    key = key ^ (key >> 14);
    key = (key + (key << 2)) + (key << 4);
    key = key ^ (key >> 28);
    key = key + (key << 31);
    return key;
}

// iterateMinimizersReal (MinimizerSeeder.cpp:104-189): all (window) minimizers,
// ties in hash reported together, restarting after non-ACGT characters
template <typename F>
static void iterateMinimizers(const std::string& str, size_t k, size_t windowSize, F callback)
{
    if (str.size() < k) return;
    const size_t realWindow = windowSize - k + 1;
    const uint64_t mask = ~(0xFFFFFFFFFFFFFFFFULL << (k * 2));
    size_t offset = 0;
    std::deque<std::tuple<size_t, uint64_t, uint64_t>> window;
start:
    while (offset < str.size() && !validChar(str[offset])) offset++;
    if (offset + windowSize > str.size()) return;
    {
        uint64_t kmer = 0;
        for (size_t i = 0; i < k; i++)
        {
            if (!validChar(str[offset + i]))
            {
                offset += i;
                goto start;
            }
            kmer <<= 2;
            kmer |= charToInt(str[offset + i]);
        }
        window.clear();
        window.emplace_back(offset + k - 1, kmer, kmerHash(kmer));
        for (size_t i = k; i < k + realWindow; i++)
        {
            if (!validChar(str[offset + i]))
            {
                offset += i;
                goto start;
            }
            kmer <<= 2;
            kmer &= mask;
            kmer |= charToInt(str[offset + i]);
            uint64_t hashed = kmerHash(kmer);
            while (!window.empty() && std::get<2>(window.back()) > hashed) window.pop_back();
            window.emplace_back(offset + i, kmer, hashed);
        }
        auto iter = window.begin();
        while (iter != window.end() && std::get<2>(*iter) == std::get<2>(window.front()))
        {
            callback(std::get<0>(*iter), std::get<1>(*iter));
            ++iter;
        }
        for (size_t i = k + realWindow; offset + i < str.size(); i++)
        {
            if (!validChar(str[offset + i]))
            {
                offset += i;
                goto start;
            }
            kmer <<= 2;
            kmer &= mask;
            kmer |= charToInt(str[offset + i]);
            uint64_t hashed = kmerHash(kmer);
            uint64_t oldMinimum = std::get<2>(window.front());
            bool frontPopped = false;
            while (!window.empty() && std::get<0>(window.front()) <= offset + i - realWindow)
            {
                frontPopped = true;
                window.pop_front();
            }
            if (frontPopped)
            {
                while (window.size() >= 2 && std::get<2>(window.front()) == std::get<2>(*(window.begin() + 1))) window.pop_front();
            }
            while (!window.empty() && std::get<2>(window.back()) > hashed) window.pop_back();
            window.emplace_back(offset + i, kmer, hashed);
            if (std::get<2>(window.front()) != oldMinimum)
            {
                auto it2 = window.begin();
                while (it2 != window.end() && std::get<2>(*it2) == std::get<2>(window.front()))
                {
                    callback(std::get<0>(*it2), std::get<1>(*it2));
                    ++it2;
                }
            }
            else if (std::get<2>(window.back()) == std::get<2>(window.front()))
            {
                callback(std::get<0>(window.back()), std::get<1>(window.back()));
            }
        }
    }
}

// MinimizerSeeder::initMinimizers + initMaxCount with one bucket (MinimizerSeeder.cpp:299-491, 557-575)
void buildMinimizerIndex(const HostGraph& g, size_t k, size_t w, double keepLeastFrequentFraction, MinimizerIndex& idx)
{
    idx.k = k;
    idx.w = w;
    std::unordered_map<size_t, size_t> nodeMinimizerStart;
    for (size_t i = 0; i < g.N; i++)
    {
        size_t id = (size_t)(int64_t)g.nodeIds[i];
        size_t& m = nodeMinimizerStart[id];
        bool skipStart = false;
        for (uint32_t e = g.inOff[i]; e < g.inOff[i + 1]; e++)
        {
            if (g.nodeIds[g.inNb[e]] != g.nodeIds[i])
            {
                skipStart = true;
                break;
            }
        }
        if (skipStart) m = std::max(m, (size_t)g.nodeOffset[i]);
    }
    // minimizers of every bigraph node in nodeLookup order: nodes are scanned on all cores
    // into per-node lists, which are then concatenated in that order (the serial order)
    const size_t numLookup = g.lookupIds.size();
    std::vector<std::vector<std::pair<uint64_t, uint64_t>>> perNode(numLookup);
    parallelFor(numLookup, [&](size_t li)
    {
        int nodeId = g.lookupIds[li];
        std::string sequence(g.originalSize[li], 'N');
        for (size_t pos = 0; pos < sequence.size(); pos++)
        {
            size_t here = g.unitigNode(nodeId, pos);
            sequence[pos] = g.charAt(here, pos - g.nodeOffset[here]);
        }
        const size_t minStart = nodeMinimizerStart.at((size_t)(int64_t)nodeId);
        auto& out = perNode[li];
        iterateMinimizers(sequence, k, w, [&](size_t pos, uint64_t kmer)
        {
            if (pos < minStart) return;
            size_t splitNode = g.unitigNode(nodeId, pos);
            size_t remaining = pos - g.nodeOffset[splitNode];
            out.emplace_back(kmer, ((uint64_t)splitNode << 6) + remaining);
        });
    });
    size_t total = 0;
    for (const auto& v : perNode) total += v.size();
    std::vector<uint64_t> kmers, positions;
    kmers.reserve(total);
    positions.reserve(total);
    for (auto& v : perNode)
    {
        for (const auto& kp : v)
        {
            kmers.push_back(kp.first);
            positions.push_back(kp.second);
        }
        std::vector<std::pair<uint64_t, uint64_t>>().swap(v);
    }
    idx.keys = kmers;
    std::sort(idx.keys.begin(), idx.keys.end());
    idx.keys.erase(std::unique(idx.keys.begin(), idx.keys.end()), idx.keys.end());
    auto rank = [&](uint64_t kmer) -> size_t { return std::lower_bound(idx.keys.begin(), idx.keys.end(), kmer) - idx.keys.begin(); };
    // the rank of every k-mer occurrence (binary searches on all cores), then the serial
    // counting sort that fixes the positions' order within a k-mer
    std::vector<uint32_t> ranks(kmers.size());
    parallelFor((kmers.size() + 4095) / 4096, [&](size_t c)
    {
        const size_t end = std::min(kmers.size(), (c + 1) * 4096);
        for (size_t i = c * 4096; i < end; i++) ranks[i] = (uint32_t)rank(kmers[i]);
    });
    idx.startPos.assign(idx.keys.size() + 1, 0);
    for (uint32_t r : ranks) idx.startPos[r] += 1;
    for (size_t i = 1; i < idx.startPos.size(); i++) idx.startPos[i] += idx.startPos[i - 1];
    idx.positions.assign(kmers.size(), 0);
    for (size_t i = 0; i < kmers.size(); i++)
    {
        const size_t r = ranks[i];
        idx.startPos[r] -= 1;
        idx.positions[idx.startPos[r]] = positions[i];
    }
    idx.maxCount = 0;
    std::vector<size_t> counts;
    if (idx.keys.size() > 0)
    {
        for (size_t i = 0; i + 1 < idx.keys.size(); i++) counts.push_back(idx.startPos[i + 1] - idx.startPos[i]);
    }
    std::sort(counts.begin(), counts.end());
    if (counts.size() == 0) return;
    size_t index = counts.size() * keepLeastFrequentFraction;
    if (index == counts.size()) index = counts.size() - 1;
    idx.maxCount = counts[index] + 1;
}

// iterateKmers + the lookup of MinimizerSeeder::getSeeds (MinimizerSeeder.cpp:59-102, 524-537)
void kmerMatchesHost(const MinimizerIndex& idx, const std::string& str, std::vector<KmerMatch>& out)
{
    out.clear();
    const size_t k = idx.k;
    const size_t realWindow = idx.w - k + 1;
    if (str.size() < k) return;
    const uint64_t mask = ~(0xFFFFFFFFFFFFFFFFULL << (k * 2));
    auto emit = [&](size_t pos, uint64_t kmer)
    {
        auto f = std::lower_bound(idx.keys.begin(), idx.keys.end(), kmer);
        if (f == idx.keys.end() || *f != kmer) return;
        size_t r = f - idx.keys.begin();
        uint64_t start = idx.startPos[r];
        uint64_t count = idx.startPos[r + 1] - start;
        if (count >= idx.maxCount) return;
        out.push_back(KmerMatch { pos, start, count });
    };
    size_t offset = 0;
start:
    while (offset < str.size() && !validChar(str[offset])) offset++;
    if (offset + k > str.size()) return;
    {
        uint64_t kmer = 0;
        for (size_t i = 0; i < k; i++)
        {
            if (!validChar(str[offset + i]))
            {
                offset += i;
                goto start;
            }
            kmer <<= 2;
            kmer |= charToInt(str[offset + i]);
        }
        emit(offset + k - 1, kmer);
        uint64_t lastKmer = kmer;
        size_t lastPos = offset + k - 1;
        for (size_t i = k; offset + i < str.size(); i++)
        {
            if (!validChar(str[offset + i]))
            {
                offset += i;
                goto start;
            }
            kmer <<= 2;
            kmer &= mask;
            kmer |= charToInt(str[offset + i]);
            if (lastKmer != kmer || lastPos <= offset + i - realWindow)
            {
                emit(offset + i, kmer);
                lastKmer = kmer;
                lastPos = offset + i;
            }
        }
    }
}

// MinimizerSeeder::addMinimizers + matchToSeedHit (MinimizerSeeder.cpp:493-519, 538-555)
void selectSeeds(const HostGraph& g, const MinimizerIndex& idx, const std::string& seq, double density,
    std::vector<KmerMatch>& matches, std::vector<SeedHit>& out)
{
    out.clear();
    size_t maxHits = seq.size() * density;
    if (density == -1) maxHits = std::numeric_limits<size_t>::max();
    std::sort(matches.begin(), matches.end(), [](const KmerMatch& a, const KmerMatch& b) { return a.count < b.count; });
    size_t seedsHere = 0;
    size_t allowedCount = 0;
    for (const auto& m : matches)
    {
        size_t start = m.start;
        size_t end = start + m.count;
        if (seedsHere >= maxHits && end - start > allowedCount) break;
        allowedCount = end - start;
        for (size_t i = start; i < end; i++)
        {
            uint64_t mergepos = idx.positions[i];
            size_t nodeId = mergepos >> 6;
            size_t offset = mergepos & 63;
            SeedHit s;
            s.nodeID = g.nodeIds[nodeId] / 2;
            s.nodeOffset = offset + g.nodeOffset[nodeId];
            s.seqPos = m.pos;
            s.matchLen = idx.k;
            s.rawSeedGoodness = idx.maxCount - (int)m.count;
            s.reverse = g.reverse[nodeId] != 0;
            s.alignmentGraphNodeId = nodeId;
            s.alignmentGraphNodeOffset = offset;
            out.push_back(s);
        }
        seedsHere += end - start;
    }
}

}
