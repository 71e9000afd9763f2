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
#include <atomic>
#include <cmath>
#include <deque>
#include <limits>
#include <tuple>
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

// A vector whose resize leaves elements uninitialised, so that large arrays are first
// touched by the threads that fill them.
template <typename T>
struct UninitAllocator : std::allocator<T>
{
    template <typename U> struct rebind { using other = UninitAllocator<U>; };
    UninitAllocator() = default;
    template <typename U> UninitAllocator(const UninitAllocator<U>&) {}
    template <typename U> void construct(U* p) noexcept { ::new ((void*)p) U; }
    template <typename U, typename... A> void construct(U* p, A&&... a) { ::new ((void*)p) U(std::forward<A>(a)...); }
};
template <typename T> using RawVec = std::vector<T, UninitAllocator<T>>;

// Stable LSD radix sort of (key, index) pairs by the low `bits` bits of key, on all
// cores: each of `parts` contiguous slices histograms a digit, the slices' buckets are
// laid out digit-major then slice-major, and each slice scatters its elements in order,
// so equal keys keep their input order.
static void radixSortPairs(RawVec<uint64_t>& key, RawVec<uint32_t>& val, unsigned bits)
{
    const size_t n = key.size();
    constexpr unsigned kDigit = 11;
    constexpr size_t kRadix = (size_t)1 << kDigit;
    const size_t parts = std::max<size_t>(1, std::min<size_t>(256, n / 65536));
    const size_t per = (n + parts - 1) / parts;
    RawVec<uint64_t> key2(n);
    RawVec<uint32_t> val2(n);
    std::vector<size_t> hist(parts * kRadix);
    for (unsigned shift = 0; shift < bits; shift += kDigit)
    {
        std::fill(hist.begin(), hist.end(), 0);
        parallelFor(parts, [&](size_t c)
        {
            size_t* h = &hist[c * kRadix];
            const size_t end = std::min(n, (c + 1) * per);
            for (size_t i = c * per; i < end; i++) h[(key[i] >> shift) & (kRadix - 1)]++;
        });
        size_t running = 0;
        for (size_t d = 0; d < kRadix; d++)
        {
            for (size_t c = 0; c < parts; c++)
            {
                const size_t count = hist[c * kRadix + d];
                hist[c * kRadix + d] = running;
                running += count;
            }
        }
        parallelFor(parts, [&](size_t c)
        {
            size_t* h = &hist[c * kRadix];
            const size_t end = std::min(n, (c + 1) * per);
            for (size_t i = c * per; i < end; i++)
            {
                const size_t to = h[(key[i] >> shift) & (kRadix - 1)]++;
                key2[to] = key[i];
                val2[to] = val[i];
            }
        });
        key.swap(key2);
        val.swap(val2);
    }
}

// MinimizerSeeder::initMinimizers + initMaxCount with one bucket (MinimizerSeeder.cpp:299-491, 557-575)
void buildMinimizerIndex(const HostGraph& g, size_t k, size_t w, double keepLeastFrequentFraction, MinimizerIndex& idx)
{
    idx.k = k;
    idx.w = w;
    const size_t numLookup = g.lookupIds.size();
    // minimizers of every bigraph node in nodeLookup order: nodes are scanned on all cores
    // into per-node lists, which are then concatenated in that order (the serial order)
    std::vector<std::vector<std::pair<uint64_t, uint64_t>>> perNode(numLookup);
    std::atomic<bool> inconsistent(false);   // a piece out of range, or a position no piece covers
    parallelFor(numLookup, [&](size_t li)
    {
        const size_t size = g.originalSize[li];
        // the node's sequence and, per position, its piece: GetUnitigNode's first piece
        // in nodeLookup order that covers the position (AlignmentGraph.cpp:812-828)
        std::string sequence(size, 'N');
        std::vector<uint32_t> pieceOf(size, UINT32_MAX);
        // minimizers start after the last piece entered from another bigraph node
        // (MinimizerSeeder.cpp:323-340)
        size_t minStart = 0;
        for (uint32_t e = g.lookupOff[li]; e < g.lookupOff[li + 1]; e++)
        {
            const uint32_t piece = g.lookupNodes[e];
            if (piece >= g.N)
            {
                inconsistent = true;
                return;
            }
            for (uint32_t p = g.inOff[piece]; p < g.inOff[piece + 1]; p++)
            {
                if (g.nodeIds[g.inNb[p]] != g.nodeIds[piece])
                {
                    minStart = std::max<size_t>(minStart, g.nodeOffset[piece]);
                    break;
                }
            }
            const size_t from = g.nodeOffset[piece], to = std::min<size_t>(size, from + g.len[piece]);
            for (size_t pos = from; pos < to; pos++)
            {
                if (pieceOf[pos] != UINT32_MAX) continue;
                pieceOf[pos] = piece;
                sequence[pos] = g.charAt(piece, pos - from);
            }
        }
        for (size_t pos = 0; pos < size; pos++)
        {
            if (pieceOf[pos] == UINT32_MAX)
            {
                inconsistent = true;
                return;
            }
        }
        auto& out = perNode[li];
        iterateMinimizers(sequence, k, w, [&](size_t pos, uint64_t kmer)
        {
            if (pos < minStart) return;
            const size_t splitNode = pieceOf[pos];
            const size_t remaining = pos - g.nodeOffset[splitNode];
            out.emplace_back(kmer, ((uint64_t)splitNode << 6) + remaining);
        });
    });
    if (inconsistent) throw IndexFailure {};
    std::vector<size_t> firstOf(numLookup + 1, 0);
    for (size_t li = 0; li < numLookup; li++) firstOf[li + 1] = firstOf[li] + perNode[li].size();
    const size_t total = firstOf[numLookup];
    if (total >= ((size_t)1 << 32)) throw IndexFailure {};
    RawVec<uint64_t> kmers(total), positions(total);
    RawVec<uint32_t> order(total);
    parallelFor(numLookup, [&](size_t li)
    {
        size_t at = firstOf[li];
        for (const auto& kp : perNode[li])
        {
            kmers[at] = kp.first;
            positions[at] = kp.second;
            order[at] = (uint32_t)at;
            at++;
        }
        std::vector<std::pair<uint64_t, uint64_t>>().swap(perNode[li]);
    });
    // k-mers in increasing order, occurrences of one k-mer in insertion order; a k-mer's id
    // is its rank among the distinct k-mers
    radixSortPairs(kmers, order, (unsigned)(2 * k));
    size_t distinct = 0;
    for (size_t i = 0; i < total; i++) distinct += i == 0 || kmers[i] != kmers[i - 1];
    idx.keys.resize(distinct);
    idx.startPos.resize(distinct + 1);
    for (size_t i = 0, r = 0; i < total; i++)
    {
        if (i == 0 || kmers[i] != kmers[i - 1])
        {
            idx.keys[r] = kmers[i];
            idx.startPos[r] = i;
            r++;
        }
    }
    idx.startPos[distinct] = total;
    RawVec<uint64_t>().swap(kmers);
    // within a k-mer, the reference's counting sort leaves the occurrences in reverse
    // insertion order
    idx.positions.assign(total, 0);
    const size_t numKeys = idx.keys.size();
    parallelFor((numKeys + 4095) / 4096, [&](size_t c)
    {
        const size_t end = std::min(numKeys, (c + 1) * 4096);
        for (size_t r = c * 4096; r < end; r++)
        {
            const size_t from = idx.startPos[r], to = idx.startPos[r + 1];
            for (size_t j = from; j < to; j++) idx.positions[from + (to - 1 - j)] = positions[order[j]];
        }
    });
    // initMaxCount: the occurrence count at the keep fraction of the sorted counts of every
    // id but the last, plus one (read off a histogram of the counts)
    idx.maxCount = 0;
    if (numKeys < 2) return;
    const size_t numCounts = numKeys - 1;
    size_t largest = 0;
    for (size_t r = 0; r < numCounts; r++) largest = std::max<size_t>(largest, idx.startPos[r + 1] - idx.startPos[r]);
    std::vector<size_t> histogram(largest + 1, 0);
    for (size_t r = 0; r < numCounts; r++) histogram[idx.startPos[r + 1] - idx.startPos[r]]++;
    size_t index = numCounts * keepLeastFrequentFraction;
    if (index == numCounts) index = numCounts - 1;
    size_t seen = 0;
    for (size_t c = 0; c <= largest; c++)
    {
        seen += histogram[c];
        if (seen > index)
        {
            idx.maxCount = c + 1;
            break;
        }
    }
}

uint64_t seedTableCapacity(const MinimizerIndex& idx)
{
    uint64_t capacity = 16;
    while (capacity < 2 * idx.keys.size()) capacity <<= 1;
    return capacity;
}

// Linear probing from seed_slot_hash.  Threads claim slots by compare-and-swap on the
// key; the keys are distinct, so each is placed once, and every slot a key's probe
// passes on its way was already taken, so a lookup finds it whatever order the claims
// came in (the slot a key lands in may differ between builds, its lookup result not).
void buildSeedTable(const MinimizerIndex& idx, gadev::SeedSlot* slots, uint64_t capacity)
{
    const size_t parts = 256;
    parallelFor(parts, [&](size_t c)
    {
        const uint64_t from = capacity * c / parts, to = capacity * (c + 1) / parts;
        for (uint64_t i = from; i < to; i++) slots[i] = gadev::SeedSlot { gadev::kEmptyKmer, 0, 0 };
    });
    const size_t numKeys = idx.keys.size();
    parallelFor((numKeys + 4095) / 4096, [&](size_t c)
    {
        const size_t end = std::min(numKeys, (c + 1) * 4096);
        for (size_t r = c * 4096; r < end; r++)
        {
            const uint64_t key = idx.keys[r];
            uint64_t h = gadev::seed_slot_hash(key) & (capacity - 1);
            while (true)
            {
                uint64_t expected = gadev::kEmptyKmer;
                if (__atomic_compare_exchange_n(&slots[h].key, &expected, key, false, __ATOMIC_RELAXED, __ATOMIC_RELAXED)) break;
                h = (h + 1) & (capacity - 1);
            }
            slots[h].start = (uint32_t)idx.startPos[r];
            slots[h].count = (uint32_t)(idx.startPos[r + 1] - idx.startPos[r]);
        }
    });
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
