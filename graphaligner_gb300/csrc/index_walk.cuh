// Per-bigraph-node minimizer walk of the GPU index build (index_build.cu): the node's
// sequence read over its split pieces and iterateMinimizersReal (MinimizerSeeder.cpp:104-189)
// on it.  Host-callable as well, so that the walk can be checked against the host build
// without a GPU.
#pragma once
#include <stdint.h>
#include "seed_table.h"

namespace gadev
{

static constexpr uint32_t kMaxRealWindow = 64;

struct IndexGraph
{
    uint32_t N;
    uint32_t firstAmbiguous;
    const uint32_t* len;
    const uint64_t* seq2;
    const uint64_t* seqAmb;
    const uint32_t* inOff;
    const uint32_t* inNb;
    const int32_t* nodeIds;
    const uint32_t* nodeOffset;
    const uint32_t* lookupOff;
    const uint32_t* lookupNodes;
    const uint32_t* originalSize;
    uint32_t numLookup;
};

// MinimizerSeeder.cpp:45-54 (Thomas Wang's 64-bit integer hash, as cited there)
GA_HOST_DEVICE inline uint64_t kmer_hash(uint64_t key)
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

// 2-bit code of the graph character at pos of piece, or -1 when it is not A, C, G or T
// (an ambiguous piece's position is a base only when its mask names one)
GA_HOST_DEVICE inline int piece_code(const IndexGraph& g, uint32_t piece, uint32_t pos)
{
    if (piece < g.firstAmbiguous) return (int)((g.seq2[(uint64_t)piece * 2 + (pos >> 5)] >> ((pos & 31) * 2)) & 3);
    const uint64_t* a = g.seqAmb + (uint64_t)(piece - g.firstAmbiguous) * 4;
    const uint32_t m = (uint32_t)((a[0] >> pos) & 1) | (uint32_t)(((a[1] >> pos) & 1) << 1) | (uint32_t)(((a[2] >> pos) & 1) << 2)
        | (uint32_t)(((a[3] >> pos) & 1) << 3);
    switch (m)
    {
        case 1: return 0;
        case 2: return 1;
        case 4: return 2;
        case 8: return 3;
    }
    return -1;
}

// Sequential access to a bigraph node's sequence over its contiguous pieces.
struct NodeCursor
{
    const IndexGraph* g;
    uint32_t first, last;   // range in lookupNodes
    uint32_t at;            // current piece index in lookupNodes
    uint32_t pieceStart;    // offset of the current piece in the bigraph node
    uint32_t size;          // the node's length
    GA_HOST_DEVICE inline void init(const IndexGraph& gr, uint32_t li)
    {
        g = &gr;
        size = gr.originalSize[li];
        first = gr.lookupOff[li];
        last = gr.lookupOff[li + 1];
        at = first;
        pieceStart = 0;
    }
    // the piece holding pos (pos never decreases between calls) and the code there; the
    // position just past the end reads as a non-ACGT character, as the terminating NUL of
    // the reference's std::string does when its initial window reaches it
    GA_HOST_DEVICE inline int code(uint32_t pos, uint32_t& piece)
    {
        if (pos >= size) return -1;
        while (pos >= pieceStart + g->len[g->lookupNodes[at]])
        {
            pieceStart += g->len[g->lookupNodes[at]];
            at++;
        }
        piece = g->lookupNodes[at];
        return piece_code(*g, piece, pos - pieceStart);
    }
};

struct WinEntry
{
    uint32_t pos;
    uint32_t piece;
    uint64_t kmer;
    uint64_t hash;
};

// Reports the node's minimizers (iterateMinimizersReal, MinimizerSeeder.cpp:104-189) that
// lie at or after minStart: counts them (out == nullptr) or writes them from out on.
GA_HOST_DEVICE inline uint32_t node_minimizers(const IndexGraph& g, uint32_t li, uint32_t k, uint32_t w, uint64_t* outKmer, uint64_t* outPos,
    bool& bad)
{
    const uint32_t size = g.originalSize[li];
    // the pieces must tile the node in order; minimizers start after the last piece
    // entered from another bigraph node
    uint32_t minStart = 0, expect = 0;
#pragma unroll 1
    for (uint32_t e = g.lookupOff[li]; e < g.lookupOff[li + 1]; e++)
    {
        const uint32_t piece = g.lookupNodes[e];
        if (piece >= g.N || g.nodeOffset[piece] != expect)
        {
            bad = true;
            return 0;
        }
        expect += g.len[piece];
#pragma unroll 1
        for (uint32_t p = g.inOff[piece]; p < g.inOff[piece + 1]; p++)
        {
            if (g.nodeIds[g.inNb[p]] != g.nodeIds[piece])
            {
                if (g.nodeOffset[piece] > minStart) minStart = g.nodeOffset[piece];
                break;
            }
        }
    }
    if (expect != size)
    {
        bad = true;
        return 0;
    }
    uint32_t n = 0;
    if (size < k) return 0;
    const uint32_t realWindow = w - k + 1;
    const uint64_t mask = ~(0xFFFFFFFFFFFFFFFFULL << (k * 2));
    WinEntry win[kMaxRealWindow + 1];
    uint32_t head = 0, count = 0;   // ring of the window's candidates, front at head
    auto at = [&](uint32_t i) -> WinEntry& { return win[(head + i) % (kMaxRealWindow + 1)]; };
    auto report = [&](const WinEntry& e)
    {
        if (e.pos < minStart) return;
        if (outKmer)
        {
            const uint32_t pieceOffset = e.pos - g.nodeOffset[e.piece];
            outKmer[n] = e.kmer;
            outPos[n] = ((uint64_t)e.piece << 6) + pieceOffset;
        }
        n++;
    };
    NodeCursor cur;
    cur.init(g, li);
    uint32_t offset = 0;
#pragma unroll 1
    while (true)
    {
        uint32_t piece = 0;
        // skip non-ACGT characters
#pragma unroll 1
        while (offset < size && cur.code(offset, piece) < 0) offset++;
        if ((uint64_t)offset + w > size) return n;
        uint64_t kmer = 0;
        bool restart = false;
#pragma unroll 1
        for (uint32_t i = 0; i < k; i++)
        {
            const int c = cur.code(offset + i, piece);
            if (c < 0)
            {
                offset += i;
                restart = true;
                break;
            }
            kmer = (kmer << 2) | (uint64_t)c;
        }
        if (restart) continue;
        head = 0;
        count = 0;
        {
            WinEntry e { offset + k - 1, piece, kmer, kmer_hash(kmer) };
            at(count++) = e;
        }
#pragma unroll 1
        for (uint32_t i = k; i < k + realWindow; i++)
        {
            const int c = cur.code(offset + i, piece);
            if (c < 0)
            {
                offset += i;
                restart = true;
                break;
            }
            kmer = ((kmer << 2) & mask) | (uint64_t)c;
            const uint64_t hashed = kmer_hash(kmer);
            while (count > 0 && at(count - 1).hash > hashed) count--;
            WinEntry e { offset + i, piece, kmer, hashed };
            at(count++) = e;
        }
        if (restart) continue;
        // the window's minimum, ties included
#pragma unroll 1
        for (uint32_t q = 0; q < count && at(q).hash == at(0).hash; q++) report(at(q));
#pragma unroll 1
        for (uint32_t i = k + realWindow; offset + i < size; i++)
        {
            const int c = cur.code(offset + i, piece);
            if (c < 0)
            {
                offset += i;
                restart = true;
                break;
            }
            kmer = ((kmer << 2) & mask) | (uint64_t)c;
            const uint64_t hashed = kmer_hash(kmer);
            const uint64_t oldMinimum = at(0).hash;
            bool frontPopped = false;
            while (count > 0 && at(0).pos <= offset + i - realWindow)
            {
                frontPopped = true;
                head = (head + 1) % (kMaxRealWindow + 1);
                count--;
            }
            if (frontPopped)
            {
                while (count >= 2 && at(0).hash == at(1).hash)
                {
                    head = (head + 1) % (kMaxRealWindow + 1);
                    count--;
                }
            }
            while (count > 0 && at(count - 1).hash > hashed) count--;
            WinEntry e { offset + i, piece, kmer, hashed };
            at(count++) = e;
            if (at(0).hash != oldMinimum)
            {
#pragma unroll 1
                for (uint32_t q = 0; q < count && at(q).hash == at(0).hash; q++) report(at(q));
            }
            else if (at(count - 1).hash == at(0).hash)
            {
                report(at(count - 1));
            }
        }
        if (!restart) return n;
    }
}

}
