// Shared declarations of the batched seed-extension kernels (fill + traceback).
#pragma once
#include <stdint.h>
#include "wordslice.cuh"

namespace gadev
{

// AlignmentGraph fields the DP reads (AlignmentGraph.h:121-139), device copies.
struct DevGraph
{
    u32 N;
    u32 firstAmbiguous;
    const u32* len;
    const u64* seq2;       // [firstAmbiguous][2] 2-bit chunks of 32 bp
    const u64* seqAmb;     // [N - firstAmbiguous][4] A,C,G,T masks
    const u32* inOff;
    const u32* inNb;
    const u32* outOff;
    const u32* outNb;
    const uint8_t* lin;
    const u32* comp;
};

// One band entry: the state of a <= 64 bp node for one 64-row slice
// (NodeSliceMapItemStruct, NodeSlice.h:15-47).  64 bytes.
struct Item
{
    u64 sVP, sVN;          // first column
    u64 eVP, eVN;          // last column
    u64 HP, HN;            // horizontal deltas along the slice's last row
    i32 sEnd, eEnd;
    i32 minScore;
    u32 node;              // bit 31: the node has been computed ("exists")
};
static constexpr u32 kExists = 0x80000000u;
static constexpr u32 kNodeMask = 0x7fffffffu;

// A committed DP slice in the per-batch arena: SliceRec (one 64-byte line), then count
// Items, then hashCap uint16 slots (band index + 1, 0 = empty) keyed by node when the
// band is larger than kInlineIds nodes.
static constexpr u32 kInlineIds = 8;

struct SliceRec
{
    i32 minScore;
    i32 quit;              // minScore + bandwidth (the slice's band quit score)
    i32 maxX;              // maxExactEndposScore
    u32 maxXNode;          // maxExactEndposNode
    u32 count;
    u32 hashCap;           // 0 when count <= kInlineIds (the ids below are the index)
    u32 notValid;          // scoresNotValid: the tangle-effort cap was hit
    u32 pad;
    u32 ids[kInlineIds];   // node of band entry k, for bands of up to kInlineIds nodes
};

// Per-extension state passed from the fill kernel to the traceback kernel.
struct ExtState
{
    u64 dir;               // arena offset of the slice directory (u64 record offsets)
    u32 committed;         // slices in the table, including the start slice
    i32 status;
    u64 steps;             // Myers column steps in the fill
};

struct Caps
{
    u32 band;              // BCAP: band entries per slice
    u32 hash;              // HCAP: build-hash slots (power of two)
    u32 heap;              // QCAP: heap entries
    u32 extras;            // ECAP: pending incoming edges per slice
};

struct FillArgs
{
    DevGraph g;
    u32 bandwidth;
    i32 xdrop;
    u64 maxCells;
    i32 cost;
    u32 num;
    const u32* order;      // processing order (longest first)
    const uint8_t* seq;
    const u64* seqOff;
    const u32* seqLen;
    const u32* startNode;
    const u32* startOffset;
    uint8_t* arena;
    u64 arenaBytes;
    unsigned long long* arenaCursor;
    uint8_t* workspace;
    u64 workspaceStride;
    Caps caps;
    const i32* prevStatus; // when non-null, only extensions whose previous status is GA_CAPACITY run
};

struct TraceArgs
{
    DevGraph g;
    i32 cost;
    u32 num;
    const u32* order;
    const uint8_t* seq;
    const u64* seqOff;
    const u32* seqLen;
    const uint8_t* arena;
    const u64* traceOffset;
    const u32* traceCap;
    i32* status;
    i32* score;
    u32* traceLen;
    u64* traceItems;
    u64* cellSteps;
    const i32* prevStatus;
};

}

void ga_launch_extend(const gadev::FillArgs& fa, const gadev::TraceArgs& ta, const uint32_t* chunks, uint32_t numChunks,
    uint32_t* counter, uint32_t slotBase, uint32_t slotLimit, int grid, int block, void* stream);
int ga_extend_occupancy(int block);
int ga_upload_tables();
void ga_set_last_error(const char* message);
uint64_t ga_workspace_bytes(const gadev::Caps& caps);
