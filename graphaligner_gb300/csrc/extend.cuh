// Shared declarations of the batched seed-extension kernels (fill, then traceback; one warp per extension).
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
struct __align__(16) Item
{
    u64 sVP, sVN;          // first column
    u64 eVP, eVN;          // last column
    u64 HP, HN;            // horizontal deltas along the slice's last row
    i32 sEnd, eEnd;
    i32 minScore;
    u32 node;              // bit 31: the node has been computed ("exists"); bit 30: it is a
                           // seed start in this slice (multiseed DP, DPSlice::seedstartNodes)
};
static constexpr u32 kExists = 0x80000000u;
static constexpr u32 kSeedStart = 0x40000000u;
static constexpr u32 kNodeMask = 0x3fffffffu;

// A committed DP slice in the arena: this 32-byte record, then the band's node ids
// (count u32, padded to 16 bytes), then count Items, all in first-pop order (the multiseed
// DP's seed starts first), then for the multiseed DP each node's best exact-end-position
// X-score (count i32, DPSlice::nodeMaxExactEndposScore).  The traceback finds a node's
// entry by a warp ballot over the ids.
struct __align__(16) SliceRec
{
    i32 minScore;
    i32 quit;              // minScore + bandwidth (the slice's band quit score)
    i32 maxX;              // maxExactEndposScore
    u32 maxXNode;          // maxExactEndposNode
    u32 count;
    u32 notValid;          // scoresNotValid: the tangle-effort cap was hit
    u32 pad0, pad1;
};

// Per-extension state passed from the fill to the traceback.
struct ExtState
{
    u64 dir;               // arena offset of the slice directory (u64 record offsets)
    u32 committed;         // slices in the table, including the start slice
    i32 status;
    u64 steps;             // Myers column steps in the fill
    u64 aux;               // multiseed DP: arena offset of the per-slice best X-scores (i32 [committed])
};

// Capacities of one warp's frontier tables.
struct Caps
{
    u32 band;              // band entries per slice
    u32 hash;              // node-table slots per slice (power of two, >= 32)
    u32 heap;              // heap entries
    u32 extras;            // pending incoming columns per slice
};

struct FillArgs
{
    DevGraph g;
    u32 bandwidth;
    i32 xdrop;
    u64 maxCells;
    i32 cost;
    u32 num;
    const u32* order;      // processing order (longest first); nullptr = index order
    const uint8_t* seq;
    const u64* seqOff;
    const u32* seqLen;
    const u32* startNode;
    const u32* startOffset;
    uint8_t* arena;        // DP tables of the batch, handed out in chunks
    u64 arenaBytes;
    unsigned long long* arenaCursor;   // [0] bytes handed out in chunks, [1] bytes the tables took (both start at 0)
    u64 chunkBytes;        // arena bytes a warp takes at once
    uint8_t* workspace;    // nullptr: the frontier tables live in shared memory
    u64 workspaceStride;   // bytes of one warp's tables
    Caps caps;
    const i32* prevStatus; // when non-null, only extensions whose previous status is GA_CAPACITY run
    ExtState* states;      // [num] where each extension's table is, for the traceback
    // multiseed DP (nullptr otherwise): read i's seeds are [seedOff[i], seedOff[i+1]),
    // slice index and split node each, in slice order
    const u64* seedOff;
    const u32* seedSlice;
    const u32* seedNode;
};

struct TraceArgs
{
    DevGraph g;
    i32 cost;
    u32 num;
    const u32* order;      // the fill's processing order; nullptr = index order
    const i32* prevStatus; // the fill's filter
    const ExtState* states;
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
};

// The multiseed DP's traceback outputs (ga_multiseed_results).
struct MultiTraceArgs
{
    DevGraph g;
    i32 cost;
    u32 num;
    const u32* order;
    const i32* prevStatus;
    const ExtState* states;
    const uint8_t* seq;
    const u64* seqOff;
    const u32* seqLen;
    const uint8_t* arena;
    const u64* traceOffset;
    const u64* traceCap;
    u32 maxTraces;
    double multimapScoreFraction;
    i32* status;
    u32* numTraces;
    i32* traceScore;
    u64* traceStart;
    u32* traceLen;
    u64* traceItems;
    u64* cellSteps;
    u64* itemsNeeded;      // [num] or null: when the traces outgrow the read's room, the room they need
    u32* tracesNeeded;
};

}

// bytes of one warp's frontier tables for these capacities (the multiseed DP's add each band
// node's best X-score)
uint64_t ga_warp_tables_bytes(const gadev::Caps& caps);
uint64_t ga_multiseed_tables_bytes(const gadev::Caps& caps);
// resident blocks of 32 * warpsPerBlock threads per SM of the fill kernel (shared: tables in
// shared memory) and of the traceback kernel
int ga_fill_blocks_per_sm(int warpsPerBlock, const gadev::Caps& caps, bool shared);
int ga_trace_blocks_per_sm(int warpsPerBlock);
// launches the fill kernel and then the traceback kernel on `stream`, blocks of warpsPerBlock
// warps, one extension per warp at a time; counters[0] and [1] must be zero
int ga_launch_extend(const gadev::FillArgs& fa, const gadev::TraceArgs& ta, uint32_t* counters, int fillBlocks, int traceBlocks,
    int warpsPerBlock, void* stream);
// the multiseed DP's fill and traceback kernels (the frontier tables always in the global workspace)
int ga_launch_multiseed(const gadev::FillArgs& fa, const gadev::MultiTraceArgs& ta, uint32_t* counters, int fillBlocks, int traceBlocks,
    int warpsPerBlock, void* stream);
int ga_upload_tables();
void ga_set_last_error(const char* message);
