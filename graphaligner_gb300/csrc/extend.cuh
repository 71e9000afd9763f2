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
// X-score (count i32, DPSlice::nodeMaxExactEndposScore) and, for a band of more than
// kHashedBand nodes, an open-addressing index of the band (hashSize u32 slots, each an
// entry's position or kEmptySlot, linear probing from the node's hash).  The traceback finds
// a node's entry through the index where there is one, else by a warp ballot over the ids.
static constexpr u32 kHashedBand = 64;
static constexpr u32 kEmptySlot = 0xffffffffu;
struct __align__(16) SliceRec
{
    i32 minScore;
    i32 quit;              // minScore + bandwidth (the slice's band quit score)
    i32 maxX;              // maxExactEndposScore
    u32 maxXNode;          // maxExactEndposNode
    u32 count;
    u32 notValid;          // scoresNotValid: the tangle-effort cap was hit
    u32 hashSize;          // slots of the band index (a power of two), 0 = none
    u32 hashOff;           // byte offset of the band index from the record
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

// One local maximum of a multiseed read's table that may start a trace: a node whose best
// X-score in a slice beats its neighbours' and reaches the multimap fraction of the slice's
// best before any trace raised it.  The traces from the candidates are independent, so one
// warp traces each; the read's own pass keeps them in getLocalMaximaTracesFromTable's order
// against the raised slice bests, in rounds: a candidate is traced only once the traces kept
// before it have not ruled it out (or as one of a few traced ahead of the read's next one).
struct MsCand
{
    u32 read;
    u32 slice;
    u32 index;             // the node's position in the slice's band
    i32 score;             // its best X-score in the slice
    u32 startNode;         // the trace's first cell
    u32 startOff;
    int64_t startSeq;
    i32 startScore;
    i32 err;               // 0 or the status the trace failed with
    i32 traceScore;
    u32 len;               // trace items
    int64_t traceStart;    // read position of the trace's last item
    u64 outOff;            // kept traces: items from the read's trace_offset
    u32 slot;              // kept traces: the trace's index in the read, else kNoSlot
    u32 state;             // kUntraced, kQueued (for this round's walks) or kTraced
    u32 lastNode;          // the trace's last item (its start in the read)
    u32 lastOff;
};

// What removeDuplicateTraces looks at in a kept trace: the read positions of its first and
// last items, its last item's cell, its score (and its length, for the room it takes).
struct MsKey
{
    int64_t first;
    int64_t last;
    u32 lastNode;
    u32 lastOff;
    i32 score;
    u32 len;
};
static constexpr u32 kNoSlot = 0xffffffffu;
static constexpr u32 kUntraced = 0, kQueued = 1, kTraced = 2;

// A multiseed read's selection so far: its candidates before `cursor` are decided.
struct MsSel
{
    u64 used;              // items of the kept traces that have their place
    u64 items;             // items of all kept traces
    u32 nt;                // kept traces that have their place
    u32 traces;            // kept traces
    u32 cursor;
    u32 full;              // the kept traces have outgrown the read's room
    u32 done;
    u32 pad;
};
// the status of a multiseed read whose traces outgrew its room (reported as GA_CAPACITY with
// the room it needs; the batch does not run it again as it does a read whose tables ran out)
static constexpr i32 kMsRoom = 100;

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
                           // (with exact room: the items of the kept traces)
    u32* tracesNeeded;
    // exact room (traceBase non-null): read i's kept traces are traceBase[i] + slot in the
    // kept list, whose summaries go to keys; after removeDuplicateTraces kept trace k is
    // written as trace keptSlot[k] (kNoSlot: a duplicate) with its items from keptItem[k], its
    // start counted from itemBias; traceOffset, traceCap and maxTraces are not used
    const u64* traceBase;
    MsKey* keys;
    const u32* keptSlot;
    const u64* keptItem;
    u64 itemBias;
    MsSel* sel;            // [num] each read's selection
    u32* work;             // this round's candidates to walk (indices into cands)
    u32* workCount;
    u32 window;            // candidates a read may have walked in this round
    MsCand* cands;         // [candCap] the batch's candidates, each read's together and in order
    u64 candCap;
    u64* candBegin;        // [num] read i's candidates are [candBegin[i], candBegin[i] + candCount[i])
    u32* candCount;
    unsigned long long* candTotal;   // candidates of the batch
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
// the multiseed DP in steps, blocks of warpsPerBlock warps, each on `stream`:
// - fill: the fill and the count of each read's trace candidates (counters[0], [1] and
//   ta.candTotal zero);
// - list: once ta.cands has room for *ta.candTotal, the candidates listed (counters[3] zero,
//   ta.sel zeroed);
// - rounds, until a resolve queues nothing: resolve (each read decides its candidates in
//   order as far as their walks are known, then queues the next ta.window walks; counters[4]
//   and *ta.workCount zero) and walk (the queued candidates' traces counted; counters[5] zero);
// - write: the kept traces written (counters[6] zero).
// counters[2] is left to the caller.
int ga_launch_multiseed_fill(const gadev::FillArgs& fa, const gadev::MultiTraceArgs& ta, uint32_t* counters, int fillBlocks, int readBlocks,
    int warpsPerBlock, void* stream);
int ga_launch_multiseed_list(const gadev::MultiTraceArgs& ta, uint32_t* counters, int readBlocks, int warpsPerBlock, void* stream);
int ga_launch_multiseed_resolve(const gadev::MultiTraceArgs& ta, uint32_t* counters, int readBlocks, int warpsPerBlock, void* stream);
int ga_launch_multiseed_walk(const gadev::MultiTraceArgs& ta, uint32_t* counters, int candBlocks, int warpsPerBlock, void* stream);
int ga_launch_multiseed_write(const gadev::MultiTraceArgs& ta, uint32_t* counters, int candBlocks, int warpsPerBlock, void* stream);
// exact room: each kept trace's summary into ta.keys
int ga_launch_multiseed_keys(const gadev::MultiTraceArgs& ta, void* stream);
int ga_upload_tables();
void ga_set_last_error(const char* message);
