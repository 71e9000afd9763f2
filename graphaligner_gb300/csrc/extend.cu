// Batched seed extension on GB300: one warp per extension.
//
// Two persistent kernels run back to back.  In the fill kernel a warp owns one
// extension at a time and runs the banded Myers DP over the graph with the
// component-ordered frontier and X-drop, writing each committed slice into the
// batch's DP-table arena; the traceback kernel then gives each warp one filled
// extension to walk back.  The DP of one extension is a sequential chain: each
// 64-row slice depends on the whole band of the previous one, and inside a slice
// nodes are computed one at a time in frontier order, the admission test using the
// running minimum.  So a warp runs that control flow warp-uniformly (every lane
// holds the same scalars, branches never diverge) and spreads over its lanes the
// work that is parallel inside it:
//   - the match masks of a slice (lane k reads rows k and k + 32; ballots),
//   - the match mask of every column of a node, before its column loop,
//   - per node: the X-score of every column (lane k scores columns k and k + 32),
//     the minimum and its first column (reduce + ballot) and the bottom-row
//     horizontal deltas (ballots), so the column loop itself only runs the
//     Myers recurrence,
//   - cellwise merges of columns and the changed-minimum test (row scores by
//     popcount, then a shuffle, ballots and a reduction),
//   - node-table lookups: 32 probes of the open-addressing table per step (ballot),
//   - committing a slice to the DP table (coalesced copies),
//   - the traceback's end-cell choice (slices and columns across lanes) and its
//     band lookups (ballot over the slice's node ids),
//   - trace output, staged in shared memory and written 32 items at a time.
// The fill's frontier tables (two bands, two node tables, the heap, the pending
// incoming columns) and a node's recorded columns live in shared memory; an
// extension that outgrows them is re-run with larger tables in global memory.
// Fill and traceback are separate kernels so that the warps of an SM share one
// phase's code: fused, the two phases' code did not fit the instruction caches.
// Cold paths (crossing rules, end-cell choice, sequential fallbacks) are out of line.
//
// Warps take extensions from a device counter over a longest-first order.
//
// Reference correspondence (GraphAligner src/):
//   fill_extension   getReverseTraceFromSeed / getXdropSlices  (GraphAlignerBitvectorBanded.h:59-76, 580-725)
//   fill_slice       calculateSlice                            (GraphAlignerBitvectorBanded.h:255-511)
//   node_calc<Fill>  calculateNodeInner                        (GraphAlignerBitvectorCommon.h:1113-1478)
//   trace_extension  getReverseTraceFromTableExactEndPos / getReverseTraceFromTable
//                                                              (GraphAlignerBitvectorCommon.h:496-758)
//   bt_corner etc.   pickBacktraceInside/HorizontalCrossing/VerticalCrossing/Corner (:770-1054)
#include <cuda_runtime.h>
#include <stdint.h>
#include "extend.cuh"
#include "../../include/graphaligner_gb300.h"

namespace gadev
{

static constexpr unsigned kFull = 0xffffffffu;

// a pending incoming column of a node (ComponentPriorityQueue::extras entry)
struct Extra
{
    u64 VP, VN;
    i32 end;
    uint16_t next;
    uint16_t skip;      // EdgeWithPriority::skipFirst
};

static constexpr uint16_t kNil = 0xffff;

// node-table slot value: where the node sits in the slice's band and its queue state
struct NodeVal
{
    int16_t band;       // index in the slice's band, -1 until the node is first popped
    uint16_t active;    // node has a heap entry (ComponentPriorityQueue::active)
    uint16_t head;      // pending incoming columns, FIFO
    uint16_t tail;
};

// one recorded column of a node-slice: the fill's epilogue and the traceback read these
struct __align__(16) Col
{
    u64 VP, VN;
    u64 Mh;             // horizontal -1 deltas of the step (the X-score's candidate mask)
    i32 end;
    u32 phTop;          // horizontal +1 delta out of the last row
};

__device__ __forceinline__ u32 hash_node(u32 node)
{
    u32 h = node * 0x9E3779B1u;
    return h ^ (h >> 15);
}

// One warp's tables.  A node-table key is (generation << 32) | node; a slot whose
// generation is not the slice's is empty, so tables are never cleared between slices.
struct WSpace
{
    Item* band[2];
    u64* key[2];
    NodeVal* val[2];
    HeapItem* heap;
    Extra* extras;
    Col* cols;          // [64]
    u64* eqcol;         // [64] match mask of each column of the current node
    u64* ring;          // [64] trace items not yet written out
    struct SliceSlot* slots;   // [2] the traceback's cached slices (odd and even)
    i32* nodeMax;       // multiseed DP: [band] each band node's best exact-end-position X-score
};

__host__ __device__ inline u64 align16(u64 x) { return (x + 15) & ~15ULL; }

__host__ __device__ inline u64 wspace_bytes(const Caps& c, bool multi = false)
{
    u64 b = multi ? align16((u64)c.band * 4) : 0;
    b += 2 * align16((u64)c.band * sizeof(Item));
    b += 2 * align16((u64)c.hash * 8);
    b += 2 * align16((u64)c.hash * sizeof(NodeVal));
    b += align16((u64)c.heap * sizeof(HeapItem));
    b += align16((u64)c.extras * sizeof(Extra));
    b += 64 * sizeof(Col) + 64 * 8 + 64 * 8;
    return align16(b);
}

__device__ __forceinline__ WSpace wspace_at(uint8_t* base, const Caps& c)
{
    WSpace w;
    u64 off = 0;
    w.band[0] = (Item*)(base + off); off += align16((u64)c.band * sizeof(Item));
    w.band[1] = (Item*)(base + off); off += align16((u64)c.band * sizeof(Item));
    w.key[0] = (u64*)(base + off); off += align16((u64)c.hash * 8);
    w.key[1] = (u64*)(base + off); off += align16((u64)c.hash * 8);
    w.val[0] = (NodeVal*)(base + off); off += align16((u64)c.hash * sizeof(NodeVal));
    w.val[1] = (NodeVal*)(base + off); off += align16((u64)c.hash * sizeof(NodeVal));
    w.heap = (HeapItem*)(base + off); off += align16((u64)c.heap * sizeof(HeapItem));
    w.extras = (Extra*)(base + off); off += align16((u64)c.extras * sizeof(Extra));
    w.cols = (Col*)(base + off); off += 64 * sizeof(Col);
    w.eqcol = (u64*)(base + off); off += 64 * 8;
    w.ring = (u64*)(base + off); off += 64 * 8;
    w.nodeMax = (i32*)(base + off);    // inside the stride only when it was sized for the multiseed DP
    w.slots = nullptr;
    return w;
}

// Node-table lookup with 32 linear probes per step (lane k probes the k-th slot of the
// step); the first slot in probe order that is the node's or empty ends the probe.
// Returns the node's slot or -1.  Every lane gets the same answer.
__device__ __forceinline__ int tbl_find(const u64* key, u32 cap, u32 gen, u32 node, u32 lane)
{
    const u32 h = hash_node(node);
    const u64 want = ((u64)gen << 32) | node;
    #pragma unroll 1
    for (u32 base = 0; base < cap; base += 32)
    {
        const u32 slot = (h + base + lane) & (cap - 1);
        const u64 k = key[slot];
        const u32 hit = __ballot_sync(kFull, k == want);
        const u32 stop = hit | __ballot_sync(kFull, (u32)(k >> 32) != gen);
        if (stop)
        {
            const u32 first = __ffs((int)stop) - 1;
            return ((hit >> first) & 1) ? (int)((h + base + first) & (cap - 1)) : -1;
        }
    }
    return -1;
}

// the node's slot, claimed (band -1, inactive, no pending columns) if it has none;
// -1 when the table would pass half full
__device__ __forceinline__ int tbl_get_or_add(u64* key, NodeVal* val, u32 cap, u32 gen, u32 node, u32& used, u32 lane)
{
    const u32 h = hash_node(node);
    const u64 want = ((u64)gen << 32) | node;
    #pragma unroll 1
    for (u32 base = 0; base < cap; base += 32)
    {
        const u32 slot = (h + base + lane) & (cap - 1);
        const u64 k = key[slot];
        const u32 hit = __ballot_sync(kFull, k == want);
        const u32 stop = hit | __ballot_sync(kFull, (u32)(k >> 32) != gen);
        if (stop)
        {
            const u32 first = __ffs((int)stop) - 1;
            const u32 s = (h + base + first) & (cap - 1);
            if ((hit >> first) & 1) return (int)s;
            if (2 * (used + 1) > cap) return -1;
            used++;
            key[s] = want;
            NodeVal v;
            v.band = -1;
            v.active = 0;
            v.head = kNil;
            v.tail = kNil;
            val[s] = v;
            return (int)s;
        }
    }
    return -1;
}

// IUPAC membership of every byte value (bit0 A, bit1 C, bit2 G, bit3 T; 0 = '-',
// -1 = not a sequence character), filled from iupac_mask on the host at load time and
// copied into shared memory by every block (lanes index it by data: the constant
// cache would serialise distinct addresses of a warp, shared memory serves them at once)
__constant__ int8_t c_iupac[256];
__shared__ int8_t s_iupac[256];

// all threads of the block must call this before any other work
__device__ __forceinline__ void load_iupac_table()
{
    for (u32 k = threadIdx.x; k < 256; k += blockDim.x) s_iupac[k] = c_iupac[k];
    __syncthreads();
}

// Match masks of the 64 rows starting at read position j (getEqVector, Common.h:279-318):
// lane k reads rows k and k + 32 and the masks come from ballots.  False when a row holds
// a non-sequence byte, or a gap inside a full 64-row window (the reference asserts).
__device__ __noinline__ bool eq_vector(const uint8_t* seq, u32 len, int64_t j, EqV4& eq, u32 lane)
{
    const bool full = j + 64 <= (int64_t)len;
    int m0 = 0, m1 = 0;
    bool bad = false;
    if (j + lane < (int64_t)len)
    {
        m0 = s_iupac[seq[j + lane]];
        bad |= m0 < 0 || (m0 == 0 && full);
    }
    if (j + lane + 32 < (int64_t)len)
    {
        m1 = s_iupac[seq[j + lane + 32]];
        bad |= m1 < 0 || (m1 == 0 && full);
    }
    eq.a = (u64)__ballot_sync(kFull, m0 & 1) | ((u64)__ballot_sync(kFull, m1 & 1) << 32);
    eq.c = (u64)__ballot_sync(kFull, m0 & 2) | ((u64)__ballot_sync(kFull, m1 & 2) << 32);
    eq.g = (u64)__ballot_sync(kFull, m0 & 4) | ((u64)__ballot_sync(kFull, m1 & 4) << 32);
    eq.t = (u64)__ballot_sync(kFull, m0 & 8) | ((u64)__ballot_sync(kFull, m1 & 8) << 32);
    return __ballot_sync(kFull, bad) == 0;
}

// graph character of node n at pos (AlignmentGraph::NodeSequences) as an IUPAC mask
__device__ __forceinline__ int node_char_mask(const DevGraph& g, u32 n, u32 pos)
{
    if (n < g.firstAmbiguous)
    {
        u64 chunk = g.seq2[(u64)n * 2 + (pos >> 5)];
        return 1 << ((chunk >> ((pos & 31) * 2)) & 3);
    }
    const u64* a = g.seqAmb + (u64)(n - g.firstAmbiguous) * 4;
    return (int)((a[0] >> pos) & 1) | (int)(((a[1] >> pos) & 1) << 1) | (int)(((a[2] >> pos) & 1) << 2) | (int)(((a[3] >> pos) & 1) << 3);
}

// GraphAlignerCommon::characterMatch on a read byte and a graph position
__device__ __forceinline__ bool char_match(const DevGraph& g, uint8_t c, u32 n, u32 pos, bool& bad)
{
    int a = s_iupac[c];
    if (a < 0) { bad = true; return false; }
    int b = node_char_mask(g, n, pos);
    // identical characters always match; for distinct ones the IUPAC sets must overlap
    return (a & b) != 0;
}

// ---------------------------------------------------------------- warp column algebra
//
// A column's scores at rows lane and lane + 32 are two prefix popcounts away from its
// row-above score.  With them the cellwise operations take one shuffle, ballot or
// reduction step instead of the bit walks of WordSlice::differenceMasksBitTwiddle
// (WordSlice.h:566-664), whose trip counts depend on the data.  They return exactly what
// ws_merge (mergeTwoSlices: the cellwise minimum) and ws_changed_min
// (changedMinScoreLocalMinima: the least score among rows, and the row above, where the
// column improved on the old one) return for valid columns.  Scores beyond +-2^29 take
// the sequential forms, so no sum here can wrap.

static constexpr i32 kWarpScoreLimit = 1 << 29;

__device__ __forceinline__ bool score_ok(i32 v) { return v > -kWarpScoreLimit && v < kWarpScoreLimit; }

// scores of rows lane and lane + 32 (WordSlice::getValue)
__device__ __forceinline__ void ws_rows(const WS& w, i32 before, u32 lane, i32& v0, i32& v1)
{
    const u32 upto = (2u << lane) - 1u;
    const u32 vpl = (u32)w.VP, vnl = (u32)w.VN;
    const i32 low = popc32(vpl) - popc32(vnl);
    v0 = before + popc32(vpl & upto) - popc32(vnl & upto);
    v1 = before + low + popc32((u32)(w.VP >> 32) & upto) - popc32((u32)(w.VN >> 32) & upto);
}

// a column from its row-above score and its scores at rows lane and lane + 32
__device__ __forceinline__ WS ws_from_rows(i32 before, i32 m0, i32 m1, u32 lane)
{
    i32 p0 = __shfl_up_sync(kFull, m0, 1);
    i32 p1 = __shfl_up_sync(kFull, m1, 1);
    const i32 m31 = __shfl_sync(kFull, m0, 31);
    if (lane == 0)
    {
        p0 = before;
        p1 = m31;
    }
    const i32 d0 = m0 - p0, d1 = m1 - p1;
    WS r;
    r.VP = (u64)__ballot_sync(kFull, d0 == 1) | ((u64)__ballot_sync(kFull, d1 == 1) << 32);
    r.VN = (u64)__ballot_sync(kFull, d0 == -1) | ((u64)__ballot_sync(kFull, d1 == -1) << 32);
    r.end = __shfl_sync(kFull, m1, 31);
    return r;
}

__device__ __noinline__ WS merge_seq(WS a, WS b) { return ws_merge(a, b); }
__device__ __noinline__ i32 changed_min_seq(WS w, WS old) { return ws_changed_min(w, old); }

// mergeTwoSlices (WordSlice.h:502-541) across the lanes
__device__ __forceinline__ WS merge_w(const WS& a, const WS& b, u32 lane)
{
    const i32 ba = ws_before(a), bb = ws_before(b);
    if (!(score_ok(ba) && score_ok(bb) && score_ok(a.end) && score_ok(b.end))) return merge_seq(a, b);
    i32 a0, a1, b0, b1;
    ws_rows(a, ba, lane, a0, a1);
    ws_rows(b, bb, lane, b0, b1);
    return ws_from_rows(imin(ba, bb), imin(a0, b0), imin(a1, b1), lane);
}

// changedMinScoreLocalMinima (WordSlice.h:438-472) across the lanes; old may be the
// never-computed column (0, 0, INT32_MAX), whose every score is INT32_MAX
__device__ __forceinline__ i32 changed_min_w(const WS& w, const WS& old, u32 lane)
{
    const i32 bw = ws_before(w), bo = ws_before(old);
    const bool oldUnset = old.VP == 0 && old.VN == 0 && old.end == kIntMax;
    if (!(score_ok(bw) && score_ok(w.end) && (oldUnset || (score_ok(bo) && score_ok(old.end))))) return changed_min_seq(w, old);
    i32 w0, w1, o0, o1;
    ws_rows(w, bw, lane, w0, w1);
    ws_rows(old, bo, lane, o0, o1);
    i32 best = bw < bo ? bw : kIntMax;
    if (w0 < o0) best = imin(best, w0);
    if (w1 < o1) best = imin(best, w1);
    return __reduce_min_sync(kFull, best);
}

struct NodeCalc
{
    i32 minScore;
    u32 minScoreNode;
    u32 minScoreOffset;
    i32 maxX;
    u32 maxXNode;
    u32 cells;
};

struct PrevInfo
{
    bool exists;
    i32 sEnd;
    u64 HP, HN;
};

// An upper bound of ws_max_xscore(w, seqOffset, cost, 64, mask): every candidate row m scores
// 100 (m + 1) - cost s(m) with s(m) >= -popc(VN), plus 100 seqOffset - cost before.
__device__ __forceinline__ int64_t xscore_bound(const WS& w, i32 seqOffset, i32 cost)
{
    const i32 vn = popc64(w.VN);
    const i32 before = w.end - (popc64(w.VP) - vn);
    return 6400 + (int64_t)cost * vn + (int64_t)seqOffset * 100 - (int64_t)cost * before;
}

// Below this read offset no term of the X-score can wrap around in 32 bits, so the bound
// above also bounds the reference's (wrapping) arithmetic.
static constexpr i32 kXBoundOffsetLimit = 10000000;

// The part of calculateNodeInner (Common.h:1209-1300) that runs when the node already
// has a column in this slice: merge the new first column into it.  Returns true when the
// reference leaves the node early (nothing changed).  Out of line: a node is computed
// again within a slice only inside cyclic components.
__device__ __noinline__ bool merge_existing(WS& ws, const Item& slice, bool hasSkipless, bool singleInEdge, u32 lane)
{
    WS s = ws_make(slice.sVP, slice.sVN, slice.sEnd);
    if (hasSkipless && singleInEdge)
    {
        if (ws.end > s.end) return true;
        if (ws.end < s.end) return false;
        u64 newBigger = (ws.VP & ~s.VP) | (s.VN & ~ws.VN);
        u64 oldBigger = (s.VP & ~ws.VP) | (ws.VN & ~s.VN);
        if (newBigger > oldBigger) return false;
        if (oldBigger > newBigger) return true;
        if (newBigger == 0 && oldBigger == 0) return true;
        WS t = merge_w(ws, s, lane);
        if (ws_eq(t, s)) return true;
        ws = t;
        return false;
    }
    WS t = merge_w(ws, s, lane);
    // the reference compares test.VP against the stored VN here (Common.h:1282)
    if (t.end == s.end && t.VP == s.VP && t.VP == s.VN) return true;
    ws = t;
    return false;
}

// The horizontal input along the slice's first row when the column enters below the
// previous slice's last row (Common.h:1310-1343): fixedHP/HN and the rows whose first
// cell is forced.  False where the reference asserts.  Out of line: rarely taken.
__device__ __noinline__ bool fix_horizontal(i32 scoreBefore, i32 scoreComparison, u64& fixedHP, u64& fixedHN, u64& forceMask)
{
    forceMask |= 1;
    #pragma unroll 1
    for (int off = 1; off < 64; off++)
    {
        i32 next = scoreComparison + (i32)((fixedHP >> off) & 1) - (i32)((fixedHN >> off) & 1);
        u64 mask = 1ULL << off;
        if (scoreBefore > next) return false;
        if (scoreBefore < next)
        {
            fixedHP |= mask;
            fixedHN &= ~mask;
            forceMask |= mask;
        }
        else
        {
            fixedHP &= ~mask;
            fixedHN &= ~mask;
        }
        scoreBefore++;
        scoreComparison = next;
        if (scoreBefore >= scoreComparison) break;
    }
    return true;
}

// The same when the node is a seed start of the multiseed DP (Common.h:1314-1362): the row
// above follows the lower of the previous slice's last row and the seed start's score
// before the slice, and every column of the first row takes its delta from that.
__device__ __noinline__ bool fix_horizontal_extra(i32 scoreBefore, i32 scoreComparison, i32 extraBefore, u32 nodeLength, u64& fixedHP,
    u64& fixedHN, u64& forceMask)
{
    scoreBefore = imin(scoreBefore, extraBefore);
    if (scoreBefore < scoreComparison) forceMask |= 1;
    i32 adjust = imin(scoreBefore, scoreComparison);
    #pragma unroll 1
    for (u32 off = 1; off < 64 && off < nodeLength; off++)
    {
        const i32 next = scoreComparison + (i32)((fixedHP >> off) & 1) - (i32)((fixedHN >> off) & 1);
        if (scoreBefore < extraBefore) scoreBefore += 1;
        const u64 mask = 1ULL << off;
        if (scoreBefore < next) forceMask |= mask;
        const i32 na = imin(next, scoreBefore);
        if (na < adjust - 1 || na > adjust + 1) return false;
        if (na == adjust - 1)
        {
            fixedHN |= mask;
            fixedHP &= ~mask;
        }
        else if (na == adjust)
        {
            fixedHP &= ~mask;
            fixedHN &= ~mask;
        }
        else
        {
            fixedHP |= mask;
            fixedHN &= ~mask;
        }
        adjust = na;
        scoreComparison = next;
    }
    return true;
}

// calculateNodeInner (Common.h:1113-1478).  Multi = false: the single-seed path, whose extra
// slice is always the fake one.  Multi = true: the multiseed DP, where `extra` (non-null for
// a node that is a seed start in this slice) is merged into every column and an incoming
// column that starts a seed forces the computation (EdgeWithPriority::forceCalculation).
// Fill = true: the slice fill (early leave allowed, calculateNodeClipPrecise).
// Fill = false: recalcNodeWordslice (no early leave); columns 0..lastColumn land in cols.
// The column loop runs the Myers recurrence warp-uniformly and records every column; the
// per-column minimum, X-score and horizontal output bits are then taken across the lanes.
template <bool Fill, bool Multi = false>
__device__ __forceinline__ NodeCalc node_calc(const DevGraph& g, i32 cost, u32 i, Item& slice, const EqV4& eqv, const PrevInfo& prev,
    const Extra* pool, uint16_t head, const WS* singleIncoming, bool singleInPrevBand, i32 seqOffset, Col* cols, u64* eqcol,
    u64& steps, int& err, u32 lane, i32 sliceMaxX = kIntMin, u32 lastColumn = 63, const WS* extra = nullptr)
{
    const bool hasExtra = Multi && extra != nullptr;
    bool forceCalculation = false;
    const bool boundOk = seqOffset < kXBoundOffsetLimit;
    NodeCalc result;
    result.minScore = kIntMax;
    result.minScoreNode = 0xffffffffu;
    result.minScoreOffset = 0xffffffffu;
    result.maxX = kIntMin;
    result.maxXNode = 0xffffffffu;
    result.cells = 0;
    const u32 nodeLength = g.len[i];
    const bool amb = i >= g.firstAmbiguous;
    u64 c0 = 0, c1 = 0, a0 = 0, a1 = 0, a2 = 0, a3 = 0;
    if (!amb)
    {
        c0 = g.seq2[(u64)i * 2];
        c1 = g.seq2[(u64)i * 2 + 1];
    }
    else
    {
        const u64* a = g.seqAmb + (u64)(i - g.firstAmbiguous) * 4;
        a0 = a[0]; a1 = a[1]; a2 = a[2]; a3 = a[3];
    }
    const u32 inDeg = g.inOff[i + 1] - g.inOff[i];
    // the match mask of every column (lane k: columns k and k + 32)
    __syncwarp();
    #pragma unroll 1
    for (u32 pos = lane; pos < nodeLength; pos += 32)
    {
        u64 e;
        if (!amb) e = eq_pick(eqv, (u32)(((pos < 32 ? c0 : c1) >> ((pos & 31) * 2)) & 3));
        else e = eq_amb(eqv, (u32)(((a0 >> pos) & 1) | (((a1 >> pos) & 1) << 1) | (((a2 >> pos) & 1) << 2) | (((a3 >> pos) & 1) << 3)));
        eqcol[pos] = e;
    }
    __syncwarp();
    const u64 eq0 = eqcol[0];

    WS ws = ws_make(0, 0, 0);
    bool hasWs = false;
    bool hasSkipless = false;
    if (singleIncoming)
    {
        result.cells = 1;
        ws = *singleIncoming;
        hasWs = true;
    }
    else
    {
        #pragma unroll 1
        for (uint16_t e = head; e != kNil; e = pool[e].next)
        {
            const Extra& inc = pool[e];
            WS incWs = ws_make(inc.VP, inc.VN, inc.end);
            result.cells++;
            if (Multi && (inc.skip & 2)) forceCalculation = true;
            if (inc.skip & 1)
            {
                ws = hasWs ? merge_w(ws, incWs, lane) : incWs;
                hasWs = true;
                continue;
            }
            hasSkipless = true;
            i32 compareHin = prev.exists ? prev.sEnd : kIntMax;
            if (hasExtra) compareHin = imin(compareHin, ws_before(*extra));
            i32 incBefore = ws_before(incWs);
            u64 hinP = 0, hinN = 0;
            if (compareHin < incBefore) hinN = 1;
            else if (compareHin > incBefore) hinP = 1;
            u64 Ph, Mh;
            WS nw = myers_step(eq0, incWs, hinP, hinN, Ph, Mh);
            steps++;
            if (!prev.exists || ws_before(nw) < prev.sEnd)
            {
                nw.VP &= kAllOnes ^ 1;
                nw.VN |= 1;
            }
            ws = hasWs ? merge_w(ws, nw, lane) : nw;
            hasWs = true;
        }
    }
    if (!hasWs) { err = GA_ASSERT; return result; }
    // column 0 as the incoming columns make it: the node's first minimum candidate and,
    // with every row a candidate, its first X-score
    const WS ws0 = ws;
    result.minScore = ws.end;
    result.minScoreNode = i;
    result.minScoreOffset = 0;
    result.maxXNode = i;
    // the seed start's column joins after the first minimum and before the first X-score
    if (hasExtra) ws = merge_w(ws, *extra, lane);
    const WS wsX = ws;
    // (the recomputation starts from the stored first column, whose merge with itself changes nothing)
    if (Fill && !forceCalculation && (slice.node & kExists) != 0 && merge_existing(ws, slice, hasSkipless, inDeg == 1 && singleInPrevBand, lane))
    {
        if (!boundOk || xscore_bound(wsX, seqOffset, cost) > (int64_t)sliceMaxX)
            result.maxX = ws_max_xscore(wsX, seqOffset, cost, 64, kAllOnes);
        return result;
    }
    if (prev.exists && ws_before(ws) > prev.sEnd) ws = merge_w(ws, ws_source(prev.sEnd), lane);
    u64 forceMask = 0;
    u64 fixedHP = prev.HP;
    u64 fixedHN = prev.HN;
    if (prev.exists)
    {
        i32 scoreBefore = ws_before(ws);
        i32 scoreComparison = prev.sEnd;
        if (scoreBefore > scoreComparison) { err = GA_ASSERT; return result; }
        if (hasExtra)
        {
            if (!fix_horizontal_extra(scoreBefore, scoreComparison, ws_before(*extra), nodeLength, fixedHP, fixedHN, forceMask))
            {
                err = GA_ASSERT;
                return result;
            }
        }
        else if (scoreBefore < scoreComparison && !fix_horizontal(scoreBefore, scoreComparison, fixedHP, fixedHN, forceMask))
        {
            err = GA_ASSERT;
            return result;
        }
    }
    else
    {
        forceMask = kAllOnes;
    }
    slice.sVP = ws.VP;
    slice.sVN = ws.VN;
    slice.sEnd = ws.end;
    slice.node = i | kExists | (slice.node & kSeedStart);
    {
        // Fill: column 0 as it enters the node, its X-score over every row; the traceback's
        // recomputation: column 0 after the merges
        Col c;
        c.VP = Fill ? ws0.VP : ws.VP;
        c.VN = Fill ? ws0.VN : ws.VN;
        c.Mh = kAllOnes;
        c.end = Fill ? ws0.end : ws.end;
        c.phTop = 0;
        cols[0] = c;
    }
    const u64 forceEq = prev.exists ? kAllOnes : (kAllOnes ^ 1);
    // the traceback's recomputation stops at the column it needs last
    const u32 columns = Fill ? nodeLength : (lastColumn + 1 < nodeLength ? lastColumn + 1 : nodeLength);
    u64 hp = fixedHP >> 1, hn = fixedHN >> 1, fm = forceMask >> 1;   // bit 0: column 1
    #pragma unroll 1
    for (u32 pos = 1; pos < columns; pos++)
    {
        const u64 eq = eqcol[pos] & forceEq;
        u64 Ph, Mh;
        WS nw = myers_step(eq, ws, hp & 1, hn & 1, Ph, Mh);
        if (fm & 1)
        {
            nw.VP &= kAllOnes ^ 1;
            nw.VN |= 1;
        }
        hp >>= 1;
        hn >>= 1;
        fm >>= 1;
        // the multiseed DP keeps both bottom-row deltas in phTop (bit 0 +1, bit 1 -1): with a
        // seed start they come from the merged column's last-row score
        u32 top = (u32)(Ph >> 63);
        if (Multi)
        {
            if (hasExtra)
            {
                const WS m = merge_w(nw, *extra, lane);
                top = (m.end == ws.end + 1 ? 1u : 0u) | (m.end == ws.end - 1 ? 2u : 0u);
                nw = m;
            }
            else top |= (u32)(Mh >> 63) << 1;
        }
        ws = nw;
        Col c;
        c.VP = ws.VP;
        c.VN = ws.VN;
        c.Mh = Mh;
        c.end = ws.end;
        c.phTop = top;
        cols[pos] = c;
    }
    steps += columns - 1;
    result.cells = columns;
    if (Fill)
    {
        // Across the lanes (lane k: columns k and k + 32; every lane wrote every column):
        // the first column of least score, the greatest X-score and the bottom-row deltas.
        // A column whose X-score bound is at most the slice's best so far cannot change the
        // slice's choice (it keeps the first node of strictly greatest X-score), so its exact
        // X-score is skipped; every column above that bound is scored exactly.
        u32 loKey = 0xffffffffu, hiKey = 0xffffffffu;
        i32 lmax = kIntMin;
        u32 hpLo = 0, hpHi = 0, hnLo = 0, hnHi = 0;
#pragma unroll
        for (u32 h = 0; h < 2; h++)
        {
            const u32 pos = lane + 32 * h;
            if (pos < columns)
            {
                const Col c = cols[pos];
                // column 0's X-score is taken after the seed start's column joins it
                const WS cw = (Multi && pos == 0) ? wsX : ws_make(c.VP, c.VN, c.end);
                const u32 key = (u32)c.end ^ 0x80000000u;   // signed order as unsigned
                if (h == 0) loKey = key; else hiKey = key;
                if (!boundOk || xscore_bound(cw, seqOffset, cost) > (int64_t)sliceMaxX)
                    lmax = imax(lmax, ws_max_xscore(cw, seqOffset, cost, 64, c.Mh));
                if (pos >= 1)
                {
                    const u32 tp = Multi ? (c.phTop & 1) : c.phTop;
                    const u32 tn = Multi ? ((c.phTop >> 1) & 1) : (u32)(c.Mh >> 63);
                    if (h == 0) { hpLo = tp; hnLo = tn; }
                    else { hpHi = tp; hnHi = tn; }
                }
            }
        }
        const u32 gkey = __reduce_min_sync(kFull, loKey < hiKey ? loKey : hiKey);
        const i32 gmax = __reduce_max_sync(kFull, lmax);
        const u32 onLo = __ballot_sync(kFull, loKey == gkey);
        const u32 onHi = __ballot_sync(kFull, hiKey == gkey);
        const u64 outHP = (u64)__ballot_sync(kFull, hpLo) | ((u64)__ballot_sync(kFull, hpHi) << 32);
        const u64 outHN = (u64)__ballot_sync(kFull, hnLo) | ((u64)__ballot_sync(kFull, hnHi) << 32);
        // column 0 always takes part, so the key is a real score
        result.minScore = (i32)(gkey ^ 0x80000000u);
        result.minScoreOffset = onLo ? (u32)(__ffs((int)onLo) - 1) : (u32)(32 + __ffs((int)onHi) - 1);
        result.maxX = gmax;
        slice.HP = outHP;
        slice.HN = outHN;
    }
    slice.eVP = ws.VP;
    slice.eVN = ws.VN;
    slice.eEnd = ws.end;
    return result;
}

// ---------------------------------------------------------------- arena

struct ArenaCursor
{
    u64 pos;
    u64 end;
    u64 used;           // bytes handed out to this warp since the launch began
};

// bytes from the warp's current chunk, else a new chunk (one atomic per chunk)
__device__ __forceinline__ bool arena_alloc(const FillArgs& a, ArenaCursor& c, u64 bytes, u64& out, u32 lane)
{
    bytes = align16(bytes);
    if (c.pos + bytes > c.end)
    {
        const u64 grab = bytes > a.chunkBytes ? bytes : a.chunkBytes;
        unsigned long long p = 0;
        if (lane == 0) p = atomicAdd(a.arenaCursor, (unsigned long long)grab);
        p = __shfl_sync(kFull, p, 0);
        if (p + grab > a.arenaBytes) return false;
        c.pos = p;
        c.end = p + grab;
    }
    out = c.pos;
    c.pos += bytes;
    c.used += bytes;
    return true;
}

__device__ __forceinline__ u64 rec_ids_bytes(u32 count) { return align16((u64)count * 4); }

// slots of a committed band's index: none up to kHashedBand nodes, else the power of two at
// least twice the band (the index is at most half full)
__device__ __forceinline__ u32 band_hash_size(u32 count)
{
    if (count <= kHashedBand) return 0;
    u32 h = 256;
    while (h < 2 * count) h <<= 1;
    return h;
}

// write one slice (record, node ids, band in first-pop order and, for the multiseed DP, each
// node's best X-score and a large band's index) into the arena, lanes copying
__device__ bool commit_slice(const FillArgs& a, ArenaCursor& c, u64* dir, u32 index, const Item* band, u32 count,
    i32 minScore, i32 quit, i32 maxX, u32 maxXNode, bool notValid, u32 lane, const i32* nodeMax = nullptr)
{
    const u64 idBytes = rec_ids_bytes(count);
    u64 off;
    const u64 maxBytes = nodeMax ? rec_ids_bytes(count) : 0;
    const u32 hashSize = nodeMax ? band_hash_size(count) : 0;
    const u64 hashOff = sizeof(SliceRec) + idBytes + (u64)count * sizeof(Item) + maxBytes;
    if (!arena_alloc(a, c, hashOff + (u64)hashSize * 4, off, lane)) return false;
    uint8_t* base = a.arena + off;
    if (lane == 0)
    {
        SliceRec r;
        r.minScore = minScore;
        r.quit = quit;
        r.maxX = maxX;
        r.maxXNode = maxXNode;
        r.count = count;
        r.notValid = notValid ? 1u : 0u;
        r.hashSize = hashSize;
        r.hashOff = hashSize ? (u32)hashOff : 0;
        *(SliceRec*)base = r;
        dir[index] = off;
    }
    u32* ids = (u32*)(base + sizeof(SliceRec));
    #pragma unroll 1
    for (u32 k = lane; k < count; k += 32) ids[k] = band[k].node & kNodeMask;
    uint4* dst = (uint4*)(base + sizeof(SliceRec) + idBytes);
    const uint4* src = (const uint4*)band;
    #pragma unroll 1
    for (u32 k = lane; k < count * 4; k += 32) dst[k] = src[k];
    if (nodeMax)
    {
        i32* m = (i32*)(base + sizeof(SliceRec) + idBytes + (u64)count * sizeof(Item));
        #pragma unroll 1
        for (u32 k = lane; k < count; k += 32) m[k] = nodeMax[k];
    }
    if (hashSize)
    {
        // every slot empty, then each entry claims the first empty slot from its node's hash
        u32* slots = (u32*)(base + hashOff);
        #pragma unroll 1
        for (u32 k = lane; k < hashSize; k += 32) slots[k] = kEmptySlot;
        __syncwarp();
        #pragma unroll 1
        for (u32 k = lane; k < count; k += 32)
        {
            u32 h = hash_node(band[k].node & kNodeMask) & (hashSize - 1);
            #pragma unroll 1
            while (atomicCAS(&slots[h], kEmptySlot, k) != kEmptySlot) h = (h + 1) & (hashSize - 1);
        }
        __syncwarp();
    }
    return true;
}

// position of node's entry in committed slice r (whose node ids are `ids`) through its band
// index: 32 slots per probe step, the first slot in probe order that is empty or the node's
// ends it.  Out of line: most bands are small, and the lookups are inlined in many places.
__device__ __noinline__ int rec_index_hashed(const SliceRec* r, const u32* ids, u32 node, u32 lane)
{
    const u32 hashSize = r->hashSize;
    const u32* slots = (const u32*)((const uint8_t*)r + r->hashOff);
    const u32 h = hash_node(node);
#pragma unroll 1
    for (u32 step = 0; step < hashSize; step += 32)
    {
        const u32 e = __ldcg(&slots[(h + step + lane) & (hashSize - 1)]);
        const bool empty = e == kEmptySlot;
        const bool hit = !empty && ids[e] == node;
        const u32 stop = __ballot_sync(kFull, empty || hit);
        if (stop) return __shfl_sync(kFull, hit ? (int)e : -1, __ffs((int)stop) - 1);
    }
    return -1;
}

// position of node's entry in committed slice r (whose node ids are `ids`), or -1; every lane
// gets the answer.  Hashed (the multiseed DP's tables): through the band index where the slice
// has one.  Else a ballot over the ids: the extension's tables have no index, and their lookups
// keep the short form.
template <bool Hashed>
__device__ __forceinline__ int rec_index(const SliceRec* r, const u32* ids, u32 node, u32 lane)
{
    if (Hashed && r->hashSize) return rec_index_hashed(r, ids, node, lane);
    const u32 n = r->count;
#pragma unroll 1
    for (u32 base = 0; base < n; base += 32)
    {
        const u32 k = base + lane;
        const u32 hit = __ballot_sync(kFull, k < n && ids[k] == node);
        if (hit) return (int)(base + __ffs((int)hit) - 1);
    }
    return -1;
}

// the multiseed DP's per-node best X-scores of a committed slice
__device__ __forceinline__ const i32* rec_node_max(const SliceRec* r)
{
    return (const i32*)((const uint8_t*)r + sizeof(SliceRec) + rec_ids_bytes(r->count) + (u64)r->count * sizeof(Item));
}

// ---------------------------------------------------------------- fill

struct SliceResult
{
    i32 minScore;
    u32 minScoreNode;
    i32 maxX;
    u32 maxXNode;
    u64 cells;
};

// getSeedSlice (Common.h:320-353): the column of starting an alignment at each row of the slice
// at j, each row scored as the X-score's error cost of the read before it (rows past the read's
// end one more each)
__device__ __noinline__ WS seed_ws(int64_t j, u32 seqLen, i32 cost)
{
    u64 vp = 0;
    i32 old = j > 0 ? (i32)((j * 100 + cost / 2) / cost) : 0;
    #pragma unroll 1
    for (u32 off = 0; off < 64; off++)
    {
        if (j + off >= (int64_t)seqLen)
        {
            vp |= 1ULL << off;
            old += 1;
            continue;
        }
        const i32 score = (i32)(((j + off + 1) * 100 + cost / 2) / cost);
        if (score == old + 1) vp |= 1ULL << off;
        old = score;
    }
    return ws_make(vp & ~1ULL, 1, old);
}

// The seeds the multiseed DP starts in one slice, with the slice's seed-start column.
struct SliceSeeds
{
    const u32* nodes;
    u32 count;
    WS ws;
};

// calculateSlice (GraphAlignerBitvectorBanded.h:255-511), component-queue branch.  Multi:
// the multiseed DP's slice, whose seeds enter the band first (addSeedHitToScoresAndQueue,
// :228-253) and whose nodes keep their best exact-end-position X-score in w.nodeMax.
template <bool Multi = false>
__device__ SliceResult fill_slice(const FillArgs& a, const WSpace& w, int cur, u32 curGen, u32 prevGen, u32& curCount, u32 prevCount,
    const uint8_t* seq, u32 seqLen, int64_t j, i32 prevQuit, i32 prevMin, u64& steps, int& err, u32 lane, const SliceSeeds* seeds = nullptr)
{
    if (Multi)
    {
        if (prevMin == kIntMax - (i32)a.bandwidth - 1)
        {
            prevMin = ws_before(seeds->ws);
            prevQuit = wadd(prevMin, (i32)a.bandwidth);
        }
        if (prevMin > seeds->ws.end)
        {
            prevMin = seeds->ws.end;
            prevQuit = wadd(seeds->ws.end, (i32)a.bandwidth);
        }
    }
    const DevGraph& g = a.g;
    const int bw = (int)a.bandwidth;
    const int prv = cur ^ 1;
    Item* curBand = w.band[cur];
    const Item* prevBand = w.band[prv];
    u64* curKey = w.key[cur];
    NodeVal* curVal = w.val[cur];
    const u64* prevKey = w.key[prv];
    const NodeVal* prevVal = w.val[prv];
    const u32 hcap = a.caps.hash;
    SliceResult res;
    res.minScore = kIntMax - bw - 1;
    res.minScoreNode = 0xffffffffu;
    res.maxX = kIntMin;
    res.maxXNode = 0;
    res.cells = 0;
    EqV4 eqv;
    if (!eq_vector(seq, seqLen, j, eqv, lane)) { err = GA_ASSERT; return res; }
    u32 heapN = 0;
    u32 poolN = 0;
    u32 used = 0;
    curCount = 0;

    // band index of node in the previous slice, or -1
    auto prevBandOf = [&](u32 node) -> int
    {
        const int s = tbl_find(prevKey, hcap, prevGen, node, lane);
        return s < 0 ? -1 : (int)prevVal[s].band;
    };

    auto insert = [&](u32 target, i32 score, u64 vp, u64 vn, i32 end, bool skip, bool force) -> bool
    {
        const int slot = tbl_get_or_add(curKey, curVal, hcap, curGen, target, used, lane);
        if (slot < 0) return false;
        NodeVal& s = curVal[slot];
        if (!s.active)
        {
            if (heapN >= a.caps.heap) return false;
            HeapItem hi; hi.component = g.comp[target]; hi.score = score; hi.node = target;
            heap_push(w.heap, heapN, hi);
            s.active = 1;
            s.head = kNil;
            s.tail = kNil;
        }
        if (poolN >= a.caps.extras) return false;
        uint16_t e = (uint16_t)poolN++;
        Extra x;
        x.VP = vp; x.VN = vn; x.end = end; x.next = kNil; x.skip = (skip ? 1 : 0) | (force ? 2 : 0);
        w.extras[e] = x;
        if (s.head == kNil) s.head = e;
        else w.extras[s.tail].next = e;
        s.tail = e;
        return true;
    };

    #pragma unroll 1
    for (u32 k = 0; k < prevCount; k++)
    {
        const Item& it = prevBand[k];
        u32 node = it.node & kNodeMask;
        if (j == 0)
        {
            if (it.minScore > prevQuit) { err = GA_ASSERT; return res; }
        }
        else
        {
            if (it.minScore > prevQuit) continue;
            if (g.lin[node])
            {
                const int pb = prevBandOf(g.inNb[g.inOff[node]]);
                if (pb >= 0)
                {
                    const Item& pn = prevBand[pb];
                    if (pn.eEnd < prevQuit && pn.minScore < prevQuit) continue;
                }
            }
        }
        WS src = ws_source(it.sEnd);
        if (!insert(node, it.minScore, src.VP, src.VN, src.end, true, false)) { err = GA_CAPACITY; return res; }
    }
    if (!Multi && heapN == 0) { err = GA_ASSERT; return res; }
    if (Multi && ws_before(seeds->ws) < wadd(prevQuit, 64))
    {
        // the seed starts: in the band before any node of the queue, computed first among equals
        #pragma unroll 1
        for (u32 k = 0; k < seeds->count; k++)
        {
            const u32 node = seeds->nodes[k];
            const int slot = tbl_get_or_add(curKey, curVal, hcap, curGen, node, used, lane);
            if (slot < 0) { err = GA_CAPACITY; return res; }
            NodeVal& sv = curVal[slot];
            if (sv.band >= 0) { err = GA_ASSERT; return res; }
            if (curCount >= a.caps.band || curCount >= 32767) { err = GA_CAPACITY; return res; }
            sv.band = (int16_t)curCount;
            Item ni;
            ni.sVP = seeds->ws.VP; ni.sVN = seeds->ws.VN; ni.sEnd = seeds->ws.end;
            ni.eVP = seeds->ws.VP; ni.eVN = seeds->ws.VN; ni.eEnd = seeds->ws.end;
            ni.HP = 0; ni.HN = 0;
            ni.minScore = seeds->ws.end;
            ni.node = node | kExists | kSeedStart;
            curBand[curCount] = ni;
            w.nodeMax[curCount] = 0;
            curCount++;
            if (!insert(node, ws_value(seeds->ws, 0), seeds->ws.VP, seeds->ws.VN, seeds->ws.end, true, true)) { err = GA_CAPACITY; return res; }
        }
    }
    i32 curMin = res.minScore;
    const i32 seqOffset = (i32)j;
    #pragma unroll 1
    while (heapN > 0)
    {
        u32 i = w.heap[0].node;
        const int slot = tbl_find(curKey, hcap, curGen, i, lane);
        if (slot < 0) { err = GA_ASSERT; return res; }
        NodeVal& s = curVal[slot];
        if (s.band < 0)
        {
            if (curCount >= a.caps.band || curCount >= 32767) { err = GA_CAPACITY; return res; }
            s.band = (int16_t)curCount;
            Item ni;
            ni.sVP = 0; ni.sVN = 0; ni.sEnd = kIntMax;
            ni.eVP = 0; ni.eVN = 0; ni.eEnd = kIntMax;
            ni.HP = 0; ni.HN = 0;
            ni.minScore = kIntMax;
            ni.node = i;
            if (Multi) w.nodeMax[curCount] = 0;
            curBand[curCount++] = ni;
        }
        Item& thisNode = curBand[s.band];
        WS oldEnd = (thisNode.node & kExists) ? ws_make(thisNode.eVP, thisNode.eVN, thisNode.eEnd) : ws_make(0, 0, kIntMax);
        const WS* extra = (Multi && (thisNode.node & kSeedStart)) ? &seeds->ws : nullptr;
        if (Multi && extra) oldEnd = merge_w(oldEnd, *extra, lane);
        PrevInfo prev;
        const int pb = prevBandOf(i);
        if (pb >= 0)
        {
            const Item& pi = prevBand[pb];
            prev.exists = true;
            prev.sEnd = pi.sEnd;
            prev.HP = pi.HP;
            prev.HN = pi.HN;
        }
        else
        {
            prev.exists = false;
            prev.sEnd = 0;
            prev.HP = kAllOnes;
            prev.HN = 0;
        }
        bool singleInPrev = false;
        if (g.inOff[i + 1] - g.inOff[i] == 1) singleInPrev = prevBandOf(g.inNb[g.inOff[i]]) >= 0;
        // a column whose X-score bound is at most both the slice's and the node's best so far
        // changes neither, so the node computation may skip its exact X-score
        const i32 skipBelow = Multi ? imin(res.maxX, w.nodeMax[s.band]) : res.maxX;
        NodeCalc nc = node_calc<true, Multi>(g, a.cost, i, thisNode, eqv, prev, w.extras, s.head, nullptr, singleInPrev, seqOffset,
            w.cols, w.eqcol, steps, err, lane, skipBelow, 63, extra);
        if (err) return res;
        if (Multi) w.nodeMax[s.band] = imax(nc.maxX, w.nodeMax[s.band]);
        heap_pop(w.heap, heapN);
        s.active = 0;
        s.head = kNil;
        s.tail = kNil;
        if (nc.minScore > wadd(wadd(seqOffset, bw), 128)) { err = GA_ASSERT; return res; }
        curMin = imin(curMin, nc.minScore);
        if (nc.minScore < thisNode.minScore) thisNode.minScore = nc.minScore;
        WS newEnd = ws_make(thisNode.eVP, thisNode.eVN, thisNode.eEnd);
        if (!ws_eq(newEnd, oldEnd))
        {
            i32 newEndMin = changed_min_w(newEnd, oldEnd, lane);
            if (newEndMin == kIntMax) { err = GA_ASSERT; return res; }
            if (newEndMin <= wadd(curMin, bw))
            {
                #pragma unroll 1
                for (u32 e = g.outOff[i]; e < g.outOff[i + 1]; e++)
                {
                    if (!insert(g.outNb[e], newEndMin, newEnd.VP, newEnd.VN, newEnd.end, false, false)) { err = GA_CAPACITY; return res; }
                }
            }
        }
        if (nc.minScore < res.minScore)
        {
            res.minScore = nc.minScore;
            res.minScoreNode = nc.minScoreNode;
        }
        if (nc.maxX > res.maxX)
        {
            res.maxX = nc.maxX;
            res.maxXNode = nc.maxXNode;
        }
        if (res.minScore != curMin || nc.cells == 0) { err = GA_ASSERT; return res; }
        res.cells += nc.cells;
        if (res.cells > a.maxCells) break;
    }
    if (res.minScoreNode == 0xffffffffu && !(Multi && seeds->count == 0)) err = GA_ASSERT;
    return res;
}

__device__ ExtState fill_extension(const FillArgs& a, const WSpace& w, u32& gen, ArenaCursor& arena, u32 ext, u32 lane)
{
    const DevGraph& g = a.g;
    ExtState st;
    st.dir = 0;
    st.committed = 0;
    st.status = GA_OK;
    st.steps = 0;
    const uint8_t* seq = a.seq + a.seqOff[ext];
    const u32 seqLen = a.seqLen[ext];
    const u32 startNode = a.startNode[ext];
    const u32 startOff = a.startOffset[ext];
    const u32 numSlices = (seqLen + 63) / 64;
    int err = 0;
    if (startNode >= g.N || startOff >= g.len[startNode])
    {
        st.status = GA_BAD_REQUEST;
        return st;
    }
    u64 dirOff;
    if (!arena_alloc(a, arena, (u64)(numSlices + 1) * 8, dirOff, lane))
    {
        st.status = GA_CAPACITY;
        return st;
    }
    u64* dir = (u64*)(a.arena + dirOff);
    st.dir = dirOff;
    // start slice (getInitialSliceExactPosition, Common.h:1551-1587): one node, scores = distance from the offset
    int prv = 0;
    gen++;
    u32 prevGen = gen;
    {
        Item it;
        u32 L = g.len[startNode];
        it.sVP = 0; it.sVN = 0; it.sEnd = (i32)startOff;
        it.eVP = 0; it.eVN = 0; it.eEnd = (i32)L - 1 - (i32)startOff;
        it.minScore = 0;
        it.node = startNode | kExists;
        u64 hn = 0, hp = 0;
        #pragma unroll 1
        for (u32 k = 1; k <= startOff; k++) hn |= 1ULL << k;
        #pragma unroll 1
        for (u32 k = startOff + 1; k < L; k++) hp |= 1ULL << k;
        it.HP = hp;
        it.HN = hn;
        w.band[prv][0] = it;
        u32 used = 0;
        const int s = tbl_get_or_add(w.key[prv], w.val[prv], a.caps.hash, prevGen, startNode, used, lane);
        w.val[prv][s].band = 0;
        if (!commit_slice(a, arena, dir, 0, w.band[prv], 1, 0, 1, 0, startNode, false, lane))
        {
            st.status = GA_CAPACITY;
            return st;
        }
    }
    u32 prevCount = 1;
    u32 committed = 1;
    i32 bestX = 0;
    i32 lastMin = 0;
    i32 lastQuit = 1;
    #pragma unroll 1
    for (u32 s = 0; s < numSlices; s++)
    {
        const int cur = prv ^ 1;
        gen++;
        const u32 curGen = gen;
        u32 curCount = 0;
        const int64_t j = (int64_t)s * 64;
        SliceResult r = fill_slice(a, w, cur, curGen, prevGen, curCount, prevCount, seq, seqLen, j, lastQuit, lastMin, st.steps, err, lane);
        if (err) break;
        if (r.maxX > bestX) bestX = r.maxX;
        const bool notValid = r.cells >= a.maxCells;
        if ((int64_t)r.maxX < (int64_t)bestX - (int64_t)a.xdrop) break;
        if (r.minScore < lastMin) { err = GA_ASSERT; break; }
        const i32 quit = wadd(r.minScore, (i32)a.bandwidth);
        if (!commit_slice(a, arena, dir, committed, w.band[cur], curCount, r.minScore, quit, r.maxX, r.maxXNode, notValid, lane))
        {
            err = GA_CAPACITY;
            break;
        }
        committed++;
        prv = cur;
        prevGen = curGen;
        prevCount = curCount;
        lastMin = r.minScore;
        lastQuit = quit;
    }
    st.committed = committed;
    if (err) st.status = err;
    else if (committed <= 1) st.status = GA_TRACE_FAILED;
    return st;
}

// GraphAlignerBitvectorBanded::getMultiseedSlices (GraphAlignerBitvectorBanded.h:727-822): every
// slice of read r from the empty initial slice, each slice's seeds started in it.  Each slice's
// best X-score also goes to a per-read array (st.aux) that the traceback lowers as it finds
// traces.
__device__ ExtState fill_multiseed(const FillArgs& a, const WSpace& w, u32& gen, ArenaCursor& arena, u32 r, u32 lane)
{
    ExtState st;
    st.dir = 0;
    st.committed = 0;
    st.status = GA_OK;
    st.steps = 0;
    st.aux = 0;
    const uint8_t* seq = a.seq + a.seqOff[r];
    const u32 seqLen = a.seqLen[r];
    const u32 numSlices = (seqLen + 63) / 64;
    const i32 bw = (i32)a.bandwidth;
    u64 dirOff, auxOff;
    if (!arena_alloc(a, arena, (u64)(numSlices + 1) * 8, dirOff, lane) || !arena_alloc(a, arena, (u64)(numSlices + 1) * 4, auxOff, lane))
    {
        st.status = GA_CAPACITY;
        return st;
    }
    u64* dir = (u64*)(a.arena + dirOff);
    i32* sliceMax = (i32*)(a.arena + auxOff);
    st.dir = dirOff;
    st.aux = auxOff;
    // getInitialEmptySlice (Common.h:1541-1549): no nodes, minimum 0, bandwidth 1
    if (!commit_slice(a, arena, dir, 0, w.band[0], 0, 0, 1, kIntMin, 0xffffffffu, false, lane, w.nodeMax))
    {
        st.status = GA_CAPACITY;
        return st;
    }
    if (lane == 0) sliceMax[0] = kIntMin;
    int prv = 0;
    gen++;
    u32 prevGen = gen;
    u32 prevCount = 0;
    u32 committed = 1;
    i32 lastMin = 0;
    i32 lastQuit = 1;
    u64 k = a.seedOff[r];
    const u64 kEnd = a.seedOff[r + 1];
    int err = 0;
    #pragma unroll 1
    for (u32 s = 0; s < numSlices; s++)
    {
        const int cur = prv ^ 1;
        gen++;
        const u32 curGen = gen;
        u32 curCount = 0;
        const int64_t j = (int64_t)s * 64;
        u64 next = k;
        while (next < kEnd && a.seedSlice[next] == s) next++;
        SliceSeeds seeds;
        seeds.nodes = a.seedNode + k;
        seeds.count = (u32)(next - k);
        seeds.ws = seed_ws(j, seqLen, a.cost);
        k = next;
        SliceResult res = fill_slice<true>(a, w, cur, curGen, prevGen, curCount, prevCount, seq, seqLen, j, lastQuit, lastMin, st.steps, err, lane, &seeds);
        if (err) break;
        // fillDPSlice's checks of a slice that started seeds (GraphAlignerBitvectorBanded.h:543-549)
        if (seeds.count > 0)
        {
            const double lim = ((double)j + 64) * (double)a.cost;
            if (res.minScore > (i32)j + 64 || res.maxX == kIntMin || (double)res.maxX < -lim || (double)res.maxX > lim) { err = GA_ASSERT; break; }
        }
        if (!(res.minScore >= lastMin || res.minScore >= ws_value(seeds.ws, 0) || lastMin == kIntMax - bw - 1)) { err = GA_ASSERT; break; }
        const bool notValid = res.cells >= a.maxCells;
        const i32 quit = wadd(res.minScore, bw);
        if (!commit_slice(a, arena, dir, committed, w.band[cur], curCount, res.minScore, quit, res.maxX, res.maxXNode, notValid, lane, w.nodeMax))
        {
            err = GA_CAPACITY;
            break;
        }
        if (lane == 0) sliceMax[committed] = res.maxX;
        committed++;
        prv = cur;
        prevGen = curGen;
        prevCount = curCount;
        lastMin = res.minScore;
        lastQuit = quit;
    }
    if (!err && k != kEnd) err = GA_ASSERT;
    st.committed = committed;
    if (err) st.status = err;
    __syncwarp();
    return st;
}

// ---------------------------------------------------------------- traceback

// A copy in shared memory of one committed slice whose band has at most kCachedBand nodes:
// the traceback works on one slice and the one before it, so two slots (by the slice's
// parity) hold both, and their band lookups are ballots over shared memory.
static constexpr u32 kCachedBand = 16;

struct __align__(16) SliceSlot
{
    SliceRec rec;
    u32 slice;             // the cached slice, 0xffffffff = none
    u32 pad[3];
    u32 ids[kCachedBand];
    Item items[kCachedBand];
};

// The record of slice s; a band of at most kCachedBand nodes is first copied into the
// slot of the slice's parity (lanes copy 16 bytes each)
__device__ __noinline__ const SliceRec* load_slice(const uint8_t* arena, const u64* dir, SliceSlot* slots, u32 s, u32 lane)
{
    const SliceRec* r = (const SliceRec*)(arena + dir[s]);
    const u32 n = r->count;
    if (n > kCachedBand) return r;
    SliceSlot& sl = slots[s & 1];
    __syncwarp();
    const uint4* src = (const uint4*)r;
    const u32* ids = (const u32*)((const uint8_t*)r + sizeof(SliceRec));
    const uint4* items = (const uint4*)((const uint8_t*)ids + rec_ids_bytes(n));
    if (lane < 2) ((uint4*)&sl.rec)[lane] = src[lane];
    if (lane < n) sl.ids[lane] = ids[lane];
#pragma unroll 1
    for (u32 k = lane; k < n * 4; k += 32) ((uint4*)sl.items)[k] = items[k];
    sl.slice = s;
    __syncwarp();
    return &sl.rec;
}

struct Table
{
    const uint8_t* arena;
    const u64* dir;
    u32 count;
    u32 lane;
    SliceSlot* slots;
    __device__ __forceinline__ void init()
    {
        slots[0].slice = 0xffffffffu;
        slots[1].slice = 0xffffffffu;
        __syncwarp();
    }
    // the slice's record: its shared copy (made on first use when the band is small), else
    // the arena's
    __device__ __forceinline__ const SliceRec* rec(u32 s)
    {
        SliceSlot& sl = slots[s & 1];
        if (sl.slice == s) return &sl.rec;
        return load_slice(arena, dir, slots, s, lane);
    }
    // the band entry of node in slice s, or nullptr (Hashed: the multiseed DP's tables)
    template <bool Hashed = false>
    __device__ __forceinline__ const Item* find(u32 s, u32 node)
    {
        const SliceRec* r = rec(s);
        const u32 n = r->count;
        const SliceSlot& sl = slots[s & 1];
        const bool cached = sl.slice == s;
        const u32* ids = cached ? sl.ids : (const u32*)((const uint8_t*)r + sizeof(SliceRec));
        const Item* items = cached ? sl.items : (const Item*)((const uint8_t*)ids + rec_ids_bytes(n));
        const int k = rec_index<Hashed>(r, ids, node, lane);
        return k < 0 ? nullptr : &items[k];
    }
};

struct TPos
{
    u32 node;
    u32 off;
    int64_t seq;      // -1 = the row above the read
};

__device__ __forceinline__ bool tpos_eq(const TPos& a, const TPos& b) { return a.node == b.node && a.off == b.off && a.seq == b.seq; }

struct TStep
{
    TPos pos;
    bool sw;
};

// writes the 32 staged trace items that end at item n (lane k writes one)
__device__ __noinline__ void flush32(u64* items, const u64* ring, u32 n, u32 lane)
{
    const u32 k = n - 32 + lane;
    items[k] = ring[k & 63];
    __syncwarp();
}

// Trace items go to a 64-entry ring in shared memory (every lane writes every item) and
// out to the caller's buffer 32 at a time, one item per lane.
// counting (MayCount only, the multiseed traceback): nothing goes out, the items are only
// counted.
template <bool MayCount>
struct TraceOutT
{
    u64* items;
    u64* ring;
    u32 cap;
    u32 n;
    u32 lane;
    TPos back;
    bool overflow;
    bool counting = false;
    __device__ __forceinline__ void push(const TPos& p, bool sw)
    {
        if (n >= cap) { overflow = true; return; }
        u64 sp1 = p.seq < 0 ? 0 : (u64)p.seq + 1;
        ring[n & 63] = (u64)p.node | ((u64)(p.off & 63) << 32) | ((u64)(sw ? 1 : 0) << 38) | (sp1 << 39);
        n++;
        back = p;
        if (!(MayCount && counting) && (n & 31) == 0) flush32(items, ring, n, lane);
    }
    // writes the items of the last, partial group of 32
    __device__ __forceinline__ void finish()
    {
        if (MayCount && counting) return;
        const u32 k = (n & ~31u) + lane;
        if (k < n) items[k] = ring[k & 63];
        __syncwarp();
    }
};
using TraceOut = TraceOutT<false>;

__device__ __forceinline__ u32 mod64(int64_t seq) { return (u32)((u64)seq & 63); }

// checkBacktraceCircularity (Common.h:760-768): the newest item must not repeat an
// earlier item of the same read position.  Items still in the ring are read there, older
// ones from the written output (a counting walk checks the ring only).
__device__ __noinline__ bool trace_circular(const u64* items, const u64* ring, u32 n, bool ringOnly = false)
{
    if (n < 2) return false;
    const u64 keyMask = ~(1ULL << 38);
    const u64 last = ring[(n - 1) & 63];
#pragma unroll 1
    for (int k = (int)n - 2; k >= 0; k--)
    {
        if (ringOnly && (u32)k + 63 < n) return false;
        const u64 x = (u32)k + 63 >= n ? ring[k & 63] : items[k];
        if ((x & keyMask) == (last & keyMask)) return true;
        if ((x >> 39) != (last >> 39)) return false;
    }
    return false;
}

// The extraSlice of a node-slice: the multiseed DP's seed-start column (getSeedSlice) where the
// node is a seed start, else the fake column (0, 0, INT32_MAX), all of whose scores are INT32_MAX.
__device__ __forceinline__ WS fake_ws() { return ws_make(0, 0, kIntMax); }
// the extraSlice's score at a row and before the slice: the seed-start column's (Multi) or
// the fake column's, INT32_MAX, which no cell reaches
template <bool Multi> __device__ __forceinline__ i32 xval(const WS& e, int row) { return Multi ? ws_value(e, row) : kIntMax; }
template <bool Multi> __device__ __forceinline__ i32 xbefore(const WS& e) { return Multi ? ws_before(e) : kIntMax; }


__device__ __forceinline__ i32 col_value(const Col& c, int row) { return ws_value(ws_make(c.VP, c.VN, c.end), row); }

// pickBacktraceCorner (Common.h:936-1054).  Out of line, like the other crossing rules:
// the walk inside a node-slice is the hot path.  t is a copy (its record cache is a hint).
template <bool Multi>
__device__ __noinline__ TStep bt_corner(const DevGraph& g, const uint8_t* seq, Table t, u32 cs, u32 node, int64_t j, int& err, WS extra)
{
    const SliceRec* cr = t.rec(cs);
    const SliceRec* pr = t.rec(cs - 1);
    const Item* self = t.template find<Multi>(cs, node);
    TStep out; out.pos.node = 0; out.pos.off = 0; out.pos.seq = 0; out.sw = false;
    if (!self) { err = GA_ASSERT; return out; }
    i32 scoreHere = ws_value(ws_make(self->sVP, self->sVN, self->sEnd), 0);
    const Item* prevSelf = t.template find<Multi>(cs - 1, node);
    if (cr->notValid || scoreHere > cr->quit)
    {
        if (scoreHere == xval<Multi>(extra, 0)) { out.pos = TPos { node, 0, j }; return out; }
        i32 smallest = scoreHere + 1;
        TPos sp = TPos { 0xffffffffu, 0xffffffffu, -2 };
        bool change = false;
        if (prevSelf)
        {
            smallest = prevSelf->sEnd;
            sp = TPos { node, 0, j - 1 };
            change = false;
        }
        #pragma unroll 1
        for (u32 e = g.inOff[node]; e < g.inOff[node + 1]; e++)
        {
            u32 nb = g.inNb[e];
            const Item* pn = t.template find<Multi>(cs - 1, nb);
            if (pn && pn->eEnd <= smallest)
            {
                smallest = pn->eEnd;
                sp = TPos { nb, g.len[nb] - 1, j - 1 };
                change = true;
            }
            const Item* cn = t.template find<Multi>(cs, nb);
            if (cn && nb != node)
            {
                i32 v = ws_value(ws_make(cn->eVP, cn->eVN, cn->eEnd), 0);
                if (v < smallest)
                {
                    smallest = v;
                    sp = TPos { nb, g.len[nb] - 1, j };
                    change = true;
                }
            }
        }
        if (sp.node == 0xffffffffu) { err = GA_ASSERT; return out; }
        out.pos = sp; out.sw = change;
        return out;
    }
    bool bad = false;
    bool eq = char_match(g, seq[j], node, 0, bad);
    if (bad) { err = GA_ASSERT; return out; }
    TPos bestInvalid = TPos { 0xffffffffu, 0xffffffffu, -2 };
    i32 bestInvalidScore = scoreHere + 1;
    bool bestInvalidSw = false;
    if (prevSelf)
    {
        i32 ps = prevSelf->sEnd;
        if (ps < scoreHere - 1) { err = GA_ASSERT; return out; }
        if (ps == scoreHere - 1) { out.pos = TPos { node, 0, j - 1 }; return out; }
        if (pr->notValid || ps > pr->quit)
        {
            if (ps < bestInvalidScore)
            {
                bestInvalidScore = ps;
                bestInvalid = TPos { node, 0, j - 1 };
                bestInvalidSw = false;
            }
        }
    }
    #pragma unroll 1
    for (u32 e = g.inOff[node]; e < g.inOff[node + 1]; e++)
    {
        u32 nb = g.inNb[e];
        const Item* cn = t.template find<Multi>(cs, nb);
        if (cn)
        {
            i32 v = ws_value(ws_make(cn->eVP, cn->eVN, cn->eEnd), 0);
            if (v < scoreHere - 1) { err = GA_ASSERT; return out; }
            if (v == scoreHere - 1) { out.pos = TPos { nb, g.len[nb] - 1, j }; out.sw = true; return out; }
        }
        const Item* pn = t.template find<Multi>(cs - 1, nb);
        if (pn)
        {
            i32 corner = pn->eEnd;
            if (pr->notValid || corner > pr->quit)
            {
                if (corner < bestInvalidScore)
                {
                    bestInvalidScore = corner;
                    bestInvalid = TPos { nb, g.len[nb] - 1, j - 1 };
                    bestInvalidSw = true;
                }
            }
            else
            {
                if (corner < scoreHere - (eq ? 0 : 1)) { err = GA_ASSERT; return out; }
                if (corner == scoreHere - (eq ? 0 : 1)) { out.pos = TPos { nb, g.len[nb] - 1, j - 1 }; out.sw = true; return out; }
            }
        }
    }
    if (eq && scoreHere == xbefore<Multi>(extra)) { out.pos = TPos { node, 0, j }; return out; }
    if (scoreHere == xval<Multi>(extra, 0)) { out.pos = TPos { node, 0, j }; return out; }
    if (bestInvalidScore < scoreHere + 1) { out.pos = bestInvalid; out.sw = bestInvalidSw; return out; }
    err = GA_ASSERT;
    return out;
}

// recalcNodeWordslice (Common.h:1078-1102): the columns 0..lastColumn of one node-slice
// into cols (the traceback only moves left inside a node, so it never needs the columns
// after the one it enters at).  When every column is recomputed the last one must equal
// the stored end column, as the reference asserts.  Returns 0 or the error status.
template <bool Multi = false>
__device__ __noinline__ int recalc(const DevGraph& g, i32 cost, Table t, u32 s, u32 node, const EqV4& eqv, Col* cols, u64* eqcol,
    u32 lane, u32 lastColumn, WS extra = fake_ws())
{
    const Item* it = t.template find<Multi>(s, node);
    if (!it) return GA_ASSERT;
    PrevInfo prev;
    const Item* pi = t.template find<Multi>(s - 1, node);
    if (pi) { prev.exists = true; prev.sEnd = pi->sEnd; prev.HP = pi->HP; prev.HN = pi->HN; }
    else { prev.exists = false; prev.sEnd = 0; prev.HP = kAllOnes; prev.HN = 0; }
    Item copy = *it;
    WS start = ws_make(it->sVP, it->sVN, it->sEnd);
    u64 steps = 0;
    int err = 0;
    int64_t j = ((int64_t)s - 1) * 64;
    node_calc<false, Multi>(g, cost, node, copy, eqv, prev, nullptr, kNil, &start, false, (i32)j, cols, eqcol, steps, err, lane, kIntMin, lastColumn,
        (Multi && extra.end != kIntMax) ? &extra : nullptr);
    if (err) return err;
    u32 L = g.len[node];
    if (!ws_eq(ws_make(cols[0].VP, cols[0].VN, cols[0].end), start)) return GA_ASSERT;
    if (lastColumn + 1 >= L && !ws_eq(ws_make(cols[L - 1].VP, cols[L - 1].VN, cols[L - 1].end), ws_make(it->eVP, it->eVN, it->eEnd)))
        return GA_ASSERT;
    return 0;
}

// pickBacktraceVerticalCrossing (Common.h:886-934), the step out of (p.node, p.off > 0, row 0)
// into the previous slice; pself is the node's entry there
template <bool Multi>
__device__ __noinline__ TStep vertical_step(const DevGraph& g, const uint8_t* seq, Table t, u32 curSlice, const Item* pself, const Col* cols,
    TPos p, int& err, WS extra)
{
    TStep second;
    second.pos = p;
    second.sw = false;
    const SliceRec* cr = t.rec(curSlice);
    const SliceRec* pr = t.rec(curSlice - 1);
    bool bad = false;
    bool eq = char_match(g, seq[p.seq], p.node, p.off, bad);
    if (bad) { err = GA_ASSERT; return second; }
    i32 here = col_value(cols[p.off], 0);
    // the previous slice's last row at column p.off - 1: its first column plus the deltas of columns 1..p.off-1
    const u64 upto = p.off >= 2 ? ((kAllOnes >> (64 - (p.off - 1))) << 1) : 0;
    i32 diag = pself->sEnd + popc64(pself->HP & upto) - popc64(pself->HN & upto);
    i32 up = diag + (i32)((pself->HP >> p.off) & 1) - (i32)((pself->HN >> p.off) & 1);
    if (pr->notValid || cr->notValid || here > cr->quit || diag > pr->quit || up > pr->quit)
    {
        if (here == xval<Multi>(extra, 0)) second = TStep { p, false };
        else if (diag < up) second = TStep { TPos { p.node, p.off - 1, p.seq - 1 }, false };
        else second = TStep { TPos { p.node, p.off, p.seq - 1 }, false };
        return second;
    }
    if (up < here - 1 || diag < here - (eq ? 0 : 1)) { err = GA_ASSERT; return second; }
    if (up == here - 1) return TStep { TPos { p.node, p.off, p.seq - 1 }, false };
    if (diag == here - (eq ? 0 : 1)) return TStep { TPos { p.node, p.off - 1, p.seq - 1 }, false };
    if (here != xval<Multi>(extra, 0)) err = GA_ASSERT;
    return second;
}

// pickBacktraceHorizontalCrossing (Common.h:817-884), the step out of (p.node, offset 0,
// row off > 0) into an in-neighbour; self is the node's entry in the slice
template <bool Multi>
__device__ __noinline__ TStep horizontal_step(const DevGraph& g, const uint8_t* seq, Table t, u32 curSlice, u32 curNode, const Item* self,
    TPos p, u32 off, int& err, WS extra)
{
    TStep second;
    second.pos = p;
    second.sw = false;
    const SliceRec* cr = t.rec(curSlice);
    bool bad = false;
    bool eq = char_match(g, seq[p.seq], p.node, p.off, bad);
    if (bad) { err = GA_ASSERT; return second; }
    WS sws = ws_make(self->sVP, self->sVN, self->sEnd);
    i32 here = ws_value(sws, (int)off);
    if (cr->notValid || here > cr->quit)
    {
        i32 smallest = ws_value(sws, (int)off - 1);
        TPos sp = TPos { curNode, 0, p.seq - 1 };
        bool change = false;
        #pragma unroll 1
        for (u32 e = g.inOff[curNode]; e < g.inOff[curNode + 1]; e++)
        {
            u32 nb = g.inNb[e];
            const Item* cn = t.template find<Multi>(curSlice, nb);
            if (cn)
            {
                WS nws = ws_make(cn->eVP, cn->eVN, cn->eEnd);
                if (ws_value(nws, (int)off - 1) <= smallest)
                {
                    smallest = ws_value(nws, (int)off - 1);
                    sp = TPos { nb, g.len[nb] - 1, p.seq - 1 };
                    change = true;
                }
                if (ws_value(nws, (int)off) < smallest && nb != curNode)
                {
                    smallest = ws_value(nws, (int)off);
                    sp = TPos { nb, g.len[nb] - 1, p.seq };
                    change = true;
                }
            }
        }
        if (tpos_eq(sp, p) && here != xval<Multi>(extra, (int)off)) { err = GA_ASSERT; return second; }
        return TStep { sp, change };
    }
    #pragma unroll 1
    for (u32 e = g.inOff[curNode]; e < g.inOff[curNode + 1]; e++)
    {
        u32 nb = g.inNb[e];
        const Item* cn = t.template find<Multi>(curSlice, nb);
        if (!cn) continue;
        WS nws = ws_make(cn->eVP, cn->eVN, cn->eEnd);
        i32 v0 = ws_value(nws, (int)off);
        i32 v1 = ws_value(nws, (int)off - 1);
        if (v0 < here - 1 || v1 < here - (eq ? 0 : 1)) { err = GA_ASSERT; return second; }
        if (v0 == here - 1) return TStep { TPos { nb, g.len[nb] - 1, p.seq }, true };
        if (v1 == here - (eq ? 0 : 1)) return TStep { TPos { nb, g.len[nb] - 1, p.seq - 1 }, true };
    }
    if (here != xval<Multi>(extra, (int)off)) { err = GA_ASSERT; return second; }
    return TStep { p, false };
}

struct EndCell
{
    u32 node;
    u32 nodeOffset;
    u32 bvOffset;
    i32 score;
    int64_t j;
    int err;
};

// getReverseTraceFromTableExactEndPos (Common.h:496-562): the first slice of greatest
// X-score (lanes stride over the slices), then across the lanes (lane k: columns k and
// k + 32 of its best node) the cell of greatest row among those scoring the slice's
// X-score, the first column on ties.  The node's columns are left in cols.
__device__ __noinline__ EndCell end_cell(const DevGraph& g, i32 cost, const uint8_t* arena, Table t, u32 committed, const uint8_t* seq,
    u32 seqLen, Col* cols, u64* eqcol, u32 lane)
{
    EndCell ec;
    ec.err = 0;
    ec.nodeOffset = 0xffffffffu;
    ec.bvOffset = 0xffffffffu;
    i32 bx = kIntMin;
    u32 bs = 0xffffffffu;
    #pragma unroll 1
    for (u32 s = 1 + lane; s < committed; s += 32)
    {
        const i32 mx = ((const SliceRec*)(arena + t.dir[s]))->maxX;
        if (mx > bx) { bx = mx; bs = s; }
    }
    const i32 gbx = __reduce_max_sync(kFull, bx);
    const u32 best = __reduce_min_sync(kFull, bx == gbx ? bs : 0xffffffffu);
    const SliceRec* br = t.rec(best);
    ec.node = br->maxXNode;
    ec.score = br->maxX;
    ec.j = ((int64_t)best - 1) * 64;
    const int64_t j = ec.j;
    EqV4 eqv;
    if (!eq_vector(seq, seqLen, j, eqv, lane)) { ec.err = GA_ASSERT; return ec; }
    ec.err = recalc(g, cost, t, best, ec.node, eqv, cols, eqcol, lane, 63);
    if (ec.err) return ec;
    const int cells = (int)((int64_t)seqLen - j < 64 ? (int64_t)seqLen - j : 64);
    const u32 L = g.len[ec.node];
    bool bad = false;
    int candOff = -1;
    u32 candCol = 0xffffffffu;
    #pragma unroll 1
    for (u32 h = 0; h < 2; h++)
    {
        const u32 i = lane + 32 * h;
        if (i >= L || bad) continue;
        const WS cw = ws_make(cols[i].VP, cols[i].VN, cols[i].end);
        i32 mx = ws_max_xscore(cw, (i32)j, cost, cells, kAllOnes);
        if (mx > ec.score) { bad = true; continue; }
        if (mx == ec.score)
        {
            #pragma unroll 1
            for (int off = 63; off >= 0; off--)
            {
                if (j + off >= (int64_t)seqLen) continue;
                i32 here = ws_xscore(cw, (i32)j, off, cost);
                if (here > ec.score) { bad = true; break; }
                if (here == ec.score && off > candOff)
                {
                    candOff = off;
                    candCol = i;
                }
            }
        }
    }
    if (__ballot_sync(kFull, bad)) { ec.err = GA_ASSERT; return ec; }
    const int gOff = __reduce_max_sync(kFull, candOff);
    const u32 gCol = __reduce_min_sync(kFull, candOff == gOff ? candCol : 0xffffffffu);
    if (gOff < 0 || j + gOff >= (int64_t)seqLen) { ec.err = GA_ASSERT; return ec; }
    ec.nodeOffset = gCol;
    ec.bvOffset = (u32)gOff;
    return ec;
}

// the start node's row above the read (Common.h:721-756): walks left along the start
// slice while the score falls by one, then into an in-neighbour at offset 0
__device__ __noinline__ int row_above(const DevGraph& g, Table t, TraceOut& to)
{
    if (to.back.seq != -1) return GA_ASSERT;
    const Item* it = t.find(0, to.back.node);
    if (!it) return GA_ASSERT;
    const u32 L = g.len[to.back.node];
    // before[k] = score of column k in the row above the read
    const u64 hp = it->HP, hn = it->HN;
    const i32 s0 = it->sEnd;
    auto before = [&](u32 k) -> i32
    {
        const u64 upto = k >= 1 ? ((kAllOnes >> (64 - k)) << 1) : 0;   // columns 1..k
        return s0 + popc64(hp & upto) - popc64(hn & upto);
    };
    if (before(L - 1) != it->eEnd) return GA_ASSERT;
    #pragma unroll 1
    while (!to.overflow)
    {
        TPos q = to.back;
        i32 bq = before(q.off);
        if (!(bq != 0 && q.off > 0 && before(q.off - 1) == bq - 1)) break;
        to.push(TPos { q.node, q.off - 1, q.seq }, false);
    }
    TPos q = to.back;
    if (!to.overflow && q.off == 0 && before(0) != 0)
    {
        #pragma unroll 1
        for (u32 e = g.inOff[q.node]; e < g.inOff[q.node + 1]; e++)
        {
            u32 nb = g.inNb[e];
            const Item* ni = t.find(0, nb);
            if (ni && ws_before(ws_make(ni->eVP, ni->eVN, ni->eEnd)) == before(0) - 1)
            {
                to.push(TPos { nb, g.len[nb] - 1, q.seq }, true);
                break;
            }
        }
    }
    return 0;
}

// The first column of the run of row-0 steps that ends at column off: the least c <= off with
// score(c') = score(c' - 1) + 1 for every c < c' <= off (pickBacktraceVerticalCrossing's walk
// along the slice's first row, Common.h:886-900).  Columns 0..off must be in cols.
__device__ __forceinline__ u32 row0_run_start(const Col* cols, u32 off, u32 lane)
{
    const i32 v0 = col_value(cols[lane], 0);
    const i32 v1 = col_value(cols[lane + 32], 0);
    i32 p0 = __shfl_up_sync(kFull, v0, 1);
    i32 p1 = __shfl_up_sync(kFull, v1, 1);
    const i32 v31 = __shfl_sync(kFull, v0, 31);
    if (lane == 0) p1 = v31;
    // bit c: column c continues the run (column 0 never does)
    const u64 cont = (u64)(__ballot_sync(kFull, lane > 0 && p0 == v0 - 1)) | ((u64)__ballot_sync(kFull, p1 == v1 - 1) << 32);
    const u64 stops = ~cont & (off == 63 ? kAllOnes : ((2ULL << off) - 1));
    return 63 - __clzll((long long)stops);
}

// getReverseTraceFromTable's walk (Common.h:571-720) from `start`, whose score is startScore,
// up to the row above the read or, in the multiseed DP (Multi), to a seed start.  resultScore:
// the trace's OnewayTrace::score.  Returns 0 or the error status.
template <bool Multi>
__device__ __forceinline__ int trace_walk(const DevGraph& g, i32 cost, const uint8_t* seq, u32 seqLen, u32 committed, Table& t, TraceOutT<Multi>& to, const WSpace& w,
    TPos start, i32 startScore, i32& resultScore, u32 lane)
{
    int err = 0;
    Col* cols = w.cols;
    const u64 guardMax = (u64)((Multi && to.counting) ? (1u << 26) : to.cap) * 4 + 1024;
    resultScore = startScore;
    to.push(start, false);
    // the extraSlice of the current node-slice and its score at a row
    WS extra = fake_ws();
    auto xv = [&](u32 row) -> i32 { return Multi ? ws_value(extra, (int)row) : kIntMax; };
    u32 curSlice = (u32)(start.seq / 64) + 1;
    u32 curNode = 0xffffffffu;
    u32 curLen = 0;
    u32 colsUpTo = 0;             // columns 0..colsUpTo of (curSlice, curNode) are in cols, their match masks in eqcol
    EqV4 eqv;
    if (!eq_vector(seq, seqLen, ((int64_t)curSlice - 1) * 64, eqv, lane)) err = GA_ASSERT;
    i32 lastScore = kIntMax - 1;
    u64 guard = 0;
    #pragma unroll 1
    while (!err && !to.overflow && to.back.seq != -1)
    {
        if (++guard > guardMax) { err = GA_CAPACITY; break; }
        TPos b = to.back;
        u32 newSlice = (u32)(b.seq / 64) + 1;
        if (newSlice >= committed) { err = GA_ASSERT; break; }
        // a self-loop can re-enter the same node-slice further right than it was computed
        if (newSlice != curSlice || b.node != curNode || b.off > colsUpTo)
        {
            if (newSlice != curSlice && !eq_vector(seq, seqLen, ((int64_t)newSlice - 1) * 64, eqv, lane)) { err = GA_ASSERT; break; }
            curSlice = newSlice;
            curNode = b.node;
            if (curSlice == 0) { err = GA_ASSERT; break; }
            if (Multi)
            {
                const Item* here = t.template find<Multi>(curSlice, curNode);
                if (!here) { err = GA_ASSERT; break; }
                extra = (here->node & kSeedStart) ? seed_ws(((int64_t)curSlice - 1) * 64, seqLen, cost) : fake_ws();
            }
            err = recalc<Multi>(g, cost, t, curSlice, curNode, eqv, cols, w.eqcol, lane, b.off, extra);
            if (err) break;
            colsUpTo = b.off;
            curLen = g.len[curNode];
        }
        const int64_t sj = ((int64_t)curSlice - 1) * 64;
        if (b.off >= curLen) { err = GA_ASSERT; break; }
        const u32 row = mod64(b.seq);
        lastScore = col_value(cols[b.off], (int)row);
        if (row == 0 && b.off == 0)
        {
            TStep bt = bt_corner<Multi>(g, seq, t, curSlice, curNode, sj, err, extra);
            if (err) break;
            if (tpos_eq(bt.pos, b) && !bt.sw && col_value(cols[bt.pos.off], (int)mod64(bt.pos.seq)) == xv(mod64(bt.pos.seq))) break;
            if (Multi && tpos_eq(bt.pos, b) && !bt.sw && col_value(cols[bt.pos.off], (int)mod64(bt.pos.seq)) == ws_before(extra)) break;
            to.push(bt.pos, bt.sw);
            if (!to.overflow && trace_circular(to.items, to.ring, to.n, Multi && to.counting)) { err = GA_ASSERT; break; }
            continue;
        }
        if (row == 0)
        {
            const Item* pself = t.template find<Multi>(curSlice - 1, curNode);
            if (!pself)
            {
                #pragma unroll 1
                for (u32 k = b.off - 1; k > 0; k--) to.push(TPos { curNode, k, b.seq }, false);
                to.push(TPos { curNode, 0, b.seq }, false);
                continue;
            }
            // pickBacktraceVerticalCrossing (Common.h:886-934)
            // step left along row 0 while the score falls by one per column: lane k tests
            // columns k and k + 32 against their left neighbours, the run ends at the
            // highest failing column at or below b.off (column 0 always ends it)
            TPos p = b;
            p.off = row0_run_start(cols, b.off, lane);
            TStep second = p.off == 0 ? bt_corner<Multi>(g, seq, t, curSlice, curNode, sj, err, extra) : vertical_step<Multi>(g, seq, t, curSlice, pself, cols, p, err, extra);
            if (err) break;
            if (second.pos.seq == b.seq && col_value(cols[second.pos.off], (int)mod64(second.pos.seq)) == xv(mod64(second.pos.seq))) break;
            if (p.off != b.off)
            {
                #pragma unroll 1
                for (u32 k = b.off - 1; k != p.off; k--) to.push(TPos { p.node, k, p.seq }, false);
            }
            if (!tpos_eq(p, to.back)) to.push(p, false);
            if (tpos_eq(second.pos, to.back)) { err = GA_ASSERT; break; }
            to.push(second.pos, second.sw);
            continue;
        }
        if (b.off == 0)
        {
            // pickBacktraceHorizontalCrossing (Common.h:817-884)
            const Item* self = t.template find<Multi>(curSlice, curNode);
            if (!self) { err = GA_ASSERT; break; }
            // step up column 0 while its score falls by one per row (the start column's VP
            // bits): the run ends at the highest row at or below this one whose bit is clear
            // (row 0 always ends it)
            TPos p = b;
            {
                const u32 r = mod64(b.seq);
                const u64 stops = (~self->sVP | 1ULL) & (r == 63 ? kAllOnes : ((2ULL << r) - 1));
                p.seq -= (int64_t)(r - (63 - __clzll((long long)stops)));
            }
            const u32 off = mod64(p.seq);
            TStep second = off == 0 ? bt_corner<Multi>(g, seq, t, curSlice, curNode, sj, err, extra) : horizontal_step<Multi>(g, seq, t, curSlice, curNode, self, p, off, err, extra);
            if (err) break;
            if (second.pos.node == b.node && !second.sw && col_value(cols[second.pos.off], (int)mod64(second.pos.seq)) == xv(mod64(second.pos.seq))) break;
            if (p.seq != b.seq)
            {
                #pragma unroll 1
                for (int64_t sp = b.seq - 1; sp != p.seq; sp--) to.push(TPos { p.node, p.off, sp }, false);
            }
            if (!tpos_eq(p, to.back)) to.push(p, false);
            if (tpos_eq(second.pos, to.back)) { err = GA_ASSERT; break; }
            to.push(second.pos, second.sw);
            if (!to.overflow && trace_circular(to.items, to.ring, to.n, Multi && to.counting)) { err = GA_ASSERT; break; }
            continue;
        }
        // pickBacktraceInside (Common.h:770-815).  The four neighbouring scores are
        // carried incrementally: a vertical step moves up one row in both columns
        // (score(r-1) = score(r) - VP_r + VN_r); a diagonal or horizontal step makes
        // the left column current and loads the next one.  The read/graph match of
        // a cell is bit `row` of the column's match mask (the fill's Eq), which is
        // GraphAlignerCommon::characterMatch for every read and graph character.
        {
            u32 hori = b.off;
            u32 vert = row;
            // the recomputation left each column's match mask (the fill's Eq) in eqcol
            const u64* eqcol = w.eqcol;
            if (hori > 0 && vert > 0)
            {
                WS colH = ws_make(cols[hori].VP, cols[hori].VN, cols[hori].end);
                WS colL = ws_make(cols[hori - 1].VP, cols[hori - 1].VN, cols[hori - 1].end);
                i32 here = ws_value(colH, (int)vert);
                i32 left = ws_value(colL, (int)vert);
                u64 eqH = eqcol[hori];
                #pragma unroll 1
                while (true)
                {
                    const i32 vs = here - (i32)((colH.VP >> vert) & 1) + (i32)((colH.VN >> vert) & 1);
                    const i32 ds = left - (i32)((colL.VP >> vert) & 1) + (i32)((colL.VN >> vert) & 1);
                    const bool eq = (eqH >> vert) & 1;
                    if (vs == here - 1)
                    {
                        vert--;
                        to.push(TPos { b.node, hori, sj + vert }, false);
                        here = vs;
                        left = ds;
                    }
                    else if (ds == here - (eq ? 0 : 1))
                    {
                        hori--;
                        vert--;
                        to.push(TPos { b.node, hori, sj + vert }, false);
                        here = ds;
                        colH = colL;
                        if (hori > 0)
                        {
                            colL = ws_make(cols[hori - 1].VP, cols[hori - 1].VN, cols[hori - 1].end);
                            left = ws_value(colL, (int)vert);
                            eqH = eqcol[hori];
                        }
                    }
                    else if (left == here - 1)
                    {
                        hori--;
                        to.push(TPos { b.node, hori, sj + vert }, false);
                        here = left;
                        colH = colL;
                        if (hori > 0)
                        {
                            colL = ws_make(cols[hori - 1].VP, cols[hori - 1].VN, cols[hori - 1].end);
                            left = ws_value(colL, (int)vert);
                            eqH = eqcol[hori];
                        }
                    }
                    else
                    {
                        if (here != xv(vert)) err = GA_ASSERT;
                        break;
                    }
                    if (to.overflow || hori == 0 || vert == 0) break;
                }
            }
            if (err || to.overflow) break;
            if (col_value(cols[to.back.off], (int)mod64(to.back.seq)) == xv(mod64(to.back.seq))) break;
        }
    }
    if (!err && !to.overflow)
    {
        if (resultScore < lastScore) err = GA_ASSERT;
        resultScore -= lastScore;
    }
    return err;
}

__device__ void trace_extension(const TraceArgs& a, u32 ext, const ExtState& st, const WSpace& w, u32 lane)
{
    const DevGraph& g = a.g;
    u64* out = a.traceItems + a.traceOffset[ext];
    const u32 cap = a.traceCap[ext];
    if (lane == 0 && a.cellSteps) a.cellSteps[ext] = st.steps;
    if (st.status != GA_OK)
    {
        if (lane == 0)
        {
            a.status[ext] = st.status;
            a.score[ext] = 0;
            a.traceLen[ext] = 0;
        }
        return;
    }
    const uint8_t* seq = a.seq + a.seqOff[ext];
    const u32 seqLen = a.seqLen[ext];
    Table t;
    t.arena = a.arena;
    t.dir = (const u64*)(a.arena + st.dir);
    t.count = st.committed;
    t.lane = lane;
    t.slots = w.slots;
    t.init();
    Col* cols = w.cols;
    TraceOut to;
    to.items = out;
    to.ring = w.ring;
    to.cap = cap;
    to.n = 0;
    to.lane = lane;
    to.overflow = false;
    int err = 0;
    i32 resultScore = 0;
    const EndCell ec = end_cell(g, a.cost, a.arena, t, st.committed, seq, seqLen, cols, w.eqcol, lane);
    err = ec.err;
    if (!err)
    {
        // getReverseTraceFromTable (Common.h:571-758)
        TPos start = TPos { ec.node, ec.nodeOffset, ec.j + ec.bvOffset };
        i32 startScore = col_value(cols[ec.nodeOffset], (int)ec.bvOffset);
        err = trace_walk<false>(g, a.cost, seq, seqLen, st.committed, t, to, w, start, startScore, resultScore, lane);
        if (!err && !to.overflow) err = row_above(g, t, to);
    }
    to.finish();
    int status = err ? err : (to.overflow ? GA_CAPACITY : GA_OK);
    if (lane == 0)
    {
        a.status[ext] = status;
        a.score[ext] = status == GA_OK ? resultScore : 0;
        a.traceLen[ext] = status == GA_OK ? to.n : 0;
    }
}

// The multiseed DP's best X-score of node in committed slice s (read from the arena); false
// when the node is not in the slice's band
__device__ __forceinline__ bool slice_node_max(const uint8_t* arena, const u64* dir, u32 s, u32 node, u32 lane, i32& out)
{
    const SliceRec* r = (const SliceRec*)(arena + dir[s]);
    const int k = rec_index<true>(r, (const u32*)((const uint8_t*)r + sizeof(SliceRec)), node, lane);
    if (k < 0) return false;
    out = rec_node_max(r)[k];
    return true;
}

// getLocalMaximaTracesFromTable's (Common.h:355-494) local-maximum test of `node` in committed
// slice cs, whose best X-score there is `score`: not below its own in the slices above and
// below, nor below its in-neighbours' in this slice and the one above or its out-neighbours'
// in this slice and the one below.
__device__ bool ms_local_max(const DevGraph& g, const uint8_t* arena, const u64* dir, u32 cs, u32 last, u32 node, i32 score, u32 lane)
{
    i32 other;
    if (slice_node_max(arena, dir, cs - 1, node, lane, other) && other > score) return false;
    if (cs < last && slice_node_max(arena, dir, cs + 1, node, lane, other) && other >= score) return false;
#pragma unroll 1
    for (u32 e = g.inOff[node]; e < g.inOff[node + 1]; e++)
    {
        const u32 nb = g.inNb[e];
        if (slice_node_max(arena, dir, cs, nb, lane, other) && other > score) return false;
        if (slice_node_max(arena, dir, cs - 1, nb, lane, other) && other > score) return false;
    }
#pragma unroll 1
    for (u32 e = g.outOff[node]; e < g.outOff[node + 1]; e++)
    {
        const u32 nb = g.outNb[e];
        if (slice_node_max(arena, dir, cs, nb, lane, other) && other > score) return false;
        if (cs < last && slice_node_max(arena, dir, cs + 1, nb, lane, other) && other > score) return false;
    }
    return true;
}

// The candidates of read r in getLocalMaximaTracesFromTable's order (slices from the last,
// band order within a slice): band nodes whose best X-score is positive, reaches the
// multimap fraction of the slice's best as the fill left it and is a local maximum.  The
// slice bests only rise as traces are taken, so the traces the read keeps are among these.
// write = false counts them and reserves the read's run of the list; write = true fills it.
__device__ void ms_candidates(const MultiTraceArgs& a, u32 r, const ExtState& st, bool write, u32 lane)
{
    u32 c = 0;
    const u64 base = write ? a.candBegin[r] : 0;
    if (st.status == GA_OK)
    {
        const u64* dir = (const u64*)(a.arena + st.dir);
        const i32* sliceMax = (const i32*)(a.arena + st.aux);
        const u32 last = st.committed - 1;
#pragma unroll 1
        for (u32 cs = last; cs >= 1; cs--)
        {
            const SliceRec* cr = (const SliceRec*)(a.arena + dir[cs]);
            if (cr->maxX <= 0) continue;
            const u32 n = cr->count;
            const u32* ids = (const u32*)((const uint8_t*)cr + sizeof(SliceRec));
            const Item* items = (const Item*)((const uint8_t*)ids + rec_ids_bytes(n));
            const i32* nodeMax = rec_node_max(cr);
            const double threshold = (double)sliceMax[cs] * a.multimapScoreFraction;
#pragma unroll 1
            for (u32 b = 0; b < n; b += 32)
            {
                const u32 k = b + lane;
                bool pass = false;
                if (k < n)
                {
                    const i32 score = nodeMax[k];
                    pass = (items[k].node & kExists) && score > 0 && !((double)score < threshold);
                }
                u32 m = __ballot_sync(kFull, pass);
#pragma unroll 1
                while (m)
                {
                    const u32 kk = b + __ffs((int)m) - 1;
                    m &= m - 1;
                    const u32 node = ids[kk];
                    const i32 score = nodeMax[kk];
                    if (!ms_local_max(a.g, a.arena, dir, cs, last, node, score, lane)) continue;
                    if (write && lane == 0 && base + c < a.candCap)
                    {
                        MsCand x {};
                        x.read = r;
                        x.slice = cs;
                        x.index = kk;
                        x.score = score;
                        x.slot = kNoSlot;
                        a.cands[base + c] = x;
                    }
                    c++;
                }
            }
        }
    }
    if (!write && lane == 0)
    {
        a.candCount[r] = c;
        a.candBegin[r] = c ? atomicAdd(a.candTotal, (unsigned long long)c) : 0;
    }
    __syncwarp();
}

// The first cell of a candidate's trace (getLocalMaximaTracesFromTable): among the node's
// columns, recomputed with its seed start, the cell of greatest row that scores the node's
// best X-score (the first column on ties); a cell above it is GA_ASSERT.
__device__ int ms_start_cell(const MultiTraceArgs& a, Table& t, const WSpace& w, const uint8_t* seq, u32 seqLen, const MsCand& c,
    TPos& start, i32& startScore, u32 lane)
{
    const DevGraph& g = a.g;
    const SliceRec* cr = (const SliceRec*)(a.arena + t.dir[c.slice]);
    const Item* items = (const Item*)((const uint8_t*)cr + sizeof(SliceRec) + rec_ids_bytes(cr->count));
    const u32 node = items[c.index].node & kNodeMask;
    const int64_t j = ((int64_t)c.slice - 1) * 64;
    EqV4 eqv;
    if (!eq_vector(seq, seqLen, j, eqv, lane)) return GA_ASSERT;
    const WS extra = (items[c.index].node & kSeedStart) ? seed_ws(j, seqLen, a.cost) : fake_ws();
    int err = recalc<true>(g, a.cost, t, c.slice, node, eqv, w.cols, w.eqcol, lane, 63, extra);
    if (err) return err;
    const Col* cols = w.cols;
    const i32 score = c.score;
    const int cells = (int)((int64_t)seqLen - j < 64 ? (int64_t)seqLen - j : 64);
    const u32 L = g.len[node];
    bool bad = false;
    int candOff = -1;
    u32 candCol = 0xffffffffu;
#pragma unroll 1
    for (u32 h = 0; h < 2; h++)
    {
        const u32 i = lane + 32 * h;
        if (i >= L || bad) continue;
        const WS cw = ws_make(cols[i].VP, cols[i].VN, cols[i].end);
        const i32 mx = ws_max_xscore(cw, (i32)j, a.cost, cells, kAllOnes);
        if (mx > score) { bad = true; continue; }
        if (mx != score) continue;
#pragma unroll 1
        for (int off = 63; off >= 0; off--)
        {
            if (j + off >= (int64_t)seqLen) continue;
            const i32 here = ws_xscore(cw, (i32)j, off, a.cost);
            if (here > score) { bad = true; break; }
            if (here == score && off > candOff)
            {
                candOff = off;
                candCol = i;
            }
        }
    }
    if (__ballot_sync(kFull, bad)) return GA_ASSERT;
    const int gOff = __reduce_max_sync(kFull, candOff);
    const u32 gCol = __reduce_min_sync(kFull, candOff == gOff ? candCol : 0xffffffffu);
    if (gOff < 0 || j + gOff >= (int64_t)seqLen) return GA_ASSERT;
    start = TPos { node, gCol, j + gOff };
    startScore = col_value(cols[gCol], gOff);
    return 0;
}

// One candidate's trace (getReverseTraceFromTable to a seed start).  write = false: finds the
// first cell and walks the trace only counting its items, recording its length, score, read
// span and last cell.  write = true (a kept trace of a read whose traces all fit and, with
// exact room, that removeDuplicateTraces kept): walks it again into the read's output at
// the place the read's selection (or the host, with exact room) gave it.
__device__ void ms_trace_cand(const MultiTraceArgs& a, MsCand* cp, const WSpace& w, bool write, u32 lane)
{
    const MsCand c = *cp;
    const u32 r = c.read;
    if (write)
    {
        // the read's status can change under other warps (a kept trace of it that failed)
        int readStatus = 0;
        if (lane == 0) readStatus = a.status[r];
        readStatus = __shfl_sync(kFull, readStatus, 0);
        if (c.slot == kNoSlot || readStatus != GA_OK) return;
    }
    const ExtState st = a.states[r];
    const uint8_t* seq = a.seq + a.seqOff[r];
    const u32 seqLen = a.seqLen[r];
    Table t;
    t.arena = a.arena;
    t.dir = (const u64*)(a.arena + st.dir);
    t.count = st.committed;
    t.lane = lane;
    t.slots = w.slots;
    t.init();
    TPos start;
    i32 startScore = 0;
    int err = 0;
    if (write)
    {
        start = TPos { c.startNode, c.startOff, c.startSeq };
        startScore = c.startScore;
    }
    else
    {
        err = ms_start_cell(a, t, w, seq, seqLen, c, start, startScore, lane);
    }
    const bool exact = a.traceBase != nullptr;
    // exact room: the kept trace's place after the duplicates went, or none
    const u64 kept = exact && write ? a.traceBase[r] + c.slot : 0;
    const u32 outSlot = exact && write ? a.keptSlot[kept] : 0;
    if (exact && write && outSlot == kNoSlot) return;
    TraceOutT<true> to;
    to.items = write ? a.traceItems + (exact ? a.keptItem[kept] : a.traceOffset[r] + c.outOff) : nullptr;
    to.ring = w.ring;
    to.lane = lane;
    to.counting = !write;
    to.cap = write ? c.len : 0xffffffffu;
    to.n = 0;
    to.overflow = false;
    to.back = start;
    i32 traceScore = 0;
    if (!err)
    {
        err = trace_walk<true>(a.g, a.cost, seq, seqLen, st.committed, t, to, w, start, startScore, traceScore, lane);
        to.finish();
        // a walk past its step guard or its counted length is broken, not short of room
        if (err == GA_CAPACITY || (!err && to.overflow)) err = GA_ASSERT;
        if (!err && (to.back.seq < 0 || start.seq < to.back.seq)) err = GA_ASSERT;
    }
    if (lane == 0)
    {
        if (!write)
        {
            cp->startNode = start.node;
            cp->startOff = start.off;
            cp->startSeq = start.seq;
            cp->startScore = startScore;
            cp->err = err;
            cp->traceScore = traceScore;
            cp->len = err ? 0 : to.n;
            cp->traceStart = to.back.seq;
            cp->lastNode = to.back.node;
            cp->lastOff = to.back.off;
            cp->state = kTraced;
        }
        else if (err || to.n != c.len || traceScore != c.traceScore)
        {
            // the walk differs from its count only where the written trace's full circularity
            // check (the counting walk checks the ring) stops it
            a.status[r] = err ? err : GA_ASSERT;
            a.numTraces[r] = 0;
        }
        else
        {
            const u64 slot = exact ? outSlot : (u64)r * a.maxTraces + c.slot;
            a.traceScore[slot] = traceScore;
            a.traceStart[slot] = exact ? a.itemBias + a.keptItem[kept] : c.outOff;
            a.traceLen[slot] = to.n;
        }
    }
    __syncwarp();
}

// getLocalMaximaTracesFromTable's selection for read r, one round: its candidates in order
// from the cursor.  A candidate below the multimap fraction of its slice's best (as raised so
// far) is passed over for good, the slice bests only rise.  One that reaches it is kept once
// its trace has been walked, and raises the best of the slices its trace spans beyond its
// first 5 %; the first one whose walk is still to come stops the round.  Then the read queues
// that walk and up to window - 1 more of the candidates after it that the slice bests do not
// yet rule out.  Kept traces get their place in the read's output while they fit its room
// (max_traces, trace_capacity); past that they are only counted, and the read reports the
// room it needs.  With exact room (a.traceBase) every kept trace gets its place, and the read
// reports the items they take.  A kept trace that failed fails the read.
__device__ void ms_resolve(const MultiTraceArgs& a, u32 r, const ExtState& st, u32 lane)
{
    MsSel* sp = a.sel + r;
    if (sp->done) return;
    if (st.status != GA_OK)
    {
        if (lane == 0)
        {
            if (a.cellSteps) a.cellSteps[r] = st.steps;
            a.status[r] = st.status;
            a.numTraces[r] = 0;
            sp->done = 1;
        }
        __syncwarp();
        return;
    }
    MsSel sel = *sp;
    i32* sliceMax = (i32*)(a.arena + st.aux);
    const bool exact = a.traceBase != nullptr;
    const u64 cap = exact ? ~0ULL : a.traceCap[r];
    const u32 maxTraces = exact ? 0xffffffffu : a.maxTraces;
    const u64 begin = a.candBegin[r];
    const u32 count = a.candCount[r];
    int err = 0;
    u32 i = sel.cursor;
#pragma unroll 1
    for (; i < count; i++)
    {
        MsCand* cp = a.cands + begin + i;
        const u32 cs = cp->slice;
        const i32 score = cp->score;
        if ((double)score < (double)sliceMax[cs] * a.multimapScoreFraction) continue;
        if (cp->state != kTraced) break;
        if (cp->err)
        {
            err = cp->err;
            break;
        }
        const u32 len = cp->len;
        if (!sel.full && (sel.nt >= maxTraces || len > cap - sel.used)) sel.full = 1;
        if (!sel.full)
        {
            if (lane == 0)
            {
                cp->slot = sel.nt;
                cp->outOff = sel.used;
            }
            sel.used += len;
            sel.nt++;
        }
        sel.items += len;
        sel.traces++;
        const int64_t traceEnd = cp->startSeq, traceStart = cp->traceStart;
        const u32 startSlice = (u32)(((double)(traceEnd - traceStart) * 0.05 + (double)traceStart + 64 - 1) / 64 + 1);
        __syncwarp();
#pragma unroll 1
        for (u32 k = startSlice + lane; k < cs; k += 32) sliceMax[k] = imax(sliceMax[k], score);
        __syncwarp();
    }
    sel.cursor = i;
    if (err || i == count)
    {
        if (lane == 0)
        {
            const bool room = !sel.full;
            if (a.cellSteps) a.cellSteps[r] = st.steps;
            a.status[r] = err ? err : (room ? GA_OK : kMsRoom);
            a.numTraces[r] = (err || !room) ? 0 : sel.nt;
            // with exact room: the items the read's traces take
            if (a.itemsNeeded) a.itemsNeeded[r] = err ? 0 : (exact ? sel.used : (!room ? sel.items : 0));
            if (a.tracesNeeded) a.tracesNeeded[r] = (!err && !room) ? sel.traces : 0;
            sel.done = 1;
            *sp = sel;
        }
        __syncwarp();
        return;
    }
    // the walk the read waits for, and a few after it that may be kept too
    u32 queued = 0;
#pragma unroll 1
    for (u32 j = i; j < count && queued < a.window; j++)
    {
        MsCand* cp = a.cands + begin + j;
        if (cp->state != kUntraced) continue;
        if ((double)cp->score < (double)sliceMax[cp->slice] * a.multimapScoreFraction) continue;
        if (lane == 0)
        {
            cp->state = kQueued;
            a.work[atomicAdd(a.workCount, 1u)] = (u32)(begin + j);
        }
        queued++;
    }
    if (lane == 0) *sp = sel;
    __syncwarp();
}

// The next extension for this warp from the work counter, or false when none is left;
// with a filter only extensions whose previous status is GA_CAPACITY are taken.
__device__ __forceinline__ bool next_extension(u32* counter, u32 num, const u32* order, const i32* prevStatus, u32 lane, u32& ext)
{
#pragma unroll 1
    while (true)
    {
        u32 k = 0;
        if (lane == 0) k = atomicAdd(counter, 1u);
        k = __shfl_sync(kFull, k, 0);
        if (k >= num) return false;
        ext = order ? order[k] : k;
        if (!prevStatus || prevStatus[ext] == GA_CAPACITY) return true;
    }
}

// The fill: a warp takes the next extension of the longest-first order, fills its DP table
// into the arena and records where it is, then takes the next.  The frontier tables are in
// dynamic shared memory (fa.workspace == nullptr) or in the global workspace, one stride
// per warp.
__global__ void __launch_bounds__(128, 4) fill_kernel(FillArgs fa, u32* counter)
{
    extern __shared__ __align__(16) uint8_t dsmem[];
    load_iupac_table();
    const u32 lane = threadIdx.x & 31;
    const u32 warpInBlock = threadIdx.x >> 5;
    const u64 gwarp = (u64)blockIdx.x * (blockDim.x >> 5) + warpInBlock;
    uint8_t* base = fa.workspace ? fa.workspace + gwarp * fa.workspaceStride : dsmem + (u64)warpInBlock * fa.workspaceStride;
    const WSpace w = wspace_at(base, fa.caps);
    // generation 0 marks every node-table slot empty
#pragma unroll 1
    for (u32 k = lane; k < fa.caps.hash; k += 32)
    {
        w.key[0][k] = 0;
        w.key[1][k] = 0;
    }
    __syncwarp();
    u32 gen = 0;
    ArenaCursor arena;
    arena.pos = 0;
    arena.end = 0;
    arena.used = 0;
    u32 ext;
#pragma unroll 1
    while (next_extension(counter, fa.num, fa.order, fa.prevStatus, lane, ext))
    {
        __syncwarp();
        const ExtState st = fill_extension(fa, w, gen, arena, ext, lane);
        if (lane == 0) fa.states[ext] = st;
        if (gen > 0xF0000000u)
        {
            // generation stamps are about to wrap: clear this warp's tables
            __syncwarp();
#pragma unroll 1
            for (u32 k2 = lane; k2 < fa.caps.hash; k2 += 32)
            {
                w.key[0][k2] = 0;
                w.key[1][k2] = 0;
            }
            __syncwarp();
            gen = 0;
        }
    }
    if (lane == 0 && arena.used) atomicAdd(fa.arenaCursor + 1, (unsigned long long)arena.used);
}

static constexpr u32 kTraceSpaceBytes = 64 * sizeof(Col) + 64 * 8 + 64 * 8 + 2 * sizeof(SliceSlot);

// The traceback: a warp takes the next filled extension and walks its table back.  Its
// shared memory holds the recomputed columns, the match masks and the trace staging.
__global__ void __launch_bounds__(128, 6) trace_kernel(TraceArgs ta, u32* counter)
{
    extern __shared__ __align__(16) uint8_t dsmem[];
    load_iupac_table();
    const u32 lane = threadIdx.x & 31;
    uint8_t* base = dsmem + (u64)(threadIdx.x >> 5) * kTraceSpaceBytes;
    WSpace w {};
    w.cols = (Col*)base;
    w.eqcol = (u64*)(base + 64 * sizeof(Col));
    w.ring = (u64*)(base + 64 * sizeof(Col) + 64 * 8);
    w.slots = (SliceSlot*)(base + 64 * sizeof(Col) + 64 * 8 + 64 * 8);
    u32 ext;
#pragma unroll 1
    while (next_extension(counter, ta.num, ta.order, ta.prevStatus, lane, ext))
    {
        __syncwarp();
        trace_extension(ta, ext, ta.states[ext], w, lane);
    }
}


// The multiseed DP's fill: a warp takes the next read and fills its whole DP table; its
// frontier tables and per-node X-scores live in the global workspace.
__global__ void __launch_bounds__(128, 4) fill_multiseed_kernel(FillArgs fa, u32* counter)
{
    load_iupac_table();
    const u32 lane = threadIdx.x & 31;
    const u64 gwarp = (u64)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
    const WSpace w = wspace_at(fa.workspace + gwarp * fa.workspaceStride, fa.caps);
#pragma unroll 1
    for (u32 k = lane; k < fa.caps.hash; k += 32)
    {
        w.key[0][k] = 0;
        w.key[1][k] = 0;
    }
    __syncwarp();
    u32 gen = 0;
    ArenaCursor arena;
    arena.pos = 0;
    arena.end = 0;
    arena.used = 0;
    u32 r;
#pragma unroll 1
    while (next_extension(counter, fa.num, fa.order, fa.prevStatus, lane, r))
    {
        __syncwarp();
        const ExtState st = fill_multiseed(fa, w, gen, arena, r, lane);
        if (lane == 0) fa.states[r] = st;
        if (gen > 0xF0000000u)
        {
            __syncwarp();
#pragma unroll 1
            for (u32 k2 = lane; k2 < fa.caps.hash; k2 += 32)
            {
                w.key[0][k2] = 0;
                w.key[1][k2] = 0;
            }
            __syncwarp();
            gen = 0;
        }
    }
    if (lane == 0 && arena.used) atomicAdd(fa.arenaCursor + 1, (unsigned long long)arena.used);
}

// The per-read passes of the multiseed traceback (write = false: count the candidates and
// reserve their run; write = true: list them), a warp per read.
__global__ void __launch_bounds__(128, 6) ms_candidates_kernel(MultiTraceArgs ta, u32* counter, int write)
{
    const u32 lane = threadIdx.x & 31;
    u32 r;
#pragma unroll 1
    while (next_extension(counter, ta.num, ta.order, ta.prevStatus, lane, r))
    {
        __syncwarp();
        ms_candidates(ta, r, ta.states[r], write != 0, lane);
    }
}

// Exact room: each kept trace of a read that finished GA_OK, summarised for the host's
// removeDuplicateTraces, a thread per candidate.
__global__ void ms_keys_kernel(MultiTraceArgs ta)
{
    const u64 total = *ta.candTotal < ta.candCap ? *ta.candTotal : ta.candCap;
    for (u64 i = (u64)blockIdx.x * blockDim.x + threadIdx.x; i < total; i += (u64)gridDim.x * blockDim.x)
    {
        const MsCand& c = ta.cands[i];
        if (c.slot == kNoSlot || ta.status[c.read] != GA_OK) continue;
        MsKey k;
        k.first = c.startSeq;
        k.last = c.traceStart;
        k.lastNode = c.lastNode;
        k.lastOff = c.lastOff;
        k.score = c.traceScore;
        k.len = c.len;
        ta.keys[ta.traceBase[c.read] + c.slot] = k;
    }
}

__global__ void __launch_bounds__(128, 6) ms_resolve_kernel(MultiTraceArgs ta, u32* counter)
{
    const u32 lane = threadIdx.x & 31;
    u32 r;
#pragma unroll 1
    while (next_extension(counter, ta.num, ta.order, ta.prevStatus, lane, r))
    {
        __syncwarp();
        ms_resolve(ta, r, ta.states[r], lane);
    }
}

// The candidates' traces, a warp per candidate (write = false: the round's queued walks,
// counted; write = true: the kept ones written).  A read's traces spread over as many warps
// as it has walks in the round.
__global__ void __launch_bounds__(128, 6) ms_trace_kernel(MultiTraceArgs ta, u32* counter, int write)
{
    extern __shared__ __align__(16) uint8_t dsmem[];
    load_iupac_table();
    const u32 lane = threadIdx.x & 31;
    uint8_t* base = dsmem + (u64)(threadIdx.x >> 5) * kTraceSpaceBytes;
    WSpace w {};
    w.cols = (Col*)base;
    w.eqcol = (u64*)(base + 64 * sizeof(Col));
    w.ring = (u64*)(base + 64 * sizeof(Col) + 64 * 8);
    w.slots = (SliceSlot*)(base + 64 * sizeof(Col) + 64 * 8 + 64 * 8);
    const u64 total = write ? (*ta.candTotal < ta.candCap ? *ta.candTotal : ta.candCap) : *ta.workCount;
#pragma unroll 1
    while (true)
    {
        u32 i = 0;
        if (lane == 0) i = atomicAdd(counter, 1u);
        i = __shfl_sync(kFull, i, 0);
        if (i >= total) break;
        __syncwarp();
        ms_trace_cand(ta, ta.cands + (write ? i : ta.work[i]), w, write != 0, lane);
    }
}
}

uint64_t ga_warp_tables_bytes(const gadev::Caps& c) { return gadev::wspace_bytes(c); }
uint64_t ga_multiseed_tables_bytes(const gadev::Caps& c) { return gadev::wspace_bytes(c, true); }

static bool set_smem(const void* kernel, size_t smem)
{
    return smem <= 48 * 1024 || cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) == cudaSuccess;
}

int ga_fill_blocks_per_sm(int warpsPerBlock, const gadev::Caps& caps, bool shared)
{
    const size_t smem = shared ? (size_t)gadev::wspace_bytes(caps) * warpsPerBlock : 0;
    if (!set_smem((const void*)gadev::fill_kernel, smem)) return 0;
    int n = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, gadev::fill_kernel, warpsPerBlock * 32, smem) != cudaSuccess) return 0;
    return n;
}

int ga_trace_blocks_per_sm(int warpsPerBlock)
{
    const size_t smem = (size_t)gadev::kTraceSpaceBytes * warpsPerBlock;
    if (!set_smem((const void*)gadev::trace_kernel, smem)) return 0;
    int n = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, gadev::trace_kernel, warpsPerBlock * 32, smem) != cudaSuccess) return 0;
    return n;
}

int ga_launch_extend(const gadev::FillArgs& fa, const gadev::TraceArgs& ta, uint32_t* counters, int fillBlocks, int traceBlocks,
    int warpsPerBlock, void* stream)
{
    const size_t fillSmem = fa.workspace ? 0 : (size_t)fa.workspaceStride * warpsPerBlock;
    const size_t traceSmem = (size_t)gadev::kTraceSpaceBytes * warpsPerBlock;
    if (!set_smem((const void*)gadev::fill_kernel, fillSmem) || !set_smem((const void*)gadev::trace_kernel, traceSmem)) return -1;
    gadev::fill_kernel<<<fillBlocks, warpsPerBlock * 32, fillSmem, (cudaStream_t)stream>>>(fa, counters);
    if (cudaGetLastError() != cudaSuccess) return -1;
    gadev::trace_kernel<<<traceBlocks, warpsPerBlock * 32, traceSmem, (cudaStream_t)stream>>>(ta, counters + 1);
    return cudaGetLastError() == cudaSuccess ? 0 : -1;
}

int ga_launch_multiseed_fill(const gadev::FillArgs& fa, const gadev::MultiTraceArgs& ta, uint32_t* counters, int fillBlocks, int readBlocks,
    int warpsPerBlock, void* stream)
{
    if (!fa.workspace) return -1;
    gadev::fill_multiseed_kernel<<<fillBlocks, warpsPerBlock * 32, 0, (cudaStream_t)stream>>>(fa, counters);
    if (cudaGetLastError() != cudaSuccess) return -1;
    gadev::ms_candidates_kernel<<<readBlocks, warpsPerBlock * 32, 0, (cudaStream_t)stream>>>(ta, counters + 1, 0);
    return cudaGetLastError() == cudaSuccess ? 0 : -1;
}

int ga_launch_multiseed_list(const gadev::MultiTraceArgs& ta, uint32_t* counters, int readBlocks, int warpsPerBlock, void* stream)
{
    gadev::ms_candidates_kernel<<<readBlocks, warpsPerBlock * 32, 0, (cudaStream_t)stream>>>(ta, counters + 3, 1);
    return cudaGetLastError() == cudaSuccess ? 0 : -1;
}

int ga_launch_multiseed_keys(const gadev::MultiTraceArgs& ta, void* stream)
{
    gadev::ms_keys_kernel<<<1024, 256, 0, (cudaStream_t)stream>>>(ta);
    return cudaGetLastError() == cudaSuccess ? 0 : -1;
}

int ga_launch_multiseed_resolve(const gadev::MultiTraceArgs& ta, uint32_t* counters, int readBlocks, int warpsPerBlock, void* stream)
{
    gadev::ms_resolve_kernel<<<readBlocks, warpsPerBlock * 32, 0, (cudaStream_t)stream>>>(ta, counters + 4);
    return cudaGetLastError() == cudaSuccess ? 0 : -1;
}

int ga_launch_multiseed_walk(const gadev::MultiTraceArgs& ta, uint32_t* counters, int candBlocks, int warpsPerBlock, void* stream)
{
    const size_t traceSmem = (size_t)gadev::kTraceSpaceBytes * warpsPerBlock;
    if (!set_smem((const void*)gadev::ms_trace_kernel, traceSmem)) return -1;
    gadev::ms_trace_kernel<<<candBlocks, warpsPerBlock * 32, traceSmem, (cudaStream_t)stream>>>(ta, counters + 5, 0);
    return cudaGetLastError() == cudaSuccess ? 0 : -1;
}

int ga_launch_multiseed_write(const gadev::MultiTraceArgs& ta, uint32_t* counters, int candBlocks, int warpsPerBlock, void* stream)
{
    const size_t traceSmem = (size_t)gadev::kTraceSpaceBytes * warpsPerBlock;
    if (!set_smem((const void*)gadev::ms_trace_kernel, traceSmem)) return -1;
    gadev::ms_trace_kernel<<<candBlocks, warpsPerBlock * 32, traceSmem, (cudaStream_t)stream>>>(ta, counters + 6, 1);
    return cudaGetLastError() == cudaSuccess ? 0 : -1;
}

int ga_upload_tables()
{
    int8_t t[256];
    for (int i = 0; i < 256; i++) t[i] = (int8_t)gadev::iupac_mask((unsigned char)i);
    return cudaMemcpyToSymbol(gadev::c_iupac, t, sizeof(t)) == cudaSuccess ? 0 : -1;
}
