// Batched seed extension on GB300: fill kernel (banded Myers DP over the graph
// with the component-ordered frontier and X-drop) and traceback kernel.
//
// Work decomposition: one thread owns one extension at a time.  The DP of one
// extension is a strictly sequential chain (each 64-row slice depends on the
// previous one; inside a slice nodes are computed one at a time in frontier
// order, and the admission test uses the running minimum), so the parallelism
// is across extensions.  Both kernels are persistent: a thread takes the next
// extension from a device work counter over a longest-first order, so short
// extensions fill in behind long ones.  The fill streams every committed slice
// into a batch arena in HBM; the traceback kernel walks it back.
//
// Reference correspondence (GraphAligner src/):
//   fill_extension   getReverseTraceFromSeed / getXdropSlices  (GraphAlignerBitvectorBanded.h:59-76, 580-725)
//   fill_slice       calculateSlice                            (GraphAlignerBitvectorBanded.h:255-511)
//   node_calc<Fill>  calculateNodeInner                        (GraphAlignerBitvectorCommon.h:1113-1478)
//   trace_extension  getReverseTraceFromTableExactEndPos / getReverseTraceFromTable
//                                                              (GraphAlignerBitvectorCommon.h:496-758)
//   bt_*             pickBacktraceInside/HorizontalCrossing/VerticalCrossing/Corner (:770-1054)
#include <cuda_runtime.h>
#include <stdint.h>
#include "extend.cuh"
#include "../../include/graphaligner_gb300.h"

namespace gadev
{

struct HSlot
{
    u32 node;
    u32 gen;
    int16_t band;       // index in the slice's band, -1 until the node is first popped
    uint16_t active;    // node has a heap entry (ComponentPriorityQueue::active)
    uint16_t head;      // pending incoming edges (ComponentPriorityQueue::extras), FIFO
    uint16_t tail;
};

struct Extra
{
    u64 VP, VN;
    i32 end;
    uint16_t next;
    uint16_t skip;      // EdgeWithPriority::skipFirst
};

static constexpr uint16_t kNil = 0xffff;

__device__ __forceinline__ u32 hash_node(u32 node)
{
    u32 h = node * 0x9E3779B1u;
    return h ^ (h >> 15);
}

struct Workspace
{
    Item* band[2];
    HSlot* hash[2];
    HeapItem* heap;
    Extra* extras;
    u32* header;
};

__host__ __device__ inline u64 align16(u64 x) { return (x + 15) & ~15ULL; }

__device__ __forceinline__ Workspace workspace_at(uint8_t* base, const Caps& c)
{
    Workspace w;
    u64 off = 16;
    w.header = (u32*)base;
    w.band[0] = (Item*)(base + off); off += align16((u64)c.band * sizeof(Item));
    w.band[1] = (Item*)(base + off); off += align16((u64)c.band * sizeof(Item));
    w.hash[0] = (HSlot*)(base + off); off += align16((u64)c.hash * sizeof(HSlot));
    w.hash[1] = (HSlot*)(base + off); off += align16((u64)c.hash * sizeof(HSlot));
    w.heap = (HeapItem*)(base + off); off += align16((u64)c.heap * sizeof(HeapItem));
    w.extras = (Extra*)(base + off);
    return w;
}

// returns the slot for node in a generation-stamped table, or nullptr
__device__ __forceinline__ HSlot* hash_find(HSlot* t, u32 cap, u32 gen, u32 node)
{
    u32 h = hash_node(node) & (cap - 1);
    for (u32 probe = 0; probe < cap; probe++)
    {
        HSlot* s = &t[h];
        if (s->gen != gen) return nullptr;
        if (s->node == node) return s;
        h = (h + 1) & (cap - 1);
    }
    return nullptr;
}

__device__ __forceinline__ HSlot* hash_get_or_add(HSlot* t, u32 cap, u32 gen, u32 node, u32& used)
{
    u32 h = hash_node(node) & (cap - 1);
    for (u32 probe = 0; probe < cap; probe++)
    {
        HSlot* s = &t[h];
        if (s->gen != gen)
        {
            if (2 * (used + 1) > cap) return nullptr;
            used++;
            s->gen = gen;
            s->node = node;
            s->band = -1;
            s->active = 0;
            s->head = kNil;
            s->tail = kNil;
            return s;
        }
        if (s->node == node) return s;
        h = (h + 1) & (cap - 1);
    }
    return nullptr;
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

__device__ __forceinline__ void eq_add(EqV4& eq, int m, u32 r, bool full, bool& ok)
{
    // a non-sequence byte always fails; a gap fails only inside a full 64-row window
    ok &= !(m < 0 || (m == 0 && full));
    const u64 bit = 1ULL << r;
    eq.a |= (m & 1) ? bit : 0;
    eq.c |= (m & 2) ? bit : 0;
    eq.g |= (m & 4) ? bit : 0;
    eq.t |= (m & 8) ? bit : 0;
}

// match masks of the 64 rows starting at read position j (getEqVector, Common.h:279-318).
// When the window and 3 bytes either side lie inside the read, it is read as aligned
// 32-bit words (every word then lies inside the read); otherwise byte by byte.
__device__ __forceinline__ bool eq_vector(const uint8_t* seq, u32 len, int64_t j, EqV4& eq)
{
    eq.a = eq.c = eq.g = eq.t = 0;
    bool ok = true;
    const bool full = j + 64 <= (int64_t)len;
    if (j >= 3 && j + 64 + 3 <= (int64_t)len)
    {
        const uint8_t* p = seq + j;
        const u32 shift = (u32)((uintptr_t)p & 3) * 8;
        const u32* w = (const u32*)((uintptr_t)p & ~(uintptr_t)3);
        u32 lo = w[0];
#pragma unroll
        for (u32 k = 0; k < 16; k++)
        {
            const u32 hi = w[k + 1];
            const u32 word = __funnelshift_r(lo, hi, shift);
            lo = hi;
#pragma unroll
            for (u32 b = 0; b < 4; b++) eq_add(eq, s_iupac[(word >> (8 * b)) & 0xff], k * 4 + b, full, ok);
        }
        return ok;
    }
    const int64_t rem = (int64_t)len - j;
    const u32 n = rem >= 64 ? 64u : (rem > 0 ? (u32)rem : 0u);
    for (u32 r = 0; r < n; r++) eq_add(eq, s_iupac[seq[j + r]], r, full, ok);
    return ok;
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

// calculateNodeInner (Common.h:1113-1478) with the single-seed fake extra slice.
// Fill = true: the slice fill (early leave allowed, calculateNodeClipPrecise).
// Fill = false: recalcNodeWordslice (no early leave, every column written to cols).
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

template <bool Fill>
__device__ NodeCalc node_calc(const DevGraph& g, i32 cost, u32 i, Item& slice, const EqV4& eqv, const PrevInfo& prev,
    const Extra* pool, uint16_t head, const WS* singleIncoming, bool singleInPrevBand, i32 seqOffset, WS* cols, u64& steps, int& err,
    i32 sliceMaxX = kIntMin, u32 lastColumn = 63)
{
    // The slice keeps the first node of strictly greatest X-score and the node keeps its
    // greatest column, so a column whose bound is at most max(slice so far, node so far)
    // changes neither: its exact X-score is skipped.
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
    u64 eq0;
    if (!amb) eq0 = eq_pick(eqv, (u32)(c0 & 3));
    else eq0 = eq_amb(eqv, (u32)((a0 & 1) | ((a1 & 1) << 1) | ((a2 & 1) << 2) | ((a3 & 1) << 3)));

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
        for (uint16_t e = head; e != kNil; e = pool[e].next)
        {
            const Extra& inc = pool[e];
            WS incWs = ws_make(inc.VP, inc.VN, inc.end);
            result.cells++;
            if (inc.skip)
            {
                ws = hasWs ? ws_merge(ws, incWs) : incWs;
                hasWs = true;
                continue;
            }
            hasSkipless = true;
            i32 compareHin = prev.exists ? prev.sEnd : kIntMax;
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
            ws = hasWs ? ws_merge(ws, nw) : nw;
            hasWs = true;
        }
    }
    if (!hasWs) { err = GA_ASSERT; return result; }
    result.minScore = ws.end;
    result.minScoreNode = i;
    result.minScoreOffset = 0;
    if (Fill && (!boundOk || xscore_bound(ws, seqOffset, cost) > (int64_t)sliceMaxX))
        result.maxX = ws_max_xscore(ws, seqOffset, cost, 64, kAllOnes);
    result.maxXNode = i;
    const bool exists = (slice.node & kExists) != 0;
    if (exists)
    {
        WS s = ws_make(slice.sVP, slice.sVN, slice.sEnd);
        if (hasSkipless && g.inOff[i + 1] - g.inOff[i] == 1 && singleInPrevBand)
        {
            if (ws.end > s.end)
            {
                if (Fill) return result;
            }
            else if (ws.end < s.end)
            {
            }
            else
            {
                u64 newBigger = (ws.VP & ~s.VP) | (s.VN & ~ws.VN);
                u64 oldBigger = (s.VP & ~ws.VP) | (ws.VN & ~s.VN);
                if (newBigger > oldBigger)
                {
                }
                else if (oldBigger > newBigger)
                {
                    if (Fill) return result;
                }
                else if (newBigger == 0 && oldBigger == 0)
                {
                    if (Fill) return result;
                }
                else
                {
                    WS t = ws_merge(ws, s);
                    if (ws_eq(t, s))
                    {
                        if (Fill) return result;
                    }
                    ws = t;
                }
            }
        }
        else
        {
            WS t = ws_merge(ws, s);
            // the reference compares test.VP against the stored VN here (Common.h:1282)
            if (t.end == s.end && t.VP == s.VP && t.VP == s.VN)
            {
                if (Fill) return result;
            }
            ws = t;
        }
    }
    if (prev.exists && ws_before(ws) > prev.sEnd) ws = ws_merge(ws, ws_source(prev.sEnd));
    u64 forceMask = 0;
    u64 fixedHP = prev.HP;
    u64 fixedHN = prev.HN;
    if (prev.exists)
    {
        i32 scoreBefore = ws_before(ws);
        i32 scoreComparison = prev.sEnd;
        if (scoreBefore > scoreComparison) { err = GA_ASSERT; return result; }
        if (scoreBefore < scoreComparison)
        {
            forceMask |= 1;
            for (int off = 1; off < 64; off++)
            {
                i32 next = scoreComparison + (i32)((fixedHP >> off) & 1) - (i32)((fixedHN >> off) & 1);
                u64 mask = 1ULL << off;
                if (scoreBefore > next) { err = GA_ASSERT; return result; }
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
        }
    }
    else
    {
        forceMask = kAllOnes;
    }
    slice.sVP = ws.VP;
    slice.sVN = ws.VN;
    slice.sEnd = ws.end;
    slice.node = i | kExists;
    if (!Fill) cols[0] = ws;
    const u64 forceEq = prev.exists ? kAllOnes : (kAllOnes ^ 1);
    u64 outHP = 0, outHN = 0;
    u32 pos = 1;
    // the traceback's recomputation stops at the column it needs last
    const u32 columns = Fill ? nodeLength : (lastColumn + 1 < nodeLength ? lastColumn + 1 : nodeLength);
    for (; pos < columns; pos++)
    {
        u64 eq;
        if (!amb)
        {
            u64 chunk = pos < 32 ? c0 : c1;
            eq = eq_pick(eqv, (u32)((chunk >> ((pos & 31) * 2)) & 3));
        }
        else
        {
            eq = eq_amb(eqv, (u32)(((a0 >> pos) & 1) | (((a1 >> pos) & 1) << 1) | (((a2 >> pos) & 1) << 2) | (((a3 >> pos) & 1) << 3)));
        }
        eq &= forceEq;
        u64 Ph, Mh;
        WS nw = myers_step(eq, ws, (fixedHP >> pos) & 1, (fixedHN >> pos) & 1, Ph, Mh);
        steps++;
        if ((forceMask >> pos) & 1)
        {
            nw.VP &= kAllOnes ^ 1;
            nw.VN |= 1;
        }
        ws = nw;
        if (ws.end < result.minScore)
        {
            result.minScore = ws.end;
            result.minScoreOffset = pos;
        }
        if (Fill && (!boundOk || xscore_bound(ws, seqOffset, cost) > (int64_t)imax(sliceMaxX, result.maxX)))
            result.maxX = imax(result.maxX, ws_max_xscore(ws, seqOffset, cost, 64, Mh));
        if (!Fill) cols[pos] = ws;
        outHP |= (Ph >> 63) << pos;
        outHN |= (Mh >> 63) << pos;
    }
    result.cells = pos;
    slice.HP = outHP;
    slice.HN = outHN;
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
};

__device__ __forceinline__ bool arena_alloc(const FillArgs& a, ArenaCursor& c, u64 bytes, u64& out)
{
    bytes = align16(bytes);
    if (c.pos + bytes > c.end)
    {
        const u64 chunk = 16 * 1024;
        u64 grab = bytes > chunk ? bytes : chunk;
        u64 p = atomicAdd(a.arenaCursor, (unsigned long long)grab);
        if (p + grab > a.arenaBytes) return false;
        c.pos = p;
        c.end = p + grab;
    }
    out = c.pos;
    c.pos += bytes;
    return true;
}

__device__ __forceinline__ u32 rec_hash_cap(u32 count)
{
    if (count <= kInlineIds) return 0;
    u32 cap = 4;
    while (cap < 2 * count) cap <<= 1;
    return cap;
}

__device__ __forceinline__ u64 rec_bytes(u32 count, u32 cap)
{
    return sizeof(SliceRec) + (u64)count * sizeof(Item) + (u64)cap * sizeof(uint16_t);
}

// write one slice (record + band in first-pop order + node hash) into the arena
__device__ bool commit_slice(const FillArgs& a, ArenaCursor& c, u64* dir, u32 index, const Item* band, u32 count,
    i32 minScore, i32 quit, i32 maxX, u32 maxXNode, bool notValid)
{
    u32 cap = rec_hash_cap(count);
    u64 off;
    if (!arena_alloc(a, c, rec_bytes(count, cap), off)) return false;
    uint8_t* base = a.arena + off;
    SliceRec* r = (SliceRec*)base;
    r->minScore = minScore;
    r->quit = quit;
    r->maxX = maxX;
    r->maxXNode = maxXNode;
    r->count = count;
    r->hashCap = cap;
    r->notValid = notValid ? 1u : 0u;
    r->pad = 0;
    for (u32 k = 0; k < kInlineIds; k++) r->ids[k] = k < count ? (band[k].node & kNodeMask) : 0xffffffffu;
    Item* items = (Item*)(base + sizeof(SliceRec));
    uint16_t* h = (uint16_t*)(base + sizeof(SliceRec) + (u64)count * sizeof(Item));
    for (u32 k = 0; k < count; k++) items[k] = band[k];
    if (cap > 0)
    {
        for (u32 k = 0; k < cap; k++) h[k] = 0;
        for (u32 k = 0; k < count; k++)
        {
            u32 node = band[k].node & kNodeMask;
            u32 p = hash_node(node) & (cap - 1);
            while (h[p] != 0) p = (p + 1) & (cap - 1);
            h[p] = (uint16_t)(k + 1);
        }
    }
    dir[index] = off;
    return true;
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

// calculateSlice (GraphAlignerBitvectorBanded.h:255-511), component-queue branch, no seed hits.
__device__ SliceResult fill_slice(const FillArgs& a, const Workspace& w, int cur, u32 curGen, u32 prevGen, u32& curCount, u32 prevCount,
    const uint8_t* seq, u32 seqLen, int64_t j, i32 prevQuit, i32 prevMin, u64& steps, int& err)
{
    const DevGraph& g = a.g;
    const int bw = (int)a.bandwidth;
    const int prv = cur ^ 1;
    Item* curBand = w.band[cur];
    const Item* prevBand = w.band[prv];
    HSlot* curHash = w.hash[cur];
    HSlot* prevHash = w.hash[prv];
    const u32 hcap = a.caps.hash;
    SliceResult res;
    res.minScore = kIntMax - bw - 1;
    res.minScoreNode = 0xffffffffu;
    res.maxX = kIntMin;
    res.maxXNode = 0;
    res.cells = 0;
    EqV4 eqv;
    if (!eq_vector(seq, seqLen, j, eqv)) { err = GA_ASSERT; return res; }
    u32 heapN = 0;
    u32 poolN = 0;
    u32 hashUsed = 0;
    curCount = 0;

    auto insert = [&](u32 target, i32 score, u64 vp, u64 vn, i32 end, bool skip) -> bool
    {
        HSlot* s = hash_get_or_add(curHash, hcap, curGen, target, hashUsed);
        if (!s) return false;
        if (!s->active)
        {
            if (heapN >= a.caps.heap) return false;
            HeapItem hi; hi.component = g.comp[target]; hi.score = score; hi.node = target;
            heap_push(w.heap, heapN, hi);
            s->active = 1;
            s->head = kNil;
            s->tail = kNil;
        }
        if (poolN >= a.caps.extras) return false;
        uint16_t e = (uint16_t)poolN++;
        Extra& x = w.extras[e];
        x.VP = vp; x.VN = vn; x.end = end; x.next = kNil; x.skip = skip ? 1 : 0;
        if (s->head == kNil) s->head = e;
        else w.extras[s->tail].next = e;
        s->tail = e;
        return true;
    };

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
                u32 nb = g.inNb[g.inOff[node]];
                HSlot* ps = hash_find(prevHash, hcap, prevGen, nb);
                if (ps && ps->band >= 0)
                {
                    const Item& pn = prevBand[ps->band];
                    if (pn.eEnd < prevQuit && pn.minScore < prevQuit) continue;
                }
            }
        }
        WS src = ws_source(it.sEnd);
        if (!insert(node, it.minScore, src.VP, src.VN, src.end, true)) { err = GA_CAPACITY; return res; }
    }
    if (heapN == 0) { err = GA_ASSERT; return res; }
    i32 curMin = res.minScore;
    const i32 seqOffset = (i32)j;
    while (heapN > 0)
    {
        u32 i = w.heap[0].node;
        HSlot* s = hash_find(curHash, hcap, curGen, i);
        if (!s) { err = GA_ASSERT; return res; }
        if (s->band < 0)
        {
            if (curCount >= a.caps.band || curCount >= 32767) { err = GA_CAPACITY; return res; }
            s->band = (int16_t)curCount;
            Item& ni = curBand[curCount++];
            ni.sVP = 0; ni.sVN = 0; ni.sEnd = kIntMax;
            ni.eVP = 0; ni.eVN = 0; ni.eEnd = kIntMax;
            ni.HP = 0; ni.HN = 0;
            ni.minScore = kIntMax;
            ni.node = i;
        }
        Item& thisNode = curBand[s->band];
        WS oldEnd = (thisNode.node & kExists) ? ws_make(thisNode.eVP, thisNode.eVN, thisNode.eEnd) : ws_make(0, 0, kIntMax);
        PrevInfo prev;
        HSlot* ps = hash_find(prevHash, hcap, prevGen, i);
        if (ps && ps->band >= 0)
        {
            const Item& pi = prevBand[ps->band];
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
        if (g.inOff[i + 1] - g.inOff[i] == 1)
        {
            HSlot* q = hash_find(prevHash, hcap, prevGen, g.inNb[g.inOff[i]]);
            singleInPrev = q && q->band >= 0;
        }
        NodeCalc nc = node_calc<true>(g, a.cost, i, thisNode, eqv, prev, w.extras, s->head, nullptr, singleInPrev, seqOffset, nullptr, steps, err, res.maxX);
        if (err) return res;
        heap_pop(w.heap, heapN);
        s->active = 0;
        s->head = kNil;
        s->tail = kNil;
        if (nc.minScore > wadd(wadd(seqOffset, bw), 128)) { err = GA_ASSERT; return res; }
        curMin = imin(curMin, nc.minScore);
        if (nc.minScore < thisNode.minScore) thisNode.minScore = nc.minScore;
        WS newEnd = ws_make(thisNode.eVP, thisNode.eVN, thisNode.eEnd);
        if (!ws_eq(newEnd, oldEnd))
        {
            i32 newEndMin = ws_changed_min(newEnd, oldEnd);
            if (newEndMin == kIntMax) { err = GA_ASSERT; return res; }
            if (newEndMin <= wadd(curMin, bw))
            {
                for (u32 e = g.outOff[i]; e < g.outOff[i + 1]; e++)
                {
                    if (!insert(g.outNb[e], newEndMin, newEnd.VP, newEnd.VN, newEnd.end, false)) { err = GA_CAPACITY; return res; }
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
    if (res.minScoreNode == 0xffffffffu) err = GA_ASSERT;
    return res;
}

__device__ ExtState fill_extension(const FillArgs& a, const Workspace& w, u32& gen, ArenaCursor& arena, u32 ext)
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
    if (!arena_alloc(a, arena, (u64)(numSlices + 1) * 8, dirOff))
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
        Item& it = w.band[prv][0];
        u32 L = g.len[startNode];
        it.sVP = 0; it.sVN = 0; it.sEnd = (i32)startOff;
        it.eVP = 0; it.eVN = 0; it.eEnd = (i32)L - 1 - (i32)startOff;
        it.minScore = 0;
        it.node = startNode | kExists;
        u64 hn = 0, hp = 0;
        for (u32 k = 1; k <= startOff; k++) hn |= 1ULL << k;
        for (u32 k = startOff + 1; k < L; k++) hp |= 1ULL << k;
        it.HP = hp;
        it.HN = hn;
        u32 used = 0;
        HSlot* s = hash_get_or_add(w.hash[prv], a.caps.hash, prevGen, startNode, used);
        s->band = 0;
        if (!commit_slice(a, arena, dir, 0, &it, 1, 0, 1, 0, startNode, false))
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
    for (u32 s = 0; s < numSlices; s++)
    {
        const int cur = prv ^ 1;
        gen++;
        const u32 curGen = gen;
        u32 curCount = 0;
        const int64_t j = (int64_t)s * 64;
        SliceResult r = fill_slice(a, w, cur, curGen, prevGen, curCount, prevCount, seq, seqLen, j, lastQuit, lastMin, st.steps, err);
        if (err) break;
        if (r.maxX > bestX) bestX = r.maxX;
        const bool notValid = r.cells >= a.maxCells;
        if ((int64_t)r.maxX < (int64_t)bestX - (int64_t)a.xdrop) break;
        if (r.minScore < lastMin) { err = GA_ASSERT; break; }
        const i32 quit = wadd(r.minScore, (i32)a.bandwidth);
        if (!commit_slice(a, arena, dir, committed, w.band[cur], curCount, r.minScore, quit, r.maxX, r.maxXNode, notValid))
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

// ---------------------------------------------------------------- traceback

struct Table
{
    const uint8_t* arena;
    const u64* dir;
    u32 count;
    // the traceback works on one slice and the one before it: their records are remembered
    u32 cs[2];
    const SliceRec* cr[2];
    __device__ __forceinline__ void init() { cs[0] = cs[1] = 0xffffffffu; cr[0] = cr[1] = nullptr; }
    __device__ __forceinline__ const SliceRec* rec(u32 s)
    {
        if (cs[0] == s) return cr[0];
        if (cs[1] == s) return cr[1];
        const SliceRec* r = (const SliceRec*)(arena + dir[s]);
        cs[1] = cs[0]; cr[1] = cr[0];
        cs[0] = s; cr[0] = r;
        return r;
    }
    __device__ __forceinline__ const Item* items(u32 s) { return (const Item*)((const uint8_t*)rec(s) + sizeof(SliceRec)); }
    __device__ __forceinline__ const Item* find(u32 s, u32 node)
    {
        const SliceRec* r = rec(s);
        const Item* it = (const Item*)((const uint8_t*)r + sizeof(SliceRec));
        const u32 count = r->count;
        if (count <= kInlineIds)
        {
            // the record's own line holds the band's node ids
            for (u32 k = 0; k < count; k++)
                if (r->ids[k] == node) return &it[k];
            return nullptr;
        }
        const uint16_t* h = (const uint16_t*)((const uint8_t*)it + (u64)count * sizeof(Item));
        u32 cap = r->hashCap;
        u32 p = hash_node(node) & (cap - 1);
        for (u32 probe = 0; probe < cap; probe++)
        {
            uint16_t v = h[p];
            if (v == 0) return nullptr;
            if ((it[v - 1].node & kNodeMask) == node) return &it[v - 1];
            p = (p + 1) & (cap - 1);
        }
        return nullptr;
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

struct TraceOut
{
    u64* items;
    u32 cap;
    u32 n;
    TPos back;
    bool overflow;
    __device__ __forceinline__ void push(const TPos& p, bool sw)
    {
        if (n >= cap) { overflow = true; return; }
        u64 sp1 = p.seq < 0 ? 0 : (u64)p.seq + 1;
        items[n++] = (u64)p.node | ((u64)(p.off & 63) << 32) | ((u64)(sw ? 1 : 0) << 38) | (sp1 << 39);
        back = p;
    }
};

__device__ __forceinline__ u32 mod64(int64_t seq) { return (u32)((u64)seq & 63); }

// checkBacktraceCircularity (Common.h:760-768): the newest item must not repeat an
// earlier item of the same read position
__device__ __forceinline__ bool trace_circular(const TraceOut& to)
{
    if (to.n < 2) return false;
    const u64 keyMask = ~(1ULL << 38);
    u64 last = to.items[to.n - 1];
    for (int k = (int)to.n - 2; k >= 0; k--)
    {
        u64 x = to.items[k];
        if ((x & keyMask) == (last & keyMask)) return true;
        if ((x >> 39) != (last >> 39)) return false;
    }
    return false;
}

struct TraceCtx
{
    const DevGraph* g;
    const uint8_t* seq;
    u32 seqLen;
    Table t;
    i32 cost;
    int err;
};

__device__ __forceinline__ i32 fake_value() { return kIntMax; }

// pickBacktraceCorner (Common.h:936-1054)
__device__ TStep bt_corner(TraceCtx& c, u32 cs, u32 node, int64_t j)
{
    const DevGraph& g = *c.g;
    const SliceRec* cr = c.t.rec(cs);
    const SliceRec* pr = c.t.rec(cs - 1);
    const Item* self = c.t.find(cs, node);
    TStep out; out.pos.node = 0; out.pos.off = 0; out.pos.seq = 0; out.sw = false;
    if (!self) { c.err = GA_ASSERT; return out; }
    i32 scoreHere = ws_value(ws_make(self->sVP, self->sVN, self->sEnd), 0);
    const Item* prevSelf = c.t.find(cs - 1, node);
    if (cr->notValid || scoreHere > cr->quit)
    {
        if (scoreHere == fake_value()) { out.pos = TPos { node, 0, j }; return out; }
        i32 smallest = scoreHere + 1;
        TPos sp = TPos { 0xffffffffu, 0xffffffffu, -2 };
        bool change = false;
        if (prevSelf)
        {
            smallest = prevSelf->sEnd;
            sp = TPos { node, 0, j - 1 };
            change = false;
        }
        for (u32 e = g.inOff[node]; e < g.inOff[node + 1]; e++)
        {
            u32 nb = g.inNb[e];
            const Item* pn = c.t.find(cs - 1, nb);
            if (pn && pn->eEnd <= smallest)
            {
                smallest = pn->eEnd;
                sp = TPos { nb, g.len[nb] - 1, j - 1 };
                change = true;
            }
            const Item* cn = c.t.find(cs, nb);
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
        if (sp.node == 0xffffffffu) { c.err = GA_ASSERT; return out; }
        out.pos = sp; out.sw = change;
        return out;
    }
    bool bad = false;
    bool eq = char_match(g, c.seq[j], node, 0, bad);
    if (bad) { c.err = GA_ASSERT; return out; }
    TPos bestInvalid = TPos { 0xffffffffu, 0xffffffffu, -2 };
    i32 bestInvalidScore = scoreHere + 1;
    bool bestInvalidSw = false;
    if (prevSelf)
    {
        i32 ps = prevSelf->sEnd;
        if (ps < scoreHere - 1) { c.err = GA_ASSERT; return out; }
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
    for (u32 e = g.inOff[node]; e < g.inOff[node + 1]; e++)
    {
        u32 nb = g.inNb[e];
        const Item* cn = c.t.find(cs, nb);
        if (cn)
        {
            i32 v = ws_value(ws_make(cn->eVP, cn->eVN, cn->eEnd), 0);
            if (v < scoreHere - 1) { c.err = GA_ASSERT; return out; }
            if (v == scoreHere - 1) { out.pos = TPos { nb, g.len[nb] - 1, j }; out.sw = true; return out; }
        }
        const Item* pn = c.t.find(cs - 1, nb);
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
                if (corner < scoreHere - (eq ? 0 : 1)) { c.err = GA_ASSERT; return out; }
                if (corner == scoreHere - (eq ? 0 : 1)) { out.pos = TPos { nb, g.len[nb] - 1, j - 1 }; out.sw = true; return out; }
            }
        }
    }
    if (eq && scoreHere == fake_value()) { out.pos = TPos { node, 0, j }; return out; }
    if (scoreHere == fake_value()) { out.pos = TPos { node, 0, j }; return out; }
    if (bestInvalidScore < scoreHere + 1) { out.pos = bestInvalid; out.sw = bestInvalidSw; return out; }
    c.err = GA_ASSERT;
    return out;
}

// recalcNodeWordslice (Common.h:1078-1102): the columns 0..lastColumn of one node-slice
// (the traceback only moves left inside a node, so it never needs the columns after the
// one it enters at).  When every column is recomputed the last one must equal the
// stored end column, as the reference asserts.
__device__ bool recalc(TraceCtx& c, u32 s, u32 node, const EqV4& eqv, WS* cols, u32 lastColumn = 63)
{
    const Item* it = c.t.find(s, node);
    if (!it) { c.err = GA_ASSERT; return false; }
    PrevInfo prev;
    const Item* pi = c.t.find(s - 1, node);
    if (pi) { prev.exists = true; prev.sEnd = pi->sEnd; prev.HP = pi->HP; prev.HN = pi->HN; }
    else { prev.exists = false; prev.sEnd = 0; prev.HP = kAllOnes; prev.HN = 0; }
    Item copy = *it;
    WS start = ws_make(it->sVP, it->sVN, it->sEnd);
    u64 steps = 0;
    int err = 0;
    int64_t j = ((int64_t)s - 1) * 64;
    node_calc<false>(*c.g, c.cost, node, copy, eqv, prev, nullptr, kNil, &start, false, (i32)j, cols, steps, err, kIntMin, lastColumn);
    if (err) { c.err = err; return false; }
    u32 L = c.g->len[node];
    if (!ws_eq(cols[0], start)) { c.err = GA_ASSERT; return false; }
    if (lastColumn + 1 >= L && !ws_eq(cols[L - 1], ws_make(it->eVP, it->eVN, it->eEnd))) { c.err = GA_ASSERT; return false; }
    return true;
}

__device__ void trace_extension(const TraceArgs& a, u32 ext, const ExtState& st, WS* cols)
{
    const DevGraph& g = a.g;
    u64* out = a.traceItems + a.traceOffset[ext];
    const u32 cap = a.traceCap[ext];
    if (a.cellSteps) a.cellSteps[ext] = st.steps;
    if (st.status != GA_OK)
    {
        a.status[ext] = st.status;
        a.score[ext] = 0;
        a.traceLen[ext] = 0;
        return;
    }
    TraceCtx c;
    c.g = &g;
    c.seq = a.seq + a.seqOff[ext];
    c.seqLen = a.seqLen[ext];
    c.t.arena = a.arena;
    c.t.dir = (const u64*)(a.arena + st.dir);
    c.t.count = st.committed;
    c.t.init();
    c.cost = a.cost;
    c.err = 0;
    TraceOut to;
    to.items = out;
    to.cap = cap;
    to.n = 0;
    to.overflow = false;
    // choose the end cell (getReverseTraceFromTableExactEndPos, Common.h:496-562)
    u32 best = 1;
    for (u32 s = 1; s < st.committed; s++)
        if (c.t.rec(s)->maxX > c.t.rec(best)->maxX) best = s;
    const SliceRec* br = c.t.rec(best);
    u32 node = br->maxXNode;
    i32 score = br->maxX;
    int64_t j = ((int64_t)best - 1) * 64;
    EqV4 eqv;
    if (!eq_vector(c.seq, c.seqLen, j, eqv)) c.err = GA_ASSERT;
    u32 nodeOffset = 0xffffffffu, bvOffset = 0xffffffffu;
    if (!c.err && recalc(c, best, node, eqv, cols))
    {
        int cells = (int)((int64_t)c.seqLen - j < 64 ? (int64_t)c.seqLen - j : 64);
        u32 L = g.len[node];
        for (u32 i = 0; i < L && !c.err; i++)
        {
            i32 mx = ws_max_xscore(cols[i], (i32)j, a.cost, cells, kAllOnes);
            if (mx > score) { c.err = GA_ASSERT; break; }
            if (mx == score)
            {
                for (int off = 63; off >= 0; off--)
                {
                    if (j + off >= (int64_t)c.seqLen) continue;
                    i32 here = ws_xscore(cols[i], (i32)j, off, a.cost);
                    if (here > score) { c.err = GA_ASSERT; break; }
                    if (here == score && (nodeOffset == 0xffffffffu || (u32)off > bvOffset))
                    {
                        nodeOffset = i;
                        bvOffset = (u32)off;
                    }
                }
            }
        }
    }
    if (!c.err && (nodeOffset == 0xffffffffu || j + bvOffset >= (int64_t)c.seqLen)) c.err = GA_ASSERT;
    i32 resultScore = 0;
    if (!c.err)
    {
        // getReverseTraceFromTable (Common.h:571-758)
        TPos start = TPos { node, nodeOffset, j + bvOffset };
        i32 startScore = ws_value(cols[nodeOffset], (int)bvOffset);
        resultScore = startScore;
        to.push(start, false);
        u32 curSlice = (u32)(start.seq / 64) + 1;
        u32 curNode = 0xffffffffu;
        u32 colsUpTo = 0;             // columns 0..colsUpTo of (curSlice, curNode) are in cols
        if (!eq_vector(c.seq, c.seqLen, ((int64_t)curSlice - 1) * 64, eqv)) c.err = GA_ASSERT;
        i32 lastScore = kIntMax - 1;
        u64 guard = 0;
        const u64 guardMax = (u64)cap * 4 + 1024;
        while (!c.err && !to.overflow && to.back.seq != -1)
        {
            if (++guard > guardMax) { c.err = GA_CAPACITY; break; }
            TPos b = to.back;
            u32 newSlice = (u32)(b.seq / 64) + 1;
            if (newSlice >= st.committed) { c.err = GA_ASSERT; break; }
            // a self-loop can re-enter the same node-slice further right than it was computed
            if (newSlice != curSlice || b.node != curNode || b.off > colsUpTo)
            {
                if (newSlice != curSlice && !eq_vector(c.seq, c.seqLen, ((int64_t)newSlice - 1) * 64, eqv)) { c.err = GA_ASSERT; break; }
                curSlice = newSlice;
                curNode = b.node;
                if (curSlice == 0) { c.err = GA_ASSERT; break; }
                if (!recalc(c, curSlice, curNode, eqv, cols, b.off)) break;
                colsUpTo = b.off;
            }
            const int64_t sj = ((int64_t)curSlice - 1) * 64;
            if (b.off >= g.len[curNode]) { c.err = GA_ASSERT; break; }
            const u32 row = mod64(b.seq);
            lastScore = ws_value(cols[b.off], (int)row);
            if (row == 0 && b.off == 0)
            {
                TStep bt = bt_corner(c, curSlice, curNode, sj);
                if (c.err) break;
                if (tpos_eq(bt.pos, b) && !bt.sw && ws_value(cols[bt.pos.off], (int)mod64(bt.pos.seq)) == fake_value()) break;
                to.push(bt.pos, bt.sw);
                if (!to.overflow && trace_circular(to)) { c.err = GA_ASSERT; break; }
                continue;
            }
            if (row == 0)
            {
                const Item* pself = c.t.find(curSlice - 1, curNode);
                if (!pself)
                {
                    for (u32 k = b.off - 1; k > 0; k--) to.push(TPos { curNode, k, b.seq }, false);
                    to.push(TPos { curNode, 0, b.seq }, false);
                    continue;
                }
                // pickBacktraceVerticalCrossing (Common.h:886-934)
                TPos p = b;
                while (p.off > 0 && ws_value(cols[p.off - 1], 0) == ws_value(cols[p.off], 0) - 1) p.off--;
                TStep second;
                if (p.off == 0)
                {
                    second = bt_corner(c, curSlice, curNode, sj);
                    if (c.err) break;
                }
                else
                {
                    const SliceRec* cr = c.t.rec(curSlice);
                    const SliceRec* pr = c.t.rec(curSlice - 1);
                    bool bad = false;
                    bool eq = char_match(g, c.seq[p.seq], p.node, p.off, bad);
                    if (bad) { c.err = GA_ASSERT; break; }
                    i32 here = ws_value(cols[p.off], 0);
                    i32 diag = pself->sEnd;
                    for (u32 k = 1; k + 1 <= p.off; k++)
                    {
                        diag += (i32)((pself->HP >> k) & 1);
                        diag -= (i32)((pself->HN >> k) & 1);
                    }
                    i32 up = diag + (i32)((pself->HP >> p.off) & 1) - (i32)((pself->HN >> p.off) & 1);
                    if (pr->notValid || cr->notValid || here > cr->quit || diag > pr->quit || up > pr->quit)
                    {
                        if (here == fake_value()) second = TStep { p, false };
                        else if (diag < up) second = TStep { TPos { p.node, p.off - 1, p.seq - 1 }, false };
                        else second = TStep { TPos { p.node, p.off, p.seq - 1 }, false };
                    }
                    else
                    {
                        if (up < here - 1 || diag < here - (eq ? 0 : 1)) { c.err = GA_ASSERT; break; }
                        if (up == here - 1) second = TStep { TPos { p.node, p.off, p.seq - 1 }, false };
                        else if (diag == here - (eq ? 0 : 1)) second = TStep { TPos { p.node, p.off - 1, p.seq - 1 }, false };
                        else { c.err = GA_ASSERT; break; }
                    }
                }
                if (second.pos.seq == b.seq && ws_value(cols[second.pos.off], (int)mod64(second.pos.seq)) == fake_value()) break;
                if (p.off != b.off)
                {
                    for (u32 k = b.off - 1; k != p.off; k--) to.push(TPos { p.node, k, p.seq }, false);
                }
                if (!tpos_eq(p, to.back)) to.push(p, false);
                if (tpos_eq(second.pos, to.back)) { c.err = GA_ASSERT; break; }
                to.push(second.pos, second.sw);
                continue;
            }
            if (b.off == 0)
            {
                // pickBacktraceHorizontalCrossing (Common.h:817-884)
                const Item* self = c.t.find(curSlice, curNode);
                if (!self) { c.err = GA_ASSERT; break; }
                TPos p = b;
                while (mod64(p.seq) != 0 && (self->sVP & (1ULL << mod64(p.seq)))) p.seq--;
                const u32 off = mod64(p.seq);
                TStep second;
                if (off == 0)
                {
                    second = bt_corner(c, curSlice, curNode, sj);
                    if (c.err) break;
                }
                else
                {
                    const SliceRec* cr = c.t.rec(curSlice);
                    bool bad = false;
                    bool eq = char_match(g, c.seq[p.seq], p.node, p.off, bad);
                    if (bad) { c.err = GA_ASSERT; break; }
                    WS sws = ws_make(self->sVP, self->sVN, self->sEnd);
                    i32 here = ws_value(sws, (int)off);
                    if (cr->notValid || here > cr->quit)
                    {
                        i32 smallest = ws_value(sws, (int)off - 1);
                        TPos sp = TPos { curNode, 0, p.seq - 1 };
                        bool change = false;
                        for (u32 e = g.inOff[curNode]; e < g.inOff[curNode + 1]; e++)
                        {
                            u32 nb = g.inNb[e];
                            const Item* cn = c.t.find(curSlice, nb);
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
                        if (tpos_eq(sp, p) && here != fake_value()) { c.err = GA_ASSERT; break; }
                        second = TStep { sp, change };
                    }
                    else
                    {
                        bool found = false;
                        for (u32 e = g.inOff[curNode]; e < g.inOff[curNode + 1] && !found; e++)
                        {
                            u32 nb = g.inNb[e];
                            const Item* cn = c.t.find(curSlice, nb);
                            if (!cn) continue;
                            WS nws = ws_make(cn->eVP, cn->eVN, cn->eEnd);
                            i32 v0 = ws_value(nws, (int)off);
                            i32 v1 = ws_value(nws, (int)off - 1);
                            if (v0 < here - 1 || v1 < here - (eq ? 0 : 1)) { c.err = GA_ASSERT; break; }
                            if (v0 == here - 1) { second = TStep { TPos { nb, g.len[nb] - 1, p.seq }, true }; found = true; }
                            else if (v1 == here - (eq ? 0 : 1)) { second = TStep { TPos { nb, g.len[nb] - 1, p.seq - 1 }, true }; found = true; }
                        }
                        if (c.err) break;
                        if (!found)
                        {
                            if (here != fake_value()) { c.err = GA_ASSERT; break; }
                            second = TStep { p, false };
                        }
                    }
                }
                if (second.pos.node == b.node && !second.sw && ws_value(cols[second.pos.off], (int)mod64(second.pos.seq)) == fake_value()) break;
                if (p.seq != b.seq)
                {
                    for (int64_t sp = b.seq - 1; sp != p.seq; sp--) to.push(TPos { p.node, p.off, sp }, false);
                }
                if (!tpos_eq(p, to.back)) to.push(p, false);
                if (tpos_eq(second.pos, to.back)) { c.err = GA_ASSERT; break; }
                to.push(second.pos, second.sw);
                if (!to.overflow && trace_circular(to)) { c.err = GA_ASSERT; break; }
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
                const bool amb = b.node >= g.firstAmbiguous;
                const u64 nc0 = amb ? 0 : g.seq2[(u64)b.node * 2];
                const u64 nc1 = amb ? 0 : g.seq2[(u64)b.node * 2 + 1];
                auto colEq = [&](u32 h) -> u64
                {
                    if (!amb) return eq_pick(eqv, (u32)(((h < 32 ? nc0 : nc1) >> ((h & 31) * 2)) & 3));
                    return eq_amb(eqv, (u32)node_char_mask(g, b.node, h));
                };
                if (hori > 0 && vert > 0)
                {
                    WS colH = cols[hori];
                    WS colL = cols[hori - 1];
                    i32 here = ws_value(colH, (int)vert);
                    i32 left = ws_value(colL, (int)vert);
                    u64 eqH = colEq(hori);
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
                                colL = cols[hori - 1];
                                left = ws_value(colL, (int)vert);
                                eqH = colEq(hori);
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
                                colL = cols[hori - 1];
                                left = ws_value(colL, (int)vert);
                                eqH = colEq(hori);
                            }
                        }
                        else
                        {
                            if (here != fake_value()) c.err = GA_ASSERT;
                            break;
                        }
                        if (to.overflow || hori == 0 || vert == 0) break;
                    }
                }
                if (c.err || to.overflow) break;
                if (ws_value(cols[to.back.off], (int)mod64(to.back.seq)) == fake_value()) break;
            }
        }
        if (!c.err && !to.overflow)
        {
            if (resultScore < lastScore) c.err = GA_ASSERT;
            resultScore -= lastScore;
        }
        // the start node's row above the read (Common.h:721-756)
        if (!c.err && !to.overflow)
        {
            if (to.back.seq != -1) c.err = GA_ASSERT;
            const Item* it = c.err ? nullptr : c.t.find(0, to.back.node);
            if (!c.err && !it) c.err = GA_ASSERT;
            if (!c.err)
            {
                const u32 L = g.len[to.back.node];
                // before[k] = score of column k in the row above the read
                auto before = [&](u32 k) -> i32
                {
                    i32 v = it->sEnd;
                    for (u32 q = 1; q <= k; q++) v += (i32)((it->HP >> q) & 1) - (i32)((it->HN >> q) & 1);
                    return v;
                };
                if (before(L - 1) != it->eEnd) c.err = GA_ASSERT;
                while (!c.err && !to.overflow)
                {
                    TPos q = to.back;
                    i32 bq = before(q.off);
                    if (!(bq != 0 && q.off > 0 && before(q.off - 1) == bq - 1)) break;
                    to.push(TPos { q.node, q.off - 1, q.seq }, false);
                }
                TPos q = to.back;
                if (!c.err && !to.overflow && q.off == 0 && before(0) != 0)
                {
                    for (u32 e = g.inOff[q.node]; e < g.inOff[q.node + 1]; e++)
                    {
                        u32 nb = g.inNb[e];
                        const Item* ni = c.t.find(0, nb);
                        if (ni && ws_before(ws_make(ni->eVP, ni->eVN, ni->eEnd)) == before(0) - 1)
                        {
                            to.push(TPos { nb, g.len[nb] - 1, q.seq }, true);
                            break;
                        }
                    }
                }
            }
        }
    }
    int status = c.err ? c.err : (to.overflow ? GA_CAPACITY : GA_OK);
    a.status[ext] = status;
    a.score[ext] = status == GA_OK ? resultScore : 0;
    a.traceLen[ext] = status == GA_OK ? to.n : 0;
}

// One persistent kernel per batch: a thread fills the DP table of an extension
// and walks it back right away.  Warps take chunks of the longest-first order from
// a chunk table the host builds (ga_launch_shape): a chunk is up to 32 consecutive
// extensions, one per lane, so the lanes of a warp hold extensions of similar
// length.  The longest extensions come in chunks of one (lane 0 alone), which keeps
// them free of divergence with other lanes; the chunk sizes trade divergence within
// a warp against the number of extensions in flight.
__global__ void __launch_bounds__(128) extend_kernel(FillArgs fa, TraceArgs ta, const u32* chunks, u32 numChunks,
    u32* counter, u32 slotBase, u32 slotLimit)
{
    load_iupac_table();
    const u32 slot = slotBase + blockIdx.x * blockDim.x + threadIdx.x;
    // a warp whose slots are not all inside [slotBase, slotLimit) touches no workspace (warp-uniform)
    if (slotBase + blockIdx.x * blockDim.x + (threadIdx.x & ~31u) + 32 > slotLimit) return;
    Workspace w = workspace_at(fa.workspace + (u64)slot * fa.workspaceStride, fa.caps);
    u32 gen = w.header[0];
    ArenaCursor arena;
    arena.pos = 0;
    arena.end = 0;
    WS cols[64];
    const u32 lane = threadIdx.x & 31;
    while (true)
    {
        u32 ci = 0;
        if (lane == 0) ci = atomicAdd(counter, 1u);
        ci = __shfl_sync(0xffffffffu, ci, 0);
        if (ci >= numChunks) break;
        // chunk = first position in the order (high 26 bits) and size - 1 (low 6 bits)
        const u32 chunk = chunks[ci];
        if (lane <= (chunk & 63u))
        {
            const u32 ext = fa.order[(chunk >> 6) + lane];
            if (!fa.prevStatus || fa.prevStatus[ext] == GA_CAPACITY)
            {
                ExtState st = fill_extension(fa, w, gen, arena, ext);
                trace_extension(ta, ext, st, cols);
                if (gen > 0xF0000000u)
                {
                    // generation stamps are about to wrap: clear this thread's tables
                    for (u32 t = 0; t < 2; t++)
                        for (u32 k2 = 0; k2 < fa.caps.hash; k2++) w.hash[t][k2].gen = 0;
                    gen = 0;
                }
            }
        }
    }
    w.header[0] = gen;
}

}

void ga_launch_extend(const gadev::FillArgs& fa, const gadev::TraceArgs& ta, const uint32_t* chunks, uint32_t numChunks,
    uint32_t* counter, uint32_t slotBase, uint32_t slotLimit, int grid, int block, void* stream)
{
    gadev::extend_kernel<<<grid, block, 0, (cudaStream_t)stream>>>(fa, ta, chunks, numChunks, counter, slotBase, slotLimit);
}

int ga_upload_tables()
{
    int8_t t[256];
    for (int i = 0; i < 256; i++) t[i] = (int8_t)gadev::iupac_mask((unsigned char)i);
    return cudaMemcpyToSymbol(gadev::c_iupac, t, sizeof(t)) == cudaSuccess ? 0 : -1;
}

int ga_extend_occupancy(int block)
{
    int n = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, gadev::extend_kernel, block, 0);
    return n;
}

uint64_t ga_workspace_bytes(const gadev::Caps& c)
{
    using namespace gadev;
    u64 b = 16;
    b += 2 * align16((u64)c.band * sizeof(Item));
    b += 2 * align16((u64)c.hash * sizeof(HSlot));
    b += align16((u64)c.heap * sizeof(HeapItem));
    b += align16((u64)c.extras * sizeof(Extra));
    return align16(b);
}

// ---------------------------------------------------------------- no-allocation entry point
//
// ga_extend_batch_noalloc serves callers that cannot call cudaMalloc when they
// extend: processes whose device memory is handed out by another allocator
// under a fixed budget (a framework's caching pool owns the GPU), and request
// paths where the device-wide synchronisation of cudaMalloc/cudaFree is not
// acceptable.  All of its scratch memory — the per-thread frontier tables and
// the DP-table arena the fill writes and the traceback reads — lives in the
// file-scope device array below, which every GPU that loads this library holds
// until the process exits.  Inputs and outputs are the caller's device buffers.

namespace gadev
{
static constexpr u64 kNoAllocScratchBytes = 128ULL << 20;       // 128 MiB per GPU
static constexpr u32 kNoAllocThreads = 2048;                     // 16 blocks of 128
static constexpr u32 kNoAllocMaxExtensions = 4096;               // per call
static constexpr u64 kNoAllocMaxReadBp = 8000000;                // per call, summed over the batch
static constexpr u64 kNoAllocHeaderBytes = 256;                  // work counter + arena cursor

static __device__ __align__(256) uint8_t g_noalloc_scratch[kNoAllocScratchBytes];

// The single-extension-per-thread fill + traceback of extend_kernel, with its
// workspace and arena carved out of the scratch array and extensions taken in
// index order (no length ordering, no second launch, no capacity retry: an
// extension that outgrows the small tables reports GA_CAPACITY).
__global__ void __launch_bounds__(128) extend_kernel_noalloc(FillArgs fa, TraceArgs ta, u32* counter)
{
    load_iupac_table();
    const u32 slot = blockIdx.x * blockDim.x + threadIdx.x;
    Workspace w = workspace_at(fa.workspace + (u64)slot * fa.workspaceStride, fa.caps);
    u32 gen = w.header[0];
    ArenaCursor arena;
    arena.pos = 0;
    arena.end = 0;
    WS cols[64];
    while (true)
    {
        const u32 ext = atomicAdd(counter, 1u);
        if (ext >= fa.num) break;
        ExtState st = fill_extension(fa, w, gen, arena, ext);
        trace_extension(ta, ext, st, cols);
    }
    w.header[0] = gen;
}
}

extern "C" int ga_extend_batch_noalloc(const ga_graph_desc* device_graph, const ga_extend_params* params,
    const ga_extend_batch_desc* device_batch, ga_extend_results* device_results, void* stream)
{
    using namespace gadev;
    if (!device_graph || !params || !device_batch || !device_results)
    {
        ga_set_last_error("ga_extend_batch_noalloc: null argument");
        return GA_ERR_ARGUMENT;
    }
    const u32 n = device_batch->num;
    if (n == 0) return GA_OK;
    if (n > kNoAllocMaxExtensions)
    {
        ga_set_last_error("ga_extend_batch_noalloc: more than 4096 extensions in one call (the limit of its fixed scratch)");
        return GA_ERR_ARGUMENT;
    }
    int device = 0;
    if (cudaGetDevice(&device) != cudaSuccess || device < 0 || device >= 64)
    {
        ga_set_last_error("ga_extend_batch_noalloc: no current CUDA device (or ordinal above 63)");
        return GA_ERR_CUDA;
    }
    // once per device, with that device current: the device address of the scratch
    // array (its host-side name is not a device address) and the IUPAC table
    static void* scratchAddress[64] = {};
    if (!scratchAddress[device])
    {
        void* p = nullptr;
        if (cudaGetSymbolAddress(&p, g_noalloc_scratch) != cudaSuccess || !p)
        {
            ga_set_last_error("ga_extend_batch_noalloc: cudaGetSymbolAddress of the scratch array failed");
            return GA_ERR_CUDA;
        }
        if (ga_upload_tables() != 0)
        {
            ga_set_last_error("ga_extend_batch_noalloc: loading the IUPAC table failed");
            return GA_ERR_CUDA;
        }
        scratchAddress[device] = p;
    }
    uint8_t* scratch = (uint8_t*)scratchAddress[device];
    cudaStream_t s = (cudaStream_t)stream;
    // the batch must fit the arena: read the lengths back into a fixed host buffer
    static thread_local uint32_t lengths[kNoAllocMaxExtensions];
    if (cudaMemcpyAsync(lengths, device_batch->seq_len, (size_t)n * 4, cudaMemcpyDeviceToHost, s) != cudaSuccess
        || cudaStreamSynchronize(s) != cudaSuccess)
    {
        ga_set_last_error("ga_extend_batch_noalloc: reading the sequence lengths back failed");
        return GA_ERR_CUDA;
    }
    u64 totalBp = 0;
    for (u32 i = 0; i < n; i++) totalBp += lengths[i];
    if (totalBp > kNoAllocMaxReadBp)
    {
        ga_set_last_error("ga_extend_batch_noalloc: more than 8,000,000 read bp in one call (the limit of its fixed scratch)");
        return GA_ERR_ARGUMENT;
    }

    Caps caps;
    caps.band = 32;
    caps.hash = 128;
    caps.heap = 32;
    caps.extras = 64;
    const u64 stride = ga_workspace_bytes(caps);
    const u64 workspaceBytes = stride * kNoAllocThreads;
    uint8_t* workspace = scratch + kNoAllocHeaderBytes;
    uint8_t* arena = workspace + workspaceBytes;
    const u64 arenaBytes = kNoAllocScratchBytes - kNoAllocHeaderBytes - workspaceBytes;
    // every call starts from zeroed counters and tables: the array keeps what the
    // previous call left in it
    if (cudaMemsetAsync(scratch, 0, kNoAllocHeaderBytes + workspaceBytes, s) != cudaSuccess)
    {
        ga_set_last_error("ga_extend_batch_noalloc: clearing the scratch tables failed");
        return GA_ERR_CUDA;
    }

    DevGraph g;
    g.N = device_graph->num_nodes;
    g.firstAmbiguous = device_graph->first_ambiguous;
    g.len = device_graph->node_length;
    g.seq2 = device_graph->seq2bit;
    g.seqAmb = device_graph->seq_ambiguous;
    g.inOff = device_graph->in_offsets;
    g.inNb = device_graph->in_neighbors;
    g.outOff = device_graph->out_offsets;
    g.outNb = device_graph->out_neighbors;
    g.lin = device_graph->linearizable;
    g.comp = device_graph->component;

    FillArgs fa {};
    fa.g = g;
    fa.bandwidth = params->bandwidth;
    fa.xdrop = params->xdrop;
    fa.maxCells = params->max_cells_per_slice;
    fa.cost = params->xscore_error_cost;
    fa.num = n;
    fa.order = nullptr;
    fa.seq = device_batch->seq;
    fa.seqOff = device_batch->seq_offset;
    fa.seqLen = device_batch->seq_len;
    fa.startNode = device_batch->start_node;
    fa.startOffset = device_batch->start_offset;
    fa.arena = arena;
    fa.arenaBytes = arenaBytes;
    fa.arenaCursor = (unsigned long long*)(scratch + 8);
    fa.workspace = workspace;
    fa.workspaceStride = stride;
    fa.caps = caps;
    fa.prevStatus = nullptr;

    TraceArgs ta {};
    ta.g = g;
    ta.cost = params->xscore_error_cost;
    ta.num = n;
    ta.order = nullptr;
    ta.seq = device_batch->seq;
    ta.seqOff = device_batch->seq_offset;
    ta.seqLen = device_batch->seq_len;
    ta.arena = arena;
    ta.traceOffset = device_batch->trace_offset;
    ta.traceCap = device_batch->trace_capacity;
    ta.status = device_results->status;
    ta.score = device_results->score;
    ta.traceLen = device_results->trace_len;
    ta.traceItems = device_results->trace_items;
    ta.cellSteps = device_results->cell_steps;
    ta.prevStatus = nullptr;

    extend_kernel_noalloc<<<kNoAllocThreads / 128, 128, 0, s>>>(fa, ta, (u32*)scratch);
    if (cudaGetLastError() != cudaSuccess)
    {
        ga_set_last_error("ga_extend_batch_noalloc: kernel launch failed");
        return GA_ERR_CUDA;
    }
    return GA_OK;
}
