// 64-row Myers bit-vector column algebra on the GPU.
//
// A column of the 64-row DP slice is (VP, VN, end): vertical +1/-1 deltas and
// the score of the last row, as GraphAligner's WordSlice<uint64_t>
// (WordSlice.h:150-765).  The 64-row word is semantic — band membership,
// X-drop and traceback corners are decided per 64 rows — so every operation
// here works on full 64-bit words (two 32-bit halves in SASS) and reproduces
// the reference's integer results bit for bit.
//
// Functions are __host__ __device__ so the host-side unit tests can exercise
// the same code paths; the product calls them from the kernels only.
#pragma once
#include <stdint.h>

#ifdef __CUDACC__
#define GA_HD __host__ __device__ __forceinline__
#else
#define GA_HD inline
#endif

namespace gadev
{
typedef uint64_t u64;
typedef int32_t i32;
typedef uint32_t u32;

static constexpr u64 kAllOnes = ~0ULL;
static constexpr u64 kLastBit = 1ULL << 63;
static constexpr i32 kIntMax = 0x7fffffff;
static constexpr i32 kIntMin = (i32)0x80000000;

GA_HD int popc64(u64 x)
{
#ifdef __CUDA_ARCH__
    return __popcll(x);
#else
    return __builtin_popcountll(x);
#endif
}

// wrapping int32 arithmetic (the reference relies on two's-complement results)
GA_HD i32 wadd(i32 a, i32 b) { return (i32)((u32)a + (u32)b); }
GA_HD i32 wsub(i32 a, i32 b) { return (i32)((u32)a - (u32)b); }
GA_HD i32 wmul(i32 a, i32 b) { return (i32)((u32)a * (u32)b); }
GA_HD i32 imax(i32 a, i32 b) { return a > b ? a : b; }
GA_HD i32 imin(i32 a, i32 b) { return a < b ? a : b; }

struct WS
{
    u64 VP;
    u64 VN;
    i32 end;
};

GA_HD WS ws_make(u64 vp, u64 vn, i32 end) { WS w; w.VP = vp; w.VN = vn; w.end = end; return w; }
GA_HD bool ws_eq(const WS& a, const WS& b) { return a.VP == b.VP && a.VN == b.VN && a.end == b.end; }

// score of row `row` (WordSlice::getValue, WordSlice.h:177-186)
GA_HD i32 ws_value(const WS& w, int row)
{
    u64 mask = row < 63 ? (kAllOnes << (row + 1)) : 0ULL;
    return wsub(wadd(w.end, popc64(w.VN & mask)), popc64(w.VP & mask));
}

// score of the row above the column (WordSlice::getScoreBeforeStart, WordSlice.h:244-247)
GA_HD i32 ws_before(const WS& w)
{
    return wadd(wsub(w.end, popc64(w.VP)), popc64(w.VN));
}

GA_HD i32 ws_xscore(const WS& w, i32 seqOffset, int offset, i32 cost)
{
    return wsub(wmul(wadd(wadd(seqOffset, offset), 1), 100), wmul(ws_value(w, offset), cost));
}

GA_HD int popc32(u32 x)
{
#ifdef __CUDA_ARCH__
    return __popc(x);
#else
    return __builtin_popcount(x);
#endif
}

GA_HD int ctz32(u32 x)
{
#ifdef __CUDA_ARCH__
    return __ffs((int)x) - 1;
#else
    return __builtin_ctz(x);
#endif
}

// Best X-score over the column's local-minimum rows (WordSlice::maxXScoreLocalMinima,
// WordSlice.h:313-347): candidates are the rows just below a run of +1 steps,
// filtered by extraMask, plus the first and the last counted row.  For row m the
// X-score is 100*(m+1) - cost * (signed popcount of rows 0..m).  The always-present
// first and last rows are evaluated directly, so the loop only visits the
// remaining candidates (about 1.3 per column on the workloads); the result is the
// same maximum.
GA_HD i32 xs_row(u32 vpl, u32 vnl, u32 vph, u32 vnh, i32 lowDelta, int m, i32 cost)
{
    i32 s;
    if (m < 32)
    {
        u32 upto = (2u << m) - 1u;
        s = popc32(vpl & upto) - popc32(vnl & upto);
    }
    else
    {
        u32 upto = (2u << (m - 32)) - 1u;
        s = lowDelta + popc32(vph & upto) - popc32(vnh & upto);
    }
    return wsub(wmul(m + 1, 100), wmul(s, cost));
}

GA_HD i32 ws_max_xscore(const WS& w, i32 seqOffset, i32 cost, int cells, u64 extraMask)
{
    const u32 vpl = (u32)w.VP, vnl = (u32)w.VN, vph = (u32)(w.VP >> 32), vnh = (u32)(w.VN >> 32);
    const i32 lowDelta = popc32(vpl) - popc32(vnl);
    const i32 allDelta = lowDelta + popc32(vph) - popc32(vnh);
    const i32 before = wsub(w.end, allDelta);
    u64 notVP = ~w.VP;
    u64 cand = (w.VP & (notVP - w.VP)) >> 1;
    cand |= kLastBit & (notVP | ~(notVP - w.VP)) & ~w.VP;
    cand &= extraMask;
    i32 best;
    // row 0
    best = wsub(100, wmul((i32)(vpl & 1) - (i32)(vnl & 1), cost));
    int last;
    if (cells < 64)
    {
        cand &= ~(kAllOnes << cells);
        last = cells - 1;
    }
    else
    {
        last = 63;
    }
    if (last == 63) best = imax(best, wsub(6400, wmul(allDelta, cost)));
    else best = imax(best, xs_row(vpl, vnl, vph, vnh, lowDelta, last, cost));
    cand &= ~1ULL;
    cand &= ~(1ULL << last);
    while (cand != 0)
    {
        u32 lo = (u32)cand;
        int m = lo != 0 ? ctz32(lo) : 32 + ctz32((u32)(cand >> 32));
        best = imax(best, xs_row(vpl, vnl, vph, vnh, lowDelta, m, cost));
        cand &= cand - 1;
    }
    return wadd(best, wsub(wmul(seqOffset, 100), wmul(before, cost)));
}

// Match masks of one 64-row slice, one per base (EqVector, Common.h:36-136)
struct EqV4
{
    u64 a, c, g, t;
};

// mask for a 2-bit base code (A=0 C=1 G=2 T=3), selected without indexing
GA_HD u64 eq_pick(const EqV4& e, u32 code)
{
    u64 x = (code & 1) ? e.c : e.a;
    u64 y = (code & 1) ? e.t : e.g;
    return (code & 2) ? y : x;
}

// mask for an ambiguous graph base given its A,C,G,T membership bits
GA_HD u64 eq_amb(const EqV4& e, u32 bits)
{
    return ((bits & 1) ? e.a : 0) | ((bits & 2) ? e.c : 0) | ((bits & 4) ? e.g : 0) | ((bits & 8) ? e.t : 0);
}

// Rows where the left column is smaller / the right column is smaller
// (WordSlice::differenceMasksBitTwiddle, WordSlice.h:566-664).  scoreDifference
// is right's score above row 0 minus left's.
struct Masks { u64 leftSmaller; u64 rightSmaller; };

GA_HD u64 lowbit(u64 x) { return x & (0ULL - x); }

GA_HD Masks difference_masks(u64 lVP, u64 lVN, u64 rVP, u64 rVN, int scoreDifference)
{
    Masks r; r.leftSmaller = 0; r.rightSmaller = 0;
    u64 vpCommon = ~(lVP & rVP);
    u64 vnCommon = ~(lVN & rVN);
    lVP &= vpCommon; lVN &= vnCommon; rVP &= vpCommon; rVN &= vnCommon;
    u64 twoSmaller = lVN & rVP;
    u64 oneSmaller = (rVP & ~lVN) | (lVN & ~rVP) | twoSmaller;
    u64 twoBigger = rVN & lVP;
    u64 oneBigger = (lVP & ~rVN) | (rVN & ~lVP) | twoBigger;
    if (scoreDifference > 0)
    {
        for (int i = 1; i < scoreDifference; i++)
        {
            u64 ls = lowbit(oneBigger);
            oneBigger ^= (~twoBigger & ls);
            twoBigger &= ~ls;
            if (oneBigger == 0) { r.leftSmaller = kAllOnes; r.rightSmaller = 0; return r; }
        }
        u64 ls = lowbit(oneBigger);
        r.leftSmaller |= ls - 1;
        oneBigger ^= (~twoBigger & ls);
        twoBigger &= ~ls;
    }
    else if (scoreDifference < 0)
    {
        for (int i = 1; i < -scoreDifference; i++)
        {
            u64 ls = lowbit(oneSmaller);
            oneSmaller ^= (~twoSmaller & ls);
            twoSmaller &= ~ls;
            if (oneSmaller == 0) { r.leftSmaller = 0; r.rightSmaller = kAllOnes; return r; }
        }
        u64 ls = lowbit(oneSmaller);
        r.rightSmaller |= ls - 1;
        oneSmaller ^= (~twoSmaller & ls);
        twoSmaller &= ~ls;
    }
    for (int i = 0; i < 64; i++)
    {
        if (oneSmaller == 0)
        {
            if (oneBigger != 0) r.rightSmaller |= 0ULL - lowbit(oneBigger);
            break;
        }
        if (oneBigger == 0)
        {
            r.leftSmaller |= 0ULL - lowbit(oneSmaller);
            break;
        }
        u64 lb = lowbit(oneBigger);
        u64 ls = lowbit(oneSmaller);
        if (lb > ls) r.leftSmaller |= lb - ls;
        else r.rightSmaller |= ls - lb;
        oneBigger ^= (~twoBigger & lb);
        twoBigger &= ~lb;
        oneSmaller ^= (~twoSmaller & ls);
        twoSmaller &= ~ls;
    }
    return r;
}

// Cellwise minimum of two columns (WordSlice::mergeTwoSlices, WordSlice.h:502-541)
GA_HD WS ws_merge(WS a, WS b)
{
    i32 ba = ws_before(a), bb = ws_before(b);
    if (ba > bb) { WS t = a; a = b; b = t; i32 u = ba; ba = bb; bb = u; }
    Masks m = difference_masks(a.VP, a.VN, b.VP, b.VN, wsub(bb, ba));
    u64 takeB = (m.rightSmaller | ((m.leftSmaller | m.rightSmaller) - (m.rightSmaller << 1))) & ~m.leftSmaller;
    u64 aRed = m.leftSmaller & (m.rightSmaller << 1);
    u64 bRed = m.rightSmaller & (m.leftSmaller << 1);
    if ((m.rightSmaller & 1) && ba < bb) bRed |= 1;
    a.VN &= ~aRed;
    b.VN &= ~bRed;
    WS r;
    r.VN = (a.VN & ~takeB) | (b.VN & takeB);
    r.VP = (a.VP & ~takeB) | (b.VP & takeB);
    r.end = imin(a.end, b.end);
    return r;
}

// Smallest score of a changed end column where it improved on the old one
// (WordSlice::changedMinScoreLocalMinima, WordSlice.h:438-472)
GA_HD i32 ws_changed_min(const WS& w, const WS& old)
{
    i32 before = ws_before(w);
    i32 oldBefore = ws_before(old);
    u64 cand = (w.VP & (w.VN - w.VP)) >> 1;
    cand |= kLastBit & (w.VN | ~(w.VN - w.VP)) & ~w.VP;
    if (wadd(w.end, popc64(w.VN)) >= wsub(old.end, popc64(old.VP)))
    {
        u64 smaller = difference_masks(w.VP, w.VN, old.VP, old.VN, wsub(oldBefore, before)).leftSmaller;
        if (smaller != kAllOnes)
        {
            cand |= (~smaller) >> 1;
            cand |= (~smaller) << 1;
            cand |= 1;
            cand |= kLastBit;
            cand &= smaller;
        }
    }
    i32 best = before < oldBefore ? before : kIntMax;
    while (cand != 0)
    {
        u64 upto = cand ^ (cand - 1);
        best = imin(best, wsub(wadd(before, popc64(w.VP & upto)), popc64(w.VN & upto)));
        cand &= ~upto;
    }
    return best;
}

// One Myers (1999) column step with horizontal inputs hinP/hinN
// (GraphAlignerBitvectorCommon::getNextSlice, Common.h:242-262).
// Ph/Mh receive the full horizontal delta words.
GA_HD WS myers_step(u64 eq, WS s, u64 hinP, u64 hinN, u64& Ph, u64& Mh)
{
    u64 Xv = eq | s.VN;
    eq |= hinN;
    u64 Xh = (((eq & s.VP) + s.VP) ^ s.VP) | eq;
    Ph = s.VN | ~(Xh | s.VP);
    Mh = s.VP & Xh;
    u64 shM = (Mh << 1) | hinN;
    u64 shP = (Ph << 1) | hinP;
    WS r;
    r.VP = shM | ~(Xv | shP);
    r.VN = shP & Xv;
    r.end = wadd(wsub(s.end, (i32)(Mh >> 63)), (i32)(Ph >> 63));
    return r;
}

// column entering from a row-above score (getSourceSliceFromScore, Common.h:1056-1060)
GA_HD WS ws_source(i32 previousScore)
{
    return ws_make(kAllOnes, 0, wadd(previousScore, 64));
}

// IUPAC bit masks: bit0 A, bit1 C, bit2 G, bit3 T; 0 = '-', -1 = not a sequence character
// (GraphAlignerCommon::ambiguousMatch, GraphAlignerCommon.h:204-279)
GA_HD int iupac_mask(unsigned char c)
{
    switch (c)
    {
        case 'A': case 'a': return 1;
        case 'C': case 'c': return 2;
        case 'G': case 'g': return 4;
        case 'T': case 't': case 'U': case 'u': return 8;
        case 'R': case 'r': return 5;
        case 'Y': case 'y': return 10;
        case 'K': case 'k': return 12;
        case 'M': case 'm': return 3;
        case 'S': case 's': return 6;
        case 'W': case 'w': return 9;
        case 'B': case 'b': return 14;
        case 'D': case 'd': return 13;
        case 'H': case 'h': return 11;
        case 'V': case 'v': return 7;
        case 'N': case 'n': return 15;
        case '-': return 0;
    }
    return -1;
}

// min-heap of the component priority queue, laid out and operated exactly as
// libstdc++'s std::priority_queue<..., std::greater<>> (push_heap / pop_heap,
// bits/stl_heap.h): ties in (component, score) then resolve the same way
// (ComponentPriorityQueue.h:11-19,153).
struct HeapItem { u32 component; i32 score; u32 node; };

GA_HD bool heap_greater(const HeapItem& a, const HeapItem& b)
{
    return a.component > b.component || (a.component == b.component && a.score > b.score);
}

GA_HD void heap_push(HeapItem* h, u32& n, HeapItem v)
{
    u32 hole = n;
    while (hole > 0)
    {
        u32 parent = (hole - 1) / 2;
        if (!heap_greater(h[parent], v)) break;
        h[hole] = h[parent];
        hole = parent;
    }
    h[hole] = v;
    n++;
}

GA_HD void heap_pop(HeapItem* h, u32& n)
{
    if (n > 1)
    {
        HeapItem v = h[n - 1];
        h[n - 1] = h[0];
        long len = (long)n - 1;
        long hole = 0;
        long child = 0;
        while (child < (len - 1) / 2)
        {
            child = 2 * (child + 1);
            if (heap_greater(h[child], h[child - 1])) child--;
            h[hole] = h[child];
            hole = child;
        }
        if ((len & 1) == 0 && child == (len - 2) / 2)
        {
            child = 2 * (child + 1);
            h[hole] = h[child - 1];
            hole = child - 1;
        }
        while (hole > 0)
        {
            long parent = (hole - 1) / 2;
            if (!heap_greater(h[parent], v)) break;
            h[hole] = h[parent];
            hole = parent;
        }
        h[hole] = v;
    }
    n--;
}

}
