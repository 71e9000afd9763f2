// Property tests of the kernels' 64-row column algebra (graphaligner_gb300/csrc/wordslice.cuh,
// compiled here for the host): every bit-parallel operation against a cell-by-cell restatement,
// as the reference's EXTRACORRECTNESSASSERTIONS checks do (WordSlice.h:263-311, 666-700;
// GraphAlignerBitvectorCommon.h:242-262), and the component queue's heap against
// std::priority_queue with std::greater (ComponentPriorityQueue.h:11-19).
// Prints "ok <cases>" or the first failing property and exits non-zero.
#include <cstdio>
#include <cstdlib>
#include <functional>
#include <queue>
#include <random>
#include <vector>
#include "../../graphaligner_gb300/csrc/wordslice.cuh"

using namespace gadev;

static std::mt19937_64 rng(12345);

static int fail(const char* what, long long i)
{
    printf("FAIL %s case %lld\n", what, i);
    return 1;
}

// a column with disjoint VP/VN; runs of one kind of step are common in DP columns
static WS randomColumn()
{
    u64 a = rng(), b = rng();
    switch (rng() % 4)
    {
        case 0: break;
        case 1: a &= rng(); b &= rng(); break;
        case 2: a = rng() & rng() & rng(); b = ~a & rng(); break;
        default: b = rng() & rng() & rng(); a = ~b & rng(); break;
    }
    WS w;
    w.VP = a & ~b;
    w.VN = b & ~a;
    w.end = (i32)(rng() % 2001) - 1000;
    return w;
}

// score of every row, from the row above (WordSlice::getValueStartBased)
static void cells(const WS& w, i32 before, i32* v)
{
    i32 s = before;
    for (int r = 0; r < 64; r++)
    {
        s += (int)((w.VP >> r) & 1) - (int)((w.VN >> r) & 1);
        v[r] = s;
    }
}

static WS fromCells(i32 before, const i32* v)
{
    WS w {0, 0, v[63]};
    i32 prev = before;
    for (int r = 0; r < 64; r++)
    {
        if (v[r] - prev == 1) w.VP |= 1ULL << r;
        else if (v[r] - prev == -1) w.VN |= 1ULL << r;
        else if (v[r] != prev) { w.end = kIntMin; return w; }
        prev = v[r];
    }
    return w;
}

int main()
{
    const long long N = 200000;
    i32 a[64], b[64];
    for (long long i = 0; i < N; i++)
    {
        WS x = randomColumn(), y = randomColumn();
        const i32 bx = ws_before(x);
        cells(x, bx, a);
        if (a[63] != x.end) return fail("before + steps != end", i);
        for (int r = 0; r < 64; r++) if (ws_value(x, r) != a[r]) return fail("ws_value", i);
        // X-score maximum over the first `cells` rows, for error costs above 100 (local minima suffice)
        {
            const int nCells = 1 + (int)(rng() % 64);
            const i32 seqOffset = (i32)(rng() % 100000);
            const i32 cost = 101 + (i32)(rng() % 400);
            i32 best = kIntMin;
            for (int r = 0; r < nCells; r++) best = imax(best, (seqOffset + r + 1) * 100 - a[r] * cost);
            if (ws_max_xscore(x, seqOffset, cost, nCells, kAllOnes) != best) return fail("ws_max_xscore", i);
        }
        // y drawn near x, so that the columns cross
        if (i % 2 == 0) y.end = x.end + (i32)(rng() % 9) - 4;
        const i32 by = ws_before(y);
        cells(y, by, b);
        // differenceMasks: rows where one column is strictly smaller (score difference = before(y) - before(x))
        {
            Masks m = difference_masks(x.VP, x.VN, y.VP, y.VN, by - bx);
            u64 ls = 0, rs = 0;
            for (int r = 0; r < 64; r++)
            {
                if (a[r] < b[r]) ls |= 1ULL << r;
                if (b[r] < a[r]) rs |= 1ULL << r;
            }
            if (m.leftSmaller != ls || m.rightSmaller != rs) return fail("difference_masks", i);
        }
        // mergeTwoSlices: the cellwise minimum
        {
            WS m = ws_merge(x, y);
            if (m.VP & m.VN) return fail("ws_merge VP&VN", i);
            for (int r = 0; r < 64; r++) if (ws_value(m, r) != imin(a[r], b[r])) return fail("ws_merge value", i);
            if (ws_before(m) != imin(bx, by)) return fail("ws_merge before", i);
        }
        // changedMinScore: the smallest score among rows (and the row above) where x improved on y
        {
            i32 best = bx < by ? bx : kIntMax;
            for (int r = 0; r < 64; r++) if (a[r] < b[r]) best = imin(best, a[r]);
            if (ws_changed_min(x, y) != best) return fail("ws_changed_min", i);
        }
        // getNextSlice: one edit-distance column step; the row above moves by -1, 0 or +1
        {
            const u64 eq = (i % 3 == 0) ? (rng() & rng()) : rng();
            const int h = (int)(rng() % 3) - 1;
            u64 Ph, Mh;
            WS n = myers_step(eq, x, h > 0 ? 1 : 0, h < 0 ? 1 : 0, Ph, Mh);
            i32 nv[64];
            i32 above = bx + h, aboveOld = bx;
            u64 ph = 0, mh = 0;
            for (int r = 0; r < 64; r++)
            {
                const i32 diag = aboveOld + (((eq >> r) & 1) ? 0 : 1);
                nv[r] = imin(imin(a[r] + 1, above + 1), diag);
                if (nv[r] - a[r] == 1) ph |= 1ULL << r;
                if (nv[r] - a[r] == -1) mh |= 1ULL << r;
                above = nv[r];
                aboveOld = a[r];
            }
            WS want = fromCells(bx + h, nv);
            if (!ws_eq(n, want)) return fail("myers_step column", i);
            if (Ph != ph || Mh != mh) return fail("myers_step horizontal deltas", i);
        }
    }
    // the component queue's heap: the same pop order as std::priority_queue<..., std::greater>,
    // ties included
    for (int t = 0; t < 2000; t++)
    {
        struct Greater
        {
            bool operator()(const HeapItem& l, const HeapItem& r) const { return heap_greater(l, r); }
        };
        std::priority_queue<HeapItem, std::vector<HeapItem>, Greater> ref;
        std::vector<HeapItem> h(512);
        u32 n = 0;
        u32 nextNode = 0;
        const int ops = 1 + (int)(rng() % 400);
        for (int k = 0; k < ops; k++)
        {
            if (n < 500 && (n == 0 || rng() % 3 != 0))
            {
                HeapItem v { (u32)(rng() % 4), (i32)(rng() % 6), nextNode++ };
                ref.push(v);
                heap_push(h.data(), n, v);
            }
            else
            {
                const HeapItem want = ref.top();
                ref.pop();
                const HeapItem got = h[0];
                heap_pop(h.data(), n);
                if (got.node != want.node || got.component != want.component || got.score != want.score) return fail("heap order", t);
            }
            if (n != ref.size()) return fail("heap size", t);
        }
    }
    // IUPAC codes: each letter's bases, either case; '-' matches nothing
    {
        const char* letters = "ACGTURYKMSWBDHVN";
        const int masks[16] = { 1, 2, 4, 8, 8, 5, 10, 12, 3, 6, 9, 14, 13, 11, 7, 15 };
        for (int k = 0; k < 16; k++)
        {
            if (iupac_mask((unsigned char)letters[k]) != masks[k]) return fail("iupac_mask upper", k);
            if (iupac_mask((unsigned char)(letters[k] + 32)) != masks[k]) return fail("iupac_mask lower", k);
        }
        if (iupac_mask('-') != 0 || iupac_mask('X') != -1 || iupac_mask('*') != -1) return fail("iupac_mask other", 0);
    }
    printf("ok %lld\n", N);
    return 0;
}
