// GAF line formatting (GraphAlignerGAFAlignment::traceToAlignment, GraphAlignerGAFAlignment.h:37-200),
// host- and device-callable: the device formats every selected alignment of a batch, one thread
// per line, and the host tests check the number formatting against std::ostream.
#pragma once
#include <stdint.h>
#include <string.h>
#include <string>
#include <vector>

#if defined(__CUDACC__)
#define GAF_HD __host__ __device__
#else
#define GAF_HD
#endif

namespace gaf
{

GAF_HD inline int clz64(uint64_t x)
{
#if defined(__CUDA_ARCH__)
    return __clzll((long long)x);
#else
    return __builtin_clzll(x);
#endif
}

// ---------------------------------------------------------------- integers

GAF_HD inline int fmt_u64(uint64_t v, char* out)
{
    char tmp[20];
    int n = 0;
    do
    {
        tmp[n++] = (char)('0' + v % 10);
        v /= 10;
    } while (v);
    if (out)
        for (int k = 0; k < n; k++) out[k] = tmp[n - 1 - k];
    return n;
}

GAF_HD inline int fmt_i64(int64_t v, char* out)
{
    if (v >= 0) return fmt_u64((uint64_t)v, out);
    if (out) out[0] = '-';
    return 1 + fmt_u64((uint64_t)0 - (uint64_t)v, out ? out + 1 : nullptr);
}

// ---------------------------------------------------------------- doubles

// An unsigned integer of up to kWords 32-bit words, little-endian: enough for a double's
// mantissa shifted by its whole exponent range times a power of ten below 10^30.
struct Big
{
    static constexpr int kWords = 40;
    uint32_t w[kWords];
    int n;   // words in use
    GAF_HD void set(uint64_t v)
    {
        n = 0;
        while (v)
        {
            w[n++] = (uint32_t)v;
            v >>= 32;
        }
    }
    GAF_HD void shl(int bits)
    {
        if (n == 0) return;
        const int words = bits / 32, rem = bits % 32;
        if (rem)
        {
            uint32_t carry = 0;
            for (int k = 0; k < n; k++)
            {
                const uint32_t x = w[k];
                w[k] = (x << rem) | carry;
                carry = x >> (32 - rem);
            }
            if (carry) w[n++] = carry;
        }
        if (words)
        {
            for (int k = n - 1; k >= 0; k--) w[k + words] = w[k];
            for (int k = 0; k < words; k++) w[k] = 0;
            n += words;
        }
    }
    GAF_HD void mul_small(uint32_t m)
    {
        uint64_t carry = 0;
        for (int k = 0; k < n; k++)
        {
            const uint64_t x = (uint64_t)w[k] * m + carry;
            w[k] = (uint32_t)x;
            carry = x >> 32;
        }
        if (carry) w[n++] = (uint32_t)carry;
    }
    GAF_HD void mul_pow10(int e)
    {
        for (; e >= 9; e -= 9) mul_small(1000000000u);
        uint32_t p = 1;
        for (; e > 0; e--) p *= 10;
        if (p > 1) mul_small(p);
    }
    GAF_HD int cmp(const Big& o) const
    {
        if (n != o.n) return n < o.n ? -1 : 1;
        for (int k = n - 1; k >= 0; k--)
            if (w[k] != o.w[k]) return w[k] < o.w[k] ? -1 : 1;
        return 0;
    }
    GAF_HD void sub(const Big& o)   // *this >= o
    {
        int64_t borrow = 0;
        for (int k = 0; k < n; k++)
        {
            int64_t x = (int64_t)w[k] - (k < o.n ? (int64_t)o.w[k] : 0) - borrow;
            borrow = x < 0;
            w[k] = (uint32_t)(x + (borrow << 32));
        }
        while (n > 0 && w[n - 1] == 0) n--;
    }
};

// floor(num / den) for a quotient below 2^32 (repeated doubling subtraction), num becomes the remainder
GAF_HD inline uint64_t big_divmod(Big& num, const Big& den)
{
    uint64_t q = 0;
    Big d = den;
    int shift = 0;
    while (true)
    {
        Big t = d;
        t.shl(1);
        if (t.cmp(num) > 0) break;
        d = t;
        shift++;
    }
    for (; shift >= 0; shift--)
    {
        q <<= 1;
        if (num.cmp(d) >= 0)
        {
            num.sub(d);
            q |= 1;
        }
        // d >>= 1
        uint32_t carry = 0;
        for (int k = d.n - 1; k >= 0; k--)
        {
            const uint32_t x = d.w[k];
            d.w[k] = (x >> 1) | carry;
            carry = x << 31;
        }
        while (d.n > 0 && d.w[d.n - 1] == 0) d.n--;
    }
    return q;
}

// a double as std::ostream writes it by default (printf's %g, precision 6): six significant
// digits correctly rounded from the double's exact value (ties to even), fixed notation for
// decimal exponents -4..5 and scientific otherwise, trailing zeros removed
GAF_HD inline int fmt_g(double v, char* out)
{
    uint64_t bits;
    memcpy(&bits, &v, 8);
    const bool neg = (bits >> 63) != 0;
    const int bexp = (int)((bits >> 52) & 0x7ff);
    uint64_t mant = bits & ((1ULL << 52) - 1);
    char buf[32];
    int n = 0;
    if (neg) buf[n++] = '-';
    if (bexp == 0x7ff)
    {
        const char* s = mant ? "nan" : "inf";
        for (int k = 0; k < 3; k++) buf[n++] = s[k];
    }
    else if (bexp == 0 && mant == 0)
    {
        buf[n++] = '0';
    }
    else
    {
        int e2;
        if (bexp == 0) e2 = -1074;
        else
        {
            mant |= 1ULL << 52;
            e2 = bexp - 1075;
        }
        // value = mant * 2^e2 = num / den
        Big num, den;
        num.set(mant);
        den.set(1);
        if (e2 >= 0) num.shl(e2);
        else den.shl(-e2);
        // decimal exponent: 10^E <= value < 10^(E+1), from an estimate corrected by comparison
        int E = (int)((63 - clz64(mant) + e2) * 0.30102999566398120) - 1;
        while (true)
        {
            Big a = num, b = den;
            if (E + 1 >= 0) b.mul_pow10(E + 1);
            else a.mul_pow10(-(E + 1));
            if (a.cmp(b) < 0) break;
            E++;
        }
        while (true)
        {
            Big a = num, b = den;
            if (E >= 0) b.mul_pow10(E);
            else a.mul_pow10(-E);
            if (a.cmp(b) >= 0) break;
            E--;
        }
        // q = value * 10^(5 - E), six digits, rounded to nearest with ties to even
        Big a = num, b = den;
        if (5 - E >= 0) a.mul_pow10(5 - E);
        else b.mul_pow10(E - 5);
        uint64_t q = big_divmod(a, b);
        a.shl(1);
        const int c = a.cmp(b);
        if (c > 0 || (c == 0 && (q & 1))) q++;
        if (q == 1000000)
        {
            q = 100000;
            E++;
        }
        char d[6];
        for (int k = 5; k >= 0; k--)
        {
            d[k] = (char)('0' + q % 10);
            q /= 10;
        }
        int last = 5;
        while (last > 0 && d[last] == '0') last--;
        if (E < -4 || E >= 6)
        {
            buf[n++] = d[0];
            if (last > 0)
            {
                buf[n++] = '.';
                for (int k = 1; k <= last; k++) buf[n++] = d[k];
            }
            buf[n++] = 'e';
            buf[n++] = E < 0 ? '-' : '+';
            const int ae = E < 0 ? -E : E;
            if (ae >= 100) buf[n++] = (char)('0' + ae / 100);
            buf[n++] = (char)('0' + (ae / 10) % 10);
            buf[n++] = (char)('0' + ae % 10);
        }
        else if (E >= 0)
        {
            for (int k = 0; k <= E; k++) buf[n++] = d[k];
            if (last > E)
            {
                buf[n++] = '.';
                for (int k = E + 1; k <= last; k++) buf[n++] = d[k];
            }
        }
        else
        {
            buf[n++] = '0';
            buf[n++] = '.';
            for (int k = 0; k < -E - 1; k++) buf[n++] = '0';
            for (int k = 0; k <= last; k++) buf[n++] = d[k];
        }
    }
    if (out)
        for (int k = 0; k < n; k++) out[k] = buf[k];
    return n;
}

// ---------------------------------------------------------------- lines

// One trace item after fixForwardTraceSeqPos / fixReverseTraceSeqPosAndOrder: bigraph node id
// (GFA id * 2 + strand), offset in that node, read position, and the read and graph characters.
struct alignas(16) Item
{
    int32_t node;
    uint32_t offset;
    uint32_t seqPos;
    uint8_t nodeSwitch;
    uint8_t seqChar;
    uint8_t graphChar;
    uint8_t pad;
};

// One GAF line as the C ABI takes it: a trace (items [item, item + count)) of read `read`.
struct Line
{
    uint64_t item;
    uint32_t count;
    uint32_t read;
    int32_t xscore100;      // alignmentXScore * 100 (AS:f is left out when the X-score is -1)
    int32_t mapq;
};

// A line after classification: its numeric fields, its edit ops (one byte per trace item,
// ops[op, op + count)) and its node-path entries (bigraph ids, entries[entry, entry + entries)).
struct LineMeta
{
    uint64_t op;
    uint64_t entry;
    uint32_t count;          // trace items: the block length
    uint32_t entries;
    uint32_t read;
    uint32_t readLen;
    uint32_t readStart;
    uint32_t readEnd;
    uint64_t nodePathLen;
    uint64_t nodePathStart;
    uint64_t nodePathEnd;
    uint64_t matches;
    uint64_t edits;          // mismatches + insertions + deletions: NM
    int32_t xscore100;
    int32_t mapq;
};

// The reads' names, and the graph's node names (GFA names by nodeLookup index, empty = the
// numeric id) with its bigraph-id lookup (open addressing) and node sizes.
struct Names
{
    const uint8_t* readNames;
    const uint64_t* readNameOff;    // [reads + 1]
    const uint32_t* readLen;
    const uint8_t* nodeNames;
    const uint64_t* nodeNameOff;    // [lookup + 1]
    const uint32_t* originalSize;   // [lookup]
    const int32_t* idKey;           // bigraph node id (GFA id * 2 + strand) per slot, INT32_MIN = empty
    const uint32_t* idVal;          // nodeLookup index per slot
    uint64_t idCap;                 // slots, a power of two
};

GAF_HD inline uint64_t id_hash(int32_t id)
{
    uint64_t x = (uint32_t)id * 0x9E3779B97F4A7C15ULL;
    return x ^ (x >> 29);
}

// nodeLookup index of a bigraph node id, or UINT32_MAX
GAF_HD inline uint32_t lookup_id(const Names& nm, int32_t bignode)
{
    uint64_t h = id_hash(bignode) & (nm.idCap - 1);
    for (uint64_t k = 0; k < nm.idCap; k++)
    {
        const int32_t key = nm.idKey[h];
        if (key == bignode) return nm.idVal[h];
        if (key == INT32_MIN) return 0xffffffffu;
        h = (h + 1) & (nm.idCap - 1);
    }
    return 0xffffffffu;
}

// IUPAC set of a read or graph byte (bit0 A, bit1 C, bit2 G, bit3 T), -1 when not a sequence character
GAF_HD inline int iupac_set(uint8_t c)
{
    switch (c)
    {
        case 'A': case 'a': return 1;
        case 'C': case 'c': return 2;
        case 'G': case 'g': return 4;
        case 'T': case 't': case 'U': case 'u': return 8;
        case 'M': case 'm': return 1 | 2;
        case 'R': case 'r': return 1 | 4;
        case 'W': case 'w': return 1 | 8;
        case 'S': case 's': return 2 | 4;
        case 'Y': case 'y': return 2 | 8;
        case 'K': case 'k': return 4 | 8;
        case 'V': case 'v': return 1 | 2 | 4;
        case 'H': case 'h': return 1 | 2 | 8;
        case 'D': case 'd': return 1 | 4 | 8;
        case 'B': case 'b': return 2 | 4 | 8;
        case 'N': case 'n': return 15;
    }
    return -1;
}

enum EditOp : uint8_t { OpMatch = 0, OpMismatch = 1, OpMatchOrMismatch = 2, OpInsertion = 3, OpDeletion = 4 };

// The walk of traceToAlignment (GraphAlignerGAFAlignment.h:37-200) over a trace: each item's
// edit op, the node-path entries (an entry at the start and wherever a node switch leaves the
// node) and the counts.  item(k) is the trace's item k; sizeOf(bignode) is the node's length,
// or 0 when the graph lacks it.  False where the reference would assert (a character outside
// the IUPAC set, an unknown node, an offset past its node, a read position out of order or
// past the read).
template <typename GetItem, typename SizeOf>
GAF_HD inline bool classify_line(GetItem item, uint32_t count, uint32_t readLen, bool cigarMerge, SizeOf sizeOf, LineMeta& m, uint8_t* ops,
    int32_t* entries)
{
    m.count = count;
    m.entries = 0;
    m.readLen = readLen;
    if (count == 0) return false;
    auto match = [&](const Item& it, bool& bad) -> bool
    {
        const int a = iupac_set(it.seqChar), b = iupac_set(it.graphChar);
        if (a < 0 || b < 0) { bad = true; return false; }
        return (a & b) != 0;
    };
    bool bad = false;
    uint64_t matches = 0, edits = 0;
    const Item first = item(0);
    int32_t curNode = first.node;
    uint32_t curOffset = first.offset;
    uint32_t curSeq = first.seqPos;
    uint64_t sz = sizeOf(curNode);
    if (sz == 0 || first.seqPos >= readLen) return false;
    uint64_t nodePathLen = sz;
    entries[m.entries++] = curNode;
    const bool m0 = match(first, bad);
    if (m0) matches++; else edits++;
    ops[0] = cigarMerge ? OpMatchOrMismatch : (m0 ? OpMatch : OpMismatch);
    Item b = first;
    for (uint32_t pos = 1; pos < count; pos++)
    {
        const Item a = b;
        b = item(pos);
        if (b.seqPos < curSeq || b.seqPos >= readLen) return false;
        const bool inside = !a.nodeSwitch || (b.node == curNode && b.offset > curOffset);
        if (!inside)
        {
            const uint64_t before = sizeOf(curNode) - 1 - a.offset;
            curNode = b.node;
            curOffset = b.offset;
            curSeq = b.seqPos;
            sz = sizeOf(curNode);
            if (sz == 0 || b.offset >= sz) return false;
            nodePathLen += sz - (before + b.offset);
            entries[m.entries++] = curNode;
        }
        uint8_t op;
        if (a.seqPos == b.seqPos)
        {
            op = OpDeletion;
            edits++;
        }
        else if (inside && a.offset == b.offset)
        {
            op = OpInsertion;
            edits++;
        }
        else
        {
            const bool mt = match(b, bad);
            if (mt) matches++; else edits++;
            op = cigarMerge ? OpMatchOrMismatch : (mt ? OpMatch : OpMismatch);
        }
        ops[pos] = op;
    }
    if (bad) return false;
    m.readStart = first.seqPos;
    m.readEnd = b.seqPos + 1;
    m.nodePathLen = nodePathLen;
    m.nodePathStart = first.offset;
    m.nodePathEnd = nodePathLen - (sizeOf(b.node) - 1 - b.offset);
    m.matches = matches;
    m.edits = edits;
    return true;
}

// Writes one classified GAF line (no newline) to out, or only measures it when out is null;
// returns its length.
GAF_HD inline int64_t write_line(const Names& nm, const LineMeta& m, const uint8_t* ops, const int32_t* entries, char* out)
{
    const char codes[5] = { '=', 'X', 'M', 'I', 'D' };
    int64_t n = 0;
    auto put = [&](char c) { if (out) out[n] = c; n++; };
    auto putU = [&](uint64_t v) { n += fmt_u64(v, out ? out + n : nullptr); };
    auto putS = [&](const uint8_t* p, uint64_t len) { if (out) for (uint64_t k = 0; k < len; k++) out[n + k] = (char)p[k]; n += len; };
    putS(nm.readNames + nm.readNameOff[m.read], nm.readNameOff[m.read + 1] - nm.readNameOff[m.read]);
    put('\t'); putU(m.readLen);
    put('\t'); putU(m.readStart);
    put('\t'); putU(m.readEnd);
    put('\t'); put('+'); put('\t');
    for (uint32_t k = 0; k < m.entries; k++)
    {
        const int32_t bignode = entries[m.entry + k];
        put((bignode % 2 == 1) ? '<' : '>');
        const uint32_t li = lookup_id(nm, bignode);
        const uint64_t from = nm.nodeNameOff[li], to = nm.nodeNameOff[li + 1];
        if (to == from) n += fmt_i64(bignode / 2, out ? out + n : nullptr);
        else putS(nm.nodeNames + from, to - from);
    }
    put('\t'); putU(m.nodePathLen);
    put('\t'); putU(m.nodePathStart);
    put('\t'); putU(m.nodePathEnd);
    put('\t'); putU(m.matches);
    put('\t'); putU(m.count);
    put('\t'); n += fmt_i64(m.mapq, out ? out + n : nullptr);
    put('\t'); putS((const uint8_t*)"NM:i:", 5); putU(m.edits);
    if (m.xscore100 != -100)
    {
        put('\t'); putS((const uint8_t*)"AS:f:", 5);
        n += fmt_g((double)m.xscore100 / 100.0, out ? out + n : nullptr);
    }
    const double total = (double)(m.matches + m.edits);
    put('\t'); putS((const uint8_t*)"dv:f:", 5);
    n += fmt_g(1.0 - ((double)m.matches / total), out ? out + n : nullptr);
    put('\t'); putS((const uint8_t*)"id:f:", 5);
    n += fmt_g((double)m.matches / total, out ? out + n : nullptr);
    put('\t'); putS((const uint8_t*)"cg:Z:", 5);
    // the CIGAR: runs of one edit op
    const uint8_t* o = ops + m.op;
    uint8_t current = o[0];
    uint64_t run = 1;
    for (uint32_t pos = 1; pos < m.count; pos++)
    {
        if (o[pos] != current)
        {
            putU(run);
            put(codes[current]);
            current = o[pos];
            run = 0;
        }
        run++;
    }
    putU(run);
    put(codes[current]);
    return n;
}

// ---------------------------------------------------------------- selection

// AlignmentSelection::alignmentIncompatible (AlignmentSelection.cpp:13-29)
GAF_HD inline bool incompatible(uint64_t ls, uint64_t le, uint64_t rs, uint64_t re)
{
    const float cutoff = 0.05f;
    const uint64_t ll = le - ls, rl = re - rs;
    const float minOverlapLen = (float)(ll < rl ? ll : rl) * cutoff;
    if (ls > rs)
    {
        uint64_t t = ls; ls = rs; rs = t;
        t = le; le = re; re = t;
    }
    int overlap = 0;
    if (le > rs) overlap = (int)(le - rs);
    return (float)overlap > minOverlapLen;
}

// AlignmentSelection::SelectAlignments (AlignmentSelection.cpp:31-95) without the E-value
// filter, for one read's n alignments: keep[k] = alignment k stays.  Both filters keep the
// order, so the kept alignments are those of the reference, in its order.
GAF_HD inline void select_read(uint32_t n, const uint64_t* start, const uint64_t* end, const double* xscore, int minAlignmentScore,
    double fractionCutoff, char* keep)
{
    const bool byScore = minAlignmentScore > INT32_MIN;
    for (uint32_t k = 0; k < n; k++) keep[k] = !byScore || xscore[k] >= (double)minAlignmentScore;
    if (fractionCutoff == 0) return;
    // the second filter compares against the alignments the first one kept
    for (uint32_t i = 0; i < n; i++)
    {
        if (!keep[i]) continue;
        bool skipped = false;
        for (uint32_t j = 0; j < n && !skipped; j++)
        {
            if (j == i || !(!byScore || xscore[j] >= (double)minAlignmentScore)) continue;
            if (!incompatible(start[i], end[i], start[j], end[j])) continue;
            if (xscore[i] < xscore[j] * fractionCutoff) skipped = true;
        }
        if (skipped) keep[i] |= 2;   // marked, cleared below so later tests still see it
    }
    for (uint32_t k = 0; k < n; k++) keep[k] = keep[k] == 1;
}

// ---------------------------------------------------------------- host-side tables

// The node names and the bigraph-id lookup of Names, from the graph's nodeLookup arrays (host).
struct NamesHost
{
    std::vector<uint8_t> nodeNames;
    std::vector<uint64_t> nodeNameOff;
    std::vector<uint32_t> originalSize;
    std::vector<int32_t> idKey;
    std::vector<uint32_t> idVal;
    uint64_t idCap = 0;
};

inline void build_names(const std::vector<int32_t>& lookupIds, const std::vector<std::string>& names, const std::vector<uint32_t>& originalSize,
    NamesHost& out)
{
    const size_t n = lookupIds.size();
    out.nodeNameOff.assign(n + 1, 0);
    out.nodeNames.clear();
    for (size_t i = 0; i < n; i++)
    {
        out.nodeNames.insert(out.nodeNames.end(), names[i].begin(), names[i].end());
        out.nodeNameOff[i + 1] = out.nodeNames.size();
    }
    if (out.nodeNames.empty()) out.nodeNames.push_back(0);
    out.originalSize = originalSize;
    out.idCap = 16;
    while (out.idCap < 2 * (uint64_t)n) out.idCap <<= 1;
    out.idKey.assign(out.idCap, INT32_MIN);
    out.idVal.assign(out.idCap, 0);
    for (size_t i = 0; i < n; i++)
    {
        uint64_t h = id_hash(lookupIds[i]) & (out.idCap - 1);
        while (out.idKey[h] != INT32_MIN && out.idKey[h] != lookupIds[i]) h = (h + 1) & (out.idCap - 1);
        out.idKey[h] = lookupIds[i];
        out.idVal[h] = (uint32_t)i;
    }
}

inline Names names_view(const NamesHost& h)
{
    Names nm {};
    nm.nodeNames = h.nodeNames.data();
    nm.nodeNameOff = h.nodeNameOff.data();
    nm.originalSize = h.originalSize.data();
    nm.idKey = h.idKey.data();
    nm.idVal = h.idVal.data();
    nm.idCap = h.idCap;
    return nm;
}

}
