// Read-level host layer of the GB300 extension path: the reference's per-read
// alignment flow restated over batched GPU extensions.
//
// For every read of a batch this follows runComponentMappings' GAF path
// (Aligner.cpp:440-592): minimizer seeds (MinimizerSeeder::getSeeds, with the
// k-mer lookup done by the seed_lookup kernel) -> OrderSeeds
// (GraphAligner::orderSeedsByChaining, GraphAligner.h:250-312) -> the seed loop of
// GraphAligner::AlignOneWay (GraphAligner.h:94-181) -> SelectAlignments
// (AlignmentSelection.cpp:31-53) -> GAF lines (GraphAlignerGAFAlignment.h:37-200).
// The seed loop is sequential per read because its skip rules read the traces
// of earlier seeds; reads advance in lock step instead: every round collects the
// two extensions (GraphAligner::getTwoDirectionalTrace, GraphAligner.h:475-520)
// of each read's next seed and runs them as one ga_extend_batch call.
#include <algorithm>
#include <chrono>
#include <atomic>
#include <thread>
#include <climits>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <deque>
#include <limits>
#include <memory>
#include <sstream>
#include <stdexcept>
#include <string>
#include <tuple>
#include <unordered_map>
#include <unordered_set>
#include <vector>
#include "../../include/graphaligner_gb300.h"
#include "readalign.h"
#include "trace_dedupe.h"

namespace gahost
{

struct ReadFailure {};
#define GAH_ASSERT(x) do { if (!(x)) throw ::gahost::ReadFailure{}; } while (0)

// ------------------------------------------------------------------ graph

int iupac(char c)
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

// GraphAlignerCommon::characterMatch (GraphAlignerCommon.h:176-200)
bool characterMatch(char s, char g)
{
    if (s == g) return true;
    int a = iupac(s), b = iupac(g);
    GAH_ASSERT(a >= 0 && b >= 0);
    return (a & b) != 0;
}

// CommonUtils::Complement (CommonUtils.cpp:78-134)
char complement(char c)
{
    switch (c)
    {
        case 'A': case 'a': return 'T';
        case 'C': case 'c': return 'G';
        case 'T': case 't': return 'A';
        case 'G': case 'g': return 'C';
        case 'N': case 'n': return 'N';
        case 'U': case 'u': return 'A';
        case 'R': case 'r': return 'Y';
        case 'Y': case 'y': return 'R';
        case 'K': case 'k': return 'M';
        case 'M': case 'm': return 'K';
        case 'S': case 's': return 'S';
        case 'W': case 'w': return 'W';
        case 'B': case 'b': return 'V';
        case 'V': case 'v': return 'B';
        case 'D': case 'd': return 'H';
        case 'H': case 'h': return 'D';
    }
    GAH_ASSERT(false);
    return 'N';
}

std::string reverseComplement(const std::string& s)
{
    std::string r;
    r.reserve(s.size());
    for (size_t i = s.size(); i > 0; i--) r += complement(s[i - 1]);
    return r;
}

HostGraph::HostGraph(const ga_host_graph_desc& d) :
    N(d.base.num_nodes), firstAmbiguous(d.base.first_ambiguous)
{
    len.assign(d.base.node_length, d.base.node_length + N);
    seq2.assign(d.base.seq2bit, d.base.seq2bit + (size_t)firstAmbiguous * 2);
    seqAmb.assign(d.base.seq_ambiguous, d.base.seq_ambiguous + (size_t)(N - firstAmbiguous) * 4);
    inOff.assign(d.base.in_offsets, d.base.in_offsets + N + 1);
    inNb.assign(d.base.in_neighbors, d.base.in_neighbors + inOff[N]);
    outOff.assign(d.base.out_offsets, d.base.out_offsets + N + 1);
    outNb.assign(d.base.out_neighbors, d.base.out_neighbors + outOff[N]);
    nodeIds.assign(d.node_ids, d.node_ids + N);
    nodeOffset.assign(d.node_offset, d.node_offset + N);
    reverse.assign(d.reverse, d.reverse + N);
    chainNumber.assign(d.chain_number, d.chain_number + N);
    chainApproxPos.assign(d.chain_approx_pos, d.chain_approx_pos + N);
    lookupIds.assign(d.lookup_ids, d.lookup_ids + d.num_lookup);
    originalSize.assign(d.original_size, d.original_size + d.num_lookup);
    lookupOff.assign(d.lookup_offsets, d.lookup_offsets + d.num_lookup + 1);
    lookupNodes.assign(d.lookup_nodes, d.lookup_nodes + lookupOff[d.num_lookup]);
    names.resize(d.num_lookup);
    for (size_t i = 0; i < d.num_lookup; i++)
    {
        if (d.names && d.names[i]) names[i] = d.names[i];
        lookupIndex[lookupIds[i]] = i;
    }
    bpSize = 0;
    for (uint32_t i = 0; i < N; i++) bpSize += len[i];
    // each split node's bigraph node size, so reversing a trace item needs no hash lookup
    bigSize.resize(N);
    for (uint32_t i = 0; i < N; i++)
    {
        auto f = lookupIndex.find(nodeIds[i]);
        bigSize[i] = f == lookupIndex.end() ? 0 : originalSize[f->second];
    }
}

size_t HostGraph::lookup(int bignode) const
{
    auto f = lookupIndex.find(bignode);
    GAH_ASSERT(f != lookupIndex.end());
    return f->second;
}

char HostGraph::charAt(size_t node, size_t pos) const
{
    GAH_ASSERT(node < N && pos < len[node]);
    if (node < firstAmbiguous)
    {
        uint64_t c = seq2[node * 2 + pos / 32];
        return "ACGT"[(c >> ((pos % 32) * 2)) & 3];
    }
    const uint64_t* a = &seqAmb[(node - firstAmbiguous) * 4];
    int m = 0;
    for (int k = 0; k < 4; k++) if ((a[k] >> pos) & 1) m |= 1 << k;
    static const char table[16] = { '?', 'A', 'C', 'M', 'G', 'R', 'S', 'V', 'T', 'W', 'Y', 'H', 'K', 'D', 'B', 'N' };
    return table[m];
}

// AlignmentGraph::GetUnitigNode (AlignmentGraph.cpp:812-828): the piece of the
// bigraph node that contains offset
size_t HostGraph::unitigNode(int bignode, size_t offset) const
{
    size_t i = lookup(bignode);
    GAH_ASSERT(offset < originalSize[i]);
    size_t lo = lookupOff[i], hi = lookupOff[i + 1];
    for (size_t k = lo; k < hi; k++)
    {
        size_t n = lookupNodes[k];
        if (nodeOffset[n] <= offset && nodeOffset[n] + len[n] > offset) return n;
    }
    GAH_ASSERT(false);
    return 0;
}

// AlignmentGraph::GetReversePosition (AlignmentGraph.cpp:830-847)
std::pair<int, size_t> HostGraph::reversePosition(int bignode, size_t offset) const
{
    size_t size = originalSize[lookup(bignode)];
    GAH_ASSERT(offset < size);
    int rev = (bignode % 2 == 0) ? (bignode / 2) * 2 + 1 : (bignode / 2) * 2;
    return { rev, size - offset - 1 };
}

size_t HostGraph::sizeOf(int bignode) const { return originalSize[lookup(bignode)]; }
const std::string& HostGraph::nameOf(int bignode) const { return names[lookup(bignode)]; }

// ------------------------------------------------------------------ seeds

// GraphAligner::orderSeedsByChaining (GraphAligner.h:250-312)
void orderSeeds(const HostGraph& g, std::vector<SeedHit>& seedHits)
{
    std::vector<size_t> chainOrder;
    std::unordered_map<size_t, std::vector<std::pair<size_t, size_t>>> seedPoses;
    for (size_t i = 0; i < seedHits.size(); i++)
    {
        int forwardNodeId = seedHits[i].reverse ? seedHits[i].nodeID * 2 + 1 : seedHits[i].nodeID * 2;
        size_t nodeIndex, realOffset;
        if (seedHits[i].alignmentGraphNodeId == std::numeric_limits<size_t>::max())
        {
            nodeIndex = g.unitigNode(forwardNodeId, seedHits[i].nodeOffset);
            GAH_ASSERT(seedHits[i].nodeOffset >= g.nodeOffset[nodeIndex]);
            realOffset = seedHits[i].nodeOffset - g.nodeOffset[nodeIndex];
        }
        else
        {
            nodeIndex = seedHits[i].alignmentGraphNodeId;
            realOffset = seedHits[i].alignmentGraphNodeOffset;
        }
        GAH_ASSERT(g.chainApproxPos[nodeIndex] + realOffset >= seedHits[i].seqPos);
        size_t chain = g.chainNumber[nodeIndex];
        auto found = seedPoses.find(chain);
        if (found == seedPoses.end())
        {
            chainOrder.push_back(chain);
            found = seedPoses.emplace(chain, std::vector<std::pair<size_t, size_t>>{}).first;
        }
        found->second.emplace_back(i, g.chainApproxPos[nodeIndex] + realOffset - seedHits[i].seqPos);
    }
    for (size_t chain : chainOrder)
    {
        auto& list = seedPoses[chain];
        std::sort(list.begin(), list.end(), [](std::pair<size_t, size_t> a, std::pair<size_t, size_t> b) { return a.second < b.second; });
        size_t clusterStart = 0;
        for (size_t i = 1; i <= list.size(); i++)
        {
            if (i < list.size() && list[i].second <= list[i - 1].second + 100) continue;
            std::sort(list.begin() + clusterStart, list.begin() + i, [&seedHits](std::pair<size_t, size_t> a, std::pair<size_t, size_t> b) { return seedHits[a.first].seqPos < seedHits[b.first].seqPos; });
            size_t matchingBps = 0;
            int lastEnd = std::numeric_limits<int>::min();
            for (size_t j = clusterStart; j < i; j++)
            {
                int thisStart = (int)seedHits[list[j].first].seqPos - (int)seedHits[list[j].first].matchLen + 1;
                int thisEnd = (int)seedHits[list[j].first].seqPos;
                GAH_ASSERT(thisEnd >= lastEnd);
                GAH_ASSERT(thisEnd > thisStart);
                matchingBps += (thisEnd - std::max(thisStart, lastEnd));
                lastEnd = thisEnd;
            }
            for (size_t j = clusterStart; j < i; j++)
            {
                seedHits[list[j].first].seedGoodness = matchingBps + seedHits[list[j].first].rawSeedGoodness;
                seedHits[list[j].first].seedClusterSize = i - clusterStart;
            }
            clusterStart = i;
        }
    }
    std::sort(seedHits.begin(), seedHits.end(), [](const SeedHit& a, const SeedHit& b) { return a.seedGoodness < b.seedGoodness; });
    std::reverse(seedHits.begin(), seedHits.end());
}

// ------------------------------------------------------------------ traces

// GraphAligner::fixForwardTraceSeqPos (GraphAligner.h:522-559)
void fixForwardTraceSeqPos(const HostGraph& g, OnewayTrace& trace, size_t start, const std::string& sequence)
{
    if (trace.trace.size() == 0) return;
    trace.score = 0;
    for (size_t i = 0; i < trace.trace.size(); i++)
    {
        auto& t = trace.trace[i];
        t.seqPos += start;
        size_t nodeIndex = t.node;
        t.node = g.nodeIds[nodeIndex];
        t.nodeOffset += g.nodeOffset[nodeIndex];
        GAH_ASSERT(t.seqPos < sequence.size());
        if (t.seqPos == start - 1)
        {
            GAH_ASSERT(t.seqChar == '-');
            t.seqChar = sequence[t.seqPos];
        }
        GAH_ASSERT(t.seqChar == sequence[t.seqPos]);
        if (i == 0 && !characterMatch(t.seqChar, t.graphChar)) trace.score += 1;
        if (i > 0)
        {
            const auto& p = trace.trace[i - 1];
            if (t.seqPos == p.seqPos) trace.score += 1;
            else if (!p.nodeSwitch && t.node == p.node && t.nodeOffset == p.nodeOffset) trace.score += 1;
            else if (!characterMatch(t.seqChar, t.graphChar)) trace.score += 1;
        }
    }
}

// GraphAligner::fixReverseTraceSeqPosAndOrder (GraphAligner.h:562-601)
// inReadOrder: the caller already put the trace in the order this function's reversal gives
void fixReverseTraceSeqPosAndOrder(const HostGraph& g, OnewayTrace& trace, size_t end, const std::string& sequence, bool inReadOrder)
{
    if (trace.trace.size() == 0) return;
    if (!inReadOrder) std::reverse(trace.trace.begin(), trace.trace.end());
    trace.score = 0;
    for (size_t i = 0; i + 1 < trace.trace.size(); i++) trace.trace[i].nodeSwitch = trace.trace[i + 1].nodeSwitch;
    trace.trace.back().nodeSwitch = false;
    for (size_t i = 0; i < trace.trace.size(); i++)
    {
        auto& t = trace.trace[i];
        GAH_ASSERT(t.seqPos <= end || t.seqPos == (size_t)-1);
        t.seqPos = end - t.seqPos;
        // reversePosition of the item's bigraph node and offset, its size from the split node
        const size_t offset = g.nodeOffset[t.node] + t.nodeOffset;
        const int bignode = g.nodeIds[t.node];
        const size_t size = g.bigSize[t.node];
        GAH_ASSERT(offset < size);
        t.node = (bignode % 2 == 0) ? (bignode / 2) * 2 + 1 : (bignode / 2) * 2;
        t.nodeOffset = size - offset - 1;
        GAH_ASSERT(t.seqPos < sequence.size());
        t.seqChar = sequence[t.seqPos];
        t.graphChar = complement(t.graphChar);
        if (i == 0 && !characterMatch(t.seqChar, t.graphChar)) trace.score += 1;
        if (i > 0)
        {
            const auto& p = trace.trace[i - 1];
            if (t.seqPos == p.seqPos) trace.score += 1;
            else if (!p.nodeSwitch && t.node == p.node && t.nodeOffset == p.nodeOffset) trace.score += 1;
            else if (!characterMatch(t.seqChar, t.graphChar)) trace.score += 1;
        }
    }
}

// GraphAligner::exactAlignmentPart (GraphAligner.h:403-457)
bool exactAlignmentPart(const AlignmentItem& aln, const SeedHit& seedHit)
{
    const auto& trace = aln.trace->trace;
    GAH_ASSERT(trace.size() > 0);
    GAH_ASSERT(trace.back().seqPos > trace[0].seqPos);
    if (trace.back().seqPos < seedHit.seqPos) return false;
    if (trace[0].seqPos > seedHit.seqPos) return false;
    size_t high = trace.size();
    size_t low = 0;
    size_t mid = (seedHit.seqPos - trace[0].seqPos) / (trace.back().seqPos - trace[0].seqPos);
    while (trace[mid].seqPos != seedHit.seqPos)
    {
        if (trace[mid].seqPos < seedHit.seqPos)
        {
            low = mid;
            mid = (high + low) / 2;
            if (mid == low) mid += 1;
            GAH_ASSERT(mid < trace.size());
        }
        if (trace[mid].seqPos > seedHit.seqPos)
        {
            high = mid;
            mid = (high + low) / 2;
            GAH_ASSERT(mid < trace.size());
        }
        GAH_ASSERT(low < mid);
        GAH_ASSERT(mid < high);
    }
    size_t down = mid;
    size_t compareNode = seedHit.nodeID * 2;
    if (seedHit.reverse) compareNode += 1;
    while (trace[down].seqPos == seedHit.seqPos)
    {
        if (compareNode == trace[down].node && seedHit.nodeOffset == trace[down].nodeOffset) return true;
        if (down == 0) break;
        down -= 1;
    }
    size_t up = mid;
    while (trace[up].seqPos == seedHit.seqPos)
    {
        if (compareNode == trace[up].node && seedHit.nodeOffset == trace[up].nodeOffset) return true;
        up += 1;
        if (up == trace.size()) break;
    }
    return false;
}

// ------------------------------------------------------------------ selection, GAF

// AlignmentSelection::alignmentIncompatible (AlignmentSelection.cpp:13-29)
static bool alignmentIncompatible(const AlignmentItem& l, const AlignmentItem& r)
{
    const float OverlapIncompatibleFractionCutoff = 0.05;
    auto minOverlapLen = std::min((l.alignmentEnd - l.alignmentStart), (r.alignmentEnd - r.alignmentStart)) * OverlapIncompatibleFractionCutoff;
    size_t leftStart = l.alignmentStart, leftEnd = l.alignmentEnd, rightStart = r.alignmentStart, rightEnd = r.alignmentEnd;
    if (leftStart > rightStart)
    {
        std::swap(leftStart, rightStart);
        std::swap(leftEnd, rightEnd);
    }
    int overlap = 0;
    if (leftEnd > rightStart) overlap = leftEnd - rightStart;
    return overlap > minOverlapLen;
}

// AlignmentSelection::SelectAlignments (AlignmentSelection.cpp:31-95) without the E-value filter
std::vector<AlignmentItem> selectAlignments(const std::vector<AlignmentItem>& all, int minAlignmentScore, double fractionCutoff)
{
    std::vector<AlignmentItem> filtered;
    bool wasFiltered = false;
    if (minAlignmentScore > std::numeric_limits<int>::min())
    {
        std::vector<AlignmentItem> r;
        for (const auto& a : all) if (a.alignmentXScore >= (double)minAlignmentScore) r.push_back(a);
        filtered = r;
        wasFiltered = true;
    }
    if (fractionCutoff != 0)
    {
        const std::vector<AlignmentItem>& in = wasFiltered ? filtered : all;
        std::vector<AlignmentItem> r;
        for (size_t i = 0; i < in.size(); i++)
        {
            bool skipped = false;
            for (size_t j = 0; j < in.size(); j++)
            {
                if (i == j) continue;
                if (!alignmentIncompatible(in[i], in[j])) continue;
                if (in[i].alignmentXScore < in[j].alignmentXScore * fractionCutoff)
                {
                    skipped = true;
                    break;
                }
            }
            if (!skipped) r.push_back(in[i]);
        }
        filtered = r;
        wasFiltered = true;
    }
    return wasFiltered ? filtered : all;
}

static void addPos(std::stringstream& s, int nodeId, bool reverse, const HostGraph& g)
{
    s << (reverse ? "<" : ">");
    const std::string& name = g.nameOf(nodeId);
    if (name == "") s << nodeId / 2;
    else s << name;
}

// GraphAlignerGAFAlignment::addCigarItem (GraphAlignerGAFAlignment.h:225-250)
static void addCigarItem(std::stringstream& s, size_t editLength, int type)
{
    if (editLength == 0) return;
    static const char codes[] = { '=', 'X', 'M', 'I', 'D' };
    s << editLength;
    if (type >= 0 && type <= 4) s << codes[type];
}

// GraphAlignerGAFAlignment::traceToAlignment (GraphAlignerGAFAlignment.h:37-200)
std::string gafLine(const HostGraph& g, const std::string& readName, const std::string& sequence, const OnewayTrace& t,
    double alignmentXScore, int mappingQuality, bool cigarMatchMismatchMerge)
{
    enum { Match = 0, Mismatch = 1, MatchOrMismatch = 2, Insertion = 3, Deletion = 4, Empty = 5 };
    const auto& trace = t.trace;
    GAH_ASSERT(trace.size() > 0);
    std::stringstream cigar;
    size_t readLen = sequence.size();
    size_t readStart = trace[0].seqPos;
    size_t readEnd = trace.back().seqPos + 1;
    std::stringstream nodePath;
    size_t nodePathLen = 0;
    size_t nodePathStart = trace[0].nodeOffset;
    size_t nodePathEnd = 0;
    size_t matches = 0, mismatches = 0, deletions = 0, insertions = 0, editLength = 0;
    size_t blockLength = trace.size();
    int curNode = (int)trace[0].node;
    bool curRev = (trace[0].node % 2) == 1;
    size_t curOffset = trace[0].nodeOffset;
    size_t curSeq = trace[0].seqPos;
    int currentEdit = Empty;
    if (cigarMatchMismatchMerge)
    {
        currentEdit = MatchOrMismatch;
        editLength = 1;
        if (characterMatch(trace[0].seqChar, trace[0].graphChar)) matches++; else mismatches++;
    }
    else if (characterMatch(trace[0].seqChar, trace[0].graphChar))
    {
        currentEdit = Match;
        editLength = 1;
        matches++;
    }
    else
    {
        currentEdit = Mismatch;
        editLength = 1;
        mismatches++;
    }
    addPos(nodePath, curNode, curRev, g);
    nodePathLen += g.sizeOf(curNode);
    for (size_t pos = 1; pos < trace.size(); pos++)
    {
        GAH_ASSERT(trace[pos].seqPos < sequence.size());
        int newNode = (int)trace[pos].node;
        bool newRev = (trace[pos].node % 2) == 1;
        size_t newOffset = trace[pos].nodeOffset;
        size_t newSeq = trace[pos].seqPos;
        bool insideNode = !trace[pos - 1].nodeSwitch || (newNode == curNode && newRev == curRev && newOffset > curOffset);
        GAH_ASSERT(newSeq >= curSeq);
        if (!insideNode)
        {
            size_t skippedBefore = g.sizeOf(curNode) - 1 - trace[pos - 1].nodeOffset;
            curNode = newNode;
            curRev = newRev;
            curOffset = newOffset;
            curSeq = newSeq;
            addPos(nodePath, curNode, curRev, g);
            GAH_ASSERT(trace[pos].nodeOffset < g.sizeOf(curNode));
            size_t skippedAfter = trace[pos].nodeOffset;
            nodePathLen += g.sizeOf(curNode) - (skippedBefore + skippedAfter);
        }
        auto step = [&](int type)
        {
            if (currentEdit == Empty) currentEdit = type;
            if (currentEdit != type)
            {
                addCigarItem(cigar, editLength, currentEdit);
                currentEdit = type;
                editLength = 0;
            }
            editLength += 1;
        };
        if (trace[pos - 1].seqPos == trace[pos].seqPos)
        {
            step(Deletion);
            deletions++;
        }
        else if (insideNode && trace[pos - 1].nodeOffset == trace[pos].nodeOffset)
        {
            step(Insertion);
            insertions++;
        }
        else if (cigarMatchMismatchMerge)
        {
            step(MatchOrMismatch);
            if (characterMatch(trace[pos].seqChar, trace[pos].graphChar)) matches++; else mismatches++;
        }
        else if (characterMatch(trace[pos].seqChar, trace[pos].graphChar))
        {
            step(Match);
            matches++;
        }
        else
        {
            step(Mismatch);
            mismatches++;
        }
    }
    GAH_ASSERT(matches + mismatches + deletions + insertions == trace.size());
    addCigarItem(cigar, editLength, currentEdit);
    nodePathEnd = nodePathLen - (g.sizeOf((int)trace.back().node) - 1 - trace.back().nodeOffset);
    std::stringstream s;
    s << readName << "\t" << readLen << "\t" << readStart << "\t" << readEnd << "\t" << "+" << "\t" << nodePath.str() << "\t" << nodePathLen << "\t" << nodePathStart << "\t" << nodePathEnd << "\t" << matches << "\t" << blockLength << "\t" << mappingQuality;
    s << "\t" << "NM:i:" << (mismatches + deletions + insertions);
    if (alignmentXScore != -1) s << "\t" << "AS:f:" << alignmentXScore;
    s << "\t" << "dv:f:" << 1.0 - ((double)matches / (double)(matches + mismatches + deletions + insertions));
    s << "\t" << "id:f:" << ((double)matches / (double)(matches + mismatches + deletions + insertions));
    s << "\t" << "cg:Z:" << cigar.str();
    return s.str();
}

// ------------------------------------------------------------------ the batched seed loop

struct ReadState
{
    std::string name;
    std::string seq;
    std::string rev;
    std::vector<SeedHit> seeds;
    size_t next = 0;
    size_t extendSeeds = 0;
    size_t seedScoreForEndToEndAln = 0;
    size_t worstExtendedSeedScore = 0;
    size_t seedsExtended = 0;
    std::vector<AlignmentItem> alignments;
    bool done = false;
    bool failed = false;
};

// advances a read's seed loop (GraphAligner.h:105-154) to the next seed that needs an
// extension; returns false when the loop ends
// the loop's cursor: the next seed to look at and the two counters that extending changes
struct SeedCursor
{
    size_t next;
    size_t worstExtendedSeedScore;
    size_t seedsExtended;
};

static bool nextSeedOn(const ReadAlignParams& p, const ReadState& r, SeedCursor& c, size_t& seedIndex)
{
    while (c.next < r.seeds.size())
    {
        const size_t i = c.next;
        const SeedHit& s = r.seeds[i];
        if (p.sloppy && (s.seedGoodness == r.seedScoreForEndToEndAln || s.seedGoodness < r.seedScoreForEndToEndAln)) return false;
        if (c.seedsExtended >= r.extendSeeds && s.seedGoodness < c.worstExtendedSeedScore) return false;
        c.next++;
        if (s.seedClusterSize < p.minClusterSize) continue;
        if (p.sloppy)
        {
            bool found = false;
            for (const auto& aln : r.alignments)
            {
                if (aln.alignmentStart <= s.seqPos && aln.alignmentEnd >= s.seqPos && aln.seedGoodness > s.seedGoodness)
                {
                    found = true;
                    break;
                }
            }
            if (found) continue;
        }
        bool found = false;
        for (const auto& aln : r.alignments)
        {
            if (exactAlignmentPart(aln, s))
            {
                found = true;
                break;
            }
        }
        if (found) continue;
        c.worstExtendedSeedScore = s.seedGoodness;
        c.seedsExtended += 1;
        seedIndex = i;
        return true;
    }
    return false;
}

static bool nextSeed(const ReadAlignParams& p, ReadState& r, size_t& seedIndex)
{
    SeedCursor c { r.next, r.worstExtendedSeedScore, r.seedsExtended };
    const bool more = nextSeedOn(p, r, c, seedIndex);
    r.next = c.next;
    r.worstExtendedSeedScore = c.worstExtendedSeedScore;
    r.seedsExtended = c.seedsExtended;
    return more;
}

// The packed items of an extension as trace items, in DP order or (reversed) read order;
// `extra` more items of room are kept for a trace that will be appended.
static OnewayTrace decodeTrace(const HostGraph& g, const ExtensionResult& e, const char* seq, size_t seqLen, bool reversed = false,
    size_t extra = 0)
{
    OnewayTrace t;
    if (e.status == GA_TRACE_FAILED)
    {
        t.score = INT32_MAX;
        return t;
    }
    GAH_ASSERT(e.status == GA_OK);
    t.score = e.score;
    const uint64_t* items = e.begin();
    const uint64_t n = e.size();
    t.trace.reserve(n + extra);
    t.trace.resize(n);
    for (uint64_t i = 0; i < n; i++)
    {
        const uint64_t x = items[i];
        TraceItem& it = t.trace[reversed ? n - 1 - i : i];
        it.node = GA_TRACE_NODE(x);
        it.nodeOffset = GA_TRACE_OFFSET(x);
        uint64_t sp1 = GA_TRACE_SEQPOS1(x);
        it.seqPos = sp1 == 0 ? (size_t)-1 : (size_t)(sp1 - 1);
        it.nodeSwitch = GA_TRACE_SWITCH(x) != 0;
        it.seqChar = it.seqPos < seqLen ? seq[it.seqPos] : '-';
        it.graphChar = g.charAt(it.node, it.nodeOffset);
    }
    return t;
}

void parallelFor(size_t n, const std::function<void(size_t)>& fn)
{
    static const size_t hw = std::max<size_t>(1, std::min<size_t>(64, std::thread::hardware_concurrency()));
    const size_t threads = std::min(hw, n / 8);
    if (threads <= 1)
    {
        for (size_t i = 0; i < n; i++) fn(i);
        return;
    }
    std::atomic<size_t> next(0);
    auto work = [&]()
    {
        while (true)
        {
            const size_t i = next.fetch_add(1);
            if (i >= n) break;
            fn(i);
        }
    };
    std::vector<std::thread> pool;
    for (size_t t = 1; t < threads; t++) pool.emplace_back(work);
    work();
    for (auto& t : pool) t.join();
}

// GraphAligner::getAlignmentFromSeed (GraphAligner.h:631-692) after the two extensions ran.
// The backward trace comes in DP order and the forward one already reversed (decodeTrace),
// so neither is reversed here: getTwoDirectionalTrace (GraphAligner.h:508-518) reverses the
// backward trace and fixReverseTraceSeqPosAndOrder reverses it back, and the forward trace
// is reversed once.
static void finishSeed(const HostGraph& g, const ReadAlignParams& p, ReadState& r, const SeedHit& seedHit,
    OnewayTrace backward, OnewayTrace forward, int backwardNodeId, int forwardNodeId)
{
    if (!backward.failed())
    {
        auto rp = g.reversePosition(forwardNodeId, seedHit.nodeOffset);
        const auto& b = backward.trace.back();
        GAH_ASSERT(b.seqPos == (size_t)-1 && g.nodeIds[b.node] == backwardNodeId && g.nodeOffset[b.node] + b.nodeOffset == rp.second);
    }
    if (!forward.failed())
    {
        const auto& b = forward.trace.front();
        GAH_ASSERT(b.seqPos == (size_t)-1 && g.nodeIds[b.node] == forwardNodeId && g.nodeOffset[b.node] + b.nodeOffset == seedHit.nodeOffset);
    }
    fixReverseTraceSeqPosAndOrder(g, backward, seedHit.seqPos - 1, r.seq, true);
    fixForwardTraceSeqPos(g, forward, seedHit.seqPos + 1, r.seq);
    if (forward.failed() && backward.failed()) return;
    GAH_ASSERT(backward.trace.size() > 0 || backward.failed());
    OnewayTrace merged = std::move(backward);
    if (merged.failed())
    {
        merged = std::move(forward);
    }
    else if (!forward.failed())
    {
        GAH_ASSERT(merged.trace.size() > 0);
        const auto& a = merged.trace.back();
        const auto& b = forward.trace[0];
        GAH_ASSERT(a.node == b.node && a.nodeOffset == b.nodeOffset && a.seqPos == b.seqPos);
        merged.trace.pop_back();
        merged.trace.insert(merged.trace.end(), forward.trace.begin(), forward.trace.end());
        merged.score += forward.score;
    }
    AlignmentItem item;
    item.trace = std::make_shared<OnewayTrace>(std::move(merged));
    GAH_ASSERT(item.trace->trace.size() > 0);
    item.alignmentScore = item.trace->score;
    item.alignmentStart = item.trace->trace[0].seqPos;
    item.alignmentEnd = item.trace->trace.back().seqPos + 1;
    GAH_ASSERT(item.alignmentEnd - 1 < r.seq.size());
    item.alignmentXScore = (int32_t)(item.alignmentEnd - item.alignmentStart) * 100 - p.xscoreErrorCost * (int32_t)item.alignmentScore;
    item.alignmentXScore /= 100.0;
    if (item.alignmentEnd == item.alignmentStart) return;
    item.seedGoodness = seedHit.seedGoodness;
    r.alignments.push_back(item);
    if (p.sloppy)
    {
        std::sort(r.alignments.begin(), r.alignments.end(), [](const AlignmentItem& a, const AlignmentItem& b) { return a.alignmentStart < b.alignmentStart; });
        if (r.alignments[0].alignmentStart == 0)
        {
            size_t minSeedGoodness = r.alignments[0].seedGoodness;
            size_t contiguousEnd = r.alignments[0].alignmentEnd;
            for (size_t i = 1; i < r.alignments.size(); i++)
            {
                if (r.alignments[i].alignmentStart <= contiguousEnd)
                {
                    minSeedGoodness = std::min(minSeedGoodness, r.alignments[i].seedGoodness);
                    contiguousEnd = std::max(contiguousEnd, r.alignments[i].alignmentEnd);
                }
            }
            if (contiguousEnd == r.seq.size()) r.seedScoreForEndToEndAln = minSeedGoodness;
        }
    }
}

// Aligner.cpp:505-548: selection (the kept ones of keep, when given), bp aligned, order by
// X-score; the lines to write in `lines`
static void finalizeSelect(const ReadAlignParams& p, ReadState& r, ReadOutput& o, std::vector<AlignmentItem>& lines, const char* keep = nullptr)
{
    lines.clear();
    if (r.failed)
    {
        o.failed = true;
        return;
    }
    if (r.alignments.empty()) return;
    try
    {
        std::vector<AlignmentItem> alns;
        if (keep)
        {
            for (size_t k = 0; k < r.alignments.size(); k++)
                if (keep[k]) alns.push_back(r.alignments[k]);
        }
        else alns = selectAlignments(r.alignments, p.minAlignmentScore, p.multimapScoreFraction);
        if (alns.empty()) return;
        std::sort(alns.begin(), alns.end(), [](const AlignmentItem& a, const AlignmentItem& b) { return a.alignmentStart < b.alignmentStart; });
        size_t bpAligned = 0, lastEnd = 0;
        for (const auto& a : alns)
        {
            size_t countStart = std::max(lastEnd, a.alignmentStart);
            if (a.alignmentEnd > countStart)
            {
                bpAligned += a.alignmentEnd - countStart;
                lastEnd = a.alignmentEnd;
            }
        }
        std::sort(alns.begin(), alns.end(), [](const AlignmentItem& a, const AlignmentItem& b) { return a.alignmentXScore > b.alignmentXScore; });
        o.bpAligned = bpAligned;
        o.alignments = alns.size();
        lines = std::move(alns);
    }
    catch (const ReadFailure&)
    {
        o.failed = true;
        o.bpAligned = 0;
        o.alignments = 0;
        lines.clear();
    }
}

static void failOutput(ReadOutput& o);

// finalizeSelect for a group of finished reads, the selection by the hook when one is set
static void finalizeGroup(const ReadAlignParams& p, const std::vector<ReadState*>& rs, const std::vector<ReadOutput*>& os,
    std::vector<std::vector<AlignmentItem>>& lines, bool hostSelect = false)
{
    const size_t n = rs.size();
    lines.assign(n, {});
    if (!p.select || hostSelect)
    {
        parallelFor(n, [&](size_t i) { finalizeSelect(p, *rs[i], *os[i], lines[i]); });
        return;
    }
    std::vector<uint64_t> first(n + 1, 0), start, end;
    std::vector<double> xscore;
    for (size_t i = 0; i < n; i++)
    {
        if (!rs[i]->failed)
            for (const auto& a : rs[i]->alignments)
            {
                start.push_back(a.alignmentStart);
                end.push_back(a.alignmentEnd);
                xscore.push_back(a.alignmentXScore);
            }
        first[i + 1] = start.size();
    }
    std::vector<char> keep(start.size(), 0);
    if (!start.empty() && !p.select(p.selectCtx, first, start, end, xscore, p.minAlignmentScore, p.multimapScoreFraction, keep))
    {
        for (size_t i = 0; i < n; i++)
        {
            rs[i]->failed = true;
            failOutput(*os[i]);
        }
        return;
    }
    parallelFor(n, [&](size_t i) { finalizeSelect(p, *rs[i], *os[i], lines[i], keep.data() + first[i]); });
}

static void failOutput(ReadOutput& o)
{
    o.failed = true;
    o.gaf.clear();
    o.bpAligned = 0;
    o.alignments = 0;
}

// Aligner.cpp:549-566: the GAF lines of finished reads.  Without a writer hook, gafLine on the
// host's cores; with one, each line's trace is walked on the host's cores (gaf::classify_line)
// into the read's pending lines, and the hook writes the text (at once, or later through
// writeFinished when `write` is false).
static void formatFinished(const HostGraph& g, const ReadAlignParams& p, const std::vector<ReadState*>& rs, const std::vector<ReadOutput*>& os,
    const std::vector<std::vector<AlignmentItem>>& lines, bool write = true)
{
    const size_t n = rs.size();
    if (!p.gafWrite)
    {
        parallelFor(n, [&](size_t i)
        {
            if (lines[i].empty()) return;
            try
            {
                std::string text;
                for (const auto& a : lines[i])
                {
                    text += gafLine(g, rs[i]->name, rs[i]->seq, *a.trace, a.alignmentXScore, a.mappingQuality, p.cigarMatchMismatchMerge);
                    text += '\n';
                }
                os[i]->gaf = std::move(text);
            }
            catch (const ReadFailure&)
            {
                failOutput(*os[i]);
            }
        });
        return;
    }
    auto sizeOf = [&g](int32_t bignode) -> uint64_t
    {
        auto f = g.lookupIndex.find(bignode);
        return f == g.lookupIndex.end() ? 0 : g.originalSize[f->second];
    };
    parallelFor(n, [&](size_t i)
    {
        if (lines[i].empty()) return;
        ClassifiedLines& c = os[i]->pending;
        size_t items = 0;
        for (const auto& a : lines[i]) items += a.trace->trace.size();
        c.lines.resize(lines[i].size());
        c.ops.resize(items);
        c.entries.clear();
        std::vector<int32_t> entries;
        uint64_t op = 0;
        for (size_t k = 0; k < lines[i].size(); k++)
        {
            const AlignmentItem& a = lines[i][k];
            const auto& t = a.trace->trace;
            auto item = [&t](uint32_t q) -> gaf::Item
            {
                const TraceItem& x = t[q];
                return gaf::Item { (int32_t)x.node, (uint32_t)x.nodeOffset, (uint32_t)x.seqPos, (uint8_t)(x.nodeSwitch ? 1 : 0),
                    (uint8_t)x.seqChar, (uint8_t)x.graphChar, 0 };
            };
            entries.resize(std::max<size_t>(t.size(), 1));
            gaf::LineMeta& m = c.lines[k];
            if (!gaf::classify_line(item, (uint32_t)t.size(), (uint32_t)rs[i]->seq.size(), p.cigarMatchMismatchMerge, sizeOf, m, c.ops.data() + op,
                    entries.data()))
            {
                c = ClassifiedLines {};
                failOutput(*os[i]);
                return;
            }
            m.op = op;
            m.entry = c.entries.size();
            m.read = 0;
            m.xscore100 = (int32_t)std::llround(a.alignmentXScore * 100);
            m.mapq = a.mappingQuality;
            c.entries.insert(c.entries.end(), entries.begin(), entries.begin() + m.entries);
            op += t.size();
        }
    });
    if (!write) return;
    std::vector<const std::string*> names;
    std::vector<const ClassifiedLines*> reads;
    std::vector<size_t> which;
    for (size_t i = 0; i < n; i++)
    {
        if (os[i]->pending.lines.empty()) continue;
        names.push_back(&rs[i]->name);
        reads.push_back(&os[i]->pending);
        which.push_back(i);
    }
    if (reads.empty()) return;
    std::string text;
    std::vector<uint64_t> readEnd;
    const bool ok = p.gafWrite(p.gafCtx, names, reads, text, readEnd);
    parallelFor(which.size(), [&](size_t k)
    {
        ReadOutput& o = *os[which[k]];
        if (!ok)
        {
            failOutput(o);
        }
        else
        {
            const uint64_t from = k == 0 ? 0 : readEnd[k - 1];
            o.gaf.assign(text.data() + from, readEnd[k] - from);
        }
        o.pending = ClassifiedLines {};
    });
}

void writeFinished(const ReadAlignParams& p, std::vector<std::pair<uint64_t, ReadOutput>>& outs, const std::vector<const std::string*>& names)
{
    if (!p.gafWrite) return;
    std::vector<const std::string*> nm;
    std::vector<const ClassifiedLines*> reads;
    std::vector<size_t> which;
    for (size_t i = 0; i < outs.size(); i++)
    {
        if (outs[i].second.pending.lines.empty()) continue;
        nm.push_back(names[i]);
        reads.push_back(&outs[i].second.pending);
        which.push_back(i);
    }
    if (reads.empty()) return;
    std::string text;
    std::vector<uint64_t> readEnd;
    const bool ok = p.gafWrite(p.gafCtx, nm, reads, text, readEnd);
    parallelFor(which.size(), [&](size_t k)
    {
        ReadOutput& o = outs[which[k]].second;
        if (!ok)
        {
            failOutput(o);
        }
        else
        {
            const uint64_t from = k == 0 ? 0 : readEnd[k - 1];
            o.gaf.assign(text.data() + from, readEnd[k] - from);
        }
        o.pending = ClassifiedLines {};
    });
}

// ------------------------------------------------------------------ multiseed DP

void prepareMultiseeds(const HostGraph& g, const std::vector<SeedHit>& seeds, size_t seqLen, std::vector<uint32_t>& slices,
    std::vector<uint32_t>& nodes)
{
    slices.clear();
    nodes.clear();
    std::vector<std::unordered_set<size_t>> actives((seqLen + 64 + 1) / 64);
    for (const auto& seed : seeds)
    {
        const size_t sliceIndex = seed.seqPos / 64;
        GAH_ASSERT(sliceIndex < actives.size());
        size_t nodeId = seed.alignmentGraphNodeId;
        if (nodeId == SIZE_MAX)
        {
            const int forwardNodeId = seed.reverse ? seed.nodeID * 2 + 1 : seed.nodeID * 2;
            nodeId = g.unitigNode(forwardNodeId, seed.nodeOffset);
        }
        actives[sliceIndex].insert(nodeId);
    }
    for (size_t i = 0; i < actives.size(); i++)
    {
        for (size_t nodeId : actives[i])
        {
            slices.push_back((uint32_t)i);
            nodes.push_back((uint32_t)nodeId);
        }
    }
}

void addMappingQualities(std::vector<AlignmentItem>& alignments)
{
    for (size_t i = 0; i < alignments.size(); i++)
    {
        double otherSum = 0;
        for (size_t j = 0; j < alignments.size(); j++)
        {
            if (i == j) continue;
            if (!alignmentIncompatible(alignments[i], alignments[j])) continue;
            if (alignments[j].alignmentXScore >= alignments[i].alignmentXScore + 1)
            {
                otherSum += 10;
                break;
            }
            otherSum += pow(10.0, alignments[j].alignmentXScore - alignments[i].alignmentXScore);
            if (otherSum >= 10) break;
        }
        if (otherSum >= 10) alignments[i].mappingQuality = 0;
        else if (otherSum <= 0.000001) alignments[i].mappingQuality = 60;
        else
        {
            alignments[i].mappingQuality = -log(1.0 - 1.0 / (1.0 + otherSum)) * 10;
            if (alignments[i].mappingQuality >= 60) alignments[i].mappingQuality = 60;
        }
    }
}

// int32 value of a size_t expression, as the reference's ScoreType assignments truncate it
static inline int32_t score32(uint64_t x) { return (int32_t)(uint32_t)x; }

// removeDuplicateTraces on the packed traces of one multiseed DP, before any is decoded
// (trace_dedupe.h); the first item is the trace's end in DP order, the last its start, whose
// cell and read position without the switch flag identify it.  Returns the surviving
// traces' indices in their final order.
static std::vector<uint32_t> dedupeMultiseedTraces(const MultiseedResult& res, int32_t cost)
{
    const uint64_t kSwitch = 1ULL << 38;
    std::vector<DedupeKey> keys(res.items.size());
    for (size_t t = 0; t < keys.size(); t++)
    {
        const uint64_t* it = res.items[t];
        const uint64_t n = res.lengths[t];
        GAH_ASSERT(n > 0);
        auto seqPos = [](uint64_t x) -> size_t { const uint64_t sp1 = GA_TRACE_SEQPOS1(x); return sp1 == 0 ? (size_t)-1 : (size_t)(sp1 - 1); };
        keys[t] = DedupeKey { dedupeScore(seqPos(it[0]), seqPos(it[n - 1]), res.scores[t], cost), (uint32_t)t, it[n - 1] & ~kSwitch };
    }
    return dedupeOrder(keys);
}

// GraphAligner::clipTraceStart (GraphAligner.h:702-738): the trace starts where its X-score
// counted from the end is highest
static void clipTraceStart(OnewayTrace& trace, int32_t cost)
{
    if (trace.trace.empty()) return;
    int32_t maxX = INT32_MIN;
    size_t maxXIndex = SIZE_MAX;
    size_t score = 0;
    size_t maxXScore = 0;
    const size_t n = trace.trace.size();
    for (size_t i = n - 1; i < n; i--)
    {
        const auto& t = trace.trace[i];
        const bool posSwitch = (i == n - 1) || t.nodeSwitch || t.nodeOffset != trace.trace[i + 1].nodeOffset || t.node != trace.trace[i + 1].node;
        if (i != n - 1 && trace.trace[i + 1].seqPos == t.seqPos) score += 1;
        else if (i != n - 1 && !posSwitch) score += 1;
        else if (!characterMatch(t.seqChar, t.graphChar)) score += 1;
        const int32_t xHere = score32((trace.trace.back().seqPos - t.seqPos + 1) * 100 - score * (uint64_t)(int64_t)cost);
        if (xHere > maxX)
        {
            maxX = xHere;
            maxXIndex = i;
            maxXScore = score;
        }
    }
    GAH_ASSERT(maxXIndex < n);
    if (maxXIndex > 0)
    {
        trace.score = (int32_t)maxXScore;
        trace.trace.erase(trace.trace.begin(), trace.trace.begin() + maxXIndex);
    }
}

// GraphAligner::mergeTraces (GraphAligner.h:316-345)
static OnewayTrace mergeTraces(OnewayTrace&& bw, OnewayTrace&& fw)
{
    GAH_ASSERT(!fw.failed() || !bw.failed());
    OnewayTrace merged;
    if (!bw.failed())
    {
        GAH_ASSERT(!bw.trace.empty());
        merged = std::move(bw);
        if (!fw.failed())
        {
            GAH_ASSERT(!merged.trace.empty() && !fw.trace.empty());
            const auto& a = merged.trace.back();
            const auto& b = fw.trace[0];
            GAH_ASSERT(a.node == b.node && a.nodeOffset == b.nodeOffset && a.seqPos == b.seqPos);
            if (!characterMatch(b.seqChar, b.graphChar))
            {
                GAH_ASSERT(merged.score >= 1 && fw.score >= 1);
                fw.score -= 1;
            }
            merged.trace.pop_back();
            merged.trace.insert(merged.trace.end(), fw.trace.begin(), fw.trace.end());
            merged.score += fw.score;
        }
    }
    else if (!fw.failed())
    {
        merged = std::move(fw);
    }
    return merged;
}

void alignBatchMultiseed(const HostGraph& g, const ReadAlignParams& p, std::vector<ReadInput>& reads, MultiseedFn multiseed, void* msCtx,
    ExtendFn extend, void* ctx, std::vector<ReadOutput>& out, BatchStats& stats)
{
    const size_t n = reads.size();
    out.assign(n, ReadOutput {});
    auto t0 = std::chrono::steady_clock::now();
    struct MsRead
    {
        ReadState r;
        std::vector<uint32_t> slices, nodes;
        std::vector<OnewayTrace> forward;     // clipped, read order, bigraph positions
        std::vector<int> backwardRequest;     // per forward trace: index in the backward batch, or -1
    };
    std::vector<MsRead> ms(n);
    parallelFor(n, [&](size_t i)
    {
        MsRead& m = ms[i];
        m.r.name = std::move(reads[i].name);
        m.r.seq = std::move(reads[i].seq);
        if (reads[i].seeds.empty())
        {
            out[i].noSeeds = true;
            m.r.done = true;
            return;
        }
        m.r.rev = reverseComplement(m.r.seq);
        try
        {
            prepareMultiseeds(g, reads[i].seeds, m.r.seq.size(), m.slices, m.nodes);
        }
        catch (const ReadFailure&)
        {
            m.r.failed = true;
        }
    });
    // the multiseed DP of every read with seeds
    std::vector<MultiseedRequest> rq;
    std::vector<size_t> rqRead;
    for (size_t i = 0; i < n; i++)
    {
        if (ms[i].r.done || ms[i].r.failed) continue;
        rq.push_back(MultiseedRequest { ms[i].r.seq.data(), (uint32_t)ms[i].r.seq.size(), ms[i].slices.data(), ms[i].nodes.data(), (uint32_t)ms[i].nodes.size() });
        rqRead.push_back(i);
    }
    std::vector<MultiseedResult> rs(rq.size());
    stats.collectMs += std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
    if (!rq.empty()) multiseed(msCtx, rq, rs);
    stats.rounds += 1;
    stats.extensions += rq.size();
    t0 = std::chrono::steady_clock::now();
    // duplicate removal, read order, clipping, and the backward extension of every trace
    // that does not start at the read's first base.  Duplicates go before any trace is
    // decoded; the survivors are decoded, reversed and clipped one trace per job (a read can
    // have thousands), then each read lists its backward extensions in trace order.
    std::vector<std::vector<ExtensionRequest>> perRead(rq.size());
    std::vector<std::vector<uint32_t>> keep(rq.size());
    parallelFor(rq.size(), [&](size_t k)
    {
        MsRead& m = ms[rqRead[k]];
        if (rs[k].status != GA_OK)
        {
            m.r.failed = true;
            return;
        }
        try
        {
            if (rs[k].deduplicated)
            {
                keep[k].resize(rs[k].items.size());
                for (uint32_t t = 0; t < keep[k].size(); t++) keep[k][t] = t;
            }
            else keep[k] = dedupeMultiseedTraces(rs[k], p.xscoreErrorCost);
            m.forward.resize(keep[k].size());
        }
        catch (const ReadFailure&)
        {
            m.r.failed = true;
            keep[k].clear();
        }
    });
    std::vector<std::pair<uint32_t, uint32_t>> jobs;     // (read, trace in its final order)
    for (size_t k = 0; k < rq.size(); k++)
        for (uint32_t q = 0; q < keep[k].size(); q++) jobs.emplace_back((uint32_t)k, q);
    std::unique_ptr<std::atomic<uint8_t>[]> broken(new std::atomic<uint8_t>[rq.size()]);
    for (size_t k = 0; k < rq.size(); k++) broken[k].store(0);
    parallelFor(jobs.size(), [&](size_t job)
    {
        const uint32_t k = jobs[job].first, q = jobs[job].second;
        if (broken[k].load(std::memory_order_relaxed)) return;
        MsRead& m = ms[rqRead[k]];
        const MultiseedResult& res = rs[k];
        const uint32_t t = keep[k][q];
        try
        {
            ExtensionResult e;
            e.status = GA_OK;
            e.score = res.scores[t];
            e.itemPtr = res.items[t];
            e.itemCount = res.lengths[t];
            OnewayTrace tr = decodeTrace(g, e, m.r.seq.data(), m.r.seq.size());
            std::reverse(tr.trace.begin(), tr.trace.end());
            clipTraceStart(tr, p.xscoreErrorCost);
            fixForwardTraceSeqPos(g, tr, 0, m.r.seq);
            m.forward[q] = std::move(tr);
        }
        catch (const ReadFailure&)
        {
            broken[k].store(1);
        }
    });
    parallelFor(rq.size(), [&](size_t k)
    {
        MsRead& m = ms[rqRead[k]];
        if (m.r.failed) return;
        if (broken[k].load())
        {
            m.r.failed = true;
            m.forward.clear();
            return;
        }
        for (const OnewayTrace& t : m.forward)
        {
            int request = -1;
            if (t.trace[0].seqPos != 0)
            {
                auto rp = g.reversePosition((int)t.trace[0].node, t.trace[0].nodeOffset);
                ExtensionRequest e;
                e.seq = m.r.rev.data() + m.r.rev.size() - t.trace[0].seqPos;
                e.len = (uint32_t)t.trace[0].seqPos;
                e.bignode = rp.first;
                e.offset = rp.second;
                const size_t node = g.unitigNode(e.bignode, e.offset);
                e.node = (uint32_t)node;
                e.nodeOffset = (uint32_t)(e.offset - g.nodeOffset[node]);
                request = (int)perRead[k].size();
                perRead[k].push_back(e);
            }
            m.backwardRequest.push_back(request);
        }
    });
    for (const auto& res : rs) stats.cellSteps += res.steps;
    std::vector<ExtensionRequest> bq;
    std::vector<size_t> firstRequest(rq.size());
    for (size_t k = 0; k < rq.size(); k++)
    {
        firstRequest[k] = bq.size();
        bq.insert(bq.end(), perRead[k].begin(), perRead[k].end());
    }
    std::vector<ExtensionResult> br(bq.size());
    stats.consumeMs += std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
    if (!bq.empty()) extend(ctx, bq, br);
    stats.rounds += 1;
    stats.extensions += bq.size();
    for (const auto& e : br) stats.cellSteps += e.steps;
    t0 = std::chrono::steady_clock::now();
    parallelFor(rq.size(), [&](size_t k)
    {
        MsRead& m = ms[rqRead[k]];
        if (m.r.failed) return;
        try
        {
            for (size_t t = 0; t < m.forward.size(); t++)
            {
                OnewayTrace fw = std::move(m.forward[t]);
                OnewayTrace bw;
                bw.score = INT32_MAX;
                if (m.backwardRequest[t] >= 0)
                {
                    const size_t q = firstRequest[k] + (size_t)m.backwardRequest[t];
                    if (br[q].status == GA_ASSERT) throw ReadFailure {};
                    GAH_ASSERT(br[q].status == GA_OK || br[q].status == GA_TRACE_FAILED);
                    bw = decodeTrace(g, br[q], bq[q].seq, bq[q].len);
                    if (!bw.failed())
                    {
                        std::reverse(bw.trace.begin(), bw.trace.end());
                        fixReverseTraceSeqPosAndOrder(g, bw, fw.trace[0].seqPos - 1, m.r.seq, false);
                    }
                }
                OnewayTrace merged = mergeTraces(std::move(bw), std::move(fw));
                if (merged.failed()) continue;
                GAH_ASSERT(!merged.trace.empty());
                const int32_t alignmentXScore = score32((merged.trace.back().seqPos - merged.trace[0].seqPos + 1) * 100)
                    - p.xscoreErrorCost * merged.score;
                if (alignmentXScore <= 0) continue;
                AlignmentItem item;
                item.trace = std::make_shared<OnewayTrace>(std::move(merged));
                item.alignmentScore = item.trace->score;
                item.alignmentStart = item.trace->trace[0].seqPos;
                item.alignmentEnd = item.trace->trace.back().seqPos + 1;
                GAH_ASSERT(item.alignmentEnd - 1 < m.r.seq.size());
                item.alignmentXScore = (double)alignmentXScore / 100.0;
                m.r.alignments.push_back(std::move(item));
            }
            addMappingQualities(m.r.alignments);
        }
        catch (const ReadFailure&)
        {
            m.r.failed = true;
            m.r.alignments.clear();
        }
    });
    stats.consumeMs += std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
    t0 = std::chrono::steady_clock::now();
    {
        // reads without seeds have no alignments and stay as they are
        std::vector<ReadState*> rsp(n);
        std::vector<ReadOutput*> osp(n);
        for (size_t i = 0; i < n; i++)
        {
            rsp[i] = &ms[i].r;
            osp[i] = &out[i];
        }
        std::vector<std::vector<AlignmentItem>> lines;
        finalizeGroup(p, rsp, osp, lines);
        formatFinished(g, p, rsp, osp, lines);
    }
    for (size_t i = 0; i < n; i++)
    {
        stats.bpAligned += out[i].bpAligned;
        stats.failedReads += out[i].failed ? 1 : 0;
    }
    stats.finishMs += std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
}

struct SeedLoopPool::Impl
{
    const HostGraph& g;
    const ReadAlignParams p;
    struct Live
    {
        std::unique_ptr<ReadState> r;
        uint64_t tag;
        bool noSeeds = false;
    };
    std::vector<Live> live;          // reads in their seed loops
    std::vector<Live> finished;      // loop ended or failed; finalized by takeFinished
    struct Pending
    {
        ReadState* r;
        size_t seed;
        int64_t backward = -1;       // request index or -1
        int64_t forward = -1;
        bool speculative = false;    // follows the read's previous pending entry
    };
    std::vector<Pending> pending;
    std::vector<ExtensionRequest> requests;
    double collectMs = 0;
    double stepsPerBp = 3.0;         // column steps per extended bp, from the last round
    Impl(const HostGraph& g_, const ReadAlignParams& p_) : g(g_), p(p_) {}
};

SeedLoopPool::SeedLoopPool(const HostGraph& g, const ReadAlignParams& p) : impl(new Impl(g, p)) {}
SeedLoopPool::~SeedLoopPool() = default;

size_t SeedLoopPool::active() const { return impl->live.size() + impl->finished.size(); }

void SeedLoopPool::addMany(std::vector<ReadInput>& reads, const std::vector<uint64_t>& tags)
{
    // orderSeeds and the reverse complement of every read on all cores, then the pool update
    std::vector<Impl::Live> ls(reads.size());
    parallelFor(reads.size(), [&](size_t i)
    {
        Impl::Live& l = ls[i];
        l.r.reset(new ReadState());
        l.tag = tags[i];
        ReadState& r = *l.r;
        r.name = std::move(reads[i].name);
        r.seq = std::move(reads[i].seq);
        r.seeds = std::move(reads[i].seeds);
        if (r.seeds.size() == 0)
        {
            r.done = true;
            l.noSeeds = true;
            return;
        }
        try
        {
            orderSeeds(impl->g, r.seeds);
            r.rev = reverseComplement(r.seq);
        }
        catch (const ReadFailure&)
        {
            r.done = true;
            r.failed = true;
            return;
        }
        r.extendSeeds = (size_t)(impl->p.seedExtendDensity * r.seq.size() + 1);
        if (impl->p.seedExtendDensity == -1) r.extendSeeds = r.seeds.size();
    });
    for (auto& l : ls)
    {
        if (l.r->done) impl->finished.push_back(std::move(l));
        else impl->live.push_back(std::move(l));
    }
}

void SeedLoopPool::add(ReadInput&& read, uint64_t tag)
{
    Impl::Live l;
    l.r.reset(new ReadState());
    l.tag = tag;
    ReadState& r = *l.r;
    r.name = std::move(read.name);
    r.seq = std::move(read.seq);
    r.seeds = std::move(read.seeds);
    if (r.seeds.size() == 0)
    {
        r.done = true;
        l.noSeeds = true;
        impl->finished.push_back(std::move(l));
        return;
    }
    try
    {
        orderSeeds(impl->g, r.seeds);
        r.rev = reverseComplement(r.seq);
    }
    catch (const ReadFailure&)
    {
        r.done = true;
        r.failed = true;
        impl->finished.push_back(std::move(l));
        return;
    }
    r.extendSeeds = (size_t)(impl->p.seedExtendDensity * r.seq.size() + 1);
    if (impl->p.seedExtendDensity == -1) r.extendSeeds = r.seeds.size();
    impl->live.push_back(std::move(l));
}

static double msSince(std::chrono::steady_clock::time_point t)
{
    return std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t).count();
}

static constexpr int kMaxSpeculation = 8;
static constexpr size_t kMinReadsToSpeculate = 16;

// the two extensions of a seed (GraphAligner::getTwoDirectionalTrace, GraphAligner.h:475-506)
static int seedRequests(const HostGraph& g, const ReadState& r, const SeedHit& s, ExtensionRequest* q, int& backward, int& forward)
{
    int n = 0;
    backward = forward = -1;
    int forwardNodeId = s.reverse ? s.nodeID * 2 + 1 : s.nodeID * 2;
    GAH_ASSERT(s.seqPos < r.seq.size());
    if (s.seqPos > 0)
    {
        auto rp = g.reversePosition(forwardNodeId, s.nodeOffset);
        ExtensionRequest& e = q[n];
        e.seq = r.rev.data() + r.rev.size() - s.seqPos;
        e.len = s.seqPos;
        e.bignode = rp.first;
        e.offset = rp.second;
        size_t node = g.unitigNode(e.bignode, e.offset);
        e.node = (uint32_t)node;
        e.nodeOffset = (uint32_t)(e.offset - g.nodeOffset[node]);
        backward = n++;
    }
    if (s.seqPos < r.seq.size() - 1)
    {
        ExtensionRequest& e = q[n];
        e.seq = r.seq.data() + s.seqPos + 1;
        e.len = r.seq.size() - s.seqPos - 1;
        e.bignode = forwardNodeId;
        e.offset = s.nodeOffset;
        size_t node = g.unitigNode(e.bignode, e.offset);
        e.node = (uint32_t)node;
        e.nodeOffset = (uint32_t)(e.offset - g.nodeOffset[node]);
        forward = n++;
    }
    return n;
}

bool SeedLoopPool::collect(std::vector<ExtensionRequest>& requests)
{
    const auto t0 = std::chrono::steady_clock::now();
    const HostGraph& g = impl->g;
    const ReadAlignParams& p = impl->p;
    auto& pending = impl->pending;
    pending.clear();
    requests.clear();
    const size_t nLive = impl->live.size();
    // speculation depth from the estimated work of a round: one seed of every read covers
    // about its length, at the previous round's column steps per extended bp
    double roundBp = 0;
    for (const auto& l : impl->live) roundBp += (double)l.r->seq.size();
    const double work = roundBp * impl->stepsPerBp;
    int spec = 1;
    // a round of a few reads waits for its slowest extension either way: more seeds per
    // read only add extensions that can be slower still
    if (nLive >= kMinReadsToSpeculate && work > 0 && work < p.speculationSteps)
        spec = (int)std::min<double>({ (double)p.maxSpeculation, (double)kMaxSpeculation, 1.0 + (p.speculationSteps - work) / work });
    // every read advances its own seed loop (all cores): its next seed for real, then up to
    // spec - 1 further candidates on a copy of its cursor (as if the seeds before them were
    // extended without changing the alignments); the requests are then gathered in read
    // order, backward extension before forward, as a serial loop would emit them
    struct Cand
    {
        size_t seed;
        int backward;
        int forward;
        int q0;
    };
    struct Next
    {
        int state = 0;           // 0 pending, 1 loop ended, 2 failed
        int count = 0;           // candidate seeds
        int nq = 0;
        Cand cand[kMaxSpeculation];
        ExtensionRequest q[2 * kMaxSpeculation];
    };
    std::vector<Next> next(nLive);
    parallelFor(nLive, [&](size_t i)
    {
        ReadState& r = *impl->live[i].r;
        Next& nx = next[i];
        size_t seedIndex = 0;
        bool more = false;
        try
        {
            more = nextSeed(p, r, seedIndex);
        }
        catch (const ReadFailure&)
        {
            r.failed = true;
        }
        if (!more)
        {
            nx.state = 1;
            return;
        }
        try
        {
            Cand& c = nx.cand[0];
            c.seed = seedIndex;
            c.q0 = 0;
            nx.nq += seedRequests(g, r, r.seeds[seedIndex], nx.q, c.backward, c.forward);
            nx.count = 1;
        }
        catch (const ReadFailure&)
        {
            r.failed = true;
            nx.state = 2;
            return;
        }
        SeedCursor cur { r.next, r.worstExtendedSeedScore, r.seedsExtended };
        while (nx.count < spec)
        {
            size_t si = 0;
            try
            {
                if (!nextSeedOn(p, r, cur, si)) break;
                Cand& c = nx.cand[nx.count];
                c.seed = si;
                c.q0 = nx.nq;
                nx.nq += seedRequests(g, r, r.seeds[si], nx.q + nx.nq, c.backward, c.forward);
                nx.count++;
            }
            catch (const ReadFailure&)
            {
                break;               // the loop may never reach this seed; if it does, it fails then
            }
        }
    });
    size_t keep = 0;
    for (size_t i = 0; i < nLive; i++)
    {
        Impl::Live& l = impl->live[i];
        Next& nx = next[i];
        if (nx.state != 0)
        {
            l.r->done = true;
            impl->finished.push_back(std::move(l));
            continue;
        }
        for (int k = 0; k < nx.count; k++)
        {
            const Cand& c = nx.cand[k];
            Impl::Pending pe;
            pe.r = l.r.get();
            pe.seed = c.seed;
            pe.speculative = k > 0;
            if (c.backward >= 0)
            {
                pe.backward = (int64_t)requests.size();
                requests.push_back(nx.q[c.q0 + c.backward]);
            }
            if (c.forward >= 0)
            {
                pe.forward = (int64_t)requests.size();
                requests.push_back(nx.q[c.q0 + c.forward]);
            }
            pending.push_back(pe);
        }
        if (keep != i) impl->live[keep] = std::move(l);
        keep++;
    }
    impl->live.resize(keep);
    impl->requests = requests;
    impl->collectMs += msSince(t0);
    return !pending.empty();
}

void SeedLoopPool::consume(const std::vector<ExtensionResult>& results, BatchStats& stats)
{
    const HostGraph& g = impl->g;
    const auto& requests = impl->requests;
    const auto t0 = std::chrono::steady_clock::now();
    stats.collectMs += impl->collectMs;
    impl->collectMs = 0;
    stats.rounds++;
    stats.extensions += requests.size();
    {
        double steps = 0, bp = 0;
        for (size_t k = 0; k < results.size(); k++)
        {
            stats.cellSteps += results[k].steps;
            steps += (double)results[k].steps;
            bp += (double)requests[k].len;
        }
        if (bp > 0) impl->stepsPerBp = std::max(1.0, steps / bp);
    }
    // every read touches only its own state: finish its seeds on all cores, a read's own
    // entries in order
    const auto& pending = impl->pending;
    const ReadAlignParams& p = impl->p;
    std::vector<size_t> groupStart;
    for (size_t i = 0; i < pending.size(); i++)
        if (!pending[i].speculative) groupStart.push_back(i);
    groupStart.push_back(pending.size());
    std::atomic<uint64_t> used(0), discarded(0);
    auto finish = [&](const Impl::Pending& pe, ReadState& r) -> bool
    {
        const SeedHit& s = r.seeds[pe.seed];
        int forwardNodeId = s.reverse ? s.nodeID * 2 + 1 : s.nodeID * 2;
        int backwardNodeId = s.reverse ? s.nodeID * 2 : s.nodeID * 2 + 1;
        try
        {
            for (int64_t k : { pe.backward, pe.forward })
            {
                if (k >= 0 && (results[k].status == GA_ASSERT || results[k].status == GA_CAPACITY || results[k].status == GA_BAD_REQUEST)) throw ReadFailure {};
            }
            OnewayTrace bw, fw;
            bw.score = INT32_MAX;
            fw.score = INT32_MAX;
            // the backward trace keeps room for the forward one, which finishSeed appends
            const size_t forwardItems = pe.forward >= 0 ? results[pe.forward].size() : 0;
            if (pe.backward >= 0) bw = decodeTrace(g, results[pe.backward], requests[pe.backward].seq, requests[pe.backward].len, false, forwardItems);
            if (pe.forward >= 0) fw = decodeTrace(g, results[pe.forward], requests[pe.forward].seq, requests[pe.forward].len, true);
            finishSeed(g, p, r, s, std::move(bw), std::move(fw), backwardNodeId, forwardNodeId);
            return true;
        }
        catch (const ReadFailure&)
        {
            r.failed = true;
            return false;
        }
    };
    parallelFor(groupStart.size() - 1, [&](size_t gi)
    {
        const size_t first = groupStart[gi], last = groupStart[gi + 1];
        ReadState& r = *pending[first].r;
        size_t k = first;
        if (finish(pending[k++], r))
        {
            // speculative entries: replay the seed loop on the read's true state; a result is
            // used only if the loop extends exactly that seed next
            for (; k < last; k++)
            {
                const Impl::Pending& pe = pending[k];
                const SeedCursor saved { r.next, r.worstExtendedSeedScore, r.seedsExtended };
                size_t idx = 0;
                bool more = false;
                try
                {
                    more = nextSeed(p, r, idx);
                }
                catch (const ReadFailure&)
                {
                    r.failed = true;
                    break;
                }
                if (!more) break;
                if (idx != pe.seed)
                {
                    // the loop goes elsewhere: leave its cursor where the next round starts
                    r.next = saved.next;
                    r.worstExtendedSeedScore = saved.worstExtendedSeedScore;
                    r.seedsExtended = saved.seedsExtended;
                    break;
                }
                used++;
                if (!finish(pe, r))
                {
                    k++;
                    break;
                }
            }
        }
        discarded += last - k;
    });
    stats.speculativeUsed += used;
    stats.speculativeDiscarded += discarded;
    impl->pending.clear();
    // a read that failed in this round leaves its loop now
    size_t keep = 0;
    for (size_t i = 0; i < impl->live.size(); i++)
    {
        Impl::Live& l = impl->live[i];
        if (l.r->failed)
        {
            l.r->done = true;
            impl->finished.push_back(std::move(l));
            continue;
        }
        if (keep != i) impl->live[keep] = std::move(l);
        keep++;
    }
    impl->live.resize(keep);
    stats.consumeMs += msSince(t0);
}

void SeedLoopPool::takeFinished(std::vector<std::pair<uint64_t, ReadOutput>>& out, BatchStats& stats, bool overlapped)
{
    const auto t0 = std::chrono::steady_clock::now();
    auto& fin = impl->finished;
    const size_t base = out.size();
    out.resize(base + fin.size());
    {
        std::vector<ReadState*> rsp(fin.size());
        std::vector<ReadOutput*> osp(fin.size());
        for (size_t i = 0; i < fin.size(); i++)
        {
            out[base + i].first = fin[i].tag;
            out[base + i].second.noSeeds = fin[i].noSeeds;
            rsp[i] = fin[i].r.get();
            osp[i] = &out[base + i].second;
        }
        std::vector<std::vector<AlignmentItem>> lines;
        finalizeGroup(impl->p, rsp, osp, lines, overlapped);
        formatFinished(impl->g, impl->p, rsp, osp, lines, !overlapped);
    }
    for (size_t i = base; i < out.size(); i++)
    {
        if (out[i].second.failed) stats.failedReads++;
        stats.bpAligned += out[i].second.bpAligned;
    }
    fin.clear();
    stats.finishMs += msSince(t0);
}

void alignBatch(const HostGraph& g, const ReadAlignParams& p, std::vector<ReadInput>& reads, ExtendFn extend, void* ctx,
    std::vector<ReadOutput>& out, BatchStats& stats)
{
    out.assign(reads.size(), ReadOutput {});
    SeedLoopPool pool(g, p);
    std::vector<uint64_t> tags(reads.size());
    for (size_t i = 0; i < reads.size(); i++) tags[i] = i;
    pool.addMany(reads, tags);
    std::vector<ExtensionRequest> requests;
    std::vector<ExtensionResult> results;
    while (pool.collect(requests))
    {
        results.assign(requests.size(), ExtensionResult {});
        if (!requests.empty()) extend(ctx, requests, results);
        pool.consume(results, stats);
    }
    std::vector<std::pair<uint64_t, ReadOutput>> done;
    pool.takeFinished(done, stats);
    for (auto& d : done) out[d.first] = std::move(d.second);
}

void alignBatchTwoLanes(const HostGraph& g, const ReadAlignParams& p, std::vector<ReadInput>& reads, ExtendFn extend,
    void* ctxA, void* ctxB, std::vector<ReadOutput>& out, BatchStats& stats)
{
    out.assign(reads.size(), ReadOutput {});
    // alternate reads between the groups after sorting by length, so both carry similar work
    std::vector<size_t> byLen(reads.size());
    for (size_t i = 0; i < reads.size(); i++) byLen[i] = i;
    std::stable_sort(byLen.begin(), byLen.end(), [&](size_t a, size_t b) { return reads[a].seq.size() > reads[b].seq.size(); });
    std::vector<ReadInput> part[2];
    std::vector<uint64_t> tags[2];
    std::vector<std::string> nameOf(reads.size());     // the reads are moved into the pools
    for (size_t i = 0; i < reads.size(); i++) nameOf[i] = reads[i].name;
    for (size_t k = 0; k < byLen.size(); k++)
    {
        part[k & 1].push_back(std::move(reads[byLen[k]]));
        tags[k & 1].push_back(byLen[k]);
    }
    SeedLoopPool pool0(g, p), pool1(g, p);
    SeedLoopPool* pool[2] = { &pool0, &pool1 };
    void* ctx[2] = { ctxA, ctxB };
    pool0.addMany(part[0], tags[0]);
    pool1.addMany(part[1], tags[1]);
    std::vector<ExtensionRequest> rq[2];
    std::vector<ExtensionResult> rs[2];
    std::vector<std::pair<uint64_t, ReadOutput>> done;
    bool active[2];
    std::thread worker[2];
    auto launch = [&](int k)
    {
        rs[k].assign(rq[k].size(), ExtensionResult {});
        if (!rq[k].empty()) worker[k] = std::thread([&, k]() { extend(ctx[k], rq[k], rs[k]); });
    };
    // finished reads are selected and their GAF lines walked between rounds on the host's
    // cores, while the other group's extensions hold the GPU; a GAF writer hook writes all the
    // text at the end
    auto finish = [&](int k)
    {
        if (worker[k].joinable()) worker[k].join();
        pool[k]->consume(rs[k], stats);
        pool[k]->takeFinished(done, stats, true);
        active[k] = pool[k]->collect(rq[k]);
        pool[k]->takeFinished(done, stats, true);
    };
    active[0] = pool0.collect(rq[0]);
    pool0.takeFinished(done, stats, true);
    if (active[0]) launch(0);
    active[1] = pool1.collect(rq[1]);
    pool1.takeFinished(done, stats, true);
    while (active[0] || active[1])
    {
        // group 1 goes to the GPU while the host finishes group 0, and the other way round
        if (active[1]) launch(1);
        if (active[0])
        {
            finish(0);
            if (active[0]) launch(0);
        }
        if (active[1]) finish(1);
    }
    for (auto& t : worker) if (t.joinable()) t.join();
    pool0.takeFinished(done, stats, true);
    pool1.takeFinished(done, stats, true);
    {
        const auto t0 = std::chrono::steady_clock::now();
        std::vector<const std::string*> names(done.size());
        for (size_t i = 0; i < done.size(); i++) names[i] = &nameOf[done[i].first];
        writeFinished(p, done, names);
        stats.finishMs += msSince(t0);
    }
    for (auto& d : done) out[d.first] = std::move(d.second);
}

}
