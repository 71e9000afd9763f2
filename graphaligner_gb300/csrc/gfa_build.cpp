// Alignment graph from GFA text (the builder behind graph.build_from_gfa), following
// DirectedGraph::BuildFromGFA (BigraphToDigraph.cpp:214-266) and AlignmentGraph's
// construction and Finalize (AlignmentGraph.cpp:47-80, 230-248, 300-724, 898-1094):
//   - both strands of every segment (GFA id * 2 forward, id * 2 + 1 reverse complement;
//     numeric GFA names keep their numbers, other names are numbered in file order);
//   - a link overlap of o bp enters the target strand at offset o: both strands get a
//     breakpoint there, and pieces of at most 64 bp are cut from every breakpoint;
//   - a link joins the source's last piece to the target's piece that starts at o;
//   - pieces with a character other than A, C, G, T, U go to the end, in reverse order;
//   - findLinearizable, the Tarjan component order of doComponentOrder, findChains with
//     union by rank (and the reference's rank bump when both sides share a root),
//     raw-parent comparisons of chainTips, and fixChainApproxPos.
// The node numbering is the builder's own (GFA order); the reference iterates hash maps
// whose order its build fixes, so the same GFA gives the same graph up to numbering.
#include "gfa_build.h"
#include <algorithm>
#include <climits>
#include <cstring>
#include <exception>
#include <new>
#include <string>
#include <unordered_map>
#include <utility>
#include <vector>
#include "../../include/graphaligner_gb300.h"

void ga_set_last_error(const char* message);

namespace
{
constexpr int64_t kPiece = 64;
constexpr uint64_t kNone = ~0ULL;

struct GfaError
{
    std::string what;
};

struct Tables
{
    unsigned char complement[256];
    unsigned char code[256];     // 2-bit code of A C G T U in either case, 255 for the rest
    unsigned char iupac[256];    // A,C,G,T mask of an upper-case IUPAC letter (U as T), 0 for the rest
    Tables()
    {
        for (int i = 0; i < 256; i++)
        {
            complement[i] = (unsigned char)i;
            code[i] = 255;
            iupac[i] = 0;
        }
        const char* from = "ACGTUacgtuRYKMSWBDHVNrykmswbdhvn";
        const char* to = "TGCAAtgcaaYRMKSWVHDBNyrmkswvhdbn";
        for (size_t i = 0; from[i]; i++) complement[(unsigned char)from[i]] = (unsigned char)to[i];
        const char* acgt = "ACGT";
        for (int i = 0; i < 4; i++)
        {
            code[(unsigned char)acgt[i]] = (unsigned char)i;
            code[(unsigned char)(acgt[i] + 32)] = (unsigned char)i;
        }
        code[(unsigned char)'U'] = 3;
        code[(unsigned char)'u'] = 3;
        const char* letters = "ACGTURYKMSWBDHVN";
        const unsigned char masks[16] = { 1, 2, 4, 8, 8, 5, 10, 12, 3, 6, 9, 14, 13, 11, 7, 15 };
        for (int i = 0; i < 16; i++) iupac[(unsigned char)letters[i]] = masks[i];
    }
};
const Tables kTables;

struct Built
{
    ga_gfa_graph_arrays view {};
    std::vector<uint32_t> nodeLength, nodeOffset, component, inOff, inNb, outOff, outNb, originalSize, lookupOff, lookupNodes;
    std::vector<int32_t> nodeIds, lookupIds;
    std::vector<uint8_t> reverse, linearizable;
    std::vector<uint64_t> chain, chainPos, seq2, seqAmb;
    std::string names;
};

struct Link
{
    uint32_t from;      // segment slots
    uint32_t to;
    bool fromForward;
    bool toForward;
    int64_t overlap;
};

struct Piece
{
    int64_t big;
    int64_t offset;
    size_t textStart;   // into the piece-text buffer
    uint32_t length;
};

typedef std::vector<std::vector<uint32_t>> Lists;

std::vector<std::string> splitTabs(const char* s, size_t n)
{
    std::vector<std::string> f;
    size_t start = 0;
    for (size_t i = 0; i <= n; i++)
    {
        if (i == n || s[i] == '\t')
        {
            f.emplace_back(s + start, i - start);
            start = i + 1;
        }
    }
    return f;
}

// int(text.rstrip("MS")) for a non-negative overlap
int64_t parseOverlap(const std::string& field)
{
    if (field == "*") return 0;
    size_t end = field.size();
    while (end > 0 && (field[end - 1] == 'M' || field[end - 1] == 'S')) end--;
    size_t i = 0;
    if (i < end && field[i] == '+') i++;
    if (i >= end) throw GfaError { "link overlap '" + field + "' is not a number of bases" };
    int64_t v = 0;
    for (; i < end; i++)
    {
        if (field[i] < '0' || field[i] > '9') throw GfaError { "link overlap '" + field + "' is not a number of bases" };
        v = v * 10 + (field[i] - '0');
        if (v > INT32_MAX) throw GfaError { "link overlap '" + field + "' is too large" };
    }
    return v;
}

bool numericName(const std::string& s)
{
    size_t i = 0;
    while (i < s.size() && s[i] == '-') i++;
    if (i == s.size()) return false;
    for (; i < s.size(); i++) if (s[i] < '0' || s[i] > '9') return false;
    return true;
}

int64_t parseId(const std::string& s)
{
    size_t i = 0;
    bool negative = false;
    if (i < s.size() && s[i] == '-')
    {
        negative = true;
        i++;
    }
    if (i == s.size() || s[i] == '-') throw GfaError { "segment name '" + s + "' is not a number" };
    int64_t v = 0;
    for (; i < s.size(); i++)
    {
        v = v * 10 + (s[i] - '0');
        if (v > ((int64_t)1 << 40)) throw GfaError { "segment id '" + s + "' does not fit a node id" };
    }
    return negative ? -v : v;
}

// AlignmentGraph::findLinearizable (AlignmentGraph.cpp:632-724), step for step: the
// reference marks a node checked before pushing it, so its walk ends on its first step
// and no node ends up linearizable.
std::vector<uint8_t> findLinearizable(const Lists& in)
{
    const size_t n = in.size();
    std::vector<uint8_t> lin(n, 0), checked(n, 0), onStack(n, 0);
    std::vector<uint32_t> stack;
    for (size_t node = 0; node < n; node++)
    {
        if (checked[node]) continue;
        if (in[node].size() != 1)
        {
            checked[node] = 1;
            continue;
        }
        checked[node] = 1;
        stack.assign(1, (uint32_t)node);
        onStack[node] = 1;
        while (true)
        {
            const uint32_t top = stack.back();
            if (in[top].size() != 1 || checked[top])
            {
                for (size_t k = 0; k + 1 < stack.size(); k++)
                {
                    checked[stack[k]] = 1;
                    lin[stack[k]] = 1;
                    onStack[stack[k]] = 0;
                }
                lin[top] = 0;
                checked[top] = 1;
                onStack[top] = 0;
                break;
            }
            const uint32_t nb = in[top][0];
            if (nb == node)
            {
                for (uint32_t s : stack)
                {
                    checked[s] = 1;
                    lin[s] = 0;
                    onStack[s] = 0;
                }
                break;
            }
            if (onStack[nb])
            {
                const size_t k = std::find(stack.begin(), stack.end(), nb) - stack.begin();
                for (size_t j = k + 1; j < stack.size(); j++)
                {
                    checked[stack[j]] = 1;
                    lin[stack[j]] = 0;
                    onStack[stack[j]] = 0;
                }
                for (size_t j = 0; j < k; j++)
                {
                    checked[stack[j]] = 1;
                    lin[stack[j]] = 1;
                    onStack[stack[j]] = 0;
                }
                break;
            }
            stack.push_back(nb);
            onStack[nb] = 1;
        }
    }
    return lin;
}

// AlignmentGraph::doComponentOrder (AlignmentGraph.cpp:987-1094): iterative Tarjan from
// node 0 upward; components numbered in reverse finishing order, so that every edge goes
// from a lower to an equal or higher component number.
std::vector<uint32_t> componentOrder(const Lists& out)
{
    const size_t n = out.size();
    std::vector<int64_t> index(n, -1), low(n, -1), comp(n, -1);
    std::vector<uint8_t> onStack(n, 0);
    std::vector<uint32_t> stack;
    std::vector<std::pair<uint32_t, uint32_t>> call;
    int64_t counter = 0, nextComp = 0;
    for (size_t root = 0; root < n; root++)
    {
        if (index[root] != -1) continue;
        call.assign(1, { (uint32_t)root, 0u });
        index[root] = low[root] = counter++;
        stack.push_back((uint32_t)root);
        onStack[root] = 1;
        while (!call.empty())
        {
            const uint32_t v = call.back().first;
            const uint32_t i = call.back().second;
            if (i < out[v].size())
            {
                const uint32_t w = out[v][i];
                call.back().second = i + 1;
                if (index[w] == -1)
                {
                    index[w] = low[w] = counter++;
                    stack.push_back(w);
                    onStack[w] = 1;
                    call.push_back({ w, 0u });
                }
                else if (onStack[w])
                {
                    low[v] = std::min(low[v], index[w]);
                }
                continue;
            }
            call.pop_back();
            if (!call.empty())
            {
                const uint32_t u = call.back().first;
                low[u] = std::min(low[u], low[v]);
            }
            if (low[v] == index[v])
            {
                while (true)
                {
                    const uint32_t w = stack.back();
                    stack.pop_back();
                    onStack[w] = 0;
                    comp[w] = nextComp;
                    if (w == v) break;
                }
                nextComp++;
            }
        }
    }
    std::vector<uint32_t> result(n);
    for (size_t i = 0; i < n; i++) result[i] = (uint32_t)(nextComp - 1 - comp[i]);
    return result;
}

// AlignmentGraph::findChains (AlignmentGraph.cpp:571-630) with chainTips (428-519),
// chainCycles (521-569), chainBubble / findBubble (300-393) and fixChainApproxPos (395-426)
struct Chains
{
    const Lists& in;
    const Lists& out;
    const std::vector<uint32_t>& comp;
    std::vector<uint32_t> parent;
    std::vector<uint64_t> rank;
    std::vector<uint8_t> ignorable;
    std::vector<uint32_t> visitedStamp, seenStamp, walkStamp;
    uint32_t generation = 0, walkGeneration = 0;

    Chains(const Lists& in_, const Lists& out_, const std::vector<uint32_t>& comp_) : in(in_), out(out_), comp(comp_)
    {
        const size_t n = in.size();
        parent.resize(n);
        for (size_t i = 0; i < n; i++) parent[i] = (uint32_t)i;
        rank.assign(n, 0);
        ignorable.assign(n, 0);
        visitedStamp.assign(n, 0);
        seenStamp.assign(n, 0);
        walkStamp.assign(n, 0);
    }

    uint32_t find(uint32_t x)
    {
        uint32_t root = x;
        while (parent[root] != root) root = parent[root];
        while (parent[x] != root)
        {
            const uint32_t next = parent[x];
            parent[x] = root;
            x = next;
        }
        return root;
    }

    // union by rank; the rank grows also when both sides already share a root
    void merge(uint32_t a, uint32_t b)
    {
        a = find(a);
        b = find(b);
        if (rank[a] < rank[b]) std::swap(a, b);
        parent[b] = a;
        if (rank[a] == rank[b]) rank[a] += 1;
    }

    // the far end of a simple bubble that starts at `start`, or kNone
    uint64_t findBubble(uint32_t start)
    {
        generation++;
        std::vector<uint32_t> stack(1, start);
        size_t seenCount = 1;
        seenStamp[start] = generation;
        while (!stack.empty())
        {
            const uint32_t v = stack.back();
            stack.pop_back();
            if (seenStamp[v] == generation)
            {
                seenStamp[v] = 0;
                seenCount--;
            }
            visitedStamp[v] = generation;
            if (out[v].empty()) return kNone;
            for (uint32_t u : out[v])
            {
                if (ignorable[u] || u == v) continue;
                if (u == start) return kNone;
                if (seenStamp[u] != generation)
                {
                    seenStamp[u] = generation;
                    seenCount++;
                }
                bool open = false;
                for (uint32_t w : in[u])
                {
                    if (w != u && !ignorable[w] && visitedStamp[w] != generation)
                    {
                        open = true;
                        break;
                    }
                }
                if (!open) stack.push_back(u);
            }
            if (stack.size() == 1 && seenCount == 1 && seenStamp[stack[0]] == generation)
            {
                const uint32_t t = stack.back();
                if (std::find(out[t].begin(), out[t].end(), start) != out[t].end()) return kNone;
                return t;
            }
        }
        return kNone;
    }

    void run(const std::vector<std::vector<uint32_t>>& lookupPieces)
    {
        const size_t n = in.size();
        for (const auto& pieces : lookupPieces)
            for (size_t k = 1; k < pieces.size(); k++) merge(pieces[0], pieces[k]);
        // chainTips
        std::vector<uint32_t> order(n);
        for (size_t i = 0; i < n; i++) order[i] = (uint32_t)i;
        std::stable_sort(order.begin(), order.end(), [&](uint32_t a, uint32_t b) { return comp[a] < comp[b]; });
        const size_t numComp = n ? (size_t)comp[order[n - 1]] + 1 : 0;
        std::vector<uint8_t> fw(numComp, 1), bw(numComp, 1);
        for (size_t k = n; k-- > 0;)
        {
            const uint32_t i = order[k];
            const uint32_t ci = comp[i];
            if (!fw[ci]) continue;
            for (uint32_t nb : out[i])
            {
                if (comp[nb] == ci || !fw[comp[nb]])
                {
                    fw[ci] = 0;
                    break;
                }
            }
        }
        for (size_t k = n; k-- > 0;)
        {
            const uint32_t i = order[k];
            if (fw[comp[i]]) for (uint32_t nb : out[i]) merge(i, nb);
        }
        for (size_t k = 0; k < n; k++)
        {
            const uint32_t i = order[k];
            const uint32_t ci = comp[i];
            if (!bw[ci]) continue;
            for (uint32_t nb : in[i])
            {
                if (comp[nb] == ci || !bw[comp[nb]])
                {
                    bw[ci] = 0;
                    break;
                }
            }
        }
        for (size_t k = 0; k < n; k++)
        {
            const uint32_t i = order[k];
            if (bw[comp[i]]) for (uint32_t nb : in[i]) merge(i, nb);
        }
        // tip chainers in first-seen order of their key; the reference compares raw
        // parent entries here, not roots
        std::vector<uint32_t> tipKeys;
        std::unordered_map<uint32_t, std::vector<uint32_t>> tipChainers;
        auto addTip = [&](uint32_t key, uint32_t nb)
        {
            auto it = tipChainers.find(key);
            if (it == tipChainers.end())
            {
                tipKeys.push_back(key);
                it = tipChainers.emplace(key, std::vector<uint32_t>()).first;
            }
            it->second.push_back(nb);
        };
        for (size_t i = 0; i < n; i++)
        {
            const bool b = bw[comp[i]] != 0, f = fw[comp[i]] != 0;
            if (b || f) ignorable[i] = 1;
            if (b) for (uint32_t nb : out[i]) if (parent[nb] != parent[i]) addTip(parent[i], nb);
            if (f) for (uint32_t nb : in[i]) if (parent[nb] != parent[i]) addTip(parent[i], nb);
        }
        // chainCycles
        for (size_t i = 0; i < n; i++)
        {
            uint64_t ufw = kNone;
            for (uint32_t u : out[i])
            {
                if (ignorable[u] || u == i) continue;
                ufw = ufw == kNone ? u : kNone - 1;
            }
            uint64_t ubw = kNone;
            for (uint32_t u : in[i])
            {
                if (ignorable[u] || u == i) continue;
                if (ubw == kNone) ubw = u;
                else if (u != ubw) ubw = kNone - 1;
            }
            if (ufw != ubw || ufw >= kNone - 1) continue;
            ignorable[i] = 1;
            merge((uint32_t)i, (uint32_t)ufw);
        }
        // chainBubble from the last piece of every bigraph node
        std::vector<uint32_t> stack;
        for (const auto& pieces : lookupPieces)
        {
            const uint32_t start = pieces.back();
            const uint64_t end = findBubble(start);
            if (end == kNone) continue;
            merge(start, (uint32_t)end);
            walkGeneration++;
            stack.assign(1, start);
            while (!stack.empty())
            {
                const uint32_t top = stack.back();
                stack.pop_back();
                if (walkStamp[top] == walkGeneration || ignorable[top]) continue;
                walkStamp[top] = walkGeneration;
                merge(start, top);
                for (uint32_t nb : out[top])
                    if (walkStamp[nb] != walkGeneration && nb != end) stack.push_back(nb);
            }
        }
        for (uint32_t key : tipKeys)
        {
            const auto& nbs = tipChainers[key];
            bool one = true;
            for (uint32_t x : nbs) if (parent[x] != parent[nbs[0]]) one = false;
            if (!one) continue;
            merge(key, nbs[0]);
        }
    }
};

void build(const char* text, size_t bytes, Built& g)
{
    // ---- GFA: segments in file order, links ----
    // one slot per segment name, holding the last sequence given for it
    std::unordered_map<std::string, uint32_t> slotOf;
    std::vector<std::string> slotName, slotSeq;
    std::vector<uint32_t> order;      // the slot of every S line, in file order
    std::vector<std::vector<std::string>> linkFields;
    slotOf.reserve(bytes / 64 + 16);
    size_t pos = 0;
    while (pos < bytes)
    {
        const char* nl = (const char*)memchr(text + pos, '\n', bytes - pos);
        size_t end = nl ? (size_t)(nl - text) : bytes;
        size_t lineEnd = end;
        if (lineEnd > pos && text[lineEnd - 1] == '\r') lineEnd--;
        const size_t len = lineEnd - pos;
        if (len > 0 && (text[pos] == 'S' || text[pos] == 'L'))
        {
            std::vector<std::string> f = splitTabs(text + pos, len);
            if (f[0] == "S")
            {
                if (f.size() < 3) throw GfaError { "segment line with fewer than 3 fields" };
                auto it = slotOf.find(f[1]);
                uint32_t slot;
                if (it == slotOf.end())
                {
                    slot = (uint32_t)slotName.size();
                    slotOf.emplace(f[1], slot);
                    slotName.push_back(f[1]);
                    slotSeq.push_back(std::move(f[2]));
                }
                else
                {
                    slot = it->second;
                    slotSeq[slot] = std::move(f[2]);
                }
                order.push_back(slot);
            }
            else if (f[0] == "L")
            {
                if (f.size() < 6) throw GfaError { "link line with fewer than 6 fields" };
                f.resize(6);
                linkFields.push_back(std::move(f));
            }
        }
        pos = end + 1;
    }
    bool numeric = true;
    for (uint32_t slot : order) numeric = numeric && numericName(slotName[slot]);
    // a repeated name takes the id of its last S line
    std::vector<int64_t> ids(slotName.size());
    for (size_t k = 0; k < order.size(); k++) ids[order[k]] = numeric ? parseId(slotName[order[k]]) : (int64_t)k + 1;
    auto slotNamed = [&](const std::string& name) -> uint32_t
    {
        auto it = slotOf.find(name);
        if (it == slotOf.end()) throw GfaError { "link to an unknown segment '" + name + "'" };
        return it->second;
    };
    std::vector<Link> links;
    links.reserve(linkFields.size());
    for (const auto& f : linkFields)
        links.push_back(Link { slotNamed(f[1]), slotNamed(f[3]), f[2] == "+", f[4] == "+", parseOverlap(f[5]) });
    std::vector<std::vector<std::string>>().swap(linkFields);
    std::unordered_map<int64_t, std::vector<int64_t>> breaks;
    for (const auto& l : links)
    {
        const int64_t la = (int64_t)slotSeq[l.from].size(), lb = (int64_t)slotSeq[l.to].size();
        if (l.overlap >= la || l.overlap >= lb)
            throw GfaError { "overlap between " + slotName[l.from] + " and " + slotName[l.to] + " is not smaller than both nodes" };
        if (l.overlap)
        {
            const int64_t fa = ids[l.from] * 2 + (l.fromForward ? 0 : 1), fb = ids[l.to] * 2 + (l.toForward ? 0 : 1);
            breaks[fb].push_back(l.overlap);
            breaks[fa ^ 1].push_back(l.overlap);
        }
    }
    // ---- pieces: both strands of every segment, cut at breakpoints and every 64 bp ----
    std::vector<Piece> pieces;
    std::string pieceText;
    std::vector<std::pair<int64_t, std::vector<uint32_t>>> lookup;
    std::vector<std::string> names;
    std::unordered_map<int64_t, uint32_t> sizeOf;
    for (uint32_t slot : order)
    {
        const std::string& name = slotName[slot];
        const std::string& s = slotSeq[slot];
        const int64_t nid = ids[slot];
        std::string rc(s.rbegin(), s.rend());
        for (auto& c : rc) c = (char)kTables.complement[(unsigned char)c];
        for (int strand = 0; strand < 2; strand++)
        {
            const std::string& t = strand == 0 ? s : rc;
            const int64_t big = nid * 2 + strand;
            if (big < INT32_MIN || big > INT32_MAX) throw GfaError { "segment id of '" + name + "' does not fit a node id" };
            if (t.empty()) throw GfaError { "segment '" + name + "' has an empty sequence" };
            if (t.size() > UINT32_MAX) throw GfaError { "segment '" + name + "' is too long" };
            std::vector<int64_t> bp = breaks.count(big) ? breaks[big] : std::vector<int64_t>();
            bp.push_back(0);
            bp.push_back((int64_t)t.size());
            std::sort(bp.begin(), bp.end());
            bp.erase(std::unique(bp.begin(), bp.end()), bp.end());
            std::vector<uint32_t> idx;
            const int64_t tl = (int64_t)t.size();
            for (size_t k = 0; k + 1 < bp.size(); k++)
            {
                const int64_t lo = bp[k], hi = bp[k + 1];
                for (int64_t o = lo; o < hi; o += kPiece)
                {
                    const int64_t e = std::min(o + kPiece, hi);
                    const int64_t from = std::min(o, tl), to = std::max(from, std::min(e, tl));
                    idx.push_back((uint32_t)pieces.size());
                    pieces.push_back(Piece { big, o, pieceText.size(), (uint32_t)(to - from) });
                    pieceText.append(t, (size_t)from, (size_t)(to - from));
                }
            }
            lookup.emplace_back(big, std::move(idx));
            names.push_back(numeric ? std::string() : name);
            sizeOf[big] = (uint32_t)t.size();
        }
    }
    if (pieces.size() >= UINT32_MAX) throw GfaError { "too many pieces" };
    const size_t n = pieces.size();
    Lists in(n), out(n);
    std::unordered_map<uint64_t, uint32_t> pieceAt;   // (bigraph node, offset) -> piece
    pieceAt.reserve(n);
    auto key = [](int64_t big, int64_t offset) { return ((uint64_t)(uint32_t)(int32_t)big << 32) | (uint64_t)(uint32_t)offset; };
    std::unordered_map<int64_t, uint32_t> lastPiece;
    lastPiece.reserve(lookup.size());
    for (const auto& l : lookup)
    {
        for (uint32_t i : l.second) pieceAt[key(l.first, pieces[i].offset)] = i;
        lastPiece[l.first] = l.second.back();
    }
    for (const auto& l : lookup)
    {
        for (size_t k = 0; k + 1 < l.second.size(); k++)
        {
            out[l.second[k]].push_back(l.second[k + 1]);
            in[l.second[k + 1]].push_back(l.second[k]);
        }
    }
    auto addEdge = [&](int64_t from, int64_t to, int64_t overlap)
    {
        const uint32_t a = lastPiece.at(from);
        auto it = pieceAt.find(key(to, overlap));
        if (it == pieceAt.end()) throw GfaError { "no piece starts at a link's overlap" };
        const uint32_t b = it->second;
        if (std::find(in[b].begin(), in[b].end(), a) == in[b].end()) in[b].push_back(a);
        if (std::find(out[a].begin(), out[a].end(), b) == out[a].end()) out[a].push_back(b);
    };
    for (const auto& l : links)
    {
        const int64_t fa = ids[l.from] * 2 + (l.fromForward ? 0 : 1), fb = ids[l.to] * 2 + (l.toForward ? 0 : 1);
        addEdge(fa, fb, l.overlap);
        addEdge(fb ^ 1, fa ^ 1, l.overlap);
    }
    // ---- ambiguous pieces to the end, in reverse order (RenumberAmbiguousToEnd, AlignmentGraph.cpp:898-985) ----
    std::vector<uint8_t> amb(n, 0);
    for (size_t i = 0; i < n; i++)
    {
        const Piece& p = pieces[i];
        for (uint32_t c = 0; c < p.length; c++)
        {
            if (kTables.code[(unsigned char)pieceText[p.textStart + c]] == 255)
            {
                amb[i] = 1;
                break;
            }
        }
    }
    std::vector<uint32_t> renum(n), perm(n);
    uint32_t numAmb = 0, numPlain = 0;
    for (size_t i = 0; i < n; i++)
    {
        renum[i] = amb[i] ? (uint32_t)(n - 1 - numAmb++) : numPlain++;
        perm[renum[i]] = (uint32_t)i;
    }
    Lists in2(n), out2(n);
    for (size_t i = 0; i < n; i++)
    {
        for (uint32_t x : in[perm[i]]) in2[i].push_back(renum[x]);
        for (uint32_t x : out[perm[i]]) out2[i].push_back(renum[x]);
    }
    Lists().swap(in);
    Lists().swap(out);
    std::vector<std::vector<uint32_t>> lookupPieces(lookup.size());
    for (size_t k = 0; k < lookup.size(); k++)
        for (uint32_t x : lookup[k].second) lookupPieces[k].push_back(renum[x]);
    // ---- arrays ----
    g.nodeLength.resize(n);
    g.nodeIds.resize(n);
    g.nodeOffset.resize(n);
    g.reverse.resize(n);
    g.seq2.assign((size_t)numPlain * 2, 0);
    g.seqAmb.assign((size_t)numAmb * 4, 0);
    uint64_t bpSize = 0;
    for (size_t i = 0; i < n; i++)
    {
        const Piece& p = pieces[perm[i]];
        g.nodeLength[i] = p.length;
        g.nodeIds[i] = (int32_t)p.big;
        g.nodeOffset[i] = (uint32_t)p.offset;
        g.reverse[i] = (uint8_t)((p.big % 2 + 2) % 2 == 1);
        bpSize += p.length;
        const char* t = pieceText.data() + p.textStart;
        if (i < numPlain)
        {
            for (uint32_t c = 0; c < p.length; c++)
                g.seq2[i * 2 + c / 32] |= (uint64_t)kTables.code[(unsigned char)t[c]] << (2 * (c % 32));
        }
        else
        {
            const size_t k = i - numPlain;
            for (uint32_t c = 0; c < p.length; c++)
            {
                unsigned char ch = (unsigned char)t[c];
                if (ch >= 'a' && ch <= 'z') ch = (unsigned char)(ch - 32);
                const unsigned char m = kTables.iupac[ch];
                if (!m) throw GfaError { "a segment has a character that is not an IUPAC code" };
                for (int b = 0; b < 4; b++)
                    if ((m >> b) & 1) g.seqAmb[k * 4 + b] |= 1ULL << c;
            }
        }
    }
    auto csr = [](const Lists& lists, std::vector<uint32_t>& off, std::vector<uint32_t>& flat)
    {
        off.assign(lists.size() + 1, 0);
        for (size_t i = 0; i < lists.size(); i++) off[i + 1] = off[i] + (uint32_t)lists[i].size();
        flat.clear();
        flat.reserve(off.back());
        for (const auto& l : lists) flat.insert(flat.end(), l.begin(), l.end());
    };
    csr(in2, g.inOff, g.inNb);
    csr(out2, g.outOff, g.outNb);
    g.linearizable = findLinearizable(in2);
    g.component = componentOrder(out2);
    csr(lookupPieces, g.lookupOff, g.lookupNodes);
    Chains chains(in2, out2, g.component);
    chains.run(lookupPieces);
    g.chain.resize(n);
    for (size_t i = 0; i < n; i++) g.chain[i] = chains.find((uint32_t)i);
    // fixChainApproxPos
    g.chainPos.assign(n, kNone);
    const uint64_t start = ((uint64_t)n + 5) * kPiece;
    std::vector<std::pair<uint32_t, uint64_t>> stack;
    for (size_t s0 = 0; s0 < n; s0++)
    {
        if (g.chainPos[s0] != kNone) continue;
        const uint64_t c = g.chain[s0];
        stack.assign(1, { (uint32_t)s0, start });
        while (!stack.empty())
        {
            const uint32_t v = stack.back().first;
            const uint64_t d = stack.back().second;
            stack.pop_back();
            if (g.chainPos[v] != kNone) continue;
            g.chainPos[v] = d;
            for (uint32_t u : out2[v])
                if (g.chain[u] == c && g.chainPos[u] == kNone) stack.push_back({ u, d + g.nodeLength[u] });
            for (uint32_t u : in2[v])
                if (g.chain[u] == c && g.chainPos[u] == kNone) stack.push_back({ u, d - g.nodeLength[v] });
        }
    }
    g.lookupIds.resize(lookup.size());
    g.originalSize.resize(lookup.size());
    for (size_t k = 0; k < lookup.size(); k++)
    {
        g.lookupIds[k] = (int32_t)lookup[k].first;
        g.originalSize[k] = sizeOf[lookup[k].first];
    }
    for (const auto& name : names)
    {
        g.names += name;
        g.names.push_back('\0');
    }
    ga_gfa_graph_arrays& v = g.view;
    v.num_nodes = (uint32_t)n;
    v.first_ambiguous = numPlain;
    v.num_lookup = (uint32_t)lookup.size();
    v.num_in_edges = g.inNb.size();
    v.num_out_edges = g.outNb.size();
    v.num_lookup_nodes = g.lookupNodes.size();
    v.bp_size = bpSize;
    v.node_length = g.nodeLength.data();
    v.node_ids = g.nodeIds.data();
    v.node_offset = g.nodeOffset.data();
    v.reverse = g.reverse.data();
    v.linearizable = g.linearizable.data();
    v.component = g.component.data();
    v.chain_number = g.chain.data();
    v.chain_approx_pos = g.chainPos.data();
    v.seq2bit = g.seq2.data();
    v.seq_ambiguous = g.seqAmb.data();
    v.in_offsets = g.inOff.data();
    v.in_neighbors = g.inNb.data();
    v.out_offsets = g.outOff.data();
    v.out_neighbors = g.outNb.data();
    v.lookup_ids = g.lookupIds.data();
    v.original_size = g.originalSize.data();
    v.lookup_offsets = g.lookupOff.data();
    v.lookup_nodes = g.lookupNodes.data();
    v.names = g.names.data();
    v.names_bytes = g.names.size();
}
}

extern "C" int ga_gfa_build(const char* text, uint64_t bytes, void** handle, ga_gfa_graph_arrays* out)
{
    if ((!text && bytes) || !handle || !out) return GA_ERR_ARGUMENT;
    Built* g = new Built();
    try
    {
        build(text, (size_t)bytes, *g);
    }
    catch (const GfaError& e)
    {
        delete g;
        ga_set_last_error(("ga_gfa_build: " + e.what).c_str());
        return GA_ERR_ARGUMENT;
    }
    catch (const std::bad_alloc&)
    {
        delete g;
        ga_set_last_error("ga_gfa_build: out of host memory");
        return GA_ERR_NOMEM;
    }
    catch (const std::exception& e)
    {
        delete g;
        ga_set_last_error((std::string("ga_gfa_build: ") + e.what()).c_str());
        return GA_ERR_ARGUMENT;
    }
    *handle = g;
    *out = g->view;
    return GA_OK;
}

extern "C" void ga_gfa_free(void* handle)
{
    delete (Built*)handle;
}
