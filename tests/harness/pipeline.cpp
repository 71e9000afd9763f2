// Test harness (CPU): the read-level host logic of the package (seeding.cpp,
// readalign.cpp) driven by the oracle's extensions, printing seeds or GAF in the
// formats oracle/_ref/ga_ref prints, so the two can be diffed.
//   pipeline <graph.gag> <reads.fa> seeds <k> <w> <density> <discard>
//   pipeline <graph.gag> <reads.fa> table <k> <w> <discard>
//   pipeline <graph.gag> <reads.fa> indexdump <k> <w> <discard> <prefix>
//       the host index build's arrays as raw u64 files <prefix>.keys/.start/.pos (none for
//       "-"), with its sizes, a checksum per array and the build time on all cores
//   pipeline <graph.gag> <reads.fa> msseeds|msseedsdbg
//       per read: name, then the (slice, split node) seeds of prepareSeedsForMultiseeding
//   pipeline <graph.gag> <reads.fa> walk <k> <w> <discard>
//       the GPU build's per-node minimizer walk (index_walk.cuh) run on the host, grouped
//       by k-mer, against the host index build
//   pipeline <graph.gag> <reads.fa> gaf|gafdbg|gafms|gafmsdbg <bandwidth> <maxcells|-> [threads (gafms*)]
//   pipeline <graph.gag> <reads.fa> gafreads|gafreadsdbg <bandwidth> <maxcells|-> <threads>
//       the reference's worker shape (Aligner.cpp:777-785, runComponentMappings :390-606): each
//       thread takes the next read and runs its seeding and whole seed loop alone, with the
//       oracle's extensions on that thread; GAF in input order
#include <algorithm>
#include <atomic>
#include <chrono>
#include <thread>
#include <cstdio>
#include <cstring>
#include <fstream>
#include <iostream>
#include <sstream>
#include <string>
#include <vector>
#include "../../include/graphaligner_gb300.h"
#include "../../graphaligner_gb300/csrc/readalign.h"
#include "../../graphaligner_gb300/csrc/index_walk.cuh"
#include "../../graphaligner_gb300/csrc/gaf_format.cuh"
#include <cmath>

extern "C" int ora_extend_batch(const ga_graph_desc*, const ga_extend_params*, const ga_extend_batch_desc*, ga_extend_results*, int);

struct Gag
{
    uint64_t h[8];
    std::vector<uint32_t> len, off, comp, inOff, inNb, outOff, outNb, origSize, lookupOff, lookupNodes, nameLen;
    std::vector<int32_t> ids, lookupIds;
    std::vector<uint8_t> rev, lin;
    std::vector<uint64_t> chain, chainPos, seq2, seqAmb;
    std::vector<std::string> names;
    std::vector<const char*> namePtr;
};

template <typename T>
static void rd(std::ifstream& f, std::vector<T>& v, size_t n)
{
    v.resize(n);
    if (n) f.read((char*)v.data(), n * sizeof(T));
}

static bool loadGag(const char* path, Gag& g)
{
    std::ifstream f(path, std::ios::binary);
    char magic[4];
    f.read(magic, 4);
    if (memcmp(magic, "GAG1", 4) != 0) return false;
    f.read((char*)g.h, sizeof(g.h));
    size_t N = g.h[0], fa = g.h[1], nIn = g.h[2], nOut = g.h[3], M = g.h[4], nL = g.h[5], nNames = g.h[6];
    rd(f, g.len, N); rd(f, g.ids, N); rd(f, g.off, N); rd(f, g.rev, N); rd(f, g.lin, N); rd(f, g.comp, N);
    rd(f, g.chain, N); rd(f, g.chainPos, N); rd(f, g.seq2, fa * 2); rd(f, g.seqAmb, (N - fa) * 4);
    rd(f, g.inOff, N + 1); rd(f, g.inNb, nIn); rd(f, g.outOff, N + 1); rd(f, g.outNb, nOut);
    rd(f, g.lookupIds, M); rd(f, g.origSize, M); rd(f, g.lookupOff, M + 1); rd(f, g.lookupNodes, nL); rd(f, g.nameLen, M);
    std::string blob(nNames, ' ');
    if (nNames) f.read(&blob[0], nNames);
    size_t p = 0;
    for (size_t i = 0; i < M; i++) { g.names.push_back(blob.substr(p, g.nameLen[i])); p += g.nameLen[i]; }
    for (auto& s : g.names) g.namePtr.push_back(s.c_str());
    return true;
}

static std::vector<std::pair<std::string, std::string>> readFasta(const char* path)
{
    std::vector<std::pair<std::string, std::string>> r;
    std::ifstream in(path);
    std::string line;
    while (std::getline(in, line))
    {
        if (line.empty()) continue;
        if (line[0] == '>')
        {
            std::string name = line.substr(1);
            auto sp = name.find_first_of(" \t");
            if (sp != std::string::npos) name = name.substr(0, sp);
            r.emplace_back(name, "");
        }
        else r.back().second += line;
    }
    return r;
}

static inline bool validChar(char c)
{
    return c == 'a' || c == 'A' || c == 'c' || c == 'C' || c == 'g' || c == 'G' || c == 't' || c == 'T';
}

static inline uint64_t charToInt(char c)
{
    switch (c)
    {
        case 'a': case 'A': return 0;
        case 'c': case 'C': return 1;
        case 'g': case 'G': return 2;
        case 't': case 'T': return 3;
    }
    return 0;
}

// iterateKmers + the lookup of MinimizerSeeder::getSeeds (MinimizerSeeder.cpp:59-102, 524-537): the
// host restatement of the GPU k-mer lookup (seed_kernel.cu), for driving the host pipeline on the CPU
static void kmerMatchesHost(const gahost::MinimizerIndex& idx, const std::string& str, std::vector<gahost::KmerMatch>& out)
{
    out.clear();
    const size_t k = idx.k;
    const size_t realWindow = idx.w - k + 1;
    if (str.size() < k) return;
    const uint64_t mask = ~(0xFFFFFFFFFFFFFFFFULL << (k * 2));
    auto emit = [&](size_t pos, uint64_t kmer)
    {
        auto f = std::lower_bound(idx.keys.begin(), idx.keys.end(), kmer);
        if (f == idx.keys.end() || *f != kmer) return;
        size_t r = f - idx.keys.begin();
        uint64_t start = idx.startPos[r];
        uint64_t count = idx.startPos[r + 1] - start;
        if (count >= idx.maxCount) return;
        out.push_back(gahost::KmerMatch { pos, start, count });
    };
    size_t offset = 0;
start:
    while (offset < str.size() && !validChar(str[offset])) offset++;
    if (offset + k > str.size()) return;
    {
        uint64_t kmer = 0;
        for (size_t i = 0; i < k; i++)
        {
            if (!validChar(str[offset + i]))
            {
                offset += i;
                goto start;
            }
            kmer <<= 2;
            kmer |= charToInt(str[offset + i]);
        }
        emit(offset + k - 1, kmer);
        uint64_t lastKmer = kmer;
        size_t lastPos = offset + k - 1;
        for (size_t i = k; offset + i < str.size(); i++)
        {
            if (!validChar(str[offset + i]))
            {
                offset += i;
                goto start;
            }
            kmer <<= 2;
            kmer &= mask;
            kmer |= charToInt(str[offset + i]);
            if (lastKmer != kmer || lastPos <= offset + i - realWindow)
            {
                emit(offset + i, kmer);
                lastKmer = kmer;
                lastPos = offset + i;
            }
        }
    }
}

struct Ctx
{
    ga_graph_desc* d;
    ga_extend_params p;
    int threads = 8;
};

static void oracleExtend(void* ctx, const std::vector<gahost::ExtensionRequest>& rq, std::vector<gahost::ExtensionResult>& rs)
{
    Ctx* c = (Ctx*)ctx;
    size_t n = rq.size();
    std::vector<uint8_t> blob;
    std::vector<uint64_t> off(n), toff(n), items, steps(n);
    std::vector<uint32_t> len(n), node(n), noff(n), cap(n), tlen(n);
    std::vector<int32_t> status(n), score(n);
    uint64_t ti = 0;
    for (size_t i = 0; i < n; i++)
    {
        off[i] = blob.size();
        blob.insert(blob.end(), rq[i].seq, rq[i].seq + rq[i].len);
        len[i] = rq[i].len; node[i] = rq[i].node; noff[i] = rq[i].nodeOffset;
        cap[i] = rq[i].len + rq[i].len / 4 + 512;
        toff[i] = ti; ti += cap[i];
    }
    if (blob.empty()) blob.push_back(0);
    items.resize(ti + 1);
    ga_extend_batch_desc b { (uint32_t)n, blob.data(), off.data(), len.data(), node.data(), noff.data(), toff.data(), cap.data() };
    ga_extend_results r { status.data(), score.data(), tlen.data(), items.data(), steps.data() };
    ora_extend_batch(c->d, &c->p, &b, &r, c->threads);
    for (size_t i = 0; i < n; i++)
    {
        rs[i].status = status[i];
        rs[i].score = score[i];
        rs[i].steps = steps[i];
        rs[i].items.assign(items.begin() + toff[i], items.begin() + toff[i] + tlen[i]);
    }
}

// GAF lines through the read flow's writer hook with gaf_format.cuh's line writer on the host
// (the read flow classifies the lines with gaf_format.cuh either way): the code the product
// runs, the writer on the device, checked here against the reference's GAF
static gaf::NamesHost g_gafNames;

static bool hostWriter(void*, const std::vector<const std::string*>& names, const std::vector<const gahost::ClassifiedLines*>& reads,
    std::string& text, std::vector<uint64_t>& readEnd)
{
    gaf::Names nm = gaf::names_view(g_gafNames);
    text.clear();
    readEnd.assign(reads.size(), 0);
    for (size_t i = 0; i < reads.size(); i++)
    {
        const uint64_t nameOff[2] = { 0, names[i]->size() };
        nm.readNames = (const uint8_t*)names[i]->data();
        nm.readNameOff = nameOff;
        for (const auto& m : reads[i]->lines)
        {
            const int64_t len = gaf::write_line(nm, m, reads[i]->ops.data(), reads[i]->entries.data(), nullptr);
            const size_t at = text.size();
            text.resize(at + (size_t)len);
            gaf::write_line(nm, m, reads[i]->ops.data(), reads[i]->entries.data(), &text[at]);
            text += '\n';
        }
        readEnd[i] = text.size();
    }
    return true;
}

static bool hostSelect(void*, const std::vector<uint64_t>& first, const std::vector<uint64_t>& start, const std::vector<uint64_t>& end,
    const std::vector<double>& xscore, int minAlignmentScore, double fractionCutoff, std::vector<char>& keep)
{
    for (size_t i = 0; i + 1 < first.size(); i++)
        gaf::select_read((uint32_t)(first[i + 1] - first[i]), start.data() + first[i], end.data() + first[i], xscore.data() + first[i],
            minAlignmentScore, fractionCutoff, keep.data() + first[i]);
    return true;
}

extern "C" int ora_multiseed_batch(const ga_graph_desc*, const ga_extend_params*, const ga_multiseed_batch_desc*, ga_multiseed_results*, int);

static void oracleMultiseed(void* ctx, const std::vector<gahost::MultiseedRequest>& rq, std::vector<gahost::MultiseedResult>& rs)
{
    Ctx* c = (Ctx*)ctx;
    std::vector<size_t> todo(rq.size());
    for (size_t i = 0; i < rq.size(); i++) todo[i] = i;
    std::vector<uint64_t> wantItems(rq.size(), 0);
    std::vector<uint32_t> wantTraces(rq.size(), 0);
    for (int attempt = 0; attempt < 2 && !todo.empty(); attempt++)
    {
        const size_t n = todo.size();
        uint32_t maxTraces = 4096;
        if (attempt > 0)
        {
            maxTraces = 1;
            for (size_t k = 0; k < n; k++) maxTraces = std::max(maxTraces, wantTraces[todo[k]]);
        }
        std::vector<uint8_t> blob;
        std::vector<uint64_t> off(n), soff(n + 1, 0), toff(n), cap(n), steps(n), needI(n);
        std::vector<uint32_t> len(n), sslice, snode, ntr(n), needT(n);
        std::vector<int32_t> status(n);
        uint64_t ti = 0;
        for (size_t k = 0; k < n; k++)
        {
            const auto& q = rq[todo[k]];
            off[k] = blob.size();
            blob.insert(blob.end(), q.seq, q.seq + q.len);
            len[k] = q.len;
            sslice.insert(sslice.end(), q.slices, q.slices + q.numSeeds);
            snode.insert(snode.end(), q.nodes, q.nodes + q.numSeeds);
            soff[k + 1] = sslice.size();
            cap[k] = attempt == 0 ? (uint64_t)q.len * 64 + 4096 : wantItems[todo[k]] + 64;
            toff[k] = ti;
            ti += cap[k];
        }
        if (blob.empty()) blob.push_back(0);
        if (sslice.empty()) { sslice.push_back(0); snode.push_back(0); }
        std::vector<uint64_t> items(ti + 1), tstart(n * maxTraces);
        std::vector<int32_t> tscore(n * maxTraces);
        std::vector<uint32_t> tlen(n * maxTraces);
        ga_multiseed_batch_desc b { (uint32_t)n, blob.data(), off.data(), len.data(), soff.data(), sslice.data(), snode.data(), toff.data(), cap.data(),
            maxTraces, 0.9 };
        ga_multiseed_results r { status.data(), ntr.data(), tscore.data(), tstart.data(), tlen.data(), items.data(), steps.data(), needI.data(), needT.data() };
        ora_multiseed_batch(c->d, &c->p, &b, &r, c->threads);
        std::vector<size_t> again;
        for (size_t k = 0; k < n; k++)
        {
            gahost::MultiseedResult& out = rs[todo[k]];
            out.status = status[k];
            out.steps = steps[k];
            out.scores.clear();
            out.items.clear();
            out.lengths.clear();
            out.own.clear();
            if (status[k] == GA_CAPACITY && attempt == 0 && (needI[k] > 0 || needT[k] > 0))
            {
                wantItems[todo[k]] = needI[k];
                wantTraces[todo[k]] = needT[k];
                again.push_back(todo[k]);
                continue;
            }
            for (uint32_t t = 0; t < ntr[k]; t++)
            {
                const size_t slot = k * maxTraces + t;
                out.scores.push_back(tscore[slot]);
                out.lengths.push_back(tlen[slot]);
                out.own.insert(out.own.end(), items.begin() + toff[k] + tstart[slot], items.begin() + toff[k] + tstart[slot] + tlen[slot]);
            }
            uint64_t at = 0;
            for (uint32_t t = 0; t < ntr[k]; t++)
            {
                out.items.push_back(out.own.data() + at);
                at += tlen[k * maxTraces + t];
            }
        }
        todo.swap(again);
    }
}

int main(int argc, char** argv)
{
    if (argc < 4) return 1;
    Gag g;
    if (!loadGag(argv[1], g)) return 2;
    ga_host_graph_desc hd {};
    hd.base = ga_graph_desc { (uint32_t)g.h[0], (uint32_t)g.h[1], g.len.data(), g.seq2.data(), g.seqAmb.data(), g.inOff.data(), g.inNb.data(),
        g.outOff.data(), g.outNb.data(), g.lin.data(), g.comp.data() };
    hd.node_ids = g.ids.data(); hd.node_offset = g.off.data(); hd.reverse = g.rev.data();
    hd.chain_number = g.chain.data(); hd.chain_approx_pos = g.chainPos.data();
    hd.num_lookup = (uint32_t)g.lookupIds.size(); hd.lookup_ids = g.lookupIds.data(); hd.original_size = g.origSize.data();
    hd.lookup_offsets = g.lookupOff.data(); hd.lookup_nodes = g.lookupNodes.data(); hd.names = g.namePtr.data();
    gahost::HostGraph graph(hd);
    auto reads = readFasta(argv[2]);
    std::string mode = argv[3];
    if (mode == "table")
    {
        // the k-mer table the lookup kernel probes: every key found with its group, and
        // k-mers that are not in the index not found
        size_t k = std::stoul(argv[4]), w = std::stoul(argv[5]);
        double discard = std::stod(argv[6]);
        gahost::MinimizerIndex idx;
        gahost::buildMinimizerIndex(graph, k, w, 1.0 - discard, idx);
        const uint64_t capacity = gahost::seedTableCapacity(idx);
        std::vector<gadev::SeedSlot> slots(capacity);
        gahost::buildSeedTable(idx, slots.data(), capacity);
        auto find = [&](uint64_t key, gadev::SeedSlot& out)
        {
            uint64_t h = gadev::seed_slot_hash(key) & (capacity - 1);
            for (uint64_t n = 0; n < capacity; n++)
            {
                if (slots[h].key == key) { out = slots[h]; return true; }
                if (slots[h].key == gadev::kEmptyKmer) return false;
                h = (h + 1) & (capacity - 1);
            }
            return false;
        };
        size_t bad = 0, used = 0;
        for (const auto& sl : slots) used += sl.key != gadev::kEmptyKmer;
        for (size_t r = 0; r < idx.keys.size(); r++)
        {
            gadev::SeedSlot sl;
            if (!find(idx.keys[r], sl) || sl.start != idx.startPos[r] || sl.count != idx.startPos[r + 1] - idx.startPos[r]) bad++;
        }
        size_t absentFound = 0, absentTried = 0;
        const uint64_t mask = (k * 2 >= 64) ? ~0ULL : ((1ULL << (k * 2)) - 1);
        for (uint64_t x = 1; absentTried < 100000; x++)
        {
            const uint64_t key = (x * 0x9e3779b97f4a7c15ULL) & mask;
            if (std::binary_search(idx.keys.begin(), idx.keys.end(), key)) continue;
            absentTried++;
            gadev::SeedSlot sl;
            absentFound += find(key, sl);
        }
        std::cout << "keys " << idx.keys.size() << " capacity " << capacity << " used " << used << " bad " << bad
                  << " absent_found " << absentFound << "\n";
        return 0;
    }
    if (mode == "msseeds" || mode == "msseedsdbg")
    {
        // per read: getSeeds, then prepareSeedsForMultiseeding's (slice, split node) pairs
        const bool dbgPreset = mode == "msseedsdbg";
        gahost::MinimizerIndex idx;
        gahost::buildMinimizerIndex(graph, dbgPreset ? 19 : 15, dbgPreset ? 30 : 20, 1.0 - (dbgPreset ? 0.0002 : 0.001), idx);
        std::vector<gahost::KmerMatch> km;
        std::vector<gahost::SeedHit> seeds;
        std::vector<uint32_t> slices, nodes;
        for (const auto& r : reads)
        {
            kmerMatchesHost(idx, r.second, km);
            gahost::selectSeeds(graph, idx, r.second, dbgPreset ? 5 : 10, km, seeds);
            gahost::prepareMultiseeds(graph, seeds, r.second.size(), slices, nodes);
            std::cout << r.first << " " << slices.size();
            for (size_t k = 0; k < slices.size(); k++) std::cout << " " << slices[k] << " " << nodes[k];
            std::cout << "\n";
        }
        return 0;
    }
    if (mode == "indexdump")
    {
        size_t k = std::stoul(argv[4]), w = std::stoul(argv[5]);
        double discard = std::stod(argv[6]);
        gahost::MinimizerIndex idx;
        const auto t0 = std::chrono::steady_clock::now();
        gahost::buildMinimizerIndex(graph, k, w, 1.0 - discard, idx);
        const double ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
        const std::string prefix = argv[7];
        auto dump = [&](const char* ext, const std::vector<uint64_t>& v)
        {
            if (prefix == "-") return;
            std::ofstream f(prefix + ext, std::ios::binary);
            f.write((const char*)v.data(), v.size() * 8);
        };
        dump(".keys", idx.keys);
        dump(".start", idx.startPos);
        dump(".pos", idx.positions);
        // sum of v[i] * (2i + 1) mod 2^64 per array
        auto sum = [](const std::vector<uint64_t>& v)
        {
            uint64_t h = 0;
            for (size_t i = 0; i < v.size(); i++) h += v[i] * (2 * (uint64_t)i + 1);
            return h;
        };
        std::cout << "maxCount " << idx.maxCount << " keys " << idx.keys.size() << " positions " << idx.positions.size() << " sumKeys "
                  << sum(idx.keys) << " sumStart " << sum(idx.startPos) << " sumPos " << sum(idx.positions) << " ms " << (uint64_t)ms
                  << " threads " << std::thread::hardware_concurrency() << "\n";
        return 0;
    }
    if (mode == "walk")
    {
        size_t k = std::stoul(argv[4]), w = std::stoul(argv[5]);
        double discard = std::stod(argv[6]);
        gahost::MinimizerIndex idx;
        gahost::buildMinimizerIndex(graph, k, w, 1.0 - discard, idx);
        gadev::IndexGraph ig {};
        ig.N = graph.N; ig.firstAmbiguous = graph.firstAmbiguous; ig.len = graph.len.data(); ig.seq2 = graph.seq2.data();
        ig.seqAmb = graph.seqAmb.data(); ig.inOff = graph.inOff.data(); ig.inNb = graph.inNb.data(); ig.nodeIds = graph.nodeIds.data();
        ig.nodeOffset = graph.nodeOffset.data(); ig.lookupOff = graph.lookupOff.data(); ig.lookupNodes = graph.lookupNodes.data();
        ig.originalSize = graph.originalSize.data(); ig.numLookup = (uint32_t)graph.lookupIds.size();
        // count pass, then write pass, in node order
        std::vector<uint64_t> first(ig.numLookup + 1, 0);
        bool bad = false;
        for (uint32_t li = 0; li < ig.numLookup; li++) first[li + 1] = first[li] + gadev::node_minimizers(ig, li, k, w, nullptr, nullptr, bad);
        std::vector<uint64_t> kmers(first.back()), pos(first.back());
        for (uint32_t li = 0; li < ig.numLookup; li++)
        {
            const uint32_t n = gadev::node_minimizers(ig, li, k, w, kmers.data() + first[li], pos.data() + first[li], bad);
            if (n != first[li + 1] - first[li]) bad = true;
        }
        // grouped by k-mer, insertion order reversed within a k-mer
        std::vector<uint32_t> order(kmers.size());
        for (size_t i = 0; i < order.size(); i++) order[i] = (uint32_t)i;
        std::stable_sort(order.begin(), order.end(), [&](uint32_t a, uint32_t b) { return kmers[a] < kmers[b]; });
        std::vector<uint64_t> keys, start, positions(order.size());
        for (size_t i = 0; i < order.size(); i++)
        {
            if (i == 0 || kmers[order[i]] != kmers[order[i - 1]])
            {
                keys.push_back(kmers[order[i]]);
                start.push_back(i);
            }
        }
        start.push_back(order.size());
        for (size_t r = 0; r + 1 < start.size(); r++)
            for (size_t j = start[r]; j < start[r + 1]; j++) positions[start[r] + (start[r + 1] - 1 - j)] = pos[order[j]];
        std::cout << "bad " << bad << " occurrences " << kmers.size() << " keys " << keys.size() << " equal "
                  << (keys == idx.keys && start == idx.startPos && positions == idx.positions) << "\n";
        if (getenv("WALK_DEBUG"))
        {
            std::cout << "host occurrences " << idx.positions.size() << " keys " << idx.keys.size() << "\n";
            std::vector<std::pair<uint64_t, uint64_t>> a, b;
            for (size_t i = 0; i < kmers.size(); i++) a.emplace_back(kmers[i], pos[i]);
            for (size_t r = 0; r < idx.keys.size(); r++)
                for (size_t j = idx.startPos[r]; j < idx.startPos[r + 1]; j++) b.emplace_back(idx.keys[r], idx.positions[j]);
            std::sort(a.begin(), a.end());
            std::sort(b.begin(), b.end());
            std::vector<std::pair<uint64_t, uint64_t>> onlyA, onlyB;
            std::set_difference(a.begin(), a.end(), b.begin(), b.end(), std::back_inserter(onlyA));
            std::set_difference(b.begin(), b.end(), a.begin(), a.end(), std::back_inserter(onlyB));
            for (auto& x : onlyA) std::cout << "walk only " << x.first << " node " << (x.second >> 6) << " off " << (x.second & 63) << " nodeOffset " << graph.nodeOffset[x.second >> 6] << " len " << graph.len[x.second >> 6] << "\n";
            for (auto& x : onlyB) std::cout << "host only " << x.first << " node " << (x.second >> 6) << " off " << (x.second & 63) << "\n";
            size_t shown = 0;
            for (size_t i = 0; i < std::min(keys.size(), idx.keys.size()) && shown < 5; i++)
                if (keys[i] != idx.keys[i]) { std::cout << "key " << i << " " << keys[i] << " " << idx.keys[i] << "\n"; shown++; }
        }
        return 0;
    }
    if (mode == "seeds")
    {
        size_t k = std::stoul(argv[4]), w = std::stoul(argv[5]);
        double density = std::stod(argv[6]), discard = std::stod(argv[7]);
        gahost::MinimizerIndex idx;
        gahost::buildMinimizerIndex(graph, k, w, 1.0 - discard, idx);
        std::cout << "maxCount " << idx.maxCount << "\n";
        std::vector<gahost::KmerMatch> km;
        std::vector<gahost::SeedHit> seeds;
        for (auto& r : reads)
        {
            kmerMatchesHost(idx, r.second, km);
            gahost::selectSeeds(graph, idx, r.second, density, km, seeds);
            std::cout << "R " << r.first << " " << seeds.size();
            for (auto& s : seeds) std::cout << " " << s.nodeID << "," << s.nodeOffset << "," << s.seqPos << "," << s.matchLen << "," << s.reverse << "," << s.alignmentGraphNodeId << "," << s.alignmentGraphNodeOffset << "," << s.rawSeedGoodness;
            std::cout << "\n";
            gahost::orderSeeds(graph, seeds);
            std::cout << "O " << r.first << " " << seeds.size();
            for (auto& s : seeds) std::cout << " " << s.nodeID << "," << s.nodeOffset << "," << s.seqPos << "," << s.seedGoodness << "," << s.seedClusterSize;
            std::cout << "\n";
        }
        return 0;
    }
    // gaf (-x vg, AlignerMain.cpp:170-177), gafdbg (-x dbg, AlignerMain.cpp:160-168), gafmix
    // (-x vg with reads joining the seed-loop pool a few per round), gaf2 (-x vg, reads in two
    // groups whose rounds alternate) or gafms / gafmsdbg (--multiseed-DP 1), with the given bandwidth
    const bool perRead = mode == "gafreads" || mode == "gafreadsdbg";
    const bool dbg = mode == "gafdbg" || mode == "gafreadsdbg" || mode == "gafmsdbg";
    const bool multiseed = mode == "gafms" || mode == "gafmsdbg";
    const bool mixed = mode == "gafmix";
    const bool twoLanes = mode == "gaf2";
    const size_t joinPerRound = 7;
    size_t bw = std::stoul(argv[4]);
    uint64_t maxCells = (argc > 5 && std::string(argv[5]) != "-") ? std::stoull(argv[5]) : (dbg ? 10000 : UINT64_MAX);
    gahost::MinimizerIndex idx;
    gahost::buildMinimizerIndex(graph, dbg ? 19 : 15, dbg ? 30 : 20, 1.0 - (dbg ? 0.0002 : 0.001), idx);
    if (perRead)
    {
        const size_t threads = argc > 6 ? std::stoul(argv[6]) : std::max(1u, std::thread::hardware_concurrency());
        gahost::ReadAlignParams p;
        if (dbg) p.seedExtendDensity = 0.002;
        std::vector<gahost::ReadOutput> out(reads.size());
        std::atomic<size_t> next(0);
        std::atomic<uint64_t> bp(0), rounds(0), extensions(0), failed(0);
        const auto t0 = std::chrono::steady_clock::now();
        auto worker = [&]()
        {
            Ctx one { &hd.base, ga_extend_params { (uint32_t)bw, 14705, maxCells, 294 }, 1 };
            std::vector<gahost::KmerMatch> km;
            while (true)
            {
                const size_t i = next.fetch_add(1);
                if (i >= reads.size()) break;
                std::vector<gahost::ReadInput> in(1);
                in[0].name = reads[i].first;
                in[0].seq = reads[i].second;
                kmerMatchesHost(idx, in[0].seq, km);
                gahost::selectSeeds(graph, idx, in[0].seq, dbg ? 5 : 10, km, in[0].seeds);
                std::vector<gahost::ReadOutput> o;
                gahost::BatchStats st;
                gahost::alignBatch(graph, p, in, oracleExtend, &one, o, st);
                out[i] = std::move(o[0]);
                bp += st.bpAligned;
                rounds += st.rounds;
                extensions += st.extensions;
                failed += st.failedReads;
            }
        };
        std::vector<std::thread> pool;
        for (size_t t = 0; t < threads; t++) pool.emplace_back(worker);
        for (auto& t : pool) t.join();
        const double seconds = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
        for (auto& o : out) std::cout << o.gaf;
        std::cerr << "rounds " << rounds << " extensions " << extensions << " bp " << bp << " failed " << failed
                  << " seconds " << seconds << " threads " << threads << std::endl;
        return 0;
    }
    const auto alignStart = std::chrono::steady_clock::now();
    std::vector<gahost::ReadInput> in(reads.size());
    std::vector<gahost::KmerMatch> km;
    for (size_t i = 0; i < reads.size(); i++)
    {
        in[i].name = reads[i].first;
        in[i].seq = reads[i].second;
        kmerMatchesHost(idx, in[i].seq, km);
        gahost::selectSeeds(graph, idx, in[i].seq, dbg ? 5 : 10, km, in[i].seeds);
    }
    if (getenv("GAF_LINE_FORMATTER")) gaf::build_names(graph.lookupIds, graph.names, graph.originalSize, g_gafNames);
    Ctx ctx { &hd.base, ga_extend_params { (uint32_t)bw, 14705, maxCells, 294 } };
    // gafms / gafmsdbg: the oracle's multiseed DPs and backward extensions on this many threads
    if (multiseed && argc > 6) ctx.threads = (int)std::stoul(argv[6]);
    gahost::ReadAlignParams p;
    if (dbg) p.seedExtendDensity = 0.002;
    // GAF_LINE_FORMATTER set: the GAF lines come from gaf_format.cuh through the formatter hook
    if (getenv("GAF_LINE_FORMATTER"))
    {
        p.gafWrite = hostWriter;
        p.select = hostSelect;
    }
    std::vector<gahost::ReadOutput> out;
    gahost::BatchStats st;
    if (mixed)
    {
        // continuous admission: a few reads join the pool before every round, so
        // rounds hold reads at different stages of their seed loops
        gahost::SeedLoopPool pool(graph, p);
        std::vector<gahost::ExtensionRequest> rq;
        std::vector<gahost::ExtensionResult> rs;
        std::vector<std::pair<uint64_t, gahost::ReadOutput>> fin;
        out.assign(in.size(), gahost::ReadOutput {});
        size_t next = 0;
        while (true)
        {
            for (size_t k = 0; k < joinPerRound && next < in.size(); k++, next++) pool.add(std::move(in[next]), next);
            const bool any = pool.collect(rq);
            if (any)
            {
                rs.assign(rq.size(), gahost::ExtensionResult {});
                if (!rq.empty()) oracleExtend(&ctx, rq, rs);
                pool.consume(rs, st);
            }
            pool.takeFinished(fin, st);
            for (auto& f : fin) out[f.first] = std::move(f.second);
            fin.clear();
            if (!any && next == in.size() && pool.active() == 0) break;
        }
    }
    else if (twoLanes)
    {
        Ctx ctx2 = ctx;
        gahost::alignBatchTwoLanes(graph, p, in, oracleExtend, &ctx, &ctx2, out, st);
    }
    else if (multiseed) gahost::alignBatchMultiseed(graph, p, in, oracleMultiseed, &ctx, oracleExtend, &ctx, out, st);
    else gahost::alignBatch(graph, p, in, oracleExtend, &ctx, out, st);
    for (auto& o : out) std::cout << o.gaf;
    const double alignSeconds = std::chrono::duration<double>(std::chrono::steady_clock::now() - alignStart).count();
    std::cerr << "rounds " << st.rounds << " extensions " << st.extensions << " bp " << st.bpAligned << " failed " << st.failedReads
              << " seconds " << alignSeconds << " speculative_used " << st.speculativeUsed << " discarded " << st.speculativeDiscarded
              << " collect_ms " << st.collectMs << " consume_ms " << st.consumeMs << " finish_ms " << st.finishMs << std::endl;
    return 0;
}
