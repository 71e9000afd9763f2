// Host-side types of the read-level layer (readalign.cpp, seeding.cpp).
#pragma once
#include "gaf_format.cuh"
#include <cstdint>
#include <functional>
#include <memory>
#include <string>
#include <unordered_map>
#include <vector>
#include "../../include/graphaligner_gb300.h"
#include "seed_table.h"

namespace gahost
{

// AlignmentGraph fields the host logic reads (AlignmentGraph.h:121-139)
struct HostGraph
{
    explicit HostGraph(const ga_host_graph_desc& d);
    uint32_t N;
    uint32_t firstAmbiguous;
    std::vector<uint32_t> len, inOff, inNb, outOff, outNb, nodeOffset;
    std::vector<uint64_t> seq2, seqAmb, chainNumber, chainApproxPos;
    std::vector<int32_t> nodeIds;
    std::vector<uint8_t> reverse;
    std::vector<int32_t> lookupIds;
    std::vector<uint32_t> originalSize, lookupOff, lookupNodes;
    std::vector<std::string> names;
    std::unordered_map<int, size_t> lookupIndex;
    std::vector<uint32_t> bigSize;      // per split node: originalSize of its bigraph node
    size_t bpSize;
    size_t lookup(int bignode) const;
    char charAt(size_t node, size_t pos) const;
    size_t unitigNode(int bignode, size_t offset) const;
    std::pair<int, size_t> reversePosition(int bignode, size_t offset) const;
    size_t sizeOf(int bignode) const;
    const std::string& nameOf(int bignode) const;
};

// SeedHit (GraphAlignerWrapper.h:11-50)
struct SeedHit
{
    int nodeID = INT32_MIN;
    size_t nodeOffset = SIZE_MAX;
    size_t seqPos = SIZE_MAX;
    size_t matchLen = SIZE_MAX;
    bool reverse = false;
    size_t alignmentGraphNodeId = SIZE_MAX;
    size_t alignmentGraphNodeOffset = SIZE_MAX;
    size_t rawSeedGoodness = 0;
    size_t seedGoodness = 0;
    size_t seedClusterSize = 0;
};

// TraceItem / OnewayTrace (GraphAlignerCommon.h:110-166)
struct TraceItem
{
    size_t node;
    size_t nodeOffset;
    size_t seqPos;
    bool nodeSwitch;
    char seqChar;
    char graphChar;
};

struct OnewayTrace
{
    std::vector<TraceItem> trace;
    int32_t score = 0;
    bool failed() const { return score == INT32_MAX; }
};

// AlignmentResult::AlignmentItem (GraphAlignerCommon.h:289-340)
struct AlignmentItem
{
    std::shared_ptr<OnewayTrace> trace;
    size_t seedGoodness = 0;
    size_t alignmentStart = 0;
    size_t alignmentEnd = 0;
    size_t alignmentScore = SIZE_MAX;
    double alignmentXScore = -1;
    int mappingQuality = 255;
};

// A finished read's GAF lines walked on the host (gaf::classify_line), their text not yet
// written: one record per line, one edit-op byte per trace item, the node-path entries (the
// records' op and entry offsets count from this read's arrays).
struct ClassifiedLines
{
    std::vector<gaf::LineMeta> lines;
    std::vector<uint8_t> ops;
    std::vector<int32_t> entries;
};

// Writes the classified GAF lines of a group of reads (the text half of traceToAlignment,
// GraphAlignerGAFAlignment.h:37-200): read i's lines, each with its newline, back to back into
// text; readEnd[i] = where read i's text ends.  False when it could not run (every read of the
// group then fails).
typedef bool (*GafWriteFn)(void* ctx, const std::vector<const std::string*>& names, const std::vector<const ClassifiedLines*>& reads,
    std::string& text, std::vector<uint64_t>& readEnd);

// AlignmentSelection::SelectAlignments (AlignmentSelection.cpp:31-95) over the alignments of
// a group of reads: read i's are [first[i], first[i+1]) of start/end/xscore, keep[k] = kept.
// False when it could not run (every read of the group then fails).
typedef bool (*SelectFn)(void* ctx, const std::vector<uint64_t>& first, const std::vector<uint64_t>& start, const std::vector<uint64_t>& end,
    const std::vector<double>& xscore, int minAlignmentScore, double fractionCutoff, std::vector<char>& keep);

struct ReadAlignParams
{
    bool sloppy = true;
    size_t minClusterSize = 1;
    double seedExtendDensity = -1;
    int32_t xscoreErrorCost = 294;
    int minAlignmentScore = 0;
    double multimapScoreFraction = 0.9;
    bool cigarMatchMismatchMerge = false;
    // speculative seeds: while a round's estimated work (read bp x the previous round's
    // column steps per extended bp) stays under speculationSteps, each read also sends its
    // next candidate seeds (up to maxSpeculation seeds per read, the extra ones together
    // within the same budget); a speculative result is used only if the seed loop, replayed
    // in order on the read's true state, extends exactly that seed next
    double speculationSteps = 6e7;
    size_t maxSpeculation = 8;
    // GAF lines of finished reads: the host's gafLine when null; else the lines are walked on
    // the host (gaf::classify_line) and this hook writes their text (the product's device writer)
    GafWriteFn gafWrite = nullptr;
    void* gafCtx = nullptr;
    // the selection of finished reads' alignments: selectAlignments on the host when null
    SelectFn select = nullptr;
    void* selectCtx = nullptr;
};

struct ReadInput
{
    std::string name;
    std::string seq;
    std::vector<SeedHit> seeds;
};

struct ReadOutput
{
    std::string gaf;
    size_t bpAligned = 0;
    size_t alignments = 0;
    bool failed = false;     // an assert would have dropped the read
    bool noSeeds = false;
    ClassifiedLines pending; // with a GAF writer: lines waiting for writeFinished
};

struct BatchStats
{
    uint64_t rounds = 0;
    uint64_t extensions = 0;
    uint64_t cellSteps = 0;
    uint64_t bpAligned = 0;
    uint64_t failedReads = 0;
    uint64_t speculativeUsed = 0;       // speculative extensions whose seed the loop then extended
    uint64_t speculativeDiscarded = 0;  // speculative extensions it did not
    double collectMs = 0;      // next seeds and extension requests
    double consumeMs = 0;      // trace decoding, fix-up and merge of every finished seed
    double finishMs = 0;       // selection and GAF of finished reads
};

struct ExtensionRequest
{
    const char* seq;
    uint32_t len;
    int bignode;
    size_t offset;
    uint32_t node;
    uint32_t nodeOffset;
};

struct ExtensionResult
{
    int32_t status = 0;
    int32_t score = 0;
    uint64_t steps = 0;
    std::vector<uint64_t> items;          // packed trace items, owned here ...
    const uint64_t* itemPtr = nullptr;    // ... or held by the extension callback until its next call
    uint64_t itemCount = 0;
    const uint64_t* begin() const { return itemPtr ? itemPtr : items.data(); }
    uint64_t size() const { return itemPtr ? itemCount : items.size(); }
};

// fn(i) for i in [0, n) on the host's cores (serially for small n); fn handles its own errors
void parallelFor(size_t n, const std::function<void(size_t)>& fn);

typedef void (*ExtendFn)(void* ctx, const std::vector<ExtensionRequest>& requests, std::vector<ExtensionResult>& results);

void orderSeeds(const HostGraph& g, std::vector<SeedHit>& seedHits);

// Reads in their seed loops (GraphAligner::AlignOneWay, GraphAligner.h:94-181), advanced
// in lock step: each round asks for the next seed's two extensions of every read.  Reads
// can join between rounds, so a round's extensions mix reads at different stages.
class SeedLoopPool
{
public:
    SeedLoopPool(const HostGraph& g, const ReadAlignParams& p);
    ~SeedLoopPool();
    void add(ReadInput&& read, uint64_t tag);
    // the same for a group of reads, prepared on all cores (reads are moved from)
    void addMany(std::vector<ReadInput>& reads, const std::vector<uint64_t>& tags);
    // reads joined and not yet taken out by takeFinished
    size_t active() const;
    // the next extension requests (they point into the pool's reads); false when no read
    // needs one.  Reads whose seed loop ended move to the finished list.
    bool collect(std::vector<ExtensionRequest>& requests);
    // results of the requests of the last collect, in the same order
    void consume(const std::vector<ExtensionResult>& results, BatchStats& stats);
    // selection, aligned bp and GAF of the finished reads (Aligner.cpp:505-566), with their tags.
    // overlapped: the call runs while another group's extensions hold the GPU, so the
    // selection runs on the host and the GAF text is left for writeFinished.
    void takeFinished(std::vector<std::pair<uint64_t, ReadOutput>>& out, BatchStats& stats, bool overlapped = false);
private:
    struct Impl;
    std::unique_ptr<Impl> impl;
};

// Writes the GAF text of outputs whose lines wait (ReadOutput::pending), in one call of the writer.
void writeFinished(const ReadAlignParams& p, std::vector<std::pair<uint64_t, ReadOutput>>& outs, const std::vector<const std::string*>& names);

void alignBatch(const HostGraph& g, const ReadAlignParams& p, std::vector<ReadInput>& reads, ExtendFn extend, void* ctx,
    std::vector<ReadOutput>& out, BatchStats& stats);
// The same with the reads in two groups, each with its own extension context: while one
// group's round runs (on a worker thread), the caller's thread finishes the other group's
// last round and collects its next requests.  Results are those of alignBatch.
void alignBatchTwoLanes(const HostGraph& g, const ReadAlignParams& p, std::vector<ReadInput>& reads, ExtendFn extend,
    void* ctxA, void* ctxB, std::vector<ReadOutput>& out, BatchStats& stats);

// ---- multiseed DP (--multiseed-DP, Aligner.cpp:461-476) ----

// GraphAligner::prepareSeedsForMultiseeding (GraphAligner.h:211-248): the distinct
// alignment-graph nodes seeded in each 64-row slice of the read, slice by slice, in the
// iteration order of the std::unordered_set the reference collects them in
void prepareMultiseeds(const HostGraph& g, const std::vector<SeedHit>& seeds, size_t seqLen, std::vector<uint32_t>& slices,
    std::vector<uint32_t>& nodes);

// AlignmentSelection::AddMappingQualities (AlignmentSelection.cpp:97-135)
void addMappingQualities(std::vector<AlignmentItem>& alignments);

// One read's multiseed DP: its seeds (prepareMultiseeds) in, its traces out in the
// reference's order, each in DP order (ga_multiseed_batch's contract).
struct MultiseedRequest
{
    const char* seq;
    uint32_t len;
    const uint32_t* slices;
    const uint32_t* nodes;
    uint32_t numSeeds;
};

struct MultiseedResult
{
    int32_t status = 0;
    uint64_t steps = 0;
    std::vector<int32_t> scores;
    // each trace's packed items: in `own`, or in the callback's buffers until its next call
    std::vector<const uint64_t*> items;
    std::vector<uint32_t> lengths;
    std::vector<uint64_t> own;
    bool deduplicated = false;   // removeDuplicateTraces already ran (its order)
};

typedef void (*MultiseedFn)(void* ctx, const std::vector<MultiseedRequest>& requests, std::vector<MultiseedResult>& results);

// AlignMultiseed per read (GraphAligner.h:77-92, 603-629): the multiseed DP, duplicate
// removal, clipping, a backward extension from each trace's start (clipAndAddBackwardTrace,
// :347-373), mapping qualities, then selection and GAF as alignBatch.
void alignBatchMultiseed(const HostGraph& g, const ReadAlignParams& p, std::vector<ReadInput>& reads, MultiseedFn multiseed, void* msCtx,
    ExtendFn extend, void* ctx, std::vector<ReadOutput>& out, BatchStats& stats);

// MinimizerSeeder with one bucket (MinimizerSeeder.h:14-47)
struct MinimizerIndex
{
    size_t k = 15;
    size_t w = 20;
    size_t maxCount = 0;
    std::vector<uint64_t> keys;        // distinct k-mers, sorted (the dense id of a k-mer is its rank)
    std::vector<uint64_t> startPos;    // [keys + 1]
    std::vector<uint64_t> positions;   // (split node << 6) | offset, grouped by id
};

void buildMinimizerIndex(const HostGraph& g, size_t k, size_t w, double keepLeastFrequentFraction, MinimizerIndex& idx);
// Slots of the open-addressing table of idx's distinct k-mers: a power of two, at least
// twice the number of keys.
uint64_t seedTableCapacity(const MinimizerIndex& idx);
// Fills the table (seed_table.h layout: key, first position, count) on all cores.
void buildSeedTable(const MinimizerIndex& idx, gadev::SeedSlot* slots, uint64_t capacity);
// k-mer hits of one read in iterateKmers order: (read position, start, count), count < maxCount
struct KmerMatch { uint64_t pos; uint64_t start; uint64_t count; };
void selectSeeds(const HostGraph& g, const MinimizerIndex& idx, const std::string& seq, double density,
    std::vector<KmerMatch>& matches, std::vector<SeedHit>& out);

}
