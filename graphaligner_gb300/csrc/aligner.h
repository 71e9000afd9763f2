// State of one read-level aligner (ga_aligner_t) shared by align_abi.cu and serve.cpp.
#pragma once
#include <cuda_runtime.h>
#include <algorithm>
#include <string>
#include <vector>
#include "readalign.h"
#include "seed_kernel.cuh"
#include "gaf_format.cuh"
#include "../../include/graphaligner_gb300.h"

// pinned host staging, grown as needed, never cleared
template <typename T>
struct Pinned
{
    T* p = nullptr;
    size_t cap = 0;
    bool reserve(size_t n)
    {
        if (n <= cap) return true;
        size_t want = std::max(n, cap + cap / 2);
        void* q = nullptr;
        if (cudaHostAlloc(&q, want * sizeof(T), cudaHostAllocDefault) != cudaSuccess) return false;
        if (p) cudaFreeHost(p);
        p = (T*)q;
        cap = want;
        return true;
    }
    void release() { if (p) cudaFreeHost(p); p = nullptr; cap = 0; }
    T* data() { return p; }
    T& operator[](size_t i) { return p[i]; }
};

// device buffers that only grow (cudaFree synchronises the device, so a steady state
// must not allocate: a serving loop seeds new reads while other lanes' rounds run)
template <typename T>
struct DevGrow
{
    T* p = nullptr;
    size_t cap = 0;
    bool reserve(size_t n)
    {
        if (n <= cap) return true;
        size_t want = std::max(n, cap + cap / 2);
        void* q = nullptr;
        if (cudaMalloc(&q, want * sizeof(T)) != cudaSuccess) return false;
        if (p) cudaFree(p);
        p = (T*)q;
        cap = want;
        return true;
    }
    void release() { if (p) cudaFree(p); p = nullptr; cap = 0; }
};

// One extender and the staging of its batches: ga_aligner_extend's context.  Two lanes
// let one group of reads extend on the GPU while the host finishes the other group.
struct ExtendLane
{
    ga_extender_t ext = nullptr;
    bool owned = false;        // created by the aligner (the second lane), freed with it
    const ga_extend_params* params = nullptr;
    Pinned<uint8_t> blob;
    Pinned<uint64_t> off, toff, items, steps;
    Pinned<uint32_t> len, node, nodeOff, cap, tlen;
    Pinned<int32_t> status, score;
    double extendMs = 0;       // ga_extend_batch calls
    double stagingMs = 0;      // packing requests and handing results over
    uint64_t launches = 0;
    ~ExtendLane()
    {
        blob.release(); off.release(); toff.release(); items.release(); steps.release();
        len.release(); node.release(); nodeOff.release(); cap.release(); tlen.release();
        status.release(); score.release();
        if (owned && ext) ga_extender_free(ext);
    }
};

// host staging of ga_multiseed_batch calls
struct MultiseedLane
{
    ga_extender_t ext = nullptr;
    const ga_extend_params* params = nullptr;
    double multimapScoreFraction = 0.9;
    std::vector<uint8_t> blob;
    std::vector<uint64_t> off, seedOff;
    std::vector<uint32_t> len, slices, nodes;
    double ms = 0;
    double kernelMs = 0;                   // of ms: the batch's kernels and trace copies
    uint64_t candidates = 0, walks = 0, traces = 0, rounds = 0;   // local maxima, walks, kept traces, rounds
};

// The device GAF formatter and alignment selection (gaf_device.cu): the graph's node names
// resident, the staging of one group of lines.
struct GafDevice
{
    int device = 0;
    cudaStream_t stream = nullptr;
    // node names by nodeLookup index, the bigraph-id lookup, node sizes
    DevGrow<uint8_t> nodeNames;
    DevGrow<uint64_t> nodeNameOff;
    DevGrow<uint32_t> originalSize, idVal;
    DevGrow<int32_t> idKey;
    uint64_t idCap = 0;
    gaf::NamesHost host;                  // the same tables on the host (node sizes for the classification)
    // one chunk of lines
    Pinned<uint8_t> hOps, hNames;
    Pinned<gaf::LineMeta> hMeta;
    Pinned<int32_t> hEntries;
    Pinned<uint64_t> hNameOff, hStart;
    Pinned<uint32_t> hLen32;
    Pinned<int64_t> hLen;
    DevGrow<uint8_t> ops, names;
    DevGrow<gaf::LineMeta> meta;
    DevGrow<int32_t> entries;
    DevGrow<uint64_t> nameOff, start;
    DevGrow<uint32_t> readLen;
    DevGrow<int64_t> len;
    DevGrow<char> text;
    // selection
    Pinned<uint64_t> hSel;
    Pinned<double> hScore;
    Pinned<char> hKeep;
    DevGrow<uint64_t> sel;
    DevGrow<double> score;
    DevGrow<char> keep;
    std::string lastText;                  // ga_aligner_format_gaf's output
    std::vector<uint64_t> lastEnds;
    std::vector<uint8_t> lastFailed;
    double ms = 0;
    void release()
    {
        nodeNames.release(); nodeNameOff.release(); originalSize.release(); idVal.release(); idKey.release();
        hOps.release(); hNames.release(); hMeta.release(); hEntries.release(); hNameOff.release(); hStart.release(); hLen32.release(); hLen.release();
        ops.release(); names.release(); meta.release(); entries.release(); nameOff.release(); start.release(); readLen.release(); len.release();
        text.release();
        hSel.release(); hScore.release(); hKeep.release(); sel.release(); score.release(); keep.release();
        if (stream) cudaStreamDestroy(stream);
        stream = nullptr;
    }
};

// uploads the graph's names (at aligner creation); GA_OK or an error code
int ga_gaf_device_init(GafDevice& d, const gahost::HostGraph& g);
// gahost::GafWriteFn and gahost::SelectFn on the device (ctx = GafDevice*)
bool ga_gaf_device_write(void* ctx, const std::vector<const std::string*>& names, const std::vector<const gahost::ClassifiedLines*>& reads,
    std::string& text, std::vector<uint64_t>& readEnd);
bool ga_gaf_device_select(void* ctx, const std::vector<uint64_t>& first, const std::vector<uint64_t>& start, const std::vector<uint64_t>& end,
    const std::vector<double>& xscore, int minAlignmentScore, double fractionCutoff, std::vector<char>& keep);

struct ga_aligner
{
    ga_extender_t ext = nullptr;
    int device = 0;
    ga_align_params params {};
    gahost::HostGraph* graph = nullptr;
    gahost::MinimizerIndex index;
    gadev::SeedSlot* slots = nullptr;
    uint64_t capacity = 0;
    double indexBuildMs = 0;   // ga_aligner_create's index build on the GPU, copies included
    std::string gaf;
    std::vector<uint64_t> readBp;
    ga_align_stats stats {};
    cudaStream_t stream = nullptr;
    ExtendLane lanes[2];       // lanes[0] uses ext; lanes[1] an extender made like it on first use
    MultiseedLane multiseed;   // the multiseed DP's calls (on ext)
    GafDevice gafDev;          // GAF lines and alignment selection on the device
    // k-mer lookup buffers
    DevGrow<uint8_t> dSeq;
    DevGrow<uint64_t> dOff, dMatchOff;
    DevGrow<uint32_t> dLen, dCount;
    DevGrow<gadev::SeedMatch> dMatch;
    Pinned<gadev::SeedMatch> hMatch;   // the matches copied back (one slot per read base)
    std::vector<ga_seed> seeds;         // ga_aligner_get_seeds' output
    std::vector<uint64_t> seedOffsets;
    ~ga_aligner()
    {
        dSeq.release(); dOff.release(); dMatchOff.release(); dLen.release(); dCount.release(); dMatch.release();
        hMatch.release();
        gafDev.release();
    }
};

// MinimizerSeeder::getSeeds for a batch of reads: k-mer lookups on the GPU, the
// least-frequent selection on the host.  Fills reads[i].name/seq/seeds.
int ga_aligner_seed(ga_aligner* a, uint32_t n, const char* const* names, const uint8_t* seq, const uint64_t* seqOffset,
    const uint32_t* seqLen, std::vector<gahost::ReadInput>& reads);

// gahost::ExtendFn over ga_extend_batch (ctx = ExtendLane*)
void ga_aligner_extend(void* ctx, const std::vector<gahost::ExtensionRequest>& rq, std::vector<gahost::ExtensionResult>& rs);

// the second lane's extender (same device graph, arena size and launch shape as the first)
int ga_aligner_second_lane(ga_aligner* a);

// the seed loop parameters of ga_align_params
gahost::ReadAlignParams ga_aligner_read_params(const ga_aligner* a);
