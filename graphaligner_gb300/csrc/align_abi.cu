// C ABI of the read-level alignment flow (ga_aligner_*): host orchestration in
// readalign.cpp / seeding.cpp, k-mer lookups in seed_kernel.cu, extensions in
// extend.cu through ga_extend_batch.
#include <cuda_runtime.h>
#include <algorithm>
#include <chrono>
#include <cstring>
#include <memory>
#include <string>
#include <vector>
#include "readalign.h"
#include "seed_kernel.cuh"
#include "extend.cuh"
#include "index_build.h"
#include "aligner.h"
#include "../../include/graphaligner_gb300.h"

// below this many reads a batch runs on one extender (a round would be too small to split)
static constexpr uint32_t kTwoLaneMinReads = 256;

static double ms_since(std::chrono::steady_clock::time_point t)
{
    return std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t).count();
}

void ga_aligner_extend(void* ctx, const std::vector<gahost::ExtensionRequest>& rq, std::vector<gahost::ExtensionResult>& rs)
{
    ExtendLane* a = (ExtendLane*)ctx;
    const size_t n = rq.size();
    const auto tStage = std::chrono::steady_clock::now();
    bool ok = a->off.reserve(n) && a->len.reserve(n) && a->node.reserve(n) && a->nodeOff.reserve(n) && a->cap.reserve(n)
        && a->toff.reserve(n) && a->status.reserve(n) && a->score.reserve(n) && a->tlen.reserve(n) && a->steps.reserve(n);
    uint64_t total = 0, totalItems = 0;
    for (size_t i = 0; ok && i < n; i++)
    {
        a->off[i] = total;
        a->len[i] = rq[i].len;
        a->node[i] = rq[i].node;
        a->nodeOff[i] = rq[i].nodeOffset;
        a->cap[i] = rq[i].len + rq[i].len / 4 + 512;
        a->toff[i] = totalItems;
        total += rq[i].len;
        totalItems += a->cap[i];
    }
    ok = ok && a->blob.reserve(std::max<uint64_t>(total, 1)) && a->items.reserve(std::max<uint64_t>(totalItems, 1));
    int rc = GA_ERR_CUDA;
    if (ok)
    {
        gahost::parallelFor(n, [&](size_t i) { memcpy(a->blob.data() + a->off[i], rq[i].seq, rq[i].len); });
        ga_extend_batch_desc b { (uint32_t)n, a->blob.data(), a->off.data(), a->len.data(), a->node.data(), a->nodeOff.data(), a->toff.data(), a->cap.data() };
        ga_extend_results r { a->status.data(), a->score.data(), a->tlen.data(), a->items.data(), a->steps.data() };
        a->stagingMs += ms_since(tStage);
        auto t0 = std::chrono::steady_clock::now();
        rc = ga_extend_batch(a->ext, a->params, &b, &r);
        a->extendMs += ms_since(t0);
        a->launches++;
    }
    else
    {
        ga_set_last_error("extension staging: pinned host memory");
    }
    for (size_t i = 0; i < n; i++)
    {
        if (rc != GA_OK)
        {
            rs[i].status = GA_CAPACITY;
            continue;
        }
        rs[i].status = a->status[i];
        rs[i].score = a->score[i];
        rs[i].steps = a->steps[i];
        rs[i].itemPtr = a->items.data() + a->toff[i];
        rs[i].itemCount = a->tlen[i];
    }
}

// The multiseed DP of a group of reads through ga_multiseed_batch_exact: every read's traces
// in the extender's buffers, which the results point into until the next call.
void ga_aligner_multiseed(void* ctx, const std::vector<gahost::MultiseedRequest>& rq, std::vector<gahost::MultiseedResult>& rs)
{
    MultiseedLane* m = (MultiseedLane*)ctx;
    const auto t0 = std::chrono::steady_clock::now();
    const size_t n = rq.size();
    m->off.assign(n, 0); m->len.assign(n, 0); m->seedOff.assign(n + 1, 0);
    m->slices.clear(); m->nodes.clear(); m->blob.clear();
    for (size_t k = 0; k < n; k++)
    {
        const auto& q = rq[k];
        m->off[k] = m->blob.size();
        m->blob.insert(m->blob.end(), q.seq, q.seq + q.len);
        m->len[k] = q.len;
        m->slices.insert(m->slices.end(), q.slices, q.slices + q.numSeeds);
        m->nodes.insert(m->nodes.end(), q.nodes, q.nodes + q.numSeeds);
        m->seedOff[k + 1] = m->slices.size();
    }
    if (m->blob.empty()) m->blob.push_back(0);
    ga_multiseed_batch_desc b { (uint32_t)n, m->blob.data(), m->off.data(), m->len.data(), m->seedOff.data(),
        m->slices.empty() ? nullptr : m->slices.data(), m->nodes.empty() ? nullptr : m->nodes.data(), nullptr, nullptr, 0,
        m->multimapScoreFraction };
    ga_multiseed_output o {};
    const int rc = ga_multiseed_batch_exact(m->ext, m->params, &b, &o);
    float kernelMs = 0;
    if (rc == GA_OK && ga_extender_last_kernel_ms(m->ext, &kernelMs) == GA_OK) m->kernelMs += kernelMs;
    uint64_t candidates = 0, walks = 0, traces = 0;
    uint32_t rounds = 0;
    if (rc == GA_OK && ga_extender_last_multiseed_counts(m->ext, &candidates, &walks, &traces, &rounds) == GA_OK)
    {
        m->candidates += candidates;
        m->walks += walks;
        m->traces += traces;
        m->rounds += rounds;
    }
    for (size_t k = 0; k < n; k++)
    {
        gahost::MultiseedResult& out = rs[k];
        out.status = rc == GA_OK ? o.status[k] : GA_CAPACITY;
        out.steps = rc == GA_OK ? o.cell_steps[k] : 0;
        out.scores.clear();
        out.items.clear();
        out.lengths.clear();
        out.own.clear();
        out.deduplicated = true;
        if (out.status != GA_OK) continue;
        for (uint32_t t = 0; t < o.num_traces[k]; t++)
        {
            const uint64_t i = o.trace_first[k] + t;
            out.scores.push_back(o.trace_score[i]);
            out.items.push_back(o.trace_items + o.trace_start[i]);
            out.lengths.push_back(o.trace_len[i]);
        }
    }
    m->ms += ms_since(t0);
}

int ga_aligner_second_lane(ga_aligner* a)
{
    ExtendLane& l = a->lanes[1];
    if (l.ext) return GA_OK;
    int rc = ga_extender_create_like(a->ext, &l.ext);
    if (rc != GA_OK) return rc;
    l.owned = true;
    l.params = &a->params.extend;
    return GA_OK;
}

gahost::ReadAlignParams ga_aligner_read_params(const ga_aligner* a)
{
    gahost::ReadAlignParams rp;
    rp.sloppy = a->params.sloppy != 0;
    rp.minClusterSize = a->params.min_cluster_size;
    rp.seedExtendDensity = a->params.seed_extend_density;
    rp.xscoreErrorCost = a->params.extend.xscore_error_cost;
    rp.minAlignmentScore = a->params.min_alignment_score;
    rp.multimapScoreFraction = a->params.multimap_score_fraction;
    rp.cigarMatchMismatchMerge = a->params.cigar_match_mismatch != 0;
    // selection and GAF lines on the device
    rp.gafWrite = ga_gaf_device_write;
    rp.gafCtx = const_cast<GafDevice*>(&a->gafDev);
    rp.select = ga_gaf_device_select;
    rp.selectCtx = const_cast<GafDevice*>(&a->gafDev);
    return rp;
}

int ga_aligner_seed(ga_aligner* a, uint32_t n, const char* const* names, const uint8_t* seq, const uint64_t* seqOffset,
    const uint32_t* seqLen, std::vector<gahost::ReadInput>& reads)
{
    const auto t0 = std::chrono::steady_clock::now();
    reads.assign(n, gahost::ReadInput {});
    if (n == 0) return GA_OK;
    uint64_t seqBytes = 0, matchSlots = 0;
    std::vector<uint64_t> matchOff(n);
    for (uint32_t i = 0; i < n; i++)
    {
        seqBytes = std::max<uint64_t>(seqBytes, seqOffset[i] + seqLen[i]);
        matchOff[i] = matchSlots;
        matchSlots += seqLen[i];
    }
    if (!a->dSeq.reserve(std::max<uint64_t>(seqBytes, 1)) || !a->dOff.reserve(n) || !a->dMatchOff.reserve(n)
        || !a->dLen.reserve(n) || !a->dCount.reserve(n) || !a->dMatch.reserve(std::max<uint64_t>(matchSlots, 1)))
    {
        ga_set_last_error("seeding: device buffers for seeding");
        return GA_ERR_CUDA;
    }
    uint8_t* dSeq = a->dSeq.p;
    uint64_t *dOff = a->dOff.p, *dMatchOff = a->dMatchOff.p;
    uint32_t *dLen = a->dLen.p, *dCount = a->dCount.p;
    gadev::SeedMatch* dMatch = a->dMatch.p;
    cudaMemcpyAsync(dSeq, seq, seqBytes, cudaMemcpyHostToDevice, a->stream);
    cudaMemcpyAsync(dOff, seqOffset, n * 8ULL, cudaMemcpyHostToDevice, a->stream);
    cudaMemcpyAsync(dMatchOff, matchOff.data(), n * 8ULL, cudaMemcpyHostToDevice, a->stream);
    cudaMemcpyAsync(dLen, seqLen, n * 4ULL, cudaMemcpyHostToDevice, a->stream);
    gadev::SeedTable table { a->slots, a->capacity, (uint32_t)std::min<uint64_t>(a->index.maxCount, 0xffffffffu) };
    ga_launch_seed_lookup(table, a->params.minimizer_length, a->params.minimizer_window, n, dSeq, dOff, dLen, dMatchOff, dMatch, dCount, a->stream);
    std::vector<uint32_t> counts(n);
    // one slot per read base, of which only the first counts[i] of each read are read below
    // (pinned and reused: a pageable copy of 16 B per read base costs more than the lookups)
    if (!a->hMatch.reserve(std::max<uint64_t>(matchSlots, 1)))
    {
        ga_set_last_error("seeding: pinned host buffer for the k-mer matches");
        return GA_ERR_CUDA;
    }
    const gadev::SeedMatch* matches = a->hMatch.data();
    cudaMemcpyAsync(counts.data(), dCount, n * 4ULL, cudaMemcpyDeviceToHost, a->stream);
    cudaMemcpyAsync(a->hMatch.data(), dMatch, std::max<uint64_t>(matchSlots, 1) * sizeof(gadev::SeedMatch), cudaMemcpyDeviceToHost, a->stream);
    cudaError_t e = cudaStreamSynchronize(a->stream);
    if (e != cudaSuccess)
    {
        ga_set_last_error("seeding: seed lookup kernel failed");
        return GA_ERR_CUDA;
    }
    a->stats.seed_lookup_ms = ms_since(t0);
    const auto t1 = std::chrono::steady_clock::now();
    gahost::parallelFor(n, [&](size_t i)
    {
        reads[i].name = names[i] ? names[i] : "";
        reads[i].seq.assign((const char*)seq + seqOffset[i], seqLen[i]);
        std::vector<gahost::KmerMatch> km(counts[i]);
        for (uint32_t k = 0; k < counts[i]; k++)
        {
            const auto& m = matches[matchOff[i] + k];
            km[k] = gahost::KmerMatch { m.pos, m.start, m.count };
        }
        gahost::selectSeeds(*a->graph, a->index, reads[i].seq, a->params.minimizer_density, km, reads[i].seeds);
    });
    a->stats.seed_select_ms = ms_since(t1);
    return GA_OK;
}

extern "C" int ga_aligner_create(ga_extender_t ext, const ga_host_graph_desc* graph, const ga_align_params* params, ga_aligner_t* out)
{
    if (!ext || !graph || !params || !out) return GA_ERR_ARGUMENT;
    if (params->minimizer_length == 0 || params->minimizer_length > 31 || params->minimizer_window < params->minimizer_length)
    {
        ga_set_last_error("ga_aligner_create: minimizer length must be 1..31 and at most the window size");
        return GA_ERR_ARGUMENT;
    }
    ga_aligner* a = new ga_aligner();
    a->ext = ext;
    a->lanes[0].ext = ext;
    a->lanes[0].params = &a->params.extend;
    a->params = *params;
    cudaGetDevice(&a->device);
    try
    {
        a->graph = new gahost::HostGraph(*graph);
    }
    catch (...)
    {
        delete a;
        ga_set_last_error("ga_aligner_create: the graph is inconsistent");
        return GA_ERR_ARGUMENT;
    }
    // minimizer index and its open-addressing lookup table, built on the GPU; the table
    // stays resident for the lookup kernel, the index's arrays come back for seed selection
    const auto t0 = std::chrono::steady_clock::now();
    std::string why;
    uint64_t capacity = 0;
    const int built = ga_build_index_gpu(*a->graph, params->minimizer_length, params->minimizer_window, 1.0 - params->minimizer_discard_fraction,
        a->index, &a->slots, &capacity, why);
    if (built != 0 || cudaStreamCreateWithFlags(&a->stream, cudaStreamNonBlocking) != cudaSuccess)
    {
        if (a->slots) cudaFree(a->slots);
        delete a->graph;
        delete a;
        ga_set_last_error(("ga_aligner_create: " + (built != 0 ? why : std::string("stream creation failed"))).c_str());
        return built == -1 ? GA_ERR_ARGUMENT : GA_ERR_CUDA;
    }
    a->indexBuildMs = ms_since(t0);
    if (ga_gaf_device_init(a->gafDev, *a->graph) != GA_OK)
    {
        cudaFree(a->slots);
        delete a->graph;
        delete a;
        ga_set_last_error("ga_aligner_create: uploading the node names failed");
        return GA_ERR_CUDA;
    }
    a->capacity = capacity;
    *out = a;
    return GA_OK;
}

extern "C" int ga_aligner_index(ga_aligner_t a, ga_index_info* info, uint64_t* keys, uint64_t* start_pos, uint64_t* positions)
{
    if (!a || !info) return GA_ERR_ARGUMENT;
    info->minimizer_length = a->index.k;
    info->minimizer_window = a->index.w;
    info->max_count = a->index.maxCount;
    info->num_keys = a->index.keys.size();
    info->num_positions = a->index.positions.size();
    info->table_capacity = a->capacity;
    info->build_ms = a->indexBuildMs;
    if (keys && !a->index.keys.empty()) std::memcpy(keys, a->index.keys.data(), a->index.keys.size() * 8);
    if (start_pos) std::memcpy(start_pos, a->index.startPos.data(), a->index.startPos.size() * 8);
    if (positions && !a->index.positions.empty()) std::memcpy(positions, a->index.positions.data(), a->index.positions.size() * 8);
    return GA_OK;
}

extern "C" int ga_aligner_free(ga_aligner_t a)
{
    if (!a) return GA_OK;
    if (a->slots) cudaFree(a->slots);
    if (a->stream) cudaStreamDestroy(a->stream);
    delete a->graph;
    delete a;
    return GA_OK;
}

extern "C" int ga_align_reads(ga_aligner_t a, uint32_t n, const char* const* names, const uint8_t* seq, const uint64_t* seqOffset, const uint32_t* seqLen)
{
    if (!a || (n > 0 && (!names || !seq || !seqOffset || !seqLen))) return GA_ERR_ARGUMENT;
    for (uint32_t i = 0; i < n; i++)
    {
        if (seqLen[i] > GA_MAX_SEQ_LEN)
        {
            ga_set_last_error(("ga_align_reads: read " + std::to_string(i) + " is longer than GA_MAX_SEQ_LEN (33,554,431 bp)").c_str());
            return GA_ERR_ARGUMENT;
        }
    }
    auto start = std::chrono::steady_clock::now();
    a->stats = ga_align_stats {};
    a->stats.reads = n;
    a->gaf.clear();
    a->readBp.assign(n, 0);
    if (n == 0) return GA_OK;
    // ---- k-mer lookups on the GPU, seed selection on the host ----
    auto ts = std::chrono::steady_clock::now();
    std::vector<gahost::ReadInput> reads;
    int rc = ga_aligner_seed(a, n, names, seq, seqOffset, seqLen, reads);
    if (rc != GA_OK) return rc;
    for (const auto& r : reads) if (!r.seeds.empty()) a->stats.reads_with_seeds++;
    a->stats.seed_ms = ms_since(ts);
    // ---- seed loops, extensions on the GPU ----
    gahost::ReadAlignParams rp = ga_aligner_read_params(a);
    std::vector<gahost::ReadOutput> outs;
    gahost::BatchStats bs;
    for (auto& l : a->lanes) { l.extendMs = 0; l.stagingMs = 0; }
    // two groups of reads on two extenders, the host finishing one group's round while
    // the other's runs on the GPU; small batches use one
    a->multiseed.ms = 0;
    a->multiseed.kernelMs = 0;
    a->multiseed.candidates = 0;
    a->multiseed.walks = 0;
    a->multiseed.traces = 0;
    a->multiseed.rounds = 0;
    if (a->params.multiseed_dp)
    {
        a->multiseed.ext = a->ext;
        a->multiseed.params = &a->params.extend;
        a->multiseed.multimapScoreFraction = a->params.multimap_score_fraction;
        gahost::alignBatchMultiseed(*a->graph, rp, reads, ga_aligner_multiseed, &a->multiseed, ga_aligner_extend, &a->lanes[0], outs, bs);
    }
    else if (n >= kTwoLaneMinReads && ga_aligner_second_lane(a) == GA_OK)
        gahost::alignBatchTwoLanes(*a->graph, rp, reads, ga_aligner_extend, &a->lanes[0], &a->lanes[1], outs, bs);
    else
        gahost::alignBatch(*a->graph, rp, reads, ga_aligner_extend, &a->lanes[0], outs, bs);
    a->stats.extend_ms = a->lanes[0].extendMs + a->lanes[1].extendMs + a->multiseed.ms;
    size_t gafBytes = 0;
    for (uint32_t i = 0; i < n; i++) gafBytes += outs[i].gaf.size();
    a->gaf.reserve(gafBytes);
    for (uint32_t i = 0; i < n; i++)
    {
        a->gaf += outs[i].gaf;
        a->readBp[i] = outs[i].bpAligned;
        if (outs[i].alignments > 0) a->stats.reads_aligned++;
    }
    a->stats.collect_ms = bs.collectMs;
    a->stats.staging_ms = a->lanes[0].stagingMs + a->lanes[1].stagingMs;
    a->stats.consume_ms = bs.consumeMs;
    a->stats.finish_ms = bs.finishMs;
    a->stats.speculative_used = bs.speculativeUsed;
    a->stats.speculative_discarded = bs.speculativeDiscarded;
    a->stats.failed_reads = bs.failedReads;
    a->stats.bp_aligned = bs.bpAligned;
    a->stats.rounds = bs.rounds;
    a->stats.extensions = bs.extensions;
    a->stats.cell_steps = bs.cellSteps;
    a->stats.multiseed_kernel_ms = a->multiseed.kernelMs;
    a->stats.multiseed_candidates = a->multiseed.candidates;
    a->stats.multiseed_walks = a->multiseed.walks;
    a->stats.multiseed_traces = a->multiseed.traces;
    a->stats.multiseed_rounds = a->multiseed.rounds;
    // with two lanes the GPU calls overlap host work: host_ms is what they do not cover
    a->stats.host_ms = std::max(0.0, ms_since(start) - a->stats.extend_ms);
    return GA_OK;
}

extern "C" int ga_aligner_gaf(ga_aligner_t a, const char** text, uint64_t* bytes)
{
    if (!a || !text || !bytes) return GA_ERR_ARGUMENT;
    *text = a->gaf.c_str();
    *bytes = a->gaf.size();
    return GA_OK;
}

extern "C" int ga_aligner_get_seeds(ga_aligner_t a, uint32_t n, const uint8_t* seq, const uint64_t* seqOffset,
    const uint32_t* seqLen, const ga_seed** seeds, const uint64_t** seedOffsets)
{
    if (!a || !seeds || !seedOffsets || (n > 0 && (!seq || !seqOffset || !seqLen))) return GA_ERR_ARGUMENT;
    for (uint32_t i = 0; i < n; i++)
    {
        if (seqLen[i] > GA_MAX_SEQ_LEN)
        {
            ga_set_last_error(("ga_aligner_get_seeds: read " + std::to_string(i) + " is longer than GA_MAX_SEQ_LEN (33,554,431 bp)").c_str());
            return GA_ERR_ARGUMENT;
        }
    }
    cudaSetDevice(a->device);
    std::vector<const char*> names(n, nullptr);
    std::vector<gahost::ReadInput> reads;
    int rc = ga_aligner_seed(a, n, names.data(), seq, seqOffset, seqLen, reads);
    if (rc != GA_OK) return rc;
    a->seedOffsets.assign(n + 1, 0);
    for (uint32_t i = 0; i < n; i++) a->seedOffsets[i + 1] = a->seedOffsets[i] + reads[i].seeds.size();
    a->seeds.resize(std::max<uint64_t>(a->seedOffsets[n], 1));
    for (uint32_t i = 0; i < n; i++)
    {
        ga_seed* o = a->seeds.data() + a->seedOffsets[i];
        for (const auto& h : reads[i].seeds)
        {
            *o++ = ga_seed { h.nodeID, h.reverse ? 1u : 0u, (uint64_t)h.nodeOffset, (uint64_t)h.seqPos, (uint32_t)h.matchLen,
                (uint32_t)h.rawSeedGoodness, (uint32_t)h.alignmentGraphNodeId, (uint32_t)h.alignmentGraphNodeOffset };
        }
    }
    *seeds = a->seeds.data();
    *seedOffsets = a->seedOffsets.data();
    return GA_OK;
}

extern "C" int ga_aligner_read_bp(ga_aligner_t a, uint64_t* bp)
{
    if (!a || !bp) return GA_ERR_ARGUMENT;
    std::copy(a->readBp.begin(), a->readBp.end(), bp);
    return GA_OK;
}

extern "C" int ga_aligner_stats(ga_aligner_t a, ga_align_stats* out)
{
    if (!a || !out) return GA_ERR_ARGUMENT;
    *out = a->stats;
    return GA_OK;
}
