// Test infrastructure: the reference-side binding of INTEGRATION.md section 2, compiled
// against the reference's own headers (GraphAligner src/) and this repository's C ABI so
// that a compiler checks it.  It is a free function with the arguments and result of
// GraphAlignerBitvectorBanded::getReverseTraceFromSeed (GraphAlignerBitvectorBanded.h:59-76);
// a maintainer pastes its body into that member.  `make -C oracle adapter` compiles it
// (-fsyntax-only: nothing is linked or run).
#define private public
#include "vg.pb.h"
#include "AlignmentGraph.h"
#include "GraphAlignerCommon.h"
#include "ThreadReadAssertion.h"
#undef private
#include <stdexcept>
#include <string_view>
#include <vector>
#include "../include/graphaligner_gb300.h"

using Common = GraphAlignerCommon<size_t, int32_t, uint64_t>;

// one extender per worker thread, like the reference's per-thread AlignerGraphsizedState;
// made once with ga_extender_create(graphHandle, 0, &gpuExtender)
thread_local ga_extender_t gpuExtender = nullptr;

Common::OnewayTrace getReverseTraceFromSeedOnGpu(const Common::Params& params, const std::string_view& sequence, int bigraphNodeId,
    size_t nodeOffset, int Xdropcutoff)
{
    const size_t node = params.graph.GetUnitigNode(bigraphNodeId, nodeOffset);
    uint32_t startNode = (uint32_t)node;
    uint32_t startOffset = (uint32_t)(nodeOffset - params.graph.nodeOffset[node]);
    uint64_t seqOffset = 0, traceOffset = 0;
    uint32_t seqLen = (uint32_t)sequence.size();
    uint32_t cap = seqLen + seqLen / 4 + 512;
    std::vector<uint64_t> items(cap);
    int32_t status = 0, score = 0;
    uint32_t n = 0;
    uint64_t steps = 0;
    ga_extend_batch_desc b { 1, (const uint8_t*)sequence.data(), &seqOffset, &seqLen, &startNode, &startOffset, &traceOffset, &cap };
    ga_extend_results r { &status, &score, &n, items.data(), &steps };
    ga_extend_params p { (uint32_t)params.alignmentBandwidth, Xdropcutoff, params.maxCellsPerSlice, params.XscoreErrorCost };
    if (ga_extend_batch(gpuExtender, &p, &b, &r) != GA_OK) throw std::runtime_error(ga_last_error());
    // a reference assert: raised the reference's way, so the worker drops the read (Aligner.cpp:493-500)
    if (status == GA_ASSERT) ThreadReadAssertion::assertFailed("GPU extension", __FILE__, __LINE__);
    if (status != GA_OK) return Common::OnewayTrace::TraceFailed();
    Common::OnewayTrace result;
    result.score = score;
    result.trace.reserve(n);
    for (uint32_t i = 0; i < n; i++)
    {
        const uint64_t x = items[i];
        const size_t seqPos = GA_TRACE_SEQPOS1(x) == 0 ? (size_t)-1 : (size_t)(GA_TRACE_SEQPOS1(x) - 1);
        result.trace.emplace_back(Common::MatrixPosition { GA_TRACE_NODE(x), GA_TRACE_OFFSET(x), seqPos }, GA_TRACE_SWITCH(x) != 0, sequence,
            params.graph);
    }
    return result;
}
