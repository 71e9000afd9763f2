// ga_extend_batch_noalloc: batched seed extension that allocates no device memory.
//
// It serves callers that cannot call cudaMalloc when they extend: processes whose
// device memory is handed out by another allocator under a fixed budget (a
// framework's caching pool owns the GPU), and request paths where the device-wide
// synchronisation of cudaMalloc/cudaFree is not acceptable.  The fill kernel keeps
// its frontier tables in shared memory; the only other scratch the two kernels need --
// work counters, the arena cursors, where each extension's DP table is, and the
// DP-table arena the fill writes and the traceback reads -- lives in the file-scope
// device array below, which every GPU that loads this library holds until the
// process exits.  Inputs and outputs are
// the caller's device buffers.
#include <cuda_runtime.h>
#include <mutex>
#include <stdint.h>
#include "extend.cuh"
#include "../../include/graphaligner_gb300.h"

namespace
{
using namespace gadev;

constexpr u64 kScratchBytes = 128ULL << 20;       // 128 MiB per GPU
constexpr u64 kHeaderBytes = 256;                 // work counters and arena cursors
constexpr u64 kStatesBytes = 4096 * 32;           // where the fill left each extension's table
constexpr u32 kWarpsPerBlock = 4;
constexpr u32 kBlocks = 64;                       // 256 warps
constexpr u32 kMaxExtensions = 4096;              // per call
constexpr u64 kMaxReadBp = 8000000;               // per call, summed over the batch
constexpr int kMaxDevices = 64;

static __device__ __align__(256) uint8_t g_scratch[kScratchBytes];

// the scratch array's device address, per device, looked up once with that device current
void* g_scratchAddress[kMaxDevices] = {};
cudaError_t g_setupError[kMaxDevices] = {};
std::once_flag g_setupOnce[kMaxDevices];

void setup_device(int device)
{
    void* p = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&p, g_scratch);
    if (e == cudaSuccess && !p) e = cudaErrorInvalidSymbol;
    if (e == cudaSuccess && ga_upload_tables() != 0) e = cudaErrorInvalidValue;
    g_setupError[device] = e;
    if (e == cudaSuccess) g_scratchAddress[device] = p;
}

// frontier-table capacities: the shared-memory layout of the regular entry point
Caps small_caps()
{
    Caps c;
    c.band = 32;
    c.hash = 64;
    c.heap = 32;
    c.extras = 64;
    return c;
}
}

extern "C" int ga_extend_batch_noalloc(const ga_graph_desc* device_graph, const ga_extend_params* params,
    const ga_extend_batch_desc* device_batch, ga_extend_results* device_results, void* stream)
{
    if (!device_graph || !params || !device_batch || !device_results)
    {
        ga_set_last_error("ga_extend_batch_noalloc: null argument");
        return GA_ERR_ARGUMENT;
    }
    const u32 n = device_batch->num;
    if (n == 0) return GA_OK;
    if (n > kMaxExtensions)
    {
        ga_set_last_error("ga_extend_batch_noalloc: more than 4096 extensions in one call (the limit of its fixed scratch)");
        return GA_ERR_ARGUMENT;
    }
    const ga_graph_desc& gd = *device_graph;
    const ga_extend_batch_desc& bd = *device_batch;
    const ga_extend_results& rd = *device_results;
    if (!gd.node_length || !gd.seq2bit || !gd.seq_ambiguous || !gd.in_offsets || !gd.in_neighbors || !gd.out_offsets
        || !gd.out_neighbors || !gd.linearizable || !gd.component || !bd.seq || !bd.seq_offset || !bd.seq_len
        || !bd.start_node || !bd.start_offset || !bd.trace_offset || !bd.trace_capacity || !rd.status || !rd.score
        || !rd.trace_len || !rd.trace_items)
    {
        ga_set_last_error("ga_extend_batch_noalloc: null array in the graph, batch or result description");
        return GA_ERR_ARGUMENT;
    }
    int device = 0;
    if (cudaGetDevice(&device) != cudaSuccess || device < 0 || device >= kMaxDevices)
    {
        ga_set_last_error("ga_extend_batch_noalloc: no current CUDA device (or ordinal above 63)");
        return GA_ERR_CUDA;
    }
    std::call_once(g_setupOnce[device], setup_device, device);
    if (g_setupError[device] != cudaSuccess)
    {
        ga_set_last_error("ga_extend_batch_noalloc: looking up the scratch array or loading the IUPAC table failed");
        return GA_ERR_CUDA;
    }
    uint8_t* scratch = (uint8_t*)g_scratchAddress[device];
    cudaStream_t s = (cudaStream_t)stream;
    // the batch must stay within the per-call limit: read the lengths back into a fixed host buffer
    static thread_local uint32_t lengths[kMaxExtensions];
    if (cudaMemcpyAsync(lengths, bd.seq_len, (size_t)n * 4, cudaMemcpyDeviceToHost, s) != cudaSuccess
        || cudaStreamSynchronize(s) != cudaSuccess)
    {
        ga_set_last_error("ga_extend_batch_noalloc: reading the sequence lengths back failed");
        return GA_ERR_CUDA;
    }
    u64 totalBp = 0;
    for (u32 i = 0; i < n; i++) totalBp += lengths[i];
    if (totalBp > kMaxReadBp)
    {
        ga_set_last_error("ga_extend_batch_noalloc: more than 8,000,000 read bp in one call (the limit of its fixed scratch)");
        return GA_ERR_ARGUMENT;
    }
    // every call starts from zeroed counters: the array keeps what the previous call left in it
    if (cudaMemsetAsync(scratch, 0, kHeaderBytes, s) != cudaSuccess)
    {
        ga_set_last_error("ga_extend_batch_noalloc: clearing the scratch counters failed");
        return GA_ERR_CUDA;
    }

    DevGraph g;
    g.N = gd.num_nodes;
    g.firstAmbiguous = gd.first_ambiguous;
    g.len = gd.node_length;
    g.seq2 = gd.seq2bit;
    g.seqAmb = gd.seq_ambiguous;
    g.inOff = gd.in_offsets;
    g.inNb = gd.in_neighbors;
    g.outOff = gd.out_offsets;
    g.outNb = gd.out_neighbors;
    g.lin = gd.linearizable;
    g.comp = gd.component;

    const u64 arenaBytes = kScratchBytes - kHeaderBytes - kStatesBytes;
    FillArgs fa {};
    fa.g = g;
    fa.bandwidth = params->bandwidth;
    fa.xdrop = params->xdrop;
    fa.maxCells = params->max_cells_per_slice;
    fa.cost = params->xscore_error_cost;
    fa.num = n;
    fa.order = nullptr;
    fa.seq = bd.seq;
    fa.seqOff = bd.seq_offset;
    fa.seqLen = bd.seq_len;
    fa.startNode = bd.start_node;
    fa.startOffset = bd.start_offset;
    fa.arena = scratch + kHeaderBytes + kStatesBytes;
    fa.arenaBytes = arenaBytes;
    fa.arenaCursor = (unsigned long long*)(scratch + 16);
    fa.chunkBytes = 16 * 1024;
    fa.workspace = nullptr;
    fa.caps = small_caps();
    fa.workspaceStride = ga_warp_tables_bytes(fa.caps);
    fa.prevStatus = nullptr;
    fa.states = (ExtState*)(scratch + kHeaderBytes);

    TraceArgs ta {};
    ta.g = g;
    ta.cost = params->xscore_error_cost;
    ta.seq = bd.seq;
    ta.seqOff = bd.seq_offset;
    ta.seqLen = bd.seq_len;
    ta.arena = fa.arena;
    ta.traceOffset = bd.trace_offset;
    ta.traceCap = bd.trace_capacity;
    ta.status = rd.status;
    ta.score = rd.score;
    ta.traceLen = rd.trace_len;
    ta.traceItems = rd.trace_items;
    ta.cellSteps = rd.cell_steps;
    ta.num = n;
    ta.order = nullptr;
    ta.prevStatus = nullptr;
    ta.states = fa.states;

    if (ga_launch_extend(fa, ta, (u32*)scratch, (int)kBlocks, (int)kBlocks, (int)kWarpsPerBlock, s) != 0)
    {
        ga_set_last_error("ga_extend_batch_noalloc: kernel launch failed");
        return GA_ERR_CUDA;
    }
    return GA_OK;
}
