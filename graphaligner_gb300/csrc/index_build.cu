// Minimizer index of the graph built on the GPU (MinimizerSeeder::initMinimizers and
// initMaxCount with one bucket, MinimizerSeeder.cpp:104-189, 299-491, 557-575).
//
// It produces the arrays of the host build in seeding.cpp, element for element:
//   1. one thread per bigraph node (AlignmentGraph::nodeLookup order) walks the node's
//      sequence over its pieces and reports its window minimizers (iterateMinimizersReal,
//      ties in hash reported together, restarts after non-ACGT characters) from the end
//      of the last piece entered from another bigraph node on (MinimizerSeeder.cpp:323-340),
//      as (k-mer, (split node << 6) | offset).  A counting pass, an exclusive scan and a
//      writing pass lay the occurrences out in node order;
//   2. a stable LSD radix sort by k-mer (8-bit digits) keeps each k-mer's occurrences in
//      insertion order;
//   3. the distinct k-mers and their first occurrences come from a scan of "new k-mer"
//      flags, and each k-mer's occurrences are written in reverse insertion order, as the
//      reference's counting sort leaves them;
//   4. initMaxCount's quantile of the occurrence counts (every k-mer but the last) is read
//      off a device histogram;
//   5. the open-addressing lookup table (seed_table.h) is filled on the device by
//      compare-and-swap claims.
#include <cuda_runtime.h>
#include <algorithm>
#include <stdint.h>
#include <string>
#include <vector>
#include "index_build.h"
#include "index_walk.cuh"

namespace gadev
{

__global__ void count_minimizers_kernel(IndexGraph g, uint32_t k, uint32_t w, uint32_t* counts, uint32_t* error)
{
    const uint32_t li = blockIdx.x * blockDim.x + threadIdx.x;
    if (li >= g.numLookup) return;
    bool bad = false;
    counts[li] = node_minimizers(g, li, k, w, nullptr, nullptr, bad);
    if (bad) atomicOr(error, 1u);
}

__global__ void write_minimizers_kernel(IndexGraph g, uint32_t k, uint32_t w, const uint32_t* first, uint64_t* kmers, uint64_t* positions,
    uint32_t* order, uint32_t* error)
{
    const uint32_t li = blockIdx.x * blockDim.x + threadIdx.x;
    if (li >= g.numLookup) return;
    const uint32_t from = first[li];
    bool bad = false;
    const uint32_t n = node_minimizers(g, li, k, w, kmers + from, positions + from, bad);
    if (bad) atomicOr(error, 1u);
    for (uint32_t i = 0; i < n; i++) order[from + i] = from + i;
}

// ---------------------------------------------------------------- exclusive scan (u32)

static constexpr uint32_t kScanBlock = 1024;   // elements per block: 256 threads x 4

// scans each block's 1024 elements in place and writes the block's total
__global__ void scan_blocks_kernel(uint32_t* data, uint32_t n, uint32_t* blockSums)
{
    __shared__ uint32_t warpTotals[8];
    const uint32_t base = blockIdx.x * kScanBlock + threadIdx.x * 4;
    uint32_t v[4];
    uint32_t local = 0;
#pragma unroll
    for (int q = 0; q < 4; q++)
    {
        v[q] = base + q < n ? data[base + q] : 0;
        local += v[q];
    }
    // inclusive scan of the per-thread totals within the warp, then across the warps
    const uint32_t lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    uint32_t incl = local;
#pragma unroll
    for (uint32_t d = 1; d < 32; d <<= 1)
    {
        const uint32_t t = __shfl_up_sync(0xffffffffu, incl, d);
        if (lane >= d) incl += t;
    }
    if (lane == 31) warpTotals[warp] = incl;
    __syncthreads();
    uint32_t warpBase = 0;
    for (uint32_t q = 0; q < warp; q++) warpBase += warpTotals[q];
    uint32_t running = warpBase + incl - local;
#pragma unroll
    for (int q = 0; q < 4; q++)
    {
        if (base + q < n) data[base + q] = running;
        running += v[q];
    }
    if (threadIdx.x == 255) blockSums[blockIdx.x] = running;
}

__global__ void add_block_offsets_kernel(uint32_t* data, uint32_t n, const uint32_t* offsets)
{
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) data[i] += offsets[i / kScanBlock];
}

// exclusive scan of n values in place; scratch holds the block sums of every level
static cudaError_t exclusive_scan(uint32_t* data, uint32_t n, cudaStream_t s, std::vector<uint32_t*>& scratch)
{
    if (n == 0) return cudaSuccess;
    const uint32_t blocks = (n + kScanBlock - 1) / kScanBlock;
    uint32_t* sums = nullptr;
    cudaError_t e = cudaMallocAsync((void**)&sums, (size_t)blocks * 4, s);
    if (e != cudaSuccess) return e;
    scratch.push_back(sums);
    scan_blocks_kernel<<<blocks, 256, 0, s>>>(data, n, sums);
    if (blocks > 1)
    {
        e = exclusive_scan(sums, blocks, s, scratch);
        if (e != cudaSuccess) return e;
        add_block_offsets_kernel<<<(n + 255) / 256, 256, 0, s>>>(data, n, sums);
    }
    return cudaGetLastError();
}

// ---------------------------------------------------------------- stable LSD radix sort

static constexpr uint32_t kSortThreads = 256;
static constexpr uint32_t kSortRounds = 16;
static constexpr uint32_t kSortTile = kSortThreads * kSortRounds;   // 4096 items per block

// digit histogram of each block's tile, digit-major: hist[d * blocks + b]
__global__ void sort_histogram_kernel(const uint64_t* key, uint32_t n, uint32_t shift, uint32_t* hist)
{
    __shared__ uint32_t h[256];
    h[threadIdx.x] = 0;
    __syncthreads();
    const uint32_t base = blockIdx.x * kSortTile;
    for (uint32_t r = 0; r < kSortRounds; r++)
    {
        const uint32_t i = base + r * kSortThreads + threadIdx.x;
        if (i < n) atomicAdd(&h[(key[i] >> shift) & 255], 1u);
    }
    __syncthreads();
    hist[threadIdx.x * gridDim.x + blockIdx.x] = h[threadIdx.x];
}

// scatters each block's tile to its digits' places, keeping the input order within a digit:
// items are taken 256 at a time in order, and an item's place among its round's items of
// the same digit is the number of them before it (match within the warp, then the earlier
// warps' counts)
__global__ void sort_scatter_kernel(const uint64_t* key, const uint32_t* val, uint32_t n, uint32_t shift, const uint32_t* offsets,
    uint64_t* keyOut, uint32_t* valOut)
{
    __shared__ uint32_t running[256];
    __shared__ uint32_t warpCount[kSortThreads / 32][256];
    const uint32_t lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    running[threadIdx.x] = offsets[threadIdx.x * gridDim.x + blockIdx.x];
    const uint32_t base = blockIdx.x * kSortTile;
    for (uint32_t r = 0; r < kSortRounds; r++)
    {
        for (uint32_t q = 0; q < kSortThreads / 32; q++) warpCount[q][threadIdx.x] = 0;
        __syncthreads();
        const uint32_t i = base + r * kSortThreads + threadIdx.x;
        const bool live = i < n;
        const uint64_t kk = live ? key[i] : 0;
        const uint32_t d = live ? (uint32_t)((kk >> shift) & 255) : 256 + lane;   // dead items match nothing live
        const uint32_t peers = __match_any_sync(0xffffffffu, d);
        const uint32_t rankInWarp = __popc(peers & ((1u << lane) - 1));
        if (live && rankInWarp == 0) warpCount[warp][d] = __popc(peers);
        __syncthreads();
        if (live)
        {
            uint32_t before = 0;
            for (uint32_t q = 0; q < warp; q++) before += warpCount[q][d];
            const uint32_t to = running[d] + before + rankInWarp;
            keyOut[to] = kk;
            valOut[to] = val[i];
        }
        __syncthreads();
        uint32_t total = 0;
        for (uint32_t q = 0; q < kSortThreads / 32; q++) total += warpCount[q][threadIdx.x];
        running[threadIdx.x] += total;
        __syncthreads();
    }
}

// ---------------------------------------------------------------- groups, table

__global__ void new_kmer_flags_kernel(const uint64_t* kmers, uint32_t n, uint32_t* flags)
{
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) flags[i] = (i == 0 || kmers[i] != kmers[i - 1]) ? 1u : 0u;
}

// rank = exclusive scan of the flags: distinct k-mer r starts at the i whose flag is set
__global__ void group_starts_kernel(const uint64_t* kmers, const uint32_t* rank, uint32_t n, uint64_t* keys, uint64_t* startPos)
{
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    if (i == 0 || kmers[i] != kmers[i - 1])
    {
        keys[rank[i]] = kmers[i];
        startPos[rank[i]] = i;
    }
}

// occurrence j of a group [from, to) goes to from + (to - 1 - j): reverse insertion order
__global__ void reverse_groups_kernel(const uint64_t* kmers, const uint32_t* rank, const uint32_t* order, const uint64_t* positions,
    const uint64_t* startPos, uint32_t n, uint64_t* out)
{
    const uint32_t j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= n) return;
    const uint32_t r = rank[j] - ((j == 0 || kmers[j] != kmers[j - 1]) ? 0u : 1u);
    const uint64_t from = startPos[r], to = startPos[r + 1];
    out[from + (to - 1 - j)] = positions[order[j]];
}

// histogram of the occurrence counts of every k-mer id but the last (counts at or above
// `cap` go to the last bin)
__global__ void count_histogram_kernel(const uint64_t* startPos, uint32_t numCounts, uint32_t cap, uint32_t* hist)
{
    const uint32_t r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= numCounts) return;
    const uint64_t c = startPos[r + 1] - startPos[r];
    atomicAdd(&hist[c < cap ? c : cap], 1u);
}

__global__ void fill_table_kernel(const uint64_t* keys, const uint64_t* startPos, uint32_t numKeys, SeedSlot* slots, uint64_t capacity)
{
    const uint32_t r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= numKeys) return;
    const uint64_t key = keys[r];
    uint64_t h = seed_slot_hash(key) & (capacity - 1);
    // every slot a key's probe passes was claimed before it looks, so lookups find it
    // whatever order the claims come in
    for (uint64_t probe = 0; probe < capacity; probe++)
    {
        const unsigned long long prev = atomicCAS((unsigned long long*)&slots[h].key, (unsigned long long)kEmptyKmer, (unsigned long long)key);
        if (prev == kEmptyKmer)
        {
            slots[h].start = (uint32_t)startPos[r];
            slots[h].count = (uint32_t)(startPos[r + 1] - startPos[r]);
            return;
        }
        h = (h + 1) & (capacity - 1);
    }
}

}

namespace
{
template <typename T>
cudaError_t up(const std::vector<T>& v, T** out, cudaStream_t s, std::vector<void*>& keep)
{
    *out = nullptr;
    cudaError_t e = cudaMallocAsync((void**)out, std::max<size_t>(v.size(), 1) * sizeof(T), s);
    if (e != cudaSuccess) return e;
    keep.push_back(*out);
    return v.empty() ? cudaSuccess : cudaMemcpyAsync(*out, v.data(), v.size() * sizeof(T), cudaMemcpyHostToDevice, s);
}
}

int ga_build_index_gpu(const gahost::HostGraph& hg, size_t k, size_t w, double keepLeastFrequentFraction, gahost::MinimizerIndex& idx,
    gadev::SeedSlot** slotsOut, uint64_t* capacityOut, std::string& error)
{
    using namespace gadev;
    idx.k = k;
    idx.w = w;
    idx.maxCount = 0;
    *slotsOut = nullptr;
    *capacityOut = 0;
    if (w < k || w - k + 1 > kMaxRealWindow || k == 0 || k > 31)
    {
        error = "minimizer length 1..31 and a window of at most 64 minimizer positions";
        return -1;
    }
    if (hg.bpSize >= ((size_t)1 << 31))
    {
        error = "graphs of 2^31 bp or more are not indexed on the GPU";
        return -1;
    }
    cudaStream_t s = nullptr;
    if (cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking) != cudaSuccess)
    {
        error = "index build: stream";
        return -2;
    }
    std::vector<void*> keep;           // device buffers freed at the end
    std::vector<uint32_t*> scanScratch;
    auto release = [&]()
    {
        for (void* p : keep) cudaFreeAsync(p, s);
        for (uint32_t* p : scanScratch) cudaFreeAsync(p, s);
        keep.clear();
        scanScratch.clear();
        cudaStreamSynchronize(s);
        cudaStreamDestroy(s);
    };
    auto fail = [&](const char* what, cudaError_t e) -> int
    {
        error = std::string("index build: ") + what + (e != cudaSuccess ? std::string(": ") + cudaGetErrorString(e) : std::string());
        release();
        return e != cudaSuccess ? -2 : -1;
    };
#define IDX_CUDA(call, what) do { cudaError_t _e = (call); if (_e != cudaSuccess) return fail(what, _e); } while (0)
    IndexGraph g {};
    g.N = hg.N;
    g.firstAmbiguous = hg.firstAmbiguous;
    g.numLookup = (uint32_t)hg.lookupIds.size();
    uint32_t *len, *inOff, *inNb, *nodeOffset, *lookupOff, *lookupNodes, *originalSize;
    uint64_t *seq2, *seqAmb;
    int32_t* nodeIds;
    IDX_CUDA(up(hg.len, &len, s, keep), "graph upload");
    IDX_CUDA(up(hg.seq2, &seq2, s, keep), "graph upload");
    IDX_CUDA(up(hg.seqAmb, &seqAmb, s, keep), "graph upload");
    IDX_CUDA(up(hg.inOff, &inOff, s, keep), "graph upload");
    IDX_CUDA(up(hg.inNb, &inNb, s, keep), "graph upload");
    IDX_CUDA(up(hg.nodeIds, &nodeIds, s, keep), "graph upload");
    IDX_CUDA(up(hg.nodeOffset, &nodeOffset, s, keep), "graph upload");
    IDX_CUDA(up(hg.lookupOff, &lookupOff, s, keep), "graph upload");
    IDX_CUDA(up(hg.lookupNodes, &lookupNodes, s, keep), "graph upload");
    IDX_CUDA(up(hg.originalSize, &originalSize, s, keep), "graph upload");
    g.len = len; g.seq2 = seq2; g.seqAmb = seqAmb; g.inOff = inOff; g.inNb = inNb; g.nodeIds = nodeIds;
    g.nodeOffset = nodeOffset; g.lookupOff = lookupOff; g.lookupNodes = lookupNodes; g.originalSize = originalSize;

    // 1. minimizers per bigraph node: count, scan, write
    const uint32_t numLookup = g.numLookup;
    uint32_t *first = nullptr, *errorFlag = nullptr;
    IDX_CUDA(cudaMallocAsync((void**)&first, ((size_t)numLookup + 1) * 4, s), "counts");
    keep.push_back(first);
    IDX_CUDA(cudaMallocAsync((void**)&errorFlag, 4, s), "flag");
    keep.push_back(errorFlag);
    IDX_CUDA(cudaMemsetAsync(errorFlag, 0, 4, s), "flag");
    IDX_CUDA(cudaMemsetAsync(first + numLookup, 0, 4, s), "counts");
    if (numLookup) count_minimizers_kernel<<<(numLookup + 127) / 128, 128, 0, s>>>(g, (uint32_t)k, (uint32_t)w, first, errorFlag);
    IDX_CUDA(cudaGetLastError(), "minimizer count");
    // counts in [0, numLookup), 0 at numLookup: the exclusive scan leaves the total there
    IDX_CUDA(exclusive_scan(first, numLookup + 1, s, scanScratch), "scan");
    uint32_t total = 0, bad = 0;
    IDX_CUDA(cudaMemcpyAsync(&total, first + numLookup, 4, cudaMemcpyDeviceToHost, s), "total");
    IDX_CUDA(cudaMemcpyAsync(&bad, errorFlag, 4, cudaMemcpyDeviceToHost, s), "flag");
    IDX_CUDA(cudaStreamSynchronize(s), "minimizer count");
    if (bad) return fail("the pieces of a bigraph node do not tile it in order", cudaSuccess);
    const uint32_t n = total;
    uint64_t *kmers, *positions, *kmers2;
    uint32_t *order, *order2;
    const size_t cells = std::max<size_t>(n, 1);
    IDX_CUDA(cudaMallocAsync((void**)&kmers, cells * 8, s), "occurrences"); keep.push_back(kmers);
    IDX_CUDA(cudaMallocAsync((void**)&positions, cells * 8, s), "occurrences"); keep.push_back(positions);
    IDX_CUDA(cudaMallocAsync((void**)&kmers2, cells * 8, s), "occurrences"); keep.push_back(kmers2);
    IDX_CUDA(cudaMallocAsync((void**)&order, cells * 4, s), "occurrences"); keep.push_back(order);
    IDX_CUDA(cudaMallocAsync((void**)&order2, cells * 4, s), "occurrences"); keep.push_back(order2);
    if (numLookup) write_minimizers_kernel<<<(numLookup + 127) / 128, 128, 0, s>>>(g, (uint32_t)k, (uint32_t)w, first, kmers, positions, order, errorFlag);
    IDX_CUDA(cudaGetLastError(), "minimizer write");

    // 2. stable LSD radix sort of (k-mer, occurrence) by the k-mer's 2k bits
    const uint32_t sortBlocks = std::max<uint32_t>(1, (n + kSortTile - 1) / kSortTile);
    uint32_t* hist;
    IDX_CUDA(cudaMallocAsync((void**)&hist, (size_t)sortBlocks * 256 * 4, s), "sort"); keep.push_back(hist);
    for (uint32_t shift = 0; shift < 2 * k && n > 0; shift += 8)
    {
        sort_histogram_kernel<<<sortBlocks, kSortThreads, 0, s>>>(kmers, n, shift, hist);
        IDX_CUDA(cudaGetLastError(), "sort histogram");
        IDX_CUDA(exclusive_scan(hist, sortBlocks * 256, s, scanScratch), "sort scan");
        sort_scatter_kernel<<<sortBlocks, kSortThreads, 0, s>>>(kmers, order, n, shift, hist, kmers2, order2);
        IDX_CUDA(cudaGetLastError(), "sort scatter");
        std::swap(kmers, kmers2);
        std::swap(order, order2);
    }

    // 3. distinct k-mers, their first occurrences, occurrences in reverse insertion order
    uint32_t* rank;
    IDX_CUDA(cudaMallocAsync((void**)&rank, (cells + 1) * 4, s), "groups"); keep.push_back(rank);
    IDX_CUDA(cudaMemsetAsync(rank + n, 0, 4, s), "groups");
    if (n) new_kmer_flags_kernel<<<(n + 255) / 256, 256, 0, s>>>(kmers, n, rank);
    IDX_CUDA(exclusive_scan(rank, n + 1, s, scanScratch), "group scan");
    uint32_t numKeys = 0;
    IDX_CUDA(cudaMemcpyAsync(&numKeys, rank + n, 4, cudaMemcpyDeviceToHost, s), "groups");
    IDX_CUDA(cudaStreamSynchronize(s), "groups");
    uint64_t *keys, *startPos, *posOut;
    IDX_CUDA(cudaMallocAsync((void**)&keys, std::max<size_t>(numKeys, 1) * 8, s), "groups"); keep.push_back(keys);
    IDX_CUDA(cudaMallocAsync((void**)&startPos, ((size_t)numKeys + 1) * 8, s), "groups"); keep.push_back(startPos);
    IDX_CUDA(cudaMallocAsync((void**)&posOut, cells * 8, s), "groups"); keep.push_back(posOut);
    const uint64_t total64 = n;
    IDX_CUDA(cudaMemcpyAsync(startPos + numKeys, &total64, 8, cudaMemcpyHostToDevice, s), "groups");
    if (n)
    {
        group_starts_kernel<<<(n + 255) / 256, 256, 0, s>>>(kmers, rank, n, keys, startPos);
        reverse_groups_kernel<<<(n + 255) / 256, 256, 0, s>>>(kmers, rank, order, positions, startPos, n, posOut);
    }
    IDX_CUDA(cudaGetLastError(), "groups");

    // 4. initMaxCount: the count at the keep fraction of the sorted counts of every id but the
    // last, plus one (MinimizerSeeder.cpp:557-575)
    const uint32_t kCap = 1u << 16;
    uint32_t* countHist;
    IDX_CUDA(cudaMallocAsync((void**)&countHist, ((size_t)kCap + 1) * 4, s), "max count"); keep.push_back(countHist);
    IDX_CUDA(cudaMemsetAsync(countHist, 0, ((size_t)kCap + 1) * 4, s), "max count");
    const uint32_t numCounts = numKeys >= 2 ? numKeys - 1 : 0;
    if (numCounts) count_histogram_kernel<<<(numCounts + 255) / 256, 256, 0, s>>>(startPos, numCounts, kCap, countHist);
    IDX_CUDA(cudaGetLastError(), "max count");

    // host copies: the selection step reads positions; keys and start positions are kept with them
    idx.keys.resize(numKeys);
    idx.startPos.resize((size_t)numKeys + 1);
    idx.positions.resize(n);
    std::vector<uint32_t> countHistHost(kCap + 1);
    if (numKeys) IDX_CUDA(cudaMemcpyAsync(idx.keys.data(), keys, (size_t)numKeys * 8, cudaMemcpyDeviceToHost, s), "copy back");
    IDX_CUDA(cudaMemcpyAsync(idx.startPos.data(), startPos, ((size_t)numKeys + 1) * 8, cudaMemcpyDeviceToHost, s), "copy back");
    if (n) IDX_CUDA(cudaMemcpyAsync(idx.positions.data(), posOut, (size_t)n * 8, cudaMemcpyDeviceToHost, s), "copy back");
    IDX_CUDA(cudaMemcpyAsync(countHistHost.data(), countHist, ((size_t)kCap + 1) * 4, cudaMemcpyDeviceToHost, s), "copy back");

    // 5. the lookup table, on the device
    uint64_t capacity = 16;
    while (capacity < 2 * (uint64_t)numKeys) capacity <<= 1;
    SeedSlot* slots = nullptr;
    IDX_CUDA(cudaMalloc((void**)&slots, capacity * sizeof(SeedSlot)), "table");
    cudaError_t e = cudaMemsetAsync(slots, 0xff, capacity * sizeof(SeedSlot), s);   // every key kEmptyKmer
    if (e == cudaSuccess && numKeys) fill_table_kernel<<<(numKeys + 255) / 256, 256, 0, s>>>(keys, startPos, numKeys, slots, capacity);
    if (e == cudaSuccess) e = cudaGetLastError();
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e != cudaSuccess)
    {
        cudaFree(slots);
        return fail("table", e);
    }
    if (numCounts)
    {
        size_t index = (size_t)(numCounts * keepLeastFrequentFraction);
        if (index == numCounts) index = numCounts - 1;
        size_t seen = 0;
        bool done = false;
        for (uint32_t c = 0; c < kCap && !done; c++)
        {
            seen += countHistHost[c];
            if (seen > index)
            {
                idx.maxCount = c + 1;
                done = true;
            }
        }
        if (!done)
        {
            // the quantile lies among counts of 2^16 or more: sort those counts on the host
            std::vector<uint64_t> big;
            for (uint32_t r = 0; r < numCounts; r++)
                if (idx.startPos[r + 1] - idx.startPos[r] >= kCap) big.push_back(idx.startPos[r + 1] - idx.startPos[r]);
            std::sort(big.begin(), big.end());
            idx.maxCount = big[index - seen] + 1;
        }
    }
    release();
    *slotsOut = slots;
    *capacityOut = capacity;
    return 0;
#undef IDX_CUDA
}
