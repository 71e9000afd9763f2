// Minimizer index lookup on the GPU (MinimizerSeeder::getSeeds, MinimizerSeeder.cpp:521-537).
//
// One warp walks one read, 32 positions per step (lane j: position base + j):
//   - the bases come in as one coalesced 32-byte load;
//   - the k-mer ending at each position is built by a shuffle-doubling pack of the
//     2-bit codes (five steps) on top of the previous step's last k-mer;
//   - a position holds a k-mer when the last non-ACGT character lies at least k
//     positions back (a ballot finds the last one at or before each lane);
//   - iterateKmers (MinimizerSeeder.cpp:59-102) looks a k-mer up when it is the first
//     after a restart, differs from the last one looked up, or that one is at least
//     w-k+1 positions back (unsigned, so every position below w-k+1 qualifies).  The last
//     one looked up always holds the previous position's k-mer, so a k-mer that differs
//     from its predecessor is looked up; only in a step that holds a repeat of its
//     predecessor (a homopolymer longer than k) are the positions resolved in order;
//   - the 32 lookups probe the index hash table resident in HBM independently, and the
//     matches with count < maxCount are compacted by ballot and prefix popcount and
//     written in read order, the order the host's selection (a std::sort by count,
//     MinimizerSeeder.cpp:493-519) needs.
#include <cuda_runtime.h>
#include <stdint.h>
#include "seed_kernel.cuh"

namespace gadev
{

static constexpr unsigned kAllLanes = 0xffffffffu;

__device__ __forceinline__ int base_code(uint8_t c)
{
    switch (c)
    {
        case 'a': case 'A': return 0;
        case 'c': case 'C': return 1;
        case 'g': case 'G': return 2;
        case 't': case 'T': return 3;
    }
    return -1;
}

__device__ __forceinline__ bool probe(const SeedTable& t, uint64_t kmer, uint32_t& start, uint32_t& count)
{
    uint64_t h = seed_slot_hash(kmer) & (t.capacity - 1);
#pragma unroll 1
    for (uint64_t n = 0; n < t.capacity; n++)
    {
        const SeedSlot s = t.slots[h];
        if (s.key == kEmptyKmer) return false;
        if (s.key == kmer)
        {
            start = s.start;
            count = s.count;
            return true;
        }
        h = (h + 1) & (t.capacity - 1);
    }
    return false;
}

__global__ void __launch_bounds__(128) seed_lookup_kernel(SeedTable t, uint32_t k, uint32_t w, uint32_t numReads,
    const uint8_t* seq, const uint64_t* seqOff, const uint32_t* seqLen, const uint64_t* outOff, SeedMatch* out, uint32_t* outCount)
{
    const uint32_t lane = threadIdx.x & 31;
    const uint32_t r = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
    if (r >= numReads) return;   // warp-uniform
    const uint8_t* s = seq + seqOff[r];
    const int64_t len = seqLen[r];
    SeedMatch* o = out + outOff[r];
    const uint64_t mask = ~(0xFFFFFFFFFFFFFFFFULL << (k * 2));
    const int64_t realWindow = (int64_t)w - (int64_t)k + 1;
    const uint32_t below = (1u << lane) - 1u;
    uint32_t n = 0;
    uint64_t prevKmer = 0;          // k-mer (2-bit packing) of the position before this step
    int64_t lastInvalid = -1;       // last non-ACGT position before this step (-1: the read start)
    int64_t lastPos = 0;            // position of the last k-mer looked up
#pragma unroll 1
    for (int64_t base = 0; base < len; base += 32)
    {
        const int64_t p = base + lane;
        const int c = p < len ? base_code(s[p]) : -1;
        // last non-ACGT position at or before p (positions past the end count as non-ACGT)
        const uint32_t inv = __ballot_sync(kAllLanes, c < 0);
        const uint32_t invUpTo = inv & (below | (1u << lane));
        const int64_t li = invUpTo ? base + (31 - __clz((int)invUpTo)) : lastInvalid;
        // codes base..p packed, then the k-mer ending at p
        uint64_t packed = c < 0 ? 0 : (uint64_t)c;
#pragma unroll
        for (uint32_t d = 1; d < 32; d <<= 1)
        {
            const uint64_t t2 = __shfl_up_sync(kAllLanes, packed, d);
            if (lane >= d) packed = (t2 << (2 * d)) | packed;
        }
        const uint64_t kmer = ((lane < 31 ? prevKmer << (2 * (lane + 1)) : 0) | packed) & mask;
        const bool valid = p < len && p - li >= (int64_t)k;
        const bool first = valid && p - li == (int64_t)k;
        uint64_t kPrev = __shfl_up_sync(kAllLanes, kmer, 1);
        if (lane == 0) kPrev = prevKmer;
        const bool repeat = valid && !first && kmer == kPrev;
        uint32_t look = __ballot_sync(kAllLanes, valid && !repeat);
        const uint32_t repeats = __ballot_sync(kAllLanes, repeat);
        if (repeats)
        {
            // positions in order: a repeat is looked up when the last lookup lies w-k+1 back
            // (or the position is below w-k+1)
            look = 0;
            const uint32_t validMask = __ballot_sync(kAllLanes, valid);
#pragma unroll 1
            for (uint32_t j = 0; j < 32; j++)
            {
                if (!((validMask >> j) & 1)) continue;
                const int64_t pj = base + j;
                if (!((repeats >> j) & 1) || pj < realWindow || pj - lastPos >= realWindow)
                {
                    look |= 1u << j;
                    lastPos = pj;
                }
            }
        }
        else if (look)
        {
            lastPos = base + (31 - __clz((int)look));
        }
        uint32_t st = 0, cnt = 0;
        const bool found = ((look >> lane) & 1) && probe(t, kmer, st, cnt) && cnt < t.maxCount;
        const uint32_t fm = __ballot_sync(kAllLanes, found);
        if (found) o[n + __popc(fm & below)] = SeedMatch { (uint64_t)p, st, cnt };
        n += __popc(fm);
        prevKmer = __shfl_sync(kAllLanes, kmer, 31);
        lastInvalid = __shfl_sync(kAllLanes, li, 31);
    }
    if (lane == 0) outCount[r] = n;
}

}

void ga_launch_seed_lookup(const gadev::SeedTable& t, uint32_t k, uint32_t w, uint32_t numReads, const uint8_t* seq,
    const uint64_t* seqOff, const uint32_t* seqLen, const uint64_t* outOff, gadev::SeedMatch* out, uint32_t* outCount, void* stream)
{
    if (numReads == 0) return;
    // one warp per read, four per block
    gadev::seed_lookup_kernel<<<(numReads + 3) / 4, 128, 0, (cudaStream_t)stream>>>(t, k, w, numReads, seq, seqOff, seqLen, outOff, out, outCount);
}
