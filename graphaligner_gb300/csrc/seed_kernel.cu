// Minimizer index lookup on the GPU (MinimizerSeeder::getSeeds, MinimizerSeeder.cpp:521-537).
//
// One thread walks one read: the rolling 2-bit k-mer of iterateKmers
// (MinimizerSeeder.cpp:59-102, a k-mer is looked up when it differs from the last
// one looked up or that one is at least w-k+1 positions back), a probe into the
// index hash table resident in HBM, and the frequency filter (count < maxCount).
// Matches are written in read order — the order the host's selection step
// (a std::sort by count, MinimizerSeeder.cpp:493-519) needs to see them in.
#include <cuda_runtime.h>
#include <stdint.h>
#include "seed_kernel.cuh"

namespace gadev
{

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
    const uint32_t r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= numReads) return;
    const uint8_t* s = seq + seqOff[r];
    const uint32_t len = seqLen[r];
    SeedMatch* o = out + outOff[r];
    uint32_t n = 0;
    const uint64_t mask = ~(0xFFFFFFFFFFFFFFFFULL << (k * 2));
    const uint64_t realWindow = w - k + 1;
    uint64_t offset = 0;
    // each restart begins a fresh window after a non-ACGT character
    while (true)
    {
        while (offset < len && base_code(s[offset]) < 0) offset++;
        if (offset + k > len) break;
        uint64_t kmer = 0;
        bool restart = false;
        for (uint32_t i = 0; i < k; i++)
        {
            int c = base_code(s[offset + i]);
            if (c < 0)
            {
                offset += i;
                restart = true;
                break;
            }
            kmer = (kmer << 2) | (uint64_t)c;
        }
        if (restart) continue;
        uint32_t st, cnt;
        if (probe(t, kmer, st, cnt) && cnt < t.maxCount) o[n++] = SeedMatch { offset + k - 1, st, cnt };
        uint64_t lastKmer = kmer;
        uint64_t lastPos = offset + k - 1;
        uint64_t i = k;
        for (; offset + i < len; i++)
        {
            int c = base_code(s[offset + i]);
            if (c < 0)
            {
                offset += i;
                restart = true;
                break;
            }
            kmer = ((kmer << 2) & mask) | (uint64_t)c;
            // unsigned arithmetic as in the reference: a wrap-around makes the test true
            if (lastKmer != kmer || lastPos <= offset + i - realWindow)
            {
                if (probe(t, kmer, st, cnt) && cnt < t.maxCount) o[n++] = SeedMatch { offset + i, st, cnt };
                lastKmer = kmer;
                lastPos = offset + i;
            }
        }
        if (!restart) break;
    }
    outCount[r] = n;
}

}

void ga_launch_seed_lookup(const gadev::SeedTable& t, uint32_t k, uint32_t w, uint32_t numReads, const uint8_t* seq,
    const uint64_t* seqOff, const uint32_t* seqLen, const uint64_t* outOff, gadev::SeedMatch* out, uint32_t* outCount, void* stream)
{
    if (numReads == 0) return;
    gadev::seed_lookup_kernel<<<(numReads + 127) / 128, 128, 0, (cudaStream_t)stream>>>(t, k, w, numReads, seq, seqOff, seqLen, outOff, out, outCount);
}
