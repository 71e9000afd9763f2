// Device layout of the minimizer index lookup table and the k-mer lookup kernel.
#pragma once
#include <stdint.h>

namespace gadev
{
static constexpr uint64_t kEmptyKmer = ~0ULL;   // k <= 31, so no k-mer uses the top bits

// open-addressing slot: a distinct k-mer of the index and its group in `positions`
struct SeedSlot
{
    uint64_t key;
    uint32_t start;
    uint32_t count;
};

struct SeedTable
{
    const SeedSlot* slots;
    uint64_t capacity;     // power of two
    uint32_t maxCount;     // MinimizerSeeder::maxCount
};

// one k-mer hit of a read: read position, first index in `positions`, number of positions
struct SeedMatch
{
    uint64_t pos;
    uint32_t start;
    uint32_t count;
};

__host__ __device__ inline uint64_t seed_slot_hash(uint64_t x)
{
    x ^= x >> 33;
    x *= 0xff51afd7ed558ccdULL;
    x ^= x >> 33;
    x *= 0xc4ceb9fe1a85ec53ULL;
    x ^= x >> 33;
    return x;
}
}

void ga_launch_seed_lookup(const gadev::SeedTable& t, uint32_t k, uint32_t w, uint32_t numReads, const uint8_t* seq,
    const uint64_t* seqOff, const uint32_t* seqLen, const uint64_t* outOff, gadev::SeedMatch* out, uint32_t* outCount, void* stream);
