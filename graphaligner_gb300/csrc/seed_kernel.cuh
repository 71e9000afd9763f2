// Device layout of the minimizer index lookup table and the k-mer lookup kernel.
#pragma once
#include <stdint.h>
#include "seed_table.h"

namespace gadev
{
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
}

void ga_launch_seed_lookup(const gadev::SeedTable& t, uint32_t k, uint32_t w, uint32_t numReads, const uint8_t* seq,
    const uint64_t* seqOff, const uint32_t* seqLen, const uint64_t* outOff, gadev::SeedMatch* out, uint32_t* outCount, void* stream);
