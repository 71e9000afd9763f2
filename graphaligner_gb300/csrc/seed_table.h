// Open-addressing table of the minimizer index's distinct k-mers: the layout the
// k-mer lookup kernel probes (seed_kernel.cu) and the host code that builds it.
#pragma once
#include <stdint.h>

#if defined(__CUDACC__)
#define GA_HOST_DEVICE __host__ __device__
#else
#define GA_HOST_DEVICE
#endif

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

GA_HOST_DEVICE inline uint64_t seed_slot_hash(uint64_t x)
{
    x ^= x >> 33;
    x *= 0xff51afd7ed558ccdULL;
    x ^= x >> 33;
    x *= 0xc4ceb9fe1a85ec53ULL;
    x ^= x >> 33;
    return x;
}
}
