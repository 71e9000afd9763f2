// Minimizer index of the graph built on the GPU (index_build.cu).
#pragma once
#include <stdint.h>
#include <string>
#include "readalign.h"
#include "seed_table.h"

// Builds idx (keys, start positions, positions, maxCount: the arrays of
// gahost::buildMinimizerIndex) on the current device and leaves the open-addressing
// lookup table of its keys there (*slots, cudaMalloc'd, *capacity slots).  Returns 0,
// -1 for a graph or parameters it cannot index (error says why) or -2 for a CUDA error.
int ga_build_index_gpu(const gahost::HostGraph& g, size_t k, size_t w, double keepLeastFrequentFraction, gahost::MinimizerIndex& idx,
    gadev::SeedSlot** slots, uint64_t* capacity, std::string& error);
