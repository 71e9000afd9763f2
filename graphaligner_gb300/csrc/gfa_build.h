// Alignment graph from GFA text, built natively for the package's Python API
// (graph.build_from_gfa).  Not part of the reference-facing C ABI: a C++ caller of
// the extension path already holds the reference's own AlignmentGraph.
#pragma once
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

// Every array of a built graph (AlignmentGraph fields and nodeLookup), owned by the handle.
typedef struct ga_gfa_graph_arrays {
    uint32_t num_nodes;
    uint32_t first_ambiguous;
    uint32_t num_lookup;
    uint64_t num_in_edges;
    uint64_t num_out_edges;
    uint64_t num_lookup_nodes;
    uint64_t bp_size;
    const uint32_t* node_length;      // [num_nodes]
    const int32_t*  node_ids;         // [num_nodes] bigraph id (GFA id * 2 + strand)
    const uint32_t* node_offset;      // [num_nodes]
    const uint8_t*  reverse;          // [num_nodes]
    const uint8_t*  linearizable;     // [num_nodes]
    const uint32_t* component;        // [num_nodes]
    const uint64_t* chain_number;     // [num_nodes]
    const uint64_t* chain_approx_pos; // [num_nodes]
    const uint64_t* seq2bit;          // [first_ambiguous * 2]
    const uint64_t* seq_ambiguous;    // [(num_nodes - first_ambiguous) * 4]
    const uint32_t* in_offsets;       // [num_nodes + 1]
    const uint32_t* in_neighbors;     // [num_in_edges]
    const uint32_t* out_offsets;      // [num_nodes + 1]
    const uint32_t* out_neighbors;    // [num_out_edges]
    const int32_t*  lookup_ids;       // [num_lookup]
    const uint32_t* original_size;    // [num_lookup]
    const uint32_t* lookup_offsets;   // [num_lookup + 1]
    const uint32_t* lookup_nodes;     // [num_lookup_nodes]
    const char*     names;            // num_lookup NUL-terminated names back to back ("" = numeric GFA id)
    uint64_t        names_bytes;
} ga_gfa_graph_arrays;

// Builds the graph of `bytes` bytes of GFA text.  GA_ERR_ARGUMENT (message in
// ga_last_error) for a GFA the builder cannot take: an unknown segment in a link, an
// overlap not smaller than both segments, an empty segment, a character outside the
// IUPAC codes, an id that does not fit.  *handle must be released by ga_gfa_free.
int ga_gfa_build(const char* text, uint64_t bytes, void** handle, ga_gfa_graph_arrays* out);
void ga_gfa_free(void* handle);

#ifdef __cplusplus
}
#endif
