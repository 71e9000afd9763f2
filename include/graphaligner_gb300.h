/*
 * graphaligner_gb300 — C ABI of the GB300 seed-extension path.
 *
 * These entry points replace GraphAligner's seed-extension hot path behind its
 * own C++ API.  Every call returns an int status (GA_OK on success) and never
 * throws; device buffers belong to the handles.  All inputs and outputs are
 * host pointers with explicit sizes unless a name says "device".
 *
 * Reference interfaces replaced (paths inside the GraphAligner project):
 *   ga_graph_upload      AlignmentGraph device-visible fields, built by
 *                        AlignmentGraph::Finalize (src/AlignmentGraph.h:121-139,
 *                        src/AlignmentGraph.cpp:252-296)
 *   ga_extend_batch      GraphAlignerBitvectorBanded::getReverseTraceFromSeed
 *                        (src/GraphAlignerBitvectorBanded.h:59-76), called twice
 *                        per seed by GraphAligner::getTwoDirectionalTrace
 *                        (src/GraphAligner.h:475-520)
 *   ga_aligner_create    the MinimizerSeeder index (src/MinimizerSeeder.cpp:299-491)
 *   ga_align_reads       the per-read body of runComponentMappings: getSeeds, AlignOneWay,
 *                        SelectAlignments and the GAF line (src/Aligner.cpp:443-592)
 *   ga_server_*          the worker loop around it, as a submit/poll request interface
 */
#ifndef GRAPHALIGNER_GB300_H
#define GRAPHALIGNER_GB300_H

#include <stdint.h>
#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

/* status codes */
#define GA_OK              0
#define GA_TRACE_FAILED    1   /* OnewayTrace::TraceFailed(): score INT32_MAX (GraphAlignerCommon.h:154-163) */
#define GA_ASSERT          2   /* a reference assert would have thrown ThreadReadAssertion::AssertionFailure */
#define GA_CAPACITY        3   /* a per-extension device capacity (band, queue, trace, arena) was exceeded */
#define GA_BAD_REQUEST     4
#define GA_ERR_ARGUMENT   -1
#define GA_ERR_CUDA       -2
#define GA_ERR_NOMEM      -3
#define GA_ERR_STATE      -4

/* The AlignmentGraph fields the DP reads, as plain arrays.  Node indices are the
 * AlignmentGraph's split-node indices (<= 64 bp per node).  Nodes below
 * first_ambiguous carry 2-bit sequence (two 64-bit chunks of 32 bp, A=0 C=1 G=2
 * T=3, AlignmentGraph.cpp:111-139); nodes from first_ambiguous on carry four
 * 64-bit masks A,C,G,T (AlignmentGraph.h:36-68).  Neighbour lists keep the
 * AlignmentGraph's order, which decides traceback ties. */
typedef struct ga_graph_desc {
    uint32_t num_nodes;
    uint32_t first_ambiguous;
    const uint32_t* node_length;      /* [num_nodes] 1..64 */
    const uint64_t* seq2bit;          /* [first_ambiguous * 2] */
    const uint64_t* seq_ambiguous;    /* [(num_nodes - first_ambiguous) * 4] A,C,G,T */
    const uint32_t* in_offsets;       /* [num_nodes + 1] */
    const uint32_t* in_neighbors;
    const uint32_t* out_offsets;      /* [num_nodes + 1] */
    const uint32_t* out_neighbors;
    const uint8_t*  linearizable;     /* [num_nodes] */
    const uint32_t* component;        /* [num_nodes] componentNumber (AlignmentGraph.cpp:987-1094) */
} ga_graph_desc;

/* Extension parameters, GraphAlignerCommon::Params (GraphAlignerCommon.h:83-109). */
typedef struct ga_extend_params {
    uint32_t bandwidth;               /* alignmentBandwidth */
    int32_t  xdrop;                   /* Xdropcutoff */
    uint64_t max_cells_per_slice;     /* maxCellsPerSlice (tangle effort); UINT64_MAX = unlimited */
    int32_t  xscore_error_cost;       /* XscoreErrorCost = int(100*(c/(1-c)+1)) */
} ga_extend_params;

/* A batch of extensions.  Extension i aligns seq[seq_offset[i] .. +seq_len[i]) starting
 * at split node start_node[i], offset start_offset[i] inside it — the node and offset
 * getInitialSliceExactPosition resolves from (bigraphNodeId, nodeOffset)
 * (GraphAlignerBitvectorCommon.h:1551-1587). */
typedef struct ga_extend_batch_desc {
    uint32_t num;
    const uint8_t*  seq;
    const uint64_t* seq_offset;
    const uint32_t* seq_len;
    const uint32_t* start_node;
    const uint32_t* start_offset;
    const uint64_t* trace_offset;     /* where extension i's trace items start in trace_items */
    const uint32_t* trace_capacity;   /* room for extension i's trace items */
} ga_extend_batch_desc;

/* Results.  A trace item packs one OnewayTrace TraceItem in DP order (end of the
 * alignment first, GraphAlignerBitvectorCommon.h:571-758):
 *   bits  0..31  split node index
 *   bits 32..37  nodeOffset inside the split node
 *   bit  38      nodeSwitch
 *   bits 39..63  seqPos + 1 (0 encodes seqPos == (size_t)-1, the row above the read) */
typedef struct ga_extend_results {
    int32_t*  status;                 /* [num] GA_OK / GA_TRACE_FAILED / GA_ASSERT / GA_CAPACITY /
                                         GA_BAD_REQUEST (start node or offset outside the graph) */
    int32_t*  score;                  /* [num] OnewayTrace::score */
    uint32_t* trace_len;              /* [num] items written */
    uint64_t* trace_items;            /* packed items, laid out by trace_offset */
    uint64_t* cell_steps;             /* [num] or NULL: Myers column steps in the fill (GCUPS numerator / 64) */
} ga_extend_results;

/* Longest extension sequence or read: seqPos + 1 must fit the item's 25 bits.  Longer
 * ones make ga_extend_batch*, ga_align_reads and ga_server_submit return GA_ERR_ARGUMENT. */
#define GA_MAX_SEQ_LEN        33554431u

#define GA_TRACE_NODE(x)      ((uint32_t)((x) & 0xffffffffu))
#define GA_TRACE_OFFSET(x)    ((uint32_t)(((x) >> 32) & 63u))
#define GA_TRACE_SWITCH(x)    ((uint32_t)(((x) >> 38) & 1u))
#define GA_TRACE_SEQPOS1(x)   ((uint64_t)((x) >> 39))

/* ---- device graph ---- */
typedef struct ga_graph* ga_graph_t;
/* Replaces the AlignmentGraph the DP reads (src/AlignmentGraph.h:121-139), as
 * AlignmentGraph::Finalize leaves it (src/AlignmentGraph.cpp:252-296): copied to
 * `device` once, read-only afterwards, shared by every extender made on it. */
int ga_graph_upload(const ga_graph_desc* desc, int device, ga_graph_t* out);
int ga_graph_free(ga_graph_t graph);

/* ---- batched extension ---- */
typedef struct ga_extender* ga_extender_t;
/* The device side of the per-thread AlignerGraphsizedState
 * (src/GraphAlignerCommon.h:52-81), for a whole batch: per-warp frontier tables and
 * the DP-table arena.  arena_bytes: device bytes for per-extension DP tables; 0 = 4 GiB. */
int ga_extender_create(ga_graph_t graph, uint64_t arena_bytes, ga_extender_t* out);
/* A second extender on the same device graph with the same arena size and launch shape
 * (no reference counterpart): two extenders let two batches run while the host works. */
int ga_extender_create_like(ga_extender_t ext, ga_extender_t* out);
int ga_extender_free(ga_extender_t ext);
/* A batch of GraphAlignerBitvectorBanded::getReverseTraceFromSeed calls
 * (src/GraphAlignerBitvectorBanded.h:59-76).  Host buffers in, host buffers out:
 * copies, launches and waits.  Status GA_TRACE_FAILED is OnewayTrace::TraceFailed(),
 * GA_ASSERT a reference assert (ThreadReadAssertion). */
int ga_extend_batch(ga_extender_t ext, const ga_extend_params* params,
                    const ga_extend_batch_desc* batch, ga_extend_results* results);
/* ---- multiseed DP ----
 * A batch of GraphAlignerBitvectorBanded::getMultiseedTraces calls (--multiseed-DP,
 * src/GraphAlignerBitvectorBanded.h:45-57): per read, the DP over every slice of the
 * read with its seeds started in their slices (getMultiseedSlices, :727-822), then a
 * trace from each local maximum of the per-node exact-end-position X-scores
 * (getLocalMaximaTracesFromTable, src/GraphAlignerBitvectorCommon.h:355-494).  The
 * traces come in the reference's order, each in DP order (end first), before
 * removeDuplicateTraces and the reversal, which stay with the caller. */
typedef struct ga_multiseed_batch_desc {
    uint32_t num;                     /* reads */
    const uint8_t*  seq;
    const uint64_t* seq_offset;
    const uint32_t* seq_len;
    const uint64_t* seed_offset;      /* [num + 1]: read i's seeds are [seed_offset[i], seed_offset[i+1]) */
    const uint32_t* seed_slice;       /* seqPos / 64 of each seed, non-decreasing within a read */
    const uint32_t* seed_node;        /* alignment-graph (split) node of each seed */
    const uint64_t* trace_offset;     /* [num] where read i's trace items start in trace_items */
    const uint64_t* trace_capacity;   /* [num] room for read i's items, all its traces together */
    uint32_t max_traces;              /* room per read in the trace tables */
    double   multimap_score_fraction; /* AlignerParams::multimapScoreFraction */
} ga_multiseed_batch_desc;

typedef struct ga_multiseed_results {
    int32_t*  status;                 /* [num] GA_OK / GA_ASSERT / GA_CAPACITY / GA_BAD_REQUEST */
    uint32_t* num_traces;             /* [num] */
    int32_t*  trace_score;            /* [num * max_traces] OnewayTrace::score */
    uint64_t* trace_start;            /* [num * max_traces] first item, counted from trace_offset[i] */
    uint32_t* trace_len;              /* [num * max_traces] items */
    uint64_t* trace_items;            /* packed items (GA_TRACE_* layout) */
    uint64_t* cell_steps;             /* [num] or NULL */
    uint64_t* items_needed;           /* [num] or NULL: for a read whose traces outgrew its room (GA_CAPACITY), */
    uint32_t* traces_needed;          /* [num] or NULL: the items and traces it needs; 0 for other statuses */
} ga_multiseed_results;

/* Host buffers in and out, like ga_extend_batch.  Seeds outside the graph or their read, or
 * out of slice order, are GA_ERR_ARGUMENT.  A read whose traces outgrow trace_capacity or
 * max_traces reports GA_CAPACITY with the room it needs in items_needed / traces_needed; run
 * it again with that room.  Of trace_items only the GA_OK reads' traces are defined after the
 * call; the rest of the span the batch's rooms cover may be overwritten. */
int ga_multiseed_batch(ga_extender_t ext, const ga_extend_params* params,
                       const ga_multiseed_batch_desc* batch, ga_multiseed_results* results);

/* The whole of GraphAlignerBitvectorBanded::getMultiseedTraces but the final reversal, with
 * no room limit: each read's traces after removeDuplicateTraces (:144-169, in its order),
 * each in DP order, land in buffers the extender owns, sized once they are counted, so no
 * read has to run twice and duplicates are neither written nor copied.  Read i's traces are
 * trace_first[i] .. trace_first[i] + num_traces[i] - 1 of the trace arrays; trace_start
 * indexes trace_items.
 * batch->trace_offset, trace_capacity and max_traces are not used (may be NULL / 0).  The
 * arrays stay valid until the extender's next call or ga_extender_free.  GA_CAPACITY now
 * means only that the read's frontier tables outgrew the largest layout. */
typedef struct ga_multiseed_output {
    const int32_t*  status;           /* [num] */
    const uint32_t* num_traces;       /* [num] */
    const uint64_t* trace_first;      /* [num] */
    const int32_t*  trace_score;      /* [total_traces] OnewayTrace::score */
    const uint64_t* trace_start;      /* [total_traces] */
    const uint32_t* trace_len;        /* [total_traces] */
    const uint64_t* trace_items;      /* [total_items] packed items (GA_TRACE_* layout) */
    const uint64_t* cell_steps;       /* [num] */
    uint64_t total_traces;
    uint64_t total_items;
} ga_multiseed_output;

int ga_multiseed_batch_exact(ga_extender_t ext, const ga_extend_params* params,
                             const ga_multiseed_batch_desc* batch, ga_multiseed_output* out);

/* Device-resident variant: every pointer in batch/results is a device pointer.
 * Work is enqueued on `stream` (a cudaStream_t; NULL = the extender's stream);
 * the call reads the lengths back once to order the work and waits for the
 * kernels, because extensions that outgrow the first pass's frontier tables
 * are re-run with larger tables before it returns. */
int ga_extend_batch_device(ga_extender_t ext, const ga_extend_params* params,
                           const ga_extend_batch_desc* batch, ga_extend_results* results,
                           void* stream);
/* No counterpart in the reference.  Extends a batch without allocating any
 * device memory, for callers that cannot call cudaMalloc while they extend
 * (device memory owned by another allocator under a fixed budget, or request
 * paths that cannot afford cudaMalloc's device-wide synchronisation).
 * device_graph, device_batch and device_results hold device pointers; a NULL
 * array in any of them is GA_ERR_ARGUMENT.  The frontier tables live in shared
 * memory; the other scratch (counters and the DP-table arena) is a 128 MiB
 * device array inside this library, kept by every GPU that loads it until the
 * process exits.  Limits per call: 4096 extensions and 8,000,000 read bp in
 * total; larger batches return GA_ERR_ARGUMENT.  Extensions whose band or
 * frontier outgrows the shared-memory tables report GA_CAPACITY (there is no
 * retry with larger tables); so do extensions that find the arena exhausted,
 * which depends on what else the batch holds (on variation graphs the tables
 * take about 5 bytes per read bp, far below the arena at the bp limit).  The
 * first call on a device looks up the array's device address and loads a
 * constant table (once per device, safe from several host threads).  Every
 * call reads the lengths back and waits for `stream` before it enqueues the
 * kernel there, so no call can be made inside a stream capture.  All calls
 * share the array: calls that overlap on the GPU (other streams, other host
 * threads) race. */
int ga_extend_batch_noalloc(const ga_graph_desc* device_graph, const ga_extend_params* params,
                            const ga_extend_batch_desc* device_batch, ga_extend_results* device_results,
                            void* stream);
/* Kernel time (fill and traceback) of the last ga_extend_batch* call in milliseconds
 * (CUDA events on the launching stream); valid after the stream has been synchronised. */
int ga_extender_last_kernel_ms(ga_extender_t ext, float* ms);
/* The same as a pair: fill_ms is the time of the fill and traceback kernels together
 * (they run back to back on one stream) and trace_ms is 0. */
int ga_extender_last_times(ga_extender_t ext, float* fill_ms, float* trace_ms);
/* Host-to-device and device-to-host copy times of the last ga_extend_batch call in
 * milliseconds (CUDA events; the trace items' copy spans the copy streams); 0 after
 * the device-resident entry points. */
int ga_extender_last_copy_ms(ga_extender_t ext, float* h2d_ms, float* d2h_ms);
/* Number of kernel launches made by the last ga_extend_batch* call. */
int ga_extender_last_launches(ga_extender_t ext, uint32_t* launches);

/* How the extension kernels are launched (no reference counterpart: it never changes a
 * result).  A fill kernel and then a traceback kernel run one extension per warp,
 * each warp taking the next of the batch's longest-first order.  warps_per_block
 * (1..4) warps share a block; blocks_per_sm caps the resident blocks per SM (0 = as
 * many as registers and shared memory allow).  first_layout picks the fill's frontier
 * tables in the first pass: 0 = small tables in shared memory (variation graphs),
 * 1 = medium tables in global memory, 2 = large tables in global memory (tangled de
 * Bruijn graphs); extensions that outgrow them (GA_CAPACITY) run again with the next
 * layout.  chunk_kib (1..2^20): the arena bytes a warp takes at once for the DP
 * tables of the extensions it fills. */
typedef struct ga_launch_shape {
    uint32_t warps_per_block;
    uint32_t blocks_per_sm;
    uint32_t first_layout;
    uint32_t chunk_kib;
} ga_launch_shape;
int ga_extender_set_launch_shape(ga_extender_t ext, const ga_launch_shape* shape);
int ga_extender_get_launch_shape(ga_extender_t ext, ga_launch_shape* shape);
/* Times `count` launch shapes on a host batch and makes the fastest the extender's
 * shape (no reference counterpart; the autotuner over warps per block, resident
 * blocks, first table layout and arena chunk).  The batch is copied to the device once; each
 * shape runs `repeats` times there (kernel time by CUDA events, the median kept) and
 * only statuses and scores come back: no trace is copied to the host.  Every shape
 * must reproduce the first one's statuses and scores, else GA_ERR_STATE and the first
 * shape is kept.  ms_out (NULL or [count]) receives each shape's median milliseconds. */
int ga_extender_autotune(ga_extender_t ext, const ga_extend_params* params,
                         const ga_extend_batch_desc* batch, const ga_launch_shape* shapes,
                         uint32_t count, uint32_t repeats, float* ms_out);
/* DP-table bytes the first pass of the last call wrote to the arena. */
int ga_extender_last_arena_bytes(ga_extender_t ext, uint64_t* bytes);
/* Extensions run with each table layout (0, 1, 2) by the last call (0 = layout not run). */
int ga_extender_last_layout_counts(ga_extender_t ext, uint32_t counts[3]);
/* The last multiseed call's local-maximum candidates, the walks that counted their traces
 * (candidates the traces kept before them ruled out are not walked), the traces it kept and
 * the rounds of walks, summed over its passes. */
int ga_extender_last_multiseed_counts(ga_extender_t ext, uint64_t* candidates, uint64_t* walks, uint64_t* traces, uint32_t* rounds);

/* ---- utilities (no reference counterpart) ---- */
/* Page-locked host memory for the host-buffer entry points. */
int ga_host_alloc(uint64_t bytes, void** out);
int ga_host_free(void* ptr);
/* Measured issue rate of independent 32-bit xor+add chains on `device`
 * (integer ops per second), the denominator of the DP kernels' ALU roofline. */
int ga_measure_int32_peak(int device, double* ops_per_second);

/* ---- read-level alignment ----
 * The per-read flow of GraphAligner's aligner (Aligner.cpp:440-592): minimizer
 * seeds (MinimizerSeeder::getSeeds, k-mer lookups on the GPU), OrderSeeds
 * (GraphAligner.h:250-312), the seed loop of GraphAligner::AlignOneWay
 * (GraphAligner.h:94-181; src/GraphAlignerWrapper.h:54) with both extensions of
 * each seed on the GPU, SelectAlignments (AlignmentSelection.cpp:31-53) and GAF
 * lines (GraphAlignerGAFAlignment.h:37-200).  Reads of a call advance through
 * their seed loops together; each round's extensions run as one GPU batch. */
typedef struct ga_host_graph_desc {
    ga_graph_desc base;               /* the DP fields, host pointers */
    const int32_t*  node_ids;         /* [num_nodes] bigraph node id of each piece (GFA id*2 + strand) */
    const uint32_t* node_offset;      /* [num_nodes] offset of the piece inside its bigraph node */
    const uint8_t*  reverse;          /* [num_nodes] */
    const uint64_t* chain_number;     /* [num_nodes] AlignmentGraph::chainNumber */
    const uint64_t* chain_approx_pos; /* [num_nodes] AlignmentGraph::chainApproxPos */
    uint32_t num_lookup;              /* bigraph nodes, in AlignmentGraph::nodeLookup order */
    const int32_t*  lookup_ids;
    const uint32_t* original_size;
    const uint32_t* lookup_offsets;   /* [num_lookup + 1] */
    const uint32_t* lookup_nodes;     /* pieces of each bigraph node, in offset order */
    const char* const* names;         /* [num_lookup] original names ("" = numeric GFA id), or NULL */
} ga_host_graph_desc;

/* AlignerParams fields of this flow (Aligner.h:10-47); -x vg: 15, 20, 10, 0.001, -1, 1, 1, 0, 0, 0.9 */
typedef struct ga_align_params {
    ga_extend_params extend;
    uint32_t minimizer_length;
    uint32_t minimizer_window;
    double   minimizer_density;
    double   minimizer_discard_fraction;
    double   seed_extend_density;
    uint64_t min_cluster_size;
    uint8_t  sloppy;                   /* not --try-all-seeds */
    uint8_t  cigar_match_mismatch;
    int32_t  min_alignment_score;
    double   multimap_score_fraction;
    uint8_t  multiseed_dp;             /* --multiseed-DP 1: one multiseed DP per read instead of the seed loop */
} ga_align_params;

typedef struct ga_align_stats {
    uint64_t reads;
    uint64_t reads_with_seeds;
    uint64_t reads_aligned;
    uint64_t failed_reads;            /* reads a reference assert would have dropped */
    uint64_t bp_aligned;              /* union of alignment intervals per read (Aligner.cpp:536-547) */
    uint64_t rounds;
    uint64_t extensions;
    uint64_t cell_steps;
    double   seed_ms;
    double   extend_ms;                /* ga_extend_batch calls: copies and kernels */
    double   host_ms;                  /* everything else */
    double   collect_ms;               /* of which: next seeds and extension requests */
    double   staging_ms;               /*           packing requests for the GPU */
    double   consume_ms;               /*           trace decoding, fix-up and merge per seed */
    double   finish_ms;                /*           selection and GAF per read */
    uint64_t speculative_used;         /* extensions of later seeds sent ahead and then used ... */
    uint64_t speculative_discarded;    /* ... and sent ahead but not used (the loop went elsewhere) */
    double   seed_lookup_ms;           /* of seed_ms: reads in, k-mer lookup kernel, matches back */
    double   seed_select_ms;           /*             least-frequent selection per read (host) */
    double   multiseed_kernel_ms;      /* of extend_ms with multiseed_dp: the multiseed DP's kernels and trace copies */
    uint64_t multiseed_candidates;     /* local maxima that could start a trace */
    uint64_t multiseed_walks;          /* of them: walked to count their traces */
    uint64_t multiseed_traces;         /* traces the multiseed DPs kept */
    uint64_t multiseed_rounds;         /* rounds of walks */
} ga_align_stats;

typedef struct ga_aligner* ga_aligner_t;
/* Builds the minimizer index of the graph (MinimizerSeeder's constructor with one bucket,
 * src/MinimizerSeeder.cpp:191-297) on the GPU and keeps its lookup table there.
 * GA_ERR_ARGUMENT for minimizer parameters out of range (length 1..31, at most 64
 * minimizer positions per window) or a graph whose split pieces do not tile their node. */
int ga_aligner_create(ga_extender_t ext, const ga_host_graph_desc* graph, const ga_align_params* params, ga_aligner_t* out);
typedef struct ga_index_info {
    uint64_t minimizer_length;
    uint64_t minimizer_window;
    uint64_t max_count;                /* MinimizerSeeder::maxCount: k-mers this frequent are not seeds */
    uint64_t num_keys;                 /* distinct k-mers */
    uint64_t num_positions;            /* minimizer occurrences in the graph */
    uint64_t table_capacity;           /* slots of the lookup table on the device */
    double   build_ms;                 /* the build in ga_aligner_create, copies included */
} ga_index_info;
/* The index built by ga_aligner_create: sizes in *info and, for each non-NULL array, the
 * distinct k-mers in increasing order (num_keys), each k-mer's first occurrence
 * (num_keys + 1, the last = num_positions) and the occurrences, (split node << 6) | offset
 * grouped by k-mer (num_positions). */
int ga_aligner_index(ga_aligner_t aligner, ga_index_info* info, uint64_t* keys, uint64_t* start_pos, uint64_t* positions);
int ga_aligner_free(ga_aligner_t aligner);
/* Aligns a batch of reads (host buffers); the GAF text stays with the aligner. */
int ga_align_reads(ga_aligner_t aligner, uint32_t num_reads, const char* const* names, const uint8_t* seq,
                   const uint64_t* seq_offset, const uint32_t* seq_len);
/* One seed of MinimizerSeeder::getSeeds (SeedHit, src/GraphAlignerWrapper.h:11-50). */
typedef struct ga_seed {
    int32_t  node_id;                 /* SeedHit::nodeID: the GFA node id */
    uint32_t reverse;                 /* SeedHit::reverse */
    uint64_t node_offset;             /* SeedHit::nodeOffset */
    uint64_t seq_pos;                 /* SeedHit::seqPos */
    uint32_t match_len;               /* SeedHit::matchLen (the minimizer length) */
    uint32_t raw_seed_goodness;       /* SeedHit::rawSeedGoodness */
    uint32_t alignment_graph_node;    /* SeedHit::alignmentGraphNodeId (split node index) */
    uint32_t alignment_graph_offset;  /* SeedHit::alignmentGraphNodeOffset */
} ga_seed;
/* MinimizerSeeder::getSeeds(sequence, density) (src/MinimizerSeeder.cpp:521-543) for a batch of
 * reads (host buffers): the k-mer lookups on the GPU, the least-frequent selection on the host.
 * Read i's seeds, in the reference's order (before OrderSeeds), are seeds[seed_offsets[i] ..
 * seed_offsets[i + 1]); both arrays stay valid until the next call on this aligner. */
int ga_aligner_get_seeds(ga_aligner_t aligner, uint32_t num_reads, const uint8_t* seq, const uint64_t* seq_offset,
                         const uint32_t* seq_len, const ga_seed** seeds, const uint64_t** seed_offsets);
/* ---- GAF lines and alignment selection on the device ----
 * What ga_align_reads does after the seed loop, for callers that keep their own: the
 * selection of one read's alignments (AlignmentSelection::SelectAlignments,
 * src/AlignmentSelection.cpp:31-95, without the E-value filter) and the GAF line of an
 * alignment (GraphAlignerGAFAlignment::traceToAlignment, src/GraphAlignerGAFAlignment.h:37-200).
 * One trace item after the fix-ups (fixForwardTraceSeqPos / fixReverseTraceSeqPosAndOrder):
 * bigraph node id, offset in it, read position, nodeSwitch and the two characters. */
typedef struct ga_gaf_item {
    int32_t  node;
    uint32_t node_offset;
    uint32_t seq_pos;
    uint8_t  node_switch;
    uint8_t  seq_char;
    uint8_t  graph_char;
    uint8_t  pad;
} ga_gaf_item;
typedef struct ga_gaf_line {
    uint64_t first_item;               /* the trace is items[first_item .. +item_count) */
    uint32_t item_count;
    uint32_t read;                     /* index into read_names / read_lens */
    int32_t  xscore100;                /* alignmentXScore * 100; -100 leaves AS:f out, as the reference does for -1 */
    int32_t  mapq;                     /* mappingQuality */
} ga_gaf_line;
/* The lines, each with its newline, into one text kept by the aligner until the next call;
 * line_ends[k] = where line k's newline ends; failed[k] = 1 where the reference would have
 * asserted (the line is then a lone newline). */
int ga_aligner_format_gaf(ga_aligner_t aligner, uint32_t num_lines, const ga_gaf_line* lines, uint64_t num_items,
                          const ga_gaf_item* items, uint32_t num_reads, const char* const* read_names, const uint32_t* read_lens,
                          uint8_t cigar_match_mismatch, const char** text, uint64_t* bytes, const uint64_t** line_ends,
                          const uint8_t** failed);
/* Read r's alignments are [first[r], first[r+1]) of starts, ends (alignmentStart / End),
 * xscores (alignmentXScore) and keep; keep[k] = 1 for the alignments SelectAlignments keeps. */
int ga_aligner_select_alignments(ga_aligner_t aligner, uint32_t num_reads, const uint64_t* first, const uint64_t* starts,
                                 const uint64_t* ends, const double* xscores, int32_t min_alignment_score,
                                 double multimap_score_fraction, uint8_t* keep);
/* GAF lines of the last ga_align_reads call, reads in input order; valid until the next call. */
int ga_aligner_gaf(ga_aligner_t aligner, const char** text, uint64_t* bytes);
/* Per-read bp aligned of the last call. */
int ga_aligner_read_bp(ga_aligner_t aligner, uint64_t* bp_per_read);
int ga_aligner_stats(ga_aligner_t aligner, ga_align_stats* out);

/* ---- serving loop ----
 * The request side of Aligner.cpp's worker loop (Aligner.cpp:440-592, one read per
 * loop iteration there) as continuous batching: reads are submitted one at a time
 * from any thread; a worker thread admits them while the reads in flight and their
 * estimated band memory stay under the limits, seeds each admitted group on the GPU,
 * and runs rounds of extensions on concurrent lanes (long reads on their own lane), so
 * reads that arrive while others are on the GPU join their lane's next round and share
 * its launch.  A read's GAF bytes do not depend on which other reads share its rounds.
 * The graph, the DP arrays and the minimizer table stay resident on the device. */
typedef struct ga_server_params {
    uint32_t max_reads_in_flight;     /* reads in their seed loops at once; 0 = 4096 */
    uint64_t max_band_bytes;          /* admission budget of estimated band + trace memory; 0 = 2 GiB */
    uint32_t band_bytes_per_bp;       /* the estimate per read bp; 0 = 32 */
    uint32_t lanes;                   /* concurrent rounds, each with its own extender; 0 = 2, at most 8;
                                         one lane if the device has no room for another extender */
    uint32_t long_read_bp;            /* with 2+ lanes, reads this long are served on lane 0 only; 0 = 15000 */
} ga_server_params;

typedef struct ga_server_result {
    uint64_t ticket;
    int32_t  status;                  /* GA_OK, GA_ASSERT (dropped as Aligner.cpp:493-500 does), or an error */
    uint32_t alignments;              /* GAF lines */
    uint64_t bp_aligned;
    const char* gaf;                  /* valid until ga_server_release(ticket) */
    uint64_t gaf_bytes;
    double   queue_ms;                /* submit -> admitted */
    double   latency_ms;              /* submit -> GAF ready */
} ga_server_result;

typedef struct ga_server_stats {
    uint64_t submitted;
    uint64_t completed;
    uint64_t rounds;                  /* extension batches launched */
    uint64_t extensions;
    uint64_t admissions;              /* admitted groups (one seeding launch each) */
    uint64_t max_in_flight;
    uint64_t mixed_rounds;            /* rounds whose reads were admitted in different groups */
    double   busy_ms;                 /* worker time spent seeding, extending and finishing */
} ga_server_stats;

typedef struct ga_server* ga_server_t;
/* Starts the worker thread.  The aligner must outlive the server and must not be
 * used by other calls meanwhile. */
/* GA_ERR_ARGUMENT for an aligner made with multiseed_dp: the loop runs the seed loop. */
int ga_server_create(ga_aligner_t aligner, const ga_server_params* params, ga_server_t* out);
/* Copies the read and queues it; returns at once with a ticket (from 1 up). */
int ga_server_submit(ga_server_t server, const char* name, const uint8_t* seq, uint32_t len, uint64_t* ticket);
/* Up to max finished reads, waiting up to wait_ms (0: no wait, -1: until one is ready). */
int ga_server_poll(ga_server_t server, ga_server_result* out, uint32_t max, uint32_t* count, int32_t wait_ms);
/* Frees the GAF text of a polled result. */
int ga_server_release(ga_server_t server, uint64_t ticket);
int ga_server_stats_get(ga_server_t server, ga_server_stats* out);
/* Finishes every submitted read, stops the worker and frees the server. */
int ga_server_free(ga_server_t server);

const char* ga_last_error(void);
const char* ga_version(void);

#ifdef __cplusplus
}
#endif

#endif
