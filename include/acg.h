/*
 * acg.h -- C ABI of the GB300 ApplicationClassification matcher.
 *
 * The reference (porumbes/application_classification) has no library API: its
 * hot path is the set of `ac::` functions in src/ac.hxx:17-186 plus the inline
 * Thrust lambdas that src/main.cu:107-247 calls between them.  This header
 * replaces that whole path -- cdist, the row log-softmax normalisers, the
 * edge->vertex max messages, the VR/VF/mu updates and the final transpose --
 * with whole-pipeline entry points, because the GB300 kernels fuse across the
 * reference's per-op boundaries.
 *
 * Conventions
 *   - Graph arrays passed to acg_data_create / acg_plan_create are DEVICE
 *     pointers owned by the caller, exactly what `loadGraph` produces
 *     (main.cu:54-62).  They must stay valid until the object built from them
 *     is destroyed.
 *   - `stream` is a cudaStream_t passed as void* (NULL = legacy default
 *     stream).  All device work of a call is enqueued on it.  Calls return once
 *     the work is enqueued, except where stated.
 *   - Every entry point returns an acg_status; 0 means success.  A failing
 *     call leaves a message for acg_last_error() (thread-local).
 *   - One host thread per plan at a time.
 */
#ifndef ACG_H
#define ACG_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef enum acg_status {
  ACG_OK = 0,
  ACG_ERR_INVALID_ARGUMENT = 1, /* null pointer, zero-sized pattern, bad option */
  ACG_ERR_OUT_OF_MEMORY = 2,    /* a device or host allocation failed */
  ACG_ERR_INDEX_OUT_OF_RANGE = 3, /* an edge endpoint >= num_nodes */
  ACG_ERR_CUDA = 4,             /* a CUDA runtime call failed */
  ACG_ERR_UNSUPPORTED = 5,      /* size or feature outside what is built */
  ACG_ERR_IO = 6,               /* file missing, truncated or malformed */
  ACG_ERR_DEVICE_TIMEOUT = 7    /* a bounded device-side wait gave up */
} acg_status;

/* Mirrors `struct Graph` (src/main.cu:8-19): u64 sizes, f64 row-major
 * features, u64 edge endpoints.  Multi-edges and self-loops are allowed. */
typedef struct acg_graph {
  uint64_t num_nodes;
  uint64_t node_feat_dim;
  uint64_t num_edges;
  uint64_t edge_feat_dim;
  const double* node_feats;  /* [num_nodes][node_feat_dim] */
  const double* edge_feats;  /* [num_edges][edge_feat_dim] */
  const uint64_t* srcs;      /* [num_edges] */
  const uint64_t* dsts;      /* [num_edges] */
} acg_graph;

/* Arithmetic used by a plan.
 *  ACG_PREC_FP64  : every value and every operation in FP64, as the reference
 *                   (helpers.hxx:3-4 `Real = double`).
 *  ACG_PREC_MIXED : cost matrices in FP32 (difference form, from FP32 copies
 *                   of the features), belief propagation in FP32 with the
 *                   values stored relative to per-column shifts, column
 *                   log-sum-exp normalisers accumulated in FP64. */
typedef enum acg_precision {
  ACG_PREC_FP64 = 0,
  ACG_PREC_MIXED = 1
} acg_precision;

typedef struct acg_options {
  int32_t precision;  /* acg_precision */
  int32_t num_iters;  /* BP iterations; < 0 means pattern num_nodes, which is
                         what the reference runs (main.cu:160) */
  int32_t kernel_timing; /* nonzero: bracket each iteration's edge and vertex
                            phases with CUDA events (acg_stats.ms_*_phase) */
  int32_t edge_blocks_per_sm;   /* resident 256-thread blocks per SM of the edge
                                   phase and the static passes (0: as many as fit) */
  int32_t vertex_blocks_per_sm; /* the same for the vertex phase (0: as many as fit) */
  int32_t cnull;      /* 1: the C-null term of the PNNL formulation, which the
                         reference leaves out (main.cu:83; test.py:93-97):
                         cnull = log-softmax over pattern edges q of
                         max(||pe_q||, max_e L(dE)[q][e]), subtracted from both
                         max-message fills of column q in every iteration.
                         0 (default): the reference's behaviour.  In a batch
                         the normaliser runs over each pattern's own edges;
                         acg_backward carries the term's gradient to the
                         pattern edge features. */
  int32_t cdist_kernel; /* the edge and vertex cost matrices of the
                           mixed-precision path: 0 (default) each on the
                           tensor cores (tcgen05, TF32 split, see
                           acg_cdist_tc.cu) when its shape allows it
                           (feature dim <= 32, <= 128 padded pattern edges /
                           vertices), else on the CUDA cores; 1 always CUDA
                           cores; 2 both on the tensor cores or
                           ACG_ERR_UNSUPPORTED.  FP64 plans always use CUDA
                           cores. */
  int32_t autotune;   /* acg_batch_create only: 1 = measure before grouping
                         (see acg_batch_create); 0 (default) = greedy packing
                         with the default launch shapes */
  int32_t edge_kernel; /* the edge phase of the mixed-precision iterations:
                          0 (default) and 1 read the stored edge cost matrix;
                          2 recompute each in-edge's costs on the tensor cores
                          inside the phase (acg_edge_tc.cu: the arithmetic of
                          the stored matrix, so the same values, without
                          reading it) or ACG_ERR_UNSUPPORTED when the shape
                          does not allow it (plans with the tensor-core edge
                          cost matrix, edge feature dim <= 24, <= 64 padded
                          pattern edges).  FP64 plans, batches and recorded
                          matches (acg_match_record) read the stored matrix. */
} acg_options;

/* Fill `opt` with the defaults (FP64, num_iters = -1). */
void acg_options_default(acg_options* opt);

/* Opaque handles. */
typedef struct acg_data acg_data; /* a data graph prepared for matching */
typedef struct acg_plan acg_plan; /* one pattern against one acg_data */

/* Timings and traffic of the last acg_match on a plan (filled by
 * acg_plan_stats, which synchronises the plan's stream). */
typedef struct acg_stats {
  double ms_total;        /* cdist + init + iterations + output */
  double ms_cdist;
  double ms_init;
  double ms_iters;
  double bytes_iters;     /* algorithmic bytes of all iterations */
  double bytes_edge_phase;   /* algorithmic bytes of one edge phase: dE rows and
                                source indices of every in-edge, each source row
                                and each output row once */
  double bytes_vertex_phase; /* algorithmic bytes of one vertex phase */
  double ms_edge_phase;   /* edge phases summed over the iterations (only with
                             acg_options.kernel_timing, else 0) */
  double ms_vertex_phase; /* vertex phases (kernel + statistics), summed */
  int64_t launches;       /* kernels launched by the last acg_match */
  int64_t num_iters;
  /* The edge phase's work split: launched warps, item ranges (the first
     edge_warps are the warps' own, the rest are claimed at run time) and
     vertices split into chunks that reduce through partial rows. */
  int64_t edge_warps;
  int64_t edge_ranges;
  int64_t edge_heavy_vertices;
} acg_stats;

/* ---------------- data graph ------------------------------------------- */
/* Validate the data graph (every endpoint < num_nodes, else
 * ACG_ERR_INDEX_OUT_OF_RANGE), build its two CSR orderings (edges sorted
 * stably by destination and by source, int32 positions) and keep them for
 * every plan made from it.  Replaces nothing in the reference, which scatters
 * with atomics instead (ac.hxx:115-149, helpers.hxx:36-55).
 * Synchronises `stream` (it reads back the validation result). */
acg_status acg_data_create(const acg_graph* data, void* stream, acg_data** out);
acg_status acg_data_destroy(acg_data* data);

/* ---------------- plan / match ----------------------------------------- */
/* Make a plan for matching `pattern` against `data`.  Allocates every device
 * workspace the match needs (the reference allocates its 13 buffers in
 * main.cu:80-99).  Pattern endpoints must be < pattern num_nodes.
 * Synchronises `stream`. */
acg_status acg_plan_create(acg_data* data, const acg_graph* pattern,
                           const acg_options* opt, void* stream,
                           acg_plan** out);
acg_status acg_plan_destroy(acg_plan* plan);

/* Run the whole match: cdist of vertex and edge features, the initial
 * normalisers and edge maxima, `num_iters` BP iterations and the output in
 * [data num_nodes][pattern num_nodes] row-major order -- the `MU` matrix the
 * reference prints (main.cu:107-247).  `mu_out` is caller-owned device
 * memory of num_nodes * pattern_nodes doubles. */
acg_status acg_match(acg_plan* plan, double* mu_out, void* stream);

/* Statistics of the last acg_match (synchronises the plan's stream). */
acg_status acg_plan_stats(acg_plan* plan, acg_stats* out);

/* One-shot convenience: data create + plan create + match + destroy.  The
 * drop-in for the body of the reference's main() between loadGraph and the
 * result copy (main.cu:77-247).  Synchronises `stream`. */
acg_status acg_match_graphs(const acg_graph* data, const acg_graph* pattern,
                            const acg_options* opt, double* mu_out,
                            void* stream);

/* One-shot from HOST buffers: the reference program's flow between reading
 * the graph files and printing MU -- loadGraph's copies (main.cu:54-62), the
 * match (main.cu:77-247) and the copy of MU back (main.cu:253) -- with the
 * graphs' arrays in host memory and mu_out_host [data num_nodes][pattern
 * num_nodes] in host memory.  The edge endpoints are copied first and the data
 * graph's CSR orderings are built while the features are still being copied
 * (on a second stream); pinned host buffers let the copies run asynchronously.
 * With ACG_PREC_MIXED the edge features go up in pieces, and each piece is
 * turned into its FP32 rows and (tensor-core plans) its rows of the edge cost
 * matrix as it lands (a third stream), so the match starts with the costs
 * written; mu is bit-identical to acg_match's.  Device memory comes from the
 * library's pool.  Synchronises `stream`. */
acg_status acg_match_graphs_host(const acg_graph* data, const acg_graph* pattern,
                                 const acg_options* opt, double* mu_out_host, void* stream);

/* ---------------- many patterns against one data graph ----------------- */
/* No counterpart in the reference, which matches one pattern per run
 * (main.cu:72-75).  The data graph is prepared once; the patterns are packed
 * into groups matched as disjoint unions (each member's mu equals its own
 * acg_match result up to summation order), groups share one set of
 * workspaces, and the whole batch is one CUDA graph launched per
 * acg_batch_match.  Patterns: device arrays as for acg_plan_create (at most
 * 128 vertices / 256 edges each); opt as for acg_plan_create (num_iters < 0:
 * each pattern's own vertex count). */
typedef struct acg_batch acg_batch;
typedef struct acg_batch_info {
  int32_t patterns;
  int32_t groups;               /* unions matched */
  int32_t widest_group_columns; /* pattern edges of the widest group */
  int32_t autotuned;            /* 1 if the grouping and launch shape were measured */
  int64_t graph_nodes;          /* nodes of the captured CUDA graph */
  double ms_last;               /* device time of the last acg_batch_match */
  /* autotune: the fitted cost model of a group with c columns running i
     iterations, ms = i * (iter_ms_per_column * c + iter_ms_fixed)
     + once_ms_per_column * c + once_ms_fixed, and the launch shape chosen */
  double iter_ms_per_column, iter_ms_fixed, once_ms_per_column, once_ms_fixed;
  double predicted_ms;          /* the model's total for the chosen grouping */
  int32_t edge_blocks_per_sm, vertex_blocks_per_sm;
} acg_batch_info;
/* With opt->autotune = 1, acg_batch_create first measures the data graph:
 * short probe matches (three BP iterations) of real pattern unions of about
 * 16, 32 and 64 columns give a linear cost model per iteration and per group,
 * a few block-per-SM launch shapes are timed on the widest probe, and the
 * grouping is then chosen by dynamic programming over the patterns sorted by
 * iteration count to minimise the model's total (a group iterates as long as
 * its longest member).  Costs a few probe matches at creation. */
acg_status acg_batch_create(acg_data* data, const acg_graph* patterns,
                            int32_t npatterns, const acg_options* opt,
                            void* stream, acg_batch** out);
/* mu_out[i]: device [Dn][patterns[i].num_nodes] f64.  The first call (and any
 * call with other outputs or another stream) captures the CUDA graph; later
 * calls only launch it.  Asynchronous on `stream`. */
acg_status acg_batch_match(acg_batch* b, double* const* mu_out, void* stream);
/* Synchronises on the last match. */
acg_status acg_batch_get_info(acg_batch* b, acg_batch_info* out);
acg_status acg_batch_destroy(acg_batch* b);

/* ---------------- no-allocation entry point ---------------------------- */
/* The match's initial mu, before any BP iteration:
 *   mu_out[v][p] = -d(v,p) - log sum_v' exp(-d(v',p)),  d = || x_v - y_p ||_2,
 * i.e. the [num_nodes][pattern_nodes] output acg_match gives with
 * num_iters = 0, computed without allocating any memory.  No counterpart in
 * the reference: it exists for callers that cannot allocate device memory at
 * the point of the call (inside stream capture, under a fixed memory budget,
 * or embedded behind another framework's allocator).  Its scratch is one
 * file-scope device array of about 1.5 MB that every GPU loading the library
 * keeps until exit.  Limits: 1..128 pattern vertices, feature dimension
 * 1..32 (else ACG_ERR_UNSUPPORTED).  The first call on each device looks the
 * array's address up (make it before any stream capture); so does the first
 * call after cudaDeviceReset, which gives the device a new context.  All
 * calls share the array: calls whose work overlaps on the GPU race and must
 * be serialised.  A CUDA error already pending on the calling thread is
 * returned (ACG_ERR_CUDA, named as earlier) before anything is launched.
 * Inputs and output are caller-owned device memory (FP64, row-major). */
acg_status acg_initial_mu_noalloc(const double* data_node_feats, uint64_t num_nodes,
                                  uint64_t feat_dim, const double* pattern_node_feats,
                                  uint64_t pattern_nodes, double* mu_out, void* stream);

/* ---------------- gradients (adjoint of a match) ----------------------- */
/* No counterpart in the reference, which runs the matcher forward only.
 * acg_match_record is acg_match (same output) that also keeps the state of
 * every `checkpoint_every`-th BP iteration (<= 0: 4) and of the last;
 * acg_backward then returns the gradients of sum(grad_mu * mu) with respect
 * to the four feature arrays (FP64 device outputs: data [num_nodes][node
 * feat dim], [num_edges][edge feat dim] in the data graph's own edge order,
 * pattern [Pn][node feat dim], [Pe][edge feat dim]), recomputing the
 * iterations between checkpoints.  Maxima pass their gradient to the first
 * maximal element (smallest data vertex; smallest edge id within a vertex's
 * edges); log-sum-exps through their softmax.  Deterministic: every sum has
 * a fixed order (the one atomic is an integer OR).
 * Limits: single plans of at most 64 pattern vertices and 64 pattern edges
 * (padded), feature dimensions <= 32 (else ACG_ERR_UNSUPPORTED).  The
 * checkpoints stay with the plan until it is destroyed or re-recorded.
 * Asynchronous on `stream`. */
acg_status acg_match_record(acg_plan* plan, double* mu_out, int32_t checkpoint_every,
                            void* stream);
acg_status acg_backward(acg_plan* plan, const double* grad_mu, double* grad_data_node_feats,
                        double* grad_data_edge_feats, double* grad_pattern_node_feats,
                        double* grad_pattern_edge_feats, void* stream);

/* ---------------- memory ----------------------------------------------- */
/* Device memory of data graphs, plans, batches and the adjoint comes from a
 * per-device stream-ordered pool that keeps freed blocks cached for the next
 * object (as a caching allocator does), so the process holds its high-water
 * mark until exit.  This returns the cached free blocks to the driver (memory
 * still in use by live objects is not touched).  No counterpart in the
 * reference.  ACG_MEMPOOL=0 in the environment (read once, at the first
 * allocation) selects plain cudaMalloc / cudaFree instead; results are the
 * same bytes either way. */
acg_status acg_release_cached_memory(void);

/* Testing aids for out-of-memory handling (no counterpart in the reference,
 * whose cudaMalloc calls go unchecked, main.cu:85-99).
 * acg_inject_alloc_failure(n): the n-th device allocation the library makes
 * from now on (counted over every thread) fails as if the device were out of
 * memory, and the call that made it returns ACG_ERR_OUT_OF_MEMORY; n <= 0
 * cancels a pending injection.
 * acg_device_memory_in_use: synchronises the device, then reports the bytes
 * in use in the library's memory pool and in the device's default pool (the
 * scratch of the CSR build); a failed call must leave it where it was. */
acg_status acg_inject_alloc_failure(int64_t nth);
acg_status acg_device_memory_in_use(int64_t* bytes);

/* ---------------- errors ----------------------------------------------- */
const char* acg_status_string(acg_status s);
/* Message of the last failing call on this host thread ("" if none). */
const char* acg_last_error(void);

/* Library version string, e.g. "acg 0.1.0 sm_103a". */
const char* acg_version(void);

#ifdef __cplusplus
}
#endif
#endif /* ACG_H */
