/*
 * kamsta_gpu.h -- C ABI of the GB300 minimum-spanning-forest solver.
 *
 * This is the drop-in boundary for KaMSTa's single-node MST hot path
 * (Boruvka rounds and filter-Boruvka).  Every entry point takes plain
 * pointers and sizes; no CUDA or C++ type appears in a signature, so the
 * header binds from C, C++ (see kamsta_gpu.hpp), ctypes, cgo or JNI alike.
 *
 * Reference interfaces replaced (paths relative to the KaMSTa tree):
 *   hybridMST::boruvka(std::vector<WEdge>, const AlgorithmConfig&)
 *       include/algorithms/hybrid_boruvka.hpp:263-301
 *   hybridMST::filter_boruvka(std::vector<WEdge>, const AlgorithmConfig&)
 *       include/algorithms/hybrid_boruvka_edgefilter.hpp:420-462
 *   hybridMST::AlgorithmConfig / LocalPreprocessing / Compression
 *       include/algorithms/algorithm_configurations.hpp:6-34
 *   hybridMST::WEdge (24-byte input edge)      include/definitions.hpp:66-84
 *   hybridMST::WEdge_4_4 (12-byte packed edge) include/edge_types.hpp:135-146
 *
 * Input contract (same as the reference, utils.hpp:388-403 and
 * benchmarks/mst.cpp:166-167): directed edge entries sorted by (src, dst),
 * both directions of every undirected edge present, no self loops, ids < n.
 * The solver reads each undirected edge from its src < dst copy, exactly like
 * the reference's local path (local_contraction/utils.hpp:38-56).
 *
 * Output: the minimum spanning forest under the total order
 * (w, min(u,v), max(u,v)) -- the order of the reference's own checker
 * (base_case_mst_algos.hpp:91-112) -- one entry per forest edge, written as
 * (min, max, w).  The order of the entries is deterministic; pass
 * KAMSTA_FLAG_SORT_OUTPUT to get them sorted by (src, dst).
 *
 * Errors: every call returns a kamsta_status; kamsta_last_error() gives a
 * thread-local message for the last failing call on the calling thread.
 * The reference aborts the process instead (include/mpi/context.hpp:77-97).
 */
#ifndef KAMSTA_GPU_H
#define KAMSTA_GPU_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes ------------------------------------------------------ */
typedef int kamsta_status;
#define KAMSTA_OK 0
#define KAMSTA_E_INPUT 1       /* malformed input (ids >= n, unsorted, sizes) */
#define KAMSTA_E_OOM 2         /* device or host allocation failed            */
#define KAMSTA_E_CUDA 3        /* a CUDA runtime call failed                  */
#define KAMSTA_E_NOCONVERGE 4  /* an iteration cap was hit (no hang, no trap) */
#define KAMSTA_E_UNSUPPORTED 5 /* option not implemented on this build        */
#define KAMSTA_E_BUDGET 6      /* request larger than the serving budget      */
#define KAMSTA_E_NOTREADY 7    /* serving: result not finished yet            */
#define KAMSTA_E_CANCELLED 8   /* serving: job withdrawn before it ran        */

/* ---- edge layouts -------------------------------------------------------- */
/* Packed 12-byte weighted edge; same field order and width as WEdge_4_4
 * (edge_types.hpp:135-146). */
typedef struct kamsta_wedge {
  uint32_t src;
  uint32_t dst;
  uint32_t w;
} kamsta_wedge;

/* The reference's std::vector<WEdge> element (definitions.hpp:66-84):
 * 64-bit ids, 32-bit weight, 4 bytes tail padding (24 bytes). */
typedef struct kamsta_wedge64 {
  uint64_t src;
  uint64_t dst;
  uint32_t w;
  uint32_t pad_;
} kamsta_wedge64;

/* ---- configuration ------------------------------------------------------- */
/* LocalPreprocessing (algorithm_configurations.hpp:6-16). */
#define KAMSTA_NO_PREPROCESSING 0
#define KAMSTA_MODIFIED_BORUVKA 1
#define KAMSTA_REDUCE_EDGES_THEN_BORUVKA 2
/* Compression (algorithm_configurations.hpp:18-25). */
#define KAMSTA_NO_COMPRESSION 0
#define KAMSTA_SEVEN_BIT_DIFF_ENCODING 1

/* flags */
#define KAMSTA_FLAG_VALIDATE 0x1u     /* check sortedness / id range on device */
#define KAMSTA_FLAG_SORT_OUTPUT 0x2u  /* sort forest edges by (src, dst)      */
#define KAMSTA_FLAG_DEDUPE_NEVER 0x4u /* never remove parallel edges          */
#define KAMSTA_FLAG_DEDUPE_ALWAYS 0x8u/* remove parallel edges every round   */
#define KAMSTA_FLAG_TRACE 0x10u       /* record per-round (m_r, n_r) in stats  */
#define KAMSTA_FLAG_FILTER 0x20u      /* batch / serving: run filter_boruvka   */

/* AlgorithmConfig (algorithm_configurations.hpp:27-34) plus GPU knobs.
 * compression = KAMSTA_SEVEN_BIT_DIFF_ENCODING: the host-buffer entry points
 * (kamsta_mst_boruvka, kamsta_mst_filter_boruvka, kamsta_mst_boruvka_wedge64)
 * encode the input on the host as the reference's boruvka() does
 * (hybrid_boruvka.hpp:277-299), copy only the compressed bytes to the device
 * and decode them there; the forest is the same as uncompressed.  Device-
 * buffer and batch entry points already hold 12-byte entries on the device
 * and solve them as they are. */
typedef struct kamsta_cfg {
  int32_t local_preprocessing; /* KAMSTA_*_PREPROCESSING / _BORUVKA         */
  int32_t compression;         /* KAMSTA_*_COMPRESSION                       */
  uint64_t filter_threshold;   /* filter_boruvka base-case average degree    */
  uint32_t flags;              /* KAMSTA_FLAG_*                              */
  uint32_t dedupe_ratio;       /* auto dedupe when m_r > ratio * n_r (0=off) */
  uint64_t seed;               /* pivot-sampling seed                        */
  uint32_t seg_items_per_thread; /* list-pass tile: 2, 4 or 8 records per   */
                               /* thread (0 = 2)                             */
  uint32_t items_per_thread;   /* first-pass tile: 6, 8 or 12 directed       */
                               /* entries per thread (0 = 6)                 */
} kamsta_cfg;

#define KAMSTA_TRACE_MAX 128
/* Phases timed in kamsta_stats (device time from CUDA events). */
#define KAMSTA_PHASE_PLAN 0         /* weight sampling for the pivots        */
#define KAMSTA_PHASE_FIRST_PASS 1   /* one streaming pass over the input     */
#define KAMSTA_PHASE_ROUND_EDGES 2  /* relabel + compact + next minimum      */
#define KAMSTA_PHASE_ROUND_VERTS 3  /* hook, jump, renumber, map             */
#define KAMSTA_PHASE_CLASS_PASS 4   /* relabel/filter of heavier classes     */
#define KAMSTA_PHASE_FINALIZE 5     /* component labels after a Boruvka call */
#define KAMSTA_PHASE_EMIT 6         /* forest output                         */
#define KAMSTA_PHASE_DEDUPE 7       /* parallel-edge removal (radix sort)    */
#define KAMSTA_PHASES 8
typedef struct kamsta_stats {
  uint64_t num_mst_edges;  /* forest edges written                         */
  uint64_t total_weight;   /* sum of forest edge weights                   */
  uint32_t rounds;         /* Boruvka rounds over all levels               */
  uint32_t levels;         /* filter recursion levels / weight classes     */
  uint32_t dedupe_passes;  /* radix-sort dedupe passes run                 */
  uint32_t gpu_launches;   /* kernels launched by the call                 */
  double device_ms;        /* device time of the solve (CUDA events)       */
  uint64_t alg_bytes;      /* algorithmic HBM bytes of the solve            */
  uint32_t trace_len;      /* entries in trace_m / trace_n                  */
  uint32_t row_scans;      /* heavy-class contractions done by row scans    */
  uint64_t trace_m[KAMSTA_TRACE_MAX]; /* live undirected edges per round   */
  uint64_t trace_n[KAMSTA_TRACE_MAX]; /* live vertices per round           */
  double phase_ms[KAMSTA_PHASES];     /* device time per phase             */
  uint64_t phase_bytes[KAMSTA_PHASES];/* algorithmic bytes per phase       */
  uint32_t phase_launches[KAMSTA_PHASES];
} kamsta_stats;

/* Fills cfg with AlgorithmConfig's defaults: NO_PREPROCESSING,
 * NO_COMPRESSION, filter_threshold 4 (algorithm_configurations.hpp:31-33). */
kamsta_status kamsta_cfg_default(kamsta_cfg* cfg);

const char* kamsta_version(void);
const char* kamsta_last_error(void);

/* ---- context: device scratch pool + stream ----------------------------- */
typedef struct kamsta_ctx kamsta_ctx;
typedef void* kamsta_stream; /* a cudaStream_t; NULL = the context's stream */

kamsta_status kamsta_ctx_create(int device, kamsta_ctx** out);
kamsta_status kamsta_ctx_destroy(kamsta_ctx* ctx);
/* Releases cached scratch memory of the context. */
kamsta_status kamsta_ctx_trim(kamsta_ctx* ctx);
/* Device bytes currently held by the context's scratch pool. */
uint64_t kamsta_ctx_pool_bytes(const kamsta_ctx* ctx);
/* Caps the device bytes the context may have in use (live allocations of
 * its scratch pool plus its arenas); 0 = no cap (the default).  A call that
 * would go over it fails with KAMSTA_E_OOM and leaves the context usable,
 * like a failed device allocation. */
kamsta_status kamsta_ctx_set_memory_limit(kamsta_ctx* ctx, uint64_t bytes);

/* ---- single-graph solve, host buffers ----------------------------------
 * edges: m_directed entries (host memory); out: capacity >= n-1 entries
 * (host memory).  Uses a per-thread default context on the current device.
 * Replaces hybridMST::boruvka (hybrid_boruvka.hpp:263-301).                 */
kamsta_status kamsta_mst_boruvka(const kamsta_wedge* edges, uint64_t m_directed,
                                 uint32_t n, const kamsta_cfg* cfg,
                                 kamsta_wedge* out, uint64_t* out_count,
                                 kamsta_stats* stats);
/* Replaces hybridMST::filter_boruvka (hybrid_boruvka_edgefilter.hpp:420-462). */
kamsta_status kamsta_mst_filter_boruvka(const kamsta_wedge* edges,
                                        uint64_t m_directed, uint32_t n,
                                        const kamsta_cfg* cfg, kamsta_wedge* out,
                                        uint64_t* out_count, kamsta_stats* stats);
/* Same as kamsta_mst_boruvka for the reference's 24-byte WEdge input; ids
 * must be < 2^32 (checked, KAMSTA_E_INPUT otherwise). */
kamsta_status kamsta_mst_boruvka_wedge64(const kamsta_wedge64* edges,
                                         uint64_t m_directed, uint64_t n,
                                         const kamsta_cfg* cfg,
                                         kamsta_wedge64* out,
                                         uint64_t* out_count,
                                         kamsta_stats* stats);

/* ---- single-graph solve, device buffers --------------------------------
 * d_edges / d_out are device pointers; the call is stream-ordered on
 * `stream` and returns after the result count is known (one host read per
 * Boruvka round).  out_count and stats are host pointers.                   */
kamsta_status kamsta_mst_boruvka_dev(kamsta_ctx* ctx, const kamsta_wedge* d_edges,
                                     uint64_t m_directed, uint32_t n,
                                     const kamsta_cfg* cfg, kamsta_wedge* d_out,
                                     uint64_t* out_count, kamsta_stats* stats,
                                     kamsta_stream stream);
kamsta_status kamsta_mst_filter_boruvka_dev(kamsta_ctx* ctx,
                                            const kamsta_wedge* d_edges,
                                            uint64_t m_directed, uint32_t n,
                                            const kamsta_cfg* cfg,
                                            kamsta_wedge* d_out,
                                            uint64_t* out_count,
                                            kamsta_stats* stats,
                                            kamsta_stream stream);

/* ---- single-graph solve without any allocation -------------------------
 * No counterpart in the reference.  For callers that cannot allocate device
 * memory (code inside another framework's fixed memory budget, allocator-
 * less runtimes, plugins handed only a stream and buffers): same result as
 * kamsta_mst_boruvka_dev, computed by one kernel whose scratch is a fixed
 * array inside the library (about 5 MB, held by every device that loads the
 * library until exit).  Limits: n <= 32768 and m_directed <= 262144, larger
 * graphs are rejected with KAMSTA_E_INPUT, and so is an entry with an id
 * >= n.  d_edges / d_out are device pointers, out_count / total_weight host
 * pointers; the call waits for `stream` and returns once the result is
 * known.  The first call on a device looks up the array's device address,
 * so make that first call before any stream capture; the address is kept
 * for the life of the device's primary context, so do not use the library
 * across a cudaDeviceReset.  Calls share the array: calls that overlap on
 * the GPU race and must be serialised. */
kamsta_status kamsta_mst_boruvka_noalloc(const kamsta_wedge* d_edges, uint64_t m_directed,
                                         uint32_t n, kamsta_wedge* d_out, uint64_t* out_count,
                                         uint64_t* total_weight, kamsta_stream stream);

/* ---- batched solve ------------------------------------------------------
 * No counterpart in the reference, whose benchmark solves one graph per job
 * (benchmarks/mst.cpp:215-228).  Graphs are solved in waves; each wave is the
 * disjoint union of consecutive graphs whose estimated device footprint fits
 * `budget_bytes` (0 = 32 GiB), solved as one graph, and the forest is split
 * back per graph.  Per graph the result equals kamsta_mst_boruvka (or
 * kamsta_mst_filter_boruvka with KAMSTA_FLAG_FILTER) on that graph alone,
 * with the forest sorted by (src, dst).  A graph whose ids are >= n (or, with
 * KAMSTA_FLAG_VALIDATE, whose entries are not (src,dst)-sorted) gets status
 * KAMSTA_E_INPUT without affecting the others. */
typedef struct kamsta_graph_desc {
  const kamsta_wedge* edges; /* in: m_directed entries, same contract as above */
  uint64_t m_directed;       /* in                                           */
  uint32_t n;                /* in: vertex count (< 2^31)                    */
  kamsta_status status;      /* out: KAMSTA_OK / KAMSTA_E_INPUT              */
  kamsta_wedge* out;         /* in: capacity >= max(n-1, 1) entries          */
  uint64_t out_count;        /* out: forest edges written                    */
  uint64_t total_weight;     /* out: forest weight                           */
} kamsta_graph_desc;

typedef struct kamsta_batch_stats {
  uint32_t graphs;           /* graphs in the call                           */
  uint32_t waves;            /* union solves                                 */
  uint32_t gpu_launches;     /* kernels launched                             */
  uint32_t pad_;
  uint64_t entries;          /* directed input entries over all graphs       */
  uint64_t vertices;         /* vertices over all graphs                     */
  uint64_t forest_edges;     /* forest edges over all graphs                 */
  double device_ms;          /* device time of the whole call (CUDA events)  */
  double solve_ms;           /* of which in the union solves                 */
} kamsta_batch_stats;

/* Device buffers: edges / out of every descriptor are device pointers; the
 * descriptors themselves are host memory. */
kamsta_status kamsta_mst_batch_dev(kamsta_ctx* ctx, kamsta_graph_desc* graphs,
                                   uint32_t count, const kamsta_cfg* cfg,
                                   uint64_t budget_bytes, kamsta_batch_stats* stats,
                                   kamsta_stream stream);
/* Host buffers (the library copies in and out; pinned memory is faster). */
kamsta_status kamsta_mst_batch(kamsta_ctx* ctx, kamsta_graph_desc* graphs, uint32_t count,
                               const kamsta_cfg* cfg, uint64_t budget_bytes,
                               kamsta_batch_stats* stats);

/* Batch tuning of a context: the CTA size of the persistent small-graph
 * kernel (256, 512 or 1024 threads) and the largest n it takes (4096 ..
 * 32768; larger graphs go to the union solve).  kamsta_batch_autotune times
 * every candidate on the given sample of graphs (device buffers; their
 * outputs are written as by kamsta_mst_batch_dev), keeps the fastest in the
 * context and reports the timings.  No counterpart in the reference. */
typedef struct kamsta_tuning {
  uint32_t small_threads;  /* chosen CTA size                                */
  uint32_t small_max_n;    /* chosen cutoff                                  */
  double threads_ms[3];    /* sample's small graphs at 256 / 512 / 1024      */
  double cutoff_ms[4];     /* whole sample at cutoff 4096 / 8192 / 16384 / 32768 */
} kamsta_tuning;
kamsta_status kamsta_batch_autotune(kamsta_ctx* ctx, kamsta_graph_desc* graphs,
                                    uint32_t count, const kamsta_cfg* cfg,
                                    kamsta_tuning* out, kamsta_stream stream);
/* Sets (e.g. from a cached autotune result) or clears (zeros) the tuning. */
kamsta_status kamsta_ctx_set_tuning(kamsta_ctx* ctx, const kamsta_tuning* tuning);

/* ---- single-graph tile autotuner ----------------------------------------
 * No counterpart in the reference.  Solves the given device input once
 * untimed, then once per (items_per_thread, seg_items_per_thread) pair of
 * {6, 8, 12} x {2, 4} with cfg's algorithm settings (KAMSTA_FLAG_FILTER
 * selects filter_boruvka), timing each solve with CUDA events, and keeps the
 * fastest pair in the context: later solves on this context whose cfg leaves
 * items_per_thread / seg_items_per_thread at 0 use it.  d_out needs room for
 * n - 1 entries (scratch).  ms[] is in the pair order (6,2) (8,2) (12,2)
 * (6,4) (8,4) (12,4). */
typedef struct kamsta_tile_tuning {
  uint32_t items_per_thread;      /* chosen first-pass entries per thread   */
  uint32_t seg_items_per_thread;  /* chosen list-pass records per thread    */
  double ms[6];                   /* device ms of each pair's solve          */
} kamsta_tile_tuning;
kamsta_status kamsta_autotune_tiles(kamsta_ctx* ctx, const kamsta_wedge* d_edges,
                                    uint64_t m_directed, uint32_t n, const kamsta_cfg* cfg,
                                    kamsta_wedge* d_out, kamsta_tile_tuning* out,
                                    kamsta_stream stream);
/* Sets (e.g. from a cached autotune result) or clears (zeros) the context's
 * single-graph tiles. */
kamsta_status kamsta_ctx_set_tiles(kamsta_ctx* ctx, uint32_t items_per_thread,
                                   uint32_t seg_items_per_thread);

/* ---- serving loop -------------------------------------------------------
 * No counterpart in the reference.  A continuous-batching request loop:
 * clients submit jobs whose edge arrays already sit in device memory (their
 * writes complete before the submit); worker threads (each with its own
 * context and stream) repeatedly take the queued jobs in arrival order while
 * their estimated device footprint fits the memory budget, and solve them as
 * one batch wave.  Jobs arriving while a wave runs join the next one; with
 * two or more workers, waves overlap on the device.  Each job's result is
 * the batch result of that graph alone (forest sorted by (src, dst)). */
typedef struct kamsta_server kamsta_server;

typedef struct kamsta_server_cfg {
  uint64_t budget_bytes;     /* admission budget, device bytes (0 = 64 GiB)   */
  uint32_t max_batch;        /* jobs per wave at most (0 = 4096)              */
  uint32_t workers;          /* worker threads / streams (1..8, default 2)   */
  kamsta_cfg solver;         /* solver options for every job (FILTER flag    */
                             /* selects filter_boruvka)                      */
  uint32_t small_threads;    /* batch tuning of the workers' contexts        */
  uint32_t small_max_n;      /* (kamsta_tuning; 0 = built-in default)        */
} kamsta_server_cfg;

typedef struct kamsta_request {
  const kamsta_wedge* d_edges; /* device, m_directed entries (input contract) */
  uint64_t m_directed;
  uint32_t n;
  uint32_t pad_;
  kamsta_wedge* d_out;         /* device, capacity >= max(n-1, 1)           */
  uint64_t user_tag;           /* returned in the completion                 */
} kamsta_request;

typedef struct kamsta_completion {
  uint64_t ticket;             /* from kamsta_server_submit                  */
  uint64_t user_tag;
  kamsta_status status;        /* KAMSTA_OK / KAMSTA_E_INPUT / solver error  */
                               /* / KAMSTA_E_CANCELLED                       */
  uint32_t batch_size;         /* jobs in the wave that solved this one      */
  uint64_t out_count;
  uint64_t total_weight;
  double submit_us;            /* steady-clock microseconds since create     */
  double start_us;             /* wave start                                 */
  double finish_us;            /* wave end (output written)                  */
} kamsta_completion;

kamsta_status kamsta_server_cfg_default(kamsta_server_cfg* cfg);
kamsta_status kamsta_server_create(int device, const kamsta_server_cfg* cfg,
                                   kamsta_server** out);
/* KAMSTA_E_BUDGET if the job alone exceeds one worker's share of the
 * budget (budget_bytes / workers), which is also the hard device-memory
 * limit of each worker's context. */
kamsta_status kamsta_server_submit(kamsta_server* server, const kamsta_request* req,
                                   uint64_t* ticket);
/* Up to `cap` completions; waits up to timeout_us for the first one.
 * KAMSTA_E_NOTREADY (count 0) when none finished in time. */
kamsta_status kamsta_server_poll(kamsta_server* server, kamsta_completion* out,
                                 uint32_t cap, uint32_t* count, uint32_t timeout_us);
/* Withdraws a job that is still queued: it completes at once with status
 * KAMSTA_E_CANCELLED (batch_size 0) and never touches its buffers.
 * KAMSTA_E_NOTREADY if the ticket is not queued (already in a wave,
 * finished, or unknown); such a job completes normally. */
kamsta_status kamsta_server_cancel(kamsta_server* server, uint64_t ticket);
kamsta_status kamsta_server_stats(kamsta_server* server, uint64_t* queued,
                                  uint64_t* in_flight, uint64_t* bytes_in_use,
                                  uint64_t* waves);
/* The per-worker device-memory limit (budget_bytes / workers) and the most
 * device memory any worker's context held during a wave so far (its pool's
 * high-water mark plus its arenas). */
kamsta_status kamsta_server_memory(kamsta_server* server, uint64_t* worker_limit,
                                   uint64_t* peak_worker_bytes);
/* Finishes every queued job, then stops the workers and frees the server. */
kamsta_status kamsta_server_destroy(kamsta_server* server);

/* ---- compressed input (Compression::SEVEN_BIT_DIFF_ENCODING) ------------
 * The reference's difference-encoded edge container
 * (datastructures/compression/difference_encoded_graph.hpp:14-261, varints
 * of variable_length_encoding.hpp:6-167): per edge varint(src - prev_src),
 * varint(dst), varint(w), 7 bits per byte, little endian, 0x80 = more bytes
 * follow.  The list is cut into chunks of chunk_edges (1..4096) edges, each
 * with its raw first edge and the byte offset of its encoded rest, so the
 * device decodes one chunk per CTA.  Input must be (src, dst) sorted. */
typedef struct kamsta_cgraph {
  uint64_t m_directed;            /* directed entries                          */
  uint32_t n;                     /* vertex count                              */
  uint32_t chunk_edges;           /* edges per chunk (the last may be shorter) */
  uint64_t num_chunks;            /* ceil(m_directed / chunk_edges)            */
  uint64_t data_bytes;            /* encoded bytes                             */
  const uint64_t* chunk_offset;   /* [num_chunks + 1] byte offsets into data   */
  const kamsta_wedge* chunk_first;/* [num_chunks] first edge of each chunk     */
  const uint8_t* data;            /* encoded edges 1.. of every chunk          */
} kamsta_cgraph;

/* Host encoder (all host cores).  With data == NULL only *data_bytes (and
 * chunk_offset, if given) is computed. */
kamsta_status kamsta_encode_7bit(const kamsta_wedge* edges, uint64_t m_directed,
                                 uint32_t chunk_edges, uint64_t* chunk_offset,
                                 kamsta_wedge* chunk_first, uint8_t* data,
                                 uint64_t data_capacity, uint64_t* data_bytes);
/* Device decoder: g holds device pointers; d_out receives m_directed entries. */
kamsta_status kamsta_decode_7bit_dev(kamsta_ctx* ctx, const kamsta_cgraph* g,
                                     kamsta_wedge* d_out, kamsta_stream stream);
/* Solve from a compressed graph held in device memory (decoded into
 * context scratch, then kamsta_mst_boruvka_dev). */
kamsta_status kamsta_mst_boruvka_7bit_dev(kamsta_ctx* ctx, const kamsta_cgraph* g,
                                          const kamsta_cfg* cfg, kamsta_wedge* d_out,
                                          uint64_t* out_count, kamsta_stats* stats,
                                          kamsta_stream stream);
/* Same from host memory: only the compressed bytes cross to the device, in
 * pieces that the device decodes as they land (keep the bytes in pinned
 * memory for the link's full rate).  The chunk table is checked on the host
 * first: byte offsets must never decrease and must end inside data_bytes
 * (KAMSTA_E_INPUT otherwise); a chunk whose bytes do not hold exactly its
 * values is KAMSTA_E_INPUT before the solve starts. */
kamsta_status kamsta_mst_boruvka_7bit(const kamsta_cgraph* g, const kamsta_cfg* cfg,
                                      kamsta_wedge* out, uint64_t* out_count,
                                      kamsta_stats* stats);

/* ---- reading the reference's binary edge files -------------------------
 * Real-world inputs of the reference (evaluation/README.md:21-22, read by
 * graphs::read_weighted_binaries(files, 4, 1),
 * benchmarks/mst_benchmarks.hpp:185-190): possibly unsorted edge lists of
 * 9-byte records (4-byte source, 4-byte destination, 1-byte weight, little
 * endian), over one or more files.  The files are streamed to the device
 * (reading and host-to-device copies overlap) and turned into the input
 * contract: sorted by (src, dst), self loops dropped, of duplicate (src,
 * dst) entries only the lightest kept; KAMSTA_LOAD_SYMMETRIZE adds the
 * reverse of every record first, so both directions are present.  n_out =
 * largest id + 1 (ids < 2^28).  kamsta_wedge9_capacity gives an upper bound
 * of the entries written (records, doubled when symmetrising). */
#define KAMSTA_LOAD_SYMMETRIZE 0x1u

/* Edge weights of the geometric generators (the reference's distance types,
 * benchmarks/mst_benchmarks.hpp:59-64): a seeded hash, or from the
 * distance d <= R of the endpoints: 1 + floor((max_weight - 1) d / R), or
 * 1 + floor((max_weight - 1) d^2 / R^2). */
#define KAMSTA_DISTANCE_RANDOM 0u
#define KAMSTA_DISTANCE_EUCLIDEAN 1u
#define KAMSTA_DISTANCE_SQUARED_EUCLIDEAN 2u
kamsta_status kamsta_wedge9_capacity(const char* const* paths, uint32_t num_paths,
                                     uint32_t flags, uint64_t* capacity);
kamsta_status kamsta_load_wedge9_dev(kamsta_ctx* ctx, const char* const* paths,
                                     uint32_t num_paths, uint32_t flags,
                                     kamsta_wedge* d_out, uint64_t capacity,
                                     uint64_t* m_directed_out, uint32_t* n_out,
                                     kamsta_stream stream);

/* MatrixMarket coordinate files (the reference's INFILE_UNWEIGHTED input,
 * read by graphs::read_unweighted_graph(file, GraphFormat::MatrixMarket) at
 * benchmarks/mst_benchmarks.hpp:181-184): entry (i, j), 1-based, is the
 * undirected edge {i-1, j-1}; values are ignored, self loops dropped,
 * repeated pairs merged; n = max(rows, cols) (< 2^31).  Every edge gets the
 * generators' weight in [1, max_weight] from `seed`.  The output is the
 * solver's input (both directions, (src, dst)-sorted).  kamsta_mtx_header
 * (host only) reads rows, cols and the stored entries; 2 * entries bounds
 * the directed entries.  Counting / capacity convention as
 * kamsta_gen_rgg2d_dev. */
kamsta_status kamsta_mtx_header(const char* path, uint64_t* rows, uint64_t* cols,
                                uint64_t* entries);
kamsta_status kamsta_load_mtx_dev(kamsta_ctx* ctx, const char* path, uint64_t seed,
                                  uint32_t max_weight, kamsta_wedge* d_out,
                                  uint64_t capacity, uint64_t* m_directed_out,
                                  uint32_t* n_out, kamsta_stream stream);

/* ---- device graph generators (seeded; identical to the oracle's CPU
 * generators).  d_out must hold 2*m entries; *m_directed_out receives the
 * number written.  Stand-ins for KaGen's get_gnm / get_rgg2D / get_rhg
 * (benchmarks/mst_benchmarks.hpp:116-199). -------------------------------- */
kamsta_status kamsta_gen_gnm_dev(kamsta_ctx* ctx, uint32_t n, uint64_t m,
                                 uint64_t seed, uint32_t max_weight,
                                 kamsta_wedge* d_out, uint64_t* m_directed_out,
                                 kamsta_stream stream);
/* 2-D random geometric graph on the unit square (radius in [0, 1]; for an
 * expected degree d away from the border, radius = sqrt(d / (pi n))).  The
 * edge count is data dependent: with d_out == NULL the call only counts
 * (*m_directed_out = entries needed); with capacity < that count it returns
 * KAMSTA_E_INPUT and the count.  `distance` is a KAMSTA_DISTANCE_* weight
 * rule (KAMSTA_DISTANCE_RANDOM: the hash weight).  Stand-in for get_rgg2D
 * (benchmarks/mst_benchmarks.hpp:133-139). */
kamsta_status kamsta_gen_rgg2d_dev(kamsta_ctx* ctx, uint32_t n, double radius,
                                   uint64_t seed, uint32_t max_weight,
                                   uint32_t distance, kamsta_wedge* d_out,
                                   uint64_t capacity, uint64_t* m_directed_out,
                                   kamsta_stream stream);
/* Threshold random hyperbolic graph: power-law exponent gamma > 2 (the
 * reference's --gamma), target average degree avg_degree; hubs of very high
 * degree.  Counting / capacity convention as kamsta_gen_rgg2d_dev.  The
 * per-point coordinates are computed on the host with the C library's
 * acosh/exp/sinh; the pair test runs on the device.  Stand-in for get_rhg
 * (benchmarks/mst_benchmarks.hpp:152-158). */
kamsta_status kamsta_gen_rhg_dev(kamsta_ctx* ctx, uint32_t n, double gamma,
                                 double avg_degree, uint64_t seed, uint32_t max_weight,
                                 kamsta_wedge* d_out, uint64_t capacity,
                                 uint64_t* m_directed_out, kamsta_stream stream);
/* Lattice of x * y * z vertices (z = 1: the 2-D grid), vertex (i, j, k) =
 * id (k y + j) x + i, joined to its -1 / +1 steps along each axis (modulo
 * the side when `periodic`); each edge kept with probability p (p >= 1: all,
 * as the reference's benchmark calls it).  Counting / capacity convention as
 * kamsta_gen_rgg2d_dev.  Stand-in for get_grid2D / get_grid3D
 * (benchmarks/mst_benchmarks.hpp:159-180). */
kamsta_status kamsta_gen_grid_dev(kamsta_ctx* ctx, uint32_t x, uint32_t y, uint32_t z,
                                  double p, int periodic, uint64_t seed,
                                  uint32_t max_weight, kamsta_wedge* d_out,
                                  uint64_t capacity, uint64_t* m_directed_out,
                                  kamsta_stream stream);
/* 3-D random geometric graph in the unit cube (radius in [0, 1]; for an
 * expected degree d away from the border, radius = cbrt(3 d / (4 pi n))).
 * Counting / capacity convention and `distance` as kamsta_gen_rgg2d_dev.
 * Stand-in for get_rgg3D (benchmarks/mst_benchmarks.hpp:140-146). */
kamsta_status kamsta_gen_rgg3d_dev(kamsta_ctx* ctx, uint32_t n, double radius,
                                   uint64_t seed, uint32_t max_weight,
                                   uint32_t distance, kamsta_wedge* d_out,
                                   uint64_t capacity, uint64_t* m_directed_out,
                                   kamsta_stream stream);
/* R-MAT graph on 2^log_n vertices (log_n <= 31): `samples` (< 2^32 - 4096)
 * recursive quadrant descents with probabilities a, b, c and d = 1 - a - b -
 * c (Graph 500: 0.57, 0.19, 0.19); the graph = the distinct pairs u != v,
 * ids not permuted (the hubs have the smallest ids).  Counting / capacity
 * convention as kamsta_gen_rgg2d_dev.  Stand-in for
 * get_rmat_edges_evenly_distributed (benchmarks/mst_benchmarks.hpp:147-151). */
kamsta_status kamsta_gen_rmat_dev(kamsta_ctx* ctx, uint32_t log_n, uint64_t samples,
                                  double a, double b, double c, uint64_t seed,
                                  uint32_t max_weight, kamsta_wedge* d_out,
                                  uint64_t capacity, uint64_t* m_directed_out,
                                  kamsta_stream stream);

#ifdef __cplusplus
} /* extern "C" */
#endif
#endif /* KAMSTA_GPU_H */
