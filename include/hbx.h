/* hbx.h -- C ABI of the GB300 rule-based blocking engine (libhbx.so).
 *
 * The engine evaluates HyperBlocker rules (equalities + Jaro-Winkler
 * similarity predicates, OR across rules, AND within a rule) over every
 * left x right pair of the reference's hash partitions and returns the
 * matching (left row, right row) pairs.  Row numbers count CSV lines from 0,
 * the header line included, because the reference reads the header as data
 * (core/components/data_mngr.h:48-51, rapidcsv LabelParams(-1, -1)).
 *
 * Every call returns an hbx_status; no C++ exception crosses this boundary.
 * hbx_last_error() gives the text of the last failure on a context.
 * A context is used by one host thread at a time.
 *
 * Reference interfaces replaced (paths inside the HyperBlocker project):
 *   examples/run_hyperblocker.cu:22-59         -> hbx_run_cli
 *   core/hyperblocker.cuh:45-131 (HyperBlocker) -> hbx_ctx_* / hbx_block
 *   core/components/execution_plan_generator.h:64-155
 *                                               -> hbx_plan_from_rule_dir,
 *                                                  hbx_plan_from_yaml,
 *                                                  hbx_plan_serialized
 *   core/components/data_mngr.h:46-79 (CSV ingest)
 *                                               -> hbx_table_from_csv,
 *                                                  hbx_table_ingest
 *   core/components/data_mngr.h:81-222 (partitioning) +
 *   core/components/host_producer.h:109-215 (AsyncSubmit) +
 *   core/gpu/global_func.cuh:104-185 (blocking_kernel)
 *                                               -> hbx_session_create /
 *                                                  hbx_session_run, hbx_block
 *   core/components/host_reducer.h:80-90 (WriteMatch)
 *                                               -> hbx_write_pairs
 */
#ifndef HBX_H_
#define HBX_H_

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef enum hbx_status {
  HBX_OK = 0,
  HBX_ERR_INVALID_ARG = 1,
  HBX_ERR_CUDA = 2,
  HBX_ERR_OOM = 3,
  HBX_ERR_CAPACITY = 4,   /* output buffer too small; n_required is set, n_written is 0 */
  HBX_ERR_WATCHDOG = 5,   /* a device loop exceeded its time budget and stopped */
  HBX_ERR_PARSE = 6,      /* malformed CSV or YAML rule */
  HBX_ERR_IO = 7,         /* file could not be read or written */
  HBX_ERR_UNSUPPORTED = 8, /* input the engine refuses (undefined in the reference) */
  HBX_ERR_TIMEOUT = 9      /* hbx_serve_poll: no result became ready within the timeout */
} hbx_status;

typedef enum hbx_mode {
  /* one launch per (partition, rule), like the reference's per-partition
   * AsyncSubmit loop (host_producer.h:75-104) */
  HBX_MODE_PLAIN = 0,
  /* every rule x partition in one persistent work-stealing launch, replayed
   * from a CUDA graph */
  HBX_MODE_BATCHED = 1
} hbx_mode;

typedef struct hbx_ctx hbx_ctx;
typedef struct hbx_plan hbx_plan;
typedef struct hbx_table hbx_table;
typedef struct hbx_session hbx_session;
typedef struct hbx_server hbx_server;

typedef struct hbx_opts {
  uint32_t struct_size;      /* sizeof(hbx_opts) */
  int32_t use_graph;         /* batched mode replays a CUDA graph (default 1) */
  int32_t tile_right;        /* right rows per work item, 0 = autotuned */
  int32_t eval_variant;      /* evaluation kernel: 1 = 3 CTAs/SM, 2 = 2 CTAs/SM with more
                                registers, 0 = autotuned */
  int32_t pred_order;        /* similarity predicates of a rule run in: 0 = order of measured
                                selectivity and cost (default), 1 = the order the rule gives */
  int32_t ingest;            /* tables are encoded: 0 = on the device (default: buckets,
                                dictionaries, composite join keys, arenas; the host
                                encoder takes over only beyond 2^30 rows, or when
                                dictionary cells collide under four hash seeds),
                                1 = on the host */
  uint64_t watchdog_cycles;  /* per-CTA SM-cycle budget of the persistent loop, 0 = none */
} hbx_opts;

/* Column-major host strings: cell (r, c) is data[c][offsets[c][r] .. offsets[c][r+1]). */
typedef struct hbx_columns {
  int64_t n_rows;
  int32_t n_cols;
  const char* const* data;
  const int64_t* const* offsets;
} hbx_columns;

/* Output pair buffer.  hbx_session_run takes device pointers, which the
 * kernels write directly (after HBX_ERR_CAPACITY their contents are
 * undefined); hbx_block takes host pointers, untouched on HBX_ERR_CAPACITY. */
typedef struct hbx_pairs {
  uint32_t* l_row;
  uint32_t* r_row;
  uint64_t capacity;
  uint64_t n_written;   /* out */
  uint64_t n_required;  /* out: total matches (also when HBX_ERR_CAPACITY) */
} hbx_pairs;

typedef struct hbx_stats {
  uint64_t pairs_covered;     /* sum over partitions of |L_p| * |R_p| */
  uint64_t pair_comparisons;  /* (rule, l, r) triples whose equalities hold */
  uint64_t n_matches;         /* distinct matching pairs */
  uint64_t fma_ambiguous;     /* JW decisions that differ with/without FMA (reported) */
  uint64_t long_string_pairs; /* JW evaluations whose shorter string > 256 bytes */
  uint64_t n_tiles;           /* work items of the last run */
  uint32_t n_partitions_used; /* partitions with both sides non-empty */
  uint32_t n_launches;        /* kernels launched by the last run */
  double ms_last_run;         /* device time of the last run (CUDA events) */
  double ms_join;             /* device time of the equality join phase */
  double ms_eval;             /* device time of the pair-evaluation kernel(s) */
  uint64_t jw_word_ops;       /* algorithmic 64-bit word operations of the JW phase */
  uint64_t h2d_bytes;         /* bytes uploaded when the session was created */
  double ms_create;           /* host wall time of the session's creation */
  uint32_t ingest_on_device;  /* 1 when the tables were encoded on the device */
  uint32_t tile_right;        /* right rows per work item of the last run */
  uint32_t eval_variant;      /* evaluation kernel of the last run (hbx_opts numbering) */
  uint32_t n_windows;         /* partition windows of the call (hbx_block_streamed), else 1 */
  uint64_t pairs_scanned;     /* JW evaluations the filters could not settle (bit-parallel scans) */
  uint64_t scan_steps;        /* steps of those scans, 4 symbols each */
  uint64_t scan_word_ops;     /* operations those scans executed, in jw_word_ops' unit (6 per
                                 64-bit mask word per character scanned) */
  uint32_t scan_words;        /* 32-bit words per scan mask in the last run (1, 2, 3, 4 or 8) */
  uint32_t reserved0;
  uint64_t scan_warp_steps;   /* warp-level scan steps: scan_steps / (4 x 32 x this) is the
                                 share of lanes busy in the scan loop */
  uint64_t rest_scans;        /* of pairs_scanned, scans of predicates after a rule's (or rule
                                 group's) first similarity predicate */
} hbx_stats;

/* ---- context ------------------------------------------------------------ */
hbx_status hbx_ctx_create(int device, const hbx_opts* opts, hbx_ctx** out);
hbx_status hbx_ctx_destroy(hbx_ctx* ctx);
const char* hbx_last_error(const hbx_ctx* ctx);
const char* hbx_status_string(hbx_status s);

/* ---- rules (yaml_config.h:37-75, execution_plan_generator.h:64-155) ----- */
/* Reads every entry of rule_dir in directory order, decodes each as a rule,
 * orders rules like the reference (std::sort on equality-list size,
 * descending) and compiles the evaluation order (equalities first, then
 * similarity predicates by measured selectivity and cost). */
hbx_status hbx_plan_from_rule_dir(hbx_ctx* ctx, const char* rule_dir, hbx_plan** out);
/* Same from in-memory YAML documents, given in directory order. */
hbx_status hbx_plan_from_yaml(hbx_ctx* ctx, const char* const* docs, int32_t n_docs,
                              hbx_plan** out);
/* The reference's serialized plan (execution_plan_generator.h:25-31). */
hbx_status hbx_plan_serialized(const hbx_plan* plan, int32_t* length,
                               const int32_t** pred_index, const char** pred_type,
                               const float** pred_threshold);
int32_t hbx_plan_n_rules(const hbx_plan* plan);
hbx_status hbx_plan_destroy(hbx_plan* plan);

/* ---- tables (data_mngr.h:46-79) ----------------------------------------- */
hbx_status hbx_table_from_csv(hbx_ctx* ctx, const char* path, char sep, hbx_table** out);
hbx_status hbx_table_ingest(hbx_ctx* ctx, const hbx_columns* cols, hbx_table** out);
int64_t hbx_table_n_rows(const hbx_table* t);
int32_t hbx_table_n_cols(const hbx_table* t);
/* Column c of a table as parsed: *bytes holds the cells back to back, cell i
 * is bytes[offsets[i] .. offsets[i + 1]) (n_rows + 1 offsets); the pointers
 * stay valid until the table is destroyed. */
hbx_status hbx_table_column(const hbx_table* t, int32_t c, const char** bytes,
                            const int64_t** offsets);
hbx_status hbx_table_destroy(hbx_table* t);

/* ---- blocking ------------------------------------------------------------ */
/* Encodes both tables for the plan (partition buckets with the reference's
 * std::hash, int32 dictionary codes for equality columns, 16-byte-aligned
 * length-prefixed string arenas), uploads them and sizes the device state.
 * prefix_idx = INT32_MAX disables the reference's prefix hash. */
hbx_status hbx_session_create(hbx_ctx* ctx, const hbx_plan* plan, const hbx_table* left,
                              const hbx_table* right, uint64_t n_partitions, int64_t prefix_idx,
                              hbx_session** out);
/* Runs the pair evaluation on device-resident inputs; out holds DEVICE
 * pointers.  stream may be NULL (the context's stream).  Returns when the
 * pairs are in out (synchronous on the stream). */
hbx_status hbx_session_run(hbx_session* s, hbx_mode mode, hbx_pairs* out, void* stream);
hbx_status hbx_session_stats(const hbx_session* s, hbx_stats* out);
hbx_status hbx_session_destroy(hbx_session* s);

/* One call from host tables to host pairs: session create + run + copy back.
 * out holds HOST pointers.  The tables are encoded on the context's stream;
 * the run and the copy of the pairs go to `stream` (a cudaStream_t, NULL =
 * the context's stream), the stream the reference's AsyncSubmit takes
 * (host_producer.h:109-112).  The pairs come back through 512 MiB of
 * page-locked host memory the context allocates on its first call (two
 * chunks, each copied into out while the next one transfers).  Returns when
 * the pairs are in out. */
hbx_status hbx_block(hbx_ctx* ctx, const hbx_plan* plan, const hbx_table* left,
                     const hbx_table* right, uint64_t n_partitions, int64_t prefix_idx,
                     hbx_mode mode, hbx_pairs* out, hbx_stats* stats, void* stream);

/* Appends "<id_l>,<id_r>\n" lines (column 0 of each table), like
 * host_reducer.h:80-90.  Pairs are written in the order given.  With a
 * context and at least 65,536 pairs the lines are formatted on its device
 * (hbx_write_pairs_device); the bytes are the same. */
hbx_status hbx_write_pairs(hbx_ctx* ctx, const hbx_table* left, const hbx_table* right,
                           const uint32_t* l_row, const uint32_t* r_row, uint64_t n,
                           const char* path);

/* hbx_write_pairs for pairs in DEVICE memory (l_row, r_row: device arrays of
 * n rows), formatted on the device: the same bytes as hbx_write_pairs, in
 * chunks of at most 64 MiB of text, each appended to path while the next is
 * formatted (replaces host_reducer.h:80-90 for large outputs). */
hbx_status hbx_write_pairs_device(hbx_ctx* ctx, const hbx_table* left, const hbx_table* right,
                                  const uint32_t* l_row, const uint32_t* r_row, uint64_t n,
                                  const char* path);

/* hbx_block for tables whose encoding need not fit the device at once (the
 * reference's per-partition pipeline, host_producer.h:75-104, with a memory
 * bound): partitions are grouped into windows of at most window_bytes of
 * device memory (a partition larger than that is split by its left rows), and
 * two workers with their own streams process windows in turn, so one
 * window's copies and encoding overlap another's evaluation.  A window's
 * pair output (up to window_bytes / 8 pairs, more if it needs them) comes on
 * top of the budget.  Same pairs as
 * hbx_block (in another order); stats->n_windows counts the windows and
 * ms_last_run is the wall time of the call.  out holds HOST pointers. */
hbx_status hbx_block_streamed(hbx_ctx* ctx, const hbx_plan* plan, const hbx_table* left,
                              const hbx_table* right, uint64_t n_partitions, int64_t prefix_idx,
                              hbx_mode mode, uint64_t window_bytes, hbx_pairs* out,
                              hbx_stats* stats);

/* The run_hyperblocker_exec command line (examples/run_hyperblocker.cu:22-59):
 * -data_l -data_r -rule_dir -o -n_partitions [-sep -scheduler -read_header
 * -prefix_hash_pred_idx], plus -hbx_mode=plain|batched.  Returns a process
 * exit code (0 on success). */
int hbx_run_cli(int argc, const char* const* argv);

/* ---- serving -------------------------------------------------------------
 * No counterpart in the reference, which runs one batch job per process.  A
 * server keeps one right table resident on the device and answers requests
 * as they arrive: each request is a batch of left records and the index of
 * one of the server's plans; its result is every (left record, right row)
 * pair that some rule of that plan accepts (equalities, then similarities,
 * as in hbx_block), over all pairs (one partition).
 *
 * A worker thread forms batches of up to max_batch_rows records from the
 * queued requests while the device memory they need fits the budget: a
 * request is dispatched in row chunks, requests with the fewest records left
 * go first (requests waiting over 200 ms go ahead of them), and each batch
 * evaluates every (chunk, rule) pair in one persistent launch.  Up to
 * max_inflight batches are on the device at once, so requests that arrive
 * while others run are admitted as soon as a batch slot and memory free up
 * (continuous batching).  A request's result does not depend on what it was
 * batched with or how it was chunked.
 *
 * hbx_serve_submit and hbx_serve_poll may be called from any threads; one
 * thread at a time should poll.  The server uses its context's device and
 * memory pool; destroy the server before the context. */
typedef struct hbx_serve_opts {
  uint32_t struct_size;     /* sizeof(hbx_serve_opts) */
  int32_t max_inflight;     /* batches on the device at once, 0 = 2 */
  int64_t max_batch_rows;   /* left records per batch, 0 = 4096 */
  uint64_t budget_bytes;    /* device memory for batches in flight, 0 = half of the free memory */
  int32_t tile_right;       /* right rows per work item, 0 = 128 */
  int32_t eval_variant;     /* evaluation kernel as hbx_opts, 0 = 2 CTAs/SM */
} hbx_serve_opts;

typedef struct hbx_serve_result {
  uint64_t req_id;
  hbx_status status;
  int32_t plan;
  uint64_t n_pairs;
  const uint32_t* l_row;     /* row of the request's records; valid until the next poll */
  const uint32_t* r_row;     /* row of the resident table */
  uint64_t pair_comparisons; /* (rule, left, right) triples whose equalities hold */
  double ms_queued;          /* submit -> admitted into a batch */
  double ms_total;           /* submit -> result ready */
  uint32_t batch_requests;   /* requests in the batch this one ran in */
  uint32_t batch_id;
} hbx_serve_result;

typedef struct hbx_serve_stats {
  uint64_t requests_done;
  uint64_t batches;
  uint64_t rows;              /* left records evaluated */
  uint64_t pair_comparisons;
  uint64_t n_pairs;
  double ms_device;           /* summed device time of the batches (CUDA events) */
  uint64_t budget_bytes;
  uint64_t peak_bytes;        /* largest device memory held by batches in flight */
  uint64_t resident_bytes;    /* device memory of the resident table and its joins */
} hbx_serve_stats;

/* plans[k] is request plan k; every plan's column indices refer to the
 * request records (left) and the resident table (right). */
hbx_status hbx_serve_open(hbx_ctx* ctx, const hbx_plan* const* plans, int32_t n_plans,
                          const hbx_table* right, const hbx_serve_opts* opts, hbx_server** out);
/* Copies the records and queues the request; returns at once.  A request
 * whose first chunk alone exceeds the budget is refused with
 * HBX_ERR_CAPACITY. */
hbx_status hbx_serve_submit(hbx_server* s, uint64_t req_id, int32_t plan, const hbx_columns* left);
/* Waits up to timeout_ms (< 0: no limit) for a finished request and returns
 * it; HBX_ERR_TIMEOUT when none finished in time.  out->status is the
 * request's own outcome. */
hbx_status hbx_serve_poll(hbx_server* s, int32_t timeout_ms, hbx_serve_result* out);
hbx_status hbx_serve_get_stats(const hbx_server* s, hbx_serve_stats* out);
/* Finishes the queued and running requests, then frees the server. */
hbx_status hbx_serve_close(hbx_server* s);
const char* hbx_serve_last_error(const hbx_server* s);

/* ---- blocking without device allocation ----------------------------------
 * No counterpart in the reference.  For callers that cannot call cudaMalloc:
 * an application whose device memory is handed out up front by another
 * runtime or pool, a process under a fixed device-memory budget, or a
 * latency-critical loop that cannot pay for cudaMalloc/cudaFree, which may
 * synchronize the device.  Same result as hbx_block, but every buffer the
 * kernels need (the device encoder's included: the tables are encoded on the
 * device, as hbx_block does) comes from one static device array of 64 MiB
 * inside libhbx.so (held on every GPU that loads the library until exit);
 * this call allocates no device memory and creates no stream, event or graph.
 *   - out holds DEVICE pointers owned by the caller; stream may be NULL;
 *   - inputs whose encoding, join state and duplicate set exceed the 64 MiB
 *     are refused with HBX_ERR_INVALID_ARG (hbx_static_last_error() gives the
 *     bytes needed);
 *   - all calls share the array: calls whose GPU work overlaps (other host
 *     threads, unordered streams) race; each call clears what must start at
 *     zero itself;
 *   - the call cannot be captured into a CUDA graph: it copies from pageable
 *     host memory and synchronizes the stream; on a failure after its first
 *     launch it still waits for its kernels, so the array is free when it
 *     returns.
 * Returns when the pairs are in out (synchronous on the stream). */
hbx_status hbx_block_static(int device, const hbx_plan* plan, const hbx_table* left,
                            const hbx_table* right, uint64_t n_partitions, int64_t prefix_idx,
                            hbx_pairs* out, void* stream, hbx_stats* stats);
/* Text of the last hbx_block_static failure on the calling thread. */
const char* hbx_static_last_error(void);

#ifdef __cplusplus
}
#endif

#endif /* HBX_H_ */
