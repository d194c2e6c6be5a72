/* sgns.h -- C ABI of the GB300 DSGL skip-gram negative-sampling trainer.
 *
 * A drop-in for the trainer DistGER's huge_walk runs over its walk corpus:
 *   int dsgl(int argc, char** argv, vector<int>* vertex_cn,
 *            vector<vertex_id_t>* new_sort, WalkEngine<real_t,uint32_t>* graph)
 *   (include/dsgl.hpp:1464 in trsenli/GDistGER-re; called from the commented-out
 *   src/examples/huge_walk.cpp:133), and its GPU sibling
 *   int train_corpus_cuda(int argc, char** argv, ...)  (src/word2vec.cu:1429).
 * The reference passes everything through argv flags and globals and exits on error;
 * here a handle owns all device memory, options are a plain struct (filled from the
 * same flags by sgns_options_from_args), and every call returns an sgns_status.
 *
 * Pointers are host pointers unless a parameter says "device".  All entry points are
 * thread-safe for distinct handles; one handle must not be used by two threads at once.
 */
#ifndef SGNS_H_
#define SGNS_H_

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef enum sgns_status {
  SGNS_OK = 0,
  SGNS_EINVAL = 1,   /* bad argument or option (message in sgns_last_error) */
  SGNS_ENOMEM = 2,   /* host or device allocation failed */
  SGNS_ECUDA = 3,    /* CUDA runtime error, or no usable GPU */
  SGNS_ETIMEOUT = 4, /* a device-side bounded wait gave up */
  SGNS_EIO = 5,      /* file could not be read or written */
  SGNS_ESTATE = 6    /* call out of order (e.g. training before sgns_set_vocab) */
} sgns_status;

typedef enum sgns_storage {
  SGNS_STORE_FP32 = 0,    /* reference precision */
  SGNS_STORE_BF16_SR = 1  /* bf16 tables, fp32 arithmetic, stochastic rounding on write-back */
} sgns_storage;

typedef enum sgns_engine {
  /* Reference memory policy (per-walk input buffers snapshot at walk load and written
   * back at walk end; per-pool negative buffer), state in HBM, one launch per step.
   * With workers = 1 it reproduces the reference's single-thread result bit for bit. */
  SGNS_ENGINE_PLAIN = 0,
  /* Persistent kernel: one launch trains the whole corpus; each worker holds its two
   * walks' context rows in shared memory over the sliding window [pos-w, pos+w] and
   * reads/updates negative rows in the table directly.  Launch captured in a CUDA
   * graph; warps per CTA and worker count chosen by the autotuner. */
  SGNS_ENGINE_PERSISTENT = 1
} sgns_engine;

typedef enum sgns_mode {
  /* Workers train concurrently and write the shared tables without locks, as the
   * reference's compute threads do (dsgl.hpp:1352-1356, 1380-1404). */
  SGNS_MODE_HOGWILD = 0,
  /* One worker: a deterministic run that replays the reference's single-compute-thread
   * order, bit for bit with the CPU oracle (and, for the plain engine, with the
   * reference itself).  workers must be 0 or 1. */
  SGNS_MODE_REPLAY_EXACT = 1
} sgns_mode;

typedef struct sgns_options {
  int32_t size;        /* -size       hidden size d (multiple of 4, <= 256)       */
  int32_t window;      /* -window     w (1..16)                                   */
  int32_t negative;    /* -negative   K (0..10)                                   */
  int32_t batch_size;  /* -batch-size accepted; the reference replaces it by 2w+1 (dsgl.hpp:832) */
  float sample;        /* -sample     subsampling threshold                       */
  float alpha;         /* -alpha      starting learning rate (linear decay)       */
  int32_t min_count;   /* -min-count  accepted; unused by the reference vocab path (dsgl.hpp:314-382) */
  int32_t iter;        /* -iter       passes over the corpus                      */
  int32_t threads;     /* -threads    partition of the unigram-table sum (dsgl.hpp:127) */
  int32_t debug;       /* -debug                                                  */
  int32_t binary;      /* -binary     1 = raw float rows in sgns_save_text        */
  int32_t storage;     /* sgns_storage                                            */
  int32_t engine;      /* sgns_engine                                             */
  int32_t workers;     /* independent trainers (the reference's compute threads); 0 = tuned */
  int32_t warps_per_cta; /* persistent engine CTA shape; 0 = tuned                */
  int32_t device;      /* CUDA device ordinal                                     */
  int32_t compute_loss;/* 1 = also accumulate the SGNS loss (fp64 reduction)      */
  int32_t mode;        /* sgns_mode (-mode hogwild|exact)                         */
  int64_t table_size;  /* unigram table entries (the reference fixes 1e8, dsgl.hpp:82) */
  uint64_t seed;       /* stochastic-rounding stream seed                         */
  int32_t forward_tile;/* persistent engine, lanes per input row in the forward dot
                          products: 1 = one lane per input; 2 = two lanes per input while
                          at most 16 inputs remain (d <= 128, K <= 5 only; the same sums);
                          0 = chosen by the autotuner                              */
  int32_t windows_per_step; /* 2 (or 0): the reference's step over two walks, target 1
                          labelling walk 1's window and target 2 walk 2's (dsgl.hpp:
                          1100-1159); 1: one walk per step -- its window and target with
                          the shared negatives (-windows-per-step 1)               */
} sgns_options;

typedef struct sgns_stats {
  uint64_t steps;              /* minibatches trained (one per target pair of walks) */
  uint64_t pairs;              /* (context, target) pairs = input rows over all steps */
  uint64_t word_count_actual;  /* tokens consumed, as the reference counts them      */
  uint64_t row_bytes;          /* algorithmic row traffic of the run: every step reads
                                  and writes its input and output rows once,
                                  2 (pairs + output_rows) d elem_bytes            */
  double loss;                 /* sum of SGNS losses (compute_loss = 1), fp64        */
  float final_alpha;
  float train_ms;              /* device time of the last training call              */
  int32_t workers;
  int32_t warps_per_cta;
  uint64_t row_loads;          /* table rows copied into worker buffers              */
  uint64_t row_stores;         /* table rows written back from worker buffers        */
  uint64_t output_rows;        /* sum over steps of the output rows (targets + negatives) */
  int32_t forward_tile;        /* persistent engine: lanes per input in the forward      */
  int32_t warps_per_worker;    /* warps that train one worker (one: its state lives in
                                  that warp's registers and shared memory)              */
} sgns_stats;

/* Defaults of dsgl.hpp:67-76, table_size 1e8, persistent engine, fp32. */
void sgns_default_options(sgns_options* opt);
/* Fills opt from word2vec-style flags exactly as dsgl.hpp:1495-1535 scans them
 * (unknown flags ignored).  Adds -storage fp32|bf16, -engine plain|persistent,
 * -mode hogwild|exact, -workers N, -table-size N, -seed N. */
sgns_status sgns_options_from_args(sgns_options* opt, int argc, const char* const* argv);

typedef struct sgns_handle sgns_handle;

/* Creates a trainer on opt->device.  Replaces dsgl()'s flag scan and globals. */
sgns_status sgns_create(const sgns_options* opt, sgns_handle** out);
void sgns_destroy(sgns_handle* h);
/* Message of the last failed call on h; with h NULL, of the calling thread's last failed
 * call that has no handle (sgns_create, sgns_options_from_args, the kernel-level entry
 * points).  Valid until the next failure on h, or of that thread. */
const char* sgns_last_error(const sgns_handle* h);

/* Vocabulary from per-vertex occurrence counts (the reference's vertex_cn), then the
 * reference's set-up: rows sorted by count (dsgl.hpp:246-252, 314-382), the unigram^0.75
 * table (dsgl.hpp:121-147), Wih from the reference LCG, Woh = 0 (dsgl.hpp:433-457), the
 * sigmoid table (dsgl.hpp:1557-1562).  Requires V >= 2 (the reference asserts V > 1000). */
sgns_status sgns_set_vocab(sgns_handle* h, const int32_t* vertex_counts, int64_t V);
/* Re-initialises Wih/Woh as sgns_set_vocab does, keeping vocabulary and tables. */
sgns_status sgns_reset_model(sgns_handle* h);

/* Copies a corpus to the device: vertex ids with -1 walk separators, the in-memory
 * walk stream the reference reads from graph->local_corpus (path.hpp:96,110). */
sgns_status sgns_upload_corpus(sgns_handle* h, const int32_t* tokens, int64_t n_tokens);
/* Trains -iter passes over the uploaded corpus (Train_SGNS_MPI, dsgl.hpp:522-1427). */
sgns_status sgns_train(sgns_handle* h);
/* Upload + train in one call: the reference's dsgl() hot path from host memory. */
sgns_status sgns_train_corpus(sgns_handle* h, const int32_t* tokens, int64_t n_tokens);
/* Reads one or more walk files (" %u" per vertex, one walk per line; path.hpp:92,108),
 * parses them on the GPU (sgns_parse_walks; the end of each file ends its last walk),
 * counts vertices (vertex_cn, path.hpp:98) on the GPU, builds the vocabulary over
 * max_vertex_id+1 vertices (or V if V > 0) and trains on the parsed corpus. */
sgns_status sgns_train_walk_files(sgns_handle* h, const char* const* paths, int32_t n_paths, int64_t V);

/* Kernel-level walk-text parser, replacing the host reader of word2vec.cu:1002-1041
 * (strtok on " \n\r\t" per line).  bytes: n bytes of walk text in device memory, read as
 * one file (the end of the buffer ends its last walk).  tokens: device output of cap
 * entries: vertex ids in text order with -1 after each line that holds at least one id
 * (the layout of graph->local_corpus, path.hpp:96,110).  *n_tokens: the number of entries
 * the text yields, also set when cap is too small (then SGNS_EINVAL is returned and
 * nothing is written); *max_id: the largest id, -1 if none.  A byte other than a digit,
 * space, tab, CR or LF, or an id above 2^31 - 1, is SGNS_EINVAL naming its offset.
 * Ordered on stream; returns after the parse has finished.  Uses library scratch memory. */
sgns_status sgns_parse_walks(const uint8_t* bytes, int64_t n, int32_t* tokens, int64_t cap, int64_t* n_tokens,
                             int64_t* max_id, void* stream);

sgns_status sgns_get_stats(const sgns_handle* h, sgns_stats* out);
int64_t sgns_vocab_size(const sgns_handle* h);
/* Row -> vertex id of the frequency-sorted rows (v_vocab[r].id). */
sgns_status sgns_get_order(const sgns_handle* h, uint32_t* order_out);
/* which: 0 = Wih (the written embedding), 1 = Woh.  V*d floats in sorted-row order.  BF16
 * tables are widened on the device; when out is 16-byte aligned pinned host memory mapped
 * for the handle's device, the widening kernel writes it in place (no staging copy). */
sgns_status sgns_get_embeddings(sgns_handle* h, int32_t which, float* out);
/* Overwrites Wih/Woh (sorted-row order, V*d floats; rounded to nearest for bf16). */
sgns_status sgns_set_embeddings(sgns_handle* h, int32_t which, const float* in);
/* Device pointers of Wih/Woh (fp32 or bf16 elements, sorted-row order). */
sgns_status sgns_device_tables(sgns_handle* h, void** wih, void** woh);
/* ---- hotness-block model sync between replicas (dsgl.hpp:548-781) ---------------------
 * Data-parallel replicas (one per GPU, each training its own walks) average a sample of
 * rows every sync period: rows sorted by count fall into blocks of equal count
 * (word_freq_block, dsgl.hpp:493-509); one row is drawn per block -- every block but the
 * last, as the reference's loop does (dsgl.hpp:645-711) -- and those rows of Wih and Woh
 * are summed over the replicas (MPI_Allreduce, dsgl.hpp:739-740) and divided by the replica
 * count (:741-746).  The library provides the row draw and the device gather / scatter;
 * the caller's collective (NCCL, MPI, torch.distributed) sums the gathered rows.
 *
 * sgns_sync_rows: the rows of one sync round, drawn from a counter-based stream of (seed,
 * round) so every replica draws the same rows (the reference broadcasts rank 0's draw,
 * :724-729); full = 1 gives every row (the reference's full sync, :602-630).  rows: host
 * output of capacity cap (V is enough); *n_rows: the count. */
sgns_status sgns_sync_rows(const sgns_handle* h, uint64_t seed, uint64_t round, int32_t full, int32_t* rows,
                           int64_t cap, int64_t* n_rows);
/* Rows rows[0..n) (device) of Wih (which = 0) or Woh (1) into buf (device, n x d fp32),
 * ordered on the handle's stream; returns when buf is written. */
sgns_status sgns_gather_rows(sgns_handle* h, int32_t which, const int32_t* rows, int64_t n, float* buf);
/* The reverse: table row rows[i] = buf[i] / divisor (fp32 division; bf16 tables round to
 * nearest even, so every replica stores identical bits). */
sgns_status sgns_scatter_rows(sgns_handle* h, int32_t which, const int32_t* rows, int64_t n, const float* buf,
                              float divisor);

/* my_saveModel (dsgl.hpp:1443-1461): "V d\n" then "<id> " + d x "%f " + "\n" per row. */
sgns_status sgns_save_text(sgns_handle* h, const char* path);

/* ---- kernel-level entry points (device pointers, caller's stream) ------------------
 * One minibatch update of the reference step (dsgl.hpp:1241-1311) for n independent
 * minibatches whose rows are given explicitly, computed by the same device code as the
 * trainers.  Per minibatch b: in_count[b] input rows (in_first[b] of them from walk 1),
 * out_count[b] output rows (row 0 = target of walk 1, last = target of walk 2),
 * out_meta = multiplicities, alpha[b].  Rows are concatenated over b (fp32).  Writes
 * d_in (the reference's updated inputM) and d_out (outputMd).  storage selects the
 * accumulation of the trainer that is mirrored (fp32 for both storages). */
sgns_status sgns_minibatch_update(int32_t d, int32_t n_batches, const int32_t* in_count,
                                  const int32_t* in_first, const int32_t* out_count,
                                  const int32_t* out_meta, const float* alpha,
                                  const float* in_rows, const float* out_rows, float* d_in,
                                  float* d_out, void* stream);

/* sgns_minibatch_update followed by the write-back of the BF16 trainers: every updated row
 * (input row j + its update, output row i + outputMd row i) is stored as bf16 bits with
 * their stochastic rounding (cvt.rs.bf16x2 fed by the counter hash of sr_seed, the
 * minibatch index and the row's index within it).  The per-minibatch error of BF16 storage
 * against an FP64 step is measured on these rows.  in_rows/out_rows: fp32 values (pass
 * widened bf16 rows to continue from a BF16 table); new_in/new_out: uint16 bf16 bits, laid
 * out like in_rows/out_rows.  Ordered on stream; returns after the rows are written. */
sgns_status sgns_minibatch_update_bf16(int32_t d, int32_t n_batches, const int32_t* in_count,
                                       const int32_t* in_first, const int32_t* out_count,
                                       const int32_t* out_meta, const float* alpha, const float* in_rows,
                                       const float* out_rows, uint16_t* new_in, uint16_t* new_out,
                                       uint64_t sr_seed, void* stream);

/* sgns_minibatch_update without any device allocation.  No counterpart in the
 * reference: it exists for callers that cannot let a library allocate device memory --
 * a process whose GPU memory belongs to its own allocator (a framework's caching
 * allocator, a serving process that reserves the device up front), where cudaMalloc
 * may fail, fragment the caller's pool, or synchronise the device mid-pipeline.
 * Its scratch (row offsets, a status word, the sigmoid table) is a statically allocated
 * device array of about 1 MiB that every GPU loading the library holds until exit;
 * n is limited to 65536 minibatches (SGNS_EINVAL beyond).  The first call on a device
 * resolves that array's address and fills the sigmoid table, so make it before any
 * stream capture.  Every call copies the kernel's status word back to the host and
 * synchronises `stream` before it returns.  All calls share the array: calls that
 * overlap on the GPU (other streams, other threads) race on it.  Same arguments,
 * results and limits otherwise. */
sgns_status sgns_minibatch_update_noalloc(int32_t d, int32_t n_batches, const int32_t* in_count,
                                          const int32_t* in_first, const int32_t* out_count,
                                          const int32_t* out_meta, const float* alpha,
                                          const float* in_rows, const float* out_rows, float* d_in,
                                          float* d_out, void* stream);

/* Link-prediction scores: scores[i] = <table[pairs[2i]], table[pairs[2i+1]]> for n pairs of
 * row indices into a table of V rows (device pointers; the dot-product scoring of the
 * holdout that src/tools/gtrain.cpp:226-385 writes).  dtype: 0 = fp32 table, 1 = bf16
 * table; fp32 arithmetic in a fixed order (per lane columns 4l..4l+3 of each 128-column
 * chunk by fused multiply-adds, then an xor butterfly over the 32 lanes).  A pair naming a
 * row outside [0, V) scores 0 and makes the call return SGNS_EINVAL.  Ordered on stream;
 * returns after the scores are written. */
sgns_status sgns_link_scores(int32_t dtype, int32_t d, const void* table, int64_t V, const int32_t* pairs,
                             int64_t n, float* scores, void* stream);

/* ---- corpus producer: information-oriented walks ------------------------------------
 * Graphs are undirected CSR in device memory: indptr (V + 1 entries, indptr[0] = 0,
 * indptr[V] = n_edges, non-decreasing) and indices (n_edges neighbour ids, each list
 * strictly increasing; an edge appears in both endpoints' lists).  A malformed graph is
 * SGNS_EINVAL, found by a device check before any kernel follows its pointers. */

/* Common-neighbour count of every edge: cn[e] = |N(u) & N(v)| for edge e = (u, v) -- the
 * edge data the information-oriented walker reads (candidate->data, include/walk.hpp:920),
 * which the reference loads from a precomputed file (include/graph.hpp:826).  cn: device
 * output of n_edges entries.  Ordered on stream; returns when the counts are written. */
sgns_status sgns_edge_common_neighbors(const int64_t* indptr, const int32_t* indices, int64_t V, int64_t n_edges,
                                       int32_t* cn, void* stream);

typedef struct sgns_walk_options {
  int64_t walker_num;  /* -w: walkers; walker k starts at vertex k % V (walk.hpp:503-506) */
  int32_t min_length;  /* --min_L: moves made before the stop test applies (walk.hpp:404, 20) */
  int32_t max_length;  /* vertices per walk at most, 1..1000 (the trainer reads at most 1000,
                          dsgl.hpp:23; the reference walker has no cap) */
  double r_threshold;  /* R of walk.hpp:24 (0.999): a walk stops once R*R < r_threshold or
                          R < 0 (walk.hpp:868-874) */
  uint64_t seed;       /* the walkers' random streams (counter-based; see below) */
  int32_t trace_steps; /* 1: the reference's trace step -- a move to a neighbour with few
                          common neighbours is followed by a return to the current vertex
                          (walk.hpp:920-1031); 0: every move goes on to the drawn neighbour,
                          with the same stop rule */
  int32_t reserved;    /* 0 */
} sgns_walk_options;

/* DistGER's information-oriented walks (InCoM, include/walk.hpp:818-1042: uniform neighbour
 * candidates, the common-neighbour "trace" step that returns to the current vertex, and the
 * stop rule on the correlation of path entropy and length, walk.hpp:260-387) over the
 * graph, one walk per walker, written as corpus tokens: vertex ids with -1 after each walk
 * in walker order (the layout of graph->local_corpus, path.hpp:96,110).  The reference
 * draws from time-seeded generators; here walker k draws from its own SplitMix64 stream of
 * `seed`, so a run is reproducible and equals the CPU restatement bit for bit.  The only
 * rule that differs: a walk whose start vertex has only itself as neighbour ends after 64
 * redraws (the reference redraws forever).  corpus: device output of cap entries;
 * *n_tokens: the entries the walks yield, also set when cap is too small (then
 * SGNS_EINVAL and nothing written; cap = 0 with corpus NULL just counts).  cn: the
 * counts of sgns_edge_common_neighbors.  Uses library scratch memory (12 bytes per walker).
 * Ordered on stream; returns after the corpus is written. */
sgns_status sgns_info_walks(const sgns_walk_options* opt, const int64_t* indptr, const int32_t* indices,
                            const int32_t* cn, int64_t V, int64_t n_edges, int32_t* corpus, int64_t cap,
                            int64_t* n_tokens, void* stream);

/* SGNS loss and its hand-written adjoint for n minibatches that index tables of V
 * rows (device pointers).  Minibatch b has inputs in_ids[in_ptr[b]..in_ptr[b+1]), the
 * first in_first[b] of them labelled by output 0 and the rest by the last output, and
 * outputs out_ids[out_ptr[b]..out_ptr[b+1]) with multiplicities out_meta (the layout of
 * one reference step, dsgl.hpp:1103-1159).  With f_ij = <Woh[o_i], Wih[x_j]>:
 *   *loss = sum meta_i * softplus(-(2*label_ij - 1) * f_ij), reduced in fp64 (device);
 *   grad_in_ids/grad_in: the distinct Wih rows of the batch in ascending order and
 *   dL/dWih for each (n_in x d); grad_out_ids/grad_out likewise for Woh.
 * dtype: 0 = fp32 tables and gradients; 1 = bf16 tables, fp32 arithmetic and gradients;
 * 2 = fp64 tables, arithmetic and gradients.  Id/gradient capacities: in_ptr[n] and
 * out_ptr[n] rows.  n_in/n_out are host pointers; the call returns once they are known.
 * A V-sized scratch is allocated by the library and cached per device. */
sgns_status sgns_loss_adjoint(int32_t dtype, int32_t d, int64_t V, int32_t n_batches,
                              const int32_t* in_ptr, const int32_t* in_ids,
                              const int32_t* in_first, const int32_t* out_ptr,
                              const int32_t* out_ids, const int32_t* out_meta,
                              const void* wih, const void* woh, double* loss,
                              int32_t* grad_in_ids, void* grad_in, int64_t* n_in,
                              int32_t* grad_out_ids, void* grad_out, int64_t* n_out,
                              void* stream);

#ifdef __cplusplus
}
#endif
#endif
