/*
 * pasqual_gb300.h — C ABI of the GB300 (sm_103a) build of PASQUAL's hot path.
 *
 * Two layers, both plain C (pointers and sizes only):
 *
 *  1. pq_* — device-resident entry points.  Each one replaces one step of the reference's
 *     construct_index()/construct_string_graph() and says which (file:line in the reference).
 *     Host buffers are copied in and out; everything in between stays in GPU memory.
 *
 *  2. The reference's own entry points with the reference's own signatures and struct layouts
 *     (construct_index, construct_string_graph, destroy_graph; src/index.h:63-68,
 *     src/string_graph.h:139-142), exported by the same library so that the reference's main()
 *     (src/test.c) and assemble() (src/assemble.c) link against it unchanged.  Those are declared
 *     in pasqual_gb300_dropin.h.
 *
 * The library is built twice, like the reference (-D__INDEX_U32__ / -D__INDEX_U64__,
 * src/common.h:31-44): libpasqual_gb300_u32.so (pq_idx = uint32_t) and
 * libpasqual_gb300_u64.so (pq_idx = uint64_t, define PQ_IDX64 before including this header).
 *
 * Errors: every int-returning function returns PQ_OK (0) or a PQ_ERR_* code and keeps a message
 * for pq_last_error().  Nothing calls exit(); the drop-in layer maps errors to the reference's
 * ERROR_EXIT behaviour (message on stderr, exit status 0, src/common.h:87-94).
 *
 * Threading: a context is used from one host thread at a time; all its work is ordered on the
 * CUDA stream given to pq_create (its own stream when NULL).
 */
#ifndef PASQUAL_GB300_H
#define PASQUAL_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#ifdef PQ_IDX64
typedef uint64_t pq_idx;
#else
typedef uint32_t pq_idx;
#endif

#define PQ_OK 0
#define PQ_ERR_ARG 1
#define PQ_ERR_CUDA 2
#define PQ_ERR_NOMEM 3
#define PQ_ERR_TOO_MANY_EDGES 4 /* a read has > 65535 edges on one side (src/string_graph.c:469-472) */
#define PQ_ERR_STATE 5          /* a step was called before the one it depends on */
#define PQ_ERR_CAPACITY 6       /* a read's interval table outgrew (2L)^2 (src/string_graph.c:542) */
#define PQ_ERR_INTERNAL 7

#if defined(__GNUC__)
#define PQ_API __attribute__ ((visibility ("default")))
#else
#define PQ_API
#endif

typedef struct pq_ctx pq_ctx;

/* Width of pq_idx in bytes (4 or 8): lets a loader check it bound the right build. */
PQ_API int pq_idx_bytes (void);

/* Create a context on CUDA device `device`; `cuda_stream` is a cudaStream_t or NULL. */
PQ_API int pq_create (pq_ctx ** out, int device, void *cuda_stream);
PQ_API void pq_destroy (pq_ctx * ctx);
PQ_API const char *pq_last_error (const pq_ctx * ctx);

/* Page-locked host memory (cudaHostAlloc) for the buffers that cross to and from the device:
 * reads in (pq_set_reads) and graphs out (pq_get_graph).  Both calls copy page-locked buffers with
 * a copy kernel that reads or writes them directly, many accesses in flight: that keeps the
 * link's rate (about 210 GB/s on GB300) right after a suffix sort or a search, where copy-engine
 * copies (cudaMemcpy) from such memory were measured at 10-17 GB/s, and from cudaHostRegister'ed
 * small-page memory at 2-35 GB/s even by kernel.  Allocate these buffers once, before the loop that
 * reuses them.  pq_host_free releases a buffer from pq_host_alloc (PQ_ERR_ARG for any other
 * pointer).  PQ_ERR_NOMEM when the memory cannot be allocated, PQ_ERR_CUDA when there is no usable
 * device. */
PQ_API int pq_host_alloc (size_t bytes, void **out);
PQ_API int pq_host_free (void *p);

/* Reads after import and de-duplication: num_reads * read_len base codes 1..4 (A,C,G,T), the
 * layout of index_t.reads after import_singlereads (src/index.c:145-405).  min_overlap is the
 * -t of the CLI, with SEQ_DEPTH(9) < min_overlap < read_len (src/test.c:306-311).
 * from_device != 0: `reads` is a device pointer.  PQ_ERR_ARG if any byte is not a base code
 * (the reference's import drops reads with N and rejects other symbols, src/index.c:304-318);
 * the context then holds no reads.  Page-locked host reads (cudaHostAlloc, pq_host_alloc,
 * cudaHostRegister) are copied by a kernel that reads them directly; pageable ones by cudaMemcpy. */
PQ_API int pq_set_reads (pq_ctx * ctx, const uint8_t * reads, pq_idx num_reads, int read_len,
                  int min_overlap, int from_device);

/* C[6], suffix_count[4], prefix_count[4] of index_t (src/index.c:336-346, 367-372). */
PQ_API int pq_get_counts (pq_ctx * ctx, pq_idx C[6], pq_idx suffix_count[4], pq_idx prefix_count[4]);

/* Suffix array of direction dir (0: the reads; 1: every read reversed), in the order the
 * reference's sufsort produces single-threaded: read-bounded suffixes, end-of-read lowest, ties
 * by text position.  Replaces transform_to_triplet[_reverse] + initial_sort + suf_sort over the
 * five slots (src/sufsort.h:29-46, driven by src/index.c:558-585). */
PQ_API int pq_sort (pq_ctx * ctx, int dir);
/* Largest number of suffixes pq_sort sorts in one pass (0, the default: 2^31 - 1, the limit of its
 * 32-bit group ranks).  Larger indexes are sorted in chunks: every suffix falls in a bucket by its
 * first 6 bases and min(length, 6), numbered in suffix order, and runs of consecutive buckets of
 * at most this many suffixes are sorted one after the other into their place -- the sort the
 * reference does over its 5 first-character slots (src/index.c:558-585), at a finer grain.  A
 * bucket larger than a chunk makes pq_sort return PQ_ERR_CAPACITY.  Same suffix array either way. */
PQ_API int pq_set_sort_chunk (pq_ctx * ctx, uint64_t max_suffixes);

/* Use a given suffix array instead of sorting (testing and external sorters). */
PQ_API int pq_set_sa (pq_ctx * ctx, int dir, const pq_idx * sa, int from_device);
PQ_API int pq_get_sa (pq_ctx * ctx, int dir, pq_idx * sa_host);

/* FM-index of direction dir from its suffix array: BWT, occurrence blocks, reads_index and the
 * k-mer seed table.  Replaces build_OCC + the occ prefix sum (src/index.c:26-142, 587-615). */
PQ_API int pq_build_fm (pq_ctx * ctx, int dir);

/* Both directions, sort + FM-index: the body of build_index (src/index.c:626-706).  The sort's
 * working memory (about 25 bytes per suffix) is kept for the next build of the same size unless
 * less than a quarter of the device memory is free afterwards. */
PQ_API int pq_build_index (pq_ctx * ctx);

/* Reference-layout copies of an FM-index (index_t.OCC_bitmap[5] back to back, each
 * (n+64)/64 words; OCC_sample (n+64)/64*5 entries; reads_index num_reads entries). */
PQ_API int pq_get_index_ref (pq_ctx * ctx, int dir, uint64_t * bitmap, pq_idx * sample,
                      pq_idx * reads_index);

/* Per-read seed intervals written into index_t.interval_start/end/depth (src/index.h:36-41):
 * the exact SA interval of the read's last (dir 0) / first, reversed (dir 1) k bases. */
PQ_API int pq_get_seeds (pq_ctx * ctx, int dir, pq_idx * start, pq_idx * size, uint16_t * depth);

/* The seed intervals the reference's sort records for every read (index_t.interval_start,
 * interval_end = the interval's size, interval_depth; src/sufsort.c:178-209, 322-334, starting from
 * the depth-1 seeds of src/index.c:495-502): the deepest depth D in 9, 12, ..., t at which the
 * reference's recursive bucket sort visits the bucket of the read's last (dir 0) / first, reversed
 * (dir 1) D bases, with that bucket's first row and size; depth 1 and the interval of that one base
 * by C[] when there is none.  Computed on the GPU from direction dir's suffix array (pq_sort or
 * pq_build_index first); field for field the reference's arrays. */
PQ_API int pq_get_sort_seeds (pq_ctx * ctx, int dir, pq_idx * start, pq_idx * size, uint16_t * depth);

/* Seed depth k of the overlap search (1 <= k <= min(14, t)): the k-mer table of 4^k entries per
 * index that seeds the walks and narrows the interval scans.  Default, per read set: 14 from 2^32
 * suffixes per index, 13 from 2^30, else 12, never above t; a value set here is kept for later
 * read sets. */
PQ_API int pq_set_seed_k (pq_ctx * ctx, int k);

/* How the candidates of each read are found.  0 walks from the depth-k seed to depth L with one
 * synchronised backward-search step per base, as the reference does from its sort-recorded seed
 * (src/string_graph.c:207-237).  1 (default) finds the depth-t interval of the walked index by
 * binary search over its suffix array inside the k-mer table interval of the pattern's first k
 * bases, reads that interval's rows once (a read r' whose suffix at offset o matches, and whose
 * first o bases continue the pattern, is a candidate at depth t + o) and takes the other index's
 * interval from the inverse suffix array.  2 is mode 1 with the learned index's window in place
 * of the k-mer table's (t >= 16).  Modes 1 and 2 apply when L - t <= 256 and
 * 4^min(t, 64) > 64 * num_reads * read_len (depth-t intervals are small; beyond 64 bases the
 * pattern is checked row by row); a read whose depth-t interval exceeds 256 rows walks.  All
 * modes give the reference's candidates.  Modes 1 and 2 also reduce each (read, side) with at
 * most 64 candidates, when L - t <= 256, from the candidates' continuations (the bases after the
 * overlap, read from the packed text) instead of the FM-index DFS of extract_*_edges: an edge is
 * emitted exactly when no other candidate's continuation is a proper prefix of its own, ordered
 * as the DFS visits them.  Mode 0 runs the reference's method throughout. */
PQ_API int pq_set_seed_mode (pq_ctx * ctx, int mode);

/* Overlap search with transitive reduction for every read: find_intervals +
 * extract_bw_edges + extract_fw_edges (src/string_graph.c:163-731) as driven by
 * construct_string_graph (src/string_graph.c:800-830). */
PQ_API int pq_overlaps (pq_ctx * ctx);

/* Sizes of the last pq_overlaps result.  probes = rank probes issued (one 32-byte sector
 * each); wide_reads = reads that needed the wide-scratch kernel. */
PQ_API int pq_get_graph_sizes (pq_ctx * ctx, uint64_t * num_edges, uint64_t * probes,
                        uint64_t * wide_reads);

/* Memory traffic of the last pq_overlaps, as the method in use defines it: load_sectors = the
 * 32-byte sectors of index data its kernels loaded (occurrence blocks, k-mer table, suffix-array
 * and inverse-SA entries, packed-text words, reads_index entries, read bytes; every load counted
 * where it is issued, so a sector loaded twice counts twice; tables that stay in L2 -- superblock
 * counts, learned models -- and the kernels' own scratch are not counted); store_bytes = the
 * bytes of per-read results and edges the search kernels write.  32 * load_sectors + store_bytes
 * is the search's algorithmic traffic. */
PQ_API int pq_get_search_traffic (pq_ctx * ctx, uint64_t * load_sectors, uint64_t * store_bytes);

/* Copy the last pq_overlaps result to host arrays.  Per read: num_B, num_F (node_t.num_B/F),
 * olp_B, olp_F (overlaps_B/F of src/string_graph.c:807-808), edge_off[num_reads+1].  Per edge,
 * B edges then F edges of each read in the reference's DFS order: dest, overlap length, type
 * (BF=0 FB=1 FF=2 BB=3) and the path_t.trans value (src/string_graph.c:940, 970).  Any pointer
 * may be NULL (that array is skipped).  Page-locked host arrays (pq_host_alloc, cudaHostAlloc) are
 * written by a copy kernel at link speed; freshly allocated pageable ones pay their first-touch
 * page faults inside this call. */
PQ_API int pq_get_graph (pq_ctx * ctx, uint16_t * num_B, uint16_t * num_F, int32_t * olp_B,
                  int32_t * olp_F, uint64_t * edge_off, pq_idx * dest, uint16_t * len,
                  uint8_t * type, int32_t * trans);

/* Time (ms, CUDA events on the context stream) of the last pq_sort/pq_build_fm/pq_overlaps. */
PQ_API int pq_get_stage_ms (pq_ctx * ctx, float *sort_ms, float *fm_ms, float *search_ms);

/* Largest num_reads * read_len that pq_suffix_sort_static accepts. */
#define PQ_STATIC_SORT_MAX_SUFFIXES (1u << 20)

/* No counterpart in the reference.  The suffix sort of pq_sort (same canonical order, same
 * kernels) for callers that cannot allocate device memory -- for example a host application that
 * owns all device memory through its own pool and forbids cudaMalloc, or a latency-critical path
 * that cannot take cudaMalloc's implicit device-wide synchronisation.  It calls no cudaMalloc,
 * cudaFree or other allocating routine: the caller passes device pointers to the reads
 * (num_reads * read_len codes 1..4) and to the output suffix array (num_reads * read_len
 * entries), and the working memory is a fixed array inside this library (about 28 MB for the
 * 32-bit build, 32 MB for the 64-bit one) that every GPU which loads the library keeps until the
 * process exits.  Sizes above PQ_STATIC_SORT_MAX_SUFFIXES return PQ_ERR_CAPACITY without doing
 * any work.  The first call on each device looks up the array's device address (once, with that
 * device current); make that first call before any stream capture.  All calls share the array:
 * calls that overlap on the GPU (other streams, other host threads) race and must be ordered by
 * the caller.  Work runs on `cuda_stream` (a cudaStream_t, NULL = the default stream) and the
 * call synchronises that stream before it returns, so the suffix array is complete on return and
 * a kernel failure comes back as PQ_ERR_CUDA.  A read byte outside the codes 1..4 returns
 * PQ_ERR_ARG before any sorting.  Returns PQ_OK, PQ_ERR_ARG, PQ_ERR_CAPACITY or PQ_ERR_CUDA. */
PQ_API int pq_suffix_sort_static (const uint8_t * reads_dev, pq_idx num_reads, int read_len,
                                  int dir, pq_idx * sa_dev, void *cuda_stream);

/* ---- Learned index (no counterpart in the reference) ---------------------------------------
 *
 * A model of each suffix array, trained on the GPU right after the index is built: the first 16
 * bases of a row's suffix, 2 bits a base (bases past the end of the read = A), form a 32-bit key
 * that never decreases down the suffix array.  The distinct keys are cut into up to 1024 segments
 * of equal key count; a piecewise-linear root maps a key onto its segment's rows and a per-segment
 * 2-layer MLP (1 -> 64 ReLU -> 1, FP32) corrects it.  After training, every key present is
 * predicted once and each segment stores the two int32 bounds e_lo, e_hi such that the key's
 * whole row group lies in [pred - e_lo, pred + e_hi).  Seed mode 2 (pq_set_seed_mode) replaces
 * the k-mer table window of mode 1 by that window: one inference per search, a bounded binary
 * search inside it, a check of the two rows just outside it, and the plain backward search of
 * mode 0 whenever the check fails. */
typedef struct pq_learned_info {
    uint64_t num_keys;          /* distinct keys in the suffix array */
    int32_t segments;           /* root segments */
    int32_t hidden;             /* hidden units of each segment's MLP (64) */
    int32_t steps;              /* Adam steps of the training */
    float keys_ms;              /* key extraction and distinct-key pass */
    float train_ms;             /* training kernel */
    float eval_ms;              /* error pass over every key */
    double mean_window;         /* mean over keys of their segment's e_lo + e_hi, trained model */
    double mean_window_root;    /* the same for the root alone (untrained network) */
    int64_t max_window;         /* largest e_lo + e_hi over segments, trained model */
    int64_t max_window_root;
    uint64_t queries;           /* window inferences of the last pq_overlaps in seed mode 2 */
    uint64_t misses;            /* of those, windows whose check failed (searches that walked) */
} pq_learned_info;

/* Build (or rebuild) direction dir's learned index with `steps` training steps (0 = the root
 * alone: the MLP outputs 0).  Needs pq_build_fm(dir).  Seed mode 2 builds missing models itself
 * with 400 steps. */
PQ_API int pq_learned_build (pq_ctx * ctx, int dir, int steps);
PQ_API int pq_learned_get_info (pq_ctx * ctx, int dir, pq_learned_info * info);
/* Copy the model out: bnd[segments], base[segments + 1], params[segments * 196] (w1[64] b1[64]
 * w2[64] b2, padded), err[2 * segments] and err_root[2 * segments] (e_lo, e_hi of each segment). */
PQ_API int pq_learned_export (pq_ctx * ctx, int dir, uint32_t * bnd, pq_idx * base, float *params,
                              int32_t * err, int32_t * err_root);
/* Predicted row (and segment) of n keys, with the search's own function; host arrays. */
PQ_API int pq_learned_predict (pq_ctx * ctx, int dir, const uint32_t * keys, uint64_t n, int64_t * pred,
                               int32_t * seg);
/* The distinct keys of direction dir's suffix array and the first row of each (up to cap of
 * them); *num_keys = their number. */
PQ_API int pq_learned_keys (pq_ctx * ctx, int dir, uint32_t * keys, pq_idx * first_row, uint64_t cap,
                            uint64_t * num_keys);
/* The network of one segment on its own, on the current CUDA device (host arrays; params is one
 * 196-float record): y[i] = mlp(x[i]), and grad[193] = d/d(w1, b1, w2, b2) of sum_i dy[i] * mlp(x[i]).
 * These are the kernels the training runs. */
PQ_API int pq_mlp_forward (const float *params, const float *x, int n, float *y);
PQ_API int pq_mlp_backward (const float *params, const float *x, const float *dy, int n, float *grad);
/* One step of the training's joint phase on one network (host arrays): the gradient of the mean
 * squared error sum_i (mlp(x[i]) - target[i])^2 / n, then Adam (beta1 0.9, beta2 0.999, eps 1e-8,
 * learning rate lr, bias correction for step number `step` >= 1) on all 193 parameters; params (one
 * 196-float record) and the moment estimates m1, m2 (193 each) are updated in place. */
PQ_API int pq_mlp_adam_step (float *params, float *m1, float *m2, const float *x, const float *target, int n,
                             int step, float lr);

/* ---- Queued search over several read sets (no counterpart in the reference) ----------------
 *
 * Each context holds one read set with its own read length L, min overlap t and index pair (the
 * reference handles one fixed-length read set per run; here several such runs share one launch).
 * pq_overlaps_batched searches all of them with ONE persistent kernel: warps take work items
 * (a batch and a group of 32 reads) from a device queue until it is empty, loading each batch's
 * index pair, L and t when they change; every context then holds the same result pq_overlaps
 * would give it.  With PQ_BATCH_GRAPH the queue reset and the kernel are captured once into a
 * CUDA graph (re-captured when a buffer moved or the launch shape changed) and replayed.  Work is
 * ordered on ctxs[0]'s stream; all contexts must be on one device, each appearing once. */
#define PQ_BATCH_GRAPH 1
PQ_API int pq_overlaps_batched (pq_ctx ** ctxs, int count, int flags);
/* Launch plan of queued searches led by `lead`: CTAs (4 warps each) per SM (0 = as many as fit),
 * groups of 32 reads per work item, and edge slots per read in the fast kernel's scratch (reads
 * with more edges go to the wide kernel). */
PQ_API int pq_set_batch_plan (pq_ctx * lead, int ctas_per_sm, int groups_per_item, int edge_slots);
PQ_API int pq_get_batch_stats (pq_ctx * lead, float *kernel_ms, int *ctas_per_sm, int *groups_per_item,
                               int *edge_slots, int *graph_used);
/* Time every plan (CTAs per SM from 2 to the occupancy limit, 1/2/4 groups per item, 32/64 edge
 * slots) on this batch set with pq_overlaps_batched(flags), keep the fastest kernel time as the
 * lead's plan; *best_ms = its time.  The contexts hold the last run's (identical) results. */
PQ_API int pq_autotune_batched (pq_ctx ** ctxs, int count, int flags, float *best_ms);

/* How the last pq_overlaps divided its reads among its tiers: reads[0] = reads the lean tier (one
 * thread a read, interval scan) handed to the fast tier (warp-level walk and DFS), reads[1] = reads
 * the block tier (one CTA a read, all-pairs reduction in shared memory) finished of those the fast
 * tier handed over, reads[2] = reads the heavy tier (the fast tier's DFS with larger capacities)
 * took, reads[3] = reads the wide tier (the reference's own bounds) took; ms[0] = the lean and
 * fast kernels (CUDA events), ms[1..3] = the block, heavy and wide tiers (host time, their
 * synchronisations included).  Either pointer may be NULL. */
PQ_API int pq_get_tier_stats (pq_ctx * ctx, uint64_t reads[4], float ms[4]);

/* Duration (ms, CUDA events on the context stream) of the fast search kernel in the last
 * pq_overlaps, and the number of kernels this library has launched since it was loaded. */
PQ_API int pq_get_kernel_stats (pq_ctx * ctx, float *search_kernel_ms,
                                unsigned long long *launches);

#ifdef __cplusplus
}
#endif

#endif
