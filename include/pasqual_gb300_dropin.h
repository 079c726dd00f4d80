/*
 * pasqual_gb300_dropin.h — the reference's own entry points and data structures, served by the
 * GB300 library.  Linking the reference's main() (src/test.c) and assemble() (src/assemble.c)
 * against libpasqual_gb300_uXX.so instead of the reference's index.o/sufsort.o/string_graph.o
 * runs suffix sort, FM-index build and overlap search on the GPU and leaves everything else
 * (CLI, graph simplification, contigs.fa writer) unchanged.
 *
 * Every structure below has the reference's field order and types so that code compiled
 * against the reference's headers (src/index.h, src/string_graph.h) reads it unchanged; the
 * library's tests compare sizeof/offsetof of each field with the reference headers.  The one
 * field whose type differs is index_t.read_lock (an omp_lock_t pointer in the reference, always
 * NULL here): both are one pointer wide.
 *
 * Index width: define PQ_IDX64 (or __INDEX_U64__, the reference's macro) for the 64-bit build
 * (libpasqual_gb300_u64.so), as src/common.h:31-44 selects INDEX_TYPE_T.
 */
#ifndef PASQUAL_GB300_DROPIN_H
#define PASQUAL_GB300_DROPIN_H

#include <stdint.h>
#include "pasqual_gb300.h"

#ifdef __cplusplus
extern "C" {
#endif

#if defined(PQ_IDX64) || defined(__INDEX_U64__)
typedef uint64_t pq_index_type;
#else
typedef uint32_t pq_index_type;
#endif

/* index_t (src/index.h:15-57) */
typedef struct pq_index_t
{
    unsigned char *bloom_array;
    pq_index_type bloom_size;
    int n_hashfunc;
    pq_index_type C[6];
    pq_index_type suffix_count[4];
    pq_index_type prefix_count[4];
    uint64_t *OCC_bitmap[5];
    uint64_t *OCC_bitmap_bw[5];
    pq_index_type *OCC_sample;
    pq_index_type *OCC_sample_bw;
    pq_index_type *reads_index;
    pq_index_type *reads_index_bw;
    pq_index_type *interval_start;
    pq_index_type *interval_end;
    uint16_t *interval_depth;
    pq_index_type *interval_start_bw;
    pq_index_type *interval_end_bw;
    uint16_t *interval_depth_bw;
    void *read_lock;
    char *reads;
    uint16_t read_len;
    pq_index_type num_reads;
    uint16_t min_overlap;
    pq_index_type size_bw[5];
    pq_index_type offset_bw[5];
    pq_index_type size_fw[5];
    pq_index_type offset_fw[5];
    pq_index_type max_size_fw;
    pq_index_type max_size_bw;
} pq_index_t;

/* path_t, path_q_t, edge_t, node_t, string_graph_t (src/string_graph.h:57-114) */
typedef struct pq_path_t
{
    pq_index_type end;
    pq_index_type hop;
    uint16_t len;
    uint16_t end_len;
    uint16_t bubble_len;
    int trans;
    char updated;
    char direction;
    char type;
} pq_path_t;

typedef struct pq_path_q_t
{
    pq_path_t *path;
    uint16_t max_F_endlen;
    uint16_t max_B_endlen;
    uint16_t max_B_len;
    uint16_t max_F_len;
    int max_F_trans;
    int max_B_trans;
} pq_path_q_t;

typedef struct pq_edge_t
{
    pq_index_type dest;
    uint16_t overlap_len;
    char type;
} pq_edge_t;

typedef struct pq_node_t
{
    pq_edge_t *edges;
    pq_path_q_t *path_q;
    uint16_t num_F;
    uint16_t num_B;
    uint16_t max_F;
    uint16_t max_B;
    char B_type;
    char F_type;
    char status;
    char marked;
} pq_node_t;

typedef struct pq_string_graph_t
{
    uint16_t read_len;
    uint16_t min_overlap;
    double average_overlap;
    pq_index_type num_reads;
    pq_node_t *nodes;
} pq_string_graph_t;

/* bucket_t (src/sufsort.h:17-23): per first-prefix rank (NUM_SLOTS = 85, src/common.h:50) the
 * number of suffixes and their offset inside the rank's slot. */
#define PQ_NUM_SLOTS 85
typedef struct pq_bucket_t
{
    pq_index_type freqs[PQ_NUM_SLOTS];
    pq_index_type offs[PQ_NUM_SLOTS];
} pq_bucket_t;

/* src/sufsort.h:32.  Recodes every read in place: byte j becomes the rank (0..84) of the read's bases
 * j .. min(j + 2, L - 1) in the order of strings of up to 3 bases with a string before its
 * extensions -- the reference's triplet code (src/sufsort.c:124-151), on every host core. */
PQ_API void transform_to_triplet (char *reads, int read_len, pq_index_type num_reads);
/* src/sufsort.h:35-36.  The same for every read reversed (src/sufsort.c:80-121). */
PQ_API void transform_to_triplet_reverse (char *reads, int read_len, pq_index_type num_reads);
/* src/sufsort.h:38-40.  Histogram of the recoded text's first-prefix ranks into bkt (frequencies,
 * offsets restarting in each of the 5 slots of 17 ranks), slot sizes bsize[5], slot offsets
 * boffset[5] and the largest slot *max_size (src/sufsort.c:386-450), on every host core. */
PQ_API void initial_sort (char *reads, pq_index_type num_elems, pq_bucket_t * bkt, pq_index_type * bsize,
                          pq_index_type * boffset, pq_index_type * max_size);
/* src/sufsort.h:42-46.  Slot `slot` of the suffix array of the recoded text: writes its bsize[slot]
 * rows (text positions, canonical order: suffix string with end-of-read lowest, then position) to
 * sa[0 ..), advances new_idx over the slot's ranks as the reference's scatter does, and deepens
 * interval_start / interval_end (the interval's size) / interval_depth with the seed records of the
 * slot's sort buckets (src/sufsort.c:178-209, 322-334).  The sort runs on the GPU (device 0): the
 * whole text is sorted on the first call and kept until a call brings another text (compared by
 * address, size, read length, min overlap and a checksum of its bytes), so the five slot calls of
 * one text sort once; the device memory stays held until the process exits or the next text.
 * read_lock is ignored (the reference's OpenMP locks).  Errors print a message on stderr and exit
 * with status 0, the reference's ERROR_EXIT convention. */
PQ_API void suf_sort (pq_index_type * sa, char *reads, int slot, pq_index_type * new_idx, pq_bucket_t * bkt0,
                      pq_index_type num_elems, int read_len, pq_index_type * interval_start,
                      pq_index_type * interval_end, uint16_t * interval_depth, void *read_lock,
                      pq_index_type bkt_offset, int min_overlap);

/* src/index.h:63-68.  Reads the FASTA (import_singlereads + bloom_filter, src/index.c:145-405,
 * src/bloom.c:91-135, restated on the host), then sorts both texts and builds both FM-indexes on
 * the GPU and fills every host field of index_t in the reference's layout.  Paired-end and
 * mate-pair files are rejected with the reference's messages.  On error: the reference's
 * ERROR_EXIT behaviour (message on stderr, exit status 0). */
PQ_API pq_index_t *construct_index (char *single_file, char *pair_file1, char *pair_file2,
                                    char *mate_file1, char *mate_file2, int min_overlap,
                                    int read_len, int bloom_m, int n_hashfunc);

/* src/string_graph.h:139.  Overlap search with transitive reduction on the GPU (using the
 * device-resident index of the construct_index call that produced `index`, or rebuilding it
 * from index->reads), then node_t construction as src/string_graph.c:832-1017. */
PQ_API pq_string_graph_t *construct_string_graph (pq_index_t * index);

/* Node construction only (src/string_graph.c:832-1017), the second half of
 * construct_string_graph: the reference's string_graph_t built from a graph in the CSR form that
 * pq_get_graph returns (per read num_B, num_F, olp_B, olp_F and edge_off[num_reads + 1]; per
 * edge dest, len, type and trans).  The nodes are built on `threads` host threads (0 = one per
 * core), as the reference builds them inside its parallel search loop; the result does not depend
 * on the thread count.  path_q->max_F_trans / max_B_trans hold the running maximum of the trans
 * values in read order (the reference's value with one thread).  average_overlap is the mean
 * edge overlap length (NaN for a graph without edges, as in the reference).  Every node, edge
 * list and path queue is malloc'd as the reference's are.  Returns NULL (nothing left allocated)
 * when memory runs out, when read_len is outside (0, 65535], or when an array the graph needs is
 * NULL (the per-edge arrays may be NULL for a graph without edges). */
PQ_API pq_string_graph_t *pq_string_graph_from_csr (pq_index_type num_reads, int read_len,
                                                    int min_overlap, const uint16_t * num_B,
                                                    const uint16_t * num_F, const int32_t * olp_B,
                                                    const int32_t * olp_F, const uint64_t * edge_off,
                                                    const pq_index_type * dest, const uint16_t * len,
                                                    const uint8_t * type, const int32_t * trans,
                                                    int threads);

/* src/string_graph.h:142 — the reference's destroy_graph is empty; so is this one. */
PQ_API void destroy_graph (pq_string_graph_t * graph);

/* Import only: the reads construct_index keeps (num_reads * read_len codes 1..4, malloc'd,
 * caller frees) and the number removed as duplicates.  Returns PQ_OK or PQ_ERR_ARG with the
 * reference's message in *err (static storage): the CLI's argument checks (read_len in
 * (0, 65535], n_hashfunc in [1, 5], bloom_m >= 1; src/test.c:300-320), then the import's own. */
PQ_API int pq_import_fasta (const char *path, int read_len, int bloom_m, int n_hashfunc,
                            uint8_t ** reads_out, pq_index_type * num_reads_out,
                            pq_index_type * removed_out, const char **err);

#ifdef __cplusplus
}
#endif

#endif
