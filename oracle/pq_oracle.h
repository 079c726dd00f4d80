/*
 * pq_oracle — CPU restatement of PASQUAL's hot path: test infrastructure, the oracle of tests/ and
 * __graft_entry__.smoke() and the timed CPU baseline of bench.py.  It is never linked into, called
 * by, or substituted for the CUDA library (pasqual_gb300/), which fails loudly instead.
 *
 * Parity of this restatement is pinned against the unmodified reference (oracle/ref_dump.c,
 * built from the reference's own sources by oracle/Makefile) in tests/test_oracle_vs_ref.py,
 * and by the committed fixtures under tests/golden/.
 *
 * Index width follows the reference's INDEX_LENGTH split (src/common.h:31-44): this file is
 * compiled twice, with and without -DPQ_IDX64.
 */
#ifndef PQ_ORACLE_H
#define PQ_ORACLE_H

#include <stdint.h>
#include <stddef.h>

#ifdef PQ_IDX64
typedef uint64_t pqo_idx;
#else
typedef uint32_t pqo_idx;
#endif

#define PQO_OK 0
#define PQO_ERR_ARG 1
#define PQO_ERR_NOMEM 2
#define PQO_ERR_TOO_MANY_EDGES 3  /* src/string_graph.c:469-472, 643-646 */
#define PQO_ERR_CAPACITY 4        /* an interval table outgrew (2L)^2 (src/string_graph.c:542) */

/* Everything the overlap search reads.  Arrays are in the reference's own layout
 * (src/index.h:15-57): bitmap[d] holds the 5 per-symbol bitmaps back to back, each
 * (n+64)/64 words; sample[d] holds 5 counts per 64-row block; d = 0 forward, 1 backward. */
typedef struct pqo_index
{
    const uint8_t *reads;       /* num_reads * read_len codes 1..4, forward orientation */
    pqo_idx num_reads;
    int read_len;
    int min_overlap;
    pqo_idx C[6];
    const uint64_t *bitmap[2];
    const pqo_idx *sample[2];
    const pqo_idx *reads_index[2];
    /* per-read seed intervals (start row, size, depth) for the F-B search on the forward index
     * and the B-F search on the backward index; NULL = start at depth 1 from C[] as
     * src/index.c:495-502 / 548-555 initialise them. */
    const pqo_idx *seed_start[2];
    const pqo_idx *seed_size[2];
    const uint16_t *seed_depth[2];
} pqo_index;

/* Per-read output of the overlap search, edges in the reference's node order: B edges
 * (extract_bw_edges) then F edges (extract_fw_edges), each in DFS emission order. */
typedef struct pqo_graph
{
    pqo_idx first;              /* first read processed */
    pqo_idx count;              /* reads processed */
    uint16_t *num_B;            /* [count] */
    uint16_t *num_F;            /* [count] */
    int32_t *olp_B;             /* [count] sum of $-counts of B candidates (overlaps_B) */
    int32_t *olp_F;             /* [count] */
    uint64_t *edge_off;         /* [count+1] */
    pqo_idx *edge_dest;         /* [num_edges] */
    uint16_t *edge_len;
    uint8_t *edge_type;         /* BF=0 FB=1 FF=2 BB=3 (src/string_graph.h:14-18) */
    int32_t *edge_trans;        /* the path_t.trans value the reference stores */
    uint64_t num_edges;
    uint64_t probes;            /* rank probes: one OCC lookup = one probe */
    int status;
    pqo_idx failed_read;
} pqo_graph;

int pqo_idx_bytes (void);

/* C[] (src/index.c:367-372), suffix_count/prefix_count (src/index.c:336-346) */
void pqo_counts (const uint8_t *reads, pqo_idx num_reads, int read_len,
                 pqo_idx C[6], pqo_idx suffix_count[4], pqo_idx prefix_count[4]);

/* Canonical suffix array of direction dir (0 = reads, 1 = reads reversed): read-bounded
 * suffixes in lexicographic order with end-of-read lowest, ties by text position -- the order
 * the reference's sufsort produces single-threaded (src/sufsort.c:386-614). */
int pqo_sort (const uint8_t *reads, pqo_idx num_reads, int read_len, int dir, pqo_idx *sa,
              int threads);

/* BWT + occurrence tables in the reference layout from a suffix array
 * (build_OCC src/index.c:26-142 and the prefix sum src/index.c:587-615).
 * fix = suffix_count (dir 0) or prefix_count (dir 1). */
int pqo_build_occ (const uint8_t *reads, pqo_idx num_reads, int read_len, int dir,
                   const pqo_idx *sa, const pqo_idx fix[4], uint64_t *bitmap, pqo_idx *sample,
                   pqo_idx *reads_index);

/* Exact SA interval of every k-mer (k <= 13): start row and size, indexed by the k-mer's 2-bit
 * code (first character most significant, A=0..T=3). */
int pqo_kmer_table (const uint8_t *reads, pqo_idx num_reads, int read_len, int dir,
                    const pqo_idx *sa, int k, pqo_idx *start, pqo_idx *size);

/* Per-read seeds at depth k from k-mer tables: forward = the read's last k bases, backward =
 * its first k bases reversed.  Any exact SA interval is a valid seed. */
int pqo_seeds_from_kmers (const uint8_t *reads, pqo_idx num_reads, int read_len, int k,
                          const pqo_idx *kstart, const pqo_idx *ksize, int dir,
                          pqo_idx *seed_start, pqo_idx *seed_size, uint16_t *seed_depth);

/* find_intervals + extract_bw_edges + extract_fw_edges for reads [first, first+count)
 * (src/string_graph.c:163-731, driven as src/string_graph.c:800-830). */
int pqo_overlaps (const pqo_index *ix, pqo_idx first, pqo_idx count, int threads,
                  pqo_graph *out);

void pqo_graph_free (pqo_graph *g);

#endif
