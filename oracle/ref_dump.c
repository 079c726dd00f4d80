/*
 * ref_dump — drives the UNMODIFIED reference through its own public C entry points and writes
 * what the hot path produces as raw little-endian arrays, so that tests can pin the C
 * restatement (oracle/pq_oracle.c) and the CUDA library against it.
 *
 * Test infrastructure only: linked against the reference objects built by oracle/Makefile.
 *
 *   ref_dump READS.fa L T OUTDIR [THREADS [BLOOM_M N_HASHFUNC]]   (Bloom defaults: 36, 2)
 *
 * Calls, in the order the reference's main() makes them (src/test.c:364-370):
 *   construct_index()        src/index.h:63-68   (run single-threaded: the canonical tie order)
 *   construct_string_graph() src/string_graph.h:139 (THREADS threads; its output is
 *                                                    thread-count invariant)
 * and, for the suffix arrays, which the reference builds chunk by chunk and never keeps, the
 * sufsort API exactly as build_idx() drives it (src/index.c:558-585), single-threaded:
 *   transform_to_triplet[_reverse] -> initial_sort -> suf_sort(slot 0..4).
 */
#include <omp.h>
#include <stdint.h>
#include <errno.h>
#include <sys/stat.h>
#include "index.h"
#include "sufsort.h"
#include "string_graph.h"

static void
dump (const char *dir, const char *name, const void *p, size_t bytes)
{
    char path[4096];
    snprintf (path, sizeof path, "%s/%s", dir, name);
    FILE *f = fopen (path, "wb");
    if (!f)
    {
        fprintf (stderr, "ref_dump: cannot write %s\n", path);
        exit (2);
    }
    if (bytes && fwrite (p, 1, bytes, f) != bytes)
    {
        fprintf (stderr, "ref_dump: short write %s\n", path);
        exit (2);
    }
    fclose (f);
}

/* Suffix array of one direction through the reference's own sort (src/index.c:558-585). */
static INDEX_TYPE_T *
reference_sa (const char *reads_fw, INDEX_TYPE_T nr, int L, int t, int dir)
{
    INDEX_TYPE_T n = nr * (INDEX_TYPE_T) L, i;
    /* +16: STNI_strcmp reads 16-byte windows past the end of the text */
    char *text = (char *) calloc (n + 32, 1);
    memcpy (text, reads_fw, n);
    omp_lock_t *lk = (omp_lock_t *) malloc ((nr ? nr : 1) * sizeof (omp_lock_t));
    for (i = 0; i < nr; i++)
        omp_init_lock (&lk[i]);
    INDEX_TYPE_T *is = calloc (nr + 1, sizeof (INDEX_TYPE_T));
    INDEX_TYPE_T *ie = calloc (nr + 1, sizeof (INDEX_TYPE_T));
    u16 *id = calloc (nr + 1, sizeof (u16));
    if (dir == 0)
        transform_to_triplet (text, L, nr);
    else
        transform_to_triplet_reverse (text, L, nr);
    bucket_t b0;
    INDEX_TYPE_T bs[SLOT_DEPTH], bo[SLOT_DEPTH], ms, ni[NUM_SLOTS];
    initial_sort (text, n, &b0, bs, bo, &ms);
    memcpy (ni, b0.offs, sizeof ni);
    INDEX_TYPE_T *sa = (INDEX_TYPE_T *) malloc ((n ? n : 1) * sizeof (INDEX_TYPE_T));
    for (int j = 0; j < SLOT_DEPTH; j++)
        suf_sort (sa + bo[j], text, j, ni, &b0, n, L, is, ie, id, lk, bo[j], t);
    for (i = 0; i < nr; i++)
        omp_destroy_lock (&lk[i]);
    free (lk);
    free (is);
    free (ie);
    free (id);
    free (text);
    return sa;
}

int
main (int argc, char **argv)
{
    if (argc < 5)
    {
        fprintf (stderr, "usage: %s READS.fa L T OUTDIR [THREADS [BLOOM_M N_HASHFUNC]]\n", argv[0]);
        return 2;
    }
    const char *fa = argv[1];
    int L = atoi (argv[2]), t = atoi (argv[3]);
    const char *out = argv[4];
    int threads = argc > 5 ? atoi (argv[5]) : omp_get_max_threads ();
    int bloom_m = argc > 7 ? atoi (argv[6]) : 36, n_hashfunc = argc > 7 ? atoi (argv[7]) : 2;
    mkdir (out, 0755);

    omp_set_num_threads (1);
    index_t *idx = construct_index ((char *) fa, NULL, NULL, NULL, NULL, t, L, bloom_m, n_hashfunc);
    INDEX_TYPE_T nr = idx->num_reads, n = nr * (INDEX_TYPE_T) L;
    INDEX_TYPE_T rowlen = (n + 64) / 64;

    FILE *m;
    char path[4096];
    snprintf (path, sizeof path, "%s/meta.txt", out);
    m = fopen (path, "w");
    fprintf (m, "idx_bytes %d\nnum_reads %llu\nread_len %d\nmin_overlap %d\n",
             (int) sizeof (INDEX_TYPE_T), (unsigned long long) nr, L, t);
    fprintf (m, "C");
    for (int c = 0; c < 6; c++)
        fprintf (m, " %llu", (unsigned long long) idx->C[c]);
    fprintf (m, "\nsuffix_count");
    for (int c = 0; c < 4; c++)
        fprintf (m, " %llu", (unsigned long long) idx->suffix_count[c]);
    fprintf (m, "\nprefix_count");
    for (int c = 0; c < 4; c++)
        fprintf (m, " %llu", (unsigned long long) idx->prefix_count[c]);
    fprintf (m, "\n");
    /* the sort-slot bookkeeping initial_sort leaves in index_t (src/index.c:466-469, 519-522) */
    const INDEX_TYPE_T *slot_f[4] = {idx->size_fw, idx->offset_fw, idx->size_bw, idx->offset_bw};
    const char *slot_n[4] = {"size_fw", "offset_fw", "size_bw", "offset_bw"};
    for (int k = 0; k < 4; k++)
    {
        fprintf (m, "%s", slot_n[k]);
        for (int c = 0; c < 5; c++)
            fprintf (m, " %llu", (unsigned long long) slot_f[k][c]);
        fprintf (m, "\n");
    }
    fprintf (m, "max_size_fw %llu\nmax_size_bw %llu\n", (unsigned long long) idx->max_size_fw,
             (unsigned long long) idx->max_size_bw);

    size_t isz = sizeof (INDEX_TYPE_T);
    dump (out, "reads.bin", idx->reads, n);
    dump (out, "occ_sample_fw.bin", idx->OCC_sample, rowlen * 5 * isz);
    dump (out, "occ_sample_bw.bin", idx->OCC_sample_bw, rowlen * 5 * isz);
    {
        u64 *bm = (u64 *) malloc (rowlen * 5 * 8);
        for (int c = 0; c < 5; c++)
            memcpy (bm + c * rowlen, idx->OCC_bitmap[c], rowlen * 8);
        dump (out, "occ_bitmap_fw.bin", bm, rowlen * 5 * 8);
        for (int c = 0; c < 5; c++)
            memcpy (bm + c * rowlen, idx->OCC_bitmap_bw[c], rowlen * 8);
        dump (out, "occ_bitmap_bw.bin", bm, rowlen * 5 * 8);
        free (bm);
    }
    dump (out, "reads_index_fw.bin", idx->reads_index, nr * isz);
    dump (out, "reads_index_bw.bin", idx->reads_index_bw, nr * isz);
    dump (out, "seed_start_fw.bin", idx->interval_start, nr * isz);
    dump (out, "seed_size_fw.bin", idx->interval_end, nr * isz);
    dump (out, "seed_depth_fw.bin", idx->interval_depth, nr * 2);
    dump (out, "seed_start_bw.bin", idx->interval_start_bw, nr * isz);
    dump (out, "seed_size_bw.bin", idx->interval_end_bw, nr * isz);
    dump (out, "seed_depth_bw.bin", idx->interval_depth_bw, nr * 2);

    for (int dir = 0; dir < 2; dir++)
    {
        INDEX_TYPE_T *sa = reference_sa (idx->reads, nr, L, t, dir);
        dump (out, dir ? "sa_bw.bin" : "sa_fw.bin", sa, n * isz);
        free (sa);
    }

    omp_set_num_threads (threads > 0 ? threads : 1);
    string_graph_t *g = construct_string_graph (idx);

    uint8_t *nodes = (uint8_t *) malloc ((nr ? nr : 1) * 8);
    size_t ne = 0, cap = 1024;
    uint64_t *dest = malloc (cap * 8);
    uint16_t *len = malloc (cap * 2);
    uint8_t *type = malloc (cap);
    int64_t *trans = malloc (cap * 8);
    for (INDEX_TYPE_T i = 0; i < nr; i++)
    {
        node_t *nd = &g->nodes[i];
        memcpy (nodes + i * 8, &nd->num_B, 2);
        memcpy (nodes + i * 8 + 2, &nd->num_F, 2);
        nodes[i * 8 + 4] = (uint8_t) nd->B_type;
        nodes[i * 8 + 5] = (uint8_t) nd->F_type;
        nodes[i * 8 + 6] = (uint8_t) nd->status;
        nodes[i * 8 + 7] = (uint8_t) nd->marked;
        int k = nd->max_B + nd->max_F;
        for (int j = 0; j < k; j++)
        {
            if (ne == cap)
            {
                cap *= 2;
                dest = realloc (dest, cap * 8);
                len = realloc (len, cap * 2);
                type = realloc (type, cap);
                trans = realloc (trans, cap * 8);
            }
            dest[ne] = nd->edges[j].dest;
            len[ne] = nd->edges[j].overlap_len;
            type[ne] = (uint8_t) nd->edges[j].type;
            trans[ne] = nd->path_q ? (int64_t) nd->path_q->path[j].trans : -1;
            ne++;
        }
    }
    dump (out, "nodes.bin", nodes, nr * 8);
    dump (out, "edges_dest.bin", dest, ne * 8);
    dump (out, "edges_len.bin", len, ne * 2);
    dump (out, "edges_type.bin", type, ne);
    dump (out, "edges_trans.bin", trans, ne * 8);
    fprintf (m, "num_edges %zu\n", ne);
    fclose (m);
    return 0;
}
