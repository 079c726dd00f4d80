/*
 * pq_oracle.c — CPU restatement of PASQUAL's hot path (TEST INFRASTRUCTURE, see pq_oracle.h).
 *
 * Each function names the reference code it restates.  The restatement keeps the reference's
 * arithmetic exactly (unsigned INDEX_TYPE_T wrap-around included) because the edge lists it
 * produces must equal the reference's bit for bit; where the reference has a latent quirk that
 * changes no output (a `tmp >= 0` test that is always true, a stale maximum that can never
 * match) the quirk is kept and commented rather than "fixed".
 */
#include "pq_oracle.h"

#include <stdlib.h>
#include <string.h>
#include <omp.h>

int
pqo_idx_bytes (void)
{
    return (int) sizeof (pqo_idx);
}

/* ntc_table (src/common.c:13): complement of a base code, `$`(0) stays 0 */
static inline int
complement (int c)
{
    return c ? 5 - c : 0;
}

/* ------------------------------------------------------------------ read statistics */

/* Restates the counting in import_singlereads (src/index.c:336-346, 367-372). */
void
pqo_counts (const uint8_t *reads, pqo_idx nr, int L, pqo_idx C[6], pqo_idx sfx[4],
            pqo_idx pfx[4])
{
    pqo_idx base[4] = { 0, 0, 0, 0 };
    memset (sfx, 0, 4 * sizeof (pqo_idx));
    memset (pfx, 0, 4 * sizeof (pqo_idx));
    for (pqo_idx r = 0; r < nr; r++)
    {
        const uint8_t *s = reads + (size_t) r * L;
        pfx[s[0] - 1]++;
        sfx[s[L - 1] - 1]++;
        for (int j = 0; j < L; j++)
            base[s[j] - 1]++;
    }
    C[0] = 0;
    C[1] = 0;
    C[2] = base[0];
    C[3] = base[0] + base[1];
    C[4] = base[0] + base[1] + base[2];
    C[5] = base[0] + base[1] + base[2] + base[3];
}

/* Character at text position p of direction dir (1 = every read reversed in place, as
 * transform_to_triplet_reverse leaves the text, src/sufsort.c:80-121). */
static inline int
text_at (const uint8_t *reads, int L, int dir, pqo_idx p)
{
    if (dir == 0)
        return reads[p];
    pqo_idx r = p / (pqo_idx) L;
    int off = (int) (p % (pqo_idx) L);
    return reads[(size_t) r * L + (L - 1 - off)];
}

/* ------------------------------------------------------------------ suffix sort */

typedef struct
{
    uint64_t key;
    pqo_idx pos;
} sort_rec;

static const uint8_t *g_text;   /* text of the sort in progress (one sort at a time) */
static int g_L;

#define HEAD 29                 /* characters packed in a sort key: 29 x 2 bits + 6-bit length */

static inline uint64_t
head_key (const uint8_t *T, int L, pqo_idx p)
{
    int m = L - (int) (p % (pqo_idx) L);
    int w = m < HEAD ? m : HEAD;
    uint64_t k = 0;
    for (int i = 0; i < HEAD; i++)
        k = (k << 2) | (uint64_t) (i < w ? T[p + i] - 1 : 0);
    return (k << 6) | (uint64_t) w;
}

/* Canonical order (pinned against src/sufsort.c single-threaded): compare the read-bounded
 * suffix strings with end-of-read lowest, then text position. */
static int
cmp_suffix (const void *pa, const void *pb)
{
    const sort_rec *a = (const sort_rec *) pa, *b = (const sort_rec *) pb;
    if (a->key != b->key)
        return a->key < b->key ? -1 : 1;
    if ((a->key & 63) == HEAD)
    {
        int la = g_L - (int) (a->pos % (pqo_idx) g_L);
        int lb = g_L - (int) (b->pos % (pqo_idx) g_L);
        int m = la < lb ? la : lb;
        int c = memcmp (g_text + a->pos + HEAD, g_text + b->pos + HEAD, (size_t) (m - HEAD));
        if (c)
            return c;
        if (la != lb)
            return la < lb ? -1 : 1;
    }
    return a->pos < b->pos ? -1 : (a->pos > b->pos);
}

int
pqo_sort (const uint8_t *reads, pqo_idx nr, int L, int dir, pqo_idx *sa, int threads)
{
    if (L <= 0)
        return PQO_ERR_ARG;
    size_t n = (size_t) nr * (size_t) L;
    if (n == 0)
        return PQO_OK;
    if (threads <= 0)
        threads = omp_get_max_threads ();
    uint8_t *T = (uint8_t *) malloc (n);
    sort_rec *rec = (sort_rec *) malloc (n * sizeof (sort_rec));
    sort_rec *tmp = (sort_rec *) malloc (n * sizeof (sort_rec));
    const int NB = 1 << 16;
    size_t *hist = (size_t *) calloc ((size_t) NB * (size_t) threads, sizeof (size_t));
    size_t *bstart = (size_t *) malloc (((size_t) NB + 1) * sizeof (size_t));
    if (!T || !rec || !tmp || !hist || !bstart)
    {
        free (T);
        free (rec);
        free (tmp);
        free (hist);
        free (bstart);
        return PQO_ERR_NOMEM;
    }
#pragma omp parallel for num_threads(threads) schedule(static)
    for (size_t p = 0; p < n; p++)
        T[p] = (uint8_t) text_at (reads, L, dir, (pqo_idx) p);

#pragma omp parallel num_threads(threads)
    {
        int tid = omp_get_thread_num ();
        size_t *h = hist + (size_t) tid * NB;
#pragma omp for schedule(static)
        for (size_t p = 0; p < n; p++)
        {
            rec[p].key = head_key (T, L, (pqo_idx) p);
            rec[p].pos = (pqo_idx) p;
            h[rec[p].key >> 48]++;
        }
    }
    /* bucket-major, thread-minor exclusive scan -> scatter positions */
    size_t run = 0;
    for (int b = 0; b < NB; b++)
    {
        bstart[b] = run;
        for (int t = 0; t < threads; t++)
        {
            size_t c = hist[(size_t) t * NB + b];
            hist[(size_t) t * NB + b] = run;
            run += c;
        }
    }
    bstart[NB] = run;
#pragma omp parallel num_threads(threads)
    {
        int tid = omp_get_thread_num ();
        size_t *h = hist + (size_t) tid * NB;
#pragma omp for schedule(static)
        for (size_t p = 0; p < n; p++)
            tmp[h[rec[p].key >> 48]++] = rec[p];
    }
    g_text = T;
    g_L = L;
#pragma omp parallel for num_threads(threads) schedule(dynamic, 16)
    for (int b = 0; b < NB; b++)
    {
        size_t s = bstart[b], e = bstart[b + 1];
        if (e - s > 1)
            qsort (tmp + s, e - s, sizeof (sort_rec), cmp_suffix);
    }
#pragma omp parallel for num_threads(threads) schedule(static)
    for (size_t i = 0; i < n; i++)
        sa[i] = tmp[i].pos;
    free (T);
    free (rec);
    free (tmp);
    free (hist);
    free (bstart);
    return PQO_OK;
}

/* ------------------------------------------------------------------ BWT + occurrence tables */

/* Restates build_OCC (src/index.c:26-142) applied to the whole suffix array at once, and the
 * prefix sum of src/index.c:587-615.  Layout: bit j+1 of word b of bitmap[c] <=> BWT[64b+j] == c,
 * for j = 0..62 (`(u64)2 << 63` is 0, so the last row of a block sets no bit -- OCCx never needs
 * it: it only reads bits 1..pos%64).  sample[5b+c] = fix[c] + #c in BWT[0, 64b), fix[0] = 0.
 * The reference builds the same arrays chunk by chunk over its 5 sort slots; the chunked and
 * whole-array results agree whenever every slot holds at least 64 rows. */
int
pqo_build_occ (const uint8_t *reads, pqo_idx nr, int L, int dir, const pqo_idx *sa,
               const pqo_idx fix[4], uint64_t *bitmap, pqo_idx *sample, pqo_idx *reads_index)
{
    size_t n = (size_t) nr * (size_t) L;
    size_t rowlen = n / 64 + 1;
    pqo_idx *blk = (pqo_idx *) calloc (rowlen * 5, sizeof (pqo_idx));
    if (!blk)
        return PQO_ERR_NOMEM;
    memset (bitmap, 0, rowlen * 5 * sizeof (uint64_t));
#pragma omp parallel for schedule(static)
    for (size_t b = 0; b < rowlen; b++)
    {
        for (int j = 0; j < 64; j++)
        {
            size_t r = b * 64 + (size_t) j;
            if (r >= n)
                break;
            pqo_idx p = sa[r];
            int c = (p % (pqo_idx) L) ? text_at (reads, L, dir, p - 1) : 0;
            blk[b * 5 + c]++;
            if (j < 63)
                bitmap[(size_t) c * rowlen + b] |= (uint64_t) 2 << j;
        }
    }
    pqo_idx run[5] = { 0, fix[0], fix[1], fix[2], fix[3] };
    for (size_t b = 0; b < rowlen; b++)
        for (int c = 0; c < 5; c++)
        {
            sample[b * 5 + c] = run[c];
            run[c] += blk[b * 5 + c];
        }
    size_t k = 0;
    for (size_t r = 0; r < n; r++)
        if (sa[r] % (pqo_idx) L == 0)
            reads_index[k++] = sa[r] / (pqo_idx) L;
    free (blk);
    return PQO_OK;
}

/* ------------------------------------------------------------------ k-mer seeds */

int
pqo_kmer_table (const uint8_t *reads, pqo_idx nr, int L, int dir, const pqo_idx *sa, int k,
                pqo_idx *start, pqo_idx *size)
{
    if (k < 1 || k > 13 || k > L)
        return PQO_ERR_ARG;
    size_t n = (size_t) nr * (size_t) L, nk = (size_t) 1 << (2 * k);
    memset (start, 0, nk * sizeof (pqo_idx));
    memset (size, 0, nk * sizeof (pqo_idx));
    for (size_t r = 0; r < n; r++)
    {
        pqo_idx p = sa[r];
        if (L - (int) (p % (pqo_idx) L) < k)
            continue;
        size_t code = 0;
        for (int j = 0; j < k; j++)
            code = (code << 2) | (size_t) (text_at (reads, L, dir, p + (pqo_idx) j) - 1);
        if (size[code] == 0)
            start[code] = (pqo_idx) r;
        else if ((size_t) start[code] + size[code] != r)
            return PQO_ERR_ARG;     /* rows of one k-mer must be contiguous in a sorted SA */
        size[code]++;
    }
    return PQO_OK;
}

int
pqo_seeds_from_kmers (const uint8_t *reads, pqo_idx nr, int L, int k, const pqo_idx *kstart,
                      const pqo_idx *ksize, int dir, pqo_idx *seed_start, pqo_idx *seed_size,
                      uint16_t *seed_depth)
{
    if (k < 1 || k > 13 || k > L)
        return PQO_ERR_ARG;
    for (pqo_idx r = 0; r < nr; r++)
    {
        const uint8_t *s = reads + (size_t) r * L;
        size_t code = 0;
        for (int j = 0; j < k; j++)
        {
            int c = dir == 0 ? s[L - k + j] : s[k - 1 - j];
            code = (code << 2) | (size_t) (c - 1);
        }
        seed_start[r] = kstart[code];
        seed_size[r] = ksize[code];
        seed_depth[r] = (uint16_t) k;
    }
    return PQO_OK;
}

/* ------------------------------------------------------------------ overlap search */

/* One candidate interval (interval_t, src/string_graph.h:47-54). */
typedef struct
{
    pqo_idx ll, uu, remain;
    uint16_t len;
    uint8_t type;
} cand_t;

enum
{ T_BF = 0, T_FB = 1, T_FF = 2, T_BB = 3 };

typedef struct
{
    pqo_idx dest;
    uint16_t len;
    uint8_t type;
    int32_t trans;
} edge_t;

typedef struct
{
    const pqo_index *ix;
    size_t rowlen;
    pqo_idx n;                  /* read being searched */
    const uint8_t *read;
    cand_t *stk[2];             /* [0] B side (I_bw), [1] F side (I_fw); (2L)^2 each */
    size_t cap;
    edge_t *edges;              /* this thread's edges, all reads */
    size_t ne, ecap;
    int side_count;             /* edges emitted on the side being reduced */
    uint64_t probes;
    int err;
} worker_t;

/* OCCx (src/string_graph.c:11-23): fix + #c in BWT[0, pos) */
static inline pqo_idx
occ (worker_t *w, int d, int c, pqo_idx pos)
{
    const pqo_index *ix = w->ix;
    size_t blk = (size_t) (pos / 64);
    pqo_idx s = ix->sample[d][blk * 5 + (size_t) c];
    uint64_t m = ix->bitmap[d][(size_t) c * w->rowlen + blk];
    return s + (pqo_idx) __builtin_popcountll (m << (63 - (int) (pos % 64)));
}

/* #symbols < c in BWT[0, pos), `$` included (the OR-of-bitmaps count inside search_2) */
static inline pqo_idx
occ_less (worker_t *w, int d, int c, pqo_idx pos)
{
    const pqo_index *ix = w->ix;
    size_t blk = (size_t) (pos / 64);
    pqo_idx s = 0;
    uint64_t m = 0;
    for (int k = 0; k < c; k++)
    {
        s += ix->sample[d][blk * 5 + (size_t) k];
        m |= ix->bitmap[d][(size_t) k * w->rowlen + blk];
    }
    return s + (pqo_idx) __builtin_popcountll (m << (63 - (int) (pos % 64)));
}

/* search_1 (src/string_graph.c:55-82): LF-map a closed interval by c */
static inline void
lf_step (worker_t *w, int d, int c, pqo_idx *l, pqo_idx *u)
{
    pqo_idx ol = occ (w, d, c, *l), ou = occ (w, d, c, *u + 1);
    w->probes += 2;
    *l = w->ix->C[c] + ol;
    *u = w->ix->C[c] + ou - 1;
}

/* search_2 (src/string_graph.c:86-131): step on index d by c and keep the other index's
 * interval [ll, uu] synchronised. */
static inline void
bi_step (worker_t *w, int d, int c, pqo_idx *l, pqo_idx *u, pqo_idx *ll, pqo_idx *uu)
{
    pqo_idx vl = *l, vu = *u + 1;
    *ll = *ll + (occ_less (w, d, c, vu) - occ_less (w, d, c, vl));
    pqo_idx ol = occ (w, d, c, vl), ou = occ (w, d, c, vu);
    w->probes += 2;
    *l = w->ix->C[c] + ol;
    *u = w->ix->C[c] + ou - 1;
    *uu = *ll + ou - ol - 1;
}

/* search_3 (src/string_graph.c:134-159): (#$ in [l, u]) - 1, wrapping to all-ones at zero */
static inline pqo_idx
dollars_m1 (worker_t *w, int d, pqo_idx l, pqo_idx u)
{
    w->probes += 2;
    return occ (w, d, 0, u + 1) - occ (w, d, 0, l) - 1;
}

/* Pattern character at depth j (1-based) of each search kind (src/string_graph.c:202-374):
 * FB walks the read leftwards from its end, BF rightwards from its start; FF/BB walk the same
 * positions with complemented bases. */
static inline int
pattern_at (const uint8_t *read, int L, int kind, int j)
{
    switch (kind)
    {
    case T_FB:
        return read[L - j];
    case T_FF:
        return complement (read[L - j]);
    case T_BF:
        return read[j - 1];
    default:
        return complement (read[j - 1]);
    }
}

/* One of the four candidate searches of find_intervals.  Kind FB and BF start from the per-read
 * seed and continue while l < u; FF and BB start at depth 1 and continue while l <= u
 * (src/string_graph.c:207/226 vs :251/:269).  Candidates at depths t..L-1 are appended with
 * their $-count; a zero count is appended as well (`tmp >= 0` is always true for an unsigned
 * index, src/string_graph.c:229), with remain 0 and uu = ll - 1. */
static void
candidate_search (worker_t *w, int kind, cand_t *out, int *nout, int32_t *olp)
{
    const pqo_index *ix = w->ix;
    const int L = ix->read_len, t = ix->min_overlap;
    const int A = (kind == T_FB || kind == T_BB) ? 0 : 1;       /* index walked */
    const int B = 1 - A;                                         /* index kept in sync */
    const int strict = (kind == T_FB || kind == T_BF);
    pqo_idx l, u, ll = 0, uu = 0;
    int d;
    const int sd = (kind == T_FB) ? 0 : 1;
    if (strict && ix->seed_depth[sd])
    {
        l = ix->seed_start[sd][w->n];
        u = l + ix->seed_size[sd][w->n] - 1;
        d = ix->seed_depth[sd][w->n];
    }
    else
    {
        int c = pattern_at (w->read, L, kind, 1);
        l = ix->C[c];
        u = ix->C[c + 1] - 1;
        d = 1;
    }
#define LIVE(l, u) (strict ? ((l) < (u)) : ((l) <= (u)))
    while (LIVE (l, u) && d < t)
    {
        lf_step (w, A, pattern_at (w->read, L, kind, d + 1), &l, &u);
        d++;
    }
    if (LIVE (l, u))
    {
        int c = pattern_at (w->read, L, kind, d);
        ll = ix->C[c];
        uu = ix->C[c + 1] - 1;
        for (int j = d - 1; j >= 1; j--)
            lf_step (w, B, pattern_at (w->read, L, kind, j), &ll, &uu);
    }
    while (LIVE (l, u) && d < L)
    {
        if (kind != T_BB || d >= t)
        {
            pqo_idx tmp = dollars_m1 (w, A, l, u);
            cand_t *c = &out[(*nout)++];
            c->ll = ll;
            c->uu = ll + tmp;
            c->len = (uint16_t) d;
            c->type = (uint8_t) kind;
            c->remain = tmp + 1;
            *olp = (int32_t) ((uint32_t) * olp + (uint32_t) (tmp + 1));
        }
        bi_step (w, A, pattern_at (w->read, L, kind, d + 1), &l, &u, &ll, &uu);
        d++;
    }
#undef LIVE
}

/* Index that holds a candidate's [ll, uu]: FB/BB on the backward index, FF/BF on the forward.
 * Extending on the forward index uses the complemented base (src/string_graph.c:522-529,
 * 696-703). */
static inline int
cand_index (int type)
{
    return (type == T_FB || type == T_BB) ? 1 : 0;
}

static void
emit (worker_t *w, pqo_idx dest, int len, int type, int32_t trans)
{
    if (w->side_count + 1 > 65535)
    {
        w->err = PQO_ERR_TOO_MANY_EDGES;
        return;
    }
    if (w->ne == w->ecap)
    {
        size_t nc = w->ecap ? 2 * w->ecap : 1024;
        edge_t *e = (edge_t *) realloc (w->edges, nc * sizeof (edge_t));
        if (!e)
        {
            w->err = PQO_ERR_NOMEM;
            return;
        }
        w->edges = e;
        w->ecap = nc;
    }
    w->edges[w->ne].dest = dest;
    w->edges[w->ne].len = (uint16_t) len;
    w->edges[w->ne].type = (uint8_t) type;
    w->edges[w->ne].trans = trans;
    w->ne++;
    w->side_count++;
}

/* extract_fw_edges / extract_bw_edges (src/string_graph.c:387-556, 560-731): depth-first
 * extension of all live candidates by a = A,C,G,T; the first candidate whose overlap plus the
 * extension covers a whole read and that holds $ rows yields the irreducible edges, and that
 * branch stops.  `maxlen` is 0 at level 0, as the reference's max_fw is there (its max_bw is a
 * stale value below L, so neither check can fire at level 0). */
static void
reduce (worker_t *w, cand_t *stk, size_t pos, int size, int level, int maxlen, int32_t trans)
{
    const pqo_index *ix = w->ix;
    const int L = ix->read_len;
    cand_t *I = stk + pos;
    if (w->err)
        return;
    if (maxlen + level == L)
    {
        int flag = 0;
        for (int i = 0; i < size; i++)
        {
            if (I[i].len + level != L)
                continue;
            int o = cand_index (I[i].type);
            w->probes += 2;
            pqo_idx lll = ix->C[0] + occ (w, o, 0, I[i].ll);
            pqo_idx uuu = ix->C[0] + occ (w, o, 0, I[i].uu + 1) - 1;
            if (lll <= uuu)
            {
                for (pqo_idx k = lll; k < uuu + 1; k++)
                {
                    pqo_idx r = ix->reads_index[o][k];
                    flag = 1;
                    if (r != w->n)
                        emit (w, r, I[i].len, I[i].type, trans);
                }
                break;
            }
        }
        if (flag)
            return;
    }
    size_t cpos = pos + (size_t) size;
    for (int a = 1; a <= 4; a++)
    {
        int cnt = 0, maxl = 0;
        uint32_t tr = 0;
        for (int i = 0; i < size; i++)
        {
            if (I[i].remain == 0)
                continue;
            int o = cand_index (I[i].type);
            int c = o == 0 ? complement (a) : a;
            pqo_idx l2 = I[i].ll, u2 = I[i].uu;
            lf_step (w, o, c, &l2, &u2);
            I[i].remain = I[i].remain - (u2 - l2 + 1);
            if (l2 <= u2)
            {
                if (cpos + (size_t) cnt >= w->cap)
                {
                    w->err = PQO_ERR_CAPACITY;
                    return;
                }
                cand_t *ch = &stk[cpos + (size_t) cnt++];
                ch->ll = l2;
                ch->uu = u2;
                ch->len = I[i].len;
                ch->type = I[i].type;
                ch->remain = u2 - l2 + 1;
                tr += (uint32_t) (u2 - l2 + 1);
                if (maxl < I[i].len)
                    maxl = I[i].len;
            }
        }
        if (cnt == 0)
            continue;
        reduce (w, stk, cpos, cnt, level + 1, maxl, (int32_t) tr);
        if (w->err)
            return;
    }
}

int
pqo_overlaps (const pqo_index *ix, pqo_idx first, pqo_idx count, int threads, pqo_graph *out)
{
    memset (out, 0, sizeof *out);
    if (!ix || ix->read_len <= 0 || first > ix->num_reads || count > ix->num_reads - first)
        return out->status = PQO_ERR_ARG;
    const int L = ix->read_len;
    size_t n = (size_t) ix->num_reads * (size_t) L;
    out->first = first;
    out->count = count;
    out->num_B = (uint16_t *) calloc (count + 1, 2);
    out->num_F = (uint16_t *) calloc (count + 1, 2);
    out->olp_B = (int32_t *) calloc (count + 1, 4);
    out->olp_F = (int32_t *) calloc (count + 1, 4);
    out->edge_off = (uint64_t *) calloc (count + 1, 8);
    /* per read: owning thread and offset into its edge buffer */
    int *owner = (int *) calloc (count + 1, sizeof (int));
    size_t *toff = (size_t *) calloc (count + 1, sizeof (size_t));
    if (threads <= 0)
        threads = omp_get_max_threads ();
    worker_t *ws = (worker_t *) calloc ((size_t) threads, sizeof (worker_t));
    if (!out->num_B || !out->num_F || !out->olp_B || !out->olp_F || !out->edge_off || !owner
        || !toff || !ws)
        return out->status = PQO_ERR_NOMEM;
    int status = PQO_OK;
    pqo_idx failed = 0;
#pragma omp parallel num_threads(threads)
    {
        worker_t *w = &ws[omp_get_thread_num ()];
        w->ix = ix;
        w->rowlen = n / 64 + 1;
        w->cap = (size_t) (2 * L) * (size_t) (2 * L);
        w->stk[0] = (cand_t *) malloc (w->cap * sizeof (cand_t));
        w->stk[1] = (cand_t *) malloc (w->cap * sizeof (cand_t));
        if (!w->stk[0] || !w->stk[1])
            w->err = PQO_ERR_NOMEM;
#pragma omp for schedule(dynamic, 64)
        for (pqo_idx q = 0; q < count; q++)
        {
            if (w->err)
                continue;
            pqo_idx r = first + q;
            int nfw = 0, nbw = 0;
            int32_t oB = 0, oF = 0;
            w->n = r;
            w->read = ix->reads + (size_t) r * L;
            candidate_search (w, T_FB, w->stk[1], &nfw, &oF);
            candidate_search (w, T_FF, w->stk[1], &nfw, &oF);
            candidate_search (w, T_BF, w->stk[0], &nbw, &oB);
            candidate_search (w, T_BB, w->stk[0], &nbw, &oB);
            owner[q] = omp_get_thread_num ();
            toff[q] = w->ne;
            w->side_count = 0;
            if (oB != 0)
                reduce (w, w->stk[0], 0, nbw, 0, 0, 0);
            out->num_B[q] = (uint16_t) w->side_count;
            w->side_count = 0;
            if (oF != 0 && !w->err)
                reduce (w, w->stk[1], 0, nfw, 0, 0, 0);
            out->num_F[q] = (uint16_t) w->side_count;
            out->olp_B[q] = oB;
            out->olp_F[q] = oF;
            if (w->err)
            {
#pragma omp critical
                {
                    if (status == PQO_OK)
                    {
                        status = w->err;
                        failed = r;
                    }
                }
            }
        }
        free (w->stk[0]);
        free (w->stk[1]);
    }
    uint64_t total = 0, probes = 0;
    for (int t = 0; t < threads; t++)
        probes += ws[t].probes;
    if (status == PQO_OK)
    {
        for (pqo_idx q = 0; q < count; q++)
        {
            out->edge_off[q] = total;
            total += (uint64_t) out->num_B[q] + out->num_F[q];
        }
        out->edge_off[count] = total;
        out->edge_dest = (pqo_idx *) malloc ((total + 1) * sizeof (pqo_idx));
        out->edge_len = (uint16_t *) malloc ((total + 1) * 2);
        out->edge_type = (uint8_t *) malloc (total + 1);
        out->edge_trans = (int32_t *) malloc ((total + 1) * 4);
        if (!out->edge_dest || !out->edge_len || !out->edge_type || !out->edge_trans)
            status = PQO_ERR_NOMEM;
        else
            for (pqo_idx q = 0; q < count; q++)
            {
                const edge_t *e = ws[owner[q]].edges + toff[q];
                uint64_t k = out->edge_off[q], m = out->edge_off[q + 1] - k;
                for (uint64_t j = 0; j < m; j++)
                {
                    out->edge_dest[k + j] = e[j].dest;
                    out->edge_len[k + j] = e[j].len;
                    out->edge_type[k + j] = e[j].type;
                    out->edge_trans[k + j] = e[j].trans;
                }
            }
    }
    for (int t = 0; t < threads; t++)
        free (ws[t].edges);
    free (ws);
    free (owner);
    free (toff);
    out->num_edges = total;
    out->probes = probes;
    out->failed_read = failed;
    return out->status = status;
}

void
pqo_graph_free (pqo_graph *g)
{
    if (!g)
        return;
    free (g->num_B);
    free (g->num_F);
    free (g->olp_B);
    free (g->olp_F);
    free (g->edge_off);
    free (g->edge_dest);
    free (g->edge_len);
    free (g->edge_type);
    free (g->edge_trans);
    memset (g, 0, sizeof *g);
}
