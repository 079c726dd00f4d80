// pq_search.cu — per-read overlap search with transitive reduction on the GPU.
//
// Replaces the body of construct_string_graph's per-read loop (src/string_graph.c:800-830):
//   find_intervals   (src/string_graph.c:163-383)  four bidirectional backward searches
//   extract_bw_edges (src/string_graph.c:560-731)  DFS irreducible-edge extraction, B side
//   extract_fw_edges (src/string_graph.c:387-556)  the same for the F side
// with the rank primitives OCCx/search_1/search_2/search_3 (src/string_graph.c:11-159) on the
// one-sector occ blocks of pq_common.cuh.
//
// One thread searches one read.  The reference's recursion becomes an explicit stack: candidate
// intervals of every open level live in a per-thread array laid out exactly as the reference's
// I_fw/I_bw (a level's children directly after it), and one frame per level remembers which
// extension base comes next.  The fast kernel keeps stack, frames and edge buffer in local
// memory with fixed capacities; a read that outgrows any of them is recorded and redone by the
// wide kernel, whose per-slot scratch has the reference's own bounds ((2L)^2 candidates,
// 65535 edges per side), so every read completes with the reference's result.
#include "pq_index.cuh"
#include "pq_learned.cuh"

#include <algorithm>

namespace pq {

// One candidate interval (interval_t, src/string_graph.h:47-54).  Its remaining size is always
// uu - ll + 1 here: zero-$ level-0 entries are not stored (see side_candidates) and no counter is
// decremented, so the field is not kept.
struct Cand {
    idx_t ll, uu;
    uint16_t len;
    uint8_t type;
};
struct Frame {
    uint32_t pos;       // first candidate of this level
    uint32_t free;      // first stack slot this level may use for its extension sets
    uint32_t cbase;     // first slot of the four extension sets (stored back to back, A..T)
    int32_t trans;      // sum of this level's interval sizes (path_t.trans of its edges)
    uint16_t size;
    uint16_t maxlen;
    uint16_t csz[4];    // non-empty extensions by A, C, G, T
    uint8_t next_a;
};
struct EdgeRec {
    idx_t dest;
    int32_t trans;
    uint16_t len;
    uint8_t type;
};

// Per-thread counters of a search: rank probes (one occurrence block each, the unit of the
// reference's OCCx/search_* calls) and the 32-byte sectors of every global load of index data the
// method issues -- occurrence blocks, k-mer table entries, suffix-array and inverse-SA entries,
// packed-text words, reads_index entries and read bytes.  Tables that stay resident in L2 (the
// superblock counts, learned models) and the search's own scratch are not counted.  `+= n` is n
// rank probes, one sector each (an occurrence block is one aligned sector).
struct Tally {
    uint32_t probes{0}, sectors{0};
    __device__ __forceinline__ Tally& operator+=(uint32_t n) {
        probes += n;
        sectors += n;
        return *this;
    }
    __device__ __forceinline__ void add(uint32_t p, uint32_t s) {
        probes += p;
        sectors += s;
    }
};

// bases from text position p to the end of its read, and the read of position p (DivL: no divide)
__device__ __forceinline__ int suffix_len(idx_t p, const DivL& dl) {
    return int(dl.L - uint32_t(uint64_t(p) - div_l(uint64_t(p), dl) * dl.L));
}
__device__ __forceinline__ idx_t read_of(idx_t p, const DivL& dl) { return idx_t(div_l(uint64_t(p), dl)); }

// 32-byte sectors spanned by `bytes` bytes at p
__device__ __forceinline__ uint32_t sectors_of(const void* p, size_t bytes) {
    const uintptr_t a = reinterpret_cast<uintptr_t>(p);
    return uint32_t(((a + bytes - 1) >> 5) - (a >> 5) + 1);
}

// ------------------------------------------------------------------------------ rank primitives

__device__ __forceinline__ void ld_block(const OccBlock* p, uint64_t& lo, uint64_t& hi, uint64_t& dol,
                                         uint32_t& c01, uint32_t& c23) {
    const uint4* q = reinterpret_cast<const uint4*>(p);
    uint4 a = __ldg(q);
    uint4 b = __ldg(q + 1);
    lo = uint64_t(a.x) | (uint64_t(a.y) << 32);
    hi = uint64_t(a.z) | (uint64_t(a.w) << 32);
    dol = uint64_t(b.x) | (uint64_t(b.y) << 32);
    c01 = b.z;
    c23 = b.w;
}

__device__ __forceinline__ uint64_t below(idx_t pos) {
    return (uint64_t(1) << (pos & 63)) - 1;   // rows [64*(pos/64), pos) of the block
}

// match mask of base c (1..4) among non-$ rows
__device__ __forceinline__ uint64_t match(uint64_t lo, uint64_t hi, uint64_t dol, int c) {
    uint64_t code = uint64_t(c - 1);
    uint64_t mlo = lo ^ ((code & 1) - 1);
    uint64_t mhi = hi ^ ((code >> 1) - 1);
    return mlo & mhi & ~dol;
}

__device__ __forceinline__ uint32_t rel_cnt(uint32_t c01, uint32_t c23, int c) {
    uint32_t w = (c <= 2) ? c01 : c23;
    return ((c & 1) ? w : (w >> 16)) & 0xffff;
}

// rank of base c (1..4) in BWT[0, pos), without the fix offset
__device__ __forceinline__ idx_t rank_c(const FmView& f, int c, idx_t pos) {
    uint64_t lo, hi, dol;
    uint32_t c01, c23;
    ld_block(f.blk + (pos >> kBlockShift), lo, hi, dol, c01, c23);
    idx_t s = __ldg(f.sb + size_t(pos >> kSuperShift) * 4 + (c - 1));
    return s + rel_cnt(c01, c23, c) + idx_t(__popcll(match(lo, hi, dol, c) & below(pos)));
}

// ranks of all four bases in BWT[0, pos)
__device__ __forceinline__ void rank_all(const FmView& f, idx_t pos, idx_t r[4]) {
    uint64_t lo, hi, dol;
    uint32_t c01, c23;
    ld_block(f.blk + (pos >> kBlockShift), lo, hi, dol, c01, c23);
    const idx_t* s4 = f.sb + size_t(pos >> kSuperShift) * 4;
    idx_t s0, s1, s2, s3;
#ifdef PQ_IDX64
    ulonglong2 a = __ldg(reinterpret_cast<const ulonglong2*>(s4));
    ulonglong2 b = __ldg(reinterpret_cast<const ulonglong2*>(s4) + 1);
    s0 = a.x; s1 = a.y; s2 = b.x; s3 = b.y;
#else
    uint4 a = __ldg(reinterpret_cast<const uint4*>(s4));
    s0 = a.x; s1 = a.y; s2 = a.z; s3 = a.w;
#endif
    uint64_t m = below(pos) & ~dol;
    r[0] = s0 + (c01 & 0xffff) + idx_t(__popcll(~hi & ~lo & m));
    r[1] = s1 + (c01 >> 16) + idx_t(__popcll(~hi & lo & m));
    r[2] = s2 + (c23 & 0xffff) + idx_t(__popcll(hi & ~lo & m));
    r[3] = s3 + (c23 >> 16) + idx_t(__popcll(hi & lo & m));
}

// # of `$` rows in BWT[0, pos) (= the reference's OCC(0, pos))
__device__ __forceinline__ idx_t rank_dollar(const FmView& f, idx_t pos) {
    idx_t r[4];
    rank_all(f, pos, r);
    return pos - (r[0] + r[1] + r[2] + r[3]);
}

// search_1: LF-map the closed interval [l, u] by base c
__device__ __forceinline__ void lf_step(const FmView& f, int c, idx_t& l, idx_t& u, Tally& probes) {
    idx_t ol = rank_c(f, c, l);
    idx_t ou = rank_c(f, c, u + 1);
    probes += 2;
    l = f.Cf[c] + ol;
    u = f.Cf[c] + ou - 1;
}

// search_2: step on this index by c, keep the other index's interval [ll, uu] in sync.
// #symbols < c in [l, u] ($ included) = (pos - sum_{k>=c} rank_k) differences; fixes cancel.
__device__ __forceinline__ void bi_step(const FmView& f, int c, idx_t& l, idx_t& u, idx_t& ll, idx_t& uu,
                                        Tally& probes) {
    idx_t vl = l, vu = u + 1;
    idx_t rl[4], ru[4];
    rank_all(f, vl, rl);
    rank_all(f, vu, ru);
    probes += 2;
    idx_t gel = 0, geu = 0;
    #pragma unroll
    for (int k = 0; k < 4; ++k) {
        if (k + 1 >= c) { gel += rl[k]; geu += ru[k]; }
    }
    idx_t less_l = vl - gel, less_u = vu - geu;
    ll = ll + (less_u - less_l);
    idx_t ol = rl[c - 1], ou = ru[c - 1];
    l = f.Cf[c] + ol;
    u = f.Cf[c] + ou - 1;
    uu = ll + ou - ol - 1;
}

// search_3: (#$ in [l, u]) - 1, wrapping to all-ones at zero
__device__ __forceinline__ idx_t dollars_m1(const FmView& f, idx_t l, idx_t u, Tally& probes) {
    probes += 2;
    return rank_dollar(f, u + 1) - rank_dollar(f, l) - 1;
}

// ------------------------------------------------------------------------------ per-read search

struct ReadView {
    const uint32_t* w;   // packed 2-bit codes (A=0..T=3), 16 per word, word i at w[i*stride]
    int stride;
    __device__ __forceinline__ int at(int i) const {   // code 1..4 of read position i
        return int((w[(i >> 4) * stride] >> ((i & 15) * 2)) & 3) + 1;
    }
};

__device__ __forceinline__ int complement(int c) { return 5 - c; }

// pattern base at depth j (1-based) of each search kind (see oracle candidate_search)
__device__ __forceinline__ int pattern_at(const ReadView& rd, int L, int kind, int j) {
    switch (kind) {
        case PQ_FB: return rd.at(L - j);
        case PQ_FF: return complement(rd.at(L - j));
        case PQ_BF: return rd.at(j - 1);
        default: return complement(rd.at(j - 1));
    }
}

// exact SA interval of pattern pat(hi) pat(hi-1) ... pat(lo) (text order) from the k-mer table
__device__ __forceinline__ void kmer_seed(const FmView& f, const ReadView& rd, int L, int kind, int first,
                                          int last, int step, idx_t& l, idx_t& u, Tally& probes) {
    uint32_t code = 0;
    for (int j = first;; j += step) {
        code = (code << 2) | uint32_t(pattern_at(rd, L, kind, j) - 1);
        if (j == last) break;
    }
    l = __ldg(f.kstart + code);
    u = __ldg(f.kend + code);
    probes.add(1, 2);
}

struct ReadResult {
    int status;
    int nB, nF;
    int32_t olpB, olpF;
    int ne;
};

__device__ __forceinline__ idx_t pick4(const idx_t r[4], int c) {   // r[c - 1] without local memory
    return c == 1 ? r[0] : (c == 2 ? r[1] : (c == 3 ? r[2] : r[3]));
}

// search_2 from ranks already loaded at vl = l and vu = u + 1 (the same two blocks also give the
// `$` count of search_3, so one pair of loads serves both).
__device__ __forceinline__ void step_from_ranks(const FmView& f, int c, idx_t vl, idx_t vu, const idx_t rl[4],
                                                const idx_t ru[4], idx_t& l, idx_t& u, idx_t& ll, idx_t& uu) {
    idx_t gel = 0, geu = 0;
    #pragma unroll
    for (int k = 0; k < 4; ++k) {
        if (k + 1 >= c) { gel += rl[k]; geu += ru[k]; }
    }
    ll = ll + ((vu - geu) - (vl - gel));
    const idx_t ol = pick4(rl, c), ou = pick4(ru, c);
    const idx_t base = f.Cf[c];
    l = base + ol;
    u = base + ou - 1;
    uu = ll + ou - ol - 1;
}

__device__ __forceinline__ bool live(int kind, idx_t l, idx_t u) {
    return (kind == PQ_FB || kind == PQ_BF) ? (l < u) : (l <= u);   // src/string_graph.c:207 vs :251
}
__device__ __forceinline__ int walked_index(int kind) { return (kind == PQ_FB || kind == PQ_BB) ? 0 : 1; }

__device__ __forceinline__ uint32_t pack_meta(int len, int type) { return uint32_t(len) | (uint32_t(type) << 16); }
__device__ __forceinline__ int meta_len(uint32_t m) { return int(m & 0xffff); }
__device__ __forceinline__ int meta_type(uint32_t m) { return int(m >> 16); }

// ---------------------------------------------------------------- candidates by interval scan
//
// A candidate of kind `kind` at depth d (t <= d < L) is a read r' whose first d bases, in the
// walked index's text, equal P_d = pat(d) .. pat(1).  Its last t bases there are P_t, so r'
// appears in the depth-t interval I_t of the walked index as the row of its suffix at offset
// o = d - t; conversely a row (r', o) of I_t with o < L - t is a candidate at depth t + o exactly
// when r'[0, o) = pat(t + o) .. pat(t + 1).  So instead of walking from depth t to L one base at a
// time (the reference's search_2/search_3 loop, src/string_graph.c:226-237), the rows of I_t are
// read once: one suffix-array entry and one text comparison each, all independent loads.
//
// The reference stores, for each depth with candidates, the other index's interval of the
// reversed pattern restricted to its `$` rows: the rows whose suffix is exactly rev(P_d) followed
// by end-of-read.  Those are precisely the candidates' suffixes of length d in the other index
// (text position r' * L + L - d), consecutive and ordered by position, so the interval is
// [ISA(r'min * L + L - d), + count - 1] with r'min the smallest candidate.
//
// Chains are alive at depth d whenever a candidate exists there (a strict kind also holds the
// read's own suffix, a second row), so the depths reported are the reference's.  I_t itself is
// found by binary search over the suffix array inside the k-mer table interval of P_t's first k
// bases, the two chains of a side searched together.  A row compares as its suffix string with
// end-of-read lowest, the order of the backward search.

constexpr int kScanWords = 2;       // bases of P_t searched by bisection: the first 64 at most
constexpr int kScanMax = 256;       // larger depth-t intervals walk instead
constexpr int kScanMaskWords = 4;   // L - t up to 256

// 64 bases of packed text starting at base p (first base in the top bits)
__device__ __forceinline__ uint64_t text_window(const uint64_t* __restrict__ pk, size_t p) {
    const size_t w = p >> 5;
    const int s = int(p & 31) * 2;
    const uint64_t a = __ldg(pk + w), b = __ldg(pk + w + 1);
    return s ? ((a << s) | (b >> (64 - s))) : a;
}

__device__ __forceinline__ uint64_t top_mask(int nbases) {      // 1 <= nbases <= 32
    return nbases >= 32 ? ~uint64_t(0) : ~(~uint64_t(0) >> (2 * nbases));
}

// P = pat(t) .. pat(1) of `kind` in the walked index's text order, its first 64 bases packed (the
// bases past t are whatever follows; every comparison masks them).  P is the read's own text in
// the walked index at self * L + L - t for a strict kind, and the complement of the other index's
// text there for FF and BB.
__device__ __forceinline__ void pattern_words(const FmView* fm, int L, int t, int kind, idx_t self,
                                              uint64_t (&P)[kScanWords], Tally& probes) {
    const bool strict = kind == PQ_FB || kind == PQ_BF;
    const uint64_t* pk = fm[strict ? walked_index(kind) : 1 - walked_index(kind)].pk;
    const size_t pos = size_t(self) * L + size_t(L - t);
    const uint64_t flip = strict ? 0 : ~uint64_t(0);
    #pragma unroll
    for (int w = 0; w < kScanWords; ++w) P[w] = text_window(pk, pos + 32 * w) ^ flip;
    probes.add(0, sectors_of(pk + (pos >> 5), 8 * (kScanWords + 1)));
}

// -1 / 0 / +1: the suffix at text position p (m bases to end-of-read) is below / starts with /
// above P (t bases)
__device__ __forceinline__ int cmp_row(const uint64_t* __restrict__ pk, idx_t p, int m,
                                       const uint64_t (&P)[kScanWords], int t) {
    const int nb = m < t ? m : t;
    const size_t w0 = size_t(p) >> 5;
    const int s = int(p & 31) * 2;
    const uint64_t a = __ldg(pk + w0), b = __ldg(pk + w0 + 1), c = __ldg(pk + w0 + 2);
    const uint64_t x0 = s ? ((a << s) | (b >> (64 - s))) : a;
    const uint64_t x1 = s ? ((b << s) | (c >> (64 - s))) : b;
    const uint64_t k0 = top_mask(nb);
    if ((x0 & k0) != (P[0] & k0)) return (x0 & k0) < (P[0] & k0) ? -1 : 1;
    if (nb > 32) {
        const uint64_t k1 = top_mask(nb - 32);
        if ((x1 & k1) != (P[1] & k1)) return (x1 & k1) < (P[1] & k1) ? -1 : 1;
    }
    return m < t ? -1 : 0;
}

// sectors cmp_row loads for a suffix at text position p
__device__ __forceinline__ uint32_t cmp_sectors(const uint64_t* pk, idx_t p) {
    return sectors_of(pk + (size_t(p) >> 5), 24);
}

// Rows [first, end) of each chain's index that start with its pattern, searched within
// [lo, hi): lower and upper bounds of both chains advance together (four independent searches).
__device__ __forceinline__ void sa_bounds2(const FmView* f0, const FmView* f1, const DivL& dl,
                                           const uint64_t (&P0)[kScanWords],
                                           const uint64_t (&P1)[kScanWords], int t, const idx_t (&lo)[2],
                                           const idx_t (&hi)[2], idx_t (&first)[2], idx_t (&end)[2],
                                           Tally& probes) {
    idx_t a0[2] = {lo[0], lo[1]}, a1[2] = {hi[0], hi[1]}, b0[2] = {lo[0], lo[1]}, b1[2] = {hi[0], hi[1]};
    const FmView* fq[2] = {f0, f1};
    while (a0[0] < a1[0] || b0[0] < b1[0] || a0[1] < a1[1] || b0[1] < b1[1]) {
        idx_t pa[2], pb[2];
        #pragma unroll
        for (int q = 0; q < 2; ++q) {
            pa[q] = a0[q] < a1[q] ? __ldg(fq[q]->sa + (a0[q] + (a1[q] - a0[q]) / 2)) : 0;
            pb[q] = b0[q] < b1[q] ? __ldg(fq[q]->sa + (b0[q] + (b1[q] - b0[q]) / 2)) : 0;
        }
        #pragma unroll
        for (int q = 0; q < 2; ++q) {
            const uint64_t (&P)[kScanWords] = q ? P1 : P0;
            if (a0[q] < a1[q]) {
                const idx_t ma = a0[q] + (a1[q] - a0[q]) / 2;
                const int c = cmp_row(fq[q]->pk, pa[q], suffix_len(pa[q], dl), P, t);
                if (c < 0) a0[q] = ma + 1;
                else a1[q] = ma;
                probes.add(2, 1 + cmp_sectors(fq[q]->pk, pa[q]));
            }
            if (b0[q] < b1[q]) {
                const idx_t mb = b0[q] + (b1[q] - b0[q]) / 2;
                const int c = cmp_row(fq[q]->pk, pb[q], suffix_len(pb[q], dl), P, t);
                if (c <= 0) b0[q] = mb + 1;
                else b1[q] = mb;
                probes.add(2, 1 + cmp_sectors(fq[q]->pk, pb[q]));
            }
        }
    }
    first[0] = a0[0]; first[1] = a0[1];
    end[0] = b0[0]; end[1] = b0[1];
}

// `o` bases of the walked index's text at ra equal those of the pattern source at rs.  The
// pattern P_d (d = t + o) of a strict kind is the read's own text in the walked index at
// self * L + L - d; of FF and BB it is the complement of the other index's text there.
// `sec` counts the sectors loaded from the walked text (the pattern source is the read's own text,
// counted once by pattern_words).
__device__ __forceinline__ bool prefix_matches(const uint64_t* __restrict__ pka, size_t ra,
                                               const uint64_t* __restrict__ pks, size_t rs, int o, bool cmpl,
                                               uint32_t& sec) {
    bool ok = true;
    int c = 0;
    for (; c < o && ok; c += 32) {
        const int m = o - c < 32 ? o - c : 32;
        const uint64_t x = text_window(pka, ra + c);
        uint64_t y = text_window(pks, rs + c);
        if (cmpl) y = ~y;
        ok = ((x ^ y) & top_mask(m)) == 0;
    }
    // windows at ra, ra + 32, ..., ra + c - 32: words (ra >> 5) .. ((ra + c - 32) >> 5) + 1
    if (c > 0) sec += sectors_of(pka + (ra >> 5), 8 * ((((ra + c - 32) >> 5) - (ra >> 5)) + 2));
    return ok;
}

// Slots of the level-0 candidates of the two chains of one side: q * M + i.
struct SlotsFast {     // fast tier: the warp's global scratch
    idx_t* ll;
    idx_t* uu;
    uint32_t* meta;
    size_t base;
    int M;
    __device__ __forceinline__ void set(int q, int i, idx_t a, idx_t b, uint32_t m) const {
        const size_t p = base + size_t(q) * M + i;
        ll[p] = a;
        uu[p] = b;
        meta[p] = m;
    }
    __device__ __forceinline__ void get(int q, int i, idx_t& a, idx_t& b) const {
        const size_t p = base + size_t(q) * M + i;
        a = ll[p];
        b = uu[p];
    }
};
struct SlotsStack {    // wide tier: the slot's candidate stack
    Cand* stk;
    int M;
    __device__ __forceinline__ void set(int q, int i, idx_t a, idx_t b, uint32_t m) const {
        Cand& c = stk[q * M + i];
        c.ll = a;
        c.uu = b;
        c.len = uint16_t(meta_len(m));
        c.type = uint8_t(meta_type(m));
    }
    __device__ __forceinline__ void get(int q, int i, idx_t& a, idx_t& b) const {
        a = stk[q * M + i].ll;
        b = stk[q * M + i].uu;
    }
};

// Candidates of both chains by interval scan; false (nothing stored) when a depth-t interval
// holds more than kScanMax rows, and the caller walks instead.
template <class Slots>
__device__ __forceinline__ bool scan_pair(const SearchArgs& A, const FmView* fm, idx_t self, int k0, int k1,
                                          int (&n)[2], int32_t& olp, Tally& probes, const Slots& slots) {
    if (!fm[0].isa || !fm[1].isa) return false;      // group intervals need the inverse SA: walk
    const int L = A.L, t = A.t, k = A.seed_k, M = L - t;
    const int tb = t < 32 * kScanWords ? t : 32 * kScanWords;    // bases bisected; the rest checked per row
    uint64_t P0[kScanWords], P1[kScanWords];
    pattern_words(fm, L, t, k0, self, P0, probes);
    pattern_words(fm, L, t, k1, self, P1, probes);
    const FmView* f0 = fm + walked_index(k0);
    const FmView* f1 = fm + walked_index(k1);
    idx_t lo[2], hi[2], first[2], end[2];
    if (A.sa_seed == 2) {
        // learned window of P_t's first 16 bases: one inference per chain
        #pragma unroll
        for (int q = 0; q < 2; ++q) {
            const LearnedView& v = (q ? f1 : f0)->lx;
            const uint32_t K = uint32_t((q ? P1 : P0)[0] >> 32);
            const int sg = lx_segment(v, K);
            const long long pr = lx_predict(v, sg, K);
            const long long b0 = (long long)__ldg(v.base + sg), b1 = (long long)__ldg(v.base + sg + 1);
            const long long a = pr - (long long)__ldg(v.err + 2 * sg), b = pr + (long long)__ldg(v.err + 2 * sg + 1);
            lo[q] = idx_t(a > b0 ? a : b0);
            hi[q] = idx_t(b < b1 ? b : b1);
            if (hi[q] < lo[q]) hi[q] = lo[q];
        }
    } else {
        const uint32_t c0 = uint32_t(P0[0] >> (64 - 2 * k)), c1 = uint32_t(P1[0] >> (64 - 2 * k));
        lo[0] = __ldg(f0->kstart + c0);
        hi[0] = __ldg(f0->kend + c0) + 1;
        lo[1] = __ldg(f1->kstart + c1);
        hi[1] = __ldg(f1->kend + c1) + 1;
        probes.add(2, 4);
        if (hi[0] < lo[0]) hi[0] = lo[0];
        if (hi[1] < lo[1]) hi[1] = lo[1];
    }
    sa_bounds2(f0, f1, A.dl, P0, P1, tb, lo, hi, first, end, probes);
    if (A.sa_seed == 2) {
        // The window holds the answer for every key present in the index; for any other key it
        // is checked: the rows just outside the window must not start with P_t.
        const idx_t n_rows = A.num_reads * idx_t(L);
        bool ok = true;
        #pragma unroll
        for (int q = 0; q < 2; ++q) {
            const FmView& fa = *(q ? f1 : f0);
            const uint64_t (&P)[kScanWords] = q ? P1 : P0;
            if (first[q] == lo[q] && lo[q] > 0) {
                const idx_t p = __ldg(fa.sa + lo[q] - 1);
                ok = ok && cmp_row(fa.pk, p, suffix_len(p, A.dl), P, tb) < 0;
                probes.add(2, 1 + cmp_sectors(fa.pk, p));
            }
            if (end[q] == hi[q] && hi[q] < n_rows) {
                const idx_t p = __ldg(fa.sa + hi[q]);
                ok = ok && cmp_row(fa.pk, p, suffix_len(p, A.dl), P, tb) > 0;
                probes.add(2, 1 + cmp_sectors(fa.pk, p));
            }
        }
        if (!ok) {
            atomicAdd(A.lx_misses, 1ull);
            return false;           // plain backward search
        }
    }
    if (end[0] - first[0] > idx_t(kScanMax) || end[1] - first[1] > idx_t(kScanMax)) return false;
    #pragma unroll
    for (int q = 0; q < 2; ++q) {
        const int kind = q ? k1 : k0;
        const FmView& fa = *(q ? f1 : f0);
        const FmView& fb = fm[1 - walked_index(kind)];
        const bool cmpl = !(kind == PQ_FB || kind == PQ_BF);
        const uint64_t* pks = cmpl ? fb.pk : fa.pk;
        const size_t src = size_t(self) * L + size_t(L - t);     // P_t in the pattern source
        uint64_t mk0 = 0, mk1 = 0, mk2 = 0, mk3 = 0;              // depths with candidates (o < 256)
        for (idx_t row = first[q]; row < end[q]; ++row) {
            const idx_t p = __ldg(fa.sa + row);
            const idx_t rp = read_of(p, A.dl);
            const int o = int(p - rp * idx_t(L));
            probes.add(2, 1);
            if (o >= M || !prefix_matches(fa.pk, size_t(rp) * L, pks, src - o, o, cmpl, probes.sectors)) continue;
            if (t > tb && !prefix_matches(fa.pk, size_t(p) + tb, pks, src + tb, t - tb, cmpl, probes.sectors))
                continue;
            const uint64_t bit = uint64_t(1) << (o & 63);
            const int hw = o >> 6;
            const uint64_t cur = hw == 0 ? mk0 : hw == 1 ? mk1 : hw == 2 ? mk2 : mk3;
            const bool seen = (cur & bit) != 0;
            mk0 |= hw == 0 ? bit : 0;
            mk1 |= hw == 1 ? bit : 0;
            mk2 |= hw == 2 ? bit : 0;
            mk3 |= hw == 3 ? bit : 0;
            if (!seen) {
                slots.set(q, o, rp, 1, 0);
            } else {
                idx_t r0, cnt;
                slots.get(q, o, r0, cnt);
                slots.set(q, o, rp < r0 ? rp : r0, cnt + 1, 0);
            }
        }
        int i = 0;
        #pragma unroll
        for (int h = 0; h < kScanMaskWords; ++h) {
            uint64_t m = h == 0 ? mk0 : h == 1 ? mk1 : h == 2 ? mk2 : mk3;
            while (m) {
                const int o = 64 * h + __ffsll((long long)m) - 1;
                m &= m - 1;
                idx_t r0, cnt;
                slots.get(q, o, r0, cnt);
                const int d = t + o;
                const idx_t l0 = __ldg(fb.isa + (size_t(r0) * M + size_t(L - d - 1)));
                probes += 1;
                slots.set(q, i++, l0, l0 + cnt - 1, pack_meta(d, kind));
                olp = int32_t(uint32_t(olp) + uint32_t(cnt));
            }
        }
        n[q] = i;
    }
    return true;
}

// find_intervals for one side: kinds k0 then k1 (B-F and B-B, or F-B and F-F), searched in
// lockstep so that each thread keeps two independent chains of loads in flight.
//
// The reference walks index A from its seed to depth t with search_1, then rebuilds the other
// index's interval of the reversed pattern from depth 1 with another t-1 search_1 steps, and
// only then continues with synchronised search_2 steps.  Here both intervals start from exact
// k-mer seeds (one per index) and every step is a synchronised step, so the other interval is
// known at every depth and the rebuild disappears; SA intervals are unique per string, so the
// intervals at depth t -- and everything after -- are the reference's.  With A.sa_seed the
// candidates come from the interval scan above instead, unless a depth-t interval is too large.
// The i-th stored candidate of kind k0 (q = 0) or k1 (q = 1) goes to slot (q, i); n[q] counts them.
// `need_read()` makes rd valid (the walk reads the read's bases; the scan reads the packed text).
template <class Slots, class NeedRead>
__device__ __forceinline__ void chain_pair(const SearchArgs& A, const FmView* fm, const ReadView& rd, idx_t self,
                                           int k0, int k1, int (&n)[2], int32_t& olp, Tally& probes,
                                           const Slots& slots, NeedRead need_read) {
    const int L = A.L, t = A.t, k = A.seed_k;
    n[0] = n[1] = 0;
    if (A.sa_seed && scan_pair(A, fm, self, k0, k1, n, olp, probes, slots)) return;
    need_read();
    idx_t l[2], u[2], ll[2], uu[2];
    bool alive[2];
    #pragma unroll
    for (int q = 0; q < 2; ++q) {
        const int kind = q ? k1 : k0;
        const int ia = walked_index(kind);
        kmer_seed(fm[ia], rd, L, kind, k, 1, -1, l[q], u[q], probes);       // pat(k) .. pat(1)
        kmer_seed(fm[1 - ia], rd, L, kind, 1, k, 1, ll[q], uu[q], probes);  // pat(1) .. pat(k)
        alive[q] = live(kind, l[q], u[q]);
    }
    int d = k;
    while (d < t && (alive[0] || alive[1])) {
        #pragma unroll
        for (int q = 0; q < 2; ++q) {
            if (!alive[q]) continue;
            const int kind = q ? k1 : k0;
            const FmView& f = fm[walked_index(kind)];
            const idx_t vl = l[q], vu = u[q] + 1;
            idx_t rl[4], ru[4];
            rank_all(f, vl, rl);
            rank_all(f, vu, ru);
            probes += 2;
            step_from_ranks(f, pattern_at(rd, L, kind, d + 1), vl, vu, rl, ru, l[q], u[q], ll[q], uu[q]);
            alive[q] = live(kind, l[q], u[q]);
        }
        ++d;
    }
    while (d < L && (alive[0] || alive[1])) {
        #pragma unroll
        for (int q = 0; q < 2; ++q) {
            if (!alive[q]) continue;
            const int kind = q ? k1 : k0;
            const FmView& f = fm[walked_index(kind)];
            const idx_t vl = l[q], vu = u[q] + 1;
            idx_t rl[4], ru[4];
            rank_all(f, vl, rl);
            rank_all(f, vu, ru);
            probes += 2;
            // (#$ in [l, u]) - 1.  The reference also appends the zero-$ case (`tmp >= 0` is
            // always true, src/string_graph.c:229) with remaining size 0; such an entry is never
            // extended, and level 0 never runs the emission check (its max length plus level 0
            // cannot reach L), so it can never contribute and is not stored.
            const idx_t tmp = (vu - (ru[0] + ru[1] + ru[2] + ru[3])) - (vl - (rl[0] + rl[1] + rl[2] + rl[3])) - 1;
            if (tmp + 1 != 0) slots.set(q, n[q]++, ll[q], ll[q] + tmp, pack_meta(d, kind));
            olp = int32_t(uint32_t(olp) + uint32_t(tmp + 1));
            step_from_ranks(f, pattern_at(rd, L, kind, d + 1), vl, vu, rl, ru, l[q], u[q], ll[q], uu[q]);
            alive[q] = live(kind, l[q], u[q]);
        }
        ++d;
    }
}

// One side's candidates into the thread's stack: kind k0 then k1, the reference's order.
__device__ __forceinline__ int side_candidates(const SearchArgs& A, const FmView* fm, const ReadView& rd, idx_t self,
                                               int k0, int k1, Cand* stk, int cap, int& n_out, int32_t& olp,
                                               Tally& probes) {
    const int M = A.L - A.t;
    if (2 * M > cap) return OVF_STACK;
    int n[2];
    chain_pair(A, fm, rd, self, k0, k1, n, olp, probes, SlotsStack{stk, M}, [] {});
    for (int i = 0; i < n[1]; ++i) stk[n[0] + i] = stk[M + i];
    n_out = n[0] + n[1];
    return OVF_NONE;
}

__device__ __forceinline__ int cand_index(int type) { return (type == PQ_FB || type == PQ_BB) ? 1 : 0; }

// extract_fw_edges / extract_bw_edges as an explicit DFS over stk[0, n0).  On entering a level the
// emission check runs as in the reference; then all four extension sets are computed at once
// from one pair of block loads per interval (the reference re-probes the same two blocks for
// every base) and stored side by side; the DFS then descends into them in base order A, C, G, T.
// Computing an extension the reference skips (its remaining-size counter reached zero) only
// finds it empty, so the sets are the reference's.
__device__ __forceinline__ int reduce_side(const SearchArgs& A, const FmView* fm, idx_t self, Cand* stk, int cap,
                                           int n0, Frame* fr, int frcap, EdgeRec* eb, int ebcap, int& ne,
                                           int& side_count, Tally& probes) {
    const int L = A.L;
    int level = 0;
    fr[0].pos = 0;
    fr[0].free = uint32_t(n0);
    fr[0].size = uint16_t(n0);
    fr[0].maxlen = 0;
    fr[0].trans = 0;
    bool entering = true;
    while (true) {
        Frame& F = fr[level];
        if (entering) {
            entering = false;
            if (int(F.maxlen) + level == L) {
                bool flag = false;
                for (int i = 0; i < F.size; ++i) {
                    const Cand& c = stk[F.pos + i];
                    if (int(c.len) + level != L) continue;
                    const FmView& fo = fm[cand_index(c.type)];
                    idx_t lll = fo.Cf[0] + rank_dollar(fo, c.ll);
                    idx_t uuu = fo.Cf[0] + rank_dollar(fo, c.uu + 1) - 1;
                    probes += 2;
                    if (lll <= uuu) {
                        probes.add(0, sectors_of(fo.reads_index + lll, size_t(uuu - lll + 1) * sizeof(idx_t)));
                        for (idx_t kk = lll; kk < uuu + 1; ++kk) {
                            idx_t r = __ldg(fo.reads_index + kk);
                            flag = true;
                            if (r != self) {
                                if (side_count + 1 > 65535) return ERR_TOO_MANY;
                                if (ne >= ebcap) return OVF_EDGES;
                                EdgeRec& e = eb[ne++];
                                e.dest = r;
                                e.len = c.len;
                                e.type = c.type;
                                e.trans = F.trans;
                                side_count++;
                            }
                        }
                        break;
                    }
                }
                if (flag) {
                    if (level == 0) return OVF_NONE;
                    --level;
                    continue;
                }
            }
            // all four extension sets from one pair of loads per interval, first in four
            // regions of P slots, then packed back to back in base order
            const int P = F.size;
            const uint32_t cbase = F.free;
            if (int(cbase) + 4 * P > cap) return OVF_STACK;
            int cnt[4] = {0, 0, 0, 0};
            for (int i = 0; i < P; ++i) {
                const Cand c = stk[F.pos + i];
                // remaining size uu - ll + 1 is 0 only for a wrapped [0, all-ones] interval (an
                // empty extension at a zero LF base); the reference keeps it but never extends it
                if (idx_t(c.uu - c.ll + 1) == 0) continue;
                const int o = cand_index(c.type);
                const FmView& f = fm[o];
                idx_t rl[4], ru[4];
                rank_all(f, c.ll, rl);
                rank_all(f, c.uu + 1, ru);
                probes += 2;
                #pragma unroll
                for (int a = 1; a <= 4; ++a) {
                    const int ch = o == 0 ? complement(a) : a;
                    const idx_t ol = pick4(rl, ch), ou = pick4(ru, ch);
                    const idx_t l2 = f.Cf[ch] + ol, u2 = f.Cf[ch] + ou - 1;
                    if (l2 <= u2) {
                        Cand& x = stk[cbase + (a - 1) * P + cnt[a - 1]++];
                        x.ll = l2;
                        x.uu = u2;
                        x.len = c.len;
                        x.type = c.type;
                    }
                }
            }
            int run = cnt[0];
            for (int a = 1; a < 4; ++a) {
                for (int j = 0; j < cnt[a]; ++j) stk[cbase + run + j] = stk[cbase + a * P + j];
                run += cnt[a];
            }
            F.cbase = cbase;
            #pragma unroll
            for (int a = 0; a < 4; ++a) F.csz[a] = uint16_t(cnt[a]);
            F.next_a = 1;
        }
        while (F.next_a <= 4 && F.csz[F.next_a - 1] == 0) F.next_a++;
        if (F.next_a > 4) {
            if (level == 0) return OVF_NONE;
            --level;
            continue;
        }
        const int a = F.next_a++;
        if (level + 1 >= frcap) return OVF_LEVELS;
        Frame& G = fr[level + 1];
        uint32_t before = 0, all = 0;
        #pragma unroll
        for (int b = 0; b < 4; ++b) {
            before += (b < a - 1) ? F.csz[b] : 0;
            all += F.csz[b];
        }
        G.pos = F.cbase + before;
        G.free = F.cbase + all;             // below it: the parent's four sets, still pending
        G.size = F.csz[a - 1];
        int maxl = 0;
        uint32_t tr = 0;
        for (int i = 0; i < G.size; ++i) {
            const Cand& c = stk[G.pos + i];
            tr += uint32_t(c.uu - c.ll + 1);
            maxl = max(maxl, int(c.len));
        }
        G.maxlen = uint16_t(maxl);
        G.trans = int32_t(tr);
        ++level;
        entering = true;
    }
}

__device__ __forceinline__ ReadResult search_read(const SearchArgs& A, const FmView* fm, idx_t self,
                                                  const ReadView& rd, Cand* stk, int cap, Frame* fr, int frcap,
                                                  EdgeRec* eb, int ebcap, Tally& probes) {
    ReadResult R;
    R.status = OVF_NONE;
    R.nB = R.nF = 0;
    R.olpB = R.olpF = 0;
    R.ne = 0;
    int n0 = 0, sc = 0;
    // B side: B-F then B-B candidates, then extract_bw_edges (src/string_graph.c:824-825)
    int s = side_candidates(A, fm, rd, self, PQ_BF, PQ_BB, stk, cap, n0, R.olpB, probes);
    if (s == OVF_NONE && R.olpB != 0)
        s = reduce_side(A, fm, self, stk, cap, n0, fr, frcap, eb, ebcap, R.ne, sc, probes);
    if (s != OVF_NONE) { R.status = s; return R; }
    R.nB = sc;
    // F side: F-B then F-F candidates, then extract_fw_edges (src/string_graph.c:828-829)
    n0 = 0;
    sc = 0;
    s = side_candidates(A, fm, rd, self, PQ_FB, PQ_FF, stk, cap, n0, R.olpF, probes);
    if (s == OVF_NONE && R.olpF != 0)
        s = reduce_side(A, fm, self, stk, cap, n0, fr, frcap, eb, ebcap, R.ne, sc, probes);
    if (s != OVF_NONE) { R.status = s; return R; }
    R.nF = sc;
    return R;
}

__device__ __forceinline__ void load_read(const SearchArgs& A, idx_t r, uint32_t* w, int stride, Tally& probes) {
    const uint8_t* src = A.reads + size_t(r) * A.L;
    probes.add(0, sectors_of(src, size_t(A.L)));
    const int words = (A.L + 15) >> 4;
    for (int i = 0; i < words; ++i) {
        uint32_t v = 0;
        const int j0 = i * 16;
        const int jn = min(16, A.L - j0);
        for (int j = 0; j < jn; ++j) v |= uint32_t(src[j0 + j] - 1) << (2 * j);
        w[i * stride] = v;
    }
}

__device__ __forceinline__ void publish(const SearchOut& O, idx_t r, const ReadResult& R, const EdgeRec* eb) {
    if (R.status != OVF_NONE) {
        O.status[r] = uint8_t(R.status);
        if (R.status != ERR_TOO_MANY) {
            unsigned k = atomicAdd(O.ovf_count, 1u);
            O.ovf_list[k] = r;
        }
        return;
    }
    unsigned long long base = 0;
    if (R.ne) {
        base = atomicAdd(O.e_count, (unsigned long long)R.ne);
        if (base + R.ne > O.e_cap) {
            O.status[r] = OVF_POOL;
            unsigned k = atomicAdd(O.ovf_count, 1u);
            O.ovf_list[k] = r;
            return;
        }
        for (int i = 0; i < R.ne; ++i) {
            O.e_dest[base + i] = eb[i].dest;
            O.e_trans[base + i] = eb[i].trans;
            O.e_len[base + i] = eb[i].len;
            O.e_type[base + i] = eb[i].type;
        }
    }
    O.status[r] = OVF_NONE;
    O.num_B[r] = uint16_t(R.nB);
    O.num_F[r] = uint16_t(R.nF);
    O.olp_B[r] = R.olpB;
    O.olp_F[r] = R.olpF;
    O.edge_src[r] = base;
}

__device__ __forceinline__ void add_probes(const SearchOut& O, const Tally& t) {
    unsigned long long v = t.probes, w = t.sectors;
    #pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        v += __shfl_down_sync(0xffffffffu, v, o);
        w += __shfl_down_sync(0xffffffffu, w, o);
    }
    if ((threadIdx.x & 31) == 0) {
        if (v) atomicAdd(O.probes, v);
        if (w) atomicAdd(O.sectors, w);
    }
}

// ------------------------------------------------------------------------------ fast tier
//
// A warp takes 32 reads.  Phase A: each lane runs the candidate searches of its read (two chains
// at a time, B side then F side) and stores the level-0 candidates in the warp's scratch.
// Phase B: the whole warp reduces one (read, side) at a time -- the extract_*_edges DFS with the
// intervals of a level spread over the lanes: every lane loads the blocks of its interval, the
// four extension sets are packed with ballots, the emission check finds the first completing
// interval with a ballot, and the edge reads are fetched by all lanes at once.  Control flow of
// phase B is uniform across the warp (all decisions come from ballots, shuffles and the frames
// in shared memory), and the stack lives in global memory as three coalesced arrays.
// Phase C: each lane publishes its read (edge-pool reservation, copy, per-read counts).

constexpr int kWarpsPerCta = 4;
constexpr int kTaskCap = 512;       // stack intervals per (read, side) task
constexpr int kTaskFrames = 48;     // DFS levels per task (deeper reads go to the wide kernel)
constexpr int kPMax = 128;          // intervals of one level of one task

__device__ __forceinline__ int csz_at(uint64_t c4, int i) { return int((c4 >> (16 * i)) & 0xffff); }

// One DFS level of one task (the reference's recursion frame of extract_*_edges).
struct TFrame {
    uint32_t pos;       // first interval of this level in the task's stack
    uint32_t free;      // first stack slot this level may use for its extension sets
    uint32_t cbase;     // first slot of the four extension sets (back to back, A..T)
    int32_t trans;      // sum of this level's interval sizes (path_t.trans of its edges)
    uint16_t size, maxlen;
    uint32_t next_a;
    uint64_t csz4;      // sizes of the four sets, 16 bits each (A lowest)
    uint64_t cml4;      // largest overlap length in each set, 16 bits each
    int32_t ctr[4];     // interval-size sum of each set
};

// Shared memory of one warp for the level-synchronous DFS of its 32 tasks (MW 64-bit mask words
// per task and base: one bit per interval of a level, up to 64 MW intervals).
template <int MW>
struct MultiSmem {
    unsigned long long mask[32][4][MW];  // extension present, by entry index
    int hit[32];                         // first entry that completes a read with $ rows
    int cml[32][4];
    unsigned ctr[32][4];
    int setoff[32][4];
    int pref[33];
    uint32_t pos[32], cbase[32];
    int lvl[32], chk[32], size[32], na[32];
};

template <int MW>
__device__ __forceinline__ int popc_words(const unsigned long long* m) {
    int c = 0;
    #pragma unroll
    for (int w = 0; w < MW; ++w) c += __popcll(m[w]);
    return c;
}
// set bits of m below bit i
template <int MW>
__device__ __forceinline__ int popc_below(const unsigned long long* m, int i) {
    int c = 0;
    #pragma unroll
    for (int w = 0; w < MW; ++w) {
        const int lo = 64 * w;
        if (i >= lo + 64) c += __popcll(m[w]);
        else if (i > lo) c += __popcll(m[w] & ((1ull << (i - lo)) - 1));
    }
    return c;
}

// exclusive prefix of v over the warp into pref[0..32] (pref[32] = total), returns the total
__device__ __forceinline__ int warp_prefix(int v, int* pref) {
    const int lane = threadIdx.x & 31;
    int x = v;
    #pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const int y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= o) x += y;
    }
    pref[lane] = x - v;
    if (lane == 31) pref[32] = x;
    __syncwarp();
    return pref[32];
}

// task owning flattened item e (pref ascending, pref[32] = total)
__device__ __forceinline__ int owner_of(const int* pref, int e) {
    int lo = 0, hi = 31;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (pref[mid] <= e) lo = mid;
        else hi = mid - 1;
    }
    return lo;
}

// ------------------------------------------------------------------------------ fast tier
//
// A warp takes 32 reads.  Phase A: each lane runs the candidate searches of its read (two chains
// at a time, B side then F side) and stores the level-0 candidates in the warp's scratch.
// Phase B, once for the B side and once for the F side: the 32 (read, side) DFS of
// extract_*_edges advance together, one level per step.  Each lane owns the control of its
// read's DFS (frames, emission, backtracking); the intervals of all tasks expanding in a step
// are spread over the lanes, so the block loads of up to 32 tasks are in flight together.  The
// order of the extension sets, the first emitting interval and the DFS order of the edges are
// fixed by entry index (bit masks with population counts, an atomic minimum), never by the order
// in which lanes happen to run, so every edge list is the reference's.
// Phase C: each lane publishes its read (edge-pool reservation, copy, per-read counts).

// ------------------------------------------------------------------------------ sorted reduction
//
// extract_*_edges as a function of the candidate set.  At DFS level j an interval of candidate
// group (kind, d) holds exactly the candidates r' whose next j bases after the overlap -- their
// continuation lambda(r') -- equal the DFS path s: extending the other index's interval by base a
// selects the candidates whose next base is a (the complement on the forward index).  So the DFS
// is a walk over the trie of continuations in base order, and:
//   * it emits at node s exactly when some candidate's continuation is s (its len + level == L),
//     taking the first interval in stack order with that length -- the group of the side's first
//     kind if it has a candidate there, else the second kind's -- and its reads (in row order,
//     i.e. ascending read id, the read itself left out), with path_t.trans = the number of
//     candidates whose continuation starts with s (the frame's interval sizes summed);
//   * an emission ends the branch, so a candidate whose continuation has another candidate's as a
//     proper prefix is never reached.
// Below, each candidate's continuation (L - d <= 256 bases) is read from the packed text -- the
// forward text from r' * L + d for candidates on the backward index, the complemented backward
// text there for candidates on the forward index -- and the emitted edges are ordered by
// continuation, then read id: the DFS order.  No FM-index step is taken.

constexpr int kRedMax = 64;          // candidates of one (read, side) reduced this way
constexpr int kLamWords = 8;         // continuations up to 256 bases (L - t <= 256)

// continuation words the kernels are built for: 2 (L - t <= 64) or kLamWords
__host__ __device__ constexpr int lam_words(int M) { return M <= 64 ? 2 : kLamWords; }

// continuation of candidate r' at overlap d: L - d bases (at most 32 W) in ceil((L - d) / 32)
// words, first base in the top bits, zero past the end; word w at out[w * plane]
// (returns the 32-byte sectors of packed text it loaded)
template <int W>
__device__ __forceinline__ uint32_t continuation(const SearchArgs& A, int type, idx_t rp, int d, uint64_t* out,
                                                 size_t plane) {
    const int L = A.L, len = L - d;
    const bool fwd = cand_index(type) == 1;
    const uint64_t* pk = A.fm[fwd ? 0 : 1].pk;
    const size_t pos = size_t(rp) * L + size_t(d);
    const uint64_t flip = fwd ? 0 : ~uint64_t(0);
    int nw = 0;
    #pragma unroll
    for (int w = 0; w < W; ++w) {
        const int left = len - 32 * w;
        if (left <= 0) break;
        out[w * plane] = (text_window(pk, pos + 32 * w) ^ flip) & top_mask(left < 32 ? left : 32);
        nw = w + 1;
    }
    return nw ? sectors_of(pk + (pos >> 5), 8 * ((((pos + 32 * (nw - 1)) >> 5) - (pos >> 5)) + 2)) : 0;
}

// the first n bases (1 <= n <= 32 W) of continuations a and b agree
template <int W>
__device__ __forceinline__ bool same_prefix(const uint64_t* a, const uint64_t* b, int n, size_t plane) {
    #pragma unroll
    for (int w = 0; w < W; ++w) {
        const int rest = n - 32 * w;
        if (rest <= 0) return true;
        const uint64_t x = a[w * plane] ^ b[w * plane];
        if (rest < 32) return (x & top_mask(rest)) == 0;
        if (x) return false;
    }
    return true;
}

// order of two continuations of la and lb bases that are equal or not prefixes of one another:
// their first differing base, else equal
template <int W>
__device__ __forceinline__ int cmp_cont(const uint64_t* a, int la, const uint64_t* b, int lb, size_t plane) {
    const int n = la < lb ? la : lb;
    #pragma unroll
    for (int w = 0; w < W; ++w) {
        if (32 * w >= n) break;
        const uint64_t x = a[w * plane], y = b[w * plane];
        if (x != y) return x < y ? -1 : 1;
    }
    return la == lb ? 0 : (la < lb ? -1 : 1);
}

template <int W>
__device__ __forceinline__ int reduce_gathered(int L, const WarpScratch& S, idx_t self, int side, size_t red, int m,
                                               size_t eb, int& ne, int& count);

// Edges of one side of one read from its level-0 candidate groups (na of the first kind, then
// n0 - na of the second) in the candidate scratch at `cand`; per-lane scratch at `red`.
template <int W>
__device__ __forceinline__ int reduce_sorted(const SearchArgs& A, const WarpScratch& S, idx_t self, int side,
                                             size_t cand, int na, int n0, size_t red, size_t eb, int& ne,
                                             int& count, Tally& probes) {
    const int L = A.L, M = L - A.t;
    int m = 0;
    for (int g = 0; g < n0; ++g) {
        const size_t src = cand + (g < na ? size_t(2 * side) * M + g : size_t(2 * side + 1) * M + (g - na));
        const idx_t ll = S.c_ll[src], uu = S.c_uu[src];
        const uint32_t mt = S.c_meta[src];
        const int d = meta_len(mt), type = meta_type(mt);
        const FmView& fb = A.fm[cand_index(type)];
        for (idx_t row = ll; row <= uu; ++row) {
            const idx_t p = __ldg(fb.sa + row);
            const idx_t rp = read_of(p, A.dl);
            const uint32_t sec = continuation<W>(A, type, rp, d, S.r_k + red + m, S.r_plane);
            S.r_id[red + m] = rp;
            S.r_meta[red + m] = mt;
            probes.add(2, 1 + sec);
            ++m;
        }
    }
    return reduce_gathered<W>(L, S, self, side, red, m, eb, ne, count);
}

// The reduction of reduce_sorted over m gathered candidates: continuations in S.r_k (word w of
// candidate i at r_k[w * r_plane + red + i]), read ids in S.r_id and (overlap, kind) in S.r_meta,
// from red on.  Emitted edges go to the edge scratch at eb + ne, in DFS order.
template <int W>
__device__ __forceinline__ int reduce_gathered(int L, const WarpScratch& S, idx_t self, int side, size_t red, int m,
                                               size_t eb, int& ne, int& count) {
    const int first_kind = side ? PQ_FB : PQ_BF;
    int nemit = 0;
    for (int c = 0; c < m; ++c) {
        const uint64_t* kc = S.r_k + red + c;
        const uint32_t mc = S.r_meta[red + c];
        const int lc = L - meta_len(mc);
        bool covered = false, first_same = false;
        int trans = 0;
        for (int e = 0; e < m; ++e) {
            const uint32_t me = S.r_meta[red + e];
            const int le = L - meta_len(me);
            if (!same_prefix<W>(kc, S.r_k + red + e, le < lc ? le : lc, S.r_plane)) continue;
            if (le < lc) {
                covered = true;
                break;
            }
            ++trans;
            if (le == lc && meta_type(me) == first_kind) first_same = true;
        }
        if (covered || S.r_id[red + c] == self || (meta_type(mc) != first_kind && first_same)) continue;
        S.r_emit[red + nemit++] = uint32_t(c) | (uint32_t(trans) << 16);
    }
    // DFS order: continuation, then read id (insertion sort; a handful of edges)
    for (int i = 1; i < nemit; ++i) {
        const uint32_t x = S.r_emit[red + i];
        const int cx = int(x & 0xffff);
        const uint64_t* kx = S.r_k + red + cx;
        const int lx = L - meta_len(S.r_meta[red + cx]);
        const idx_t xi = S.r_id[red + cx];
        int j = i - 1;
        while (j >= 0) {
            const int cy = int(S.r_emit[red + j] & 0xffff);
            const int o = cmp_cont<W>(S.r_k + red + cy, L - meta_len(S.r_meta[red + cy]), kx, lx, S.r_plane);
            const bool greater = o != 0 ? o > 0 : S.r_id[red + cy] > xi;
            if (!greater) break;
            S.r_emit[red + j + 1] = S.r_emit[red + j];
            --j;
        }
        S.r_emit[red + j + 1] = x;
    }
    for (int i = 0; i < nemit; ++i) {
        const uint32_t x = S.r_emit[red + i];
        const int c = int(x & 0xffff);
        if (ne >= S.ebcap) return OVF_EDGES;
        S.e_dest[eb + ne] = S.r_id[red + c];
        S.e_trans[eb + ne] = int32_t(x >> 16);
        S.e_meta[eb + ne] = S.r_meta[red + c];
        ++ne;
    }
    count = nemit;
    return OVF_NONE;
}

// ------------------------------------------------------------------------ lean tier: candidate scan
//
// The interval scan already yields every candidate of a side with its read id and overlap -- row
// (r', o) of I_t is a candidate at depth t + o -- and its continuation is the rest of r' after the
// overlap: the walked index's text right after the matched pattern, at the row's text position
// plus t (complemented for the kinds walked on the backward index, B-F and F-F).  So the lean tier
// gathers each side's candidates for reduce_gathered straight from the scan, without the
// depth-indexed candidate slots, the inverse-SA load of every candidate depth and the suffix-array
// reload of every candidate that the group form (scan_pair + reduce_sorted) needs.

// Candidates of both kinds of one side, gathered for reduce_gathered at red + m: false when the
// scan does not apply to this read (a depth-t interval of more than kScanMax rows, or a learned
// window that missed) or the side has more than kRedMax candidates -- the fast tier then redoes
// the read.
template <int W>
__device__ __forceinline__ bool scan_planes(const SearchArgs& A, const FmView* fm, idx_t self, int k0, int k1,
                                            const WarpScratch& S, size_t red, int& m, int32_t& olp, Tally& probes) {
    const int L = A.L, t = A.t, k = A.seed_k, M = L - t;
    const int m0 = m;
    const int tb = t < 32 * kScanWords ? t : 32 * kScanWords;
    uint64_t P0[kScanWords], P1[kScanWords];
    pattern_words(fm, L, t, k0, self, P0, probes);
    pattern_words(fm, L, t, k1, self, P1, probes);
    const FmView* f0 = fm + walked_index(k0);
    const FmView* f1 = fm + walked_index(k1);
    idx_t lo[2], hi[2], first[2], end[2];
    if (A.sa_seed == 2) {
        #pragma unroll
        for (int q = 0; q < 2; ++q) {
            const LearnedView& v = (q ? f1 : f0)->lx;
            const uint32_t K = uint32_t((q ? P1 : P0)[0] >> 32);
            const int sg = lx_segment(v, K);
            const long long pr = lx_predict(v, sg, K);
            const long long b0 = (long long)__ldg(v.base + sg), b1 = (long long)__ldg(v.base + sg + 1);
            const long long a = pr - (long long)__ldg(v.err + 2 * sg), b = pr + (long long)__ldg(v.err + 2 * sg + 1);
            lo[q] = idx_t(a > b0 ? a : b0);
            hi[q] = idx_t(b < b1 ? b : b1);
            if (hi[q] < lo[q]) hi[q] = lo[q];
        }
    } else {
        const uint32_t c0 = uint32_t(P0[0] >> (64 - 2 * k)), c1 = uint32_t(P1[0] >> (64 - 2 * k));
        lo[0] = __ldg(f0->kstart + c0);
        hi[0] = __ldg(f0->kend + c0) + 1;
        lo[1] = __ldg(f1->kstart + c1);
        hi[1] = __ldg(f1->kend + c1) + 1;
        probes.add(2, 4);
        if (hi[0] < lo[0]) hi[0] = lo[0];
        if (hi[1] < lo[1]) hi[1] = lo[1];
    }
    sa_bounds2(f0, f1, A.dl, P0, P1, tb, lo, hi, first, end, probes);
    if (A.sa_seed == 2) {
        const idx_t n_rows = A.num_reads * idx_t(L);
        bool ok = true;
        #pragma unroll
        for (int q = 0; q < 2; ++q) {
            const FmView& fa = *(q ? f1 : f0);
            const uint64_t (&P)[kScanWords] = q ? P1 : P0;
            if (first[q] == lo[q] && lo[q] > 0) {
                const idx_t p = __ldg(fa.sa + lo[q] - 1);
                ok = ok && cmp_row(fa.pk, p, suffix_len(p, A.dl), P, tb) < 0;
                probes.add(2, 1 + cmp_sectors(fa.pk, p));
            }
            if (end[q] == hi[q] && hi[q] < n_rows) {
                const idx_t p = __ldg(fa.sa + hi[q]);
                ok = ok && cmp_row(fa.pk, p, suffix_len(p, A.dl), P, tb) > 0;
                probes.add(2, 1 + cmp_sectors(fa.pk, p));
            }
        }
        if (!ok) {
            atomicAdd(A.lx_misses, 1ull);
            return false;
        }
    }
    if (end[0] - first[0] > idx_t(kScanMax) || end[1] - first[1] > idx_t(kScanMax)) return false;
    #pragma unroll
    for (int q = 0; q < 2; ++q) {
        const int kind = q ? k1 : k0;
        const FmView& fa = *(q ? f1 : f0);
        const FmView& fb = fm[1 - walked_index(kind)];
        const bool cmpl = !(kind == PQ_FB || kind == PQ_BF);
        const uint64_t* pks = cmpl ? fb.pk : fa.pk;
        const uint64_t flip = walked_index(kind) ? ~uint64_t(0) : 0;
        const size_t src = size_t(self) * L + size_t(L - t);
        for (idx_t row = first[q]; row < end[q]; ++row) {
            const idx_t p = __ldg(fa.sa + row);
            const idx_t rp = read_of(p, A.dl);
            const int o = int(p - rp * idx_t(L));
            probes.add(2, 1);
            if (o >= M || !prefix_matches(fa.pk, size_t(rp) * L, pks, src - o, o, cmpl, probes.sectors)) continue;
            if (t > tb && !prefix_matches(fa.pk, size_t(p) + tb, pks, src + tb, t - tb, cmpl, probes.sectors))
                continue;
            if (m - m0 >= kRedMax) return false;
            // the continuation: M - o bases of the walked text after the pattern
            const int len = M - o;
            const size_t pos = size_t(p) + size_t(t);
            int nw = 0;
            #pragma unroll
            for (int w = 0; w < W; ++w) {
                const int left = len - 32 * w;
                if (left <= 0) break;
                S.r_k[w * S.r_plane + red + m] =
                    (text_window(fa.pk, pos + 32 * w) ^ flip) & top_mask(left < 32 ? left : 32);
                nw = w + 1;
            }
            if (nw) probes.add(0, sectors_of(fa.pk + (pos >> 5), 8 * ((((pos + 32 * (nw - 1)) >> 5) - (pos >> 5)) + 2)));
            S.r_id[red + m] = rp;
            S.r_meta[red + m] = pack_meta(t + o, kind);
            ++m;
            olp = int32_t(uint32_t(olp) + 1u);
        }
    }
    return true;
}

// warp-cooperative copy of one batch description into shared memory
__device__ __forceinline__ void load_batch(SearchBatch& dst, const SearchBatch* src, int lane) {
    static_assert(sizeof(SearchBatch) % 4 == 0, "batch description is copied in 32-bit words");
    const uint32_t* s = reinterpret_cast<const uint32_t*>(src);
    uint32_t* d = reinterpret_cast<uint32_t*>(&dst);
    for (int i = lane; i < int(sizeof(SearchBatch) / 4); i += 32) d[i] = s[i];
    __syncwarp();
}

// Without a queue (Q.count == 0) the kernel searches the one read set of (A0, O0), warp w taking
// groups of 32 reads w, w + #warps, ...  With a queue, each warp takes the next item (a batch and
// a group of its reads) from a shared counter until the queue is empty; the batch's description
// (index pair, L, t, outputs) is loaded into the warp's shared memory when it changes.
template <int W, int CAP, int FRAMES, int PMAX>
__global__ void __launch_bounds__(128, 6) k_search_fast(SearchArgs A0, SearchOut O0, WarpScratch S, SearchQueue Q) {
    constexpr int MW = PMAX / 64;
    extern __shared__ uint32_t s_reads[];
    __shared__ SearchBatch s_b[kWarpsPerCta];
    __shared__ MultiSmem<MW> s_ms[kWarpsPerCta];
    __shared__ int s_n[kWarpsPerCta][32][4];
    __shared__ int32_t s_olp[kWarpsPerCta][32][2];
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    const size_t gw = size_t(blockIdx.x) * kWarpsPerCta + wid;
    const size_t nw = size_t(gridDim.x) * kWarpsPerCta;
    SearchBatch& B = s_b[wid];
    const SearchArgs& A = B.a;
    const SearchOut& O = B.o;
    if (Q.count == 0) {
        if (lane == 0) {
            B.a = A0;
            B.o = O0;
        }
        __syncwarp();
    }
    MultiSmem<MW>& sm = s_ms[wid];
    const size_t cbase_w = gw * 32 * 4 * size_t(S.mstride);    // level-0 candidates of this warp
    const size_t ebase_w = gw * 32 * size_t(S.ebcap);          // edge slots of this warp
    const size_t tbase_w = gw * 32 * size_t(CAP);         // task stacks
    const size_t xbase_w = gw * 32 * 4 * size_t(PMAX);        // sparse extension slots
    const size_t mbase_w = gw * 32 * size_t(PMAX);            // emission bounds
    const size_t rbase_w = gw * 32 * size_t(kRedMax);          // sorted-reduction candidates
    TFrame* const frw = S.frames + gw * 32 * FRAMES;
    Tally probes;
    int cur = -1;
    // reads of the current batch (or of the list of reads handed over by the lean tier)
    const size_t list_n = Q.read_list ? size_t(*Q.list_count) : 0;
    for (size_t iter = 0;; ++iter) {
        size_t group, gend;
        if (Q.count) {
            unsigned it = 0;
            if (lane == 0) it = atomicAdd(Q.next, 1u);
            it = __shfl_sync(0xffffffffu, it, 0);
            if (it >= Q.count) break;
            const int b = int(Q.item_batch[it]);
            group = Q.item_group[it];
            gend = group + Q.groups_per_item;
            if (b != cur) {
                if (cur >= 0) add_probes(O, probes);
                probes = Tally{};
                __syncwarp();
                load_batch(B, Q.batches + b, lane);
                cur = b;
            }
        } else {
            group = gw + iter * nw;
            gend = group + 1;
            if (group * 32 >= (Q.read_list ? list_n : size_t(A.num_reads))) break;
        }
        const size_t n_items = Q.read_list ? list_n : size_t(A.num_reads);
        for (; group < gend && group * 32 < n_items; ++group) {
        const int M = A.L - A.t;
        const int L = A.L;
        const size_t item = group * 32 + lane;
        const bool have = item < n_items;
        const size_t r = Q.read_list ? (have ? size_t(Q.read_list[item]) : 0) : item;
        const idx_t self = idx_t(r);
        // ---- phase A
        if (have) {
            load_read(A, idx_t(r), s_reads + threadIdx.x, blockDim.x, probes);
            ReadView rd{s_reads + threadIdx.x, int(blockDim.x)};
            const size_t cb = cbase_w + size_t(lane) * 4 * size_t(S.mstride);
            int nb[2], nf[2];
            int32_t ob = 0, of = 0;
            chain_pair(A, A.fm, rd, self, PQ_BF, PQ_BB, nb, ob, probes, SlotsFast{S.c_ll, S.c_uu, S.c_meta, cb, M},
                       [] {});
            chain_pair(A, A.fm, rd, self, PQ_FB, PQ_FF, nf, of, probes,
                       SlotsFast{S.c_ll, S.c_uu, S.c_meta, cb + 2 * size_t(M), M}, [] {});
            s_n[wid][lane][0] = nb[0];
            s_n[wid][lane][1] = nb[1];
            s_n[wid][lane][2] = nf[0];
            s_n[wid][lane][3] = nf[1];
            s_olp[wid][lane][0] = ob;
            s_olp[wid][lane][1] = of;
        }
        __syncwarp();
        // ---- phase B
        int status = have ? OVF_NONE : -1;
        int ne = 0, count_b = 0, count_f = 0;
        const size_t tb = tbase_w + size_t(lane) * CAP;    // this lane's task stack
        TFrame* const fr = frw + lane * FRAMES;
        const size_t eb = ebase_w + size_t(lane) * S.ebcap;
        #pragma unroll 1
        for (int side = 0; side < 2; ++side) {
            bool active = have && status == OVF_NONE && s_olp[wid][lane][side] != 0;   // src/string_graph.c:824, 828
            const int na = active ? s_n[wid][lane][2 * side] : 0;
            const int n0 = active ? na + s_n[wid][lane][2 * side + 1] : 0;
            int sc_sorted = -1;
            if (active && A.sorted_reduce && s_olp[wid][lane][side] <= kRedMax) {
                const int st = reduce_sorted<W>(A, S, self, side, cbase_w + size_t(lane) * 4 * size_t(S.mstride), na,
                                             n0, rbase_w + size_t(lane) * kRedMax, eb, ne, sc_sorted, probes);
                if (st != OVF_NONE) status = st;
                active = false;
            }
            if (active && n0 > CAP) { status = OVF_STACK; active = false; }
            // level 0 = kind-0 candidates then kind-1 candidates, copied into the task stacks
            sm.na[lane] = na;
            const int tot0 = warp_prefix(active ? n0 : 0, sm.pref);
            for (int e = lane; e < tot0; e += 32) {
                const int j = owner_of(sm.pref, e);
                const int i = e - sm.pref[j];
                const int nj = sm.na[j];
                const size_t src = cbase_w + size_t(j) * 4 * size_t(S.mstride) +
                                   (i < nj ? size_t(2 * side) * M + i : size_t(2 * side + 1) * M + (i - nj));
                const size_t dst = tbase_w + size_t(j) * CAP + i;
                S.t_ll[dst] = S.c_ll[src];
                S.t_uu[dst] = S.c_uu[src];
                S.t_meta[dst] = S.c_meta[src];
            }
            __syncwarp();
            TFrame F;
            F.pos = 0;
            F.free = uint32_t(n0);
            F.cbase = 0;
            F.trans = 0;
            F.size = uint16_t(n0);
            F.maxlen = 0;
            F.next_a = 1;
            F.csz4 = 0;
            F.cml4 = 0;
            F.ctr[0] = F.ctr[1] = F.ctr[2] = F.ctr[3] = 0;
            bool entering = true;
            int level = 0, sc = 0;
            while (__any_sync(0xffffffffu, active)) {
                // (1) own control: backtrack / descend until this task needs an expansion
                if (active && !entering) {
                    while (true) {
                        int a = int(F.next_a);
                        while (a <= 4 && csz_at(F.csz4, a - 1) == 0) ++a;
                        if (a > 4) {
                            if (level == 0) { active = false; break; }
                            --level;
                            F = fr[level];
                            continue;
                        }
                        if (level + 1 >= FRAMES) { status = OVF_LEVELS; active = false; break; }
                        F.next_a = uint32_t(a + 1);
                        fr[level] = F;
                        uint32_t before = 0, all = 0;
                        #pragma unroll
                        for (int b = 0; b < 4; ++b) {
                            before += (b < a - 1) ? csz_at(F.csz4, b) : 0;
                            all += csz_at(F.csz4, b);
                        }
                        TFrame G;
                        G.pos = F.cbase + before;
                        G.free = F.cbase + all;      // below it: the parent's four sets, still pending
                        G.cbase = 0;
                        G.size = uint16_t(csz_at(F.csz4, a - 1));
                        G.maxlen = uint16_t(csz_at(F.cml4, a - 1));
                        G.trans = a == 1 ? F.ctr[0] : (a == 2 ? F.ctr[1] : (a == 3 ? F.ctr[2] : F.ctr[3]));
                        G.next_a = 1;
                        G.csz4 = 0;
                        G.cml4 = 0;
                        G.ctr[0] = G.ctr[1] = G.ctr[2] = G.ctr[3] = 0;
                        F = G;
                        ++level;
                        entering = true;
                        break;
                    }
                }
                const bool expand = active && entering;
                if (expand && F.size > PMAX) { status = OVF_STACK; active = false; }
                const bool go = active && entering;
                sm.size[lane] = go ? int(F.size) : 0;
                sm.pos[lane] = F.pos;
                sm.lvl[lane] = level;
                sm.chk[lane] = int(F.maxlen) + level == L;
                sm.hit[lane] = 0x7fffffff;
                #pragma unroll
                for (int a = 0; a < 4; ++a) {
                    #pragma unroll
                    for (int w = 0; w < MW; ++w) sm.mask[lane][a][w] = 0;
                    sm.cml[lane][a] = 0;
                    sm.ctr[lane][a] = 0;
                }
                // (2) every interval of every expanding task: one pair of block loads serves the
                // emission check and the four extensions
                const int tot = warp_prefix(go ? int(F.size) : 0, sm.pref);
                for (int e = lane; e < tot; e += 32) {
                    const int j = owner_of(sm.pref, e);
                    const int i = e - sm.pref[j];
                    const size_t tj = tbase_w + size_t(j) * CAP + sm.pos[j] + i;
                    const idx_t cl = S.t_ll[tj], cu = S.t_uu[tj];
                    const uint32_t m = S.t_meta[tj];
                    const bool ext = idx_t(cu - cl + 1) != 0;   // wrapped [0, all-ones]: kept, never extended
                    const bool ends = sm.chk[j] && meta_len(m) + sm.lvl[j] == L;
                    const int o = cand_index(meta_type(m));
                    const FmView& f = A.fm[o];
                    idx_t rl[4] = {0, 0, 0, 0}, ru[4] = {0, 0, 0, 0};
                    if (ext || ends) {
                        rank_all(f, cl, rl);
                        rank_all(f, cu + 1, ru);
                        probes += 2;
                    }
                    if (ends) {
                        const idx_t ea = f.Cf[0] + (cl - (rl[0] + rl[1] + rl[2] + rl[3]));
                        const idx_t eb2 = f.Cf[0] + ((cu + 1) - (ru[0] + ru[1] + ru[2] + ru[3])) - 1;
                        if (ea <= eb2) {
                            const size_t me = mbase_w + size_t(j) * PMAX + i;
                            S.em_l[me] = ea;
                            S.em_u[me] = eb2;
                            atomicMin(&sm.hit[j], i);
                        }
                    }
                    if (ext) {
                        #pragma unroll
                        for (int a = 1; a <= 4; ++a) {
                            const int ch = o == 0 ? complement(a) : a;
                            const idx_t lo = f.Cf[ch] + pick4(rl, ch);
                            const idx_t hi = f.Cf[ch] + pick4(ru, ch) - 1;
                            if (lo <= hi) {
                                const size_t x = xbase_w + (size_t(j) * 4 + (a - 1)) * PMAX + i;
                                S.x_ll[x] = lo;
                                S.x_uu[x] = hi;
                                S.x_meta[x] = m;
                                atomicOr(&sm.mask[j][a - 1][i >> 6], 1ull << (i & 63));
                                atomicMax(&sm.cml[j][a - 1], meta_len(m));
                                atomicAdd(&sm.ctr[j][a - 1], unsigned(hi - lo + 1));
                            }
                        }
                    }
                }
                __syncwarp();
                // (3) own control: emit, or record the four sets
                bool place = false;
                if (go) {
                    const int h = sm.hit[lane];
                    bool popped = false;
                    if (h != 0x7fffffff) {
                        const size_t me = mbase_w + size_t(lane) * PMAX + h;
                        const idx_t lll = S.em_l[me], uuu = S.em_u[me];
                        const uint32_t hm = S.t_meta[tb + F.pos + h];
                        const idx_t endk = uuu + 1;      // k < uuu + 1: no iteration when uuu + 1 wraps
                        const idx_t cnt = endk > lll ? endk - lll : 0;
                        const idx_t* rix = A.fm[cand_index(meta_type(hm))].reads_index;
                        if (cnt > 0) probes.add(0, sectors_of(rix + lll, size_t(cnt) * sizeof(idx_t)));
                        for (idx_t k = 0; k < cnt; ++k) {
                            const idx_t rr = __ldg(rix + (lll + k));
                            if (rr == self) continue;
                            if (sc + 1 > 65535) { status = ERR_TOO_MANY; break; }
                            if (ne + 1 > S.ebcap) { status = OVF_EDGES; break; }
                            S.e_dest[eb + ne] = rr;
                            S.e_trans[eb + ne] = F.trans;
                            S.e_meta[eb + ne] = hm;
                            ++ne;
                            ++sc;
                        }
                        if (status != OVF_NONE) {
                            active = false;
                        } else if (cnt > 0) {           // flag: this branch is finished
                            popped = true;
                            entering = false;
                            if (level == 0) active = false;
                            else {
                                --level;
                                F = fr[level];
                            }
                        }
                    }
                    if (!popped && active) {
                        int c[4];
                        int run = 0;
                        #pragma unroll
                        for (int a = 0; a < 4; ++a) {
                            c[a] = popc_words<MW>(sm.mask[lane][a]);
                            sm.setoff[lane][a] = run;
                            run += c[a];
                        }
                        if (int(F.free) + run > CAP) {
                            status = OVF_STACK;
                            active = false;
                        } else {
                            F.cbase = F.free;
                            F.csz4 = uint64_t(c[0]) | (uint64_t(c[1]) << 16) | (uint64_t(c[2]) << 32) |
                                     (uint64_t(c[3]) << 48);
                            F.cml4 = uint64_t(sm.cml[lane][0]) | (uint64_t(sm.cml[lane][1]) << 16) |
                                     (uint64_t(sm.cml[lane][2]) << 32) | (uint64_t(sm.cml[lane][3]) << 48);
                            F.ctr[0] = int32_t(sm.ctr[lane][0]);
                            F.ctr[1] = int32_t(sm.ctr[lane][1]);
                            F.ctr[2] = int32_t(sm.ctr[lane][2]);
                            F.ctr[3] = int32_t(sm.ctr[lane][3]);
                            F.next_a = 1;
                            entering = false;
                            place = true;
                        }
                    }
                }
                // (4) pack the sets of every expanded task into its stack, in entry order
                sm.cbase[lane] = F.cbase;
                const int totx = warp_prefix(place ? 4 * int(F.size) : 0, sm.pref);
                __syncwarp();
                for (int e = lane; e < totx; e += 32) {
                    const int j = owner_of(sm.pref, e);
                    const int rel = e - sm.pref[j];
                    const int Pj = (sm.pref[j + 1] - sm.pref[j]) >> 2;
                    const int a = rel / Pj, i = rel - a * Pj;
                    const unsigned long long* mk = sm.mask[j][a];
                    if ((mk[i >> 6] >> (i & 63)) & 1) {
                        const int dst = int(sm.cbase[j]) + sm.setoff[j][a] + popc_below<MW>(mk, i);
                        const size_t x = xbase_w + (size_t(j) * 4 + a) * PMAX + i;
                        const size_t t = tbase_w + size_t(j) * CAP + dst;
                        S.t_ll[t] = S.x_ll[x];
                        S.t_uu[t] = S.x_uu[x];
                        S.t_meta[t] = S.x_meta[x];
                    }
                }
                __syncwarp();
            }
            if (sc_sorted >= 0) sc = sc_sorted;
            if (side == 0) count_b = sc;
            else count_f = sc;
        }
        // ---- phase C: publish
        if (have) {
            if (status != OVF_NONE) {
                O.status[r] = uint8_t(status);
                if (status != ERR_TOO_MANY) {
                    unsigned k = atomicAdd(O.ovf_count, 1u);
                    O.ovf_list[k] = idx_t(r);
                }
            } else {
                unsigned long long base = 0;
                bool ok = true;
                if (ne) {
                    base = atomicAdd(O.e_count, (unsigned long long)ne);
                    if (base + ne > O.e_cap) {
                        ok = false;
                        O.status[r] = OVF_POOL;
                        unsigned k = atomicAdd(O.ovf_count, 1u);
                        O.ovf_list[k] = idx_t(r);
                    } else {
                        for (int e = 0; e < ne; ++e) {
                            const uint32_t mt = S.e_meta[eb + e];
                            O.e_dest[base + e] = S.e_dest[eb + e];
                            O.e_trans[base + e] = S.e_trans[eb + e];
                            O.e_len[base + e] = uint16_t(meta_len(mt));
                            O.e_type[base + e] = uint8_t(meta_type(mt));
                        }
                    }
                }
                if (ok) {
                    O.status[r] = OVF_NONE;
                    O.num_B[r] = uint16_t(count_b);
                    O.num_F[r] = uint16_t(count_f);
                    O.olp_B[r] = s_olp[wid][lane][0];
                    O.olp_F[r] = s_olp[wid][lane][1];
                    O.edge_src[r] = base;
                }
            }
        }
        __syncwarp();
        }
    }
    if (Q.count == 0 || cur >= 0) add_probes(O, probes);
}

// ------------------------------------------------------------------------------ lean tier
//
// One thread per read, no warp-level phases: each side's candidates by the interval scan as a list
// of records, and its edges by sorted continuations.  A read the scan does not serve (a depth-t
// interval beyond kScanMax rows, a learned window that missed) or with more than kRedMax
// candidates on a side is listed in `defer` for the fast tier (which walks and runs the DFS there).
// With no shared-memory DFS state and fewer registers, more warps stay resident to hide the latency
// of the independent suffix-array and text loads.
constexpr int kLeanThreads = 128;

template <int W>
__global__ void __launch_bounds__(kLeanThreads, 8) k_search_lean(SearchArgs A0, SearchOut O0, WarpScratch S,
                                                                SearchQueue Q) {
    extern __shared__ uint32_t s_reads[];
    __shared__ SearchBatch s_b[kLeanThreads / 32];
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    const size_t gw = size_t(blockIdx.x) * (kLeanThreads / 32) + wid;
    const size_t nw = size_t(gridDim.x) * (kLeanThreads / 32);
    SearchBatch& B = s_b[wid];
    const SearchArgs& A = B.a;
    const SearchOut& O = B.o;
    if (Q.count == 0) {
        if (lane == 0) {
            B.a = A0;
            B.o = O0;
        }
        __syncwarp();
    }
    const size_t tid = gw * 32 + lane;
    const size_t eb = tid * size_t(S.ebcap);
    const size_t red = tid * size_t(kRedMax);
    Tally probes;
    int cur = -1;
    for (size_t iter = 0;; ++iter) {
        size_t group, gend;
        if (Q.count) {
            unsigned it = 0;
            if (lane == 0) it = atomicAdd(Q.next, 1u);
            it = __shfl_sync(0xffffffffu, it, 0);
            if (it >= Q.count) break;
            const int b = int(Q.item_batch[it]);
            group = Q.item_group[it];
            gend = group + Q.groups_per_item;
            if (b != cur) {
                if (cur >= 0) add_probes(O, probes);
                probes = Tally{};
                __syncwarp();
                load_batch(B, Q.batches + b, lane);
                cur = b;
            }
        } else {
            group = gw + iter * nw;
            gend = group + 1;
            if (group * 32 >= size_t(A.num_reads)) break;
        }
        for (; group < gend && group * 32 < size_t(A.num_reads); ++group) {
            const size_t r = group * 32 + lane;
            if (r >= size_t(A.num_reads)) continue;
            const idx_t self = idx_t(r);
            // B side: B-F then B-B candidates, then extract_bw_edges (src/string_graph.c:824-825);
            // then the F side: F-B, F-F, extract_fw_edges (:828-829)
            int32_t ob = 0, of = 0;
            int m = 0, ne = 0, count_b = 0, count_f = 0;
            int status = OVF_NONE;
            bool ok = scan_planes<W>(A, A.fm, self, PQ_BF, PQ_BB, S, red, m, ob, probes);
            if (ok && ob != 0) status = reduce_gathered<W>(A.L, S, self, 0, red, m, eb, ne, count_b);
            m = 0;
            if (ok) ok = scan_planes<W>(A, A.fm, self, PQ_FB, PQ_FF, S, red, m, of, probes);
            if (ok && of != 0 && status == OVF_NONE)
                status = reduce_gathered<W>(A.L, S, self, 1, red, m, eb, ne, count_f);
            if (!ok) {              // the fast tier redoes this read (walk, or more candidates)
                const unsigned k = atomicAdd(A.defer_count, 1u);
                A.defer[k] = self;
                continue;
            }
            if (status != OVF_NONE) {
                O.status[r] = uint8_t(status);
                const unsigned k = atomicAdd(O.ovf_count, 1u);
                O.ovf_list[k] = self;
                continue;
            }
            unsigned long long base = 0;
            if (ne) {
                base = atomicAdd(O.e_count, (unsigned long long)ne);
                if (base + ne > O.e_cap) {
                    O.status[r] = OVF_POOL;
                    const unsigned k = atomicAdd(O.ovf_count, 1u);
                    O.ovf_list[k] = self;
                    continue;
                }
                for (int e = 0; e < ne; ++e) {
                    const uint32_t mt = S.e_meta[eb + e];
                    O.e_dest[base + e] = S.e_dest[eb + e];
                    O.e_trans[base + e] = S.e_trans[eb + e];
                    O.e_len[base + e] = uint16_t(meta_len(mt));
                    O.e_type[base + e] = uint8_t(meta_type(mt));
                }
            }
            O.status[r] = OVF_NONE;
            O.num_B[r] = uint16_t(count_b);
            O.num_F[r] = uint16_t(count_f);
            O.olp_B[r] = ob;
            O.olp_F[r] = of;
            O.edge_src[r] = base;
        }
        __syncwarp();
    }
    if (Q.count == 0 || cur >= 0) add_probes(O, probes);
}

int search_lean_blocks(int L, int M, int num_sms) {
    const int words = (L + 15) / 16;
    const size_t smem = size_t(words) * kLeanThreads * sizeof(uint32_t);
    int per_sm = 0;
    const cudaError_t e = lam_words(M) == 2
        ? cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_search_lean<2>, kLeanThreads, smem)
        : cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_search_lean<kLamWords>, kLeanThreads, smem);
    if (e != cudaSuccess ||
        per_sm < 1)
        per_sm = 1;
    return per_sm * num_sms;
}

int search_fast_blocks(int L, int M, int num_sms) {
    const int words = (L + 15) / 16;
    const size_t smem = size_t(words) * 32 * kWarpsPerCta * sizeof(uint32_t);
    int per_sm = 0;
    const cudaError_t e = lam_words(M) == 2
        ? cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_search_fast<2, kTaskCap, kTaskFrames, kPMax>, 32 * kWarpsPerCta, smem)
        : cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_search_fast<kLamWords, kTaskCap, kTaskFrames, kPMax>, 32 * kWarpsPerCta, smem);
    if (e != cudaSuccess || per_sm < 1)
        per_sm = 1;
    return per_sm * num_sms;
}

static size_t scratch_layout(int M_max, size_t nwarps, int ebcap, void* base, WarpScratch* S, int cap = kTaskCap,
                             int frames = kTaskFrames, int pmax = kPMax) {
    const size_t M = size_t(M_max);
    const size_t cand = nwarps * 32 * 4 * M, edg = nwarps * 32 * size_t(ebcap);
    const size_t tsk = nwarps * 32 * size_t(cap), spr = nwarps * 32 * 4 * size_t(pmax);
    const size_t emb = nwarps * 32 * size_t(pmax), frm = nwarps * 32 * size_t(frames);
    char* p = static_cast<char*>(base);
    size_t used = 0;
    auto take = [&](size_t bytes) {
        char* q = p ? p + used : nullptr;
        used += (bytes + 255) & ~size_t(255);
        return q;
    };
    WarpScratch T{};
    T.c_ll = reinterpret_cast<idx_t*>(take(cand * sizeof(idx_t)));
    T.c_uu = reinterpret_cast<idx_t*>(take(cand * sizeof(idx_t)));
    T.c_meta = reinterpret_cast<uint32_t*>(take(cand * 4));
    T.e_dest = reinterpret_cast<idx_t*>(take(edg * sizeof(idx_t)));
    T.e_trans = reinterpret_cast<int32_t*>(take(edg * 4));
    T.e_meta = reinterpret_cast<uint32_t*>(take(edg * 4));
    T.t_ll = reinterpret_cast<idx_t*>(take(tsk * sizeof(idx_t)));
    T.t_uu = reinterpret_cast<idx_t*>(take(tsk * sizeof(idx_t)));
    T.t_meta = reinterpret_cast<uint32_t*>(take(tsk * 4));
    T.x_ll = reinterpret_cast<idx_t*>(take(spr * sizeof(idx_t)));
    T.x_uu = reinterpret_cast<idx_t*>(take(spr * sizeof(idx_t)));
    T.x_meta = reinterpret_cast<uint32_t*>(take(spr * 4));
    T.em_l = reinterpret_cast<idx_t*>(take(emb * sizeof(idx_t)));
    T.em_u = reinterpret_cast<idx_t*>(take(emb * sizeof(idx_t)));
    T.frames = reinterpret_cast<TFrame*>(take(frm * sizeof(TFrame)));
    const size_t red = nwarps * 32 * size_t(kRedMax);
    T.r_k = reinterpret_cast<uint64_t*>(take(red * 8 * kLamWords));
    T.r_plane = red;
    T.r_id = reinterpret_cast<idx_t*>(take(red * sizeof(idx_t)));
    T.r_meta = reinterpret_cast<uint32_t*>(take(red * 4));
    T.r_emit = reinterpret_cast<uint32_t*>(take(red * 4));
    T.ebcap = ebcap;
    T.mstride = int(M);
    if (S) *S = T;
    return used;
}

size_t warp_scratch_bytes(int L, int t, size_t nwarps, int ebcap) {
    return scratch_layout(L - t, nwarps, ebcap, nullptr, nullptr);
}

cudaError_t search_fast(const SearchArgs& a, const SearchOut& o, int blocks, void* scratch, size_t scratch_bytes,
                        int ebcap, cudaStream_t st) {
    const size_t nwarps = size_t(blocks) * kWarpsPerCta;
    WarpScratch S;
    if (scratch_bytes < scratch_layout(a.L - a.t, nwarps, ebcap, scratch, &S)) return cudaErrorInvalidValue;
    const int words = (a.L + 15) / 16;
    size_t smem = size_t(words) * 32 * kWarpsPerCta * sizeof(uint32_t);
    SearchQueue Q{};
    if (lam_words(a.L - a.t) == 2) k_search_fast<2, kTaskCap, kTaskFrames, kPMax><<<blocks, 32 * kWarpsPerCta, smem, st>>>(a, o, S, Q);
    else k_search_fast<kLamWords, kTaskCap, kTaskFrames, kPMax><<<blocks, 32 * kWarpsPerCta, smem, st>>>(a, o, S, Q);
    note_launch();
    return cudaGetLastError();
}

cudaError_t search_lean(const SearchArgs& a, const SearchOut& o, int lean_blocks, int fast_blocks, void* scratch,
                        size_t scratch_bytes, int ebcap, cudaStream_t st) {
    const size_t nwarps = size_t(std::max(lean_blocks * (kLeanThreads / 32), fast_blocks * kWarpsPerCta));
    WarpScratch S;
    if (scratch_bytes < scratch_layout(a.L - a.t, nwarps, ebcap, scratch, &S)) return cudaErrorInvalidValue;
    const int words = (a.L + 15) / 16;
    cudaError_t e = cudaMemsetAsync(a.defer_count, 0, sizeof(unsigned), st);
    if (e != cudaSuccess) return e;
    const size_t lsm = size_t(words) * kLeanThreads * 4, fsm = size_t(words) * 32 * kWarpsPerCta * 4;
    SearchQueue none{};
    if (lam_words(a.L - a.t) == 2) k_search_lean<2><<<lean_blocks, kLeanThreads, lsm, st>>>(a, o, S, none);
    else k_search_lean<kLamWords><<<lean_blocks, kLeanThreads, lsm, st>>>(a, o, S, none);
    note_launch();
    // the handed-over reads, whatever their number (read on the device): the fast tier's DFS
    SearchQueue Q{};
    Q.read_list = a.defer;
    Q.list_count = a.defer_count;
    if (lam_words(a.L - a.t) == 2) k_search_fast<2, kTaskCap, kTaskFrames, kPMax><<<fast_blocks, 32 * kWarpsPerCta, fsm, st>>>(a, o, S, Q);
    else k_search_fast<kLamWords, kTaskCap, kTaskFrames, kPMax><<<fast_blocks, 32 * kWarpsPerCta, fsm, st>>>(a, o, S, Q);
    note_launch();
    return cudaGetLastError();
}

// Queued lean search: one persistent lean launch over the queue (kernel built for the words of
// M_max), then the fast tier over the handed-over reads of each batch in `batches` (one launch per
// batch, counts read on the device; no host sync).
cudaError_t search_lean_queue(const SearchQueue& q, const SearchBatch* host_batches, const int* batches, int nbatch,
                              int L_max, int M_max, int lean_blocks, int fast_blocks, void* scratch,
                              size_t scratch_bytes, int ebcap, cudaStream_t st) {
    const size_t nwarps = size_t(std::max(lean_blocks * (kLeanThreads / 32), fast_blocks * kWarpsPerCta));
    WarpScratch S;
    if (scratch_bytes < scratch_layout(M_max, nwarps, ebcap, scratch, &S)) return cudaErrorInvalidValue;
    const int words = (L_max + 15) / 16;
    const size_t lsm = size_t(words) * kLeanThreads * 4, fsm = size_t(words) * 32 * kWarpsPerCta * 4;
    const bool two = lam_words(M_max) == 2;
    SearchArgs a0{};
    SearchOut o0{};
    if (two) k_search_lean<2><<<lean_blocks, kLeanThreads, lsm, st>>>(a0, o0, S, q);
    else k_search_lean<kLamWords><<<lean_blocks, kLeanThreads, lsm, st>>>(a0, o0, S, q);
    note_launch();
    for (int i = 0; i < nbatch; ++i) {
        const SearchBatch& hbt = host_batches[batches[i]];
        SearchQueue Q{};
        Q.read_list = hbt.a.defer;
        Q.list_count = hbt.a.defer_count;
        if (two) k_search_fast<2, kTaskCap, kTaskFrames, kPMax><<<fast_blocks, 32 * kWarpsPerCta, fsm, st>>>(hbt.a, hbt.o, S, Q);
        else k_search_fast<kLamWords, kTaskCap, kTaskFrames, kPMax><<<fast_blocks, 32 * kWarpsPerCta, fsm, st>>>(hbt.a, hbt.o, S, Q);
        note_launch();
    }
    return cudaGetLastError();
}

size_t lean_scratch_bytes(int L, int t, int lean_blocks, int fast_blocks, int ebcap) {
    const size_t nwarps = size_t(std::max(lean_blocks * (kLeanThreads / 32), fast_blocks * kWarpsPerCta));
    return scratch_layout(L - t, nwarps, ebcap, nullptr, nullptr);
}

// ------------------------------------------------------------------------------ block tier
//
// Reads the fast tier hands over are the ones with many candidates -- low-complexity sequence,
// where a read's side can have thousands.  The block tier gives each such read one CTA: two
// threads walk the two sides (chain_pair, from exact k-mer seeds, with the reference's depths),
// the CTA expands every candidate group into its candidates (read id from the suffix array,
// continuation from the packed text), and reduces each side as reduce_gathered does, with the
// m x m ordered pairs of candidates spread over the CTA's threads: candidate c is covered when
// another candidate's continuation is a proper prefix of its own, trans(c) counts the
// continuations that start with c's, first_same(c) tells whether a candidate of the side's first
// kind has exactly c's continuation.  The emitted candidates are then ranked in DFS order
// (continuation, read id) by counting, again over pairs.  In this variant everything lives in
// shared memory; a side with more candidates than fit goes to the variant with its arrays in
// global memory, which reduces by sorting (block_sorted_side), and only a side beyond that one's
// capacity goes on to the heavy and wide tiers.

constexpr int kBlockThreads = 256;
constexpr size_t kBlockSmemBudget = 200 * 1024;     // dynamic shared memory of one block-tier CTA

struct BlockSmem {      // the block tier's dynamic shared memory (offsets in bytes)
    size_t words, ids, metas, cnts, elist, e_ids, e_metas, e_trans, groups, prefs, read, bytes;
    size_t perm0, perm1, info;      // the sorted reduction's order and walk arrays (global variant)
    int cap;            // candidates a side (and B-side edges kept while the F side is reduced)
    int nw;             // continuation words per candidate
};

// bytes a candidate takes (continuation words, read id, meta, counter, emitted list, B-side edge;
// with `sorted`, two order arrays and the walk's array) and the fixed part (both sides' candidate
// groups, their prefix sums, the read)
size_t block_per_cand(int L, int t, bool sorted = false) {
    return size_t((L - t + 31) / 32) * 8 + sizeof(idx_t) + 4 + 4 + 4 + sizeof(idx_t) + 4 + 4 + (sorted ? 12 : 0);
}
size_t block_fixed(int L, int t) {
    const int M = L - t;
    return size_t(2) * size_t(2 * M) * sizeof(Cand) + size_t(2 * M + 1) * sizeof(unsigned) +
           size_t((L + 15) / 16) * sizeof(uint32_t) + 16 * 16;
}

BlockSmem block_smem_layout(int L, int t, size_t budget, bool sorted = false) {
    BlockSmem b{};
    const int M = L - t;
    b.nw = (M + 31) / 32;
    const size_t groups = size_t(2) * size_t(2 * M) * sizeof(Cand);
    const size_t prefs = size_t(2 * M + 1) * sizeof(unsigned);
    const size_t read = size_t((L + 15) / 16) * sizeof(uint32_t);
    const size_t per = block_per_cand(L, t, sorted);
    const size_t fixed = block_fixed(L, t);
    int cap = budget > fixed ? int(std::min<size_t>((budget - fixed) / per, 65535)) : 0;
    cap &= ~31;
    b.cap = cap;
    size_t o = 0;
    auto take = [&](size_t n) {
        const size_t r = o;
        o += (n + 15) & ~size_t(15);
        return r;
    };
    b.words = take(size_t(cap) * size_t(b.nw) * 8);
    b.ids = take(size_t(cap) * sizeof(idx_t));
    b.e_ids = take(size_t(cap) * sizeof(idx_t));
    b.metas = take(size_t(cap) * 4);
    b.cnts = take(size_t(cap) * 4);
    b.elist = take(size_t(cap) * 4);
    b.e_metas = take(size_t(cap) * 4);
    b.e_trans = take(size_t(cap) * 4);
    b.groups = take(groups);
    b.prefs = take(prefs);
    b.read = take(read);
    b.perm0 = b.perm1 = b.info = 0;
    if (sorted) {
        b.perm0 = take(size_t(cap) * 4);
        b.perm1 = take(size_t(cap) * 4);
        b.info = take(size_t(cap) * 4);
    }
    b.bytes = o;
    return b;
}

// the first n bases of continuations a and b (word k of candidate i at w[k * cap + i]) agree
__device__ __forceinline__ bool block_same_prefix(const uint64_t* w, int cap, int a, int b, int n) {
    for (int k = 0; n > 0; ++k, n -= 32) {
        const uint64_t x = w[size_t(k) * cap + a] ^ w[size_t(k) * cap + b];
        if (n < 32) return (x & top_mask(n)) == 0;
        if (x) return false;
    }
    return true;
}
// order of two continuations that are equal or not prefixes of one another
__device__ __forceinline__ int block_cmp(const uint64_t* w, int cap, int nw, int a, int la, int b, int lb) {
    const int n = la < lb ? la : lb;
    for (int k = 0; k < nw && 32 * k < n; ++k) {
        const uint64_t x = w[size_t(k) * cap + a], y = w[size_t(k) * cap + b];
        if (x != y) return x < y ? -1 : 1;
    }
    return la == lb ? 0 : (la < lb ? -1 : 1);
}

constexpr int kBlockMaxWords = 8;       // continuation words a candidate (L - t <= 256)
// the digit counts' index with one pad word after every 16, so that a thread summing 16
// consecutive counts and its neighbours hit different banks
__device__ __forceinline__ int block_pad(int f) { return f + (f >> 4); }

// 4-bit digit q (0 = least significant) of candidate c's sort key: the continuation words (word 0
// most significant), then the continuation length (16 bits), then the read id.
__device__ __forceinline__ unsigned block_digit(const uint64_t* cw, int cap, int nw, const idx_t* cid,
                                                const uint32_t* cmeta, int L, int c, int q) {
    constexpr int kIdDigits = 2 * int(sizeof(idx_t));
    if (q < kIdDigits) return unsigned(uint64_t(cid[c]) >> (4 * q)) & 15u;
    q -= kIdDigits;
    if (q < 4) return (unsigned(L - meta_len(cmeta[c])) >> (4 * q)) & 15u;
    q -= 4;
    return unsigned(cw[size_t(nw - 1 - q / 16) * cap + c] >> (4 * (q % 16))) & 15u;
}

// One side's reduction by sorting, for the global-memory block tier (m up to 32768 candidates,
// where the m x m pair tests cost too much).  The candidates are ordered by (continuation, read id)
// with a stable LSD radix sort on 4-bit digits of (continuation words, length, read id): each
// thread counts and then places one contiguous run of the current order, and a digit that is the
// same for every candidate skips its placing.  Comparing the words (zero past each continuation's
// end) and then the length is the order in which a continuation precedes its extensions, so the
// candidates whose continuation starts with a given one follow it contiguously.  One walk then
// decides what the pair tests decide: a run of equal continuations with no earlier prefix among
// them is uncovered, the candidates after it that extend it are covered, trans = the run plus its
// extensions, and the run's second-kind candidates yield when a first-kind one is in it.  The
// emitted candidates come out in sorted order, which is the DFS order; they are written as the
// pair version writes them (B side: e_id/e_meta/e_trans by rank; F side: elist by rank, ccnt[c] =
// rank).  Returns the number emitted (in thread 0).
__device__ int block_sorted_side(int m, int L, int nw, int cap, const uint64_t* cw, const idx_t* cid,
                                 const uint32_t* cmeta, uint32_t* perm0, uint32_t* perm1, uint32_t* info,
                                 unsigned* scnt, unsigned* s_misc, int first_kind, idx_t self, int side,
                                 idx_t* e_id, uint32_t* e_meta, int32_t* e_trans, uint32_t* elist, uint32_t* ccnt) {
    constexpr int T = kBlockThreads;
    const int tid = threadIdx.x, lane = tid & 31, wid = tid >> 5;
    const int per = (m + T - 1) / T;
    const int b0 = min(m, tid * per), b1 = min(m, b0 + per);
    for (int i = tid; i < m; i += T) perm0[i] = uint32_t(i);
    uint32_t* src = perm0;
    uint32_t* dst = perm1;
    const int digits = 2 * int(sizeof(idx_t)) + 4 + 16 * nw;
    unsigned* s_wsum = s_misc;             // [T / 32]
    unsigned* s_dstart = s_misc + 8;       // [17]
    // which key bits differ between candidates: each key XOR candidate 0's, OR-reduced (id, length,
    // words); a digit whose bits never differ needs no pass at all
    unsigned long long* s_diff = reinterpret_cast<unsigned long long*>(s_misc + 26);   // [2 + nw]
    if (tid < 2 + nw) s_diff[tid] = 0;
    __syncthreads();
    {
        unsigned long long did = 0, dlen = 0, dw[kBlockMaxWords];
        #pragma unroll
        for (int w = 0; w < kBlockMaxWords; ++w) dw[w] = 0;
        const unsigned long long id0 = uint64_t(cid[0]), len0 = unsigned(L - meta_len(cmeta[0]));
        for (int c = tid; c < m; c += T) {
            did |= uint64_t(cid[c]) ^ id0;
            dlen |= unsigned(L - meta_len(cmeta[c])) ^ len0;
            #pragma unroll
            for (int w = 0; w < kBlockMaxWords; ++w)
                if (w < nw) dw[w] |= cw[size_t(w) * cap + c] ^ cw[size_t(w) * cap];
        }
        if (did) atomicOr(&s_diff[0], did);
        if (dlen) atomicOr(&s_diff[1], dlen);
        #pragma unroll
        for (int w = 0; w < kBlockMaxWords; ++w)
            if (w < nw && dw[w]) atomicOr(&s_diff[2 + w], dw[w]);
    }
    __syncthreads();
    for (int q = 0; q < digits; ++q) {
        {   // the digit's bits in the OR of differences: zero means every candidate has the same digit
            constexpr int kIdDigits = 2 * int(sizeof(idx_t));
            unsigned long long bits;
            if (q < kIdDigits) bits = s_diff[0] >> (4 * q);
            else if (q < kIdDigits + 4) bits = s_diff[1] >> (4 * (q - kIdDigits));
            else {
                const int r = q - kIdDigits - 4;
                bits = s_diff[2 + nw - 1 - r / 16] >> (4 * (r % 16));
            }
            if ((bits & 15ull) == 0) continue;
        }
        #pragma unroll
        for (int d = 0; d < 16; ++d) scnt[block_pad(d * T + tid)] = 0;
        for (int e = b0; e < b1; ++e)
            ++scnt[block_pad(block_digit(cw, cap, nw, cid, cmeta, L, int(src[e]), q) * T + tid)];
        __syncthreads();
        // exclusive scan of the 16 x T counts, digit-major: thread tid owns entries [16 tid, 16 tid + 16)
        unsigned mine = 0;
        #pragma unroll
        for (int j = 0; j < 16; ++j) mine += scnt[block_pad(16 * tid + j)];
        unsigned x = mine;
        #pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const unsigned y = __shfl_up_sync(0xffffffffu, x, o);
            if (lane >= o) x += y;
        }
        if (lane == 31) s_wsum[wid] = x;
        __syncthreads();
        unsigned run = x - mine;
        for (int w = 0; w < wid; ++w) run += s_wsum[w];
        #pragma unroll
        for (int j = 0; j < 16; ++j) {
            const unsigned v = scnt[block_pad(16 * tid + j)];
            scnt[block_pad(16 * tid + j)] = run;
            run += v;
        }
        if ((16 * tid) % T == 0) s_dstart[(16 * tid) / T] = run - mine;   // the digit's first place
        if (tid == 0) s_dstart[16] = unsigned(m);
        __syncthreads();
        bool trivial = false;
        #pragma unroll
        for (int d = 0; d < 16; ++d) trivial |= s_dstart[d + 1] - s_dstart[d] == unsigned(m);
        if (!trivial) {
            for (int e = b0; e < b1; ++e) {
                const uint32_t c = src[e];
                dst[scnt[block_pad(block_digit(cw, cap, nw, cid, cmeta, L, int(c), q) * T + tid)]++] = c;
            }
            uint32_t* tmp = src;
            src = dst;
            dst = tmp;
        }
        __syncthreads();
    }
    // per position of the order: common prefix with the previous candidate (bases, capped at both
    // lengths) and the continuation length
    for (int k = tid; k < m; k += T) {
        const int c = int(src[k]);
        const int lc = L - meta_len(cmeta[c]);
        int lcp = 0;
        if (k > 0) {
            const int a = int(src[k - 1]);
            const int la = L - meta_len(cmeta[a]);
            lcp = 32 * nw;
            for (int w = 0; w < nw; ++w) {
                const uint64_t z = cw[size_t(w) * cap + a] ^ cw[size_t(w) * cap + c];
                if (z) {
                    lcp = 32 * w + (__clzll(z) >> 1);
                    break;
                }
            }
            lcp = min(lcp, min(la, lc));
        }
        info[k] = uint32_t(lcp) | (uint32_t(lc) << 16);
    }
    __syncthreads();
    int ne = 0;
    if (tid == 0) {
        for (int i = 0; i < m;) {
            const int lr = int(info[i] >> 16);
            int k = i + 1;
            while (k < m && int(info[k] & 0xffffu) >= lr && int(info[k] >> 16) == lr) ++k;
            const int eq_end = k;
            while (k < m && int(info[k] & 0xffffu) >= lr) ++k;
            const int32_t trans = int32_t(k - i);
            bool first_same = false;
            for (int j = i; j < eq_end; ++j) first_same |= meta_type(cmeta[src[j]]) == first_kind;
            for (int j = i; j < eq_end; ++j) {
                const int c = int(src[j]);
                if (cid[c] == self || (meta_type(cmeta[c]) != first_kind && first_same)) continue;
                if (side == 0) {
                    e_id[ne] = cid[c];
                    e_meta[ne] = cmeta[c];
                    e_trans[ne] = trans;
                } else {
                    elist[ne] = uint32_t(c) | (uint32_t(trans) << 16);
                    ccnt[c] = uint32_t(ne);
                }
                ++ne;
            }
            i = k;
        }
    }
    return ne;
}

// kGlobal: the candidate arrays live in a per-CTA region of `scratch` (global memory, cached in
// L1/L2) instead of shared memory, for sides with more candidates than shared memory holds; each
// side is then reduced by sorting (block_sorted_side) instead of by pair tests.
template <bool kGlobal>
__global__ void __launch_bounds__(kBlockThreads) k_search_block(SearchArgs A, SearchOut O, const idx_t* list,
                                                                const unsigned* list_count, BlockSmem lay,
                                                                idx_t* next_list, unsigned* next_count,
                                                                unsigned char* scratch) {
    extern __shared__ __align__(16) unsigned char smem_dyn[];
    unsigned char* smem = kGlobal ? scratch + size_t(blockIdx.x) * lay.bytes : smem_dyn;
    uint64_t* cw = reinterpret_cast<uint64_t*>(smem + lay.words);
    uint32_t* perm0 = reinterpret_cast<uint32_t*>(smem + lay.perm0);
    uint32_t* perm1 = reinterpret_cast<uint32_t*>(smem + lay.perm1);
    uint32_t* sinfo = reinterpret_cast<uint32_t*>(smem + lay.info);
    unsigned* scnt = reinterpret_cast<unsigned*>(smem_dyn);              // global variant: 16 x 256 counts, padded
    unsigned* smisc = scnt + 16 * kBlockThreads + 16 * kBlockThreads / 16;
    idx_t* cid = reinterpret_cast<idx_t*>(smem + lay.ids);
    uint32_t* cmeta = reinterpret_cast<uint32_t*>(smem + lay.metas);
    uint32_t* ccnt = reinterpret_cast<uint32_t*>(smem + lay.cnts);
    uint32_t* elist = reinterpret_cast<uint32_t*>(smem + lay.elist);
    idx_t* e_id = reinterpret_cast<idx_t*>(smem + lay.e_ids);
    uint32_t* e_meta = reinterpret_cast<uint32_t*>(smem + lay.e_metas);
    int32_t* e_trans = reinterpret_cast<int32_t*>(smem + lay.e_trans);
    Cand* grp = reinterpret_cast<Cand*>(smem + lay.groups);
    unsigned* pref = reinterpret_cast<unsigned*>(smem + lay.prefs);
    uint32_t* rdw = reinterpret_cast<uint32_t*>(smem + lay.read);
    __shared__ int s_n[2][2];
    __shared__ int32_t s_olp[2];
    __shared__ int s_ok, s_ne, s_cnt[2];
    __shared__ unsigned s_wsum[kBlockThreads / 32];
    __shared__ unsigned long long s_base;
    const int tid = threadIdx.x, lane = tid & 31, wid = tid >> 5;
    const int L = A.L, M = L - A.t, cap = lay.cap, nw = lay.nw;
    const unsigned count = *list_count;
    Tally probes;
    for (unsigned item = blockIdx.x; item < count; item += gridDim.x) {
        const idx_t self = list[item];
        if (tid == 0) {
            load_read(A, self, rdw, 1, probes);
            s_ok = 1;
        }
        __syncthreads();
        // the candidate groups of side B (thread 0) and side F (thread 32)
        if (tid == 0 || tid == 32) {
            const int side = tid ? 1 : 0;
            ReadView rd{rdw, 1};
            int n[2];
            int32_t olp = 0;
            chain_pair(A, A.fm, rd, self, side ? PQ_FB : PQ_BF, side ? PQ_FF : PQ_BB, n, olp, probes,
                       SlotsStack{grp + size_t(side) * 2 * M, M}, [] {});
            s_n[side][0] = n[0];
            s_n[side][1] = n[1];
            s_olp[side] = olp;
        }
        __syncthreads();
        for (int side = 0; side < 2; ++side) {
            if (tid == 0) s_cnt[side] = 0;
            if (s_olp[side] == 0) {      // src/string_graph.c:824, 828
                __syncthreads();
                continue;
            }
            const int n0 = s_n[side][0], ng = n0 + s_n[side][1];
            const Cand* g = grp + size_t(side) * 2 * M;
            if (tid == 0) {       // group sizes are index-wide: summed in 64 bits, stopped past cap
                unsigned long long s = 0;
                for (int i = 0; i < ng && s <= (unsigned long long)cap; ++i) {
                    const Cand& c = g[i < n0 ? i : M + (i - n0)];
                    pref[i] = unsigned(s);
                    s += (unsigned long long)(c.uu - c.ll) + 1ull;
                }
                pref[ng] = unsigned(s);
                if (s > (unsigned long long)cap) s_ok = 0;
            }
            __syncthreads();
            if (!s_ok) break;
            const int m = int(pref[ng]);
            // every candidate's read id and continuation
            for (int i = tid; i < m; i += kBlockThreads) {
                int lo = 0, hi = ng - 1;
                while (lo < hi) {
                    const int mid = (lo + hi + 1) >> 1;
                    if (pref[mid] <= unsigned(i)) lo = mid;
                    else hi = mid - 1;
                }
                const Cand& c = g[lo < n0 ? lo : M + (lo - n0)];
                const idx_t row = c.ll + idx_t(unsigned(i) - pref[lo]);
                const FmView& fb = A.fm[cand_index(c.type)];
                const idx_t rp = read_of(__ldg(fb.sa + row), A.dl);
                const int d = int(c.len), len = L - d;
                const bool fwd = cand_index(c.type) == 1;
                const uint64_t* pk = A.fm[fwd ? 0 : 1].pk;
                const size_t pos = size_t(rp) * L + size_t(d);
                const uint64_t flip = fwd ? 0 : ~uint64_t(0);
                int used = 0;
                for (int w = 0; w < nw; ++w) {
                    const int left = len - 32 * w;
                    uint64_t x = 0;
                    if (left > 0) {
                        x = (text_window(pk, pos + 32 * w) ^ flip) & top_mask(left < 32 ? left : 32);
                        used = w + 1;
                    }
                    cw[size_t(w) * cap + i] = x;
                }
                probes.add(2, 1 + (used ? sectors_of(pk + (pos >> 5),
                                                     8 * ((((pos + 32 * (used - 1)) >> 5) - (pos >> 5)) + 2))
                                        : 0));
                cid[i] = rp;
                cmeta[i] = pack_meta(d, c.type);
            }
            __syncthreads();
            const int first_kind = side ? PQ_FB : PQ_BF;
            if constexpr (kGlobal) {
                const int nsorted = block_sorted_side(m, L, nw, cap, cw, cid, cmeta, perm0, perm1, sinfo, scnt, smisc,
                                                      first_kind, self, side, e_id, e_meta, e_trans, elist, ccnt);
                if (tid == 0) s_cnt[side] = nsorted;
                __syncthreads();
                continue;
            }
            // all pairs: covered (bit 0), first_same (bit 1), trans (bits 2..)
            for (int c = tid; c < m; c += kBlockThreads) {
                const int lc = L - meta_len(cmeta[c]);
                uint32_t v = 0;
                for (int x = 0; x < m; ++x) {
                    const uint32_t mx = cmeta[x];
                    const int lx = L - meta_len(mx);
                    if (!block_same_prefix(cw, cap, c, x, lx < lc ? lx : lc)) continue;
                    if (lx < lc) {
                        v |= 1u;
                        break;
                    }
                    v += 4u;
                    if (lx == lc && meta_type(mx) == first_kind) v |= 2u;
                }
                ccnt[c] = v;
            }
            if (tid == 0) s_ne = 0;
            __syncthreads();
            // the emitted candidates, listed (index | trans << 16) in candidate order
            for (int c0 = 0; c0 < m; c0 += kBlockThreads) {
                const int c = c0 + tid;
                bool em = false;
                if (c < m) {
                    const uint32_t v = ccnt[c];
                    em = !(v & 1u) && cid[c] != self && (meta_type(cmeta[c]) == first_kind || !(v & 2u));
                }
                const unsigned bal = __ballot_sync(0xffffffffu, em);
                if (lane == 0) s_wsum[wid] = __popc(bal);
                __syncthreads();
                unsigned before = 0, all = 0;
                for (int w = 0; w < kBlockThreads / 32; ++w) {
                    before += w < wid ? s_wsum[w] : 0u;
                    all += s_wsum[w];
                }
                if (em) elist[s_ne + int(before) + __popc(bal & ((1u << lane) - 1))] = uint32_t(c) | ((ccnt[c] >> 2) << 16);
                __syncthreads();
                if (tid == 0) s_ne += int(all);
                __syncthreads();
            }
            const int ne = s_ne;
            // DFS order: each emitted candidate's rank among the emitted ones; B-side edges are
            // kept in place, F-side ranks wait in ccnt for the pool reservation
            for (int i = tid; i < ne; i += kBlockThreads) {
                const uint32_t v = elist[i];
                const int c = int(v & 0xffff), lc = L - meta_len(cmeta[c]);
                int rank = 0;
                for (int j = 0; j < ne; ++j) {
                    const int x = int(elist[j] & 0xffff);
                    const int o = block_cmp(cw, cap, nw, x, L - meta_len(cmeta[x]), c, lc);
                    rank += (o != 0 ? o < 0 : cid[x] < cid[c]) ? 1 : 0;
                }
                if (side == 0) {
                    e_id[rank] = cid[c];
                    e_meta[rank] = cmeta[c];
                    e_trans[rank] = int32_t(v >> 16);
                } else {
                    ccnt[c] = uint32_t(rank);
                }
            }
            if (tid == 0) s_cnt[side] = ne;
            __syncthreads();
        }
        if (!s_ok) {             // more candidates than fit: the next tier
            if (tid == 0) {
                const unsigned k = atomicAdd(next_count, 1u);
                next_list[k] = self;
            }
            __syncthreads();
            continue;
        }
        const int nb = s_cnt[0], nf = s_cnt[1], ne = nb + nf;
        if (tid == 0) {
            s_base = ne ? atomicAdd(O.e_count, (unsigned long long)ne) : 0ull;
            if (s_base + ne > O.e_cap) {         // edge pool full: the host grows it, runs the read again
                O.status[self] = OVF_POOL;
                const unsigned k = atomicAdd(next_count, 1u);
                next_list[k] = self;
            } else {
                O.status[self] = OVF_NONE;
                O.num_B[self] = uint16_t(nb);
                O.num_F[self] = uint16_t(nf);
                O.olp_B[self] = s_olp[0];
                O.olp_F[self] = s_olp[1];
                O.edge_src[self] = s_base;
            }
        }
        __syncthreads();
        const unsigned long long base = s_base;
        if (base + ne <= O.e_cap) {
            for (int e = tid; e < nb; e += kBlockThreads) {
                O.e_dest[base + e] = e_id[e];
                O.e_trans[base + e] = e_trans[e];
                O.e_len[base + e] = uint16_t(meta_len(e_meta[e]));
                O.e_type[base + e] = uint8_t(meta_type(e_meta[e]));
            }
            for (int i = tid; i < nf; i += kBlockThreads) {       // the F side's candidates are still in place
                const uint32_t v = elist[i];
                const int c = int(v & 0xffff);
                const unsigned long long q = base + nb + ccnt[c];
                O.e_dest[q] = cid[c];
                O.e_trans[q] = int32_t(v >> 16);
                O.e_len[q] = uint16_t(meta_len(cmeta[c]));
                O.e_type[q] = uint8_t(meta_type(cmeta[c]));
            }
        }
        __syncthreads();
    }
    add_probes(O, probes);
}

bool block_tier_holds(int L, int t) { return block_smem_layout(L, t, kBlockSmemBudget).cap >= 128; }

cudaError_t search_block(const SearchArgs& a, const SearchOut& o, const idx_t* list, const unsigned* count,
                         unsigned count_host, idx_t* next_list, unsigned* next_count, cudaStream_t st) {
    const BlockSmem lay = block_smem_layout(a.L, a.t, kBlockSmemBudget);
    if (lay.cap < 128 || !count_host) return cudaSuccess;     // nothing this tier can hold
    cudaError_t e = cudaFuncSetAttribute(k_search_block<false>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         int(lay.bytes));
    if (e != cudaSuccess) return e;
    int dev = 0, sms = 152;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    const unsigned blocks = count_host < unsigned(sms) ? count_host : unsigned(sms);
    k_search_block<false><<<blocks, kBlockThreads, lay.bytes, st>>>(a, o, list, count, lay, next_list, next_count,
                                                                    nullptr);
    note_launch();
    return cudaGetLastError();
}

// The same tier with the candidate arrays in global memory: kBlockGlobalCap candidates a side, one
// region of block_global_bytes / blocks bytes per CTA.
constexpr int kBlockGlobalCap = 32768;

int block_global_blocks(unsigned count) {
    int dev = 0, sms = 152;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    const unsigned most = unsigned(sms) * 2;
    return int(count < most ? count : most);
}

BlockSmem block_global_layout(int L, int t) {
    return block_smem_layout(L, t, block_per_cand(L, t, true) * kBlockGlobalCap + block_fixed(L, t), true);
}
// the global variant's dynamic shared memory: the sort's 16 x kBlockThreads digit counts and a
// few words of scan state
constexpr size_t kBlockSortSmem = (16 * kBlockThreads + 16 * kBlockThreads / 16 + 64) * sizeof(unsigned);

size_t block_global_bytes(int L, int t, int blocks) { return size_t(blocks) * block_global_layout(L, t).bytes; }

cudaError_t search_block_global(const SearchArgs& a, const SearchOut& o, const idx_t* list, const unsigned* count,
                                unsigned count_host, int blocks, void* scratch, size_t scratch_bytes,
                                idx_t* next_list, unsigned* next_count, cudaStream_t st) {
    if (!count_host || blocks <= 0) return cudaSuccess;
    const BlockSmem lay = block_global_layout(a.L, a.t);
    if (scratch_bytes < size_t(blocks) * lay.bytes) return cudaErrorInvalidValue;
    k_search_block<true><<<blocks, kBlockThreads, kBlockSortSmem, st>>>(a, o, list, count, lay, next_list, next_count,
                                                                        static_cast<unsigned char*>(scratch));
    note_launch();
    return cudaGetLastError();
}

// Heavy tier: the fast kernel's DFS with 32 times the stack, 4 times the level width and 256
// levels, over a list of reads (the ones the fast tier could not hold: low-complexity sequence
// gives thousands of candidates a side).  Its own overflow goes to the wide tier.
constexpr int kHeavyCap = 16384, kHeavyFrames = 256, kHeavyPMax = 512;

size_t heavy_scratch_bytes(int L, int t, int blocks, int ebcap) {
    return scratch_layout(L - t, size_t(blocks) * kWarpsPerCta, ebcap, nullptr, nullptr, kHeavyCap, kHeavyFrames,
                          kHeavyPMax);
}

cudaError_t search_heavy(const SearchArgs& a, const SearchOut& o, const idx_t* list, const unsigned* count, int blocks,
                         void* scratch, size_t scratch_bytes, int ebcap, cudaStream_t st) {
    WarpScratch S;
    if (scratch_bytes < scratch_layout(a.L - a.t, size_t(blocks) * kWarpsPerCta, ebcap, scratch, &S, kHeavyCap,
                                       kHeavyFrames, kHeavyPMax))
        return cudaErrorInvalidValue;
    const int words = (a.L + 15) / 16;
    const size_t smem = size_t(words) * 32 * kWarpsPerCta * sizeof(uint32_t);
    SearchQueue Q{};
    Q.read_list = list;
    Q.list_count = count;
    // static shared memory (~47 KB) plus the reads: past the 48 KB a launch may take unasked
    cudaError_t e = lam_words(a.L - a.t) == 2
        ? cudaFuncSetAttribute(k_search_fast<2, kHeavyCap, kHeavyFrames, kHeavyPMax>,
                               cudaFuncAttributeMaxDynamicSharedMemorySize, int(smem))
        : cudaFuncSetAttribute(k_search_fast<kLamWords, kHeavyCap, kHeavyFrames, kHeavyPMax>,
                               cudaFuncAttributeMaxDynamicSharedMemorySize, int(smem));
    if (e != cudaSuccess) return e;
    if (lam_words(a.L - a.t) == 2)
        k_search_fast<2, kHeavyCap, kHeavyFrames, kHeavyPMax><<<blocks, 32 * kWarpsPerCta, smem, st>>>(a, o, S, Q);
    else
        k_search_fast<kLamWords, kHeavyCap, kHeavyFrames, kHeavyPMax><<<blocks, 32 * kWarpsPerCta, smem, st>>>(a, o, S,
                                                                                                            Q);
    note_launch();
    return cudaGetLastError();
}

size_t queue_scratch_bytes(int L_max, int M_max, size_t nwarps, int ebcap) {
    (void)L_max;
    return scratch_layout(M_max, nwarps, ebcap, nullptr, nullptr);
}

cudaError_t search_fast_queue(const SearchQueue& q, int L_max, int M_max, int blocks, void* scratch,
                              size_t scratch_bytes, int ebcap, cudaStream_t st) {
    const size_t nwarps = size_t(blocks) * kWarpsPerCta;
    WarpScratch S;
    if (scratch_bytes < scratch_layout(M_max, nwarps, ebcap, scratch, &S)) return cudaErrorInvalidValue;
    const int words = (L_max + 15) / 16;
    size_t smem = size_t(words) * 32 * kWarpsPerCta * sizeof(uint32_t);
    SearchArgs a{};
    SearchOut o{};
    if (lam_words(M_max) == 2) k_search_fast<2, kTaskCap, kTaskFrames, kPMax><<<blocks, 32 * kWarpsPerCta, smem, st>>>(a, o, S, q);
    else k_search_fast<kLamWords, kTaskCap, kTaskFrames, kPMax><<<blocks, 32 * kWarpsPerCta, smem, st>>>(a, o, S, q);
    note_launch();
    return cudaGetLastError();
}

// Wide tier: the reference's own capacity bounds, scratch in global memory, one slot per thread.
__global__ void __launch_bounds__(64) k_search_wide(SearchArgs A, SearchOut O, const idx_t* list, unsigned count,
                                                    WideScratch W) {
    extern __shared__ uint32_t s_reads[];
    __shared__ FmView s_fm[2];
    if (threadIdx.x < 2) s_fm[threadIdx.x] = A.fm[threadIdx.x];
    __syncthreads();
    const unsigned slot = blockIdx.x * blockDim.x + threadIdx.x;
    Tally probes;
    if (slot < unsigned(W.slots)) {
        Cand* stk = reinterpret_cast<Cand*>(W.stack) + size_t(slot) * W.stack_cap;
        Frame* fr = reinterpret_cast<Frame*>(W.frames) + size_t(slot) * W.frame_cap;
        EdgeRec* eb = reinterpret_cast<EdgeRec*>(W.edges) + size_t(slot) * W.edge_cap;
        for (unsigned i = slot; i < count; i += unsigned(W.slots)) {
            idx_t r = list[i];
            load_read(A, r, s_reads + threadIdx.x, blockDim.x, probes);
            ReadView rd{s_reads + threadIdx.x, int(blockDim.x)};
            ReadResult R = search_read(A, s_fm, r, rd, stk, int(W.stack_cap), fr, int(W.frame_cap), eb,
                                       int(W.edge_cap), probes);
            if (R.status == OVF_STACK || R.status == OVF_LEVELS) R.status = ERR_CAP;
            if (R.status == ERR_CAP || R.status == ERR_TOO_MANY || R.status == OVF_EDGES) {
                O.status[r] = uint8_t(R.status == OVF_EDGES ? ERR_CAP : R.status);
                continue;
            }
            // pool overflow is reported through status and the host grows the pool and retries
            unsigned long long base = 0;
            if (R.ne) {
                base = atomicAdd(O.e_count, (unsigned long long)R.ne);
                if (base + R.ne > O.e_cap) { O.status[r] = OVF_POOL; continue; }
                for (int e = 0; e < R.ne; ++e) {
                    O.e_dest[base + e] = eb[e].dest;
                    O.e_trans[base + e] = eb[e].trans;
                    O.e_len[base + e] = eb[e].len;
                    O.e_type[base + e] = eb[e].type;
                }
            }
            O.status[r] = OVF_NONE;
            O.num_B[r] = uint16_t(R.nB);
            O.num_F[r] = uint16_t(R.nF);
            O.olp_B[r] = R.olpB;
            O.olp_F[r] = R.olpF;
            O.edge_src[r] = base;
        }
    }
    if (probes.probes) atomicAdd(O.probes, (unsigned long long)probes.probes);
    if (probes.sectors) atomicAdd(O.sectors, (unsigned long long)probes.sectors);
}

size_t wide_slot_bytes(int L) {
    size_t cap = size_t(2 * L) * size_t(2 * L);
    return cap * sizeof(Cand) + size_t(L + 2) * sizeof(Frame) + size_t(2 * 65535 + 2) * sizeof(EdgeRec);
}

cudaError_t search_wide(const SearchArgs& a, const SearchOut& o, const idx_t* list, unsigned count,
                        const WideScratch& ws, cudaStream_t st) {
    if (!count) return cudaSuccess;
    const int tpb = 64;
    const int words = (a.L + 15) / 16;
    size_t smem = size_t(words) * tpb * sizeof(uint32_t);
    int blocks = (ws.slots + tpb - 1) / tpb;
    { k_search_wide<<<blocks, tpb, smem, st>>>(a, o, list, count, ws); note_launch(); }
    return cudaGetLastError();
}

// ------------------------------------------------------------------------------ CSR assembly

__global__ void k_edge_counts(const uint16_t* nB, const uint16_t* nF, idx_t n, unsigned long long* cnt) {
    const size_t stride = size_t(gridDim.x) * blockDim.x;
    for (size_t r = size_t(blockIdx.x) * blockDim.x + threadIdx.x; r < n; r += stride)
        cnt[r] = (unsigned long long)nB[r] + nF[r];
}

// exclusive scan of 64-bit counts: tiles of 1024 per CTA (3 passes)
__global__ void k_scan_tiles(const unsigned long long* in, size_t n, unsigned long long* out,
                             unsigned long long* tile_sums) {
    __shared__ unsigned long long warp_sum[32];
    const size_t tile = blockIdx.x;
    const size_t i = tile * 1024 + threadIdx.x;
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    unsigned long long v = i < n ? in[i] : 0, x = v;
    #pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        unsigned long long y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= o) x += y;
    }
    if (lane == 31) warp_sum[wid] = x;
    __syncthreads();
    if (wid == 0) {
        unsigned long long w = warp_sum[lane], z = w;
        #pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            unsigned long long y = __shfl_up_sync(0xffffffffu, z, o);
            if (lane >= o) z += y;
        }
        warp_sum[lane] = z - w;
        if (lane == 31 && tile_sums) tile_sums[tile] = z;
    }
    __syncthreads();
    if (i < n) out[i] = warp_sum[wid] + x - v;
}

__global__ void k_scan_add(unsigned long long* out, size_t n, const unsigned long long* tile_off) {
    const size_t i = size_t(blockIdx.x) * 1024 + threadIdx.x;
    if (i < n) out[i] += tile_off[blockIdx.x];
}

static void scan_u64(const unsigned long long* in, size_t n, unsigned long long* out, unsigned long long* tmp,
                     cudaStream_t st) {
    if (n == 0) return;
    size_t tiles = (n + 1023) / 1024;
    if (tiles == 1) {
        { k_scan_tiles<<<1, 1024, 0, st>>>(in, n, out, nullptr); note_launch(); }
        return;
    }
    unsigned long long* sums = tmp;
    unsigned long long* sums_scan = tmp + tiles;
    { k_scan_tiles<<<unsigned(tiles), 1024, 0, st>>>(in, n, out, sums); note_launch(); }
    scan_u64(sums, tiles, sums_scan, tmp + 2 * tiles, st);
    { k_scan_add<<<unsigned(tiles), 1024, 0, st>>>(out, n, sums_scan); note_launch(); }
}

size_t assemble_tmp_bytes(idx_t num_reads) {
    size_t n = size_t(num_reads) + 1, total = n;   // counts
    size_t t = (n + 1023) / 1024;
    while (t > 1) { total += 2 * t; t = (t + 1023) / 1024; }
    return (total + 64) * sizeof(unsigned long long);
}

__global__ void k_gather_edges(const SearchOut O, idx_t n, const unsigned long long* off, idx_t* dest,
                               uint16_t* len, uint8_t* type, int32_t* trans) {
    const size_t stride = size_t(gridDim.x) * blockDim.x;
    for (size_t r = size_t(blockIdx.x) * blockDim.x + threadIdx.x; r < n; r += stride) {
        unsigned long long o = off[r], m = off[r + 1] - o, s = O.edge_src[r];
        for (unsigned long long j = 0; j < m; ++j) {
            dest[o + j] = O.e_dest[s + j];
            len[o + j] = O.e_len[s + j];
            type[o + j] = O.e_type[s + j];
            trans[o + j] = O.e_trans[s + j];
        }
    }
}

cudaError_t assemble_counts_total(const SearchOut& o, idx_t num_reads, unsigned long long* out_off, void* scan_tmp,
                                  size_t scan_tmp_bytes, cudaStream_t st) {
    const size_t n = size_t(num_reads);
    if (scan_tmp_bytes < assemble_tmp_bytes(num_reads)) return cudaErrorInvalidValue;
    unsigned long long* cnt = reinterpret_cast<unsigned long long*>(scan_tmp);
    unsigned long long* tmp = cnt + n + 1;
    cudaMemsetAsync(cnt, 0, (n + 1) * sizeof(unsigned long long), st);
    unsigned g = unsigned(std::min<size_t>((n + 255) / 256 + 1, 152 * 32));
    if (n) { k_edge_counts<<<g, 256, 0, st>>>(o.num_B, o.num_F, idx_t(n), cnt); note_launch(); }
    scan_u64(cnt, n + 1, out_off, tmp, st);
    return cudaGetLastError();
}

cudaError_t assemble_gather(const SearchOut& o, idx_t num_reads, const unsigned long long* off, idx_t* dest,
                            uint16_t* len, uint8_t* type, int32_t* trans, cudaStream_t st) {
    const size_t n = size_t(num_reads);
    unsigned g = unsigned(std::min<size_t>((n + 255) / 256 + 1, 152 * 32));
    if (n) { k_gather_edges<<<g, 256, 0, st>>>(o, idx_t(n), off, dest, len, type, trans); note_launch(); }
    return cudaGetLastError();
}

const size_t kCandBytes = sizeof(Cand);
const size_t kFrameBytes = sizeof(Frame);

}  // namespace pq
