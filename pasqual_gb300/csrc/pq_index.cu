// pq_index.cu — FM-index construction from a suffix array (both directions).
//
// Replaces the BWT/occurrence-table build of the reference: build_OCC (src/index.c:26-142), the
// occ prefix sum (src/index.c:587-615), C[] and the prefix/suffix counts (src/index.c:336-372).
// The reference fills five per-symbol bitmaps plus 5 counts per 64 rows; here one 32-byte occ
// block per 64 rows holds everything a rank query needs (see pq_common.cuh), and the
// reference-layout arrays are produced from it on demand for the drop-in host interface.
#include "pq_index.cuh"
#include "pq_sort.cuh"

#include <algorithm>

namespace pq {

// Text character at position p (codes 1..4).  dir 1 = every read reversed in place, the text
// transform_to_triplet_reverse sorts (src/sufsort.c:80-121).
__device__ __forceinline__ int text_at(const uint8_t* __restrict__ reads, idx_t L, int dir, idx_t p) {
    if (dir == 0) return reads[p];
    idx_t r = p / L, off = p - r * L;
    return reads[r * L + (L - 1 - off)];
}

// Base code (1..4) at position p of the packed text of a direction (32 bases per word, first base
// in the top two bits).
__device__ __forceinline__ int packed_at(const uint64_t* __restrict__ pk, size_t p) {
    return int((pk[p >> 5] >> (62 - 2 * int(p & 31))) & 3) + 1;
}

// One warp per 64-row block: BWT symbol of each row (`$` for a read-start suffix, else the
// preceding base), packed into lo/hi/dol masks with ballots; per-block symbol counts go into
// cnt[] for the superblock pass.  A row's symbol comes from the sort's hints when it left one
// (hint != 0xff: the rows its group refinement placed), else from the packed text when given (a
// quarter of the bytes of the text, so more of it stays in L2), else from the text.
__global__ void k_bwt_blocks(const idx_t* __restrict__ sa, const uint8_t* __restrict__ reads,
                             const uint64_t* __restrict__ pk, const uint8_t* __restrict__ hint, idx_t n, idx_t L,
                             int dir, idx_t nblk, OccBlock* __restrict__ blk) {
    constexpr int G = 4;                    // blocks per warp and round: 8 independent rows per lane
    const int lane = threadIdx.x & 31;
    const size_t warp = (size_t(blockIdx.x) * blockDim.x + threadIdx.x) >> 5;
    const size_t nwarps = (size_t(gridDim.x) * blockDim.x) >> 5;
    for (size_t b0 = warp * G; b0 < nblk; b0 += nwarps * G) {
        int sym[2 * G];
        #pragma unroll
        for (int x = 0; x < 2 * G; ++x) {
            const size_t r = b0 * 64 + size_t(x) * 32 + lane;
            sym[x] = r < n ? (hint ? int(hint[r]) : 0xff) : -1;
        }
        idx_t p[2 * G];
        #pragma unroll
        for (int x = 0; x < 2 * G; ++x) {
            const size_t r = b0 * 64 + size_t(x) * 32 + lane;
            p[x] = sym[x] == 0xff ? sa[r] : idx_t(0);
        }
        #pragma unroll
        for (int x = 0; x < 2 * G; ++x) {
            if (sym[x] == 0xff) {
                const idx_t off = p[x] % L;
                sym[x] = off ? (pk ? packed_at(pk, size_t(p[x]) - 1) : text_at(reads, L, dir, p[x] - 1)) : 0;
            }
        }
        #pragma unroll
        for (int g = 0; g < G; ++g) {
            if (b0 + g >= nblk) break;
            uint32_t lo2[2], hi2[2], dl2[2], va2[2];
            #pragma unroll
            for (int h = 0; h < 2; ++h) {
                const int sy = sym[2 * g + h];
                const int code = sy > 0 ? sy - 1 : 0;
                lo2[h] = __ballot_sync(0xffffffffu, code & 1);
                hi2[h] = __ballot_sync(0xffffffffu, code >> 1);
                dl2[h] = __ballot_sync(0xffffffffu, sy == 0);
                va2[h] = __ballot_sync(0xffffffffu, sy >= 0);
            }
            if (lane == 0) {
                OccBlock ob;
                ob.lo = uint64_t(lo2[0]) | (uint64_t(lo2[1]) << 32);
                ob.hi = uint64_t(hi2[0]) | (uint64_t(hi2[1]) << 32);
                ob.dol = uint64_t(dl2[0]) | (uint64_t(dl2[1]) << 32);
                const uint64_t valid = uint64_t(va2[0]) | (uint64_t(va2[1]) << 32);
                const uint64_t base = valid & ~ob.dol;
                ob.cnt[0] = (uint16_t)__popcll(base & ~ob.hi & ~ob.lo);
                ob.cnt[1] = (uint16_t)__popcll(base & ~ob.hi & ob.lo);
                ob.cnt[2] = (uint16_t)__popcll(base & ob.hi & ~ob.lo);
                ob.cnt[3] = (uint16_t)__popcll(base & ob.hi & ob.lo);
                blk[b0 + g] = ob;
            }
        }
    }
}

// One CTA (256 threads x 4 blocks) per superblock: in-superblock exclusive prefix of the block
// counts, written back as the blocks' relative counts; superblock totals to sbtot.
__global__ void k_super_prefix(OccBlock* __restrict__ blk, idx_t nblk, idx_t* __restrict__ sbtot) {
    __shared__ uint32_t warp_tot[8][4];
    const size_t s = blockIdx.x;
    const int tid = threadIdx.x, lane = tid & 31, wid = tid >> 5;
    const size_t b0 = s * kBlocksPerSuper + size_t(tid) * 4;
    uint32_t c[4][4];
    uint32_t mine[4] = {0, 0, 0, 0};
    #pragma unroll
    for (int i = 0; i < 4; ++i) {
        size_t b = b0 + i;
        #pragma unroll
        for (int k = 0; k < 4; ++k) c[i][k] = 0;
        if (b < nblk) {
            uint2 w = *reinterpret_cast<const uint2*>(&blk[b].cnt[0]);
            c[i][0] = w.x & 0xffff; c[i][1] = w.x >> 16; c[i][2] = w.y & 0xffff; c[i][3] = w.y >> 16;
        }
        #pragma unroll
        for (int k = 0; k < 4; ++k) mine[k] += c[i][k];
    }
    // warp inclusive scan of the per-thread totals, per symbol
    uint32_t incl[4];
    #pragma unroll
    for (int k = 0; k < 4; ++k) {
        uint32_t v = mine[k];
        #pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            uint32_t y = __shfl_up_sync(0xffffffffu, v, o);
            if (lane >= o) v += y;
        }
        incl[k] = v;
        if (lane == 31) warp_tot[wid][k] = v;
    }
    __syncthreads();
    uint32_t run[4];
    #pragma unroll
    for (int k = 0; k < 4; ++k) {
        uint32_t before = 0;
        for (int w = 0; w < wid; ++w) before += warp_tot[w][k];
        run[k] = before + incl[k] - mine[k];
    }
    #pragma unroll
    for (int i = 0; i < 4; ++i) {
        size_t b = b0 + i;
        if (b < nblk) {
            uint2 w;
            w.x = run[0] | (run[1] << 16);
            w.y = run[2] | (run[3] << 16);
            *reinterpret_cast<uint2*>(&blk[b].cnt[0]) = w;
        }
        #pragma unroll
        for (int k = 0; k < 4; ++k) run[k] += c[i][k];
    }
    if (tid == 255) {
        #pragma unroll
        for (int k = 0; k < 4; ++k) sbtot[s * 4 + k] = idx_t(run[k]);
    }
}

// Single CTA: exclusive scan of superblock totals (in place), per symbol.
__global__ void k_super_scan(idx_t* __restrict__ sb, size_t nsb) {
    __shared__ idx_t carry[4];
    __shared__ idx_t part[1024][4];
    const int tid = threadIdx.x;
    if (tid < 4) carry[tid] = 0;
    __syncthreads();
    for (size_t base = 0; base < nsb; base += 1024) {
        size_t s = base + tid;
        idx_t v[4];
        #pragma unroll
        for (int k = 0; k < 4; ++k) v[k] = s < nsb ? sb[s * 4 + k] : 0;
        #pragma unroll
        for (int k = 0; k < 4; ++k) part[tid][k] = v[k];
        __syncthreads();
        // Hillis-Steele inclusive scan over 1024 entries
        for (int o = 1; o < 1024; o <<= 1) {
            idx_t t[4];
            #pragma unroll
            for (int k = 0; k < 4; ++k) t[k] = tid >= o ? part[tid - o][k] : 0;
            __syncthreads();
            #pragma unroll
            for (int k = 0; k < 4; ++k) part[tid][k] += t[k];
            __syncthreads();
        }
        if (s < nsb) {
            #pragma unroll
            for (int k = 0; k < 4; ++k) sb[s * 4 + k] = carry[k] + part[tid][k] - v[k];
        }
        __syncthreads();
        if (tid < 4) carry[tid] += part[1023][tid];
        __syncthreads();
    }
}

// reads_index (src/index.c:71-79): read id of every `$` row, in row order.
__global__ void k_reads_index(const idx_t* __restrict__ sa, const OccBlock* __restrict__ blk,
                              const idx_t* __restrict__ sb, idx_t n, idx_t L, idx_t nblk,
                              idx_t* __restrict__ reads_index) {
    const int lane = threadIdx.x & 31;
    const size_t warp = (size_t(blockIdx.x) * blockDim.x + threadIdx.x) >> 5;
    const size_t nwarps = (size_t(gridDim.x) * blockDim.x) >> 5;
    for (size_t b = warp; b < nblk; b += nwarps) {
        OccBlock ob = blk[b];
        if (!ob.dol) continue;
        const idx_t* s4 = sb + (b >> (kSuperShift - kBlockShift)) * 4;
        idx_t row0 = idx_t(b * 64);
        idx_t before = row0 - (s4[0] + s4[1] + s4[2] + s4[3] +
                               idx_t(ob.cnt[0]) + ob.cnt[1] + ob.cnt[2] + ob.cnt[3]);
        #pragma unroll
        for (int h = 0; h < 2; ++h) {
            int j = h * 32 + lane;
            if ((ob.dol >> j) & 1) {
                uint64_t below = j ? (ob.dol & ((uint64_t(1) << j) - 1)) : 0;
                idx_t k = before + idx_t(__popcll(below));
                reads_index[k] = sa[row0 + j] / L;
            }
        }
    }
}

// Read statistics: C[] (src/index.c:367-372), suffix_count / prefix_count (src/index.c:336-346),
// and the number of bytes that are not base codes 1..4.  The base counts stream the read set
// 16 bytes a thread at a time (coalesced); the first and last base of every read are a strided
// pass over the reads.
__device__ __forceinline__ void count_word(uint32_t w, unsigned (&loc)[5]) {
    // per code c: the bytes of w equal to c (per-byte compare masks, 8 bits a match)
    unsigned hit = 0;
    #pragma unroll
    for (int c = 1; c <= 4; ++c) {
        const unsigned h = uint32_t(__popc(__vcmpeq4(w, 0x01010101u * unsigned(c)))) >> 3;
        loc[c - 1] += h;
        hit += h;
    }
    loc[4] += 4 - hit;
}

__global__ void k_read_counts(const uint8_t* __restrict__ reads, idx_t nr, idx_t L,
                              unsigned long long* __restrict__ out /* base[4], sfx[4], pfx[4], bad */) {
    __shared__ unsigned long long acc[13];
    if (threadIdx.x < 13) acc[threadIdx.x] = 0;
    __syncthreads();
    unsigned loc[5] = {0, 0, 0, 0, 0};                  // per thread: < 2^32 bytes each
    unsigned long long ends[8] = {0, 0, 0, 0, 0, 0, 0, 0};
    const size_t n = size_t(nr) * size_t(L);
    const size_t tid = size_t(blockIdx.x) * blockDim.x + threadIdx.x;
    const size_t stride = size_t(gridDim.x) * blockDim.x;
    const size_t n16 = reinterpret_cast<uintptr_t>(reads) % 16 == 0 ? n / 16 : 0;
    const uint4* v = reinterpret_cast<const uint4*>(reads);
    for (size_t i = tid; i < n16; i += stride) {
        const uint4 q = v[i];
        count_word(q.x, loc);
        count_word(q.y, loc);
        count_word(q.z, loc);
        count_word(q.w, loc);
    }
    for (size_t i = n16 * 16 + tid; i < n; i += stride) {
        const uint32_t c = reads[i];
        #pragma unroll
        for (int k = 1; k <= 4; ++k) loc[k - 1] += c == uint32_t(k);
        loc[4] += c < 1u || c > 4u;
    }
    for (size_t r = tid; r < size_t(nr); r += stride) {
        const uint32_t last = reads[r * L + L - 1], first = reads[r * L];
        #pragma unroll
        for (int c = 1; c <= 4; ++c) {
            ends[c - 1] += last == uint32_t(c);
            ends[4 + c - 1] += first == uint32_t(c);
        }
    }
    #pragma unroll
    for (int k = 0; k < 4; ++k) if (loc[k]) atomicAdd(&acc[k], (unsigned long long)loc[k]);
    #pragma unroll
    for (int k = 0; k < 8; ++k) if (ends[k]) atomicAdd(&acc[4 + k], ends[k]);
    if (loc[4]) atomicAdd(&acc[12], (unsigned long long)loc[4]);
    __syncthreads();
    if (threadIdx.x < 13 && acc[threadIdx.x]) atomicAdd(&out[threadIdx.x], acc[threadIdx.x]);
}

// k-mer table from the packed text, one pass: a warp takes 32 consecutive rows, each lane the
// k-mer of its row's suffix (all-ones when shorter than k) from one 64-bit window of the packed
// text; neighbours' k-mers come by shuffle (the warp's edge lanes fetch theirs).
__device__ __forceinline__ uint32_t kmer_at(const idx_t* __restrict__ sa, const uint64_t* __restrict__ pk,
                                            size_t r, idx_t L, int k) {
    const size_t p = size_t(sa[r]);
    const idx_t off = idx_t(p % size_t(L));
    if (L - off < idx_t(k)) return 0xffffffffu;
    const size_t w = p >> 5;
    const int sh = int(p & 31) * 2;
    const uint64_t x = sh ? ((pk[w] << sh) | (pk[w + 1] >> (64 - sh))) : pk[w];
    return uint32_t(x >> (64 - 2 * k));
}

__global__ void k_kmer_bounds_pk(const idx_t* __restrict__ sa, const uint64_t* __restrict__ pk, size_t n, idx_t L,
                                 int k, idx_t* __restrict__ kstart, idx_t* __restrict__ kend) {
    const int lane = threadIdx.x & 31;
    const size_t warp = (size_t(blockIdx.x) * blockDim.x + threadIdx.x) >> 5;
    const size_t nwarps = (size_t(gridDim.x) * blockDim.x) >> 5;
    for (size_t base = warp * 32; base < n; base += nwarps * 32) {
        const size_t r = base + lane;
        const uint32_t c = r < n ? kmer_at(sa, pk, r, L, k) : 0xffffffffu;
        uint32_t prev = __shfl_up_sync(0xffffffffu, c, 1);
        uint32_t next = __shfl_down_sync(0xffffffffu, c, 1);
        if (lane == 0) prev = r > 0 && r < n ? kmer_at(sa, pk, r - 1, L, k) : 0xfffffffeu;
        if (lane == 31) next = r + 1 < n ? kmer_at(sa, pk, r + 1, L, k) : 0xfffffffeu;
        if (r < n && c != 0xffffffffu) {
            if (r == 0 || prev != c) kstart[c] = idx_t(r);
            if (r + 1 == n || next != c) kend[c] = idx_t(r);
        }
    }
}

// k-mer table straight from the sorted suffix keys (first 14 bases in bits 31..4, min(length, 14)
// in bits 3..0), read in order: a row's k-mer is the key's top 2k bits when the suffix has k bases
__device__ __forceinline__ uint32_t key_code(uint32_t key, int k) {
    return int(key & 15) >= k ? (key >> (32 - 2 * k)) : 0xffffffffu;
}

// four rows a thread from one 16-byte load (the key array starts 16-byte aligned), plus the
// neighbours on either side; key[i] is the key of row off + i (the keys of one chunk of a chunked
// sort: for k >= 6 a k-mer's rows share one 6-base bucket of that sort, so never span two chunks)
__global__ void k_kmer_bounds_keys(const uint32_t* __restrict__ key, idx_t n, int k, idx_t* __restrict__ kstart,
                                   idx_t* __restrict__ kend, size_t off) {
    const size_t stride = size_t(gridDim.x) * blockDim.x;
    const size_t nn = size_t(n);
    for (size_t q = size_t(blockIdx.x) * blockDim.x + threadIdx.x; 4 * q < nn; q += stride) {
        const size_t r0 = 4 * q;
        uint32_t c[6];                               // rows r0 - 1 .. r0 + 4
        if (r0 + 4 <= nn) {
            const uint4 v = *reinterpret_cast<const uint4*>(key + r0);
            c[1] = key_code(v.x, k);
            c[2] = key_code(v.y, k);
            c[3] = key_code(v.z, k);
            c[4] = key_code(v.w, k);
        } else {
            #pragma unroll
            for (int u = 0; u < 4; ++u) c[1 + u] = r0 + u < nn ? key_code(key[r0 + u], k) : 0xfffffffeu;
        }
        c[0] = r0 > 0 ? key_code(key[r0 - 1], k) : 0xfffffffeu;
        c[5] = r0 + 4 < nn ? key_code(key[r0 + 4], k) : 0xfffffffeu;
        #pragma unroll
        for (int u = 1; u <= 4; ++u) {
            const size_t r = r0 + u - 1;
            if (r >= nn || c[u] == 0xffffffffu) continue;
            if (c[u - 1] != c[u]) kstart[c[u]] = idx_t(off + r);
            if (c[u + 1] != c[u]) kend[c[u]] = idx_t(off + r);
        }
    }
}


// inverse suffix array restricted to read offsets 1..M: isa[read * M + offset - 1] = row of the
// suffix at that offset (the rows the interval scan looks up: suffixes of length L - M .. L - 1)
// hint (or null): the sort's BWT symbols; rows with one (!= 0xff) already have their entry
__global__ void k_isa(const idx_t* __restrict__ sa, size_t n, idx_t L, idx_t M, idx_t* __restrict__ isa,
                      const uint8_t* __restrict__ hint) {
    const size_t stride = size_t(gridDim.x) * blockDim.x;
    for (size_t r = size_t(blockIdx.x) * blockDim.x + threadIdx.x; r < n; r += stride) {
        if (hint && hint[r] != 0xff) continue;
        const idx_t p = sa[r];
        const idx_t rd = p / L, off = p - rd * L;
        if (off >= 1 && off <= M) isa[size_t(rd) * M + (off - 1)] = idx_t(r);
    }
}

__global__ void k_fill_idx(idx_t* __restrict__ a, size_t m, idx_t v) {
    const size_t stride = size_t(gridDim.x) * blockDim.x;
    for (size_t i = size_t(blockIdx.x) * blockDim.x + threadIdx.x; i < m; i += stride) a[i] = v;
}

// Reference-layout export (src/index.h:26-30): bitmap[c] word b bit j+1 <=> BWT[64b+j] == c for
// j <= 62, and sample[5b+c] = fix[c] + #c in BWT[0, 64b) (fix[0] = 0).
__global__ void k_export_ref(const OccBlock* __restrict__ blk, const idx_t* __restrict__ sb,
                             idx_t n, idx_t nblk, idx_t f1, idx_t f2, idx_t f3, idx_t f4,
                             uint64_t* __restrict__ bitmap, idx_t* __restrict__ sample) {
    const size_t stride = size_t(gridDim.x) * blockDim.x;
    for (size_t b = size_t(blockIdx.x) * blockDim.x + threadIdx.x; b < nblk; b += stride) {
        OccBlock ob = blk[b];
        uint64_t valid = (size_t(n) >= (b + 1) * 64) ? ~uint64_t(0)
                       : (size_t(n) > b * 64 ? ((uint64_t(1) << (size_t(n) - b * 64)) - 1) : 0);
        uint64_t base = valid & ~ob.dol;
        uint64_t m[5];
        m[0] = ob.dol;
        m[1] = base & ~ob.hi & ~ob.lo;
        m[2] = base & ~ob.hi & ob.lo;
        m[3] = base & ob.hi & ~ob.lo;
        m[4] = base & ob.hi & ob.lo;
        #pragma unroll
        for (int c = 0; c < 5; ++c) bitmap[size_t(c) * nblk + b] = m[c] << 1;
        const idx_t* s4 = sb + (b >> (kSuperShift - kBlockShift)) * 4;
        idx_t r1 = s4[0] + ob.cnt[0], r2 = s4[1] + ob.cnt[1], r3 = s4[2] + ob.cnt[2], r4 = s4[3] + ob.cnt[3];
        idx_t row0 = idx_t(b * 64);
        sample[b * 5 + 0] = row0 - (r1 + r2 + r3 + r4);
        sample[b * 5 + 1] = f1 + r1;
        sample[b * 5 + 2] = f2 + r2;
        sample[b * 5 + 3] = f3 + r3;
        sample[b * 5 + 4] = f4 + r4;
    }
}

// Per-read seeds (index_t.interval_start/end/depth, src/index.h:36-41): forward = the read's
// last k bases, backward = its first k bases reversed; both exact SA intervals from the table.
__global__ void k_read_seeds(const uint8_t* __restrict__ reads, idx_t nr, int L, int dir, int k,
                             const idx_t* __restrict__ kstart, const idx_t* __restrict__ kend,
                             idx_t* __restrict__ start, idx_t* __restrict__ size) {
    const size_t stride = size_t(gridDim.x) * blockDim.x;
    for (size_t r = size_t(blockIdx.x) * blockDim.x + threadIdx.x; r < nr; r += stride) {
        const uint8_t* s = reads + r * size_t(L);
        uint32_t code = 0;
        for (int j = 0; j < k; ++j) {
            int c = dir == 0 ? s[L - k + j] : s[k - 1 - j];
            code = (code << 2) | uint32_t(c - 1);
        }
        start[r] = kstart[code];
        size[r] = kend[code] - kstart[code] + 1;
    }
}

static inline unsigned grid_for(size_t work, int threads, int per_sm = 8) {
    size_t g = (work + threads - 1) / threads;
    size_t cap = size_t(152) * per_sm * 4;
    if (g > cap) g = cap;
    if (g < 1) g = 1;
    return unsigned(g);
}

cudaError_t build_occ(const idx_t* sa, const uint8_t* reads, idx_t num_reads, idx_t L, int dir,
                      OccBlock* blk, idx_t* sb, idx_t* reads_index, cudaStream_t st, const uint64_t* pk,
                      const uint8_t* hint) {
    const size_t n = size_t(num_reads) * L;
    const size_t nblk = n / 64 + 1;
    const size_t nsb = (nblk + kBlocksPerSuper - 1) / kBlocksPerSuper;
    { k_bwt_blocks<<<grid_for(nblk * 32, 256), 256, 0, st>>>(sa, reads, pk, hint, idx_t(n), L, dir, idx_t(nblk), blk); note_launch(); }
    { k_super_prefix<<<unsigned(nsb), 256, 0, st>>>(blk, idx_t(nblk), sb); note_launch(); }
    { k_super_scan<<<1, 1024, 0, st>>>(sb, nsb); note_launch(); }
    { k_reads_index<<<grid_for(nblk * 32, 256), 256, 0, st>>>(sa, blk, sb, idx_t(n), L, idx_t(nblk), reads_index); note_launch(); }
    return cudaGetLastError();
}

// Copy of n bytes between page-locked host memory and device memory by a kernel (either side may
// be the host's, at its device-accessible address): four independent 16-byte accesses a thread,
// 32 CTAs per SM.  So many accesses in flight keep the copy at the link's rate right after a sort
// or a search over most of device memory, where a copy-engine cudaMemcpy from the same
// (cudaHostAlloc'd) buffer was measured at ~10 GB/s.  Bytes before the first 16-byte boundary
// and after the last go one by one; when the two sides are not equally aligned the whole copy
// goes byte by byte.
__global__ void __launch_bounds__(256) k_copy_bytes(uint8_t* __restrict__ dst, const uint8_t* __restrict__ src,
                                                    size_t n) {
    const size_t tid = size_t(blockIdx.x) * blockDim.x + threadIdx.x, stride = size_t(gridDim.x) * blockDim.x;
    const size_t mis = reinterpret_cast<uintptr_t>(src) & 15;
    if (mis != (reinterpret_cast<uintptr_t>(dst) & 15)) {
        for (size_t i = tid; i < n; i += stride) dst[i] = src[i];
        return;
    }
    const size_t head = mis ? (16 - mis < n ? 16 - mis : n) : 0;
    const size_t n16 = (n - head) / 16, tail = head + n16 * 16;
    if (tid < head) dst[tid] = src[tid];
    if (tid < n - tail) dst[tail + tid] = src[tail + tid];
    uint4* d = reinterpret_cast<uint4*>(dst + head);
    const uint4* s = reinterpret_cast<const uint4*>(src + head);
    size_t i = tid;
    for (; i + 3 * stride < n16; i += 4 * stride) {
        const uint4 a = s[i], b = s[i + stride], c = s[i + 2 * stride], e = s[i + 3 * stride];
        d[i] = a;
        d[i + stride] = b;
        d[i + 2 * stride] = c;
        d[i + 3 * stride] = e;
    }
    for (; i < n16; i += stride) d[i] = s[i];
}

cudaError_t kernel_copy(void* dst, const void* src, size_t n, cudaStream_t st) {
    if (!n) return cudaSuccess;
    int dev = 0, sms = 152;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    const size_t want = (n / 16 + 255) / 256;
    const unsigned blocks = unsigned(std::max<size_t>(1, std::min<size_t>(want, size_t(sms) * 32)));
    k_copy_bytes<<<blocks, 256, 0, st>>>(static_cast<uint8_t*>(dst), static_cast<const uint8_t*>(src), n);
    note_launch();
    return cudaGetLastError();
}

cudaError_t read_counts(const uint8_t* reads, idx_t num_reads, idx_t L, unsigned long long* out13,
                        cudaStream_t st) {
    cudaMemsetAsync(out13, 0, 13 * sizeof(unsigned long long), st);
    if (num_reads) { k_read_counts<<<grid_for(size_t(num_reads) * L / 16 + 1, 256), 256, 0, st>>>(reads, num_reads, L, out13); note_launch(); }
    return cudaGetLastError();
}

cudaError_t kmer_table_clear(int k, idx_t* kstart, idx_t* kend, cudaStream_t st) {
    const size_t nk = size_t(1) << (2 * k);
    { k_fill_idx<<<grid_for(nk, 256), 256, 0, st>>>(kstart, nk, idx_t(1)); note_launch(); }
    { k_fill_idx<<<grid_for(nk, 256), 256, 0, st>>>(kend, nk, idx_t(0)); note_launch(); }
    return cudaGetLastError();
}

cudaError_t kmer_table_from_keys(const uint32_t* keys, size_t m, size_t off, int k, idx_t* kstart, idx_t* kend,
                                 cudaStream_t st) {
    if (m) { k_kmer_bounds_keys<<<grid_for((m + 3) / 4, 256), 256, 0, st>>>(keys, idx_t(m), k, kstart, kend, off); note_launch(); }
    return cudaGetLastError();
}

cudaError_t build_kmer_table(const idx_t* sa, idx_t num_reads, idx_t L, int k, idx_t* kstart, idx_t* kend,
                             cudaStream_t st, const uint32_t* sorted_keys, const uint64_t* pk) {
    const size_t n = size_t(num_reads) * L;
    cudaError_t e = kmer_table_clear(k, kstart, kend, st);
    if (e != cudaSuccess) return e;
    if (n && sorted_keys && k <= kSortKeyBases && reinterpret_cast<uintptr_t>(sorted_keys) % 16 == 0) {
        return kmer_table_from_keys(sorted_keys, n, 0, k, kstart, kend, st);
    } else if (n) {
        { k_kmer_bounds_pk<<<grid_for(n, 256), 256, 0, st>>>(sa, pk, n, L, k, kstart, kend); note_launch(); }
    }
    return cudaGetLastError();
}

cudaError_t read_seeds(const uint8_t* reads, idx_t num_reads, int L, int dir, int k, const idx_t* kstart,
                       const idx_t* kend, idx_t* start, idx_t* size, cudaStream_t st) {
    if (num_reads)
        { k_read_seeds<<<grid_for(num_reads, 256), 256, 0, st>>>(reads, num_reads, L, dir, k, kstart, kend, start, size); note_launch(); }
    return cudaGetLastError();
}

cudaError_t build_isa(const idx_t* sa, size_t n, idx_t L, idx_t M, idx_t* isa, cudaStream_t st,
                      const uint8_t* hint) {
    if (n && M) { k_isa<<<grid_for(n, 256), 256, 0, st>>>(sa, n, L, M, isa, hint); note_launch(); }
    return cudaGetLastError();
}

cudaError_t export_ref_layout(const OccBlock* blk, const idx_t* sb, idx_t num_reads, idx_t L,
                              const idx_t fix[4], uint64_t* bitmap, idx_t* sample, cudaStream_t st) {
    const size_t n = size_t(num_reads) * L;
    const size_t nblk = n / 64 + 1;
    { k_export_ref<<<grid_for(nblk, 256), 256, 0, st>>>(blk, sb, idx_t(n), idx_t(nblk), fix[0], fix[1],
                                                      fix[2], fix[3], bitmap, sample); note_launch(); }
    return cudaGetLastError();
}

}  // namespace pq
