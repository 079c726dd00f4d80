// pq_seeds.cu — the per-read seed intervals the reference's suffix sort records as a side effect
// (index_t.interval_start / interval_end / interval_depth; src/sufsort.c:178-209, 322-334),
// computed from a finished suffix array.
//
// The reference sorts each slot by counting passes on triplets at depths 3 and 6, then recurses
// from depth 9 (process_slot_1) three bases at a time; a bucket holding suffixes that share D
// bases is recursed into when it has more than one suffix, except that a bucket whose size times
// (L - D + 3) is below INSERT_SORT_SIZE (3500, src/common.h:57) is finished by insertion sort
// instead.  Whenever a bucket of depth D <= t is visited -- by the recursion or by the insertion
// sort -- every suffix in it that is exactly D bases long (the last D bases of its read) records
// the bucket as its read's seed, if D is deeper than the read's seed so far.  So read r's seed is
// the deepest such D together with the bucket's first row and size.
//
// Given the suffix array, bucket structure is a question of longest common prefixes: the rows of
// one depth-D bucket are a run of rows in which consecutive suffixes share at least D bases.  This
// file computes the common prefix of every pair of adjacent rows (capped at the deepest depth
// that matters, 3 * floor(t / 3)) and then walks the depths 9, 12, ... once each over the rows,
// level by level, carrying one flag per row: "this row's bucket at the previous depth was
// recursed into".  A bucket at depth D is visited when its parent was recursed into and it holds
// more than one suffix; it is recursed into itself when it was visited and (D == 9 or its size
// times (L - D + 3) is at least 3500, in the index width's unsigned arithmetic, as the
// reference's test wraps).  Within one depth every read has at most one suffix of that length, so
// records need no atomics; the depths run in increasing order, so the deepest record wins.
//
// Buckets never span the reference's five sort slots (they share at least 3 bases), so running
// this over the rows of one slot gives exactly the records that slot's suf_sort call makes.
#include "pq_index.cuh"

namespace pq {

namespace {

constexpr size_t kSeedChunk = 2048;          // rows per warp work item (a multiple of 32)
constexpr idx_t kInsertSortSize = 3500;      // INSERT_SORT_SIZE

__device__ __forceinline__ uint64_t seed_window(const uint64_t* __restrict__ pk, size_t p) {
    const size_t w = p >> 5;
    const int s = int(p & 31) * 2;
    const uint64_t a = __ldg(pk + w), b = __ldg(pk + w + 1);
    return s ? ((a << s) | (b >> (64 - s))) : a;
}

// lcp[i - r0] = bases shared by the suffixes at rows i - 1 and i, at most `cap` (0 for i = r0)
__global__ void k_seed_lcp(const idx_t* __restrict__ sa, const uint64_t* __restrict__ pk, idx_t L, size_t r0,
                           size_t r1, int cap, uint16_t* __restrict__ lcp) {
    for (size_t i = r0 + size_t(blockIdx.x) * blockDim.x + threadIdx.x; i < r1;
         i += size_t(gridDim.x) * blockDim.x) {
        if (i == r0) {
            lcp[0] = 0;
            continue;
        }
        const idx_t p = __ldg(sa + i - 1), q = __ldg(sa + i);
        const int lp = int(L - p % L), lq = int(L - q % L);
        int m = lp < lq ? lp : lq;
        m = m < cap ? m : cap;
        int c = 0;
        while (c < m) {
            const uint64_t x = seed_window(pk, size_t(p) + c) ^ seed_window(pk, size_t(q) + c);
            if (x) {
                c += __clzll((long long)x) >> 1;
                break;
            }
            c += 32;
        }
        lcp[i - r0] = uint16_t(c < m ? c : m);
    }
}

// One depth D over rows [r0, r1): every bucket (run of rows sharing D bases) that starts in an
// active chunk is handled by the warp owning that chunk (it scans on past the chunk for the end).
// proc[row - r0] != 0: the row's bucket at depth D - 3 was recursed into (all rows at D = 9).
__global__ void k_seed_level(const uint16_t* __restrict__ lcp, const idx_t* __restrict__ sa, idx_t L, int t, int D,
                             size_t r0, size_t r1, uint8_t* __restrict__ proc, const uint8_t* __restrict__ act_in,
                             uint8_t* __restrict__ act_out, uint16_t* __restrict__ depth,
                             idx_t* __restrict__ start, idx_t* __restrict__ size) {
    const int lane = threadIdx.x & 31;
    const size_t gw = (size_t(blockIdx.x) * blockDim.x + threadIdx.x) >> 5;
    const size_t nw = (size_t(gridDim.x) * blockDim.x) >> 5;
    const size_t rows = r1 - r0;
    const size_t nchunks = (rows + kSeedChunk - 1) / kSeedChunk;
    for (size_t c = gw; c < nchunks; c += nw) {
        if (act_in && !act_in[c]) continue;
        const size_t c0 = r0 + c * kSeedChunk;
        const size_t c1 = c0 + kSeedChunk < r1 ? c0 + kSeedChunk : r1;
        for (size_t w0 = c0; w0 < c1; w0 += 32) {
            const size_t row = w0 + lane;
            const bool head = row < c1 && (row == r0 || lcp[row - r0] < D);
            unsigned m = __ballot_sync(0xffffffffu, head);
            while (m) {
                const size_t s = w0 + size_t(__ffs(m) - 1);
                m &= m - 1;
                // end of the bucket: the next head (in this window, or further on)
                size_t e;
                if (m) {
                    e = w0 + size_t(__ffs(m) - 1);
                } else {
                    e = r1;
                    for (size_t x = w0 + 32; x < r1; x += 32) {
                        const size_t rr = x + lane;
                        const unsigned b = __ballot_sync(0xffffffffu, rr < r1 && lcp[rr - r0] < D);
                        if (b) {
                            e = x + size_t(__ffs(b) - 1);
                            break;
                        }
                    }
                }
                if (D > 9 && !proc[s - r0]) continue;    // the parent bucket was not recursed into
                const idx_t n = idx_t(e - s);
                const bool visited = n > 1;
                const bool recurse = visited && (D == 9 || idx_t(n * idx_t(L - (D - 3))) >= kInsertSortSize);
                for (size_t x = s + lane; x < e; x += 32) {
                    if (visited && D <= t) {
                        const idx_t p = __ldg(sa + x);
                        if (int(L - p % L) == D) {
                            const idx_t r = p / L;
                            if (depth[r] < D) {
                                depth[r] = uint16_t(D);
                                start[r] = idx_t(s);
                                size[r] = n;
                            }
                        }
                    }
                    proc[x - r0] = recurse ? 1 : 0;
                    if (recurse) act_out[(x - r0) / kSeedChunk] = 1;
                }
            }
        }
    }
}

// the seed every read starts from in build_idx (src/index.c:495-502, 548-555): the interval of its
// last base (forward) or first base (backward) by C[], depth 1
struct SeedC {
    idx_t c[6];
};
__global__ void k_seed_init(const uint8_t* __restrict__ reads, idx_t num_reads, idx_t L, int dir, SeedC C,
                            uint16_t* __restrict__ depth, idx_t* __restrict__ start, idx_t* __restrict__ size) {
    for (size_t r = size_t(blockIdx.x) * blockDim.x + threadIdx.x; r < size_t(num_reads);
         r += size_t(gridDim.x) * blockDim.x) {
        const int ch = reads[r * size_t(L) + (dir ? 0 : size_t(L) - 1)];
        start[r] = C.c[ch];
        size[r] = C.c[ch + 1] - C.c[ch];
        depth[r] = 1;
    }
}

int grid_for_rows(size_t n, int per_block) {
    size_t g = (n + per_block - 1) / per_block;
    if (g > 152 * 64) g = 152 * 64;
    return int(g ? g : 1);
}

}  // namespace

cudaError_t seed_init(const uint8_t* reads, idx_t num_reads, idx_t L, int dir, const idx_t C[6], uint16_t* depth,
                      idx_t* start, idx_t* size, cudaStream_t st) {
    if (!num_reads) return cudaSuccess;
    SeedC c;
    for (int i = 0; i < 6; ++i) c.c[i] = C[i];
    k_seed_init<<<grid_for_rows(num_reads, 256), 256, 0, st>>>(reads, num_reads, L, dir, c, depth, start, size);
    note_launch();
    return cudaGetLastError();
}

size_t sort_seeds_tmp_bytes(size_t rows) {
    const size_t nchunks = (rows + kSeedChunk - 1) / kSeedChunk;
    auto al = [](size_t b) { return (b + 255) & ~size_t(255); };
    return al(rows * sizeof(uint16_t)) + al(rows) + 2 * al(nchunks) + 256;
}

cudaError_t sort_seeds(const idx_t* sa, const uint64_t* pk, idx_t L, int t, size_t r0, size_t r1, uint16_t* depth,
                       idx_t* start, idx_t* size, void* tmp, size_t tmp_bytes, cudaStream_t st) {
    if (r1 <= r0 || t < 9) return cudaSuccess;
    const size_t rows = r1 - r0;
    if (tmp_bytes < sort_seeds_tmp_bytes(rows)) return cudaErrorInvalidValue;
    const size_t nchunks = (rows + kSeedChunk - 1) / kSeedChunk;
    auto al = [](size_t b) { return (b + 255) & ~size_t(255); };
    char* p = static_cast<char*>(tmp);
    uint16_t* lcp = reinterpret_cast<uint16_t*>(p);
    p += al(rows * sizeof(uint16_t));
    uint8_t* proc = reinterpret_cast<uint8_t*>(p);
    p += al(rows);
    uint8_t* act[2] = {reinterpret_cast<uint8_t*>(p), reinterpret_cast<uint8_t*>(p + al(nchunks))};
    const int dmax = 3 * (t / 3);
    k_seed_lcp<<<grid_for_rows(rows, 256), 256, 0, st>>>(sa, pk, L, r0, r1, dmax, lcp);
    note_launch();
    const int warps_per_block = 8;
    const int blocks = grid_for_rows(nchunks, warps_per_block);
    int cur = 0;
    for (int D = 9; D <= dmax; D += 3) {
        cudaError_t e = cudaMemsetAsync(act[cur], 0, nchunks, st);
        if (e != cudaSuccess) return e;
        k_seed_level<<<blocks, 32 * warps_per_block, 0, st>>>(lcp, sa, L, t, D, r0, r1, proc,
                                                               D == 9 ? nullptr : act[cur ^ 1], act[cur], depth,
                                                               start, size);
        note_launch();
        cur ^= 1;
    }
    return cudaGetLastError();
}

}  // namespace pq
