// pq_sort.cu — suffix sort of the reads (forward) or of the reversed reads (backward).
//
// Replaces transform_to_triplet[_reverse], initial_sort and suf_sort (src/sufsort.c:80-614) as
// driven by build_idx (src/index.c:558-585).  The reference sorts in 5 slots by an MSD counting
// sort on 3-character "triplet" ranks with insertion sort for small buckets; its single-threaded
// output order is: read-bounded suffix strings, end-of-read lowest, ties by text position.
//
// GB300 design: the text is packed 2 bits per base; every suffix gets a 32-bit key made of its
// first 14 bases (padded with A) and the number of those bases that exist (0..14) -- comparing
// (padded bases, length) is exactly the end-of-read-lowest order on the first 14 bases.  Four
// stable radix passes sort the keys; every group of equal keys whose suffixes go on past base 14
// is then finished where it lies (group refinement, below).  At read coverage c such a group
// holds about c suffixes of one genome locus whatever the key length, so a short key costs the
// refinement little and halves the radix passes of a 29-base key.  Every radix pass is stable and
// the input starts in text order, so equal suffixes stay in text order: the canonical tie-break.
// Inputs the refinement cannot finish (groups larger than its scratch, reads longer than
// 268 bases) are sorted by prefix doubling on 29-base 64-bit keys instead: ranks by
// (rank(p), rank(p+h) or "empty" past the read end) for h = 29, 58, 116, ...
#include "pq_sort.cuh"
#include "pq_index.cuh"

#include <algorithm>
#include <vector>

namespace pq {

constexpr int kHead = kSortKeyBases;     // bases per 32-bit head key (4 radix passes)
constexpr int kWide = 29;                 // bases per 64-bit key (big groups, prefix doubling)

// Key layouts: the bases (padded with A, first base highest) above the number of them that exist.
//   uint32_t: 14 bases in bits 31..4, length 0..14 in bits 3..0
//   uint64_t: 29 bases in bits 63..6, length 0..29 in bits 5..0
template <class K> struct KeyFmt;
template <> struct KeyFmt<uint32_t> {
    static constexpr int bases = kHead, len_bits = 4;
};
template <> struct KeyFmt<uint64_t> {
    static constexpr int bases = kWide, len_bits = 6;
};
template <class K>
__device__ __forceinline__ int key_len(K k) { return int(k & K((1u << KeyFmt<K>::len_bits) - 1)); }
constexpr int RS_THREADS = 256;
constexpr int RS_IPT = 8;
constexpr int RS_WARPS = RS_THREADS / 32;
constexpr int RS_MAX_CTAS = 152 * 4;

__host__ __device__ __forceinline__ size_t zmin(size_t a, size_t b) { return a < b ? a : b; }

static inline unsigned grid_for(size_t work, int threads, int per_sm = 8) {
    size_t g = (work + threads - 1) / threads;
    size_t cap = size_t(152) * per_sm * 4;
    return unsigned(std::max<size_t>(1, std::min(g, cap)));
}

// ------------------------------------------------------------------------------ packed text

// 32 bases per word, first base in the top two bits (A=0 .. T=3).  The forward text of a whole
// word comes in two 16-byte loads; the backward text walks the word's positions with one
// division for the first (the read offset then steps and wraps).
__global__ void k_pack_text(const uint8_t* __restrict__ reads, size_t n, idx_t L, int dir, size_t nwords,
                            uint64_t* __restrict__ pk) {
    const size_t stride = size_t(gridDim.x) * blockDim.x;
    const bool vec = dir == 0 && reinterpret_cast<uintptr_t>(reads) % 16 == 0;
    for (size_t w = size_t(blockIdx.x) * blockDim.x + threadIdx.x; w < nwords; w += stride) {
        const size_t p0 = w * 32;
        uint64_t v = 0;
        if (vec && p0 + 32 <= n) {
            const uint4 a = *reinterpret_cast<const uint4*>(reads + p0);
            const uint4 b = *reinterpret_cast<const uint4*>(reads + p0 + 16);
            const uint32_t q[8] = {a.x, a.y, a.z, a.w, b.x, b.y, b.z, b.w};
            #pragma unroll
            for (int i = 0; i < 8; ++i) {
                #pragma unroll
                for (int by = 0; by < 4; ++by) v = (v << 2) | uint64_t(((q[i] >> (8 * by)) & 0xffu) - 1);
            }
        } else if (p0 < n) {
            size_t r = p0 / size_t(L);
            idx_t off = idx_t(p0 - r * size_t(L));
            for (int j = 0; j < 32; ++j) {
                const size_t p = p0 + size_t(j);
                uint64_t c = 0;
                if (p < n) c = uint64_t((dir == 0 ? reads[p] : reads[r * size_t(L) + size_t(L - 1 - off)]) - 1);
                v = (v << 2) | c;
                if (++off == L) {
                    off = 0;
                    ++r;
                }
            }
        }
        pk[w] = v;
    }
}

__device__ __forceinline__ uint64_t window(const uint64_t* __restrict__ pk, size_t p) {
    size_t w = p >> 5;
    int s = int(p & 31) * 2;
    uint64_t a = pk[w];
    uint64_t b = pk[w + 1];
    return s ? ((a << s) | (b >> (64 - s))) : a;
}

// the key of a suffix whose bases start the 64-bit window x and of which m exist (m >= 0)
template <class K>
__device__ __forceinline__ K make_key(uint64_t x, int m) {
    constexpr int B = KeyFmt<K>::bases;
    const int w = m < B ? m : B;
    if (w <= 0) return K(0);
    const uint64_t top = x & (~uint64_t(0) << (64 - 2 * w));
    return K(K(top >> (64 - 8 * int(sizeof(K)))) | K(w));
}

template <class K>
__global__ void k_init_keys(const uint64_t* __restrict__ pk, size_t n, idx_t L, K* __restrict__ key,
                            idx_t* __restrict__ val) {
    const size_t stride = size_t(gridDim.x) * blockDim.x;
    for (size_t p = size_t(blockIdx.x) * blockDim.x + threadIdx.x; p < n; p += stride) {
        key[p] = make_key<K>(window(pk, p), int(L - idx_t(p % L)));
        val[p] = idx_t(p);
    }
}

// The 32-bit head keys four positions a thread: one division for the first position's read
// offset, the windows of all four from the same two packed-text words, and 16-byte stores of the
// keys (and of the values when they are 32-bit); the key and value arrays start 16-byte aligned.
__global__ void k_init_keys4(const uint64_t* __restrict__ pk, size_t n, idx_t L, uint32_t* __restrict__ key,
                             idx_t* __restrict__ val) {
    const size_t stride = size_t(gridDim.x) * blockDim.x;
    for (size_t q = size_t(blockIdx.x) * blockDim.x + threadIdx.x; 4 * q < n; q += stride) {
        const size_t p0 = 4 * q;
        int off = int(p0 % size_t(L));
        const size_t w = p0 >> 5;
        const uint64_t a = pk[w], b = pk[w + 1];
        uint32_t kk[4];
        idx_t vv[4];
        #pragma unroll
        for (int u = 0; u < 4; ++u) {
            const int s = int((p0 + u) & 31) * 2;
            const uint64_t x = s ? ((a << s) | (b >> (64 - s))) : a;
            kk[u] = make_key<uint32_t>(x, int(L) - off);
            vv[u] = idx_t(p0 + u);
            if (++off == int(L)) off = 0;
        }
        if (p0 + 4 <= n) {
            *reinterpret_cast<uint4*>(key + p0) = make_uint4(kk[0], kk[1], kk[2], kk[3]);
            if (sizeof(idx_t) == 4) {
                *reinterpret_cast<uint4*>(val + p0) = make_uint4(uint32_t(vv[0]), uint32_t(vv[1]), uint32_t(vv[2]),
                                                                 uint32_t(vv[3]));
            } else {
                #pragma unroll
                for (int u = 0; u < 4; ++u) val[p0 + u] = vv[u];
            }
        } else {
            for (int u = 0; p0 + u < n; ++u) {
                key[p0 + u] = kk[u];
                val[p0 + u] = vv[u];
            }
        }
    }
}

// ------------------------------------------------------------------------------ radix sort

// Digit histograms of all byte positions over the whole key array (order independent): a pass
// whose digit is constant over all keys is the identity and is skipped.
template <class K>
__global__ void k_digit_hist(const K* __restrict__ key, size_t n, unsigned long long* __restrict__ hist) {
    constexpr int D = int(sizeof(K));
    __shared__ unsigned int h[D][256];
    for (int i = threadIdx.x; i < D * 256; i += blockDim.x) (&h[0][0])[i] = 0;
    __syncthreads();
    const size_t stride = size_t(gridDim.x) * blockDim.x;
    for (size_t i = size_t(blockIdx.x) * blockDim.x + threadIdx.x; i < n; i += stride) {
        const K k = key[i];
        #pragma unroll
        for (int d = 0; d < D; ++d) atomicAdd(&h[d][(k >> (8 * d)) & 255], 1u);
    }
    __syncthreads();
    for (int i = threadIdx.x; i < D * 256; i += blockDim.x)
        if ((&h[0][0])[i]) atomicAdd(&hist[i], (unsigned long long)(&h[0][0])[i]);
}

template <class K>
__global__ void __launch_bounds__(RS_THREADS) k_rs_upsweep(const K* __restrict__ key, size_t n, int shift,
                                                           size_t part, unsigned long long* __restrict__ cnt) {
    __shared__ unsigned int h[RS_WARPS][256];
    const int warp = threadIdx.x >> 5;
    for (int i = threadIdx.x; i < RS_WARPS * 256; i += RS_THREADS) (&h[0][0])[i] = 0;
    __syncthreads();
    const size_t beg = size_t(blockIdx.x) * part;
    const size_t end = zmin(n, beg + part);
    for (size_t i = beg + threadIdx.x; i < end; i += RS_THREADS)
        atomicAdd(&h[warp][(key[i] >> shift) & 255], 1u);
    __syncthreads();
    for (int d = threadIdx.x; d < 256; d += RS_THREADS) {
        unsigned long long s = 0;
        #pragma unroll
        for (int w = 0; w < RS_WARPS; ++w) s += h[w][d];
        cnt[size_t(d) * gridDim.x + blockIdx.x] = s;
    }
}

// single-CTA exclusive scan of m 64-bit counts, in place: each of the 1024 threads sums one
// contiguous segment, the segment totals are scanned once, and each thread rewrites its segment
__global__ void k_scan_small(unsigned long long* __restrict__ a, size_t m) {
    __shared__ unsigned long long wsum[32];
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    const size_t seg = (m + 1023) / 1024;
    const size_t b = zmin(m, size_t(threadIdx.x) * seg), e = zmin(m, b + seg);
    unsigned long long mine = 0;
    for (size_t i = b; i < e; ++i) mine += a[i];
    unsigned long long x = mine;
    #pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        unsigned long long y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= o) x += y;
    }
    if (lane == 31) wsum[wid] = x;
    __syncthreads();
    if (wid == 0) {
        unsigned long long w = wsum[lane], z = w;
        #pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            unsigned long long y = __shfl_up_sync(0xffffffffu, z, o);
            if (lane >= o) z += y;
        }
        wsum[lane] = z - w;
    }
    __syncthreads();
    unsigned long long run = wsum[wid] + x - mine;
    for (size_t i = b; i < e; ++i) {
        unsigned long long v = a[i];
        a[i] = run;
        run += v;
    }
}

// 16-byte asynchronous global -> shared copies (bypassing registers and L1)
__device__ __forceinline__ void cp_async16(void* smem, const void* gmem) {
    const unsigned s = unsigned(__cvta_generic_to_shared(smem));
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(s), "l"(gmem) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
__device__ __forceinline__ void cp_async_wait_all() { asm volatile("cp.async.wait_group 0;\n" ::: "memory"); }

// Downsweep configuration: 512 threads (tiles of 4096) for 32-bit keys and values, whose tile,
// staging buffer and reorder buffer fit two CTAs per SM; 256 threads otherwise.
template <class K, class V>
struct RsCfg {
    static constexpr int threads = (sizeof(K) == 4 && sizeof(V) == 4) ? 512 : 256;
    static constexpr int tile = threads * RS_IPT;
    static constexpr int min_blocks = threads == 512 ? 2 : (sizeof(K) == 4 ? 4 : 3);   // CTAs per SM
};
constexpr int RS_TILE_MAX = 4096;           // parts are whole multiples of every tile size

// One CTA per contiguous part of the input, tiles in order.  Per tile: every thread takes its
// RS_IPT (key, value) pairs, from the staging buffer when the tile was prefetched there (whole,
// 16-byte aligned tiles: the next tile's copy runs while this one is ranked and written), else
// straight from global memory; each warp ranks its rows by digit (8 ballots per row give the lanes
// with the same digit; a per-warp count per digit in shared memory carries the rank from row to
// row), the tile is reordered by digit in shared memory and written out in runs per digit at the
// part's running digit offsets.
template <class K, class V>
__global__ void __launch_bounds__(RsCfg<K, V>::threads, RsCfg<K, V>::min_blocks)
k_rs_downsweep(const K* __restrict__ kin, const V* __restrict__ vin, K* __restrict__ kout, V* __restrict__ vout,
               size_t n, int shift, size_t part, const unsigned long long* __restrict__ offs, int staged) {
    constexpr int T = RsCfg<K, V>::threads;
    constexpr int TILE = RsCfg<K, V>::tile;
    constexpr int NW = T / 32;
    extern __shared__ __align__(16) unsigned char rs_smem[];
    K* stk = reinterpret_cast<K*>(rs_smem);                          // staging: keys, values
    V* stv = reinterpret_cast<V*>(stk + TILE);
    K* sk = reinterpret_cast<K*>(stv + TILE);                         // reorder buffer
    V* sv = reinterpret_cast<V*>(sk + TILE);
    unsigned (*wcnt)[256] = reinterpret_cast<unsigned (*)[256]>(sv + TILE);
    unsigned* tcount = &wcnt[NW][0];
    unsigned* dstart = tcount + 256;
    unsigned* wtot = dstart + 256;
    unsigned long long* base = reinterpret_cast<unsigned long long*>(wtot + 32);

    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const unsigned lt_mask = (1u << lane) - 1;
    for (int d = tid; d < 256; d += T) base[d] = offs[size_t(d) * gridDim.x + blockIdx.x];
    const size_t beg = size_t(blockIdx.x) * part;
    const size_t end = zmin(n, beg + part);
    auto prefetch = [&](size_t t) {
        constexpr int KC = TILE * int(sizeof(K)) / 16, VC = TILE * int(sizeof(V)) / 16;
        for (int i = tid; i < KC; i += T)
            cp_async16(reinterpret_cast<char*>(stk) + 16 * i, reinterpret_cast<const char*>(kin + t) + 16 * size_t(i));
        for (int i = tid; i < VC; i += T)
            cp_async16(reinterpret_cast<char*>(stv) + 16 * i, reinterpret_cast<const char*>(vin + t) + 16 * size_t(i));
        cp_async_commit();
    };
    if (staged && beg + TILE <= end) prefetch(beg);
    for (size_t t0 = beg; t0 < end; t0 += TILE) {
        for (int i = lane; i < 256; i += 32) wcnt[warp][i] = 0;
        K k[RS_IPT];
        V v[RS_IPT];
        unsigned int lr[RS_IPT];
        const int j0 = warp * 32 * RS_IPT + lane;
        const size_t row0 = t0 + j0;
        if (staged && t0 + TILE <= end) {
            cp_async_wait_all();
            __syncthreads();
            #pragma unroll
            for (int r = 0; r < RS_IPT; ++r) {
                k[r] = stk[j0 + r * 32];
                v[r] = stv[j0 + r * 32];
            }
            __syncthreads();                                    // the staging buffer is free again
            if (t0 + 2 * size_t(TILE) <= end) prefetch(t0 + TILE);
        } else {
            #pragma unroll
            for (int r = 0; r < RS_IPT; ++r) {
                const size_t idx = row0 + r * 32;
                k[r] = idx < end ? kin[idx] : K(0);
                v[r] = idx < end ? vin[idx] : V(0);
            }
            __syncwarp();
        }
        #pragma unroll
        for (int r = 0; r < RS_IPT; ++r) {
            const bool valid = row0 + r * 32 < end;
            const int d = valid ? int((k[r] >> shift) & 255) : -1;
            unsigned peers = __ballot_sync(0xffffffffu, valid);
            #pragma unroll
            for (int b = 0; b < 8; ++b) {
                unsigned bits = __ballot_sync(0xffffffffu, (d >> b) & 1);
                peers &= ((d >> b) & 1) ? bits : ~bits;
            }
            unsigned before = 0;
            if (valid) before = wcnt[warp][d];
            __syncwarp();
            if (valid && (peers & lt_mask) == 0) wcnt[warp][d] = before + __popc(peers);
            __syncwarp();
            lr[r] = before + __popc(peers & lt_mask);
        }
        __syncthreads();
        // per digit: warp prefixes and tile count
        for (int d = tid; d < 256; d += T) {
            unsigned run = 0;
            #pragma unroll
            for (int w = 0; w < NW; ++w) {
                unsigned c = wcnt[w][d];
                wcnt[w][d] = run;
                run += c;
            }
            tcount[d] = run;
        }
        __syncthreads();
        // exclusive scan of tcount over the 256 digits (one per thread of the first 8 warps)
        {
            unsigned v0 = 0, x = 0;
            if (tid < 256) {
                v0 = tcount[tid];
                x = v0;
                #pragma unroll
                for (int o = 1; o < 32; o <<= 1) {
                    unsigned y = __shfl_up_sync(0xffffffffu, x, o);
                    if (lane >= o) x += y;
                }
                if (lane == 31) wtot[warp] = x;
            }
            __syncthreads();
            if (tid < 256) {
                unsigned pre = 0;
                for (int w = 0; w < warp; ++w) pre += wtot[w];
                dstart[tid] = pre + x - v0;
            }
        }
        __syncthreads();
        #pragma unroll
        for (int r = 0; r < RS_IPT; ++r) {
            if (row0 + r * 32 < end) {
                const int d = int((k[r] >> shift) & 255);
                const unsigned pos = dstart[d] + wcnt[warp][d] + lr[r];
                sk[pos] = k[r];
                sv[pos] = v[r];
            }
        }
        __syncthreads();
        const int cnt = int(zmin(size_t(TILE), end - t0));
        for (int j = tid; j < cnt; j += T) {
            const K key = sk[j];
            int d = int((key >> shift) & 255);
            unsigned long long g = base[d] + (unsigned)(j - dstart[d]);
            kout[g] = key;
            vout[g] = sv[j];
        }
        __syncthreads();
        for (int d = tid; d < 256; d += T) base[d] += tcount[d];
        __syncthreads();
    }
}

template <class K, class V>
static size_t rs_down_smem() {
    constexpr int T = RsCfg<K, V>::threads, TILE = RsCfg<K, V>::tile;
    return 2 * size_t(TILE) * (sizeof(K) + sizeof(V)) + size_t(T / 32 + 2) * 256 * 4 + 32 * 4 + 256 * 8;
}

cudaError_t pack_text(const uint8_t* reads, size_t n, idx_t L, int dir, uint64_t* pk, cudaStream_t st) {
    const size_t nwords = n / 32 + 4;
    { k_pack_text<<<grid_for(nwords, 256), 256, 0, st>>>(reads, n, L, dir, nwords, pk); note_launch(); }
    return cudaGetLastError();
}

size_t radix_tmp_bytes(size_t n) {
    (void)n;
    return (size_t(256) * RS_MAX_CTAS + 8 * 256 + 64) * sizeof(unsigned long long);
}

template <class K, class V>
int radix_sort_pairs(K** k0, V** v0, K** k1, V** v1, size_t n, int lo_bit, int hi_bit, void* tmp,
                     size_t tmp_bytes, cudaStream_t st, bool skip_trivial) {
    constexpr int D = int(sizeof(K));
    if (hi_bit > 8 * D) hi_bit = 8 * D;
    if (n <= 1) return 0;
    if (tmp_bytes < radix_tmp_bytes(n)) return int(cudaErrorInvalidValue);
    unsigned long long* cnt = reinterpret_cast<unsigned long long*>(tmp);
    unsigned long long* gh = cnt + size_t(256) * RS_MAX_CTAS;
    std::vector<unsigned long long> h(size_t(D) * 256, 0);
    if (skip_trivial) {
        cudaMemsetAsync(gh, 0, 8 * 256 * sizeof(unsigned long long), st);
        { k_digit_hist<K><<<grid_for(n, 256, 4), 256, 0, st>>>(*k0, n, gh); note_launch(); }
        cudaMemcpyAsync(h.data(), gh, h.size() * sizeof(unsigned long long), cudaMemcpyDeviceToHost, st);
        cudaError_t e = cudaStreamSynchronize(st);
        if (e != cudaSuccess) return int(e);
    }
    size_t tiles = (n + RS_TILE_MAX - 1) / RS_TILE_MAX;
    // one wave of resident CTAs: as many per SM as the downsweep's shared memory and registers
    // allow (a grid sized for more ran a second, partial wave on a fraction of the SMs)
    const size_t smem = rs_down_smem<K, V>();
    cudaFuncSetAttribute(k_rs_downsweep<K, V>, cudaFuncAttributeMaxDynamicSharedMemorySize, int(smem));
    int dev = 0, sms = 152, per_sm = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_rs_downsweep<K, V>, RsCfg<K, V>::threads, smem) !=
            cudaSuccess || per_sm < 1) {
        cudaGetLastError();
        per_sm = 1;
    }
    size_t ctas = std::min<size_t>(tiles, std::min<size_t>(RS_MAX_CTAS, size_t(sms) * size_t(per_sm)));
    size_t part = ((tiles + ctas - 1) / ctas) * RS_TILE_MAX;
    ctas = (n + part - 1) / part;
    for (int d = lo_bit / 8; d * 8 < hi_bit; ++d) {
        bool trivial = false;
        for (int b = 0; b < 256; ++b)
            if (h[size_t(d) * 256 + b] == n) trivial = true;
        if (trivial) continue;
        { k_rs_upsweep<K><<<unsigned(ctas), RS_THREADS, 0, st>>>(*k0, n, 8 * d, part, cnt); note_launch(); }
        { k_scan_small<<<1, 1024, 0, st>>>(cnt, 256 * ctas); note_launch(); }
        // whole tiles are prefetched by 16-byte copies when both inputs are 16-byte aligned
        const int staged = (reinterpret_cast<uintptr_t>(*k0) % 16 == 0 && reinterpret_cast<uintptr_t>(*v0) % 16 == 0);
        { k_rs_downsweep<K, V><<<unsigned(ctas), RsCfg<K, V>::threads, smem, st>>>(*k0, *v0, *k1, *v1, n, 8 * d, part,
                                                                                   cnt, staged); note_launch(); }
        std::swap(*k0, *k1);
        std::swap(*v0, *v1);
    }
    return int(cudaGetLastError());
}

template int radix_sort_pairs<uint64_t, uint32_t>(uint64_t**, uint32_t**, uint64_t**, uint32_t**, size_t, int, int,
                                                  void*, size_t, cudaStream_t, bool);
template int radix_sort_pairs<uint64_t, uint64_t>(uint64_t**, uint64_t**, uint64_t**, uint64_t**, size_t, int, int,
                                                  void*, size_t, cudaStream_t, bool);
template int radix_sort_pairs<uint32_t, uint32_t>(uint32_t**, uint32_t**, uint32_t**, uint32_t**, size_t, int, int,
                                                  void*, size_t, cudaStream_t, bool);
template int radix_sort_pairs<uint32_t, uint64_t>(uint32_t**, uint64_t**, uint32_t**, uint64_t**, size_t, int, int,
                                                  void*, size_t, cudaStream_t, bool);

// ------------------------------------------------------------------------------ group ranks

constexpr int HT_THREADS = 256;
constexpr int HT_IPT = 8;
constexpr int HT_TILE = HT_THREADS * HT_IPT;

// per tile: max over i of (key[i] != key[i-1] ? i : 0), and the number of group starts
__global__ void k_head_tiles(const uint64_t* __restrict__ key, size_t n, unsigned long long* __restrict__ tmax,
                             unsigned long long* __restrict__ tcnt) {
    __shared__ unsigned long long smax[HT_THREADS / 32], scnt[HT_THREADS / 32];
    const size_t t0 = size_t(blockIdx.x) * HT_TILE;
    unsigned long long m = 0, c = 0;
    for (int j = threadIdx.x; j < HT_TILE; j += HT_THREADS) {
        size_t i = t0 + j;
        if (i >= n) break;
        bool f = (i == 0) || key[i] != key[i - 1];
        if (f) { m = i; c++; }
    }
    #pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        m = max(m, __shfl_down_sync(0xffffffffu, m, o));
        c += __shfl_down_sync(0xffffffffu, c, o);
    }
    if ((threadIdx.x & 31) == 0) { smax[threadIdx.x >> 5] = m; scnt[threadIdx.x >> 5] = c; }
    __syncthreads();
    if (threadIdx.x == 0) {
        unsigned long long M = 0, Cn = 0;
        for (int w = 0; w < HT_THREADS / 32; ++w) { M = max(M, smax[w]); Cn += scnt[w]; }
        tmax[blockIdx.x] = M;
        tcnt[blockIdx.x] = Cn;
    }
}

// single CTA: exclusive max-scan of tile maxima (in place), total of tile counts into *groups
__global__ void k_head_carry(unsigned long long* __restrict__ tmax, const unsigned long long* __restrict__ tcnt,
                             size_t m, unsigned long long* __restrict__ groups) {
    __shared__ unsigned long long wv[32], carry, total;
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    if (threadIdx.x == 0) { carry = 0; total = 0; }
    __syncthreads();
    for (size_t base = 0; base < m; base += 1024) {
        size_t i = base + threadIdx.x;
        unsigned long long v = i < m ? tmax[i] : 0, x = v;
        unsigned long long c = i < m ? tcnt[i] : 0;
        #pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            unsigned long long y = __shfl_up_sync(0xffffffffu, x, o);
            if (lane >= o) x = max(x, y);
        }
        #pragma unroll
        for (int o = 16; o > 0; o >>= 1) c += __shfl_down_sync(0xffffffffu, c, o);
        if (lane == 31) wv[wid] = x;
        if (lane == 0) atomicAdd(&total, c);
        __syncthreads();
        unsigned long long pre = carry;
        for (int w = 0; w < wid; ++w) pre = max(pre, wv[w]);
        unsigned long long up = __shfl_up_sync(0xffffffffu, x, 1);
        unsigned long long excl = lane ? max(pre, up) : pre;
        if (i < m) tmax[i] = excl;
        __syncthreads();
        if (threadIdx.x == 1023) carry = max(pre, x);
        __syncthreads();
    }
    if (threadIdx.x == 0) *groups = total;
}

// head[i] = last group start <= i; rank[val[i]] = head[i]; kout[i] = head[i] << 32
// (kout != key: neighbouring threads still read key[i0-1])
template <class V>
__global__ void k_head_apply(const uint64_t* __restrict__ key, uint64_t* __restrict__ kout, const V* __restrict__ val,
                             size_t n, const unsigned long long* __restrict__ carry, uint32_t* __restrict__ rank) {
    __shared__ unsigned long long wv[HT_THREADS / 32];
    const size_t t0 = size_t(blockIdx.x) * HT_TILE;
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    // thread owns HT_IPT consecutive items
    const size_t i0 = t0 + size_t(threadIdx.x) * HT_IPT;
    unsigned long long h[HT_IPT];
    uint64_t prevk = (i0 > 0 && i0 < n) ? key[i0 - 1] : 0;
    unsigned long long run = 0;
    #pragma unroll
    for (int j = 0; j < HT_IPT; ++j) {
        size_t i = i0 + j;
        uint64_t kk = i < n ? key[i] : 0;
        bool f = i < n && (i == 0 || kk != prevk);
        if (f) run = i;
        h[j] = run;
        prevk = kk;
    }
    unsigned long long x = run;
    #pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        unsigned long long y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= o) x = max(x, y);
    }
    if (lane == 31) wv[wid] = x;
    __syncthreads();
    unsigned long long pre = carry[blockIdx.x];
    for (int w = 0; w < wid; ++w) pre = max(pre, wv[w]);
    unsigned long long up = __shfl_up_sync(0xffffffffu, x, 1);
    unsigned long long excl = lane ? max(pre, up) : pre;
    #pragma unroll
    for (int j = 0; j < HT_IPT; ++j) {
        size_t i = i0 + j;
        if (i < n) {
            unsigned long long hd = max(excl, h[j]);
            rank[val[i]] = uint32_t(hd);
            kout[i] = uint64_t(hd) << 32;
        }
    }
}

// key[i] |= rank of the suffix h bases further (+1), or 0 when that lies past the read end
template <class V>
__global__ void k_second_keys(uint64_t* __restrict__ key, const V* __restrict__ val, size_t n, idx_t L, size_t h,
                              const uint32_t* __restrict__ rank) {
    const size_t stride = size_t(gridDim.x) * blockDim.x;
    for (size_t i = size_t(blockIdx.x) * blockDim.x + threadIdx.x; i < n; i += stride) {
        size_t p = val[i];
        size_t off = p % L;
        uint64_t second = (off + h < size_t(L)) ? uint64_t(rank[p + h]) + 1 : 0;
        key[i] |= second;
    }
}

template <class V>
__global__ void k_copy_vals(const V* __restrict__ v, size_t n, idx_t* __restrict__ sa) {
    const size_t stride = size_t(gridDim.x) * blockDim.x;
    for (size_t i = size_t(blockIdx.x) * blockDim.x + threadIdx.x; i < n; i += stride) sa[i] = idx_t(v[i]);
}

// ------------------------------------------------------------------------------ group refinement
//
// After the sort on 14-base keys, every group of equal keys whose suffixes all go on past base 14
// still has to be ordered.  At read coverage c such groups hold about c suffixes, so instead of
// more whole-array passes each group is finished where it lies: every suffix loads the rest of
// its bases as W 64-bit words (bases past its end read as A) and the group is sorted by
// (words, suffix length, position) -- the end-of-read-lowest order, ties by position.  Groups of
// up to 32 and up to 128 suffixes are sorted by one warp in registers (1 or 4 per lane, several
// groups packed per warp), up to 1024 by one CTA in shared memory, all with bitonic networks;
// larger ones by a radix sort of their range on the next 29 bases.

constexpr int kRefineMaxWords = 8;          // suffixes up to 14 + 30 + 224 bases
constexpr int kGroupWarp4 = 128;            // largest group sorted by one warp, 4 per lane
constexpr int kGroupCta = 1024;             // largest group sorted in shared memory

// Group classes: 0 = 2..32 suffixes, 1 = 33..128, 2 = 129..1024 (entries (start << 24) | size),
// 3 = larger (start, size pairs).
struct GroupLists {
    unsigned long long* list[4];
    unsigned long long* counts;             // [4]
    size_t cap[4];                          // entries (pairs for class 3)
    uint8_t* bwt;                           // BWT symbols of the rows the refinement places, or null
    idx_t* isa;                             // their inverse-SA entries (offsets 1..M), or null
    idx_t isa_m;                            // M
    size_t row_base;                        // suffix-array row of val[0]
};

// side outputs of a row the refinement has placed: its BWT symbol and, for read offsets 1..M,
// its inverse-SA entry isa[read * M + offset - 1] = row (written here, where the refinement's
// ALU-bound networks leave DRAM idle, instead of by a separate scatter over every row)
__device__ __forceinline__ void row_outputs(uint8_t* __restrict__ bwt, idx_t* __restrict__ isa, idx_t M,
                                            size_t row, idx_t pos, idx_t L, uint8_t sym) {
    if (bwt) bwt[row] = sym;
    if (isa) {
        const idx_t rd = pos / L, off = pos - rd * L;
        if (off >= 1 && off <= M) isa[size_t(rd) * M + (off - 1)] = idx_t(row);
    }
}

// BWT symbol of the suffix at p: 0 (`$`) at a read start, else the preceding base (1..4)
__device__ __forceinline__ uint8_t bwt_symbol(const uint64_t* __restrict__ pk, size_t p, idx_t L) {
    if (p % size_t(L) == 0) return 0;
    const size_t q = p - 1;
    return uint8_t(((pk[q >> 5] >> (62 - 2 * int(q & 31))) & 3) + 1);
}

__device__ __forceinline__ int group_class(size_t m) {
    if (m < 2) return -1;
    if (m <= 32) return 0;
    if (m <= size_t(kGroupWarp4)) return 1;
    return m <= size_t(kGroupCta) ? 2 : 3;
}

// One CTA per tile of 4096 sorted keys.  Two bit masks per tile, by ballots: group heads, and
// keys whose suffix is longer than the key's bases.  Then one thread per mask word walks the set
// bits of (head & long) only: a group ends at the next head bit (in the mask; a group running past
// the tile end is followed in global memory by a galloping search), and the groups are listed by
// size class.  List slots are taken with one atomic per list per tile, after a block-wide prefix
// of the per-thread counts; the walk runs twice (count, then write).
constexpr int kGlTile = 4096;
constexpr int kGlThreads = 256;
constexpr int kGlPer = kGlTile / kGlThreads;      // positions per thread (j = tid + 256 i)
constexpr int kGlWords = kGlTile / 32;

__device__ __forceinline__ void block_scan4(unsigned (&c)[4], unsigned (&excl)[4], unsigned (*wsum)[4],
                                            unsigned* tot) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    unsigned x[4] = {c[0], c[1], c[2], c[3]};
    #pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        #pragma unroll
        for (int q = 0; q < 4; ++q) {
            const unsigned y = __shfl_up_sync(0xffffffffu, x[q], o);
            if (lane >= o) x[q] += y;
        }
    }
    if (lane == 31) {
        #pragma unroll
        for (int q = 0; q < 4; ++q) wsum[warp][q] = x[q];
    }
    __syncthreads();
    #pragma unroll
    for (int q = 0; q < 4; ++q) {
        unsigned before = 0, all = 0;
        for (int w = 0; w < kGlThreads / 32; ++w) {
            before += w < warp ? wsum[w][q] : 0u;
            all += wsum[w][q];
        }
        excl[q] = before + x[q] - c[q];
        tot[q] = all;
    }
}

// first index >= e0 whose key differs from k (keys sorted; key[e0 - 1] == k), or n
template <class K>
__device__ size_t run_end(const K* __restrict__ key, size_t n, size_t e0, K k) {
    size_t lo = e0, step = 32;                      // key[lo - 1] == k
    size_t hi = lo;
    while (true) {                                  // gallop: hi = first probe that differs (or n)
        hi = lo + step < n ? lo + step : n;
        if (hi == n || key[hi] != k) break;
        lo = hi + 1;
        step *= 2;
    }
    // the answer lies in [lo, hi]: the first index there with key != k (hi qualifies)
    while (lo < hi) {
        const size_t mid = lo + (hi - lo) / 2;
        if (key[mid] != k) hi = mid;
        else lo = mid + 1;
    }
    return lo;
}

template <class K>
__global__ void __launch_bounds__(kGlThreads, 5) k_group_lists(const K* __restrict__ key, size_t n, GroupLists G,
                                                           size_t base) {
    __shared__ uint32_t hm[kGlWords + 1];               // heads; sentinel word at the end
    __shared__ uint32_t lm[kGlWords];                   // long suffixes
    __shared__ unsigned wsum[kGlThreads / 32][4];
    __shared__ unsigned long long sbase[4];
    __shared__ K last[kGlPer][kGlThreads / 32];         // each warp's lane-31 key, per round
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    for (size_t t0 = size_t(blockIdx.x) * kGlTile; t0 < n; t0 += size_t(gridDim.x) * kGlTile) {
        // all of the thread's keys in flight at once; a key's predecessor comes from the lane
        // before, or for lane 0 from the warp before (or the round before) through shared memory
        K kk[kGlPer];
        #pragma unroll
        for (int q = 0; q < kGlPer; ++q) {
            const size_t i = t0 + threadIdx.x + size_t(kGlThreads) * q;
            kk[q] = i < n ? key[i] : K(0);
        }
        const K before_tile = (t0 > 0 && threadIdx.x == 0) ? key[t0 - 1] : K(0);
        if (lane == 31) {
            #pragma unroll
            for (int q = 0; q < kGlPer; ++q) last[q][warp] = kk[q];
        }
        __syncthreads();
        #pragma unroll
        for (int q = 0; q < kGlPer; ++q) {
            const int j = threadIdx.x + kGlThreads * q;
            const size_t i = t0 + j;
            K prev = __shfl_up_sync(0xffffffffu, kk[q], 1);
            if (lane == 0) prev = warp ? last[q][warp - 1] : (q ? last[q - 1][kGlThreads / 32 - 1] : before_tile);
            const bool head = i < n && (i == 0 || kk[q] != prev);
            const uint32_t hb = __ballot_sync(0xffffffffu, head);
            const uint32_t lb = __ballot_sync(0xffffffffu, i < n && key_len<K>(kk[q]) == KeyFmt<K>::bases);
            if (lane == 0) {
                hm[j >> 5] = hb;
                lm[j >> 5] = lb;
            }
        }
        if (threadIdx.x == 0) hm[kGlWords] = 1u;        // sentinel: the tile end
        __syncthreads();
        // walk: thread t < kGlWords owns mask word t
        auto group_size = [&](int j) -> size_t {
            int w = (j + 1) >> 5;
            uint32_t bits = (j + 1 < kGlTile) ? hm[w] & (~0u << ((j + 1) & 31)) : hm[w];
            while (!bits) bits = hm[++w];               // ends at the sentinel word at the latest
            const int nxt = 32 * w + __ffs(bits) - 1;
            const size_t i = t0 + size_t(j);
            size_t e = t0 + size_t(nxt);
            if (nxt >= kGlTile) e = t0 + kGlTile < n ? run_end<K>(key, n, t0 + kGlTile, key[i]) : n;
            if (e > n) e = n;
            return e - i;
        };
        const int tw = threadIdx.x;
        const uint32_t mine = tw < kGlWords ? (hm[tw] & lm[tw]) : 0u;
        unsigned c[4] = {0, 0, 0, 0};
        for (uint32_t bits = mine; bits; bits &= bits - 1) {
            const int cl = group_class(group_size(32 * tw + __ffs(bits) - 1));
            #pragma unroll
            for (int z = 0; z < 4; ++z) c[z] += cl == z ? 1u : 0u;
        }
        unsigned excl[4], tot[4];
        block_scan4(c, excl, wsum, tot);
        if (threadIdx.x == 0) {
            #pragma unroll
            for (int q = 0; q < 4; ++q) sbase[q] = tot[q] ? atomicAdd(&G.counts[q], (unsigned long long)tot[q]) : 0ull;
        }
        __syncthreads();
        unsigned long long at[4] = {sbase[0] + excl[0], sbase[1] + excl[1], sbase[2] + excl[2], sbase[3] + excl[3]};
        for (uint32_t bits = mine; bits; bits &= bits - 1) {
            const int j = 32 * tw + __ffs(bits) - 1;
            const size_t m = group_size(j);
            const int cl = group_class(m);
            const size_t i = base + t0 + size_t(j);
            if (cl == 3) {
                if (at[3] < G.cap[3]) {
                    G.list[3][2 * at[3]] = i;
                    G.list[3][2 * at[3] + 1] = m;
                }
                ++at[3];
            } else if (cl >= 0) {
                if (at[cl] < G.cap[cl]) G.list[cl][at[cl]] = (uint64_t(i) << 24) | m;
                ++at[cl];
            }
        }
        __syncthreads();
    }
}

// the W words of bases off, off+32, ... of the suffix at p (length m_len), zero past its end
template <int W>
__device__ __forceinline__ void suffix_words(const uint64_t* __restrict__ pk, size_t p, int m_len, int off,
                                             uint64_t w[W]) {
    #pragma unroll
    for (int j = 0; j < W; ++j) {
        const int rem = m_len - off - 32 * j;
        uint64_t x = 0;
        if (rem > 0) {
            x = window(pk, p + off + 32 * size_t(j));
            if (rem < 32) x &= ~uint64_t(0) << (64 - 2 * rem);
        }
        w[j] = x;
    }
}

template <int W>
__device__ __forceinline__ bool tuple_less(const uint64_t a[W], uint64_t alen, uint64_t apos, const uint64_t b[W],
                                           uint64_t blen, uint64_t bpos) {
    #pragma unroll
    for (int j = 0; j < W; ++j)
        if (a[j] != b[j]) return a[j] < b[j];
    if (alen != blen) return alen < blen;
    return apos < bpos;
}

// Groups of 2..32E suffixes, several per warp: a warp takes 8 list entries at a time and packs
// consecutive ones into its 32E slots (slot e * 32 + lane is register set e of that lane) while
// they fit; one bitonic network over the 32E slots on (segment, bases from `from` on, length,
// slot) then sorts every packed group in place (each segment keeps its slots, since segments are
// numbered in slot order and empty slots sort last).  The segment number (3 bits) rides in the top
// of the first word, which holds the next 30 bases; the other words hold 32 each.  A group's
// members arrive in ascending position (every radix pass is stable from text order), so the
// original slot breaks ties exactly as the position does; the positions wait in shared memory
// and are gathered by slot at the end.  Distances below 32 exchange by shuffle, larger ones swap
// registers within a lane.
template <int W>
struct RefineItem {
    uint64_t w[W];                              // w[0] = segment (3 bits) | 30 bases | 0
    uint32_t tail;                              // (length << 8) | original slot
};

// the words of RefineItem for the suffix at p (length m_len): bases from `off` on, zero past its end
template <int W>
__device__ __forceinline__ void refine_words(const uint64_t* __restrict__ pk, size_t p, int m_len, int off, uint32_t seg,
                                             uint64_t w[W]) {
    const int rem0 = m_len - off;
    uint64_t x = 0;
    if (rem0 > 0) {
        x = window(pk, p + off) & (~uint64_t(0) << 4);            // 30 bases
        if (rem0 < 30) x &= ~uint64_t(0) << (64 - 2 * rem0);
    }
    w[0] = (uint64_t(seg) << 61) | (x >> 3);
    #pragma unroll
    for (int j = 1; j < W; ++j) {
        const int rem = rem0 - 30 - 32 * (j - 1);
        uint64_t y = 0;
        if (rem > 0) {
            y = window(pk, p + off + 30 + 32 * size_t(j - 1));
            if (rem < 32) y &= ~uint64_t(0) << (64 - 2 * rem);
        }
        w[j] = y;
    }
}

// a < b on (w[0..W-1], tail) as one unsigned multi-word number: the borrow out of the
// subtraction a - b, least significant word first, in one chain of subtract-with-borrow
// instructions (no branches; the chain must sit in one asm statement to keep the carry flag).
#define PQ_SUBC(x, y) "subc.cc.u64 t, %" #x ", %" #y ";\n\t"
#define PQ_LT_HEAD "{\n\t.reg .u64 t;\n\t.reg .u32 s, z;\n\tmov.u32 z, 0;\n\tsub.cc.u32 s, %1, %2;\n\t"
#define PQ_LT_TAIL "subc.u32 %0, z, z;\n\t}"
#define PQ_WORD(j) "l"(a.w[j]), "l"(b.w[j])

template <int W>
__device__ __forceinline__ bool item_less(const RefineItem<W>& a, const RefineItem<W>& b);

template <>
__device__ __forceinline__ bool item_less<1>(const RefineItem<1>& a, const RefineItem<1>& b) {
    unsigned r;
    asm(PQ_LT_HEAD PQ_SUBC(3, 4) PQ_LT_TAIL
        : "=r"(r)
        : "r"(a.tail), "r"(b.tail), PQ_WORD(0));
    return r != 0;
}

template <>
__device__ __forceinline__ bool item_less<2>(const RefineItem<2>& a, const RefineItem<2>& b) {
    unsigned r;
    asm(PQ_LT_HEAD PQ_SUBC(3, 4) PQ_SUBC(5, 6) PQ_LT_TAIL
        : "=r"(r)
        : "r"(a.tail), "r"(b.tail), PQ_WORD(1), PQ_WORD(0));
    return r != 0;
}

template <>
__device__ __forceinline__ bool item_less<3>(const RefineItem<3>& a, const RefineItem<3>& b) {
    unsigned r;
    asm(PQ_LT_HEAD PQ_SUBC(3, 4) PQ_SUBC(5, 6) PQ_SUBC(7, 8) PQ_LT_TAIL
        : "=r"(r)
        : "r"(a.tail), "r"(b.tail), PQ_WORD(2), PQ_WORD(1), PQ_WORD(0));
    return r != 0;
}

template <>
__device__ __forceinline__ bool item_less<4>(const RefineItem<4>& a, const RefineItem<4>& b) {
    unsigned r;
    asm(PQ_LT_HEAD PQ_SUBC(3, 4) PQ_SUBC(5, 6) PQ_SUBC(7, 8) PQ_SUBC(9, 10) PQ_LT_TAIL
        : "=r"(r)
        : "r"(a.tail), "r"(b.tail), PQ_WORD(3), PQ_WORD(2), PQ_WORD(1), PQ_WORD(0));
    return r != 0;
}

template <>
__device__ __forceinline__ bool item_less<5>(const RefineItem<5>& a, const RefineItem<5>& b) {
    unsigned r;
    asm(PQ_LT_HEAD PQ_SUBC(3, 4) PQ_SUBC(5, 6) PQ_SUBC(7, 8) PQ_SUBC(9, 10) PQ_SUBC(11, 12) PQ_LT_TAIL
        : "=r"(r)
        : "r"(a.tail), "r"(b.tail), PQ_WORD(4), PQ_WORD(3), PQ_WORD(2), PQ_WORD(1), PQ_WORD(0));
    return r != 0;
}

template <>
__device__ __forceinline__ bool item_less<6>(const RefineItem<6>& a, const RefineItem<6>& b) {
    unsigned r;
    asm(PQ_LT_HEAD PQ_SUBC(3, 4) PQ_SUBC(5, 6) PQ_SUBC(7, 8) PQ_SUBC(9, 10) PQ_SUBC(11, 12) PQ_SUBC(13, 14) PQ_LT_TAIL
        : "=r"(r)
        : "r"(a.tail), "r"(b.tail), PQ_WORD(5), PQ_WORD(4), PQ_WORD(3), PQ_WORD(2), PQ_WORD(1), PQ_WORD(0));
    return r != 0;
}

template <>
__device__ __forceinline__ bool item_less<7>(const RefineItem<7>& a, const RefineItem<7>& b) {
    unsigned r;
    asm(PQ_LT_HEAD PQ_SUBC(3, 4) PQ_SUBC(5, 6) PQ_SUBC(7, 8) PQ_SUBC(9, 10) PQ_SUBC(11, 12) PQ_SUBC(13, 14) PQ_SUBC(15, 16) PQ_LT_TAIL
        : "=r"(r)
        : "r"(a.tail), "r"(b.tail), PQ_WORD(6), PQ_WORD(5), PQ_WORD(4), PQ_WORD(3), PQ_WORD(2), PQ_WORD(1), PQ_WORD(0));
    return r != 0;
}

template <>
__device__ __forceinline__ bool item_less<8>(const RefineItem<8>& a, const RefineItem<8>& b) {
    unsigned r;
    asm(PQ_LT_HEAD PQ_SUBC(3, 4) PQ_SUBC(5, 6) PQ_SUBC(7, 8) PQ_SUBC(9, 10) PQ_SUBC(11, 12) PQ_SUBC(13, 14) PQ_SUBC(15, 16) PQ_SUBC(17, 18) PQ_LT_TAIL
        : "=r"(r)
        : "r"(a.tail), "r"(b.tail), PQ_WORD(7), PQ_WORD(6), PQ_WORD(5), PQ_WORD(4), PQ_WORD(3), PQ_WORD(2), PQ_WORD(1), PQ_WORD(0));
    return r != 0;
}

#undef PQ_SUBC
#undef PQ_LT_HEAD
#undef PQ_LT_TAIL
#undef PQ_WORD

constexpr int kRefineThreads = 256;

template <int W, int E>
__global__ void __launch_bounds__(kRefineThreads, E == 1 ? (W <= 3 ? 5 : 1) : (W <= 4 ? 3 : 1)) k_refine_warp(const unsigned long long* __restrict__ list,
                                                                const unsigned long long* __restrict__ cnt,
                                                                const uint64_t* __restrict__ pk, idx_t L,
                                                                idx_t* __restrict__ val, int from,
                                                                uint8_t* __restrict__ bwt, idx_t* __restrict__ isa,
                                                                idx_t isa_m, size_t row_base) {
    constexpr int kChunk = 8;
    constexpr int N = 32 * E;
    __shared__ idx_t spos[kRefineThreads / 32][N];
    __shared__ uint8_t ssym[kRefineThreads / 32][N];
    const int lane = threadIdx.x & 31;
    idx_t* const mypos = spos[threadIdx.x >> 5];
    uint8_t* const mysym = ssym[threadIdx.x >> 5];
    const size_t warp = (size_t(blockIdx.x) * blockDim.x + threadIdx.x) >> 5;
    const size_t nwarps = (size_t(gridDim.x) * blockDim.x) >> 5;
    const size_t groups = *cnt;
    for (size_t c0 = warp * kChunk; c0 < groups; c0 += nwarps * kChunk) {
        const unsigned long long mine = (lane < kChunk && c0 + lane < groups) ? list[c0 + lane] : 0ull;
        int next = 0;
        while (next < kChunk) {
            // consecutive entries next .. next + taken - 1 fit in N slots
            int taken = 0, total = 0;
            uint32_t seg[E];
            size_t at[E];
            #pragma unroll
            for (int e = 0; e < E; ++e) {
                seg[e] = 255;
                at[e] = 0;
            }
            for (int q = next; q < kChunk; ++q) {
                const unsigned long long x = __shfl_sync(0xffffffffu, mine, q);
                const int m = int(x & 0xffffff);
                if (m == 0 || total + m > N) break;
                #pragma unroll
                for (int e = 0; e < E; ++e) {
                    const int slot = e * 32 + lane;
                    if (slot >= total && slot < total + m) {
                        seg[e] = uint32_t(q - next);
                        at[e] = size_t(x >> 24) + size_t(slot - total);
                    }
                }
                total += m;
                ++taken;
            }
            if (taken == 0) break;
            RefineItem<W> it[E];
            #pragma unroll
            for (int e = 0; e < E; ++e) {
                if (seg[e] != 255) {
                    const idx_t pos = val[at[e]];
                    const uint32_t len = uint32_t(L - pos % L);
                    refine_words<W>(pk, size_t(pos), int(len), from, seg[e], it[e].w);
                    it[e].tail = (len << 8) | uint32_t(e * 32 + lane);
                    mypos[e * 32 + lane] = pos;
                    if (bwt) mysym[e * 32 + lane] = bwt_symbol(pk, size_t(pos), L);
                } else {
                    #pragma unroll
                    for (int j = 0; j < W; ++j) it[e].w[j] = ~uint64_t(0);
                    it[e].tail = ~0u;
                }
            }
            #pragma unroll
            for (int k = 2; k <= N; k <<= 1) {
                #pragma unroll
                for (int j = k >> 1; j > 0; j >>= 1) {
                    if (j >= 32) {
                        #pragma unroll
                        for (int e = 0; e < E; ++e) {
                            const int f = e ^ (j >> 5);
                            if (f > e) {
                                const bool asc = ((e * 32 + lane) & k) == 0;
                                if (item_less<W>(it[f], it[e]) == asc) {
                                    const RefineItem<W> t = it[e];
                                    it[e] = it[f];
                                    it[f] = t;
                                }
                            }
                        }
                    } else {
                        #pragma unroll
                        for (int e = 0; e < E; ++e) {
                            RefineItem<W> o;
                            #pragma unroll
                            for (int q = 0; q < W; ++q) o.w[q] = __shfl_xor_sync(0xffffffffu, it[e].w[q], j);
                            o.tail = __shfl_xor_sync(0xffffffffu, it[e].tail, j);
                            const bool keep_min = ((lane & j) == 0) == (((e * 32 + lane) & k) == 0);
                            if (keep_min == item_less<W>(o, it[e])) it[e] = o;
                        }
                    }
                }
            }
            __syncwarp();
            #pragma unroll
            for (int e = 0; e < E; ++e) {
                if (seg[e] != 255) {
                    const idx_t pos = mypos[it[e].tail & 255u];
                    val[at[e]] = pos;
                    row_outputs(bwt, isa, isa_m, row_base + at[e], pos, L, bwt ? mysym[it[e].tail & 255u] : 0);
                }
            }
            __syncwarp();
            next += taken;
        }
    }
}

// bitonic sort of one group of m suffixes held as columns: words w[j][P2], len[P2], pos[P2]
template <int W>
__device__ void cta_bitonic(uint64_t* cols, int P2) {
    uint64_t* lenc = cols + size_t(W) * P2;
    uint64_t* posc = lenc + P2;
    for (int k = 2; k <= P2; k <<= 1) {
        for (int j = k >> 1; j > 0; j >>= 1) {
            for (int i = threadIdx.x; i < P2; i += blockDim.x) {
                const int o = i ^ j;
                if (o <= i) continue;
                uint64_t a[W], b[W];
                #pragma unroll
                for (int q = 0; q < W; ++q) {
                    a[q] = cols[size_t(q) * P2 + i];
                    b[q] = cols[size_t(q) * P2 + o];
                }
                const bool asc = (i & k) == 0;
                const bool b_less = tuple_less<W>(b, lenc[o], posc[o], a, lenc[i], posc[i]);
                if (b_less == asc) {
                    #pragma unroll
                    for (int q = 0; q < W; ++q) {
                        cols[size_t(q) * P2 + i] = b[q];
                        cols[size_t(q) * P2 + o] = a[q];
                    }
                    const uint64_t tl = lenc[i], tp = posc[i];
                    lenc[i] = lenc[o];
                    posc[i] = posc[o];
                    lenc[o] = tl;
                    posc[o] = tp;
                }
            }
            __syncthreads();
        }
    }
}

template <int W>
__device__ void cta_load_group(uint64_t* cols, int P2, size_t start, int m, const uint64_t* __restrict__ pk, idx_t L,
                               const idx_t* __restrict__ val, int off) {
    uint64_t* lenc = cols + size_t(W) * P2;
    uint64_t* posc = lenc + P2;
    for (int i = threadIdx.x; i < P2; i += blockDim.x) {
        uint64_t w[W];
        uint64_t len = ~uint64_t(0), pos = ~uint64_t(0);
        if (i < m) {
            pos = uint64_t(val[start + i]);
            len = uint64_t(L - idx_t(pos % L));
            suffix_words<W>(pk, size_t(pos), int(len), off, w);
        } else {
            #pragma unroll
            for (int q = 0; q < W; ++q) w[q] = ~uint64_t(0);
        }
        #pragma unroll
        for (int q = 0; q < W; ++q) cols[size_t(q) * P2 + i] = w[q];
        lenc[i] = len;
        posc[i] = pos;
    }
    __syncthreads();
}

template <int W>
__global__ void k_refine_cta(const unsigned long long* __restrict__ list, const unsigned long long* __restrict__ cnt,
                             const uint64_t* __restrict__ pk, idx_t L, idx_t* __restrict__ val, int off,
                             uint8_t* __restrict__ bwt, idx_t* __restrict__ isa, idx_t isa_m, size_t row_base) {
    extern __shared__ uint64_t s_cols[];
    const size_t groups = *cnt;
    for (size_t g = blockIdx.x; g < groups; g += gridDim.x) {
        const unsigned long long e = list[g];
        const size_t start = size_t(e >> 24);
        const int m = int(e & 0xffffff);
        int P2 = 32;
        while (P2 < m) P2 <<= 1;
        cta_load_group<W>(s_cols, P2, start, m, pk, L, val, off);
        cta_bitonic<W>(s_cols, P2);
        const uint64_t* posc = s_cols + size_t(W + 1) * P2;
        for (int i = threadIdx.x; i < m; i += blockDim.x) {
            const idx_t pos = idx_t(posc[i]);
            val[start + i] = pos;
            row_outputs(bwt, isa, isa_m, row_base + start + i, pos, L, bwt ? bwt_symbol(pk, size_t(pos), L) : 0);
        }
        __syncthreads();
    }
}

// 64-bit keys of a range of suffixes on their bases [off, off + 29): those bases (padded) and how
// many of them exist (0..29)
__global__ void k_range_keys(const uint64_t* __restrict__ pk, const idx_t* __restrict__ val, size_t m, idx_t L,
                             int off, uint64_t* __restrict__ key, idx_t* __restrict__ out) {
    const size_t stride = size_t(gridDim.x) * blockDim.x;
    for (size_t i = size_t(blockIdx.x) * blockDim.x + threadIdx.x; i < m; i += stride) {
        const idx_t p = val[i];
        const int rem = int(L - p % L) - off;
        key[i] = rem > 0 ? make_key<uint64_t>(window(pk, size_t(p) + off), rem) : 0;
        out[i] = p;
    }
}

// the groups of classes 0..2 (c: their counts)
template <int W>
static void refine_small_mid(const GroupLists& G, const unsigned long long* c, const uint64_t* pk, idx_t L,
                             idx_t* val, int off, cudaStream_t st) {
    if (c[0]) {
        unsigned g = unsigned(std::min<unsigned long long>((c[0] + 63) / 64, 152ull * 64));
        { k_refine_warp<W, 1><<<g, kRefineThreads, 0, st>>>(G.list[0], G.counts + 0, pk, L, val, off, G.bwt, G.isa, G.isa_m, G.row_base); note_launch(); }
    }
    if (c[1]) {
        unsigned g = unsigned(std::min<unsigned long long>((c[1] + 15) / 16, 152ull * 64));
        { k_refine_warp<W, 4><<<g, kRefineThreads, 0, st>>>(G.list[1], G.counts + 1, pk, L, val, off, G.bwt, G.isa, G.isa_m, G.row_base); note_launch(); }
    }
    if (c[2]) {
        const size_t smem = size_t(W + 2) * kGroupCta * sizeof(uint64_t);
        cudaFuncSetAttribute(k_refine_cta<W>, cudaFuncAttributeMaxDynamicSharedMemorySize, int(smem));
        unsigned g = unsigned(std::min<unsigned long long>(c[2], 152ull * 8));
        { k_refine_cta<W><<<g, 512, smem, st>>>(G.list[2], G.counts + 2, pk, L, val, off, G.bwt, G.isa, G.isa_m, G.row_base); note_launch(); }
    }
}

// Groups of up to 1024 suffixes are finished in place by the warp and CTA kernels.  A larger group
// (low-complexity or highly repeated sequence) gets a device-wide radix sort of its range on the
// next 29 bases (64-bit keys), and its subgroups are finished the same way, 29 bases further on
// each time.
template <int W>
static int refine_groups_w(const GroupLists& G, const unsigned long long* c0,
                           const std::vector<unsigned long long>& big, const uint64_t* pk, idx_t L, idx_t* val,
                           uint64_t* cols, size_t cols_cap, void* rtmp, size_t rtmp_bytes, cudaStream_t st) {
    refine_small_mid<W>(G, c0, pk, L, val, kHead, st);
    struct Item {
        size_t start, m;
        int off;
    };
    std::vector<Item> work;
    for (size_t i = 0; i + 1 < big.size(); i += 2) work.push_back({size_t(big[i]), size_t(big[i + 1]), kHead});
    std::vector<unsigned long long> sub;
    while (!work.empty()) {
        const Item it = work.back();
        work.pop_back();
        const size_t m = it.m;
        // range scratch in the column area: two key arrays, two value arrays
        const size_t kw = m, vw = (m * sizeof(idx_t) + 7) / 8;
        if (2 * kw + 2 * vw + 64 > cols_cap) return -1;
        uint64_t* ka = cols;
        uint64_t* kb = cols + kw;
        idx_t* va = reinterpret_cast<idx_t*>(cols + 2 * kw);
        idx_t* vb = reinterpret_cast<idx_t*>(cols + 2 * kw + vw);
        { k_range_keys<<<grid_for(m, 256), 256, 0, st>>>(pk, val + it.start, m, L, it.off, ka, va); note_launch(); }
        int rc = radix_sort_pairs<uint64_t, idx_t>(&ka, &va, &kb, &vb, m, 0, 64, rtmp, rtmp_bytes, st, true);
        if (rc) return rc;
        { k_copy_vals<idx_t><<<grid_for(m, 256), 256, 0, st>>>(va, m, val + it.start); note_launch(); }
        if (it.off + kWide >= int(L)) continue;          // every suffix is now fully compared
        cudaMemsetAsync(G.counts, 0, 4 * sizeof(unsigned long long), st);
        { k_group_lists<uint64_t><<<unsigned(std::min<size_t>((m + kGlTile - 1) / kGlTile, size_t(152) * 64)), 256, 0, st>>>(
              ka, m, G, it.start); note_launch(); }
        unsigned long long c[4];
        cudaMemcpyAsync(c, G.counts, sizeof c, cudaMemcpyDeviceToHost, st);
        cudaError_t e = cudaStreamSynchronize(st);
        if (e != cudaSuccess) return int(e);
        for (int z = 0; z < 4; ++z)
            if (c[z] > G.cap[z]) return -1;
        refine_small_mid<W>(G, c, pk, L, val, it.off + kWide, st);
        if (c[3]) {
            sub.resize(2 * c[3]);
            cudaMemcpyAsync(sub.data(), G.list[3], sub.size() * 8, cudaMemcpyDeviceToHost, st);
            e = cudaStreamSynchronize(st);
            if (e != cudaSuccess) return int(e);
            for (size_t i = 0; i + 1 < sub.size(); i += 2)
                work.push_back({size_t(sub[i]), size_t(sub[i + 1]), it.off + kWide});
        }
    }
    return int(cudaGetLastError());
}

// lists_mem holds the four group lists: (n/2 + n/33 + n/129 + 2 n/1025 + 5) 64-bit entries,
// under 0.55 n
static int refine_groups(const uint32_t* key, idx_t* val, size_t n, idx_t L, const uint64_t* pk, uint64_t* lists_mem,
                         uint64_t* cols, size_t cols_cap, unsigned long long* counters, void* rtmp, size_t rtmp_bytes,
                         cudaStream_t st, uint8_t* bwt = nullptr, idx_t* isa = nullptr, idx_t isa_m = 0,
                         size_t row_base = 0) {
    // words from base 14 on: 30 bases in the first (beside the segment number), 32 in each other
    const int W = 1 + int((size_t(L) > size_t(kHead) + 30 ? size_t(L) - kHead - 30 + 31 : 0) / 32);
    if (W < 1 || W > kRefineMaxWords) return -1;
    GroupLists G;
    G.cap[0] = n / 2 + 1;
    G.cap[1] = n / 33 + 1;
    G.cap[2] = n / (kGroupWarp4 + 1) + 1;
    G.cap[3] = n / (kGroupCta + 1) + 1;
    G.list[0] = reinterpret_cast<unsigned long long*>(lists_mem);
    G.list[1] = G.list[0] + G.cap[0];
    G.list[2] = G.list[1] + G.cap[1];
    G.list[3] = G.list[2] + G.cap[2];
    G.counts = counters;
    G.bwt = bwt;
    G.isa = isa;
    G.isa_m = isa_m;
    G.row_base = row_base;
    cudaMemsetAsync(counters, 0, 4 * sizeof(unsigned long long), st);
    { k_group_lists<uint32_t><<<unsigned(std::min<size_t>((n + kGlTile - 1) / kGlTile, size_t(152) * 64)), 256, 0, st>>>(
          key, n, G, 0); note_launch(); }
    unsigned long long c[4];
    cudaMemcpyAsync(c, counters, sizeof c, cudaMemcpyDeviceToHost, st);
    cudaError_t e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) return int(e);
    std::vector<unsigned long long> big(2 * c[3]);
    if (c[3]) {
        cudaMemcpyAsync(big.data(), G.list[3], big.size() * 8, cudaMemcpyDeviceToHost, st);
        e = cudaStreamSynchronize(st);
        if (e != cudaSuccess) return int(e);
    }
    switch (W) {
        case 1: return refine_groups_w<1>(G, c, big, pk, L, val, cols, cols_cap, rtmp, rtmp_bytes, st);
        case 2: return refine_groups_w<2>(G, c, big, pk, L, val, cols, cols_cap, rtmp, rtmp_bytes, st);
        case 3: return refine_groups_w<3>(G, c, big, pk, L, val, cols, cols_cap, rtmp, rtmp_bytes, st);
        case 4: return refine_groups_w<4>(G, c, big, pk, L, val, cols, cols_cap, rtmp, rtmp_bytes, st);
        case 5: return refine_groups_w<5>(G, c, big, pk, L, val, cols, cols_cap, rtmp, rtmp_bytes, st);
        case 6: return refine_groups_w<6>(G, c, big, pk, L, val, cols, cols_cap, rtmp, rtmp_bytes, st);
        case 7: return refine_groups_w<7>(G, c, big, pk, L, val, cols, cols_cap, rtmp, rtmp_bytes, st);
        default: return refine_groups_w<8>(G, c, big, pk, L, val, cols, cols_cap, rtmp, rtmp_bytes, st);
    }
}

// ------------------------------------------------------------------------------ driver

static size_t al(size_t b) { return (b + 255) & ~size_t(255); }

size_t suffix_sort_tmp_bytes(size_t n) {
    size_t tiles = (n + HT_TILE - 1) / HT_TILE + 1;
    return 2 * al(n * sizeof(uint64_t)) + al(n * sizeof(idx_t)) + al(n * sizeof(uint32_t)) +
           al((n / 32 + 4) * sizeof(uint64_t)) + al(radix_tmp_bytes(n)) + al(3 * tiles * sizeof(unsigned long long)) +
           al(n) + 1024;
}

int suffix_sort(const uint8_t* reads, idx_t num_reads, int L, int dir, idx_t* sa, void* tmp, size_t tmp_bytes,
                cudaStream_t st, const uint32_t** keys_out, const uint8_t** bwt_out, uint64_t* pk_out,
                idx_t* isa_out, idx_t isa_m) {
    if (keys_out) *keys_out = nullptr;
    if (bwt_out) *bwt_out = nullptr;
    const size_t n = size_t(num_reads) * size_t(L);
    if (n == 0) return 0;
    if (n >= (size_t(1) << 31)) return int(cudaErrorNotSupported);   // 32-bit group ranks
    if (tmp_bytes < suffix_sort_tmp_bytes(n)) return int(cudaErrorInvalidValue);
    char* p = static_cast<char*>(tmp);
    uint64_t* ka = reinterpret_cast<uint64_t*>(p); p += al(n * sizeof(uint64_t));
    uint64_t* kb = reinterpret_cast<uint64_t*>(p); p += al(n * sizeof(uint64_t));
    // the values start in the suffix array itself (four radix passes bring them back there)
    idx_t* va = sa;
    idx_t* vb = reinterpret_cast<idx_t*>(p); p += al(n * sizeof(idx_t));
    uint32_t* rank = reinterpret_cast<uint32_t*>(p); p += al(n * sizeof(uint32_t));
    const size_t nwords = n / 32 + 4;
    uint64_t* pk = pk_out ? pk_out : reinterpret_cast<uint64_t*>(p);
    p += al(nwords * sizeof(uint64_t));
    void* rtmp = p; p += al(radix_tmp_bytes(n));
    const size_t tiles = (n + HT_TILE - 1) / HT_TILE;
    unsigned long long* tmax = reinterpret_cast<unsigned long long*>(p);
    unsigned long long* tcnt = tmax + tiles + 1;
    unsigned long long* groups = tcnt + tiles + 1;
    p += al(3 * (tiles + 1) * sizeof(unsigned long long));
    // BWT symbols of the refined rows (0xff elsewhere), kept only when asked for
    uint8_t* bwt = bwt_out ? reinterpret_cast<uint8_t*>(p) : nullptr;

    idx_t* const vb0 = vb;                 // followed by rank in memory
    auto finish = [&](const uint32_t* keys) {
        if (va != sa) { k_copy_vals<idx_t><<<grid_for(n, 256), 256, 0, st>>>(va, n, sa); note_launch(); }
        if (keys_out) *keys_out = keys;
        return int(cudaGetLastError());
    };
    { k_pack_text<<<grid_for(nwords, 256), 256, 0, st>>>(reads, n, idx_t(L), dir, nwords, pk); note_launch(); }
    // 32-bit head keys in the two 64-bit key buffers
    uint32_t* ha = reinterpret_cast<uint32_t*>(ka);
    uint32_t* hb = reinterpret_cast<uint32_t*>(kb);
    if (reinterpret_cast<uintptr_t>(va) % 16 == 0 && reinterpret_cast<uintptr_t>(ha) % 16 == 0)
        { k_init_keys4<<<grid_for((n + 3) / 4, 256), 256, 0, st>>>(pk, n, idx_t(L), ha, va); note_launch(); }
    else    // a caller's suffix array that is not 16-byte aligned
        { k_init_keys<uint32_t><<<grid_for(n, 256), 256, 0, st>>>(pk, n, idx_t(L), ha, va); note_launch(); }
    // all four digits vary on any real read set: no histogram pass, no host round trip
    int rc = radix_sort_pairs<uint32_t, idx_t>(&ha, &va, &hb, &vb, n, 0, 32, rtmp, radix_tmp_bytes(n), st, false);
    if (rc) return rc;
    if (size_t(L) <= size_t(kHead)) return finish(ha);   // every suffix fits in its key: final order
    {
        // finish the groups where they lie; lists go to the free key buffer, big-group scratch to
        // the free value buffer (and rank behind it when that buffer is the scratch one; when the
        // values ended in the scratch, the free one is the suffix array, exactly n entries)
        uint64_t* cols = reinterpret_cast<uint64_t*>(vb);
        const size_t cols_cap = vb == vb0 ? (al(n * sizeof(idx_t)) + al(n * sizeof(uint32_t))) / sizeof(uint64_t)
                                          : n * sizeof(idx_t) / sizeof(uint64_t);
        if (bwt) cudaMemsetAsync(bwt, 0xff, n, st);
        rc = refine_groups(ha, va, n, idx_t(L), pk, reinterpret_cast<uint64_t*>(hb), cols, cols_cap, tcnt, rtmp,
                           radix_tmp_bytes(n), st, bwt, isa_out, isa_m);
        if (rc > 0) return rc;
        if (rc == 0) {   // the refinement permutes suffixes within groups of equal keys only
            if (bwt_out) *bwt_out = bwt;
            return finish(ha);
        }
        // a group too large for the scratch (or reads longer than 268 bases): prefix doubling on
        // 29-base keys
        ka = reinterpret_cast<uint64_t*>(ha);
        kb = reinterpret_cast<uint64_t*>(hb);
        { k_init_keys<uint64_t><<<grid_for(n, 256), 256, 0, st>>>(pk, n, idx_t(L), ka, va); note_launch(); }
        rc = radix_sort_pairs<uint64_t, idx_t>(&ka, &va, &kb, &vb, n, 0, 64, rtmp, radix_tmp_bytes(n), st, true);
        if (rc) return rc;
    }
    for (size_t h = kWide;; h *= 2) {
        { k_head_tiles<<<unsigned(tiles), HT_THREADS, 0, st>>>(ka, n, tmax, tcnt); note_launch(); }
        { k_head_carry<<<1, 1024, 0, st>>>(tmax, tcnt, tiles, groups); note_launch(); }
        { k_head_apply<idx_t><<<unsigned(tiles), HT_THREADS, 0, st>>>(ka, kb, va, n, tmax, rank); note_launch(); }
        std::swap(ka, kb);
        unsigned long long g = 0;
        cudaMemcpyAsync(&g, groups, sizeof g, cudaMemcpyDeviceToHost, st);
        cudaError_t e = cudaStreamSynchronize(st);
        if (e != cudaSuccess) return int(e);
        if (g == n || h >= size_t(L)) break;
        { k_second_keys<idx_t><<<grid_for(n, 256), 256, 0, st>>>(ka, va, n, idx_t(L), h, rank); note_launch(); }
        int bits = 1;
        while ((size_t(1) << bits) <= n + 1) ++bits;
        rc = radix_sort_pairs<uint64_t, idx_t>(&ka, &va, &kb, &vb, n, 0, 32 + bits, rtmp, radix_tmp_bytes(n), st, true);
        if (rc) return rc;
    }
    return finish(nullptr);
}

// ------------------------------------------------------------------------------ chunked sort
//
// For indexes too large for one pass (group ranks are 32-bit, and the working memory grows with
// n): every suffix falls in a bucket by its first 6 bases (padded with A) and min(length, 6),
// numbered in suffix order, so the suffix array is the concatenation of the buckets' own sorted
// suffixes.  Consecutive buckets are gathered into chunks of at most `cap` suffixes; each chunk is
// listed in text order (stable compaction), keyed, radix sorted and refined exactly as a whole
// sort, and written at its offset.

constexpr int kBucketBases = 6;
constexpr int kBuckets = (1 << (2 * kBucketBases)) * 8;
constexpr int kCkTile = 8192;

__device__ __forceinline__ uint32_t bucket_of(const uint64_t* __restrict__ pk, size_t p, const DivL& dl) {
    const int m = int(dl.L - uint32_t(p - div_l(p, dl) * dl.L));
    const int w = m < kBucketBases ? m : kBucketBases;
    const uint32_t pre = uint32_t(window(pk, p) >> (64 - 2 * kBucketBases)) & (~0u << (2 * (kBucketBases - w)));
    return (pre << 3) | uint32_t(w);
}

// every position's bucket (kept for the chunk passes, which then read 2 bytes a position) and the
// bucket histogram, counted in shared memory (kBuckets 32-bit counters, one CTA per SM) and added
// to the global histogram once per CTA
constexpr int kHistThreads = 1024;
__global__ void __launch_bounds__(kHistThreads) k_bucket_hist(const uint64_t* __restrict__ pk, size_t n, DivL dl,
                                                              uint16_t* __restrict__ bid,
                                                              unsigned long long* __restrict__ hist) {
    extern __shared__ unsigned s_hist[];
    for (int i = threadIdx.x; i < kBuckets; i += blockDim.x) s_hist[i] = 0;
    __syncthreads();
    // eight consecutive positions a thread a step: their windows come from the same two words of
    // the packed text (the first position is a multiple of 8), their read offsets from one
    // multiply-high, their buckets go out in one 16-byte store
    const size_t groups = (n + 7) / 8;
    const size_t stride = size_t(gridDim.x) * blockDim.x;
    for (size_t g = size_t(blockIdx.x) * blockDim.x + threadIdx.x; g < groups; g += stride) {
        const size_t p0 = g * 8;
        const uint64_t a = pk[p0 >> 5], b = pk[(p0 >> 5) + 1];
        const int s0 = int(p0 & 31);
        int off = int(uint32_t(p0 - div_l(p0, dl) * dl.L));
        uint32_t v[8];
        #pragma unroll
        for (int j = 0; j < 8; ++j) {
            const int sh = 2 * (s0 + j);
            const uint64_t x = sh ? ((a << sh) | (b >> (64 - sh))) : a;
            const int m = int(dl.L) - off;
            const int w = m < kBucketBases ? m : kBucketBases;
            const uint32_t pre = uint32_t(x >> (64 - 2 * kBucketBases)) & (~0u << (2 * (kBucketBases - w)));
            v[j] = (pre << 3) | uint32_t(w);
            if (p0 + size_t(j) < n) atomicAdd(&s_hist[v[j]], 1u);
            off = off + 1 == int(dl.L) ? 0 : off + 1;
        }
        if (p0 + 8 <= n) {
            *reinterpret_cast<uint4*>(bid + p0) =
                make_uint4(v[0] | (v[1] << 16), v[2] | (v[3] << 16), v[4] | (v[5] << 16), v[6] | (v[7] << 16));
        } else {
            for (int j = 0; j < 8; ++j)
                if (p0 + size_t(j) < n) bid[p0 + j] = uint16_t(v[j]);
        }
    }
    __syncthreads();
    for (int i = threadIdx.x; i < kBuckets; i += blockDim.x)
        if (s_hist[i]) atomicAdd(&hist[i], (unsigned long long)s_hist[i]);
}

// Chunk passes over tiles of kCkTile positions; warp w of a tile takes its positions
// [w * kCkSpan, (w + 1) * kCkSpan), 32 consecutive ones a step.  A bucket's chunk comes from a
// kBuckets-byte map (chunk numbers below kNoChunk).
constexpr int kCkThreads = 256;
constexpr int kCkWarps = kCkThreads / 32;
constexpr int kCkSpan = kCkTile / kCkWarps;
constexpr int kMaxChunks = 255;
constexpr unsigned kNoChunk = 0xffu;

// per tile and chunk: how many of the tile's positions fall in the chunk, into
// tcnt[chunk * ntiles + tile]
__global__ void __launch_bounds__(kCkThreads) k_chunk_tiles(const uint16_t* __restrict__ bid, size_t n,
                                                            const uint8_t* __restrict__ cmap, int nchunks,
                                                            size_t ntiles, unsigned long long* __restrict__ tcnt) {
    __shared__ uint8_t s_map[kBuckets];
    __shared__ unsigned s_cnt[kMaxChunks];
    for (int i = threadIdx.x; i < kBuckets; i += blockDim.x) s_map[i] = cmap[i];
    for (int c = threadIdx.x; c < nchunks; c += blockDim.x) s_cnt[c] = 0;
    __syncthreads();
    const int lane = threadIdx.x & 31;
    for (size_t tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
        const size_t t0 = tile * kCkTile;
        #pragma unroll 4
        for (int j = threadIdx.x; j < kCkTile; j += kCkThreads) {
            const size_t p = t0 + size_t(j);
            const unsigned c = p < n ? unsigned(s_map[bid[p]]) : kNoChunk;
            const unsigned peers = __match_any_sync(0xffffffffu, c);
            if (c != kNoChunk && lane == __ffs(peers) - 1) atomicAdd(&s_cnt[c], unsigned(__popc(peers)));
        }
        __syncthreads();
        for (int c = threadIdx.x; c < nchunks; c += blockDim.x) {
            tcnt[size_t(c) * ntiles + tile] = s_cnt[c];
            s_cnt[c] = 0;
        }
        __syncthreads();
    }
}

// Every position into its chunk's slice of `out`, in text order within the chunk.  toff is the
// exclusive scan of tcnt in chunk-major order: the chunk's slice start plus the tile's place in
// it.  A first walk over the tile counts each warp's positions per chunk, the warps' starts follow
// from those counts, and a second walk (over the same bytes, from L1) writes, each warp keeping a
// running offset per chunk.
template <class V>
__global__ void __launch_bounds__(kCkThreads) k_chunk_scatter(const uint16_t* __restrict__ bid, size_t n,
                                                              const uint8_t* __restrict__ cmap, int nchunks,
                                                              size_t ntiles,
                                                              const unsigned long long* __restrict__ toff,
                                                              V* __restrict__ out) {
    __shared__ uint8_t s_map[kBuckets];
    __shared__ unsigned s_run[kCkWarps][kMaxChunks];     // per warp and chunk: place within the tile
    __shared__ unsigned long long s_base[kMaxChunks];    // per chunk: the tile's start in `out`
    for (int i = threadIdx.x; i < kBuckets; i += blockDim.x) s_map[i] = cmap[i];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const unsigned below = (1u << lane) - 1u;
    for (size_t tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
        const size_t w0 = tile * kCkTile + size_t(warp) * kCkSpan;
        for (int c = lane; c < nchunks; c += 32) s_run[warp][c] = 0;
        __syncthreads();
        for (int k = 0; k < kCkSpan; k += 32) {
            const size_t p = w0 + size_t(k + lane);
            const unsigned c = p < n ? unsigned(s_map[bid[p]]) : kNoChunk;
            const unsigned peers = __match_any_sync(0xffffffffu, c);
            if (c != kNoChunk && lane == __ffs(peers) - 1) s_run[warp][c] += unsigned(__popc(peers));
            __syncwarp();
        }
        __syncthreads();
        for (int c = threadIdx.x; c < nchunks; c += blockDim.x) {
            s_base[c] = toff[size_t(c) * ntiles + tile];
            unsigned run = 0;
            for (int w = 0; w < kCkWarps; ++w) {
                const unsigned x = s_run[w][c];
                s_run[w][c] = run;
                run += x;
            }
        }
        __syncthreads();
        for (int k = 0; k < kCkSpan; k += 32) {
            const size_t p = w0 + size_t(k + lane);
            const unsigned c = p < n ? unsigned(s_map[bid[p]]) : kNoChunk;
            const unsigned peers = __match_any_sync(0xffffffffu, c);
            if (c != kNoChunk) out[s_base[c] + s_run[warp][c] + __popc(peers & below)] = V(p);
            __syncwarp();
            if (c != kNoChunk && lane == __ffs(peers) - 1) s_run[warp][c] += unsigned(__popc(peers));
            __syncwarp();
        }
        __syncthreads();
    }
}

// The counting pass for at most kFewChunks chunks (every index up to 8 G suffixes at the default
// capacity), without __match_any_sync: thread tid of a tile takes its 32 consecutive positions
// [tile * kCkTile + 32 tid, + 32) in four 16-byte loads, and keeps one counter per chunk in its own
// column of a shared array (no atomics, no bank conflicts): 3.3 times faster than k_chunk_tiles.
// (Scatters built the same way -- per-thread runs, or per-chunk ballots over 32 consecutive
// positions -- measured slower than k_chunk_scatter's __match_any_sync groups.)
constexpr int kFewChunks = 16;
constexpr int kCkPer = kCkTile / kCkThreads;          // 32 positions a thread

__device__ __forceinline__ void load_bids32(const uint16_t* __restrict__ bid, size_t p0, size_t n, uint32_t (&w)[16]) {
    if (p0 + kCkPer <= n) {
        #pragma unroll
        for (int q = 0; q < 4; ++q) {
            const uint4 x = *reinterpret_cast<const uint4*>(bid + p0 + 8 * q);
            w[4 * q] = x.x;
            w[4 * q + 1] = x.y;
            w[4 * q + 2] = x.z;
            w[4 * q + 3] = x.w;
        }
    } else {
        #pragma unroll
        for (int q = 0; q < 16; ++q) {
            const uint32_t lo = p0 + 2 * q < n ? bid[p0 + 2 * q] : 0xffffu;
            const uint32_t hi = p0 + 2 * q + 1 < n ? bid[p0 + 2 * q + 1] : 0xffffu;
            w[q] = lo | (hi << 16);
        }
    }
}

__global__ void __launch_bounds__(kCkThreads) k_chunk_tiles_few(const uint16_t* __restrict__ bid, size_t n,
                                                                const uint8_t* __restrict__ cmap, int nchunks,
                                                                size_t ntiles, unsigned long long* __restrict__ tcnt) {
    __shared__ uint8_t s_map[kBuckets + 1];
    __shared__ unsigned s_cnt[kFewChunks][kCkThreads];
    for (int i = threadIdx.x; i < kBuckets; i += blockDim.x) s_map[i] = cmap[i];
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    for (size_t tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
        #pragma unroll
        for (int c = 0; c < kFewChunks; ++c) s_cnt[c][tid] = 0;
        __syncthreads();
        const size_t p0 = tile * kCkTile + size_t(tid) * kCkPer;
        if (p0 < n) {
            uint32_t w[16];
            load_bids32(bid, p0, n, w);
            #pragma unroll
            for (int j = 0; j < kCkPer; ++j) {
                const uint32_t b = (w[j >> 1] >> (16 * (j & 1))) & 0xffffu;
                if (b != 0xffffu) ++s_cnt[s_map[b]][tid];
            }
        }
        __syncthreads();
        for (int c = warp; c < nchunks; c += kCkWarps) {
            unsigned sum = 0;
            for (int i = lane; i < kCkThreads; i += 32) sum += s_cnt[c][i];
            #pragma unroll
            for (int o = 16; o > 0; o >>= 1) sum += __shfl_down_sync(0xffffffffu, sum, o);
            if (lane == 0) tcnt[size_t(c) * ntiles + tile] = sum;
        }
        __syncthreads();
    }
}

// the chunk's keys, and its positions copied from their slice of the suffix array into the radix
// sort's value buffer (which starts 16-byte aligned, as the sort's staged tiles want)
template <class V>
__global__ void k_init_keys_list(const uint64_t* __restrict__ pk, const V* __restrict__ list, size_t m, DivL dl,
                                 uint32_t* __restrict__ key, V* __restrict__ val) {
    const size_t stride = size_t(gridDim.x) * blockDim.x;
    for (size_t i = size_t(blockIdx.x) * blockDim.x + threadIdx.x; i < m; i += stride) {
        const V v = list[i];
        const size_t p = size_t(v);
        key[i] = make_key<uint32_t>(window(pk, p), int(dl.L - uint32_t(p - div_l(p, dl) * dl.L)));
        val[i] = v;
    }
}

// chunks a greedy packing of buckets into `cap` can make: every chunk but the last is over half
// full or ends before a bucket of more than half a chunk, so at most 2 n / cap + 2
static size_t chunk_bound(size_t n, size_t cap) {
    return std::min<size_t>(size_t(kMaxChunks), 2 * ((n + cap - 1) / cap) + 2);
}

static size_t chunk_parts(size_t n, size_t cap, size_t (&b)[11]) {
    const size_t ntiles = (n + kCkTile - 1) / kCkTile;
    b[0] = cap * sizeof(uint64_t);                    // ka (32-bit head keys; 64-bit for big groups)
    b[1] = cap * sizeof(uint64_t);                    // kb (also the group lists)
    b[2] = cap * sizeof(idx_t);                       // va
    b[3] = cap * sizeof(idx_t);                       // vb (with rank: big-group columns)
    b[4] = cap * sizeof(uint32_t);                    // rank
    b[5] = (n / 32 + 4) * sizeof(uint64_t);           // packed text
    b[6] = radix_tmp_bytes(cap);
    b[7] = (chunk_bound(n, cap) * ntiles + 1) * sizeof(unsigned long long);   // tile counts / offsets
    b[8] = (size_t(kBuckets) + 8) * sizeof(unsigned long long) + size_t(kBuckets);   // histogram, counters, map
    b[9] = n;                                         // BWT symbols of the refined rows
    b[10] = n * sizeof(uint16_t);                     // every position's 6-base bucket
    size_t t = 0;
    for (size_t x : b) t += al(x);
    return t + 1024;
}

size_t suffix_sort_chunked_tmp_bytes(size_t n, size_t cap) {
    size_t b[11];
    return chunk_parts(n, cap, b);
}

int suffix_sort_chunked(const uint8_t* reads, idx_t num_reads, int L, int dir, idx_t* sa, size_t cap, void* tmp,
                        size_t tmp_bytes, cudaStream_t st, const uint8_t** bwt_out, uint64_t* pk_out,
                        idx_t* isa_out, idx_t isa_m, idx_t* kstart, idx_t* kend, int kmer_k) {
    if (bwt_out) *bwt_out = nullptr;
    const size_t n = size_t(num_reads) * size_t(L);
    if (n == 0) return 0;
    if (cap < 2 || cap >= (size_t(1) << 31)) return int(cudaErrorInvalidValue);
    size_t b[11];
    if (tmp_bytes < chunk_parts(n, cap, b)) return int(cudaErrorInvalidValue);
    char* q = static_cast<char*>(tmp);
    char* part[11];
    for (int i = 0; i < 11; ++i) {
        part[i] = q;
        q += al(b[i]);
    }
    uint64_t* ka0 = reinterpret_cast<uint64_t*>(part[0]);
    uint64_t* kb0 = reinterpret_cast<uint64_t*>(part[1]);
    idx_t* va0 = reinterpret_cast<idx_t*>(part[2]);
    idx_t* vb0 = reinterpret_cast<idx_t*>(part[3]);
    uint64_t* pk = pk_out ? pk_out : reinterpret_cast<uint64_t*>(part[5]);
    void* rtmp = part[6];
    uint8_t* bwt = bwt_out ? reinterpret_cast<uint8_t*>(part[9]) : nullptr;
    if (bwt) cudaMemsetAsync(bwt, 0xff, n, st);
    unsigned long long* tcnt = reinterpret_cast<unsigned long long*>(part[7]);
    unsigned long long* hist = reinterpret_cast<unsigned long long*>(part[8]);
    unsigned long long* counters = hist + kBuckets;
    uint16_t* bid = reinterpret_cast<uint16_t*>(part[10]);
    uint8_t* cmap = reinterpret_cast<uint8_t*>(counters + 8);
    const DivL dl = make_divl(uint32_t(L));
    const size_t nwords = n / 32 + 4;
    const size_t ntiles = (n + kCkTile - 1) / kCkTile;
    int dev = 0, sms = 152;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    { k_pack_text<<<grid_for(nwords, 256), 256, 0, st>>>(reads, n, idx_t(L), dir, nwords, pk); note_launch(); }
    cudaMemsetAsync(hist, 0, size_t(kBuckets) * sizeof(unsigned long long), st);
    const size_t hsm = size_t(kBuckets) * sizeof(unsigned);
    cudaFuncSetAttribute(k_bucket_hist, cudaFuncAttributeMaxDynamicSharedMemorySize, int(hsm));
    { k_bucket_hist<<<unsigned(sms), kHistThreads, hsm, st>>>(pk, n, dl, bid, hist); note_launch(); }
    std::vector<unsigned long long> h(kBuckets);
    cudaMemcpyAsync(h.data(), hist, h.size() * sizeof(unsigned long long), cudaMemcpyDeviceToHost, st);
    cudaError_t e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) return int(e);
    // chunks: runs of consecutive buckets that fit the capacity, each a slice of the suffix array
    std::vector<uint8_t> map(kBuckets, uint8_t(kNoChunk));
    struct Chunk {
        size_t offset, m;
    };
    std::vector<Chunk> chunks;
    {
        size_t offset = 0;
        uint32_t lo = 0;
        while (lo < uint32_t(kBuckets)) {
            uint32_t hi = lo;
            size_t m = 0;
            while (hi < uint32_t(kBuckets) && m + h[hi] <= cap) m += h[hi++];
            if (hi == lo) return int(cudaErrorNotSupported);          // one bucket larger than a chunk
            if (m) {
                if (chunks.size() >= chunk_bound(n, cap)) return int(cudaErrorNotSupported);
                for (uint32_t b = lo; b < hi; ++b) map[b] = uint8_t(chunks.size());
                chunks.push_back({offset, m});
            }
            offset += m;
            lo = hi;
        }
    }
    const int nchunks = int(chunks.size());
    cudaMemcpyAsync(cmap, map.data(), map.size(), cudaMemcpyHostToDevice, st);
    // every position into its chunk's slice of the suffix array, in text order: tile counts per
    // chunk, their scan in chunk-major order (the slices' starts included), the scatter
    const unsigned cgrid = unsigned(std::min<size_t>(ntiles, size_t(sms) * 8));
    if (nchunks <= kFewChunks) {
        k_chunk_tiles_few<<<cgrid, kCkThreads, 0, st>>>(bid, n, cmap, nchunks, ntiles, tcnt);
    } else {
        k_chunk_tiles<<<cgrid, kCkThreads, 0, st>>>(bid, n, cmap, nchunks, ntiles, tcnt);
    }
    note_launch();
    { k_scan_small<<<1, 1024, 0, st>>>(tcnt, size_t(nchunks) * ntiles); note_launch(); }
    { k_chunk_scatter<idx_t><<<cgrid, kCkThreads, 0, st>>>(bid, n, cmap, nchunks, ntiles, tcnt, sa); note_launch(); }
    for (const Chunk& ck : chunks) {
        const size_t offset = ck.offset, m = ck.m;
        {
            uint32_t* ka = reinterpret_cast<uint32_t*>(ka0);
            uint32_t* kb = reinterpret_cast<uint32_t*>(kb0);
            { k_init_keys_list<idx_t><<<grid_for(m, 256), 256, 0, st>>>(pk, sa + offset, m, dl, ka, va0); note_launch(); }
            idx_t* va = va0;
            idx_t* vb = vb0;
            int rc = radix_sort_pairs<uint32_t, idx_t>(&ka, &va, &kb, &vb, m, 0, 32, rtmp, radix_tmp_bytes(m), st, false);
            if (rc) return rc;
            if (size_t(L) > size_t(kHead)) {
                // scratch: the free value buffer, and rank behind it when that is the second buffer
                uint64_t* cols = reinterpret_cast<uint64_t*>(vb);
                const size_t cols_cap = (vb == vb0 ? al(b[3]) + b[4] : al(b[2])) / sizeof(uint64_t);
                rc = refine_groups(ka, va, m, idx_t(L), pk, reinterpret_cast<uint64_t*>(kb), cols, cols_cap, counters,
                                   rtmp, radix_tmp_bytes(m), st, bwt, isa_out, isa_m, offset);
                if (rc > 0) return rc;
                if (rc < 0) return int(cudaErrorNotSupported);      // would need prefix doubling
            }
            { k_copy_vals<idx_t><<<grid_for(m, 256), 256, 0, st>>>(va, m, sa + offset); note_launch(); }
            // the chunk's keys are still sorted and aligned with its rows (the refinement only
            // reorders rows of equal keys): its k-mers' row ranges
            if (kstart && kmer_k >= 6 && kmer_k <= kSortKeyBases) {
                const cudaError_t ek = kmer_table_from_keys(ka, m, offset, kmer_k, kstart, kend, st);
                if (ek != cudaSuccess) return int(ek);
            }
        }
    }
    if (bwt_out) *bwt_out = bwt;
    return int(cudaGetLastError());
}

}  // namespace pq
