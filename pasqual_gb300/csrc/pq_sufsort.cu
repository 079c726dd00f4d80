// pq_sufsort.cu — the reference's suffix-sort entry points (src/sufsort.h:29-46) with their own
// signatures, served by this library: transform_to_triplet, transform_to_triplet_reverse,
// initial_sort and suf_sort.  A caller that drives them the way build_idx does
// (src/index.c:558-585) gets, slot by slot, the reference's suffix array and seed intervals.
//
// The triplet recoding and the first-prefix histogram are single streaming passes over host
// memory, so they run on the host (every core).  suf_sort runs on the GPU: the recoded text is
// decoded back to base codes (the first base of each triplet), its whole suffix array is sorted
// once on the device and kept, keyed by the text's address, size and a checksum of its bytes, so
// the five slot calls over one text sort once; each call copies its slot's rows out and applies
// the seed records of the sort buckets inside the slot (pq_seeds.cu).  The reference's per-read
// OpenMP locks are not needed and the read_lock argument is ignored.
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <mutex>
#include <string>
#include <thread>
#include <vector>

#include "pq_common.cuh"
#include "../../include/pasqual_gb300.h"
#include "../../include/pasqual_gb300_dropin.h"

static_assert(sizeof(pq_index_type) == sizeof(idx_t), "index widths must agree");

// pq_api.cu (not in the public header)
extern "C" int pq_get_sa_rows(pq_ctx* ctx, int dir, uint64_t first, uint64_t count, pq_idx* host);
extern "C" int pq_apply_sort_seeds(pq_ctx* ctx, int dir, uint64_t r0, uint64_t r1, pq_idx* start, pq_idx* size,
                                   uint16_t* depth);

namespace {

constexpr int kSlotDepth = 5;    // SLOT_DEPTH, src/common.h:51
constexpr int kSlotNum = 17;     // SLOT_NUM, src/common.h:52

// Rank of a string of 1..3 bases (codes 1..4) in the order of all strings of length 0..3 with a
// string before its extensions: the first base spans 21 ranks, the second 5, the third 1.  This is
// the order-preserving code the reference tabulates (triplet_table, src/sufsort.c:21-30).
inline char triplet_rank(int n, int c0, int c1, int c2) {
    int r = 1 + 21 * (c0 - 1);
    if (n > 1) r += 1 + 5 * (c1 - 1);
    if (n > 2) r += 1 + (c2 - 1);
    return char(r);
}

template <class F>
void parallel_reads(size_t num_reads, F f) {
    const size_t hw = std::max(1u, std::thread::hardware_concurrency());
    const size_t threads = std::max<size_t>(1, std::min(hw, (num_reads + 4095) / 4096));
    if (threads == 1) {
        f(size_t(0), num_reads);
        return;
    }
    std::vector<std::thread> th;
    const size_t chunk = (num_reads + threads - 1) / threads;
    for (size_t t = 0; t < threads; ++t) {
        const size_t b = t * chunk, e = std::min(num_reads, b + chunk);
        if (b >= e) break;
        th.emplace_back([&f, b, e] { f(b, e); });
    }
    for (auto& x : th) x.join();
}

// byte j of a read becomes the rank of its bases j .. min(j + 2, L - 1), read in `dir` order
void recode(char* reads, int L, size_t num_reads, bool reverse) {
    if (L <= 0) return;
    parallel_reads(num_reads, [&](size_t b, size_t e) {
        std::vector<char> tmp(static_cast<size_t>(L));
        for (size_t r = b; r < e; ++r) {
            char* s = reads + r * size_t(L);
            auto at = [&](int j) { return int(reverse ? s[L - 1 - j] : s[j]); };
            for (int j = 0; j < L; ++j) {
                const int n = L - j < 3 ? L - j : 3;
                tmp[size_t(j)] = triplet_rank(n, at(j), n > 1 ? at(j + 1) : 1, n > 2 ? at(j + 2) : 1);
            }
            memcpy(s, tmp.data(), size_t(L));
        }
    });
}

uint64_t text_checksum(const char* p, size_t n) {
    const size_t hw = std::max(1u, std::thread::hardware_concurrency());
    const size_t threads = std::max<size_t>(1, std::min(hw, n >> 22));
    std::vector<uint64_t> part(threads, 0);
    std::vector<std::thread> th;
    const size_t chunk = (n + threads - 1) / threads;
    for (size_t t = 0; t < threads; ++t) {
        th.emplace_back([&, t] {
            const size_t b = std::min(n, t * chunk), e = std::min(n, b + chunk);
            uint64_t h = 0x9e3779b97f4a7c15ull ^ (t + 1);
            size_t i = b;
            for (; i + 8 <= e; i += 8) {
                uint64_t w;
                memcpy(&w, p + i, 8);
                h = (h ^ w) * 0xff51afd7ed558ccdull;
                h ^= h >> 29;
            }
            for (; i < e; ++i) h = (h ^ uint8_t(p[i])) * 0xc4ceb9fe1a85ec53ull;
            part[t] = h;
        });
    }
    for (auto& x : th) x.join();
    uint64_t h = n;
    for (uint64_t v : part) h = (h ^ v) * 0x9e3779b97f4a7c15ull;
    return h;
}

[[noreturn]] void sufsort_error(const std::string& msg) {
    // the reference's ERROR_EXIT convention (src/common.h:87-94)
    fprintf(stderr, "Error: %s\n", msg.c_str());
    fflush(stderr);
    exit(0);
}

// The sorted text of the last suf_sort calls.
struct SortedText {
    std::mutex mu;
    pq_ctx* ctx = nullptr;
    const char* text = nullptr;
    size_t n = 0;
    int L = 0, t = 0;
    uint64_t sum = 0;
};
SortedText g_sorted;

}  // namespace

extern "C" {

void transform_to_triplet(char* reads, int read_len, pq_index_type num_reads) {
    recode(reads, read_len, size_t(num_reads), false);
}

void transform_to_triplet_reverse(char* reads, int read_len, pq_index_type num_reads) {
    recode(reads, read_len, size_t(num_reads), true);
}

void initial_sort(char* reads, pq_index_type num_elems, pq_bucket_t* bkt, pq_index_type* bsize,
                  pq_index_type* boffset, pq_index_type* max_size) {
    const size_t n = size_t(num_elems);
    const size_t hw = std::max(1u, std::thread::hardware_concurrency());
    const size_t threads = std::max<size_t>(1, std::min(hw, n >> 20));
    std::vector<std::vector<uint64_t>> part(threads, std::vector<uint64_t>(PQ_NUM_SLOTS, 0));
    std::vector<std::thread> th;
    const size_t chunk = (n + threads - 1) / threads;
    for (size_t t = 0; t < threads; ++t) {
        th.emplace_back([&, t] {
            const size_t b = std::min(n, t * chunk), e = std::min(n, b + chunk);
            for (size_t i = b; i < e; ++i) part[t][size_t(uint8_t(reads[i]))]++;
        });
    }
    for (auto& x : th) x.join();
    for (int k = 0; k < PQ_NUM_SLOTS; ++k) {
        uint64_t f = 0;
        for (size_t t = 0; t < threads; ++t) f += part[t][size_t(k)];
        bkt->freqs[k] = pq_index_type(f);
    }
    // offsets restart at 0 in every slot; slots follow one another (src/sufsort.c:429-449)
    pq_index_type msize = 0;
    for (int k = 0; k < kSlotDepth; ++k) {
        bkt->offs[k * kSlotNum] = 0;
        bsize[k] = bkt->freqs[k * kSlotNum];
        for (int j = 1; j < kSlotNum; ++j) {
            bsize[k] += bkt->freqs[k * kSlotNum + j];
            bkt->offs[k * kSlotNum + j] = bkt->offs[k * kSlotNum + j - 1] + bkt->freqs[k * kSlotNum + j - 1];
        }
        if (bsize[k] > msize) msize = bsize[k];
    }
    boffset[0] = 0;
    for (int k = 1; k < kSlotDepth; ++k) boffset[k] = boffset[k - 1] + bsize[k - 1];
    *max_size = msize;
}

void suf_sort(pq_index_type* sa, char* reads, int slot, pq_index_type* new_idx, pq_bucket_t* bkt0,
              pq_index_type num_elems, int read_len, pq_index_type* interval_start, pq_index_type* interval_end,
              uint16_t* interval_depth, void* read_lock, pq_index_type bkt_offset, int min_overlap) {
    (void)read_lock;
    if (slot < 0 || slot >= kSlotDepth || read_len <= 0) sufsort_error("invalid suf_sort slot or read length");
    const size_t n = size_t(num_elems);
    if (n % size_t(read_len)) sufsort_error("num_elems is not a multiple of read_len");
    const size_t nr = n / size_t(read_len);
    std::lock_guard<std::mutex> g(g_sorted.mu);
    const uint64_t sum = text_checksum(reads, n);
    if (!g_sorted.ctx || g_sorted.text != reads || g_sorted.n != n || g_sorted.L != read_len ||
        g_sorted.t != min_overlap || g_sorted.sum != sum) {
        if (!g_sorted.ctx && pq_create(&g_sorted.ctx, 0, nullptr) != PQ_OK) sufsort_error("no usable CUDA device.");
        g_sorted.text = nullptr;
        // the first base of each triplet: (rank - 1) / 21 + 1
        std::vector<uint8_t> codes(n);
        parallel_reads(nr, [&](size_t b, size_t e) {
            for (size_t i = b * size_t(read_len); i < e * size_t(read_len); ++i)
                codes[i] = uint8_t((uint8_t(reads[i]) - 1) / 21 + 1);
        });
        if (pq_set_reads(g_sorted.ctx, codes.data(), pq_idx(nr), read_len, min_overlap, 0) != PQ_OK ||
            pq_sort(g_sorted.ctx, 0) != PQ_OK)
            sufsort_error(pq_last_error(g_sorted.ctx));
        g_sorted.text = reads;
        g_sorted.n = n;
        g_sorted.L = read_len;
        g_sorted.t = min_overlap;
        g_sorted.sum = sum;
    }
    // the slot's rows, and the scatter offsets step 1 of the reference advances
    // (src/sufsort.c:485-538): every first-prefix rank of the slot by its frequency
    pq_index_type size = 0;
    for (int j = 0; j < kSlotNum; ++j) {
        const int k = slot * kSlotNum + j;
        size += bkt0->freqs[k];
        new_idx[k] += bkt0->freqs[k];
    }
    if (pq_get_sa_rows(g_sorted.ctx, 0, uint64_t(bkt_offset), uint64_t(size), reinterpret_cast<pq_idx*>(sa)) !=
            PQ_OK ||
        pq_apply_sort_seeds(g_sorted.ctx, 0, uint64_t(bkt_offset), uint64_t(bkt_offset) + uint64_t(size),
                            reinterpret_cast<pq_idx*>(interval_start), reinterpret_cast<pq_idx*>(interval_end),
                            interval_depth) != PQ_OK)
        sufsort_error(pq_last_error(g_sorted.ctx));
}

}  // extern "C"
