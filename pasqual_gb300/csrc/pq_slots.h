// pq_slots.h — the sort-slot sizes of the reference's initial_sort (src/sufsort.c:386-450), for
// the index_t fields size_fw/offset_fw/max_size_fw and their _bw twins (host code).
//
// Every suffix of every read falls in one of 85 first-prefix ranks: its first min(3, remaining)
// bases in the order of strings of length 1..3 where a string comes before its extensions
// (rank = sum over its bases i of base_i * span(i + 1) + 1, spans 21, 5, 1); slot k holds the
// ranks 17k .. 17k + 16.  Direction 1 is every read reversed.  The reads are counted in parallel
// (one 85-bin histogram per thread), three bases at a time.
#pragma once
#include <algorithm>
#include <cstddef>
#include <cstdint>
#include <thread>
#include <vector>

namespace pq_slots {

// histogram of the 85 first-prefix ranks over all suffixes (reads: codes 1..4, read-major)
inline void prefix_rank_histogram(const uint8_t* reads, size_t num_reads, int L, int dir, uint64_t hist[85],
                                  int threads) {
    for (int i = 0; i < 85; ++i) hist[i] = 0;
    if (num_reads == 0 || L <= 0) return;
    threads = std::max(1, std::min<int>(threads, int((num_reads + 1023) / 1024)));
    std::vector<std::vector<uint64_t>> part(threads, std::vector<uint64_t>(85, 0));
    auto work = [&](size_t b, size_t e, std::vector<uint64_t>& h) {
        for (size_t r = b; r < e; ++r) {
            const uint8_t* s = reads + r * size_t(L);
            // base j of the read in this direction, 0..3
            auto at = [&](int j) { return int(dir ? s[L - 1 - j] : s[j]) - 1; };
            for (int j = 0; j + 2 < L; ++j) h[21 * at(j) + 5 * at(j + 1) + at(j + 2) + 3]++;
            if (L >= 2) h[21 * at(L - 2) + 5 * at(L - 1) + 2]++;
            h[21 * at(L - 1) + 1]++;
        }
    };
    std::vector<std::thread> th;
    const size_t chunk = (num_reads + threads - 1) / threads;
    for (int t = 0; t < threads; ++t) {
        const size_t b = size_t(t) * chunk, e = std::min(num_reads, b + chunk);
        if (b >= e) break;
        th.emplace_back([&, b, e, t] { work(b, e, part[t]); });
    }
    for (auto& x : th) x.join();
    for (const auto& p : part)
        for (int i = 0; i < 85; ++i) hist[i] += p[i];
}

// size[k] = suffixes in slot k, off[k] = suffixes in the slots before it, *max_size = the largest
template <class IDX>
inline void slot_sizes(const uint8_t* reads, size_t num_reads, int L, int dir, IDX size[5], IDX off[5], IDX* max_size,
                       int threads) {
    uint64_t hist[85];
    prefix_rank_histogram(reads, num_reads, L, dir, hist, threads);
    IDX mx = 0;
    for (int k = 0; k < 5; ++k) {
        size[k] = 0;
        for (int j = 0; j < 17; ++j) size[k] += IDX(hist[k * 17 + j]);
        off[k] = k ? off[k - 1] + size[k - 1] : 0;
        mx = std::max(mx, size[k]);
    }
    *max_size = mx;
}

}  // namespace pq_slots
