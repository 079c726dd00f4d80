// pq_sort.cuh — GPU suffix sort of read-bounded suffixes (internal).
#pragma once
#include "pq_common.cuh"

namespace pq {

size_t suffix_sort_tmp_bytes(size_t n);

// Suffix array of direction dir in the canonical order (suffix string with end-of-read lowest,
// then text position).  Returns 0 or a cudaError_t value.  When keys_out is given it receives
// the sorted 32-bit keys (first 14 bases in bits 31..4, then min(length, 14) in bits 3..0)
// aligned with the suffix array, inside tmp (valid until tmp is reused), or nullptr when the sort
// ended by prefix doubling (the key array then holds ranks).  When bwt_out is given it receives
// the BWT symbols (0 = `$`, 1..4) of the rows the group refinement placed, 0xff for the others,
// inside tmp, or nullptr.  pk_out (n/32 + 4 words), when given, receives the packed text of the
// direction (see pack_text) instead of tmp.  isa_out (num_reads * isa_m entries), when given
// together with bwt_out, receives the inverse-SA entries isa[read * isa_m + offset - 1] of the
// rows the refinement placed (those with a BWT symbol); the other rows' entries are left for the
// caller.  Without bwt_out the sort computes neither (suffix array only).
constexpr int kSortKeyBases = 14;
int suffix_sort(const uint8_t* reads, idx_t num_reads, int L, int dir, idx_t* sa, void* tmp,
                size_t tmp_bytes, cudaStream_t st, const uint32_t** keys_out = nullptr,
                const uint8_t** bwt_out = nullptr, uint64_t* pk_out = nullptr, idx_t* isa_out = nullptr,
                idx_t isa_m = 0);

// The same order for inputs too large for one pass: suffixes bucketed by their first 6 bases,
// consecutive buckets sorted in chunks of at most cap (< 2^31) suffixes.  Returns
// cudaErrorNotSupported if one bucket exceeds cap.  bwt_out and pk_out as for suffix_sort.
size_t suffix_sort_chunked_tmp_bytes(size_t n, size_t cap);
// kstart/kend (cleared by the caller), when given, receive the k-mer table (6 <= k <= 14) from each
// chunk's sorted keys.
int suffix_sort_chunked(const uint8_t* reads, idx_t num_reads, int L, int dir, idx_t* sa, size_t cap, void* tmp,
                        size_t tmp_bytes, cudaStream_t st, const uint8_t** bwt_out = nullptr,
                        uint64_t* pk_out = nullptr, idx_t* isa_out = nullptr, idx_t isa_m = 0,
                        idx_t* kstart = nullptr, idx_t* kend = nullptr, int kmer_k = 0);

// Per-read seeds from a k-mer table (pq_index.cu).
cudaError_t read_seeds(const uint8_t* reads, idx_t num_reads, int L, int dir, int k, const idx_t* kstart,
                       const idx_t* kend, idx_t* start, idx_t* size, cudaStream_t st);

// Stable LSD radix sort of (key, value) pairs on the bits [lo_bit, hi_bit) of the key (K is
// uint32_t or uint64_t).  Buffers are ping-ponged; the sorted result ends in (*k0, *v0) (pointers
// may be swapped).  skip_trivial: first histogram every digit (one pass and a host round trip)
// and skip the digits that are constant over all keys; else run every digit pass.
template <class K, class V>
int radix_sort_pairs(K** k0, V** v0, K** k1, V** v1, size_t n, int lo_bit, int hi_bit,
                     void* tmp, size_t tmp_bytes, cudaStream_t st, bool skip_trivial = true);
size_t radix_tmp_bytes(size_t n);

// The text of direction dir packed 32 bases per 64-bit word, first base in the top bits
// (n/32 + 4 words; the last words are zero padding).
cudaError_t pack_text(const uint8_t* reads, size_t n, idx_t L, int dir, uint64_t* pk, cudaStream_t st);

}  // namespace pq
