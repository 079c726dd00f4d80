// pq_common.cuh — shared types for the GB300 build of PASQUAL's hot path.
//
// Index width follows the reference's INDEX_LENGTH split (src/common.h:31-44): the library is
// compiled twice, with and without -DPQ_IDX64, exactly as the reference builds
// bin/pasqual_omp_u32 and _u64.
#pragma once

#include <cstdint>
#include <cstddef>
#include <cuda_runtime.h>

#ifdef PQ_IDX64
typedef uint64_t idx_t;
#else
typedef uint32_t idx_t;
#endif

// Base codes, as the reference stores them after import (src/index.c:282-303): $=0 A=1 C=2 G=3 T=4.
// Edge types (src/string_graph.h:14-18).
enum : int { PQ_BF = 0, PQ_FB = 1, PQ_FF = 2, PQ_BB = 3 };

// ---------------------------------------------------------------------------------------------
// Occurrence structure ("occ block"): one 32-byte sector covers 64 BWT rows, so one rank query is
// one sector (plus an L2-resident superblock word).
//
//   lo, hi : bit j = low / high bit of the 2-bit base code (A=0..T=3) of row 64b+j
//   dol    : bit j set <=> row 64b+j is a `$` row (read-start suffix); lo = hi = 0 there
//   cnt[c] : # of base c+1 in rows [65536*(b/1024), 64b)  (relative to the superblock)
//
// Superblock (65536 rows): sb[4*s + c] = # of base c+1 in rows [0, 65536*s).
// rank_c(pos) = sb + cnt + popc(match_c & below(pos));  rank_$(pos) = pos - sum_c rank_c(pos).
// The reference's OCC(c, pos) (src/string_graph.c:11-23) equals fix[c] + rank_c(pos) for c >= 1
// and rank_$(pos) for c = 0, where fix = suffix_count (forward) / prefix_count (backward).
// ---------------------------------------------------------------------------------------------
struct __align__(32) OccBlock {
    uint64_t lo, hi, dol;
    uint16_t cnt[4];
};
static_assert(sizeof(OccBlock) == 32, "occ block must be one 32-byte sector");

constexpr int kBlockShift = 6;                    // 64 rows per block
constexpr int kSuperShift = 16;                   // 65536 rows per superblock
constexpr int kBlocksPerSuper = 1 << (kSuperShift - kBlockShift);

// Device view of one direction's learned index (pq_learned.cuh): segment boundary keys, the
// root's row at each boundary, per-segment MLP parameters, per-segment window bounds
// (e_lo, e_hi) and the segment of each 16-bit key prefix.
struct LearnedView {
    const uint32_t* bnd;      // [S] first key of each segment (bnd[0] = 0); segment S-1 ends at 2^32
    const idx_t* base;        // [S + 1] rows with a smaller key; base[S] = number of rows
    const float* par;         // [S * 196] w1[64] b1[64] w2[64] b2, padded
    const int32_t* err;       // [2 S] e_lo, e_hi
    const uint16_t* segof;    // [65537] segment holding key h << 16 (segof[65536] = S - 1)
    int segs;                 // S (0 = no model)
};

// Device view of one FM-index direction.
struct FmView {
    const OccBlock* blk;      // n/64 + 1 blocks
    const idx_t* sb;          // 4 per superblock
    const idx_t* reads_index; // read id of the k-th `$` row
    const idx_t* kstart;      // k-mer seed table: first row of each k-mer (or nullptr)
    const idx_t* kend;        // last row (kend < kstart when the k-mer is absent)
    const idx_t* sa;          // suffix array (for seeds found by binary search), or nullptr
    const uint64_t* pk;       // the text, 32 bases per word, first base in the top bits
    const idx_t* isa;         // row of the suffix at read offset o (1 <= o <= L - t) of read r at
                              // isa[r * (L - t) + o - 1], or nullptr
    LearnedView lx;           // learned index of 16-base keys (lx.segs = 0 when absent)
    idx_t Cf[5];              // Cf[0] = C[0]; Cf[c] = C[c] + fix[c]  (LF-mapping base)
};

// Division of a text position by the read length L without a 64-bit divide: with
// m = floor((2^64 - 1) / L) + 1, floor(p / L) = high 64 bits of p * m for every p < 2^64 / L (so
// for every position of an index below 2^48 suffixes, L <= 65535): the product's excess over p / L
// is below p / 2^64 < 1 / L, too small to reach the next integer.
struct DivL {
    uint64_t m;
    uint32_t L;
};
inline DivL make_divl(uint32_t L) { return DivL{~uint64_t(0) / L + 1, L}; }
__device__ __forceinline__ uint64_t div_l(uint64_t p, const DivL& d) { return __umul64hi(p, d.m); }

namespace pq {
// Count of kernels this library has launched (reported through pq_get_kernel_stats).
void note_launch();
unsigned long long launch_count();
}  // namespace pq

// Status codes returned through the C ABI.
enum : int {
    PQ_OK = 0,
    PQ_ERR_ARG = 1,
    PQ_ERR_CUDA = 2,
    PQ_ERR_NOMEM = 3,
    PQ_ERR_TOO_MANY_EDGES = 4,   // a read has more than 65535 edges on one side
    PQ_ERR_STATE = 5,
    PQ_ERR_CAPACITY = 6,
    PQ_ERR_INTERNAL = 7,
};

// Per-read overflow reasons recorded by the fast search kernel (the read is redone by the
// wide-scratch kernel).
enum : uint8_t { OVF_NONE = 0, OVF_STACK = 1, OVF_EDGES = 2, OVF_LEVELS = 3, OVF_POOL = 4,
                 ERR_TOO_MANY = 16, ERR_CAP = 17 };
