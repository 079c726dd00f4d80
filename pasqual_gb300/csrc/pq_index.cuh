// pq_index.cuh — device-side index construction and search entry points (internal).
#pragma once
#include "pq_common.cuh"

namespace pq {

// FM-index build from a suffix array (pq_index.cu)
// pk: the packed text of direction dir (preferred for the BWT gathers), or nullptr; hint: the
// sort's per-row BWT symbols (0xff = none), or nullptr
cudaError_t build_occ(const idx_t* sa, const uint8_t* reads, idx_t num_reads, idx_t L, int dir,
                      OccBlock* blk, idx_t* sb, idx_t* reads_index, cudaStream_t st, const uint64_t* pk = nullptr,
                      const uint8_t* hint = nullptr);
// out13: base counts [4], last-base counts [4], first-base counts [4], bytes outside 1..4
// n bytes between device memory and page-locked host memory (at its device-accessible address),
// copied by a kernel
cudaError_t kernel_copy(void* dst, const void* src, size_t n, cudaStream_t st);
cudaError_t read_counts(const uint8_t* reads, idx_t num_reads, idx_t L, unsigned long long* out13,
                        cudaStream_t st);
// k-mer table of direction dir: from the sort's keys when sorted_keys is given, else from the
// suffix array and the packed text pk (each one streaming pass)
cudaError_t build_kmer_table(const idx_t* sa, idx_t num_reads, idx_t L, int k, idx_t* kstart, idx_t* kend,
                             cudaStream_t st, const uint32_t* sorted_keys, const uint64_t* pk);
// The k-mer table in parts: cleared (every k-mer absent), then entered from runs of sorted keys
// (rows off .. off + m - 1), as each chunk of a chunked sort finishes.
cudaError_t kmer_table_clear(int k, idx_t* kstart, idx_t* kend, cudaStream_t st);
cudaError_t kmer_table_from_keys(const uint32_t* keys, size_t m, size_t off, int k, idx_t* kstart, idx_t* kend,
                                 cudaStream_t st);
// rows of the suffixes at read offsets 1..M (isa[read * M + offset - 1]); M = L - t.  hint: the
// sort's BWT symbols, whose rows (symbol != 0xff) the sort has already entered, or null (all rows)
cudaError_t build_isa(const idx_t* sa, size_t n, idx_t L, idx_t M, idx_t* isa, cudaStream_t st,
                      const uint8_t* hint = nullptr);
// The per-read seed intervals the reference's sort records (index_t.interval_start/end/depth,
// src/sufsort.c:178-209, 322-334) from a finished suffix array and the packed text of its
// direction (pq_seeds.cu).  seed_init writes the depth-1 seeds build_idx starts from; sort_seeds
// then deepens them with the records of the buckets in rows [r0, r1).
cudaError_t seed_init(const uint8_t* reads, idx_t num_reads, idx_t L, int dir, const idx_t C[6], uint16_t* depth,
                      idx_t* start, idx_t* size, cudaStream_t st);
size_t sort_seeds_tmp_bytes(size_t rows);
cudaError_t sort_seeds(const idx_t* sa, const uint64_t* pk, idx_t L, int t, size_t r0, size_t r1, uint16_t* depth,
                       idx_t* start, idx_t* size, void* tmp, size_t tmp_bytes, cudaStream_t st);
cudaError_t export_ref_layout(const OccBlock* blk, const idx_t* sb, idx_t num_reads, idx_t L,
                              const idx_t fix[4], uint64_t* bitmap, idx_t* sample, cudaStream_t st);

// Overlap search (pq_search.cu)
struct SearchOut {
    uint16_t* num_B;            // [num_reads]
    uint16_t* num_F;
    int32_t* olp_B;
    int32_t* olp_F;
    uint8_t* status;            // OVF_* / ERR_* per read (0 = done)
    unsigned long long* edge_src;  // per read: offset into pool 1, or (1<<63 | offset) into pool 2
    // edge pool (struct of arrays)
    idx_t* e_dest;
    int32_t* e_trans;
    uint16_t* e_len;
    uint8_t* e_type;
    unsigned long long* e_count;   // atomic bump counter
    unsigned long long e_cap;
    idx_t* ovf_list;               // reads handed to the wide kernel
    unsigned int* ovf_count;
    unsigned long long* probes;    // total rank probes (one 32-byte sector each)
    unsigned long long* sectors;   // total 32-byte sectors of index data loaded (see Tally)
};

struct SearchArgs {
    FmView fm[2];               // 0 forward, 1 backward
    const uint8_t* reads;       // codes 1..4, forward orientation
    idx_t num_reads;
    int L;
    int t;
    DivL dl;                    // division by L
    int seed_k;                 // k-mer seed depth (0 = start at depth 1 from C[])
    int sa_seed;                // 1: candidates by depth-t interval scan (needs fm[].sa/pk/isa),
                                // 2: the same with learned windows (needs fm[].lx)
    unsigned long long* lx_misses;  // learned windows that missed (those chains walk)
    int sorted_reduce;          // 1: edges from sorted continuations (L - t <= 256)
    idx_t* defer;               // lean tier: reads handed to the fast tier ...
    unsigned* defer_count;      //   ... and their number (zero before the search)
};

// Global scratch of the fast kernel, per warp of 32 reads: level-0 candidates (4 kinds x (L - t)
// slots per read), ebcap edge slots per read, and per (read, side) task a DFS stack, sparse
// extension slots, emission bounds and DFS frames.
struct TFrame;
struct WarpScratch {
    idx_t *c_ll, *c_uu;
    uint32_t* c_meta;
    idx_t* e_dest;
    int32_t* e_trans;
    uint32_t* e_meta;
    idx_t *t_ll, *t_uu;
    uint32_t* t_meta;
    idx_t *x_ll, *x_uu;
    uint32_t* x_meta;
    idx_t *em_l, *em_u;
    TFrame* frames;
    uint64_t* r_k;              // sorted reduction: continuation words (word w of slot i at
    size_t r_plane;             //   r_k[w * r_plane + i]),
    idx_t* r_id;                //   read ids,
    uint32_t *r_meta, *r_emit;  //   (overlap, type) and emitted (index, trans)
    int ebcap;
    int mstride;                // candidate slots per kind and read (largest L - t searched)
};

// One read set of a queued search: its index pair, L and t, and its outputs.
struct SearchBatch {
    SearchArgs a;
    SearchOut o;
};
// Work items of a queued search: item i is group item_group[i] (reads 32 g .. 32 g + 31, and
// the following groups_per_item - 1 groups) of batch item_batch[i].  Warps take items in order
// from *next, which is zero at launch.
struct SearchQueue {
    const SearchBatch* batches;
    const uint32_t* item_batch;
    const uint32_t* item_group;
    unsigned count;             // 0: no queue
    unsigned groups_per_item;
    unsigned* next;
    // without a queue: search only the reads read_list[0, *list_count) (nullptr: every read)
    const idx_t* read_list;
    const unsigned* list_count;
};
size_t warp_scratch_bytes(int L, int t, size_t nwarps, int ebcap);
int search_fast_blocks(int L, int M, int num_sms);   // resident blocks of the fast kernel (M = L - t)
// blocks of 128 threads (4 warps); reads that outgrow the shared-memory stack, ebcap edges or
// the frame count are listed for the wide kernel.
cudaError_t search_fast(const SearchArgs& a, const SearchOut& o, int blocks, void* scratch, size_t scratch_bytes,
                        int ebcap, cudaStream_t st);
// Lean tier (thread per read, sorted reduction) over every read, then the fast tier over the reads
// it hands over (more than 64 candidates on a side); needs a.sorted_reduce.
int search_lean_blocks(int L, int M, int num_sms);
size_t lean_scratch_bytes(int L, int t, int lean_blocks, int fast_blocks, int ebcap);
cudaError_t search_lean(const SearchArgs& a, const SearchOut& o, int lean_blocks, int fast_blocks, void* scratch,
                        size_t scratch_bytes, int ebcap, cudaStream_t st);
// Block tier over reads[0, *count) (count_host of them): one CTA a read, all-pairs reduction of each
// side's candidates in shared memory; reads it cannot hold (or whose edges overflow the pool) are
// appended to next_list for the heavy tier.
cudaError_t search_block(const SearchArgs& a, const SearchOut& o, const idx_t* list, const unsigned* count,
                         unsigned count_host, idx_t* next_list, unsigned* next_count, cudaStream_t st);
bool block_tier_holds(int L, int t);      // false: reads of this L and t skip the block tier
// The block tier with each CTA's candidate arrays in its own region of a global scratch buffer
// (block_global_bytes for `blocks` CTAs): sides of up to 32768 candidates.
int block_global_blocks(unsigned count);
size_t block_global_bytes(int L, int t, int blocks);
cudaError_t search_block_global(const SearchArgs& a, const SearchOut& o, const idx_t* list, const unsigned* count,
                                unsigned count_host, int blocks, void* scratch, size_t scratch_bytes,
                                idx_t* next_list, unsigned* next_count, cudaStream_t st);
// Heavy tier over reads[0, *count) with a wider DFS (reads the fast tier could not hold).
size_t heavy_scratch_bytes(int L, int t, int blocks, int ebcap);
cudaError_t search_heavy(const SearchArgs& a, const SearchOut& o, const idx_t* list, const unsigned* count, int blocks,
                         void* scratch, size_t scratch_bytes, int ebcap, cudaStream_t st);
// One persistent lean launch over a queue of batches, then the fast tier over the handed-over
// reads of the batches listed in `batches` (host_batches: the descriptions the queue holds).
cudaError_t search_lean_queue(const SearchQueue& q, const SearchBatch* host_batches, const int* batches, int nbatch,
                              int L_max, int M_max, int lean_blocks, int fast_blocks, void* scratch,
                              size_t scratch_bytes, int ebcap, cudaStream_t st);
constexpr int lam_words_host(int M) { return M <= 64 ? 2 : 8; }
// One persistent launch over a queue of batches (L_max, M_max: the largest L and L - t).
size_t queue_scratch_bytes(int L_max, int M_max, size_t nwarps, int ebcap);
cudaError_t search_fast_queue(const SearchQueue& q, int L_max, int M_max, int blocks, void* scratch,
                              size_t scratch_bytes, int ebcap, cudaStream_t st);

struct WideScratch {
    void* stack;                // slots * stack_cap candidates
    void* frames;               // slots * frame_cap
    void* edges;                // slots * edge_cap
    size_t stack_cap, frame_cap, edge_cap;
    int slots;
};
size_t wide_slot_bytes(int L);
cudaError_t search_wide(const SearchArgs& a, const SearchOut& o, const idx_t* list, unsigned count,
                        const WideScratch& ws, cudaStream_t st);

// Final CSR assembly: out_off = exclusive scan of num_B+num_F (out_off[num_reads] = total),
// then the edges are gathered from the pool in read order.
cudaError_t assemble_counts_total(const SearchOut& o, idx_t num_reads, unsigned long long* out_off,
                                  void* scan_tmp, size_t scan_tmp_bytes, cudaStream_t st);
cudaError_t assemble_gather(const SearchOut& o, idx_t num_reads, const unsigned long long* off,
                            idx_t* dest, uint16_t* len, uint8_t* type, int32_t* trans, cudaStream_t st);
size_t assemble_tmp_bytes(idx_t num_reads);
extern const size_t kCandBytes;    // sizeof one stack entry of the search kernels
extern const size_t kFrameBytes;   // sizeof one DFS frame

}  // namespace pq
