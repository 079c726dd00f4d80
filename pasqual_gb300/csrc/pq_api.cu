// pq_api.cu — the C ABI (include/pasqual_gb300.h): a context owning the device buffers of both
// FM-indexes and the overlap-search output, and the entry points that sequence the kernels.
#include <cmath>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>
#include <chrono>
#include <algorithm>

#include "pq_index.cuh"
#include "pq_sort.cuh"
#include "pq_learned_build.cuh"
#include "../../include/pasqual_gb300.h"

static_assert(sizeof(pq_idx) == sizeof(idx_t), "pq_idx and idx_t must agree");

#include <atomic>
#include <mutex>
#include <thread>
#include <unordered_map>
namespace pq {
static std::atomic<unsigned long long> g_launches{0};
void note_launch() { g_launches.fetch_add(1, std::memory_order_relaxed); }
unsigned long long launch_count() { return g_launches.load(std::memory_order_relaxed); }
}  // namespace pq

namespace {

struct DevBuf {
    void* p = nullptr;
    size_t bytes = 0;
    cudaError_t ensure(size_t want) {
        if (want <= bytes && p) return cudaSuccess;
        if (p) cudaFree(p);
        p = nullptr;
        bytes = 0;
        cudaError_t e = cudaMalloc(&p, want ? want : 16);
        if (e == cudaSuccess) bytes = want;
        return e;
    }
    // grow keeping the first `keep` bytes
    cudaError_t grow(size_t want, size_t keep, cudaStream_t st) {
        if (want <= bytes && p) return cudaSuccess;
        void* q = nullptr;
        cudaError_t e = cudaMalloc(&q, want);
        if (e != cudaSuccess) return e;
        if (p && keep) cudaMemcpyAsync(q, p, std::min(keep, bytes), cudaMemcpyDeviceToDevice, st);
        cudaStreamSynchronize(st);
        if (p) cudaFree(p);
        p = q;
        bytes = want;
        return cudaSuccess;
    }
    void release() {
        if (p) cudaFree(p);
        p = nullptr;
        bytes = 0;
    }
    template <class T> T* as() const { return reinterpret_cast<T*>(p); }
};

}  // namespace

struct pq_ctx {
    int device = 0;
    cudaStream_t st = nullptr;
    bool own_stream = false;
    std::string err;
    cudaEvent_t ev0 = nullptr, ev1 = nullptr, evk0 = nullptr, evk1 = nullptr;
    float ms_sort = 0, ms_fm = 0, ms_search = 0, ms_fast = 0;

    idx_t num_reads = 0;
    int L = 0, t = 0;
    int seed_k = 0;
    int seed_k_user = 0;      // set by pq_set_seed_k: kept for every later read set
    int seed_mode = 1;        // 1: candidates by depth-t interval scan, 0: walk from the k-mer seed
    DevBuf reads;
    idx_t C[6] = {0}, sfx[4] = {0}, pfx[4] = {0};
    bool have_reads = false;

    // per direction
    DevBuf sa[2], blk[2], sb[2], ri[2], kstart[2], kend[2], pk[2], isa[2];
    bool sa_ok[2] = {false, false}, fm_ok[2] = {false, false};
    int fm_k[2] = {0, 0};
    DevBuf sort_tmp, counts;
    const uint32_t* sorted_keys[2] = {nullptr, nullptr};   // the last sort's keys, inside sort_tmp
    int kmer_from_sort[2] = {0, 0};                         // k of the k-mer table a chunked sort entered
    const uint8_t* bwt_hint[2] = {nullptr, nullptr};       // the last sort's BWT symbols, inside sort_tmp
    bool pk_ok[2] = {false, false};                        // pk[dir] holds this read set's packed text
    uint64_t sort_chunk = 0;                                // suffixes per sort chunk (0: automatic)

    // learned index per direction (pq_learned.cu)
    DevBuf lx_bnd[2], lx_base[2], lx_par[2], lx_err[2], lx_err_root[2], lx_segof[2], lx_tmp;
    int lx_segs[2] = {0, 0};
    bool lx_ok[2] = {false, false};
    pq_learned_info lx_info[2] = {};
    uint64_t lx_queries = 0, lx_misses = 0;

    // queued search over several contexts (this context leading): plan, queue buffers, graph
    int q_ctas_per_sm = 0;          // 0: as many as fit
    int q_groups_per_item = 1;
    int q_ebcap = 64;
    DevBuf q_batches, q_items, q_next;
    cudaGraph_t q_graph = nullptr;
    cudaGraphExec_t q_exec = nullptr;
    std::vector<uintptr_t> q_key;
    float q_kernel_ms = 0;
    int q_graph_used = 0;

    // overlap-search output
    DevBuf nB, nF, oB, oF, status, esrc, e_dest, e_trans, e_len, e_type, ctrs, ovf_list;
    DevBuf off, g_dest, g_len, g_type, g_trans, asm_tmp, wide, warp_scratch, defer, heavy_scratch, ovf2, ovf3, ovf4, block_scratch;
    uint64_t block_reads = 0;               // reads the block tier finished
    float ms_block = 0;
    uint64_t heavy_reads = 0, deferred_reads = 0;
    float ms_heavy = 0, ms_wide = 0;        // host time of the heavy and wide tiers
    bool graph_ok = false;
    uint64_t num_edges = 0, probes = 0, sectors = 0, wide_reads = 0;
};

static int fail(pq_ctx* c, int code, const std::string& msg) {
    if (c) c->err = msg;
    return code;
}

#define CK(call)                                                                                   \
    do {                                                                                           \
        cudaError_t e_ = (call);                                                                   \
        if (e_ != cudaSuccess)                                                                     \
            return fail(ctx, e_ == cudaErrorMemoryAllocation ? PQ_ERR_NOMEM : PQ_ERR_CUDA,        \
                        std::string(#call) + ": " + cudaGetErrorString(e_));                      \
    } while (0)

static inline size_t n_rows(const pq_ctx* c) { return size_t(c->num_reads) * size_t(c->L); }
static inline size_t n_blocks(const pq_ctx* c) { return n_rows(c) / 64 + 1; }
static inline size_t n_supers(const pq_ctx* c) {
    return (n_blocks(c) + kBlocksPerSuper - 1) / kBlocksPerSuper;
}

static constexpr int kLxDefaultSteps = 400;

static LearnedView lx_view(const pq_ctx* c, int d) {
    LearnedView v;
    v.bnd = c->lx_bnd[d].as<uint32_t>();
    v.base = c->lx_base[d].as<idx_t>();
    v.par = c->lx_par[d].as<float>();
    v.err = c->lx_err[d].as<int32_t>();
    v.segof = c->lx_segof[d].as<uint16_t>();
    v.segs = c->lx_ok[d] ? c->lx_segs[d] : 0;
    return v;
}

extern "C" {

int pq_idx_bytes(void) { return int(sizeof(idx_t)); }

namespace {
// Host buffers handed out by pq_host_alloc (pq_host_free accepts only these).
std::mutex g_host_mu;
std::unordered_map<void*, size_t> g_host;
}  // namespace

int pq_host_alloc(size_t bytes, void** out) {
    if (!out) return PQ_ERR_ARG;
    *out = nullptr;
    void* p = nullptr;
    const cudaError_t e = cudaHostAlloc(&p, std::max<size_t>(bytes, 1), cudaHostAllocDefault);
    if (e != cudaSuccess) {
        cudaGetLastError();
        return e == cudaErrorMemoryAllocation ? PQ_ERR_NOMEM : PQ_ERR_CUDA;
    }
    std::lock_guard<std::mutex> g(g_host_mu);
    g_host[p] = bytes;
    *out = p;
    return PQ_OK;
}

int pq_host_free(void* p) {
    if (!p) return PQ_OK;
    {
        std::lock_guard<std::mutex> g(g_host_mu);
        auto it = g_host.find(p);
        if (it == g_host.end()) return PQ_ERR_ARG;
        g_host.erase(it);
    }
    return cudaFreeHost(p) == cudaSuccess ? PQ_OK : PQ_ERR_CUDA;
}

// The device-accessible address of page-locked host memory (cudaHostAlloc'd or registered), or
// null for pageable memory.
static void* locked_device_ptr(const void* host) {
    cudaPointerAttributes pa{};
    const bool ok = cudaPointerGetAttributes(&pa, host) == cudaSuccess && pa.type == cudaMemoryTypeHost;
    cudaGetLastError();
    return ok ? pa.devicePointer : nullptr;
}

int pq_create(pq_ctx** out, int device, void* cuda_stream) {
    if (!out) return PQ_ERR_ARG;
    *out = nullptr;
    pq_ctx* ctx = new (std::nothrow) pq_ctx();
    if (!ctx) return PQ_ERR_NOMEM;
    ctx->device = device;
    cudaError_t e = cudaSetDevice(device);
    if (e != cudaSuccess) {
        delete ctx;
        return PQ_ERR_CUDA;
    }
    if (cuda_stream) {
        ctx->st = reinterpret_cast<cudaStream_t>(cuda_stream);
    } else {
        if (cudaStreamCreateWithFlags(&ctx->st, cudaStreamNonBlocking) != cudaSuccess) {
            delete ctx;
            return PQ_ERR_CUDA;
        }
        ctx->own_stream = true;
    }
    cudaEventCreate(&ctx->ev0);
    cudaEventCreate(&ctx->ev1);
    cudaEventCreate(&ctx->evk0);
    cudaEventCreate(&ctx->evk1);
    *out = ctx;
    return PQ_OK;
}

void pq_destroy(pq_ctx* ctx) {
    if (!ctx) return;
    cudaSetDevice(ctx->device);
    cudaStreamSynchronize(ctx->st);
    DevBuf* bufs[] = {&ctx->reads, &ctx->sort_tmp, &ctx->counts, &ctx->nB, &ctx->nF, &ctx->oB,
                      &ctx->oF, &ctx->status, &ctx->esrc, &ctx->e_dest, &ctx->e_trans, &ctx->e_len,
                      &ctx->e_type, &ctx->ctrs, &ctx->ovf_list, &ctx->off, &ctx->g_dest, &ctx->g_len,
                      &ctx->g_type, &ctx->g_trans, &ctx->asm_tmp, &ctx->wide, &ctx->warp_scratch, &ctx->defer,
                      &ctx->heavy_scratch, &ctx->ovf2, &ctx->ovf3, &ctx->ovf4, &ctx->block_scratch};
    for (DevBuf* b : bufs) b->release();
    for (int d = 0; d < 2; ++d) {
        ctx->sa[d].release();
        ctx->blk[d].release();
        ctx->sb[d].release();
        ctx->ri[d].release();
        ctx->kstart[d].release();
        ctx->kend[d].release();
        ctx->pk[d].release();
        ctx->isa[d].release();
        ctx->lx_bnd[d].release();
        ctx->lx_base[d].release();
        ctx->lx_par[d].release();
        ctx->lx_err[d].release();
        ctx->lx_err_root[d].release();
        ctx->lx_segof[d].release();
    }
    if (ctx->ev0) cudaEventDestroy(ctx->ev0);
    if (ctx->ev1) cudaEventDestroy(ctx->ev1);
    if (ctx->evk0) cudaEventDestroy(ctx->evk0);
    if (ctx->evk1) cudaEventDestroy(ctx->evk1);
    if (ctx->own_stream) cudaStreamDestroy(ctx->st);
    if (ctx->q_exec) cudaGraphExecDestroy(ctx->q_exec);
    if (ctx->q_graph) cudaGraphDestroy(ctx->q_graph);
    ctx->q_batches.release();
    ctx->q_items.release();
    ctx->q_next.release();
    delete ctx;
}

const char* pq_last_error(const pq_ctx* ctx) { return ctx ? ctx->err.c_str() : "no context"; }

int pq_set_reads(pq_ctx* ctx, const uint8_t* reads, pq_idx num_reads, int read_len, int min_overlap,
                 int from_device) {
    if (!ctx) return PQ_ERR_ARG;
    if (read_len <= 0 || read_len > 65535)
        return fail(ctx, PQ_ERR_ARG, "invalid read length, valid range (0, 65535]");
    if (min_overlap <= 9 || min_overlap >= read_len)
        return fail(ctx, PQ_ERR_ARG, "invalid minimum overlap length, valid range (9, read_len)");
    const unsigned __int128 n = (unsigned __int128)num_reads * (unsigned)read_len;
    if (n >> (8 * sizeof(idx_t) - 1))
        return fail(ctx, PQ_ERR_ARG, "num_reads * read_len does not fit the index width");
    if (num_reads && !reads) return fail(ctx, PQ_ERR_ARG, "reads is NULL");
    cudaSetDevice(ctx->device);
    ctx->num_reads = num_reads;
    ctx->L = read_len;
    ctx->t = min_overlap;
    // default seed depth by index size: a k-mer's rows number about n / 4^k, and each halving of
    // them saves a bisection step of every interval scan (the 250 Mbp workload's search: 189 ms at
    // k = 12, 166 at 13, 148 at 14), for 4^k table entries (2 per index, IDX bytes each)
    if (!ctx->seed_k_user) {
        const unsigned long long n_sfx = (unsigned long long)num_reads * (unsigned)read_len;
        ctx->seed_k = n_sfx >= (1ull << 32) ? 14 : (n_sfx >= (1ull << 30) ? 13 : 12);
    }
    ctx->seed_k = std::min(ctx->seed_k, min_overlap);
    size_t bytes = size_t(num_reads) * read_len;
    CK(ctx->reads.ensure(bytes + 64));
    if (bytes) {
        // page-locked host memory (cudaHostAlloc'd or registered) is read by the copy kernel;
        // pageable memory goes through cudaMemcpy
        const void* locked = from_device ? nullptr : locked_device_ptr(reads);
        if (locked)
            CK(pq::kernel_copy(ctx->reads.p, locked, bytes, ctx->st));
        else
            CK(cudaMemcpyAsync(ctx->reads.p, reads, bytes,
                               from_device ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice, ctx->st));
    }
    CK(ctx->counts.ensure(13 * sizeof(unsigned long long)));
    CK(pq::read_counts(ctx->reads.as<uint8_t>(), num_reads, idx_t(read_len),
                       ctx->counts.as<unsigned long long>(), ctx->st));
    unsigned long long h[13];
    CK(cudaMemcpyAsync(h, ctx->counts.p, sizeof h, cudaMemcpyDeviceToHost, ctx->st));
    CK(cudaStreamSynchronize(ctx->st));
    if (h[12]) {   // the reference's import drops reads with N and rejects any other symbol
        ctx->have_reads = false;
        ctx->num_reads = 0;
        ctx->pk_ok[0] = ctx->pk_ok[1] = false;
        ctx->sa_ok[0] = ctx->sa_ok[1] = false;
        ctx->fm_ok[0] = ctx->fm_ok[1] = false;
        ctx->graph_ok = false;
        return fail(ctx, PQ_ERR_ARG, "reads must hold base codes 1..4 (A, C, G, T) only");
    }
    ctx->C[0] = 0;
    ctx->C[1] = 0;
    ctx->C[2] = idx_t(h[0]);
    ctx->C[3] = idx_t(h[0] + h[1]);
    ctx->C[4] = idx_t(h[0] + h[1] + h[2]);
    ctx->C[5] = idx_t(h[0] + h[1] + h[2] + h[3]);
    for (int c = 0; c < 4; ++c) {
        ctx->sfx[c] = idx_t(h[4 + c]);
        ctx->pfx[c] = idx_t(h[8 + c]);
    }
    ctx->have_reads = true;
    ctx->pk_ok[0] = ctx->pk_ok[1] = false;
    ctx->sa_ok[0] = ctx->sa_ok[1] = false;
    ctx->fm_ok[0] = ctx->fm_ok[1] = false;
    ctx->graph_ok = false;
    return PQ_OK;
}

int pq_get_counts(pq_ctx* ctx, pq_idx C[6], pq_idx suffix_count[4], pq_idx prefix_count[4]) {
    if (!ctx) return PQ_ERR_ARG;
    if (!ctx->have_reads) return fail(ctx, PQ_ERR_STATE, "pq_set_reads first");
    if (C) memcpy(C, ctx->C, sizeof ctx->C);
    if (suffix_count) memcpy(suffix_count, ctx->sfx, sizeof ctx->sfx);
    if (prefix_count) memcpy(prefix_count, ctx->pfx, sizeof ctx->pfx);
    return PQ_OK;
}

// side_outputs: also the BWT symbols of the rows the group refinement places (FM-index work done
// where the refinement leaves DRAM idle; pq_build_index asks for them), and for a chunked sort the
// k-mer table from its chunks' keys.  pq_sort itself computes the suffix array only.
static int sort_dir(pq_ctx* ctx, int dir, bool side_outputs) {
    if (!ctx || (dir != 0 && dir != 1)) return PQ_ERR_ARG;
    if (!ctx->have_reads) return fail(ctx, PQ_ERR_STATE, "pq_set_reads first");
    cudaSetDevice(ctx->device);
    const size_t n = n_rows(ctx);
    CK(ctx->sa[dir].ensure(n * sizeof(idx_t) + 64));
    CK(ctx->pk[dir].ensure((n / 32 + 4) * sizeof(uint64_t)));
    // one pass below 2^31 suffixes (32-bit group ranks), else chunks of 6-base buckets
    const size_t one_pass_max = (size_t(1) << 31) - 1;
    const bool chunked = n > one_pass_max || (ctx->sort_chunk && n > ctx->sort_chunk);
    const size_t cap = std::min(ctx->sort_chunk ? size_t(ctx->sort_chunk) : (size_t(1) << 30), one_pass_max);
    size_t tmp_bytes = chunked ? pq::suffix_sort_chunked_tmp_bytes(n, cap) : pq::suffix_sort_tmp_bytes(n);
    CK(ctx->sort_tmp.ensure(tmp_bytes));
    CK(cudaEventRecord(ctx->ev0, ctx->st));
    ctx->sorted_keys[0] = ctx->sorted_keys[1] = nullptr;     // the scratch is about to be reused
    ctx->bwt_hint[0] = ctx->bwt_hint[1] = nullptr;
    const uint8_t** hint_out = side_outputs ? &ctx->bwt_hint[dir] : nullptr;
    idx_t* isa_out = nullptr;       // the search needs no inverse suffix array
    // a chunked index-build sort also enters the k-mer table from its chunks' keys (k >= 6: a
    // k-mer's rows then lie in one 6-base bucket, so in one chunk)
    ctx->kmer_from_sort[dir] = 0;
    const int kk = ctx->seed_k;
    const bool kmer_in_sort = side_outputs && chunked && kk >= 6 && kk <= pq::kSortKeyBases;
    if (kmer_in_sort) {
        const size_t nk = size_t(1) << (2 * kk);
        CK(ctx->kstart[dir].ensure(nk * sizeof(idx_t)));
        CK(ctx->kend[dir].ensure(nk * sizeof(idx_t)));
        CK(pq::kmer_table_clear(kk, ctx->kstart[dir].as<idx_t>(), ctx->kend[dir].as<idx_t>(), ctx->st));
    }
    int rc = chunked ? pq::suffix_sort_chunked(ctx->reads.as<uint8_t>(), ctx->num_reads, ctx->L, dir,
                                               ctx->sa[dir].as<idx_t>(), cap, ctx->sort_tmp.p, tmp_bytes, ctx->st,
                                               hint_out, ctx->pk[dir].as<uint64_t>(), isa_out,
                                               idx_t(ctx->L - ctx->t),
                                               kmer_in_sort ? ctx->kstart[dir].as<idx_t>() : nullptr,
                                               kmer_in_sort ? ctx->kend[dir].as<idx_t>() : nullptr, kk)
                     : pq::suffix_sort(ctx->reads.as<uint8_t>(), ctx->num_reads, ctx->L, dir,
                                       ctx->sa[dir].as<idx_t>(), ctx->sort_tmp.p, tmp_bytes, ctx->st,
                                       &ctx->sorted_keys[dir], hint_out, ctx->pk[dir].as<uint64_t>(), isa_out,
                                       idx_t(ctx->L - ctx->t));
    ctx->pk_ok[dir] = rc == 0;
    if (rc == int(cudaErrorNotSupported))
        return fail(ctx, PQ_ERR_CAPACITY, "suffix sort: a 6-base bucket holds more suffixes than a sort chunk");
    if (rc != 0) return fail(ctx, PQ_ERR_CUDA, std::string("suffix sort failed: ") + cudaGetErrorString(cudaGetLastError()));
    CK(cudaEventRecord(ctx->ev1, ctx->st));
    CK(cudaEventSynchronize(ctx->ev1));
    cudaEventElapsedTime(&ctx->ms_sort, ctx->ev0, ctx->ev1);
    if (kmer_in_sort) ctx->kmer_from_sort[dir] = kk;
    ctx->sa_ok[dir] = true;
    ctx->fm_ok[dir] = false;
    ctx->graph_ok = false;
    return PQ_OK;
}

int pq_sort(pq_ctx* ctx, int dir) { return sort_dir(ctx, dir, false); }

// The sort of an index build (with the FM side outputs), for the reference's own entry points
// (pq_dropin.cu), which build one direction at a time; not part of the C ABI.
int pq_sort_for_index(pq_ctx* ctx, int dir) { return sort_dir(ctx, dir, true); }

int pq_set_sa(pq_ctx* ctx, int dir, const pq_idx* sa, int from_device) {
    if (!ctx || (dir != 0 && dir != 1)) return PQ_ERR_ARG;
    if (!ctx->have_reads) return fail(ctx, PQ_ERR_STATE, "pq_set_reads first");
    cudaSetDevice(ctx->device);
    const size_t n = n_rows(ctx);
    CK(ctx->sa[dir].ensure(n * sizeof(idx_t) + 64));
    if (n)
        CK(cudaMemcpyAsync(ctx->sa[dir].p, sa, n * sizeof(idx_t),
                           from_device ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice, ctx->st));
    CK(cudaStreamSynchronize(ctx->st));
    ctx->sorted_keys[dir] = nullptr;
    ctx->bwt_hint[dir] = nullptr;
    ctx->kmer_from_sort[dir] = 0;
    ctx->sa_ok[dir] = true;
    ctx->fm_ok[dir] = false;
    ctx->graph_ok = false;
    return PQ_OK;
}

int pq_get_sa(pq_ctx* ctx, int dir, pq_idx* sa_host) {
    if (!ctx || (dir != 0 && dir != 1) || !sa_host) return PQ_ERR_ARG;
    if (!ctx->sa_ok[dir]) return fail(ctx, PQ_ERR_STATE, "no suffix array for this direction");
    const size_t n = n_rows(ctx);
    if (n) CK(cudaMemcpyAsync(sa_host, ctx->sa[dir].p, n * sizeof(idx_t), cudaMemcpyDeviceToHost, ctx->st));
    CK(cudaStreamSynchronize(ctx->st));
    return PQ_OK;
}

// Rows [first, first + count) of direction dir's suffix array into host memory (the slot a
// drop-in suf_sort call returns).  Not part of the public header.
int pq_get_sa_rows(pq_ctx* ctx, int dir, uint64_t first, uint64_t count, pq_idx* host) {
    if (!ctx || (dir != 0 && dir != 1) || (count && !host)) return PQ_ERR_ARG;
    if (!ctx->sa_ok[dir]) return fail(ctx, PQ_ERR_STATE, "no suffix array for this direction");
    if (first > n_rows(ctx) || count > n_rows(ctx) - first) return fail(ctx, PQ_ERR_ARG, "rows out of range");
    if (count)
        CK(cudaMemcpyAsync(host, ctx->sa[dir].as<idx_t>() + first, count * sizeof(idx_t), cudaMemcpyDeviceToHost,
                           ctx->st));
    CK(cudaStreamSynchronize(ctx->st));
    return PQ_OK;
}

// The seed records of the sort buckets in rows [r0, r1) of direction dir applied to the host arrays
// start/size/depth (one entry per read): a record replaces a read's seed when it is deeper, as in
// src/sufsort.c:182-189.  Not part of the public header.
int pq_apply_sort_seeds(pq_ctx* ctx, int dir, uint64_t r0, uint64_t r1, pq_idx* start, pq_idx* size,
                        uint16_t* depth) {
    if (!ctx || (dir != 0 && dir != 1) || !start || !size || !depth) return PQ_ERR_ARG;
    if (!ctx->sa_ok[dir]) return fail(ctx, PQ_ERR_STATE, "no suffix array for this direction");
    const size_t nr = ctx->num_reads, n = n_rows(ctx);
    if (r0 > r1 || r1 > n) return fail(ctx, PQ_ERR_ARG, "rows out of range");
    if (!nr || r0 == r1) return PQ_OK;
    cudaSetDevice(ctx->device);
    if (!ctx->pk_ok[dir]) {
        CK(ctx->pk[dir].ensure((n / 32 + 4) * sizeof(uint64_t)));
        CK(pq::pack_text(ctx->reads.as<uint8_t>(), n, idx_t(ctx->L), dir, ctx->pk[dir].as<uint64_t>(), ctx->st));
        ctx->pk_ok[dir] = true;
    }
    DevBuf s, z, d, tmp;
    CK(s.ensure(nr * sizeof(idx_t)));
    CK(z.ensure(nr * sizeof(idx_t)));
    CK(d.ensure(nr * sizeof(uint16_t)));
    const size_t tb = pq::sort_seeds_tmp_bytes(size_t(r1 - r0));
    CK(tmp.ensure(tb));
    CK(cudaMemcpyAsync(s.p, start, nr * sizeof(idx_t), cudaMemcpyHostToDevice, ctx->st));
    CK(cudaMemcpyAsync(z.p, size, nr * sizeof(idx_t), cudaMemcpyHostToDevice, ctx->st));
    CK(cudaMemcpyAsync(d.p, depth, nr * sizeof(uint16_t), cudaMemcpyHostToDevice, ctx->st));
    CK(pq::sort_seeds(ctx->sa[dir].as<idx_t>(), ctx->pk[dir].as<uint64_t>(), idx_t(ctx->L), ctx->t, size_t(r0),
                      size_t(r1), d.as<uint16_t>(), s.as<idx_t>(), z.as<idx_t>(), tmp.p, tb, ctx->st));
    CK(cudaMemcpyAsync(start, s.p, nr * sizeof(idx_t), cudaMemcpyDeviceToHost, ctx->st));
    CK(cudaMemcpyAsync(size, z.p, nr * sizeof(idx_t), cudaMemcpyDeviceToHost, ctx->st));
    CK(cudaMemcpyAsync(depth, d.p, nr * sizeof(uint16_t), cudaMemcpyDeviceToHost, ctx->st));
    CK(cudaStreamSynchronize(ctx->st));
    return PQ_OK;
}

int pq_set_seed_k(pq_ctx* ctx, int k) {
    if (!ctx) return PQ_ERR_ARG;
    if (k < 1 || k > pq::kSortKeyBases) return fail(ctx, PQ_ERR_ARG, "seed depth must be in [1, 14]");
    if (ctx->have_reads && k > ctx->t) return fail(ctx, PQ_ERR_ARG, "seed depth must not exceed t");
    ctx->seed_k = k;
    ctx->seed_k_user = 1;
    return PQ_OK;
}

int pq_set_sort_chunk(pq_ctx* ctx, uint64_t max_suffixes) {
    if (!ctx) return PQ_ERR_ARG;
    if (max_suffixes == 1 || max_suffixes >= (uint64_t(1) << 31))
        return fail(ctx, PQ_ERR_ARG, "sort chunk must be 0 (automatic) or 2 .. 2^31 - 1 suffixes");
    ctx->sort_chunk = max_suffixes;
    return PQ_OK;
}

int pq_set_seed_mode(pq_ctx* ctx, int mode) {
    if (!ctx) return PQ_ERR_ARG;
    if (mode < 0 || mode > 2)
        return fail(ctx, PQ_ERR_ARG, "seed mode must be 0 (walk), 1 (interval scan) or 2 (learned windows)");
    ctx->seed_mode = mode;
    ctx->graph_ok = false;
    return PQ_OK;
}

int pq_build_fm(pq_ctx* ctx, int dir) {
    if (!ctx || (dir != 0 && dir != 1)) return PQ_ERR_ARG;
    if (!ctx->sa_ok[dir]) return fail(ctx, PQ_ERR_STATE, "no suffix array for this direction");
    cudaSetDevice(ctx->device);
    const size_t n = n_rows(ctx);
    CK(ctx->blk[dir].ensure(n_blocks(ctx) * sizeof(OccBlock)));
    CK(ctx->sb[dir].ensure(n_supers(ctx) * 4 * sizeof(idx_t) + 64));
    CK(ctx->ri[dir].ensure(size_t(ctx->num_reads) * sizeof(idx_t) + 64));
    const int k = ctx->seed_k;
    const size_t nk = size_t(1) << (2 * k);
    CK(ctx->kstart[dir].ensure(nk * sizeof(idx_t)));
    CK(ctx->kend[dir].ensure(nk * sizeof(idx_t)));
    CK(ctx->pk[dir].ensure((n / 32 + 4) * sizeof(uint64_t)));
    ctx->isa[dir].release();
    CK(cudaEventRecord(ctx->ev0, ctx->st));
    if (!ctx->pk_ok[dir])
        CK(pq::pack_text(ctx->reads.as<uint8_t>(), n, idx_t(ctx->L), dir, ctx->pk[dir].as<uint64_t>(), ctx->st));
    ctx->pk_ok[dir] = true;
    CK(pq::build_occ(ctx->sa[dir].as<idx_t>(), ctx->reads.as<uint8_t>(), ctx->num_reads, idx_t(ctx->L), dir,
                     ctx->blk[dir].as<OccBlock>(), ctx->sb[dir].as<idx_t>(), ctx->ri[dir].as<idx_t>(), ctx->st,
                     ctx->pk[dir].as<uint64_t>(), ctx->bwt_hint[dir]));
    if (ctx->kmer_from_sort[dir] != k)
        CK(pq::build_kmer_table(ctx->sa[dir].as<idx_t>(), ctx->num_reads, idx_t(ctx->L), k,
                                ctx->kstart[dir].as<idx_t>(), ctx->kend[dir].as<idx_t>(), ctx->st,
                                ctx->sorted_keys[dir], ctx->pk[dir].as<uint64_t>()));
    ctx->kmer_from_sort[dir] = 0;
    CK(cudaEventRecord(ctx->ev1, ctx->st));
    CK(cudaEventSynchronize(ctx->ev1));
    cudaEventElapsedTime(&ctx->ms_fm, ctx->ev0, ctx->ev1);
    ctx->fm_ok[dir] = true;
    ctx->fm_k[dir] = k;
    ctx->lx_ok[dir] = false;
    ctx->graph_ok = false;
    return PQ_OK;
}

int pq_build_index(pq_ctx* ctx) {
    if (!ctx) return PQ_ERR_ARG;
    float s = 0, f = 0;
    for (int d = 0; d < 2; ++d) {
        int rc = sort_dir(ctx, d, true);
        if (rc) return rc;
        s += ctx->ms_sort;
        rc = pq_build_fm(ctx, d);
        if (rc) return rc;
        f += ctx->ms_fm;
    }
    ctx->ms_sort = s;
    ctx->ms_fm = f;
    // the sort's working memory is not needed by the search: give it back when device
    // memory is short (under a quarter free), else keep it for the next build of the same size
    // (a cudaMalloc and cudaFree of tens of GB per build)
    ctx->sorted_keys[0] = ctx->sorted_keys[1] = nullptr;
    ctx->bwt_hint[0] = ctx->bwt_hint[1] = nullptr;
    size_t free_b = 0, total_b = 0;
    if (cudaMemGetInfo(&free_b, &total_b) != cudaSuccess || free_b < total_b / 4) {
        ctx->sort_tmp.release();
    }
    return PQ_OK;
}

int pq_get_index_ref(pq_ctx* ctx, int dir, uint64_t* bitmap, pq_idx* sample, pq_idx* reads_index) {
    if (!ctx || (dir != 0 && dir != 1)) return PQ_ERR_ARG;
    if (!ctx->fm_ok[dir]) return fail(ctx, PQ_ERR_STATE, "no FM-index for this direction");
    cudaSetDevice(ctx->device);
    const size_t nblk = n_blocks(ctx);
    if (bitmap || sample) {
        DevBuf bm, smp;
        CK(bm.ensure(nblk * 5 * sizeof(uint64_t)));
        CK(smp.ensure(nblk * 5 * sizeof(idx_t)));
        const idx_t* fix = dir == 0 ? ctx->sfx : ctx->pfx;
        CK(pq::export_ref_layout(ctx->blk[dir].as<OccBlock>(), ctx->sb[dir].as<idx_t>(), ctx->num_reads,
                                 idx_t(ctx->L), fix, bm.as<uint64_t>(), smp.as<idx_t>(), ctx->st));
        if (bitmap) CK(cudaMemcpyAsync(bitmap, bm.p, nblk * 5 * sizeof(uint64_t), cudaMemcpyDeviceToHost, ctx->st));
        if (sample) CK(cudaMemcpyAsync(sample, smp.p, nblk * 5 * sizeof(idx_t), cudaMemcpyDeviceToHost, ctx->st));
        CK(cudaStreamSynchronize(ctx->st));
        bm.release();
        smp.release();
    }
    if (reads_index && ctx->num_reads)
        CK(cudaMemcpyAsync(reads_index, ctx->ri[dir].p, size_t(ctx->num_reads) * sizeof(idx_t),
                           cudaMemcpyDeviceToHost, ctx->st));
    CK(cudaStreamSynchronize(ctx->st));
    return PQ_OK;
}

int pq_get_seeds(pq_ctx* ctx, int dir, pq_idx* start, pq_idx* size, uint16_t* depth) {
    if (!ctx || (dir != 0 && dir != 1)) return PQ_ERR_ARG;
    if (!ctx->fm_ok[dir]) return fail(ctx, PQ_ERR_STATE, "no FM-index for this direction");
    cudaSetDevice(ctx->device);
    const size_t nr = ctx->num_reads;
    if (!nr) return PQ_OK;
    DevBuf s, z;
    CK(s.ensure(nr * sizeof(idx_t)));
    CK(z.ensure(nr * sizeof(idx_t)));
    CK(pq::read_seeds(ctx->reads.as<uint8_t>(), ctx->num_reads, ctx->L, dir, ctx->fm_k[dir],
                      ctx->kstart[dir].as<idx_t>(), ctx->kend[dir].as<idx_t>(), s.as<idx_t>(), z.as<idx_t>(), ctx->st));
    if (start) CK(cudaMemcpyAsync(start, s.p, nr * sizeof(idx_t), cudaMemcpyDeviceToHost, ctx->st));
    if (size) CK(cudaMemcpyAsync(size, z.p, nr * sizeof(idx_t), cudaMemcpyDeviceToHost, ctx->st));
    CK(cudaStreamSynchronize(ctx->st));
    if (depth)
        for (size_t i = 0; i < nr; ++i) depth[i] = uint16_t(ctx->fm_k[dir]);
    return PQ_OK;
}

int pq_get_sort_seeds(pq_ctx* ctx, int dir, pq_idx* start, pq_idx* size, uint16_t* depth) {
    if (!ctx || (dir != 0 && dir != 1)) return PQ_ERR_ARG;
    if (!ctx->sa_ok[dir]) return fail(ctx, PQ_ERR_STATE, "no suffix array for this direction");
    cudaSetDevice(ctx->device);
    const size_t nr = ctx->num_reads, n = n_rows(ctx);
    if (!nr) return PQ_OK;
    if (!ctx->pk_ok[dir]) {
        CK(ctx->pk[dir].ensure((n / 32 + 4) * sizeof(uint64_t)));
        CK(pq::pack_text(ctx->reads.as<uint8_t>(), n, idx_t(ctx->L), dir, ctx->pk[dir].as<uint64_t>(), ctx->st));
        ctx->pk_ok[dir] = true;
    }
    DevBuf s, z, d, tmp;
    CK(s.ensure(nr * sizeof(idx_t)));
    CK(z.ensure(nr * sizeof(idx_t)));
    CK(d.ensure(nr * sizeof(uint16_t)));
    const size_t tb = pq::sort_seeds_tmp_bytes(n);
    CK(tmp.ensure(tb));
    CK(pq::seed_init(ctx->reads.as<uint8_t>(), ctx->num_reads, idx_t(ctx->L), dir, ctx->C, d.as<uint16_t>(),
                     s.as<idx_t>(), z.as<idx_t>(), ctx->st));
    CK(pq::sort_seeds(ctx->sa[dir].as<idx_t>(), ctx->pk[dir].as<uint64_t>(), idx_t(ctx->L), ctx->t, 0, n,
                      d.as<uint16_t>(), s.as<idx_t>(), z.as<idx_t>(), tmp.p, tb, ctx->st));
    if (start) CK(cudaMemcpyAsync(start, s.p, nr * sizeof(idx_t), cudaMemcpyDeviceToHost, ctx->st));
    if (size) CK(cudaMemcpyAsync(size, z.p, nr * sizeof(idx_t), cudaMemcpyDeviceToHost, ctx->st));
    if (depth) CK(cudaMemcpyAsync(depth, d.p, nr * sizeof(uint16_t), cudaMemcpyDeviceToHost, ctx->st));
    CK(cudaStreamSynchronize(ctx->st));
    return PQ_OK;
}

// Output buffers, search arguments and zeroed counters of one context's overlap search.
static int search_prepare(pq_ctx* ctx, pq::SearchArgs& A, pq::SearchOut& O) {
    if (!ctx->fm_ok[0] || !ctx->fm_ok[1]) return fail(ctx, PQ_ERR_STATE, "build both FM-indexes first");
    if (ctx->fm_k[0] != ctx->fm_k[1]) return fail(ctx, PQ_ERR_STATE, "seed tables of different depth");
    cudaSetDevice(ctx->device);
    const size_t nr = ctx->num_reads;
    const size_t nrp = nr + 1;
    CK(ctx->nB.ensure(nrp * 2));
    CK(ctx->nF.ensure(nrp * 2));
    CK(ctx->oB.ensure(nrp * 4));
    CK(ctx->oF.ensure(nrp * 4));
    CK(ctx->status.ensure(nrp));
    CK(ctx->esrc.ensure(nrp * 8));
    CK(ctx->ovf_list.ensure(nrp * sizeof(idx_t)));
    CK(ctx->ctrs.ensure(128));
    size_t ecap = std::max<size_t>(ctx->e_dest.bytes / sizeof(idx_t), nr * 6 + 4096);
    CK(ctx->e_dest.ensure(ecap * sizeof(idx_t)));
    CK(ctx->e_trans.ensure(ecap * 4));
    CK(ctx->e_len.ensure(ecap * 2));
    CK(ctx->e_type.ensure(ecap));

    for (int d = 0; d < 2; ++d) {
        FmView& f = A.fm[d];
        f.blk = ctx->blk[d].as<OccBlock>();
        f.sb = ctx->sb[d].as<idx_t>();
        f.reads_index = ctx->ri[d].as<idx_t>();
        f.kstart = ctx->kstart[d].as<idx_t>();
        f.kend = ctx->kend[d].as<idx_t>();
        f.sa = ctx->sa[d].as<idx_t>();
        f.pk = ctx->pk[d].as<uint64_t>();
        f.isa = nullptr;          // no inverse suffix array: reads the lean tier hands over walk
        const idx_t* fix = d == 0 ? ctx->sfx : ctx->pfx;
        f.Cf[0] = ctx->C[0];
        for (int c = 1; c <= 4; ++c) f.Cf[c] = ctx->C[c] + fix[c - 1];
    }
    A.reads = ctx->reads.as<uint8_t>();
    A.num_reads = ctx->num_reads;
    A.L = ctx->L;
    A.dl = make_divl(uint32_t(ctx->L));
    A.t = ctx->t;
    A.seed_k = ctx->fm_k[0];
    // Interval scan where depth-t intervals are small (4^min(t, 64) well above 64 n: chance hits
    // rare) and L - t <= 256; otherwise the walk.  Learned windows need 16-base keys.
    {
        const double n = double(n_rows(ctx)) + 1.0;
        const bool small_intervals = 2.0 * std::min(ctx->t, 64) > std::log2(n) + 6.0;
        const bool scan = small_intervals && ctx->L - ctx->t <= 256 && ctx->t > A.seed_k;
        A.sa_seed = 0;
        if (scan && ctx->seed_mode == 1) A.sa_seed = 1;
        if (scan && ctx->seed_mode == 2 && ctx->t >= pq::kLxKeyBases && nr) {
            for (int d = 0; d < 2; ++d) {
                if (!ctx->lx_ok[d]) {
                    const int rc = pq_learned_build(ctx, d, kLxDefaultSteps);
                    if (rc != PQ_OK) return rc;
                }
            }
            if (ctx->lx_segs[0] && ctx->lx_segs[1]) A.sa_seed = 2;
        }
        for (int d = 0; d < 2; ++d) A.fm[d].lx = lx_view(ctx, d);
    }
    ctx->lx_queries = A.sa_seed == 2 ? 4 * uint64_t(nr) : 0;
    // seed mode 0 is the reference's method throughout (walk + FM-index DFS); 1 and 2 reduce by
    // sorted continuations wherever those fit in 256 bases
    A.sorted_reduce = (ctx->seed_mode != 0 && ctx->L - ctx->t <= 256) ? 1 : 0;

    // [0] e_count [1] probes [2] ovf (u32) [3] learned misses [4] defer (u32) [5] heavy ovf [6] sectors
    unsigned long long* ctr = ctx->ctrs.as<unsigned long long>();
    O.num_B = ctx->nB.as<uint16_t>();
    O.num_F = ctx->nF.as<uint16_t>();
    O.olp_B = ctx->oB.as<int32_t>();
    O.olp_F = ctx->oF.as<int32_t>();
    O.status = ctx->status.as<uint8_t>();
    O.edge_src = ctx->esrc.as<unsigned long long>();
    O.e_dest = ctx->e_dest.as<idx_t>();
    O.e_trans = ctx->e_trans.as<int32_t>();
    O.e_len = ctx->e_len.as<uint16_t>();
    O.e_type = ctx->e_type.as<uint8_t>();
    O.e_count = ctr + 0;
    O.e_cap = ecap;
    O.ovf_list = ctx->ovf_list.as<idx_t>();
    O.ovf_count = reinterpret_cast<unsigned int*>(ctr + 2);
    O.probes = ctr + 1;
    O.sectors = ctr + 6;
    A.lx_misses = ctr + 3;
    CK(ctx->defer.ensure((nr + 1) * sizeof(idx_t)));
    A.defer = ctx->defer.as<idx_t>();
    A.defer_count = reinterpret_cast<unsigned*>(ctr + 4);

    CK(cudaMemsetAsync(ctr, 0, 64, ctx->st));
    return PQ_OK;
}

// After the fast kernel: the wide tier for the reads it handed over, then the CSR in read order.
static int search_finish(pq_ctx* ctx, pq::SearchArgs& A, pq::SearchOut& O) {
    const size_t nr = ctx->num_reads;
    const size_t nrp = nr + 1;
    unsigned long long* ctr = ctx->ctrs.as<unsigned long long>();
    unsigned long long hc[5];
    CK(cudaMemcpyAsync(hc, ctr, sizeof hc, cudaMemcpyDeviceToHost, ctx->st));
    CK(cudaStreamSynchronize(ctx->st));
    ctx->lx_misses = hc[3];
    ctx->deferred_reads = A.sorted_reduce ? (hc[4] & 0xffffffffu) : 0;
    unsigned ovf = unsigned(hc[2] & 0xffffffffu);
    const idx_t* ovf_src = ctx->ovf_list.as<idx_t>();
    const unsigned* ovf_cnt = reinterpret_cast<const unsigned*>(ctr + 2);     // device count of ovf_src
    ctx->heavy_reads = 0;
    ctx->ms_heavy = ctx->ms_wide = 0;
    auto wall_ms = [] {
        return std::chrono::duration<float, std::milli>(std::chrono::steady_clock::now().time_since_epoch()).count();
    };
    ctx->block_reads = 0;
    ctx->ms_block = 0;
    if (ovf && A.sorted_reduce) {
        // block tier (one CTA a read, all-pairs reduction in shared memory) over the reads the fast
        // tier could not hold; the ones it cannot hold either go on to the heavy tier.  Seed mode 0
        // keeps the reference's DFS for every read and skips it.
        const float tb0 = wall_ms();
        CK(ctx->ovf3.ensure(nrp * sizeof(idx_t)));
        CK(cudaMemsetAsync(ctr + 7, 0, sizeof(unsigned long long), ctx->st));
        CK(pq::search_block(A, O, ctx->ovf_list.as<idx_t>(), reinterpret_cast<const unsigned*>(ctr + 2), ovf,
                            ctx->ovf3.as<idx_t>(), reinterpret_cast<unsigned*>(ctr + 7), ctx->st));
        unsigned long long h7 = 0;
        CK(cudaMemcpyAsync(&h7, ctr + 7, sizeof h7, cudaMemcpyDeviceToHost, ctx->st));
        CK(cudaStreamSynchronize(ctx->st));
        const unsigned left = unsigned(h7 & 0xffffffffu);
        if (pq::block_tier_holds(ctx->L, ctx->t)) {
            ctx->block_reads = ovf - left;
            ovf = left;
            ovf_src = ctx->ovf3.as<idx_t>();
            ovf_cnt = reinterpret_cast<const unsigned*>(ctr + 7);
            if (ovf) {
                // the same tier with its candidate arrays in global memory, for sides of up to
                // 32768 candidates
                const int gb = pq::block_global_blocks(ovf);
                const size_t gbytes = pq::block_global_bytes(ctx->L, ctx->t, gb);
                CK(ctx->block_scratch.ensure(gbytes));
                CK(ctx->ovf4.ensure(nrp * sizeof(idx_t)));
                CK(cudaMemsetAsync(ctr + 8, 0, sizeof(unsigned long long), ctx->st));
                CK(pq::search_block_global(A, O, ovf_src, ovf_cnt, ovf, gb, ctx->block_scratch.p, gbytes,
                                           ctx->ovf4.as<idx_t>(), reinterpret_cast<unsigned*>(ctr + 8), ctx->st));
                unsigned long long h8 = 0;
                CK(cudaMemcpyAsync(&h8, ctr + 8, sizeof h8, cudaMemcpyDeviceToHost, ctx->st));
                CK(cudaStreamSynchronize(ctx->st));
                const unsigned left2 = unsigned(h8 & 0xffffffffu);
                ctx->block_reads += ovf - left2;
                ovf = left2;
                ovf_src = ctx->ovf4.as<idx_t>();
                ovf_cnt = reinterpret_cast<const unsigned*>(ctr + 8);
                // reads that found the edge pool full: grow it past everything reserved so far
                // (twice that covers every failed reservation made again) and run them once more
                unsigned long long reserved = 0;
                if (ovf) {
                    CK(cudaMemcpyAsync(&reserved, ctr + 0, sizeof reserved, cudaMemcpyDeviceToHost, ctx->st));
                    CK(cudaStreamSynchronize(ctx->st));
                }
                if (ovf && reserved > O.e_cap) {
                    const size_t need = size_t(2 * reserved + 4096), keep = O.e_cap;
                    CK(ctx->e_dest.grow(need * sizeof(idx_t), keep * sizeof(idx_t), ctx->st));
                    CK(ctx->e_trans.grow(need * 4, keep * 4, ctx->st));
                    CK(ctx->e_len.grow(need * 2, keep * 2, ctx->st));
                    CK(ctx->e_type.grow(need, keep, ctx->st));
                    O.e_dest = ctx->e_dest.as<idx_t>();
                    O.e_trans = ctx->e_trans.as<int32_t>();
                    O.e_len = ctx->e_len.as<uint16_t>();
                    O.e_type = ctx->e_type.as<uint8_t>();
                    O.e_cap = need;
                    const int gb2 = pq::block_global_blocks(ovf);
                    const size_t gbytes2 = pq::block_global_bytes(ctx->L, ctx->t, gb2);
                    CK(ctx->block_scratch.ensure(gbytes2));
                    CK(cudaMemsetAsync(ctr + 7, 0, sizeof(unsigned long long), ctx->st));
                    CK(pq::search_block_global(A, O, ovf_src, ovf_cnt, ovf, gb2, ctx->block_scratch.p, gbytes2,
                                               ctx->ovf3.as<idx_t>(), reinterpret_cast<unsigned*>(ctr + 7), ctx->st));
                    unsigned long long h7b = 0;
                    CK(cudaMemcpyAsync(&h7b, ctr + 7, sizeof h7b, cudaMemcpyDeviceToHost, ctx->st));
                    CK(cudaStreamSynchronize(ctx->st));
                    const unsigned left3 = unsigned(h7b & 0xffffffffu);
                    ctx->block_reads += ovf - left3;
                    ovf = left3;
                    ovf_src = ctx->ovf3.as<idx_t>();
                    ovf_cnt = reinterpret_cast<const unsigned*>(ctr + 7);
                }
            }
        }
        ctx->ms_block = wall_ms() - tb0;
    }
    const float th0 = wall_ms();
    if (ovf) {
        // heavy tier (the fast kernel's DFS with larger capacities) over the reads the fast tier
        // could not hold; what it cannot hold either goes on to the wide tier
        const int hebcap = 4096;
        const int hblocks = int(std::min<size_t>((size_t(ovf) + 127) / 128, size_t(152) * 2));
        const size_t hbytes = pq::heavy_scratch_bytes(ctx->L, ctx->t, hblocks, hebcap);
        CK(ctx->heavy_scratch.ensure(hbytes));
        CK(ctx->ovf2.ensure(nrp * sizeof(idx_t)));
        pq::SearchOut O2 = O;
        O2.ovf_list = ctx->ovf2.as<idx_t>();
        O2.ovf_count = reinterpret_cast<unsigned int*>(ctr + 5);
        CK(cudaMemsetAsync(ctr + 5, 0, sizeof(unsigned long long), ctx->st));
        // the heavy tier's list: the block tiers' leftovers, or the fast tier's own
        CK(pq::search_heavy(A, O2, ovf_src, ovf_cnt, hblocks, ctx->heavy_scratch.p, hbytes, hebcap, ctx->st));
        unsigned long long h5 = 0;
        CK(cudaMemcpyAsync(&h5, ctr + 5, sizeof h5, cudaMemcpyDeviceToHost, ctx->st));
        CK(cudaStreamSynchronize(ctx->st));
        ctx->heavy_reads = ovf;
        ovf = unsigned(h5 & 0xffffffffu);
        ovf_src = ctx->ovf2.as<idx_t>();
        ctx->ms_heavy = wall_ms() - th0;
    }
    const float tw0 = wall_ms();
    ctx->wide_reads = ovf;
    if (ovf) {
        // wide tier over the overflow list; retried after growing the edge pool if needed
        std::vector<idx_t> list(ovf);
        CK(cudaMemcpyAsync(list.data(), ovf_src, ovf * sizeof(idx_t), cudaMemcpyDeviceToHost, ctx->st));
        CK(cudaStreamSynchronize(ctx->st));
        const size_t slot_bytes = pq::wide_slot_bytes(ctx->L);
        // one thread per read: as many slots as a quarter of the free memory holds (at most 32 GB)
        size_t free_b = 0, total_b = 0;
        if (cudaMemGetInfo(&free_b, &total_b) != cudaSuccess) free_b = size_t(16) << 30;
        const size_t budget = std::min(free_b / 4, size_t(32) << 30);
        int slots = int(std::max<size_t>(1, std::min<size_t>({size_t(ovf), size_t(16384), budget / slot_bytes})));
        pq::WideScratch W{};
        W.stack_cap = size_t(2 * ctx->L) * size_t(2 * ctx->L);
        W.frame_cap = size_t(ctx->L + 2);
        W.edge_cap = size_t(2 * 65535 + 2);
        W.slots = slots;
        CK(ctx->wide.ensure(slot_bytes * slots + 1024));
        const size_t st_bytes = W.stack_cap * slots * pq::kCandBytes;
        const size_t fr_bytes = W.frame_cap * slots * pq::kFrameBytes;
        W.stack = ctx->wide.p;
        W.frames = static_cast<char*>(ctx->wide.p) + ((st_bytes + 255) & ~size_t(255));
        W.edges = static_cast<char*>(W.frames) + ((fr_bytes + 255) & ~size_t(255));
        DevBuf dlist;
        for (int attempt = 0; attempt < 8 && !list.empty(); ++attempt) {
            CK(dlist.ensure(list.size() * sizeof(idx_t)));
            CK(cudaMemcpyAsync(dlist.p, list.data(), list.size() * sizeof(idx_t), cudaMemcpyHostToDevice, ctx->st));
            CK(pq::search_wide(A, O, dlist.as<idx_t>(), unsigned(list.size()), W, ctx->st));
            std::vector<uint8_t> stv(nr);
            CK(cudaMemcpyAsync(stv.data(), ctx->status.p, nr, cudaMemcpyDeviceToHost, ctx->st));
            CK(cudaMemcpyAsync(hc, ctr, sizeof hc, cudaMemcpyDeviceToHost, ctx->st));
            CK(cudaStreamSynchronize(ctx->st));
            std::vector<idx_t> again;
            for (idx_t r : list) {
                uint8_t s = stv[r];
                if (s == ERR_TOO_MANY) {
                    dlist.release();
                    return fail(ctx, PQ_ERR_TOO_MANY_EDGES, "assembly failed. Try a larger min overlap length.");
                }
                if (s == ERR_CAP) {
                    dlist.release();
                    return fail(ctx, PQ_ERR_CAPACITY, "interval table exceeded (2L)^2 entries for read " +
                                                          std::to_string((unsigned long long)r));
                }
                if (s == OVF_POOL) again.push_back(r);
                else if (s != OVF_NONE) {
                    dlist.release();
                    return fail(ctx, PQ_ERR_INTERNAL, "wide search left read unfinished");
                }
            }
            if (again.empty()) { list.clear(); break; }
            // grow the pool past everything reserved so far plus a full worst case per retried read
            size_t need = size_t(hc[0]) + again.size() * size_t(2 * 65535 + 2);
            size_t keep = std::min<size_t>(size_t(hc[0]), O.e_cap);
            CK(ctx->e_dest.grow(need * sizeof(idx_t), keep * sizeof(idx_t), ctx->st));
            CK(ctx->e_trans.grow(need * 4, keep * 4, ctx->st));
            CK(ctx->e_len.grow(need * 2, keep * 2, ctx->st));
            CK(ctx->e_type.grow(need, keep, ctx->st));
            O.e_dest = ctx->e_dest.as<idx_t>();
            O.e_trans = ctx->e_trans.as<int32_t>();
            O.e_len = ctx->e_len.as<uint16_t>();
            O.e_type = ctx->e_type.as<uint8_t>();
            O.e_cap = need;
            list.swap(again);
        }
        dlist.release();
        if (!list.empty()) return fail(ctx, PQ_ERR_INTERNAL, "edge pool retries exhausted");
    }
    if (ctx->wide_reads) ctx->ms_wide = wall_ms() - tw0;
    // CSR in read order
    CK(ctx->off.ensure(nrp * 8));
    unsigned long long total = 0;
    size_t atb = pq::assemble_tmp_bytes(ctx->num_reads);
    CK(ctx->asm_tmp.ensure(atb));
    // size the CSR from the per-read counts
    {
        CK(pq::assemble_counts_total(O, ctx->num_reads, ctx->off.as<unsigned long long>(), ctx->asm_tmp.p, atb,
                                     ctx->st));
        CK(cudaMemcpyAsync(&total, ctx->off.as<unsigned long long>() + nr, 8, cudaMemcpyDeviceToHost, ctx->st));
        CK(cudaStreamSynchronize(ctx->st));
    }
    CK(ctx->g_dest.ensure((total + 1) * sizeof(idx_t)));
    CK(ctx->g_len.ensure((total + 1) * 2));
    CK(ctx->g_type.ensure(total + 1));
    CK(ctx->g_trans.ensure((total + 1) * 4));
    CK(pq::assemble_gather(O, ctx->num_reads, ctx->off.as<unsigned long long>(), ctx->g_dest.as<idx_t>(),
                           ctx->g_len.as<uint16_t>(), ctx->g_type.as<uint8_t>(), ctx->g_trans.as<int32_t>(), ctx->st));
    CK(cudaEventRecord(ctx->ev1, ctx->st));
    CK(cudaMemcpyAsync(hc, ctr, sizeof hc, cudaMemcpyDeviceToHost, ctx->st));
    unsigned long long sec = 0;
    CK(cudaMemcpyAsync(&sec, ctr + 6, sizeof sec, cudaMemcpyDeviceToHost, ctx->st));
    CK(cudaEventSynchronize(ctx->ev1));
    CK(cudaStreamSynchronize(ctx->st));
    cudaEventElapsedTime(&ctx->ms_search, ctx->ev0, ctx->ev1);
    cudaEventElapsedTime(&ctx->ms_fast, ctx->evk0, ctx->evk1);
    ctx->num_edges = total;
    ctx->probes = hc[1];
    ctx->sectors = sec;
    ctx->graph_ok = true;
    return PQ_OK;
}

int pq_overlaps(pq_ctx* ctx) {
    if (!ctx) return PQ_ERR_ARG;
    pq::SearchArgs A{};
    pq::SearchOut O{};
    int rc = search_prepare(ctx, A, O);
    if (rc != PQ_OK) return rc;
    const size_t nr = ctx->num_reads;
    CK(cudaEventRecord(ctx->ev0, ctx->st));
    int dev_sms = 152;
    cudaDeviceGetAttribute(&dev_sms, cudaDevAttrMultiProcessorCount, ctx->device);
    CK(cudaEventRecord(ctx->evk0, ctx->st));
    if (nr && A.sorted_reduce) {
        // lean tier over every read (thread per read), then the fast tier over what it hands over
        const int ebcap = 64;
        const int lean = int(std::min<size_t>((nr + 127) / 128, size_t(pq::search_lean_blocks(ctx->L, ctx->L - ctx->t, dev_sms))));
        const int fast = pq::search_fast_blocks(ctx->L, ctx->L - ctx->t, dev_sms);
        const size_t wsb = pq::lean_scratch_bytes(ctx->L, ctx->t, lean, fast, ebcap);
        CK(ctx->warp_scratch.ensure(wsb));
        CK(pq::search_lean(A, O, lean, fast, ctx->warp_scratch.p, wsb, ebcap, ctx->st));
    } else if (nr) {
        // 4 warps per block, each warp 32 reads per batch; enough blocks to fill every SM
        const int ebcap = 64;
        int blocks = int(std::min<size_t>((nr + 127) / 128, size_t(pq::search_fast_blocks(ctx->L, ctx->L - ctx->t, dev_sms))));
        const size_t wsb = pq::warp_scratch_bytes(ctx->L, ctx->t, size_t(blocks) * 4, ebcap);
        CK(ctx->warp_scratch.ensure(wsb));
        CK(pq::search_fast(A, O, blocks, ctx->warp_scratch.p, wsb, ebcap, ctx->st));
    }
    CK(cudaEventRecord(ctx->evk1, ctx->st));
    return search_finish(ctx, A, O);
}

int pq_get_graph_sizes(pq_ctx* ctx, uint64_t* num_edges, uint64_t* probes, uint64_t* wide_reads) {
    if (!ctx) return PQ_ERR_ARG;
    if (!ctx->graph_ok) return fail(ctx, PQ_ERR_STATE, "pq_overlaps first");
    if (num_edges) *num_edges = ctx->num_edges;
    if (probes) *probes = ctx->probes;
    if (wide_reads) *wide_reads = ctx->wide_reads;
    return PQ_OK;
}

int pq_get_search_traffic(pq_ctx* ctx, uint64_t* load_sectors, uint64_t* store_bytes) {
    if (!ctx) return PQ_ERR_ARG;
    if (!ctx->graph_ok) return fail(ctx, PQ_ERR_STATE, "pq_overlaps first");
    if (load_sectors) *load_sectors = ctx->sectors;
    // per read: num_B, num_F (2 + 2), olp_B, olp_F (4 + 4), edge-pool offset (8), status (1);
    // per edge: dest, trans (4), length (2), type (1)
    if (store_bytes) *store_bytes = uint64_t(ctx->num_reads) * 21 + ctx->num_edges * (sizeof(idx_t) + 7);
    return PQ_OK;
}

int pq_get_graph(pq_ctx* ctx, uint16_t* num_B, uint16_t* num_F, int32_t* olp_B, int32_t* olp_F, uint64_t* edge_off,
                 pq_idx* dest, uint16_t* len, uint8_t* type, int32_t* trans) {
    if (!ctx) return PQ_ERR_ARG;
    if (!ctx->graph_ok) return fail(ctx, PQ_ERR_STATE, "pq_overlaps first");
    const size_t nr = ctx->num_reads, ne = ctx->num_edges;
    cudaStream_t s = ctx->st;
    // page-locked destinations are written by the copy kernel, pageable ones by cudaMemcpy
    auto d2h = [&](void* h, const DevBuf& b, size_t bytes) -> cudaError_t {
        if (!h || !bytes) return cudaSuccess;
        if (void* locked = locked_device_ptr(h)) return pq::kernel_copy(locked, b.p, bytes, s);
        return cudaMemcpyAsync(h, b.p, bytes, cudaMemcpyDeviceToHost, s);
    };
    CK(d2h(num_B, ctx->nB, nr * 2));
    CK(d2h(num_F, ctx->nF, nr * 2));
    CK(d2h(olp_B, ctx->oB, nr * 4));
    CK(d2h(olp_F, ctx->oF, nr * 4));
    CK(d2h(edge_off, ctx->off, (nr + 1) * 8));
    CK(d2h(dest, ctx->g_dest, ne * sizeof(idx_t)));
    CK(d2h(len, ctx->g_len, ne * 2));
    CK(d2h(type, ctx->g_type, ne));
    CK(d2h(trans, ctx->g_trans, ne * 4));
    CK(cudaStreamSynchronize(s));
    return PQ_OK;
}

int pq_get_stage_ms(pq_ctx* ctx, float* sort_ms, float* fm_ms, float* search_ms) {
    if (!ctx) return PQ_ERR_ARG;
    if (sort_ms) *sort_ms = ctx->ms_sort;
    if (fm_ms) *fm_ms = ctx->ms_fm;
    if (search_ms) *search_ms = ctx->ms_search;
    return PQ_OK;
}

int pq_get_tier_stats(pq_ctx* ctx, uint64_t* reads, float* ms) {
    if (!ctx) return PQ_ERR_ARG;
    if (!ctx->graph_ok) return fail(ctx, PQ_ERR_STATE, "pq_overlaps first");
    if (reads) {
        reads[0] = ctx->deferred_reads;
        reads[1] = ctx->block_reads;
        reads[2] = ctx->heavy_reads;
        reads[3] = ctx->wide_reads;
    }
    if (ms) {
        ms[0] = ctx->ms_fast;
        ms[1] = ctx->ms_block;
        ms[2] = ctx->ms_heavy;
        ms[3] = ctx->ms_wide;
    }
    return PQ_OK;
}

int pq_get_kernel_stats(pq_ctx* ctx, float* search_kernel_ms, unsigned long long* launches) {
    if (!ctx) return PQ_ERR_ARG;
    if (search_kernel_ms) *search_kernel_ms = ctx->ms_fast;
    if (launches) *launches = pq::launch_count();
    return PQ_OK;
}

// ---------------------------------------------------------------------------- learned index

int pq_learned_build(pq_ctx* ctx, int dir, int steps) {
    if (!ctx || (dir != 0 && dir != 1) || steps < 0) return PQ_ERR_ARG;
    if (!ctx->fm_ok[dir]) return fail(ctx, PQ_ERR_STATE, "pq_learned_build needs pq_build_fm first");
    cudaSetDevice(ctx->device);
    const size_t n = n_rows(ctx);
    ctx->lx_ok[dir] = false;
    pq_learned_info info = {};
    info.hidden = pq::kLxHidden;
    info.steps = steps;
    if (n == 0) {
        ctx->lx_segs[dir] = 0;
        ctx->lx_info[dir] = info;
        ctx->lx_ok[dir] = true;
        return PQ_OK;
    }
    CK(ctx->lx_tmp.ensure(pq::lx_tmp_bytes(n)));
    const pq::LxTmp T = pq::lx_tmp_layout(ctx->lx_tmp.p, n);
    unsigned long long m = 0;
    CK(cudaEventRecord(ctx->ev0, ctx->st));
    CK(pq::lx_distinct_keys(ctx->sa[dir].as<idx_t>(), ctx->pk[dir].as<uint64_t>(), n, idx_t(ctx->L), T, &m, ctx->st));
    CK(cudaEventRecord(ctx->ev1, ctx->st));
    CK(cudaEventSynchronize(ctx->ev1));
    cudaEventElapsedTime(&info.keys_ms, ctx->ev0, ctx->ev1);
    const int S = int(std::min<unsigned long long>(pq::kLxMaxSegs, m));
    CK(ctx->lx_bnd[dir].ensure(size_t(S) * 4 + 64));
    CK(ctx->lx_base[dir].ensure(size_t(S + 1) * sizeof(idx_t) + 64));
    CK(ctx->lx_par[dir].ensure(size_t(S) * pq::kLxStride * sizeof(float) + 64));
    CK(ctx->lx_err[dir].ensure(size_t(S) * 8 + 64));
    CK(ctx->lx_err_root[dir].ensure(size_t(S) * 8 + 64));
    CK(ctx->lx_segof[dir].ensure(65537 * 2 + 64));
    CK(pq::lx_root(T, m, n, S, ctx->lx_bnd[dir].as<uint32_t>(), ctx->lx_base[dir].as<idx_t>(),
                   ctx->lx_segof[dir].as<uint16_t>(), ctx->st));
    CK(cudaEventRecord(ctx->ev0, ctx->st));
    CK(pq::lx_train(T, ctx->lx_bnd[dir].as<uint32_t>(), ctx->lx_base[dir].as<idx_t>(), S, steps, 0.03f,
                    0x51ed5eedu + uint32_t(dir), ctx->lx_par[dir].as<float>(), ctx->st));
    CK(cudaEventRecord(ctx->ev1, ctx->st));
    CK(cudaEventSynchronize(ctx->ev1));
    cudaEventElapsedTime(&info.train_ms, ctx->ev0, ctx->ev1);
    ctx->lx_segs[dir] = S;
    ctx->lx_ok[dir] = true;
    const LearnedView v = lx_view(ctx, dir);
    CK(cudaEventRecord(ctx->ev0, ctx->st));
    CK(pq::lx_errors(T, v, ctx->lx_err[dir].as<int32_t>(), ctx->lx_err_root[dir].as<int32_t>(), ctx->st));
    CK(cudaEventRecord(ctx->ev1, ctx->st));
    CK(cudaEventSynchronize(ctx->ev1));
    cudaEventElapsedTime(&info.eval_ms, ctx->ev0, ctx->ev1);
    // window statistics, weighted by the keys of each segment
    std::vector<int32_t> e(2 * S), er(2 * S);
    std::vector<unsigned long long> dsi(S + 1);
    CK(cudaMemcpy(e.data(), ctx->lx_err[dir].p, 8 * size_t(S), cudaMemcpyDeviceToHost));
    CK(cudaMemcpy(er.data(), ctx->lx_err_root[dir].p, 8 * size_t(S), cudaMemcpyDeviceToHost));
    CK(cudaMemcpy(dsi.data(), T.dsi, 8 * size_t(S + 1), cudaMemcpyDeviceToHost));
    double sw = 0, swr = 0;
    for (int s = 0; s < S; ++s) {
        const double keys = double(dsi[s + 1] - dsi[s]);
        const int64_t w = int64_t(e[2 * s]) + e[2 * s + 1], wr = int64_t(er[2 * s]) + er[2 * s + 1];
        sw += keys * double(w);
        swr += keys * double(wr);
        info.max_window = std::max(info.max_window, w);
        info.max_window_root = std::max(info.max_window_root, wr);
    }
    info.num_keys = m;
    info.segments = S;
    info.mean_window = m ? sw / double(m) : 0.0;
    info.mean_window_root = m ? swr / double(m) : 0.0;
    ctx->lx_info[dir] = info;
    ctx->lx_tmp.release();
    ctx->graph_ok = false;
    return PQ_OK;
}

int pq_learned_get_info(pq_ctx* ctx, int dir, pq_learned_info* info) {
    if (!ctx || (dir != 0 && dir != 1) || !info) return PQ_ERR_ARG;
    if (!ctx->lx_ok[dir]) return fail(ctx, PQ_ERR_STATE, "no learned index for this direction");
    *info = ctx->lx_info[dir];
    info->queries = ctx->lx_queries;
    info->misses = ctx->lx_misses;
    return PQ_OK;
}

int pq_learned_export(pq_ctx* ctx, int dir, uint32_t* bnd, pq_idx* base, float* params, int32_t* err,
                      int32_t* err_root) {
    if (!ctx || (dir != 0 && dir != 1)) return PQ_ERR_ARG;
    if (!ctx->lx_ok[dir]) return fail(ctx, PQ_ERR_STATE, "no learned index for this direction");
    const size_t S = size_t(ctx->lx_segs[dir]);
    if (!S) return PQ_OK;
    if (bnd) CK(cudaMemcpy(bnd, ctx->lx_bnd[dir].p, S * 4, cudaMemcpyDeviceToHost));
    if (base) CK(cudaMemcpy(base, ctx->lx_base[dir].p, (S + 1) * sizeof(idx_t), cudaMemcpyDeviceToHost));
    if (params) CK(cudaMemcpy(params, ctx->lx_par[dir].p, S * pq::kLxStride * 4, cudaMemcpyDeviceToHost));
    if (err) CK(cudaMemcpy(err, ctx->lx_err[dir].p, S * 8, cudaMemcpyDeviceToHost));
    if (err_root) CK(cudaMemcpy(err_root, ctx->lx_err_root[dir].p, S * 8, cudaMemcpyDeviceToHost));
    return PQ_OK;
}

int pq_learned_predict(pq_ctx* ctx, int dir, const uint32_t* keys, uint64_t n, int64_t* pred, int32_t* seg) {
    if (!ctx || (dir != 0 && dir != 1) || (n && (!keys || !pred || !seg))) return PQ_ERR_ARG;
    if (!ctx->lx_ok[dir] || !ctx->lx_segs[dir]) return fail(ctx, PQ_ERR_STATE, "no learned index for this direction");
    if (!n) return PQ_OK;
    cudaSetDevice(ctx->device);
    DevBuf dk, dp, ds;
    CK(dk.ensure(n * 4));
    CK(dp.ensure(n * 8));
    CK(ds.ensure(n * 4));
    CK(cudaMemcpyAsync(dk.p, keys, n * 4, cudaMemcpyHostToDevice, ctx->st));
    CK(pq::lx_predict_keys(lx_view(ctx, dir), dk.as<uint32_t>(), n, dp.as<long long>(), ds.as<int32_t>(), ctx->st));
    CK(cudaMemcpyAsync(pred, dp.p, n * 8, cudaMemcpyDeviceToHost, ctx->st));
    CK(cudaMemcpyAsync(seg, ds.p, n * 4, cudaMemcpyDeviceToHost, ctx->st));
    CK(cudaStreamSynchronize(ctx->st));
    dk.release();
    dp.release();
    ds.release();
    return PQ_OK;
}

int pq_learned_keys(pq_ctx* ctx, int dir, uint32_t* keys, pq_idx* first_row, uint64_t cap, uint64_t* num_keys) {
    if (!ctx || (dir != 0 && dir != 1) || !num_keys) return PQ_ERR_ARG;
    if (!ctx->fm_ok[dir]) return fail(ctx, PQ_ERR_STATE, "pq_learned_keys needs pq_build_fm first");
    cudaSetDevice(ctx->device);
    const size_t n = n_rows(ctx);
    *num_keys = 0;
    if (!n) return PQ_OK;
    CK(ctx->lx_tmp.ensure(pq::lx_tmp_bytes(n)));
    const pq::LxTmp T = pq::lx_tmp_layout(ctx->lx_tmp.p, n);
    unsigned long long m = 0;
    CK(pq::lx_distinct_keys(ctx->sa[dir].as<idx_t>(), ctx->pk[dir].as<uint64_t>(), n, idx_t(ctx->L), T, &m, ctx->st));
    const size_t c = size_t(std::min<unsigned long long>(m, cap));
    if (keys && c) CK(cudaMemcpy(keys, T.kd, c * 4, cudaMemcpyDeviceToHost));
    if (first_row && c) CK(cudaMemcpy(first_row, T.fd, c * sizeof(idx_t), cudaMemcpyDeviceToHost));
    *num_keys = m;
    ctx->lx_tmp.release();
    return PQ_OK;
}

int pq_mlp_forward(const float* params, const float* x, int n, float* y) {
    if (!params || n < 0 || (n && (!x || !y))) return PQ_ERR_ARG;
    DevBuf dp, dx, dy;
    if (dp.ensure(pq::kLxStride * 4) || dx.ensure(size_t(n) * 4 + 4) || dy.ensure(size_t(n) * 4 + 4)) return PQ_ERR_NOMEM;
    int rc = PQ_OK;
    if (cudaMemcpy(dp.p, params, pq::kLxStride * 4, cudaMemcpyHostToDevice) != cudaSuccess ||
        (n && cudaMemcpy(dx.p, x, size_t(n) * 4, cudaMemcpyHostToDevice) != cudaSuccess) ||
        pq::mlp_forward(dp.as<float>(), dx.as<float>(), n, dy.as<float>(), 0) != cudaSuccess ||
        (n && cudaMemcpy(y, dy.p, size_t(n) * 4, cudaMemcpyDeviceToHost) != cudaSuccess))
        rc = PQ_ERR_CUDA;
    dp.release();
    dx.release();
    dy.release();
    return rc;
}

int pq_mlp_backward(const float* params, const float* x, const float* dy, int n, float* grad) {
    if (!params || !grad || n < 0 || (n && (!x || !dy))) return PQ_ERR_ARG;
    DevBuf dp, dx, dg, dd;
    if (dp.ensure(pq::kLxStride * 4) || dx.ensure(size_t(n) * 4 + 4) || dd.ensure(size_t(n) * 4 + 4) ||
        dg.ensure(pq::kLxParams * 4))
        return PQ_ERR_NOMEM;
    int rc = PQ_OK;
    if (cudaMemcpy(dp.p, params, pq::kLxStride * 4, cudaMemcpyHostToDevice) != cudaSuccess ||
        (n && cudaMemcpy(dx.p, x, size_t(n) * 4, cudaMemcpyHostToDevice) != cudaSuccess) ||
        (n && cudaMemcpy(dd.p, dy, size_t(n) * 4, cudaMemcpyHostToDevice) != cudaSuccess) ||
        pq::mlp_backward(dp.as<float>(), dx.as<float>(), dd.as<float>(), n, dg.as<float>(), 0) != cudaSuccess ||
        cudaMemcpy(grad, dg.p, pq::kLxParams * 4, cudaMemcpyDeviceToHost) != cudaSuccess)
        rc = PQ_ERR_CUDA;
    dp.release();
    dx.release();
    dd.release();
    dg.release();
    return rc;
}

int pq_mlp_adam_step(float* params, float* m1, float* m2, const float* x, const float* target, int n, int step,
                     float lr) {
    if (!params || !m1 || !m2 || n <= 0 || !x || !target || step < 1) return PQ_ERR_ARG;
    DevBuf dp, dm1, dm2, dx, dt;
    if (dp.ensure(pq::kLxStride * 4) || dm1.ensure(pq::kLxParams * 4) || dm2.ensure(pq::kLxParams * 4) ||
        dx.ensure(size_t(n) * 4) || dt.ensure(size_t(n) * 4))
        return PQ_ERR_NOMEM;
    int rc = PQ_OK;
    if (cudaMemcpy(dp.p, params, pq::kLxStride * 4, cudaMemcpyHostToDevice) != cudaSuccess ||
        cudaMemcpy(dm1.p, m1, pq::kLxParams * 4, cudaMemcpyHostToDevice) != cudaSuccess ||
        cudaMemcpy(dm2.p, m2, pq::kLxParams * 4, cudaMemcpyHostToDevice) != cudaSuccess ||
        cudaMemcpy(dx.p, x, size_t(n) * 4, cudaMemcpyHostToDevice) != cudaSuccess ||
        cudaMemcpy(dt.p, target, size_t(n) * 4, cudaMemcpyHostToDevice) != cudaSuccess ||
        pq::mlp_adam_step(dp.as<float>(), dm1.as<float>(), dm2.as<float>(), dx.as<float>(), dt.as<float>(), n, step,
                          lr, 0) != cudaSuccess ||
        cudaMemcpy(params, dp.p, pq::kLxParams * 4, cudaMemcpyDeviceToHost) != cudaSuccess ||
        cudaMemcpy(m1, dm1.p, pq::kLxParams * 4, cudaMemcpyDeviceToHost) != cudaSuccess ||
        cudaMemcpy(m2, dm2.p, pq::kLxParams * 4, cudaMemcpyDeviceToHost) != cudaSuccess)
        rc = PQ_ERR_CUDA;
    dp.release();
    dm1.release();
    dm2.release();
    dx.release();
    dt.release();
    return rc;
}

// ---------------------------------------------------------------------------- queued search

static uint64_t fnv1a(const void* p, size_t n) {
    const unsigned char* c = static_cast<const unsigned char*>(p);
    uint64_t h = 1469598103934665603ull;
    for (size_t i = 0; i < n; ++i) h = (h ^ c[i]) * 1099511628211ull;
    return h;
}

// One queued search over the batch descriptions already on the device (lead->q_batches, copies
// of hb).  Lean path (every batch reduces by sorted continuations): the batches are split by the
// continuation words their kernels are built for (L - t <= 64 or not); each class is one
// persistent lean launch over its own queue, followed by the fast tier over its batches'
// handed-over reads.  Otherwise one fast-kernel launch over the whole queue.
static int queue_launch(pq_ctx* lead, const std::vector<pq::SearchBatch>& hb, const std::vector<int>& order,
                        int use_graph) {
    pq_ctx* ctx = lead;
    int dev_sms = 152;
    cudaDeviceGetAttribute(&dev_sms, cudaDevAttrMultiProcessorCount, lead->device);
    bool lean = true;
    for (const auto& b : hb) lean = lean && b.a.sorted_reduce;
    const unsigned gpi = unsigned(std::max(1, lead->q_groups_per_item));
    // classes of batches, each with its items (batch, first group), longest reads first
    struct Class {
        std::vector<int> batches;
        std::vector<uint32_t> ib, ig;
        int L_max = 1, M_max = 1;
    };
    std::vector<Class> cls(lean ? 2 : 1);
    for (int b : order) {
        const int M = hb[b].a.L - hb[b].a.t;
        Class& c = cls[lean && pq::lam_words_host(M) != 2 ? 1 : 0];
        c.batches.push_back(b);
        c.L_max = std::max(c.L_max, hb[b].a.L);
        c.M_max = std::max(c.M_max, M);
        const size_t groups = (size_t(hb[b].a.num_reads) + 31) / 32;
        for (size_t g = 0; g < groups; g += gpi) {
            c.ib.push_back(uint32_t(b));
            c.ig.push_back(uint32_t(g));
        }
    }
    size_t nitems = 0, scratch = 0;
    struct Plan {
        int blocks, fast_blocks;
        size_t wsb, first;
    };
    std::vector<Plan> plan(cls.size());
    for (size_t k = 0; k < cls.size(); ++k) {
        const Class& c = cls[k];
        const int fast_max = pq::search_fast_blocks(c.L_max, c.M_max, 1);
        const int lean_max = pq::search_lean_blocks(c.L_max, c.M_max, 1);
        int per_sm = lean ? lean_max : fast_max;
        if (lead->q_ctas_per_sm > 0) per_sm = std::min(lead->q_ctas_per_sm, per_sm);
        Plan& p = plan[k];
        p.blocks = int(std::max<size_t>(1, std::min<size_t>(size_t(per_sm) * dev_sms, (c.ib.size() + 3) / 4)));
        p.fast_blocks = fast_max * dev_sms;
        const size_t nwarps = size_t(lean ? std::max(p.blocks, p.fast_blocks) : p.blocks) * 4;
        p.wsb = pq::queue_scratch_bytes(c.L_max, c.M_max, nwarps, lead->q_ebcap);
        p.first = nitems;
        nitems += c.ib.size();
        scratch = std::max(scratch, p.wsb);
    }
    CK(lead->warp_scratch.ensure(scratch));
    CK(lead->q_items.ensure(nitems * 8 + 64));
    CK(lead->q_next.ensure(64));
    uint32_t* d_items = lead->q_items.as<uint32_t>();
    for (size_t k = 0; k < cls.size(); ++k) {
        if (cls[k].ib.empty()) continue;
        CK(cudaMemcpyAsync(d_items + plan[k].first, cls[k].ib.data(), cls[k].ib.size() * 4, cudaMemcpyHostToDevice,
                           lead->st));
        CK(cudaMemcpyAsync(d_items + nitems + plan[k].first, cls[k].ig.data(), cls[k].ig.size() * 4,
                           cudaMemcpyHostToDevice, lead->st));
    }
    auto enqueue = [&]() -> cudaError_t {
        cudaError_t e = cudaMemsetAsync(lead->q_next.p, 0, 64, lead->st);
        for (size_t k = 0; k < cls.size() && e == cudaSuccess; ++k) {
            const Class& c = cls[k];
            if (c.ib.empty()) continue;
            pq::SearchQueue Q{};
            Q.batches = lead->q_batches.as<pq::SearchBatch>();
            Q.item_batch = d_items + plan[k].first;
            Q.item_group = d_items + nitems + plan[k].first;
            Q.count = unsigned(c.ib.size());
            Q.groups_per_item = gpi;
            Q.next = lead->q_next.as<unsigned>() + k;
            if (lean)
                e = pq::search_lean_queue(Q, hb.data(), c.batches.data(), int(c.batches.size()), c.L_max, c.M_max,
                                          plan[k].blocks, plan[k].fast_blocks, lead->warp_scratch.p, plan[k].wsb,
                                          lead->q_ebcap, lead->st);
            else
                e = pq::search_fast_queue(Q, c.L_max, c.M_max, plan[k].blocks, lead->warp_scratch.p, plan[k].wsb,
                                          lead->q_ebcap, lead->st);
        }
        return e;
    };
    lead->q_graph_used = 0;
    if (!use_graph) {
        CK(cudaEventRecord(lead->evk0, lead->st));
        CK(enqueue());
        CK(cudaEventRecord(lead->evk1, lead->st));
    } else {
        // one captured graph per launch shape and batch set: queue reset + the search launches
        std::vector<uintptr_t> key = {uintptr_t(lead->q_batches.p), uintptr_t(d_items), uintptr_t(lead->q_next.p),
                                      uintptr_t(lead->warp_scratch.p), nitems, gpi, uintptr_t(lead->q_ebcap),
                                      uintptr_t(lean), uintptr_t(fnv1a(hb.data(), hb.size() * sizeof(hb[0])))};
        for (const Plan& p : plan) {
            key.push_back(uintptr_t(p.blocks));
            key.push_back(p.first);
        }
        if (!lead->q_exec || lead->q_key != key) {
            if (lead->q_exec) cudaGraphExecDestroy(lead->q_exec);
            if (lead->q_graph) cudaGraphDestroy(lead->q_graph);
            lead->q_exec = nullptr;
            lead->q_graph = nullptr;
            CK(cudaStreamSynchronize(lead->st));
            CK(cudaStreamBeginCapture(lead->st, cudaStreamCaptureModeThreadLocal));
            const cudaError_t e1 = enqueue();
            cudaGraph_t g = nullptr;
            const cudaError_t e2 = cudaStreamEndCapture(lead->st, &g);
            CK(e1);
            CK(e2);
            lead->q_graph = g;
            CK(cudaGraphInstantiate(&lead->q_exec, g, 0));
            lead->q_key = key;
        }
        CK(cudaEventRecord(lead->evk0, lead->st));
        CK(cudaGraphLaunch(lead->q_exec, lead->st));
        pq::note_launch();
        CK(cudaEventRecord(lead->evk1, lead->st));
        lead->q_graph_used = 1;
    }
    CK(cudaEventSynchronize(lead->evk1));
    cudaEventElapsedTime(&lead->q_kernel_ms, lead->evk0, lead->evk1);
    return PQ_OK;
}

int pq_overlaps_batched(pq_ctx** ctxs, int count, int flags) {
    if (!ctxs || count <= 0) return PQ_ERR_ARG;
    pq_ctx* lead = ctxs[0];
    if (!lead) return PQ_ERR_ARG;
    for (int b = 0; b < count; ++b) {
        if (!ctxs[b]) return fail(lead, PQ_ERR_ARG, "null context in batch");
        if (ctxs[b]->device != lead->device) return fail(lead, PQ_ERR_ARG, "batched contexts must share a device");
        for (int c = 0; c < b; ++c)
            if (ctxs[c] == ctxs[b]) return fail(lead, PQ_ERR_ARG, "a context appears twice in the batch");
    }
    cudaSetDevice(lead->device);
    std::vector<pq::SearchBatch> hb(count);
    int L_max = 1, M_max = 1;
    for (int b = 0; b < count; ++b) {
        const int rc = search_prepare(ctxs[b], hb[b].a, hb[b].o);
        if (rc != PQ_OK) {
            if (b) fail(lead, rc, std::string("batch ") + std::to_string(b) + ": " + ctxs[b]->err);
            return rc;
        }
        if (ctxs[b]->st != lead->st && cudaStreamSynchronize(ctxs[b]->st) != cudaSuccess)
            return fail(lead, PQ_ERR_CUDA, "batch stream synchronisation failed");
        L_max = std::max(L_max, ctxs[b]->L);
        M_max = std::max(M_max, ctxs[b]->L - ctxs[b]->t);
    }
    // batches longest reads first (they take longest); items are built per class in queue_launch
    std::vector<int> order(count);
    for (int b = 0; b < count; ++b) order[b] = b;
    std::stable_sort(order.begin(), order.end(), [&](int x, int y) { return ctxs[x]->L > ctxs[y]->L; });
    size_t total_reads = 0;
    for (int b = 0; b < count; ++b) total_reads += ctxs[b]->num_reads;
    pq_ctx* ctx = lead;
    CK(lead->q_batches.ensure(sizeof(pq::SearchBatch) * size_t(count)));
    CK(cudaMemcpyAsync(lead->q_batches.p, hb.data(), sizeof(pq::SearchBatch) * size_t(count), cudaMemcpyHostToDevice,
                       lead->st));
    for (int b = 0; b < count; ++b) CK(cudaEventRecord(ctxs[b]->ev0, lead->st));
    if (total_reads) {
        const int rc = queue_launch(lead, hb, order, (flags & PQ_BATCH_GRAPH) ? 1 : 0);
        if (rc != PQ_OK) return rc;
    } else {
        lead->q_kernel_ms = 0;
    }
    CK(cudaStreamSynchronize(lead->st));
    for (int b = 0; b < count; ++b) {
        const int rc = search_finish(ctxs[b], hb[b].a, hb[b].o);
        if (rc != PQ_OK) {
            if (b) fail(lead, rc, std::string("batch ") + std::to_string(b) + ": " + ctxs[b]->err);
            return rc;
        }
        ctxs[b]->ms_fast = lead->q_kernel_ms;
    }
    return PQ_OK;
}

int pq_set_batch_plan(pq_ctx* lead, int ctas_per_sm, int groups_per_item, int edge_slots) {
    if (!lead || ctas_per_sm < 0 || ctas_per_sm > 32 || groups_per_item < 1 || groups_per_item > 64 ||
        edge_slots < 8 || edge_slots > 4096)
        return PQ_ERR_ARG;
    lead->q_ctas_per_sm = ctas_per_sm;
    lead->q_groups_per_item = groups_per_item;
    lead->q_ebcap = edge_slots;
    return PQ_OK;
}

int pq_get_batch_stats(pq_ctx* lead, float* kernel_ms, int* ctas_per_sm, int* groups_per_item, int* edge_slots,
                       int* graph_used) {
    if (!lead) return PQ_ERR_ARG;
    if (kernel_ms) *kernel_ms = lead->q_kernel_ms;
    if (ctas_per_sm) *ctas_per_sm = lead->q_ctas_per_sm;
    if (groups_per_item) *groups_per_item = lead->q_groups_per_item;
    if (edge_slots) *edge_slots = lead->q_ebcap;
    if (graph_used) *graph_used = lead->q_graph_used;
    return PQ_OK;
}

int pq_autotune_batched(pq_ctx** ctxs, int count, int flags, float* best_ms) {
    if (!ctxs || count <= 0 || !ctxs[0]) return PQ_ERR_ARG;
    pq_ctx* lead = ctxs[0];
    int max_per_sm = 0;
    int L_max = 1;
    for (int b = 0; b < count; ++b)
        if (ctxs[b]) L_max = std::max(L_max, ctxs[b]->L);
    max_per_sm = std::max(pq::search_fast_blocks(L_max, 256, 1), pq::search_lean_blocks(L_max, 256, 1));
    float best = -1.f;
    int bc = 0, bg = 1, be = 64;
    const int edge_opts[2] = {32, 64};
    for (int c = 2; c <= max_per_sm; ++c) {
        for (int g = 1; g <= 4; g *= 2) {
            for (int e : edge_opts) {
                lead->q_ctas_per_sm = c;
                lead->q_groups_per_item = g;
                lead->q_ebcap = e;
                float t = 0.f;
                for (int rep = 0; rep < 2; ++rep) {     // first run warms up, second is timed
                    const int rc = pq_overlaps_batched(ctxs, count, flags);
                    if (rc != PQ_OK) return rc;
                    t = lead->q_kernel_ms;
                }
                if (best < 0.f || t < best) {
                    best = t;
                    bc = c;
                    bg = g;
                    be = e;
                }
            }
        }
    }
    lead->q_ctas_per_sm = bc;
    lead->q_groups_per_item = bg;
    lead->q_ebcap = be;
    if (best_ms) *best_ms = best;
    return PQ_OK;
}

}  // extern "C"
