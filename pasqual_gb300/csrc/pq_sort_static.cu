// pq_sort_static.cu — a suffix sort that allocates no device memory.
//
// pq_sort() allocates its working memory (keys, values, ranks, packed text, BWT symbols, radix
// histograms: about 25 bytes per suffix) with cudaMalloc on first use.  Some callers cannot do that: code
// that runs inside a host application which owns every byte of device memory through its own
// pool and forbids direct cudaMalloc (an assembler or read-correction tool that embeds this sort
// for many small per-bucket sorts), and code on latency-critical paths where cudaMalloc's
// implicit device-wide synchronisation is not acceptable.  For them, pq_suffix_sort_static()
// sorts from caller-owned device buffers with its working memory in a fixed array compiled
// into this library, sized for PQ_STATIC_SORT_MAX_SUFFIXES suffixes.
//
// The array lives in every GPU that loads the library until the process exits.  All calls on
// a device share it: calls whose work overlaps on the GPU (different streams, or different
// host threads) race on it and must be ordered by the caller.  Every call writes all of the
// scratch it reads back, and clears the histogram it accumulates, before use.
//
// Each call first counts the read bytes outside the base codes 1..4 (a count kept in a second
// fixed device variable, cleared by the call) and refuses such input with PQ_ERR_ARG: the sort
// packs 2 bits a base, so another byte would corrupt its neighbours' bits and give a wrong order.
// The call synchronises its stream before it returns, so the suffix array is complete and any
// kernel error is reported as PQ_ERR_CUDA.
#include <cstdio>
#include <mutex>

#include "pq_sort.cuh"
#include "../../include/pasqual_gb300.h"

namespace {

constexpr size_t al256(size_t b) { return (b + 255) & ~size_t(255); }
constexpr size_t kMax = PQ_STATIC_SORT_MAX_SUFFIXES;

// Upper bound of pq::suffix_sort_tmp_bytes(kMax): key double buffer, one value buffer (the other
// is the caller's suffix array), 32-bit ranks, packed text, radix histograms of up to 608 CTAs
// plus 8 digit histograms, per-tile head data, one BWT-symbol byte per suffix.
constexpr size_t kScratchBytes =
    2 * al256(kMax * sizeof(uint64_t)) + al256(kMax * sizeof(idx_t)) + al256(kMax * sizeof(uint32_t)) +
    al256((kMax / 32 + 4) * sizeof(uint64_t)) + al256((256 * 608 + 8 * 256 + 64) * sizeof(unsigned long long)) +
    al256(3 * (kMax / 2048 + 2) * sizeof(unsigned long long)) + al256(kMax) + 1024;

__device__ __align__(256) unsigned char g_sort_scratch[kScratchBytes];
__device__ unsigned long long g_bad_codes;

__global__ void k_clear_bad_codes() { g_bad_codes = 0; }

// Bytes of reads[0, n) that are not a base code 1..4, added to g_bad_codes.
__global__ void k_count_bad_codes(const uint8_t* __restrict__ reads, size_t n) {
    unsigned long long bad = 0;
    for (size_t i = size_t(blockIdx.x) * blockDim.x + threadIdx.x; i < n; i += size_t(gridDim.x) * blockDim.x)
        bad += unsigned(reads[i] - 1u) > 3u;
    for (int o = 16; o; o >>= 1) bad += __shfl_xor_sync(0xffffffffu, bad, o);
    if ((threadIdx.x & 31) == 0 && bad) atomicAdd(&g_bad_codes, bad);
}

// Device address of g_sort_scratch per device, looked up once per device with that device
// current (host code must not pass the symbol itself: it is a host-side stand-in).
constexpr int kMaxDevices = 64;
void* g_addr[kMaxDevices] = {nullptr};
std::mutex g_mu;

int scratch_address(void** out) {
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices) return PQ_ERR_CUDA;
    std::lock_guard<std::mutex> g(g_mu);
    if (!g_addr[dev]) {
        void* p = nullptr;
        cudaError_t e = cudaGetSymbolAddress(&p, g_sort_scratch);
        if (e != cudaSuccess || !p) return PQ_ERR_CUDA;
        g_addr[dev] = p;
    }
    *out = g_addr[dev];
    return PQ_OK;
}

}  // namespace

extern "C" int pq_suffix_sort_static(const uint8_t* reads_dev, pq_idx num_reads, int read_len, int dir,
                                     pq_idx* sa_dev, void* cuda_stream) {
    if ((dir != 0 && dir != 1) || read_len <= 0 || read_len > 65535) return PQ_ERR_ARG;
    const unsigned __int128 n = (unsigned __int128)num_reads * (unsigned)read_len;
    if (n > kMax) return PQ_ERR_CAPACITY;
    if (n == 0) return PQ_OK;
    if (!reads_dev || !sa_dev) return PQ_ERR_ARG;
    const size_t need = pq::suffix_sort_tmp_bytes(size_t(n));
    if (need > kScratchBytes) return PQ_ERR_INTERNAL;
    void* scratch = nullptr;
    int rc = scratch_address(&scratch);
    if (rc != PQ_OK) return rc;
    cudaStream_t st = reinterpret_cast<cudaStream_t>(cuda_stream);
    const size_t nn = size_t(n);
    k_clear_bad_codes<<<1, 1, 0, st>>>();
    k_count_bad_codes<<<unsigned((nn + 255) / 256 < 1024 ? (nn + 255) / 256 : 1024), 256, 0, st>>>(reads_dev, nn);
    unsigned long long bad = 0;
    if (cudaMemcpyFromSymbolAsync(&bad, g_bad_codes, sizeof bad, 0, cudaMemcpyDeviceToHost, st) != cudaSuccess ||
        cudaStreamSynchronize(st) != cudaSuccess)
        return PQ_ERR_CUDA;
    if (bad) return PQ_ERR_ARG;
    int e = pq::suffix_sort(reads_dev, idx_t(num_reads), read_len, dir, reinterpret_cast<idx_t*>(sa_dev), scratch,
                            kScratchBytes, st);
    if (e != 0) return PQ_ERR_CUDA;
    return cudaStreamSynchronize(st) == cudaSuccess && cudaGetLastError() == cudaSuccess ? PQ_OK : PQ_ERR_CUDA;
}
