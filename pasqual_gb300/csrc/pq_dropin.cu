// pq_dropin.cu — the reference's own entry points (construct_index, construct_string_graph,
// destroy_graph; src/index.h:63-68, src/string_graph.h:139-142) served by the GPU library, with
// the reference's struct layouts (include/pasqual_gb300_dropin.h).
//
// Host work that stays on the CPU is restated here in plain C-style code: the FASTA import with
// its Bloom-filter de-duplication (src/index.c:145-405, src/bloom.c:18-135) -- sequential by
// definition, because which read of a duplicate pair survives depends on input order -- and
// the node_t construction of src/string_graph.c:832-1017.
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <sys/time.h>
#include <sys/stat.h>
#include <sys/mman.h>
#include <fcntl.h>
#include <unistd.h>
#include <unordered_map>
#include <memory>
#include <mutex>
#include <vector>
#include <string>
#include <algorithm>
#include <thread>
#include <type_traits>

#include "pq_common.cuh"
#include "pq_slots.h"
#include "../../include/pasqual_gb300.h"
#include "../../include/pasqual_gb300_dropin.h"

static_assert(sizeof(pq_index_type) == sizeof(idx_t), "index widths must agree");

// pq_api.cu: the sort of an index build, which also leaves the FM side outputs
extern "C" int pq_sort_for_index(pq_ctx* ctx, int dir);

// The reference's main() prints total time minus this (src/test.c:417-419).
extern "C" {
__attribute__((visibility("default"))) double time_importreads = 0.0;
}

namespace {

double now_ms() {
    struct timeval tv;
    gettimeofday(&tv, nullptr);
    return tv.tv_sec * 1000.0 + tv.tv_usec / 1000.0;
}

[[noreturn]] void error_exit(const char* msg) {
    // ERROR_EXIT (src/common.h:87-94): message on stderr, exit status 0
    fprintf(stderr, "Error: ");
    fprintf(stderr, "%s", msg);
    fflush(stderr);
    exit(0);
}

// ---------------------------------------------------------------- Bloom filter (src/bloom.c)
// Five string hashes over the 1..4 base codes, in index-width arithmetic; a read is a duplicate
// when all of its own hash bits are already set, or all bits of its reverse complement's hashes
// are; otherwise its own bits are set.
typedef pq_index_type (*hash_fn)(const char*, pq_index_type);

pq_index_type h_shift_xor(const char* k, pq_index_type m) {
    pq_index_type h = 0;
    while (*k) h ^= (h << 5) + (h >> 2) + (unsigned char)*k++;
    return h % m;
}
pq_index_type h_sdbm(const char* k, pq_index_type m) {
    pq_index_type h = 0;
    while (*k) h = (unsigned char)*k++ + (h << 6) + (h << 16) - h;
    return h % m;
}
pq_index_type h_sum(const char* k, pq_index_type m) {
    pq_index_type h = 0;
    while (*k) h += *k++;
    return h % m;
}
pq_index_type h_xor(const char* k, pq_index_type m) {
    pq_index_type h = 0;
    while (*k) h ^= *k++;
    return h % m;
}
pq_index_type h_times33(const char* k, pq_index_type m) {
    pq_index_type h = 0;
    while (*k) h = 33 * h + *k++;
    return h % m;
}
const hash_fn kHashes[5] = {h_shift_xor, h_sdbm, h_sum, h_xor, h_times33};

inline bool bit_get(const unsigned char* a, pq_index_type n) { return (a[n / 8] >> (n % 8)) & 1; }
inline void bit_set(unsigned char* a, pq_index_type n) { a[n / 8] |= (unsigned char)(1u << (n % 8)); }

// returns true when the read is a duplicate (src/bloom.c:91-135)
bool bloom_seen(unsigned char* bits, pq_index_type m, int nfunc, const char* fw, const char* rc) {
    pq_index_type hv[5];
    bool all = true;
    for (int i = 0; i < nfunc; ++i) {
        hv[i] = kHashes[i](fw, m);
        if (!bit_get(bits, hv[i])) all = false;
    }
    if (all) return true;
    for (int i = 0; i < nfunc; ++i) {
        if (!bit_get(bits, kHashes[i](rc, m))) {
            for (int j = 0; j < nfunc; ++j) bit_set(bits, hv[j]);
            return false;
        }
    }
    return true;
}

std::string g_import_err;

// ---------------------------------------------------------------- registry of GPU contexts
std::mutex g_mu;
std::unordered_map<const void*, pq_ctx*> g_ctx;


}  // namespace

namespace {

// The import one line at a time, exactly as the reference reads the file (fgets into 1000
// bytes); import_fasta_parallel falls back to it for inputs where a whole-file parse could
// differ from that (lines of 999 or more characters, NUL bytes).
int import_fasta_serial(const char* path, int read_len, int bloom_m, int n_hashfunc, uint8_t** reads_out,
                        pq_index_type* num_reads_out, pq_index_type* removed_out, const char** err) {
    char line[1000];
    char msg[512];
    auto bad = [&](pq_index_type kept) {
        snprintf(msg, sizeof msg, "incorrect reads file at line %llu.\n", (unsigned long long)(kept * 2 + 2));
        g_import_err = msg;
        if (err) *err = g_import_err.c_str();
        return PQ_ERR_ARG;
    };
    FILE* fp = fopen(path, "r");
    if (!fp) {
        snprintf(msg, sizeof msg, "open reads file %s failed.\n", path);
        g_import_err = msg;
        if (err) *err = g_import_err.c_str();
        return PQ_ERR_ARG;
    }
    pq_index_type records = 0;
    while (fgets(line, 1000, fp))
        if (line[0] == '>') records++;
    const pq_index_type m = records * (pq_index_type)bloom_m;
    std::vector<unsigned char> bits((size_t(m) + 7) / 8 + 1, 0);
    std::vector<uint8_t> out;
    out.reserve(size_t(records) * read_len);
    std::vector<char> fw(read_len + 1), rc(read_len + 1);
    pq_index_type kept = 0, removed = 0;
    fseek(fp, 0, SEEK_SET);
    while (fgets(line, 1000, fp)) {
        if (line[0] != '>') { fclose(fp); return bad(kept); }
        if (!fgets(line, 1000, fp)) { fclose(fp); return bad(kept); }
        const size_t got = strlen(line);     // 0 when the line starts with a NUL byte
        if (got == 0) { fclose(fp); return bad(kept); }   // the length check below fails then too
        line[got - 1] = '\0';
        if ((int)strlen(line) != read_len) { fclose(fp); return bad(kept); }
        bool with_n = false;
        for (int i = 0; i < read_len; ++i) {
            int c, r;
            switch (line[i]) {
                case 'a': case 'A': c = 1; r = 4; break;
                case 'c': case 'C': c = 2; r = 3; break;
                case 'g': case 'G': c = 3; r = 2; break;
                case 't': case 'T': c = 4; r = 1; break;
                case 'n': case 'N': with_n = true; c = 'N'; r = 0; break;
                default: fclose(fp); return bad(kept);
            }
            fw[i] = (char)c;
            rc[read_len - 1 - i] = (char)r;
        }
        fw[read_len] = 0;
        rc[read_len] = 0;
        if (with_n || bloom_seen(bits.data(), m, n_hashfunc, fw.data(), rc.data())) {
            removed++;
            continue;
        }
        out.insert(out.end(), fw.begin(), fw.begin() + read_len);
        kept++;
    }
    fclose(fp);
    uint8_t* buf = (uint8_t*)malloc(out.size() ? out.size() : 1);
    if (!buf) return PQ_ERR_NOMEM;
    if (!out.empty()) memcpy(buf, out.data(), out.size());
    *reads_out = buf;
    *num_reads_out = kept;
    if (removed_out) *removed_out = removed;
    return PQ_OK;
}

// Base symbol -> code (A=1 C=2 G=3 T=4, either case), the code of its complement, and a class:
// 0 = base, 1 = N (either case), 2 = any other byte.  Tables make the decode branch-free.
struct BaseTables {
    uint8_t fw[256], rc[256], cls[256];
    BaseTables() {
        for (int i = 0; i < 256; ++i) { fw[i] = 0; rc[i] = 0; cls[i] = 2; }
        const char* up = "ACGT";
        const char* lo = "acgt";
        for (int b = 0; b < 4; ++b) {
            for (const char* s : {up, lo}) {
                const unsigned char ch = (unsigned char)s[b];
                fw[ch] = uint8_t(b + 1);
                rc[ch] = uint8_t(4 - b);
                cls[ch] = 0;
            }
        }
        cls['N'] = cls['n'] = 1;
        fw['N'] = fw['n'] = 'N';
    }
};
const BaseTables kBases;

// The first NF string hashes of src/bloom.c over a record's base codes and over its reverse
// complement's, read straight from the sequence line through the base tables (forward codes front
// to back, complement codes back to front) in one pass of 2 * NF independent chains, in
// index-width arithmetic; hf[f] / hr[f] = hash f mod m.  Returns the OR of (1 << class) over the
// line's bytes; the hashes are stored only when no N and no other byte was seen.
template <int NF>
inline unsigned hash_line(const unsigned char* sq, int RL, pq_index_type m, pq_index_type* hf,
                          pq_index_type* hr) {
    pq_index_type a0 = 0, a1 = 0, a2 = 0, a3 = 0, a4 = 0, r0 = 0, r1 = 0, r2 = 0, r3 = 0, r4 = 0;
    unsigned cls = 0;
    for (int j = 0; j < RL; ++j) {
        const unsigned char ch = sq[j];
        cls |= 1u << kBases.cls[ch];
        const pq_index_type c = kBases.fw[ch], d = kBases.rc[sq[RL - 1 - j]];
        if (NF > 0) { a0 ^= (a0 << 5) + (a0 >> 2) + c; r0 ^= (r0 << 5) + (r0 >> 2) + d; }   // shift-xor
        if (NF > 1) { a1 = c + (a1 << 6) + (a1 << 16) - a1; r1 = d + (r1 << 6) + (r1 << 16) - r1; }   // sdbm
        if (NF > 2) { a2 += c; r2 += d; }                                                     // sum
        if (NF > 3) { a3 ^= c; r3 ^= d; }                                                     // xor
        if (NF > 4) { a4 = 33 * a4 + c; r4 = 33 * r4 + d; }                                 // times 33
    }
    if ((cls & 6u) == 0) {
        const pq_index_type av[5] = {a0, a1, a2, a3, a4}, rv[5] = {r0, r1, r2, r3, r4};
        for (int f = 0; f < NF; ++f) {
            hf[f] = av[f] % m;
            hr[f] = rv[f] % m;
        }
    }
    return cls;
}

// malloc-compatible (free()-able) memory in 2 MB-aligned whole huge pages where the kernel
// grants them on request: random accesses then miss the TLB far less often
void* alloc_huge(size_t bytes) {
    constexpr size_t kHuge = size_t(2) << 20;
    const size_t sz = (bytes + kHuge - 1) / kHuge * kHuge;
    void* p = aligned_alloc(kHuge, sz ? sz : kHuge);
    if (p && sz) madvise(p, sz, MADV_HUGEPAGE);        // advice only: ignored where unsupported
    return p;
}

template <class F>
void parallel_ranges(size_t n, int threads, F f) {
    if (n == 0) return;
    threads = std::max(1, std::min<int>(threads, int((n + 4095) / 4096)));
    if (threads == 1) { f(size_t(0), n, 0); return; }
    std::vector<std::thread> th;
    const size_t chunk = (n + threads - 1) / threads;
    for (int t = 0; t < threads; ++t) {
        const size_t b = size_t(t) * chunk, e = std::min(n, b + chunk);
        if (b >= e) break;
        th.emplace_back([=, &f] { f(b, e, t); });
    }
    for (auto& x : th) x.join();
}

// Whole-file import with the reference's outcome: the file is read once; line boundaries,
// record count, validation, base codes and the Bloom hashes of every record are computed in
// parallel; only the Bloom filter pass runs in input order (it decides which of two duplicates
// survives), touching a few bits per record with the bits of the next records prefetched.
int import_fasta_parallel(const char* path, int read_len, int bloom_m, int n_hashfunc, uint8_t** reads_out,
                          pq_index_type* num_reads_out, pq_index_type* removed_out, const char** err) {
    char msg[512];
    const int fd = open(path, O_RDONLY);
    if (fd < 0) {
        snprintf(msg, sizeof msg, "open reads file %s failed.\n", path);
        g_import_err = msg;
        if (err) *err = g_import_err.c_str();
        return PQ_ERR_ARG;
    }
    struct stat stt;
    if (fstat(fd, &stt) != 0 || !S_ISREG(stt.st_mode)) {   // not a regular file: read line by line
        close(fd);
        return -1;
    }
    const int threads = std::max(1, int(std::thread::hardware_concurrency()));
    const size_t nbytes = size_t(stt.st_size);
    std::unique_ptr<char, decltype(&free)> text((char*)malloc(nbytes ? nbytes : 1), &free);
    if (!text) { close(fd); return -1; }
    bool read_ok = true;
    std::mutex read_mu;
    parallel_ranges(nbytes, threads, [&](size_t b, size_t e, int) {
        size_t at = b;
        while (at < e) {
            const ssize_t got = pread(fd, text.get() + at, e - at, off_t(at));
            if (got <= 0) {
                std::lock_guard<std::mutex> g(read_mu);
                read_ok = false;
                return;
            }
            at += size_t(got);
        }
    });
    close(fd);
    if (!read_ok) return -1;
    const char* T = text.get();
    // lines: per chunk count of newlines and NUL bytes, then the line starts
    std::vector<size_t> nl_count(threads + 1, 0), nul_count(threads + 1, 0);
    parallel_ranges(nbytes, threads, [&](size_t b, size_t e, int t) {
        size_t c = 0;
        for (const char* q = T + b; (q = (const char*)memchr(q, '\n', size_t(T + e - q))) != nullptr; ++q) ++c;
        nl_count[t] = c;
        nul_count[t] = memchr(T + b, 0, e - b) != nullptr;
    });
    size_t nuls = 0, nls = 0;
    for (int t = 0; t <= threads; ++t) { nuls += nul_count[t]; nls += nl_count[t]; }
    const bool last_open = nbytes && T[nbytes - 1] != '\n';
    const size_t nlines = nls + (last_open ? 1 : 0);
    if (nuls) return -1;
    std::unique_ptr<size_t[]> start(new size_t[nlines + 1]);
    {
        std::vector<size_t> base(threads + 1, 0);
        for (int t = 0; t < threads; ++t) base[t + 1] = base[t] + nl_count[t];
        if (nlines) start[0] = 0;
        parallel_ranges(nbytes, threads, [&](size_t b, size_t e, int t) {
            size_t k = base[t];
            for (const char* q = T + b; (q = (const char*)memchr(q, '\n', size_t(T + e - q))) != nullptr; ++q)
                if (k + 1 <= nlines) start[++k] = size_t(q - T) + 1;
        });
        start[nlines] = nbytes + (last_open ? 1 : 0);   // one past the (virtual) newline
    }
    // line i: bytes [start[i], start[i+1] - 1) without its newline
    auto line_len = [&](size_t i) { return start[i + 1] - 1 - start[i]; };
    std::vector<size_t> hdr_count(threads + 1, 0), long_count(threads + 1, 0);
    parallel_ranges(nlines, threads, [&](size_t b, size_t e, int t) {
        size_t h = 0, lg = 0;
        for (size_t i = b; i < e; ++i) {
            h += line_len(i) > 0 && T[start[i]] == '>';
            lg += line_len(i) >= 999;
        }
        hdr_count[t] = h;
        long_count[t] = lg;
    });
    pq_index_type records = 0;
    size_t longs = 0;
    for (int t = 0; t <= threads; ++t) { records += pq_index_type(hdr_count[t]); longs += long_count[t]; }
    if (longs) return -1;
    // record i: header line 2i, sequence line 2i + 1; status 0 = ok, 1 = has N, 2 = error
    const size_t pairs = (nlines + 1) / 2;
    const pq_index_type m = records * (pq_index_type)bloom_m;
    const int nf = std::max(0, std::min(n_hashfunc, 5));
    // not zero-filled: each worker touches (and page-faults) only its own records
    std::unique_ptr<uint8_t[]> status(new uint8_t[pairs ? pairs : 1]);
    std::unique_ptr<pq_index_type[]> hfw(new pq_index_type[pairs * size_t(nf) + 1]);
    std::unique_ptr<pq_index_type[]> hrc(new pq_index_type[pairs * size_t(nf) + 1]);
    // the sequence line of record i (valid records only)
    const size_t* __restrict__ const st = start.get();
    auto seq_of = [st, T](size_t i) { return T + st[2 * i + 1]; };
    auto classify = [&, st, T](auto nf_tag) {
        constexpr int NF = decltype(nf_tag)::value;
        parallel_ranges(pairs, threads, [&, st, T](size_t b, size_t e, int) {
            const int RL = read_len;
            const size_t NL = nlines;
            const bool open_end = last_open;
            const pq_index_type M = m;
            uint8_t* __restrict__ const sta = status.get();
            pq_index_type* __restrict__ const hf = hfw.get();
            pq_index_type* __restrict__ const hr = hrc.get();
            for (size_t i = b; i < e; ++i) {
                const size_t h = 2 * i, q = h + 1;
                const size_t hlen = st[h + 1] - 1 - st[h];
                if (hlen == 0 || T[st[h]] != '>' || q >= NL) { sta[i] = 2; continue; }
                // the reference drops the last character of the buffer: the newline, or the last
                // base of a final line without one
                const size_t slen = (st[q + 1] - 1 - st[q]) + (q + 1 == NL && open_end ? 0 : 1) - 1;
                if (slen != size_t(RL)) { sta[i] = 2; continue; }
                const unsigned cls = hash_line<NF>((const unsigned char*)(T + st[q]), RL, M, hf + i * NF, hr + i * NF);
                // a byte that is no base and no N: error; an N: dropped before the filter
                sta[i] = (cls & 4u) ? 2 : ((cls & 2u) ? 1 : 0);
            }
        });
    };
    switch (nf) {
        case 0: classify(std::integral_constant<int, 0>{}); break;
        case 1: classify(std::integral_constant<int, 1>{}); break;
        case 2: classify(std::integral_constant<int, 2>{}); break;
        case 3: classify(std::integral_constant<int, 3>{}); break;
        case 4: classify(std::integral_constant<int, 4>{}); break;
        default: classify(std::integral_constant<int, 5>{}); break;
    }
    // the Bloom pass in input order (src/bloom.c:91-135), up to the first bad record
    const size_t nbits_bytes = (size_t(m) + 7) / 8 + 1;
    std::unique_ptr<unsigned char, decltype(&free)> bits_mem((unsigned char*)alloc_huge(nbits_bytes), &free);
    if (!bits_mem) return PQ_ERR_NOMEM;
    unsigned char* const bits = bits_mem.get();
    memset(bits, 0, nbits_bytes);
    std::vector<uint8_t> keep(pairs, 0);
    pq_index_type kept = 0, removed = 0;
    constexpr size_t kAhead = 16;
    for (size_t i = 0; i < pairs; ++i) {
        if (i + kAhead < pairs && status[i + kAhead] == 0) {
            for (int f = 0; f < nf; ++f) {
                __builtin_prefetch(&bits[hfw[(i + kAhead) * nf + f] / 8]);
                __builtin_prefetch(&bits[hrc[(i + kAhead) * nf + f] / 8]);
            }
        }
        if (status[i] == 2) {
            snprintf(msg, sizeof msg, "incorrect reads file at line %llu.\n", (unsigned long long)(kept * 2 + 2));
            g_import_err = msg;
            if (err) *err = g_import_err.c_str();
            return PQ_ERR_ARG;
        }
        if (status[i] == 1) { removed++; continue; }
        const pq_index_type* hv = &hfw[i * nf];
        bool all = true;
        for (int f = 0; f < nf; ++f)
            if (!bit_get(bits, hv[f])) all = false;
        bool dup = true;
        if (!all) {
            for (int f = 0; f < nf; ++f) {
                if (!bit_get(bits, hrc[i * nf + f])) {
                    for (int j = 0; j < nf; ++j) bit_set(bits, hv[j]);
                    dup = false;
                    break;
                }
            }
        }
        if (dup) { removed++; continue; }
        keep[i] = 1;
        kept++;
    }
    // kept reads in input order
    std::vector<size_t> kc(threads + 1, 0);
    parallel_ranges(pairs, threads, [&](size_t b, size_t e, int t) {
        size_t c = 0;
        for (size_t i = b; i < e; ++i) c += keep[i];
        kc[t] = c;
    });
    std::vector<size_t> kb(threads + 1, 0);
    for (int t = 0; t < threads; ++t) kb[t + 1] = kb[t] + kc[t];
    const size_t out_bytes = size_t(kept) * size_t(read_len);
    uint8_t* buf = (uint8_t*)alloc_huge(out_bytes ? out_bytes : 1);
    if (!buf) return PQ_ERR_NOMEM;
    parallel_ranges(pairs, threads, [&](size_t b, size_t e, int t) {
        const int RL = read_len;
        uint8_t* __restrict__ o = buf + kb[t] * size_t(RL);
        for (size_t i = b; i < e; ++i) {
            if (!keep[i]) continue;
            const unsigned char* sq = (const unsigned char*)seq_of(i);   // all bases (kept)
            for (int j = 0; j < RL; ++j) o[j] = kBases.fw[sq[j]];
            o += RL;
        }
    });
    *reads_out = buf;
    *num_reads_out = kept;
    if (removed_out) *removed_out = removed;
    return PQ_OK;
}

}  // namespace

extern "C" {

int pq_import_fasta(const char* path, int read_len, int bloom_m, int n_hashfunc, uint8_t** reads_out,
                    pq_index_type* num_reads_out, pq_index_type* removed_out, const char** err) {
    // the CLI's own argument checks (src/test.c:300-320), which run before the reference imports
    const char* bad = nullptr;
    char msg[160];
    if (read_len <= 0 || read_len > 65535) {
        snprintf(msg, sizeof msg, "invalid read length (%d), valid range (0, 65535].\n", read_len);
        bad = msg;
    } else if (n_hashfunc < 1 || n_hashfunc > 5) {
        snprintf(msg, sizeof msg, "invalid number of hash functions (%d), valid range [1, MAX_FUNC].\n", n_hashfunc);
        bad = msg;
    } else if (bloom_m < 1) {
        bad = "length of bloom filter array must be larger than 1.\n";
    }
    if (bad || !path || !reads_out || !num_reads_out) {
        g_import_err = bad ? bad : "invalid argument.\n";
        if (err) *err = g_import_err.c_str();
        return PQ_ERR_ARG;
    }
    const int rc = import_fasta_parallel(path, read_len, bloom_m, n_hashfunc, reads_out, num_reads_out, removed_out,
                                         err);
    if (rc >= 0) return rc;
    return import_fasta_serial(path, read_len, bloom_m, n_hashfunc, reads_out, num_reads_out, removed_out, err);
}

pq_index_t* construct_index(char* single_file, char* pair_file1, char* pair_file2, char* mate_file1,
                            char* mate_file2, int min_overlap, int read_len, int bloom_m, int n_hashfunc) {
    pq_index_t* ix = (pq_index_t*)calloc(1, sizeof(pq_index_t));
    if (!ix) error_exit("out of memory.\n");
    ix->min_overlap = (uint16_t)min_overlap;
    ix->read_len = (uint16_t)read_len;
    ix->bloom_size = (pq_index_type)bloom_m;
    ix->n_hashfunc = n_hashfunc;

    if (single_file) {
        double t0 = now_ms();
        printf("Importing reads from %s ... ", single_file);
        fflush(stdout);
        uint8_t* reads = nullptr;
        pq_index_type nr = 0, removed = 0;
        const char* err = nullptr;
        int rc = pq_import_fasta(single_file, read_len, bloom_m, n_hashfunc, &reads, &nr, &removed, &err);
        if (rc) error_exit(err ? err : "import failed.\n");
        ix->reads = (char*)reads;
        ix->num_reads = nr;
        ix->bloom_size = nr + removed == 0 ? 0 : (nr + removed) * (pq_index_type)bloom_m;
        printf("done\n");
        printf("  has imported %llu reads (removed %llu duplicate reads)\n", (unsigned long long)nr,
               (unsigned long long)removed);
        time_importreads = now_ms() - t0;
        printf("  takes %.3lf ms\n", time_importreads);
        fflush(stdout);
    } else if (pair_file1 && pair_file2) {
        error_exit("We do not support paired end reads.\nPlease input them as single reads.\n");
    } else if (mate_file1 && mate_file2) {
        error_exit("We do not support mate pair reads.\nPlease input them as single reads.\n");
    }

    pq_ctx* ctx = nullptr;
    if (pq_create(&ctx, 0, nullptr) != PQ_OK) error_exit("no usable CUDA device.\n");
    auto ck = [&](int rc) {
        if (rc != PQ_OK) {
            std::string m = std::string(pq_last_error(ctx)) + "\n";
            error_exit(m.c_str());
        }
    };
    ck(pq_set_reads(ctx, (const uint8_t*)ix->reads, ix->num_reads, read_len, min_overlap, 0));
    ck(pq_get_counts(ctx, ix->C, ix->suffix_count, ix->prefix_count));
    const size_t nr = ix->num_reads, n = nr * size_t(read_len), rowlen = n / 64 + 1;
    for (int dir = 0; dir < 2; ++dir) {
        double t0 = now_ms();
        printf(dir ? "Sorting backward suffixes ... " : "Sorting forward suffixes ... ");
        fflush(stdout);
        ck(pq_sort_for_index(ctx, dir));
        ck(pq_build_fm(ctx, dir));
        std::vector<uint64_t> bm(rowlen * 5);
        pq_index_type* sample = (pq_index_type*)malloc(rowlen * 5 * sizeof(pq_index_type));
        pq_index_type* ri = (pq_index_type*)malloc((nr ? nr : 1) * sizeof(pq_index_type));
        pq_index_type* ss = (pq_index_type*)malloc((nr ? nr : 1) * sizeof(pq_index_type));
        pq_index_type* sz = (pq_index_type*)malloc((nr ? nr : 1) * sizeof(pq_index_type));
        uint16_t* sd = (uint16_t*)malloc((nr ? nr : 1) * sizeof(uint16_t));
        if (!sample || !ri || !ss || !sz || !sd) error_exit("out of memory.\n");
        ck(pq_get_index_ref(ctx, dir, bm.data(), sample, ri));
        ck(pq_get_sort_seeds(ctx, dir, ss, sz, sd));
        uint64_t** dst = dir ? ix->OCC_bitmap_bw : ix->OCC_bitmap;
        for (int c = 0; c < 5; ++c) {
            dst[c] = (uint64_t*)malloc(rowlen * sizeof(uint64_t));
            if (!dst[c]) error_exit("out of memory.\n");
            memcpy(dst[c], bm.data() + size_t(c) * rowlen, rowlen * sizeof(uint64_t));
        }
        // sort-slot sizes (src/sufsort.c:386-450): 5 slots of 17 first-prefix ranks
        pq_index_type* size = dir ? ix->size_bw : ix->size_fw;
        pq_index_type* off = dir ? ix->offset_bw : ix->offset_fw;
        pq_index_type mx = 0;
        pq_slots::slot_sizes<pq_index_type>((const uint8_t*)ix->reads, nr, read_len, dir, size, off, &mx,
                                            int(std::max(1u, std::thread::hardware_concurrency())));
        if (dir) {
            ix->OCC_sample_bw = sample;
            ix->reads_index_bw = ri;
            ix->interval_start_bw = ss;
            ix->interval_end_bw = sz;
            ix->interval_depth_bw = sd;
            ix->max_size_bw = mx;
        } else {
            ix->OCC_sample = sample;
            ix->reads_index = ri;
            ix->interval_start = ss;
            ix->interval_end = sz;
            ix->interval_depth = sd;
            ix->max_size_fw = mx;
        }
        printf("done\n");
        printf("  takes %.3lf ms\n", now_ms() - t0);
        fflush(stdout);
    }
    {
        std::lock_guard<std::mutex> g(g_mu);
        auto it = g_ctx.find(ix);
        if (it != g_ctx.end()) pq_destroy(it->second);
        g_ctx[ix] = ctx;
    }
    return ix;
}

pq_string_graph_t* construct_string_graph(pq_index_t* ix) {
    double t0 = now_ms();
    printf("Building overlap graph ... ");
    fflush(stdout);
    pq_ctx* ctx = nullptr;
    {
        std::lock_guard<std::mutex> g(g_mu);
        auto it = g_ctx.find(ix);
        if (it != g_ctx.end()) {
            ctx = it->second;
            g_ctx.erase(it);
        }
    }
    auto ck = [&](int rc) {
        if (rc != PQ_OK) {
            if (rc == PQ_ERR_TOO_MANY_EDGES) error_exit("assembly failed. Try a larger min overlap length.\n");
            std::string m = std::string(pq_last_error(ctx)) + "\n";
            error_exit(m.c_str());
        }
    };
    if (!ctx) {   // index built elsewhere: rebuild the device index from its reads
        if (pq_create(&ctx, 0, nullptr) != PQ_OK) error_exit("no usable CUDA device.\n");
        ck(pq_set_reads(ctx, (const uint8_t*)ix->reads, ix->num_reads, ix->read_len, ix->min_overlap, 0));
        ck(pq_build_index(ctx));
    }
    ck(pq_overlaps(ctx));
    uint64_t ne = 0;
    ck(pq_get_graph_sizes(ctx, &ne, nullptr, nullptr));
    const size_t nr = ix->num_reads;
    // uninitialised host arrays: pq_get_graph writes every entry
    std::unique_ptr<uint16_t[]> nB(new uint16_t[nr + 1]), nF(new uint16_t[nr + 1]), len(new uint16_t[ne + 1]);
    std::unique_ptr<int32_t[]> oB(new int32_t[nr + 1]), oF(new int32_t[nr + 1]), trans(new int32_t[ne + 1]);
    std::unique_ptr<uint64_t[]> off(new uint64_t[nr + 1]);
    std::unique_ptr<pq_index_type[]> dest(new pq_index_type[ne + 1]);
    std::unique_ptr<uint8_t[]> type(new uint8_t[ne + 1]);
    ck(pq_get_graph(ctx, nB.get(), nF.get(), oB.get(), oF.get(), off.get(), dest.get(), len.get(), type.get(),
                    trans.get()));
    pq_destroy(ctx);
    pq_string_graph_t* g = pq_string_graph_from_csr(ix->num_reads, ix->read_len, ix->min_overlap, nB.get(), nF.get(),
                                                    oB.get(), oF.get(), off.get(), dest.get(), len.get(), type.get(),
                                                    trans.get(), 0);
    if (!g) error_exit("out of memory.\n");
    printf("  takes %.3lf ms\n", now_ms() - t0);
    printf("  average overlap length: %lf\n", g->average_overlap);
    fflush(stdout);
    return g;
}

// Frees what pq_string_graph_from_csr allocated for the nodes [0, n).
static void free_nodes(pq_node_t* nodes, size_t n) {
    for (size_t i = 0; i < n; ++i) {
        free(nodes[i].edges);
        if (nodes[i].path_q) free(nodes[i].path_q->path);
        free(nodes[i].path_q);
    }
}

pq_string_graph_t* pq_string_graph_from_csr(pq_index_type num_reads, int read_len, int min_overlap,
                                            const uint16_t* num_B, const uint16_t* num_F, const int32_t* olp_B,
                                            const int32_t* olp_F, const uint64_t* edge_off, const pq_index_type* dest,
                                            const uint16_t* len, const uint8_t* type, const int32_t* trans,
                                            int threads) {
    const size_t nr = num_reads;
    if (read_len <= 0 || read_len > 65535 || min_overlap < 0 || min_overlap > 65535) return nullptr;
    if (nr && (!num_B || !num_F || !olp_B || !olp_F || !edge_off)) return nullptr;
    if (nr && edge_off[nr] && (!dest || !len || !type || !trans)) return nullptr;
    pq_string_graph_t* g = (pq_string_graph_t*)malloc(sizeof(pq_string_graph_t));
    if (!g) return nullptr;
    g->nodes = (pq_node_t*)calloc(nr ? nr : 1, sizeof(pq_node_t));
    if (!g->nodes) {
        free(g);
        return nullptr;
    }
    g->num_reads = num_reads;
    g->read_len = (uint16_t)read_len;
    g->min_overlap = (uint16_t)min_overlap;
    if (threads <= 0) threads = std::max(1, int(std::thread::hardware_concurrency()));
    threads = std::max(1, std::min<int>(threads, int((nr + 4095) / 4096)));
    const size_t chunk = nr ? (nr + threads - 1) / threads : 0;

    // The running maximum of trans in read order (I_F[1].uu / I_B[1].uu of one reference thread):
    // each range's own maximum first, then every range starts from the maximum of those before it.
    std::vector<pq_index_type> mx_B(threads, 0), mx_F(threads, 0);
    std::vector<uint64_t> olen(threads, 0), cnt(threads, 0);   // integer sums: exact, any order
    std::vector<char> oom(threads, 0);
    auto run = [&](auto&& body) {
        if (threads == 1) {
            body(0);
            return;
        }
        std::vector<std::thread> th;
        for (int t = 0; t < threads; ++t) th.emplace_back([&, t] { body(t); });
        for (auto& x : th) x.join();
    };
    run([&](int t) {
        const size_t b = std::min(nr, size_t(t) * chunk), e = std::min(nr, b + chunk);
        pq_index_type mB = 0, mF = 0;
        for (size_t i = b; i < e; ++i) {
            const uint64_t e0 = edge_off[i];
            for (int j = 0; j < num_B[i]; ++j) mB = std::max(mB, (pq_index_type)trans[e0 + j]);
            for (int j = 0; j < num_F[i]; ++j) mF = std::max(mF, (pq_index_type)trans[e0 + num_B[i] + j]);
        }
        mx_B[t] = mB;
        mx_F[t] = mF;
    });
    {   // exclusive prefix maximum over the ranges
        pq_index_type pB = 0, pF = 0;
        for (int t = 0; t < threads; ++t) {
            const pq_index_type rB = mx_B[t], rF = mx_F[t];
            mx_B[t] = pB;
            mx_F[t] = pF;
            pB = std::max(pB, rB);
            pF = std::max(pF, rF);
        }
    }
    const char ONE = 1, BRANCH = 2, ENDING = 4, REMOVED = 8, SUSPECT = 4, NONE = 0;
    const char BB = 3, FB = 1;
    run([&](int t) {
        const size_t b = std::min(nr, size_t(t) * chunk), e = std::min(nr, b + chunk);
        pq_index_type run_max_B = mx_B[t], run_max_F = mx_F[t];
        uint64_t sum_len = 0, sum_cnt = 0;
        for (size_t i = b; i < e; ++i) {
            pq_node_t* nd = &g->nodes[i];
            const int nb = num_B[i], nf = num_F[i];
            const uint64_t e0 = edge_off[i];
            for (int j = 0; j < nb; ++j) run_max_B = std::max(run_max_B, (pq_index_type)trans[e0 + j]);
            for (int j = 0; j < nf; ++j) run_max_F = std::max(run_max_F, (pq_index_type)trans[e0 + nb + j]);
            nd->max_B = nd->num_B = (uint16_t)nb;
            nd->max_F = nd->num_F = (uint16_t)nf;
            nd->status = 0;
            nd->path_q = nullptr;
            nd->edges = (pq_edge_t*)malloc((size_t(nb) + nf) * sizeof(pq_edge_t));
            if (!nd->edges && nb + nf) {
                oom[t] = 1;
                return;
            }
            const int ob = olp_B[i], of = olp_F[i];
            const int mo = std::max(ob, of);
            const double ratio = mo == 0 ? 0 : ((double)abs(ob - of)) / mo;
            nd->marked = ratio > 0.6 ? SUSPECT : 0;
            if (nb || nf) {
                nd->B_type = nb == 1 ? ONE : (nb > 1 ? BRANCH : ENDING);
                nd->F_type = nf == 1 ? ONE : (nf > 1 ? BRANCH : ENDING);
            } else {
                nd->B_type = nd->F_type = ENDING;
                nd->status = REMOVED;
            }
            for (int j = 0; j < nb + nf; ++j) {
                nd->edges[j].dest = dest[e0 + j];
                nd->edges[j].overlap_len = len[e0 + j];
                nd->edges[j].type = (char)type[e0 + j];
                sum_len += len[e0 + j];
            }
            if ((nd->B_type == BRANCH && nd->F_type != ENDING) || (nd->F_type == BRANCH && nd->B_type != ENDING)) {
                pq_path_q_t* q = (pq_path_q_t*)malloc(sizeof(pq_path_q_t));
                pq_path_t* path = (pq_path_t*)malloc(sizeof(pq_path_t) * (size_t(nb) + nf));
                if (!q || !path) {
                    free(q);
                    free(path);
                    oom[t] = 1;
                    return;
                }
                q->max_B_endlen = q->max_F_endlen = q->max_B_len = q->max_F_len = 0;
                q->path = path;
                q->max_F_trans = (int)run_max_F;
                q->max_B_trans = (int)run_max_B;
                for (int j = 0; j < nb + nf; ++j) {
                    pq_path_t* p = &path[j];
                    const pq_edge_t* ed = &nd->edges[j];
                    p->end = ed->dest;
                    p->hop = ed->dest;
                    p->len = 1;
                    p->end_len = (uint16_t)(read_len - ed->overlap_len);
                    p->bubble_len = 0;
                    p->type = NONE;
                    p->updated = 0;
                    p->direction = j < nb ? (ed->type == BB ? 1 : 0) : (ed->type == FB ? 1 : 0);
                    p->trans = trans[e0 + j];
                }
                nd->path_q = q;
            }
            sum_cnt += uint64_t(nb + nf);
        }
        olen[t] = sum_len;
        cnt[t] = sum_cnt;
    });
    double overlap_len = 0;
    pq_index_type overlaps = 0;
    for (int t = 0; t < threads; ++t) {
        if (oom[t]) {
            free_nodes(g->nodes, nr);
            free(g->nodes);
            free(g);
            return nullptr;
        }
        overlap_len += (double)olen[t];
        overlaps += (pq_index_type)cnt[t];
    }
    g->average_overlap = overlap_len / overlaps;
    return g;
}

void destroy_graph(pq_string_graph_t* graph) { (void)graph; }

}  // extern "C"
