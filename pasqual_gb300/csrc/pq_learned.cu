// pq_learned.cu — build of the learned index of pq_learned.cuh from a suffix array just built.
//
//   1. row keys      key16 of every SA row (SA entry, then 32 bits of packed text)
//   2. distinct keys one pass in tiles of 4096 rows: group starts F (rows where the key changes)
//   3. segments      S = min(1024, #keys) segments of equal key count; root = (bnd, base)
//   4. training      one CTA per segment: Adam on the MLP with this file's forward and backward
//   5. max errors    every present key predicted with the search's own function; per segment the
//                    largest (pred - F(K)) and (F(K + 1) - pred)
//
// Training.  The hidden layer starts as 64 ReLU knots spread evenly over the segment
// (w1 = 1, b1 = -(j + 0.5) / 64) and stays there; the output layer (w2, b2) is trained.  The
// output weights are updated in knot-value coordinates -- v_j = network value at knot j, so that
// w2 = D v and b2 = v_0 with D the fixed second-difference map of the knots -- because Adam on
// w2 directly stalls: the 64 ramp features overlap and their Gram matrix is badly conditioned.
// The gradient with respect to v is the chain rule through D applied to the backward kernel's
// gradient with respect to w2 and b2.  Targets are the centre of each key's row group, relative
// to the root and divided by their RMS over a sample (folded back into w2 and b2 at the end).
// Everything runs in FP32 and in a fixed order, so a build is reproducible.
#include "pq_learned.cuh"
#include "pq_learned_build.cuh"

namespace pq {

static inline unsigned grid_cap(size_t work, int threads) {
    size_t g = (work + threads - 1) / threads;
    const size_t cap = size_t(152) * 32;
    if (g > cap) g = cap;
    if (g < 1) g = 1;
    return unsigned(g);
}

constexpr int kTileRows = 4096;      // 256 threads x 16 rows
constexpr int kTrainThreads = 256;   // samples per training step
constexpr float kJointLr = 1e-3f;    // learning rate of the joint phase (all parameters)

// ---------------------------------------------------------------------------------- keys

__global__ void k_lx_row_keys(const idx_t* __restrict__ sa, const uint64_t* __restrict__ pk, size_t n, idx_t L,
                              uint32_t* __restrict__ keys) {
    const size_t stride = size_t(gridDim.x) * blockDim.x;
    for (size_t r = size_t(blockIdx.x) * blockDim.x + threadIdx.x; r < n; r += stride) {
        const idx_t p = sa[r];
        const int m = int(L - p % L);
        const size_t w = size_t(p) >> 5;
        const int s = int(p & 31) * 2;
        const uint64_t a = __ldg(pk + w), b = __ldg(pk + w + 1);
        const uint64_t x = s ? ((a << s) | (b >> (64 - s))) : a;
        uint32_t key = uint32_t(x >> 32);
        if (m < kLxKeyBases) key &= ~(0xffffffffu >> (2 * m));
        keys[r] = key;
    }
}

__device__ __forceinline__ bool is_head(const uint32_t* __restrict__ keys, size_t n, size_t r) {
    return r < n && (r == 0 || keys[r] != keys[r - 1]);
}

__global__ void __launch_bounds__(256) k_lx_tile_count(const uint32_t* __restrict__ keys, size_t n,
                                                      unsigned long long* __restrict__ tcnt) {
    __shared__ unsigned red[8];
    const size_t r0 = size_t(blockIdx.x) * kTileRows + size_t(threadIdx.x) * 16;
    unsigned c = 0;
    for (int j = 0; j < 16; ++j) c += is_head(keys, n, r0 + j) ? 1u : 0u;
    for (int o = 16; o > 0; o >>= 1) c += __shfl_down_sync(0xffffffffu, c, o);
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = c;
    __syncthreads();
    if (threadIdx.x == 0) {
        unsigned t = 0;
        for (int w = 0; w < 8; ++w) t += red[w];
        tcnt[blockIdx.x] = t;
    }
}

// exclusive prefix of tcnt[0, m) in place, total in tcnt[m]; one CTA of 1024 threads
__global__ void __launch_bounds__(1024) k_lx_tile_scan(unsigned long long* __restrict__ tcnt, size_t m) {
    __shared__ unsigned long long part[1024];
    const size_t per = (m + 1023) / 1024;
    const size_t a = size_t(threadIdx.x) * per, b = a + per < m ? a + per : m;
    unsigned long long s = 0;
    for (size_t i = a; i < b; ++i) s += tcnt[i];
    part[threadIdx.x] = s;
    __syncthreads();
    for (int o = 1; o < 1024; o <<= 1) {
        const unsigned long long v = threadIdx.x >= unsigned(o) ? part[threadIdx.x - o] : 0;
        __syncthreads();
        part[threadIdx.x] += v;
        __syncthreads();
    }
    unsigned long long run = part[threadIdx.x] - s;
    for (size_t i = a; i < b; ++i) {
        const unsigned long long v = tcnt[i];
        tcnt[i] = run;
        run += v;
    }
    if (threadIdx.x == 1023) tcnt[m] = part[1023];
}

__global__ void __launch_bounds__(256) k_lx_tile_write(const uint32_t* __restrict__ keys, size_t n,
                                                      const unsigned long long* __restrict__ toff,
                                                      uint32_t* __restrict__ kd, idx_t* __restrict__ fd) {
    __shared__ unsigned wsum[8];
    const size_t r0 = size_t(blockIdx.x) * kTileRows + size_t(threadIdx.x) * 16;
    unsigned flags = 0;
    for (int j = 0; j < 16; ++j) flags |= is_head(keys, n, r0 + j) ? (1u << j) : 0u;
    const unsigned c = __popc(flags);
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    unsigned x = c;
    for (int o = 1; o < 32; o <<= 1) {
        const unsigned y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= o) x += y;
    }
    if (lane == 31) wsum[w] = x;
    __syncthreads();
    unsigned before = 0;
    for (int i = 0; i < w; ++i) before += wsum[i];
    unsigned long long off = toff[blockIdx.x] + before + (x - c);
    while (flags) {
        const int j = __ffs(flags) - 1;
        flags &= flags - 1;
        kd[off] = keys[r0 + j];
        fd[off] = idx_t(r0 + j);
        ++off;
    }
}

// ---------------------------------------------------------------------------------- root

__global__ void k_lx_segments(const uint32_t* __restrict__ kd, idx_t* __restrict__ fd, unsigned long long m,
                              size_t n, int S, uint32_t* __restrict__ bnd, idx_t* __restrict__ base,
                              unsigned long long* __restrict__ dsi) {
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s < S) {
        const unsigned long long ds = (unsigned long long)s * m / unsigned(S);
        bnd[s] = s ? kd[ds] : 0u;
        base[s] = s ? fd[ds] : idx_t(0);
        dsi[s] = ds;
    }
    if (s == 0) {
        base[S] = idx_t(n);
        dsi[S] = m;
        fd[m] = idx_t(n);
    }
}

__global__ void k_lx_segof(const uint32_t* __restrict__ bnd, int S, uint16_t* __restrict__ segof) {
    const int h = blockIdx.x * blockDim.x + threadIdx.x;
    if (h > 65536) return;
    if (h == 65536) { segof[h] = uint16_t(S - 1); return; }
    const uint32_t key = uint32_t(h) << 16;
    int a = 0, b = S - 1;
    while (a < b) {
        const int mid = (a + b + 1) >> 1;
        if (bnd[mid] <= key) a = mid;
        else b = mid - 1;
    }
    segof[h] = uint16_t(a);
}

// ---------------------------------------------------------------------------------- MLP

// forward of one sample with the parameters in shared memory (same operation order as lx_mlp)
__device__ __forceinline__ float mlp_forward_smem(const float* w1, const float* b1, const float* w2, float b2,
                                                  float x) {
    float y = b2;
    #pragma unroll 8
    for (int j = 0; j < kLxHidden; ++j) y = fmaf(w2[j], fmaxf(fmaf(w1[j], x, b1[j]), 0.f), y);
    return y;
}

// Backward of a batch of nb <= 256 samples (x, dy) in shared memory, run by 256 threads:
// adds d/dw1, d/db1, d/dw2 (64 each) and d/db2 of sum_i dy_i * y_i into acc[0..192].  Thread
// (j = tid % 64, part = tid / 64) sums samples part, part + 4, ...; parts are added in order.
__device__ __forceinline__ void mlp_backward_block(const float* w1, const float* b1, const float* w2,
                                                   const float* sx, const float* sg, int nb, float* acc,
                                                   float (*part)[3][kLxHidden], float* red) {
    const int tid = threadIdx.x, j = tid & (kLxHidden - 1), pi = tid >> 6;
    float gw1 = 0.f, gb1 = 0.f, gw2 = 0.f;
    for (int i = pi; i < nb; i += 4) {
        const float x = sx[i], g = sg[i];
        const float a = fmaf(w1[j], x, b1[j]);
        if (a > 0.f) {
            gw2 = fmaf(g, a, gw2);
            const float dz = g * w2[j];
            gw1 = fmaf(dz, x, gw1);
            gb1 += dz;
        }
    }
    part[pi][0][j] = gw1;
    part[pi][1][j] = gb1;
    part[pi][2][j] = gw2;
    float gb = tid < nb ? sg[tid] : 0.f;
    for (int o = 16; o > 0; o >>= 1) gb += __shfl_down_sync(0xffffffffu, gb, o);
    if ((tid & 31) == 0) red[tid >> 5] = gb;
    __syncthreads();
    if (tid < kLxHidden) {
        acc[tid] += ((part[0][0][tid] + part[1][0][tid]) + part[2][0][tid]) + part[3][0][tid];
        acc[kLxHidden + tid] += ((part[0][1][tid] + part[1][1][tid]) + part[2][1][tid]) + part[3][1][tid];
        acc[2 * kLxHidden + tid] += ((part[0][2][tid] + part[1][2][tid]) + part[2][2][tid]) + part[3][2][tid];
    }
    if (tid == 0) {
        float s = 0.f;
        for (int w = 0; w < 8; ++w) s += red[w];
        acc[3 * kLxHidden] += s;
    }
    __syncthreads();
}

// One Adam step (beta1 0.9, beta2 0.999, eps 1e-8) of the block on k parameters p with gradient g;
// p1 = 0.9^t and p2 = 0.999^t for this step t (bias correction).
__device__ __forceinline__ void adam_params(float* p, float* m1, float* m2, const float* g, int k, float lr, float p1,
                                            float p2) {
    for (int i = threadIdx.x; i < k; i += blockDim.x) {
        const float gi = g[i];
        m1[i] = 0.9f * m1[i] + 0.1f * gi;
        m2[i] = 0.999f * m2[i] + 0.001f * gi * gi;
        const float mh = m1[i] / (1.f - p1), vh = m2[i] / (1.f - p2);
        p[i] -= lr * mh / (sqrtf(vh) + 1e-8f);
    }
}

// Mean squared error of the network (parameters P in shared memory) on batches of 256 samples
// (x, target): sg = d loss / d y of every sample, and the gradient of the loss in acc[0..192].
__device__ __forceinline__ void mse_gradient(const float* P, const float* x, const float* tgt, int n, float* sx,
                                             float* sg, float* acc, float (*part)[3][kLxHidden], float* red) {
    const int tid = threadIdx.x;
    if (tid < kLxParams) acc[tid] = 0.f;
    __syncthreads();
    for (int c = 0; c < n; c += 256) {
        const int nb = n - c < 256 ? n - c : 256;
        if (tid < nb) {
            const float xi = x[c + tid];
            const float y = mlp_forward_smem(P, P + kLxHidden, P + 2 * kLxHidden, P[3 * kLxHidden], xi);
            sx[tid] = xi;
            sg[tid] = 2.f * (y - tgt[c + tid]) / float(n);
        }
        __syncthreads();
        mlp_backward_block(P, P + kLxHidden, P + 2 * kLxHidden, sx, sg, nb, acc, part, red);
    }
}

// One training step of one network on its own (the step the joint phase of k_lx_train takes):
// gradient of the mean squared error on (x, target), then Adam on all 193 parameters; par
// (one kLxStride record), m1, m2 (193 each) are read and written; t is the 1-based step number.
__global__ void __launch_bounds__(256) k_mlp_adam_step(float* __restrict__ par, float* __restrict__ m1g,
                                                      float* __restrict__ m2g, const float* __restrict__ x,
                                                      const float* __restrict__ tgt, int n, int t, float lr) {
    __shared__ float P[kLxParams], m1[kLxParams], m2[kLxParams], acc[kLxParams];
    __shared__ float sx[256], sg[256];
    __shared__ float part[4][3][kLxHidden];
    __shared__ float red[8];
    const int tid = threadIdx.x;
    if (tid < kLxParams) {
        P[tid] = par[tid];
        m1[tid] = m1g[tid];
        m2[tid] = m2g[tid];
    }
    __syncthreads();
    mse_gradient(P, x, tgt, n, sx, sg, acc, part, red);
    adam_params(P, m1, m2, acc, kLxParams, lr, powf(0.9f, float(t)), powf(0.999f, float(t)));
    __syncthreads();
    if (tid < kLxParams) {
        par[tid] = P[tid];
        m1g[tid] = m1[tid];
        m2g[tid] = m2[tid];
    }
}

__global__ void k_mlp_forward(const float* __restrict__ par, const float* __restrict__ x, int n,
                              float* __restrict__ y) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) y[i] = lx_mlp(par, x[i]);
}

__global__ void __launch_bounds__(256) k_mlp_backward(const float* __restrict__ par, const float* __restrict__ x,
                                                     const float* __restrict__ dy, int n, float* __restrict__ grad) {
    __shared__ float w1[kLxHidden], b1[kLxHidden], w2[kLxHidden];
    __shared__ float sx[256], sg[256], acc[kLxParams];
    __shared__ float part[4][3][kLxHidden];
    __shared__ float red[8];
    const int tid = threadIdx.x;
    if (tid < kLxHidden) {
        w1[tid] = par[tid];
        b1[tid] = par[kLxHidden + tid];
        w2[tid] = par[2 * kLxHidden + tid];
    }
    if (tid < kLxParams) acc[tid] = 0.f;
    __syncthreads();
    for (int c = 0; c < n; c += 256) {
        const int nb = n - c < 256 ? n - c : 256;
        if (tid < nb) {
            sx[tid] = x[c + tid];
            sg[tid] = dy[c + tid];
        }
        __syncthreads();
        mlp_backward_block(w1, b1, w2, sx, sg, nb, acc, part, red);
    }
    if (tid < kLxParams) grad[tid] = acc[tid];
}

// ---------------------------------------------------------------------------------- training

__device__ __forceinline__ uint32_t mix32(uint32_t x) {      // integer hash (xorshift-multiply)
    x ^= x >> 16;
    x *= 0x7feb352du;
    x ^= x >> 15;
    x *= 0x846ca68bu;
    x ^= x >> 16;
    return x;
}

struct SegData {
    const uint32_t* kd;
    const idx_t* fd;
    uint32_t b0;
    double span;
    double base;
    double R;
    __device__ __forceinline__ float x_of(unsigned long long i) const { return float(double(kd[i] - b0) / span); }
    // centre of key i's row group relative to the root, in units of the segment's rows
    __device__ __forceinline__ float target(unsigned long long i, float x) const {
        const double c = 0.5 * (double(fd[i]) + double(fd[i + 1])) - base;
        return float(c / R) - x;
    }
};

__global__ void __launch_bounds__(kTrainThreads) k_lx_train(const uint32_t* __restrict__ kd, const idx_t* __restrict__ fd,
                                                           const unsigned long long* __restrict__ dsi,
                                                           const uint32_t* __restrict__ bnd,
                                                           const idx_t* __restrict__ base, int S, int steps, float lr,
                                                           uint32_t seed, float* __restrict__ par) {
    constexpr int H = kLxHidden;
    __shared__ float w1[H], b1[H], w2[H], v[H + 1], m1[H + 1], m2[H + 1], hk[H];
    __shared__ float sx[kTrainThreads], sg[kTrainThreads], acc[kLxParams];
    __shared__ float part[4][3][H];
    __shared__ float red[8];
    __shared__ float s_b2, s_sigma;
    __shared__ float jp[kLxParams], jq[kLxParams], jm1[kLxParams], jm2[kLxParams];
    __shared__ float ex[kTrainThreads], et[kTrainThreads];
    __shared__ float s_loss0, s_loss1;
    const int s = blockIdx.x, tid = threadIdx.x;
    const unsigned long long ds = dsi[s], cnt = dsi[s + 1] - ds;
    SegData sd;
    sd.kd = kd;
    sd.fd = fd;
    sd.b0 = bnd[s];
    sd.span = (s + 1 < S ? double(bnd[s + 1]) : 4294967296.0) - double(sd.b0);
    sd.base = double(base[s]);
    sd.R = double(base[s + 1] - base[s]);
    if (sd.R <= 0.0) sd.R = 1.0;
    if (tid < H) {
        w1[tid] = 1.f;
        b1[tid] = -(float(tid) + 0.5f) / float(H);
        // knot spacing: c_{j+1} - c_j, with c_H = 1
        hk[tid] = tid + 1 < H ? 1.f / float(H) : 1.f - (float(H) - 0.5f) / float(H);
        w2[tid] = 0.f;
    }
    if (tid <= H) {
        v[tid] = 0.f;
        m1[tid] = 0.f;
        m2[tid] = 0.f;
    }
    if (tid == 0) s_b2 = 0.f;
    // target scale: RMS of the root's residual over an even sample of the segment's keys
    {
        float q = 0.f;
        if (cnt) {
            const unsigned long long i = ds + (unsigned long long)tid * cnt / kTrainThreads;
            const float x = sd.x_of(i);
            const float r = sd.target(i, x);
            q = r * r;
        }
        for (int o = 16; o > 0; o >>= 1) q += __shfl_down_sync(0xffffffffu, q, o);
        if ((tid & 31) == 0) red[tid >> 5] = q;
        __syncthreads();
        if (tid == 0) {
            float t = 0.f;
            for (int w = 0; w < 8; ++w) t += red[w];
            const float rms = sqrtf(t / kTrainThreads);
            s_sigma = rms > 0.f ? rms : 1.f;
        }
        __syncthreads();
    }
    const float inv_sigma = 1.f / s_sigma;
    const float beta1 = 0.9f, beta2 = 0.999f, eps = 1e-8f;
    float p1 = 1.f, p2 = 1.f;
    for (int step = 0; step < steps && cnt; ++step) {
        // forward and loss gradient of one random batch
        const unsigned long long i = ds + mix32(seed ^ mix32(uint32_t(s) * 0x9e3779b9u + uint32_t(step) * 0x85ebca6bu + uint32_t(tid))) % cnt;
        const float x = sd.x_of(i);
        const float tgt = sd.target(i, x) * inv_sigma;
        const float y = mlp_forward_smem(w1, b1, w2, s_b2, x);
        sx[tid] = x;
        sg[tid] = 2.f * (y - tgt) / float(kTrainThreads);
        if (tid < kLxParams) acc[tid] = 0.f;
        __syncthreads();
        mlp_backward_block(w1, b1, w2, sx, sg, kTrainThreads, acc, part, red);
        // chain rule into knot values: w2_j = s_j - s_{j-1}, s_j = (v_{j+1} - v_j) / hk_j, b2 = v_0
        p1 *= beta1;
        p2 *= beta2;
        if (tid <= H) {
            const int k = tid;
            auto gs = [&](int j) { return acc[2 * H + j] - (j + 1 < H ? acc[2 * H + j + 1] : 0.f); };   // dL/ds_j
            float g = 0.f;
            if (k >= 1) g += gs(k - 1) / hk[k - 1];
            if (k < H) g -= gs(k) / hk[k];
            if (k == 0) g += acc[3 * H];
            m1[k] = beta1 * m1[k] + (1.f - beta1) * g;
            m2[k] = beta2 * m2[k] + (1.f - beta2) * g * g;
            const float mh = m1[k] / (1.f - p1), vh = m2[k] / (1.f - p2);
            const float lr_t = lr * (1.f - float(step) / float(steps));
            v[k] -= lr_t * mh / (sqrtf(vh) + eps);
        }
        __syncthreads();
        if (tid < H) {
            const float sj = (v[tid + 1] - v[tid]) / hk[tid];
            const float sp = tid ? (v[tid] - v[tid - 1]) / hk[tid - 1] : 0.f;
            w2[tid] = sj - sp;
        }
        if (tid == 0) s_b2 = v[0];
        __syncthreads();
    }
    // Joint phase: every parameter (knot slopes and offsets w1, b1 as well as w2, b2) by Adam on the
    // same loss, from the knot-value solution; kept only if it lowers the squared error on an even
    // sample of the segment's keys.
    if (tid < H) {
        jp[tid] = w1[tid];
        jp[H + tid] = b1[tid];
        jp[2 * H + tid] = w2[tid];
    }
    if (tid == 0) jp[3 * H] = s_b2;
    if (tid < kLxParams) {
        jq[tid] = 0.f;
        jm1[tid] = 0.f;
        jm2[tid] = 0.f;
    }
    if (cnt) {
        const unsigned long long i = ds + ((unsigned long long)tid * cnt + cnt / 2) / kTrainThreads;
        ex[tid] = sd.x_of(i);
        et[tid] = sd.target(i, ex[tid]) * inv_sigma;
    }
    __syncthreads();
    auto sample_loss = [&](float* out_loss) {
        float q = 0.f;
        if (cnt) {
            const float y = mlp_forward_smem(jp, jp + H, jp + 2 * H, jp[3 * H], ex[tid]);
            q = (y - et[tid]) * (y - et[tid]);
        }
        for (int o = 16; o > 0; o >>= 1) q += __shfl_down_sync(0xffffffffu, q, o);
        if ((tid & 31) == 0) red[tid >> 5] = q;
        __syncthreads();
        if (tid == 0) {
            float t = 0.f;
            for (int w = 0; w < 8; ++w) t += red[w];
            *out_loss = t;
        }
        __syncthreads();
    };
    sample_loss(&s_loss0);
    if (tid < kLxParams) jq[tid] = jp[tid];
    const int steps2 = steps / 2;
    float q1 = 1.f, q2 = 1.f;
    for (int step = 0; step < steps2 && cnt; ++step) {
        const unsigned long long i = ds + mix32(~seed ^ mix32(uint32_t(s) * 0x2545f491u + uint32_t(step) * 0x9e3779b9u + uint32_t(tid))) % cnt;
        const float x = sd.x_of(i);
        sx[tid] = x;
        const float y = mlp_forward_smem(jp, jp + H, jp + 2 * H, jp[3 * H], x);
        sg[tid] = 2.f * (y - sd.target(i, x) * inv_sigma) / float(kTrainThreads);
        if (tid < kLxParams) acc[tid] = 0.f;
        __syncthreads();
        mlp_backward_block(jp, jp + H, jp + 2 * H, sx, sg, kTrainThreads, acc, part, red);
        q1 *= 0.9f;
        q2 *= 0.999f;
        adam_params(jp, jm1, jm2, acc, kLxParams, kJointLr * (1.f - float(step) / float(steps2)), q1, q2);
        __syncthreads();
    }
    sample_loss(&s_loss1);
    if (!(s_loss1 < s_loss0) && tid < kLxParams) jp[tid] = jq[tid];     // keep the knot-value solution
    __syncthreads();
    float* out = par + size_t(s) * kLxStride;
    if (tid < H) {
        out[tid] = jp[tid];
        out[H + tid] = jp[H + tid];
        out[2 * H + tid] = jp[2 * H + tid] * s_sigma;
    }
    if (tid == 0) out[3 * H] = jp[3 * H] * s_sigma;
    if (tid >= kLxParams && tid < kLxStride) out[tid] = 0.f;
}

// ---------------------------------------------------------------------------------- errors

__global__ void __launch_bounds__(256) k_lx_errors(const uint32_t* __restrict__ kd, const idx_t* __restrict__ fd,
                                                  const unsigned long long* __restrict__ dsi, LearnedView v,
                                                  int32_t* __restrict__ err, int32_t* __restrict__ err_root) {
    __shared__ long long red[4][8];
    const int s = blockIdx.x, tid = threadIdx.x;
    const unsigned long long a = dsi[s], b = dsi[s + 1];
    long long e[4] = {0, 0, 0, 0};      // trained lo, hi; root lo, hi
    for (unsigned long long i = a + tid; i < b; i += blockDim.x) {
        const uint32_t K = kd[i];
        const long long f0 = (long long)fd[i], f1 = (long long)fd[i + 1];
        const long long p = lx_predict(v, s, K, true), q = lx_predict(v, s, K, false);
        e[0] = max(e[0], p - f0);
        e[1] = max(e[1], f1 - p);
        e[2] = max(e[2], q - f0);
        e[3] = max(e[3], f1 - q);
    }
    #pragma unroll
    for (int c = 0; c < 4; ++c) {
        long long x = e[c];
        for (int o = 16; o > 0; o >>= 1) x = max(x, __shfl_down_sync(0xffffffffu, x, o));
        if ((tid & 31) == 0) red[c][tid >> 5] = x;
    }
    __syncthreads();
    if (tid < 4) {
        long long x = 0;
        for (int w = 0; w < 8; ++w) x = max(x, red[tid][w]);
        if (x > 0x7fffffffLL) x = 0x7fffffffLL;
        int32_t* dst = tid < 2 ? err : err_root;
        dst[2 * s + (tid & 1)] = int32_t(x);
    }
}

__global__ void k_lx_predict(LearnedView v, const uint32_t* __restrict__ keys, size_t n, long long* __restrict__ pred,
                             int32_t* __restrict__ seg) {
    const size_t i = size_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const int s = lx_segment(v, keys[i]);
    pred[i] = lx_predict(v, s, keys[i], true);
    seg[i] = s;
}

// ---------------------------------------------------------------------------------- host

// sizes of the working arrays, in layout order; each starts on a 256-byte boundary
static void lx_tmp_parts(size_t n, size_t (&bytes)[5], size_t& ntiles) {
    ntiles = (n + kTileRows - 1) / kTileRows;
    bytes[0] = 4 * n;                          // row keys
    bytes[1] = 8 * (ntiles + 1);               // tile offsets
    bytes[2] = 4 * n;                          // distinct keys
    bytes[3] = sizeof(idx_t) * (n + 1);        // group starts
    bytes[4] = 8 * (kLxMaxSegs + 1);           // segment starts in key order
}

static size_t round256(size_t b) { return (b + 255) & ~size_t(255); }

size_t lx_tmp_bytes(size_t n) {
    size_t b[5], nt;
    lx_tmp_parts(n, b, nt);
    size_t total = 0;
    for (size_t x : b) total += round256(x);
    return total;
}

LxTmp lx_tmp_layout(void* tmp, size_t n) {
    size_t b[5], nt;
    lx_tmp_parts(n, b, nt);
    char* p = static_cast<char*>(tmp);
    char* q[5];
    for (int i = 0; i < 5; ++i) {
        q[i] = p;
        p += round256(b[i]);
    }
    LxTmp t;
    t.keys = reinterpret_cast<uint32_t*>(q[0]);
    t.toff = reinterpret_cast<unsigned long long*>(q[1]);
    t.kd = reinterpret_cast<uint32_t*>(q[2]);
    t.fd = reinterpret_cast<idx_t*>(q[3]);
    t.dsi = reinterpret_cast<unsigned long long*>(q[4]);
    t.ntiles = nt;
    return t;
}

cudaError_t lx_distinct_keys(const idx_t* sa, const uint64_t* pk, size_t n, idx_t L, const LxTmp& t,
                             unsigned long long* num_keys, cudaStream_t st) {
    *num_keys = 0;
    if (!n) return cudaSuccess;
    { k_lx_row_keys<<<grid_cap(n, 256), 256, 0, st>>>(sa, pk, n, L, t.keys); note_launch(); }
    { k_lx_tile_count<<<unsigned(t.ntiles), 256, 0, st>>>(t.keys, n, t.toff); note_launch(); }
    { k_lx_tile_scan<<<1, 1024, 0, st>>>(t.toff, t.ntiles); note_launch(); }
    { k_lx_tile_write<<<unsigned(t.ntiles), 256, 0, st>>>(t.keys, n, t.toff, t.kd, t.fd); note_launch(); }
    cudaError_t e = cudaMemcpyAsync(num_keys, t.toff + t.ntiles, sizeof(unsigned long long), cudaMemcpyDeviceToHost, st);
    if (e != cudaSuccess) return e;
    e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) return e;
    return cudaGetLastError();
}

cudaError_t lx_root(const LxTmp& t, unsigned long long m, size_t n, int S, uint32_t* bnd, idx_t* base,
                    uint16_t* segof, cudaStream_t st) {
    { k_lx_segments<<<(S + 255) / 256, 256, 0, st>>>(t.kd, t.fd, m, n, S, bnd, base, t.dsi); note_launch(); }
    { k_lx_segof<<<(65537 + 255) / 256, 256, 0, st>>>(bnd, S, segof); note_launch(); }
    return cudaGetLastError();
}

cudaError_t lx_train(const LxTmp& t, const uint32_t* bnd, const idx_t* base, int S, int steps, float lr, uint32_t seed,
                     float* par, cudaStream_t st) {
    { k_lx_train<<<S, kTrainThreads, 0, st>>>(t.kd, t.fd, t.dsi, bnd, base, S, steps, lr, seed, par); note_launch(); }
    return cudaGetLastError();
}

cudaError_t lx_errors(const LxTmp& t, const LearnedView& v, int32_t* err, int32_t* err_root, cudaStream_t st) {
    { k_lx_errors<<<v.segs, 256, 0, st>>>(t.kd, t.fd, t.dsi, v, err, err_root); note_launch(); }
    return cudaGetLastError();
}

cudaError_t lx_predict_keys(const LearnedView& v, const uint32_t* keys, size_t n, long long* pred, int32_t* seg,
                            cudaStream_t st) {
    if (n) { k_lx_predict<<<unsigned((n + 255) / 256), 256, 0, st>>>(v, keys, n, pred, seg); note_launch(); }
    return cudaGetLastError();
}

cudaError_t mlp_forward(const float* par, const float* x, int n, float* y, cudaStream_t st) {
    if (n > 0) { k_mlp_forward<<<(n + 255) / 256, 256, 0, st>>>(par, x, n, y); note_launch(); }
    return cudaGetLastError();
}

cudaError_t mlp_backward(const float* par, const float* x, const float* dy, int n, float* grad, cudaStream_t st) {
    { k_mlp_backward<<<1, 256, 0, st>>>(par, x, dy, n, grad); note_launch(); }
    return cudaGetLastError();
}

cudaError_t mlp_adam_step(float* par, float* m1, float* m2, const float* x, const float* tgt, int n, int t, float lr,
                          cudaStream_t st) {
    { k_mlp_adam_step<<<1, 256, 0, st>>>(par, m1, m2, x, tgt, n, t, lr); note_launch(); }
    return cudaGetLastError();
}

}  // namespace pq
