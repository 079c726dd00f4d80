// pq_learned.cuh — learned index over a suffix array: 2-bit-packed 16-base key -> SA rank.
//
// Keys.  Row r of a suffix array gets key16(r) = the first 16 bases of its suffix, 2 bits a base
// (A=0 .. T=3, first base in the top bits), bases past the end of the read set to 0.  Padding with
// the smallest code keeps key16 non-decreasing in r, and for a pattern P of t >= 16 bases with
// first 16 bases K every row whose suffix starts with P lies in the key group
// [F(K), F(K + 1)), F(K) = number of rows with key16 < K.
//
// Model.  The distinct keys present are cut into S <= 1024 segments of equal key count.  The root
// maps a key of segment s linearly from the segment's key range onto its row range
// [base[s], base[s + 1]) (piecewise linear over the whole key space); a per-segment 2-layer MLP
// (1 -> 64 ReLU -> 1, FP32) adds a correction in units of the segment's row range:
//
//     x = (K - bnd[s]) / (bnd[s + 1] - bnd[s]),   pred = base[s] + (x + mlp_s(x)) * (base[s+1] - base[s]).
//
// Every present key's whole group lies in [pred - e_lo[s], pred + e_hi[s]); the two per-segment
// int32 bounds are measured over all present keys after training with this same prediction
// function.  A query searches that window exactly (binary search on the suffix array and the
// packed text) and checks the rows just outside it; a key that is absent, or a window that does
// not hold the answer, is a miss and the search falls back to the plain backward search.
#pragma once
#include "pq_common.cuh"

namespace pq {

constexpr int kLxMaxSegs = 1024;
constexpr int kLxHidden = 64;
constexpr int kLxParams = 3 * kLxHidden + 1;     // w1[64] b1[64] w2[64] b2
constexpr int kLxStride = 196;                    // floats per segment (49 float4)
constexpr int kLxKeyBases = 16;

__device__ __forceinline__ float lx_mlp(const float* __restrict__ p, float x) {
    const float4* q = reinterpret_cast<const float4*>(p);
    float y = __ldg(p + 3 * kLxHidden);
    #pragma unroll 4
    for (int j4 = 0; j4 < kLxHidden / 4; ++j4) {
        const float4 w1 = __ldg(q + j4), b1 = __ldg(q + kLxHidden / 4 + j4), w2 = __ldg(q + kLxHidden / 2 + j4);
        y = fmaf(w2.x, fmaxf(fmaf(w1.x, x, b1.x), 0.f), y);
        y = fmaf(w2.y, fmaxf(fmaf(w1.y, x, b1.y), 0.f), y);
        y = fmaf(w2.z, fmaxf(fmaf(w1.z, x, b1.z), 0.f), y);
        y = fmaf(w2.w, fmaxf(fmaf(w1.w, x, b1.w), 0.f), y);
    }
    return y;
}

__device__ __forceinline__ double lx_key_span(const LearnedView& v, int s) {
    const double hi = s + 1 < v.segs ? double(__ldg(v.bnd + s + 1)) : 4294967296.0;
    return hi - double(__ldg(v.bnd + s));
}

// segment of key K: the last s with bnd[s] <= K
__device__ __forceinline__ int lx_segment(const LearnedView& v, uint32_t K) {
    const uint32_t h = K >> 16;
    int a = __ldg(v.segof + h), b = __ldg(v.segof + h + 1);     // answer in [a, b]
    while (a < b) {
        const int m = (a + b + 1) >> 1;
        if (__ldg(v.bnd + m) <= K) a = m;
        else b = m - 1;
    }
    return a;
}

// predicted row of key K in segment s; with_mlp = false gives the root alone
__device__ __forceinline__ long long lx_predict(const LearnedView& v, int s, uint32_t K, bool with_mlp = true) {
    const float x = float(double(K - __ldg(v.bnd + s)) / lx_key_span(v, s));
    float r = x;
    if (with_mlp) r += lx_mlp(v.par + size_t(s) * kLxStride, x);
    const idx_t b0 = __ldg(v.base + s), b1 = __ldg(v.base + s + 1);
    const float R = float(b1 - b0);
    float o = r * R;
    o = fminf(fmaxf(o, 0.f), R);
    const long long p = (long long)b0 + __float2ll_rd(o);
    return p < (long long)b1 ? p : (long long)b1;
}

}  // namespace pq
