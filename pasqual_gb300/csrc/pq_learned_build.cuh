// pq_learned_build.cuh — host entry points of the learned-index build (pq_learned.cu).
#pragma once
#include "pq_learned.cuh"

namespace pq {

// Working memory of one build: row keys, tile offsets, distinct keys (kd), their group starts
// (fd, with fd[m] = n) and the segment starts in key order (dsi).
struct LxTmp {
    uint32_t* keys;
    unsigned long long* toff;
    uint32_t* kd;
    idx_t* fd;
    unsigned long long* dsi;
    size_t ntiles;
};
size_t lx_tmp_bytes(size_t n);
LxTmp lx_tmp_layout(void* tmp, size_t n);

// key16 of every row, then the distinct keys and group starts; *num_keys on return (synchronises)
cudaError_t lx_distinct_keys(const idx_t* sa, const uint64_t* pk, size_t n, idx_t L, const LxTmp& t,
                             unsigned long long* num_keys, cudaStream_t st);
// root: S segments of equal key count (bnd[S], base[S + 1], segof[65537]; dsi in t)
cudaError_t lx_root(const LxTmp& t, unsigned long long m, size_t n, int S, uint32_t* bnd, idx_t* base,
                    uint16_t* segof, cudaStream_t st);
// per-segment MLP training (par[S * kLxStride])
cudaError_t lx_train(const LxTmp& t, const uint32_t* bnd, const idx_t* base, int S, int steps, float lr, uint32_t seed,
                     float* par, cudaStream_t st);
// per-segment window bounds of the trained model (err) and of the root alone (err_root), 2 S each
cudaError_t lx_errors(const LxTmp& t, const LearnedView& v, int32_t* err, int32_t* err_root, cudaStream_t st);
// predictions (and segments) of arbitrary keys with the search's own function
cudaError_t lx_predict_keys(const LearnedView& v, const uint32_t* keys, size_t n, long long* pred, int32_t* seg,
                            cudaStream_t st);

// The network of one segment on its own (parameters as one kLxStride record): forward of n
// inputs, and the gradient of sum_i dy_i * y_i with respect to the 193 parameters.
cudaError_t mlp_forward(const float* par, const float* x, int n, float* y, cudaStream_t st);
cudaError_t mlp_backward(const float* par, const float* x, const float* dy, int n, float* grad, cudaStream_t st);
// one training step of one network: Adam on the mean squared error of (x, tgt) (t = step number)
cudaError_t mlp_adam_step(float* par, float* m1, float* m2, const float* x, const float* tgt, int n, int t, float lr,
                          cudaStream_t st);

}  // namespace pq
