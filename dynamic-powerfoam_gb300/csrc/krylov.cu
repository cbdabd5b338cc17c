// Per-request Arnoldi for served batches: the building blocks of one FGMRES
// per request over a batch whose requests are contiguous site ranges
// (segments).  The basis vectors and the preconditioned directions are
// shared (N, 6) rows; every inner product, norm and coefficient is per
// segment, so each request follows its own Krylov recurrence
// (experiments/bonded_dem_newton.py:13-60 per request) while the operator
// and preconditioner launches cover all active requests at once.
//
// Reductions: each segment is cut into kChunks equal site ranges; one block
// per (chunk, segment) writes its partial sums, and a finishing kernel adds a
// segment's chunks in chunk order (deterministic, independent of the other
// segments).  Segments flagged inactive are skipped (their results are 0 and
// their rows are left untouched, or zeroed where stated).
#include "common.cuh"

namespace dpf {
namespace kry {

constexpr int kChunks = 16;
constexpr int kMaxBasis = 40;  // basis vectors per Arnoldi process (restart + 1 and then some)

struct Chunk {
    int64_t lo, hi;  // doubles
};

__device__ __forceinline__ Chunk chunk_of(const int64_t *seg_ptr, int r, int c) {
    const int64_t s0 = seg_ptr[r], s1 = seg_ptr[r + 1];
    const int64_t per = (s1 - s0 + kChunks - 1) / kChunks;
    const int64_t lo = s0 + c * per < s1 ? s0 + c * per : s1, hi = lo + per < s1 ? lo + per : s1;
    return Chunk{6 * lo, 6 * hi};
}

// partial[(r kChunks + c) count + k] = sum over the chunk of basis_k . w
__global__ void __launch_bounds__(kThreads) segment_dots_kernel(const int64_t *seg_ptr, const uint8_t *active,
                                                                const double *basis, int64_t ld, int count,
                                                                const double *w, double *partial) {
    const int r = blockIdx.y, c = blockIdx.x;
    if (active && !active[r]) return;
    const Chunk ch = chunk_of(seg_ptr, r, c);
    for (int k = 0; k < count; ++k) {
        const double *v = basis + (int64_t)k * ld;
        double t = 0.0;
        for (int64_t e = ch.lo + threadIdx.x; e < ch.hi; e += blockDim.x) t = fma(v[e], w[e], t);
        t = block_sum(t);
        if (threadIdx.x == 0) partial[((int64_t)r * kChunks + c) * count + k] = t;
    }
}

// out[r count + k] = sum of the segment's chunk partials (0 for inactive segments).
__global__ void segment_finish_kernel(int n_segments, const uint8_t *active, int count, const double *partial,
                                      double *out) {
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i >= (int64_t)n_segments * count) return;
    const int r = (int)(i / count), k = (int)(i % count);
    double t = 0.0;
    if (!active || active[r])
        for (int c = 0; c < kChunks; ++c) t += partial[((int64_t)r * kChunks + c) * count + k];
    out[i] = t;
}

// w -= sum_k h[seg, k] basis_k on active segments; partial |w|^2 per chunk.
__global__ void __launch_bounds__(kThreads) segment_project_kernel(const int64_t *seg_ptr, const uint8_t *active,
                                                                   const double *basis, int64_t ld, int count,
                                                                   const double *h, double *w, double *partial) {
    const int r = blockIdx.y, c = blockIdx.x;
    if (active && !active[r]) return;
    const Chunk ch = chunk_of(seg_ptr, r, c);
    __shared__ double coef[kMaxBasis];
    for (int k = threadIdx.x; k < count; k += blockDim.x) coef[k] = h[(int64_t)r * count + k];
    __syncthreads();
    double sq = 0.0;
    for (int64_t e = ch.lo + threadIdx.x; e < ch.hi; e += blockDim.x) {
        double proj = 0.0;
        for (int k = 0; k < count; ++k) proj = fma(basis[(int64_t)k * ld + e], coef[k], proj);
        const double v = w[e] - proj;
        w[e] = v;
        sq = fma(v, v, sq);
    }
    sq = block_sum(sq);
    if (threadIdx.x == 0) partial[(int64_t)r * kChunks + c] = sq;
}

// out = scale[seg] * a on active segments (inactive segments: 0).
__global__ void __launch_bounds__(kThreads) segment_scale_kernel(int64_t n, const int32_t *seg, const uint8_t *active,
                                                                 const double *scale, const double *a, double *out) {
    const int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (e >= 6 * n) return;
    const int r = seg[e / 6];
    out[e] = (!active || active[r]) ? scale[r] * a[e] : 0.0;
}

// x += sum_k y[seg, k] rows_k (y padded with zeros beyond each segment's length).
__global__ void __launch_bounds__(kThreads) segment_combine_kernel(int64_t n, const int32_t *seg, const double *rows,
                                                                   int64_t ld, int count, const double *y,
                                                                   double *x) {
    const int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (e >= 6 * n) return;
    const int r = seg[e / 6];
    double acc = 0.0;
    for (int k = 0; k < count; ++k) acc = fma(rows[(int64_t)k * ld + e], y[(int64_t)r * count + k], acc);
    x[e] += acc;
}

inline int blocks_for(int64_t n, int threads) { return (int)((n + threads - 1) / threads); }

}  // namespace kry
}  // namespace dpf

using namespace dpf;
using namespace dpf::kry;

extern "C" {

int64_t dpf_segment_krylov_partials_doubles(int n_segments, int count) {
    return n_segments <= 0 || count <= 0 ? 0 : (int64_t)n_segments * kChunks * (count > 1 ? count : 1);
}

int dpf_segment_dots(int n_segments, const int64_t *seg_ptr, const uint8_t *active, const double *basis, int64_t ld,
                     int count, const double *w, double *out, double *partials, void *stream) {
    if (n_segments <= 0 || n_segments > 65535 || !seg_ptr || !basis || !w || !out || !partials || count < 1 ||
        count > kMaxBasis || ld < 0)
        return DPF_ERR_ARGUMENT;
    cudaStream_t st = (cudaStream_t)stream;
    segment_dots_kernel<<<dim3(kChunks, n_segments), kThreads, 0, st>>>(seg_ptr, active, basis, ld, count, w,
                                                                          partials);
    segment_finish_kernel<<<blocks_for((int64_t)n_segments * count, 128), 128, 0, st>>>(n_segments, active, count,
                                                                                        partials, out);
    DPF_CHECK_LAUNCH();
    return DPF_OK;
}

int dpf_segment_project(int n_segments, const int64_t *seg_ptr, const uint8_t *active, const double *basis,
                        int64_t ld, int count, const double *h, double *w, double *norm2, double *partials,
                        void *stream) {
    if (n_segments <= 0 || n_segments > 65535 || !seg_ptr || !basis || !h || !w || !norm2 || !partials ||
        count < 1 || count > kMaxBasis || ld < 0)
        return DPF_ERR_ARGUMENT;
    cudaStream_t st = (cudaStream_t)stream;
    segment_project_kernel<<<dim3(kChunks, n_segments), kThreads, 0, st>>>(seg_ptr, active, basis, ld, count, h, w,
                                                                             partials);
    segment_finish_kernel<<<blocks_for(n_segments, 128), 128, 0, st>>>(n_segments, active, 1, partials, norm2);
    DPF_CHECK_LAUNCH();
    return DPF_OK;
}

int dpf_segment_scale(int64_t n_sites, const int32_t *seg, const uint8_t *active, const double *scale,
                      const double *a, double *out, void *stream) {
    if (n_sites <= 0 || !seg || !scale || !a || !out) return DPF_ERR_ARGUMENT;
    segment_scale_kernel<<<blocks_for(6 * n_sites, kThreads), kThreads, 0, (cudaStream_t)stream>>>(n_sites, seg, active,
                                                                                                   scale, a, out);
    DPF_CHECK_LAUNCH();
    return DPF_OK;
}

int dpf_segment_combine(int64_t n_sites, const int32_t *seg, const double *rows, int64_t ld, int count,
                        const double *y, double *x, void *stream) {
    if (n_sites <= 0 || !seg || !rows || !y || !x || count < 0 || count > kMaxBasis || ld < 0)
        return DPF_ERR_ARGUMENT;
    if (count == 0) return DPF_OK;
    segment_combine_kernel<<<blocks_for(6 * n_sites, kThreads), kThreads, 0, (cudaStream_t)stream>>>(
        n_sites, seg, rows, ld, count, y, x);
    DPF_CHECK_LAUNCH();
    return DPF_OK;
}

}  // extern "C"
