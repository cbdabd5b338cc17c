// Shared device code for the bonded-DEM kernels: 3-vector math, the contact
// transport of the rate law, block reductions and a time-limited grid barrier.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "dpf_gb300.h"

namespace dpf {

constexpr int kThreads = 256;
// cos(0.25) rounded to double, the threshold of the reference transport guard.
constexpr double kCosQuarter = 0.9689124217106447;
// Grid barriers give up after this many nanoseconds and report
// DPF_ERR_BARRIER_TIMEOUT instead of waiting forever.
constexpr unsigned long long kBarrierTimeoutNs = 1000000000ull;

struct d3 {
    double x, y, z;
};

__device__ __forceinline__ d3 mk(double a, double b, double c) { return {a, b, c}; }
__device__ __forceinline__ d3 operator+(d3 a, d3 b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
__device__ __forceinline__ d3 operator-(d3 a, d3 b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
__device__ __forceinline__ d3 operator-(d3 a) { return {-a.x, -a.y, -a.z}; }
__device__ __forceinline__ d3 operator*(double s, d3 a) { return {s * a.x, s * a.y, s * a.z}; }
// One reciprocal and three products: a float64 division costs many times a
// multiply on GB300's float64 pipe.
__device__ __forceinline__ d3 operator/(d3 a, double s) {
    const double inv = 1.0 / s;
    return {a.x * inv, a.y * inv, a.z * inv};
}
__device__ __forceinline__ double dot(d3 a, d3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
__device__ __forceinline__ d3 cross(d3 a, d3 b) {
    return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x};
}
__device__ __forceinline__ double norm(d3 a) { return sqrt(dot(a, a)); }

__device__ __forceinline__ d3 ld3(const double *p) { return {p[0], p[1], p[2]}; }
__device__ __forceinline__ d3 ld3(const double *p, int64_t i) { return ld3(p + 3 * i); }
__device__ __forceinline__ void st3(double *p, d3 v) { p[0] = v.x; p[1] = v.y; p[2] = v.z; }
__device__ __forceinline__ void st3(double *p, int64_t i, d3 v) { st3(p + 3 * i, v); }

__device__ __forceinline__ void edge(const int64_t *edges, int64_t b, int64_t &i, int64_t &j) {
    const longlong2 e = reinterpret_cast<const longlong2 *>(edges)[b];
    i = e.x;
    j = e.y;
}

// Rotation that carries vectors from a bond frame with normal n0 to one with
// normal n1 (shortest arc) and then spins them about n1 by spin . bisector:
// the `transport` of experiments/bonded_dem_finite_gpu.py:22-32.
struct Transport {
    d3 k, n1;
    double inv1pc, c, s;
};

__device__ __forceinline__ Transport make_transport(d3 n0, d3 n1, d3 spin, int &flags) {
    Transport t;
    t.k = cross(n0, n1);
    const double cosine = fmin(fmax(dot(n0, n1), -1.0), 1.0);
    if (cosine < kCosQuarter) flags |= DPF_ERR_NORMAL_TURN;
    t.inv1pc = 1.0 / (1.0 + cosine);
    d3 b = n0 + n1;
    b = b / fmax(norm(b), 1e-12);
    sincos(dot(spin, b), &t.s, &t.c);
    t.n1 = n1;
    return t;
}

__device__ __forceinline__ d3 apply(const Transport &t, d3 v) {
    const d3 kv = cross(t.k, v);
    d3 out = v + kv;
    out = out + t.inv1pc * cross(t.k, kv);
    return t.c * out + t.s * cross(t.n1, out) + ((1.0 - t.c) * dot(t.n1, out)) * t.n1;
}

// Sum over the incidences of site s of the bond wrenches [F, T_i, T_j]
// (nine doubles per bond; the j end receives (-F, T_j)), in incidence order.
__device__ __forceinline__ void gather_wrench(const int32_t *__restrict__ ptr, const int32_t *__restrict__ inc,
                                              const double *__restrict__ w, int64_t s, double acc[6]) {
#pragma unroll
    for (int c = 0; c < 6; ++c) acc[c] = 0.0;
    const int e1 = ptr[s + 1];
    for (int e = ptr[s]; e < e1; ++e) {
        const int v = inc[e];
        if (v >= 0) {
            const double *p = w + 9 * (int64_t)v;
#pragma unroll
            for (int c = 0; c < 6; ++c) acc[c] += p[c];
        } else {
            const double *p = w + 9 * (int64_t)(~v);
            acc[0] -= p[0];
            acc[1] -= p[1];
            acc[2] -= p[2];
            acc[3] += p[6];
            acc[4] += p[7];
            acc[5] += p[8];
        }
    }
}

// Inverse of a symmetric positive definite 6x6 matrix via Cholesky
// (A = L L^T, A^-1 = L^-T L^-1), fully unrolled into registers: every loop
// has a constant trip count so all indices fold.
__device__ __forceinline__ void spd_inverse6(const double A[36], double P[36]) {
    double L[36];
#pragma unroll
    for (int c = 0; c < 36; ++c) L[c] = 0.0;
#pragma unroll
    for (int jj = 0; jj < 6; ++jj) {
        double s = A[6 * jj + jj];
#pragma unroll
        for (int kk = 0; kk < 6; ++kk)
            if (kk < jj) s -= L[6 * jj + kk] * L[6 * jj + kk];
        const double ljj = sqrt(s);
        L[6 * jj + jj] = ljj;
        const double inv = 1.0 / ljj;
#pragma unroll
        for (int ii = 0; ii < 6; ++ii) {
            if (ii > jj) {
                double v = A[6 * ii + jj];
#pragma unroll
                for (int kk = 0; kk < 6; ++kk)
                    if (kk < jj) v -= L[6 * ii + kk] * L[6 * jj + kk];
                L[6 * ii + jj] = v * inv;
            }
        }
    }
    double W[36];  // W = L^-1 (lower triangular)
#pragma unroll
    for (int c = 0; c < 36; ++c) W[c] = 0.0;
#pragma unroll
    for (int ii = 0; ii < 6; ++ii) {
        W[6 * ii + ii] = 1.0 / L[6 * ii + ii];
#pragma unroll
        for (int jj = 0; jj < 6; ++jj) {
            if (jj < ii) {
                double v = 0.0;
#pragma unroll
                for (int kk = 0; kk < 6; ++kk)
                    if (kk >= jj && kk < ii) v += L[6 * ii + kk] * W[6 * kk + jj];
                W[6 * ii + jj] = -v * W[6 * ii + ii];
            }
        }
    }
#pragma unroll
    for (int ii = 0; ii < 6; ++ii)
#pragma unroll
        for (int jj = 0; jj < 6; ++jj) {
            if (jj <= ii) {
                double v = 0.0;
#pragma unroll
                for (int kk = 0; kk < 6; ++kk)
                    if (kk >= ii) v += W[6 * kk + ii] * W[6 * kk + jj];
                P[6 * ii + jj] = v;
                P[6 * jj + ii] = v;
            }
        }
}

// ---- reductions -----------------------------------------------------------

__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}
__device__ __forceinline__ double warp_max(double v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v = fmax(v, __shfl_xor_sync(0xffffffffu, v, o));
    return v;
}

// Block-wide sum (all threads get the result).  Fixed order: deterministic.
__device__ __forceinline__ double block_sum(double v) {
    __shared__ double buf[32];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    v = warp_sum(v);
    __syncthreads();
    if (lane == 0) buf[warp] = v;
    __syncthreads();
    const int nw = (blockDim.x + 31) >> 5;
    v = (threadIdx.x < nw) ? buf[threadIdx.x] : 0.0;
    if (warp == 0) v = warp_sum(v);
    if (threadIdx.x == 0) buf[0] = v;
    __syncthreads();
    v = buf[0];
    __syncthreads();
    return v;
}

__device__ __forceinline__ double block_max(double v) {
    __shared__ double buf[32];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    v = warp_max(v);
    __syncthreads();
    if (lane == 0) buf[warp] = v;
    __syncthreads();
    const int nw = (blockDim.x + 31) >> 5;
    v = (threadIdx.x < nw) ? buf[threadIdx.x] : -INFINITY;
    if (warp == 0) v = warp_max(v);
    if (threadIdx.x == 0) buf[0] = v;
    __syncthreads();
    v = buf[0];
    __syncthreads();
    return v;
}

// Sum of `count` values spaced `stride` apart, in a fixed order (every block
// that calls this with the same data gets the bit-identical result).
__device__ __forceinline__ double block_sum_array(const double *p, int count, int stride = 1) {
    double v = 0.0;
    for (int k = threadIdx.x; k < count; k += blockDim.x) v += p[(int64_t)k * stride];
    return block_sum(v);
}

__device__ __forceinline__ double block_max_array(const double *p, int count, int stride = 1) {
    double v = -INFINITY;
    for (int k = threadIdx.x; k < count; k += blockDim.x) v = fmax(v, p[(int64_t)k * stride]);
    return block_max(v);
}

// ---- sums as float32 pairs ---------------------------------------------------
// A float32 pair (hi, lo) carries a sum to about 48 bits with float32
// arithmetic only (TwoSum); float64 arithmetic is scarce on this part, and a
// block reduction of doubles costs every thread a float64 add per shuffle
// level.  TwoSum's error term is exact whatever the order of its operands,
// so an xor-shuffle tree leaves the same pair in every lane.

__device__ __forceinline__ void pair_add(float &hi, float &lo, float h, float l) {
    const float t = hi + h;
    const float hp = t - hi;
    lo += ((hi - (t - hp)) + (h - hp)) + l;
    hi = t;
}

__device__ __forceinline__ void warp_pair_sum(float &hi, float &lo) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        const float h = __shfl_xor_sync(0xffffffffu, hi, o), l = __shfl_xor_sync(0xffffffffu, lo, o);
        pair_add(hi, lo, h, l);
    }
}

// Block sum of per-thread pairs; every thread gets the total pair.
__device__ __forceinline__ float2 block_pair_sum(float hi, float lo) {
    __shared__ float2 buf[32];
    __shared__ float2 total;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    warp_pair_sum(hi, lo);
    __syncthreads();
    if (lane == 0) buf[warp] = make_float2(hi, lo);
    __syncthreads();
    if (warp == 0) {
        const int nw = (blockDim.x + 31) >> 5;
        float h = lane < nw ? buf[lane].x : 0.0f, l = lane < nw ? buf[lane].y : 0.0f;
        warp_pair_sum(h, l);
        if (lane == 0) total = make_float2(h, l);
    }
    __syncthreads();
    return total;
}

__device__ __forceinline__ float block_max_float(float v) {
    __shared__ float buf[32];
    __shared__ float total;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v = fmaxf(v, __shfl_xor_sync(0xffffffffu, v, o));
    __syncthreads();
    if (lane == 0) buf[warp] = v;
    __syncthreads();
    if (warp == 0) {
        const int nw = (blockDim.x + 31) >> 5;
        float m = lane < nw ? buf[lane] : -INFINITY;
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) m = fmaxf(m, __shfl_xor_sync(0xffffffffu, m, o));
        if (lane == 0) total = m;
    }
    __syncthreads();
    return total;
}

// The block's partial of a per-thread float32 value, as a pair, into part[blockIdx.x].
__device__ __forceinline__ void block_pair_partial(float v, float2 *part) {
    const float2 t = block_pair_sum(v, 0.0f);
    if (threadIdx.x == 0) part[blockIdx.x] = t;
}

// Sum of `count` block partial pairs, in float64, the same in every block
// (one warp adds them in a fixed order; the others wait at the block barrier).
__device__ __forceinline__ double pair_total(const float2 *part, int count) {
    __shared__ double total;
    __syncthreads();  // the previous total has been read
    if (threadIdx.x < 32) {
        float hi = 0.0f, lo = 0.0f;
        for (int k = threadIdx.x; k < count; k += 32) {
            const float2 p = part[k];
            pair_add(hi, lo, p.x, p.y);
        }
        warp_pair_sum(hi, lo);
        if (threadIdx.x == 0) total = (double)hi + (double)lo;
    }
    __syncthreads();
    return total;
}

// a / b formed by thread 0 and shared with the block: one float64 division
// per block instead of one per thread (float64 division is slow on this
// part).  Every thread of the block calls it, with the same a and b.
__device__ __forceinline__ double block_divide(double a, double b) {
    __shared__ double quotient;
    __syncthreads();  // the previous quotient has been read
    if (threadIdx.x == 0) quotient = a / b;
    __syncthreads();
    return quotient;
}

// "Last block finishes" protocol: every block has written its partial(s);
// returns true in exactly one block, after all partials are visible.  The
// counter lives in device memory, starts at zero and is reset by the last block.
__device__ __forceinline__ bool last_block(unsigned *counter) {
    __shared__ bool is_last;
    __threadfence();
    __syncthreads();
    if (threadIdx.x == 0) {
        const unsigned ticket = atomicAdd(counter, 1u);
        is_last = (ticket == gridDim.x - 1);
        if (is_last) *counter = 0u;
    }
    __syncthreads();
    if (is_last) __threadfence();
    return is_last;
}

// ---- grid barrier for cooperative (co-resident) launches --------------------

__device__ __forceinline__ unsigned ld_acquire(const unsigned *p) {
    unsigned v;
    asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}

__device__ __forceinline__ unsigned long long global_ns() {
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

// One atomic per block and barrier: block 0 adds 2^31 - (parties - 1), every
// other block 1, so the top bit of barrier[0] flips exactly when all parties
// have arrived (and the low bits return to where they were); a block waits
// until the bit differs from the value its own add returned.  Release add and
// acquire loads order the blocks' writes before and after the barrier.
// barrier[0] starts at 0 (the launching entry point clears it); barrier[1] is
// unused.  Returns false when the wait ran past timeout_ns (the status word
// then carries the error).  parties: arrivals that release the barrier (0 =
// every block of the grid).
__device__ __forceinline__ bool grid_barrier(unsigned *barrier, int *status,
                                             unsigned long long timeout_ns = kBarrierTimeoutNs,
                                             unsigned parties = 0) {
    __shared__ int ok;
    __syncthreads();
    if (threadIdx.x == 0) {
        ok = 1;
        const unsigned n = parties ? parties : gridDim.x;
        const unsigned add = blockIdx.x == 0 ? 0x80000000u - (n - 1) : 1u;
        unsigned old;
        asm volatile("atom.add.release.gpu.global.u32 %0, [%1], %2;" : "=r"(old) : "l"(barrier), "r"(add) : "memory");
        unsigned polls = 0;
        const unsigned long long t0 = global_ns();
        while (((ld_acquire(barrier) ^ old) & 0x80000000u) == 0) {
            if ((++polls & 63u) == 0 && global_ns() - t0 > timeout_ns) {
                atomicOr(status, DPF_ERR_BARRIER_TIMEOUT);
                ok = 0;
                break;
            }
        }
    }
    __syncthreads();
    return ok != 0;
}

}  // namespace dpf

#define DPF_CHECK_LAUNCH()                                   \
    do {                                                     \
        if (cudaGetLastError() != cudaSuccess) return DPF_ERR_CUDA; \
    } while (0)
