// Solver kernels of the Newton path (float64): the elastic block-Jacobi PCG
// as one cooperative launch, the FGMRES Arnoldi building blocks, reductions,
// the accepted-step update and the energy.
#include "common.cuh"

namespace dpf {

constexpr int kMaxReduceBlocks = 1024;
constexpr int64_t kPartialsOffset = 8;
constexpr int kMaxArnoldi = 64;
constexpr int kMaxPcgBlocks = 4096;

inline int blocks_for(int64_t n, int threads) { return (int)((n + threads - 1) / threads); }
inline int reduce_grid(int64_t n) {
    int g = blocks_for(n, kThreads);
    if (g > kMaxReduceBlocks) g = kMaxReduceBlocks;
    if (g < 1) g = 1;
    return g;
}

__device__ __forceinline__ unsigned *counter_slot(double *partials, int slot) {
    return reinterpret_cast<unsigned *>(partials) + slot;
}

__device__ __forceinline__ void matvec6(const double *P, const double x[6], double y[6]) {
#pragma unroll
    for (int row = 0; row < 6; ++row) {
        double v = 0.0;
#pragma unroll
        for (int c = 0; c < 6; ++c) v += P[6 * row + c] * x[c];
        y[row] = v;
    }
}

// ---------------------------------------------------------------------------
// Elastic PCG (experiments/bonded_dem_newton.py:107-130) in one cooperative
// launch.  Every block reduces the per-block partials in the same order, so
// all blocks take the same (deterministic) stopping decision without a flag.

struct PcgArgs {
    int64_t n, m;
    const int32_t *ptr, *inc;
    const int64_t *edges;
    dpf_stiffness k;
    dpf_tangent t;
    const double *mass, *block, *P, *units, *vector;
    const uint8_t *fixed;
    double alpha_op, tol2;
    int max_it;
    double *out;
    int *iterations;
    double *wrench, *x, *r, *z, *d, *ad, *part_a, *part_b;
    unsigned *barrier;
    int *status;
};

__global__ void __launch_bounds__(kThreads) pcg_kernel(PcgArgs a) {
    const int64_t tid = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    double p = 0.0;
    for (int64_t s = tid; s < a.n; s += stride) {
        double u[6], rr[6], zz[6];
#pragma unroll
        for (int c = 0; c < 6; ++c) u[c] = a.units[6 * s + c] * a.vector[6 * s + c];
        if (a.fixed[s]) {
#pragma unroll
            for (int c = 0; c < 6; ++c) rr[c] = 0.0;
        } else {
            matvec6(a.block + 36 * s, u, rr);
        }
        matvec6(a.P + 36 * s, rr, zz);
#pragma unroll
        for (int c = 0; c < 6; ++c) {
            a.x[6 * s + c] = 0.0;
            a.r[6 * s + c] = rr[c];
            a.d[6 * s + c] = zz[c];
            p += rr[c] * zz[c];
        }
    }
    p = block_sum(p);
    if (threadIdx.x == 0) a.part_b[blockIdx.x] = p;
    if (!grid_barrier(a.barrier, a.status)) return;
    double rz = block_sum_array(a.part_b, gridDim.x);
    const double initial = rz;
    if (initial == 0.0) {
        for (int64_t e = tid; e < 6 * a.n; e += stride) a.out[e] = 0.0;
        return;
    }
    int it = 0;
    for (; it < a.max_it; ++it) {
        // ad = (diag M + alpha K) d with identity rows on fixed sites
        for (int64_t b = tid; b < a.m; b += stride) {
            int64_t i, j;
            edge(a.edges, b, i, j);
            const double *qi = a.d + 6 * i, *qj = a.d + 6 * j;
            const d3 n = ld3(a.t.n, b), ri = ld3(a.t.ri, b), rj = ld3(a.t.rj, b);
            const d3 wi = ld3(qi + 3), wj = ld3(qj + 3);
            const d3 du = ld3(qj) - ld3(qi) + cross(wj, rj) - cross(wi, ri);
            const d3 dw = wj - wi;
            const double kn = a.k.kn[b], ks = a.k.ks[b], kb = a.k.kb[b], kt = a.k.kt[b];
            const d3 f = ks * du + ((kn - ks) * dot(du, n)) * n;
            const d3 mm = kb * dw + ((kt - kb) * dot(dw, n)) * n;
            double *w = a.wrench + 9 * b;
            st3(w, -f);
            st3(w + 3, -cross(ri, f) - mm);
            st3(w + 6, cross(rj, f) + mm);
        }
        if (!grid_barrier(a.barrier, a.status)) return;
        p = 0.0;
        for (int64_t s = tid; s < a.n; s += stride) {
            double acc[6];
            gather_wrench(a.ptr, a.inc, a.wrench, s, acc);
            const bool fx = a.fixed[s] != 0;
#pragma unroll
            for (int c = 0; c < 6; ++c) {
                const double dv = a.d[6 * s + c];
                const double v = fx ? dv : a.mass[6 * s + c] * dv + a.alpha_op * acc[c];
                a.ad[6 * s + c] = v;
                p += dv * v;
            }
        }
        p = block_sum(p);
        if (threadIdx.x == 0) a.part_a[blockIdx.x] = p;
        if (!grid_barrier(a.barrier, a.status)) return;
        const double alpha = block_divide(rz, block_sum_array(a.part_a, gridDim.x));
        p = 0.0;
        for (int64_t s = tid; s < a.n; s += stride) {
            double rr[6], zz[6];
#pragma unroll
            for (int c = 0; c < 6; ++c) {
                a.x[6 * s + c] += alpha * a.d[6 * s + c];
                rr[c] = a.r[6 * s + c] - alpha * a.ad[6 * s + c];
                a.r[6 * s + c] = rr[c];
            }
            matvec6(a.P + 36 * s, rr, zz);
#pragma unroll
            for (int c = 0; c < 6; ++c) {
                a.z[6 * s + c] = zz[c];
                p += rr[c] * zz[c];
            }
        }
        p = block_sum(p);
        if (threadIdx.x == 0) a.part_b[blockIdx.x] = p;
        if (!grid_barrier(a.barrier, a.status)) return;
        const double following = block_sum_array(a.part_b, gridDim.x);
        if (it % 5 == 0 && following <= a.tol2 * initial) break;
        const double beta = block_divide(following, rz);
        for (int64_t e = tid; e < 6 * a.n; e += stride) a.d[e] = a.z[e] + beta * a.d[e];
        rz = following;
        if (!grid_barrier(a.barrier, a.status)) return;
    }
    for (int64_t e = tid; e < 6 * a.n; e += stride) a.out[e] = a.x[e] / a.units[e];
    if (tid == 0) atomicAdd(a.iterations, it < a.max_it ? it + 1 : a.max_it);
}

// ---------------------------------------------------------------------------
// Arnoldi CGS2 (experiments/bonded_dem_newton.py:35-43).

__global__ void __launch_bounds__(kThreads) arnoldi_dots(int64_t len, const double *basis, int64_t ld, int count,
                                                         const double *w, double *part) {
    const int64_t tid = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    for (int k = 0; k < count; ++k) {
        const double *row = basis + k * ld;
        double p = 0.0;
        for (int64_t e = tid; e < len; e += stride) p += row[e] * w[e];
        p = block_sum(p);
        if (threadIdx.x == 0) part[k * gridDim.x + blockIdx.x] = p;
    }
}

// values_k = sum of part_in; h[k] (=|+=) values_k; w -= sum_k values_k basis_k;
// then optionally the next pass's partial dots (part_out) or |w|^2 (part_out[blk]).
__global__ void __launch_bounds__(kThreads) arnoldi_update(int64_t len, const double *basis, int64_t ld, int count,
                                                           double *w, const double *part_in, double *h,
                                                           int accumulate, double *part_out, int want_dots) {
    __shared__ double values[kMaxArnoldi];
    for (int k = 0; k < count; ++k) {
        const double v = block_sum_array(part_in + k * gridDim.x, gridDim.x);
        if (threadIdx.x == 0) values[k] = v;
    }
    __syncthreads();
    if (blockIdx.x == 0 && threadIdx.x == 0)
        for (int k = 0; k < count; ++k) h[k] = accumulate ? h[k] + values[k] : values[k];
    const int64_t tid = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    double sq = 0.0;
    for (int64_t e = tid; e < len; e += stride) {
        double proj = 0.0;
        for (int k = 0; k < count; ++k) proj += basis[k * ld + e] * values[k];
        const double wv = w[e] - proj;
        w[e] = wv;
        sq += wv * wv;
    }
    if (want_dots) {
        for (int k = 0; k < count; ++k) {
            const double *row = basis + k * ld;
            double p = 0.0;
            for (int64_t e = tid; e < len; e += stride) p += row[e] * w[e];
            p = block_sum(p);
            if (threadIdx.x == 0) part_out[k * gridDim.x + blockIdx.x] = p;
        }
    } else {
        sq = block_sum(sq);
        if (threadIdx.x == 0) part_out[blockIdx.x] = sq;
    }
}

__global__ void __launch_bounds__(kThreads) arnoldi_normalize(int64_t len, double *basis, int64_t ld, int j,
                                                              const double *w, const double *part, double *h) {
    const double nrm = sqrt(block_sum_array(part, gridDim.x));
    if (blockIdx.x == 0 && threadIdx.x == 0) h[j + 1] = nrm;
    if (!(nrm >= 1e-14)) return;
    const int64_t tid = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    double *row = basis + (int64_t)(j + 1) * ld;
    // one float64 division per block, then products (float64 divides are slow on this part)
    const double inv = 1.0 / nrm;
    for (int64_t e = tid; e < len; e += stride) row[e] = w[e] * inv;
}

struct Coefficients {
    double c[kMaxArnoldi];
};

__global__ void __launch_bounds__(kThreads) combine_rows_kernel(int64_t len, const double *rows, int64_t ld, int count,
                                                                Coefficients coef, double *x) {
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < len; e += stride) {
        double acc = 0.0;
        for (int k = 0; k < count; ++k) acc += rows[k * ld + e] * coef.c[k];
        x[e] += acc;
    }
}

__global__ void __launch_bounds__(kThreads) dot_norm_kernel(int64_t len, const double *a, const double *b,
                                                            double *result, double *partials) {
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    double ab = 0.0, aa = 0.0;
    for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < len; e += stride) {
        const double av = a[e];
        ab += av * (b ? b[e] : av);
        aa += av * av;
    }
    ab = block_sum(ab);
    aa = block_sum(aa);
    double *part = partials + kPartialsOffset;
    if (threadIdx.x == 0) {
        part[2 * blockIdx.x] = ab;
        part[2 * blockIdx.x + 1] = aa;
    }
    if (last_block(counter_slot(partials, 1))) {
        const double s_ab = block_sum_array(part, gridDim.x, 2);
        const double s_aa = block_sum_array(part + 1, gridDim.x, 2);
        if (threadIdx.x == 0) {
            result[0] = s_ab;
            result[1] = sqrt(s_aa);
        }
    }
}

__global__ void __launch_bounds__(kThreads) axpby_kernel(int64_t len, double alpha, const double *a, double beta,
                                                         const double *b, double *out) {
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < len; e += stride)
        out[e] = alpha * a[e] + beta * b[e];
}

// Scaled residual s = P r / units and [|r|, max|s|, |s|] (bonded_dem_newton.py:104-105, 147).
__global__ void __launch_bounds__(kThreads) scale_kernel(int64_t n, const double *P, const double *units,
                                                         const double *r, double *scaled, double *norms,
                                                         double *partials) {
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    double sum_r = 0.0, max_s = 0.0, sum_s = 0.0;
    for (int64_t s = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; s < n; s += stride) {
        double rr[6], ss[6];
#pragma unroll
        for (int c = 0; c < 6; ++c) {
            rr[c] = r[6 * s + c];
            sum_r += rr[c] * rr[c];
        }
        matvec6(P + 36 * s, rr, ss);
#pragma unroll
        for (int c = 0; c < 6; ++c) {
            const double v = ss[c] / units[6 * s + c];
            if (scaled) scaled[6 * s + c] = v;
            max_s = fmax(max_s, fabs(v));
            sum_s += v * v;
        }
    }
    if (!norms) return;
    sum_r = block_sum(sum_r);
    max_s = block_max(max_s);
    sum_s = block_sum(sum_s);
    double *part = partials + kPartialsOffset;
    if (threadIdx.x == 0) {
        part[3 * blockIdx.x] = sum_r;
        part[3 * blockIdx.x + 1] = max_s;
        part[3 * blockIdx.x + 2] = sum_s;
    }
    if (last_block(counter_slot(partials, 2))) {
        const double r2 = block_sum_array(part, gridDim.x, 3);
        const double mx = block_max_array(part + 1, gridDim.x, 3);
        const double s2 = block_sum_array(part + 2, gridDim.x, 3);
        if (threadIdx.x == 0) {
            norms[0] = sqrt(r2);
            norms[1] = mx;
            norms[2] = sqrt(s2);
        }
    }
}

// v <- 2 y / dt - v;  R <- exp(y_w) R   (bonded_dem_newton.py:150-153, bonded_dem_finite_gpu.py:35-43)
__global__ void __launch_bounds__(kThreads) accept_kernel(int64_t n, const double *y, double dt, double *v,
                                                          double *rotation) {
    const int64_t s = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (s >= n) return;
    const double two_over_dt = 2.0 / dt;  // one float64 division per site, not six
#pragma unroll
    for (int c = 0; c < 6; ++c) v[6 * s + c] = two_over_dt * y[6 * s + c] - v[6 * s + c];
    const d3 w = ld3(y + 6 * s + 3);
    // Rodrigues coefficients A = sin(a)/a and B = (1 - cos a)/a^2 of a = |w|.
    // Both are even in a: for a^2 < 1/4 (every step the rotation guard lets
    // through has a <= 0.25) their Maclaurin series in a^2, 8 terms each,
    // are exact to a few 1e-17 and need no float64 transcendental, which is
    // slow on this part.  Larger angles take the closed form.
    const double theta = w.x * w.x + w.y * w.y + w.z * w.z;
    double A, B;
    if (theta < 0.25) {
        // Horner in theta: A = sum (-theta)^k/(2k+1)!, B = sum (-theta)^k/(2k+2)!, k = 0..7
        A = 1.0 / 1307674368000.0;                 // 1/15!
        A = fma(-theta, A, 1.0 / 6227020800.0);    // 1/13!
        A = fma(-theta, A, 1.0 / 39916800.0);      // 1/11!
        A = fma(-theta, A, 1.0 / 362880.0);        // 1/9!
        A = fma(-theta, A, 1.0 / 5040.0);          // 1/7!
        A = fma(-theta, A, 1.0 / 120.0);           // 1/5!
        A = fma(-theta, A, 1.0 / 6.0);             // 1/3!
        A = fma(-theta, A, 1.0);
        B = 1.0 / 20922789888000.0;                // 1/16!
        B = fma(-theta, B, 1.0 / 87178291200.0);   // 1/14!
        B = fma(-theta, B, 1.0 / 479001600.0);     // 1/12!
        B = fma(-theta, B, 1.0 / 3628800.0);       // 1/10!
        B = fma(-theta, B, 1.0 / 40320.0);         // 1/8!
        B = fma(-theta, B, 1.0 / 720.0);           // 1/6!
        B = fma(-theta, B, 1.0 / 24.0);            // 1/4!
        B = fma(-theta, B, 0.5);
    } else {
        const double angle = sqrt(theta);
        double sh, ch;
        sincos(0.5 * angle, &sh, &ch);
        A = sin(angle) / angle;
        const double q = sh / (0.5 * angle);
        B = 0.5 * q * q;
    }
    const double S[9] = {0.0, -w.z, w.y, w.z, 0.0, -w.x, -w.y, w.x, 0.0};
    double E[9];
#pragma unroll
    for (int p = 0; p < 3; ++p)
#pragma unroll
        for (int q = 0; q < 3; ++q) {
            const double ss = S[3 * p] * S[q] + S[3 * p + 1] * S[3 + q] + S[3 * p + 2] * S[6 + q];
            E[3 * p + q] = (p == q ? 1.0 : 0.0) + A * S[3 * p + q] + B * ss;
        }
    double *R = rotation + 9 * s;
    double Rn[9];
#pragma unroll
    for (int p = 0; p < 3; ++p)
#pragma unroll
        for (int q = 0; q < 3; ++q) Rn[3 * p + q] = E[3 * p] * R[q] + E[3 * p + 1] * R[3 + q] + E[3 * p + 2] * R[6 + q];
#pragma unroll
    for (int c = 0; c < 9; ++c) R[c] = Rn[c];
}

// Elastic + kinetic energy (bonded_dem_finite_gpu.py:122-125).
__global__ void __launch_bounds__(kThreads) energy_kernel(int64_t m, int64_t n, dpf_stiffness k, dpf_history h,
                                                          const double *mass, const double *v, double *energy,
                                                          double *partials) {
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    const int64_t tid = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    double el = 0.0, kin = 0.0;
    for (int64_t b = tid; b < m; b += stride) {
        const d3 fs = ld3(h.fs, b), mb = ld3(h.mb, b);
        const double fn = h.fn[b], mt = h.mt[b];
        el += fn * fn / k.kn[b] + dot(fs, fs) / k.ks[b] + mt * mt / k.kt[b] + dot(mb, mb) / k.kb[b];
    }
    for (int64_t e = tid; e < 6 * n; e += stride) kin += mass[e] * v[e] * v[e];
    el = block_sum(el);
    kin = block_sum(kin);
    double *part = partials + kPartialsOffset;
    if (threadIdx.x == 0) {
        part[2 * blockIdx.x] = el;
        part[2 * blockIdx.x + 1] = kin;
    }
    if (last_block(counter_slot(partials, 3))) {
        const double se = block_sum_array(part, gridDim.x, 2);
        const double sk = block_sum_array(part + 1, gridDim.x, 2);
        if (threadIdx.x == 0) *energy = 0.5 * se + 0.5 * sk;
    }
}

// [|dt M v + dt^2/2 ext|, |loads on free sites|] (bonded_dem_newton.py:138-139).
__global__ void __launch_bounds__(kThreads) rhs_scale_kernel(int64_t n, const double *mass, const double *v,
                                                             const double *external, const double *loads,
                                                             const uint8_t *fixed, double dt, double half_dt2,
                                                             double *out, double *partials) {
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    double a2 = 0.0, l2 = 0.0;
    for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < 6 * n; e += stride) {
        const double a = dt * mass[e] * v[e] + half_dt2 * external[e];
        a2 += a * a;
        if (!fixed[e / 6]) l2 += loads[e] * loads[e];
    }
    a2 = block_sum(a2);
    l2 = block_sum(l2);
    double *part = partials + kPartialsOffset;
    if (threadIdx.x == 0) {
        part[2 * blockIdx.x] = a2;
        part[2 * blockIdx.x + 1] = l2;
    }
    if (last_block(counter_slot(partials, 4))) {
        const double sa = block_sum_array(part, gridDim.x, 2);
        const double sl = block_sum_array(part + 1, gridDim.x, 2);
        if (threadIdx.x == 0) {
            out[0] = sqrt(sa);
            out[1] = sqrt(sl);
        }
    }
}

// out = units * a with zero rows on fixed sites (bonded_dem_newton.py:186-187).
__global__ void __launch_bounds__(kThreads) masked_scale_kernel(int64_t n, const double *a, const double *units,
                                                                const uint8_t *fixed, double *out) {
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < 6 * n; e += stride)
        out[e] = fixed[e / 6] ? 0.0 : units[e] * a[e];
}

struct DeviceInfo {
    int sms = 0;
    int pcg_blocks_per_sm = 0;
};

static DeviceInfo &device_info() {
    static DeviceInfo info[64];
    int dev = 0;
    cudaGetDevice(&dev);
    DeviceInfo &d = info[dev & 63];
    if (d.sms == 0) {
        cudaDeviceGetAttribute(&d.sms, cudaDevAttrMultiProcessorCount, dev);
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&d.pcg_blocks_per_sm, pcg_kernel, kThreads, 0);
    }
    return d;
}

}  // namespace dpf

using namespace dpf;

namespace dpf {

// ---------------------------------------------------------------------------
// Krylov vectors in float32 with exactly accumulated float32 pairs.  The
// mixed Newton path's Krylov inputs (PCG and JVP outputs, the scaled residual)
// carry float32 precision; storing the basis in float32 and forming dot
// products and updates as float32 pairs (TwoProd by FMA, TwoSum) gives
// float64-quality sums without float64 arithmetic per entry, which is scarce
// on this part (the float64 form of these kernels ran at 77-82% of the FP64
// pipe).  Block partials and the Hessenberg entries stay float64.

__device__ __forceinline__ void ff_two_sum(float &s, float &e, float b) {
    const float t = s + b;
    const float bp = t - s;
    e += (s - (t - bp)) + (b - bp);
    s = t;
}

// (hi, lo) += a b exactly up to the pair's precision
__device__ __forceinline__ void ff_add_product(float &hi, float &lo, float a, float b) {
    const float p = a * b;
    const float e = fmaf(a, b, -p);
    ff_two_sum(hi, lo, p);
    lo += e;
}

__device__ __forceinline__ double ff_value(float hi, float lo) { return (double)hi + (double)lo; }

// float64 value v as hi + lo float32 (lo the rounded remainder)
__device__ __forceinline__ void ff_split(double v, float &hi, float &lo) {
    hi = (float)v;
    lo = (float)(v - (double)hi);
}

// x += sum_k c_k rows_k, the sum as a float32 pair, added to float64 x
__global__ void __launch_bounds__(kThreads) combine32_kernel(int64_t len, const float *rows, int64_t ld, int count,
                                                             Coefficients coef, double *x) {
    __shared__ float chi[kMaxArnoldi], clo[kMaxArnoldi];
    if (threadIdx.x < count) ff_split(coef.c[threadIdx.x], chi[threadIdx.x], clo[threadIdx.x]);
    __syncthreads();
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < len; e += stride) {
        float hi = 0.0f, lo = 0.0f;
        for (int k = 0; k < count; ++k) {
            const float r = rows[k * ld + e];
            ff_add_product(hi, lo, chi[k], r);
            lo = fmaf(clo[k], r, lo);
        }
        x[e] += ff_value(hi, lo);
    }
}

// CGS2 of one Arnoldi step in one cooperative launch: dots, projection,
// dots, projection and norm, normalisation, with grid barriers between them
// and pairs of floats per access.  Block partials are float32 pairs; every
// block sums them in the same order, so all take the same values.  Partials:
// part1 = count x grid, part2 = count x grid, part3 = grid pairs.
struct Arnoldi32Args {
    int64_t half;        // length / 2 (the length is even: 6 per site)
    const float2 *basis;  // rows of ld2 float2
    float2 *next;         // row count (written)
    int64_t ld2;
    int count;
    const float2 *v;
    float2 *w;
    double *h, *part1, *part2, *part3;
    unsigned *barrier;
    int *status;
};

// per-thread float32-pair dots of rows 0..count-1 with x, reduced per block
// into part[k * gridDim.x + blockIdx.x]
__device__ __forceinline__ void arnoldi_dots_pass(const Arnoldi32Args &a, const float2 *x, double *part) {
    const int64_t tid = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    for (int k0 = 0; k0 < a.count; k0 += 4) {
        float hi[4] = {0.0f, 0.0f, 0.0f, 0.0f}, lo[4] = {0.0f, 0.0f, 0.0f, 0.0f};
        const int kn = a.count - k0 < 4 ? a.count - k0 : 4;
        for (int64_t e = tid; e < a.half; e += stride) {
            const float2 xv = x[e];
#pragma unroll
            for (int q = 0; q < 4; ++q) {
                if (q < kn) {
                    const float2 b = a.basis[(k0 + q) * a.ld2 + e];
                    ff_add_product(hi[q], lo[q], b.x, xv.x);
                    ff_add_product(hi[q], lo[q], b.y, xv.y);
                }
            }
        }
        for (int q = 0; q < kn; ++q) {
            const float2 p = block_pair_sum(hi[q], lo[q]);
            if (threadIdx.x == 0) reinterpret_cast<float2 *>(part)[(k0 + q) * gridDim.x + blockIdx.x] = p;
        }
    }
}

// w = in - sum_k values_k basis_k (values from the partials of the last pass),
// the projection as float32 pairs; returns this thread's |w|^2 pair
__device__ __forceinline__ void arnoldi_project(const Arnoldi32Args &a, const float2 *in, const double *part,
                                               bool second, float &sq_hi, float &sq_lo) {
    __shared__ float vhi[kMaxArnoldi], vlo[kMaxArnoldi];
    for (int k = 0; k < a.count; ++k) {
        const double v = pair_total(reinterpret_cast<const float2 *>(part) + k * gridDim.x, gridDim.x);
        if (threadIdx.x == 0) {
            ff_split(v, vhi[k], vlo[k]);
            if (blockIdx.x == 0) a.h[k] = second ? a.h[k] + v : v;
        }
    }
    __syncthreads();
    const int64_t tid = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    for (int64_t e = tid; e < a.half; e += stride) {
        float2 ph = make_float2(0.0f, 0.0f), pl = make_float2(0.0f, 0.0f);
        for (int k = 0; k < a.count; ++k) {
            const float2 b = a.basis[k * a.ld2 + e];
            ff_add_product(ph.x, pl.x, vhi[k], b.x);
            ff_add_product(ph.y, pl.y, vhi[k], b.y);
            pl.x = fmaf(vlo[k], b.x, pl.x);
            pl.y = fmaf(vlo[k], b.y, pl.y);
        }
        const float2 iv = in[e];
        float dx = iv.x, ex = 0.0f, dy = iv.y, ey = 0.0f;
        ff_two_sum(dx, ex, -ph.x);
        ff_two_sum(dy, ey, -ph.y);
        const float2 wv = make_float2(dx + (ex - pl.x), dy + (ey - pl.y));
        a.w[e] = wv;
        ff_add_product(sq_hi, sq_lo, wv.x, wv.x);
        ff_add_product(sq_hi, sq_lo, wv.y, wv.y);
    }
}

__global__ void __launch_bounds__(kThreads) arnoldi32_fused_kernel(Arnoldi32Args a) {
    arnoldi_dots_pass(a, a.v, a.part1);
    if (!grid_barrier(a.barrier, a.status)) return;
    float sh = 0.0f, sl = 0.0f;
    arnoldi_project(a, a.v, a.part1, false, sh, sl);
    // the second pass reads w only after every block has written it
    if (!grid_barrier(a.barrier, a.status)) return;
    arnoldi_dots_pass(a, a.w, a.part2);
    if (!grid_barrier(a.barrier, a.status)) return;
    sh = sl = 0.0f;
    arnoldi_project(a, a.w, a.part2, true, sh, sl);
    const float2 sq = block_pair_sum(sh, sl);
    if (threadIdx.x == 0) reinterpret_cast<float2 *>(a.part3)[blockIdx.x] = sq;
    if (!grid_barrier(a.barrier, a.status)) return;
    const double nrm = sqrt(pair_total(reinterpret_cast<const float2 *>(a.part3), gridDim.x));
    if (blockIdx.x == 0 && threadIdx.x == 0) a.h[a.count] = nrm;
    if (!(nrm >= 1e-14)) return;
    const float inv = (float)(1.0 / nrm);
    const int64_t tid = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    for (int64_t e = tid; e < a.half; e += stride) {
        const float2 wv = a.w[e];
        a.next[e] = make_float2(wv.x * inv, wv.y * inv);
    }
}

__global__ void __launch_bounds__(kThreads) scale_to_float_kernel(int64_t len, double alpha, const double *a,
                                                                  float *out) {
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < len; e += stride)
        out[e] = (float)(alpha * a[e]);
}

}  // namespace dpf

extern "C" {

int64_t dpf_elastic_workspace_doubles(int64_t n_sites) { return 30 * n_sites + 2 * (int64_t)kMaxPcgBlocks; }

int dpf_elastic_precondition(const dpf_graph *g, const dpf_stiffness *k, const dpf_tangent *t, const double *mass,
                             const uint8_t *fixed, const double *block, const double *preconditioner,
                             const double *units, const double *vector, double dt, double tolerance,
                             int max_iterations, double *out, int *iterations, double *wrench, double *workspace,
                             unsigned *barrier, int *status, void *stream) {
    if (!g || g->n_sites <= 0 || !g->inc_ptr || (g->n_bonds && !g->inc_bond) || !k || !t || !mass || !fixed ||
        !block ||
        !preconditioner || !units || !vector || !out || !iterations || !workspace || !barrier || !status ||
        max_iterations < 1 || (g->n_bonds && (!wrench || !g->edges)))
        return DPF_ERR_ARGUMENT;
    cudaStream_t st = (cudaStream_t)stream;
    DeviceInfo &info = device_info();
    if (info.sms <= 0 || info.pcg_blocks_per_sm <= 0) return DPF_ERR_CUDA;
    int64_t want = blocks_for(g->n_sites > g->n_bonds ? g->n_sites : g->n_bonds, kThreads);
    int64_t cap = (int64_t)info.sms * info.pcg_blocks_per_sm;
    if (cap > kMaxPcgBlocks) cap = kMaxPcgBlocks;
    const int grid = (int)(want < cap ? (want < 1 ? 1 : want) : cap);
    const int64_t n6 = 6 * g->n_sites;
    PcgArgs a{};
    a.n = g->n_sites;
    a.m = g->n_bonds;
    a.ptr = g->inc_ptr;
    a.inc = g->inc_bond;
    a.edges = g->edges;
    a.k = *k;
    a.t = *t;
    a.mass = mass;
    a.block = block;
    a.P = preconditioner;
    a.units = units;
    a.vector = vector;
    a.fixed = fixed;
    a.alpha_op = 0.25 * dt * dt;
    a.tol2 = tolerance * tolerance;
    a.max_it = max_iterations;
    a.out = out;
    a.iterations = iterations;
    a.wrench = wrench;
    a.x = workspace;
    a.r = workspace + n6;
    a.z = workspace + 2 * n6;
    a.d = workspace + 3 * n6;
    a.ad = workspace + 4 * n6;
    a.part_a = workspace + 5 * n6;
    a.part_b = workspace + 5 * n6 + kMaxPcgBlocks;
    a.barrier = barrier;
    a.status = status;
    if (cudaMemsetAsync(barrier, 0, 2 * sizeof(unsigned), st) != cudaSuccess) return DPF_ERR_CUDA;
    void *args[] = {&a};
    if (cudaLaunchCooperativeKernel((const void *)pcg_kernel, grid, kThreads, args, 0, st) != cudaSuccess) {
        cudaGetLastError();
        return DPF_ERR_CUDA;
    }
    return DPF_OK;
}

int dpf_arnoldi_cgs2(int64_t length, double *basis, int64_t ld, int j, double *w, double *h, double *partials,
                     void *stream) {
    if (length <= 0 || !basis || !w || !h || !partials || j < 0 || j + 1 >= kMaxArnoldi || ld < length)
        return DPF_ERR_ARGUMENT;
    cudaStream_t st = (cudaStream_t)stream;
    const int grid = reduce_grid(length);
    const int count = j + 1;
    double *pa = partials + kPartialsOffset;
    double *pb = pa + (int64_t)kMaxArnoldi * kMaxReduceBlocks;
    arnoldi_dots<<<grid, kThreads, 0, st>>>(length, basis, ld, count, w, pa);
    arnoldi_update<<<grid, kThreads, 0, st>>>(length, basis, ld, count, w, pa, h, 0, pb, 1);
    arnoldi_update<<<grid, kThreads, 0, st>>>(length, basis, ld, count, w, pb, h, 1, pa, 0);
    arnoldi_normalize<<<grid, kThreads, 0, st>>>(length, basis, ld, j, w, pa, h);
    DPF_CHECK_LAUNCH();
    return DPF_OK;
}

int dpf_arnoldi_cgs2_f32(int64_t length, float *basis, int64_t ld, int j, const float *v, float *w, double *h,
                         double *partials, unsigned *barrier, int *status, void *stream) {
    if (length <= 0 || (length & 1) || (ld & 1) || !basis || !v || !w || !h || !partials || !barrier || !status ||
        j < 0 || j + 1 >= kMaxArnoldi || ld < length || (((uintptr_t)basis | (uintptr_t)v | (uintptr_t)w) & 7u))
        return DPF_ERR_ARGUMENT;
    cudaStream_t st = (cudaStream_t)stream;
    static int per_sm[64] = {0}, sms[64] = {0};
    int dev = 0;
    cudaGetDevice(&dev);
    if (per_sm[dev & 63] == 0) {
        cudaDeviceGetAttribute(&sms[dev & 63], cudaDevAttrMultiProcessorCount, dev);
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm[dev & 63], arnoldi32_fused_kernel, kThreads, 0);
    }
    int grid = sms[dev & 63] * (per_sm[dev & 63] < 4 ? per_sm[dev & 63] : 4);
    const int64_t need = (length / 2 + kThreads - 1) / kThreads;
    if (grid > need) grid = (int)need;
    if (grid > kMaxReduceBlocks) grid = kMaxReduceBlocks;
    if (grid < 1) return DPF_ERR_CUDA;
    Arnoldi32Args a;
    a.half = length / 2;
    a.basis = reinterpret_cast<const float2 *>(basis);
    a.ld2 = ld / 2;
    a.next = reinterpret_cast<float2 *>(basis + (int64_t)(j + 1) * ld);
    a.count = j + 1;
    a.v = reinterpret_cast<const float2 *>(v);
    a.w = reinterpret_cast<float2 *>(w);
    a.h = h;
    a.part1 = partials + kPartialsOffset;
    a.part2 = a.part1 + (int64_t)kMaxArnoldi * kMaxReduceBlocks;
    a.part3 = a.part2 + (int64_t)(kMaxArnoldi - 1) * kMaxReduceBlocks;
    a.barrier = barrier;
    a.status = status;
    // a wait that timed out in an earlier launch leaves a partial arrival count
    if (cudaMemsetAsync(barrier, 0, 2 * sizeof(unsigned), st) != cudaSuccess) {
        cudaGetLastError();
        return DPF_ERR_CUDA;
    }
    void *args[] = {&a};
    if (cudaLaunchCooperativeKernel((const void *)arnoldi32_fused_kernel, grid, kThreads, args, 0, st) !=
        cudaSuccess) {
        cudaGetLastError();
        return DPF_ERR_CUDA;
    }
    return DPF_OK;
}

int dpf_combine_rows_f32(int64_t length, const float *rows, int64_t ld, int count, const double *coefficients,
                         double *x, void *stream) {
    if (length <= 0 || !rows || !x || count < 0 || count > kMaxArnoldi || (count && !coefficients))
        return DPF_ERR_ARGUMENT;
    Coefficients c{};
    for (int k = 0; k < count; ++k) c.c[k] = coefficients[k];
    combine32_kernel<<<reduce_grid(length), kThreads, 0, (cudaStream_t)stream>>>(length, rows, ld, count, c, x);
    DPF_CHECK_LAUNCH();
    return DPF_OK;
}

int dpf_scale_to_float(int64_t length, double alpha, const double *a, float *out, void *stream) {
    if (length <= 0 || !a || !out) return DPF_ERR_ARGUMENT;
    scale_to_float_kernel<<<reduce_grid(length), kThreads, 0, (cudaStream_t)stream>>>(length, alpha, a, out);
    DPF_CHECK_LAUNCH();
    return DPF_OK;
}

int dpf_combine_rows(int64_t length, const double *rows, int64_t ld, int count, const double *coefficients, double *x,
                     void *stream) {
    if (length <= 0 || !rows || !x || count < 0 || count > kMaxArnoldi || (count && !coefficients))
        return DPF_ERR_ARGUMENT;
    Coefficients c{};
    for (int k = 0; k < count; ++k) c.c[k] = coefficients[k];
    combine_rows_kernel<<<reduce_grid(length), kThreads, 0, (cudaStream_t)stream>>>(length, rows, ld, count, c, x);
    DPF_CHECK_LAUNCH();
    return DPF_OK;
}

int dpf_dot_norm(int64_t length, const double *a, const double *b, double *result, double *partials, void *stream) {
    if (length <= 0 || !a || !result || !partials) return DPF_ERR_ARGUMENT;
    dot_norm_kernel<<<reduce_grid(length), kThreads, 0, (cudaStream_t)stream>>>(length, a, b, result, partials);
    DPF_CHECK_LAUNCH();
    return DPF_OK;
}

int dpf_axpby(int64_t length, double alpha, const double *a, double beta, const double *b, double *out,
              void *stream) {
    if (length <= 0 || !a || !b || !out) return DPF_ERR_ARGUMENT;
    axpby_kernel<<<reduce_grid(length), kThreads, 0, (cudaStream_t)stream>>>(length, alpha, a, beta, b, out);
    DPF_CHECK_LAUNCH();
    return DPF_OK;
}

int dpf_scale_residual(int64_t n_sites, const double *preconditioner, const double *units, const double *residual,
                       double *scaled, double *norms, double *partials, void *stream) {
    if (n_sites <= 0 || !preconditioner || !units || !residual || (norms && !partials)) return DPF_ERR_ARGUMENT;
    scale_kernel<<<reduce_grid(n_sites), kThreads, 0, (cudaStream_t)stream>>>(n_sites, preconditioner, units,
                                                                               residual, scaled, norms, partials);
    DPF_CHECK_LAUNCH();
    return DPF_OK;
}

int dpf_accept_step(int64_t n_sites, const double *y, double dt, double *v, double *rotation, void *stream) {
    if (n_sites <= 0 || !y || !v || !rotation) return DPF_ERR_ARGUMENT;
    accept_kernel<<<blocks_for(n_sites, kThreads), kThreads, 0, (cudaStream_t)stream>>>(n_sites, y, dt, v, rotation);
    DPF_CHECK_LAUNCH();
    return DPF_OK;
}

int dpf_energy(const dpf_graph *g, const dpf_stiffness *k, const dpf_history *h, const double *mass, const double *v,
               double *energy, double *partials, void *stream) {
    if (!g || g->n_sites <= 0 || !k || !h || !mass || !v || !energy || !partials) return DPF_ERR_ARGUMENT;
    const int64_t work = g->n_bonds > 6 * g->n_sites ? g->n_bonds : 6 * g->n_sites;
    energy_kernel<<<reduce_grid(work), kThreads, 0, (cudaStream_t)stream>>>(g->n_bonds, g->n_sites, *k, *h, mass, v,
                                                                            energy, partials);
    DPF_CHECK_LAUNCH();
    return DPF_OK;
}

int dpf_rhs_scale(int64_t n_sites, const double *mass, const double *v, const double *external, const double *loads,
                  const uint8_t *fixed, double dt, double *out, double *partials, void *stream) {
    if (n_sites <= 0 || !mass || !v || !external || !loads || !fixed || !out || !partials) return DPF_ERR_ARGUMENT;
    rhs_scale_kernel<<<reduce_grid(6 * n_sites), kThreads, 0, (cudaStream_t)stream>>>(
        n_sites, mass, v, external, loads, fixed, dt, 0.5 * dt * dt, out, partials);
    DPF_CHECK_LAUNCH();
    return DPF_OK;
}

int dpf_masked_scale(int64_t n_sites, const double *a, const double *units, const uint8_t *fixed, double *out,
                     void *stream) {
    if (n_sites <= 0 || !a || !units || !fixed || !out) return DPF_ERR_ARGUMENT;
    masked_scale_kernel<<<reduce_grid(6 * n_sites), kThreads, 0, (cudaStream_t)stream>>>(n_sites, a, units, fixed,
                                                                                         out);
    DPF_CHECK_LAUNCH();
    return DPF_OK;
}

}  // extern "C"
