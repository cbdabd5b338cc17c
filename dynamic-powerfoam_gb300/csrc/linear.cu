// Float64 linear solves of the reference's linearised model and of its
// previous (Anderson) solver, as library kernels:
//   * the operator (diag M + alpha K) q with identity rows on fixed sites;
//   * one cooperative launch of block-Jacobi PCG with either stopping test
//     (the linear model's, or the previous solver's "balanced" test with the
//     local pose defect and a true-residual exit check);
//   * the vector updates of the linear implicit-midpoint step and its energy;
//   * the small reductions of Anderson mixing over device history buffers;
//   * a self-test of the time-limited grid barrier.
// Every reduction is per block then in a fixed order: results are bitwise
// reproducible run to run.
#include "common.cuh"

namespace dpf {
namespace lin {

constexpr int kMaxBlocks = 4096;
constexpr int kMaxHistory = 8;  // Anderson slots (the reference keeps 6 iterates)
constexpr int64_t kCounter = 8;  // doubles reserved for "last block" counters at the head of partials

inline int blocks_for(int64_t n, int threads) { return (int)((n + threads - 1) / threads); }
inline int reduce_grid(int64_t n) {
    int g = blocks_for(n, kThreads);
    if (g > 1024) g = 1024;
    return g < 1 ? 1 : g;
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

// Wrench of K v on bond b, stored as [F_i, T_i, T_j] (F_j = -F_i).
__device__ __forceinline__ void stiffness_wrench(const int64_t *edges, const dpf_stiffness &k, const dpf_tangent &t,
                                                 const double *v, int64_t b, double *wrench) {
    int64_t i, j;
    edge(edges, b, i, j);
    const double *vi = v + 6 * i, *vj = v + 6 * j;
    const d3 n = ld3(t.n, b), ri = ld3(t.ri, b), rj = ld3(t.rj, b);
    const d3 wi = ld3(vi + 3), wj = ld3(vj + 3);
    const d3 du = ld3(vj) - ld3(vi) + cross(wj, rj) - cross(wi, ri);
    const d3 dw = wj - wi;
    const double kn = k.kn[b], ks = k.ks[b], kb = k.kb[b], kt = k.kt[b];
    const d3 f = ks * du + ((kn - ks) * dot(du, n)) * n;
    const d3 m = kb * dw + ((kt - kb) * dot(dw, n)) * n;
    double *w = wrench + 9 * b;
    st3(w, -f);
    st3(w + 3, -cross(ri, f) - m);
    st3(w + 6, cross(rj, f) + m);
}

struct Operator {
    int64_t n, m;
    const int32_t *ptr, *inc;
    const int64_t *edges;
    dpf_stiffness k;
    dpf_tangent t;
    const double *mass;
    const uint8_t *fixed;
    double alpha;
    double *wrench;
};

// (diag M + alpha K) v at site s from the bond wrenches of v; v on fixed sites.
__device__ __forceinline__ void operator_site(const Operator &A, const double *v, int64_t s, double out[6]) {
    double acc[6];
    gather_wrench(A.ptr, A.inc, A.wrench, s, acc);
    const bool fx = A.fixed[s] != 0;
#pragma unroll
    for (int c = 0; c < 6; ++c) {
        const double vv = v[6 * s + c];
        out[c] = fx ? vv : A.mass[6 * s + c] * vv + A.alpha * acc[c];
    }
}

__global__ void __launch_bounds__(kThreads) operator_bonds(Operator A, const double *v) {
    const int64_t b = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (b < A.m) stiffness_wrench(A.edges, A.k, A.t, v, b, A.wrench);
}

__global__ void __launch_bounds__(kThreads) operator_sites(Operator A, const double *v, double *out) {
    const int64_t s = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (s >= A.n) return;
    double o[6];
    operator_site(A, v, s, o);
#pragma unroll
    for (int c = 0; c < 6; ++c) out[6 * s + c] = o[c];
}

// ---------------------------------------------------------------------------
// Block-Jacobi PCG on (diag M + alpha K) x = b, identity rows on fixed sites
// and b's fixed rows read as zero, in one cooperative launch.
//
// kLinear (LinearBondsGPU.solve_increment, bonded_dem_linear_gpu.py:79-112):
//   start from the guess (fixed rows zeroed); every 10th iteration stop when
//   |r| / |b| < tol; afterwards the true residual |b - A x| / |b| is returned.
// kBalanced (FiniteBondsGPU.solve_increment, bonded_dem_finite_gpu.py:133-167):
//   start from zero; every 10th iteration, when |r| / |b| < tol and the pose
//   defect max |P r / scale| < 2e-8, check the true residual a = b - A x:
//   stop when |a| / |b| < 5 tol and max |P a / scale| < 1e-7.
// Both flag a non-finite residual at a test.  info = [iterations, relative
// residual (kLinear: true residual; kBalanced: the accepted true residual or
// the last tested one), state (0 converged, 1 iteration cap, 2 non-finite), |b|].

enum { kLinear = 0, kBalanced = 1 };

struct BlockPcgArgs {
    Operator A;
    const double *P, *scale, *rhs;
    double tol, zero_norm;
    int max_it, mode, use_guess;
    double *x, *info;
    double *r, *z, *d, *ad, *part;  // part: 2 x 3 x kMaxBlocks
    unsigned *barrier;
    int *status;
};

struct Reducer {
    double *part;
    int buf;
    // Block partials (sum, sum, max) -> grid barrier -> the same totals in every block.
    __device__ __forceinline__ bool operator()(double s0, double s1, double m2, unsigned *barrier, int *status,
                                               double out[3]) {
        s0 = block_sum(s0);
        s1 = block_sum(s1);
        m2 = block_max(m2);
        double *p = part + (int64_t)buf * 3 * kMaxBlocks;
        if (threadIdx.x == 0) {
            p[3 * blockIdx.x] = s0;
            p[3 * blockIdx.x + 1] = s1;
            p[3 * blockIdx.x + 2] = m2;
        }
        if (!grid_barrier(barrier, status)) return false;
        out[0] = block_sum_array(p, gridDim.x, 3);
        out[1] = block_sum_array(p + 1, gridDim.x, 3);
        out[2] = block_max_array(p + 2, gridDim.x, 3);
        buf ^= 1;  // the other buffer: no block still reads it after the next barrier
        return true;
    }
};

__device__ __forceinline__ bool sweep_bonds(const BlockPcgArgs &a, const double *v, int64_t tid, int64_t stride) {
    for (int64_t b = tid; b < a.A.m; b += stride) stiffness_wrench(a.A.edges, a.A.k, a.A.t, v, b, a.A.wrench);
    return grid_barrier(a.barrier, a.status);
}

__device__ __forceinline__ void rhs_site(const BlockPcgArgs &a, int64_t s, double b6[6]) {
    const bool fx = a.A.fixed[s] != 0;
#pragma unroll
    for (int c = 0; c < 6; ++c) b6[c] = fx ? 0.0 : a.rhs[6 * s + c];
}

__device__ __forceinline__ double scaled_max(const BlockPcgArgs &a, int64_t s, const double z6[6], double m) {
    if (!a.scale) return m;
#pragma unroll
    for (int c = 0; c < 6; ++c) m = fmax(m, fabs(z6[c] / a.scale[6 * s + c]));
    return m;
}

__global__ void __launch_bounds__(kThreads) block_pcg_kernel(BlockPcgArgs a) {
    const int64_t tid = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    const int64_t n = a.A.n;
    Reducer reduce{a.part, 0};
    double tot[3];
    // x0: the guess with fixed rows zeroed, or zero
    for (int64_t s = tid; s < n; s += stride) {
        const bool keep = a.use_guess && !a.A.fixed[s];
#pragma unroll
        for (int c = 0; c < 6; ++c) a.x[6 * s + c] = keep ? a.x[6 * s + c] : 0.0;
    }
    if (a.use_guess) {
        if (!grid_barrier(a.barrier, a.status)) return;
        if (!sweep_bonds(a, a.x, tid, stride)) return;
    }
    // r = b - A x0, z = P r, d = z
    double rz = 0.0, bb = 0.0;
    for (int64_t s = tid; s < n; s += stride) {
        double b6[6], rr[6], zz[6];
        rhs_site(a, s, b6);
        if (a.use_guess) {
            double ax[6];
            operator_site(a.A, a.x, s, ax);
#pragma unroll
            for (int c = 0; c < 6; ++c) rr[c] = b6[c] - ax[c];
        } else {
#pragma unroll
            for (int c = 0; c < 6; ++c) rr[c] = b6[c];
        }
        matvec6(a.P + 36 * s, rr, zz);
#pragma unroll
        for (int c = 0; c < 6; ++c) {
            a.r[6 * s + c] = rr[c];
            a.z[6 * s + c] = zz[c];
            a.d[6 * s + c] = zz[c];
            rz += rr[c] * zz[c];
            bb += b6[c] * b6[c];
        }
    }
    if (!reduce(rz, bb, 0.0, a.barrier, a.status, tot)) return;
    rz = tot[0];
    const double norm = sqrt(tot[1]);
    if (norm < a.zero_norm) {
        for (int64_t e = tid; e < 6 * n; e += stride) a.x[e] = 0.0;
        if (tid == 0) {
            a.info[0] = 0.0;
            a.info[1] = 0.0;
            a.info[2] = 0.0;
            a.info[3] = norm;
        }
        return;
    }
    int it = 0, state = 1;
    double relative = 0.0;
    for (; it < a.max_it; ++it) {
        // ad = A d, (d, ad)
        if (!sweep_bonds(a, a.d, tid, stride)) return;
        double dad = 0.0;
        for (int64_t s = tid; s < n; s += stride) {
            double v[6];
            operator_site(a.A, a.d, s, v);
#pragma unroll
            for (int c = 0; c < 6; ++c) {
                a.ad[6 * s + c] = v[c];
                dad += a.d[6 * s + c] * v[c];
            }
        }
        if (!reduce(dad, 0.0, 0.0, a.barrier, a.status, tot)) return;
        const double step = block_divide(rz, tot[0]);
        // x += step d, r -= step ad, z = P r; (r, z), |r|^2, max |z / scale|
        double rz1 = 0.0, rr2 = 0.0, zmax = 0.0;
        for (int64_t s = tid; s < n; s += stride) {
            double rr[6], zz[6];
#pragma unroll
            for (int c = 0; c < 6; ++c) {
                a.x[6 * s + c] += step * a.d[6 * s + c];
                rr[c] = a.r[6 * s + c] - step * a.ad[6 * s + c];
                a.r[6 * s + c] = rr[c];
                rr2 += rr[c] * rr[c];
            }
            matvec6(a.P + 36 * s, rr, zz);
#pragma unroll
            for (int c = 0; c < 6; ++c) {
                a.z[6 * s + c] = zz[c];
                rz1 += rr[c] * zz[c];
            }
            zmax = scaled_max(a, s, zz, zmax);
        }
        if (!reduce(rz1, rr2, zmax, a.barrier, a.status, tot)) return;
        rz1 = tot[0];
        if (it % 10 == 0) {
            relative = sqrt(tot[1]) / norm;
            if (a.mode == kLinear) {
                if (relative < a.tol) {
                    state = 0;
                    break;
                }
            } else if (relative < a.tol && tot[2] < 2e-8) {
                // true residual of the balanced test (x is complete after the last barrier)
                if (!sweep_bonds(a, a.x, tid, stride)) return;
                double e2 = 0.0, emax = 0.0;
                for (int64_t s = tid; s < n; s += stride) {
                    double b6[6], ax[6], res[6], pr[6];
                    rhs_site(a, s, b6);
                    operator_site(a.A, a.x, s, ax);
#pragma unroll
                    for (int c = 0; c < 6; ++c) {
                        res[c] = b6[c] - ax[c];
                        e2 += res[c] * res[c];
                    }
                    matvec6(a.P + 36 * s, res, pr);
                    emax = scaled_max(a, s, pr, emax);
                }
                double tr[3];
                if (!reduce(e2, 0.0, emax, a.barrier, a.status, tr)) return;
                const double actual = sqrt(tr[0]) / norm;
                if (actual < 5.0 * a.tol && tr[2] < 1e-7) {
                    relative = actual;
                    state = 0;
                    break;
                }
            }
            if (!isfinite(relative)) {
                state = 2;
                break;
            }
        }
        const double beta = block_divide(rz1, rz);
        for (int64_t e = tid; e < 6 * n; e += stride) a.d[e] = a.z[e] + beta * a.d[e];
        rz = rz1;
        if (!grid_barrier(a.barrier, a.status)) return;
    }
    const int iterations = it < a.max_it ? it + 1 : a.max_it;
    if (a.mode == kLinear && state != 2) {
        if (!sweep_bonds(a, a.x, tid, stride)) return;
        double e2 = 0.0;
        for (int64_t s = tid; s < n; s += stride) {
            double b6[6], ax[6];
            rhs_site(a, s, b6);
            operator_site(a.A, a.x, s, ax);
#pragma unroll
            for (int c = 0; c < 6; ++c) e2 += (b6[c] - ax[c]) * (b6[c] - ax[c]);
        }
        if (!reduce(e2, 0.0, 0.0, a.barrier, a.status, tot)) return;
        relative = sqrt(tot[0]) / norm;
    }
    if (tid == 0) {
        a.info[0] = (double)iterations;
        a.info[1] = relative;
        a.info[2] = (double)state;
        a.info[3] = norm;
    }
}

// ---------------------------------------------------------------------------
// Block preconditioner of the linear solves: B = diag M + alpha D per site
// (the identity on fixed sites) and P = B^-1 by the register Cholesky
// inverse (bonded_dem_linear_gpu.py:82-86, bonded_dem_finite_gpu.py:141-143).
__global__ void __launch_bounds__(128) block_inverse_kernel(int64_t n, const double *mass, const uint8_t *fixed,
                                                            const double *diagonal, double alpha, double *block,
                                                            double *P) {
    const int64_t s = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (s >= n) return;
    double B[36], Pi[36];
    const bool fx = fixed[s] != 0;
#pragma unroll
    for (int e = 0; e < 36; ++e) {
        const int row = e / 6, col = e % 6;
        const double eye = row == col ? 1.0 : 0.0;
        B[e] = fx ? eye : eye * mass[6 * s + row] + alpha * diagonal[36 * s + e];
    }
    spd_inverse6(B, Pi);
#pragma unroll
    for (int e = 0; e < 36; ++e) {
        if (block) block[36 * s + e] = B[e];
        P[36 * s + e] = Pi[e];
    }
}

// ---------------------------------------------------------------------------
// Linear implicit midpoint (bonded_dem_linear_gpu.py:114-121):
//   rhs = dt M v + dt^2/2 (external - K q),  guess = dt v;
//   after the solve: v <- 2 dq / dt - v,  q <- q + dq.

__global__ void __launch_bounds__(kThreads) linear_rhs_kernel(int64_t len, const double *mass, const double *v,
                                                              const double *external, const double *kq, double dt,
                                                              double *rhs, double *guess) {
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    const double h = 0.5 * dt * dt;
    for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < len; e += stride) {
        rhs[e] = dt * mass[e] * v[e] + h * (external[e] - kq[e]);
        guess[e] = dt * v[e];
    }
}

__global__ void __launch_bounds__(kThreads) linear_advance_kernel(int64_t len, const double *dq, double dt, double *v,
                                                                  double *q) {
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < len; e += stride) {
        v[e] = 2.0 * dq[e] / dt - v[e];
        q[e] += dq[e];
    }
}

// [sum a.b, 1/2 (sum m v^2 + sum q kq)] with the "last block" protocol.
__global__ void __launch_bounds__(kThreads) pair_sums_kernel(int64_t len, const double *a, const double *b,
                                                             const double *mass, const double *v, const double *q,
                                                             const double *kq, double *out, double *partials) {
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    double ab = 0.0, en = 0.0;
    for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < len; e += stride) {
        if (a) ab += a[e] * b[e];
        if (mass) en += mass[e] * v[e] * v[e] + q[e] * kq[e];
    }
    ab = block_sum(ab);
    en = block_sum(en);
    double *part = partials + kCounter;
    if (threadIdx.x == 0) {
        part[2 * blockIdx.x] = ab;
        part[2 * blockIdx.x + 1] = en;
    }
    if (last_block(reinterpret_cast<unsigned *>(partials))) {
        const double s_ab = block_sum_array(part, gridDim.x, 2);
        const double s_en = block_sum_array(part + 1, gridDim.x, 2);
        if (threadIdx.x == 0) {
            out[0] = s_ab;
            out[1] = 0.5 * s_en;
        }
    }
}

// ---------------------------------------------------------------------------
// Anderson mixing over device history slots (bonded_dem_finite_gpu.py:215-229).
// Slots hold iterates y_k and corrections c_k as (N, 6) rows of two
// (slots, N, 6) arrays; order[0..count) lists the slots oldest first.  With
// dc_h = c_{h+1} - c_h and the weights u = [1, 1, 1, r, r, r]:
//   gram[h][l] = sum (u dc_h)(u dc_l),  proj[h] = sum (u dc_h)(u c_last).

struct History {
    const double *y, *c;
    int64_t ld;  // doubles per slot (6 N)
    int order[kMaxHistory];
    int count;
};

__global__ void __launch_bounds__(kThreads) anderson_gram_kernel(int64_t n, History H, const double *radii,
                                                                 double *out, double *partials) {
    constexpr int kPairs = (kMaxHistory - 1) * kMaxHistory / 2;
    const int dh = H.count - 1;
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    double acc[kPairs + kMaxHistory - 1];
    const int terms = dh * (dh + 1) / 2 + dh;
    for (int k = 0; k < terms; ++k) acc[k] = 0.0;
    const double *last = H.c + (int64_t)H.order[H.count - 1] * H.ld;
    for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < 6 * n; e += stride) {
        const double u = (e % 6) < 3 ? 1.0 : radii[e / 6];
        double w[kMaxHistory - 1];
        for (int h = 0; h < dh; ++h)
            w[h] = u * (H.c[(int64_t)H.order[h + 1] * H.ld + e] - H.c[(int64_t)H.order[h] * H.ld + e]);
        const double cl = u * last[e];
        int k = 0;
        for (int h = 0; h < dh; ++h)
            for (int l = h; l < dh; ++l) acc[k++] += w[h] * w[l];
        for (int h = 0; h < dh; ++h) acc[k++] += w[h] * cl;
    }
    double *part = partials + kCounter;
    for (int k = 0; k < terms; ++k) {
        const double v = block_sum(acc[k]);
        if (threadIdx.x == 0) part[(int64_t)k * gridDim.x + blockIdx.x] = v;
    }
    if (last_block(reinterpret_cast<unsigned *>(partials) + 1)) {
        for (int k = 0; k < terms; ++k) {
            const double v = block_sum_array(part + (int64_t)k * gridDim.x, gridDim.x);
            if (threadIdx.x == 0) out[k] = v;
        }
    }
}

struct Coefficients {
    double c[kMaxHistory];
};

// out = c_last - sum_h coef_h (dy_h + dc_h); flag[0] = 1 if any entry is not finite.
__global__ void __launch_bounds__(kThreads) anderson_mix_kernel(int64_t len, History H, Coefficients coef,
                                                                double *out, int *flag) {
    const int dh = H.count - 1;
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    const double *last = H.c + (int64_t)H.order[H.count - 1] * H.ld;
    bool bad = false;
    for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < len; e += stride) {
        double v = last[e];
        for (int h = 0; h < dh; ++h) {
            const int64_t a = (int64_t)H.order[h] * H.ld + e, b = (int64_t)H.order[h + 1] * H.ld + e;
            v -= coef.c[h] * ((H.y[b] + H.c[b]) - (H.y[a] + H.c[a]));
        }
        out[e] = v;
        bad |= !isfinite(v);
    }
    if (bad) atomicOr(flag, 1);
}

// ---------------------------------------------------------------------------
// Self-test of the bounded grid barrier: every block waits for `parties`
// arrivals; with parties above the grid size nobody releases the barrier and
// each wait gives up after timeout_ns, setting DPF_ERR_BARRIER_TIMEOUT.
__global__ void barrier_selftest_kernel(unsigned *barrier, int *status, unsigned long long timeout_ns,
                                        unsigned parties, int *passed) {
    if (grid_barrier(barrier, status, timeout_ns, parties) && threadIdx.x == 0) atomicAdd(passed, 1);
}

struct DeviceInfo {
    int sms = 0, per_sm = 0;
};

DeviceInfo &device_info() {
    static DeviceInfo info[64];
    int dev = 0;
    cudaGetDevice(&dev);
    DeviceInfo &d = info[dev & 63];
    if (d.sms == 0) {
        cudaDeviceGetAttribute(&d.sms, cudaDevAttrMultiProcessorCount, dev);
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&d.per_sm, block_pcg_kernel, kThreads, 0);
    }
    return d;
}

bool graph_ok(const dpf_graph *g) {
    return g && g->n_sites > 0 && g->n_bonds >= 0 && g->n_bonds < (int64_t(1) << 31) && g->inc_ptr &&
           (g->n_bonds == 0 || (g->edges && g->inc_bond));
}

Operator make_operator(const dpf_graph *g, const dpf_stiffness *k, const dpf_tangent *t, const double *mass,
                       const uint8_t *fixed, double alpha, double *wrench) {
    return Operator{g->n_sites, g->n_bonds, g->inc_ptr, g->inc_bond, g->edges, *k, *t, mass, fixed, alpha, wrench};
}

bool history_ok(const double *y, const double *c, int64_t n, int slots, const int32_t *order, int count) {
    if (!y || !c || !order || n <= 0 || slots < 1 || slots > kMaxHistory || count < 2 || count > slots) return false;
    for (int h = 0; h < count; ++h)
        if (order[h] < 0 || order[h] >= slots) return false;
    return true;
}

History make_history(const double *y, const double *c, int64_t n, const int32_t *order, int count) {
    History H{};
    H.y = y;
    H.c = c;
    H.ld = 6 * n;
    H.count = count;
    for (int h = 0; h < count; ++h) H.order[h] = order[h];
    return H;
}

}  // namespace lin
}  // namespace dpf

using namespace dpf;
using namespace dpf::lin;

extern "C" {

int dpf_operator_apply(const dpf_graph *g, const dpf_stiffness *k, const dpf_tangent *t, const double *mass,
                       const uint8_t *fixed, double alpha, const double *q, double *out, double *wrench,
                       void *stream) {
    if (!graph_ok(g) || !k || !t || !mass || !fixed || !q || !out || (g->n_bonds && !wrench))
        return DPF_ERR_ARGUMENT;
    cudaStream_t st = (cudaStream_t)stream;
    const Operator A = make_operator(g, k, t, mass, fixed, alpha, wrench);
    if (g->n_bonds) operator_bonds<<<blocks_for(g->n_bonds, kThreads), kThreads, 0, st>>>(A, q);
    operator_sites<<<blocks_for(g->n_sites, kThreads), kThreads, 0, st>>>(A, q, out);
    DPF_CHECK_LAUNCH();
    return DPF_OK;
}

int dpf_block_inverse(int64_t n_sites, const double *mass, const uint8_t *fixed, const double *diagonal, double alpha,
                      double *block, double *preconditioner, void *stream) {
    if (n_sites <= 0 || !mass || !fixed || !diagonal || !preconditioner) return DPF_ERR_ARGUMENT;
    block_inverse_kernel<<<blocks_for(n_sites, 128), 128, 0, (cudaStream_t)stream>>>(n_sites, mass, fixed, diagonal,
                                                                                     alpha, block, preconditioner);
    DPF_CHECK_LAUNCH();
    return DPF_OK;
}

int64_t dpf_block_pcg_workspace_doubles(int64_t n_sites) { return 24 * n_sites + 6 * (int64_t)kMaxBlocks; }

int dpf_block_pcg(const dpf_graph *g, const dpf_stiffness *k, const dpf_tangent *t, const double *mass,
                  const uint8_t *fixed, const double *preconditioner, const double *scale, const double *rhs,
                  double alpha, double tolerance, int max_iterations, int mode, int use_guess, double *x,
                  double *info, double *wrench, double *workspace, unsigned *barrier, int *status, void *stream) {
    if (!graph_ok(g) || !k || !t || !mass || !fixed || !preconditioner || !rhs || !x || !info || !workspace ||
        !barrier || !status || (g->n_bonds && !wrench) || max_iterations < 1 || (mode != kLinear && mode != kBalanced) ||
        (mode == kBalanced && !scale) || !(tolerance >= 0.0))
        return DPF_ERR_ARGUMENT;
    cudaStream_t st = (cudaStream_t)stream;
    DeviceInfo &info_d = device_info();
    if (info_d.sms <= 0 || info_d.per_sm <= 0) return DPF_ERR_CUDA;
    const int64_t work = g->n_sites > g->n_bonds ? g->n_sites : g->n_bonds;
    int64_t cap = (int64_t)info_d.sms * info_d.per_sm;
    if (cap > kMaxBlocks) cap = kMaxBlocks;
    int64_t want = blocks_for(work, kThreads);
    const int grid = (int)(want < cap ? (want < 1 ? 1 : want) : cap);
    const int64_t n6 = 6 * g->n_sites;
    BlockPcgArgs a{};
    a.A = make_operator(g, k, t, mass, fixed, alpha, wrench);
    a.P = preconditioner;
    a.scale = scale;
    a.rhs = rhs;
    a.tol = tolerance;
    a.zero_norm = mode == kLinear ? 1e-30 : 1e-40;
    a.max_it = max_iterations;
    a.mode = mode;
    a.use_guess = use_guess ? 1 : 0;
    a.x = x;
    a.info = info;
    a.r = workspace;
    a.z = workspace + n6;
    a.d = workspace + 2 * n6;
    a.ad = workspace + 3 * n6;
    a.part = workspace + 4 * n6;
    a.barrier = barrier;
    a.status = status;
    if (cudaMemsetAsync(barrier, 0, 2 * sizeof(unsigned), st) != cudaSuccess) {
        cudaGetLastError();
        return DPF_ERR_CUDA;
    }
    void *args[] = {&a};
    if (cudaLaunchCooperativeKernel((const void *)block_pcg_kernel, grid, kThreads, args, 0, st) != cudaSuccess) {
        cudaGetLastError();
        return DPF_ERR_CUDA;
    }
    return DPF_OK;
}

int dpf_linear_midpoint_rhs(int64_t n_sites, const double *mass, const double *v, const double *external,
                            const double *kq, double dt, double *rhs, double *guess, void *stream) {
    if (n_sites <= 0 || !mass || !v || !external || !kq || !rhs || !guess || !(dt > 0.0)) return DPF_ERR_ARGUMENT;
    linear_rhs_kernel<<<reduce_grid(6 * n_sites), kThreads, 0, (cudaStream_t)stream>>>(6 * n_sites, mass, v, external,
                                                                                       kq, dt, rhs, guess);
    DPF_CHECK_LAUNCH();
    return DPF_OK;
}

int dpf_linear_midpoint_advance(int64_t n_sites, const double *dq, double dt, double *v, double *q, void *stream) {
    if (n_sites <= 0 || !dq || !v || !q || !(dt > 0.0)) return DPF_ERR_ARGUMENT;
    linear_advance_kernel<<<reduce_grid(6 * n_sites), kThreads, 0, (cudaStream_t)stream>>>(6 * n_sites, dq, dt, v,
                                                                                           q);
    DPF_CHECK_LAUNCH();
    return DPF_OK;
}

int64_t dpf_small_partials_doubles(void) { return kCounter + 64 * 1024; }

int dpf_linear_sums(int64_t n_sites, const double *a, const double *b, const double *mass, const double *v,
                    const double *q, const double *kq, double *out, double *partials, void *stream) {
    if (n_sites <= 0 || !out || !partials || (a && !b) || (mass && (!v || !q || !kq)) || (!a && !mass))
        return DPF_ERR_ARGUMENT;
    pair_sums_kernel<<<reduce_grid(6 * n_sites), kThreads, 0, (cudaStream_t)stream>>>(6 * n_sites, a, b, mass, v, q,
                                                                                      kq, out, partials);
    DPF_CHECK_LAUNCH();
    return DPF_OK;
}

int dpf_anderson_gram(int64_t n_sites, const double *iterates, const double *corrections, int slots,
                      const int32_t *order, int count, const double *radii, double *out, double *partials,
                      void *stream) {
    if (!history_ok(iterates, corrections, n_sites, slots, order, count) || !radii || !out || !partials)
        return DPF_ERR_ARGUMENT;
    // one reduction term per block row: keep the grid within the partials' rows
    const int dh = count - 1, terms = dh * (dh + 1) / 2 + dh;
    int grid = reduce_grid(6 * n_sites);
    if ((int64_t)terms * grid > 64 * 1024) grid = (64 * 1024) / terms;
    anderson_gram_kernel<<<grid, kThreads, 0, (cudaStream_t)stream>>>(
        n_sites, make_history(iterates, corrections, n_sites, order, count), radii, out, partials);
    DPF_CHECK_LAUNCH();
    return DPF_OK;
}

int dpf_anderson_mix(int64_t n_sites, const double *iterates, const double *corrections, int slots,
                     const int32_t *order, int count, const double *coefficients, double *out, int *flag,
                     void *stream) {
    if (!history_ok(iterates, corrections, n_sites, slots, order, count) || !coefficients || !out || !flag)
        return DPF_ERR_ARGUMENT;
    Coefficients c{};
    for (int h = 0; h < count - 1; ++h) c.c[h] = coefficients[h];
    anderson_mix_kernel<<<reduce_grid(6 * n_sites), kThreads, 0, (cudaStream_t)stream>>>(
        6 * n_sites, make_history(iterates, corrections, n_sites, order, count), c, out, flag);
    DPF_CHECK_LAUNCH();
    return DPF_OK;
}

int dpf_barrier_selftest(int blocks, int64_t timeout_ns, int missing, unsigned *barrier, int *status, int *passed,
                         void *stream) {
    if (blocks < 1 || blocks > 64 || timeout_ns <= 0 || timeout_ns > 2000000000LL || missing < 0 || missing > 64 ||
        !barrier || !status || !passed)
        return DPF_ERR_ARGUMENT;
    cudaStream_t st = (cudaStream_t)stream;
    if (cudaMemsetAsync(barrier, 0, 2 * sizeof(unsigned), st) != cudaSuccess) {
        cudaGetLastError();
        return DPF_ERR_CUDA;
    }
    void *args[5];
    unsigned long long t = (unsigned long long)timeout_ns;
    unsigned parties = (unsigned)(blocks + missing);
    args[0] = &barrier;
    args[1] = &status;
    args[2] = &t;
    args[3] = &parties;
    args[4] = &passed;
    if (cudaLaunchCooperativeKernel((const void *)barrier_selftest_kernel, blocks, 32, args, 0, st) != cudaSuccess) {
        cudaGetLastError();
        return DPF_ERR_CUDA;
    }
    return DPF_OK;
}

}  // extern "C"
