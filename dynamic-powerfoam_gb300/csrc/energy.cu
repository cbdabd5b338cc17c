// Bond energy law of the energy-based foam (experiments/foam_dem_energy.py,
// EnergyFoam with volume=False, kinematics='small'): per bond, with body
// rotations R = R(q) (unit quaternions w, x, y, z) and rest levers r_i, r_j,
//   D = x_j + R_j r_j - x_i - R_i r_i,   d = (R_i^T D + R_j^T D) / 2,
//   phi = axial(R_i^T R_j - R_j^T R_i) / 2,  k = k0 exp((theta_i + theta_j) / 2),
//   E = kn dn^2/2 + ks |d_t|^2/2 + kb |phi_t|^2/2 + kt phi_n^2/2  (n0 components),
// and the closed-form force and world torque (foam_dem_energy.py:797-811).
// One thread per bond writes the bond's wrench [a, -t_i, -t_j]; the site pass
// sums them over the incidence CSR in its fixed order; the energy is summed
// per block and then over blocks in a fixed order (deterministic).
#include "common.cuh"

namespace dpf {
namespace energy {

constexpr int kMaxBlocks = 4096;

struct M3 {
    d3 r0, r1, r2;  // rows
};

__device__ __forceinline__ M3 quat_matrix(const double *q) {
    const double w = q[0], x = q[1], y = q[2], z = q[3];
    return M3{mk(1 - 2 * (y * y + z * z), 2 * (x * y - w * z), 2 * (x * z + w * y)),
              mk(2 * (x * y + w * z), 1 - 2 * (x * x + z * z), 2 * (y * z - w * x)),
              mk(2 * (x * z - w * y), 2 * (y * z + w * x), 1 - 2 * (x * x + y * y))};
}
__device__ __forceinline__ d3 mul(const M3 &R, d3 v) { return mk(dot(R.r0, v), dot(R.r1, v), dot(R.r2, v)); }
// R^T v
__device__ __forceinline__ d3 tmul(const M3 &R, d3 v) { return v.x * R.r0 + v.y * R.r1 + v.z * R.r2; }
__device__ __forceinline__ d3 col(const M3 &R, int c) {
    return c == 0 ? mk(R.r0.x, R.r1.x, R.r2.x) : c == 1 ? mk(R.r0.y, R.r1.y, R.r2.y) : mk(R.r0.z, R.r1.z, R.r2.z);
}

struct BondArgs {
    int64_t m;
    const int64_t *edges;
    const double *base, *theta;
    int64_t theta_stride;
    const double *x, *q, *n0, *ri, *rj;
    double *wrench;    // 9 per bond or null
    double *partials;  // per-block energy sums or null
};

__global__ void __launch_bounds__(kThreads) bond_energy_kernel(BondArgs a) {
    double e_sum = 0.0;
    for (int64_t b = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; b < a.m; b += (int64_t)gridDim.x * blockDim.x) {
        int64_t i, j;
        edge(a.edges, b, i, j);
        const M3 Ri = quat_matrix(a.q + 4 * i), Rj = quat_matrix(a.q + 4 * j);
        const d3 pi = mul(Ri, ld3(a.ri, b)), pj = mul(Rj, ld3(a.rj, b));
        const d3 D = ld3(a.x, j) + pj - ld3(a.x, i) - pi;
        const d3 d = 0.5 * (tmul(Ri, D) + tmul(Rj, D));
        // Psi = R_i^T R_j: Psi[r][c] = col_r(R_i) . col_c(R_j)
        const d3 ci0 = col(Ri, 0), ci1 = col(Ri, 1), ci2 = col(Ri, 2);
        const d3 cj0 = col(Rj, 0), cj1 = col(Rj, 1), cj2 = col(Rj, 2);
        const double P00 = dot(ci0, cj0), P01 = dot(ci0, cj1), P02 = dot(ci0, cj2);
        const double P10 = dot(ci1, cj0), P11 = dot(ci1, cj1), P12 = dot(ci1, cj2);
        const double P20 = dot(ci2, cj0), P21 = dot(ci2, cj1), P22 = dot(ci2, cj2);
        const d3 phi = mk(0.5 * (P21 - P12), 0.5 * (P02 - P20), 0.5 * (P10 - P01));
        const d3 n0 = ld3(a.n0, b);
        const double *ti = a.theta + a.theta_stride * i, *tj = a.theta + a.theta_stride * j;
        const double *k0 = a.base + 4 * b;
        const double kn = k0[0] * exp(0.5 * (ti[0] + tj[0])), ks = k0[1] * exp(0.5 * (ti[1] + tj[1]));
        const double kb = k0[2] * exp(0.5 * (ti[2] + tj[2])), kt = k0[3] * exp(0.5 * (ti[3] + tj[3]));
        const double dn = dot(d, n0), pn = dot(phi, n0);
        const d3 dt = d - dn * n0, pt = phi - pn * n0;
        e_sum += 0.5 * kn * dn * dn + 0.5 * (ks * dot(dt, dt) + kb * dot(pt, pt) + kt * pn * pn);
        if (a.wrench) {
            const d3 gd = (kn * dn) * n0 + ks * dt, gp = (kt * pn) * n0 + kb * pt;
            const d3 Rgi = mul(Ri, gd), Rgj = mul(Rj, gd);
            const d3 av = 0.5 * (Rgi + Rgj);
            const double trace = P00 + P11 + P22;
            // M = (tr Psi gp - Psi^T gp) / 2
            const d3 PTgp = mk(P00 * gp.x + P10 * gp.y + P20 * gp.z, P01 * gp.x + P11 * gp.y + P21 * gp.z,
                               P02 * gp.x + P12 * gp.y + P22 * gp.z);
            const d3 Mv = 0.5 * (trace * gp - PTgp);
            const d3 T = mul(Ri, Mv);
            const d3 tjv = cross(pj, av) - 0.5 * cross(D, Rgj) + T;
            const d3 tiv = -cross(pi, av) - 0.5 * cross(D, Rgi) - T;
            double *w = a.wrench + 9 * b;
            st3(w, av);
            st3(w + 3, -tiv);
            st3(w + 6, -tjv);
        }
    }
    if (a.partials) {
        const double s = block_sum(e_sum);
        if (threadIdx.x == 0) a.partials[blockIdx.x] = s;
    }
}

__global__ void __launch_bounds__(kThreads) sum_partials_kernel(int count, const double *partials, double *out) {
    const double s = block_sum_array(partials, count);
    if (threadIdx.x == 0) *out = s;
}

// f_s = sum of a over i ends minus a over j ends; tau_s = -t_i / -t_j terms.
__global__ void __launch_bounds__(kThreads) site_forces_kernel(int64_t n, const int32_t *ptr, const int32_t *inc,
                                                               const double *w, double *force, double *torque) {
    const int64_t s = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (s >= n) return;
    double f[3] = {0.0, 0.0, 0.0}, t[3] = {0.0, 0.0, 0.0};
    const int e1 = ptr[s + 1];
    for (int e = ptr[s]; e < e1; ++e) {
        const int v = inc[e];
        if (v >= 0) {
            const double *p = w + 9 * (int64_t)v;
#pragma unroll
            for (int c = 0; c < 3; ++c) {
                f[c] += p[c];
                t[c] += p[3 + c];
            }
        } else {
            const double *p = w + 9 * (int64_t)(~v);
#pragma unroll
            for (int c = 0; c < 3; ++c) {
                f[c] -= p[c];
                t[c] += p[6 + c];
            }
        }
    }
    if (force)
#pragma unroll
        for (int c = 0; c < 3; ++c) force[3 * s + c] = f[c];
    if (torque)
#pragma unroll
        for (int c = 0; c < 3; ++c) torque[3 * s + c] = t[c];
}

// Frozen tangent of the bond potential at the current configuration, for
// the Newton direction of the energy-law solver: the bond axis
// n = (x_j - x_i) / |x_j - x_i|, the current contact point c (the mean of the
// two body-attached contact points x_i + R_i r_i and x_j + R_j r_j), levers
// c - x_i and c - x_j (so that r_i - r_j = L n exactly), and the bond
// stiffnesses; written as the float32 tangent records (n, kn) (r_i, ks)
// (r_j, kb) (kt, 0, 0, 0) that the bond-end sweep and the 6x6 block scaling
// read.  At the reference configuration this is the stiffness of
// LinearBondsGPU, the exact Hessian of the potential there.
__global__ void __launch_bounds__(kThreads) energy_tangent_kernel(int64_t m, const int64_t *edges, const double *base,
                                                                  const double *theta, int64_t theta_stride,
                                                                  const double *x, const double *q, const double *ri0,
                                                                  const double *rj0, float4 *t0, float4 *t1, float4 *t2,
                                                                  float4 *t3) {
    const int64_t b = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (b >= m) return;
    int64_t i, j;
    edge(edges, b, i, j);
    const d3 xi = ld3(x, i), xj = ld3(x, j);
    const M3 Ri = quat_matrix(q + 4 * i), Rj = quat_matrix(q + 4 * j);
    const d3 c = 0.5 * ((xi + mul(Ri, ld3(ri0, b))) + (xj + mul(Rj, ld3(rj0, b))));
    const d3 d = xj - xi;
    const d3 n = d / norm(d);
    const d3 ri = c - xi, rj = c - xj;
    const double *ti = theta + theta_stride * i, *tj = theta + theta_stride * j;
    const double *k0 = base + 4 * b;
    const float kn = (float)(k0[0] * exp(0.5 * (ti[0] + tj[0]))), ks = (float)(k0[1] * exp(0.5 * (ti[1] + tj[1])));
    const float kb = (float)(k0[2] * exp(0.5 * (ti[2] + tj[2]))), kt = (float)(k0[3] * exp(0.5 * (ti[3] + tj[3])));
    t0[b] = make_float4((float)n.x, (float)n.y, (float)n.z, kn);
    t1[b] = make_float4((float)ri.x, (float)ri.y, (float)ri.z, ks);
    t2[b] = make_float4((float)rj.x, (float)rj.y, (float)rj.z, kb);
    t3[b] = make_float4(kt, 0.0f, 0.0f, 0.0f);
}

}  // namespace energy
}  // namespace dpf

using namespace dpf;
using namespace dpf::energy;

extern "C" {

int64_t dpf_energy_partials_doubles(void) { return kMaxBlocks; }

int dpf_bond_energy(const dpf_graph *g, const double *base, const double *theta, int64_t theta_stride,
                    const double *x, const double *q, const double *n0, const double *ri, const double *rj,
                    double *force, double *torque, double *energy, double *wrench, double *partials,
                    void *stream) {
    const bool want_forces = force || torque;
    if (!g || g->n_sites <= 0 || (g->n_bonds && (!g->edges || !base || !theta || !n0 || !ri || !rj)) || !x ||
        !q || theta_stride < 4 || (want_forces && (!g->inc_ptr || (g->n_bonds && (!g->inc_bond || !wrench)))) ||
        (energy && !partials) || (!want_forces && !energy))
        return DPF_ERR_ARGUMENT;
    cudaStream_t st = (cudaStream_t)stream;
    int grid = 1;
    if (g->n_bonds) {
        int64_t want = (g->n_bonds + kThreads - 1) / kThreads;
        grid = (int)(want < kMaxBlocks ? want : kMaxBlocks);
        BondArgs a{g->n_bonds, g->edges, base, theta, theta_stride, x, q, n0, ri, rj,
                   want_forces ? wrench : nullptr, energy ? partials : nullptr};
        bond_energy_kernel<<<grid, kThreads, 0, st>>>(a);
    } else if (energy) {
        cudaMemsetAsync(partials, 0, sizeof(double), st);
    }
    if (energy) sum_partials_kernel<<<1, kThreads, 0, st>>>(grid, partials, energy);
    if (want_forces)
        site_forces_kernel<<<(int)((g->n_sites + kThreads - 1) / kThreads), kThreads, 0, st>>>(
            g->n_sites, g->inc_ptr, g->inc_bond, wrench, force, torque);
    DPF_CHECK_LAUNCH();
    return DPF_OK;
}

int dpf_energy_tangent(const dpf_graph *g, const double *base, const double *theta, int64_t theta_stride,
                       const double *x, const double *q, const double *ri0, const double *rj0, float *bond_data,
                       void *stream) {
    if (!g || g->n_sites <= 0 || g->n_bonds < 0 || !x || !q || theta_stride < 4 ||
        (g->n_bonds && (!g->edges || !base || !theta || !ri0 || !rj0 || !bond_data)) ||
        ((uintptr_t)bond_data & 15u))
        return DPF_ERR_ARGUMENT;
    const int64_t m = g->n_bonds;
    if (m) {
        float4 *p = reinterpret_cast<float4 *>(bond_data);
        energy_tangent_kernel<<<(int)((m + kThreads - 1) / kThreads), kThreads, 0, (cudaStream_t)stream>>>(
            m, g->edges, base, theta, theta_stride, x, q, ri0, rj0, p + 7 * m, p + 8 * m, p + 9 * m, p + 10 * m);
    }
    DPF_CHECK_LAUNCH();
    return DPF_OK;
}

}  // extern "C"
