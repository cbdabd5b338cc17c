// Parallel-bond component with brittle failure (experiments/bonded_dem_core.py:45-208),
// float64: one thread per bond integrates the midpoint rate law (shortest-arc
// transports of the shear force and bending couple to the midpoint frame and
// on to the end frame, rotation about the normal by the average spin), tests
// the tensile and shear strengths, and writes the bond's new history to
// separate output arrays, so a step rejected by a guard leaves the committed
// state untouched.  Work, elastic energy, removed (broken-bond) energy and
// the number of newly broken bonds are summed per block and then over blocks
// in a fixed order; loads are gathered per site over the incidence CSR.
#include "common.cuh"

namespace dpf {
namespace core {

constexpr int kMaxBlocks = 4096;
constexpr int kSums = 4;  // work, elastic energy, removed energy, newly broken

struct AdvanceArgs {
    int64_t n, m;
    const int64_t *edges;
    dpf_parallel_params p;
    const double *radii, *x, *end, *mid, *v, *w;
    double dt;
    dpf_parallel_state in, out;
    double *partials;
    int *status;
};

__device__ __forceinline__ d3 midpoint(const AdvanceArgs &a, int64_t s) {
    return a.mid ? ld3(a.mid, s) : 0.5 * (ld3(a.x, s) + ld3(a.end, s));
}

__global__ void __launch_bounds__(kThreads) advance_kernel(AdvanceArgs a) {
    int flags = 0;
    double sums[kSums] = {0.0, 0.0, 0.0, 0.0};
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    const int64_t tid = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    // body rotation guard (bonded_dem_core.py:171-172)
    for (int64_t s = tid; s < a.n; s += stride)
        if (norm(ld3(a.w, s)) * a.dt > 0.25) flags |= DPF_ERR_ROTATION;
    for (int64_t b = tid; b < a.m; b += stride) {
        int64_t i, j;
        edge(a.edges, b, i, j);
        const d3 mi = midpoint(a, i), mj = midpoint(a, j);
        const d3 dm = mj - mi;
        const double lm = norm(dm);
        if (lm <= 1e-12) flags |= DPF_ERR_COINCIDENT;
        const d3 nm = dm / lm;
        const d3 contact = 0.5 * (mi + mj) + (0.5 * (a.radii[i] - a.radii[j])) * nm;
        const d3 de = ld3(a.end, j) - ld3(a.end, i);
        const double le = norm(de);
        if (le <= 1e-12) flags |= DPF_ERR_COINCIDENT;
        const d3 ne = de / le;
        const d3 wi = ld3(a.w, i), wj = ld3(a.w, j);
        const d3 half = (0.25 * a.dt) * (wi + wj);
        const Transport to_mid = make_transport(ld3(a.in.normal, b), nm, half, flags);
        const Transport to_end = make_transport(nm, ne, half, flags);
        const d3 fs0 = apply(to_mid, ld3(a.in.fs, b)), mb0 = apply(to_mid, ld3(a.in.mb, b));
        const d3 du = a.dt * (ld3(a.v, j) + cross(wj, contact - mj) - ld3(a.v, i) - cross(wi, contact - mi));
        const d3 dth = a.dt * (wj - wi);
        const bool intact = a.in.failure[b] == 0;
        const double on = intact ? 1.0 : 0.0;
        const double dun = dot(du, nm), dthn = dot(dth, nm);
        const double dn = on * dun, tw = on * dthn;
        const d3 ds = on * (du - dun * nm), bend = on * (dth - dthn * nm);
        const double kn = a.p.kn[b], ks = a.p.ks[b], kb = a.p.kb[b], kt = a.p.kt[b];
        const double fn_old = a.in.fn[b], mt_old = a.in.mt[b];
        double fn = fn_old + kn * dn, mt = mt_old + kt * tw;
        d3 fs = fs0 + ks * ds, mb = mb0 + kb * bend;
        sums[0] += 0.5 * ((fn_old + fn) * dn + dot(fs0 + fs, ds) + (mt_old + mt) * tw + dot(mb0 + mb, bend));
        const double A = a.p.area[b], I = a.p.second_moment[b], J = a.p.polar_moment[b], rb = a.p.radius[b];
        const double sigma = fn / A + a.p.beta * norm(mb) * rb / I;
        const double tau = norm(fs) / A + a.p.beta * fabs(mt) * rb / J;
        const bool tensile = intact && sigma > a.p.tensile[b];
        const bool shear = intact && !tensile && tau > a.p.cohesion[b] - fn / A * a.p.tan_phi;
        double removed = a.in.break_energy[b];
        int8_t failure = a.in.failure[b];
        if (tensile || shear) {
            removed += 0.5 * (fn * fn / kn + dot(fs, fs) / ks + mt * mt / kt + dot(mb, mb) / kb);
            failure = tensile ? 1 : 2;
            fn = mt = 0.0;
            fs = mk(0.0, 0.0, 0.0);
            mb = mk(0.0, 0.0, 0.0);
            sums[3] += 1.0;
        }
        const d3 fs_end = apply(to_end, fs), mb_end = apply(to_end, mb);
        a.out.fn[b] = fn;
        a.out.mt[b] = mt;
        st3(a.out.fs, b, fs_end);
        st3(a.out.mb, b, mb_end);
        st3(a.out.normal, b, ne);
        a.out.failure[b] = failure;
        a.out.break_energy[b] = removed;
        sums[1] += 0.5 * (fn * fn / kn + dot(fs_end, fs_end) / ks + mt * mt / kt + dot(mb_end, mb_end) / kb);
        sums[2] += removed;
    }
    if (flags) atomicOr(a.status, flags);
#pragma unroll
    for (int k = 0; k < kSums; ++k) {
        const double s = block_sum(sums[k]);
        if (threadIdx.x == 0) a.partials[kSums * blockIdx.x + k] = s;
    }
}

__global__ void __launch_bounds__(kThreads) sums_kernel(int blocks, const double *partials, double *out) {
#pragma unroll
    for (int k = 0; k < kSums; ++k) {
        const double s = block_sum_array(partials + k, blocks, kSums);
        if (threadIdx.x == 0) out[k] = s;
    }
}

// Bond loads about the centres (bonded_dem_core.py:132-142): W = [f, (c - x_i) x f
// + couple, -(c - x_j) x f - couple]; site i adds (f, T_i), site j (-f, T_j).
__global__ void __launch_bounds__(kThreads) load_bonds_kernel(int64_t m, const int64_t *edges, const double *radii,
                                                              const double *x, const double *fn, const double *fs,
                                                              const double *mt, const double *mb, double *wrench,
                                                              int *status) {
    const int64_t b = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (b >= m) return;
    int64_t i, j;
    edge(edges, b, i, j);
    const d3 xi = ld3(x, i), xj = ld3(x, j);
    const d3 d = xj - xi;
    const double l = norm(d);
    if (l <= 1e-12) atomicOr(status, DPF_ERR_COINCIDENT);
    const d3 n = d / l;
    const d3 c = 0.5 * (xi + xj) + (0.5 * (radii[i] - radii[j])) * n;
    const d3 f = fn[b] * n + ld3(fs, b);
    const d3 couple = mt[b] * n + ld3(mb, b);
    double *w = wrench + 9 * b;
    st3(w, f);
    st3(w + 3, cross(c - xi, f) + couple);
    st3(w + 6, -cross(c - xj, f) - couple);
}

__global__ void __launch_bounds__(kThreads) load_sites_kernel(int64_t n, const int32_t *ptr, const int32_t *inc,
                                                              const double *w, double *force, double *torque) {
    const int64_t s = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (s >= n) return;
    double f[3] = {0.0, 0.0, 0.0}, t[3] = {0.0, 0.0, 0.0};
    const int e1 = ptr[s + 1];
    for (int e = ptr[s]; e < e1; ++e) {
        const int v = inc[e];
        const double *p = w + 9 * (int64_t)(v >= 0 ? v : ~v);
        const double sg = v >= 0 ? 1.0 : -1.0;
        const int off = v >= 0 ? 3 : 6;
#pragma unroll
        for (int c = 0; c < 3; ++c) {
            f[c] += sg * p[c];
            t[c] += p[off + c];
        }
    }
#pragma unroll
    for (int c = 0; c < 3; ++c) {
        force[3 * s + c] = f[c];
        torque[3 * s + c] = t[c];
    }
}

inline int grid_for(int64_t n) {
    const int64_t want = (n + kThreads - 1) / kThreads;
    return (int)(want < 1 ? 1 : (want < kMaxBlocks ? want : kMaxBlocks));
}

bool params_ok(const dpf_parallel_params *p) {
    return p && p->kn && p->ks && p->kb && p->kt && p->area && p->second_moment && p->polar_moment && p->radius &&
           p->tensile && p->cohesion;
}

bool state_ok(const dpf_parallel_state *s) {
    return s && s->normal && s->fn && s->fs && s->mt && s->mb && s->break_energy && s->failure;
}

}  // namespace core
}  // namespace dpf

using namespace dpf;
using namespace dpf::core;

extern "C" {

int64_t dpf_parallel_partials_doubles(void) { return (int64_t)kSums * kMaxBlocks; }

int dpf_parallel_advance(const dpf_graph *g, const dpf_parallel_params *p, const double *radii, const double *x,
                         const double *end, const double *mid, const double *v, const double *w, double dt,
                         const dpf_parallel_state *in, const dpf_parallel_state *out, double *sums,
                         double *partials, int *status, void *stream) {
    if (!g || g->n_sites <= 0 || g->n_bonds <= 0 || !g->edges || !params_ok(p) || !radii || !x || !end || !v ||
        !w || !state_ok(in) || !state_ok(out) || !sums || !partials || !status || !(dt > 0.0))
        return DPF_ERR_ARGUMENT;
    cudaStream_t st = (cudaStream_t)stream;
    const int grid = grid_for(g->n_bonds > g->n_sites ? g->n_bonds : g->n_sites);
    AdvanceArgs a{g->n_sites, g->n_bonds, g->edges, *p, radii, x, end, mid, v, w, dt, *in, *out, partials, status};
    advance_kernel<<<grid, kThreads, 0, st>>>(a);
    sums_kernel<<<1, kThreads, 0, st>>>(grid, partials, sums);
    DPF_CHECK_LAUNCH();
    return DPF_OK;
}

int dpf_parallel_loads(const dpf_graph *g, const double *radii, const double *x, const double *fn, const double *fs,
                       const double *mt, const double *mb, double *force, double *torque, double *wrench,
                       int *status, void *stream) {
    if (!g || g->n_sites <= 0 || !g->inc_ptr || (g->n_bonds && !g->inc_bond) || !radii || !x || !force ||
        !torque || !status ||
        (g->n_bonds && (!g->edges || !fn || !fs || !mt || !mb || !wrench)))
        return DPF_ERR_ARGUMENT;
    cudaStream_t st = (cudaStream_t)stream;
    if (g->n_bonds)
        load_bonds_kernel<<<(int)((g->n_bonds + kThreads - 1) / kThreads), kThreads, 0, st>>>(
            g->n_bonds, g->edges, radii, x, fn, fs, mt, mb, wrench, status);
    load_sites_kernel<<<(int)((g->n_sites + kThreads - 1) / kThreads), kThreads, 0, st>>>(
        g->n_sites, g->inc_ptr, g->inc_bond, wrench, force, torque);
    DPF_CHECK_LAUNCH();
    return DPF_OK;
}

}  // extern "C"
