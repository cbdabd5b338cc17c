// Adjoint of the rate-law implicit step (implicit-function theorem).
//
// The per-bond constitutive trial (experiments/bonded_dem_finite_gpu.py:87-116:
// midpoint wrench and end-of-step history) is written once, templated on the
// scalar type; with a forward-mode dual number it yields one column of the
// bond's local Jacobian per pass.  From those columns:
//   * dpf_adjoint_local_jacobian stores B_b = d[F, T_i, T_j]/d[y_i, y_j] (9 x 12)
//     per bond, so J^T lambda costs one sparse transposed product;
//   * dpf_adjoint_apply_jt applies J^T (free rows) for the adjoint Krylov solve;
//   * dpf_adjoint_bond_vjp contracts output adjoints (wrench adjoints from a
//     site vector, end-history adjoints per bond) with every input column and
//     returns input adjoints per bond (history, stiffness) and per site
//     (increment, position), the latter by a deterministic incidence gather.
#include "common.cuh"

namespace dpf {
namespace adj {

struct DD {
    double v, d;
    DD() = default;
    __device__ constexpr DD(double value, double derivative = 0.0) : v(value), d(derivative) {}
};
__device__ __forceinline__ DD operator+(DD a, DD b) { return {a.v + b.v, a.d + b.d}; }
__device__ __forceinline__ DD operator-(DD a, DD b) { return {a.v - b.v, a.d - b.d}; }
__device__ __forceinline__ DD operator-(DD a) { return {-a.v, -a.d}; }
__device__ __forceinline__ DD operator*(DD a, DD b) { return {a.v * b.v, fma(a.d, b.v, a.v * b.d)}; }
__device__ __forceinline__ DD operator*(double s, DD a) { return {s * a.v, s * a.d}; }
__device__ __forceinline__ DD operator/(DD a, DD b) {
    const double inv = 1.0 / b.v, q = a.v * inv;
    return {q, (a.d - q * b.d) * inv};
}
__device__ __forceinline__ DD operator+(DD a, double b) { return {a.v + b, a.d}; }
__device__ __forceinline__ DD operator+(double b, DD a) { return {a.v + b, a.d}; }
__device__ __forceinline__ DD operator-(double b, DD a) { return {b - a.v, -a.d}; }
__device__ __forceinline__ DD dsqrt(DD a) {
    const double s = sqrt(a.v);
    return {s, a.d * 0.5 / s};
}
__device__ __forceinline__ double dsqrt(double a) { return sqrt(a); }
__device__ __forceinline__ void dsincos(DD a, DD &s, DD &c) {
    double sv, cv;
    sincos(a.v, &sv, &cv);
    s = {sv, cv * a.d};
    c = {cv, -sv * a.d};
}
__device__ __forceinline__ void dsincos(double a, double &s, double &c) { sincos(a, &s, &c); }
// clamp to [-1, 1]: derivative zero outside (torch's clamp derivative)
__device__ __forceinline__ DD dclamp1(DD a) {
    if (a.v < -1.0) return {-1.0, 0.0};
    if (a.v > 1.0) return {1.0, 0.0};
    return a;
}
__device__ __forceinline__ double dclamp1(double a) { return fmin(fmax(a, -1.0), 1.0); }
// max(a, eps): derivative of a when a > eps
__device__ __forceinline__ DD dmax(DD a, double e) { return a.v > e ? a : DD{e, 0.0}; }
__device__ __forceinline__ double dmax(double a, double e) { return fmax(a, e); }
__device__ __forceinline__ double val(DD a) { return a.v; }
__device__ __forceinline__ double val(double a) { return a; }

template <class S>
struct W3 {
    S x, y, z;
};
template <class S>
__device__ __forceinline__ W3<S> operator+(W3<S> a, W3<S> b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
template <class S>
__device__ __forceinline__ W3<S> operator-(W3<S> a, W3<S> b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
template <class S>
__device__ __forceinline__ W3<S> operator-(W3<S> a) { return {-a.x, -a.y, -a.z}; }
template <class S, class T>
__device__ __forceinline__ W3<S> operator*(T s, W3<S> a) { return {s * a.x, s * a.y, s * a.z}; }
template <class S>
__device__ __forceinline__ S wdot(W3<S> a, W3<S> b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
template <class S>
__device__ __forceinline__ W3<S> wcross(W3<S> a, W3<S> b) {
    return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x};
}
template <class S>
__device__ __forceinline__ W3<S> wdiv(W3<S> a, S s) {
    const S inv = S(1.0) / s;
    return {a.x * inv, a.y * inv, a.z * inv};
}
__device__ __forceinline__ DD mkdd(double v) { return {v, 0.0}; }

// Bond inputs and outputs (index order defines the dual directions).
constexpr int kInputs = 36;   // ui wi uj wj xi xj normal offset fn fs mt mb kn ks kb kt
constexpr int kOutputs = 23;  // F Ti Tj normal_end offset_end fn_end fs_end mt_end mb_end

template <class S>
struct BondIn {
    S v[kInputs];
    double radi, radj;
};

template <class S>
__device__ __forceinline__ W3<S> in3(const BondIn<S> &a, int k) {
    return {a.v[k], a.v[k + 1], a.v[k + 2]};
}

template <class S>
struct Rot {
    W3<S> k, n1;
    S inv1pc, c, s;
};

template <class S>
__device__ __forceinline__ Rot<S> make_rot(W3<S> n0, W3<S> n1, W3<S> spin) {
    Rot<S> t;
    t.k = wcross(n0, n1);
    const S cosine = dclamp1(wdot(n0, n1));
    t.inv1pc = S(1.0) / (1.0 + cosine);
    const W3<S> b0 = n0 + n1;
    const W3<S> b = wdiv(b0, dmax(dsqrt(wdot(b0, b0)), 1e-12));
    dsincos(wdot(spin, b), t.s, t.c);
    t.n1 = n1;
    return t;
}

template <class S>
__device__ __forceinline__ W3<S> rot_apply(const Rot<S> &t, W3<S> v) {
    const W3<S> kv = wcross(t.k, v);
    W3<S> out = v + kv;
    out = out + t.inv1pc * wcross(t.k, kv);
    return t.c * out + t.s * wcross(t.n1, out) + ((1.0 - t.c) * wdot(t.n1, out)) * t.n1;
}

// The trial of one bond: midpoint wrench [F, T_i, T_j] (site i gets (F, T_i),
// site j (-F, T_j)) and the end-of-step history.
template <class S>
__device__ __forceinline__ void bond_trial(const BondIn<S> &a, S out[kOutputs]) {
    const W3<S> ui = in3(a, 0), wi = in3(a, 3), uj = in3(a, 6), wj = in3(a, 9);
    const W3<S> xi = in3(a, 12), xj = in3(a, 15), normal = in3(a, 18), offset = in3(a, 21);
    const S fn = a.v[24], mt = a.v[28];
    const W3<S> fs = in3(a, 25), mb = in3(a, 29);
    const S kn = a.v[32], ks = a.v[33], kb = a.v[34], kt = a.v[35];
    const W3<S> mi = xi + 0.5 * ui, mj = xj + 0.5 * uj;
    const W3<S> ei = xi + ui, ej = xj + uj;
    const W3<S> dm = mj - mi;
    const W3<S> nm = wdiv(dm, dsqrt(wdot(dm, dm)));
    W3<S> contact = 0.5 * (mi + mj) + (0.5 * (a.radi - a.radj)) * nm;
    const W3<S> de = ej - ei;
    const W3<S> ne = wdiv(de, dsqrt(wdot(de, de)));
    const W3<S> hs = 0.5 * (0.5 * (wi + wj));
    const Rot<S> r1 = make_rot(normal, nm, hs);
    const W3<S> offset_mid = rot_apply(r1, offset);
    contact = contact + offset_mid;
    const W3<S> ri = contact - mi, rj = contact - mj;
    const W3<S> fs0 = rot_apply(r1, fs), mb0 = rot_apply(r1, mb);
    const W3<S> du = uj - ui + wcross(wj, rj) - wcross(wi, ri);
    const W3<S> dw = wj - wi;
    const S dn = wdot(du, nm), twist = wdot(dw, nm);
    const S fn1 = fn + kn * dn;
    const W3<S> fs1 = fs0 + ks * (du - dn * nm);
    const S mt1 = mt + kt * twist;
    const W3<S> mb1 = mb0 + kb * (dw - twist * nm);
    const W3<S> f = (0.5 * (fn + fn1)) * nm + 0.5 * (fs0 + fs1);
    const W3<S> couple = (0.5 * (mt + mt1)) * nm + 0.5 * (mb0 + mb1);
    const W3<S> ti = wcross(ri, f) + couple, tj = -wcross(rj, f) - couple;
    const Rot<S> r2 = make_rot(nm, ne, hs);
    const W3<S> fse = rot_apply(r2, fs1), mbe = rot_apply(r2, mb1), offe = rot_apply(r2, offset_mid);
    out[0] = f.x; out[1] = f.y; out[2] = f.z;
    out[3] = ti.x; out[4] = ti.y; out[5] = ti.z;
    out[6] = tj.x; out[7] = tj.y; out[8] = tj.z;
    out[9] = ne.x; out[10] = ne.y; out[11] = ne.z;
    out[12] = offe.x; out[13] = offe.y; out[14] = offe.z;
    out[15] = fn1;
    out[16] = fse.x; out[17] = fse.y; out[18] = fse.z;
    out[19] = mt1;
    out[20] = mbe.x; out[21] = mbe.y; out[22] = mbe.z;
}

struct BondSources {
    const int64_t *edges;
    const double *y, *x, *radii, *normal, *offset, *fn, *fs, *mt, *mb, *kn, *ks, *kb, *kt;
};

__device__ __forceinline__ void load_inputs(const BondSources &s, int64_t b, double in[kInputs], int64_t &i,
                                            int64_t &j, double &radi, double &radj) {
    edge(s.edges, b, i, j);
#pragma unroll
    for (int c = 0; c < 6; ++c) {
        in[c] = s.y[6 * i + c];
        in[6 + c] = s.y[6 * j + c];
    }
#pragma unroll
    for (int c = 0; c < 3; ++c) {
        in[12 + c] = s.x[3 * i + c];
        in[15 + c] = s.x[3 * j + c];
        in[18 + c] = s.normal[3 * b + c];
        in[21 + c] = s.offset[3 * b + c];
        in[25 + c] = s.fs[3 * b + c];
        in[29 + c] = s.mb[3 * b + c];
    }
    in[24] = s.fn[b];
    in[28] = s.mt[b];
    in[32] = s.kn[b];
    in[33] = s.ks[b];
    in[34] = s.kb[b];
    in[35] = s.kt[b];
    radi = s.radii[i];
    radj = s.radii[j];
}

// Column `dir` of the bond's local Jacobian (all 23 outputs).
__device__ __forceinline__ void column(const double in[kInputs], double radi, double radj, int dir,
                                       double col[kOutputs]) {
    BondIn<DD> a;
#pragma unroll
    for (int c = 0; c < kInputs; ++c) a.v[c] = {in[c], c == dir ? 1.0 : 0.0};
    a.radi = radi;
    a.radj = radj;
    DD out[kOutputs];
    bond_trial(a, out);
#pragma unroll
    for (int o = 0; o < kOutputs; ++o) col[o] = out[o].d;
}

// B_b (9 x 12, row-major by output) for every bond.
__global__ void __launch_bounds__(128) local_jacobian_kernel(int64_t m, BondSources s, double *B) {
    const int64_t b = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (b >= m) return;
    double in[kInputs], radi, radj;
    int64_t i, j;
    load_inputs(s, b, in, i, j, radi, radj);
    double *Bb = B + 108 * b;
    for (int dir = 0; dir < 12; ++dir) {
        double col[kOutputs];
        column(in, radi, radj, dir, col);
#pragma unroll
        for (int o = 0; o < 9; ++o) Bb[12 * o + dir] = col[o];
    }
}

// Per-bond adjoints of the 9 wrench outputs from a site vector lam (N, 6):
// F -> lam_i[0:3] - lam_j[0:3], T_i -> lam_i[3:6], T_j -> lam_j[3:6].
__device__ __forceinline__ void wrench_adjoint(const double *lam, int64_t i, int64_t j, double w[9]) {
#pragma unroll
    for (int c = 0; c < 3; ++c) {
        w[c] = lam[6 * i + c] - lam[6 * j + c];
        w[3 + c] = lam[6 * i + 3 + c];
        w[6 + c] = lam[6 * j + 3 + c];
    }
}

// J^T product, bond pass: slots[b] = [ (B_b^T w)_i (6), (B_b^T w)_j (6) ].
__global__ void __launch_bounds__(kThreads) jt_bonds_kernel(int64_t m, const int64_t *edges, const double *B,
                                                            const double *lam, double *slots) {
    const int64_t b = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (b >= m) return;
    int64_t i, j;
    edge(edges, b, i, j);
    double w[9];
    wrench_adjoint(lam, i, j, w);
    const double *Bb = B + 108 * b;
#pragma unroll
    for (int k = 0; k < 12; ++k) {
        double acc = 0.0;
#pragma unroll
        for (int o = 0; o < 9; ++o) acc += w[o] * Bb[12 * o + k];
        slots[12 * b + k] = acc;
    }
}

// Site gather of per-bond slots of width 2K ([i-side K, j-side K]).
template <int K>
__device__ __forceinline__ void gather_slots(const int32_t *ptr, const int32_t *inc, const double *slots, int64_t s,
                                             double acc[K]) {
#pragma unroll
    for (int c = 0; c < K; ++c) acc[c] = 0.0;
    const int e1 = ptr[s + 1];
    for (int e = ptr[s]; e < e1; ++e) {
        const int v = inc[e];
        const double *p = v >= 0 ? slots + 2 * K * (int64_t)v : slots + 2 * K * (int64_t)(~v) + K;
#pragma unroll
        for (int c = 0; c < K; ++c) acc[c] += p[c];
    }
}

// out = M lam - h sum B^T w on free rows, lam on fixed rows (lam's fixed rows are zero).
__global__ void __launch_bounds__(kThreads) jt_sites_kernel(int64_t n, const int32_t *ptr, const int32_t *inc,
                                                            const double *slots, const double *mass,
                                                            const uint8_t *fixed, double half_dt2, const double *lam,
                                                            double *out) {
    const int64_t s = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (s >= n) return;
    double acc[6];
    gather_slots<6>(ptr, inc, slots, s, acc);
    const bool fx = fixed[s] != 0;
#pragma unroll
    for (int c = 0; c < 6; ++c) {
        const double l = lam[6 * s + c];
        out[6 * s + c] = fx ? l : mass[6 * s + c] * l - half_dt2 * acc[c];
    }
}

// Input adjoints of one bond for output adjoints: wrench part = coef * (wrench
// adjoint of lam), end part = end-history adjoints of the bond (optional).
// Per-bond inputs: history adjoints (14: normal 3, offset 3, fn, fs 3, mt, mb 3,
// the end-history layout) ADDED to hist_adj, stiffness adjoints (kn ks kb kt)
// ADDED to stiff_adj; per-site inputs (y_i, y_j, x_i, x_j) written to slots
// [i: y 6, x 3 | j: y 6, x 3] (18 per bond) for the site gather.
struct VjpArgs {
    int64_t m;
    BondSources s;
    const double *lam;        // (N, 6) or null
    double coef;
    const double *end_adj;    // (M, 14) or null
    int first_dir;            // 0: all inputs; 12: skip the increment columns
    double *hist_adj;         // (M, 14) accumulated
    double *stiff_adj;        // (M, 4) accumulated
    double *slots;            // (M, 18) written
};

__global__ void __launch_bounds__(128) vjp_kernel(VjpArgs a) {
    const int64_t b = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (b >= a.m) return;
    double in[kInputs], radi, radj;
    int64_t i, j;
    load_inputs(a.s, b, in, i, j, radi, radj);
    double w[kOutputs];
#pragma unroll
    for (int o = 0; o < kOutputs; ++o) w[o] = 0.0;
    if (a.lam) {
        double wr[9];
        wrench_adjoint(a.lam, i, j, wr);
#pragma unroll
        for (int o = 0; o < 9; ++o) w[o] = a.coef * wr[o];
    }
    if (a.end_adj) {
        const double *e = a.end_adj + 14 * b;
#pragma unroll
        for (int o = 0; o < 14; ++o) w[9 + o] = e[o];
    }
    double *sl = a.slots + 18 * b;
    double *ha = a.hist_adj + 14 * b;
    double *ka = a.stiff_adj + 4 * b;
    if (a.first_dir > 0) {
#pragma unroll
        for (int c = 0; c < 6; ++c) sl[c] = sl[9 + c] = 0.0;
    }
    for (int dir = a.first_dir; dir < kInputs; ++dir) {
        double col[kOutputs];
        column(in, radi, radj, dir, col);
        double g = 0.0;
#pragma unroll
        for (int o = 0; o < kOutputs; ++o) g += w[o] * col[o];
        if (dir < 6) sl[dir] = g;                       // y_i
        else if (dir < 12) sl[3 + dir] = g;             // y_j -> 9..14
        else if (dir < 15) sl[dir - 6] = g;             // x_i -> 6..8
        else if (dir < 18) sl[dir] = g;                 // x_j -> 15..17
        else if (dir < 32) ha[dir - 18] += g;
        else ka[dir - 32] += g;
    }
}

// Site adjoints from the VJP slots: y_adj (N, 6) and x_adj (N, 3), ADDED.
__global__ void __launch_bounds__(kThreads) vjp_sites_kernel(int64_t n, const int32_t *ptr, const int32_t *inc,
                                                             const double *slots, double *y_adj, double *x_adj) {
    const int64_t s = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (s >= n) return;
    double acc[9];
    gather_slots<9>(ptr, inc, slots, s, acc);
    if (y_adj) {
#pragma unroll
        for (int c = 0; c < 6; ++c) y_adj[6 * s + c] += acc[c];
    }
    if (x_adj) {
#pragma unroll
        for (int c = 0; c < 3; ++c) x_adj[3 * s + c] += acc[6 + c];
    }
}

inline int blocks_for(int64_t n, int threads) { return (int)((n + threads - 1) / threads); }

}  // namespace adj
}  // namespace dpf

using namespace dpf;
using namespace dpf::adj;

extern "C" {

static bool adj_ok(const dpf_graph *g, const dpf_stiffness *k, const dpf_history *h, const double *y) {
    return g && g->n_sites > 0 && g->inc_ptr && (g->n_bonds == 0 || (g->edges && g->inc_bond)) && k && h && h->x &&
           h->radii && h->normal && h->offset && h->fn && h->fs && h->mt && h->mb && y;
}

static BondSources sources(const dpf_graph *g, const dpf_stiffness *k, const dpf_history *h, const double *y) {
    return BondSources{g->edges, y, h->x, h->radii, h->normal, h->offset, h->fn, h->fs, h->mt, h->mb,
                       k->kn, k->ks, k->kb, k->kt};
}

int64_t dpf_adjoint_jacobian_doubles(int64_t n_bonds) { return 108 * n_bonds; }

int64_t dpf_adjoint_slot_doubles(int64_t n_bonds) { return 18 * n_bonds; }

int dpf_adjoint_local_jacobian(const dpf_graph *g, const dpf_stiffness *k, const dpf_history *h, const double *y,
                               double *jacobian, void *stream) {
    if (!adj_ok(g, k, h, y) || (g->n_bonds && !jacobian)) return DPF_ERR_ARGUMENT;
    if (g->n_bonds)
        local_jacobian_kernel<<<blocks_for(g->n_bonds, 128), 128, 0, (cudaStream_t)stream>>>(
            g->n_bonds, sources(g, k, h, y), jacobian);
    DPF_CHECK_LAUNCH();
    return DPF_OK;
}

int dpf_adjoint_apply_jt(const dpf_graph *g, const double *jacobian, const double *mass, const uint8_t *fixed,
                         double dt, const double *lam, double *out, double *slots, void *stream) {
    if (!g || g->n_sites <= 0 || !mass || !fixed || !lam || !out || (g->n_bonds && (!jacobian || !slots)))
        return DPF_ERR_ARGUMENT;
    cudaStream_t st = (cudaStream_t)stream;
    if (g->n_bonds)
        jt_bonds_kernel<<<blocks_for(g->n_bonds, kThreads), kThreads, 0, st>>>(g->n_bonds, g->edges, jacobian, lam,
                                                                               slots);
    jt_sites_kernel<<<blocks_for(g->n_sites, kThreads), kThreads, 0, st>>>(
        g->n_sites, g->inc_ptr, g->inc_bond, slots, mass, fixed, 0.5 * dt * dt, lam, out);
    DPF_CHECK_LAUNCH();
    return DPF_OK;
}

int dpf_adjoint_bond_vjp(const dpf_graph *g, const dpf_stiffness *k, const dpf_history *h, const double *y,
                         const double *lam, double coef, const double *end_adjoint, int with_increment,
                         double *history_adjoint, double *stiffness_adjoint, double *y_adjoint, double *x_adjoint,
                         double *slots, void *stream) {
    if (!adj_ok(g, k, h, y) || (g->n_bonds && (!slots || !history_adjoint || !stiffness_adjoint)))
        return DPF_ERR_ARGUMENT;
    cudaStream_t st = (cudaStream_t)stream;
    if (g->n_bonds) {
        VjpArgs a{g->n_bonds, sources(g, k, h, y), lam, coef, end_adjoint, with_increment ? 0 : 12,
                  history_adjoint, stiffness_adjoint, slots};
        vjp_kernel<<<blocks_for(g->n_bonds, 128), 128, 0, st>>>(a);
    }
    if ((y_adjoint || x_adjoint) && g->n_bonds)
        vjp_sites_kernel<<<blocks_for(g->n_sites, kThreads), kThreads, 0, st>>>(
            g->n_sites, g->inc_ptr, g->inc_bond, slots, with_increment ? y_adjoint : nullptr, x_adjoint);
    DPF_CHECK_LAUNCH();
    return DPF_OK;
}

}  // extern "C"
