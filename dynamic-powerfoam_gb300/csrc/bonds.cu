// Bond sweeps of the finite-motion rate law (float64).
//
// Every sweep is two passes with no atomics: a bond pass computes, once per
// bond, the wrench it applies to its two endpoints and stores it as nine
// doubles [F, T_i, T_j] (endpoint i receives (F, T_i), endpoint j (-F, T_j));
// a site pass walks the site's incidence list in the reference's index_add_
// order and sums them.  Results are deterministic run to run.

#include "common.cuh"

namespace dpf {

constexpr int kMaxReduceBlocks = 1024;
constexpr int64_t kPartialsOffset = 8;  // doubles reserved for counters

__device__ __forceinline__ unsigned *counter_slot(double *partials, int slot) {
    return reinterpret_cast<unsigned *>(partials) + slot;
}

__device__ __forceinline__ void store_wrench(double *w, int64_t b, d3 f, d3 ti, d3 tj) {
    double *p = w + 9 * b;
    st3(p, f);
    st3(p + 3, ti);
    st3(p + 6, tj);
}

// ---------------------------------------------------------------------------
// Constitutive trial (experiments/bonded_dem_finite_gpu.py:87-116).

struct TrialBondArgs {
    int64_t m;
    const int64_t *edges;
    dpf_stiffness k;
    dpf_history h;
    const double *y, *mid, *end;
    int want_end;
    double *n, *ri, *rj;
    double *normal_end, *offset_end, *fs_end, *mb_end, *fn_end, *mt_end;
    double *wrench;
    int *status;
};

__global__ void __launch_bounds__(kThreads) trial_bonds(TrialBondArgs a) {
    const int64_t b = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (b >= a.m) return;
    int flags = 0;
    int64_t i, j;
    edge(a.edges, b, i, j);
    const double *yi = a.y + 6 * i, *yj = a.y + 6 * j;
    const d3 ui = ld3(yi), wi = ld3(yi + 3), uj = ld3(yj), wj = ld3(yj + 3);
    const d3 xi = ld3(a.h.x, i), xj = ld3(a.h.x, j);
    const d3 mi = a.mid ? ld3(a.mid, i) : xi + 0.5 * ui;
    const d3 mj = a.mid ? ld3(a.mid, j) : xj + 0.5 * uj;
    const d3 ei = a.end ? ld3(a.end, i) : xi + ui;
    const d3 ej = a.end ? ld3(a.end, j) : xj + uj;
    const double radi = a.h.radii[i], radj = a.h.radii[j];
    // geometry(mid), geometry(end)  (bonded_dem_finite_gpu.py:66-73)
    const d3 dm = mj - mi;
    const double lm = norm(dm);
    if (lm <= 1e-12) flags |= DPF_ERR_COINCIDENT;
    const d3 nm = dm / lm;
    d3 contact = 0.5 * (mi + mj) + (0.5 * (radi - radj)) * nm;
    const d3 de = ej - ei;
    const double le = norm(de);
    if (le <= 1e-12) flags |= DPF_ERR_COINCIDENT;
    const d3 ne = de / le;
    const d3 half_spin = 0.5 * (0.5 * (wi + wj));
    const Transport to_mid = make_transport(ld3(a.h.normal, b), nm, half_spin, flags);
    const d3 offset_mid = apply(to_mid, ld3(a.h.offset, b));
    contact = contact + offset_mid;
    const d3 ri = contact - mi, rj = contact - mj;
    const d3 fs0 = apply(to_mid, ld3(a.h.fs, b));
    const d3 mb0 = apply(to_mid, ld3(a.h.mb, b));
    const d3 du = uj - ui + cross(wj, rj) - cross(wi, ri);
    const d3 dw = wj - wi;
    const double dn = dot(du, nm), twist = dot(dw, nm);
    const double kn = a.k.kn[b], ks = a.k.ks[b], kb = a.k.kb[b], kt = a.k.kt[b];
    const double fn_c = a.h.fn[b], mt_c = a.h.mt[b];
    const double fn1 = fn_c + kn * dn;
    const d3 fs1 = fs0 + ks * (du - dn * nm);
    const double mt1 = mt_c + kt * twist;
    const d3 mb1 = mb0 + kb * (dw - twist * nm);
    const d3 f = (0.5 * (fn_c + fn1)) * nm + 0.5 * (fs0 + fs1);
    const d3 couple = (0.5 * (mt_c + mt1)) * nm + 0.5 * (mb0 + mb1);
    store_wrench(a.wrench, b, f, cross(ri, f) + couple, -cross(rj, f) - couple);
    if (a.n) st3(a.n, b, nm);
    if (a.ri) st3(a.ri, b, ri);
    if (a.rj) st3(a.rj, b, rj);
    // End-of-step transports; the guard is evaluated even when unused.
    const Transport to_end = make_transport(nm, ne, half_spin, flags);
    if (a.want_end) {
        if (a.normal_end) st3(a.normal_end, b, ne);
        if (a.fn_end) a.fn_end[b] = fn1;
        if (a.mt_end) a.mt_end[b] = mt1;
        if (a.fs_end) st3(a.fs_end, b, apply(to_end, fs1));
        if (a.mb_end) st3(a.mb_end, b, apply(to_end, mb1));
        if (a.offset_end) st3(a.offset_end, b, apply(to_end, offset_mid));
    }
    if (flags) atomicOr(a.status, flags);
}

// Site pass of trial/residual: force gather, rotation guard, end positions,
// midpoint residual (bonded_dem_newton.py:83-86), block scaling
// (bonded_dem_newton.py:104-105) and the three norms of NewtonBonds.step.
struct SiteResidualArgs {
    int64_t n;
    const int32_t *ptr, *inc;
    const double *wrench;
    const double *y, *x, *end;
    double *force, *x_end;
    // residual part (residual != nullptr)
    const double *v, *external, *mass;
    const uint8_t *fixed;
    double dt, half_dt2;
    double *residual;
    const double *P, *units;
    double *scaled, *norms, *partials;
    int *status;
};

__global__ void __launch_bounds__(kThreads) site_residual(SiteResidualArgs a) {
    double sum_r = 0.0, max_s = 0.0, sum_s = 0.0;
    int flags = 0;
    for (int64_t s = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; s < a.n;
         s += (int64_t)gridDim.x * blockDim.x) {
        double acc[6];
        gather_wrench(a.ptr, a.inc, a.wrench, s, acc);
        const double *ys = a.y + 6 * s;
        if (a.force) {
#pragma unroll
            for (int c = 0; c < 6; ++c) a.force[6 * s + c] = acc[c];
        }
        if (norm(ld3(ys + 3)) > 0.25) flags |= DPF_ERR_ROTATION;
        if (a.x_end) st3(a.x_end, s, a.end ? ld3(a.end, s) : ld3(a.x, s) + ld3(ys));
        if (a.residual) {
            double r[6];
            const bool fx = a.fixed[s] != 0;
#pragma unroll
            for (int c = 0; c < 6; ++c) {
                const double val = a.mass[6 * s + c] * (ys[c] - a.dt * a.v[6 * s + c]) -
                                   a.half_dt2 * (acc[c] + a.external[6 * s + c]);
                r[c] = fx ? ys[c] : val;
                a.residual[6 * s + c] = r[c];
                sum_r += r[c] * r[c];
            }
            if (a.P) {
                const double *P = a.P + 36 * s;
#pragma unroll
                for (int row = 0; row < 6; ++row) {
                    double val = 0.0;
#pragma unroll
                    for (int c = 0; c < 6; ++c) val += P[6 * row + c] * r[c];
                    val = val / a.units[6 * s + row];
                    if (a.scaled) a.scaled[6 * s + row] = val;
                    max_s = fmax(max_s, fabs(val));
                    sum_s += val * val;
                }
            }
        }
    }
    if (flags) atomicOr(a.status, flags);
    if (!a.norms) return;
    sum_r = block_sum(sum_r);
    max_s = block_max(max_s);
    sum_s = block_sum(sum_s);
    double *part = a.partials + kPartialsOffset;
    if (threadIdx.x == 0) {
        part[3 * blockIdx.x + 0] = sum_r;
        part[3 * blockIdx.x + 1] = max_s;
        part[3 * blockIdx.x + 2] = sum_s;
    }
    if (last_block(counter_slot(a.partials, 0))) {
        const double r2 = block_sum_array(part + 0, gridDim.x, 3);
        const double mx = block_max_array(part + 1, gridDim.x, 3);
        const double s2 = block_sum_array(part + 2, gridDim.x, 3);
        if (threadIdx.x == 0) {
            a.norms[0] = sqrt(r2);
            a.norms[1] = mx;
            a.norms[2] = sqrt(s2);
            if (!isfinite(r2) || !isfinite(s2)) atomicOr(a.status, DPF_ERR_NONFINITE);
        }
    }
}

// ---------------------------------------------------------------------------
// Analytic JVP of the midpoint force (experiments/bonded_dem_jvp_warp.py:17-97).

// Shared part of `transport` and its derivative for one bond: the same
// (n0, n, spin) rotate offset, fs and mb.
struct TransportJvp {
    d3 k, dk, n, dn, b;
    double inv, dc, c, s, da;
};

__device__ __forceinline__ TransportJvp make_transport_jvp(d3 n0, d3 n, d3 dn, d3 spin, d3 dspin) {
    TransportJvp t;
    const double raw = dot(n0, n);
    const double cosine = fmin(fmax(raw, -1.0), 1.0);
    t.dc = (raw < -1.0 || raw > 1.0) ? 0.0 : dot(n0, dn);
    t.k = cross(n0, n);
    t.dk = cross(n0, dn);
    t.inv = 1.0 / (1.0 + cosine);
    const d3 sum = n0 + n;
    const double length = norm(sum);
    t.b = sum / length;
    const d3 db = (dn - dot(t.b, dn) * t.b) / length;
    const double angle = dot(spin, t.b);
    t.da = dot(dspin, t.b) + dot(spin, db);
    sincos(angle, &t.s, &t.c);
    t.n = n;
    t.dn = dn;
    return t;
}

__device__ __forceinline__ void apply_jvp(const TransportJvp &t, d3 v, d3 &value, d3 &deriv) {
    const d3 kv = cross(t.k, v);
    const d3 kkv = cross(t.k, kv);
    const d3 tv = v + kv + t.inv * kkv;
    const d3 dkv = cross(t.dk, v);
    d3 dt = dkv + t.inv * (cross(t.dk, kv) + cross(t.k, dkv));
    dt = dt - (t.dc * t.inv * t.inv) * kkv;
    const double nt = dot(t.n, tv);
    const d3 nxt = cross(t.n, tv);
    value = t.c * tv + t.s * nxt + ((1.0 - t.c) * nt) * t.n;
    d3 d = t.c * dt - (t.s * t.da) * tv + (t.c * t.da) * nxt;
    d = d + t.s * (cross(t.dn, tv) + cross(t.n, dt)) + (t.s * t.da * nt) * t.n;
    deriv = d + (1.0 - t.c) * ((dot(t.dn, tv) + dot(t.n, dt)) * t.n + nt * t.dn);
}

struct JvpBondArgs {
    int64_t m;
    const int64_t *edges;
    dpf_stiffness k;
    dpf_history h;
    const double *y, *direction, *units;
    double *wrench;
};

__device__ __forceinline__ void load_direction(const double *d, const double *units, int64_t s, d3 &u, d3 &w) {
    const double *p = d + 6 * s;
    u = ld3(p);
    w = ld3(p + 3);
    if (units) {
        const double *q = units + 6 * s;
        u = mk(u.x * q[0], u.y * q[1], u.z * q[2]);
        w = mk(w.x * q[3], w.y * q[4], w.z * q[5]);
    }
}

__global__ void __launch_bounds__(kThreads) jvp_bonds(JvpBondArgs a) {
    const int64_t b = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (b >= a.m) return;
    int64_t i, j;
    edge(a.edges, b, i, j);
    const d3 ui = ld3(a.y + 6 * i), wi = ld3(a.y + 6 * i + 3);
    const d3 uj = ld3(a.y + 6 * j), wj = ld3(a.y + 6 * j + 3);
    d3 dui, dwi, duj, dwj;
    load_direction(a.direction, a.units, i, dui, dwi);
    load_direction(a.direction, a.units, j, duj, dwj);
    const d3 mi = ld3(a.h.x, i) + 0.5 * ui, mj = ld3(a.h.x, j) + 0.5 * uj;
    const d3 disp = mj - mi;
    const double length = norm(disp);
    const d3 n = disp / length;
    const d3 dd = 0.5 * (duj - dui);
    const d3 dn = (dd - dot(n, dd) * n) / length;
    const d3 spin = 0.25 * (wi + wj), dspin = 0.25 * (dwi + dwj);
    const TransportJvp t = make_transport_jvp(ld3(a.h.normal, b), n, dn, spin, dspin);
    d3 rotated, drotated, fs0, dfs0, mb0, dmb0;
    apply_jvp(t, ld3(a.h.offset, b), rotated, drotated);
    apply_jvp(t, ld3(a.h.fs, b), fs0, dfs0);
    apply_jvp(t, ld3(a.h.mb, b), mb0, dmb0);
    const double rad = 0.5 * (a.h.radii[i] - a.h.radii[j]);
    const d3 contact = 0.5 * (mi + mj) + rad * n + rotated;
    const d3 dcontact = 0.25 * (dui + duj) + rad * dn + drotated;
    const d3 ri = contact - mi, rj = contact - mj;
    const d3 dri = dcontact - 0.5 * dui, drj = dcontact - 0.5 * duj;
    const d3 du = uj - ui + cross(wj, rj) - cross(wi, ri);
    const d3 ddu = duj - dui + cross(dwj, rj) + cross(wj, drj) - cross(dwi, ri) - cross(wi, dri);
    const d3 dw = wj - wi, ddw = dwj - dwi;
    const double nd = dot(du, n), tw = dot(dw, n);
    const double dnd = dot(ddu, n) + dot(du, dn);
    const double dtw = dot(ddw, n) + dot(dw, dn);
    const double kn = a.k.kn[b], ks = a.k.ks[b], kb = a.k.kb[b], kt = a.k.kt[b];
    const double fn_mid = a.h.fn[b] + 0.5 * kn * nd;
    const double dfn_mid = 0.5 * kn * dnd;
    const d3 fs_mid = fs0 + (0.5 * ks) * (du - nd * n);
    const d3 dfs_mid = dfs0 + (0.5 * ks) * (ddu - dnd * n - nd * dn);
    const double mt_mid = a.h.mt[b] + 0.5 * kt * tw;
    const double dmt_mid = 0.5 * kt * dtw;
    const d3 dmb_mid = dmb0 + (0.5 * kb) * (ddw - dtw * n - tw * dn);
    const d3 f = fn_mid * n + fs_mid;
    const d3 df = dfn_mid * n + fn_mid * dn + dfs_mid;
    const d3 dcouple = dmt_mid * n + mt_mid * dn + dmb_mid;
    const d3 dti = cross(dri, f) + cross(ri, df) + dcouple;
    const d3 dtj = -cross(drj, f) - cross(rj, df) - dcouple;
    store_wrench(a.wrench, b, df, dti, dtj);
}

// Site pass of the JVP: out = M d - dt^2/2 g, fixed rows d; optional P(.)/units.
struct SiteJvpArgs {
    int64_t n;
    const int32_t *ptr, *inc;
    const double *wrench, *direction, *units, *mass, *P;
    const uint8_t *fixed;
    double half_dt2;
    double *out;
};

__global__ void __launch_bounds__(kThreads) site_jvp(SiteJvpArgs a) {
    const int64_t s = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (s >= a.n) return;
    double acc[6], r[6];
    gather_wrench(a.ptr, a.inc, a.wrench, s, acc);
    const bool fx = a.fixed[s] != 0;
#pragma unroll
    for (int c = 0; c < 6; ++c) {
        double d = a.direction[6 * s + c];
        if (a.units) d *= a.units[6 * s + c];
        r[c] = fx ? d : a.mass[6 * s + c] * d - a.half_dt2 * acc[c];
    }
    if (a.P) {
        const double *P = a.P + 36 * s;
#pragma unroll
        for (int row = 0; row < 6; ++row) {
            double val = 0.0;
#pragma unroll
            for (int c = 0; c < 6; ++c) val += P[6 * row + c] * r[c];
            a.out[6 * s + row] = val / a.units[6 * s + row];
        }
    } else {
#pragma unroll
        for (int c = 0; c < 6; ++c) a.out[6 * s + c] = r[c];
    }
}

// ---------------------------------------------------------------------------
// Frozen tangent K q (experiments/bonded_dem_linear_gpu.py:42-52).

struct StiffnessBondArgs {
    int64_t m;
    const int64_t *edges;
    dpf_stiffness k;
    dpf_tangent t;
    const double *q;
    double *wrench;
};

__device__ __forceinline__ void stiffness_bond(const StiffnessBondArgs &a, int64_t b) {
    int64_t i, j;
    edge(a.edges, b, i, j);
    const double *qi = a.q + 6 * i, *qj = a.q + 6 * j;
    const d3 n = ld3(a.t.n, b), ri = ld3(a.t.ri, b), rj = ld3(a.t.rj, b);
    const d3 wi = ld3(qi + 3), wj = ld3(qj + 3);
    const d3 du = ld3(qj) - ld3(qi) + cross(wj, rj) - cross(wi, ri);
    const d3 dw = wj - wi;
    const double kn = a.k.kn[b], ks = a.k.ks[b], kb = a.k.kb[b], kt = a.k.kt[b];
    const d3 f = ks * du + ((kn - ks) * dot(du, n)) * n;
    const d3 m = kb * dw + ((kt - kb) * dot(dw, n)) * n;
    store_wrench(a.wrench, b, -f, -cross(ri, f) - m, cross(rj, f) + m);
}

__global__ void __launch_bounds__(kThreads) stiffness_bonds(StiffnessBondArgs a) {
    const int64_t b = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (b < a.m) stiffness_bond(a, b);
}

__global__ void __launch_bounds__(kThreads) site_gather(int64_t n, const int32_t *ptr, const int32_t *inc,
                                                         const double *wrench, double *out) {
    const int64_t s = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (s >= n) return;
    double acc[6];
    gather_wrench(ptr, inc, wrench, s, acc);
#pragma unroll
    for (int c = 0; c < 6; ++c) out[6 * s + c] = acc[c];
}

// ---------------------------------------------------------------------------
// Diagonal blocks (bonded_dem_linear_gpu.py:54-72) and block scaling
// (bonded_dem_newton.py:94-102), one thread per site over its incidences.

__device__ __forceinline__ void add_bond_block(double D[36], d3 n, d3 r, double kn, double ks, double kb, double kt) {
    const double nv[3] = {n.x, n.y, n.z};
    double d[9], h[9];
#pragma unroll
    for (int p = 0; p < 3; ++p)
#pragma unroll
        for (int q = 0; q < 3; ++q) {
            const double nn = nv[p] * nv[q];
            d[3 * p + q] = (p == q ? ks : 0.0) + (kn - ks) * nn;
            h[3 * p + q] = (p == q ? kb : 0.0) + (kt - kb) * nn;
        }
    // S = skew(r)
    const double S[9] = {0.0, -r.z, r.y, r.z, 0.0, -r.x, -r.y, r.x, 0.0};
    double dS[9];
#pragma unroll
    for (int p = 0; p < 3; ++p)
#pragma unroll
        for (int q = 0; q < 3; ++q)
            dS[3 * p + q] = d[3 * p] * S[q] + d[3 * p + 1] * S[3 + q] + d[3 * p + 2] * S[6 + q];
#pragma unroll
    for (int p = 0; p < 3; ++p)
#pragma unroll
        for (int q = 0; q < 3; ++q) {
            D[6 * p + q] += d[3 * p + q];
            D[6 * p + 3 + q] += -dS[3 * p + q];
            D[6 * (3 + q) + p] += -dS[3 * p + q];
            // (S^T d S)_{pq} = sum_c S_{cp} (dS)_{cq}
            const double sds = S[p] * dS[q] + S[3 + p] * dS[3 + q] + S[6 + p] * dS[6 + q];
            D[6 * (3 + p) + 3 + q] += sds + h[3 * p + q];
        }
}

__device__ __forceinline__ void site_diagonal(const int32_t *ptr, const int32_t *inc, const dpf_stiffness &k,
                                              const dpf_tangent &t, int64_t s, double D[36]) {
#pragma unroll
    for (int c = 0; c < 36; ++c) D[c] = 0.0;
    const int e1 = ptr[s + 1];
    for (int e = ptr[s]; e < e1; ++e) {
        const int v = inc[e];
        const int64_t b = v >= 0 ? v : ~v;
        const d3 r = v >= 0 ? ld3(t.ri, b) : ld3(t.rj, b);
        add_bond_block(D, ld3(t.n, b), r, k.kn[b], k.ks[b], k.kb[b], k.kt[b]);
    }
}


struct ScalingArgs {
    int64_t n;
    const int32_t *ptr, *inc;
    dpf_stiffness k;
    dpf_tangent t;
    const double *mass, *radii;
    const uint8_t *fixed;
    double alpha;  // dt^2 / 4
    double *diagonal, *block, *P, *units;
};

__global__ void __launch_bounds__(128) scaling_sites(ScalingArgs a) {
    const int64_t s = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (s >= a.n) return;
    double D[36];
    site_diagonal(a.ptr, a.inc, a.k, a.t, s, D);
    if (a.diagonal) {
#pragma unroll
        for (int c = 0; c < 36; ++c) a.diagonal[36 * s + c] = D[c];
    }
    if (!a.P && !a.block) return;
    const bool fx = a.fixed[s] != 0;
    double B[36];
#pragma unroll
    for (int p = 0; p < 6; ++p)
#pragma unroll
        for (int q = 0; q < 6; ++q) {
            const double val = (p == q ? a.mass[6 * s + p] : 0.0) + a.alpha * D[6 * p + q];
            B[6 * p + q] = fx ? (p == q ? 1.0 : 0.0) : val;
        }
    if (a.block) {
#pragma unroll
        for (int c = 0; c < 36; ++c) a.block[36 * s + c] = B[c];
    }
    if (a.P) {
        double P[36];
        spd_inverse6(B, P);
#pragma unroll
        for (int c = 0; c < 36; ++c) a.P[36 * s + c] = P[c];
    }
    if (a.units) {
        const double r = fx ? 1.0 : a.radii[s];
#pragma unroll
        for (int c = 0; c < 6; ++c) a.units[6 * s + c] = c < 3 ? r : 1.0;
    }
}

__global__ void __launch_bounds__(128) diagonal_sites(int64_t n, const int32_t *ptr, const int32_t *inc,
                                                      dpf_stiffness k, dpf_tangent t, double *out) {
    const int64_t s = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (s >= n) return;
    double D[36];
    site_diagonal(ptr, inc, k, t, s, D);
#pragma unroll
    for (int c = 0; c < 36; ++c) out[36 * s + c] = D[c];
}

// ---------------------------------------------------------------------------
// Loads of the committed state (experiments/bonded_dem_finite_gpu.py:82-85).

__global__ void __launch_bounds__(kThreads) loads_bonds(int64_t m, const int64_t *edges, dpf_history h,
                                                         double *wrench, int *status) {
    const int64_t b = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (b >= m) return;
    int64_t i, j;
    edge(edges, b, i, j);
    const d3 xi = ld3(h.x, i), xj = ld3(h.x, j);
    const d3 d = xj - xi;
    const double length = norm(d);
    if (length <= 1e-12 && status) atomicOr(status, DPF_ERR_COINCIDENT);
    const d3 n = d / length;
    const d3 c = 0.5 * (xi + xj) + (0.5 * (h.radii[i] - h.radii[j])) * n + ld3(h.offset, b);
    const d3 ri = c - xi, rj = c - xj;
    const d3 f = h.fn[b] * n + ld3(h.fs, b);
    const d3 couple = h.mt[b] * n + ld3(h.mb, b);
    store_wrench(wrench, b, f, cross(ri, f) + couple, -cross(rj, f) - couple);
}

inline int blocks_for(int64_t n, int threads) { return (int)((n + threads - 1) / threads); }

// Bond setup of LinearBondsGPU / FiniteBondsGPU (experiments/bonded_dem_linear_gpu.py:15-40,
// experiments/bonded_dem_finite_gpu.py:49-63) on the device: normal, contact
// levers, stiffnesses and the contact offset from the classical contact.
struct BondSetupArgs {
    int64_t m;
    const int64_t *edges;
    const double *points, *radii, *areas, *contacts, *young_b, *shear_b;
    double young, shear;
    double *n, *ri, *rj, *kn, *ks, *kb, *kt, *offset;
};

// One-time setup arithmetic, written with correctly rounded divisions and no
// fused multiply-adds so that it gives the bits of the reference's host
// formulas (n = d / |d|, c = (p_i + p_j)/2 + (r_i - r_j)/2 n, k = E A / L, ..).
__global__ void __launch_bounds__(kThreads) bond_setup_kernel(BondSetupArgs a) {
    const int64_t b = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (b >= a.m) return;
    int64_t i, j;
    edge(a.edges, b, i, j);
    const d3 pi = ld3(a.points, i), pj = ld3(a.points, j);
    const d3 d = mk(__dsub_rn(pj.x, pi.x), __dsub_rn(pj.y, pi.y), __dsub_rn(pj.z, pi.z));
    const double length = __dsqrt_rn(__dadd_rn(__dadd_rn(__dmul_rn(d.x, d.x), __dmul_rn(d.y, d.y)), __dmul_rn(d.z, d.z)));
    const d3 n = mk(__ddiv_rn(d.x, length), __ddiv_rn(d.y, length), __ddiv_rn(d.z, length));
    const double half = __dmul_rn(0.5, __dsub_rn(a.radii[i], a.radii[j]));
    const d3 classical = mk(__dadd_rn(__dmul_rn(0.5, __dadd_rn(pi.x, pj.x)), __dmul_rn(half, n.x)),
                            __dadd_rn(__dmul_rn(0.5, __dadd_rn(pi.y, pj.y)), __dmul_rn(half, n.y)),
                            __dadd_rn(__dmul_rn(0.5, __dadd_rn(pi.z, pj.z)), __dmul_rn(half, n.z)));
    const d3 c = a.contacts ? ld3(a.contacts, b) : classical;
    st3(a.n, b, n);
    st3(a.ri, b, mk(__dsub_rn(c.x, pi.x), __dsub_rn(c.y, pi.y), __dsub_rn(c.z, pi.z)));
    st3(a.rj, b, mk(__dsub_rn(c.x, pj.x), __dsub_rn(c.y, pj.y), __dsub_rn(c.z, pj.z)));
    if (a.offset)
        st3(a.offset, b, mk(__dsub_rn(c.x, classical.x), __dsub_rn(c.y, classical.y), __dsub_rn(c.z, classical.z)));
    const double area = a.areas[b];
    const double second = __ddiv_rn(__dmul_rn(area, area), 4.0 * 3.14159265358979323846);
    const double E = a.young_b ? a.young_b[b] : a.young, G = a.shear_b ? a.shear_b[b] : a.shear;
    a.kn[b] = __ddiv_rn(__dmul_rn(E, area), length);
    a.ks[b] = __ddiv_rn(__dmul_rn(G, area), length);
    a.kb[b] = __ddiv_rn(__dmul_rn(E, second), length);
    a.kt[b] = __ddiv_rn(__dmul_rn(G, __dmul_rn(2.0, second)), length);
}

__global__ void __launch_bounds__(kThreads) site_mass_kernel(int64_t n, const double *masses, const double *radii,
                                                             double *mass6) {
    const int64_t s = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (s >= n) return;
    const double m = masses[s], r = radii[s];
    const double inertia = __dmul_rn(__dmul_rn(__dmul_rn(0.4, m), r), r);
#pragma unroll
    for (int c = 0; c < 6; ++c) mass6[6 * s + c] = c < 3 ? m : inertia;
}

}  // namespace dpf

using namespace dpf;

extern "C" {

int64_t dpf_wrench_scratch_doubles(int64_t n_bonds) { return 9 * n_bonds; }

int64_t dpf_partials_doubles(void) { return kPartialsOffset + 2 * 64 * (int64_t)kMaxReduceBlocks; }

static bool graph_ok(const dpf_graph *g) {
    return g && g->n_sites > 0 && g->n_bonds >= 0 && g->n_bonds < (int64_t(1) << 31) && g->inc_ptr &&
           (g->n_bonds == 0 || (g->edges && g->inc_bond));
}

int dpf_stiffness_apply(const dpf_graph *g, const dpf_stiffness *k, const dpf_tangent *t, const double *q,
                        double *out, double *wrench, void *stream) {
    if (!graph_ok(g) || !k || !t || !q || !out || (g->n_bonds && !wrench)) return DPF_ERR_ARGUMENT;
    cudaStream_t st = (cudaStream_t)stream;
    if (g->n_bonds) {
        StiffnessBondArgs a{g->n_bonds, g->edges, *k, *t, q, wrench};
        stiffness_bonds<<<blocks_for(g->n_bonds, kThreads), kThreads, 0, st>>>(a);
    }
    site_gather<<<blocks_for(g->n_sites, kThreads), kThreads, 0, st>>>(g->n_sites, g->inc_ptr, g->inc_bond,
                                                                        wrench, out);
    DPF_CHECK_LAUNCH();
    return DPF_OK;
}

int dpf_diagonal_blocks(const dpf_graph *g, const dpf_stiffness *k, const dpf_tangent *t, double *diagonal,
                        void *stream) {
    if (!graph_ok(g) || !k || !t || !diagonal) return DPF_ERR_ARGUMENT;
    diagonal_sites<<<blocks_for(g->n_sites, 128), 128, 0, (cudaStream_t)stream>>>(
        g->n_sites, g->inc_ptr, g->inc_bond, *k, *t, diagonal);
    DPF_CHECK_LAUNCH();
    return DPF_OK;
}

int dpf_prepare_scaling(const dpf_graph *g, const dpf_stiffness *k, const dpf_tangent *t, const double *mass,
                        const uint8_t *fixed, const double *radii, double dt, double *diagonal, double *block,
                        double *preconditioner, double *units, void *stream) {
    if (!graph_ok(g) || !k || !t || !mass || !fixed || !radii || !preconditioner) return DPF_ERR_ARGUMENT;
    ScalingArgs a{g->n_sites, g->inc_ptr, g->inc_bond, *k, *t, mass, radii, fixed, 0.25 * dt * dt,
                  diagonal, block, preconditioner, units};
    scaling_sites<<<blocks_for(g->n_sites, 128), 128, 0, (cudaStream_t)stream>>>(a);
    DPF_CHECK_LAUNCH();
    return DPF_OK;
}

static int launch_trial_bonds(const dpf_graph *g, const dpf_stiffness *k, const dpf_history *h, const double *y,
                              const double *mid, const double *end, int want_end, const dpf_trial_out *out,
                              double *wrench, int *status, cudaStream_t st) {
    if (!g->n_bonds) return DPF_OK;
    TrialBondArgs a{};
    a.m = g->n_bonds;
    a.edges = g->edges;
    a.k = *k;
    a.h = *h;
    a.y = y;
    a.mid = mid;
    a.end = end;
    a.want_end = want_end;
    if (out) {
        a.n = out->n;
        a.ri = out->ri;
        a.rj = out->rj;
        a.normal_end = out->normal_end;
        a.offset_end = out->offset_end;
        a.fs_end = out->fs_end;
        a.mb_end = out->mb_end;
        a.fn_end = out->fn_end;
        a.mt_end = out->mt_end;
    }
    a.wrench = wrench;
    a.status = status;
    trial_bonds<<<blocks_for(g->n_bonds, kThreads), kThreads, 0, st>>>(a);
    return DPF_OK;
}

// Per-bond history arrays may be null (empty) when the graph has no bonds.
static bool history_ok(const dpf_history *h, int64_t n_bonds = 1) {
    return h && h->x && h->radii &&
           (n_bonds == 0 || (h->normal && h->offset && h->fn && h->fs && h->mt && h->mb));
}

int dpf_trial(const dpf_graph *g, const dpf_stiffness *k, const dpf_history *h, const double *y,
              const double *mid_positions, const double *end_positions, int want_end, const dpf_trial_out *out,
              double *wrench, int *status, void *stream) {
    if (!graph_ok(g) || !k || !history_ok(h, g->n_bonds) || !y || !out || !out->force || !status ||
        (g->n_bonds && !wrench))
        return DPF_ERR_ARGUMENT;
    cudaStream_t st = (cudaStream_t)stream;
    launch_trial_bonds(g, k, h, y, mid_positions, end_positions, want_end, out, wrench, status, st);
    SiteResidualArgs a{};
    a.n = g->n_sites;
    a.ptr = g->inc_ptr;
    a.inc = g->inc_bond;
    a.wrench = wrench;
    a.y = y;
    a.x = h->x;
    a.end = end_positions;
    a.force = out->force;
    a.x_end = want_end ? out->x_end : nullptr;
    a.status = status;
    site_residual<<<blocks_for(g->n_sites, kThreads), kThreads, 0, st>>>(a);
    DPF_CHECK_LAUNCH();
    return DPF_OK;
}

int dpf_residual(const dpf_graph *g, const dpf_stiffness *k, const dpf_history *h, const double *y,
                 const double *v, const double *external, const double *mass, const uint8_t *fixed, double dt,
                 const dpf_trial_out *trial, const double *preconditioner, const double *units, double *residual,
                 double *scaled, double *norms, double *wrench, double *partials, int *status, void *stream) {
    if (!graph_ok(g) || !k || !history_ok(h, g->n_bonds) || !y || !v || !external || !mass || !fixed || !residual ||
        !status || (g->n_bonds && !wrench) || (norms && !partials) || (preconditioner && !units))
        return DPF_ERR_ARGUMENT;
    cudaStream_t st = (cudaStream_t)stream;
    launch_trial_bonds(g, k, h, y, nullptr, nullptr, 0, trial, wrench, status, st);
    SiteResidualArgs a{};
    a.n = g->n_sites;
    a.ptr = g->inc_ptr;
    a.inc = g->inc_bond;
    a.wrench = wrench;
    a.y = y;
    a.x = h->x;
    a.force = trial ? trial->force : nullptr;
    a.v = v;
    a.external = external;
    a.mass = mass;
    a.fixed = fixed;
    a.dt = dt;
    a.half_dt2 = 0.5 * dt * dt;
    a.residual = residual;
    a.P = preconditioner;
    a.units = units;
    a.scaled = scaled;
    a.norms = norms;
    a.partials = partials;
    a.status = status;
    int grid = blocks_for(g->n_sites, kThreads);
    if (grid > kMaxReduceBlocks) grid = kMaxReduceBlocks;
    site_residual<<<grid, kThreads, 0, st>>>(a);
    DPF_CHECK_LAUNCH();
    return DPF_OK;
}

int dpf_jacobian_vector(const dpf_graph *g, const dpf_stiffness *k, const dpf_history *h, const double *y,
                        const double *direction, const double *mass, const uint8_t *fixed, double dt,
                        const double *units, const double *preconditioner, double *out, double *wrench,
                        void *stream) {
    if (!graph_ok(g) || !k || !history_ok(h, g->n_bonds) || !y || !direction || !mass || !fixed || !out ||
        (g->n_bonds && !wrench) || (preconditioner && !units))
        return DPF_ERR_ARGUMENT;
    cudaStream_t st = (cudaStream_t)stream;
    if (g->n_bonds) {
        JvpBondArgs a{g->n_bonds, g->edges, *k, *h, y, direction, units, wrench};
        jvp_bonds<<<blocks_for(g->n_bonds, kThreads), kThreads, 0, st>>>(a);
    }
    SiteJvpArgs s{g->n_sites, g->inc_ptr, g->inc_bond, wrench, direction, units, mass, preconditioner, fixed,
                  0.5 * dt * dt, out};
    site_jvp<<<blocks_for(g->n_sites, kThreads), kThreads, 0, st>>>(s);
    DPF_CHECK_LAUNCH();
    return DPF_OK;
}

int dpf_bond_setup(int64_t n_sites, int64_t n_bonds, const int64_t *edges, const double *points, const double *radii,
                   const double *areas, const double *contacts, const double *masses, double young, double shear,
                   const double *young_b, const double *shear_b, double *n, double *ri, double *rj, double *kn,
                   double *ks, double *kb, double *kt, double *offset, double *mass6, void *stream) {
    if (n_sites <= 0 || n_bonds < 0 || (n_bonds && (!edges || !areas || !n || !ri || !rj || !kn || !ks || !kb || !kt)) ||
        !points || !radii || (mass6 && !masses))
        return DPF_ERR_ARGUMENT;
    cudaStream_t st = (cudaStream_t)stream;
    if (n_bonds) {
        BondSetupArgs a{n_bonds, edges, points, radii, areas, contacts, young_b, shear_b, young, shear,
                        n, ri, rj, kn, ks, kb, kt, offset};
        bond_setup_kernel<<<blocks_for(n_bonds, kThreads), kThreads, 0, st>>>(a);
    }
    if (mass6) site_mass_kernel<<<blocks_for(n_sites, kThreads), kThreads, 0, st>>>(n_sites, masses, radii, mass6);
    DPF_CHECK_LAUNCH();
    return DPF_OK;
}

int dpf_loads(const dpf_graph *g, const dpf_history *h, double *out, double *wrench, void *stream) {
    if (!graph_ok(g) || !history_ok(h, g->n_bonds) || !out || (g->n_bonds && !wrench)) return DPF_ERR_ARGUMENT;
    cudaStream_t st = (cudaStream_t)stream;
    if (g->n_bonds)
        loads_bonds<<<blocks_for(g->n_bonds, kThreads), kThreads, 0, st>>>(g->n_bonds, g->edges, *h, wrench,
                                                                            nullptr);
    site_gather<<<blocks_for(g->n_sites, kThreads), kThreads, 0, st>>>(g->n_sites, g->inc_ptr, g->inc_bond,
                                                                        wrench, out);
    DPF_CHECK_LAUNCH();
    return DPF_OK;
}

}  // extern "C"

// ---------------------------------------------------------------------------
// K q without any allocation by anyone: the bond-wrench scratch lives in a
// file-scope device array instead of a caller buffer.  For callers that
// cannot call cudaMalloc (see dpf_stiffness_apply_static in dpf_gb300.h).

namespace {

__device__ __align__(256) double g_static_wrench[9 * DPF_STATIC_MAX_BONDS];

// Device address of g_static_wrench on the current device.  The host-side
// name is only a stand-in for the device symbol, so the address is looked up
// with cudaGetSymbolAddress while the device is current.  It is looked up on
// every call (cheap once the module is loaded) rather than cached, so a
// device reset or a re-created primary context never leaves a stale address.
int static_wrench(double **out) {
    void *ptr = nullptr;
    if (cudaGetSymbolAddress(&ptr, g_static_wrench) != cudaSuccess || !ptr) {
        cudaGetLastError();
        return DPF_ERR_CUDA;
    }
    *out = static_cast<double *>(ptr);
    return DPF_OK;
}

}  // namespace

extern "C" {

int64_t dpf_static_max_bonds(void) { return DPF_STATIC_MAX_BONDS; }

int dpf_stiffness_apply_static(const dpf_graph *g, const dpf_stiffness *k, const dpf_tangent *t, const double *q,
                               double *out, void *stream) {
    if (!graph_ok(g) || !k || !t || !q || !out) return DPF_ERR_ARGUMENT;
    if (g->n_bonds > DPF_STATIC_MAX_BONDS) return DPF_ERR_TOO_LARGE;
    double *wrench = nullptr;
    const int rc = static_wrench(&wrench);
    if (rc) return rc;
    cudaStream_t st = (cudaStream_t)stream;
    // Every bond slot read by site_gather is written by stiffness_bonds first
    // in the same call, so the array needs no clearing between calls.
    if (g->n_bonds) {
        StiffnessBondArgs a{g->n_bonds, g->edges, *k, *t, q, wrench};
        stiffness_bonds<<<blocks_for(g->n_bonds, kThreads), kThreads, 0, st>>>(a);
    }
    site_gather<<<blocks_for(g->n_sites, kThreads), kThreads, 0, st>>>(g->n_sites, g->inc_ptr, g->inc_bond,
                                                                        wrench, out);
    DPF_CHECK_LAUNCH();
    return DPF_OK;
}

}  // extern "C"
