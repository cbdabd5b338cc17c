// Mixed-precision Newton path: float32 bond sweeps, float64 reductions and a
// float64-accurate residual.
//
// Per time step, one float64 pass (mixed_setup) builds the float32 bond
// records and the float64 constant part of the residual,
//     r0 = -dt M v - dt^2/2 (loads(x) + external),
// so that for any increment y
//     r(y) = r0 + M y - dt^2/2 sum_bonds [f_mid(y) - f_mid(0)],
// where the bond increments are evaluated in float32 from small quantities
// only (normal change, transport increments, lever changes; see mixed.cuh)
// and summed per site in float64.  The JVP is the forward-mode derivative of
// the same float32 increment.  Site sums walk the incidence CSR (no atomics).
#include "mixed.cuh"

namespace dpf {
namespace mp {

constexpr int kMaxReduceBlocks = 1024;
constexpr int64_t kPartialsOffset = 8;
constexpr int kMaxPcgBlocks = 4096;
// Lanes per site in the segmented (lane-group) site gathers: each lane of a
// group walks every kGroup-th incidence of the site, then the group reduces
// with xor shuffles.  Groups never straddle a warp.
constexpr int kGroup = 4;

inline int blocks_for(int64_t n, int threads) { return (int)((n + threads - 1) / threads); }
inline int reduce_grid(int64_t n) {
    int g = blocks_for(n, kThreads);
    return g > kMaxReduceBlocks ? kMaxReduceBlocks : (g < 1 ? 1 : g);
}

__device__ __forceinline__ unsigned *counter_slot(double *partials, int slot) {
    return reinterpret_cast<unsigned *>(partials) + slot;
}

// Bond data block: records (7 float4 per bond) then the float32 tangent used
// by K q and the blocks (4 float4 per bond: (n, kn), (ri, ks), (rj, kb), (kt, i, j, 0)).
struct BondData {
    Records rec;
    float4 *t0, *t1, *t2, *t3;
};

inline BondData split_bond_data(float *base, int64_t m) {
    float4 *p = reinterpret_cast<float4 *>(base);
    BondData d;
    d.rec = {p, p + m, p + 2 * m, p + 3 * m, p + 4 * m, p + 5 * m, p + 6 * m};
    d.t0 = p + 7 * m;
    d.t1 = p + 8 * m;
    d.t2 = p + 9 * m;
    d.t3 = p + 10 * m;
    return d;
}

__device__ __forceinline__ V3<float> f3(const double *p) {
    return {(float)p[0], (float)p[1], (float)p[2]};
}
__device__ __forceinline__ float3 tof3(d3 a) { return make_float3((float)a.x, (float)a.y, (float)a.z); }

// Float32 bond wrench record [F, T_i, T_j] in 12 floats (48 B, 16-byte
// aligned): (F.x F.y F.z Ti.x) (Ti.y Ti.z Tj.x Tj.y) (Tj.z 0 0 0), so that a
// site pass reads an end's six numbers with two or three 16-byte loads.
constexpr int kWrenchFloats = 12;

__device__ __forceinline__ void store9(float *w, int64_t b, V3<float> f, V3<float> ti, V3<float> tj) {
    float4 *p = reinterpret_cast<float4 *>(w + kWrenchFloats * b);
    p[0] = make_float4(f.x, f.y, f.z, ti.x);
    p[1] = make_float4(ti.y, ti.z, tj.x, tj.y);
    p[2] = make_float4(tj.z, 0.0f, 0.0f, 0.0f);
}

// The signed share of incidence v (v >= 0: the i end, F and T_i; ~v: the j
// end, -F and T_j) of a wrench record.
__device__ __forceinline__ void end_share(const float *__restrict__ w, int v, float out[6]) {
    const bool at_i = v >= 0;
    const float4 *p = reinterpret_cast<const float4 *>(w + kWrenchFloats * (int64_t)(at_i ? v : ~v));
    const float4 q0 = p[0], q1 = p[1];
    if (at_i) {
        out[0] = q0.x; out[1] = q0.y; out[2] = q0.z;
        out[3] = q0.w; out[4] = q1.x; out[5] = q1.y;
    } else {
        const float tz = reinterpret_cast<const float *>(p)[8];
        out[0] = -q0.x; out[1] = -q0.y; out[2] = -q0.z;
        out[3] = q1.z; out[4] = q1.w; out[5] = tz;
    }
}

// Error-free sum a + b = s + e (Knuth's TwoSum), float32.
__device__ __forceinline__ void two_sum(float &s, float &e, float b) {
    const float t = s + b;
    const float bp = t - s;
    e += (s - (t - bp)) + (b - bp);
    s = t;
}


// Segmented site sum by groups of kGroupJ lanes (xor-shuffle reduction),
// compensated: used by the residual, JVP and commit site passes.  The group
// width is a launch-shape choice (4, 8 or 16 lanes; the build may set it):
// on the 64^3 foam 4 lanes measured fastest (residual 157 / 186 / 258 us,
// JVP 169 / 176 / 205 us for 4 / 8 / 16 lanes).
#ifndef DPF_SITE_LANES
#define DPF_SITE_LANES 4
#endif
constexpr int kGroupJ = DPF_SITE_LANES;
static_assert(kGroupJ == 4 || kGroupJ == 8 || kGroupJ == 16, "site groups of 4, 8 or 16 lanes");

__device__ __forceinline__ void group_gather9c_j(const int32_t *__restrict__ ptr, const int32_t *__restrict__ inc,
                                                 const float *__restrict__ w, int64_t s, bool valid, int lane,
                                                 float hi[6], float lo[6]) {
#pragma unroll
    for (int c = 0; c < 6; ++c) hi[c] = lo[c] = 0.0f;
    if (valid) {
        const int e1 = ptr[s + 1];
        for (int e = ptr[s] + lane; e < e1; e += kGroupJ) {
            float sh[6];
            end_share(w, inc[e], sh);
#pragma unroll
            for (int c = 0; c < 6; ++c) two_sum(hi[c], lo[c], sh[c]);
        }
    }
#pragma unroll
    for (int o = 1; o < kGroupJ; o <<= 1)
#pragma unroll
        for (int c = 0; c < 6; ++c) {
            const float h = __shfl_xor_sync(0xffffffffu, hi[c], o);
            const float l = __shfl_xor_sync(0xffffffffu, lo[c], o);
            two_sum(hi[c], lo[c], h);
            lo[c] += l;
        }
}

// Site sum of a float32 bond wrench in float64.
__device__ __forceinline__ void gather9(const int32_t *__restrict__ ptr, const int32_t *__restrict__ inc,
                                        const float *__restrict__ w, int64_t s, double acc[6]) {
#pragma unroll
    for (int c = 0; c < 6; ++c) acc[c] = 0.0;
    const int e1 = ptr[s + 1];
    for (int e = ptr[s]; e < e1; ++e) {
        float sh[6];
        end_share(w, inc[e], sh);
#pragma unroll
        for (int c = 0; c < 6; ++c) acc[c] += (double)sh[c];
    }
}

// ---------------------------------------------------------------------------
// Per-step setup (float64): records, loads(x) wrench.

struct SetupArgs {
    int64_t m;
    const int64_t *edges;
    dpf_stiffness k;
    dpf_history h;
    BondData out;
    double *wrench;
    float4 *corr;  // optional: the records' float32 rounding errors (the lazy history's corrections)
    int *status;
};

// What float32 rounding drops from a float64 history value (the lazy
// history's correction of a record just written from it).
__device__ __forceinline__ float history_gap(double h) { return (float)(h - (double)(float)h); }

// One thread per bond, float64 (this pass is float64-bound on this part: one
// reciprocal square root gives the length and the unit normal, no divisions).
__global__ void __launch_bounds__(kThreads) setup_bonds(SetupArgs a) {
    const int64_t b = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (b >= a.m) return;
    int64_t i, j;
    edge(a.edges, b, i, j);
    const d3 xi = ld3(a.h.x, i), xj = ld3(a.h.x, j);
    const d3 dx = xj - xi;
    const double l2 = dot(dx, dx);
    if (l2 <= 1e-24) atomicOr(a.status, DPF_ERR_COINCIDENT);
    const double inv = rsqrt(l2);
    const double L0 = l2 * inv;
    const d3 nx = inv * dx;
    const d3 n0 = ld3(a.h.normal, b);
    const double rh = 0.5 * (a.h.radii[i] - a.h.radii[j]);
    const d3 off = ld3(a.h.offset, b), fs = ld3(a.h.fs, b), mb = ld3(a.h.mb, b);
    const double fn = a.h.fn[b], mt = a.h.mt[b];
    const d3 c = 0.5 * (xi + xj) + rh * nx + off;
    const d3 ri = c - xi, rj = c - xj;
    // A bond without force and couple (every bond of a request's first step):
    // its wrench and its force records are zero, and the float64 arithmetic
    // for them (about half of this pass) is skipped.  Only the sign of a zero
    // can differ from the full form, which no site sum sees (0 + -0 = +0).
    const bool quiet = fn == 0.0 && mt == 0.0 && fs.x == 0.0 && fs.y == 0.0 && fs.z == 0.0 && mb.x == 0.0 &&
                       mb.y == 0.0 && mb.z == 0.0;
    // loads(x) exactly as dpf_loads (experiments/bonded_dem_finite_gpu.py:82-85)
    double *w = a.wrench + 9 * b;
    const float kn = (float)a.k.kn[b], ks = (float)a.k.ks[b], kb = (float)a.k.kb[b], kt = (float)a.k.kt[b];
    const float3 n0f = tof3(n0), dn0 = tof3(nx - n0), rif = tof3(ri);
    const int64_t m = a.m;
    if (quiet) {
        const d3 zero = mk(0.0, 0.0, 0.0);
        st3(w, zero);
        st3(w + 3, zero);
        st3(w + 6, zero);
        a.out.rec.r2[b] = make_float4(rif.x, rif.y, rif.z, 0.0f);
        a.out.rec.r3[b] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
        a.out.rec.r4[b] = make_float4(0.0f, 0.0f, 0.0f, kn);
        if (a.corr) {
            a.corr[b] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
            a.corr[m + b] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
        }
    } else {
        const d3 f = fn * nx + fs;
        const d3 couple = mt * nx + mb;
        st3(w, f);
        st3(w + 3, cross(ri, f) + couple);
        st3(w + 6, -cross(rj, f) - couple);
        a.out.rec.r2[b] = make_float4(rif.x, rif.y, rif.z, (float)fn);
        a.out.rec.r3[b] = make_float4((float)fs.x, (float)fs.y, (float)fs.z, (float)mt);
        a.out.rec.r4[b] = make_float4((float)mb.x, (float)mb.y, (float)mb.z, kn);
        if (a.corr) {
            a.corr[b] = make_float4(history_gap(fs.x), history_gap(fs.y), history_gap(fs.z), history_gap(fn));
            a.corr[m + b] = make_float4(history_gap(mb.x), history_gap(mb.y), history_gap(mb.z), history_gap(mt));
        }
    }
    a.out.rec.r0[b] = make_float4(n0f.x, n0f.y, n0f.z, (float)L0);
    a.out.rec.r1[b] = make_float4(dn0.x, dn0.y, dn0.z, (float)rh);
    a.out.rec.r5[b] = make_float4((float)off.x, (float)off.y, (float)off.z, ks);
    a.out.rec.r6[b] = make_float4(kb, kt, __int_as_float((int)i), __int_as_float((int)j));
    a.out.t3[b] = make_float4(kt, __int_as_float((int)i), __int_as_float((int)j), 0.0f);
    if (a.corr)
        a.corr[2 * m + b] = make_float4(history_gap(off.x), history_gap(off.y), history_gap(off.z), 0.0f);
}

// r0 = -dt M v - dt^2/2 (L + ext); norms [|dt M v + dt^2/2 ext|, |L on free sites|].
struct SetupSiteArgs {
    int64_t n;
    const int32_t *ptr, *inc;
    const double *wrench, *mass, *v, *external;
    const uint8_t *fixed;
    double dt, half_dt2;
    double *r0, *loads, *scales, *partials;
};

__global__ void __launch_bounds__(kThreads) setup_sites(SetupSiteArgs a) {
    double a2 = 0.0, l2 = 0.0;
    for (int64_t s = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; s < a.n; s += (int64_t)gridDim.x * blockDim.x) {
        double acc[6];
#pragma unroll
        for (int c = 0; c < 6; ++c) acc[c] = 0.0;
        const int e1 = a.ptr[s + 1];
        for (int e = a.ptr[s]; e < e1; ++e) {
            const int v = a.inc[e];
            if (v >= 0) {
                const double *p = a.wrench + 9 * (int64_t)v;
#pragma unroll
                for (int c = 0; c < 6; ++c) acc[c] += p[c];
            } else {
                const double *p = a.wrench + 9 * (int64_t)(~v);
                acc[0] -= p[0];
                acc[1] -= p[1];
                acc[2] -= p[2];
                acc[3] += p[6];
                acc[4] += p[7];
                acc[5] += p[8];
            }
        }
        const bool fx = a.fixed[s] != 0;
#pragma unroll
        for (int c = 0; c < 6; ++c) {
            const int64_t e = 6 * s + c;
            const double mv = a.dt * a.mass[e] * a.v[e];
            const double rhs = mv + a.half_dt2 * a.external[e];
            a2 += rhs * rhs;
            if (!fx) l2 += acc[c] * acc[c];
            a.r0[e] = -mv - a.half_dt2 * (acc[c] + a.external[e]);
            if (a.loads) a.loads[e] = acc[c];
        }
    }
    a2 = block_sum(a2);
    l2 = block_sum(l2);
    double *part = a.partials + kPartialsOffset;
    if (threadIdx.x == 0) {
        part[2 * blockIdx.x] = a2;
        part[2 * blockIdx.x + 1] = l2;
    }
    if (last_block(counter_slot(a.partials, 5))) {
        const double sa = block_sum_array(part, gridDim.x, 2);
        const double sl = block_sum_array(part + 1, gridDim.x, 2);
        if (threadIdx.x == 0) {
            a.scales[0] = sqrt(sa);
            a.scales[1] = sqrt(sl);
        }
    }
}

// ---------------------------------------------------------------------------
// Residual increment (float32 bonds) and the float64 residual (sites).

struct ResidualBondArgs {
    int64_t m;
    BondData bd;
    const float *y;
    int want_tangent;
    float *wrench;
    int *status;
    const int32_t *seg;      // optional per-bond segment: status[seg[b]]
    const uint8_t *active;   // optional per-segment flag: bonds of inactive segments are skipped
};

__device__ __forceinline__ void load_y(const float *y, int s, V3<float> &u, V3<float> &w) {
    const float *p = y + 6 * (int64_t)s;
    u = {p[0], p[1], p[2]};
    w = {p[3], p[4], p[5]};
}

__device__ __forceinline__ void store_zero9(float *w, int64_t b) {
    float4 *p = reinterpret_cast<float4 *>(w + kWrenchFloats * b);
    p[0] = p[1] = p[2] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
}

__global__ void __launch_bounds__(kThreads) residual_bonds(ResidualBondArgs a) {
    const int64_t b = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (b >= a.m) return;
    if (a.active && !a.active[a.seg[b]]) {  // a converged request of a batch: its rows are not read
        store_zero9(a.wrench, b);
        return;
    }
    const Bond B = load_bond(a.bd.rec, b);
    V3<float> ui, wi, uj, wj;
    load_y(a.y, B.i, ui, wi);
    load_y(a.y, B.j, uj, wj);
    const BondIncrement<float> o = bond_increment<float>(B, ui, wi, uj, wj);
    store9(a.wrench, b, o.dF, o.dTi, o.dTj);
    int flags = 0;
    if (!(o.length > 1e-12f)) flags |= DPF_ERR_COINCIDENT;
    if (o.turn2 > kTurn2) flags |= DPF_ERR_NORMAL_TURN;
    // end-of-step guards: end length and the mid -> end normal turn
    const V3<float> nx = lift3<float>(B.n0) + lift3<float>(B.dn0);
    float le;
    const V3<float> dnx_e = normal_change(B.L0, nx, uj - ui, le);
    const V3<float> turn = dnx_e - o.dn_x;
    if (!(le > 1e-12f)) flags |= DPF_ERR_COINCIDENT;
    if (dot(turn, turn) > kTurn2) flags |= DPF_ERR_NORMAL_TURN;
    if (flags) atomicOr(a.status + (a.seg ? a.seg[b] : 0), flags);
    if (a.want_tangent) {
        a.bd.t0[b] = make_float4(o.n.x, o.n.y, o.n.z, B.kn);
        a.bd.t1[b] = make_float4(o.ri.x, o.ri.y, o.ri.z, B.ks);
        a.bd.t2[b] = make_float4(o.rj.x, o.rj.y, o.rj.z, B.kb);
    }
}

struct ResidualSiteArgs {
    int64_t n;
    const int32_t *ptr, *inc;
    const float *wrench;
    const double *y, *mass, *r0;
    const uint8_t *fixed;
    double half_dt2;
    const float *P, *units32;
    double *residual, *scaled, *norms, *partials;
    int *status;
    const int32_t *seg;  // optional per-site segment: status[seg[s]]
};

__device__ __forceinline__ void matvec6f(const float *P, const float x[6], float y[6]) {
#pragma unroll
    for (int row = 0; row < 6; ++row) {
        float v = 0.0f;
#pragma unroll
        for (int c = 0; c < 6; ++c) v = fmaf(P[6 * row + c], x[c], v);
        y[row] = v;
    }
}

// Block partials of [|r|^2, max |s|, |s|^2] from per-thread float64 |r|^2,
// float32 max |s| and the float32 pair |s|^2, reduced as float32 pairs
// (float64 is scarce on this part: three float64 operations per thread
// instead of a float64 add per shuffle level), then in the last block the
// grid totals.
__device__ __forceinline__ void finish_norms(double sum_r, float max_s, float s_hi, float s_lo, double *partials,
                                             int slot, double *norms, int *status) {
    const float r_hi = (float)sum_r, r_lo = (float)(sum_r - (double)r_hi);
    const float2 r2 = block_pair_sum(r_hi, r_lo);
    const float mx = block_max_float(max_s);
    const float2 s2 = block_pair_sum(s_hi, s_lo);
    double *part = partials + kPartialsOffset;
    if (threadIdx.x == 0) {
        part[3 * blockIdx.x] = (double)r2.x + (double)r2.y;
        part[3 * blockIdx.x + 1] = mx;
        part[3 * blockIdx.x + 2] = (double)s2.x + (double)s2.y;
    }
    if (last_block(counter_slot(partials, slot))) {
        const double r2 = block_sum_array(part, gridDim.x, 3);
        const double mx = block_max_array(part + 1, gridDim.x, 3);
        const double s2 = block_sum_array(part + 2, gridDim.x, 3);
        if (threadIdx.x == 0) {
            norms[0] = sqrt(r2);
            norms[1] = mx;
            norms[2] = sqrt(s2);
            if (status && (!isfinite(r2) || !isfinite(s2))) atomicOr(status, DPF_ERR_NONFINITE);
        }
    }
}

// One scaled row of a site: (P r)_row / units_row in float32 (the fmaf order
// of matvec6f), from the float32 copy rf of the site's residual.
__device__ __forceinline__ float scale_row(const float *P, const float rf[6], int row, float unit) {
    const float2 *p = reinterpret_cast<const float2 *>(P + 6 * row);
    const float2 p01 = p[0], p23 = p[1], p45 = p[2];
    float v = 0.0f;
    v = fmaf(p01.x, rf[0], v);
    v = fmaf(p01.y, rf[1], v);
    v = fmaf(p23.x, rf[2], v);
    v = fmaf(p23.y, rf[3], v);
    v = fmaf(p45.x, rf[4], v);
    v = fmaf(p45.y, rf[5], v);
    return v / unit;
}

// (hi, lo) += v^2 without rounding error beyond float32 pairs: the square by
// FMA (TwoProd) and the sum by TwoSum.  Keeps |s|^2 to about 48 bits without
// float64 arithmetic per entry (float64 is scarce on this part).
__device__ __forceinline__ void add_square(float &hi, float &lo, float v) {
    const float p = v * v;
    const float e = fmaf(v, v, -p);
    two_sum(hi, lo, p);
    lo += e;
}

// A group of kGroupJ lanes per site: the lanes gather the site's bond
// wrench, lanes 0-2 then form two residual components each (16-byte loads and
// stores), the group exchanges them by shuffles, and with a preconditioner
// lane l scales rows l, l + kGroupJ, ... of the six.
__global__ void __launch_bounds__(kThreads) residual_sites(ResidualSiteArgs a) {
    double sum_r = 0.0;
    float max_s = 0.0f;
    float s_hi = 0.0f, s_lo = 0.0f;
    int flags = 0;
    const int lane = threadIdx.x & (kGroupJ - 1);
    const int64_t groups = (int64_t)gridDim.x * blockDim.x / kGroupJ;
    const int64_t n_padded = (a.n + groups - 1) / groups * groups;
    for (int64_t s = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) / kGroupJ; s < n_padded; s += groups) {
        const bool valid = s < a.n;
        float hi[6], lo[6];
        group_gather9c_j(a.ptr, a.inc, a.wrench, s, valid, lane, hi, lo);
        double r0v = 0.0, r1v = 0.0;
        if (valid && lane < 3) {
            const float h0 = lane == 0 ? hi[0] : (lane == 1 ? hi[2] : hi[4]);
            const float l0 = lane == 0 ? lo[0] : (lane == 1 ? lo[2] : lo[4]);
            const float h1 = lane == 0 ? hi[1] : (lane == 1 ? hi[3] : hi[5]);
            const float l1 = lane == 0 ? lo[1] : (lane == 1 ? lo[3] : lo[5]);
            const int64_t e = 6 * s + 2 * lane;
            const double2 yv = *reinterpret_cast<const double2 *>(a.y + e);
            const double2 mv = *reinterpret_cast<const double2 *>(a.mass + e);
            const double2 rv = *reinterpret_cast<const double2 *>(a.r0 + e);
            const bool fx = a.fixed[s] != 0;
            r0v = fx ? yv.x : fma(mv.x, yv.x, rv.x) - a.half_dt2 * ((double)h0 + (double)l0);
            r1v = fx ? yv.y : fma(mv.y, yv.y, rv.y) - a.half_dt2 * ((double)h1 + (double)l1);
            *reinterpret_cast<double2 *>(a.residual + e) = make_double2(r0v, r1v);
            sum_r = fma(r0v, r0v, sum_r);
            sum_r = fma(r1v, r1v, sum_r);
        }
        if (valid && lane == 0) {
            const double *ys = a.y + 6 * s;
            const float w0 = (float)ys[3], w1 = (float)ys[4], w2 = (float)ys[5];
            if (sqrtf(w0 * w0 + w1 * w1 + w2 * w2) > 0.25f) {
                if (a.seg)
                    atomicOr(a.status + a.seg[s], DPF_ERR_ROTATION);
                else
                    flags |= DPF_ERR_ROTATION;
            }
        }
        if (a.P) {  // uniform over the grid: every lane takes part in the shuffles
            // lanes 0-2 round their two entries to float32, the group shares them
            const float f0 = (float)r0v, f1 = (float)r1v;
            float rf[6];
#pragma unroll
            for (int k = 0; k < 3; ++k) {
                rf[2 * k] = __shfl_sync(0xffffffffu, f0, k, kGroupJ);
                rf[2 * k + 1] = __shfl_sync(0xffffffffu, f1, k, kGroupJ);
            }
            if (valid) {
                const float *P = a.P + 36 * s;
                const float *u = a.units32 + 6 * s;
#pragma unroll
                for (int k = 0; k < (6 + kGroupJ - 1) / kGroupJ; ++k) {
                    const int row = lane + kGroupJ * k;
                    if (row < 6) {
                        const float v = scale_row(P, rf, row, u[row]);
                        if (a.scaled) a.scaled[6 * s + row] = v;
                        max_s = fmaxf(max_s, fabsf(v));
                        add_square(s_hi, s_lo, v);
                    }
                }
            }
        }
    }
    if (flags) atomicOr(a.status, flags);
    if (!a.norms) return;
    finish_norms(sum_r, max_s, s_hi, s_lo, a.partials, 6, a.norms, a.status);
}

// One thread per site, 16-byte loads: the six residual entries (rounded to
// float32 once), the 36-float P block, the six units; s = P r / units.
__global__ void __launch_bounds__(kThreads) scale_sites_f32(int64_t n, const float *P, const float *units32,
                                                            const double *r, double *scaled, double *norms,
                                                            double *partials) {
    double sum_r = 0.0;
    float max_s = 0.0f;
    float s_hi = 0.0f, s_lo = 0.0f;
    for (int64_t s = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; s < n; s += (int64_t)gridDim.x * blockDim.x) {
        const double2 *rp = reinterpret_cast<const double2 *>(r + 6 * s);
        const double2 a0 = rp[0], a1 = rp[1], a2 = rp[2];
        const double rr[6] = {a0.x, a0.y, a1.x, a1.y, a2.x, a2.y};
        float rf[6];
#pragma unroll
        for (int c = 0; c < 6; ++c) {
            sum_r = fma(rr[c], rr[c], sum_r);
            rf[c] = (float)rr[c];
        }
        const float4 *pp = reinterpret_cast<const float4 *>(P + 36 * s);
        float pm[36];
#pragma unroll
        for (int k = 0; k < 9; ++k) {
            const float4 q = pp[k];
            pm[4 * k] = q.x;
            pm[4 * k + 1] = q.y;
            pm[4 * k + 2] = q.z;
            pm[4 * k + 3] = q.w;
        }
        const float2 *up = reinterpret_cast<const float2 *>(units32 + 6 * s);
        const float2 u0 = up[0], u1 = up[1], u2 = up[2];
        const float un[6] = {u0.x, u0.y, u1.x, u1.y, u2.x, u2.y};
        double out[6];
#pragma unroll
        for (int row = 0; row < 6; ++row) {
            float v = 0.0f;
#pragma unroll
            for (int c = 0; c < 6; ++c) v = fmaf(pm[6 * row + c], rf[c], v);
            v = v / un[row];
            max_s = fmaxf(max_s, fabsf(v));
            add_square(s_hi, s_lo, v);
            out[row] = (double)v;
        }
        if (scaled) {
            double2 *sp = reinterpret_cast<double2 *>(scaled + 6 * s);
            sp[0] = make_double2(out[0], out[1]);
            sp[1] = make_double2(out[2], out[3]);
            sp[2] = make_double2(out[4], out[5]);
        }
    }
    if (!norms) return;
    finish_norms(sum_r, max_s, s_hi, s_lo, partials, 7, norms, nullptr);
}

// ---------------------------------------------------------------------------
// JVP: forward-mode derivative of the float32 increment.

struct JvpArgs {
    int64_t m;
    BondData bd;
    const float *y, *d;
    float *wrench;
    const int32_t *seg;     // optional: bonds of inactive segments give zero
    const uint8_t *active;
};

__device__ __forceinline__ V3<Dual> dual3(V3<float> v, V3<float> d) {
    return {{v.x, d.x}, {v.y, d.y}, {v.z, d.z}};
}

// d32 = units * direction in float32 (one conversion per entry; a float32
// direction is taken as it is).
__global__ void __launch_bounds__(kThreads) prepare_direction(int64_t count, const double *direction,
                                                              const float *direction32, const float *units32,
                                                              float *d32) {
    const int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (e >= count) return;
    const float d = direction32 ? direction32[e] : (float)direction[e];
    d32[e] = units32 ? d * units32[e] : d;
}

// Resident 256-thread blocks per SM the JVP bond pass is compiled for (the
// dual-number increment is register heavy); 0 leaves the register count to
// the compiler (99 registers, 2 blocks).  3 blocks (80 registers, 88 bytes of
// spills) measured 156 us per JVP on the 64^3 foam against 168 us for 2 and
// 164 us for 4 (64 registers).  The build may set it.
#ifndef DPF_JVP_BLOCKS_PER_SM
#define DPF_JVP_BLOCKS_PER_SM 3
#endif
#if DPF_JVP_BLOCKS_PER_SM > 0
#define DPF_JVP_BOUNDS __launch_bounds__(kThreads, DPF_JVP_BLOCKS_PER_SM)
#else
#define DPF_JVP_BOUNDS __launch_bounds__(kThreads)
#endif

__global__ void DPF_JVP_BOUNDS jvp_bonds_mixed(JvpArgs a) {
    const int64_t b = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (b >= a.m) return;
    if (a.active && !a.active[a.seg[b]]) {
        store_zero9(a.wrench, b);
        return;
    }
    const Bond B = load_bond(a.bd.rec, b);
    V3<float> ui, wi, uj, wj, dui, dwi, duj, dwj;
    load_y(a.y, B.i, ui, wi);
    load_y(a.y, B.j, uj, wj);
    load_y(a.d, B.i, dui, dwi);
    load_y(a.d, B.j, duj, dwj);
    const BondIncrement<Dual> o =
        bond_increment<Dual>(B, dual3(ui, dui), dual3(wi, dwi), dual3(uj, duj), dual3(wj, dwj));
    store9(a.wrench, b, der3(o.dF), der3(o.dTi), der3(o.dTj));
}

struct JvpSiteArgs {
    int64_t n;
    const int32_t *ptr, *inc;
    const float *wrench, *d, *mass32, *P, *units32;
    const uint8_t *fixed;
    float half_dt2;
    double *out;
    float *out32;  // float32 output instead of out (one of the two)
};

__global__ void __launch_bounds__(kThreads) jvp_sites_mixed(JvpSiteArgs a) {
    const int64_t g = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) / kGroupJ;
    const int lane = threadIdx.x & (kGroupJ - 1);
    const bool valid = g < a.n;
    float hi[6], lo[6], r[6];
    group_gather9c_j(a.ptr, a.inc, a.wrench, g, valid, lane, hi, lo);
    if (!valid) return;
    // every lane of the group holds the sums: each forms the six entries of
    // r (the site's d and mass are one cache line) and writes its rows
    const int64_t s = g;
    const bool fx = a.fixed[s] != 0;
#pragma unroll
    for (int c = 0; c < 6; ++c) {
        // m d - h (hi + lo) with the rounding errors of both products recovered by FMA
        const float d = a.d[6 * s + c], m = a.mass32[6 * s + c];
        const float p = m * d, q = a.half_dt2 * hi[c];
        const float e = fmaf(m, d, -p) - fmaf(a.half_dt2, hi[c], -q) - a.half_dt2 * lo[c];
        r[c] = fx ? d : (p - q) + e;
    }
#pragma unroll
    for (int k = 0; k < (6 + kGroupJ - 1) / kGroupJ; ++k) {
        const int row = lane + kGroupJ * k;
        if (row < 6) {
            float v;
            if (a.P)
                v = scale_row(a.P + 36 * s, r, row, a.units32[6 * s + row]);
            else
                v = row == 0 ? r[0] : row == 1 ? r[1] : row == 2 ? r[2] : row == 3 ? r[3] : row == 4 ? r[4] : r[5];
            if (a.out32)
                a.out32[6 * s + row] = v;
            else
                a.out[6 * s + row] = (double)v;
        }
    }
}

// ---------------------------------------------------------------------------
// Frozen tangent K q in float32 (experiments/bonded_dem_linear_gpu.py:42-52).

__device__ __forceinline__ void stiffness_bond_f32(const BondData &bd, const float *q, float *wrench, int64_t b) {
    const float4 a = __ldg(bd.t0 + b), c = __ldg(bd.t1 + b), e = __ldg(bd.t2 + b), g = __ldg(bd.t3 + b);
    const int i = __float_as_int(g.y), j = __float_as_int(g.z);
    const V3<float> n = {a.x, a.y, a.z}, ri = {c.x, c.y, c.z}, rj = {e.x, e.y, e.z};
    const float kn = a.w, ks = c.w, kb = e.w, kt = g.x;
    const float *qi = q + 6 * (int64_t)i, *qj = q + 6 * (int64_t)j;
    const V3<float> wi = {qi[3], qi[4], qi[5]}, wj = {qj[3], qj[4], qj[5]};
    const V3<float> du = V3<float>{qj[0] - qi[0], qj[1] - qi[1], qj[2] - qi[2]} + cross(wj, rj) - cross(wi, ri);
    const V3<float> dw = wj - wi;
    const V3<float> f = ks * du + ((kn - ks) * dot(du, n)) * n;
    const V3<float> m = kb * dw + ((kt - kb) * dot(dw, n)) * n;
    store9(wrench, b, -f, -cross(ri, f) - m, cross(rj, f) + m);
}

__global__ void __launch_bounds__(kThreads) stiffness_bonds_f32(int64_t m, BondData bd, const float *q, float *w) {
    const int64_t b = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (b < m) stiffness_bond_f32(bd, q, w, b);
}

__global__ void __launch_bounds__(kThreads) to_f32(int64_t n, const double *a, float *out) {
    const int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (e < n) out[e] = (float)a[e];
}

__global__ void __launch_bounds__(kThreads) gather_to_f64(int64_t n, const int32_t *ptr, const int32_t *inc,
                                                          const float *w, double *out) {
    const int64_t s = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (s >= n) return;
    double acc[6];
    gather9(ptr, inc, w, s, acc);
#pragma unroll
    for (int c = 0; c < 6; ++c) out[6 * s + c] = acc[c];
}

// ---------------------------------------------------------------------------
// Blocks and their inverse in float32 (experiments/bonded_dem_newton.py:94-102).

__device__ __forceinline__ void add_block_f32(float D[36], V3<float> n, V3<float> r, float kn, float ks, float kb,
                                              float kt) {
    const float nv[3] = {n.x, n.y, n.z};
    float d[9], h[9];
#pragma unroll
    for (int p = 0; p < 3; ++p)
#pragma unroll
        for (int q = 0; q < 3; ++q) {
            const float nn = nv[p] * nv[q];
            d[3 * p + q] = (p == q ? ks : 0.0f) + (kn - ks) * nn;
            h[3 * p + q] = (p == q ? kb : 0.0f) + (kt - kb) * nn;
        }
    const float S[9] = {0.0f, -r.z, r.y, r.z, 0.0f, -r.x, -r.y, r.x, 0.0f};
    float dS[9];
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
            D[6 * p + 3 + q] -= dS[3 * p + q];
            D[6 * (3 + q) + p] -= dS[3 * p + q];
            D[6 * (3 + p) + 3 + q] += S[p] * dS[q] + S[3 + p] * dS[3 + q] + S[6 + p] * dS[6 + q] + h[3 * p + q];
        }
}

// In-place inverse of a symmetric positive definite 6x6 after symmetric
// diagonal scaling (Jacobi), Cholesky based; A is overwritten with A^-1.
// Every loop has a constant trip count so all indices fold to registers.
__device__ __forceinline__ void spd_inverse6_f32(float A[36]) {
    float sc[6];
#pragma unroll
    for (int p = 0; p < 6; ++p) sc[p] = rsqrtf(A[7 * p]);
#pragma unroll
    for (int p = 0; p < 6; ++p)
#pragma unroll
        for (int q = 0; q < 6; ++q) A[6 * p + q] *= sc[p] * sc[q];
    // Cholesky: the lower triangle of A becomes L
#pragma unroll
    for (int jj = 0; jj < 6; ++jj) {
        float s = A[7 * jj];
#pragma unroll
        for (int kk = 0; kk < 6; ++kk)
            if (kk < jj) s -= A[6 * jj + kk] * A[6 * jj + kk];
        const float l = sqrtf(s);
        A[7 * jj] = l;
        const float inv = 1.0f / l;
#pragma unroll
        for (int ii = 0; ii < 6; ++ii) {
            if (ii > jj) {
                float v = A[6 * ii + jj];
#pragma unroll
                for (int kk = 0; kk < 6; ++kk)
                    if (kk < jj) v -= A[6 * ii + kk] * A[6 * jj + kk];
                A[6 * ii + jj] = v * inv;
            }
        }
    }
    // W = L^-1 (lower triangular), kept in the upper triangle of A as W^T
    float W[36];
#pragma unroll
    for (int ii = 0; ii < 6; ++ii) {
        W[7 * ii] = 1.0f / A[7 * ii];
#pragma unroll
        for (int jj = 0; jj < 6; ++jj) {
            if (jj < ii) {
                float v = 0.0f;
#pragma unroll
                for (int kk = 0; kk < 6; ++kk)
                    if (kk >= jj && kk < ii) v += A[6 * ii + kk] * W[6 * kk + jj];
                W[6 * ii + jj] = -v * W[7 * ii];
            }
        }
    }
    // A^-1 = W^T W, unscaled
#pragma unroll
    for (int ii = 0; ii < 6; ++ii)
#pragma unroll
        for (int jj = 0; jj < 6; ++jj) {
            if (jj <= ii) {
                float v = 0.0f;
#pragma unroll
                for (int kk = 0; kk < 6; ++kk)
                    if (kk >= ii) v += W[6 * kk + ii] * W[6 * kk + jj];
                v *= sc[ii] * sc[jj];
                A[6 * ii + jj] = v;
                A[6 * jj + ii] = v;
            }
        }
}

struct ScalingArgs {
    int64_t n;
    const int32_t *ptr, *inc;
    BondData bd;
    const float *mass32;
    const double *radii;
    const uint8_t *fixed;
    float alpha;
    float *block, *P, *units32;
    double *units;
};

// Packed upper triangle of a symmetric 6x6: k(p, q), p <= q.
__host__ __device__ __forceinline__ constexpr int sym6(int p, int q) {
    return (p < q ? p : q) * 6 - (p < q ? p : q) * ((p < q ? p : q) - 1) / 2 + ((p < q ? q : p) - (p < q ? p : q));
}

// Adds the site-diagonal block of one bond to the packed upper triangle
// (same block as add_block_f32 / experiments/bonded_dem_linear_gpu.py:54-72).
__device__ __forceinline__ void add_block_sym(float D[21], V3<float> n, V3<float> r, float kn, float ks, float kb,
                                              float kt) {
    const float nv[3] = {n.x, n.y, n.z};
    float d[9], h[9];
#pragma unroll
    for (int p = 0; p < 3; ++p)
#pragma unroll
        for (int q = 0; q < 3; ++q) {
            const float nn = nv[p] * nv[q];
            d[3 * p + q] = (p == q ? ks : 0.0f) + (kn - ks) * nn;
            h[3 * p + q] = (p == q ? kb : 0.0f) + (kt - kb) * nn;
        }
    const float S[9] = {0.0f, -r.z, r.y, r.z, 0.0f, -r.x, -r.y, r.x, 0.0f};
    float dS[9];
#pragma unroll
    for (int p = 0; p < 3; ++p)
#pragma unroll
        for (int q = 0; q < 3; ++q)
            dS[3 * p + q] = d[3 * p] * S[q] + d[3 * p + 1] * S[3 + q] + d[3 * p + 2] * S[6 + q];
#pragma unroll
    for (int p = 0; p < 3; ++p)
#pragma unroll
        for (int q = 0; q < 3; ++q) {
            if (p <= q) {
                D[sym6(p, q)] += d[3 * p + q];
                D[sym6(3 + p, 3 + q)] += S[p] * dS[q] + S[3 + p] * dS[3 + q] + S[6 + p] * dS[6 + q] + h[3 * p + q];
            }
            D[sym6(p, 3 + q)] -= dS[3 * p + q];
        }
}

// kScalingLanes lanes per site sum the incident bonds' blocks (more loads in
// flight than one thread walking the site's ~15 incidences), an xor-shuffle
// tree adds the lanes' sums, and lane 0 inverts.
constexpr int kScalingLanes = 4;

__global__ void __launch_bounds__(128) scaling_sites_f32(ScalingArgs a) {
    const int64_t s = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) / kScalingLanes;
    const int lane = threadIdx.x & (kScalingLanes - 1);
    const bool valid = s < a.n;
    float D[21];
#pragma unroll
    for (int c = 0; c < 21; ++c) D[c] = 0.0f;
    if (valid) {
        const int e1 = a.ptr[s + 1];
        for (int e = a.ptr[s] + lane; e < e1; e += kScalingLanes) {
            const int v = a.inc[e];
            const int64_t b = v >= 0 ? v : ~v;
            // (n, kn), this end's (lever, ks or kb), the other stiffness and kt:
            // two 16-byte and two 4-byte loads
            const bool at_i = v >= 0;
            const float4 t0 = __ldg(a.bd.t0 + b), tr = __ldg((at_i ? a.bd.t1 : a.bd.t2) + b);
            const float other_k = __ldg(reinterpret_cast<const float *>((at_i ? a.bd.t2 : a.bd.t1) + b) + 3);
            const float kt = __ldg(reinterpret_cast<const float *>(a.bd.t3 + b));
            const float ks = at_i ? tr.w : other_k, kb = at_i ? other_k : tr.w;
            add_block_sym(D, {t0.x, t0.y, t0.z}, {tr.x, tr.y, tr.z}, t0.w, ks, kb, kt);
        }
    }
#pragma unroll
    for (int o = 1; o < kScalingLanes; o <<= 1)
#pragma unroll
        for (int c = 0; c < 21; ++c) D[c] += __shfl_xor_sync(0xffffffffu, D[c], o);
    if (!valid || lane != 0) return;
    const bool fx = a.fixed[s] != 0;
    float B[36];
#pragma unroll
    for (int p = 0; p < 6; ++p)
#pragma unroll
        for (int q = 0; q < 6; ++q) {
            const float val = (p == q ? a.mass32[6 * s + p] : 0.0f) + a.alpha * D[sym6(p, q)];
            B[6 * p + q] = fx ? (p == q ? 1.0f : 0.0f) : val;
        }
    if (a.block) {
        float4 *out = reinterpret_cast<float4 *>(a.block + 36 * s);
#pragma unroll
        for (int c = 0; c < 9; ++c) out[c] = make_float4(B[4 * c], B[4 * c + 1], B[4 * c + 2], B[4 * c + 3]);
    }
    spd_inverse6_f32(B);
    float4 *out = reinterpret_cast<float4 *>(a.P + 36 * s);
#pragma unroll
    for (int c = 0; c < 9; ++c) out[c] = make_float4(B[4 * c], B[4 * c + 1], B[4 * c + 2], B[4 * c + 3]);
    const double r = fx ? 1.0 : a.radii[s];
#pragma unroll
    for (int c = 0; c < 6; ++c) {
        a.units[6 * s + c] = c < 3 ? r : 1.0;
        a.units32[6 * s + c] = c < 3 ? (float)r : 1.0f;
    }
}

// ---------------------------------------------------------------------------


__device__ __forceinline__ void mv6(const float *P, const float x[6], float y[6]) {
#pragma unroll
    for (int row = 0; row < 6; ++row) {
        float v = 0.0f;
#pragma unroll
        for (int c = 0; c < 6; ++c) v = fmaf(P[6 * row + c], x[c], v);
        y[row] = v;
    }
}



// Elastic PCG in float32 with float64 dot products, one cooperative launch
// (experiments/bonded_dem_newton.py:107-130).  Three grid barriers per
// iteration: the direction update d = z + beta d is folded into the next
// iteration's bond pass (recomputed per endpoint) and site pass (stored).
// Work vectors are 16-byte aligned per site: zd = [z, 0, 0, d, 0, 0] (64 B),
// x, r, ad = [v, 0, 0] (32 B); the bond wrench is three float4 [F, T_i, T_j].

constexpr int kPcgThreads = 1024;

struct PcgArgs {
    int64_t n, m;
    const int32_t *ptr, *inc;
    BondData bd;
    const float *mass32, *units32;
    const double *vector;
    const float *block, *P;
    const uint8_t *fixed;
    float alpha_op;
    double tol2;
    int max_it;
    double *out;
    int *iterations;
    float4 *wrench, *zd, *x, *r, *ad;
    double *part_a, *part_b;
    unsigned *barrier;
    int *status;
    const int32_t *seg;     // optional: bonds of inactive segments are skipped (their direction is zero)
    const uint8_t *active;
};

__device__ __forceinline__ void ld8(const float4 *p, float v[6]) {
    const float4 a = p[0], b = p[1];
    v[0] = a.x; v[1] = a.y; v[2] = a.z; v[3] = a.w; v[4] = b.x; v[5] = b.y;
}
__device__ __forceinline__ void st8(float4 *p, const float v[6]) {
    p[0] = make_float4(v[0], v[1], v[2], v[3]);
    p[1] = make_float4(v[4], v[5], 0.0f, 0.0f);
}

// Direction at a site: z + beta d from the interleaved record.
__device__ __forceinline__ void direction_at(const float4 *zd, int64_t s, float beta, float q[6]) {
    const float4 *p = zd + 4 * s;
    const float4 z0 = p[0], z1 = p[1], d0 = p[2], d1 = p[3];
    q[0] = fmaf(beta, d0.x, z0.x); q[1] = fmaf(beta, d0.y, z0.y); q[2] = fmaf(beta, d0.z, z0.z);
    q[3] = fmaf(beta, d0.w, z0.w); q[4] = fmaf(beta, d1.x, z1.x); q[5] = fmaf(beta, d1.y, z1.y);
}

__device__ __forceinline__ void stiffness_bond_dir(const BondData &bd, const float4 *zd, float beta, float4 *wrench,
                                                   int64_t b) {
    const float4 a = __ldg(bd.t0 + b), c = __ldg(bd.t1 + b), e = __ldg(bd.t2 + b), g = __ldg(bd.t3 + b);
    const int i = __float_as_int(g.y), j = __float_as_int(g.z);
    const V3<float> n = {a.x, a.y, a.z}, ri = {c.x, c.y, c.z}, rj = {e.x, e.y, e.z};
    const float kn = a.w, ks = c.w, kb = e.w, kt = g.x;
    float qi[6], qj[6];
    direction_at(zd, i, beta, qi);
    direction_at(zd, j, beta, qj);
    const V3<float> wi = {qi[3], qi[4], qi[5]}, wj = {qj[3], qj[4], qj[5]};
    const V3<float> du = V3<float>{qj[0] - qi[0], qj[1] - qi[1], qj[2] - qi[2]} + cross(wj, rj) - cross(wi, ri);
    const V3<float> dw = wj - wi;
    const V3<float> f = ks * du + ((kn - ks) * dot(du, n)) * n;
    const V3<float> mm = kb * dw + ((kt - kb) * dot(dw, n)) * n;
    const V3<float> ti = -cross(ri, f) - mm, tj = cross(rj, f) + mm;
    float4 *w = wrench + 3 * b;
    w[0] = make_float4(-f.x, -f.y, -f.z, 0.0f);
    w[1] = make_float4(ti.x, ti.y, ti.z, 0.0f);
    w[2] = make_float4(tj.x, tj.y, tj.z, 0.0f);
}

__device__ __forceinline__ void group_gather_w4(const int32_t *__restrict__ ptr, const int32_t *__restrict__ inc,
                                                const float4 *__restrict__ w, int64_t s, bool valid, int lane,
                                                float acc[6]) {
#pragma unroll
    for (int c = 0; c < 6; ++c) acc[c] = 0.0f;
    if (valid) {
        const int e1 = ptr[s + 1];
        for (int e = ptr[s] + lane; e < e1; e += kGroup) {
            const int v = inc[e];
            const int64_t b = v >= 0 ? v : ~v;
            const float4 f = w[3 * b];
            const float4 t = w[3 * b + (v >= 0 ? 1 : 2)];
            const float sg = v >= 0 ? 1.0f : -1.0f;
            acc[0] = fmaf(sg, f.x, acc[0]);
            acc[1] = fmaf(sg, f.y, acc[1]);
            acc[2] = fmaf(sg, f.z, acc[2]);
            acc[3] += t.x;
            acc[4] += t.y;
            acc[5] += t.z;
        }
    }
#pragma unroll
    for (int o = 1; o < kGroup; o <<= 1)
#pragma unroll
        for (int c = 0; c < 6; ++c) acc[c] += __shfl_xor_sync(0xffffffffu, acc[c], o);
}

__global__ void __launch_bounds__(kPcgThreads) pcg_kernel_f32(PcgArgs a) {
    const int64_t tid = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    const float zero6[6] = {0.0f, 0.0f, 0.0f, 0.0f, 0.0f, 0.0f};
    float pf = 0.0f;
    for (int64_t s = tid; s < a.n; s += stride) {
        float u[6], rr[6], zz[6];
#pragma unroll
        for (int c = 0; c < 6; ++c) u[c] = a.units32[6 * s + c] * (float)a.vector[6 * s + c];
        if (a.fixed[s]) {
#pragma unroll
            for (int c = 0; c < 6; ++c) rr[c] = 0.0f;
        } else {
            mv6(a.block + 36 * s, u, rr);
        }
        mv6(a.P + 36 * s, rr, zz);
        st8(a.x + 2 * s, zero6);
        st8(a.r + 2 * s, rr);
        st8(a.zd + 4 * s, zz);
        st8(a.zd + 4 * s + 2, zero6);
#pragma unroll
        for (int c = 0; c < 6; ++c) pf = fmaf(rr[c], zz[c], pf);
    }
    double p = block_sum((double)pf);
    if (threadIdx.x == 0) a.part_b[blockIdx.x] = p;
    if (!grid_barrier(a.barrier, a.status)) return;
    double rz = block_sum_array(a.part_b, gridDim.x);
    const double initial = rz;
    if (initial == 0.0) {
        for (int64_t e = tid; e < 6 * a.n; e += stride) a.out[e] = 0.0;
        return;
    }
    const int lane = threadIdx.x & (kGroup - 1);
    const int64_t groups = stride / kGroup;
    const int64_t n_padded = (a.n + groups - 1) / groups * groups;
    float beta = 0.0f;
    int it = 0;
    for (; it < a.max_it; ++it) {
        // K d_k with d_k = z_k + beta d_{k-1} formed per endpoint
#pragma unroll 2
        for (int64_t b = tid; b < a.m; b += stride) {
            if (a.active && !a.active[a.seg[b]]) {
                float4 *w = a.wrench + 3 * b;
                w[0] = w[1] = w[2] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
                continue;
            }
            stiffness_bond_dir(a.bd, a.zd, beta, a.wrench, b);
        }
        if (!grid_barrier(a.barrier, a.status)) return;
        // ad = (diag M + alpha K) d_k with identity rows on fixed sites; store d_k
        pf = 0.0f;
        for (int64_t s = tid / kGroup; s < n_padded; s += groups) {
            const bool valid = s < a.n;
            float acc[6];
            group_gather_w4(a.ptr, a.inc, a.wrench, s, valid, lane, acc);
            if (valid && lane == 0) {
                const bool fx = a.fixed[s] != 0;
                float dv[6], v[6];
                direction_at(a.zd, s, beta, dv);
#pragma unroll
                for (int c = 0; c < 6; ++c) {
                    const float m = a.mass32[6 * s + c];
                    v[c] = fx ? dv[c] : fmaf(m, dv[c], a.alpha_op * acc[c]);
                    pf = fmaf(dv[c], v[c], pf);
                }
                st8(a.zd + 4 * s + 2, dv);
                st8(a.ad + 2 * s, v);
            }
        }
        p = block_sum((double)pf);
        if (threadIdx.x == 0) a.part_a[blockIdx.x] = p;
        if (!grid_barrier(a.barrier, a.status)) return;
        const float alpha = (float)block_divide(rz, block_sum_array(a.part_a, gridDim.x));
        pf = 0.0f;
        for (int64_t s = tid; s < a.n; s += stride) {
            float xv[6], rv[6], dv[6], av[6], zz[6];
            ld8(a.x + 2 * s, xv);
            ld8(a.r + 2 * s, rv);
            ld8(a.zd + 4 * s + 2, dv);
            ld8(a.ad + 2 * s, av);
#pragma unroll
            for (int c = 0; c < 6; ++c) {
                xv[c] = fmaf(alpha, dv[c], xv[c]);
                rv[c] = fmaf(-alpha, av[c], rv[c]);
            }
            mv6(a.P + 36 * s, rv, zz);
            st8(a.x + 2 * s, xv);
            st8(a.r + 2 * s, rv);
            st8(a.zd + 4 * s, zz);
#pragma unroll
            for (int c = 0; c < 6; ++c) pf = fmaf(rv[c], zz[c], pf);
        }
        p = block_sum((double)pf);
        if (threadIdx.x == 0) a.part_b[blockIdx.x] = p;
        if (!grid_barrier(a.barrier, a.status)) return;
        const double following = block_sum_array(a.part_b, gridDim.x);
        if (it % 5 == 0 && following <= a.tol2 * initial) break;
        beta = (float)block_divide(following, rz);
        rz = following;
    }
    for (int64_t s = tid; s < a.n; s += stride) {
        float xv[6];
        ld8(a.x + 2 * s, xv);
#pragma unroll
        for (int c = 0; c < 6; ++c) a.out[6 * s + c] = (double)(xv[c] / a.units32[6 * s + c]);
    }
    if (tid == 0) atomicAdd(a.iterations, it < a.max_it ? it + 1 : a.max_it);
}

// ---------------------------------------------------------------------------
// End state of an accepted increment (experiments/bonded_dem_finite_gpu.py:102-116):
// float32 increments added to the float64 committed history.

struct CommitArgs {
    int64_t m;
    BondData bd;
    dpf_history h;
    const float *y32;
    const double *x_end;  // end positions x + y, formed first by end_positions
    double *normal_end, *offset_end, *fs_end, *mb_end, *fn_end, *mt_end;
    float *dloads;  // optional: increment of the committed loads (a wrench record per bond)
    float4 *corr;   // lazy form: corrections of the records' float32 state (3 float4 arrays of m)
};

// Lazy float64 history: the bond records carry fn, mt, fs, mb and offset in
// float32 and advance them every step; per bond three float4 corrections
// (fs, fn), (mb, mt), (offset, -) hold what float32 rounding dropped, so that
// (double)record + (double)correction is the float64 history (to about 48
// bits).  A float64 setup writes the records and their corrections from the
// history; each lazy commit adds the exact rounding error of each record
// update (TwoSum) to the correction; a fold forms the history from both.
constexpr int kCorrArrays = 3;

// s = a + b rounded as the record update rounds it; returns the exact error
// a + b - s (Knuth's TwoSum)
__device__ __forceinline__ float sum_error(float a, float b, float s) {
    const float bp = s - a;
    return (a - (s - bp)) + (b - bp);
}

// x_end = x + u per site, before the bond pass reads it.
__global__ void __launch_bounds__(kThreads) end_positions(int64_t n, const double *x, const double *y, double *x_end) {
    const int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (e >= 3 * n) return;
    const int64_t s = e / 3;
    x_end[e] = x[e] + y[6 * s + (e - 3 * s)];
}

// End state of the accepted increment; with dloads it also rewrites the bond
// records for the next step in place (the bond's own record only) and emits
// loads(x_end) - loads(x) per bond as float32 increments.
// 3 resident blocks per SM (80 registers) rather than 2 (88 registers).
// end normal and length in float64 from the end positions (geometry(end));
// one reciprocal square root instead of a square root and a division (float64
// arithmetic is scarce on this part).  The fold of the lazy form uses it too.
__device__ __forceinline__ d3 end_normal(const double *x, int64_t i, int64_t j, double &length) {
    const d3 de = ld3(x, j) - ld3(x, i);
    const double l2 = dot(de, de);
    const double inv = rsqrt(l2);
    length = l2 * inv;
    return inv * de;
}

// kLazy: the float64 end state is not written; the records' rounding errors
// go to the corrections a.corr (dpf_mixed_fold_history forms the history).
template <bool kLazy>
__global__ void __launch_bounds__(kThreads, 3) commit_bonds(CommitArgs a) {
    const int64_t b = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (b >= a.m) return;
    const Bond B = load_bond(a.bd.rec, b);
    V3<float> ui, wi, uj, wj;
    load_y(a.y32, B.i, ui, wi);
    load_y(a.y32, B.j, uj, wj);
    const BondIncrement<float> o = bond_increment<float>(B, ui, wi, uj, wj);
    const float dfn = B.kn * value(o.dn), dmt = B.kt * value(o.tw);
    if (!kLazy) {
        a.fn_end[b] = a.h.fn[b] + (double)dfn;
        a.mt_end[b] = a.h.mt[b] + (double)dmt;
    }
    double le64;
    const d3 ne = end_normal(a.x_end, B.i, B.j, le64);
    if (!kLazy) st3(a.normal_end, b, ne);
    const V3<float> nx = lift3<float>(B.n0) + lift3<float>(B.dn0);
    float le;
    const V3<float> dnx_e = normal_change(B.L0, nx, uj - ui, le);
    const TransportInc<float> t2 = make_transport_inc(o.n, dnx_e - o.dn_x, 0.25f * (wi + wj));
    const V3<float> fs1 = lift3<float>(B.fs) + o.dfs1;
    const V3<float> mb1 = lift3<float>(B.mb) + o.dmb1;
    const V3<float> off1 = lift3<float>(B.off) + o.doff;
    const V3<float> dfs = o.dfs1 + t2.apply(fs1);
    const V3<float> dmb = o.dmb1 + t2.apply(mb1);
    const V3<float> doff = o.doff + t2.apply(off1);
    if (!kLazy) {
        st3(a.fs_end, b, ld3(a.h.fs, b) + mk(dfs.x, dfs.y, dfs.z));
        st3(a.mb_end, b, ld3(a.h.mb, b) + mk(dmb.x, dmb.y, dmb.z));
        st3(a.offset_end, b, ld3(a.h.offset, b) + mk(doff.x, doff.y, doff.z));
    }
    if (!a.dloads) return;
    // loads(x_end) - loads(x) of this bond from the small increments
    const V3<float> ne32 = nx + dnx_e;
    const V3<float> fx = B.fn * nx + lift3<float>(B.fs);
    const V3<float> dF = dfn * ne32 + B.fn * dnx_e + dfs;
    const V3<float> dcp = dmt * ne32 + B.mt * dnx_e + dmb;
    const V3<float> f_new = fx + dF;
    const V3<float> dc = 0.5f * (ui + uj) + B.rh * dnx_e + doff;
    const V3<float> ri_x = lift3<float>(B.ri_x), rj_x = ri_x - B.L0 * nx;
    const V3<float> dTi = cross(dc - ui, f_new) + cross(ri_x, dF) + dcp;
    const V3<float> dTj = -(cross(dc - uj, f_new) + cross(rj_x, dF) + dcp);
    store9(a.dloads, b, dF, dTi, dTj);
    // records of the next step: n0 = normal_end (= geometry(x_end), so dn0 = 0);
    // the other fields are float32 quantities, formed in float32
    const float3 ne32f = tof3(ne);
    const float le32 = (float)le64;
    const V3<float> nef = {ne32f.x, ne32f.y, ne32f.z};
    const V3<float> ri_end = (0.5f * le32) * nef + B.rh * nef + (lift3<float>(B.off) + doff);
    const V3<float> fsr = lift3<float>(B.fs) + dfs, mbr = lift3<float>(B.mb) + dmb, offr = lift3<float>(B.off) + doff;
    const float fnr = B.fn + dfn, mtr = B.mt + dmt;
    if (kLazy) {
        float4 *C = a.corr;
        const int64_t m = a.m;
        float4 c0 = C[b], c1 = C[m + b], c2 = C[2 * m + b];
        c0.x += sum_error(B.fs.x, dfs.x, fsr.x);
        c0.y += sum_error(B.fs.y, dfs.y, fsr.y);
        c0.z += sum_error(B.fs.z, dfs.z, fsr.z);
        c0.w += sum_error(B.fn, dfn, fnr);
        c1.x += sum_error(B.mb.x, dmb.x, mbr.x);
        c1.y += sum_error(B.mb.y, dmb.y, mbr.y);
        c1.z += sum_error(B.mb.z, dmb.z, mbr.z);
        c1.w += sum_error(B.mt, dmt, mtr);
        c2.x += sum_error(B.off.x, doff.x, offr.x);
        c2.y += sum_error(B.off.y, doff.y, offr.y);
        c2.z += sum_error(B.off.z, doff.z, offr.z);
        C[b] = c0;
        C[m + b] = c1;
        C[2 * m + b] = c2;
    }
    a.bd.rec.r0[b] = make_float4(ne32f.x, ne32f.y, ne32f.z, le32);
    a.bd.rec.r1[b] = make_float4(0.0f, 0.0f, 0.0f, B.rh);
    a.bd.rec.r2[b] = make_float4(ri_end.x, ri_end.y, ri_end.z, fnr);
    // the next step's tangent at y = 0 (dn0 = 0: n = n0, ri = ri_x, rj = ri_x - L0 n0,
    // what the residual pass forms there), so that its first residual needs no bond pass
    const V3<float> rj_end = ri_end - le32 * nef;
    a.bd.t0[b] = make_float4(nef.x, nef.y, nef.z, B.kn);
    a.bd.t1[b] = make_float4(ri_end.x, ri_end.y, ri_end.z, B.ks);
    a.bd.t2[b] = make_float4(rj_end.x, rj_end.y, rj_end.z, B.kb);
    a.bd.rec.r3[b] = make_float4(fsr.x, fsr.y, fsr.z, mtr);
    a.bd.rec.r4[b] = make_float4(mbr.x, mbr.y, mbr.z, B.kn);
    a.bd.rec.r5[b] = make_float4(offr.x, offr.y, offr.z, B.ks);
}

// loads += site sum of the load increments.
__global__ void __launch_bounds__(kThreads) commit_sites(int64_t n, const int32_t *ptr, const int32_t *inc,
                                                         const float *dloads, double *loads) {
    const int64_t g = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) / kGroupJ;
    const int lane = threadIdx.x & (kGroupJ - 1);
    const bool valid = g < n;
    float hi[6], lo[6];
    group_gather9c_j(ptr, inc, dloads, g, valid, lane, hi, lo);
    if (valid && lane == 0) {
#pragma unroll
        for (int c = 0; c < 6; ++c) loads[6 * g + c] += (double)hi[c] + (double)lo[c];
    }
}

struct FoldArgs {
    int64_t m;
    const int64_t *edges;
    const double *x;
    Records rec;
    const float4 *corr;
    double *normal, *offset, *fn, *fs, *mt, *mb;
};

// history = (double)record + (double)correction, normal = geometry(x)
__global__ void __launch_bounds__(kThreads) fold_history(FoldArgs a) {
    const int64_t b = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (b >= a.m) return;
    double length;
    st3(a.normal, b, end_normal(a.x, a.edges[2 * b], a.edges[2 * b + 1], length));
    const int64_t m = a.m;
    const float4 c0 = a.corr[b], c1 = a.corr[m + b], c2 = a.corr[2 * m + b];
    const float4 r2 = a.rec.r2[b], r3 = a.rec.r3[b], r4 = a.rec.r4[b], r5 = a.rec.r5[b];
    const auto pair = [](float v, float c) { return (double)v + (double)c; };
    a.fn[b] = pair(r2.w, c0.w);
    a.mt[b] = pair(r3.w, c1.w);
    st3(a.fs, b, mk(pair(r3.x, c0.x), pair(r3.y, c0.y), pair(r3.z, c0.z)));
    st3(a.mb, b, mk(pair(r4.x, c1.x), pair(r4.y, c1.y), pair(r4.z, c1.z)));
    st3(a.offset, b, mk(pair(r5.x, c2.x), pair(r5.y, c2.y), pair(r5.z, c2.z)));
}

// corrections = history - (double)record after a float64 setup wrote the records
struct CorrArgs {
    int64_t m;
    dpf_history h;
    Records rec;
    float4 *corr;
};

__global__ void __launch_bounds__(kThreads) history_corrections(CorrArgs a) {
    const int64_t b = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (b >= a.m) return;
    const float4 r2 = a.rec.r2[b], r3 = a.rec.r3[b], r4 = a.rec.r4[b], r5 = a.rec.r5[b];
    const auto gap = [](double h, float v) { return (float)(h - (double)v); };
    const d3 fs = ld3(a.h.fs, b), mb = ld3(a.h.mb, b), off = ld3(a.h.offset, b);
    const int64_t m = a.m;
    a.corr[b] = make_float4(gap(fs.x, r3.x), gap(fs.y, r3.y), gap(fs.z, r3.z), gap(a.h.fn[b], r2.w));
    a.corr[m + b] = make_float4(gap(mb.x, r4.x), gap(mb.y, r4.y), gap(mb.z, r4.z), gap(a.h.mt[b], r3.w));
    a.corr[2 * m + b] = make_float4(gap(off.x, r5.x), gap(off.y, r5.y), gap(off.z, r5.z), 0.0f);
}

// Residual at y = 0 after a commit: the records' increments vanish there, so
// r = r0 on free sites and 0 (= y) on fixed ones; y32 = 0.
__global__ void __launch_bounds__(kThreads) initial_residual(int64_t n, const double *r0, const uint8_t *fixed,
                                                             float *y32, double *residual) {
    const int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (e >= 6 * n) return;
    residual[e] = fixed[e / 6] ? 0.0 : r0[e];
    y32[e] = 0.0f;
}

// Per-step constants from maintained loads: r0 and the rhs scale terms.
struct BeginArgs {
    int64_t n;
    const double *loads, *mass, *v, *external;
    const uint8_t *fixed;
    double dt, half_dt2;
    double *r0, *scales, *partials;
};

__global__ void __launch_bounds__(kThreads) begin_sites(BeginArgs a) {
    double a2 = 0.0, l2 = 0.0;
    for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < 6 * a.n; e += (int64_t)gridDim.x * blockDim.x) {
        const double mv = a.dt * a.mass[e] * a.v[e];
        const double rhs = mv + a.half_dt2 * a.external[e];
        a2 += rhs * rhs;
        const double L = a.loads[e];
        if (!a.fixed[e / 6]) l2 += L * L;
        a.r0[e] = -mv - a.half_dt2 * (L + a.external[e]);
    }
    a2 = block_sum(a2);
    l2 = block_sum(l2);
    double *part = a.partials + kPartialsOffset;
    if (threadIdx.x == 0) {
        part[2 * blockIdx.x] = a2;
        part[2 * blockIdx.x + 1] = l2;
    }
    if (last_block(counter_slot(a.partials, 5))) {
        const double sa = block_sum_array(part, gridDim.x, 2);
        const double sl = block_sum_array(part + 1, gridDim.x, 2);
        if (threadIdx.x == 0) {
            a.scales[0] = sqrt(sa);
            a.scales[1] = sqrt(sl);
        }
    }
}


// ---------------------------------------------------------------------------
// Segmented (per-request) reductions and updates for batches of requests
// stored as contiguous site ranges [seg_ptr[r], seg_ptr[r+1]).

// out[r] = [|a|_2, max|a|, |b|_2 or a.b] over the segment's 6-vectors,
// skipping masked sites (mask[s] != 0) when mask is given.  kSegChunks blocks
// per segment (blockIdx.x), each over a fixed slice of it, write partials; a
// second pass adds a segment's partials in slice order: deterministic and
// independent of the other segments.
constexpr int kSegChunks = 16;

__global__ void __launch_bounds__(kThreads) segment_norms_kernel(const int64_t *seg_ptr, const double *a,
                                                                 const double *b, int b_dot, const uint8_t *mask,
                                                                 double *partials) {
    const int r = blockIdx.y, c = blockIdx.x;
    const int64_t s0 = seg_ptr[r], s1 = seg_ptr[r + 1];
    const int64_t per = (s1 - s0 + kSegChunks - 1) / kSegChunks;
    const int64_t lo = s0 + c * per < s1 ? s0 + c * per : s1, hi = lo + per < s1 ? lo + per : s1;
    double s2 = 0.0, mx = 0.0, t = 0.0;
    for (int64_t e = 6 * lo + threadIdx.x; e < 6 * hi; e += blockDim.x) {
        if (mask && mask[e / 6]) continue;
        const double v = a[e];
        s2 = fma(v, v, s2);
        mx = fmax(mx, fabs(v));
        if (b) t = fma(b_dot ? v : b[e], b[e], t);
    }
    s2 = block_sum(s2);
    mx = block_max(mx);
    t = block_sum(t);
    if (threadIdx.x == 0) {
        double *p = partials + 3 * ((int64_t)r * kSegChunks + c);
        p[0] = s2;
        p[1] = mx;
        p[2] = t;
    }
}

__global__ void segment_finish_kernel(int n_segments, const double *partials, int b_dot, double *out) {
    const int r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= n_segments) return;
    double s2 = 0.0, mx = 0.0, t = 0.0;
    for (int c = 0; c < kSegChunks; ++c) {
        const double *p = partials + 3 * ((int64_t)r * kSegChunks + c);
        s2 += p[0];
        mx = fmax(mx, p[1]);
        t += p[2];
    }
    out[3 * r] = sqrt(s2);
    out[3 * r + 1] = mx;
    out[3 * r + 2] = b_dot ? t : sqrt(t);
}

// out = a + factor[seg[s]] * c on every site (factor 0 leaves a).
__global__ void __launch_bounds__(kThreads) segment_axpy_kernel(int64_t n, const int32_t *seg, const double *factor,
                                                                const double *a, const double *c, double *out) {
    const int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (e >= 6 * n) return;
    out[e] = fma(factor[seg[e / 6]], c[e], a[e]);
}

// out = keep[seg[s]] ? a : b  (per-segment select of 6-vectors).
__global__ void __launch_bounds__(kThreads) segment_select_kernel(int64_t n, const int32_t *seg,
                                                                  const uint8_t *keep, const double *a,
                                                                  const double *b, double *out) {
    const int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (e >= 6 * n) return;
    out[e] = keep[seg[e / 6]] ? a[e] : b[e];
}

}  // namespace mp
}  // namespace dpf

using namespace dpf;
using namespace dpf::mp;

extern "C" {

int64_t dpf_mixed_bond_floats(int64_t n_bonds) { return 4 * 11 * n_bonds; }

int64_t dpf_mixed_wrench_floats(int64_t n_bonds) { return n_bonds < 0 ? 0 : kWrenchFloats * n_bonds; }

static bool aligned16(const void *p) { return ((uintptr_t)p & 15u) == 0; }

int64_t dpf_mixed_workspace_floats(int64_t n_sites, int64_t n_bonds) {
    return 40 * n_sites + 12 * n_bonds + 4 * (int64_t)kMaxPcgBlocks;
}

static bool mixed_graph_ok(const dpf_graph *g) {
    return g && g->n_sites > 0 && g->n_bonds >= 0 && g->n_bonds < (int64_t(1) << 31) && g->inc_ptr &&
           (g->n_bonds == 0 || g->inc_bond);
}

int dpf_mixed_setup(const dpf_graph *g, const dpf_stiffness *k, const dpf_history *h, const double *mass,
                    const double *v, const double *external, const uint8_t *fixed, double dt, float *bond_data,
                    double *r0, double *loads, double *scales, double *wrench, float *corrections,
                    double *partials, int *status, void *stream) {
    if (!mixed_graph_ok(g) || !k || !h || !h->x || !h->radii ||
        (g->n_bonds && (!h->normal || !h->offset || !h->fn || !h->fs || !h->mt || !h->mb)) || !mass || !v ||
        !external || !fixed || !bond_data || !r0 || !scales || !partials || !status ||
        (g->n_bonds && (!wrench || !g->edges)) || ((uintptr_t)corrections & 15u))
        return DPF_ERR_ARGUMENT;
    cudaStream_t st = (cudaStream_t)stream;
    if (g->n_bonds) {
        SetupArgs a{g->n_bonds, g->edges, *k, *h, split_bond_data(bond_data, g->n_bonds), wrench,
                    reinterpret_cast<float4 *>(corrections), status};
        setup_bonds<<<blocks_for(g->n_bonds, kThreads), kThreads, 0, st>>>(a);
    }
    SetupSiteArgs s{g->n_sites, g->inc_ptr, g->inc_bond, wrench, mass, v, external, fixed, dt, 0.5 * dt * dt,
                    r0, loads, scales, partials};
    setup_sites<<<reduce_grid(g->n_sites), kThreads, 0, st>>>(s);
    DPF_CHECK_LAUNCH();
    return DPF_OK;
}

int dpf_mixed_residual_segmented(const dpf_graph *g, float *bond_data, const double *y, const float *y32,
                                 const double *mass, const uint8_t *fixed, double dt, const double *r0,
                                 int want_tangent, const float *preconditioner, const float *units32, double *residual,
                                 double *scaled, double *norms, float *wrench, double *partials, int *status,
                                 const int32_t *seg_bond, const int32_t *seg_site, const uint8_t *active,
                                 void *stream);

int dpf_mixed_residual(const dpf_graph *g, float *bond_data, const double *y, const float *y32, const double *mass,
                       const uint8_t *fixed, double dt, const double *r0, int want_tangent, const float *preconditioner,
                       const float *units32, double *residual, double *scaled, double *norms, float *wrench,
                       double *partials, int *status, void *stream) {
    return dpf_mixed_residual_segmented(g, bond_data, y, y32, mass, fixed, dt, r0, want_tangent, preconditioner,
                                        units32, residual, scaled, norms, wrench, partials, status, nullptr, nullptr,
                                        nullptr, stream);
}

int dpf_mixed_residual_segmented(const dpf_graph *g, float *bond_data, const double *y, const float *y32,
                                 const double *mass, const uint8_t *fixed, double dt, const double *r0,
                                 int want_tangent, const float *preconditioner, const float *units32, double *residual,
                                 double *scaled, double *norms, float *wrench, double *partials, int *status,
                                 const int32_t *seg_bond, const int32_t *seg_site, const uint8_t *active,
                                 void *stream) {
    if (!mixed_graph_ok(g) || !bond_data || !y || !y32 || !mass || !fixed || !r0 || !residual || !status ||
        (g->n_bonds && !wrench) || (norms && !partials) || (preconditioner && !units32) || (active && !seg_bond))
        return DPF_ERR_ARGUMENT;
    // the site pass moves y, mass, r0 and the residual in 16-byte pairs and P in 8-byte pairs;
    // wrench records are 16-byte quads
    if ((((uintptr_t)y | (uintptr_t)mass | (uintptr_t)r0 | (uintptr_t)residual) & 15u) ||
        ((uintptr_t)preconditioner & 7u) || !aligned16(wrench))
        return DPF_ERR_ARGUMENT;
    cudaStream_t st = (cudaStream_t)stream;
    if (g->n_bonds) {
        ResidualBondArgs a{g->n_bonds, split_bond_data(bond_data, g->n_bonds), y32, want_tangent, wrench, status,
                           seg_bond, active};
        residual_bonds<<<blocks_for(g->n_bonds, kThreads), kThreads, 0, st>>>(a);
    }
    ResidualSiteArgs s{g->n_sites, g->inc_ptr, g->inc_bond, wrench, y, mass, r0, fixed, 0.5 * dt * dt,
                       preconditioner, units32, residual, scaled, norms, partials, status, seg_site};
    residual_sites<<<reduce_grid(kGroupJ * g->n_sites), kThreads, 0, st>>>(s);
    DPF_CHECK_LAUNCH();
    return DPF_OK;
}

int dpf_mixed_scaling(const dpf_graph *g, float *bond_data, const float *mass32, const uint8_t *fixed,
                      const double *radii, double dt, float *block, float *preconditioner, double *units,
                      float *units32, void *stream) {
    if (!mixed_graph_ok(g) || !bond_data || !mass32 || !fixed || !radii || !preconditioner || !units || !units32)
        return DPF_ERR_ARGUMENT;
    ScalingArgs a{g->n_sites, g->inc_ptr, g->inc_bond, split_bond_data(bond_data, g->n_bonds), mass32, radii, fixed,
                  (float)(0.25 * dt * dt), block, preconditioner, units32, units};
    scaling_sites_f32<<<blocks_for(kScalingLanes * g->n_sites, 128), 128, 0, (cudaStream_t)stream>>>(a);
    DPF_CHECK_LAUNCH();
    return DPF_OK;
}

int dpf_mixed_scale_residual(int64_t n_sites, const float *preconditioner, const float *units32,
                             const double *residual, double *scaled, double *norms, double *partials, void *stream) {
    // P in 16-byte quads, units in 8-byte pairs, residual and scaled in 16-byte pairs
    if (n_sites <= 0 || !preconditioner || !units32 || !residual || (norms && !partials) ||
        ((uintptr_t)preconditioner & 15u) || ((uintptr_t)units32 & 7u) || ((uintptr_t)residual & 15u) ||
        ((uintptr_t)scaled & 15u))
        return DPF_ERR_ARGUMENT;
    scale_sites_f32<<<reduce_grid(n_sites), kThreads, 0, (cudaStream_t)stream>>>(n_sites, preconditioner, units32,
                                                                                  residual, scaled, norms, partials);
    DPF_CHECK_LAUNCH();
    return DPF_OK;
}

static int mixed_jvp(const dpf_graph *g, float *bond_data, const float *y32, const double *direction,
                     const float *direction32, const float *mass32, const uint8_t *fixed, double dt,
                     const float *units32, const float *preconditioner, double *out, float *out32, float *d32,
                     float *wrench, const int32_t *seg_bond, const uint8_t *active, void *stream) {
    if (!mixed_graph_ok(g) || !bond_data || !y32 || (!direction && !direction32) || !mass32 || !fixed ||
        (!out && !out32) || !d32 || (g->n_bonds && !wrench) || (preconditioner && !units32) ||
        (active && !seg_bond) || ((uintptr_t)preconditioner & 7u) ||  // rows of P are read in 8-byte pairs
        !aligned16(wrench))
        return DPF_ERR_ARGUMENT;
    cudaStream_t st = (cudaStream_t)stream;
    const int64_t n6 = 6 * g->n_sites;
    prepare_direction<<<blocks_for(n6, kThreads), kThreads, 0, st>>>(n6, direction32 ? nullptr : direction,
                                                                     direction32, units32, d32);
    if (g->n_bonds) {
        JvpArgs a{g->n_bonds, split_bond_data(bond_data, g->n_bonds), y32, d32, wrench, seg_bond, active};
        jvp_bonds_mixed<<<blocks_for(g->n_bonds, kThreads), kThreads, 0, st>>>(a);
    }
    JvpSiteArgs s{g->n_sites, g->inc_ptr, g->inc_bond, wrench, d32, mass32, preconditioner, units32, fixed,
                  (float)(0.5 * dt * dt), out32 ? nullptr : out, out32};
    jvp_sites_mixed<<<blocks_for(kGroupJ * g->n_sites, kThreads), kThreads, 0, st>>>(s);
    DPF_CHECK_LAUNCH();
    return DPF_OK;
}

int dpf_mixed_jacobian_vector(const dpf_graph *g, float *bond_data, const float *y32, const double *direction,
                              const float *mass32, const uint8_t *fixed, double dt, const float *units32,
                              const float *preconditioner, double *out, float *d32, float *wrench,
                              const int32_t *seg_bond, const uint8_t *active, void *stream) {
    if (!direction || !out) return DPF_ERR_ARGUMENT;
    return mixed_jvp(g, bond_data, y32, direction, nullptr, mass32, fixed, dt, units32, preconditioner, out, nullptr,
                     d32, wrench, seg_bond, active, stream);
}

int dpf_mixed_jacobian_vector_f32(const dpf_graph *g, float *bond_data, const float *y32, const float *direction,
                                  const float *mass32, const uint8_t *fixed, double dt, const float *units32,
                                  const float *preconditioner, float *out, float *d32, float *wrench, void *stream) {
    if (!direction || !out) return DPF_ERR_ARGUMENT;
    return mixed_jvp(g, bond_data, y32, nullptr, direction, mass32, fixed, dt, units32, preconditioner, nullptr, out,
                     d32, wrench, nullptr, nullptr, stream);
}

int dpf_mixed_stiffness_apply(const dpf_graph *g, float *bond_data, const float *q, double *out, float *wrench,
                              void *stream) {
    if (!mixed_graph_ok(g) || !bond_data || !q || !out || (g->n_bonds && !wrench) || !aligned16(wrench))
        return DPF_ERR_ARGUMENT;
    cudaStream_t st = (cudaStream_t)stream;
    if (g->n_bonds)
        stiffness_bonds_f32<<<blocks_for(g->n_bonds, kThreads), kThreads, 0, st>>>(
            g->n_bonds, split_bond_data(bond_data, g->n_bonds), q, wrench);
    gather_to_f64<<<blocks_for(g->n_sites, kThreads), kThreads, 0, st>>>(g->n_sites, g->inc_ptr, g->inc_bond,
                                                                          wrench, out);
    DPF_CHECK_LAUNCH();
    return DPF_OK;
}

int dpf_to_float(int64_t count, const double *a, float *out, void *stream) {
    if (count <= 0 || !a || !out) return DPF_ERR_ARGUMENT;
    to_f32<<<blocks_for(count, kThreads), kThreads, 0, (cudaStream_t)stream>>>(count, a, out);
    DPF_CHECK_LAUNCH();
    return DPF_OK;
}

struct MixedDeviceInfo {
    int sms = 0, blocks_per_sm = 0;
};

static MixedDeviceInfo &mixed_info() {
    static MixedDeviceInfo info[64];
    int dev = 0;
    cudaGetDevice(&dev);
    MixedDeviceInfo &d = info[dev & 63];
    if (d.sms == 0) {
        cudaDeviceGetAttribute(&d.sms, cudaDevAttrMultiProcessorCount, dev);
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&d.blocks_per_sm, pcg_kernel_f32, kPcgThreads, 0);
    }
    return d;
}

int dpf_mixed_precondition(const dpf_graph *g, float *bond_data, const float *mass32, const uint8_t *fixed,
                           const float *block, const float *preconditioner, const float *units32,
                           const double *vector, double dt, double tolerance, int max_iterations, double *out,
                           int *iterations, float *wrench, float *workspace, unsigned *barrier, int *status,
                           const int32_t *seg_bond, const uint8_t *active, void *stream) {
    if (!mixed_graph_ok(g) || !bond_data || !mass32 || !fixed || !block || !preconditioner || !units32 || !vector ||
        !out || !iterations || !workspace || !barrier || !status || max_iterations < 1 || (g->n_bonds && !wrench) ||
        (active && !seg_bond))
        return DPF_ERR_ARGUMENT;
    cudaStream_t st = (cudaStream_t)stream;
    MixedDeviceInfo &info = mixed_info();
    if (info.sms <= 0 || info.blocks_per_sm <= 0) return DPF_ERR_CUDA;
    const int64_t want = blocks_for(g->n_sites > g->n_bonds ? g->n_sites : g->n_bonds, kPcgThreads);
    int64_t cap = (int64_t)info.sms * info.blocks_per_sm;
    if (cap > kMaxPcgBlocks) cap = kMaxPcgBlocks;
    const int grid = (int)(want < cap ? (want < 1 ? 1 : want) : cap);
    const int64_t n6 = 6 * g->n_sites;
    PcgArgs a{};
    a.n = g->n_sites;
    a.m = g->n_bonds;
    a.ptr = g->inc_ptr;
    a.inc = g->inc_bond;
    a.bd = split_bond_data(bond_data, g->n_bonds);
    a.mass32 = mass32;
    a.units32 = units32;
    a.vector = vector;
    a.block = block;
    a.P = preconditioner;
    a.fixed = fixed;
    a.alpha_op = (float)(0.25 * dt * dt);
    a.tol2 = tolerance * tolerance;
    a.max_it = max_iterations;
    a.out = out;
    a.iterations = iterations;
    a.seg = seg_bond;
    a.active = active;
    float4 *w4 = reinterpret_cast<float4 *>(workspace);
    const int64_t n = g->n_sites;
    a.zd = w4;                 // 4 float4 per site
    a.x = w4 + 4 * n;          // 2 float4 per site
    a.r = w4 + 6 * n;
    a.ad = w4 + 8 * n;
    a.wrench = w4 + 10 * n;    // 3 float4 per bond
    double *parts = reinterpret_cast<double *>(w4 + 10 * n + 3 * g->n_bonds);
    a.part_a = parts;
    a.part_b = parts + kMaxPcgBlocks;
    (void)n6;
    (void)wrench;
    a.barrier = barrier;
    a.status = status;
    if (cudaMemsetAsync(barrier, 0, 2 * sizeof(unsigned), st) != cudaSuccess) return DPF_ERR_CUDA;
    void *args[] = {&a};
    if (cudaLaunchCooperativeKernel((const void *)pcg_kernel_f32, grid, kPcgThreads, args, 0, st) != cudaSuccess) {
        cudaGetLastError();
        return DPF_ERR_CUDA;
    }
    return DPF_OK;
}

int dpf_mixed_commit(const dpf_graph *g, float *bond_data, const dpf_history *h, const double *y, const float *y32,
                     double *x_end, double *normal_end, double *offset_end, double *fn_end, double *fs_end,
                     double *mt_end, double *mb_end, float *dloads, double *loads, void *stream) {
    if (!mixed_graph_ok(g) || !bond_data || !h || !h->x ||
        (g->n_bonds && (!h->fn || !h->fs || !h->mt || !h->mb || !h->offset)) || !y || !y32 || !x_end ||
        (dloads && (!loads || !aligned16(dloads))) ||
        ((g->n_bonds) && (!normal_end || !offset_end || !fn_end || !fs_end || !mt_end || !mb_end)))
        return DPF_ERR_ARGUMENT;
    cudaStream_t st = (cudaStream_t)stream;
    end_positions<<<blocks_for(3 * g->n_sites, kThreads), kThreads, 0, st>>>(g->n_sites, h->x, y, x_end);
    if (g->n_bonds) {
        CommitArgs a{g->n_bonds, split_bond_data(bond_data, g->n_bonds), *h, y32, x_end, normal_end, offset_end,
                     fs_end, mb_end, fn_end, mt_end, dloads, nullptr};
        commit_bonds<false><<<blocks_for(g->n_bonds, kThreads), kThreads, 0, st>>>(a);
        if (dloads)
            commit_sites<<<blocks_for(kGroupJ * g->n_sites, kThreads), kThreads, 0, st>>>(
                g->n_sites, g->inc_ptr, g->inc_bond, dloads, loads);
    }
    DPF_CHECK_LAUNCH();
    return DPF_OK;
}

int dpf_mixed_initial_residual(int64_t n_sites, const double *r0, const uint8_t *fixed, float *y32, double *residual,
                               void *stream) {
    if (n_sites <= 0 || !r0 || !fixed || !y32 || !residual) return DPF_ERR_ARGUMENT;
    initial_residual<<<blocks_for(6 * n_sites, kThreads), kThreads, 0, (cudaStream_t)stream>>>(n_sites, r0, fixed,
                                                                                              y32, residual);
    DPF_CHECK_LAUNCH();
    return DPF_OK;
}

int64_t dpf_history_correction_floats(int64_t n_bonds) { return n_bonds < 0 ? 0 : 4 * kCorrArrays * n_bonds; }

int dpf_mixed_history_corrections(const dpf_graph *g, const dpf_history *h, const float *bond_data,
                                  float *corrections, void *stream) {
    if (!mixed_graph_ok(g) || !h || !bond_data) return DPF_ERR_ARGUMENT;
    if (!g->n_bonds) return DPF_OK;
    if (!h->fn || !h->fs || !h->mt || !h->mb || !h->offset || !corrections || ((uintptr_t)corrections & 15u))
        return DPF_ERR_ARGUMENT;
    CorrArgs a{g->n_bonds, *h, split_bond_data(const_cast<float *>(bond_data), g->n_bonds).rec,
               reinterpret_cast<float4 *>(corrections)};
    history_corrections<<<blocks_for(g->n_bonds, kThreads), kThreads, 0, (cudaStream_t)stream>>>(a);
    DPF_CHECK_LAUNCH();
    return DPF_OK;
}

int dpf_mixed_commit_lazy(const dpf_graph *g, float *bond_data, const double *x, const double *y, const float *y32,
                          double *x_end, float *corrections, float *dloads, double *loads, void *stream) {
    if (!mixed_graph_ok(g) || !bond_data || !x || !y || !y32 || !x_end || (g->n_bonds && (!corrections || !dloads ||
        !loads || ((uintptr_t)corrections & 15u) || !aligned16(dloads))))
        return DPF_ERR_ARGUMENT;
    cudaStream_t st = (cudaStream_t)stream;
    end_positions<<<blocks_for(3 * g->n_sites, kThreads), kThreads, 0, st>>>(g->n_sites, x, y, x_end);
    if (g->n_bonds) {
        dpf_history h{};
        h.x = x;
        CommitArgs a{g->n_bonds, split_bond_data(bond_data, g->n_bonds), h, y32, x_end, nullptr, nullptr, nullptr,
                     nullptr, nullptr, nullptr, dloads, reinterpret_cast<float4 *>(corrections)};
        commit_bonds<true><<<blocks_for(g->n_bonds, kThreads), kThreads, 0, st>>>(a);
        commit_sites<<<blocks_for(kGroupJ * g->n_sites, kThreads), kThreads, 0, st>>>(g->n_sites, g->inc_ptr,
                                                                                       g->inc_bond, dloads, loads);
    }
    DPF_CHECK_LAUNCH();
    return DPF_OK;
}

int dpf_mixed_fold_history(const dpf_graph *g, const double *x, const float *bond_data, const float *corrections,
                           double *normal, double *offset, double *fn, double *fs, double *mt, double *mb,
                           void *stream) {
    if (!mixed_graph_ok(g) || !x || !g->edges || !bond_data)
        return DPF_ERR_ARGUMENT;
    if (!g->n_bonds) return DPF_OK;
    if (!corrections || !normal || !offset || !fn || !fs || !mt || !mb || ((uintptr_t)corrections & 15u))
        return DPF_ERR_ARGUMENT;
    FoldArgs a{g->n_bonds, g->edges, x, split_bond_data(const_cast<float *>(bond_data), g->n_bonds).rec,
               reinterpret_cast<const float4 *>(corrections), normal, offset, fn, fs, mt, mb};
    fold_history<<<blocks_for(g->n_bonds, kThreads), kThreads, 0, (cudaStream_t)stream>>>(a);
    DPF_CHECK_LAUNCH();
    return DPF_OK;
}

int dpf_mixed_begin(int64_t n_sites, const double *loads, const double *mass, const double *v, const double *external,
                    const uint8_t *fixed, double dt, double *r0, double *scales, double *partials, void *stream) {
    if (n_sites <= 0 || !loads || !mass || !v || !external || !fixed || !r0 || !scales || !partials)
        return DPF_ERR_ARGUMENT;
    BeginArgs a{n_sites, loads, mass, v, external, fixed, dt, 0.5 * dt * dt, r0, scales, partials};
    begin_sites<<<reduce_grid(6 * n_sites), kThreads, 0, (cudaStream_t)stream>>>(a);
    DPF_CHECK_LAUNCH();
    return DPF_OK;
}

int64_t dpf_segment_partials_doubles(int n_segments) { return n_segments < 0 ? 0 : 3LL * kSegChunks * n_segments; }

int dpf_segment_norms(int n_segments, const int64_t *seg_ptr, const double *a, const double *b, int b_dot,
                      const uint8_t *mask, double *out, double *partials, void *stream) {
    if (n_segments <= 0 || n_segments > 65535 || !seg_ptr || !a || !out || !partials) return DPF_ERR_ARGUMENT;
    cudaStream_t st = (cudaStream_t)stream;
    segment_norms_kernel<<<dim3(kSegChunks, n_segments), kThreads, 0, st>>>(seg_ptr, a, b, b_dot, mask, partials);
    segment_finish_kernel<<<(n_segments + 127) / 128, 128, 0, st>>>(n_segments, partials, b_dot, out);
    DPF_CHECK_LAUNCH();
    return DPF_OK;
}

int dpf_segment_axpy(int64_t n_sites, const int32_t *seg, const double *factor, const double *a, const double *c,
                     double *out, void *stream) {
    if (n_sites <= 0 || !seg || !factor || !a || !c || !out) return DPF_ERR_ARGUMENT;
    segment_axpy_kernel<<<blocks_for(6 * n_sites, kThreads), kThreads, 0, (cudaStream_t)stream>>>(n_sites, seg, factor,
                                                                                                    a, c, out);
    DPF_CHECK_LAUNCH();
    return DPF_OK;
}

int dpf_segment_select(int64_t n_sites, const int32_t *seg, const uint8_t *keep, const double *a, const double *b,
                       double *out, void *stream) {
    if (n_sites <= 0 || !seg || !keep || !a || !b || !out) return DPF_ERR_ARGUMENT;
    segment_select_kernel<<<blocks_for(6 * n_sites, kThreads), kThreads, 0, (cudaStream_t)stream>>>(n_sites, seg, keep,
                                                                                                      a, b, out);
    DPF_CHECK_LAUNCH();
    return DPF_OK;
}

}  // extern "C"
