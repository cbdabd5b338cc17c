// float32 arithmetic of the mixed-precision Newton path: 3-vectors, forward-mode
// dual numbers, the per-bond record layout and the incremental midpoint force.
#pragma once

#include "common.cuh"

namespace dpf {
namespace mp {

// 1 - cos(0.25): the transport guard cos(angle) < cos(0.25) is evaluated as
// |n1 - n0|^2 > 2 (1 - cos 0.25), which stays accurate for small turns.
constexpr float kTurn2 = 2.0f * 0.031087578289355f;

// ---- forward-mode dual number (value, directional derivative) -------------
struct Dual {
    float v, d;
};
__device__ __forceinline__ Dual operator+(Dual a, Dual b) { return {a.v + b.v, a.d + b.d}; }
__device__ __forceinline__ Dual operator-(Dual a, Dual b) { return {a.v - b.v, a.d - b.d}; }
__device__ __forceinline__ Dual operator-(Dual a) { return {-a.v, -a.d}; }
__device__ __forceinline__ Dual operator*(Dual a, Dual b) { return {a.v * b.v, fmaf(a.d, b.v, a.v * b.d)}; }
__device__ __forceinline__ Dual operator/(Dual a, Dual b) {
    const float inv = 1.0f / b.v;
    const float q = a.v * inv;
    return {q, (a.d - q * b.d) * inv};
}
__device__ __forceinline__ Dual operator*(float s, Dual a) { return {s * a.v, s * a.d}; }
__device__ __forceinline__ Dual operator+(Dual a, float b) { return {a.v + b, a.d}; }
__device__ __forceinline__ Dual operator+(float b, Dual a) { return {a.v + b, a.d}; }
__device__ __forceinline__ Dual operator-(float b, Dual a) { return {b - a.v, -a.d}; }
__device__ __forceinline__ Dual dsqrt(Dual a) {
    const float s = sqrtf(a.v);
    return {s, a.d * 0.5f / s};
}
__device__ __forceinline__ float dsqrt(float a) { return sqrtf(a); }
__device__ __forceinline__ void dsincos(Dual a, Dual &s, Dual &c) {
    float sv, cv;
    sincosf(a.v, &sv, &cv);
    s = {sv, cv * a.d};
    c = {cv, -sv * a.d};
}
__device__ __forceinline__ void dsincos(float a, float &s, float &c) { sincosf(a, &s, &c); }

// sin t and 1 - cos t (= 2 sin^2(t/2), without cancellation).  For |t| < 1/2
// (every spin increment the rotation guards admit) from their Maclaurin
// series in t^2, five terms each (truncation below 3e-11 relative), instead of
// two sincos evaluations; larger |t| through sincos of t and t/2.
__device__ __forceinline__ void sin_omc(float t, float &s, float &omc) {
    const float t2 = t * t;
    if (t2 < 0.25f) {
        float p = 1.0f / 362880.0f;               // 1/9!
        p = fmaf(p, t2, -1.0f / 5040.0f);         // 1/7!
        p = fmaf(p, t2, 1.0f / 120.0f);           // 1/5!
        p = fmaf(p, t2, -1.0f / 6.0f);            // 1/3!
        p = fmaf(p, t2, 1.0f);
        s = t * p;
        float q = 1.0f / 3628800.0f;              // 1/10!
        q = fmaf(q, t2, -1.0f / 40320.0f);        // 1/8!
        q = fmaf(q, t2, 1.0f / 720.0f);           // 1/6!
        q = fmaf(q, t2, -1.0f / 24.0f);           // 1/4!
        q = fmaf(q, t2, 0.5f);                    // 1/2!
        omc = t2 * q;
    } else {
        float sh, ch, c;
        sincosf(0.5f * t, &sh, &ch);
        sincosf(t, &s, &c);
        omc = 2.0f * sh * sh;
    }
}
__device__ __forceinline__ void sin_omc(Dual t, Dual &s, Dual &omc) {
    float sv, ov;
    sin_omc(t.v, sv, ov);
    s = {sv, (1.0f - ov) * t.d};   // d sin = cos dt
    omc = {ov, sv * t.d};          // d (1 - cos) = sin dt
}
__device__ __forceinline__ float value(float a) { return a; }
__device__ __forceinline__ float value(Dual a) { return a.v; }
__device__ __forceinline__ float deriv(Dual a) { return a.d; }

template <class T>
__device__ __forceinline__ T lift(float a);
template <>
__device__ __forceinline__ float lift<float>(float a) { return a; }
template <>
__device__ __forceinline__ Dual lift<Dual>(float a) { return {a, 0.0f}; }

template <class T>
struct V3 {
    T x, y, z;
};
template <class T>
__device__ __forceinline__ V3<T> operator+(V3<T> a, V3<T> b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
template <class T>
__device__ __forceinline__ V3<T> operator-(V3<T> a, V3<T> b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
template <class T>
__device__ __forceinline__ V3<T> operator-(V3<T> a) { return {-a.x, -a.y, -a.z}; }
template <class T, class S>
__device__ __forceinline__ V3<T> operator*(S s, V3<T> a) { return {s * a.x, s * a.y, s * a.z}; }
template <class T>
__device__ __forceinline__ T dot(V3<T> a, V3<T> b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
template <class T>
__device__ __forceinline__ V3<T> cross(V3<T> a, V3<T> b) {
    return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x};
}
template <class T>
__device__ __forceinline__ V3<T> operator/(V3<T> a, T s) {
    const T inv = lift<T>(1.0f) / s;
    return {a.x * inv, a.y * inv, a.z * inv};
}
template <class T>
__device__ __forceinline__ V3<T> lift3(float3 a) { return {lift<T>(a.x), lift<T>(a.y), lift<T>(a.z)}; }
__device__ __forceinline__ V3<float> val3(V3<Dual> a) { return {a.x.v, a.y.v, a.z.v}; }
__device__ __forceinline__ V3<float> der3(V3<Dual> a) { return {a.x.d, a.y.d, a.z.d}; }
__device__ __forceinline__ V3<float> val3(V3<float> a) { return a; }

// ---- per-bond record (float32, bond-sorted structure of float4 arrays) ------
// Constant over one time step, built from the committed state in float64:
//   r0 = (n0, L0)          committed normal, rest-of-step length |x_j - x_i|
//   r1 = (dn0, rh)         geometry(x) normal minus n0; (rad_i - rad_j)/2
//   r2 = (ri_x, fn)        contact lever of i at x; normal force
//   r3 = (fs, mt)          shear force; twist couple
//   r4 = (mb, kn)          bending couple; normal stiffness
//   r5 = (offset, ks)      contact offset; shear stiffness
//   r6 = (kb, kt, i, j)    bending, twist stiffness; endpoints (int bits)
struct Records {
    float4 *r0, *r1, *r2, *r3, *r4, *r5, *r6;
};
constexpr int kRecordFloat4s = 7;

struct Bond {
    float3 n0, dn0, ri_x, fs, mb, off;
    float L0, rh, fn, mt, kn, ks, kb, kt;
    int i, j;
};

__device__ __forceinline__ Bond load_bond(const Records &R, int64_t b) {
    const float4 a = __ldg(R.r0 + b), c = __ldg(R.r1 + b), e = __ldg(R.r2 + b), f = __ldg(R.r3 + b);
    const float4 g = __ldg(R.r4 + b), h = __ldg(R.r5 + b), k = __ldg(R.r6 + b);
    Bond o;
    o.n0 = make_float3(a.x, a.y, a.z);
    o.L0 = a.w;
    o.dn0 = make_float3(c.x, c.y, c.z);
    o.rh = c.w;
    o.ri_x = make_float3(e.x, e.y, e.z);
    o.fn = e.w;
    o.fs = make_float3(f.x, f.y, f.z);
    o.mt = f.w;
    o.mb = make_float3(g.x, g.y, g.z);
    o.kn = g.w;
    o.off = make_float3(h.x, h.y, h.z);
    o.ks = h.w;
    o.kb = k.x;
    o.kt = k.y;
    o.i = __float_as_int(k.z);
    o.j = __float_as_int(k.w);
    return o;
}

// n(x + u) - n(x) for a bond of rest vector L0 * nx, stretched by du_half =
// (u_j - u_i)/2, computed from the small quantities only.
template <class T>
__device__ __forceinline__ V3<T> normal_change(float L0, V3<T> nx, V3<T> du_half, T &length) {
    const T e = (2.0f * L0 * dot(nx, du_half) + dot(du_half, du_half)) / lift<T>(L0 * L0);
    const T s = dsqrt(1.0f + e);
    length = L0 * s;
    const T dL = (L0 * e) / (1.0f + s);
    return (du_half - dL * nx) / length;
}
// Rotation of the rate-law transport from n0 to n0 + dn with axial spin
// angle hs . bisector, in increment form: apply(v) returns T(v) - v.
template <class T>
struct TransportInc {
    V3<T> k, n;
    T inv1pc, s, omc;
    __device__ __forceinline__ V3<T> apply(V3<T> v) const {
        const V3<T> kv = cross(k, v);
        const V3<T> d1 = kv + inv1pc * cross(k, kv);
        const V3<T> out = v + d1;
        return d1 + s * cross(n, out) - omc * (out - dot(n, out) * n);
    }
};

template <class T>
__device__ __forceinline__ TransportInc<T> make_transport_inc(V3<T> n0, V3<T> dn, V3<T> hs) {
    TransportInc<T> t;
    t.k = cross(n0, dn);
    t.n = n0 + dn;
    const T dn2 = dot(dn, dn);
    t.inv1pc = lift<T>(1.0f) / (2.0f - 0.5f * dn2);
    const V3<T> bv = 2.0f * n0 + dn;
    const T bl = dsqrt(dot(bv, bv));
    const V3<T> b = bv / bl;
    const T theta = dot(hs, b);
    sin_omc(theta, t.s, t.omc);
    return t;
}

// Increment of the midpoint bond wrench, f_mid(y) - f_mid(0) restricted to the
// bond (experiments/bonded_dem_newton.py:64-81 with experiments/bonded_dem_finite_gpu.py:22-32),
// as [dF, dT_i, dT_j]; also the midpoint tangent geometry and the guard terms.
template <class T>
struct BondIncrement {
    V3<T> dF, dTi, dTj;
    V3<T> n, ri, rj;
    V3<T> dn_x;     // n - n_x
    V3<T> dfs1, dmb1;  // fs1 - fs, mb1 - mb (for the end state)
    V3<T> doff;        // offset_mid - offset
    T dn, tw, length;
    float turn2;       // |n - n0|^2
};

template <class T>
__device__ __forceinline__ BondIncrement<T> bond_increment(const Bond &B, V3<T> ui, V3<T> wi, V3<T> uj, V3<T> wj) {
    BondIncrement<T> o;
    const V3<T> n0 = lift3<T>(B.n0), dn0 = lift3<T>(B.dn0);
    const V3<T> nx = n0 + dn0;
    o.dn_x = normal_change(B.L0, nx, 0.5f * (uj - ui), o.length);
    const V3<T> dn = o.dn_x + dn0;  // n - n0
    o.n = n0 + dn;
    o.turn2 = value(dot(dn, dn));
    const V3<T> hs = 0.25f * (wi + wj);
    const TransportInc<T> tr = make_transport_inc(n0, dn, hs);
    o.doff = tr.apply(lift3<T>(B.off));
    const V3<T> dfs = tr.apply(lift3<T>(B.fs));
    const V3<T> dmb = tr.apply(lift3<T>(B.mb));
    const V3<T> dc = 0.25f * (ui + uj) + B.rh * o.dn_x + o.doff;
    const V3<T> ri_x = lift3<T>(B.ri_x);
    const V3<T> rj_x = ri_x - B.L0 * nx;
    const V3<T> dri = dc - 0.5f * ui, drj = dc - 0.5f * uj;
    o.ri = ri_x + dri;
    o.rj = rj_x + drj;
    const V3<T> du = uj - ui + cross(wj, o.rj) - cross(wi, o.ri);
    const V3<T> dw = wj - wi;
    o.dn = dot(du, o.n);
    o.tw = dot(dw, o.n);
    const V3<T> ds = du - o.dn * o.n, db = dw - o.tw * o.n;
    o.dfs1 = dfs + B.ks * ds;
    o.dmb1 = dmb + B.kb * db;
    o.dF = B.fn * o.dn_x + dfs + (0.5f * B.kn) * o.dn * o.n + (0.5f * B.ks) * ds;
    const V3<T> dcp = B.mt * o.dn_x + dmb + (0.5f * B.kt) * o.tw * o.n + (0.5f * B.kb) * db;
    const V3<T> f = (B.fn * nx + lift3<T>(B.fs)) + o.dF;
    o.dTi = cross(dri, f) + cross(ri_x, o.dF) + dcp;
    o.dTj = -(cross(drj, f) + cross(rj_x, o.dF) + dcp);
    return o;
}

}  // namespace mp
}  // namespace dpf
