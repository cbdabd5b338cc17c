// Site tiles of the bond graph and the tiled float32 Hessian-vector product
// y = (diag M + dt^2/4 K) q (experiments/bonded_dem_linear_gpu.py:42-52, 74-77)
// with the elastic block-Jacobi PCG built on it
// (experiments/bonded_dem_newton.py:107-130).
//
// A tile is a contiguous range of sites (the foam generator orders sites along
// a Morton curve, so a range is a compact patch) plus every bond touching it
// ("entries"; a bond between two tiles is an entry of both) and the outside
// endpoints of those bonds ("halo").  Persistent CTAs walk their tiles with
// a ring of three or four shared-memory buffers: while one tile computes, the
// entry records and incidence metadata of the tiles after it arrive by TMA
// bulk copies (completing on an mbarrier) and the next tile's site vectors by
// cp.async.  Per tile:
//   1. each thread computes its entries' wrenches [F_i, T_i, T_j] and writes
//      them over the same entries' records;
//   2. after one block barrier, each site sums its wrench contributions over
//      its incidence list in the list's order (no atomics: deterministic) and
//      hands the sum to the caller's epilogue (y of the HVP, w and (w, u) of
//      the PCG).
// Only bonds cut by tile boundaries are read twice; wrenches never go to
// global memory.
#include <algorithm>
#include <mutex>
#include <vector>

#include "common.cuh"

namespace dpf {
namespace tiles {

#ifndef DPF_TILE_LANES
#define DPF_TILE_LANES 4
#endif

constexpr int kLanes = DPF_TILE_LANES;  // lanes per site in the site sums
constexpr int kPer = 2;                 // entries per thread and tile (read to registers before W overwrites them)
#ifndef DPF_TILE_THREADS_MAX
#define DPF_TILE_THREADS_MAX 192  // consumer threads; the tiled kernels add a bulk and a halo warp
#endif
#ifndef DPF_TILE_MIN_BLOCKS
#define DPF_TILE_MIN_BLOCKS 3
#endif
constexpr int kTileThreadsMax = DPF_TILE_THREADS_MAX;
constexpr unsigned long long kWaitNs = 1000000000ull;  // mbarrier waits give up after 1 s

struct TileGraph {
    int32_t n_tiles;
    const int4 *desc;            // per tile (first site, sites, entries, halo), (first entry, -, meta word, words)
    const uint32_t *tile_meta;
    const float4 *e0, *e1, *e2;  // entry planes: (n, ri.x), (ri.y, ri.z, L, a kn), (a ks, a kb, a kt, ends)
    const float4 *site;          // per site (mass, inertia, 1 free / 0 fixed, -); fixed sites (1, 1, 0, -)
};

// Byte offsets inside one of the shared-memory tile buffers.
struct Layout {
    uint32_t plane;   // bytes of one record plane (16 * max entries)
    uint32_t qown, qhalo, site, meta, head, size;  // head: the tile's descriptor (two int4)
    int stages;       // tile buffers in the ring
};

// ---- asynchronous copies (TMA bulk + mbarrier, cp.async) -------------------

__device__ __forceinline__ uint32_t saddr(const void *p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void mbar_init(uint64_t *bar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(saddr(bar)), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_init_fence() {
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}
__device__ __forceinline__ void mbar_expect_tx(uint64_t *bar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(saddr(bar)), "r"(bytes) : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(uint64_t *bar, uint32_t parity) {
    uint32_t ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(ok)
        : "r"(saddr(bar)), "r"(parity)
        : "memory");
    return ok != 0;
}
// Global -> shared bulk copy completing on `bar` (16-byte aligned, multiple of 16 bytes).
__device__ __forceinline__ void bulk_load(void *dst, const void *src, uint32_t bytes, uint64_t *bar) {
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                     saddr(dst)),
                 "l"(src), "r"(bytes), "r"(saddr(bar))
                 : "memory");
}
// Order this thread's earlier generic-proxy shared accesses before later bulk writes.
__device__ __forceinline__ void fence_proxy_async() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }
__device__ __forceinline__ void cp_async8(void *dst, const void *src) {
    asm volatile("cp.async.ca.shared.global [%0], [%1], 8;" ::"r"(saddr(dst)), "l"(src) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
__device__ __forceinline__ void cp_async_wait_all() { asm volatile("cp.async.wait_group 0;" ::: "memory"); }

// Wait for phase `parity` of `bar`; false (and the status bit) after kWaitNs.
__device__ __forceinline__ bool mbar_wait(uint64_t *bar, uint32_t parity, int *status) {
    if (mbar_try_wait(bar, parity)) return true;
    const unsigned long long t0 = global_ns();
    while (!mbar_try_wait(bar, parity)) {
        if (global_ns() - t0 > kWaitNs) {
            atomicOr(status, DPF_ERR_BARRIER_TIMEOUT);
            return false;
        }
    }
    return true;
}

// ---- one entry -------------------------------------------------------------------

// alpha K q wrench of one entry, written over the entry's own records (slot e
// of the three record planes, so no other thread's records are touched):
// W0 = (F, Ti.x), W1 = (Ti.y, Ti.z, Tj.x, Tj.y), W2.x = Tj.z with F = F_i
// (site i adds F_i, T_i; site j adds -F_i, T_j).
__device__ __forceinline__ void entry_wrench(float4 a, float4 b, float4 c, const float *qown, const float *qhalo,
                                             int T, float4 *W0, float4 *W1, float *W2) {
    const uint32_t ends = __float_as_uint(c.w);
    const int li = (int)(ends & 0xffffu), lj = (int)(ends >> 16);
    const float2 *qi = reinterpret_cast<const float2 *>(li < T ? qown + 6 * li : qhalo + 6 * (li - T));
    const float2 *qj = reinterpret_cast<const float2 *>(lj < T ? qown + 6 * lj : qhalo + 6 * (lj - T));
    const float2 ui0 = qi[0], ui1 = qi[1], ui2 = qi[2], uj0 = qj[0], uj1 = qj[1], uj2 = qj[2];
    const float nx = a.x, ny = a.y, nz = a.z;
    const float rix = a.w, riy = b.x, riz = b.y, L = b.z;
    const float rjx = rix - L * nx, rjy = riy - L * ny, rjz = riz - L * nz;
    const float kn = b.w, ks = c.x, kb = c.y, kt = c.z;
    const float wix = ui1.y, wiy = ui2.x, wiz = ui2.y, wjx = uj1.y, wjy = uj2.x, wjz = uj2.y;
    // du = u_j - u_i + w_j x r_j - w_i x r_i ; dw = w_j - w_i
    const float dux = uj0.x - ui0.x + (wjy * rjz - wjz * rjy) - (wiy * riz - wiz * riy);
    const float duy = uj0.y - ui0.y + (wjz * rjx - wjx * rjz) - (wiz * rix - wix * riz);
    const float duz = uj1.x - ui1.x + (wjx * rjy - wjy * rjx) - (wix * riy - wiy * rix);
    const float dwx = wjx - wix, dwy = wjy - wiy, dwz = wjz - wiz;
    const float un = (kn - ks) * (dux * nx + duy * ny + duz * nz);
    const float wn = (kt - kb) * (dwx * nx + dwy * ny + dwz * nz);
    const float fx = ks * dux + un * nx, fy = ks * duy + un * ny, fz = ks * duz + un * nz;
    const float mx = kb * dwx + wn * nx, my = kb * dwy + wn * ny, mz = kb * dwz + wn * nz;
    const float tix = -(riy * fz - riz * fy) - mx, tiy = -(riz * fx - rix * fz) - my;
    const float tiz = -(rix * fy - riy * fx) - mz;
    const float tjx = (rjy * fz - rjz * fy) + mx, tjy = (rjz * fx - rjx * fz) + my;
    const float tjz = (rjx * fy - rjy * fx) + mz;
    *W0 = make_float4(-fx, -fy, -fz, tix);
    *W1 = make_float4(tiy, tiz, tjx, tjy);
    *W2 = tjz;
}

struct TileView {
    int64_t a, e0, meta;
    int T, E, H, words, halo_word;  // halo_word: first halo-site word in the metadata
};

__device__ __forceinline__ TileView view_of(int4 d0, int4 d1) {
    TileView v;
    v.a = d0.x;
    v.T = d0.y;
    v.E = d0.z;
    v.H = d0.w;
    v.e0 = d1.x;
    v.meta = d1.z;
    v.words = d1.w;
    v.halo_word = v.words - ((v.H + 3) & ~3);
    return v;
}

// Own-site q of a tile in shared memory starts at buf + L.qown + (24 a mod 16),
// so the 16-byte-aligned interior of its global range maps to an aligned
// shared address (bulk copy) and the at most two 8-byte ends go by cp.async.
struct OwnRange {
    uint64_t begin, end, lo, hi;  // global byte offsets in q; [lo, hi) 16-aligned interior
    uint32_t shift;               // (24 a) mod 16
};

__device__ __forceinline__ OwnRange own_range(const TileView &v) {
    OwnRange r;
    r.begin = 24ull * (uint64_t)v.a;
    r.end = r.begin + 24ull * (uint64_t)v.T;
    r.lo = (r.begin + 15) & ~15ull;
    r.hi = r.end & ~15ull;
    if (r.hi < r.lo) r.hi = r.lo;
    r.shift = (uint32_t)(r.begin & 15u);
    return r;
}

// Bulk warp, lane 0: the tile's descriptor into the buffer header, then bulk copies of
// the tile's entry records, metadata, site records and own-site q interior.
__device__ __forceinline__ void issue_bulk(const TileGraph &G, const Layout &L, int4 d0, int4 d1, const float *q,
                                           unsigned char *buf, uint64_t *bar) {
    const TileView v = view_of(d0, d1);
    int4 *head = reinterpret_cast<int4 *>(buf + L.head);  // read by the consumers after the bulk barrier
    head[0] = d0;
    head[1] = d1;
    fence_proxy_async();
    const uint32_t plane = 16u * (uint32_t)v.E, meta = 4u * (uint32_t)v.words;
    const OwnRange o = own_range(v);
    const uint32_t own = (uint32_t)(o.hi - o.lo), sites = 16u * (uint32_t)v.T;
    mbar_expect_tx(bar, 3 * plane + meta + own + sites);
    bulk_load(buf + L.site, G.site + v.a, sites, bar);
    if (v.E) {
        bulk_load(buf, G.e0 + v.e0, plane, bar);
        bulk_load(buf + L.plane, G.e1 + v.e0, plane, bar);
        bulk_load(buf + 2 * L.plane, G.e2 + v.e0, plane, bar);
    }
    bulk_load(buf + L.meta, G.tile_meta + v.meta, meta, bar);
    if (own)
        bulk_load(buf + L.qown + o.shift + (uint32_t)(o.lo - o.begin),
                  reinterpret_cast<const unsigned char *>(q) + o.lo, own, bar);
}

// Halo sites of a tile held in registers by the halo warp: slot lane + 32 k.
constexpr int kHaloRegs = 8;

__device__ __forceinline__ void load_halo(const TileView &v, const uint32_t *meta, int lane, int h[kHaloRegs]) {
    const int32_t *src = reinterpret_cast<const int32_t *>(meta) + v.meta + v.halo_word;
#pragma unroll
    for (int k = 0; k < kHaloRegs; ++k) {
        const int slot = lane + 32 * k;
        h[k] = slot < v.H ? __ldg(src + slot) : 0;
    }
}

// The halo warp, once the buffer is free: cp.async of the own-site q ends
// outside the bulk interior and of the halo sites' q (the first 32 kHaloRegs
// halo sites from registers, loaded a tile ahead; any further ones read from
// the tile's metadata in global memory), then each lane's asynchronous
// arrival on `bar` (it fires when that lane's copies have landed).
__device__ __forceinline__ void issue_q(const TileView &v, const Layout &L, const uint32_t *meta, const int h[kHaloRegs],
                                        unsigned char *buf, const float *q, int lane, uint64_t *bar) {
    const OwnRange o = own_range(v);
    const unsigned char *qb = reinterpret_cast<const unsigned char *>(q);
    unsigned char *own = buf + L.qown + o.shift;
    const int head = (int)((o.lo - o.begin) >> 3), tail = (int)((o.end - o.hi) >> 3);
    for (int k = lane; k < head + tail; k += 32) {
        const uint64_t off = k < head ? 8ull * k : (o.hi - o.begin) + 8ull * (k - head);
        cp_async8(own + off, qb + o.begin + off);
    }
    float2 *hal = reinterpret_cast<float2 *>(buf + L.qhalo);
#pragma unroll
    for (int k = 0; k < kHaloRegs; ++k) {
        const int slot = lane + 32 * k;
        if (slot < v.H) {
            const float2 *src = reinterpret_cast<const float2 *>(q + 6 * (int64_t)h[k]);
            cp_async8(hal + 3 * slot, src);
            cp_async8(hal + 3 * slot + 1, src + 1);
            cp_async8(hal + 3 * slot + 2, src + 2);
        }
    }
    const int32_t *list = reinterpret_cast<const int32_t *>(meta) + v.meta + v.halo_word;
    for (int slot = lane + 32 * kHaloRegs; slot < v.H; slot += 32) {
        const float2 *src = reinterpret_cast<const float2 *>(q + 6 * (int64_t)__ldg(list + slot));
        cp_async8(hal + 3 * slot, src);
        cp_async8(hal + 3 * slot + 1, src + 1);
        cp_async8(hal + 3 * slot + 2, src + 2);
    }
    asm volatile("cp.async.mbarrier.arrive.noinc.shared::cta.b64 [%0];" ::"r"(saddr(bar)) : "memory");
}

// The alpha K q part of local site sl from the tile's wrench planes (all
// kLanes lanes of a group call it together).  span[sl] = start | mid << 16:
// the site's incidences [start, mid) are i ends, [mid, next start) j ends, in
// incidence order with a fixed lane split.
__device__ __forceinline__ void site_sum(const float4 *W0, const float4 *W1, const float4 *W2, const uint32_t *span,
                                         const uint16_t *codes, int sl, bool valid, int lane, float acc[6]) {
#pragma unroll
    for (int c = 0; c < 6; ++c) acc[c] = 0.0f;
    if (valid) {
        const uint32_t sp = span[sl];
        const int k0 = (int)(sp & 0xffffu), mid = (int)(sp >> 16), k1 = (int)(span[sl + 1] & 0xffffu);
        for (int k = k0 + lane; k < mid; k += kLanes) {
            const int e = codes[k];
            const float4 w0 = W0[e], w1 = W1[e];
            acc[0] += w0.x;
            acc[1] += w0.y;
            acc[2] += w0.z;
            acc[3] += w0.w;
            acc[4] += w1.x;
            acc[5] += w1.y;
        }
        for (int k = mid + lane; k < k1; k += kLanes) {
            const int e = codes[k];
            const float4 w0 = W0[e], w1 = W1[e];
            const float w2 = reinterpret_cast<const float *>(W2 + e)[0];
            acc[0] -= w0.x;
            acc[1] -= w0.y;
            acc[2] -= w0.z;
            acc[3] += w1.z;
            acc[4] += w1.w;
            acc[5] += w2;
        }
    }
#pragma unroll
    for (int o = 1; o < kLanes; o <<= 1)
#pragma unroll
        for (int c = 0; c < 6; ++c) acc[c] += __shfl_xor_sync(0xffffffffu, acc[c], o);
}

// Ring of L.stages shared-memory tile buffers.  Per buffer three mbarriers:
// bulk (the tile's bulk copies: one arrival with the byte count), halo (the
// 32 lanes of the halo warp, each when its q copies have landed) and empty
// (one arrival per consumer warp when it is done with the buffer).
struct Pipe {
    unsigned char *base;
    uint64_t *bulk, *halo, *empty;
    uint32_t parity;  // this thread's next phase parity: bit b bulk, 8 + b halo, 16 + b empty
};

__device__ __forceinline__ Pipe pipe_init(unsigned char *smem, const Layout &L, int consumer_warps) {
    Pipe P;
    P.base = smem;
    P.bulk = reinterpret_cast<uint64_t *>(smem + (size_t)L.stages * L.size);
    P.halo = P.bulk + L.stages;
    P.empty = P.halo + L.stages;
    P.parity = 0u;
    if (threadIdx.x == 0) {
        for (int b = 0; b < L.stages; ++b) {
            mbar_init(P.bulk + b, 1);
            mbar_init(P.halo + b, 32);
            mbar_init(P.empty + b, (uint32_t)consumer_warps);
        }
        mbar_init_fence();
    }
    __syncthreads();
    return P;
}

// This thread's wait for the next phase of barrier `bar` (parity bit `bit`);
// false after the time limit.
__device__ __forceinline__ bool pipe_wait(Pipe &P, uint64_t *bar, int bit, int *status) {
    const bool ok = mbar_wait(bar, (P.parity >> bit) & 1u, status);
    P.parity ^= 1u << bit;
    return ok;
}

__device__ __forceinline__ void mbar_arrive(uint64_t *bar) {
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(saddr(bar)) : "memory");
}

// OR of `pred` over the `count` consumer threads (named barrier 1).
__device__ __forceinline__ bool consumers_or(bool pred, int count) {
    uint32_t out;
    asm volatile(
        "{\n\t.reg .pred p, q;\n\t"
        "setp.ne.u32 p, %1, 0;\n\t"
        "bar.red.or.pred q, 1, %2, p;\n\t"
        "selp.u32 %0, 1, 0, q;\n\t}"
        : "=r"(out)
        : "r"((uint32_t)pred), "r"(count)
        : "memory");
    return out != 0;
}

// For each own site s of every tile of this block: epi(s, q_s (shared), site
// record, acc) with acc the alpha K q sum.  Warp roles (blockDim = consumer
// threads + 64):
//   * bulk warp (lane 0): for tile j in buffer j mod S, once the consumers
//     have released the buffer's previous tile, the tile's bulk copies;
//   * halo warp: once the buffer is free, the q gather of the tile's halo
//     sites (list read from global memory) and own-site ends, arriving on
//     halo[b];
// (both producer warps read the descriptors of 32 tiles at a time, one per
// lane; the consumers read the tile's descriptor from the buffer header).
//   * consumer warps: wait for bulk[b] and halo[b], compute the entry
//     wrenches in place, one named barrier among consumers, the site sums and
//     the epilogue, then release the buffer (empty[b]).
// So up to S - 1 tiles stream in while one computes.  False (for the whole
// block) on a wait timeout.
template <class Epi>
__device__ __forceinline__ bool for_tiles(const TileGraph &G, const Layout &L, Pipe &P, const float *q, int *status,
                                          Epi &epi) {
    bool ok = true;
    if ((int)blockIdx.x < G.n_tiles) {
        const int S = L.stages;
        const int n_local = (G.n_tiles - 1 - (int)blockIdx.x) / (int)gridDim.x + 1;
        const int consumers = (int)blockDim.x - 64, warp = (int)threadIdx.x >> 5, lane32 = (int)threadIdx.x & 31;
        auto tile_of = [&](int j) { return (int)blockIdx.x + j * (int)gridDim.x; };
        auto buf_of = [&](int b) { return P.base + (size_t)b * L.size; };
        // the descriptors of tiles j .. j + 31 of this block, one per lane
        auto fetch = [&](int j, int4 &d0, int4 &d1) {
            const int t = j + lane32 < n_local ? tile_of(j + lane32) : tile_of(j);
            d0 = __ldg(G.desc + 2 * t);
            d1 = __ldg(G.desc + 2 * t + 1);
        };
        auto pick = [&](const int4 &d, int src) {
            return make_int4(__shfl_sync(0xffffffffu, d.x, src), __shfl_sync(0xffffffffu, d.y, src),
                             __shfl_sync(0xffffffffu, d.z, src), __shfl_sync(0xffffffffu, d.w, src));
        };
        if (warp == consumers / 32) {  // bulk warp
            int4 d0, d1;
            for (int j = 0; j < n_local && ok; ++j) {
                if ((j & 31) == 0) fetch(j, d0, d1);
                const int4 t0 = pick(d0, j & 31), t1 = pick(d1, j & 31);
                const int b = j % S;
                if (lane32 == 0) {
                    if (j >= S) ok = pipe_wait(P, P.empty + b, 16 + b, status);
                    if (ok) issue_bulk(G, L, t0, t1, q, buf_of(b), P.bulk + b);
                }
                ok = __shfl_sync(0xffffffffu, ok, 0);
            }
            // the consumers' release of the last tiles (keeps the phases in step)
            if (lane32 == 0)
                for (int j = n_local > S ? n_local - S : 0; j < n_local && ok; ++j)
                    ok = pipe_wait(P, P.empty + j % S, 16 + j % S, status);
            ok = __shfl_sync(0xffffffffu, ok, 0);
        } else if (warp == consumers / 32 + 1) {  // halo warp
            int4 d0, d1;
            int h[kHaloRegs], hn[kHaloRegs];
            fetch(0, d0, d1);
            TileView vn = view_of(pick(d0, 0), pick(d1, 0));
            load_halo(vn, G.tile_meta, lane32, hn);
            for (int j = 0; j < n_local && ok; ++j) {
                const TileView v = vn;
#pragma unroll
                for (int k = 0; k < kHaloRegs; ++k) h[k] = hn[k];
                if (j + 1 < n_local) {  // the next tile's halo list, loaded while this one waits
                    if (((j + 1) & 31) == 0) fetch(j + 1, d0, d1);
                    vn = view_of(pick(d0, (j + 1) & 31), pick(d1, (j + 1) & 31));
                    load_halo(vn, G.tile_meta, lane32, hn);
                }
                const int b = j % S;
                if (j >= S) ok = __all_sync(0xffffffffu, pipe_wait(P, P.empty + b, 16 + b, status));
                if (ok) issue_q(v, L, G.tile_meta, h, buf_of(b), q, lane32, P.halo + b);
            }
            for (int j = n_local > S ? n_local - S : 0; j < n_local && ok; ++j)
                ok = __all_sync(0xffffffffu, pipe_wait(P, P.empty + j % S, 16 + j % S, status));
            cp_async_wait_all();
        } else {  // consumer warps
            const int lane = threadIdx.x & (kLanes - 1);
            const int groups = consumers / kLanes;
            for (int j = 0; j < n_local; ++j) {
                const int b = j % S;
                bool here = pipe_wait(P, P.bulk + b, b, status);
                here = pipe_wait(P, P.halo + b, 8 + b, status) && here;
                unsigned char *buf = buf_of(b);
                const int4 *head = reinterpret_cast<const int4 *>(buf + L.head);
                const TileView v = view_of(head[0], head[1]);
                float4 *p0 = reinterpret_cast<float4 *>(buf);
                float4 *p1 = reinterpret_cast<float4 *>(buf + L.plane);
                float4 *p2 = reinterpret_cast<float4 *>(buf + 2 * L.plane);
                const float *qown = reinterpret_cast<const float *>(buf + L.qown + own_range(v).shift);
                const float *qhalo = reinterpret_cast<const float *>(buf + L.qhalo);
                if (here) {
#pragma unroll
                    for (int u = 0; u < kPer; ++u) {
                        const int e = threadIdx.x + u * consumers;
                        if (e < v.E)
                            entry_wrench(p0[e], p1[e], p2[e], qown, qhalo, v.T, p0 + e, p1 + e,
                                         reinterpret_cast<float *>(p2 + e));
                    }
                }
                if (consumers_or(!here, consumers)) {  // the wrenches of tile j are written
                    ok = false;
                    break;
                }
                const uint32_t *span = reinterpret_cast<const uint32_t *>(buf + L.meta);
                const uint16_t *codes = reinterpret_cast<const uint16_t *>(span + v.T + 1);
                const int rounds = (v.T + groups - 1) / groups;
                for (int rd = 0; rd < rounds; ++rd) {
                    const int sl = rd * groups + (int)threadIdx.x / kLanes;
                    const bool valid = sl < v.T;
                    float acc[6];
                    site_sum(p0, p1, p2, span, codes, sl, valid, lane, acc);
                    if (valid && lane == 0)
                        epi(v.a + sl, qown + 6 * sl, reinterpret_cast<const float4 *>(buf + L.site)[sl], acc);
                }
                __syncwarp();
                if (lane32 == 0) mbar_arrive(P.empty + b);
            }
        }
    }
    return !__syncthreads_or(!ok);
}

__device__ __forceinline__ void ld6(const float *p, float v[6]) {
    const float2 *q = reinterpret_cast<const float2 *>(p);
    const float2 a = q[0], b = q[1], c = q[2];
    v[0] = a.x; v[1] = a.y; v[2] = b.x; v[3] = b.y; v[4] = c.x; v[5] = c.y;
}
__device__ __forceinline__ void st6(float *p, const float v[6]) {
    float2 *q = reinterpret_cast<float2 *>(p);
    q[0] = make_float2(v[0], v[1]);
    q[1] = make_float2(v[2], v[3]);
    q[2] = make_float2(v[4], v[5]);
}

// (diag M) q + alpha K q; fixed sites (record (1, 1, 0, -)) give q.
__device__ __forceinline__ void operator_row(float4 rec, const float *qs, const float acc[6], float out[6]) {
#pragma unroll
    for (int c = 0; c < 6; ++c) out[c] = fmaf(c < 3 ? rec.x : rec.y, qs[c], rec.z * acc[c]);
}

// ---- standalone HVP ------------------------------------------------------------

struct HvpArgs {
    TileGraph G;
    Layout L;
    const float *q;
    float *y;
    int *status;
};

struct HvpEpi {
    const HvpArgs &a;
    __device__ __forceinline__ void operator()(int64_t s, const float *qs, float4 rec, const float acc[6]) const {
        float out[6];
        operator_row(rec, qs, acc, out);
        st6(a.y + 6 * s, out);
    }
};

__global__ void __launch_bounds__(kTileThreadsMax + 64, DPF_TILE_MIN_BLOCKS) tiled_hvp_kernel(HvpArgs a) {
    extern __shared__ __align__(16) unsigned char smem[];
    Pipe P = pipe_init(smem, a.L, ((int)blockDim.x - 64) / 32);
    HvpEpi epi{a};
    for_tiles(a.G, a.L, P, a.q, a.status, epi);
}

// ---- packing -----------------------------------------------------------------

struct PackArgs {
    int64_t n_entries;
    const int32_t *entry_bond;
    const uint32_t *entry_ends;
    const float4 *t0, *t1, *t2, *t3;  // tangent records (n, kn), (ri, ks), (rj, kb), (kt, i, j, -)
    float alpha;
    float4 *e0, *e1, *e2;
};

__global__ void __launch_bounds__(kThreads) pack_entries_kernel(PackArgs a) {
    const int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (e >= a.n_entries) return;
    const int64_t b = a.entry_bond[e];
    const float4 n = a.t0[b], ri = a.t1[b], rj = a.t2[b], g = a.t3[b];
    const float L = (ri.x - rj.x) * n.x + (ri.y - rj.y) * n.y + (ri.z - rj.z) * n.z;
    a.e0[e] = make_float4(n.x, n.y, n.z, ri.x);
    a.e1[e] = make_float4(ri.y, ri.z, L, a.alpha * n.w);
    a.e2[e] = make_float4(a.alpha * ri.w, a.alpha * rj.w, a.alpha * g.x, __uint_as_float(a.entry_ends[e]));
}

// P (36 floats, symmetric) -> 21 upper-triangle floats padded to 24; site
// records (m, I, 1, 0), fixed sites (1, 1, 0, 0).
__global__ void __launch_bounds__(kThreads) pack_sites_kernel(int64_t n, const float *P36, const float *mass32,
                                                              const uint8_t *fixed, float4 *P24, float4 *site) {
    const int64_t s = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (s >= n) return;
    const float *p = P36 + 36 * s;
    float u[24];
    int k = 0;
#pragma unroll
    for (int r = 0; r < 6; ++r)
#pragma unroll
        for (int c = r; c < 6; ++c) u[k++] = p[6 * r + c];
    u[21] = u[22] = u[23] = 0.0f;
#pragma unroll
    for (int q = 0; q < 6; ++q) P24[6 * s + q] = make_float4(u[4 * q], u[4 * q + 1], u[4 * q + 2], u[4 * q + 3]);
    if (site)
        site[s] = fixed[s] ? make_float4(1.0f, 1.0f, 0.0f, 0.0f)
                           : make_float4(mass32[6 * s], mass32[6 * s + 3], 1.0f, 0.0f);
}

__device__ __forceinline__ void sym6(const float4 *P24, float P[21]) {
    float u[24];
#pragma unroll
    for (int q = 0; q < 6; ++q) {
        const float4 v = P24[q];
        u[4 * q] = v.x;
        u[4 * q + 1] = v.y;
        u[4 * q + 2] = v.z;
        u[4 * q + 3] = v.w;
    }
#pragma unroll
    for (int k = 0; k < 21; ++k) P[k] = u[k];
}

__device__ __forceinline__ void sym_mv6(const float P[21], const float x[6], float y[6]) {
    // upper-triangle row-major index of (r, c), r <= c
#define DPF_SYM(r, c) P[(r) * 6 - ((r) * ((r)-1)) / 2 + (c) - (r)]
#pragma unroll
    for (int r = 0; r < 6; ++r) {
        float v = 0.0f;
#pragma unroll
        for (int c = 0; c < 6; ++c) v = fmaf(r <= c ? DPF_SYM(r, c) : DPF_SYM(c, r), x[c], v);
        y[r] = v;
    }
#undef DPF_SYM
}

// ---- bond-end sweep ------------------------------------------------------------
//
// The same operator over the site-sorted incidence CSR instead of tiles: one
// end record per incidence (bond b seen from site s), in the CSR's order,
//   (n', r_s.x) (r_s.y, r_s.z, L, a kn) (a ks, a kb, a kt, other site)
// with n' the unit normal from s towards the other end o and r_s the lever
// of s, so that r_o = r_s - L n' and the end's share of alpha K q is
//   du = u_o - u_s + w_o x r_o - w_s x r_s,  dw = w_o - w_s,
//   f = ks du + (kn - ks)(du.n') n',  m = kb dw + (kt - kb)(dw.n') n',
//   F_s = -f,  T_s = -(r_s x f) - m
// (for the i end this is the bond's wrench on i; for the j end n' = -n and the
// same formula gives the wrench on j).  A group of L lanes owns a site, each
// lane sums the ends k = start + lane, start + lane + L, ..
// in registers and a fixed xor-shuffle tree adds the lanes: no shared
// memory, no atomics, bitwise reproducible.  Records stream from HBM once per
// sweep (evict-first); q of the other ends is gathered from L2.

// Launch shapes of the bond-end sweep: L lanes per site (4, 8 or 16) and B
// resident 256-thread CTAs per SM (the register budget: 64 registers at 4,
// 80 at 3, 128 at 2).  The variants are compiled side by side; callers pick
// one per graph size (dpf_end_variant_shape lists them; variant 0 is 8 lanes,
// 4 CTAs per SM).
constexpr int kEndThreads = 256;
constexpr int kEndPcgThreads = 256;
constexpr int kEndVariants = 6;
constexpr int kEndVariantLanes[kEndVariants] = {8, 4, 16, 8, 4, 8};
constexpr int kEndVariantBlocks[kEndVariants] = {4, 4, 4, 3, 2, 2};

struct EndGraph {
    int64_t n;
    const int32_t *ptr;           // incidence CSR pointers (n + 1)
    const float4 *e0, *e1, *e2;   // end records in incidence order
    const float4 *site;           // per site (mass, inertia, 1 free / 0 fixed, -); fixed sites (1, 1, 0, -)
    const int32_t *seg;           // optional per-site segment (a request of a batch) ...
    const uint8_t *active;        // ... and per-segment flag: sites of inactive segments skip their ends
};

__device__ __forceinline__ void end_wrench(float4 a, float4 b, float4 c, const float qs[6], const float qo[6],
                                           float acc[6]) {
    const float nx = a.x, ny = a.y, nz = a.z;
    const float rx = a.w, ry = b.x, rz = b.y, L = b.z;
    const float ox = rx - L * nx, oy = ry - L * ny, oz = rz - L * nz;
    const float kn = b.w, ks = c.x, kb = c.y, kt = c.z;
    const float wsx = qs[3], wsy = qs[4], wsz = qs[5], wox = qo[3], woy = qo[4], woz = qo[5];
    const float dux = qo[0] - qs[0] + (woy * oz - woz * oy) - (wsy * rz - wsz * ry);
    const float duy = qo[1] - qs[1] + (woz * ox - wox * oz) - (wsz * rx - wsx * rz);
    const float duz = qo[2] - qs[2] + (wox * oy - woy * ox) - (wsx * ry - wsy * rx);
    const float dwx = wox - wsx, dwy = woy - wsy, dwz = woz - wsz;
    const float un = (kn - ks) * (dux * nx + duy * ny + duz * nz);
    const float wn = (kt - kb) * (dwx * nx + dwy * ny + dwz * nz);
    const float fx = ks * dux + un * nx, fy = ks * duy + un * ny, fz = ks * duz + un * nz;
    const float mx = kb * dwx + wn * nx, my = kb * dwy + wn * ny, mz = kb * dwz + wn * nz;
    acc[0] -= fx;
    acc[1] -= fy;
    acc[2] -= fz;
    acc[3] -= (ry * fz - rz * fy) + mx;
    acc[4] -= (rz * fx - rx * fz) + my;
    acc[5] -= (rx * fy - ry * fx) + mz;
}

// ---- L2 residency of the PCG's per-site vectors ----------------------------
// Every CG iteration streams the end records (about 190 MB at 64^3, loaded
// evict-first) through L2 and reads the site vectors u, p, x, w, s, r and the
// block inverses (about 65 MB) again.  Their loads and stores carry an L2
// evict-last policy so that the record stream does not push them out.
__device__ __forceinline__ uint64_t keep_policy() {
    uint64_t pol;
    asm volatile("createpolicy.fractional.L2::evict_last.b64 %0, 1.0;" : "=l"(pol));
    return pol;
}
__device__ __forceinline__ float2 ld2_keep(const float2 *p, uint64_t pol) {
    float2 v;
    asm volatile("ld.global.L2::cache_hint.v2.f32 {%0, %1}, [%2], %3;" : "=f"(v.x), "=f"(v.y) : "l"(p), "l"(pol));
    return v;
}
__device__ __forceinline__ float4 ld4_keep(const float4 *p, uint64_t pol) {
    float4 v;
    asm volatile("ld.global.L2::cache_hint.v4.f32 {%0, %1, %2, %3}, [%4], %5;"
                 : "=f"(v.x), "=f"(v.y), "=f"(v.z), "=f"(v.w)
                 : "l"(p), "l"(pol));
    return v;
}
__device__ __forceinline__ void st2_keep(float2 *p, float2 v, uint64_t pol) {
    asm volatile("st.global.L2::cache_hint.v2.f32 [%0], {%1, %2}, %3;" ::"l"(p), "f"(v.x), "f"(v.y), "l"(pol)
                 : "memory");
}
__device__ __forceinline__ void ld6_keep(const float *p, float v[6], uint64_t pol) {
    const float2 *q = reinterpret_cast<const float2 *>(p);
    const float2 a = ld2_keep(q, pol), b = ld2_keep(q + 1, pol), c = ld2_keep(q + 2, pol);
    v[0] = a.x; v[1] = a.y; v[2] = b.x; v[3] = b.y; v[4] = c.x; v[5] = c.y;
}
__device__ __forceinline__ void st6_keep(float *p, const float v[6], uint64_t pol) {
    float2 *q = reinterpret_cast<float2 *>(p);
    st2_keep(q, make_float2(v[0], v[1]), pol);
    st2_keep(q + 1, make_float2(v[2], v[3]), pol);
    st2_keep(q + 2, make_float2(v[4], v[5]), pol);
}

// q of a site: read-only for the whole launch (kConst) through the
// non-coherent path, else (a PCG updates q between sweeps) with plain loads
// under the evict-last policy.
template <bool kConst>
__device__ __forceinline__ void load_q(const float *q, int64_t s, float v[6]) {
    if (kConst) {
        const float2 *p = reinterpret_cast<const float2 *>(q + 6 * s);
        const float2 a = __ldg(p), b = __ldg(p + 1), c = __ldg(p + 2);
        v[0] = a.x; v[1] = a.y; v[2] = b.x; v[3] = b.y; v[4] = c.x; v[5] = c.y;
    } else {
        ld6_keep(q + 6 * s, v, keep_policy());
    }
}

// For every site s: epi(s, q_s, site record, acc) with acc the alpha K q sum.
// Warp w of the grid takes the chunks w, w + W, ... of 32 / L
// consecutive sites (W warps in the grid).  The round count is the same for
// every warp, so the shuffles see full warps.  A round is a chain of
// dependent loads (CSR bounds, end records, gathers of q_o, site record); the
// next round's CSR bounds are loaded at the start of this one and the site
// record before the shuffle tree, so a round waits on the records and the
// gathers only.  (An L2 prefetch of the next round's records as well made
// the PCG slower: 1.40 vs 1.32 ms per 20 iterations at 64^3.)
template <int L, bool kConst, class Epi>
__device__ __forceinline__ void for_ends(const EndGraph &G, const float *q, Epi &epi) {
    constexpr int kSites = 32 / L;  // sites per warp and round
    const int warps = (int)((int64_t)gridDim.x * blockDim.x / 32);
    const int warp = (int)(((int64_t)blockIdx.x * blockDim.x + threadIdx.x) / 32);
    const int lane32 = (int)threadIdx.x & 31, lane = lane32 & (L - 1);
    const int n = (int)G.n;  // callers bound the site count by 2^31 - 1
    const int64_t chunks = (G.n + kSites - 1) / kSites;
    const int64_t rounds = (chunks + warps - 1) / warps;
    const int step = warps * kSites;  // site stride between rounds (< 2^31: a grid of at most 2^26 warps)
    int s = warp * kSites + lane32 / L;
    int k0 = 0, k1 = 0;
    if (s < n) {
        k0 = G.ptr[s];
        k1 = G.ptr[s + 1];
    }
    for (int64_t r = 0; r < rounds; ++r) {
        const bool valid = s < n;
        const int following = s < n - step ? s + step : n;  // the next round's site (n: none)
        int n0 = 0, n1 = 0;
        if (following < n) {
            n0 = G.ptr[following];
            n1 = G.ptr[following + 1];
        }
        float acc[6] = {0.0f, 0.0f, 0.0f, 0.0f, 0.0f, 0.0f}, qs[6];
        if (valid) load_q<kConst>(q, s, qs);
        if (valid && !(G.active && !G.active[G.seg[s]])) {
            // two ends per step: both ends' records, then both gathers, are in
            // flight together
            for (int k = k0 + lane; k < k1; k += 2 * L) {
                const int k2 = k + L;
                const bool two = k2 < k1;
                const float4 a = __ldcs(G.e0 + k), b = __ldcs(G.e1 + k), c = __ldcs(G.e2 + k);
                float4 a2 = a, b2 = b, c2 = c;
                if (two) {
                    a2 = __ldcs(G.e0 + k2);
                    b2 = __ldcs(G.e1 + k2);
                    c2 = __ldcs(G.e2 + k2);
                }
                float qo[6], qo2[6];
                load_q<kConst>(q, (int64_t)__float_as_int(c.w), qo);
                load_q<kConst>(q, (int64_t)__float_as_int(c2.w), qo2);
                end_wrench(a, b, c, qs, qo, acc);
                if (two) end_wrench(a2, b2, c2, qs, qo2, acc);
            }
        }
        float4 rec = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
        if (valid && lane == 0) rec = G.site[s];
#pragma unroll
        for (int o = 1; o < L; o <<= 1)
#pragma unroll
            for (int c = 0; c < 6; ++c) acc[c] += __shfl_xor_sync(0xffffffffu, acc[c], o);
        if (valid && lane == 0) epi((int64_t)s, qs, rec, acc);
        s = following;
        k0 = n0;
        k1 = n1;
    }
}

struct EndHvpEpi {
    float *y;
    __device__ __forceinline__ void operator()(int64_t s, const float *qs, float4 rec, const float acc[6]) const {
        float out[6];
#pragma unroll
        for (int c = 0; c < 6; ++c) out[c] = fmaf(c < 3 ? rec.x : rec.y, qs[c], rec.z * acc[c]);
        float2 *p = reinterpret_cast<float2 *>(y + 6 * s);
        p[0] = make_float2(out[0], out[1]);
        p[1] = make_float2(out[2], out[3]);
        p[2] = make_float2(out[4], out[5]);
    }
};

template <int L, int B>
__global__ void __launch_bounds__(kEndThreads, B) end_hvp_kernel(EndGraph G, const float *q, float *y) {
    EndHvpEpi epi{y};
    for_ends<L, true>(G, q, epi);
}

// One thread per incidence k of site s (site-major): the end record of bond
// v = inc_bond[k] (v >= 0: s is its i end; ~v: its j end).
struct EndPackArgs {
    int64_t n_inc;
    const int32_t *inc_bond;
    const int64_t *edges;
    const float4 *t0, *t1, *t2, *t3;  // tangent records (n, kn), (ri, ks), (rj, kb), (kt, -, -, -)
    float alpha;
    float4 *e0, *e1, *e2;
};

__global__ void __launch_bounds__(kThreads) pack_ends_kernel(EndPackArgs a) {
    const int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (k >= a.n_inc) return;
    const int v = a.inc_bond[k];
    const bool at_i = v >= 0;
    const int64_t b = at_i ? v : ~v;
    const float4 n = a.t0[b], ri = a.t1[b], rj = a.t2[b], g = a.t3[b];
    const float L = (ri.x - rj.x) * n.x + (ri.y - rj.y) * n.y + (ri.z - rj.z) * n.z;
    const longlong2 e = reinterpret_cast<const longlong2 *>(a.edges)[b];
    const int other = (int)(at_i ? e.y : e.x);
    const float sg = at_i ? 1.0f : -1.0f;
    const float4 r = at_i ? ri : rj;
    a.e0[k] = make_float4(sg * n.x, sg * n.y, sg * n.z, r.x);
    a.e1[k] = make_float4(r.y, r.z, L, a.alpha * n.w);
    a.e2[k] = make_float4(a.alpha * ri.w, a.alpha * rj.w, a.alpha * g.x, __int_as_float(other));
}

// ---- tiled elastic PCG (single-reduction form: two grid barriers per iteration) ----
//
// Same equations and stopping rule as the reference loop: after iteration k's
// update, following = (r, z) is tested when k % 5 == 0 against tol^2 (r0, z0).
// The single-reduction recurrence keeps s = A p and forms (p, A p) from
// (u, A u) = (z, A z):  p = z + beta p, s = w + beta s,
// alpha = gamma / (delta - beta gamma / alpha_prev).

struct PcgArgs {
    int64_t n;
    TileGraph G;  // tiled operator
    Layout L;
    EndGraph E;   // bond-end operator
    const uint8_t *fixed;
    const float4 *P24;
    const float *block, *units32;
    const double *vector;
    const float *vector32;  // float32 input instead of vector (one of the two)
    double tol2;
    int max_it;
    double *out;
    float *out32;           // float32 output instead of out (one of the two)
    int *iterations;
    float *x, *r, *u, *p, *s, *w;  // (N, 6) each
    double *part_a, *part_b;
    unsigned *barrier;
    int *status;
};

struct PcgEpi {
    const PcgArgs &a;
    float dot;
    __device__ __forceinline__ void operator()(int64_t s, const float *qs, float4 rec, const float acc[6]) {
        float wv[6];
        operator_row(rec, qs, acc, wv);
#pragma unroll
        for (int c = 0; c < 6; ++c) dot = fmaf(wv[c], qs[c], dot);
        st6_keep(a.w + 6 * s, wv, keep_policy());
    }
};

__device__ __forceinline__ void mv36(const float *B, const float x[6], float y[6]) {
#pragma unroll
    for (int row = 0; row < 6; ++row) {
        float v = 0.0f;
#pragma unroll
        for (int c = 0; c < 6; ++c) v = fmaf(B[6 * row + c], x[c], v);
        y[row] = v;
    }
}

// One site of the single-reduction update: p = u + beta p, x += alpha p,
// s = w + beta s, r -= alpha s, u = P r; returns (r, u).  Every load of the
// site comes before any store.
__device__ __forceinline__ float update_site(const PcgArgs &a, int64_t s, float fa, float fb) {
    float uv[6], pv[6], xv[6], wv[6], sv[6], rv[6], Pm[21];
    const uint64_t pol = keep_policy();
    ld6_keep(a.u + 6 * s, uv, pol);
    ld6_keep(a.p + 6 * s, pv, pol);
    ld6_keep(a.x + 6 * s, xv, pol);
    ld6_keep(a.w + 6 * s, wv, pol);
    ld6_keep(a.s + 6 * s, sv, pol);
    ld6_keep(a.r + 6 * s, rv, pol);
    {
        float q24[24];
#pragma unroll
        for (int k = 0; k < 6; ++k) {
            const float4 v = ld4_keep(a.P24 + 6 * s + k, pol);
            q24[4 * k] = v.x;
            q24[4 * k + 1] = v.y;
            q24[4 * k + 2] = v.z;
            q24[4 * k + 3] = v.w;
        }
#pragma unroll
        for (int k = 0; k < 21; ++k) Pm[k] = q24[k];
    }
#pragma unroll
    for (int c = 0; c < 6; ++c) {
        pv[c] = fmaf(fb, pv[c], uv[c]);
        xv[c] = fmaf(fa, pv[c], xv[c]);
        sv[c] = fmaf(fb, sv[c], wv[c]);
        rv[c] = fmaf(-fa, sv[c], rv[c]);
    }
    sym_mv6(Pm, rv, uv);
    st6_keep(a.p + 6 * s, pv, pol);
    st6_keep(a.x + 6 * s, xv, pol);
    st6_keep(a.s + 6 * s, sv, pol);
    st6_keep(a.r + 6 * s, rv, pol);
    st6_keep(a.u + 6 * s, uv, pol);
    float dot = 0.0f;
#pragma unroll
    for (int c = 0; c < 6; ++c) dot = fmaf(rv[c], uv[c], dot);
    return dot;
}

// kTiles: w = A u by the tiled sweep, else by the bond-end sweep.
template <bool kTiles, int L>
__device__ __forceinline__ void pcg_body(PcgArgs &a, unsigned char *smem) {
    const int64_t tid = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    const float zero6[6] = {0.0f, 0.0f, 0.0f, 0.0f, 0.0f, 0.0f};
    Pipe P;
    if (kTiles) P = pipe_init(smem, a.L, ((int)blockDim.x - 64) / 32);
    // r0 = B (units v) with fixed rows zero, u0 = P r0, x = p = s = 0
    float pf = 0.0f;
    for (int64_t s = tid; s < a.n; s += stride) {
        float v[6], rr[6], zz[6], Pm[21];
#pragma unroll
        for (int c = 0; c < 6; ++c)
            v[c] = a.units32[6 * s + c] * (a.vector32 ? a.vector32[6 * s + c] : (float)a.vector[6 * s + c]);
        if (a.fixed[s]) {
#pragma unroll
            for (int c = 0; c < 6; ++c) rr[c] = 0.0f;
        } else {
            mv36(a.block + 36 * s, v, rr);
        }
        sym6(a.P24 + 6 * s, Pm);
        sym_mv6(Pm, rr, zz);
        st6(a.r + 6 * s, rr);
        st6(a.u + 6 * s, zz);
        st6(a.x + 6 * s, zero6);
        st6(a.p + 6 * s, zero6);
        st6(a.s + 6 * s, zero6);
#pragma unroll
        for (int c = 0; c < 6; ++c) pf = fmaf(rr[c], zz[c], pf);
    }
    // CG scalars as float32-pair block partials (no float64 per thread)
    float2 *part_a = reinterpret_cast<float2 *>(a.part_a), *part_b = reinterpret_cast<float2 *>(a.part_b);
    block_pair_partial(pf, part_b);
    if (!grid_barrier(a.barrier, a.status)) return;
    double gamma = pair_total(part_b, gridDim.x);
    const double initial = gamma;
    if (initial == 0.0) {
        for (int64_t e = tid; e < 6 * a.n; e += stride) {
            if (a.out32)
                a.out32[e] = 0.0f;
            else
                a.out[e] = 0.0;
        }
        return;
    }
    double alpha_prev = 1.0, gamma_prev = 1.0;
    int it = 0;
    for (; it < a.max_it; ++it) {
        // w = A u over the tiles of this block, delta partial (w, u)
        PcgEpi epi{a, 0.0f};
        bool ok = true;
        if (kTiles)
            ok = for_tiles(a.G, a.L, P, a.u, a.status, epi);
        else
            for_ends<L, false>(a.E, a.u, epi);
        block_pair_partial(epi.dot, part_a);
        if (!ok) return;
        if (!grid_barrier(a.barrier, a.status)) return;
        const double delta = pair_total(part_a, gridDim.x);
        // the recurrence's three float64 divisions once per block (thread 0),
        // not once per thread: float64 division is slow on this part
        __shared__ double shared_ab[2];
        if (threadIdx.x == 0) {
            double beta, alpha;
            if (it == 0) {
                beta = 0.0;
                alpha = gamma / delta;
            } else {
                beta = gamma / gamma_prev;
                alpha = gamma / (delta - beta * gamma / alpha_prev);
            }
            shared_ab[0] = alpha;
            shared_ab[1] = beta;
        }
        __syncthreads();
        const double alpha = shared_ab[0], beta = shared_ab[1];
        const float fa = (float)alpha, fb = (float)beta;
        pf = 0.0f;
        for (int64_t s = tid; s < a.n; s += stride) pf += update_site(a, s, fa, fb);
        block_pair_partial(pf, part_b);
        if (!grid_barrier(a.barrier, a.status)) return;
        const double following = pair_total(part_b, gridDim.x);
        if (it % 5 == 0 && following <= a.tol2 * initial) break;
        gamma_prev = gamma;
        gamma = following;
        alpha_prev = alpha;
    }
    for (int64_t s = tid; s < a.n; s += stride) {
        float xv[6];
        ld6(a.x + 6 * s, xv);
#pragma unroll
        for (int c = 0; c < 6; ++c) {
            const float v = xv[c] / a.units32[6 * s + c];
            if (a.out32)
                a.out32[6 * s + c] = v;
            else
                a.out[6 * s + c] = (double)v;
        }
    }
    if (tid == 0) atomicAdd(a.iterations, it < a.max_it ? it + 1 : a.max_it);
}

__global__ void __launch_bounds__(kTileThreadsMax + 64, DPF_TILE_MIN_BLOCKS) tiled_pcg_kernel(PcgArgs a) {
    extern __shared__ __align__(16) unsigned char smem[];
    pcg_body<true, 8>(a, smem);
}

template <int L, int B>
__global__ void __launch_bounds__(kEndPcgThreads, B) end_pcg_kernel(PcgArgs a) {
    pcg_body<false, L>(a, nullptr);
}

// The kernels of variant v (0 <= v < kEndVariants).
using EndHvpKernel = void (*)(EndGraph, const float *, float *);
using EndPcgKernel = void (*)(PcgArgs);
inline EndHvpKernel end_hvp_variant(int v) {
    switch (v) {
    case 1: return end_hvp_kernel<4, 4>;
    case 2: return end_hvp_kernel<16, 4>;
    case 3: return end_hvp_kernel<8, 3>;
    case 4: return end_hvp_kernel<4, 2>;
    case 5: return end_hvp_kernel<8, 2>;
    default: return end_hvp_kernel<8, 4>;
    }
}
inline EndPcgKernel end_pcg_variant(int v) {
    switch (v) {
    case 1: return end_pcg_kernel<4, 4>;
    case 2: return end_pcg_kernel<16, 4>;
    case 3: return end_pcg_kernel<8, 3>;
    case 4: return end_pcg_kernel<4, 2>;
    case 5: return end_pcg_kernel<8, 2>;
    default: return end_pcg_kernel<8, 4>;
    }
}

inline int blocks_for(int64_t n, int threads) { return (int)((n + threads - 1) / threads); }

}  // namespace tiles
}  // namespace dpf

using namespace dpf;
using namespace dpf::tiles;

namespace {

constexpr int kMaxPcgBlocksTiled = 4096;
// dynamic shared memory cap per CTA (the static reduction buffers need the rest)
constexpr size_t kMaxTileSmem = 220 * 1024;

bool tiles_ok(const dpf_tiles *t) {
    return t && t->n_tiles > 0 && t->tile_desc && t->tile_meta && t->max_entries >= 0 && t->max_sites > 0 &&
           t->max_meta_words > 0 && (t->n_entries == 0 || (t->entry_ends && t->entry_bond)) &&
           ((uintptr_t)t->tile_desc & 15u) == 0;
}

TileGraph tile_graph(const dpf_tiles *t, const float *entries, const float *site) {
    const float4 *p = reinterpret_cast<const float4 *>(entries);
    return TileGraph{(int32_t)t->n_tiles, reinterpret_cast<const int4 *>(t->tile_desc), t->tile_meta, p,
                     p + t->n_entries, p + 2 * t->n_entries, reinterpret_cast<const float4 *>(site)};
}

size_t round16(size_t v) { return (v + 15) & ~(size_t)15; }

Layout layout_of(const dpf_tiles *t, int stages) {
    Layout L;
    L.plane = 16u * (uint32_t)t->max_entries;
    L.qown = 3 * L.plane;
    L.qhalo = L.qown + (uint32_t)round16(24 * (size_t)t->max_sites + 16);
    L.site = L.qhalo + (uint32_t)round16(24 * (size_t)(t->max_halo > 0 ? t->max_halo : 1));
    L.meta = L.site + 16u * (uint32_t)t->max_sites;
    L.head = (uint32_t)round16(L.meta + 4u * (uint32_t)t->max_meta_words);
    L.size = L.head + 32u;
    L.stages = stages;
    return L;
}

size_t smem_bytes(const Layout &L) { return (size_t)L.stages * L.size + 24 * (size_t)L.stages; }

// A ring of `stages` buffers (3..4); 0 picks the deepest within the cap.
Layout pick_layout(const dpf_tiles *t, int stages) {
    if (stages >= 3) return layout_of(t, stages);
    const Layout L = layout_of(t, 4);
    return smem_bytes(L) <= kMaxTileSmem ? L : layout_of(t, 3);
}

bool aligned16(const void *p) { return ((uintptr_t)p & 15u) == 0; }

// Launch checks shared by the tiled kernels; returns the dynamic shared memory.
int tile_launch_check(const dpf_tiles *t, int threads, int stages, size_t &smem) {
    if (threads < 64 || threads > kTileThreadsMax || threads % 32 || stages < 0 || stages == 1 || stages == 2 ||
        stages > 4)
        return DPF_ERR_ARGUMENT;
    if (t->max_entries > kPer * threads) return DPF_ERR_TOO_LARGE;
    smem = smem_bytes(pick_layout(t, stages));
    if (smem > kMaxTileSmem) return DPF_ERR_TOO_LARGE;
    return DPF_OK;
}

// Launch shape of a persistent tiled kernel: shared-memory attributes and the
// occupancy query run once per (device, kernel, threads, shared memory) and
// are cached, so a launch costs no extra driver calls.
struct GridKey {
    int dev;
    const void *kernel;
    int threads;
    size_t smem;
};

template <class K>
int persistent_grid(K kernel, int threads, size_t smem, int64_t n_tiles, int64_t cap, int &grid, bool tiled = true) {
    static GridKey keys[64];
    static int values[64];
    static int used = 0;
    static std::mutex lock;
    std::lock_guard<std::mutex> guard(lock);
    int dev = 0;
    cudaGetDevice(&dev);
    int per_grid = 0;
    for (int k = 0; k < used; ++k)
        if (keys[k].dev == dev && keys[k].kernel == (const void *)kernel && keys[k].threads == threads &&
            keys[k].smem == smem)
            per_grid = values[k];
    if (per_grid == 0) {
        // the attribute is the cap (not this shape's size): any cached shape stays
        // launchable; the bond-end sweep uses no shared memory and prefers L1
        if ((tiled && cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kMaxTileSmem) !=
                          cudaSuccess) ||
            cudaFuncSetAttribute(kernel, cudaFuncAttributePreferredSharedMemoryCarveout, tiled ? 100 : 0) !=
                cudaSuccess) {
            cudaGetLastError();
            return DPF_ERR_CUDA;
        }
        int sms = 0, per_sm = 0;
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, threads, smem);
        if (sms <= 0 || per_sm <= 0) return DPF_ERR_CUDA;
        per_grid = sms * per_sm;
        const int slot = used < 64 ? used++ : (int)(((uintptr_t)kernel + (uintptr_t)smem + threads) % 64);
        keys[slot] = GridKey{dev, (const void *)kernel, threads, smem};
        values[slot] = per_grid;
    }
    int64_t g = per_grid;
    if (g > n_tiles) g = n_tiles;
    if (g > cap) g = cap;
    grid = (int)g;
    return DPF_OK;
}

}  // namespace

extern "C" {

int dpf_tile_graph(int64_t n_sites, int64_t n_bonds, const int64_t *edges, const int32_t *inc_ptr,
                   const int32_t *inc_bond, int32_t max_entries, int32_t max_stage, int32_t *tile_site,
                   int32_t *tile_entry, int32_t *tile_halo, int32_t *tile_meta_off, int32_t *halo_site,
                   int32_t *entry_bond, uint32_t *entry_ends, uint32_t *tile_meta, int64_t meta_capacity,
                   int32_t *tile_desc, int64_t *counts) {
    if (n_sites <= 0 || n_sites > INT32_MAX || n_bonds < 0 || n_bonds > INT32_MAX / 2 || !inc_ptr || !counts ||
        (n_bonds && (!edges || !inc_bond || !entry_bond || !entry_ends || !halo_site)) || !tile_site ||
        !tile_entry || !tile_halo || !tile_meta_off || !tile_meta || !tile_desc || max_entries < 1 ||
        max_entries > 32767 ||
        max_stage < 1 || max_stage > 65535 || meta_capacity < 4)
        return DPF_ERR_ARGUMENT;
    if (inc_ptr[0] != 0 || inc_ptr[n_sites] != 2 * n_bonds) return DPF_ERR_ARGUMENT;
    for (int64_t b = 0; b < n_bonds; ++b) {
        const int64_t i = edges[2 * b], j = edges[2 * b + 1];
        if (i < 0 || j < 0 || i >= n_sites || j >= n_sites || i == j) return DPF_ERR_ARGUMENT;
    }
    std::vector<int32_t> bond_mark((size_t)n_bonds, -1), site_mark((size_t)n_sites, -1);
    // the far end of incidence v (v >= 0: the site is the bond's i end)
    auto other = [&](int32_t v) -> int64_t {
        const int64_t b = v >= 0 ? v : ~v;
        return v >= 0 ? edges[2 * b + 1] : edges[2 * b];
    };
    // pass 1: tile boundaries (greedy in site order: grow while the entries and
    // the staged own + halo sites fit)
    int32_t t = 0;
    int64_t s0 = 0, ent = 0, stage = 0;
    tile_site[0] = 0;
    for (int64_t s = 0; s < n_sites; ++s) {
        int64_t ne = 0, nst = site_mark[s] != t ? 1 : 0;
        for (int32_t k = inc_ptr[s]; k < inc_ptr[s + 1]; ++k) {
            const int32_t v = inc_bond[k];
            const int64_t b = v >= 0 ? v : ~v;
            if (bond_mark[b] != t) ++ne;
            if (site_mark[other(v)] != t) ++nst;
        }
        if (s > s0 && (ent + ne > max_entries || stage + nst > max_stage)) {
            ++t;
            tile_site[t] = (int32_t)s;
            s0 = s;
            ent = stage = 0;
            ne = inc_ptr[s + 1] - inc_ptr[s];
            nst = 1 + ne;
        }
        if (ne > max_entries || nst > max_stage) return DPF_ERR_TOO_LARGE;
        for (int32_t k = inc_ptr[s]; k < inc_ptr[s + 1]; ++k) {
            const int32_t v = inc_bond[k];
            bond_mark[v >= 0 ? v : ~v] = t;
            site_mark[other(v)] = t;
        }
        site_mark[s] = t;
        ent += ne;
        stage += nst;
    }
    const int32_t n_tiles = t + 1;
    tile_site[n_tiles] = (int32_t)n_sites;
    // pass 2: entries (first-encounter order), halo slots, local ends, metadata
    std::fill(bond_mark.begin(), bond_mark.end(), -1);
    std::fill(site_mark.begin(), site_mark.end(), -1);
    std::vector<int32_t> bond_local((size_t)n_bonds, 0), site_local((size_t)n_sites, 0);
    int64_t e = 0, h = 0, words = 0, max_e = 0, max_st = 0, max_t = 0, max_h = 0, max_w = 0;
    for (int32_t tt = 0; tt < n_tiles; ++tt) {
        const int64_t a = tile_site[tt], bnd = tile_site[tt + 1], T = bnd - a;
        tile_entry[tt] = (int32_t)e;
        tile_halo[tt] = (int32_t)h;
        for (int64_t s = a; s < bnd; ++s)
            for (int32_t k = inc_ptr[s]; k < inc_ptr[s + 1]; ++k) {
                const int32_t v = inc_bond[k];
                const int64_t b = v >= 0 ? v : ~v;
                if (bond_mark[b] != tt) {
                    bond_mark[b] = tt;
                    bond_local[b] = (int32_t)(e - tile_entry[tt]);
                    entry_bond[e++] = (int32_t)b;
                }
                const int64_t o = other(v);
                if ((o < a || o >= bnd) && site_mark[o] != tt) {
                    site_mark[o] = tt;
                    site_local[o] = (int32_t)(T + (h - tile_halo[tt]));
                    halo_site[h++] = (int32_t)o;
                }
            }
        const int64_t n_e = e - tile_entry[tt], n_h = h - tile_halo[tt];
        if (n_e > max_entries || T + n_h > max_stage) return DPF_ERR_TOO_LARGE;
        max_e = std::max(max_e, n_e);
        max_st = std::max(max_st, T + n_h);
        max_t = std::max(max_t, T);
        max_h = std::max(max_h, n_h);
        for (int64_t k = tile_entry[tt]; k < e; ++k) {
            const int64_t b = entry_bond[k];
            const int64_t i = edges[2 * b], j = edges[2 * b + 1];
            const uint32_t li = (uint32_t)(i >= a && i < bnd ? i - a : site_local[i]);
            const uint32_t lj = (uint32_t)(j >= a && j < bnd ? j - a : site_local[j]);
            entry_ends[k] = li | (lj << 16);
        }
        // metadata: T + 1 incidence offsets, the uint16 codes (padded to 16
        // bytes), then the halo sites (int32, padded to 16 bytes)
        const int64_t k0 = inc_ptr[a], n_inc = inc_ptr[bnd] - k0;
        const int64_t w_codes = ((T + 1 + (n_inc + 1) / 2) + 3) & ~(int64_t)3;
        const int64_t w = w_codes + ((n_h + 3) & ~(int64_t)3);
        if (words + w > meta_capacity) return DPF_ERR_TOO_LARGE;
        tile_meta_off[tt] = (int32_t)words;
        uint32_t *m = tile_meta + words;
        for (int64_t k = 0; k < w; ++k) m[k] = 0u;
        if (n_inc > 65535) return DPF_ERR_TOO_LARGE;
        for (int64_t k = 0; k <= T; ++k) {
            const int64_t s = a + k, start = inc_ptr[s] - k0;
            int64_t mid = start;
            if (k < T) {
                while (mid < inc_ptr[s + 1] - k0 && inc_bond[k0 + mid] >= 0) ++mid;
                for (int64_t r = mid; r < inc_ptr[s + 1] - k0; ++r)
                    if (inc_bond[k0 + r] >= 0) return DPF_ERR_ARGUMENT;  // i ends must precede j ends
            }
            m[k] = (uint32_t)start | ((uint32_t)mid << 16);
        }
        for (int64_t k = 0; k < n_inc; ++k) {
            const int32_t v = inc_bond[k0 + k];
            const uint32_t code = (uint32_t)bond_local[v >= 0 ? v : ~v];
            const int64_t word = T + 1 + k / 2;
            m[word] |= (k & 1) ? (code << 16) : code;  // little-endian uint16 pairs
        }
        for (int64_t k = 0; k < n_h; ++k) m[w_codes + k] = (uint32_t)halo_site[tile_halo[tt] + k];
        words += w;
        max_w = std::max(max_w, w);
    }
    tile_entry[n_tiles] = (int32_t)e;
    tile_halo[n_tiles] = (int32_t)h;
    tile_meta_off[n_tiles] = (int32_t)words;
    for (int32_t tt = 0; tt < n_tiles; ++tt) {
        int32_t *d = tile_desc + 8 * (int64_t)tt;
        d[0] = tile_site[tt];
        d[1] = tile_site[tt + 1] - tile_site[tt];
        d[2] = tile_entry[tt + 1] - tile_entry[tt];
        d[3] = tile_halo[tt + 1] - tile_halo[tt];
        d[4] = tile_entry[tt];
        d[5] = tile_halo[tt];
        d[6] = tile_meta_off[tt];
        d[7] = tile_meta_off[tt + 1] - tile_meta_off[tt];
    }
    counts[0] = n_tiles;
    counts[1] = e;
    counts[2] = h;
    counts[3] = words;
    counts[4] = max_e;
    counts[5] = max_t;
    counts[6] = max_h;
    counts[7] = max_w;
    counts[8] = max_st;
    return DPF_OK;
}

int64_t dpf_tile_entry_floats(int64_t n_entries) { return 12 * n_entries; }

int64_t dpf_tile_meta_capacity(int64_t n_sites, int64_t n_bonds) { return 9 * n_sites + 3 * n_bonds + 16; }

int dpf_tile_pack(const dpf_tiles *t, const float *bond_data, int64_t n_bonds, double alpha, const float *P36,
                  const float *mass32, const uint8_t *fixed, int64_t n_sites, float *entries, float *P24,
                  float *site4, void *stream) {
    if (!tiles_ok(t) || !bond_data || !entries || !aligned16(bond_data) || !aligned16(entries) ||
        (P24 && (!P36 || !aligned16(P24) || n_sites <= 0)) ||
        (site4 && (!mass32 || !fixed || !aligned16(site4) || n_sites <= 0)))
        return DPF_ERR_ARGUMENT;
    cudaStream_t st = (cudaStream_t)stream;
    // tangent planes of the mixed bond data: records (7 M float4) then t0..t3
    const float4 *base = reinterpret_cast<const float4 *>(bond_data);
    if (t->n_entries) {
        float4 *e = reinterpret_cast<float4 *>(entries);
        PackArgs a{t->n_entries, t->entry_bond, t->entry_ends, base + 7 * n_bonds, base + 8 * n_bonds,
                   base + 9 * n_bonds, base + 10 * n_bonds, (float)alpha, e, e + t->n_entries,
                   e + 2 * t->n_entries};
        pack_entries_kernel<<<blocks_for(t->n_entries, kThreads), kThreads, 0, st>>>(a);
    }
    if (P24 || site4)
        pack_sites_kernel<<<blocks_for(n_sites, kThreads), kThreads, 0, st>>>(
            n_sites, P36, mass32, fixed, reinterpret_cast<float4 *>(P24), reinterpret_cast<float4 *>(site4));
    DPF_CHECK_LAUNCH();
    return DPF_OK;
}

int dpf_tiled_hvp(const dpf_graph *g, const dpf_tiles *t, const float *entries, const float *site4, const float *q,
                  float *y, int *status, int threads, int stages, void *stream) {
    if (!g || !tiles_ok(t) || !entries || !site4 || !q || !y || !status || !aligned16(entries) ||
        !aligned16(site4) || !aligned16(q) || !aligned16(y))
        return DPF_ERR_ARGUMENT;
    size_t smem = 0;
    int rc = tile_launch_check(t, threads, stages, smem);
    if (rc) return rc;
    int grid = 0;
    rc = persistent_grid(tiled_hvp_kernel, threads + 64, smem, t->n_tiles, INT32_MAX, grid);
    if (rc) return rc;
    HvpArgs a{tile_graph(t, entries, site4), pick_layout(t, stages), q, y, status};
    tiled_hvp_kernel<<<grid, threads + 64, smem, (cudaStream_t)stream>>>(a);
    DPF_CHECK_LAUNCH();
    return DPF_OK;
}

int64_t dpf_tiled_workspace_floats(int64_t n_sites) { return 36 * n_sites; }

int dpf_tiled_precondition(const dpf_graph *g, const dpf_tiles *t, const float *entries, const float *site4,
                           const uint8_t *fixed, const float *block32, const float *P24, const float *units32,
                           const double *vector, double tolerance, int max_iterations, double *out, int *iterations,
                           float *workspace, double *partials, unsigned *barrier, int *status, int threads,
                           int stages, void *stream) {
    if (!g || !tiles_ok(t) || g->n_sites <= 0 || !entries || !site4 || !fixed || !block32 || !P24 || !units32 ||
        !vector || !out || !iterations || !workspace || !partials || !barrier || !status || max_iterations < 1 ||
        !aligned16(entries) || !aligned16(workspace) || !aligned16(P24) || !aligned16(site4))
        return DPF_ERR_ARGUMENT;
    size_t smem = 0;
    int rc = tile_launch_check(t, threads, stages, smem);
    if (rc) return rc;
    int grid = 0;
    rc = persistent_grid(tiled_pcg_kernel, threads + 64, smem, t->n_tiles, kMaxPcgBlocksTiled, grid);
    if (rc) return rc;
    const int64_t n6 = 6 * g->n_sites;
    PcgArgs a{};
    a.n = g->n_sites;
    a.G = tile_graph(t, entries, site4);
    a.L = pick_layout(t, stages);
    a.fixed = fixed;
    a.P24 = reinterpret_cast<const float4 *>(P24);
    a.block = block32;
    a.units32 = units32;
    a.vector = vector;
    a.tol2 = tolerance * tolerance;
    a.max_it = max_iterations;
    a.out = out;
    a.iterations = iterations;
    a.x = workspace;
    a.r = workspace + n6;
    a.u = workspace + 2 * n6;
    a.p = workspace + 3 * n6;
    a.s = workspace + 4 * n6;
    a.w = workspace + 5 * n6;
    a.part_a = partials;
    a.part_b = partials + kMaxPcgBlocksTiled;
    a.barrier = barrier;
    a.status = status;
    // a wait that timed out in an earlier launch leaves a partial arrival count
    if (cudaMemsetAsync(barrier, 0, 2 * sizeof(unsigned), (cudaStream_t)stream) != cudaSuccess) {
        cudaGetLastError();
        return DPF_ERR_CUDA;
    }
    void *args[] = {&a};
    if (cudaLaunchCooperativeKernel((const void *)tiled_pcg_kernel, grid, threads + 64, args, smem,
                                    (cudaStream_t)stream) != cudaSuccess) {
        cudaGetLastError();  // report it here, not at the next caller's launch check
        return DPF_ERR_CUDA;
    }
    return DPF_OK;
}

int64_t dpf_tiled_partials_doubles(void) { return 2 * kMaxPcgBlocksTiled; }

int64_t dpf_end_floats(int64_t n_bonds) { return n_bonds < 0 ? 0 : 24 * n_bonds; }

int dpf_end_pack(const dpf_graph *g, const float *bond_data, double alpha, const float *P36, const float *mass32,
                 const uint8_t *fixed, float *ends, float *P24, float *site4, void *stream) {
    if (!g || g->n_sites <= 0 || !g->inc_ptr || (g->n_bonds && (!g->edges || !g->inc_bond || !bond_data || !ends ||
                                                                !aligned16(bond_data) || !aligned16(ends))) ||
        (P24 && (!P36 || !aligned16(P24))) || (site4 && (!mass32 || !fixed || !aligned16(site4))))
        return DPF_ERR_ARGUMENT;
    cudaStream_t st = (cudaStream_t)stream;
    const int64_t m = g->n_bonds, n_inc = 2 * m;
    if (m) {
        const float4 *base = reinterpret_cast<const float4 *>(bond_data);
        float4 *e = reinterpret_cast<float4 *>(ends);
        EndPackArgs a{n_inc, g->inc_bond, g->edges, base + 7 * m, base + 8 * m, base + 9 * m, base + 10 * m,
                      (float)alpha, e, e + n_inc, e + 2 * n_inc};
        pack_ends_kernel<<<blocks_for(n_inc, kThreads), kThreads, 0, st>>>(a);
    }
    if (P24 || site4)
        pack_sites_kernel<<<blocks_for(g->n_sites, kThreads), kThreads, 0, st>>>(
            g->n_sites, P36, mass32, fixed, reinterpret_cast<float4 *>(P24), reinterpret_cast<float4 *>(site4));
    DPF_CHECK_LAUNCH();
    return DPF_OK;
}

static EndGraph end_graph(const dpf_graph *g, const float *ends, const float *site4,
                          const int32_t *seg_site = nullptr, const uint8_t *active = nullptr) {
    const float4 *e = reinterpret_cast<const float4 *>(ends);
    const int64_t n_inc = 2 * g->n_bonds;
    return EndGraph{g->n_sites, g->inc_ptr, e, e + n_inc, e + 2 * n_inc, reinterpret_cast<const float4 *>(site4),
                    seg_site, active};
}

int dpf_end_variant_count(void) { return kEndVariants; }

int dpf_end_variant_shape(int variant, int *lanes, int *blocks_per_sm) {
    if (variant < 0 || variant >= kEndVariants) return DPF_ERR_ARGUMENT;
    if (lanes) *lanes = kEndVariantLanes[variant];
    if (blocks_per_sm) *blocks_per_sm = kEndVariantBlocks[variant];
    return DPF_OK;
}

int dpf_end_hvp(const dpf_graph *g, const float *ends, const float *site4, const float *q, float *y, int variant,
                void *stream) {
    if (!g || g->n_sites <= 0 || !g->inc_ptr || (g->n_bonds && (!ends || !aligned16(ends))) || !site4 ||
        !aligned16(site4) || !q || !y || ((uintptr_t)q & 7u) || ((uintptr_t)y & 7u) || variant < 0 ||
        variant >= kEndVariants)
        return DPF_ERR_ARGUMENT;
    int grid = 0;
    const EndHvpKernel kernel = end_hvp_variant(variant);
    const int rc = persistent_grid(kernel, kEndThreads, 0, INT32_MAX, INT32_MAX, grid, false);
    if (rc) return rc;
    kernel<<<grid, kEndThreads, 0, (cudaStream_t)stream>>>(end_graph(g, ends, site4), q, y);
    DPF_CHECK_LAUNCH();
    return DPF_OK;
}

static int end_precondition(const dpf_graph *g, const float *ends, const float *site4, const uint8_t *fixed,
                            const float *block32, const float *P24, const float *units32, const double *vector,
                            const float *vector32, double tolerance, int max_iterations, double *out, float *out32,
                            int *iterations, float *workspace, double *partials, unsigned *barrier, int *status,
                            const int32_t *seg_site, const uint8_t *active, int variant, void *stream) {
    if (!g || g->n_sites <= 0 || !g->inc_ptr || (g->n_bonds && (!ends || !aligned16(ends))) || !site4 || !fixed ||
        !block32 || !P24 || !units32 || (!vector && !vector32) || (!out && !out32) || !iterations || !workspace ||
        !partials || !barrier || !status || max_iterations < 1 || !aligned16(workspace) || !aligned16(P24) ||
        !aligned16(site4) || (active && !seg_site) || variant < 0 || variant >= kEndVariants)
        return DPF_ERR_ARGUMENT;
    int grid = 0;
    const EndPcgKernel kernel = end_pcg_variant(variant);
    int rc = persistent_grid(kernel, kEndPcgThreads, 0, INT32_MAX, kMaxPcgBlocksTiled, grid, false);
    if (rc) return rc;
    const int64_t n6 = 6 * g->n_sites;
    PcgArgs a{};
    a.n = g->n_sites;
    a.E = end_graph(g, ends, site4, seg_site, active);
    a.fixed = fixed;
    a.P24 = reinterpret_cast<const float4 *>(P24);
    a.block = block32;
    a.units32 = units32;
    a.vector = vector32 ? nullptr : vector;
    a.vector32 = vector32;
    a.tol2 = tolerance * tolerance;
    a.max_it = max_iterations;
    a.out = out32 ? nullptr : out;
    a.out32 = out32;
    a.iterations = iterations;
    a.x = workspace;
    a.r = workspace + n6;
    a.u = workspace + 2 * n6;
    a.p = workspace + 3 * n6;
    a.s = workspace + 4 * n6;
    a.w = workspace + 5 * n6;
    a.part_a = partials;
    a.part_b = partials + kMaxPcgBlocksTiled;
    a.barrier = barrier;
    a.status = status;
    // a wait that timed out in an earlier launch leaves a partial arrival count
    if (cudaMemsetAsync(barrier, 0, 2 * sizeof(unsigned), (cudaStream_t)stream) != cudaSuccess) {
        cudaGetLastError();
        return DPF_ERR_CUDA;
    }
    void *args[] = {&a};
    if (cudaLaunchCooperativeKernel((const void *)kernel, grid, kEndPcgThreads, args, 0,
                                    (cudaStream_t)stream) !=
        cudaSuccess) {
        cudaGetLastError();
        return DPF_ERR_CUDA;
    }
    return DPF_OK;
}

int dpf_end_precondition(const dpf_graph *g, const float *ends, const float *site4, const uint8_t *fixed,
                         const float *block32, const float *P24, const float *units32, const double *vector,
                         double tolerance, int max_iterations, double *out, int *iterations, float *workspace,
                         double *partials, unsigned *barrier, int *status, const int32_t *seg_site,
                         const uint8_t *active, int variant, void *stream) {
    if (!vector || !out) return DPF_ERR_ARGUMENT;
    return end_precondition(g, ends, site4, fixed, block32, P24, units32, vector, nullptr, tolerance, max_iterations,
                            out, nullptr, iterations, workspace, partials, barrier, status, seg_site, active, variant,
                            stream);
}

int dpf_end_precondition_f32(const dpf_graph *g, const float *ends, const float *site4, const uint8_t *fixed,
                             const float *block32, const float *P24, const float *units32, const float *vector,
                             double tolerance, int max_iterations, float *out, int *iterations, float *workspace,
                             double *partials, unsigned *barrier, int *status, int variant, void *stream) {
    if (!vector || !out) return DPF_ERR_ARGUMENT;
    return end_precondition(g, ends, site4, fixed, block32, P24, units32, nullptr, vector, tolerance, max_iterations,
                            nullptr, out, iterations, workspace, partials, barrier, status, nullptr, nullptr, variant,
                            stream);
}

}  // extern "C"
