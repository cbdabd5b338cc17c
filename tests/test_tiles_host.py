"""Host-side checks of the site tiler (``dpf_tile_graph``, plain C++ in the
CUDA library; no GPU needed) and of the tiled operator's data semantics,
emulated in NumPy against the direct (diag M + alpha K) q."""
import numpy as np
import pytest

from tests.conftest import ROOT  # noqa: F401  (puts the repo on sys.path)


def _lib_or_skip():
    from dpf_gb300 import _lib
    try:
        return _lib.load()
    except _lib.LibraryError as e:
        pytest.skip(str(e))


def _graph(m=6, seed=2):
    from dpf_gb300 import foam, newton
    f = foam.jittered_lattice_foam(m, seed=seed)
    edges = np.asarray(f['pairs'], dtype=np.int64)
    ptr, inc = newton.incidence(edges, len(f['points']))
    return f, edges, np.asarray(ptr), np.asarray(inc)


def _decode(t, tile, edges):
    a, b = t['tile_site'][tile], t['tile_site'][tile + 1]
    e0, e1 = t['tile_entry'][tile], t['tile_entry'][tile + 1]
    h0, h1 = t['tile_halo'][tile], t['tile_halo'][tile + 1]
    T = b - a

    def site(local):
        return a + local if local < T else t['halo_site'][h0 + local - T]
    return a, b, e0, e1, h0, h1, site


@pytest.mark.parametrize('max_entries', [48, 200, 2048])
def test_tiles_cover_graph(max_entries):
    _lib_or_skip()
    from dpf_gb300.tiles import host_tiles, tile_codes
    f, edges, ptr, inc = _graph()
    n = len(f['points'])
    t = host_tiles(edges, ptr, inc, n, max_entries)
    ts = t['tile_site']
    assert ts[0] == 0 and ts[-1] == n and np.all(np.diff(ts) > 0)
    assert t['max_entries'] <= max_entries
    total = 0
    for tile in range(t['n_tiles']):
        a, b, e0, e1, h0, h1, site = _decode(t, tile, edges)
        own = set(range(a, b))
        bonds = set(np.nonzero(np.isin(edges[:, 0], list(own)) | np.isin(edges[:, 1], list(own)))[0].tolist())
        entry_bonds = t['entry_bond'][e0:e1].tolist()
        assert len(entry_bonds) == len(set(entry_bonds)) == len(bonds) and set(entry_bonds) == bonds
        assert e1 - e0 <= max_entries and (b - a) + (h1 - h0) <= t['max_stage']
        halo = t['halo_site'][h0:h1].tolist()
        assert len(set(halo)) == len(halo) and not (set(halo) & own)
        for k, bond in enumerate(entry_bonds):
            ends = int(t['entry_ends'][e0 + k])
            assert site(ends & 0xffff) == edges[bond, 0] and site(ends >> 16) == edges[bond, 1]
        lptr, mid, codes = tile_codes(t, tile)
        assert t['tile_meta_off'][tile] % 4 == 0 and len(lptr) == b - a + 1
        assert np.array_equal(lptr, ptr[a:b + 1] - ptr[a])
        for s in range(a, b):
            for k in range(ptr[s], ptr[s + 1]):
                v = int(inc[k])
                code = int(codes[k - ptr[a]])
                assert t['entry_bond'][e0 + code] == (v if v >= 0 else ~v)
                assert (k - ptr[a] >= mid[s - a]) == (v < 0)
        assert t['max_sites'] >= b - a and t['max_halo'] >= h1 - h0
        assert list(t['tile_desc'][8*tile:8*tile + 8]) == [a, b - a, e1 - e0, h1 - h0, e0, h0, t['tile_meta_off'][tile],
                                                           t['tile_meta_off'][tile + 1] - t['tile_meta_off'][tile]]
        words = t['tile_meta'][t['tile_meta_off'][tile]:t['tile_meta_off'][tile + 1]]
        n_halo_words = (h1 - h0 + 3) // 4*4
        assert np.array_equal(words[len(words) - n_halo_words:][:h1 - h0].view(np.int32), t['halo_site'][h0:h1])
        assert t['max_meta_words'] >= t['tile_meta_off'][tile + 1] - t['tile_meta_off'][tile]
        total += e1 - e0
    assert total == t['n_entries'] and t['tile_meta_off'][-1] == t['meta_words']


def test_tiler_rejects_oversized_sites():
    from dpf_gb300 import _lib
    _lib_or_skip()
    from dpf_gb300.tiles import host_tiles
    f, edges, ptr, inc = _graph()
    degree = int(np.diff(ptr).max())
    with pytest.raises(_lib.LibraryError):
        host_tiles(edges, ptr, inc, len(f['points']), max_entries=degree - 1)


def _stiffness_apply(edges, n, ri, rj, k, q):
    """Direct K q in float64 (experiments/bonded_dem_linear_gpu.py:42-52)."""
    i, j = edges[:, 0], edges[:, 1]
    kn, ks, kb, kt = k.T
    du = q[j, :3] - q[i, :3] + np.cross(q[j, 3:], rj) - np.cross(q[i, 3:], ri)
    dw = q[j, 3:] - q[i, 3:]
    f = ks[:, None]*du + ((kn - ks)*np.einsum('bc,bc->b', du, n))[:, None]*n
    m = kb[:, None]*dw + ((kt - kb)*np.einsum('bc,bc->b', dw, n))[:, None]*n
    out = np.zeros_like(q)
    np.add.at(out, i, np.concatenate([-f, -np.cross(ri, f) - m], 1))
    np.add.at(out, j, np.concatenate([f, np.cross(rj, f) + m], 1))
    return out


def test_tiled_operator_semantics_match_direct_product():
    """Emulate the kernel's three steps (stage own + halo q, entry wrenches with
    r_j = r_i - L n, incidence-ordered site sums) from the tiler's arrays."""
    _lib_or_skip()
    from dpf_gb300.tiles import host_tiles, tile_codes
    f, edges, ptr, inc = _graph(m=5, seed=4)
    n_sites, m = len(f['points']), len(edges)
    rng = np.random.default_rng(0)
    p = np.asarray(f['points'])
    nvec = p[edges[:, 1]] - p[edges[:, 0]]
    L = np.linalg.norm(nvec, axis=1)
    nvec /= L[:, None]
    ri = .5*L[:, None]*nvec + rng.normal(0, .01, (m, 3))
    rj = ri - L[:, None]*nvec
    k = rng.uniform(1, 2, (m, 4))
    mass = rng.uniform(1, 2, (n_sites, 2))
    fixed = rng.uniform(size=n_sites) < .1
    alpha = .3
    q = rng.normal(size=(n_sites, 6))
    direct = np.where(fixed[:, None], q, np.repeat(mass, 3, axis=1)*q + alpha*_stiffness_apply(edges, nvec, ri, rj, k, q))
    t = host_tiles(edges, ptr, inc, n_sites, 64)
    y = np.zeros_like(q)
    for tile in range(t['n_tiles']):
        a, b, e0, e1, h0, h1, site = _decode(t, tile, edges)
        stage = np.concatenate([q[a:b], q[t['halo_site'][h0:h1]]])
        W = np.zeros((e1 - e0, 9))
        for e in range(e0, e1):
            bond = t['entry_bond'][e]
            ends = int(t['entry_ends'][e])
            qi, qj = stage[ends & 0xffff], stage[ends >> 16]
            r_i, Lb, nb = ri[bond], L[bond], nvec[bond]
            r_j = r_i - Lb*nb
            kn, ks, kb, kt = alpha*k[bond]
            du = qj[:3] - qi[:3] + np.cross(qj[3:], r_j) - np.cross(qi[3:], r_i)
            dw = qj[3:] - qi[3:]
            fv = ks*du + (kn - ks)*du.dot(nb)*nb
            mv = kb*dw + (kt - kb)*dw.dot(nb)*nb
            W[e - e0] = np.concatenate([-fv, -np.cross(r_i, fv) - mv, np.cross(r_j, fv) + mv])
        lptr, mid, codes = tile_codes(t, tile)
        for s in range(a, b):
            acc = np.zeros(6)
            for kk in range(lptr[s - a], lptr[s - a + 1]):
                w = W[int(codes[kk])]
                acc += w[:6] if kk < mid[s - a] else np.concatenate([-w[:3], w[6:]])
            y[s] = q[s] if fixed[s] else np.repeat(mass[s], 3)*q[s] + acc
    assert np.abs(y - direct).max() <= 1e-12*np.abs(direct).max()


def test_end_sweep_tuner_borrows_the_nearest_tuned_class():
    """An untuned size class takes the launch shape of the closest tuned class
    within ``nearest`` classes (the larger one on a tie); the cache is keyed by
    (device, log2 of incidences)."""
    from types import SimpleNamespace
    from dpf_gb300 import tiles
    saved = dict(tiles._END_TUNED)
    try:
        tiles._END_TUNED.clear()
        tiles._END_TUNED[(0, 20)] = (3, {})
        tiles._END_TUNED[(0, 24)] = (5, {})
        tiles._END_TUNED[(1, 22)] = (1, {})
        solver = lambda bonds: SimpleNamespace(device=SimpleNamespace(index=0), n_sites=1, n_bonds=bonds)
        assert tiles.end_size_class(1, 1 << 20) == 21
        assert tiles.tune_end_sweep(solver(1 << 19), None, nearest=0) == 3       # class 20 itself
        assert tiles.tune_end_sweep(solver(1 << 20), None, nearest=2) == 3       # 21: 20 is one away
        assert tiles.tune_end_sweep(solver(1 << 21), None, nearest=2) == 5       # 22: 20 and 24 tie, larger wins
        assert tiles.tune_end_sweep(solver(1 << 24), None, nearest=1) == 5       # 25: 24 is one away
        assert (0, 22) not in tiles._END_TUNED                                   # borrowed, not cached
    finally:
        tiles._END_TUNED.clear()
        tiles._END_TUNED.update(saved)
