"""Host side of the serving form (no GPU): the request sets of the served
stream and of the large served mix, and the HBM footprint used for admission."""
import numpy as np


def test_large_mix_requests():
    from dpf_gb300 import serving
    reqs = serving.large_mix(big=10, small=5, count=4, seed=1, big_steps=3, dt=2e-3)
    assert len(reqs) == 5
    big, small = reqs[0], reqs[1:]
    assert big.sites == 1000 and big.steps == 3 and all(r.steps == 1 for r in small)
    assert all(r.sites == 125 for r in small)
    assert all(r.arrival == 0. and r.dt == 2e-3 for r in reqs)
    assert [r.rid for r in reqs] == list(range(5))
    # the foam: gravity on free sites, nothing on the clamped bottom layer
    f = big.foam
    assert np.allclose(big.load[~f['fixed'], 2], -9.81*f['masses'][~f['fixed']])
    assert not big.load[f['fixed']].any()
    # the requests: their own material and top load
    youngs = {r.foam['young'] for r in small}
    assert len(youngs) == 4 and all(1e4 <= e <= 1e6 for e in youngs)
    for r in small:
        nu = r.foam['young']/(2*r.foam['shear']) - 1
        assert .2 <= nu <= .4
        top = (r.foam['unit'][:, 2] > .95) & ~r.foam['fixed']
        assert (r.load[top, 2] < -9.81*r.foam['masses'][top]).all()


def test_synthetic_stream_is_seeded():
    from dpf_gb300 import serving
    a = serving.synthetic_stream(6, seed=4, sites=(500, 4000), rate=100.)
    b = serving.synthetic_stream(6, seed=4, sites=(500, 4000), rate=100.)
    assert [r.sites for r in a] == [r.sites for r in b]
    assert [r.arrival for r in a] == [r.arrival for r in b]
    assert all(np.array_equal(x.load, y.load) for x, y in zip(a, b))
    assert all(x < y for x, y in zip([r.arrival for r in a], [r.arrival for r in a][1:]))


def test_footprint_grows_with_size():
    from dpf_gb300.serving import footprint_bytes
    assert 0 < footprint_bytes(1000, 7000) < footprint_bytes(2000, 7000) < footprint_bytes(2000, 14000)


def test_concatenated_incidence_equals_the_sorted_one():
    """A batch's incidence CSR laid end to end from its parts' CSRs equals the
    stable device sort of the concatenated edges entry for entry, and slicing a
    request's rows back out gives that request's own CSR."""
    import torch
    from dpf_gb300.newton import device_incidence
    from dpf_gb300.serving import concat_incidence, slice_incidence
    from types import SimpleNamespace
    rng = np.random.default_rng(4)
    parts, edges_all, site_off, bond_off = [], [], [0], [0]
    for n, m in ((7, 12), (1, 0), (30, 80), (5, 9)):
        e = rng.integers(0, n, (m, 2)) if n > 1 else np.zeros((0, 2), dtype=np.int64)
        e = e[e[:, 0] != e[:, 1]]
        edges = torch.as_tensor(e, dtype=torch.int64).reshape(-1, 2)
        ptr, inc = device_incidence(edges, n)
        parts.append(SimpleNamespace(_inc_ptr=ptr, _inc_bond=inc, n_sites=n, n_bonds=len(e)))
        edges_all.append(edges + site_off[-1])
        site_off.append(site_off[-1] + n)
        bond_off.append(bond_off[-1] + len(e))
    ptr, inc = concat_incidence(parts, site_off, bond_off)
    ref_ptr, ref_inc = device_incidence(torch.cat(edges_all), site_off[-1])
    assert torch.equal(ptr, ref_ptr) and torch.equal(inc, ref_inc)
    for k, p in enumerate(parts):
        sp, si = slice_incidence(ptr, inc, (site_off[k], site_off[k + 1]), (2*bond_off[k], 2*bond_off[k + 1]),
                                 bond_off[k])
        assert torch.equal(sp, p._inc_ptr) and torch.equal(si, p._inc_bond)
