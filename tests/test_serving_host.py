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
