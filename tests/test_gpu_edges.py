"""Edge cases of the CUDA solvers: isolated sites, graphs without bonds,
all sites fixed, a high-degree site, an empty step; float64 and mixed
forms, checked against the oracle or the closed form."""
import numpy as np
import pytest

from tests.helpers import host

pytestmark = pytest.mark.gpu

CLASSES = ('NewtonBonds', 'MixedNewtonBonds')


def _solver(cls, points, pairs, masses, fixed, radii=.3, areas=None):
    import dpf_gb300
    pairs = np.asarray(pairs, dtype=np.int64).reshape(-1, 2)
    areas = np.full(len(pairs), .01) if areas is None else areas
    return getattr(dpf_gb300, cls)(np.asarray(points, float), np.full(len(points), radii), pairs, areas,
                                   np.asarray(masses, float), np.asarray(fixed, bool), device='cuda')


def _oracle(points, pairs, masses, fixed, radii=.3, areas=None):
    from oracle import dem
    pairs = np.asarray(pairs, dtype=np.int64).reshape(-1, 2)
    areas = np.full(len(pairs), .01) if areas is None else areas
    return dem.NewtonBonds(np.asarray(points, float), np.full(len(points), radii), pairs, areas,
                           np.asarray(masses, float), np.asarray(fixed, bool))


@pytest.mark.parametrize('cls', CLASSES)
def test_graph_without_bonds_falls_freely(cls):
    points = np.array([[0., 0, 0], [1, 0, 0], [0, 1, 0]])
    s = _solver(cls, points, np.zeros((0, 2)), [1., 2., 3.], [False, False, True])
    load = np.zeros((3, 6))
    load[:, 2] = -9.81*np.array([1., 2., 3.])
    load[2] = 0
    dt = 1e-2
    for _ in range(3):
        s.step(dt, s.tensor(load))
    # implicit midpoint with no bonds: v grows by dt g per step on free sites
    # (float64: exact to rounding; mixed: its float32 linear operator, 1e-6)
    rtol = 1e-12 if cls == 'NewtonBonds' else 1e-6
    v = host(s.v)
    assert np.allclose(v[:2, 2], -9.81*3*dt, rtol=rtol, atol=0)
    assert np.allclose(host(s.x)[:2, 2], -.5*9.81*(3*dt)**2, rtol=rtol, atol=0)
    assert np.array_equal(host(s.x)[2], points[2]) and not v[2].any()


@pytest.mark.parametrize('cls', CLASSES)
def test_all_sites_fixed_keep_their_state(cls):
    points = np.array([[0., 0, 0], [.5, 0, 0], [1, 0, 0]])
    s = _solver(cls, points, [[0, 1], [1, 2]], [1., 1., 1.], [True, True, True])
    load = np.random.default_rng(1).normal(size=(3, 6))
    work, info = s.step(1e-3, s.tensor(load))
    assert info['nonlinear_iterations'] == 0 and work == 0.
    assert np.array_equal(host(s.x), points) and not host(s.v).any()


@pytest.mark.parametrize('cls', CLASSES)
def test_isolated_site_beside_a_bond(cls):
    """A free site with no bond next to a bonded pair, against the oracle."""
    points = np.array([[0., 0, 0], [.5, .02, 0], [3, 3, 3]])
    pairs = [[0, 1]]
    masses, fixed = [1., .5, .2], [True, False, False]
    load = np.zeros((3, 6))
    load[1] = [.3, -.2, .1, .01, .02, -.01]
    load[2, 2] = -1.
    s = _solver(cls, points, pairs, masses, fixed)
    ref = _oracle(points, pairs, masses, fixed)
    for _ in range(3):
        s.step(1e-2, s.tensor(load), tolerance=1e-10, pose_tolerance=1e-9)
        ref.step(1e-2, load, tolerance=1e-10, pose_tolerance=1e-9)
    tol = 1e-9 if cls == 'NewtonBonds' else 1e-6
    assert np.abs(host(s.x) - ref.x).max() <= tol*np.abs(ref.x - points).max()
    assert np.abs(host(s.v) - ref.v).max() <= tol*np.abs(ref.v).max()


@pytest.mark.parametrize('cls', CLASSES)
def test_high_degree_site(cls):
    """One centre bonded to 96 sites on a sphere (the hub's incidence list is
    long enough to span many lanes and tile entries)."""
    rng = np.random.default_rng(3)
    d = rng.normal(size=(96, 3))
    d /= np.linalg.norm(d, axis=1)[:, None]
    points = np.vstack([[0., 0, 0], d*.5])
    pairs = [[0, k] for k in range(1, 97)]
    masses = np.full(97, .2)
    fixed = np.zeros(97, bool)
    fixed[1:10] = True
    load = np.zeros((97, 6))
    load[0] = [1., -2., .5, .1, 0, .05]
    s = _solver(cls, points, pairs, masses, fixed, radii=.1)
    ref = _oracle(points, pairs, masses, fixed, radii=.1)
    for _ in range(2):
        s.step(1e-3, s.tensor(load), tolerance=1e-10, pose_tolerance=1e-9)
        ref.step(1e-3, load, tolerance=1e-10, pose_tolerance=1e-9)
    tol = 1e-9 if cls == 'NewtonBonds' else 1e-6
    assert np.abs(host(s.x) - ref.x).max() <= tol*np.abs(ref.x - points).max()


@pytest.mark.parametrize('cls', CLASSES)
def test_nothing_to_do(cls):
    points = np.array([[0., 0, 0], [.5, 0, 0]])
    s = _solver(cls, points, [[0, 1]], [1., 1.], [True, False])
    work, info = s.step(1e-3, s.tensor(np.zeros((2, 6))))
    assert info['nonlinear_iterations'] == 0 and work == 0.
    assert np.array_equal(host(s.x), points)
