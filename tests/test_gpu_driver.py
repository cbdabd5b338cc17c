"""The library's native step driver (dpf_mixed_newton_step) against the
Python control path of MixedNewtonBonds.step: the same launches and host
decisions, so every committed array, the returned work and every iteration
count and residual-trace entry must be bit-identical.  Both solvers are given
the same bond-end launch shape, since the autotuner may pick different shapes
for two instances and the shape changes the PCG's summation order."""
import numpy as np
import pytest

from tests.conftest import STATE

pytestmark = pytest.mark.gpu

torch = pytest.importorskip('torch')


@pytest.fixture(scope='module', autouse=True)
def _cuda():
    if not torch.cuda.is_available():
        pytest.skip('needs a CUDA GPU')


def pair(m=10, seed=3, refresh=32):
    import dpf_gb300
    foam = dpf_gb300.jittered_lattice_foam(m, seed=seed)
    args = (foam['points'], foam['radii'], foam['pairs'], foam['areas'], foam['masses'], foam['fixed'])
    kw = dict(young=foam['young'], shear=foam['shear'])
    python, native = dpf_gb300.MixedNewtonBonds(*args, **kw), dpf_gb300.MixedNewtonBonds(*args, **kw)
    python.native = False
    for s in (python, native):
        s._end_variant = 0
        s.refresh_interval = refresh
    return foam, python, native


def assert_same_info(a, b):
    """Every entry bit-identical but the largest rotation, which the driver
    reduces with its own kernel (torch's norm may round the last bit apart)."""
    a, b = dict(a), dict(b)
    ra, rb = a.pop('max_step_rotation'), b.pop('max_step_rotation')
    assert a == b
    assert abs(ra - rb) <= 1e-14*max(abs(ra), 1e-300)


def assert_same_state(a, b):
    for k in STATE:
        ta, tb = getattr(a, k), getattr(b, k)
        assert torch.equal(ta, tb), k


def test_driver_matches_python_path_bit_for_bit():
    import dpf_gb300
    from dpf_gb300 import _lib
    foam, python, native = pair(refresh=3)       # steps 0, 3 refresh the float64 records
    load = dpf_gb300.gravity_load(foam)*4.0
    for step in range(6):
        ext_p, ext_n = python.tensor(load), native.tensor(load)
        before = _lib.LAUNCHES['count']
        wp, ip = python.step(2e-3, ext_p, tolerance=1e-6)
        launched = _lib.LAUNCHES['count']
        wn, inn = native.step(2e-3, ext_n, tolerance=1e-6)
        if step > 0:      # the first step of each solver runs in Python (it sets up the sweep buffers)
            assert native._native_ready('fgmres', 'elastic')
            assert _lib.LAUNCHES['count'] - launched > 10
        assert wp == wn, step
        assert_same_info(ip, inn)
        assert_same_state(python, native)
        assert launched > before
    assert native.time == python.time


def test_driver_timing_fills_the_profile():
    import dpf_gb300
    foam, python, native = pair(m=8)
    load = dpf_gb300.gravity_load(foam)
    native.step(1e-3, native.tensor(load), tolerance=1e-6)      # Python path: sweep buffers
    native.profile = {}
    native.step(1e-3, native.tensor(load), tolerance=1e-6)
    profile, native.profile = native.profile, None
    for key in ('setup', 'residual', 'scaling', 'pcg', 'jvp', 'commit', 'pack', 'krylov', 'norms', 'vector',
                'accept'):
        assert key in profile and all(isinstance(v, float) and v > 0 for v in profile[key]), key


def test_driver_reports_the_same_failures():
    """A load that turns bodies by more than 0.25 rad in a step: both paths raise
    the same Subdivide error and keep the committed state."""
    import dpf_gb300
    foam, python, native = pair(m=8)
    load = dpf_gb300.gravity_load(foam)
    for s in (python, native):
        s.step(1e-3, s.tensor(load), tolerance=1e-6)
    rng = np.random.default_rng(0)
    wild = np.zeros((len(foam['points']), 6))
    wild[:, 3:] = rng.normal(0, 1, (len(foam['points']), 3))*1e6
    errors = []
    for s in (python, native):
        x0 = s.x.clone()
        with pytest.raises(dpf_gb300.SubdivideError) as e:
            s.step(5e-2, s.tensor(wild), tolerance=1e-6)
        errors.append(str(e.value))
        assert torch.equal(s.x, x0)
    assert errors[0] == errors[1]
    # and both go on from there identically
    wp, ip = python.step(1e-3, python.tensor(load), tolerance=1e-6)
    wn, inn = native.step(1e-3, native.tensor(load), tolerance=1e-6)
    assert wp == wn
    assert_same_info(ip, inn)
    assert_same_state(python, native)


def test_lazy_history_matches_eager_commit():
    """Committing steps as exact float32-pair increments and folding them into
    the float64 history on access (or at a refresh) agrees with writing the
    float64 end state every step: bit for bit until the first float64 refresh
    (the records advance the same way), to float64 rounding afterwards."""
    import dpf_gb300
    foam, lazy, eager = pair(m=10, seed=5, refresh=4)
    eager.lazy_history = False
    load = dpf_gb300.gravity_load(foam)*4.0
    for step in range(9):      # the history is read only after the loop: 9 steps, refreshes at 4 and 8
        lazy.step(2e-3, lazy.tensor(load), tolerance=1e-6)
        eager.step(2e-3, eager.tensor(load), tolerance=1e-6)
        if step < 4:
            assert torch.equal(lazy.x, eager.x) and torch.equal(lazy.v, eager.v)
        scale = float(torch.linalg.vector_norm(eager.x - torch.as_tensor(foam['points'], device=eager.x.device)))
        assert float(torch.linalg.vector_norm(lazy.x - eager.x)) <= 1e-12*scale
    assert lazy._pending_fold
    for k in ('fn', 'fs', 'mt', 'mb', 'offset', 'normal'):
        a, b = getattr(lazy, k), getattr(eager, k)
        assert float(torch.linalg.vector_norm(a - b)) <= 1e-12*max(float(torch.linalg.vector_norm(b)), 1e-300), k
    assert not lazy._pending_fold
    # a fold leaves nothing pending and new tensors behind: an old reference keeps its values
    fn_before = lazy.fn.clone()
    held = lazy.fn
    lazy.step(2e-3, lazy.tensor(load), tolerance=1e-6)
    assert torch.equal(held, fn_before)
    assert not torch.equal(lazy.fn, fn_before)
    assert lazy.fn is lazy.fn


def test_committed_start_equals_the_full_first_residual():
    """After a commit the first residual of the next step is r0 (0 on fixed
    sites) and the tangent the commit stored equals the one the residual pass
    forms at y = 0."""
    import dpf_gb300
    foam, s, _ = pair(m=10, seed=7)
    load = dpf_gb300.gravity_load(foam)*4.0
    for _ in range(2):
        s.step(2e-3, s.tensor(load), tolerance=1e-6)
    assert s._committed_start
    m, dt = s.n_bonds, 2e-3
    stored = s._bond_data[7*4*m:10*4*m].clone()
    s._v = s._vec(s.v).clone()
    s._step_begin(dt, s.tensor(load))
    assert s._zero_start
    y = torch.zeros_like(s._v)
    quick = torch.empty_like(y)
    s._call('dpf_mixed_initial_residual', s.n_sites, s._r0.data_ptr(), s.fixed.data_ptr(), s._y32.data_ptr(),
            quick.data_ptr(), s._stream())
    full = s._mixed_residual(y, dt, want_tangent=True, use_p=False)
    assert torch.equal(quick, full)
    recomputed = s._bond_data[7*4*m:10*4*m]
    assert torch.allclose(stored, recomputed, rtol=2e-7, atol=0)
