"""CUDA path vs the reference's golden vectors and the CPU oracle (float64).

Tolerances are the reference's own bars: K q 1e-12, blocks 1e-12, JVP 2e-11
(scaled norm, bonded_dem_jvp_checks.py:44), inner CG 1e-8
(bonded_dem_precondition_checks.py:54), full step dx < 1e-8, rotation < 1e-7
(bonded_dem_jvp_checks.py:68).
"""
import numpy as np
import pytest

from tests.conftest import golden, STATE
from tests.helpers import gpu_newton, oracle_newton, rel, host

pytestmark = pytest.mark.gpu

torch = pytest.importorskip('torch')


@pytest.fixture(scope='module', autouse=True)
def _cuda():
    if not torch.cuda.is_available():
        pytest.skip('needs a CUDA GPU')
    import dpf_gb300  # noqa: F401
    from dpf_gb300 import _lib
    _lib.load()


CASES = ['newton_prestressed', 'newton_unstressed']


@pytest.mark.parametrize('case', CASES)
def test_trial_residual_loads_energy(case):
    g = golden(case)
    s = gpu_newton(g)
    y, dt, ext = s.tensor(g['y']), float(g['dt']), s.tensor(g['external'])
    trial = s.trial(y)
    for k in ('force', 'n', 'ri', 'rj', 'x', 'normal', 'fn', 'fs', 'mt', 'mb', 'offset'):
        assert rel(trial[k], g[f'trial_{k}']) < 1e-12, k
    assert rel(s.midpoint_force(y), g['midpoint_force']) < 1e-12
    assert rel(s.residual(y, dt, ext), g['residual']) < 1e-12
    assert rel(s.loads(), g['loads']) < 1e-12
    assert abs(s.energy() - float(g['energy'])) <= 1e-12*abs(float(g['energy']))


@pytest.mark.parametrize('case', CASES)
def test_scaling_jvp_stiffness_precondition(case):
    g = golden(case)
    s = gpu_newton(g)
    y, dt, ext = s.tensor(g['y']), float(g['dt']), s.tensor(g['external'])
    s.prepare_scaling(s.trial(y), dt)
    for k in ('diagonal', 'block', 'units'):
        assert rel(getattr(s, k), g[f'scaling_{k}']) < 1e-12, k
    assert rel(s.preconditioner, g['scaling_preconditioner']) < 1e-9
    ref = s.tensor(g['jvp'])
    jv = s.jacobian_vector(y, s.tensor(g['jvp_direction']), dt, ext)
    err = float(torch.linalg.vector_norm(s.scale_residual(jv - ref))/torch.linalg.vector_norm(s.scale_residual(ref)))
    assert err < 2e-11
    assert rel(s.scale_residual(ref), g['scaled_jvp']) < 1e-9
    assert rel(s.stiffness(s.tensor(g['q'])), g['stiffness_q']) < 1e-12
    s.inner_iterations = 0
    x = s.elastic_precondition(s.tensor(g['vector']), dt)
    assert rel(x, g['elastic_precondition']) < 1e-8
    assert s.inner_iterations == int(g['elastic_inner_iterations'])
    assert torch.equal(x[s.fixed], torch.zeros_like(x[s.fixed]))
    assert torch.equal(s.elastic_precondition(torch.zeros_like(x), dt), torch.zeros_like(x))


@pytest.mark.parametrize('case', CASES)
@pytest.mark.parametrize('tag,backend,pc', [('fgmres_elastic', 'fgmres', 'elastic'),
                                            ('fgmres_block', 'fgmres', 'block'),
                                            ('dense', 'dense', 'elastic')])
def test_full_step_matches_reference(case, tag, backend, pc):
    g = golden(case)
    s = gpu_newton(g)
    energy0 = s.energy()
    work, info = s.step(float(g['dt']), s.tensor(g['step_load']), tolerance=2e-7, backend=backend,
                        preconditioning=pc, linear_tolerance=1e-7)
    assert info['nonlinear_iterations'] == int(g[f'step_{tag}_nonlinear_iterations'])
    assert info['krylov_iterations'] == int(g[f'step_{tag}_krylov_iterations'])
    assert info['cg_iterations'] == int(g[f'step_{tag}_cg_iterations'])
    assert np.abs(host(s.x) - g[f'step_{tag}_state_x']).max() < 1e-8
    assert np.abs(host(s.rotation) - g[f'step_{tag}_state_rotation']).max() < 1e-7
    for k in ('v', 'normal', 'offset', 'fn', 'fs', 'mt', 'mb'):
        ref = g[f'step_{tag}_state_{k}']
        assert np.abs(host(getattr(s, k)) - ref).max() <= 1e-7*max(1., np.abs(ref).max()), k
    assert abs(work - float(g[f'step_{tag}_work'])) <= 1e-8*abs(float(g[f'step_{tag}_work']))
    # work-energy balance (bonded_dem_newton_checks.py:117-118)
    assert abs(s.energy() - energy0 - work)/max(energy0, abs(work), 1e-30) < 1e-5


def test_tangent_81_and_linear_217():
    import dpf_gb300
    g = golden('tangent_81')
    s = dpf_gb300.LinearBonds(g['points'], np.ones(50), g['pairs'], np.ones(len(g['pairs'])), g['contacts'],
                              np.ones(50), np.zeros(50, bool))
    assert rel(s.stiffness(s.tensor(g['q'])), g['stiffness_q']) < 1e-12
    assert rel(s.diagonal, g['diagonal']) < 1e-12
    g = golden('linear_217')
    p = g['points']
    s = dpf_gb300.LinearBonds(p, g['radii'], g['pairs'], g['areas'], g['contacts'], np.ones(len(p)),
                              np.zeros(len(p), bool))
    q = g['q']
    assert rel(s.stiffness(s.tensor(q)).cpu().numpy().ravel(), g['dense_k']@q.ravel()) < 1e-12
    assert np.abs(host(s.diagonal) - g['diagonal']).max() < 1e-10


def test_linear_step_217_matches_reference_and_dense_solve():
    """LinearBonds.step (library PCG, linear stopping test) against the
    reference's own step and the check's dense midpoint solve: positions
    1e-6 of the dense solve and work = energy to 1e-6, as
    bonded_dem_linear_gpu.py:144-155 asserts; the reference's step to 1e-10."""
    import dpf_gb300
    g = golden('linear_step_217')
    p = g['points']
    s = dpf_gb300.LinearBonds(p, g['radii'], g['pairs'], g['areas'], g['contacts'], np.ones(len(p)), g['fixed'])
    work, metrics = s.step(float(g['dt']), s.tensor(g['force']))
    assert rel(s.q, g['dense_q']) < 1e-6
    assert rel(s.q, g['step_q']) < 1e-10
    assert rel(s.v, g['step_v']) < 1e-10
    assert rel(s.kq, g['step_kq']) < 1e-10
    assert abs(work - float(g['step_work'])) <= 1e-10*abs(float(g['step_work']))
    assert abs(s.energy() - work)/work < 1e-6
    assert abs(metrics['iterations'] - int(g['step_iterations'])) <= 10
    assert metrics['relative_residual'] < 5*2e-8
    # the operator and the solve on their own: (diag M + a K) x = b
    alpha = .25*float(g['dt'])**2
    b = s.tensor(np.random.default_rng(1).normal(size=(len(p), 6)))
    x, info = s.solve_increment(b, float(g['dt']))
    r = s._operator(x, alpha) - b
    r[s.fixed] = 0
    assert float(torch.linalg.vector_norm(r)/torch.linalg.vector_norm(b[~s.fixed])) < 5*2e-8
    assert info['relative_residual'] < 5*2e-8


def test_finite_history_953_matches_parallel_bonds():
    import dpf_gb300
    g = golden('finite_953')
    s = dpf_gb300.FiniteBonds(g['points'], g['radii'], g['pairs'], g['areas'], np.ones(8), np.zeros(8, bool))
    for end, v, w in zip(g['ends'], g['vs'], g['ws']):
        s.commit(s.trial(s.tensor(np.c_[v, w]*.01), end_positions=s.tensor(end)))
    for k in ('fn', 'fs', 'mt', 'mb'):
        assert rel(getattr(s, k), g[f'cpu_{k}']) < 1e-12, k
    loads = host(s.loads())
    assert np.linalg.norm(loads[:, :3] - g['cpu_force']) + np.linalg.norm(loads[:, 3:] - g['cpu_torque']) < 1e-10
    assert np.linalg.norm(loads[:, :3].sum(0)) < 1e-10


def test_fgmres_381_dense_system():
    import dpf_gb300
    g = golden('fgmres_381')
    a = torch.as_tensor(g['a'], device='cuda')
    b = torch.as_tensor(g['b'], device='cuda')
    calls = [0]
    diag = torch.diag(a)

    def variable_precondition(v):
        calls[0] += 1
        return v/(diag*(1+.08*np.sin(calls[0])))
    x, info = dpf_gb300.fgmres(lambda z: a@z, b, variable_precondition, tolerance=1e-10, restart=24)
    assert info['iterations'] == int(g['iterations'])
    assert rel(x, g['x']) < 1e-11


def test_lattice8_three_steps():
    import dpf_gb300
    g = golden('lattice8')
    s = dpf_gb300.NewtonBonds(g['points'], g['radii'], g['pairs'], g['areas'], g['masses'], g['fixed'],
                              young=float(g['young']), shear=float(g['shear']))
    infos = []
    for step in range(3):
        work, info = s.step(float(g['dt']), s.tensor(g['load']), tolerance=1e-6)
        infos.append([info['nonlinear_iterations'], info['krylov_iterations'], info['cg_iterations']])
        assert abs(work - float(g[f'work_{step}'])) <= 1e-8*abs(float(g[f'work_{step}']))
    assert np.array_equal(np.array(infos), g['iterations'])
    for k in STATE:
        ref = g[f'state_{k}']
        assert np.abs(host(getattr(s, k)) - ref).max() <= 1e-8*max(1., np.abs(ref).max()), k


def test_lattice16_step_vs_oracle():
    """A 4,096-site foam (about 30k bonds): one GPU step vs the oracle."""
    import dpf_gb300
    from oracle import dem
    foam = dpf_gb300.jittered_lattice_foam(16, seed=0)
    load = dpf_gb300.gravity_load(foam)
    args = (foam['points'], foam['radii'], foam['pairs'], foam['areas'], foam['masses'], foam['fixed'])
    kw = dict(young=foam['young'], shear=foam['shear'])
    s = dpf_gb300.NewtonBonds(*args, **kw)
    o = dem.NewtonBonds(*args, **kw)
    work, info = s.step(1e-3, s.tensor(load), tolerance=1e-6)
    ow, oinfo = o.step(1e-3, load, tolerance=1e-6)
    assert info['nonlinear_iterations'] == oinfo['nonlinear_iterations']
    assert info['krylov_iterations'] == oinfo['krylov_iterations']
    assert abs(info['cg_iterations'] - oinfo['cg_iterations']) <= 5
    assert np.abs(host(s.x) - o.x).max() < 1e-10
    assert abs(work - ow) <= 1e-8*abs(ow)


def test_jvp_and_stiffness_are_deterministic():
    g = golden('newton_prestressed')
    s = gpu_newton(g)
    y, dt = s.tensor(g['y']), float(g['dt'])
    d = s.tensor(g['jvp_direction'])
    a = s.jacobian_vector(y, d, dt, None)
    b = s.jacobian_vector(y, d, dt, None)
    assert torch.equal(a, b)
    q = s.tensor(g['q'])
    assert torch.equal(s.stiffness(q), s.stiffness(q))


def test_guards_raise_and_leave_state_untouched():
    import dpf_gb300
    g = golden('newton_prestressed')
    s = gpu_newton(g)
    before = {k: getattr(s, k).clone() for k in STATE}
    with pytest.raises(dpf_gb300.SubdivideError, match='Subdivide: body rotation'):
        s.trial(torch.ones_like(s.mass))
    big = torch.zeros_like(s.mass)
    big[:, :3] = 5.
    big[0, :3] = -5.
    with pytest.raises(RuntimeError, match='Subdivide:'):
        s.trial(big)
    assert all(torch.equal(getattr(s, k), v) for k, v in before.items())
    # a failed step (Newton iteration cap) raises Subdivide and commits nothing
    with pytest.raises(RuntimeError, match='Subdivide:'):
        s.step(float(g['dt']), s.tensor(g['step_load']), max_iterations=0)
    assert all(torch.equal(getattr(s, k), v) for k, v in before.items())


def test_advance_interval_bisects_on_subdivide():
    """advance_interval halves dt after a Subdivide failure (bonded_dem_finite_gpu.py:252-261)."""
    g = golden('newton_unstressed')
    s = gpu_newton(g)
    o = oracle_newton(g)
    load = np.zeros_like(g['step_load']); load[:, 2] = -.6; load[g['in_fixed']] = 0
    work, records = s.advance_interval(.02, lambda t: s.tensor(load))
    ow, orecords = o.advance_interval(.02, lambda t: load)
    assert [r['subdivision_depth'] for r in orecords] == [1, 1]
    assert [r['subdivision_depth'] for r in records] == [r['subdivision_depth'] for r in orecords]
    assert np.abs(host(s.x) - o.x).max() < 1e-8
    assert abs(work - ow) <= 1e-8*abs(ow)


@pytest.mark.parametrize('case', CASES)
def test_previous_solver_step_matches_reference(case):
    """FiniteBondsGPU.step (PCG + Anderson + merit backtracking) on the GPU."""
    import dpf_gb300
    from tests.conftest import newton_inputs
    g = golden(case)
    s = dpf_gb300.FiniteBonds(**newton_inputs(g))
    for k in STATE:
        setattr(s, k, torch.as_tensor(np.array(g['state_' + k]), dtype=torch.float64, device=s.device).contiguous())
    work, info = s.step(float(g['dt']), s.tensor(g['step_load']), tolerance=2e-7)
    assert info['nonlinear_iterations'] == int(g['step_previous_nonlinear_iterations'])
    assert abs(info['cg_iterations'] - int(g['step_previous_cg_iterations'])) <= 10
    assert np.abs(host(s.x) - g['step_previous_state_x']).max() < 1e-8
    assert np.abs(host(s.rotation) - g['step_previous_state_rotation']).max() < 1e-7
    assert abs(work - float(g['step_previous_work'])) <= 1e-8*abs(float(g['step_previous_work']))
