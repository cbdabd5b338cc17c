"""Pin the NumPy oracle against vectors produced by the reference's own code."""
import numpy as np
import pytest

from oracle import dem
from tests.conftest import golden, newton_inputs, STATE


def rel(a, b):
    return float(np.linalg.norm(np.asarray(a) - np.asarray(b))/max(np.linalg.norm(b), 1e-300))


def oracle_newton(g, prefix='state_'):
    s = dem.NewtonBonds(**newton_inputs(g))
    for k in STATE:
        setattr(s, k, np.array(g[prefix + k]))
    return s


@pytest.mark.parametrize('case', ['newton_prestressed', 'newton_unstressed'])
def test_trial_force_jvp_precondition(case):
    g = golden(case)
    s = oracle_newton(g)
    y, dt, ext = g['y'], float(g['dt']), g['external']
    trial = s.trial(y)
    for k in ('force', 'n', 'ri', 'rj', 'x', 'normal', 'fn', 'fs', 'mt', 'mb', 'offset'):
        assert rel(trial[k], g[f'trial_{k}']) < 1e-13, k
    assert rel(s.midpoint_force(y), g['midpoint_force']) < 1e-13
    assert rel(s.residual(y, dt, ext), g['residual']) < 1e-13
    assert rel(s.loads(), g['loads']) < 1e-13
    assert abs(s.energy() - float(g['energy'])) <= 1e-13*abs(float(g['energy']))
    s.prepare_scaling(trial, dt)
    for k in ('diagonal', 'block', 'units'):
        assert rel(getattr(s, k), g[f'scaling_{k}']) < 1e-13, k
    assert rel(s.preconditioner, g['scaling_preconditioner']) < 1e-9
    # analytic JVP vs the reference's torch.func.jvp (reference bar 2e-11, scaled norm)
    jv = s.jacobian_vector(y, g['jvp_direction'], dt, ext)
    ref = g['jvp']
    err = np.linalg.norm(s.scale_residual(jv - ref))/np.linalg.norm(s.scale_residual(ref))
    assert err < 2e-11
    assert rel(s.stiffness(g['q']), g['stiffness_q']) < 1e-13
    s.inner_iterations = 0
    x = s.elastic_precondition(g['vector'], dt)
    assert rel(x, g['elastic_precondition']) < 1e-8
    assert s.inner_iterations == int(g['elastic_inner_iterations'])


@pytest.mark.parametrize('case', ['newton_prestressed', 'newton_unstressed'])
@pytest.mark.parametrize('tag,backend,pc', [('fgmres_elastic', 'fgmres', 'elastic'),
                                            ('fgmres_block', 'fgmres', 'block'),
                                            ('dense', 'dense', 'elastic')])
def test_full_step(case, tag, backend, pc):
    g = golden(case)
    s = oracle_newton(g)
    work, info = s.step(float(g['dt']), g['step_load'], tolerance=2e-7, backend=backend,
                        preconditioning=pc, linear_tolerance=1e-7)
    assert info['nonlinear_iterations'] == int(g[f'step_{tag}_nonlinear_iterations'])
    assert info['krylov_iterations'] == int(g[f'step_{tag}_krylov_iterations'])
    assert info['cg_iterations'] == int(g[f'step_{tag}_cg_iterations'])
    # the reference's own cross-solver bars (bonded_dem_newton_checks.py:130-132)
    assert np.abs(s.x - g[f'step_{tag}_state_x']).max() < 1e-9
    assert np.abs(s.rotation - g[f'step_{tag}_state_rotation']).max() < 1e-8
    assert abs(work - float(g[f'step_{tag}_work'])) <= 1e-9*abs(float(g[f'step_{tag}_work']))


def test_linear_217_against_dense_k():
    g = golden('linear_217')
    p, pairs = g['points'], g['pairs']
    s = dem.LinearBonds(p, g['radii'], pairs, g['areas'], g['contacts'], np.ones(len(p)),
                        np.zeros(len(p), bool))
    q = g['q']
    assert rel(s.stiffness(q), g['stiffness_q']) < 1e-13
    assert rel(s.stiffness(q).ravel(), g['dense_k']@q.ravel()) < 1e-12
    assert np.abs(s.diagonal - g['diagonal']).max() < 1e-12
    k = dem.reference_stiffness(p, pairs, g['contacts'], s.kn, s.ks, s.kb, s.kt)
    assert np.abs(k - g['dense_k']).max() < 1e-10


def test_linear_step_217_matches_reference_and_dense_solve():
    """The oracle's linear implicit-midpoint step against the reference's own
    step and the dense solve of ``bonded_dem_linear_gpu.checks`` (1e-6 bar)."""
    g = golden('linear_step_217')
    p = g['points']
    s = dem.LinearBonds(p, g['radii'], g['pairs'], g['areas'], g['contacts'], np.ones(len(p)), g['fixed'])
    work, metrics = s.step(float(g['dt']), g['force'])
    assert rel(s.q, g['step_q']) < 1e-12
    assert rel(s.q, g['dense_q']) < 1e-6
    assert abs(work - float(g['step_work'])) <= 1e-12*abs(float(g['step_work']))
    assert abs(s.energy() - work)/work < 1e-6
    assert metrics['iterations'] == int(g['step_iterations'])


def test_tangent_81():
    g = golden('tangent_81')
    s = dem.LinearBonds(g['points'], np.ones(50), g['pairs'], np.ones(len(g['pairs'])), g['contacts'],
                        np.ones(50), np.zeros(50, bool))
    assert rel(s.stiffness(g['q']), g['stiffness_q']) < 1e-13
    assert rel(s.diagonal, g['diagonal']) < 1e-13


def test_finite_history_953():
    g = golden('finite_953')
    s = dem.FiniteBonds(g['points'], g['radii'], g['pairs'], g['areas'], np.ones(8), np.zeros(8, bool))
    for end, v, w in zip(g['ends'], g['vs'], g['ws']):
        s.commit(s.trial(np.c_[v, w]*.01, end_positions=end))
    for k in ('fn', 'fs', 'mt', 'mb'):
        assert rel(getattr(s, k), g[f'fin_{k}']) < 1e-12
        assert rel(getattr(s, k), g[f'cpu_{k}']) < 1e-12
    loads = s.loads()
    assert rel(loads, g['fin_loads']) < 1e-12
    assert np.linalg.norm(loads[:, :3] - g['cpu_force']) + np.linalg.norm(loads[:, 3:] - g['cpu_torque']) < 1e-10


def test_fgmres_381():
    g = golden('fgmres_381')
    a, b = g['a'], g['b']
    calls = [0]

    def variable_precondition(v):
        calls[0] += 1
        return v/(np.diag(a)*(1+.08*np.sin(calls[0])))
    x, info = dem.fgmres(lambda z: a@z, b, variable_precondition, tolerance=1e-10, restart=24)
    assert info['iterations'] == int(g['iterations'])
    assert rel(x, g['x']) < 1e-12
    assert rel(x, np.linalg.solve(a, b)) < 1e-9


def test_lattice8_three_steps():
    g = golden('lattice8')
    s = dem.NewtonBonds(g['points'], g['radii'], g['pairs'], g['areas'], g['masses'], g['fixed'],
                        young=float(g['young']), shear=float(g['shear']))
    infos = []
    for step in range(3):
        work, info = s.step(float(g['dt']), g['load'], tolerance=1e-6)
        infos.append([info['nonlinear_iterations'], info['krylov_iterations'], info['cg_iterations']])
        assert abs(work - float(g[f'work_{step}'])) <= 1e-9*abs(float(g[f'work_{step}']))
    assert np.array_equal(np.array(infos), g['iterations'])
    for k in STATE:
        assert np.abs(getattr(s, k) - g[f'state_{k}']).max() <= 1e-9*max(1., np.abs(g[f'state_{k}']).max()), k


def test_transport_guard_and_transactional_trial():
    g = golden('newton_prestressed')
    s = oracle_newton(g)
    before = {k: getattr(s, k).copy() for k in STATE}
    with pytest.raises(RuntimeError, match='Subdivide:'):
        s.trial(np.ones_like(s.mass))
    assert all(np.array_equal(getattr(s, k), v) for k, v in before.items())


@pytest.mark.parametrize('case', ['newton_prestressed', 'newton_unstressed'])
def test_previous_solver_step(case):
    """FiniteBondsGPU.step (Anderson + merit backtracking) restated."""
    g = golden(case)
    s = dem.FiniteBonds(**newton_inputs(g))
    for k in STATE:
        setattr(s, k, np.array(g['state_' + k]))
    work, info = s.step(float(g['dt']), g['step_load'], tolerance=2e-7)
    assert info['nonlinear_iterations'] == int(g['step_previous_nonlinear_iterations'])
    assert info['cg_iterations'] == int(g['step_previous_cg_iterations'])
    assert np.abs(s.x - g['step_previous_state_x']).max() < 1e-9
    assert abs(work - float(g['step_previous_work'])) <= 1e-9*abs(float(g['step_previous_work']))


@pytest.mark.parametrize('name', ['energy_fixture', 'energy_foam5'])
def test_energy_law_matches_reference(name):
    """EnergyFoam (volume=False, small kinematics) energy, force and torque."""
    from oracle import dem
    g = golden(name)
    inputs = {k[3:]: g[k] for k in g if k.startswith('in_')}
    model = dem.EnergyBonds(inputs['points'], inputs['radii'], inputs['pairs'], inputs['areas'], inputs['contacts'],
                            inputs['masses'], inputs['fixed'], float(g['young']), float(g['shear']))
    e = model.energy(g['theta'], g['x'], g['q'])
    f, tau = model.forces(g['theta'], g['x'], g['q'])
    assert abs(e - float(g['energy'])) <= 1e-13*abs(float(g['energy']))
    assert np.abs(f - g['force']).max() <= 1e-12*np.abs(g['force']).max()
    assert np.abs(tau - g['torque']).max() <= 1e-12*np.abs(g['torque']).max()


def test_parallel_bonds_with_failure_match_reference():
    """bonded_dem_core.ParallelBonds history with tensile and shear failure."""
    from oracle import dem
    g = golden('parallel_512')
    b = dem.ParallelBonds(g['points'], g['pairs'], g['radii'], float(g['bond_radius']), g['kbar_n'], g['kbar_s'],
                          g['tensile'], g['cohesion'], float(g['friction_angle']), float(g['moment_factor']))
    for k, (end, v, w) in enumerate(zip(g['ends'], g['vs'], g['ws'])):
        info = b.advance(end, v, w, float(g['dt']))
        nb, e, removed = g['steps'][k]
        assert info['newly_broken'] == int(nb)
        assert abs(info['energy'] - e) <= 1e-10*max(abs(e), 1e-30)
        assert abs(info['removed_bond_energy'] - removed) <= 1e-10*max(abs(removed), 1e-30)
    assert np.array_equal(b.failure, g['failure'])
    for k in ('fn', 'fs', 'mt', 'mb', 'break_energy', 'normal'):
        assert np.abs(getattr(b, k) - g[k]).max() <= 1e-10*max(np.abs(g[k]).max(), 1e-30), k
    assert abs(b.work - float(g['work'])) <= 1e-10*abs(float(g['work']))
    f, t = b.loads()
    assert np.abs(f - g['force']).max() <= 1e-10*np.abs(g['force']).max()
    assert np.abs(t - g['torque']).max() <= 1e-10*np.abs(g['torque']).max()


def test_static_equilibrium_matches_reference():
    """reference_stiffness + solve_prescribed on the reference's jittered specimen."""
    from oracle import dem
    g = golden('static_specimen')
    b = dem.ParallelBonds(g['points'], g['pairs'], g['radii'], g['bond_radius'], g['kbar_n'], g['kbar_s'])
    _, contacts = b.geometry(b.x)
    k = dem.reference_stiffness(g['points'], g['pairs'], contacts, b.kn, b.ks, b.kb, b.kt)
    assert np.abs(k - g['dense_k']).max() <= 1e-12*np.abs(g['dense_k']).max()
    q, residual = dem.solve_prescribed(k, g['prescribed'], g['values'], g['load'])
    assert np.abs(q.reshape(-1, 6) - g['q']).max() <= 1e-9*np.abs(g['q']).max()
    assert residual < 1e-8


def _platen_foam(m, seed=0):
    """A jittered m^3 foam with its bottom lattice layer held and its top layer
    pushed down by 5% of its height (the static configuration's boundary
    conditions on whole sites: a clamped platen)."""
    import dpf_gb300
    foam = dpf_gb300.jittered_lattice_foam(m, seed=seed)
    unit, h = foam['unit'], 1./m
    bottom, top = unit[:, 2] < h, unit[:, 2] > 1 - h
    n = len(unit)
    prescribed = np.zeros((n, 3))
    prescribed[top, 2] = -.05*foam['points'][top, 2]
    contacts = dpf_gb300.newton.classical_contacts(foam['points'], foam['radii'], foam['pairs'])
    return foam, contacts, bottom | top, prescribed


def test_energy_newton_linear_limit_matches_reference_stiffness():
    """For a vanishing platen displacement the minimiser of the bond potential
    is the linear static solution of the reference stiffness (the reference
    Hessian of the potential, foam_dem_energy.py:14-16, assembled as in
    bonded_dem_dynamics.py:22-47)."""
    foam, contacts, fixed, prescribed = _platen_foam(5)
    b = dem.EnergyBonds(foam['points'], foam['radii'], foam['pairs'], foam['areas'], contacts, foam['masses'],
                        fixed, foam['young'], foam['shear'])
    n = len(foam['points'])
    eps = 1e-6
    q0 = np.zeros((n, 4))
    q0[:, 0] = 1
    u, t, info = dem.energy_newton(b, np.zeros((n, 4)), foam['points'], q0, np.zeros((n, 6)), fixed,
                                   eps*prescribed, tolerance=1e-12)
    assert info['relative_gradient'] <= 1e-12
    k = dem.reference_stiffness(foam['points'], foam['pairs'], contacts, b.base[:, 0], b.base[:, 1], b.base[:, 2],
                                b.base[:, 3])
    mask = np.repeat(fixed, 6)
    values = np.zeros((n, 6))
    values[:, :3] = eps*prescribed
    q, _ = dem.solve_prescribed(k, mask, values)
    q = q.reshape(n, 6)
    assert np.linalg.norm(np.c_[u, t] - q)/np.linalg.norm(q) < 1e-5


def test_energy_newton_minimises_the_potential():
    """The oracle's static minimiser: relative gradient below the tolerance, and
    the potential grows along random admissible perturbations."""
    foam, contacts, fixed, prescribed = _platen_foam(6, seed=1)
    b = dem.EnergyBonds(foam['points'], foam['radii'], foam['pairs'], foam['areas'], contacts, foam['masses'],
                        fixed, foam['young'], foam['shear'])
    n = len(foam['points'])
    q0 = np.zeros((n, 4))
    q0[:, 0] = 1
    theta = np.zeros((n, 4))
    u, t, info = dem.energy_newton(b, theta, foam['points'], q0, np.zeros((n, 6)), fixed, prescribed,
                                   tolerance=1e-11)
    assert info['relative_gradient'] <= 1e-11

    def energy(du, dt):
        q = dem.quaternion_product(dem.rotation_quaternion(t + dt), q0)
        return b.energy(theta, foam['points'] + u + du, q)
    e0 = energy(0., 0.)
    rng = np.random.default_rng(3)
    for _ in range(3):
        d = rng.normal(size=(n, 6))*1e-4
        d[fixed] = 0
        assert energy(d[:, :3], d[:, 3:]) > e0
