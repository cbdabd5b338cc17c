"""Energy law on the GPU against the reference's EnergyFoam outputs (golden)
and against its own energy by central differences."""
import numpy as np
import pytest

from tests.conftest import golden

pytestmark = pytest.mark.gpu


def _model(g):
    import dpf_gb300
    geometry = {k[3:]: g[k] for k in g if k.startswith('in_')}
    return dpf_gb300.EnergyFoam(geometry, volume=False, device='cuda', young=float(g['young']),
                                shear=float(g['shear']))


@pytest.mark.parametrize('name', ['energy_fixture', 'energy_foam5'])
def test_energy_and_forces_match_reference(name):
    g = golden(name)
    model = _model(g)
    e = float(model.energy(g['theta'], g['x'], g['q']))
    f, tau = model.forces(g['theta'], g['x'], g['q'])
    assert abs(e - float(g['energy'])) <= 1e-12*abs(float(g['energy']))
    assert np.abs(f.cpu().numpy() - g['force']).max() <= 1e-11*np.abs(g['force']).max()
    assert np.abs(tau.cpu().numpy() - g['torque']).max() <= 1e-11*np.abs(g['torque']).max()


def test_forces_are_energy_gradients():
    """-dE/dx and -dE/d(world rotation) by central differences of the GPU energy
    (rotation perturbed as q <- quat(exp(eps w)) q)."""
    g = golden('energy_foam5')
    model = _model(g)
    rng = np.random.default_rng(5)
    theta, x, q = g['theta'], g['x'], g['q']
    f, tau = (t.cpu().numpy() for t in model.forces(theta, x, q))
    dx = rng.normal(size=x.shape)
    h = 1e-6
    fd = (float(model.energy(theta, x + h*dx, q)) - float(model.energy(theta, x - h*dx, q)))/(2*h)
    assert abs(fd + (f*dx).sum()) <= 1e-6*abs(fd)

    def rotate(w):
        # left-multiply each quaternion by the rotation exp(w) (w small)
        ang = np.linalg.norm(w, axis=1, keepdims=True)
        axis = w/np.maximum(ang, 1e-300)
        dq = np.concatenate([np.cos(ang/2), np.sin(ang/2)*axis], 1)
        w0, v0 = dq[:, :1], dq[:, 1:]
        w1, v1 = q[:, :1], q[:, 1:]
        return np.concatenate([w0*w1 - (v0*v1).sum(1, keepdims=True), w0*v1 + w1*v0 + np.cross(v0, v1)], 1)
    dw = rng.normal(size=(len(q), 3))
    fd = (float(model.energy(theta, x, rotate(h*dw))) - float(model.energy(theta, x, rotate(-h*dw))))/(2*h)
    assert abs(fd + (tau*dw).sum()) <= 1e-6*abs(fd)


def test_energy_is_deterministic():
    g = golden('energy_foam5')
    model = _model(g)
    a = model.forces(g['theta'], g['x'], g['q'])
    b = model.forces(g['theta'], g['x'], g['q'])
    assert all(bool((u == v).all()) for u, v in zip(a, b))
    assert float(model.energy(g['theta'], g['x'], g['q'])) == float(model.energy(g['theta'], g['x'], g['q']))


def _platen(m, seed=0):
    """Static configuration: jittered m^3 foam, bottom lattice layer held, top
    layer pushed down by 5% of its height (whole sites held: a clamped platen)."""
    import dpf_gb300
    foam = dpf_gb300.jittered_lattice_foam(m, seed=seed)
    unit, h = foam['unit'], 1./m
    bottom, top = unit[:, 2] < h, unit[:, 2] > 1 - h
    prescribed = np.zeros((len(unit), 3))
    prescribed[top, 2] = -.05*foam['points'][top, 2]
    geometry = dict(points=foam['points'], radii=foam['radii'], pairs=foam['pairs'], areas=foam['areas'],
                    contacts=None, masses=foam['masses'], fixed=bottom | top)
    return foam, geometry, prescribed


def _oracle(foam, geometry, prescribed=None, inertia=None, load=None, tolerance=1e-12):
    from oracle import dem
    import dpf_gb300
    contacts = dpf_gb300.newton.classical_contacts(foam['points'], foam['radii'], foam['pairs'])
    b = dem.EnergyBonds(foam['points'], foam['radii'], foam['pairs'], foam['areas'], contacts, foam['masses'],
                        geometry['fixed'], foam['young'], foam['shear'])
    n = len(foam['points'])
    q0 = np.zeros((n, 4))
    q0[:, 0] = 1
    load = np.zeros((n, 6)) if load is None else load
    return dem.energy_newton(b, np.zeros((n, 4)), foam['points'], q0, load, geometry['fixed'], prescribed, inertia,
                             tolerance=tolerance)


def test_static_platen_16cube_matches_oracle():
    """The static configuration at 16^3 (4,096 sites): the line-searched Newton
    equilibrium of the bond potential on the GPU against the NumPy oracle's
    minimiser, both to a relative gradient of 1e-12: displacements and
    rotations agree to 1e-8."""
    import dpf_gb300
    foam, geometry, prescribed = _platen(16)
    solver = dpf_gb300.EnergyNewton(geometry, young=foam['young'], shear=foam['shear'])
    info = solver.solve(prescribed=prescribed, tolerance=1e-12)
    assert info['relative_gradient'] <= 1e-12
    u_ref, t_ref, ref = _oracle(foam, geometry, prescribed)
    u = (solver.x - solver.X).cpu().numpy()
    assert np.linalg.norm(u - u_ref)/np.linalg.norm(u_ref) < 1e-8
    qw = solver.q.cpu().numpy()
    from oracle import dem
    q_ref = dem.rotation_quaternion(t_ref)
    q_ref *= np.sign(q_ref[:, :1])
    qw *= np.sign(qw[:, :1])
    assert np.linalg.norm(qw - q_ref)/np.linalg.norm(t_ref) < 1e-8
    assert abs(info['energy'] - ref['energy']) <= 1e-10*abs(ref['energy'])


def test_implicit_euler_steps_match_oracle():
    """Implicit-Euler steps of the bond potential under gravity (8^3 foam,
    bottom layer held, dt = 1e-3): two GPU steps against the oracle's
    minimisations of the same incremental potentials."""
    import dpf_gb300
    foam = dpf_gb300.jittered_lattice_foam(8, seed=2)
    unit = foam['unit']
    fixed = unit[:, 2] < 1./8
    geometry = dict(points=foam['points'], radii=foam['radii'], pairs=foam['pairs'], areas=foam['areas'],
                    contacts=None, masses=foam['masses'], fixed=fixed)
    load = dpf_gb300.gravity_load(dict(foam, fixed=fixed))
    load[:, 2] *= 50.            # a visible response within two steps
    solver = dpf_gb300.EnergyNewton(geometry, young=foam['young'], shear=foam['shear'])
    from oracle import dem
    contacts = dpf_gb300.newton.classical_contacts(foam['points'], foam['radii'], foam['pairs'])
    b = dem.EnergyBonds(foam['points'], foam['radii'], foam['pairs'], foam['areas'], contacts, foam['masses'],
                        fixed, foam['young'], foam['shear'])
    n = len(unit)
    x, q = foam['points'].copy(), np.zeros((n, 4))
    q[:, 0] = 1
    v, w = np.zeros((n, 3)), np.zeros((n, 3))
    dt = 1e-3
    for _ in range(2):
        info = solver.step(dt, solver.law._bonds.tensor(load), tolerance=1e-12)
        assert info['relative_gradient'] <= 1e-12
        u, t, _ = dem.energy_newton(b, np.zeros((n, 4)), x, q, load, fixed, None, (dt, v, w), tolerance=1e-12)
        x, q = x + u, dem.quaternion_product(dem.rotation_quaternion(t), q)
        v, w = u/dt, t/dt
    disp = x - foam['points']
    assert np.linalg.norm(solver.x.cpu().numpy() - x)/np.linalg.norm(disp) < 1e-8
    assert np.linalg.norm(solver.v.cpu().numpy() - v)/np.linalg.norm(v) < 1e-8
    assert np.linalg.norm(solver.w.cpu().numpy() - w)/max(np.linalg.norm(w), 1e-30) < 1e-6


def test_energy_newton_at_rest_stays_put():
    import dpf_gb300
    foam, geometry, _ = _platen(6)
    solver = dpf_gb300.EnergyNewton(geometry, young=foam['young'], shear=foam['shear'])
    info = solver.solve(tolerance=1e-10)
    assert info['newton_iterations'] == 0
    assert float((solver.x - solver.X).abs().max()) == 0.
