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
