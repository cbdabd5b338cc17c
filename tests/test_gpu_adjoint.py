"""Adjoint rollouts (DifferentiableBonds) against the reference's own
gradients (``experiments/bonded_dem_differentiable.py``, dense autograd
Jacobians) and against central finite differences of the CUDA forward."""
import numpy as np
import pytest

from tests.conftest import golden
from tests.helpers import rel

pytestmark = pytest.mark.gpu


def _golden_model(g, **kw):
    import dpf_gb300
    return dpf_gb300.DifferentiableBonds(points=g['points'], radii=g['radii'], pairs=g['pairs'],
                                         areas=g['areas'], masses=g['masses'], fixed=g['fixed'],
                                         contacts=g['contacts'], device='cuda', **kw)


@pytest.mark.parametrize('every', [1, 2, 3])
def test_rollout_matches_reference_gradients(every):
    import torch
    g = golden('adjoint_unstressed')
    model = _golden_model(g, checkpoint_every=every)
    theta = torch.tensor(g['theta'], device='cuda', requires_grad=True)
    loads = [torch.tensor(l, device='cuda', requires_grad=True) for l in g['loads']]
    positions, state = model.rollout(theta, loads, float(g['dt']))
    loss = (positions*torch.tensor(g['weights'], device='cuda')).sum()
    # forward: the reference solves to a max scaled residual of 1e-11
    assert rel(positions, g['positions']) < 1e-10
    assert rel(positions - positions[0], g['positions'] - g['positions'][0]) < 1e-8
    assert abs(float(loss.detach()) - float(g["loss"])) <= 1e-10*abs(float(g["loss"]))
    grads = torch.autograd.grad(loss, [theta] + loads)
    # gradients: transposed Krylov solve to 1e-10 against the reference's dense solve
    assert rel(grads[0], g['grad_theta']) < 1e-7
    assert rel(torch.stack(grads[1:]), g['grad_loads']) < 1e-7


def _foam(n=4, seed=5):
    import dpf_gb300
    foam = dpf_gb300.jittered_lattice_foam(n, seed=seed)
    keys = ('points', 'radii', 'pairs', 'areas', 'masses', 'fixed', 'contacts', 'young', 'shear')
    return foam, {k: foam[k] for k in keys}


def _loss_parts(model, foam, steps, seed):
    """A loss touching positions, final velocity, rotation and history."""
    import torch
    import dpf_gb300
    s = model.solver
    rng = np.random.default_rng(seed)
    t = lambda a: torch.as_tensor(a, dtype=torch.float64, device='cuda')
    weights = dict(x=t(rng.normal(size=(steps+1, s.n_sites, 3))), v=t(rng.normal(size=(s.n_sites, 6))),
                   rotation=t(rng.normal(size=(s.n_sites, 3, 3))), fn=t(rng.normal(size=s.n_bonds)),
                   fs=t(rng.normal(size=(s.n_bonds, 3))), mb=t(rng.normal(size=(s.n_bonds, 3))))
    load = dpf_gb300.gravity_load(foam)
    loads = np.stack([load*(1 + .5*k) + rng.normal(0, 50, load.shape)*(~np.asarray(foam['fixed']))[:, None]
                      for k in range(steps)])

    def loss(stiffness, loads_t, state, dt):
        positions, v, rotation, normal, offset, fn, fs, mt, mb = model.rollout_bonds(stiffness, loads_t, state, dt)
        return ((positions*weights['x']).sum() + 1e-3*(v*weights['v']).sum()
                + (rotation*weights['rotation']).sum() + 1e-2*(fn*weights['fn']).sum()
                + 1e-2*(fs*weights['fs']).sum() + 1e-2*(mb*weights['mb']).sum())
    return loss, t(loads)


@pytest.mark.parametrize('which', ['stiffness', 'positions', 'loads', 'velocity', 'history'])
def test_directional_derivative_matches_central_differences(which):
    import torch
    import dpf_gb300
    foam, kwargs = _foam()
    steps, dt = 4, 2e-3
    model = dpf_gb300.DifferentiableBonds(**kwargs, device='cuda', checkpoint_every=3)
    s = model.solver
    loss, loads = _loss_parts(model, foam, steps, seed=11)
    state0 = list(model.initial_state())
    # start from a moving, loaded state so every history input matters
    rng = np.random.default_rng(17)
    free = torch.as_tensor(~np.asarray(foam['fixed']), device='cuda')[:, None].double()
    state0[1] = torch.as_tensor(rng.normal(0, .05, (s.n_sites, 6)), device='cuda')*free
    state0[5] = torch.as_tensor(rng.normal(0, 1., s.n_bonds), device='cuda')
    state0[6] = torch.as_tensor(rng.normal(0, .3, (s.n_bonds, 3)), device='cuda')
    stiffness = model.base_stiffness.clone()
    inputs = dict(stiffness=stiffness, loads=loads, x=state0[0], v=state0[1], fn=state0[5], fs=state0[6])
    h = foam['h']
    directions = dict(
        stiffness=dict(stiffness=stiffness*torch.as_tensor(rng.normal(size=stiffness.shape), device='cuda')),
        positions=dict(x=torch.as_tensor(rng.normal(0, 1e-3*h, (s.n_sites, 3)), device='cuda')),
        loads=dict(loads=torch.as_tensor(rng.normal(0, 30., loads.shape), device='cuda')*free),
        velocity=dict(v=torch.as_tensor(rng.normal(0, .01, (s.n_sites, 6)), device='cuda')*free),
        history=dict(fn=torch.as_tensor(rng.normal(0, .5, s.n_bonds), device='cuda'),
                     fs=torch.as_tensor(rng.normal(0, .2, (s.n_bonds, 3)), device='cuda')))[which]

    def evaluate(eps, grad=False):
        vals = {k: (v + eps*directions[k] if k in directions else v).detach().clone().requires_grad_(grad)
                for k, v in inputs.items()}
        state = list(state0)
        state[0], state[1], state[5], state[6] = vals['x'], vals['v'], vals['fn'], vals['fs']
        out = loss(vals['stiffness'], vals['loads'], tuple(state), dt)
        if not grad:
            return float(out)
        grads = torch.autograd.grad(out, [vals[k] for k in directions])
        return sum(float((gk*directions[k]).sum()) for gk, k in zip(grads, directions))

    analytic = evaluate(0., grad=True)
    eps = 1e-4
    numeric = (evaluate(eps) - evaluate(-eps))/(2*eps)
    assert abs(analytic - numeric) <= 1e-5*max(abs(numeric), 1e-12), (analytic, numeric)


def test_checkpointing_is_exact():
    """Replayed segments give bit-identical gradients for every checkpoint spacing."""
    import torch
    import dpf_gb300
    foam, kwargs = _foam(n=4, seed=7)
    steps, dt = 5, 2e-3
    results = []
    for every in (1, 2, 5):
        model = dpf_gb300.DifferentiableBonds(**kwargs, device='cuda', checkpoint_every=every)
        loss, loads = _loss_parts(model, foam, steps, seed=3)
        stiffness = model.base_stiffness.clone().requires_grad_(True)
        state = list(model.initial_state())
        state[0] = state[0].clone().requires_grad_(True)
        loads = loads.clone().requires_grad_(True)
        out = loss(stiffness, loads, tuple(state), dt)
        results.append([t.clone() for t in torch.autograd.grad(out, [stiffness, loads, state[0]])])
    for other in results[1:]:
        for a, b in zip(results[0], other):
            assert torch.equal(a, b)


def test_cell_parameters_chain_to_bond_stiffness():
    """rollout(parameters) = rollout_bonds(stiffness(parameters)) with the
    per-cell chain rule of bonded_dem_differentiable.py:67-78."""
    import torch
    g = golden('adjoint_unstressed')
    model = _golden_model(g)
    theta = torch.tensor(g['theta'], device='cuda', requires_grad=True)
    loads = torch.tensor(g['loads'], device='cuda')
    weights = torch.tensor(g['weights'], device='cuda')
    positions, _ = model.rollout(theta, loads, float(g['dt']))
    grad_theta, = torch.autograd.grad((positions*weights).sum(), [theta])
    stiffness = model.stiffness(theta.detach()).requires_grad_(True)
    positions2, *_ = model.rollout_bonds(stiffness, loads, model.initial_state(), float(g['dt']))
    grad_k, = torch.autograd.grad((positions2*weights).sum(), [stiffness])
    s = model.solver
    per_bond = .5*(grad_k*stiffness.detach())
    manual = torch.zeros_like(theta).index_add_(0, s.i, per_bond).index_add_(0, s.j, per_bond)
    assert torch.allclose(manual, grad_theta, rtol=1e-12, atol=1e-14)


def test_inverse_fit_gradient_matches_central_differences():
    """The inverse material fit workload (per-bond log stiffness, position MSE)
    at 6^3, 12 steps, checkpoints every 5: per-bond gradients of the largest
    entries vs central differences with h = 1e-4 within 1e-4."""
    import torch
    from dpf_gb300.adjoint import inverse_fit_problem
    model, theta0, loss = inverse_fit_problem(6, 4, 'cuda', 12, 2e-3, 5, 1e-12)
    theta = theta0.clone().requires_grad_(True)
    grad, = torch.autograd.grad(loss(theta), [theta])
    bonds = torch.topk(grad.abs(), 4).indices.tolist()
    h = 1e-4
    with torch.no_grad():
        for b in bonds:
            e = torch.zeros_like(theta0)
            e[b] = h
            fd = (float(loss(theta0 + e)) - float(loss(theta0 - e)))/(2*h)
            assert abs(fd - float(grad[b])) <= 1e-4*abs(fd), (b, fd, float(grad[b]))
