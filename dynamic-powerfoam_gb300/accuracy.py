"""Accuracy of the mixed-precision and served solves against float64 solves.

Every result of the mixed-precision form (float32 bond sweeps with float64
reductions and residual) and of the served batches is reported against a
float64 ``NewtonBonds`` solve of the same inputs, started from the same
state (``NewtonBonds`` is the drop-in of the reference's
``experiments/bonded_dem_newton.py:132-201`` and is held to the reference's
own outputs by the parity tests):

* force residual: the float64 implicit-midpoint residual of the result's
  increment y = dt (v_before + v_after) / 2 (the commit rule
  ``v_after = 2 y / dt - v_before``), relative to the step's right-hand-side
  scale max(|dt M v + dt^2/2 f_ext|, dt^2/2 |loads on free sites|), exactly
  the quantity the solver's own stopping test bounds;
* displacement: |x - x_64| / |x_64 - x_before| with x_64 the positions of a
  float64 solve of the same step at relative residual 1e-10.
"""
import numpy as np
import torch

from .newton import NewtonBonds

STATE = ('x', 'v', 'rotation', 'normal', 'offset', 'fn', 'fs', 'mt', 'mb')
REFERENCE_TOLERANCE = 1e-10


def snapshot_state(solver):
    """Copies of the committed physical state and the time."""
    return {name: getattr(solver, name).clone() for name in STATE}, solver.time


def restore(solver, state, time_):
    """Set a solver's committed state (copies) and time."""
    for name, value in state.items():
        setattr(solver, name, value.clone())
    solver.time = time_


def float64_check(p64, state, time_, y, dt, external, tolerance=REFERENCE_TOLERANCE):
    """From ``state``: the float64 force residual of the increment ``y``
    (relative to the step's rhs scale) and the positions of the float64 solve
    of the same step at ``tolerance``.  ``p64`` is a float64 solver of the
    same foam; its state is overwritten."""
    restore(p64, state, time_)
    r = p64.residual(y, dt, external)
    a = torch.linalg.vector_norm(dt*p64.mass*state['v'] + .5*dt*dt*external)
    b = .5*dt*dt*torch.linalg.vector_norm(p64.loads()[~p64.fixed])
    scale = max(float(a), float(b), 1e-30)
    residual = float(torch.linalg.vector_norm(r))/scale
    p64.step(dt, external, tolerance=tolerance)
    return residual, p64.x


def _relative(a, b, origin):
    return float(torch.linalg.vector_norm(a - b)/torch.linalg.vector_norm(b - origin))


def trajectory_accuracy(solver, foam, external, dt, tolerance, steps, start, device):
    """``steps`` steps of ``solver`` from ``start`` (a ``snapshot_state``),
    each against a float64 solve of the same state, plus the whole trajectory
    against a float64 trajectory from the same start."""
    args = (foam['points'], foam['radii'], foam['pairs'], foam['areas'], foam['masses'], foam['fixed'])
    kw = dict(young=foam['young'], shear=foam['shear'], device=device)
    p64, trajectory = NewtonBonds(*args, **kw), NewtonBonds(*args, **kw)
    restore(solver, *start)
    restore(trajectory, *start)
    x0 = solver.x.clone()
    displacement, force = [], []
    for _ in range(steps):
        state, time_ = snapshot_state(solver)
        solver.step(dt, external, tolerance=tolerance)
        y = .5*dt*(state['v'] + solver.v)
        residual, x64 = float64_check(p64, state, time_, y, dt, external)
        force.append(residual)
        displacement.append(_relative(solver.x, x64, state['x']))
        trajectory.step(dt, external, tolerance=REFERENCE_TOLERANCE)
    return dict(reference=f'float64 NewtonBonds at tolerance {REFERENCE_TOLERANCE:g} from the same state, '
                          'every step', steps=steps, displacement_rel_max=max(displacement),
                displacement_rel_median=float(np.median(displacement)), force_residual_rel_max=max(force),
                trajectory_displacement_rel=_relative(solver.x, trajectory.x, x0),
                bars=dict(displacement=1e-6, force_residual=1e-6))


def served_accuracy(finished, count, device, seed=7):
    """A seeded sample of ``count`` finished one-step served requests, each
    against a float64 solve of the same request."""
    ok = [r for r in finished if r.error is None and r.steps == 1]
    if not ok or count <= 0:
        return None
    pick = np.random.default_rng(seed).choice(len(ok), min(count, len(ok)), replace=False)
    displacement, force = [], []
    for k in sorted(pick):
        req = ok[k]
        f = req.foam
        p64 = NewtonBonds(f['points'], f['radii'], f['pairs'], f['areas'], f['masses'], f['fixed'],
                          young=f['young'], shear=f['shear'], device=device)
        external = p64.tensor(req.load)
        state, time_ = snapshot_state(p64)
        y = .5*req.dt*(state['v'] + req.state['v'])
        residual, x64 = float64_check(p64, state, time_, y, req.dt, external)
        force.append(residual)
        displacement.append(_relative(req.state['x'], x64, state['x']))
    return dict(requests=len(displacement), reference=f'float64 NewtonBonds at tolerance {REFERENCE_TOLERANCE:g} '
                                                      'of the same request',
                displacement_rel_max=max(displacement), displacement_rel_median=float(np.median(displacement)),
                force_residual_rel_max=max(force), bars=dict(displacement=1e-6, force_residual=1e-6))
