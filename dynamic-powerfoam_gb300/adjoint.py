"""Differentiable rollouts of the rate-law implicit step (drop-in for
``DifferentiableBonds``, ``experiments/bonded_dem_differentiable.py:41-152``).

The reference differentiates one step with dense ``torch.autograd``
Jacobians (limited to 240 free DOFs).  Here the forward step is the CUDA
``NewtonBonds`` solve and the backward pass is a hand-written adjoint:

* the implicit-function theorem gives the increment's adjoint from one
  transposed solve ``J^T lam = y_bar`` (FGMRES on the block-scaled system with
  the transposed elastic preconditioner, ``J^T`` applied through stored
  per-bond 9 x 12 local Jacobians of the float64 trial);
* every input adjoint (committed history, per-bond stiffness, initial
  positions, loads, velocities) comes from per-bond vector-Jacobian products
  of the trial, evaluated with forward-mode dual numbers on the device and
  summed per site in the incidence order (deterministic);
* states are checkpointed every ``checkpoint_every`` steps together with the
  accepted increments; the backward pass replays each segment's commits from
  its checkpoint (one trial per step, no Newton solve) instead of keeping
  every state.
"""
import ctypes

import numpy as np
import torch

from . import _lib
from .newton import F64, NewtonBonds, _Krylov, _addr, fgmres

STATE_NAMES = ('x', 'v', 'rotation', 'normal', 'offset', 'fn', 'fs', 'mt', 'mb')
STIFFNESS_NAMES = ('kn', 'ks', 'kb', 'kt')
HISTORY_NAMES = ('normal', 'offset', 'fn', 'fs', 'mt', 'mb')


def exp_rotation(w):
    """Rotation matrices exp([w]x) (``bonded_dem_finite_gpu.py:35-43``), in torch
    for the rotation adjoint."""
    angle = torch.linalg.vector_norm(w, dim=1)
    s = torch.zeros((len(w), 3, 3), dtype=w.dtype, device=w.device)
    s[:, 0, 1], s[:, 0, 2] = -w[:, 2], w[:, 1]
    s[:, 1, 0], s[:, 1, 2] = w[:, 2], -w[:, 0]
    s[:, 2, 0], s[:, 2, 1] = -w[:, 1], w[:, 0]
    return (torch.eye(3, dtype=w.dtype, device=w.device)
            + torch.sinc(angle/np.pi)[:, None, None]*s
            + (.5*torch.sinc(angle/(2*np.pi))**2)[:, None, None]*(s@s))


def _pack_history(normal, offset, fn, fs, mt, mb):
    return torch.cat((normal, offset, fn[:, None], fs, mt[:, None], mb), dim=1).contiguous()


def _unpack_history(h):
    return h[:, 0:3], h[:, 3:6], h[:, 6], h[:, 7:10], h[:, 10], h[:, 11:14]


class _RecordingNewton(NewtonBonds):
    """NewtonBonds that keeps the accepted increment of its last step."""

    accepted_increment = None

    def _accept(self, y, dt):
        self.accepted_increment = y.clone()
        super()._accept(y, dt)


class _Rollout(torch.autograd.Function):
    """positions (T+1, N, 3) and the final state of T implicit steps as a
    function of per-bond stiffness (M, 4), loads (T, N, 6) and the initial state."""

    @staticmethod
    def forward(ctx, model, dt, stiffness, loads, *state):
        positions, final, checkpoints, increments = model._run(stiffness.detach(), loads.detach(),
                                                               tuple(t.detach() for t in state), dt)
        ctx.model, ctx.dt = model, dt
        ctx.stiffness = stiffness.detach()
        ctx.checkpoints, ctx.increments = checkpoints, increments
        return (positions, *final)

    @staticmethod
    def backward(ctx, g_positions, *g_final):
        grads = ctx.model._adjoint(ctx.stiffness, ctx.checkpoints, ctx.increments, ctx.dt, g_positions, g_final)
        ctx.checkpoints = ctx.increments = None
        return (None, None, *grads)


class DifferentiableBonds:
    """Differentiable implicit rollouts on the CUDA solver.

    Constructor arguments are those of ``FiniteBonds`` (``points, radii,
    pairs, areas, masses, fixed, contacts, young, shear, device``).
    ``parameters`` are per-cell log stiffness multipliers (N, 4): bond b
    scales its base (kn, ks, kb, kt) by ``exp((theta_i + theta_j)/2)``
    (``bonded_dem_differentiable.py:67-78``).  ``rollout_bonds`` takes
    per-bond stiffness and the initial state directly.
    """

    def __init__(self, volume_term=None, *, tolerance=1e-10, pose_tolerance=1e-9, checkpoint_every=8,
                 adjoint_tolerance=1e-10, max_iterations=16, **kwargs):
        if volume_term is not None:
            raise NotImplementedError('volume terms are not part of the CUDA adjoint')
        if checkpoint_every < 1:
            raise ValueError('checkpoint_every must be positive')
        self.solver = _RecordingNewton(**kwargs)
        s = self.solver
        self.base_stiffness = torch.stack([getattr(s, k) for k in STIFFNESS_NAMES], dim=1).clone()
        self.tolerance, self.pose_tolerance = tolerance, pose_tolerance
        self.max_iterations = max_iterations
        self.checkpoint_every = checkpoint_every
        self.adjoint_tolerance = adjoint_tolerance
        self._initial = tuple(getattr(s, k).clone() for k in STATE_NAMES)
        self._lib = _lib.load()
        self.stats = []

    @property
    def device(self):
        return self.solver.device

    # ---- reference interface ------------------------------------------------
    def initial_state(self):
        return tuple(t.clone() for t in self._initial)

    def stiffness(self, parameters):
        """Per-bond (M, 4) stiffness of per-cell log multipliers."""
        s = self.solver
        if parameters.shape != (s.n_sites, 4):
            raise ValueError('Expected 4 log multipliers per cell.')
        return self.base_stiffness*torch.exp(.5*(parameters[s.i] + parameters[s.j]))

    def step(self, state, parameters, external, dt):
        """One differentiable implicit step (``bonded_dem_differentiable.py:139-144``)."""
        positions, *final = self.rollout_bonds(self.stiffness(parameters), external[None], state, dt)
        return (positions[1], *final)

    def rollout(self, parameters, loads, dt):
        """``bonded_dem_differentiable.py:146-152``: (positions (T+1, N, 3), final state)."""
        loads = torch.stack(list(loads)) if not torch.is_tensor(loads) else loads
        positions, *final = self.rollout_bonds(self.stiffness(parameters), loads, self.initial_state(), dt)
        return positions, (positions[-1], *final)

    def rollout_bonds(self, stiffness, loads, state, dt):
        """Differentiable in per-bond stiffness (M, 4), loads (T, N, 6) and every
        entry of ``state`` (x, v, rotation, normal, offset, fn, fs, mt, mb).
        Returns positions (T+1, N, 3) and the final (v, rotation, normal,
        offset, fn, fs, mt, mb)."""
        dt = float(dt)
        if not np.isfinite(dt) or dt <= 0:
            raise ValueError('Positive finite dt required')
        loads = loads.to(device=self.device, dtype=F64)
        if loads.dim() != 3 or loads.shape[1:] != (self.solver.n_sites, 6):
            raise ValueError('loads must be (steps, n_sites, 6)')
        stiffness = stiffness.to(device=self.device, dtype=F64)
        state = tuple(t.to(device=self.device, dtype=F64) for t in state)
        return _Rollout.apply(self, dt, stiffness, loads, *state)

    # ---- forward -------------------------------------------------------------
    def _set(self, stiffness, state):
        s = self.solver
        for k, column in zip(STIFFNESS_NAMES, stiffness.T):
            setattr(s, k, column.contiguous())
        for k, value in zip(STATE_NAMES, state):
            setattr(s, k, value.contiguous())

    def _state(self):
        return tuple(getattr(self.solver, k) for k in STATE_NAMES)

    @torch.no_grad()
    def _run(self, stiffness, loads, state, dt):
        s = self.solver
        self._set(stiffness, state)
        positions, increments, checkpoints = [s.x], [], {}
        for t in range(len(loads)):
            if t % self.checkpoint_every == 0:
                checkpoints[t] = self._state()
            _, info = s.step(dt, loads[t], tolerance=self.tolerance, pose_tolerance=self.pose_tolerance,
                             max_iterations=self.max_iterations)
            self.stats.append(dict(iterations=info['nonlinear_iterations'],
                                   relative_residual=info['nonlinear_relative_residual']))
            increments.append(s.accepted_increment)
            positions.append(s.x)
        final = self._state()[1:]
        return torch.stack(positions), tuple(t.clone() for t in final), checkpoints, increments

    @torch.no_grad()
    def _replay(self, state, increments, dt):
        """States reached from ``state`` by committing the stored increments."""
        s = self.solver
        out = [state]
        for y in increments[:-1]:
            self._set_history(state)
            trial = s.trial(y)
            # the forward's own accept kernel: replayed states are bit-identical
            v, rotation = state[1].clone(), state[2].contiguous().clone()
            _lib.check(self._lib.dpf_accept_step(s.n_sites, y.data_ptr(), dt, v.data_ptr(), rotation.data_ptr(),
                                                 s._stream()), 'dpf_accept_step')
            state = (trial['x'], v, rotation, trial['normal'], trial['offset'], trial['fn'], trial['fs'],
                     trial['mt'], trial['mb'])
            out.append(state)
        return out

    def _set_history(self, state):
        s = self.solver
        for k, value in zip(STATE_NAMES, state):
            setattr(s, k, value.contiguous())

    # ---- backward ------------------------------------------------------------
    def _vjp(self, y, lam, coef, end_adjoint, with_increment, hist_adj, stiff_adj, y_adj, x_adj, slots):
        s = self.solver
        _lib.check(self._lib.dpf_adjoint_bond_vjp(
            ctypes.byref(s._graph), ctypes.byref(s._stiffness_struct()), ctypes.byref(s._history_struct()),
            y.data_ptr(), _addr(lam), float(coef), _addr(end_adjoint), int(with_increment), hist_adj.data_ptr(),
            stiff_adj.data_ptr(), _addr(y_adj), _addr(x_adj), slots.data_ptr(), s._stream()),
            'dpf_adjoint_bond_vjp')

    @torch.no_grad()
    def _adjoint(self, stiffness, checkpoints, increments, dt, g_positions, g_final):
        s = self.solver
        lib = self._lib
        n, m, steps = s.n_sites, s.n_bonds, len(increments)
        stream = s._stream()
        self._set(stiffness, checkpoints[0])
        zeros = lambda *shape: torch.zeros(shape, dtype=F64, device=self.device)
        g_v, g_rotation, *g_history = (g if g is not None else None for g in g_final)
        dense = lambda g: g.to(F64).contiguous().clone()
        x_bar = dense(g_positions[steps])
        v_bar = dense(g_v) if g_v is not None else zeros(n, 6)
        r_bar = dense(g_rotation) if g_rotation is not None else zeros(n, 3, 3)
        h_bar = _pack_history(*(g.to(F64) if g is not None else zeros(*shape) for g, shape in
                                zip(g_history, ((m, 3), (m, 3), (m,), (m, 3), (m,), (m, 3)))))
        stiff_bar = zeros(m, 4)
        load_bar = zeros(steps, n, 6)
        slots = torch.empty(max(1, lib.dpf_adjoint_slot_doubles(m)), dtype=F64, device=self.device)
        jac = torch.empty(max(1, lib.dpf_adjoint_jacobian_doubles(m)), dtype=F64, device=self.device)
        jt_out = torch.empty((n, 6), dtype=F64, device=self.device)
        identity = torch.eye(6, dtype=F64, device=self.device).expand(n, 6, 6).contiguous()
        ones = torch.ones((n, 6), dtype=F64, device=self.device)
        krylov = _Krylov(6*n, 32, self.device)
        half = .5*dt*dt
        free = (~s.fixed)[:, None].to(F64)
        starts = sorted(checkpoints)
        for c, start in reversed(list(enumerate(starts))):
            stop = starts[c+1] if c+1 < len(starts) else steps
            states = self._replay(checkpoints[start], increments[start:stop], dt)
            for t in reversed(range(start, stop)):
                state, y = states[t-start], increments[t]
                self._set_history(state)
                # (1) the commit map: x' = x + u, v' = 2y/dt - v, R' = exp(w) R, history' = trial end
                y_bar = torch.zeros_like(y)
                y_bar[:, :3] += x_bar
                y_bar += (2/dt)*v_bar
                if bool(torch.any(r_bar != 0)):
                    with torch.enable_grad():
                        w = y[:, 3:].clone().requires_grad_(True)
                        exp_w = exp_rotation(w)
                        w_bar, = torch.autograd.grad(exp_w@state[2], (w,), r_bar)
                    y_bar[:, 3:] += w_bar
                    r_bar = exp_w.detach().transpose(1, 2)@r_bar
                x_next, v_next = x_bar.clone(), -v_bar
                h_next = torch.zeros_like(h_bar)
                self._vjp(y, None, 0., h_bar, True, h_next, stiff_bar, y_bar, x_next, slots)
                y_bar *= free
                # (2) the implicit solve: J^T lam = y_bar on the block-scaled system
                trial = s.trial(y)
                s.prepare_scaling(trial, dt)
                lam = self._transposed_solve(y, y_bar, dt, jac, jt_out, slots, identity, ones, krylov)
                load_bar[t] = half*lam
                v_next += dt*s.mass*lam
                # (3) the residual's direct dependence on history, stiffness and positions
                self._vjp(y, lam, half, None, False, h_next, stiff_bar, None, x_next, slots)
                x_bar, v_bar, h_bar = x_next, v_next, h_next
                x_bar += g_positions[t]
        self._set(stiffness, checkpoints[0])
        normal, offset, fn, fs, mt, mb = (t.contiguous() for t in _unpack_history(h_bar))
        return stiff_bar, load_bar, x_bar, v_bar, r_bar, normal, offset, fn, fs, mt, mb

    def _transposed_solve(self, y, rhs, dt, jac, jt_out, slots, identity, ones, krylov):
        """lam with J^T lam = rhs (fixed rows zero), solved as (U^-1 P J U)^T mu = U rhs."""
        s = self.solver
        lib = self._lib
        stream = s._stream()
        _lib.check(lib.dpf_adjoint_local_jacobian(ctypes.byref(s._graph), ctypes.byref(s._stiffness_struct()),
                                                  ctypes.byref(s._history_struct()), y.data_ptr(), jac.data_ptr(),
                                                  stream), 'dpf_adjoint_local_jacobian')
        units, P, block = s.units, s.preconditioner, s.block

        def to_lambda(mu):
            return torch.einsum('nij,nj->ni', P, mu/units).contiguous()

        def operator(mu):
            lam = to_lambda(mu)
            _lib.check(lib.dpf_adjoint_apply_jt(ctypes.byref(s._graph), jac.data_ptr(), s.mass.data_ptr(),
                                                s.fixed.data_ptr(), float(dt), lam.data_ptr(), jt_out.data_ptr(),
                                                slots.data_ptr(), stream), 'dpf_adjoint_apply_jt')
            return units*jt_out

        if s._pcg_workspace is None:
            s._pcg_workspace = torch.empty(lib.dpf_elastic_workspace_doubles(s.n_sites), dtype=F64,
                                           device=self.device)

        def precondition(v):
            r = (v/units).contiguous()
            x = torch.empty_like(r)
            _lib.check(lib.dpf_elastic_precondition(
                ctypes.byref(s._graph), ctypes.byref(s._stiffness_struct()), ctypes.byref(s._tangent_struct()),
                s.mass.data_ptr(), s.fixed.data_ptr(), identity.data_ptr(), P.data_ptr(), ones.data_ptr(),
                r.data_ptr(), float(dt), .03, 80, x.data_ptr(), s._inner.data_ptr(), s._wrench.data_ptr(),
                s._pcg_workspace.data_ptr(), s._barrier.data_ptr(), s._status.data_ptr(), stream),
                'dpf_elastic_precondition')
            return units*torch.einsum('nij,nj->ni', block, x)

        mu, info = fgmres(operator, (units*rhs).contiguous(), precondition, tolerance=self.adjoint_tolerance,
                          workspace=krylov)
        self.stats.append(dict(adjoint_krylov=info['iterations'], adjoint_relative=info['relative_residual']))
        return to_lambda(mu)


def inverse_fit_problem(m, seed, device, steps, dt, checkpoint_every, tolerance):
    """The differentiable inverse material fit: an m^3 jittered foam with its
    bottom layer fixed, under gravity and a 3% top indentation (equivalent load
    E * 0.03 * top area spread over the top layer's sites), a hidden per-bond log-stiffness field (smooth Gaussian random
    field by 512 random Fourier features of the bond midpoints: squared-
    exponential covariance, length scale 0.2, mean log(1e5), std 0.5), and the
    MSE of all site positions of a ``steps``-step trajectory against the
    trajectory of the hidden field.  Returns (model, uniform initial guess
    theta0 (M,), loss(theta)) with theta the per-bond log stiffness."""
    from .foam import gravity_load, jittered_lattice_foam
    # bottom lattice layer fixed, top layer loaded (jitter is +-0.2 spacing)
    foam = jittered_lattice_foam(m, seed=seed, young=1.0, poisson=.3, fixed_below=1./m)
    model = DifferentiableBonds(points=foam['points'], radii=foam['radii'], pairs=foam['pairs'],
                                          areas=foam['areas'], masses=foam['masses'], fixed=foam['fixed'],
                                          young=1.0, shear=1/2.6, device=device, checkpoint_every=checkpoint_every,
                                          tolerance=tolerance, pose_tolerance=max(tolerance, 1e-12),
                                          adjoint_tolerance=1e-11, max_iterations=24)
    rng = np.random.default_rng(seed + 1)
    pairs = np.asarray(foam['pairs'])
    mid = .5*(foam['unit'][pairs[:, 0]] + foam['unit'][pairs[:, 1]])
    k = 512
    omega = rng.normal(0., 1/.2, (k, 3))
    phase = rng.uniform(0., 2*np.pi, k)
    field = np.sqrt(2./k)*np.cos(mid@omega.T + phase).sum(1)
    hidden = np.log(1e5) + .5*field
    load = gravity_load(foam)
    top = (foam['unit'][:, 2] > 1. - 1./m) & ~np.asarray(foam['fixed'])
    load[top, 2] -= 1e5*.03*1.0/max(1, top.sum())
    t = lambda a: torch.as_tensor(a, dtype=torch.float64, device=device)
    loads = t(np.repeat(load[None], steps, 0))
    base = model.base_stiffness

    def rollout(theta):
        return model.rollout_bonds(base*torch.exp(theta)[:, None], loads, model.initial_state(), dt)[0]
    with torch.no_grad():
        target = rollout(t(hidden))
    theta0 = t(np.full(len(pairs), np.log(1e5)))

    def loss(theta):
        return ((rollout(theta) - target)**2).mean()
    return model, theta0, loss
