"""Parallel-bond component with brittle failure on the GPU: drop-in for
``ParallelBonds`` (``experiments/bonded_dem_core.py:45-208``).

Same constructor arguments, validation, attributes and methods
(``geometry``, ``loads``, ``advance``, ``elastic_energy_per_bond``,
``intact``); the state lives in float64 CUDA tensors.  ``advance`` runs one
bond pass that writes the new history to spare buffers and swaps them in only
when no guard fired, so a rejected step (``ValueError``, as in the
reference) leaves the model unchanged.
"""
import ctypes

import numpy as np
import torch

from . import _lib
from .newton import F64, incidence

_GUARDS = ((_lib.DPF_ERR_ROTATION, 'Body rotation > 0.25 rad per step; subdivide'),
           (_lib.DPF_ERR_NORMAL_TURN, 'Contact normal turns > 0.25 rad per half-step; subdivide'),
           (_lib.DPF_ERR_COINCIDENT, 'Coincident centers are outside this baseline'))
_STATE = ('normal', 'fn', 'fs', 'mt', 'mb', 'break_energy', 'failure')


class ParallelBonds:
    """Stateful bonded interaction; advance exactly once per physical step."""

    def __init__(self, reference, pairs, radii, bond_radius, kbar_n, kbar_s, tensile_strength=np.inf,
                 cohesion=np.inf, friction_angle=0., moment_factor=1., device='cuda'):
        x = np.asarray(reference, dtype=np.float64)
        if x.ndim != 2 or x.shape[1] != 3 or not np.isfinite(x).all():
            raise ValueError('reference must be a finite (N, 3) array')
        raw = np.asarray(pairs)
        if raw.ndim != 2 or raw.shape[1] != 2 or len(raw) == 0 or not np.issubdtype(raw.dtype, np.integer):
            raise ValueError('pairs must be a nonempty integer (M, 2) array')
        pairs = raw.astype(np.int64)
        if np.any(pairs < 0) or np.any(pairs >= len(x)):
            raise ValueError('Invalid endpoint index')
        canonical = np.sort(pairs, axis=1)
        if np.any(canonical[:, 0] == canonical[:, 1]) or len(np.unique(canonical, axis=0)) != len(canonical):
            raise ValueError('Self-bonds and duplicate undirected bonds are invalid')
        radii = np.broadcast_to(np.asarray(radii, dtype=float), (len(x),)).copy()
        if not np.isfinite(radii).all() or np.any(radii <= 0):
            raise ValueError('Particle radii must be positive and finite')
        m = len(pairs)

        def parameter(value, name, allow_inf=False):
            out = np.broadcast_to(np.asarray(value, dtype=float), (m,)).copy()
            valid = ~np.isnan(out) if allow_inf else np.isfinite(out)
            if not valid.all() or np.any(out <= 0):
                raise ValueError(f'{name} must be positive' + (' or +inf' if allow_inf else ' and finite'))
            return out
        rb = parameter(bond_radius, 'bond_radius')
        kbn, kbs = parameter(kbar_n, 'kbar_n'), parameter(kbar_s, 'kbar_s')
        tensile = parameter(tensile_strength, 'tensile_strength', True)
        cohesion_a = parameter(cohesion, 'cohesion', True)
        if not np.isfinite(friction_angle) or not 0 <= friction_angle < np.pi/2:
            raise ValueError('friction_angle must be in [0, pi/2) radians')
        if not np.isfinite(moment_factor) or not 0 <= moment_factor <= 1:
            raise ValueError('moment_factor must be in [0, 1]')
        self.device = torch.device(device)
        if self.device.type != 'cuda':
            raise ValueError('dpf_gb300 solvers run on CUDA devices only')
        self._lib = _lib.load()
        t = lambda a: torch.as_tensor(np.ascontiguousarray(a), dtype=F64, device=self.device)
        self.x = t(x)
        self.pairs = torch.as_tensor(pairs, device=self.device).contiguous()
        self.i, self.j = self.pairs.T
        self.radii = t(radii)
        area = np.pi*rb**2
        second = np.pi*rb**4/4
        polar = 2*second
        self.rb, self.area, self.second_moment, self.polar_moment = t(rb), t(area), t(second), t(polar)
        self.kn, self.ks, self.kb, self.kt = t(kbn*area), t(kbs*area), t(kbn*second), t(kbs*polar)
        self.tensile_strength, self.cohesion = t(tensile), t(cohesion_a)
        self.tan_phi, self.beta = float(np.tan(friction_angle)), float(moment_factor)
        ptr, inc = incidence(pairs, len(x))
        self._inc_ptr = torch.as_tensor(ptr, device=self.device)
        self._inc_bond = torch.as_tensor(inc, device=self.device)
        self._graph = _lib.Graph(len(x), m, self.pairs.data_ptr(), self._inc_ptr.data_ptr(), self._inc_bond.data_ptr())
        self._params = _lib.ParallelParams(*(a.data_ptr() for a in (
            self.kn, self.ks, self.kb, self.kt, self.area, self.second_moment, self.polar_moment, self.rb,
            self.tensile_strength, self.cohesion)), self.tan_phi, self.beta)
        self.normal, _ = self.geometry(self.x)
        self.reference_length = torch.linalg.vector_norm(self.x[self.j] - self.x[self.i], dim=1)
        z = lambda *shape: torch.zeros(shape, dtype=F64, device=self.device)
        self.fn, self.mt, self.fs, self.mb = z(m), z(m), z(m, 3), z(m, 3)
        self.failure = torch.zeros(m, dtype=torch.int8, device=self.device)
        self.break_energy = z(m)
        self._spare = {k: torch.empty_like(getattr(self, k)) for k in _STATE}
        self._sums = z(4)
        self._partials = z(self._lib.dpf_parallel_partials_doubles())
        self._wrench = z(9*m)
        self._status = torch.zeros(1, dtype=torch.int32, device=self.device)
        self.work, self.time = 0., 0.

    @property
    def intact(self):
        return self.failure == 0

    def _stream(self):
        return torch.cuda.current_stream(self.device).cuda_stream

    def _vec(self, a, name):
        out = torch.as_tensor(a, dtype=F64, device=self.device).contiguous()
        if out.shape != self.x.shape or not bool(torch.isfinite(out).all()):
            raise ValueError(f'{name} must be finite with shape {tuple(self.x.shape)}')
        return out

    def geometry(self, x):
        """Classical ball-ball contact point (bonded_dem_core.py:117-126)."""
        x = torch.as_tensor(x, dtype=F64, device=self.device)
        d = x[self.j] - x[self.i]
        length = torch.linalg.vector_norm(d, dim=1)
        if bool(torch.any(length <= 1e-12)):
            raise ValueError('Coincident centers are outside this baseline')
        n = d/length[:, None]
        return n, .5*(x[self.i] + x[self.j]) + .5*(self.radii[self.i] - self.radii[self.j])[:, None]*n

    def elastic_energy_per_bond(self):
        return .5*(self.fn**2/self.kn + (self.fs*self.fs).sum(1)/self.ks + self.mt**2/self.kt
                   + (self.mb*self.mb).sum(1)/self.kb)

    def _struct(self, d):
        return _lib.ParallelState(*(d[k].data_ptr() for k in _STATE))

    @torch.no_grad()
    def loads(self):
        """Forces and torques about the centres (bonded_dem_core.py:132-142)."""
        n = len(self.x)
        force = torch.empty((n, 3), dtype=F64, device=self.device)
        torque = torch.empty_like(force)
        self._status.zero_()
        _lib.check(self._lib.dpf_parallel_loads(
            ctypes.byref(self._graph), self.radii.data_ptr(), self.x.data_ptr(), self.fn.data_ptr(),
            self.fs.data_ptr(), self.mt.data_ptr(), self.mb.data_ptr(), force.data_ptr(), torque.data_ptr(),
            self._wrench.data_ptr(), self._status.data_ptr(), self._stream()), 'dpf_parallel_loads')
        if int(self._status.item()):
            raise ValueError('Coincident centers are outside this baseline')
        return force, torque

    @torch.no_grad()
    def advance(self, x_next, velocity_mid, omega_mid, dt, *, x_mid=None):
        """One step of the bond history from midpoint samples (bonded_dem_core.py:144-208)."""
        if not np.isfinite(dt) or dt <= 0:
            raise ValueError('dt must be positive and finite')
        end = self._vec(x_next, 'x_next')
        mid = None if x_mid is None else self._vec(x_mid, 'x_mid')
        v = self._vec(velocity_mid, 'velocity_mid')
        w = self._vec(omega_mid, 'omega_mid')
        current = {k: getattr(self, k) for k in _STATE}
        self._status.zero_()
        _lib.check(self._lib.dpf_parallel_advance(
            ctypes.byref(self._graph), ctypes.byref(self._params), self.radii.data_ptr(), self.x.data_ptr(),
            end.data_ptr(), None if mid is None else mid.data_ptr(), v.data_ptr(), w.data_ptr(), float(dt),
            ctypes.byref(self._struct(current)), ctypes.byref(self._struct(self._spare)), self._sums.data_ptr(),
            self._partials.data_ptr(), self._status.data_ptr(), self._stream()), 'dpf_parallel_advance')
        status = int(self._status.item())
        for bit, message in _GUARDS:
            if status & bit:
                raise ValueError(message)
        work, energy, removed, broken = self._sums.tolist()
        for k in _STATE:
            setattr(self, k, self._spare[k])
        self._spare = current
        self.work += work
        self.x = end.clone()
        self.time += dt
        return dict(newly_broken=int(round(broken)), energy=energy, removed_bond_energy=removed)
