"""Energy-based bond law on the GPU: drop-in for the bond part of
``EnergyFoam`` (``experiments/foam_dem_energy.py:127-168, 303-315, 405-421,
797-811``) with ``volume=False`` and ``kinematics='small'``.

The bond potential of rest normal n0 and body-frame levers r_i, r_j,
E_b = kn dn^2/2 + ks |d_t|^2/2 + kb |phi_t|^2/2 + kt phi_n^2/2 with the
averaged-frame stretch d and the sin-angle relative rotation phi, stiffness
k = k0 exp((theta_i + theta_j)/2), and its closed-form force and world torque
are evaluated by one CUDA bond pass and a deterministic incidence gather.
"""
import ctypes

import torch

from . import _lib
from .newton import F64, LinearBonds

UNSUPPORTED = ('residual', 'enhanced', 'cosserat', 'bond_level', 'nonlinear_bonds')


class EnergyFoam:
    """``EnergyFoam(geometry, volume=False, kinematics='small', young, shear, device)``;
    ``energy(theta, x, q)`` and ``forces(theta, x, q) -> (force, torque)``."""

    def __init__(self, geometry, k_v=400., volume=True, device='cuda', young=1200., shear=480.,
                 kinematics='small', **options):
        if volume:
            raise NotImplementedError('volume terms are not part of the CUDA energy law; pass volume=False')
        if kinematics != 'small':
            raise NotImplementedError("only kinematics='small' is built")
        for key in UNSUPPORTED:
            if options.get(key):
                raise NotImplementedError(f'{key} is not part of the CUDA energy law')
        b = LinearBonds(geometry['points'], geometry['radii'], geometry['pairs'], geometry['areas'],
                        geometry['contacts'], geometry['masses'], geometry['fixed'], young, shear, device=device)
        self._bonds = b
        self.device = b.device
        self.X = b.p
        self.n = b.n_sites
        self.i, self.j = b.i, b.j
        self.n0, self.ri, self.rj = b.n.contiguous(), b.ri.contiguous(), b.rj.contiguous()
        self.base = torch.stack((b.kn, b.ks, b.kb, b.kt), 1).contiguous()
        self.mass, self.inertia = b.mass[:, 0], b.mass[:, 3]
        self.fixed = b.fixed
        self._lib = b._lib
        self._wrench = torch.empty(max(1, 9*b.n_bonds), dtype=F64, device=self.device)
        self._partials = torch.empty(self._lib.dpf_energy_partials_doubles(), dtype=F64, device=self.device)

    def _run(self, theta, x, q, forces, energy):
        theta = torch.as_tensor(theta, dtype=F64, device=self.device).contiguous()
        x = torch.as_tensor(x, dtype=F64, device=self.device).contiguous()
        q = torch.as_tensor(q, dtype=F64, device=self.device).contiguous()
        if theta.dim() != 2 or theta.shape[0] != self.n or theta.shape[1] < 4:
            raise ValueError('theta must be (n_sites, >= 4)')
        if x.shape != (self.n, 3) or q.shape != (self.n, 4):
            raise ValueError('x must be (n_sites, 3) and q (n_sites, 4)')
        f = torch.empty((self.n, 3), dtype=F64, device=self.device) if forces else None
        tau = torch.empty((self.n, 3), dtype=F64, device=self.device) if forces else None
        e = torch.empty(1, dtype=F64, device=self.device) if energy else None
        addr = lambda t: None if t is None else t.data_ptr()
        b = self._bonds
        _lib.check(self._lib.dpf_bond_energy(
            ctypes.byref(b._graph), self.base.data_ptr(), theta.data_ptr(), theta.shape[1], x.data_ptr(),
            q.data_ptr(), self.n0.data_ptr(), self.ri.data_ptr(), self.rj.data_ptr(), addr(f), addr(tau), addr(e),
            self._wrench.data_ptr(), self._partials.data_ptr(), b._stream()), 'dpf_bond_energy')
        return f, tau, e

    @torch.no_grad()
    def energy(self, theta, x, q):
        """Total bond energy (0-d float64 tensor)."""
        return self._run(theta, x, q, False, True)[2][0]

    @torch.no_grad()
    def forces(self, theta, x, q):
        """-dE/dx and -dE/d(world rotation), (n_sites, 3) each."""
        f, tau, _ = self._run(theta, x, q, True, False)
        return f, tau
