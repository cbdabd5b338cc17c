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

import numpy as np
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


# ---------------------------------------------------------------------------
# Line-searched Newton on the bond potential: static equilibrium and implicit
# Euler steps.

def rotation_quaternion(theta):
    """Unit quaternions (w, x, y, z) of rotation vectors (N, 3)."""
    angle = torch.linalg.vector_norm(theta, dim=1, keepdim=True)
    half = .5*angle
    # sin(t/2)/t, with its series below 1e-4
    scale = torch.where(angle > 1e-4, torch.sin(half)/angle.clamp_min(1e-300), .5 - angle*angle/48)
    return torch.cat((torch.cos(half), scale*theta), 1)


def quaternion_product(a, b):
    """Hamilton product a b of (N, 4) quaternions (w, x, y, z)."""
    aw, ax, ay, az = a.unbind(1)
    bw, bx, by, bz = b.unbind(1)
    return torch.stack((aw*bw - ax*bx - ay*by - az*bz, aw*bx + ax*bw + ay*bz - az*by,
                        aw*by - ax*bz + ay*bw + az*bx, aw*bz + ax*by - ay*bx + az*bw), 1)


def left_jacobian_transpose_apply(theta, v):
    """J_l(theta)^T v for the left Jacobian of SO(3), exp(theta + e) = exp(J_l e) exp(theta):
    J_l^T v = v - a theta x v + b theta x (theta x v), a = (1 - cos t)/t^2,
    b = (t - sin t)/t^3 (series below t = 1e-3)."""
    t = torch.linalg.vector_norm(theta, dim=1, keepdim=True)
    small = t < 1e-3
    tt = t.clamp_min(1e-300)
    a = torch.where(small, .5 - t*t/24, (1 - torch.cos(t))/(tt*tt))
    b = torch.where(small, 1/6 - t*t/120, (t - torch.sin(t))/(tt*tt*tt))
    c = torch.linalg.cross(theta, v, dim=1)
    return v - a*c + b*torch.linalg.cross(theta, c, dim=1)


class EnergyNewton:
    """Line-searched Newton on the bond potential of ``EnergyFoam``
    (``volume=False, kinematics='small'``: ``foam_dem_energy.py:303-315,
    405-421, 797-811``) for static equilibrium and implicit-Euler steps.

    Unknowns per site: a displacement u and a rotation vector t of the body
    rotation relative to the start of the solve (q = exp(t) q_0).  Potentials:

    * static: ``Pi(u, t) = E_b(X + u, exp(t) q_0) - f . u - tau . t``;
    * implicit Euler (dt): ``Phi = sum m |u - dt v|^2 / (2 dt^2) +
      sum I |t - dt w|^2 / (2 dt^2) + Pi``, after which v = u / dt, w = t / dt.

    Sites flagged ``fixed`` are held (static: at ``prescribed`` displacements,
    rotation held); their rows are removed from the gradient.  Each Newton
    direction solves ``(M/dt^2 + K) d = -g`` (static: ``K d = -g``) by the
    float32 block-Jacobi PCG over the bond-end sweep, with K the frozen tangent
    of the potential at the current configuration (``dpf_energy_tangent``; at
    the reference configuration K is the exact Hessian).  The step length
    follows an Armijo backtracking search on the float64 potential; the
    gradient (float64 forces and torques, ``dpf_bond_energy``; the rotation
    rows ``-J_l(t)^T tau``) decides convergence: ``|g| <= tolerance * scale``
    with scale the largest of the first gradient norm, |external load| and
    the roundoff level of the bond forces divided by the tolerance.
    """

    def __init__(self, geometry, young=1200., shear=480., device='cuda', theta=None, inner_tolerance=1e-2,
                 inner_iterations=200):
        self.law = EnergyFoam(geometry, volume=False, young=young, shear=shear, device=device)
        b = self.law._bonds
        self.device, self._lib = b.device, b._lib
        n, m = b.n_sites, b.n_bonds
        self.n_sites, self.n_bonds = n, m
        f64, f32, dev = F64, torch.float32, self.device
        self.theta = torch.zeros((n, 4), dtype=f64, device=dev) if theta is None else \
            torch.as_tensor(theta, dtype=f64, device=dev).contiguous()
        self.X = self.law.X
        self.x = self.X.clone()
        self.q = torch.zeros((n, 4), dtype=f64, device=dev)
        self.q[:, 0] = 1.
        self.v = torch.zeros((n, 3), dtype=f64, device=dev)
        self.w = torch.zeros((n, 3), dtype=f64, device=dev)
        self.fixed = b.fixed
        self.mass, self.inertia = self.law.mass, self.law.inertia
        self.inner_tolerance, self.inner_iterations = inner_tolerance, inner_iterations
        lib = self._lib
        self._bond_data = torch.zeros(max(4, lib.dpf_mixed_bond_floats(m)), dtype=f32, device=dev)
        self._ends = torch.empty(max(4, lib.dpf_end_floats(m)), dtype=f32, device=dev)
        self._mass32 = torch.cat((self.mass[:, None].expand(n, 3), self.inertia[:, None].expand(n, 3)), 1).float()
        self._zero32 = torch.zeros((n, 6), dtype=f32, device=dev)
        eye = torch.eye(6, dtype=f32, device=dev)
        self._identity32 = eye.expand(n, 6, 6).contiguous()
        self._ones32 = torch.ones((n, 6), dtype=f32, device=dev)
        self._block32 = torch.empty((n, 6, 6), dtype=f32, device=dev)
        self._p32 = torch.empty((n, 6, 6), dtype=f32, device=dev)
        self._units = torch.empty((n, 6), dtype=f64, device=dev)
        self._units32 = torch.empty((n, 6), dtype=f32, device=dev)
        self._site4 = torch.empty((n, 4), dtype=f32, device=dev)
        self._p24 = torch.empty(24*n, dtype=f32, device=dev)
        self._workspace = torch.empty(lib.dpf_tiled_workspace_floats(n), dtype=f32, device=dev)
        self._partials = torch.zeros(lib.dpf_tiled_partials_doubles(), dtype=f64, device=dev)
        self._cg = torch.zeros(1, dtype=torch.int32, device=dev)
        self._barrier = torch.zeros(2, dtype=torch.int32, device=dev)
        self._status = torch.zeros(1, dtype=torch.int32, device=dev)
        self.time = 0.

    def _stream(self):
        return torch.cuda.current_stream(self.device).cuda_stream

    def _evaluate(self, x0, q0, u, t, load, inertia):
        """Potential and its gradient (N, 6) at (u, t); fixed rows of the gradient zeroed."""
        law = self.law
        x = x0 + u
        q = quaternion_product(rotation_quaternion(t), q0)
        f, tau, e = law._run(self.theta, x, q, True, True)
        g = torch.cat((-f - load[:, :3], -left_jacobian_transpose_apply(t, tau) - load[:, 3:]), 1)
        phi = e[0] - (load[:, :3]*u).sum() - (load[:, 3:]*t).sum()
        if inertia is not None:
            dt, v, w = inertia
            du, dw = u - dt*v, t - dt*w
            g[:, :3] += self.mass[:, None]*du/(dt*dt)
            g[:, 3:] += self.inertia[:, None]*dw/(dt*dt)
            phi = phi + .5*((self.mass[:, None]*du*du).sum() + (self.inertia[:, None]*dw*dw).sum())/(dt*dt)
        g[self.fixed] = 0.
        return float(phi), g, x, q

    def _direction(self, x, q, g, inertia):
        """d with (M/dt^2 + K) d = -g (static: K d = -g) by the float32 bond-end PCG."""
        b = self.law._bonds
        stream = self._stream()
        _lib.check(self._lib.dpf_energy_tangent(ctypes.byref(b._graph), self.law.base.data_ptr(),
                                                self.theta.data_ptr(), self.theta.shape[1], x.data_ptr(),
                                                q.data_ptr(), self.law.ri.data_ptr(), self.law.rj.data_ptr(),
                                                self._bond_data.data_ptr(), stream), 'dpf_energy_tangent')
        # operator diag(mass32) + alpha K: alpha = dt^2 (the system times dt^2) or 1 (static)
        if inertia is None:
            mass32, alpha, rhs = self._zero32, 1., -g
        else:
            dt = inertia[0]
            mass32, alpha, rhs = self._mass32, dt*dt, -(dt*dt)*g
        # dpf_mixed_scaling takes the midpoint step: its alpha is dt'^2/4
        _lib.check(self._lib.dpf_mixed_scaling(ctypes.byref(b._graph), self._bond_data.data_ptr(), mass32.data_ptr(),
                                               self.fixed.data_ptr(), b._site_radii.data_ptr(), 2.*alpha**.5,
                                               self._block32.data_ptr(), self._p32.data_ptr(), self._units.data_ptr(),
                                               self._units32.data_ptr(), stream), 'dpf_mixed_scaling')
        _lib.check(self._lib.dpf_end_pack(ctypes.byref(b._graph), self._bond_data.data_ptr(), alpha,
                                          self._p32.data_ptr(), mass32.data_ptr(), self.fixed.data_ptr(),
                                          self._ends.data_ptr(), self._p24.data_ptr(), self._site4.data_ptr(),
                                          stream), 'dpf_end_pack')
        rhs = rhs.contiguous()
        out = torch.empty_like(rhs)
        _lib.check(self._lib.dpf_end_precondition(
            ctypes.byref(b._graph), self._ends.data_ptr(), self._site4.data_ptr(), self.fixed.data_ptr(),
            self._identity32.data_ptr(), self._p24.data_ptr(), self._ones32.data_ptr(), rhs.data_ptr(),
            float(self.inner_tolerance), int(self.inner_iterations), out.data_ptr(), self._cg.data_ptr(),
            self._workspace.data_ptr(), self._partials.data_ptr(), self._barrier.data_ptr(), self._status.data_ptr(),
            None, None, 0, stream), 'dpf_end_precondition')
        out[self.fixed] = 0.
        return out

    def _minimize(self, load, prescribed, inertia, tolerance, max_iterations):
        load = torch.as_tensor(load, dtype=F64, device=self.device).reshape(self.n_sites, 6)
        load = load.masked_fill(self.fixed[:, None], 0.)
        x0, q0 = self.x, self.q
        u = torch.zeros_like(x0)
        if prescribed is not None:
            prescribed = torch.as_tensor(prescribed, dtype=F64, device=self.device).reshape(self.n_sites, 3)
            u = torch.where(self.fixed[:, None], prescribed, u)
        t = torch.zeros_like(x0)
        self._cg.zero_()
        self._status.zero_()
        phi, g, x, q = self._evaluate(x0, q0, u, t, load, inertia)
        gnorm = float(torch.linalg.vector_norm(g))
        # floor: the roundoff level of bond forces (1e-13 of the stiffest bond times the largest coordinate)
        floor = 1e-13*float(self.law.base[:, 0].max())*float(x0.abs().max())/max(tolerance, 1e-300) \
            if self.n_bonds else 0.
        scale = max(gnorm, float(torch.linalg.vector_norm(load)), floor, 1e-300)
        trace = [gnorm/scale]
        for iteration in range(max_iterations + 1):
            if gnorm <= tolerance*scale:
                return u, t, x, q, dict(newton_iterations=iteration, relative_gradient=gnorm/scale,
                                        cg_iterations=int(self._cg.item()), gradient_trace=trace, energy=phi)
            if iteration == max_iterations:
                break
            d = self._direction(x, q, g, inertia)
            slope = float((g*d).sum())
            if not slope < 0:                      # not a descent direction: precondition the gradient only
                d = -g
                slope = -gnorm*gnorm
            du, dtheta = d[:, :3], d[:, 3:]
            step, accepted = 1., False
            for _ in range(30):
                cand = self._evaluate(x0, q0, u + step*du, t + step*dtheta, load, inertia)
                cnorm = float(torch.linalg.vector_norm(cand[1]))
                drop = cand[0] - phi
                if drop <= 1e-4*step*slope or (abs(drop) <= 1e-13*max(abs(phi), 1.) and cnorm < gnorm):
                    accepted = True
                    break
                step *= .5
            if not accepted:
                raise RuntimeError(f'energy Newton line search failed at relative gradient {gnorm/scale:g}')
            u, t = u + step*du, t + step*dtheta
            phi, g, x, q = cand
            gnorm = cnorm
            trace.append(gnorm/scale)
        if int(self._status.item()):
            raise RuntimeError(f'device status {int(self._status.item()):#x}')
        raise RuntimeError(f'energy Newton did not converge ({gnorm/scale:g})')

    @torch.no_grad()
    def solve(self, load=None, prescribed=None, tolerance=1e-10, max_iterations=60):
        """Static equilibrium under ``load`` (N, 6) [force, torque] with the
        fixed sites held at ``prescribed`` (N, 3) displacements from the
        current positions (rows of free sites ignored; None: held in place);
        the state moves to the equilibrium.  Returns info."""
        load = torch.zeros((self.n_sites, 6), dtype=F64, device=self.device) if load is None else load
        u, t, x, q, info = self._minimize(load, prescribed, None, tolerance, max_iterations)
        self.x, self.q = x, q
        return info

    @torch.no_grad()
    def step(self, dt, load, tolerance=1e-10, max_iterations=40):
        """One implicit-Euler step of length dt under ``load`` (N, 6); returns info."""
        if not np.isfinite(dt) or dt <= 0:
            raise ValueError('Positive finite dt required')
        u, t, x, q, info = self._minimize(load, None, (float(dt), self.v, self.w), tolerance, max_iterations)
        self.v, self.w = u/dt, t/dt
        self.x, self.q = x, q
        self.time += dt
        return info
