"""Drop-in GPU bonded-DEM solvers: ``LinearBonds``, ``FiniteBonds``, ``NewtonBonds``.

The classes keep the constructors, attributes (tensor names, shapes and
layouts), methods, plug-in points and error behaviour of the reference's
``LinearBondsGPU`` (``experiments/bonded_dem_linear_gpu.py``),
``FiniteBondsGPU`` (``experiments/bonded_dem_finite_gpu.py``) and
``NewtonBonds`` / ``FastNewtonBonds`` (``experiments/bonded_dem_newton.py``,
``experiments/bonded_dem_newton_fast.py``).  All tensors are float64 CUDA
tensors in the reference layouts; every bond sweep, block operation, Krylov
vector operation and reduction of the Newton path runs in the sm_103a kernels
of ``libdpf_gb300.so`` on ``torch.cuda.current_stream()``.

A method the caller replaces on an instance (``s.jacobian_vector = f`` as
``FastNewtonBonds`` does) is honoured: ``step`` then calls the replacement
through the reference's generic code path.
"""
import ctypes
import threading

import numpy as np
import torch

from . import _lib

F64 = torch.float64


class SubdivideError(RuntimeError):
    """Recoverable failure; the message starts with 'Subdivide:' as in the reference."""


_GUARD_MESSAGES = (
    (_lib.DPF_ERR_ROTATION, 'Subdivide: body rotation exceeds .25 rad in a step'),
    (_lib.DPF_ERR_COINCIDENT, 'Subdivide: coincident centers'),
    (_lib.DPF_ERR_NORMAL_TURN, 'Subdivide: normal turns more than .25 rad per half-step'),
    (_lib.DPF_ERR_NONFINITE, 'Subdivide: non-finite residual'),
    (_lib.DPF_ERR_BARRIER_TIMEOUT, 'Subdivide: device barrier timed out'),
)


def guard_error(status):
    """The reference's exception for a device status bitmask (first guard in reference order)."""
    for bit, message in _GUARD_MESSAGES:
        if status & bit:
            return SubdivideError(message)
    return SubdivideError(f'Subdivide: device status {status:#x}')


def _addr(t):
    return None if t is None else t.data_ptr()


def incidence(edges, n_sites):
    """Incidence CSR of the bond graph in the reference's index_add_ order.

    For every site: first the bonds whose first endpoint it is (value b, in
    increasing b), then those whose second endpoint it is (value ~b).
    """
    edges = np.asarray(edges, dtype=np.int64).reshape(-1, 2)
    m = len(edges)
    site = np.concatenate((edges[:, 0], edges[:, 1]))
    value = np.concatenate((np.arange(m, dtype=np.int64), ~np.arange(m, dtype=np.int64)))
    order = np.argsort(site, kind='stable')
    counts = np.bincount(site, minlength=n_sites)
    ptr = np.zeros(n_sites + 1, dtype=np.int64)
    np.cumsum(counts, out=ptr[1:])
    return ptr.astype(np.int32), value[order].astype(np.int32)


def device_incidence(edges, n_sites):
    """``incidence`` built on the device by one stable sort of the endpoint sites
    (int32 pointers and entries)."""
    m = edges.shape[0]
    site = torch.cat((edges[:, 0], edges[:, 1]))
    ids = torch.arange(m, dtype=torch.int64, device=edges.device)
    value = torch.cat((ids, -ids - 1))
    order = torch.sort(site, stable=True).indices
    ptr = torch.zeros(n_sites + 1, dtype=torch.int64, device=edges.device)
    ptr[1:] = torch.cumsum(torch.bincount(site, minlength=n_sites), 0)
    return ptr.to(torch.int32).contiguous(), value[order].to(torch.int32).contiguous()


_PINNED = threading.local()


def _pinned_buffers():
    """Pinned host buffers for device-scalar reads, one set per host thread and
    shared by every solver of that thread (a read copies, syncs and consumes
    them at once), so constructing a solver allocates no pinned memory."""
    if not hasattr(_PINNED, 'buffers'):
        _PINNED.buffers = (torch.zeros(1, dtype=torch.int32).pin_memory(), torch.zeros(64, dtype=F64).pin_memory(),
                           torch.zeros(64, dtype=F64).pin_memory())
    return _PINNED.buffers


def bond_setup(points, radii, pairs, areas, contacts, masses, young, shear):
    """Host-side setup arithmetic of ``LinearBondsGPU.__init__``
    (``experiments/bonded_dem_linear_gpu.py:15-40``): bond normals, contact
    levers, stiffnesses kn = E A/L, ks = G A/L, kb = E I/L, kt = 2 G I/L with
    I = A^2/(4 pi), and the (N, 6) mass [m, m, m, 0.4 m r^2 x 3]."""
    p = np.array(points, dtype=np.float64)
    edges = np.array(pairs, dtype=np.int64).reshape(-1, 2)
    if len(edges) and (edges.min() < 0 or edges.max() >= len(p)):
        raise ValueError('Invalid endpoint index')
    r = np.broadcast_to(np.asarray(radii, dtype=np.float64), (len(p),))
    area = np.broadcast_to(np.asarray(areas, dtype=np.float64), (len(edges),))
    c = np.asarray(contacts, dtype=np.float64).reshape(-1, 3)
    i, j = edges[:, 0], edges[:, 1]
    distance = p[j] - p[i]
    length = np.linalg.norm(distance, axis=1)
    second = area**2/(4*np.pi)
    mass = np.broadcast_to(np.asarray(masses, dtype=np.float64), (len(p),))
    inertia = .4*mass*r*r
    mass6 = np.concatenate((np.repeat(mass[:, None], 3, 1), np.repeat(inertia[:, None], 3, 1)), 1)
    if np.any(mass6 <= 0):
        raise ValueError('Only positive-mass bodies can enter this solver')
    return dict(p=p, edges=edges, n=distance/length[:, None], ri=c - p[i], rj=c - p[j], kn=young*area/length,
                ks=shear*area/length, kb=young*second/length, kt=shear*(2*second)/length, mass=mass6)


def classical_contacts(points, radii, pairs):
    """Classical ball contacts ``bonded_dem_finite_gpu.py:49-53``: midpoint shifted by the radius difference."""
    p = np.asarray(points, dtype=np.float64)
    i, j = np.asarray(pairs, dtype=np.int64).reshape(-1, 2).T
    radii_a = np.broadcast_to(np.asarray(radii, dtype=np.float64), (len(p),))
    n = p[j] - p[i]
    n /= np.linalg.norm(n, axis=1)[:, None]
    return .5*(p[i] + p[j]) + .5*(radii_a[i] - radii_a[j])[:, None]*n


class LinearBonds:
    """Stress-free linearised bonds (drop-in for ``LinearBondsGPU``,
    ``experiments/bonded_dem_linear_gpu.py:14-124``)."""

    def __init__(self, points, radii, pairs, areas, contacts, masses, fixed,
                 young=1200., shear=480., device='cuda'):
        self.device = torch.device(device)
        if self.device.type != 'cuda':
            raise ValueError('dpf_gb300 solvers run on CUDA devices only')
        if self.device.index is None:
            self.device = torch.device('cuda', torch.cuda.current_device())
        self._lib = _lib.load()
        self.tensor = lambda x: torch.as_tensor(x, dtype=F64, device=self.device)
        self._offset = self._setup(points, radii, pairs, areas, contacts, masses, fixed, young, shear)
        n_sites, n_bonds = self.p.shape[0], self.edges.shape[0]
        self._inc_ptr, self._inc_bond = device_incidence(self.edges, n_sites)
        self._graph = _lib.Graph(n_sites, n_bonds, self.edges.data_ptr() if n_bonds else None,
                                 self._inc_ptr.data_ptr(), self._inc_bond.data_ptr())
        self._wrench = torch.empty(max(1, self._lib.dpf_wrench_scratch_doubles(n_bonds)), dtype=F64,
                                   device=self.device)
        self._partials = torch.zeros(self._lib.dpf_partials_doubles(), dtype=F64, device=self.device)
        self._status = torch.zeros(1, dtype=torch.int32, device=self.device)
        self._scalars = torch.zeros(8, dtype=F64, device=self.device)
        self._host_status, self._host_scalars, _ = _pinned_buffers()
        self.q, self.v = torch.zeros_like(self.mass), torch.zeros_like(self.mass)
        self.kq = torch.zeros_like(self.mass)
        self.diagonal = self._diagonal_blocks()
        self.preconditioner = None
        self.preconditioner_dt = None

    def _setup(self, points, radii, pairs, areas, contacts, masses, fixed, young, shear):
        """Setup arithmetic of ``LinearBondsGPU.__init__`` (``bonded_dem_linear_gpu.py:15-40``)
        in one device pass over the bonds and one over the sites (``dpf_bond_setup``):
        normals, contact levers (classical ball contacts when ``contacts`` is
        None), kn = E A/L, ks = G A/L, kb = E I/L, kt = 2 G I/L with I = A^2/(4 pi),
        and the (N, 6) mass [m, m, m, 0.4 m r^2 x 3].  Returns the contact offsets
        (contacts - classical)."""
        p = np.array(points, dtype=np.float64).reshape(-1, 3)
        n = len(p)
        edges = np.array(pairs, dtype=np.int64).reshape(-1, 2)
        m = len(edges)
        if m and (edges.min() < 0 or edges.max() >= n):
            raise ValueError('Invalid endpoint index')
        r = np.array(np.broadcast_to(np.asarray(radii, dtype=np.float64), (n,)))
        mass = np.array(np.broadcast_to(np.asarray(masses, dtype=np.float64), (n,)))
        if np.any(mass <= 0) or np.any(.4*mass*r*r <= 0):
            raise ValueError('Only positive-mass bodies can enter this solver')
        area = np.array(np.broadcast_to(np.asarray(areas, dtype=np.float64), (m,)))
        dev = self.device
        self.p = self.tensor(p)
        self.edges = torch.as_tensor(edges, device=dev).contiguous()
        self.i, self.j = self.edges.T
        self._site_radii = self.tensor(r)
        mass_d = self.tensor(mass)
        area_d = self.tensor(area)
        contacts_d = None if contacts is None else self.tensor(np.array(contacts, dtype=np.float64).reshape(-1, 3))
        e = lambda *shape: torch.empty(shape, dtype=F64, device=dev)
        self.n, self.ri, self.rj, offset = e(m, 3), e(m, 3), e(m, 3), e(m, 3)
        self.kn, self.ks, self.kb, self.kt = e(m), e(m), e(m), e(m)
        self.mass = e(n, 6)
        self._call('dpf_bond_setup', n, m, self.edges.data_ptr() if m else None, self.p.data_ptr(),
                   self._site_radii.data_ptr(), area_d.data_ptr(), _addr(contacts_d), mass_d.data_ptr(),
                   float(young), float(shear), None, None, self.n.data_ptr(), self.ri.data_ptr(), self.rj.data_ptr(),
                   self.kn.data_ptr(), self.ks.data_ptr(), self.kb.data_ptr(), self.kt.data_ptr(), offset.data_ptr(),
                   self.mass.data_ptr(), self._stream())
        self.fixed = torch.as_tensor(np.array(fixed, dtype=bool), device=dev)
        return offset

    # ---- plumbing ---------------------------------------------------------
    @property
    def n_sites(self):
        return int(self._graph.n_sites)

    @property
    def n_bonds(self):
        return int(self._graph.n_bonds)

    def _stream(self):
        return torch.cuda.current_stream(self.device).cuda_stream

    def _vec(self, a, shape=None):
        a = torch.as_tensor(a, dtype=F64, device=self.device)
        return a.contiguous()

    def _stiffness_struct(self):
        return _lib.Stiffness(*(_addr(t.contiguous()) for t in (self.kn, self.ks, self.kb, self.kt)))

    def _tangent_struct(self):
        for name in ('n', 'ri', 'rj'):
            t = getattr(self, name)
            if not t.is_contiguous():
                setattr(self, name, t.contiguous())
        return _lib.Tangent(self.n.data_ptr(), self.ri.data_ptr(), self.rj.data_ptr())

    def _call(self, name, *args):
        calls = self.__dict__.get('call_profile')
        if calls is None:
            _lib.check(getattr(self._lib, name)(*args), name)
            return
        # CUDA events around the library call on the current stream, by entry point
        start, end = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        start.record()
        _lib.check(getattr(self._lib, name)(*args), name)
        end.record()
        calls.setdefault(name, []).append((start, end))

    def _fetch(self, scalars=0, status=False):
        """Copy device scalars (and the status word) to the host with one sync;
        a step's deferred scale (see ``MixedNewtonBonds._step_begin``) rides along."""
        stream = torch.cuda.current_stream(self.device)
        if scalars:
            self._host_scalars[:scalars].copy_(self._scalars[:scalars], non_blocking=True)
        if status:
            self._host_status.copy_(self._status[:1], non_blocking=True)
        deferred = getattr(self, '_deferred_scale', None)
        if deferred is not None:
            self._host_scalars[8:10].copy_(deferred, non_blocking=True)
            self._deferred_scale = None
        stream.synchronize()
        return self._host_scalars[:scalars].tolist(), int(self._host_status[0]) if status else 0

    # ---- reference methods ------------------------------------------------
    @torch.no_grad()
    def stiffness(self, q):
        """Frozen-tangent K q (``bonded_dem_linear_gpu.py:42-52``)."""
        q = self._vec(q)
        out = torch.empty_like(q)
        self._call('dpf_stiffness_apply', ctypes.byref(self._graph), ctypes.byref(self._stiffness_struct()),
                   ctypes.byref(self._tangent_struct()), q.data_ptr(), out.data_ptr(), self._wrench.data_ptr(),
                   self._stream())
        return out

    @torch.no_grad()
    def _diagonal_blocks(self):
        """Per-site 6x6 diagonal blocks of K (``bonded_dem_linear_gpu.py:54-72``)."""
        out = torch.empty((self.n_sites, 6, 6), dtype=F64, device=self.device)
        self._call('dpf_diagonal_blocks', ctypes.byref(self._graph), ctypes.byref(self._stiffness_struct()),
                   ctypes.byref(self._tangent_struct()), out.data_ptr(), self._stream())
        return out

    def _operator(self, q, alpha):
        """(diag M + alpha K) q, identity rows on fixed sites (``bonded_dem_linear_gpu.py:74-77``)."""
        q = self._vec(q)
        if 'stiffness' in self.__dict__:       # an instance plug-in supplies K q
            return torch.where(self.fixed[:, None], q, torch.addcmul(alpha*self.stiffness(q), self.mass, q))
        out = torch.empty_like(q)
        self._call('dpf_operator_apply', ctypes.byref(self._graph), ctypes.byref(self._stiffness_struct()),
                   ctypes.byref(self._tangent_struct()), self.mass.data_ptr(), self.fixed.data_ptr(), float(alpha),
                   q.data_ptr(), out.data_ptr(), self._wrench.data_ptr(), self._stream())
        return out

    # ---- linear solves on the library's cooperative block PCG ----------------
    def _solver_buffers(self):
        """Workspace, barrier, info and reduction partials of the library PCG and sums."""
        if getattr(self, '_lin', None) is None:
            lib, dev = self._lib, self.device
            self._lin = dict(work=torch.empty(lib.dpf_block_pcg_workspace_doubles(self.n_sites), dtype=F64, device=dev),
                             barrier=torch.zeros(2, dtype=torch.int32, device=dev),
                             aux=torch.zeros(64, dtype=F64, device=dev),
                             flag=torch.zeros(1, dtype=torch.int32, device=dev),
                             partials=torch.zeros(lib.dpf_small_partials_doubles(), dtype=F64, device=dev))
        self._lin['host'] = _pinned_buffers()[2]
        return self._lin

    def _read_aux(self, count, status=False):
        """aux[:count] (and the status word) on the host after one stream sync."""
        buf = self._solver_buffers()
        buf['host'][:count].copy_(buf['aux'][:count], non_blocking=True)
        if status:
            self._host_status.copy_(self._status[:1], non_blocking=True)
        torch.cuda.current_stream(self.device).synchronize()
        return buf['host'][:count].tolist(), int(self._host_status[0]) if status else 0

    def _block_inverse(self, alpha):
        """(diag M + alpha D)^-1 per site from ``self.diagonal`` (identity on fixed sites)."""
        out = torch.empty((self.n_sites, 6, 6), dtype=F64, device=self.device)
        diagonal = self.diagonal.to(F64).contiguous()
        self._call('dpf_block_inverse', self.n_sites, self.mass.data_ptr(), self.fixed.data_ptr(),
                   diagonal.data_ptr(), float(alpha), None, out.data_ptr(), self._stream())
        return out

    def _block_pcg(self, rhs, alpha, tolerance, max_iterations, mode, x, use_guess, scale=None, info_at=0):
        """Launch the library PCG (mode 0: linear test, 1: balanced test); its
        [iterations, relative, state, |rhs|] land in aux[info_at:info_at+4]."""
        buf = self._solver_buffers()
        self._call('dpf_block_pcg', ctypes.byref(self._graph), ctypes.byref(self._stiffness_struct()),
                   ctypes.byref(self._tangent_struct()), self.mass.data_ptr(), self.fixed.data_ptr(),
                   self.preconditioner.data_ptr(), _addr(scale), rhs.data_ptr(), float(alpha), float(tolerance),
                   int(max_iterations), int(mode), int(use_guess), x.data_ptr(), buf['aux'][info_at:].data_ptr(),
                   self._wrench.data_ptr(), buf['work'].data_ptr(), buf['barrier'].data_ptr(), self._status.data_ptr(),
                   self._stream())

    @torch.no_grad()
    def solve_increment(self, rhs, dt, guess=None, tolerance=2e-8, max_iterations=1000):
        """Block-Jacobi PCG of the linear model (``bonded_dem_linear_gpu.py:79-112``):
        one cooperative launch with the reference's stopping test, then one read
        of its iteration count and true residual."""
        alpha = .25*dt*dt
        if self.preconditioner_dt != dt:
            self.preconditioner = self._block_inverse(alpha)
            self.preconditioner_dt = dt
        x = torch.zeros_like(self.mass) if guess is None else self._vec(guess).clone()
        return x, self._linear_result(self._vec(rhs), alpha, x, guess is not None, tolerance, max_iterations)

    def _linear_result(self, rhs, alpha, x, use_guess, tolerance, max_iterations):
        self._block_pcg(rhs, alpha, tolerance, max_iterations, 0, x, use_guess)
        (iterations, relative, state, norm), _ = self._read_aux(4)
        if norm < 1e-30:
            return dict(iterations=0, relative_residual=0.)
        if state == 2:
            raise RuntimeError('Nonfinite conjugate-gradient residual')
        if not relative <= 5*tolerance:
            raise RuntimeError(f'Linear solve failed after {int(iterations)} iterations: {relative}')
        return dict(iterations=int(iterations), relative_residual=relative)

    @torch.no_grad()
    def step(self, dt, external):
        """Linear implicit midpoint (``bonded_dem_linear_gpu.py:114-121``): the
        right-hand side and the dt v guess in one kernel, the library PCG, then
        the velocity/displacement update, K q and the work on the device."""
        external, v, kq = self._vec(external), self._vec(self.v).clone(), self._vec(self.kq)
        rhs, dq = torch.empty_like(v), torch.empty_like(v)
        n, stream = self.n_sites, self._stream()
        self._call('dpf_linear_midpoint_rhs', n, self.mass.data_ptr(), v.data_ptr(), external.data_ptr(),
                   kq.data_ptr(), float(dt), rhs.data_ptr(), dq.data_ptr(), stream)
        alpha = .25*dt*dt
        if self.preconditioner_dt != dt:
            self.preconditioner = self._block_inverse(alpha)
            self.preconditioner_dt = dt
        metrics = self._linear_result(rhs, alpha, dq, True, 2e-8, 1000)   # a vanishing rhs leaves dq = 0
        self.q = self._vec(self.q)
        self._call('dpf_linear_midpoint_advance', n, dq.data_ptr(), float(dt), v.data_ptr(), self.q.data_ptr(), stream)
        self.v = v
        self.kq = self.stiffness(self.q)
        buf = self._solver_buffers()
        self._call('dpf_linear_sums', n, external.data_ptr(), dq.data_ptr(), None, None, None, None,
                   buf['aux'].data_ptr(), buf['partials'].data_ptr(), stream)
        (work,), _ = self._read_aux(1)
        return work, metrics

    @torch.no_grad()
    def energy(self):
        """(sum m v^2 + q . K q) / 2 (``bonded_dem_linear_gpu.py:123-124``)."""
        buf = self._solver_buffers()
        v, q, kq = self._vec(self.v), self._vec(self.q), self._vec(self.kq)
        self._call('dpf_linear_sums', self.n_sites, None, None, self.mass.data_ptr(), v.data_ptr(), q.data_ptr(),
                   kq.data_ptr(), buf['aux'].data_ptr(), buf['partials'].data_ptr(), self._stream())
        (_, value), _ = self._read_aux(2)
        return value


class FiniteBonds(LinearBonds):
    """Finite-motion rate law (drop-in for ``FiniteBondsGPU``,
    ``experiments/bonded_dem_finite_gpu.py:46-261``)."""

    PHYSICAL_STATE = ('x', 'v', 'rotation', 'normal', 'offset', 'fn', 'fs', 'mt', 'mb')

    def __init__(self, points, radii, pairs, areas, masses, fixed, contacts=None,
                 young=1200., shear=480., device='cuda'):
        # contacts=None: classical ball contacts, computed with the levers on the device
        super().__init__(points, radii, pairs, areas, contacts, masses, fixed, young, shear, device)
        self.x = self.p.clone()
        self.radii = self._site_radii
        self.normal = self.n.clone()
        self.offset = self._offset
        self.fn, self.mt = torch.zeros_like(self.kn), torch.zeros_like(self.kn)
        self.fs, self.mb = torch.zeros_like(self.n), torch.zeros_like(self.n)
        self.rotation = torch.eye(3, dtype=F64, device=self.device).repeat(self.n_sites, 1, 1)
        self.time = 0.

    def _history_struct(self):
        for name in ('x', 'radii', 'normal', 'offset', 'fn', 'fs', 'mt', 'mb'):
            t = getattr(self, name)
            if not (t.is_contiguous() and t.dtype == F64):
                setattr(self, name, t.to(F64).contiguous())
        return _lib.History(self.x.data_ptr(), self.radii.data_ptr(), self.normal.data_ptr(), self.offset.data_ptr(),
                            self.fn.data_ptr(), self.fs.data_ptr(), self.mt.data_ptr(), self.mb.data_ptr())

    def _raise_status(self):
        _, status = self._fetch(status=True)
        if status:
            raise guard_error(status)

    def geometry(self, x):
        """Bond normal and classical contact (``bonded_dem_finite_gpu.py:66-73``)."""
        d = x[self.j] - x[self.i]
        length = torch.linalg.vector_norm(d, dim=1)
        if bool(torch.any(length <= 1e-12)):
            raise SubdivideError('Subdivide: coincident centers')
        n = d/length[:, None]
        c = .5*(x[self.i] + x[self.j]) + .5*(self.radii[self.i] - self.radii[self.j])[:, None]*n
        return n, c

    def assemble(self, fn, fs, mt, mb, n, ri, rj):
        """Scatter bond force and couple to sites (``bonded_dem_finite_gpu.py:75-80``)."""
        f, couple = fn[:, None]*n + fs, mt[:, None]*n + mb
        out = torch.zeros_like(self.mass)
        out.index_add_(0, self.i, torch.cat((f, torch.linalg.cross(ri, f) + couple), 1))
        out.index_add_(0, self.j, torch.cat((-f, -torch.linalg.cross(rj, f) - couple), 1))
        return out

    @torch.no_grad()
    def loads(self):
        """Net force and torque of the committed state (``bonded_dem_finite_gpu.py:82-85``)."""
        out = torch.empty_like(self.mass)
        self._call('dpf_loads', ctypes.byref(self._graph), ctypes.byref(self._history_struct()), out.data_ptr(),
                   self._wrench.data_ptr(), self._stream())
        return out

    def _new_trial(self):
        m, n = self.n_bonds, self.n_sites
        e = lambda *shape: torch.empty(shape, dtype=F64, device=self.device)
        return dict(force=e(n, 6), n=e(m, 3), ri=e(m, 3), rj=e(m, 3), x=e(n, 3), normal=e(m, 3), fn=e(m),
                    mt=e(m), fs=e(m, 3), mb=e(m, 3), offset=e(m, 3))

    @staticmethod
    def _trial_struct(t, end=True):
        g = lambda k: _addr(t.get(k)) if t is not None else None
        if not end:
            return _lib.TrialOut(g('force'), g('n'), g('ri'), g('rj'))
        return _lib.TrialOut(g('force'), g('n'), g('ri'), g('rj'), g('x'), g('normal'), g('offset'), g('fs'),
                             g('mb'), g('fn'), g('mt'))

    @torch.no_grad()
    def trial(self, increment, *, mid_positions=None, end_positions=None, _check=True):
        """Pure constitutive trial from committed history (``bonded_dem_finite_gpu.py:87-116``)."""
        y = self._vec(increment)
        mid = None if mid_positions is None else self._vec(mid_positions)
        end = None if end_positions is None else self._vec(end_positions)
        out = self._new_trial()
        self._status.zero_()
        self._call('dpf_trial', ctypes.byref(self._graph), ctypes.byref(self._stiffness_struct()),
                   ctypes.byref(self._history_struct()), y.data_ptr(), _addr(mid), _addr(end), 1,
                   ctypes.byref(self._trial_struct(out)), self._wrench.data_ptr(), self._status.data_ptr(),
                   self._stream())
        if _check:
            self._raise_status()
        return out

    def commit(self, trial):
        """Adopt a trial's end state (``bonded_dem_finite_gpu.py:118-120``)."""
        for name in ('x', 'normal', 'fn', 'fs', 'mt', 'mb', 'offset'):
            setattr(self, name, trial[name])

    @torch.no_grad()
    def energy(self):
        """Elastic plus kinetic energy (``bonded_dem_finite_gpu.py:122-125``)."""
        v = self._vec(self.v)
        self._call('dpf_energy', ctypes.byref(self._graph), ctypes.byref(self._stiffness_struct()),
                   ctypes.byref(self._history_struct()), self.mass.data_ptr(), v.data_ptr(),
                   self._scalars.data_ptr(), self._partials.data_ptr(), self._stream())
        values, _ = self._fetch(1)
        return values[0]

    def _pose_scale(self):
        """Per-DOF scale of the pose defect: [r, r, r, 1, 1, 1] (``bonded_dem_finite_gpu.py:129-130``)."""
        scale = torch.ones_like(self.mass)
        scale[:, :3] = self._vec(self.radii)[:, None]
        return scale

    @torch.no_grad()
    def local_defect(self, residual):
        """Max block-scaled pose defect max |P r / scale| (``bonded_dem_finite_gpu.py:127-131``)."""
        buf = self._solver_buffers()
        r = self._vec(residual)
        self._call('dpf_scale_residual', self.n_sites, self.preconditioner.data_ptr(), self._pose_scale().data_ptr(),
                   r.data_ptr(), None, buf['aux'].data_ptr(), self._partials.data_ptr(), self._stream())
        (_, value), _ = self._read_aux(2)
        return value

    def _balanced_solve(self, rhs, dt, tolerance, max_iterations, scale, info_at=0):
        """Launch the balanced PCG of the previous solver on the blocks of
        ``self.diagonal`` (the preconditioner is rebuilt every call, as the
        reference does); nothing is read back here."""
        alpha = .25*dt*dt
        self.preconditioner = self._block_inverse(alpha)
        x = torch.empty_like(self.mass)
        self._block_pcg(rhs, alpha, tolerance, max_iterations, 1, x, False, scale=scale, info_at=info_at)
        return x

    @staticmethod
    def _balanced_outcome(info):
        iterations, _, state, norm = info
        if norm < 1e-40:
            return 0
        if state == 2:
            raise RuntimeError('Nonfinite PCG residual')
        if state != 0:
            raise SubdivideError('Subdivide: balanced PCG did not converge')
        return int(iterations)

    @torch.no_grad()
    def solve_increment(self, rhs, dt, tolerance=2e-7, max_iterations=1600):
        """Block-Jacobi PCG with the local pose-defect and global residual tests
        and a true-residual exit check (``bonded_dem_finite_gpu.py:133-167``),
        one cooperative launch."""
        x = self._balanced_solve(self._vec(rhs), dt, tolerance, max_iterations, self._pose_scale())
        info, _ = self._read_aux(4)
        return x, dict(iterations=self._balanced_outcome(info))

    def _previous_residual(self, y, dt, external, v, preconditioner, scale, tangent=None):
        """Midpoint residual at y (fixed rows y = 0) with [|r|, max |P r / scale|]
        in aux[0:2] and the trial guards in the status word; returns r."""
        r = torch.empty_like(y)
        self._status.zero_()
        use_p = preconditioner is not None
        self._call('dpf_residual', ctypes.byref(self._graph), ctypes.byref(self._stiffness_struct()),
                   ctypes.byref(self._history_struct()), y.data_ptr(), v.data_ptr(), external.data_ptr(),
                   self.mass.data_ptr(), self.fixed.data_ptr(), float(dt),
                   ctypes.byref(self._trial_struct(tangent, end=False)) if tangent else None,
                   preconditioner.data_ptr() if use_p else None, scale.data_ptr() if use_p else None, r.data_ptr(),
                   None, self._solver_buffers()['aux'].data_ptr(), self._wrench.data_ptr(), self._partials.data_ptr(),
                   self._status.data_ptr(), self._stream())
        return r

    @torch.no_grad()
    def step(self, dt, external, tolerance=2e-7, max_iterations=18):
        """The reference's previous solver (``bonded_dem_finite_gpu.py:169-250``):
        nonlinear implicit midpoint by block-PCG corrections, type-II Anderson
        mixing over the last six iterates and merit backtracking.  Every bond
        sweep, solve, mixing reduction and norm runs in library kernels; the host
        reads a few scalars per iteration and solves the at most 5 x 5 mixing
        system."""
        if not np.isfinite(dt) or dt <= 0:
            raise ValueError('Positive finite dt required')
        dt = float(dt)
        external, v = self._vec(external), self._vec(self.v)
        n, stream, buf = self.n_sites, self._stream(), self._solver_buffers()
        self._call('dpf_rhs_scale', n, self.mass.data_ptr(), v.data_ptr(), external.data_ptr(),
                   self.loads().data_ptr(), self.fixed.data_ptr(), dt, buf['aux'][8:].data_ptr(),
                   self._partials.data_ptr(), stream)
        scale = self._pose_scale()
        mixing = _Mixing(self, 6)
        y = torch.zeros_like(self.mass)
        m = self.n_bonds
        tangent = {k: torch.empty((m, 3), dtype=F64, device=self.device) for k in ('n', 'ri', 'rj')}
        tangent['force'] = None
        solved = 0
        relative = float('nan')
        rhs_scale = None
        for iteration in range(max_iterations):
            r = self._previous_residual(y, dt, external, v, self.preconditioner if iteration else None, scale, tangent)
            values, status = self._read_aux(10, status=True)
            if rhs_scale is None:
                rhs_scale = max(values[8], .5*dt*dt*values[9], 1e-30)
            if status:
                raise guard_error(status)
            relative = values[0]/rhs_scale
            local = values[1] if iteration else (0. if relative == 0 else float('inf'))
            if relative < tolerance and local < 2e-6:
                return self._accept_previous(y, dt, external, v, dict(
                    nonlinear_iterations=iteration, nonlinear_relative_residual=relative, cg_iterations=solved,
                    local_pose_defect=local))
            # frozen tangent of this iterate, its blocks, the balanced correction
            self.n, self.ri, self.rj = tangent['n'], tangent['ri'], tangent['rj']
            tangent = {k: torch.empty((m, 3), dtype=F64, device=self.device) for k in ('n', 'ri', 'rj')}
            tangent['force'] = None
            self.diagonal = self._diagonal_blocks()
            self.preconditioner_dt = None
            rhs = torch.empty_like(r)
            self._call('dpf_axpby', 6*n, -1., r.data_ptr(), 0., r.data_ptr(), rhs.data_ptr(), stream)
            correction = self._balanced_solve(rhs, dt, 2e-7, 1600, scale, info_at=4)
            self._call('dpf_scale_residual', n, self.preconditioner.data_ptr(), scale.data_ptr(), r.data_ptr(), None,
                       buf['aux'][1:].data_ptr(), self._partials.data_ptr(), stream)
            mixing.push(y, correction)
            terms = mixing.reduce(buf['aux'][16:])
            values, _ = self._read_aux(16 + terms)
            solved += self._balanced_outcome(values[4:8])
            merit = max(relative/tolerance, values[2]/2e-6)
            directions = []
            accelerated = mixing.mix(values[16:16 + terms])
            if accelerated is not None:
                directions.append(accelerated)
            directions.append(correction)
            y = self._backtrack(y, directions, merit, dt, external, v, scale, rhs_scale, tolerance)
        raise SubdivideError(f'Subdivide: nonlinear residual {relative} did not converge')

    def _backtrack(self, y, directions, merit, dt, external, v, scale, rhs_scale, tolerance):
        """First candidate y + f d (d in order, f = 1, 1/2, .., 1/16) whose trial
        passes every guard and whose merit max(|r|/scale/tol, defect/2e-6) is
        below the iterate's (``bonded_dem_finite_gpu.py:231-249``)."""
        candidate = torch.empty_like(y)
        for direction in directions:
            for halvings in range(5):
                self._call('dpf_axpby', 6*self.n_sites, 1., y.data_ptr(), 2.**-halvings, direction.data_ptr(),
                           candidate.data_ptr(), self._stream())
                self._previous_residual(candidate, dt, external, v, self.preconditioner, scale)
                (norm, defect), status = self._read_aux(2, status=True)
                if not status and max(norm/rhs_scale/tolerance, defect/2e-6) < merit:
                    return candidate
        raise SubdivideError('Subdivide: nonlinear line search failed')

    def _accept_previous(self, y, dt, external, v, info):
        """Commit the trial at y, v <- 2 y/dt - v, R <- exp(y_w) R; work = external . y."""
        state = self.trial(y)
        velocity, rotation = v.clone(), self._vec(self.rotation).clone()
        self._call('dpf_accept_step', self.n_sites, y.data_ptr(), dt, velocity.data_ptr(), rotation.data_ptr(),
                   self._stream())
        buf = self._solver_buffers()
        self._call('dpf_linear_sums', self.n_sites, external.data_ptr(), y.data_ptr(), None, None, None, None,
                   buf['aux'].data_ptr(), buf['partials'].data_ptr(), self._stream())
        buf['aux'][1:2].copy_(torch.linalg.vector_norm(y[:, 3:], dim=1).max().reshape(1) if len(y) else
                              torch.zeros(1, dtype=F64, device=self.device))
        (work, turn), _ = self._read_aux(2)
        self.commit(state)
        self.v, self.rotation = velocity, rotation
        self.time += dt
        return work, dict(info, max_step_rotation=turn)

    def advance_interval(self, dt, force_at_time, depth=0):
        """Advance by dt; an interval whose step fails with 'Subdivide:' is
        replaced by its two halves, down to depth 8 (``bonded_dem_finite_gpu.py:252-261``).
        The halves are walked depth first from an explicit stack; records come
        out in time order."""
        work, records = 0., []
        pending = [(float(dt), depth)]
        while pending:
            h, level = pending.pop()
            try:
                value, info = self.step(h, force_at_time(self.time + .5*h))
            except RuntimeError as error:
                if level >= 8 or 'Subdivide:' not in str(error):
                    raise
                pending += [(.5*h, level + 1), (.5*h, level + 1)]
                continue
            work += value
            records.append(dict(dt=h, subdivision_depth=level, **info))
        return work, records


class _Mixing:
    """Type-II Anderson mixing of the previous solver over device slots holding
    the last ``depth`` (iterate, correction) pairs (``bonded_dem_finite_gpu.py:215-229``):
    one kernel reduces the weighted Gram system of the correction differences,
    the host solves it (at most 5 x 5, ridge 1e-10 trace), one kernel forms
    c - sum_h a_h (dy_h + dc_h)."""

    def __init__(self, solver, depth):
        self.solver, self.depth = solver, depth
        shape = (depth, solver.n_sites, 6)
        self.y = torch.empty(shape, dtype=F64, device=solver.device)
        self.c = torch.empty(shape, dtype=F64, device=solver.device)
        self.slots = []       # oldest first

    def push(self, y, correction):
        slot = self.slots.pop(0) if len(self.slots) == self.depth else len(self.slots)
        self.y[slot].copy_(y)
        self.c[slot].copy_(correction)
        self.slots.append(slot)

    def _order(self):
        return (ctypes.c_int32*len(self.slots))(*self.slots)

    def reduce(self, out):
        """Launch the Gram reduction into ``out``; returns the number of terms (0: nothing to mix)."""
        count = len(self.slots)
        if count < 2:
            return 0
        s = self.solver
        s._call('dpf_anderson_gram', s.n_sites, self.y.data_ptr(), self.c.data_ptr(), self.depth, self._order(), count,
                s._vec(s.radii).data_ptr(), out.data_ptr(), s._solver_buffers()['partials'].data_ptr(), s._stream())
        return (count - 1)*count//2 + count - 1

    def mix(self, terms):
        """Mixed direction from the reduced terms, or None when it is not finite."""
        count = len(self.slots)
        if count < 2:
            return None
        k = count - 1
        gram = np.zeros((k, k))
        upper = iter(terms[:k*(k + 1)//2])
        for h in range(k):
            for l in range(h, k):
                gram[h, l] = gram[l, h] = next(upper)
        proj = np.asarray(terms[k*(k + 1)//2:k*(k + 1)//2 + k])
        ridge = 1e-10*max(np.trace(gram), 1e-40)
        coefficients = np.ascontiguousarray(np.linalg.solve(gram + ridge*np.eye(k), proj), dtype=np.float64)
        s = self.solver
        out = torch.empty_like(s.mass)
        flag = s._solver_buffers()['flag']
        flag.zero_()
        s._call('dpf_anderson_mix', s.n_sites, self.y.data_ptr(), self.c.data_ptr(), self.depth, self._order(), count,
                coefficients.ctypes.data_as(ctypes.POINTER(ctypes.c_double)), out.data_ptr(), flag.data_ptr(),
                s._stream())
        return None if int(flag.item()) else out


class _Krylov:
    """Device workspace of one FGMRES cycle (basis, transformed rows, h column)."""

    def __init__(self, length, width, device):
        self.length, self.width = length, width
        self.basis = torch.empty((width+1, length), dtype=F64, device=device)
        self.transformed = torch.empty((width, length), dtype=F64, device=device)
        self.h = torch.zeros(72, dtype=F64, device=device)


class _Krylov32:
    """Float32 Krylov vectors of the mixed Newton path's FGMRES (basis,
    transformed rows, the Arnoldi vector) with its float64 h column, partials
    and vectors (x, true residual)."""

    def __init__(self, length, width, device):
        self.length, self.width = length, width
        f32 = torch.float32
        self.basis = torch.empty((width+1, length), dtype=f32, device=device)
        self.transformed = torch.empty((width, length), dtype=f32, device=device)
        self.products = torch.empty((width, length), dtype=f32, device=device)   # J z_k
        self.w = torch.empty(length, dtype=f32, device=device)
        self.h = torch.zeros(72, dtype=F64, device=device)
        self.partials = torch.zeros(_lib.load().dpf_partials_doubles(), dtype=F64, device=device)
        self.scalars = torch.zeros(2, dtype=F64, device=device)
        self.x = torch.empty(length, dtype=F64, device=device)
        self.product = torch.empty(length, dtype=F64, device=device)    # J x
        self.residual = torch.empty(length, dtype=F64, device=device)


def _back_substitute(h, g, k):
    """Solve the k x k upper-triangular h[:k, :k] c = g[:k] (the Givens-reduced
    Hessenberg system) row by row from the bottom, float64 operation for
    operation as the library's step driver does."""
    c = np.zeros(k)
    for i in range(k-1, -1, -1):
        acc = g[i]
        for col in range(i+1, k):
            acc -= h[i, col]*c[col]
        c[i] = acc/h[i, i]
    return c


def fgmres(operator, rhs, precondition, tolerance=1e-6, restart=32, max_iterations=256, *, workspace=None,
           strict=True, rhs_norm=None):
    """Right-preconditioned flexible GMRES with CGS2 Arnoldi on CUDA tensors.

    Same signature, iteration and stopping rules as the reference
    (``experiments/bonded_dem_newton.py:13-60``); the Arnoldi
    orthogonalisation, row combination and norms run in library kernels and
    the (restart+1) x restart Hessenberg/Givens recurrence stays on the host,
    read back once per Arnoldi step as in the reference.  ``strict=False``
    returns the last iterate (with ``converged=False`` in the info) instead of
    raising when the iteration budget runs out.  ``rhs_norm``: the float64
    2-norm of ``rhs`` when the caller already holds it (saves one device read).
    """
    lib = _lib.load()
    device = rhs.device
    stream = torch.cuda.current_stream(device).cuda_stream
    shape = rhs.shape
    b = rhs.reshape(-1).to(F64).contiguous()
    length = b.numel()
    partials = torch.zeros(lib.dpf_partials_doubles(), dtype=F64, device=device)
    scal = torch.zeros(2, dtype=F64, device=device)

    def norm_of(v):
        _lib.check(lib.dpf_dot_norm(length, v.data_ptr(), None, scal.data_ptr(), partials.data_ptr(), stream),
                   'dpf_dot_norm')
        return float(scal[1])

    norm = norm_of(b) if rhs_norm is None else float(rhs_norm)
    x = torch.zeros_like(b)
    if norm == 0:
        return x.reshape(shape), dict(iterations=0, relative_residual=0.)
    residual = b.clone(); iterations = 0
    relative = float('nan')
    residual_norm = norm      # the first cycle starts from x = 0
    while iterations < max_iterations:
        width = min(restart, max_iterations - iterations)
        ws = workspace if (workspace is not None and workspace.width >= width and workspace.length == length) \
            else _Krylov(length, width, device)
        h = np.zeros((width+1, width)); cs, sn = np.zeros(width), np.zeros(width)
        g = np.zeros(width+1); g[0] = residual_norm if residual_norm is not None else norm_of(residual)
        residual_norm = None
        _lib.check(lib.dpf_axpby(length, 1./g[0], residual.data_ptr(), 0., residual.data_ptr(),
                                 ws.basis[0].data_ptr(), stream), 'dpf_axpby')
        for j in range(width):
            z = precondition(ws.basis[j].reshape(shape)).reshape(-1).to(F64).contiguous()
            _lib.check(lib.dpf_axpby(length, 1., z.data_ptr(), 0., z.data_ptr(), ws.transformed[j].data_ptr(),
                                     stream), 'dpf_axpby')
            w = operator(ws.transformed[j].reshape(shape)).reshape(-1).to(F64).contiguous()
            if w.data_ptr() == ws.transformed[j].data_ptr():
                w = w.clone()
            _lib.check(lib.dpf_arnoldi_cgs2(length, ws.basis.data_ptr(), length, j, w.data_ptr(), ws.h.data_ptr(),
                                            partials.data_ptr(), stream), 'dpf_arnoldi_cgs2')
            column = ws.h[:j+2].cpu().numpy()
            h[:j+1, j] = column[:j+1]
            h[j+1, j] = column[j+1]
            breakdown = h[j+1, j] < 1e-14
            for k in range(j):
                h[k, j], h[k+1, j] = cs[k]*h[k, j] + sn[k]*h[k+1, j], -sn[k]*h[k, j] + cs[k]*h[k+1, j]
            denominator = np.hypot(h[j, j], h[j+1, j])
            if denominator == 0:
                raise SubdivideError('Subdivide: singular Newton linear system')
            cs[j], sn[j] = h[j, j]/denominator, h[j+1, j]/denominator
            h[j, j], h[j+1, j] = denominator, 0.
            g[j+1], g[j] = -sn[j]*g[j], cs[j]*g[j]
            iterations += 1
            if abs(g[j+1]) <= tolerance*norm or breakdown or j+1 == width:
                coefficients = _back_substitute(h, g, j+1)
                _lib.check(lib.dpf_combine_rows(length, ws.transformed.data_ptr(), length, j+1,
                                                coefficients.ctypes.data_as(ctypes.POINTER(ctypes.c_double)),
                                                x.data_ptr(), stream), 'dpf_combine_rows')
                ax = operator(x.reshape(shape)).reshape(-1).to(F64).contiguous()
                _lib.check(lib.dpf_axpby(length, 1., b.data_ptr(), -1., ax.data_ptr(), residual.data_ptr(), stream),
                           'dpf_axpby')
                relative = norm_of(residual)/norm
                if relative <= 1.05*tolerance:
                    return x.reshape(shape), dict(iterations=iterations, relative_residual=relative)
                break
    if not strict:
        return x.reshape(shape), dict(iterations=iterations, relative_residual=relative, converged=False)
    raise SubdivideError(f'Subdivide: FGMRES did not converge ({relative:g})')


class NewtonBonds(FiniteBonds):
    """Scaled Newton-FGMRES on the unchanged rate law (drop-in for ``NewtonBonds``
    and ``FastNewtonBonds``, ``experiments/bonded_dem_newton.py:63-201``)."""

    PLUGINS = ('jacobian_vector', 'elastic_precondition', '_diagonal_blocks', 'stiffness')

    def __init__(self, *args, **kwargs):
        super().__init__(*args, **kwargs)
        self._inner = torch.zeros(1, dtype=torch.int32, device=self.device)
        self._inner_host = 0
        self._pcg_workspace = None
        self._barrier = torch.zeros(2, dtype=torch.int32, device=self.device)
        self._krylov = None
        self.block = None
        self.units = None
        # Optional {name: [(start_event, end_event), ...]} timing of the hot launches.
        self.profile = None

    def _timed(self, key, fn):
        if self.profile is None:
            return fn()
        start, end = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        start.record()
        out = fn()
        end.record()
        self.profile.setdefault(key, []).append((start, end))
        return out

    # inner_iterations accumulates on the device; reading it synchronises.
    @property
    def inner_iterations(self):
        return self._inner_host + int(self._inner.item())

    @inner_iterations.setter
    def inner_iterations(self, value):
        self._inner.zero_()
        self._inner_host = int(value)

    def _overridden(self, name):
        return name in self.__dict__

    @torch.no_grad()
    def midpoint_force(self, y):
        """Midpoint force of the trial (``bonded_dem_newton.py:64-81``)."""
        return self.trial(y, _check=False)['force']

    @torch.no_grad()
    def residual(self, y, dt, external):
        """``bonded_dem_newton.py:83-86``."""
        y, v, ext = self._vec(y), self._vec(self.v), self._vec(external)
        r = torch.empty_like(y)
        self._status.zero_()
        self._call('dpf_residual', ctypes.byref(self._graph), ctypes.byref(self._stiffness_struct()),
                   ctypes.byref(self._history_struct()), y.data_ptr(), v.data_ptr(), ext.data_ptr(),
                   self.mass.data_ptr(), self.fixed.data_ptr(), float(dt), None, None, None, r.data_ptr(), None,
                   None, self._wrench.data_ptr(), self._partials.data_ptr(), self._status.data_ptr(),
                   self._stream())
        self._raise_status()
        return r

    @torch.no_grad()
    def jacobian_vector(self, y, direction, dt, external):
        """J d of the midpoint residual (``bonded_dem_newton.py:88-92``,
        ``bonded_dem_jvp_warp.py:45-116``)."""
        return self._jvp(self._vec(y), self._vec(direction), dt)

    def _jvp(self, y, direction, dt, units=None, preconditioner=None):
        out = torch.empty_like(direction)
        self._timed('jvp', lambda: self._call('dpf_jacobian_vector', ctypes.byref(self._graph), ctypes.byref(self._stiffness_struct()),
                   ctypes.byref(self._history_struct()), y.data_ptr(), direction.data_ptr(), self.mass.data_ptr(),
                   self.fixed.data_ptr(), float(dt), _addr(units), _addr(preconditioner), out.data_ptr(),
                   self._wrench.data_ptr(), self._stream()))
        return out

    @torch.no_grad()
    def prepare_scaling(self, trial, dt):
        """Block scaling of the Newton system (``bonded_dem_newton.py:94-102``)."""
        self.n, self.ri, self.rj = trial['n'], trial['ri'], trial['rj']
        if self._overridden('_diagonal_blocks'):
            self.diagonal = self._diagonal_blocks()
            self.block = torch.diag_embed(self.mass) + .25*dt*dt*self.diagonal
            self.block[self.fixed] = torch.eye(6, dtype=F64, device=self.device)
            self.preconditioner = torch.linalg.inv(self.block)
            self.units = torch.ones_like(self.mass)
            self.units[:, :3] = self.radii[:, None]
            self.units[self.fixed] = 1.
            return
        n = self.n_sites
        if self.block is None or self.block.shape[0] != n:
            self.diagonal = torch.empty((n, 6, 6), dtype=F64, device=self.device)
            self.block = torch.empty_like(self.diagonal)
            self.preconditioner = torch.empty_like(self.diagonal)
            self.units = torch.empty_like(self.mass)
        self._call('dpf_prepare_scaling', ctypes.byref(self._graph), ctypes.byref(self._stiffness_struct()),
                   ctypes.byref(self._tangent_struct()), self.mass.data_ptr(), self.fixed.data_ptr(),
                   self.radii.data_ptr(), float(dt), self.diagonal.data_ptr(), self.block.data_ptr(),
                   self.preconditioner.data_ptr(), self.units.data_ptr(), self._stream())

    @torch.no_grad()
    def scale_residual(self, r):
        """P r / units (``bonded_dem_newton.py:104-105``)."""
        r = self._vec(r)
        out = torch.empty_like(r)
        self._call('dpf_scale_residual', self.n_sites, self.preconditioner.data_ptr(), self.units.data_ptr(),
                   r.data_ptr(), out.data_ptr(), None, None, self._stream())
        return out

    @torch.no_grad()
    def elastic_precondition(self, vector, dt, tolerance=.03, max_iterations=80):
        """Block-Jacobi PCG on M + dt^2/4 K (``bonded_dem_newton.py:107-130``,
        ``bonded_dem_precondition_warp.py:127-151``), one cooperative launch."""
        vector = self._vec(vector)
        if self._overridden('stiffness'):
            return self._elastic_precondition_generic(vector, dt, tolerance, max_iterations)
        if self._pcg_workspace is None:
            self._pcg_workspace = torch.empty(self._lib.dpf_elastic_workspace_doubles(self.n_sites), dtype=F64,
                                              device=self.device)
        out = torch.empty_like(vector)
        self._timed('pcg', lambda: self._call('dpf_elastic_precondition', ctypes.byref(self._graph), ctypes.byref(self._stiffness_struct()),
                   ctypes.byref(self._tangent_struct()), self.mass.data_ptr(), self.fixed.data_ptr(),
                   self.block.data_ptr(), self.preconditioner.data_ptr(), self.units.data_ptr(), vector.data_ptr(),
                   float(dt), float(tolerance), int(max_iterations), out.data_ptr(), self._inner.data_ptr(),
                   self._wrench.data_ptr(), self._pcg_workspace.data_ptr(), self._barrier.data_ptr(),
                   self._status.data_ptr(), self._stream()))
        return out

    def _elastic_precondition_generic(self, vector, dt, tolerance, max_iterations):
        """The elastic PCG with K q from an instance ``stiffness`` plug-in: the
        recurrence and stopping rule of the library kernel, driven from the
        host with one plug-in K q per iteration."""
        def blocks(matrices, v):
            return (matrices @ v.unsqueeze(-1)).squeeze(-1)

        def inner(a, b):
            return torch.dot(a.reshape(-1), b.reshape(-1))
        b = torch.where(self.fixed[:, None], 0., blocks(self.block, self.units*vector))
        x = torch.zeros_like(b)
        r, z = b, blocks(self.preconditioner, b)
        p, gamma = z, inner(b, z)
        gamma0 = float(gamma)
        if gamma0 == 0:
            return x
        done = max_iterations
        for k in range(max_iterations):
            w = self._operator(p, .25*dt*dt)
            step = gamma/inner(p, w)
            x, r = x + step*p, r - step*w
            z = blocks(self.preconditioner, r)
            gamma_next = inner(r, z)
            if k % 5 == 0 and float(gamma_next) <= tolerance*tolerance*gamma0:
                done = k + 1
                break
            p, gamma = z + (gamma_next/gamma)*p, gamma_next
        self._inner_host += done
        return x/self.units

    # ---- the Newton step ---------------------------------------------------
    def _evaluate(self, y, dt, external, tangent_out=None, scaled=None):
        """Residual at y with every trial guard (status in self._status)."""
        r = torch.empty_like(y)
        self._status.zero_()
        use_p = tangent_out is None
        self._timed('residual', lambda: self._call(
            'dpf_residual', ctypes.byref(self._graph), ctypes.byref(self._stiffness_struct()),
            ctypes.byref(self._history_struct()), y.data_ptr(), self._v.data_ptr(), external.data_ptr(),
            self.mass.data_ptr(), self.fixed.data_ptr(), float(dt),
            ctypes.byref(self._trial_struct(tangent_out, end=False)) if tangent_out else None,
            self.preconditioner.data_ptr() if use_p else None, self.units.data_ptr() if use_p else None,
            r.data_ptr(), _addr(scaled) if use_p else None, self._scalars.data_ptr() if use_p else None,
            self._wrench.data_ptr(), self._partials.data_ptr(), self._status.data_ptr(), self._stream()))
        return r

    # Precision-specific stages of step(); the control flow in step() is the
    # reference's (bonded_dem_newton.py:132-201).
    def _step_begin(self, dt, external):
        """rhs_scale of the step (bonded_dem_newton.py:138-139)."""
        loads = self.loads()
        self._call('dpf_rhs_scale', self.n_sites, self.mass.data_ptr(), self._v.data_ptr(), external.data_ptr(),
                   loads.data_ptr(), self.fixed.data_ptr(), dt, self._scalars.data_ptr(), self._partials.data_ptr(),
                   self._stream())
        (a, l), _ = self._fetch(2)
        return max(a, .5*dt*dt*l, 1e-30)

    def _iteration_residual(self, y, dt, external):
        """trial + prepare_scaling + residual + scaling at the iterate; returns
        (scaled residual, [|r|, max|s|, |s|]) and raises on a trial guard."""
        m = self.n_bonds
        tangent = dict(force=None, n=torch.empty((m, 3), dtype=F64, device=self.device),
                       ri=torch.empty((m, 3), dtype=F64, device=self.device),
                       rj=torch.empty((m, 3), dtype=F64, device=self.device))
        r = self._evaluate(y, dt, external, tangent_out=tangent)
        _, status = self._fetch(status=True)
        if status:
            raise guard_error(status)
        self.prepare_scaling(tangent, dt)
        scaled = torch.empty_like(r)
        self._call('dpf_scale_residual', self.n_sites, self.preconditioner.data_ptr(), self.units.data_ptr(),
                   r.data_ptr(), scaled.data_ptr(), self._scalars.data_ptr(), self._partials.data_ptr(),
                   self._stream())
        norms, _ = self._fetch(3)
        return scaled, norms

    def _newton_operator(self, y, dt, external):
        units, pre = self.units, self.preconditioner
        if self._overridden('jacobian_vector'):
            return lambda v: self.scale_residual(self.jacobian_vector(y, units*v, dt, external))
        return lambda v: self._jvp(y, self._vec(v), dt, units=units, preconditioner=pre)

    def _newton_preconditioner(self, dt):
        return lambda v: self.elastic_precondition(v, dt)

    def _line_merit(self, candidate, dt, external):
        """|P r(candidate) / units| and the guard status (one device sync)."""
        self._evaluate(candidate, dt, external)
        (_, _, value), status = self._fetch(3, status=True)
        return value, status

    def _accept(self, y, dt):
        """Commit the trial at y and update velocity and rotation (bonded_dem_newton.py:149-154)."""
        state = self.trial(y)
        rotation = self._vec(self.rotation).clone()
        self._call('dpf_accept_step', self.n_sites, y.data_ptr(), dt, self._v.data_ptr(), rotation.data_ptr(),
                   self._stream())
        self.commit(state)
        self.v, self.rotation = self._v, rotation

    def _krylov_solve(self, operator, rhs, precondition, tolerance, rhs_norm, dt):
        """FGMRES on the scaled Newton system (``bonded_dem_newton.py:160-162``)."""
        return fgmres(operator, rhs, precondition, tolerance=tolerance, workspace=self._krylov, rhs_norm=rhs_norm)

    def _dense_direction(self, operator, scaled):
        """Newton direction of the 'dense' backend (``bonded_dem_newton.py:163-175``):
        the scaled Jacobian restricted to the free DOFs is built one unit
        column at a time through ``operator`` and solved by LU."""
        free = (~self.fixed)[:, None].expand(-1, 6).reshape(-1)
        index = free.nonzero().reshape(-1)
        size = int(index.numel())
        if size > 400:
            raise ValueError('Dense reference limited to 400 free DOFs')
        n6 = 6*self.n_sites
        jacobian = torch.empty((size, size), dtype=F64, device=self.device)
        unit = torch.zeros(n6, dtype=F64, device=self.device)
        for column, dof in enumerate(index.tolist()):
            unit[dof] = 1.
            jacobian[:, column] = operator(unit.view(-1, 6)).reshape(-1).index_select(0, index)
            unit[dof] = 0.
        delta = torch.zeros(n6, dtype=F64, device=self.device)
        delta.index_copy_(0, index, torch.linalg.solve(jacobian, -scaled.reshape(-1).index_select(0, index)))
        return delta.view(-1, 6)

    @torch.no_grad()
    def step(self, dt, external, tolerance=2e-7, max_iterations=12, *,
             pose_tolerance=2e-6, backend='fgmres', linear_tolerance=1e-6,
             preconditioning='elastic'):
        """Line-searched Newton on the implicit-midpoint residual (``bonded_dem_newton.py:132-201``)."""
        if not np.isfinite(dt) or dt <= 0:
            raise ValueError('Positive finite dt required')
        dt = float(dt)
        external = self._vec(external)
        self._v = self._vec(self.v).clone()
        y = torch.zeros_like(self._v)
        stream = self._stream()
        rhs_scale = self._step_begin(dt, external)    # a number, or a callable read after the first fetch
        krylov = 0
        self.inner_iterations = 0
        residual_trace = []
        relative = local = float('nan')
        n6 = 6*self.n_sites
        for iteration in range(max_iterations+1):
            scaled, (rnorm, local, merit) = self._iteration_residual(y, dt, external)
            if callable(rhs_scale):
                rhs_scale = rhs_scale()
            relative = rnorm/rhs_scale
            if not np.isfinite(relative) or not np.isfinite(local):
                raise SubdivideError(f'Subdivide: non-finite Newton residual ({relative:g}, {local:g})')
            residual_trace.append([relative, local])
            if relative < tolerance and local < pose_tolerance:
                self._accept(y, dt)
                self.time += dt
                self._call('dpf_dot_norm', n6, external.data_ptr(), y.data_ptr(), self._scalars.data_ptr(),
                           self._partials.data_ptr(), stream)
                if len(y):
                    self._scalars[2:3].copy_(torch.linalg.vector_norm(y[:, 3:], dim=1).max().reshape(1))
                self._scalars[3:4].copy_(self._inner)   # the device CG count rides along
                (work, _, max_rotation, inner), _ = self._fetch(4)
                return work, dict(nonlinear_iterations=iteration, nonlinear_relative_residual=relative,
                                  local_pose_defect=local, krylov_iterations=krylov,
                                  cg_iterations=self._inner_host + int(inner), residual_trace=residual_trace,
                                  max_step_rotation=max_rotation)
            if iteration == max_iterations:
                break
            operator = self._newton_operator(y, dt, external)
            if backend == 'dense':
                delta = self._dense_direction(operator, scaled)
            elif backend == 'fgmres':
                if preconditioning == 'elastic':
                    precondition = self._newton_preconditioner(dt)
                elif preconditioning == 'block':
                    precondition = (lambda v: v)
                else:
                    raise ValueError(preconditioning)
                if self._krylov is None or self._krylov.length != n6:
                    self._krylov = _Krylov(n6, 32, self.device)
                rhs = torch.empty_like(scaled)
                self._call('dpf_axpby', n6, -1., scaled.data_ptr(), 0., scaled.data_ptr(), rhs.data_ptr(), stream)
                # rhs = -scaled, whose float64 norm the residual pass returned (merit)
                delta, metrics = self._krylov_solve(operator, rhs, precondition, linear_tolerance, merit, dt)
                krylov += metrics['iterations']
            else:
                raise ValueError(backend)
            delta = self._vec(delta)
            correction = torch.empty_like(delta)
            self._call('dpf_masked_scale', self.n_sites, delta.data_ptr(), self.units.data_ptr(),
                       self.fixed.data_ptr(), correction.data_ptr(), stream)
            accepted = False
            candidate = torch.empty_like(y)
            for power in range(10):
                factor = 2.**(-power)
                self._call('dpf_axpby', n6, 1., y.data_ptr(), factor, correction.data_ptr(), candidate.data_ptr(),
                           stream)
                value, status = self._line_merit(candidate, dt, external)
                if status:
                    continue
                if value < (1 - 1e-4*factor)*merit:
                    y = candidate; accepted = True; break
            if not accepted:
                raise SubdivideError('Subdivide: Newton line search failed')
        raise SubdivideError(f'Subdivide: Newton did not converge ({relative:g}, {local:g})')


FastNewtonBonds = NewtonBonds


_HISTORY = ('x', 'normal', 'offset', 'fn', 'fs', 'mt', 'mb')


def _history_property(name):
    key = '_h_' + name

    def get(self):
        if name != 'x' and self.__dict__.get('_pending_fold'):
            self._fold_history()
        return self.__dict__[key]

    def put(self, value):
        if self.__dict__.get('_pending_fold'):
            self._fold_history()
        self.__dict__[key] = value
    return property(get, put, doc=f'Committed {name} (float64; pending step increments are folded in on access).')


class AdaptiveIntervals:
    """Interval controller that keeps the subdivision depth which last worked
    (``experiments/bonded_dem_adaptive.py:4-23``): an interval is advanced as
    2^depth equal pieces, each bisected further on demand; the deepest piece
    sets the next depth, and after ``coarsen_after`` consecutive easy
    intervals (no piece needed more than ``easy_newton`` Newton iterations)
    the depth drops by one."""

    coarsen_after = 8
    easy_newton = 3

    def __init__(self, solver):
        self.solver = solver
        self.depth = 0
        self.easy_intervals = 0

    def advance(self, dt, load):
        pieces = 1 << self.depth
        results = [self.solver.advance_interval(dt/pieces, load, depth=self.depth) for _ in range(pieces)]
        records = [record for _, part in results for record in part]
        self._remember(records)
        return sum(value for value, _ in results), records

    def _remember(self, records):
        self.depth = max(record['subdivision_depth'] for record in records)
        easy = all(record['nonlinear_iterations'] <= self.easy_newton for record in records)
        self.easy_intervals = self.easy_intervals + 1 if easy else 0
        if self.depth and self.easy_intervals >= self.coarsen_after:
            self.depth, self.easy_intervals = self.depth - 1, 0


class MixedNewtonBonds(NewtonBonds):
    """Mixed-precision form of ``NewtonBonds.step``: the same equations, control
    flow, tolerances and ``info`` as the reference solver
    (``experiments/bonded_dem_newton.py:132-201``) with float32 bond sweeps
    (residual increment, JVP, K q, 6x6 blocks, elastic PCG), float64
    reductions and Krylov vectors, and a float64-accurate residual:
    r(y) = r0 + M y - dt^2/2 sum of float32 bond increments, with r0 computed
    in float64 once per step and site sums compensated.  The accepted line-search
    evaluation (with its tangent) is reused as the next iteration's residual,
    as the reference's next trial at the same increment gives the same values.
    Every other method is the float64 one it inherits.

    The JVP is a float32 operator (relative accuracy ~1e-7), so FGMRES cannot
    certify linear tolerances below ``min_linear_tolerance`` (1e-6): smaller
    requests are raised to it.  The float64-accurate nonlinear residual still
    decides convergence of the step.
    """

    min_linear_tolerance = 1e-6
    # Steps between float64 rebuilds of the bond records and committed loads
    # (in between they are advanced by the commit's float32 increments).
    refresh_interval = 32
    # Operator sweep of the elastic PCG (one cooperative launch, two grid
    # barriers per iteration): 'ends' -- bond ends over the site-sorted
    # incidence CSR, lanes of a site sum in registers; 'tiles' -- site tiles
    # staged in shared memory (tile size and CTA width autotuned at the first
    # use); 'bonds' -- a bond pass and a site gather through HBM per iteration.
    sweep = 'ends'

    # Drive eligible steps (bond-end sweep, FGMRES, elastic preconditioning, no
    # overridden hook) from the library's host step driver: the same launches
    # and decisions as the Python control path, bit for bit, without Python
    # between the launches.  False keeps every step on the Python path.
    native = True

    # the hooks the native driver replaces; a subclass that overrides one keeps the Python path
    _NATIVE_HOOKS = ('_step_begin', '_iteration_residual', '_mixed_residual', '_newton_operator',
                     '_newton_preconditioner', '_line_merit', '_accept', '_bond_mask', '_site_mask', '_end_pcg',
                     '_pack_ends', 'step', '_native_step')

    def step(self, dt, external, tolerance=2e-7, max_iterations=12, *, pose_tolerance=2e-6, backend='fgmres',
             linear_tolerance=1e-6, preconditioning='elastic'):
        linear_tolerance = max(linear_tolerance, self.min_linear_tolerance)
        if self._native_ready(backend, preconditioning):
            return self._native_step(dt, external, tolerance, max_iterations, pose_tolerance, linear_tolerance)
        return super().step(dt, external, tolerance, max_iterations, pose_tolerance=pose_tolerance, backend=backend,
                            linear_tolerance=linear_tolerance, preconditioning=preconditioning)

    def _native_ready(self, backend, preconditioning):
        if not (self.native and backend == 'fgmres' and preconditioning == 'elastic' and self.sweep == 'ends'):
            return False
        if self._end_variant is None or self._ends is None or not self._sweep_ready:
            return False        # the first step runs in Python: it autotunes the sweep's launch shape
        cls = type(self)
        return all(getattr(cls, name) is getattr(MixedNewtonBonds, name) for name in self._NATIVE_HOOKS)

    def _native_buffers(self):
        """Descriptor of this solver's buffers for ``dpf_mixed_newton_step`` (cached
        while the tensors it points to stay the same)."""
        key = tuple(t.data_ptr() for t in (self.mass, self.fixed, self.radii, self.kn, self.ks, self.kb, self.kt,
                                           self._ends, self._p32)) + (self._end_variant, self.lazy_history)
        cached = getattr(self, '_native_desc', None)
        if cached is not None and cached[0] == key:
            return cached[1]
        n, dev, lib = self.n_sites, self.device, self._lib
        ws = self._krylov_workspace32()
        if getattr(self, '_native_vectors', None) is None:
            # the second scaling set (a line-search candidate's blocks, inverses and units)
            self._scaling_b = (torch.empty_like(self._block32), torch.empty_like(self._p32),
                               torch.empty_like(self._units), torch.empty_like(self._units32))
            self._native_vectors = torch.empty((_lib.NEWTON_VECTORS, n, 6), dtype=F64, device=dev)
            self._native_partials = torch.zeros(lib.dpf_partials_doubles(), dtype=F64, device=dev)
            self._native_scalars = torch.zeros(2, dtype=F64, device=dev)
            self._native_host = torch.zeros(_lib.NEWTON_HOST_DOUBLES, dtype=F64).pin_memory()
        for name in ('mass', 'fixed', 'radii'):
            t = getattr(self, name)
            if not t.is_contiguous():
                setattr(self, name, t.contiguous())
        ptr = lambda t: t.data_ptr()
        desc = _lib.MixedNewton(
            graph=ctypes.addressof(self._graph), stiffness=self._stiffness_struct(), radii=ptr(self.radii),
            mass=ptr(self.mass), mass32=ptr(self._mass32), fixed=ptr(self.fixed), bond_data=ptr(self._bond_data),
            r0=ptr(self._r0), loads=ptr(self._loads), scales=ptr(self._begin_scales), wrench64=ptr(self._wrench),
            partials=ptr(self._partials), scalars=ptr(self._scalars), status=ptr(self._status), y32=ptr(self._y32),
            d32=ptr(self._d32), wrench32=ptr(self._wrench32), block32=ptr(self._block32), p32=ptr(self._p32),
            units=ptr(self._units), units32=ptr(self._units32), block32_b=ptr(self._scaling_b[0]),
            p32_b=ptr(self._scaling_b[1]), units_b=ptr(self._scaling_b[2]), units32_b=ptr(self._scaling_b[3]),
            ends=ptr(self._ends), site4=ptr(self._site4),
            p24=ptr(self._p24), end_workspace=ptr(self._tiled_workspace), end_partials=ptr(self._tiled_partials),
            barrier=ptr(self._barrier), inner=ptr(self._inner), basis=ptr(ws.basis),
            transformed=ptr(ws.transformed), products=ptr(ws.products), w32=ptr(ws.w), h=ptr(ws.h),
            krylov_width=ws.width,
            krylov_partials=ptr(self._native_partials), krylov_scalars=ptr(self._native_scalars),
            vectors=ptr(self._native_vectors), host=ptr(self._native_host), end_variant=int(self._end_variant),
            history_corrections=ptr(self._history_corrections()) if self.lazy_history else None)
        # the descriptor holds only addresses: keep what they point into alive with it
        self._native_desc = (key, desc, ws)
        return desc

    def _krylov_workspace32(self):
        ws = getattr(self, '_krylov32', None)
        if ws is None or ws.length != 6*self.n_sites:
            ws = self._krylov32 = _Krylov32(6*self.n_sites, 32, self.device)
        return ws

    def _krylov_solve(self, operator, rhs, precondition, tolerance, rhs_norm, dt):
        cls = type(self)
        if self.sweep == 'ends' and cls._newton_operator is MixedNewtonBonds._newton_operator and \
                cls._newton_preconditioner is MixedNewtonBonds._newton_preconditioner:
            return self._fgmres32(rhs, tolerance, rhs_norm, dt)
        return super()._krylov_solve(operator, rhs, precondition, tolerance, rhs_norm, dt)

    def _fgmres32(self, b, tolerance, norm, dt, restart=32, max_iterations=256):
        """``fgmres`` with float32 Krylov vectors: the elastic PCG and the JVP read
        and write float32 rows (their values carry float32 precision either
        way), the Arnoldi sums are exact float32 pairs with float64 partials
        and h, and x, b and the true residual stay float64.  The Hessenberg
        recurrence, stopping rules and restarts are those of ``fgmres``
        (``bonded_dem_newton.py:13-60``), except that the true residual's J x
        is sum_k c_k J z_k from the kept products (J is linear; the reference
        applies the operator to x once more, a fourth JVP per two Arnoldi
        steps).  The library's step driver runs the same launches."""
        lib, stream = self._lib, self._stream()
        n6 = 6*self.n_sites
        ws = self._krylov_workspace32()
        b = b.reshape(-1)
        x, res = ws.x, ws.residual
        x.zero_()
        if norm == 0:
            return x.view(-1, 6), dict(iterations=0, relative_residual=0.)

        def norm_of(v):
            self._call('dpf_dot_norm', n6, v.data_ptr(), None, ws.scalars.data_ptr(), ws.partials.data_ptr(),
                       stream)
            return float(ws.scalars[1])

        iterations, relative, first = 0, float('nan'), True
        while iterations < max_iterations:
            width = min(restart, max_iterations - iterations)
            h = np.zeros((width+1, width)); cs, sn = np.zeros(width), np.zeros(width)
            g = np.zeros(width+1)
            g[0] = norm if first else norm_of(res)
            start = b if first else res
            first = False
            self._call('dpf_scale_to_float', n6, 1./g[0], start.data_ptr(), ws.basis[0].data_ptr(), stream)
            for j in range(width):
                bj, tj, pj = ws.basis[j], ws.transformed[j], ws.products[j]
                if self._packed != ('ends', dt):     # at the first PCG of a tangent, as the step driver does
                    self._pack_ends(dt)
                if self._end_variant is None:
                    from .tiles import tune_end_sweep
                    self._end_variant = tune_end_sweep(self, b.view(-1, 6), nearest=self._tune_nearest)
                self._timed('pcg', lambda: self._call(
                    'dpf_end_precondition_f32', ctypes.byref(self._graph), self._ends.data_ptr(),
                    self._site4.data_ptr(), self.fixed.data_ptr(), self._block32.data_ptr(), self._p24.data_ptr(),
                    self._units32.data_ptr(), bj.data_ptr(), .03, 80, tj.data_ptr(), self._inner.data_ptr(),
                    self._tiled_workspace.data_ptr(), self._tiled_partials.data_ptr(), self._barrier.data_ptr(),
                    self._status.data_ptr(), int(self._end_variant), stream))
                self._timed('jvp', lambda: self._call(
                    'dpf_mixed_jacobian_vector_f32', ctypes.byref(self._graph), self._bond_data.data_ptr(),
                    self._y32.data_ptr(), tj.data_ptr(), self._mass32.data_ptr(), self.fixed.data_ptr(), dt,
                    self._units32.data_ptr(), self._p32.data_ptr(), pj.data_ptr(), self._d32.data_ptr(),
                    self._wrench32.data_ptr(), stream))
                self._call('dpf_arnoldi_cgs2_f32', n6, ws.basis.data_ptr(), n6, j, pj.data_ptr(), ws.w.data_ptr(),
                           ws.h.data_ptr(), ws.partials.data_ptr(), self._barrier.data_ptr(),
                           self._status.data_ptr(), stream)
                column = ws.h[:j+2].cpu().numpy()
                h[:j+1, j] = column[:j+1]
                h[j+1, j] = column[j+1]
                breakdown = h[j+1, j] < 1e-14
                for k in range(j):
                    h[k, j], h[k+1, j] = cs[k]*h[k, j] + sn[k]*h[k+1, j], -sn[k]*h[k, j] + cs[k]*h[k+1, j]
                denominator = np.hypot(h[j, j], h[j+1, j])
                if denominator == 0:
                    raise SubdivideError('Subdivide: singular Newton linear system')
                cs[j], sn[j] = h[j, j]/denominator, h[j+1, j]/denominator
                h[j, j], h[j+1, j] = denominator, 0.
                g[j+1], g[j] = -sn[j]*g[j], cs[j]*g[j]
                iterations += 1
                if abs(g[j+1]) <= tolerance*norm or breakdown or j+1 == width:
                    coefficients = _back_substitute(h, g, j+1)
                    c = coefficients.ctypes.data_as(ctypes.POINTER(ctypes.c_double))
                    self._call('dpf_combine_rows_f32', n6, ws.transformed.data_ptr(), n6, j+1, c, x.data_ptr(),
                               stream)
                    ax = ws.product
                    ax.zero_()
                    self._call('dpf_combine_rows_f32', n6, ws.products.data_ptr(), n6, j+1, c, ax.data_ptr(), stream)
                    self._call('dpf_axpby', n6, 1., b.data_ptr(), -1., ax.data_ptr(), res.data_ptr(), stream)
                    relative = norm_of(res)/norm
                    if relative <= 1.05*tolerance:
                        return x.view(-1, 6), dict(iterations=iterations, relative_residual=relative)
                    break
        raise SubdivideError(f'Subdivide: FGMRES did not converge ({relative:g})')

    @torch.no_grad()
    def _native_step(self, dt, external, tolerance, max_iterations, pose_tolerance, linear_tolerance):
        """``step`` through ``dpf_mixed_newton_step``: one library call per step
        (the host work around it is kept small: the GPU idles meanwhile)."""
        if not (dt > 0 and np.isfinite(dt)):
            raise ValueError('Positive finite dt required')
        dt = float(dt)
        external = self._vec(external)
        v0, r0 = self._vec(self.v), self._vec(self.rotation)
        self._v, rotation = torch.empty_like(v0), torch.empty_like(r0)   # the driver copies the start values in
        if getattr(self, '_begin_scales', None) is None:
            self._begin_scales = torch.zeros(2, dtype=F64, device=self.device)
        self._cached = None
        refresh = not (self._token is not None and self._since_refresh < self.refresh_interval and
                       self._token == self._state_token())
        if refresh:
            self._since_refresh = 0
        # a float64 setup reads the whole (folded) history; the lazy commit only x
        history = self._history_struct() if (refresh or not self.lazy_history) else self._stored_history()
        desc = self._native_buffers()
        m, n = self.n_bonds, self.n_sites
        e = lambda *shape: torch.empty(shape, dtype=F64, device=self.device)
        if self.lazy_history:
            state = dict(x=e(n, 3))
            ends = (None,)*6
        else:
            state = dict(x=e(n, 3), normal=e(m, 3), offset=e(m, 3), fn=e(m), fs=e(m, 3), mt=e(m), mb=e(m, 3))
            ends = tuple(state[k].data_ptr() for k in ('normal', 'offset', 'fn', 'fs', 'mt', 'mb'))
        timing = self.profile is not None
        args = self.__dict__.get('_native_args')
        if args is None:
            args = self._native_args = _lib.NewtonStep()
            self._native_info = _lib.NewtonInfo()
        args.dt, args.external, args.v, args.rotation, args.history = \
            dt, external.data_ptr(), self._v.data_ptr(), rotation.data_ptr(), history
        args.x_end = state['x'].data_ptr()
        args.normal_end, args.offset_end, args.fn_end, args.fs_end, args.mt_end, args.mb_end = ends
        args.tolerance, args.pose_tolerance, args.linear_tolerance = float(tolerance), float(pose_tolerance), \
            float(linear_tolerance)
        args.max_iterations, args.refresh, args.timing = int(max_iterations), int(refresh), int(timing)
        args.v_in, args.rotation_in = v0.data_ptr(), r0.data_ptr()
        args.committed_start = int(self.__dict__.get('_committed_start', False) and not refresh)
        self._committed_start = False      # until this step commits
        info = self._native_info
        self._inner_host = 0
        self._call('dpf_mixed_newton_step', ctypes.byref(desc), ctypes.byref(args), ctypes.byref(info),
                   self._stream())
        _lib.LAUNCHES['count'] += info.launches
        if info.scaling_alternate:      # the last scaling went to the second set: it is now the first
            b = self._scaling_b
            self._scaling_b = (self._block32, self._p32, self._units, self._units32)
            self._block32, self._p32, self._units, self._units32 = b
        self.units = self._units
        self._packed = None
        if timing:
            for k, key in enumerate(_lib.NEWTON_TIMERS):
                count = info.timed_launches[k]
                if count:
                    self.profile.setdefault(key, []).extend([info.time_ms[k]/count]*count)
        relative, local = info.relative, info.local
        outcome = info.outcome
        if outcome == _lib.NEWTON_GUARD:
            raise guard_error(info.guard)
        if outcome == _lib.NEWTON_NONFINITE:
            raise SubdivideError(f'Subdivide: non-finite Newton residual ({relative:g}, {local:g})')
        if outcome == _lib.NEWTON_SINGULAR:
            raise SubdivideError('Subdivide: singular Newton linear system')
        if outcome == _lib.NEWTON_KRYLOV:
            raise SubdivideError(f'Subdivide: FGMRES did not converge ({info.krylov_relative:g})')
        if outcome == _lib.NEWTON_LINE_SEARCH:
            raise SubdivideError('Subdivide: Newton line search failed')
        if outcome != _lib.NEWTON_CONVERGED:
            raise SubdivideError(f'Subdivide: Newton did not converge ({relative:g}, {local:g})')
        if self.lazy_history:
            self._commit_lazy(state['x'])
        else:
            self.commit(state)
        self.v, self.rotation = self._v, rotation
        self._committed_start = True
        self._token = self._state_token()
        self._since_refresh += 1
        self.time += dt
        trace = [[info.trace[2*k], info.trace[2*k + 1]] for k in range(info.trace_len)]
        return info.work, dict(nonlinear_iterations=info.nonlinear_iterations, nonlinear_relative_residual=relative,
                               local_pose_defect=local, krylov_iterations=info.krylov_iterations,
                               cg_iterations=info.cg_iterations, residual_trace=trace,
                               max_step_rotation=info.max_rotation)

    def __init__(self, *args, **kwargs):
        super().__init__(*args, **kwargs)
        lib, n, m = self._lib, self.n_sites, self.n_bonds
        dev = self.device
        f32 = torch.float32
        self._bond_data = torch.empty(max(4, lib.dpf_mixed_bond_floats(m)), dtype=f32, device=dev)
        self._wrench32 = torch.empty(max(4, lib.dpf_mixed_wrench_floats(m)), dtype=f32, device=dev)
        self._r0 = torch.empty((n, 6), dtype=F64, device=dev)
        self._block32 = torch.empty((n, 6, 6), dtype=f32, device=dev)
        self._p32 = torch.empty((n, 6, 6), dtype=f32, device=dev)
        self._units = torch.empty((n, 6), dtype=F64, device=dev)
        self._units32 = torch.empty((n, 6), dtype=f32, device=dev)
        self._mass32 = torch.empty((n, 6), dtype=f32, device=dev)
        self._y32 = torch.empty((n, 6), dtype=f32, device=dev)
        self._d32 = torch.empty((n, 6), dtype=f32, device=dev)
        self._mixed_workspace = torch.empty(lib.dpf_mixed_workspace_floats(n, m), dtype=f32, device=dev)
        self._call('dpf_to_float', 6*n, self.mass.data_ptr(), self._mass32.data_ptr(), self._stream())
        self._cached = None
        self._loads = torch.empty((n, 6), dtype=F64, device=dev)
        self._token = None
        self._since_refresh = 0
        self._init_tiles()

    def _init_tiles(self):
        self._tiles = None
        self._ends = None
        self._end_variant = None       # launch shape of the bond-end sweep (autotuned at the first PCG)
        self._sweep_ready = False
        self.tile_timings = {}
        self._packed = None

    def _sweep_buffers(self):
        """Packed block inverses, site records and PCG workspace of the 'ends' and
        'tiles' sweeps (allocated at the first use)."""
        if self._sweep_ready:
            return
        n, dev, lib = self.n_sites, self.device, self._lib
        self._site4 = torch.empty((n, 4), dtype=torch.float32, device=dev)
        self._p24 = torch.empty(24*n, dtype=torch.float32, device=dev)
        self._tiled_workspace = torch.empty(lib.dpf_tiled_workspace_floats(n), dtype=torch.float32, device=dev)
        self._tiled_partials = torch.zeros(lib.dpf_tiled_partials_doubles(), dtype=F64, device=dev)
        self._tune_iterations = torch.zeros(1, dtype=torch.int32, device=dev)
        self._sweep_ready = True

    def _pack_ends(self, dt):
        """End records (alpha = dt^2/4 folded in), packed P and site records."""
        self._sweep_buffers()
        if self._ends is None:
            self._ends = torch.empty(max(4, self._lib.dpf_end_floats(self.n_bonds)), dtype=torch.float32,
                                     device=self.device)
        self._call('dpf_end_pack', ctypes.byref(self._graph), self._bond_data.data_ptr(), .25*dt*dt,
                   self._p32.data_ptr(), self._mass32.data_ptr(), self.fixed.data_ptr(), self._ends.data_ptr(),
                   self._p24.data_ptr(), self._site4.data_ptr(), self._stream())
        self._packed = ('ends', dt)

    # size classes an untuned graph may borrow the launch shape from (0: time the shapes)
    _tune_nearest = 0

    def _end_pcg(self, vector, out, tolerance, max_iterations, iterations, variant=None):
        if variant is None:
            if self._end_variant is None:
                from .tiles import tune_end_sweep
                self._end_variant = tune_end_sweep(self, vector, nearest=self._tune_nearest)
            variant = self._end_variant
        self._call('dpf_end_precondition', ctypes.byref(self._graph), self._ends.data_ptr(), self._site4.data_ptr(),
                   self.fixed.data_ptr(), self._block32.data_ptr(), self._p24.data_ptr(), self._units32.data_ptr(),
                   vector.data_ptr(), float(tolerance), int(max_iterations), out.data_ptr(), iterations.data_ptr(),
                   self._tiled_workspace.data_ptr(), self._tiled_partials.data_ptr(), self._barrier.data_ptr(),
                   self._status.data_ptr(), *self._site_mask(), int(variant), self._stream())

    def _site_mask(self):
        """(per-site segment, per-segment active flag) device pointers that let the
        bond-end sweep skip sites of finished segments; (None, None) here."""
        return None, None

    def _pack_tiles(self, tiles, dt):
        """Entry records (alpha = dt^2/4 folded in), packed P and site records for ``tiles``."""
        self._sweep_buffers()
        self._call('dpf_tile_pack', ctypes.byref(tiles.struct), self._bond_data.data_ptr(), self.n_bonds,
                   .25*dt*dt, self._p32.data_ptr(), self._mass32.data_ptr(), self.fixed.data_ptr(), self.n_sites,
                   tiles.entries.data_ptr(), self._p24.data_ptr(), self._site4.data_ptr(), self._stream())
        self._packed = (tiles, dt)

    def _tiled_pcg(self, tiles, vector, out, tolerance, max_iterations, iterations):
        self._call('dpf_tiled_precondition', ctypes.byref(self._graph), ctypes.byref(tiles.struct),
                   tiles.entries.data_ptr(), self._site4.data_ptr(), self.fixed.data_ptr(),
                   self._block32.data_ptr(), self._p24.data_ptr(), self._units32.data_ptr(), vector.data_ptr(),
                   float(tolerance), int(max_iterations), out.data_ptr(), iterations.data_ptr(),
                   self._tiled_workspace.data_ptr(), self._tiled_partials.data_ptr(), self._barrier.data_ptr(),
                   self._status.data_ptr(), tiles.threads, tiles.stages, self._stream())

    def _ensure_tiles(self, dt, vector, tolerance, max_iterations):
        if self._tiles is None:
            from .tiles import autotune
            scratch = torch.empty_like(vector)

            def run(tiles):
                self._pack_tiles(tiles, dt)
                self._tiled_pcg(tiles, vector, scratch, tolerance, max_iterations, self._tune_iterations)
            self._tiles, self.tile_timings = autotune(self, run)
            self._packed = None
        if self._packed != (self._tiles, dt):
            self._pack_tiles(self._tiles, dt)

    def _state_token(self):
        # identity and in-place version of every committed tensor the records
        # depend on (the stored tensors: reading the history would fold it)
        d = self.__dict__
        return tuple((t.data_ptr(), t._version) for t in [d['_h_' + name] for name in _HISTORY] + [self.radii])

    # ---- lazily folded float64 history -------------------------------------
    # The bond records carry fn, mt, fs, mb and offset in float32 and every
    # accepted step advances them; a per-bond float32 correction keeps what
    # float32 rounding dropped (the exact TwoSum error of each update), so
    # record + correction is the float64 history.  An accepted step therefore
    # writes no float64 per bond; reading a history attribute (or a float64
    # setup, every refresh_interval steps) first folds records and corrections
    # into new float64 tensors, with normal = geometry(x) as the eager commit
    # forms it.
    lazy_history = True

    def _history_corrections(self):
        size = max(4, self._lib.dpf_history_correction_floats(self.n_bonds))
        corr = getattr(self, '_history_corr', None)
        if corr is None or corr.numel() != size:
            corr = self._history_corr = torch.zeros(size, dtype=torch.float32, device=self.device)
        return corr

    def _stored_history(self):
        """History struct of the stored tensors (no fold: only x is read by the lazy commit)."""
        d = self.__dict__
        return _lib.History(*(d['_h_' + name].data_ptr() if name != 'radii' else self.radii.data_ptr()
                              for name in ('x', 'radii', 'normal', 'offset', 'fn', 'fs', 'mt', 'mb')))

    def _fold_history(self):
        d = self.__dict__
        d['_pending_fold'] = False
        valid = self._token is not None and self._token == self._state_token()
        for name in _HISTORY:
            t = d['_h_' + name]
            if not (t.is_contiguous() and t.dtype == F64):
                d['_h_' + name] = t.to(F64).contiguous()
        out = {name: torch.empty_like(d['_h_' + name]) for name in _HISTORY if name != 'x'}
        self._call('dpf_mixed_fold_history', ctypes.byref(self._graph), d['_h_x'].data_ptr(),
                   self._bond_data.data_ptr(), self._history_corrections().data_ptr(), out['normal'].data_ptr(),
                   out['offset'].data_ptr(), out['fn'].data_ptr(), out['fs'].data_ptr(), out['mt'].data_ptr(),
                   out['mb'].data_ptr(), self._stream())
        for name, t in out.items():
            d['_h_' + name] = t
        if valid:                  # the records describe the folded state as well
            self._token = self._state_token()

    def _commit_lazy(self, x_end):
        """Adopt the end positions of a lazily committed step."""
        self.__dict__['_h_x'] = x_end
        self.__dict__['_pending_fold'] = self.n_bonds > 0

    def _to_y32(self, y):
        self._call('dpf_to_float', 6*self.n_sites, y.data_ptr(), self._y32.data_ptr(), self._stream())

    def _step_begin(self, dt, external):
        self._cached = None
        self._status.zero_()
        if getattr(self, '_begin_scales', None) is None:
            self._begin_scales = torch.zeros(2, dtype=F64, device=self.device)
        scales = self._begin_scales
        self._zero_start = False
        if self._token is not None and self._token == self._state_token() and \
                self._since_refresh < self.refresh_interval:
            self._zero_start = self.__dict__.get('_committed_start', False)
            self._timed('setup', lambda: self._call(
                'dpf_mixed_begin', self.n_sites, self._loads.data_ptr(), self.mass.data_ptr(), self._v.data_ptr(),
                external.data_ptr(), self.fixed.data_ptr(), dt, self._r0.data_ptr(), scales.data_ptr(),
                self._partials.data_ptr(), self._stream()))
        else:
            self._since_refresh = 0
            self._committed_start = False
            history = self._history_struct()     # folds a lazily committed history first
            # the lazy history's corrections come out of the same pass
            corrections = self._history_corrections().data_ptr() if self.lazy_history else None
            self._timed('setup', lambda: self._call(
                'dpf_mixed_setup', ctypes.byref(self._graph), ctypes.byref(self._stiffness_struct()),
                ctypes.byref(history), self.mass.data_ptr(), self._v.data_ptr(), external.data_ptr(),
                self.fixed.data_ptr(), dt, self._bond_data.data_ptr(), self._r0.data_ptr(), self._loads.data_ptr(),
                scales.data_ptr(), self._wrench.data_ptr(), corrections, self._partials.data_ptr(),
                self._status.data_ptr(), self._stream()))
        # the scales reach the host with the first residual's fetch (one sync
        # less per step); a setup guard is raised by that residual's own trial
        self._deferred_scale = scales

        def rhs_scale():
            a, l = self._host_scalars[8:10].tolist()
            return max(a, .5*dt*dt*l, 1e-30)
        return rhs_scale

    def _mixed_residual(self, y, dt, want_tangent, use_p, scaled=None):
        self._committed_start = False      # the tangent is no longer the one the last commit stored
        r = torch.empty_like(y)
        self._to_y32(y)
        self._status.zero_()
        self._timed('residual', lambda: self._call(
            'dpf_mixed_residual', ctypes.byref(self._graph), self._bond_data.data_ptr(), y.data_ptr(),
            self._y32.data_ptr(), self.mass.data_ptr(), self.fixed.data_ptr(), dt, self._r0.data_ptr(),
            int(want_tangent), self._p32.data_ptr() if use_p else None, self._units32.data_ptr() if use_p else None,
            r.data_ptr(), _addr(scaled) if use_p else None, self._scalars.data_ptr() if use_p else None,
            self._wrench32.data_ptr(), self._partials.data_ptr(), self._status.data_ptr(), self._stream()))
        return r

    def _iteration_residual(self, y, dt, external):
        reuse = self._cached is not None and self._cached[0] is y
        if self.__dict__.get('_zero_start'):
            # y = 0 on records and tangent from the last commit: r = r0 (0 on fixed sites)
            self._zero_start = False
            r = torch.empty_like(y)
            self._status.zero_()
            self._timed('residual', lambda: self._call(
                'dpf_mixed_initial_residual', self.n_sites, self._r0.data_ptr(), self.fixed.data_ptr(),
                self._y32.data_ptr(), r.data_ptr(), self._stream()))
        else:
            r = self._cached[1] if reuse else self._mixed_residual(y, dt, want_tangent=True, use_p=False)
        self._cached = None
        self._timed('scaling', lambda: self._call(
            'dpf_mixed_scaling', ctypes.byref(self._graph), self._bond_data.data_ptr(), self._mass32.data_ptr(),
            self.fixed.data_ptr(), self.radii.data_ptr(), dt, self._block32.data_ptr(), self._p32.data_ptr(),
            self._units.data_ptr(), self._units32.data_ptr(), self._stream()))
        scaled = torch.empty_like(r)
        self._call('dpf_mixed_scale_residual', self.n_sites, self._p32.data_ptr(), self._units32.data_ptr(),
                   r.data_ptr(), scaled.data_ptr(), self._scalars.data_ptr(), self._partials.data_ptr(),
                   self._stream())
        norms, status = self._fetch(3, status=not reuse)
        if status:
            raise guard_error(status)
        self.units = self._units
        self._packed = None  # new tangent: repack before the next swept PCG
        return scaled, norms

    def _newton_operator(self, y, dt, external):
        def operator(v):
            v = self._vec(v)
            out = torch.empty_like(v)
            self._timed('jvp', lambda: self._call(
                'dpf_mixed_jacobian_vector', ctypes.byref(self._graph), self._bond_data.data_ptr(),
                self._y32.data_ptr(), v.data_ptr(), self._mass32.data_ptr(), self.fixed.data_ptr(), dt,
                self._units32.data_ptr(), self._p32.data_ptr(), out.data_ptr(), self._d32.data_ptr(),
                self._wrench32.data_ptr(), *self._bond_mask(), self._stream()))
            return out
        return operator

    def _bond_mask(self):
        """(per-bond segment, per-segment active flag) device pointers that let
        the bond passes skip bonds of finished segments; (None, None) here."""
        return None, None

    def _newton_preconditioner(self, dt):
        def precondition(vector, tolerance=.03, max_iterations=80):
            vector = self._vec(vector)
            out = torch.empty_like(vector)
            if self.sweep == 'ends':
                if self._packed != ('ends', dt):
                    self._pack_ends(dt)
                self._timed('pcg', lambda: self._end_pcg(vector, out, tolerance, max_iterations, self._inner))
                return out
            if self.sweep == 'tiles':
                self._ensure_tiles(dt, vector, tolerance, max_iterations)
                self._timed('pcg', lambda: self._tiled_pcg(self._tiles, vector, out, tolerance, max_iterations,
                                                           self._inner))
                return out
            self._timed('pcg', lambda: self._call(
                'dpf_mixed_precondition', ctypes.byref(self._graph), self._bond_data.data_ptr(),
                self._mass32.data_ptr(), self.fixed.data_ptr(), self._block32.data_ptr(), self._p32.data_ptr(),
                self._units32.data_ptr(), vector.data_ptr(), dt, tolerance, max_iterations, out.data_ptr(),
                self._inner.data_ptr(), self._wrench32.data_ptr(), self._mixed_workspace.data_ptr(),
                self._barrier.data_ptr(), self._status.data_ptr(), *self._bond_mask(), self._stream()))
            return out
        return precondition

    def _line_merit(self, candidate, dt, external):
        # The candidate's tangent overwrites the iterate's (FGMRES is done with it);
        # an accepted candidate's residual and tangent start the next iteration.
        r = self._mixed_residual(candidate, dt, want_tangent=True, use_p=True)
        (_, _, value), status = self._fetch(3, status=True)
        self._cached = (candidate, r)
        return value, status

    def _accept(self, y, dt):
        m, n = self.n_bonds, self.n_sites
        e = lambda *shape: torch.empty(shape, dtype=F64, device=self.device)
        self._to_y32(y)
        if self.lazy_history:
            x_end = e(n, 3)
            x = self.__dict__['_h_x']
            self._timed('commit', lambda: self._call(
                'dpf_mixed_commit_lazy', ctypes.byref(self._graph), self._bond_data.data_ptr(), x.data_ptr(),
                y.data_ptr(), self._y32.data_ptr(), x_end.data_ptr(), self._history_corrections().data_ptr(),
                self._wrench32.data_ptr(), self._loads.data_ptr(), self._stream()))
        else:
            state = dict(x=e(n, 3), normal=e(m, 3), offset=e(m, 3), fn=e(m), fs=e(m, 3), mt=e(m), mb=e(m, 3))
            history = self._history_struct()
            self._timed('commit', lambda: self._call(
                'dpf_mixed_commit', ctypes.byref(self._graph), self._bond_data.data_ptr(), ctypes.byref(history),
                y.data_ptr(), self._y32.data_ptr(), state['x'].data_ptr(), state['normal'].data_ptr(),
                state['offset'].data_ptr(), state['fn'].data_ptr(), state['fs'].data_ptr(), state['mt'].data_ptr(),
                state['mb'].data_ptr(), self._wrench32.data_ptr(), self._loads.data_ptr(), self._stream()))
        rotation = self._vec(self.rotation).clone()
        self._call('dpf_accept_step', self.n_sites, y.data_ptr(), dt, self._v.data_ptr(), rotation.data_ptr(),
                   self._stream())
        if self.lazy_history:
            self._commit_lazy(x_end)
        else:
            self.commit(state)
        self.v, self.rotation = self._v, rotation
        self._committed_start = True       # records and the tangent at y = 0 of the next step
        self._cached = None
        self._token = self._state_token()
        self._since_refresh += 1


for _name in _HISTORY:
    setattr(MixedNewtonBonds, _name, _history_property(_name))
