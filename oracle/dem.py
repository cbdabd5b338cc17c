"""NumPy FP64 restatement of the reference bonded-DEM Newton path.

TEST INFRASTRUCTURE ONLY: the checker for the CUDA path and the CPU baseline
that ``bench.py`` times.  Nothing in the product imports this module.

Every function cites the reference file:line (paths inside the reference
project) whose algorithm it restates.  Parity of this restatement with the
reference itself is pinned by ``tests/test_oracle_golden.py`` against vectors
generated by the reference's own code (``tests/golden/make_golden.py``).

Layouts follow the reference: per-site 6-vectors ``[tx, ty, tz, rx, ry, rz]``
as (N, 6) float64; per-bond vectors (M, 3); ``edges`` (M, 2) int64 with the
bond normal pointing from ``edges[:, 0]`` to ``edges[:, 1]``.
"""
import numpy as np

COS_QUARTER = float(np.cos(.25))


class SubdivideError(RuntimeError):
    """Recoverable failure; message starts with 'Subdivide:' as in the reference."""


def dot(a, b):
    return np.einsum('...i,...i->...', a, b)


def cross(a, b):
    return np.cross(a, b)


def scatter_add(n, index, values):
    """out[index[k]] += values[k] for (K, C) values; deterministic bincount per column."""
    out = np.empty((n, values.shape[1]))
    for c in range(values.shape[1]):
        out[:, c] = np.bincount(index, weights=values[:, c], minlength=n)
    return out


def transport(v, n0, n1, spin):
    """Shortest-arc transport n0 -> n1 then rotation about n1 by spin . bisector.

    Restates ``experiments/bonded_dem_finite_gpu.py:22-32`` (same algorithm as
    ``experiments/bonded_dem_core.py:31-42``); raises when a normal turns by
    more than 0.25 rad.
    """
    k = cross(n0, n1)
    cosine = np.clip(dot(n0, n1), -1., 1.)
    if np.any(cosine < COS_QUARTER):
        raise SubdivideError('Subdivide: normal turns more than .25 rad per half-step')
    out = v + cross(k, v)
    out = out + cross(k, cross(k, v))/(1+cosine)[:, None]
    b = n0 + n1
    b = b/np.maximum(np.linalg.norm(b, axis=1), 1e-12)[:, None]
    angle = dot(spin, b)[:, None]
    c, s = np.cos(angle), np.sin(angle)
    return c*out + s*cross(n1, out) + (1-c)*dot(n1, out)[:, None]*n1


def skew(v):
    s = np.zeros(v.shape[:-1] + (3, 3))
    s[..., 0, 1], s[..., 0, 2] = -v[..., 2], v[..., 1]
    s[..., 1, 0], s[..., 1, 2] = v[..., 2], -v[..., 0]
    s[..., 2, 0], s[..., 2, 1] = -v[..., 1], v[..., 0]
    return s


def exp_rotation(v):
    """SO(3) exponential via sinc; ``experiments/bonded_dem_finite_gpu.py:35-43``."""
    angle = np.linalg.norm(v, axis=1)
    s = skew(v)
    a = np.sinc(angle/np.pi)
    b = .5*np.sinc(angle/(2*np.pi))**2
    return np.eye(3) + a[:, None, None]*s + b[:, None, None]*(s@s)


class LinearBonds:
    """Stress-free linearised bonds; ``experiments/bonded_dem_linear_gpu.py:14-124``."""

    def __init__(self, points, radii, pairs, areas, contacts, masses, fixed,
                 young=1200., shear=480.):
        # bonded_dem_linear_gpu.py:15-40
        self.p = np.array(points, dtype=np.float64)
        self.edges = np.array(pairs, dtype=np.int64)
        self.i, self.j = self.edges[:, 0].copy(), self.edges[:, 1].copy()
        r = np.broadcast_to(np.asarray(radii, dtype=np.float64), (len(self.p),)).copy()
        area = np.broadcast_to(np.asarray(areas, dtype=np.float64), (len(self.edges),)).copy()
        c = np.asarray(contacts, dtype=np.float64)
        distance = self.p[self.j] - self.p[self.i]
        length = np.linalg.norm(distance, axis=1)
        self.n = distance/length[:, None]
        self.ri, self.rj = c - self.p[self.i], c - self.p[self.j]
        self.kn, self.ks = young*area/length, shear*area/length
        second = area**2/(4*np.pi)
        self.kb, self.kt = young*second/length, shear*(2*second)/length
        mass = np.broadcast_to(np.asarray(masses, dtype=np.float64), (len(self.p),)).copy()
        inertia = .4*mass*r*r
        self.mass = np.concatenate((np.repeat(mass[:, None], 3, 1), np.repeat(inertia[:, None], 3, 1)), 1)
        if np.any(self.mass <= 0):
            raise ValueError('Only positive-mass bodies can enter this solver')
        self.fixed = np.array(fixed, dtype=bool)
        self.q, self.v = np.zeros_like(self.mass), np.zeros_like(self.mass)
        self.kq = np.zeros_like(self.mass)
        self.diagonal = self._diagonal_blocks()
        self.preconditioner = None
        self.preconditioner_dt = None

    @property
    def n_sites(self):
        return len(self.p)

    def stiffness(self, q):
        """Frozen-tangent K q; ``bonded_dem_linear_gpu.py:42-52``."""
        a, b = q[self.i], q[self.j]
        du = b[:, :3] - a[:, :3] + cross(b[:, 3:], self.rj) - cross(a[:, 3:], self.ri)
        dw = b[:, 3:] - a[:, 3:]
        f = self.ks[:, None]*du + (self.kn-self.ks)[:, None]*dot(du, self.n)[:, None]*self.n
        m = self.kb[:, None]*dw + (self.kt-self.kb)[:, None]*dot(dw, self.n)[:, None]*self.n
        out = scatter_add(self.n_sites, self.i, np.concatenate((-f, -cross(self.ri, f) - m), 1))
        out += scatter_add(self.n_sites, self.j, np.concatenate((f, cross(self.rj, f) + m), 1))
        return out

    def _diagonal_blocks(self):
        """Per-site 6x6 diagonal blocks of K; ``bonded_dem_linear_gpu.py:54-72``."""
        eye = np.eye(3)
        nn = self.n[:, :, None]*self.n[:, None, :]
        d = self.ks[:, None, None]*eye + (self.kn-self.ks)[:, None, None]*nn
        h = self.kb[:, None, None]*eye + (self.kt-self.kb)[:, None, None]*nn
        diagonal = np.zeros((self.n_sites, 36))
        for indices, r in ((self.i, self.ri), (self.j, self.rj)):
            s = skew(r)
            block = np.zeros((len(indices), 6, 6))
            block[:, :3, :3] = d
            block[:, :3, 3:] = -d@s
            block[:, 3:, :3] = np.transpose(block[:, :3, 3:], (0, 2, 1))
            block[:, 3:, 3:] = np.transpose(s, (0, 2, 1))@d@s + h
            diagonal += scatter_add(self.n_sites, indices, block.reshape(-1, 36))
        return diagonal.reshape(-1, 6, 6)

    def _operator(self, q, alpha):
        """(diag M + alpha K) q with identity fixed rows; ``bonded_dem_linear_gpu.py:74-77``."""
        out = self.mass*q + alpha*self.stiffness(q)
        out[self.fixed] = q[self.fixed]
        return out

    def solve_increment(self, rhs, dt, guess=None, tolerance=2e-8, max_iterations=1000):
        """Block-Jacobi PCG; ``bonded_dem_linear_gpu.py:79-112``."""
        alpha = dt*dt/4
        if self.preconditioner_dt != dt:
            diagonal = np.einsum('ni,ij->nij', self.mass, np.eye(6)) + alpha*self.diagonal
            diagonal[self.fixed] = np.eye(6)
            self.preconditioner = np.linalg.inv(diagonal)
            self.preconditioner_dt = dt
        rhs = rhs.copy(); rhs[self.fixed] = 0
        norm = float(np.linalg.norm(rhs))
        if norm < 1e-30:
            return np.zeros_like(rhs), dict(iterations=0, relative_residual=0.)
        x = np.zeros_like(rhs) if guess is None else guess.copy()
        x[self.fixed] = 0
        residual = rhs - self._operator(x, alpha)
        z = np.einsum('nij,nj->ni', self.preconditioner, residual)
        direction = z.copy(); rz = (residual*z).sum()
        for iteration in range(max_iterations):
            ad = self._operator(direction, alpha)
            step = rz/(direction*ad).sum()
            x += step*direction; residual -= step*ad
            if iteration % 10 == 0:
                relative = float(np.linalg.norm(residual))/norm
                if relative < tolerance:
                    break
                if not np.isfinite(relative):
                    raise RuntimeError('Nonfinite conjugate-gradient residual')
            z = np.einsum('nij,nj->ni', self.preconditioner, residual)
            next_rz = (residual*z).sum()
            direction = z + (next_rz/rz)*direction; rz = next_rz
        actual = float(np.linalg.norm(rhs - self._operator(x, alpha)))/norm
        if actual > 5*tolerance or not np.isfinite(actual):
            raise RuntimeError(f'Linear solve failed after {iteration+1} iterations: {actual}')
        return x, dict(iterations=iteration+1, relative_residual=actual)

    def step(self, dt, external):
        """Linear implicit midpoint; ``bonded_dem_linear_gpu.py:114-121``."""
        rhs = dt*self.mass*self.v + .5*dt*dt*(external - self.kq)
        dq, metrics = self.solve_increment(rhs, dt, guess=dt*self.v)
        self.v = 2*dq/dt - self.v
        self.q = self.q + dq; self.kq = self.stiffness(self.q)
        return float((external*dq).sum()), metrics

    def energy(self):
        return float(.5*((self.mass*self.v*self.v).sum() + (self.q*self.kq).sum()))


class FiniteBonds(LinearBonds):
    """Finite-motion rate law; ``experiments/bonded_dem_finite_gpu.py:46-261``."""

    STATE = ('x', 'v', 'rotation', 'normal', 'offset', 'fn', 'fs', 'mt', 'mb')

    def __init__(self, points, radii, pairs, areas, masses, fixed, contacts=None,
                 young=1200., shear=480.):
        # bonded_dem_finite_gpu.py:47-64
        p = np.asarray(points, dtype=np.float64)
        i, j = np.asarray(pairs).T
        radii_a = np.broadcast_to(np.asarray(radii, dtype=np.float64), (len(p),))
        n = p[j] - p[i]
        n /= np.linalg.norm(n, axis=1)[:, None]
        classical = .5*(p[i]+p[j])
        classical += .5*(radii_a[i]-radii_a[j])[:, None]*n
        if contacts is None:
            contacts = classical
        contacts = np.asarray(contacts, dtype=np.float64)
        super().__init__(p, radii_a, pairs, areas, contacts, masses, fixed, young, shear)
        self.x = self.p.copy()
        self.radii = np.array(radii_a)
        self.normal = self.n.copy()
        self.offset = contacts - classical
        self.fn, self.mt = np.zeros_like(self.kn), np.zeros_like(self.kn)
        self.fs, self.mb = np.zeros_like(self.n), np.zeros_like(self.n)
        self.rotation = np.repeat(np.eye(3)[None], len(p), 0)
        self.time = 0.

    def geometry(self, x):
        """Normal and classical contact; ``bonded_dem_finite_gpu.py:66-73``."""
        d = x[self.j] - x[self.i]
        length = np.linalg.norm(d, axis=1)
        if np.any(length <= 1e-12):
            raise SubdivideError('Subdivide: coincident centers')
        n = d/length[:, None]
        c = .5*(x[self.i]+x[self.j]) + .5*(self.radii[self.i]-self.radii[self.j])[:, None]*n
        return n, c

    def assemble(self, fn, fs, mt, mb, n, ri, rj):
        """Scatter bond force and couple; ``bonded_dem_finite_gpu.py:75-80``."""
        f, couple = fn[:, None]*n + fs, mt[:, None]*n + mb
        out = scatter_add(self.n_sites, self.i, np.concatenate((f, cross(ri, f)+couple), 1))
        out += scatter_add(self.n_sites, self.j, np.concatenate((-f, -cross(rj, f)-couple), 1))
        return out

    def loads(self):
        """``bonded_dem_finite_gpu.py:82-85``."""
        n, c = self.geometry(self.x)
        c = c + self.offset
        return self.assemble(self.fn, self.fs, self.mt, self.mb, n, c-self.x[self.i], c-self.x[self.j])

    def trial(self, increment, *, mid_positions=None, end_positions=None):
        """Pure constitutive trial; ``bonded_dem_finite_gpu.py:87-116``."""
        if float(np.linalg.norm(increment[:, 3:], axis=1).max()) > .25:
            raise SubdivideError('Subdivide: body rotation exceeds .25 rad in a step')
        mid = self.x + .5*increment[:, :3] if mid_positions is None else mid_positions
        end = self.x + increment[:, :3] if end_positions is None else end_positions
        nm, contact = self.geometry(mid)
        ne, _ = self.geometry(end)
        spin = .5*(increment[self.i, 3:] + increment[self.j, 3:])
        offset_mid = transport(self.offset, self.normal, nm, .5*spin)
        contact = contact + offset_mid
        ri, rj = contact - mid[self.i], contact - mid[self.j]
        fs0 = transport(self.fs, self.normal, nm, .5*spin)
        mb0 = transport(self.mb, self.normal, nm, .5*spin)
        du = (increment[self.j, :3] - increment[self.i, :3]
              + cross(increment[self.j, 3:], rj) - cross(increment[self.i, 3:], ri))
        dw = increment[self.j, 3:] - increment[self.i, 3:]
        dn, twist = dot(du, nm), dot(dw, nm)
        fn = self.fn + self.kn*dn
        fs = fs0 + self.ks[:, None]*(du - dn[:, None]*nm)
        mt = self.mt + self.kt*twist
        mb = mb0 + self.kb[:, None]*(dw - twist[:, None]*nm)
        force = self.assemble(.5*(self.fn+fn), .5*(fs0+fs), .5*(self.mt+mt), .5*(mb0+mb), nm, ri, rj)
        return dict(force=force, n=nm, ri=ri, rj=rj, x=end, normal=ne, fn=fn, mt=mt,
                    fs=transport(fs, nm, ne, .5*spin),
                    mb=transport(mb, nm, ne, .5*spin),
                    offset=transport(offset_mid, nm, ne, .5*spin))

    def commit(self, trial):
        """``bonded_dem_finite_gpu.py:118-120``."""
        for name in ('x', 'normal', 'fn', 'fs', 'mt', 'mb', 'offset'):
            setattr(self, name, np.array(trial[name]))

    def energy(self):
        """Elastic + kinetic; ``bonded_dem_finite_gpu.py:122-125``."""
        elastic = .5*(self.fn**2/self.kn + dot(self.fs, self.fs)/self.ks
                      + self.mt**2/self.kt + dot(self.mb, self.mb)/self.kb).sum()
        return float(elastic + .5*(self.mass*self.v*self.v).sum())

    def local_defect(self, residual):
        """``bonded_dem_finite_gpu.py:127-131``."""
        correction = np.einsum('nij,nj->ni', self.preconditioner, residual)
        scale = np.ones_like(correction)
        scale[:, :3] = self.radii[:, None]
        return float(np.abs(correction/scale).max())

    def solve_increment(self, rhs, dt, tolerance=2e-7, max_iterations=1600):
        """PCG with local and global checks; ``bonded_dem_finite_gpu.py:133-167``."""
        diagonal = np.einsum('ni,ij->nij', self.mass, np.eye(6)) + dt*dt*self.diagonal/4
        diagonal[self.fixed] = np.eye(6)
        self.preconditioner = np.linalg.inv(diagonal)
        rhs = rhs.copy(); rhs[self.fixed] = 0
        norm = float(np.linalg.norm(rhs))
        if norm < 1e-40:
            return np.zeros_like(rhs), dict(iterations=0)
        x, residual = np.zeros_like(rhs), rhs.copy()
        z = np.einsum('nij,nj->ni', self.preconditioner, residual)
        direction = z.copy(); rz = dot(residual.ravel(), z.ravel())
        for iteration in range(max_iterations):
            ad = self._operator(direction, dt*dt/4)
            step = rz/(direction*ad).sum()
            x += step*direction; residual -= step*ad
            if iteration % 10 == 0:
                relative = float(np.linalg.norm(residual))/norm
                if relative < tolerance and self.local_defect(residual) < 2e-8:
                    actual = rhs - self._operator(x, dt*dt/4)
                    if float(np.linalg.norm(actual))/norm < 5*tolerance and self.local_defect(actual) < 1e-7:
                        return x, dict(iterations=iteration+1)
                if not np.isfinite(relative):
                    raise RuntimeError('Nonfinite PCG residual')
            z = np.einsum('nij,nj->ni', self.preconditioner, residual)
            next_rz = (residual*z).sum()
            direction = z + (next_rz/rz)*direction; rz = next_rz
        raise SubdivideError('Subdivide: balanced PCG did not converge')

    def step(self, dt, external, tolerance=2e-7, max_iterations=18):
        """Anderson-accelerated implicit midpoint; ``bonded_dem_finite_gpu.py:169-250``."""
        if not np.isfinite(dt) or dt <= 0:
            raise ValueError('Positive finite dt required')
        y = np.zeros_like(self.v)
        rhs_scale = float(np.linalg.norm(dt*self.mass*self.v + .5*dt*dt*external))
        rhs_scale = max(rhs_scale, .5*dt*dt*float(np.linalg.norm(self.loads()[~self.fixed])), 1e-30)
        cg_total = 0
        iterates, corrections = [], []
        units = np.ones_like(self.mass)
        units[:, 3:] = self.radii[:, None]
        relative = float('nan')
        for iteration in range(max_iterations):
            trial = self.trial(y)
            residual = self.mass*(y - dt*self.v) - .5*dt*dt*(trial['force'] + external)
            residual[self.fixed] = 0
            relative = float(np.linalg.norm(residual))/rhs_scale
            local = self.local_defect(residual) if iteration else (0. if relative == 0 else float('inf'))
            if relative < tolerance and local < 2e-6:
                velocity = 2*y/dt - self.v
                rotation = exp_rotation(y[:, 3:])@self.rotation
                self.commit(trial)
                self.v, self.rotation = velocity, rotation
                self.time += dt
                return float((external*y).sum()), dict(
                    nonlinear_iterations=iteration, nonlinear_relative_residual=relative, cg_iterations=cg_total,
                    local_pose_defect=local, max_step_rotation=float(np.linalg.norm(y[:, 3:], axis=1).max()))
            self.n, self.ri, self.rj = trial['n'], trial['ri'], trial['rj']
            self.diagonal = self._diagonal_blocks()
            self.preconditioner_dt = None
            correction, cg = self.solve_increment(-residual, dt)
            cg_total += cg['iterations']
            merit = max(relative/tolerance, self.local_defect(residual)/2e-6)
            iterates.append(y.copy()); corrections.append(correction.copy())
            iterates, corrections = iterates[-6:], corrections[-6:]
            directions = []
            if len(corrections) > 1:
                dc = np.stack([b - a for a, b in zip(corrections[:-1], corrections[1:])])
                dg = np.stack([b + db - a - da for a, b, da, db in
                               zip(iterates[:-1], iterates[1:], corrections[:-1], corrections[1:])])
                weighted = (dc*units).reshape(len(dc), -1)
                gram = weighted@weighted.T
                ridge = 1e-10*max(np.trace(gram), 1e-40)
                coefficients = np.linalg.solve(gram + ridge*np.eye(len(gram)), weighted@(correction*units).ravel())
                accelerated = correction - np.einsum('h,hij->ij', coefficients, dg)
                if np.isfinite(accelerated).all():
                    directions.append(accelerated)
            directions.append(correction)
            accepted = False
            for direction in directions:
                for factor in (1., .5, .25, .125, .0625):
                    candidate = y + factor*direction
                    try:
                        state = self.trial(candidate)
                    except RuntimeError:
                        continue
                    r = self.mass*(candidate - dt*self.v) - .5*dt*dt*(state['force'] + external)
                    r[self.fixed] = 0
                    candidate_merit = max(float(np.linalg.norm(r))/rhs_scale/tolerance, self.local_defect(r)/2e-6)
                    if candidate_merit < merit:
                        y = candidate; accepted = True; break
                if accepted:
                    break
            if not accepted:
                raise SubdivideError('Subdivide: nonlinear line search failed')
        raise SubdivideError(f'Subdivide: nonlinear residual {relative} did not converge')

    def advance_interval(self, dt, force_at_time, depth=0):
        """Recursive dt bisection on 'Subdivide:'; ``bonded_dem_finite_gpu.py:252-261``."""
        try:
            work, info = self.step(dt, force_at_time(self.time + .5*dt))
            return work, [dict(dt=dt, subdivision_depth=depth, **info)]
        except RuntimeError as error:
            if depth >= 8 or 'Subdivide:' not in str(error):
                raise
            a, ia = self.advance_interval(.5*dt, force_at_time, depth+1)
            b, ib = self.advance_interval(.5*dt, force_at_time, depth+1)
            return a+b, ia+ib


def fgmres(operator, rhs, precondition, tolerance=1e-6, restart=32, max_iterations=256):
    """Right-preconditioned flexible GMRES with CGS2 Arnoldi.

    Restates ``experiments/bonded_dem_newton.py:13-60``.
    """
    shape = rhs.shape
    b = rhs.ravel(); norm = float(np.linalg.norm(b))
    x = np.zeros_like(b)
    if norm == 0:
        return x.reshape(shape), dict(iterations=0, relative_residual=0.)
    residual = b.copy(); iterations = 0
    relative = float('nan')
    while iterations < max_iterations:
        width = min(restart, max_iterations - iterations)
        basis = np.empty((width+1, len(b)))
        transformed = np.empty((width, len(b)))
        h = np.zeros((width+1, width)); cs, sn = np.zeros(width), np.zeros(width)
        g = np.zeros(width+1); g[0] = float(np.linalg.norm(residual))
        basis[0] = residual/g[0]
        for j in range(width):
            z = precondition(basis[j].reshape(shape)).ravel()
            transformed[j] = z
            w = operator(z.reshape(shape)).ravel()
            projections = np.zeros(j+1)
            for _ in range(2):
                values = basis[:j+1]@w
                projections += values
                w = w - basis[:j+1].T@values
            h[:j+1, j] = projections
            h[j+1, j] = float(np.linalg.norm(w))
            breakdown = h[j+1, j] < 1e-14
            if not breakdown:
                basis[j+1] = w/h[j+1, j]
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
                coefficients = np.linalg.solve(h[:j+1, :j+1], g[:j+1])
                x = x + transformed[:j+1].T@coefficients
                residual = b - operator(x.reshape(shape)).ravel()
                relative = float(np.linalg.norm(residual))/norm
                if relative <= 1.05*tolerance:
                    return x.reshape(shape), dict(iterations=iterations, relative_residual=relative)
                break
    raise SubdivideError(f'Subdivide: FGMRES did not converge ({relative:g})')


def rotate_jvp(v, n0, n, dn, spin, dspin):
    """Value and directional derivative of ``transport`` with respect to (n, spin).

    Restates the analytic derivative of ``experiments/bonded_dem_jvp_warp.py:17-42``
    (vectorised over bonds).
    """
    raw = dot(n0, n)
    cosine = np.clip(raw, -1., 1.)
    dc = dot(n0, dn)
    dc = np.where((raw < -1.) | (raw > 1.), 0., dc)
    k, dk = cross(n0, n), cross(n0, dn)
    kv = cross(k, v)
    kkv = cross(k, kv)
    one_c = (1. + cosine)[:, None]
    t = v + kv + kkv/one_c
    dt = cross(dk, v) + (cross(dk, kv) + cross(k, cross(dk, v)))/one_c
    dt = dt - kkv*dc[:, None]/(one_c*one_c)
    length = np.linalg.norm(n0 + n, axis=1)[:, None]
    b = (n0 + n)/length
    db = (dn - b*dot(b, dn)[:, None])/length
    angle = dot(spin, b)
    da = (dot(dspin, b) + dot(spin, db))[:, None]
    c, s = np.cos(angle)[:, None], np.sin(angle)[:, None]
    nt = dot(n, t)[:, None]
    value = c*t + s*cross(n, t) + (1-c)*nt*n
    derivative = c*dt - s*da*t + c*da*cross(n, t)
    derivative = derivative + s*(cross(dn, t) + cross(n, dt)) + s*da*nt*n
    derivative = derivative + (1-c)*((dot(dn, t) + dot(n, dt))[:, None]*n + nt*dn)
    return value, derivative


class NewtonBonds(FiniteBonds):
    """Scaled Newton-FGMRES; ``experiments/bonded_dem_newton.py:63-201``."""

    def midpoint_force(self, y):
        """``bonded_dem_newton.py:64-81``."""
        mid = self.x + .5*y[:, :3]
        n, contact = self.geometry(mid)
        half_spin = .25*(y[self.i, 3:] + y[self.j, 3:])
        contact = contact + transport(self.offset, self.normal, n, half_spin)
        ri, rj = contact - mid[self.i], contact - mid[self.j]
        fs0 = transport(self.fs, self.normal, n, half_spin)
        mb0 = transport(self.mb, self.normal, n, half_spin)
        du = y[self.j, :3] - y[self.i, :3] + cross(y[self.j, 3:], rj) - cross(y[self.i, 3:], ri)
        dw = y[self.j, 3:] - y[self.i, 3:]
        dn, twist = dot(du, n), dot(dw, n)
        return self.assemble(self.fn + .5*self.kn*dn, fs0 + .5*self.ks[:, None]*(du - dn[:, None]*n),
                             self.mt + .5*self.kt*twist, mb0 + .5*self.kb[:, None]*(dw - twist[:, None]*n),
                             n, ri, rj)

    def residual(self, y, dt, external):
        """``bonded_dem_newton.py:83-86``."""
        trial = self.trial(y)
        r = self.mass*(y - dt*self.v) - .5*dt*dt*(trial['force'] + external)
        return np.where(self.fixed[:, None], y, r)

    def midpoint_force_jvp(self, y, direction):
        """Analytic d f_mid(y)[direction]; ``bonded_dem_jvp_warp.py:45-97``."""
        i, j = self.i, self.j
        ui, uj, wi, wj = y[i, :3], y[j, :3], y[i, 3:], y[j, 3:]
        dui, duj, dwi, dwj = direction[i, :3], direction[j, :3], direction[i, 3:], direction[j, 3:]
        mi, mj = self.x[i] + .5*ui, self.x[j] + .5*uj
        displacement = mj - mi
        length = np.linalg.norm(displacement, axis=1)[:, None]
        n = displacement/length
        dd = .5*(duj - dui)
        dn = (dd - n*dot(n, dd)[:, None])/length
        spin, dspin = .25*(wi + wj), .25*(dwi + dwj)
        rotated, drotated = rotate_jvp(self.offset, self.normal, n, dn, spin, dspin)
        rad = .5*(self.radii[i] - self.radii[j])[:, None]
        contact = .5*(mi + mj) + rad*n + rotated
        dcontact = .25*(dui + duj) + rad*dn + drotated
        ri, rj = contact - mi, contact - mj
        dri, drj = dcontact - .5*dui, dcontact - .5*duj
        fs0, dfs0 = rotate_jvp(self.fs, self.normal, n, dn, spin, dspin)
        mb0, dmb0 = rotate_jvp(self.mb, self.normal, n, dn, spin, dspin)
        du = uj - ui + cross(wj, rj) - cross(wi, ri)
        ddu = duj - dui + cross(dwj, rj) + cross(wj, drj) - cross(dwi, ri) - cross(wi, dri)
        dw, ddw = wj - wi, dwj - dwi
        nd, tw = dot(du, n)[:, None], dot(dw, n)[:, None]
        dnd = dot(ddu, n)[:, None] + dot(du, dn)[:, None]
        dtw = dot(ddw, n)[:, None] + dot(dw, dn)[:, None]
        kn, ks, kt, kb = (k[:, None] for k in (self.kn, self.ks, self.kt, self.kb))
        fn_mid = self.fn[:, None] + .5*kn*nd
        dfn_mid = .5*kn*dnd
        fs_mid = fs0 + .5*ks*(du - nd*n)
        dfs_mid = dfs0 + .5*ks*(ddu - dnd*n - nd*dn)
        mt_mid = self.mt[:, None] + .5*kt*tw
        dmt_mid = .5*kt*dtw
        dmb_mid = dmb0 + .5*kb*(ddw - dtw*n - tw*dn)
        f = fn_mid*n + fs_mid
        df = dfn_mid*n + fn_mid*dn + dfs_mid
        dcouple = dmt_mid*n + mt_mid*dn + dmb_mid
        dti = cross(dri, f) + cross(ri, df) + dcouple
        dtj = -cross(drj, f) - cross(rj, df) - dcouple
        out = scatter_add(self.n_sites, i, np.concatenate((df, dti), 1))
        out += scatter_add(self.n_sites, j, np.concatenate((-df, dtj), 1))
        return out

    def jacobian_vector(self, y, direction, dt, external):
        """J d of the midpoint residual; ``bonded_dem_newton.py:88-92`` (torch.func.jvp
        there) with the derivative of ``bonded_dem_jvp_warp.py:106-116``."""
        result = self.mass*direction - .5*dt*dt*self.midpoint_force_jvp(y, direction)
        return np.where(self.fixed[:, None], direction, result)

    def prepare_scaling(self, trial, dt):
        """``bonded_dem_newton.py:94-102``."""
        self.n, self.ri, self.rj = trial['n'], trial['ri'], trial['rj']
        self.diagonal = self._diagonal_blocks()
        self.block = np.einsum('ni,ij->nij', self.mass, np.eye(6)) + .25*dt*dt*self.diagonal
        self.block[self.fixed] = np.eye(6)
        self.preconditioner = np.linalg.inv(self.block)
        self.units = np.ones_like(self.mass)
        self.units[:, :3] = self.radii[:, None]
        self.units[self.fixed] = 1.

    def scale_residual(self, r):
        """``bonded_dem_newton.py:104-105``."""
        return np.einsum('nij,nj->ni', self.preconditioner, r)/self.units

    def elastic_precondition(self, vector, dt, tolerance=.03, max_iterations=80):
        """Block-Jacobi PCG on M + dt^2/4 K; ``bonded_dem_newton.py:107-130``."""
        rhs = np.einsum('nij,nj->ni', self.block, self.units*vector)
        rhs[self.fixed] = 0
        x = np.zeros_like(rhs); r = rhs.copy()
        z = np.einsum('nij,nj->ni', self.preconditioner, r)
        direction = z.copy(); rz = (r*z).sum(); initial = float(rz)
        if initial == 0:
            return x
        for iteration in range(max_iterations):
            ad = self._operator(direction, .25*dt*dt)
            denominator = (direction*ad).sum()
            alpha = rz/denominator
            x += alpha*direction; r -= alpha*ad
            z = np.einsum('nij,nj->ni', self.preconditioner, r)
            following = (r*z).sum()
            if iteration % 5 == 0 and float(following) <= tolerance*tolerance*initial:
                break
            direction = z + (following/rz)*direction; rz = following
        self.inner_iterations += iteration+1
        return x/self.units

    def step(self, dt, external, tolerance=2e-7, max_iterations=12, *,
             pose_tolerance=2e-6, backend='fgmres', linear_tolerance=1e-6,
             preconditioning='elastic'):
        """Line-searched Newton on the implicit-midpoint residual; ``bonded_dem_newton.py:132-201``."""
        if not np.isfinite(dt) or dt <= 0:
            raise ValueError('Positive finite dt required')
        y = np.zeros_like(self.v)
        rhs_scale = max(float(np.linalg.norm(dt*self.mass*self.v + .5*dt*dt*external)),
                        .5*dt*dt*float(np.linalg.norm(self.loads()[~self.fixed])), 1e-30)
        krylov, self.inner_iterations = 0, 0
        residual_trace = []
        relative = local = float('nan')
        for iteration in range(max_iterations+1):
            trial = self.trial(y)
            self.prepare_scaling(trial, dt)
            r = self.residual(y, dt, external)
            scaled = self.scale_residual(r)
            relative, local = float(np.linalg.norm(r))/rhs_scale, float(np.abs(scaled).max())
            residual_trace.append([relative, local])
            if relative < tolerance and local < pose_tolerance:
                velocity = 2*y/dt - self.v
                rotation = exp_rotation(y[:, 3:])@self.rotation
                self.commit(trial)
                self.v, self.rotation = velocity, rotation
                self.time += dt
                return float((external*y).sum()), dict(
                    nonlinear_iterations=iteration, nonlinear_relative_residual=relative,
                    local_pose_defect=local, krylov_iterations=krylov,
                    cg_iterations=self.inner_iterations, residual_trace=residual_trace,
                    max_step_rotation=float(np.linalg.norm(y[:, 3:], axis=1).max()))
            if iteration == max_iterations:
                break

            def operator(v):
                return self.scale_residual(self.jacobian_vector(y, self.units*v, dt, external))
            if backend == 'dense':
                free = np.flatnonzero(~np.repeat(self.fixed, 6))
                if len(free) > 400:
                    raise ValueError('Dense reference limited to 400 free DOFs')
                columns = []
                for col in np.eye(len(free)):
                    direction = np.zeros(y.size); direction[free] = col
                    columns.append(operator(direction.reshape(y.shape)).ravel()[free])
                jac = np.stack(columns, 1)
                delta = np.zeros(y.size)
                delta[free] = np.linalg.solve(jac, -scaled.ravel()[free])
                delta = delta.reshape(y.shape)
            elif backend == 'fgmres':
                if preconditioning == 'elastic':
                    precondition = lambda v: self.elastic_precondition(v, dt)
                elif preconditioning == 'block':
                    precondition = lambda v: v
                else:
                    raise ValueError(preconditioning)
                delta, metrics = fgmres(operator, -scaled, precondition, tolerance=linear_tolerance)
                krylov += metrics['iterations']
            else:
                raise ValueError(backend)
            correction = self.units*delta
            correction[self.fixed] = 0
            merit = float(np.linalg.norm(scaled))
            accepted = False
            for power in range(10):
                factor = 2.**(-power)
                candidate = y + factor*correction
                try:
                    value = self.scale_residual(self.residual(candidate, dt, external))
                except RuntimeError as error:
                    if 'Subdivide:' not in str(error):
                        raise
                    continue
                if float(np.linalg.norm(value)) < (1-1e-4*factor)*merit:
                    y = candidate; accepted = True; break
            if not accepted:
                raise SubdivideError('Subdivide: Newton line search failed')
        raise SubdivideError(f'Subdivide: Newton did not converge ({relative:g}, {local:g})')


class AdaptiveIntervals:
    """Remembered subdivision depth; ``experiments/bonded_dem_adaptive.py:4-23``."""

    def __init__(self, solver):
        self.solver = solver
        self.depth = 0
        self.easy_intervals = 0

    def advance(self, dt, load):
        work, records = 0., []
        for _ in range(2**self.depth):
            value, info = self.solver.advance_interval(dt/(2**self.depth), load, depth=self.depth)
            work += value; records.extend(info)
        self.depth = max(item['subdivision_depth'] for item in records)
        if max(item['nonlinear_iterations'] for item in records) <= 3:
            self.easy_intervals += 1
        else:
            self.easy_intervals = 0
        if self.easy_intervals >= 8 and self.depth:
            self.depth -= 1
            self.easy_intervals = 0
        return work, records


def reference_stiffness(points, pairs, contacts, kn, ks, kb, kt):
    """Dense 6N x 6N stress-free K from B^T D B + A^T H A.

    Restates ``experiments/bonded_dem_dynamics.py:22-47`` (returned dense for
    the small oracle cases instead of SciPy CSR).
    """
    x = np.asarray(points, dtype=np.float64)
    i, j = np.asarray(pairs).T
    d = x[j] - x[i]
    n = d/np.linalg.norm(d, axis=1)[:, None]
    ri, rj = contacts - x[i], contacts - x[j]
    count = len(n)
    b, a = np.zeros((count, 3, 12)), np.zeros((count, 3, 12))
    b[:, :, :3], b[:, :, 3:6] = -np.eye(3), skew(ri)
    b[:, :, 6:9], b[:, :, 9:12] = np.eye(3), -skew(rj)
    a[:, :, 3:6], a[:, :, 9:12] = -np.eye(3), np.eye(3)
    nn = n[:, :, None]*n[:, None, :]
    dd = ks[:, None, None]*np.eye(3) + (kn-ks)[:, None, None]*nn
    hh = kb[:, None, None]*np.eye(3) + (kt-kb)[:, None, None]*nn
    local = np.einsum('eai,eab,ebj->eij', b, dd, b) + np.einsum('eai,eab,ebj->eij', a, hh, a)
    idx = np.concatenate((6*i[:, None] + np.arange(6), 6*j[:, None] + np.arange(6)), 1)
    k = np.zeros((6*len(x), 6*len(x)))
    for e in range(count):
        k[np.ix_(idx[e], idx[e])] += local[e]
    return k


def solve_prescribed(k, prescribed, values, load=None):
    """Static linear equilibrium with the prescribed DOFs eliminated exactly
    (restates ``experiments/bonded_dem_material.py:53-65`` with a dense solve)."""
    q = np.array(values, dtype=np.float64).ravel()
    mask = np.asarray(prescribed, dtype=bool).ravel()
    free, fixed = np.flatnonzero(~mask), np.flatnonzero(mask)
    rhs = np.zeros(len(q)) if load is None else np.asarray(load, dtype=np.float64).ravel()
    q[free] = np.linalg.solve(k[np.ix_(free, free)], rhs[free] - k[np.ix_(free, fixed)]@q[fixed])
    reaction = k@q - rhs
    scale = max(np.linalg.norm(rhs), np.linalg.norm(reaction[fixed]), 1e-30)
    residual = np.linalg.norm(reaction[free])/scale
    if not np.isfinite(q).all() or residual > 1e-8:
        raise AssertionError(f'Unresolved static equilibrium, relative residual {residual}')
    return q, float(residual)


# ---------------------------------------------------------------------------
# Energy law (experiments/foam_dem_energy.py, EnergyFoam with volume=False and
# kinematics='small'): bond potential, closed-form force and world torque.

def quat_matrix(q):
    """Rotation matrix of unit quaternions (w, x, y, z) (foam_dem_energy.py:61-65)."""
    w, x, y, z = np.moveaxis(np.asarray(q, dtype=np.float64), -1, 0)
    return np.stack((1 - 2*(y*y + z*z), 2*(x*y - w*z), 2*(x*z + w*y),
                     2*(x*y + w*z), 1 - 2*(x*x + z*z), 2*(y*z - w*x),
                     2*(x*z - w*y), 2*(y*z + w*x), 1 - 2*(x*x + y*y)), -1).reshape(np.shape(q)[:-1] + (3, 3))


class EnergyBonds:
    """Bond part of ``EnergyFoam`` (foam_dem_energy.py:127-168 with volume=False):
    rest normal n0 and levers ri, rj and base stiffness (kn, ks, kb, kt) of
    ``LinearBonds`` (bonded_dem_linear_gpu.py:15-40)."""

    def __init__(self, points, radii, pairs, areas, contacts, masses, fixed, young=1200., shear=480.):
        b = LinearBonds(points, radii, pairs, areas, contacts, masses, fixed, young, shear)
        self.X = b.p
        self.i, self.j = b.i, b.j
        self.n0, self.ri, self.rj = b.n, b.ri, b.rj
        self.base = np.stack((b.kn, b.ks, b.kb, b.kt), 1)
        self.mass, self.inertia = b.mass[:, 0], b.mass[:, 3]

    def kinematics(self, theta, x, q):
        """foam_dem_energy.py:303-315 (averaged-frame stretch, sin-angle rotation)."""
        R = quat_matrix(q)
        Ri, Rj = R[self.i], R[self.j]
        pi = np.einsum('bij,bj->bi', Ri, self.ri)
        pj = np.einsum('bij,bj->bi', Rj, self.rj)
        D = x[self.j] + pj - x[self.i] - pi
        d = .5*(np.einsum('bji,bj->bi', Ri, D) + np.einsum('bji,bj->bi', Rj, D))
        Psi = np.einsum('bki,bkj->bij', Ri, Rj)
        A = Psi - np.swapaxes(Psi, 1, 2)
        phi = .5*np.stack((A[:, 2, 1], A[:, 0, 2], A[:, 1, 0]), -1)
        k = self.base*np.exp(.5*(theta[self.i, :4] + theta[self.j, :4]))
        dn, pn = dot(d, self.n0), dot(phi, self.n0)
        dt, pt = d - dn[:, None]*self.n0, phi - pn[:, None]*self.n0
        return Ri, Rj, pi, pj, D, Psi, k, dn, dt, pn, pt

    def energy(self, theta, x, q):
        """foam_dem_energy.py:405-421 (linear bond energy)."""
        *_, k, dn, dt, pn, pt = self.kinematics(theta, x, q)
        return float((.5*k[:, 0]*dn**2 + .5*(k[:, 1]*dot(dt, dt) + k[:, 2]*dot(pt, pt) + k[:, 3]*pn**2)).sum())

    def forces(self, theta, x, q):
        """-dE/dx and -dE/d(world rotation) (foam_dem_energy.py:797-811)."""
        Ri, Rj, pi, pj, D, Psi, k, dn, dt, pn, pt = self.kinematics(theta, x, q)
        gd = k[:, :1]*dn[:, None]*self.n0 + k[:, 1:2]*dt
        gp = k[:, 3:4]*pn[:, None]*self.n0 + k[:, 2:3]*pt
        Rgi, Rgj = np.einsum('bij,bj->bi', Ri, gd), np.einsum('bij,bj->bi', Rj, gd)
        a = .5*(Rgi + Rgj)
        trace = np.trace(Psi, axis1=1, axis2=2)
        M = .5*(trace[:, None]*gp - np.einsum('bji,bj->bi', Psi, gp))
        T = np.einsum('bij,bj->bi', Ri, M)
        tj = cross(pj, a) - .5*cross(D, Rgj) + T
        ti = -cross(pi, a) - .5*cross(D, Rgi) - T
        n = len(x)
        f = scatter_add(n, self.i, a) + scatter_add(n, self.j, -a)
        tau = scatter_add(n, self.i, -ti) + scatter_add(n, self.j, -tj)
        return f, tau


# ---------------------------------------------------------------------------
# Parallel-bond component with brittle failure (experiments/bonded_dem_core.py:45-208).

class ParallelBonds:
    """Stateful parallel bonds advanced once per step from midpoint samples.

    Section constants (bonded_dem_core.py:86-93): A = pi r_b^2, I = pi r_b^4/4,
    J = 2 I; kn = kbar_n A, ks = kbar_s A, kb = kbar_n I, kt = kbar_s J.
    """

    def __init__(self, reference, pairs, radii, bond_radius, kbar_n, kbar_s, tensile_strength=np.inf,
                 cohesion=np.inf, friction_angle=0., moment_factor=1.):
        self.x = np.array(reference, dtype=np.float64)
        self.pairs = np.array(pairs, dtype=np.int64)
        self.i, self.j = self.pairs.T
        m = len(self.pairs)
        per_bond = lambda v: np.broadcast_to(np.asarray(v, dtype=np.float64), (m,)).copy()
        self.radii = np.broadcast_to(np.asarray(radii, dtype=np.float64), (len(self.x),)).copy()
        self.rb = per_bond(bond_radius)
        self.area = np.pi*self.rb**2
        self.second_moment = np.pi*self.rb**4/4
        self.polar_moment = 2*self.second_moment
        kbn, kbs = per_bond(kbar_n), per_bond(kbar_s)
        self.kn, self.ks = kbn*self.area, kbs*self.area
        self.kb, self.kt = kbn*self.second_moment, kbs*self.polar_moment
        self.tensile_strength, self.cohesion = per_bond(tensile_strength), per_bond(cohesion)
        self.tan_phi, self.beta = np.tan(friction_angle), float(moment_factor)
        self.normal, _ = self.geometry(self.x)
        self.fn, self.mt = np.zeros(m), np.zeros(m)
        self.fs, self.mb = np.zeros((m, 3)), np.zeros((m, 3))
        self.failure = np.zeros(m, dtype=np.int8)
        self.break_energy = np.zeros(m)
        self.work, self.time = 0., 0.

    def geometry(self, x):
        """bonded_dem_core.py:117-126: unit normal i -> j and classical contact point."""
        d = x[self.j] - x[self.i]
        length = np.linalg.norm(d, axis=1)
        if np.any(length <= 1e-12):
            raise ValueError('Coincident centers are outside this baseline')
        n = d/length[:, None]
        return n, .5*(x[self.i] + x[self.j]) + .5*(self.radii[self.i] - self.radii[self.j])[:, None]*n

    def elastic_energy_per_bond(self):
        return .5*(self.fn**2/self.kn + dot(self.fs, self.fs)/self.ks + self.mt**2/self.kt
                   + dot(self.mb, self.mb)/self.kb)

    def loads(self):
        """bonded_dem_core.py:132-142: forces and torques about the centres."""
        n, c = self.geometry(self.x)
        f = self.fn[:, None]*n + self.fs
        couple = self.mt[:, None]*n + self.mb
        size = len(self.x)
        force = scatter_add(size, self.i, f) - scatter_add(size, self.j, f)
        torque = (scatter_add(size, self.i, cross(c - self.x[self.i], f) + couple)
                  + scatter_add(size, self.j, -cross(c - self.x[self.j], f) - couple))
        return force, torque

    def advance(self, x_next, velocity_mid, omega_mid, dt, *, x_mid=None):
        """bonded_dem_core.py:144-208: midpoint increments, transports, failure."""
        end = np.asarray(x_next, dtype=np.float64)
        mid = .5*(self.x + end) if x_mid is None else np.asarray(x_mid, dtype=np.float64)
        v, w = np.asarray(velocity_mid, dtype=np.float64), np.asarray(omega_mid, dtype=np.float64)
        if np.max(np.linalg.norm(w, axis=1))*dt > .25:
            raise ValueError('Body rotation > 0.25 rad per step; subdivide')
        nm, contact = self.geometry(mid)
        ne, _ = self.geometry(end)
        half = .25*(w[self.i] + w[self.j])*dt
        try:
            fs0 = transport(self.fs, self.normal, nm, half)
            mb0 = transport(self.mb, self.normal, nm, half)
            transport(np.zeros_like(fs0), nm, ne, half)
        except SubdivideError as e:
            raise ValueError(str(e)) from e
        du = (v[self.j] + cross(w[self.j], contact - mid[self.j]) - v[self.i]
              - cross(w[self.i], contact - mid[self.i]))*dt
        dth = (w[self.j] - w[self.i])*dt
        on = (self.failure == 0).astype(np.float64)
        dn, tw = dot(du, nm)*on, dot(dth, nm)*on
        ds = (du - dot(du, nm)[:, None]*nm)*on[:, None]
        bend = (dth - dot(dth, nm)[:, None]*nm)*on[:, None]
        fn, mt = self.fn + self.kn*dn, self.mt + self.kt*tw
        fs, mb = fs0 + self.ks[:, None]*ds, mb0 + self.kb[:, None]*bend
        work = .5*((self.fn + fn)*dn + dot(fs0 + fs, ds) + (self.mt + mt)*tw + dot(mb0 + mb, bend))
        sigma = fn/self.area + self.beta*np.linalg.norm(mb, axis=1)*self.rb/self.second_moment
        tau = np.linalg.norm(fs, axis=1)/self.area + self.beta*np.abs(mt)*self.rb/self.polar_moment
        intact = on > 0
        tensile = intact & (sigma > self.tensile_strength)
        shear = intact & ~tensile & (tau > self.cohesion - fn/self.area*self.tan_phi)
        broken = tensile | shear
        trial_energy = .5*(fn**2/self.kn + dot(fs, fs)/self.ks + mt**2/self.kt + dot(mb, mb)/self.kb)
        self.break_energy = self.break_energy + np.where(broken, trial_energy, 0.)
        self.failure = np.where(tensile, 1, np.where(shear, 2, self.failure)).astype(np.int8)
        keep = (~broken).astype(np.float64)
        fn, mt, fs, mb = fn*keep, mt*keep, fs*keep[:, None], mb*keep[:, None]
        self.fn, self.mt = fn, mt
        self.fs, self.mb = transport(fs, nm, ne, half), transport(mb, nm, ne, half)
        self.work += float(work.sum())
        self.x, self.normal = end.copy(), ne
        self.time += dt
        return dict(newly_broken=int(broken.sum()), energy=float(self.elastic_energy_per_bond().sum()),
                    removed_bond_energy=float(self.break_energy.sum()))


# ---------------------------------------------------------------------------
# Line-searched Newton on the bond potential (static equilibrium and implicit
# Euler).  The reference integrates EnergyFoam explicitly; these minimisations
# of its bond potential (foam_dem_energy.py:303-315, 405-421, 797-811) are
# restated here in NumPy with exact sparse solves so that the CUDA solver's
# minimiser can be checked.  Unknowns per site: displacement u and rotation
# vector t with q = exp(t) q0.

def rotation_quaternion(t):
    """Unit quaternions (w, x, y, z) of rotation vectors (N, 3)."""
    angle = np.linalg.norm(t, axis=1, keepdims=True)
    with np.errstate(invalid='ignore', divide='ignore'):
        scale = np.where(angle > 1e-4, np.sin(.5*angle)/np.where(angle > 0, angle, 1.), .5 - angle*angle/48)
    return np.concatenate((np.cos(.5*angle), scale*t), 1)


def quaternion_product(a, b):
    """Hamilton product of (N, 4) quaternions (w, x, y, z)."""
    aw, ax, ay, az = a.T
    bw, bx, by, bz = b.T
    return np.stack((aw*bw - ax*bx - ay*by - az*bz, aw*bx + ax*bw + ay*bz - az*by,
                     aw*by - ax*bz + ay*bw + az*bx, aw*bz + ax*by - ay*bx + az*bw), 1)


def left_jacobian_transpose_apply(t, v):
    """J_l(t)^T v, exp(t + e) = exp(J_l(t) e) exp(t)."""
    a_ = np.linalg.norm(t, axis=1, keepdims=True)
    small = a_ < 1e-3
    s = np.where(small, 1., a_)
    a = np.where(small, .5 - a_*a_/24, (1 - np.cos(a_))/(s*s))
    b = np.where(small, 1/6 - a_*a_/120, (a_ - np.sin(a_))/(s*s*s))
    c = cross(t, v)
    return v - a*c + b*cross(t, c)


def bond_blocks(n, ri, rj, kn, ks, kb, kt):
    """Per-bond 12 x 12 stiffness B^T D B + A^T H A (bonded_dem_dynamics.py:22-47)."""
    count = len(n)
    b, a = np.zeros((count, 3, 12)), np.zeros((count, 3, 12))
    b[:, :, :3], b[:, :, 3:6] = -np.eye(3), skew(ri)
    b[:, :, 6:9], b[:, :, 9:12] = np.eye(3), -skew(rj)
    a[:, :, 3:6], a[:, :, 9:12] = -np.eye(3), np.eye(3)
    nn = n[:, :, None]*n[:, None, :]
    dd = ks[:, None, None]*np.eye(3) + (kn-ks)[:, None, None]*nn
    hh = kb[:, None, None]*np.eye(3) + (kt-kb)[:, None, None]*nn
    return np.einsum('eai,eab,ebj->eij', b, dd, b) + np.einsum('eai,eab,ebj->eij', a, hh, a)


def sparse_stiffness(n_sites, pairs, n, ri, rj, kn, ks, kb, kt):
    """The 6N x 6N stiffness of ``bond_blocks`` as a SciPy CSR matrix."""
    import scipy.sparse as sp
    i, j = np.asarray(pairs).T
    local = bond_blocks(n, ri, rj, kn, ks, kb, kt)
    idx = np.concatenate((6*i[:, None] + np.arange(6), 6*j[:, None] + np.arange(6)), 1)
    rows = np.repeat(idx, 12, axis=1).ravel()
    cols = np.tile(idx, (1, 12)).ravel()
    return sp.coo_matrix((local.ravel(), (rows, cols)), shape=(6*n_sites, 6*n_sites)).tocsr()


def energy_tangent(bonds, theta, x, q):
    """Frozen tangent of the bond potential at (x, q): axis n = (x_j - x_i)/L,
    contact point c = ((x_i + R_i r_i) + (x_j + R_j r_j))/2, levers c - x_i,
    c - x_j, stiffness base exp((theta_i + theta_j)/2)."""
    R = quat_matrix(q)
    i, j = bonds.i, bonds.j
    ci = x[i] + np.einsum('bij,bj->bi', R[i], bonds.ri)
    cj = x[j] + np.einsum('bij,bj->bi', R[j], bonds.rj)
    c = .5*(ci + cj)
    d = x[j] - x[i]
    n = d/np.linalg.norm(d, axis=1)[:, None]
    k = bonds.base*np.exp(.5*(theta[i, :4] + theta[j, :4]))
    return n, c - x[i], c - x[j], k


def _block_jacobi_cg(a, b, tolerance):
    """Solve a x = b (SPD, rows in whole sites of 6) by CG preconditioned with
    the inverse 6 x 6 diagonal blocks, to |r| <= tolerance |b|."""
    import scipy.sparse.linalg as spla
    n = a.shape[0]//6
    blocks = np.stack([a[6*k:6*k + 6, 6*k:6*k + 6].toarray() for k in range(n)]) if n < 64 else \
        a.tobsr(blocksize=(6, 6)).data[_diagonal_block_index(a.tobsr(blocksize=(6, 6)))]
    inverse = np.linalg.inv(blocks)
    precondition = spla.LinearOperator(a.shape, matvec=lambda v: np.einsum('kij,kj->ki', inverse,
                                                                           v.reshape(-1, 6)).ravel())
    x, info = spla.cg(a, b, rtol=tolerance, atol=0., maxiter=20*n + 200, M=precondition)
    if info != 0:
        raise RuntimeError(f'energy Newton: inner CG did not converge ({info})')
    return x


def _diagonal_block_index(bsr):
    """Positions of the diagonal blocks in a BSR matrix's data (every block row has one)."""
    rows = np.repeat(np.arange(bsr.shape[0]//6), np.diff(bsr.indptr))
    where = np.flatnonzero(bsr.indices == rows)
    return where[np.argsort(rows[where], kind='stable')]


def energy_newton(bonds, theta, x0, q0, load, fixed, prescribed=None, inertia=None, tolerance=1e-10,
                  max_iterations=60):
    """Minimise the bond potential over (u, t) (static: E_b - f . u - tau . t;
    implicit Euler with inertia = (dt, v, w): plus sum m |u - dt v|^2/(2 dt^2)
    + sum I |t - dt w|^2/(2 dt^2)).  Fixed sites are held at ``prescribed``
    displacements with their rotation held.  Newton directions solve the
    frozen-tangent system on the free DOFs by block-Jacobi CG to 1e-10; Armijo
    backtracking on the potential; stop at |g| <= tolerance * scale, scale the
    largest of the first gradient norm, |load| and the roundoff level of the
    bond forces divided by the tolerance.  Returns (u, t, info)."""
    import scipy.sparse as sp
    import scipy.sparse.linalg as spla
    n_sites = len(x0)
    fixed = np.asarray(fixed, dtype=bool)
    load = np.where(fixed[:, None], 0., np.asarray(load, dtype=np.float64))
    free = np.flatnonzero(~np.repeat(fixed, 6))
    u = np.zeros((n_sites, 3))
    if prescribed is not None:
        u[fixed] = np.asarray(prescribed, dtype=np.float64)[fixed]
    t = np.zeros((n_sites, 3))

    def evaluate(u, t):
        x = x0 + u
        q = quaternion_product(rotation_quaternion(t), q0)
        e = bonds.energy(theta, x, q)
        f, tau = bonds.forces(theta, x, q)
        g = np.concatenate((-f - load[:, :3], -left_jacobian_transpose_apply(t, tau) - load[:, 3:]), 1)
        phi = e - (load[:, :3]*u).sum() - (load[:, 3:]*t).sum()
        if inertia is not None:
            dt, v, w = inertia
            du, dw = u - dt*v, t - dt*w
            g[:, :3] += bonds.mass[:, None]*du/(dt*dt)
            g[:, 3:] += bonds.inertia[:, None]*dw/(dt*dt)
            phi += .5*((bonds.mass[:, None]*du*du).sum() + (bonds.inertia[:, None]*dw*dw).sum())/(dt*dt)
        g[fixed] = 0.
        return phi, g, x, q

    phi, g, x, q = evaluate(u, t)
    gnorm = np.linalg.norm(g)
    # floor: the roundoff level of bond forces (1e-13 of the stiffest bond times the largest coordinate)
    floor = 1e-13*float(bonds.base[:, 0].max(initial=0.))*float(np.abs(x0).max(initial=1.))/max(tolerance, 1e-300)
    scale = max(gnorm, np.linalg.norm(load), floor, 1e-300)
    for iteration in range(max_iterations + 1):
        if gnorm <= tolerance*scale:
            return u, t, dict(newton_iterations=iteration, relative_gradient=gnorm/scale, energy=phi)
        if iteration == max_iterations:
            break
        n, ri, rj, k = energy_tangent(bonds, theta, x, q)
        h = sparse_stiffness(n_sites, np.stack((bonds.i, bonds.j), 1), n, ri, rj, *k.T)
        if inertia is not None:
            dt = inertia[0]
            h = h + sp.diags(np.repeat(np.stack((bonds.mass, bonds.inertia), 1), 3, axis=1).ravel()/(dt*dt))
        d = np.zeros(6*n_sites)
        d[free] = _block_jacobi_cg(h[free][:, free].tocsr(), -g.ravel()[free], 1e-10)
        d = d.reshape(-1, 6)
        slope = float((g*d).sum())
        if not slope < 0:
            d, slope = -g, -gnorm*gnorm
        step = 1.
        for _ in range(30):
            cand = evaluate(u + step*d[:, :3], t + step*d[:, 3:])
            cnorm = np.linalg.norm(cand[1])
            drop = cand[0] - phi
            if drop <= 1e-4*step*slope or (abs(drop) <= 1e-13*max(abs(phi), 1.) and cnorm < gnorm):
                break
            step *= .5
        else:
            raise RuntimeError('energy Newton line search failed')
        u, t = u + step*d[:, :3], t + step*d[:, 3:]
        phi, g, x, q = cand
        gnorm = cnorm
    raise RuntimeError(f'energy Newton did not converge ({gnorm/scale:g})')
