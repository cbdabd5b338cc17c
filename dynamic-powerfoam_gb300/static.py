"""Static linear equilibrium of bonded networks on the GPU.

``reference_stiffness`` (``experiments/bonded_dem_dynamics.py:22-47``)
assembles the stress-free 6N x 6N stiffness as a CUDA sparse CSR tensor;
``solve_prescribed`` (``experiments/bonded_dem_material.py:53-65``) solves
K q = load with prescribed DOFs eliminated, matrix-free: conjugate gradients
on the free DOFs with the CUDA K q product (``dpf_stiffness_apply``) and a
block-Jacobi preconditioner from the CUDA 6x6 diagonal blocks restricted to
each site's free DOFs, and the reference's acceptance test on the true
residual.
"""
import ctypes

import numpy as np
import torch

from . import _lib
from .newton import F64


def _skew(v):
    s = torch.zeros(v.shape[:-1] + (3, 3), dtype=v.dtype, device=v.device)
    s[..., 0, 1], s[..., 0, 2] = -v[..., 2], v[..., 1]
    s[..., 1, 0], s[..., 1, 2] = v[..., 2], -v[..., 0]
    s[..., 2, 0], s[..., 2, 1] = -v[..., 1], v[..., 0]
    return s


class _Tangent:
    """Frozen stress-free tangent of a bonded network: graph, stiffnesses,
    normal and levers, with the CUDA K q and diagonal blocks."""

    def __init__(self, bonds):
        self.lib = _lib.load()
        if hasattr(bonds, 'failure'):         # ParallelBonds
            if bool(torch.any(bonds.failure != 0)) or any(bool(torch.any(getattr(bonds, k) != 0))
                                                          for k in ('fn', 'fs', 'mt', 'mb')):
                raise ValueError('Reference tangent requires an intact, stress-free state')
            n, c = bonds.geometry(bonds.x)
            self.n = n.contiguous()
            self.ri = (c - bonds.x[bonds.i]).contiguous()
            self.rj = (c - bonds.x[bonds.j]).contiguous()
            self.n_sites = len(bonds.x)
        else:                                  # LinearBonds and its subclasses
            self.n, self.ri, self.rj = (getattr(bonds, k).contiguous() for k in ('n', 'ri', 'rj'))
            self.n_sites = bonds.n_sites
        self.k = tuple(getattr(bonds, k).contiguous() for k in ('kn', 'ks', 'kb', 'kt'))
        self.i, self.j = bonds.i, bonds.j
        self.device = self.n.device
        self.graph = bonds._graph
        m = int(self.graph.n_bonds)
        self.wrench = torch.empty(max(1, 9*m), dtype=F64, device=self.device)
        self.stiffness = _lib.Stiffness(*(t.data_ptr() for t in self.k))
        self.tangent = _lib.Tangent(self.n.data_ptr(), self.ri.data_ptr(), self.rj.data_ptr())

    def stream(self):
        return torch.cuda.current_stream(self.device).cuda_stream

    def apply(self, q):
        q = q.contiguous()
        out = torch.empty_like(q)
        _lib.check(self.lib.dpf_stiffness_apply(ctypes.byref(self.graph), ctypes.byref(self.stiffness),
                                                ctypes.byref(self.tangent), q.data_ptr(), out.data_ptr(),
                                                self.wrench.data_ptr(), self.stream()), 'dpf_stiffness_apply')
        return out

    def diagonal(self):
        out = torch.empty((self.n_sites, 6, 6), dtype=F64, device=self.device)
        _lib.check(self.lib.dpf_diagonal_blocks(ctypes.byref(self.graph), ctypes.byref(self.stiffness),
                                                ctypes.byref(self.tangent), out.data_ptr(), self.stream()),
                   'dpf_diagonal_blocks')
        return out


@torch.no_grad()
def reference_stiffness(bonds):
    """Sparse K (CUDA CSR, float64) for q = [u, theta] per body from
    U = du.D.du/2 + dtheta.H.dtheta/2 at the stress-free state
    (``bonded_dem_dynamics.py:22-47``): per bond B^T D B + A^T H A."""
    t = _Tangent(bonds)
    m, dev = len(t.n), t.device
    eye = torch.eye(3, dtype=F64, device=dev).expand(m, 3, 3)
    b = torch.zeros((m, 3, 12), dtype=F64, device=dev)
    a = torch.zeros((m, 3, 12), dtype=F64, device=dev)
    b[:, :, :3], b[:, :, 3:6], b[:, :, 6:9], b[:, :, 9:12] = -eye, _skew(t.ri), eye, -_skew(t.rj)
    a[:, :, 3:6], a[:, :, 9:12] = -eye, eye
    kn, ks, kb, kt = t.k
    nn = t.n[:, :, None]*t.n[:, None, :]
    d = ks[:, None, None]*eye + (kn - ks)[:, None, None]*nn
    h = kb[:, None, None]*eye + (kt - kb)[:, None, None]*nn
    local = torch.einsum('eai,eab,ebj->eij', b, d, b) + torch.einsum('eai,eab,ebj->eij', a, h, a)
    ar6 = torch.arange(6, device=dev)
    idx = torch.cat((6*t.i[:, None] + ar6, 6*t.j[:, None] + ar6), 1)
    rows = idx[:, :, None].expand(m, 12, 12).reshape(-1)
    cols = idx[:, None, :].expand(m, 12, 12).reshape(-1)
    size = 6*t.n_sites
    k = torch.sparse_coo_tensor(torch.stack((rows, cols)), local.reshape(-1), (size, size)).coalesce()
    import warnings
    with warnings.catch_warnings():
        warnings.simplefilter("ignore", UserWarning)  # torch marks sparse CSR as beta
        return k.to_sparse_csr()


@torch.no_grad()
def solve_prescribed(k, prescribed, values, load=None, tolerance=1e-12, max_iterations=20000):
    """Static equilibrium with exact elimination of the prescribed DOFs
    (``bonded_dem_material.py:53-65``).

    ``k`` is a bonded network on the GPU (``ParallelBonds``, ``LinearBonds``
    or a subclass; solved matrix-free) or a CUDA matrix (dense or sparse CSR
    from ``reference_stiffness``).  ``prescribed`` (N, 6) bool, ``values``
    (N, 6), ``load`` (N, 6) or None.  Returns (q flattened (6N,), relative
    residual); raises AssertionError like the reference when the true
    residual exceeds 1e-8.
    """
    if torch.is_tensor(k):
        device, size = k.device, k.shape[0]
        if size > 6*4096:
            raise ValueError('pass the bonded network itself (matrix-free) for systems above 4096 sites')
        matvec = lambda q: (k@q.reshape(-1)).reshape(q.shape)
        dense = k.to_dense() if k.layout != torch.strided else k
        sites = torch.arange(size//6, device=device)
        blocks = dense.reshape(size//6, 6, size//6, 6)[sites, :, sites, :]
    else:
        t = _Tangent(k)
        device, size = t.device, 6*t.n_sites
        matvec = t.apply
        blocks = t.diagonal()
    n = size//6
    mask = torch.as_tensor(np.asarray(prescribed, dtype=bool), device=device).reshape(n, 6)
    free = (~mask).to(F64)
    q = torch.as_tensor(np.asarray(values, dtype=np.float64), device=device).reshape(n, 6).clone()
    rhs = torch.zeros((n, 6), dtype=F64, device=device) if load is None else \
        torch.as_tensor(np.asarray(load, dtype=np.float64), device=device).reshape(n, 6).clone()
    fixed_part = q*mask.to(F64)
    b = (rhs - matvec(fixed_part))*free
    # block-Jacobi on the free DOFs: each site's 6x6 block with prescribed rows
    # and columns replaced by the identity
    eye = torch.eye(6, dtype=F64, device=device)
    fm = free[:, :, None]*free[:, None, :]
    pre = torch.linalg.inv(blocks*fm + torch.diag_embed(1. - free)*eye)
    precondition = lambda r: torch.einsum('nij,nj->ni', pre, r)*free
    operator = lambda d: matvec(d*free)*free
    norm_b = float(torch.linalg.vector_norm(b))
    x = torch.zeros_like(b)
    if norm_b > 0:
        r = b.clone()
        z = precondition(r)
        d = z.clone()
        rz = float((r*z).sum())
        for _ in range(max_iterations):
            ad = operator(d)
            alpha = rz/float((d*ad).sum())
            x += alpha*d
            r -= alpha*ad
            if float(torch.linalg.vector_norm(r)) <= tolerance*norm_b:
                break
            z = precondition(r)
            following = float((r*z).sum())
            d = z + (following/rz)*d
            rz = following
    q = x*free + fixed_part
    reaction = matvec(q) - rhs
    fixed_mask = mask.to(F64)
    scale = max(float(torch.linalg.vector_norm(rhs)), float(torch.linalg.vector_norm(reaction*fixed_mask)), 1e-30)
    residual = float(torch.linalg.vector_norm(reaction*free))/scale
    if not bool(torch.isfinite(q).all()) or residual > 1e-8:
        raise AssertionError(f'Unresolved static equilibrium, relative residual {residual}')
    return q.reshape(-1), residual
