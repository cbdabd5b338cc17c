"""Serving form: continuous batching of Newton solve requests on one GPU.

A *batch* is the disjoint union of the active requests' bond graphs
(concatenated sites, bonds and incidence lists, built on the device from the
requests' resident tensors).  Every kernel launch of a batched Newton step
covers all requests at once; each request still follows its own control flow
of ``NewtonBonds.step`` (``experiments/bonded_dem_newton.py:132-201``):

* per-request scalars (rhs scale, residual norm, pose defect, merit, work) come
  from segmented reductions (``dpf_segment_norms``), guard failures from
  per-request status words (``dpf_mixed_residual_segmented``);
* a request that has converged is frozen: its rows of the Newton right-hand
  side are zero, which keeps its blocks exactly zero through FGMRES and the
  block-diagonal PCG, so its increment stays put while others iterate;
* the backtracking line search runs with one step factor per request.

The shared FGMRES/PCG over the batch only changes how accurately each Newton
direction is computed, not the converged answer: every request stops at its
own relative residual and pose tolerance, so a request's result agrees alone
and in any mix within that tolerance.

``Service`` admits requests by HBM footprint into free batch capacity at the
boundaries of batched steps (requests arriving while a batch runs join the
next one), keeps each request's state resident until it has done all its time
steps, and records per-request latency.
"""
import ctypes
import threading
import time
from concurrent.futures import ThreadPoolExecutor
from dataclasses import dataclass, field

import numpy as np
import torch

from . import _lib
from .newton import (MixedNewtonBonds, NewtonBonds, SubdivideError, guard_error, _Krylov, fgmres, F64, incidence,
                     device_incidence)

_PER_SITE = ('p', 'mass', 'fixed', 'radii', 'x', 'v', 'rotation', '_mass32')
_PER_BOND = ('n', 'ri', 'rj', 'kn', 'ks', 'kb', 'kt', 'normal', 'offset', 'fn', 'fs', 'mt', 'mb')
_STATE = ('x', 'v', 'rotation', 'normal', 'offset', 'fn', 'fs', 'mt', 'mb')


class Staging:
    """Reusable pinned host buffers for uploads (pinned allocations are slow)."""

    def __init__(self):
        self.buffers = {}

    def host(self, kind, count):
        """A pinned host array of ``count`` elements of numpy kind ``kind`` to fill."""
        dtype = np.dtype(kind)
        buf = self.buffers.get(dtype.str)
        if buf is None or buf.numel() < count:
            buf = torch.empty(max(count, 1 << 20), dtype=torch.from_numpy(np.zeros(0, dtype)).dtype).pin_memory()
            self.buffers[dtype.str] = buf
        return buf[:count].numpy()

    def send(self, kind, count, device):
        """Upload the first ``count`` elements of the pinned buffer of ``kind``."""
        buf = self.buffers[np.dtype(kind).str][:count]
        out = buf.to(device, non_blocking=True)
        torch.cuda.current_stream(device).synchronize()
        return out

    def upload(self, array, device):
        array = np.ascontiguousarray(array)
        key = array.dtype.str
        need = array.size
        buf = self.buffers.get(key)
        if buf is None or buf.numel() < need:
            buf = torch.empty(max(need, 1 << 20), dtype=torch.from_numpy(array[:0]).dtype).pin_memory()
            self.buffers[key] = buf
        view = buf[:need]
        view.numpy()[...] = array.ravel()
        out = view.to(device, non_blocking=True)
        # the pinned buffer is reused by the next upload: wait for this copy
        torch.cuda.current_stream(device).synchronize()
        return out.view(array.shape)


_LOCAL = threading.local()
_PREFETCH = ThreadPoolExecutor(max_workers=1)
_COPIERS = ThreadPoolExecutor(max_workers=8)


def _staging():
    """The calling thread's pinned staging buffers."""
    if not hasattr(_LOCAL, 'staging'):
        _LOCAL.staging = Staging()
    return _LOCAL.staging


class RequestState:
    """Resident state of one or several requests: exactly what a ``Batch``
    concatenates (the attributes of fresh ``MixedNewtonBonds`` solvers, without
    solver scratch), set up on the device with one ``dpf_bond_setup`` and one
    device sort of the incidence list for the whole group."""

    def __init__(self, points, radii, pairs, areas, masses, fixed, contacts=None, young=1200., shear=480.,
                 device='cuda'):
        self._build([dict(points=points, radii=radii, pairs=pairs, areas=areas, masses=masses, fixed=fixed,
                          contacts=contacts, young=young, shear=shear)], device)

    @classmethod
    def group(cls, foams, device='cuda', loads=None):
        """Several requests' foams as one resident state (sites and bonds in
        order); with ``loads`` (one (n, 6) array per foam) also their external
        loads, uploaded with the rest as ``external``."""
        self = cls.__new__(cls)
        self._build(foams, device, loads)
        return self

    def _build(self, foams, device, loads=None):
        self.device = torch.device(device)
        if self.device.index is None:
            self.device = torch.device('cuda', torch.cuda.current_device())
        self._lib = _lib.load()
        self.tensor = lambda a: torch.as_tensor(a, dtype=F64, device=self.device)
        if any(f.get('contacts') is not None for f in foams):
            raise ValueError('explicit contacts are not supported in a group; use MixedNewtonBonds')
        sites = [len(f['points']) for f in foams]
        bonds = [len(f['pairs']) for f in foams]
        self.sites, self.bonds = sites, bonds
        so = np.concatenate(([0], np.cumsum(sites))).astype(np.int64)
        bo = np.concatenate(([0], np.cumsum(bonds))).astype(np.int64)
        n, m = int(so[-1]), int(bo[-1])
        # one copy of each input into pinned staging: per-site float64 [points, radii,
        # masses], per-bond float64 areas, int32 endpoints (global ids), uint8 flags
        staging = _staging()
        n_load = 6*n if loads is not None else 0
        f64 = staging.host('f8', 5*n + m + n_load)
        u8 = staging.host('u1', n)
        i32 = staging.host('i4', 2*m)
        pts, rad, mas, are = f64[:3*n].reshape(n, 3), f64[3*n:4*n], f64[4*n:5*n], f64[5*n:5*n + m]
        ext = f64[5*n + m:5*n + m + n_load].reshape(-1, 6)
        ends = i32.reshape(-1, 2)
        bad = []

        def copy(k):
            f = foams[k]
            a, b, c, d = so[k], so[k+1], bo[k], bo[k+1]
            pts[a:b] = f['points']
            rad[a:b] = f['radii']
            mas[a:b] = f['masses']
            are[c:d] = f['areas']
            u8[a:b] = np.asarray(f['fixed'], dtype=bool)
            if n_load:
                ext[a:b] = loads[k]
            # the request's bonds with group-wide site ids (int32)
            pairs = np.asarray(f['pairs']).reshape(-1, 2)
            if len(pairs) and (pairs.min() < 0 or pairs.max() >= sites[k]):
                bad.append(k)
            np.add(pairs, a, out=ends[c:d], casting='unsafe')
        # numpy releases the GIL for these copies: spread the requests over threads
        list(_COPIERS.map(copy, range(len(foams))))
        if bad:
            raise ValueError('Invalid endpoint index')
        if np.any(mas <= 0):
            raise ValueError('Only positive-mass bodies can enter this solver')
        dev64 = staging.send('f8', 5*n + m + n_load, self.device)
        # one upload of the group's bonds and one device sort for its incidence CSR
        edges = staging.send('i4', 2*m, self.device).view(-1, 2).to(torch.int64).contiguous()
        inc_ptr, inc_bond = device_incidence(edges, n)
        self.external = dev64[5*n + m:].view(n, 6) if n_load else None
        self.fixed = staging.send('u1', n, self.device).view(torch.bool)
        self.p = dev64[:3*n].view(n, 3)
        self.radii = dev64[3*n:4*n]
        masses_d, areas_d = dev64[4*n:5*n], dev64[5*n:5*n + m]
        self.n_sites, self.n_bonds = n, m
        e = lambda *shape: torch.empty(shape, dtype=F64, device=self.device)
        self.n, self.ri, self.rj, self.offset = e(m, 3), e(m, 3), e(m, 3), e(m, 3)
        self.kn, self.ks, self.kb, self.kt = e(m), e(m), e(m), e(m)
        self.mass = e(n, 6)
        stream = torch.cuda.current_stream(self.device).cuda_stream
        _lib.check(self._lib.dpf_bond_setup(n, m, edges.data_ptr() if m else None, self.p.data_ptr(),
                                            self.radii.data_ptr(), areas_d.data_ptr(), None, masses_d.data_ptr(),
                                            1., 1., None, None, self.n.data_ptr(), self.ri.data_ptr(),
                                            self.rj.data_ptr(), self.kn.data_ptr(), self.ks.data_ptr(),
                                            self.kb.data_ptr(), self.kt.data_ptr(), self.offset.data_ptr(),
                                            self.mass.data_ptr(), stream), 'dpf_bond_setup')
        # per-request moduli (kn, kb scale with E; ks, kt with G)
        counts = torch.as_tensor(bonds, device=self.device)
        E = torch.repeat_interleave(self.tensor([float(f['young']) for f in foams]), counts)
        G = torch.repeat_interleave(self.tensor([float(f['shear']) for f in foams]), counts)
        self.kn.mul_(E); self.kb.mul_(E); self.ks.mul_(G); self.kt.mul_(G)
        self.edges = edges
        self._mass32 = self.mass.float()
        self.x = self.p.clone()
        self.normal = self.n.clone()
        self.fn, self.mt = torch.zeros_like(self.kn), torch.zeros_like(self.kn)
        self.fs, self.mb = torch.zeros_like(self.n), torch.zeros_like(self.n)
        self.v = torch.zeros_like(self.mass)
        self.rotation = torch.eye(3, dtype=F64, device=self.device).repeat(n, 1, 1)
        self._inc_ptr, self._inc_bond = inc_ptr, inc_bond
        self.time = 0.


def concat_incidence(parts, site_off, bond_off):
    """Incidence CSR of parts laid end to end (part k's sites from
    ``site_off[k]``, its bonds from ``bond_off[k]``) from the parts' own CSRs:
    the rows of part k follow the rows of part k - 1 with its bond ids
    shifted (v >= 0: the site is the i end of bond v; ~v: the j end).  Equal,
    entry for entry, to ``device_incidence`` of the concatenated edges: that
    stable sort orders a site's ends by (side, bond), which the shift keeps."""
    ptrs, incs = [], []
    for k, p in enumerate(parts):
        ptr = p._inc_ptr[:-1] if k + 1 < len(parts) else p._inc_ptr
        ptrs.append(ptr + 2*int(bond_off[k]))
        v, b = p._inc_bond, int(bond_off[k])
        incs.append(torch.where(v >= 0, v + b, v - b))
    return torch.cat(ptrs).contiguous(), torch.cat(incs).contiguous()


def slice_incidence(inc_ptr, inc_bond, sites, incidences, first_bond):
    """The rows of sites [s0, s1) of an incidence CSR (their incidences
    [e0, e1), bonds from ``first_bond`` on) as a CSR of their own sites and
    bonds: the inverse of ``concat_incidence``."""
    (s0, s1), (e0, e1) = sites, incidences
    ptr = inc_ptr[s0:s1 + 1]
    v = inc_bond[e0:e1]
    return ptr - ptr[0], torch.where(v >= 0, v - first_bond, v + first_bond)


def _warm_incidence_ops(device):
    """Run ``concat_incidence`` and ``slice_incidence`` once on a two-part toy
    graph: the first launch of a device kernel in a process can cost a module
    load (about 3 s was measured on a GB300 host for these int32 ops), which
    should not land inside the first batch that joins two parts."""
    ptr = torch.tensor([0, 1, 2], dtype=torch.int32, device=device)
    inc = torch.tensor([0, -1], dtype=torch.int32, device=device)
    part = _IncidencePart(ptr, inc)
    joined = concat_incidence([part, part], [0, 2, 4], [0, 1, 2])
    slice_incidence(*joined, (2, 4), (2, 4), 1)
    if device.type == 'cuda':
        torch.cuda.synchronize(device)


@dataclass
class _IncidencePart:
    _inc_ptr: torch.Tensor
    _inc_bond: torch.Tensor


class Slice:
    """One request's state inside a previous batch (views, no copies), ready
    to be concatenated into the next batch."""

    def __init__(self, batch, k):
        s0, s1 = batch.site_range[k]
        b0, b1 = batch.bond_range[k]
        self.device, self._lib, self.tensor = batch.device, batch._lib, batch.tensor
        self.n_sites, self.n_bonds = s1 - s0, b1 - b0
        for name in _PER_SITE:
            setattr(self, name, getattr(batch, name)[s0:s1])
        for name in _PER_BOND:
            setattr(self, name, getattr(batch, name)[b0:b1])
        self.edges = batch.edges[b0:b1] - s0
        self._inc_ptr, self._inc_bond = slice_incidence(batch._inc_ptr, batch._inc_bond, (s0, s1),
                                                        batch.inc_range[k], b0)
        self.time = batch.time


class Pool:
    """Batch scratch, allocated once for the largest batch and carved per batch."""

    def __init__(self, device, max_sites, max_bonds):
        lib = _lib.load()
        self.max_sites, self.max_bonds = int(max_sites), int(max_bonds)
        n, m = self.max_sites, self.max_bonds
        self.f64 = torch.empty(9*m + 3*6*n + 65*6*n + 1024, dtype=F64, device=device)
        self.f32 = torch.empty(lib.dpf_mixed_bond_floats(m) + lib.dpf_mixed_wrench_floats(m) + 2*36*n + 3*6*n +
                               lib.dpf_mixed_workspace_floats(n, m) + lib.dpf_end_floats(m) +
                               (4 + 24)*n + lib.dpf_tiled_workspace_floats(n) + 4096,
                               dtype=torch.float32, device=device)

    def carve(self, n, m):
        if n > self.max_sites or m > self.max_bonds:
            raise ValueError('batch exceeds the pool')
        o64, o32 = [0], [0]

        def take64(count, shape=None):
            start = o64[0]; o64[0] += (count + 31)//32*32
            v = self.f64[start:start + count]
            return v.view(shape) if shape else v

        def take32(count, shape=None):
            start = o32[0]; o32[0] += (count + 63)//64*64
            v = self.f32[start:start + count]
            return v.view(shape) if shape else v
        return take64, take32


class Batch(MixedNewtonBonds):
    """Union of resident ``MixedNewtonBonds`` requests (no host-side rebuild)."""

    _active_mask = None
    # a batch of a size class not yet tuned takes the launch shape of a tuned
    # class up to two classes (4x in incidences) away: batch sizes follow the
    # arrivals, and timing the shapes inside a step costs more than it saves
    _tune_nearest = 2

    def __init__(self, parts, pool=None):
        if not parts:
            raise ValueError('empty batch')
        first = parts[0]
        self.parts = list(parts)
        self.device = first.device
        self._lib = first._lib
        self.tensor = first.tensor
        # segments: one per request (a group part holds several requests)
        seg_sites, seg_bonds = [], []
        for p in parts:
            seg_sites += list(getattr(p, 'sites', [p.n_sites]))
            seg_bonds += list(getattr(p, 'bonds', [p.n_bonds]))
        self.n_requests = len(seg_sites)
        sites = [p.n_sites for p in parts]
        bonds = [p.n_bonds for p in parts]
        site_off = np.concatenate(([0], np.cumsum(sites)))
        bond_off = np.concatenate(([0], np.cumsum(bonds)))
        n, m = int(site_off[-1]), int(bond_off[-1])
        rs = np.concatenate(([0], np.cumsum(seg_sites)))
        rb = np.concatenate(([0], np.cumsum(seg_bonds)))
        self.site_ptr = torch.as_tensor(rs, dtype=torch.int64, device=self.device)
        self.site_range = [(int(rs[k]), int(rs[k+1])) for k in range(self.n_requests)]
        self.bond_range = [(int(rb[k]), int(rb[k+1])) for k in range(self.n_requests)]
        # a request's incidences: the CSR rows of its sites (two per bond, contiguous)
        self.inc_range = [(2*int(rb[k]), 2*int(rb[k+1])) for k in range(self.n_requests)]
        if len(parts) == 1 and isinstance(first, RequestState):
            # a freshly set-up group alone: use its tensors and incidence as they
            # are (the step replaces state tensors, it never writes into them)
            for name in _PER_SITE + _PER_BOND:
                setattr(self, name, getattr(first, name))
            self.edges = first.edges
            self._inc_ptr, self._inc_bond = first._inc_ptr, first._inc_bond
        else:
            for name in _PER_SITE + _PER_BOND:
                setattr(self, name, torch.cat([getattr(p, name).contiguous() for p in parts]))
            self.edges = torch.cat([p.edges + int(site_off[k]) for k, p in enumerate(parts)]).contiguous()
            self._inc_ptr, self._inc_bond = concat_incidence(parts, site_off, bond_off)
        self.i, self.j = self.edges.T
        R = self.n_requests
        self.seg_site = torch.repeat_interleave(torch.arange(R, dtype=torch.int32, device=self.device),
                                                torch.as_tensor(seg_sites, device=self.device)).contiguous()
        self.seg_bond = torch.repeat_interleave(torch.arange(R, dtype=torch.int32, device=self.device),
                                                torch.as_tensor(seg_bonds, device=self.device)).contiguous()
        self._graph = _lib.Graph(n, m, self.edges.data_ptr() if m else None, self._inc_ptr.data_ptr(),
                                 self._inc_bond.data_ptr())
        lib, dev, f32 = self._lib, self.device, torch.float32
        if pool is not None:
            take64, take32 = pool.carve(n, m)
        else:
            take64 = lambda count, shape=None: torch.empty(shape or (count,), dtype=F64, device=dev)
            take32 = lambda count, shape=None: torch.empty(shape or (count,), dtype=f32, device=dev)
        self._wrench = take64(max(1, 9*m))
        self._partials = torch.zeros(lib.dpf_partials_doubles(), dtype=F64, device=dev)
        self._status = torch.zeros(max(1, R), dtype=torch.int32, device=dev)
        self._scalars = torch.zeros(8, dtype=F64, device=dev)
        self._host_status = torch.zeros(1, dtype=torch.int32).pin_memory()
        self._host_scalars = torch.zeros(64, dtype=F64).pin_memory()
        self.q = self.kq = self.diagonal = None
        self.preconditioner, self.preconditioner_dt = None, None
        self.time = 0.
        self._inner = torch.zeros(1, dtype=torch.int32, device=dev)
        self._inner_host = 0
        self._pcg_workspace = None
        self._barrier = torch.zeros(2, dtype=torch.int32, device=dev)
        self._krylov = _Krylov.__new__(_Krylov)
        self._krylov.length, self._krylov.width = 6*n, 32
        self._krylov.basis = take64(33*6*n, (33, 6*n))
        self._krylov.transformed = take64(32*6*n, (32, 6*n))
        self._krylov.h = torch.zeros(72, dtype=F64, device=dev)
        self.block = self.units = None
        self.profile = None
        self._bond_data = take32(max(4, lib.dpf_mixed_bond_floats(m)))
        self._wrench32 = take32(max(4, lib.dpf_mixed_wrench_floats(m)))
        self._r0 = take64(6*n, (n, 6))
        self._block32 = take32(36*n, (n, 6, 6))
        self._p32 = take32(36*n, (n, 6, 6))
        self._units = take64(6*n, (n, 6))
        self._units32 = take32(6*n, (n, 6))
        self._y32 = take32(6*n, (n, 6))
        self._d32 = take32(6*n, (n, 6))
        self._mixed_workspace = take32(lib.dpf_mixed_workspace_floats(n, m))
        # bond-end sweep of the elastic PCG
        self._ends = take32(max(4, lib.dpf_end_floats(m)))
        self._site4 = take32(4*n, (n, 4))
        self._p24 = take32(24*n)
        self._tiled_workspace = take32(lib.dpf_tiled_workspace_floats(n))
        self._tiled_partials = torch.zeros(lib.dpf_tiled_partials_doubles(), dtype=F64, device=dev)
        self._tune_iterations = torch.zeros(1, dtype=torch.int32, device=dev)
        self._sweep_ready = True
        self._packed = None
        self._tiles = None
        self._end_variant = None       # bond-end sweep launch shape, from the autotuner's size-class cache
        self.tile_timings = {}
        self._cached = None
        self._loads = take64(6*n, (n, 6))
        self._token = None
        self._since_refresh = 0
        self._seg_norms = torch.zeros((R, 3), dtype=F64, device=dev)
        self._seg_norms2 = torch.zeros((R, 3), dtype=F64, device=dev)
        self._seg_partials = torch.empty(max(1, lib.dpf_segment_partials_doubles(R)), dtype=F64, device=dev)
        self._host_seg = torch.zeros((2, R, 3), dtype=F64).pin_memory()
        self._host_seg_status = torch.zeros(R, dtype=torch.int32).pin_memory()

    @property
    def n_segments(self):
        return self.n_requests

    def request_state(self, k):
        """Views of request k's committed state inside the batch."""
        s0, s1 = self.site_range[k]
        b0, b1 = self.bond_range[k]
        return {name: getattr(self, name)[s0:s1] if name in ('x', 'v', 'rotation') else getattr(self, name)[b0:b1]
                for name in _STATE}

    def scatter_state(self):
        """Copy the batch's committed state back into its parts' own tensors."""
        site0 = bond0 = 0
        for p in self.parts:
            for name in _STATE:
                src = getattr(self, name)
                rows = (slice(site0, site0 + p.n_sites) if name in ('x', 'v', 'rotation')
                        else slice(bond0, bond0 + p.n_bonds))
                setattr(p, name, src[rows].clone())
            p.time = self.time
            site0 += p.n_sites
            bond0 += p.n_bonds

    # ---- per-request reductions ---------------------------------------------------
    def _segment(self, a, b=None, b_dot=False, mask=None, out=None):
        out = self._seg_norms if out is None else out
        self._call('dpf_segment_norms', self.n_segments, self.site_ptr.data_ptr(), a.data_ptr(),
                   None if b is None else b.data_ptr(), int(b_dot), None if mask is None else mask.data_ptr(),
                   out.data_ptr(), self._seg_partials.data_ptr(), self._stream())
        return out

    def _fetch_segments(self, second=False, status=False):
        self._host_seg[0].copy_(self._seg_norms, non_blocking=True)
        if second:
            self._host_seg[1].copy_(self._seg_norms2, non_blocking=True)
        if status:
            self._host_seg_status.copy_(self._status[:self.n_segments], non_blocking=True)
        torch.cuda.current_stream(self.device).synchronize()
        return (self._host_seg[0].numpy().copy(), self._host_seg[1].numpy().copy() if second else None,
                self._host_seg_status.numpy().copy() if status else None)

    def _residual_segmented(self, y, dt, want_tangent, use_p, scaled=None):
        r = torch.empty_like(y)
        self._to_y32(y)
        self._status.zero_()
        self._call('dpf_mixed_residual_segmented', ctypes.byref(self._graph), self._bond_data.data_ptr(),
                   y.data_ptr(), self._y32.data_ptr(), self.mass.data_ptr(), self.fixed.data_ptr(), dt,
                   self._r0.data_ptr(), int(want_tangent), self._p32.data_ptr() if use_p else None,
                   self._units32.data_ptr() if use_p else None, r.data_ptr(),
                   _addr_or_none(scaled) if use_p else None, None, self._wrench32.data_ptr(),
                   self._partials.data_ptr(), self._status.data_ptr(), self.seg_bond.data_ptr(),
                   self.seg_site.data_ptr(), self._bond_mask()[1], self._stream())
        return r

    def _bond_mask(self):
        if self._active_mask is None:
            return None, None
        return self.seg_bond.data_ptr(), self._active_mask.data_ptr()

    def _site_mask(self):
        if self._active_mask is None:
            return None, None
        return self.seg_site.data_ptr(), self._active_mask.data_ptr()

    def _set_active(self, requests):
        """Bond passes of the following launches skip every request not in
        ``requests`` (their sites' rows of those passes are not read)."""
        if len(requests) == self.n_segments:
            self._active_mask = None
            return
        flags = np.zeros(self.n_segments, dtype=np.uint8)
        flags[list(requests)] = 1
        self._active_mask = torch.as_tensor(flags).to(self.device)

    # ---- the batched Newton step ------------------------------------------------------
    @torch.no_grad()
    def step_batch(self, dt, external, tolerance=1e-6, max_iterations=12, *, pose_tolerance=2e-6,
                   linear_tolerance=1e-6):
        """One implicit-midpoint Newton solve for every request of the batch.

        Returns one entry per request: ``(work, info)`` or the ``SubdivideError``
        that request raised (its state is left untouched).
        """
        R, dt = self.n_segments, float(dt)
        linear_tolerance = max(linear_tolerance, self.min_linear_tolerance)
        external = self._vec(external)
        self._v = self._vec(self.v).clone()
        self._status.zero_()
        MixedNewtonBonds._step_begin(self, dt, external)     # r0, maintained loads (global)
        self._deferred_scale = None                           # per-request scales come from segments
        h = .5*dt*dt
        rhs_vec = -(self._r0 + h*self._loads)                 # dt M v + dt^2/2 ext
        self._segment(rhs_vec)
        self._segment(self._loads, mask=self.fixed, out=self._seg_norms2)
        first, second, _ = self._fetch_segments(second=True)
        rhs_scale = np.maximum(np.maximum(first[:, 0], h*second[:, 0]), 1e-30)
        y = torch.zeros_like(self._v)
        n6 = 6*self.n_sites
        stream = self._stream()
        done = [None]*R                 # None: active; dict: converged info; Exception: failed
        trace = [[] for _ in range(R)]
        iters = np.zeros(R, dtype=np.int64)
        krylov = np.zeros(R, dtype=np.int64)
        cg = np.zeros(R, dtype=np.int64)
        self._active_mask = None
        for iteration in range(max_iterations+1):
            self._set_active([k for k in range(R) if done[k] is None])
            r = self._residual_segmented(y, dt, want_tangent=True, use_p=False)
            self._call('dpf_mixed_scaling', ctypes.byref(self._graph), self._bond_data.data_ptr(),
                       self._mass32.data_ptr(), self.fixed.data_ptr(), self.radii.data_ptr(), dt,
                       self._block32.data_ptr(), self._p32.data_ptr(), self._units.data_ptr(),
                       self._units32.data_ptr(), stream)
            self._packed = None  # new tangent and blocks: repack the end records before the PCG
            scaled = torch.empty_like(r)
            self._call('dpf_mixed_scale_residual', self.n_sites, self._p32.data_ptr(), self._units32.data_ptr(),
                       r.data_ptr(), scaled.data_ptr(), None, None, stream)
            self._segment(r)
            self._segment(scaled, out=self._seg_norms2)
            rn, sn, status = self._fetch_segments(second=True, status=True)
            for k in range(R):
                if done[k] is not None:
                    continue
                if status[k]:
                    done[k] = guard_error(int(status[k]))
                    continue
                relative, local = rn[k, 0]/rhs_scale[k], sn[k, 1]
                if not (np.isfinite(relative) and np.isfinite(local)):
                    done[k] = SubdivideError(f'Subdivide: non-finite Newton residual ({relative:g}, {local:g})')
                    continue
                trace[k].append([relative, local])
                if relative < tolerance and local < pose_tolerance:
                    done[k] = dict(nonlinear_iterations=iteration, nonlinear_relative_residual=relative,
                                   local_pose_defect=local)
            active = [k for k in range(R) if done[k] is None]
            if not active:
                break
            if iteration == max_iterations:
                for k in active:
                    relative, local = trace[k][-1]
                    done[k] = SubdivideError(f'Subdivide: Newton did not converge ({relative:g}, {local:g})')
                break
            self._set_active(active)
            # Each active request's block of the right-hand side is normalised to
            # unit norm (frozen requests: zero), so that the shared Krylov
            # tolerance weighs every request's own relative linear residual
            # alike; the direction is then judged by each request's line search.
            scale = np.zeros(R)
            for k in active:
                scale[k] = -1./max(sn[k, 0], 1e-300)
            sdev = torch.as_tensor(scale, dtype=F64).to(self.device)
            zero = torch.zeros_like(scaled)
            rhs = torch.empty_like(scaled)
            self._call('dpf_segment_axpy', self.n_sites, self.seg_site.data_ptr(), sdev.data_ptr(), zero.data_ptr(),
                       scaled.data_ptr(), rhs.data_ptr(), stream)
            self.inner_iterations = 0
            delta, metrics = fgmres(self._newton_operator(y, dt, external), rhs, self._newton_preconditioner(dt),
                                    tolerance=linear_tolerance, workspace=self._krylov, strict=False)
            unscale = torch.as_tensor(np.where(scale != 0, -1./np.where(scale != 0, scale, 1.), 0.),
                                      dtype=F64).to(self.device)
            delta = delta.contiguous()
            self._call('dpf_segment_axpy', self.n_sites, self.seg_site.data_ptr(), unscale.data_ptr(),
                       zero.data_ptr(), delta.data_ptr(), delta.data_ptr(), stream)
            inner = self.inner_iterations
            for k in active:
                krylov[k] += metrics['iterations']
                cg[k] += inner
                iters[k] = iteration + 1
            correction = torch.empty_like(delta)
            self._call('dpf_masked_scale', self.n_sites, delta.data_ptr(), self._units.data_ptr(),
                       self.fixed.data_ptr(), correction.data_ptr(), stream)
            merit = {k: sn[k, 0] for k in active}
            factor = {k: 1. for k in active}
            pending = list(active)
            candidate = torch.empty_like(y)
            for power in range(10):
                f = np.zeros(R)
                for k in pending:
                    f[k] = factor[k]
                fdev = torch.as_tensor(f, dtype=F64).to(self.device)
                self._call('dpf_segment_axpy', self.n_sites, self.seg_site.data_ptr(), fdev.data_ptr(),
                           y.data_ptr(), correction.data_ptr(), candidate.data_ptr(), stream)
                cscaled = torch.empty_like(y)
                self._set_active(pending)
                self._residual_segmented(candidate, dt, want_tangent=False, use_p=True, scaled=cscaled)
                self._segment(cscaled)
                values, _, status = self._fetch_segments(status=True)
                accept = torch.zeros(R, dtype=torch.uint8)
                still = []
                for k in pending:
                    if status[k] == 0 and values[k, 0] < (1 - 1e-4*factor[k])*merit[k]:
                        accept[k] = 1
                    else:
                        factor[k] *= .5
                        still.append(k)
                if int(accept.sum()):
                    self._call('dpf_segment_select', self.n_sites, self.seg_site.data_ptr(),
                               accept.to(self.device).data_ptr(), candidate.data_ptr(), y.data_ptr(),
                               y.data_ptr(), stream)
                pending = still
                if not pending:
                    break
            for k in pending:
                done[k] = SubdivideError('Subdivide: Newton line search failed')
        self._active_mask = None
        # commit the converged requests; failed ones keep their state
        failed = [k for k in range(R) if isinstance(done[k], Exception)]
        if failed:
            keep_y = torch.zeros(R, dtype=torch.uint8)
            keep_y[[k for k in range(R) if k not in failed]] = 1
            zero = torch.zeros_like(y)
            self._call('dpf_segment_select', self.n_sites, self.seg_site.data_ptr(), keep_y.to(self.device).data_ptr(),
                       y.data_ptr(), zero.data_ptr(), y.data_ptr(), stream)
            saved = {name: getattr(self, name).clone() for name in _STATE}
        self._accept(y, dt)
        self.time += dt
        if failed:
            for k in failed:
                s0, s1 = self.site_range[k]
                b0, b1 = self.bond_range[k]
                for name in _STATE:
                    rows = slice(s0, s1) if name in ('x', 'v', 'rotation') else slice(b0, b1)
                    getattr(self, name)[rows] = saved[name][rows]
            self._token = None
        self._segment(external, b=y, b_dot=True)
        work, _, _ = self._fetch_segments()
        out = []
        for k in range(R):
            if isinstance(done[k], Exception):
                out.append(done[k])
            else:
                info = dict(done[k], krylov_iterations=int(krylov[k]), cg_iterations=int(cg[k]),
                            residual_trace=trace[k])
                out.append((float(work[k, 2]), info))
        return out


def _addr_or_none(t):
    return None if t is None else t.data_ptr()


# ---------------------------------------------------------------------------------
# Requests and the continuous-batching service


@dataclass(order=True)
class Request:
    """One served job: ``steps`` implicit Newton solves of one foam."""
    arrival: float
    rid: int = field(compare=False)
    foam: dict = field(compare=False, repr=False)
    load: np.ndarray = field(compare=False, repr=False)
    dt: float = field(compare=False, default=1e-3)
    steps: int = field(compare=False, default=1)
    # filled by the service
    solver: object = field(compare=False, default=None, repr=False)
    done_steps: int = field(compare=False, default=0)
    started: float = field(compare=False, default=None)
    finished: float = field(compare=False, default=None)
    infos: list = field(compare=False, default_factory=list, repr=False)
    error: Exception = field(compare=False, default=None)
    device_load: object = field(compare=False, default=None, repr=False)

    @property
    def sites(self):
        return len(self.foam['points'])

    @property
    def bonds(self):
        return len(self.foam['pairs'])


def footprint_bytes(sites, bonds):
    """HBM bytes of a resident request's state plus its copy inside a batch.

    Per site: positions, reference points, velocity, rotation, mass (float64
    and float32), radius, flag and incidence pointer; per bond: edges, tangent,
    stiffnesses, history and two incidence entries.  Batch scratch (Krylov
    basis, float32 records, bond-end records, CG vectors) comes from the
    service's pool, counted once.
    """
    per_site = 8*(3 + 3 + 6 + 9 + 6 + 1) + 4*6 + 1 + 4
    per_bond = 16 + 8*(3*3 + 4 + 3*2 + 2 + 3*2) + 8
    return int(2*(per_site*sites + per_bond*bonds))


class Service:
    """Continuous batching of solve requests under an HBM budget.

    ``run(requests)`` plays the request stream in real time (``arrival`` in
    seconds from the start): a request is constructed (resident state on the
    device) once it has arrived, admitted when its footprint fits the budget
    and the batch has room, and solved by batched Newton steps together with
    every other admitted request.  Requests that arrive while a batch step is
    running are set up meanwhile (a collector thread builds them as groups on a
    side stream) and join at the next step boundary.  A batch steps all its
    requests with one dt: admission is in arrival order and stops at a request
    with another dt, which starts the next batch once the current one drains.
    Latency = completion - arrival.
    """

    def __init__(self, device='cuda', hbm_budget=150e9, max_batch_sites=4_000_000, tolerance=1e-6,
                 profile=False):
        self.device = torch.device(device)
        # profile: per batched step, the wall time (with a device sync on either
        # side) and the device time of every library call by entry point
        self.profile = [] if profile else None
        self.hbm_budget = float(hbm_budget)
        self.max_batch_sites = int(max_batch_sites)
        self.tolerance = float(tolerance)
        self.in_use = 0.
        self.batches = 0
        self.timers = dict(setup=0., batch=0., solve=0.)
        self.batch_sizes = []
        self.pool = None
        _warm_incidence_ops(self.device)

    def run(self, requests, clock=time.perf_counter):
        pending = sorted(requests)
        waiting, active, finished = [], [], []
        ready = []           # (requests, group, event): admitted and set up, not yet in a batch
        if self.pool is None:
            largest = max((r.bonds for r in requests), default=1)
            max_bonds = int(self.max_batch_sites*max(r.bonds/max(r.sites, 1) for r in requests)*1.05) + largest
            self.pool = Pool(self.device, self.max_batch_sites + max(r.sites for r in requests), max_bonds)
            self.in_use += self.pool.f64.numel()*8 + self.pool.f32.numel()*4
            # Reserve half of the rest of the budget in the caching allocator up
            # front, so request state is carved from it instead of waiting on
            # device allocations while batches run.
            free = torch.cuda.mem_get_info(self.device)[0]
            spare = int(min(.5*(self.hbm_budget - self.in_use), .5*free))
            if spare > 0:
                block = torch.empty(spare, dtype=torch.uint8, device=self.device)
                del block
        t0 = clock()
        now = lambda: clock() - t0
        batch, members = None, []
        side = torch.cuda.Stream(device=self.device)

        def build(reqs):
            with torch.cuda.stream(side):
                group = RequestState.group([r.foam for r in reqs], device=self.device,
                                           loads=[r.load for r in reqs])
                event = torch.cuda.Event()
                event.record(side)
            for (a, b), r in zip(zip(np.cumsum([0] + group.sites[:-1]), np.cumsum(group.sites)), reqs):
                r.device_load = group.external[int(a):int(b)]
            return group, event

        def admit(room, first_free, dt=None):
            """Arrived requests in arrival order that fit the HBM budget and ``room``
            sites (the first one regardless of ``room`` when ``first_free``) and step
            with ``dt`` (a batch steps all its requests with one dt; None: the
            first one's)."""
            while pending and pending[0].arrival <= now():
                waiting.append(pending.pop(0))
            taken, sites = [], 0
            while waiting:
                req = waiting[0]
                need = footprint_bytes(req.sites, req.bonds)
                if self.in_use + need > self.hbm_budget or \
                        (sites + req.sites > room and not (first_free and not taken)) or \
                        (dt is not None and req.dt != dt) or (taken and req.dt != taken[0].dt):
                    break
                waiting.pop(0)
                self.in_use += need
                req.started = now()
                taken.append(req)
                sites += req.sites
            return taken

        def collect(stop, room, first_free, dt):
            """While a batch step runs: set up the requests that arrive, as groups on
            the side stream, so they join at the next step boundary ready to go."""
            built = []
            while not stop.is_set():
                taken = admit(room, first_free and not built, dt)
                if taken:
                    room -= sum(r.sites for r in taken)
                    built.append((taken, *build(taken)))
                    continue
                wait = pending[0].arrival - now() if pending else .005
                stop.wait(max(2e-4, min(wait, .005)))
            return built

        while pending or waiting or active or ready:
            if not active and not ready:
                # nothing to run: set up what has arrived here (otherwise the
                # collector takes it during the next step)
                taken = admit(self.max_batch_sites, True)
                if taken:
                    t1 = clock()
                    ready.append((taken, *build(taken)))
                    self.timers['setup'] += clock() - t1
            if not active and not ready:
                if pending:
                    time.sleep(max(0., min(pending[0].arrival - now(), .001)))
                continue
            if ready or batch is None:
                # staying requests keep their resident state; the admitted ones join
                # as the groups they were set up in
                t1 = clock()
                parts = [r.part for r in active]
                stream = torch.cuda.current_stream(self.device)
                for reqs, group, event in ready:
                    stream.wait_event(event)
                    for value in vars(group).values():   # set up on the side stream, used here
                        if torch.is_tensor(value) and value.is_cuda:
                            value.record_stream(stream)
                    parts.append(group)
                    active += reqs
                ready = []
                t2 = clock()
                members = list(active)
                batch = Batch(parts, pool=self.pool)
                ext = parts[0].external if len(parts) == 1 and isinstance(parts[0], RequestState) else \
                    torch.cat([r.device_load for r in members])
                t3 = clock()
                self.timers['setup'] += t2 - t1
                self.timers['batch'] += t3 - t2
            # requests arriving during this step are set up meanwhile
            staying = sum(r.sites for r in members if r.done_steps + 1 < r.steps)
            stop = threading.Event()
            future = _PREFETCH.submit(collect, stop, self.max_batch_sites - staying, not staying, members[0].dt)
            if self.profile is not None:
                torch.cuda.synchronize(self.device)
                batch.call_profile = {}
            t4 = clock()
            try:
                results = batch.step_batch(members[0].dt, ext, tolerance=self.tolerance)
                if self.profile is not None:
                    torch.cuda.synchronize(self.device)
                    self.profile.append(_step_profile(batch, results, clock() - t4))
            finally:
                stop.set()
                ready += future.result()
            self.timers['solve'] += clock() - t4
            self.batch_sizes.append([len(members), batch.n_sites])
            self.batches += 1
            leaving = []
            for req, res in zip(members, results):
                if isinstance(res, Exception):
                    req.error = res
                    leaving.append(req)
                    continue
                req.infos.append(res[1])
                req.done_steps += 1
                if req.done_steps >= req.steps:
                    leaving.append(req)
            if leaving or ready or waiting or (pending and pending[0].arrival <= now()):
                stamp = now()
                gone = {id(r) for r in leaving}      # identity: requests compare by arrival time
                for k, req in enumerate(members):
                    if id(req) in gone:
                        req.state = batch.request_state(k)
                        req.finished = stamp
                        finished.append(req)
                        self.in_use -= footprint_bytes(req.sites, req.bonds)
                    else:
                        req.part = Slice(batch, k)
                active = [r for r in active if id(r) not in gone]
                batch = None
        return finished


def _step_profile(batch, results, wall):
    """One batched step of a profiled ``Service``: requests, sites, wall ms,
    the largest Newton / FGMRES / CG counts of its requests and the device ms
    and launch count of every library entry point it called."""
    calls, batch.call_profile = batch.call_profile, None
    infos = [r[1] for r in results if not isinstance(r, Exception)]
    device = {name: [len(ev), round(sum(a.elapsed_time(b) for a, b in ev), 3)] for name, ev in calls.items()}
    return dict(requests=batch.n_segments, sites=batch.n_sites, wall_ms=round(1e3*wall, 2),
                device_ms=round(sum(v[1] for v in device.values()), 2),
                newton=max((i['nonlinear_iterations'] for i in infos), default=0),
                krylov=max((i['krylov_iterations'] for i in infos), default=0),
                cg=max((i['cg_iterations'] for i in infos), default=0), calls=device)


def latency_stats(finished):
    lat = np.array([r.finished - r.arrival for r in finished if r.error is None])
    if not len(lat):
        return dict(p50=None, p99=None, mean=None)
    return dict(p50=float(np.percentile(lat, 50)), p99=float(np.percentile(lat, 99)), mean=float(lat.mean()))


# ---------------------------------------------------------------------------------
# Synthetic request stream (the mixed-size served workload)

_UNIT_FOAMS = {}


def _unit_foam(m, seed):
    """Jittered unit-cube foam of lattice size m (bond graph computed once per (m, seed))."""
    from .foam import jittered_lattice_foam
    key = (m, seed)
    if key not in _UNIT_FOAMS:
        _UNIT_FOAMS[key] = jittered_lattice_foam(m, seed=seed)
    return _UNIT_FOAMS[key]


def compressed_foam_request(m, rng, *, aspect=None, young=None, poisson=None, strain=None, seed=0, density=1000.,
                            base=None):
    """A jittered ``m^3`` foam stretched by box aspect ratios, with its material and top load.

    The bond graph is that of the unit-cube foam ``base`` (default: the cached
    foam of lattice size ``m`` and ``seed``); positions, cross sections, masses
    and lever radii follow the stretched box.  The top layer (unit z > 0.95)
    carries a compressive force equivalent to the nominal strain ``strain``:
    E * strain * (top area) spread over the top sites; gravity acts on every
    free site.
    """
    from .foam import gravity_load
    base = _unit_foam(m, seed) if base is None else base
    aspect = rng.uniform(.5, 2., 3) if aspect is None else np.asarray(aspect, dtype=float)
    young = float(np.exp(rng.uniform(np.log(1e4), np.log(1e6)))) if young is None else young
    poisson = float(rng.uniform(.2, .4)) if poisson is None else poisson
    strain = float(rng.uniform(.01, .1)) if strain is None else strain
    h = base['h']
    scale = float(np.prod(aspect))**(1/3)
    foam = dict(points=base['unit']*aspect, radii=np.full(len(base['unit']), .5*h*scale), pairs=base['pairs'],
                areas=rng.uniform(.5, 1., len(base['pairs']))*(h*scale)**2,
                masses=np.full(len(base['unit']), density*h**3*float(np.prod(aspect))), fixed=base['fixed'],
                contacts=None, young=young, shear=young/(2*(1+poisson)), h=h, unit=base['unit'])
    load = gravity_load(foam)
    top = (base['unit'][:, 2] > .95) & ~base['fixed']
    if top.any():
        load[top, 2] -= young*strain*aspect[0]*aspect[1]/top.sum()
    return foam, load


def stream_plan(count, seed=0, sites=(1024, 131072), rate=None):
    """Per-request parameters of a mixed-size stream in which every request has
    its own foam: lattice size m (m^3 log-uniform in ``sites``, rounded to the
    nearest lattice), foam seed, box aspect ratios U[0.5, 2], E log-uniform
    [1e4, 1e6], nu U[0.2, 0.4], top strain U[1%, 10%] and a Poisson arrival
    time at ``rate`` per second (None: all at t = 0).  The foams themselves
    (the expensive part) are built from the plan by ``planned_stream``."""
    rng = np.random.default_rng(seed)
    arrival, plan = 0., []
    for rid in range(count):
        target = np.exp(rng.uniform(np.log(sites[0]), np.log(sites[1])))
        m = max(2, int(round(target**(1/3))))
        if rate:
            arrival += float(rng.exponential(1./rate))
        plan.append(dict(rid=rid, m=m, foam_seed=int(rng.integers(1 << 31)), aspect=rng.uniform(.5, 2., 3),
                         young=float(np.exp(rng.uniform(np.log(1e4), np.log(1e6)))), poisson=float(rng.uniform(.2, .4)),
                         strain=float(rng.uniform(.01, .1)), area_seed=int(rng.integers(1 << 31)), arrival=arrival))
    return plan


def planned_stream(plan, bases, steps=1):
    """Requests of a ``stream_plan`` from their unit-cube foams ``bases``
    (``bases[k]`` = ``jittered_lattice_foam(plan[k]['m'], seed=plan[k]['foam_seed'])``)."""
    out = []
    for spec, base in zip(plan, bases):
        foam, load = compressed_foam_request(spec['m'], np.random.default_rng(spec['area_seed']), aspect=spec['aspect'],
                                             young=spec['young'], poisson=spec['poisson'], strain=spec['strain'],
                                             base=base)
        out.append(Request(arrival=spec['arrival'], rid=spec['rid'], foam=foam, load=load, steps=steps))
    return out


def large_mix(big=128, small=32, count=64, seed=0, big_steps=10, dt=1e-3):
    """The large served mix: one jittered ``big^3`` foam under gravity with its
    bottom layer fixed (``big_steps`` implicit steps of ``dt``) and ``count``
    requests of ``small^3`` sites with randomized E, nu, box and top load as in
    ``synthetic_stream`` (one step each), all arriving at t = 0."""
    from .foam import gravity_load, jittered_lattice_foam
    rng = np.random.default_rng(seed)
    foam = jittered_lattice_foam(big, seed=seed)
    foam['contacts'] = None
    out = [Request(arrival=0., rid=0, foam=foam, load=gravity_load(foam), dt=dt, steps=big_steps)]
    for rid in range(1, count + 1):
        f, load = compressed_foam_request(small, rng, seed=seed + 1)
        out.append(Request(arrival=0., rid=rid, foam=f, load=load, dt=dt, steps=1))
    return out


def large_mix_requests(big_foam, small_bases, seed=0, big_steps=10, dt=1e-3):
    """The large served mix from prepared foams: ``big_foam`` (a jittered
    lattice foam) under gravity with its bottom layer fixed for ``big_steps``
    implicit steps, and one request per unit-cube foam of ``small_bases``
    (each its own foam; randomized E, nu, box and top load as in
    ``stream_plan``, one step each), all arriving at t = 0."""
    from .foam import gravity_load
    rng = np.random.default_rng(seed)
    big_foam = dict(big_foam, contacts=None)
    out = [Request(arrival=0., rid=0, foam=big_foam, load=gravity_load(big_foam), dt=dt, steps=big_steps)]
    for rid, base in enumerate(small_bases, 1):
        m = round(len(base['points'])**(1/3))
        f, load = compressed_foam_request(m, rng, base=base)
        out.append(Request(arrival=0., rid=rid, foam=f, load=load, dt=dt, steps=1))
    return out


def synthetic_stream(count, seed=0, sites=(1024, 131072), rate=None, buckets=8, steps=1):
    """Mixed-size requests: site counts log-uniform in ``sites`` (rounded to
    ``buckets`` lattice sizes so that bond graphs are generated once per size),
    random box aspect ratios U[0.5, 2], E log-uniform [1e4, 1e6], nu U[0.2, 0.4],
    top strain U[1%, 10%]; Poisson arrivals at ``rate`` per second (None: all
    at t = 0)."""
    rng = np.random.default_rng(seed)
    lo, hi = np.log(sites[0])/3, np.log(sites[1])/3
    sizes = np.unique(np.round(np.exp(np.linspace(lo, hi, buckets))).astype(int))
    arrival = 0.
    out = []
    for rid in range(count):
        target = np.exp(rng.uniform(np.log(sites[0]), np.log(sites[1])))
        m = int(sizes[np.argmin(abs(np.log(sizes**3) - np.log(target)))])
        foam, load = compressed_foam_request(m, rng, seed=seed)
        if rate:
            arrival += float(rng.exponential(1./rate))
        out.append(Request(arrival=arrival, rid=rid, foam=foam, load=load, steps=steps))
    return out
