"""The float32 operator sweeps (site tiles, bond ends) and their elastic
PCGs against float64 products and the bond-pass float32 PCG on the same
tangent."""
import ctypes

import pytest

pytestmark = pytest.mark.gpu


def _solver(m=8, seed=1, dt=1e-3):
    import torch
    import dpf_gb300
    foam = dpf_gb300.jittered_lattice_foam(m, seed=seed)
    s = dpf_gb300.MixedNewtonBonds(foam['points'], foam['radii'], foam['pairs'], foam['areas'], foam['masses'],
                                   foam['fixed'], young=foam['young'], shear=foam['shear'], device='cuda')
    load = s.tensor(dpf_gb300.gravity_load(foam))
    s.step(dt, load)
    # a fresh scaling (tangent, blocks, P, units) at a nonzero iterate
    y = torch.randn((s.n_sites, 6), dtype=torch.float64, device='cuda')*1e-5
    y[s.fixed] = 0
    s._step_begin(dt, load)
    s._iteration_residual(y, dt, load)
    return s, dt


def _direct_operator(s, alpha, q):
    """(diag M + alpha K) q in float64 from the float32 tangent in the bond data."""
    import torch
    m = s.n_bonds
    planes = s._bond_data[:44*m].view(11*m, 4).double()
    t0, t1, t2, t3 = planes[7*m:8*m], planes[8*m:9*m], planes[9*m:10*m], planes[10*m:11*m]
    n, ri, rj = t0[:, :3], t1[:, :3], t2[:, :3]
    kn, ks, kb, kt = t0[:, 3], t1[:, 3], t2[:, 3], t3[:, 0]
    i, j = s.i, s.j
    du = q[j, :3] - q[i, :3] + torch.linalg.cross(q[j, 3:], rj) - torch.linalg.cross(q[i, 3:], ri)
    dw = q[j, 3:] - q[i, 3:]
    f = ks[:, None]*du + ((kn - ks)*(du*n).sum(1))[:, None]*n
    mm = kb[:, None]*dw + ((kt - kb)*(dw*n).sum(1))[:, None]*n
    out = torch.zeros_like(q)
    out.index_add_(0, i, torch.cat([-f, -torch.linalg.cross(ri, f) - mm], 1))
    out.index_add_(0, j, torch.cat([f, torch.linalg.cross(rj, f) + mm], 1))
    y = s._mass32.double()*q + alpha*out
    y[s.fixed] = q[s.fixed]
    return y


@pytest.mark.parametrize('max_entries,threads,stages', [(256, 128, 3), (320, 160, 4), (384, 192, 3)])
def test_tiled_hvp_matches_float64_product(max_entries, threads, stages):
    import torch
    from dpf_gb300 import _lib
    from dpf_gb300.tiles import Tiles
    s, dt = _solver()
    edges, ptr, inc = s.edges.cpu().numpy(), s._inc_ptr.cpu().numpy(), s._inc_bond.cpu().numpy()
    tiles = Tiles.build(edges, ptr, inc, s.n_sites, s.device, max_entries, threads, stages)
    s._pack_tiles(tiles, dt)
    q = torch.randn((s.n_sites, 6), dtype=torch.float64, device='cuda')
    q32 = q.float().contiguous()
    y = torch.empty_like(q32)
    _lib.call('dpf_tiled_hvp', ctypes.byref(s._graph), ctypes.byref(tiles.struct), tiles.entries.data_ptr(),
              s._site4.data_ptr(), q32.data_ptr(), y.data_ptr(), tiles.status.data_ptr(), threads,
              stages, s._stream())
    assert int(tiles.status.item()) == 0
    ref = _direct_operator(s, .25*dt*dt, q32.double())
    err = (y.double() - ref).norm()/ref.norm()
    assert float(err) < 2e-6


def test_end_hvp_matches_float64_product():
    import torch
    from dpf_gb300 import _lib
    s, dt = _solver(m=9, seed=4)
    s._pack_ends(dt)
    q = torch.randn((s.n_sites, 6), dtype=torch.float64, device='cuda')
    q32 = q.float().contiguous()
    y = torch.empty_like(q32)
    _lib.call('dpf_end_hvp', ctypes.byref(s._graph), s._ends.data_ptr(), s._site4.data_ptr(), q32.data_ptr(),
              y.data_ptr(), 0, s._stream())
    ref = _direct_operator(s, .25*dt*dt, q32.double())
    err = (y.double() - ref).norm()/ref.norm()
    assert float(err) < 2e-6
    # bitwise reproducible: fixed lane split and shuffle tree, no atomics
    y2 = torch.empty_like(q32)
    _lib.call('dpf_end_hvp', ctypes.byref(s._graph), s._ends.data_ptr(), s._site4.data_ptr(), q32.data_ptr(),
              y2.data_ptr(), 0, s._stream())
    assert torch.equal(y, y2)
    # every launch shape gives the same operator
    lib = _lib.load()
    for variant in range(1, lib.dpf_end_variant_count()):
        lanes, blocks = ctypes.c_int(), ctypes.c_int()
        assert lib.dpf_end_variant_shape(variant, ctypes.byref(lanes), ctypes.byref(blocks)) == 0
        y3 = torch.empty_like(q32)
        _lib.call('dpf_end_hvp', ctypes.byref(s._graph), s._ends.data_ptr(), s._site4.data_ptr(), q32.data_ptr(),
                  y3.data_ptr(), variant, s._stream())
        err = (y3.double() - ref).norm()/ref.norm()
        assert float(err) < 2e-6, (variant, lanes.value, blocks.value)


@pytest.mark.parametrize('sweep', ['ends', 'tiles'])
def test_swept_pcg_matches_bond_pass_pcg(sweep):
    import torch
    s, dt = _solver()
    v = torch.randn((s.n_sites, 6), dtype=torch.float64, device='cuda')
    pre = s._newton_preconditioner(dt)
    s.sweep = sweep
    a = pre(v, tolerance=1e-7, max_iterations=2000)
    if sweep == 'tiles':
        from dpf_gb300.tiles import _TUNED
        assert s._tiles is not None and (s.n_sites, s.n_bonds) in _TUNED, 'autotuner did not run'
    s.sweep = 'bonds'
    b = pre(v, tolerance=1e-7, max_iterations=2000)
    rel = float((a - b).norm()/b.norm())
    assert rel < 1e-4, rel
    # the reference tolerance: comparable iteration counts
    s.sweep = sweep
    s.inner_iterations = 0
    pre(v)
    swept_its = s.inner_iterations
    s.sweep = 'bonds'
    s.inner_iterations = 0
    pre(v)
    assert abs(swept_its - s.inner_iterations) <= max(2, .2*s.inner_iterations)


@pytest.mark.parametrize('sweep', ['ends', 'tiles'])
def test_swept_pcg_is_deterministic(sweep):
    import torch
    s, dt = _solver(m=10, seed=3)
    s.sweep = sweep
    v = torch.randn((s.n_sites, 6), dtype=torch.float64, device='cuda')
    pre = s._newton_preconditioner(dt)
    a = pre(v).clone()
    b = pre(v).clone()
    assert torch.equal(a, b)
