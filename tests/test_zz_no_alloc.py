"""The allocation-free K q entry point, checked against the allocating one (GPU).

Some callers cannot call cudaMalloc: a host application that passes this
library only its inputs and outputs, taken from a device-memory pool it
manages itself under a fixed budget, cannot let a plug-in allocate scratch (an
extra allocation could fail, a cudaFree could stall the whole device in the
middle of the host's work).  For them ``dpf_stiffness_apply_static`` keeps its
bond-wrench scratch in a file-scope device array of fixed capacity
(``DPF_STATIC_MAX_BONDS`` bonds).  This file is collected last so that a run
stopping at the first failure has already run every other test; it passes
alone in a fresh process as well as after the others.
"""
import ctypes

import numpy as np
import pytest

from tests.conftest import golden

pytestmark = pytest.mark.gpu

torch = pytest.importorskip('torch')


@pytest.fixture(scope='module')
def lib():
    if not torch.cuda.is_available():
        pytest.skip('needs a CUDA GPU')
    from dpf_gb300 import _lib
    return _lib.load()


def _both(lib, s, q):
    """K q through the allocating entry point and through the static-scratch one."""
    stream = torch.cuda.current_stream().cuda_stream
    ref, out = torch.empty_like(q), torch.empty_like(q)
    graph, stiffness, tangent = s._graph, s._stiffness_struct(), s._tangent_struct()
    rc = lib.dpf_stiffness_apply(ctypes.byref(graph), ctypes.byref(stiffness), ctypes.byref(tangent),
                                 q.data_ptr(), ref.data_ptr(), s._wrench.data_ptr(), stream)
    assert rc == 0
    rc = lib.dpf_stiffness_apply_static(ctypes.byref(graph), ctypes.byref(stiffness), ctypes.byref(tangent),
                                        q.data_ptr(), out.data_ptr(), stream)
    assert rc == 0
    torch.cuda.synchronize()
    return ref, out


def _rel(a, b):
    return float(torch.linalg.vector_norm(a - b)/torch.linalg.vector_norm(b))


def test_static_scratch_matches_allocating_entry_point(lib):
    import dpf_gb300
    g = golden('tangent_81')
    s = dpf_gb300.LinearBonds(g['points'], np.ones(50), g['pairs'], np.ones(len(g['pairs'])), g['contacts'],
                              np.ones(50), np.zeros(50, bool))
    foam = dpf_gb300.jittered_lattice_foam(16, seed=1)
    big = dpf_gb300.FiniteBonds(foam['points'], foam['radii'], foam['pairs'], foam['areas'], foam['masses'],
                                foam['fixed'], young=foam['young'], shear=foam['shear'])
    assert big.n_bonds <= lib.dpf_static_max_bonds()
    generator = torch.Generator(device='cuda').manual_seed(11)
    for solver in (s, big, s, big):          # calls in a row share (and reuse) the static array
        for _ in range(2):
            q = torch.randn((solver.n_sites, 6), dtype=torch.float64, device='cuda', generator=generator)
            ref, out = _both(lib, solver, q)
            assert _rel(out, ref) < 1e-12     # the K q tolerance of the parity tests
    ref, out = _both(lib, s, s.tensor(g['q']))
    assert _rel(out, s.tensor(g['stiffness_q'])) < 1e-12


def test_static_scratch_rejects_graphs_above_capacity(lib):
    import dpf_gb300
    from dpf_gb300 import _lib
    g = golden('tangent_81')
    s = dpf_gb300.LinearBonds(g['points'], np.ones(50), g['pairs'], np.ones(len(g['pairs'])), g['contacts'],
                              np.ones(50), np.zeros(50, bool))
    graph = _lib.Graph(s._graph.n_sites, lib.dpf_static_max_bonds() + 1, s._graph.edges, s._graph.inc_ptr,
                       s._graph.inc_bond)
    q = torch.zeros((s.n_sites, 6), dtype=torch.float64, device='cuda')
    out = torch.empty_like(q)
    # rejected on the host before any launch
    rc = lib.dpf_stiffness_apply_static(ctypes.byref(graph), ctypes.byref(s._stiffness_struct()),
                                        ctypes.byref(s._tangent_struct()), q.data_ptr(), out.data_ptr(),
                                        torch.cuda.current_stream().cuda_stream)
    assert rc == _lib.DPF_ERR_TOO_LARGE
