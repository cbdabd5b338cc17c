"""CPU tests: the C-ABI library loads and exports every declared symbol, and
the host-side logic (incidence order, status mapping, foam generator) is right.
No kernel is launched here."""
import ctypes
import re
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parent.parent


def declared_functions():
    text = (ROOT/'include'/'dpf_gb300.h').read_text()
    text = re.sub(r'/\*.*?\*/', '', text, flags=re.S)
    return sorted(set(re.findall(r'\b(dpf_[a-z0-9_]+)\s*\(', text)))


@pytest.fixture(scope='module')
def library():
    import __graft_entry__
    lib_path = ROOT/'dynamic-powerfoam_gb300'/'libdpf_gb300.so'
    if not lib_path.exists():
        __graft_entry__.build()
    return ctypes.CDLL(str(lib_path))


def test_library_exports_every_declared_symbol(library):
    names = declared_functions()
    assert len(names) >= 20
    missing = [n for n in names if not hasattr(library, n)]
    assert not missing, missing


def test_binding_covers_header():
    from dpf_gb300 import _lib
    assert set(declared_functions()) == set(_lib.SIGNATURES)
    assert set(_lib.KERNELS) <= set(_lib.SIGNATURES)


def test_step_driver_struct_layouts_match_the_binding(library):
    from dpf_gb300 import _lib
    out = (ctypes.c_int64*3)()
    library.dpf_newton_struct_sizes.argtypes = [ctypes.POINTER(ctypes.c_int64)]
    assert library.dpf_newton_struct_sizes(out) == 0
    assert list(out) == [ctypes.sizeof(_lib.MixedNewton), ctypes.sizeof(_lib.NewtonStep),
                         ctypes.sizeof(_lib.NewtonInfo)]


def test_size_queries(library):
    library.dpf_wrench_scratch_doubles.restype = ctypes.c_int64
    library.dpf_wrench_scratch_doubles.argtypes = [ctypes.c_int64]
    assert library.dpf_wrench_scratch_doubles(1000) == 9000
    library.dpf_elastic_workspace_doubles.restype = ctypes.c_int64
    library.dpf_elastic_workspace_doubles.argtypes = [ctypes.c_int64]
    assert library.dpf_elastic_workspace_doubles(10) >= 300


def test_incidence_order_matches_index_add():
    """Per site: bonds as endpoint i in increasing b, then as endpoint j (~b)."""
    from dpf_gb300 import incidence
    rng = np.random.default_rng(5)
    edges = rng.integers(0, 40, size=(300, 2))
    edges = edges[edges[:, 0] != edges[:, 1]]
    ptr, inc = incidence(edges, 40)
    assert ptr[0] == 0 and ptr[-1] == 2*len(edges)
    for s in range(40):
        got = list(inc[ptr[s]:ptr[s+1]])
        want = [b for b in range(len(edges)) if edges[b, 0] == s] + [~b for b in range(len(edges)) if edges[b, 1] == s]
        assert got == want


def test_guard_error_order_and_messages():
    from dpf_gb300 import guard_error, SubdivideError
    from dpf_gb300 import _lib
    e = guard_error(_lib.DPF_ERR_NORMAL_TURN | _lib.DPF_ERR_ROTATION)
    assert isinstance(e, SubdivideError) and isinstance(e, RuntimeError)
    assert str(e).startswith('Subdivide: body rotation')
    assert 'coincident' in str(guard_error(_lib.DPF_ERR_COINCIDENT | _lib.DPF_ERR_NORMAL_TURN))
    assert str(guard_error(_lib.DPF_ERR_NORMAL_TURN)).startswith('Subdivide: normal turns')


def test_foam_generator():
    import dpf_gb300
    foam = dpf_gb300.jittered_lattice_foam(8, seed=0)
    n, m = len(foam['points']), len(foam['pairs'])
    assert n == 512 and 6.5 < m/n < 7.7
    used = np.unique(foam['pairs'])
    assert len(used) == n                     # no hidden sites
    assert np.all(foam['pairs'][:, 0] < foam['pairs'][:, 1])
    assert foam['fixed'].sum() > 0 and not foam['fixed'].all()
    a = dpf_gb300.jittered_lattice_foam(8, seed=0)
    assert np.array_equal(a['pairs'], foam['pairs']) and np.array_equal(a['points'], foam['points'])
    g = dpf_gb300.morton_order(4)
    assert len(np.unique(g, axis=0)) == 64 and tuple(g[0]) == (0, 0, 0) and tuple(g[1]) == (1, 0, 0)


def test_equal_weights_give_delaunay_edges():
    """Regular triangulation with equal weights is the Delaunay triangulation
    (the reference's own graph audit, powersim_bread_demo.py:139-153)."""
    from scipy.spatial import Delaunay
    import dpf_gb300
    rng = np.random.default_rng(928)
    x = rng.normal(size=(30, 3))
    pairs = dpf_gb300.regular_edges(x, np.ones(30))
    tetra = Delaunay(x).simplices
    expected = np.concatenate([tetra[:, [i, j]] for i in range(4) for j in range(i+1, 4)])
    expected = np.unique(np.sort(expected, axis=1), axis=0)
    assert np.array_equal(pairs, expected)


def test_solver_refuses_cpu_device():
    import dpf_gb300
    with pytest.raises(ValueError):
        dpf_gb300.NewtonBonds(np.eye(3), 1., [[0, 1]], 1., 1., [False]*3, device='cpu')


def test_mechanics_sources_cover_every_cuda_source():
    from dpf_gb300.checkpoint import mechanics_sources
    from pathlib import Path
    hashes = mechanics_sources()
    csrc = Path(__file__).resolve().parent.parent/'dynamic-powerfoam_gb300'/'csrc'
    for f in list(csrc.glob('*.cu')) + list(csrc.glob('*.cuh')):
        assert f.name in hashes and len(hashes[f.name]) == 64
    assert 'dpf_gb300.h' in hashes and 'newton.py' in hashes
