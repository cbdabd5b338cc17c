"""Static linear equilibrium on the GPU against the reference's
reference_stiffness / solve_prescribed (golden) and matrix-free vs matrix."""
import numpy as np
import pytest

from tests.conftest import golden
from tests.helpers import host

pytestmark = pytest.mark.gpu


def _specimen_bonds(g):
    import dpf_gb300
    return dpf_gb300.ParallelBonds(g['points'], g['pairs'], g['radii'], g['bond_radius'], g['kbar_n'], g['kbar_s'],
                                   device='cuda')


def test_reference_stiffness_matches_reference():
    import dpf_gb300
    g = golden('static_specimen')
    k = dpf_gb300.reference_stiffness(_specimen_bonds(g)).to_dense()
    assert np.abs(host(k) - g['dense_k']).max() <= 1e-12*np.abs(g['dense_k']).max()


@pytest.mark.parametrize('matrix', [False, True])
def test_solve_prescribed_matches_reference(matrix):
    import dpf_gb300
    g = golden('static_specimen')
    bonds = _specimen_bonds(g)
    k = dpf_gb300.reference_stiffness(bonds) if matrix else bonds
    q, residual = dpf_gb300.solve_prescribed(k, g['prescribed'], g['values'], g['load'])
    assert residual < 1e-8
    assert np.abs(host(q).reshape(-1, 6) - g['q']).max() <= 1e-8*np.abs(g['q']).max()


def test_matrix_free_solve_on_a_foam():
    """A 10^3 foam clamped at the bottom with its top pushed down: the
    matrix-free solve equals the sparse-matrix solve and satisfies the
    reference's residual test."""
    import torch
    import dpf_gb300
    foam = dpf_gb300.jittered_lattice_foam(10, seed=2)
    s = dpf_gb300.LinearBonds(foam['points'], foam['radii'], foam['pairs'], foam['areas'],
                              dpf_gb300.newton.classical_contacts(foam['points'], foam['radii'], foam['pairs']),
                              foam['masses'], foam['fixed'], young=foam['young'], shear=foam['shear'], device='cuda')
    unit = foam['unit']
    prescribed = np.zeros((s.n_sites, 6), bool)
    values = np.zeros((s.n_sites, 6))
    prescribed[unit[:, 2] < .1] = True
    top = unit[:, 2] > .9
    prescribed[top, 2] = True
    values[top, 2] = -.01
    q1, r1 = dpf_gb300.solve_prescribed(s, prescribed, values)
    q2, r2 = dpf_gb300.solve_prescribed(dpf_gb300.reference_stiffness(s), prescribed, values)
    assert r1 < 1e-8 and r2 < 1e-8
    assert float(torch.linalg.vector_norm(q1 - q2)/torch.linalg.vector_norm(q2)) < 1e-8


def test_static_16cube_matches_direct_solve():
    """The small static configuration: a 16^3 foam (4,096 sites), bottom layer
    (z < 0.05) clamped, top layer (z > 0.95) displaced by -5% of its height in z;
    the matrix-free CUDA solve against a direct sparse solve (SciPy) of the same
    stiffness on the host."""
    import time
    import torch
    import scipy.sparse as sp
    import scipy.sparse.linalg as spla
    import dpf_gb300
    foam = dpf_gb300.jittered_lattice_foam(16, seed=0)
    s = dpf_gb300.LinearBonds(foam['points'], foam['radii'], foam['pairs'], foam['areas'],
                              dpf_gb300.newton.classical_contacts(foam['points'], foam['radii'], foam['pairs']),
                              foam['masses'], foam['fixed'], young=foam['young'], shear=foam['shear'], device='cuda')
    z = foam['points'][:, 2]
    prescribed = np.zeros((s.n_sites, 6), bool)
    values = np.zeros((s.n_sites, 6))
    prescribed[z < .05] = True
    top = z > .95
    prescribed[top, 2] = True
    values[top, 2] = -.05*z[top]
    q, residual = dpf_gb300.solve_prescribed(s, prescribed, values)
    assert residual < 1e-8
    k = dpf_gb300.reference_stiffness(s).to('cpu')
    K = sp.csr_matrix((k.values().numpy(), k.col_indices().numpy(), k.crow_indices().numpy()), shape=k.shape)
    mask = prescribed.ravel()
    free, fixed = np.flatnonzero(~mask), np.flatnonzero(mask)
    t = time.time()
    ref = values.ravel().copy()
    ref[free] = spla.spsolve(K[free][:, free].tocsc(), -K[free][:, fixed]@ref[fixed])
    assert time.time() - t < 120
    q = host(q)
    assert np.abs(q - ref).max() <= 1e-7*np.abs(ref).max()
