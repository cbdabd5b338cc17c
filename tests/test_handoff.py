"""Render hand-off (state_from_bodies) against the reference's outputs; the
quaternion conversion against matrices (q and -q are the same frame)."""
import numpy as np
import pytest

from tests.conftest import golden


def _run(device):
    import torch
    from dpf_gb300.handoff import quat_to_matrix, state_from_bodies
    g = golden('handoff_30')
    base = {k[5:]: g[k] for k in g if k.startswith('base_')}
    rot = torch.as_tensor(g['rotations'], device=device)
    out = state_from_bodies(base, torch.as_tensor(g['positions'], device=device), rot)
    want = {k[6:]: g[k] for k in g if k.startswith('state_')}
    assert np.allclose(out['points'].cpu().numpy(), want['points'], atol=0, rtol=0)
    assert np.abs(out['texel_sv_axis'].cpu().numpy() - want['texel_sv_axis']).max() < 1e-14
    # reference quaternions are (w, x, y, z) up to sign: compare the frames
    ours = quat_to_matrix(out['quaternions']).cpu().numpy()
    theirs = quat_to_matrix(torch.as_tensor(want['quaternions'])).numpy()
    assert np.abs(ours - theirs).max() < 1e-14
    for k in ('radii', 'density', 'texel_sites', 'texel_height', 'texel_sv_rgb'):
        assert np.array_equal(np.asarray(out[k]), want[k])


def test_handoff_matches_reference_cpu_tensors():
    _run('cpu')


@pytest.mark.gpu
def test_handoff_matches_reference_on_gpu():
    _run('cuda')


def test_matrix_to_quat_round_trip():
    import torch
    from dpf_gb300.handoff import matrix_to_quat, quat_to_matrix
    rng = np.random.default_rng(1)
    q = torch.as_tensor(rng.normal(size=(200, 4)))
    q = q/torch.linalg.vector_norm(q, dim=1, keepdim=True)
    q[:5, 0] = 0   # 180-degree rotations
    q[:5] = q[:5]/torch.linalg.vector_norm(q[:5], dim=1, keepdim=True)
    m = quat_to_matrix(q)
    assert float((quat_to_matrix(matrix_to_quat(m)) - m).abs().max()) < 1e-14
