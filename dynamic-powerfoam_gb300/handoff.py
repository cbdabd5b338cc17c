"""Hand-off of simulated body poses to the Power Foam renderer's state
(drop-in for ``state_from_bodies``, ``experiments/bonded_dem_powerfoam.py:123-130``),
on the device that holds the trajectory.

Each body's render frame follows its rotation: frame = frame0 R^T, with the
frame stored as a unit quaternion (w, x, y, z); the texel shading axes are
rotated by R; positions replace the points.  Quaternions are defined up to
sign (q and -q are the same frame).
"""
import torch


def quat_to_matrix(q):
    """Rotation matrices of unit quaternions (w, x, y, z)."""
    w, x, y, z = q.unbind(-1)
    return torch.stack((1 - 2*(y*y + z*z), 2*(x*y - w*z), 2*(x*z + w*y),
                        2*(x*y + w*z), 1 - 2*(x*x + z*z), 2*(y*z - w*x),
                        2*(x*z - w*y), 2*(y*z + w*x), 1 - 2*(x*x + y*y)), -1).reshape(q.shape[:-1] + (3, 3))


def matrix_to_quat(m):
    """Unit quaternions (w, x, y, z) of rotation matrices, with w >= 0.

    Shepperd's method: the largest of the four squared components
    (1 + tr, 1 + 2 m00 - tr, ...) is recovered first and the others from
    off-diagonal sums and differences, so no branch divides by a small number.
    """
    m00, m11, m22 = m[..., 0, 0], m[..., 1, 1], m[..., 2, 2]
    tr = m00 + m11 + m22
    cand = torch.stack((1 + tr, 1 + 2*m00 - tr, 1 + 2*m11 - tr, 1 + 2*m22 - tr), -1)
    k = cand.argmax(-1)
    s = torch.sqrt(cand.gather(-1, k[..., None]).clamp_min(0))[..., 0]      # 2 |q_k|
    a21, a12, a02, a20, a10, a01 = (m[..., 2, 1], m[..., 1, 2], m[..., 0, 2], m[..., 2, 0], m[..., 1, 0],
                                    m[..., 0, 1])
    qs = [torch.stack((s/2, (a21 - a12)/(2*s), (a02 - a20)/(2*s), (a10 - a01)/(2*s)), -1),
          torch.stack(((a21 - a12)/(2*s), s/2, (a01 + a10)/(2*s), (a02 + a20)/(2*s)), -1),
          torch.stack(((a02 - a20)/(2*s), (a01 + a10)/(2*s), s/2, (a12 + a21)/(2*s)), -1),
          torch.stack(((a10 - a01)/(2*s), (a02 + a20)/(2*s), (a12 + a21)/(2*s), s/2), -1)]
    q = torch.stack(qs, 0).gather(0, k[None, ..., None].expand((1,) + k.shape + (4,)))[0]
    q = torch.where(q[..., :1] < 0, -q, q)
    return q/torch.linalg.vector_norm(q, dim=-1, keepdim=True)


def state_from_bodies(base, positions, rotations):
    """Renderer state of bodies at ``positions`` (N, 3) with rotations (N, 3, 3).

    ``base`` is the renderer state at the reference configuration (``points``,
    ``quaternions`` (N, 4) w-first, ``texel_sv_axis`` (N, 8, 24), ...); the
    other entries are passed through.  Tensors stay on their device.
    """
    dev = rotations.device if torch.is_tensor(rotations) else None
    t = lambda a: torch.as_tensor(a, dtype=torch.float64, device=dev)
    rotations, positions = t(rotations), t(positions)
    frame0 = quat_to_matrix(t(base['quaternions']))
    frame = frame0@rotations.transpose(1, 2)
    axes = t(base['texel_sv_axis']).reshape(-1, 8, 8, 3)
    rotated = torch.einsum('nab,nsdb->nsda', rotations, axes)
    return dict(base, points=positions, quaternions=matrix_to_quat(frame),
                texel_sv_axis=rotated.reshape(-1, 8, 24))
