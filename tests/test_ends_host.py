"""The bond-end form of the frozen-tangent operator, emulated on the host (no GPU):
every incidence's share F_s = -f, T_s = -(r_s x f) - m with n' pointing from the
site to the other end and r_o = r_s - L n' adds up, over the incidence CSR, to the
bond-wise K q of the reference (experiments/bonded_dem_linear_gpu.py:42-52)."""
import numpy as np


def _graph(rng, n=40, m=150):
    pairs = set()
    while len(pairs) < m:
        i, j = sorted(rng.choice(n, 2, replace=False))
        pairs.add((int(i), int(j)))
    edges = np.array(sorted(pairs))
    nrm = rng.normal(size=(m, 3))
    nrm /= np.linalg.norm(nrm, axis=1)[:, None]
    ri = rng.normal(size=(m, 3))
    L = rng.uniform(.5, 1.5, m)
    rj = ri - L[:, None]*nrm
    k = rng.uniform(.5, 2., (m, 4))
    return edges, nrm, ri, rj, L, k


def _bondwise(n, edges, nrm, ri, rj, k, q):
    """K q as the reference: per bond du, dw, f, m scattered to both ends."""
    i, j = edges.T
    kn, ks, kb, kt = k.T
    du = q[j, :3] - q[i, :3] + np.cross(q[j, 3:], rj) - np.cross(q[i, 3:], ri)
    dw = q[j, 3:] - q[i, 3:]
    f = ks[:, None]*du + ((kn - ks)*(du*nrm).sum(1))[:, None]*nrm
    mm = kb[:, None]*dw + ((kt - kb)*(dw*nrm).sum(1))[:, None]*nrm
    out = np.zeros((n, 6))
    np.add.at(out, i, np.hstack([-f, -np.cross(ri, f) - mm]))
    np.add.at(out, j, np.hstack([f, np.cross(rj, f) + mm]))
    return out


def _endwise(n, edges, nrm, ri, rj, L, k, q):
    """K q from one end record per incidence, summed per site in CSR order."""
    m = len(edges)
    site = np.concatenate([edges[:, 0], edges[:, 1]])
    code = np.concatenate([np.arange(m), ~np.arange(m)])
    order = np.argsort(site, kind='stable')
    out = np.zeros((n, 6))
    for s, v in zip(site[order], code[order]):
        b = v if v >= 0 else ~v
        at_i = v >= 0
        nn = nrm[b] if at_i else -nrm[b]           # n' from s towards the other end
        rs = ri[b] if at_i else rj[b]
        o = edges[b, 1] if at_i else edges[b, 0]
        ro = rs - L[b]*nn                          # the other end's lever
        kn, ks, kb, kt = k[b]
        du = q[o, :3] - q[s, :3] + np.cross(q[o, 3:], ro) - np.cross(q[s, 3:], rs)
        dw = q[o, 3:] - q[s, 3:]
        f = ks*du + (kn - ks)*du.dot(nn)*nn
        mm = kb*dw + (kt - kb)*dw.dot(nn)*nn
        out[s, :3] -= f
        out[s, 3:] -= np.cross(rs, f) + mm
    return out


def test_end_shares_sum_to_the_bondwise_product():
    rng = np.random.default_rng(5)
    n = 40
    edges, nrm, ri, rj, L, k = _graph(rng, n)
    q = rng.normal(size=(n, 6))
    ref = _bondwise(n, edges, nrm, ri, rj, k, q)
    got = _endwise(n, edges, nrm, ri, rj, L, k, q)
    assert np.abs(got - ref).max() <= 1e-12*np.abs(ref).max()


def test_end_levers_recover_the_other_lever():
    """The pack derives r_o from r_s, L and n' (L = (r_i - r_j).n): exact for the
    tangent's levers, whose difference is the bond vector."""
    rng = np.random.default_rng(6)
    edges, nrm, ri, rj, L, k = _graph(rng)
    L_packed = ((ri - rj)*nrm).sum(1)
    assert np.allclose(L_packed, L, rtol=1e-14, atol=0)
    assert np.allclose(rj + L_packed[:, None]*nrm, ri, rtol=0, atol=1e-14)   # from the j end: n' = -n
