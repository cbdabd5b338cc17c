"""Shared helpers for the GPU parity tests (build the solver from golden inputs)."""
import numpy as np

from tests.conftest import golden, newton_inputs, STATE


def gpu_newton(g, prefix='state_', device='cuda'):
    import torch
    import dpf_gb300
    s = dpf_gb300.NewtonBonds(**newton_inputs(g), device=device)
    for k in STATE:
        setattr(s, k, torch.as_tensor(np.array(g[prefix + k]), dtype=torch.float64, device=s.device).contiguous())
    return s


def oracle_newton(g, prefix='state_'):
    from oracle import dem
    s = dem.NewtonBonds(**newton_inputs(g))
    for k in STATE:
        setattr(s, k, np.array(g[prefix + k]))
    return s


def rel(a, b):
    a = a.detach().cpu().numpy() if hasattr(a, 'detach') else np.asarray(a)
    b = b.detach().cpu().numpy() if hasattr(b, 'detach') else np.asarray(b)
    return float(np.linalg.norm(a - b)/max(np.linalg.norm(b), 1e-300))


def host(t):
    return t.detach().cpu().numpy() if hasattr(t, 'detach') else np.asarray(t)
