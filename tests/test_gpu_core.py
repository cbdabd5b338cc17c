"""Parallel-bond component with brittle failure on the GPU against the
reference's ParallelBonds history (golden) and its guard semantics."""
import numpy as np
import pytest

from tests.conftest import golden
from tests.helpers import host

pytestmark = pytest.mark.gpu


def _bonds(g):
    import dpf_gb300
    return dpf_gb300.ParallelBonds(g['points'], g['pairs'], g['radii'], float(g['bond_radius']), g['kbar_n'],
                                   g['kbar_s'], g['tensile'], g['cohesion'], float(g['friction_angle']),
                                   float(g['moment_factor']), device='cuda')


def test_history_with_failure_matches_reference():
    g = golden('parallel_512')
    b = _bonds(g)
    for k, (end, v, w) in enumerate(zip(g['ends'], g['vs'], g['ws'])):
        info = b.advance(end, v, w, float(g['dt']))
        nb, e, removed = g['steps'][k]
        assert info['newly_broken'] == int(nb), k
        assert abs(info['energy'] - e) <= 1e-10*max(abs(e), 1e-30)
        assert abs(info['removed_bond_energy'] - removed) <= 1e-10*max(abs(removed), 1e-30)
    assert np.array_equal(host(b.failure), g['failure'])
    for k in ('fn', 'fs', 'mt', 'mb', 'break_energy', 'normal', 'x'):
        assert np.abs(host(getattr(b, k)) - g[k]).max() <= 1e-10*max(np.abs(g[k]).max(), 1e-30), k
    assert abs(b.work - float(g['work'])) <= 1e-10*abs(float(g['work']))
    f, t = b.loads()
    assert np.abs(host(f) - g['force']).max() <= 1e-10*np.abs(g['force']).max()
    assert np.abs(host(t) - g['torque']).max() <= 1e-10*np.abs(g['torque']).max()
    assert np.abs(host(b.elastic_energy_per_bond()).sum() - g['steps'][-1][1]) <= 1e-10*abs(g['steps'][-1][1])


def test_rejected_step_leaves_state_unchanged():
    g = golden('parallel_512')
    b = _bonds(g)
    end, v, w = g['ends'][0], g['vs'][0], g['ws'][0]
    b.advance(end, v, w, float(g['dt']))
    before = {k: host(getattr(b, k)).copy() for k in ('fn', 'fs', 'mt', 'mb', 'failure', 'normal', 'x')}
    work = b.work
    with pytest.raises(ValueError, match='rotation'):
        b.advance(g['ends'][1], g['vs'][1], np.full_like(w, 10.), float(g['dt']))
    for k, val in before.items():
        assert np.array_equal(host(getattr(b, k)), val), k
    assert b.work == work
    b.advance(g['ends'][1], g['vs'][1], g['ws'][1], float(g['dt']))
