"""Trajectory checkpoints and verified resume: a run interrupted and resumed
reproduces the uninterrupted run bit for bit."""
import json

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _solver():
    import dpf_gb300
    foam = dpf_gb300.jittered_lattice_foam(6, seed=4, fixed_below=1/6)
    s = dpf_gb300.NewtonBonds(foam['points'], foam['radii'], foam['pairs'], foam['areas'], foam['masses'],
                              foam['fixed'], young=foam['young'], shear=foam['shear'], device='cuda')
    base = s.tensor(dpf_gb300.gravity_load(foam))
    return s, (lambda t: base*(1 + 20*np.sin(40*t)**2))


def test_resume_reproduces_uninterrupted_run(tmp_path):
    from dpf_gb300.checkpoint import TrajectoryRun
    s, load = _solver()
    full = TrajectoryRun(s, load, 2e-3, 6, tmp_path/'full', checkpoint_every=2).run()
    assert full['complete'] and full['checks_pass']
    s, load = _solver()
    part = TrajectoryRun(s, load, 2e-3, 4, tmp_path/'part', checkpoint_every=2).run()
    assert part['completed_intervals'] == 4
    s, load = _solver()
    resumed = TrajectoryRun(s, load, 2e-3, 6, tmp_path/'resumed', checkpoint_every=2,
                            resume=tmp_path/'part').run()
    assert resumed['complete'] and resumed['resumed_from'] == str(tmp_path/'part')
    with np.load(tmp_path/'full'/'final_state.npz') as a, np.load(tmp_path/'resumed'/'final_state.npz') as b:
        for k in a.files:
            assert np.array_equal(a[k], b[k]), k
    rows = lambda d: [json.loads(line) for line in (d/'progress.jsonl').read_text().splitlines()]
    strip = lambda r: {k: v for k, v in r.items() if k != 'elapsed_seconds'}
    assert [strip(r) for r in rows(tmp_path/'full')] == [strip(r) for r in rows(tmp_path/'resumed')]


def test_resume_refuses_changed_mechanics(tmp_path):
    from dpf_gb300.checkpoint import TrajectoryRun
    s, load = _solver()
    TrajectoryRun(s, load, 2e-3, 2, tmp_path/'part', checkpoint_every=2).run()
    report = json.loads((tmp_path/'part'/'mechanics.json').read_text())
    name = sorted(report['source_sha256'])[0]
    report['source_sha256'][name] = '0'*64
    (tmp_path/'part'/'mechanics.json').write_text(json.dumps(report))
    s, load = _solver()
    with pytest.raises(ValueError, match='unchanged mechanics'):
        TrajectoryRun(s, load, 2e-3, 4, tmp_path/'again', resume=tmp_path/'part')
