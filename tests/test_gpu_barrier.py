"""Bounded device waits: a grid barrier that nobody releases gives up, reports
DPF_ERR_BARRIER_TIMEOUT and returns, and the context stays usable.

The failure is made without any fault: the self-test kernel waits for one
more arrival than its grid has (a flag that nothing sets), under a 5 ms
limit.  The barrier word it leaves behind (a partial arrival count) is then
handed to the cooperative PCG launches, which must reset it before use.
"""
import ctypes
import time

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

torch = pytest.importorskip('torch')


@pytest.fixture(scope='module')
def lib():
    if not torch.cuda.is_available():
        pytest.skip('needs a CUDA GPU')
    from dpf_gb300 import _lib
    return _lib.load()


def _selftest(lib, blocks, missing, timeout_ns=5_000_000):
    barrier = torch.zeros(2, dtype=torch.int32, device='cuda')
    status = torch.zeros(1, dtype=torch.int32, device='cuda')
    passed = torch.zeros(1, dtype=torch.int32, device='cuda')
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    rc = lib.dpf_barrier_selftest(blocks, timeout_ns, missing, barrier.data_ptr(), status.data_ptr(),
                                  passed.data_ptr(), torch.cuda.current_stream().cuda_stream)
    torch.cuda.synchronize()
    return rc, int(status.item()), int(passed.item()), barrier.cpu().tolist(), time.perf_counter() - t0


def test_barrier_passes_with_every_arrival(lib):
    rc, status, passed, _, _ = _selftest(lib, 8, 0)
    assert rc == 0 and status == 0 and passed == 8


def test_barrier_wait_runs_out_and_reports(lib):
    from dpf_gb300 import _lib
    rc, status, passed, barrier, elapsed = _selftest(lib, 8, 1)
    assert rc == 0
    assert status & _lib.DPF_ERR_BARRIER_TIMEOUT
    assert passed == 0
    # the arrivals stay behind in the barrier word: block 0 added 2^31 - 8 (nine
    # parties), the seven others 1 each, so the top bit never flipped
    assert barrier[0] == 0x7FFFFFFF
    assert elapsed < 2.0
    # the context still works
    x = torch.arange(10, dtype=torch.float64, device='cuda')
    assert float((x*x).sum()) == 285.0


def test_pcg_resets_a_barrier_left_by_a_timeout(lib):
    """A barrier word with stale arrivals (as a timed-out wait leaves it) must not
    release the next cooperative PCG early: both the float64 elastic PCG and the
    bond-end PCG zero it on their stream before launching."""
    import dpf_gb300
    foam = dpf_gb300.jittered_lattice_foam(8, seed=4)
    load = dpf_gb300.gravity_load(foam)
    args = (foam['points'], foam['radii'], foam['pairs'], foam['areas'], foam['masses'], foam['fixed'])
    kw = dict(young=foam['young'], shear=foam['shear'])
    for cls in (dpf_gb300.NewtonBonds, dpf_gb300.MixedNewtonBonds):
        clean, dirty = cls(*args, **kw), cls(*args, **kw)
        clean.step(1e-3, clean.tensor(load), tolerance=1e-6)
        dirty._barrier.fill_(3)      # three stale arrivals
        dirty.step(1e-3, dirty.tensor(load), tolerance=1e-6)
        assert int(dirty._status.item()) & 32 == 0
        assert torch.equal(clean.x, dirty.x), cls.__name__
    # and the tiled sweep's PCG, through its own entry point
    s = dpf_gb300.MixedNewtonBonds(*args, **kw)
    s.sweep = 'tiles'
    ref = dpf_gb300.MixedNewtonBonds(*args, **kw)
    ref.sweep = 'tiles'
    ref.step(1e-3, ref.tensor(load), tolerance=1e-6)
    s._barrier.fill_(5)
    s.step(1e-3, s.tensor(load), tolerance=1e-6)
    assert int(s._status.item()) & 32 == 0
    # the autotuner may pick another tile shape per instance: compare displacements
    u, u_ref = s.x.cpu().numpy() - foam['points'], ref.x.cpu().numpy() - foam['points']
    assert np.linalg.norm(u - u_ref) <= 1e-6*np.linalg.norm(u_ref)
