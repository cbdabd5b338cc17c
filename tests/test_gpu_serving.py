"""Serving form: batched Newton steps over concatenated graphs and the
continuous-batching service.  A request's result must be the same alone and
in the mix: each result (served in a batch, and the same request solved
alone by the mixed-precision solver) is held to the spec bars against a
float64 solve of the same request at relative residual 1e-10 -- displacement
error at most 1e-6 of the float64 displacement -- so the two agree within
2e-6 of the displacement, which is also asserted."""
import pytest

pytestmark = pytest.mark.gpu

torch = pytest.importorskip('torch')


@pytest.fixture(scope='module', autouse=True)
def _cuda():
    if not torch.cuda.is_available():
        pytest.skip('needs a CUDA GPU')


def _solver(req):
    import dpf_gb300
    f = req.foam
    return dpf_gb300.MixedNewtonBonds(f['points'], f['radii'], f['pairs'], f['areas'], f['masses'], f['fixed'],
                                      young=f['young'], shear=f['shear'])


def _alone(req, steps):
    s = _solver(req)
    x0 = s.x.clone()
    for _ in range(steps):
        s.step(req.dt, s.tensor(req.load), tolerance=1e-6)
    return s, x0


def _float64(req, steps):
    """The request solved by the float64 solver at relative residual 1e-10."""
    import dpf_gb300
    f = req.foam
    s = dpf_gb300.NewtonBonds(f['points'], f['radii'], f['pairs'], f['areas'], f['masses'], f['fixed'],
                              young=f['young'], shear=f['shear'])
    x0 = s.x.clone()
    for _ in range(steps):
        s.step(req.dt, s.tensor(req.load), tolerance=1e-10)
    return s.x, x0


def _same_alone_and_in_mix(req, x_mix, steps):
    """Alone and in the mix, each within 1e-6 of the float64 displacement; so
    within 2e-6 of each other."""
    x64, x0 = _float64(req, steps)
    alone, _ = _alone(req, steps)
    disp = float(torch.linalg.vector_norm(x64 - x0))
    mix = float(torch.linalg.vector_norm(x_mix - x64))/disp
    solo = float(torch.linalg.vector_norm(alone.x - x64))/disp
    both = float(torch.linalg.vector_norm(x_mix - alone.x))/disp
    assert mix <= 1e-6 and solo <= 1e-6 and both <= 2e-6, (req.rid, mix, solo, both)
    return alone


def test_batch_matches_alone():
    from dpf_gb300 import serving
    reqs = serving.synthetic_stream(4, seed=3, sites=(800, 9000))
    parts = [_solver(r) for r in reqs]
    batch = serving.Batch(parts)
    ext = torch.cat([p.tensor(r.load) for p, r in zip(parts, reqs)])
    for step in range(2):
        results = batch.step_batch(1e-3, ext, tolerance=1e-6)
        for res in results:
            assert not isinstance(res, Exception), res
            assert res[1]['nonlinear_relative_residual'] < 1e-6
    batch.scatter_state()
    for req, part in zip(reqs, parts):
        alone = _same_alone_and_in_mix(req, part.x, 2)
        ev = float(torch.linalg.vector_norm(part.v - alone.v)/torch.linalg.vector_norm(alone.v))
        assert ev < 1e-4, ev


def test_failed_request_is_isolated():
    """A request whose step trips a guard fails alone; the others commit."""
    from dpf_gb300 import serving
    reqs = serving.synthetic_stream(3, seed=5, sites=(800, 3000))
    reqs[1].load = reqs[1].load*1e7          # rotation/turn guards everywhere
    parts = [_solver(r) for r in reqs]
    before = {k: getattr(parts[1], k).clone() for k in ('x', 'v', 'fn', 'fs')}
    batch = serving.Batch(parts)
    ext = torch.cat([p.tensor(r.load) for p, r in zip(parts, reqs)])
    results = batch.step_batch(1e-3, ext, tolerance=1e-6)
    assert isinstance(results[1], RuntimeError) and 'Subdivide:' in str(results[1])
    assert not isinstance(results[0], Exception) and not isinstance(results[2], Exception)
    batch.scatter_state()
    for k, v in before.items():
        assert torch.equal(getattr(parts[1], k), v), k
    _same_alone_and_in_mix(reqs[0], parts[0].x, 1)


def test_service_stream_with_arrivals():
    from dpf_gb300 import serving
    reqs = serving.synthetic_stream(6, seed=7, sites=(700, 6000), rate=200., steps=2)
    service = serving.Service(hbm_budget=8e9, max_batch_sites=12000)
    finished = service.run(reqs)
    assert len(finished) == 6
    assert all(r.error is None and r.done_steps == 2 for r in finished)
    stats = serving.latency_stats(finished)
    assert stats['p50'] > 0 and stats['p99'] >= stats['p50']
    assert service.batches >= 2
    for req in finished[:3]:
        _same_alone_and_in_mix(req, req.state['x'], 2)


def test_group_state_matches_solver_setup():
    """Device setup of a group of requests equals the float64 host setup of each."""
    from dpf_gb300 import serving
    reqs = serving.synthetic_stream(3, seed=9, sites=(700, 3000))
    group = serving.RequestState.group([r.foam for r in reqs])
    # the concatenated cached graphs give the incidence of the group's own edges
    ptr, inc = serving.device_incidence(group.edges, group.n_sites)
    assert torch.equal(ptr, group._inc_ptr) and torch.equal(inc, group._inc_bond)
    site0 = bond0 = 0
    for r in reqs:
        s = _solver(r)
        for name in ('n', 'ri', 'rj', 'kn', 'ks', 'kb', 'kt', 'offset'):
            got = getattr(group, name)[bond0:bond0 + s.n_bonds]
            assert float(torch.linalg.vector_norm(got - getattr(s, name))) <= 1e-12*max(
                1., float(torch.linalg.vector_norm(getattr(s, name)))), name
        assert torch.allclose(group.mass[site0:site0 + s.n_sites], s.mass, rtol=1e-14, atol=0)
        site0 += s.n_sites
        bond0 += s.n_bonds


def test_large_mix_small_scale():
    """The large served mix at small sizes: a multi-step foam served together
    with single-step requests; each result agrees with its request solved alone."""
    from dpf_gb300 import serving
    reqs = serving.large_mix(big=12, small=6, count=5, seed=2, big_steps=4)
    service = serving.Service(hbm_budget=8e9, max_batch_sites=20000)
    finished = service.run(reqs)
    assert len(finished) == 6 and all(r.error is None for r in finished)
    by_id = {r.rid: r for r in finished}
    assert by_id[0].done_steps == 4 and all(by_id[k].done_steps == 1 for k in range(1, 6))
    # the single-step requests leave after the first batch step; the foam continues alone
    assert service.batch_sizes[0][0] == 6 and service.batch_sizes[-1][0] == 1
    for rid, steps in ((0, 4), (1, 1), (5, 1)):
        req = by_id[rid]
        _same_alone_and_in_mix(req, req.state['x'], steps)


def test_requests_with_other_dt_get_their_own_batch():
    """A batch steps with one dt: a request with another dt waits for its own batch."""
    from dpf_gb300 import serving
    reqs = serving.synthetic_stream(3, seed=13, sites=(600, 2000))
    reqs[1].dt = 2e-3
    service = serving.Service(hbm_budget=8e9, max_batch_sites=20000)
    finished = service.run(reqs)
    assert len(finished) == 3 and all(r.error is None for r in finished)
    assert service.batches >= 2
    for req in finished:
        _same_alone_and_in_mix(req, req.state['x'], 1)


def test_served_stream_of_own_foams_meets_float64_bars():
    """A stream in which every request has its own seeded foam (as the served
    benchmark): every result's float64 force residual and displacement error
    against a float64 solve of the same request are at most 1e-6."""
    from dpf_gb300 import serving
    from dpf_gb300.accuracy import served_accuracy
    from dpf_gb300.foam import jittered_lattice_foam
    plan = serving.stream_plan(12, seed=21, sites=(1000, 12000), rate=500.)
    stream = serving.planned_stream(plan, [jittered_lattice_foam(p['m'], seed=p['foam_seed']) for p in plan])
    assert len({id(r.foam['pairs']) for r in stream}) == len(stream)
    service = serving.Service(hbm_budget=8e9, max_batch_sites=40000)
    finished = service.run(stream)
    assert len(finished) == 12 and all(r.error is None for r in finished)
    report = served_accuracy(finished, 12, 'cuda')
    assert report['requests'] == 12
    assert report['force_residual_rel_max'] <= 1e-6, report
    assert report['displacement_rel_max'] <= 1e-6, report
