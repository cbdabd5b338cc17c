#!/usr/bin/env python
"""Benchmark: implicit Newton solves per second of the bonded-DEM solver.

Workload (one "step" = one Newton solve of one implicit-midpoint time step,
``NewtonBonds.step`` at relative residual 1e-6): a 64^3 jittered-lattice foam
(262,144 sites, ~1.95M bonds; seeded synthetic input, generator in
``dynamic-powerfoam_gb300/foam.py``) with density 1000, gravity -9.81 z,
bottom layer fixed, dt = 1e-3, successive steps of one trajectory.

Prints one JSON line.  ``value`` is solves/s with the load already in HBM;
``e2e`` is the same through the public API with the load copied from pinned
host memory and the new positions copied back every step.  The working set
(about 0.5 GB of bond state) is larger than L2, so no flush is needed.

``--impl reference`` times the reference algorithm on the host CPU instead
(the NumPy restatement in ``oracle/``, the reference code itself does not
travel), on a bounded sample of the same workload.
Multi-GPU (torchrun): independent replicas, one foam per rank, no collective
on the data path; rank 0 prints the aggregate.
"""
import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

import numpy as np  # noqa: E402

# DRAM bytes (dram__bytes_read.sum + dram__bytes_write.sum, one ncu capture on
# the 64^3 bench foam, profiles/end_pcg_hvp_64cube.txt): a bond-end PCG launch
# of exactly 20 iterations, and one bond-end HVP launch.
PCG_DRAM_BYTES_PER_ITERATION_64 = (4027809536 + 134359296)/20
HVP_DRAM_BYTES_PER_LAUNCH_64 = 199288576 + 3624960

METRIC = 'implicit Newton solves/s at rel. residual 1e-6 (64^3 jittered foam, 262k sites, ~1.95M bonds)'
UNIT = 'solves/s'
SMI_FIELDS = ('clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,'
              'clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,'
              'clocks_event_reasons.sw_power_cap')


def parse():
    p = argparse.ArgumentParser()
    p.add_argument('--gpus', type=int, default=1)
    p.add_argument('--steps', type=int, default=10)
    p.add_argument('--warmup', type=int, default=3)
    p.add_argument('--impl', default='ours', choices=('ours', 'reference'))
    p.add_argument('--lattice', type=int, default=64)
    p.add_argument('--dt', type=float, default=1e-3)
    p.add_argument('--tolerance', type=float, default=1e-6)
    p.add_argument('--seed', type=int, default=0)
    p.add_argument('--no-cpu-baseline', action='store_true')
    p.add_argument('--precision', default='mixed', choices=('mixed', 'f64'))
    p.add_argument('--plain-steps', type=int, default=3,
                   help='solves of the plain float64 solver timed beside the mixed one (0: skip)')
    p.add_argument('--hvp-launches', type=int, default=50, help='timed launches of the standalone HVP (0: skip)')
    p.add_argument('--profile-pcg', type=int, default=0,
                   help='run one elastic PCG launch of exactly this many iterations in an NVTX range "profile_pcg" '
                        '(for an ncu capture of its DRAM traffic)')
    p.add_argument('--adjoint-lattice', type=int, default=32, help='lattice size of the inverse-fit workload (0: skip)')
    p.add_argument('--adjoint-steps', type=int, default=50)
    p.add_argument('--adjoint-fd', type=int, default=4, help='bonds checked against central differences')
    p.add_argument('--served', type=int, default=512, help='requests of the served mixed-size stream (0: skip)')
    p.add_argument('--large-mix', type=int, default=0,
                   help='lattice size of the large served mix (128: one 128^3 foam for 10 steps with '
                        '--large-mix-count requests of 32^3 sites; 0: skip)')
    p.add_argument('--large-mix-count', type=int, default=64)
    p.add_argument('--large-mix-small', type=int, default=32)
    p.add_argument('--served-plain', type=int, default=64,
                   help='requests of the same stream solved one at a time by the plain float64 solver')
    p.add_argument('--served-rate', type=float, default=4000., help='Poisson arrival rate of the stream (1/s)')
    p.add_argument('--served-batch-sites', type=int, default=8_000_000, help='site capacity of one batch')
    return p.parse_args()


def foam_and_load(m, seed):
    import dpf_gb300
    foam = dpf_gb300.jittered_lattice_foam(m, seed=seed)
    return foam, dpf_gb300.gravity_load(foam)


def corner_subfoam(foam, load):
    """Sites with all unit coordinates < 1/2 (one eighth of the foam, same spacing)."""
    keep = np.all(foam['unit'] < .5, axis=1)
    index = -np.ones(len(keep), dtype=np.int64)
    index[keep] = np.arange(keep.sum())
    pairs = foam['pairs']
    both = keep[pairs[:, 0]] & keep[pairs[:, 1]]
    sub = dict(points=foam['points'][keep], radii=foam['radii'][keep], pairs=index[pairs[both]],
               areas=foam['areas'][both], masses=foam['masses'][keep], fixed=foam['fixed'][keep],
               young=foam['young'], shear=foam['shear'])
    return sub, load[keep]


def oracle_rate(foam, load, dt, tol, steps, warmup, budget_s):
    """Solves/s of the NumPy reference restatement on the one-eighth corner sub-foam,
    scaled to the full foam by bond count."""
    from oracle import dem
    sub, sload = corner_subfoam(foam, load)
    s = dem.NewtonBonds(sub['points'], sub['radii'], sub['pairs'], sub['areas'], sub['masses'], sub['fixed'],
                        young=sub['young'], shear=sub['shear'])
    for _ in range(warmup):
        s.step(dt, sload, tolerance=tol)
    t0 = time.perf_counter()
    done = 0
    while done < steps:
        s.step(dt, sload, tolerance=tol)
        done += 1
        if time.perf_counter() - t0 > budget_s:
            break
    elapsed = time.perf_counter() - t0
    scale = len(sub['pairs'])/len(foam['pairs'])
    sample = (f'{done} Newton step(s) of the NumPy float64 restatement of NewtonBonds.step on the one-eighth '
              f'corner sub-foam ({len(sub["points"])} sites, {len(sub["pairs"])} bonds, same spacing), '
              f'{elapsed:.1f} s, solves/s scaled by the bond-count ratio {scale:.4f}')
    return done/elapsed*scale, sample


class ClockSampler:
    def __init__(self, index):
        self.index = index
        self.file = tempfile.NamedTemporaryFile('w+', suffix='.csv', delete=False)
        self.proc = None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(['nvidia-smi', f'--id={self.index}', f'--query-gpu={SMI_FIELDS}',
                                          '--format=csv,noheader,nounits', '-lms', '200'],
                                         stdout=self.file, stderr=subprocess.DEVNULL)
        except OSError:
            self.proc = None
        return self

    def __exit__(self, *exc):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def ready(self, limit=3.):
        """Wait (up to ``limit`` s) for the first sample, so that nvidia-smi's own
        start-up (driver queries) stays out of the timed region."""
        t0 = time.time()
        while self.proc is not None and time.time() - t0 < limit:
            if os.path.getsize(self.file.name) > 0:
                return
            time.sleep(.02)

    def summary(self):
        self.file.flush()
        rows = []
        with open(self.file.name) as f:
            for line in f:
                parts = [x.strip() for x in line.split(',')]
                if len(parts) >= 8:
                    rows.append(parts)
        os.unlink(self.file.name)
        if not rows:
            return dict(sm_mhz=None, sm_max_mhz=None, reasons=['unsampled'], samples=0)
        sm = [float(r[0]) for r in rows if r[0].replace('.', '').isdigit()]
        mx = [float(r[1]) for r in rows if r[1].replace('.', '').isdigit()]
        names = ('hw_slowdown', 'hw_thermal_slowdown', 'sw_thermal_slowdown', 'sw_power_cap')
        reasons = sorted({n for r in rows for n, v in zip(names, r[4:8]) if v.lower() == 'active'})
        return dict(sm_mhz=statistics.median(sm) if sm else None, sm_max_mhz=max(mx) if mx else None,
                    reasons=reasons, samples=len(rows))


def run_hvp(s, dt, peak, peaks, launches=50):
    """Bond-HVPs/s of the float32 operator y = (diag M + dt^2/4 K) q of the
    elastic PCG (the bond-end sweep) on the bench foam: each launch timed
    alone with CUDA events on the launching stream, L2 flushed (a 256 MB
    write) between launches; also back to back (the end records, 188 MB, are
    larger than L2)."""
    import ctypes
    import torch
    from dpf_gb300 import _lib
    s._pack_ends(dt)
    stream = torch.cuda.current_stream()
    n, m = s.n_sites, s.n_bonds
    q = torch.randn((n, 6), dtype=torch.float32, device=s.device)
    y = torch.empty_like(q)
    flush = torch.empty(64 << 20, dtype=torch.float32, device=s.device)

    def launch():
        _lib.call('dpf_end_hvp', ctypes.byref(s._graph), s._ends.data_ptr(), s._site4.data_ptr(), q.data_ptr(),
                  y.data_ptr(), stream.cuda_stream)
    for _ in range(3):
        launch()
    times = []
    for _ in range(launches):
        flush.fill_(1.0)
        start, end = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        start.record(stream)
        launch()
        end.record(stream)
        times.append((start, end))
    start, end = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    start.record(stream)
    for _ in range(launches):
        launch()
    end.record(stream)
    torch.cuda.synchronize()
    ms = [a.elapsed_time(b) for a, b in times]
    mean = sum(ms)/len(ms)
    back_to_back = start.elapsed_time(end)/launches
    # algorithmic bytes of one float32 HVP: per bond i,j 8 + n, ri, rj 36 + k 16 = 60 B;
    # per site q 24 + y 24 + (m, I) 8 = 56 B
    alg = 60*m + 56*n
    achieved = alg/(mean*1e-3)/1e9
    return dict(kernel='end_hvp_kernel', bond_hvps_per_s=m/(mean*1e-3), mean_ms=mean, min_ms=min(ms),
                launches=len(ms), algorithmic_bytes=alg, traffic=HVP_DRAM_BYTES_PER_LAUNCH_64 if n == 262144 else None,
                achieved=achieved, peak=peak, unit='GB/s',
                frac=achieved/peak, peak_source='measured' if peaks else 'fallback', l2='flushed between launches',
                back_to_back_ms=back_to_back, back_to_back_frac=alg/(back_to_back*1e-3)/1e9/peak,
                end_records_bytes=int(s._ends.numel())*4)


def run_adjoint(args, device):
    """Gradient of the inverse-fit loss by the adjoint (implicit-function
    theorem, checkpoints every 10 steps), timed; checked against central
    differences (h = 1e-4) of the loss in ``args.adjoint_fd`` random bonds."""
    import torch
    steps, dt = args.adjoint_steps, 2e-3
    from dpf_gb300.adjoint import inverse_fit_problem
    model, theta0, loss = inverse_fit_problem(args.adjoint_lattice, 4, device, steps, dt, 10, 1e-12)
    theta = theta0.clone().requires_grad_(True)
    with torch.no_grad():
        loss(theta0)       # warm-up rollout (allocations, first launches), not timed
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    value = loss(theta)
    torch.cuda.synchronize()
    t1 = time.perf_counter()
    grad, = torch.autograd.grad(value, [theta])
    torch.cuda.synchronize()
    t2 = time.perf_counter()
    value = value.detach()
    out = dict(workload=f'{args.adjoint_lattice}^3 jittered foam, {model.solver.n_bonds} bonds, {steps} implicit '
                        f'steps dt={dt}, gravity + 3% top indentation load, hidden per-bond log-stiffness GRF '
                        '(l=0.2, mean log 1e5, std 0.5), MSE of positions; adjoint with checkpoints every 10 steps',
               loss=float(value), forward_s=t1 - t0, backward_s=t2 - t1, forward_ms_per_step=1e3*(t1 - t0)/steps,
               backward_ms_per_step=1e3*(t2 - t1)/steps, gradient_norm=float(grad.norm()),
               newton_tolerance=1e-12)
    if args.adjoint_fd > 0:
        rng = np.random.default_rng(5)
        # bonds with the largest gradients are the ones the loss sees best; mix
        # them with uniformly random bonds
        bonds = np.unique(np.concatenate([rng.choice(len(theta0), args.adjoint_fd//2, replace=False),
                                          torch.topk(grad.abs(), args.adjoint_fd - args.adjoint_fd//2)
                                          .indices.cpu().numpy()]))
        h, errs, rows = 1e-4, [], []
        with torch.no_grad():
            for b in bonds:
                e = torch.zeros_like(theta0)
                e[b] = h
                fd = (float(loss(theta0 + e)) - float(loss(theta0 - e)))/(2*h)
                g = float(grad[b])
                errs.append(abs(fd - g)/max(abs(fd), 1e-300))
                rows.append([int(b), g, fd])
        out.update(fd_bonds=len(bonds), fd_h=h, fd_max_relative_error=float(max(errs)),
                   fd_median_relative_error=float(np.median(errs)), fd_samples=rows[:8])
    return out


def run_large_mix(args, device, peak, peaks):
    """The large served mix: one jittered ``L^3`` foam under gravity (10 implicit
    steps at dt = 1e-3) served together with requests of 32^3 sites (randomized
    material, box and top load, one step each), all arriving at t = 0, under a
    150 GB budget; then the bond-end HVP on the large foam alone."""
    import torch
    import dpf_gb300
    from dpf_gb300 import serving
    t = time.time()
    reqs = serving.large_mix(big=args.large_mix, small=args.large_mix_small, count=args.large_mix_count,
                             seed=args.seed)
    build_s = time.time() - t
    sites = sum(r.sites for r in reqs)
    service = serving.Service(device=device, hbm_budget=150e9, max_batch_sites=max(8_000_000, sites))
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    finished = service.run(reqs)
    torch.cuda.synchronize()
    wall = time.perf_counter() - t0
    ok = [r for r in finished if r.error is None]
    solves = sum(r.done_steps for r in ok)
    lat = np.array([r.finished - r.arrival for r in ok])
    big = reqs[0]
    out = dict(workload=f'{args.large_mix}^3 foam x 10 steps + {args.large_mix_count} x {args.large_mix_small}^3 '
                        'requests, all at t = 0, 150 GB budget', requests=len(reqs), failed=len(reqs) - len(ok),
               big_sites=big.sites, big_bonds=big.bonds, sites=sites, solves=solves, wall_s=wall,
               solves_per_s=solves/wall, p50_ms=1e3*float(np.percentile(lat, 50)),
               p99_ms=1e3*float(np.percentile(lat, 99)), batched_steps=service.batches,
               phase_s={k: round(v, 4) for k, v in service.timers.items()}, foam_build_s=build_s,
               max_relative_residual=float(max(i['nonlinear_relative_residual'] for r in ok for i in r.infos)))
    del service, finished, ok
    f = big.foam
    s = dpf_gb300.MixedNewtonBonds(f['points'], f['radii'], f['pairs'], f['areas'], f['masses'], f['fixed'],
                                   young=f['young'], shear=f['shear'], device=device)
    s.step(big.dt, s.tensor(big.load), tolerance=args.tolerance)
    out['hvp'] = run_hvp(s, big.dt, peak, peaks, launches=20)
    del s
    torch.cuda.empty_cache()
    return out


def run_served(args, device):
    """Served stream vs the plain float64 solver (one request at a time).

    Stream: ``args.served`` requests, site counts log-uniform 1,024-131,072,
    box aspect U[0.5, 2], E log-uniform [1e4, 1e6], nu U[0.2, 0.4], top strain
    U[1%, 10%] (as a top load), Poisson arrivals; one implicit Newton solve per
    request at relative residual 1e-6.  Served: continuous batching of mixed-
    precision batched Newton steps under a 150 GB HBM budget.  Plain: float64
    ``NewtonBonds`` constructed and solved per request in arrival order.
    Latency = completion - arrival, request construction included in both arms.
    """
    import torch
    import dpf_gb300
    from dpf_gb300 import serving
    stream = serving.synthetic_stream(args.served, seed=11, sites=(1024, 131072), rate=args.served_rate)
    warm = serving.synthetic_stream(4, seed=12, sites=(1024, 4096))
    serving.Service(device=device).run(warm)
    torch.cuda.synchronize()
    service = serving.Service(device=device, hbm_budget=150e9, max_batch_sites=args.served_batch_sites)
    t0 = time.perf_counter()
    finished = service.run(stream)
    torch.cuda.synchronize()
    wall = time.perf_counter() - t0
    ok = [r for r in finished if r.error is None]
    stats = serving.latency_stats(finished)
    served = dict(requests=len(stream), solved=len(ok), failed=len(stream) - len(ok), wall_s=wall,
                  solves_per_s=len(ok)/wall, p50_ms=1e3*stats['p50'], p99_ms=1e3*stats['p99'],
                  batched_steps=service.batches, sites=int(sum(r.sites for r in stream)),
                  phase_s={k: round(v, 4) for k, v in service.timers.items()},
                  batch_sizes=service.batch_sizes,
                  newton_per_solve=float(np.mean([r.infos[0]['nonlinear_iterations'] for r in ok])),
                  max_relative_residual=float(max(r.infos[0]['nonlinear_relative_residual'] for r in ok)))
    del finished, ok, stream
    plain = None
    if args.served_plain > 0:
        stream = serving.synthetic_stream(args.served_plain, seed=11, sites=(1024, 131072), rate=args.served_rate)
        lat = []
        t0 = time.perf_counter()
        for req in stream:
            wait = req.arrival - (time.perf_counter() - t0)
            if wait > 0:
                time.sleep(wait)
            f = req.foam
            s = dpf_gb300.NewtonBonds(f['points'], f['radii'], f['pairs'], f['areas'], f['masses'], f['fixed'],
                                      young=f['young'], shear=f['shear'], device=device)
            s.step(req.dt, s.tensor(req.load), tolerance=args.tolerance)
            lat.append(time.perf_counter() - t0 - req.arrival)
        torch.cuda.synchronize()
        pwall = time.perf_counter() - t0
        plain = dict(requests=len(stream), solves_per_s=len(stream)/pwall, p50_ms=1e3*float(np.percentile(lat, 50)),
                     p99_ms=1e3*float(np.percentile(lat, 99)), dtype='f64', sample='first requests of the same stream')
        served['speedup_vs_plain'] = served['solves_per_s']/plain['solves_per_s']
    served['plain_f64'] = plain
    return served


_WORKER = {}


def _reference_worker_init(sub, sload):
    """Process-pool initializer: one NumPy reference solver per worker process."""
    from oracle import dem
    _WORKER['s'] = dem.NewtonBonds(sub['points'], sub['radii'], sub['pairs'], sub['areas'], sub['masses'],
                                   sub['fixed'], young=sub['young'], shear=sub['shear'])
    _WORKER['load'] = sload


def _reference_worker_step(args):
    dt, tol = args
    t0 = time.perf_counter()
    _WORKER['s'].step(dt, _WORKER['load'], tolerance=tol)
    return time.perf_counter() - t0


def replica_rates(ms, e_ms, steps, world, device='cpu'):
    """Whole-job rates of ``world`` replicas that each timed ``steps`` solves: the
    slowest rank's device and end-to-end times (all-reduce MAX over the process
    group when world > 1) and ``world * steps`` solves over those times."""
    import torch
    times = torch.tensor([ms, e_ms], dtype=torch.float64, device=device)
    if world > 1:
        import torch.distributed as dist
        dist.all_reduce(times, op=dist.ReduceOp.MAX)
    ms, e_ms = times.tolist()
    return ms, e_ms, world*steps/(ms*1e-3), world*steps/(e_ms*1e-3)


def run_reference(args):
    """The reference algorithm (NumPy restatement) on all host cores: one worker
    process per core, each advancing its own copy of the one-eighth corner
    sub-foam; a step is one Newton solve in every worker, solves/s scaled to
    the full foam by bond count."""
    import multiprocessing
    rank = int(os.environ.get('RANK', '0'))
    if rank != 0:
        return
    foam, load = foam_and_load(args.lattice, args.seed)
    sub, sload = corner_subfoam(foam, load)
    cores = os.cpu_count() or 1
    for var in ('OMP_NUM_THREADS', 'OPENBLAS_NUM_THREADS', 'MKL_NUM_THREADS'):
        os.environ[var] = '1'
    scale = len(sub['pairs'])/len(foam['pairs'])
    with multiprocessing.get_context('spawn').Pool(cores, initializer=_reference_worker_init,
                                                   initargs=(sub, sload)) as pool:
        task = [(args.dt, args.tolerance)]*cores
        for _ in range(max(1, min(args.warmup, 1))):
            pool.map(_reference_worker_step, task)
        t0 = time.perf_counter()
        for _ in range(max(1, args.steps)):
            pool.map(_reference_worker_step, task)
        elapsed = time.perf_counter() - t0
    steps = max(1, args.steps)
    rate = cores*steps/elapsed*scale
    sample = (f'{steps} step(s) x {cores} worker processes, each one Newton step of the NumPy float64 '
              f'restatement of NewtonBonds.step on the one-eighth corner sub-foam ({len(sub["points"])} sites, '
              f'{len(sub["pairs"])} bonds, same spacing), {elapsed:.1f} s, solves/s scaled by the bond-count '
              f'ratio {scale:.4f}')
    line = dict(impl='reference', metric=METRIC, value=rate, unit=UNIT, n_gpus=args.gpus, steps=args.steps,
                warmup=args.warmup, ms_per_step=1e3/rate if rate else None, higher_is_better=True,
                scaling='weak', vs_baseline=None, dtype='f64', data='synthetic',
                config=dict(workload=f'{args.lattice}^3 jittered-lattice foam, gravity, bottom fixed, '
                                     f'dt={args.dt}, NewtonBonds.step tol={args.tolerance}', lattice=args.lattice,
                            sites=len(foam['points']), bonds=len(foam['pairs'])),
                cpu_baseline=dict(value=rate, unit=UNIT, cores=cores, kind='port', sample=sample),
                e2e=dict(value=rate, unit=UNIT, h2d_bytes_per_step=0, d2h_bytes_per_step=0))
    print(json.dumps(line), flush=True)


def run_ours(args):
    import torch
    import torch.distributed as dist
    import dpf_gb300
    from dpf_gb300 import _lib

    world = int(os.environ.get('WORLD_SIZE', '1'))
    rank = int(os.environ.get('RANK', '0'))
    local = int(os.environ.get('LOCAL_RANK', '0'))
    torch.cuda.set_device(local)
    device = torch.device('cuda', local)
    if world > 1:
        dist.init_process_group('nccl', device_id=device)

    def barrier():
        if world > 1:
            dist.barrier()

    foam, load = foam_and_load(args.lattice, args.seed + rank)
    cls = dpf_gb300.MixedNewtonBonds if args.precision == 'mixed' else dpf_gb300.NewtonBonds
    s = cls(foam['points'], foam['radii'], foam['pairs'], foam['areas'], foam['masses'],
            foam['fixed'], young=foam['young'], shear=foam['shear'], device=device)
    ext = s.tensor(load)
    n_sites, n_bonds = s.n_sites, s.n_bonds
    for _ in range(args.warmup):
        s.step(args.dt, ext, tolerance=args.tolerance)
    torch.cuda.synchronize()

    # device-resident throughput
    infos = []
    launches0 = _lib.LAUNCHES['count']
    start, end = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    host_load = torch.from_numpy(load).pin_memory()
    host_x = torch.empty((n_sites, 3), dtype=torch.float64).pin_memory()
    dev_load = torch.empty_like(ext)
    # the end-to-end run below replays the same K steps from the same state
    snapshot = {name: getattr(s, name).clone() for name in s.PHYSICAL_STATE}
    snapshot_time = s.time
    with ClockSampler(local) as clocks:
        clocks.ready()
        barrier()
        torch.cuda.synchronize()
        start.record()
        for _ in range(args.steps):
            infos.append(s.step(args.dt, ext, tolerance=args.tolerance)[1])
        end.record()
        torch.cuda.synchronize()
        barrier()
        launches = _lib.LAUNCHES['count'] - launches0

        # end to end through the public API: pinned host load in, positions out, every step
        for name, value in snapshot.items():
            setattr(s, name, value.clone())
        s.time = snapshot_time
        barrier()
        torch.cuda.synchronize()
        e_start, e_end = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e_start.record()
        for _ in range(args.steps):
            dev_load.copy_(host_load, non_blocking=True)
            s.step(args.dt, dev_load, tolerance=args.tolerance)
            host_x.copy_(s.x, non_blocking=True)
        e_end.record()
        torch.cuda.synchronize()
        barrier()
    ms = start.elapsed_time(end)
    e_ms = e_start.elapsed_time(e_end)
    clock = clocks.summary()

    # launch timing of the hot kernels: the same steps again with CUDA events
    # around every launch (kept out of the timed regions above)
    s.profile = {}
    profiled = [s.step(args.dt, ext, tolerance=args.tolerance)[1] for _ in range(args.steps)]
    torch.cuda.synchronize()
    profile, s.profile = s.profile, None

    ms, e_ms, value, e2e = replica_rates(ms, e_ms, args.steps, world, device)

    # the plain float64 solver on the same foam, one step at a time (the comparator of the mixed and served forms)
    plain = None
    if args.precision == 'mixed' and args.plain_steps > 0:
        p64 = dpf_gb300.NewtonBonds(foam['points'], foam['radii'], foam['pairs'], foam['areas'], foam['masses'],
                                    foam['fixed'], young=foam['young'], shear=foam['shear'], device=device)
        p64.step(args.dt, ext, tolerance=args.tolerance)
        torch.cuda.synchronize()
        p_start, p_end = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        p_start.record()
        for _ in range(args.plain_steps):
            p64.step(args.dt, ext, tolerance=args.tolerance)
        p_end.record()
        torch.cuda.synchronize()
        p_ms = p_start.elapsed_time(p_end)
        plain = dict(value=args.plain_steps/(p_ms*1e-3), unit=UNIT, steps=args.plain_steps, dtype='f64',
                     ms_per_step=p_ms/args.plain_steps)
        del p64

    # roofline of the dominant launch
    kernels = {}
    for key, pairs in profile.items():
        durations = [a.elapsed_time(b) for a, b in pairs]
        kernels[key] = dict(launches=len(durations), total_ms=sum(durations),
                            mean_ms=sum(durations)/len(durations))
    cg = sum(i['cg_iterations'] for i in profiled)
    pcg_launches = max(1, kernels.get('pcg', {}).get('launches', 1))
    if args.precision == 'f64':
        # float64: JVP 160 B/bond + 192 B/site; one PCG iteration's K d sweep
        # 120 B/bond + 112 B/site plus 6x6 block and vector traffic (576 B/site).
        bytes_jvp = 160*n_bonds + 192*n_sites
        alg = dict(jvp=bytes_jvp, pcg=(120*n_bonds + 688*n_sites)*cg/pcg_launches, residual=bytes_jvp)
    else:
        # float32 bond data: JVP 80 B/bond + 96 B/site; HVP (K d) 60 B/bond +
        # 56 B/site plus the vector traffic of a single-reduction CG iteration
        # (read u, w, p, s, x, r and the 21-float block inverse, write p, s, x,
        # r, u: 348 B/site); residual 80 B/bond + 72 B/site; blocks 128 B/bond
        # (two incidences of the tangent) + 296 B/site; setup 160 B/bond of
        # float64 state read + 112 B/bond of records written + 144 B/site.
        alg = dict(jvp=80*n_bonds + 96*n_sites, pcg=(60*n_bonds + 404*n_sites)*cg/pcg_launches,
                   residual=80*n_bonds + 72*n_sites, scaling=128*n_bonds + 296*n_sites,
                   setup=272*n_bonds + 144*n_sites, commit=112*n_bonds + 208*n_bonds + 48*n_sites)
    dominant = max(kernels, key=lambda k: kernels[k]['total_ms']) if kernels else None
    peaks = {}
    try:
        with open(os.path.join(ROOT, 'MEASURED_PEAKS.json')) as f:
            peaks = json.load(f)
    except OSError:
        pass
    peak = float(peaks.get('hbm_gbs', 6800.))
    roof = None
    if dominant:
        achieved = alg[dominant]/(kernels[dominant]['mean_ms']*1e-3)/1e9
        traffic = None
        if dominant == 'pcg' and args.precision == 'mixed' and args.lattice == 64 and args.seed == 0 and \
                PCG_DRAM_BYTES_PER_ITERATION_64:
            traffic = PCG_DRAM_BYTES_PER_ITERATION_64*cg/pcg_launches
        roof = dict(bound='hbm', kernel=dominant, achieved=achieved, peak=peak, unit='GB/s', frac=achieved/peak,
                    traffic=traffic, algorithmic_bytes=alg[dominant],
                    traffic_source='ncu capture of this workload, scaled by CG iterations per launch'
                    if traffic else None, peak_source='measured' if peaks else 'fallback',
                    launches=kernels[dominant]['launches'], mean_ms=kernels[dominant]['mean_ms'])

    hvp = run_hvp(s, args.dt, peak, peaks, launches=args.hvp_launches) \
        if args.precision == 'mixed' and args.hvp_launches > 0 and s.sweep == 'ends' else None
    if args.profile_pcg > 0 and args.precision == 'mixed' and s.sweep == 'ends':
        s._pack_ends(args.dt)
        vec = torch.randn((n_sites, 6), dtype=torch.float64, device=device)
        out = torch.empty_like(vec)
        its = torch.zeros(1, dtype=torch.int32, device=device)
        torch.cuda.synchronize()
        torch.cuda.nvtx.range_push('profile_pcg')
        s._end_pcg(vec, out, 0.0, args.profile_pcg, its)
        torch.cuda.nvtx.range_pop()
        torch.cuda.synchronize()
    served = run_served(args, device) if args.served > 0 and args.precision == 'mixed' else None
    adjoint = run_adjoint(args, device) if args.adjoint_lattice > 0 and world == 1 else None
    large = run_large_mix(args, device, peak, peaks) if args.large_mix > 0 and world == 1 else None
    if rank != 0:
        return
    cpu = None
    if not args.no_cpu_baseline and world == 1:
        rate, sample = oracle_rate(foam, load, args.dt, args.tolerance, steps=1, warmup=0, budget_s=30.)
        cpu = dict(value=rate, unit=UNIT, cores=1, kind='port', sample=sample)
    mean = lambda k: sum(i[k] for i in infos)/len(infos)
    line = dict(metric=METRIC, value=value, unit=UNIT, n_gpus=world, steps=args.steps, warmup=args.warmup,
                ms_per_step=ms/args.steps, higher_is_better=True, scaling='weak', vs_baseline=None,
                dtype='f32+f64' if args.precision == 'mixed' else 'f64',
                data='synthetic (seeded jittered-lattice foam; no dataset)',
                config=dict(workload=f'{args.lattice}^3 jittered-lattice foam, gravity, bottom fixed, dt={args.dt}, '
                                     f'NewtonBonds.step tol={args.tolerance}, fgmres+elastic PCG, '
                                     + ('float32 bond sweeps + float64 reductions/residual'
                                        if args.precision == 'mixed' else 'float64'),
                            lattice=args.lattice, sites=n_sites, bonds=n_bonds, parallelism=f'replicas{world}',
                            l2='working set > L2 (no flush)',
                            newton_per_solve=mean('nonlinear_iterations'),
                            krylov_per_solve=mean('krylov_iterations'), cg_per_solve=mean('cg_iterations')),
                e2e=dict(value=e2e, unit=UNIT, h2d_bytes_per_step=int(load.nbytes),
                         d2h_bytes_per_step=int(n_sites*3*8)),
                gpu_launches=launches, kernels=kernels, roofline=roof, hvp=hvp, cpu_baseline=cpu, plain_f64=plain,
                served=served, adjoint=adjoint, large_mix=large,
                relative_residual_max=max(i['nonlinear_relative_residual'] for i in infos),
                clocks=dict(sm_mhz=clock['sm_mhz'], sm_max_mhz=clock['sm_max_mhz'], reasons=clock['reasons']))
    print(json.dumps(line), flush=True)
    if world > 1:
        dist.destroy_process_group()


def main():
    args = parse()
    if args.impl == 'reference':
        run_reference(args)
    else:
        run_ours(args)


if __name__ == '__main__':
    main()
