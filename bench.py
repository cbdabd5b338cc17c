#!/usr/bin/env python
"""Benchmark: implicit Newton solves per second of the bonded-DEM solver.

Workload (one "step" = one Newton solve of one implicit-midpoint time step,
``NewtonBonds.step`` at relative residual 1e-6): a 64^3 jittered-lattice foam
(262,144 sites, ~1.95M bonds; seeded synthetic input, generator in
``dynamic-powerfoam_gb300/foam.py``) with density 1000, gravity -9.81 z,
bottom layer fixed, dt = 1e-3, successive steps of one trajectory, solved by
the mixed-precision form (float32 bond sweeps, float64 reductions and
residual).

Prints one JSON line.  ``value`` is solves/s with the load already in HBM;
``e2e`` is the same through the public API with the load copied from pinned
host memory and the new positions copied back every step.  The working set
(about 0.5 GB of bond state) is larger than L2, so no flush is needed.
``accuracy`` holds every timed step's error against a float64 solve of the
same inputs; ``served`` the mixed-size request stream (every request its own
foam) against the plain float64 solver over the same requests; ``large_mix``
the 128^3 foam served with 64 requests of 32^3 sites; ``adjoint`` the inverse
material fit.  The foams of the served workloads are triangulated on the
host in spawned worker processes (lowest priority) while the GPU measures
the rest; every timed region starts after its inputs exist.

``--impl reference`` times the reference algorithm on the host CPU instead
(the NumPy restatement in ``oracle/``; the reference code itself does not
travel) on the same full foam, one solver process per host core.
Multi-GPU (torchrun): independent replicas, one foam per rank, no collective
on the data path; rank 0 prints the aggregate.
"""
import argparse
import importlib.util
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

# DRAM bytes per algorithmic byte of the bond-end PCG and HVP launches, from
# one ncu capture (dram__bytes_read.sum + dram__bytes_write.sum) of the 64^3
# bench foam; applied to the algorithmic bytes of the measured size.
PCG_TRAFFIC_PER_ALGORITHMIC_BYTE = 0.921
HVP_TRAFFIC_PER_ALGORITHMIC_BYTE = 1.545

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
    p.add_argument('--accuracy', type=int, default=1, help='check every timed step against float64 solves (0: skip)')
    p.add_argument('--hvp-launches', type=int, default=50, help='timed launches of the standalone HVP (0: skip)')
    p.add_argument('--profile-pcg', type=int, default=0,
                   help='run one elastic PCG launch of exactly this many iterations in an NVTX range "profile_pcg" '
                        '(for an ncu capture of its DRAM traffic)')
    p.add_argument('--adjoint-lattice', type=int, default=32, help='lattice size of the inverse-fit workload (0: skip)')
    p.add_argument('--adjoint-steps', type=int, default=50)
    p.add_argument('--adjoint-fd', type=int, default=16, help='bonds checked against central differences')
    p.add_argument('--served', type=int, default=512, help='requests of the served mixed-size stream (0: skip)')
    p.add_argument('--served-plain', type=int, default=-1,
                   help='requests of the same stream solved one at a time by the plain float64 solver (-1: all)')
    p.add_argument('--served-accuracy', type=int, default=16,
                   help='served requests checked against a float64 solve of the same request')
    p.add_argument('--served-rate', type=float, default=4000., help='Poisson arrival rate of the stream (1/s)')
    p.add_argument('--served-batch-sites', type=int, default=8_000_000, help='site capacity of one batch')
    p.add_argument('--served-profile', action='store_true',
                   help='one more pass of the served stream, untimed, with every batched step profiled')
    p.add_argument('--large-mix', type=int, default=128,
                   help='lattice size of the large served mix (128: one 128^3 foam for 10 steps with '
                        '--large-mix-count requests of 32^3 sites; 0: skip)')
    p.add_argument('--large-mix-count', type=int, default=64)
    p.add_argument('--large-mix-small', type=int, default=32)
    p.add_argument('--foam-workers', type=int, default=0, help='host processes triangulating foams (0: cores - 1)')
    p.add_argument('--static-lattice', type=int, default=16,
                   help='lattice of the static energy-law configuration (bottom held, top pushed 5%%; 0: skip)')
    return p.parse_args()


def _foam_module():
    """The foam generator alone (NumPy/SciPy), without the package or torch."""
    spec = importlib.util.spec_from_file_location('_dpf_foam', os.path.join(ROOT, 'dynamic-powerfoam_gb300', 'foam.py'))
    module = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(module)
    return module


def _foam_worker_init():
    try:
        os.nice(19)
    except OSError:
        pass


def _foam_job(m, seed):
    return _foam_module().jittered_lattice_foam(m, seed=seed)


class FoamPool:
    """Jittered-lattice foams triangulated on the host in spawned worker
    processes at the lowest priority, so that the SciPy regular triangulation
    of the served workloads runs while the GPU measures the others."""

    def __init__(self, workers):
        import multiprocessing
        from concurrent.futures import ProcessPoolExecutor
        self.workers = workers
        self.executor = ProcessPoolExecutor(workers, mp_context=multiprocessing.get_context('spawn'),
                                            initializer=_foam_worker_init)

    def submit(self, m, seed):
        return self.executor.submit(_foam_job, m, seed)

    def close(self):
        self.executor.shutdown(wait=True, cancel_futures=True)


def foam_and_load(m, seed):
    import dpf_gb300
    foam = dpf_gb300.jittered_lattice_foam(m, seed=seed)
    return foam, dpf_gb300.gravity_load(foam)


def _single_thread_env():
    for var in ('OMP_NUM_THREADS', 'OPENBLAS_NUM_THREADS', 'MKL_NUM_THREADS'):
        os.environ[var] = '1'


_WORKER = {}


def _reference_worker_init(foam, load):
    """Process-pool initializer: one NumPy reference solver of the full foam per worker."""
    from oracle import dem
    _WORKER['s'] = dem.NewtonBonds(foam['points'], foam['radii'], foam['pairs'], foam['areas'], foam['masses'],
                                   foam['fixed'], young=foam['young'], shear=foam['shear'])
    _WORKER['load'] = load


def _reference_worker_step(args):
    """One Newton solve of the worker's own trajectory: (seconds, Newton, Krylov, CG)."""
    dt, tol = args
    t0 = time.perf_counter()
    _, info = _WORKER['s'].step(dt, _WORKER['load'], tolerance=tol)
    return (time.perf_counter() - t0, info['nonlinear_iterations'], info['krylov_iterations'],
            info['cg_iterations'])


def reference_rate(foam, load, dt, tol, workers, warmup, steps):
    """Solves/s of the NumPy restatement of ``NewtonBonds.step`` on the full
    foam: ``workers`` spawned processes (one thread each) each advance their
    own copy of the trajectory; ``warmup`` untimed solves, then ``steps`` timed
    solves spread over the processes.  Returns (rate, per-solve iteration
    means, sample text)."""
    import multiprocessing
    _single_thread_env()
    with multiprocessing.get_context('spawn').Pool(workers, initializer=_reference_worker_init,
                                                   initargs=(foam, load)) as pool:
        if warmup:
            pool.map(_reference_worker_step, [(dt, tol)]*min(warmup, workers), chunksize=1)
        t0 = time.perf_counter()
        rows = pool.map(_reference_worker_step, [(dt, tol)]*steps, chunksize=1)
        elapsed = time.perf_counter() - t0
    rows = np.array(rows)
    iterations = dict(newton_per_solve=float(rows[:, 1].mean()), krylov_per_solve=float(rows[:, 2].mean()),
                      cg_per_solve=float(rows[:, 3].mean()), seconds_per_solve=float(rows[:, 0].mean()))
    sample = (f'{steps} Newton solve(s) of the NumPy float64 restatement of NewtonBonds.step on the full '
              f'{len(foam["points"])}-site, {len(foam["pairs"])}-bond foam, {workers} single-threaded process(es) '
              f'each advancing its own trajectory, {min(warmup, workers) if warmup else 0} untimed warm-up solve(s), '
              f'{elapsed:.1f} s')
    return steps/elapsed, iterations, sample


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
    write) between launches; also back to back."""
    import ctypes
    import torch
    from dpf_gb300 import _lib
    s._pack_ends(dt)
    variant = s._end_variant or 0
    stream = torch.cuda.current_stream()
    n, m = s.n_sites, s.n_bonds
    q = torch.randn((n, 6), dtype=torch.float32, device=s.device)
    y = torch.empty_like(q)
    flush = torch.empty(64 << 20, dtype=torch.float32, device=s.device)

    def launch():
        _lib.call('dpf_end_hvp', ctypes.byref(s._graph), s._ends.data_ptr(), s._site4.data_ptr(), q.data_ptr(),
                  y.data_ptr(), variant, stream.cuda_stream)
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
                launches=len(ms), algorithmic_bytes=alg, traffic=HVP_TRAFFIC_PER_ALGORITHMIC_BYTE*alg,
                achieved=achieved, peak=peak, unit='GB/s', frac=achieved/peak,
                peak_source='measured' if peaks else 'fallback', l2='flushed between launches',
                back_to_back_ms=back_to_back, back_to_back_frac=alg/(back_to_back*1e-3)/1e9/peak,
                end_records_bytes=int(s._ends.numel())*4, variant=_end_shape(variant))


def run_adjoint(args, device):
    """Gradient of the inverse-fit loss by the adjoint (implicit-function
    theorem, checkpoints every 10 steps), timed after one untimed forward and
    backward pass; checked against central differences (h = 1e-4) of the loss
    on ``args.adjoint_fd`` bonds (half uniformly drawn, half the largest
    gradients)."""
    import torch
    steps, dt = args.adjoint_steps, 2e-3
    from dpf_gb300.adjoint import inverse_fit_problem
    model, theta0, loss = inverse_fit_problem(args.adjoint_lattice, 4, device, steps, dt, 10, 1e-12)
    theta = theta0.clone().requires_grad_(True)
    torch.autograd.grad(loss(theta), [theta])       # warm-up forward and backward, not timed
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
               newton_tolerance=1e-12, warmup='one forward and backward pass')
    if args.adjoint_fd > 0:
        rng = np.random.default_rng(5)
        bonds = np.unique(np.concatenate([rng.choice(len(theta0), args.adjoint_fd//2, replace=False),
                                          torch.topk(grad.abs(), args.adjoint_fd - args.adjoint_fd//2)
                                          .indices.cpu().numpy()]))
        h, errs, rows = 1e-4, [], []
        t3 = time.perf_counter()
        with torch.no_grad():
            for b in bonds:
                e = torch.zeros_like(theta0)
                e[b] = h
                fd = (float(loss(theta0 + e)) - float(loss(theta0 - e)))/(2*h)
                g = float(grad[b])
                errs.append(abs(fd - g)/max(abs(fd), 1e-300))
                rows.append([int(b), g, fd])
        out.update(fd_bonds=len(bonds), fd_h=h, fd_max_relative_error=float(max(errs)),
                   fd_median_relative_error=float(np.median(errs)), fd_samples=rows[:8],
                   fd_seconds=time.perf_counter() - t3)
    return out


def run_served(args, device, plan, bases):
    """Served stream vs the plain float64 solver (one request at a time).

    Stream: ``args.served`` requests, each its own seeded jittered-lattice
    foam with m^3 sites log-uniform in 1,024-131,072, box aspect U[0.5, 2],
    E log-uniform [1e4, 1e6], nu U[0.2, 0.4], top strain U[1%, 10%] (as a top
    load), Poisson arrivals; one implicit Newton solve per request at
    relative residual 1e-6.  Served: continuous batching of mixed-precision
    batched Newton steps under a 150 GB HBM budget.  Plain: float64
    ``NewtonBonds`` constructed (on the device) and solved per request, in
    arrival order, over the same requests.  Latency = completion - arrival.
    Warm-up: one untimed pass of the same stream (fresh request objects),
    which also lets the bond-end sweep's autotuner see the stream's batch
    size classes.
    """
    import torch
    import dpf_gb300
    from dpf_gb300 import serving
    from dpf_gb300.accuracy import served_accuracy
    serving.Service(device=device, hbm_budget=150e9, max_batch_sites=args.served_batch_sites).run(
        serving.planned_stream(plan, bases))
    torch.cuda.synchronize()
    stream = serving.planned_stream(plan, bases)
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
                  distinct_foams=len({id(r.foam['pairs']) for r in stream}),
                  phase_s={k: round(v, 4) for k, v in service.timers.items()},
                  batch_sizes=service.batch_sizes,
                  newton_per_solve=float(np.mean([r.infos[0]['nonlinear_iterations'] for r in ok])),
                  max_relative_residual=float(max(r.infos[0]['nonlinear_relative_residual'] for r in ok)))
    served['accuracy'] = served_accuracy(finished, args.served_accuracy, device)
    del finished, ok
    if getattr(args, 'served_profile', False):
        # per batched step: wall ms (device synced on either side) and the device
        # ms of every library entry point (the generic FGMRES's Arnoldi launches
        # are in the wall time only)
        profiled = serving.Service(device=device, hbm_budget=150e9, max_batch_sites=args.served_batch_sites,
                                   profile=True)
        profiled.run(serving.planned_stream(plan, bases))
        torch.cuda.synchronize()
        served['profile'] = profiled.profile
    plain = None
    count = len(stream) if args.served_plain < 0 else min(args.served_plain, len(stream))
    if count > 0:
        requests = sorted(stream)[:count]
        lat, build, solve = [], 0., 0.
        t0 = time.perf_counter()
        for req in requests:
            wait = req.arrival - (time.perf_counter() - t0)
            if wait > 0:
                time.sleep(wait)
            f = req.foam
            t1 = time.perf_counter()
            s = dpf_gb300.NewtonBonds(f['points'], f['radii'], f['pairs'], f['areas'], f['masses'], f['fixed'],
                                      young=f['young'], shear=f['shear'], device=device)
            ext = s.tensor(req.load)
            torch.cuda.synchronize()
            t2 = time.perf_counter()
            s.step(req.dt, ext, tolerance=args.tolerance)
            t3 = time.perf_counter()
            build += t2 - t1
            solve += t3 - t2
            lat.append(t3 - t0 - req.arrival)
            del s, ext
        torch.cuda.synchronize()
        pwall = time.perf_counter() - t0
        plain = dict(requests=count, solves_per_s=count/pwall, p50_ms=1e3*float(np.percentile(lat, 50)),
                     p99_ms=1e3*float(np.percentile(lat, 99)), dtype='f64', construction_s=build, solve_s=solve,
                     solve_only_solves_per_s=count/solve,
                     sample='every request of the same stream' if count == len(stream) else
                     f'the first {count} requests of the same stream')
        served['speedup_vs_plain'] = served['solves_per_s']/plain['solves_per_s']
        served['speedup_vs_plain_solve_only'] = served['solves_per_s']/plain['solve_only_solves_per_s']
    served['plain_f64'] = plain
    return served


def run_large_mix(args, device, peak, peaks, requests, build_s):
    """The large served mix: one jittered ``L^3`` foam under gravity (10 implicit
    steps at dt = 1e-3) served together with requests of 32^3 sites (each its
    own foam; randomized material, box and top load, one step each), all
    arriving at t = 0, under a 150 GB budget; then the bond-end HVP on the
    large foam alone."""
    import torch
    import dpf_gb300
    from dpf_gb300 import serving
    from dpf_gb300.accuracy import served_accuracy
    sites = sum(r.sites for r in requests)
    service = serving.Service(device=device, hbm_budget=150e9, max_batch_sites=max(8_000_000, sites))
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    finished = service.run(requests)
    torch.cuda.synchronize()
    wall = time.perf_counter() - t0
    ok = [r for r in finished if r.error is None]
    solves = sum(r.done_steps for r in ok)
    lat = np.array([r.finished - r.arrival for r in ok])
    big = requests[0]
    out = dict(workload=f'{args.large_mix}^3 foam x 10 steps + {args.large_mix_count} x {args.large_mix_small}^3 '
                        'requests (each its own foam), all at t = 0, 150 GB budget', requests=len(requests),
               failed=len(requests) - len(ok), big_sites=big.sites, big_bonds=big.bonds, sites=sites, solves=solves,
               wall_s=wall, solves_per_s=solves/wall, p50_ms=1e3*float(np.percentile(lat, 50)),
               p99_ms=1e3*float(np.percentile(lat, 99)), batched_steps=service.batches,
               phase_s={k: round(v, 4) for k, v in service.timers.items()}, foam_build_s=build_s,
               max_relative_residual=float(max(i['nonlinear_relative_residual'] for r in ok for i in r.infos)))
    out['accuracy'] = served_accuracy(finished, 8, device)
    del service, finished, ok
    f = big.foam
    s = dpf_gb300.MixedNewtonBonds(f['points'], f['radii'], f['pairs'], f['areas'], f['masses'], f['fixed'],
                                   young=f['young'], shear=f['shear'], device=device)
    s.step(big.dt, s.tensor(big.load), tolerance=args.tolerance)
    out['hvp'] = run_hvp(s, big.dt, peak, peaks, launches=20)
    del s
    torch.cuda.empty_cache()
    return out


def _end_shape(variant):
    """(lanes per site, CTAs per SM) of a bond-end sweep variant."""
    import ctypes
    from dpf_gb300 import _lib
    lanes, blocks = ctypes.c_int(), ctypes.c_int()
    _lib.check(_lib.load().dpf_end_variant_shape(int(variant), ctypes.byref(lanes), ctypes.byref(blocks)),
               'dpf_end_variant_shape')
    return dict(variant=int(variant), lanes_per_site=lanes.value, ctas_per_sm=blocks.value)


def _platen_problem(m, seed=0):
    """The static configuration: jittered m^3 foam, bottom lattice layer held,
    top layer pushed down by 5% of its height (whole sites held: a clamped
    platen)."""
    import dpf_gb300
    foam = dpf_gb300.jittered_lattice_foam(m, seed=seed)
    unit, h = foam['unit'], 1./m
    bottom, top = unit[:, 2] < h, unit[:, 2] > 1 - h
    prescribed = np.zeros((len(unit), 3))
    prescribed[top, 2] = -.05*foam['points'][top, 2]
    geometry = dict(points=foam['points'], radii=foam['radii'], pairs=foam['pairs'], areas=foam['areas'],
                    contacts=None, masses=foam['masses'], fixed=bottom | top)
    return foam, geometry, prescribed


def _static_oracle_job(m):
    """One static solve of the NumPy restatement (single thread, own process): (seconds, info, u)."""
    import dpf_gb300
    from oracle import dem
    foam, geometry, prescribed = _platen_problem(m)
    contacts = dpf_gb300.newton.classical_contacts(foam['points'], foam['radii'], foam['pairs'])
    b = dem.EnergyBonds(foam['points'], foam['radii'], foam['pairs'], foam['areas'], contacts, foam['masses'],
                        geometry['fixed'], foam['young'], foam['shear'])
    n = len(foam['points'])
    q0 = np.zeros((n, 4))
    q0[:, 0] = 1
    t0 = time.perf_counter()
    u, _, info = dem.energy_newton(b, np.zeros((n, 4)), foam['points'], q0, np.zeros((n, 6)), geometry['fixed'],
                                   prescribed, tolerance=1e-10)
    return time.perf_counter() - t0, {k: float(v) for k, v in info.items()}, u


def run_static(args, device):
    """The static configuration on the energy law: line-searched Newton to a
    relative gradient of 1e-10, timed on the GPU (CUDA events, after one
    untimed solve), beside one solve of the NumPy restatement on one host
    core; displacements compared."""
    import multiprocessing
    import torch
    import dpf_gb300
    foam, geometry, prescribed = _platen_problem(args.static_lattice)
    times, infos = [], []
    for k in range(4):
        solver = dpf_gb300.EnergyNewton(geometry, young=foam['young'], shear=foam['shear'], device=device)
        torch.cuda.synchronize()
        start, end = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        start.record()
        info = solver.solve(prescribed=prescribed, tolerance=1e-10)
        end.record()
        torch.cuda.synchronize()
        if k:
            times.append(start.elapsed_time(end))
            infos.append(info)
    u = (solver.x - solver.X).cpu().numpy()
    _single_thread_env()
    with multiprocessing.get_context('spawn').Pool(1) as pool:
        cpu_s, cpu_info, u_ref = pool.apply(_static_oracle_job, (args.static_lattice,))
    ms = float(np.mean(times))
    return dict(workload=f'{args.static_lattice}^3 jittered foam, energy law (EnergyFoam bond potential), bottom '
                         'layer held, top layer pushed down 5% (clamped platen), static equilibrium to relative '
                         'gradient 1e-10', sites=solver.n_sites, bonds=solver.n_bonds, solves_per_s=1e3/ms,
                ms_per_solve=ms, newton_iterations=infos[-1]['newton_iterations'],
                cg_iterations=infos[-1]['cg_iterations'], relative_gradient=infos[-1]['relative_gradient'],
                cpu=dict(kind='port', cores=1, seconds_per_solve=cpu_s, solves_per_s=1./cpu_s,
                         newton_iterations=cpu_info['newton_iterations'],
                         sample='one solve of the NumPy restatement (block-Jacobi CG Newton directions)'),
                displacement_rel_vs_cpu=float(np.linalg.norm(u - u_ref)/np.linalg.norm(u_ref)))


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
    """The reference algorithm (NumPy restatement of ``NewtonBonds.step``) on
    all host cores, on the same full foam and solver settings as our arm:
    one single-threaded process per core, each advancing its own copy of the
    trajectory; K timed solves spread over the processes."""
    rank = int(os.environ.get('RANK', '0'))
    if rank != 0:
        return
    foam, load = foam_and_load(args.lattice, args.seed)
    cores = os.cpu_count() or 1
    steps = max(1, args.steps)
    rate, iterations, sample = reference_rate(foam, load, args.dt, args.tolerance, cores, args.warmup, steps)
    line = dict(impl='reference', metric=METRIC, value=rate, unit=UNIT, n_gpus=args.gpus, steps=args.steps,
                warmup=args.warmup, ms_per_step=1e3/rate if rate else None, higher_is_better=True,
                scaling='weak', vs_baseline=None, dtype='f64',
                data='synthetic (seeded jittered-lattice foam; no dataset)',
                config=_config(args, len(foam['points']), len(foam['pairs']), int(os.environ.get('WORLD_SIZE', '1'))),
                iterations=iterations,
                cpu_baseline=dict(value=rate, unit=UNIT, cores=cores, kind='port', sample=sample),
                e2e=dict(value=rate, unit=UNIT, h2d_bytes_per_step=0, d2h_bytes_per_step=0))
    print(json.dumps(line), flush=True)


def _config(args, sites, bonds, world):
    """The workload description, identical in both arms (each arm reports its
    own iteration counts beside it)."""
    return dict(workload=f'{args.lattice}^3 jittered-lattice foam, gravity, bottom fixed, dt={args.dt}, '
                         f'NewtonBonds.step tol={args.tolerance}, fgmres+elastic PCG',
                lattice=args.lattice, sites=sites, bonds=bonds, dt=args.dt, tolerance=args.tolerance,
                parallelism=f'replicas{world}', l2='working set > L2 (no flush)')


def run_ours(args):
    import torch
    import torch.distributed as dist

    world = int(os.environ.get('WORLD_SIZE', '1'))
    rank = int(os.environ.get('RANK', '0'))
    local = int(os.environ.get('LOCAL_RANK', '0'))

    # host triangulation of the served workloads (largest first), in worker
    # processes that start only after the main leg's timed regions: the step
    # driver's host side must not share the cores with them while it is timed
    pool, large_jobs, served_jobs, plan = None, [], [], None

    def start_pool():
        nonlocal pool, plan
        if not (world == 1 and (args.served > 0 or args.large_mix > 0) and args.precision == 'mixed'):
            return None
        from dpf_gb300 import serving
        cores = os.cpu_count() or 2
        pool = FoamPool(args.foam_workers or max(1, cores - 1))
        if args.large_mix > 0:
            large_jobs.append(pool.submit(args.large_mix, args.seed))
            for k in range(args.large_mix_count):
                large_jobs.append(pool.submit(args.large_mix_small, args.seed + 1 + k))
        if args.served > 0:
            plan = serving.stream_plan(args.served, seed=11, sites=(1024, 131072), rate=args.served_rate)
            order = sorted(range(len(plan)), key=lambda k: -plan[k]['m'])
            futures = {k: pool.submit(plan[k]['m'], plan[k]['foam_seed']) for k in order}
            served_jobs.extend(futures[k] for k in range(len(plan)))
        return time.time()

    import dpf_gb300
    from dpf_gb300 import _lib
    from dpf_gb300.accuracy import restore, snapshot_state, trajectory_accuracy
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
    # the end-to-end run and the accuracy check replay the same K steps from the same state
    snapshot = snapshot_state(s)
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
        restore(s, *snapshot)
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
    restore(s, *snapshot)
    s.profile = {}
    profiled = [s.step(args.dt, ext, tolerance=args.tolerance)[1] for _ in range(args.steps)]
    torch.cuda.synchronize()
    profile, s.profile = s.profile, None

    ms, e_ms, value, e2e = replica_rates(ms, e_ms, args.steps, world, device)
    t_pool = start_pool()

    accuracy = None
    if args.accuracy and args.precision == 'mixed':
        accuracy = trajectory_accuracy(s, foam, ext, args.dt, args.tolerance, args.steps, snapshot, device)

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
    for key, entries in profile.items():
        # (start, end) CUDA events of the Python control path, or milliseconds
        # per launch measured by the library's step driver
        durations = [e if isinstance(e, float) else e[0].elapsed_time(e[1]) for e in entries]
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
        if dominant == 'pcg' and args.precision == 'mixed' and s.sweep == 'ends':
            traffic = PCG_TRAFFIC_PER_ALGORITHMIC_BYTE*alg[dominant]
        roof = dict(bound='hbm', kernel=dominant, achieved=achieved, peak=peak, unit='GB/s', frac=achieved/peak,
                    traffic=traffic, algorithmic_bytes=alg[dominant],
                    traffic_source='ncu DRAM bytes per algorithmic byte of this launch on the 64^3 foam'
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
    del s
    torch.cuda.empty_cache()
    served = None
    if served_jobs:
        from dpf_gb300 import serving
        bases = [job.result() for job in served_jobs]
        for base in bases:     # the requests' bonds as int32 site ids, as a server would receive them
            base['pairs'] = base['pairs'].astype(np.int32)
        served = run_served(args, device, plan, bases)
        served['foam_pool_s'] = time.time() - t_pool
        del bases
    adjoint = run_adjoint(args, device) if args.adjoint_lattice > 0 and world == 1 else None
    large = None
    if large_jobs:
        from dpf_gb300 import serving
        foams = [job.result() for job in large_jobs]
        build_s = time.time() - t_pool
        requests = serving.large_mix_requests(foams[0], foams[1:], seed=args.seed)
        large = run_large_mix(args, device, peak, peaks, requests, build_s)
        del foams, requests
    if pool is not None:
        pool.close()
    static = run_static(args, device) if args.static_lattice > 0 and world == 1 else None
    if rank != 0:
        return
    cpu = None
    if not args.no_cpu_baseline and world == 1:
        rate, iterations, sample = reference_rate(foam, load, args.dt, args.tolerance, 1, 0, 1)
        cpu = dict(value=rate, unit=UNIT, cores=1, kind='port', sample=sample, **iterations)
    mean = lambda k: sum(i[k] for i in infos)/len(infos)
    iterations = dict(newton_per_solve=mean('nonlinear_iterations'), krylov_per_solve=mean('krylov_iterations'),
                      cg_per_solve=mean('cg_iterations'))
    config = _config(args, n_sites, n_bonds, world)
    line = dict(metric=METRIC, value=value, unit=UNIT, n_gpus=world, steps=args.steps, warmup=args.warmup,
                ms_per_step=ms/args.steps, higher_is_better=True, scaling='weak', vs_baseline=None,
                dtype='f32+f64' if args.precision == 'mixed' else 'f64',
                data='synthetic (seeded jittered-lattice foam; no dataset)', config=config, iterations=iterations,
                precision='float32 bond sweeps + float64 reductions/residual' if args.precision == 'mixed'
                else 'float64',
                e2e=dict(value=e2e, unit=UNIT, h2d_bytes_per_step=int(load.nbytes),
                         d2h_bytes_per_step=int(n_sites*3*8)),
                gpu_launches=launches, kernels=kernels, roofline=roof, hvp=hvp, cpu_baseline=cpu, plain_f64=plain,
                accuracy=accuracy, served=served, adjoint=adjoint, large_mix=large, static=static,
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
