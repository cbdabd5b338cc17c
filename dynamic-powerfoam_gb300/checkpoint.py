"""Trajectory runs with checkpoints and verified resume, in the reference's
output format (``experiments/bread_solver_run.py:46-53, 125-219``).

A run directory holds

* ``config.json`` -- the run's parameters and the SHA-256 of every mechanics
  source of this package (CUDA sources, headers, solver modules);
* ``progress.jsonl`` -- one record per completed output interval (step, time,
  energy, work, substeps, failed attempts, subdivision depth, iteration
  counts, local pose defect);
* ``attempts.jsonl`` -- one record per solve attempt (accepted or failed);
* ``final_state.npz`` -- ``x, rotation, fn, fs, mt, mb, normal, offset,
  velocity, time`` (the reference's keys), written atomically every
  ``checkpoint_every`` intervals;
* ``mechanics.json`` -- the report (completed intervals, time, counts,
  work-energy balance, orientation orthogonality, checks, failure).

``resume`` continues a saved run into a new directory after checking that the
mechanics sources are unchanged, the state's time matches the report, and
rebuilding the adaptive controller's memory from the accepted attempts.
"""
import hashlib
import json
import time
from pathlib import Path

import numpy as np
import torch

from .newton import AdaptiveIntervals

STATE_KEYS = ('x', 'rotation', 'fn', 'fs', 'mt', 'mb', 'normal', 'offset')
HERE = Path(__file__).resolve().parent


def mechanics_sources():
    """SHA-256 of the sources that define the mechanics (a resume needs them unchanged)."""
    files = sorted((HERE/'csrc').glob('*.cu')) + sorted((HERE/'csrc').glob('*.cuh')) + \
        sorted((HERE.parent/'include').glob('*.h')) + [HERE/name for name in ('newton.py', '_lib.py', 'tiles.py')]
    return {f.name: hashlib.sha256(f.read_bytes()).hexdigest() for f in files if f.exists()}


def save_state(solver, path):
    """``final_state.npz`` of a FiniteBonds/NewtonBonds solver, written atomically."""
    path = Path(path)
    tmp = path.with_name(path.stem + '.tmp.npz')
    np.savez_compressed(tmp, **{k: getattr(solver, k).detach().cpu().numpy() for k in STATE_KEYS},
                        velocity=solver.v.detach().cpu().numpy(), time=solver.time)
    tmp.replace(path)


def load_state(solver, path):
    """Set a solver's committed state from ``final_state.npz``."""
    with np.load(path) as a:
        for k in STATE_KEYS:
            setattr(solver, k, solver.tensor(a[k]))
        solver.v = solver.tensor(a['velocity'])
        solver.time = float(a['time'])


def _write_json(path, obj):
    tmp = path.with_name(path.stem + '.tmp.json')
    tmp.write_text(json.dumps(obj, indent=2) + '\n')
    tmp.replace(path)


class TrajectoryRun:
    """Advance ``solver`` by ``intervals`` output intervals of ``dt`` under
    ``load(t)`` with ``AdaptiveIntervals``; progress, attempts and checkpoints
    go to ``out`` (a new directory).  ``resume`` names a saved run to continue."""

    def __init__(self, solver, load, dt, intervals, out, checkpoint_every=8, resume=None, config=None):
        if intervals < 1 or dt <= 0 or checkpoint_every < 1:
            raise ValueError('positive intervals, dt and checkpoint_every required')
        self.s, self.load, self.dt, self.intervals = solver, load, float(dt), int(intervals)
        self.out = Path(out)
        self.out.mkdir(parents=True, exist_ok=True)
        if (self.out/'config.json').exists():
            raise ValueError('output already contains a run; select a new directory')
        self.checkpoint_every = int(checkpoint_every)
        self.hashes = mechanics_sources()
        self.controller = AdaptiveIntervals(solver)
        self.attempts, self.records = [], []
        self.work, self.elapsed, self.completed = 0., 0., 0
        previous = None
        if resume is not None:
            resume = Path(resume)
            previous = json.loads((resume/'mechanics.json').read_text())
            if previous['failure'] is not None or not previous['checks_pass']:
                raise ValueError('cannot resume a failed run')
            if previous['completed_intervals'] >= self.intervals:
                raise ValueError('the saved run already covers the requested intervals')
            for name, digest in previous['source_sha256'].items():
                if self.hashes.get(name) != digest:
                    raise ValueError(f'Resume requires unchanged mechanics: {name}')
            if not np.isclose(previous['dt'], self.dt, rtol=1e-13, atol=0):
                raise ValueError('resume needs the same dt')
            load_state(solver, resume/'final_state.npz')
            if abs(solver.time - previous['actual_time']) >= 1e-14:
                raise ValueError('saved state time does not match the report')
        self.config = dict(config or {}, intervals=self.intervals, dt=self.dt,
                           start_time=previous['start_time'] if previous else solver.time,
                           checkpoint_every=self.checkpoint_every, source_sha256=self.hashes)
        if previous:
            state = resume/'final_state.npz'
            self.config.update(resumed_from=str(resume), resume_source_sha256=previous['source_sha256'],
                               resume_state_sha256=hashlib.sha256(state.read_bytes()).hexdigest())
        _write_json(self.out/'config.json', self.config)
        self.initial_energy = solver.energy() if not previous else previous['initial_energy']
        self.peak_energy, self.worst_balance = self.initial_energy, 0.
        if previous:
            self._restore(resume, previous)

    def _restore(self, resume, previous):
        first = previous['completed_intervals']
        records = [json.loads(line) for line in (resume/'progress.jsonl').read_text().splitlines()]
        self.records = [r for r in records if r['step'] <= first]
        if len(self.records) != first or self.records[-1]['step'] != first:
            raise ValueError('progress records do not reach the checkpoint')
        self.attempts = [a for a in (json.loads(line) for line in (resume/'attempts.jsonl').read_text().splitlines())
                         if a['output_interval'] <= first]
        if len(self.attempts) != previous['attempts']:
            raise ValueError('attempt records do not match the report')
        # the controller's memory from the accepted attempts of every interval
        accepted = {}
        for a in self.attempts:
            if a['success']:
                accepted.setdefault(a['output_interval'], []).append(a)
        c = self.controller
        for row in self.records:
            c.depth = row['max_subdivision_depth']
            easy = max(a['nonlinear_iterations'] for a in accepted[row['step']]) <= 3
            c.easy_intervals = c.easy_intervals + 1 if easy else 0
            if c.easy_intervals >= 8 and c.depth:
                c.depth -= 1
                c.easy_intervals = 0
        self.work = self.records[-1]['work']
        self.elapsed = previous['elapsed_seconds']
        self.completed = first
        self.peak_energy = max([self.initial_energy, *(r['energy'] for r in self.records)])
        self.worst_balance = max(abs(r['energy'] - self.initial_energy - r['work']) for r in self.records)
        if abs(self.s.energy() - self.records[-1]['energy']) > 1e-12*max(1., abs(self.records[-1]['energy'])):
            raise ValueError('saved state energy does not match the progress record')
        (self.out/'progress.jsonl').write_text(''.join(json.dumps(r) + '\n' for r in self.records))
        (self.out/'attempts.jsonl').write_text(''.join(json.dumps(a) + '\n' for a in self.attempts))

    def _tracked(self):
        solver, attempts = self.s, self.attempts
        original = solver.step

        def step(dt, external, *args, **kwargs):
            torch.cuda.synchronize()
            tick = time.perf_counter()
            try:
                work, info = original(dt, external, *args, **kwargs)
                attempts.append(dict(dt=dt, success=True, elapsed_seconds=0.,
                                     **{k: v for k, v in info.items() if k != 'residual_trace'}))
                return work, info
            except RuntimeError as error:
                attempts.append(dict(dt=dt, success=False, elapsed_seconds=0., reason=str(error)))
                raise
            finally:
                torch.cuda.synchronize()
                attempts[-1]['elapsed_seconds'] = time.perf_counter() - tick
        return original, step

    def save(self, failure=None):
        s = self.s
        accepted = [a for a in self.attempts if a['success']]
        balance = self.worst_balance/max(self.peak_energy, abs(self.work), 1e-30)
        eye = torch.eye(3, dtype=s.rotation.dtype, device=s.rotation.device)
        orthogonality = float((s.rotation.transpose(1, 2)@s.rotation - eye).abs().max())
        fixed_ok = bool(torch.equal(s.x[s.fixed], s.p[s.fixed])) and not bool(s.v[s.fixed].any())
        report = dict(self.config, complete=self.completed == self.intervals and failure is None,
                      completed_intervals=self.completed, actual_time=s.time, elapsed_seconds=self.elapsed,
                      steps=self.completed, actual_substeps=len(accepted), attempts=len(self.attempts),
                      failed_attempts=len(self.attempts) - len(accepted),
                      solve_seconds=sum(a['elapsed_seconds'] for a in self.attempts),
                      max_subdivision_depth=max((r['max_subdivision_depth'] for r in self.records), default=0),
                      max_local_pose_defect=max((a['local_pose_defect'] for a in accepted), default=0),
                      max_nonlinear_relative_residual=max((a['nonlinear_relative_residual'] for a in accepted),
                                                          default=0),
                      initial_energy=self.initial_energy, work_energy_error_over_peak=balance,
                      orientation_orthogonality_max_error=orthogonality, fixed_state_unchanged=fixed_ok,
                      checks_pass=balance < .002 and orthogonality < 1e-10 and fixed_ok, failure=failure)
        if mechanics_sources() != self.hashes:
            raise RuntimeError('mechanics sources changed during the run')
        save_state(s, self.out/'final_state.npz')
        _write_json(self.out/'mechanics.json', report)
        return report

    def run(self):
        s = self.s
        original, tracked = self._tracked()
        s.step = tracked
        report = None
        try:
            for step in range(self.completed, self.intervals):
                before = len(self.attempts)
                torch.cuda.synchronize()
                tick = time.perf_counter()
                delta, info = self.controller.advance(self.dt, self.load)
                torch.cuda.synchronize()
                self.elapsed += time.perf_counter() - tick
                self.work += delta
                self.completed = step + 1
                energy = s.energy()
                self.peak_energy = max(self.peak_energy, energy)
                self.worst_balance = max(self.worst_balance, abs(energy - self.initial_energy - self.work))
                row = dict(step=self.completed, time=s.time, elapsed_seconds=self.elapsed, energy=energy,
                           work=self.work, substeps=len(info),
                           failed_attempts=sum(not a['success'] for a in self.attempts[before:]),
                           max_subdivision_depth=max(a['subdivision_depth'] for a in info),
                           nonlinear_iterations=sum(a['nonlinear_iterations'] for a in info),
                           cg_iterations=sum(a['cg_iterations'] for a in info),
                           krylov_iterations=sum(a.get('krylov_iterations', 0) for a in info),
                           max_local_pose_defect=max(a['local_pose_defect'] for a in info))
                self.records.append(row)
                with (self.out/'progress.jsonl').open('a') as f:
                    f.write(json.dumps(row) + '\n')
                with (self.out/'attempts.jsonl').open('a') as f:
                    for a in self.attempts[before:]:
                        f.write(json.dumps(dict(output_interval=self.completed, **a)) + '\n')
                for a in self.attempts[before:]:
                    a['output_interval'] = self.completed
                if self.completed % self.checkpoint_every == 0 or self.completed == self.intervals:
                    report = self.save()
        except Exception as error:
            self.save(repr(error))
            raise
        finally:
            s.step = original
        return report
