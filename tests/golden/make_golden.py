"""Generate golden vectors by running the reference's own Python code on CPU.

Run from the repository root in a container that has the reference checked
out (read-only) and torch/numpy/scipy installed:

    PYTHONDONTWRITEBYTECODE=1 python tests/golden/make_golden.py /path/to/reference [--only-linear-step]

It imports ``experiments.bonded_dem_*`` from the reference with
``device='cpu'``, builds the fixtures of the reference's own check scripts
(``bonded_dem_newton_checks.fixture`` seed 906, the complete graphs of
``bonded_dem_linear_gpu.checks`` seed 217, ``bonded_dem_tangent_warp.check``
seed 81 and ``bonded_dem_finite_checks`` seed 953, the FGMRES system of
``bonded_dem_newton_checks.main`` seed 381) plus one jittered 8^3 lattice
foam, and stores inputs and reference outputs as compressed ``.npz`` files
next to this script.  The tests read only those files; the reference itself
is never needed at test time.
"""
import os
import sys
from pathlib import Path

import numpy as np

os.environ.setdefault('PYTHONDONTWRITEBYTECODE', '1')
sys.dont_write_bytecode = True
HERE = Path(__file__).resolve().parent
REPO = HERE.parent.parent


def main(reference):
    sys.path.insert(0, str(reference))
    sys.path.insert(0, str(REPO))
    import torch
    from scipy.spatial.transform import Rotation
    torch.set_num_threads(1)
    from experiments.bonded_dem_core import ParallelBonds
    from experiments.bonded_dem_dynamics import reference_stiffness
    from experiments.bonded_dem_finite_gpu import FiniteBondsGPU, exp_rotation
    from experiments.bonded_dem_linear_gpu import LinearBondsGPU
    from experiments.bonded_dem_newton import NewtonBonds, fgmres
    import dpf_gb300

    def np64(t):
        return t.detach().cpu().numpy().astype(np.float64) if torch.is_tensor(t) else np.asarray(t)

    def state_of(s):
        return {f'state_{k}': np64(getattr(s, k)) for k in
                ('x', 'v', 'rotation', 'normal', 'offset', 'fn', 'fs', 'mt', 'mb')}

    # ---- bonded_dem_newton_checks.fixture (restated inputs, reference state) ----
    def newton_fixture(prestress, minimum_mass=1e-14, cls=NewtonBonds):
        rng = np.random.default_rng(906)
        p = np.array(np.meshgrid(np.arange(3), np.arange(2), np.arange(2))).reshape(3, -1).T*.4
        p = p + rng.normal(0, .008, p.shape)
        pairs = np.array([(i, j) for i in range(len(p)) for j in range(i+1, len(p))
                          if np.linalg.norm(p[i]-p[j]) < .65])
        radii = rng.uniform(.3, .4, len(p))
        area = rng.uniform(.008, .016, len(pairs))
        contacts = .5*(p[pairs[:, 0]]+p[pairs[:, 1]]) + rng.normal(0, .025, (len(pairs), 3))
        mass = np.geomspace(minimum_mass, 1., len(p)); rng.shuffle(mass)
        fixed = p[:, 0] < .1
        s = cls(p, radii, pairs, area, mass, fixed, contacts=contacts, device='cpu')
        if prestress:
            y = torch.zeros_like(s.mass)
            y[:, 1] = .025*s.p[:, 0]
            y[:, 3] = .02*s.p[:, 2]
            s.commit(s.trial(y)); s.rotation = exp_rotation(y[:, 3:])@s.rotation
            axis = np.array([.3, -.4, .6]); axis /= np.linalg.norm(axis)
            initial = s.x.cpu().numpy().copy()
            for step in range(12):
                rm = Rotation.from_rotvec(axis*1.2*(step+.5)/12).as_matrix()
                re = Rotation.from_rotvec(axis*1.2*(step+1)/12).as_matrix()
                mid, end = initial@rm.T, initial@re.T
                y = s.tensor(np.c_[np.cross(axis*.1, mid), np.tile(axis*.1, (len(p), 1))])
                s.commit(s.trial(y, mid_positions=s.tensor(mid), end_positions=s.tensor(end)))
                s.rotation = exp_rotation(y[:, 3:])@s.rotation
        inputs = dict(points=p, radii=radii, pairs=pairs, areas=area, masses=mass, fixed=fixed,
                      contacts=contacts, young=1200., shear=480.)
        return s, inputs

    def newton_case(name, prestress, minimum_mass=1e-14, dt=.02, seed=381):
        s, inputs = newton_fixture(prestress, minimum_mass)
        out = {f'in_{k}': np.asarray(v) for k, v in inputs.items()}
        out.update(state_of(s))
        rng = np.random.default_rng(seed)
        external = s.tensor(rng.normal(0, .01, s.mass.shape)); external[s.fixed] = 0
        y = s.tensor(rng.normal(0, .006, s.mass.shape)); y[s.fixed] = 0
        direction = s.tensor(rng.normal(size=s.mass.shape)); direction[s.fixed] = 0
        q = s.tensor(rng.normal(size=s.mass.shape))
        vector = s.tensor(rng.normal(size=s.mass.shape)); vector[s.fixed] = 0
        out.update(dt=dt, external=np64(external), y=np64(y), direction=np64(direction), q=np64(q),
                   vector=np64(vector))
        trial = s.trial(y)
        for k, v in trial.items():
            out[f'trial_{k}'] = np64(v)
        out['midpoint_force'] = np64(s.midpoint_force(y))
        out['residual'] = np64(s.residual(y, dt, external))
        out['loads'] = np64(s.loads())
        out['energy'] = s.energy()
        s.prepare_scaling(trial, dt)
        for k in ('diagonal', 'block', 'preconditioner', 'units'):
            out[f'scaling_{k}'] = np64(getattr(s, k))
        scaled_direction = direction*s.units
        jv = s.jacobian_vector(y, scaled_direction, dt, external)
        out['jvp_direction'] = np64(scaled_direction)
        out['jvp'] = np64(jv)
        out['scaled_jvp'] = np64(s.scale_residual(jv))
        out['stiffness_q'] = np64(s.stiffness(q))
        s.inner_iterations = 0
        out['elastic_precondition'] = np64(s.elastic_precondition(vector, dt))
        out['elastic_inner_iterations'] = s.inner_iterations
        # Full steps with the three solver configurations of the reference checks.
        load = torch.zeros_like(s.mass)
        load[:, 2] = -.03*s.mass[:, 0]; load[s.fixed] = 0
        out['step_load'] = np64(load)
        for tag, backend, pc in (('fgmres_elastic', 'fgmres', 'elastic'),
                                 ('fgmres_block', 'fgmres', 'block'), ('dense', 'dense', 'elastic')):
            solver, _ = newton_fixture(prestress, minimum_mass)
            work, info = solver.step(dt, load, tolerance=2e-7, backend=backend, preconditioning=pc,
                                     linear_tolerance=1e-7)
            for k, v in state_of(solver).items():
                out[f'step_{tag}_{k}'] = v
            out[f'step_{tag}_work'] = work
            out[f'step_{tag}_energy'] = solver.energy()
            for k in ('nonlinear_iterations', 'krylov_iterations', 'cg_iterations'):
                out[f'step_{tag}_{k}'] = info[k]
            out[f'step_{tag}_relative'] = info['nonlinear_relative_residual']
            out[f'step_{tag}_local'] = info['local_pose_defect']
        # the previous solver (FiniteBondsGPU.step, Anderson), as in bonded_dem_newton_checks.py:107-112
        solver, _ = newton_fixture(prestress, minimum_mass, cls=FiniteBondsGPU)
        work, info = solver.step(dt, load, tolerance=2e-7)
        for k, v in state_of(solver).items():
            out[f'step_previous_{k}'] = v
        out['step_previous_work'] = work
        out['step_previous_nonlinear_iterations'] = info['nonlinear_iterations']
        out['step_previous_cg_iterations'] = info['cg_iterations']
        np.savez_compressed(HERE/f'{name}.npz', **out)
        print(name, {k: out[k] for k in out if k.endswith('iterations')})

    newton_case('newton_prestressed', True)
    newton_case('newton_unstressed', False)

    # ---- complete graph, seed 217 (bonded_dem_linear_gpu.checks) ----
    rng = np.random.default_rng(217)
    p = rng.normal(size=(12, 3))
    pairs = np.array([(i, j) for i in range(len(p)) for j in range(i+1, len(p))])
    r = rng.uniform(.8, 1.2, len(p))
    lengths = np.linalg.norm(p[pairs[:, 1]]-p[pairs[:, 0]], axis=1)
    cpu = ParallelBonds(p, pairs, r, .12, 1200/lengths, 480/lengths)
    k = reference_stiffness(cpu).toarray()
    contacts = cpu.geometry(p)[1]
    gpu = LinearBondsGPU(p, r, pairs, cpu.area, contacts, np.ones(len(p)), np.zeros(len(p), bool), device='cpu')
    q = rng.normal(size=(len(p), 6))
    np.savez_compressed(HERE/'linear_217.npz', points=p, pairs=pairs, radii=r, areas=cpu.area,
                        contacts=contacts, q=q, stiffness_q=np64(gpu.stiffness(gpu.tensor(q))),
                        dense_k=k, diagonal=np64(gpu.diagonal), kn=np64(gpu.kn), ks=np64(gpu.ks),
                        kb=np64(gpu.kb), kt=np64(gpu.kt))

    # ---- complete graph, seed 81, offset contacts (bonded_dem_tangent_warp.check) ----
    rng = np.random.default_rng(81)
    p = rng.normal(size=(50, 3))
    pairs = np.array([(i, j) for i in range(50) for j in range(i+1, 50)])
    contacts = .5*(p[pairs[:, 0]]+p[pairs[:, 1]]) + rng.normal(0, .1, (len(pairs), 3))
    s = LinearBondsGPU(p, np.ones(50), pairs, np.ones(len(pairs)), contacts, np.ones(50),
                       np.zeros(50, bool), device='cpu')
    q = rng.normal(size=(50, 6))
    np.savez_compressed(HERE/'tangent_81.npz', points=p, pairs=pairs, contacts=contacts, q=q,
                        stiffness_q=np64(s.stiffness(s.tensor(q))), diagonal=np64(s.diagonal))

    # ---- finite law vs ParallelBonds history, seed 953 (bonded_dem_finite_checks) ----
    rng = np.random.default_rng(953)
    p = rng.normal(size=(8, 3)); r = rng.uniform(.6, 1.1, len(p))
    pairs = np.array([(i, j) for i in range(len(p)) for j in range(i+1, len(p))])
    length = np.linalg.norm(p[pairs[:, 1]]-p[pairs[:, 0]], axis=1)
    cpu = ParallelBonds(p, pairs, r, .12, 1200/length, 480/length)
    fin = FiniteBondsGPU(p, r, pairs, cpu.area, np.ones(len(p)), np.zeros(len(p), bool), device='cpu')
    ends, vs, ws = [], [], []
    for _ in range(80):
        v, w = rng.normal(0, .2, (len(p), 3)), rng.normal(0, 1., (len(p), 3))
        end = cpu.x + .01*v
        cpu.advance(end, v, w, .01)
        y = fin.tensor(np.c_[v, w]*.01)
        fin.commit(fin.trial(y, end_positions=fin.tensor(end)))
        ends.append(end); vs.append(v); ws.append(w)
    fc, tc = cpu.loads()
    np.savez_compressed(HERE/'finite_953.npz', points=p, radii=r, pairs=pairs, areas=cpu.area,
                        ends=np.array(ends), vs=np.array(vs), ws=np.array(ws),
                        cpu_fn=cpu.fn, cpu_fs=cpu.fs, cpu_mt=cpu.mt, cpu_mb=cpu.mb,
                        cpu_force=fc, cpu_torque=tc, fin_fn=np64(fin.fn), fin_fs=np64(fin.fs),
                        fin_mt=np64(fin.mt), fin_mb=np64(fin.mb), fin_loads=np64(fin.loads()),
                        fin_x=np64(fin.x), fin_normal=np64(fin.normal))

    # ---- parallel bonds with brittle failure (bonded_dem_core.ParallelBonds):
    # a jittered block pulled apart and sheared until bonds break ----
    rng = np.random.default_rng(512)
    g3 = np.array(np.meshgrid(np.arange(4), np.arange(3), np.arange(3), indexing='ij')).reshape(3, -1).T*.5
    p = g3 + rng.normal(0, .02, g3.shape)
    pairs = np.array([(i, j) for i in range(len(p)) for j in range(i+1, len(p))
                      if np.linalg.norm(p[i]-p[j]) < .75])
    r = rng.uniform(.25, .35, len(p))
    length = np.linalg.norm(p[pairs[:, 1]]-p[pairs[:, 0]], axis=1)
    core = ParallelBonds(p, pairs, r, .1, 1200/length, 480/length, tensile_strength=rng.uniform(40, 80, len(pairs)),
                         cohesion=rng.uniform(30, 60, len(pairs)), friction_angle=.3, moment_factor=.7)
    steps, ends, vs, ws = [], [], [], []
    x = p.copy()
    for step in range(40):
        v = np.zeros_like(p)
        v[:, 0] = .03*(p[:, 0] - p[:, 0].mean())          # stretch along x
        v[:, 2] = .02*(p[:, 1] - p[:, 1].mean())          # shear z along y
        v += rng.normal(0, .005, p.shape)
        w = rng.normal(0, .05, p.shape)
        dt = .05
        end = x + v*dt
        info = core.advance(end, v, w, dt)
        steps.append([info['newly_broken'], info['energy'], info['removed_bond_energy']])
        ends.append(end); vs.append(v); ws.append(w)
        x = end
    fc, tc = core.loads()
    np.savez_compressed(HERE/'parallel_512.npz', points=p, radii=r, pairs=pairs, bond_radius=.1,
                        kbar_n=1200/length, kbar_s=480/length, tensile=core.tensile_strength, cohesion=core.cohesion,
                        friction_angle=.3, moment_factor=.7, dt=.05, ends=np.array(ends), vs=np.array(vs),
                        ws=np.array(ws), steps=np.array(steps), fn=core.fn, fs=core.fs,
                        mt=core.mt, mb=core.mb, failure=core.failure, break_energy=core.break_energy, work=core.work,
                        x=core.x, normal=core.normal, force=fc, torque=tc)
    print('parallel_512 broken', int((core.failure > 0).sum()), 'of', len(pairs), 'tension',
          int((core.failure == 1).sum()), 'shear', int((core.failure == 2).sum()))

    # ---- static linear equilibrium (bonded_dem_material.solve_prescribed on the
    # reference_stiffness of a jittered specimen): clamped face, prescribed
    # stretch of the opposite face, random body loads ----
    from experiments.bonded_dem_material import solve_prescribed, specimen
    spec = specimen(3, length=2., jitter=.08)
    sb, sx = spec['bonds'], spec['x']
    k = reference_stiffness(sb)
    prescribed = np.zeros((len(sx), 6), bool)
    values = np.zeros((len(sx), 6))
    left, right = sx[:, 0] < 1e-9, sx[:, 0] > spec['length'] - 1e-9
    prescribed[left] = True
    prescribed[right, 0] = True
    values[right, 0] = .01
    srng = np.random.default_rng(733)
    load = srng.normal(0, 1e-3, (len(sx), 6))
    q, residual = solve_prescribed(k, prescribed, values, load)
    np.savez_compressed(HERE/'static_specimen.npz', points=sx, pairs=sb.pairs, radii=sb.radii, bond_radius=sb.rb,
                        kbar_n=sb.kn/sb.area, kbar_s=sb.ks/sb.area, dense_k=k.toarray(), prescribed=prescribed,
                        values=values, load=load, q=q.reshape(-1, 6), residual=residual)
    print('static_specimen', len(sx), 'sites', len(sb.pairs), 'bonds', residual)

    # ---- render hand-off (bonded_dem_powerfoam.state_from_bodies) of body poses ----
    from experiments.bonded_dem_powerfoam import appearance, state_from_bodies
    hrng = np.random.default_rng(4040)
    ref = hrng.uniform(0, 1, (30, 3))
    base = appearance(ref, np.full(30, .12), hrng.uniform(size=30) < .2)
    positions = ref + hrng.normal(0, .01, ref.shape)
    rotations = Rotation.from_rotvec(hrng.normal(0, .3, (30, 3))).as_matrix()
    state = state_from_bodies(base, positions, rotations)
    np.savez_compressed(HERE/'handoff_30.npz', positions=positions, rotations=rotations,
                        **{f'base_{k}': np.asarray(v) for k, v in base.items()},
                        **{f'state_{k}': np.asarray(v) for k, v in state.items()})

    # ---- FGMRES vs dense with a variable preconditioner, seed 381 ----
    rng = np.random.default_rng(381)
    a = torch.tensor(rng.normal(size=(36, 36)), dtype=torch.float64) + 8*torch.eye(36, dtype=torch.float64)
    b = torch.tensor(rng.normal(size=36), dtype=torch.float64)
    calls = [0]

    def variable_precondition(v):
        calls[0] += 1
        return v/(torch.diag(a)*(1+.08*np.sin(calls[0])))
    x, info = fgmres(lambda z: a@z, b, variable_precondition, tolerance=1e-10, restart=24)
    np.savez_compressed(HERE/'fgmres_381.npz', a=np64(a), b=np64(b), x=np64(x),
                        iterations=info['iterations'], relative=info['relative_residual'])

    # ---- differentiable rollout (bonded_dem_differentiable.py): per-cell log
    # stiffness multipliers, three implicit steps, weighted-position loss ----
    from experiments.bonded_dem_differentiable import DifferentiableBonds
    for name, prestress_case in (('adjoint_unstressed', False),):
        rng = np.random.default_rng(906)
        p = np.array(np.meshgrid(np.arange(3), np.arange(2), np.arange(2))).reshape(3, -1).T*.4
        p = p + rng.normal(0, .008, p.shape)
        pairs = np.array([(i, j) for i in range(len(p)) for j in range(i+1, len(p))
                          if np.linalg.norm(p[i]-p[j]) < .65])
        radii = rng.uniform(.3, .4, len(p))
        area = rng.uniform(.008, .016, len(pairs))
        contacts = .5*(p[pairs[:, 0]]+p[pairs[:, 1]]) + rng.normal(0, .025, (len(pairs), 3))
        mass = np.geomspace(.01, 1., len(p)); rng.shuffle(mass)
        fixed = p[:, 0] < .1
        model = DifferentiableBonds(points=p, radii=radii, pairs=pairs, areas=area, masses=mass, fixed=fixed,
                                    contacts=contacts, device='cpu')
        arng = np.random.default_rng(4242)
        theta = torch.tensor(arng.normal(0, .1, (len(p), 4)), dtype=torch.float64, requires_grad=True)
        steps, dt = 3, .02
        loads = []
        for t in range(steps):
            load = torch.zeros((len(p), 6), dtype=torch.float64)
            load[:, :3] = torch.tensor(arng.normal(0, .05, (len(p), 3)))
            load[:, 2] -= .3*torch.tensor(mass)
            load[torch.tensor(fixed)] = 0
            loads.append(load.requires_grad_(True))
        weights = torch.tensor(arng.normal(size=(steps+1, len(p), 3)), dtype=torch.float64)
        positions, _ = model.rollout(theta, loads, dt)
        loss = (positions*weights).sum()
        grads = torch.autograd.grad(loss, [theta] + loads)
        np.savez_compressed(HERE/f'{name}.npz', points=p, radii=radii, pairs=pairs, areas=area, masses=mass,
                            fixed=fixed, contacts=contacts, theta=np64(theta), loads=np.stack([np64(l) for l in loads]),
                            weights=np64(weights), dt=dt, positions=np64(positions), loss=float(loss.detach()),
                            grad_theta=np64(grads[0]), grad_loads=np.stack([np64(g) for g in grads[1:]]))
        print(name, float(loss), np.abs(np64(grads[0])).max())

    # ---- energy law (foam_dem_energy.py EnergyFoam, volume=False, small
    # kinematics): bond energy, force and world torque at a perturbed state ----
    from experiments.foam_dem_energy import EnergyFoam, quat_small
    for name, geometry in (('energy_fixture', None), ('energy_foam5', 5)):
        if geometry is None:
            _, g = newton_fixture(False)
            g = dict(g)
        else:
            foam = dpf_gb300.jittered_lattice_foam(geometry, seed=3)
            g = dict(points=foam['points'], radii=foam['radii'], pairs=foam['pairs'], areas=foam['areas'],
                     masses=foam['masses'], fixed=foam['fixed'], young=1200., shear=480.,
                     contacts=dpf_gb300.newton.classical_contacts(foam['points'], foam['radii'], foam['pairs']))
        young, shear = g.pop('young'), g.pop('shear')
        model = EnergyFoam(g, volume=False, device='cpu', young=young, shear=shear, kinematics='small')
        erng = np.random.default_rng(77)
        n = len(g['points'])
        scale = float(np.median(np.linalg.norm(g['points'][g['pairs'][:, 1]] - g['points'][g['pairs'][:, 0]], axis=1)))
        theta = torch.tensor(erng.normal(0, .2, (n, 5)), dtype=torch.float64)
        x = model.X + torch.tensor(erng.normal(0, .02*scale, (n, 3)), dtype=torch.float64)
        q = quat_small(torch.tensor(erng.normal(0, .1, (n, 3)), dtype=torch.float64))
        energy = model.energy(theta, x, q)
        f, tau = model.forces(theta, x, q)
        np.savez_compressed(HERE/f'{name}.npz', young=young, shear=shear, theta=np64(theta), x=np64(x), q=np64(q),
                            energy=float(energy), force=np64(f), torque=np64(tau),
                            **{f'in_{k}': np.asarray(v) for k, v in g.items()})
        print(name, float(energy), float(np.abs(np64(f)).max()))

    # ---- jittered 8^3 lattice foam under gravity, three reference steps ----
    foam = dpf_gb300.jittered_lattice_foam(8, seed=0)
    load = dpf_gb300.gravity_load(foam)
    s = NewtonBonds(foam['points'], foam['radii'], foam['pairs'], foam['areas'], foam['masses'],
                    foam['fixed'], young=foam['young'], shear=foam['shear'], device='cpu')
    out = dict(points=foam['points'], radii=foam['radii'], pairs=foam['pairs'], areas=foam['areas'],
               masses=foam['masses'], fixed=foam['fixed'], young=foam['young'], shear=foam['shear'],
               load=load, dt=1e-3)
    infos = []
    for step in range(3):
        work, info = s.step(1e-3, s.tensor(load), tolerance=1e-6)
        infos.append([info['nonlinear_iterations'], info['krylov_iterations'], info['cg_iterations']])
        out[f'work_{step}'] = work
    out.update(state_of(s))
    out['iterations'] = np.array(infos)
    np.savez_compressed(HERE/'lattice8.npz', **out)
    print('lattice8', infos)
    linear_step(reference)


def linear_step(reference):
    """The linear implicit-midpoint step of ``bonded_dem_linear_gpu.checks``
    (seed 217: 12 random points, complete graph, site 0 fixed, random load,
    dt = 0.03), run by the reference's LinearBondsGPU on the CPU, with the
    check's independent dense solve of the same step."""
    sys.path.insert(0, str(reference))
    import torch
    torch.set_num_threads(1)
    from experiments.bonded_dem_core import ParallelBonds
    from experiments.bonded_dem_dynamics import reference_stiffness
    from experiments.bonded_dem_linear_gpu import LinearBondsGPU
    rng = np.random.default_rng(217)
    p = rng.normal(size=(12, 3))
    pairs = np.array([(i, j) for i in range(len(p)) for j in range(i+1, len(p))])
    r = rng.uniform(.8, 1.2, len(p))
    lengths = np.linalg.norm(p[pairs[:, 1]]-p[pairs[:, 0]], axis=1)
    cpu = ParallelBonds(p, pairs, r, .12, 1200/lengths, 480/lengths)
    k = reference_stiffness(cpu).toarray()
    contacts = cpu.geometry(p)[1]
    gpu = LinearBondsGPU(p, r, pairs, cpu.area, contacts, np.ones(len(p)), np.zeros(len(p), bool), device='cpu')
    rng.normal(size=(len(p), 6))      # the K q probe vector of the check
    gpu.fixed[0] = True
    mass = gpu.mass.cpu().numpy().ravel()
    free = np.arange(6, len(mass))
    force = rng.normal(size=(len(p), 6))
    force[0] = 0
    dt = .03
    dense = np.zeros(len(mass))
    dense[free] = np.linalg.solve(np.diag(mass[free]) + dt*dt*k[np.ix_(free, free)]/4, .5*dt*dt*force.ravel()[free])
    work, metrics = gpu.step(dt, gpu.tensor(force))
    np.savez_compressed(HERE/'linear_step_217.npz', points=p, pairs=pairs, radii=r, areas=cpu.area, contacts=contacts,
                        fixed=gpu.fixed.numpy(), force=force, dt=dt, dense_q=dense.reshape(-1, 6),
                        step_q=gpu.q.numpy(), step_v=gpu.v.numpy(), step_kq=gpu.kq.numpy(), step_work=work,
                        step_energy=gpu.energy(), step_iterations=metrics['iterations'],
                        step_relative=metrics['relative_residual'])
    print('linear_step_217', metrics, work)


if __name__ == '__main__':
    args = [a for a in sys.argv[1:] if not a.startswith('--')]
    where = Path(args[0] if args else os.environ['DPF_REFERENCE'])
    if '--only-linear-step' in sys.argv:
        linear_step(where)
    else:
        main(where)
