"""ctypes binding of ``libdpf_gb300.so`` (declared in ``include/dpf_gb300.h``).

There is no fallback: if the library cannot be loaded the import of the
solver fails with an error naming the missing file and how to build it.
"""
import ctypes
import os
from pathlib import Path

HERE = Path(__file__).resolve().parent
LIBRARY = HERE/'libdpf_gb300.so'

DPF_ERR_ROTATION = 1
DPF_ERR_COINCIDENT = 2
DPF_ERR_NORMAL_TURN = 4
DPF_ERR_NONFINITE = 8
DPF_ERR_NOT_CONVERGED = 16
DPF_ERR_BARRIER_TIMEOUT = 32
DPF_ERR_ARGUMENT = 1 << 16
DPF_ERR_CUDA = 1 << 17
DPF_ERR_TOO_LARGE = 1 << 18

c_double_p = ctypes.c_void_p
i64, i32, f64, vp = ctypes.c_int64, ctypes.c_int, ctypes.c_double, ctypes.c_void_p


class Graph(ctypes.Structure):
    _fields_ = [('n_sites', i64), ('n_bonds', i64), ('edges', vp), ('inc_ptr', vp), ('inc_bond', vp)]


class Stiffness(ctypes.Structure):
    _fields_ = [('kn', vp), ('ks', vp), ('kb', vp), ('kt', vp)]


class History(ctypes.Structure):
    _fields_ = [('x', vp), ('radii', vp), ('normal', vp), ('offset', vp), ('fn', vp), ('fs', vp),
                ('mt', vp), ('mb', vp)]


class Tangent(ctypes.Structure):
    _fields_ = [('n', vp), ('ri', vp), ('rj', vp)]


class TrialOut(ctypes.Structure):
    _fields_ = [('force', vp), ('n', vp), ('ri', vp), ('rj', vp), ('x_end', vp), ('normal_end', vp),
                ('offset_end', vp), ('fs_end', vp), ('mb_end', vp), ('fn_end', vp), ('mt_end', vp)]


class ParallelParams(ctypes.Structure):
    _fields_ = [(k, vp) for k in ('kn', 'ks', 'kb', 'kt', 'area', 'second_moment', 'polar_moment', 'radius',
                                  'tensile', 'cohesion')] + [('tan_phi', f64), ('beta', f64)]


class ParallelState(ctypes.Structure):
    _fields_ = [(k, vp) for k in ('normal', 'fn', 'fs', 'mt', 'mb', 'break_energy', 'failure')]


class Tiles(ctypes.Structure):
    _fields_ = [('n_tiles', i64), ('n_entries', i64), ('n_halo', i64), ('meta_words', i64), ('max_entries', i32),
                ('max_sites', i32), ('max_halo', i32), ('max_meta_words', i32), ('tile_site', vp),
                ('tile_entry', vp), ('tile_halo', vp), ('tile_meta_off', vp), ('halo_site', vp), ('entry_bond', vp),
                ('entry_ends', vp), ('tile_desc', vp), ('tile_meta', vp)]


class MixedNewton(ctypes.Structure):
    """dpf_mixed_newton: buffers of a MixedNewtonBonds solver for the native step driver."""
    _fields_ = ([('graph', vp), ('stiffness', Stiffness)] +
                [(k, vp) for k in ('radii', 'mass', 'mass32', 'fixed', 'bond_data', 'r0', 'loads', 'scales',
                                   'wrench64', 'partials', 'scalars', 'status', 'y32', 'd32', 'wrench32', 'block32',
                                   'p32', 'units', 'units32', 'block32_b', 'p32_b', 'units_b', 'units32_b', 'ends',
                                   'site4', 'p24', 'end_workspace',
                                   'end_partials', 'barrier', 'inner', 'basis', 'transformed', 'products', 'w32',
                                   'h')] +
                [('krylov_width', i32)] +
                [(k, vp) for k in ('krylov_partials', 'krylov_scalars', 'vectors', 'host')] +
                [('end_variant', i32), ('history_corrections', vp)])


class NewtonStep(ctypes.Structure):
    """dpf_newton_step: one step's inputs and end-state outputs."""
    _fields_ = ([('dt', f64), ('external', vp), ('v', vp), ('rotation', vp), ('history', History)] +
                [(k, vp) for k in ('x_end', 'normal_end', 'offset_end', 'fn_end', 'fs_end', 'mt_end', 'mb_end')] +
                [('tolerance', f64), ('pose_tolerance', f64), ('linear_tolerance', f64),
                 ('max_iterations', i32), ('refresh', i32), ('timing', i32), ('v_in', vp), ('rotation_in', vp),
                 ('committed_start', i32)])


NEWTON_VECTORS = 10
NEWTON_HOST_DOUBLES = 128
NEWTON_TRACE = 32
NEWTON_TIMERS = ('setup', 'residual', 'scaling', 'pcg', 'jvp', 'commit', 'pack', 'krylov', 'norms', 'vector', 'accept')
(NEWTON_CONVERGED, NEWTON_GUARD, NEWTON_NONFINITE, NEWTON_SINGULAR, NEWTON_KRYLOV, NEWTON_LINE_SEARCH,
 NEWTON_DIVERGED) = range(7)


class NewtonInfo(ctypes.Structure):
    """dpf_newton_info: outcome, iteration counts, norms, trace and launch times of a step."""
    _fields_ = ([(k, i32) for k in ('outcome', 'guard', 'scaling_alternate', 'nonlinear_iterations', 'krylov_iterations',
                                    'cg_iterations', 'launches')] +
                [(k, f64) for k in ('relative', 'local', 'work', 'max_rotation', 'krylov_relative')] +
                [('trace_len', i32), ('trace', f64*(2*NEWTON_TRACE)), ('time_ms', f64*len(NEWTON_TIMERS)),
                 ('timed_launches', i32*len(NEWTON_TIMERS))])


P = ctypes.POINTER
SIGNATURES = {
    'dpf_wrench_scratch_doubles': (i64, [i64]),
    'dpf_partials_doubles': (i64, []),
    'dpf_elastic_workspace_doubles': (i64, [i64]),
    'dpf_stiffness_apply': (i32, [P(Graph), P(Stiffness), P(Tangent), vp, vp, vp, vp]),
    'dpf_diagonal_blocks': (i32, [P(Graph), P(Stiffness), P(Tangent), vp, vp]),
    'dpf_prepare_scaling': (i32, [P(Graph), P(Stiffness), P(Tangent), vp, vp, vp, f64, vp, vp, vp, vp, vp]),
    'dpf_trial': (i32, [P(Graph), P(Stiffness), P(History), vp, vp, vp, i32, P(TrialOut), vp, vp, vp]),
    'dpf_residual': (i32, [P(Graph), P(Stiffness), P(History), vp, vp, vp, vp, vp, f64, P(TrialOut), vp, vp,
                           vp, vp, vp, vp, vp, vp, vp]),
    'dpf_scale_residual': (i32, [i64, vp, vp, vp, vp, vp, vp, vp]),
    'dpf_jacobian_vector': (i32, [P(Graph), P(Stiffness), P(History), vp, vp, vp, vp, f64, vp, vp, vp, vp, vp]),
    'dpf_elastic_precondition': (i32, [P(Graph), P(Stiffness), P(Tangent), vp, vp, vp, vp, vp, vp, f64, f64, i32,
                                       vp, vp, vp, vp, vp, vp, vp]),
    'dpf_loads': (i32, [P(Graph), P(History), vp, vp, vp]),
    'dpf_bond_setup': (i32, [i64, i64, vp, vp, vp, vp, vp, vp, f64, f64, vp, vp, vp, vp, vp, vp, vp, vp, vp, vp, vp,
                             vp]),
    'dpf_accept_step': (i32, [i64, vp, f64, vp, vp, vp]),
    'dpf_energy': (i32, [P(Graph), P(Stiffness), P(History), vp, vp, vp, vp, vp]),
    'dpf_arnoldi_cgs2': (i32, [i64, vp, i64, i32, vp, vp, vp, vp]),
    'dpf_combine_rows': (i32, [i64, vp, i64, i32, P(ctypes.c_double), vp, vp]),
    'dpf_dot_norm': (i32, [i64, vp, vp, vp, vp, vp]),
    'dpf_axpby': (i32, [i64, f64, vp, f64, vp, vp, vp]),
    'dpf_rhs_scale': (i32, [i64, vp, vp, vp, vp, vp, f64, vp, vp, vp]),
    'dpf_masked_scale': (i32, [i64, vp, vp, vp, vp, vp]),
    'dpf_stiffness_apply_static': (i32, [P(Graph), P(Stiffness), P(Tangent), vp, vp, vp]),
    'dpf_mixed_bond_floats': (i64, [i64]),
    'dpf_mixed_workspace_floats': (i64, [i64, i64]),
    'dpf_mixed_setup': (i32, [P(Graph), P(Stiffness), P(History), vp, vp, vp, vp, f64, vp, vp, vp, vp, vp, vp, vp,
                              vp, vp]),
    'dpf_mixed_residual': (i32, [P(Graph), vp, vp, vp, vp, vp, f64, vp, i32, vp, vp, vp, vp, vp, vp, vp, vp, vp]),
    'dpf_mixed_scaling': (i32, [P(Graph), vp, vp, vp, vp, f64, vp, vp, vp, vp, vp]),
    'dpf_mixed_scale_residual': (i32, [i64, vp, vp, vp, vp, vp, vp, vp]),
    'dpf_mixed_jacobian_vector': (i32, [P(Graph), vp, vp, vp, vp, vp, f64, vp, vp, vp, vp, vp, vp, vp, vp]),
    'dpf_mixed_stiffness_apply': (i32, [P(Graph), vp, vp, vp, vp, vp]),
    'dpf_to_float': (i32, [i64, vp, vp, vp]),
    'dpf_mixed_precondition': (i32, [P(Graph), vp, vp, vp, vp, vp, vp, vp, f64, f64, i32, vp, vp, vp, vp, vp, vp,
                                     vp, vp, vp]),
    'dpf_mixed_commit': (i32, [P(Graph), vp, P(History), vp, vp, vp, vp, vp, vp, vp, vp, vp, vp, vp, vp]),
    'dpf_mixed_begin': (i32, [i64, vp, vp, vp, vp, vp, f64, vp, vp, vp, vp]),
    'dpf_mixed_residual_segmented': (i32, [P(Graph), vp, vp, vp, vp, vp, f64, vp, i32, vp, vp, vp, vp, vp, vp, vp, vp,
                                           vp, vp, vp, vp]),
    'dpf_segment_partials_doubles': (i64, [i32]),
    'dpf_segment_norms': (i32, [i32, vp, vp, vp, i32, vp, vp, vp, vp]),
    'dpf_segment_axpy': (i32, [i64, vp, vp, vp, vp, vp, vp]),
    'dpf_segment_select': (i32, [i64, vp, vp, vp, vp, vp, vp]),
    'dpf_static_max_bonds': (i64, []),
    'dpf_tile_graph': (i32, [i64, i64, vp, vp, vp, i32, i32, vp, vp, vp, vp, vp, vp, vp, vp, i64, vp, vp]),
    'dpf_tile_meta_capacity': (i64, [i64, i64]),
    'dpf_tile_entry_floats': (i64, [i64]),
    'dpf_tile_pack': (i32, [P(Tiles), vp, i64, f64, vp, vp, vp, i64, vp, vp, vp, vp]),
    'dpf_tiled_hvp': (i32, [P(Graph), P(Tiles), vp, vp, vp, vp, vp, i32, i32, vp]),
    'dpf_tiled_workspace_floats': (i64, [i64]),
    'dpf_end_floats': (i64, [i64]),
    'dpf_end_pack': (i32, [P(Graph), vp, f64, vp, vp, vp, vp, vp, vp, vp]),
    'dpf_end_variant_count': (i32, []),
    'dpf_end_variant_shape': (i32, [i32, P(ctypes.c_int), P(ctypes.c_int)]),
    'dpf_end_hvp': (i32, [P(Graph), vp, vp, vp, vp, i32, vp]),
    'dpf_end_precondition': (i32, [P(Graph), vp, vp, vp, vp, vp, vp, vp, f64, i32, vp, vp, vp, vp, vp, vp, vp, vp,
                                   i32, vp]),
    'dpf_tiled_partials_doubles': (i64, []),
    'dpf_tiled_precondition': (i32, [P(Graph), P(Tiles), vp, vp, vp, vp, vp, vp, vp, f64, i32, vp, vp, vp, vp, vp, vp,
                                     i32, i32, vp]),
    'dpf_energy_partials_doubles': (i64, []),
    'dpf_parallel_partials_doubles': (i64, []),
    'dpf_parallel_advance': (i32, [P(Graph), P(ParallelParams), vp, vp, vp, vp, vp, vp, f64, P(ParallelState),
                                   P(ParallelState), vp, vp, vp, vp]),
    'dpf_parallel_loads': (i32, [P(Graph), vp, vp, vp, vp, vp, vp, vp, vp, vp, vp, vp]),
    'dpf_bond_energy': (i32, [P(Graph), vp, vp, i64, vp, vp, vp, vp, vp, vp, vp, vp, vp, vp, vp]),
    'dpf_energy_tangent': (i32, [P(Graph), vp, vp, i64, vp, vp, vp, vp, vp, vp]),
    'dpf_adjoint_jacobian_doubles': (i64, [i64]),
    'dpf_adjoint_slot_doubles': (i64, [i64]),
    'dpf_adjoint_local_jacobian': (i32, [P(Graph), P(Stiffness), P(History), vp, vp, vp]),
    'dpf_adjoint_apply_jt': (i32, [P(Graph), vp, vp, vp, f64, vp, vp, vp, vp]),
    'dpf_adjoint_bond_vjp': (i32, [P(Graph), P(Stiffness), P(History), vp, vp, f64, vp, i32, vp, vp, vp, vp, vp,
                                   vp]),
    'dpf_operator_apply': (i32, [P(Graph), P(Stiffness), P(Tangent), vp, vp, f64, vp, vp, vp, vp]),
    'dpf_block_inverse': (i32, [i64, vp, vp, vp, f64, vp, vp, vp]),
    'dpf_block_pcg_workspace_doubles': (i64, [i64]),
    'dpf_block_pcg': (i32, [P(Graph), P(Stiffness), P(Tangent), vp, vp, vp, vp, vp, f64, f64, i32, i32, i32, vp, vp,
                            vp, vp, vp, vp, vp]),
    'dpf_linear_midpoint_rhs': (i32, [i64, vp, vp, vp, vp, f64, vp, vp, vp]),
    'dpf_linear_midpoint_advance': (i32, [i64, vp, f64, vp, vp, vp]),
    'dpf_small_partials_doubles': (i64, []),
    'dpf_linear_sums': (i32, [i64, vp, vp, vp, vp, vp, vp, vp, vp, vp]),
    'dpf_anderson_gram': (i32, [i64, vp, vp, i32, P(ctypes.c_int32), i32, vp, vp, vp, vp]),
    'dpf_anderson_mix': (i32, [i64, vp, vp, i32, P(ctypes.c_int32), i32, P(ctypes.c_double), vp, vp, vp]),
    'dpf_barrier_selftest': (i32, [i32, i64, i32, vp, vp, vp, vp]),
    'dpf_mixed_newton_step': (i32, [P(MixedNewton), P(NewtonStep), P(NewtonInfo), vp]),
    'dpf_end_precondition_f32': (i32, [P(Graph), vp, vp, vp, vp, vp, vp, vp, f64, i32, vp, vp, vp, vp, vp, vp, i32,
                                       vp]),
    'dpf_mixed_jacobian_vector_f32': (i32, [P(Graph), vp, vp, vp, vp, vp, f64, vp, vp, vp, vp, vp, vp]),
    'dpf_arnoldi_cgs2_f32': (i32, [i64, vp, i64, i32, vp, vp, vp, vp, vp, vp, vp]),
    'dpf_combine_rows_f32': (i32, [i64, vp, i64, i32, P(ctypes.c_double), vp, vp]),
    'dpf_scale_to_float': (i32, [i64, f64, vp, vp, vp]),
    'dpf_mixed_initial_residual': (i32, [i64, vp, vp, vp, vp, vp]),
    'dpf_mixed_wrench_floats': (i64, [i64]),
    'dpf_history_correction_floats': (i64, [i64]),
    'dpf_mixed_history_corrections': (i32, [P(Graph), P(History), vp, vp, vp]),
    'dpf_mixed_commit_lazy': (i32, [P(Graph), vp, vp, vp, vp, vp, vp, vp, vp, vp]),
    'dpf_mixed_fold_history': (i32, [P(Graph), vp, vp, vp, vp, vp, vp, vp, vp, vp, vp]),
    'dpf_newton_struct_sizes': (i32, [P(ctypes.c_int64)]),
}


# Kernels each entry point launches (the launch counter's unit).
KERNELS = {
    'dpf_stiffness_apply': 2, 'dpf_diagonal_blocks': 1, 'dpf_prepare_scaling': 1, 'dpf_trial': 2,
    'dpf_residual': 2, 'dpf_scale_residual': 1, 'dpf_jacobian_vector': 2, 'dpf_elastic_precondition': 1,
    'dpf_loads': 2, 'dpf_bond_setup': 2, 'dpf_accept_step': 1, 'dpf_energy': 1, 'dpf_arnoldi_cgs2': 4, 'dpf_combine_rows': 1,
    'dpf_dot_norm': 1, 'dpf_axpby': 1, 'dpf_rhs_scale': 1, 'dpf_masked_scale': 1,
    'dpf_stiffness_apply_static': 2, 'dpf_mixed_setup': 2, 'dpf_mixed_residual': 2, 'dpf_mixed_scaling': 1,
    'dpf_mixed_scale_residual': 1, 'dpf_mixed_jacobian_vector': 3, 'dpf_mixed_stiffness_apply': 2,
    'dpf_to_float': 1, 'dpf_mixed_precondition': 1, 'dpf_mixed_commit': 3, 'dpf_mixed_begin': 1, 'dpf_mixed_residual_segmented': 2, 'dpf_segment_norms': 2,
    'dpf_segment_axpy': 1, 'dpf_segment_select': 1,
    'dpf_adjoint_local_jacobian': 1, 'dpf_adjoint_apply_jt': 2, 'dpf_adjoint_bond_vjp': 2,
    'dpf_tile_pack': 2, 'dpf_tiled_hvp': 1, 'dpf_tiled_precondition': 1, 'dpf_end_pack': 2, 'dpf_end_hvp': 1,
    'dpf_end_precondition': 1, 'dpf_bond_energy': 3, 'dpf_parallel_advance': 2, 'dpf_parallel_loads': 2,
    'dpf_energy_tangent': 1, 'dpf_operator_apply': 2, 'dpf_block_inverse': 1, 'dpf_block_pcg': 1, 'dpf_linear_midpoint_rhs': 1, 'dpf_linear_midpoint_advance': 1,
    'dpf_linear_sums': 1, 'dpf_anderson_gram': 1, 'dpf_anderson_mix': 1, 'dpf_barrier_selftest': 1,
    'dpf_end_precondition_f32': 1, 'dpf_mixed_jacobian_vector_f32': 3, 'dpf_arnoldi_cgs2_f32': 1,
    'dpf_combine_rows_f32': 1, 'dpf_scale_to_float': 1, 'dpf_mixed_commit_lazy': 3, 'dpf_mixed_fold_history': 1, 'dpf_mixed_history_corrections': 1, 'dpf_mixed_initial_residual': 1,
}
LAUNCHES = {'count': 0}


class LibraryError(RuntimeError):
    pass


_LIB = None


def load():
    """Load the CUDA library once; raise if it is missing or incomplete."""
    global _LIB
    if _LIB is not None:
        return _LIB
    path = Path(os.environ.get('DPF_GB300_LIBRARY', LIBRARY))
    if not path.exists():
        raise LibraryError(f'{path} is missing: build it with `python -c "import __graft_entry__ as g; g.build()"` '
                           'or `python dynamic-powerfoam_gb300/build.py` (needs nvcc); there is no CPU fallback')
    lib = ctypes.CDLL(str(path))
    for name, (restype, argtypes) in SIGNATURES.items():
        fn = getattr(lib, name)
        fn.restype = restype
        fn.argtypes = argtypes
    _LIB = lib
    return lib


def check(code, name):
    """Raise for argument/launch errors returned by an entry point; count its kernels."""
    if code:
        raise LibraryError(f'{name} failed with status {code:#x}')
    LAUNCHES['count'] += KERNELS.get(name, 0)


def call(name, *args):
    """Call an entry point of the loaded library and check its status."""
    check(getattr(load(), name)(*args), name)
