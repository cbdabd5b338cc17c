"""Site tiles of a bond graph for the tiled float32 HVP and elastic PCG
(``dpf_tile_graph`` / ``dpf_tiled_hvp`` / ``dpf_tiled_precondition``), and the
autotuner that picks the tile size and CTA width per graph.

The tiled kernels compute ``(diag M + dt^2/4 K) q`` -- the operator of
``LinearBondsGPU._operator`` (``experiments/bonded_dem_linear_gpu.py:74-77``)
inside ``NewtonBonds.elastic_precondition``
(``experiments/bonded_dem_newton.py:107-130``) -- persistent CTAs stream the
tiles through a ring of shared-memory buffers (a bulk-copy warp, a halo-gather
warp, consumer warps).  ``MixedNewtonBonds`` uses them with ``sweep = 'tiles'``;
its default is the bond-end sweep, which needs no tiling.
"""
import ctypes

import numpy as np
import torch

from . import _lib

# Candidate (max entries per tile, consumer threads per CTA, tile buffers per CTA) of
# the autotuner; a CTA handles at most two entries per thread.
CANDIDATES = ((256, 128, 3), (256, 128, 4), (320, 160, 3), (384, 192, 3), (384, 192, 4))
DEFAULT = (384, 192, 3)


def host_tiles(edges, inc_ptr, inc_bond, n_sites, max_entries=DEFAULT[0], max_stage=65535):
    """Tile a graph on the host (``dpf_tile_graph``); returns numpy arrays and counts."""
    lib = _lib.load()
    edges = np.ascontiguousarray(edges, dtype=np.int64).reshape(-1, 2)
    inc_ptr = np.ascontiguousarray(inc_ptr, dtype=np.int32)
    inc_bond = np.ascontiguousarray(inc_bond, dtype=np.int32)
    m = len(edges)
    capacity = int(lib.dpf_tile_meta_capacity(n_sites, m))
    out = dict(tile_site=np.zeros(n_sites + 1, np.int32), tile_entry=np.zeros(n_sites + 1, np.int32),
               tile_halo=np.zeros(n_sites + 1, np.int32), tile_meta_off=np.zeros(n_sites + 1, np.int32),
               halo_site=np.zeros(max(1, 2*m), np.int32), entry_bond=np.zeros(max(1, 2*m), np.int32),
               entry_ends=np.zeros(max(1, 2*m), np.uint32), tile_meta=np.zeros(capacity, np.uint32),
               tile_desc=np.zeros(8*n_sites, np.int32))
    counts = np.zeros(9, np.int64)
    p = lambda a: a.ctypes.data_as(ctypes.c_void_p)
    _lib.check(lib.dpf_tile_graph(n_sites, m, p(edges), p(inc_ptr), p(inc_bond), int(max_entries), int(max_stage),
                                  p(out['tile_site']), p(out['tile_entry']), p(out['tile_halo']),
                                  p(out['tile_meta_off']), p(out['halo_site']), p(out['entry_bond']),
                                  p(out['entry_ends']), p(out['tile_meta']), capacity, p(out['tile_desc']),
                                  p(counts)),
               'dpf_tile_graph')
    (n_tiles, n_entries, n_halo, meta_words, max_e, max_sites, max_halo, max_meta,
     max_stage_used) = (int(c) for c in counts)
    for k in ('tile_site', 'tile_entry', 'tile_halo', 'tile_meta_off'):
        out[k] = out[k][:n_tiles + 1]
    out['halo_site'] = out['halo_site'][:max(1, n_halo)]
    out['entry_bond'] = out['entry_bond'][:max(1, n_entries)]
    out['entry_ends'] = out['entry_ends'][:max(1, n_entries)]
    out['tile_meta'] = out['tile_meta'][:meta_words]
    out['tile_desc'] = out['tile_desc'][:8*n_tiles]
    out.update(n_tiles=n_tiles, n_entries=n_entries, n_halo=n_halo, meta_words=meta_words, max_entries=max_e,
               max_sites=max_sites, max_halo=max_halo, max_meta_words=max_meta, max_stage=max_stage_used)
    return out


def tile_codes(host, tile):
    """(incidence offsets, first j-end offsets, entry codes) of one tile from
    its metadata words."""
    off, T = host['tile_meta_off'][tile], host['tile_site'][tile + 1] - host['tile_site'][tile]
    words = host['tile_meta'][off:host['tile_meta_off'][tile + 1]]
    ptr = (words[:T + 1] & 0xffff).astype(np.int64)
    mid = (words[:T] >> 16).astype(np.int64)
    codes = words[T + 1:].view(np.uint16)[:ptr[-1]]
    return ptr, mid, codes


class Tiles:
    """Device copy of a tiling plus its ``dpf_tiles`` descriptor and the
    packed entry records."""

    def __init__(self, host, device, threads=DEFAULT[1], stages=DEFAULT[2]):
        self.host = host
        self.threads = int(threads)
        self.stages = int(stages)
        dev = lambda k: torch.as_tensor(host[k].view(np.int32), device=device).contiguous()
        for k in ('tile_site', 'tile_entry', 'tile_halo', 'tile_meta_off', 'halo_site', 'entry_bond', 'entry_ends',
                  'tile_desc', 'tile_meta'):
            setattr(self, k, dev(k))
        self.n_entries = host['n_entries']
        lib = _lib.load()
        self.entries = torch.empty(max(4, lib.dpf_tile_entry_floats(self.n_entries)), dtype=torch.float32,
                                   device=device)
        self.status = torch.zeros(1, dtype=torch.int32, device=device)
        self.struct = _lib.Tiles(host['n_tiles'], host['n_entries'], host['n_halo'], host['meta_words'],
                                 host['max_entries'], host['max_sites'], host['max_halo'], host['max_meta_words'],
                                 *(getattr(self, k).data_ptr() for k in (
                                     'tile_site', 'tile_entry', 'tile_halo', 'tile_meta_off', 'halo_site',
                                     'entry_bond', 'entry_ends', 'tile_desc', 'tile_meta')))

    @classmethod
    def build(cls, edges, inc_ptr, inc_bond, n_sites, device, max_entries=DEFAULT[0], threads=DEFAULT[1],
              stages=DEFAULT[2]):
        return cls(host_tiles(edges, inc_ptr, inc_bond, n_sites, max_entries), device, threads, stages)

    @property
    def key(self):
        return (int(self.host['max_entries']), self.threads, self.stages)


def _graph_arrays(solver):
    return (solver.edges.cpu().numpy(), solver._inc_ptr.cpu().numpy(), solver._inc_bond.cpu().numpy())


# Autotuner results per graph shape: (n_sites, n_bonds) -> (max_entries, threads, stages).
_TUNED = {}


def autotune(solver, run, candidates=CANDIDATES, repeats=3):
    """Pick (max entries per tile, threads per CTA, buffers per CTA) for ``solver``'s graph.

    ``run(tiles)`` performs one representative launch sequence with a tiling
    (the caller packs entries first); each candidate is timed with CUDA
    events over ``repeats`` runs after one warm-up and the fastest median
    wins.  Results are cached per (sites, bonds); returns the winning
    ``Tiles`` and the timings {(max_entries, threads, stages): ms}.
    """
    key = (solver.n_sites, solver.n_bonds)
    edges, ptr, inc = _graph_arrays(solver)
    if key in _TUNED:
        max_entries, threads, stages = _TUNED[key]
        return Tiles.build(edges, ptr, inc, solver.n_sites, solver.device, max_entries, threads, stages), {}
    timings, built = {}, {}
    for max_entries, threads, stages in candidates:
        if max_entries not in built:
            try:
                built[max_entries] = host_tiles(edges, ptr, inc, solver.n_sites, max_entries)
            except _lib.LibraryError:
                continue
        tiles = Tiles(built[max_entries], solver.device, threads, stages)
        try:
            run(tiles)
        except _lib.LibraryError:
            continue
        samples = []
        for _ in range(repeats):
            start, end = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            start.record()
            run(tiles)
            end.record()
            end.synchronize()
            samples.append(start.elapsed_time(end))
        timings[(max_entries, threads, stages)] = float(np.median(samples))
        del tiles
    if not timings:
        raise _lib.LibraryError('no tiling candidate fits this graph')
    best = min(timings, key=timings.get)
    _TUNED[key] = best
    return Tiles(built[best[0]], solver.device, best[1], best[2]), timings


# Launch shape of the bond-end sweep per (device, size class): the autotuner
# times each compiled variant (lanes per site x CTAs per SM, see
# dpf_end_variant_shape) on the first elastic PCG of a graph of that size
# class and keeps the fastest for every later graph of the class.
_END_TUNED = {}


def end_size_class(n_sites, n_bonds):
    """Size class of a graph for the bond-end sweep: log2 of its incidences."""
    return int(np.log2(max(2*n_bonds, 1)))


def tune_end_sweep(solver, vector, iterations=5, nearest=0):
    """Variant index of the bond-end PCG for ``solver``'s graph: cached per
    (device, size class); otherwise each variant runs an elastic PCG of exactly
    ``iterations`` iterations on the solver's own packed records and
    ``vector`` (tolerance 0), once to warm up and once timed with CUDA events
    on the current stream, and the fastest is kept.  With ``nearest`` > 0 an
    untuned class takes the choice of the closest tuned class at most
    ``nearest`` classes away (the larger on a tie) instead of timing the
    variants: a served batch of a new size meets the timing's dozen launches
    (tens of ms at millions of sites) inside its step otherwise."""
    device, size = solver.device.index, end_size_class(solver.n_sites, solver.n_bonds)
    key = (device, size)
    if key in _END_TUNED:
        return _END_TUNED[key][0]
    for distance in range(1, nearest + 1):
        for near in (size + distance, size - distance):
            if (device, near) in _END_TUNED:
                return _END_TUNED[(device, near)][0]
    scratch = torch.empty_like(vector)
    count = torch.zeros(1, dtype=torch.int32, device=solver.device)
    stream = torch.cuda.current_stream(solver.device)
    times = {}
    for variant in range(_lib.load().dpf_end_variant_count()):
        solver._end_pcg(vector, scratch, 0., iterations, count, variant=variant)
        start, end = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        start.record(stream)
        solver._end_pcg(vector, scratch, 0., iterations, count, variant=variant)
        end.record(stream)
        end.synchronize()
        times[variant] = start.elapsed_time(end)
    best = min(times, key=times.get)
    _END_TUNED[key] = (best, times)
    return best
