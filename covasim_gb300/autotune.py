"""Autotuner for the stored layers' edge pass.

The pass runs either one 256-thread block per tile of edges (small tiles give
more blocks and shorter tails, large tiles amortise the per-block set-up), or
one wave of blocks each walking a balanced range of tiles ('w': the tile size
only sets how finely the ranges are balanced), or, for one sim, one block per
SM with the source bitmap resident in shared memory ('r'). The best choice
depends on the population, the layers and the epidemic's course, and on how
the redrawn layers' pass, which runs beside it, fills the device; so
``tune_edge_tile`` times whole runs of the actual sim with each variant (CUDA
events around the graph launch, state rewound between runs) and keeps the
fastest. Results are cached per workload signature and device name in memory
and, optionally, in a JSON file.
"""
import json
import os

import numpy as np
import torch

from . import _lib as L
from .sim import init_infections
from .state import parse_edge_tile

__all__ = ['tune_edge_tile', 'workload_signature']

_CACHE = {}


def workload_signature(state):
    """Edge counts per (stored, dynamic) layer kind, agents, sims, and the device."""
    stored = sum(int(r.n_edges) for r in state.segments if not r.dynamic)
    dynamic = sum(int(r.n_edges) for r in state.segments if r.dynamic)
    name = torch.cuda.get_device_name(state.device)
    return f'{name}|n={state.n}|sims={len(state.specs)}|stored={stored}|dynamic={dynamic}'


def _one_run(state, snap, t1):
    state.restore(snap)
    for k, sp in enumerate(state.specs):
        init_infections(state, k, sp.pars)
    state.run_days(0, t1, open_prev=False, close_last=True, use_graph=True)


def _candidates(state, tiles):
    """Labels: every tile, the one-wave variant of the stored layers' pass with each
    tile, and the resident-bitmap variant where it can run."""
    out = [str(int(t)) for t in tiles] + [f'{int(t)}w' for t in tiles]
    if state.resident_possible():
        out += [f'{int(t)}r' for t in tiles if int(t) >= 4096]
    return out


def tune_edge_tile(state, days=None, candidates=L.EDGE_TILES, reps=2, cache_file=None):
    """Pick the edge-pass variant for ``state`` (a freshly initialised ``BatchState``
    whose sims have not run): each tile size with one block per tile and as one
    wave, and for one sim also the variant with the source bitmap resident in
    shared memory, timed over ``reps`` whole runs of ``days`` days (default: all).
    Leaves the state rewound with the best variant set. Returns (best label,
    {label: ms per run}); a label is the tile size, suffixed 'w' for the one-wave
    pass and 'r' for the resident variant."""
    key = workload_signature(state) + f'|days={days}'
    if cache_file and os.path.exists(cache_file) and key not in _CACHE:
        with open(cache_file) as f:
            _CACHE.update(json.load(f))
    snap = state.snapshot()
    if key in _CACHE:
        best = str(_CACHE[key]['best'])
        state.set_edge_tile(**parse_edge_tile(best))
        return best, dict(_CACHE[key]['ms'])
    t1 = min(sp.npts for sp in state.specs) if days is None else int(days)
    stream = torch.cuda.current_stream()
    ms = {}
    for label in _candidates(state, candidates):
        state.set_edge_tile(**parse_edge_tile(label))
        for _ in range(2):  # a direct run, then the one that captures the graph the timed runs replay
            _one_run(state, snap, t1)
        times = []
        for _ in range(reps):
            a = torch.cuda.Event(enable_timing=True)
            b = torch.cuda.Event(enable_timing=True)
            a.record(stream)
            _one_run(state, snap, t1)
            b.record(stream)
            b.synchronize()
            times.append(a.elapsed_time(b))
        ms[label] = float(np.median(times))
    best = min(ms, key=ms.get)
    state.set_edge_tile(**parse_edge_tile(best))
    state.restore(snap)
    _CACHE[key] = {'best': best, 'ms': ms}
    if cache_file:
        os.makedirs(os.path.dirname(os.path.abspath(cache_file)), exist_ok=True)
        with open(cache_file, 'w') as f:
            json.dump(_CACHE, f, indent=1)
    return best, ms
