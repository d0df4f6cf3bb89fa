"""Autotuner for the edge pass's tile size.

The edge pass runs one 256-thread block per tile of edges. Small tiles give
more blocks (better balance between the cheap stored-edge tiles and the
Philox-bound dynamic-layer tiles, shorter tails); large tiles amortise the
per-block set-up (segment lookup, queue drains) over more edges. The best
size depends on the population, the layers and the epidemic's course, so
``tune_edge_tile`` times whole runs of the actual sim with each supported size
(CUDA events around the graph launch, state rewound between runs) and keeps
the fastest. Results are cached per workload signature and device name in
memory and, optionally, in a JSON file.
"""
import json
import os

import numpy as np
import torch

from . import _lib as L
from .sim import init_infections

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
    """(tile, resident) pairs: every tile, and the resident-bitmap variant where it can run."""
    out = [(int(t), False) for t in tiles]
    if state.resident_possible():
        out += [(int(t), True) for t in tiles if int(t) >= 4096]
    return out


def _label(tile, resident):
    return f'{tile}{"r" if resident else ""}'


def tune_edge_tile(state, days=None, candidates=L.EDGE_TILES, reps=2, cache_file=None):
    """Pick the edge-pass variant for ``state`` (a freshly initialised ``BatchState``
    whose sims have not run): each tile size, and for one sim also the variant
    with the source bitmap resident in shared memory, timed over ``reps`` whole
    runs of ``days`` days (default: all). Leaves the state rewound with the best
    variant set. Returns (best label, {label: ms per run}); a label is the tile
    size, suffixed 'r' for the resident variant."""
    key = workload_signature(state) + f'|days={days}'
    if cache_file and os.path.exists(cache_file) and key not in _CACHE:
        with open(cache_file) as f:
            _CACHE.update(json.load(f))
    snap = state.snapshot()
    if key in _CACHE:
        best = str(_CACHE[key]['best'])
        state.set_edge_tile(int(best.rstrip('r')), resident=best.endswith('r'))
        return best, dict(_CACHE[key]['ms'])
    t1 = min(sp.npts for sp in state.specs) if days is None else int(days)
    stream = torch.cuda.current_stream()
    ms = {}
    for tile, resident in _candidates(state, candidates):
        state.set_edge_tile(tile, resident=resident)
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
        ms[_label(tile, resident)] = float(np.median(times))
    best = min(ms, key=ms.get)
    state.set_edge_tile(int(best.rstrip('r')), resident=best.endswith('r'))
    state.restore(snap)
    _CACHE[key] = {'best': best, 'ms': ms}
    if cache_file:
        os.makedirs(os.path.dirname(os.path.abspath(cache_file)), exist_ok=True)
        with open(cache_file, 'w') as f:
            json.dump(_CACHE, f, indent=1)
    return best, ms
