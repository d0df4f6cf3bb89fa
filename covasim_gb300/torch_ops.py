"""The day path's C ABI as torch custom ops ``torch.ops.covgpu.*``.

Every entry point of include/covgpu.h that ``BatchState`` calls goes through
one of these ops, so the day path is visible to torch as operators (tracing,
stream semantics, profiling) rather than as opaque ctypes calls. The
arguments keep the C ABI's meaning:

* ``state`` is the address of the ``covgpu_state`` descriptor (a ctypes
  structure owned by the BatchState; its device pointers name the state's
  tensors);
* ``status`` is the state's device status word (int32[1]). Every day kernel
  may write it, and it stands for the state's device arrays in the ops'
  ``mutates_args``, so that torch orders the ops as the C calls are ordered
  and never drops one as unused;
* tensors passed explicitly (index lists, outputs) are device tensors.

The ops enqueue on the current CUDA stream and return without synchronising,
like the C entry points; a non-OK status from the C call raises
``covasim_gb300._lib.CovgpuError``.
"""
import ctypes as C
from typing import Optional

import numpy as np
import torch

from . import _lib as L

__all__ = ['state_arg']


def _stream():
    return C.c_void_p(torch.cuda.current_stream().cuda_stream)


def _st(state):
    return C.cast(C.c_void_p(state), C.POINTER(L.State))


def _p(t):
    return None if t is None else t.data_ptr()


def state_arg(cstate):
    """The ``state`` argument of the ops for a ctypes ``covgpu_state``."""
    return C.addressof(cstate)


@torch.library.custom_op('covgpu::agent_step', mutates_args=('status',))
def agent_step(state: int, t: int, do_prev: bool, do_day: bool, steady: bool, status: torch.Tensor) -> None:
    """covgpu_agent_step: update_states_pre + check_immunity + update_nab + counts (people.py:164-186);
    steady: COVGPU_DAY_STEADY (a full pass has run since the state last changed outside the day kernels)."""
    L.call('covgpu_agent_step', _st(state), int(t), int(do_prev),
           int(do_day) | (L.DAY_STEADY if (steady and do_day) else 0), _stream())


@torch.library.custom_op('covgpu::edge_pass', mutates_args=('status',))
def edge_pass(state: int, t: int, status: torch.Tensor) -> None:
    """covgpu_edge_pass: compute_trans_sus + compute_infections over every layer and variant (sim.py:601-649)."""
    L.call('covgpu_edge_pass', _st(state), int(t), _stream())


@torch.library.custom_op('covgpu::infect_claims', mutates_args=('status',))
def infect_claims(state: int, t: int, status: torch.Tensor) -> None:
    """covgpu_infect_claims: People.infect for the day's first infectors (people.py:435-586)."""
    L.call('covgpu_infect_claims', _st(state), int(t), _stream())


@torch.library.custom_op('covgpu::infect_list', mutates_args=('status', 'infected'))
def infect_list(state: int, t: int, inds: torch.Tensor, sources: Optional[torch.Tensor], sim: int, variant: int,
                layer_tag: int, call_tag: int, infected: Optional[torch.Tensor], status: torch.Tensor) -> None:
    """covgpu_infect_list: People.infect for explicit global agent indices (people.py:435-586)."""
    L.call('covgpu_infect_list', _st(state), int(t), _p(inds), _p(sources), inds.numel(), int(sim), int(variant),
           int(layer_tag), int(call_tag), _p(infected), _stream())


@torch.library.custom_op('covgpu::import_day', mutates_args=('status',))
def import_day(state: int, t: int, status: torch.Tensor) -> None:
    """covgpu_import_day: the day's Poisson importations (sim.py:582-587)."""
    L.call('covgpu_import_day', _st(state), int(t), _stream())


@torch.library.custom_op('covgpu::test_trace', mutates_args=('status',))
def test_trace(state: int, t: int, status: torch.Tensor) -> None:
    """covgpu_test_trace: test_prob, contact_tracing and update_states_post (sim.py:596-600)."""
    L.call('covgpu_test_trace', _st(state), int(t), _stream())


@torch.library.custom_op('covgpu::lik_targets', mutates_args=('status',))
def lik_targets(state: int, t: int, status: torch.Tensor) -> None:
    """covgpu_lik_targets: the per-target half of the day's likelihood terms."""
    L.call('covgpu_lik_targets', _st(state), int(t), _stream())


@torch.library.custom_op('covgpu::rescale_check', mutates_args=('status',))
def rescale_check(state: int, t: int, status: torch.Tensor) -> None:
    """covgpu_rescale_check: whether a dynamic rescaling falls due on day t (sim.py:535-547)."""
    L.call('covgpu_rescale_check', _st(state), int(t), _stream())


@torch.library.custom_op('covgpu::run_days', mutates_args=('status',))
def run_days(state: int, t0: int, t1: int, open_prev: bool, close_last: bool, use_graph: bool,
             status: torch.Tensor) -> None:
    """covgpu_run_days: days [t0, t1) of every sim, captured as a CUDA graph (Sim.run, sim.py:733-755)."""
    L.call('covgpu_run_days', _st(state), int(t0), int(t1), int(open_prev), int(close_last), int(use_graph),
           _stream())


@torch.library.custom_op('covgpu::layer_lists', mutates_args=('status', 'counts', 'partners'))
def layer_lists(state: int, segment: int, t: int, agent_begin: int, n_agents: int, counts: torch.Tensor,
                offsets: Optional[torch.Tensor], partners: Optional[torch.Tensor], status: torch.Tensor) -> None:
    """covgpu_layer_lists: a dynamic layer's day-t contact lists (base.py:1849-1876)."""
    L.call('covgpu_layer_lists', _st(state), int(segment), int(t), int(agent_begin), int(n_agents), _p(counts),
           _p(offsets), _p(partners), _stream())


@torch.library.custom_op('covgpu::check', mutates_args=('status', 'out', 'counts'))
def check(state: int, t: int, which: int, sim: int, filter_exposed: bool, inds: Optional[torch.Tensor],
          n_agents: int, out: torch.Tensor, counts: torch.Tensor, status: torch.Tensor) -> None:
    """covgpu_check: one of People.check_infectious ... check_death, check_exit_iso (people.py:222-312, 368-374)."""
    L.call('covgpu_check', _st(state), int(t), int(which), int(sim), int(filter_exposed), _p(inds),
           0 if inds is None else inds.numel(), int(n_agents), _p(out), out.numel(), _p(counts), _stream())


@torch.library.custom_op('covgpu::check_immunity', mutates_args=('status',))
def check_immunity(state: int, t: int, sim: int, variant_mask: int, status: torch.Tensor) -> None:
    """covgpu_check_immunity: check_immunity(people, variants) (immunity.py:303-350)."""
    L.call('covgpu_check_immunity', _st(state), int(t), int(sim), int(variant_mask), _stream())


@torch.library.custom_op('covgpu::update_nab', mutates_args=('status',))
def update_nab(state: int, t: int, sim: int, inds: torch.Tensor, status: torch.Tensor) -> None:
    """covgpu_update_nab: update_nab(people, inds) (immunity.py:205-213)."""
    L.call('covgpu_update_nab', _st(state), int(t), int(sim), _p(inds), inds.numel(), _stream())


@torch.library.custom_op('covgpu::update_peak_nab', mutates_args=('status',))
def update_peak_nab(state: int, t: int, sim: int, inds: torch.Tensor, symp_class: Optional[torch.Tensor],
                    init_code: int, init_a: float, init_b: float, nab_boost: float, norm_factor: float,
                    call_tag: int, status: torch.Tensor) -> None:
    """covgpu_update_peak_nab: update_peak_nab(people, inds, nab_pars, symp) (immunity.py:138-202)."""
    L.call('covgpu_update_peak_nab', _st(state), int(t), int(sim), _p(inds), inds.numel(), _p(symp_class),
           L.DurPar(int(init_code), 0, float(init_a), float(init_b)), float(np.float32(nab_boost)),
           float(norm_factor), int(call_tag), _stream())
