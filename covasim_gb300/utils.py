"""The reference's three numba kernels as GPU drop-ins (covasim/utils.py:38-128).

Same names, arguments and return values as ``cv.compute_viral_load``,
``cv.compute_trans_sus`` and ``cv.compute_infections``. numpy inputs give
numpy outputs (copied through the device); torch CUDA tensors stay on the
device. They are also registered as torch custom ops ``covgpu::*``.
"""
import ctypes as C

import numpy as np
import torch

from . import _lib as L

__all__ = ['compute_viral_load', 'compute_trans_sus', 'compute_infections']

_F32, _I32, _U8, _F64 = torch.float32, torch.int32, torch.uint8, torch.float64


def _stream():
    return C.c_void_p(torch.cuda.current_stream().cuda_stream)


def _dev(x, dtype):
    if torch.is_tensor(x):
        return x.to(device='cuda', dtype=dtype).contiguous()
    return torch.from_numpy(np.ascontiguousarray(np.asarray(x), dtype=torch.empty(0, dtype=dtype).numpy().dtype)).cuda()


def _ptr(t):
    return t.data_ptr() if t is not None and t.numel() else None


# ---------------------------------------------------------------- torch custom ops
@torch.library.custom_op('covgpu::compute_viral_load', mutates_args=())
def _viral_load_op(t: int, time_start: torch.Tensor, time_recovered: torch.Tensor, time_dead: torch.Tensor,
                   frac_time: float, load_ratio: float, high_cap: float) -> torch.Tensor:
    n = time_start.numel()
    out = torch.empty(n, dtype=_F32, device=time_start.device)
    L.call('covgpu_viral_load', int(t), _ptr(time_start), _ptr(time_recovered), _ptr(time_dead), n,
           float(np.float32(frac_time)), float(np.float32(load_ratio)), float(np.float32(high_cap)), _ptr(out),
           _stream())
    return out


@torch.library.custom_op('covgpu::compute_trans_sus', mutates_args=())
def _trans_sus_op(rel_trans: torch.Tensor, rel_sus: torch.Tensor, inf: torch.Tensor, sus: torch.Tensor,
                  beta_layer: float, viral_load: torch.Tensor, symp: torch.Tensor, iso: torch.Tensor,
                  quar: torch.Tensor, asymp_factor: float, iso_factor: float, quar_factor: float,
                  immunity_factors: torch.Tensor) -> tuple[torch.Tensor, torch.Tensor]:
    n = rel_trans.numel()
    a = torch.empty(n, dtype=_F32, device=rel_trans.device)
    b = torch.empty(n, dtype=_F32, device=rel_trans.device)
    f = lambda x: float(np.float32(x))  # noqa: E731 -- the numba signature's float32 cast
    L.call('covgpu_trans_sus', _ptr(rel_trans), _ptr(rel_sus), _ptr(inf), _ptr(sus), f(beta_layer), _ptr(viral_load),
           _ptr(symp), _ptr(iso), _ptr(quar), f(asymp_factor), f(iso_factor), f(quar_factor), _ptr(immunity_factors),
           n, _ptr(a), _ptr(b), _stream())
    return a, b


@torch.library.custom_op('covgpu::compute_infections', mutates_args=())
def _infections_op(beta: float, p1: torch.Tensor, p2: torch.Tensor, layer_betas: torch.Tensor,
                   rel_trans: torch.Tensor, rel_sus: torch.Tensor, uniforms: torch.Tensor, seed: int, day: int,
                   variant: int, layer: int) -> tuple[torch.Tensor, torch.Tensor]:
    E = p1.numel()
    dev = p1.device
    cap = 2 * E
    src = torch.empty(max(cap, 1), dtype=_I32, device=dev)
    tgt = torch.empty(max(cap, 1), dtype=_I32, device=dev)
    count = torch.zeros(1, dtype=torch.int64, device=dev)
    status = torch.zeros(1, dtype=_I32, device=dev)
    nbytes = int(L.lib().covgpu_infections_scratch_bytes(E))
    scratch = torch.empty(nbytes, dtype=_U8, device=dev)
    L.call('covgpu_infections', float(np.float32(beta)), _ptr(p1), _ptr(p2), _ptr(layer_betas), E, _ptr(rel_trans),
           _ptr(rel_sus), min(rel_trans.numel(), rel_sus.numel()), _ptr(uniforms), int(seed) & 0xFFFFFFFFFFFFFFFF, int(day), int(variant), int(layer),
           _ptr(src), _ptr(tgt), cap, _ptr(count), _ptr(status), scratch.data_ptr(), nbytes, _stream())
    n = int(count.item())
    if int(status.item()) & L.BADARG:
        raise IndexError('compute_infections: an edge index is outside the agent arrays')
    return src[:n].clone(), tgt[:n].clone()


# ---------------------------------------------------------------- reference-signature drop-ins
def compute_viral_load(t, time_start, time_recovered, time_dead, frac_time, load_ratio, high_cap):
    """utils.py:39-79."""
    as_np = not torch.is_tensor(time_start)
    out = torch.ops.covgpu.compute_viral_load(int(t), _dev(time_start, _F32), _dev(time_recovered, _F32),
                                              _dev(time_dead, _F32), float(frac_time), float(load_ratio),
                                              float(high_cap))
    return out.cpu().numpy() if as_np else out


def compute_trans_sus(rel_trans, rel_sus, inf, sus, beta_layer, viral_load, symp, iso, quar, asymp_factor,
                      iso_factor, quar_factor, immunity_factors):
    """utils.py:82-90."""
    as_np = not torch.is_tensor(rel_trans)
    b = lambda x: _dev(x, _U8) if not torch.is_tensor(x) else x.to('cuda').to(_U8).contiguous()  # noqa: E731
    a, c = torch.ops.covgpu.compute_trans_sus(_dev(rel_trans, _F32), _dev(rel_sus, _F32), b(inf), b(sus),
                                              float(beta_layer), _dev(viral_load, _F32), b(symp), b(iso), b(quar),
                                              float(asymp_factor), float(iso_factor), float(quar_factor),
                                              _dev(immunity_factors, _F32))
    return (a.cpu().numpy(), c.cpu().numpy()) if as_np else (a, c)


def compute_infections(beta, p1, p2, layer_betas, rel_trans, rel_sus, legacy=False, uniforms=None, seed=0, day=0,
                       variant=0, layer=0):
    """utils.py:93-128 (non-legacy). Returns (sources, targets): direction p1->p2
    in edge order, then p2->p1. ``uniforms`` ([2, E] float64 draws by direction
    and edge) replays given draws; otherwise Bernoullis come from Philox keyed
    by (seed, day, variant, layer, edge)."""
    if legacy:
        raise NotImplementedError('the legacy (pre-3.1.1) transmission path is not supported on the GPU')
    as_np = not torch.is_tensor(p1)
    uni = _dev(uniforms, _F64) if uniforms is not None else torch.empty(0, dtype=_F64, device='cuda')
    src, tgt = torch.ops.covgpu.compute_infections(float(beta), _dev(p1, _I32), _dev(p2, _I32), _dev(layer_betas, _F32),
                                                   _dev(rel_trans, _F32), _dev(rel_sus, _F32), uni, int(seed),
                                                   int(day), int(variant), int(layer))
    return (src.cpu().numpy(), tgt.cpu().numpy()) if as_np else (src, tgt)
