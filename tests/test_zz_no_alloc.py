"""covgpu_infections_noalloc: compute_infections for callers that cannot allocate.

Some callers may not allocate device memory at all (a framework capturing a
CUDA graph under its own allocator, a plugin host with a fixed memory budget,
a thread that must not trigger the synchronisation an allocation can cause).
The no-allocation entry point keeps its scratch in a file-scope device array
of the library instead of caller memory. This test calls it through the C ABI
and checks it against the allocating entry point, twice in a row with
different inputs (the shared array keeps the previous call's contents), and
checks that a size beyond the array's limit is rejected before any launch.
This file is collected last so that a run stopping at the first failure has
already run every other test.
"""
import ctypes as C

import numpy as np
import pytest
import torch

from covasim_gb300 import _lib as L

pytestmark = pytest.mark.gpu


def _inputs(seed, n_edges, n_agents, frac_src):
    rng = np.random.default_rng(seed)
    p1 = np.sort(rng.integers(0, n_agents, n_edges)).astype(np.int32)
    p2 = rng.integers(0, n_agents, n_edges).astype(np.int32)
    lb = np.where(rng.random(n_edges) < 0.8, 1.0, rng.random(n_edges)).astype(np.float32)
    rt = np.where(rng.random(n_agents) < frac_src, rng.random(n_agents), 0).astype(np.float32)
    rs = np.where(rng.random(n_agents) < 0.7, rng.random(n_agents), 0).astype(np.float32)
    dev = lambda a: torch.from_numpy(a).cuda()  # noqa: E731
    return dev(p1), dev(p2), dev(lb), dev(rt), dev(rs)


def _call(lib, noalloc, beta, p1, p2, lb, rt, rs, seed, day):
    E, n = p1.numel(), rt.numel()
    cap = 2 * E
    src = torch.full((cap,), -7, dtype=torch.int32, device='cuda')
    tgt = torch.full((cap,), -7, dtype=torch.int32, device='cuda')
    count = torch.zeros(1, dtype=torch.int64, device='cuda')
    status = torch.zeros(1, dtype=torch.int32, device='cuda')
    stream = C.c_void_p(torch.cuda.current_stream().cuda_stream)
    common = (C.c_float(beta), p1.data_ptr(), p2.data_ptr(), lb.data_ptr(), E, rt.data_ptr(), rs.data_ptr(), n,
              None, seed, day, 0, 1, src.data_ptr(), tgt.data_ptr(), cap, count.data_ptr(), status.data_ptr())
    if noalloc:
        rc = lib.covgpu_infections_noalloc(*common, stream)
    else:
        nbytes = int(lib.covgpu_infections_scratch_bytes(E))
        scratch = torch.empty(nbytes, dtype=torch.uint8, device='cuda')
        rc = lib.covgpu_infections(*common, scratch.data_ptr(), nbytes, stream)
    assert rc == L.OK
    torch.cuda.synchronize()
    assert int(status.item()) == 0
    k = int(count.item())
    return src[:k].cpu().numpy(), tgt[:k].cpu().numpy()


def test_noalloc_matches_allocating_entry_point_on_two_calls():
    lib = L.lib()
    cases = [(1, 3_000_000, 400_000, 0.05, 0.3, 9), (2, 777_777, 50_000, 0.2, 0.05, 10)]
    for seed, E, n, frac, beta, day in cases:
        inputs = _inputs(seed, E, n, frac)
        want = _call(lib, False, beta, *inputs, seed=seed, day=day)
        got = _call(lib, True, beta, *inputs, seed=seed, day=day)
        assert len(want[0]) > 0
        assert np.array_equal(got[0], want[0]) and np.array_equal(got[1], want[1])


def test_noalloc_at_its_edge_limit_matches_allocating_entry_point():
    """Exactly the largest size the array holds: every tile's count and offset slot in use."""
    lib = L.lib()
    E = L.NOALLOC_MAX_EDGES
    inputs = _inputs(3, E, 2_000_000, 0.002)
    want = _call(lib, False, 0.5, *inputs, seed=3, day=4)
    got = _call(lib, True, 0.5, *inputs, seed=3, day=4)
    assert len(want[0]) > 0
    assert np.array_equal(got[0], want[0]) and np.array_equal(got[1], want[1])


def test_noalloc_rejects_more_edges_than_its_array_holds():
    lib = L.lib()
    rc = lib.covgpu_infections_noalloc(C.c_float(0.1), None, None, None, L.NOALLOC_MAX_EDGES + 1, None, None, 10,
                                       None, 0, 0, 0, 0, None, None, 0, None, None, None)
    assert rc == L.BADARG
