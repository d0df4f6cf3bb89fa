"""CPU oracle for the Covasim 3.1.7 per-day step hot path.

TEST INFRASTRUCTURE ONLY. Only ``tests/``, ``__graft_entry__.smoke()`` and the
CPU-baseline leg of ``bench.py`` import this package, and only as the checker
or the timed CPU baseline; the ``covasim_gb300`` product never imports it and
has no CPU fallback.

Contents (each function cites the reference file:line it restates):

* ``kernels``: compute_viral_load, compute_trans_sus, compute_infections
  (covasim/utils.py:39-128), float32-faithful under numba's typing rules;
* ``people``: agent arrays, update_states_pre and its checks, infect,
  update_peak_nab, update_nab, check_immunity, nab_growth_decay
  (covasim/people.py, covasim/immunity.py);
* ``sim``: the day loop (covasim/sim.py:558-685) in Philox mode (draws keyed
  like the CUDA library's) or MT19937 mode (reference call order);
* ``philox``: Philox-4x32-10 and the draw conversions shared with the GPU.

Parity pinning: the oracle is checked against golden vectors produced by
running the reference's own function bodies (loaded from the reference source
with small stand-ins for numba and sciris, which are not installed here) on
seeded inputs with recorded draws; see ``tests/golden/make_golden.py``.
"""
