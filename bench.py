"""Benchmark: agent-days/s of the per-day step on the 1M-agent hybrid 180-day sim.

Workload (one "step" = one full run of the sim): pop_size=1,000,000,
pop_type='hybrid' (layers h/s/w/c, c redrawn every day), pop_infected=100,
use_waning=True, n_days=180, float32. Synthetic population from the
package's generators (same distributions as the reference's). Inputs
(agents ~160 MB + edges ~62 MB) are larger than L2 (129 MB).

  value        device-resident throughput: the population is in HBM, each
               step rewinds the state (device copy) and runs 181 days as one
               CUDA-graph launch (the rewind is inside the timed region)
  e2e          the same metric through the public API: per step the pinned
               host population is uploaded by cv.Sim(...).initialize(), run,
               and the results copied back (finalize)
  roofline     the dominant kernel, from per-kernel CUDA-event timing of one
               extra ungraphed run; algorithmic bytes per launch: 28 B per
               undirected edge per day for the edge pass (p1, p2, beta streamed,
               rel_trans and rel_sus of both endpoints gathered), 76 + 12 nv B
               per agent per day for the agent pass
  cpu_baseline the CPU oracle (numpy restatement) on a bounded sample of the
               same workload: a few days of the 1M hybrid sim

python bench.py [--gpus N] [--steps K] [--warmup W] [--impl reference]
Under torchrun (N > 1) every rank runs its own replica (seed + rank); value
is the sum over ranks, timed as the max over ranks (weak scaling).
"""
import argparse
import json
import os
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

POP = 1_000_000
DAYS = 180
PEAKS = os.path.join(ROOT, 'MEASURED_PEAKS.json')
# From ncu captures of the 1M-agent workload (day 85, near the epidemic's peak;
# the launch list of a whole ungraphed run gives the kernels' shares): DRAM bytes
# (dram__bytes_read.sum + dram__bytes_write.sum) per launch and the share of
# cycles the schedulers issued (smsp__issue_active), per kernel.
# Cumulative infections of the default workload's run with seed 1 (1M agents, 180
# days). The runs are deterministic (Philox streams keyed by the seed; bit-identical
# to the oracle's, checked at this scale by the tests), so the bench asserts it.
RECORDED_CUM_INFECTIONS = {(1_000_000, 180, 1): 1_055_079}

MEASURED_NCU = {
    ('agent_step', 1_000_000): {
        'dram_bytes': 69_901_568, 'issue_active': 0.602, 'bound': 'issue',
        'note': 'ncu section capture, day 85 of the 1M-agent run: 69.9 MB of DRAM traffic against 88 MB '
                'algorithmic; instruction issue 60% busy, 35.0 M warp instructions for 1M agents, so the pass '
                'is issue-bound on the float-float efficacies, not HBM-bound'},
    ('edge_stored', 1_000_000): {
        'dram_bytes': 83_445_760, 'issue_active': 0.533, 'bound': 'latency',
        'note': 'ncu section capture, day 85 (one-wave pass, 2048-edge tiles): 83 MB of DRAM traffic (the 62 MB '
                'of stored edge lists and the candidates\' records); long-scoreboard stalls dominate'},
}


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument('--gpus', type=int, default=1)
    ap.add_argument('--steps', type=int, default=5)
    ap.add_argument('--warmup', type=int, default=3)
    ap.add_argument('--impl', default='gb300', choices=['gb300', 'reference'])
    ap.add_argument('--pop-size', type=int, default=POP)
    ap.add_argument('--days', type=int, default=DAYS)
    ap.add_argument('--no-cpu', action='store_true')
    ap.add_argument('--no-e2e', action='store_true')
    ap.add_argument('--batch', type=int, default=16, help='sims of the batched measurement (0: skip)')
    ap.add_argument('--no-adjoint', action='store_true', help='skip the forward/adjoint cost measurement')
    ap.add_argument('--no-large', action='store_true',
                    help='skip the 20M-agent, 365-day measurement (one run, device population) in the default line')
    ap.add_argument('--no-batch256', action='store_true',
                    help='skip the 256-sim batched measurement (batched vs one by one) in the default line')
    ap.add_argument('--edge-tile', default='auto',
                    help="edge-pass tile (1024/2048/4096/8192, suffix 'w' for the one-wave stored-layer pass, "
                         "'r' for the resident bitmap) or 'auto' (autotuner)")
    ap.add_argument('--src-walk', type=int, default=None,
                    help='walk of the stored layers from the day\'s sources: k walks while infectious x k < agents, '
                         '0 never, -1 always (default: the library\'s)')
    ap.add_argument('--seeds', type=int, default=1,
                    help='large workload: this many seeds of the 20M-agent sim in one BatchSim')
    ap.add_argument('--gpu-population', action='store_true',
                    help='large / batch256 workloads: build the populations on the device')
    ap.add_argument('--workload', default='hybrid1m', choices=['hybrid1m', 'large', 'batch256'],
                    help='hybrid1m: the headline run; large: 20M-agent hybrid, 3 variants, testing and tracing, '
                         '365 days; batch256: 256 random-population sims of 10k-500k agents, batched vs one by one')
    ap.add_argument('--json-out', default=None)
    ap.add_argument('--profile-run', action='store_true',
                    help='run one sim of --pop-size agents for --days days, one launch per kernel (no graph), '
                         'for profilers, and exit')
    ap.add_argument('--profile-testing', action='store_true',
                    help='profile run: with test_prob(symp_prob=0.1), contact_tracing(trace_probs=0.5) and the '
                         'likelihood passes, so that every per-day kernel runs')
    return ap.parse_args()


def sim_pars(args, seed):
    return dict(pop_size=args.pop_size, pop_type='hybrid', pop_infected=100, use_waning=True, n_days=args.days,
                rand_seed=seed, dynam_layer=dict(h=0, s=0, w=0, c=1))


# ----------------------------------------------------------------------------- distributed
def dist_setup():
    world = int(os.environ.get('WORLD_SIZE', '1'))
    rank = int(os.environ.get('RANK', '0'))
    local = int(os.environ.get('LOCAL_RANK', '0'))
    if world > 1:
        import torch
        import torch.distributed as dist
        backend = 'nccl' if torch.cuda.is_available() else 'gloo'
        if torch.cuda.is_available():
            torch.cuda.set_device(local)
        dist.init_process_group(backend=backend)
    return world, rank, local


def barrier(world):
    if world > 1:
        import torch.distributed as dist
        dist.barrier()


def max_over_ranks(x, world):
    if world == 1:
        return x
    import torch
    import torch.distributed as dist
    t = torch.tensor([x], dtype=torch.float64, device='cuda' if torch.cuda.is_available() else 'cpu')
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


# ----------------------------------------------------------------------------- clocks
class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled every 200 ms during the timed region."""
    Q = ('index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,'
         'clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,'
         'clocks_event_reasons.sw_power_cap')

    def __init__(self, gpu_index=0):
        self.gpu = gpu_index
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(['nvidia-smi', f'--id={self.gpu}', f'--query-gpu={self.Q}',
                                          '--format=csv,noheader,nounits', '-lms', '200'],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except FileNotFoundError:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if self.proc is None:
            return {'sm_mhz': None, 'sm_max_mhz': None, 'reasons': ['nvidia-smi unavailable']}
        time.sleep(0.25)
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        sm, smax, reasons = [], [], set()
        names = ['hw_slowdown', 'hw_thermal_slowdown', 'sw_thermal_slowdown', 'sw_power_cap']
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(',')]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                smax.append(float(parts[2]))
            except ValueError:
                continue
            for name, val in zip(names, parts[5:9]):
                if val.lower().startswith('active'):
                    reasons.add(name)
        return {'sm_mhz': float(np.median(sm)) if sm else None, 'sm_max_mhz': max(smax) if smax else None,
                'reasons': sorted(reasons), 'samples': len(sm)}


# ----------------------------------------------------------------------------- algorithmic bytes
# Algorithmic bytes per unit of work (the HBM roofline's numerator), the
# per-unit figures of the reference's own algorithm:
#   edge pass  28 B per undirected edge per day: p1, p2 and beta streamed
#              (12 B) plus rel_trans and rel_sus of both endpoints gathered
#              (16 B), over every layer including the redrawn one;
#   agent pass 76 + 12*nv B per agent per day: six date reads (24), two
#              end-of-isolation/quarantine dates (8), base rel_trans/rel_sus
#              (8), nab/peak_nab/t_nab_event (12), variant fields (4), flags
#              read+write (8), nab write (4), effective rel_trans/rel_sus
#              writes (8), and 3*nv immunity writes (12*nv).
EDGE_BYTES_PER_EDGE = 28
AGENT_BYTES_BASE, AGENT_BYTES_PER_VARIANT = 76, 12


def agent_pass_bytes(n, nv):
    return (AGENT_BYTES_BASE + AGENT_BYTES_PER_VARIANT * nv) * n


# ----------------------------------------------------------------------------- GPU arm
def kernel_profile(sim, npts, head_start_cycles=2_000_000):
    """One ungraphed run with CUDA events around each kernel (on the launching
    stream): the agent pass, the stored layers' edge pass, the dynamic layers'
    per-source pass and the infect pass, each launched on its own. Each day
    starts with a short spin of the stream (about 1 ms, outside the timed pairs)
    so that the host has queued the day's launches and events before the GPU
    reaches them: an event pair then times its kernel, not the host's launch
    latency."""
    import torch
    st = sim.state
    times = {'agent_step': [], 'edge_stored': [], 'edge_dynamic': [], 'infect_claims': []}
    stream = torch.cuda.current_stream()

    def timed(name, fn):
        a = torch.cuda.Event(enable_timing=True)
        b = torch.cuda.Event(enable_timing=True)
        a.record(stream)
        fn()
        b.record(stream)
        times[name].append((a, b))

    for t in range(npts):
        torch.cuda._sleep(head_start_cycles)
        timed('agent_step', lambda: st.agent_step(t, do_prev=t > 0, do_day=True, steady=t > 0))
        timed('edge_stored', lambda: st.edge_pass(t, parts=1))
        timed('edge_dynamic', lambda: st.edge_pass(t, parts=2))
        timed('infect_claims', lambda: st.infect_claims(t))
    torch.cuda._sleep(head_start_cycles)
    timed('agent_step', lambda: st.agent_step(npts, do_prev=True, do_day=False))
    torch.cuda.synchronize()
    return {k: [a.elapsed_time(b) for a, b in v] for k, v in times.items()}


KERNEL_NAMES = {'agent_step': 'k_agent_step', 'edge_stored': 'k_edge_pass', 'edge_dynamic': 'k_dyn_pass',
                'infect_claims': 'k_infect_claims'}


def roofline_block(dom, totals, kt, sim, n, st, res):
    """The roofline of the dominant kernel: algorithmic bytes per launch (the
    reference algorithm's per-unit bytes x the units of one launch) over its
    CUDA-event average duration, against the measured copy bandwidth; beside it
    the DRAM traffic ncu measured for that kernel and what bounds it."""
    nv = 1
    if dom == 'agent_step':
        bytes_launch = agent_pass_bytes(n, nv)
        unit_desc = f'{AGENT_BYTES_BASE + AGENT_BYTES_PER_VARIANT * nv} B/agent/day'
    elif dom == 'edge_stored':
        bytes_launch = EDGE_BYTES_PER_EDGE * sum(len(ly['p1']) for ly in sim.spec.layers if not ly['dynamic'])
        unit_desc = f'{EDGE_BYTES_PER_EDGE} B/stored undirected edge/day'
    elif dom == 'edge_dynamic':
        bytes_launch = EDGE_BYTES_PER_EDGE * sum(len(ly['p1']) for ly in sim.spec.layers if ly['dynamic'])
        unit_desc = (f'{EDGE_BYTES_PER_EDGE} B/redrawn undirected edge/day (the reference streams the whole '
                     'redrawn layer; this pass draws the sources\' lists only)')
    else:
        bytes_launch = 16.0 * max(float(np.mean(res['new_infections'])), 1.0)
        unit_desc = '16 B/new infection'
    avg_ms = totals[dom] / len(kt[dom])
    achieved = bytes_launch / (avg_ms / 1e3) / 1e9
    peak, peak_kind = peaks()
    m = MEASURED_NCU.get((dom, n), {})
    traffic = m.get('dram_bytes')
    out = {'bound': m.get('bound', 'hbm'), 'kernel': KERNEL_NAMES[dom], 'achieved': round(achieved, 1), 'peak': peak,
           'peak_source': peak_kind, 'unit': 'GB/s', 'frac': round(achieved / peak, 4), 'traffic': traffic,
           'algorithmic_bytes_per_launch': round(bytes_launch), 'bytes_per_unit': unit_desc,
           'avg_launch_ms': round(avg_ms, 5)}
    if traffic:
        out['dram_achieved'] = round(traffic / (avg_ms / 1e3) / 1e9, 1)
        out['dram_frac'] = round(traffic / (avg_ms / 1e3) / 1e9 / peak, 4)
        out['traffic_note'] = m.get('note')
    if 'issue_active' in m:
        out['issue_active'] = m['issue_active']
    out['kernel_ms_total'] = {KERNEL_NAMES[k]: round(v, 3) for k, v in totals.items()}
    out['kernel_share'] = {KERNEL_NAMES[k]: round(v / sum(totals.values()), 4) for k, v in totals.items()}
    return out


def peaks():
    try:
        with open(PEAKS) as f:
            p = json.load(f)
        return float(p['hbm_gbs']), 'measured'
    except Exception:
        return 6800.0, 'fallback'


def gpu_arm(args, world, rank):
    import torch
    import covasim_gb300 as cv
    from covasim_gb300.sim import choose_seed_infections, CALL_SEED
    from covasim_gb300 import _lib as L

    seed = 1 + rank
    sim = cv.Sim(sim_pars(args, seed))
    t0 = time.perf_counter()
    sim.initialize()
    init_s = time.perf_counter() - t0
    st = sim.state
    npts = sim.npts
    if args.src_walk is not None:
        st.set_src_walk(args.src_walk)
    tile_ms = None
    if args.edge_tile == 'auto':  # before the snapshot: tuning leaves the state rewound
        from covasim_gb300.autotune import tune_edge_tile
        _, tile_ms = tune_edge_tile(st)
    else:
        st.apply_edge_tile(args.edge_tile)
    snap = st.snapshot()
    seeds = choose_seed_infections(sim['rand_seed'], sim['pop_size'], sim['pop_infected'])

    def one_run():
        st.restore(snap)
        st.infect_list(0, seeds, sim=0, variant=0, layer_tag=L.LOG_SEED, call_tag=CALL_SEED)
        st.run_days(0, npts, open_prev=False, close_last=True, use_graph=True)

    for _ in range(args.warmup):
        one_run()
    torch.cuda.synchronize()
    if st.status():
        raise RuntimeError(f'device status {st.status()}')
    clocks = ClockSampler(torch.cuda.current_device())
    clocks.start()
    barrier(world)
    torch.cuda.synchronize()
    ev0 = torch.cuda.Event(enable_timing=True)
    ev1 = torch.cuda.Event(enable_timing=True)
    ev0.record()
    for _ in range(args.steps):
        one_run()
    ev1.record()
    torch.cuda.synchronize()
    barrier(world)
    elapsed = ev0.elapsed_time(ev1) / 1e3
    clk = clocks.stop()
    elapsed = max_over_ranks(elapsed, world)
    res = st.results(0)
    n = sim['pop_size']
    agent_days = n * args.days
    value = world * agent_days * args.steps / elapsed

    # per-kernel timing (one extra ungraphed run) for the roofline
    st.restore(snap)
    st.infect_list(0, seeds, sim=0, variant=0, layer_tag=L.LOG_SEED, call_tag=CALL_SEED)
    kt = kernel_profile(sim, npts)
    res = st.results(0)
    totals = {k: float(np.sum(v)) for k, v in kt.items()}
    dom = max(totals, key=totals.get)
    roofline = roofline_block(dom, totals, kt, sim, n, st, res)
    launches_per_step = 1 + 4 * npts + 1  # seed infect, per day agent/stored/dynamic/infect, closing pass

    # end to end through the public API, from pinned host memory
    e2e = None
    if not args.no_e2e:
        pop = sim.popdict
        pin = lambda a, dt: torch.from_numpy(np.ascontiguousarray(a, dtype=dt)).pin_memory()  # noqa: E731
        host_pop = {'uid': pop['uid'], 'age': pop['age'], 'sex': pop['sex'], 'contacts': {}}
        h2d = 0
        for k, c in pop['contacts'].items():
            host_pop['contacts'][k] = dict(p1=pin(c['p1'], np.int32), p2=pin(c['p2'], np.int32))
            h2d += 8 * len(c['p1']) if not sim['dynam_layer'].get(k) else 0
        host_person = {k: pin(v, np.float32) for k, v in sim._person.items()}
        h2d += sum(4 * len(v) for v in host_person.values())
        d2h = 0

        def e2e_step():
            s = cv.Sim(sim_pars(args, seed), popdict=host_pop, person=host_person, edge_tile=st.edge_tile_label)
            s.run()
            return s

        for _ in range(max(1, args.warmup)):
            e2e_step()
        torch.cuda.synchronize()
        barrier(world)
        t0 = time.perf_counter()
        for _ in range(args.steps):
            s = e2e_step()
        torch.cuda.synchronize()
        e2e_s = max_over_ranks(time.perf_counter() - t0, world)
        d2h = 8 * (L.N_RES_INT + L.N_RES_VAR + L.N_RES_F) * npts
        e2e = {'value': round(world * agent_days * args.steps / e2e_s, 1), 'unit': 'agent-days/s',
               'h2d_bytes_per_step': int(h2d), 'd2h_bytes_per_step': int(d2h),
               'ms_per_step': round(1e3 * e2e_s / args.steps, 3)}
        check_recorded(args, seed, float(s.results['cum_infections'].values[-1]))

    batched = batched_arm(args, sim, value, world) if args.batch else None
    adjoint = adjoint_arm(args) if not args.no_adjoint else None
    batch256 = None
    if not args.no_batch256 and world == 1:
        batch256 = batch_arm(args, steps=min(args.steps, 3), warmup=2, emit=False)
    large = None
    if not args.no_large and world == 1:
        large = large_arm(args, steps=1, warmup=1, gpu_population=True, emit=False)

    check_recorded(args, seed, float(res['new_infections'].sum() + sim['pop_infected']))
    return dict(value=value, elapsed=elapsed, clocks=clk, roofline=roofline, e2e=e2e, batched=batched, adjoint=adjoint,
                batch256=batch256, large=large,
                edge_tile=st.edge_tile_label, tile_ms=tile_ms, popdict=sim.popdict, person=sim._person,
                launches=launches_per_step * args.steps, init_s=init_s, res=res, spec=sim.spec,
                cum_infections=float(res['new_infections'].sum() + sim['pop_infected']))


def adjoint_arm(args, n=100_000, days=120, every=10, reps=3):
    """Forward and forward + adjoint cost on the differentiable workload: a
    100,000-agent hybrid sim, 120 days, change_beta on days 30 and 60, gradients
    with respect to beta, the 4 layer betas and the 2 multipliers, a state
    checkpoint every 10 days. The forward runs the sim with the likelihood
    passes and the gradient accumulators, so the adjoint at the forward's own
    parameters only combines them; the adjoint at other parameters (a
    fixed-states step) rewinds to each checkpoint and recomputes its days.
    Wall-clock with device synchronisation."""
    import torch
    import covasim_gb300 as cv
    from covasim_gb300.adjoint import LikelihoodRun
    pars = dict(pop_size=n, pop_type='hybrid', pop_infected=100, use_waning=True, n_days=days, rand_seed=1,
                dynam_layer=dict(h=0, s=0, w=0, c=1), interventions=[cv.change_beta(days=[30, 60], changes=[0.7, 0.9])])
    sim = cv.Sim(pars)
    sim.initialize()
    run = LikelihoodRun(sim, checkpoint_every=every)
    th = run.params.theta0
    g_exp = np.ones(run.npts)

    def timed(fn):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for _ in range(reps):
            fn()
        torch.cuda.synchronize()
        return (time.perf_counter() - t0) / reps

    def plain():
        st = run.state
        st.disable_lik()
        st.restore(run.initial)
        init_infections(st, 0, run.sim.pars)
        st.run_days(0, run.npts, open_prev=False, close_last=True, use_graph=True)
        torch.cuda.synchronize()

    from covasim_gb300.sim import init_infections
    for _ in range(2):  # warm-up: graph captures of every segment in both modes
        plain()
        run.forward(th)
        run.backward(1.0, g_exp)
    t_plain = timed(plain)
    t_fwd = timed(lambda: run.forward(th))
    t_both = timed(lambda: (run.forward(th), run.backward(1.0, g_exp)))
    th_other = th * 1.05
    t_other = timed(lambda: run.backward(1.0, g_exp, theta_eval=th_other))
    grad = run.backward(1.0, g_exp)
    return {'workload': f'hybrid {n} agents, {days} days, change_beta days 30/60, {len(th)} parameters, '
                        f'checkpoint every {every} days',
            'plain_ms': round(1e3 * t_plain, 3), 'forward_ms': round(1e3 * t_fwd, 3),
            'forward_adjoint_ms': round(1e3 * t_both, 3), 'adjoint_over_forward': round(t_both / t_fwd, 3),
            'forward_over_plain': round(t_fwd / t_plain, 3),
            'adjoint_other_theta_ms': round(1e3 * t_other, 3),
            'grad': {k: float(v) for k, v in zip(run.params.names, grad)}}


def batched_arm(args, sim, plain_value, world):
    """B copies of the workload (seeds differ, population shared) in one BatchState:
    one agent pass, one edge pass and one infect pass per day over all of them,
    the whole run one CUDA graph. Each batched sim is bit-identical to its solo
    run (tested), so outcome statistics match the plain path by construction;
    sim 0 is checked against the plain run here."""
    import torch
    import covasim_gb300 as cv
    from covasim_gb300.sim import choose_seed_infections, CALL_SEED
    from covasim_gb300 import _lib as L
    B = args.batch
    sims = [cv.Sim(sim_pars(args, 1 + k), popdict=sim.popdict, person=sim._person) for k in range(B)]
    batch = cv.BatchSim(sims, edge_tile=args.edge_tile).initialize()
    st = batch.state
    snap = st.snapshot()
    seeds = [choose_seed_infections(s['rand_seed'], s['pop_size'], s['pop_infected']) for s in sims]
    npts = batch.npts

    def one_run():
        st.restore(snap)
        for k in range(B):
            st.infect_list(0, seeds[k], sim=k, variant=0, layer_tag=L.LOG_SEED, call_tag=CALL_SEED)
        st.run_days(0, npts, open_prev=False, close_last=True, use_graph=True)

    for _ in range(args.warmup):
        one_run()
    torch.cuda.synchronize()
    barrier(world)
    ev0 = torch.cuda.Event(enable_timing=True)
    ev1 = torch.cuda.Event(enable_timing=True)
    ev0.record()
    for _ in range(args.steps):
        one_run()
    ev1.record()
    torch.cuda.synchronize()
    elapsed = max_over_ranks(ev0.elapsed_time(ev1) / 1e3, world)
    if st.status():
        raise RuntimeError(f'device status {st.status()}')
    value = world * B * args.pop_size * args.days * args.steps / elapsed
    solo = sim.state.results(0)['new_infections']
    same = bool(np.array_equal(st.results(0)['new_infections'], solo))
    cum = [float(st.results(k)['new_infections'].sum()) for k in range(B)]
    return {'value': round(value, 1), 'unit': 'agent-days/s', 'n_sims': B, 'edge_tile': st.edge_tile_label,
            'ms_per_step': round(1e3 * elapsed / args.steps, 3), 'vs_plain': round(value / plain_value, 3),
            'sim0_equals_plain_run': same, 'cum_infections_mean': round(float(np.mean(cum)), 1),
            'cum_infections_sd': round(float(np.std(cum)), 1)}


# ----------------------------------------------------------------------------- CPU oracle
def check_recorded(args, seed, cum):
    """The run's cumulative infections equal the recorded ones of its workload."""
    want = RECORDED_CUM_INFECTIONS.get((args.pop_size, args.days, seed))
    if want is not None and cum != want:
        raise AssertionError(f'cum_infections {cum} differs from the recorded {want} of this workload and seed')
    assert cum > 100


def workload_config(args):
    """The ``config`` both arms print: the workload alone (step and sampling details are top-level keys)."""
    return {'workload': f'hybrid {args.pop_size} agents (h/s/w/c, c redrawn daily), {args.days} days, waning, '
                        f'pop_infected 100'}


def host_cores():
    """The host cores this process may use (its affinity mask) and their count."""
    try:
        mask = sorted(os.sched_getaffinity(0))
    except AttributeError:
        mask = list(range(os.cpu_count() or 1))
    return mask, len(mask)


def _oracle_sim(pop_size, days, seed):
    """The workload on the CPU oracle in MT19937 mode: the reference's algorithm
    (the whole redrawn layer every day, every edge's draw) with the reference's
    streams; population and prognoses from the same generators as the GPU arm."""
    import covasim_gb300 as cv
    from oracle.sim import OracleSim, set_prognoses
    from oracle.people import OraclePeople
    pars = cv.make_pars(pop_size=pop_size, pop_type='hybrid', pop_infected=100, use_waning=True,
                        n_days=days, rand_seed=seed, dynam_layer=dict(h=0, s=0, w=0, c=1))
    pars['prognoses'] = cv.get_prognoses(True)
    cv.init_immunity(pars, days + 1)
    pop = cv.make_randpop(pars, rng=np.random.default_rng(seed))
    tmp = OraclePeople(pars, pop_size)
    tmp.age = np.asarray(pop['age'], np.float32)
    set_prognoses(tmp, pars, np.random.RandomState(seed))
    person = {k: tmp[k] for k in ('symp_prob', 'severe_prob', 'crit_prob', 'death_prob', 'rel_trans', 'rel_sus')}
    contacts = {k: dict(p1=c['p1'], p2=c['p2'], beta=np.ones(len(c['p1']), np.float32))
                for k, c in ((k, pop['contacts'][k]) for k in pars['beta_layer'])}
    return OracleSim(pars, person, contacts, rng='mt')


def _reference_worker(job):
    """One process of the reference arm: its own sim, ``warm`` untimed days on a
    copy, then the whole run (days 0..days) in ``k`` timed slices of consecutive
    days. Returns the slices' seconds and the run's cumulative infections."""
    import copy
    pop_size, days, seed, warm, k = job
    sys.path.insert(0, ROOT)
    sim = _oracle_sim(pop_size, days, seed)
    if warm:
        w = copy.deepcopy(sim)
        for _ in range(warm):
            w.step()
        del w
    bounds = np.linspace(0, days + 1, k + 1).round().astype(int)
    out = []
    for j in range(k):
        t0 = time.perf_counter()
        for _ in range(bounds[j], bounds[j + 1]):
            sim.step()
        out.append(time.perf_counter() - t0)
    return out, float(sim.results['new_infections'].sum()) + 100


def cpu_baseline(args, gpu_sim_factory, samples=5, days_each=2):
    """The CPU oracle (MT19937 mode, one process) on a bounded sample of the
    workload: ``samples`` stretches of ``days_each`` days spread evenly over the
    epidemic, each started from the GPU run's state of the evening before (the
    same trajectory), so early, peak and late days are all in the sample."""
    import covasim_gb300 as cv  # noqa: F401
    from oracle.people import (PERSON, STATES, VARIANT_STATES, BY_VARIANT_STATES, IMM_STATES, NAB_STATES,
                               VACC_STATES, DATES, DURS)
    keys = [k for k in PERSON + STATES + VARIANT_STATES + BY_VARIANT_STATES + IMM_STATES + NAB_STATES +
            VACC_STATES + DATES + DURS if k not in ('age', 'sex', 'uid', 'doses')]
    starts = np.linspace(args.days / (samples + 1), args.days * samples / (samples + 1), samples).round().astype(int)
    sim = gpu_sim_factory()
    orc = _oracle_sim(args.pop_size, args.days, 1)
    total, n_days = 0.0, 0
    for d in starts:
        sim.run(until=int(d))
        for k in keys:
            orc.people[k] = np.array(sim.people.gpu(k).cpu().numpy(), dtype=orc.people[k].dtype)
        orc.t = int(d)
        t0 = time.perf_counter()
        for _ in range(days_each):
            orc.step()
        total += time.perf_counter() - t0
        n_days += days_each
    mask, _ = host_cores()
    return {'value': round(args.pop_size * n_days / total, 1), 'unit': 'agent-days/s', 'cores': 1, 'kind': 'port',
            'sample': f'days {", ".join(f"{d}-{d + days_each - 1}" for d in starts)} of the {args.pop_size}-agent '
                      f'hybrid sim, each stretch started from the GPU run\'s state of the evening before; numpy '
                      f'oracle (the reference\'s algorithm restated) in MT19937 mode, one process, '
                      f'{total:.1f} s',
            'affinity': f'{len(mask)} cores available ({mask[0]}-{mask[-1]})'}


def reference_arm(args, world, rank):
    """The reference's CPU implementation of the path (its numpy restatement: the
    reference needs numba and sciris, which are not installed) on every host core
    the process may use: one independent sim per core (seeds differ), each running
    the whole 180-day epidemic. The K timed steps are K consecutive slices of that
    run, so every day of the epidemic is timed once; the W warm-up steps are W
    untimed days on a copy of each sim."""
    if rank != 0:
        return
    import multiprocessing as mp
    mask, n_cores = host_cores()
    procs = max(1, min(n_cores, 16))
    t0 = time.perf_counter()
    jobs = [(args.pop_size, args.days, 1 + i, args.warmup, args.steps) for i in range(procs)]
    with mp.get_context('spawn').Pool(procs) as pool:
        res = pool.map(_reference_worker, jobs)
    run_s = max(sum(r[0]) for r in res)
    value = procs * args.pop_size * args.days / run_s
    line = {'metric': 'agent-days/s', 'value': round(value, 1), 'unit': 'agent-days/s', 'impl': 'reference',
            'n_gpus': args.gpus, 'steps': args.steps, 'warmup': args.warmup,
            'ms_per_step': round(1e3 * run_s / args.steps, 3), 'higher_is_better': True, 'scaling': 'weak',
            'vs_baseline': None, 'dtype': 'f32', 'data': 'synthetic', 'config': workload_config(args),
            'step': f'1/{args.steps} of one whole run ({args.days + 1} days) on each of {procs} cores; the steps '
                    f'cover every day once',
            'cpu_baseline': {'value': round(value, 1), 'unit': 'agent-days/s', 'cores': procs, 'kind': 'port',
                             'sample': f'{procs} independent {args.pop_size}-agent hybrid sims (seeds 1-{procs}), '
                                       f'each its whole {args.days + 1}-day run (numpy oracle, MT19937 mode)',
                             'affinity': f'{len(mask)} cores available ({mask[0]}-{mask[-1]})'},
            'e2e': {'value': round(value, 1), 'unit': 'agent-days/s', 'h2d_bytes_per_step': 0,
                    'd2h_bytes_per_step': 0},
            'cum_infections_per_run': round(float(np.mean([r[1] for r in res])), 1),
            'wall_s': round(time.perf_counter() - t0, 1)}
    print(json.dumps(line), flush=True)


def _line(metric_value, unit, args, ms, workload, extra):
    line = {'metric': 'agent-days/s', 'value': round(metric_value, 1), 'unit': unit, 'n_gpus': 1,
            'steps': args.steps, 'warmup': args.warmup, 'ms_per_step': round(ms, 3), 'higher_is_better': True,
            'scaling': 'weak', 'vs_baseline': None, 'dtype': 'f32', 'data': 'synthetic',
            'config': {'workload': workload}}
    line.update(extra)
    print(json.dumps(line), flush=True)
    if args.json_out:
        with open(args.json_out, 'w') as f:
            json.dump(line, f, indent=1)


def large_arm(args, n=20_000_000, days=365, steps=None, warmup=None, gpu_population=None, emit=True):
    """20M-agent hybrid sim, 3 co-circulating variants (rel_beta 1.0 / 1.5 / 1.7,
    the second and third imported on days 60 and 120), waning, test_prob(symp_prob=0.1)
    and contact_tracing(trace_probs=0.5), 365 days. A step is one whole run: the
    state is rewound in HBM, the days between importations run as CUDA graphs and
    the two importation days as single steps."""
    import torch
    import covasim_gb300 as cv
    pars = dict(pop_size=n, pop_type='hybrid', pop_infected=200, use_waning=True, n_days=days, rand_seed=1,
                dynam_layer=dict(h=0, s=0, w=0, c=1),
                variants=[cv.variant(dict(rel_beta=1.5), days=60, n_imports=100, label='v1.5'),
                          cv.variant(dict(rel_beta=1.7), days=120, n_imports=100, label='v1.7')],
                interventions=[cv.test_prob(symp_prob=0.1), cv.contact_tracing(trace_probs=0.5)])
    t0 = time.perf_counter()
    tile = None if args.edge_tile == 'auto' else args.edge_tile
    seeds = max(1, args.seeds)
    gpu_population = args.gpu_population if gpu_population is None else gpu_population
    steps = args.steps if steps is None else steps
    warmup = args.warmup if warmup is None else warmup
    if seeds == 1:
        sim = cv.Sim(pars, edge_tile=tile, gpu_population=gpu_population)
        sim.initialize()
        st = sim.state
    else:  # the batched form: several seeds in one BatchSim
        sims = [cv.Sim(dict(pars, rand_seed=1 + k), gpu_population=gpu_population) for k in range(seeds)]
        batch = cv.BatchSim(sims, edge_tile=tile).initialize()
        sim, st = sims[0], batch.state
    if args.src_walk is not None:
        st.set_src_walk(args.src_walk)
    init_s = time.perf_counter() - t0
    snap = st.snapshot()

    def one_run():
        if seeds == 1:
            sim.rewind(snap)
            sim.run()
        else:
            st.restore(snap)
            batch.run()

    for _ in range(warmup):
        one_run()
    torch.cuda.synchronize()
    clocks = ClockSampler(torch.cuda.current_device())
    clocks.start()
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    ev0.record()
    for _ in range(steps):
        one_run()
    ev1.record()
    torch.cuda.synchronize()
    clk = clocks.stop()
    el = ev0.elapsed_time(ev1) / 1e3
    res = st.results(0)
    e_all = sum(len(ly['p1']) for ly in sim.spec.layers)
    workload = (f'{seeds} x ' * (seeds > 1) + f'hybrid {n} agents, {e_all} edges, 3 variants (days 0/60/120), '
                f'waning, test_prob(symp_prob=0.1), contact_tracing(trace_probs=0.5), {days} days')
    extra = {'edge_evaluations_per_s': round(seeds * 2 * e_all * days * steps / el, 1), 'init_s': round(init_s, 1),
             'seeds': seeds, 'population': 'device' if gpu_population else 'host',
             'cum_infections': float(res['new_infections'].sum() + sim['pop_infected']),
             'cum_tests': float(res['new_tests'].sum()), 'cum_quarantined': float(res['new_quarantined'].sum()),
             'clocks': clk}
    value = seeds * n * days * steps / el
    if emit:
        _line(value, 'agent-days/s', args, 1e3 * el / steps, workload, extra)
    return dict({'workload': workload, 'value': round(value, 1), 'unit': 'agent-days/s', 'steps': steps,
                 'warmup': warmup, 'ms_per_step': round(1e3 * el / steps, 3)}, **extra)


def batch_arm(args, n_sims=256, days=120, steps=None, warmup=None, emit=True):
    """256 random-population sims (pop_size log-uniform in [10k, 500k], contacts
    10/20/30, beta U[0.010, 0.025], change_beta(days=30, changes=U[0.3, 1])), 120
    days: all in one BatchSim (one launch sequence per day over every sim, one
    CUDA graph) against the same sims run one by one (one graph each). Each
    batched sim is bit-identical to its own run, so outcome statistics match
    exactly; value is the batched agent-days/s, with the one-by-one figure beside it."""
    import torch
    import covasim_gb300 as cv
    from covasim_gb300._lib import MAX_LAYERS
    from covasim_gb300.sim import CALL_SEED as CALL_SEED_TAG
    rng = np.random.default_rng(2024)
    sizes = np.exp(rng.uniform(np.log(10_000), np.log(500_000), n_sims)).astype(int)
    contacts = rng.choice([10, 20, 30], n_sims)
    betas = rng.uniform(0.010, 0.025, n_sims)
    changes = rng.uniform(0.3, 1.0, n_sims)

    def make(k):
        return cv.Sim(dict(pop_size=int(sizes[k]), pop_type='random', contacts=dict(a=int(contacts[k])),
                           beta=float(betas[k]), n_days=days, rand_seed=100 + k, pop_infected=20,
                           interventions=[cv.change_beta(days=30, changes=float(changes[k]))]),
                      gpu_population=args.gpu_population)
    t0 = time.perf_counter()
    sims = [make(k) for k in range(n_sims)]
    batch = cv.BatchSim(sims, edge_tile=args.edge_tile).initialize()
    init_s = time.perf_counter() - t0
    st = batch.state
    if args.src_walk is not None:
        st.set_src_walk(args.src_walk)
    snap = st.snapshot()
    seeds = [choose_seed(s) for s in sims]
    npts = days + 1

    def batched():
        st.restore(snap)
        for k, inds in enumerate(seeds):
            st.infect_list(0, inds, sim=k, variant=0, layer_tag=MAX_LAYERS, call_tag=CALL_SEED_TAG)
        st.run_days(0, npts, open_prev=False, close_last=True, use_graph=True)

    singles = []
    for k in range(n_sims):
        s = cv.Sim(dict(sims[k].pars), popdict=sims[k].popdict, person=sims[k]._person,
                   edge_tile=st.edge_tile_label)
        s.initialize()
        if args.src_walk is not None:
            s.state.set_src_walk(args.src_walk)
        singles.append((s, s.state.snapshot()))

    def one_by_one():
        for s, sn in singles:
            s.state.restore(sn)
            s.state.infect_list(0, choose_seed(s), sim=0, variant=0, layer_tag=MAX_LAYERS, call_tag=CALL_SEED_TAG)
            s.state.run_days(0, npts, open_prev=False, close_last=True, use_graph=True)

    steps = args.steps if steps is None else steps
    warmup = args.warmup if warmup is None else warmup

    def timed(fn):
        for _ in range(warmup):
            fn()
        torch.cuda.synchronize()
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record()
        for _ in range(steps):
            fn()
        b.record()
        torch.cuda.synchronize()
        return a.elapsed_time(b) / 1e3 / steps

    clocks = ClockSampler(torch.cuda.current_device())
    clocks.start()
    t_batch = timed(batched)
    t_single = timed(one_by_one)
    clk = clocks.stop()
    agent_days = float(sizes.sum()) * days
    same = all(np.array_equal(st.results(k)['new_infections'], singles[k][0].state.results(0)['new_infections'])
               for k in range(n_sims))
    workload = (f'{n_sims} random-population sims, {int(sizes.sum())} agents in all (10k-500k each), contacts '
                f'10/20/30, beta U[0.010,0.025], change_beta day 30 x U[0.3,1], {days} days')
    extra = {'one_by_one': {'value': round(agent_days / t_single, 1), 'ms_per_step': round(1e3 * t_single, 3)},
             'batched_over_one_by_one': round(t_single / t_batch, 3), 'every_sim_equals_its_own_run': same,
             'edge_tile': st.edge_tile_label, 'init_s': round(init_s, 1),
             'population': 'device' if args.gpu_population else 'host', 'clocks': clk}
    if emit:
        _line(agent_days / t_batch, 'agent-days/s', args, 1e3 * t_batch, workload, extra)
    return dict({'workload': workload, 'value': round(agent_days / t_batch, 1), 'unit': 'agent-days/s',
                 'steps': steps, 'warmup': warmup, 'ms_per_step': round(1e3 * t_batch, 3)}, **extra)


def choose_seed(sim):
    from covasim_gb300.sim import choose_seed_infections
    return choose_seed_infections(sim['rand_seed'], sim['pop_size'], sim['pop_infected'])


def profile_run(args):
    """One ungraphed run (kernels launched one by one) for ncu captures."""
    import torch
    import covasim_gb300 as cv
    pars = sim_pars(args, 1)
    if args.profile_testing:
        from covasim_gb300.adjoint import Parameters
        pars['interventions'] = [cv.test_prob(symp_prob=0.1), cv.contact_tracing(trace_probs=0.5)]
        sim = cv.Sim(pars, edge_tile=None if args.edge_tile == 'auto' else args.edge_tile)
        sim.initialize()
        st = sim.state
        st.enable_lik(grad=True)
        params = Parameters(sim)
        st.set_lik_factor(params.factor(params.theta0))
        st.zero_lik()
    else:
        sim = cv.Sim(pars, edge_tile=None if args.edge_tile == 'auto' else args.edge_tile)
        sim.initialize()
    if args.src_walk is not None:
        sim.state.set_src_walk(args.src_walk)
    sim.run(use_graph=False)
    torch.cuda.synchronize()
    print(json.dumps({'profile_run': True, 'pop_size': args.pop_size, 'days': args.days,
                      'testing': bool(args.profile_testing),
                      'cum_infections': float(sim.results['cum_infections'].values[-1])}))


def main():
    args = parse()
    if args.profile_run:
        profile_run(args)
        return
    world, rank, local = dist_setup()
    if args.impl == 'reference':
        reference_arm(args, world, rank)
        return
    if args.workload != 'hybrid1m':
        if rank == 0:
            (large_arm if args.workload == 'large' else batch_arm)(args)
        return
    out = gpu_arm(args, world, rank)
    cpu = None
    if rank == 0 and not args.no_cpu:
        import covasim_gb300 as cv
        cpu = cpu_baseline(args, lambda: cv.Sim(sim_pars(args, 1), popdict=out['popdict'], person=out['person'],
                                                 edge_tile=out['edge_tile']))
    if rank == 0:
        line = {'metric': 'agent-days/s', 'value': round(out['value'], 1), 'unit': 'agent-days/s',
                'n_gpus': world, 'steps': args.steps, 'warmup': args.warmup,
                'ms_per_step': round(1e3 * out['elapsed'] / args.steps, 3), 'higher_is_better': True,
                'scaling': 'weak', 'vs_baseline': None, 'dtype': 'f32', 'data': 'synthetic',
                'config': workload_config(args),
                'step': f'one full run: rewind the state in HBM, seed, {args.days + 1} days as one CUDA graph',
                'edge_tile': out['edge_tile'], 'edge_tile_autotune_ms_per_run': out['tile_ms'],
                'l2': 'inputs larger than L2 (agents ~160 MB + stored edges ~62 MB)',
                'replicas': world, 'cum_infections_per_run': out['cum_infections'],
                'edge_evaluations_per_s': None,
                'roofline': out['roofline'], 'cpu_baseline': cpu, 'e2e': out['e2e'], 'batched': out['batched'],
                'adjoint': out['adjoint'], 'batch256': out['batch256'], 'large': out['large'],
                'gpu_launches': out['launches'], 'clocks': out['clocks']}
        spec = out['spec']
        e_all = sum(len(ly['p1']) for ly in spec.layers)
        line['edge_evaluations_per_s'] = round(world * 2 * e_all * args.days * args.steps / out['elapsed'], 1)
        print(json.dumps(line), flush=True)
        if args.json_out:
            with open(args.json_out, 'w') as f:
                json.dump(line, f, indent=1)
    if world > 1:
        import torch.distributed as dist
        dist.destroy_process_group()


if __name__ == '__main__':
    main()
