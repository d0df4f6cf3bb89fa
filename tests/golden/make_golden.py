"""Generate the golden fixtures from Covasim 3.1.7's own code.

Run from the repository root, where the reference source tree is available:

    python tests/golden/make_golden.py --reference PATH            # all fixtures
    python tests/golden/make_golden.py --reference PATH --only day # one group

(PATH is the reference source tree, the directory holding covasim/; the
COVASIM_REFERENCE environment variable may stand in for --reference.)

It executes the reference's function bodies through ``refload`` (see its
docstring), records every random draw they make, and writes small compressed
fixtures next to this script. Tests replay the recorded draws, so the oracle
and the CUDA kernels are checked against the reference's own outputs for the
reference's own draws. Nothing at test time reads the reference tree.

Fixtures:
  ref_pars.json        make_pars() + prognoses + nab_kin + immunity (random and hybrid)
  ref_kernels.npz      compute_viral_load / compute_trans_sus / compute_infections cases
  ref_day_<name>.npz   one day of the hot path on a mid-epidemic state: states before and
                       after update_states_pre (with check_immunity), viral load, per
                       (variant, layer) trans/sus, infections and infect() results with the
                       draws mapped to per-edge / per-agent slots, and update_nab
  ref_sims.npz         whole reference runs (inputs and daily results) for MT-mode replay
  ref_testing.npz      whole reference runs with test_prob + contact_tracing (inputs,
                       intervention arguments, daily results, final testing/quarantine state)
  ref_reporting.npz    compute_yield / compute_doubling / compute_r_eff / compute_gen_time
                       inputs and outputs on a reference run (sciris' smooth restated)
  ref_analysis.npz     TransTree / Fit / compute_gof outputs of the reference's own code on a
                       reference run with testing (pandas and sciris replaced by stand-ins)
  state_diagram.json   the state-implication matrices of tests/state_diagram.xlsx
  ref_distribution.npz daily new infections / severe / deaths of 200 seeds of the default
                       20k-agent random sim (60 days), reference code with MT19937 streams
  ref_distribution_hybrid.npz  the same for 200 seeds of a 30k-agent hybrid sim with waning
                       immunity and the community layer redrawn daily (150 days)
"""
import argparse
import copy
import json
import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, HERE)
sys.path.insert(0, ROOT)

import refload  # noqa: E402
from oracle import philox as ph  # noqa: E402
from oracle.kernels import compute_infections as o_compute_infections  # noqa: E402
from oracle.people import OraclePeople, TableDraws, dist_consumes_draws  # noqa: E402
from oracle.people import STATES, PERSON, VARIANT_STATES, BY_VARIANT_STATES, IMM_STATES  # noqa: E402
from oracle.people import NAB_STATES, VACC_STATES, DATES, DURS  # noqa: E402

ALL_KEYS = PERSON + STATES + VARIANT_STATES + BY_VARIANT_STATES + IMM_STATES + NAB_STATES + VACC_STATES + DATES + DURS


def jsonable(x):
    if isinstance(x, dict):
        return {str(k): jsonable(v) for k, v in x.items()}
    if isinstance(x, (list, tuple)):
        return [jsonable(v) for v in x]
    if isinstance(x, np.ndarray):
        return {'__array__': x.tolist(), 'dtype': str(x.dtype)}
    if isinstance(x, (np.floating,)):
        return float(x)
    if isinstance(x, (np.integer,)):
        return int(x)
    if callable(x):
        return None
    return x


def snapshot(people, prefix):
    return {f'{prefix}.{k}': np.array(people[k], copy=True) for k in ALL_KEYS}


# ------------------------------------------------------------------------- draw mapping
class LogDraws:
    """Replays a recorded numpy-stream log through oracle.infect and fills a per-agent table."""

    def __init__(self, log):
        self.log = list(log)
        self.table = {}

    def begin(self, inds):
        self.inds = np.asarray(inds)
        for a in self.inds:
            self.table.setdefault(int(a), np.full(ph.N_DRAWS, np.nan))

    def _pop(self, kind, n):
        k, vals, info = self.log.pop(0)
        assert k == kind and len(vals) == n, (k, kind, len(vals), n)
        return vals, info

    def normal(self, slot, inds, dist):
        from oracle.people import sample_from_normal
        if not dist_consumes_draws(dist):
            return sample_from_normal(dist, np.zeros(len(inds)))
        z, _ = self._pop('normal', len(inds))
        for a, v in zip(inds, z):
            self.table[int(a)][slot] = v
        return sample_from_normal(dist, z)

    def uniform(self, slot, inds):
        u, _ = self._pop('uniform', len(inds))
        for a, v in zip(inds, u):
            self.table[int(a)][slot] = v
        return u

    def as_arrays(self):
        keys = np.array(sorted(self.table), dtype=np.int64)
        tab = np.array([self.table[k] for k in keys]).reshape(len(keys), ph.N_DRAWS)
        return keys, tab


def map_edge_uniforms(log, beta, p1, p2, layer_betas, rel_trans, rel_sus):
    """Slot table [2, E] of the reference's compute_infections draws (2.0 = not drawn)."""
    U = np.full((2, len(p1)), 2.0)
    log = list(log)

    def uni(d, edge_inds):
        k, vals, _ = log.pop(0)
        assert k == 'uniform' and len(vals) == len(edge_inds)
        U[d, edge_inds] = vals
        return vals
    src, tgt = o_compute_infections(beta, p1, p2, layer_betas, rel_trans, rel_sus, uni)
    assert not log
    return U, src, tgt


# ------------------------------------------------------------------------- fixtures
class _SimPars(dict):
    """What init_immunity needs of a sim: item access to the pars and ``npts``."""

    def __init__(self, pars, npts):
        super().__init__(pars)
        self.npts = npts


def make_pars_fixture(ref):
    out = {}
    for pop_type in ('random', 'hybrid'):
        pars = ref.make_pars(pop_type=pop_type)
        s = _SimPars(pars, int(pars['n_days']) + 1)
        ref.cvi.init_immunity(s)
        pars['nab_kin'] = s['nab_kin']
        pars['immunity'] = s['immunity']
        out[pop_type] = jsonable(pars)
    pars = ref.make_pars(pop_type='hybrid')
    pars['variant_map'] = {0: 'wild', 1: 'alpha', 2: 'delta'}
    pars['variant_pars'] = {k: ref.cvpar.get_variant_pars(variant=k) for k in ('wild', 'alpha', 'delta')}
    pars['n_variants'] = 3
    s = _SimPars(pars, 61)
    ref.cvi.init_immunity(s, create=True)
    out['immunity_3var'] = jsonable(s['immunity'])
    with open(os.path.join(HERE, 'ref_pars.json'), 'w') as f:
        json.dump(out, f)
    print('ref_pars.json written')


def make_kernels_fixture(ref):
    rng = np.random.default_rng(20240611)
    out = {}
    # --- compute_viral_load: NaN starts, dead vs recovered, capped/uncapped, zero-length, ties
    n = 4096
    ts = rng.integers(0, 40, n).astype(np.float32)
    rec = ts + rng.integers(0, 30, n).astype(np.float32)
    dead = np.where(rng.random(n) < 0.2, ts + rng.integers(0, 25, n), np.nan).astype(np.float32)
    ts[rng.random(n) < 0.1] = np.nan
    rec[rng.random(n) < 0.1] = np.nan
    vl_cases = []
    for i, (t, fr, lr, hc) in enumerate([(20, 0.3, 2.0, 4.0), (5, 0.3, 2.0, 4.0), (33, 0.5, 3.0, 2.0),
                                         (0, 0.3, 2.0, 100.0)]):
        vl = ref.cvu.compute_viral_load(t, ts, rec, dead, fr, lr, hc)
        out[f'vl{i}.out'] = vl
        vl_cases.append([t, fr, lr, hc])
    out['vl.ts'], out['vl.rec'], out['vl.dead'] = ts, rec, dead
    out['vl.cases'] = np.array(vl_cases, dtype=np.float64)

    # --- compute_trans_sus
    rt = (rng.random(n) * 2).astype(np.float32)
    rt[rng.random(n) < 0.1] = 0
    rs = rng.choice([0.34, 0.67, 1.0, 1.24, 1.47], n).astype(np.float32)
    inf, sus, symp, iso, quar = (rng.random((5, n)) < np.array([[0.3], [0.6], [0.5], [0.2], [0.2]]))
    vl = ref.cvu.compute_viral_load(20, ts, rec, dead, 0.3, 2.0, 4.0)
    imm = np.where(rng.random(n) < 0.3, rng.random(n), 0).astype(np.float32)
    ts_cases = [(3.0, 1.0, 0.3, 0.6), (0.3, 0.8, 0.1, 0.2), (1.0, 0.0, 0.0, 1.0)]
    for i, (bl, af, isf, qf) in enumerate(ts_cases):
        a, b = ref.cvu.compute_trans_sus(rt, rs, inf, sus, bl, vl, symp, iso, quar, af, isf, qf, imm)
        out[f'ts{i}.rel_trans'], out[f'ts{i}.rel_sus'] = a, b
    for k, v in dict(rt=rt, rs=rs, inf=inf, sus=sus, symp=symp, iso=iso, quar=quar, vl=vl, imm=imm).items():
        out[f'ts.{k}'] = v
    out['ts.cases'] = np.array(ts_cases, dtype=np.float64)

    # --- compute_infections: sparse sources, self-loops, duplicate targets, p > 1, empty layer
    n_agents = 3000
    inf_cases = []
    for i, (E, beta, frac_src, big) in enumerate([(20000, 0.016, 0.05, False), (15000, 0.3, 0.2, False),
                                                 (5000, 50.0, 0.1, True), (0, 0.016, 0.1, False),
                                                 (40000, 0.05, 0.5, False)]):
        p1 = np.sort(rng.integers(0, n_agents, E)).astype(np.int32)
        p2 = rng.integers(0, n_agents, E).astype(np.int32)
        if E:
            p2[:10] = p1[:10]  # self-loops
        lb = np.where(rng.random(E) < 0.5, 1.0, rng.random(E) * 2).astype(np.float32)
        rtr = np.where(rng.random(n_agents) < frac_src, rng.random(n_agents), 0).astype(np.float32)
        rsu = np.where(rng.random(n_agents) < 0.7, rng.random(n_agents) * 1.5, 0).astype(np.float32)
        if big:
            rtr *= 10
        ref.cvu.set_seed(100 + i)
        ref.draws()
        src, tgt = ref.cvu.compute_infections(beta, p1, p2, lb, rtr, rsu)
        nb_log, _ = ref.draws()
        U, osrc, otgt = map_edge_uniforms(nb_log, np.float32(beta), p1, p2, lb, rtr, rsu)
        assert np.array_equal(src, osrc) and np.array_equal(tgt, otgt)
        for k, v in dict(p1=p1, p2=p2, lb=lb, rt=rtr, rs=rsu, U=U, src=src, tgt=tgt).items():
            out[f'inf{i}.{k}'] = v
        inf_cases.append(beta)
    out['inf.betas'] = np.array(inf_cases, dtype=np.float64)
    np.savez_compressed(os.path.join(HERE, 'ref_kernels.npz'), **out)
    print('ref_kernels.npz written')


def ref_sim_with_variants(ref, n, seed, days_before, nv=1, pop_type='hybrid', n_beds=None):
    pars = ref.make_pars(pop_size=n, n_days=days_before + 5, pop_type=pop_type, rand_seed=seed)
    if nv > 1:
        labels = ['wild', 'alpha', 'delta'][:nv]
        pars['variant_map'] = {i: k for i, k in enumerate(labels)}
        pars['variant_pars'] = {k: ref.cvpar.get_variant_pars(variant=k) for k in labels}
        pars['n_variants'] = nv
        pars['immunity'] = None
    if n_beds is not None:
        pars['n_beds_hosp'], pars['n_beds_icu'] = n_beds
    sim = refload.RefSim(ref, pars)
    if nv > 1:
        sim.pars['immunity'] = None
        ref.cvi.init_immunity(sim, create=True)
    rs = np.random.RandomState(seed + 1000)
    while sim.t < days_before:
        if nv > 1 and sim.t in (6, 12):  # import later variants, as variant.apply would
            v = 1 if sim.t == 6 else min(2, nv - 1)
            sus = sim.people.susceptible.nonzero()[0]
            imp = rs.choice(sus, min(15, len(sus)), replace=False)
            sim.people.infect(inds=imp, layer='importation', variant=v)
        sim.step()
    return sim


def run_day(ref, sim, out, prefix):
    """One day of the hot path on a copy of sim.people, with every output recorded."""
    people = copy.deepcopy(sim.people)
    people.pars = sim.pars
    t = sim.t
    p = sim.pars
    out.update(snapshot(people, f'{prefix}.S0'))
    ref.draws()
    people.update_states_pre(t=t)
    out.update(snapshot(people, f'{prefix}.S1'))
    for k, v in people.flows.items():
        out[f'{prefix}.flows.{k}'] = np.array(v)
    for k, v in people.flows_variant.items():
        out[f'{prefix}.flows_variant.{k}'] = np.array(v)
    hosp_max = people.count('severe') > p['n_beds_hosp'] if p['n_beds_hosp'] is not None else False
    icu_max = people.count('critical') > p['n_beds_icu'] if p['n_beds_icu'] is not None else False
    out[f'{prefix}.hosp_icu'] = np.array([hosp_max, icu_max])
    vd = p['viral_dist']
    vl = ref.cvu.compute_viral_load(t, people.date_infectious, people.date_recovered, people.date_dead,
                                    np.float32(vd['frac_time']), np.float32(vd['load_ratio']),
                                    np.float32(vd['high_cap']))
    out[f'{prefix}.viral_load'] = vl
    nv = p['n_variants']
    layers = list(people.contacts.keys())
    out[f'{prefix}.layer_keys'] = np.array(layers)
    for li, lkey in enumerate(layers):
        L = people.contacts[lkey]
        out[f'{prefix}.L{li}.p1'], out[f'{prefix}.L{li}.p2'], out[f'{prefix}.L{li}.beta'] = L['p1'], L['p2'], L['beta']
    for v in range(nv):
        label = p['variant_map'][v]
        beta = np.float32(p['beta'] * p['rel_beta'] * p['variant_pars'][label]['rel_beta'])
        inf_variant = people.infectious * (people.infectious_variant == v)
        out[f'{prefix}.v{v}.beta'] = np.array(beta)
        for li, lkey in enumerate(layers):
            L = people.contacts[lkey]
            rt, rs = ref.cvu.compute_trans_sus(people.rel_trans, people.rel_sus, inf_variant, people.susceptible,
                                               np.float32(p['beta_layer'][lkey]), vl, people.symptomatic,
                                               people.isolated, people.quarantined, p['asymp_factor'],
                                               np.float32(p['iso_factor'][lkey]), np.float32(p['quar_factor'][lkey]),
                                               people.sus_imm[v, :])
            key = f'{prefix}.v{v}.L{li}'
            out[f'{key}.rel_trans'], out[f'{key}.rel_sus'] = rt, rs
            ref.draws()
            src, tgt = ref.cvu.compute_infections(beta, L['p1'], L['p2'], L['beta'], rt, rs)
            nb_log, _ = ref.draws()
            U, osrc, otgt = map_edge_uniforms(nb_log, beta, L['p1'], L['p2'], L['beta'], rt, rs)
            assert np.array_equal(src, osrc) and np.array_equal(tgt, otgt)
            out[f'{key}.U'], out[f'{key}.src'], out[f'{key}.tgt'] = U, src, tgt
            inds = people.infect(inds=tgt, hosp_max=hosp_max, icu_max=icu_max, source=src, layer=lkey, variant=v)
            _, np_log = ref.draws()
            out[f'{key}.infected'] = np.asarray(inds)
            out[f'{key}.n_draw_log'] = np.array(len(np_log))
            out[f'{key}.np_log'] = np.concatenate([e[1].ravel() for e in np_log]) if np_log else np.zeros(0)
            out[f'{key}.np_log_lens'] = np.array([len(e[1]) for e in np_log], dtype=np.int64)
            out[f'{key}.np_log_kinds'] = np.array([e[0] == 'normal' for e in np_log], dtype=bool)
            out.update(snapshot(people, f'{key}.after'))
    out.update(snapshot(people, f'{prefix}.S2'))
    if p['use_waning']:
        has_nabs = people.peak_nab.nonzero()[0]
        if len(has_nabs):
            ref.cvi.update_nab(people, inds=has_nabs)
    out.update(snapshot(people, f'{prefix}.S3'))
    return people


def map_infect_tables(out, prefix, pars):
    """Turn each (variant, layer)'s recorded infect log into a per-agent draw table."""
    from oracle.people import OraclePeople as OP
    nv = pars['n_variants']
    n = len(out[f'{prefix}.S0.uid'])
    people = OP(pars, n)
    for k in ALL_KEYS:
        people[k] = np.array(out[f'{prefix}.S1.{k}'], copy=True)
    people.t = int(out[f'{prefix}.t'])
    nlayers = len([k for k in out if k.startswith(f'{prefix}.L') and k.endswith('.p1')])
    hosp_max, icu_max = out[f'{prefix}.hosp_icu']
    for v in range(nv):
        for li in range(nlayers):
            key = f'{prefix}.v{v}.L{li}'
            flat, lens, kinds = out[f'{key}.np_log'], out[f'{key}.np_log_lens'], out[f'{key}.np_log_kinds']
            log, pos = [], 0
            for ln, isn in zip(lens, kinds):
                log.append(('normal' if isn else 'uniform', flat[pos:pos + ln], {}))
                pos += ln
            ld = LogDraws(log)
            people.infect(inds=out[f'{key}.tgt'], hosp_max=hosp_max, icu_max=icu_max, source=out[f'{key}.src'],
                          layer=str(li), variant=v, draws=ld)
            assert not ld.log, 'unconsumed draws'
            agents, tab = ld.as_arrays()
            out[f'{key}.draw_agents'], out[f'{key}.draw_table'] = agents, tab
            for k in ALL_KEYS:
                a, b = people[k], out[f'{key}.after.{k}']
                assert np.array_equal(a, b, equal_nan=True), (key, k)
            del out[f'{key}.np_log'], out[f'{key}.np_log_lens'], out[f'{key}.np_log_kinds'], out[f'{key}.n_draw_log']


def make_day_fixtures(ref):
    cases = [
        # name, n, seed, day, variants, pop_type, beds
        ('hybrid', 2000, 11, 24, 1, 'hybrid', None),
        ('variants', 2000, 12, 30, 3, 'hybrid', (2, 1)),
        ('random', 1500, 13, 35, 1, 'random', None),
    ]
    for name, n, seed, day, nv, pop_type, beds in cases:
        sim = ref_sim_with_variants(ref, n, seed, day, nv=nv, pop_type=pop_type, n_beds=beds)
        out = {}
        prefix = 'd'
        out[f'{prefix}.t'] = np.array(sim.t)
        run_day(ref, sim, out, prefix)
        map_infect_tables(out, prefix, sim.pars)
        out['pars'] = np.array(json.dumps(jsonable(sim.pars)))
        # drop redundant per-layer 'after' snapshots except the last (keeps the fixture small)
        for k in [k for k in out if '.after.' in k]:
            del out[k]
        np.savez_compressed(os.path.join(HERE, f'ref_day_{name}.npz'), **out)
        print(f'ref_day_{name}.npz written', sum(v.nbytes for v in out.values()) // 1024, 'KiB raw')


def make_sims_fixture(ref):
    out = {}
    # (pop_type, n, days, seed, dynamic c, extra pars); cases 3 and 4 import agents every
    # day (sim.py:582-587), one at a rate that float32 does not hold exactly; cases 5
    # and 6 start with part of the population non-naive (sim.py:519-522)
    cases = [('random', 1500, 40, 3, 0, {}), ('hybrid', 1500, 50, 4, 0, {}), ('hybrid', 1200, 45, 9, 1, {}),
             ('hybrid', 1500, 45, 12, 1, dict(n_imports=0.7)), ('random', 1200, 40, 13, 0, dict(n_imports=3)),
             ('hybrid', 1500, 45, 14, 0, dict(frac_susceptible=0.55)),
             ('random', 1300, 40, 15, 0, dict(frac_susceptible=0.8, n_imports=1.5, pop_infected=40)),
             # dynamic rescaling (sim.py:535-556), with importations scaled by it, and a fixed scale
             ('hybrid', 2000, 60, 16, 0, dict(pop_scale=10, pop_infected=20)),
             ('random', 1500, 50, 17, 0, dict(pop_scale=4, n_imports=2, rescale_factor=1.5, rescale_threshold=0.1)),
             ('random', 1200, 40, 18, 0, dict(pop_scale=3, rescale=False, n_imports=3))]
    for i, (pop_type, n, days, seed, dyn, extra) in enumerate(cases):
        pars = ref.make_pars(pop_size=n, n_days=days, pop_type=pop_type, rand_seed=seed, **extra)
        if dyn:
            pars['dynam_layer']['c'] = 1
        sim = refload.RefSim(ref, pars)
        for k in ('age', 'sex', 'symp_prob', 'severe_prob', 'crit_prob', 'death_prob', 'rel_trans', 'rel_sus'):
            out[f's{i}.person.{k}'] = sim.people[k].copy()
        layers = list(sim.people.contacts.keys())
        for li, lk in enumerate(layers):
            for c in ('p1', 'p2', 'beta'):
                out[f's{i}.L{li}.{c}'] = sim.people.contacts[lk][c].copy()
        out[f's{i}.pars'] = np.array(json.dumps(jsonable(sim.pars)))
        sim.run()
        for k, v in sim.results.items():
            if k == 'variant':
                for kk, vv in v.items():
                    out[f's{i}.res.{kk}'] = vv
            else:
                out[f's{i}.res.{k}'] = v
        for k in ('exposed', 'recovered', 'dead', 'susceptible', 'date_recovered', 'peak_nab', 'nab'):
            out[f's{i}.final.{k}'] = sim.people[k].copy()
        out[f's{i}.rescale_vec'] = sim.rescale_vec.copy()
    out['n'] = np.array(len(cases))
    np.savez_compressed(os.path.join(HERE, 'ref_sims.npz'), **out)
    print('ref_sims.npz written')


TESTING_CASES = [  # (pop_type, n, days, seed, use_waning, dynamic c, test_prob kwargs, contact_tracing kwargs)
    ('hybrid', 1500, 40, 3, True, 0, dict(symp_prob=0.2, asymp_prob=0.01), dict(trace_probs=0.5, trace_time=1)),
    ('hybrid', 1500, 40, 4, True, 1,
     dict(symp_prob=0.3, asymp_prob=0.02, symp_quar_prob=0.5, asymp_quar_prob=0.1, quar_policy='both',
          sensitivity=0.9, loss_prob=0.1, test_delay=2),
     dict(trace_probs={'h': 1.0, 's': 0.5, 'w': 0.5, 'c': 0.2}, trace_time={'h': 0, 's': 1, 'w': 2, 'c': 3})),
    ('random', 1200, 40, 5, True, 0, dict(symp_prob=0.3, quar_policy='daily', start_day=5, end_day=30),
     dict(trace_probs=0.8, presumptive=True, start_day=8)),
    ('hybrid', 1200, 40, 6, False, 0, dict(symp_prob=0.3, quar_policy=[0, 2]),
     dict(trace_probs=0.7, trace_time=0.5, quar_period=10)),
    # influenza-like illness and fixed subtargets
    ('hybrid', 1500, 40, 7, True, 1,
     dict(symp_prob=0.2, asymp_prob=0.005, quar_policy='both', ili_prev=0.02,
          subtarget=dict(inds=list(range(0, 1500, 7)), vals=0.3)),
     dict(trace_probs=0.5, trace_time=1)),
    ('random', 1200, 40, 8, False, 0,
     dict(symp_prob=0.3, start_day=3, ili_prev=[0.01] * 8 + [0.05] * 12,
          subtarget=dict(inds=list(range(3, 1200, 11)), vals=[0.05 + 0.9 * (k % 3) / 2 for k in range(109)])),
     dict(trace_probs=0.6)),
    # a distribution of delays from symptom onset to swab
    ('hybrid', 1500, 40, 9, True, 0,
     dict(symp_prob=0.25, asymp_prob=0.01, swab_delay=dict(dist='lognormal', par1=3, par2=4)),
     dict(trace_probs=0.5, trace_time=1)),
    ('random', 1200, 40, 10, False, 0,
     dict(symp_prob=0.4, quar_policy='daily', swab_delay=dict(dist='uniform', par1=0, par2=5), ili_prev=0.01),
     dict(trace_probs=0.7)),
    # a tracing capacity below the day's cases
    ('hybrid', 1500, 40, 11, True, 0, dict(symp_prob=0.4, asymp_prob=0.02), dict(trace_probs=0.8, capacity=3)),
    ('random', 1200, 40, 12, False, 0, dict(symp_prob=0.5, test_delay=1),
     dict(trace_probs=0.9, presumptive=True, capacity=2)),
]
TESTING_FINAL = ['diagnosed', 'quarantined', 'isolated', 'known_contact', 'tested', 'date_diagnosed',
                 'date_quarantined', 'date_end_quarantine', 'date_known_contact', 'date_pos_test', 'date_tested',
                 'date_end_isolation', 'exposed', 'recovered', 'dead']


def make_testing_fixture(ref):
    """Whole runs with the reference's own test_prob and contact_tracing."""
    out = {}
    for i, (pop_type, n, days, seed, waning, dyn, tp_kw, ct_kw) in enumerate(TESTING_CASES):
        pars = ref.make_pars(pop_size=n, n_days=days, pop_type=pop_type, rand_seed=seed, use_waning=waning)
        if dyn:
            pars['dynam_layer']['c'] = 1
        pars['interventions'] = [ref.cvint.test_prob(**tp_kw), ref.cvint.contact_tracing(**ct_kw)]
        sim = refload.RefSim(ref, pars)
        for k in ('age', 'sex', 'symp_prob', 'severe_prob', 'crit_prob', 'death_prob', 'rel_trans', 'rel_sus'):
            out[f's{i}.person.{k}'] = sim.people[k].copy()
        for li, lk in enumerate(sim.people.contacts.keys()):
            for c in ('p1', 'p2', 'beta'):
                out[f's{i}.L{li}.{c}'] = sim.people.contacts[lk][c].copy()
        out[f's{i}.pars'] = np.array(json.dumps(jsonable({k: v for k, v in sim.pars.items() if k != 'interventions'})))
        out[f's{i}.interventions'] = np.array(json.dumps({'test_prob': tp_kw, 'contact_tracing': ct_kw}))
        sim.run()
        for k, v in sim.results.items():
            if k == 'variant':
                for kk, vv in v.items():
                    out[f's{i}.res.{kk}'] = vv
            else:
                out[f's{i}.res.{k}'] = v
        for k in TESTING_FINAL:
            out[f's{i}.final.{k}'] = sim.people[k].copy()
    out['n'] = np.array(len(TESTING_CASES))
    np.savez_compressed(os.path.join(HERE, 'ref_testing.npz'), **out)
    print('ref_testing.npz written')


class _Res:
    """The part of the reference's Result the reporting methods use."""

    def __init__(self, values):
        self.values = np.asarray(values, dtype=np.float64)

    def __getitem__(self, k):
        return self.values[k]

    def __setitem__(self, k, v):
        self.values[k] = v


def make_reporting_fixture(ref):
    """Inputs and outputs of the reference's compute_yield, compute_doubling,
    compute_r_eff (all three methods) and compute_gen_time (sim.py:853-1040) on
    a whole reference run with testing; sciris' smooth is restated (sciris is
    not installed)."""
    from covasim_gb300.sim import _smooth
    import types
    pop_type, n, days, seed, waning, dyn, tp_kw, ct_kw = TESTING_CASES[0]
    pars = ref.make_pars(pop_size=3000, n_days=60, pop_type=pop_type, rand_seed=seed, use_waning=waning)
    pars['interventions'] = [ref.cvint.test_prob(**tp_kw), ref.cvint.contact_tracing(**ct_kw)]
    sim = refload.RefSim(ref, pars).run()
    r = sim.results
    res = {k: _Res(v) for k, v in r.items() if k != 'variant'}
    for key in ref.cvd.result_flows:
        res[f'cum_{key}'] = _Res(np.cumsum(r[f'new_{key}']))
    res['cum_infections'].values += pars['pop_infected']
    res['n_alive'] = _Res(pars['pop_size'] - res['cum_deaths'].values)
    for key in ('test_yield', 'rel_test_yield', 'doubling_time', 'r_eff'):
        res[key] = _Res(np.zeros(sim.npts))
    sc_ns = types.SimpleNamespace(**vars(refload.sc))
    sc_ns.smooth = _smooth
    ns = {'np': np, 'sc': sc_ns, 'cvu': ref.cvu, 'cvm': types.SimpleNamespace(warn=print)}
    fns = refload.load_functions('sim.py', classname='Sim', namespace=ns,
                                 names=['compute_yield', 'compute_doubling', 'compute_r_eff', 'compute_gen_time'])
    class RefSimStub:
        def __getitem__(self, k):
            return self.pars[k]
    stub = RefSimStub()
    stub.results, stub.people, stub.npts, stub.tvec, stub.pars = res, sim.people, sim.npts, np.arange(sim.npts), pars
    out = {}
    fns['compute_yield'](stub)
    out['out.test_yield'] = res['test_yield'].values.copy()
    out['out.rel_test_yield'] = res['rel_test_yield'].values.copy()
    out['out.doubling_time'] = fns['compute_doubling'](stub).copy()
    for method in ('daily', 'infectious', 'outcome'):
        out[f'out.r_eff_{method}'] = np.array(fns['compute_r_eff'](stub, method=method), dtype=np.float64).copy()
    gt = fns['compute_gen_time'](stub)
    out['out.gen_time'] = np.array([gt['true'], gt['true_std'], gt['clinical'], gt['clinical_std']])
    for k in ('new_tests', 'new_diagnoses', 'n_infectious', 'n_alive', 'cum_diagnoses', 'cum_infections',
              'new_infections', 'n_imports'):
        out[f'res.{k}'] = res[k].values.copy()
    for k in ('date_recovered', 'date_dead', 'date_infectious', 'date_exposed', 'date_symptomatic'):
        out[f'people.{k}'] = sim.people[k].copy()
    log = sim.people.infection_log
    out['log.source'] = np.array([-1 if e['source'] is None else e['source'] for e in log], dtype=np.int64)
    out['log.target'] = np.array([e['target'] for e in log], dtype=np.int64)
    out['dur'] = np.array(json.dumps(jsonable(pars['dur'])))
    np.savez_compressed(os.path.join(HERE, 'ref_reporting.npz'), **out)
    print('ref_reporting.npz written')


class _Col(np.ndarray):
    """A numpy column with the two pandas Series attributes the reference's consumers use."""

    def __array_finalize__(self, obj):
        self._index = getattr(obj, '_index', None)

    @property
    def values(self):
        return np.asarray(self)

    def items(self):
        return zip(list(self._index), np.asarray(self).tolist())


class _Frame:
    """The few DataFrame operations of the reference's Fit and TransTree
    (pandas is not installed): records or dict construction, columns, column
    get/set with scalar broadcast, rename, boolean .loc get/set."""

    def __init__(self, data=None, index=None):
        if isinstance(data, list):
            keys = list(dict.fromkeys(k for r in data for k in r))
            data = {k: [r.get(k) for r in data] for k in keys}
        self._cols = {k: self._arr(v) for k, v in dict(data or {}).items()}
        self._index = index

    @staticmethod
    def _arr(v):
        if isinstance(v, np.ndarray):
            return v
        v = list(v)
        if all(x is None or isinstance(x, (int, float, np.integer, np.floating)) for x in v):
            if any(x is None for x in v):  # pandas: numbers with None -> float64 with NaN
                return np.array([np.nan if x is None else x for x in v], dtype=np.float64)
            return np.asarray(v)
        return np.array(v, dtype=object)

    @property
    def columns(self):
        return list(self._cols)

    def __len__(self):
        return len(next(iter(self._cols.values()))) if self._cols else 0

    def __getitem__(self, k):
        c = np.asarray(self._cols[k]).view(_Col)
        c._index = self._index if self._index is not None else np.arange(len(c))
        return c

    def __setitem__(self, k, v):
        self._cols[k] = np.full(len(self), v, dtype=object) if np.isscalar(v) else np.asarray(v)

    def rename(self, columns):
        return _Frame({columns.get(k, k): v for k, v in self._cols.items()})

    @property
    def loc(self):
        frame = self

        class _Loc:
            def __getitem__(lself, mask):
                m = np.asarray(mask, dtype=bool)
                return _Frame({k: v[m] for k, v in frame._cols.items()})

            def __setitem__(lself, key, val):
                mask, col = key
                frame._cols[col][np.asarray(mask, dtype=bool)] = val
        return _Loc()


class _ObjDict(dict):
    """sciris' objdict: attribute access, and [:] for the values as an array."""

    def __getattr__(self, k):
        try:
            return self[k]
        except KeyError as E:
            raise AttributeError(k) from E

    def __setattr__(self, k, v):
        self[k] = v

    def __getitem__(self, k):
        if isinstance(k, slice):
            return np.array(list(self.values()))[k]
        return dict.__getitem__(self, k)


class _ODict(dict):
    """sciris' odict with a default factory."""

    def __init__(self, defaultdict=None):
        super().__init__()
        self._factory = defaultdict

    def __missing__(self, k):
        self[k] = v = self._factory()
        return v


def make_analysis_fixture(ref):
    """Outputs of the reference's own TransTree (analysis.py:1772-2056), Fit
    (analysis.py:991-1235) and compute_gof (misc.py:707-790) on a reference run
    with testing and tracing; pandas and sciris are replaced by the small
    stand-ins above."""
    import types
    pop_type, n, days, seed, waning, dyn, tp_kw, ct_kw = TESTING_CASES[0]
    pars = ref.make_pars(pop_size=n, n_days=days, pop_type=pop_type, rand_seed=seed, use_waning=waning)
    pars['interventions'] = [ref.cvint.test_prob(**tp_kw), ref.cvint.contact_tracing(**ct_kw)]
    sim = refload.RefSim(ref, pars).run()
    people = sim.people
    log = people.infection_log

    sc_ns = types.SimpleNamespace(**vars(refload.sc))
    sc_ns.objdict = _ObjDict
    sc_ns.odict = _ODict
    sc_ns.isiterable = lambda x: np.iterable(x)
    sc_ns.prettyobj = object
    sc_ns.day = lambda d, start_date=None: int(d)  # integer days only in these cases
    misc_ns = {'np': np, 'sc': sc_ns}
    gof_fn = refload.load_functions('misc.py', ['compute_gof'], namespace=misc_ns)['compute_gof']
    cvm = types.SimpleNamespace(warn=print, compute_gof=gof_fn)
    pd_stub = types.SimpleNamespace(DataFrame=_Frame)
    ns = {'np': np, 'sc': sc_ns, 'pd': pd_stub, 'cvm': cvm}
    classes = refload.load_classes('analysis.py', ['Analyzer', 'Fit', 'TransTree'], ns)

    out = {}
    # -- transmission tree (agent 0 made a source on purpose: the `if source:` convention)
    log = [dict(e) for e in log]
    zero_rec = next((k for k, e in enumerate(log) if e['source'] is not None), None)
    if zero_rec is not None:
        log[zero_rec]['source'] = 0

    class PeopleStub:
        def __init__(self):
            self.t = sim.npts - 1
            self.infection_log = log

        def __len__(self):
            return n

        def __getitem__(self, k):
            return people[k]

    class SimStub:
        def __init__(self):
            self.people = PeopleStub()
            self.results = {'t': np.arange(sim.npts), 'cum_infections': _Res(np.cumsum(sim.results['new_infections']))}

        def __getitem__(self, k):
            return {'start_day': '2020-03-01', 'rescale': False, 'pop_scale': 1}[k]

    tt = classes['TransTree'](SimStub(), to_networkx=True)
    out['tt.sources'] = np.array([-1 if s is None else s for s in tt.sources], dtype=np.int64)
    out['tt.source_dates'] = np.array([-1 if s is None else s for s in tt.source_dates], dtype=np.int64)
    out['tt.targets_count'] = np.array([len(t) for t in tt.targets], dtype=np.int64)
    out['tt.targets_flat'] = np.array([g for t in tt.targets for g in t], dtype=np.int64)
    out['tt.target_dates_flat'] = np.array([d for t in tt.target_dates for d in t], dtype=np.int64)
    out['tt.n_targets'] = np.asarray(tt.n_targets, dtype=np.float64)
    out['tt.n_targets_10_25'] = np.asarray(tt.count_targets(10, 25), dtype=np.float64)
    out['tt.transmissions'] = np.array(tt.transmissions, dtype=np.int64).reshape(-1, 2)
    out['tt.r0_0'] = np.array(tt.r0(False))
    out['tt.r0_1'] = np.array(tt.r0(True))
    det = tt.detailed
    for k in det.columns:
        col = det[k].values
        out[f'tt.detailed.{k}'] = (np.array([str(x) for x in col]) if col.dtype == object
                                   else np.asarray(col, dtype=np.float64))
    for k in tt.df.columns:
        col = tt.df[k].values
        out[f'tt.df.{k}'] = np.array([str(x) for x in col]) if col.dtype == object else np.asarray(col)
    out['log.source'] = np.array([-1 if e['source'] is None else e['source'] for e in log], dtype=np.int64)
    out['log.target'] = np.array([e['target'] for e in log], dtype=np.int64)
    out['log.date'] = np.array([e['date'] for e in log], dtype=np.int64)
    out['log.layer'] = np.array([e['layer'] for e in log])
    out['log.variant'] = np.array([str(e['variant']) for e in log])
    for k in ('age', 'date_exposed', 'date_symptomatic', 'date_tested', 'date_diagnosed', 'date_severe',
              'date_critical', 'date_known_contact', 'date_quarantined', 'date_end_quarantine', 'date_recovered'):
        out[f'people.{k}'] = np.asarray(people[k]).copy()
    out['meta'] = np.array([n, sim.npts - 1])

    # -- goodness of fit
    rng = np.random.RandomState(11)
    a = np.cumsum(rng.poisson(5, 40)).astype(float)
    b = a * rng.uniform(0.8, 1.2, 40)
    gof_cases = [dict(), dict(normalize=False), dict(use_frac=True), dict(use_squared=True, as_scalar='mean'),
                 dict(as_scalar='median'), dict(normalize=False, use_squared=True, as_scalar='sum'),
                 dict(use_frac=True, eps=1e-3, as_scalar='sum')]
    out['gof.actual'], out['gof.predicted'] = a, b
    out['gof.cases'] = np.array(json.dumps(gof_cases))
    for i, kw in enumerate(gof_cases):
        out[f'gof.out{i}'] = np.asarray(gof_fn(a, b, **kw), dtype=np.float64)

    # -- Fit against synthetic data: some dates outside the sim, missing values, a custom key
    import datetime as dt
    start = dt.date(2020, 3, 1)
    sim_dates = [start + dt.timedelta(days=d) for d in range(sim.npts)]
    res = {}
    for key in ref.cvd.result_flows:
        res[f'cum_{key}'] = _Res(np.cumsum(sim.results[f'new_{key}']))
        res[f'new_{key}'] = _Res(sim.results[f'new_{key}'])
    res['cum_infections'].values += pars['pop_infected']
    data_days = np.arange(-5, sim.npts + 5, 2)
    data_dates = [start + dt.timedelta(days=int(d)) for d in data_days]
    dcols = {}
    for key in ('cum_diagnoses', 'cum_deaths', 'cum_tests', 'new_infections'):
        base = np.interp(data_days, np.arange(sim.npts), res[key].values)
        vals = np.round(base * rng.uniform(0.7, 1.3, len(base)) + rng.poisson(2, len(base)))
        vals[rng.rand(len(vals)) < 0.15] = np.nan
        dcols[key] = vals
    data = _Frame(dcols, index=data_dates)

    class FitSim:
        def __init__(self):
            self.data = data
            self.results_ready = True
            self.results = dict(res, t=np.arange(sim.npts), date=np.array(sim_dates, dtype=object))
            self.npts = sim.npts
            self.datevec = np.array(sim_dates, dtype=object)

        def result_keys(self):
            return [k for k in res]

    fit_cases = [dict(), dict(keys=['cum_diagnoses', 'new_infections'], weights={'new_infections': 2.0}),
                 dict(use_frac=True, as_scalar='sum'),
                 dict(weights={'cum_tests': np.linspace(0.5, 2, sim.npts)}),
                 dict(custom={'extra': {'data': np.array([1.0, 2.0, 4.0]), 'sim': np.array([1.5, 2.0, 3.0]), 'weight': 3.0}})]
    out['fit.cases'] = np.array(json.dumps(jsonable(fit_cases)))
    for i, kw in enumerate(fit_cases):
        f = classes['Fit'](FitSim(), **copy.deepcopy(kw))
        out[f'fit.mismatch{i}'] = np.array(f.mismatch, dtype=np.float64)
        out[f'fit.keys{i}'] = np.array(list(f.mismatches.keys()))
        out[f'fit.mismatches{i}'] = np.array(list(f.mismatches.values()), dtype=np.float64)
    for key, vals in dcols.items():
        out[f'data.{key}'] = vals
    out['data.days'] = data_days
    for key in ('cum_diagnoses', 'cum_deaths', 'cum_tests', 'new_infections', 'cum_infections'):
        out[f'simres.{key}'] = res[key].values.copy()
    np.savez_compressed(os.path.join(HERE, 'ref_analysis.npz'), **out)
    print('ref_analysis.npz written', len(log), 'records')


def make_state_diagram_fixture(ref=None):
    """The state-implication matrices of the reference's tests/state_diagram.xlsx
    (sheets 'Without waning' and 'With waning', read by test_immunity.py's
    test_states): relation[s1][s2] = 1 if being s1 implies s2, -1 if it implies
    not s2, 0 if either. Read with zipfile and the sheet XML (no openpyxl)."""
    import re
    import zipfile
    import xml.etree.ElementTree as ET
    path = os.path.join(refload.REF_ROOT, 'tests', 'state_diagram.xlsx')
    z = zipfile.ZipFile(path)
    ns = {'m': 'http://schemas.openxmlformats.org/spreadsheetml/2006/main'}
    rel_ns = '{http://schemas.openxmlformats.org/officeDocument/2006/relationships}id'
    strings = [''.join(t.text or '' for t in si.iter(f'{{{ns["m"]}}}t'))
               for si in ET.fromstring(z.read('xl/sharedStrings.xml')).findall('m:si', ns)]
    rels = ET.fromstring(z.read('xl/_rels/workbook.xml.rels'))
    targets = {r.get('Id'): r.get('Target') for r in rels}
    wb = ET.fromstring(z.read('xl/workbook.xml'))
    out = {}
    for sheet in wb.find('m:sheets', ns):
        name = sheet.get('name')
        if name not in ('Without waning', 'With waning'):
            continue
        xml = ET.fromstring(z.read('xl/' + targets[sheet.get(rel_ns)].lstrip('/').replace('xl/', '')))
        rows = []
        for row in xml.find('m:sheetData', ns):
            cells = {}
            for c in row:
                v = c.find('m:v', ns)
                if v is None:
                    continue
                col = re.match(r'[A-Z]+', c.get('r')).group(0)
                cells[col] = strings[int(v.text)] if c.get('t') == 's' else v.text
            rows.append(cells)
        cols = sorted((k for k in rows[0] if k != 'A'), key=lambda c: (len(c), c))
        states = [rows[0][c] for c in cols]
        rel = {}
        for r in rows[1:]:
            if r.get('A') in states:
                rel[r['A']] = {states[j]: int(float(r[c])) for j, c in enumerate(cols)}
        out[name] = {'states': states, 'relation': rel}
    with open(os.path.join(HERE, 'state_diagram.json'), 'w') as f:
        json.dump(out, f, indent=1, ensure_ascii=False)
    print('state_diagram.json written', {k: len(v['relation']) for k, v in out.items()})


def make_distribution_fixture(ref, n_seeds=200, pop_size=20000, n_days=60):
    keys = ['new_infections', 'new_severe', 'new_deaths', 'new_infectious', 'new_recoveries', 'new_critical',
            'new_symptomatic', 'n_exposed']
    res = {k: np.zeros((n_seeds, n_days + 1)) for k in keys}
    t0 = time.time()
    for s in range(n_seeds):
        pars = ref.make_pars(pop_size=pop_size, n_days=n_days, pop_type='random', rand_seed=s)
        sim = refload.RefSim(ref, pars).run()
        for k in keys:
            res[k][s] = sim.results[k]
        if s % 20 == 0:
            print(f'  seed {s}: {time.time() - t0:.1f}s, cum inf {sim.results["new_infections"].sum()}')
    out = {k: v.astype(np.int32) for k, v in res.items()}
    out['meta'] = np.array([n_seeds, pop_size, n_days])
    np.savez_compressed(os.path.join(HERE, 'ref_distribution.npz'), **out)
    print('ref_distribution.npz written', time.time() - t0, 's')


# The hybrid distribution fixture: the model the 1M-agent benchmark runs (hybrid
# layers, waning immunity with NAb kinetics, the community layer redrawn daily),
# at a size the reference's code finishes in seconds per seed.
HYBRID_DIST = dict(pop_size=30000, n_days=150, pop_type='hybrid', use_waning=True,
                   dynam_layer=dict(h=0, s=0, w=0, c=1))
HYBRID_DIST_KEYS = ['new_infections', 'new_severe', 'new_deaths', 'new_critical', 'new_symptomatic',
                    'new_reinfections', 'new_recoveries', 'n_exposed', 'n_susceptible']


def _hybrid_dist_worker(job):
    root, seeds = job
    refload.set_reference_root(root)
    ref = refload.Reference()
    rows = []
    for s in seeds:
        pars = ref.make_pars(rand_seed=int(s), **copy.deepcopy(HYBRID_DIST))
        sim = refload.RefSim(ref, pars)
        while sim.t < sim.npts:
            sim.step()
            ref.draws()  # drop the recorded draws as the run goes (this fixture replays none)
        rows.append((int(s), {k: np.asarray(sim.results[k]) for k in HYBRID_DIST_KEYS},
                     np.asarray(sim.results['pop_nabs'])))
        del sim
    return rows


def make_distribution_hybrid_fixture(ref, n_seeds=200, procs=None):
    """n_seeds runs of the reference's own Sim.step on HYBRID_DIST, seeds 0..n_seeds-1,
    in a spawn pool (each worker loads the reference's code itself)."""
    import multiprocessing as mp
    procs = procs or max(1, min(os.cpu_count() or 1, 16))
    t0 = time.time()
    jobs = [(refload.REF_ROOT, list(range(k, n_seeds, procs))) for k in range(procs)]
    with mp.get_context('spawn').Pool(procs) as pool:
        parts = pool.map(_hybrid_dist_worker, jobs)
    npts = HYBRID_DIST['n_days'] + 1
    out = {k: np.zeros((n_seeds, npts), np.int32) for k in HYBRID_DIST_KEYS}
    out['pop_nabs'] = np.zeros((n_seeds, npts), np.float64)
    for rows in parts:
        for s, r, nabs in rows:
            for k in HYBRID_DIST_KEYS:
                out[k][s] = r[k]
            out['pop_nabs'][s] = nabs
    out['meta'] = np.array([n_seeds, HYBRID_DIST['pop_size'], HYBRID_DIST['n_days']])
    out['pars'] = np.array(json.dumps(HYBRID_DIST))
    np.savez_compressed(os.path.join(HERE, 'ref_distribution_hybrid.npz'), **out)
    print('ref_distribution_hybrid.npz written', round(time.time() - t0, 1), 's; mean cum infections',
          out['new_infections'].sum(1).mean())


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument('--only', default=None)
    ap.add_argument('--seeds', type=int, default=200)
    ap.add_argument('--reference', default=os.environ.get('COVASIM_REFERENCE'),
                    help='the reference source tree (the directory holding covasim/)')
    args = ap.parse_args()
    if not args.reference:
        ap.error('pass --reference PATH (or set COVASIM_REFERENCE)')
    refload.set_reference_root(args.reference)
    ref = refload.Reference()
    groups = dict(pars=make_pars_fixture, kernels=make_kernels_fixture, day=make_day_fixtures,
                  sims=make_sims_fixture, testing=make_testing_fixture, reporting=make_reporting_fixture,
                  analysis=make_analysis_fixture, states=make_state_diagram_fixture,
                  distribution=lambda r: make_distribution_fixture(r, n_seeds=args.seeds),
                  distribution_hybrid=lambda r: make_distribution_hybrid_fixture(r, n_seeds=args.seeds))
    for name, fn in groups.items():
        if args.only is None or args.only == name:
            fn(ref)


if __name__ == '__main__':
    main()
