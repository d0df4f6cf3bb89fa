"""CPU restatement of Covasim 3.1.7's day loop (covasim/sim.py:558-685).

TEST INFRASTRUCTURE ONLY. The product never imports this module; tests and
the CPU-baseline leg of bench.py do.

Two random-number modes:

* ``rng='philox'``: every draw is keyed exactly like the CUDA library keys it
  (edge Bernoullis by (seed, day, layer, variant, edge); infection draws by
  (seed, day, agent, call); a dynamic layer's day as per-agent contact lists
  keyed by (seed, day, layer, agent), drawn for the day's sources), so a GPU
  run and this loop agree draw for draw.
* ``rng='mt'``: two MT19937 streams seeded with the sim's seed, one standing in
  for numba's (edge Bernoullis, ``choose``/``choose_r``) and one for numpy's
  (``infect`` and ``set_prognoses``), consumed in the reference's call order.

Philox mode also evaluates the NAb efficacy and update_nab with the CUDA
library's float-float formulation (``gpu_arith``) by default, so that a GPU
run and this loop agree bit for bit; MT mode uses the reference's float64.
"""
import numpy as np

from . import philox as ph
from .kernels import compute_viral_load, compute_trans_sus, compute_infections
from .people import (OraclePeople, TableDraws, SequentialDraws, philox_table, philox_table_ff, update_nab,
                     STATES, FLOWS, FLOWS_VARIANT)
from .gpu_arith import update_nab_gpu

F32 = np.float32

RESULT_STOCKS = ['susceptible', 'exposed', 'infectious', 'symptomatic', 'severe', 'critical',
                 'recovered', 'dead', 'diagnosed', 'known_dead', 'quarantined', 'isolated',
                 'vaccinated']
RESULT_STOCKS_BY_VARIANT = ['exposed_by_variant', 'infectious_by_variant']

# call tags of infect() draws in philox mode (shared with the CUDA library)
CALL_TRANSMISSION = 0
CALL_SEED = 1
CALL_IMPORT = 2

SEED_INFECTION_TAG = 0x5EED
IMPORT_TAG = 0x1B1B
NONNAIVE_TAG = 0x4A4A
RESCALE_TAG = 0x5C5C


def choose_seed_infections(seed, n, k):
    """Agents infected on day 0 in philox mode: a PCG64 stream keyed by the seed."""
    rng = np.random.Generator(np.random.PCG64([int(seed) & 0xFFFFFFFFFFFFFFFF, SEED_INFECTION_TAG]))
    return np.sort(rng.choice(n, size=int(k), replace=False)).astype(np.int64)


def philox_mode_importations(seed, rate, n, t):
    """Agents imported on day t in philox mode (the CUDA library's host-side
    schedule): Poisson(float32 rate) agents chosen without replacement, from a
    PCG64 stream keyed by (seed, 0x1B1B, t)."""
    rng = np.random.Generator(np.random.PCG64([int(seed) & 0xFFFFFFFFFFFFFFFF, IMPORT_TAG, int(t)]))
    k = int(rng.poisson(float(np.float32(rate))))
    return np.sort(rng.choice(int(n), size=k, replace=False)).astype(np.int64)


def set_prognoses(people, pars, rs):
    """covasim/people.py:139-161 with draws from ``rs`` (numpy RandomState)."""
    progs = pars['prognoses']
    inds = np.digitize(people.age, progs['age_cutoffs']) - 1
    people.symp_prob[:] = progs['symp_probs'][inds]
    people.severe_prob[:] = progs['severe_probs'][inds] * progs['comorbidities'][inds]
    people.crit_prob[:] = progs['crit_probs'][inds]
    people.death_prob[:] = progs['death_probs'][inds]
    people.rel_sus[:] = progs['sus_ORs'][inds]
    bd = pars['beta_dist']
    nbn_n = bd['par2']
    nbn_p = bd['par2'] / (bd['par1'] / bd.get('step', 1) + bd['par2'])
    draws = rs.negative_binomial(n=nbn_n, p=nbn_p, size=len(inds)) * bd.get('step', 1)
    people.rel_trans[:] = progs['trans_ORs'][inds] * draws


class OracleSim:
    """One simulation on the CPU.

    Args:
        pars: full parameter dict (prognoses, nab_kin and immunity filled in)
        person: dict of initial per-person arrays (at least age, symp_prob,
            severe_prob, crit_prob, death_prob, rel_trans, rel_sus)
        contacts: {layer key: dict(p1, p2, beta)}; layer order is layer index
        rng: 'philox' or 'mt'
        beta_schedule: optional per-day overall beta (change_beta), length npts
        interventions: optional list of ``oracle.interventions`` objects (testing, tracing)
    """

    def __init__(self, pars, person, contacts, rng='philox', beta_schedule=None, seed_inds=None, arith=None,
                 interventions=None):
        self.pars = pars
        self.n = int(pars['pop_size'])
        self.npts = int(pars['n_days']) + 1
        self.people = OraclePeople(pars, self.n)
        # 'reference': the reference's float64 NAb math; 'gpu': the CUDA library's float-float
        # formulation of it (gpu_arith), for draw-for-draw comparisons with a GPU run
        self.arith = arith or ('gpu' if rng == 'philox' else 'reference')
        self.people.arith = self.arith
        for k, v in person.items():
            self.people[k] = np.array(v, dtype=self.people[k].dtype)
        self.contacts = {k: {c: np.array(v[c]) for c in ('p1', 'p2', 'beta')} for k, v in contacts.items()}
        self.layer_keys = list(self.contacts.keys())
        self.rng = rng
        # philox mode: a dynamic layer's day is drawn as per-agent lists (ph.dyn_lists)
        self.dyn_tables = {}
        self.dyn_rse_max = {}  # the thinning bound of each dynamic layer: the largest rel_sus' it can meet
        if rng == 'philox':
            rs_max = np.float32(np.max(self.people.rel_sus)) if self.n else np.float32(0)
            for lkey in self.layer_keys:
                if pars['dynam_layer'].get(lkey, 0) and len(self.contacts[lkey]['p1']):
                    self.dyn_tables[lkey] = ph.dyn_count_table(len(self.contacts[lkey]['p1']), self.n)
                    self.dyn_rse_max[lkey] = max(rs_max, np.float32(rs_max * F32(pars['quar_factor'][lkey])))
        self.seed = int(pars['rand_seed'])
        self.k0, self.k1 = ph.seed_key(self.seed)
        if rng == 'mt':
            self.rs_numba = np.random.RandomState(self.seed)
            self.rs_numpy = np.random.RandomState(self.seed)
        self.beta_schedule = beta_schedule
        self.seed_inds = seed_inds
        self.exposure_hook = None  # optional f(sim, t, viral_load) before each day's transmission
        self.interventions = list(interventions or [])  # oracle.interventions objects, applied in order
        for iv in self.interventions:
            if hasattr(iv, 'initialize'):
                iv.initialize(self)
        self.t = 0
        # sim.py:342-346: the scale of each day, 1 to start with when rescaling dynamically
        pop_scale = pars.get('pop_scale') or 1
        self.rescale_vec = (1.0 if pars.get('rescale', True) else float(pop_scale)) * np.ones(self.npts)
        self.results = {}
        for key in FLOWS + [f'n_{k}' for k in RESULT_STOCKS] + ['n_imports', 'pop_nabs', 'pop_protection',
                                                                'pop_symp_protection']:
            self.results[key] = np.zeros(self.npts)
        nv = pars['n_variants']
        for key in FLOWS_VARIANT + [f'n_{k}' for k in RESULT_STOCKS_BY_VARIANT]:
            self.results[key] = np.zeros((nv, self.npts))

    # ------------------------------------------------------------------
    def _draws(self, call_tag):
        if self.rng == 'philox':
            if self.arith == 'gpu':  # the CUDA library's float-float normals and samples
                return TableDraws(None, ff_fn=philox_table_ff(self.seed, self.t, call_tag))
            return TableDraws(philox_table(self.seed, self.t, call_tag))
        return SequentialDraws(self.rs_numpy)

    def init_infections(self):
        """sim.py:505-532: the non-susceptible fraction made non-naive
        (people.py:414-431 on fresh agents: susceptible and naive cleared), then
        the seed infections."""
        p = self.pars
        frac = p.get('frac_susceptible', 1.0)
        if frac < 1:
            k = int(np.round((1 - frac) * self.n))
            if self.rng == 'philox':
                rng = np.random.Generator(np.random.PCG64([self.seed & 0xFFFFFFFFFFFFFFFF, NONNAIVE_TAG]))
                inds = np.sort(rng.choice(self.n, size=k, replace=False))
            else:  # cvu.choose: numba's stream
                inds = self.rs_numba.choice(self.n, k, replace=False)
            self.people.susceptible[inds] = False
            self.people.naive[inds] = False
        if p['pop_infected']:
            if self.seed_inds is not None:
                inds = np.asarray(self.seed_inds)
            elif self.rng == 'philox':
                inds = choose_seed_infections(self.seed, self.n, p['pop_infected'])
            else:
                inds = self.rs_numba.choice(self.n, int(p['pop_infected']), replace=False)
            self.people.infect(inds=inds, layer='seed_infection', draws=self._draws(CALL_SEED))

    def rescale(self):
        """sim.py:535-556: once the agents not naive exceed rescale_threshold of the
        population (and the scale has room to grow), scale up by at least
        rescale_factor and make that share of them naive again."""
        p = self.pars
        if not p.get('rescale', True):
            return
        pop_scale = p.get('pop_scale') or 1
        current = self.rescale_vec[self.t]
        if current < pop_scale:
            not_naive = np.nonzero(~self.people.naive)[0]
            m = len(not_naive)
            ratio = m / self.n
            if ratio > p['rescale_threshold']:
                scaling = min(max(ratio / p['rescale_threshold'], p['rescale_factor']), pop_scale / current)
                self.rescale_vec[self.t:] *= scaling
                k = int(round(m * (1.0 - 1.0 / scaling)))
                if self.rng == 'philox':
                    rng = np.random.Generator(np.random.PCG64([self.seed & 0xFFFFFFFFFFFFFFFF, RESCALE_TAG, self.t]))
                    choices = rng.choice(m, size=k, replace=False)
                else:  # cvu.choose: numba's stream, int32 arguments
                    choices = self.rs_numba.choice(int(np.int32(m)), int(np.int32(k)), replace=False)
                self.people.make_naive(not_naive[choices])

    def _import_variant(self, v, t):
        """immunity.py:117-130 in philox mode (the CUDA library's host draws): n_imports
        over the day's scale, rounded at random, agents chosen among the susceptible
        from a PCG64 stream keyed by (seed, 0x1A1A, day, variant); infect() without
        bed limits, as variant.apply calls it."""
        if self.rng != 'philox':
            raise NotImplementedError('variant importations are replayed in philox mode only')
        sus = np.nonzero(self.people.susceptible)[0]
        rng = np.random.default_rng([self.seed, 0x1A1A, t, v.index])
        x = v.n_imports / (self.rescale_vec[t] if getattr(v, 'rescale', True) else 1.0)
        n_imp = int(x) if x == int(x) else int(np.floor(x + rng.random()))  # more than len(sus): ValueError below
        inds = rng.choice(sus, n_imp, replace=False)
        if len(inds):
            self.people.infect(inds=inds, layer='importation', variant=v.index, draws=self._draws(CALL_IMPORT + v.index))
        self.results['n_imports'][t] += n_imp

    def update_contacts(self):
        """people.py:199-206 -> base.py:1849-1876 (Layer.update, frac=1). In philox
        mode a dynamic layer is not materialised: its day's edges are the per-agent
        lists that ``dynamic_lists`` draws where they are needed."""
        for li, lkey in enumerate(self.layer_keys):
            if self.pars['dynam_layer'].get(lkey, 0):
                layer = self.contacts[lkey]
                n_new = len(layer['p1'])
                if self.rng == 'philox':
                    continue
                inds = self.rs_numba.permutation(n_new)
                layer['p1'][inds] = self.rs_numba.randint(0, self.n, n_new).astype(np.int32)
                layer['p2'][inds] = self.rs_numba.randint(0, self.n, n_new).astype(np.int32)
                layer['beta'] = np.ones(n_new, dtype=F32)

    def dynamic_lists(self, lkey, agents):
        """Day t's contact lists of ``agents`` in dynamic layer lkey (philox mode):
        arrays (agent, d, j, partner), d = 0 for the agent as p1, 1 as p2."""
        li = self.layer_keys.index(lkey)
        return ph.dyn_lists(self.k0, self.k1, self.t, li, agents, self.dyn_tables[lkey], self.n)

    def exposures(self, li, variant, beta, rel_trans, rel_sus):
        """The day's exposed directions of layer li (source rel_trans != 0, target
        rel_sus != 0, p != 0) with their transmission outcome, as the CUDA library
        draws them: arrays (source, target, direction, edge identity, edge beta,
        float32 p, transmitted). Stored layers: every edge in both directions, the
        identity its index, transmitted when the edge's uniform u < p. Dynamic
        layers in philox mode: every entry of every source's lists (identity
        ph.dyn_edge_id), transmitted when it is a potential transmission of the
        thinning and u < p * 2**m (see dynamic_infections)."""
        lkey = self.layer_keys[li]
        if lkey in self.dyn_tables:
            return self._dyn_entries(li, variant, beta, rel_trans, rel_sus, every_entry=True)
        layer = self.contacts[lkey]
        e = np.arange(len(layer['p1']), dtype=np.int64)
        src = np.concatenate([layer['p1'], layer['p2']]).astype(np.int64)
        tgt = np.concatenate([layer['p2'], layer['p1']]).astype(np.int64)
        d = np.repeat(np.array([0, 1], dtype=np.int64), len(e))
        eb = np.concatenate([layer['beta'], layer['beta']]).astype(F32)
        eid = np.concatenate([e, e])
        p = (F32(beta) * eb) * rel_trans[src] * rel_sus[tgt]
        keep = p != 0
        src, tgt, d, eid, eb, p = src[keep], tgt[keep], d[keep], eid[keep], eb[keep], p[keep]
        u0, u1 = ph.edge_uniforms(self.k0, self.k1, self.t, li, variant, eid)
        hit = np.where(d == 0, u0, u1) < p.astype(np.float64)
        return src, tgt, d, eid, eb, p, hit

    def _dyn_entries(self, li, variant, beta, rel_trans, rel_sus, every_entry=False):
        """The list entries of dynamic layer li's sources (rel_trans != 0) with
        p != 0: the potential transmissions of the thinning, or every entry."""
        lkey = self.layer_keys[li]
        t, k0, k1 = self.t, self.k0, self.k1
        S = rel_trans.nonzero()[0].astype(np.int64)
        q = (F32(beta) * F32(1.0)) * rel_trans[S]  # beta * layer beta (1 for a redrawn layer) * rel_trans'
        m = ph.thin_shift(q * F32(self.dyn_rse_max[lkey]))
        counts = ph.dyn_counts(k0, k1, t, li, S, self.dyn_tables[lkey]).reshape(-1)
        pos = np.repeat(np.repeat(np.arange(len(S)), 2), counts)  # source position of each entry
        d = np.repeat(np.tile(np.array([0, 1], dtype=np.int64), len(S)), counts)
        j = np.arange(len(pos), dtype=np.int64) - np.repeat(np.cumsum(counts) - counts, counts)
        a = S[pos]
        pot = ph.dyn_potential(k0, k1, t, li, a, d, j, m[pos])
        if not every_entry:
            a, d, j, pos, pot = a[pot], d[pot], j[pot], pos[pot], pot[pot]
        g = ph.dyn_partners(k0, k1, t, li, a, d, j, self.n)
        p = q[pos] * rel_sus[g]
        keep = p != 0
        a, g, d, j, pos, pot, p = a[keep], g[keep], d[keep], j[keep], pos[keep], pot[keep], p[keep]
        eid = ph.dyn_edge_id(a, j, t, li)
        u0, u1 = ph.edge_uniforms(k0, k1, t, li, variant, eid)
        scaled = p * np.ldexp(np.float32(1), m[pos]).astype(F32)  # p * 2**m, exact in float32
        hit = pot & (np.where(d == 0, u0, u1) < scaled.astype(np.float64))
        return a, g, d, eid, np.ones(len(a), dtype=F32), p, hit

    def dynamic_infections(self, li, variant, beta, rel_trans, rel_sus):
        """compute_infections (utils.py:93-128) over dynamic layer li in philox
        mode, with the sources' list entries thinned: entry j of list d of source
        s (p(s, g) = beta * rel_trans'[s] * rel_sus'[g] <= pmax = beta *
        rel_trans'[s] * rse_max) is a potential transmission with probability
        2**-m >= pmax (ph.thin_shift, ph.dyn_potential); only then is its partner
        g drawn, and it transmits when its edge uniform u < p * 2**m. The
        transmissions are ordered by (direction, identity), as the reference
        orders direction then edge."""
        s, g, d, eid, _, _, hit = self._dyn_entries(li, variant, beta, rel_trans, rel_sus)
        s, g, d, eid = s[hit], g[hit], d[hit], eid[hit]
        order = np.lexsort((eid, d))
        return s[order].astype(np.int32), g[order].astype(np.int32)

    def step(self):
        p = self.pars
        t = self.t
        people = self.people
        if t == 0:
            self.init_infections()
        self.rescale()
        people.update_states_pre(t=t)
        self.update_contacts()
        hosp_max = people.severe.sum() > p['n_beds_hosp'] if p['n_beds_hosp'] is not None else False
        icu_max = people.critical.sum() > p['n_beds_icu'] if p['n_beds_icu'] is not None else False
        if p.get('n_imports'):  # sim.py:582-587
            rate = p['n_imports'] / self.rescale_vec[t]
            if self.rng == 'philox':
                inds = philox_mode_importations(self.seed, rate, self.n, t)
            else:  # cvu.poisson / cvu.choose are numba functions: numba's stream; the rate is typed float32
                k = int(self.rs_numba.poisson(float(F32(rate)), 1)[0])
                inds = self.rs_numba.choice(self.n, k, replace=False) if k > 0 else np.zeros(0, dtype=np.int64)
            if len(inds):
                people.infect(inds=inds, hosp_max=hosp_max, icu_max=icu_max, layer='importation',
                              draws=self._draws(CALL_IMPORT))
                self.results['n_imports'][t] += len(inds)
        for v in p.get('variants') or []:  # sim.py:590-592 -> immunity.py:117-130 variant.apply
            if t in np.atleast_1d(v.days):
                self._import_variant(v, t)
        if self.beta_schedule is not None:
            p['beta'] = self.beta_schedule[t]
        for iv in self.interventions:  # sim.py:596-598
            iv.apply(self)
        people.update_states_post()  # sim.py:600

        vd = p['viral_dist']
        viral_load = compute_viral_load(t, people.date_infectious, people.date_recovered, people.date_dead,
                                        F32(vd['frac_time']), F32(vd['load_ratio']), F32(vd['high_cap']))
        if self.exposure_hook is not None:  # test hook: the state the transmission draws see
            self.exposure_hook(self, t, viral_load)
        nv = p['n_variants']
        for variant in range(nv):
            label = p['variant_map'][variant]
            beta = F32(p['beta'] * p['rel_beta'] * p['variant_pars'][label]['rel_beta'])
            inf_variant = people.infectious * (people.infectious_variant == variant)
            if not inf_variant.any():
                continue
            for li, lkey in enumerate(self.layer_keys):
                layer = self.contacts[lkey]
                rel_trans, rel_sus = compute_trans_sus(
                    people.rel_trans, people.rel_sus, inf_variant, people.susceptible,
                    F32(p['beta_layer'][lkey]), viral_load, people.symptomatic, people.isolated,
                    people.quarantined, F32(p['asymp_factor']), F32(p['iso_factor'][lkey]),
                    F32(p['quar_factor'][lkey]), people.sus_imm[variant, :])
                if lkey in self.dyn_tables:
                    src, tgt = self.dynamic_infections(li, variant, beta, rel_trans, rel_sus)
                else:
                    if self.rng == 'philox':  # keyed draws for the surviving edges only
                        k0, k1 = self.k0, self.k1
                        uniforms = lambda d, edge_inds: ph.edge_uniforms(k0, k1, t, li, variant, edge_inds)[d]  # noqa: E731
                    else:
                        rs = self.rs_numba
                        uniforms = lambda d, edge_inds: rs.random_sample(len(edge_inds))  # noqa: E731
                    src, tgt = compute_infections(beta, layer['p1'], layer['p2'], layer['beta'],
                                                  rel_trans, rel_sus, uniforms)
                people.infect(inds=tgt, hosp_max=hosp_max, icu_max=icu_max, source=src, layer=lkey,
                              variant=variant, draws=self._draws(CALL_TRANSMISSION))

        # sim.py:651-663: stocks and flows
        for key in RESULT_STOCKS:
            self.results[f'n_{key}'][t] = np.count_nonzero(people[key])
        for key in RESULT_STOCKS_BY_VARIANT:
            for v in range(nv):
                self.results[f'n_{key}'][v, t] = np.count_nonzero(people[key][v, :])
        for key, count in people.flows.items():
            self.results[key][t] += count
        for key, count in people.flows_variant.items():
            for v in range(nv):
                self.results[key][v, t] += count[v]
        # sim.py:666-674: NAb update and population means
        if p['use_waning']:
            has_nabs = people.peak_nab.nonzero()[0]
            if len(has_nabs):
                if self.arith == 'gpu':
                    update_nab_gpu(people, inds=has_nabs)
                else:
                    update_nab(people, inds=has_nabs)
        inds_alive = (~people.dead).nonzero()[0]
        nab_alive = people.nab[inds_alive]
        self.results['pop_nabs'][t] = np.sum(nab_alive[nab_alive.nonzero()[0]]) / len(inds_alive)
        self.results['pop_protection'][t] = np.nanmean(people.sus_imm)
        self.results['pop_symp_protection'][t] = np.nanmean(people.symp_imm)
        self.t += 1

    def run(self, until=None):
        until = self.npts if until is None else until
        while self.t < until:
            self.step()
        return self
