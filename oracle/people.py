"""CPU restatement of Covasim 3.1.7's agent state, transitions, infect and NAb logic.

TEST INFRASTRUCTURE ONLY. The product never imports this module; tests and
the CPU-baseline leg of bench.py do.

``OraclePeople`` holds the same keys as ``cv.People`` (covasim/defaults.py:37-138)
as numpy arrays with the reference's dtypes, and its methods restate
covasim/people.py and covasim/immunity.py line by line. Random draws go
through a draw provider so that the same code runs with

* ``TableDraws``: a per-agent table (Philox draws, or the reference's own
  recorded draws replayed per agent), or
* ``SequentialDraws``: a numpy ``RandomState`` consumed in the reference's
  call order (MT19937 mode, as the reference does it).
"""
import numpy as np

from . import philox as ph
from .kernels import lognormal_params

F32 = np.float32
I32 = np.int32

PERSON = ['uid', 'age', 'sex', 'symp_prob', 'severe_prob', 'crit_prob', 'death_prob',
          'rel_trans', 'rel_sus', 'n_infections', 'n_breakthroughs']
STATES = ['susceptible', 'naive', 'exposed', 'infectious', 'symptomatic', 'severe', 'critical',
          'tested', 'diagnosed', 'recovered', 'known_dead', 'dead', 'known_contact',
          'quarantined', 'isolated', 'vaccinated']
VARIANT_STATES = ['exposed_variant', 'infectious_variant', 'recovered_variant']
BY_VARIANT_STATES = ['exposed_by_variant', 'infectious_by_variant']
IMM_STATES = ['sus_imm', 'symp_imm', 'sev_imm']
NAB_STATES = ['peak_nab', 'nab', 't_nab_event']
VACC_STATES = ['doses', 'vaccine_source']
DATES = [f'date_{s}' for s in STATES] + ['date_pos_test', 'date_end_quarantine', 'date_end_isolation']
DURS = ['dur_exp2inf', 'dur_inf2sym', 'dur_sym2sev', 'dur_sev2crit', 'dur_disease']

FLOWS = ['new_infections', 'new_reinfections', 'new_infectious', 'new_symptomatic', 'new_severe',
         'new_critical', 'new_recoveries', 'new_deaths', 'new_tests', 'new_diagnoses',
         'new_known_deaths', 'new_quarantined', 'new_isolated', 'new_doses', 'new_vaccinated']
FLOWS_VARIANT = ['new_infections_by_variant', 'new_symptomatic_by_variant',
                 'new_severe_by_variant', 'new_infectious_by_variant']


def sample_from_normal(dist, z):
    """covasim/utils.py:156-236 (sample) for the distributions that are a
    function of one standard normal per draw; ``dist`` is the reference's
    dict(dist=..., par1=..., par2=...)."""
    name, p1, p2 = dist['dist'], dist['par1'], dist['par2']
    z = np.asarray(z, dtype=np.float64)
    if name in ('norm', 'normal'):
        return p1 + p2 * z
    if name == 'normal_pos':
        return np.abs(p1 + p2 * z)
    if name == 'normal_int':
        return np.round(np.abs(p1 + p2 * z))
    if name in ('lognorm', 'lognormal', 'lognorm_int', 'lognormal_int'):
        if p1 > 0:
            mean, sigma = lognormal_params(p1, p2)
            out = np.exp(mean + sigma * z)
        else:
            out = np.zeros(z.shape)
        if '_int' in name:
            out = np.round(out)
        return out
    raise NotImplementedError(f'distribution "{name}" is not a function of one normal draw')


def dist_consumes_draws(dist):
    """Whether the reference's sample() draws from the stream for this dist."""
    name = dist['dist']
    return not (name.startswith('lognorm') and not dist['par1'] > 0)


class TableDraws:
    """Per-agent draw table [N_DRAWS] indexed by agent (see philox.N_*).

    With ``ff_fn`` (the CUDA library's arithmetic) the normals are float-float
    pairs and samples are formed in float-float (``gpu_arith.sample_ff``)."""

    def __init__(self, table_fn, ff_fn=None):
        self.table_fn = table_fn  # inds -> float64 [len(inds), N_DRAWS]
        self.ff_fn = ff_fn        # inds -> (z_hi [n, 6], z_lo [n, 6], u [n, 4])

    def begin(self, inds):
        self._inds = np.asarray(inds)
        if self.ff_fn is not None:
            if len(self._inds):
                self._zh, self._zl, self._u = self.ff_fn(self._inds)
            else:
                self._zh = self._zl = np.zeros((0, 6), np.float32)
                self._u = np.zeros((0, 4))
            return
        self._tab = self.table_fn(self._inds) if len(self._inds) else np.zeros((0, ph.N_DRAWS))

    def _rows(self, inds):
        # infect() draws for subsets of its sorted, unique index array
        return np.searchsorted(self._inds, np.asarray(inds))

    def normal(self, slot, inds, dist):
        if self.ff_fn is not None:
            from .gpu_arith import sample_ff
            r = self._rows(inds)
            return sample_ff(dist, self._zh[r, slot], self._zl[r, slot])
        return sample_from_normal(dist, self._tab[self._rows(inds), slot])

    def uniform(self, slot, inds):
        if self.ff_fn is not None:
            return self._u[self._rows(inds), slot - ph.U_SYMP]
        return self._tab[self._rows(inds), slot]


class SequentialDraws:
    """numpy MT19937 stream consumed in the reference's call order."""

    def __init__(self, rs):
        self.rs = rs

    def begin(self, inds):
        pass

    def normal(self, slot, inds, dist):
        n = len(inds)
        if not dist_consumes_draws(dist) or n == 0:
            return sample_from_normal(dist, np.zeros(n))
        return sample_from_normal(dist, self.rs.standard_normal(n))

    def uniform(self, slot, inds):
        return self.rs.random_sample(len(inds))


def philox_table(seed, day, call_tag):
    k0, k1 = ph.seed_key(seed)
    return lambda inds: ph.infect_draws(k0, k1, day, call_tag, inds)


def philox_table_ff(seed, day, call_tag):
    k0, k1 = ph.seed_key(seed)
    return lambda inds: ph.infect_draws_ff(k0, k1, day, call_tag, inds)


class OraclePeople:
    """Agent arrays with the reference's keys and dtypes (covasim/people.py:47-118)."""

    def __init__(self, pars, n):
        self.pars = pars
        nv = pars['n_variants']
        self.n = n
        self.t = 0
        for key in PERSON:
            if key == 'uid':
                setattr(self, key, np.arange(n, dtype=I32))
            elif key in ('n_infections', 'n_breakthroughs'):
                setattr(self, key, np.zeros(n, dtype=I32))
            else:
                setattr(self, key, np.full(n, np.nan, dtype=F32))
        for key in STATES:
            setattr(self, key, np.full(n, key in ('susceptible', 'naive'), dtype=bool))
        for key in VARIANT_STATES:
            setattr(self, key, np.full(n, np.nan, dtype=F32))
        for key in BY_VARIANT_STATES:
            setattr(self, key, np.zeros((nv, n), dtype=bool))
        for key in IMM_STATES:
            setattr(self, key, np.zeros((nv, n), dtype=F32))
        for key in NAB_STATES:
            setattr(self, key, np.zeros(n, dtype=I32 if key == 't_nab_event' else F32))
        for key in VACC_STATES:
            setattr(self, key, np.zeros(n, dtype=I32))
        for key in DATES + DURS:
            setattr(self, key, np.full(n, np.nan, dtype=F32))
        self.infection_log = []
        self._pending = {}  # people.py:115 _pending_quarantine
        self.init_flows()

    def make_naive(self, inds, reset_vx=False):
        """people.py:378-412: states back to the initial ones (vaccination kept),
        variant fields undefined, immunity, NAb and vaccine fields of the
        unvaccinated zeroed, every date (but date_vaccinated) and duration undefined."""
        inds = np.asarray(inds, dtype=np.int64)
        for key in STATES:
            if key in ('susceptible', 'naive'):
                self[key][inds] = True
            elif key != 'vaccinated' or reset_vx:
                self[key][inds] = False
        for key in VARIANT_STATES:
            self[key][inds] = np.nan
        for key in BY_VARIANT_STATES:
            self[key][:, inds] = False
        non_vx = inds if reset_vx else inds[~self.vaccinated[inds]]
        for key in IMM_STATES:
            self[key][:, non_vx] = 0
        for key in NAB_STATES + VACC_STATES:
            self[key][non_vx] = 0
        for key in DATES + DURS:
            if key != 'date_vaccinated' or reset_vx:
                self[key][inds] = np.nan

    def __getitem__(self, key):
        return getattr(self, key)

    def __setitem__(self, key, value):
        setattr(self, key, value)

    def keys(self):
        return (PERSON + STATES + VARIANT_STATES + BY_VARIANT_STATES + IMM_STATES + NAB_STATES
                + VACC_STATES + DATES + DURS)

    def init_flows(self):
        """people.py:121-127."""
        self.flows = {k: 0 for k in FLOWS}
        self.flows_variant = {k: np.zeros(self.pars['n_variants'], dtype=F32) for k in FLOWS_VARIANT}

    # ---------------------------------------------------------------- transitions
    def update_states_pre(self, t):
        """people.py:164-186."""
        self.t = t
        self.is_exp = self.exposed.nonzero()[0]
        self.init_flows()
        self.flows['new_infectious'] += len(self.check_infectious())
        self.flows['new_symptomatic'] += len(self.check_symptomatic())
        self.flows['new_severe'] += len(self.check_severe())
        self.flows['new_critical'] += len(self.check_critical())
        self.flows['new_recoveries'] += len(self.check_recovery())
        self.check_exit_iso()
        _, new_deaths, new_known_deaths = self.check_death()
        self.flows['new_deaths'] += new_deaths
        self.flows['new_known_deaths'] += new_known_deaths
        if self.pars['use_waning']:
            if getattr(self, 'arith', 'reference') == 'gpu':
                from .gpu_arith import check_immunity_gpu
                check_immunity_gpu(self)
            else:
                check_immunity(self)

    def check_inds(self, current, date, filter_inds=None):
        """people.py:211-219."""
        if filter_inds is None:
            not_current = (~current).nonzero()[0]
        else:
            not_current = filter_inds[~current[filter_inds]]
        has_date = not_current[~np.isnan(date[not_current])]
        return has_date[self.t >= date[has_date]]

    def check_infectious(self):
        """people.py:222-232."""
        inds = self.check_inds(self.infectious, self.date_infectious, filter_inds=self.is_exp)
        self.infectious[inds] = True
        self.infectious_variant[inds] = self.exposed_variant[inds]
        for variant in range(self.pars['n_variants']):
            this = inds[self.infectious_variant[inds] == variant]
            self.flows_variant['new_infectious_by_variant'][variant] += len(this)
            self.infectious_by_variant[variant, this] = True
        return inds

    def check_symptomatic(self):
        """people.py:235-239."""
        inds = self.check_inds(self.symptomatic, self.date_symptomatic, filter_inds=self.is_exp)
        self.symptomatic[inds] = True
        return inds

    def check_severe(self):
        """people.py:242-246."""
        inds = self.check_inds(self.severe, self.date_severe, filter_inds=self.is_exp)
        self.severe[inds] = True
        return inds

    def check_critical(self):
        """people.py:249-253."""
        inds = self.check_inds(self.critical, self.date_critical, filter_inds=self.is_exp)
        self.critical[inds] = True
        return inds

    def check_recovery(self, inds=None, filter_inds='is_exp'):
        """people.py:256-291."""
        if isinstance(filter_inds, str) and filter_inds == 'is_exp':
            filter_inds = self.is_exp
        if inds is None:
            inds = self.check_inds(self.recovered, self.date_recovered, filter_inds=filter_inds)
        self.exposed[inds] = False
        self.infectious[inds] = False
        self.symptomatic[inds] = False
        self.severe[inds] = False
        self.critical[inds] = False
        self.recovered[inds] = True
        self.recovered_variant[inds] = self.exposed_variant[inds]
        self.infectious_variant[inds] = np.nan
        self.exposed_variant[inds] = np.nan
        self.exposed_by_variant[:, inds] = False
        self.infectious_by_variant[:, inds] = False
        if self.pars['use_waning']:
            self.susceptible[inds] = True
            self.diagnosed[inds] = False
        return inds

    def check_death(self):
        """people.py:294-312."""
        inds = self.check_inds(self.dead, self.date_dead, filter_inds=self.is_exp)
        self.dead[inds] = True
        diag_inds = inds[self.diagnosed[inds]]
        self.known_dead[diag_inds] = True
        for key in ('susceptible', 'exposed', 'infectious', 'symptomatic', 'severe', 'critical',
                    'known_contact', 'quarantined', 'recovered'):
            self[key][inds] = False
        self.infectious_variant[inds] = np.nan
        self.exposed_variant[inds] = np.nan
        self.recovered_variant[inds] = np.nan
        return inds, len(inds), len(diag_inds)

    def check_exit_iso(self):
        """people.py:368-374."""
        end_inds = self.check_inds(~self.isolated, self.date_end_isolation, filter_inds=None)
        self.isolated[end_inds] = False
        return end_inds

    # ---------------------------------------------------------------- after interventions
    def update_states_post(self):
        """people.py:189-196."""
        self.flows['new_diagnoses'] += len(self.check_diagnosed())
        self.flows['new_quarantined'] += self.check_quar()
        self.flows['new_isolated'] += len(self.check_enter_iso())

    def check_diagnosed(self):
        """people.py:315-332."""
        test_pos_inds = self.check_inds(self.diagnosed, self.date_pos_test, filter_inds=None)
        self.date_pos_test[test_pos_inds] = np.nan
        diag_inds = self.check_inds(self.diagnosed, self.date_diagnosed, filter_inds=None)
        self.diagnosed[diag_inds] = True
        return test_pos_inds

    def check_quar(self):
        """people.py:335-358; ``_pending_quarantine`` maps a start day to (agent, end day) requests."""
        n_quarantined = 0
        for ind, end_day in self._pending.pop(self.t, []):
            if self.quarantined[ind]:
                # Python's max keeps its first argument unless the second compares greater
                cur = self.date_end_quarantine[ind]
                self.date_end_quarantine[ind] = end_day if end_day > cur else cur
            elif not (self.dead[ind] or self.recovered[ind] or self.diagnosed[ind] or self.isolated[ind]):
                self.quarantined[ind] = True
                self.date_quarantined[ind] = self.t
                self.date_end_quarantine[ind] = end_day
                n_quarantined += 1
        diag_inds = (self.quarantined & (self.date_diagnosed == self.t)).nonzero()[0]
        self.date_end_quarantine[diag_inds] = self.t
        end_inds = self.check_inds(~self.quarantined, self.date_end_quarantine, filter_inds=None)
        self.quarantined[end_inds] = False
        return n_quarantined

    def check_enter_iso(self):
        """people.py:361-366."""
        iso_inds = (self.date_diagnosed == self.t).nonzero()[0]
        self.isolated[iso_inds] = True
        self.date_end_isolation[iso_inds] = self.date_recovered[iso_inds]
        return iso_inds

    def test(self, inds, u_sens, u_keep, test_sensitivity=1.0, loss_prob=0.0, test_delay=0):
        """people.py:589-617. ``u_sens(is_infectious)`` and ``u_keep(not_diagnosed)``
        give the uniforms of the sensitivity and loss-to-follow-up trials."""
        inds = np.unique(inds)
        self.tested[inds] = True
        self.date_tested[inds] = self.t
        is_infectious = inds[self.infectious[inds]]
        pos_test = u_sens(is_infectious) < test_sensitivity
        is_inf_pos = is_infectious[pos_test]
        not_diagnosed = is_inf_pos[np.isnan(self.date_diagnosed[is_inf_pos])]
        not_lost = u_keep(not_diagnosed) < 1.0 - loss_prob
        final_inds = not_diagnosed[not_lost]
        self.date_diagnosed[final_inds] = self.t + test_delay
        self.date_pos_test[final_inds] = self.t
        return final_inds

    def schedule_quarantine(self, inds, start_date=None, period=None):
        """people.py:620-640."""
        start_date = self.t if start_date is None else int(start_date)
        period = self.pars['quar_period'] if period is None else int(period)
        for ind in inds:
            self._pending.setdefault(start_date, []).append((ind, start_date + period))

    # ---------------------------------------------------------------- infection
    def infect(self, inds, hosp_max=None, icu_max=None, source=None, layer=None, variant=0,
               draws=None):
        """people.py:435-586; ``draws`` is a TableDraws or SequentialDraws."""
        inds = np.asarray(inds)
        if len(inds) == 0:
            return inds
        inds, unique = np.unique(inds, return_index=True)
        if source is not None:
            source = np.asarray(source)[unique]
        keep = self.susceptible[inds]
        inds = inds[keep]
        if source is not None:
            source = source[keep]
        draws.begin(inds)

        pars = self.pars
        variant_keys = ['rel_symp_prob', 'rel_severe_prob', 'rel_crit_prob', 'rel_death_prob']
        infect_pars = {k: pars[k] for k in variant_keys}
        variant_label = pars['variant_map'][variant]
        if variant:
            for k in variant_keys:
                infect_pars[k] *= pars['variant_pars'][variant_label][k]
        durpars = pars['dur']

        breakthrough_inds = inds[self.peak_nab[inds].nonzero()[0]]
        if len(breakthrough_inds):
            no_prior = self.n_breakthroughs[breakthrough_inds] == 0
            self.rel_trans[breakthrough_inds[no_prior]] *= pars['trans_redux']

        n_infections = len(inds)
        self.susceptible[inds] = False
        self.naive[inds] = False
        self.recovered[inds] = False
        self.diagnosed[inds] = False
        self.exposed[inds] = True
        self.n_infections[inds] += 1
        self.n_breakthroughs[breakthrough_inds] += 1
        self.exposed_variant[inds] = variant
        self.exposed_by_variant[variant, inds] = True
        self.flows['new_infections'] += n_infections
        self.flows['new_reinfections'] += int((~np.isnan(self.date_recovered[inds])).sum())
        self.flows_variant['new_infections_by_variant'][variant] += n_infections

        for i, target in enumerate(inds):
            self.infection_log.append(dict(source=source[i] if source is not None else None,
                                           target=int(target), date=self.t, layer=layer,
                                           variant=variant_label))

        self.dur_exp2inf[inds] = draws.normal(ph.N_EXP2INF, inds, durpars['exp2inf'])
        self.date_exposed[inds] = self.t
        self.date_infectious[inds] = self.dur_exp2inf[inds] + self.t
        for key in ('date_symptomatic', 'date_severe', 'date_critical', 'date_diagnosed',
                    'date_recovered'):
            self[key][inds] = np.nan

        symp_probs = infect_pars['rel_symp_prob'] * self.symp_prob[inds] * (1 - self.symp_imm[variant, inds])
        is_symp = draws.uniform(ph.U_SYMP, inds) < symp_probs
        symp_inds = inds[is_symp]
        asymp_inds = inds[~is_symp]
        self.flows_variant['new_symptomatic_by_variant'][variant] += len(symp_inds)

        dur_asym2rec = draws.normal(ph.N_FINAL, asymp_inds, durpars['asym2rec'])
        self.date_recovered[asymp_inds] = self.date_infectious[asymp_inds] + dur_asym2rec
        self.dur_disease[asymp_inds] = self.dur_exp2inf[asymp_inds] + dur_asym2rec

        self.dur_inf2sym[symp_inds] = draws.normal(ph.N_INF2SYM, symp_inds, durpars['inf2sym'])
        self.date_symptomatic[symp_inds] = self.date_infectious[symp_inds] + self.dur_inf2sym[symp_inds]
        sev_probs = infect_pars['rel_severe_prob'] * self.severe_prob[symp_inds] * (1 - self.sev_imm[variant, symp_inds])
        is_sev = draws.uniform(ph.U_SEV, symp_inds) < sev_probs
        sev_inds = symp_inds[is_sev]
        mild_inds = symp_inds[~is_sev]
        self.flows_variant['new_severe_by_variant'][variant] += len(sev_inds)

        dur_mild2rec = draws.normal(ph.N_FINAL, mild_inds, durpars['mild2rec'])
        self.date_recovered[mild_inds] = self.date_symptomatic[mild_inds] + dur_mild2rec
        self.dur_disease[mild_inds] = self.dur_exp2inf[mild_inds] + self.dur_inf2sym[mild_inds] + dur_mild2rec

        self.dur_sym2sev[sev_inds] = draws.normal(ph.N_SYM2SEV, sev_inds, durpars['sym2sev'])
        self.date_severe[sev_inds] = self.date_symptomatic[sev_inds] + self.dur_sym2sev[sev_inds]
        crit_probs = infect_pars['rel_crit_prob'] * self.crit_prob[sev_inds] * (pars['no_hosp_factor'] if hosp_max else 1.)
        is_crit = draws.uniform(ph.U_CRIT, sev_inds) < crit_probs
        crit_inds = sev_inds[is_crit]
        non_crit_inds = sev_inds[~is_crit]

        dur_sev2rec = draws.normal(ph.N_FINAL, non_crit_inds, durpars['sev2rec'])
        self.date_recovered[non_crit_inds] = self.date_severe[non_crit_inds] + dur_sev2rec
        self.dur_disease[non_crit_inds] = (self.dur_exp2inf[non_crit_inds] + self.dur_inf2sym[non_crit_inds]
                                           + self.dur_sym2sev[non_crit_inds] + dur_sev2rec)

        self.dur_sev2crit[crit_inds] = draws.normal(ph.N_SEV2CRIT, crit_inds, durpars['sev2crit'])
        self.date_critical[crit_inds] = self.date_severe[crit_inds] + self.dur_sev2crit[crit_inds]
        death_probs = infect_pars['rel_death_prob'] * self.death_prob[crit_inds] * (pars['no_icu_factor'] if icu_max else 1.)
        is_dead = draws.uniform(ph.U_DEATH, crit_inds) < death_probs
        dead_inds = crit_inds[is_dead]
        alive_inds = crit_inds[~is_dead]

        dur_crit2rec = draws.normal(ph.N_FINAL, alive_inds, durpars['crit2rec'])
        self.date_recovered[alive_inds] = self.date_critical[alive_inds] + dur_crit2rec
        self.dur_disease[alive_inds] = (self.dur_exp2inf[alive_inds] + self.dur_inf2sym[alive_inds]
                                        + self.dur_sym2sev[alive_inds] + self.dur_sev2crit[alive_inds] + dur_crit2rec)

        dur_crit2die = draws.normal(ph.N_FINAL, dead_inds, durpars['crit2die'])
        self.date_dead[dead_inds] = self.date_critical[dead_inds] + dur_crit2die
        self.dur_disease[dead_inds] = (self.dur_exp2inf[dead_inds] + self.dur_inf2sym[dead_inds]
                                       + self.dur_sym2sev[dead_inds] + self.dur_sev2crit[dead_inds] + dur_crit2die)
        self.date_recovered[dead_inds] = np.nan

        if pars['use_waning']:
            symp = dict(asymp=asymp_inds, mild=mild_inds, sev=sev_inds)
            update_peak_nab(self, inds, nab_pars=pars, symp=symp, draws=draws)
        return inds


# -------------------------------------------------------------------- immunity
def update_peak_nab(people, inds, nab_pars, symp=None, draws=None):
    """covasim/immunity.py:138-202 (natural-infection branch)."""
    pars = people.pars
    has_nabs = people.nab[inds] > 0
    no_prior_nab_inds = inds[~has_nabs]
    prior_nab_inds = inds[has_nabs]
    if len(prior_nab_inds):
        people.peak_nab[prior_nab_inds] *= nab_pars['nab_boost']
    if len(no_prior_nab_inds):
        init_nab = draws.normal(ph.N_NAB, no_prior_nab_inds, nab_pars['nab_init'])
        if getattr(people, 'arith', 'reference') == 'gpu':
            from .gpu_arith import exp2_ff
            no_prior_nab = exp2_ff(init_nab)  # 2**init in float-float, as the GPU forms it
        else:
            no_prior_nab = 2 ** init_nab
        if symp is not None:
            prior_symp = np.full(pars['pop_size'], np.nan)
            prior_symp[symp['asymp']] = pars['rel_imm_symp']['asymp']
            prior_symp[symp['mild']] = pars['rel_imm_symp']['mild']
            prior_symp[symp['sev']] = pars['rel_imm_symp']['severe']
            prior_symp[prior_nab_inds] = np.nan
            prior_symp = prior_symp[~np.isnan(prior_symp)]
            norm_factor = 1 + nab_pars['nab_eff']['alpha_inf_diff']
            no_prior_nab = no_prior_nab * prior_symp * norm_factor
        people.peak_nab[no_prior_nab_inds] = no_prior_nab
    people.t_nab_event[inds] = people.t


def update_nab(people, inds):
    """covasim/immunity.py:205-213."""
    t_since_boost = people.t - people.t_nab_event[inds]
    people.nab[inds] += people.pars['nab_kin'][t_since_boost] * people.peak_nab[inds]
    people.nab[inds] = np.where(people.nab[inds] < 0, 0, people.nab[inds])
    people.nab[inds] = np.where(people.nab[inds] > people.peak_nab[inds], people.peak_nab[inds], people.nab[inds])


def calc_VE(nab, ax, pars):
    """covasim/immunity.py:216-247."""
    if ax == 'sus':
        alpha, beta = pars['alpha_inf'], pars['beta_inf']
    elif ax == 'symp':
        alpha, beta = pars['alpha_symp_inf'], pars['beta_symp_inf']
    else:
        alpha, beta = pars['alpha_sev_symp'], pars['beta_sev_symp']
    exp_lo = np.exp(alpha) * nab ** beta
    return exp_lo / (1 + exp_lo)


def check_immunity(people, variants=None):
    """covasim/immunity.py:303-350 (natural and vaccine immunity, float64 math)."""
    pars = people.pars
    nab_eff = pars['nab_eff']
    if variants is None:
        variants = range(pars['n_variants'])
    n = people.n
    for variant in variants:
        natural_imm = np.zeros(n)
        vaccine_imm = np.zeros(n)
        with np.errstate(invalid='ignore'):
            was_inf = (people.t >= people.date_recovered).nonzero()[0]
        recovered_variant = people.recovered_variant[was_inf]
        immunity = pars['immunity'][variant, :]
        natural_imm[was_inf] = immunity[recovered_variant.astype(int)]
        is_vacc = people.vaccinated.nonzero()[0]
        vacc_source = people.vaccine_source[is_vacc]
        if len(is_vacc) and len(pars['vaccine_pars']):
            vx_pars, vx_map = pars['vaccine_pars'], pars['vaccine_map']
            var_key = pars['variant_map'][variant]
            imm_arr = np.zeros(max(vx_map.keys()) + 1)
            for num, key in vx_map.items():
                imm_arr[num] = vx_pars[key][var_key]
            vaccine_imm[is_vacc] = imm_arr[vacc_source]
        imm = np.maximum(natural_imm, vaccine_imm)
        effective_nabs = people.nab * imm
        people.sus_imm[variant, :] = calc_VE(effective_nabs, 'sus', nab_eff)
        people.symp_imm[variant, :] = calc_VE(effective_nabs, 'symp', nab_eff)
        people.sev_imm[variant, :] = calc_VE(effective_nabs, 'sev', nab_eff)


def nab_growth_decay(length, growth_time, decay_rate1, decay_time1, decay_rate2, decay_time2):
    """covasim/immunity.py:406-448."""
    def f1(t, growth_time):
        return (1 / growth_time) * t

    def f2(t, decay_time1, decay_time2, decay_rate1, decay_rate2):
        decay_rate = np.full(len(t), fill_value=decay_rate1)
        decay_rate[(t > decay_time2).nonzero()[0]] = decay_rate2
        slowing = (1 / (decay_time2 - decay_time1)) * (decay_rate1 - decay_rate2)
        mid = ((t > decay_time1) * (t <= decay_time2)).nonzero()[0]
        decay_rate[mid] = decay_rate1 - slowing * np.arange(len(mid), dtype=I32)
        titre = np.zeros(len(t))
        for i in range(1, len(t)):
            titre[i] = titre[i - 1] + decay_rate[i]
        return np.exp(-titre)

    if decay_time2 < decay_time1:
        raise ValueError('Decay time 2 must be larger than decay time 1')
    length = length + 1
    t1 = np.arange(growth_time, dtype=I32)
    t2 = np.arange(length - growth_time, dtype=I32)
    y = np.concatenate([f1(t1, growth_time), f2(t2, decay_time1, decay_time2, decay_rate1, decay_rate2)])
    return np.diff(y)[0:length]
