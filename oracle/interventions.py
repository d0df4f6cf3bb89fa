"""CPU restatement of Covasim 3.1.7's testing and contact-tracing interventions.

TEST INFRASTRUCTURE ONLY. The product never imports this module; tests import
it as the checker.

``TestProb`` restates ``test_prob`` (covasim/interventions.py:858-981) and
``ContactTracing`` restates ``contact_tracing`` (covasim/interventions.py:984-1145),
for the options the GPU path supports (swab delays, ILI prevalence, fixed
subtargets and tracing capacity). Their random draws come
from the oracle sim: the numpy MT19937 stream in the reference's call order
(``rng='mt'``), or Philox keyed by (agent, day) and (agent, layer, day) like
the CUDA library's, with the day's ILI agents from a PCG64 stream keyed by
(seed, 0x111E, day) (``rng='philox'``).
"""
import numpy as np

from . import philox as ph


def get_quar_inds(quar_policy, sim):
    """interventions.py:682-710 (string and number policies)."""
    t = sim.t
    p = sim.people
    if quar_policy is None:
        return np.array([], dtype=np.int64)
    if quar_policy == 'start':
        return (p.date_quarantined == t - 1).nonzero()[0]
    if quar_policy == 'end':
        return (p.date_end_quarantine == t + 1).nonzero()[0]
    if quar_policy == 'both':
        return np.concatenate([(p.date_quarantined == t - 1).nonzero()[0], (p.date_end_quarantine == t + 1).nonzero()[0]])
    if quar_policy == 'daily':
        return p.quarantined.nonzero()[0]
    qp = np.atleast_1d(np.asarray(quar_policy))
    return np.unique(np.concatenate([(p.date_quarantined == t - 1 - q).nonzero()[0] for q in qp]))


def find_contacts(p1, p2, inds):
    """utils.py:131-147 + base.py:1808-1846 (as a sorted array): partners of ``inds``."""
    p1 = np.asarray(p1)
    p2 = np.asarray(p2)
    out = np.concatenate([p2[np.isin(p1, inds)], p1[np.isin(p2, inds)]])
    return np.unique(out).astype(np.int64)


def _active(t, start_day, end_day):
    return not (t < start_day or (end_day is not None and t > end_day))


ILI_TAG = 0x111E


def ili_agents(seed, t, n, n_ili):
    """Philox mode: the n_ili distinct agents with influenza-like symptoms on day t
    (interventions.py:942-947 draws them with cvu.choose), from a PCG64 stream keyed
    by (seed, 0x111E, t): they do not depend on the sim's state."""
    rng = np.random.Generator(np.random.PCG64([int(seed) & 0xFFFFFFFFFFFFFFFF, ILI_TAG, int(t)]))
    return np.sort(rng.choice(int(n), int(n_ili), replace=False)).astype(np.int64)


def swab_pdf(dist=None, par1=None, par2=None):
    """get_pdf (utils.py:240-268): the frozen scipy distribution of the delay from
    symptom onset to swab, or None."""
    import scipy.stats as sps
    if dist in ('None', 'none', None):
        return None
    if dist == 'uniform':
        return sps.uniform(loc=par1, scale=par2)
    if dist == 'lognormal':
        mean = np.log(par1**2 / np.sqrt(par2 + par1**2))
        sigma = np.sqrt(np.log(par2 / par1**2 + 1))
        return sps.lognorm(sigma, loc=-0.5, scale=np.exp(mean))
    raise NotImplementedError(f'The selected distribution "{dist}" is not implemented')


def daily_series(x, npts):
    """process_daily_data (interventions.py:111-147) for a number or a sequence."""
    if isinstance(x, (int, float, np.integer, np.floating)):
        return np.array([x] * npts)
    return np.asarray(x)


class TestProb:
    """interventions.py:858-981 (subtarget a dict of fixed ``inds`` and ``vals``)."""

    __test__ = False  # not a pytest test class

    def __init__(self, symp_prob, asymp_prob=0.0, symp_quar_prob=None, asymp_quar_prob=None, quar_policy=None,
                 subtarget=None, ili_prev=None, sensitivity=1.0, loss_prob=0.0, test_delay=0, start_day=0,
                 end_day=None, swab_delay=None):
        self.symp_prob = symp_prob
        self.asymp_prob = asymp_prob
        self.symp_quar_prob = symp_quar_prob if symp_quar_prob is not None else symp_prob
        self.asymp_quar_prob = asymp_quar_prob if asymp_quar_prob is not None else asymp_prob
        self.quar_policy = quar_policy if quar_policy else 'start'
        self.subtarget = subtarget
        self.ili_prev = ili_prev
        self.pdf = swab_pdf(**(swab_delay or {}))
        self.sensitivity = sensitivity
        self.loss_prob = loss_prob
        self.test_delay = test_delay
        self.start_day = start_day
        self.end_day = end_day

    def apply(self, sim):
        t = sim.t
        if not _active(t, self.start_day, self.end_day):
            return None
        people = sim.people
        n = sim.n
        symp_inds = people.symptomatic.nonzero()[0]
        symp_prob = self.symp_prob
        if self.pdf:  # the swab delay's distribution (interventions.py:930-938)
            symp_time = (t - people.date_symptomatic[symp_inds]).astype(np.int32)
            inv_count = np.bincount(symp_time) / len(symp_time)
            count = np.nan * np.ones(inv_count.shape)
            count[inv_count != 0] = 1 / inv_count[inv_count != 0]
            symp_prob = np.ones(len(symp_time))
            inds = 1 > (symp_time * self.symp_prob)
            symp_prob[inds] = self.symp_prob / (1 - symp_time[inds] * self.symp_prob)
            symp_prob = self.pdf.pdf(symp_time) * symp_prob * count[symp_time]
        # symptomatics of influenza-like illness, drawn before the tests (interventions.py:941-947)
        ili_inds = np.array([], dtype=np.int64)
        if self.ili_prev is not None:
            ili = daily_series(self.ili_prev, sim.npts)
            rel_t = t - self.start_day
            if rel_t < len(ili):
                n_ili = int(ili[rel_t] * n)
                if sim.rng == 'philox':
                    ili_inds = ili_agents(sim.seed, t, n, n_ili)
                else:  # cvu.choose is a numba function (utils.py:430-443): numba's stream
                    ili_inds = sim.rs_numba.choice(n, n_ili, replace=False)
                ili_inds = np.setdiff1d(ili_inds, symp_inds)
        asymp_inds = np.setdiff1d(np.setdiff1d(np.arange(n), symp_inds), ili_inds)
        quar_test_inds = get_quar_inds(self.quar_policy, sim)
        symp_quar_inds = np.intersect1d(quar_test_inds, symp_inds)
        asymp_quar_inds = np.intersect1d(quar_test_inds, asymp_inds)
        diag_inds = people.diagnosed.nonzero()[0]
        test_probs = np.zeros(n)
        test_probs[symp_inds] = symp_prob
        test_probs[ili_inds] = self.symp_prob
        test_probs[asymp_inds] = self.asymp_prob
        test_probs[symp_quar_inds] = self.symp_quar_prob
        test_probs[asymp_quar_inds] = self.asymp_quar_prob
        if self.subtarget is not None:  # get_subtargets (interventions.py:150-187), fixed inds and vals
            test_probs[np.asarray(self.subtarget['inds'], dtype=np.int64)] = self.subtarget['vals']
        test_probs[diag_inds] = 0.0
        if sim.rng == 'philox':
            u_test, u_sens, u_keep = ph.test_draws(sim.k0, sim.k1, t, np.arange(n))
            test_inds = (u_test < test_probs).nonzero()[0]
            sens = lambda inds: u_sens[inds]  # noqa: E731
            keep = lambda inds: u_keep[inds]  # noqa: E731
        else:
            rs = sim.rs_numpy
            test_inds = (rs.random_sample(n) < test_probs).nonzero()[0]
            sens = keep = lambda inds: rs.random_sample(len(inds))  # noqa: E731
        people.test(test_inds, sens, keep, test_sensitivity=self.sensitivity, loss_prob=self.loss_prob,
                    test_delay=self.test_delay)
        sim.results['new_tests'][t] += len(test_inds)
        return test_inds


class ContactTracing:
    """interventions.py:984-1145."""

    def __init__(self, trace_probs=None, trace_time=None, start_day=0, end_day=None, presumptive=False,
                 quar_period=None, capacity=None):
        self.trace_probs = trace_probs
        self.trace_time = trace_time
        self.start_day = start_day
        self.end_day = end_day
        self.presumptive = presumptive
        self.quar_period = quar_period
        self.capacity = capacity

    def initialize(self, sim):
        """interventions.py:1023-1041."""
        if self.trace_probs is None:
            self.trace_probs = 1.0
        if self.trace_time is None:
            self.trace_time = 0.0
        if self.quar_period is None:
            self.quar_period = sim.pars['quar_period']
        if np.isscalar(self.trace_probs):
            self.trace_probs = {k: self.trace_probs for k in sim.layer_keys}
        if np.isscalar(self.trace_time):
            self.trace_time = {k: self.trace_time for k in sim.layer_keys}

    def apply(self, sim):
        t = sim.t
        if not _active(t, self.start_day, self.end_day):
            return None
        people = sim.people
        if not self.presumptive:
            trace_inds = (people.date_diagnosed == t).nonzero()[0]
        else:
            just_tested = (people.date_tested == t).nonzero()[0]
            trace_inds = just_tested[people.exposed[just_tested]]
        if self.capacity is not None:  # interventions.py:1074-1078
            capacity = int(self.capacity / sim.rescale_vec[t])
            if len(trace_inds) > capacity:
                if sim.rng == 'philox':  # the capacity cases with the smallest keys
                    keys = ph.capacity_keys(sim.k0, sim.k1, t, trace_inds)
                    trace_inds = np.sort(trace_inds[np.argsort(keys, kind='stable')[:capacity]])
                else:
                    trace_inds = sim.rs_numpy.choice(trace_inds, capacity, replace=False)
        if not len(trace_inds):
            return {}
        contacts = {}
        for lkey, prob in self.trace_probs.items():
            if prob == 0:
                continue
            if lkey in getattr(sim, 'dyn_tables', {}):  # philox mode: the traced agents' own lists
                traceable = np.unique(sim.dynamic_lists(lkey, trace_inds)[3])
            else:
                layer = sim.contacts[lkey]
                traceable = find_contacts(layer['p1'], layer['p2'], trace_inds)
            if len(traceable):
                if sim.rng == 'philox':
                    u = ph.trace_draws(sim.k0, sim.k1, t, sim.layer_keys.index(lkey), traceable)
                else:
                    u = sim.rs_numpy.random_sample(len(traceable))
                contacts.setdefault(self.trace_time[lkey], []).extend(traceable[(u < prob).nonzero()[0]])
        is_dead = people.dead.nonzero()[0]
        for trace_time, inds in contacts.items():
            contact_inds = np.setdiff1d(np.asarray(inds, dtype=np.int64), is_dead)
            people.known_contact[contact_inds] = True
            people.date_known_contact[contact_inds] = np.fmin(people.date_known_contact[contact_inds], t + trace_time)
            people.schedule_quarantine(contact_inds, start_date=t + trace_time, period=self.quar_period - trace_time)
        return contacts
