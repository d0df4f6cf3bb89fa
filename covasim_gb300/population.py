"""Synthetic populations (random and hybrid), vectorised on the host.

Same distributions as Covasim 3.1.7's generators (covasim/population.py):
ages from the default age table (population.py:143-226), random layers with
round(Poisson(n)/2) partners per agent drawn uniformly (population.py:241-284),
household clusters of Poisson(h) size with all pairs inside each cluster
(population.py:287-329), and the hybrid school/work/community layers
(population.py:332-364). Draws come from a numpy ``Generator`` (PCG64); the
loops over agents of the reference become array operations. Population
building runs once per sim, before the day loop.
"""
import numpy as np

from . import defaults as cvd

__all__ = ['make_randpop', 'make_random_contacts', 'make_microstructured_contacts', 'make_hybrid_contacts',
           'sample_ages']


def _rng(rng):
    return rng if isinstance(rng, np.random.Generator) else np.random.default_rng(rng)


def sample_ages(pop_size, rng, age_data=None):
    """population.py:196-204: a bin by its weight, then uniform within the bin."""
    rng = _rng(rng)
    age_data = cvd.default_age_data if age_data is None else np.asarray(age_data, dtype=float)
    lo = age_data[:, 0]
    rng_ = age_data[:, 1] + 1 - lo
    prob = age_data[:, 2] / age_data[:, 2].sum()
    bins = np.searchsorted(np.cumsum(prob), rng.random(pop_size))
    bins = np.minimum(bins, len(prob) - 1)
    return lo[bins] + rng_[bins] * rng.random(pop_size)


def make_random_contacts(pop_size, n, rng=None, dispersion=None, mapping=None):
    """population.py:241-284: round(Poisson(n)/2) (or negative-binomial) uniform partners per agent.

    Returns dict(p1, p2) with p1 sorted ascending.
    """
    rng = _rng(rng)
    pop_size = int(pop_size)
    if dispersion is None:
        counts = rng.poisson(n, pop_size)
    else:
        counts = rng.negative_binomial(n=dispersion, p=dispersion / (n + dispersion), size=pop_size)
    counts = np.round(counts / 2.0).astype(np.int64)
    p1 = np.repeat(np.arange(pop_size, dtype=np.int64), counts)
    p2 = rng.integers(0, pop_size, len(p1)) if pop_size else np.zeros(0, dtype=np.int64)
    if mapping is not None:
        mapping = np.asarray(mapping, dtype=np.int64)
        p1, p2 = mapping[p1], mapping[p2]
    return dict(p1=p1.astype(cvd.default_int), p2=p2.astype(cvd.default_int))


def make_microstructured_contacts(pop_size, cluster_size, rng=None):
    """population.py:287-329: consecutive clusters of Poisson(cluster_size) agents,
    every pair inside a cluster once (source < target)."""
    rng = _rng(rng)
    pop_size = int(pop_size)
    if pop_size == 0:
        return dict(p1=np.zeros(0, cvd.default_int), p2=np.zeros(0, cvd.default_int))
    chunks, total = [], 0
    mean = max(float(cluster_size), 0.5)
    while total < pop_size:
        draw = rng.poisson(cluster_size, size=int((pop_size - total) / mean * 1.1) + 64)
        chunks.append(draw)
        total += int(draw.sum())
    sizes = np.concatenate(chunks).astype(np.int64)
    cs = np.cumsum(sizes)
    k = int(np.searchsorted(cs, pop_size))  # first cluster reaching the population size
    sizes = sizes[:k + 1].copy()
    sizes[-1] -= int(cs[k]) - pop_size
    sizes = sizes[sizes > 0]
    starts = np.cumsum(sizes) - sizes
    cluster = np.repeat(np.arange(len(sizes)), sizes)
    agent = np.arange(pop_size, dtype=np.int64)
    n_targets = (starts + sizes)[cluster] - agent - 1
    p1 = np.repeat(agent, n_targets)
    group_start = np.cumsum(n_targets) - n_targets
    pos = np.arange(len(p1), dtype=np.int64) - np.repeat(group_start, n_targets)
    p2 = p1 + 1 + pos
    return dict(p1=p1.astype(cvd.default_int), p2=p2.astype(cvd.default_int))


def make_hybrid_contacts(pop_size, ages, contacts, rng=None, school_ages=None, work_ages=None):
    """population.py:332-364: households (h), community (c), school (s), work (w)."""
    rng = _rng(rng)
    contacts = {**dict(h=4, s=20, w=20, c=20), **(contacts or {})}
    school_ages = [6, 22] if school_ages is None else school_ages
    work_ages = [22, 65] if work_ages is None else work_ages
    ages = np.asarray(ages)
    out = {}
    out['h'] = make_microstructured_contacts(pop_size, contacts['h'], rng)
    out['c'] = make_random_contacts(pop_size, contacts['c'], rng)
    s_inds = np.nonzero((ages >= school_ages[0]) * (ages < school_ages[1]))[0]
    w_inds = np.nonzero((ages >= work_ages[0]) * (ages < work_ages[1]))[0]
    out['s'] = make_random_contacts(len(s_inds), contacts['s'], rng, mapping=s_inds)
    out['w'] = make_random_contacts(len(w_inds), contacts['w'], rng, mapping=w_inds)
    return out


def make_randpop(pars, rng=None, microstructure=None, sex_ratio=0.5):
    """population.py:143-226: uid/age/sex and the contact layers of a random or hybrid population."""
    rng = _rng(rng if rng is not None else pars.get('rand_seed', 0))
    pop_size = int(pars['pop_size'])
    microstructure = microstructure or pars['pop_type']
    ages = sample_ages(pop_size, rng)
    sexes = rng.binomial(1, sex_ratio, pop_size)
    if microstructure == 'random':
        contacts = {lkey: make_random_contacts(pop_size, n, rng) for lkey, n in pars['contacts'].items()}
    elif microstructure == 'hybrid':
        contacts = make_hybrid_contacts(pop_size, ages, pars['contacts'], rng)
    else:
        raise NotImplementedError(f'Microstructure type "{microstructure}" not found; choices are random or hybrid')
    return dict(uid=np.arange(pop_size, dtype=cvd.default_int), age=ages, sex=sexes, contacts=contacts,
                layer_keys=list(pars['contacts'].keys()))


def set_prognoses(age, pars, rng):
    """people.py:139-161: per-agent prognosis probabilities and rel_trans/rel_sus from age."""
    rng = _rng(rng)
    progs = pars['prognoses']
    inds = np.digitize(age, progs['age_cutoffs']) - 1
    out = {}
    out['symp_prob'] = progs['symp_probs'][inds].astype(cvd.default_float)
    out['severe_prob'] = (progs['severe_probs'][inds] * progs['comorbidities'][inds]).astype(cvd.default_float)
    out['crit_prob'] = progs['crit_probs'][inds].astype(cvd.default_float)
    out['death_prob'] = progs['death_probs'][inds].astype(cvd.default_float)
    out['rel_sus'] = progs['sus_ORs'][inds].astype(cvd.default_float)
    bd = pars['beta_dist']
    if bd['dist'] == 'neg_binomial':
        step = bd.get('step', 1)
        nbn_n = bd['par2']
        nbn_p = bd['par2'] / (bd['par1'] / step + bd['par2'])
        draws = rng.negative_binomial(n=nbn_n, p=nbn_p, size=len(inds)) * step
    elif bd['dist'] in ('lognormal', 'lognorm'):
        m, s = bd['par1'], bd['par2']
        mu = np.log(m ** 2 / np.sqrt(s ** 2 + m ** 2))
        sg = np.sqrt(np.log(s ** 2 / m ** 2 + 1))
        draws = rng.lognormal(mu, sg, len(inds))
    elif bd['dist'] in ('uniform', 'unif'):
        draws = rng.uniform(bd['par1'], bd['par2'], len(inds))
    elif bd['dist'] in ('normal', 'norm'):
        draws = rng.normal(bd['par1'], bd['par2'], len(inds))
    else:
        raise NotImplementedError(f'beta_dist "{bd["dist"]}"')
    out['rel_trans'] = (progs['trans_ORs'][inds] * draws).astype(cvd.default_float)
    return out
