"""Populations built on the device (covgpu_pop.cu) against the distributions of
covasim/population.py and people.py:139-161, and a whole sim on such a
population against the oracle."""
import numpy as np
import pytest
import torch
from scipy import stats

import covasim_gb300 as cv
from covasim_gb300 import defaults as cvd, parameters as cvpar
from covasim_gb300.population import make_randpop_device, set_prognoses_device
from test_gpu_sim import compare_runs, oracle_for, RES_KEYS

pytestmark = pytest.mark.gpu


def chi2_p(observed, probs):
    probs = np.asarray(probs, dtype=float)
    keep = probs * observed.sum() >= 5
    obs = np.append(observed[keep], observed[~keep].sum())
    exp = np.append(probs[keep], probs[~keep].sum()) * observed.sum()
    if exp[-1] == 0:
        obs, exp = obs[:-1], exp[:-1]
    return stats.chisquare(obs, exp * obs.sum() / exp.sum()).pvalue


def half_even_pmf(lam, kmax):
    """pmf of round(X / 2) (halves to even) for X ~ Poisson(lam)."""
    x = np.arange(0, 2 * kmax + 2)
    px = stats.poisson.pmf(x, lam)
    h = x // 2 + ((x % 2 == 1) & ((x // 2) % 2 == 1))
    return np.bincount(h, weights=px, minlength=kmax + 2)[:kmax + 1]


def test_ages_sexes_and_random_layer_follow_the_reference_distributions():
    pars = cvpar.make_pars(pop_size=400_000, pop_type='random', contacts=dict(a=20))
    pop = make_randpop_device(pars, seed=11)
    ad = np.asarray(cvd.default_age_data, dtype=float)
    lo, hi = ad[:, 0], ad[:, 1] + 1
    bins = np.searchsorted(hi, pop['age'], side='right')
    assert pop['age'].min() >= 0 and pop['age'].max() < hi[-1]
    assert chi2_p(np.bincount(bins, minlength=len(ad)), ad[:, 2] / ad[:, 2].sum()) > 1e-3
    assert abs(pop['sex'].mean() - 0.5) < 0.005
    p1 = pop['contacts']['a']['p1'].cpu().numpy()
    p2 = pop['contacts']['a']['p2'].cpu().numpy()
    assert np.all(p1[1:] >= p1[:-1]) and p2.min() >= 0 and p2.max() < 400_000
    counts = np.bincount(p1, minlength=400_000)
    pmf = half_even_pmf(20, counts.max() + 5)
    assert chi2_p(np.bincount(counts, minlength=len(pmf))[:len(pmf)], pmf) > 1e-3
    assert chi2_p(np.bincount(p2 * 50 // 400_000, minlength=50), np.full(50, 1 / 50)) > 1e-3


def test_hybrid_households_and_age_layers():
    n = 300_000
    pars = cvpar.make_pars(pop_size=n, pop_type='hybrid')
    pop = make_randpop_device(pars, seed=5)
    age = pop['age']
    h1 = pop['contacts']['h']['p1'].cpu().numpy()
    h2 = pop['contacts']['h']['p2'].cpu().numpy()
    assert np.all(h2 > h1) and np.all(h1[1:] >= h1[:-1])
    # each agent's targets are the next agents of its cluster: p2 - p1 runs 1..k
    first = np.ones(len(h1), dtype=bool)
    first[1:] = h1[1:] != h1[:-1]
    run = np.arange(len(h1)) - np.maximum.accumulate(np.where(first, np.arange(len(h1)), 0))
    assert np.array_equal(h2 - h1, run + 1)
    # cluster sizes: an agent that is no one's target starts a cluster of (its targets + 1)
    is_target = np.zeros(n, dtype=bool)
    is_target[h2] = True
    n_targets = np.bincount(h1, minlength=n)
    sizes = n_targets[~is_target] + 1
    mean_h = pars['contacts']['h']
    pmf = stats.poisson.pmf(np.arange(1, 15), mean_h) / (1 - stats.poisson.pmf(0, mean_h))
    assert chi2_p(np.bincount(sizes[:-1], minlength=15)[1:15], pmf) > 1e-3
    for key, (a0, a1) in (('s', (6, 22)), ('w', (22, 65))):
        m1 = pop['contacts'][key]['p1'].cpu().numpy()
        m2 = pop['contacts'][key]['p2'].cpu().numpy()
        for m in (m1, m2):
            assert np.all((age[m] >= a0) & (age[m] < a1)), key
        members = np.nonzero((age >= a0) & (age < a1))[0]
        counts = np.bincount(m1, minlength=n)[members]
        lam = pars['contacts'][key]
        pmf = half_even_pmf(lam, counts.max() + 5)
        assert chi2_p(np.bincount(counts, minlength=len(pmf))[:len(pmf)], pmf) > 1e-3, key


def test_prognoses_tables_and_rel_trans_distribution():
    n = 500_000
    pars = cvpar.make_pars(pop_size=n, pop_type='random')
    pars['prognoses'] = cvpar.get_prognoses()
    age = torch.linspace(0, 99.9, n, device='cuda')
    out = {k: v.cpu().numpy() for k, v in set_prognoses_device(age, pars, seed=3).items()}
    progs = pars['prognoses']
    inds = np.digitize(age.cpu().numpy(), progs['age_cutoffs']) - 1
    np.testing.assert_array_equal(out['symp_prob'], progs['symp_probs'][inds].astype(np.float32))
    np.testing.assert_array_equal(out['severe_prob'],
                                  (progs['severe_probs'][inds] * progs['comorbidities'][inds]).astype(np.float32))
    np.testing.assert_array_equal(out['rel_sus'], progs['sus_ORs'][inds].astype(np.float32))
    bd = pars['beta_dist']
    mu, k, step = bd['par1'] / bd['step'], bd['par2'], bd['step']
    draws = out['rel_trans'] / progs['trans_ORs'][inds]
    se_mean = np.sqrt(step ** 2 * (mu + mu ** 2 / k) / n)
    assert abs(draws.mean() - bd['par1']) < 4 * se_mean
    var = step ** 2 * (mu + mu ** 2 / k)
    assert abs(draws.var() / var - 1) < 0.05
    counts = np.rint(draws[:200_000].astype(np.float64) / step).astype(np.int64)  # the integer NB draws
    ref = np.random.default_rng(0).negative_binomial(k, k / (mu + k), 200_000)
    assert stats.ks_2samp(counts, ref).pvalue > 1e-3


def test_sim_on_a_device_population_matches_the_oracle_and_is_deterministic():
    pars = dict(pop_type='hybrid', pop_size=4000, n_days=40, rand_seed=8, pop_infected=30,
                dynam_layer=dict(h=0, s=0, w=0, c=1))
    sim = cv.Sim(pars, gpu_population=True)
    sim.initialize()
    orc = oracle_for(sim).run()
    sim.run()
    compare_runs(sim, orc)
    again = cv.Sim(pars, gpu_population=True).run().raw_results()
    for k in RES_KEYS:
        np.testing.assert_array_equal(again[k], sim.raw_results()[k], err_msg=k)


def test_batch_of_device_populations_leaves_them_intact():
    """A batch places each sim's agents at an offset; the caller's device layers must not move."""
    sims = [cv.Sim(pop_type='random', pop_size=n, n_days=20, rand_seed=s, gpu_population=True)
            for n, s in ((3000, 1), (5000, 2))]
    batch = cv.BatchSim(sims).run()
    for k, s in enumerate(sims):
        p2 = s.popdict['contacts']['a']['p2']
        assert int(p2.max()) < s['pop_size']
        single = cv.Sim(dict(s.pars), popdict=s.popdict, person=s._person).run().raw_results()
        np.testing.assert_array_equal(batch.results(k)['new_infections'], single['new_infections'])
