"""The likelihood passes and their adjoint (covasim_gb300.adjoint): gradients
of the transmission log-likelihood and of the expected daily infections
with respect to beta, the layer betas and the change_beta multipliers,
against float64 central finite differences on the run's fixed states, against
torch autograd on the oracle's exposures, and a calibration of beta."""
import numpy as np
import pytest
import torch

import covasim_gb300 as cv
from covasim_gb300.adjoint import LikelihoodRun, SimLikelihood, fit_parameters
from oracle import philox as ph
from oracle.kernels import compute_trans_sus
from common import oracle_for

pytestmark = pytest.mark.gpu


def make_run(n=6000, days=40, seed=3, every=10, dyn=True):
    pars = dict(pop_type='hybrid', pop_size=n, n_days=days, rand_seed=seed, pop_infected=40,
                interventions=[cv.change_beta(days=[15, 25], changes=[0.6, 0.8])])
    if dyn:
        pars['dynam_layer'] = dict(h=0, s=0, w=0, c=1)
    sim = cv.Sim(pars)
    sim.initialize()
    return sim, LikelihoodRun(sim, checkpoint_every=every)


def test_forward_reproduces_plain_run_and_checkpoints_are_exact():
    sim, run = make_run()
    ll, expected = run.forward(run.params.theta0)
    plain = cv.Sim(dict(sim.pars)).run().raw_results()
    got = sim.state.results(0)
    for k in ('new_infections', 'n_exposed', 'new_recoveries'):
        np.testing.assert_array_equal(got[k], plain[k], err_msg=k)
    again = run.recompute(grad=True)  # checkpointed recomputation sees the same states
    np.testing.assert_allclose(again['ll'], run.last['ll'], rtol=1e-12, atol=1e-9)
    np.testing.assert_allclose(again['expected'], run.last['expected'], rtol=1e-12, atol=1e-9)
    for k in ('new_infections', 'n_exposed', 'new_recoveries'):
        np.testing.assert_array_equal(sim.state.results(0)[k], plain[k], err_msg=k)
    assert np.isfinite(ll) and ll < 0 and expected.sum() > 0
    # expected infections track the realised ones
    real = got['new_infections']
    assert abs(expected.sum() - real.sum()) < 0.1 * real.sum()


@pytest.mark.parametrize('objective', ['ll', 'expected'])
def test_gradients_match_central_finite_differences(objective):
    sim, run = make_run()
    th = run.params.theta0
    run.forward(th)
    w = np.random.default_rng(0).uniform(0.5, 1.5, run.npts)

    def f(theta):
        ll, e = run.loglik(theta)
        return ll if objective == 'll' else float(w @ e)

    g = run.backward(1.0, np.zeros(run.npts)) if objective == 'll' else run.backward(0.0, w)
    h = 1e-4
    for k, name in enumerate(run.params.names):
        tp, tm = th.copy(), th.copy()
        tp[k] *= 1 + h
        tm[k] *= 1 - h
        fd = (f(tp) - f(tm)) / (2 * h * th[k])
        assert abs(g[k] - fd) <= 1e-4 * abs(fd) + 1e-9, (name, g[k], fd)


def torch_reference(sim, run, theta):
    """LL and expected[t] on the oracle's exposures (same Philox draws as the GPU
    run), as torch float64 functions of theta."""
    orc = oracle_for(sim)
    days = []
    p = sim.pars

    def hook(o, t, vl):
        pp = o.people
        recs = []
        for v in range(p['n_variants']):
            beta32 = np.float32(o.pars['beta'] * p['rel_beta'] * p['variant_pars'][p['variant_map'][v]]['rel_beta'])
            inf_v = pp.infectious & (pp.infectious_variant == v)
            for li, lk in enumerate(o.layer_keys):
                qf, isf, af = (np.float32(p['quar_factor'][lk]), np.float32(p['iso_factor'][lk]),
                               np.float32(p['asymp_factor']))
                rt32, rs32 = compute_trans_sus(pp.rel_trans, pp.rel_sus, inf_v, pp.susceptible,
                                               np.float32(o.pars['beta_layer'][lk]), vl, pp.symptomatic,
                                               pp.isolated, pp.quarantined, af, isf, qf, pp.sus_imm[v])
                rte = pp.rel_trans.astype(np.float64) * np.where(pp.quarantined, qf, 1.0) \
                    * np.where(pp.symptomatic, 1.0, af) * np.where(pp.isolated, isf, 1.0) * vl.astype(np.float64)
                rse = pp.rel_sus.astype(np.float64) * np.where(pp.quarantined, qf, 1.0) \
                    * (1.0 - pp.sus_imm[v].astype(np.float64))
                # every exposed direction with its outcome as the GPU draws it (a dynamic
                # layer: the entries of the sources' lists, thinned)
                s, g, d, eid, eb, p32, hit = o.exposures(li, v, beta32, rt32, rs32)
                m = (p32 > 0) & inf_v[s] & pp.susceptible[g]
                recs.append(dict(l=li, v=v, g=g[m], infected=hit[m],
                                 c=eb[m].astype(np.float64) * rte[s[m]] * rse[g[m]]))
        days.append(recs)

    orc.exposure_hook = hook
    orc.run()
    A = torch.from_numpy(run.params.A)
    rb = torch.from_numpy(run.params._rb)
    logF = torch.einsum('tlk,k->tl', A, torch.log(theta))
    ll = torch.zeros((), dtype=torch.float64)
    expected = []
    for t, recs in enumerate(days):
        logq = torch.zeros(sim['pop_size'], dtype=torch.float64)
        for r in recs:
            pr = torch.exp(logF[t, r['l']]) * rb[r['v']] * torch.from_numpy(r['c'])
            inf = torch.from_numpy(r['infected'])
            capped = pr >= 1  # certain transmission (u < p for every u): log p = 0, no sensitivity
            ps = torch.where(capped, torch.full_like(pr, 0.5), pr)
            zero = torch.zeros_like(pr)
            ll = ll + torch.where(inf, torch.where(capped, zero, torch.log(ps)), torch.log1p(-ps)).sum()
            logq = logq.index_add(0, torch.from_numpy(r['g']),
                                  torch.where(capped, torch.full_like(pr, -np.inf), torch.log1p(-ps)))
        expected.append((1 - torch.exp(logq[logq != 0])).sum())
    return ll, torch.stack(expected)


def test_gradients_match_torch_autograd_on_the_oracle():
    sim, run = make_run(n=2500, days=30, seed=5, every=7)
    th0 = run.params.theta0
    theta = torch.tensor(th0, dtype=torch.float64, requires_grad=True)
    ll_t, e_t = torch_reference(sim, run, theta)
    w = torch.from_numpy(np.random.default_rng(1).uniform(0.5, 1.5, run.npts))
    (g_ll_t,) = torch.autograd.grad(ll_t, theta, retain_graph=True)
    (g_e_t,) = torch.autograd.grad((w * e_t).sum(), theta)
    ll, e = run.forward(th0)
    assert abs(ll - ll_t.item()) <= 1e-9 * abs(ll_t.item())
    np.testing.assert_allclose(e, e_t.detach().numpy(), rtol=1e-9, atol=1e-9)
    np.testing.assert_allclose(run.backward(1.0, np.zeros(run.npts)), g_ll_t.numpy(), rtol=1e-8, atol=1e-9)
    np.testing.assert_allclose(run.backward(0.0, w.numpy()), g_e_t.numpy(), rtol=1e-8, atol=1e-9)


def test_autograd_function_and_calibration_recover_beta():
    target_sim = cv.Sim(pop_type='hybrid', pop_size=30000, n_days=60, rand_seed=21, beta=0.018, pop_infected=60)
    target = target_sim.run().raw_results()['new_infections']
    sim = cv.Sim(pop_type='hybrid', pop_size=30000, n_days=60, rand_seed=22, beta=0.012, pop_infected=60)
    sim.initialize()
    run = LikelihoodRun(sim, which=('beta',))
    theta = torch.tensor(run.params.theta0, dtype=torch.float64, requires_grad=True)
    ll, e = SimLikelihood.apply(theta, run)
    (e.sum() + 0.0 * ll).backward()
    assert theta.grad is not None and theta.grad[0] > 0  # more beta, more expected infections
    fitted, hist = fit_parameters(run, target, fit=('beta',), steps=30, lr=0.08)
    assert abs(fitted[0] - 0.018) < 0.1 * 0.018, hist[-5:]


def test_calibration_to_daily_diagnoses_recovers_beta():
    """Config 4's calibration: beta fitted to the daily diagnoses (test_prob) of a
    sim run at beta = 0.018, through the expected infections convolved with the
    run's infection-to-diagnosis delays, starting from beta = 0.012."""
    tp = dict(symp_prob=0.1)
    base = dict(pop_type='hybrid', pop_size=30000, n_days=80, pop_infected=60)
    target_sim = cv.Sim(dict(base, rand_seed=31, beta=0.018), interventions=[cv.test_prob(**tp)])
    target = target_sim.run().raw_results()['new_diagnoses']
    assert target.sum() > 500
    sim = cv.Sim(dict(base, rand_seed=32, beta=0.012), interventions=[cv.test_prob(**tp)])
    sim.initialize()
    run = LikelihoodRun(sim, which=('beta',))
    fitted, hist = fit_parameters(run, target, fit=('beta',), steps=30, lr=0.08, observe='diagnoses')
    assert abs(fitted[0] - 0.018) < 0.1 * 0.018, hist[-5:]

