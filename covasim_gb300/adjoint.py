"""Gradients of a simulation's transmission likelihood and expected infections.

For a sim run at parameters theta, every exposed direction source -> target
of day t (infectious source, susceptible target, on some layer l) has the
transmission probability of compute_infections (covasim/utils.py:93-128)

    p = F[t, l, v] * edge beta * rel_trans' * rel_sus'

where F = beta(t) * rel_beta * (variant rel_beta) * beta_layer[l](t) holds every
parameter (covasim/sim.py:626-643) and rel_trans', rel_sus' are the per-agent
factors of compute_trans_sus (utils.py:82-90) without beta_layer. Holding the
run's states and transmission outcomes fixed, the library's likelihood passes
return, per day,

    ll[t]       = sum over infecting directions of log p + others log(1 - p)
    expected[t] = sum over targets of 1 - prod over their directions (1 - p)

and their derivatives with respect to log F[t, l, .] (G[t, l] and H[t, l]).
Each parameter theta_k enters F[t, l] with exponent A[t, l, k] in {0, 1}:
``beta`` on every day and layer, ``beta_layer:<key>`` on its layer, and each
change_beta multiplier (interventions.py:530-586) on the days and layers it
governs. So d/d theta_k = sum over t, l of A[t, l, k] * G[t, l] / theta_k.

``LikelihoodRun`` runs the sim with a state checkpoint every few days and the
gradient accumulators on (with a handful of parameters the sensitivities G and
H cost little beside the run itself), so the backward pass at the forward's
parameters reuses them; a backward or likelihood at other parameters rewinds
to each checkpoint and recomputes its days on the run's fixed states, so
memory stays at one state per checkpoint. ``SimLikelihood`` wraps it as a
``torch.autograd.Function``.
"""
import numpy as np
import torch

from . import _lib as L
from .interventions import change_beta
from .sim import init_infections

__all__ = ['Parameters', 'LikelihoodRun', 'SimLikelihood', 'fit_parameters', 'delay_matrix']


class Parameters:
    """The differentiable parameters of one sim and their day/layer structure.

    Args:
        sim: an initialised ``Sim``
        which: any of 'beta', 'beta_layer', 'change_beta'; the others stay at
            the sim's values
    """

    def __init__(self, sim, which=('beta', 'beta_layer', 'change_beta')):
        spec = sim.spec
        p = sim.pars
        self.npts = T = spec.npts
        self.keys = [ly['key'] for ly in spec.layers]
        nl, nv = len(self.keys), spec.nv
        names = ['beta'] + [f'beta_layer:{k}' for k in self.keys]
        values = [float(p['beta'])] + [float(p['beta_layer'][k]) for k in self.keys]
        kinds = ['beta'] + ['beta_layer'] * nl
        # the change_beta multiplier in force on each day for each target ('overall' or
        # a layer), following change_beta.apply (interventions.py:575-586)
        active = {tgt: np.full(T, -1) for tgt in ['overall'] + self.keys}
        for j, iv in enumerate([iv for iv in sim['interventions'] if isinstance(iv, change_beta)]):
            for day, ch in zip(iv.days, iv.changes):
                k = len(names)
                names.append(f'change_beta[{j}]:day{int(day)}')
                values.append(float(ch))
                kinds.append('change_beta')
                for lkey in iv.orig_betas:
                    if 0 <= int(day) < T:
                        active[lkey][int(day):] = k
        K = len(names)
        A = np.zeros((T, nl, K), dtype=np.float64)
        A[:, :, 0] = 1
        for li in range(nl):
            A[:, li, 1 + li] = 1
        for t in range(T):
            if active['overall'][t] >= 0:
                A[t, :, active['overall'][t]] = 1
            for li, lk in enumerate(self.keys):
                if active[lk][t] >= 0:
                    A[t, li, active[lk][t]] = 1
        self._values0 = np.array(values, dtype=np.float64)
        self._active = active
        self._sel = [i for i, kd in enumerate(kinds) if kd in which]
        self.names = [names[i] for i in self._sel]
        self.theta0 = self._values0[self._sel].copy()
        self.A = A[:, :, self._sel]
        self._rb = np.array([p['rel_beta'] * p['variant_pars'][p['variant_map'][v]]['rel_beta'] for v in range(nv)])

    def _full(self, theta):
        v = self._values0.copy()
        v[self._sel] = np.asarray(theta, dtype=np.float64)
        return v

    def schedules(self, theta):
        """Per-day overall beta and per-layer beta under ``theta``: the products
        change_beta forms (original value times the multiplier in force), so that
        ``theta0`` reproduces the sim's own tables exactly."""
        v = self._full(theta)
        T, nl = self.npts, len(self.keys)
        beta = np.empty(T)
        bl = np.empty((T, nl))
        for t in range(T):
            k = self._active['overall'][t]
            beta[t] = v[0] * v[k] if k >= 0 else v[0]
            for li, lk in enumerate(self.keys):
                k = self._active[lk][t]
                bl[t, li] = v[1 + li] * v[k] if k >= 0 else v[1 + li]
        return beta, bl

    def factor(self, theta):
        """F[t, l, v] = beta(t) * beta_layer[l](t) * rel_beta * variant rel_beta."""
        beta, bl = self.schedules(theta)
        return beta[:, None, None] * bl[:, :, None] * self._rb[None, None, :]

    def chain(self, theta, G):
        """sum over (t, l) of A[t, l, k] * G[t, l] / theta_k."""
        return np.einsum('tlk,tl->k', self.A, G) / np.asarray(theta, dtype=np.float64)


class LikelihoodRun:
    """A sim whose runs report the transmission log-likelihood and expected
    infections per day, with gradients by checkpointed recomputation.

    Args:
        sim: a ``Sim`` (initialised here if needed)
        which: parameters to differentiate (see ``Parameters``)
        checkpoint_every: days between state checkpoints
        use_graph: capture each checkpoint segment in a CUDA graph
    """

    def __init__(self, sim, which=('beta', 'beta_layer', 'change_beta'), checkpoint_every=10, use_graph=True):
        if not sim.initialized:
            sim.initialize()
        if sim.state.hold is not None:
            raise NotImplementedError('likelihood runs do not support dynamic rescaling (pop_scale > 1 with rescale)')
        if sim['variants']:
            raise NotImplementedError('likelihood runs support sims without host-side days (no variants imports)')
        self.sim = sim
        self.state = sim.state
        self.params = Parameters(sim, which)
        self.every = int(checkpoint_every)
        self.use_graph = use_graph
        self.npts = sim.npts
        self.initial = self.state.snapshot()
        self.state.enable_lik(grad=False)
        self.theta = None
        self.checkpoints = []
        self._ck_buffers = []  # checkpoint storage, reused by every forward
        self._grads = None      # G and H of the last forward, at its own parameters

    def _segments(self):
        return [(t0, min(t0 + self.every, self.npts)) for t0 in range(0, self.npts, self.every)]

    def _set_dynamics(self, theta):
        beta, bl = self.params.schedules(theta)
        self.state.set_beta_tables(beta, bl)

    def _read(self, grad):
        lk = self.state.lik
        T = self.npts
        nl = len(self.params.keys)
        out = dict(ll=lk['ll'][0, :T].cpu().numpy().copy(), expected=lk['expected'][0, :T].cpu().numpy().copy())
        if grad:
            out['G'] = lk['g_ll'][0, :T, :nl].cpu().numpy().copy()
            out['H'] = lk['g_exp'][0, :T, :nl].cpu().numpy().copy()
        return out

    def forward(self, theta):
        """Run the sim at ``theta`` (checkpointing); returns (ll, expected[npts])."""
        theta = np.asarray(theta, dtype=np.float64)
        st = self.state
        self.theta = theta.copy()
        self._set_dynamics(theta)
        st.enable_lik(grad=True)
        st.set_lik_factor(self.params.factor(theta))
        st.zero_lik()
        st.restore(self.initial)
        init_infections(st, 0, self.sim.pars)
        self.checkpoints = []
        for k, (t0, t1) in enumerate(self._segments()):
            if k < len(self._ck_buffers):
                self.checkpoints.append(st.checkpoint(into=self._ck_buffers[k]))
            else:
                self._ck_buffers.append(st.checkpoint())
                self.checkpoints.append(self._ck_buffers[k])
            st.run_days(t0, t1, open_prev=t0 > 0, close_last=t1 == self.npts, use_graph=self.use_graph)
        if st.status():
            raise L.CovgpuError('likelihood run', st.status())
        out = self._read(grad=True)
        self._grads = out
        self.last = out  # per-day ll and expected of this run
        return float(out['ll'].sum()), out['expected']

    def recompute(self, theta_eval=None, grad=True):
        """Rerun every checkpoint segment of the last forward run (same states and
        outcomes) with the likelihood evaluated at ``theta_eval`` (default: the
        run's own parameters). Returns dict(ll, expected, G, H) per day."""
        if self.theta is None:
            raise RuntimeError('call forward() first')
        st = self.state
        theta_eval = self.theta if theta_eval is None else np.asarray(theta_eval, dtype=np.float64)
        st.enable_lik(grad=grad)
        st.set_lik_factor(self.params.factor(theta_eval))
        st.zero_lik()
        for (t0, t1), ck in zip(self._segments(), self.checkpoints):
            st.rewind(ck)
            st.run_days(t0, t1, open_prev=t0 > 0, close_last=t1 == self.npts, use_graph=self.use_graph)
        if st.status():
            raise L.CovgpuError('likelihood recompute', st.status())
        return self._read(grad=grad)

    def backward(self, g_ll, g_expected, theta_eval=None):
        """Vector-Jacobian product: d(g_ll * ll + g_expected . expected) / d theta,
        from the forward's own sensitivities at its parameters, else by
        recomputing from the checkpoints at ``theta_eval``."""
        if theta_eval is None or np.array_equal(np.asarray(theta_eval, dtype=np.float64), self.theta):
            if self._grads is None:
                raise RuntimeError('call forward() first')
            theta_eval, out = self.theta, self._grads
        else:
            theta_eval = np.asarray(theta_eval, dtype=np.float64)
            out = self.recompute(theta_eval, grad=True)
        G = float(g_ll) * out['G'] + np.asarray(g_expected, dtype=np.float64)[:, None] * out['H']
        return self.params.chain(theta_eval, G)

    def diagnosis_kernel(self):
        """K[k]: the fraction of the last run's infected agents diagnosed k days
        after their exposure (date_diagnosed - date_exposed), an estimate of the
        delay distribution from infection to a positive test result."""
        st = self.state
        e = st.get('date_exposed').cpu().numpy()
        d = st.get('date_diagnosed').cpu().numpy()
        exposed = ~np.isnan(e)
        K = np.zeros(self.npts)
        if not exposed.any():
            return K
        diag = exposed & ~np.isnan(d)
        lag = np.clip(np.rint(d[diag] - e[diag]).astype(np.int64), 0, self.npts - 1)
        np.add.at(K, lag, 1.0)
        return K / exposed.sum()

    def loglik(self, theta_eval):
        """ll and expected[npts] at ``theta_eval`` on the last run's fixed states."""
        out = self.recompute(theta_eval, grad=False)
        return float(out['ll'].sum()), out['expected']


class SimLikelihood(torch.autograd.Function):
    """(ll, expected[npts]) = SimLikelihood.apply(theta, run): the forward runs the
    sim at ``theta`` (float64 CPU tensor, ``run.params.names`` order); the
    backward is the library's adjoint on the run's fixed states."""

    @staticmethod
    def forward(ctx, theta, run):
        ll, expected = run.forward(theta.detach().cpu().numpy())
        ctx.run = run
        return (torch.tensor(ll, dtype=torch.float64),
                torch.from_numpy(np.asarray(expected, dtype=np.float64)))

    @staticmethod
    def backward(ctx, g_ll, g_expected):
        g_ll = 0.0 if g_ll is None else float(g_ll)
        g_exp = (np.zeros(ctx.run.npts) if g_expected is None
                 else g_expected.detach().cpu().numpy().astype(np.float64))
        grad = ctx.run.backward(g_ll, g_exp)
        return torch.from_numpy(grad), None


def delay_matrix(K):
    """M[t, s] = K[t - s] (t >= s): M @ expected gives the expected diagnoses of each day."""
    T = len(K)
    idx = np.arange(T)
    lag = idx[:, None] - idx[None, :]
    return np.where(lag >= 0, np.asarray(K)[np.clip(lag, 0, T - 1)], 0.0)


def fit_parameters(run, target, theta0=None, fit=('beta',), steps=40, lr=0.05, fixed_states=False,
                   observe='infections'):
    """Gradient-based calibration: minimise sum_t (model[t] - target[t])^2 / sum(target^2)
    over log theta of the parameters named in ``fit`` (Adam). The model of the
    target series is the expected new infections of each day (observe =
    'infections'), or the expected diagnoses (observe = 'diagnoses': the expected
    infections convolved with the run's own infection-to-diagnosis delay
    distribution, ``LikelihoodRun.diagnosis_kernel``, which is held fixed within
    a step), the series a sim with test_prob reports as new_diagnoses. With
    ``fixed_states`` the states of one run at ``theta0`` are kept and only the
    likelihood is re-evaluated; otherwise each step re-simulates at the
    current parameters. Returns (theta, history of (loss, theta))."""
    if observe not in ('infections', 'diagnoses'):
        raise ValueError("observe must be 'infections' or 'diagnoses'")
    names = run.params.names
    theta0 = run.params.theta0 if theta0 is None else np.asarray(theta0, dtype=np.float64)
    idx = [names.index(n) for n in fit]
    logt = torch.tensor(np.log(theta0[idx]), dtype=torch.float64, requires_grad=True)
    opt = torch.optim.Adam([logt], lr=lr)
    target = torch.as_tensor(np.asarray(target, dtype=np.float64))
    scale = float((target ** 2).sum()) or 1.0
    hist = []
    if fixed_states:
        run.forward(theta0)
    for _ in range(steps):
        theta = torch.tensor(theta0, dtype=torch.float64)
        theta = theta.index_put((torch.tensor(idx),), torch.exp(logt))
        if fixed_states:
            th = theta.detach().numpy()
            ll, expected = run.loglik(th)
            M = delay_matrix(run.diagnosis_kernel()) if observe == 'diagnoses' else np.eye(len(expected))
            e = torch.from_numpy(M @ expected)
            resid = e - target[:len(e)]
            loss = float((resid ** 2).sum()) / scale
            g_exp = M.T @ (2.0 * resid / scale).numpy()
            g_theta = torch.from_numpy(run.backward(0.0, g_exp, theta_eval=th))
            opt.zero_grad()
            logt.grad = g_theta[idx] * torch.exp(logt.detach())
        else:
            _, expected = SimLikelihood.apply(theta, run)
            model = expected
            if observe == 'diagnoses':
                model = torch.from_numpy(delay_matrix(run.diagnosis_kernel())) @ expected
            resid = model - target[:len(model)]
            loss_t = (resid ** 2).sum() / scale
            opt.zero_grad()
            loss_t.backward()
            loss = float(loss_t.detach())
        opt.step()
        hist.append((loss, np.exp(logt.detach().numpy()).copy()))
    out = np.array(theta0)
    out[idx] = np.exp(logt.detach().numpy())
    return out, hist
