"""``BatchSim``: many independent sims in one device state and one launch sequence.

Replaces the process fan-out of ``cv.MultiSim`` / ``multi_run``
(covasim/run.py:36-180, 1406-1519): every sim's agents and edges are
concatenated in HBM with per-sim offsets, each sim keeps its own parameter
block (seed, beta, change_beta schedule, population size ...), and each day is
one agent pass, one edge pass and one infect pass over all sims together; the
whole day loop is captured as one CUDA graph. Because every draw is keyed by
the sim's own seed and its local agent/edge indices, a sim gives the same
results alone or in any batch.
"""
import copy

import numpy as np

from . import parameters as cvpar
from . import immunity as cvimm
from . import defaults as cvd
from . import _lib as L
from .sim import Sim, build_spec, init_infections, variant_import_count, CALL_IMPORT
from .state import BatchState

__all__ = ['BatchSim']


class BatchSim:
    """Run a list of sims (or ``n_runs`` reseeded copies of one) as one batch.

    Args:
        sims: a Sim, or a list of Sims (not yet run)
        n_runs: with a single Sim, run this many copies with rand_seed + i (run.py:1363-1365)
        use_graph: capture the day loop in a CUDA graph
    """

    def __init__(self, sims, n_runs=None, use_graph=True, log=False, edge_tile=None):
        if isinstance(sims, Sim):
            base = sims
            n_runs = n_runs or 1
            sims = []
            for i in range(n_runs):
                s = copy.deepcopy(base)
                s['rand_seed'] = base['rand_seed'] + i
                sims.append(s)
        self.sims = list(sims)
        self.use_graph = use_graph
        self.log = log
        self.edge_tile = edge_tile  # as Sim's: None (the default, '2048w'), a tile, a label such as '8192r', or 'auto'
        self.state = None

    def initialize(self):
        specs = []
        self.npts = None
        for s in self.sims:
            s.validate_pars()
            s.init_variants()
            if s['prognoses'] is None:
                s['prognoses'] = cvpar.get_prognoses(s['prog_by_age'])
            cvimm.init_immunity(s.pars, s.npts)
            s.init_results()
            s.init_interventions()
            spec, popdict, person = build_spec(s.pars, s.popdict, getattr(s, '_person', None), s['interventions'],
                                               gpu_population=getattr(s, 'gpu_population', False))
            s.popdict, s._person, s.spec = popdict, person, spec
            specs.append(spec)
        npts = {sp.npts for sp in specs}
        if len(npts) != 1:
            raise ValueError('all sims of a batch must have the same number of days')
        self.npts = npts.pop()
        self.state = BatchState(specs, log=self.log)
        self.state.apply_edge_tile(self.edge_tile)
        return self

    def seed_infections(self):
        for k, s in enumerate(self.sims):
            init_infections(self.state, k, s.pars)

    def _import_variants(self, t):
        """Each sim's variant importations of day t, with the sim's own draws
        (immunity.py:117-130, as Sim does them)."""
        for k, s in enumerate(self.sims):
            for v in s['variants']:
                if t in np.atleast_1d(v.days):
                    sus = np.nonzero(self.state.get('susceptible', k).cpu().numpy())[0]
                    rng = np.random.default_rng([int(s['rand_seed']), 0x1A1A, t, v.index])
                    n_imp = variant_import_count(v, self.state.rescale_vecs[k][t], rng)  # more than len(sus): ValueError
                    inds = rng.choice(sus, n_imp, replace=False)
                    self.state.set_hospicu([[0, 0]] * len(self.sims))  # variant.apply: no bed limits
                    self.state.infect_list(t, inds, sim=k, variant=v.index, layer_tag=L.LOG_IMPORT,
                                           call_tag=CALL_IMPORT + v.index)
                    self.state.set_hospicu(None)
                    self.state.note_imports(k, t, len(inds))

    def run(self, use_graph=None):
        if self.state is None:
            self.initialize()
        use_graph = self.use_graph if use_graph is None else use_graph
        self.seed_infections()
        # the days with importations (any sim's) run as single steps, the rest as graphs
        host_days = sorted({d for s in self.sims for d in s._variant_days() if 0 <= d < self.npts})
        st, t = self.state, 0
        for d in host_days + [self.npts]:
            while d > t:
                st.run_days(t, d, open_prev=False, close_last=True, use_graph=use_graph)
                held = st.held_day()
                if held is not None and held < d:  # a rescaling fell due on day `held` (sim.py:535-556)
                    st.rescale_day(held)
                    t = held
                else:
                    t = d
            if t < self.npts:
                st.rescale_day(t)
                st.agent_step(t, do_prev=False, do_day=True)
                st.import_day(t)
                self._import_variants(t)
                st.test_trace(t)
                st.edge_pass(t)
                st.infect_claims(t)
                st.agent_step(t + 1, do_prev=True, do_day=False)
                t += 1
        status = self.state.status()
        if status:
            raise L.CovgpuError('device status', status)
        return self

    def results(self, k):
        """Raw per-day device results of sim k (see BatchState.results)."""
        return self.state.results(k)

    def series(self, key):
        """[n_sims, npts] array of one per-day result."""
        return np.stack([self.state.results(k)[key] for k in range(len(self.sims))])

    def finalize(self):
        """Fill each Sim's results as Sim.finalize does."""
        for k, s in enumerate(self.sims):
            s.state = self.state
            s.t = self.npts
            s.complete = True
            s._fill_results(self.state.results(k), self.state.rescale_vecs[k])
            s.results_ready = True
            s.t -= 1
            s.compute_states()
        return self.sims
