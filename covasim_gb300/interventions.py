"""Interventions that the GPU day loop consumes as per-day device tables.

``change_beta`` (covasim/interventions.py:530-586) changes the overall beta or a
layer's beta from given days on. On the GPU path its effect is folded into the
per-day beta tables before the run, so the whole day loop can be captured in a
CUDA graph without a host round trip per day.
"""
import numpy as np

__all__ = ['Intervention', 'change_beta']


class Intervention:
    """Base class (interventions.py:223-410): ``initialize(sim)`` then ``apply(sim)`` per day.

    Subclasses that only change per-day parameters implement ``apply_day(t, betas)``,
    which the GPU sim folds into its per-day tables; other interventions are
    called on the host between the agent pass and the transmission pass.
    """

    def __init__(self, label=None, show_label=False, do_plot=None, line_args=None):
        self.label = label or self.__class__.__name__
        self.show_label = show_label
        self.do_plot = do_plot if do_plot is not None else True
        self.days = []
        self.initialized = False
        self.finalized = False

    def initialize(self, sim=None):
        self.initialized = True

    def finalize(self, sim=None):
        self.finalized = True

    def apply(self, sim):
        raise NotImplementedError

    def __call__(self, *args, **kwargs):
        if not self.initialized:
            raise RuntimeError(f'Intervention (label={self.label}, {type(self)}) has not been initialized')
        return self.apply(*args, **kwargs)


def _process_days(days):
    if not isinstance(days, (list, tuple, np.ndarray)):
        days = [days]
    return np.sort(np.asarray(days, dtype=int))


def _process_changes(changes, days):
    if not isinstance(changes, (list, tuple, np.ndarray)):
        changes = [changes] * len(days)
    changes = np.asarray(changes, dtype=float)
    if len(changes) != len(days):
        raise ValueError(f'Number of days supplied ({len(days)}) does not match number of changes ({len(changes)})')
    return changes


class change_beta(Intervention):
    """Multiply beta (or layer betas) by ``changes[i]`` from ``days[i]`` on (interventions.py:530-586).

    The multiplier applies to the beta the sim had at initialisation, as in
    the reference.
    """

    def __init__(self, days, changes, layers=None, **kwargs):
        super().__init__(**kwargs)
        self.days = days
        self.changes = changes
        self.layers = layers
        self.orig_betas = None

    def initialize(self, sim):
        super().initialize()
        self.days = _process_days(self.days)
        self.changes = _process_changes(self.changes, self.days)
        layers = self.layers
        self.layers = [layers] if (layers is None or isinstance(layers, str)) else list(layers)
        self.orig_betas = {}
        for lkey in self.layers:
            if lkey is None:
                self.orig_betas['overall'] = sim['beta']
            else:
                self.orig_betas[lkey] = sim['beta_layer'][lkey]

    def apply_day(self, t, betas):
        """Day-t effect on ``betas`` = {'overall': beta, layer key: beta_layer} (in place)."""
        for ind in np.nonzero(self.days == t)[0]:
            for lkey, orig in self.orig_betas.items():
                betas[lkey] = orig * self.changes[ind]

    def apply(self, sim):
        betas = {'overall': sim['beta'], **sim['beta_layer']}
        self.apply_day(sim.t, betas)
        sim['beta'] = betas.pop('overall')
        sim['beta_layer'].update(betas)
