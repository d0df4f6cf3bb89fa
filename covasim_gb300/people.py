"""``People``: the reference's People interface over one sim's agents in HBM.

Keys are those of covasim/defaults.py:37-138. Reading ``people[key]`` or
``people.key`` returns a numpy copy (the reference's arrays are numpy);
``people.gpu(key)`` returns the device tensor (a view for float and int
arrays; booleans are unpacked from the state word). Writing
``people[key] = values`` updates the device state. The transition and
infection methods run the CUDA kernels.
"""
import numpy as np
import torch

from . import defaults as cvd
from . import _lib as L

__all__ = ['People', 'Layer', 'Contacts']


def log_layer_tag(layer, layer_keys, extra):
    """The infection-log tag of an infect() call's ``layer`` (people.py:508-511):
    a contact layer's index, LOG_SEED / LOG_IMPORT for 'seed_infection' /
    'importation', LOG_NONE for None, else a tag registered in ``extra``."""
    if layer in layer_keys:
        return layer_keys.index(layer)
    if layer is None:
        return L.LOG_NONE
    named = {'seed_infection': L.LOG_SEED, 'importation': L.LOG_IMPORT}
    if layer in named:
        return named[layer]
    if layer not in extra:
        if L.LOG_EXTRA + len(extra) > 0xFF:
            raise ValueError('too many distinct infection-log layer labels')
        extra.append(layer)
    return L.LOG_EXTRA + extra.index(layer)


def log_layer_label(tag, layer_keys, extra):
    """Inverse of log_layer_tag."""
    if tag < len(layer_keys):
        return layer_keys[tag]
    if tag == L.LOG_SEED:
        return 'seed_infection'
    if tag == L.LOG_IMPORT:
        return 'importation'
    if L.LOG_EXTRA <= tag < L.LOG_EXTRA + len(extra):
        return extra[tag - L.LOG_EXTRA]
    return None


class Layer(dict):
    """One contact layer (covasim/base.py:1610-1876): p1, p2, beta arrays."""

    def __init__(self, p1=None, p2=None, beta=None, label=None, **kwargs):
        super().__init__()
        self.label = label
        self['p1'] = np.asarray([] if p1 is None else p1, dtype=cvd.default_int)
        self['p2'] = np.asarray([] if p2 is None else p2, dtype=cvd.default_int)
        self['beta'] = (np.ones(len(self['p1']), dtype=cvd.default_float) if beta is None
                        else np.asarray(beta, dtype=cvd.default_float))
        for k, v in kwargs.items():
            self[k] = v

    def __len__(self):
        return len(self['p1'])

    def meta_keys(self):
        return ['p1', 'p2', 'beta']

    def validate(self):
        n = len(self['p1'])
        for key in ('p2', 'beta'):
            if len(self[key]) != n:
                raise TypeError(f'Expecting length {n} for layer key "{key}"; got {len(self[key])}')

    def find_contacts(self, inds, as_array=True):
        """base.py:1808-1846: partners of ``inds`` in either direction."""
        inds = np.asarray(inds)
        m1 = np.isin(self['p1'], inds)
        m2 = np.isin(self['p2'], inds)
        out = set(self['p2'][m1].tolist()) | set(self['p1'][m2].tolist())
        if as_array:
            out = np.fromiter(out, dtype=cvd.default_int)
            out.sort()
        return out

    @property
    def members(self):
        return np.unique(np.concatenate([self['p1'], self['p2']]))


class Contacts(dict):
    """Contact layers by key (covasim/base.py:1509-1606)."""

    def __len__(self):
        return sum(len(v) for v in self.values())

    def add_layer(self, **kwargs):
        for lkey, layer in kwargs.items():
            if not isinstance(layer, Layer):
                layer = Layer(**layer, label=lkey)
            layer.validate()
            self[lkey] = layer


class People:
    """One sim's agents (covasim/people.py:20-118), state kept in device memory."""

    def __init__(self, state, sim_index, pars, contacts):
        self.__dict__['_state'] = state
        self.__dict__['_sim'] = sim_index
        self.__dict__['pars'] = pars
        self.__dict__['contacts'] = contacts
        self.__dict__['t'] = 0
        self.__dict__['flows'] = {k: 0 for k in cvd.new_result_flows}
        self.__dict__['flows_variant'] = {k: np.zeros(pars['n_variants']) for k in cvd.new_result_flows_by_variant}

    # ------------------------------------------------------------------ access
    def gpu(self, key):
        """Device tensor for ``key``."""
        return self._state.get(key, self._sim)

    def __getitem__(self, key):
        if key in ('age', 'sex') and key in self.__dict__:
            return self.__dict__[key]
        try:
            return self.gpu(key).cpu().numpy()
        except KeyError as E:
            raise AttributeError(f'Key "{key}" is not a valid attribute of people') from E

    def __setitem__(self, key, value):
        if key in ('age', 'sex', 't', 'pars', 'contacts', 'flows', 'flows_variant', 'infection_log_'):
            self.__dict__[key] = value
            return
        self._state.set(key, value, self._sim)

    def __getattr__(self, key):
        if key.startswith('__'):
            raise AttributeError(key)
        return self[key]

    def __setattr__(self, key, value):
        self[key] = value

    def __len__(self):
        return int(self.pars['pop_size'])

    def keys(self):
        return cvd.ALL_STATES[:]

    def person_keys(self):
        return cvd.PERSON[:]

    def state_keys(self):
        return cvd.STATES[:]

    def layer_keys(self):
        return list(self.contacts.keys())

    # ------------------------------------------------------------------ counts (base.py:1118-1145)
    def count(self, key):
        return int(torch.count_nonzero(self.gpu(key)).item())

    def count_by_variant(self, key, variant):
        return int(torch.count_nonzero(self.gpu(key)[variant]).item())

    def count_not(self, key):
        return len(self) - self.count(key)

    def true(self, key):
        return self[key].nonzero()[0]

    def false(self, key):
        return (~self[key]).nonzero()[0]

    def defined(self, key):
        return (~np.isnan(self[key])).nonzero()[0]

    def undefined(self, key):
        return np.isnan(self[key]).nonzero()[0]

    # ------------------------------------------------------------------ transitions
    def update_states_pre(self, t, close_prev=False):
        """people.py:164-186 (+ check_immunity), on the device for every agent.

        ``close_prev`` also closes day t-1 first (stocks and update_nab), which
        the fused kernel does in the same pass.
        """
        self.__dict__['t'] = t
        self._state.agent_step(t, do_prev=close_prev, do_day=True)

    def infect(self, inds, hosp_max=None, icu_max=None, source=None, layer=None, variant=0, call_tag=2):
        """people.py:435-586 on the device for an explicit list of agents (seed
        infections, importations, interventions); the day's transmissions are
        infected on the device by the edge pass. As the reference: duplicates
        are removed keeping each agent's first source, only the susceptible are
        infected, each infection is logged with its source and layer, and the
        agents actually infected are returned (sorted)."""
        inds = np.asarray(inds, dtype=np.int64)
        if len(inds) == 0:
            return inds
        if source is not None and len(source) != len(inds):
            raise ValueError('infect: source must have one entry per target')
        if hosp_max is not None or icu_max is not None:
            self._state.set_hospicu([[int(bool(hosp_max)), int(bool(icu_max))]] * len(self._state.specs))
        layer_tag = log_layer_tag(layer, self.layer_keys(), self._state.log_labels)
        u, infected = self._state.infect_list(self.t, inds, sim=self._sim, variant=variant, layer_tag=layer_tag,
                                              call_tag=call_tag, sources=source, want_infected=True)
        if hosp_max is not None or icu_max is not None:
            self._state.set_hospicu(None)
        done = u[infected.cpu().numpy().astype(bool)]
        self.flows['new_infections'] += len(done)
        self.flows_variant['new_infections_by_variant'][variant] += len(done)
        return done

    # ------------------------------------------------------------------ one check at a time (people.py:222-312)
    def _check(self, which, filter_exposed=True, inds=None):
        got, known = self._state.check(self.t, which, sim=self._sim, filter_exposed=filter_exposed, inds=inds)
        return got.cpu().numpy().astype(cvd.default_int), known

    def check_infectious(self):
        """people.py:222-232: the exposed whose infectious date has come become
        infectious with their exposed variant; returns their indices."""
        inds, _ = self._check(L.CHECK_INFECTIOUS)
        iv = self['infectious_variant'][inds]
        for v in range(self.pars['n_variants']):
            self.flows_variant['new_infectious_by_variant'][v] += int(np.count_nonzero(iv == v))
        return inds

    def check_symptomatic(self):
        """people.py:235-239."""
        return self._check(L.CHECK_SYMPTOMATIC)[0]

    def check_severe(self):
        """people.py:242-246."""
        return self._check(L.CHECK_SEVERE)[0]

    def check_critical(self):
        """people.py:249-253."""
        return self._check(L.CHECK_CRITICAL)[0]

    def check_recovery(self, inds=None, filter_inds='is_exp'):
        """people.py:256-291: recovery of the exposed whose date has come (or of
        exactly ``inds`` when given); with waning they become susceptible again.
        filter_inds 'is_exp' checks the exposed, None every agent."""
        if inds is not None:
            return self._check(L.CHECK_RECOVERY, inds=np.asarray(inds))[0]
        if filter_inds is not None and not (isinstance(filter_inds, str) and filter_inds == 'is_exp'):
            raise NotImplementedError("check_recovery: filter_inds must be 'is_exp' or None on the GPU path")
        return self._check(L.CHECK_RECOVERY, filter_exposed=filter_inds is not None)[0]

    def check_death(self):
        """people.py:294-312: returns (indices, deaths, deaths of the diagnosed)."""
        inds, known = self._check(L.CHECK_DEATH)
        return inds, len(inds), int(known)

    def check_exit_iso(self):
        """people.py:368-374: isolation ends on its date; returns the released."""
        return self._check(L.CHECK_EXIT_ISO, filter_exposed=False)[0]

    @property
    def infection_log(self):
        """people.py:508-511 records: dict(source, target, date, layer, variant)."""
        rec = self._state.infection_log(self._sim)
        keys = self.layer_keys()
        vmap = self.pars['variant_map']
        out = []
        for src, tgt, day, layer, v in rec.tolist():
            lk = log_layer_label(layer, keys, self._state.log_labels)
            out.append(dict(source=None if src < 0 else src, target=tgt, date=day, layer=lk, variant=vmap[v]))
        return out
