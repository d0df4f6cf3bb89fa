"""Consumers of a finished sim: ``Fit`` and ``compute_gof`` (covasim/analysis.py:991-1235,
covasim/misc.py:707-790), ``TransTree`` (covasim/analysis.py:1772-2057) and
``Calibration`` (covasim/analysis.py:1358-1660), with ``load_data``
(covasim/misc.py:33-91) for the data they compare against.

The reference keeps data files and the detailed transmission tree in pandas
DataFrames; here they are ``DataTable`` objects (named numpy columns with the
same keys), since the consumers only read columns, and pandas is not a
dependency of this package.

``TransTree`` is built on the device from the infection log that the infect
kernels write (one record per infection, in the reference's order): the
last-infection-per-target maps, the per-source transmission counts and the
distinct-edge out-degrees are scatter/bincount passes over the log instead of
the reference's Python loops over every agent and every record.

``Calibration`` keeps the reference's interface (``calib_pars`` as
``dict(key=[best, low, high])``, ``fit_args``, ``custom_fn``, ``calibrate``,
``best_pars``, ``before``/``after``, ``summarize``, ``to_json``). The reference
draws trials with Optuna, one sim per worker process; Optuna is not a
dependency here, so trials are drawn by a seeded cross-entropy search
(Rubinstein's method: sample, keep the elite quarter, refit a truncated normal
per parameter) and each generation of ``n_workers`` trials runs as one
``BatchSim`` -- all of a generation's sims in one launch sequence on the GPU.
"""
import copy
import csv
import datetime as dt
import json
import math
import os
import time
import warnings

import numpy as np
import torch

from .people import log_layer_label

__all__ = ['Analyzer', 'DataTable', 'load_data', 'compute_gof', 'Fit', 'TransTree', 'Calibration',
           'to_date', 'to_day']


# ----------------------------------------------------------------------------- dates
def to_date(x):
    """A date from a 'YYYY-MM-DD' string, a date, a datetime or a numpy datetime64."""
    if isinstance(x, dt.datetime):
        return x.date()
    if isinstance(x, dt.date):
        return x
    if isinstance(x, np.datetime64):
        return x.astype('datetime64[D]').astype(dt.date)
    if isinstance(x, str):
        return dt.date.fromisoformat(x.strip()[:10])
    raise TypeError(f'cannot convert {x!r} to a date')


def to_day(day, start_day):
    """Days since ``start_day`` for a date (string or object); integers pass through
    (sciris' ``sc.day`` as the reference uses it)."""
    if day is None:
        return None
    if isinstance(day, (list, tuple, np.ndarray)):
        return [to_day(d, start_day) for d in day]
    if isinstance(day, (int, np.integer)):
        return int(day)
    if isinstance(day, (float, np.floating)) and float(day).is_integer():
        return int(day)
    return (to_date(day) - to_date(start_day)).days


class Analyzer:
    """Base of the analyzers (covasim/analysis.py:37-100): a label and the
    initialize / finalize flags."""

    def __init__(self, label=None):
        self.label = label or self.__class__.__name__
        self.initialized = False
        self.finalized = False

    def initialize(self, sim=None):
        self.initialized = True

    def finalize(self, sim=None):
        self.finalized = True

    def __repr__(self):
        return f'{self.__class__.__name__}(label={self.label!r})'


# ----------------------------------------------------------------------------- data
class DataTable:
    """Named columns of equal length (numpy arrays), indexed by the 'date' column
    when there is one: the part of a pandas DataFrame that the consumers use."""

    def __init__(self, columns=None):
        self._cols = {}
        for k, v in (columns or {}).items():
            self[k] = v

    @property
    def columns(self):
        return list(self._cols.keys())

    def keys(self):
        return self.columns

    def __contains__(self, key):
        return key in self._cols

    def __getitem__(self, key):
        return self._cols[key]

    def __setitem__(self, key, value):
        arr = value if isinstance(value, np.ndarray) else np.asarray(value)
        if self._cols and len(arr) != len(self):
            raise ValueError(f'column {key!r} has {len(arr)} rows, the table {len(self)}')
        self._cols[key] = arr

    def __len__(self):
        return len(next(iter(self._cols.values()))) if self._cols else 0

    @property
    def index(self):
        return self._cols['date'] if 'date' in self._cols else np.arange(len(self))

    def items(self, key):
        """(index, value) pairs of one column, as ``df[key].items()``."""
        return zip(self.index.tolist(), self._cols[key].tolist())

    def rows(self, mask):
        """The rows where ``mask`` holds, as a new table."""
        return DataTable({k: v[mask] for k, v in self._cols.items()})

    def to_dict(self):
        return {k: v.tolist() for k, v in self._cols.items()}

    def __repr__(self):
        return f'DataTable({len(self)} rows: {", ".join(self.columns)})'


def _parse_column(values):
    """Strings of one CSV column -> float64 (empty cells NaN), or the strings."""
    out = np.empty(len(values), dtype=np.float64)
    for i, v in enumerate(values):
        v = v.strip()
        if v == '':
            out[i] = np.nan
            continue
        try:
            out[i] = float(v)
        except ValueError:
            return np.asarray(values, dtype=object)
    return out


def _nan_cumsum(x):
    """Running sum that skips missing values and keeps them missing (pandas'
    ``cumsum``, which ``np.cumsum`` dispatches to for a Series)."""
    x = np.asarray(x, dtype=np.float64)
    out = np.nancumsum(x)
    out[np.isnan(x)] = np.nan
    return out


def load_data(datafile, calculate=True, check_date=True, verbose=True, start_day=None, **kwargs):
    """Data to compare with the model (misc.py:33-91): a .csv or .json file, a
    dict of columns or a DataTable. Missing ``cum_`` columns are added from the
    ``new_`` ones; the 'date' column becomes dates (integers count days from
    ``start_day``)."""
    if isinstance(datafile, os.PathLike):
        datafile = str(datafile)
    if isinstance(datafile, str):
        low = datafile.lower()
        if low.endswith('csv'):
            with open(datafile, newline='') as fh:
                rows = list(csv.reader(fh, **kwargs))
            header, body = rows[0], [r for r in rows[1:] if r]
            cols = {h: _parse_column([r[j] if j < len(r) else '' for r in body]) for j, h in enumerate(header)}
            data = DataTable(cols)
        elif low.endswith('json'):
            with open(datafile) as fh:
                raw = json.load(fh)
            if isinstance(raw, list):  # records
                keys = list(dict.fromkeys(k for r in raw for k in r))
                raw = {k: [r.get(k, np.nan) for r in raw] for k in keys}
            data = DataTable({k: (np.asarray(v, dtype=np.float64) if k != 'date' else np.asarray(v, dtype=object))
                              for k, v in raw.items()})
        else:
            raise NotImplementedError(f'Currently loading is only supported from .csv and .json files, not "{datafile}"')
    elif isinstance(datafile, DataTable):
        data = datafile
    elif isinstance(datafile, dict):
        data = DataTable({k: (np.asarray(v, dtype=object) if k == 'date' else np.asarray(v)) for k, v in datafile.items()})
    else:
        raise TypeError(f'Could not interpret data {type(datafile)}: must be a file name, a dict or a DataTable')

    if calculate:
        for col in data.columns:
            if col.startswith('new'):
                cum_col = col.replace('new_', 'cum_')
                if cum_col not in data:
                    data[cum_col] = _nan_cumsum(data[col])
                    if verbose:
                        print(f'  Automatically adding cumulative column {cum_col} from {col}')

    if check_date:
        if 'date' not in data:
            raise ValueError(f'Required column "date" not found; columns are {data.columns}')
        raw = data['date']
        if raw.dtype.kind in 'iuf' or all(isinstance(d, (int, np.integer)) for d in raw.tolist()):
            if start_day is None:
                raise ValueError('integer dates count days from start_day, which was not given')
            base = to_date(start_day)
            dates = [base + dt.timedelta(days=int(d)) for d in raw.tolist()]
        else:
            dates = [to_date(d) for d in raw.tolist()]
        data['date'] = np.asarray(dates, dtype=object)
    return data


# ----------------------------------------------------------------------------- goodness of fit
def compute_gof(actual, predicted, normalize=True, use_frac=False, use_squared=False, as_scalar='none', eps=1e-9,
                skestimator=None, estimator=None, **kwargs):
    """Goodness of fit (misc.py:707-790): normalised absolute error by default;
    ``use_frac`` for fractional errors, ``use_squared``, ``as_scalar`` in
    sum / mean / median, or a scikit-learn / custom estimator."""
    actual = np.array(copy.deepcopy(actual), dtype=float)
    predicted = np.array(copy.deepcopy(predicted), dtype=float)

    if skestimator is not None:
        try:
            import sklearn.metrics as sm
            sklearn_gof = getattr(sm, skestimator)
        except ImportError as E:
            raise ImportError(f'You must have scikit-learn >=0.22.2 installed: {str(E)}') from E
        except AttributeError as E:
            raise AttributeError(f'Estimator {skestimator} is not available in sklearn.metrics') from E
        return sklearn_gof(actual, predicted, **kwargs)

    if estimator is not None:
        try:
            return estimator(actual, predicted, **kwargs)
        except Exception as E:
            raise RuntimeError(f'Custom estimator "{estimator}" must be a callable function that accepts actual and '
                               'predicted arrays, plus optional kwargs') from E

    gofs = abs(np.array(actual) - np.array(predicted))
    if normalize and not use_frac:
        actual_max = abs(actual).max()
        if actual_max > 0:
            gofs /= actual_max
    if use_frac:
        if (actual < 0).any() or (predicted < 0).any():
            print('Warning: Calculating fractional errors for non-positive quantities is ill-advised!')
        else:
            maxvals = np.maximum(actual, predicted) + eps
            gofs /= maxvals
    if use_squared:
        gofs = gofs ** 2
    if as_scalar == 'sum':
        gofs = np.sum(gofs)
    elif as_scalar == 'mean':
        gofs = np.mean(gofs)
    elif as_scalar == 'median':
        gofs = np.median(gofs)
    return gofs


class Fit(Analyzer):
    """The fit between a finished sim and its data (analysis.py:991-1235):
    paired points by date -> differences -> goodness of fit (``compute_gof``)
    -> losses (times ``weights``: 10 for cum_deaths, 5 for cum_diagnoses, 1
    otherwise) -> one mismatch per key -> their sum, ``mismatch``."""

    def __init__(self, sim, weights=None, keys=None, custom=None, compute=True, verbose=False, die=True, label=None,
                 **kwargs):
        super().__init__(label=label)
        self.custom = dict(custom or {})
        self.verbose = verbose
        self.weights = {'cum_deaths': 10, 'cum_diagnoses': 5, **(weights or {})}
        self.keys = keys
        self.gof_kwargs = kwargs
        self.die = die

        if sim.data is None:
            errormsg = 'Model fit cannot be calculated until data are loaded'
            if self.die:
                raise RuntimeError(errormsg)
            warnings.warn(errormsg)
            sim.data = DataTable()
        self.data = sim.data

        if not sim.results_ready:
            errormsg = 'Model fit cannot be calculated until results are run'
            if self.die:
                raise RuntimeError(errormsg)
            warnings.warn(errormsg)
        self.sim_results = {}
        for key in sim.result_keys() + ['t', 'date']:
            self.sim_results[key] = sim.results[key]
        self.sim_npts = sim.npts
        self.sim_dates = list(sim.datevec)

        self.inds = {'sim': {}, 'data': {}}
        self.date_matches = {}
        self.pair = {}
        self.diffs = {}
        self.gofs = {}
        self.losses = {}
        self.mismatches = {}
        self.mismatch = None
        if compute:
            self.compute()

    def compute(self):
        self.reconcile_inputs()
        self.compute_diffs()
        self.compute_gofs()
        self.compute_losses()
        self.compute_mismatch()
        return self.mismatch

    def reconcile_inputs(self):
        """Matching keys and dates of the model and the data (analysis.py:1085-1170)."""
        data_cols = self.data.columns
        if self.keys is None:
            sim_keys = [k for k in self.sim_results.keys() if k.startswith('cum_')]
            self.keys = [key for key in sim_keys if key in data_cols]
            if not len(self.keys):
                errormsg = f'No matches found between simulation result keys {sim_keys} and data columns {data_cols}'
                if self.die:
                    raise KeyError(errormsg)
                warnings.warn(errormsg)
        missing = [key for key in self.keys if key not in data_cols]
        if missing:
            errormsg = f'The following requested key(s) were not found in the data: {", ".join(missing)}'
            if self.die:
                raise KeyError(errormsg)
            warnings.warn(errormsg)

        date_pos = {d: i for i, d in reversed(list(enumerate(self.sim_dates)))}  # first position of each date
        for key in self.keys:
            sim_inds, data_inds, matches = [], [], []
            for count, (d, datum) in enumerate(self.data.items(key)):
                if np.isfinite(datum) and d in date_pos:
                    matches.append(d)
                    sim_inds.append(date_pos[d])
                    data_inds.append(count)
            self.date_matches[key] = matches
            self.inds['sim'][key] = np.array(sim_inds)
            self.inds['data'][key] = np.array(data_inds)

        n_matches = 0
        for key in self.keys:
            sim_inds, data_inds = self.inds['sim'][key], self.inds['data'][key]
            n = len(sim_inds)
            n_matches += n
            sim_vals = np.asarray(self.sim_results[key].values)
            data_vals = np.asarray(self.data[key])
            self.pair[key] = {'sim': np.zeros(n), 'data': np.zeros(n)}
            if n:
                self.pair[key]['sim'][:] = sim_vals[sim_inds]
                self.pair[key]['data'][:] = data_vals[data_inds]

        self.custom_keys = list(self.custom.keys())
        for key, custom in self.custom.items():
            n_matches += 1
            c_keys = list(custom.keys())
            if 'sim' not in c_keys or 'data' not in c_keys:
                raise KeyError(f'Custom input must have "sim" and "data" keys, not {c_keys}')
            c_data, c_sim = custom['data'], custom['sim']
            try:
                assert len(c_data) == len(c_sim)
            except Exception as E:
                raise ValueError(f'Custom data and sim must be arrays of the same length: data = {c_data}, '
                                 f'sim = {c_sim} could not be processed') from E
            if key in self.pair:
                raise ValueError(f'You cannot use a custom key "{key}" that matches one of the existing keys: '
                                 f'{list(self.pair.keys())}')
            self.pair[key] = {'sim': c_sim, 'data': c_data}
            wt = custom.get('weight', 1.0)
            self.weights[key] = custom.get('weights', wt)

        if n_matches == 0:
            errormsg = ('No paired data points were found between the supplied data and the simulation; '
                        'please check the dates for each')
            if self.die:
                raise ValueError(errormsg)
            warnings.warn(errormsg)

    def compute_diffs(self, absolute=False):
        for key, pair in self.pair.items():
            self.diffs[key] = pair['sim'] - pair['data']
            if absolute:
                self.diffs[key] = np.abs(self.diffs[key])

    def compute_gofs(self, **kwargs):
        kwargs = {**self.gof_kwargs, **kwargs}
        for key, pair in self.pair.items():
            self.gofs[key] = compute_gof(pair['data'], pair['sim'], **kwargs)

    def compute_losses(self):
        for key, gof in self.gofs.items():
            weight = self.weights.get(key, 1.0)
            if np.iterable(weight):
                len_wt, len_match = len(weight), len(gof)
                if len_wt == len_match:
                    pass
                elif len_wt == self.sim_npts:
                    weight = np.asarray(weight)[self.inds['sim'][key]]
                else:
                    raise ValueError(f'Could not map weight array of length {len_wt} onto simulation of length '
                                     f'{self.sim_npts} or data-model matches of length {len_match}')
            self.losses[key] = gof * weight

    def compute_mismatch(self, use_median=False):
        for key, loss in self.losses.items():
            self.mismatches[key] = np.median(loss) if use_median else np.sum(loss)
        self.mismatch = np.array(list(self.mismatches.values())).sum()
        return self.mismatch

    def summarize(self):
        if self.mismatch is not None:
            print('Mismatch values for:')
            print(self.mismatches)
            print('\nTotal mismatch value:')
            print(self.mismatch)
        else:
            print('Mismatch values not yet calculated; please run sim.compute_fit().')


# ----------------------------------------------------------------------------- transmission tree
_ATTRS = ['age', 'date_exposed', 'date_symptomatic', 'date_tested', 'date_diagnosed', 'date_severe', 'date_critical',
          'date_known_contact']
_QUAR_ATTRS = ['date_quarantined', 'date_end_quarantine']
_NODE_ATTRS = ['age', 'date_exposed', 'date_symptomatic', 'date_tested', 'date_diagnosed', 'date_quarantined',
               'date_severe', 'date_critical', 'date_known_contact', 'date_recovered']


def _last_per_target(tgt, mask, n_agents):
    """Position in the log of the last record (among ``mask``) of each target, -1 for none."""
    pos = torch.arange(tgt.numel(), device=tgt.device, dtype=torch.int64)
    last = torch.full((n_agents,), -1, dtype=torch.int64, device=tgt.device)
    if mask is not None:
        tgt, pos = tgt[mask], pos[mask]
    if tgt.numel():
        last.scatter_reduce_(0, tgt, pos, reduce='amax')
    return last


class TransTree(Analyzer):
    """The transmission tree of a finished sim (analysis.py:1772-2057).

    ``infection_log``, ``sources``, ``targets``, ``source_dates``,
    ``target_dates``, ``n_targets``, ``transmissions``, ``source_inds``,
    ``target_inds``, ``detailed`` and ``df`` hold what the reference's hold
    (``detailed`` and ``df`` as DataTables); ``graph`` is the networkx DiGraph
    with ``to_networkx=True``. The reference's own conventions are kept: the
    source/target maps skip records whose source is agent 0 (its ``if source:``
    test), a target's source and date are those of its last infection, and
    ``detailed`` describes each target's last infection.

    Device work: ``source_of`` / ``source_date`` (int64 per agent, -1 for none)
    and ``n_targets_all`` (records per source) are scatter and bincount passes
    over the device log; the per-agent Python lists are built on first use.
    """

    def __init__(self, sim, to_networkx=False, **kwargs):
        super().__init__(**kwargs)
        people = sim.people
        self.sim_start = sim['start_day']
        self.sim_results = {'t': sim.results['t'], 'cum_infections': sim.results['cum_infections'].values}
        self.n_days = people.t
        self.pop_size = len(people)
        if sim['rescale'] and sim['pop_scale'] > 1:
            warnings.warn('Warning: transmission tree results are unreliable when dynamic rescaling is on, since '
                          'agents are reused! Please rerun with rescale=False and pop_scale=1 for reliable results.')
        self._people = people
        self._layer_names = people.layer_keys()
        self._log_labels = list(getattr(sim.state, 'log_labels', []))
        log = sim.state.infection_log_tensor(people._sim)
        self._log = log
        src, tgt, day = log[:, 0], log[:, 1], log[:, 2]
        n = self.pop_size
        truthy = src > 0  # the reference's `if source:` (agent 0 and seeds skipped)
        last = _last_per_target(tgt, truthy, n)
        has = last >= 0
        li = last.clamp(min=0)
        self.source_of = torch.where(has, src[li], torch.full_like(li, -1))
        self.source_date = torch.where(has, day[li], torch.full_like(li, -1))
        self.n_targets_all = torch.bincount(src[truthy], minlength=n)[:n]
        self._lists = None
        self._inflog = None
        self.count_targets()
        self.count_transmissions()
        self.make_detailed(people)
        if to_networkx:
            import networkx as nx
            self.graph = nx.DiGraph()
            node_vals = {a: people[a] for a in _NODE_ATTRS}
            for i in range(n):
                self.graph.add_node(i, **{a: node_vals[a][i] for a in _NODE_ATTRS})
            for entry in self.infection_log:
                if entry['source'] is not None:
                    self.graph.add_edge(entry['source'], entry['target'], date=entry['date'], layer=entry['layer'])

    def _person_array(self, people, attr):
        """An agent array on the log's device (ages are host arrays of People)."""
        try:
            return people.gpu(attr)
        except (KeyError, AttributeError):
            return torch.as_tensor(np.asarray(people[attr]), device=self._log.device)

    def _layer_name(self, layer, src, day):
        return log_layer_label(layer, self._layer_names, self._log_labels)

    @property
    def infection_log(self):
        """people.py:508-511 records: dict(source, target, date, layer, variant)."""
        if self._inflog is None:
            self._inflog = self._people.infection_log
        return self._inflog

    def _build_lists(self):
        log = self._log.cpu().numpy()
        n = self.pop_size
        src_of = self.source_of.cpu().numpy()
        src_date = self.source_date.cpu().numpy()
        sources = [None if s < 0 else int(s) for s in src_of.tolist()]
        source_dates = [None if s < 0 else int(d) for s, d in zip(src_of.tolist(), src_date.tolist())]
        targets = [[] for _ in range(n)]
        target_dates = [[] for _ in range(n)]
        for s, g, d in log[log[:, 0] > 0][:, :3].tolist():
            targets[s].append(g)
            target_dates[s].append(d)
        self._lists = (sources, targets, source_dates, target_dates)

    @property
    def sources(self):
        if self._lists is None:
            self._build_lists()
        return self._lists[0]

    @property
    def targets(self):
        if self._lists is None:
            self._build_lists()
        return self._lists[1]

    @property
    def source_dates(self):
        if self._lists is None:
            self._build_lists()
        return self._lists[2]

    @property
    def target_dates(self):
        if self._lists is None:
            self._build_lists()
        return self._lists[3]

    def __len__(self):
        return int(self._log.shape[0])

    def day(self, day=None, which=None):
        if day is not None:
            return to_day(day, self.sim_start)
        if which == 'start':
            return 0
        if which == 'end':
            return self.n_days
        return None

    def count_targets(self, start_day=None, end_day=None):
        """Targets of each agent who was infected by someone (a source other than
        agent 0) between start_day and end_day, in agent order (analysis.py:1888-1912)."""
        start_day = self.day(start_day, which='start')
        end_day = self.day(end_day, which='end')
        keep = (self.source_of >= 0) & (self.source_date >= start_day) & (self.source_date <= end_day)
        self.n_targets = self.n_targets_all[keep].cpu().numpy().astype(np.float64)
        return self.n_targets

    def count_transmissions(self):
        """[source, target] of every record with a source (analysis.py:1915-1934)."""
        log = self._log
        with_src = log[log[:, 0] >= 0]
        pairs = with_src[:, :2].cpu().numpy()
        self.source_inds = pairs[:, 0].tolist()
        self.target_inds = pairs[:, 1].tolist()
        self.transmissions = pairs.tolist()
        return self.transmissions

    def make_detailed(self, people, reset=False):
        """Per-agent columns of each target's last infection and its source, and the
        per-transmission table ``df`` (analysis.py:1937-2032)."""
        log = self._log
        n = self.pop_size
        dev = log.device
        src, tgt, day, layer = log[:, 0], log[:, 1], log[:, 2], log[:, 3]
        last = _last_per_target(tgt, None, n)
        infected = last >= 0
        li = last.clamp(min=0)
        nan = torch.full((n,), float('nan'), dtype=torch.float64, device=dev)
        src_last = src[li]
        src_arr = torch.where(infected & (src_last >= 0), src_last.double(), nan)
        trg_arr = torch.where(infected, torch.arange(n, device=dev, dtype=torch.float64), nan)
        date_arr = torch.where(infected, day[li].double(), nan)

        vi_t = torch.nonzero(torch.isfinite(trg_arr) & torch.isfinite(src_arr)).flatten()
        vs_t = src_arr[vi_t].long()
        ti_t = torch.nonzero(infected).flatten()
        vinf = date_arr[vi_t]
        tinf = date_arr[ti_t]
        vi, vs, ti = vi_t.cpu().numpy(), vs_t.cpu().numpy(), ti_t.cpu().numpy()
        vinfdates, tinfdates = vinf.cpu().numpy(), tinf.cpu().numpy()

        def col():
            return np.full(n, np.nan)

        dd = {}
        dd['source'] = col()
        dd['source'][vi] = vs
        dd['target'] = col()
        dd['target'][ti] = ti
        dd['date'] = col()
        dd['date'][ti] = tinfdates
        layer_col = np.array(col(), dtype=object)
        if len(ti):
            rec = log[li[ti_t]].cpu().numpy()  # each target's last record
            layer_col[ti] = [self._layer_name(a, s, d) for s, d, a in rec[:, [0, 2, 3]].tolist()]
        dd['layer'] = layer_col

        for attr in _ATTRS + _QUAR_ATTRS:
            vals = self._person_array(people, attr)
            dd['trg_' + attr] = vals.cpu().numpy()
            dd['src_' + attr] = col()
            if len(vi):
                dd['src_' + attr][vi] = vals[vs_t].double().cpu().numpy()

        lnot = np.logical_not
        dd['src_is_quarantined'] = col()
        q = dd['src_date_quarantined'][vi]
        dd['src_is_quarantined'][vi] = (q <= vinfdates) & lnot(q <= vinfdates)  # as the reference writes it
        date_attrs = [a for a in _ATTRS if a.startswith('date_')]
        for date_attr in date_attrs:
            is_attr = 'src_' + date_attr.replace('date_', 'is_')
            dd[is_attr] = col()
            dd[is_attr][vi] = np.array(dd['src_' + date_attr][vi] <= vinfdates, dtype=bool)
        dd['src_is_asymp'] = col()
        dd['src_is_asymp'][vi] = np.isnan(dd['src_date_symptomatic'][vi])
        dd['src_is_presymp'] = col()
        dd['src_is_presymp'][vi] = lnot(dd['src_is_asymp'][vi].astype(bool)) & lnot(
            dd['src_is_symptomatic'][vi].astype(bool))
        dd['trg_is_quarantined'] = col()
        dd['trg_is_quarantined'][ti] = ((dd['trg_date_quarantined'][ti] <= tinfdates)
                                        & lnot(dd['trg_date_end_quarantine'][ti] <= tinfdates))

        targets = np.array(self.target_inds, dtype=np.int64)
        infdates = dd['date'][targets]
        dtr = {}
        dtr['Day'] = infdates
        dtr['layer'] = dd['layer'][targets]
        dtr['s_asymp'] = np.isnan(dd['src_date_symptomatic'][targets])
        dtr['s_presymp'] = ~(dtr['s_asymp'][:]) & (infdates < dd['src_date_symptomatic'][targets])
        dtr['s_sev'] = dd['src_date_severe'][targets] < infdates
        dtr['s_crit'] = dd['src_date_critical'][targets] < infdates
        dtr['s_diag'] = dd['src_date_diagnosed'][targets] < infdates
        dtr['s_quar'] = ((dd['src_date_quarantined'][targets] < infdates)
                         & lnot(dd['src_date_end_quarantine'][targets] <= infdates))
        dtr['t_quar'] = ((dd['trg_date_quarantined'][targets] < infdates)
                         & lnot(dd['trg_date_end_quarantine'][targets] <= infdates))
        df = DataTable(dtr)
        df = df.rows(np.array([lay != 'seed_infection' for lay in df['layer'].tolist()], dtype=bool))
        stage = np.array(['Symptomatic'] * len(df), dtype=object)
        stage[df['s_asymp']] = 'Asymptomatic'
        stage[df['s_presymp']] = 'Presymptomatic'
        df['Stage'] = stage
        severity = np.array(['Mild'] * len(df), dtype=object)
        severity[df['s_sev']] = 'Severe'
        severity[df['s_crit']] = 'Critical'
        df['Severity'] = severity
        self.detailed = DataTable(dd)
        self.df = df

    def r0(self, recovered_only=False):
        """Mean number of distinct agents each exposed agent infected (analysis.py:2035-2056):
        the mean out-degree of the transmission graph over the agents with a
        date_exposed (with ``recovered_only``, excluding those whose recovery
        falls after the last day). Computed from the device log; the networkx
        graph is not needed."""
        log = self._log
        n = self.pop_size
        with_src = log[log[:, 0] >= 0]
        pairs = torch.unique(with_src[:, 0] * n + with_src[:, 1])
        out_deg = torch.bincount(torch.div(pairs, n, rounding_mode='floor'), minlength=n)[:n]
        de = self._person_array(self._people, 'date_exposed')
        keep = ~torch.isnan(de)
        if recovered_only:
            keep &= ~(self._person_array(self._people, 'date_recovered') > self.n_days)
        if not bool(keep.any()):
            return float('nan')
        return float(out_deg[keep].double().mean().item())


# ----------------------------------------------------------------------------- calibration
class Calibration(Analyzer):
    """Fit parameters of a sim to its data (analysis.py:1358-1660), trials on the GPU in batches.

    Args:
        sim: the sim to calibrate (with data; not run)
        calib_pars (dict): dict(key=[best, low, high]) of the parameters to fit
        fit_args (dict): passed to ``sim.compute_fit()``
        custom_fn (func): ``custom_fn(sim, calib_pars) -> sim`` for parameters that are not sim pars
        par_samplers (dict): per key 'suggest_float' (default), 'suggest_int' or
            'suggest_loguniform' / 'suggest_float_log' (uniform in the logarithm)
        n_trials (int): trials per worker (default 20)
        n_workers (int): trials per generation, run as one batch of sims (default 8)
        total_trials (int): if given, n_trials = ceil(total_trials / n_workers)
        elite_frac (float): the fraction of trials that shapes the next generation
        seed (int): the sampler's seed
        die (bool): raise when a trial fails (else its mismatch is inf)
        verbose (bool): print progress
    """

    def __init__(self, sim, calib_pars=None, fit_args=None, custom_fn=None, par_samplers=None, n_trials=None,
                 n_workers=None, total_trials=None, name=None, db_name=None, keep_db=None, storage=None, label=None,
                 die=False, verbose=True, elite_frac=0.25, seed=0):
        super().__init__(label=label)
        n_trials = 20 if n_trials is None else n_trials
        n_workers = 8 if n_workers is None else n_workers
        if total_trials is not None:
            n_trials = np.ceil(total_trials / n_workers)
        self.run_args = dict(n_trials=int(n_trials), n_workers=int(n_workers), name=name or 'covasim_calibration')
        self.sim = sim
        self.calib_pars = calib_pars
        self.fit_args = dict(fit_args or {})
        self.par_samplers = dict(par_samplers or {})
        self.custom_fn = custom_fn
        self.die = die
        self.verbose = verbose
        self.elite_frac = elite_frac
        self.seed = seed
        self.calibrated = False
        if self.sim.complete:
            warnings.warn('Sim has already been run; re-initializing, but in future, use a sim that has not been run')
            self.sim = self.sim.copy()

    # -- one trial --
    def _make_sim(self, calib_pars, label=None):
        sim = self.sim.copy()
        if label:
            sim.label = label
        valid = {k: v for k, v in calib_pars.items() if k in sim.pars}
        sim.update_pars(valid)
        if self.custom_fn:
            sim = self.custom_fn(sim, calib_pars)
        elif len(valid) != len(calib_pars):
            extra = set(calib_pars) - set(valid)
            raise ValueError('The following parameters are not part of the sim, nor is a custom function specified '
                             f'to use them: {", ".join(sorted(extra))}')
        return sim

    def run_sim(self, calib_pars, label=None, return_sim=False):
        """Run one sim with these parameters; its mismatch (or the sim)."""
        sim = self._make_sim(calib_pars, label)
        try:
            sim.run()
            sim.compute_fit(**self.fit_args)
            return sim if return_sim else sim.fit.mismatch
        except Exception as E:
            if self.die:
                raise
            warnings.warn(f'Encountered error running sim with parameters {calib_pars}: {E}')
            return None if return_sim else np.inf

    def run_batch(self, par_sets):
        """Mismatches of a generation of trials, run together as one BatchSim."""
        from .batch import BatchSim
        try:
            sims = [self._make_sim(p) for p in par_sets]
        except Exception:
            if self.die:
                raise
            return [self.run_sim(p) for p in par_sets]
        try:
            BatchSim(sims).run().finalize()
            out = []
            for s in sims:
                s.compute_fit(**self.fit_args)
                out.append(float(s.fit.mismatch))
            return out
        except Exception as E:
            if self.die:
                raise
            warnings.warn(f'Encountered error running a batch of {len(sims)} trials: {E}')
            return [np.inf] * len(sims)

    # -- the sampler --
    def _kind(self, key):
        s = self.par_samplers.get(key, 'suggest_float')
        if s in ('suggest_float', 'suggest_uniform'):
            return 'float'
        if s == 'suggest_int':
            return 'int'
        if s in ('suggest_loguniform', 'suggest_float_log'):
            return 'log'
        raise AttributeError(f'The requested sampler function {s!r} is not supported')

    def _to_unit(self, key, x):
        _, low, high = self.calib_pars[key]
        if self._kind(key) == 'log':
            return (math.log(x) - math.log(low)) / (math.log(high) - math.log(low))
        return (x - low) / (high - low)

    def _from_unit(self, key, u):
        _, low, high = self.calib_pars[key]
        u = min(max(u, 0.0), 1.0)
        kind = self._kind(key)
        if kind == 'log':
            return float(math.exp(math.log(low) + u * (math.log(high) - math.log(low))))
        x = low + u * (high - low)
        return int(round(x)) if kind == 'int' else float(x)

    def _sample(self, rng, n, elite):
        keys = list(self.calib_pars.keys())
        if elite is None:
            units = rng.random((n, len(keys)))
        else:
            e = np.array([[self._to_unit(k, p[k]) for k in keys] for p in elite])
            mu = e.mean(axis=0)
            sd = np.maximum(e.std(axis=0), 0.02)
            units = np.empty((n, len(keys)))
            for j in range(len(keys)):  # truncated normal on [0, 1] by resampling
                col = rng.normal(mu[j], sd[j], size=n)
                for _ in range(64):
                    bad = (col < 0) | (col > 1)
                    if not bad.any():
                        break
                    col[bad] = rng.normal(mu[j], sd[j], size=int(bad.sum()))
                units[:, j] = np.clip(col, 0, 1)
        return [{k: self._from_unit(k, units[i, j]) for j, k in enumerate(keys)} for i in range(n)]

    def calibrate(self, calib_pars=None, verbose=True, **kwargs):
        """Run n_trials generations of n_workers trials; keep the best."""
        if calib_pars is not None:
            self.calib_pars = calib_pars
        if self.calib_pars is None:
            raise ValueError('You must supply calibration parameters either when creating the calibration object '
                             'or when calling calibrate().')
        self.run_args.update(kwargs)
        t0 = time.perf_counter()
        rng = np.random.default_rng(self.seed)
        n_gen, width = self.run_args['n_trials'], self.run_args['n_workers']
        self.trials = []
        elite = None
        for g in range(n_gen):
            par_sets = self._sample(rng, width, elite)
            mism = self.run_batch(par_sets)
            for p, m in zip(par_sets, mism):
                self.trials.append({'number': len(self.trials), 'value': None if not np.isfinite(m) else float(m),
                                    'params': p})
            done = [t for t in self.trials if t['value'] is not None]
            if done:
                k = max(2, int(math.ceil(self.elite_frac * len(done))))
                elite = [t['params'] for t in sorted(done, key=lambda t: t['value'])[:k]]
            if self.verbose and verbose:
                best = min((t['value'] for t in done), default=None)
                print(f'  generation {g + 1}/{n_gen}: {len(done)} trials, best mismatch {best}')
        done = [t for t in self.trials if t['value'] is not None]
        if not done:
            raise RuntimeError('every calibration trial failed')
        self.best_pars = dict(min(done, key=lambda t: t['value'])['params'])
        self.elapsed = time.perf_counter() - t0
        self.initial_pars = {k: v[0] for k, v in self.calib_pars.items()}
        self.par_bounds = {k: np.array([v[1], v[2]]) for k, v in self.calib_pars.items()}
        self.before = self.run_sim(calib_pars=self.initial_pars, label='Before calibration', return_sim=True)
        self.after = self.run_sim(calib_pars=self.best_pars, label='After calibration', return_sim=True)
        self.parse_study()
        self.calibrated = True
        if verbose and self.verbose:
            self.summarize()
        return self

    def summarize(self):
        if not self.calibrated:
            print('Calibration not yet run; please run calib.calibrate()')
            return None
        before, after = self.before.fit.mismatch, self.after.fit.mismatch
        print(f'Calibration for {len(self.trials)} total trials completed in {self.elapsed:0.1f} s.')
        print('\nInitial parameter values:')
        print(self.initial_pars)
        print('\nBest parameter values:')
        print(self.best_pars)
        print(f'\nMismatch before calibration: {before:n}')
        print(f'Mismatch after calibration:  {after:n}')
        print(f'Percent improvement:         {((before - after) / before) * 100:0.1f}%')
        return before, after

    def parse_study(self):
        """The trials as columns: index, mismatch and one per parameter (analysis.py:1600-1630)."""
        best = self.best_pars
        keys = ['index', 'mismatch'] + list(best.keys())
        data = {k: [] for k in keys}
        for t in self.trials:
            if t['value'] is None:
                continue
            row = {'index': t['number'], 'mismatch': t['value'], **t['params']}
            for k in keys:
                data[k].append(row.get(k, best.get(k)))
        self.data = data
        self.df = DataTable({k: np.asarray(v) for k, v in data.items()})

    def to_json(self, filename=None):
        order = np.argsort(self.df['mismatch'], kind='stable')
        out = []
        for o in order:
            row = {k: self.df[k][o].item() for k in self.df.columns}
            out.append(dict(index=row.pop('index'), mismatch=row.pop('mismatch'), pars=row))
        if filename:
            with open(filename, 'w') as fh:
                json.dump(out, fh, indent=2)
            return None
        return out
