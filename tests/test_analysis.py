"""Result consumers: TransTree, Fit, compute_gof, load_data and the calibration
sampler, against the outputs of the reference's own code (ref_analysis.npz)
and the oracle's restatement. CPU only: the transmission tree's device passes
run here on CPU tensors fed from the fixture's infection log."""
import datetime as dt
import json
import os

import numpy as np
import pytest
import torch

from covasim_gb300 import analysis as cva
from covasim_gb300 import _lib as L
from oracle import analysis as oa

HERE = os.path.dirname(os.path.abspath(__file__))
FIX = np.load(os.path.join(HERE, 'golden', 'ref_analysis.npz'))
LAYERS = ['h', 's', 'w', 'c']
START = dt.date(2020, 3, 1)


def fixture_log():
    src, tgt, day, lay = FIX['log.source'], FIX['log.target'], FIX['log.date'], FIX['log.layer']
    return [dict(source=None if s < 0 else int(s), target=int(g), date=int(d), layer=str(l), variant='wild')
            for s, g, d, l in zip(src, tgt, day, lay)]


def fixture_people():
    return {k.split('.', 1)[1]: FIX[k] for k in FIX.files if k.startswith('people.')}


# ----------------------------------------------------------------------------- stand-in sim for TransTree
class _Res:
    def __init__(self, v):
        self.values = np.asarray(v)


class _People:
    def __init__(self, arrays, n, t, log):
        self._arrays = {k: torch.as_tensor(v) for k, v in arrays.items()}
        self._n, self.t, self._sim = n, t, 0
        self.infection_log = log

    def gpu(self, key):
        return self._arrays[key]

    def __getitem__(self, key):
        return self._arrays[key].numpy()

    def __len__(self):
        return self._n

    def layer_keys(self):
        return LAYERS


class _State:
    def __init__(self, log):
        rows = []
        for e in log:
            if e['layer'] in LAYERS:
                li = LAYERS.index(e['layer'])
            else:  # seeds and importations carry tags above the layer indices
                li = {'seed_infection': L.LOG_SEED, 'importation': L.LOG_IMPORT}[e['layer']]
            rows.append([-1 if e['source'] is None else e['source'], e['target'], e['date'], li, 0])
        self._log = torch.tensor(rows, dtype=torch.int64).reshape(-1, 5)

    def infection_log_tensor(self, sim):
        return self._log


class _Sim:
    def __init__(self, log, people, n, n_days):
        self.people = _People(people, n, n_days, log)
        self.state = _State(log)
        self.results = {'t': np.arange(n_days + 1), 'cum_infections': _Res(np.zeros(n_days + 1))}

    def __getitem__(self, k):
        return {'start_day': '2020-03-01', 'rescale': True, 'pop_scale': 1}[k]


def check_transtree(tt_get, prefix='tt.'):
    """Compare a dict-like of TransTree outputs with the fixture."""
    np.testing.assert_array_equal(tt_get('sources'), FIX[prefix + 'sources'])
    np.testing.assert_array_equal(tt_get('source_dates'), FIX[prefix + 'source_dates'])
    np.testing.assert_array_equal(tt_get('targets_count'), FIX[prefix + 'targets_count'])
    np.testing.assert_array_equal(tt_get('targets_flat'), FIX[prefix + 'targets_flat'])
    np.testing.assert_array_equal(tt_get('target_dates_flat'), FIX[prefix + 'target_dates_flat'])
    np.testing.assert_array_equal(tt_get('n_targets'), FIX[prefix + 'n_targets'])
    np.testing.assert_array_equal(tt_get('n_targets_10_25'), FIX[prefix + 'n_targets_10_25'])
    np.testing.assert_array_equal(tt_get('transmissions'), FIX[prefix + 'transmissions'])
    assert tt_get('r0_0') == pytest.approx(float(FIX[prefix + 'r0_0']), rel=1e-12)
    assert tt_get('r0_1') == pytest.approx(float(FIX[prefix + 'r0_1']), rel=1e-12)
    det = tt_get('detailed')
    for k in FIX.files:
        if k.startswith(prefix + 'detailed.'):
            col = k.split('.', 2)[2]
            ref = FIX[k]
            got = det[col]
            if ref.dtype.kind == 'U':
                np.testing.assert_array_equal(np.array([str(x) for x in got]), ref, err_msg=col)
            else:
                np.testing.assert_array_equal(np.asarray(got, dtype=np.float64), ref, err_msg=col)
    df = tt_get('df')
    for k in FIX.files:
        if k.startswith(prefix + 'df.'):
            col = k.split('.', 2)[2]
            ref = FIX[k]
            got = np.asarray(df[col])
            if ref.dtype.kind == 'U':
                got = np.array([str(x) for x in got])
            np.testing.assert_array_equal(got, ref, err_msg=col)


def _flat(lists):
    return np.array([x for sub in lists for x in sub], dtype=np.int64)


def test_oracle_transtree_matches_the_reference():
    n, n_days = (int(x) for x in FIX['meta'])
    o = oa.transtree(fixture_log(), fixture_people(), n, n_days, start_day=10, end_day=25)

    def get(k):
        if k in ('sources', 'source_dates'):
            return np.array([-1 if s is None else s for s in o[k]], dtype=np.int64)
        if k == 'targets_count':
            return np.array([len(t) for t in o['targets']], dtype=np.int64)
        if k == 'targets_flat':
            return _flat(o['targets'])
        if k == 'target_dates_flat':
            return _flat(o['target_dates'])
        if k == 'n_targets_10_25':
            return o['n_targets_window']
        if k == 'transmissions':
            return np.array(o['transmissions'], dtype=np.int64).reshape(-1, 2)
        return o[k]
    check_transtree(get)


def test_transtree_device_passes_match_the_reference():
    n, n_days = (int(x) for x in FIX['meta'])
    sim = _Sim(fixture_log(), fixture_people(), n, n_days)
    tt = cva.TransTree(sim)
    assert len(tt) == len(FIX['log.target'])

    def get(k):
        if k in ('sources', 'source_dates'):
            return np.array([-1 if s is None else s for s in getattr(tt, k)], dtype=np.int64)
        if k == 'targets_count':
            return np.array([len(t) for t in tt.targets], dtype=np.int64)
        if k == 'targets_flat':
            return _flat(tt.targets)
        if k == 'target_dates_flat':
            return _flat(tt.target_dates)
        if k == 'n_targets':
            return tt.count_targets()
        if k == 'n_targets_10_25':
            return tt.count_targets(10, '2020-03-26')  # day 25 as a date
        if k == 'transmissions':
            return np.array(tt.transmissions, dtype=np.int64).reshape(-1, 2)
        if k == 'r0_0':
            return tt.r0()
        if k == 'r0_1':
            return tt.r0(recovered_only=True)
        return getattr(tt, k)
    check_transtree(get)


def test_transtree_networkx_graph():
    nx = pytest.importorskip('networkx')
    n, n_days = (int(x) for x in FIX['meta'])
    sim = _Sim(fixture_log(), fixture_people(), n, n_days)
    tt = cva.TransTree(sim, to_networkx=True)
    assert isinstance(tt.graph, nx.DiGraph)
    assert tt.graph.number_of_nodes() == n
    assert tt.graph.number_of_edges() == len({tuple(t) for t in FIX['tt.transmissions'].tolist()})


# ----------------------------------------------------------------------------- goodness of fit
def test_compute_gof_matches_the_reference():
    a, b = FIX['gof.actual'], FIX['gof.predicted']
    for i, kw in enumerate(json.loads(str(FIX['gof.cases']))):
        ref = FIX[f'gof.out{i}']
        np.testing.assert_allclose(cva.compute_gof(a, b, **kw), ref, rtol=1e-15, atol=0, err_msg=str(kw))
        np.testing.assert_allclose(oa.gof(a, b, **kw), ref, rtol=1e-12, atol=0, err_msg=str(kw))


def test_compute_gof_custom_estimator():
    a, b = FIX['gof.actual'], FIX['gof.predicted']
    assert cva.compute_gof(a, b, estimator=lambda x, y: float(np.max(np.abs(x - y)))) == np.max(np.abs(a - b))
    with pytest.raises(RuntimeError):
        cva.compute_gof(a, b, estimator=lambda x: 0)


def _decode(obj):
    if isinstance(obj, dict):
        if '__array__' in obj:
            return np.array(obj['__array__'], dtype=obj.get('dtype', None))
        return {k: _decode(v) for k, v in obj.items()}
    if isinstance(obj, list):
        return [_decode(x) for x in obj]
    return obj


class _FitSim:
    def __init__(self):
        npts = len(FIX['simres.cum_deaths'])
        self.npts = npts
        self.datevec = np.array([START + dt.timedelta(days=d) for d in range(npts)], dtype=object)
        self.results = {k.split('.', 1)[1]: _Res(FIX[k]) for k in FIX.files if k.startswith('simres.')}
        self.results['t'] = np.arange(npts)
        self.results['date'] = self.datevec
        self.results_ready = True
        cols = {k.split('.', 1)[1]: FIX[k] for k in FIX.files if k.startswith('data.') and k != 'data.days'}
        cols['date'] = [START + dt.timedelta(days=int(d)) for d in FIX['data.days']]
        self.data = cva.load_data(cols, calculate=False)

    def result_keys(self):
        # the reference's result order: cum_ keys in flow order (tests, diagnoses ... deaths)
        order = ['cum_infections', 'cum_tests', 'cum_diagnoses', 'cum_deaths', 'new_infections']
        return [k for k in order if k in self.results]


def test_fit_matches_the_reference():
    for i, kw in enumerate(_decode(json.loads(str(FIX['fit.cases'])))):
        sim = _FitSim()
        fit = cva.Fit(sim, **kw)
        ref_keys = list(FIX[f'fit.keys{i}'])
        assert sorted(fit.mismatches) == sorted(ref_keys)
        for k, v in zip(ref_keys, FIX[f'fit.mismatches{i}']):
            assert fit.mismatches[k] == pytest.approx(v, rel=1e-13), (i, k)
        assert fit.mismatch == pytest.approx(float(FIX[f'fit.mismatch{i}']), rel=1e-13)


def test_oracle_fit_matches_the_reference():
    sim = _FitSim()
    series = {k: v.values for k, v in sim.results.items() if hasattr(v, 'values')}
    cols = {k.split('.', 1)[1]: FIX[k] for k in FIX.files if k.startswith('data.') and k != 'data.days'}
    dates = [START + dt.timedelta(days=int(d)) for d in FIX['data.days']]
    for i, kw in enumerate(_decode(json.loads(str(FIX['fit.cases'])))):
        if 'custom' in kw:
            continue
        gkw = {k: v for k, v in kw.items() if k not in ('keys', 'weights')}
        mism, total = oa.fit(series, list(sim.datevec), cols, dates, keys=kw.get('keys'), weights=kw.get('weights'),
                             **gkw)
        assert total == pytest.approx(float(FIX[f'fit.mismatch{i}']), rel=1e-12)


def test_fit_errors():
    sim = _FitSim()
    sim.data = None
    with pytest.raises(RuntimeError):
        cva.Fit(sim)
    sim = _FitSim()
    with pytest.raises(KeyError):
        cva.Fit(sim, keys=['cum_severe'])


# ----------------------------------------------------------------------------- data
def test_load_data_csv(tmp_path):
    path = tmp_path / 'data.csv'
    path.write_text('date,new_diagnoses,new_deaths,cum_deaths\n'
                    '2020-03-02,1,0,0\n2020-03-03,,1,1\n2020-03-05,4,0,1\n')
    d = cva.load_data(str(path), verbose=False)
    assert d.columns == ['date', 'new_diagnoses', 'new_deaths', 'cum_deaths', 'cum_diagnoses']
    assert list(d['date']) == [dt.date(2020, 3, 2), dt.date(2020, 3, 3), dt.date(2020, 3, 5)]
    np.testing.assert_array_equal(d['cum_diagnoses'], [1.0, np.nan, 5.0])  # missing stays missing
    np.testing.assert_array_equal(d['cum_deaths'], [0.0, 1.0, 1.0])  # present: not recomputed
    path2 = tmp_path / 'days.csv'
    path2.write_text('date,cum_tests\n0,3\n2,8\n')
    d2 = cva.load_data(str(path2), start_day='2020-03-01', verbose=False)
    assert list(d2['date']) == [dt.date(2020, 3, 1), dt.date(2020, 3, 3)]
    with pytest.raises(ValueError):
        cva.load_data({'cum_tests': [1, 2]}, verbose=False)
    with pytest.raises(NotImplementedError):
        cva.load_data('data.xlsx')


def test_dates():
    assert cva.to_day('2020-03-11', '2020-03-01') == 10
    assert cva.to_day(dt.date(2020, 2, 28), '2020-03-01') == -2
    assert cva.to_day(7, '2020-03-01') == 7
    assert cva.to_date('2021-01-05T00:00') == dt.date(2021, 1, 5)


# ----------------------------------------------------------------------------- calibration sampler
class _CalSim:
    complete = False
    pars = {'beta': 0.016, 'n_imports': 0}


def test_calibration_sampler_stays_in_bounds():
    cal = cva.Calibration(_CalSim(), calib_pars=dict(beta=[0.015, 0.01, 0.03], n_imports=[0, 0, 5],
                                                     rel_death_prob=[1.0, 0.1, 10.0]),
                          par_samplers=dict(n_imports='suggest_int', rel_death_prob='suggest_loguniform'))
    rng = np.random.default_rng(1)
    first = cal._sample(rng, 200, None)
    assert all(0.01 <= p['beta'] <= 0.03 for p in first)
    assert all(isinstance(p['n_imports'], int) and 0 <= p['n_imports'] <= 5 for p in first)
    logs = np.log10([p['rel_death_prob'] for p in first])
    assert logs.min() >= -1 and logs.max() <= 1 and abs(np.median(logs)) < 0.2  # uniform in the logarithm
    elite = [dict(beta=0.02, n_imports=2, rel_death_prob=2.0), dict(beta=0.021, n_imports=3, rel_death_prob=2.5)]
    nxt = cal._sample(rng, 200, elite)
    betas = np.array([p['beta'] for p in nxt])
    assert 0.01 <= betas.min() and betas.max() <= 0.03
    assert abs(np.median(betas) - 0.0205) < 0.002  # concentrated on the elite
    with pytest.raises(AttributeError):
        cva.Calibration(_CalSim(), calib_pars=dict(beta=[0.015, 0.01, 0.03]),
                        par_samplers=dict(beta='suggest_categorical'))._sample(rng, 2, None)
