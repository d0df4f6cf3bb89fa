"""Oracle (test infrastructure only): plain-Python restatement of the reference's
result consumers, for checking ``covasim_gb300.analysis``.

* ``transtree``  covasim/analysis.py:1796-2056 (TransTree.__init__,
  count_targets, count_transmissions, make_detailed, r0)
* ``gof``        covasim/misc.py:707-790 (compute_gof, default estimator)
* ``fit``        covasim/analysis.py:1022-1222 (Fit: pairing by date, diffs,
  goodness of fit, weighted losses, mismatch)

Pinned by ``tests/golden/ref_analysis.npz``, which holds the outputs of the
reference's own TransTree / Fit / compute_gof code on a reference run.
Records are dicts (source None for seeds and importations, target, date,
layer name, variant), the people arrays a dict of numpy arrays.
"""
import math

import numpy as np

ATTRS = ['age', 'date_exposed', 'date_symptomatic', 'date_tested', 'date_diagnosed', 'date_severe', 'date_critical',
         'date_known_contact']
QUAR_ATTRS = ['date_quarantined', 'date_end_quarantine']


def transtree(log, people, pop_size, n_days, start_day=None, end_day=None):
    """Every output of the reference's TransTree for one infection log."""
    out = {}
    # analysis.py:1823-1836: per-agent maps; `if source:` skips agent 0 and seeds
    sources = [None] * pop_size
    targets = [[] for _ in range(pop_size)]
    source_dates = [None] * pop_size
    target_dates = [[] for _ in range(pop_size)]
    for rec in log:
        s, g, d = rec['source'], rec['target'], rec['date']
        if s:
            sources[g] = s
            targets[s].append(g)
            source_dates[g] = d
            target_dates[s].append(d)
    out.update(sources=sources, targets=targets, source_dates=source_dates, target_dates=target_dates)

    # analysis.py:1888-1912
    def count_targets(start, end):
        start = 0 if start is None else start
        end = n_days if end is None else end
        res = []
        for i in range(pop_size):
            if sources[i] is not None and start <= source_dates[i] <= end:
                res.append(float(len(targets[i])))
        return np.array(res, dtype=np.float64)
    out['n_targets'] = count_targets(None, None)
    out['n_targets_window'] = count_targets(start_day, end_day)

    # analysis.py:1915-1934
    trans = [[r['source'], r['target']] for r in log if r['source'] is not None]
    out['transmissions'] = trans
    out['source_inds'] = [t[0] for t in trans]
    out['target_inds'] = [t[1] for t in trans]

    # analysis.py:1937-2032: each target's last record
    last = {}
    for k, rec in enumerate(log):
        last[rec['target']] = k
    nanarr = lambda: np.full(pop_size, np.nan)  # noqa: E731
    dd = {'source': nanarr(), 'target': nanarr(), 'date': nanarr(), 'layer': np.array(nanarr(), dtype=object)}
    vi, vs, vdates = [], [], []
    for g in sorted(last):
        rec = log[last[g]]
        dd['target'][g] = g
        dd['date'][g] = rec['date']
        dd['layer'][g] = rec['layer']
        if rec['source'] is not None:
            dd['source'][g] = rec['source']
            vi.append(g)
            vs.append(rec['source'])
            vdates.append(rec['date'])
    vi = np.array(vi, dtype=np.int64)
    vs = np.array(vs, dtype=np.int64)
    vdates = np.array(vdates, dtype=np.float64)
    ti = np.array(sorted(last), dtype=np.int64)
    tdates = dd['date'][ti]
    for attr in ATTRS + QUAR_ATTRS:
        dd['trg_' + attr] = np.asarray(people[attr]).copy()
        col = nanarr()
        col[vi] = np.asarray(people[attr])[vs]
        dd['src_' + attr] = col
    col = nanarr()
    col[vi] = 0.0  # (q <= d) & not (q <= d): never true, as the reference writes it
    dd['src_is_quarantined'] = col
    for attr in ATTRS:
        if attr.startswith('date_'):
            col = nanarr()
            col[vi] = (dd['src_' + attr][vi] <= vdates).astype(np.float64)
            dd['src_' + attr.replace('date_', 'is_')] = col
    col = nanarr()
    col[vi] = np.isnan(dd['src_date_symptomatic'][vi]).astype(np.float64)
    dd['src_is_asymp'] = col
    col = nanarr()
    col[vi] = ((dd['src_is_asymp'][vi] == 0) & (dd['src_is_symptomatic'][vi] == 0)).astype(np.float64)
    dd['src_is_presymp'] = col
    col = nanarr()
    col[ti] = ((dd['trg_date_quarantined'][ti] <= tdates)
               & ~(dd['trg_date_end_quarantine'][ti] <= tdates)).astype(np.float64)
    dd['trg_is_quarantined'] = col
    out['detailed'] = dd

    tg = np.array(out['target_inds'], dtype=np.int64)
    day = dd['date'][tg]
    df = {'Day': day, 'layer': dd['layer'][tg]}
    df['s_asymp'] = np.isnan(dd['src_date_symptomatic'][tg])
    df['s_presymp'] = ~df['s_asymp'] & (day < dd['src_date_symptomatic'][tg])
    df['s_sev'] = dd['src_date_severe'][tg] < day
    df['s_crit'] = dd['src_date_critical'][tg] < day
    df['s_diag'] = dd['src_date_diagnosed'][tg] < day
    df['s_quar'] = (dd['src_date_quarantined'][tg] < day) & ~(dd['src_date_end_quarantine'][tg] <= day)
    df['t_quar'] = (dd['trg_date_quarantined'][tg] < day) & ~(dd['trg_date_end_quarantine'][tg] <= day)
    keep = np.array([lay != 'seed_infection' for lay in df['layer']], dtype=bool)
    df = {k: v[keep] for k, v in df.items()}
    stage = []
    sev = []
    for a, p, s, c in zip(df['s_asymp'], df['s_presymp'], df['s_sev'], df['s_crit']):
        stage.append('Presymptomatic' if p else ('Asymptomatic' if a else 'Symptomatic'))
        sev.append('Critical' if c else ('Severe' if s else 'Mild'))
    df['Stage'] = np.array(stage, dtype=object)
    df['Severity'] = np.array(sev, dtype=object)
    out['df'] = df

    # analysis.py:2035-2056: mean out-degree of the (deduplicated) transmission graph
    succ = [set() for _ in range(pop_size)]
    for s, g in trans:
        succ[s].add(g)
    de = np.asarray(people['date_exposed'])
    dr = np.asarray(people['date_recovered'])
    for flag in (False, True):
        vals = [len(succ[i]) for i in range(pop_size)
                if not (math.isnan(de[i]) or (flag and dr[i] > n_days))]
        out[f'r0_{int(flag)}'] = float(np.mean(vals)) if vals else float('nan')
    return out


def gof(actual, predicted, normalize=True, use_frac=False, use_squared=False, as_scalar='none', eps=1e-9):
    """misc.py:765-790, one element at a time."""
    actual = [float(a) for a in actual]
    predicted = [float(p) for p in predicted]
    g = [abs(a - p) for a, p in zip(actual, predicted)]
    if normalize and not use_frac:
        amax = max(abs(a) for a in actual) if actual else 0.0
        if amax > 0:
            g = [x / amax for x in g]
    if use_frac and not (any(a < 0 for a in actual) or any(p < 0 for p in predicted)):
        g = [x / (max(a, p) + eps) for x, a, p in zip(g, actual, predicted)]
    if use_squared:
        g = [x * x for x in g]
    g = np.array(g)
    if as_scalar == 'sum':
        return float(np.sum(g))
    if as_scalar == 'mean':
        return float(np.mean(g))
    if as_scalar == 'median':
        return float(np.median(g))
    return g


def fit(sim_series, sim_dates, data_cols, data_dates, keys=None, weights=None, **gof_kwargs):
    """Mismatch of sim series (dict key -> values per sim day) against data
    columns (dict key -> values per data row), paired by date; returns
    (mismatches by key, total)."""
    w = {'cum_deaths': 10, 'cum_diagnoses': 5, **(weights or {})}
    if keys is None:
        keys = [k for k in sim_series if k.startswith('cum_') and k in data_cols]
    mism = {}
    for key in keys:
        sim_vals, dat_vals = [], []
        for j, d in enumerate(data_dates):
            v = data_cols[key][j]
            if np.isfinite(v) and d in sim_dates:
                sim_vals.append(sim_series[key][sim_dates.index(d)])
                dat_vals.append(v)
        g = gof(dat_vals, sim_vals, **gof_kwargs)
        wt = w.get(key, 1.0)
        if np.iterable(wt):
            wt = np.asarray(wt)
            if len(wt) == len(sim_dates):
                wt = wt[[sim_dates.index(d) for j, d in enumerate(data_dates)
                         if np.isfinite(data_cols[key][j]) and d in sim_dates]]
        mism[key] = float(np.sum(g * wt))
    return mism, float(np.array(list(mism.values())).sum())
