"""Synthetic populations (random and hybrid), vectorised on the host.

Same distributions as Covasim 3.1.7's generators (covasim/population.py):
ages from the default age table (population.py:143-226), random layers with
round(Poisson(n)/2) partners per agent drawn uniformly (population.py:241-284),
household clusters of Poisson(h) size with all pairs inside each cluster
(population.py:287-329), and the hybrid school/work/community layers
(population.py:332-364). Draws come from a numpy ``Generator`` (PCG64); the
loops over agents of the reference become array operations. Population
building runs once per sim, before the day loop. ``make_randpop_device`` and
``set_prognoses_device`` build the same distributions on the GPU
(covgpu_pop.cu), with Philox draws.
"""
import numpy as np

from . import defaults as cvd

__all__ = ['make_randpop', 'make_random_contacts', 'make_microstructured_contacts', 'make_hybrid_contacts',
           'sample_ages', 'make_randpop_device', 'set_prognoses_device']


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


# ----------------------------------------------------------------------------- on the device
def _dev_call(name, *args):
    from . import _lib as L
    from .state import _stream
    L.call(name, *args, _stream())


def _dev_scan_scratch(n, device):
    import torch
    from . import _lib as L
    return torch.empty(int(L.lib().covgpu_pop_scan_scratch(int(n))) + 1, dtype=torch.int64, device=device)


def _dev_random_layer(n_members, mean, seed, layer, status, device, members=None, dispersion=None):
    """population.py:241-284 on the device: (p1, p2) int32 tensors, p1 ascending."""
    import torch
    if n_members == 0:
        z = torch.zeros(0, dtype=torch.int32, device=device)
        return z, z.clone()
    counts = torch.empty(n_members, dtype=torch.int64, device=device)
    offsets = torch.empty(n_members + 1, dtype=torch.int64, device=device)
    _dev_call('covgpu_pop_random_counts', n_members, float(mean), float(dispersion or 0.0), seed, layer,
              counts.data_ptr(), offsets.data_ptr(), _dev_scan_scratch(n_members, device).data_ptr(),
              status.data_ptr())
    n_edges = int(offsets[-1].item())
    p1 = torch.empty(n_edges, dtype=torch.int32, device=device)
    p2 = torch.empty(n_edges, dtype=torch.int32, device=device)
    if n_edges:
        _dev_call('covgpu_pop_random_fill', n_members, None if members is None else members.data_ptr(),
                  offsets.data_ptr(), seed, layer, p1.data_ptr(), p2.data_ptr())
    return p1, p2


def _dev_clusters(pop_size, mean, seed, layer, status, device):
    """population.py:287-329 on the device: every pair inside consecutive Poisson(mean) clusters."""
    import torch
    k = int(pop_size / max(float(mean), 0.5) * 1.2) + 64
    while True:
        sizes = torch.empty(k, dtype=torch.int64, device=device)
        starts = torch.empty(k + 1, dtype=torch.int64, device=device)
        _dev_call('covgpu_pop_cluster_sizes', k, float(mean), seed, layer, sizes.data_ptr(), starts.data_ptr(),
                  _dev_scan_scratch(k, device).data_ptr(), status.data_ptr())
        if int(starts[-1].item()) >= pop_size:
            break
        k *= 2  # more clusters, same draws for the first k (keyed by cluster index)
    counts = torch.empty(pop_size, dtype=torch.int64, device=device)
    offsets = torch.empty(pop_size + 1, dtype=torch.int64, device=device)
    _dev_call('covgpu_pop_cluster_counts', pop_size, k, starts.data_ptr(), counts.data_ptr(), offsets.data_ptr(),
              _dev_scan_scratch(pop_size, device).data_ptr())
    n_edges = int(offsets[-1].item())
    p1 = torch.empty(n_edges, dtype=torch.int32, device=device)
    p2 = torch.empty(n_edges, dtype=torch.int32, device=device)
    if n_edges:
        _dev_call('covgpu_pop_cluster_fill', pop_size, offsets.data_ptr(), p1.data_ptr(), p2.data_ptr())
    return p1, p2


def make_randpop_device(pars, seed, device='cuda', sex_ratio=0.5):
    """``make_randpop`` built on the device (covgpu_pop_*): the same distributions,
    draws from Philox keyed by ``seed``; ages and sexes come back as numpy
    arrays, the layers as device tensors (p1 ascending)."""
    import torch
    from . import _lib as L
    if sex_ratio != 0.5:
        raise NotImplementedError('the device generator draws sexes with ratio 0.5')
    pop_size = int(pars['pop_size'])
    seed = int(seed) & 0xFFFFFFFFFFFFFFFF
    status = torch.zeros(1, dtype=torch.int32, device=device)
    ad = np.asarray(cvd.default_age_data, dtype=float)
    lo, width, cdf = ad[:, 0], ad[:, 1] + 1 - ad[:, 0], np.cumsum(ad[:, 2] / ad[:, 2].sum())
    tabs = [torch.from_numpy(np.ascontiguousarray(x, dtype=np.float64)).to(device) for x in (lo, width, cdf)]
    age = torch.empty(pop_size, dtype=torch.float32, device=device)
    sex = torch.empty(pop_size, dtype=torch.int32, device=device)
    _dev_call('covgpu_pop_ages', pop_size, tabs[0].data_ptr(), tabs[1].data_ptr(), tabs[2].data_ptr(), len(ad), seed,
              age.data_ptr(), sex.data_ptr())
    contacts = {}
    microstructure = pars['pop_type']
    keys = list(pars['contacts'].keys())
    if microstructure == 'random':
        for li, (lkey, n) in enumerate(pars['contacts'].items()):
            p1, p2 = _dev_random_layer(pop_size, n, seed, li, status, device)
            contacts[lkey] = dict(p1=p1, p2=p2)
    elif microstructure == 'hybrid':
        cts = {**dict(h=4, s=20, w=20, c=20), **pars['contacts']}
        p1, p2 = _dev_clusters(pop_size, cts['h'], seed, 0, status, device)
        contacts['h'] = dict(p1=p1, p2=p2)
        p1, p2 = _dev_random_layer(pop_size, cts['c'], seed, 3, status, device)
        contacts['c'] = dict(p1=p1, p2=p2)
        for li, (lkey, (a0, a1)) in ((1, ('s', (6, 22))), (2, ('w', (22, 65)))):
            flags = torch.empty(pop_size, dtype=torch.int64, device=device)
            pos = torch.empty(pop_size + 1, dtype=torch.int64, device=device)
            members = torch.empty(pop_size, dtype=torch.int32, device=device)
            _dev_call('covgpu_pop_members', pop_size, age.data_ptr(), float(a0), float(a1), flags.data_ptr(),
                      pos.data_ptr(), _dev_scan_scratch(pop_size, device).data_ptr(), members.data_ptr())
            m = int(pos[-1].item())
            p1, p2 = _dev_random_layer(m, cts[lkey], seed, li, status, device, members=members[:m])
            contacts[lkey] = dict(p1=p1, p2=p2)
    else:
        raise NotImplementedError(f'Microstructure type "{microstructure}" not found; choices are random or hybrid')
    if int(status.item()) & L.TIMEOUT:
        raise L.CovgpuError('population generation (a sampler ran out of tries)', L.TIMEOUT)
    return dict(uid=np.arange(pop_size, dtype=cvd.default_int), age=age.cpu().numpy().astype(np.float64),
                sex=sex.cpu().numpy(), contacts=contacts, layer_keys=keys, _age_device=age)


def set_prognoses_device(age, pars, seed, device='cuda'):
    """``set_prognoses`` on the device: dict of float32 device tensors."""
    import torch
    from . import _lib as L
    age = age if torch.is_tensor(age) else torch.as_tensor(np.asarray(age, dtype=np.float32))
    age = age.to(device, torch.float32).contiguous()
    n = age.numel()
    progs = pars['prognoses']
    cut = torch.from_numpy(np.ascontiguousarray(progs['age_cutoffs'], dtype=np.float64)).to(device)
    tabs = np.stack([progs['symp_probs'], progs['severe_probs'] * progs['comorbidities'], progs['crit_probs'],
                     progs['death_probs'], progs['sus_ORs'], progs['trans_ORs']]).astype(np.float64)
    tabs_d = torch.from_numpy(np.ascontiguousarray(tabs)).to(device)
    bd = pars['beta_dist']
    if bd['dist'] == 'neg_binomial':
        code, p1, p2, step = 0, float(bd['par1']), float(bd['par2']), float(bd.get('step', 1))
    elif bd['dist'] in ('lognormal', 'lognorm'):
        code, p1, p2, step = 1, float(bd['par1']), float(bd['par2']), 1.0
    else:
        raise NotImplementedError(f'beta_dist "{bd["dist"]}" on the device')
    out = {k: torch.empty(n, dtype=torch.float32, device=device)
           for k in ('symp_prob', 'severe_prob', 'crit_prob', 'death_prob', 'rel_sus', 'rel_trans')}
    status = torch.zeros(1, dtype=torch.int32, device=device)
    _dev_call('covgpu_pop_prognoses', n, age.data_ptr(), cut.data_ptr(), len(progs['age_cutoffs']), tabs_d.data_ptr(),
              code, p1, p2, step, int(seed) & 0xFFFFFFFFFFFFFFFF, *(out[k].data_ptr() for k in
                                                                  ('symp_prob', 'severe_prob', 'crit_prob',
                                                                   'death_prob', 'rel_sus', 'rel_trans')),
              status.data_ptr())
    if int(status.item()) & L.TIMEOUT:
        raise L.CovgpuError('prognoses (a sampler ran out of tries)', L.TIMEOUT)
    return out
