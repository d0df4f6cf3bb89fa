"""CPU restatement of Covasim 3.1.7's three numba transmission kernels.

TEST INFRASTRUCTURE ONLY. The product never imports this module; tests and
the CPU-baseline leg of bench.py do.

Each function restates covasim/utils.py with the dtypes numba gives it under
the reference's signatures (``cvd.nbfloat`` = float32, ``cvd.nbint`` = int32):
numba types mixed integer/float ufunc inputs as float32 (its
``ufunc_can_cast`` rule), so ``t - time_start`` is a float32 subtraction and
``1 - immunity_factors`` is float32; the Bernoulli comparison is float64
uniform < float32 probability (``utils.py:123``), i.e. it is done in float64.
"""
import numpy as np

F32 = np.float32


def compute_viral_load(t, time_start, time_recovered, time_dead, frac_time, load_ratio, high_cap):
    """covasim/utils.py:39-79 (compute_viral_load)."""
    time_start = np.asarray(time_start, dtype=F32)
    time_recovered = np.asarray(time_recovered, dtype=F32)
    time_dead = np.asarray(time_dead, dtype=F32)
    frac_time, load_ratio, high_cap = F32(frac_time), F32(load_ratio), F32(high_cap)
    n = len(time_dead)
    # utils.py:59-61: stop date is the death date where defined, else recovery
    time_stop = time_recovered.copy()
    dead = ~np.isnan(time_dead)
    time_stop[dead] = time_dead[dead]
    # utils.py:64-71: high-load phase capped at high_cap days
    with np.errstate(divide='ignore', invalid='ignore'):
        infect_days_total = time_stop - time_start
        trans_day = frac_time * infect_days_total
        capped = trans_day > high_cap
        trans_point = np.full(n, frac_time, dtype=F32)
        trans_point[capped] = high_cap / infect_days_total[capped]
        # utils.py:74-77: float32 throughout (t is an int32 scalar -> float32)
        early = (F32(t) - time_start) / infect_days_total < trans_point
    one = F32(1.0)
    num = np.where(early, load_ratio, one).astype(F32)
    den = one + frac_time * (load_ratio - one)
    return (num / den).astype(F32)


def compute_trans_sus(rel_trans, rel_sus, inf, sus, beta_layer, viral_load, symp, iso, quar,
                      asymp_factor, iso_factor, quar_factor, immunity_factors):
    """covasim/utils.py:82-90 (compute_trans_sus); float32 left-to-right products."""
    rel_trans = np.asarray(rel_trans, dtype=F32)
    rel_sus = np.asarray(rel_sus, dtype=F32)
    inf, sus, symp, iso, quar = (np.asarray(x, dtype=bool) for x in (inf, sus, symp, iso, quar))
    one = F32(1.0)
    f_asymp = np.where(symp, one, F32(asymp_factor)).astype(F32)
    f_iso = np.where(iso, F32(iso_factor), one).astype(F32)
    f_quar = np.where(quar, F32(quar_factor), one).astype(F32)
    rt = rel_trans * inf.astype(F32)
    rt = rt * f_quar
    rt = rt * f_asymp
    rt = rt * f_iso
    rt = rt * F32(beta_layer)
    rt = rt * np.asarray(viral_load, dtype=F32)
    rs = rel_sus * sus.astype(F32)
    rs = rs * f_quar
    rs = rs * (one - np.asarray(immunity_factors, dtype=F32))
    return rt.astype(F32), rs.astype(F32)


def infection_probs(beta, sources, targets, layer_betas, rel_trans, rel_sus):
    """Per-edge probability for one direction, utils.py:115-117, float32."""
    return (F32(beta) * layer_betas) * rel_trans[sources] * rel_sus[targets]


def compute_infections(beta, p1, p2, layer_betas, rel_trans, rel_sus, uniforms):
    """covasim/utils.py:93-128 (compute_infections, non-legacy).

    ``uniforms`` supplies the draws: a callable ``uniforms(direction, edge_inds)``
    returning float64 draws for the surviving edges of that direction (in edge
    order), or an array of shape (2, E) indexed by (direction, edge).

    Returns (sources, targets) int32, direction p1->p2 first, then p2->p1, each
    in edge order.
    """
    p1 = np.asarray(p1, dtype=np.int32)
    p2 = np.asarray(p2, dtype=np.int32)
    layer_betas = np.asarray(layer_betas, dtype=F32)
    rel_trans = np.asarray(rel_trans, dtype=F32)
    rel_sus = np.asarray(rel_sus, dtype=F32)
    beta = F32(beta)
    slist, tlist = [], []
    for d, (sources, targets) in enumerate(((p1, p2), (p2, p1))):
        source_trans = rel_trans[sources]
        inf_inds = source_trans.nonzero()[0]
        betas = beta * layer_betas[inf_inds] * source_trans[inf_inds] * rel_sus[targets[inf_inds]]
        nz = betas.nonzero()[0]
        edge_inds = inf_inds[nz]
        if callable(uniforms):
            u = np.asarray(uniforms(d, edge_inds), dtype=np.float64)
        else:
            u = np.asarray(uniforms, dtype=np.float64)[d, edge_inds]
        hit = (u < betas[nz].astype(np.float64)).nonzero()[0]
        slist.append(sources[edge_inds[hit]])
        tlist.append(targets[edge_inds[hit]])
    return (np.concatenate(slist).astype(np.int32), np.concatenate(tlist).astype(np.int32))


def lognormal_params(par1, par2):
    """utils.py:223-226: mean and sigma of the underlying normal (float64)."""
    mean = np.log(par1 ** 2 / np.sqrt(par2 ** 2 + par1 ** 2))
    sigma = np.sqrt(np.log(par2 ** 2 / par1 ** 2 + 1))
    return mean, sigma


def lognormal_int_from_normal(par1, par2, z):
    """utils.py:222-231 with the standard normal z made explicit: round(exp(mu + sigma z))."""
    z = np.asarray(z, dtype=np.float64)
    if par1 > 0:
        mean, sigma = lognormal_params(par1, par2)
        return np.round(np.exp(mean + sigma * z))
    return np.zeros(z.shape)
