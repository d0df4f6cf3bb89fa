"""Philox-4x32-10 counter-based generator in numpy, plus the draw conversions.

TEST INFRASTRUCTURE ONLY (part of the CPU oracle): the CUDA library implements
the same generator and the same conversions, so that the oracle run in
"philox" mode reproduces a GPU simulation draw for draw.

Philox-4x32-10 is the published generator of Salmon et al., "Parallel random
numbers: as easy as 1, 2, 3" (SC'11). Round function, multipliers and Weyl key
increments follow that paper.

Stream layout (shared with the CUDA side; all words little-endian uint32):

  key     = (seed_lo, seed_hi)                        64-bit per-sim seed
  counter = (c0, c1, c2, c3)
    edge Bernoulli      : (edge_lo, edge_hi, day, TAG_EDGE  | variant << 8 | layer)
    dynamic-layer lists : counts (agent, 0, day, TAG_DYN | layer); partners (agent, 1 + d * 256 + j // 4,
                          day, TAG_DYN | layer); redraws (agent, d << 10 | j, day, TAG_DYN_RETRY | try << 8 | layer)
    infect draws        : (agent,   block,   day, TAG_INFECT | call_tag)
    testing draws       : (agent,   block,   day, TAG_TEST)  block 0: test, sensitivity; 1: follow-up
    tracing draws       : (agent,   layer,   day, TAG_TRACE)

Draw conversions:
  u52(a, b)  = ((a >> 6) << 26 | (b >> 6)) ... see ``u01_52``: exact doubles in (0, 1)
  u32(a)     = (a + 0.5) * 2**-32, exact double in (0, 1)
  Box-Muller = sqrt(-2 ln u1) * (cos 2 pi u2, sin 2 pi u2)
"""
import numpy as np

PHILOX_M0 = np.uint64(0xD2511F53)
PHILOX_M1 = np.uint64(0xCD9E8D57)
PHILOX_W0 = np.uint32(0x9E3779B9)
PHILOX_W1 = np.uint32(0xBB67AE85)

TAG_EDGE = 0x01000000
TAG_INFECT = 0x03000000
TAG_TEST = 0x04000000
TAG_TRACE = 0x05000000
TAG_DYN = 0x08000000
TAG_DYN_RETRY = 0x09000000

_MASK32 = np.uint64(0xFFFFFFFF)


def philox4x32_10(c0, c1, c2, c3, k0, k1):
    """Vectorised Philox-4x32-10. All inputs broadcast; returns 4 uint32 arrays."""
    c0 = np.asarray(c0, dtype=np.uint32).astype(np.uint64)
    c1 = np.asarray(c1, dtype=np.uint32).astype(np.uint64)
    c2 = np.asarray(c2, dtype=np.uint32).astype(np.uint64)
    c3 = np.asarray(c3, dtype=np.uint32).astype(np.uint64)
    c0, c1, c2, c3 = np.broadcast_arrays(c0, c1, c2, c3)
    k0 = np.uint64(np.uint32(k0))
    k1 = np.uint64(np.uint32(k1))
    w0 = np.uint64(PHILOX_W0)
    w1 = np.uint64(PHILOX_W1)
    for r in range(10):
        if r:
            k0 = (k0 + w0) & _MASK32
            k1 = (k1 + w1) & _MASK32
        p0 = PHILOX_M0 * c0
        p1 = PHILOX_M1 * c2
        hi0, lo0 = p0 >> np.uint64(32), p0 & _MASK32
        hi1, lo1 = p1 >> np.uint64(32), p1 & _MASK32
        c0, c1, c2, c3 = hi1 ^ c1 ^ k0, lo1, hi0 ^ c3 ^ k1, lo0
    return (c0.astype(np.uint32), c1.astype(np.uint32),
            c2.astype(np.uint32), c3.astype(np.uint32))


def seed_key(seed):
    """Split a (non-negative) integer seed into the two 32-bit key words."""
    s = int(seed) & 0xFFFFFFFFFFFFFFFF
    return s & 0xFFFFFFFF, s >> 32


def u01_52(a, b):
    """Exact double in (0, 1) from two words: (k + 0.5) * 2**-52, k = 52 random bits."""
    a = np.asarray(a, dtype=np.uint64)
    b = np.asarray(b, dtype=np.uint64)
    k = ((a >> np.uint64(6)) << np.uint64(26)) | (b >> np.uint64(6))
    return (k.astype(np.float64) + 0.5) * (2.0 ** -52)


def u01_32(a):
    """Exact double in (0, 1) from one word: (a + 0.5) * 2**-32."""
    return (np.asarray(a, dtype=np.uint32).astype(np.float64) + 0.5) * (2.0 ** -32)


def box_muller(w_a, w_b):
    """Two standard normals from two words (32-bit uniforms)."""
    u1 = u01_32(w_a)
    u2 = u01_32(w_b)
    r = np.sqrt(-2.0 * np.log(u1))
    th = 2.0 * np.pi * u2
    return r * np.cos(th), r * np.sin(th)


def uniform_index(a, b, n):
    """Uniform integer in [0, n) from a 64-bit word pair: floor(x * n / 2**64)."""
    a = np.asarray(a, dtype=np.uint64)
    b = np.asarray(b, dtype=np.uint64)
    n = np.uint64(n)
    # 64x64 -> high 64 bits, computed from 32-bit halves (x = a<<32 | b).
    n_lo = n & _MASK32
    n_hi = n >> np.uint64(32)
    t0 = b * n_lo
    t1 = a * n_lo + (t0 >> np.uint64(32))
    t2 = b * n_hi + (t1 & _MASK32)
    hi = a * n_hi + (t1 >> np.uint64(32)) + (t2 >> np.uint64(32))
    return hi.astype(np.int64)


def edge_uniforms(k0, k1, day, layer, variant, edges):
    """Per-edge Bernoulli uniforms for both directions: (u_dir0, u_dir1)."""
    e = np.asarray(edges, dtype=np.int64)
    w = philox4x32_10(e & 0xFFFFFFFF, e >> 32, day,
                      TAG_EDGE | (int(variant) << 8) | int(layer), k0, k1)
    return u01_52(w[0], w[1]), u01_52(w[2], w[3])


# ----------------------------------------------------------------------------- redrawn layers
# A layer redrawn every day (covasim/base.py:1849-1876, Layer.update with frac=1)
# has E edges with i.i.d. uniform endpoints over n agents. In philox mode the
# day's edges of agent a are two lists (d = 0: a as p1, d = 1: a as p2), each of
# Binomial(E, 1/n) entries with uniform partners; the lists of an agent are drawn
# only where they are needed (the day's sources for transmission, the traced
# agents for contact tracing).
DYN_MAX_LIST = 1024
_M40 = (1 << 40) - 1


def dyn_count_table(n_edges, n_agents):
    """The list-length distribution Binomial(n_edges, 1 / n_agents) as 64-bit
    thresholds: entry k = floor(2**64 * P(count <= k)), the last entry 2**64 - 1
    (the first k where the upper tail falls below 2**-64, at most DYN_MAX_LIST
    entries). Computed in 50-digit decimal arithmetic, so every platform gets
    the same table."""
    from decimal import Decimal, localcontext
    E, n = int(n_edges), int(n_agents)
    top = (1 << 64) - 1
    with localcontext() as ctx:
        ctx.prec = 50
        if n == 1:  # every edge is the agent's own
            if E >= DYN_MAX_LIST:
                raise ValueError('dynamic layer lists longer than the supported maximum')
            return np.array([0] * E + [top], dtype=np.uint64)
        p = Decimal(1) / Decimal(n)
        q = 1 - p
        pmf = (Decimal(E) * q.ln()).exp()
        cdf = Decimal(0)
        eps = Decimal(2) ** -64
        out = []
        for k in range(DYN_MAX_LIST):
            cdf += pmf
            if 1 - cdf < eps or k == E:
                out.append(top)
                return np.array(out, dtype=np.uint64)
            out.append(min(int(cdf * (1 << 64)), top))
            pmf = pmf * Decimal(E - k) / Decimal(k + 1) * p / q
        if 1 - cdf > Decimal(2) ** -40:
            raise ValueError('dynamic layer lists longer than the supported maximum (mean contacts too high)')
        out[-1] = top
        return np.array(out, dtype=np.uint64)


def dyn_edge_id(a, j, day, layer):
    """Identity of entry j of an agent's list: a bijection of a << 10 | j on 40
    bits, salted by the day and layer (its order decides the first infector
    among one layer's transmissions to the same target)."""
    a = np.asarray(a, dtype=np.uint64)
    j = np.asarray(j, dtype=np.uint64)
    salt = np.uint64(((((int(day) << 8) | int(layer)) * 0x9E3779B97F) & _M40))
    m40 = np.uint64(_M40)
    x = ((a << np.uint64(10)) | j) ^ salt
    x = (x * np.uint64(0xD6E8FEB86659D)) & m40
    x ^= x >> np.uint64(21)
    x = (x * np.uint64(0xA0761D6478BD)) & m40
    x ^= x >> np.uint64(19)
    return x.astype(np.int64)


def dyn_counts(k0, k1, day, layer, agents, table):
    """Lengths of the two lists of each agent: [m, 2] int64 (64-bit uniforms from
    words x:y and z:w of Philox (agent, 0, day, TAG_DYN | layer))."""
    a = np.asarray(agents, dtype=np.int64)
    w = philox4x32_10(a, 0, day, TAG_DYN | int(layer), k0, k1)
    out = np.empty((len(a), 2), dtype=np.int64)
    for d, (hi, lo) in enumerate(((w[0], w[1]), (w[2], w[3]))):
        u = (hi.astype(np.uint64) << np.uint64(32)) | lo.astype(np.uint64)
        out[:, d] = np.minimum(np.searchsorted(table, u, side='right'), len(table) - 1)
    return out


TAG_DYN_HIT = 0x0A000000


def dyn_partners(k0, k1, day, layer, agents, d, j, n_agents):
    """Partner j of list d of each agent (the entries dyn_lists draws), for
    given (agent, d, j) triples."""
    ag = np.asarray(agents, dtype=np.int64)
    dd = np.asarray(d, dtype=np.int64)
    jj = np.asarray(j, dtype=np.int64)
    w = philox4x32_10(ag, 1 + 256 * dd + (jj >> 2), day, TAG_DYN | int(layer), k0, k1)
    x = np.choose(jj & 3, [w[0], w[1], w[2], w[3]]).astype(np.uint64)
    n = np.uint64(n_agents)
    thr = np.uint64((2 ** 32 - int(n_agents)) % int(n_agents))
    m = x * n
    mask32 = np.uint64(0xFFFFFFFF)
    bad = (m & mask32) < thr
    for r in range(16):
        if not bad.any():
            break
        idx = np.nonzero(bad)[0]
        rw = philox4x32_10(ag[idx], (dd[idx] << 10) | jj[idx], day, TAG_DYN_RETRY | (r << 8) | int(layer), k0, k1)
        m[idx] = rw[0].astype(np.uint64) * n
        bad[idx] = (m[idx] & mask32) < thr
    return (m >> np.uint64(32)).astype(np.int64)


def thin_shift(pmax):
    """m with 2**-m the power of two just above each float32 bound pmax (0 for
    pmax >= 1, at most 32): an entry is a potential transmission with
    probability 2**-m."""
    pm = np.asarray(pmax, dtype=np.float32)
    ex = ((pm.view(np.uint32) >> np.uint32(23)) & np.uint32(0xFF)).astype(np.int64)
    m = np.where(ex == 0, 32, np.minimum(32, 126 - ex))
    return np.where(pm >= 1, 0, m).astype(np.int64)


def dyn_potential(k0, k1, day, layer, agents, d, j, m):
    """Whether entry j of list d of each agent is a potential transmission: the
    top m bits of word j % 4 of Philox (agent, 256 d + j // 4, day,
    TAG_DYN_HIT | layer) are zero."""
    ag = np.asarray(agents, dtype=np.int64)
    dd = np.asarray(d, dtype=np.int64)
    jj = np.asarray(j, dtype=np.int64)
    w = philox4x32_10(ag, 256 * dd + (jj >> 2), day, TAG_DYN_HIT | int(layer), k0, k1)
    x = np.choose(jj & 3, [w[0], w[1], w[2], w[3]]).astype(np.uint64)
    m = np.asarray(m, dtype=np.int64)
    return (m == 0) | ((x >> (32 - np.minimum(np.maximum(m, 1), 32)).astype(np.uint64)) == 0)


def dyn_lists(k0, k1, day, layer, agents, table, n_agents):
    """Every entry of the two lists of each agent: arrays (agent, d, j, partner),
    ordered by agent, then d, then j. Partner j of list d is word j % 4 of
    Philox (agent, 1 + 256 d + j // 4, day, TAG_DYN | layer), made an unbiased
    integer below n_agents (Lemire 2019: the high half of x * n, redrawn while
    the low half is below 2**32 mod n; redraw r is word x of Philox
    (agent, d << 10 | j, day, TAG_DYN_RETRY | r << 8 | layer), at most 16)."""
    a = np.asarray(agents, dtype=np.int64)
    counts = dyn_counts(k0, k1, day, layer, a, table)
    reps = counts.reshape(-1)
    ag = np.repeat(np.repeat(a, 2), reps)
    dd = np.repeat(np.tile(np.array([0, 1], dtype=np.int64), len(a)), reps)
    starts = np.cumsum(reps) - reps
    jj = np.arange(len(ag), dtype=np.int64) - np.repeat(starts, reps)
    w = philox4x32_10(ag, 1 + 256 * dd + (jj >> 2), day, TAG_DYN | int(layer), k0, k1)
    x = np.choose(jj & 3, [w[0], w[1], w[2], w[3]]).astype(np.uint64)
    n = np.uint64(n_agents)
    thr = np.uint64((2 ** 32 - int(n_agents)) % int(n_agents))
    m = x * n
    mask32 = np.uint64(0xFFFFFFFF)
    bad = (m & mask32) < thr
    for r in range(16):
        if not bad.any():
            break
        idx = np.nonzero(bad)[0]
        rw = philox4x32_10(ag[idx], (dd[idx] << 10) | jj[idx], day, TAG_DYN_RETRY | (r << 8) | int(layer), k0, k1)
        m[idx] = rw[0].astype(np.uint64) * n
        bad[idx] = (m[idx] & mask32) < thr
    return ag, dd, jj, (m >> np.uint64(32)).astype(np.int64)


# Slots of the per-infection draw table (shared with the CUDA side).
N_EXP2INF, N_INF2SYM, N_SYM2SEV, N_SEV2CRIT, N_FINAL, N_NAB = 0, 1, 2, 3, 4, 5
U_SYMP, U_SEV, U_CRIT, U_DEATH = 6, 7, 8, 9
N_DRAWS = 10


def infect_draws(k0, k1, day, call_tag, agents):
    """The ten draws one infection consumes, as a float64 table [n, 10].

    Three Philox blocks per agent: block 0 gives the normals for exp2inf,
    inf2sym, sym2sev, sev2crit; block 1 the normals for the final duration and
    the initial NAb level plus the symptomatic and severe uniforms; block 2 the
    critical and death uniforms.
    """
    a = np.asarray(agents, dtype=np.int64)
    tag = TAG_INFECT | int(call_tag)
    out = np.empty((len(a), N_DRAWS), dtype=np.float64)
    b0 = philox4x32_10(a, 0, day, tag, k0, k1)
    b1 = philox4x32_10(a, 1, day, tag, k0, k1)
    b2 = philox4x32_10(a, 2, day, tag, k0, k1)
    out[:, N_EXP2INF], out[:, N_INF2SYM] = box_muller(b0[0], b0[1])
    out[:, N_SYM2SEV], out[:, N_SEV2CRIT] = box_muller(b0[2], b0[3])
    out[:, N_FINAL], out[:, N_NAB] = box_muller(b1[0], b1[1])
    out[:, U_SYMP] = u01_32(b1[2])
    out[:, U_SEV] = u01_32(b1[3])
    out[:, U_CRIT] = u01_32(b2[0])
    out[:, U_DEATH] = u01_32(b2[1])
    return out


def test_draws(k0, k1, day, agents):
    """The three uniforms of one agent's testing on one day: (test, sensitivity,
    not lost to follow-up), each a 52-bit exact double."""
    a = np.asarray(agents, dtype=np.int64)
    b0 = philox4x32_10(a, 0, day, TAG_TEST, k0, k1)
    b1 = philox4x32_10(a, 1, day, TAG_TEST, k0, k1)
    return u01_52(b0[0], b0[1]), u01_52(b0[2], b0[3]), u01_52(b1[0], b1[1])


def capacity_keys(k0, k1, day, agents):
    """contact_tracing's capacity in philox mode: each case's 64-bit selection key,
    the x word of Philox (agent, 2, day, TAG_TEST) above the agent's index (unique);
    the day's ``capacity`` cases with the smallest keys are traced."""
    a = np.asarray(agents, dtype=np.int64)
    b = philox4x32_10(a, 2, day, TAG_TEST, k0, k1)
    return (np.asarray(b[0], dtype=np.uint64) << np.uint64(32)) | a.astype(np.uint64)


def trace_draws(k0, k1, day, layer, agents):
    """The uniform deciding whether a contact of a traced case in ``layer`` is reached."""
    a = np.asarray(agents, dtype=np.int64)
    b = philox4x32_10(a, int(layer), day, TAG_TRACE, k0, k1)
    return u01_52(b[0], b[1])


def infect_draws_ff(k0, k1, day, call_tag, agents):
    """The draws of ``infect_draws`` as the CUDA library forms them: the six
    normals as float-float pairs (Box-Muller in float-float, oracle.gpu_arith)
    and the four uniforms. Returns (z_hi [n, 6], z_lo [n, 6], u [n, 4])."""
    from .gpu_arith import box_muller_ff
    a = np.asarray(agents, dtype=np.int64)
    tag = TAG_INFECT | int(call_tag)
    b0 = philox4x32_10(a, 0, day, tag, k0, k1)
    b1 = philox4x32_10(a, 1, day, tag, k0, k1)
    b2 = philox4x32_10(a, 2, day, tag, k0, k1)
    zh = np.empty((len(a), 6), dtype=np.float32)
    zl = np.empty((len(a), 6), dtype=np.float32)
    for (wa, wb), (i, j) in (((b0[0], b0[1]), (0, 1)), ((b0[2], b0[3]), (2, 3)), ((b1[0], b1[1]), (4, 5))):
        (z0h, z0l), (z1h, z1l) = box_muller_ff(wa, wb)
        zh[:, i], zl[:, i], zh[:, j], zl[:, j] = z0h, z0l, z1h, z1l
    u = np.stack([u01_32(b1[2]), u01_32(b1[3]), u01_32(b2[0]), u01_32(b2[1])], axis=1)
    return zh, zl, u
