"""State consistency against the reference's state diagram (tests/state_diagram.xlsx,
as tests/test_immunity.py:23-85 test_states uses it): for every pair of states
s1 != s2, being s1 implies s2 (1), implies not s2 (-1), or allows either (0).
The matrices are committed as tests/golden/state_diagram.json (read from the
workbook by make_golden.py). The oracle is checked on the reference's own
testing + tracing cases (CPU, MT19937 mode, which reproduces the reference's
runs exactly); the GPU sim on the reference's test_states configuration."""
import json
import os

import numpy as np
import pytest

from common import load_npz, load_testing_case
from oracle.sim import OracleSim
from oracle.interventions import TestProb, ContactTracing

HERE = os.path.dirname(os.path.abspath(__file__))
DIAGRAM = json.load(open(os.path.join(HERE, 'golden', 'state_diagram.json'), encoding='utf-8'))


def check_states(get, use_waning, label=''):
    """Every relation of the sheet on the arrays that ``get(state)`` returns; the
    number of (s1, s2) pairs that had agents in s1."""
    sheet = DIAGRAM['With waning' if use_waning else 'Without waning']
    states, rel = sheet['states'], sheet['relation']
    arrays = {s: np.asarray(get(s), dtype=bool) for s in states}
    checked = 0
    for s1 in states:
        inds = np.nonzero(arrays[s1])[0]
        if not len(inds):
            continue
        for s2 in states:
            if s1 == s2:
                continue
            r = rel[s1][s2]
            vals = arrays[s2][inds]
            if r == 1:
                assert vals.all(), f'{label}: {s1} implies {s2}, but only {vals.sum()}/{len(inds)} are'
            elif r == -1:
                assert not vals.any(), f'{label}: {s1} implies not {s2}, but {vals.sum()}/{len(inds)} are'
            checked += 1
    return checked


def test_diagram_fixture_is_complete():
    for name in ('Without waning', 'With waning'):
        sheet = DIAGRAM[name]
        assert len(sheet['states']) == 14 and set(sheet['relation']) == set(sheet['states'])
        assert all(sheet['relation'][s][s] == 1 for s in sheet['states'])


def test_oracle_runs_of_the_reference_cases_respect_the_diagram():
    d = load_npz('ref_testing.npz')
    seen = set()
    for i in range(int(d['n'])):
        pars, person, contacts, tp, ct = load_testing_case(d, i)
        sim = OracleSim(pars, person, contacts, rng='mt', interventions=[TestProb(**tp), ContactTracing(**ct)]).run()
        n = check_states(lambda s: sim.people[s], bool(pars['use_waning']), label=f'case {i}')
        assert n > 50
        seen.add(bool(pars['use_waning']))
    assert seen == {False, True}


@pytest.mark.gpu
def test_gpu_runs_respect_the_diagram():
    import covasim_gb300 as cv
    for use_waning in (False, True):
        pars = dict(pop_size=1000, pop_infected=20, n_days=70, use_waning=use_waning, rand_seed=1,
                    interventions=[cv.test_prob(symp_prob=0.4, asymp_prob=0.01), cv.contact_tracing(trace_probs=0.1)])
        sim = cv.Sim(pars)
        for until in (20, 35, 50, 71):
            sim.run(until=until)
            n = check_states(lambda s: sim.people[s], use_waning, label=f'waning {use_waning} day {until}')
            assert n > 20
