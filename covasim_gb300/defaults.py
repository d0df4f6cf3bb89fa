"""State schema, dtypes and result keys of the GPU path.

Mirrors covasim/defaults.py:20-243 (Covasim 3.1.7): the same keys and dtypes
are exposed through ``People``; on the device the sixteen boolean states and
the two by-variant boolean arrays are packed into one ``uint32`` word per agent
and the three variant fields into one ``uint32`` word (one byte each, 0xFF for
"undefined", which the reference stores as NaN).
"""
import numpy as np

default_float = np.float32   # defaults.py:24 (precision 32 is the only precision on the GPU path)
default_int = np.int32       # defaults.py:25
result_float = np.float64    # defaults.py:20

# defaults.py:44-56
PERSON = ['uid', 'age', 'sex', 'symp_prob', 'severe_prob', 'crit_prob', 'death_prob',
          'rel_trans', 'rel_sus', 'n_infections', 'n_breakthroughs']
# defaults.py:59-76: bit i of the flag word is STATES[i]
STATES = ['susceptible', 'naive', 'exposed', 'infectious', 'symptomatic', 'severe', 'critical',
          'tested', 'diagnosed', 'recovered', 'known_dead', 'dead', 'known_contact',
          'quarantined', 'isolated', 'vaccinated']
STATE_BIT = {k: i for i, k in enumerate(STATES)}
EXPOSED_BY_VARIANT_SHIFT = 16    # bits 16..23: exposed_by_variant[v]
INFECTIOUS_BY_VARIANT_SHIFT = 24  # bits 24..31: infectious_by_variant[v]
MAX_VARIANTS = 8
# defaults.py:79-83: byte i of the variant word
VARIANT_STATES = ['exposed_variant', 'infectious_variant', 'recovered_variant']
NO_VARIANT = 0xFF
BY_VARIANT_STATES = ['exposed_by_variant', 'infectious_by_variant']
IMM_STATES = ['sus_imm', 'symp_imm', 'sev_imm']
NAB_STATES = ['peak_nab', 'nab', 't_nab_event']
VACC_STATES = ['doses', 'vaccine_source']
# defaults.py:118-121: index i of the date block is DATES[i]
DATES = [f'date_{s}' for s in STATES] + ['date_pos_test', 'date_end_quarantine', 'date_end_isolation']
DURS = ['dur_exp2inf', 'dur_inf2sym', 'dur_sym2sev', 'dur_sev2crit', 'dur_disease']

ALL_STATES = PERSON + STATES + VARIANT_STATES + BY_VARIANT_STATES + IMM_STATES + NAB_STATES + VACC_STATES + DATES + DURS

# defaults.py:145-159
result_stocks = {
    'susceptible': 'Number susceptible',
    'exposed': 'Number exposed',
    'infectious': 'Number infectious',
    'symptomatic': 'Number symptomatic',
    'severe': 'Number of severe cases',
    'critical': 'Number of critical cases',
    'recovered': 'Number recovered',
    'dead': 'Number dead',
    'diagnosed': 'Number of confirmed cases',
    'known_dead': 'Number of confirmed deaths',
    'quarantined': 'Number in quarantine',
    'isolated': 'Number in isolation',
    'vaccinated': 'Number of people vaccinated',
}
result_stocks_by_variant = {
    'exposed_by_variant': 'Number exposed by variant',
    'infectious_by_variant': 'Number infectious by variant',
}
# defaults.py:167-183
result_flows = {
    'infections': 'infections',
    'reinfections': 'reinfections',
    'infectious': 'infectious',
    'symptomatic': 'symptomatic cases',
    'severe': 'severe cases',
    'critical': 'critical cases',
    'recoveries': 'recoveries',
    'deaths': 'deaths',
    'tests': 'tests',
    'diagnoses': 'diagnoses',
    'known_deaths': 'known deaths',
    'quarantined': 'quarantined people',
    'isolated': 'isolated people',
    'doses': 'vaccine doses',
    'vaccinated': 'vaccinated people',
}
result_flows_by_variant = {
    'infections_by_variant': 'infections by variant',
    'symptomatic_by_variant': 'symptomatic by variant',
    'severe_by_variant': 'severe by variant',
    'infectious_by_variant': 'infectious by variant',
}
new_result_flows = [f'new_{k}' for k in result_flows]
new_result_flows_by_variant = [f'new_{k}' for k in result_flows_by_variant]

# Order of the per-day integer counters the device writes (one row per sim-day).
# Flows, then stocks, then the two bed-occupancy counts used for hosp/icu_max.
RES_FLOWS = new_result_flows
RES_STOCKS = [f'n_{k}' for k in result_stocks]
RES_INT_KEYS = RES_FLOWS + RES_STOCKS
# Per-variant integer counters: [variant flows (4), variant stocks (2)]
RES_VAR_KEYS = new_result_flows_by_variant + [f'n_{k}' for k in result_stocks_by_variant]
# Per-day float64 results
RES_FLOAT_KEYS = ['pop_nabs', 'pop_protection', 'pop_symp_protection']

# variant_pars keys that can differ by variant (defaults.py:204-210)
variant_pars = ['rel_beta', 'rel_symp_prob', 'rel_severe_prob', 'rel_crit_prob', 'rel_death_prob']

# Default age data, Seattle 2018 census (defaults.py:223-243): [min age, max age, fraction]
default_age_data = np.array([
    [0, 4, 0.0605],
    [5, 9, 0.0607],
    [10, 14, 0.0566],
    [15, 19, 0.0557],
    [20, 24, 0.0612],
    [25, 29, 0.0843],
    [30, 34, 0.0848],
    [35, 39, 0.0764],
    [40, 44, 0.0697],
    [45, 49, 0.0701],
    [50, 54, 0.0681],
    [55, 59, 0.0653],
    [60, 64, 0.0591],
    [65, 69, 0.0453],
    [70, 74, 0.0312],
    [75, 79, 0.02016],
    [80, 84, 0.01344],
    [85, 89, 0.01008],
    [90, 99, 0.00672],
])
