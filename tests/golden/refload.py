"""Execute Covasim 3.1.7's own hot-path functions in this container.

Used only by ``make_golden.py`` to produce the committed golden fixtures; it
reads the reference source tree, which exists only where the fixtures are
generated (never at test time).

The reference cannot be imported here (numba, sciris, pandas and matplotlib
are not installed), so this module parses the reference's source files with
``ast`` and executes the selected function bodies unchanged, with:

* numba's ``@njit`` decorators dropped; the three numba kernels are called
  through a wrapper that casts the arguments to the declared numba signature
  (float32 / int32 / bool arrays, float32 and int32 scalars), which is what
  numba's dispatcher does before running the compiled code;
* a small stand-in for the few ``sciris`` helpers those bodies call;
* ``np.random`` replaced by a recorder backed by two MT19937 ``RandomState``
  streams -- one for the functions the reference JIT-compiles with numba (which
  has its own generator state) and one for plain numpy calls -- that records
  every draw so that the fixtures can replay the reference's own draws.
"""
import ast
import copy
import os
import types

import numpy as np

# The reference source tree: set by ``set_reference_root`` (make_golden.py's
# ``--reference`` argument) or the COVASIM_REFERENCE environment variable.
REF_ROOT = os.environ.get('COVASIM_REFERENCE') or None


def set_reference_root(path):
    global REF_ROOT
    REF_ROOT = path


def _ref_pkg():
    if not REF_ROOT:
        raise RuntimeError('the reference source tree is not set: pass --reference PATH to make_golden.py '
                           'or set COVASIM_REFERENCE')
    return os.path.join(REF_ROOT, 'covasim')


# ----------------------------------------------------------------------------- stand-ins
class _SciStub(types.SimpleNamespace):
    """The sciris helpers used by the loaded function bodies."""


def _mergedicts(*args, **kwargs):
    out = {}
    for a in args:
        if a:
            out.update(a)
    out.update(kwargs)
    return out


class _objdict(dict):
    def __getattr__(self, k):
        try:
            return self[k]
        except KeyError as E:
            raise AttributeError(k) from E

    def __setattr__(self, k, v):
        self[k] = v


sc = _SciStub(
    dcp=copy.deepcopy, cp=copy.copy, mergedicts=_mergedicts, odict=dict, objdict=_objdict,
    prettyobj=object, findinds=lambda arr, val=None: (np.nonzero(arr)[0] if val is None else np.nonzero(np.asarray(arr) == val)[0]),
    strjoin=lambda *a, **k: ', '.join(str(x) for x in (a[0] if len(a) == 1 else a)),
    newlinejoin=lambda x: '\n'.join(str(i) for i in x), KeyNotFoundError=KeyError,
    isnumber=lambda x: isinstance(x, (int, float, np.integer, np.floating)),
    tolist=lambda x, keepnone=False: (list(x) if isinstance(x, (list, tuple, np.ndarray)) else [x]),
    toarray=np.asarray, printv=lambda *a, **k: None,
)


class _NbType:
    def __getitem__(self, _):
        return self

    def __call__(self, *a, **k):
        return self


_nb = types.SimpleNamespace(
    njit=lambda *a, **k: (lambda f: f), bool_=_NbType(), int32=_NbType(), int64=_NbType(),
    float32=_NbType(), float64=_NbType())

_cvo = types.SimpleNamespace(numba_parallel='none', numba_cache=False, precision=32, verbose=0)


class DrawRecorder:
    """Stand-in for ``np.random`` on one stream: draws from a RandomState and logs them."""

    def __init__(self, name):
        self.name = name
        self.rs = np.random.RandomState(0)
        self.log = []

    def seed(self, seed=None):
        self.rs = np.random.RandomState(seed)

    def _rec(self, kind, vals, **info):
        self.log.append((kind, np.array(vals, copy=True), info))
        return vals

    def random(self, size=None):
        return self._rec('uniform', self.rs.random_sample(size))

    rand = random
    random_sample = random

    def normal(self, loc=0.0, scale=1.0, size=None):
        z = self.rs.standard_normal(size)
        self._rec('normal', z, loc=loc, scale=scale)
        return loc + scale * z

    def lognormal(self, mean=0.0, sigma=1.0, size=None):
        z = self.rs.standard_normal(size)
        self._rec('normal', z, mean=mean, sigma=sigma)
        return np.exp(mean + sigma * z)

    def poisson(self, lam=1.0, size=None):
        return self._rec('poisson', self.rs.poisson(lam, size))

    def negative_binomial(self, n, p, size=None):
        return self._rec('negbin', self.rs.negative_binomial(n, p, size))

    def binomial(self, n, p, size=None):
        return self._rec('binomial', self.rs.binomial(n, p, size))

    def choice(self, a, size=None, replace=True, p=None):
        return self._rec('choice', self.rs.choice(a, size, replace=replace, p=p))

    def randint(self, low, high=None, size=None):
        return self._rec('randint', self.rs.randint(low, high, size))

    def uniform(self, low=0.0, high=1.0, size=None):
        return self._rec('uniform_lh', self.rs.uniform(low, high, size))


class _NpProxy(types.ModuleType):
    """numpy with ``random`` swapped for a DrawRecorder."""

    def __init__(self, recorder):
        super().__init__('numpy_proxy')
        self.random = recorder

    def __getattr__(self, k):
        return getattr(np, k)


# ----------------------------------------------------------------------------- loading
def _read_tree(fname):
    path = os.path.join(_ref_pkg(), fname)
    with open(path) as f:
        return path, ast.parse(f.read())


def _is_njit(node):
    for d in node.decorator_list:
        src = ast.unparse(d)
        if 'njit' in src:
            return True
    return False


def load_module_body(fname, namespace, skip_imports=True):
    """Execute a whole reference module (minus its imports) into ``namespace``."""
    path, tree = _read_tree(fname)
    body = [n for n in tree.body if not (skip_imports and isinstance(n, (ast.Import, ast.ImportFrom)))]
    exec(compile(ast.Module(body=body, type_ignores=[]), path, 'exec'), namespace)
    return namespace


def load_classes(fname, names, namespace):
    """Execute selected top-level class and function definitions of a module
    into ``namespace`` in file order (so base classes precede subclasses)."""
    path, tree = _read_tree(fname)
    body = [n for n in tree.body if isinstance(n, (ast.ClassDef, ast.FunctionDef)) and n.name in names]
    exec(compile(ast.Module(body=body, type_ignores=[]), path, 'exec'), namespace)
    return {n.name: namespace[n.name] for n in body}


def load_functions(fname, names=None, classname=None, namespace=None, njit_namespace=None):
    """Execute selected function definitions (decorators stripped).

    Functions that the reference decorates with numba's ``njit`` are executed
    in ``njit_namespace`` (so they see the numba-stream recorder), the rest in
    ``namespace``. Returns {name: function}.
    """
    path, tree = _read_tree(fname)
    body = tree.body
    if classname is not None:
        body = [n for n in body if isinstance(n, ast.ClassDef) and n.name == classname][0].body
    out = {}
    for node in body:
        if isinstance(node, ast.FunctionDef) and (names is None or node.name in names):
            ns = njit_namespace if (njit_namespace is not None and _is_njit(node)) else namespace
            node.decorator_list = [d for d in node.decorator_list if 'njit' not in ast.unparse(d)]
            exec(compile(ast.Module(body=[node], type_ignores=[]), path, 'exec'), ns)
            out[node.name] = ns[node.name]
    return out


# ----------------------------------------------------------------------------- numba casts
F32, I32 = np.float32, np.int32


def _cast_args(args, spec):
    out = []
    for a, s in zip(args, spec):
        if s == 'f':
            out.append(F32(a))
        elif s == 'i':
            out.append(int(np.int32(a)))  # int32 scalar; Python int keeps numba's float32 typing
        elif s == 'F':
            out.append(np.ascontiguousarray(a, dtype=F32))
        elif s == 'I':
            out.append(np.ascontiguousarray(a, dtype=I32))
        elif s == 'B':
            out.append(np.ascontiguousarray(a, dtype=bool))
        elif s == 'L':
            out.append(np.ascontiguousarray(a, dtype=np.int64))
        else:
            out.append(a)
    return out


NUMBA_SIGNATURES = {  # covasim/utils.py:38,81,92,131,378,430
    'compute_viral_load': 'iFFFfff',
    'compute_trans_sus': 'FFBBfFBBBfffF',
    'compute_infections': 'fIIFFF?',
    'find_contacts': 'IIL',
    'poisson': 'f',
    'choose': 'ii',
}


def numba_wrapped(fn, name):
    spec = NUMBA_SIGNATURES[name]

    def call(*args, **kwargs):
        return fn(*_cast_args(args, spec), **kwargs)
    call.__name__ = name
    return call


# ----------------------------------------------------------------------------- assembly
class Reference:
    """The reference's functions, wired together as the package wires them."""

    def __init__(self):
        self.rec_numba = DrawRecorder('numba')
        self.rec_numpy = DrawRecorder('numpy')
        np_numba = _NpProxy(self.rec_numba)
        np_numpy = _NpProxy(self.rec_numpy)

        # defaults.py, executed whole (imports stubbed)
        cvd_ns = {'np': np, 'nb': _nb, 'sc': sc, 'cvo': _cvo, '__name__': 'covasim.defaults'}
        load_module_body('defaults.py', cvd_ns)
        self.cvd = types.SimpleNamespace(**{k: v for k, v in cvd_ns.items() if not k.startswith('__')})

        # utils.py: plain functions see numpy's stream, numba ones numba's
        # inside the jitted bodies the numba dtype names stand for these numpy dtypes
        utils_ns = {'np': np_numpy, 'nb': _nb, 'sc': sc, 'cvo': _cvo, 'cvd': self.cvd,
                    'random': __import__('random'), 'nbint': np.int32, 'nbfloat': np.float32,
                    'nbbool': np.bool_}
        utils_nb_ns = dict(utils_ns, np=np_numba)
        fns = load_functions('utils.py', namespace=utils_ns, njit_namespace=utils_nb_ns)
        for k, f in fns.items():  # cross-link so each body finds the others
            utils_ns[k] = f
            utils_nb_ns[k] = f
        self.cvu = types.SimpleNamespace(**fns)
        for k in NUMBA_SIGNATURES:
            setattr(self.cvu, k, numba_wrapped(fns[k], k))

        def set_seed(seed=None):  # utils.py:271-298: seed both streams identically
            seed = int(seed)
            self.rec_numpy.seed(seed)
            self.rec_numba.seed(seed)
        self.cvu.set_seed = set_seed

        # parameters.py (values)
        par_ns = {'np': np, 'sc': sc, 'cvo': _cvo, 'cvd': self.cvd, 'cvm': None,
                  '__name__': 'covasim.parameters'}
        load_module_body('parameters.py', par_ns)
        self.cvpar = types.SimpleNamespace(**{k: v for k, v in par_ns.items() if not k.startswith('__')})

        # immunity.py
        imm_ns = {'np': np_numpy, 'sc': sc, 'cvu': self.cvu, 'cvd': self.cvd, 'cvpar': self.cvpar}
        self.cvi = types.SimpleNamespace(**load_functions(
            'immunity.py', ['update_peak_nab', 'update_nab', 'calc_VE', 'check_immunity',
                            'init_immunity', 'precompute_waning', 'nab_growth_decay'], namespace=imm_ns))
        imm_ns.update(vars(self.cvi))

        # people.py and base.py methods, attached to a light People class
        from collections import defaultdict
        ppl_ns = {'np': np_numpy, 'sc': sc, 'cvu': self.cvu, 'cvd': self.cvd, 'cvi': self.cvi,
                  'defaultdict': defaultdict}
        people_methods = load_functions('people.py', classname='People', namespace=ppl_ns,
                                        names=['init_flows', 'set_prognoses', 'update_states_pre',
                                               'update_states_post', 'update_contacts', 'check_inds',
                                               'check_infectious', 'check_symptomatic', 'check_severe',
                                               'check_critical', 'check_recovery', 'check_death',
                                               'check_diagnosed', 'check_quar', 'check_enter_iso',
                                               'check_exit_iso', 'make_naive', 'make_nonnaive', 'infect', 'test',
                                               'schedule_quarantine'])
        base_ns = {'np': np, 'sc': sc, 'cvu': self.cvu, 'cvd': self.cvd}
        base_methods = load_functions('base.py', classname='BasePeople', namespace=base_ns,
                                      names=['true', 'false', 'defined', 'undefined', 'count',
                                             'count_by_variant', 'count_not', '__getitem__',
                                             '__setitem__', '__len__'])
        layer_ns = {'np': np_numba, 'sc': sc, 'cvu': self.cvu, 'cvd': self.cvd}
        layer_methods = load_functions('base.py', classname='Layer', namespace=layer_ns,
                                       names=['update', 'find_contacts'])

        meta = self.cvd.PeopleMeta

        class RefPeople:
            def __init__(pself, pars):
                pself.__dict__['_lock'] = False
                pself.pars = pars
                pself.t = 0
                pself.meta = meta()
                pself.infection_log = []
                n = int(pars['pop_size'])
                nv = pars['n_variants']
                m = pself.meta
                for key in m.person:
                    if key == 'uid':
                        pself[key] = np.arange(n, dtype=I32)
                    elif key in ('n_infections', 'n_breakthroughs'):
                        pself[key] = np.zeros(n, dtype=I32)
                    else:
                        pself[key] = np.full(n, np.nan, dtype=F32)
                for key in m.states:
                    pself[key] = np.full(n, key in ('susceptible', 'naive'), dtype=bool)
                for key in m.variant_states:
                    pself[key] = np.full(n, np.nan, dtype=F32)
                for key in m.by_variant_states:
                    pself[key] = np.full((nv, n), False, dtype=bool)
                for key in m.imm_states:
                    pself[key] = np.zeros((nv, n), dtype=F32)
                for key in m.nab_states:
                    pself[key] = np.zeros(n, dtype=I32 if key == 't_nab_event' else F32)
                for key in m.vacc_states:
                    pself[key] = np.zeros(n, dtype=I32)
                for key in m.dates + m.durs:
                    pself[key] = np.full(n, np.nan, dtype=F32)
                pself._pending_quarantine = defaultdict(list)
                pself.contacts = {}
                pself.init_flows()

            def keys(pself):
                return pself.meta.all_states[:]

            def layer_keys(pself):
                return list(pself.contacts.keys())

        for k, f in {**base_methods, **people_methods}.items():
            setattr(RefPeople, k, f)
        self.People = RefPeople

        class RefLayer(dict):
            def __init__(lself, p1, p2, beta=None, label=None):
                super().__init__()
                lself.label = label
                lself['p1'] = np.asarray(p1, dtype=I32)
                lself['p2'] = np.asarray(p2, dtype=I32)
                lself['beta'] = (np.ones(len(lself['p1']), dtype=F32) if beta is None
                                 else np.asarray(beta, dtype=F32))

            def __len__(lself):
                return len(lself['p1'])

        for k, f in layer_methods.items():
            setattr(RefLayer, k, f)
        self.Layer = RefLayer

        # population.py generators
        pop_ns = {'np': np_numpy, 'sc': sc, 'cvu': self.cvu, 'cvd': self.cvd}
        self.cvpop = types.SimpleNamespace(**load_functions(
            'population.py', ['make_randpop', '_tidy_edgelist', 'make_random_contacts',
                              'make_microstructured_contacts', 'make_hybrid_contacts'], namespace=pop_ns))
        pop_ns.update(vars(self.cvpop))

        # interventions.py: the base class, test_prob and contact_tracing with the
        # helpers they call (their draws come from numpy's stream, as in the package)
        from collections import defaultdict as _dd
        iv_sc = types.SimpleNamespace(**vars(sc))
        iv_sc.ddict = _dd
        iv_sc.isstring = lambda x: isinstance(x, str)
        iv_sc.isiterable = lambda x: hasattr(x, '__iter__')
        iv_sc.pr = print
        pd_stub = types.SimpleNamespace(Series=type('Series', (), {}), DataFrame=type('DataFrame', (), {}))
        iv_ns = {'np': np_numpy, 'sc': iv_sc, 'cvu': self.cvu, 'cvd': self.cvd, 'inspect': __import__('inspect'),
                 'pd': pd_stub,
                 '__all__': ['Intervention', 'test_prob', 'contact_tracing'], '__name__': 'covasim.interventions'}
        self.cvint = types.SimpleNamespace(**load_classes(
            'interventions.py', ['preprocess_day', 'get_day', 'process_daily_data', 'get_subtargets',
                                 'get_quar_inds', 'Intervention', 'test_prob', 'contact_tracing'], iv_ns))

        # sim.py day loop
        sim_ns = {'np': np_numpy, 'sc': sc, 'cvu': self.cvu, 'cvd': self.cvd, 'cvimm': self.cvi,
                  'cvi': types.SimpleNamespace(Intervention=self.cvint.Intervention)}
        self.sim_methods = load_functions('sim.py', classname='Sim', namespace=sim_ns,
                                          names=['step', 'init_infections', 'rescale'])
        sim_ns['AlreadyRunError'] = RuntimeError

    # ------------------------------------------------------------------ helpers
    def make_pars(self, **kwargs):
        pars = self.cvpar.make_pars(**kwargs)
        pars['prognoses'] = self.cvpar.get_prognoses(pars['prog_by_age'])
        return pars

    def draws(self):
        """Pop the recorded draw logs: (numba-stream log, numpy-stream log)."""
        a, b = self.rec_numba.log, self.rec_numpy.log
        self.rec_numba.log, self.rec_numpy.log = [], []
        return a, b


class RefSim:
    """A light ``Sim`` whose ``step`` is the reference's own (sim.py:558-685)."""

    def __init__(self, ref, pars, popdict=None):
        self.ref = ref
        self.pars = pars
        self.t = 0
        self.npts = int(pars['n_days']) + 1
        self.complete = False
        self._legacy_trans = False
        self.rescale_vec = (1.0 if pars['rescale'] else pars['pop_scale']) * np.ones(self.npts)  # sim.py:342-346
        if pars['use_waning']:
            ref.cvi.init_immunity(self)
        cvd = ref.cvd
        self.results = {}
        for key in cvd.result_flows:
            self.results[f'new_{key}'] = np.zeros(self.npts)
        for key in cvd.result_stocks:
            self.results[f'n_{key}'] = np.zeros(self.npts)
        for key in ('n_imports', 'pop_nabs', 'pop_protection', 'pop_symp_protection'):
            self.results[key] = np.zeros(self.npts)
        nv = pars['n_variants']
        self.results['variant'] = {}
        for key in cvd.result_flows_by_variant:
            self.results['variant'][f'new_{key}'] = np.zeros((nv, self.npts))
        for key in cvd.result_stocks_by_variant:
            self.results['variant'][f'n_{key}'] = np.zeros((nv, self.npts))
        ref.cvu.set_seed(pars['rand_seed'])
        if popdict is None:
            popdict = ref.cvpop.make_randpop(pars, microstructure=pars['pop_type'])
        self.popdict = popdict
        people = ref.People(pars)
        # base.py:1357-1368 + 1173-1182: People.__init__ creates its Contacts from the
        # beta_layer keys (the contacts do not exist yet), then add_contacts fills them
        people.contacts = {k: ref.Layer(popdict['contacts'][k]['p1'], popdict['contacts'][k]['p2'], label=k)
                           for k in pars['beta_layer'].keys()}
        people['age'] = np.asarray(popdict['age'], dtype=F32)
        people['sex'] = np.asarray(popdict['sex'], dtype=F32)
        people.set_prognoses()
        self.people = people
        ref.cvu.set_seed(pars['rand_seed'])
        for iv in self.pars['interventions']:  # sim.py:457-474 init_interventions
            if isinstance(iv, ref.cvint.Intervention):
                iv.initialize(self)

    def day(self, day, *args):
        """base.py:356-370 for integer days (and None)."""
        return None if day is None else int(day)

    def __getitem__(self, k):
        return self.pars[k]

    def __setitem__(self, k, v):
        self.pars[k] = v

    def step(self):
        return self.ref.sim_methods['step'](self)

    def init_infections(self, **kw):
        return self.ref.sim_methods['init_infections'](self, **kw)

    def rescale(self):
        return self.ref.sim_methods['rescale'](self)

    @property
    def npts_(self):
        return self.npts

    def run(self):
        while self.t < self.npts:
            self.step()
        return self
