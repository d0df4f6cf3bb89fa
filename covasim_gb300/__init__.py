"""covasim_gb300: Covasim 3.1.7's per-day step hot path on one GB300 GPU.

Drop-in pieces of the reference's API (``import covasim_gb300 as cv``):

* ``cv.Sim`` / ``cv.People`` / ``cv.Layer`` / ``cv.Contacts`` -- a sim whose
  day loop (transitions, NAb/immunity, transmission, infection) runs as CUDA
  kernels for sm_103a, reached through the C ABI in include/covgpu.h;
* ``cv.compute_viral_load`` / ``cv.compute_trans_sus`` /
  ``cv.compute_infections`` -- the reference's numba kernels, on the GPU;
* ``cv.BatchSim`` -- many sims in one launch (replaces MultiSim's processes);
* ``cv.make_pars``, ``cv.change_beta``, ``cv.variant`` and the population
  generators;
* ``cv.Fit`` / ``cv.compute_gof`` / ``cv.load_data``, ``cv.TransTree`` and
  ``cv.Calibration`` (trials run as batches of sims).

There is no CPU fallback: the kernels need the in-tree ``libcovgpu.so`` and a
CUDA device, and fail loudly without them.
"""
from .version import __version__
from .defaults import *  # noqa: F401,F403
from .parameters import *  # noqa: F401,F403
from .population import *  # noqa: F401,F403
from .immunity import *  # noqa: F401,F403
from .interventions import *  # noqa: F401,F403
from .people import *  # noqa: F401,F403
from .sim import *  # noqa: F401,F403
from .batch import *  # noqa: F401,F403
from .analysis import *  # noqa: F401,F403
from .utils import *  # noqa: F401,F403
from ._lib import CovgpuError  # noqa: F401
