"""gbsgmc: the SG-MCMC sampling hot path of jax_sgmc on one GB300.

The modules mirror jax_sgmc's (``alias``, ``potential``, ``integrator``,
``adaption``, ``scheduler``, ``solver``, ``io``, ``data``); the arithmetic runs
in hand-written sm_103a CUDA kernels reached through the C ABI of
``libgbsgmc.so`` (``include/gbsgmc.h``).
"""

from . import _lib
from . import likelihoods
from . import util
from . import data
from . import potential
from . import adaption
from . import scheduler
from . import integrator
from . import io
from . import engine
from . import solver
from . import alias

__version__ = "0.1.0"
