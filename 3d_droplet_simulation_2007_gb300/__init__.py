"""GB300-native projection hot path of the 3D VOF droplet solver
farzan-t/3D_Droplet_simulation_2007.

The compute lives in ``libdsg.so`` (hand-written sm_103a CUDA kernels behind
the C ABI of ``include/dsg.h``); this package is the host-side mirror of the
reference driver (``Solver``), the ``inputdata.in`` interface (``config``) and
the build recipe (``build``).  The package directory name starts with a digit,
so import it with ``importlib.import_module("3d_droplet_simulation_2007_gb300")``.
"""
from . import config  # noqa: F401
from .config import InputData, parse_inputdata, format_inputdata  # noqa: F401
from ._lib import DsgError, load  # noqa: F401
from .solver import Solver  # noqa: F401
from .ensemble import Ensemble, study_configs  # noqa: F401
from . import kernels  # noqa: F401
