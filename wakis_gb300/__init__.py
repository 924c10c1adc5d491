"""wakis_gb300: the Finite Integration Technique leapfrog path of Wakis on one GB300.

Drop-in classes with the reference's names and arguments: GridFIT3D, SolverFIT3D (with
one_step / emsolve / wakesolve), WakeSolver, Field, sources.Beam / PlaneWave / WavePacket,
Logger, materials.material_lib.  The time step runs in hand-written sm_103a kernels of
libwakis_fit.so (C ABI: include/wakis_fit.h); there is no CPU fallback.
"""

__version__ = "0.1.0"

from . import materials, sources  # noqa: F401
from .field import Field  # noqa: F401
from .field_monitors import FieldMonitor  # noqa: F401
from .gridFIT3D import GridFIT3D  # noqa: F401
from .logger import Logger  # noqa: F401
from .solverFIT3D import SolverFIT3D  # noqa: F401
from .wakeSolver import WakeSolver  # noqa: F401
