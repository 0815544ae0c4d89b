"""rectv_gpu_gb300: GB300-native (sm_103a) time-resolved tomographic
reconstruction with a drop-in ``rectv`` / ``Solver`` API of nikitinvv/rectv_gpu.

The compute path is librectv_gb300.so (hand-written CUDA + cuFFT, C ABI in
include/rectv_gb300.h); importing the classes does not require a GPU, creating
a solver does.
"""

from .rectv import plan_directions, rectv
from .solver import Solver, getp, takephi
from . import phantom

__all__ = ["rectv", "plan_directions", "Solver", "getp", "takephi", "phantom"]
__version__ = "1.0.0"
