"""seistorch_gb300: GB300-native (sm_103a) wave-propagation hot path of seistorch.

The 2D acoustic (PML / HABC) and isotropic elastic time loops, with source
injection, receiver sampling and a boundary-saving adjoint, run in
hand-written CUDA kernels behind a C ABI (include/seistorch_gb300.h).  The
Python modules mirror seistorch's names (``WaveRNN``, ``WaveCell``,
``equations2d.<eq>._time_step`` ...) so the path is a drop-in.
"""
from .cell import WaveCell
from .eqconfigure import Parameters, Wavefield
from .geom import WaveGeometryFreeForm
from .model import build_model
from .probe import WaveIntensityProbe, WaveProbe
from .rnn import WaveRNN
from .source import WaveSource
from .type import TensorList

__version__ = "0.1.0"
