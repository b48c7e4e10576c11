"""
fractalshades_gb300 -- GB300-native (sm_103a) iteration path for Fractalshades.

Drop-in replacement of Fractalshades' per-pixel escape-time hot path: the
model classes, zoom / calc_std_div options and postproc API of the reference,
with the standard and perturbation loops (BLA, rebasing, derivatives, interior
detection, Xrange deltas, Burning Ship sign folding) running as CUDA kernels
behind the C-ABI of include/fsgpu.h.  The arbitrary-precision reference orbit
stays on the host.
"""
__version__ = "0.1.0"

from . import settings
from .utils import zoom_options, calc_options, interactive_options
from .core import Fractal
from .perturbation import PerturbationFractal
from . import models
from . import postproc
from . import projection

__all__ = ["settings", "zoom_options", "calc_options", "interactive_options", "Fractal",
           "PerturbationFractal", "models", "postproc", "projection"]
