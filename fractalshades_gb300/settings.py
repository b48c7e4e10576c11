"""
Application-level settings (module globals), same names and defaults as the
reference's settings.py.  Only the flags the iteration path reads are kept,
plus the GPU options of this package.
"""
enable_multithreading: bool = True
"""Kept for API compatibility: tiles are batched into GPU launches."""

skip_calc: bool = False
"""If True, no calculation is performed (core.py is_interrupted)."""

newton_zoom_level: float = 1.e-5
"""Minimal zoom level for Newton search; shallower zooms use the critical
point as reference.  Also gates the BLA (mandelbrot_M2.py:521-524)."""

std_zoom_level: float = 1.e-8

xrange_zoom_level: float = 1.e-300
"""Zoom level (dx) which triggers the Xrange branches."""

no_newton: bool = False
"""Veto all Newton iterations: keep the reference point as is."""

inspect_calc: bool = False

chunk_size: int = 200
"""Side of the basic calculation tile (chunk_size x chunk_size)."""

BLA_compression: int = 3
"""Number of BLA levels which are not stored (fixed at 3 in the kernels)."""

postproc_dtype: str = "float32"

verbosity: int = 2
log_directory: str = None

# --- GPU options ------------------------------------------------------------
gpu_device: int = 0
"""CUDA device of the calculations."""

precision_mode: str = "auto"
"""Delta arithmetic of the perturbation kernels:
"auto" follows the reference (Xrange deltas when dx < xrange_zoom_level,
double deltas otherwise); "fp64", "xr64" force one of the reference's two
forms; "fe32" selects the FP32-mantissa + int32-exponent fast form."""
