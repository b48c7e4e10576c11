"""
Fractal: zoom, pixel grid, calculation hook and tile driver.

Mirrors the reference's ``Fractal`` (core.py:1264-2931) for the iteration path:
same zoom / calc_options API, same pixel -> c mapping (chunk_pixel_pos,
core.py:1767-1830), same per-tile arrays (Z, U, stop_reason, stop_iter) and the
same static ``numba_cycle_call(cycle_dep_args, cycle_indep_args)`` plug-in
point -- which here launches the GPU kernel instead of a numba loop.

Where the reference runs one numba call per 200 x 200 tile on a thread pool
(mthreading.py:48-68), ``calc_raw`` launches all tiles of the image in one
persistent GPU launch and keeps the raw arrays in memory.
"""
import copy
import inspect
import logging
import types

import numpy as np

from . import settings
from . import utils
from . import projection as fsproj
from . import gpu

logger = logging.getLogger(__name__)

USER_INTERRUPTED = 1


class Fractal:
    REPORT_ITEMS = ["chunk1d_begin", "chunk1d_end", "chunk_pts", "done"]
    SAVE_ARRS = ["Z", "U", "stop_reason", "stop_iter"]
    USER_INTERRUPTED = 1

    def __init__(self, directory: str):
        """Base class for escape-time fractals (core.py:1280-1339).

        Parameters
        ----------
        directory : str
            Path for the working base directory (kept for API compatibility:
            raw results are held in memory)."""
        self.directory = directory
        self.subset = None
        self._interrupted = np.array([0], dtype=np.bool_)
        self.float_postproc_type = np.dtype(settings.postproc_dtype)
        self.termination_type = np.int8
        self.int_type = np.int32

    @property
    def init_kwargs(self):
        """Parameters of the __init__ call (stored as attributes by contract)."""
        return {name: getattr(self, name)
                for name in inspect.signature(self.__init__).parameters}

    def __reduce__(self):
        return (self.__class__, tuple(self.init_kwargs.values()))

    # ------------------------------------------------------------------
    # zoom
    # ------------------------------------------------------------------
    @utils.zoom_options
    def zoom(self, *,
             x: float = 0.,
             y: float = 0.,
             dx: float = 8.,
             nx: int = 800,
             xy_ratio: float = 1.,
             theta_deg: float = 0.,
             projection: fsproj.Projection = fsproj.Cartesian(),
             has_skew: bool = False,
             skew_00: float = 1.,
             skew_01: float = 0.,
             skew_10: float = 0.,
             skew_11: float = 1.):
        """Zoom parameters of the next calculation (core.py:1387-1468)."""
        if isinstance(x, str) or isinstance(y, str) or isinstance(dx, str):
            raise RuntimeError("Float expected for x, y, dx")
        if isinstance(projection, str):
            self.projection = projection = fsproj.Cartesian()
        self._skew = None
        if has_skew:
            self._skew = np.array(((skew_00, skew_01), (skew_10, skew_11)), dtype=np.float64)
        self.lin_mat = self.get_lin_mat()
        projection.adjust_to_zoom(self)
        self.proj_impl = projection.f

    def get_lin_mat(self):
        """Rotation (+ skew) matrix (core.py:1470-1484)."""
        theta = self.theta_deg / 180. * np.pi
        c = np.cos(theta)
        s = np.sin(theta)
        lin_mat = np.array(((c, -s), (s, c)), dtype=np.float64)
        skew = getattr(self, "_skew", None)
        if skew is not None:
            lin_mat = np.matmul(skew, lin_mat)
        return lin_mat

    @property
    def ny(self):
        return int(self.nx / self.xy_ratio + 0.5)

    @property
    def dy(self):
        return self.dx / self.xy_ratio

    @property
    def px(self):
        if not hasattr(self, "_px"):
            self._px = self.dx / self.nx
        return self._px

    @property
    def skew(self):
        return getattr(self, "_skew", None)

    @property
    def float_type(self):
        return np.float64

    # ------------------------------------------------------------------
    # tiles (chunks)
    # ------------------------------------------------------------------
    def chunk_slices(self):
        """Yields (ix, ixx, iy, iyy) for tiles of chunk_size x chunk_size
        (core.py:1644-1658)."""
        cs = settings.chunk_size
        for ix in range(0, self.nx, cs):
            ixx = min(ix + cs, self.nx)
            for iy in range(0, self.ny, cs):
                iyy = min(iy + cs, self.ny)
                yield (ix, ixx, iy, iyy)

    @property
    def chunks_count(self):
        cs = settings.chunk_size
        return -(-self.nx // cs) * -(-self.ny // cs)

    def chunk_rank(self, chunk_slice):
        cs = settings.chunk_size
        ix, _, iy, _ = chunk_slice
        cy = -(-self.ny // cs)
        return (ix // cs) * cy + iy // cs

    def chunk_from_rank(self, rank):
        cs = settings.chunk_size
        cy = -(-self.ny // cs)
        cx_, cy_ = divmod(rank, cy)
        ix, iy = cx_ * cs, cy_ * cs
        return (ix, min(ix + cs, self.nx), iy, min(iy + cs, self.ny))

    def pts_count(self, calc_name=None, chunk_slice=None):
        if chunk_slice is None:
            return self.nx * self.ny
        ix, ixx, iy, iyy = chunk_slice
        return (ixx - ix) * (iyy - iy)

    def _axis_1d(self, i0, i1, n, jitter_gap=0.):
        k = 0.5 / (n - 1)
        return np.linspace(k * (2 * i0 - n + 1), k * (2 * i1 - n - 1), num=(i1 - i0),
                           dtype=self.float_type)

    def chunk_axes(self, chunk_slice):
        """Screen coordinates of the columns and rows of a tile, as
        chunk_pixel_pos computes them (core.py:1775-1830): x in
        [-0.5, 0.5] by linspace over the tile, y likewise, negated and divided
        by xy_ratio."""
        ix, ixx, iy, iyy = chunk_slice
        xs = self._axis_1d(ix, ixx, self.nx)
        ys = self._axis_1d(iy, iyy, self.ny)
        ys = (-ys) / self.xy_ratio
        return np.ascontiguousarray(xs), np.ascontiguousarray(ys)

    def image_axes(self):
        """Column / row coordinates of the full image, built tile by tile so
        that every pixel gets exactly the value of its tile's linspace."""
        cs = settings.chunk_size
        xs = np.empty(self.nx)
        ys = np.empty(self.ny)
        for ix in range(0, self.nx, cs):
            ixx = min(ix + cs, self.nx)
            xs[ix:ixx] = self._axis_1d(ix, ixx, self.nx)
        for iy in range(0, self.ny, cs):
            iyy = min(iy + cs, self.ny)
            ys[iy:iyy] = (-self._axis_1d(iy, iyy, self.ny)) / self.xy_ratio
        return xs, ys

    def chunk_pixel_pos(self, chunk_slice, jitter=False, supersampling=None):
        """Pixel positions of a tile in fraction of dx, as a complex array of
        shape (ny, nx) (core.py:1767-1830)."""
        (nx, ny) = (self.nx, self.ny)
        (ix, ixx, iy, iyy) = chunk_slice
        kx = 0.5 / (nx - 1)
        ky = 0.5 / (ny - 1)
        if supersampling is None:
            x_1d = np.linspace(kx * (2 * ix - nx + 1), kx * (2 * ixx - nx - 1),
                               num=(ixx - ix), dtype=self.float_type)
            y_1d = np.linspace(ky * (2 * iy - ny + 1), ky * (2 * iyy - ny - 1),
                               num=(iyy - iy), dtype=self.float_type)
        else:
            ssg = supersampling
            ssg_gap = (ssg - 1.) / ssg
            x_1d = np.linspace(kx * (2 * ix - nx + 1 - ssg_gap),
                               kx * (2 * ixx - nx - 1 + ssg_gap),
                               num=(ixx - ix) * ssg, dtype=self.float_type)
            y_1d = np.linspace(ky * (2 * iy - ny + 1 - ssg_gap),
                               ky * (2 * iyy - ny - 1 + ssg_gap),
                               num=(iyy - iy) * ssg, dtype=self.float_type)
        dx_screen, dy_screen = np.meshgrid(x_1d, -y_1d, indexing='xy')
        if jitter:
            rg = np.random.default_rng(0)
            rand_x = rg.random(dx_screen.shape, dtype=self.float_type)
            rand_y = rg.random(dy_screen.shape, dtype=self.float_type)
            k = 0.7071067811865476
            jitter_x = (0.5 - rand_x) * k / (nx - 1) * jitter
            jitter_y = (0.5 - rand_y) * k / (ny - 1) * jitter
            if supersampling is not None:
                jitter_x /= supersampling
                jitter_y /= supersampling
            dx_screen += jitter_x
            dy_screen += jitter_y
        dy_screen /= self.xy_ratio
        return dx_screen + 1j * dy_screen

    # ------------------------------------------------------------------
    # calculation hook (core.py:1918-2009)
    # ------------------------------------------------------------------
    def calc_hook(self, calc_callable, calc_kwargs, return_dic):
        """Called after a @calc_options method: stores the state and the
        cycle-independent arguments of the calculation."""
        calc_name = calc_kwargs["calc_name"]
        if not hasattr(self, "_calc_data"):
            self._calc_data = dict()
        state = types.SimpleNamespace()
        for k, v in calc_kwargs.items():
            setattr(state, k, v)
            setattr(self, k, v)
        set_state = return_dic["set_state"]()
        set_state(state)
        set_state(self)
        initialize = return_dic["initialize"]()
        iterate = return_dic["iterate"]()
        cycle_indep_args = self.get_cycle_indep_args(initialize, iterate)
        self._calc_data[calc_name] = {
            "calc_class": type(self).__name__,
            "calc_callable": calc_callable,
            "calc_kwargs": calc_kwargs,
            "zoom_kwargs": copy.copy(getattr(self, "zoom_kwargs", {})),
            "state": state,
            "cycle_indep_args": cycle_indep_args,
            "saved_codes": self.saved_codes(state.codes),
            "init_kwargs": self.init_kwargs,
            "raw": None,
        }
        state.fingerprint = {k: self._calc_data[calc_name][k] for k in (
            "calc_class", "calc_callable", "calc_kwargs", "zoom_kwargs", "init_kwargs")}

    @staticmethod
    def saved_codes(codes):
        """Codes of the stored fields: names starting with '_' are not kept
        (core.py:2148-2159)."""
        complex_codes, int_codes, stop_codes = codes
        return ([c for c in complex_codes if not c.startswith("_")],
                [c for c in int_codes if not c.startswith("_")], stop_codes)

    def raise_interruption(self):
        self._interrupted[0] = True
        gpu.cancel()

    def lower_interruption(self):
        self._interrupted[0] = False
        gpu.clear_cancel()

    def is_interrupted(self):
        return bool(self._interrupted[0] or settings.skip_calc)

    # ------------------------------------------------------------------
    # the plug-in point
    # ------------------------------------------------------------------
    @staticmethod
    def numba_cycle_call(cycle_dep_args, cycle_indep_args):
        """Iterate the pixels of one tile in place: same contract as the
        reference (core.py:2022-2027, numba_cycles core.py:2935-2963):
        cycle_dep_args = (c_pix, Z, U, stop_reason, stop_iter) filled in place;
        returns 0, or USER_INTERRUPTED."""
        return gpu.run_std_pixels(cycle_dep_args, cycle_indep_args)

    def get_cycle_indep_args(self, initialize, iterate):
        """Digest of the zoom and calculation parameters (core.py:2029-2041):
        here the GPU calculation options returned by ``iterate``."""
        center = self.x + 1j * self.y
        return (initialize, iterate, complex(center), self.proj_impl, self.lin_mat,
                float(self.dx), self._interrupted)

    def get_cycling_dep_args(self, calc_name, chunk_slice, final=False, jitter=False,
                             supersampling=None):
        """The input / output arrays of one tile (core.py:2044-2075)."""
        c_pix = np.ravel(self.chunk_pixel_pos(chunk_slice, jitter, supersampling))
        state = self._calc_data[calc_name]["state"]
        subset = state.subset
        chunk_subset = None
        if subset is not None:
            chunk_subset = subset[chunk_slice]
            c_pix = c_pix[chunk_subset]
        (n_pts,) = c_pix.shape
        n_Z, n_U, n_stop = (len(code) for code in self.codes)
        Z = np.zeros([n_Z, n_pts], dtype=self.complex_type)
        U = np.zeros([n_U, n_pts], dtype=self.int_type)
        stop_reason = - np.ones([1, n_pts], dtype=self.termination_type)
        stop_iter = np.zeros([1, n_pts], dtype=self.int_type)
        return (c_pix, Z, U, stop_reason, stop_iter), chunk_subset

    def compute_tile(self, calc_name, chunk_slice):
        """One tile through numba_cycle_call (compute_rawdata_dev,
        core.py:2515-2554, without the memmap storage)."""
        (cycle_dep_args, chunk_subset) = self.get_cycling_dep_args(calc_name, chunk_slice)
        cycle_indep_args = self._calc_data[calc_name]["cycle_indep_args"]
        ret_code = self.numba_cycle_call(cycle_dep_args, cycle_indep_args)
        if ret_code == self.USER_INTERRUPTED:
            logger.warning("Interruption signal received")
            return None
        return cycle_dep_args, chunk_subset

    # ------------------------------------------------------------------
    # whole image
    # ------------------------------------------------------------------
    def calc_raw(self, calc_name, tile_validator=None):
        """Compute every tile of the image in one GPU launch; the raw arrays
        are kept in memory, in image layout (ny, nx) per field."""
        if self.is_interrupted():
            return None
        cia = self._calc_data[calc_name]["cycle_indep_args"]
        state = self._calc_data[calc_name]["state"]
        if state.subset is not None:
            raise NotImplementedError("calc_raw with a subset: use compute_tile")
        xs, ys = self.image_axes()
        res = gpu.run_image(self, xs, ys, cia)
        if res is None:
            return None
        self._calc_data[calc_name]["raw"] = res
        return res

    def get_raw(self, calc_name, key):
        """A raw field of the last calc_raw, in image layout (ny, nx):
        a complex code (e.g. "zn"), an int code, "stop_reason" or "stop_iter"."""
        raw = self._calc_data[calc_name]["raw"]
        if raw is None:
            raise RuntimeError(f"calc_raw has not been run for {calc_name}")
        complex_codes, int_codes, _ = self.codes
        ny, nx = self.ny, self.nx
        if key in complex_codes:
            return raw["Z"][complex_codes.index(key)].reshape(ny, nx)
        if key in int_codes:
            return raw["U"][int_codes.index(key)].reshape(ny, nx)
        if key in ("stop_reason", "stop_iter", "potential", "dem"):
            return raw[key].reshape(ny, nx)
        raise KeyError(key)

    def get_std_cpt(self, c_pix):
        """c = center + dx * lin_mat . pix (core.py:2781-2794)."""
        center = complex(self.x + 1j * self.y)
        x, y = c_pix.real, c_pix.imag
        m = self.lin_mat
        x1 = m[0, 0] * x + m[0, 1] * y
        y1 = m[1, 0] * x + m[1, 1] * y
        return center + self.dx * (x1 + 1j * y1)
