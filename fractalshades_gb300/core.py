"""
Fractal: zoom, pixel grid, calculation hook and tile driver.

Mirrors the reference's ``Fractal`` (core.py:1264-2931) for the iteration path:
same zoom / calc_options API, same pixel -> c mapping (chunk_pixel_pos,
core.py:1767-1830), same per-tile arrays (Z, U, stop_reason, stop_iter) and the
same static ``numba_cycle_call(cycle_dep_args, cycle_indep_args)`` plug-in
point -- which here launches the GPU kernel instead of a numba loop.

Where the reference runs one numba call per 200 x 200 tile on a thread pool
(mthreading.py:48-68), ``calc_raw`` launches all tiles of the image in one
persistent GPU launch.  The raw arrays are then written to the reference's
on-disk layout (core.py:2125-2510): ``data/<calc>_{Z,U,stop_reason,
stop_iter}.arr`` npy-format memory maps in chunk-compressed order, the
``data/<calc>.report`` chunk table and the ``data/<calc>.fingerprint``
pickle, so that stored results are found again (and only missing tiles
recomputed) exactly as the reference does.
"""
import copy
import inspect
import logging
import os
import pickle
import types

from numpy.lib.format import open_memmap

import numpy as np

from . import settings
from . import utils
from . import projection as fsproj
from . import gpu

logger = logging.getLogger(__name__)

USER_INTERRUPTED = 1

# core.py:60-72: supersampling option -> points per pixel side
SUPERSAMPLING_DIC = {"None": None, None: None, "2x2": 2, "3x3": 3, "4x4": 4, "5x5": 5,
                     "6x6": 6, "7x7": 7}


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
        """Compressed 1-d points of the calculation (of one chunk, or all):
        the subset's true entries when there is a subset (core.py:1743-1765)."""
        subset = None
        if calc_name is not None and calc_name in getattr(self, "_calc_data", {}):
            subset = self._calc_data[calc_name]["state"].subset
        if subset is not None:
            if chunk_slice is None:
                return int(sum(np.count_nonzero(subset[cs]) for cs in self.chunk_slices()))
            return int(np.count_nonzero(subset[chunk_slice]))
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
        # stored results: reuse them when the fingerprint matches and every
        # file is there, else start a new set (core.py:1976-2009)
        if self.res_available(calc_name):
            try:
                self.get_report_memmap(calc_name, mode="r+")
                for key in self.SAVE_ARRS:
                    self.get_data_memmap(calc_name, key, mode="r+")
                if state.subset is not None:
                    self.get_data_memmap(calc_name, "subset", mode="r+")
                self._calc_data[calc_name]["need_new_mmap"] = False
            except FileNotFoundError:
                self._calc_data[calc_name]["need_new_mmap"] = True
        else:
            self._calc_data[calc_name]["need_new_mmap"] = True
            self.save_fingerprint(calc_name, state.fingerprint)

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
        # the projection as the kernels' fields (fsg_tile.proj*), in place of
        # the reference's numba proj_impl
        return (initialize, iterate, complex(center), fsproj.kernel_params(self.projection),
                self.lin_mat, float(self.dx), self._interrupted)

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
    # final render: raw arrays computed on the fly (core.py:2572-2610)
    # ------------------------------------------------------------------
    def evaluate_rawdata_final(self, calc_name, chunk_slice, postproc_options):
        """Raw arrays of one chunk for a final render, with the
        postproc_options' jitter and supersampling ("None", "2x2" .. "7x7");
        nothing is stored.  Returns (subset, c_pix, Z, U, stop_reason,
        stop_iter), or None when interrupted."""
        jitter = float(postproc_options.get("jitter", False))
        supersampling = SUPERSAMPLING_DIC[postproc_options.get("supersampling", "None")]
        if supersampling is not None and self._calc_data[calc_name]["state"].subset is not None:
            raise NotImplementedError("supersampling of a subset calculation")
        (cycle_dep_args, chunk_subset) = self.get_cycling_dep_args(
            calc_name, chunk_slice, final=True, jitter=jitter, supersampling=supersampling)
        cycle_indep_args = self._calc_data[calc_name]["cycle_indep_args"]
        ret_code = self.numba_cycle_call(cycle_dep_args, cycle_indep_args)
        if ret_code == self.USER_INTERRUPTED:
            logger.error("Interruption signal received")
            return None
        (c_pix, Z, U, stop_reason, stop_iter) = cycle_dep_args
        return (chunk_subset, c_pix, Z, U, stop_reason, stop_iter)

    def evaluate_data(self, calc_name, chunk_slice, postproc_options):
        """Raw arrays of a chunk: computed on the fly for a final render,
        else reloaded from the stored memory maps (core.py:2595-2610)."""
        if postproc_options.get("final_render", False):
            return self.evaluate_rawdata_final(calc_name, chunk_slice, postproc_options)
        return self.reload_data(chunk_slice, calc_name)

    # ------------------------------------------------------------------
    # whole image
    # ------------------------------------------------------------------
    def calc_raw(self, calc_name, tile_validator=None):
        """Compute the image and store its raw arrays (core.py:2724-2737).

        Without a subset every tile of the image is computed in one GPU launch
        (kept in memory in image layout (ny, nx) for ``get_raw``) and written
        to the memory maps; with a subset, or when stored results exist, only
        the tiles whose report entry is not done are computed, one launch per
        tile as the reference's compute_rawdata_dev (core.py:2518-2554)."""
        if self.is_interrupted():
            return None
        data = self._calc_data[calc_name]
        if data["need_new_mmap"]:
            self.init_report_mmap(calc_name)
            self.init_data_mmaps(calc_name)
            data["need_new_mmap"] = False
        state = data["state"]
        todo = [cs for cs in self.chunk_slices()
                if (tile_validator is None or tile_validator(cs))
                and not self.res_available(calc_name, cs)]
        if not todo:
            return data.get("raw")
        if state.subset is None and len(todo) == self.chunks_count:
            xs, ys = self.image_axes()
            res = gpu.run_image(self, xs, ys, data["cycle_indep_args"])
            if res is None:
                return None
            data["raw"] = res
            self._store_image(calc_name, res)
            return res
        for cs in todo:
            out = self.compute_tile(calc_name, cs)
            if out is None:
                return None
            (_c_pix, Z, U, stop_reason, stop_iter), _subset = out
            self.update_report_mmap(calc_name, cs, stop_reason)
            self.update_data_mmaps(calc_name, cs, Z, U, stop_reason, stop_iter)
        data["raw"] = None
        return None

    def _store_image(self, calc_name, res):
        """Whole-image raw arrays (image layout) -> per-chunk compressed
        memory maps, every chunk marked done.  The layout is the one
        update_data_mmaps writes tile by tile; here each map is opened and
        flushed once for the whole image."""
        ny, nx = self.ny, self.nx
        state = self._calc_data[calc_name]["state"]
        complex_codes, int_codes, _ = state.codes
        f_complex, f_int, _ = self._calc_data[calc_name]["saved_codes"]
        rows = {"Z": [complex_codes.index(c) for c in f_complex],
                "U": [int_codes.index(c) for c in f_int],
                "stop_reason": [0], "stop_iter": [0]}
        src = {"Z": res["Z"].reshape(res["Z"].shape[0], ny, nx),
               "U": res["U"].reshape(res["U"].shape[0], ny, nx),
               "stop_reason": res["stop_reason"].reshape(1, ny, nx),
               "stop_iter": res["stop_iter"].reshape(1, ny, nx)}
        chunks = []
        for cs in self.chunk_slices():
            rank = self.chunk_rank(cs)
            chunks.append((rank, self.compressed_beg_end(calc_name, rank), cs))
        for key in self.SAVE_ARRS:
            mmap = self.get_data_memmap(calc_name, key, mode="r+")
            for _rank, (beg, end), (ix, ixx, iy, iyy) in chunks:
                for field, r in enumerate(rows[key]):
                    mmap[field, beg:end] = src[key][r, iy:iyy, ix:ixx].ravel()
            mmap.flush()
            del mmap
        mmap = self.get_report_memmap(calc_name, mode="r+")
        mmap[[c[0] for c in chunks], self.REPORT_ITEMS.index("done")] = 1
        mmap.flush()
        del mmap

    def get_raw(self, calc_name, key):
        """A raw field in image layout (ny, nx): a complex code (e.g. "zn"),
        an int code, "stop_reason" or "stop_iter" -- from the last calc_raw,
        else reassembled from the stored memory maps ("potential" and "dem"
        exist only after a calc_raw of this session)."""
        raw = self._calc_data[calc_name].get("raw")
        complex_codes, int_codes, _ = self.codes
        ny, nx = self.ny, self.nx
        if raw is None:
            if key in ("potential", "dem"):
                raise RuntimeError(f"calc_raw has not been run for {calc_name}")
            if self._calc_data[calc_name]["state"].subset is not None:
                raise NotImplementedError("image layout of a subset calculation")
            if key in complex_codes:
                arr_key, row = "Z", self._calc_data[calc_name]["saved_codes"][0].index(key)
            elif key in int_codes:
                arr_key, row = "U", self._calc_data[calc_name]["saved_codes"][1].index(key)
            elif key in ("stop_reason", "stop_iter"):
                arr_key, row = key, 0
            else:
                raise KeyError(key)
            mmap = self.get_data_memmap(calc_name, arr_key, mode="r")
            img = np.empty((ny, nx), dtype=mmap.dtype)
            for rank, cs in enumerate(self.chunk_slices()):
                ix, ixx, iy, iyy = cs
                beg, end = self.compressed_beg_end(calc_name, self.chunk_rank(cs))
                img[iy:iyy, ix:ixx] = np.asarray(mmap[row, beg:end]).reshape(iyy - iy, ixx - ix)
            return img
        if key in complex_codes:
            return raw["Z"][complex_codes.index(key)].reshape(ny, nx)
        if key in int_codes:
            return raw["U"][int_codes.index(key)].reshape(ny, nx)
        if key in ("stop_reason", "stop_iter", "potential", "dem"):
            return raw[key].reshape(ny, nx)
        raise KeyError(key)

    # ------------------------------------------------------------------
    # raw-array storage (core.py:2125-2510)
    # ------------------------------------------------------------------
    def fingerprint_path(self, calc_name):
        return os.path.join(self.directory, "data", calc_name + ".fingerprint")

    def save_fingerprint(self, calc_name, fingerprint):
        path = self.fingerprint_path(calc_name)
        os.makedirs(os.path.dirname(path), exist_ok=True)
        with open(path, "wb+") as f:
            pickle.dump(fingerprint, f, pickle.HIGHEST_PROTOCOL)

    def reload_fingerprint(self, calc_name):
        with open(self.fingerprint_path(calc_name), "rb") as f:
            return pickle.load(f)

    def fingerprint_matching(self, calc_name, test_fingerprint, log=False):
        """Every flattened key of the current fingerprint equals the stored
        one (core.py:1851-1881)."""
        flat = utils.dic_flatten(test_fingerprint)
        expected = utils.dic_flatten(self._calc_data[calc_name]["state"].fingerprint)
        for key, val in expected.items():
            if key not in flat:
                return False
            try:
                same = flat[key] == val
                if isinstance(same, np.ndarray):
                    same = bool(same.all()) and np.shape(flat[key]) == np.shape(val)
            except Exception:      # noqa: BLE001 -- incomparable values differ
                same = False
            if not same:
                if log:
                    logger.debug(f"Parameter mismatch: {key}, {flat[key]} --> {val}")
                return False
        return True

    def res_available(self, calc_name, chunk_slice=None):
        """Fingerprint match (chunk_slice None), or the chunk's report entry
        is done (core.py:1883-1915)."""
        try:
            fingerprint = self.reload_fingerprint(calc_name)
        except (IOError, EOFError, pickle.UnpicklingError):
            return False
        if not self.fingerprint_matching(calc_name, fingerprint, chunk_slice is None):
            return False
        if chunk_slice is None:
            return True
        try:
            report = self.reload_report(calc_name, chunk_slice)
        except (IOError, ValueError):
            return False
        return report["done"] > 0

    def report_path(self, calc_name):
        return os.path.join(self.directory, "data", calc_name + ".report")

    def init_report_mmap(self, calc_name):
        """int32 [chunks_count, (chunk1d_begin, chunk1d_end, chunk_pts, done)]
        (core.py:2173-2209)."""
        items = self.REPORT_ITEMS
        path = self.report_path(calc_name)
        os.makedirs(os.path.dirname(path), exist_ok=True)
        mmap = open_memmap(filename=path, mode="w+", dtype=np.dtype(np.int32),
                           shape=(self.chunks_count, len(items)), fortran_order=False,
                           version=None)
        mmap[:, items.index("done")] = 0
        pts = np.array([self.pts_count(calc_name, cs) for cs in self.chunk_slices()],
                       dtype=np.int32)
        cum = np.zeros(self.chunks_count + 1, dtype=np.int32)
        np.cumsum(pts, out=cum[1:])
        mmap[:, items.index("chunk_pts")] = pts
        mmap[:, items.index("chunk1d_begin")] = cum[:-1]
        mmap[:, items.index("chunk1d_end")] = cum[1:]
        mmap.flush()
        del mmap

    def get_report_memmap(self, calc_name, mode="r+"):
        return open_memmap(filename=self.report_path(calc_name), mode=mode)

    def update_report_mmap(self, calc_name, chunk_slice, stop_reason):
        mmap = self.get_report_memmap(calc_name, mode="r+")
        mmap[self.chunk_rank(chunk_slice), self.REPORT_ITEMS.index("done")] = 1
        mmap.flush()
        del mmap

    def reload_report(self, calc_name, chunk_slice):
        """The chunk's report entry as a dict, or (items, full report) when
        chunk_slice is None (core.py:2253-2271)."""
        mmap = self.get_report_memmap(calc_name, mode="r")
        items = self.REPORT_ITEMS
        if chunk_slice is None:
            return items, np.array(mmap)
        rank = self.chunk_rank(chunk_slice)
        return dict(zip(items, (int(mmap[rank, items.index(it)]) for it in items)))

    def compressed_beg_end(self, calc_name, rank):
        mmap = self.get_report_memmap(calc_name, mode="r")
        items = self.REPORT_ITEMS
        return (int(mmap[rank, items.index("chunk1d_begin")]),
                int(mmap[rank, items.index("chunk1d_end")]))

    def uncompressed_beg_end(self, rank):
        """Span of the chunk in the (full-size) subset mask, chunks in rank
        order (core.py:1700-1727)."""
        arr = np.zeros(self.chunks_count + 1, dtype=np.int64)
        for i, (ix, ixx, iy, iyy) in enumerate(self.chunk_slices()):
            arr[i + 1] = arr[i] + (ixx - ix) * (iyy - iy)
        return int(arr[rank]), int(arr[rank + 1])

    def data_path(self, calc_name):
        keys = ["subset"] + self.SAVE_ARRS
        return {k: os.path.join(self.directory, "data", f"{calc_name}_{k}.arr") for k in keys}

    def init_data_mmaps(self, calc_name):
        """Z [n_Z, pts], U [n_U, pts], stop_reason / stop_iter [1, pts] with
        the stored codes only, and the subset mask (core.py:2362-2430)."""
        state = self._calc_data[calc_name]["state"]
        f_complex, f_int, _stop = self._calc_data[calc_name]["saved_codes"]
        pts = self.pts_count(calc_name)
        dtypes = {"Z": self.complex_type, "U": self.int_type,
                  "stop_reason": self.termination_type, "stop_iter": self.int_type}
        dims = {"Z": (len(f_complex), pts), "U": (len(f_int), pts),
                "stop_reason": (1, pts), "stop_iter": (1, pts)}
        paths = self.data_path(calc_name)
        os.makedirs(os.path.dirname(paths["Z"]), exist_ok=True)
        for key in self.SAVE_ARRS:
            mmap = open_memmap(filename=paths[key], mode="w+", dtype=np.dtype(dtypes[key]),
                               shape=dims[key], fortran_order=False, version=None)
            del mmap
        if state.subset is not None:
            mmap = open_memmap(filename=paths["subset"], mode="w+", dtype=bool,
                               shape=(self.ny * self.nx,), fortran_order=False, version=None)
            for rank, cs in enumerate(self.chunk_slices()):
                beg, end = self.uncompressed_beg_end(rank)
                mmap[beg:end] = np.ravel(state.subset[cs])
            del mmap

    def get_data_memmap(self, calc_name, key, mode="r+"):
        return open_memmap(filename=self.data_path(calc_name)[key], mode=mode)

    def update_data_mmaps(self, calc_name, chunk_slice, Z, U, stop_reason, stop_iter):
        """The chunk's columns [beg, end) of each stored array; codes starting
        with '_' are not stored (core.py:2441-2473)."""
        state = self._calc_data[calc_name]["state"]
        complex_codes, int_codes, _ = state.codes
        f_complex, f_int, _ = self._calc_data[calc_name]["saved_codes"]
        rank = self.chunk_rank(chunk_slice)
        beg, end = self.compressed_beg_end(calc_name, rank)
        rows = {"Z": [complex_codes.index(c) for c in f_complex],
                "U": [int_codes.index(c) for c in f_int],
                "stop_reason": [0], "stop_iter": [0]}
        arrs = {"Z": Z, "U": U, "stop_reason": stop_reason, "stop_iter": stop_iter}
        for key in self.SAVE_ARRS:
            mmap = self.get_data_memmap(calc_name, key, mode="r+")
            for field, src in enumerate(rows[key]):
                mmap[field, beg:end] = arrs[key][src, :]
            mmap.flush()
            del mmap

    def reload_data(self, chunk_slice, calc_name):
        """(subset, c_pix, Z, U, stop_reason, stop_iter) of a chunk from the
        memory maps (core.py:2476-2510)."""
        rank = self.chunk_rank(chunk_slice)
        beg, end = self.compressed_beg_end(calc_name, rank)
        arr = {}
        for key in self.SAVE_ARRS:
            mmap = self.get_data_memmap(calc_name, key, mode="r")
            arr[key] = np.array(mmap[:, beg:end])
            del mmap
        subset = self._calc_data[calc_name]["state"].subset
        if subset is not None:
            ub, ue = self.uncompressed_beg_end(rank)
            mmap = self.get_data_memmap(calc_name, "subset", mode="r")
            arr["subset"] = np.array(mmap[ub:ue])
            del mmap
        else:
            arr["subset"] = None
        c_pix = np.ravel(self.chunk_pixel_pos(chunk_slice, jitter=False, supersampling=None))
        if arr["subset"] is not None:
            c_pix = c_pix[arr["subset"]]
        return arr["subset"], c_pix, arr["Z"], arr["U"], arr["stop_reason"], arr["stop_iter"]

    def get_std_cpt(self, c_pix):
        """c = center + dx * lin_mat . proj(pix) (core.py:2781-2794,
        c_from_pix :3161-3194)."""
        center = complex(self.x + 1j * self.y)
        if getattr(self.projection, "kernel_kind", 0):
            c_pix = self.projection.f(np.asarray(c_pix))
        x, y = c_pix.real, c_pix.imag
        m = self.lin_mat
        x1 = m[0, 0] * x + m[0, 1] * y
        y1 = m[1, 0] * x + m[1, 1] * y
        return center + self.dx * (x1 + 1j * y1)
