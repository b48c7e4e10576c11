"""
Post-processing of the raw iteration results: continuous iteration count
(potential), distance estimate, field lines, DEM normal map and raw field
access.

Restates the reference's Continuous_iter_pp (postproc.py:267-406,
Continuous_iter_pp_infinity :1001-1009), DEM_pp (:662-731), Raw_pp
(:217-264), Fieldlines_pp (:409-530) and DEM_normal_pp (:533-628) over the
raw arrays of ``Fractal.calc_raw``.  The GPU kernels also produce the
potential and the distance estimate in their epilogue; Continuous_iter_pp
and DEM_pp compute them from Z, U, stop_iter in numpy with the reference's
formulas, so both can be compared.  Field lines and normals run on the GPU
(csrc/fsg_postproc.cu, fsg_postproc_fieldlines / fsg_postproc_normal).
"""
import numpy as np


def Continuous_iter_pp_infinity(zn, d, a_d, M):
    """nu_frac = -log(log|k zn| / log(M k)) / log d, k = |a_d|^(1/(d-1))."""
    k = np.abs(a_d) ** (1. / (d - 1.))
    return -(np.log(np.log(np.abs(zn * k)) / np.log(M * k)) / np.log(d))


class Postproc:
    field_count = 1

    def link(self, batch):
        self.batch = batch

    @property
    def fractal(self):
        return self.batch.fractal

    @property
    def state(self):
        return self.fractal._calc_data[self.batch.calc_name]["state"]

    @property
    def holomorphic(self):
        return self.fractal.holomorphic

    def raw(self, key):
        return self.batch.raw(key)

    def get_zn(self):
        if self.holomorphic:
            return self.raw("zn")
        return self.raw("xn") + 1j * self.raw("yn")


class Raw_pp(Postproc):
    def __init__(self, key, func=None):
        """Direct access to a raw field (postproc.py:217-264)."""
        self.key = key
        self.func = func

    def evaluate(self, context):
        arr = self.raw(self.key)
        if np.iscomplexobj(arr) and self.func is None:
            raise ValueError(f"complex field {self.key}: provide `func`")
        return (arr if self.func is None else self.func(arr)), {}


class Continuous_iter_pp(Postproc):
    def __init__(self, kind=None, d=None, a_d=None, M=None, epsilon_cv=None, floor_iter=0):
        """Continuous iteration number (postproc.py:267-406), kind
        "infinity" only."""
        self.post_dic = {k: v for k, v in dict(kind=kind, d=d, a_d=a_d, M=M,
                                               epsilon_cv=epsilon_cv).items() if v is not None}
        self._floor_iter = floor_iter

    @property
    def potential_dic(self):
        dic = {}
        for prop in ["kind", "d", "a_d", "M_cutoff"]:
            dic[prop] = self.post_dic.get(prop, getattr(self.fractal, "potential_" + prop, None))
        for prop in ["M", "epsilon_cv"]:
            dic[prop] = self.post_dic.get(prop, getattr(self.state, "potential_" + prop, None))
        return dic

    def evaluate(self, context):
        # stop_iter's int32, as the reference's n (postproc.py:392)
        n = self.raw("stop_iter").astype(np.int32)
        pd = self.potential_dic
        if pd["kind"] != "infinity":
            raise NotImplementedError(f"Potential kind: {pd['kind']} unsupported")
        zn = self.get_zn()
        with np.errstate(all="ignore"):
            nu_frac = Continuous_iter_pp_infinity(zn, pd["d"], pd["a_d"], pd["M"])
            nu_div, nu_mod = np.divmod(-nu_frac, 1.)
            # a NaN nu_div (pixel not escaped) casts to a platform-dependent int
            n = n - nu_div.astype(n.dtype)
        nu_frac = -nu_mod
        val = (n - self._floor_iter) + nu_frac
        return val, {"potential_dic": pd, "nu_frac": nu_frac, "n": n,
                     "backshift": getattr(self.state, "backshift", None)}


class DEM_pp(Postproc):
    def __init__(self, px_snap=None):
        """Distance estimation |zn| log|zn| / |dzndc| (postproc.py:662-731)."""
        self.px_snap = px_snap

    def evaluate(self, context):
        zn = self.get_zn()
        with np.errstate(all="ignore"):
            abs_zn = np.abs(zn)
            if self.holomorphic:
                abs_dzndc = np.abs(self.raw("dzndc"))
            else:
                a, b = self.raw("dxnda"), self.raw("dxndb")
                c, d = self.raw("dynda"), self.raw("dyndb")
                abs_dzndc = 0.5 * (np.hypot(a + d, b - c) + np.hypot(a - d, b + c))
            val = abs_zn * np.log(abs_zn) / abs_dzndc
        if self.px_snap is not None:
            val = np.where(val < self.px_snap, 0., val)
        return val, {}


class Fieldlines_pp(Postproc):
    def __init__(self, n_iter=5, swirl=0., endpoint_k=1.0):
        """Orbit-averaged angle revealing field lines (postproc.py:409-530):
        n_iter orbit points from zn_orbit (else zn), geometric weights from
        1 to endpoint_k, random phases scaled by swirl.  Needs
        Continuous_iter_pp earlier in the batch."""
        self.n_iter = int(n_iter)
        self.swirl = swirl
        self.endpoint_k = endpoint_k
        if not 1 <= self.n_iter <= 64:
            raise ValueError("n_iter must be in 1 .. 64")

    def _model(self):
        """The map the orbit is continued with: 0 z^2 + c (M2_iterate), n
        z^n + c (the power-n models' Mn_iterate), -flavor (BS_iterate)."""
        f = self.fractal
        if not self.holomorphic:
            return -int(f.flavor_int)
        return int(getattr(f, "exponent", 0))

    def evaluate(self, context):
        from . import gpu
        pd = context["potential_dic"]
        if pd["kind"] != "infinity":
            raise ValueError(f"Unsupported potential '{pd['kind']}' for field lines")
        k_arr = np.geomspace(1., self.endpoint_k, num=self.n_iter)
        k_arr = k_arr / np.sum(k_arr)
        rg = np.random.default_rng(0)
        phi_arr = rg.random(self.n_iter) * self.swirl * np.pi
        codes = self.fractal.codes[0]
        backshift = context.get("backshift")
        if self.holomorphic:
            key = "zn_orbit" if "zn_orbit" in codes else "zn"
            z = self.raw(key)
        else:
            key = "xn_orbit" if "xn_orbit" in codes else "xn"
            z = self.raw(key) + 1j * self.raw("yn_orbit" if key == "xn_orbit" else "yn")
        is_backward = key.endswith("_orbit")
        if is_backward and backshift is None:
            raise ValueError("zn_orbit stored without a backshift in the calculation state")
        c_pt = self.fractal.get_std_cpt(self.batch.c_pix())
        val = gpu.context().fieldlines(
            model=self._model(), c=c_pt, z=z, nu_frac=context["nu_frac"], n=context["n"],
            k=k_arr, phi=phi_arr, is_backward=is_backward,
            backshift=backshift if is_backward else 0)
        return val, {}


class DEM_normal_pp(Postproc):
    field_count = 2

    def __init__(self, kind="potential"):
        """Unit normal of the distance estimate (postproc.py:533-628): kind
        "potential" (z / dzndc, Burning Ship: J^T z) or "Milnor" (needs the
        d2zndc2 field); the view's skew is undone.  Evaluates to complex."""
        if kind not in ("potential", "Milnor"):
            raise ValueError(kind)
        self.kind = kind

    def evaluate(self, context):
        from . import gpu
        skew = self.fractal.skew
        if self.kind == "Milnor":
            out = gpu.context().normal(kind=1, zn=self.raw("zn"), dzndc=self.raw("dzndc"),
                                       d2zndc2=self.raw("d2zndc2"), skew=skew)
        elif self.holomorphic:
            out = gpu.context().normal(kind=0, zn=self.raw("zn"), dzndc=self.raw("dzndc"),
                                       skew=skew)
        else:
            jac = np.stack([self.raw(k) for k in ("dxnda", "dxndb", "dynda", "dyndb")])
            out = gpu.context().normal(kind=2, zn=self.get_zn(), dzndc=jac, skew=skew)
        return out, {}


class Postproc_batch:
    def __init__(self, fractal, calc_name):
        """A set of post-processings of one calculation."""
        self.fractal = fractal
        self.calc_name = calc_name
        self.posts = {}
        self._final = None

    def add_postproc(self, postname, postproc):
        postproc.link(self)
        self.posts[postname] = postproc

    def raw(self, key):
        """A raw field, flat: from the final-render arrays being evaluated,
        else from the calculation's stored results."""
        if self._final is None:
            return self.fractal.get_raw(self.calc_name, key).ravel()
        (_subset, _c_pix, Z, U, sr, si) = self._final
        complex_codes, int_codes, _ = self.fractal.codes
        if key in complex_codes:
            return Z[complex_codes.index(key)]
        if key in int_codes:
            return U[int_codes.index(key)]
        if key == "stop_reason":
            return sr[0]
        if key == "stop_iter":
            return si[0]
        raise KeyError(key)

    def c_pix(self):
        """Screen positions of the evaluated points (fractions of dx)."""
        if self._final is not None:
            return self._final[1]
        xs, ys = self.fractal.image_axes()
        return (xs[None, :] + 1j * ys[:, None]).ravel()

    def evaluate(self, postproc_options=None):
        """Evaluate every post-processing on the whole image; returns
        {postname: float array (ny, nx)}.  With postproc_options
        {"final_render": True, "supersampling": "None" | "2x2" .. "7x7",
        "jitter": False | float} the raw arrays are computed on the fly on the
        jittered / supersampled grid (core.py:2572-2593) and the arrays are
        (ny * s, nx * s)."""
        from .core import SUPERSAMPLING_DIC
        opts = postproc_options or {}
        ssg = 1
        if opts.get("final_render", False):
            chunk = (0, self.fractal.nx, 0, self.fractal.ny)
            self._final = self.fractal.evaluate_rawdata_final(self.calc_name, chunk, opts)
            if self._final is None:
                return None
            ssg = SUPERSAMPLING_DIC[opts.get("supersampling", "None")] or 1
        try:
            return self._evaluate(ssg)
        finally:
            self._final = None

    def _evaluate(self, ssg):
        out = {}
        context = {}
        for name, pp in self.posts.items():
            val, upd = pp.evaluate(context)
            context.update(upd)
            shape = (self.fractal.ny * ssg, self.fractal.nx * ssg)
            if getattr(pp, "field_count", 1) == 2:
                # the two components, as the reference's XYCoord_wrapper_pp
                out[name + "_x"] = np.asarray(val.real, self.fractal.float_postproc_type).reshape(shape)
                out[name + "_y"] = np.asarray(val.imag, self.fractal.float_postproc_type).reshape(shape)
                continue
            out[name] = np.asarray(val, dtype=self.fractal.float_postproc_type).reshape(shape)
        return out
