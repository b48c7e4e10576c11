"""
Post-processing of the raw iteration results: continuous iteration count
(potential), distance estimate and raw field access.

Restates the reference's Continuous_iter_pp (postproc.py:267-406,
Continuous_iter_pp_infinity :1001-1009), DEM_pp (:662-731) and Raw_pp
(:217-264) over the in-memory raw arrays of ``Fractal.calc_raw``.  The GPU
kernels also produce the potential and the distance estimate in their
epilogue; these classes compute them from Z, U, stop_iter in numpy with the
reference's formulas, so both can be compared.
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
        return self.fractal.get_raw(self.batch.calc_name, key).ravel()

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
        n = self.raw("stop_iter").astype(np.int64)
        pd = self.potential_dic
        if pd["kind"] != "infinity":
            raise NotImplementedError(f"Potential kind: {pd['kind']} unsupported")
        zn = self.get_zn()
        with np.errstate(all="ignore"):
            nu_frac = Continuous_iter_pp_infinity(zn, pd["d"], pd["a_d"], pd["M"])
            nu_div, nu_mod = np.divmod(-nu_frac, 1.)
        nu_frac = -nu_mod
        n = n - nu_div.astype(n.dtype)
        val = (n - self._floor_iter) + nu_frac
        return val, {"potential_dic": pd, "nu_frac": nu_frac, "n": n}


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


class Postproc_batch:
    def __init__(self, fractal, calc_name):
        """A set of post-processings of one calculation."""
        self.fractal = fractal
        self.calc_name = calc_name
        self.posts = {}

    def add_postproc(self, postname, postproc):
        postproc.link(self)
        self.posts[postname] = postproc

    def evaluate(self):
        """Evaluate every post-processing on the whole image; returns
        {postname: float array (ny, nx)}."""
        out = {}
        context = {}
        for name, pp in self.posts.items():
            val, upd = pp.evaluate(context)
            context.update(upd)
            out[name] = np.asarray(val, dtype=self.fractal.float_postproc_type).reshape(
                self.fractal.ny, self.fractal.nx)
        return out
