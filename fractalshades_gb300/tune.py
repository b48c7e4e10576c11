"""
Launch-shape autotuner for the iteration kernels.

The kernels run as one persistent wave: pixels are claimed one at a time
from a device counter, so the launch shape -- threads per CTA
(``fsg_calc.block``) and resident CTAs per SM (``fsg_calc.ctas_per_sm``,
0 = the occupancy limit) -- changes speed, never results.  ``autotune`` times
the candidate shapes of a calculation's kernel on the caller's own tiles
(kernel time from the library's CUDA events), keeps the fastest per device
and kernel kind in a JSON cache, and ``apply`` gives later calculations of
that kind the cached shape.

Cache file: ``$FSG_TUNE_CACHE`` if set, else
``~/.cache/fractalshades_gb300/launch_shapes.json``.
"""
import copy
import json
import os
import threading

from . import _native as nat

_lock = threading.Lock()

#: resident-CTA caps tried besides the occupancy limit (0)
CTA_CAPS = (0, 4, 2)


def cache_path():
    p = os.environ.get("FSG_TUNE_CACHE")
    if p:
        return p
    return os.path.join(os.path.expanduser("~"), ".cache", "fractalshades_gb300",
                        "launch_shapes.json")


def kernel_kind(calc, perturb):
    """The kernel a calculation launches, as a cache key."""
    mode = {v: k for k, v in nat.MODES.items()}.get(int(calc.mode), str(calc.mode))
    parts = ["perturb" if perturb else "std", mode if perturb else "fp64"]
    parts.append("bs%d" % calc.flavor if calc.flavor else ("mn" if calc.nexp else "m2"))
    if calc.interior:
        parts.append("interior")
    if calc.calc_dzndc:
        parts.append("deriv")
    if calc.backshift > 0 or calc.calc_d2zndc2:
        parts.append("options")
    return "/".join(parts)


def max_block(calc, perturb):
    """The largest threads per CTA the kernel's launch bounds allow."""
    fe32_m2 = perturb and calc.flavor == 0 and calc.nexp == 0 and calc.mode == nat.MODES["fe32"]
    return 128 if fe32_m2 else 256


def candidates(calc, perturb):
    blocks = [b for b in (64, 128, 256) if b <= max_block(calc, perturb)]
    return [(b, k) for b in blocks for k in CTA_CAPS]


def _device_name(ctx):
    try:
        import torch
        return torch.cuda.get_device_name(getattr(ctx, "device", 0))
    except Exception:
        return "cuda"


_mem = {}      # path -> (mtime, contents): one read per change of the file


def _load(path):
    try:
        mt = os.path.getmtime(path)
    except OSError:
        return {}
    hit = _mem.get(path)
    if hit and hit[0] == mt:
        return hit[1]
    try:
        with open(path) as f:
            data = json.load(f)
    except (OSError, ValueError):
        return {}
    _mem[path] = (mt, data)
    return data


def _store(path, key, entry):
    with _lock:
        data = dict(_load(path))
        data[key] = entry
        os.makedirs(os.path.dirname(os.path.abspath(path)), exist_ok=True)
        tmp = path + ".tmp"
        with open(tmp, "w") as f:
            json.dump(data, f, indent=1, sort_keys=True)
        os.replace(tmp, path)


def _shaped(calc, block, ctas):
    c = copy.copy(calc)
    c.block, c.ctas_per_sm = int(block), int(ctas)
    return c


def autotune(ctx, calc, tiles, *, perturb, where=None, repeats=2, store=True, device=None,
             shapes=None):
    """Time every candidate shape (the best of ``repeats`` launches each) of
    ``calc`` on ``tiles`` and return {"block", "ctas_per_sm", "kernel_ms",
    "kind", "table"}; with ``store`` the winner goes to the cache.  The tiles'
    outputs hold the last launch's results, which do not depend on the
    shape."""
    where = nat.DEVICE if where is None else where
    run = ctx.perturb_tiles if perturb else ctx.std_tiles
    table = []
    for block, ctas in (shapes or candidates(calc, perturb)):
        c = _shaped(calc, block, ctas)
        best = None
        for _ in range(max(1, int(repeats))):
            run(c, tiles, where)
            ms = float(ctx.stats()["kernel_ms"])
            best = ms if best is None else min(best, ms)
        table.append({"block": block, "ctas_per_sm": ctas, "kernel_ms": best})
    win = min(table, key=lambda e: e["kernel_ms"])
    kind = kernel_kind(calc, perturb)
    out = {"block": win["block"], "ctas_per_sm": win["ctas_per_sm"],
           "kernel_ms": win["kernel_ms"], "kind": kind, "table": table}
    if store:
        dev = device or _device_name(ctx)
        _store(cache_path(), dev + "|" + kind,
               {"block": win["block"], "ctas_per_sm": win["ctas_per_sm"],
                "kernel_ms": win["kernel_ms"]})
    return out


def lookup(calc, perturb, device):
    """The cached (block, ctas_per_sm) of this kernel kind, or None."""
    e = _load(cache_path()).get(device + "|" + kernel_kind(calc, perturb))
    if not e:
        return None
    block, ctas = int(e["block"]), int(e["ctas_per_sm"])
    if block % 32 or not 0 <= block <= max_block(calc, perturb) or ctas < 0:
        return None
    return block, ctas


def apply(calc, perturb, device):
    """``calc`` with the cached shape of its kernel kind (unchanged when the
    cache has none)."""
    shape = lookup(calc, perturb, device)
    return calc if shape is None else _shaped(calc, *shape)
