"""
Writes data/nuclei.json: the nuclei of the seeded deep-zoom workloads (the
period-p nuclei of synthetic.config2_workload, config3_workload and the
eight centres of the serving stream), found by synthetic.find_nucleus (Newton
at the workload's digits, period confirmed by the ball method).  Each entry
"p:dps" holds the real and imaginary parts as decimal strings with dps + 10
digits.  Run:  python -m fractalshades_gb300.data.make_nuclei
"""
import json
import os

import mpmath
import numpy as np

from fractalshades_gb300 import synthetic as syn


def periods():
    out = []
    out.append((int(np.random.default_rng(2).integers(300, 3001)), 400))      # config 2
    out.append((int(np.random.default_rng(3).integers(2000, 20001)), 1100))   # config 3
    for p in np.random.default_rng(5).integers(300, 3001, 8):                 # serving
        out.append((int(p), 1100))
    return out


def main():
    data = {}
    if os.path.exists(syn.NUCLEI_FILE):
        with open(syn.NUCLEI_FILE) as f:
            data = json.load(f)
    for p, dps in periods():
        key = f"{p}:{dps}"
        if key in data:
            continue
        c = syn.find_nucleus(p, dps)
        with mpmath.workdps(dps):
            data[key] = [mpmath.nstr(c.real, dps + 10), mpmath.nstr(c.imag, dps + 10)]
        print(key, flush=True)
    with open(syn.NUCLEI_FILE, "w") as f:
        json.dump(data, f, indent=1, sort_keys=True)


if __name__ == "__main__":
    main()
