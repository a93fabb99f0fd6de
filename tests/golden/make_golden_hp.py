"""Adds the high-precision answer to the golden fixtures in this directory.

For every golden image case whose pixel function the CPU oracle restates,
the oracle is evaluated in quadruple precision (oracle/quad_oracle.cpp: the
reference's algorithm, its operations, branches and stop rules, without FP64
rounding) on the case's prepared block, and stored as "hp" (rounded to
double) with "hp_cond": the value's largest relative change when q moves by
4 double ulps or the series coefficients by 2 ulps
(oracle.cpu_oracle.quad_condition). Where the reference's own FP64 value is
ill-conditioned ("cond" > 1e-12), the GPU paths are compared with "hp",
within their tolerance or 10 x "hp_cond" where the exact value itself moves
more. Usage (after make_golden.py; --only a,b for selected cases):

    python tests/golden/make_golden_hp.py
"""
import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from oracle import cpu_oracle  # noqa: E402


def main():
    with open(os.path.join(HERE, "cases.json")) as f:
        cases = json.load(f)
    only = None
    if "--only" in sys.argv:
        only = set(sys.argv[sys.argv.index("--only") + 1].split(","))
    for name, c in sorted(cases["images"].items()):
        if c.get("ign_new_switch") or (only is not None and name not in only):
            continue
        P = cpu_oracle.prepare(c["params"], c["ign_cbs"])
        if not cpu_oracle.supported(P):
            continue
        path = os.path.join(HERE, f"{name}.npz")
        rec = dict(np.load(path))
        H, spread = cpu_oracle.quad_condition(P, nthreads=os.cpu_count())
        rec["hp"] = H
        rec["hp_cond"] = spread.astype(np.float32)
        np.savez_compressed(path, **rec)
        ill = rec["cond"] > 1e-12
        print(name, "ill", int(ill.sum()), "hp unstable (>1e-6)", int((ill & (spread > 1e-6)).sum()))
        c["hp"] = True
    with open(os.path.join(HERE, "cases.json"), "w") as f:
        json.dump(cases, f, indent=1, sort_keys=True)


if __name__ == "__main__":
    main()
