"""Regenerates the golden fixtures in this directory from the reference's own test data.

Reads (never executes) the reference repository:
  * test/inchworm.h5           /inchworm/P/{1,2}, /inchworm/g   (written by test/inchworm.jl:180-212),
                                /diff_inchworm/P/{1,2}           (test/inchworm.jl:214-239)
  * test/topology_eval.h5      /x1_list, /xs_list, /values       (test/topology_eval.jl:53-140)
  * test/scrambled_sobol.jl    MockRNG-scrambled Sobol vectors   (test/scrambled_sobol.jl:136-179)
  * README.md                  Z and rho of the README Anderson run (README.md:203-204)
and writes small JSON files that the tests use on machines without the reference.

Usage:  python tests/golden/make_golden.py /path/to/QInchworm.jl   (or QINCHWORM_REF=/path/to/QInchworm.jl)
"""
from __future__ import annotations

import json
import os
import re
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)

from h5mini import H5File  # noqa: E402


def _cplx(a):
    a = a.ravel()
    return {"re": [float(x) for x in a.real], "im": [float(x) for x in a.imag]}


def inchworm_h5(ref: str):
    f = H5File(os.path.join(ref, "test", "inchworm.h5"))
    out = {
        "source": "test/inchworm.h5 (written by test/inchworm.jl:180-212)",
        "model": {"beta": 10.0, "mu": 0.1, "eps": 0.1, "V": -0.1, "n_tau": 20,
                  "orders": [0, 1, 2, 3], "orders_bare": [0, 1, 2], "N_samples": 256,
                  "spline_delta": True, "interpolate_ppgf": True},
        "P": [_cplx(f.read(f"/inchworm/P/{s}")) for s in (1, 2)],
        "g": _cplx(f.read("/inchworm/g")),
        # diff_inchworm! of the same model, orders 0:3, N = 2^8 (test/inchworm.jl:214-239)
        "diff_P": [_cplx(f.read(f"/diff_inchworm/P/{s}")) for s in (1, 2)],
    }
    with open(os.path.join(HERE, "inchworm_h5.json"), "w") as fh:
        json.dump(out, fh, indent=1)


def topology_eval_h5(ref: str):
    """TopologyEvaluator values of the order-3, n_pts_after = 1 topologies of the single-level
    model at 100 explicit time sets (test/topology_eval.jl:53-140)."""
    f = H5File(os.path.join(ref, "test", "topology_eval.h5"))
    vals = f.read("/values")   # [100][2]: sectors 1 and 2
    out = {
        "source": "test/topology_eval.h5 (read by test/topology_eval.jl:95-140)",
        "model": {"beta": 10.0, "mu": 0.1, "eps": 0.1, "V": -0.1, "n_tau": 30, "order": 3,
                  "n_pts_after": 1, "tau_index_w": 6, "tau_index_f": 7},
        "x1_list": [float(x) for x in f.read("/x1_list")],
        "xs_list": [[float(x) for x in row] for row in f.read("/xs_list")],   # [5][100]
        "values": [_cplx(vals[:, s]) for s in range(vals.shape[1])],
    }
    with open(os.path.join(HERE, "topology_eval_h5.json"), "w") as fh:
        json.dump(out, fh, indent=1)


def _parse_ref_block(text: str, start: int):
    """Parse the `ref = [[...], ...]` literal following `start`."""
    i = text.index("ref = [", start)
    depth, j = 0, i + len("ref = ")
    for k in range(j, len(text)):
        if text[k] == "[":
            depth += 1
        elif text[k] == "]":
            depth -= 1
            if depth == 0:
                lit = text[j:k + 1]
                break
    rows = re.findall(r"\[([^\[\]]*)\]", lit)
    return [[float(x) for x in re.split(r"[,\s]+", r.strip()) if x] for r in rows]


def sobol_vectors(ref: str):
    text = open(os.path.join(ref, "test", "scrambled_sobol.jl")).read()
    scr = text.index('@testset "Scrambled"')
    uns = text.index('@testset "Unscrambled"')
    out = {"source": "test/scrambled_sobol.jl", "tolerance_scrambled": 1e-10}
    for name, base in (("unscrambled", uns), ("scrambled_mockrng", scr)):
        d1 = text.index('@testset "D=1"', base)
        d5 = text.index('@testset "D=5"', base)
        out[name] = {"D1": _parse_ref_block(text, d1), "D5": _parse_ref_block(text, d5)}
    with open(os.path.join(HERE, "sobol_vectors.json"), "w") as fh:
        json.dump(out, fh, indent=1)


def readme_output(ref: str):
    text = open(os.path.join(ref, "README.md")).read()
    z = float(re.search(r"Z = ([0-9.eE+-]+)", text).group(1))
    rho = [float(x) for x in re.findall(r"\[([0-9.eE+-]+) \+ 0\.0im;;\]", text)]
    out = {"source": "README.md:203-204 ('a possible text output')", "Z": z, "rho": rho,
           "model": {"eps": 0.1, "U": 1.0, "D": 2.0, "V": 0.5, "beta": 10.0, "n_tau": 200,
                     "orders": [0, 1, 2, 3, 4], "orders_bare": [0, 1, 2, 3, 4], "N_samples": 1024},
           "topology_counts_bare": [1, 1, 3, 15, 105],
           "topology_counts_bold": [[1], [1], [1, 2, 1], [4, 6, 7, 6, 4], [27, 36, 40, 42, 40, 36, 27]]}
    with open(os.path.join(HERE, "readme_anderson.json"), "w") as fh:
        json.dump(out, fh, indent=1)


if __name__ == "__main__":
    ref = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("QINCHWORM_REF")
    if not ref:
        sys.exit("usage: make_golden.py <path to a QInchworm.jl checkout> (or set QINCHWORM_REF)")
    inchworm_h5(ref)
    topology_eval_h5(ref)
    sobol_vectors(ref)
    readme_output(ref)
    print("fixtures written to", HERE)
