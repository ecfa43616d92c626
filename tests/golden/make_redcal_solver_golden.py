"""What the reference's solver-level Omnical does with a solver's
dictionaries, for tests/test_redcal_solver.py.

Runs the unmodified ``OmnicalSolverGPU.solve_iteratively`` of
hera_gpu/redcal.py:747-837 -- and through it the reference's ``omnical``,
its kernels compiled for the host -- on the CPU via oracle/redcal_ref.py,
for a 19-antenna hexagonal array of 3 x 2 problems whose solution is
complex64 or complex128, with the precision taken from it or given.
linsolve's ``get_name`` is its published rule (a trailing '_' marks a
conjugated variable).  Records the arrays the reference hands to
``omnical``, what ``omnical`` returned, and the (meta, sol) it returned.

Writes redcal_solver_reference.npz: per case ``<case>_in_<g0|u0|d|w>``
(the problem), ``<case>_precision`` (-1: None), ``<case>_omnical_<arg>``,
``<case>_result_<key>``, ``<case>_meta_<key>``, and ``<case>_sol_names`` /
``<case>_sol_values``.

Usage (needs the reference sources; the fixture is committed):

    python tests/golden/make_redcal_solver_golden.py /path/to/reference
"""
from __future__ import annotations

import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))
sys.path.insert(0, os.path.dirname(HERE))

SHAPE = (3, 2)
GAIN = 0.3
SCHEDULE = dict(conv_crit=1e-10, maxiter=60, check_every=4, check_after=1)
CASES = {"c64_auto": (np.complex64, None), "c128_auto": (np.complex128, None),
         "c128_p1": (np.complex128, 1)}
OMNICAL_ARGS = ("ggu", "gains", "ubls", "data", "wgts")


def problem(dtype):
    from hera_gpu_gb300 import synth
    ggu, nubls = synth.hex_redundant_layout(19)
    g0, u0, d, w = synth.redundant_data(ggu, nubls, int(np.prod(SHAPE)), 11, noise=1e-3)
    return ggu, g0.astype(dtype), u0.astype(dtype), d.astype(dtype), w


def main(ref_root):
    from oracle.redcal_ref import reference_solve_iteratively
    from solver_cases import solver_attributes

    out = {}
    for case, (dtype, precision) in CASES.items():
        ggu, g0, u0, d, w = problem(dtype)
        attrs = solver_attributes(ggu, g0, u0, d, w, SHAPE, GAIN)
        meta, sol, calls = reference_solve_iteratively(ref_root, attrs, precision=precision,
                                                       **SCHEDULE)
        assert len(calls) == 1
        call = calls[0]
        out.update({f"{case}_in_g0": g0, f"{case}_in_u0": u0, f"{case}_in_d": d,
                    f"{case}_in_w": w, f"{case}_precision": -1 if precision is None else precision})
        for name, value in zip(OMNICAL_ARGS, call["args"][:5]):
            out[f"{case}_omnical_{name}"] = value
        out[f"{case}_omnical_precision"] = call["kwargs"]["precision"]
        out[f"{case}_omnical_gain"] = call["kwargs"]["gain"]
        for k, v in call["result"].items():
            out[f"{case}_result_{k}"] = v
        for k, v in meta.items():
            out[f"{case}_meta_{k}"] = v
        names = sorted(sol)
        out[f"{case}_sol_names"] = np.array(names)
        out[f"{case}_sol_values"] = np.stack([sol[n] for n in names])
        print(case, "iters", np.unique(meta["iter"]))
    np.savez_compressed(os.path.join(HERE, "redcal_solver_reference.npz"), **out)


if __name__ == "__main__":
    main(sys.argv[1])
