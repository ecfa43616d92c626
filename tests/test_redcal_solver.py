"""The solver-level Omnical API (hera_gpu.redcal.OmnicalSolverGPU /
RedundantCalibratorGPU, redcal.py:746-883).

CPU: packing a solver's equations and starting solution into ``omnical``'s
arrays (names numbered in first-appearance order, conjugation marks
dropped), unpacking a result by name into the solution's shape, and the two
classes made on hera_cal's -- with a stand-in ``hera_cal.redcal`` module and
a stand-in ``omnical`` that records its arguments.  Pinned to the
reference's own solve_iteratively run on the CPU
(tests/golden/make_redcal_solver_golden.py): the same arrays handed to
``omnical``, and from the same ``omnical`` result the same meta and
solution, types included.  GPU: the solver path
against ``omnical`` on the same arrays (the same launch, so equal) and
against the oracle, on a 19-antenna hexagonal array in float64.
"""
import os
import sys
import types

import numpy as np
import pytest

from hera_gpu_gb300 import redcal, synth
from oracle import omnical_oracle
from solver_cases import FakeSolver, gain_name, ubl_name

SHAPE = (6, 4)       # (times, frequencies): 24 problems


def hex_solver(dtype=np.complex128, seed=3, gain=0.3):
    ggu, nubls = synth.hex_redundant_layout(19)
    g0, u0, d, w = synth.redundant_data(ggu, nubls, int(np.prod(SHAPE)), seed, noise=1e-3)
    solver = FakeSolver(ggu, g0.astype(dtype), u0.astype(dtype), d.astype(dtype), w, SHAPE,
                        gain)
    return solver, ggu, (g0, u0, d, w)


# ---------------------------------------------------------------- CPU

def test_variable_name_drops_the_conjugation_mark():
    assert redcal.variable_name("g_3_Jxx_") == "g_3_Jxx"
    assert redcal.variable_name("g_3_Jxx") == "g_3_Jxx"
    assert redcal.variable_name(7) == "7"


@pytest.mark.parametrize("dtype,precision", [(np.complex64, 1), (np.complex128, 2)])
def test_pack_solver_restates_the_problem(dtype, precision):
    solver, ggu, (g0, u0, d, w) = hex_solver(dtype)
    p = redcal.pack_solver(solver)
    assert p["precision"] == precision and p["shape"] == SHAPE
    assert p["ggu"].dtype == np.uint32 and p["ggu"].shape == ggu.shape
    gains_of = {v: k for k, v in p["gain_map"].items()}
    ubls_of = {v: k for k, v in p["ubl_map"].items()}
    # every equation names the same variables as the layout it came from
    for (i, j, k), (pi, pj, pk) in zip(ggu, p["ggu"]):
        assert (gains_of[pi], gains_of[pj], ubls_of[pk]) == (gain_name(i), gain_name(j),
                                                            ubl_name(k))
    # numbered in the order the names first appear
    first = list(dict.fromkeys(n for i, j, _ in ggu for n in (gain_name(i), gain_name(j))))
    assert list(p["gain_map"]) == first and list(p["gain_map"].values()) == list(range(19))
    for name, col in p["gain_map"].items():
        np.testing.assert_array_equal(p["gains"][:, col], solver.sol0[name].ravel())
    for name, col in p["ubl_map"].items():
        np.testing.assert_array_equal(p["ubls"][:, col], solver.sol0[name].ravel())
    assert p["data"].dtype == dtype and p["wgts"].dtype == (np.float32 if precision == 1
                                                            else np.float64)
    np.testing.assert_array_equal(p["data"], d.astype(dtype))
    np.testing.assert_array_equal(p["wgts"], w)
    # an explicit precision sets the weights' type; the solution keeps its own
    assert redcal.pack_solver(solver, precision=3 - precision)["gains"].dtype == dtype


def test_pack_solver_rejects_real_solutions():
    solver, _, _ = hex_solver()
    solver.sol0 = {k: v.real.copy() for k, v in solver.sol0.items()}
    with pytest.raises(AssertionError):
        redcal.pack_solver(solver)


class RecordingOmnical:
    """Stands in for ``omnical``: records its arguments and returns
    recognisable arrays (gains x 2, ubls x 3, iters / chisq / conv counting
    the problems)."""

    def __call__(self, ggu, gains, ubls, data, wgts, conv_crit, maxiter, check_every,
                 check_after, gain, precision, verbose, context):
        self.args = dict(ggu=ggu, conv_crit=conv_crit, maxiter=maxiter, check_every=check_every,
                         check_after=check_after, gain=gain, precision=precision,
                         verbose=verbose, context=context)
        n = gains.shape[0]
        return {"gains": gains * 2, "ubls": ubls * 3, "iters": np.arange(n, dtype=np.uint32),
                "chisq": np.arange(n) * 0.5, "conv": np.arange(n) * 0.25}


def test_solve_iteratively_unpacks_by_name(monkeypatch):
    fake = RecordingOmnical()
    monkeypatch.setattr(redcal, "omnical", fake)
    solver, _, _ = hex_solver(gain=0.4)
    start = {k: v.copy() for k, v in solver.sol0.items()}
    meta, sol = redcal.solve_iteratively(solver, conv_crit=1e-8, maxiter=30, check_every=6,
                                         check_after=5)
    assert sol is solver.sol0          # written into the solver's solution, as the reference
    for name in start:
        factor = 2 if name.startswith("g_") else 3
        assert sol[name].shape == SHAPE
        np.testing.assert_array_equal(sol[name], start[name] * factor)
    n = int(np.prod(SHAPE))
    np.testing.assert_array_equal(meta["iter"], np.arange(n).reshape(SHAPE))
    np.testing.assert_array_equal(meta["chisq"], (np.arange(n) * 0.5).reshape(SHAPE))
    np.testing.assert_array_equal(meta["conv_crit"], (np.arange(n) * 0.25).reshape(SHAPE))
    assert fake.args["gain"] == 0.4 and fake.args["precision"] == 2
    assert (fake.args["conv_crit"], fake.args["maxiter"], fake.args["check_every"],
            fake.args["check_after"]) == (1e-8, 30, 6, 5)


@pytest.fixture
def stand_in_hera_cal(monkeypatch):
    """A ``hera_cal.redcal`` module whose RedundantCalibrator keys solutions
    by tuples outside and by names inside, and builds solvers from a layout."""
    ggu, nubls = synth.hex_redundant_layout(19)
    g0, u0, d, w = synth.redundant_data(ggu, nubls, int(np.prod(SHAPE)), 5, noise=1e-3)

    class OmnicalSolver:
        pass

    class RedundantCalibrator:
        def pack_sol_key(self, k):
            return gain_name(k[0]) if k[1] == "Jxx" else ubl_name(k[0])

        def unpack_sol_key(self, name):
            kind, idx = name.split("_")[:2]
            return (int(idx), "Jxx") if kind == "g" else (int(idx), "ubl")

        def _solver(self, cls, data, sol0, wgts, gain):
            s = cls()
            ref = FakeSolver(ggu, g0, u0, d, w, SHAPE, gain)
            s.keys, s.all_terms, s.data, s.wgts = ref.keys, ref.all_terms, data, ref.wgts
            s.sol0, s.gain, s.wgts_given = sol0, gain, wgts
            self.solver = s
            return s

    mod = types.ModuleType("hera_cal.redcal")
    mod.OmnicalSolver, mod.RedundantCalibrator = OmnicalSolver, RedundantCalibrator
    pkg = types.ModuleType("hera_cal")
    pkg.redcal = mod
    monkeypatch.setitem(sys.modules, "hera_cal", pkg)
    monkeypatch.setitem(sys.modules, "hera_cal.redcal", mod)
    return mod, FakeSolver(ggu, g0, u0, d, w, SHAPE)


def test_classes_subclass_hera_cal(stand_in_hera_cal):
    mod, _ = stand_in_hera_cal
    from hera_gpu_gb300.redcal import OmnicalSolverGPU, RedundantCalibratorGPU
    assert issubclass(OmnicalSolverGPU, mod.OmnicalSolver)
    assert issubclass(RedundantCalibratorGPU, mod.RedundantCalibrator)
    assert redcal.OmnicalSolverGPU is OmnicalSolverGPU      # made once
    with pytest.raises(AttributeError):
        redcal.NoSuchSolver


def test_classes_need_hera_cal(monkeypatch):
    monkeypatch.setitem(sys.modules, "hera_cal", None)
    monkeypatch.setitem(sys.modules, "hera_cal.redcal", None)
    with pytest.raises(ImportError):
        redcal.RedundantCalibratorGPU


def test_omnical_gpu_keys_and_arguments(stand_in_hera_cal, monkeypatch):
    _, ref = stand_in_hera_cal
    fake = RecordingOmnical()
    monkeypatch.setattr(redcal, "omnical", fake)
    info = redcal.RedundantCalibratorGPU()
    sol0 = {(int(n.split("_")[1]), "Jxx" if n.startswith("g_") else "ubl"): v
            for n, v in ref.sol0.items()}
    meta, sol = info.omnical_gpu(ref.data, sol0, gain=0.5, conv_crit=1e-12, maxiter=500,
                                 check_every=6, check_after=30, precision=1)
    assert set(sol) == set(sol0)
    for k in sol0:
        np.testing.assert_array_equal(sol[k], sol0[k] * (2 if k[1] == "Jxx" else 3))
    assert isinstance(info.solver, redcal.OmnicalSolverGPU)
    assert info.solver.wgts_given == {} and info.solver.gain == 0.5
    assert (fake.args["conv_crit"], fake.args["maxiter"], fake.args["check_every"],
            fake.args["check_after"], fake.args["precision"]) == (1e-12, 500, 6, 30, 1)
    assert meta["iter"].shape == SHAPE


REFERENCE = os.path.join(os.path.dirname(__file__), "golden", "redcal_solver_reference.npz")
REFERENCE_CASES = ["c64_auto", "c128_auto", "c128_p1"]


def reference_case(case):
    """The reference's own solve_iteratively on a 19-antenna hex array of
    3 x 2 problems (tests/golden/make_redcal_solver_golden.py): the solver
    it ran on, its precision argument and what it did."""
    z = np.load(REFERENCE)
    ggu, _ = synth.hex_redundant_layout(19)
    solver = FakeSolver(ggu, z[f"{case}_in_g0"], z[f"{case}_in_u0"], z[f"{case}_in_d"],
                        z[f"{case}_in_w"], (3, 2), 0.3)
    p = int(z[f"{case}_precision"])
    return z, solver, (None if p < 0 else p)


@pytest.mark.parametrize("case", REFERENCE_CASES)
def test_pack_solver_matches_the_reference(case):
    # the arrays the reference's solve_iteratively handed to its omnical
    z, solver, precision = reference_case(case)
    p = redcal.pack_solver(solver, precision)
    np.testing.assert_array_equal(p["ggu"].astype(np.int64),
                                  z[f"{case}_omnical_ggu"].astype(np.int64))
    for k in ("gains", "ubls", "data", "wgts"):
        ref = z[f"{case}_omnical_{k}"]
        assert p[k].dtype == ref.dtype, k
        np.testing.assert_array_equal(p[k], ref)
    assert p["precision"] == int(z[f"{case}_omnical_precision"])
    assert solver.gain == float(z[f"{case}_omnical_gain"])


@pytest.mark.parametrize("case", REFERENCE_CASES)
def test_solve_iteratively_matches_the_reference(case, monkeypatch):
    # given what the reference's omnical returned, the same meta and solution
    z, solver, precision = reference_case(case)
    result = {k: z[f"{case}_result_{k}"].copy() for k in ("gains", "ubls", "chisq", "iters", "conv")}
    monkeypatch.setattr(redcal, "omnical", lambda *args, **kwargs: result)
    meta, sol = redcal.solve_iteratively(solver, conv_crit=1e-10, maxiter=60,
                                         precision=precision)
    for k in ("iter", "chisq", "conv_crit"):
        ref = z[f"{case}_meta_{k}"]
        assert meta[k].dtype == ref.dtype, k
        np.testing.assert_array_equal(meta[k], ref)
    names = [str(n) for n in z[f"{case}_sol_names"]]
    assert sorted(sol) == names
    for name, value in zip(names, z[f"{case}_sol_values"]):
        np.testing.assert_array_equal(sol[name], value)
        assert sol[name].shape == value.shape and sol[name].dtype == value.dtype


# ---------------------------------------------------------------- GPU

@pytest.mark.gpu
def test_solver_path_on_the_gpu():
    solver, ggu, _ = hex_solver(np.complex128)
    p = redcal.pack_solver(solver)
    # every problem converges, after 144 to 360 iterations
    direct = redcal.omnical(p["ggu"], p["gains"], p["ubls"], p["data"], p["wgts"], 1e-10, 500,
                            4, 1, gain=0.3, precision=2)
    ref = omnical_oracle(p["ggu"], p["gains"], p["ubls"], p["data"], p["wgts"], 1e-10, 500, 4,
                         1, 0.3, precision=2)
    meta, sol = redcal.solve_iteratively(solver, conv_crit=1e-10, maxiter=500)
    for name, col in p["gain_map"].items():
        np.testing.assert_array_equal(sol[name].ravel(), direct["gains"][:, col])
        np.testing.assert_allclose(sol[name].ravel(), ref["gains"][:, col], rtol=0,
                                   atol=1e-9 * np.abs(ref["gains"]).max())
    for name, col in p["ubl_map"].items():
        np.testing.assert_array_equal(sol[name].ravel(), direct["ubls"][:, col])
    np.testing.assert_array_equal(meta["iter"].ravel(), direct["iters"])
    np.testing.assert_array_equal(meta["chisq"].ravel(), direct["chisq"])
    assert (meta["iter"].ravel() == ref["iters"]).mean() >= 0.95
