"""Drop-in for hera_gpu's Omnical solver (``hera_gpu.redcal.omnical``).

The reference (hera_gpu/redcal.py:358-743) solves many independent Omnical
problems -- one per "pixel" (frequency x time sample) -- 64 at a time, with
a dozen kernel launches per iteration and a host round trip at every
convergence check.  Here every problem of the call goes through one launch of
libheravis.so's omnical kernel (``hv_omnical``): one CTA per problem, all
iterations inside the kernel, deterministic sums.

The reference's ``OmnicalSolverGPU`` / ``RedundantCalibratorGPU``
(redcal.py:746-883) subclass ``hera_cal.redcal``'s ``OmnicalSolver`` and
``RedundantCalibrator``.  ``hera_cal`` is not a dependency of this package:
the two classes are made on first access, from the installed ``hera_cal``
(ImportError without it).  Their work -- packing a solver's equations and
starting solution into ``omnical``'s arrays and unpacking the result by
name -- is ``pack_solver`` / ``solve_iteratively`` below, which take any
object with an OmnicalSolver's attributes.
"""
from __future__ import annotations

import numpy as np

from . import _native

NTHREADS = 1024
_CLASSES = {}


def omnical(ggu_indices, gains, ubls, data, wgts, conv_crit=1e-10, maxiter=50, check_every=4,
            check_after=1, gain=0.3, nthreads=NTHREADS, precision=1, verbose=False,
            context=None):
    """Omnical iterations for ``ndata`` independent problems.

    Args (as hera_gpu.redcal.omnical, redcal.py:358-389):
        ggu_indices: (nbls, 3) indices (i, j, k): data = gains[i] gains[j]* ubls[k]
        gains: (ndata, nants) starting gains
        ubls: (ndata, nubls) starting unique-baseline visibilities
        data: (ndata, nbls) data; wgts: (ndata, nbls) weights
        conv_crit, maxiter, check_every, check_after, gain: as the reference
        nthreads: accepted and not needed (the library picks its launch)
        precision: 1 = float32 / complex64, 2 = float64 / complex128

    Returns {'gains', 'ubls', 'chisq', 'iters', 'conv'} (new arrays; the
    inputs are not modified, as the reference's astype copies).
    """
    nbls = ggu_indices.shape[0]
    assert ggu_indices.shape == (nbls, 3)
    ndata = data.shape[0]
    assert data.shape == (ndata, nbls)
    assert wgts.shape == (ndata, nbls)
    nants = gains.shape[1]
    assert gains.shape == (ndata, nants)
    nubls = ubls.shape[1]
    assert ubls.shape == (ndata, nubls)
    assert precision in (1, 2)
    assert check_every > 1
    if verbose:
        print("PRECISION:", precision)
        print("NDATA:", ndata)
        print("NANTS:", nants)
        print("NUBLS:", nubls)
        print("NBLS:", nbls)
    rt, ct = (np.float32, np.complex64) if precision == 1 else (np.float64, np.complex128)
    ggu = np.ascontiguousarray(ggu_indices, dtype=np.uint32)
    data = np.ascontiguousarray(data, dtype=ct)
    wgts = np.ascontiguousarray(wgts, dtype=rt)
    gains = np.array(gains, dtype=ct, order="C", copy=True)
    ubls = np.array(ubls, dtype=ct, order="C", copy=True)
    chisq = np.empty((ndata,), dtype=rt)
    conv = np.empty((ndata,), dtype=rt)
    iters = np.empty((ndata,), dtype=np.uint32)
    ctx = context or _native.default_context()
    ctx.omnical(precision, ggu, gains, ubls, data, wgts, conv_crit, maxiter, check_every,
                check_after, gain, chisq, iters, conv)
    return {"gains": gains, "ubls": ubls, "chisq": chisq, "iters": iters, "conv": conv}


def variable_name(factor):
    """The variable a factor of a linsolve product term names (the
    reference's ``linsolve.get_name``, redcal.py:10, 781): a string with any
    trailing '_' (linsolve's mark of a conjugated variable) removed; any
    other factor as ``str``."""
    return factor.rstrip("_") if isinstance(factor, str) else str(factor)


def pack_solver(solver, precision=None):
    """``omnical``'s inputs from an OmnicalSolver (redcal.py:780-823).

    ``solver`` has ``sol0`` (variable name -> array, every array of one
    shape), ``all_terms`` (per equation, a list of (gi, gj*, uij) factor
    triples), ``keys`` (the data keys, one per equation), ``data`` and
    ``wgts`` (key -> array of the solution's shape) and ``gain``.  Gains and
    unique baselines are numbered in the order their names first appear in
    the terms, as the reference numbers them.

    Returns a dict: ggu (nbls, 3) uint32, gains (ndata, ngains), ubls
    (ndata, nubls), data (ndata, nbls) in the solution's complex type, wgts
    (ndata, nbls) in precision's real type, gain_map / ubl_map (name ->
    column), shape (of one solution array) and precision.
    """
    sol = solver.sol0
    terms = [tuple(variable_name(f) for f in term) for eq in solver.all_terms for term in eq]
    assert terms, "no equations"
    gain_map, ubl_map = {}, {}
    for gi, gj, uij in terms:
        gain_map.setdefault(gi, len(gain_map))
        gain_map.setdefault(gj, len(gain_map))
        ubl_map.setdefault(uij, len(ubl_map))
    ggu = np.array([(gain_map[gi], gain_map[gj], ubl_map[uij]) for gi, gj, uij in terms],
                   dtype=np.uint32).reshape(-1, 3)
    # the reference takes shape and type from the last term's first gain
    v = np.asarray(sol[terms[-1][0]])
    shape, dtype, ndata = v.shape, v.dtype, v.size
    assert dtype in (np.complex64, np.complex128)
    if precision is None:
        precision = 1 if dtype == np.complex64 else 2
    real_dtype = np.float32 if precision == 1 else np.float64
    gains = np.empty((ndata, len(gain_map)), dtype=dtype)
    for k, col in gain_map.items():
        gains[:, col] = np.asarray(sol[k]).ravel()
    ubls = np.empty((ndata, len(ubl_map)), dtype=dtype)
    for k, col in ubl_map.items():
        ubls[:, col] = np.asarray(sol[k]).ravel()
    nbls = len(solver.keys)
    data = np.empty((ndata, nbls), dtype=dtype)
    wgts = np.empty((ndata, nbls), dtype=real_dtype)
    for i, k in enumerate(solver.keys):
        data[:, i] = np.asarray(solver.data[k]).ravel()
        wgts[:, i] = np.asarray(solver.wgts[k]).ravel()
    return {"ggu": ggu, "gains": gains, "ubls": ubls, "data": data, "wgts": wgts,
            "gain_map": gain_map, "ubl_map": ubl_map, "shape": shape, "precision": precision}


def solve_iteratively(solver, conv_crit=1e-10, maxiter=50, check_every=4, check_after=1,
                      precision=None, verbose=False, context=None):
    """``OmnicalSolverGPU.solve_iteratively`` (redcal.py:747-837) for any
    object with an OmnicalSolver's attributes (see ``pack_solver``):
    ``omnical`` over every sample of the solution, with the solver's
    ``gain`` as the step.  ``precision`` None takes it from the solution's
    type.

    Returns (meta, sol).  meta: 'iter', 'chisq', 'conv_crit', each of the
    solution's shape.  sol: ``solver.sol0`` with every gain and unique
    baseline replaced by its solution (the reference writes into sol0 too).
    """
    p = pack_solver(solver, precision)
    result = omnical(p["ggu"], p["gains"], p["ubls"], p["data"], p["wgts"], conv_crit, maxiter,
                     check_every, check_after, gain=solver.gain, precision=p["precision"],
                     verbose=verbose, context=context)
    sol, shape = solver.sol0, p["shape"]
    for k, col in p["gain_map"].items():
        sol[k] = np.reshape(result["gains"][:, col], shape)
    for k, col in p["ubl_map"].items():
        sol[k] = np.reshape(result["ubls"][:, col], shape)
    meta = {"iter": np.reshape(result["iters"], shape),
            "chisq": np.reshape(result["chisq"], shape),
            "conv_crit": np.reshape(result["conv"], shape)}
    return meta, sol


def _make_classes():
    """OmnicalSolverGPU / RedundantCalibratorGPU on the installed hera_cal's
    classes (redcal.py:746, 839), made once per pair of base classes."""
    from hera_cal.redcal import OmnicalSolver, RedundantCalibrator
    key = (OmnicalSolver, RedundantCalibrator)
    if key in _CLASSES:
        return _CLASSES[key]

    class OmnicalSolverGPU(OmnicalSolver):
        """hera_cal's OmnicalSolver with ``solve_iteratively`` on the GPU."""

        def solve_iteratively(self, conv_crit=1e-10, maxiter=50, check_every=4,
                              check_after=1, precision=None, verbose=False):
            return solve_iteratively(self, conv_crit, maxiter, check_every, check_after,
                                     precision, verbose)

    class RedundantCalibratorGPU(RedundantCalibrator):
        """hera_cal's RedundantCalibrator with ``omnical_gpu``."""

        def omnical_gpu(self, data, sol0, wgts=None, gain=.3, conv_crit=1e-10, maxiter=50,
                        check_every=4, check_after=1, precision=None):
            """Drop-in for RedundantCalibrator.omnical on the GPU
            (redcal.py:840-883): sol0 and the returned sol are keyed by
            antenna / baseline tuples."""
            sol0 = {self.pack_sol_key(k): sol0[k] for k in sol0.keys()}
            ls = self._solver(OmnicalSolverGPU, data, sol0=sol0,
                              wgts={} if wgts is None else wgts, gain=gain)
            meta, sol = ls.solve_iteratively(conv_crit=conv_crit, maxiter=maxiter,
                                             check_every=check_every, check_after=check_after,
                                             precision=precision)
            return meta, {self.unpack_sol_key(k): sol[k] for k in sol.keys()}

    _CLASSES[key] = {"OmnicalSolverGPU": OmnicalSolverGPU,
                     "RedundantCalibratorGPU": RedundantCalibratorGPU}
    return _CLASSES[key]


def __getattr__(name):
    if name in ("OmnicalSolverGPU", "RedundantCalibratorGPU"):
        return _make_classes()[name]
    raise AttributeError(f"module {__name__!r} has no attribute {name!r}")
