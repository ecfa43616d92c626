"""Omnical solver objects for tests: the attributes of hera_cal's
OmnicalSolver that the solver-level API reads, built from a layout."""
import types


def gain_name(a):
    return f"g_{a}_Jxx"


def ubl_name(k):
    return f"u_{k}_xx"


def solver_attributes(ggu, gains, ubls, data, wgts, shape, gain=0.3):
    """One product term g_i * conj(g_j) * u_k per data key (i, j, 'xx'), the
    conjugated factor named with linsolve's trailing '_'; arrays of
    ``shape`` from columns of the (ndata, n) matrices."""
    keys = [(int(i), int(j), "xx") for i, j, _ in ggu]
    sol0 = {gain_name(a): gains[:, a].reshape(shape) for a in range(gains.shape[1])}
    sol0.update({ubl_name(k): ubls[:, k].reshape(shape) for k in range(ubls.shape[1])})
    return {"keys": keys,
            "all_terms": [[(gain_name(i), gain_name(j) + "_", ubl_name(k))] for i, j, k in ggu],
            "sol0": sol0,
            "data": {key: data[:, b].reshape(shape) for b, key in enumerate(keys)},
            "wgts": {key: wgts[:, b].reshape(shape) for b, key in enumerate(keys)},
            "gain": gain}


def FakeSolver(ggu, gains, ubls, data, wgts, shape, gain=0.3):
    return types.SimpleNamespace(**solver_attributes(ggu, gains, ubls, data, wgts, shape, gain))
