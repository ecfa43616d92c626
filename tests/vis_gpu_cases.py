"""The reference's own vis_gpu outputs (tests/golden/vis_gpu_reference.npz,
made by tests/golden/make_vis_gpu_golden.py): its host loop and kernels run
on the CPU, on the inputs of small_config / random_inputs / edge_inputs and
on a ragged case of 1003 sources, of which the reference sums the first
1000 (hera_gpu/vis.py:176-177)."""
import os

import numpy as np

GOLDEN = os.path.join(os.path.dirname(__file__), "golden")
VIS_GPU_CASES = ["small_config", "random_inputs", "edge_inputs", "ragged"]
ARGS = ("antpos", "freq", "eq2tops", "crd_eq", "I_sky", "bm_cube")


def load_vis_gpu_case(name):
    """(inputs restricted to the sources the reference sums, all inputs,
    the reference's vis_gpu outputs {1: precision 1, 2: precision 2})."""
    z = np.load(os.path.join(GOLDEN, "vis_gpu_reference.npz"))
    if name == "ragged":
        a = {k: z["ragged_" + k] for k in ARGS}
    else:
        d = np.load(os.path.join(GOLDEN, name + ".npz"))
        a = {k: d[k] for k in ARGS}
    full = (a["antpos"], float(a["freq"]), a["eq2tops"], a["crd_eq"], a["I_sky"], a["bm_cube"])
    n = int(z[name + "_nsrc_used"])
    used = full[:3] + (full[3][:, :n], full[4][:n], full[5])
    return used, full, {1: z[name + "_p1"], 2: z[name + "_p2"]}
