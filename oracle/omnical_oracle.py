"""CPU oracle of hera_gpu's omnical solver -- TEST INFRASTRUCTURE ONLY.

Restates the algorithm of hera_gpu/redcal.py:358-743 (`omnical`, the host
loop) and its kernels (redcal.py:19-355) in numpy, vectorised over the
independent problems ("pixels"), for data modelled as
    data[p, b] = gains[p, i_b] * conj(gains[p, j_b]) * ubls[p, k_b]
with (i_b, j_b, k_b) = ggu_indices[b]:

  * dmdl = g_i conj(g_j) u_k (gen_dmdl, :70-94); chisq = sum_b |data - dmdl|^2 w
    (calc_chisq, :97-114);
  * initial chisq before the loop (host :566-577);
  * iteration it = 1 .. maxiter (host :587) while the problem is active:
      - when it % check_every == 1, dwgts = |dmdl|^2 w (calc_dwgts, :117-132)
        and the weights gwgt[a] / uwgt[k] = sums of dwgts over the baselines
        that touch antenna a (as i or as j) / unique baseline k
        (calc_gu_wgt, :171-196; host :590-604);
      - d_b = data_b conj(dmdl_b) dwgts_b / |dmdl_b|^2, gbuf[i_b] += d_b,
        gbuf[j_b] += conj(d_b), ubuf[k_b] += d_b (calc_gu_buf, :199-236);
      - the step: x *= (1 - gain) + gain * buf / wgt (update_gains / update_ubls,
        :239-280, the real part of the factor carrying the 1 - gain); the
        reference passes the gain as a float32 (host :625,630,657,662) and forms
        1 - gain in float32 at both precisions;
      - if it < maxiter and (it < check_after or it % check_every != 0)
        (host :619): take the step and regenerate dmdl;
        otherwise check (host :644-702): with the stepped solution, new chisq
        and conv = sqrt(sum |new - old|^2 / sum |new|^2) over gains and ubls
        (calc_conv, :283-311); conv < conv_crit (rounded to the working
        precision, host :691) ends the problem keeping the old solution,
        so does new chisq > chisq; otherwise the step is taken, chisq and
        iters (= it) are updated (update_active, :314-354);
  * returns gains, ubls, chisq, iters (0 if no check ever accepted: the
    reference leaves that buffer uninitialised) and conv.

Sums are taken in float64 here.  Pinned by the reference's own known answers
(hera_gpu/tests/test_redcal.py:64-101, restated in tests/test_omnical.py) and
by the reference's own omnical -- its host loop and its kernels, run on the
CPU by oracle/redcal_ref.py -- on seven seeded problems
(tests/golden/omnical_*.npz): in float64 the gains agree to ~1e-15 and the
stopping iteration is the same.  Only tests/ and bench.py's CPU baseline use
this module.
"""
import numpy as np


def omnical_oracle(ggu_indices, gains, ubls, data, wgts, conv_crit=1e-10, maxiter=50,
                   check_every=4, check_after=1, gain=0.3, precision=2):
    # a unique baseline or antenna whose baselines all have zero weight
    # gives 0 / 0 = NaN, as in the reference
    with np.errstate(invalid="ignore", divide="ignore"):
        return _omnical(ggu_indices, gains, ubls, data, wgts, conv_crit, maxiter, check_every,
                        check_after, gain, precision)


def _omnical(ggu_indices, gains, ubls, data, wgts, conv_crit, maxiter, check_every,
             check_after, gain, precision):
    assert check_every > 1
    gstep = float(np.float32(gain))
    one_m = float(np.float32(1) - np.float32(gain))
    crit = float(np.float32(conv_crit)) if precision == 1 else float(conv_crit)
    ggu = np.asarray(ggu_indices, dtype=np.int64)
    gi, gj, uk = ggu[:, 0], ggu[:, 1], ggu[:, 2]
    g = np.array(gains, dtype=np.complex128)
    u = np.array(ubls, dtype=np.complex128)
    d = np.asarray(data, dtype=np.complex128)
    w = np.asarray(wgts, dtype=np.float64)
    ndata, nants = g.shape
    nubls = u.shape[1]
    # incidence of baselines on antennas and unique baselines
    Ai = np.zeros((len(ggu), nants))
    Aj = np.zeros((len(ggu), nants))
    Au = np.zeros((len(ggu), nubls))
    Ai[np.arange(len(ggu)), gi] = 1
    Aj[np.arange(len(ggu)), gj] = 1
    Au[np.arange(len(ggu)), uk] = 1

    def model(g_, u_):
        return g_[:, gi] * np.conj(g_[:, gj]) * u_[:, uk]

    def chisq_of(m):
        return np.sum(np.abs(d - m) ** 2 * w, axis=1)

    dmdl = model(g, u)
    chisq = chisq_of(dmdl)
    iters = np.zeros(ndata, dtype=np.int64)
    conv = np.zeros(ndata)
    active = np.ones(ndata, dtype=bool)
    dwgts = np.zeros_like(w)
    gwgt = np.zeros((ndata, nants))
    uwgt = np.zeros((ndata, nubls))
    for it in range(1, maxiter + 1):
        a = active
        if not a.any():
            break
        if it % check_every == 1:
            dwgts[a] = np.abs(dmdl[a]) ** 2 * w[a]
            gwgt[a] = dwgts[a] @ (Ai + Aj)
            uwgt[a] = dwgts[a] @ Au
        dd = d[a] * np.conj(dmdl[a]) * (dwgts[a] / np.abs(dmdl[a]) ** 2)
        gbuf = dd @ Ai + np.conj(dd) @ Aj
        ubuf = dd @ Au
        fg = one_m + gstep * gbuf.real / gwgt[a] + 1j * (gstep * gbuf.imag / gwgt[a])
        fu = one_m + gstep * ubuf.real / uwgt[a] + 1j * (gstep * ubuf.imag / uwgt[a])
        new_g = g[a] * fg
        new_u = u[a] * fu
        idx = np.flatnonzero(a)
        if it < maxiter and (it < check_after or it % check_every != 0):
            g[idx] = new_g
            u[idx] = new_u
            dmdl[idx] = model(new_g, new_u)
            continue
        new_m = model(new_g, new_u)
        dmdl[idx] = new_m
        new_chisq = chisq_of_rows(d[idx], new_m, w[idx])
        cs = np.sum(np.abs(new_g - g[idx]) ** 2, axis=1) + np.sum(np.abs(new_u - u[idx]) ** 2, axis=1)
        cw = np.sum(np.abs(new_g) ** 2, axis=1) + np.sum(np.abs(new_u) ** 2, axis=1)
        conv[idx] = np.sqrt(cs / cw)
        done = (conv[idx] < crit) | (new_chisq > chisq[idx])
        keep = idx[~done]
        sel = ~done
        g[keep] = new_g[sel]
        u[keep] = new_u[sel]
        chisq[keep] = new_chisq[sel]
        iters[keep] = it
        active[idx[done]] = False
    return {"gains": g, "ubls": u, "chisq": chisq, "iters": iters, "conv": conv}


def chisq_of_rows(d, m, w):
    return np.sum(np.abs(d - m) ** 2 * w, axis=1)


def redundant_problem(nants, ndata, seed=0, gain_scatter=0.05, noise=0.0, spacing=14.6):
    """A redundant linear array: baselines (i, j), i > j, in unique-baseline
    groups by separation i - j - 1 (the reference's test layout,
    test_redcal.py:57-64), true gains 1 + scatter and true unique baselines
    of unit order; returns (ggu_indices, true_gains, true_ubls, data, wgts)."""
    rng = np.random.default_rng(seed)
    ggu = np.array([(i, j, i - j - 1) for i in range(nants) for j in range(i)], dtype=np.uint32)
    nubls = nants - 1
    g = 1 + gain_scatter * (rng.normal(size=(ndata, nants)) + 1j * rng.normal(size=(ndata, nants)))
    u = rng.normal(size=(ndata, nubls)) + 1j * rng.normal(size=(ndata, nubls))
    gi, gj, uk = ggu[:, 0], ggu[:, 1], ggu[:, 2]
    d = g[:, gi] * np.conj(g[:, gj]) * u[:, uk]
    if noise:
        d = d + noise * (rng.normal(size=d.shape) + 1j * rng.normal(size=d.shape))
    w = np.ones(d.shape)
    return ggu, g, u, d, w
