"""Generate the golden vectors in tests/golden/ from the reference itself.

Run on a machine that has the reference sources (they are compiled into
oracle/_ref/libglassref.so by oracle/Makefile.ref; nothing is copied):

    python tests/golden/make_golden.py

Every output value below comes from the reference's own functions:
ucb_waveform (ucb/src/glass_ucb_waveform.c:738), ucb_bandwidth (:698),
ucb_alignment (:727), AEnoise_FF (utils/src/glass_lisa.c:1137),
generate_ucb_model + gaussian_log_likelihood (ucb/src/glass_ucb_model.c:55,
utils/src/glass_model.c:726), snr (utils/src/glass_math.c:403) and ucb_fisher
(ucb/src/glass_ucb_waveform.c:364), the WDM transforms
(utils/src/glass_wavelet.c:293, :351, :544, :327), ucb_waveform_wavelet
(ucb/src/glass_ucb_waveform.c:1061) with initialize_interpolated_analytic_orbits
(utils/src/glass_lisa.c:271), delta_log_likelihood and
gaussian_log_likelhood_wavelet (utils/src/glass_model.c:624, :805) and
snr_wavelet (utils/src/glass_math.c:428), get_Fstat_logL
(ucb/src/glass_ucb_fstatistic.c:646) and build_fstatistic_proposal
(ucb/src/glass_ucb_proposal.c:1085), and the noise module's
generate_instrument_noise_model, generate_galactic_foreground_model,
invert_noise_covariance_matrix and my_noise_log_likelihood
(noise/src/glass_noise_model.c:389, :612, utils/src/glass_math.c:240,
noise/src/glass_noise_model.c:1243) with their wavelet-domain, coarse-grained
forms (:561, :656, :923, :983, :1057, :1211), and the UCB sampler's noise
step (noise_model_mcmc, ucb/src/glass_ucb_sampler.c:29), and the
parallel-tempering exchange ptmcmc (utils/src/glass_sampler.c:19).  Inputs are
seeded numpy draws.

    python tests/golden/make_golden.py            # every fixture
    python tests/golden/make_golden.py fstat noise   # only the named ones
"""
from __future__ import annotations

import math
import os
import sys

# one OpenMP thread for the reference: build_fstatistic_proposal opens a
# parallel region per frequency, and nested regions with the default team
# size make it several hundred times slower
os.environ.setdefault("OMP_NUM_THREADS", "1")

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(ROOT, "oracle"))
sys.path.insert(0, ROOT)

from oracle import Ref  # noqa: E402
from glass_gb300 import workloads as wl  # noqa: E402

T = wl.T_YEAR


def waveforms(ref, rng):
    cases = []
    for fmt in ("sangria", "phase", "frequency"):
        for N in (32, 64, 128, 256, 512, 1024):
            f0 = 10 ** rng.uniform(np.log10(0.5e-3), np.log10(15e-3))
            amp = 10 ** rng.uniform(-23, -21)
            fdot = 10 ** rng.uniform(-18, -15)
            cases.append((fmt, N, wl.draw_source(rng, f0, amp, fdot)))
    cases.append(("sangria", 4096, wl.draw_source(rng, 12e-3, 1e-22, 1e-15)))
    cases.append(("sangria", 2048, wl.draw_source(rng, 0.7e-3, 1e-22, 1e-18)))
    # t0 != 0 and NI = 1 variants
    out = {"fmt": [], "N": [], "NI": [], "t0": [], "params": [], "XYZAE": []}
    for fmt, N, p in cases:
        for t0, NI in ((0.0, 2),) + (((1.5e6, 2), (0.0, 1)) if N == 128 else ()):
            h = ref.waveform(p, N, T, t0=t0, fmt=fmt, NI=NI)
            out["fmt"].append(fmt)
            out["N"].append(N)
            out["NI"].append(NI)
            out["t0"].append(t0)
            out["params"].append(p)
            out["XYZAE"].append(h)
    np.savez_compressed(os.path.join(HERE, "waveforms.npz"), fmt=np.array(out["fmt"]), N=np.array(out["N"]),
                        NI=np.array(out["NI"]), t0=np.array(out["t0"]), params=np.array(out["params"]),
                        **{f"h{i}": h for i, h in enumerate(out["XYZAE"])})


def bandwidth(ref, rng):
    n = 3000
    f = 10 ** rng.uniform(-4.3, -1.3, n)
    fdot = 10 ** rng.uniform(-20, -12, n)
    ct = rng.uniform(-1, 1, n)
    amp = 10 ** rng.uniform(-24, -19.5, n)
    nfft = 2 ** rng.integers(5, 15, n)
    bw = np.array([ref.bandwidth(f[i], fdot[i], ct[i], amp[i], T, int(nfft[i])) for i in range(n)], np.int32)
    # alignment on a config-1 like grid
    params = np.array([wl.draw_source(rng, 10 ** rng.uniform(np.log10(0.5e-3), np.log10(15e-3)),
                                      10 ** rng.uniform(-23, -21)) for _ in range(300)])
    qmin = np.array([int(p[0]) - 512 + int(rng.integers(-600, 600)) for p in params], np.int32)
    al = np.array([ref.alignment(T, 1024, int(qmin[i]), params[i]) for i in range(len(params))], np.int32)
    fgrid = np.geomspace(1e-5, 5e-2, 200)
    S = ref.aenoise_ff(fgrid, "scirdv1")
    np.savez_compressed(os.path.join(HERE, "bandwidth.npz"), f=f, fdot=fdot, costh=ct, amp=amp, nfft=nfft, bw=bw,
                        align_params=params, align_qmin=qmin, align=al, noise_f=fgrid, noise_S=S)


def likelihood(ref, rng):
    """Config-0-like segments: the injected source plus noise, and Gaussian
    jump proposals; logL of each proposal from the reference."""
    cases = []
    for k in range(3):
        f0 = rng.uniform(3.0e-3, 3.5e-3) if k < 2 else rng.uniform(0.5e-3, 15e-3)
        amp = 1e-22 if k < 2 else 10 ** rng.uniform(-23, -21)
        inj = wl.draw_source(rng, f0, amp, 1e-17)
        extra = []
        if k == 1:  # a second source near the first one, part of the residual
            extra = [wl.draw_source(rng, f0 + 40 / T, 5e-23, 1e-17)]

        def wf(p):
            al = ref.alignment(T, 1024, 0, p)
            h = ref.waveform(p, int(al[0]), T)
            return int(al[0]), h[3], h[4]

        qmin, dA, dE, iA, iE = wl.make_segment(rng, [inj] + extra, wf, NFFT=1024, T=T)
        dA_i = np.empty(2048)
        dA_i[0::2], dA_i[1::2] = dA.real, dA.imag
        dE_i = np.empty(2048)
        dE_i[0::2], dE_i[1::2] = dE.real, dE.imag
        snr0 = ref.log_likelihood(T, 1024, qmin, dA_i, dE_i, iA, iE, inj)[1][0]
        props = wl.gaussian_jumps(rng, inj, wl.jump_scales(inj, snr0), 12)
        props = np.vstack([inj[None], props])
        logL = []
        snr = []
        for p in props:
            ll, s = ref.log_likelihood(T, 1024, qmin, dA_i, dE_i, iA, iE, np.vstack([p[None]] + [e[None] for e in extra]))
            logL.append(ll)
            snr.append(s[0])
        # model with no sources at all: logL of the bare data
        ll0, _ = ref.log_likelihood(T, 1024, qmin, dA_i, dE_i, iA, iE, np.zeros((0, 8)))
        cases.append(dict(qmin=qmin, dA=dA_i, dE=dE_i, invCA=iA, invCE=iE, props=props, logL=np.array(logL),
                          snr=np.array(snr), logL_empty=ll0,
                          extra=np.array(extra) if extra else np.zeros((0, 8))))
    flat = {}
    for k, c in enumerate(cases):
        for key, v in c.items():
            flat[f"c{k}_{key}"] = v
    np.savez_compressed(os.path.join(HERE, "likelihood.npz"), ncase=len(cases), **flat)


def fisher(ref, rng):
    out = {"params": [], "F": [], "qmin": [], "invC": []}
    for k in range(4):
        f0 = rng.uniform(1e-3, 5e-3)
        p = wl.draw_source(rng, f0, 10 ** rng.uniform(-23, -21), 1e-17)
        qmin = int(p[0]) - 512
        invC = 1.0 / wl.aenoise_ff((qmin + np.arange(1024)) / T)
        F, ev, evec = ref.fisher(p, T, 1024, qmin, invC, invC)
        out["params"].append(p)
        out["F"].append(F)
        out["qmin"].append(qmin)
        out["invC"].append(invC)
    np.savez_compressed(os.path.join(HERE, "fisher.npz"), **{k: np.array(v) for k, v in out.items()})


def fisher_big(ref, rng):
    """ucb_fisher on 8192-bin segments with templates of 2048 and 4096
    samples (two each): loud sources at 5-20 mHz, redrawn until the
    reference's own alignment gives the wanted size."""
    NFFT = 8192
    out = {"params": [], "F": [], "qmin": [], "invC": [], "N": []}
    for want in (2048, 2048, 4096, 4096):
        while True:
            p = wl.draw_source(rng, rng.uniform(5e-3, 2e-2), 10 ** rng.uniform(-21, -20), 1e-17)
            qmin = int(p[0]) - NFFT // 2
            N = int(ref.alignment(T, NFFT, qmin, p)[0])
            if N == want:
                break
        invC = 1.0 / wl.aenoise_ff((qmin + np.arange(NFFT)) / T)
        F, ev, evec = ref.fisher(p, T, NFFT, qmin, invC, invC)
        out["params"].append(p)
        out["F"].append(F)
        out["qmin"].append(qmin)
        out["invC"].append(invC)
        out["N"].append(N)
    np.savez_compressed(os.path.join(HERE, "fisher_big.npz"), **{k: np.array(v) for k, v in out.items()})


def fisher_wavelet(ref, rng):
    """ucb_fisher_wavelet (ucb/src/glass_ucb_waveform.c:524) on the 64 x 256
    test grid of tests/test_wavelet_gpu.py (pixels of layers 10..39, time
    indices 4..251 counted), five sources of that band with a positive
    definite matrix (the reference regularises others)."""
    NF, NT, wdt, Tobs = 64, 256, 15.0 * 64, 2.0**14 * 15.0
    wdf = 1 / (2 * wdt)
    kmin, kmax = 10 * NT, 40 * NT
    imin, imax = 4, NT - 4
    invC = wl.wavelet_invC(kmax - kmin, NT, kmin, 1e-22)
    out = {"params": [], "F": []}
    while len(out["F"]) < 5:
        p = wl.draw_source(rng, rng.uniform(12 * wdf, 38 * wdf), 10 ** rng.uniform(-22, -21), 1e-14, Tobs)
        F, reg = ref.fisher_wavelet(p, Tobs, 0.0, NF, NT, wdt, wdf, kmin, kmax, imin, imax, invC)
        if reg:
            continue
        out["params"].append(p)
        out["F"].append(F)
    np.savez_compressed(os.path.join(HERE, "fisher_wavelet.npz"), grid=np.array([NF, NT, wdt, Tobs]),
                        kmin=kmin, kmax=kmax, imin=imin, imax=imax, **{k: np.array(v) for k, v in out.items()})


def priors(ref, rng):
    """draw_from_uniform_prior (utils/src/glass_sampler.c:96) for 64 chains,
    three draws each, and evaluate_ucb_prior (ucb/src/glass_ucb_prior.c:536)
    on 200 parameter sets (in range, out of range, NaN, wrapped longitude,
    polarisation and phase) with the uniform sky and with a sky histogram."""
    T = wl.T_YEAR
    q0 = 1000.0
    prior = np.array([[q0, q0 + 512.0], [-1.0, 1.0], [0.0, 2 * np.pi], [np.log(1e-24), np.log(1e-20)],
                      [-1.0, 1.0], [0.0, np.pi], [0.0, 2 * np.pi], [-10.0, 10.0]])
    logPV = np.log(prior[:, 1] - prior[:, 0])
    seeds0 = rng.integers(1, 2**31, 64).astype(np.uint32)
    draws, logQ, seeds = [], [], []
    s = seeds0.copy()
    for k in range(3):
        row_p, row_q = [], []
        for c in range(64):
            p, q, s[c] = ref.draw_uniform_prior(prior.reshape(-1), logPV, int(s[c]))
            row_p.append(p)
            row_q.append(q)
        draws.append(row_p), logQ.append(row_q), seeds.append(s.copy())
    params = np.column_stack([rng.uniform(q0 - 20, q0 + 532, 200), rng.uniform(-1.1, 1.1, 200),
                              rng.uniform(-7, 14, 200), rng.uniform(np.log(1e-25), np.log(1e-19), 200),
                              rng.uniform(-1.05, 1.05, 200), rng.uniform(-4, 7, 200), rng.uniform(-8, 15, 200),
                              rng.uniform(-11, 11, 200)])
    params[5, 3] = np.nan
    nphi, ncos = 16, 8
    skyhist = np.log(rng.uniform(0.5, 2.0, ncos * nphi) / (4 * np.pi))
    lp_u, p_u, lp_g, p_g = [], [], [], []
    for p in params:
        a, b = ref.ucb_prior(p, prior.reshape(-1), logPV)
        lp_u.append(a), p_u.append(b)
        a, b = ref.ucb_prior(p, prior.reshape(-1), logPV, skyhist, 2.0 / ncos, 2 * np.pi / nphi, nphi)
        lp_g.append(a), p_g.append(b)
    np.savez_compressed(os.path.join(HERE, "priors.npz"), prior=prior, logPV=logPV, seeds0=seeds0,
                        draws=np.array(draws), logQ=np.array(logQ), seeds=np.array(seeds), params=params,
                        logP_uniform=np.array(lp_u), params_uniform=np.array(p_u), skyhist=skyhist, nphi=nphi,
                        dcostheta=2.0 / ncos, dphi=2 * np.pi / nphi, logP_galaxy=np.array(lp_g),
                        params_galaxy=np.array(p_g))
    del T


def wdm(ref, rng):
    """WDM windows, forward and inverse transforms on small grids (the window
    exponent is the reference's fixed 6, A = 0), and the per-layer transform."""
    out = {}
    grids = [(32, 64), (48, 64), (16, 256), (1536, 8)]
    for NF, NT in grids:
        key = f"{NF}x{NT}"
        x = rng.standard_normal(NF * NT)
        out[f"win_{key}"] = ref.wdm_window(NF, NT)
        out[f"winv_{key}"] = ref.wdm_window(NF, NT, forward=False)
        out[f"x_{key}"] = x
        out[f"fwd_{key}"] = ref.wdm_forward(NF, NT, x)
        w = rng.standard_normal(NF * NT)
        out[f"w_{key}"] = w
        out[f"inv_{key}"] = ref.wdm_inverse(NF, NT, w)
    NF, NT, jmin, NL = 64, 32, 10, 3
    x = rng.standard_normal(NT * (NL + 1))
    out["layers_in"] = x
    out["layers_out"] = ref.wdm_by_layers(NF, NT, jmin, NL, x)
    np.savez_compressed(os.path.join(HERE, "wdm.npz"), grids=np.array(grids), **out)


WAVELET_GRIDS = {
    # name: (NF, NT, pixel duration, Tobs); 15 s samples, 1024 layers x 2048 pixels
    "nf1024": (1024, 2048, 15.0 * 1024, 2.0**21 * 15.0),
    # the reference's own grid (initialize_wavelet, utils/src/glass_wavelet.c:210): 5 s samples
    "nf1536": (1536, 4096, 7680.0, 4096 * 7680.0),
}


def wavelet_segment(rng, params, grid, below=3, above=3, cut=0):
    from oracle import Port

    NF, NT, wdt, T = WAVELET_GRIDS[grid]
    j, nl = Port().wavelet_layers(T, params, 1.0 / (2 * wdt))
    lmin, lmax = j - below + cut, j + nl + above
    return lmin * NT, lmax * NT


def wavelet_waveforms(ref, rng):
    """ucb_waveform_wavelet: the pixel list and the X, Y, Z values on it."""
    out = {"grid": [], "params": [], "t0": [], "kmin": [], "kmax": []}
    cases = []
    for k in range(8):
        f0 = 10 ** rng.uniform(np.log10(0.5e-3), np.log10(15e-3))
        fdot = 10 ** rng.uniform(-18, -16) * (-1 if k == 5 else 1)
        p = wl.draw_source(rng, f0, 10 ** rng.uniform(-23, -21), fdot)
        grid = "nf1536" if k in (2, 7) else "nf1024"
        t0 = 2.5e5 if k in (1, 7) else 0.0
        cut = 1 if k in (3, 6) else 0  # the segment starts above the signal's first layer
        cases.append((grid, p, t0, cut))
    for i, (grid, p, t0, cut) in enumerate(cases):
        NF, NT, wdt, T = WAVELET_GRIDS[grid]
        kmin, kmax = wavelet_segment(rng, p, grid, cut=cut)
        lst, xyz = ref.wavelet_waveform(p, T, t0, NF, NT, wdt, 1.0 / (2 * wdt), kmin, kmax)
        out["grid"].append(grid)
        out["params"].append(p)
        out["t0"].append(t0)
        out["kmin"].append(kmin)
        out["kmax"].append(kmax)
        out[f"list{i}"] = lst
        out[f"xyz{i}"] = xyz[:, lst]
    t, pos = ref.orbit_grid(WAVELET_GRIDS["nf1024"][3], 0.0)
    np.savez_compressed(os.path.join(HERE, "wavelet_waveform.npz"), orbit_t=t, orbit_pos=pos,
                        **{k: np.array(v) for k, v in out.items()})


def wavelet_likelihood(ref, rng):
    """Sparse-pixel delta logL (delta_log_likelihood), the full-segment logL
    (gaussian_log_likelhood_wavelet) and snr_wavelet on a segment holding an
    injected source plus white noise, for Gaussian jumps around it."""
    grid = "nf1024"
    NF, NT, wdt, T = WAVELET_GRIDS[grid]
    wdf = 1.0 / (2 * wdt)
    out = {}
    for c in range(2):
        f0 = rng.uniform(2e-3, 6e-3)
        inj = wl.draw_source(rng, f0, 10 ** rng.uniform(-21.7, -21.2), 1e-17)
        kmin, kmax = wavelet_segment(rng, inj, grid, below=2, above=2)
        N = kmax - kmin
        lst, h = ref.wavelet_waveform(inj, T, 0.0, NF, NT, wdt, wdf, kmin, kmax)
        # noise with covariance C per pixel, scaled to the injection
        scale = 0.5 * np.abs(h).max()
        invC_s = wl.wavelet_invC(N, NT, kmin, scale)
        L = np.linalg.cholesky(np.linalg.inv(invC_s.transpose(2, 0, 1)))
        d = h + np.einsum("kab,kb->ak", L, rng.standard_normal((N, 3)))
        props = np.vstack([inj[None], wl.gaussian_jumps(rng, inj, wl.jump_scales(inj, 20.0), 9)])
        dl, full, snr, lists = [], [], [], []
        for q, p in enumerate(props):
            ly, hy = ref.wavelet_waveform(p, T, 0.0, NF, NT, wdt, wdf, kmin, kmax)
            dl.append(ref.wavelet_delta_logl(d, invC_s, h, lst, hy, ly))
            imin, imax = 100, NT - 100
            full.append(ref.wavelet_logl_full(NT, kmin, imin, imax, d, hy, ly, invC_s))
            snr.append(ref.wavelet_snr(hy, ly, invC_s))
        out.update({f"c{c}_kmin": kmin, f"c{c}_kmax": kmax, f"c{c}_d": d, f"c{c}_scale": scale,
                    f"c{c}_inj": inj, f"c{c}_props": props, f"c{c}_dlogl": np.array(dl),
                    f"c{c}_logl_full": np.array(full), f"c{c}_snr": np.array(snr)})
    np.savez_compressed(os.path.join(HERE, "wavelet_likelihood.npz"), ncase=2, grid=grid, edge=100, **out)


def _fstat_segment(ref, rng, f0, amp, fdot, NFFT, fmt="sangria"):
    inj = wl.draw_source(rng, f0, amp, fdot)

    def wf(p):
        al = ref.alignment(T, NFFT, 0, p)
        h = ref.waveform(p, int(al[0]), T, fmt=fmt)
        return int(al[0]), h[3], h[4]

    qmin, dA, dE, iA, _ = wl.make_segment(rng, [inj], wf, NFFT=NFFT, T=T)
    il = np.empty((2, 2 * NFFT))
    il[0, 0::2], il[0, 1::2] = dA.real, dA.imag
    il[1, 0::2], il[1, 1::2] = dE.real, dE.imag
    return inj, qmin, il[0].copy(), il[1].copy(), iA


def fstat(ref, rng):
    """get_Fstat_logL on cells scattered over (and a little beyond) segments
    holding one injected source, and build_fstatistic_proposal on a short
    segment.  Cells whose filters miss the segment entirely are included: the
    reference returns logL = 0 there."""
    out = {}
    cases = [("sangria", 3.2e-3, 3e-22, 1e-17, 160), ("sangria", 0.8e-3, 2e-22, 1e-18, 120),
             ("sangria", 12e-3, 1e-22, 1e-15, 120), ("phase", 2.5e-3, 2e-22, 1e-17, 40),
             ("frequency", 6e-3, 2e-22, 1e-16, 40)]
    for c, (fmt, f0, amp, fdot, n) in enumerate(cases):
        inj, qmin, dA, dE, iA = _fstat_segment(ref, rng, f0, amp, fdot, 1024, fmt)
        f = (qmin + rng.uniform(-24, 1048, n)) / T
        fd = np.where(rng.random(n) < 0.5, 0.0, 10 ** rng.uniform(-18, -13, n))
        th = np.arccos(rng.uniform(-1, 1, n))
        ph = rng.uniform(0, 2 * np.pi, n)
        cells = np.stack([f, fd, th, ph], 1)
        # a few cells at the source and next to it
        src = np.array([inj[0] / T, inj[7] / T ** 2, np.arccos(inj[1]), inj[2]])
        near = src + np.array([[0, 0, 0, 0], [0.5 / T, 0, 0.05, -0.1], [-1.0 / T, 0, -0.1, 0.2], [0.0, 0, 0.3, 0.0]])
        cells = np.vstack([near, cells])
        out[f"c{c}_fmt"] = fmt
        out[f"c{c}_qmin"] = qmin
        out[f"c{c}_dA"], out[f"c{c}_dE"], out[f"c{c}_invCA"] = dA, dE, iA
        out[f"c{c}_cells"] = cells
        out[f"c{c}_out"] = ref.fstat_logl(T, 1024, qmin, dA, dE, iA, cells, fmt=fmt)
    # the proposal grid of one short segment
    inj, qmin, dA, dE, iA = _fstat_segment(ref, rng, 4e-3, 4e-22, 1e-17, 64)
    tensor, norm, maxp = ref.fstat_proposal(T, 64, qmin, dA, dE, iA, 4, 5)
    out.update(p_qmin=qmin, p_dA=dA, p_dE=dE, p_invCA=iA, p_n_theta=4, p_n_phi=5, p_tensor=tensor, p_norm=norm,
               p_maxp=maxp)
    np.savez_compressed(os.path.join(HERE, "fstat.npz"), ncase=len(cases), **out)


def noise(ref, rng):
    """The noise module's XYZ likelihood (instrument covariance, optionally
    plus the galactic foreground, inverse, my_noise_log_likelihood) for noise
    models around the starting point, on 1024-bin grids at 0.1 mHz, at 2 mHz
    (where the foreground dominates), across the acceleration-noise cutoff
    (10 mHz) and across the foreground's high-frequency cutoff (~20 mHz); data
    drawn from the starting point's covariance."""
    from oracle import Port

    port = Port()
    NF = 1024
    inst0, sgal0 = wl.default_noise_params(T)
    out = {}
    starts = [int(1e-4 * T), int(2e-3 * T), int(1e-2 * T) - 500, int(10 * math.exp(sgal0[1]) * T) - 500]
    for c, q in enumerate(starts):
        fmin = q / T
        X, Y, Z = wl.xyz_from_covariance(rng, port.noise_covariance(T, fmin, NF, inst0, sgal0))
        inst = inst0 * np.exp(rng.uniform(-0.3, 0.3, (12, 12)))
        sgal = sgal0 + rng.uniform(-0.2, 0.2, (12, 5))
        out[f"c{c}_qmin"] = q
        out[f"c{c}_X"], out[f"c{c}_Y"], out[f"c{c}_Z"] = X, Y, Z
        out[f"c{c}_inst"], out[f"c{c}_sgal"] = inst, sgal
        out[f"c{c}_logl_inst"] = ref.noise_logl(T, fmin, X, Y, Z, inst)
        out[f"c{c}_logl_gal"] = ref.noise_logl(T, fmin, X, Y, Z, inst, sgal)
    np.savez_compressed(os.path.join(HERE, "noise.npz"), ncase=len(starts), NFFT=NF, **out)


def noise_wavelet(ref, rng):
    """The noise module's coarse-grained wavelet-domain likelihood: instrument
    only, with the stationary foreground and with the modulated foreground
    (a smooth modulation cache of galaxy_modulation_cache_for_Q's shape), at
    Q = 1 (full resolution) and Q = 8, on 16 layers of a 1024 x 256 grid at
    0.3 mHz and across the 10 mHz acceleration cutoff; data drawn per layer
    from the starting model's covariance."""
    from oracle import Port

    port = Port()
    NF, NT = 1024, 256
    dt = 15.0 * NF
    df = 1.0 / (2 * dt)
    Nl = 16
    inst0, sgal0 = wl.default_noise_params(T)
    out = {}
    c = 0
    for band, lmin in enumerate((10, 300)):
        C6 = np.array([port.noise_covariance(T, (lmin + j) * df, 1, inst0, sgal0)[0] for j in range(Nl)]) / (NF * NT)
        X, Y, Z = wl.wavelet_noise_data(rng, C6, NT)
        out[f"b{band}_X"], out[f"b{band}_Y"], out[f"b{band}_Z"] = X, Y, Z
        inst = inst0 * np.exp(rng.uniform(-0.3, 0.3, (8, 12)))
        sgal = sgal0 + rng.uniform(-0.2, 0.2, (8, 5))
        for Q in (1, 8):
            mod = wl.galaxy_modulation_like(NT // Q, phase=0.3 * c)
            out[f"c{c}_lmin"], out[f"c{c}_Q"], out[f"c{c}_band"] = lmin, Q, band
            out[f"c{c}_inst"], out[f"c{c}_sgal"], out[f"c{c}_mod"] = inst, sgal, mod
            for mode in (0, 1, 2):
                out[f"c{c}_logl{mode}"], P = ref.noise_wavelet_logl(NF, NT, dt, df, lmin, Q, X, Y, Z, inst, sgal, mode,
                                                                    mod if mode == 2 else None)
            c += 1
    np.savez_compressed(os.path.join(HERE, "noise_wavelet.npz"), ncase=c, NF=NF, NT=NT, dt=dt, df=df, **out)


def sgwb(ref, rng):
    """The noise module's stochastic background (generate_sgwb_model, all three
    templates) with the synthetic response table of
    glass_gb300.workloads.sgwb_response_table (the reference reads its table
    from a file in the same layout): the covariance on a frequency grid; the
    XYZ likelihood with instrument + foreground + background for models around
    the starting point on 1024-bin grids at 0.1 and 2 mHz; the coarse wavelet
    likelihood (modes 0, 1, 2 with the background) at Q = 1 and 8."""
    from oracle import Port

    port = Port()
    resp = wl.sgwb_response_table()
    inst0, sgal0 = wl.default_noise_params(T)
    out = {"resp": resp}
    fgrid = np.exp(np.linspace(math.log(5e-5), math.log(0.05), 97))
    for t in range(3):
        params = wl.sgwb_params_draw(rng, t, 4)
        if t == 1:
            params[3, 2] = 0.98  # Delta = 10^0.98 >= 9: the asymptotic branch
        if t == 2:
            # b + 4 < m: the template's base goes negative at low frequency and
            # the reference gives NaN there
            params[0] = (1.2, 0.5, -18.0, -2.5)
        out[f"t{t}_params"] = params
        npar = len(wl.default_sgwb_params(t))
        out[f"t{t}_C"] = np.array([ref.sgwb_model(t, params[k, :npar], resp, fgrid) for k in range(4)])
    out["fgrid"] = fgrid
    # Fourier likelihood
    NF = 1024
    for c, q in enumerate((int(2e-3 * T), int(8e-3 * T))):
        fmin = q / T
        X, Y, Z = wl.xyz_from_covariance(rng, port.noise_covariance(T, fmin, NF, inst0, sgal0))
        out[f"c{c}_qmin"] = q
        out[f"c{c}_X"], out[f"c{c}_Y"], out[f"c{c}_Z"] = X, Y, Z
        inst = inst0 * np.exp(rng.uniform(-0.3, 0.3, (6, 12)))
        sgal = sgal0 + rng.uniform(-0.2, 0.2, (6, 5))
        out[f"c{c}_inst"], out[f"c{c}_sgal"] = inst, sgal
        for t in range(3):
            sg = wl.sgwb_params_draw(rng, t, 6)
            out[f"c{c}_t{t}_sgwb"] = sg
            out[f"c{c}_t{t}_logl"] = ref.noise_logl_sgwb(T, fmin, X, Y, Z, inst, sgal, t, sg, resp)
            out[f"c{c}_t{t}_logl_inst"] = ref.noise_logl_sgwb(T, fmin, X, Y, Z, inst, None, t, sg, resp)
    # wavelet likelihood
    NFw, NT = 1024, 256
    dt = 15.0 * NFw
    df = 1.0 / (2 * dt)
    Nl, lmin = 16, 60
    C6 = np.array([port.noise_covariance(T, (lmin + j) * df, 1, inst0, sgal0)[0] for j in range(Nl)]) / (NFw * NT)
    X, Y, Z = wl.wavelet_noise_data(rng, C6, NT)
    out["w_X"], out["w_Y"], out["w_Z"] = X, Y, Z
    inst = inst0 * np.exp(rng.uniform(-0.3, 0.3, (4, 12)))
    sgal = sgal0 + rng.uniform(-0.2, 0.2, (4, 5))
    out["w_inst"], out["w_sgal"] = inst, sgal
    for Q in (1, 8):
        mod = wl.galaxy_modulation_like(NT // Q, phase=0.2)
        out[f"w_Q{Q}_mod"] = mod
        for t in range(3):
            sg = wl.sgwb_params_draw(rng, t, 4)
            out[f"w_Q{Q}_t{t}_sgwb"] = sg
            for mode in (0, 1, 2):
                out[f"w_Q{Q}_t{t}_logl{mode}"] = ref.noise_wavelet_logl_sgwb(NFw, NT, dt, df, lmin, Q, X, Y, Z, inst,
                                                                            sgal, mode, mod if mode == 2 else None,
                                                                            t, sg, resp)
    np.savez_compressed(os.path.join(HERE, "sgwb.npz"), NFFT=NF, NF=NFw, NT=NT, dt=dt, df=df, lmin=lmin, Nl=Nl,
                        **out)


def noise_eta(ref, rng):
    """noise_model_mcmc's likelihood change (ucb/src/glass_ucb_sampler.c:29-73)
    for chains with one source on a config-0-like segment: small eta jumps as
    the sampler draws them (0.001) and larger ones."""
    out = {}
    for c in range(2):
        f0 = rng.uniform(3.0e-3, 3.5e-3)
        inj = wl.draw_source(rng, f0, 2e-22, 1e-17)

        def wf(p):
            al = ref.alignment(T, 1024, 0, p)
            h = ref.waveform(p, int(al[0]), T)
            return int(al[0]), h[3], h[4]

        qmin, dA, dE, iA, iE = wl.make_segment(rng, [inj], wf, NFFT=1024, T=T)
        iE = iE * rng.uniform(0.9, 1.1)  # the two channels' noise need not be equal
        il = np.empty((2, 2048))
        il[0, 0::2], il[0, 1::2] = dA.real, dA.imag
        il[1, 0::2], il[1, 1::2] = dE.real, dE.imag
        props = np.vstack([inj[None], wl.gaussian_jumps(rng, inj, wl.jump_scales(inj, 20.0), 15)])
        ex = rng.uniform(0.8, 1.25, (16, 2))
        ey = np.where(np.arange(16)[:, None] < 8, ex + 0.001 * rng.standard_normal((16, 2)),
                      ex * rng.uniform(0.5, 2.0, (16, 2)))
        eta = np.column_stack([ex, ey])
        out[f"c{c}_qmin"] = qmin
        out[f"c{c}_dA"], out[f"c{c}_dE"], out[f"c{c}_invCA"], out[f"c{c}_invCE"] = il[0], il[1], iA, iE
        out[f"c{c}_params"], out[f"c{c}_eta"] = props, eta
        out[f"c{c}_delta"] = ref.noise_eta(T, 1024, qmin, il[0].copy(), il[1].copy(), iA, iE, props, eta)
    np.savez_compressed(os.path.join(HERE, "noise_eta.npz"), ncase=2, **out)


def sampler(ref, rng):
    """ptmcmc (utils/src/glass_sampler.c:19) of 16 ladders of 12 chains with a
    geometric temperature ladder, 40 successive exchange sweeps each on fixed
    log-likelihoods: the permutation, acceptance and seeds after the first
    sweep and after the last."""
    NC, nens, sweeps = 12, 16, 40
    temperature = 1.3 ** np.arange(NC)
    logL = rng.normal(1000.0, 20.0, (nens, NC))
    logLn = rng.normal(-50.0, 5.0, (nens, NC))
    seed0 = rng.integers(1, 2**31, (nens, NC)).astype(np.uint32)
    idx1, acc1, s1 = [], [], []
    idxN, accN, sN = [], [], []
    for e in range(nens):
        index = np.arange(NC, dtype=np.int32)
        seed = seed0[e].copy()
        acc = np.zeros(NC)
        for k in range(sweeps):
            ref.ptmcmc(temperature, logL[e], index, seed, acc, logLn[e])
            if k == 0:
                idx1.append(index.copy()), acc1.append(acc.copy()), s1.append(seed.copy())
        idxN.append(index), accN.append(acc), sN.append(seed)
    np.savez_compressed(os.path.join(HERE, "sampler.npz"), NC=NC, sweeps=sweeps, temperature=temperature, logL=logL,
                        logLnorm=logLn, seed0=seed0, index1=np.array(idx1), acc1=np.array(acc1),
                        seed1=np.array(s1), indexN=np.array(idxN), accN=np.array(accN), seedN=np.array(sN))


def fisher_draw(ref, rng):
    """draw_from_fisher (ucb/src/glass_ucb_proposal.c:348) of 64 chains, four
    successive draws each from the same state: the drawn parameters, the
    return values and the seeds after every draw."""
    x, evec, evalue, seed0 = wl.fisher_draw_inputs(rng)
    seed = seed0.copy()
    ys, qs, ss = [], [], []
    for k in range(4):
        y, q = ref.fisher_draw(x, evec, evalue, seed)
        ys.append(y), qs.append(q), ss.append(seed.copy())
    np.savez_compressed(os.path.join(HERE, "fisher_draw.npz"), x=x, evec=evec, evalue=evalue, seed0=seed0,
                        y=np.array(ys), logQ=np.array(qs), seeds=np.array(ss))


def spline_noise(ref, rng):
    """The noise module's spline noise model (generate_spline_noise_model +
    noise_log_likelihood, one and two channels): models around a synthetic
    excess over the A/E noise PSD, at 2 mHz on 1000 bins (one channel, 24
    knots at most, 2-knot models among them), 4 mHz on 1024 bins (two
    channels, 24 knots), and 512 knots on 2048 bins (two channels, the
    kernel's largest knot count)."""
    out = {}
    for name, q, NFFT, nch, n, kmax, kmin in (("one", int(2e-3 * T), 1000, 1, 10, 24, 2),
                                             ("two", int(4e-3 * T), 1024, 2, 10, 24, 2),
                                             ("max", int(3e-3 * T), 2048, 2, 2, 512, 512)):
        tr, d, ex = wl.spline_noise_data(rng, T, q, NFFT, nch, excess=2.0)
        nk, kf, kC = wl.spline_noise_models(rng, T, q, NFFT, ex, n, kmax, kmin)
        if name == "one":
            nk[1] = 2  # the smallest model: a straight line
            kf[1, :] = 0.0
            kf[1, 0], kf[1, 1] = q / T - 0.5 / T, (q + NFFT) / T
            kC[1, :, 2:] = 0.0
        out[f"{name}_qmin"] = q
        out[f"{name}_transfer"], out[f"{name}_d"] = tr, d
        out[f"{name}_nknots"], out[f"{name}_knot_f"], out[f"{name}_knot_C"] = nk, kf, kC
        out[f"{name}_logl"] = ref.spline_noise_logl(T, q / T, d, tr, nk, kf, kC)
    np.savez_compressed(os.path.join(HERE, "spline_noise.npz"), **out)


def noise_channels(ref, rng):
    """The noise module's one- and two-channel instrument (+ foreground)
    models (generate_instrument_noise_model's case 1 and case 2,
    generate_galactic_foreground_model's case 1 and 2, noise_log_likelihood):
    Michelson X and A/E data drawn from the three-channel model's X and A/E
    covariance, at 0.1 mHz (acceleration noise on), 2 mHz and 12 mHz (above
    the acceleration cut), six models each around the starting point, with
    and without the foreground."""
    from oracle import Port

    port = Port()
    inst0, sgal0 = wl.default_noise_params(T)
    out = {}
    for c, (q, N) in enumerate(((int(1e-4 * T), 512), (int(2e-3 * T), 1000), (int(12e-3 * T), 512))):
        C6 = port.noise_covariance(T, q / T, N, inst0, sgal0)
        xx, yy, zz, xy, xz, yz = C6.T
        var = {1: [xx], 2: [(zz + xx - 2 * xz) / 2, (xx + 4 * yy + zz - 4 * xy + 2 * xz - 4 * yz) / 6]}
        for nch in (1, 2):
            d = np.empty((nch, 2 * N))
            for k in range(nch):
                sd = np.sqrt(0.5 * var[nch][k])
                d[k, 0::2] = rng.standard_normal(N) * sd
                d[k, 1::2] = rng.standard_normal(N) * sd
            inst = inst0 * np.exp(rng.uniform(-0.3, 0.3, (6, 12)))
            sgal = sgal0 + rng.uniform(-0.2, 0.2, (6, 5))
            key = f"c{c}_n{nch}"
            out[f"{key}_qmin"], out[f"{key}_d"], out[f"{key}_inst"], out[f"{key}_sgal"] = q, d, inst, sgal
            out[f"{key}_logl"] = ref.noise_logl_channels(T, q / T, d, inst, sgal)
            out[f"{key}_logl_inst"] = ref.noise_logl_channels(T, q / T, d, inst, None)
    np.savez_compressed(os.path.join(HERE, "noise_channels.npz"), **out)


def rj(ref, rng):
    """ucb_rjmcmc (ucb/src/glass_ucb_sampler.c:454), the birth/death step, run
    by the reference itself: 48 chains on one 256-bin A/E segment at 3.2 mHz
    with three injected sources, starting from 0 to 3 sources (injections
    and prior draws), six successive calls each, the reference's cocktail of
    the prior draw (rj weight 0.2) and the F-statistic draw (0.8) on a
    synthetic 64 x 10 x 10 density grid peaked at the injections, and
    temperatures 1.5^(c mod 12).  Recorded per call: the proposed state's
    logL when the reference evaluated it, a birth's new source and SNR, and
    logL, Nlive and the seed after the call; the final source lists."""
    NFFT, NC, maxsrc, nsteps = 256, 48, 6, 6
    injs = [wl.draw_source(rng, 3.2e-3 + k * 30 / T, 10 ** rng.uniform(-22.0, -21.3), 1e-17) for k in range(3)]

    def wf(p):
        al = ref.alignment(T, NFFT, 0, p)
        h = ref.waveform(p, int(al[0]), T)
        return int(al[0]), h[3], h[4]

    qmin, dA, dE, iA, iE = wl.make_segment(rng, injs, wf, NFFT=NFFT, T=T, center_f0=3.2e-3 + 30 / T)
    dA_i = np.empty(2 * NFFT)
    dA_i[0::2], dA_i[1::2] = dA.real, dA.imag
    dE_i = np.empty(2 * NFFT)
    dE_i[0::2], dE_i[1::2] = dE.real, dE.imag
    prior = np.array([[qmin, qmin + NFFT], [-1.0, 1.0], [0.0, 2 * np.pi], [np.log(1e-23), np.log(2e-21)],
                      [-1.0, 1.0], [0.0, np.pi], [0.0, 2 * np.pi], [-1.0, 1.0]])
    logPV = np.log(prior[:, 1] - prior[:, 0])
    nf, nt, npp = 64, 10, 10
    df, dt, dp = (NFFT / nf) / T, 2.0 / nt, 2 * np.pi / npp
    tensor = rng.uniform(0.5, 1.5, (nf, nt, npp))
    for p in injs:
        i = int((p[0] - qmin) / (df * T))
        j = int((p[1] + 1) / dt)
        k = int((p[2] % (2 * np.pi)) / dp)
        tensor[min(i, nf - 1), min(j, nt - 1), min(k, npp - 1)] += 200.0
    maxp = float(tensor.max())
    Nlive = rng.integers(0, 4, NC).astype(np.int32)
    Neff = np.full(NC, maxsrc, np.int32)
    Neff[::7] = Nlive[::7] + 1  # births refused on these chains
    src = np.zeros((NC, maxsrc, 8))
    for c in range(NC):
        for s in range(Nlive[c]):
            if s < 3 and rng.uniform() < 0.6:
                src[c, s] = wl.gaussian_jumps(rng, injs[s], wl.jump_scales(injs[s], 30.0), 1)[0]
            else:
                src[c, s] = prior[:, 0] + rng.uniform(0, 1, 8) * (prior[:, 1] - prior[:, 0])
    temperature = 1.5 ** (np.arange(NC) % 12)
    seed0 = rng.integers(1, 2**31, NC).astype(np.uint32)
    rjw = np.array([0.2, 0.8, 0, 0, 0, 0, 0, 0, 0])
    Nl, sr, sd = Nlive.copy(), src.copy(), seed0.copy()
    out = ref.rj_steps(T, NFFT, qmin, dA_i, dE_i, iA, iE, Neff, Nl, sr, prior, logPV, rjw,
                       (tensor, df, dt, dp, maxp), temperature, sd, nsteps)
    # a death's likelihood change: logL of the first eight chains' starting
    # models with and without their first source
    full, without = np.full(8, np.nan), np.full(8, np.nan)
    for c in range(8):
        if Nlive[c] > 0:
            full[c] = ref.log_likelihood(T, NFFT, qmin, dA_i, dE_i, iA, iE, src[c, :Nlive[c]])[0]
            without[c] = ref.log_likelihood(T, NFFT, qmin, dA_i, dE_i, iA, iE, src[c, 1:Nlive[c]])[0]
    out["death_full"], out["death_without"] = full, without
    np.savez_compressed(os.path.join(HERE, "rj.npz"), NFFT=NFFT, qmin=qmin, dA=dA_i, dE=dE_i, invCA=iA, invCE=iE,
                        prior=prior, logPV=logPV, tensor=tensor, df=df, dt=dt, dp=dp, maxp=maxp, Nlive0=Nlive,
                        Neff=Neff, src0=src, temperature=temperature, seed0=seed0, rjw=rjw, Nlive_end=Nl,
                        src_end=sr, seed_end=sd, **out)


OWN_SEEDS = {"fstat": 20261204, "noise": 20261205, "noise_wavelet": 20261206, "noise_eta": 20261207,
             "sampler": 20261208, "fisher_draw": 20261209, "fisher_big": 20261210,
             "fisher_wavelet": 20261211, "priors": 20261212, "sgwb": 20261213,
             "spline_noise": 20261214, "noise_channels": 20261215, "rj": 20261216}


def main(names=()):
    ref = Ref()
    if names:  # fixtures with a seed of their own can be regenerated alone
        for name in names:
            globals()[name](ref, np.random.default_rng(OWN_SEEDS[name]))
        return
    rng = np.random.default_rng(20261203)
    waveforms(ref, rng)
    bandwidth(ref, rng)
    likelihood(ref, rng)
    fisher(ref, rng)
    wdm(ref, rng)
    wavelet_waveforms(ref, rng)
    wavelet_likelihood(ref, rng)
    fstat(ref, np.random.default_rng(OWN_SEEDS["fstat"]))
    noise(ref, np.random.default_rng(OWN_SEEDS["noise"]))
    noise_wavelet(ref, np.random.default_rng(OWN_SEEDS["noise_wavelet"]))
    noise_eta(ref, np.random.default_rng(OWN_SEEDS["noise_eta"]))
    sampler(ref, np.random.default_rng(OWN_SEEDS["sampler"]))
    fisher_draw(ref, np.random.default_rng(OWN_SEEDS["fisher_draw"]))
    fisher_big(ref, np.random.default_rng(OWN_SEEDS["fisher_big"]))
    fisher_wavelet(ref, np.random.default_rng(OWN_SEEDS["fisher_wavelet"]))
    priors(ref, np.random.default_rng(OWN_SEEDS["priors"]))
    sgwb(ref, np.random.default_rng(OWN_SEEDS["sgwb"]))
    spline_noise(ref, np.random.default_rng(OWN_SEEDS["spline_noise"]))
    noise_channels(ref, np.random.default_rng(OWN_SEEDS["noise_channels"]))
    rj(ref, np.random.default_rng(OWN_SEEDS["rj"]))
    for name in sorted(os.listdir(HERE)):
        if name.endswith(".npz"):
            print(name, os.path.getsize(os.path.join(HERE, name)))


if __name__ == "__main__":
    main(sys.argv[1:])
