"""Calibration of the mixed-precision error estimate.

    python -m glass_gb300.error_study [--batches 10] [--out error_study.npz]

The mixed-precision delta logL lists for double-float re-evaluation every
proposal whose estimate

    Ka sqrt(hw_full rr / N) + Ks |(h|r - h)|

exceeds the tolerance (hw, rr: the whitened |h|^2 and |r - h|^2 over the
template's support; hw_full: hw scaled to the whole template when the segment
edge clips it; N: the template size).  This script measures the two constants
on three workloads: the 64-segment parallel-tempering benchmark (3072
proposals a batch), loud sources (amplitudes 1e-22..1e-21) with proposals
around them and louder copies far from the data, and the 1e4-source
global-fit population (512 segments of 8192 bins, N up to 4096, births and
updates).  Each proposal is evaluated in FP64 and in mixed precision with the
re-evaluation off; the sums of the estimate come from the FP64 template
(ucb_waveform on the GPU) and the bank.  Printed per workload and template
size: the largest error over the random predictor after the systematic part
(Ks_fit |(h|r - h)|) is taken off, and, for the constants in use, the
proposals listed per 3072 and the largest error / estimate where the error
exceeds 1e-4.
"""
from __future__ import annotations

import argparse
import math

import numpy as np

KA, KS = 9e-7, 2e-7  # the constants the engine uses (glass_gb300/csrc/capi.cu)
KS_FIT = 1.5e-7


def _features(gg, wl, bank, seg, params, d64, dmx, status, nmax=4096):
    """Per proposal: N, hw, rr, in-segment bins, |error|, |(h|r - h)|, hw_full."""
    T = bank.T
    rows = []
    for i in range(len(seg)):
        p, s = params[i], seg[i]
        N = 2 * gg.ucb_bandwidth(wl.LARM, wl.FSTAR, p[0] / T, p[7] / T / T, p[1], math.exp(p[3]), T, bank.NFFT)
        if status[i] != 0 or N > nmax or not (np.isfinite(d64[i]) and np.isfinite(dmx[i])):
            continue
        h = gg.ucb_waveform(p, N, T)
        hA, hE = h[3][0::2] + 1j * h[3][1::2], h[4][0::2] + 1j * h[4][1::2]
        i0 = int(p[0]) - N // 2 - int(bank.qmin[s])
        lo, hi = max(0, i0), min(bank.NFFT, i0 + N)
        if hi <= lo:
            continue
        wA, wE = np.sqrt(bank.invCA[s, lo:hi]), np.sqrt(bank.invCE[s, lo:hi])
        ha, he = hA[lo - i0:hi - i0] * wA, hE[lo - i0:hi - i0] * wE
        ea, eb = bank.dA[s, lo:hi] * wA - ha, bank.dE[s, lo:hi] * wE - he
        hw = np.sum(abs(ha) ** 2 + abs(he) ** 2)
        rr = np.sum(abs(ea) ** 2 + abs(eb) ** 2)
        hr = abs(np.sum(np.conj(ha) * ea + np.conj(he) * eb))
        pall = np.sum(abs(hA) ** 2 + abs(hE) ** 2)
        pseg = np.sum(abs(hA[lo - i0:hi - i0]) ** 2 + abs(hE[lo - i0:hi - i0]) ** 2)
        rows.append((N, hw, rr, hi - lo, abs(dmx[i] - d64[i]), hr, hw * pall / max(pseg, 1e-300)))
    return np.array(rows)


def _run(gg, wl, eng, bank, seg, batches, txs):
    out = []
    for b in range(len(batches)):
        tx = None if txs is None else txs[b]
        d, _, _, st = eng.dlogl_host(seg, batches[b], term_x=tx, precision=gg.PREC_FP64)
        eng.set_mixed_tolerance(0.0)
        dm, _, _, stm = eng.dlogl_host(seg, batches[b], term_x=tx, precision=gg.PREC_MIXED)
        eng.set_mixed_tolerance(1e-3)
        out.append(_features(gg, wl, bank, seg, batches[b], d, dm, st | stm))
    return np.concatenate(out)


def study(nb: int = 10, seed: int = 7) -> dict:
    import glass_gb300 as gg
    from . import workloads as wl

    T = wl.T_YEAR

    def wf_rule(NFFT, cap=4096):
        def wf(p):
            N = min(cap, 2 * gg.ucb_bandwidth(wl.LARM, wl.FSTAR, p[0] / T, p[7] / T / T, p[1], math.exp(p[3]), T,
                                              NFFT))
            h = gg.ucb_waveform(p, N, T)
            return N, h[3], h[4]

        return wf

    res = {}
    rng = np.random.default_rng(seed)
    # 1. the benchmark workload
    bank, inj, _, item_seg, temps = wl.tempered_bank(rng, wf_rule(1024))
    eng = gg.Engine(0)
    try:
        eng.upload(bank)
        _, t_inj, hh, _ = eng.dlogl_host(np.arange(len(inj), dtype=np.int32), inj, precision=gg.PREC_FP64)
        batches = wl.tempered_proposals(rng, inj, np.sqrt(np.maximum(hh, 1.0)), item_seg, temps, nb)
        res["benchmark"] = _run(gg, wl, eng, bank, item_seg, batches, [t_inj[item_seg]] * nb)
    finally:
        eng.close()
    # 2. loud sources: jumps around them at 12 temperatures, and copies x3..x30
    # louder moved by 0..40 bins (where the FP32 error is largest)
    bank, inj, _, _, _ = wl.tempered_bank(rng, wf_rule(1024), log10_amp_range=(-22.0, -21.0))
    eng = gg.Engine(0)
    try:
        eng.upload(bank)
        seg, batches = [], []
        for s in range(len(inj)):
            seg += [s] * 21
        seg = np.array(seg, np.int32)
        for _ in range(nb):
            ps = []
            for s in range(len(inj)):
                for k in range(12):
                    ps.append(wl.gaussian_jumps(rng, inj[s], wl.jump_scales(inj[s], 20.0) * 1.5 ** (k / 2), 1)[0])
                for fa in (3.0, 10.0, 30.0):
                    for df in (0.0, 2.0, 40.0):
                        p = inj[s].copy()
                        p[3] += math.log(fa)
                        p[0] += df
                        ps.append(p)
            batches.append(np.array(ps))
        res["loud"] = _run(gg, wl, eng, bank, seg, batches, None)
    finally:
        eng.close()
    # 3. the global-fit population
    bank, src, seg_of = wl.global_fit_bank(rng, wf_rule(8192))
    eng = gg.Engine(0)
    try:
        eng.upload(bank)
        _, t_src, hh, _ = eng.dlogl_host(seg_of, src, precision=gg.PREC_FP64)
        batches, birth = wl.global_fit_proposals(rng, bank, src, seg_of, np.sqrt(np.maximum(hh, 1.0)), nb)
        res["global_fit"] = _run(gg, wl, eng, bank, seg_of, batches, np.where(birth, 0.0, t_src[None, :]))
    finally:
        eng.close()
    return res


def report(res: dict, ka: float = KA, ks: float = KS) -> None:
    for name, v in res.items():
        N, hw, rr, nb, err, hr, hf = v.T
        rnd = np.sqrt(hf * rr / N)
        print(f"{name}: {len(v)} proposals, {int((err > 1e-3).sum())} with |error| > 1e-3")
        for n in np.unique(N):
            m = N == n
            # where |error| > 1e-6: below that the FP64 reference's own rounding
            # (~1e-12 absolute) makes the ratio meaningless for tiny templates
            mm = m & (err > 1e-6)
            r = np.maximum(err[mm] - KS_FIT * hr[mm], 0.0) / rnd[mm]
            print(f"  N = {int(n):5d}: {int(m.sum()):6d} proposals, (|error| - {KS_FIT:.1e} |(h|r-h)|) / "
                  f"sqrt(hw_full rr / N) <= {r.max() if r.size else 0.0:.2e} where |error| > 1e-6")
        est = ka * rnd + ks * hr
        big = err > 1e-4
        print(f"  Ka {ka:.1e}, Ks {ks:.1e}: listed {np.mean(est > 1e-3) * 3072:.1f} per 3072, "
              f"missed {int(((err > 1e-3) & (est <= 1e-3)).sum())}, "
              f"max |error| / estimate where |error| > 1e-4: {(err[big] / est[big]).max() if big.any() else 0:.2f}")


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--batches", type=int, default=10)
    ap.add_argument("--out", default=None)
    args = ap.parse_args()
    res = study(args.batches)
    report(res)
    if args.out:
        np.savez_compressed(args.out, **res)


if __name__ == "__main__":
    main()
