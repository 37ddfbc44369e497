"""Parity of the CUDA wavelet-domain UCB waveform and sparse-pixel likelihood
with the reference (golden vectors) and the oracle, through the C ABI.

FP64 tolerances: waveform values within 1e-10 of the channel's largest value
(they agree to the FFTs' rounding, ~1e-14), pixel lists identical; delta logL
within 1e-10 relative to max(1, |delta logL|).

Mixed precision (FP64 phase, FP32 amplitude, FFTs and products, double-float
sums) against FP64: waveform values within 1e-5 of the channel's largest
value; delta logL within 1e-3 absolute for every source at the default
tolerance (sources whose error estimate exceeds it are evaluated again in
FP64), and without the re-evaluation within 1e-3 where |delta logL| is small
and 1e-5 of |delta logL| elsewhere; <h|h> within 1e-5 relative.
"""
import numpy as np
import pytest

import glass_gb300 as gg
from glass_gb300 import workloads as wl

pytestmark = pytest.mark.gpu
REL = 1e-10
MIXED_ABS = 1e-3
MIXED_REL_FAR = 1e-5
GRIDS = {"nf1024": (1024, 2048, 15.0 * 1024, 2.0**21 * 15.0), "nf1536": (1536, 4096, 7680.0, 4096 * 7680.0)}
SMALL = (64, 256, 15.0 * 64, 2.0**14 * 15.0)  # NF, NT, pixel duration, Tobs


@pytest.fixture(scope="module")
def engine():
    from glass_gb300 import build

    build.build()
    eng = gg.Engine(0)
    yield eng
    eng.close()


def setup_grid(engine, grid, t0, kmin, kmax):
    NF, NT, wdt, Tobs = grid
    engine.wavelet_setup(Tobs, t0, NF, NT, wdt, 1 / (2 * wdt), kmin, kmax)


def compact(engine, info, xyz):
    lst = engine.wavelet_list(info)
    return lst, xyz[:, : len(lst)]


def test_waveform_matches_reference(engine, golden):
    g = golden("wavelet_waveform.npz")
    for i in range(len(g["grid"])):
        grid = GRIDS[str(g["grid"][i])]
        setup_grid(engine, grid, float(g["t0"][i]), int(g["kmin"][i]), int(g["kmax"][i]))
        info, xyz, st = engine.wavelet_waveform_host(g["params"][i][None])
        assert st[0] == 0
        lst, vals = compact(engine, info[0], xyz[0])
        np.testing.assert_array_equal(lst, g[f"list{i}"])
        ref = g[f"xyz{i}"]
        for c in range(3):
            err = np.abs(vals[c] - ref[c]).max() / np.abs(ref[c]).max()
            assert err < REL, (i, c, err)


def test_sparse_likelihood_matches_reference(engine, golden):
    """delta_log_likelihood(model with the injection -> model with each proposal)
    and snr_wavelet, on the data of the golden segment."""
    g = golden("wavelet_likelihood.npz")
    NF, NT, wdt, Tobs = GRIDS[str(g["grid"])]
    for c in range(int(g["ncase"])):
        kmin, kmax = int(g[f"c{c}_kmin"]), int(g[f"c{c}_kmax"])
        setup_grid(engine, (NF, NT, wdt, Tobs), 0.0, kmin, kmax)
        invC = wl.wavelet_invC(kmax - kmin, NT, kmin, float(g[f"c{c}_scale"]))
        engine.wavelet_set_data(g[f"c{c}_d"], invC)
        _, tx, _, st = engine.wavelet_dlogl_host(g[f"c{c}_inj"][None])
        assert st[0] == 0
        props = g[f"c{c}_props"]
        dl, ty, hh, st = engine.wavelet_dlogl_host(props, term_x=np.full(len(props), tx[0]))
        assert (st == 0).all()
        ref = g[f"c{c}_dlogl"]
        err = np.abs(dl - ref) / np.maximum(1.0, np.abs(ref))
        assert err.max() < REL, err
        np.testing.assert_allclose(np.sqrt(hh), g[f"c{c}_snr"], rtol=REL)


def test_batch_matches_oracle_small_grid(engine, port):
    """Many sources at once (different layer counts, segments that cut the
    signal, t0 != 0) on a small grid, against the oracle."""
    NF, NT, wdt, Tobs = SMALL
    wdf = 1 / (2 * wdt)
    rng = np.random.default_rng(21)
    for t0 in (0.0, 3.3e4):
        lmin, lmax = 10, 40
        kmin, kmax = lmin * NT, lmax * NT
        engine.wavelet_setup(Tobs, t0, NF, NT, wdt, wdf, kmin, kmax)
        n = 40
        f0 = rng.uniform((lmin - 1) * wdf, (lmax + 1) * wdf, n)
        params = np.array([wl.draw_source(rng, f, 10 ** rng.uniform(-22, -21), 10 ** rng.uniform(-15, -13), Tobs)
                           for f in f0])
        params[::7, 7] *= -1  # frequency decreasing
        info, xyz, st = engine.wavelet_waveform_host(params)
        assert (st == 0).all()
        for i in range(n):
            lst_o, xyz_o, j, nl = port.wavelet_waveform(params[i], Tobs, t0, NF, NT, wdt, wdf, kmin, kmax)
            assert (info[i, 0], info[i, 1]) == (j, nl)
            lst, vals = compact(engine, info[i], xyz[i])
            np.testing.assert_array_equal(lst, lst_o)
            if len(lst):
                ref = xyz_o[:, lst]
                assert np.abs(vals - ref).max() <= REL * np.abs(ref).max(), i


def test_dlogl_matches_oracle_and_edge_cases(engine, port):
    NF, NT, wdt, Tobs = SMALL
    wdf = 1 / (2 * wdt)
    kmin, kmax = 10 * NT, 40 * NT
    N = kmax - kmin
    engine.wavelet_setup(Tobs, 0.0, NF, NT, wdt, wdf, kmin, kmax)
    rng = np.random.default_rng(5)
    invC = wl.wavelet_invC(N, NT, kmin, 1e-22)
    d = rng.standard_normal((3, N)) * 1e-22
    engine.wavelet_set_data(d, invC)
    f0 = rng.uniform(9 * wdf, 41 * wdf, 30)
    params = np.array([wl.draw_source(rng, f, 10 ** rng.uniform(-22, -21), 1e-14, Tobs) for f in f0])
    params[3, 1] = 1.5  # invalid cos(theta)
    params[4, 0] = np.nan
    params[5, 0] = 2 * wdf * Tobs  # far below the segment
    dl, ty, hh, st = engine.wavelet_dlogl_host(params)
    assert st[3] == 1 and st[4] == 1 and np.isnan(dl[3]) and np.isnan(dl[4])
    assert st[5] == 4 and ty[5] == 0.0
    for i in np.where(st == 0)[0]:
        lst, h, _, _ = port.wavelet_waveform(params[i], Tobs, 0.0, NF, NT, wdt, wdf, kmin, kmax)
        dh, hh_o = port.wavelet_dh_hh(d, h, invC, lst)
        term = hh_o - 2 * dh
        assert abs(ty[i] - term) <= REL * max(1.0, abs(term)), i
        assert abs(hh[i] - hh_o) <= REL * hh_o


def test_given_orbit_arrays_are_used(engine, port):
    """Orbit node arrays passed by the caller (struct Orbit's t, x, y, z) give
    the same waveform as the built-in interpolated analytic orbit when they hold
    the same nodes."""
    NF, NT, wdt, Tobs = SMALL
    wdf = 1 / (2 * wdt)
    kmin, kmax = 10 * NT, 40 * NT
    t, pos = port.orbit_grid(Tobs, 0.0)
    rng = np.random.default_rng(9)
    p = wl.draw_source(rng, 20 * wdf, 1e-21, 1e-14, Tobs)
    engine.wavelet_setup(Tobs, 0.0, NF, NT, wdt, wdf, kmin, kmax)
    a = engine.wavelet_waveform_host(p[None])
    engine.wavelet_setup(Tobs, 0.0, NF, NT, wdt, wdf, kmin, kmax, orbit=(t, pos))
    b = engine.wavelet_waveform_host(p[None])
    np.testing.assert_array_equal(a[0], b[0])
    np.testing.assert_array_equal(a[1], b[1])


def test_mixed_waveform_close_to_fp64(engine, golden):
    g = golden("wavelet_likelihood.npz")
    NF, NT, wdt, Tobs = GRIDS[str(g["grid"])]
    kmin, kmax = int(g["c0_kmin"]), int(g["c0_kmax"])
    setup_grid(engine, (NF, NT, wdt, Tobs), 0.0, kmin, kmax)
    invC = wl.wavelet_invC(kmax - kmin, NT, kmin, float(g["c0_scale"]))
    props = g["c0_props"]
    with pytest.raises(gg.GlassError):  # mixed precision needs the data's noise level
        engine.wavelet_waveform_host(props, precision=gg.PREC_MIXED)
    engine.wavelet_set_data(g["c0_d"], invC)
    i64, x64, s64 = engine.wavelet_waveform_host(props)
    i32, x32, s32 = engine.wavelet_waveform_host(props, precision=gg.PREC_MIXED)
    assert (s64 == 0).all() and (s32 == 0).all()
    np.testing.assert_array_equal(i32, i64)
    for i in range(len(props)):
        lst = engine.wavelet_list(i64[i])
        for c in range(3):
            ref = x64[i, c, : len(lst)]
            assert np.abs(x32[i, c, : len(lst)] - ref).max() < 1e-5 * np.abs(ref).max(), (i, c)


def test_mixed_dlogl_error_budget(engine, golden):
    """Golden segments (noise + one injection) with their proposals, plus wider
    jumps from the injection: near the injection the error is absolute, far
    from it relative."""
    g = golden("wavelet_likelihood.npz")
    NF, NT, wdt, Tobs = GRIDS[str(g["grid"])]
    rng = np.random.default_rng(17)
    for c in range(int(g["ncase"])):
        kmin, kmax = int(g[f"c{c}_kmin"]), int(g[f"c{c}_kmax"])
        setup_grid(engine, (NF, NT, wdt, Tobs), 0.0, kmin, kmax)
        invC = wl.wavelet_invC(kmax - kmin, NT, kmin, float(g[f"c{c}_scale"]))
        engine.wavelet_set_data(g[f"c{c}_d"], invC)
        inj = g[f"c{c}_inj"]
        _, tx, hh0, _ = engine.wavelet_dlogl_host(inj[None])
        scales = wl.jump_scales(inj, float(np.sqrt(hh0[0])))
        wide = np.array([wl.gaussian_jumps(rng, inj, scales * f, 1)[0] for f in np.geomspace(0.3, 30, 40)])
        props = np.concatenate([g[f"c{c}_props"], wide])
        txs = np.full(len(props), tx[0])
        dl64, _, hh64, s64 = engine.wavelet_dlogl_host(props, term_x=txs)
        engine.set_mixed_tolerance(0.0)  # the mixed values alone
        dl32, _, hh32, s32 = engine.wavelet_dlogl_host(props, term_x=txs, precision=gg.PREC_MIXED)
        engine.set_mixed_tolerance(1e-3)
        np.testing.assert_array_equal(s32, s64)
        ok = s64 == 0
        assert ok.sum() >= len(g[f"c{c}_props"])
        err = np.abs(dl32 - dl64)[ok]
        ref = np.abs(dl64[ok])
        near = ref < 100.0
        assert (err[near] < MIXED_ABS).all(), err[near].max()
        assert (err[~near] < MIXED_REL_FAR * ref[~near]).all()
        np.testing.assert_allclose(hh32[ok], hh64[ok], rtol=MIXED_REL_FAR)
        # at the default tolerance: every source within 1e-3
        dlt, _, _, st = engine.wavelet_dlogl_host(props, term_x=txs, precision=gg.PREC_MIXED)
        np.testing.assert_array_equal(st, s64)
        assert (np.abs(dlt - dl64)[ok] < MIXED_ABS).all(), np.abs(dlt - dl64)[ok].max()


def test_mixed_tolerance_loud_templates(engine, golden):
    """Loud templates against data that do not contain them (the injection
    made 30 to 3000 times louder and moved in frequency by up to two layers):
    the mixed values alone miss 1e-3, the default tolerance's
    FP64 re-evaluation brings every source within it, and the re-evaluated
    sources are counted."""
    g = golden("wavelet_likelihood.npz")
    NF, NT, wdt, Tobs = GRIDS[str(g["grid"])]
    kmin, kmax = int(g["c0_kmin"]), int(g["c0_kmax"])
    setup_grid(engine, (NF, NT, wdt, Tobs), 0.0, kmin, kmax)
    engine.wavelet_set_data(g["c0_d"], wl.wavelet_invC(kmax - kmin, NT, kmin, float(g["c0_scale"])))
    inj = g["c0_inj"]
    props = []
    for fa in (30.0, 300.0, 3000.0):
        for df in (0.0, 0.5, 1.0, 2.0):
            p = inj.copy()
            p[3] += np.log(fa)
            p[0] += df * 0.5 * NT  # bins of 1/Tobs: half a layer per NT/2
            props.append(p)
    props = np.array(props)
    dl64, _, _, s64 = engine.wavelet_dlogl_host(props)
    ok = s64 == 0
    assert ok.sum() >= 8
    engine.set_mixed_tolerance(0.0)
    raw, _, _, _ = engine.wavelet_dlogl_host(props, precision=gg.PREC_MIXED)
    engine.set_mixed_tolerance(1e-3)
    assert (np.abs(raw - dl64)[ok] > MIXED_ABS).any()
    n0 = engine.wavelet_reevaluated()
    dlt, _, _, st = engine.wavelet_dlogl_host(props, precision=gg.PREC_MIXED)
    np.testing.assert_array_equal(st, s64)
    assert (np.abs(dlt - dl64)[ok] < MIXED_ABS).all(), np.abs(dlt - dl64)[ok].max()
    assert engine.wavelet_reevaluated() - n0 >= int((np.abs(raw - dl64)[ok] > MIXED_ABS).sum())


def _fisher_oracle(port, p, grid, t0, kmin, kmax, invC, imin, imax):
    """ucb_fisher_wavelet (ucb/src/glass_ucb_waveform.c:524-640) restated on
    the oracle's wavelet waveforms: central differences of step 1e-6 on the +
    waveform's pixels with imin < t < imax, nine XYZ cross terms of invC."""
    NF, NT, wdt, Tobs = grid
    wdf = 1 / (2 * wdt)
    N = kmax - kmin
    eps = 1e-6
    dh = np.zeros((8, 3, N))
    for i in range(8):
        pp, pm = p.copy(), p.copy()
        pp[i] += eps / 2
        pm[i] -= eps / 2
        if i in (1, 4):
            pp[i] = min(pp[i], 1.0)
            pm[i] = max(pm[i], -1.0)
        lp, xp, _, _ = port.wavelet_waveform(pp, Tobs, t0, NF, NT, wdt, wdf, kmin, kmax)
        _, xm, _, _ = port.wavelet_waveform(pm, Tobs, t0, NF, NT, wdt, wdf, kmin, kmax)
        for k in lp:
            t = (k + kmin) % NT
            if imin < t < imax and 0 <= k < N:
                dh[i][:, k] = (xp[:, k] - xm[:, k]) * (1.0 / eps)
    return np.einsum("iak,abk,jbk->ij", dh, invC, dh)


def test_fisher_batch_matches_restated_reference(engine, port):
    NF, NT, wdt, Tobs = SMALL
    wdf = 1 / (2 * wdt)
    kmin, kmax = 10 * NT, 40 * NT
    N = kmax - kmin
    imin, imax = 4, NT - 4
    engine.wavelet_setup(Tobs, 0.0, NF, NT, wdt, wdf, kmin, kmax)
    rng = np.random.default_rng(33)
    invC = wl.wavelet_invC(N, NT, kmin, 1e-22)
    engine.wavelet_set_data(np.zeros((3, N)), invC)
    params = np.array([wl.draw_source(rng, f, 10 ** rng.uniform(-22, -21), 1e-14, Tobs)
                       for f in rng.uniform(12 * wdf, 38 * wdf, 5)])
    params[2, 1] = 1.0 - 2e-7  # the + step of cos(theta) is clamped at 1
    params[3, 4] = -1.0 + 1e-7  # the - step of cos(iota) is clamped at -1
    bad = params[0].copy()
    bad[4] = 1.5
    F, st = engine.wavelet_fisher_host(np.vstack([params, bad[None]]), imin, imax)
    assert (st[:-1] == 0).all() and st[-1] != 0 and np.isnan(F[-1]).all()
    for s in range(len(params)):
        ref = _fisher_oracle(port, params[s], SMALL, 0.0, kmin, kmax, invC, imin, imax)
        scale = np.sqrt(np.outer(np.diag(ref), np.diag(ref)))
        np.testing.assert_array_equal(F[s], F[s].T)
        assert (np.abs(F[s] - ref) <= 1e-6 * scale + 1e-300).all(), (s, (np.abs(F[s] - ref) / scale).max())


def test_fisher_batch_matches_reference_ucb_fisher_wavelet(engine, golden):
    """The reference's own ucb_fisher_wavelet (central differences of its
    wavelet waveform, ucb/src/glass_ucb_waveform.c:524-640) on the same grid:
    golden matrices from its sources (tests/golden/fisher_wavelet.npz)."""
    g = golden("fisher_wavelet.npz")
    NF, NT, wdt, Tobs = (float(x) for x in g["grid"])
    NF, NT = int(NF), int(NT)
    kmin, kmax, imin, imax = int(g["kmin"]), int(g["kmax"]), int(g["imin"]), int(g["imax"])
    engine.wavelet_setup(Tobs, 0.0, NF, NT, wdt, 1 / (2 * wdt), kmin, kmax)
    invC = wl.wavelet_invC(kmax - kmin, NT, kmin, 1e-22)
    engine.wavelet_set_data(np.zeros((3, kmax - kmin)), invC)
    F, st = engine.wavelet_fisher_host(g["params"], imin, imax)
    assert (st == 0).all()
    for s in range(len(g["params"])):
        ref = g["F"][s]
        scale = np.sqrt(np.outer(np.diag(ref), np.diag(ref)))
        err = np.abs(F[s] - ref) / scale
        assert err.max() < 1e-6, (s, err.max(), np.unravel_index(err.argmax(), err.shape))
