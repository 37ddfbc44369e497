"""The trans-dimensional (birth/death) step of ucb_rjmcmc: tests/golden/rj.npz
holds six successive calls of the reference's own ucb_rjmcmc on 48 chains
(prior and F-statistic draws, the reference's likelihood), with the proposed
state's logL and a birth's SNR recorded per call.  The oracle (CPU) and the
device kernels (gpu) replay the calls from the same seeds with those
likelihoods and must reproduce every new source, decision, seed and source
list; a GPU test checks the death's likelihood change from the engine's
term and (h|h) against the reference."""
import numpy as np
import pytest

from glass_gb300 import workloads as wl

T = wl.T_YEAR


def _grid(g):
    return (g["tensor"], float(g["df"]), float(g["dt"]), float(g["dp"]), float(g["maxp"]), int(g["qmin"]), T)


def _replay(g, propose, accept):
    """Replays the golden's calls through propose(Nlive, src, seed) ->
    (move, slot, kind, params_y, logQxy, logQyx, logPy) and
    accept(Nlive, src, proposal, dlogl, hh, seed, logL); checks each call."""
    Nlive = g["Nlive0"].astype(np.int32).copy()
    src = g["src0"].copy()
    seed = g["seed0"].astype(np.uint32).copy()
    logL = g["logL0"].copy()
    steps = g["rec_gen"].shape[0]
    for k in range(steps):
        prop = propose(Nlive, src, seed)
        move, y, lpy = prop[0], prop[3], prop[6]
        gen = (move > 0) & (lpy > -np.inf)
        np.testing.assert_array_equal(gen.astype(np.int32), g["rec_gen"][k], err_msg=f"call {k}: births generated")
        np.testing.assert_array_equal(y[gen], g["rec_params"][k][gen], err_msg=f"call {k}: new sources")
        ly = g["rec_logLy"][k]
        dlogl = np.where(np.isfinite(ly), ly - logL, 0.0)
        snr = g["rec_snr"][k]
        hh = np.where(np.isfinite(snr), snr * snr, 1e6)
        Nlive, src, seed, logL = accept(Nlive, src, prop, dlogl, hh, seed, logL)
        np.testing.assert_array_equal(Nlive, g["Nlive"][k], err_msg=f"call {k}: Nlive")
        np.testing.assert_array_equal(seed, g["seed"][k], err_msg=f"call {k}: seeds")
        np.testing.assert_allclose(logL, g["logL"][k], rtol=1e-12, atol=1e-9, err_msg=f"call {k}: logL")
    for c in range(len(Nlive)):
        n = Nlive[c]
        np.testing.assert_array_equal(src[c, :n], g["src_end"][c, :n], err_msg=f"chain {c}: sources")
    np.testing.assert_array_equal(seed, g["seed_end"])


def test_oracle_rj_matches_reference(golden, port):
    g = golden("rj.npz")
    grid = _grid(g)

    def propose(Nlive, src, seed):
        return port.rj_propose(Nlive, g["Neff"], src, g["prior"], g["logPV"], g["rjw"], grid, seed)

    def accept(Nlive, src, prop, dlogl, hh, seed, logL):
        move, slot, kind, y, qxy, qyx, lpy = prop
        port.rj_accept(Nlive, src, move, slot, y, qxy, qyx, lpy, g["temperature"], dlogl, hh, g["prior"],
                       g["logPV"], seed, logL)
        return Nlive, src, seed, logL

    _replay(g, propose, accept)


def test_rj_golden_covers_both_moves(golden):
    """The golden exercises births (generated, accepted and cut by SNR),
    deaths, refused births (Nlive + 1 = Neff) and deaths of empty models."""
    g = golden("rj.npz")
    before = np.vstack([g["Nlive0"][None], g["Nlive"][:-1]])
    up, down = (g["Nlive"] > before).sum(), (g["Nlive"] < before).sum()
    assert up >= 3 and down >= 3, (up, down)
    assert (g["rec_snr"][np.isfinite(g["rec_snr"])] < 5).any()
    assert (g["Neff"] == g["Nlive0"] + 1).any() and (g["Nlive0"] == 0).any()


@pytest.fixture(scope="module")
def engine():
    import glass_gb300 as gg
    from glass_gb300 import build

    build.build()
    eng = gg.Engine(0)
    yield eng
    eng.close()


@pytest.mark.gpu
def test_gpu_rj_matches_reference(engine, golden):
    torch = pytest.importorskip("torch")
    dev = torch.device("cuda", 0)
    g = golden("rj.npz")
    NC, maxsrc = g["src0"].shape[0], g["src0"].shape[1]
    tensor = torch.from_numpy(np.ascontiguousarray(g["tensor"])).to(dev)
    grid = engine.fstat_grid(tensor, float(g["df"]), float(g["dt"]), float(g["dp"]), float(g["maxp"]), int(g["qmin"]),
                             T)
    prior = torch.from_numpy(np.ascontiguousarray(g["prior"]).reshape(16)).to(dev)
    logPV = torch.from_numpy(np.ascontiguousarray(g["logPV"])).to(dev)
    Neff = torch.from_numpy(g["Neff"].astype(np.int32)).to(dev)
    temps = torch.from_numpy(g["temperature"]).to(dev)
    d = {}

    def propose(Nlive, src, seed):
        d["Nlive"] = torch.from_numpy(Nlive.astype(np.int32)).to(dev)
        d["src"] = torch.from_numpy(np.ascontiguousarray(src)).to(dev)
        d["seed"] = torch.from_numpy(seed.view(np.int32).copy()).to(dev)
        d["prop"] = engine.rj_propose_device(d["Nlive"], Neff, d["src"], prior, logPV, g["rjw"], grid, d["seed"])
        torch.cuda.synchronize()
        return tuple(x.cpu().numpy() for x in d["prop"][:7])

    def accept(Nlive, src, prop, dlogl, hh, seed, logL):
        lg = torch.from_numpy(logL.copy()).to(dev)
        engine.rj_accept_device(d["Nlive"], d["src"], d["prop"], temps, torch.from_numpy(dlogl).to(dev),
                                torch.from_numpy(hh).to(dev), prior, logPV, d["seed"], lg)
        torch.cuda.synchronize()
        return (d["Nlive"].cpu().numpy(), d["src"].cpu().numpy(), d["seed"].cpu().numpy().view(np.uint32),
                lg.cpu().numpy())

    _replay(g, propose, accept)
    # status: no chain hit the draw edge or the rejection limit
    assert int(d["prop"][7].abs().sum()) == 0
    assert NC == 48 and maxsrc == 6


@pytest.mark.gpu
def test_gpu_rj_death_change_from_term(engine, golden, port):
    """A death's likelihood change from the engine's term of the removed
    source against the chain's residual and its (h|h):
    -(term + hh) = logL(without it) - logL(with it), against the reference's
    logL of the first chains' starting models with and without their first
    source."""
    import glass_gb300 as gg

    g = golden("rj.npz")
    NFFT, qmin = int(g["NFFT"]), int(g["qmin"])
    dA, dE = g["dA"], g["dE"]
    checked = 0
    for c in range(8):
        n = int(g["Nlive0"][c])
        if n == 0:
            continue
        srcs = g["src0"][c, :n]
        rA, rE = dA.copy(), dE.copy()  # the chain's residual: the data minus its sources
        for p in srcs:
            N = int(port.alignment(T, NFFT, qmin, p)[0])
            h = port.waveform(p, N, T)
            i0 = int(p[0]) - N // 2 - qmin
            for r, hc in ((rA, h[3]), (rE, h[4])):
                for m in range(N):
                    j = i0 + m
                    if 0 <= j < NFFT:
                        r[2 * j] -= hc[2 * m]
                        r[2 * j + 1] -= hc[2 * m + 1]
        bank = wl.SegmentBank(T=T, NFFT=NFFT, qmin=np.array([qmin], np.int32),
                              dA=(rA[0::2] + 1j * rA[1::2])[None], dE=(rE[0::2] + 1j * rE[1::2])[None],
                              invCA=g["invCA"][None].copy(), invCE=g["invCE"][None].copy())
        engine.upload(bank)
        term, _, hh, st = engine.dlogl_host(np.zeros(1, np.int32), srcs[:1], precision=gg.PREC_FP64)
        assert st[0] == 0
        want = g["death_without"][c] - g["death_full"][c]
        assert abs(-(term[0] + hh[0]) - want) <= 1e-8 * max(1.0, abs(g["death_full"][c])), (c, term, hh, want)
        checked += 1
    assert checked >= 3
