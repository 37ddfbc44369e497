"""The on-device sampler kernels against the C library's rand_r, the
reference's ptmcmc (golden vectors) and the oracle's restatement of
ucb_mcmc's accept/reject tail, bit for bit: same seeds in, same decisions,
states and seeds out."""
import numpy as np
import pytest

import glass_gb300 as gg

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def engine():
    from glass_gb300 import build

    build.build()
    eng = gg.Engine(0)
    yield eng
    eng.close()


def _u32(a):
    return np.ascontiguousarray(a, np.uint32).view(np.int32)


def test_rand_r_stream_matches_c_library(engine, port):
    import torch

    rng = np.random.default_rng(31)
    seeds = np.concatenate([[0, 1, 12345, 2**31 - 1, 2**32 - 1], rng.integers(0, 2**32, 995, dtype=np.uint64)])
    seeds = seeds.astype(np.uint32)
    ref, ref_next = port.rand_r_seq(seeds, 64)
    ds = torch.tensor(_u32(seeds), device="cuda")
    out = torch.empty((len(seeds), 64), dtype=torch.int32, device="cuda")
    torch.cuda.synchronize()
    engine.rand_r_fill_device(ds, out)
    torch.cuda.synchronize()
    np.testing.assert_array_equal(out.cpu().numpy(), ref)
    np.testing.assert_array_equal(ds.cpu().numpy().view(np.uint32), ref_next)


def test_ptmcmc_matches_reference(engine, golden):
    import torch

    g = golden("sampler.npz")
    NC = int(g["NC"])
    nens = len(g["seed0"])
    dT = torch.tensor(g["temperature"], device="cuda")
    dL = torch.tensor(g["logL"], device="cuda")
    dLn = torch.tensor(g["logLnorm"], device="cuda")
    didx = torch.tensor(np.tile(np.arange(NC, dtype=np.int32), (nens, 1)), device="cuda")
    dseed = torch.tensor(_u32(g["seed0"]), device="cuda")
    dacc = torch.zeros((nens, NC), dtype=torch.float64, device="cuda")
    torch.cuda.synchronize()
    for k in range(int(g["sweeps"])):
        engine.ptmcmc_device(dT, dL, didx, dseed, dacc, logLnorm=dLn)
        if k == 0:
            torch.cuda.synchronize()
            np.testing.assert_array_equal(didx.cpu().numpy(), g["index1"])
            np.testing.assert_array_equal(dseed.cpu().numpy().view(np.uint32), g["seed1"])
            np.testing.assert_array_equal(dacc.cpu().numpy(), g["acc1"])
    torch.cuda.synchronize()
    np.testing.assert_array_equal(didx.cpu().numpy(), g["indexN"])
    np.testing.assert_array_equal(dseed.cpu().numpy().view(np.uint32), g["seedN"])
    np.testing.assert_array_equal(dacc.cpu().numpy(), g["accN"])


def test_mh_accept_matches_restated_reference(engine, port):
    """ucb_mcmc's tail (ucb/src/glass_ucb_sampler.c:141-172): infinite priors
    (no draw), SNR below 5 (a draw, then rejection), non-finite logH, and
    ordinary proposals at a range of temperatures; 20 successive steps."""
    import torch

    rng = np.random.default_rng(32)
    n = 4096
    T = 1.3 ** rng.integers(0, 12, n)
    logL = rng.normal(1000, 10, n)
    px = rng.normal(0, 1, (n, 8))
    seed = rng.integers(1, 2**32, n, dtype=np.uint64).astype(np.uint32)
    d = {k: torch.tensor(v, device="cuda") for k, v in (("T", T), ("logL", logL.copy()), ("px", px.copy()))}
    dseed = torch.tensor(_u32(seed), device="cuda")
    for step in range(20):
        dlogl = rng.normal(-2, 3, n)
        dlogl[rng.random(n) < 0.01] = np.nan
        logPx = rng.normal(-5, 1, n)
        logPy = rng.normal(-5, 1, n)
        logPy[rng.random(n) < 0.1] = -np.inf
        logQxy, logQyx = rng.normal(0, 1, n), rng.normal(0, 1, n)
        snr = rng.uniform(0, 20, n)
        py = rng.normal(0, 1, (n, 8))
        acc_ref = port.mh_accept(T, logL, dlogl, logPx, logPy, logQxy, logQyx, seed, px, py, snr=snr)
        dd = {k: torch.tensor(v, device="cuda") for k, v in (("dl", dlogl), ("lpx", logPx), ("lpy", logPy),
                                                            ("qxy", logQxy), ("qyx", logQyx), ("snr", snr),
                                                            ("py", py))}
        dacc = torch.empty(n, dtype=torch.int32, device="cuda")
        torch.cuda.synchronize()
        engine.mh_accept_device(d["T"], dd["dl"], dd["lpx"], dd["lpy"], dd["qxy"], dd["qyx"], dseed, d["logL"],
                                d["px"], dd["py"], accepted=dacc, snr=dd["snr"])
        torch.cuda.synchronize()
        np.testing.assert_array_equal(dacc.cpu().numpy(), acc_ref)
        np.testing.assert_array_equal(dseed.cpu().numpy().view(np.uint32), seed)
        np.testing.assert_array_equal(d["logL"].cpu().numpy(), logL)
        np.testing.assert_array_equal(d["px"].cpu().numpy(), px)
    assert 0.05 < acc_ref.mean() < 0.9


def _fisher_draw_device(engine, x, evec, evalue, seed, draws):
    import torch

    dx, dev, del_ = (torch.tensor(np.ascontiguousarray(a, np.float64), device="cuda") for a in (x, evec, evalue))
    ds = torch.tensor(_u32(seed), device="cuda")
    n = len(x)
    dy = torch.empty((n, 8), dtype=torch.float64, device="cuda")
    dq = torch.empty(n, dtype=torch.float64, device="cuda")
    dst = torch.empty(n, dtype=torch.int32, device="cuda")
    out = []
    torch.cuda.synchronize()
    for _ in range(draws):
        engine.fisher_draw_device(dx, dev, del_, ds, dy, dq, dst)
        torch.cuda.synchronize()
        out.append((dy.cpu().numpy().copy(), dq.cpu().numpy().copy(), dst.cpu().numpy().copy(),
                    ds.cpu().numpy().view(np.uint32).copy()))
    return out


def test_fisher_draw_matches_reference(engine, golden):
    """draw_from_fisher on the device against the reference's own draws
    (golden vectors): seeds and return values exactly, parameters to 1e-14
    relative (the device's log against the C library's)."""
    g = golden("fisher_draw.npz")
    res = _fisher_draw_device(engine, g["x"], g["evec"], g["evalue"], g["seed0"], 4)
    for k, (y, q, st, s) in enumerate(res):
        np.testing.assert_array_equal(s, g["seeds"][k])
        np.testing.assert_array_equal(q, g["logQ"][k])
        np.testing.assert_allclose(y, g["y"][k], rtol=1e-14, atol=0)
        np.testing.assert_array_equal(st, np.where(np.isinf(q), gg.DRAW_NAN, gg.DRAW_OK))


def test_fisher_draw_many_chains(engine, port):
    """3072 chains, eight successive draws, against the oracle's restatement.
    The first six seeds start draws that need more than the 48 rand_r values
    the kernel's lanes generate at once (fewer than eight accepted polar pairs
    in them, or the eighth in the last pair), so those chains take the
    one-lane path; the test checks that they do need more."""
    from glass_gb300 import workloads as wl

    x, evec, evalue, seed = wl.fisher_draw_inputs(np.random.default_rng(33), n=3072)
    long_seeds = np.array([620013, 1277705, 2079646, 1627781, 2377129, 3502334], np.uint32)
    seed[:6] = long_seeds
    for k in range(6):  # values one draw consumes from each of these seeds
        s1 = seed[k:k + 1].copy()
        port.fisher_draw(x[k:k + 1], evec[k:k + 1], evalue[k:k + 1], s1)
        st, used = seed[k:k + 1].copy(), 0
        while st[0] != s1[0]:
            _, st = port.rand_r_seq(st, 1)
            used += 1
        assert used > 48, (k, used)
    res = _fisher_draw_device(engine, x, evec, evalue, seed, 8)
    s = seed.copy()
    for y, q, st, sd in res:
        yr, qr = port.fisher_draw(x, evec, evalue, s)
        np.testing.assert_array_equal(sd, s)
        np.testing.assert_array_equal(q, qr)
        np.testing.assert_allclose(y, yr, rtol=1e-14, atol=0)


def test_prior_draw_matches_reference(engine, golden):
    """draw_from_uniform_prior: three successive draws of 64 chains, bit for
    bit (parameters, logQ and the seeds after each draw)."""
    import torch

    g = golden("priors.npz")
    prior = torch.tensor(g["prior"].reshape(-1), device="cuda")
    logPV = torch.tensor(g["logPV"], device="cuda")
    seed = torch.tensor(_u32(g["seeds0"]), device="cuda")
    params = torch.empty((64, 8), dtype=torch.float64, device="cuda")
    logQ = torch.empty(64, dtype=torch.float64, device="cuda")
    for k in range(3):
        engine.prior_draw_device(prior, logPV, seed, params, logQ)
        torch.cuda.synchronize()
        np.testing.assert_array_equal(params.cpu().numpy(), g["draws"][k])
        np.testing.assert_array_equal(logQ.cpu().numpy(), g["logQ"][k])
        np.testing.assert_array_equal(seed.cpu().numpy().view(np.uint32), g["seeds"][k])


def test_ucb_prior_matches_reference(engine, golden):
    """evaluate_ucb_prior on 200 parameter sets, uniform and galaxy sky:
    the same -inf decisions, log priors and wrapped parameters."""
    import torch

    g = golden("priors.npz")
    prior = torch.tensor(g["prior"].reshape(-1), device="cuda")
    logPV = torch.tensor(g["logPV"], device="cuda")
    sky = torch.tensor(g["skyhist"], device="cuda")
    for key, kw in (("uniform", {}), ("galaxy", dict(skyhist=sky, dcostheta=float(g["dcostheta"]),
                                                        dphi=float(g["dphi"]), nphi=int(g["nphi"])))):
        p = torch.tensor(g["params"], device="cuda")
        lp = torch.empty(len(g["params"]), dtype=torch.float64, device="cuda")
        engine.ucb_prior_device(p, prior, logPV, lp, **kw)
        torch.cuda.synchronize()
        ref = g[f"logP_{key}"]
        got = lp.cpu().numpy()
        np.testing.assert_array_equal(np.isinf(got), np.isinf(ref))
        fin = np.isfinite(ref)
        np.testing.assert_allclose(got[fin], ref[fin], rtol=1e-14, atol=0)
        # the reference wraps longitude, polarisation and phase in place
        np.testing.assert_allclose(p.cpu().numpy()[fin], g[f"params_{key}"][fin], rtol=1e-13, atol=1e-13)


def test_device_fisher_jump_pipeline(engine, port, golden):
    """gradient/Fisher kernel -> device eigen-decomposition -> draw_from_fisher
    with no host round trip: the decomposition reconstructs each Fisher matrix
    (sorted eigenvalues, unit vectors), agrees with the drop-in
    matrix_eigenstuff, and the jumps drawn from it equal those drawn from the
    host decomposition."""
    import ctypes

    import torch

    from glass_gb300 import workloads as wl
    from glass_gb300.refstructs import Keep, bind_dropins

    g = golden("fisher.npz")
    T = wl.T_YEAR
    invC = g["invC"][0]
    zero = np.zeros((1, 1024), complex)
    engine.upload(wl.SegmentBank(T=T, NFFT=1024, qmin=np.array([g["qmin"][0]], np.int32), dA=zero, dE=zero,
                                 invCA=invC[None], invCE=invC[None]))
    rng = np.random.default_rng(12)
    base = g["params"][0]
    props = base + rng.standard_normal((96, 8)) * wl.jump_scales(base, 30.0)
    props[:, 1] = np.clip(props[:, 1], -0.99, 0.99)
    props[:, 4] = np.clip(props[:, 4], -0.99, 0.99)
    n = len(props)
    d_seg = torch.zeros(n, dtype=torch.int32, device="cuda")
    d_p = torch.tensor(props, device="cuda")
    ty = torch.empty(n, dtype=torch.float64, device="cuda")
    grad = torch.empty((n, 8), dtype=torch.float64, device="cuda")
    F = torch.empty((n, 8, 8), dtype=torch.float64, device="cuda")
    st = torch.empty(n, dtype=torch.int32, device="cuda")
    evec = torch.empty((n, 8, 8), dtype=torch.float64, device="cuda")
    eval_ = torch.empty((n, 8), dtype=torch.float64, device="cuda")
    seeds0 = rng.integers(1, 2**31, n).astype(np.uint32)
    seed = torch.tensor(_u32(seeds0), device="cuda")
    y = torch.empty((n, 8), dtype=torch.float64, device="cuda")
    engine.grad_fisher_device(d_seg, d_p, ty, grad, F, st)
    engine.sym_eigen8_device(F, evec, eval_)
    engine.fisher_draw_device(d_p, evec, eval_, seed, y)
    torch.cuda.synchronize()
    Fh, V, lam = F.cpu().numpy(), evec.cpu().numpy(), eval_.cpu().numpy()
    assert (st.cpu().numpy() == 0).all()
    L = bind_dropins(gg.load_library())
    Vh, lh = np.zeros_like(V), np.zeros_like(lam)
    for i in range(n):
        assert (np.diff(lam[i]) <= 0).all()
        np.testing.assert_allclose(np.linalg.norm(V[i], axis=0), 1.0, rtol=1e-12)
        np.testing.assert_allclose(V[i] @ np.diag(lam[i]) @ V[i].T, Fh[i], rtol=0, atol=1e-10 * np.abs(Fh[i]).max())
        # the drop-in on the host: the same convention
        keep = Keep()
        vp = keep.ptrs(np.zeros((8, 8)))
        L.matrix_eigenstuff(keep.ptrs(Fh[i]), vp, lh[i].ctypes.data_as(ctypes.POINTER(ctypes.c_double)), 8)
        Vh[i] = np.array([[vp[r][c] for c in range(8)] for r in range(8)])
    np.testing.assert_allclose(lh, lam, rtol=1e-9, atol=0)
    # the same draw from the host decomposition: the same chains' choices and seeds,
    # jumps equal to the decompositions' agreement
    seed2 = torch.tensor(_u32(seeds0), device="cuda")
    y2 = torch.empty_like(y)
    engine.fisher_draw_device(d_p, torch.tensor(Vh, device="cuda"), torch.tensor(lh, device="cuda"), seed2, y2)
    torch.cuda.synchronize()
    np.testing.assert_array_equal(seed.cpu().numpy(), seed2.cpu().numpy())
    jump, jump2 = y.cpu().numpy() - props, y2.cpu().numpy() - props
    np.testing.assert_allclose(jump, jump2, rtol=1e-6, atol=1e-9 * np.abs(jump).max())
