"""The adjoint kernels behind a torch.autograd.Function, in the test harness
only (the engine's interface is the C ABI): forward = term_y of each proposal
from glass_gpu_grad_fisher_batch, backward = the chain rule through its
gradient d term_y / d params.  Checked with torch.autograd.gradcheck-style
central differences of the FP64 path, through a downstream scalar (a weighted
sum of the terms, as a tempered likelihood sum is), and the Fisher matrix as
the Gauss-Newton Hessian of the same function."""
import numpy as np
import pytest

import glass_gb300 as gg
from glass_gb300 import workloads as wl

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")
T = wl.T_YEAR


class DeltaLogL(torch.autograd.Function):
    """term_y(params) of a batch of proposals on the engine's bank."""

    @staticmethod
    def forward(ctx, params, item_seg, engine):
        n = item_seg.numel()
        term = torch.empty(n, dtype=torch.float64, device=params.device)
        grad = torch.empty((n, 8), dtype=torch.float64, device=params.device)
        status = torch.empty(n, dtype=torch.int32, device=params.device)
        p = params.detach().contiguous()
        engine.grad_fisher_device(item_seg, p, term, grad, None, status)
        torch.cuda.synchronize()
        if bool((status != 0).any()):
            raise RuntimeError("invalid proposal in the batch")
        ctx.save_for_backward(grad)
        return term

    @staticmethod
    def backward(ctx, g_term):
        (grad,) = ctx.saved_tensors
        return g_term[:, None] * grad, None, None


@pytest.fixture(scope="module")
def engine():
    from glass_gb300 import build

    build.build()
    eng = gg.Engine(0)
    yield eng
    eng.close()


def _bank(rng, port, nseg=4, NFFT=1024):
    qmin, dA, dE, iA, iE, inj = [], [], [], [], [], []

    def wf(p):
        al = port.alignment(T, NFFT, 0, p)
        h = port.waveform(p, int(al[0]), T)
        return int(al[0]), h[3], h[4]

    for s in range(nseg):
        p = wl.draw_source(rng, rng.uniform(1e-3, 5e-3), 10 ** rng.uniform(-22.5, -21.5), 1e-17)
        p[1] = np.clip(p[1], -0.9, 0.9)
        p[4] = np.clip(p[4], -0.9, 0.9)
        q, a, e, ia, ie = wl.make_segment(rng, [p], wf, NFFT=NFFT, T=T)
        qmin.append(q), dA.append(a), dE.append(e), iA.append(ia), iE.append(ie), inj.append(p)
    return wl.SegmentBank(T=T, NFFT=NFFT, qmin=np.array(qmin, np.int32), dA=np.array(dA), dE=np.array(dE),
                          invCA=np.array(iA), invCE=np.array(iE)), np.array(inj)


def test_autograd_function_matches_central_differences(engine, port):
    rng = np.random.default_rng(41)
    bank, inj = _bank(rng, port)
    engine.upload(bank)
    dev = torch.device("cuda", 0)
    seg = np.repeat(np.arange(len(inj), dtype=np.int32), 3)
    props = np.array([wl.gaussian_jumps(rng, inj[s], wl.jump_scales(inj[s], 30.0), 1)[0] for s in seg])
    temps = torch.tensor(1.5 ** (np.arange(len(seg)) % 4), dtype=torch.float64, device=dev)
    d_seg = torch.from_numpy(seg).to(dev)
    x = torch.tensor(props, dtype=torch.float64, device=dev, requires_grad=True)
    # a downstream scalar: the tempered sum of the terms
    y = (DeltaLogL.apply(x, d_seg, engine) / temps).sum()
    y.backward()
    g = x.grad.cpu().numpy()
    # central differences of the same scalar on the FP64 path
    eps = 1e-6
    Tn = temps.cpu().numpy()
    fd = np.zeros_like(g)
    for k in range(8):
        pp, pm = props.copy(), props.copy()
        pp[:, k] += eps
        pm[:, k] -= eps
        tp = engine.dlogl_host(seg, pp, precision=gg.PREC_FP64)[1]
        tm = engine.dlogl_host(seg, pm, precision=gg.PREC_FP64)[1]
        fd[:, k] = (tp - tm) / (2 * eps) / Tn
    _, _, F, _ = engine.grad_fisher_host(seg, props)
    sig = np.sqrt(np.maximum(np.einsum("nkk->nk", F), 1e-30)) / Tn[:, None]
    err = np.abs(g - fd) / (sig + np.abs(fd))
    assert err.max() < 2e-3, err.max(axis=0)
    # forward value: the FP64 term to the mixed path's accuracy
    t64 = engine.dlogl_host(seg, props, precision=gg.PREC_FP64)[1]
    assert abs(float(y.detach()) - float((t64 / Tn).sum())) < 1e-3 * len(seg)


def test_fisher_is_the_gauss_newton_hessian_of_the_term(engine, port):
    """Near the injection the residual is noise, and d^2 term / dp dp' is
    -F + O(noise): the Hessian from differences of the autograd gradient
    (one backward per parameter) agrees with -F at the level of the
    expected noise term, ~ sqrt(F_kk F_ll)/SNR."""
    rng = np.random.default_rng(43)
    bank, inj = _bank(rng, port, nseg=2)
    engine.upload(bank)
    dev = torch.device("cuda", 0)
    seg = np.arange(2, dtype=np.int32)
    d_seg = torch.from_numpy(seg).to(dev)
    _, _, F, _ = engine.grad_fisher_host(seg, inj)
    H = np.zeros((2, 8, 8))
    for k in range(8):
        eps = 1e-2 / np.sqrt(F[:, k, k])  # a hundredth of each source's Fisher sigma
        gs = []
        for sgn in (1.0, -1.0):
            p = inj.copy()
            p[:, k] += sgn * eps
            x = torch.tensor(p, dtype=torch.float64, device=dev, requires_grad=True)
            DeltaLogL.apply(x, d_seg, engine).sum().backward()
            gs.append(x.grad.cpu().numpy())
        H[:, :, k] = (gs[0] - gs[1]) / (2 * eps[:, None])
    for s in range(2):
        snr = np.sqrt(max(F[s, 3, 3], 1.0))
        scale = np.sqrt(np.outer(np.diag(F[s]), np.diag(F[s])))
        rel = np.abs(H[s] + F[s]) / scale
        assert rel.max() < 10.0 / snr + 1e-2, (s, rel.max(), snr)
