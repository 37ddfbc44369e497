"""Seeded synthetic workloads for the UCB likelihood engine.

Every input here is generated from numpy's PCG64 with a fixed seed, so the
GPU path, the oracle and the CPU baseline all see identical arrays.  The
shapes and value distributions are the ones the benchmark configurations
describe:

* ``segment_config0`` -- one A/E segment of NFFT = 1024 bins around a source
  with f0 ~ U[3.0, 3.5] mHz, fdot = 1e-17, A = 1e-22, N = 128 slow-part
  samples, plus Gaussian-jump proposals around it;
* ``segments_config1`` -- 64 independent one-year segments, f0 log-uniform in
  [0.5, 15] mHz, A log-uniform in [1e-23, 1e-21], 256 chains x 12
  temperatures, one proposal per (chain, temperature);
* ``proposals_config2`` -- 16384 proposals, f0 ~ U[1, 5] mHz, A log-uniform.

Noise follows the reference's convention (utils/src/glass_data.c:1323-1403):
each bin's real and imaginary parts are N(0, C/2) with C the A/E PSD of
utils/src/glass_lisa.c:1137-1145 at the "scirdv1" levels
(acceleration 3e-15 m/s^2/rtHz, optical metrology 1.5e-11 m/rtHz).
"""
from __future__ import annotations

import dataclasses
import math

import numpy as np

T_YEAR = 31457280.0
CLIGHT = 299792458.0
LARM = 2.5e9
PI2 = 6.283185307179586
FSTAR = CLIGHT / (2.0 * math.pi * LARM)


def noise_levels_scirdv1(f):
    """utils/src/glass_lisa.c:1089-1106: (Spm, Sop) for the "scirdv1" model."""
    f = np.asarray(f, np.float64)
    fonc = PI2 * f / CLIGHT
    sa_a = 9.00e-30 * (1.0 + (0.4e-3 / f) * (0.4e-3 / f)) * (1.0 + (f / 8.0e-3) ** 4)
    sa_d = sa_a * (PI2 * f) ** -4.0
    spm = sa_d * fonc * fonc
    soms_d = 2.25e-22 * (1.0 + (2.0e-3 / f) ** 4.0)
    return spm, soms_d * fonc * fonc


def aenoise_ff(f):
    """utils/src/glass_lisa.c:1137-1145: A/E noise PSD (fractional frequency)."""
    f = np.asarray(f, np.float64)
    spm, sop = noise_levels_scirdv1(f)
    x = f / FSTAR
    return 8.0 * np.sin(x) ** 2 * (2.0 * spm * (3.0 + 2.0 * np.cos(x) + np.cos(2.0 * x)) + sop * (2.0 + np.cos(x)))


@dataclasses.dataclass
class SegmentBank:
    """A set of A/E frequency segments of equal length NFFT.

    dA, dE: (S, NFFT) complex data (or residual); invCA, invCE: (S, NFFT) real;
    qmin: (S,) first DFT bin of each segment.
    """

    T: float
    NFFT: int
    qmin: np.ndarray
    dA: np.ndarray
    dE: np.ndarray
    invCA: np.ndarray
    invCE: np.ndarray
    t0: float = 0.0

    @property
    def nseg(self) -> int:
        return len(self.qmin)

    def interleaved(self):
        """(S, 2*NFFT) float64 arrays in the reference's re/im layout."""
        def il(z):
            out = np.empty(z.shape[:-1] + (2 * z.shape[-1],))
            out[..., 0::2] = z.real
            out[..., 1::2] = z.imag
            return out

        return il(self.dA), il(self.dE)


def make_params(f0, costh, phi, amp, cosi, psi, phi0, fdot, T=T_YEAR):
    """The reference's params array (ucb/src/glass_ucb_model.c:40-53)."""
    return np.array([f0 * T, costh, phi, math.log(amp), cosi, psi, phi0, fdot * T * T], np.float64)


def draw_source(rng, f0, amp, fdot=1e-17, T=T_YEAR):
    return make_params(f0, rng.uniform(-1, 1), rng.uniform(0, 2 * math.pi), amp, rng.uniform(-1, 1),
                       rng.uniform(0, math.pi), rng.uniform(0, 2 * math.pi), fdot, T)


def make_segment(rng, params_list, waveform_fn, NFFT=1024, T=T_YEAR, center_f0=None, noise=True):
    """One segment centred on the first source, with every source injected.

    ``waveform_fn(params, N) -> (A, E)`` returns 2N-double interleaved arrays for
    a template of N bins starting at bin floor(f0 T) - N/2 (the layout of
    ucb_waveform, ucb/src/glass_ucb_waveform.c:738), and ``bandwidth_fn`` is
    folded into waveform_fn's caller.
    """
    f0c = params_list[0][0] / T if center_f0 is None else center_f0
    qmin = int(f0c * T) - NFFT // 2
    f = (qmin + np.arange(NFFT)) / T
    C = aenoise_ff(f)
    dA = np.zeros(NFFT, np.complex128)
    dE = np.zeros(NFFT, np.complex128)
    for p in params_list:
        N, A, E = waveform_fn(p)
        q = int(p[0])  # (long)(f0*T)
        i0 = q - N // 2 - qmin
        for arr, h in ((dA, A), (dE, E)):
            hc = h[0::2] + 1j * h[1::2]
            lo, hi = max(0, i0), min(NFFT, i0 + N)
            if hi > lo:
                arr[lo:hi] += hc[lo - i0:hi - i0]
    if noise:
        sig = np.sqrt(C / 2.0)
        dA += sig * rng.standard_normal(NFFT) + 1j * sig * rng.standard_normal(NFFT)
        dE += sig * rng.standard_normal(NFFT) + 1j * sig * rng.standard_normal(NFFT)
    return qmin, dA, dE, 1.0 / C, 1.0 / C


def jump_scales(params, snr):
    """Per-parameter Gaussian jump widths of roughly one Fisher sigma for a
    source of the given SNR (frequency in bins, angles in radians)."""
    s = 1.0 / max(float(snr), 1.0)
    return np.array([0.3 * s, 0.5 * s, 0.5 * s, 1.0 * s, 0.5 * s, 0.5 * s, 1.0 * s, 1.0 * s])


def gaussian_jumps(rng, params, scales, n):
    """n proposals params + N(0, scales^2), with the cos-parameters kept in
    (-1, 1) the way draw_from_fisher does (ucb/src/glass_ucb_proposal.c:382-386)."""
    jump = rng.standard_normal((n, 8)) * scales
    out = params[None, :] + jump
    for k in (1, 4):
        bad = (out[:, k] >= 1.0) | (out[:, k] <= -1.0)
        out[bad, k] = params[k] - jump[bad, k]
    return out


def tempered_bank(rng, waveform_fn, nseg=64, NFFT=1024, nchain=256, ntemp=12, f_range=(0.5e-3, 15e-3),
                  log10_amp_range=(-23.0, -21.0), T=T_YEAR):
    """A parallel-tempering likelihood workload: nseg independent segments of
    NFFT bins, each the injection of one source (f0 log-uniform over f_range,
    log10 amplitude uniform over log10_amp_range) in Gaussian A/E noise; nchain x
    ntemp proposals per batch, chain c of segment c mod nseg at temperature
    1.5^(i mod ntemp).  waveform_fn(params) -> (N, A, E) places a template.
    Returns bank, injections, template sizes, item_seg and temperatures."""
    inj, Ns = [], []
    qmin, dA, dE, iA, iE = [], [], [], [], []
    for s in range(nseg):
        f0 = 10 ** rng.uniform(math.log10(f_range[0]), math.log10(f_range[1]))
        amp = 10 ** rng.uniform(log10_amp_range[0], log10_amp_range[1])
        p = draw_source(rng, f0, amp, 1e-17, T=T)
        q, a, e, ia, ie = make_segment(rng, [p], waveform_fn, NFFT=NFFT, T=T)
        qmin.append(q), dA.append(a), dE.append(e), iA.append(ia), iE.append(ie), inj.append(p)
        Ns.append(waveform_fn(p)[0])
    bank = SegmentBank(T=T, NFFT=NFFT, qmin=np.array(qmin, np.int32), dA=np.array(dA), dE=np.array(dE),
                       invCA=np.array(iA), invCE=np.array(iE))
    items = nchain * ntemp
    item_seg = (np.arange(items) // ntemp % nseg).astype(np.int32)
    temps = 1.5 ** (np.arange(items) % ntemp)
    return bank, np.array(inj), np.array(Ns), item_seg, temps


def tempered_proposals(rng, inj, snr, item_seg, temps, nbatch):
    """nbatch batches of Gaussian jumps around each chain's state, widened by
    sqrt(temperature); cos-parameters reflected back inside (-1, 1) as
    draw_from_fisher does (ucb/src/glass_ucb_proposal.c:382-386), and left
    unchanged when even the reflection falls outside."""
    scales = np.array([jump_scales(inj[s], max(snr[s], 5.0)) for s in range(len(inj))])
    out = np.empty((nbatch, len(item_seg), 8))
    x = inj[item_seg]
    for b in range(nbatch):
        jump = rng.standard_normal((len(item_seg), 8)) * scales[item_seg] * np.sqrt(temps)[:, None]
        p = x + jump
        for k in (1, 4):
            bad = (p[:, k] >= 1.0) | (p[:, k] <= -1.0)
            p[bad, k] = x[bad, k] - jump[bad, k]
            bad = (p[:, k] >= 1.0) | (p[:, k] <= -1.0)
            p[bad, k] = x[bad, k]
        out[b] = p
    return out


def global_fit_bank(rng, waveform_fn, nsrc=10000, nseg=512, NFFT=8192, T=T_YEAR):
    """A global-fit-scale population: nsrc sources of a synthetic Galactic
    population (f0 log-uniform over 0.1-10 mHz, fdot from the GR chirp with
    chirp mass ~U[0.2, 0.8] Msun, amplitude from the chirp mass, f0 and a
    distance ~U[1, 15] kpc, isotropic sky and orientation) injected into nseg
    segments of NFFT A/E bins centred on log-spaced frequencies (each source
    in the nearest), with Gaussian noise.  Returns (bank, sources [nsrc, 8],
    segment of each source)."""
    MSUN_S, KPC_M = 4.925491025543576e-06, 3.0856775814913673e19
    f = 10 ** rng.uniform(math.log10(1e-4), math.log10(1e-2), nsrc)
    mc = rng.uniform(0.2, 0.8, nsrc) * MSUN_S
    dist = rng.uniform(1.0, 15.0, nsrc) * KPC_M
    amp = 2.0 * mc ** (5.0 / 3.0) * (math.pi * f) ** (2.0 / 3.0) * CLIGHT / dist
    fdot = 96.0 / 5.0 * math.pi ** (8.0 / 3.0) * mc ** (5.0 / 3.0) * f ** (11.0 / 3.0)
    src = np.array([make_params(f[i], rng.uniform(-1, 1), rng.uniform(0, 2 * math.pi), amp[i], rng.uniform(-1, 1),
                                rng.uniform(0, math.pi), rng.uniform(0, 2 * math.pi), fdot[i], T)
                    for i in range(nsrc)])
    centres = np.exp(np.linspace(math.log(1.3e-4), math.log(9.7e-3), nseg))
    centres = np.maximum(centres, (NFFT // 2 + 16) / T)  # every segment starts above 0 Hz
    seg_of = np.clip(np.searchsorted((centres[1:] + centres[:-1]) / 2, f), 0, nseg - 1).astype(np.int32)
    qmin, dA, dE, iA, iE = [], [], [], [], []
    for s in range(nseg):
        members = [src[i] for i in np.nonzero(seg_of == s)[0]]
        q, a, e, ia, ie = make_segment(rng, members, waveform_fn, NFFT=NFFT, T=T, center_f0=centres[s])
        qmin.append(q), dA.append(a), dE.append(e), iA.append(ia), iE.append(ie)
    bank = SegmentBank(T=T, NFFT=NFFT, qmin=np.array(qmin, np.int32), dA=np.array(dA), dE=np.array(dE),
                       invCA=np.array(iA), invCE=np.array(iE))
    return bank, src, seg_of


def global_fit_proposals(rng, bank, src, seg_of, snr, nb, nchain=64, ntemp=16, T=T_YEAR):
    """nb batches of one RJMCMC move per source of global_fit_bank, the
    sources owned by nchain x ntemp chains (temperature 1.5^(i mod ntemp)):
    an update (Gaussian jump of about a Fisher sigma at the source's SNR,
    widened by sqrt(T)) or, for one source in five, a birth (a prior draw in
    the source's segment, nothing there yet).  Returns (batches [nb, nsrc, 8],
    birth mask [nb, nsrc])."""
    nsrc = len(src)
    temps = 1.5 ** (np.arange(nsrc) % (nchain * ntemp) % ntemp)
    batches, births = np.empty((nb, nsrc, 8)), np.empty((nb, nsrc), bool)
    for b in range(nb):
        birth = rng.uniform(size=nsrc) < 0.2
        scales = np.array([jump_scales(src[i], max(snr[i], 5.0)) for i in range(nsrc)])
        jump = rng.standard_normal((nsrc, 8)) * scales * np.sqrt(temps)[:, None]
        p = src + jump
        for k in (1, 4):
            bad = np.abs(p[:, k]) >= 1.0
            p[bad, k] = src[bad, k]
        qs = bank.qmin[seg_of] + rng.uniform(0.1, 0.9, nsrc) * bank.NFFT
        bp = np.array([make_params(qs[i] / T, rng.uniform(-1, 1), rng.uniform(0, 2 * math.pi),
                                   10 ** rng.uniform(-23, -21), rng.uniform(-1, 1), rng.uniform(0, math.pi),
                                   rng.uniform(0, 2 * math.pi), 0.0, T) for i in range(nsrc)])
        p[birth] = bp[birth]
        batches[b] = p
        births[b] = birth
    return batches, births


def wavelet_invC(N, NT, kmin, scale=1.0):
    """Inverse noise covariance of a wavelet segment of N pixels starting at
    pixel kmin of a grid with NT pixels per layer: per pixel the inverse of
    scale^2 * s(i) * [[1, -0.45, -0.45], [-0.45, 1, -0.45], [-0.45, -0.45, 1]]
    (X, Y, Z noise correlated as in the equal-arm Michelson channels), with
    s(i) = 1 + 0.2 sin(2 pi i / NT) + 0.1 sin(2 pi k / 97)^2 a slow trend in the
    time index i = k mod NT.  Returned as [3][3][N] (the reference's
    invC[i][j][k] layout)."""
    k = np.arange(N) + kmin
    s = (1.0 + 0.2 * np.sin(2 * np.pi * (k % NT) / NT) + 0.1 * np.sin(2 * np.pi * k / 97.0) ** 2) * scale**2
    base = np.full((3, 3), -0.45) + np.eye(3) * 1.45
    inv = np.linalg.inv(base)
    return np.ascontiguousarray(inv[:, :, None] / s[None, None, :])


# Noise-model defaults of the noise module (noise/src/glass_noise_model.c:1378-1458):
# link levels and the galactic foreground for a one-year observation.
NOISE_SACC0 = 5.76e-30
NOISE_SOMS0 = 1.28e-22


def default_noise_params(T=T_YEAR):
    """(inst [12], sgal [5]) at the noise module's starting point."""
    inst = np.array([NOISE_SACC0] * 6 + [NOISE_SOMS0] * 6)
    f1 = 10.0 ** (-2.235e-1 * math.log10(T / 3.15581497632e7) - 2.7040844)
    fk = 10.0 ** (-3.60976122e-1 * math.log10(T / 3.15581497632e7) - 2.37822436)
    sgal = np.array([math.log(1.2826e-44), math.log(f1), 1.629667, math.log(fk), math.log(4.810781e-4)])
    return inst, sgal


def sgwb_response_table(n=1000, fmin=1e-5, fmax=1.0):
    """A synthetic instrument response to an isotropic stochastic background
    in the layout of the noise module's response file (rows f, XX, YY, ZZ, XY,
    XZ, YZ; f log-evenly spaced): a smooth equal-arm-like shape, x^6 at low
    frequency (x = f / f*) with transfer-function ripples above f*, slightly
    unequal channels, cross-responses near -1/2 of the auto-responses at low
    frequency that change sign above f*.  Stands in for the response file the
    reference reads, which is data, not part of this library."""
    f = np.exp(np.linspace(math.log(fmin), math.log(fmax), n))
    x = f / FSTAR
    auto = 27.0 * np.sin(x) ** 2 * x ** 4 / (1.0 + 0.6 * x ** 2) + 1e-30 * x ** 2
    rows = np.empty((n, 7))
    rows[:, 0] = f
    rows[:, 1] = auto
    rows[:, 2] = auto * (1.0 + 1e-3 * np.sin(x))
    rows[:, 3] = auto * (1.0 - 1e-3 * np.sin(2 * x))
    cross = -0.5 * auto * np.cos(x) / (1.0 + 0.05 * x ** 2)
    rows[:, 4] = cross
    rows[:, 5] = cross * (1.0 + 2e-3 * np.cos(x))
    rows[:, 6] = cross * (1.0 - 2e-3 * np.sin(x))
    return rows


def default_sgwb_params(sgwb_type):
    """The noise module's starting point per SGWB template
    (default_sgwb_injection, noise/src/glass_noise_model.c:1459-1486)."""
    return {0: np.array([-8.45, 2.0 / 3.0]), 1: np.array([-2.5, math.log(2e-3) / math.log(10.0), 0.0]),
            2: np.array([1.0, 1.0, -18.0, -2.5])}[int(sgwb_type)]


def sgwb_params_draw(rng, sgwb_type, n):
    """n parameter sets [n, 4] of an SGWB template around its starting point,
    the amplitude raised so that the background rivals the instrument noise
    near 2 mHz (power law x30, lognormal x3 in A, phase transition x1e9);
    phase transitions kept where their spectrum is finite at every
    frequency (rb^4 (5 - b) < 4, i.e. b + 4 > m)."""
    t = int(sgwb_type)
    p0 = default_sgwb_params(t)
    lift = {0: 1.5, 1: 0.5, 2: 9.0}[t]
    out = np.zeros((n, 4))
    for k in range(n):
        while True:
            p = p0 + rng.uniform(-0.3, 0.3, len(p0))
            p[0 if t < 2 else 2] += lift
            if t == 2:
                p[1] = rng.uniform(1.5, 3.0)
                if p[0] ** 4 * (5.0 - p[1]) >= 3.6:
                    continue
            break
        out[k, :len(p0)] = p
    return out


def spline_noise_data(rng, T, qmin, NFFT, nch, excess=1.0):
    """Data for the spline noise model on bins qmin/T + n/T: the A/E noise
    PSD as the transfer function (initialize_spline_model,
    noise/src/glass_noise_model.c:1346-1355, with the A/E form for one channel
    too) and, per channel, complex bins with E|d|^2 = transfer (1 + excess
    bump), a smooth excess (a Gaussian in log f centred in the band, as a
    foreground would add) that the spline has to fit.  Returns (transfer
    [NFFT], d [nch, 2 NFFT], the excess spectrum [nch, NFFT] over transfer)."""
    f = (qmin + np.arange(NFFT)) / T
    tr = aenoise_ff(f)
    lf = np.log(f)
    mid, wid = 0.5 * (lf[0] + lf[-1]), max(0.25 * (lf[-1] - lf[0]), 1e-12)
    d = np.empty((nch, 2 * NFFT))
    ex = np.empty((nch, NFFT))
    for c in range(nch):
        ex[c] = tr * excess * (1.0 + 0.2 * c) * np.exp(-0.5 * ((lf - mid) / wid) ** 2)
        sd = np.sqrt(0.5 * (tr + ex[c]))
        d[c, 0::2] = rng.standard_normal(NFFT) * sd
        d[c, 1::2] = rng.standard_normal(NFFT) * sd
    return tr, d, ex


def spline_noise_models(rng, T, qmin, NFFT, excess, n, kmax, kmin=2, first_full=True):
    """n spline noise models [knots in the layout the batched likelihood
    takes]: nknots [n], knot_f [n, kmax], knot_C [n, nch, kmax].  The first
    (first_full) has kmax knots log-evenly spaced over fmin .. fmax with the
    first moved down half a bin (initialize_spline_model,
    noise/src/glass_noise_model.c:1357-1372); the others a knot count drawn
    from kmin .. kmax (the trans-dimensional sampler's range) with the end
    knots kept and the interior knots on an even grid moved by up to 0.3 of
    its spacing.  Control values: the excess (excess [nch, NFFT], linearly
    interpolated) times 1 + U(-0.1, 0.1)."""
    nch = len(excess)
    fmin, fmax = qmin / T, (qmin + NFFT) / T
    f = (qmin + np.arange(NFFT)) / T
    nk = np.zeros(n, np.int32)
    kf = np.zeros((n, kmax))
    kC = np.zeros((n, nch, kmax))
    for p in range(n):
        if p == 0 and first_full:
            K = kmax
            x = np.exp(np.linspace(math.log(fmin), math.log(fmax), K))
        else:
            K = int(rng.integers(kmin, kmax + 1))
            x = np.linspace(fmin, fmax, K)
            x[1:-1] += rng.uniform(-0.3, 0.3, K - 2) * (fmax - fmin) / (K - 1)
        x[0] -= 0.5 / T
        nk[p] = K
        kf[p, :K] = x
        for c in range(nch):
            kC[p, c, :K] = np.interp(x, f, excess[c]) * (1.0 + rng.uniform(-0.1, 0.1, K))
    return nk, kf, kC


def xyz_from_covariance(rng, C6):
    """Complex XYZ bins with E[x x^H] = C for real symmetric per-bin C given as
    [N, 6] = xx, yy, zz, xy, xz, yz; returned interleaved (3, 2N)."""
    N = len(C6)
    C = np.empty((N, 3, 3))
    C[:, 0, 0], C[:, 1, 1], C[:, 2, 2] = C6[:, 0], C6[:, 1], C6[:, 2]
    C[:, 0, 1] = C[:, 1, 0] = C6[:, 3]
    C[:, 0, 2] = C[:, 2, 0] = C6[:, 4]
    C[:, 1, 2] = C[:, 2, 1] = C6[:, 5]
    L = np.linalg.cholesky(C)
    g = (rng.standard_normal((N, 3)) + 1j * rng.standard_normal((N, 3))) * math.sqrt(0.5)
    x = np.einsum("nij,nj->ni", L, g)
    out = np.empty((3, 2 * N))
    out[:, 0::2] = x.real.T
    out[:, 1::2] = x.imag.T
    return out


def wavelet_noise_data(rng, C6_layers, NT):
    """Real wavelet coefficients X, Y, Z (pixel i of layer j at i + j NT) drawn
    per layer with covariance C6_layers [Nlayer, 6] (xx, yy, zz, xy, xz, yz)."""
    Nl = len(C6_layers)
    C = np.empty((Nl, 3, 3))
    C[:, 0, 0], C[:, 1, 1], C[:, 2, 2] = C6_layers[:, 0], C6_layers[:, 1], C6_layers[:, 2]
    C[:, 0, 1] = C[:, 1, 0] = C6_layers[:, 3]
    C[:, 0, 2] = C[:, 2, 0] = C6_layers[:, 4]
    C[:, 1, 2] = C[:, 2, 1] = C6_layers[:, 5]
    L = np.linalg.cholesky(C)
    x = np.einsum("jab,jbi->aji", L, rng.standard_normal((Nl, 3, NT)))
    return x.reshape(3, Nl * NT)


def galaxy_modulation_like(Ncoarse, phase=0.0):
    """A smooth modulation cache (6, Ncoarse) with the structure of
    galaxy_modulation_cache_for_Q's output (XX, YY, ZZ, XY, XZ, YZ): yearly
    variation of the three auto terms, cross terms -0.45 sqrt(auto auto), so
    that the modulated foreground stays a covariance."""
    q = np.arange(Ncoarse)
    a = [1.0 + 0.3 * np.cos(2 * np.pi * q / Ncoarse + phase + 2.1 * k) for k in range(3)]
    return np.stack(a + [-0.45 * np.sqrt(a[0] * a[1]), -0.45 * np.sqrt(a[0] * a[2]), -0.45 * np.sqrt(a[1] * a[2])])


def fisher_draw_inputs(rng, n=64):
    """Chains for draw_from_fisher: UCB parameter arrays (f0 T, cos theta, phi,
    ln A, cos iota, psi, phi0, fdot T^2), Fisher eigenvectors from random
    orthogonal matrices and eigenvalues from 1e2 to 1e12; the last chains are
    edge cases: cosines near +-1 with wide jumps (reflections), a zero and a
    negative eigenvalue (infinite and NaN amplitudes), a NaN parameter."""
    T = 31457280.0
    x = np.column_stack([rng.uniform(1e-3, 1e-2, n) * T, rng.uniform(-1, 1, n), rng.uniform(0, 2 * np.pi, n),
                         np.log(10 ** rng.uniform(-23, -21, n)), rng.uniform(-1, 1, n), rng.uniform(0, np.pi, n),
                         rng.uniform(0, 2 * np.pi, n), rng.normal(0, 1, n)])
    evec = np.zeros((n, 8, 8))
    evalue = np.zeros((n, 8))
    for i in range(n):
        q, r = np.linalg.qr(rng.normal(size=(8, 8)))
        evec[i] = q * np.sign(np.diag(r))
        evalue[i] = 10 ** rng.uniform(2, 12, 8)
    for i in range(n - 8, n - 4):  # cosines at the edge, jumps of order 1
        x[i, 1] = 0.9999 if i % 2 else -0.9999
        x[i, 4] = -0.9998 if i % 2 else 0.9998
        evalue[i] = 1.0
    evalue[n - 4, 3] = 0.0
    evalue[n - 3, 5] = -1.0
    evalue[n - 3, 2] = 0.0
    x[n - 2, 6] = np.nan
    seed = rng.integers(1, 2**31, n).astype(np.uint32)
    return x, evec, evalue, seed
