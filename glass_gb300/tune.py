"""Autotuner of the mixed-precision likelihood's launch shapes.

    python -m glass_gb300.tune [--steps 40] [--rounds 2] [--out glass_gb300/tuning.json]

Times the batched step - CUDA-graph replays of glass_gpu_dlogl_batch on a
parallel-tempering workload of 64 segments of 1024 bins and 3072 proposals
over 12 temperatures (sizes 32..1024 from the bandwidth rule), L2 flushed
between steps - for the values of each launch-shape knob of the engine
(glass_gpu_set_tuning: slow-part block size and CTAs per SM, persistent
spectral CTAs per SM, proposals per plan CTA), by coordinate descent from the
built-in choice: each knob in turn is set to its fastest value with the others
fixed, for a few rounds.  The result is recorded per GPU model (with the
sweep's timings) in a JSON table; Engine.apply_tuning() reads it.
"""
from __future__ import annotations

import argparse
import json
import math
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
TABLE = os.path.join(HERE, "tuning.json")

KNOBS = {
    "slow_block": [128, 256, 512],
    "slow_ctas_per_sm": [0, 2, 4, 6, 8],
    "spec_ctas_per_sm": [0, 1, 2, 3],
    "plan_per_cta": [0, 8, 12, 16, 24, 32],
}


def gpu_name(device: int = 0) -> str:
    import torch

    return torch.cuda.get_device_name(device)


def _workload(gg, eng, nbatch: int, seed: int = 7):
    from . import workloads as wl

    T = wl.T_YEAR
    rng = np.random.default_rng(seed)

    def wf(p):
        N = 2 * gg.ucb_bandwidth(wl.LARM, wl.FSTAR, p[0] / T, p[7] / T / T, p[1], math.exp(p[3]), T, 1024)
        h = gg.ucb_waveform(p, N, T)
        return N, h[3], h[4]

    bank, inj, _, item_seg, temps = wl.tempered_bank(rng, wf)
    eng.upload(bank)
    _, t_inj, hh, _ = eng.dlogl_host(np.arange(len(inj), dtype=np.int32), inj, precision=gg.PREC_FP64)
    batches = wl.tempered_proposals(rng, inj, np.sqrt(np.maximum(hh, 1.0)), item_seg, temps, nbatch)
    return item_seg, t_inj[item_seg], batches


def time_step(eng, gg, torch, dev, d_seg, d_batches, d_tx, outs, steps: int) -> float:
    """Mean device time (ms) of one mixed step, graph replays, L2 flushed."""
    stream = torch.cuda.Stream(dev)
    eng.set_stream(stream.cuda_stream)
    dl, ty, hh, st = outs
    nb = d_batches.shape[0]
    with torch.cuda.stream(stream):
        eng.dlogl_device(d_seg, d_batches[0], dl, ty, hh, st, term_x=d_tx, precision=gg.PREC_MIXED)
    stream.synchronize()
    graphs = []
    for k in range(nb):
        g = torch.cuda.CUDAGraph()
        with torch.cuda.graph(g, stream=stream):
            eng.dlogl_device(d_seg, d_batches[k], dl, ty, hh, st, term_x=d_tx, precision=gg.PREC_MIXED)
        graphs.append(g)
    flush = torch.empty(64 * 1024 * 1024, dtype=torch.float32, device=dev)  # 256 MB > L2
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(steps)]
    with torch.cuda.stream(stream):
        for k in range(3):
            graphs[k % nb].replay()
        for k in range(steps):
            flush.zero_()
            ev[k][0].record(stream)
            graphs[k % nb].replay()
            ev[k][1].record(stream)
    stream.synchronize()
    eng.set_stream(None)
    ts = sorted(a.elapsed_time(b) for a, b in ev)
    return float(np.mean(ts[: max(1, len(ts) * 3 // 4)]))  # the slowest quarter dropped (other users' noise)


def tune(device: int = 0, steps: int = 40, rounds: int = 2, verbose: bool = True) -> dict:
    import torch

    import glass_gb300 as gg

    dev = torch.device("cuda", device)
    torch.cuda.set_device(dev)
    eng = gg.Engine(device)
    try:
        item_seg, tx, batches = _workload(gg, eng, 8)
        n = len(item_seg)
        d_seg = torch.from_numpy(item_seg).to(dev)
        d_batches = torch.from_numpy(batches).to(dev)
        d_tx = torch.from_numpy(tx).to(dev)
        outs = (torch.empty(n, dtype=torch.float64, device=dev), torch.empty(n, dtype=torch.float64, device=dev),
                torch.empty(n, dtype=torch.float64, device=dev), torch.empty(n, dtype=torch.int32, device=dev))
        best = {k: eng.get_tuning(k) for k in KNOBS}
        sweeps = []
        base = time_step(eng, gg, torch, dev, d_seg, d_batches, d_tx, outs, steps)
        for r in range(rounds):
            for knob, values in KNOBS.items():
                res = {}
                for v in values:
                    eng.set_tuning(knob, v)
                    res[v] = time_step(eng, gg, torch, dev, d_seg, d_batches, d_tx, outs, steps)
                v_best = min(res, key=res.get)
                best[knob] = v_best
                eng.set_tuning(knob, v_best)
                sweeps.append({"round": r, "knob": knob, "ms": {str(k): v for k, v in res.items()}, "best": v_best})
                if verbose:
                    print(f"round {r} {knob}: " + ", ".join(f"{k}={v:.4f}" for k, v in res.items()) +
                          f" -> {v_best}", flush=True)
        final = time_step(eng, gg, torch, dev, d_seg, d_batches, d_tx, outs, steps)
    finally:
        eng.close()
    return {"gpu": gpu_name(device), "knobs": best, "ms_builtin": base, "ms_tuned": final,
            "workload": "64 segments x 1024 bins, 3072 proposals, 12 temperatures, mixed precision, "
                        "graph replay, L2 flushed", "sweeps": sweeps}


def load(path: str | None = None) -> dict:
    path = path or TABLE
    if not os.path.exists(path):
        return {}
    with open(path) as fh:
        return json.load(fh)


def apply(eng, path: str | None = None, device: int = 0) -> dict:
    """Sets the knobs recorded for this GPU model; returns them ({} if none)."""
    table = load(path)
    try:
        entry = table.get(gpu_name(device))
    except Exception:  # no torch / no device name: nothing to apply
        entry = None
    if not entry:
        return {}
    for k, v in entry["knobs"].items():
        eng.set_tuning(k, int(v))
    return dict(entry["knobs"])


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--device", type=int, default=0)
    ap.add_argument("--steps", type=int, default=40)
    ap.add_argument("--rounds", type=int, default=2)
    ap.add_argument("--out", default=TABLE)
    args = ap.parse_args()
    res = tune(args.device, args.steps, args.rounds)
    table = load(args.out)
    table[res["gpu"]] = res
    with open(args.out, "w") as fh:
        json.dump(table, fh, indent=1)
    print(f"{res['gpu']}: {res['ms_builtin']:.4f} ms -> {res['ms_tuned']:.4f} ms with {res['knobs']}")


if __name__ == "__main__":
    main()
