"""Partition of a segment bank over ranks for multi-GPU runs: the likelihood of
a proposal reads only its own segment, so ranks take disjoint sets of segments
(and the proposals on them) and exchange nothing on the data path; only the
timing reduction crosses ranks.  Contiguous blocks keep each rank's segments
adjacent in frequency (one rank's templates stay within its band)."""
from __future__ import annotations

import numpy as np

from .workloads import SegmentBank


def segments_of_rank(nseg: int, rank: int, world: int) -> np.ndarray:
    """Segment indices of one rank: the rank-th of `world` contiguous blocks,
    sizes differing by at most one."""
    if not (0 <= rank < world):
        raise ValueError("rank out of range")
    lo = rank * nseg // world
    hi = (rank + 1) * nseg // world
    return np.arange(lo, hi, dtype=np.int32)


def shard_bank(bank: SegmentBank, rank: int, world: int) -> tuple[SegmentBank, np.ndarray]:
    """The rank's sub-bank and the global indices of its segments."""
    idx = segments_of_rank(len(bank.qmin), rank, world)
    sub = SegmentBank(T=bank.T, NFFT=bank.NFFT, qmin=bank.qmin[idx], dA=bank.dA[idx], dE=bank.dE[idx],
                      invCA=bank.invCA[idx], invCE=bank.invCE[idx], t0=bank.t0)
    return sub, idx


def shard_proposals(item_seg: np.ndarray, seg_idx: np.ndarray) -> tuple[np.ndarray, np.ndarray]:
    """Of a batch's proposals, those on the rank's segments: (positions in the
    batch, segment indices local to the rank's sub-bank)."""
    local = np.full(int(max(item_seg.max(initial=-1), seg_idx.max(initial=-1))) + 1, -1, np.int32)
    local[seg_idx] = np.arange(len(seg_idx), dtype=np.int32)
    pos = np.nonzero(local[item_seg] >= 0)[0]
    return pos, local[item_seg[pos]]
