"""Rotation-range sharding over ranks and the gather of their peaks.

The reference parallelises a scan by splitting the rotation set into
contiguous ranges, one ``rot-scan`` process each, and merging their records
in a ``gather`` task (``python/lib/PRODDL/dock.py:86-133``).  Here one rank
(one GPU) takes each range, no collective touches the data path, and rank 0
merges the ranks' peaks with the ``Foreman`` rule: every peak becomes a pose
(rotation, translation), the ``max_matches`` lowest energies are kept,
ascending, ties in rotation order.
"""
from __future__ import annotations

import numpy as np


def rotation_range(n_rot, rank, world):
    """Contiguous [start, end) of the rotation set for ``rank``; ranges
    differ in length by at most one and cover the set in rank order."""
    if world < 1 or not (0 <= rank < world):
        raise ValueError("bad rank/world")
    base, extra = divmod(n_rot, world)
    start = rank * base + min(rank, extra)
    return start, start + base + (1 if rank < extra else 0)


def merge_peaks(parts, rotations, max_matches):
    """Foreman-style merge of per-rank peak lists.

    ``parts``: list (rank order) of (first_rot_id, peaks, n_peaks) with
    ``peaks`` structured fftdock_peak arrays (n_rot_rank, P).  Returns a
    structured pose array (value, rot[9], t[3]) ascending."""
    from . import _lib
    rot = np.asarray(rotations, dtype=np.float64).reshape(-1, 9)
    entries = []
    seq = 0
    for first, peaks, npk in parts:
        for i in range(peaks.shape[0]):
            for j in range(int(npk[i])):
                p = peaks[i, j]
                entries.append((float(p["score"]), seq, int(p["rot_id"]), p["t"].copy()))
                seq += 1
    entries = [e for e in entries if e[0] < 1e16]
    entries.sort(key=lambda e: (e[0], e[1]))
    entries = entries[:max_matches]
    out = np.zeros(len(entries), dtype=_lib.pose_dtype())
    for k, (v, _, rid, t) in enumerate(entries):
        out[k]["value"] = v
        out[k]["rot"] = rot[rid]
        out[k]["t"] = t
    return out


def scan_sharded(scan_fn, rotations, max_matches, group=None):
    """Scan this rank's range with ``scan_fn(rot_slice, first_rot_id) ->
    (peaks, n_peaks)`` and merge on rank 0 (other ranks return None).  Uses
    torch.distributed object gather when a process group is initialised."""
    import torch.distributed as dist
    rotations = np.asarray(rotations, dtype=np.float64).reshape(-1, 9)
    world = dist.get_world_size(group) if dist.is_initialized() else 1
    rank = dist.get_rank(group) if dist.is_initialized() else 0
    lo, hi = rotation_range(rotations.shape[0], rank, world)
    peaks, npk = scan_fn(rotations[lo:hi], lo)
    mine = (lo, peaks, npk)
    if world == 1:
        return merge_peaks([mine], rotations, max_matches)
    gathered = [None] * world if rank == 0 else None
    dist.gather_object(mine, gathered, dst=0, group=group)
    if rank != 0:
        return None
    return merge_peaks(gathered, rotations, max_matches)
