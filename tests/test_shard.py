"""Rotation sharding over ranks (gloo, 2 processes, CPU): the merged result
equals the single-process scan.  Each rank's scan is the FP64 oracle on a
small case, standing in for one GPU's scan."""
import os
import socket

import numpy as np
import pytest
import torch.multiprocessing as mp

from oracle import fftdock_oracle as O


def test_rotation_ranges_cover_in_order():
    from proddl2_gb300.shard import rotation_range
    for n in (0, 1, 7, 64, 9000):
        for w in (1, 2, 3, 8):
            rs = [rotation_range(n, r, w) for r in range(w)]
            assert rs[0][0] == 0 and rs[-1][1] == n
            assert all(a[1] == b[0] for a, b in zip(rs, rs[1:]))
            assert max(b - a for a, b in rs) - min(b - a for a, b in rs) <= 1


def _case():
    from proddl2_gb300 import synth
    pair = synth.make_pair(60, 15, 9, seed=31)
    geom = O.Geometry.centred(1.2, 16)
    tp = O.TermParams(term_set=O.TERMS_SHAPE_ACE, ace_matrix=pair.ace)
    rg = O.receptor_terms(geom, pair.receptor.xyz, pair.receptor.ace_type, tp)
    rs = O.receptor_spectra(rg)
    w = O.ligand_term_weights(pair.ligand.ace_type, tp)
    return pair, geom, rg, rs, w


def _oracle_scan(case, rot, first, k=3):
    from proddl2_gb300 import _lib
    pair, geom, rg, rs, w = case
    peaks = np.zeros((rot.shape[0], k), dtype=_lib.peak_dtype())
    npk = np.zeros(rot.shape[0], dtype=np.int32)
    for i, r in enumerate(rot.reshape(-1, 3, 3)):
        res = O.scan_rotation(geom, rg, rs, pair.ligand.xyz, w, r, k)
        npk[i] = len(res.scores)
        for j in range(npk[i]):
            peaks[i, j]["rot_id"] = first + i
            peaks[i, j]["cell"] = res.cells[j]
            peaks[i, j]["t"] = res.translations[j]
            peaks[i, j]["score"] = res.scores[j]
    return peaks, npk


def _worker(rank, world, port, out_path):
    import torch.distributed as dist
    from proddl2_gb300.shard import scan_sharded
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    case = _case()
    merged = scan_sharded(lambda rot, first: _oracle_scan(case, rot, first), case[0].rotations, 10)
    if rank == 0:
        np.save(out_path, merged)
    dist.destroy_process_group()


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def test_sharded_scan_equals_single_process(tmp_path):
    from proddl2_gb300.shard import merge_peaks
    out = str(tmp_path / "merged.npy")
    mp.spawn(_worker, args=(2, _free_port(), out), nprocs=2, join=True)
    merged = np.load(out)
    case = _case()
    rot = case[0].rotations.reshape(-1, 9)
    single = merge_peaks([(0, *_oracle_scan(case, rot, 0))], rot, 10)
    assert np.array_equal(merged, single)
    # and the merge keeps the 10 smallest energies of all rotations
    allv = sorted(float(v) for v in _oracle_scan(case, rot, 0)[0]["score"].reshape(-1))
    assert list(merged["value"]) == allv[:10]
