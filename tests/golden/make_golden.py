"""Generate the golden scan fixtures in this directory from the FP64 oracle.

Run from the repository root: ``python tests/golden/make_golden.py``.
Each fixture holds its seeded synthetic inputs and the oracle's outputs
(per-rotation top-k offsets and scores, plus the FP64 correlation grid of the
first rotation), so the GPU parity tests can check against committed values
without regenerating them.
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from oracle import fftdock_oracle as O  # noqa: E402
from proddl2_gb300 import synth  # noqa: E402

CASES = {
    "scan_shape_ace_n32": dict(seed=21, n_rec=300, n_lig=80, n=32, term_set=O.TERMS_SHAPE_ACE, n_rot=6, k=4),
    "scan_shape_n48": dict(seed=22, n_rec=600, n_lig=150, n=48, term_set=O.TERMS_SHAPE, n_rot=6, k=4),
    "scan_shape_ace_n64": dict(seed=23, n_rec=900, n_lig=250, n=64, term_set=O.TERMS_SHAPE_ACE, n_rot=3, k=8),
}
H = 1.2


def make(name, seed, n_rec, n_lig, n, term_set, n_rot, k):
    pair = synth.make_pair(n_rec, n_lig, n_rot, seed=seed)
    geom = O.Geometry.centred(H, n)
    tp = O.TermParams(term_set=term_set, ace_matrix=pair.ace)
    rg = O.receptor_terms(geom, pair.receptor.xyz, pair.receptor.ace_type, tp)
    rs = O.receptor_spectra(rg)
    w = O.ligand_term_weights(pair.ligand.ace_type, tp)
    offs = np.zeros((n_rot, k), np.int64)
    scores = np.zeros((n_rot, k))
    corr0 = None
    for i, rot in enumerate(pair.rotations):
        res = O.scan_rotation(geom, rg, rs, pair.ligand.xyz, w, rot, k, keep_corr=(i == 0))
        assert res.in_grid
        offs[i] = res.offsets
        scores[i] = res.scores
        if i == 0:
            corr0 = res.corr
    np.savez_compressed(
        os.path.join(HERE, name + ".npz"),
        rec_xyz=pair.receptor.xyz, rec_type=pair.receptor.ace_type,
        lig_xyz=pair.ligand.xyz, lig_type=pair.ligand.ace_type,
        ace=pair.ace, rotations=pair.rotations, grid_n=n, grid_step=H, term_set=term_set, k=k,
        offsets=offs, scores=scores,
        corr0=corr0.astype(np.float32) if n <= 48 else np.zeros(0, np.float32),
    )


if __name__ == "__main__":
    for name, kw in CASES.items():
        make(name, **kw)
        print("wrote", name)
