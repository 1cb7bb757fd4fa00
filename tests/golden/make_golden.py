"""Generate the golden scan fixtures in this directory from the FP64 oracle.

Run from the repository root: ``python tests/golden/make_golden.py [name ...]``
(no names: every fixture).  Each fixture holds its seeded synthetic inputs
and the oracle's outputs (per-rotation top-k offsets and scores, plus the
FP64 correlation grid of the first rotation at small sizes), so the GPU
parity tests check against committed values without regenerating them.

The ``config*`` fixtures are the benchmark workloads themselves (seed 1, the
seed the benchmark uses):
* config1_shape64: receptor 1800 / ligand 450 atoms, 64^3 at 1.2 A, shape
  only, all 2000 rotations, 4 peaks per rotation, and the ranked top 100 of
  the whole scan (the reference's Foreman gather over the per-rotation
  records);
* config2_shape_ace128: receptor 4000 / ligand 1500 atoms, 128^3 at 1.2 A,
  shape + 18 desolvation terms, 256 of the 9000 rotations (every 35th), 4
  peaks per rotation, and the ranked top 100 of those 256.
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
    "config1_shape64": dict(seed=1, n_rec=1800, n_lig=450, n=64, term_set=O.TERMS_SHAPE, n_rot=2000, k=4,
                            top=100),
    "config2_shape_ace128": dict(seed=1, n_rec=4000, n_lig=1500, n=128, term_set=O.TERMS_SHAPE_ACE, n_rot=9000,
                                 k=4, every=35, keep=256, top=100),
}
H = 1.2


def make(name, seed, n_rec, n_lig, n, term_set, n_rot, k, every=1, keep=None, top=0):
    pair = synth.make_pair(n_rec, n_lig, n_rot, seed=seed)
    rots = pair.rotations[::every][:keep]
    geom = O.Geometry.centred(H, n)
    tp = O.TermParams(term_set=term_set, ace_matrix=pair.ace)
    rg = O.receptor_terms(geom, pair.receptor.xyz, pair.receptor.ace_type, tp)
    rs = O.receptor_spectra(rg, workers=os.cpu_count() or 1)
    w = O.ligand_term_weights(pair.ligand.ace_type, tp)
    m = len(rots)
    offs = np.zeros((m, k), np.int64)
    scores = np.zeros((m, k))
    corr0 = None
    records = []
    for i, rot in enumerate(rots):
        res = O.scan_rotation(geom, rg, rs, pair.ligand.xyz, w, rot, k, keep_corr=(i == 0),
                              workers=os.cpu_count() or 1)
        assert res.in_grid
        offs[i] = res.offsets
        scores[i] = res.scores
        if i == 0:
            corr0 = res.corr
        if top:
            cells = O.offsets_to_cells(res.offsets, n)
            records.append((rot, O.translation(cells, geom), res.scores))
    extra = {}
    if top:
        # Foreman gather over the per-rotation records: the `top` lowest
        # values, ascending, ties in arrival (rotation) order
        best = O.gather_records(records, top)
        rot_flat = rots.reshape(m, 9)
        extra = dict(top_value=np.array([v for v, _, _ in best]),
                     top_rot=np.array([int(np.nonzero((rot_flat == r.reshape(9)).all(1))[0][0]) for _, r, _ in best]),
                     top_t=np.array([t for _, _, t in best]))
    np.savez_compressed(
        os.path.join(HERE, name + ".npz"),
        rec_xyz=pair.receptor.xyz, rec_type=pair.receptor.ace_type,
        lig_xyz=pair.ligand.xyz, lig_type=pair.ligand.ace_type,
        ace=pair.ace, rotations=rots, grid_n=n, grid_step=H, term_set=term_set, k=k,
        offsets=offs, scores=scores,
        corr0=corr0.astype(np.float32) if n <= 48 else np.zeros(0, np.float32),
        **extra,
    )


if __name__ == "__main__":
    names = sys.argv[1:] or list(CASES)
    for name in names:
        make(name, **CASES[name])
        print("wrote", name)
