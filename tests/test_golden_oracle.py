"""The committed golden fixtures still reproduce from the oracle (CPU)."""
from pathlib import Path

import numpy as np
import pytest

from oracle import fftdock_oracle as O

GOLDEN = Path(__file__).resolve().parent / "golden"


@pytest.mark.parametrize("name", sorted(p.stem for p in GOLDEN.glob("*.npz")))
def test_golden_fixture_reproduces(name):
    f = np.load(GOLDEN / (name + ".npz"))
    n = int(f["grid_n"])
    geom = O.Geometry.centred(float(f["grid_step"]), n)
    tp = O.TermParams(term_set=int(f["term_set"]), ace_matrix=f["ace"])
    rg = O.receptor_terms(geom, f["rec_xyz"], f["rec_type"], tp)
    rs = O.receptor_spectra(rg)
    w = O.ligand_term_weights(f["lig_type"], tp)
    k = int(f["k"])
    for i, rot in enumerate(f["rotations"]):
        res = O.scan_rotation(geom, rg, rs, f["lig_xyz"], w, rot, k)
        assert np.array_equal(res.offsets, f["offsets"][i])
        assert np.allclose(res.scores, f["scores"][i], rtol=1e-12, atol=1e-9)
        # every fixture score is the exact direct-space energy of its cell
        cells, _ = O.bin_ligand(geom, rot, f["lig_xyz"])
        for off, s in zip(f["offsets"][i], f["scores"][i]):
            c = O.offsets_to_cells([off], n)[0]
            assert abs(O.direct_score(rg, cells, w, c) - s) <= 1e-9 * max(1.0, abs(s))
