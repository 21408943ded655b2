"""Golden fixtures (tests/golden/, made by make_golden.py from the oracle): the oracle must
reproduce them on the CPU, and the CUDA path must match them on the GPU."""
import sys
from pathlib import Path

import numpy as np
import pytest

from _util import rel

GOLD = Path(__file__).resolve().parent / "golden" / "oracle_cylinder_64x48.npz"
sys.path.insert(0, str(GOLD.parent))


@pytest.fixture(scope="module")
def gold():
    return dict(np.load(GOLD))


def test_oracle_reproduces_golden(gold):
    import make_golden as mg
    fresh = mg.cylinder_case()
    for k in ("gamma", "psi", "q", "fb", "cd", "cl", "bmat"):
        assert rel(fresh[k], gold[k]) < 1e-12, k
    kat = mg.kat_vectors()
    for k in kat:
        assert rel(kat[k], gold[k]) < 1e-12, k
    # the parity bar presumes a well-conditioned Schur matrix (points spaced ~h)
    assert np.linalg.cond(gold["bmat"]) < 1e7
    # analytic answers
    assert rel(gold["kat_lap_inv"], gold["kat_expected_lap_inv"]) < 1e-13
    d = gold["kat_dst"]
    assert abs(d[1, 2] - 4 * 24 * 20 / 4) < 1e-10 and np.sum(np.abs(d)) - abs(d[1, 2]) < 1e-9


@pytest.mark.gpu
def test_cuda_matches_golden(ib, gold):
    nx, ny, L = int(gold["nx"]), int(gold["ny"]), int(gold["L"])
    h = float(gold["h"])
    x0, y0 = float(gold["x0"]), float(gold["y0"])
    grid = ib.MultiLevel(ib.UniformGrid(h, (x0, x0 + nx * h), (y0, y0 + ny * h)), L)
    body = ib.RigidBody(ib.GridFrame(), gold["xb"], gold["ds"])
    prob = ib.Problem(ib.StreamFcnFluid(grid, (1.0, 0.0), float(gold["Re"])), ib.BodyGroup(body),
                      ib.SchemeCNAB(float(gold["dt"])))
    st = ib.initstate(prob)
    st._gamma[:] = gold["gamma0"].reshape(L, -1)
    s = ib.initsolver(prob, st)
    s.vort2flux(st)
    cd = []
    for i in range(len(gold["cd"])):
        ib.advance_(st, s, i * float(gold["dt"]))
        cd.append(st.qty.stress[0].CD)
    assert rel(st.qty.gamma, gold["gamma"].reshape(L, -1)) < 1e-10
    assert rel(st.qty.psi, gold["psi"].reshape(L, -1)) < 1e-10
    assert rel(st.qty.q, gold["q"]) < 1e-10
    assert np.max(np.abs(np.array(cd) - gold["cd"]) / np.maximum(1, np.abs(gold["cd"]))) < 1e-8
    s.close()
