"""Training features on the GPU (mlipg_features) against the oracle.

The oracle restates the reference's prepare_features (structural, polynomial,
force and stress features) and is pinned to its own energy, forces and virial
through the linear model (tests/test_oracle.py).  Here the device path, FP64
on an image-coded device neighbour list of the periodic cell, matches it to
1e-10 of each array's scale on the three fitted regression potentials, and
reproduces the FP64 energy, forces and virial of the evaluation path
through E = sum_i P_i . w, F = FF . w, virial = SF . w.
"""
import numpy as np
import pytest

import mlipg
from conftest import structure
from mlipg.structures import build_system, fcc_cell, jitter, random_types
from oracle import Oracle

pytestmark = pytest.mark.gpu


def close(a, b, rel=1e-10):
    return np.abs(a - b).max() <= rel * max(np.abs(b).max(), 1e-300)


@pytest.mark.parametrize("pot", ["gtinv-820", "gtinv-434", "gtinv-197"])
def test_features_match_oracle(potdir, pot):
    cell = structure("structure.lammps")
    o = Oracle(potdir[pot], threads=16)
    s = build_system(cell, o.cutoff, skin=2.0)
    ref = o.features(s)
    g = mlipg.Potential(potdir[pot], mlipg.PREC_FP64)
    got = g.features(cell)
    for k in ("d", "p", "ff", "sf"):
        assert got[k].shape == ref[k].shape
        assert close(got[k], ref[k]), k
    # the linear model reproduces the evaluation path, to the rounding of the
    # contraction (fitted coefficients cancel: sum |w_p| |X_p| can exceed the
    # result by orders of magnitude, so the bound scales with that sum)
    w = o.coefficients()
    aw = np.abs(w)
    r = g.compute(s)
    P = got["p"].sum(0)
    assert abs(P @ w - r["energy"]) <= 1e-12 * (np.abs(P) @ aw)
    F = np.einsum("ipk,p->ik", got["ff"], w)
    Fs = np.einsum("ipk,p->ik", np.abs(got["ff"]), aw)
    assert np.all(np.abs(F - s.fold_forces(r["f_all"])) <= 1e-12 * Fs + 1e-14)
    v = w @ got["sf"]
    vs = aw @ np.abs(got["sf"])
    assert np.all(np.abs(v[[0, 1, 2, 5, 4, 3]] - r["virial"]) <= 1e-12 * vs[[0, 1, 2, 5, 4, 3]])


def test_features_subset_and_three_elements(tmp_path):
    """A ternary potential (orders to 4, l <= [4, 4, 2]) on a small
    random-element fcc cell, with only some outputs requested."""
    from mlipg.potential import gaussian_params, write_potential
    p = str(tmp_path / "tern.mlip")
    write_potential(p, ["A", "B", "C"], 5.0, gaussian_params(5, 5.0), 3, 2, 4, 4, [4, 4, 2],
                    [0, 0, 0], masses=[27.0, 58.7, 55.8], seed=4)
    rng = np.random.default_rng(3)
    cell = random_types(jitter(fcc_cell(2, 2, 2, 3.8), 0.08, rng), 3, rng)
    o = Oracle(p, threads=16)
    s = build_system(cell, o.cutoff, skin=1.0)
    ref = o.features(s)
    g = mlipg.Potential(p, mlipg.PREC_FP64)
    got = g.features(cell, want=("p", "sf"))
    assert set(got) == {"p", "sf"}
    assert close(got["p"], ref["p"]) and close(got["sf"], ref["sf"])
