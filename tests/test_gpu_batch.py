"""Batched cells (one persistent launch over many periodic cells) vs the oracle.

Cells are small random triclinic cells (8-64 atoms, many narrower than twice
the cutoff, so atoms see their own periodic images) with the order-3,
l <= [12, 8] two-element potential of the batched workload.  FP64: energy,
forces and virial of every cell agree with the oracle (ghost-atom form) to
1e-10 relative; a cell's result does not depend on the rest of the batch.
"""
import numpy as np
import pytest

import mlipg
from mlipg.potential import workload_potential
from mlipg.structures import build_system, random_triclinic_cell
from oracle import Oracle

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def setup(tmp_path_factory):
    d = tmp_path_factory.mktemp("batch")
    pot = str(d / "tric.mlip")
    workload_potential(pot, "triclinic-batch", seed=5)
    rng = np.random.default_rng(11)
    sizes = [8, 9, 12, 17, 24, 31, 40, 64, 10, 50, 8, 20]
    cells = [random_triclinic_cell(n, 0.06, 2, rng) for n in sizes]
    orc = Oracle(pot, threads=16)
    refs = []
    for c in cells:
        s = build_system(c, orc.cutoff)
        r = orc.compute(s)
        refs.append((r["energy"], s.fold_forces(r["f_all"]), r["virial"]))
    return pot, cells, refs


def rel(a, b):
    return np.abs(np.asarray(a) - np.asarray(b)).max() / max(np.abs(b).max(), 1e-300)


def test_batch_fp64_matches_oracle(setup):
    pot, cells, refs = setup
    b = mlipg.Batch(mlipg.Potential(pot, mlipg.PREC_FP64), cells)
    e, f, v = b.compute()
    for k, (er, fr, vr) in enumerate(refs):
        fk = f[b.offsets[k]:b.offsets[k + 1]]
        assert abs(e[k] - er) <= 1e-10 * abs(er), k
        assert rel(fk, fr) <= 1e-10, k
        assert rel(v[k], vr) <= 1e-10, k


def test_batch_mixed_accuracy(setup):
    pot, cells, refs = setup
    b = mlipg.Batch(mlipg.Potential(pot, mlipg.PREC_MIXED), cells)
    e, f, v = b.compute()
    for k, (er, fr, vr) in enumerate(refs):
        fk = f[b.offsets[k]:b.offsets[k + 1]]
        assert abs(e[k] - er) / cells[k].natoms <= 1e-6
        assert np.sqrt(np.mean((fk - fr) ** 2)) <= 1e-4


def test_cell_alone_equals_cell_in_batch(setup):
    pot, cells, _ = setup
    g = mlipg.Potential(pot, mlipg.PREC_FP64)
    e_all, f_all, v_all = mlipg.Batch(g, cells).compute()
    for k in (0, 5, 7):
        e1, f1, v1 = mlipg.Batch(g, [cells[k]]).compute()
        assert e1[0] == pytest.approx(e_all[k], rel=1e-12)
        off = np.concatenate([[0], np.cumsum([c.natoms for c in cells])])
        np.testing.assert_allclose(f1, f_all[off[k]:off[k + 1]], rtol=0, atol=1e-11)
