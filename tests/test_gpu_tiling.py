"""Tile shapes of the fused kernel and the autotuner.

Every candidate tiling (terms per batched unit, warp dealing order, CTAs per
SM) evaluates the same physics: FP64 energies, forces and virials match the
oracle to 1e-10 relative for the two- and three-element potentials (the
three-element one exercises the slot-0 split of order-3 units); the mixed
path stays within 1e-4 eV/A RMS.  The autotuner times every candidate, keeps
the fastest, and an MD run whose tiling changes between two segments
re-captures its step graph and follows the unchanged trajectory.
"""
import numpy as np
import pytest

import mlipg
from mlipg.potential import workload_potential
from mlipg.structures import build_system, fcc_cell, jitter, random_triclinic_cell, random_types
from oracle import Oracle

pytestmark = pytest.mark.gpu

TILINGS = [(12, 0, 0), (12, 1, 1), (24, 1, 0), (48, 0, 1), (48, 1, 0), (24, 2, 0), (48, 2, 1)]


def rel(a, b):
    return np.abs(np.asarray(a) - np.asarray(b)).max() / max(np.abs(b).max(), 1e-300)


@pytest.fixture(scope="module", params=["triclinic-batch", "fcc-ternary-1m"])
def case(request, tmp_path_factory):
    pot = str(tmp_path_factory.mktemp("tiling") / (request.param + ".mlip"))
    workload_potential(pot, request.param, seed=3)
    rng = np.random.default_rng(4)
    if request.param == "triclinic-batch":
        cells = [random_triclinic_cell(n, 0.06, 2, rng) for n in (9, 24, 40)]
    else:
        cells = [random_types(jitter(fcc_cell(2, 2, 2, 4.0), 0.1, rng), 3, rng)]
    orc = Oracle(pot, threads=16)
    refs = []
    for c in cells:
        s = build_system(c, orc.cutoff)
        r = orc.compute(s)
        refs.append((r["energy"], s.fold_forces(r["f_all"]), r["virial"]))
    return pot, cells, refs


@pytest.mark.parametrize("tiling", TILINGS)
def test_tiling_fp64_matches_oracle(case, tiling):
    pot, cells, refs = case
    g = mlipg.Potential(pot, mlipg.PREC_FP64)
    g.set_tiling(*tiling)
    b = mlipg.Batch(g, cells)
    e, f, v = b.compute()
    for k, (er, fr, vr) in enumerate(refs):
        assert abs(e[k] - er) <= 1e-10 * abs(er)
        assert rel(f[b.offsets[k]:b.offsets[k + 1]], fr) <= 1e-10
        assert rel(v[k], vr) <= 1e-10
    g.set_precision(mlipg.PREC_MIXED)
    e, f, v = b.compute()
    for k, (er, fr, vr) in enumerate(refs):
        assert abs(e[k] - er) / cells[k].natoms <= 1e-6
        assert np.sqrt(np.mean((f[b.offsets[k]:b.offsets[k + 1]] - fr) ** 2)) <= 1e-4


def test_autotune_picks_fastest_and_keeps_parity(case):
    pot, cells, refs = case
    g = mlipg.Potential(pot, mlipg.PREC_FP64)
    b = mlipg.Batch(g, cells * 8)
    rows = b.autotune()
    assert len(rows) >= 6
    assert all(r["ms"] > 0 for r in rows)
    best = min(rows, key=lambda r: r["ms"])
    t = g.tiling()
    assert (t["irr_chunk"], t["warp_order"], t["ctas_per_sm"]) == \
        (best["irr_chunk"], best["warp_order"], best["ctas_per_sm"])
    e, f, v = mlipg.Batch(g, cells).compute()
    for k, (er, fr, vr) in enumerate(refs):
        assert abs(e[k] - er) <= 1e-10 * abs(er)


def test_md_recaptures_graph_after_tiling_change(case):
    pot, cells, _ = case
    cell = cells[-1]
    g = mlipg.Potential(pot, mlipg.PREC_FP64)
    m = np.array(g.masses)[cell.types]
    v0 = mlipg.maxwell_boltzmann(m, 300.0, np.random.default_rng(2))
    ref = mlipg.MD(g, cell, v0)
    ref.run(10, 0.001, True)
    x_ref, _, _ = ref.state()
    ref.close()
    md = mlipg.MD(g, cell, v0)
    md.run(5, 0.001, True)
    g.set_tiling(12, 1, 1)
    md.run(5, 0.001, True)
    x, _, _ = md.state()
    md.close()
    assert np.abs(x - x_ref).max() <= 1e-9


def test_md_autotune_keeps_trajectory(case):
    pot, cells, _ = case
    cell = cells[-1]
    g = mlipg.Potential(pot, mlipg.PREC_FP64)
    m = np.array(g.masses)[cell.types]
    v0 = mlipg.maxwell_boltzmann(m, 300.0, np.random.default_rng(8))
    ref = mlipg.MD(g, cell, v0)
    ref.run(6, 0.001, True)
    x_ref, v_ref, _ = ref.state()
    ref.close()
    md = mlipg.MD(g, cell, v0)
    md.run(3, 0.001, True)
    rows = md.autotune()
    assert len(rows) >= 6
    md.run(3, 0.001, True)
    x, v, _ = md.state()
    md.close()
    assert np.abs(x - x_ref).max() <= 1e-9
    assert np.abs(v - v_ref).max() <= 1e-8
