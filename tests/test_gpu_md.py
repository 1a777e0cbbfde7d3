"""NVE molecular dynamics on the device against the reference's trajectories.

The reference's regression runs (test/regression/{gtinv,pair}-*.in: read the
32-atom TiAl3 cell, `fix nve`, 100 steps of 1 fs) end in `dump.atom.*` and the
step-100 thermo line of their logs.  The FP64 path must reproduce the final
coordinates within the reference's own tolerance (mean |dx| < 1e-4 A,
test/regression/regression.py:9) and the printed thermo to its last printed
digit.  The stress run (5 fs steps) pins the pressure tensor at steps 50 and
100.
"""
import os

import numpy as np
import pytest

import mlipg
from conftest import GOLDEN, structure

pytestmark = pytest.mark.gpu


def read_dump(name):
    lines = open(os.path.join(GOLDEN, name)).read().splitlines()
    rows = sorted((int(l.split()[0]), [float(v) for v in l.split()[2:5]]) for l in lines[9:]
                  if l.strip())
    return np.array([r[1] for r in rows])


def run_nve(pot_path, nsteps, dt, skin=2.0, graph=True, prec=mlipg.PREC_FP64):
    g = mlipg.Potential(pot_path, prec)
    md = mlipg.MD(g, structure("structure.lammps"), skin=skin)
    md.run(nsteps, dt, graph=graph)
    x, v, f = md.state()
    th = md.thermo()
    md.close()
    return x, th


@pytest.mark.parametrize("pot", ["gtinv-820", "gtinv-434", "gtinv-197", "pair-60", "pair-17"])
def test_nve_100_steps_match_reference(potdir, golden, pot):
    x, th = run_nve(potdir[pot], 100, 0.001)
    ref = read_dump("dump.atom." + pot)
    assert np.abs(x - ref).mean() < 1e-4          # the reference's L1_TOL
    assert np.abs(x - ref).max() < 1e-6           # FP64 trajectories agree far closer
    g = golden["nve"][pot]["rows"]["100"]
    assert th["temp"] == pytest.approx(g["Temp"], abs=1e-4)
    assert th["pe"] == pytest.approx(g["E_pair"], abs=1e-5)
    assert th["etotal"] == pytest.approx(g["TotEng"], abs=1e-5)
    assert th["press"] == pytest.approx(g["Press"], abs=2e-3)


def test_nve_stress_run(potdir, golden):
    rows = golden["nve"]["gtinv-197-stress"]["rows"]
    g = mlipg.Potential(potdir["gtinv-197"], mlipg.PREC_FP64)
    md = mlipg.MD(g, structure("structure.lammps"), skin=2.0)
    for step in (50, 100):
        md.run(50, 0.005)
        th = md.thermo()
        r = rows[str(step)]
        for k, key in [("pxx", "Pxx"), ("pyy", "Pyy"), ("pzz", "Pzz"), ("pxy", "Pxy"),
                       ("pxz", "Pxz"), ("pyz", "Pyz")]:
            assert th[k] == pytest.approx(r[key], abs=2e-3), (step, key)
        assert th["temp"] == pytest.approx(r["Temp"], abs=1e-4)
        assert th["etotal"] == pytest.approx(r["TotEng"], abs=1e-5)
    md.close()


def test_graph_equals_eager_and_rebuilds_keep_physics(potdir):
    xg, tg = run_nve(potdir["gtinv-820"], 30, 0.002, graph=True)
    xe, te = run_nve(potdir["gtinv-820"], 30, 0.002, graph=False)
    np.testing.assert_allclose(xg, xe, rtol=0, atol=1e-10)
    assert tg["etotal"] == pytest.approx(te["etotal"], abs=1e-10)
    # a tiny skin forces list rebuilds (positions are re-wrapped into the cell)
    xs, ts = run_nve(potdir["gtinv-820"], 30, 0.002, skin=0.02, graph=True)
    assert ts["rebuilds"] >= 1
    cell = structure("structure.lammps")
    d = (xs - xg) @ np.linalg.inv(cell.lattice)
    d -= np.round(d)
    assert np.abs(d @ cell.lattice).max() < 1e-9
    assert ts["etotal"] == pytest.approx(tg["etotal"], abs=1e-9)


def test_nve_energy_conservation_mixed(potdir):
    """Velocity Verlet itself moves the total energy of this cell by ~1e-5
    eV/atom per 100 steps (the reference's own FP64 log: TotEng -135.40507 ->
    -135.40539), so the mixed run's drift is compared with the FP64 run's:
    the FP32 adjoint products may add no more than the integrator's own drift
    scale, 2e-5 eV/atom over 200 steps (measured: ~6e-6)."""
    drift = {}
    for prec in (mlipg.PREC_FP64, mlipg.PREC_MIXED):
        _, t0 = run_nve(potdir["gtinv-820"], 1, 0.001, prec=prec)
        _, t1 = run_nve(potdir["gtinv-820"], 200, 0.001, prec=prec)
        drift[prec] = (t1["etotal"] - t0["etotal"]) / 32
    assert abs(drift[mlipg.PREC_MIXED] - drift[mlipg.PREC_FP64]) < 2e-5
    assert abs(drift[mlipg.PREC_FP64]) < 5e-5
