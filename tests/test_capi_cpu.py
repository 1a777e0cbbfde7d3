"""C-ABI library checks that need no GPU: symbols, model structure, errors."""
import ctypes
import hashlib
import os
import re

import numpy as np
import pytest

import mlipg
from conftest import REPO


def header_functions():
    text = open(os.path.join(REPO, "include", "mlipg.h")).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(mlipg_[a-z0-9_]+)\s*\(", text)))


def test_library_exports_every_declared_symbol():
    L = mlipg.lib()
    names = header_functions()
    assert len(names) >= 15
    for n in names:
        assert hasattr(L, n), n


def test_model_structure_matches_reference(potdir, golden):
    for pot, fp in golden["model"].items():
        p = mlipg.Potential(potdir[pot])
        for k, key in [("n_irreps", "n_irreps"), ("n_terms", "n_terms"), ("ITC", "ITC"),
                       ("D", "D"), ("n_coeffs", "n_coeffs"), ("T", "T"), ("F", "F")]:
            assert p.info[k] == fp[key], (pot, k)
        assert hashlib.sha256(p.itc_list().astype(np.int64).tobytes()).hexdigest() == \
            fp["itc_sha256"]
        assert hashlib.sha256(p.poly_list().astype(np.int64).tobytes()).hexdigest() == \
            fp["poly_sha256"]
        # every conjugate pair folded into one canonical term
        assert p.info["n_folded_terms"] <= p.info["n_terms"]


@pytest.mark.parametrize("spec,expected", [
    # (T, model_type, maxp, maxl, order, gtinv_maxl, sym, n_fn) -> (C, D)
    ((1, 2, 2, 4, 3, [4, 4], [0, 0], 10), (20300, 200)),
    ((2, 3, 2, 12, 4, [12, 8, 4], [0, 0, 0], 15), (14340, 13530)),
    ((3, 3, 2, 12, 4, [12, 8, 4], [0, 0, 0], 15), (68535, 65790)),
    ((2, 3, 2, 12, 3, [12, 8], [0, 0], 15), (11805, 10995)),
])
def test_count_coefficients_workloads(spec, expected):
    assert mlipg.count_coefficients(*spec) == expected


def test_count_matches_regression_potentials(potdir, golden):
    # gtinv-197: 2 el, model_type 2, max_p 2, max_l 4, order 2, [4]
    assert mlipg.count_coefficients(2, 2, 2, 4, 2, [4], [0], 15)[0] == \
        golden["model"]["gtinv-197"]["n_coeffs"]
    assert mlipg.count_coefficients(2, 3, 3, 4, 4, [4, 4, 2], [0, 0, 0], 10)[0] == \
        golden["model"]["gtinv-820"]["n_coeffs"]
    assert mlipg.count_coefficients(2, 4, 2, 0, 3, [0, 0], [0, 0], 15)[0] == \
        golden["model"]["gtinv-434"]["n_coeffs"]


def test_type_map_semantics(potdir):
    p = mlipg.Potential(potdir["gtinv-820"])
    assert p.elements == ["Ti", "Al"]
    assert p.masses == pytest.approx([47.88, 26.98])
    assert p.cutoff == 6.0
    p.set_type_map(["Al", "Ti", "NULL"])
    with pytest.raises(mlipg.MlipgError, match="No matching element"):
        p.set_type_map(["Ti", "Xx"])
    with pytest.raises(mlipg.MlipgError, match="Incorrect args"):
        p.set_type_map(["NULL", "NULL"])


def test_precision_values(potdir):
    """The four precisions are accepted at creation and by set_precision;
    anything else is EINVAL and leaves the handle as it was."""
    for prec in (mlipg.PREC_FP64, mlipg.PREC_MIXED, mlipg.PREC_MIXED_A64,
                 mlipg.PREC_FP64_NATIVE):
        p = mlipg.Potential(potdir["gtinv-434"], prec)
        p.set_precision(mlipg.PREC_MIXED_A64)
        p.set_precision(prec)
        for bad in (-1, 4):
            with pytest.raises(mlipg.MlipgError) as e:
                p.set_precision(bad)
            assert e.value.code == 1
        p.close()
    with pytest.raises(mlipg.MlipgError) as e:
        mlipg.Potential(potdir["gtinv-434"], 4)
    assert e.value.code == 1


def test_bad_potential_files(tmp_path):
    with pytest.raises(mlipg.MlipgError) as e:
        mlipg.Potential(str(tmp_path / "missing.mlip"))
    assert e.value.code == 2
    bad = tmp_path / "bad.mlip"
    bad.write_text("A # element\n6.0\ngaussian\nspline\n")
    with pytest.raises(mlipg.MlipgError, match="des_type"):
        mlipg.Potential(str(bad))
    # a radial-only (pair) file cut short
    bad.write_text("A # element\n6.0\ngaussian\npair\n")
    with pytest.raises(mlipg.MlipgError) as e:
        mlipg.Potential(str(bad))
    assert e.value.code == 2


def test_pair_potential_model(potdir):
    """Radial-only potentials load without a GPU: the legacy enumeration gives
    the file's coefficient count (pair-60: 60 features, 1,430 pair and 21,420
    triple terms; pair-17: 30 features squared and cubed)."""
    for name, d, c in (("pair-60", 60, 22910), ("pair-17", 30, 90)):
        p = mlipg.Potential(potdir[name])
        assert p.info["D"] == d and p.info["n_coeffs"] == c
        assert p.elements == ["Ti", "Al"]


@pytest.mark.skipif(os.environ.get("CUDA_VISIBLE_DEVICES") is None and
                    os.path.exists("/dev/nvidia0"), reason="a GPU is present")
def test_compute_without_gpu_fails_loudly(potdir):
    p = mlipg.Potential(potdir["gtinv-434"])
    with pytest.raises(mlipg.MlipgError) as e:
        p.compute_lammps(1, 1, np.zeros((1, 3)), [1], [0], [0], [np.zeros(0, np.int32)])
    assert e.value.code == 7


def test_tiling_candidates_build_on_host(tmp_path):
    """Every autotuner candidate builds a schedule that covers each feature once
    (the library checks coverage and fails otherwise); invalid shapes are
    rejected and leave the previous tiling in place."""
    import mlipg
    from mlipg.potential import workload_potential
    for name in ("fcc-ternary-1m", "triclinic-batch", "fcc-al-256"):
        p = str(tmp_path / (name + ".mlip"))
        workload_potential(p, name)
        g = mlipg.Potential(p, mlipg.PREC_MIXED)
        for chunk in (12, 24, 48):
            for order in (0, 1, 2):
                g.set_tiling(chunk, order, 1)
                assert g.tiling() == {"irr_chunk": chunk, "warp_order": order, "ctas_per_sm": 1}
        for bad in ((13, 0, 0), (24, 3, 0), (24, 0, -1), (0, 0, 0)):
            with pytest.raises(mlipg.MlipgError):
                g.set_tiling(*bad)
        assert g.tiling()["irr_chunk"] == 48
        g.close()
