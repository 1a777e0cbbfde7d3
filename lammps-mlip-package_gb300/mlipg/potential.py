"""Writer for potential files in the reference's ``mlp.lammps`` format.

Line layout read by the reference parser (mlipkk_potential_parser.cpp:14-105):
elements + "# element", cutoff, pair_type, des_type, model_type, max_p,
max_l, gtinv_order, gtinv_maxl, gtinv_sym, number of coefficients,
coefficients, scales, number of radial parameters, one "beta mu" line each,
masses.  Synthetic potentials for the benchmark workloads are written with
seeded N(0, sigma) coefficients and unit scales.
"""
from __future__ import annotations

import numpy as np

from . import count_coefficients


def write_potential(path, elements, cutoff, params, model_type, maxp, maxl, gtinv_order,
                    gtinv_maxl, gtinv_sym, coeffs=None, masses=None, seed=0, sigma=1e-3):
    n_fn = len(params)
    nc, _ = count_coefficients(len(elements), model_type, maxp, maxl, gtinv_order, gtinv_maxl,
                               gtinv_sym, n_fn)
    if coeffs is None:
        coeffs = np.random.default_rng(seed).normal(0.0, sigma, nc)
    coeffs = np.asarray(coeffs, dtype=np.float64)
    if coeffs.size != nc:
        raise ValueError("model needs %d coefficients, got %d" % (nc, coeffs.size))
    if masses is None:
        masses = [1.0] * len(elements)
    lines = [
        " ".join(elements) + " # element",
        "%r # cutoff" % float(cutoff),
        "gaussian # pair_type",
        "gtinv # des_type",
        "%d # model_type" % model_type,
        "%d # max_p" % maxp,
        "%d # max_l" % maxl,
        "%d # gtinv_order" % gtinv_order,
        " ".join(str(int(v)) for v in gtinv_maxl) + "  # gtinv_maxl",
        " ".join(str(int(v)) for v in gtinv_sym) + "  # gtinv_sym",
        "%d # number of regression coefficients" % nc,
        " ".join("%.17g" % v for v in coeffs) + "  # reg. coeffs",
        " ".join("1" for _ in range(nc)) + "  # scales",
        "%d # number of parameters" % n_fn,
    ]
    for b, m in params:
        lines.append("%.17g %.17g # pair func. params" % (b, m))
    lines.append(" ".join("%.17g" % m for m in masses) + "  # atomic mass")
    with open(path, "w") as f:
        f.write("\n".join(lines) + "\n")
    return nc


def gaussian_params(n, rmax, beta=1.0):
    """n Gaussians with centres linspace(0, rmax, n) and a common width beta."""
    return [(beta, float(m)) for m in np.linspace(0.0, rmax, n)]


# Potentials of the benchmark workloads (synthetic weights, seeded).
def workload_potential(path, name, seed=1):
    """Writes the potential of a named workload; returns its coefficient count.

    fcc-al-256:       1 element, rc 6, 10 Gaussians, order 3, l <= [4, 4],
                      model_type 2, max_p 2 (linear + 2nd-order polynomial)
    bcc-binary-16k:   2 elements, rc 6, 15 Gaussians, order 4, l <= [12, 8, 4],
                      model_type 3, max_p 2 (pair-feature quadratic terms;
                      model_type 2 would need ~9e7 coefficients)
    fcc-ternary-1m:   the bcc-binary potential with 3 elements
    triclinic-batch:  the bcc-binary potential truncated to order 3, l <= [12, 8]
    """
    if name == "fcc-al-256":
        return write_potential(path, ["Al"], 6.0, gaussian_params(10, 6.0), 2, 2, 4, 3, [4, 4],
                               [0, 0], masses=[27.0], seed=seed)
    if name == "bcc-binary-16k":
        return write_potential(path, ["A", "B"], 6.0, gaussian_params(15, 6.0), 3, 2, 12, 4,
                               [12, 8, 4], [0, 0, 0], masses=[55.845, 58.693], seed=seed)
    if name == "fcc-ternary-1m":
        return write_potential(path, ["A", "B", "C"], 6.0, gaussian_params(15, 6.0), 3, 2, 12, 4,
                               [12, 8, 4], [0, 0, 0], masses=[26.98, 58.69, 55.85], seed=seed)
    if name == "triclinic-batch":
        return write_potential(path, ["A", "B"], 6.0, gaussian_params(15, 6.0), 3, 2, 12, 3,
                               [12, 8], [0, 0], masses=[55.845, 58.693], seed=seed)
    raise ValueError("unknown workload " + name)
