"""Serving loop: continuous batching of differently sized requests.

Each request's result in the mix (many requests in flight, FP64 and mixed
interleaved) equals the same structure evaluated alone: energies to 1e-13
relative (they are reduced per cell in a fixed order), forces and virials to
1e-12 of the force / virial scale in FP64 and 1e-7 in the mixed path.  Both
accumulate the adjoint in exact fixed point whose scale adapts from the
centres a CTA ran before, which depend on the batch: the FP64 precision's
double-float flushes are rounded 64 bits below the CTA's largest flush (far
below FP64 rounding; the FP64 force scatter's order differs too), the mixed
path's FP32 flushes 31 .. 37 bits below it (measured differences up to 1.2e-8
of the force scale, below the 6e-8 rounding of the FP32 products
themselves).
"""
import threading

import numpy as np
import pytest

import mlipg
from mlipg.potential import workload_potential
from mlipg.structures import random_triclinic_cell

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def pot(tmp_path_factory):
    p = str(tmp_path_factory.mktemp("serve") / "tric.mlip")
    workload_potential(p, "triclinic-batch", seed=9)
    return p


def cells(n, seed):
    rng = np.random.default_rng(seed)
    sizes = np.exp(rng.uniform(np.log(16), np.log(160), n)).astype(int)
    return [random_triclinic_cell(int(k), 0.06, 2, rng) for k in sizes]


_pots = {}


def alone(pot, cell, prec):
    if prec not in _pots:
        _pots[prec] = mlipg.Potential(pot, prec)
    b = mlipg.Batch(_pots[prec], [cell])
    e, f, v = b.compute()
    b.close()
    return e[0], f, v[0]


def test_results_in_the_mix_equal_alone(pot):
    cs = cells(24, 3)
    precs = [mlipg.PREC_FP64 if k % 2 else mlipg.PREC_MIXED for k in range(len(cs))]
    srv = mlipg.Server(pot, budget_bytes=1 << 30, max_batch_atoms=600)
    tickets = []
    # submit from two threads to interleave arrivals
    lock = threading.Lock()

    def submit(idx):
        for k in idx:
            t = srv.submit(cs[k], precs[k])
            with lock:
                tickets.append((k, t))

    th = [threading.Thread(target=submit, args=(range(i, len(cs), 2),)) for i in range(2)]
    for t in th:
        t.start()
    for t in th:
        t.join()
    res = {k: srv.wait(t) for k, t in tickets}
    st = srv.stats()
    srv.close()
    assert st["completed"] == len(cs)
    assert st["batches"] >= 2
    for k, c in enumerate(cs):
        e, f, v = res[k]
        e1, f1, v1 = alone(pot, c, precs[k])
        assert abs(e - e1) <= 1e-13 * abs(e1)
        tol = 1e-12 if precs[k] == mlipg.PREC_FP64 else 1e-7
        assert np.abs(f - f1).max() <= tol * max(np.abs(f1).max(), 1e-30)
        assert np.abs(v - v1).max() <= tol * max(np.abs(v1).max(), 1e-30)


def test_tiny_budget_still_completes(pot):
    cs = cells(10, 4)
    srv = mlipg.Server(pot, budget_bytes=200_000, max_batch_atoms=100000)
    tk = [srv.submit(c, mlipg.PREC_MIXED) for c in cs]
    out = [srv.wait(t) for t in tk]
    st = srv.stats()
    srv.close()
    assert st["completed"] == len(cs)
    assert st["batches"] >= 5          # the budget forces small batches
    for (e, f, v), c in zip(out, cs):
        assert f.shape == (c.natoms, 3) and np.isfinite(e)


def test_unknown_ticket_and_deadline(pot):
    srv = mlipg.Server(pot, budget_bytes=1 << 30)
    with pytest.raises(mlipg.MlipgError):
        srv.wait(12345, timeout_ms=10)
    srv.close()
