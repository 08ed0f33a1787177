"""GPU: EPSGB300Server, the continuous-batching request loop.

Requests arrive while others are on the GPU and join them at the next restart cycle; the HBM budget bounds the
admitted footprint; every result is bit-identical to the same problem solved alone (a batch of one) -- the served
form changes when work runs, not what it computes."""
import threading
import time

import numpy as np
import pytest

import slepc_gb300 as sg
from slepc_gb300 import matgen

pytestmark = pytest.mark.gpu


def make(csr, hermitian, which, nev, ncv, tol, seed):
    A = sg.Mat(*csr)
    eps = sg.EPS().create()
    eps.setOperators(A)
    eps.setProblemType(sg.EPS.ProblemType.HEP if hermitian else sg.EPS.ProblemType.NHEP)
    eps.setDimensions(nev, ncv)
    eps.setTolerances(tol)
    eps.setWhichEigenpairs(which)
    eps.setInitialSpace(matgen.start_vector(len(csr[0]) - 1, seed))
    eps._A = A
    return eps


def results(eps):
    n = eps._A.m
    vals, vecs = [], []
    for i in range(eps.getConverged()):
        x = np.zeros(n)
        vals.append(eps.getEigenpair(i, x))
        vecs.append(x)
    return eps.getConverged(), eps.getIterationNumber(), eps.getConvergedReason(), vals, vecs


def requests():
    out = []
    for i, n in enumerate([2000, 5000, 9000, 3000, 12000, 2500]):
        nev = 4 + 3 * i
        out.append((matgen.laplacian_2d_randdiag(n, 50 + i), True, "LR", nev, max(2 * nev + 8, 24), 1e-10, 70 + i))
    out.append((matgen.convection_diffusion_2d(50, 25.0), False, "LR", 6, 24, 1e-10, 80))
    out.append((matgen.laplacian_3d_randdiag(18, 81), True, "LR", 10, 28, 1e-10, 82))
    return out


def test_served_equals_alone(lib):
    reqs = requests()
    alone = []
    for p in reqs:
        e = make(*p)
        sg.solve_batch([e])
        alone.append(results(e))
    srv = sg.Server(hbm_budget_bytes=8e9, max_requests=64, max_ncv=48)
    try:
        served = [make(*p) for p in reqs]
        # staggered arrivals from two client threads: later requests join solves already on the GPU
        def client(idx, delay):
            for k in idx:
                time.sleep(delay)
                srv.submit(served[k])
        t1 = threading.Thread(target=client, args=([0, 2, 4, 6], 0.01))
        t2 = threading.Thread(target=client, args=([1, 3, 5, 7], 0.015))
        t1.start(); t2.start(); t1.join(); t2.join()
        for e in served:
            assert srv.wait(e, timeout=120.0)
        st = srv.stats()
        assert st["completed"] == len(reqs) and st["failed"] == 0
        assert st["max_live"] >= 2  # the solves did overlap on the device
    finally:
        srv.destroy()
    for a, e in zip(alone, served):
        r = results(e)
        assert r[0] == a[0] and r[1] == a[1] and r[2] == a[2] == 1
        assert r[3] == a[3]
        for xa, xb in zip(a[4], r[4]):
            assert np.array_equal(xa, xb)
        assert e.getStats()["solve_seconds"] > 0.0


def test_server_budget_admission(lib):
    reqs = requests()[:6]
    eps = [make(*p) for p in reqs]
    # footprint n (ncv+1) 8 + nnz 12 of the two largest requests
    foot = sorted(((len(p[0][0]) - 1) * (p[4] + 1) * 8 + len(p[0][1]) * 12 for p in reqs))
    budget = foot[-1] + foot[-2]
    srv = sg.Server(hbm_budget_bytes=budget, max_requests=64, max_ncv=48)
    try:
        for e in eps:
            srv.submit(e)
        for e in eps:
            assert srv.wait(e, timeout=120.0)
        st = srv.stats()
        assert st["completed"] == len(eps)
        assert st["peak_bytes"] <= budget
        assert st["bytes_in_use"] == 0.0
    finally:
        srv.destroy()
    for e in eps:
        assert e.getConvergedReason() == 1


def test_server_two_lanes(lib):
    """Small and large requests run in separate lanes (engines, graphs, streams) under one budget: each result is
    bit-identical to the same problem solved alone, and the admitted footprint of both lanes together stays within
    the budget while the large requests' reservation keeps the small ones from starving them."""
    small = requests()[:4]
    large = [(matgen.laplacian_3d_randdiag(64, 90 + i), True, "LR", 6, 24, 1e-10, 92 + i) for i in range(2)]
    reqs = [small[0], large[0], small[1], small[2], large[1], small[3]]

    def foot(p):
        return (len(p[0][0]) - 1) * (p[4] + 1) * 8 + len(p[0][1]) * 12

    assert min(foot(p) for p in large) > 64 * 1024 * 1024 >= max(foot(p) for p in small)
    alone = []
    for p in reqs:
        e = make(*p)
        sg.solve_batch([e])
        alone.append(results(e))
    budget = max(foot(p) for p in large) + 2 * max(foot(p) for p in small)
    srv = sg.Server(hbm_budget_bytes=budget, max_requests=16, max_ncv=48)
    try:
        served = [make(*p) for p in reqs]
        for e in served:
            srv.submit(e)
        for e in served:
            assert srv.wait(e, timeout=300.0)
        st = srv.stats()
        assert st["completed"] == len(reqs) and st["failed"] == 0
        assert st["peak_bytes"] <= budget and st["bytes_in_use"] == 0.0
    finally:
        srv.destroy()
    for a, e in zip(alone, served):
        r = results(e)
        assert r[0] == a[0] and r[1] == a[1] and r[2] == a[2] == 1
        assert r[3] == a[3]
        for xa, xb in zip(a[4], r[4]):
            assert np.array_equal(xa, xb)
