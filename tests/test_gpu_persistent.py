"""Persistent PCG kernels (one cooperative launch per iteration tail, or per
group of whole FP64 iterations, with grid-wide barriers) against the
separate scatter/update/finish kernels of p121.f90:90-104: the iterates,
the stopping iteration and the final residual must be bitwise the same.
Also the error path of the bounded bulk-copy waits."""
import numpy as np
import pytest

import parafem_gb300 as P

pytestmark = pytest.mark.gpu


def _solve(prob, mode, persistent, graphs=True, tol=1e-8, limit=20000, material=(100.0, 0.3), shared=False):
    with P.Solver() as s:
        s.setup(prob["g_num"], prob["g_g"], prob["g_coord"], prob["nn"], prob["neq"])
        s.set_material(*material)
        if shared:
            s.set_shared_km(s.form_km(1, 27))
        else:
            s.form_storkm(27)
            s.set_tuning(0)
        s.set_persistent(persistent)
        s.set_graphs(graphs)
        x, it, rel = s.solve(prob["r"], tol, limit, mode)
        return x, it, rel


def _same(a, b):
    assert a[1] == b[1], (a[1], b[1])
    assert a[2] == b[2], (a[2], b[2])
    assert np.array_equal(a[0], b[0])


@pytest.mark.parametrize("mode", [P.MODE_P121, P.MODE_FP64_RES, P.MODE_MIXED, P.MODE_MIXED16])
def test_persistent_iterates_bitwise_equal_separate_kernels(mode):
    prob = P.cube_problem(7, 6, 5)
    tol = 1e-6 if mode == P.MODE_P121 else 1e-8
    _same(_solve(prob, mode, True, tol=tol), _solve(prob, mode, False, tol=tol))


def test_persistent_without_graphs_and_heterogeneous_material():
    prob = P.cube_problem(6, 6, 6)
    nels = 6 ** 3
    mat = P.random_material(nels, 7, 1.0, 1000.0, 0.2, 0.35)
    a = _solve(prob, P.MODE_MIXED, True, graphs=False, material=mat)
    b = _solve(prob, P.MODE_MIXED, False, graphs=True, material=mat)
    _same(a, b)


def test_persistent_shared_km_mixed_and_fp64():
    prob = P.cube_problem(8, 8, 8)
    for mode in (P.MODE_MIXED, P.MODE_FP64_RES):
        _same(_solve(prob, mode, True, shared=True), _solve(prob, mode, False, shared=True))


def test_persistent_more_virtual_blocks_than_resident_blocks():
    """26^3: 213k slots, so the vector kernels have more 256-slot blocks than
    a cooperative launch holds, and each block runs several of them; the
    limit (37) ends the run inside a launch of whole FP64 iterations."""
    prob = P.cube_problem(26, 26, 26)
    for mode in (P.MODE_FP64_RES, P.MODE_P121):
        a = _solve(prob, mode, True, tol=1e-30, limit=37)
        b = _solve(prob, mode, False, tol=1e-30, limit=37)
        assert a[1] == 37
        _same(a, b)


def test_persistent_p121_demo_matches_oracle(demo_problem):
    """The demo deck (98,360 equations, nip 8) through the persistent FP64
    iterations against the C restatement, at the golden iteration."""
    from oracle import oracle as O
    dp = demo_problem
    d = dp["deck"]
    it_ref, x_ref, _ = O.pcg(dp["g_g"], dp["km"], dp["diag"], dp["r"], 0.0, 295, 0)
    with P.Solver() as s:
        gc = dp["gc"]
        s.setup(d.g_num, dp["g_g"], gc, d.nn, dp["neq"])
        s.set_material(d.e, d.v)
        s.form_storkm(d.nip)
        s.set_persistent(True)
        x, it, _ = s.solve(dp["r"], 0.0, 295, P.MODE_P121)
    assert it == 295 == it_ref
    assert np.abs(x - x_ref).max() <= 1e-6 * np.abs(x_ref).max()


def test_bounded_wait_timeout_is_reported_and_context_recovers():
    prob = P.cube_problem(4, 4, 4)
    with P.Solver() as s:
        s.setup(prob["g_num"], prob["g_g"], prob["g_coord"], prob["nn"], prob["neq"])
        s.set_material(100.0, 0.3)
        s.form_storkm(27)
        x0, it0, _ = s.solve(prob["r"], 1e-8, 5000, P.MODE_MIXED)
        rc, msg = s.check_wait_timeout(64)
        assert rc != 0
        assert "bulk-copy wait timed out (code 2)" in msg
        x1, it1, rel1 = s.solve(prob["r"], 1e-8, 5000, P.MODE_MIXED)
        assert it1 == it0 and rel1 <= 1e-8
        assert np.array_equal(x0, x1)
