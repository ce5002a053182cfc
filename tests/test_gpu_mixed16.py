"""PF_MODE_MIXED16: the mixed solver with FP16 storkm (scaled per element) in
its inner products, and pf_ebe_matvec prec 16."""
import numpy as np
import pytest

import parafem_gb300 as P

pytestmark = pytest.mark.gpu


def cube_solver(n, hetero):
    prob = P.cube_problem(n, n, n)
    nels = prob["g_num"].shape[0]
    if hetero:
        e, v = P.random_material(nels, 2024, 1.0, 1000.0, 0.2, 0.35)
    else:
        e, v = np.array([100.0]), np.array([0.3])
    s = P.Solver()
    s.setup(prob["g_num"], prob["g_g"], prob["g_coord"], prob["nn"], prob["neq"])
    s.set_material(e, v)
    s.form_storkm(27)
    return s, prob


@pytest.mark.parametrize("hetero", [False, True])
def test_fp16_product_is_within_fp16_rounding_of_fp64(hetero):
    s, prob = cube_solver(8, hetero)
    try:
        x = np.random.default_rng(5).standard_normal(prob["neq"])
        u64, u16 = s.ebe_matvec(x, 64), s.ebe_matvec(x, 16)
        u16b = s.ebe_matvec(x, 16)
    finally:
        s.close()
    assert np.array_equal(u16, u16b)
    # storkm rounded to 11 significant bits: about 1.5e-4 of the result here
    assert np.abs(u16 - u64).max() <= 1e-3 * np.abs(u64).max()
    assert np.abs(u16 - u64).max() > 1e-7 * np.abs(u64).max()   # it is the FP16 copy


@pytest.mark.parametrize("hetero", [False, True])
def test_mixed16_reaches_the_fp64_solution(hetero):
    s, prob = cube_solver(8, hetero)
    try:
        xr, _, relr = s.solve(prob["r"], 1e-12, 20000, P.MODE_FP64_RES)
        x64, _, _ = s.solve(prob["r"], 1e-8, 20000, P.MODE_FP64_RES)
        x16, it16, rel16 = s.solve(prob["r"], 1e-8, 40000, P.MODE_MIXED16)
        st = s.stats()
    finally:
        s.close()
    assert relr <= 1e-11
    assert rel16 <= 1e-8
    assert st["outer"] >= 1
    nrm = np.linalg.norm(xr)
    err64 = np.linalg.norm(x64 - xr) / nrm
    err16 = np.linalg.norm(x16 - xr) / nrm
    assert err16 <= max(1e-7, 3.0 * err64), (err16, err64)


def test_fp16_copy_follows_a_new_storkm():
    """storkm is linear in E, and the per-element scale absorbs a factor 2
    exactly, so the FP16 product after re-forming storkm with 2E is exactly
    twice the first -- which also shows that the FP16 copy was repacked."""
    prob = P.cube_problem(5, 5, 5)
    x = np.random.default_rng(6).standard_normal(prob["neq"])
    with P.Solver() as s:
        s.setup(prob["g_num"], prob["g_g"], prob["g_coord"], prob["nn"], prob["neq"])
        s.set_material(100.0, 0.3)
        s.form_storkm(27)
        u1 = s.ebe_matvec(x, 16)
        s.set_material(200.0, 0.3)
        s.form_storkm(27)
        u2 = s.ebe_matvec(x, 16)
    assert np.array_equal(u2, 2.0 * u1)


def test_mixed16_refuses_shared_km_contexts():
    prob = P.cube_problem(4, 4, 4)
    with P.Solver() as s:
        s.setup(prob["g_num"], prob["g_g"], prob["g_coord"], prob["nn"], prob["neq"])
        s.set_material(100.0, 0.3)
        km = s.form_km(1, 27)
        s.set_shared_km(km)
        with pytest.raises(P.PfError):
            s.solve(prob["r"], 1e-8, 1000, P.MODE_MIXED16)
        with pytest.raises(P.PfError):
            s.ebe_matvec(np.ones(prob["neq"]), 16)
