"""One element matrix shared by every element (PCG_KM, maths.f90:1152-1323):
pf_set_shared_km against the per-element path and the oracle."""
import numpy as np
import pytest

import parafem_gb300 as P
from oracle import oracle as O

pytestmark = pytest.mark.gpu


def uniform_cube(n):
    prob = P.cube_problem(n, n, n)
    km = O.form_storkm(prob["g_coord"][:1], 27, 100.0, 0.3)[0]
    km = 0.5 * (km + km.T)            # exactly symmetric
    tiled = np.ascontiguousarray(np.broadcast_to(km, (n ** 3, 60, 60)))
    return prob, km, tiled


def solver_for(prob):
    s = P.Solver()
    s.setup(prob["g_num"], prob["g_g"], prob["g_coord"], prob["nn"], prob["neq"])
    return s


@pytest.mark.parametrize("n", [5, 11])       # 11^3 = 1331 elements: 11 tiles of 128, a partial last tile
def test_shared_products_match_oracle(n):
    prob, km, tiled = uniform_cube(n)
    x = np.random.default_rng(n).standard_normal(prob["neq"])
    ref = O.ebe_matvec(prob["g_g"], tiled, x)
    with solver_for(prob) as s:
        s.set_shared_km(km)
        u64 = s.ebe_matvec(x, 64)
        u32 = s.ebe_matvec(x, 32)
        dg = s.get_diag()
        with pytest.raises(P.PfError):
            s.get_storkm(0, 1)
    scale = np.abs(ref).max()
    assert np.abs(u64 - ref).max() <= 1e-13 * scale
    assert np.abs(u32 - ref).max() <= 3e-6 * scale        # FP32-class tensor-core products
    assert np.array_equal(dg, O.diag(prob["g_g"], tiled, prob["neq"]))


def test_shared_fp64_solve_bitwise_equals_per_element_path():
    prob, km, tiled = uniform_cube(6)
    with solver_for(prob) as s:
        s.set_storkm(tiled)
        x1, it1, r1 = s.solve(prob["r"], 1e-6, 5000, P.MODE_P121)
        s.set_shared_km(km)
        x2, it2, r2 = s.solve(prob["r"], 1e-6, 5000, P.MODE_P121)
    assert it1 == it2
    assert np.array_equal(x1, x2)    # same FMA order per row, same scatter order


def test_shared_mixed_solve_reaches_1e8_and_matches_fp64():
    prob, km, tiled = uniform_cube(9)
    with solver_for(prob) as s:
        s.set_shared_km(km)
        xr, _, relr = s.solve(prob["r"], 1e-12, 20000, P.MODE_FP64_RES)
        xm, itm, relm = s.solve(prob["r"], 1e-8, 20000, P.MODE_MIXED)
        st = s.stats()
        with pytest.raises(P.PfError):
            s.solve_multi(np.zeros((prob["neq"], 16)), 1e-8, 10)
    assert relr <= 1e-11 and relm <= 1e-8
    assert st["outer"] >= 1
    assert np.linalg.norm(xm - xr) <= 1e-7 * np.linalg.norm(xr)


def test_form_km_matches_oracle():
    prob = P.cube_problem(3, 2, 2)
    with solver_for(prob) as s:
        s.set_material(100.0, 0.3)
        km = s.form_km(4, 27)
    ref = O.form_storkm(prob["g_coord"][3:4], 27, 100.0, 0.3)[0]
    assert np.abs(km - ref).max() <= 1e-13 * np.abs(ref).max()


def test_shared_tensor_core_product_keeps_translations_out_of_the_rounding():
    """The tensor-core product is P km P p_e (P removes each element's mean
    translation), so on a nearly rigid p its error away from the restrained
    elements is set by the small non-rigid part.  The full-FP32 per-element
    product of the same km (no projection) errs by the rounding of the
    translation itself."""
    prob, km, tiled = uniform_cube(8)
    g_g, neq = prob["g_g"], prob["neq"]
    x = 1.0 + 1e-4 * np.random.default_rng(13).standard_normal(neq)
    with solver_for(prob) as s:
        s.set_shared_km(km)
        u64, u32 = s.ebe_matvec(x, 64), s.ebe_matvec(x, 32)
    with solver_for(prob) as s:
        s.set_storkm(tiled)
        u31 = s.ebe_matvec(x, 31)
    touched = np.zeros(neq + 1, bool)
    touched[g_g[(g_g == 0).any(axis=1)].ravel()] = True
    inner = ~touched[1:]
    assert inner.sum() > neq // 2
    e32 = np.abs(u32 - u64)[inner].max()
    e31 = np.abs(u31 - u64)[inner].max()
    assert e31 > 0.0
    assert e32 <= 1e-2 * e31, (e32, e31)
