"""Edge cases through the C-ABI: zero loads, iteration limits, one element,
nodes no element uses, a single-slice mesh."""
import numpy as np
import pytest

import parafem_gb300 as P
from oracle import oracle as O

pytestmark = pytest.mark.gpu

MODES = [P.MODE_P121, P.MODE_FP64_RES, P.MODE_MIXED, P.MODE_MIXED_RESTART]


def solver(prob):
    s = P.Solver()
    s.setup(prob["g_num"], prob["g_g"], prob["g_coord"], prob["nn"], prob["neq"])
    s.set_material(100.0, 0.3)
    s.form_storkm(27)
    return s


@pytest.mark.parametrize("mode", MODES)
def test_zero_load_is_solved_by_zero(mode):
    prob = P.cube_problem(3, 2, 2)
    with solver(prob) as s:
        x, it, rel = s.solve(np.zeros(prob["neq"]), 1e-8, 100, mode)
    assert it == 0 and not x.any() and rel == 0.0


@pytest.mark.parametrize("mode", [P.MODE_P121, P.MODE_FP64_RES])
def test_iteration_limit_is_honoured(mode):
    prob = P.cube_problem(4, 4, 4)
    with solver(prob) as s:
        for limit in (1, 2, 7):
            x, it, rel = s.solve(prob["r"], 1e-14, limit, mode)
            assert it == limit and np.isfinite(x).all() and rel > 1e-14


def test_one_element_mesh_matches_oracle():
    prob = P.cube_problem(1, 1, 1)
    km = O.form_storkm(prob["g_coord"], 27, 100.0, 0.3)
    dg = O.diag(prob["g_g"], km, prob["neq"])
    it_ref, x_ref, _ = O.pcg(prob["g_g"], km, dg, prob["r"], 1e-10, 500, 0)
    with solver(prob) as s:
        x, it, _ = s.solve(prob["r"], 1e-10, 500, P.MODE_P121)
    assert abs(it - it_ref) <= 1
    assert np.abs(x - x_ref).max() <= 1e-9 * np.abs(x_ref).max()


def test_nodes_used_by_no_element_are_ignored():
    prob = P.cube_problem(2, 2, 2)
    nn = prob["nn"] + 3                      # three trailing nodes no element names
    with P.Solver() as s:
        s.setup(prob["g_num"], prob["g_g"], prob["g_coord"], nn, prob["neq"])
        s.set_material(100.0, 0.3)
        s.form_storkm(27)
        x, it, rel = s.solve(prob["r"], 1e-10, 500, P.MODE_FP64_RES)
    with solver(prob) as s:
        x0, it0, _ = s.solve(prob["r"], 1e-10, 500, P.MODE_FP64_RES)
    assert it == it0 and np.array_equal(x, x0)


def test_single_slice_mesh_in_every_mode():
    prob = P.cube_problem(9, 1, 1)           # one element thick in y and z
    with solver(prob) as s:
        xr, _, _ = s.solve(prob["r"], 1e-12, 5000, P.MODE_FP64_RES)
        for mode in MODES:
            x, it, rel = s.solve(prob["r"], 1e-8, 5000, mode)
            assert it > 0
            if mode != P.MODE_P121:
                assert rel <= 1e-8
                assert np.linalg.norm(x - xr) <= 1e-6 * np.linalg.norm(xr)
