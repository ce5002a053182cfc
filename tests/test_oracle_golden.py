"""The oracle pinned against the reference's own recorded p121 runs
(examples/5th_ed/p121: demo deck + p121_demo.res + DISPL; book p121.res)."""
import hashlib

import numpy as np
import pytest

from oracle import oracle as O
from tests.conftest import fortran_e


def test_demo_deck_regenerated_byte_identical(demo_job, golden):
    for ext, sha in golden["demo_deck_sha256"].items():
        with open(demo_job + "." + ext, "rb") as f:
            assert hashlib.sha256(f.read()).hexdigest() == sha, ext


def test_demo_sizes(demo_problem, golden):
    d = demo_problem["deck"]
    g = golden["demo"]
    assert (d.nn, d.nr, demo_problem["neq"]) == (g["nn"], g["nr"], g["neq"])


def test_demo_total_load_line(demo_problem, golden):
    q = O._seq_sum(demo_problem["r"])
    assert "The total load is:" + fortran_e(q) == golden["demo"]["lines"]["total_load"]


@pytest.fixture(scope="module")
def demo_oracle_run(demo_problem):
    p = demo_problem
    d = p["deck"]
    it, x, metric, hist = O.pcg(p["g_g"], p["km"], p["diag"], p["r"], d.tol, d.limit, 0, history=True)
    it295, x295, _ = O.pcg(p["g_g"], p["km"], p["diag"], p["r"], 0.0, 295, 0)
    return dict(it=it, x=x, hist=hist, x295=x295)


def test_demo_iterations_within_rounding_window(demo_oracle_run, golden):
    # The 4-rank reference stopped at 295; the checon metric there sits 0.9%
    # above tol and moves by ~0.5% with the reduction order alone, so the
    # stop is pinned to +-2 iterations.
    it = demo_oracle_run["it"]
    assert abs(it - golden["demo"]["iterations"]) <= 2
    h = demo_oracle_run["hist"]
    assert h[294] > 1e-5 and h[294] < 1.01e-5


def test_demo_central_displacement_line(demo_oracle_run, golden):
    x = demo_oracle_run["x"]
    assert "The central nodal displacement is :" + fortran_e(x[0]) == golden["demo"]["lines"]["central"]


def test_demo_stresses_at_golden_iteration(demo_oracle_run, demo_problem, golden):
    p = demo_problem
    d = p["deck"]
    x0 = np.concatenate([[0.0], demo_oracle_run["x295"]])
    sig = O.centroid_stress(p["gc"][0], x0[p["g_g"][0]], d.e, d.v)
    assert "".join(fortran_e(s) for s in sig) == golden["demo"]["lines"]["stress"]


def test_demo_displacement_field_at_golden_iteration(demo_oracle_run, demo_problem, golden_displ):
    p = demo_problem
    disp = O.nodal_displacements(p["deck"].g_num, p["g_g"], demo_oracle_run["x295"], p["deck"].nn)
    # golden is E12.4 text: half a unit in the 4th digit is <= 5e-5 for |u| < 1
    assert np.abs(disp - golden_displ).max() <= 5.2e-5


def test_book_deck_sizes(book_job, golden):
    d = O.read_deck(book_job)
    g = golden["book"]
    g_g = O.steering(d.g_num, d.rest)
    assert (d.nn, d.nr, int(g_g.max())) == (g["nn"], g["nr"], g["neq"])
