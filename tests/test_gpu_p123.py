"""p123 (3-D Laplace, 8-node bricks) on the GPU against the oracle and the
reference's recorded book run, through the C-ABI of libpfgpu.so."""
import json
import os

import numpy as np
import pytest

import parafem_gb300 as P
from oracle import oracle as O
from tests.conftest import GOLDEN_DIR, fortran_e

pytestmark = pytest.mark.gpu


def distorted_box8(nxe, nye, nze, seed=3, amp=0.1):
    prob = P.box8_problem(nxe, nye, nze, 1.0, 1.0, 1.0)
    g_num, g_coord = prob["g_num"], prob["g_coord"]
    coords = np.zeros((prob["nn"], 3))
    for e in range(g_num.shape[0]):
        coords[g_num[e] - 1] = g_coord[e].T
    coords += np.random.default_rng(seed).uniform(-amp, amp, size=coords.shape)
    prob["g_coord"] = np.ascontiguousarray(coords[g_num - 1].transpose(0, 2, 1))
    return prob


def scalar_solver(prob, nip=8, k=(2.0, 1.0, 3.0)):
    s = P.Solver()
    s.setup_scalar8(prob["g_num"], prob["g_g"], prob["g_coord"], prob["nn"], prob["neq"])
    s.form_storkc(nip, *k)
    return s


@pytest.mark.parametrize("nip", [8, 27])
def test_storkc_products_and_diag_match_oracle(nip):
    prob = distorted_box8(4, 3, 5)
    ref = O.form_storkc(prob["g_coord"], nip, 2.0, 1.0, 3.0)
    x = np.random.default_rng(nip).standard_normal(prob["neq"])
    with scalar_solver(prob, nip) as s:
        kc = s.get_storkc()
        u = s.ebe_matvec(x, 64)
        dg = s.get_diag()
        with pytest.raises(P.PfError):
            s.ebe_matvec(x, 32)
    # storkc(i,j) at i + 8j: the GPU's (nels, 8, 8) array holds column j in row j
    assert np.abs(kc - ref).max() <= 1e-13 * np.abs(ref).max()
    uref = O.ebe_matvec8(prob["g_g"], ref, x)
    assert np.abs(u - uref).max() <= 1e-12 * np.abs(uref).max()
    assert np.abs(dg - O.diag8(prob["g_g"], ref, prob["neq"])).max() <= 1e-13 * np.abs(dg).max()


def test_p123_pcg_matches_oracle():
    prob = P.box8_problem(24, 20, 16, 0.1, 0.1, 0.1)
    kc = O.form_storkc(prob["g_coord"], 8, 2.0, 2.0, 2.0)
    dg = O.diag8(prob["g_g"], kc, prob["neq"])
    it_ref, x_ref, _ = O.pcg123(prob["g_g"], kc, dg, prob["r"], 1e-8, 5000)
    with scalar_solver(prob, 8, (2.0, 2.0, 2.0)) as s:
        x, it, rel = s.solve(prob["r"], 1e-8, 5000, P.MODE_P121)
        x2, it2, _ = s.solve(prob["r"], 1e-8, 5000, P.MODE_P121)
        xr, itr, relr = s.solve(prob["r"], 1e-10, 5000, P.MODE_FP64_RES)
        with pytest.raises(P.PfError):
            s.solve(prob["r"], 1e-8, 5000, P.MODE_MIXED)
    assert abs(it - it_ref) <= 1
    assert np.linalg.norm(x - x_ref) <= 1e-7 * np.linalg.norm(x_ref)
    assert it2 == it and np.array_equal(x, x2)
    assert relr <= 1e-10


def test_fixed_freedoms_by_penalty_match_oracle():
    prob = P.box8_problem(10, 8, 6, 0.2, 0.2, 0.2)
    neq = prob["neq"]
    fix_eq = np.array([3, 17, neq // 2], np.int32)
    vals = np.array([100.0, -20.0, 5.0])
    kc = O.form_storkc(prob["g_coord"], 8, 1.0, 2.0, 3.0)
    dg = O.diag8(prob["g_g"], kc, neq)
    dg[fix_eq - 1] += 1e20
    store = dg[fix_eq - 1].copy()
    r = prob["r"].copy()
    r[fix_eq - 1] = store * vals
    it_ref, x_ref, _ = O.pcg123(prob["g_g"], kc, dg, r, 1e-9, 5000, fix_eq, store)
    with scalar_solver(prob, 8, (1.0, 2.0, 3.0)) as s:
        s.set_fixed(fix_eq, 1e20)
        gdg = s.get_diag()
        r2 = prob["r"].copy()
        r2[fix_eq - 1] = gdg[fix_eq - 1] * vals
        x, it, _ = s.solve(r2, 1e-9, 5000, P.MODE_P121)
    assert np.array_equal(gdg[fix_eq - 1], store)
    assert abs(it - it_ref) <= 1
    assert np.abs(x[fix_eq - 1] - vals).max() <= 1e-12 * np.abs(vals).max()
    assert np.linalg.norm(x - x_ref) <= 1e-7 * np.linalg.norm(x_ref)


def test_p123_job_writes_res_and_potentials(tmp_path):
    job = str(tmp_path / "p123_small")
    with open(job + ".mg", "w") as f:
        f.write("'p123'\n'parafem' 4000  20  20  8\n.05  .05  .05  2.0  2.0  2.0\n1.e-5  1000\n1  0\n")
    P.p12meshgen(job)
    it, pot = P.p123_run(job)
    ref = O.run_p123_box(20, 10, 20, .05, .05, .05, 2.0, 2.0, 2.0, 1e-5, 1000)
    assert abs(it - ref["iters"]) <= 1
    res = open(job + ".res").read()
    assert "The total load is   0.1000E+02" in res
    nres = ref["nres"]
    for i in range(4):
        assert f"{nres + i:8d}     {fortran_e(ref['x'][nres - 1 + i])}" in res
        assert abs(pot[i] - ref["x"][nres - 1 + i]) <= 1e-6 * abs(ref["x"][nres - 1])
    ndptl = open(job + ".ensi.NDPTL-000001").read().splitlines()
    assert ndptl[:4] == ["Alya Ensight Gold --- Scalar per-node variable file", "part", "    1", "coordinates"]
    assert len(ndptl) == 4 + 21 * 11 * 21


@pytest.mark.slow
def test_p123_book_run_on_the_gpu():
    """examples/5th_ed/p123/book: 8,000,000 bricks, 180 iterations, the four
    printed potentials (E12.4)."""
    with open(os.path.join(GOLDEN_DIR, "p123_golden.json")) as f:
        g = json.load(f)["book"]
    prob = P.box8_problem(200, 200, 200, .005, .005, .005)
    assert prob["neq"] == g["neq"]
    with scalar_solver(prob, 8, (2.0, 2.0, 2.0)) as s:
        x, it, _ = s.solve(prob["r"], 1e-5, 10000, P.MODE_P121)
    assert abs(it - g["iterations"]) <= 2
    for fq, text in g["potentials"]:
        assert fortran_e(x[fq - 1]).strip() == text
