"""GPU path vs the oracle, through the C-ABI of libpfgpu.so."""
import numpy as np
import pytest

import parafem_gb300 as P
from oracle import oracle as O
from tests.conftest import fortran_e

pytestmark = pytest.mark.gpu


def distorted_cube(nxe, nye, nze, seed=7, amp=0.08):
    """A cube mesh with every node moved by a seeded random offset."""
    g_num, g_coord, nn = P.mesh_cube(nxe, nye, nze)
    rng = np.random.default_rng(seed)
    shift = rng.uniform(-amp, amp, size=(nn, 3))
    coords = np.zeros((nn, 3))
    for e in range(g_num.shape[0]):
        coords[g_num[e] - 1] = g_coord[e].T
    coords = coords + shift
    g_coord = np.ascontiguousarray(coords[g_num - 1].transpose(0, 2, 1))
    fix = P.cube_restraints(nxe, nye, nze, 1, nn)
    g_g, neq = P.number_equations(g_num, fix)
    return g_num, g_coord, nn, g_g, neq


@pytest.mark.parametrize("nip", [8, 27])
@pytest.mark.parametrize("per_element", [False, True])
def test_storkm_formation_matches_oracle(nip, per_element):
    g_num, g_coord, nn, g_g, neq = distorted_cube(3, 2, 3)
    nels = g_num.shape[0]
    if per_element:
        e, v = P.random_material(nels, 99, 1.0, 1000.0, 0.2, 0.35)
    else:
        e, v = np.array([100.0]), np.array([0.3])
    ref = O.form_storkm(g_coord, nip, e, v)
    with P.Solver() as s:
        s.setup(g_num, g_g, g_coord, nn, neq)
        s.set_material(e, v)
        s.form_storkm(nip)
        km = s.get_storkm()
        dg = s.get_diag()
    scale = np.abs(ref).max(axis=(1, 2), keepdims=True)
    assert (np.abs(km - ref) / scale).max() <= 1e-13
    assert np.abs(dg - O.diag(g_g, ref, neq)).max() <= 1e-13 * np.abs(dg).max()
    # symmetric, positive diagonal
    assert (np.abs(km - km.transpose(0, 2, 1)) / scale).max() <= 1e-13
    assert (np.einsum("eii->ei", km) > 0).all()


def test_exact_weights_switch():
    g_num, g_coord, nn, g_g, neq = distorted_cube(2, 2, 2)
    with P.Solver() as s:
        s.setup(g_num, g_g, g_coord, nn, neq)
        s.set_material(100.0, 0.3)
        s.form_storkm(27, exact_weights=False)
        k1 = s.get_storkm()
        s.form_storkm(27, exact_weights=True)
        k2 = s.get_storkm()
    ref2 = O.form_storkm(g_coord, 27, 100.0, 0.3, exact_weights=True)
    rel = np.abs(k1 - k2).max() / np.abs(k2).max()
    assert 1e-9 < rel < 1e-6        # the single-precision 5./9. factor
    assert np.abs(k2 - ref2).max() <= 1e-13 * np.abs(ref2).max()


def test_diag_bitwise_equals_serial_scatter(demo_problem):
    p = demo_problem
    d = p["deck"]
    with P.Solver() as s:
        s.setup(d.g_num, p["g_g"], p["gc"], d.nn, p["neq"])
        s.set_storkm(p["km"])
        dg = s.get_diag()
    assert np.array_equal(dg, p["diag"])


@pytest.mark.parametrize("prec,tol", [(64, 1e-13), (32, 3e-6), (31, 3e-6)])
def test_ebe_matvec_matches_oracle(demo_problem, prec, tol):
    """64: FP64 storkm; 32: packed-symmetric FP32 (bulk-copy staged); 31: full FP32."""
    p = demo_problem
    d = p["deck"]
    rng = np.random.default_rng(3)
    x = rng.standard_normal(p["neq"])
    ref = O.ebe_matvec(p["g_g"], p["km"], x)
    with P.Solver() as s:
        s.setup(d.g_num, p["g_g"], p["gc"], d.nn, p["neq"])
        s.set_storkm(p["km"])
        u = s.ebe_matvec(x, prec)
    assert np.abs(u - ref).max() <= tol * np.abs(ref).max()


def test_demo_pcg_matches_oracle_iterates(demo_problem):
    p = demo_problem
    d = p["deck"]
    it_ref, x_ref, _ = O.pcg(p["g_g"], p["km"], p["diag"], p["r"], 0.0, 295, 0)
    with P.Solver() as s:
        s.setup(d.g_num, p["g_g"], p["gc"], d.nn, p["neq"])
        s.set_storkm(p["km"])
        x, it, rel = s.solve(p["r"], 0.0, 295, P.MODE_P121)
        x2, it2, _ = s.solve(p["r"], 0.0, 295, P.MODE_P121)
    assert it == 295
    # 295 iterations amplify FMA / reduction-order rounding; p121's own bound
    assert np.abs(x - x_ref).max() <= 1e-6 * np.abs(x_ref).max()
    assert np.array_equal(x, x2)            # bitwise reproducible


def test_p121_job_reproduces_golden_res(demo_job, golden, golden_displ):
    it, central = P.p121_run(demo_job, P.MODE_P121)
    res = open(demo_job + ".res").read().splitlines()
    g = golden["demo"]["lines"]
    assert g["total_load"] in res
    assert g["central"] in res
    assert abs(it - golden["demo"]["iterations"]) <= 2
    vals = open(demo_job + ".ensi.DISPL-000001").read().split("\n")[4:]
    disp = np.array([float(t) for t in vals if t.strip()]).reshape(3, -1).T
    # converged iterate vs the golden one two iterations earlier: E12.4 text
    # (<= 5e-5) plus the change over those iterations
    assert np.abs(disp - golden_displ).max() <= 1e-4


def test_demo_stresses_via_gpu_at_golden_iteration(demo_problem, golden):
    p = demo_problem
    d = p["deck"]
    _, x_ref, _ = O.pcg(p["g_g"], p["km"], p["diag"], p["r"], 0.0, 295, 0)
    x0 = np.concatenate([[0.0], x_ref])
    sig_ref = O.centroid_stress(p["gc"][0], x0[p["g_g"][0]], d.e, d.v)
    with P.Solver() as s:
        s.setup(d.g_num, p["g_g"], p["gc"], d.nn, p["neq"])
        s.set_material(d.e, d.v)
        s.form_storkm(d.nip)
        x, it, _ = s.solve(p["r"], 0.0, 295, P.MODE_P121)
        sig = s.centroid_stress(x, 1)
    # the oracle's stresses print as the golden line (test_oracle_golden); the
    # GPU's agree with the oracle's to the displacement bound
    assert np.abs(sig - sig_ref).max() <= 1e-6 * np.abs(sig_ref).max()
    normal = "".join(fortran_e(v) for v in sig[:3])
    assert normal == golden["demo"]["lines"]["stress"][:36]


def test_element_stresses_of_every_element_match_oracle():
    g_num, g_coord, nn, g_g, neq = distorted_cube(4, 3, 3)
    nels = g_num.shape[0]
    e, v = P.random_material(nels, 5, 1.0, 1000.0, 0.2, 0.35)
    x = np.random.default_rng(12).standard_normal(neq)
    x0 = np.concatenate([[0.0], x])
    ref = np.array([O.centroid_stress(g_coord[k], x0[g_g[k]], e[k], v[k]) for k in range(nels)])
    with P.Solver() as s:
        s.setup(g_num, g_g, g_coord, nn, neq)
        s.set_material(e, v)
        sig = s.element_stresses(x)
        part = s.element_stresses(x, 7, 5)
        one = s.centroid_stress(x, 9)
    assert np.abs(sig - ref).max() <= 1e-12 * np.abs(ref).max()
    assert np.array_equal(part, sig[6:11])
    assert np.array_equal(one, sig[8])


def test_config1_fp64_drop_in_matches_oracle():
    """10^3 cube, nip=27, E=100, v=0.3, fixed base, top pressure, checon tol 1e-6."""
    prob = P.cube_problem(10, 10, 10)
    gc = prob["g_coord"]
    km = O.form_storkm(gc, 27, 100.0, 0.3)
    dg = O.diag(prob["g_g"], km, prob["neq"])
    it_ref, x_ref, _ = O.pcg(prob["g_g"], km, dg, prob["r"], 1e-6, 5000, 0)
    with P.Solver() as s:
        s.setup(prob["g_num"], prob["g_g"], gc, prob["nn"], prob["neq"])
        s.set_material(100.0, 0.3)
        s.form_storkm(27)
        x, it, rel = s.solve(prob["r"], 1e-6, 5000, P.MODE_P121)
    assert abs(it - it_ref) <= 3
    assert np.linalg.norm(x - x_ref) <= 1e-6 * np.linalg.norm(x_ref)


@pytest.mark.parametrize("hetero", [False, True])
def test_mixed_precision_reaches_1e8_and_matches_fp64(hetero):
    prob = P.cube_problem(8, 8, 8)
    nels = prob["g_num"].shape[0]
    if hetero:
        e, v = P.random_material(nels, 2024, 1.0, 1000.0, 0.2, 0.35)
    else:
        e, v = np.array([100.0]), np.array([0.3])
    with P.Solver() as s:
        s.setup(prob["g_num"], prob["g_g"], prob["g_coord"], prob["nn"], prob["neq"])
        s.set_material(e, v)
        s.form_storkm(27)
        xr, itr, relr = s.solve(prob["r"], 1e-12, 20000, P.MODE_FP64_RES)
        x64, it64, rel64 = s.solve(prob["r"], 1e-8, 20000, P.MODE_FP64_RES)
        xm, itm, relm = s.solve(prob["r"], 1e-8, 20000, P.MODE_MIXED)
        st = s.stats()
        xt, itt, relt = s.solve(prob["r"], 1e-10, 20000, P.MODE_MIXED)
    assert relr <= 1e-11
    assert relm <= 1e-8 and relt <= 1e-10
    assert st["outer"] >= 1
    nrm = np.linalg.norm(xr)
    err64 = np.linalg.norm(x64 - xr) / nrm
    errm = np.linalg.norm(xm - xr) / nrm
    # at the same residual the mixed solution is as accurate as the FP64 one
    assert errm <= max(1e-7, 3.0 * err64), (errm, err64)
    assert np.linalg.norm(xt - xr) <= 1e-7 * nrm


def test_packed_symmetric_product_is_symmetric_and_deterministic(demo_problem):
    p = demo_problem
    d = p["deck"]
    rng = np.random.default_rng(8)
    a, b = rng.standard_normal(p["neq"]), rng.standard_normal(p["neq"])
    with P.Solver() as s:
        s.setup(d.g_num, p["g_g"], p["gc"], d.nn, p["neq"])
        s.set_storkm(p["km"])
        ka, kb = s.ebe_matvec(a, 32), s.ebe_matvec(b, 32)
        ka2 = s.ebe_matvec(a, 32)
    assert np.array_equal(ka, ka2)
    # the packed operator is exactly symmetric up to FP32 rounding of the products
    assert abs(b @ ka - a @ kb) <= 1e-6 * abs(b @ ka)


def test_packed_product_keeps_rigid_translations_out_of_the_rounding():
    """K_e t = 0 for a translation t; the packed FP32 product subtracts each
    element's mean translation in FP64 before rounding, so on a nearly rigid
    p its error away from the restrained elements is set by the small
    non-rigid part, while the full-FP32 product (no projection) errs by the
    rounding of the translation itself."""
    prob = P.cube_problem(8, 8, 8)
    g_g, neq = prob["g_g"], prob["neq"]
    rng = np.random.default_rng(12)
    x = 1.0 + 1e-4 * rng.standard_normal(neq)
    with P.Solver() as s:
        s.setup(prob["g_num"], g_g, prob["g_coord"], prob["nn"], prob["neq"])
        s.set_material(100.0, 0.3)
        s.form_storkm(27)
        u64, u32, u31 = s.ebe_matvec(x, 64), s.ebe_matvec(x, 32), s.ebe_matvec(x, 31)
    # equations of elements with no restrained freedom, minus every equation
    # that also belongs to an element with one
    touched = np.zeros(neq + 1, bool)
    touched[g_g[(g_g == 0).any(axis=1)].ravel()] = True
    inner = ~touched[1:]
    assert inner.sum() > neq // 2
    e32 = np.abs(u32 - u64)[inner].max()
    e31 = np.abs(u31 - u64)[inner].max()
    assert e31 > 0.0
    assert e32 <= 1e-2 * e31, (e32, e31)


def test_autotuned_configurations_give_bitwise_equal_products(demo_problem):
    p = demo_problem
    d = p["deck"]
    a = np.random.default_rng(9).standard_normal(p["neq"])
    with P.Solver() as s:
        s.setup(d.g_num, p["g_g"], p["gc"], d.nn, p["neq"])
        s.set_storkm(p["km"])
        t = s.tuning()
        assert (t["warps"], t["stages"]) in ((14, 2), (12, 2), (8, 3))
        assert all(v > 0 for v in t["ms"].values())
        outs = []
        for cfg in (0, 1, 2):
            s.set_tuning(cfg)
            outs.append(s.ebe_matvec(a, 32))
        s.set_tuning(-1)
        with pytest.raises(P.PfError):
            s.set_tuning(3)
    assert np.array_equal(outs[0], outs[1]) and np.array_equal(outs[0], outs[2])


@pytest.mark.parametrize("mode", [P.MODE_P121, P.MODE_MIXED])
def test_graph_replay_gives_bitwise_equal_iterates(mode):
    prob = P.cube_problem(7, 7, 7)
    res = []
    for graphs in (True, False):
        with P.Solver() as s:
            s.setup(prob["g_num"], prob["g_g"], prob["g_coord"], prob["nn"], prob["neq"])
            s.set_material(100.0, 0.3)
            s.form_storkm(27)
            s.set_graphs(graphs)
            s.set_tuning(0)
            x, it, rel = s.solve(prob["r"], 1e-8, 5000, mode)
            res.append((x, it, rel, s.launches()))
    (xa, ia, ra, la), (xb, ib, rb, lb) = res
    assert ia == ib and ra == rb
    assert np.array_equal(xa, xb)
    # a replay launches every kernel of its iterations, counted the same way
    assert abs(la - lb) <= 5 * 8 * 4


def test_mixed_restart_mode_also_converges():
    prob = P.cube_problem(6, 6, 6)
    with P.Solver() as s:
        s.setup(prob["g_num"], prob["g_g"], prob["g_coord"], prob["nn"], prob["neq"])
        s.set_material(100.0, 0.3)
        s.form_storkm(27)
        xr, _, _ = s.solve(prob["r"], 1e-12, 20000, P.MODE_FP64_RES)
        x3, it3, rel3 = s.solve(prob["r"], 1e-8, 20000, P.MODE_MIXED_RESTART)
    assert rel3 <= 1e-8
    assert np.linalg.norm(x3 - xr) <= 1e-6 * np.linalg.norm(xr)


def test_xx3_matrix_vector_multiplies():
    import ctypes
    L = P.lib()
    rng = np.random.default_rng(5)
    for n_mat, n_row, n_col in [(37, 60, 60), (5, 7, 3)]:
        mats = rng.standard_normal((n_mat, n_col, n_row))     # column-major per matrix
        lhs = rng.standard_normal((n_mat, n_col))
        ref = np.einsum("mji,mj->mi", mats, lhs)
        I = lambda v: ctypes.byref(ctypes.c_int(v))
        ptr = [ctypes.c_void_p() for _ in range(3)]
        sizes = [mats.size, lhs.size, n_mat * n_row]
        for pv, n in zip(ptr, sizes):
            assert L.allocate_memory_on_gpu(I(n), I(8), ctypes.byref(pv)) == 0
        assert L.copy_data_to_gpu(I(mats.size), I(8), mats.ctypes.data, ctypes.byref(ptr[0])) == 0
        assert L.copy_data_to_gpu(I(lhs.size), I(8), lhs.ctypes.data, ctypes.byref(ptr[1])) == 0
        assert L.matrix_vector_multiplies(I(n_mat), I(n_row), I(n_col), ctypes.byref(ptr[1]),
                                          ctypes.byref(ptr[0]), ctypes.byref(ptr[2])) == 0
        out = np.zeros((n_mat, n_row))
        assert L.copy_data_from_gpu(I(out.size), I(8), out.ctypes.data, ctypes.byref(ptr[2])) == 0
        for pv in ptr:
            assert L.free_memory_on_gpu(ctypes.byref(pv)) == 0
        assert np.abs(out - ref).max() <= 1e-12 * np.abs(ref).max()


def test_invalid_inputs_fail_loudly():
    with P.Solver() as s:
        with pytest.raises(P.PfError):
            s.form_storkm(8)                     # before setup
        g_num, g_coord, nn, g_g, neq = distorted_cube(1, 1, 1)
        bad = g_num.copy()
        bad[0, 0] = nn + 5
        with pytest.raises(P.PfError, match="outside"):
            s.setup(bad, g_g, g_coord, nn, neq)
        s.setup(g_num, g_g, g_coord, nn, neq)
        with pytest.raises(P.PfError, match="nip"):
            s.set_material(100.0, 0.3)
            s.form_storkm(9)


@pytest.mark.slow
@pytest.mark.parametrize("mode", [P.MODE_MIXED, P.MODE_MIXED16])
def test_mixed_40cube_within_1e7_of_fp64_at_1e12(mode):
    """The mixed modes on a 40^3 cube (797,040 equations, heterogeneous E and
    v) solved to relres 1e-8: within 1e-7 (2-norm, relative) of FP64 solved
    as far as FP64 goes on this mesh (the recursive residual to 1e-12; the
    true residual levels off near 1e-11), as the 100^3 benchmark measures."""
    prob = P.cube_problem(40, 40, 40)
    nels = prob["g_num"].shape[0]
    e, v = P.random_material(nels, 40, 1.0, 1000.0, 0.2, 0.35)
    with P.Solver() as s:
        s.setup(prob["g_num"], prob["g_g"], prob["g_coord"], prob["nn"], prob["neq"])
        s.set_material(e, v)
        s.form_storkm(27)
        xr, _, relr = s.solve(prob["r"], 1e-12, 50000, P.MODE_FP64_RES)
        xm, _, relm = s.solve(prob["r"], 1e-8, 50000, mode)
    assert relr <= 5e-11 and relm <= 1e-8
    assert np.linalg.norm(xm - xr) <= 1e-7 * np.linalg.norm(xr)
