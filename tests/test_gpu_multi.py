"""Several load cases per mesh (pf_solve_multi / pf_ebe_matvec_multi): the
tensor-core block product (tcgen05, two-term FP16 splits of K_e and P_e,
FP32 accumulation) against FP32 CUDA cores and FP64, for k = 8 .. 72 load
cases, and the block solve against sequential FP64 solves and against the
C restatement of p121's PCG."""
import numpy as np
import pytest

import parafem_gb300 as P

pytestmark = pytest.mark.gpu


def setup_solver(nxe, nye, nze, seed=3):
    prob = P.cube_problem(nxe, nye, nze)
    nels = nxe * nye * nze
    e, v = P.random_material(nels, seed, 10.0, 1000.0, 0.2, 0.35)
    s = P.Solver()
    s.setup(prob["g_num"], prob["g_g"], prob["g_coord"], prob["nn"], prob["neq"])
    s.set_material(e, v)
    s.form_storkm(27)
    return s, prob, (e, v)


@pytest.mark.parametrize("k", [8, 16, 24, 40, 64, 72])
def test_block_products_agree(k):
    s, prob, _ = setup_solver(4, 3, 3)
    try:
        rng = np.random.default_rng(k)
        Pm = rng.standard_normal((prob["neq"], k))
        u64 = s.ebe_matvec_multi(Pm, 64)
        ref = np.stack([s.ebe_matvec(Pm[:, j], 64) for j in range(k)], axis=1)
        assert np.abs(u64 - ref).max() <= 1e-13 * np.abs(ref).max()
        for prec in (32, 16):
            u = s.ebe_matvec_multi(Pm, prec)
            # per case: FP32-class products (FP16 hi + lo terms, FP32 accumulation)
            err = np.abs(u - u64).max(axis=0) / np.abs(u64).max(axis=0)
            assert err.max() <= 3e-6, (prec, err.max())
        tune = s.multi_tuning()
        assert tune["kb"] <= 64 and tune["kb"] % 8 == 0
        assert tune["kb"] == min(k, 64) or tune["kb"] in tune["ms"]
    finally:
        s.close()


def test_invalid_case_counts_are_rejected():
    s, prob, _ = setup_solver(3, 3, 3)
    try:
        for k in (4, 12, 136):
            with pytest.raises(P.PfError, match="multiple of 8"):
                s.ebe_matvec_multi(np.zeros((prob["neq"], k)), 16)
    finally:
        s.close()


@pytest.mark.parametrize("k", [16, 24])
def test_block_solve_matches_sequential_fp64(k):
    s, prob, _ = setup_solver(6, 5, 4)
    try:
        R = P.random_top_loads(prob["g_g"], 6, 4, prob["neq"], k, seed=7)
        X, it, rel = s.solve_multi(R, 1e-9, 20000, prec=16)
        assert (rel <= 1e-9).all()
        for j in (0, 5, k - 1):
            x64, it64, rel64 = s.solve(R[:, j], 1e-12, 20000, P.MODE_FP64_RES)
            assert np.linalg.norm(X[:, j] - x64) <= 1e-7 * np.linalg.norm(x64), j
        X32, it32, rel32 = s.solve_multi(R, 1e-9, 20000, prec=32)
        assert (rel32 <= 1e-9).all()
        assert np.abs(X32 - X).max() <= 1e-6 * np.abs(X).max()
    finally:
        s.close()


def test_block_solve_matches_oracle_pcg():
    """8 load cases on a small heterogeneous mesh: every block-solve column
    against the C restatement of p121's PCG (relative-residual stop at 1e-12)
    on the oracle's own storkm."""
    from oracle import oracle as O
    s, prob, (e, v) = setup_solver(5, 4, 3, seed=11)
    try:
        R = P.random_top_loads(prob["g_g"], 5, 3, prob["neq"], 8, seed=12)
        X, it, rel = s.solve_multi(R, 1e-10, 20000, prec=16)
    finally:
        s.close()
    assert (rel <= 1e-10).all()
    km = O.form_storkm(prob["g_coord"], 27, e, v)
    dg = O.diag(prob["g_g"], km, prob["neq"])
    for j in range(8):
        _, xr, _ = O.pcg(prob["g_g"], km, dg, np.ascontiguousarray(R[:, j]), 1e-12, 20000, 1)
        assert np.linalg.norm(X[:, j] - xr) <= 1e-7 * np.linalg.norm(xr), j


def test_tensor_core_block_product_keeps_translations_out_of_the_rounding():
    """The tensor-core block product removes a translation of each load case
    before rounding (and the mean translation of the result); on nearly
    rigid load cases its error away from the restrained elements is far
    below that of the FP32 CUDA-core block product (no projection)."""
    s, prob, _ = setup_solver(6, 6, 6)
    try:
        g_g, neq = prob["g_g"], prob["neq"]
        Pm = 1.0 + 1e-4 * np.random.default_rng(14).standard_normal((neq, 16))
        u64, u16, u32 = s.ebe_matvec_multi(Pm, 64), s.ebe_matvec_multi(Pm, 16), s.ebe_matvec_multi(Pm, 32)
    finally:
        s.close()
    touched = np.zeros(neq + 1, bool)
    touched[g_g[(g_g == 0).any(axis=1)].ravel()] = True
    inner = ~touched[1:]
    assert inner.sum() > neq // 3
    e16 = np.abs(u16 - u64)[inner].max()
    e32 = np.abs(u32 - u64)[inner].max()
    assert e32 > 0.0
    assert e16 <= 1e-2 * e32, (e16, e32)


def test_block_buffers_belong_to_the_context():
    """Each context keeps its own block-solve buffers: products of two
    meshes interleave, and pf_multi_free releases one context's buffers
    without touching the other's; a change of k reallocates them."""
    s1, p1, _ = setup_solver(4, 3, 3)
    s2, p2, _ = setup_solver(5, 4, 3, seed=4)
    try:
        rng = np.random.default_rng(15)
        X1 = rng.standard_normal((p1["neq"], 16))
        X2 = rng.standard_normal((p2["neq"], 16))
        a1 = s1.ebe_matvec_multi(X1, 16)
        a2 = s2.ebe_matvec_multi(X2, 16)
        b1 = s1.ebe_matvec_multi(X1, 16)
        s2.multi_free()
        b2 = s2.ebe_matvec_multi(X2, 16)
        s1.ebe_matvec_multi(X1[:, :8], 16)
        c1 = s1.ebe_matvec_multi(X1, 16)
    finally:
        s1.close()
        s2.close()
    assert np.array_equal(a1, b1) and np.array_equal(a1, c1)
    assert np.array_equal(a2, b2)
