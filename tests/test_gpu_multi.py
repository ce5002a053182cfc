"""Several load cases per mesh (pf_solve_multi / pf_ebe_matvec_multi): the
tensor-core block product (tcgen05, three-term BF16 splits, FP32
accumulation) against FP32 CUDA cores and FP64, and the block solve against
sequential FP64 solves."""
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
    return s, prob


def test_block_products_agree():
    s, prob = setup_solver(4, 3, 3)
    try:
        rng = np.random.default_rng(1)
        Pm = rng.standard_normal((prob["neq"], 16))
        u64 = s.ebe_matvec_multi(Pm, 64)
        ref = np.stack([s.ebe_matvec(Pm[:, j], 64) for j in range(16)], axis=1)
        assert np.abs(u64 - ref).max() <= 1e-13 * np.abs(ref).max()
        for prec in (32, 16):
            u = s.ebe_matvec_multi(Pm, prec)
            assert np.abs(u - u64).max() <= 3e-6 * np.abs(u64).max(), prec
    finally:
        s.close()


def test_block_solve_matches_sequential_fp64():
    s, prob = setup_solver(6, 5, 4)
    try:
        R = P.random_top_loads(prob["g_g"], 6, 4, prob["neq"], 16, seed=7)
        X, it, rel = s.solve_multi(R, 1e-9, 20000, prec=16)
        assert (rel <= 1e-9).all()
        for j in (0, 5, 15):
            x64, it64, rel64 = s.solve(R[:, j], 1e-12, 20000, P.MODE_FP64_RES)
            assert np.linalg.norm(X[:, j] - x64) <= 1e-7 * np.linalg.norm(x64), j
        X32, it32, rel32 = s.solve_multi(R, 1e-9, 20000, prec=32)
        assert (rel32 <= 1e-9).all()
        assert np.abs(X32 - X).max() <= 1e-6 * np.abs(X).max()
    finally:
        s.close()


def test_tensor_core_block_product_keeps_translations_out_of_the_rounding():
    """The tensor-core block product is P K_e P P_e per load case; on nearly
    rigid load cases its error away from the restrained elements is far
    below that of the FP32 CUDA-core block product (no projection)."""
    s, prob = setup_solver(6, 6, 6)
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
    without touching the other's."""
    s1, p1 = setup_solver(4, 3, 3)
    s2, p2 = setup_solver(5, 4, 3, seed=4)
    try:
        rng = np.random.default_rng(15)
        X1 = rng.standard_normal((p1["neq"], 16))
        X2 = rng.standard_normal((p2["neq"], 16))
        a1 = s1.ebe_matvec_multi(X1, 16)
        a2 = s2.ebe_matvec_multi(X2, 16)
        b1 = s1.ebe_matvec_multi(X1, 16)
        s2.multi_free()
        b2 = s2.ebe_matvec_multi(X2, 16)
        c1 = s1.ebe_matvec_multi(X1, 16)
    finally:
        s1.close()
        s2.close()
    assert np.array_equal(a1, b1) and np.array_equal(a1, c1)
    assert np.array_equal(a2, b2)
