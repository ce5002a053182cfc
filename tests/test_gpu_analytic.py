"""Analytic checks of the GPU path: storkm annihilates the rigid-body modes,
and the solve passes a patch test (a uniform stress state is reproduced
exactly by 20-node bricks, also with distorted interior nodes)."""
import numpy as np
import pytest

import parafem_gb300 as P

pytestmark = pytest.mark.gpu


def node_coords(g_num, g_coord, nn):
    X = np.zeros((nn, 3))
    for e in range(g_num.shape[0]):
        X[g_num[e] - 1] = g_coord[e].T
    return X


def test_storkm_annihilates_rigid_body_modes():
    """K_e r = 0 for the three translations and three rotations of each
    element of a distorted mesh (p121's B'DB: rigid motions are strain free)."""
    g_num, g_coord, nn = P.mesh_cube(3, 2, 3)
    X = node_coords(g_num, g_coord, nn) + np.random.default_rng(4).uniform(-0.08, 0.08, size=(nn, 3))
    g_coord = np.ascontiguousarray(X[g_num - 1].transpose(0, 2, 1))
    fix = P.cube_restraints(3, 2, 3, 1, nn)
    g_g, neq = P.number_equations(g_num, fix)
    with P.Solver() as s:
        s.setup(g_num, g_g, g_coord, nn, neq)
        s.set_material(100.0, 0.3)
        s.form_storkm(27)
        km = s.get_storkm()
    for e in range(g_num.shape[0]):
        Xe = g_coord[e].T - g_coord[e].T.mean(axis=0)        # 20 x 3 about the centroid
        R = np.zeros((60, 6))
        for a in range(20):
            x, y, z = Xe[a]
            R[3 * a:3 * a + 3, :3] = np.eye(3)
            R[3 * a:3 * a + 3, 3] = [0.0, -z, y]
            R[3 * a:3 * a + 3, 4] = [z, 0.0, -x]
            R[3 * a:3 * a + 3, 5] = [-y, x, 0.0]
        assert np.abs(km[e] @ R).max() <= 1e-12 * np.abs(km[e]).max()


@pytest.mark.parametrize("mode,tol", [(P.MODE_FP64_RES, 1e-12), (P.MODE_MIXED, 1e-11), (P.MODE_MIXED16, 1e-11)])
def test_patch_test_uniform_stress_on_a_distorted_mesh(mode, tol):
    """Rollers on the planes x = 0, y = 0 and on the base, uniform pressure p
    on the top face: the exact field is uz = -p (z - z0)/E, ux = nu p x/E,
    uy = nu p y/E, which every element reproduces (interior nodes moved)."""
    n, E, nu, pr = 3, 100.0, 0.3, 0.3
    g_num, g_coord, nn = P.mesh_cube(n, n, n)
    X = node_coords(g_num, g_coord, nn)
    lo, hi = X.min(axis=0), X.max(axis=0)
    inner = np.all((X > lo + 1e-9) & (X < hi - 1e-9), axis=1)
    X[inner] += np.random.default_rng(3).uniform(-0.12, 0.12, size=(inner.sum(), 3))
    g_coord = np.ascontiguousarray(X[g_num - 1].transpose(0, 2, 1))
    fix = np.ones((nn, 3), np.int32)
    for d in range(3):
        fix[np.abs(X[:, d] - lo[d]) < 1e-9, d] = 0
    g_g, neq = P.number_equations(g_num, fix)
    r = P.cube_top_pressure(n, n, g_g, neq, pr)
    with P.Solver() as s:
        s.setup(g_num, g_g, g_coord, nn, neq)
        s.set_material(E, nu)
        s.form_storkm(27)
        x, it, rel = s.solve(r, tol, 20000, mode)
    assert rel <= tol
    node = np.zeros(neq, int)
    dof = np.zeros(neq, int)
    for e in range(g_num.shape[0]):
        for a in range(20):
            for d in range(3):
                q = g_g[e, 3 * a + d]
                if q > 0:
                    node[q - 1], dof[q - 1] = g_num[e, a] - 1, d
    strain = np.array([nu * pr / E, nu * pr / E, -pr / E])   # sigma_zz = -p
    exact = strain[dof] * (X[node, dof] - lo[dof])
    assert np.abs(x - exact).max() <= 1e-6 * np.abs(exact).max()
