"""Analytic checks of the oracle's element matrices (CPU, no recorded run).

K_e = sum over the Gauss points of B'DB det w (p121.f90:54-64 for 20-node
bricks, p122.f90:76-84 with nod = 8) and kc = sum of (kx dx dx' + ky dy dy' +
kz dz dz') det w (p123.f90:70-85) must be symmetric and positive
semi-definite, with null spaces that are exactly the rigid-body modes (six
for elasticity, the constant for the Laplace brick) under full integration.
A linear displacement field (constant strain) must store exactly the strain
energy of that strain over the element's volume.  The Gauss rule must
integrate its polynomial degree exactly and the shape-function derivatives
must be complete.  These pin the oracle's SAMPLE, SHAPE_DER, DEEMAT, BEEMAT,
DETERMINANT and INVERT, and its assembly and PCG (a patch test),
independently of the reference's recorded runs.
"""
import numpy as np
import pytest

from oracle import oracle as O


def _brick(nod, aa, bb, cc, distort, seed):
    """One element of GEOMETRY_20BXZ / GEOMETRY_8BXZ, coord (3, nod); with
    distort, every node moved by up to distort * the element size."""
    coord = np.zeros((3, nod))
    num = np.zeros(nod, np.int32)
    geo = O.lib().orc_geometry_20bxz if nod == 20 else O.lib().orc_geometry_8bxz
    geo(1, 1, 1, aa, bb, cc, coord, num)
    if distort:
        rng = np.random.default_rng(seed)
        coord = coord + distort * rng.uniform(-1.0, 1.0, coord.shape) * np.array([[aa], [bb], [cc]])
    return np.ascontiguousarray(coord)


def _rigid_modes(coord):
    """The six rigid-body modes of an elasticity element, dofs (x, y, z) per node."""
    x, y, z = coord
    nod = coord.shape[1]
    r = np.zeros((6, 3 * nod))
    for d in range(3):
        r[d, d::3] = 1.0
    r[3, 0::3], r[3, 1::3] = -y, x      # rotation about z
    r[4, 1::3], r[4, 2::3] = -z, y      # about x
    r[5, 0::3], r[5, 2::3] = z, -x      # about y
    return r


def _elasticity_k(nod, coord, nip, e, v, exact=False):
    if nod == 20:
        km = O.form_storkm(coord[None], nip, e, v, exact_weights=exact)[0]
    else:
        km = O.form_storkm8(coord[None], nip, e, v)[0]
    return km.T   # km[j, i] = K(i, j)


@pytest.mark.parametrize("nod,nip", [(20, 27), (20, 8), (8, 8)])
@pytest.mark.parametrize("distort", [0.0, 0.12])
def test_elasticity_matrix_is_symmetric_psd_with_rigid_null_space(nod, nip, distort):
    coord = _brick(nod, 1.0, 2.0, 0.5, distort, seed=nod * 100 + nip)
    k = _elasticity_k(nod, coord, nip, 100.0, 0.3)
    scale = np.abs(k).max()
    assert np.abs(k - k.T).max() <= 1e-13 * scale
    r = _rigid_modes(coord)
    for mode in r:
        assert np.linalg.norm(k @ mode) <= 1e-12 * scale * np.linalg.norm(mode)
    lam = np.linalg.eigvalsh(0.5 * (k + k.T))
    assert lam.min() >= -1e-11 * lam.max()
    # full integration: the rigid-body modes are the whole null space; the
    # 20-node brick under the 2x2x2 rule has six spurious zero-energy modes
    # besides them, the known rank deficiency of that reduced rule
    n0 = int((lam <= 1e-9 * lam.max()).sum())
    assert n0 == (12 if (nod, nip) == (20, 8) else 6), (n0, lam[:14] / lam.max())


@pytest.mark.parametrize("nod,nip", [(20, 27), (20, 8), (8, 8)])
def test_constant_strain_stores_its_exact_energy(nod, nip):
    aa, bb, cc, e, v = 1.0, 2.0, 0.5, 100.0, 0.3
    coord = _brick(nod, aa, bb, cc, 0.0, seed=0)
    exact = nod == 20   # exact Gauss weights (the 27-point rule's default factors are FP32)
    k = _elasticity_k(nod, coord, nip, e, v, exact=exact)
    rng = np.random.default_rng(7 + nod + nip)
    a = rng.normal(size=(3, 3))
    eps = 0.5 * (a + a.T)
    u = (eps @ coord).T.reshape(-1)     # u(node) = eps x(node), dofs (x, y, z) per node
    lam_ = e * v / ((1 + v) * (1 - 2 * v))
    mu = e / (2 * (1 + v))
    energy = (lam_ * np.trace(eps) ** 2 + 2 * mu * np.sum(eps * eps)) * aa * bb * cc
    assert abs(u @ k @ u - energy) <= 1e-11 * abs(energy)


def test_default_27_point_weights_follow_the_single_precision_factors():
    """SAMPLE's 27-point weights are products of 5./9. and 8./9. in single
    precision (new_library.f90:1491-1514): the energy of a constant strain
    then differs from the exact one by the FP32 rounding of those factors,
    about 1e-8 relative, not by zero."""
    coord = _brick(20, 1.0, 1.0, 1.0, 0.0, seed=0)
    rng = np.random.default_rng(3)
    a = rng.normal(size=(3, 3))
    eps = 0.5 * (a + a.T)
    u = (eps @ coord).T.reshape(-1)
    w_exact = u @ _elasticity_k(20, coord, 27, 100.0, 0.3, exact=True) @ u
    w_fp32 = u @ _elasticity_k(20, coord, 27, 100.0, 0.3, exact=False) @ u
    rel = abs(w_fp32 - w_exact) / abs(w_exact)
    assert 1e-10 < rel < 1e-6


@pytest.mark.parametrize("distort", [0.0, 0.12])
def test_laplace_matrix_has_the_constant_as_its_null_space(distort):
    aa, bb, cc, kx, ky, kz = 1.0, 2.0, 0.5, 1.0, 2.0, 3.0
    coord = _brick(8, aa, bb, cc, distort, seed=11)
    kc = O.form_storkc(coord[None], 8, kx, ky, kz)[0].T
    scale = np.abs(kc).max()
    assert np.abs(kc - kc.T).max() <= 1e-13 * scale
    assert np.abs(kc.sum(axis=1)).max() <= 1e-12 * scale
    lam = np.linalg.eigvalsh(0.5 * (kc + kc.T))
    assert lam.min() >= -1e-12 * lam.max()
    assert int((lam <= 1e-9 * lam.max()).sum()) == 1
    if distort == 0.0:
        g = np.array([0.3, -1.2, 0.7])
        phi = g @ coord                  # a linear potential, constant gradient g
        energy = (kx * g[0] ** 2 + ky * g[1] ** 2 + kz * g[2] ** 2) * aa * bb * cc
        assert abs(phi @ kc @ phi - energy) <= 1e-11 * energy


@pytest.mark.parametrize("exact_weights,bound", [(True, 1e-10), (False, 1e-7)])
def test_oracle_solve_passes_the_patch_test(exact_weights, bound):
    """The oracle's assembly, Jacobi diagonal and PCG (p121.f90:65-104) on a
    3x3x3 cube with distorted interior nodes: rollers on the planes x = 0,
    y = 0 and on the base, uniform pressure p on the top face.  The exact
    field is uz = -p (z - z0)/E, ux = nu p x/E, uy = nu p y/E, a constant
    stress state that every 20-node brick reproduces.  With SAMPLE's
    single-precision 27-point factors (the reference's default) the stiffness
    and the exactly integrated pressure loads differ by those factors'
    rounding, a few 1e-8 relative."""
    import parafem_gb300 as P   # host-side mesh, numbering and load functions (no GPU)
    n, e, nu, pr = 3, 100.0, 0.3, 0.3
    g_num, g_coord, nn = P.mesh_cube(n, n, n)
    X = np.zeros((nn, 3))
    for el in range(g_num.shape[0]):
        X[g_num[el] - 1] = g_coord[el].T
    lo, hi = X.min(axis=0), X.max(axis=0)
    inner = np.all((X > lo + 1e-9) & (X < hi - 1e-9), axis=1)
    X[inner] += np.random.default_rng(3).uniform(-0.12, 0.12, size=(inner.sum(), 3))
    g_coord = np.ascontiguousarray(X[g_num - 1].transpose(0, 2, 1))
    fix = np.ones((nn, 3), np.int32)
    for d in range(3):
        fix[np.abs(X[:, d] - lo[d]) < 1e-9, d] = 0
    g_g, neq = P.number_equations(g_num, fix)
    r = P.cube_top_pressure(n, n, g_g, neq, pr)
    km = O.form_storkm(g_coord, 27, e, nu, exact_weights=exact_weights)
    dg = O.diag(g_g, km, neq)
    it, x, rel = O.pcg(g_g, km, dg, r, 1e-12, 20000, 1)
    assert rel <= 1e-12 and it < 20000
    node = np.zeros(neq, int)
    dof = np.zeros(neq, int)
    for el in range(g_num.shape[0]):
        for a in range(20):
            for d in range(3):
                q = g_g[el, 3 * a + d]
                if q > 0:
                    node[q - 1], dof[q - 1] = g_num[el, a] - 1, d
    strain = np.array([nu * pr / e, nu * pr / e, -pr / e])   # sigma_zz = -p
    exact = strain[dof] * (X[node, dof] - lo[dof])
    assert np.abs(x - exact).max() <= bound * np.abs(exact).max()


@pytest.mark.parametrize("nip,deg", [(8, 3), (27, 5)])
def test_gauss_rule_integrates_its_polynomial_degree_exactly(nip, deg):
    """SAMPLE('hexahedron', nip) (new_library.f90:1397-1520) with exact
    weights: the tensor Gauss rule integrates xi^a eta^b zeta^c over the
    reference cube exactly for a, b, c <= deg."""
    pts, wts = np.zeros(3 * nip), np.zeros(nip)
    O.lib().orc_sample(nip, pts, wts, 1)
    s = pts.reshape(3, nip)
    for a in range(deg + 1):
        for b in range(deg + 1):
            for c in range(deg + 1):
                exact = np.prod([0.0 if k % 2 else 2.0 / (k + 1) for k in (a, b, c)])
                got = np.sum(wts * s[0] ** a * s[1] ** b * s[2] ** c)
                assert abs(got - exact) <= 1e-14, (a, b, c, got, exact)


@pytest.mark.parametrize("nod", [20, 8])
def test_shape_derivatives_are_complete(nod):
    """SHAPE_DER (new_library.f90:865-896 for 20 nodes; the 8-node brick):
    the derivatives sum to zero over the nodes at any point, and on a
    box-shaped element the Jacobian is the same at every point, with
    8 det J the element's volume."""
    aa, bb, cc = 1.0, 2.0, 0.5
    coord = _brick(nod, aa, bb, cc, 0.0, seed=0)
    f = O.lib().orc_shape_der20 if nod == 20 else O.lib().orc_shape_der8
    rng = np.random.default_rng(5)
    jac0 = None
    for xi, eta, zeta in rng.uniform(-1.0, 1.0, size=(20, 3)):
        der = np.zeros(3 * nod)
        f(der, xi, eta, zeta)
        d = der.reshape(nod, 3).T          # d[direction, node]
        assert np.abs(d.sum(axis=1)).max() <= 1e-14
        jac = d @ coord.T
        jac0 = jac if jac0 is None else jac0
        assert np.abs(jac - jac0).max() <= 1e-13
    assert abs(8.0 * abs(np.linalg.det(jac0)) - aa * bb * cc) <= 1e-13


def test_p123_oracle_passes_the_laplace_patch_test():
    """p123's storkc, diagonal, penalty fixed freedoms and PCG
    (p123.f90:70-148) on a 3x3x3 box of 8-node bricks with distorted
    interior nodes: the potential fixed to 0 on x = 0 and to g on x = 1 by
    the penalty method, no flux elsewhere.  The exact potential g x is
    linear, which every 8-node brick reproduces."""
    n, g, penalty = 3, 2.5, 1e20
    g_num, g_coord = O.box8_mesh(n, n, n, 1.0 / n, 1.0 / n, 1.0 / n)
    nn = (n + 1) ** 3
    X = np.zeros((nn, 3))
    for el in range(g_num.shape[0]):
        X[g_num[el] - 1] = g_coord[el].T
    lo, hi = X.min(axis=0), X.max(axis=0)
    inner = np.all((X > lo + 1e-9) & (X < hi - 1e-9), axis=1)
    X[inner] += np.random.default_rng(9).uniform(-0.04, 0.04, size=(inner.sum(), 3))
    g_coord = np.ascontiguousarray(X[g_num - 1].transpose(0, 2, 1))
    g_g, neq = np.ascontiguousarray(g_num, dtype=np.int32), nn   # no restrained node: equation = node
    kc = O.form_storkc(g_coord, 8, 1.0, 1.0, 1.0)
    dg = O.diag8(g_g, kc, neq)
    fixed = np.flatnonzero((np.abs(X[:, 0] - lo[0]) < 1e-9) | (np.abs(X[:, 0] - hi[0]) < 1e-9))
    value = g * (X[fixed, 0] - lo[0])
    dg[fixed] += penalty
    store = dg[fixed].copy()
    r = np.zeros(neq)
    r[fixed] = store * value
    it, x, _ = O.pcg123(g_g, kc, dg, r, 1e-12, 5000, fix_eq=fixed + 1, fix_store=store)
    assert it < 5000
    exact = g * (X[:, 0] - lo[0])
    assert np.abs(x - exact).max() <= 1e-9 * g
