"""The timed CPU build of p121's PCG (oracle/p121_cpu.c, the bench's CPU
baseline and reference arm) against the serial-order C restatement: the
same cube, storkm, iterates and stopping iteration."""
import numpy as np

from oracle import oracle as O


def _oracle_cube(n):
    L = O.lib()
    nels = n ** 3
    g_num = np.zeros((nels, 20), np.int32)
    gc = np.zeros((nels, 3, 20))
    coord = np.zeros(60)
    num = np.zeros(20, np.int32)
    for e in range(nels):
        L.orc_geometry_20bxz(e + 1, n, n, 1.0, 1.0, 1.0, coord, num)
        g_num[e] = num
        gc[e] = coord.reshape(3, 20)
    base = np.unique(g_num[:, [0, 6, 7, 8, 11, 12, 18, 19]][np.arange(nels) % (n * n) >= n * (n - 1)])
    rest = np.zeros((len(base) + 1, 4), np.int32)
    rest[0] = [1, 1, 1, 1]
    rest[1:, 0] = base
    return gc, O.steering(g_num, rest)


def test_cpu_build_matches_restatement():
    n = 4
    c = O.CpuP121(n, n, n)
    try:
        g_g, r = c.problem()
        gc, g_ref = _oracle_cube(n)
        assert np.array_equal(g_g, g_ref)
        km = O.form_storkm(gc, 27, 100.0, 0.3)
        kc = c.storkm(0, n ** 3)
        assert np.abs(km - kc).max() <= 1e-13 * np.abs(km).max()
        dg = O.diag(g_g, km, c.neq)
        _, x10, _ = O.pcg(g_g, km, dg, r, 0.0, 10, 0)
        c.init()
        assert c.iterate(10) == 10
        assert np.abs(c.x() - x10).max() <= 1e-12 * np.abs(x10).max()
        it, x, _ = O.pcg(g_g, km, dg, r, 1e-6, 5000, 0)
        c.init()
        assert c.iterate(5000, 1e-6, 0) == it
        assert np.abs(c.x() - x).max() <= 1e-6 * np.abs(x).max()
    finally:
        c.close()
