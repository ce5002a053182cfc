"""Continuous batching (pf_batch_*): each result is the same alone and in the
mix, agrees with the single-mesh solver, and admission respects the budget."""
import numpy as np
import pytest

import parafem_gb300 as P

pytestmark = pytest.mark.gpu

SPECS = [  # (nxe, nye, nze, E seed, pressure)
    (3, 4, 2, 1, 1.0),
    (5, 3, 3, 2, 0.7),
    (4, 4, 4, 3, 1.6),
    (2, 6, 3, 4, 1.2),
]


def request(spec):
    nxe, nye, nze, seed, pres = spec
    prob = P.cube_problem(nxe, nye, nze, pressure=pres)
    nels = nxe * nye * nze
    e, v = P.random_material(nels, seed, 10.0, 1000.0, 0.2, 0.35)
    return prob, e, v


def admit(b, prob, e, v, tol=1e-9):
    return b.admit(prob["g_num"], prob["g_g"], prob["g_coord"], prob["nn"], prob["neq"], e, v, prob["r"], tol=tol)


def test_same_alone_and_in_the_mix():
    reqs = [request(sp) for sp in SPECS]
    cap = max(p["neq"] for p, _, _ in reqs)
    alone = []
    for prob, e, v in reqs:
        with P.Batch(2 << 30, 8) as b:
            sid = admit(b, prob, e, v)
            res = b.run_all(cap)
            alone.append(res[sid])
    with P.Batch(2 << 30, 8) as b:
        ids = [admit(b, *r) for r in reqs[:2]]
        b.launch(5)                       # two solves iterate ...
        b.sync()
        ids += [admit(b, *r) for r in reqs[2:]]   # ... while two more arrive
        res = b.run_all(cap, chunk=3)
    for k, sid in enumerate(ids):
        it_a, rel_a, x_a = alone[k]
        it_m, rel_m, x_m = res[sid]
        assert it_a == it_m
        assert np.array_equal(x_a, x_m)          # bitwise: per-mesh reduction order
        assert rel_m <= 1e-9


def test_batch_matches_single_solver():
    prob, e, v = request(SPECS[2])
    with P.Solver() as s:
        s.setup(prob["g_num"], prob["g_g"], prob["g_coord"], prob["nn"], prob["neq"])
        s.set_material(e, v)
        s.form_storkm(27)
        x_ref, it_ref, rel_ref = s.solve(prob["r"], 1e-9, 20000, P.MODE_FP64_RES)
    with P.Batch(1 << 30, 4) as b:
        sid = admit(b, prob, e, v)
        it, rel, x = b.run_all(prob["neq"])[sid]
    assert abs(it - it_ref) <= 3
    assert np.linalg.norm(x - x_ref) <= 1e-7 * np.linalg.norm(x_ref)
    # the reported FP64 true residual equals one computed from the returned x
    with P.Solver() as s:
        s.setup(prob["g_num"], prob["g_g"], prob["g_coord"], prob["nn"], prob["neq"])
        s.set_material(e, v)
        s.form_storkm(27)
        kx = s.ebe_matvec(x, 64)
    rel_py = np.linalg.norm(prob["r"] - kx) / np.linalg.norm(prob["r"])
    assert 0.0 < rel <= 1e-9, (rel, rel_py)
    assert abs(rel - rel_py) <= 0.05 * rel_py, (rel, rel_py)


def test_admission_is_bounded_by_the_budget():
    prob, e, v = request(SPECS[2])        # 64 elements
    with P.Batch(64 * 32_000 * 2 + (1 << 20), 16) as b:   # room for about two such meshes
        cap_el, _ = b.capacity()
        admitted = []
        for _ in range(6):
            sid = admit(b, prob, e, v)
            if sid is None:
                break
            admitted.append(sid)
        assert 1 <= len(admitted) < 6
        assert len(admitted) * 64 <= cap_el
        res = b.run_all(prob["neq"])
        assert sorted(res) == admitted
        # retired solves freed their ranges: the next request fits again
        assert admit(b, prob, e, v) is not None


@pytest.mark.parametrize("prec", [32, 16])
def test_mixed_batch_same_alone_and_in_the_mix_and_accurate(prec):
    reqs = [request(sp) for sp in SPECS[:3]]
    cap = max(p["neq"] for p, _, _ in reqs)
    alone = []
    for prob, e, v in reqs:
        with P.Batch(2 << 30, 8, prec=prec) as b:
            sid = admit(b, prob, e, v)
            alone.append(b.run_all(cap)[sid])
    with P.Batch(2 << 30, 8, prec=prec) as b:
        ids = [admit(b, *r) for r in reqs]
        res = b.run_all(cap, chunk=5)
    for k, sid in enumerate(ids):
        assert alone[k][0] == res[sid][0]
        assert np.array_equal(alone[k][2], res[sid][2])
        prob, e, v = reqs[k]
        with P.Solver() as s:
            s.setup(prob["g_num"], prob["g_g"], prob["g_coord"], prob["nn"], prob["neq"])
            s.set_material(e, v)
            s.form_storkm(27)
            x_ref, _, _ = s.solve(prob["r"], 1e-12, 20000, P.MODE_FP64_RES)
        it, rel, x = res[sid]
        assert 0.0 < rel <= 1e-9
        assert np.linalg.norm(x - x_ref) <= 1e-7 * np.linalg.norm(x_ref)


@pytest.mark.parametrize("prec", [64, 32, 16])
def test_graph_replay_matches_direct_launches(prec):
    reqs = [request(sp) for sp in SPECS]
    cap = max(p["neq"] for p, _, _ in reqs)
    runs = []
    for graphs in (True, False):
        with P.Batch(2 << 30, 8, prec=prec) as b:
            b.set_graphs(graphs)
            ids = [admit(b, *r) for r in reqs[:3]]
            b.launch(6)
            b.sync()
            ids += [admit(b, *reqs[3])]      # the tables change: a new graph
            res = b.run_all(cap, chunk=4)
            runs.append([res[i] for i in ids])
    for (it_g, rel_g, x_g), (it_d, rel_d, x_d) in zip(*runs):
        assert it_g == it_d and rel_g == rel_d
        assert np.array_equal(x_g, x_d)


def test_batch_solution_matches_oracle_pcg():
    """A batched solve of a small heterogeneous mesh against the C
    restatement of p121's PCG (relative-residual stop at 1e-12) on the
    oracle's own storkm, so the serving engine is pinned to the oracle
    directly, not only through the single-mesh solver."""
    from oracle import oracle as O
    prob, e, v = request(SPECS[1])
    with P.Batch(1 << 30, 4) as b:
        sid = admit(b, prob, e, v, tol=1e-10)
        it, rel, x = b.run_all(prob["neq"])[sid]
    assert rel <= 1e-10
    km = O.form_storkm(prob["g_coord"], 27, e, v)
    dg = O.diag(prob["g_g"], km, prob["neq"])
    _, xr, _ = O.pcg(prob["g_g"], km, dg, np.ascontiguousarray(prob["r"]), 1e-12, 20000, 1)
    assert np.linalg.norm(x - xr) <= 1e-7 * np.linalg.norm(xr)
