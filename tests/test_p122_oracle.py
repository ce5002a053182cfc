"""p122 (Mohr-Coulomb viscoplasticity, 20-node bricks) on the CPU: the
oracle against the reference's recorded book run (16 ranks)."""
import json
import os

import numpy as np
import pytest

from oracle import oracle as O
from tests.conftest import GOLDEN_DIR


def book():
    with open(os.path.join(GOLDEN_DIR, "p122_golden.json")) as f:
        g = json.load(f)
    tok = g["book_mg"].replace("'", " ").split()
    mg = dict(nels=int(tok[2]), nxe=int(tok[3]), nze=int(tok[4]), nod=int(tok[5]), nip=int(tok[6]),
              aa=float(tok[7]), bb=float(tok[8]), cc=float(tok[9]), incs=int(tok[10]), phi=float(tok[11]),
              c=float(tok[12]), psi=float(tok[13]), e=float(tok[14]), v=float(tok[15]), plasits=int(tok[16]),
              cjits=int(tok[17]), plastol=float(tok[18]), cjtol=float(tok[19]),
              qinc=[float(t) for t in tok[20:20 + int(tok[10])]])
    return g["book"], mg


def book_problem(mg):
    # p12meshgen's p122 case, 20-node bricks: val = -val * aa * bb / 12 (p12meshgen.f90:420)
    return O.cube20_problem(mg["nels"], mg["nxe"], mg["nze"], mg["aa"], mg["bb"], mg["cc"],
                            -mg["aa"] * mg["bb"] / 12.0)


def printed_ulp(text):
    """One unit in the last place of an E12.4 value 0.ddddE+xx."""
    return 10.0 ** (int(text.split("E")[1]) - 4)


def check_increment(res, gold, rel=2e-4):
    """Displacement and stresses to the printed 4 digits (half a unit of
    rounding plus the PCG tolerance), iteration counts within the spread that
    16 ranks' reduction order gives."""
    t = gold["displacement_text"]
    assert abs(res[0] - float(t)) <= 0.5 * printed_ulp(t) + rel * abs(res[0]), (res[0], t)
    for k in range(3):
        t = gold["stress_text"][k]
        assert abs(res[1 + k] - float(t)) <= 0.5 * printed_ulp(t) + rel * abs(res[1 + k]), (k, res[1 + k], t)
    assert abs(res[5] - gold["plastic_iterations"]) <= 2
    assert abs(res[4] - gold["cj_iterations"]) <= 0.02 * gold["cj_iterations"] + 5


@pytest.mark.slow
def test_oracle_reproduces_p122_book_increments():
    gold, mg = book()
    prob = book_problem(mg)
    assert (prob["nn"], prob["nr"], prob["neq"]) == (gold["nn"], gold["nr"], gold["neq"])
    out, _ = O.run_p122(prob, mg["nip"], mg["phi"], mg["c"], mg["psi"], mg["e"], mg["v"], mg["qinc"][:3],
                        mg["plasits"], mg["cjits"], mg["plastol"], mg["cjtol"])
    assert out.shape[0] == 3
    for k in range(3):
        check_increment(out[k], gold["increments"][k])


def test_mohr_coulomb_routines():
    L = O.lib()
    import ctypes
    s = np.array([-10.0, -4.0, -7.0, 1.5, -0.5, 2.0])
    sigm, dsbar, theta = ctypes.c_double(), ctypes.c_double(), ctypes.c_double()
    L.orc_invar(s, ctypes.byref(sigm), ctypes.byref(dsbar), ctypes.byref(theta))
    assert abs(sigm.value - (-7.0)) < 1e-15
    # dsbar = sqrt(3 J2); J2 from the deviator
    dev = s[:3] - sigm.value
    j2 = 0.5 * (dev @ dev) + s[3] ** 2 + s[4] ** 2 + s[5] ** 2
    assert abs(dsbar.value - np.sqrt(3 * j2)) < 1e-12 * dsbar.value
    assert -np.pi / 6 <= theta.value <= np.pi / 6
    # phi = 0: Tresca-like, f = dsbar cos(theta)/sqrt(3) - c
    f = L.orc_mocouf(0.0, 2.0, sigm.value, dsbar.value, theta.value)
    assert abs(f - (dsbar.value * np.cos(theta.value) / np.sqrt(3.0) - 2.0)) < 1e-12
    m1, m2, m3 = np.zeros(36), np.zeros(36), np.zeros(36)
    L.orc_formm(s, m1, m2, m3)
    for m in (m1, m2, m3):
        mm = m.reshape(6, 6)
        assert np.array_equal(mm, mm.T)


def demo_node_displacements(prob, totd):
    """Nodal displacements (nn, 3) of an equation vector, 0 at restrained freedoms."""
    node_eq = np.zeros((prob["nn"], 3), np.int64)
    for e in range(prob["g_num"].shape[0]):
        node_eq[prob["g_num"][e] - 1] = prob["g_g"][e].reshape(-1, 3)
    return np.concatenate([[0.0], totd])[node_eq]


def within_printed(x, gold):
    """x against E12.4 text values: within half a unit in the fourth digit."""
    ulp = np.where(gold != 0, 10.0 ** (np.floor(np.log10(np.abs(np.where(gold != 0, gold, 1.0)))) - 3), 0.0)
    return np.abs(x - gold) <= 0.5 * ulp * (1 + 1e-9) + 1e-15


def test_oracle_reproduces_p122_demo_run():
    """The reference's demo run (8-node bricks, 19 fixed freedoms under
    displacement control, 4 ranks): every increment's .res figures, iteration
    counts included, and all ten ensi.DISPL fields."""
    prob = O.p122_demo_problem(GOLDEN_DIR)
    m, gold = prob["mat"], prob["gold"]
    assert (prob["nn"], prob["nr"], prob["neq"]) == (gold["nn"], gold["nr"], gold["neq"])
    out, totd = O.run_p122n(prob, m["nip"], m["phi"], m["c"], m["psi"], m["e"], m["v"], prob["qinc"], m["plasits"],
                            m["cjits"], m["plastol"], m["cjtol"], fix_eq=prob["fix_eq"], fix_val=prob["fix_val"],
                            keep_totd=True)
    assert out.shape[0] == len(gold["increments"]) == 10
    for k, g in enumerate(gold["increments"]):
        assert within_printed(out[k, 0], float(g["displacement_text"])), (k, out[k, 0])
        for j in range(3):
            assert within_printed(out[k, 1 + j], float(g["stress_text"][j])), (k, j, out[k, 1 + j])
        assert (out[k, 4], out[k, 5]) == (g["cj_iterations"], g["plastic_iterations"]), k
        assert np.all(within_printed(demo_node_displacements(prob, totd[k]), prob["displ"][k])), k


def test_p122_demo_numbering_is_find_g():
    """find_g's numbering (freedoms in node order) gives every equation one
    freedom; 3,636 equations as the reference printed."""
    prob = O.p122_demo_problem(GOLDEN_DIR)
    g = prob["g_g"]
    owners = {}
    for e in range(g.shape[0]):
        for a in range(8):
            for d in range(3):
                if g[e, 3 * a + d]:
                    owners.setdefault(int(g[e, 3 * a + d]), set()).add((int(prob["g_num"][e, a]), d))
    assert sorted(owners) == list(range(1, prob["neq"] + 1))
    assert all(len(o) == 1 for o in owners.values())
    assert prob["neq"] == prob["gold"]["neq"] == 3636
