"""p122 (Mohr-Coulomb viscoplasticity, 20-node bricks, load control) on the
GPU against the oracle and the reference's recorded book run."""
import numpy as np
import pytest

import parafem_gb300 as P
from oracle import oracle as O
from tests.test_p122_oracle import book, book_problem, check_increment

pytestmark = pytest.mark.gpu


def gpu_run(prob, mg, nincs, keep_totd=False):
    with P.Solver() as s:
        s.setup(prob["g_num"], prob["g_g"], prob["g_coord"], prob["nn"], prob["neq"])
        s.set_material(mg["e"], mg["v"])
        s.form_storkm(mg["nip"])
        return s.p122_solve(mg["nip"], mg["phi"], mg["c"], mg["psi"], mg["qinc"][:nincs], mg["plasits"],
                            mg["cjits"], mg["plastol"], mg["cjtol"], prob["ld0"], keep_totd)


def small_case():
    # examples/5th_ed/p122/mg/p122_small.mg sizes; c = 30 and phi = 20 yield from the first increment
    mg = dict(nels=1000, nxe=10, nze=10, nip=8, aa=1.0, bb=1.0, cc=1.0, phi=20.0, c=30.0, psi=5.0, e=1.0e4,
              v=0.3, plasits=200, cjits=1000, plastol=1e-4, cjtol=1e-6, qinc=[200.0, 100.0])
    return O.cube20_problem(mg["nels"], mg["nxe"], mg["nze"], mg["aa"], mg["bb"], mg["cc"],
                            -mg["aa"] * mg["bb"] / 12.0), mg


def test_p122_small_matches_oracle():
    prob, mg = small_case()
    ref, tref = O.run_p122(prob, mg["nip"], mg["phi"], mg["c"], mg["psi"], mg["e"], mg["v"], mg["qinc"],
                           mg["plasits"], mg["cjits"], mg["plastol"], mg["cjtol"], keep_totd=True)
    out, totd = gpu_run(prob, mg, len(mg["qinc"]), keep_totd=True)
    assert out.shape == ref.shape
    assert ref[0, 5] > 5                                        # the case yields
    for k in range(out.shape[0]):
        # FP64 on both sides, different summation orders: the plastic loop may stop an iteration apart
        assert abs(out[k, 5] - ref[k, 5]) <= 2
        assert abs(out[k, 4] - ref[k, 4]) <= 0.03 * ref[k, 4] + 5
        np.testing.assert_allclose(out[k, :4], ref[k, :4], rtol=5e-4)
        assert np.linalg.norm(totd[k] - tref[k]) <= 5e-4 * np.linalg.norm(tref[k])


@pytest.mark.slow
def test_p122_book_increments_on_the_gpu():
    gold, mg = book()
    prob = book_problem(mg)
    out, _ = gpu_run(prob, mg, 4)
    assert out.shape[0] == 4
    for k in range(4):
        check_increment(out[k], gold["increments"][k])


def test_p122_job_writes_res_and_displacements(tmp_path):
    job = str(tmp_path / "p122s")
    with open(job + ".mg", "w") as f:
        f.write("'p122'\n'parafem' 1000 10 10 20 8\n1.0 1.0 1.0 2\n20.0 30.0 5.0 1.0e4 0.3\n"
                "200 1000 1.e-4 1.e-6\n200.0 100.0\n")
    P.p12meshgen(job)
    assert P.p122_run(job) == 2
    prob, mg = small_case()
    ref, tref = O.run_p122(prob, 8, 20.0, 30.0, 5.0, 1.0e4, 0.3, [200.0, 100.0], 200, 1000, 1e-4, 1e-6,
                           keep_totd=True)
    res = open(job + ".res").read().splitlines()
    # p122.f90:62-63 writes '(A,3(I7,A))' with " restrained and   " before neq.
    assert res[1] == "There are    4961 nodes   1541 restrained and   %7d equations" % prob["neq"]
    incs = [k for k, ln in enumerate(res) if ln.startswith("Load Increment")]
    assert len(incs) == 2
    for i, k in enumerate(incs):
        disp = float(res[k + 1].split()[-1])
        assert abs(disp - ref[i, 0]) <= 1e-3 * abs(ref[i, 0])
        sig = [float(t) for t in res[k + 3].split()]
        np.testing.assert_allclose(sig, ref[i, 1:4], rtol=1e-3)
    disp = open(job + ".ensi.DISPL-000002").read().splitlines()
    assert disp[:4] == ["Alya Ensight Gold --- Vector per-node variable file", "part", "    1", "coordinates"]
    assert len(disp) == 4 + 3 * 4961


# ---------------------------------------------------------------------------
# The reference's demo deck: 8-node bricks, 19 fixed freedoms (displacement
# control), no loaded nodes (examples/5th_ed/p122/demo)
from tests.conftest import GOLDEN_DIR  # noqa: E402
from tests.test_p122_oracle import demo_node_displacements, within_printed  # noqa: E402


def demo_gpu(prob, keep_totd=True):
    m = prob["mat"]
    with P.Solver() as s:
        s.setup_solid8(prob["g_num"], prob["g_g"], prob["g_coord"], prob["nn"], prob["neq"])
        s.set_material(m["e"], m["v"])
        s.form_storkm(m["nip"])
        return s.p122_solve_fixed(m["nip"], m["phi"], m["c"], m["psi"], prob["qinc"], m["plasits"], m["cjits"],
                                  m["plastol"], m["cjtol"], fix_eqs=prob["fix_eq"], fix_vals=prob["fix_val"],
                                  keep_totd=keep_totd)


def test_p122_demo_on_the_gpu_reproduces_the_reference_run():
    """Every increment of the demo run against the reference's .res (the
    printed 4 digits; the iteration counts within the window that summation
    order opens) and the ten ensi.DISPL fields, and against the oracle."""
    prob = O.p122_demo_problem(GOLDEN_DIR)
    out, totd = demo_gpu(prob)
    m = prob["mat"]
    ref, tref = O.run_p122n(prob, m["nip"], m["phi"], m["c"], m["psi"], m["e"], m["v"], prob["qinc"],
                            m["plasits"], m["cjits"], m["plastol"], m["cjtol"], fix_eq=prob["fix_eq"],
                            fix_val=prob["fix_val"], keep_totd=True)
    gold = prob["gold"]["increments"]
    assert out.shape[0] == ref.shape[0] == 10
    for k in range(10):
        assert abs(out[k, 5] - gold[k]["plastic_iterations"]) <= 1, (k, out[k, 5])
        assert abs(out[k, 4] - gold[k]["cj_iterations"]) <= 0.02 * gold[k]["cj_iterations"] + 2, (k, out[k, 4])
        np.testing.assert_allclose(out[k, :4], ref[k, :4], rtol=2e-4)
        check = [within_printed(out[k, 0], float(gold[k]["displacement_text"]))]
        check += [within_printed(out[k, 1 + j], float(gold[k]["stress_text"][j])) for j in range(3)]
        # the printed figures, allowing 2e-4 relative beyond half a unit of rounding
        for ok, val, txt in zip(check, out[k, :4], [gold[k]["displacement_text"]] + gold[k]["stress_text"]):
            assert ok or abs(val - float(txt)) <= 2e-4 * abs(val) + 0.5 * 10.0 ** (int(txt.split("E")[1]) - 4), \
                (k, val, txt)
        assert np.linalg.norm(totd[k] - tref[k]) <= 2e-4 * np.linalg.norm(tref[k])
        disp = demo_node_displacements(prob, totd[k])
        gd = prob["displ"][k]
        assert np.abs(disp - gd).max() <= 1e-3 * np.abs(gd).max(), k


def test_p122_demo_deck_files_through_p122_run(tmp_path):
    """The demo deck written as the reference's files (.dat, .d, .bnd, .fix)
    and run as the p122 program: its .res lines and DISPL files."""
    prob = O.p122_demo_problem(GOLDEN_DIR)
    job = str(tmp_path / "p122_demo")
    with open(job + ".dat", "w") as f:
        f.write(prob["dat"])
    with open(job + ".d", "w") as f:
        f.write("*THREE_DIMENSIONAL\n*NODES\n")
        for i, (x, y, z) in enumerate(prob["coords"]):
            f.write("%6d %.17g %.17g %.17g\n" % (i + 1, x, y, z))
        f.write("*ELEMENTS\n")
        for e, row in enumerate(prob["g_num"]):
            f.write("%6d 3 8 1 %s %d\n" % (e + 1, " ".join(str(int(v)) for v in row), int(prob["matid"][e])))
    with open(job + ".bnd", "w") as f:
        for row in prob["rest"]:
            f.write("%d %d %d %d\n" % tuple(int(v) for v in row))
    with open(job + ".fix", "w") as f:
        for nd, sn, val in zip(prob["fix_node"], prob["fix_sense"], prob["fix_val"]):
            f.write("%d %d %.17g\n" % (nd, sn, val))
    assert P.p122_run(job) == 10
    res = open(job + ".res").read().splitlines()
    assert res[1] == "There are    1469 nodes    497 restrained and      3636 equations"
    assert res[3] == "The critical timestep is     0.5200E-03"
    incs = [k for k, ln in enumerate(res) if ln.startswith("Load Increment")]
    gold = prob["gold"]["increments"]
    assert len(incs) == 10
    for i, k in enumerate(incs):
        assert abs(float(res[k + 1].split()[-1]) - float(gold[i]["displacement_text"])) <= \
            2e-3 * abs(float(gold[i]["displacement_text"]))
        assert abs(int(res[k + 5].split()[-1]) - gold[i]["plastic_iterations"]) <= 1
        disp = open(job + ".ensi.DISPL-%06d" % (i + 1)).read().splitlines()
        assert disp[:4] == ["Alya Ensight Gold --- Vector per-node variable file", "part", "    1", "coordinates"]
        vals = np.array([float(t) for t in disp[4:]]).reshape(3, -1).T
        gd = prob["displ"][i]
        assert np.abs(vals - gd).max() <= 1e-3 * np.abs(gd).max(), i
