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
