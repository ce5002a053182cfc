"""p123 (3-D Laplace, 8-node bricks) on the CPU: the oracle against the
reference's recorded book run, and the library's host side (mesh, restraints,
numbering, deck writer) against the oracle's restatement."""
import json
import os

import numpy as np
import pytest

import parafem_gb300 as P
from oracle import oracle as O
from tests.conftest import GOLDEN_DIR, fortran_e


@pytest.fixture(scope="module")
def golden123():
    with open(os.path.join(GOLDEN_DIR, "p123_golden.json")) as f:
        return json.load(f)


def _mg_values(mg_text):
    tok = mg_text.replace("'", " ").split()
    return dict(nels=int(tok[2]), nxe=int(tok[3]), nze=int(tok[4]), nip=int(tok[5]), aa=float(tok[6]),
                bb=float(tok[7]), cc=float(tok[8]), kx=float(tok[9]), ky=float(tok[10]), kz=float(tok[11]),
                tol=float(tok[12]), limit=int(tok[13]), loaded=int(tok[14]), fixed=int(tok[15]))


@pytest.mark.slow
def test_oracle_reproduces_p123_book_run(golden123):
    """examples/5th_ed/p123/book: 200^3 bricks, 16 ranks on the reference
    machine; the restatement reproduces its counts, load and potentials."""
    g = golden123["book"]
    m = _mg_values(golden123["book_mg"])
    nye = m["nels"] // m["nxe"] // m["nze"]
    res = O.run_p123_box(m["nxe"], nye, m["nze"], m["aa"], m["bb"], m["cc"], m["kx"], m["ky"], m["kz"],
                         m["tol"], m["limit"], m["nip"])
    assert (res["nn"], res["nr"], res["neq"]) == (g["nn"], g["nr"], g["neq"])
    assert fortran_e(res["q"]).strip() == g["total_load_text"]
    # the reference ran on 16 ranks: the reduction order moves the stop by an iteration or two
    assert abs(res["iters"] - g["iterations"]) <= 2
    for (fq, text) in g["potentials"]:
        assert fq == res["nres"] + g["potentials"].index([fq, text])
        assert fortran_e(res["x"][fq - 1]).strip() == text


def test_host_mesh_restraints_and_numbering_match_oracle():
    nxe, nye, nze = 5, 4, 6
    prob = P.box8_problem(nxe, nye, nze, 0.3, 0.4, 0.5)
    g_num, g_coord = O.box8_mesh(nxe, nye, nze, 0.3, 0.4, 0.5)
    assert np.array_equal(prob["g_num"], g_num)
    assert np.array_equal(prob["g_coord"], g_coord)
    rest = O.box8_rest(nxe, nye, nze)
    assert rest.shape[0] == (nxe + 1) * (nye + 1) + (nxe + 1) * nze + nye * nze
    assert np.array_equal(np.nonzero(prob["fix"] == 0)[0] + 1, rest[:, 0])
    g_g, neq = O.steering8(g_num, rest)
    assert neq == prob["neq"] and np.array_equal(g_g, prob["g_g"])


def test_p12meshgen_writes_p123_decks(tmp_path):
    job = str(tmp_path / "box")
    with open(job + ".mg", "w") as f:
        f.write("'p123'\n'parafem' 120  5  4  8\n.3  .4  .5  2.0  1.0  3.0\n1.e-6  500\n1  1\n")
    P.p12meshgen(job)
    dat = open(job + ".dat").read().split()
    nels, nn, nr, nip, nod, nl, nf = (int(t) for t in dat[3:10])
    kx, ky, kz, tol = (float(t) for t in dat[10:14])
    limit, nres = int(dat[14]), int(dat[15])
    nye = 120 // 5 // 4
    assert (nels, nn, nip, nod, nl, nf) == (120, 6 * (nye + 1) * 5, 8, 8, 1, 1)
    assert (kx, ky, kz, tol, limit) == (2.0, 1.0, 3.0, 1e-6, 500)
    assert nres == 5 * (4 - 1) + 1
    lines = open(job + ".d").read().splitlines()
    assert lines[:2] == ["*THREE_DIMENSIONAL", "*NODES"] and lines[2 + nn] == "*ELEMENTS"
    el = np.array([[int(t) for t in ln.split()] for ln in lines[3 + nn:3 + nn + nels]])
    g_abaqus = np.ascontiguousarray(el[:, 4:12], dtype=np.int32)
    O.lib().orc_abaqus2sg8(nels, g_abaqus)
    g_num, g_coord = O.box8_mesh(5, nye, 4, .3, .4, .5)
    assert np.array_equal(g_abaqus, g_num)
    coords = np.array([[float(t) for t in ln.split()[1:]] for ln in lines[2:2 + nn]])
    assert np.allclose(coords[g_num - 1].transpose(0, 2, 1), g_coord, atol=5e-7)
    bnd = np.loadtxt(job + ".bnd", dtype=np.int64, ndmin=2)
    assert bnd.shape[0] == nr and np.array_equal(bnd, O.box8_rest(5, nye, 4))
    lds = open(job + ".lds").read().split()
    assert int(lds[0]) == nres and float(lds[1]) == 10.0
    fix = open(job + ".fix").read().split()
    assert (int(fix[0]), int(fix[1]), float(fix[2])) == (nres, 1, 100.0)
