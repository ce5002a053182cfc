"""Shared fixtures.  Tests marked ``gpu`` need a CUDA device; the rest run on CPU."""
import json
import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

GOLDEN_DIR = os.path.join(ROOT, "tests", "golden")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (run with -m gpu)")
    config.addinivalue_line("markers", "slow: takes more than a few seconds")


@pytest.fixture(scope="session")
def golden():
    with open(os.path.join(GOLDEN_DIR, "p121_golden.json")) as f:
        return json.load(f)


@pytest.fixture(scope="session")
def golden_displ():
    return np.load(os.path.join(GOLDEN_DIR, "p121_demo_displ.npz"))["disp"].astype(np.float64)


def _write_deck(tmpdir, name, mg_text):
    import parafem_gb300 as P
    job = os.path.join(str(tmpdir), name)
    with open(job + ".mg", "w") as f:
        f.write(mg_text)
    P.p12meshgen(job)
    return job


@pytest.fixture(scope="session")
def demo_job(tmp_path_factory, golden):
    """The p121 demo deck regenerated from its .mg by the library's p12meshgen."""
    return _write_deck(tmp_path_factory.mktemp("demo"), "p121_demo", golden["demo_mg"])


@pytest.fixture(scope="session")
def book_job(tmp_path_factory, golden):
    return _write_deck(tmp_path_factory.mktemp("book"), "p121", golden["book_mg"])


@pytest.fixture(scope="session")
def demo_deck(demo_job):
    from oracle import oracle as O
    return O.read_deck(demo_job)


@pytest.fixture(scope="session")
def demo_problem(demo_deck):
    """Oracle set-up of the demo: numbering, storkm, diag, loads."""
    from oracle import oracle as O
    d = demo_deck
    g_g = O.steering(d.g_num, d.rest)
    neq = int(g_g.max())
    gc = O.element_coords(d.coords, d.g_num)
    km = O.form_storkm(gc, d.nip, d.e, d.v)
    dg = O.diag(g_g, km, neq)
    r = O.load_vector(d.g_num, g_g, d.load_node, d.load_val, neq)
    return dict(deck=d, g_g=g_g, neq=neq, gc=gc, km=km, diag=dg, r=r)


def fortran_e(v, w=12, d=4):
    """Fortran Ew.d text of v (gfortran style, 0.dddE+xx)."""
    a = abs(v)
    if a == 0.0:
        digits, ex = "0" * d, 0
    else:
        s = "%.*e" % (d - 1, a)
        digits = s[0] + s[2:2 + d - 1]
        ex = int(s.split("e")[1]) + 1
    t = ("-" if np.signbit(v) else "") + "0." + digits + "E" + ("-" if ex < 0 else "+") + "%02d" % abs(ex)
    return t.rjust(w)
