"""Host-side logic of libpfgpu.so (no GPU): exports, generators, numbering."""
import ctypes
import os
import re

import numpy as np
import pytest

import parafem_gb300 as P
from oracle import oracle as O

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def header_functions():
    txt = open(os.path.join(ROOT, "include", "pfgpu.h")).read()
    txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
    return re.findall(r"^\s*int\s+(\w+)\s*\(", txt, flags=re.M)


def test_library_exports_every_declared_symbol():
    names = header_functions()
    assert len(names) >= 25
    lib = ctypes.CDLL(P.library_path() if os.path.exists(P.library_path()) else P.lib()._name)
    for n in names:
        assert hasattr(lib, n), n
    assert set(names) == set(P.pfgpu.exported_symbols())


def test_integration_notes_cover_every_declared_symbol():
    """Every entry point of the C-ABI is described in the integration notes."""
    notes = open(os.path.join(ROOT, "INTEGRATION.md")).read()
    missing = [n for n in header_functions() if not re.search(r"\b%s\b" % n, notes)]
    assert not missing, missing


@pytest.mark.parametrize("nxe,nye,nze", [(1, 1, 1), (2, 3, 4), (5, 2, 3)])
def test_mesh_cube_matches_geometry_20bxz(nxe, nye, nze):
    aa, bb, cc = 0.5, 0.25, 0.75
    g_num, g_coord, nn = P.mesh_cube(nxe, nye, nze, aa, bb, cc)
    L = O.lib()
    coord = np.zeros(60)
    num = np.zeros(20, np.int32)
    for e in range(nxe * nye * nze):
        L.orc_geometry_20bxz(e + 1, nxe, nze, aa, bb, cc, coord, num)
        assert np.array_equal(num, g_num[e])
        assert np.array_equal(coord.reshape(3, 20), g_coord[e])
    assert nn == g_num.max()
    assert len(np.unique(g_num)) == nn


@pytest.mark.parametrize("nxe,nye,nze", [(1, 1, 1), (3, 2, 4), (5, 5, 5)])
def test_cube_bc20_matches(nxe, nye, nze):
    g_num, _, nn = P.mesh_cube(nxe, nye, nze)
    fix = P.cube_restraints(nxe, nye, nze, 0, nn)
    rest = np.zeros((nn, 4), np.int32)
    nr = O.lib().orc_cube_bc20(nxe, nye, nze, rest)
    rest = rest[:nr]
    ref = np.ones((nn, 3), np.int32)
    ref[rest[:, 0] - 1] = rest[:, 1:]
    assert np.array_equal(fix, ref)
    listed = np.nonzero((fix == 0).any(axis=1))[0] + 1
    assert np.array_equal(listed, rest[:, 0])


@pytest.mark.parametrize("bc", [0, 1])
def test_numbering_matches_rearrange_find_g3(bc):
    nxe, nye, nze = 4, 3, 5
    g_num, _, nn = P.mesh_cube(nxe, nye, nze)
    fix = P.cube_restraints(nxe, nye, nze, bc, nn)
    g_g, neq = P.number_equations(g_num, fix)
    rows = np.nonzero((fix == 0).any(axis=1))[0]
    rest = np.concatenate([(rows + 1)[:, None], fix[rows]], axis=1).astype(np.int32)
    if bc == 1:
        # node 1 precedes the first restrained node: list it free so that the
        # reference's find_g3 stays inside rest (new_library.f90:3130-3212)
        rest = np.concatenate([[[1, 1, 1, 1]], rest]).astype(np.int32)
    ref = O.steering(g_num, rest)
    assert np.array_equal(g_g, ref)
    assert neq == ref.max()


def test_demo_numbering(demo_problem):
    d = demo_problem["deck"]
    fix = np.ones((d.nn, 3), np.int32)
    fix[d.rest[:, 0] - 1] = (d.rest[:, 1:] != 0)
    g_g, neq = P.number_equations(d.g_num, fix)
    assert np.array_equal(g_g, demo_problem["g_g"])


def test_config1_sizes_and_total_load():
    prob = P.cube_problem(10, 10, 10)
    assert prob["nn"] == 4961 and prob["neq"] == 13860
    assert abs(prob["r"].sum() + 1.0) < 1e-14
    assert (prob["g_g"] >= 0).all()


def test_load_p121_pattern_is_patch_pressure(demo_deck):
    # load_p121 values are the consistent loads of a uniform pressure of 25 on
    # the nle x nle corner patch: total -25 * (nle*aa)^2 = -100 for the demo
    assert abs(demo_deck.load_val[:, 2].sum() + 100.0) < 1e-6


def test_random_material_deterministic_and_in_range():
    e1, v1 = P.random_material(10000, 1234, 1.0, 1000.0, 0.2, 0.35)
    e2, v2 = P.random_material(10000, 1234, 1.0, 1000.0, 0.2, 0.35)
    e3, _ = P.random_material(10000, 1235, 1.0, 1000.0, 0.2, 0.35)
    assert np.array_equal(e1, e2) and np.array_equal(v1, v2) and not np.array_equal(e1, e3)
    assert e1.min() >= 1.0 and e1.max() <= 1000.0 and v1.min() >= 0.2 and v1.max() <= 0.35
    # log-uniform: mean of ln(E) ~ ln(1000)/2
    assert abs(np.log(e1).mean() - np.log(1000.0) / 2) < 0.1


def test_errors_are_reported_not_printed(tmp_path):
    with pytest.raises(P.PfError, match="cannot read"):
        P.p12meshgen(str(tmp_path / "missing"))


@pytest.mark.parametrize("run", ["p121_run", "p122_run", "p123_run"])
def test_whole_jobs_report_a_missing_deck(tmp_path, run):
    """The deck is read before any GPU work, so this runs without a GPU."""
    with pytest.raises(P.PfError, match=r"cannot read .*missing\.dat"):
        getattr(P, run)(str(tmp_path / "missing"))


@pytest.mark.parametrize("ext,what", [("bnd", "restraints"), ("lds", "loads")])
def test_truncated_deck_is_reported(tmp_path, demo_job, ext, what):
    job = str(tmp_path / "cut")
    for e in ("dat", "d", "bnd", "lds"):
        with open(f"{demo_job}.{e}") as src, open(f"{job}.{e}", "w") as dst:
            lines = src.readlines()
            dst.writelines(lines[: len(lines) // 2] if e == ext else lines)
    with pytest.raises(P.PfError, match=rf"cannot read \d+ {what} from .*cut\.{ext}"):
        P.p121_run(job)


def test_numbering_without_restraints_is_the_identity():
    """No restrained node: the product numbers freedom d of node l as
    3 (l - 1) + d, as the oracle's find_g3 does for an empty list, and the
    8-node scalar numbering gives each node its own number."""
    g_num, _, nn = P.mesh_cube(2, 2, 2)
    g_g, neq = P.number_equations(g_num, np.ones((nn, 3), np.int32))
    assert neq == 3 * nn
    assert np.array_equal(g_g, O.steering(g_num, np.zeros((0, 4), np.int32)))
    g8, _ = O.box8_mesh(2, 2, 2, 1.0, 1.0, 1.0, coords=False)
    s8, neq8 = O.steering8(g8, np.zeros((0, 2), np.int32))
    assert neq8 == 27 and np.array_equal(s8, g8)


_RUN_LIMITED = r"""
import resource, sys
resource.setrlimit(resource.RLIMIT_AS, (8 << 30, 8 << 30))   # a runaway allocation fails, not the machine
sys.path.insert(0, sys.argv[1])
import parafem_gb300 as P
try:
    getattr(P, sys.argv[2])(sys.argv[3])
    print("NO ERROR")
except P.PfError as e:
    print("PfError:", e)
"""


def _run_limited(fn, job):
    import subprocess
    import sys
    r = subprocess.run([sys.executable, "-c", _RUN_LIMITED, ROOT, fn, job], capture_output=True, text=True,
                       timeout=120)
    assert r.returncode == 0, r.stderr[-2000:]   # no abort: every failure comes back as an error status
    return r.stdout


@pytest.mark.parametrize("token,value,match", [
    (4, "2000000000", "short node list"),   # nn far beyond the node lines of the .d file
    (3, "2000000000", "short element list"),
    (4, "-7", "elements and -7 nodes"),
    (3, "0", "0 elements and"),
])
def test_deck_counts_the_files_do_not_hold_are_reported(tmp_path, demo_job, token, value, match):
    """The .dat record's counts do not size any array before the lines are
    read, and a count the .d file does not hold is an error, not an
    allocation the size of the claim."""
    job = str(tmp_path / "claim")
    for e in ("d", "bnd", "lds"):
        with open(f"{demo_job}.{e}") as src, open(f"{job}.{e}", "w") as dst:
            dst.write(src.read())
    toks = open(f"{demo_job}.dat").read().split()
    toks[token] = value
    with open(f"{job}.dat", "w") as f:
        f.write(" ".join(toks) + "\n")
    out = _run_limited("p121_run", job)
    assert out.startswith("PfError:") and match in out, out


@pytest.mark.parametrize("case,body", [
    ("p121", "p121\nparafem\n-6 2 3 20 27 1.0 1.0 1.0 100.0 0.3 1e-6 5000\n"),
    ("p121", "p121\nparafem\n6 200000 300000 20 27 1.0 1.0 1.0 100.0 0.3 1e-6 5000\n"),
    ("p123", "p123\nparafem\n-6 2 3 8 1.0 1.0 1.0 1.0 1.0 1.0 1e-5 500 1 0\n"),
])
def test_mesh_generator_rejects_element_counts_it_cannot_form(tmp_path, case, body):
    job = str(tmp_path / case)
    with open(job + ".mg", "w") as f:
        f.write(body)
    out = _run_limited("p12meshgen", job)
    assert out.startswith("PfError:") and "supported" in out, out


def test_host_memory_exhaustion_is_an_error_status(tmp_path):
    """A valid request that the host cannot hold (a 1000^3 cube's deck, about
    100 GB of node and element arrays, under an 8 GB address-space limit)
    comes back as PF_FAILURE through the entry point's exception handler."""
    job = str(tmp_path / "huge")
    with open(job + ".mg", "w") as f:
        f.write("p121\nparafem\n1000000000 1000 1000 20 27 1.0 1.0 1.0 100.0 0.3 1e-6 5000\n")
    out = _run_limited("p12meshgen", job)
    assert out.startswith("PfError:") and "pf_p12meshgen: out of host memory" in out, out


_DEGENERATE = r"""
import ctypes, sys
sys.path.insert(0, sys.argv[1])
import numpy as np
import parafem_gb300 as P
L = P.lib()
i = lambda v: ctypes.byref(ctypes.c_int(v))
dd = lambda v: ctypes.byref(ctypes.c_double(v))
buf_i = np.ones(64, np.int32)
buf_d = np.zeros(64)
out = ctypes.c_int()
calls = {
    "mesh_cube nxe 0": lambda: L.pf_mesh_cube(i(0), i(1), i(1), dd(1), dd(1), dd(1), ctypes.byref(out),
                                              ctypes.byref(out), None, None),
    "cube_restraints nxe 0": lambda: L.pf_cube_restraints(i(0), i(1), i(1), i(0), buf_i.ctypes.data),
    "cube_restraints nze -2": lambda: L.pf_cube_restraints(i(1), i(1), i(-2), i(0), buf_i.ctypes.data),
    "number_equations nels -1": lambda: L.pf_number_equations(i(-1), i(1), buf_i.ctypes.data, buf_i.ctypes.data,
                                                              buf_i.ctypes.data, ctypes.byref(out)),
    "number_equations nn 0": lambda: L.pf_number_equations(i(1), i(0), buf_i.ctypes.data, buf_i.ctypes.data,
                                                           buf_i.ctypes.data, ctypes.byref(out)),
    "cube_top_pressure nxe 0": lambda: L.pf_cube_top_pressure(i(0), i(1), i(1), dd(1), dd(1), dd(1),
                                                              buf_i.ctypes.data, i(1), buf_d.ctypes.data),
    "random_material nels -1": lambda: L.pf_random_material(i(-1), ctypes.byref(ctypes.c_longlong(1)), dd(1),
                                                            dd(2), dd(0.2), dd(0.3), buf_d.ctypes.data,
                                                            buf_d.ctypes.data),
    "patch_loads nels -1": lambda: L.pf_patch_loads(i(5), i(1), dd(1), i(-1), buf_i.ctypes.data, buf_i.ctypes.data,
                                                    i(1), buf_d.ctypes.data),
    "number_equations1 nels -1": lambda: L.pf_number_equations1(i(-1), i(1), i(8), buf_i.ctypes.data,
                                                                buf_i.ctypes.data, buf_i.ctypes.data,
                                                                ctypes.byref(out)),
}
for name, call in calls.items():
    print(name, "=>", call(), P.pfgpu.last_error())
"""


def test_host_helpers_reject_degenerate_sizes():
    """Zero, negative or overflowing sizes come back as PF_FAILURE with a
    message: no division by zero, no loop over a wrapped count."""
    import subprocess
    import sys
    r = subprocess.run([sys.executable, "-c", _DEGENERATE, ROOT], capture_output=True, text=True, timeout=120)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = r.stdout.strip().splitlines()
    assert len(lines) == 9, r.stdout
    for ln in lines:
        name, rest = ln.split(" => ")
        status, msg = rest.split(" ", 1)
        assert status == "1" and msg.startswith("pf_"), ln
