"""CPU oracle for the p121, p122 and p123 EBE-PCG paths (TEST INFRASTRUCTURE ONLY).

Wraps ``p121_oracle.c`` (a plain-C restatement of ParaFEM's p121 solve),
``p122_oracle.c`` and ``p123_oracle.c`` (the same for p122 and p123) and
``p121_cpu.c`` (the timed CPU build of p121's PCG), and adds a numpy reader
for p121 decks.  Only the tests, the smoke check and the
CPU-baseline leg of ``bench.py`` import this module; the product library never
does.

Reference routines restated (paths inside the ParaFEM tree):
  src/programs/5th_ed/p121/p121.f90:27-141           driver
  src/modules/mpi/input.f90:3336 (READ_P121), :1037-1060 (READ_G_NUM_PP),
    :893-896 (READ_G_COORD_PP), :2622 (READ_REST), :2399 (READ_LOADS)
  src/modules/shared/new_library.f90 SAMPLE/SHAPE_DER/DEEMAT/BEEMAT/REARRANGE/
    find_g3/ABAQUS2SG, src/modules/mpi/maths.f90 DOT_PRODUCT_P/INVERT/
    DETERMINANT/checon_par, src/modules/mpi/loading.f90 LOAD/load_p121,
    src/modules/shared/geometry.f90 GEOMETRY_20BXZ/cube_bc20
"""
from __future__ import annotations

import ctypes
import os
import subprocess
import threading
from dataclasses import dataclass

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD_DIR = os.path.join(HERE, "_build")
LIB_PATH = os.path.join(BUILD_DIR, "liborc.so")
_lock = threading.Lock()
_lib = None

_I = ctypes.c_int
_D = ctypes.c_double
_PI = np.ctypeslib.ndpointer(dtype=np.int32, flags="C_CONTIGUOUS")
_PD = np.ctypeslib.ndpointer(dtype=np.float64, flags="C_CONTIGUOUS")


def build(force: bool = False) -> str:
    """Compile the C restatement into ``oracle/_build/liborc.so`` (gcc, OpenMP)."""
    srcs = [os.path.join(HERE, "p121_oracle.c"), os.path.join(HERE, "p123_oracle.c"),
            os.path.join(HERE, "p122_oracle.c")]
    os.makedirs(BUILD_DIR, exist_ok=True)
    if (not force and os.path.exists(LIB_PATH)
            and os.path.getmtime(LIB_PATH) >= max(os.path.getmtime(s) for s in srcs)):
        return LIB_PATH
    tmp = LIB_PATH + f".tmp{os.getpid()}"
    subprocess.check_call(["gcc", "-O2", "-fPIC", "-shared", "-fopenmp",
                           "-ffp-contract=off", "-o", tmp] + srcs + ["-lm"])
    os.replace(tmp, LIB_PATH)
    return LIB_PATH


CPU_LIB_PATH = os.path.join(BUILD_DIR, "libcpu121.so")
_cpu_lib = None


def build_cpu(force: bool = False) -> str:
    """Compile the timed CPU baseline (``p121_cpu.c`` with the routines of
    ``p121_oracle.c`` it calls) into ``oracle/_build/libcpu121.so``: -O3,
    OpenMP, floating-point contraction allowed.  The parity oracle keeps its
    own -O2 -ffp-contract=off build."""
    srcs = [os.path.join(HERE, "p121_cpu.c"), os.path.join(HERE, "p121_oracle.c")]
    os.makedirs(BUILD_DIR, exist_ok=True)
    if (not force and os.path.exists(CPU_LIB_PATH)
            and os.path.getmtime(CPU_LIB_PATH) >= max(os.path.getmtime(s) for s in srcs)):
        return CPU_LIB_PATH
    tmp = CPU_LIB_PATH + f".tmp{os.getpid()}"
    subprocess.check_call(["gcc", "-O3", "-fPIC", "-shared", "-fopenmp", "-ffp-contract=fast",
                           "-o", tmp] + srcs + ["-lm"])
    os.replace(tmp, CPU_LIB_PATH)
    return CPU_LIB_PATH


def cpu_lib():
    global _cpu_lib
    with _lock:
        if _cpu_lib is None:
            L = ctypes.CDLL(build_cpu())
            L.cpu121_create.argtypes = [_I, _I, _I, _I, _D, _D]
            L.cpu121_create.restype = ctypes.c_void_p
            L.cpu121_destroy.argtypes = [ctypes.c_void_p]
            L.cpu121_neq.argtypes = [ctypes.c_void_p]
            L.cpu121_neq.restype = _I
            L.cpu121_threads.argtypes = [ctypes.c_void_p]
            L.cpu121_threads.restype = _I
            L.cpu121_metric.argtypes = [ctypes.c_void_p]
            L.cpu121_metric.restype = _D
            L.cpu121_get_storkm.argtypes = [ctypes.c_void_p, _I, _I, _PD]
            L.cpu121_get_problem.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p]
            L.cpu121_init.argtypes = [ctypes.c_void_p]
            L.cpu121_iterate.argtypes = [ctypes.c_void_p, _I, _D, _I]
            L.cpu121_iterate.restype = _I
            L.cpu121_get_x.argtypes = [ctypes.c_void_p, _PD]
            _cpu_lib = L
    return _cpu_lib


class CpuP121:
    """The timed CPU baseline of p121's solve on the fixed-base, top-pressure
    cube (``p121_cpu.c``): every loop of the PCG iteration on all host threads."""

    def __init__(self, nxe, nye, nze, nip=27, e=100.0, v=0.3):
        self.L = cpu_lib()
        self.h = self.L.cpu121_create(nxe, nye, nze, nip, e, v)
        if not self.h:
            raise MemoryError(f"CPU baseline: cannot allocate the {nxe}x{nye}x{nze} cube")
        self.nels = nxe * nye * nze
        self.neq = self.L.cpu121_neq(self.h)
        self.threads = self.L.cpu121_threads(self.h)

    def problem(self):
        g_g = np.zeros((self.nels, 60), np.int32)
        r = np.zeros(self.neq)
        self.L.cpu121_get_problem(self.h, g_g.ctypes.data, r.ctypes.data)
        return g_g, r

    def storkm(self, e0, count):
        out = np.zeros((count, 60, 60))
        self.L.cpu121_get_storkm(self.h, e0, count, out)
        return out

    def init(self):
        self.L.cpu121_init(self.h)

    def iterate(self, k, tol=0.0, stop_mode=0):
        return self.L.cpu121_iterate(self.h, k, tol, stop_mode)

    def x(self):
        out = np.zeros(self.neq)
        self.L.cpu121_get_x(self.h, out)
        return out

    def metric(self):
        return self.L.cpu121_metric(self.h)

    def close(self):
        if self.h:
            self.L.cpu121_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def lib():
    global _lib
    with _lock:
        if _lib is None:
            L = ctypes.CDLL(build())
            L.orc_geometry_20bxz.argtypes = [_I, _I, _I, _D, _D, _D, _PD, _PI]
            L.orc_cube_bc20.argtypes = [_I, _I, _I, _PI]
            L.orc_cube_bc20.restype = _I
            L.orc_load_p121.argtypes = [_I, _I, _I, _PI, _PD]
            L.orc_load_p121.restype = _I
            L.orc_rearrange.argtypes = [_I, _PI]
            L.orc_find_g3.argtypes = [_PI, _PI, _I, _PI]
            L.orc_abaqus2sg.argtypes = [_I, _PI]
            L.orc_sample.argtypes = [_I, _PD, _PD, _I]
            L.orc_sample.restype = _I
            L.orc_shape_der20.argtypes = [_PD, _D, _D, _D]
            L.orc_deemat.argtypes = [_PD, _D, _D]
            L.orc_form_storkm.argtypes = [_I, _I, _I, _PD, _PD, _PD, _I, _PD]
            L.orc_diag.argtypes = [_I, _I, _PI, _PD, _PD]
            L.orc_load.argtypes = [_I, _I, _PI, _PI, _I, _PI, _PD, _PD]
            L.orc_pcg.argtypes = [_I, _I, _PI, _PD, _PD, _PD, _D, _I, _I, _PD,
                                  ctypes.POINTER(ctypes.c_double), ctypes.c_void_p]
            L.orc_pcg.restype = _I
            L.orc_ebe_matvec.argtypes = [_I, _I, _PI, _PD, _PD, _PD]
            L.orc_centroid_stress.argtypes = [_PD, _PD, _D, _D, _PD]
            L.orc_num_threads.restype = _I
            L.orc_set_num_threads.argtypes = [_I]
            # p123 (p123_oracle.c)
            L.orc_geometry_8bxz.argtypes = [_I, _I, _I, _D, _D, _D, _PD, _PI]
            L.orc_box_bc8.argtypes = [_I, _I, _I, _PI]
            L.orc_box_bc8.restype = _I
            L.orc_rearrange_2.argtypes = [_I, _PI]
            L.orc_find_g4.argtypes = [_PI, _I, _PI, _I, _PI]
            L.orc_abaqus2sg8.argtypes = [_I, _PI]
            L.orc_shape_der8.argtypes = [_PD, _D, _D, _D]
            L.orc_form_storkc.argtypes = [_I, _I, _PD, _D, _D, _D, _PD]
            L.orc_diag8.argtypes = [_I, _I, _PI, _PD, _I, _PD]
            L.orc_pcg123.argtypes = [_I, _I, _PI, _PD, _I, _PD, _PD, _I, _PI, _PD, _D, _I, _PD,
                                     ctypes.POINTER(ctypes.c_double)]
            L.orc_pcg123.restype = _I
            L.orc_ebe_matvec8.argtypes = [_I, _I, _PI, _PD, _I, _PD, _PD]
            L.orc_mesh_box8.argtypes = [_I, _I, _I, _D, _D, _D, _PI, ctypes.c_void_p]
            L.orc_steering8.argtypes = [_I, _PI, _I, _PI, _PI]
            # p122 (p122_oracle.c)
            L.orc_p122.argtypes = [_I, _I, _PI, _PD, _I, _D, _D, _D, _D, _D, _I, _PD, _I, _I, _D, _D, _PD, _PD,
                                   ctypes.c_void_p]
            L.orc_p122.restype = _I
            L.orc_p122n.argtypes = [_I, _I, _I, _PI, _PD, _I, _D, _D, _D, _D, _D, _I, _PD, _I, _I, _D, _D,
                                    ctypes.c_void_p, _I, ctypes.c_void_p, ctypes.c_void_p, _PD, ctypes.c_void_p]
            L.orc_p122n.restype = _I
            L.orc_invar.argtypes = [_PD, ctypes.POINTER(_D), ctypes.POINTER(_D), ctypes.POINTER(_D)]
            L.orc_mocouf.argtypes = [_D, _D, _D, _D, _D]
            L.orc_mocouf.restype = _D
            L.orc_mocouq.argtypes = [_D, _D, _D, ctypes.POINTER(_D), ctypes.POINTER(_D), ctypes.POINTER(_D)]
            L.orc_formm.argtypes = [_PD, _PD, _PD, _PD]
            L.orc_form_storkm8.argtypes = [_I, _I, _PD, _D, _D, _PD]
            _lib = L
    return _lib


# ---------------------------------------------------------------------------
# Deck reading (p121 text formats)
# ---------------------------------------------------------------------------
@dataclass
class Deck:
    element: str
    meshgen: int
    partitioner: int
    nels: int
    nn: int
    nr: int
    nip: int
    nod: int
    loaded_nodes: int
    e: float
    v: float
    tol: float
    limit: int
    coords: np.ndarray      # (nn, 3) float64, node id i at row i-1
    g_num: np.ndarray       # (nels, 20) int32, Smith-Griffiths order after abaqus2sg
    rest: np.ndarray        # (nr, 4) int32 as read (1 = free, 0 = fixed)
    load_node: np.ndarray   # (loaded_nodes,) int32
    load_val: np.ndarray    # (loaded_nodes, 3) float64


def _fortran_float(tok: str) -> float:
    return float(tok.replace("D", "E").replace("d", "e"))


def read_deck(job: str) -> Deck:
    """Read job.dat/.d/.bnd/.lds as READ_P121 and friends do."""
    with open(job + ".dat") as f:
        toks = f.read().split()
    element = toks[0].strip("'\"")
    meshgen, part, nels, nn, nr, nip, nod, ln = (int(t) for t in toks[1:9])
    e, v, tol = (_fortran_float(t) for t in toks[9:12])
    limit = int(toks[12])
    with open(job + ".d") as f:
        lines = f.read().splitlines()
    i0 = lines.index("*NODES") + 1
    i1 = lines.index("*ELEMENTS")
    coords = np.loadtxt(lines[i0:i1], dtype=np.float64)[:, 1:4]
    if coords.shape[0] != nn:
        raise ValueError(f"{job}.d has {coords.shape[0]} nodes, .dat says {nn}")
    el = np.loadtxt(lines[i1 + 1:i1 + 1 + nels], dtype=np.int64)
    g_num = np.ascontiguousarray(el[:, 4:4 + nod], dtype=np.int32)
    if meshgen == 2:
        lib().orc_abaqus2sg(nels, g_num)
    rest = np.loadtxt(job + ".bnd", dtype=np.int32, ndmin=2).reshape(-1, 4)[:nr]
    if ln > 0:
        lds = np.loadtxt(job + ".lds", dtype=np.float64, ndmin=2).reshape(-1, 4)[:ln]
        load_node = np.ascontiguousarray(lds[:, 0].astype(np.int32))
        load_val = np.ascontiguousarray(lds[:, 1:4])
    else:
        load_node = np.zeros(0, np.int32)
        load_val = np.zeros((0, 3))
    return Deck(element, meshgen, part, nels, nn, nr, nip, nod, ln, e, v, tol, limit,
                coords, g_num, np.ascontiguousarray(rest), load_node, load_val)


# ---------------------------------------------------------------------------
# Restated steps
# ---------------------------------------------------------------------------
def steering(g_num: np.ndarray, rest: np.ndarray) -> np.ndarray:
    """REARRANGE + find_g3 for every element -> g_g (nels, 60), 1-based, 0 = fixed."""
    L = lib()
    rr = np.ascontiguousarray(rest, dtype=np.int32).copy()
    L.orc_rearrange(rr.shape[0], rr)
    nels = g_num.shape[0]
    g_g = np.zeros((nels, 60), np.int32)
    row = np.zeros(60, np.int32)
    for e in range(nels):
        L.orc_find_g3(np.ascontiguousarray(g_num[e]), row, rr.shape[0], rr)
        g_g[e] = row
    return g_g


def element_coords(coords: np.ndarray, g_num: np.ndarray) -> np.ndarray:
    """g_coord_pp(nod,ndim,nels) as a C array (nels, 3, 20)."""
    return np.ascontiguousarray(coords[g_num - 1].transpose(0, 2, 1))


def form_storkm(g_coord: np.ndarray, nip: int, e, v, exact_weights: bool = False) -> np.ndarray:
    nels = g_coord.shape[0]
    e_arr = np.ascontiguousarray(np.atleast_1d(np.asarray(e, np.float64)))
    v_arr = np.ascontiguousarray(np.atleast_1d(np.asarray(v, np.float64)))
    per = int(e_arr.size > 1)
    km = np.zeros((nels, 60, 60), np.float64)   # km[e, j, i] = K_e(i, j)
    lib().orc_form_storkm(nels, nip, int(exact_weights), g_coord, e_arr, v_arr, per, km)
    return km


def diag(g_g: np.ndarray, storkm: np.ndarray, neq: int) -> np.ndarray:
    out = np.zeros(neq)
    lib().orc_diag(g_g.shape[0], neq, np.ascontiguousarray(g_g), storkm, out)
    return out


def load_vector(g_num, g_g, load_node, load_val, neq) -> np.ndarray:
    r = np.zeros(neq)
    lib().orc_load(g_num.shape[0], neq, np.ascontiguousarray(g_num), np.ascontiguousarray(g_g),
                   int(load_node.size), np.ascontiguousarray(load_node, dtype=np.int32),
                   np.ascontiguousarray(load_val, dtype=np.float64), r)
    return r


def pcg(g_g, storkm, dg, rhs, tol, limit, stop_mode=0, history=False):
    """p121 PCG.  stop_mode 0: checon_par; 1: relative residual.

    Returns (iterations, x, final stopping metric[, metric history])."""
    neq = rhs.size
    x = np.zeros(neq)
    m = ctypes.c_double(0.0)
    hist = np.zeros(max(int(limit), 1)) if history else None
    it = lib().orc_pcg(g_g.shape[0], neq, np.ascontiguousarray(g_g), storkm, dg,
                       np.ascontiguousarray(rhs, dtype=np.float64), float(tol), int(limit),
                       int(stop_mode), x, ctypes.byref(m),
                       hist.ctypes.data if history else None)
    if history:
        return it, x, m.value, hist[:it].copy()
    return it, x, m.value


def ebe_matvec(g_g, storkm, p):
    u = np.zeros(p.size)
    lib().orc_ebe_matvec(g_g.shape[0], p.size, np.ascontiguousarray(g_g), storkm,
                         np.ascontiguousarray(p, dtype=np.float64), u)
    return u


def centroid_stress(coord_e: np.ndarray, eld: np.ndarray, e: float, v: float) -> np.ndarray:
    s = np.zeros(6)
    lib().orc_centroid_stress(np.ascontiguousarray(coord_e.reshape(-1)),
                              np.ascontiguousarray(eld), float(e), float(v), s)
    return s


def nodal_displacements(g_num, g_g, x, nn) -> np.ndarray:
    """Node-wise displacement field (nn, 3); fixed dofs are zero."""
    disp = np.zeros((nn, 3))
    x0 = np.concatenate([[0.0], x])
    disp[g_num.reshape(-1) - 1] = x0[g_g.reshape(-1, 3)]
    return disp


@dataclass
class P121Result:
    nn: int
    nr: int
    neq: int
    total_load: float
    iters: int
    x: np.ndarray
    central: float
    stress: np.ndarray
    disp: np.ndarray
    storkm: np.ndarray
    g_g: np.ndarray


def run_p121(deck: Deck, exact_weights: bool = False, keep_storkm: bool = True) -> P121Result:
    """The whole p121 job of p121.f90:27-141 on one rank."""
    g_g = steering(deck.g_num, deck.rest)
    neq = int(g_g.max())
    gc = element_coords(deck.coords, deck.g_num)
    km = form_storkm(gc, deck.nip, deck.e, deck.v, exact_weights)
    dg = diag(g_g, km, neq)
    r = load_vector(deck.g_num, g_g, deck.load_node, deck.load_val, neq)
    q = _seq_sum(r)
    it, x, _ = pcg(g_g, km, dg, r, deck.tol, deck.limit, 0)
    x0 = np.concatenate([[0.0], x])
    eld = x0[g_g[0]]
    sig = centroid_stress(gc[0], eld, deck.e, deck.v)
    disp = nodal_displacements(deck.g_num, g_g, x, deck.nn)
    return P121Result(deck.nn, deck.nr, neq, q, it, x, float(x[0]), sig, disp,
                      km if keep_storkm else None, g_g)


def _seq_sum(a: np.ndarray) -> float:
    """SUM_P on one rank: a left-to-right sum (src/modules/mpi/maths.f90:271)."""
    s = 0.0
    for val in a.tolist():
        s += val
    return s


# ---------------------------------------------------------------------------
# p123: 3-D Laplace with 8-node bricks (src/programs/5th_ed/p123/p123.f90),
# restated in p123_oracle.c
# ---------------------------------------------------------------------------
def box8_mesh(nxe, nye, nze, aa, bb, cc, coords=True):
    """GEOMETRY_8BXZ over the box: g_num (nels, 8) and, if asked, g_coord (nels, 3, 8)."""
    nels = nxe * nye * nze
    g_num = np.zeros((nels, 8), np.int32)
    g_coord = np.zeros((nels, 3, 8)) if coords else None
    lib().orc_mesh_box8(nxe, nye, nze, aa, bb, cc, g_num, g_coord.ctypes.data if coords else None)
    return g_num, g_coord


def box8_rest(nxe, nye, nze):
    """box_bc8 rows (node, 0), sorted by node."""
    nn = (nxe + 1) * (nye + 1) * (nze + 1)
    rest = np.zeros(2 * nn, np.int32)
    nr = lib().orc_box_bc8(nxe, nye, nze, rest)
    return np.ascontiguousarray(rest[:2 * nr].reshape(nr, 2))


def steering8(g_num, rest):
    """rearrange_2 + find_g4 for every element -> g_g (nels, 8), and neq."""
    rr = np.ascontiguousarray(rest, dtype=np.int32).copy()
    lib().orc_rearrange_2(rr.shape[0], rr)
    g_g = np.zeros(g_num.shape, np.int32)
    lib().orc_steering8(g_num.shape[0], np.ascontiguousarray(g_num, dtype=np.int32), rr.shape[0], rr, g_g)
    return g_g, int(g_g.max())


def form_storkc(g_coord, nip, kx, ky, kz):
    g_coord = np.ascontiguousarray(g_coord, dtype=np.float64)
    nels = g_coord.shape[0]
    kc = np.zeros((nels, 8, 8))
    lib().orc_form_storkc(nels, nip, g_coord, kx, ky, kz, kc)
    return kc


def form_storkm8(g_coord, nip, e, v):
    """storkm of 8-node elasticity bricks (p122 with nod = 8): g_coord
    (nels, 3, 8) -> (nels, 24, 24) with km[e, j, i] = K_e(i, j)."""
    g_coord = np.ascontiguousarray(g_coord, dtype=np.float64)
    nels = g_coord.shape[0]
    km = np.zeros((nels, 24, 24))
    lib().orc_form_storkm8(nels, nip, g_coord, e, v, km)
    return km


def diag8(g_g, storkc, neq, shared=False):
    out = np.zeros(neq)
    lib().orc_diag8(g_g.shape[0], neq, np.ascontiguousarray(g_g, dtype=np.int32),
                    np.ascontiguousarray(storkc, dtype=np.float64), 0 if shared else 64, out)
    return out


def pcg123(g_g, storkc, dg, rhs, tol, limit, fix_eq=(), fix_store=(), shared=False):
    """p123's PCG with checon_par; dg already holds the penalties. Returns (iters, x, metric)."""
    neq = dg.shape[0]
    x = np.zeros(neq)
    metric = ctypes.c_double(0.0)
    fe = np.ascontiguousarray(np.asarray(fix_eq, dtype=np.int32))
    fs = np.ascontiguousarray(np.asarray(fix_store, dtype=np.float64))
    it = lib().orc_pcg123(g_g.shape[0], neq, np.ascontiguousarray(g_g, dtype=np.int32),
                          np.ascontiguousarray(storkc, dtype=np.float64), 0 if shared else 64,
                          np.ascontiguousarray(dg, dtype=np.float64), np.ascontiguousarray(rhs, dtype=np.float64),
                          fe.size, fe if fe.size else np.zeros(1, np.int32), fs if fs.size else np.zeros(1),
                          tol, limit, x, ctypes.byref(metric))
    return it, x, metric.value


def ebe_matvec8(g_g, storkc, p, shared=False):
    u = np.zeros_like(p)
    lib().orc_ebe_matvec8(g_g.shape[0], p.shape[0], np.ascontiguousarray(g_g, dtype=np.int32),
                          np.ascontiguousarray(storkc, dtype=np.float64), 0 if shared else 64,
                          np.ascontiguousarray(p, dtype=np.float64), u)
    return u


def run_p123_box(nxe, nye, nze, aa, bb, cc, kx, ky, kz, tol, limit, nip=8, load=10.0):
    """The p123 job on p12meshgen's box (p12meshgen.f90:658-801 + p123.f90),
    in memory: every element of the uniform box has element 1's storkc,
    which the solve shares.  Returns dict(nn, nr, neq, iters, q, nres, x)."""
    g_num, _ = box8_mesh(nxe, nye, nze, aa, bb, cc, coords=False)
    co = np.zeros(24)
    num = np.zeros(8, np.int32)
    lib().orc_geometry_8bxz(1, nxe, nze, aa, bb, cc, co, num)
    kc = form_storkc(co.reshape(1, 3, 8), nip, kx, ky, kz)
    rest = box8_rest(nxe, nye, nze)
    g_g, neq = steering8(g_num, rest)
    del g_num
    dg = diag8(g_g, kc, neq, shared=True)
    nres = nxe * (nze - 1) + 1
    r = np.zeros(neq)
    r[nres - 1] = load                       # loaded freedom used as an equation (p123.f90:98-103)
    it, x, _ = pcg123(g_g, kc, dg, r, tol, limit, shared=True)
    return dict(nn=(nxe + 1) * (nye + 1) * (nze + 1), nr=rest.shape[0], neq=neq, iters=it, q=float(r.sum()),
                nres=nres, x=x)


# ---------------------------------------------------------------------------
# p122: elastic-plastic (Mohr-Coulomb) solid, viscoplastic strain method,
# 20-node bricks (src/programs/5th_ed/p122/p122.f90), restated in p122_oracle.c
# ---------------------------------------------------------------------------
def cube20_problem(nels, nxe, nze, aa, bb, cc, load_factor):
    """p12meshgen's p121/p122 box of 20-node bricks (GEOMETRY_20BXZ,
    cube_bc20, load_p121 with val = val * load_factor): returns
    dict(g_num, g_coord, g_g, neq, nn, nr, ld0)."""
    L = lib()
    nye = nels // nxe // nze
    g_num = np.zeros((nels, 20), np.int32)
    g_coord = np.zeros((nels, 3, 20))
    co = np.zeros(60)
    num = np.zeros(20, np.int32)
    for iel in range(1, nels + 1):
        L.orc_geometry_20bxz(iel, nxe, nze, aa, bb, cc, co, num)
        g_num[iel - 1] = num
        g_coord[iel - 1] = co.reshape(3, 20)
    nn = int(g_num.max())
    rest = np.zeros(4 * nn, np.int32)
    nr = L.orc_cube_bc20(nxe, nye, nze, rest)
    rest = np.ascontiguousarray(rest[:4 * nr].reshape(nr, 4))
    g_g = steering(g_num, rest)
    neq = int(g_g.max())
    nle = nxe // 5
    node = np.zeros(4 * (nle + 1) ** 2 + 8, np.int32)
    val = np.zeros(node.size)
    nl = L.orc_load_p121(nle, nxe, nze, node, val)
    lv = np.zeros((nl, 3))
    lv[:, 2] = val[:nl] * load_factor
    ld0 = load_vector(g_num, g_g, np.ascontiguousarray(node[:nl]), lv, neq)
    return dict(g_num=g_num, g_coord=g_coord, g_g=g_g, neq=neq, nn=nn, nr=nr, ld0=ld0)


def run_p122(prob, nip, phi, c, psi, e, v, qinc, plasits, cjits, plastol, cjtol, keep_totd=False):
    """The p122 solve: per increment (totd(1), sigma z, sigma x, sigma y of
    element 1 Gauss point 1, cj iterations, plastic iterations)."""
    qinc = np.ascontiguousarray(qinc, dtype=np.float64)
    incs = qinc.size
    out = np.zeros((incs, 6))
    totd = np.zeros((incs, prob["neq"])) if keep_totd else None
    n = lib().orc_p122(prob["g_num"].shape[0], prob["neq"], np.ascontiguousarray(prob["g_g"]),
                       np.ascontiguousarray(prob["g_coord"]), nip, phi, c, psi, e, v, incs, qinc, plasits, cjits,
                       plastol, cjtol, np.ascontiguousarray(prob["ld0"]), out,
                       totd.ctypes.data if keep_totd else None)
    return out[:n], (totd[:n] if keep_totd else None)


def steering_n(g_num, rest):
    """find_g (src/modules/shared/new_library.f90:3218-3243), which p122 calls
    after REARRANGE, for bricks of any node count -> g_g (nels, 3 nod),
    1-based, 0 = restrained.  For freedom k of node l it counts the
    restrained freedoms of the listed nodes below l and of node l before k:
    g = 3 l - count - (3 - k), the freedoms numbered in node order.
    (REARRANGE leaves a restrained flag 0 and makes free ones nonzero, and
    find_g tests only for 0, so the original flags serve.)"""
    nels, nod = g_num.shape
    nn = int(max(g_num.max(), np.asarray(rest)[:, 0].max()))
    free = np.ones((nn, 3), bool)
    rest = np.asarray(rest)
    free[rest[:, 0] - 1] = rest[:, 1:4] != 0
    eq = np.zeros((nn, 3), np.int64)
    eq[free] = np.arange(1, int(free.sum()) + 1)
    return np.ascontiguousarray(eq[g_num - 1].reshape(nels, 3 * nod).astype(np.int32))


def fixed_equations(g_num, g_g, node, sense):
    """find_no: the equation of freedom `sense` (1..3) of each node."""
    eq = np.zeros(len(node), np.int32)
    nod = g_num.shape[1]
    for i, (nd, sn) in enumerate(zip(node, sense)):
        e, a = np.argwhere(g_num == nd)[0]
        eq[i] = g_g[e, 3 * a + sn - 1]
    assert np.all(eq > 0), "a fixed freedom is restrained"
    return eq


def p122_demo_problem(golden_dir):
    """The p122 demo deck (8-node bricks, 19 fixed freedoms) from its fixtures:
    dict(g_num, g_coord, g_g, neq, nn, nr, fix_eq, fix_val, mat, qinc, gold,
    displ)."""
    import json
    import os
    with open(os.path.join(golden_dir, "p122_golden.json")) as f:
        g = json.load(f)
    z = np.load(os.path.join(golden_dir, "p122_demo.npz"))
    tok = g["demo_dat"].replace("'", " ").split()
    incs = int(tok[15])
    mat = dict(nip=int(tok[6]), nod=int(tok[7]), phi=float(tok[10]), c=float(tok[11]), psi=float(tok[12]),
               e=float(tok[13]), v=float(tok[14]), plasits=int(tok[16]), cjits=int(tok[17]),
               plastol=float(tok[18]), cjtol=float(tok[19]))
    g_num = np.ascontiguousarray(z["g_num"])
    g_g = steering_n(g_num, z["rest"])
    g_coord = np.ascontiguousarray(z["coords"][g_num - 1].transpose(0, 2, 1))
    fix_eq = fixed_equations(g_num, g_g, z["fix_node"], z["fix_sense"])
    return dict(g_num=g_num, g_coord=g_coord, g_g=g_g, neq=int(g_g.max()), nn=z["coords"].shape[0],
                nr=z["rest"].shape[0], coords=z["coords"], rest=z["rest"], matid=z["matid"],
                fix_node=z["fix_node"], fix_sense=z["fix_sense"], fix_eq=fix_eq,
                fix_val=np.ascontiguousarray(z["fix_val"], dtype=np.float64), mat=mat,
                qinc=[float(t) for t in tok[20:20 + incs]], gold=g["demo"], displ=z["displ"], dat=g["demo_dat"])


def run_p122n(prob, nip, phi, c, psi, e, v, qinc, plasits, cjits, plastol, cjtol, ld0=None, fix_eq=(),
              fix_val=(), keep_totd=False):
    """The p122 solve for bricks of prob["g_num"].shape[1] nodes, with fixed
    freedoms (1-based equations fix_eq, values fix_val) and optional nodal
    loads ld0: per increment (totd(1), sigma z, sigma x, sigma y of element 1
    Gauss point 1, cj iterations, plastic iterations)."""
    qinc = np.ascontiguousarray(qinc, dtype=np.float64)
    incs = qinc.size
    out = np.zeros((incs, 6))
    totd = np.zeros((incs, prob["neq"])) if keep_totd else None
    fe = np.ascontiguousarray(fix_eq, dtype=np.int32)
    fv = np.ascontiguousarray(fix_val, dtype=np.float64)
    ld = np.ascontiguousarray(ld0, dtype=np.float64) if ld0 is not None else None
    n = lib().orc_p122n(prob["g_num"].shape[1], prob["g_num"].shape[0], prob["neq"],
                        np.ascontiguousarray(prob["g_g"]), np.ascontiguousarray(prob["g_coord"]), nip, phi, c, psi,
                        e, v, incs, qinc, plasits, cjits, plastol, cjtol, ld.ctypes.data if ld is not None else None,
                        int(fe.size), fe.ctypes.data if fe.size else None, fv.ctypes.data if fv.size else None, out,
                        totd.ctypes.data if keep_totd else None)
    return out[:n], (totd[:n] if keep_totd else None)
