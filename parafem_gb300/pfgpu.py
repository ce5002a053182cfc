"""ctypes binding of libpfgpu.so, the GB300 element-by-element PCG library.

The host arrays follow p121's Fortran layouts, expressed as C-contiguous
numpy arrays with the Fortran leading index last:
    g_num   (nels, 20)      int32   == g_num_pp(20, nels)
    g_g     (nels, 60)      int32   == g_g_pp(60, nels)
    g_coord (nels, 3, 20)   float64 == g_coord_pp(20, 3, nels)
    storkm  (nels, 60, 60)  float64 == storkm_pp(60, 60, nels): km[e, j, i] = K_e(i, j)

There is no CPU fallback: every call below runs in the compiled library and
raises PfError when the library reports a failure.
"""
from __future__ import annotations

import ctypes
import os

import numpy as np

from . import _build

MODE_P121 = 0
MODE_FP64_RES = 1
MODE_MIXED = 2
MODE_MIXED_RESTART = 3
MODE_MIXED16 = 4
FORM_EXACT_WEIGHTS = 1

_I = ctypes.c_int
_IP = ctypes.POINTER(ctypes.c_int)
_DP = ctypes.POINTER(ctypes.c_double)
_VPP = ctypes.POINTER(ctypes.c_void_p)
_LLP = ctypes.POINTER(ctypes.c_longlong)

_lib = None

# (name, argtypes) for every entry point of include/pfgpu.h
_SIGS = {
    "set_gpu": [_IP],
    "allocate_memory_on_gpu": [_IP, _IP, _VPP],
    "free_memory_on_gpu": [_VPP],
    "copy_data_to_gpu": [_IP, _IP, ctypes.c_void_p, _VPP],
    "copy_data_from_gpu": [_IP, _IP, ctypes.c_void_p, _VPP],
    "matrix_vector_multiplies": [_IP, _IP, _IP, _VPP, _VPP, _VPP],
    "pf_last_error": [ctypes.c_char_p, _IP],
    "pf_ctx_create": [_IP, _VPP],
    "pf_ctx_destroy": [_VPP],
    "pf_setup": [_VPP, _IP, _IP, _IP, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p],
    "pf_set_material": [_VPP, _IP, ctypes.c_void_p, ctypes.c_void_p],
    "pf_form_storkm": [_VPP, _IP, _IP],
    "pf_set_storkm": [_VPP, ctypes.c_void_p],
    "pf_set_shared_km": [_VPP, ctypes.c_void_p],
    "pf_form_km": [_VPP, _IP, _IP, _IP, ctypes.c_void_p],
    "pf_get_storkm": [_VPP, _IP, _IP, ctypes.c_void_p],
    "pf_get_diag": [_VPP, ctypes.c_void_p],
    "pf_ebe_matvec": [_VPP, _IP, ctypes.c_void_p, ctypes.c_void_p],
    "pf_solve": [_VPP, ctypes.c_void_p, _DP, _IP, _IP, ctypes.c_void_p, _IP, _DP],
    "pf_solve_stats": [_VPP, ctypes.c_void_p, _IP],
    "pf_bench_iterations": [_VPP, _IP, _IP, _DP, _DP, _DP],
    "pf_centroid_stress": [_VPP, _IP, ctypes.c_void_p, ctypes.c_void_p],
    "pf_element_stresses": [_VPP, ctypes.c_void_p, _IP, _IP, ctypes.c_void_p],
    "pf_kernel_launches": [_VPP, _LLP],
    "pf_tuning": [_VPP, _IP, _IP, ctypes.c_void_p],
    "pf_tuning16": [_VPP, _IP, _IP, ctypes.c_void_p],
    "pf_set_tuning": [_VPP, _IP],
    "pf_set_graphs": [_VPP, _IP],
    "pf_set_persistent": [_VPP, _IP],
    "pf_check_wait_timeout": [_VPP, _IP],
    "pf_ebe_matvec_noalloc": [_IP, _IP, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p,
                              ctypes.c_void_p],
    "pf_solve_multi": [_VPP, _IP, ctypes.c_void_p, _DP, _IP, _IP, ctypes.c_void_p, ctypes.c_void_p,
                       ctypes.c_void_p],
    "pf_ebe_matvec_multi": [_VPP, _IP, _IP, ctypes.c_void_p, ctypes.c_void_p],
    "pf_multi_free": [_VPP],
    "pf_multi_tuning": [_VPP, _IP, ctypes.c_void_p, ctypes.c_void_p],
    "pf_multi_product_ms": [_VPP, _IP, ctypes.c_void_p, _IP, ctypes.c_void_p],
    "pf_batch_create": [_IP, _LLP, _IP, _IP, _VPP],
    "pf_batch_destroy": [_VPP],
    "pf_batch_capacity": [_VPP, _LLP, _LLP],
    "pf_batch_admit": [_VPP, _IP, _IP, _IP, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, _IP,
                       ctypes.c_void_p, ctypes.c_void_p, _IP, ctypes.c_void_p, _DP, _IP, _IP],
    "pf_batch_launch": [_VPP, _IP],
    "pf_batch_sync": [_VPP, _IP, _IP],
    "pf_batch_collect": [_VPP, _IP, _IP, _DP, ctypes.c_void_p, _IP, _IP],
    "pf_batch_launches": [_VPP, _LLP],
    "pf_batch_set_graphs": [_VPP, _IP],
    "pf_p12meshgen": [ctypes.c_char_p],
    "pf_p121_run": [ctypes.c_char_p, _IP, _IP, _IP, _DP],
    "pf_p123_run": [ctypes.c_char_p, _IP, _IP, ctypes.c_void_p],
    "pf_p122_run": [ctypes.c_char_p, _IP, _IP],
    "pf_mesh_box8": [_IP, _IP, _IP, _DP, _DP, _DP, ctypes.c_void_p, ctypes.c_void_p],
    "pf_box8_restraints": [_IP, _IP, _IP, ctypes.c_void_p],
    "pf_number_equations1": [_IP, _IP, _IP, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, _IP],
    "pf_setup_scalar8": [_VPP, _IP, _IP, _IP, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p],
    "pf_form_storkc": [_VPP, _IP, _DP, _DP, _DP],
    "pf_get_storkc": [_VPP, _IP, _IP, ctypes.c_void_p],
    "pf_set_fixed": [_VPP, _IP, ctypes.c_void_p, _DP],
    "pf_p122_solve": [_VPP, _IP, _DP, _DP, _DP, _IP, ctypes.c_void_p, _IP, _IP, _DP, _DP, ctypes.c_void_p,
                      ctypes.c_void_p, ctypes.c_void_p, _IP],
    "pf_setup_solid8": [_VPP, _IP, _IP, _IP, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p],
    "pf_p122_solve_fixed": [_VPP, _IP, _DP, _DP, _DP, _IP, ctypes.c_void_p, _IP, _IP, _DP, _DP, ctypes.c_void_p,
                            _IP, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, _IP],
    "pf_mesh_cube": [_IP, _IP, _IP, _DP, _DP, _DP, _IP, _IP, ctypes.c_void_p, ctypes.c_void_p],
    "pf_cube_restraints": [_IP, _IP, _IP, _IP, ctypes.c_void_p],
    "pf_number_equations": [_IP, _IP, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, _IP],
    "pf_cube_top_pressure": [_IP, _IP, _IP, _DP, _DP, _DP, ctypes.c_void_p, _IP, ctypes.c_void_p],
    "pf_patch_loads": [_IP, _IP, _DP, _IP, ctypes.c_void_p, ctypes.c_void_p, _IP, ctypes.c_void_p],
    "pf_random_material": [_IP, _LLP, _DP, _DP, _DP, _DP, ctypes.c_void_p, ctypes.c_void_p],
}


class PfError(RuntimeError):
    pass


def library_path() -> str:
    return _build.LIB


def lib():
    """Load libpfgpu.so, building it first when a source is newer."""
    global _lib
    if _lib is None:
        path = _build.build()
        L = ctypes.CDLL(path)
        for name, args in _SIGS.items():
            fn = getattr(L, name)
            fn.argtypes = args
            fn.restype = ctypes.c_int
        _lib = L
    return _lib


def exported_symbols():
    return list(_SIGS)


def _i(v):
    return ctypes.byref(ctypes.c_int(int(v)))


def _d(v):
    return ctypes.byref(ctypes.c_double(float(v)))


def last_error() -> str:
    buf = ctypes.create_string_buffer(1024)
    lib().pf_last_error(buf, _i(1024))
    return buf.value.decode(errors="replace")


def _check(rc, what):
    if rc != 0:
        raise PfError(f"{what}: {last_error()}")


def _arr(a, dtype):
    a = np.ascontiguousarray(a, dtype=dtype)
    return a, a.ctypes.data


# ---------------------------------------------------------------------------
# host-side helpers (no GPU)
def mesh_cube(nxe, nye, nze, aa=1.0, bb=1.0, cc=1.0):
    """GEOMETRY_20BXZ cube: returns (g_num (nels,20), g_coord (nels,3,20), nn)."""
    L = lib()
    nels, nn = ctypes.c_int(0), ctypes.c_int(0)
    args = [_i(nxe), _i(nye), _i(nze), _d(aa), _d(bb), _d(cc)]
    _check(L.pf_mesh_cube(*args, ctypes.byref(nels), ctypes.byref(nn), None, None), "pf_mesh_cube")
    g_num = np.zeros((nels.value, 20), np.int32)
    g_coord = np.zeros((nels.value, 3, 20), np.float64)
    _check(L.pf_mesh_cube(*args, ctypes.byref(nels), ctypes.byref(nn), g_num.ctypes.data,
                          g_coord.ctypes.data), "pf_mesh_cube")
    return g_num, g_coord, nn.value


def cube_restraints(nxe, nye, nze, bc, nn):
    fix = np.zeros((nn, 3), np.int32)
    _check(lib().pf_cube_restraints(_i(nxe), _i(nye), _i(nze), _i(bc), fix.ctypes.data),
           "pf_cube_restraints")
    return fix


def number_equations(g_num, node_fix):
    g_num, pn = _arr(g_num, np.int32)
    node_fix, pf = _arr(node_fix, np.int32)
    g_g = np.zeros((g_num.shape[0], 60), np.int32)
    neq = ctypes.c_int(0)
    _check(lib().pf_number_equations(_i(g_num.shape[0]), _i(node_fix.shape[0]), pn, pf, g_g.ctypes.data,
                                     ctypes.byref(neq)), "pf_number_equations")
    return g_g, neq.value


def cube_top_pressure(nxe, nze, g_g, neq, p, aa=1.0, bb=1.0, r=None):
    g_g, pg = _arr(g_g, np.int32)
    if r is None:
        r = np.zeros(neq)
    _check(lib().pf_cube_top_pressure(_i(nxe), _i(nze), _i(g_g.shape[0]), _d(aa), _d(bb), _d(p), pg,
                                      _i(neq), r.ctypes.data), "pf_cube_top_pressure")
    return r


def patch_loads(nxe, nze, g_num, g_g, neq, factor):
    """load_p121's top-face patch as a load vector (see pf_patch_loads)."""
    g_num, pn = _arr(g_num, np.int32)
    g_g, pg = _arr(g_g, np.int32)
    r = np.zeros(neq)
    _check(lib().pf_patch_loads(_i(nxe), _i(nze), _d(factor), _i(g_num.shape[0]), pn, pg, _i(neq), r.ctypes.data),
           "pf_patch_loads")
    return r


def random_material(nels, seed, e_lo, e_hi, v_lo, v_hi):
    e = np.zeros(nels)
    v = np.zeros(nels)
    _check(lib().pf_random_material(_i(nels), ctypes.byref(ctypes.c_longlong(int(seed))), _d(e_lo), _d(e_hi),
                                    _d(v_lo), _d(v_hi), e.ctypes.data, v.ctypes.data), "pf_random_material")
    return e, v


def p12meshgen(job: str):
    _check(lib().pf_p12meshgen(os.fsencode(job)), "pf_p12meshgen")


def p121_run(job: str, mode: int = MODE_P121, device: int = 0):
    it, cen = ctypes.c_int(0), ctypes.c_double(0.0)
    _check(lib().pf_p121_run(os.fsencode(job), _i(device), _i(mode), ctypes.byref(it), ctypes.byref(cen)),
           "pf_p121_run")
    return it.value, cen.value


# ---------------------------------------------------------------------------
class Solver:
    """One solver context on one GPU (pf_ctx_create .. pf_ctx_destroy)."""

    def __init__(self, device: int = 0):
        self._h = ctypes.c_void_p(None)
        _check(lib().pf_ctx_create(_i(device), ctypes.byref(self._h)), "pf_ctx_create")
        self.nels = self.nn = self.neq = 0

    @property
    def _ref(self):
        if not self._h.value:
            raise PfError("solver context is closed")
        return ctypes.byref(self._h)

    def close(self):
        if self._h.value:
            lib().pf_ctx_destroy(ctypes.byref(self._h))

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def setup(self, g_num, g_g, g_coord, nn, neq):
        g_num, pn = _arr(g_num, np.int32)
        g_g, pg = _arr(g_g, np.int32)
        g_coord, pc = _arr(g_coord, np.float64)
        nels = g_num.shape[0]
        if g_g.shape != (nels, 60) or g_coord.shape != (nels, 3, 20):
            raise ValueError("g_num (nels,20), g_g (nels,60), g_coord (nels,3,20) expected")
        _check(lib().pf_setup(self._ref, _i(nels), _i(nn), _i(neq), pn, pg, pc), "pf_setup")
        self.nels, self.nn, self.neq = nels, int(nn), int(neq)

    def setup_scalar8(self, g_num, g_g, g_coord, nn, neq):
        """8-node bricks with one freedom per node (p123)."""
        g_num, pn = _arr(g_num, np.int32)
        g_g, pg = _arr(g_g, np.int32)
        g_coord, pc = _arr(g_coord, np.float64)
        nels = g_num.shape[0]
        if g_num.shape != (nels, 8) or g_g.shape != (nels, 8) or g_coord.shape != (nels, 3, 8):
            raise ValueError("g_num (nels,8), g_g (nels,8), g_coord (nels,3,8) expected")
        _check(lib().pf_setup_scalar8(self._ref, _i(nels), _i(nn), _i(neq), pn, pg, pc), "pf_setup_scalar8")
        self.nels, self.nn, self.neq = nels, int(nn), int(neq)

    def setup_solid8(self, g_num, g_g, g_coord, nn, neq):
        """8-node elasticity bricks, three freedoms per node (p122's demo deck)."""
        g_num, pn = _arr(g_num, np.int32)
        g_g, pg = _arr(g_g, np.int32)
        g_coord, pc = _arr(g_coord, np.float64)
        nels = g_num.shape[0]
        if g_num.shape != (nels, 8) or g_g.shape != (nels, 24) or g_coord.shape != (nels, 3, 8):
            raise ValueError("g_num (nels,8), g_g (nels,24), g_coord (nels,3,8) expected")
        _check(lib().pf_setup_solid8(self._ref, _i(nels), _i(nn), _i(neq), pn, pg, pc), "pf_setup_solid8")
        self.nels, self.nn, self.neq = nels, int(nn), int(neq)

    def form_storkc(self, nip, kx, ky, kz):
        _check(lib().pf_form_storkc(self._ref, _i(nip), _d(kx), _d(ky), _d(kz)), "pf_form_storkc")

    def get_storkc(self, first=0, count=None):
        count = self.nels - first if count is None else count
        out = np.zeros((max(count, 1), 8, 8))
        _check(lib().pf_get_storkc(self._ref, _i(first), _i(count), out.ctypes.data), "pf_get_storkc")
        return out[:count]

    def set_fixed(self, eqs, penalty=1.0e20):
        eqs, pe = _arr(np.atleast_1d(eqs), np.int32)
        _check(lib().pf_set_fixed(self._ref, _i(eqs.size), pe, _d(penalty)), "pf_set_fixed")

    def p122_solve(self, nip, phi, c, psi, qinc, plasits, cjits, plastol, cjtol, ld0, keep_totd=False):
        """p122's load increments (see pf_p122_solve): results (incs_done, 6), totd (incs_done, neq) or None."""
        qinc = np.ascontiguousarray(np.atleast_1d(qinc), dtype=np.float64)
        ld0 = np.ascontiguousarray(ld0, dtype=np.float64)
        res = np.zeros((qinc.size, 6))
        totd = np.zeros((qinc.size, self.neq)) if keep_totd else None
        done = ctypes.c_int(0)
        _check(lib().pf_p122_solve(self._ref, _i(nip), _d(phi), _d(c), _d(psi), _i(qinc.size), qinc.ctypes.data,
                                   _i(plasits), _i(cjits), _d(plastol), _d(cjtol), ld0.ctypes.data, res.ctypes.data,
                                   totd.ctypes.data if keep_totd else None, ctypes.byref(done)), "pf_p122_solve")
        n = done.value
        return res[:n], (totd[:n] if keep_totd else None)

    def p122_solve_fixed(self, nip, phi, c, psi, qinc, plasits, cjits, plastol, cjtol, fix_eqs=(), fix_vals=(),
                         ld0=None, keep_totd=False):
        """p122's load increments with fixed freedoms (see pf_p122_solve_fixed):
        results (incs_done, 6), totd (incs_done, neq) or None."""
        qinc = np.ascontiguousarray(np.atleast_1d(qinc), dtype=np.float64)
        fe = np.ascontiguousarray(np.atleast_1d(fix_eqs), dtype=np.int32)
        fv = np.ascontiguousarray(np.atleast_1d(fix_vals), dtype=np.float64)
        if fe.size != fv.size:
            raise ValueError("fix_eqs and fix_vals differ in length")
        ld = None if ld0 is None else np.ascontiguousarray(ld0, dtype=np.float64)
        res = np.zeros((qinc.size, 6))
        totd = np.zeros((qinc.size, self.neq)) if keep_totd else None
        done = ctypes.c_int(0)
        _check(lib().pf_p122_solve_fixed(self._ref, _i(nip), _d(phi), _d(c), _d(psi), _i(qinc.size),
                                         qinc.ctypes.data, _i(plasits), _i(cjits), _d(plastol), _d(cjtol),
                                         ld.ctypes.data if ld is not None else None, _i(fe.size),
                                         fe.ctypes.data if fe.size else None, fv.ctypes.data if fv.size else None,
                                         res.ctypes.data, totd.ctypes.data if keep_totd else None,
                                         ctypes.byref(done)), "pf_p122_solve_fixed")
        n = done.value
        return res[:n], (totd[:n] if keep_totd else None)

    def set_material(self, e, v):
        e, pe = _arr(np.atleast_1d(e), np.float64)
        v, pv = _arr(np.atleast_1d(v), np.float64)
        _check(lib().pf_set_material(self._ref, _i(e.size), pe, pv), "pf_set_material")

    def form_storkm(self, nip: int, exact_weights: bool = False):
        _check(lib().pf_form_storkm(self._ref, _i(nip), _i(FORM_EXACT_WEIGHTS if exact_weights else 0)),
               "pf_form_storkm")

    def set_storkm(self, km):
        km, pk = _arr(km, np.float64)
        _check(lib().pf_set_storkm(self._ref, pk), "pf_set_storkm")

    def form_km(self, iel=1, nip=27, exact_weights=False):
        """The (60, 60) stiffness matrix of element iel (1-based), formed on the GPU."""
        km = np.zeros((60, 60))
        _check(lib().pf_form_km(self._ref, _i(iel), _i(nip), _i(FORM_EXACT_WEIGHTS if exact_weights else 0),
                                km.ctypes.data), "pf_form_km")
        return km

    def set_shared_km(self, km):
        """One element matrix (60, 60) for every element (PCG_KM); see pf_set_shared_km."""
        km = np.asarray(km, np.float64)
        if km.shape != (60, 60):
            raise ValueError("km must be 60 x 60")
        km, pk = _arr(km, np.float64)
        _check(lib().pf_set_shared_km(self._ref, pk), "pf_set_shared_km")

    def get_storkm(self, first=0, count=None):
        count = self.nels - first if count is None else count
        out = np.zeros((count, 60, 60))
        _check(lib().pf_get_storkm(self._ref, _i(first), _i(count), out.ctypes.data), "pf_get_storkm")
        return out

    def get_diag(self):
        out = np.zeros(self.neq)
        _check(lib().pf_get_diag(self._ref, out.ctypes.data), "pf_get_diag")
        return out

    def ebe_matvec(self, p, prec: int = 64):
        p, pp = _arr(p, np.float64)
        u = np.zeros(self.neq)
        _check(lib().pf_ebe_matvec(self._ref, _i(prec), pp, u.ctypes.data), "pf_ebe_matvec")
        return u

    def solve(self, r, tol, limit, mode=MODE_P121):
        r, pr = _arr(r, np.float64)
        x = np.zeros(self.neq)
        it = ctypes.c_int(0)
        rel = ctypes.c_double(0.0)
        _check(lib().pf_solve(self._ref, pr, _d(tol), _i(limit), _i(mode), x.ctypes.data, ctypes.byref(it),
                              ctypes.byref(rel)), "pf_solve")
        return x, it.value, rel.value

    def stats(self):
        """Statistics of the last pf_solve (see pf_solve_stats)."""
        keys = ["iters", "outer", "solve_ms", "metric", "matvec64", "matvec32", "relres"]
        return dict(zip(keys, self.stats_raw().tolist()))

    def stats_raw(self):
        """The 8 raw statistics words; after pf_solve_multi: [0] max iterations,
        [1] corrections, [2] solve ms, [3] element-product ms, [4] scatter ms,
        [5] iteration ms, [6] iterations launched."""
        s = np.zeros(8)
        _check(lib().pf_solve_stats(self._ref, s.ctypes.data, _i(8)), "pf_solve_stats")
        return s

    def bench_iterations(self, prec: int, steps: int):
        a, b, c = ctypes.c_double(0), ctypes.c_double(0), ctypes.c_double(0)
        _check(lib().pf_bench_iterations(self._ref, _i(prec), _i(steps), ctypes.byref(a), ctypes.byref(b),
                                         ctypes.byref(c)), "pf_bench_iterations")
        return a.value, b.value, c.value

    def multi_free(self):
        """Releases this context's block-solve buffers (pf_multi_free); the
        next block solve or product allocates them again."""
        _check(lib().pf_multi_free(self._ref), "pf_multi_free")

    def solve_multi(self, R, tol, limit, prec=16):
        """k load cases together (k = R.shape[1], a multiple of 8): R (neq, k)
        -> X (neq, k), iters (k,), relres (k,)."""
        Rf = np.asfortranarray(R, dtype=np.float64)
        if Rf.ndim != 2 or Rf.shape[0] != self.neq:
            raise ValueError("R must be (neq, k)")
        k = Rf.shape[1]
        X = np.zeros((self.neq, k), order="F")
        it = np.zeros(k, np.int32)
        rel = np.zeros(k)
        _check(lib().pf_solve_multi(self._ref, _i(k), Rf.ctypes.data, _d(tol), _i(limit), _i(prec),
                                    X.ctypes.data, it.ctypes.data, rel.ctypes.data), "pf_solve_multi")
        return X, it, rel

    def ebe_matvec_multi(self, Pm, prec=16):
        Pf = np.asfortranarray(Pm, dtype=np.float64)
        k = Pf.shape[1]
        U = np.zeros((self.neq, k), order="F")
        _check(lib().pf_ebe_matvec_multi(self._ref, _i(k), _i(prec), Pf.ctypes.data, U.ctypes.data),
               "pf_ebe_matvec_multi")
        return U

    def multi_product_ms(self, Pm, reps: int = 5) -> float:
        """Average device time of one tensor-core block product U = K P over
        the k columns of Pm (resident on the device; CUDA events)."""
        Pf = np.asfortranarray(Pm, dtype=np.float64)
        ms = ctypes.c_double(0)
        _check(lib().pf_multi_product_ms(self._ref, _i(Pf.shape[1]), Pf.ctypes.data, _i(reps), ctypes.byref(ms)),
               "pf_multi_product_ms")
        return ms.value

    def multi_tuning(self):
        """The tensor-core block product's pass width for the current k and
        the candidates' timings (ms per full product)."""
        kb = ctypes.c_int(0)
        cand = np.zeros(4, np.int32)
        ms = np.zeros(4, np.float32)
        _check(lib().pf_multi_tuning(self._ref, ctypes.byref(kb), cand.ctypes.data, ms.ctypes.data),
               "pf_multi_tuning")
        return {"kb": kb.value, "ms": {int(c): float(m) for c, m in zip(cand, ms) if c}}

    def centroid_stress(self, x, iel: int = 1):
        x, px = _arr(x, np.float64)
        s = np.zeros(6)
        _check(lib().pf_centroid_stress(self._ref, _i(iel), px, s.ctypes.data), "pf_centroid_stress")
        return s

    def element_stresses(self, x, first: int = 1, count=None):
        """Centroid stresses of elements first..first+count-1 (1-based): (count, 6)."""
        x, px = _arr(x, np.float64)
        count = self.nels - first + 1 if count is None else count
        s = np.zeros((max(count, 1), 6))
        _check(lib().pf_element_stresses(self._ref, px, _i(first), _i(count), s.ctypes.data),
               "pf_element_stresses")
        return s

    def launches(self) -> int:
        n = ctypes.c_longlong(0)
        _check(lib().pf_kernel_launches(self._ref, ctypes.byref(n)), "pf_kernel_launches")
        return n.value

    def tuning(self):
        """The autotuned (warps, stages) of the packed-symmetric kernel and the timed configurations."""
        w, st = ctypes.c_int(0), ctypes.c_int(0)
        ms = np.zeros(3, np.float32)
        _check(lib().pf_tuning(self._ref, ctypes.byref(w), ctypes.byref(st), ms.ctypes.data), "pf_tuning")
        return {"warps": w.value, "stages": st.value,
                "ms": {"14x2": float(ms[0]), "12x2": float(ms[1]), "8x3": float(ms[2])}}

    def tuning16(self):
        """The autotuned (warps, stages) of the packed FP16 kernel and the timed configurations."""
        w, st = ctypes.c_int(0), ctypes.c_int(0)
        ms = np.zeros(3, np.float32)
        _check(lib().pf_tuning16(self._ref, ctypes.byref(w), ctypes.byref(st), ms.ctypes.data), "pf_tuning16")
        return {"warps": w.value, "stages": st.value,
                "ms": {"20x2": float(ms[0]), "24x2": float(ms[1]), "28x2": float(ms[2])}}

    def set_graphs(self, on: bool) -> None:
        """Replay PCG iterations from a CUDA graph (default) or launch each kernel directly."""
        _check(lib().pf_set_graphs(self._ref, ctypes.byref(ctypes.c_int(1 if on else 0))), "pf_set_graphs")

    def set_persistent(self, on: bool) -> None:
        """Run the PCG iteration's scatter, updates and finish (and whole FP64
        iterations) as persistent cooperative kernels, or as the separate
        kernels (the default)."""
        _check(lib().pf_set_persistent(self._ref, ctypes.byref(ctypes.c_int(1 if on else 0))), "pf_set_persistent")

    def check_wait_timeout(self, polls: int) -> tuple[int, str]:
        """Runs one bounded bulk-copy wait that nothing completes; returns the
        status code and the recorded error message (PF_FAILURE and the
        timeout message when the error path works)."""
        rc = lib().pf_check_wait_timeout(self._ref, ctypes.byref(ctypes.c_int(polls)))
        return rc, last_error()

    def set_tuning(self, config: int) -> None:
        """Force configuration 0 (14x2), 1 (12x2) or 2 (8x3); -1 re-runs the autotuner."""
        _check(lib().pf_set_tuning(self._ref, ctypes.byref(ctypes.c_int(config))), "pf_set_tuning")


PF_BUSY = 2


class Batch:
    """Continuous-batching engine (pf_batch_*): many solves resident at once,
    admitted by a device-memory budget, retired when converged."""

    def __init__(self, budget_bytes: int, max_meshes: int = 256, device: int = 0, prec: int = 64):
        """prec 64: FP64 element products; 32: FP32 products with FP64 residual replacement;
        16: FP16 storkm in the products, with the same replacement."""
        self._h = ctypes.c_void_p(None)
        _check(lib().pf_batch_create(_i(device), ctypes.byref(ctypes.c_longlong(int(budget_bytes))),
                                     _i(max_meshes), _i(prec), ctypes.byref(self._h)), "pf_batch_create")

    @property
    def _ref(self):
        if not self._h.value:
            raise PfError("batch is closed")
        return ctypes.byref(self._h)

    def close(self):
        if self._h.value:
            lib().pf_batch_destroy(ctypes.byref(self._h))

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def capacity(self):
        a, b = ctypes.c_longlong(0), ctypes.c_longlong(0)
        _check(lib().pf_batch_capacity(self._ref, ctypes.byref(a), ctypes.byref(b)), "pf_batch_capacity")
        return a.value, b.value

    def admit(self, g_num, g_g, g_coord, nn, neq, e, v, r, tol=1e-8, limit=20000, nip=27):
        """Returns the solve id, or None when the budget is full right now."""
        g_num, pn = _arr(g_num, np.int32)
        g_g, pg = _arr(g_g, np.int32)
        g_coord, pc = _arr(g_coord, np.float64)
        e, pe = _arr(np.atleast_1d(e), np.float64)
        v, pv = _arr(np.atleast_1d(v), np.float64)
        r, pr = _arr(r, np.float64)
        sid = ctypes.c_int(-1)
        rc = lib().pf_batch_admit(self._ref, _i(g_num.shape[0]), _i(nn), _i(neq), pn, pg, pc, _i(e.size), pe, pv,
                                  _i(nip), pr, _d(tol), _i(limit), ctypes.byref(sid))
        if rc == PF_BUSY:
            return None
        _check(rc, "pf_batch_admit")
        return sid.value

    def launch(self, iters: int):
        _check(lib().pf_batch_launch(self._ref, _i(iters)), "pf_batch_launch")

    def sync(self):
        a, d = ctypes.c_int(0), ctypes.c_int(0)
        _check(lib().pf_batch_sync(self._ref, ctypes.byref(a), ctypes.byref(d)), "pf_batch_sync")
        return a.value, d.value

    def collect(self, x_cap: int):
        sid, it, neq = ctypes.c_int(0), ctypes.c_int(0), ctypes.c_int(0)
        rel = ctypes.c_double(0.0)
        x = np.zeros(max(int(x_cap), 1))
        _check(lib().pf_batch_collect(self._ref, ctypes.byref(sid), ctypes.byref(it), ctypes.byref(rel),
                                      x.ctypes.data, _i(x.size), ctypes.byref(neq)), "pf_batch_collect")
        return sid.value, it.value, rel.value, x[:neq.value].copy()

    def launches(self) -> int:
        n = ctypes.c_longlong(0)
        _check(lib().pf_batch_launches(self._ref, ctypes.byref(n)), "pf_batch_launches")
        return n.value

    def set_graphs(self, on: bool) -> None:
        """Replay iteration chunks from a CUDA graph (default) or launch each kernel directly."""
        _check(lib().pf_batch_set_graphs(self._ref, ctypes.byref(ctypes.c_int(1 if on else 0))),
               "pf_batch_set_graphs")

    def run_all(self, x_cap: int, chunk: int = 8):
        """Iterates until every resident solve has retired; returns the results."""
        out = {}
        while True:
            self.launch(chunk)
            active, done = self.sync()
            for _ in range(done):
                sid, it, rel, x = self.collect(x_cap)
                out[sid] = (it, rel, x)
            if active == 0:
                return out


def top_face_z_equations(g_g, nxe, nze):
    """Equations (1-based) of the z dofs of the top-face nodes of a GEOMETRY_20BXZ cube."""
    g_g = np.asarray(g_g)
    top = np.nonzero(np.arange(g_g.shape[0]) % (nxe * nze) < nxe)[0]
    local = np.array([3, 4, 5, 10, 11, 15, 16, 17]) - 1
    eqs = g_g[top][:, 3 * local + 2].ravel()
    return np.unique(eqs[eqs > 0])


def random_top_loads(g_g, nxe, nze, neq, k, seed):
    """k load cases of i.i.d. N(0,1) vertical forces on the top-face nodes (seeded)."""
    eqs = top_face_z_equations(g_g, nxe, nze)
    rng = np.random.default_rng(seed)
    R = np.zeros((neq, k), order="F")
    R[eqs - 1, :] = rng.standard_normal((eqs.size, k))
    return R


def mesh_box8(nxe, nye, nze, aa=1.0, bb=1.0, cc=1.0):
    """GEOMETRY_8BXZ box of 8-node bricks: (g_num (nels,8), g_coord (nels,3,8), nn)."""
    nels = nxe * nye * nze
    g_num = np.zeros((nels, 8), np.int32)
    g_coord = np.zeros((nels, 3, 8), np.float64)
    _check(lib().pf_mesh_box8(_i(nxe), _i(nye), _i(nze), _d(aa), _d(bb), _d(cc), g_num.ctypes.data,
                              g_coord.ctypes.data), "pf_mesh_box8")
    return g_num, g_coord, (nxe + 1) * (nye + 1) * (nze + 1)


def box8_restraints(nxe, nye, nze):
    """box_bc8: per node 1 = free, 0 = restrained."""
    fix = np.zeros((nxe + 1) * (nye + 1) * (nze + 1), np.int32)
    _check(lib().pf_box8_restraints(_i(nxe), _i(nye), _i(nze), fix.ctypes.data), "pf_box8_restraints")
    return fix


def number_equations1(g_num, node_fix):
    """One freedom per node: g_g (nels, nod), 0 = restrained, and neq."""
    g_num, pn = _arr(g_num, np.int32)
    node_fix, pf = _arr(node_fix, np.int32)
    g_g = np.zeros(g_num.shape, np.int32)
    neq = ctypes.c_int(0)
    _check(lib().pf_number_equations1(_i(g_num.shape[0]), _i(node_fix.shape[0]), _i(g_num.shape[1]), pn, pf,
                                      g_g.ctypes.data, ctypes.byref(neq)), "pf_number_equations1")
    return g_g, neq.value


def box8_problem(nxe, nye, nze, aa=1.0, bb=1.0, cc=1.0, load=10.0):
    """p123's box: 8-node bricks, box_bc8 restraints, a load at equation
    nres = nxe*(nze-1)+1 (the freedom p12meshgen loads).  Host only."""
    g_num, g_coord, nn = mesh_box8(nxe, nye, nze, aa, bb, cc)
    fix = box8_restraints(nxe, nye, nze)
    g_g, neq = number_equations1(g_num, fix)
    nres = nxe * (nze - 1) + 1
    r = np.zeros(neq)
    r[nres - 1] = load
    return dict(g_num=g_num, g_coord=g_coord, nn=nn, g_g=g_g, neq=neq, r=r, fix=fix, nres=nres,
                nxe=nxe, nye=nye, nze=nze)


def p123_run(job: str, device: int = 0):
    it = ctypes.c_int(0)
    pot = np.zeros(4)
    _check(lib().pf_p123_run(os.fsencode(job), _i(device), ctypes.byref(it), pot.ctypes.data), "pf_p123_run")
    return it.value, pot


def p122_run(job: str, device: int = 0):
    incs = ctypes.c_int(0)
    _check(lib().pf_p122_run(os.fsencode(job), _i(device), ctypes.byref(incs)), "pf_p122_run")
    return incs.value


def cube_problem(nxe, nye, nze, bc=1, pressure=None, aa=1.0, bb=1.0, cc=1.0):
    """Synthetic cube problem: mesh, restraints (bc 1 = fixed base), numbering and
    the top-pressure load vector (total load -1 by default).  Host only."""
    g_num, g_coord, nn = mesh_cube(nxe, nye, nze, aa, bb, cc)
    fix = cube_restraints(nxe, nye, nze, bc, nn)
    g_g, neq = number_equations(g_num, fix)
    if pressure is None:
        pressure = 1.0 / (nxe * aa * nye * bb)
    r = cube_top_pressure(nxe, nze, g_g, neq, pressure, aa, bb)
    return dict(g_num=g_num, g_coord=g_coord, nn=nn, g_g=g_g, neq=neq, r=r, fix=fix,
                nxe=nxe, nye=nye, nze=nze)
