"""pf_ebe_matvec_noalloc: the element-by-element product for callers that
cannot allocate device memory while they run.

The test allocates the caller's buffers itself (through the xx3-layer entry
points, as such a caller would at start-up) and checks two calls in a row
against pf_ebe_matvec, the allocating entry point, through the C-ABI.
"""
import ctypes

import numpy as np
import pytest

import parafem_gb300 as P

pytestmark = pytest.mark.gpu


def _i(v):
    return ctypes.byref(ctypes.c_int(int(v)))


class DeviceBuffer:
    """A caller-owned device buffer made with allocate_memory_on_gpu."""

    def __init__(self, host):
        self.host = np.ascontiguousarray(host)
        self.ptr = ctypes.c_void_p()
        L = P.lib()
        assert L.allocate_memory_on_gpu(_i(self.host.size), _i(self.host.itemsize), ctypes.byref(self.ptr)) == 0
        assert L.copy_data_to_gpu(_i(self.host.size), _i(self.host.itemsize), self.host.ctypes.data,
                                  ctypes.byref(self.ptr)) == 0

    def read(self):
        out = np.empty_like(self.host)
        assert P.lib().copy_data_from_gpu(_i(out.size), _i(out.itemsize), out.ctypes.data,
                                          ctypes.byref(self.ptr)) == 0
        return out

    def free(self):
        P.lib().free_memory_on_gpu(ctypes.byref(self.ptr))


def test_noalloc_matches_allocating_entry_point_twice():
    prob = P.cube_problem(6, 5, 4)
    nels, neq = prob["g_num"].shape[0], prob["neq"]
    rng = np.random.default_rng(11)
    with P.Solver() as s:
        s.setup(prob["g_num"], prob["g_g"], prob["g_coord"], prob["nn"], neq)
        s.set_material(*P.random_material(nels, 5, 1.0, 1000.0, 0.2, 0.35))
        s.form_storkm(27)
        km = s.get_storkm()
        ps = [rng.standard_normal(neq) for _ in range(2)]
        refs = [s.ebe_matvec(p, 64) for p in ps]
    bufs = [DeviceBuffer(km), DeviceBuffer(prob["g_g"].astype(np.int32)), DeviceBuffer(np.zeros(neq)),
            DeviceBuffer(np.zeros(neq))]
    d_km, d_gg, d_p, d_u = bufs
    L = P.lib()
    try:
        for p, ref in zip(ps, refs):
            d_p.host[:] = p
            assert L.copy_data_to_gpu(_i(neq), _i(8), d_p.host.ctypes.data, ctypes.byref(d_p.ptr)) == 0
            rc = L.pf_ebe_matvec_noalloc(_i(nels), _i(neq), d_km.ptr, d_gg.ptr, d_p.ptr, d_u.ptr)
            assert rc == 0, P.last_error()
            u = d_u.read()
            assert np.abs(u - ref).max() <= 1e-13 * np.abs(ref).max()
    finally:
        for b in bufs:
            b.free()


def test_noalloc_rejects_sizes_beyond_its_scratch():
    L = P.lib()
    dummy = ctypes.c_void_p(1)
    rc = L.pf_ebe_matvec_noalloc(_i(16385), _i(1000), dummy, dummy, dummy, dummy)
    assert rc == 1 and "scratch limits" in P.last_error()


def test_noalloc_takes_no_device_memory_per_call_and_keeps_u_on_failure():
    """After the set-up call, calls change the device's free memory by
    nothing; a g_g entry out of range fails the call and leaves u as it was."""
    torch = pytest.importorskip("torch")
    L = P.lib()
    torch.cuda.mem_get_info(0)   # the runtime context exists before the measurements
    assert L.pf_ebe_matvec_noalloc(_i(0), _i(0), None, None, None, None) == 0, P.last_error()
    prob = P.cube_problem(3, 3, 3)
    nels, neq = prob["g_num"].shape[0], prob["neq"]
    rng = np.random.default_rng(12)
    km = rng.standard_normal((nels, 60, 60))
    g_g = prob["g_g"].astype(np.int32)
    bufs = [DeviceBuffer(km), DeviceBuffer(g_g), DeviceBuffer(rng.standard_normal(neq)),
            DeviceBuffer(np.full(neq, 7.0))]
    d_km, d_gg, d_p, d_u = bufs
    try:
        free0, _ = torch.cuda.mem_get_info(0)
        for _ in range(2):
            assert L.pf_ebe_matvec_noalloc(_i(nels), _i(neq), d_km.ptr, d_gg.ptr, d_p.ptr, d_u.ptr) == 0
        free1, _ = torch.cuda.mem_get_info(0)
        assert free1 == free0
        good = d_u.read()
        bad = g_g.copy()
        bad[0, 0] = neq + 5
        d_bad = DeviceBuffer(bad)
        bufs.append(d_bad)
        rc = L.pf_ebe_matvec_noalloc(_i(nels), _i(neq), d_km.ptr, d_bad.ptr, d_p.ptr, d_u.ptr)
        assert rc == 1 and "outside 0.." in P.last_error()
        assert np.array_equal(d_u.read(), good)
    finally:
        for b in bufs:
            b.free()
