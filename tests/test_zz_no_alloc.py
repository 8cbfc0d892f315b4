"""The allocation-free reduction entry point (mpm_energy_reduce_noalloc).

It serves hosts that cannot allocate device memory inside a solver call: the
caller owns every device array and passes pointers; the entry point's own
scratch is a fixed __device__ array. This test calls it through the C ABI on
device arrays the test allocates itself, twice in a row (the second call must
not see the first call's leftovers), and checks both results bit for bit
against the context path (the FP64 strict form's calcEnergy reduction) on the
same particle state. Two sizes: the small Taylor bar (66 blocks) and a block
of 327,680 particles, which reaches the 1024-block cap, so that every thread
loops over several particles and the last block combines four block partials
per thread -- the paths that use the whole partial-sum area of the scratch
array and its arrival counter.
The file name makes pytest collect it last.
"""
import ctypes
import glob
import os

import numpy as np
import pytest


def _cudart():
    cands = []
    for pat in ("/usr/local/cuda/lib64/libcudart.so*", "/usr/local/cuda/targets/*/lib/libcudart.so*",
                "/usr/lib/*/libcudart.so*"):
        cands += sorted(glob.glob(pat))
    for c in cands:
        try:
            lib = ctypes.CDLL(c)
            lib.cudaMalloc.argtypes = [ctypes.POINTER(ctypes.c_void_p), ctypes.c_size_t]
            lib.cudaMemcpy.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_size_t, ctypes.c_int]
            lib.cudaFree.argtypes = [ctypes.c_void_p]
            lib.cudaDeviceSynchronize.argtypes = []
            return lib
        except OSError:
            continue
    pytest.skip("libcudart not found")


def _to_device(rt, a):
    a = np.ascontiguousarray(a, dtype=np.float64)
    p = ctypes.c_void_p()
    assert rt.cudaMalloc(ctypes.byref(p), a.nbytes) == 0
    assert rt.cudaMemcpy(p, a.ctypes.data, a.nbytes, 1) == 0  # host -> device
    return p


def _decks():
    from mpm3d_gb300 import decks

    return {
        "taylor_bar_2080": decks.taylor_bar(dp=8e-4),
        "elastic_block_327680": decks.generic_block("1 elas 1000 1e7 0.3", counts=(80, 64, 64),
                                                    velocity=(1.0, -2.0, -5.0)),
    }


@pytest.mark.gpu
@pytest.mark.parametrize("case", ["taylor_bar_2080", "elastic_block_327680"])
def test_noalloc_energy_matches_context(gpu_mod, case):
    lib = gpu_mod.library()
    rt = _cudart()
    deck = gpu_mod.Deck.parse(_decks()[case])
    step = gpu_mod.MpmStep(deck, precision="fp64", device=0)
    step.run(3, graph=False)
    step.calcEnergy()
    ref = step.scalars()
    vxp, mass, ie = step.download("VXp"), step.download("mass"), step.download("ie")
    np_ = mass.size
    if case.startswith("elastic_block"):
        assert np_ > 1024 * 256  # more particles than one pass of the capped grid
    d_v, d_m, d_e = _to_device(rt, vxp), _to_device(rt, mass), _to_device(rt, ie)
    d_out = ctypes.c_void_p()
    assert rt.cudaMalloc(ctypes.byref(d_out), 6 * 8) == 0
    want = np.array([ref["EngKinetic"], ref["EngInternal"], ref["Momentum_x"], ref["Momentum_y"],
                     ref["Momentum_z"], float(np.max(np.abs(vxp)))])
    try:
        for call in range(2):
            st = lib.mpm_energy_reduce_noalloc(d_v, d_m, d_e, np_, d_out, None)
            assert st == 0, f"call {call}: status {st}"
            got = np.zeros(6)
            assert rt.cudaMemcpy(got.ctypes.data, d_out, 6 * 8, 2) == 0  # device -> host
            # the same block tree and combine order as the step's reduction
            np.testing.assert_array_equal(got, want, err_msg=f"call {call}")
        # sizes beyond the stated maximum are refused before any work
        assert lib.mpm_energy_reduce_noalloc(d_v, d_m, d_e, (1 << 27) + 1, d_out, None) == 1
        assert lib.mpm_energy_reduce_noalloc(d_v, d_m, d_e, 0, d_out, None) == 1
    finally:
        for p in (d_v, d_m, d_e, d_out):
            rt.cudaFree(p)
        step.close()
