"""afar_adjustTimeStep_noalloc, the entry point for callers that cannot allocate device memory
(an application that hands out all GPU memory from its own pool, or has reserved its budget up
front, and forbids libraries to allocate): it takes device pointers the caller owns, keeps its only
scratch in a static device array, and must give the same Courant step as afar_adjustTimeStep.

This file sorts last so that a run which stops at the first failure has run every other test."""
import numpy as np
import pytest

from conftest import gpu_available, small_cases

pytestmark = pytest.mark.gpu

BLOCK = 256  # faces per block minimum in the entry point's scratch


def test_noalloc_courant_step_matches_adjust_time_step_on_two_calls():
    if not gpu_available():
        pytest.skip("no CUDA device")
    import torch

    from afar_cudaeuler2dmixo3rk3solver_gb300 import CaseConfig, CudaSolver, _ffi, precompute

    L = _ffi.lib()
    cases = small_cases()
    # two calls in a row; the second mesh has fewer blocks of faces than the first, so it reads only
    # scratch entries the first call also wrote, and must not see that call's minima
    names = ("mixed_riemann", "quad_riemann")
    nblocks = []
    for i, name in enumerate(names):
        m, W, Wb, st = cases[name]
        cfg = CaseConfig(stencilType=st)
        hf = precompute(m, cfg, W, Wb)
        nblocks.append((hf.nf + BLOCK - 1) // BLOCK)
        s = CudaSolver(hf, cfg, policy="ref")
        s.run(3)  # a non-uniform state
        FD = s.state()["FD"]
        expected = s.set_delta_t()  # the existing entry point
        s.close()

        def dev(a):
            return torch.from_numpy(np.ascontiguousarray(a)).cuda()

        FD_d, CELL_d, FACE_d, NB_d = dev(FD), dev(hf.CELL), dev(hf.FACE), dev(hf.neighbour)
        out = torch.full((1,), -1.0, dtype=torch.float64, device="cuda")
        torch.cuda.synchronize()
        free0 = torch.cuda.mem_get_info()[0]
        _ffi.check(L.afar_adjustTimeStep_noalloc(FD_d.data_ptr(), CELL_d.data_ptr(), FACE_d.data_ptr(),
                                                 NB_d.data_ptr(), hf.nf, cfg.R, cfg.Cv, cfg.CFL, out.data_ptr(), None))
        torch.cuda.synchronize()
        free1 = torch.cuda.mem_get_info()[0]
        got = out.item()
        assert got == pytest.approx(expected, rel=1e-15, abs=0), (name, got, expected)
        if i > 0:
            # the first call on a device may load this file's device code (with its static scratch
            # array) once; every later call must leave the device's free memory as it found it
            assert free1 == free0, f"free device memory changed by {free0 - free1} bytes over the call"
    assert nblocks[1] < nblocks[0], nblocks


def test_noalloc_rejects_meshes_beyond_its_scratch():
    from afar_cudaeuler2dmixo3rk3solver_gb300 import _ffi

    L = _ffi.lib()
    import ctypes as C

    dummy = C.c_double()
    st = L.afar_adjustTimeStep_noalloc(C.addressof(dummy), C.addressof(dummy), C.addressof(dummy),
                                       C.addressof(dummy), 16_777_217, 1 / 1.4, 2.5, 0.5, C.addressof(dummy), None)
    assert st == 3  # AFAR_ERR_LIMIT, before anything touches the GPU
    assert b"exceeds the limit" in L.afar_last_error()
