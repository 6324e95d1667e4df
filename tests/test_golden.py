"""The CPU oracle against golden vectors produced by the reference's own CUDA kernels (compiled from
its sources, run on a GB300 by tests/golden/make_golden.py): same inputs, one RK3 step, every
intermediate compared stage by stage.  No GPU needed.

Tolerances: flags identical; gradients and face values within 1e-12 relative (double arithmetic of
float-staged values, identical up to FMA contraction); limiters within 1e-6 (float); fluxes and
residuals within 1e-5 of the flux scale (the reference's Roe/KFVS dissipation is float with CUDA's
erfcf/expf, the oracle's uses libm's); states within 1e-6 of the state scale after the update."""
import glob
import os

import numpy as np
import pytest

from conftest import ROOT, rel_err

FILES = sorted(glob.glob(os.path.join(ROOT, "tests", "golden", "*.npz")))
SIZE_KEYS = ["cellsNum", "facesNum", "patchesNum", "totalBoundaryFacesNum", "maxStencilSize", "maxCompactStencilSize",
             "maxLocalBlockStencilSize", "maxCompactLocalBlockStencilSize"]


def _load(path):
    from afar_cudaeuler2dmixo3rk3solver_gb300.solver import HostFields

    z = np.load(path)
    sizes = dict(zip(SIZE_KEYS, [int(v) for v in z["sizes"]]))
    arrays = {k[3:]: np.ascontiguousarray(z[k]) for k in z.files if k.startswith("in_")}
    hf = HostFields(sizes, arrays)
    R, Cv, CFL, dt = [float(v) for v in z["gas"]]
    return z, hf, R, Cv, CFL, dt


def test_golden_files_present():
    assert len(FILES) >= 2


@pytest.mark.parametrize("path", FILES, ids=[os.path.basename(f)[:-4] for f in FILES])
def test_oracle_matches_reference_kernels(path):
    from oracle.oracle import Oracle

    z, hf, R, Cv, CFL, dt = _load(path)
    o = Oracle(hf, R, Cv, "ref", matrix32=hf.matrix)
    # the oracle's own LS matrix equals the reference kernel's to float rounding
    assert np.abs(o.mat64.astype(np.float32) - hf.matrix).max() <= 2e-7 * np.abs(hf.matrix).max()
    st = {"FD": hf.FD.copy(), "cFD": hf.cFD.copy(), "cFDold": hf.cFD.copy(),
          "si": np.zeros(2 * (hf.nc + hf.nb), dtype=np.int8)}
    assert o.delta_t(st["FD"], CFL) == pytest.approx(dt, rel=1e-13)
    for k in range(3):
        c = o.stage(st, k, dt)
        ref = {n: z[f"stage{k}_{n}"] for n in ("faceFD", "gradFD", "limiter", "shockIndicator", "Flux", "Res", "FD",
                                               "cFD")}
        assert np.array_equal(c["shockIndicator"], ref["shockIndicator"]), f"switch flags differ at stage {k}"
        assert rel_err(c["faceFD"], ref["faceFD"]) <= 1e-12
        assert rel_err(c["gradFD"], ref["gradFD"]) <= 1e-12
        assert rel_err(c["limiter"], ref["limiter"]) <= 1e-6
        scale = np.abs(ref["Flux"]).max()
        assert np.abs(c["Flux"] - ref["Flux"]).max() <= 1e-5 * scale
        assert np.abs(c["Res"] - ref["Res"]).max() <= 1e-5 * scale
        assert np.abs(c["FD"] - ref["FD"]).max() <= 1e-6 * np.abs(ref["FD"]).max()
        # continue from the reference's state so the next stage starts from identical inputs
        st["FD"][:] = ref["FD"]
        st["cFD"][:] = ref["cFD"]
        if k == 2:
            st["cFDold"][:] = ref["cFD"]


@pytest.mark.parametrize("path", FILES, ids=[os.path.basename(f)[:-4] for f in FILES])
def test_golden_step_exercises_every_switch(path):
    z = np.load(path)
    flags = z["stage0_shockIndicator"][1::2]
    assert set(np.unique(flags)) >= {-2, -1, 0, 1}
