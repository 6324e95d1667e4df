"""A reference-style OpenFOAM case run on the GPU (the reference application's time loop): the
forward-step case written by the tests, stepped to endTime with the device CFL step, landing on
every write time like OpenFOAM's adjustableRunTime, fields written in OpenFOAM format."""
import os

import numpy as np
import pytest

from conftest import gpu_available
from foam_case import write_case

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def need_gpu():
    if not gpu_available():
        pytest.skip("no CUDA device")


def test_run_case_writes_every_write_time(tmp_path):
    from afar_cudaeuler2dmixo3rk3solver_gb300 import foam

    case_dir = write_case(str(tmp_path / "case"), n=4, end=0.02, wi=0.005)
    out = str(tmp_path / "out")
    res = foam.run_case(case_dir, out, policy="mixed")
    assert res["write_times"] == pytest.approx([0.005, 0.01, 0.015, 0.02])
    assert res["time"] == pytest.approx(0.02, rel=1e-12) and res["steps"] > 4
    for t in ("0", "0.005", "0.01", "0.015", "0.02"):
        p = foam.read_field(os.path.join(out, t, "p"))
        assert p.shape == (res["cells"],) and np.isfinite(p).all() and (p > 0).all()
    assert os.path.exists(os.path.join(out, "constant", "polyMesh", "faces"))


def test_write_interval_spreads_the_steps_to_the_write_time(tmp_path):
    from afar_cudaeuler2dmixo3rk3solver_gb300 import CudaSolver, foam, precompute

    case = foam.load_case(write_case(str(tmp_path / "case"), n=4))
    hf = precompute(case.mesh, case.config, case.W, case.Wb)
    wi = 0.003
    for landing in (False, True):
        s = CudaSolver(hf, case.config, policy="fp64")
        if landing:
            s.set_write_interval(wi)
        dts = []
        t_prev = 0.0
        for _ in range(500):
            s.run(1, t_end=wi)
            t, last, n = s.time()
            if t <= t_prev:
                break
            dts.append(t - t_prev)
            t_prev = t
        s.close()
        assert t == pytest.approx(wi, rel=1e-12)
        if landing:
            # OpenFOAM's rule spreads the remainder: no step is cut to a sliver at the write time
            assert min(dts) >= 0.2 * max(dts)
            assert dts[-1] == pytest.approx(dts[-2], rel=0.2)
        else:
            plain = dts
    assert len(dts) <= len(plain) + 1


def test_recalc_basis_false_reuses_the_written_weights(tmp_path):
    """A first run computes the O3 weights and writes system/basisOwnList/basisNeiList; a case with
    recalcBasis false reads them and steps to bit-identical fields (the weights read back exactly)."""
    import shutil

    from afar_cudaeuler2dmixo3rk3solver_gb300 import foam

    first = write_case(str(tmp_path / "a"), n=2, end=0.004, wi=0.002)
    foam.run_case(first, first, policy="fp64")
    assert os.path.exists(os.path.join(first, "system", "basisOwnList"))
    second = write_case(str(tmp_path / "b"), n=2, end=0.004, wi=0.002, recalc_basis=False)
    for name in foam.BASIS_FILES:
        shutil.copy(os.path.join(first, "system", name), os.path.join(second, "system", name))
    res = foam.run_case(second, second, policy="fp64")
    assert res["time"] == pytest.approx(0.004, rel=1e-12)
    for t in ("0.002", "0.004"):
        for f in ("p", "U", "T"):
            a = foam.read_field(os.path.join(first, t, f))
            b = foam.read_field(os.path.join(second, t, f))
            assert np.array_equal(a, b), (t, f)


def test_run_case_in_binary_write_format(tmp_path):
    """writeFormat binary (the reference case's setting): the fields, the polyMesh and the O3
    weight files come out in OpenFOAM's binary form, hold the same values as the ascii run (to the
    ascii files' 9 digits; the state is the same, bit for bit), and the binary weight files feed a
    recalcBasis false run that reproduces the first."""
    from afar_cudaeuler2dmixo3rk3solver_gb300 import foam

    res, outs = {}, {}
    for fmt in ("ascii", "binary"):
        case_dir = write_case(str(tmp_path / f"case_{fmt}"), n=4, end=0.01, wi=0.005, write_format=fmt)
        outs[fmt] = str(tmp_path / f"out_{fmt}")
        res[fmt] = foam.run_case(case_dir, outs[fmt], policy="fp64")
    assert res["ascii"]["steps"] == res["binary"]["steps"]
    for t in ("0.005", "0.01"):
        for name in ("p", "U", "T"):
            head = open(os.path.join(outs["binary"], t, name), "rb").read(200)
            assert b"format      binary;" in head
            a = foam.read_field(os.path.join(outs["ascii"], t, name))
            b = foam.read_field(os.path.join(outs["binary"], t, name))
            assert np.allclose(a, b, rtol=1e-8, atol=1e-12), (t, name)
    m = foam.read_poly_mesh(outs["binary"], {0: 3, 1: 4, 2: 2})
    assert m.n_cells == res["binary"]["cells"]
    # rerun from the binary weight files (recalcBasis false): the same final fields, bit for bit
    again = write_case(str(tmp_path / "again"), n=4, end=0.01, wi=0.005, recalc_basis=False, write_format="binary")
    import shutil
    for f in foam.BASIS_FILES:
        shutil.copy(os.path.join(outs["binary"], "system", f), os.path.join(again, "system", f))
    out2 = str(tmp_path / "out_again")
    foam.run_case(again, out2, policy="fp64")
    for name in ("p", "U", "T"):
        assert np.array_equal(foam.read_field(os.path.join(out2, "0.01", name)),
                              foam.read_field(os.path.join(outs["binary"], "0.01", name)))
