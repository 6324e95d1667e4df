"""Edge-case meshes through the CUDA path, stage by stage against the CPU oracle: a single cell
with no internal face (every stencil member a ghost), 130 cells (one full 128-cell tile and a
ragged second one), and a one-cell-high strip of 257 cells (every cell on the boundary, two full
tiles and one cell).  A fixed step size, since a mesh without internal faces has no CFL step.
Policies: fp64 within 1e-10 of the FP64 oracle, ref within 1e-12 of the oracle in the face values
and gradients with identical flags, mixed within 1e-5 of the fp64 policy after whole steps, and its
tile-staged reconstruct (TMA boxes of 128 cells reaching past the rows' ends, which read zeros)
bitwise equal to its register pass."""
import numpy as np
import pytest

from conftest import gpu_available, rel_err

pytestmark = pytest.mark.gpu

FIELDS = ["faceFD", "gradFD", "Flux", "Res", "FD", "cFD"]
DT = 2.0e-4


def _meshes():
    from afar_cudaeuler2dmixo3rk3solver_gb300 import mesh as M

    out = {}
    walls = dict(classify=lambda x, y: np.zeros(x.shape[0], dtype=np.int64), patch_defs=[("walls", M.BC_SLIP)])
    for name, m in (("one_cell", M.quad_grid(1, 1, **walls)), ("ragged_130", M.quad_grid(13, 10, jitter=0.2, seed=2)),
                    ("strip_257", M.quad_grid(257, 1, 0.0, 25.7, 0.0, 0.1))):
        W, Wb = M.riemann_fields(m) if name != "strip_257" else M.uniform_fields(m, 1.0, 0.5, 0.0, 1.0)
        if name == "strip_257":  # a pressure jump in the middle of the strip
            W = W.copy()
            W[m.cell_centres()[:, 0] > 12.85, 0] = 0.3
        if name == "one_cell":  # a moving cell in a box of slip walls
            W = np.array([[1.0, 0.3, -0.2, 1.1]])
        out[name] = (m, W, Wb)
    return out


@pytest.fixture(scope="module")
def cases():
    if not gpu_available():
        pytest.skip("no CUDA device")
    from afar_cudaeuler2dmixo3rk3solver_gb300 import CaseConfig, precompute

    out = {}
    for name, (m, W, Wb) in _meshes().items():
        cfg = CaseConfig(stencilType="edgeNeighbour")
        out[name] = (precompute(m, cfg, W, Wb, want_rbf64=True), cfg)
    return out


NAMES = ["one_cell", "ragged_130", "strip_257"]


@pytest.mark.parametrize("name", NAMES)
def test_sizes(cases, name):
    hf, _ = cases[name]
    assert (hf.nc, hf.nf) == {"one_cell": (1, 0), "ragged_130": (130, 237), "strip_257": (257, 256)}[name]


@pytest.mark.parametrize("name", NAMES)
def test_fp64_policy_vs_oracle(cases, name):
    from afar_cudaeuler2dmixo3rk3solver_gb300 import CudaSolver
    from oracle.oracle import Oracle

    hf, cfg = cases[name]
    s = CudaSolver(hf, cfg, policy="fp64")
    o = Oracle(hf, cfg.R, cfg.Cv, "fp64")
    st = o.new_state()
    for step in range(2):
        for k in range(3):
            a = s.stage_debug(k, DT)
            c = o.stage(st, k, DT)
            assert np.array_equal(a["shockIndicator"], c["shockIndicator"]), f"flags differ step {step} stage {k}"
            for f in FIELDS:
                assert rel_err(a[f], c[f]) <= 1e-10, (f, step, k)
            s.upload_state(FD=c["FD"], cFD=c["cFD"], cFDold=c["cFD"] if k == 2 else None)
    s.close()


@pytest.mark.parametrize("name", NAMES)
def test_ref_policy_vs_oracle(cases, name):
    from afar_cudaeuler2dmixo3rk3solver_gb300 import CudaSolver
    from oracle.oracle import Oracle

    hf, cfg = cases[name]
    s = CudaSolver(hf, cfg, policy="ref")
    o = Oracle(hf, cfg.R, cfg.Cv, "ref", matrix32=s.ls_matrix())
    st = o.new_state()
    for k in range(3):
        a = s.stage_debug(k, DT)
        c = o.stage(st, k, DT)
        assert np.array_equal(a["shockIndicator"], c["shockIndicator"]), f"flags differ stage {k}"
        for f in ("faceFD", "gradFD"):
            assert rel_err(a[f], c[f]) <= 1e-12, (f, k)
        scale = max(np.abs(c["Flux"]).max(), 1e-300)
        assert np.abs(a["Flux"] - c["Flux"]).max() <= 1e-5 * scale
        s.upload_state(FD=c["FD"], cFD=c["cFD"], cFDold=c["cFD"] if k == 2 else None)
    s.close()


@pytest.mark.parametrize("name", NAMES)
def test_mixed_policy_close_to_fp64(cases, name):
    from afar_cudaeuler2dmixo3rk3solver_gb300 import CudaSolver

    hf, cfg = cases[name]
    res = {}
    for policy in ("fp64", "mixed"):
        s = CudaSolver(hf, cfg, policy=policy)
        s.run(5, dt=DT)
        res[policy] = s.state()
        assert s.time()[2] == 5
        s.close()
    a, b = res["mixed"]["FD"][:hf.nc], res["fp64"]["FD"][:hf.nc]
    assert np.isfinite(a).all()
    assert np.abs(a - b).max() <= 1e-5 * np.abs(b).max()


@pytest.mark.parametrize("name", NAMES)
def test_mixed_tile_reconstruct_equals_register_pass(cases, name):
    from afar_cudaeuler2dmixo3rk3solver_gb300 import CudaSolver

    hf, cfg = cases[name]
    res = []
    for variant in (0, 1):  # tile-staged, register pass
        s = CudaSolver(hf, cfg, policy="mixed")
        s.set_tuning(variant)
        s.run(5, dt=DT)
        res.append(s.state())
        s.close()
    for k in ("FD", "cFD", "shockIndicator"):
        assert np.array_equal(res[0][k], res[1][k]), k
