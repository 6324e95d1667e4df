"""The RBF stage of the precompute on the GPU (afar_precompute_fields_device): every array of the
bundle bit-identical to the host precompute's, on the four small meshes (both stencil types,
triangles, quads, mixed, a fixed-value inlet), a periodic mesh and a 100k-cell forward step."""
import numpy as np
import pytest

from conftest import gpu_available, small_cases

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def need_gpu():
    if not gpu_available():
        pytest.skip("no CUDA device")


def _same_bundle(a, b):
    assert a.sizes == b.sizes
    assert sorted(a.a) == sorted(b.a)
    for k in a.a:
        x, y = np.ascontiguousarray(a.a[k]), np.ascontiguousarray(b.a[k])
        assert x.dtype == y.dtype and x.shape == y.shape, k
        assert np.array_equal(x.view(np.uint8), y.view(np.uint8)), k


@pytest.mark.parametrize("name", ["quad_riemann", "ffs_tri", "ffs_tri_hilbert", "mixed_riemann", "corner_flow"])
def test_device_rbf_stage_is_bit_identical(name):
    from afar_cudaeuler2dmixo3rk3solver_gb300 import CaseConfig, precompute

    m, W, Wb, st = small_cases()[name]
    cfg = CaseConfig(stencilType=st)
    host = precompute(m, cfg, W, Wb, want_rbf64=True)
    dev = precompute(m, cfg, W, Wb, want_rbf64=True, device=0)
    _same_bundle(host, dev)


def test_device_rbf_stage_periodic_and_large():
    from afar_cudaeuler2dmixo3rk3solver_gb300 import CaseConfig, mesh, precompute

    m = mesh.periodic_quad_grid(48, 40, 0.0, 10.0, 0.0, 10.0)
    W = mesh.vortex_fields(m.cell_centres())
    cfg = CaseConfig(stencilType="edgeNeighbour")
    _same_bundle(precompute(m, cfg, W, None, want_rbf64=True), precompute(m, cfg, W, None, want_rbf64=True, device=0))
    m = mesh.forward_step_triangles(50_000, seed=11)
    W, Wb = mesh.uniform_fields(m, 1.0, 3.0, 0.0, 1.0)
    host = precompute(m, cfg, W, Wb)
    dev = precompute(m, cfg, W, Wb, device=0)
    assert dev.nc > 90_000
    _same_bundle(host, dev)


def test_device_precompute_bad_device_is_an_error():
    from afar_cudaeuler2dmixo3rk3solver_gb300 import AfarError, CaseConfig, mesh, precompute
    from afar_cudaeuler2dmixo3rk3solver_gb300 import _ffi

    m = mesh.quad_grid(6, 5)
    W, Wb = mesh.uniform_fields(m, 1.0, 0.0, 0.0, 1.0)
    with pytest.raises(AfarError, match="device"):
        precompute(m, CaseConfig(), W, Wb, device=4096)
    assert _ffi.lib().afar_precompute_fields_device(None, None, None, None, -1, None, None, None) == 1
