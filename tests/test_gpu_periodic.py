"""Periodic meshes on the GPU: a uniform stream stays uniform, mass is conserved (no boundary
faces: every face flux leaves one cell and enters another), the isentropic vortex of the standard
periodic test ([0,10]^2, centre (5,5), moving with (1,1), t = 2) converges, and the ref policy,
whose flux takes raw cell centres like the reference's kernel, refuses a periodic mesh."""
import numpy as np
import pytest

from conftest import gpu_available

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def need_gpu():
    if not gpu_available():
        pytest.skip("no CUDA device")


def _solver(n, policy, W=None, stencil="edgeNeighbour"):
    from afar_cudaeuler2dmixo3rk3solver_gb300 import CaseConfig, CudaSolver, gauss_quadrature, mesh, precompute

    m = mesh.periodic_quad_grid(n, n, 0.0, 10.0, 0.0, 10.0)
    cfg = CaseConfig(stencilType=stencil, CFL=0.5)
    q = gauss_quadrature(m, cfg)
    if W is None:
        U0 = mesh.vortex_cell_averages(m, q, 0.0, centre=(5.0, 5.0))
        W0 = mesh.primitive_from_conserved(U0)
    else:
        W0 = np.tile(W, (m.n_cells, 1))
        U0 = mesh.conserved_from_primitive(W0)
    hf = precompute(m, cfg, W0, None, want_rbf64=policy == "fp64")
    s = CudaSolver(hf, cfg, policy=policy)
    s.upload_state(FD=W0, cFD=U0, cFDold=U0)
    return m, q, s


@pytest.mark.parametrize("policy,tol", [("fp64", 1e-12), ("mixed", 1e-6)])
def test_uniform_stream_stays_uniform(policy, tol):
    W = np.array([1.0, 1.0, 0.5, 1.0 / (1.0 / 1.4)])
    m, q, s = _solver(32, policy, W=W)
    s.run(20)
    st = s.state()
    assert np.abs(st["FD"] - W).max() <= tol * np.abs(W).max()
    s.close()


@pytest.mark.parametrize("policy,tol", [("fp64", 1e-12), ("mixed", 1e-6)])
def test_mass_is_conserved(policy, tol):
    m, q, s = _solver(48, policy)
    V = m.cell_areas() * m.depth
    mass0 = float(np.sum(s.state()["cFD"][:, 0] * V))
    s.run(30)
    mass = float(np.sum(s.state()["cFD"][:, 0] * V))
    assert abs(mass - mass0) <= tol * mass0, (mass, mass0)
    s.close()


@pytest.mark.parametrize("policy", ["fp64", "mixed"])
def test_periodic_vortex_converges(policy):
    from afar_cudaeuler2dmixo3rk3solver_gb300 import mesh

    errs = []
    for n in (40, 80):
        m, q, s = _solver(n, policy)
        s.run(8 * n, t_end=2.0)
        t = s.time()[0]
        assert t == pytest.approx(2.0, rel=1e-12)
        rho = s.state()["cFD"][:, 0]
        exact = mesh.vortex_cell_averages(m, q, 2.0, centre=(5.0, 5.0))[:, 0]
        a = m.cell_areas()
        errs.append(float(np.sum(np.abs(rho - exact) * a) / a.sum()))
        s.close()
    print(policy, "periodic vortex L1(rho)", errs)
    assert errs[1] < 0.6 * errs[0] and errs[1] < 5e-4


def test_ref_policy_refuses_periodic_meshes():
    from afar_cudaeuler2dmixo3rk3solver_gb300 import AfarError

    with pytest.raises(AfarError, match="periodic"):
        _solver(8, "ref")
