"""Supersonic compression ramps (the batched workload's solves): the label-6 inflow keeps the state
given at set-up, the flow stays finite through the shock's formation, and the ramp raises the
pressure above the inflow's."""
import numpy as np
import pytest

from conftest import gpu_available

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("policy", ["mixed", "fp64"])
@pytest.mark.parametrize("mach,angle", [(1.5, 20.0), (4.0, 5.0)])
def test_ramp_runs_with_fixed_inflow(policy, mach, angle):
    if not gpu_available():
        pytest.skip("no CUDA device")
    from afar_cudaeuler2dmixo3rk3solver_gb300 import CaseConfig, CudaSolver, mesh, precompute

    m = mesh.wedge_quads(80, 40, angle)
    u0 = mach * np.sqrt(1.4)
    W = mesh.vortex_fields(m.cell_centres(), strength=3.0, xc=0.5, yc=0.6, u0=u0, v0=0.0)
    Wb = mesh.vortex_fields(m.boundary_face_centres(), strength=0.0, xc=0.5, yc=0.6, u0=u0, v0=0.0)
    cfg = CaseConfig(stencilType="faceNeighbour", CFL=0.3)
    s = CudaSolver(precompute(m, cfg, W, Wb, want_rbf64=policy == "fp64"), cfg, policy=policy)
    s.run(200)
    FD = s.state()["FD"]
    nc = m.n_cells
    inflow = [p for p in m.patches if p[0] == "inflow"][0]
    b0 = inflow[2] - m.n_internal_faces
    ghosts = FD[nc + b0:nc + b0 + inflow[3]]
    assert np.allclose(ghosts, Wb[b0:b0 + inflow[3]], rtol=1e-6)  # float-stored in mixed
    assert np.isfinite(FD).all() and (FD[:nc, 0] > 0).all() and (FD[:nc, 3] > 0).all()
    assert FD[:nc, 0].max() > 1.2  # the ramp's shock compresses the stream
    s.close()
