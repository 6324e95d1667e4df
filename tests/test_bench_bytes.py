"""The roofline numerators of bench.py (algorithmic bytes of a step and of one reconstruct launch)
restated cell by cell and face by face in plain loops on a small mesh, for every policy."""
import numpy as np
import pytest

WORDS = {"mixed": (4, 4, 4, 4), "fp64": (8, 8, 8, 8), "ref": (8, 4, 8, 4)}  # wW, wO, wG, wS


@pytest.fixture(scope="module")
def hf():
    from afar_cudaeuler2dmixo3rk3solver_gb300 import CaseConfig, mesh, precompute

    m = mesh.forward_step_triangles(600, seed=7)
    W, Wb = mesh.uniform_fields(m, 1.0, 3.0, 0.0, 1.0)
    return precompute(m, CaseConfig(stencilType="edgeNeighbour"), W, Wb)


@pytest.mark.parametrize("policy", ["mixed", "fp64", "ref"])
def test_step_bytes(hf, policy):
    import bench

    wW, wO, _, _ = WORDS[policy]
    S = [int(v) for v in hf.stencilSize]
    M = [int(v) for v in hf.compactStencilSize]
    stage = 0
    for c in range(hf.nc):  # W in/out, U^n, U in/out, x y V, LS rows, stencil and face ids, counts
        stage += 8 * wW + 96 + 24 + 2 * M[c] * wO + 4 * S[c] + 4 * M[c] + 2
    for f in range(hf.nf):  # geometry, owner/neighbour, O3 weights of both sides
        o, n = int(hf.neighbour[2 * f]), int(hf.neighbour[2 * f + 1])
        stage += 40 + 8 + (S[o] + 1 + S[n] + 1) * wO
    stage += hf.nb * (40 + 4 + 1 + 4 * wW)  # geometry, owner, label, ghost write
    step = 3 * stage + hf.nc * (4 * wW + 16) + 48 * hf.nf  # + the CFL step
    assert bench.algorithmic_bytes_per_step(hf, policy) == pytest.approx(step, rel=1e-15)


@pytest.mark.parametrize("policy", ["mixed", "fp64", "ref"])
def test_reconstruct_launch_bytes(hf, policy):
    import bench

    wW, wO, wG, wS = WORDS[policy]
    S = [int(v) for v in hf.stencilSize]
    M = [int(v) for v in hf.compactStencilSize]
    total = 0
    for c in range(hf.nc):
        total += 4 * wW                 # own state
        total += 2 * M[c] * wO          # LS rows
        total += 4 * S[c] + 4 * M[c] + 2  # stencil ids, face ids, counts
        total += 4 * M[c] * wG          # face geometry (dx, dy) and (delta r, fraction)
        total += 8 * wG + 4 * wS + 1    # gradient, limiter, troubled flag out
    own = 0 if policy == "mixed" else 1  # the mixed sums (difference form) read no own-cell weight
    for f in range(hf.nf):
        o, n = int(hf.neighbour[2 * f]), int(hf.neighbour[2 * f + 1])
        total += (S[o] + own + S[n] + own) * wO + 8 * wG  # O3 weights in, face values of both sides out
    assert bench.reconstruct_bytes_per_launch(hf, policy) == pytest.approx(total, rel=1e-15)
