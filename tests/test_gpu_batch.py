"""Batched stepping (afar_batch_*): several solves of different meshes, sizes, step controls and end
times advanced by one graph whose launches cover the blocks of every member.  The contract tested
here is exact: after any sequence of batch runs, joins and leaves, each member's state, time and
step count are bitwise the ones the same solve reaches when stepped alone with afar_run."""
import numpy as np
import pytest

from conftest import gpu_available, small_cases

pytestmark = pytest.mark.gpu

STEPS = 8


@pytest.fixture(scope="module")
def cases():
    if not gpu_available():
        pytest.skip("no CUDA device")
    from afar_cudaeuler2dmixo3rk3solver_gb300 import CaseConfig, precompute

    out = {}
    for name, (m, W, Wb, st) in small_cases().items():
        if name == "corner_flow":
            cfg = CaseConfig(R=0.7142857, Cv=1.7857142857, CFL=0.1, stencilType=st, cOrder=7, fOrder=5)
        elif name == "ffs_tri":
            cfg = CaseConfig(stencilType=st, CFL=0.2)
        else:
            cfg = CaseConfig(stencilType=st)
        out[name] = (precompute(m, cfg, W, Wb, want_rbf64=True), cfg)
    return out


def _make(cases, name, policy):
    from afar_cudaeuler2dmixo3rk3solver_gb300 import CudaSolver

    hf, cfg = cases[name]
    return CudaSolver(hf, cfg, policy=policy)


def _same(a, b):
    sa, sb = a.state(), b.state()
    for k in ("FD", "cFD", "shockIndicator"):
        assert np.array_equal(sa[k], sb[k]), f"{k} differs"
    assert a.time() == b.time()


def _controls(cases, policy):
    """Per-solve step controls: CFL stepping, a fixed step, and an end time reached mid-run."""
    probe = _make(cases, "quad_riemann", policy)
    probe.run(STEPS)
    t_end = 0.6 * probe.time()[0]
    probe.close()
    return {
        "quad_riemann": dict(dt=0.0, cfl=None, t_end=t_end),
        "ffs_tri": dict(dt=0.0, cfl=None, t_end=0.0),
        "mixed_riemann": dict(dt=2.0e-4, cfl=None, t_end=0.0),
        "corner_flow": dict(dt=0.0, cfl=0.08, t_end=0.0),
    }


@pytest.mark.parametrize("policy", ["mixed", "fp64"])
def test_batch_matches_solo(cases, policy):
    from afar_cudaeuler2dmixo3rk3solver_gb300 import Batch

    ctl = _controls(cases, policy)
    names = list(ctl)
    solo = {n: _make(cases, n, policy) for n in names}
    for n in names:
        solo[n].run(STEPS, **ctl[n])
    members = {n: _make(cases, n, policy) for n in names}
    b = Batch(policy)
    for n in names:
        members[n].set_step_params(**ctl[n])
        b.add(members[n])
    assert len(b) == len(names)
    b.run(STEPS)
    for n in names:
        _same(members[n], solo[n])
    # the member with an end time stopped there; the others took every step
    assert members["quad_riemann"].time()[2] < STEPS
    assert members["ffs_tri"].time()[2] == STEPS
    b.close()


def test_batch_join_and_leave(cases):
    from afar_cudaeuler2dmixo3rk3solver_gb300 import Batch

    a, b_, c = (_make(cases, n, "mixed") for n in ("ffs_tri", "mixed_riemann", "quad_riemann"))
    sa, sb, sc = (_make(cases, n, "mixed") for n in ("ffs_tri", "mixed_riemann", "quad_riemann"))
    sa.run(7)
    sb.run(3 + 2)
    sc.run(4)
    batch = Batch("mixed")
    for s in (a, b_):
        s.set_step_params()
        batch.add(s)
    batch.run(3)
    batch.remove(b_)
    c.set_step_params()
    batch.add(c)
    batch.run(4)
    b_.run(2)  # a solve that left the batch continues alone
    _same(a, sa)
    _same(b_, sb)
    _same(c, sc)
    assert len(batch) == 2
    batch.close()


def test_batch_checkpoint_restore_inside(cases):
    """A member's device snapshot taken between batch runs restores to a state that replays bitwise."""
    from afar_cudaeuler2dmixo3rk3solver_gb300 import Batch

    a = _make(cases, "mixed_riemann", "mixed")
    a.set_step_params()
    batch = Batch("mixed")
    batch.add(a)
    batch.run(2)
    a.save()
    batch.run(3)
    first = a.state()
    t_first = a.time()
    a.restore()
    batch.run(3)
    second = a.state()
    assert np.array_equal(first["FD"], second["FD"]) and np.array_equal(first["cFD"], second["cFD"])
    assert a.time() == t_first
    batch.close()


def test_batch_rejects_bad_members(cases):
    from afar_cudaeuler2dmixo3rk3solver_gb300 import AfarError, Batch

    batch = Batch("mixed")
    assert batch.run(1) == 0.0  # empty batch: nothing to do
    f = _make(cases, "quad_riemann", "fp64")
    with pytest.raises(AfarError) as e:
        batch.add(f)  # policy differs
    assert e.value.status == 1
    m = _make(cases, "quad_riemann", "mixed")
    batch.add(m)
    with pytest.raises(AfarError) as e:
        batch.add(m)  # already a member
    assert e.value.status == 5
    with pytest.raises(AfarError):
        batch.remove(f)
    batch.close()
