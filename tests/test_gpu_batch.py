"""Batched stepping (afar_batch_*): several solves of different meshes, sizes, step controls and end
times advanced by one graph whose launches cover the blocks of every member.

* Composition independence, exact: after any sequence of batch runs, joins and leaves, a member's
  state, time and step count are bitwise the ones it reaches stepped in a batch of its own.
* Agreement with afar_run: a batched member matches the same solve stepped alone within the
  policy's tolerance (the batched kernels read their arguments from a device table, the single-solve
  kernels from the parameter bank; the compiler may contract a multiply-add differently between the
  two, one rounding apart): 1e-5 of the state scale for mixed (FP32 arithmetic), 1e-11 for fp64.
"""
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
        elif name.startswith("ffs_tri"):
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


TOL = {"mixed": 1e-5, "fp64": 1e-11}


def _close(a, b, policy):
    sa, sb = a.state(), b.state()
    for k in ("FD", "cFD"):
        scale = np.abs(sb[k]).max(axis=0)
        assert (np.abs(sa[k] - sb[k]) <= TOL[policy] * scale).all(), f"{k} differs"
    flips = np.count_nonzero(sa["shockIndicator"] != sb["shockIndicator"])
    assert flips <= 0.005 * sa["shockIndicator"].size
    ta, tb = a.time(), b.time()
    assert ta[2] == tb[2] and ta[0] == pytest.approx(tb[0], rel=10 * TOL[policy])


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


def _alone_in_batch(cases, name, policy, steps, ctl):
    from afar_cudaeuler2dmixo3rk3solver_gb300 import Batch

    s = _make(cases, name, policy)
    s.set_step_params(**ctl)
    b = Batch(policy)
    b.add(s)
    b.run(steps)
    b.close()
    return s


@pytest.mark.parametrize("policy", ["mixed", "fp64"])
def test_batch_composition_independent_and_close_to_solo(cases, policy):
    from afar_cudaeuler2dmixo3rk3solver_gb300 import Batch

    ctl = _controls(cases, policy)
    names = list(ctl)
    members = {n: _make(cases, n, policy) for n in names}
    b = Batch(policy)
    for n in names:
        members[n].set_step_params(**ctl[n])
        b.add(members[n])
    assert len(b) == len(names)
    b.run(STEPS)
    for n in names:
        _same(members[n], _alone_in_batch(cases, n, policy, STEPS, ctl[n]))
        solo = _make(cases, n, policy)
        solo.run(STEPS, **ctl[n])
        _close(members[n], solo, policy)
    # the member with an end time stopped there; the others took every step
    assert members["quad_riemann"].time()[2] < STEPS
    assert members["ffs_tri"].time()[2] == STEPS
    b.close()


def test_batch_join_and_leave(cases):
    from afar_cudaeuler2dmixo3rk3solver_gb300 import Batch

    a, b_, c = (_make(cases, n, "mixed") for n in ("ffs_tri", "mixed_riemann", "quad_riemann"))
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
    assert len(batch) == 2
    batch.close()
    _same(a, _alone_in_batch(cases, "ffs_tri", "mixed", 7, {}))
    _same(c, _alone_in_batch(cases, "quad_riemann", "mixed", 4, {}))
    rb = _alone_in_batch(cases, "mixed_riemann", "mixed", 3, {})
    rb.run(2)
    _same(b_, rb)


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
    with pytest.raises(AfarError) as e:
        m.run(1)  # a member is stepped by its batch only
    assert e.value.status == 5
    other = Batch("mixed")
    with pytest.raises(AfarError) as e:
        other.add(m)  # one batch at a time
    assert e.value.status == 5
    m2 = _make(cases, "mixed_riemann", "mixed")
    batch.add(m2)
    assert len(batch) == 2
    batch.members.remove(m2)
    m2.close()  # freeing a member takes it out of its batch
    assert len(batch) == 1
    assert batch.run(1) > 0.0
    batch.remove(m)
    m.run(1)  # stepping alone again after leaving
    other.close()
    batch.close()


@pytest.mark.parametrize("policy", ["mixed", "fp64"])
def test_batch_schedule_block_sizes_do_not_change_results(cases, policy):
    """The batch autotuner's choices: every forced BVD/flux block size gives bitwise the same member
    results (the only reductions are exact minima); the autotuned schedule reports what it timed and
    a second batch of the same shape takes the cached decision."""
    from afar_cudaeuler2dmixo3rk3solver_gb300 import Batch

    names = ["quad_riemann", "ffs_tri", "mixed_riemann"]
    runs = []
    for bvd, flux in ((64, 128), (128, 256), (256, 128), (0, 0)):
        solvers = [_make(cases, n, policy) for n in names]
        b = Batch(policy)
        for s in solvers:
            s.set_step_params()
            b.add(s)
        b.set_schedule(bvd, flux)
        b.run(STEPS)
        sch = b.schedule()
        if bvd:
            assert (sch["bvd_block"], sch["flux_block"]) == (bvd, flux)
        else:
            assert sch["bvd_block"] in (64, 128, 256) and sch["flux_block"] in (128, 256)
        runs.append(([s.state() for s in solvers], [s.time() for s in solvers], sch))
        b.close()
        for s in solvers:
            s.close()
    for states, times, _ in runs[1:]:
        for a, b_ in zip(runs[0][0], states):
            for k in ("FD", "cFD", "shockIndicator"):
                assert np.array_equal(a[k], b_[k]), k
        assert times == runs[0][1]
    # the same shape again: the decision comes from the cache (no launch times measured)
    solvers = [_make(cases, n, policy) for n in names]
    b = Batch(policy)
    for s in solvers:
        s.set_step_params()
        b.add(s)
    sch = b.schedule()
    auto = runs[-1][2]
    assert (sch["bvd_block"], sch["flux_block"]) == (auto["bvd_block"], auto["flux_block"])
    if max(auto["ms_bvd"].values()) > 0:  # this process timed the shape first
        assert max(sch["ms_bvd"].values()) == 0 and max(sch["ms_flux"].values()) == 0
    b.close()
    for s in solvers:
        s.close()


def test_batch_member_keeps_its_own_reconstruct_choice(cases):
    """A mixed-policy member whose solver forces the register-pass reconstruct keeps it in a batch
    (the others run the tile-staged one): the schedule counts it, and its result is bitwise the same
    in a batch with other members as in a batch of its own."""
    from afar_cudaeuler2dmixo3rk3solver_gb300 import Batch

    def run(with_others):
        s = _make(cases, "ffs_tri", "mixed")
        s.set_tuning(1)
        others = [_make(cases, n, "mixed") for n in (["quad_riemann", "mixed_riemann"] if with_others else [])]
        for o in others:
            o.set_tuning(-1)  # autotuned solo; in the batch the tile-staged kernel
        b = Batch("mixed")
        for x in [s] + others:
            x.set_step_params()
            b.add(x)
        b.run(STEPS)
        sch = b.schedule()
        st = s.state()
        b.close()
        for x in [s] + others:
            x.close()
        return st, sch

    alone, sch1 = run(False)
    mixed, sch3 = run(True)
    assert sch1["register_members"] == 1 and sch1["tile_members"] == 0
    assert sch3["register_members"] == 1 and sch3["tile_members"] == 2
    for k in ("FD", "cFD", "shockIndicator"):
        assert np.array_equal(alone[k], mixed[k]), k
