"""Batched 1D instances (nufi_batch_*): every instance of a batch of uneven
grid sizes against the same configuration run alone through a handle, and
the batched adjoint against the single-instance adjoint and central
differences.

Tolerances: FP64 energy histories 1e-12 of max (the batch sums rho over
other partial rows than a handle; the difference is the FP64 summation
floor); FP32-split within the 1e-6 gate of the FP64 history; gradients
1e-9 of max |dJ| against the single-instance adjoint (FP64 atomics in the
slab adjoints), 1e-5 per component against central differences.
"""
import numpy as np
import pytest

from numericalflowiteration_gb300.config import batched_bump_on_tail, bump_on_tail_1d, landau_1d

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def nufi():
    import numericalflowiteration_gb300 as m
    from numericalflowiteration_gb300 import build
    build.build()
    m.load()
    return m


def small_batch(precision="fp64", count=7, Nt=40):
    return batched_bump_on_tail(count=count, seed=7, Nt=Nt, nx=(16, 32, 64), nv=(32, 64, 128), precision=precision)


def rel(a, b):
    return float(np.max(np.abs(np.asarray(a) - np.asarray(b))) / np.max(np.abs(b)))


def test_batch_fp64_matches_single_handles(nufi):
    cfgs = small_batch()
    with nufi.Batch(cfgs) as b:
        J = b.forward()
        E = [b.energy(i) for i in range(len(cfgs))]
        d = b.describe()
    assert d["instances"] == len(cfgs) and d["autotune"]["chosen"]["ppt"] in (1, 2, 4)
    for i, c in enumerate(cfgs):
        with nufi.Simulation(c) as s:
            Js = s.forward()
            Es = s.energy()
        assert rel(E[i], Es) <= 1e-12, i
        assert abs(J[i] - Js) <= 1e-12 * abs(Js)


def test_batch_split_within_gate(nufi):
    cfgs = small_batch()
    with nufi.Batch([c.replace(precision="fp32split") for c in cfgs]) as b:
        b.forward()
        E = [b.energy(i) for i in range(len(cfgs))]
        d = b.describe()
    assert d["autotune"]["chosen"]["ppt"] in (2, 4, 8)
    for i, c in enumerate(cfgs):
        with nufi.Simulation(c) as s:
            Es = s.run()
        assert rel(E[i], Es) <= 1e-6, i


def test_batch_backward_matches_single_adjoint(nufi):
    cfgs = small_batch()
    with nufi.Batch(cfgs) as b:
        with pytest.raises(IndexError):
            b.backward()
        b.forward()
        G = b.backward()
        G2 = b.backward()
    assert rel(G2, G) <= 1e-13
    for i, c in enumerate(cfgs):
        with nufi.Simulation(c) as s:
            s.forward()
            g = s.backward()
        assert rel(G[i], g) <= 1e-9, (i, G[i], g)


def test_batch_gradient_matches_central_differences(nufi):
    cfgs = small_batch(count=3, Nt=30)
    with nufi.Batch(cfgs) as b:
        b.forward()
        G = b.backward()
    h = 1e-6
    for i in range(4):
        plus, minus = [], []
        for c in cfgs:
            pp = list(c.f0_params)
            pp[i] += h
            plus.append(c.replace(f0_params=list(pp)))
            pp[i] -= 2 * h
            minus.append(c.replace(f0_params=list(pp)))
        with nufi.Batch(plus) as bp:
            Jp = bp.forward()
        with nufi.Batch(minus) as bm:
            Jm = bm.forward()
        fd = (Jp - Jm) / (2 * h)
        assert np.all(np.abs(G[:, i] - fd) <= 1e-5 * np.abs(fd)), (i, G[:, i], fd)


def test_batch_rejects_unsupported(nufi):
    with pytest.raises(NotImplementedError):
        nufi.Batch([landau_1d(Nx=48, Nv=32, Nt=4)])
    with pytest.raises(NotImplementedError):
        nufi.Batch([landau_1d(Nx=16, Nv=32, Nt=4), landau_1d(Nx=16, Nv=32, Nt=4, precision="fp32split")])


def test_batch_split_adjoint_matches_fp64_and_differences(nufi):
    """The FP32-split adjoint (fixed-point reversible characteristics) of a
    split batch against the FP64 adjoint of the same instances and against
    central differences of the FP64 forward: max_i |dG_i| <= 1e-5 max_i |G_i|
    per instance (components far below the largest one carry the FP32
    rounding of the largest)."""
    cfgs = batched_bump_on_tail(count=4, seed=11, Nt=80, nx=(32, 64), nv=(64, 128))
    with nufi.Batch(cfgs) as b:
        b.forward()
        G64 = b.backward()
    with nufi.Batch([c.replace(precision="fp32split") for c in cfgs]) as b:
        b.forward()
        Gs = b.backward()
        Gs2 = b.backward()
    assert rel(Gs2, Gs) <= 1e-6
    for i in range(len(cfgs)):
        assert np.max(np.abs(Gs[i] - G64[i])) <= 1e-5 * np.max(np.abs(G64[i])), (i, Gs[i], G64[i])
    h = 1e-6
    for i in range(4):
        plus, minus = [], []
        for c in cfgs[:2]:
            pp = list(c.f0_params)
            pp[i] += h
            plus.append(c.replace(f0_params=list(pp)))
            pp[i] -= 2 * h
            minus.append(c.replace(f0_params=list(pp)))
        with nufi.Batch(plus) as bp, nufi.Batch(minus) as bm:
            fd = (bp.forward() - bm.forward()) / (2 * h)
        for j in range(2):
            assert abs(Gs[j, i] - fd[j]) <= 1e-5 * np.max(np.abs(G64[j])), (i, j, Gs[j, i], fd[j])


def test_batch_split_one_launch_matches_per_step_launches(nufi):
    """The whole FP32-split batched forward as one cooperative launch
    (batch_run_split_kernel: all steps of all instances, grid barriers
    between the phases) against the CUDA graph of per-step launches: the
    same arithmetic in the same order, so the same bits; the adjoint runs
    on either forward's history."""
    cfgs = [c.replace(precision="fp32split") for c in small_batch()]
    with nufi.Batch(cfgs, opts={"batch_no_autotune": 1}) as a:
        d = a.describe()
        assert d["forward_launch"].startswith("batch_run_split_kernel") and d["forward_ctas"] > 0
        Ja = a.forward()
        Ea = [a.energy(i) for i in range(len(cfgs))]
        assert np.array_equal(a.forward(), Ja)
        Ga = a.backward()
    with nufi.Batch(cfgs, opts={"batch_no_autotune": 1, "no_persistent": 1}) as b:
        assert b.describe()["forward_launch"] == "graph of per-step launches"
        Jb = b.forward()
        Eb = [b.energy(i) for i in range(len(cfgs))]
        Gb = b.backward()
    assert np.array_equal(Ja, Jb)
    for i in range(len(cfgs)):
        assert np.array_equal(Ea[i], Eb[i]), i
    assert rel(Ga, Gb) <= 1e-6
