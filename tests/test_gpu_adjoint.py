"""GPU adjoint (nufi_backward): dJ/d(alpha, k, u_b, sigma_b) of
J = 2 dt sum_n W_n against the oracle's FP64 forward-mode derivative and
against central finite differences (h = 1e-6) of the GPU FP64 forward.

Tolerances: 1e-8 of max |dJ| against forward mode (both FP64; the adjoint
recomputes the characteristics by inverting the substeps, which rounds
differently), 1e-5 relative per component against finite differences (the
gradient's accuracy target; the difference quotient itself is good to
~1e-7).
"""
import numpy as np
import pytest

from numericalflowiteration_gb300.config import bump_on_tail_1d, landau_1d, landau_2d, two_stream_1d

pytestmark = pytest.mark.gpu

CASES = {
    "landau_32x64_n40": landau_1d(Nx=32, Nv=64, Nt=40),
    "two_stream_32x128_n60": two_stream_1d(Nx=32, Nv=128, Nt=60),
    "bump_on_tail_64x128_n80": bump_on_tail_1d(Nx=64, Nv=128, Nt=80),
    "landau_order6_32x64_n30": landau_1d(Nx=32, Nv=64, Nt=30, order=6),
}


@pytest.fixture(scope="module")
def nufi():
    import numericalflowiteration_gb300 as m
    from numericalflowiteration_gb300 import build
    build.build()
    m.load()
    return m


def _nparams(cfg):
    return 4 if cfg.f0 == "bump_on_tail" else 2


@pytest.mark.parametrize("name", sorted(CASES))
def test_adjoint_matches_forward_mode(nufi, oracle_mod, name):
    cfg = CASES[name]
    J_ref, dJ_ref = oracle_mod.objective_tangent(cfg)
    with nufi.Simulation(cfg) as sim:
        J = sim.forward()
        g = sim.backward()
    assert abs(J - J_ref) <= 1e-12 * abs(J_ref)
    k = _nparams(cfg)
    assert np.max(np.abs(g[:k] - dJ_ref[:k])) <= 1e-8 * np.max(np.abs(dJ_ref[:k])), (g, dJ_ref)
    assert np.all(g[k:] == 0)


@pytest.mark.parametrize("name", ["landau_32x64_n40", "bump_on_tail_64x128_n80"])
def test_adjoint_matches_central_differences(nufi, name):
    cfg = CASES[name]
    h = 1e-6
    with nufi.Simulation(cfg) as sim:
        sim.forward()
        g = sim.backward()
    for i in range(_nparams(cfg)):
        Js = []
        for sgn in (1, -1):
            pp = list(cfg.f0_params)
            pp[i] += sgn * h
            with nufi.Simulation(cfg.replace(f0_params=pp)) as s:
                Js.append(s.forward())
        fd = (Js[0] - Js[1]) / (2 * h)
        assert abs(g[i] - fd) <= 1e-5 * abs(fd), (i, g[i], fd)


def test_adjoint_repeat_and_partial_horizon(nufi, oracle_mod):
    """backward(n1) for n1 < Nt differentiates J up to n1; repeated calls
    agree to the last bits (FP64 atomics in the slab adjoints)."""
    cfg = CASES["landau_32x64_n40"]
    with nufi.Simulation(cfg) as sim:
        sim.forward()
        g1 = sim.backward(25)
        g2 = sim.backward(25)
        J25 = sim.objective(25)
    J_ref, dJ_ref = oracle_mod.objective_tangent(cfg, 25)
    assert abs(J25 - J_ref) <= 1e-12 * abs(J_ref)
    assert np.max(np.abs(g1 - g2)) <= 1e-13 * np.max(np.abs(g1))
    assert np.max(np.abs(g1[:2] - dJ_ref[:2])) <= 1e-8 * np.max(np.abs(dJ_ref[:2]))


def test_adjoint_errors(nufi):
    cfg = CASES["landau_32x64_n40"]
    with nufi.Simulation(cfg) as sim:
        with pytest.raises(IndexError):
            sim.backward()  # no forward yet
        with pytest.raises(IndexError):
            sim.objective()
        sim.forward(10)
        with pytest.raises(IndexError):
            sim.backward(11)
        sim.backward(10)
    with nufi.Simulation(landau_2d(Nx=8, Nv=8, Nt=4)) as sim:
        sim.forward()
        with pytest.raises(NotImplementedError):
            sim.backward()
