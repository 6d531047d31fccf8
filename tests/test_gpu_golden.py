"""libswgb300 (C ABI) against the committed golden fixtures
(tests/golden/*.npz): the oracle's FP64 traces, misfit and gradients of
three seeded cases (constant density with a free top, variable density with
harmonic 1/rho averaging, elastic moment tensor with a free top), compared
without running the oracle.  Bars: traces 1e-5, misfit 1e-6, gradients 1e-5."""
import pytest

import golden_cases as G
from cases import GpuRun, rel_l2

pytestmark = pytest.mark.gpu

TRACE_TOL, MISFIT_TOL, GRAD_TOL = 1e-5, 1e-6, 1e-5


def test_gpu_golden_acoustic_cd2d(sw):
    case, shot, K, exp = G.acoustic_cd2d()
    run = GpuRun(sw, case, gradient=True, check_freq=K)
    g, m, tr = run.gradient([shot])
    run.close()
    assert rel_l2(tr[0], exp["traces"]) < TRACE_TOL
    assert abs(m - exp["misfit"]) <= MISFIT_TOL * exp["misfit"]
    assert rel_l2(g, exp["grad"]) < GRAD_TOL


def test_gpu_golden_acoustic_vd2d(sw):
    from vd_cases import GpuVD
    case, shot, obs, K, exp = G.acoustic_vd2d()
    ctx = sw._lib.Context(0)
    run = GpuVD(ctx, case, gradient=True, check_freq=K)
    g, m, tr = run.gradient([shot], [obs])
    run.close()
    ctx.close()
    assert rel_l2(tr[0], exp["traces"]) < TRACE_TOL
    assert abs(m - exp["misfit"]) <= MISFIT_TOL * exp["misfit"]
    for k in ("vp", "rho"):
        assert rel_l2(g[k], exp[k]) < GRAD_TOL, k


def test_gpu_golden_elastic2d(sw):
    from elastic_cases import GpuElastic
    case, shot, obs, K, exp = G.elastic2d()
    ctx = sw._lib.Context(0)
    run = GpuElastic(ctx, case, gradient=True, check_freq=K)
    g, m, tr = run.gradient([shot], [obs])
    run.close()
    ctx.close()
    assert rel_l2(tr[0], exp["traces"]) < TRACE_TOL
    assert abs(m - exp["misfit"]) <= MISFIT_TOL * exp["misfit"]
    for k in ("rho", "lambda", "mu"):
        assert rel_l2(g[k], exp[k]) < GRAD_TOL, k
