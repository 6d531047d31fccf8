"""The oracle against the committed golden fixtures (tests/golden/*.npz, made
by tests/golden/make_golden.py): re-run on the stored inputs it reproduces
its stored FP64 traces, misfit and gradients to 1e-10 (compiler contraction
and thread count change only the last bits), so a change to the oracle that
alters results does not pass unnoticed."""
import numpy as np

import golden_cases as G
from cases import oracle_gradient, rel_l2

TOL = 1e-10


def test_golden_acoustic_cd2d(sw, oracle):
    case, shot, K, exp = G.acoustic_cd2d()
    g, m, tr = oracle_gradient(oracle, sw, case, shot, check_freq=K)
    assert rel_l2(tr, exp["traces"]) < TOL
    assert abs(m - exp["misfit"]) <= TOL * exp["misfit"]
    assert rel_l2(g, exp["grad"]) < TOL


def test_golden_acoustic_vd2d():
    from vd_cases import oracle_gradient as vd_gradient
    case, shot, obs, K, exp = G.acoustic_vd2d()
    g, m, tr = vd_gradient(case, shot, obs, check_freq=K)
    assert rel_l2(tr, exp["traces"]) < TOL
    assert abs(m - exp["misfit"]) <= TOL * exp["misfit"]
    for k in ("vp", "rho"):
        assert rel_l2(g[k], exp[k]) < TOL, k


def test_golden_elastic2d():
    from elastic_cases import oracle_gradient as el_gradient
    case, shot, obs, K, exp = G.elastic2d()
    g, m, tr = el_gradient(case, shot, obs, check_freq=K)
    assert rel_l2(tr, exp["traces"]) < TOL
    assert abs(m - exp["misfit"]) <= TOL * exp["misfit"]
    for k in ("rho", "lambda", "mu"):
        assert rel_l2(g[k], exp[k]) < TOL, k


def test_golden_fixtures_are_nontrivial():
    for load in (G.acoustic_cd2d,):
        case, shot, _, exp = load()
        assert np.abs(exp["traces"]).max() > 0 and exp["misfit"] > 0 and np.abs(exp["grad"]).max() > 0
    for load, keys in ((G.acoustic_vd2d, ("vp", "rho")), (G.elastic2d, ("rho", "lambda", "mu"))):
        case, shot, obs, _, exp = load()
        assert exp["misfit"] > 0 and all(np.abs(exp[k]).max() > 0 for k in keys)
