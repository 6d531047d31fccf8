"""GPU parity of the elastic 2D (P-SV) path against the FP64 CPU oracle.

Every test calls libswgb300 through its C ABI (tests/elastic_cases.py:
GpuElastic) with the inputs the oracle gets.  Tolerances: traces within 1e-5
relative L2, misfit within 1e-6 and each gradient (rho, lambda, mu) within
1e-5 of the FP64 restatement.
"""
import numpy as np
import pytest

from elastic_cases import (ElCase, ElShot, GpuElastic, homogeneous, oracle_forward, oracle_gradient, rel_l2,
                           small_case, stable_dt, sw)

pytestmark = pytest.mark.gpu

TRACE_TOL = 1e-5
MISFIT_TOL = 1e-6
GRAD_TOL = 1e-5


@pytest.fixture(scope="module")
def ctx():
    c = sw._lib.Context(0)
    yield c
    c.close()


def _observed(case, shot, scale=1.3):
    """Observed data from the oracle on a perturbed model, rounded to FP32 (the
    precision the library takes them in), so both sides see the same data.  The
    perturbation keeps the residuals well above the FP32 rounding of the
    traces, which the misfit (a difference of nearby numbers) would amplify."""
    pert = ElCase(case.nx, case.nz, case.h, case.dt, case.halo, case.lam * scale, case.mu * 0.88, case.rho * 0.92,
                  [shot], freetop=case.freetop, sinc=case.sinc, interp_rho=case.interp_rho, interp_mu=case.interp_mu)
    return oracle_forward(pert, shot).astype(np.float32).astype(np.float64)


@pytest.mark.parametrize("kind,freetop,sinc,interp", [
    ("mt", False, True, (0, 0)), ("mt", True, True, (0, 0)), ("force", False, True, (0, 0)),
    ("force", True, True, (1, 1)), ("mt", False, False, (0, 0)), ("mt", True, False, (1, 0))])
def test_elastic_forward_matches_oracle(ctx, kind, freetop, sinc, interp):
    case = small_case(kind, freetop=freetop, sinc=sinc, interp=interp, nt=500)
    shot = case.shots[0]
    ref = oracle_forward(case, shot)
    run = GpuElastic(ctx, case)
    tr = run.forward([shot])[0]
    run.close()
    err = rel_l2(tr, ref)
    print(f"elastic forward {kind} freetop={freetop} sinc={sinc} interp={interp}: rel L2 {err:.2e}")
    assert np.abs(ref).max() > 0
    assert err < TRACE_TOL


def test_elastic_forward_small_halo(ctx):
    for halo in (0, 1, 4):
        case = small_case("mt", nt=300, halo=halo, nx=60, nz=50)
        shot = case.shots[0]
        ref = oracle_forward(case, shot)
        run = GpuElastic(ctx, case)
        tr = run.forward([shot])[0]
        run.close()
        assert rel_l2(tr, ref) < TRACE_TOL, halo


def test_elastic_batched_equals_single(ctx):
    case = small_case("mt", nt=300)
    base = case.shots[0]
    shots = [ElShot("mt", base.src + [[30.0 * k, 5.0 * k]], base.rec[: 5 + k], 300 - 40 * k) for k in range(3)]
    run = GpuElastic(ctx, case)
    batched = run.forward(shots)
    singles = [run.forward([s])[0] for s in shots]
    run.close()
    for a, b in zip(batched, singles):
        assert np.array_equal(a, b)


@pytest.mark.parametrize("kind,freetop,K", [("mt", False, 1), ("mt", False, 23), ("force", True, 17),
                                             ("mt", True, 40)])
def test_elastic_gradient_matches_oracle(ctx, kind, freetop, K):
    case = small_case(kind, freetop=freetop, nt=400)
    shot = case.shots[0]
    obs = _observed(case, shot)
    gref, mref, tref = oracle_gradient(case, shot, obs, check_freq=K)
    run = GpuElastic(ctx, case, gradient=True, check_freq=K)
    g, m, tr = run.gradient([shot], [obs])
    run.close()
    errs = {k: rel_l2(g[k], gref[k]) for k in g}
    print(f"elastic gradient {kind} freetop={freetop} K={K}: traces {rel_l2(tr[0], tref):.2e} "
          f"misfit {abs(m - mref) / abs(mref):.2e} " + " ".join(f"{k} {v:.2e}" for k, v in errs.items()))
    assert rel_l2(tr[0], tref) < TRACE_TOL
    assert abs(m - mref) <= MISFIT_TOL * abs(mref)
    for k, v in errs.items():
        assert np.abs(gref[k]).max() > 0
        assert v < GRAD_TOL, k


def test_elastic_gradient_windows_invcov_mute(ctx):
    case = small_case("force", nt=360)
    shot = case.shots[0]
    obs = _observed(case, shot, 1.35)
    ic = np.linspace(0.5, 1.5, shot.nt)
    win = [(20, 150), (200, 330)]
    gref, mref, _ = oracle_gradient(case, shot, obs, check_freq=19, invcov=ic, windows=win, mute_src=6, mute_rec=3)
    run = GpuElastic(ctx, case, gradient=True, check_freq=19, mute_src=6, mute_rec=3)
    g, m, _ = run.gradient([shot], [obs], invcov=[ic], windows=[win])
    run.close()
    assert abs(m - mref) <= MISFIT_TOL * abs(mref)
    for k in g:
        assert rel_l2(g[k], gref[k]) < GRAD_TOL, k


def test_elastic_gradient_shot_sum(ctx):
    """Three shots with different record lengths in one call = the sum of the oracle's per-shot gradients."""
    case = small_case("mt", nt=330)
    base = case.shots[0]
    shots = [ElShot("mt", base.src + [[40.0 * k - 40.0, 3.0 * k]], base.rec[k:], 330 - 30 * k) for k in range(3)]
    obs = [_observed(case, s) for s in shots]
    run = GpuElastic(ctx, case, gradient=True, check_freq=25)
    g, m, _ = run.gradient(shots, obs)
    run.close()
    gsum = {k: 0.0 for k in g}
    msum = 0.0
    for s, o in zip(shots, obs):
        gr, mr, _ = oracle_gradient(case, s, o, check_freq=25)
        msum += mr
        for k in g:
            gsum[k] = gsum[k] + gr[k]
    assert abs(m - msum) <= MISFIT_TOL * abs(msum)
    for k in g:
        assert rel_l2(g[k], gsum[k]) < GRAD_TOL, k


def test_elastic_rejects_boundary_stress_source(ctx):
    nx, nz, h = 60, 50, 5.0
    lam, mu, rho = homogeneous(nx, nz)
    dt = stable_dt(lam, mu, rho, h)
    shot = ElShot("mt", np.array([[0.0, 100.0]]), np.array([[100.0, 100.0]]), 50)
    case = ElCase(nx, nz, h, dt, 10, lam, mu, rho, [shot], sinc=False)
    run = GpuElastic(ctx, case)
    with pytest.raises(sw._lib.SwError) as ei:
        run.forward([shot])
    run.close()
    assert ei.value.code == sw._lib.SW_ERR_UNSUPPORTED


def test_elastic_gradient_dense_invcov(ctx):
    """Full inverse covariance applied per component (cuBLAS on the device)."""
    case = small_case("mt", nt=300)
    shot = case.shots[0]
    obs = _observed(case, shot)
    i = np.arange(shot.nt)
    ic = np.linalg.inv(np.exp(-np.abs(i[:, None] - i[None, :]) / 3.0) + 0.1 * np.eye(shot.nt))
    gref, mref, _ = oracle_gradient(case, shot, obs, check_freq=20, invcov=ic)
    run = GpuElastic(ctx, case, gradient=True, check_freq=20)
    g, m, _ = run.gradient([shot], [obs], invcov=[ic])
    run.close()
    print(f"elastic dense invcov: misfit {abs(m - mref) / abs(mref):.2e} "
          + " ".join(f"{k} {rel_l2(g[k], gref[k]):.2e}" for k in g))
    assert abs(m - mref) <= MISFIT_TOL * abs(mref)
    for k in g:
        assert rel_l2(g[k], gref[k]) < GRAD_TOL, k


@pytest.mark.parametrize("kind,freetop", [("mt", True), ("force", False)])
def test_elastic_split_displacement_matches(ctx, kind, freetop):
    """The displacement update as two launches (ux, then uz; the default) runs
    the same per-point arithmetic as the single launch (sw_elastic_set_tuning
    + 128): the traces and gradients agree with it and with the oracle."""
    case = small_case(kind, freetop=freetop, nt=360)
    shot = case.shots[0]
    obs = _observed(case, shot)
    out = {}
    for tz in (8, 136):
        run = GpuElastic(ctx, case, gradient=True, check_freq=19)
        run.ctx.check(run.ctx.lib.sw_elastic_set_tuning(run.h, tz), "sw_elastic_set_tuning")
        out[tz] = run.gradient([shot], [obs])
        run.close()
    g0, m0, t0 = out[8]
    g1, m1, t1 = out[136]
    assert rel_l2(t1[0], t0[0]) < 1e-6 and abs(m1 - m0) <= 1e-6 * abs(m0)
    for k in g0:
        assert rel_l2(g1[k], g0[k]) < 1e-6, k
    gref, mref, tref = oracle_gradient(case, shot, obs, check_freq=19)
    assert rel_l2(t1[0], tref) < TRACE_TOL
    for k in g1:
        assert rel_l2(g1[k], gref[k]) < GRAD_TOL, k
