"""GPU parity of the variable-density acoustic 2D path against the FP64 CPU oracle.

Every test calls libswgb300 through its C ABI (tests/vd_cases.py: GpuVD)
with the inputs the oracle gets.  Tolerances: traces within 1e-5 relative
L2, misfit within 1e-6 and each gradient (vp, rho) within 1e-5 of the FP64
restatement.
"""
import numpy as np
import pytest

from vd_cases import GpuVD, VDCase, VDShot, nearest, oracle_forward, oracle_gradient, rel_l2, ricker, small_case, sw

pytestmark = pytest.mark.gpu

TRACE_TOL = 1e-5
MISFIT_TOL = 1e-6
GRAD_TOL = 1e-5


@pytest.fixture(scope="module")
def ctx():
    c = sw._lib.Context(0)
    yield c
    c.close()


def _observed(case, shot, scale=1.10):
    """Observed data from the oracle on a perturbed model, rounded to FP32 (the
    precision the library takes them in), so both sides see the same data.  The
    perturbation keeps the residuals well above the FP32 rounding of the
    traces, which the misfit (a difference of nearby numbers) would amplify."""
    pert = VDCase(case.vp * scale, case.rho * (2.0 - scale), case.h, case.dt, case.halo, freetop=case.freetop,
                  interp=case.interp, shots=[shot])
    return oracle_forward(pert, shot).astype(np.float32).astype(np.float64)


@pytest.mark.parametrize("freetop,interp,halo,nsrc", [(False, 0, 20, 1), (True, 0, 20, 1), (False, 1, 20, 2),
                                                       (True, 1, 12, 3), (False, 0, 0, 1), (False, 0, 1, 1)])
def test_vd_forward_matches_oracle(ctx, freetop, interp, halo, nsrc):
    case = small_case(nt=600, freetop=freetop, interp=interp, halo=halo, nsrc=nsrc)
    shot = case.shots[0]
    ref = oracle_forward(case, shot)
    run = GpuVD(ctx, case)
    tr = run.forward([shot])[0]
    run.close()
    err = rel_l2(tr, ref)
    print(f"VD forward freetop={freetop} interp={interp} halo={halo} nsrc={nsrc}: rel L2 {err:.2e}")
    assert np.abs(ref).max() > 0
    assert err < TRACE_TOL


def test_vd_forward_edge_sources_and_shared_points(ctx):
    """Sources on boundary nodes (never updated: they accumulate their source),
    two sources and two receivers on one node, receivers on the edges."""
    case = small_case(nt=300, nx=70, nz=60, halo=8)
    h = case.h
    ex, ez = (case.vp.shape[0] - 1) * h, (case.vp.shape[1] - 1) * h
    src = np.array([[0.0, 0.5 * ez], [0.5 * ex, 0.5 * ez], [0.5 * ex + 1.0, 0.5 * ez - 1.0], [ex, ez]])
    rec = np.array([[0.0, 0.5 * ez], [0.25 * ex, 0.3 * ez], [0.25 * ex, 0.3 * ez], [ex, 0.0], [0.6 * ex, ez]])
    t = np.arange(300) * case.dt
    tf = np.stack([ricker(t, 0.08 + 0.01 * k, 15.0) for k in range(4)], 1)
    shot = VDShot(src, rec, tf, 15.0)
    ref = oracle_forward(case, shot)
    run = GpuVD(ctx, case)
    tr = run.forward([shot])[0]
    run.close()
    assert rel_l2(tr, ref) < TRACE_TOL


def test_vd_batched_equals_single(ctx):
    case = small_case(nt=300)
    base = case.shots[0]
    t = np.arange(300) * case.dt
    shots = [VDShot(base.src + [[25.0 * k, 5.0 * k]], base.rec[: 5 + k],
                    ricker(t[: 300 - 40 * k], 0.08, 15.0).reshape(-1, 1), 15.0) for k in range(3)]
    run = GpuVD(ctx, case)
    batched = run.forward(shots)
    singles = [run.forward([s])[0] for s in shots]
    run.close()
    for a, b in zip(batched, singles):
        assert np.array_equal(a, b)


@pytest.mark.parametrize("freetop,interp,K", [(False, 0, 1), (False, 0, 23), (True, 1, 17), (False, 1, 40),
                                               (True, 0, 64)])
def test_vd_gradient_matches_oracle(ctx, freetop, interp, K):
    case = small_case(nt=400, freetop=freetop, interp=interp)
    shot = case.shots[0]
    obs = _observed(case, shot)
    gref, mref, tref = oracle_gradient(case, shot, obs, check_freq=K)
    run = GpuVD(ctx, case, gradient=True, check_freq=K)
    g, m, tr = run.gradient([shot], [obs])
    run.close()
    errs = {k: rel_l2(g[k], gref[k]) for k in g}
    print(f"VD gradient freetop={freetop} interp={interp} K={K}: traces {rel_l2(tr[0], tref):.2e} "
          f"misfit {abs(m - mref) / abs(mref):.2e} " + " ".join(f"{k} {v:.2e}" for k, v in errs.items()))
    assert rel_l2(tr[0], tref) < TRACE_TOL
    assert abs(m - mref) <= MISFIT_TOL * abs(mref)
    for k, v in errs.items():
        assert np.abs(gref[k]).max() > 0
        assert v < GRAD_TOL, k


def test_vd_gradient_windows_invcov_mute(ctx):
    case = small_case(nt=360)
    shot = case.shots[0]
    obs = _observed(case, shot, 1.12)
    ic = np.linspace(0.5, 1.5, shot.nt)
    win = [(20, 150), (200, 330)]
    gref, mref, _ = oracle_gradient(case, shot, obs, check_freq=19, invcov=ic, windows=win, mute_src=6, mute_rec=3)
    run = GpuVD(ctx, case, gradient=True, check_freq=19, mute_src=6, mute_rec=3)
    g, m, _ = run.gradient([shot], [obs], invcov=[ic], windows=[win])
    run.close()
    assert abs(m - mref) <= MISFIT_TOL * abs(mref)
    for k in g:
        assert rel_l2(g[k], gref[k]) < GRAD_TOL, k


def test_vd_gradient_shot_sum(ctx):
    """Three shots with different record lengths in one call = the sum of the oracle's per-shot gradients."""
    case = small_case(nt=330)
    base = case.shots[0]
    shots = []
    for k in range(3):
        nt = 330 - 35 * k
        t = np.arange(nt) * case.dt
        shots.append(VDShot(base.src + [[30.0 * k - 30.0, 4.0 * k]], base.rec[k:],
                            ricker(t, 0.07, 15.0).reshape(-1, 1), 15.0))
    obs = [_observed(case, s) for s in shots]
    run = GpuVD(ctx, case, gradient=True, check_freq=25)
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


def test_vd_gradient_dense_invcov(ctx):
    case = small_case(nt=300)
    shot = case.shots[0]
    obs = _observed(case, shot)
    i = np.arange(shot.nt)
    ic = np.linalg.inv(np.exp(-np.abs(i[:, None] - i[None, :]) / 3.0) + 0.1 * np.eye(shot.nt))
    gref, mref, _ = oracle_gradient(case, shot, obs, check_freq=20, invcov=ic)
    run = GpuVD(ctx, case, gradient=True, check_freq=20)
    g, m, _ = run.gradient([shot], [obs], invcov=[ic])
    run.close()
    assert abs(m - mref) <= MISFIT_TOL * abs(mref)
    for k in g:
        assert rel_l2(g[k], gref[k]) < GRAD_TOL, k


def test_vd_snapshots_match_oracle(ctx):
    case = small_case(nt=240, nx=80, nz=70, halo=10)
    shot = case.shots[0]
    tref, sref = oracle_forward(case, shot, snapevery=60)
    run = GpuVD(ctx, case)
    tr, snaps = run.forward_snapshots([shot], 60)
    run.close()
    assert rel_l2(tr[0], tref) < TRACE_TOL
    assert len(snaps[0]) == len(sref) == 4
    for a, b in zip(snaps[0], sref):
        for x, y in zip(a, b):
            assert rel_l2(x, y) < TRACE_TOL


def test_vd_mirror_api_gradient(ctx):
    """swgradient through the host mirror (VpRhoAcousticVDMaterialProperties) == the oracle."""
    case = small_case(nt=300, nx=90, nz=80, halo=10)
    shot = case.shots[0]
    obs = _observed(case, shot)
    gref, mref, _ = oracle_gradient(case, shot, obs, check_freq=15)
    nx, nz = case.vp.shape
    params = sw.InputParametersAcoustic(shot.nt, case.dt, (nx, nz), (case.h, case.h),
                                        sw.CPMLBoundaryConditionParameters(halo=case.halo, rcoef=case.rcoef,
                                                                           freeboundtop=False))
    mp = sw.VpRhoAcousticVDMaterialProperties(case.vp, case.rho)
    shots = [sw.ScalarShot(srcs=sw.ScalarSources(shot.src, shot.tf, shot.f0),
                           recs=sw.ScalarReceivers(shot.rec, shot.nt))]
    misfit = [sw.L2Misfit(observed=obs)]
    rp = sw.RunParameters(erroronPPW=False)
    g, m = sw.swgradient(params, mp, shots, misfit, runparams=rp,
                         gradparams=sw.GradParameters(check_freq=15, compute_misfit=True))
    assert abs(m - mref) <= MISFIT_TOL * abs(mref)
    for k in ("vp", "rho"):
        assert rel_l2(g[k], gref[k]) < GRAD_TOL, k
