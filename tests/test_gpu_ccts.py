"""GPU parity of the device CCTS misfit (k_ccts) on the constant- and
variable-density acoustic gradients and on the elastic gradient (one trace
per receiver component), against the FP64 oracle's restatement of
CCTSMisfit.jl:17-80.  The per-trace time shifts are integers times dt, so
the misfit matches to FP64 rounding once every argmax agrees; the gradient is
held to the usual 1e-5."""
import numpy as np
import pytest

import __graft_entry__
from vd_cases import GpuVD, VDCase, oracle_forward as vd_forward, oracle_gradient as vd_gradient, rel_l2, small_case

sw = __graft_entry__.load_package()
pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def ctx():
    c = sw._lib.Context(0)
    yield c
    c.close()


def test_ccts_gradient_constant_density_matches_oracle():
    import oracle

    nx, nz, h = 140, 110, 5.0
    x = np.arange(nx)[:, None] * h
    z = np.arange(nz)[None, :] * h
    vp = np.asfortranarray(2000.0 + 800.0 * z / z.max() + 0.0 * x)
    nt = 700
    dt = 0.5 * h / (float(vp.max()) * np.sqrt(2))
    f0 = 15.0
    t = np.arange(nt) * dt
    tf = (1 - 2 * (np.pi * f0 * (t - 0.08)) ** 2) * np.exp(-(np.pi * f0 * (t - 0.08)) ** 2)
    src = np.array([[0.5 * (nx - 1) * h + 1.0, 0.4 * (nz - 1) * h]])
    rec = np.stack([np.linspace(0.2, 0.8, 12) * (nx - 1) * h, np.full(12, 0.25 * (nz - 1) * h)], 1)
    halo = 15
    si, ri = sw.nearest_grid_points(src, (h, h)), sw.nearest_grid_points(rec, (h, h))
    cp = oracle.cpml_blocks(vp, (h, h), dt, halo, 1e-4, f0, False)

    def scaled(v):
        return np.asarray(sw.scale_srctf(tf.reshape(nt, 1), si, v, (h, h), dt), dtype=np.float64)

    obs = oracle.acoustic_forward(vp * 1.06, (h, h), dt, halo, cp, scaled(vp), si, ri)
    obs = obs.astype(np.float32).astype(np.float64)
    gref, mref, _ = oracle.acoustic_gradient(vp, (h, h), dt, halo, cp, scaled(vp), si, ri, obs, check_freq=20,
                                             ccts_dt=dt)
    params = sw.InputParametersAcoustic(nt, dt, (nx, nz), (h, h),
                                        sw.CPMLBoundaryConditionParameters(halo=halo, rcoef=1e-4, freeboundtop=False))
    shots = [sw.ScalarShot(srcs=sw.ScalarSources(src, tf.reshape(nt, 1), f0), recs=sw.ScalarReceivers(rec, nt))]
    g, m = sw.swgradient(params, sw.VpAcousticCDMaterialProperties(vp), shots, [sw.CCTSMisfit(dt, observed=obs)],
                         runparams=sw.RunParameters(erroronPPW=False),
                         gradparams=sw.GradParameters(check_freq=20, compute_misfit=True))
    err = rel_l2(g["vp"], gref)
    print(f"CCTS CD: misfit {m:.6e} vs {mref:.6e}, gradient rel L2 {err:.2e}")
    assert mref > 0 and m == pytest.approx(mref, rel=1e-9)
    assert err < 1e-5


def test_ccts_gradient_variable_density_matches_oracle(ctx):
    case = small_case(nt=500)
    shot = case.shots[0]
    pert = VDCase(case.vp * 1.08, case.rho, case.h, case.dt, case.halo, shots=[shot])
    obs = vd_forward(pert, shot).astype(np.float32).astype(np.float64)
    gref, mref, _ = vd_gradient(case, shot, obs, check_freq=20, ccts_dt=case.dt)
    run = GpuVD(ctx, case, gradient=True, check_freq=20)
    g, m, _ = run.gradient([shot], [obs], ccts_dt=case.dt)
    run.close()
    errs = {k: rel_l2(g[k], gref[k]) for k in g}
    print(f"CCTS VD: misfit {m:.6e} vs {mref:.6e}, " + " ".join(f"{k} {v:.2e}" for k, v in errs.items()))
    assert mref > 0 and m == pytest.approx(mref, rel=1e-9)
    for k, v in errs.items():
        assert v < 1e-5, k


def test_ccts_gradient_elastic_matches_oracle(ctx):
    """CCTSMisfit{T,3} on vector receivers (CCTSMisfit.jl:30-44, :63-80): a
    time shift per receiver and component, summed into the misfit; the
    adjoint sources carry the elastic path's power-of-two scale."""
    import elastic_cases as EC
    case = EC.small_case(nt=500, seed=3)
    shot = case.shots[0]
    pert = EC.ElCase(case.nx, case.nz, case.h, case.dt, case.halo, case.lam * 1.15, case.mu * 0.9, case.rho,
                     [shot], freetop=case.freetop, sinc=case.sinc)
    obs = EC.oracle_forward(pert, shot).astype(np.float32).astype(np.float64)
    gref, mref, _ = EC.oracle_gradient(case, shot, obs, check_freq=20, ccts_dt=case.dt)
    run = EC.GpuElastic(ctx, case, gradient=True, check_freq=20)
    g, m, _ = run.gradient([shot], [obs], ccts_dt=case.dt)
    run.close()
    errs = {k: rel_l2(g[k], gref[k]) for k in g}
    print(f"CCTS elastic: misfit {m:.6e} vs {mref:.6e}, " + " ".join(f"{k} {v:.2e}" for k, v in errs.items()))
    assert mref > 0 and m == pytest.approx(mref, rel=1e-9)
    for k, v in errs.items():
        assert v < 1e-5, k
