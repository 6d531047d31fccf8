"""The reverse-mode rule on the GPU, through the host mirror (build_wavesim,
swforward, swgradient) and libswgb300: for the constant-density, the
variable-density and the elastic simulations, chi equals the forward misfit,
the pullback equals the sign of the physics times swgradient's field, and the
torch adapter's dchi/dm matches the central difference of its own misfit
along a Gaussian perturbation (FP32 simulations: within 2 %)."""
import copy

import numpy as np
import pytest

import __graft_entry__

sw = __graft_entry__.load_package()
R = __import__(sw.__name__ + ".rrules", fromlist=["rrules"])
pytestmark = pytest.mark.gpu

FD_TOL = 0.02


def _rp():
    return sw.RunParameters(erroronPPW=False)


def _blob(shape, cx, cz, s=6.0):
    x = np.arange(shape[0])[:, None]
    z = np.arange(shape[1])[None, :]
    return np.exp(-((x - cx) ** 2 + (z - cz) ** 2) / (2 * s * s))


def _fd_check(chi, matprop, key, attr, dv, eps):
    torch = pytest.importorskip("torch")
    base = np.asarray(getattr(matprop, attr), dtype=np.float64)
    t = torch.tensor(base, requires_grad=True)
    y = chi(**{key: t})
    y.backward()
    an = float(np.sum(t.grad.numpy() * dv))
    ms = [float(chi(**{key: torch.tensor(base + s * eps * dv)})) for s in (1, -1)]
    fd = (ms[0] - ms[1]) / (2 * eps)
    print(f"{key}: <dchi/dm, dv> = {an:.6e}, central difference = {fd:.6e}")
    assert abs(fd) > 0 and abs(an - fd) <= FD_TOL * abs(fd), key


def _check_rule(params, matprop, shots, misfit, gradparams, sign):
    chi, pb = R.rrule_swmisfit(params, matprop, shots, misfit, runparams=_rp(), gradparams=gradparams)
    ref = sw.swmisfit(params, matprop, shots, misfit, runparams=_rp())
    assert chi > 0 and abs(chi - ref) <= 1e-6 * ref
    g = sw.swgradient(params, matprop, shots, misfit, runparams=_rp(), gradparams=gradparams)
    tang = pb(1.0)
    for k, v in g.items():
        np.testing.assert_allclose(tang[k], sign * v, rtol=1e-12, atol=0)


def test_rrule_constant_density():
    from cases import ricker, smooth_model, stable_dt
    n, h, nt, f0 = (90, 80), (5.0, 5.0), 500, 15.0
    vp = smooth_model(n, 1800.0, 3000.0, seed=3)
    dt = stable_dt(vp, h)
    params = sw.InputParametersAcoustic(nt, dt, n, h, sw.CPMLBoundaryConditionParameters(halo=10, rcoef=1e-4,
                                                                                         freeboundtop=False))
    tf = ricker(np.arange(nt) * dt, 1.2 / f0, f0).reshape(nt, 1)
    rec = np.array([[x, 120.0] for x in np.linspace(80, 360, 9)])
    shots = [sw.ScalarShot(srcs=sw.ScalarSources([[200.0, 200.0]], tf, f0), recs=sw.ScalarReceivers(rec, nt))]
    sw.swforward(params, sw.VpAcousticCDMaterialProperties(np.asfortranarray(vp * 1.03)), shots, runparams=_rp())
    misfit = [sw.L2Misfit(observed=shots[0].recs.seismograms.copy())]
    matprop = sw.VpAcousticCDMaterialProperties(vp)
    gp = sw.GradParameters(check_freq=7)
    _check_rule(params, matprop, shots, misfit, gp, -1.0)
    ws = sw.build_wavesim(params, matprop, runparams=_rp(), gradparams=gp, gradient=True)
    chi = R.misfit_function(ws, matprop, shots, misfit)
    _fd_check(chi, matprop, "vp", "vp", _blob(n, 60, 30), 2.0)


def test_rrule_variable_density():
    from vd_cases import small_case
    case = small_case(nt=500, nx=90, nz=80, halo=10)
    shot = case.shots[0]
    nx, nz = case.vp.shape
    params = sw.InputParametersAcoustic(shot.nt, case.dt, (nx, nz), (case.h, case.h),
                                        sw.CPMLBoundaryConditionParameters(halo=case.halo, rcoef=case.rcoef,
                                                                           freeboundtop=False))
    shots = [sw.ScalarShot(srcs=sw.ScalarSources(shot.src, shot.tf, shot.f0),
                           recs=sw.ScalarReceivers(shot.rec, shot.nt))]
    sw.swforward(params, sw.VpRhoAcousticVDMaterialProperties(np.asfortranarray(case.vp * 1.03),
                                                              np.asfortranarray(case.rho * 0.97)), shots,
                 runparams=_rp())
    misfit = [sw.L2Misfit(observed=shots[0].recs.seismograms.copy())]
    matprop = sw.VpRhoAcousticVDMaterialProperties(case.vp, case.rho)
    gp = sw.GradParameters(check_freq=7)
    _check_rule(params, matprop, shots, misfit, gp, -1.0)
    # a wavesim built without compute_misfit: chi is summed from the recorded seismograms
    ws = sw.build_wavesim(params, matprop, runparams=_rp(), gradparams=gp, gradient=True)
    chi_ws, _ = R.rrule_swmisfit(ws, matprop, shots, misfit)
    chi_ref, _ = R.rrule_swmisfit(params, matprop, shots, misfit, runparams=_rp(), gradparams=gp)
    assert abs(chi_ws - chi_ref) <= 1e-6 * chi_ref
    chi = R.misfit_function(ws, matprop, shots, misfit)
    _fd_check(chi, matprop, "vp", "vp", _blob((nx, nz), 60, 30), 2.0)
    _fd_check(chi, matprop, "rho", "rho", _blob((nx, nz), 40, 55), 2.0)


def test_rrule_elastic():
    import elastic_cases as ec
    case = ec.small_case("mt", nt=400, nx=90, nz=80, halo=10)
    shot = case.shots[0]
    E = ec.E
    params = E.InputParametersElastic(shot.nt, case.dt, (case.nx, case.nz), (case.h, case.h),
                                      sw.CPMLBoundaryConditionParameters(halo=case.halo, rcoef=case.rcoef,
                                                                         freeboundtop=False))
    tf = ec.ricker(shot.nt, case.dt, shot.f0).reshape(-1, 1)

    def shots_():
        return [E.MomentTensorShot(srcs=E.MomentTensorSources(shot.src, tf, [E.MomentTensor2D(1.0, 1.0, 0.0)],
                                                              shot.f0),
                                   recs=E.VectorReceivers(shot.rec, shot.nt))]

    obs_shots = shots_()
    sw.swforward(params, E.ElasticIsoMaterialProperties(case.lam * 1.05, case.mu * 0.97, case.rho * 0.98),
                 obs_shots, runparams=_rp())
    misfit = [sw.L2Misfit(observed=obs_shots[0].recs.seismograms.copy())]
    shots = shots_()
    matprop = E.ElasticIsoMaterialProperties(case.lam, case.mu, case.rho)
    gp = sw.GradParameters(check_freq=7)
    _check_rule(params, matprop, shots, misfit, gp, 1.0)
    ws = sw.build_wavesim(params, copy.deepcopy(matprop), runparams=_rp(), gradparams=gp, gradient=True)
    chi = R.misfit_function(ws, matprop, shots, misfit)
    dv = _blob((case.nx, case.nz), 40, 55)
    for key, attr in (("lambda", "λ"), ("mu", "μ"), ("rho", "ρ")):
        _fd_check(chi, matprop, key, attr, dv, 1e-2 * float(np.mean(getattr(matprop, attr))))
