"""Parity at the sizes of the benchmark configurations, against the FP64
oracle where it finishes in seconds to a minute: the 201 x 201 forward, the
801 x 801 forward + L2 misfit + adjoint gradient with checkpoint period 50,
two shots of the 2001 x 801 batch (shortest and longest record) and one of
its variable-density twin, two elastic shots on the full 1200 x 600 grid
(records capped at 600 steps) and the 3D generator at 200^3; plus the whole
64-shot 2001 x 801 batch through properties that hold at any size."""
import numpy as np
import pytest

from cases import Case, GpuRun, Shot, oracle_forward, oracle_gradient, rel_l2

pytestmark = pytest.mark.gpu

TRACE_TOL = 1e-5     # traces, relative L2 against the FP64 oracle
MISFIT_TOL = 1e-6    # misfit, relative
GRAD_TOL = 1e-5      # gradient (FP32 checkpoints), relative L2


def _case(w):
    shots = [Shot(src_pos=s.src_pos, rec_pos=s.rec_pos, tf=np.asfortranarray(s.stf(w.dt)), f0=s.f0, nt=s.nt)
             for s in w.shots]
    return Case(vp=w.vp, h=w.h, dt=w.dt, halo=w.halo, freetop=w.freetop, shots=shots)


def test_acoustic2d_201_forward(sw, oracle):
    from seismicwaves_gb300 import configs
    case = _case(configs.acoustic2d_201())
    run = GpuRun(sw, case)
    tr = run.forward(case.shots)[0]
    run.close()
    assert rel_l2(tr, oracle_forward(oracle, sw, case, case.shots[0])) < TRACE_TOL


def test_acoustic2d_801_gradient(sw, oracle):
    from seismicwaves_gb300 import configs
    w = configs.acoustic2d_801()
    case = _case(w)
    shot = case.shots[0]
    obs_case = Case(vp=w.vp_observed, h=w.h, dt=w.dt, halo=w.halo, freetop=w.freetop)
    shot.observed = oracle_forward(oracle, sw, obs_case, shot)
    run = GpuRun(sw, case, gradient=True, check_freq=w.check_freq)
    g, msf, tr = run.gradient([shot])
    run.close()
    gref, mref, tref = oracle_gradient(oracle, sw, case, shot, check_freq=w.check_freq)
    errs = (rel_l2(tr[0], tref), abs(msf - mref) / mref, rel_l2(g, gref))
    print(f"acoustic2d_801: traces {errs[0]:.3e}  misfit {errs[1]:.3e}  gradient {errs[2]:.3e}")
    assert errs[0] < TRACE_TOL
    assert errs[1] < MISFIT_TOL
    assert errs[2] < GRAD_TOL


def _misfit_bound(trs, trefs, obs):
    """Relative misfit difference that the trace differences alone imply: with
    chi = |r|^2 / 2 and r = traces - observed, |chi - chi_ref| <= sum over
    shots of |r_ref| |d| + |d|^2 / 2, d = traces - traces_ref (exact, by
    Cauchy-Schwarz).  At full record lengths the FP32 traces differ from the
    FP64 ones by about 1e-6, which this quadratic form doubles or more; the
    misfit reduction itself must add nothing beyond it."""
    num = chi = 0.0
    for t, tref, o in zip(trs, trefs, obs):
        nr = float(np.linalg.norm(np.asarray(tref, np.float64) - o))
        nd = float(np.linalg.norm(np.asarray(t, np.float64) - tref))
        num += nr * nd + 0.5 * nd * nd
        chi += 0.5 * nr * nr
    return num / chi


def _shot(s, dt, nt=None):
    nt = nt or s.nt
    return Shot(src_pos=s.src_pos, rec_pos=s.rec_pos, tf=np.asfortranarray(s.stf(dt)[:nt]), f0=s.f0, nt=nt)


def _gpu_observed(sw, case, vp_obs, shots):
    run = GpuRun(sw, Case(vp=np.asfortranarray(vp_obs), h=case.h, dt=case.dt, halo=case.halo, freetop=case.freetop))
    obs = run.forward(shots)
    run.close()
    for s, o in zip(shots, obs):
        s.observed = np.asfortranarray(o, dtype=np.float64)


def _sample_shots(w, k=8, seed=2024):
    """k shots of the workload spanning its record lengths: the shortest, the
    longest and k-2 seeded picks among the rest."""
    order = sorted(range(len(w.shots)), key=lambda i: w.shots[i].nt)
    rng = np.random.default_rng(seed)
    mid = sorted(rng.choice(order[1:-1], size=k - 2, replace=False).tolist(), key=lambda i: w.shots[i].nt)
    return [order[0]] + mid + [order[-1]]


def test_acoustic2d_2001x801_batch_matches_oracle(sw, oracle):
    """The headline grid (2001 x 801, 20-point C-PML, K = 50) at full size: 8
    of its 64 shots (the shortest and longest records, nt 2002 and 3982, and 6
    seeded picks between), with their different receiver counts, in one
    batched gradient call against the sum of the oracle's per-shot FP64
    gradients (each shot with its own nt), and each shot alone against its
    own oracle gradient.  Observed data: the GPU forward of 1.05 vp, so that
    the misfit is a well-conditioned comparison."""
    from seismicwaves_gb300 import configs
    w = configs.acoustic2d_2001x801()
    sel = _sample_shots(w)
    shots = [_shot(w.shots[i], w.dt) for i in sel]
    case = Case(vp=w.vp, h=w.h, dt=w.dt, halo=w.halo, freetop=w.freetop)
    _gpu_observed(sw, case, w.vp * 1.05, shots)
    run = GpuRun(sw, case, gradient=True, check_freq=w.check_freq)
    g, msf, tr = run.gradient(shots)
    singles = [run.gradient([s])[0] for s in shots]
    run.close()
    gref, mref, trefs, gerrs = 0.0, 0.0, [], []
    for k, s in enumerate(shots):
        gk, mk, tk = oracle_gradient(oracle, sw, case, s, check_freq=w.check_freq)
        assert rel_l2(tr[k], tk) < TRACE_TOL, k
        gerrs.append(rel_l2(singles[k], gk))
        gref, mref = gref + gk, mref + mk
        trefs.append(tk)
    bound = _misfit_bound(tr, trefs, [s.observed for s in shots])
    errs = (abs(msf - mref) / mref, rel_l2(g, gref))
    # the compensated forward (sw_wavesim_set_precision 1) on the same batch
    hp = GpuRun(sw, case, gradient=True, check_freq=w.check_freq, precision=1)
    g_hp, msf_hp, tr_hp = hp.gradient(shots)
    hp.close()
    hp_errs = (abs(msf_hp - mref) / mref, rel_l2(g_hp, gref), max(rel_l2(a, b) for a, b in zip(tr_hp, trefs)))
    print(f"acoustic2d_2001x801, shots {sel} (nt {[s.nt for s in shots]}): FP32 traces "
          f"{[f'{rel_l2(a, b):.2e}' for a, b in zip(tr, trefs)]} misfit {errs[0]:.3e} (trace-implied bound "
          f"{bound:.3e})  batched gradient {errs[1]:.3e}  per-shot gradients {[f'{e:.2e}' for e in gerrs]}; "
          f"compensated: traces <= {hp_errs[2]:.2e} misfit {hp_errs[0]:.3e} gradient {hp_errs[1]:.3e}")
    assert errs[0] <= max(MISFIT_TOL, 1.1 * bound)  # FP32 state: about 2e-6 at these record lengths
    assert errs[1] < GRAD_TOL
    assert max(gerrs) < GRAD_TOL
    assert hp_errs[0] < MISFIT_TOL  # the misfit bar, met by the compensated forward
    assert hp_errs[1] < GRAD_TOL and hp_errs[2] < TRACE_TOL


def test_acoustic2d_2001x801_all_shots_consistency(sw):
    """All 64 shots of the headline workload at full size, through properties
    that hold at any size: the gradient call's misfit equals the misfit of a
    forward call's traces (summed on the host in FP64), and the 64-shot
    gradient equals the sum of two 32-shot calls (batch composition changes
    only the FP32 rounding of the correlation sums)."""
    from seismicwaves_gb300 import configs
    w = configs.acoustic2d_2001x801()
    shots = [_shot(s, w.dt) for s in w.shots]
    case = Case(vp=w.vp, h=w.h, dt=w.dt, halo=w.halo, freetop=w.freetop)
    _gpu_observed(sw, case, w.vp_observed, shots)
    run = GpuRun(sw, case, gradient=True, check_freq=w.check_freq)
    g, msf, _ = run.gradient(shots)
    fw = run.forward(shots)
    ga, ma, _ = run.gradient(shots[:32])
    gb, mb, _ = run.gradient(shots[32:])
    run.close()
    mfw = sum(0.5 * float(np.sum((t - s.observed) ** 2)) for t, s in zip(fw, shots))
    print(f"64 shots: misfit {msf:.6e} (forward {mfw:.6e}), split gradient rel diff {rel_l2(ga + gb, g):.2e}")
    assert msf > 0 and abs(msf - mfw) <= 1e-6 * mfw
    assert abs((ma + mb) - msf) <= 1e-9 * msf
    assert rel_l2(ga + gb, g) < 1e-5


def test_acoustic_vd2d_2001x801_shot_matches_oracle(sw, oracle):
    """The variable-density headline grid at full size: its shortest shot's vp
    and rho gradients against the FP64 oracle (observed: 1.05 vp, 0.97 rho)."""
    from seismicwaves_gb300 import configs
    from vd_cases import GpuVD, VDCase, VDShot, oracle_forward as vd_forward, oracle_gradient as vd_gradient
    w = configs.acoustic_vd2d_2001x801()
    s = min(w.shots, key=lambda s: s.nt)
    shot = VDShot(s.src_pos, s.rec_pos, s.stf(w.dt), s.f0)
    case = VDCase(w.vp, w.rho, w.h[0], w.dt, w.halo, shots=[shot])
    ctx = sw._lib.Context(0)
    obs_run = GpuVD(ctx, VDCase(np.asfortranarray(w.vp * 1.05), np.asfortranarray(w.rho * 0.97), w.h[0], w.dt,
                                w.halo, shots=[shot]))
    obs = obs_run.forward([shot])[0]
    obs_run.close()
    run = GpuVD(ctx, case, gradient=True, check_freq=w.check_freq)
    g, msf, tr = run.gradient([shot], [obs])
    run.close()
    hp = GpuVD(ctx, case, gradient=True, check_freq=w.check_freq, precision=1)  # the compensated forward
    g_hp, msf_hp, tr_hp = hp.gradient([shot], [obs])
    hp.close()
    ctx.close()
    gref, mref, tref = vd_gradient(case, shot, obs, check_freq=w.check_freq)
    errs = (rel_l2(tr[0], tref), abs(msf - mref) / mref, rel_l2(g["vp"], gref["vp"]), rel_l2(g["rho"], gref["rho"]))
    hp_errs = (rel_l2(tr_hp[0], tref), abs(msf_hp - mref) / mref, rel_l2(g_hp["vp"], gref["vp"]),
               rel_l2(g_hp["rho"], gref["rho"]))
    bound = _misfit_bound(tr, [tref], [obs])
    print(f"acoustic_vd2d_2001x801 (nt {shot.nt}): traces {errs[0]:.3e} misfit {errs[1]:.3e} (trace-implied "
          f"bound {bound:.3e}) vp {errs[2]:.3e} rho {errs[3]:.3e}; compensated: traces {hp_errs[0]:.3e} misfit "
          f"{hp_errs[1]:.3e} vp {hp_errs[2]:.3e} rho {hp_errs[3]:.3e}")
    assert errs[0] < TRACE_TOL and errs[1] <= max(MISFIT_TOL, 1.1 * bound)  # FP32 state: about 1.8e-6
    assert errs[2] < GRAD_TOL and errs[3] < GRAD_TOL
    assert hp_errs[0] < TRACE_TOL and hp_errs[1] < MISFIT_TOL  # the misfit bar, met by the compensated forward
    assert hp_errs[2] < GRAD_TOL and hp_errs[3] < GRAD_TOL


def test_elastic2d_1200x600_batch_matches_oracle(sw):
    """The elastic grid at full size (1200 x 600, 300 receivers per shot, sinc
    spreading, K = 50) with records capped at 600 steps: its first and last
    shots in one batched gradient call against the sum of the oracle's
    lambda, mu and rho gradients (observed: the GPU forward of lambda 1.3x,
    mu 0.88x, rho 0.92x)."""
    from seismicwaves_gb300 import configs
    from elastic_cases import ElCase, ElShot, GpuElastic, oracle_gradient as el_gradient
    w = configs.elastic2d_1200x600()
    nx, nz = w.lam.shape
    shots = [ElShot("mt", s.src_pos, s.rec_pos, 600, s.f0, momtens=[w.momtens]) for s in (w.shots[0], w.shots[-1])]
    case = ElCase(nx, nz, w.h[0], w.dt, w.halo, w.lam, w.mu, w.rho, shots)
    pert = ElCase(nx, nz, w.h[0], w.dt, w.halo, w.lam * 1.3, w.mu * 0.88, w.rho * 0.92, shots)
    ctx = sw._lib.Context(0)
    obs_run = GpuElastic(ctx, pert)
    obs = obs_run.forward(shots)
    obs_run.close()
    run = GpuElastic(ctx, case, gradient=True, check_freq=w.check_freq)
    g, msf, tr = run.gradient(shots, obs)
    run.close()
    ctx.close()
    gref, mref = {k: 0.0 for k in ("rho", "lambda", "mu")}, 0.0
    for k, s in enumerate(shots):
        gk, mk, tk = el_gradient(case, s, obs[k], check_freq=w.check_freq)
        assert rel_l2(tr[k], tk) < TRACE_TOL, k
        gref = {n: gref[n] + gk[n] for n in gref}
        mref += mk
    errs = {n: rel_l2(g[n], gref[n]) for n in gref}
    print(f"elastic2d_1200x600: misfit {abs(msf - mref) / mref:.3e} gradients {errs}")
    assert abs(msf - mref) / mref < MISFIT_TOL
    assert all(e < GRAD_TOL for e in errs.values())


def test_acoustic3d_generator_200_matches_oracle(sw, oracle):
    """The 3D workload's generator (smooth random velocity, surface source,
    receiver patch) at 200^3, the size the FP64 oracle finishes in seconds:
    one shot, 150 steps, K = 50.  FP32 recompute buffer against the 1e-5 bar;
    the FP16 buffer of the benchmark against 1e-3; the BF16 buffer reported
    and bounded at 5e-3 (its error relative to the gradient grows as the
    residual shrinks: 2.4e-3 here, with a 3 % velocity perturbation over 150
    steps); the compensated forward against the misfit bar."""
    from seismicwaves_gb300 import configs
    w = configs.acoustic3d_400(n=200, nshots_side=1, patch=10, nt=150)
    shots = [_shot(s, w.dt) for s in w.shots]
    case = Case(vp=w.vp, h=w.h, dt=w.dt, halo=w.halo, freetop=w.freetop)
    _gpu_observed(sw, case, w.vp_observed, shots)
    gref, mref, tref = oracle_gradient(oracle, sw, case, shots[0], check_freq=50)
    out = {}
    for bf16, prec in ((0, 0), (1, 0), (3, 0), (0, 1)):
        run = GpuRun(sw, case, gradient=True, check_freq=50, bf16=bf16, precision=prec)
        out[(bf16, prec)] = run.gradient(shots)
        run.close()
    g, msf, tr = out[(0, 0)]
    g_hp, msf_hp, tr_hp = out[(0, 1)]
    bound = _misfit_bound(tr, [tref], [shots[0].observed])
    errs = (rel_l2(tr[0], tref), abs(msf - mref) / mref, rel_l2(g, gref), rel_l2(out[(1, 0)][0], gref))
    hp_errs = (rel_l2(tr_hp[0], tref), abs(msf_hp - mref) / mref, rel_l2(g_hp, gref))
    e16 = rel_l2(out[(3, 0)][0], gref)
    print(f"acoustic3d 200^3: traces {errs[0]:.3e} misfit {errs[1]:.3e} (trace-implied bound {bound:.3e}) "
          f"gradient {errs[2]:.3e}, with the BF16 buffer {errs[3]:.3e}, with the FP16 buffer {e16:.3e}; "
          f"compensated forward: traces {hp_errs[0]:.3e} misfit {hp_errs[1]:.3e} gradient {hp_errs[2]:.3e}")
    assert errs[0] < TRACE_TOL and errs[1] <= max(MISFIT_TOL, 1.1 * bound)
    assert errs[2] < GRAD_TOL
    assert errs[3] < 5e-3  # BF16 buffer: about 2.4e-3 here
    assert e16 < 1e-3     # the bar of the reduced-precision buffer, met by the FP16 one
    assert hp_errs[0] < TRACE_TOL and hp_errs[1] < MISFIT_TOL and hp_errs[2] < GRAD_TOL
