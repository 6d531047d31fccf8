"""The compensated forward (sw_wavesim_set_precision(ws, 1)) against the FP64
oracle and against the FP32 forward on the same inputs.

FP32 state drifts to ~1e-6 relative trace error over a few thousand steps
(mostly the cancellation in the second differences); the compensated step
keeps p, d, fact and 1/h^2 as pairs of FP32 numbers and must bring the
traces several times closer to the oracle, the misfit under the 1e-6 bar,
and leave the gradient (FP32 recompute and adjoint) within its 1e-5 bar.
Cases: 2D with free surface and C-PML, several sources (two on one point),
a source on the grid's outer line (its node keeps the FP32 ring update), 3D,
BF16 recompute buffers, snapshots, and the variable-density path
(sw_acoustic_vd_set_precision: p, vx, vz compensated)."""
import ctypes

import numpy as np
import pytest

from cases import Case, GpuRun, make_shot, oracle_forward, oracle_gradient, rel_l2, smooth_model, stable_dt

pytestmark = pytest.mark.gpu

MISFIT_TOL = 1e-6
GRAD_TOL = 1e-5


def _case2d(nx=401, nz=201, halo=20, freetop=True, seed=11):
    vp = smooth_model((nx, nz), 1600.0, 3400.0, seed)
    h = (8.0, 8.0)
    return Case(vp=vp, h=h, dt=stable_dt(vp, h), halo=halo, freetop=freetop)


def _shot2d(case, nt, srcs=None, seed=0):
    ex = [h * (n - 1) for n, h in zip(case.vp.shape, case.h)]
    rng = np.random.default_rng(seed)
    if srcs is None:
        p = [rng.uniform(0.3, 0.7) * ex[0], rng.uniform(0.1, 0.3) * ex[1]]
        srcs = [p, p, [rng.uniform(0.2, 0.8) * ex[0], rng.uniform(0.2, 0.6) * ex[1]]]
    rec = [[x, 0.05 * ex[1]] for x in np.linspace(0.05, 0.95, 41) * ex[0]]
    return make_shot(case.h, ex, nt, case.dt, 12.0, srcs, rec)


def test_compensated_forward_2d_closer_to_oracle(sw, oracle):
    case = _case2d()
    shot = _shot2d(case, 2500)
    ref = oracle_forward(oracle, sw, case, shot)
    out = {}
    for prec in (0, 1):
        run = GpuRun(sw, case, precision=prec)
        out[prec] = run.forward([shot])[0]
        run.close()
    e32, ehp = rel_l2(out[0], ref), rel_l2(out[1], ref)
    print(f"2D 401 x 201, 2500 steps: FP32 traces {e32:.3e}, compensated {ehp:.3e}")
    assert ehp < 0.35 * e32
    assert ehp < 3e-7


def test_compensated_gradient_2d_meets_misfit_bar(sw, oracle):
    case = _case2d(seed=5)
    shots = [_shot2d(case, 2200, seed=1), _shot2d(case, 1900, seed=2)]
    obs_case = Case(vp=np.asfortranarray(case.vp * 1.04), h=case.h, dt=case.dt, halo=case.halo,
                    freetop=case.freetop)
    run = GpuRun(sw, obs_case)
    for s, o in zip(shots, run.forward(shots)):
        s.observed = np.asfortranarray(o, dtype=np.float64)
    run.close()
    gref, mref = 0.0, 0.0
    for s in shots:
        gk, mk, _ = oracle_gradient(oracle, sw, case, s, check_freq=40)
        gref, mref = gref + gk, mref + mk
    res = {}
    for prec, bf16 in ((0, 0), (1, 0), (1, 1)):
        run = GpuRun(sw, case, gradient=True, check_freq=40, precision=prec, bf16=bf16)
        g, m, _ = run.gradient(shots)
        run.close()
        res[(prec, bf16)] = (abs(m - mref) / mref, rel_l2(g, gref))
    print("misfit / gradient errors (precision, bf16):", {k: f"{v[0]:.2e} / {v[1]:.2e}" for k, v in res.items()})
    assert res[(1, 0)][0] < MISFIT_TOL
    assert res[(1, 0)][1] < GRAD_TOL
    assert res[(1, 1)][0] < MISFIT_TOL  # the BF16 buffer changes the recompute only
    assert res[(1, 1)][1] < 1e-2


def test_compensated_boundary_source_and_halo0(sw, oracle):
    """A source on the outermost grid line (its node evolves through the FP32
    ring of the injection kernel) and a grid without C-PML."""
    for halo, freetop in ((6, False), (0, False)):
        case = _case2d(nx=150, nz=90, halo=halo, freetop=freetop, seed=3)
        ex = [h * (n - 1) for n, h in zip(case.vp.shape, case.h)]
        shot = _shot2d(case, 700, srcs=[[0.0, 0.5 * ex[1]], [0.4 * ex[0], 0.5 * ex[1]]])
        ref = oracle_forward(oracle, sw, case, shot)
        run = GpuRun(sw, case, precision=1)
        tr = run.forward([shot])[0]
        run.close()
        assert rel_l2(tr, ref) < 1e-6, (halo, rel_l2(tr, ref))


def test_compensated_forward_3d_closer_to_oracle(sw, oracle):
    n = 72
    vp = smooth_model((n, n, n), 1800.0, 3000.0, 9)
    h = (10.0, 10.0, 10.0)
    case = Case(vp=vp, h=h, dt=stable_dt(vp, h), halo=10, freetop=True)
    ex = [hh * (k - 1) for k, hh in zip(vp.shape, h)]
    rec = [[x, y, 0.05 * ex[2]] for x in np.linspace(0.1, 0.9, 7) * ex[0] for y in np.linspace(0.1, 0.9, 5) * ex[1]]
    shot = make_shot(h, ex, 900, case.dt, 15.0, [[0.5 * ex[0], 0.45 * ex[1], 0.3 * ex[2]]], rec)
    ref = oracle_forward(oracle, sw, case, shot)
    out = {}
    for prec in (0, 1):
        run = GpuRun(sw, case, precision=prec)
        out[prec] = run.forward([shot])[0]
        run.close()
    e32, ehp = rel_l2(out[0], ref), rel_l2(out[1], ref)
    print(f"3D 72^3, 900 steps: FP32 traces {e32:.3e}, compensated {ehp:.3e}")
    assert ehp < 0.5 * e32


def test_compensated_snapshots_match_traces(sw):
    """Snapshots in compensated mode are the high parts of p: equal to the
    FP32-rounded state to within one rounding of the low part."""
    case = _case2d(nx=160, nz=80, halo=8, seed=4)
    shot = _shot2d(case, 120, seed=3)
    run = GpuRun(sw, case, precision=1)
    arr, keep, outs = run._structs([shot], False)
    buf = np.zeros((120 // 4) * case.vp.size, np.float32)
    ptrs = (ctypes.c_void_p * 1)(buf.ctypes.data)
    run.ctx.check(run.ctx.lib.sw_acoustic_forward_snapshots(run.h, 1, arr, 0, 4, ptrs), "snapshots")
    tr = run.forward([shot])[0]
    run.close()
    assert np.allclose(outs[0], tr, rtol=1e-6, atol=1e-6 * np.abs(tr).max())
    last = buf[-case.vp.size:]
    assert np.isfinite(last).all() and np.abs(last).max() > 0


def test_precision_rejects_bad_mode(sw):
    case = _case2d(nx=64, nz=40, halo=4, seed=1)
    run = GpuRun(sw, case)
    assert run.ctx.lib.sw_wavesim_set_precision(run.h, 2) != 0
    assert run.ctx.lib.sw_wavesim_set_precision(run.h, -1) != 0
    assert run.ctx.lib.sw_wavesim_set_precision(None, 1) != 0
    assert run.ctx.lib.sw_wavesim_set_precision(run.h, 0) == 0
    run.close()


def test_compensated_vd_forward_and_gradient(sw):
    """The variable-density path: compensated traces several times closer to
    the FP64 oracle than FP32 ones, and the gradient's misfit under the bar
    (free surface, C-PML, harmonic and arithmetic 1/rho)."""
    from vd_cases import GpuVD, VDCase, VDShot, oracle_forward as vd_forward, oracle_gradient as vd_gradient
    vp = smooth_model((260, 140), 1600.0, 3200.0, 31)
    rho = np.asfortranarray(310.0 * vp ** 0.25)
    h = 8.0
    dt = 0.45 * h / float(vp.max())
    ex = (259 * h, 139 * h)
    for interp, freetop in ((0, True), (1, False)):
        src = np.array([[0.5 * ex[0], 0.12 * ex[1]]])
        rec = np.stack([np.linspace(0.05, 0.95, 31) * ex[0], np.full(31, 0.05 * ex[1])], 1)
        shot = VDShot(src, rec, _ricker(1800, dt, 14.0), 14.0)
        case = VDCase(vp, rho, h, dt, 16, shots=[shot], interp=interp, freetop=freetop)
        ctx = sw._lib.Context(0)
        out = {}
        for prec in (0, 1):
            run = GpuVD(ctx, case, precision=prec)
            out[prec] = run.forward([shot])[0]
            run.close()
        ref = vd_forward(case, shot)
        e32, ehp = rel_l2(out[0], ref), rel_l2(out[1], ref)
        print(f"VD interp {interp}: FP32 traces {e32:.3e}, compensated {ehp:.3e}")
        assert ehp < 0.35 * e32 and ehp < 3e-7
        obs_case = VDCase(np.asfortranarray(vp * 1.04), np.asfortranarray(rho * 0.98), h, dt, 16, shots=[shot],
                          interp=interp, freetop=freetop)
        run = GpuVD(ctx, obs_case)
        obs = run.forward([shot])[0]
        run.close()
        run = GpuVD(ctx, case, gradient=True, check_freq=30, precision=1)
        g, m, _ = run.gradient([shot], [obs])
        run.close()
        ctx.close()
        gref, mref, _ = vd_gradient(case, shot, obs, check_freq=30)
        assert abs(m - mref) / mref < MISFIT_TOL
        assert rel_l2(g["vp"], gref["vp"]) < GRAD_TOL and rel_l2(g["rho"], gref["rho"]) < GRAD_TOL


def _ricker(nt, dt, f0):
    t = np.arange(nt) * dt - 1.2 / f0
    a = (np.pi * f0 * t) ** 2
    return ((1 - 2 * a) * np.exp(-a)).reshape(-1, 1)
