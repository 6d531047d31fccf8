"""CPU checks of the variable-density acoustic 2D oracle.

Known answers from the reference's own tests:
  * analytical 2D Green's function, 1 % integrated-error criterion
    (test/test_analytical_vs_numerical_acoustic_variable_density.jl:68-115,
    test/utils/setup_models.jl:101-123, 241-259);
  * gradient with checkpointing == without, non-zero vp and rho gradients,
    misfit of the gradient run == misfit of a forward run
    (test/test_gradient_acoustic_variable_density.jl);
plus a central finite-difference check of the vp gradient and the FP32
error budget.

Sign convention.  The reference injects the adjoint source -C^-1 r and
returns -2 g0 / (vp^3 rho) with g0 = -sum adjp dp/dt * dt^-1
(acou_gradient.jl:146-201); central differences of the misfit show that this
is the negative of d(chi)/d(vp) (a descent direction), as for its
constant-density path.  The restatement keeps the reference's sign.
"""
from __future__ import annotations

import math

import numpy as np
import pytest

import oracle
from vd_cases import VDCase, VDShot, gaussderiv, nearest, oracle_forward, oracle_gradient, rel_l2, ricker, small_case


def _const_setup(n, h, c0, rho0, f0, nt, dt, halo, rcoef):
    """setup_constant_vel_rho_2D_CPML: gaussderivstf source at the centre, receiver at lx/3."""
    lx, ly = (n[0] - 1) * h, (n[1] - 1) * h
    t = np.arange(nt) * dt
    tf = gaussderiv(t, 2 / f0, f0).reshape(nt, 1)
    shot = VDShot(np.array([[lx / 2, ly / 2]]), np.array([[lx / 3, ly / 2]]), tf, f0)
    vp = np.full(n, c0, order="F")
    rho = np.full(n, rho0, order="F")
    return VDCase(vp, rho, h, dt, halo, rcoef=rcoef, shots=[shot])


def _analytical(c0, rho, dt, nt, t0, f0, src, rec):
    """analytical_solution_constant_vel_constant_density_2D (setup_models.jl:241-259)."""
    times = dt / 2 + np.arange(nt) * dt
    dist = np.linalg.norm(src[0] - rec[0])
    s = c0 ** 2 * rho * ricker(times, t0, f0)
    G = np.zeros(nt)
    m = times - dist / c0 >= 0
    G[m] = 1.0 / (2 * np.pi * c0 ** 2 * np.sqrt(times[m] ** 2 - dist ** 2 / c0 ** 2))
    return times, np.convolve(G, s * dt)[:nt]


@pytest.mark.parametrize("halo", [0, 20])
def test_vd_analytical_green(halo):
    c0, rho0, f0, h = 1000.0, 1500.0, 5.0, 5.0
    n = (401, 401)
    nt = 350 if halo == 0 else 350 * 4
    dt = 0.99 * h / c0 / math.sqrt(2) * 6 / 7
    case = _const_setup(n, h, c0, rho0, f0, nt, dt, halo, 1.0 if halo == 0 else 1e-4)
    shot = case.shots[0]
    tr = oracle_forward(case, shot)
    times, Gc = _analytical(c0, rho0, dt, nt, 2 / f0, f0, shot.src, shot.rec)
    err = np.trapezoid(np.abs(tr[:, 0] - Gc), times)
    assert err <= np.max(np.abs(Gc)) * 0.01 * (dt * nt)


def _gradient_setup():
    """The 2D case of test_gradient_acoustic_variable_density.jl: 101 x 101, nt 1000."""
    c0, rho0, f0, h = 2000.0, 1500.0, 10.0, 10.0
    nt = 1000
    dt = 0.99 * h / c0 / math.sqrt(2) * 6 / 7
    case = _const_setup((101, 101), h, c0, rho0, f0, nt, dt, 20, 1e-4)
    observed = case.shots[0].tf.copy()  # L2Misfit(observed=copy(srctf), invcov=I)
    return case, case.shots[0], observed


def test_vd_checkpoint_equivalence_and_misfit():
    case, shot, obs = _gradient_setup()
    g1, m1, tr1 = oracle_gradient(case, shot, obs, check_freq=1)
    gk, mk, _ = oracle_gradient(case, shot, obs, check_freq=int(math.floor(math.sqrt(shot.nt))))
    for k in ("vp", "rho"):
        assert np.any(g1[k] != 0.0)
        np.testing.assert_allclose(gk[k], g1[k], rtol=1e-12, atol=0)
    tr = oracle_forward(case, shot)
    assert np.array_equal(tr, tr1)
    mf = 0.5 * np.sum((tr - obs) ** 2)
    assert m1 > 0 and m1 == pytest.approx(mf, rel=1e-12) and mk == pytest.approx(mf, rel=1e-12)


def test_vd_vp_gradient_finite_difference():
    """<g_vp, dv> against the central difference of the misfit along dv: the
    reference's gradient is -d(chi)/d(vp); its magnitude agrees to 3 %."""
    case = small_case(nt=500, nx=90, nz=80, halo=10)
    shot = case.shots[0]
    pert = VDCase(case.vp * 1.03, case.rho, case.h, case.dt, case.halo, shots=[shot])
    obs = oracle_forward(pert, shot)
    g, m0, _ = oracle_gradient(case, shot, obs, check_freq=7)
    x = np.arange(case.vp.shape[0])[:, None]
    z = np.arange(case.vp.shape[1])[None, :]
    dv = np.exp(-((x - 40) ** 2 + (z - 55) ** 2) / (2 * 6.0 ** 2))
    eps = 2.0
    mis = []
    for s in (1, -1):
        c = VDCase(case.vp + s * eps * dv, case.rho, case.h, case.dt, case.halo, shots=[shot])
        _, m, _ = oracle_gradient(c, shot, obs, check_freq=7)
        mis.append(m)
    fd = (mis[0] - mis[1]) / (2 * eps)
    an = float(np.sum(g["vp"] * dv))
    print(f"VD vp gradient: <g, dv> = {an:.6e}, central difference = {fd:.6e}")
    assert abs(fd) > 0
    assert abs(an + fd) <= 0.03 * abs(fd)


def test_vd_interp_methods_differ_and_agree_on_constant_rho():
    case = small_case(nt=200, nx=70, nz=60, halo=8)
    shot = case.shots[0]
    a = oracle_forward(case, shot)
    case.interp = 1
    b = oracle_forward(case, shot)
    assert rel_l2(a, b) > 1e-8  # harmonic and arithmetic 1/rho at half points differ on a varying rho
    c0 = VDCase(case.vp, np.full(case.vp.shape, 2000.0, order="F"), case.h, case.dt, case.halo, shots=[shot])
    x = oracle_forward(c0, shot)
    c0.interp = 1
    y = oracle_forward(c0, shot)
    assert rel_l2(x, y) < 1e-14


@pytest.mark.parametrize("freetop", [False, True])
def test_vd_fp32_budget(freetop):
    case = small_case(nt=600, nx=110, nz=90, freetop=freetop)
    shot = case.shots[0]
    t64 = oracle_forward(case, shot)
    t32 = oracle_forward(case, shot, f32=True)
    assert np.abs(t64).max() > 0
    assert rel_l2(t32, t64) < 1e-5


def test_vd_snapshots_match_forward_state():
    case = small_case(nt=120, nx=60, nz=50, halo=6)
    shot = case.shots[0]
    tr, snaps = oracle_forward(case, shot, snapevery=40)
    assert len(snaps) == 3
    ri = nearest(shot.rec, case.h) - 1
    for k, (p, vx, vz) in enumerate(snaps):
        it = 40 * (k + 1)
        assert vx.shape == (59, 50) and vz.shape == (60, 49)
        np.testing.assert_array_equal(tr[it - 1], p[ri[:, 0], ri[:, 1]])


def test_vd_rho_gradient_finite_difference():
    """The rho gradient carries the same sign as vp's (-d(chi)/d(rho)); it agrees
    with the central difference of the misfit to 1 %."""
    case = small_case(nt=500, nx=90, nz=80, halo=10)
    shot = case.shots[0]
    pert = VDCase(case.vp * 1.03, case.rho * 0.97, case.h, case.dt, case.halo, shots=[shot])
    obs = oracle_forward(pert, shot)
    g, _, _ = oracle_gradient(case, shot, obs, check_freq=7)
    x = np.arange(case.vp.shape[0])[:, None]
    z = np.arange(case.vp.shape[1])[None, :]
    dv = np.exp(-((x - 40) ** 2 + (z - 55) ** 2) / (2 * 6.0 ** 2))
    eps = 2.0
    ms = [oracle_gradient(VDCase(case.vp, np.asfortranarray(case.rho + s * eps * dv), case.h, case.dt, case.halo,
                                 shots=[shot]), shot, obs, check_freq=7)[1] for s in (1, -1)]
    fd = (ms[0] - ms[1]) / (2 * eps)
    an = float(np.sum(g["rho"] * dv))
    assert abs(fd) > 0 and abs(an + fd) <= 0.01 * abs(fd)
