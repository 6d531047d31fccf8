"""CPU checks of the elastic oracle and of the elastic host logic.

Known answers from the reference's own tests:
  * interpolation and back-interpolation KATs (test/test_interpolations.jl);
  * gradient checkpoint equivalence, non-zero gradients and misfit consistency
    (test/test_gradient_elastic_homogeneous.jl);
plus the sinc spreading of the host mirror against the oracle's independent
restatement (src/utils/utils.jl:62-214) and the modified Bessel function I0.
"""
from __future__ import annotations

import math

import numpy as np
import pytest

import oracle
from elastic_cases import E, ElCase, ElShot, homogeneous, oracle_forward, oracle_gradient, rel_l2, ricker, small_case, sw


M3 = np.array([[1.0, 2.0, 3.0], [4.0, 5.0, 6.0], [7.0, 8.0, 9.0]])


def test_interpolation_kats_1d():
    m = np.array([[1.0], [2.0], [3.0], [4.0]])
    assert np.array_equal(oracle.interp(m, [1])[:, 0], [1.5, 2.5, 3.5])
    assert np.allclose(oracle.interp(m, [1], 1)[:, 0], [1.333, 2.4, 3.428], atol=1e-3)
    g = np.array([[0.1], [0.2], [0.3]])
    exp = np.zeros(4)
    exp[:-1] += g[:, 0] * 0.5
    exp[1:] += g[:, 0] * 0.5
    assert np.allclose(oracle.back_interp(m, g, [1])[:, 0], exp)
    # harmonic: d f / d m = (-2/g^2) (-1/m^2) with g = 1/m_i + 1/m_{i+1}
    mm = m[:, 0]
    gg = 1 / mm[:-1] + 1 / mm[1:]
    exp = np.zeros(4)
    exp[:-1] += g[:, 0] * (2 / gg ** 2) / mm[:-1] ** 2
    exp[1:] += g[:, 0] * (2 / gg ** 2) / mm[1:] ** 2
    assert np.allclose(oracle.back_interp(m, g, [1], 1)[:, 0], exp)


def test_interpolation_kats_2d():
    m = M3
    assert np.array_equal(oracle.interp(m, [1]), [[2.5, 3.5, 4.5], [5.5, 6.5, 7.5]])
    assert np.array_equal(oracle.interp(m, [2]), [[1.5, 2.5], [4.5, 5.5], [7.5, 8.5]])
    assert np.array_equal(oracle.interp(m, [1, 2]), [[3.0, 4.0], [6.0, 7.0]])
    g4 = np.array([[1 / m[a, b] + 1 / m[a + 1, b] + 1 / m[a, b + 1] + 1 / m[a + 1, b + 1] for b in range(2)]
                   for a in range(2)])
    assert np.allclose(oracle.interp(m, [1, 2], 1), 4 / g4)
    assert np.allclose(oracle.interp(m, [1], 1), [[2 / (1 / m[a, b] + 1 / m[a + 1, b]) for b in range(3)]
                                                 for a in range(2)])
    d = np.array([[0.1, 0.2], [0.3, 0.4]])
    exp = np.zeros((3, 3))
    for pa in range(2):
        for pb in range(2):
            exp[pa:pa + 2, pb:pb + 2] += d * 0.25
    assert np.allclose(oracle.back_interp(m, d, [1, 2]), exp)
    exp = np.zeros((3, 3))
    for pa in range(2):
        for pb in range(2):
            exp[pa:pa + 2, pb:pb + 2] += d * (4 / g4 ** 2) / m[pa:pa + 2, pb:pb + 2] ** 2
    assert np.allclose(oracle.back_interp(m, d, [1, 2], 1), exp)
    d1 = np.array([[0.1, 0.2, 0.3], [0.4, 0.5, 0.6]])
    g15 = 1 / m[:-1, :] + 1 / m[1:, :]
    exp = np.zeros((3, 3))
    exp[0:2, :] += d1 * (2 / g15 ** 2) / m[0:2, :] ** 2
    exp[1:3, :] += d1 * (2 / g15 ** 2) / m[1:3, :] ** 2
    assert np.allclose(oracle.back_interp(m, d1, [1], 1), exp)
    d2 = np.array([[0.1, 0.2], [0.3, 0.4], [0.5, 0.6]])
    g25 = 1 / m[:, :-1] + 1 / m[:, 1:]
    exp = np.zeros((3, 3))
    exp[:, 0:2] += d2 * (2 / g25 ** 2) / m[:, 0:2] ** 2
    exp[:, 1:3] += d2 * (2 / g25 ** 2) / m[:, 1:3] ** 2
    assert np.allclose(oracle.back_interp(m, d2, [2], 1), exp)


def test_bessel_i0_series():
    sp = pytest.importorskip("scipy.special")
    for x in (0.0, 0.5, 3.0, 6.31, 9.0):
        assert oracle.bessel_i0(x) == pytest.approx(float(sp.i0(x)), rel=1e-14)


@pytest.mark.parametrize("shift,mirror", [((0, 0), True), ((2.5, 2.5), True), ((2.5, 0), False), ((0, 2.5), False)])
def test_spread_positions_host_vs_oracle(shift, mirror):
    n, h = (100, 80), (5.0, 5.0)
    pos = np.array([[250.0, 200.0], [252.5, 101.3], [0.0, 3.0], [497.0, 395.0], [13.1, 7.7]])
    a = E.spread_positions(n, h, pos, shift=shift, mirror=mirror)
    b = oracle.spread_positions(n, h, pos, shift=shift, mirror=mirror)
    for (ia, ca), (ib, cb) in zip(a, b):
        da = {tuple(x): c for x, c in zip(ia, ca)}
        db = {tuple(x): c for x, c in zip(ib, cb)}
        assert da.keys() == db.keys()
        assert max(abs(da[k] - db[k]) for k in da) < 1e-13


def test_spread_positions_delta_on_node():
    # a position on a grid node: sinc is 0 at every other node, a single weight 1
    (ij, c), = E.spread_positions((100, 80), (5.0, 5.0), np.array([[250.0, 200.0]]))
    assert ij.tolist() == [[51, 41]] and c.tolist() == [1.0]
    # interior off-node: the weights sum to about 1 and fill an 8 x 8 window
    (ij, c), = E.spread_positions((100, 80), (5.0, 5.0), np.array([[252.5, 201.3]]))
    assert len(c) == 64 and abs(c.sum() - 1.0) < 2e-3


def _reference_test_setup(kind):
    """setup_constant_elastic_2D_CPML (test/utils/setup_models.jl:125-152), shrunk."""
    rho0, vp0 = 2100.0, 3210.5
    vs0 = vp0 / math.sqrt(3)
    nx, nz, h, dt, halo = 120, 90, 4.5, 0.0005, 20
    nt = 150
    lam, mu, rho = homogeneous(nx, nz, vp0, rho0)
    lx, lz = (nx - 1) * h, (nz - 1) * h
    shot = ElShot(kind, np.array([[lx / 2, lz / 2]]), np.array([[lx / 3, lz / 2]]), nt, f0=12.0)
    case = ElCase(nx, nz, h, dt, halo, lam, mu, rho, [shot], rcoef=1e-4)
    # observed = the source wavelet on both components (as the reference test does)
    w = ricker(nt, dt, 12.0)
    obs = np.zeros((nt, 2, 1))
    obs[:, 0, 0] = w
    obs[:, 1, 0] = w
    return case, shot, obs * 1e-12


@pytest.mark.parametrize("kind", ["force", "mt"])
def test_elastic_checkpoint_equivalence(kind):
    case, shot, obs = _reference_test_setup(kind)
    K = int(math.floor(math.sqrt(shot.nt)))
    g1, m1, _ = oracle_gradient(case, shot, obs, check_freq=1)
    gk, mk, _ = oracle_gradient(case, shot, obs, check_freq=K)
    for k in ("rho", "lambda", "mu"):
        assert np.any(g1[k] != 0.0)
        assert np.allclose(gk[k], g1[k], rtol=1e-12, atol=0)
    assert m1 != 0.0 and mk == pytest.approx(m1, rel=1e-12)


def test_elastic_misfit_consistency():
    case, shot, obs = _reference_test_setup("force")
    _, msf, traces = oracle_gradient(case, shot, obs, check_freq=5)
    tr = oracle_forward(case, shot)
    assert np.array_equal(tr, traces)
    m = sw.L2Misfit(observed=obs)
    recs = E.VectorReceivers(shot.rec, shot.nt)
    recs.seismograms[...] = tr
    assert msf == pytest.approx(m.calcmisfit(recs), rel=1e-12)


def test_elastic_symmetry():
    """Explosive source at the centre of a symmetric homogeneous grid: ux is
    odd and uz even under x -> -x about the source (staggered grids included)."""
    nx, nz, h = 101, 81, 5.0
    lam, mu, rho = homogeneous(nx, nz)
    from elastic_cases import stable_dt
    dt = stable_dt(lam, mu, rho, h)
    xc = (nx - 1) * h / 2
    rec = np.array([[xc - 60.0, 150.0], [xc + 60.0, 150.0]])
    shot = ElShot("mt", np.array([[xc, 200.0]]), rec, 300)
    case = ElCase(nx, nz, h, dt, 20, lam, mu, rho, [shot])
    tr = oracle_forward(case, shot)
    assert np.abs(tr).max() > 0
    scale = np.abs(tr).max()
    assert np.abs(tr[:, 0, 0] + tr[:, 0, 1]).max() < 1e-9 * scale
    assert np.abs(tr[:, 1, 0] - tr[:, 1, 1]).max() < 1e-9 * scale


@pytest.mark.parametrize("freetop", [False, True])
def test_elastic_fp32_budget(freetop):
    """The FP32 restatement stays within the trace tolerance of the FP64 one
    on a short run (the error budget the GPU path is held to)."""
    case = small_case("mt", freetop=freetop, nt=300, nx=100, nz=90)
    shot = case.shots[0]
    t64 = oracle_forward(case, shot)
    t32 = oracle_forward(case, shot, f32=True)
    assert rel_l2(t32, t64) < 1e-5


def test_elastic_gradients_finite_difference():
    """Unlike the acoustic paths, the reference's elastic gradients are
    +d(chi)/d(lambda, mu, rho): central differences of the misfit along a
    Gaussian perturbation agree to 1e-4 (the discrete adjoint is exact)."""
    import copy
    case = small_case(nt=400, nx=90, nz=80, halo=10)
    shot = case.shots[0]
    pert = copy.deepcopy(case)
    pert.lam, pert.mu, pert.rho = case.lam * 1.05, case.mu * 0.97, case.rho * 0.98
    obs = oracle_forward(pert, shot)
    g, _, _ = oracle_gradient(case, shot, obs, check_freq=7)
    x = np.arange(case.nx)[:, None]
    z = np.arange(case.nz)[None, :]
    dv = np.exp(-((x - 40) ** 2 + (z - 55) ** 2) / (2 * 6.0 ** 2))
    for name, attr in (("lambda", "lam"), ("mu", "mu"), ("rho", "rho")):
        base = getattr(case, attr)
        eps = 1e-3 * float(np.mean(base))
        ms = []
        for s in (1, -1):
            c = copy.deepcopy(case)
            setattr(c, attr, base + s * eps * dv)
            ms.append(oracle_gradient(c, shot, obs, check_freq=7)[1])
        fd = (ms[0] - ms[1]) / (2 * eps)
        an = float(np.sum(g[name] * dv))
        assert abs(fd) > 0 and abs(an - fd) <= 1e-4 * abs(fd), name


def test_elastic_ccts_misfit_matches_host_definition():
    """The oracle's elastic CCTS misfit equals the host restatement of
    CCTSMisfit{T,3} (seismicwaves.jl_gb300/api.py, numpy correlate) on the
    oracle's own traces: one time shift per receiver and component."""
    import elastic_cases as EC

    import __graft_entry__
    sw = __graft_entry__.load_package()
    case = EC.small_case(nt=240, nx=70, nz=60, halo=10, seed=4)
    shot = case.shots[0]
    pert = EC.ElCase(case.nx, case.nz, case.h, case.dt, case.halo, case.lam * 1.2, case.mu, case.rho * 0.9,
                     [shot], freetop=case.freetop, sinc=case.sinc)
    obs = EC.oracle_forward(pert, shot)
    _, m, tr = EC.oracle_gradient(case, shot, obs, check_freq=10, ccts_dt=case.dt)
    mis = sw.CCTSMisfit(case.dt, observed=obs)
    recs = type("R", (), {"seismograms": tr})()
    assert m > 0 and m == pytest.approx(mis.calcmisfit(recs), rel=1e-12)
