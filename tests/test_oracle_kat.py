"""Pins the CPU oracle against the known-answer tests of the reference's own
test-suite (SeismicWaves.jl test/), re-run on the oracle:

* analytical Green's functions, 1 % integrated-error criterion
  (test_analytical_vs_numerical_acoustic_constant_density.jl:63-152,
  test/utils/setup_models.jl:76-99, 155-179, 221-280);
* invariance of the traces under reversing the source/receiver order
  (test_forward_constant_density.jl:152-266);
* gradient with checkpointing == without (test_gradient_acoustic_constant_density.jl:234-312);
* misfit returned by the gradient == misfit of a forward run (:124-195).
"""
import numpy as np
import pytest

from cases import ricker


def _nearest(pos, h):
    return np.floor(np.atleast_2d(pos) / np.asarray(h) + 1 + 0.5).astype(np.int32)


def _scaled(tf, si, vp, h, dt):
    scal = tf / np.prod(h) * dt ** 2
    for s in range(scal.shape[1]):
        scal[:, s] = scal[:, s] * vp[tuple(si[s] - 1)] ** 2
    return scal


def _const_setup(n, h, c0, f0, nt, dt):
    """setup_constant_vel_{2,3}D_CPML: source at the centre, receiver at lx/3."""
    ext = [(k - 1) * hh for k, hh in zip(n, h)]
    vp = np.full(n, c0, order="F")
    times = np.arange(nt) * dt
    srctf = ricker(times, 2 / f0, f0).reshape(nt, 1)
    possrc = np.array([[e / 2 for e in ext]])
    posrec = np.array([[ext[0] / 3] + [e / 2 for e in ext[1:]]])
    return vp, srctf, possrc, posrec


def _analytical(dim, c0, dt, nt, srctf, possrc, posrec):
    times = np.arange(1, nt + 1) * dt
    dist = np.linalg.norm(possrc[0] - posrec[0])
    src = c0 ** 2 * srctf[:, 0]
    G = np.zeros(nt)
    if dim == 2:
        m = times - dist / c0 >= 0
        G[m] = 1.0 / (2 * np.pi * c0 ** 2 * np.sqrt(times[m] ** 2 - dist ** 2 / c0 ** 2))
        Gc = np.convolve(G, src * dt)[:nt]
    else:
        k = np.argmax(times - dist / c0 >= 0)
        G[k] = 1.0 / (4 * np.pi * c0 ** 2 * dist)
        Gc = np.convolve(G, src)[:nt]
    return times, Gc


@pytest.mark.parametrize("dim,halo", [(2, 0), (2, 20), (3, 0), (3, 20)])
def test_analytical_green(oracle, dim, halo):
    c0, f0 = 1000.0, 5.0
    if dim == 2:
        n, h, nt = (801, 801), (2.5, 2.5), (700 if halo == 0 else 1400)
        dt = (1.0 if halo == 0 else 0.99) * 2.5 / c0 / np.sqrt(2)
    else:
        n, h, nt = (121, 121, 121), (8.0, 8.0, 8.0), (200 if halo == 0 else 400)
        dt = 0.99 * 8.0 / c0 / np.sqrt(3)
    rcoef = 1.0 if halo == 0 else 1e-4
    vp, srctf, possrc, posrec = _const_setup(n, h, c0, f0, nt, dt)
    si, ri = _nearest(possrc, h), _nearest(posrec, h)
    cp = oracle.cpml_blocks(vp, h, dt, halo, rcoef, f0, False)
    tr = oracle.acoustic_forward(vp, h, dt, halo, cp, _scaled(srctf, si, vp, h, dt), si, ri)
    times, Gc = _analytical(dim, c0, dt, nt, srctf, possrc, posrec)
    err = np.trapezoid(np.abs(tr[:, 0] - Gc), times)
    assert err <= np.max(np.abs(Gc)) * 0.01 * (dt * nt)


def _gaussian_vel_2d(nx, ny, c0, c0max, r):
    sigma = r / 3
    x, y = np.meshgrid(np.arange(1, nx + 1), np.arange(1, ny + 1), indexing="ij")
    o = ((nx + 1) / 2, (ny + 1) / 2)
    return np.asfortranarray(c0 + (c0max - c0) * np.exp(-0.5 * ((x - o[0]) ** 2 + (y - o[1]) ** 2) / sigma ** 2))


@pytest.mark.parametrize("nsrcs", [1, 3])
def test_reversal_invariance(oracle, nsrcs):
    nx = ny = 801
    vp = _gaussian_vel_2d(nx, ny, 1000.0, 1300.0, 150)
    nt, dx, halo, f0 = 700, 2.5, 20, 5.0
    lx, ly = (nx - 1) * dx, (ny - 1) * dx
    dt = 0.99 * dx / 1300.0 / np.sqrt(2)
    times = np.arange(nt) * dt
    dist = 20 if nsrcs > 1 else 0
    xs = lx / 2 - dist * ((nsrcs + 1) / 2 - np.arange(1, nsrcs + 1)) * dx
    possrc = np.stack([xs, np.full(nsrcs, (halo + 10) * dx)], 1)
    srctf = np.repeat(ricker(times, 2 / f0, f0).reshape(nt, 1), nsrcs, axis=1)
    xr = lx / 2 - 50 * ((4 + 1) / 2 - np.arange(1, 5)) * dx
    posrec = np.stack([xr, np.full(4, ly - (halo + 10) * dx)], 1)
    cp = oracle.cpml_blocks(vp, (dx, dx), dt, halo, 1e-4, f0, False)

    def run(ps, pr):
        si, ri = _nearest(ps, (dx, dx)), _nearest(pr, (dx, dx))
        return oracle.acoustic_forward(vp, (dx, dx), dt, halo, cp, _scaled(srctf.copy(), si, vp, (dx, dx), dt), si, ri)

    a = run(possrc, posrec)
    b = run(possrc[::-1] if nsrcs > 1 else possrc, posrec[::-1])
    for i in range(4):
        np.testing.assert_allclose(a[:, i], b[:, 3 - i], rtol=np.sqrt(np.finfo(float).eps), atol=0)


@pytest.mark.parametrize("dim", [2, 3])
def test_checkpointing_equivalence_and_misfit(oracle, dim):
    c0, f0 = 2000.0, 10.0
    if dim == 2:
        n, h, nt = (101, 101), (10.0, 10.0), 1000
        dt = 0.99 * 10.0 / c0 / np.sqrt(2)
    else:
        n, h, nt = (81, 81, 81), (10.0, 10.0, 10.0), 150
        dt = 0.99 * 10.0 / c0 / np.sqrt(3)
    vp, srctf, possrc, posrec = _const_setup(n, h, c0, f0, nt, dt)
    si, ri = _nearest(possrc, h), _nearest(posrec, h)
    cp = oracle.cpml_blocks(vp, h, dt, 20, 1e-4, f0, False)
    scal = _scaled(srctf, si, vp, h, dt)
    observed = srctf.copy()  # L2Misfit(observed=srctf, invcov=I)
    g1, m1, tr1 = oracle.acoustic_gradient(vp, h, dt, 20, cp, scal, si, ri, observed, check_freq=1)
    g2, m2, _ = oracle.acoustic_gradient(vp, h, dt, 20, cp, scal, si, ri, observed,
                                         check_freq=int(np.sqrt(nt)))
    assert np.any(g1 != 0)
    np.testing.assert_allclose(g2, g1, rtol=np.sqrt(np.finfo(float).eps) * 10, atol=0)
    # misfit of the gradient run == misfit of a plain forward (swmisfit!)
    tr = oracle.acoustic_forward(vp, h, dt, 20, cp, scal, si, ri)
    mf = 0.5 * np.sum((tr - observed) ** 2)
    assert m1 > 0 and abs(m1 - mf) <= 1e-12 * mf and abs(m2 - mf) <= 1e-12 * mf


def test_fp32_restatement_error_budget(oracle):
    """The FP32 instantiation stays within the trace tolerance the GPU is held to."""
    nx = nz = 301
    h, f0, nt = 5.0, 10.0, 3000
    rng = np.random.default_rng(0)
    vp = np.asfortranarray(1500.0 + 2000.0 * np.linspace(0, 1, nz)[None, :] + 50 * rng.standard_normal((nx, nz)) * 0)
    dt = 0.6 * h / (np.max(vp) * np.sqrt(2))
    times = np.arange(nt) * dt
    srctf = ricker(times, 1.2 / f0, f0).reshape(nt, 1)
    si = _nearest(np.array([[750.0, 100.0]]), (h, h))
    ri = _nearest(np.stack([np.linspace(50, 1450, 29), np.full(29, 60.0)], 1), (h, h))
    cp = oracle.cpml_blocks(vp, (h, h), dt, 20, 1e-4, f0, False)
    scal = _scaled(srctf, si, vp, (h, h), dt)
    a = oracle.acoustic_forward(vp, (h, h), dt, 20, cp, scal, si, ri)
    b = oracle.acoustic_forward(vp, (h, h), dt, 20, cp, scal, si, ri, f32=True)
    assert np.linalg.norm(a - b) / np.linalg.norm(a) < 1e-5


# --------------------------------------------------------------------------- CCTS misfit
def test_ccts_time_shift_known_answer(oracle):
    """A wavelet delayed by L samples gives dtau = (L + 1) dt: the reference's
    (argmax - (nt - 1)) indexing of DSP's 1-based xcorr (CCTSMisfit.jl:23).
    The host mirror and the oracle agree on misfit and adjoint source."""
    import __graft_entry__

    sw = __graft_entry__.load_package()
    nt, dt, f0 = 400, 1e-3, 25.0
    t = np.arange(nt) * dt
    syn = np.stack([ricker(t, 0.1, f0), 0.5 * ricker(t, 0.15, f0)], 1)
    shifts = (7, -4)
    obs = np.stack([np.roll(syn[:, r], s) for r, s in enumerate(shifts)], 1)
    m = sw.CCTSMisfit(dt, observed=obs)
    recs = sw.ScalarReceivers(np.zeros((2, 2)), nt)
    recs.seismograms[...] = syn
    want = sum(((s + 1) * dt) ** 2 / 2 for s in shifts)
    assert m.calcmisfit(recs) == pytest.approx(want, rel=1e-12)
    g = m.dchi_du(recs)
    assert np.sign(g[np.argmax(np.abs(g[:, 0])), 0]) != 0 and g.shape == syn.shape


def test_ccts_gradient_misfit_consistency(oracle):
    """2D counterpart of the reference's CCTS gradient test
    (test_gradient_acoustic_constant_density.jl:53-86): non-zero gradient and
    the gradient run's misfit == CCTS misfit of a forward run (host mirror)."""
    import __graft_entry__

    sw = __graft_entry__.load_package()
    c0, f0 = 2000.0, 10.0
    n, h, nt = (101, 101), (10.0, 10.0), 600
    dt = 0.99 * 10.0 / c0 / np.sqrt(2)
    vp, srctf, possrc, posrec = _const_setup(n, h, c0, f0, nt, dt)
    si, ri = _nearest(possrc, h), _nearest(posrec, h)
    cp = oracle.cpml_blocks(vp, h, dt, 20, 1e-4, f0, False)
    scal = _scaled(srctf, si, vp, h, dt)
    observed = srctf.copy()
    g, m, tr = oracle.acoustic_gradient(vp, h, dt, 20, cp, scal, si, ri, observed, check_freq=24, ccts_dt=dt)
    assert np.any(g != 0) and m > 0
    mis = sw.CCTSMisfit(dt, observed=observed)
    recs = sw.ScalarReceivers(posrec, nt)
    recs.seismograms[...] = tr
    assert m == pytest.approx(mis.calcmisfit(recs), rel=1e-12)


def test_vp_gradient_finite_difference_sign(oracle, sw):
    """The reference's constant-density gradient is -d(chi)/d(vp): <g, dv> against
    the central difference of the misfit along a Gaussian dv agrees to 1 % with
    the opposite sign (the reverse-mode rule of the backend relies on it)."""
    from cases import Case, make_shot, oracle_forward, oracle_gradient, smooth_model, stable_dt
    n, h = (90, 80), (5.0, 5.0)
    vp = smooth_model(n, 1800.0, 3000.0, seed=3)
    dt = stable_dt(vp, h)
    shot = make_shot(h, None, 500, dt, 15.0, [[200.0, 200.0]], [[x, 120.0] for x in np.linspace(80, 360, 9)])
    case = Case(vp, h, dt, 10, False, shots=[shot])
    shot.observed = oracle_forward(oracle, sw, Case(np.asfortranarray(vp * 1.03), h, dt, 10, False), shot)
    g, _, _ = oracle_gradient(oracle, sw, case, shot, check_freq=7)
    x = np.arange(n[0])[:, None]
    z = np.arange(n[1])[None, :]
    dv = np.exp(-((x - 60) ** 2 + (z - 30) ** 2) / (2 * 6.0 ** 2))
    eps = 2.0
    ms = [oracle_gradient(oracle, sw, Case(np.asfortranarray(vp + s * eps * dv), h, dt, 10, False), shot,
                          check_freq=7)[1] for s in (1, -1)]
    fd = (ms[0] - ms[1]) / (2 * eps)
    an = float(np.sum(g * dv))
    assert abs(fd) > 0 and abs(an + fd) <= 0.01 * abs(fd)
