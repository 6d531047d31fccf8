"""GPU parity of the acoustic constant-density path against the FP64 CPU oracle.

Every test calls libswgb300 through its C ABI (tests/cases.py:GpuRun) with
the same inputs the oracle gets.  Tolerances are the ones the FP32 backend is
held to against the FP64 restatement of the reference: traces within 1e-5
relative L2, misfit within 1e-6, gradient within 1e-5.
"""
import numpy as np
import pytest

from cases import Case, GpuRun, make_shot, oracle_forward, oracle_gradient, rel_l2, smooth_model, stable_dt

pytestmark = pytest.mark.gpu

TRACE_TOL = 1e-5
MISFIT_TOL = 1e-6
GRAD_TOL = 1e-5
# Gradient with the recompute buffer in BF16: its 8-bit significand bounds each
# stored second difference to 2^-9 relative, and the correlation sums near the
# source are dominated by a few time samples, so the error sits at about 1e-3
# (measured 0.96e-3 in 2D, 1.09e-3 in 3D); the bound leaves 50 % headroom.
GRAD_TOL_BF16 = 1.5e-3


def _case2d(nx, nz, h, halo, freetop, seed=1, frac=0.6, vmin=1500.0, vmax=3000.0):
    vp = smooth_model((nx, nz), vmin, vmax, seed)
    return Case(vp=vp, h=(h, h), dt=stable_dt(vp, (h, h), frac), halo=halo, freetop=freetop)


def _extent(case):
    return [h * (n - 1) for n, h in zip(case.vp.shape, case.h)]


@pytest.mark.parametrize("halo,freetop", [(20, False), (20, True), (8, True), (3, False), (2, False), (1, False),
                                          (0, False)])
def test_forward_2d_matches_oracle(sw, oracle, halo, freetop):
    case = _case2d(120 + 3, 97, 8.0, halo, freetop, seed=halo)
    ex = _extent(case)
    nt = 500
    recx = np.linspace(0.1 * ex[0], 0.9 * ex[0], 13)
    shot = make_shot(case.h, ex, nt, case.dt, 14.0, [[0.43 * ex[0], 0.37 * ex[1]]],
                     np.stack([recx, np.full_like(recx, 0.6 * ex[1])], 1))
    run = GpuRun(sw, case)
    tr = run.forward([shot])[0]
    run.close()
    ref = oracle_forward(oracle, sw, case, shot)
    assert np.all(np.isfinite(tr))
    assert rel_l2(tr, ref) < TRACE_TOL


def test_forward_2d_odd_grid_duplicates_and_boundary(sw, oracle):
    """Ragged 23x29 grid, halo 3: sources and receivers sharing grid points,
    receivers on the outermost lines and a source on the free surface."""
    case = _case2d(23, 29, 5.0, 3, True, seed=7)
    ex = _extent(case)
    nt = 240
    src = [[0.5 * ex[0], 0.0], [0.5 * ex[0], 0.0], [0.3 * ex[0], 0.5 * ex[1]]]
    rec = [[0.0, 0.2 * ex[1]], [ex[0], ex[1]], [0.3 * ex[0], 0.5 * ex[1]], [0.3 * ex[0], 0.5 * ex[1]],
           [0.7 * ex[0], 0.4 * ex[1]], [0.5 * ex[0], 0.0]]
    shot = make_shot(case.h, ex, nt, case.dt, 20.0, src, rec)
    run = GpuRun(sw, case)
    tr = run.forward([shot])[0]
    run.close()
    ref = oracle_forward(oracle, sw, case, shot)
    assert rel_l2(tr, ref) < TRACE_TOL
    # the duplicated receivers see the same value
    assert np.array_equal(tr[:, 2], tr[:, 3])


def test_forward_batched_equals_single(sw, oracle):
    """Shots with different nt and receiver counts in one call: each matches
    the oracle and is bit-identical to running it alone."""
    case = _case2d(150, 110, 10.0, 12, False, seed=3)
    ex = _extent(case)
    rng = np.random.default_rng(5)
    shots = []
    for k, nt in enumerate([420, 300, 511, 300]):
        nrec = int(rng.integers(3, 17))
        recx = np.linspace(0.15 * ex[0], 0.85 * ex[0], nrec)
        shots.append(make_shot(case.h, ex, nt, case.dt, 12.0, [[(0.2 + 0.2 * k) * ex[0], 0.3 * ex[1]]],
                               np.stack([recx, np.full_like(recx, 0.5 * ex[1])], 1)))
    run = GpuRun(sw, case)
    batched = run.forward(shots)
    singles = [run.forward([s])[0] for s in shots]
    run.close()
    for s, b, one in zip(shots, batched, singles):
        assert b.shape == (s.nt, s.rec_pos.shape[0])
        assert np.array_equal(b, one)
        assert rel_l2(b, oracle_forward(oracle, sw, case, s)) < TRACE_TOL


def test_forward_2d_long_run(sw, oracle):
    """3000 steps on a 301x201 smooth model: FP32 error growth stays inside the bound."""
    case = _case2d(301, 201, 5.0, 20, False, seed=11, vmin=1500.0, vmax=3500.0)
    ex = _extent(case)
    recx = np.linspace(0.05 * ex[0], 0.95 * ex[0], 41)
    shot = make_shot(case.h, ex, 3000, case.dt, 10.0, [[0.5 * ex[0], 0.12 * ex[1]]],
                     np.stack([recx, np.full_like(recx, 0.1 * ex[1])], 1))
    run = GpuRun(sw, case)
    tr = run.forward([shot])[0]
    run.close()
    assert rel_l2(tr, oracle_forward(oracle, sw, case, shot)) < TRACE_TOL


def _grad_case(sw, oracle, nt=400, freetop=False, halo=10, seed=2):
    case = _case2d(110, 90, 10.0, halo, freetop, seed=seed)
    ex = _extent(case)
    recx = np.linspace(0.1 * ex[0], 0.9 * ex[0], 9)
    shot = make_shot(case.h, ex, nt, case.dt, 12.0, [[0.35 * ex[0], 0.25 * ex[1]]],
                     np.stack([recx, np.full_like(recx, 0.2 * ex[1])], 1))
    pert = Case(vp=np.asfortranarray(case.vp * 1.05), h=case.h, dt=case.dt, halo=case.halo,
                freetop=case.freetop)
    shot.observed = oracle_forward(oracle, sw, pert, shot)
    return case, shot


@pytest.mark.parametrize("check_freq", [1, 7, 20])
def test_gradient_2d_matches_oracle(sw, oracle, check_freq):
    case, shot = _grad_case(sw, oracle)
    run = GpuRun(sw, case, gradient=True, check_freq=check_freq)
    g, msf, tr = run.gradient([shot])
    run.close()
    gref, mref, tref = oracle_gradient(oracle, sw, case, shot, check_freq=check_freq)
    assert rel_l2(tr[0], tref) < TRACE_TOL
    assert abs(msf - mref) / abs(mref) < MISFIT_TOL
    assert rel_l2(g, gref) < GRAD_TOL


def test_gradient_checkpointing_is_exact(sw, oracle):
    """check_freq = floor(sqrt(nt)) gives the same gradient bits as storing every step."""
    case, shot = _grad_case(sw, oracle, nt=500)
    r1 = GpuRun(sw, case, gradient=True, check_freq=1)
    g1, m1, _ = r1.gradient([shot])
    r1.close()
    r2 = GpuRun(sw, case, gradient=True, check_freq=int(np.sqrt(500)))
    g2, m2, _ = r2.gradient([shot])
    r2.close()
    assert np.array_equal(g1, g2) and m1 == m2
    assert np.any(g1 != 0)


def test_gradient_windows_invcov_mute_freetop(sw, oracle):
    case, shot = _grad_case(sw, oracle, nt=360, freetop=True, halo=8, seed=4)
    rng = np.random.default_rng(3)
    shot.invcov = rng.uniform(0.5, 2.0, shot.nt)
    shot.windows = [(20, 150), (200, 330)]
    run = GpuRun(sw, case, gradient=True, check_freq=9, mute_src=4, mute_rec=2)
    g, msf, _ = run.gradient([shot])
    run.close()
    gref, mref, _ = oracle_gradient(oracle, sw, case, shot, check_freq=9, mute_src=4, mute_rec=2)
    assert abs(msf - mref) / abs(mref) < MISFIT_TOL
    assert rel_l2(g, gref) < GRAD_TOL


def test_gradient_batched_shots_sum(sw, oracle):
    """Several shots with different nt in one call: gradient = sum of the
    oracle's per-shot gradients, misfit = sum of misfits."""
    case = _case2d(120, 100, 10.0, 10, False, seed=9)
    ex = _extent(case)
    shots = []
    pert = Case(vp=np.asfortranarray(case.vp * 0.97), h=case.h, dt=case.dt, halo=case.halo, freetop=False)
    for k, nt in enumerate([350, 280, 401]):
        nrec = 5 + 3 * k
        recx = np.linspace(0.1 * ex[0], 0.9 * ex[0], nrec)
        s = make_shot(case.h, ex, nt, case.dt, 12.0, [[(0.25 + 0.25 * k) * ex[0], 0.2 * ex[1]]],
                      np.stack([recx, np.full_like(recx, 0.15 * ex[1])], 1))
        s.observed = oracle_forward(oracle, sw, pert, s)
        shots.append(s)
    run = GpuRun(sw, case, gradient=True, check_freq=10)
    g, msf, _ = run.gradient(shots)
    run.close()
    gref = np.zeros_like(g)
    mref = 0.0
    for s in shots:
        gg, mm, _ = oracle_gradient(oracle, sw, case, s, check_freq=10)
        gref += gg
        mref += mm
    assert abs(msf - mref) / abs(mref) < MISFIT_TOL
    assert rel_l2(g, gref) < GRAD_TOL


def test_gradient_rejects_boundary_source_with_checkpoints(sw, oracle):
    case, shot = _grad_case(sw, oracle, nt=200, freetop=True)
    shot.src_pos = np.array([[0.5 * _extent(case)[0], 0.0]])
    run = GpuRun(sw, case, gradient=True, check_freq=10)
    with pytest.raises(sw._lib.SwError) as e:
        run.gradient([shot])
    assert e.value.code == sw._lib.SW_ERR_UNSUPPORTED
    run.close()


def _case3d(n, h, halo, freetop, seed=1):
    vp = smooth_model(n, 1800.0, 3200.0, seed, blobs=3)
    return Case(vp=vp, h=(h, h, h), dt=stable_dt(vp, (h, h, h), 0.6), halo=halo, freetop=freetop)


@pytest.mark.parametrize("variant", [0, 2])
@pytest.mark.parametrize("halo,freetop", [(5, False), (6, True), (0, False)])
def test_forward_3d_matches_oracle(sw, oracle, halo, freetop, variant):
    case = _case3d((37, 29, 33), 10.0, halo, freetop, seed=halo + 1)
    ex = _extent(case)
    rec = [[0.2 * ex[0], 0.3 * ex[1], 0.5 * ex[2]], [0.8 * ex[0], 0.6 * ex[1], 0.4 * ex[2]],
           [0.5 * ex[0], 0.5 * ex[1], 0.9 * ex[2]]]
    shot = make_shot(case.h, ex, 260, case.dt, 15.0, [[0.45 * ex[0], 0.55 * ex[1], 0.35 * ex[2]]], rec)
    run = GpuRun(sw, case, variant=variant)
    tr = run.forward([shot])[0]
    run.close()
    assert rel_l2(tr, oracle_forward(oracle, sw, case, shot)) < TRACE_TOL


@pytest.mark.parametrize("variant", [0, 2])
def test_gradient_3d_matches_oracle(sw, oracle, variant):
    """3D gradient with 4 (variant 0) or 8 (variant 2) y rows per block; the
    y extent (30) leaves a partly filled last tile in both."""
    case = _case3d((34, 30, 32), 10.0, 5, False, seed=4)
    ex = _extent(case)
    rec = [[x, 0.5 * ex[1], 0.3 * ex[2]] for x in np.linspace(0.2 * ex[0], 0.8 * ex[0], 5)]
    shot = make_shot(case.h, ex, 200, case.dt, 15.0, [[0.5 * ex[0], 0.5 * ex[1], 0.6 * ex[2]]], rec)
    pert = Case(vp=np.asfortranarray(case.vp * 1.04), h=case.h, dt=case.dt, halo=case.halo, freetop=False)
    shot.observed = oracle_forward(oracle, sw, pert, shot)
    run = GpuRun(sw, case, gradient=True, check_freq=13, variant=variant)
    g, msf, _ = run.gradient([shot])
    run.close()
    gref, mref, _ = oracle_gradient(oracle, sw, case, shot, check_freq=13)
    assert abs(msf - mref) / abs(mref) < MISFIT_TOL
    assert rel_l2(g, gref) < GRAD_TOL


@pytest.mark.parametrize("check_freq", [1, 7, 20])
def test_gradient_bf16_buffer_2d(sw, oracle, check_freq):
    """BF16 snapshots of the recompute buffer: traces and misfit unchanged (the
    forward pass is exact), gradient within 1e-3 of the FP64 oracle."""
    case, shot = _grad_case(sw, oracle, nt=600)
    run = GpuRun(sw, case, gradient=True, check_freq=check_freq, bf16=1)
    g, msf, tr = run.gradient([shot])
    run.close()
    gref, mref, tref = oracle_gradient(oracle, sw, case, shot, check_freq=check_freq)
    err = rel_l2(g, gref)
    print(f"bf16 buffer K={check_freq}: gradient rel L2 {err:.2e}")
    assert rel_l2(tr[0], tref) < TRACE_TOL
    assert abs(msf - mref) / abs(mref) < MISFIT_TOL
    assert err < GRAD_TOL_BF16


def test_gradient_bf16_buffer_3d(sw, oracle):
    case = _case3d((34, 30, 32), 10.0, 5, False, seed=4)
    ex = _extent(case)
    rec = [[x, 0.5 * ex[1], 0.3 * ex[2]] for x in np.linspace(0.2 * ex[0], 0.8 * ex[0], 5)]
    shot = make_shot(case.h, ex, 200, case.dt, 15.0, [[0.5 * ex[0], 0.5 * ex[1], 0.6 * ex[2]]], rec)
    pert = Case(vp=np.asfortranarray(case.vp * 1.04), h=case.h, dt=case.dt, halo=case.halo, freetop=False)
    shot.observed = oracle_forward(oracle, sw, pert, shot)
    run = GpuRun(sw, case, gradient=True, check_freq=13, bf16=1)
    g, msf, _ = run.gradient([shot])
    run.close()
    gref, mref, _ = oracle_gradient(oracle, sw, case, shot, check_freq=13)
    err = rel_l2(g, gref)
    print(f"bf16 buffer 3D: gradient rel L2 {err:.2e}")
    assert abs(msf - mref) / abs(mref) < MISFIT_TOL
    assert err < GRAD_TOL_BF16


def test_gradient_bf16_buffer_batched_grouped(sw, oracle):
    """The grouped 2D adjoint (4+ shots) reads the BF16 buffer too."""
    case, shot = _grad_case(sw, oracle, nt=400)
    shots = [shot] * 4
    run = GpuRun(sw, case, gradient=True, check_freq=10, bf16=1)
    g, msf, _ = run.gradient(shots)
    run.close()
    gref, mref, _ = oracle_gradient(oracle, sw, case, shot, check_freq=10)
    assert abs(msf - 4 * mref) / abs(4 * mref) < MISFIT_TOL
    assert rel_l2(g, 4 * gref) < GRAD_TOL_BF16


@pytest.mark.parametrize("check_freq", [7, 20])
def test_gradient_bf16_checkpoints_2d(sw, oracle, check_freq):
    """snapshot_bf16 = 2 also keeps the checkpoints' (p, d) in BF16: the
    quantisation noise of p seeds grid-scale noise in every recomputed window,
    so this mode trades accuracy (a few 1e-3) for memory; the bound here is 1e-2."""
    case, shot = _grad_case(sw, oracle, nt=600)
    run = GpuRun(sw, case, gradient=True, check_freq=check_freq, bf16=2)
    g, msf, tr = run.gradient([shot])
    run.close()
    gref, mref, tref = oracle_gradient(oracle, sw, case, shot, check_freq=check_freq)
    err = rel_l2(g, gref)
    print(f"bf16 checkpoints K={check_freq}: gradient rel L2 {err:.2e}")
    assert rel_l2(tr[0], tref) < TRACE_TOL
    assert abs(msf - mref) / abs(mref) < MISFIT_TOL
    assert err < 1e-2


@pytest.mark.parametrize("tz", [0, 7, 64])
def test_2d_stencil_variants_match_oracle(sw, oracle, tz):
    """The register-pipelined 2D stencil (variant 0), the TMA-pipelined one
    (variant 1) and the cp.async-staged one (variant 512) give the oracle's
    traces and gradient for any tile height."""
    case, shot = _grad_case(sw, oracle, nt=300, freetop=True, halo=12, seed=8)
    gref, mref, tref = oracle_gradient(oracle, sw, case, shot, check_freq=11)
    for variant in (0, 1, 512):
        run = GpuRun(sw, case, gradient=True, check_freq=11, variant=variant, tz=tz)
        g, msf, tr = run.gradient([shot])
        fw = run.forward([shot])[0]
        run.close()
        assert rel_l2(tr[0], tref) < TRACE_TOL
        assert rel_l2(fw, tref) < TRACE_TOL
        assert abs(msf - mref) / abs(mref) < MISFIT_TOL
        assert rel_l2(g, gref) < GRAD_TOL


def test_graph_replay_is_bitwise_identical(sw, oracle):
    """Calls 1 (direct), 2 (captured) and 3 (replayed) give the same bits as
    a simulation with graphs switched off, for the forward and the gradient."""
    case, shot = _grad_case(sw, oracle, nt=300)
    shots = [shot] * 5
    off = GpuRun(sw, case, gradient=True, check_freq=10)
    off.ctx.check(off.ctx.lib.sw_wavesim_use_graphs(off.h, 0), "use_graphs")
    g0, m0, t0 = off.gradient(shots)
    f0 = off.forward(shots)
    off.close()
    on = GpuRun(sw, case, gradient=True, check_freq=10)
    for _ in range(3):
        g, m, t = on.gradient(shots)
        assert np.array_equal(g, g0) and m == m0
        assert all(np.array_equal(a, b) for a, b in zip(t, t0))
        f = on.forward(shots)
        assert all(np.array_equal(a, b) for a, b in zip(f, f0))
    on.close()


@pytest.mark.parametrize("variant", [0, 256, 264, 512, 768])
def test_gradient_grouped_adjoint_variants(sw, oracle, variant):
    """The per-shot 2D adjoint with plain FP32 sums flushed into FP64 every 32
    steps (default), the grouped adjoint (256: 4+ shots, one Kahan update per
    group) with 4 or 5 (264) resident blocks per SM, and both with the
    cp.async-staged stencil (512, 768) match the oracle's shot sum."""
    case, shot = _grad_case(sw, oracle, nt=300)
    run = GpuRun(sw, case, gradient=True, check_freq=10, variant=variant)
    g, msf, _ = run.gradient([shot] * 5)
    run.close()
    gref, mref, _ = oracle_gradient(oracle, sw, case, shot, check_freq=10)
    assert abs(msf - 5 * mref) / abs(5 * mref) < MISFIT_TOL
    assert rel_l2(g, 5 * gref) < GRAD_TOL


def _dense_invcov(nt, seed=0):
    """A symmetric positive-definite inverse covariance with off-diagonal terms
    (exponentially correlated noise)."""
    i = np.arange(nt)
    c = np.exp(-np.abs(i[:, None] - i[None, :]) / 3.0)
    return np.linalg.inv(c + 0.1 * np.eye(nt))


def test_gradient_dense_invcov(sw, oracle):
    """A full inverse covariance (cuBLAS product on the device) against the oracle's dense C^-1 r."""
    case, shot = _grad_case(sw, oracle, nt=300)
    ic = _dense_invcov(shot.nt)
    shot.invcov = ic
    run = GpuRun(sw, case, gradient=True, check_freq=10)
    g, msf, _ = run.gradient([shot])
    run.close()
    gref, mref, _ = oracle_gradient(oracle, sw, case, shot, check_freq=10)
    print(f"dense invcov: misfit {abs(msf - mref) / abs(mref):.2e} gradient {rel_l2(g, gref):.2e}")
    assert abs(msf - mref) / abs(mref) < MISFIT_TOL
    assert rel_l2(g, gref) < GRAD_TOL


def test_cpa_stencil_agrees_with_register_pipeline(sw, oracle):
    """The cp.async-staged 2D kernels (variant 512) run the same row update as
    the register-pipelined ones: forward traces, misfit and gradient of a
    5-shot batch agree to rounding, with FP32 and with BF16 D buffers and
    with muting (the per-shot Kahan adjoint)."""
    case, shot = _grad_case(sw, oracle, nt=320, seed=6)
    shots = [shot] * 5
    for bf16, mute in ((0, 0), (1, 0), (0, 3)):
        out = []
        for variant in (0, 512):
            run = GpuRun(sw, case, gradient=True, check_freq=9, variant=variant, bf16=bf16, mute_src=mute)
            g, m, t = run.gradient(shots)
            f = run.forward(shots)
            run.close()
            out.append((g, m, t, f))
        (g0, m0, t0, f0), (g1, m1, t1, f1) = out
        same = np.array_equal(g0, g1) and m0 == m1 and all(np.array_equal(a, b) for a, b in zip(f0, f1))
        print(f"bf16={bf16} mute={mute}: bitwise equal {same}, gradient rel diff {rel_l2(g1, g0):.2e}")
        assert abs(m1 - m0) <= 1e-7 * abs(m0)
        assert rel_l2(g1, g0) < 1e-6
        assert all(rel_l2(a, b) < 1e-7 for a, b in zip(t1, t0))
        assert all(rel_l2(a, b) < 1e-7 for a, b in zip(f1, f0))
