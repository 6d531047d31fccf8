"""Two time steps per stencil launch (k_ac2d_pair: forward, recompute and
adjoint kinds, tuning variant 1024) against one step per launch (the default).

The two-step kernel rounds exactly as two one-step launches do, so traces,
misfits and gradients must be bit-identical whether the library pairs steps
or not, across grid shapes that leave
partial warps and bands, free surface or not, halo 0, several sources (two on
one point), receivers on several rows, odd and even checkpoint periods (which
mix paired and single steps), BF16 recompute buffers and checkpoints, and
snapshots.  Each case also checks, through the per-kernel launch counts, that
steps were actually paired."""
import ctypes

import numpy as np
import pytest

from cases import Case, GpuRun, make_shot, oracle_forward, rel_l2, smooth_model, stable_dt

pytestmark = pytest.mark.gpu

PAIR = 1024


def _case(nx, nz, halo, freetop, seed):
    vp = smooth_model((nx, nz), 1500.0, 3200.0, seed)
    h = (7.0, 6.0)
    return Case(vp=vp, h=h, dt=stable_dt(vp, h), halo=halo, freetop=freetop)


def _shot(case, nt, seed):
    rng = np.random.default_rng(seed)
    ex = [h * (n - 1) for n, h in zip(case.vp.shape, case.h)]
    p = [rng.uniform(0.15, 0.85) * ex[0], rng.uniform(0.2, 0.8) * ex[1]]
    src = [p, p, [rng.uniform(0.1, 0.9) * ex[0], rng.uniform(0.1, 0.9) * ex[1]]]
    rec = []
    for zf in (0.1, 0.45, 0.8):  # three receiver rows
        for xf in np.linspace(0.05, 0.95, 9):
            rec.append([xf * ex[0], zf * ex[1]])
    return make_shot(case.h, ex, nt, case.dt, 15.0, src, rec)


def _launches(run, kind=0):
    """Launches of one kernel kind (0 forward stencil, 1 adjoint, 4 recompute) since profiling was enabled."""
    ms, n, b = ctypes.c_double(), ctypes.c_int64(), ctypes.c_double()
    run.ctx.check(run.ctx.lib.sw_profile_read(run.ctx.h, kind, ctypes.byref(ms), ctypes.byref(n),
                                              ctypes.byref(b)), "profile_read")
    return n.value


CASES = [  # nx, nz, halo, freetop, pair band selector (variant >> 11)
    (123, 97, 20, False, 0),
    (250, 61, 8, True, 1),
    (37, 40, 0, False, 2),
    (481, 130, 20, True, 4),
    (150, 50, 6, False, 6),
]


@pytest.mark.parametrize("nx,nz,halo,freetop,tzsel", CASES)
def test_two_step_forward_is_bitwise_one_step(sw, oracle, nx, nz, halo, freetop, tzsel):
    case = _case(nx, nz, halo, freetop, seed=nx + nz)
    shots = [_shot(case, 301, seed=k) for k in range(3)]
    shots[1].nt = 250  # a shorter record: the active set changes mid-run
    out = {}
    for v in (PAIR | tzsel << 11, 0):
        run = GpuRun(sw, case, variant=v)
        run.ctx.profile(True)
        out[v] = run.forward(shots)
        n = _launches(run)
        run.ctx.profile(False)
        run.close()
        if v == 0:
            assert n == 301
        else:
            assert n < 0.6 * 301, n  # steps were paired
    for a, b in zip(out[PAIR | tzsel << 11], out[0]):
        assert np.array_equal(a, b)
    ref = oracle_forward(oracle, sw, case, shots[0])
    assert rel_l2(out[0][0], ref) < 1e-5


@pytest.mark.parametrize("check_freq,bf16", [(1, 0), (10, 0), (7, 0), (10, 1), (6, 2)])
def test_two_step_gradient_is_bitwise_one_step(sw, check_freq, bf16):
    case = _case(203, 88, 12, True, seed=5)
    shots = [_shot(case, 240, seed=10 + k) for k in range(2)]
    shots[0].nt = 221
    obs_case = Case(vp=np.asfortranarray(case.vp * 1.04), h=case.h, dt=case.dt, halo=case.halo, freetop=case.freetop)
    obs_run = GpuRun(sw, obs_case)
    for s, o in zip(shots, obs_run.forward(shots)):
        s.observed = np.asfortranarray(o, dtype=np.float64)
    obs_run.close()
    out = {}
    for v in (PAIR, 0):
        run = GpuRun(sw, case, gradient=True, check_freq=check_freq, variant=v, bf16=bf16)
        run.ctx.profile(True)
        out[v] = run.gradient(shots)
        adj = _launches(run, 1)
        run.ctx.profile(False)
        run.close()
        if v == 0:
            assert adj == 240
        else:
            assert adj < 0.75 * 240, adj  # adjoint steps were paired
    g0, m0, t0 = out[PAIR]
    g1, m1, t1 = out[0]
    assert m0 == m1
    assert np.array_equal(g0, g1), rel_l2(g0, g1)
    for a, b in zip(t0, t1):
        assert np.array_equal(a, b)


def test_two_step_snapshots_are_bitwise_one_step(sw):
    case = _case(150, 70, 10, False, seed=9)
    shot = _shot(case, 200, seed=3)
    snaps = {}
    for v in (PAIR, 0):
        run = GpuRun(sw, case, variant=v)
        arr, keep, outs = run._structs([shot], False)
        buf = np.zeros((200 // 3) * case.vp.size, np.float32)
        ptrs = (ctypes.c_void_p * 1)(buf.ctypes.data)
        run.ctx.check(run.ctx.lib.sw_acoustic_forward_snapshots(run.h, 1, arr, 0, 3, ptrs), "snapshots")
        snaps[v] = (buf, outs[0])
        run.close()
    assert np.array_equal(snaps[PAIR][0], snaps[0][0])
    assert np.array_equal(snaps[PAIR][1], snaps[0][1])


def test_boundary_source_falls_back_to_one_step(sw, oracle):
    """A source on the outermost grid line keeps the one-step path (its node
    evolves through the 3-value ring of the injection kernel)."""
    case = _case(90, 60, 5, False, seed=2)
    ex = [h * (n - 1) for n, h in zip(case.vp.shape, case.h)]
    shot = make_shot(case.h, ex, 150, case.dt, 15.0, [[0.0, 0.5 * ex[1]]], [[0.5 * ex[0], 0.3 * ex[1]]])
    run = GpuRun(sw, case, variant=PAIR)
    run.ctx.profile(True)
    tr = run.forward([shot])[0]
    n = _launches(run)
    run.ctx.profile(False)
    run.close()
    assert n == 150
    assert rel_l2(tr, oracle_forward(oracle, sw, case, shot)) < 1e-5
