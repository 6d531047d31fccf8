"""The 2D one-step stencil with its x strips split off (the default:
k_ac2d_step with XS, whose main blocks leave the 4-point lane groups that
meet an x strip to extra blocks at the end of the launch, one group per
thread) against the single path (tuning variant bit 18).  Every point is
advanced exactly once with the same arithmetic, so traces, misfit and
gradient must be bit-identical: grids whose x strips end inside a lane group
(odd nx, halo not a multiple of 4), no strips, strips that leave a single
interior group, checkpointing (K > 1), BF16 recompute buffers, the per-shot
Kahan adjoint (muting) and sources and receivers inside the strips."""
import numpy as np
import pytest

from cases import Case, GpuRun, make_shot, oracle_forward, rel_l2, smooth_model, stable_dt

pytestmark = pytest.mark.gpu

UNSPLIT = 262144

CASES = [  # nx, nz, halo, freetop
    (157, 90, 12, True),
    (201, 75, 5, False),
    (130, 60, 0, False),
    (61, 40, 7, True),
    (45, 45, 20, False),  # one interior lane group between the strips
]


def _case(nx, nz, halo, freetop, seed):
    vp = smooth_model((nx, nz), 1700.0, 3200.0, seed)
    h = (9.0, 8.0)
    return Case(vp=vp, h=h, dt=stable_dt(vp, h), halo=halo, freetop=freetop)


def _shots(case, nt, k=3):
    ex = [hh * (n - 1) for n, hh in zip(case.vp.shape, case.h)]
    rng = np.random.default_rng(11)
    out = []
    for i in range(k):
        srcs = [[rng.uniform(0.3, 0.7) * ex[0], rng.uniform(0.2, 0.6) * ex[1]]]
        if i == 0:  # a source inside the left x strip (two grid points from the edge)
            srcs.append([2 * case.h[0], 0.5 * ex[1]])
        rec = [[x, 0.1 * ex[1]] for x in np.linspace(0.0, 1.0, 17) * ex[0]]
        out.append(make_shot(case.h, ex, nt - 7 * i, case.dt, 16.0, srcs, rec))
    return out


@pytest.mark.parametrize("nx,nz,halo,freetop", CASES)
def test_xsplit_forward_is_bitwise_single_launch(sw, oracle, nx, nz, halo, freetop):
    case = _case(nx, nz, halo, freetop, seed=nx + nz)
    shots = _shots(case, 120)
    out = {}
    for v in (0, UNSPLIT):
        run = GpuRun(sw, case, variant=v)
        out[v] = run.forward(shots)
        run.close()
    for a, b in zip(out[0], out[UNSPLIT]):
        assert np.array_equal(a, b)
    assert rel_l2(out[0][1], oracle_forward(oracle, sw, case, shots[1])) < 1e-5


@pytest.mark.parametrize("nx,nz,halo,freetop,bf16,mute", [
    (157, 90, 12, True, 0, 0),
    (201, 75, 5, False, 1, 0),
    (61, 40, 7, True, 0, 3),
    (45, 45, 20, False, 0, 0),
])
def test_xsplit_gradient_is_bitwise_single_launch(sw, nx, nz, halo, freetop, bf16, mute):
    case = _case(nx, nz, halo, freetop, seed=3 * nx)
    shots = _shots(case, 110)
    obs_case = Case(vp=np.asfortranarray(case.vp * 1.03), h=case.h, dt=case.dt, halo=case.halo, freetop=freetop)
    run = GpuRun(sw, obs_case)
    for s, o in zip(shots, run.forward(shots)):
        s.observed = np.asfortranarray(o, dtype=np.float64)
    run.close()
    out = {}
    for v in (0, UNSPLIT):
        run = GpuRun(sw, case, gradient=True, check_freq=7, variant=v, bf16=bf16, mute_src=mute)
        out[v] = run.gradient(shots)
        run.close()
    (g0, m0, t0), (g1, m1, t1) = out[0], out[UNSPLIT]
    assert m0 == m1 and np.array_equal(g0, g1)
    assert all(np.array_equal(a, b) for a, b in zip(t0, t1))
