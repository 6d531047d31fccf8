"""The 3D step as three launches (rows outside the y / z C-PML strips, the z
slabs, the y slabs: k_ac3d_inner / k_ac3d_inner_np, k_ac3d_zslab, k_ac3d_yslab; the default)
against the single-launch kernels (tuning variant bit 16).  Every point is
computed by exactly one launch with the same arithmetic, so traces, misfit
and gradient must be bit-identical, for the pipelined and unpipelined inner
kernel (bit 17), 4 and 8 rows per block (variant 2), the shallowest grid a
halo allows (three inner rows), halo 0 (no strips) and BF16 recompute
buffers."""
import numpy as np
import pytest

from cases import Case, GpuRun, make_shot, oracle_forward, rel_l2, smooth_model, stable_dt

pytestmark = pytest.mark.gpu

SINGLE, NOPIPE = 65536, 131072


def _case(shape, halo, freetop, seed):
    vp = smooth_model(shape, 1700.0, 3100.0, seed)
    h = (9.0, 8.0, 7.0)
    return Case(vp=vp, h=h, dt=stable_dt(vp, h), halo=halo, freetop=freetop)


def _shots(case, nt, k=2):
    ex = [hh * (n - 1) for n, hh in zip(case.vp.shape, case.h)]
    rng = np.random.default_rng(7)
    out = []
    for i in range(k):
        src = [[rng.uniform(0.2, 0.8) * ex[0], rng.uniform(0.2, 0.8) * ex[1], rng.uniform(0.1, 0.6) * ex[2]]]
        rec = [[x, y, 0.1 * ex[2]] for x in np.linspace(0.05, 0.95, 6) * ex[0] for y in (0.3 * ex[1], 0.7 * ex[1])]
        out.append(make_shot(case.h, ex, nt - 9 * i, case.dt, 18.0, src, rec))
    return out


CASES = [  # shape, halo, freetop
    ((70, 50, 45), 6, True),
    ((61, 40, 33), 5, False),
    ((50, 36, 15), 6, True),   # the smallest depth for this halo: three inner rows
    ((40, 30, 28), 0, False),  # no strips: the slab launches cover nothing
]


@pytest.mark.parametrize("shape,halo,freetop", CASES)
def test_split_forward_is_bitwise_single_launch(sw, oracle, shape, halo, freetop):
    case = _case(shape, halo, freetop, seed=sum(shape))
    shots = _shots(case, 80)
    out = {}
    for v in (0, NOPIPE, 2, 2 | NOPIPE, SINGLE):
        run = GpuRun(sw, case, variant=v)
        out[v] = run.forward(shots)
        run.close()
    for v in (NOPIPE, 2, 2 | NOPIPE, SINGLE):
        for a, b in zip(out[v], out[0]):
            assert np.array_equal(a, b), v
    assert rel_l2(out[0][0], oracle_forward(oracle, sw, case, shots[0])) < 1e-5


@pytest.mark.parametrize("bf16", [0, 1])
def test_split_gradient_is_bitwise_single_launch(sw, bf16):
    case = _case((58, 44, 40), 5, True, seed=3)
    shots = _shots(case, 90)
    obs_case = Case(vp=np.asfortranarray(case.vp * 1.03), h=case.h, dt=case.dt, halo=case.halo, freetop=True)
    run = GpuRun(sw, obs_case)
    for s, o in zip(shots, run.forward(shots)):
        s.observed = np.asfortranarray(o, dtype=np.float64)
    run.close()
    out = {}
    for v in (0, NOPIPE, SINGLE):
        run = GpuRun(sw, case, gradient=True, check_freq=7, variant=v, bf16=bf16)
        out[v] = run.gradient(shots)
        run.close()
    g0, m0, t0 = out[SINGLE]
    for v in (0, NOPIPE):
        g, m, t = out[v]
        assert m == m0 and np.array_equal(g, g0), v
        assert all(np.array_equal(a, b) for a, b in zip(t, t0))
