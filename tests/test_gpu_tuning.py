"""Per-kind band heights (sw_wavesim_set_band_heights) and the autotuner on
the GPU.  Every band height runs the same rounded arithmetic, so traces,
misfit and gradient must be bit-identical to the default configuration; the
autotuner, run on the same batch with gradient trials, must leave the
results unchanged too and report its per-kind choices."""
import numpy as np
import pytest

from cases import Case, GpuRun, make_shot, smooth_model, stable_dt

pytestmark = pytest.mark.gpu


def _setup(sw):
    vp = smooth_model((301, 140), 1500.0, 3000.0, 17)
    h = (6.0, 6.0)
    case = Case(vp=vp, h=h, dt=stable_dt(vp, h), halo=14, freetop=True)
    ex = [hh * (n - 1) for n, hh in zip(vp.shape, h)]
    rng = np.random.default_rng(4)
    shots = []
    for k in range(5):
        src = [[rng.uniform(0.1, 0.9) * ex[0], rng.uniform(0.1, 0.5) * ex[1]]]
        rec = [[x, 0.05 * ex[1]] for x in np.linspace(0.02, 0.98, 31) * ex[0]]
        shots.append(make_shot(h, ex, 180 - 13 * k, case.dt, 14.0, src, rec))
    obs_case = Case(vp=np.asfortranarray(vp * 1.03), h=h, dt=case.dt, halo=case.halo, freetop=True)
    run = GpuRun(sw, obs_case)
    for s, o in zip(shots, run.forward(shots)):
        s.observed = np.asfortranarray(o, dtype=np.float64)
    run.close()
    return case, shots


@pytest.mark.parametrize("bands", [(4, 16, 8), (16, 4, 32), (8, 8, 4)])
def test_band_heights_are_bitwise_default(sw, bands):
    case, shots = _setup(sw)
    out = {}
    for b in (bands, None):
        run = GpuRun(sw, case, gradient=True, check_freq=9)
        if b:
            run.ctx.check(run.ctx.lib.sw_wavesim_set_band_heights(run.h, *b), "set_band_heights")
        out[b] = run.gradient(shots)
        run.close()
    g0, m0, t0 = out[bands]
    g1, m1, t1 = out[None]
    assert m0 == m1
    assert np.array_equal(g0, g1)
    for a, b in zip(t0, t1):
        assert np.array_equal(a, b)


def test_band_heights_reject_bad_arguments(sw):
    case, _ = _setup(sw)
    run = GpuRun(sw, case, gradient=True, check_freq=9)
    lib = run.ctx.lib
    assert lib.sw_wavesim_set_band_heights(run.h, -1, 0, 0) != 0
    assert lib.sw_wavesim_set_band_heights(run.h, 0, 0, 5000) != 0
    assert lib.sw_wavesim_set_band_heights(None, 8, 8, 8) != 0
    assert lib.sw_wavesim_set_band_heights(run.h, 0, 0, 0) == 0
    run.close()


def test_autotuned_gradient_is_bitwise_default(sw):
    tune = __import__(sw.__name__ + ".tune", fromlist=["tune"])
    case, shots = _setup(sw)
    ref = GpuRun(sw, case, gradient=True, check_freq=9)
    g1, m1, t1 = ref.gradient(shots)
    ref.close()
    run = GpuRun(sw, case, gradient=True, check_freq=9)
    arr, keep, _ = run._structs(shots, True)
    n = case.vp.size
    gbuf = np.zeros(n, np.float64)
    mbuf = np.zeros(1, np.float64)
    r = tune.autotune(run.ctx, run.h, ("test", case.vp.shape, case.halo), arr, len(shots), 2,
                      gradient_out=(gbuf.ctypes.data, mbuf.ctypes.data), check_freq=9,
                      candidates=[(0, 4), (0, 8), (2, 8), (1024, 0)])
    assert [s.nt for s in arr] == [s.nt for s in shots]
    assert set(r["per_kind_ms"]) == {(0, 4), (0, 8), (2, 8), (1024, 0)}
    assert all(set(d) == {"forward", "recompute", "adjoint"} for d in r["per_kind_ms"].values())
    del keep  # the trial structs' buffers
    g0, m0, t0 = run.gradient(shots)
    run.close()
    assert m0 == m1
    assert np.array_equal(g0, g1)
    for a, b in zip(t0, t1):
        assert np.array_equal(a, b)
