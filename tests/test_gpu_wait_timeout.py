"""Bounded device-side waits of the TMA-pipelined stencil (variant 1).

The library's test hook (sw_wavesim_set_wait_test) makes the producer warp of
each launch's first block stop before one stage of its row pipeline, so the
consumer warps' mbarrier wait on that stage can never complete.  With a short
wait limit (2e7 cycles, about 10 ms) the consumers give up, raise the
context's error flag and leave -- no copy is in flight then, since they have
consumed every stage issued before the withheld one -- and the call returns
SW_ERR_TIMEOUT.  The context stays usable: with the hook off the same
simulation gives the same traces as before, bit for bit.  The grid is small
(6 blocks per launch, one resident wave) and the record short (40 steps),
so the whole test waits under a second on the device."""
import numpy as np
import pytest

from cases import Case, GpuRun, make_shot, smooth_model, stable_dt

pytestmark = pytest.mark.gpu

SW_ERR_TIMEOUT = 4


def test_tma_wait_gives_up_and_context_recovers(sw):
    vp = smooth_model((600, 40), 1500.0, 2800.0, 3)
    h = (5.0, 5.0)
    case = Case(vp=vp, h=h, dt=stable_dt(vp, h), halo=8, freetop=False)
    ex = [hh * (n - 1) for n, hh in zip(vp.shape, h)]
    shot = make_shot(h, ex, 40, case.dt, 20.0, [[0.5 * ex[0], 0.5 * ex[1]]],
                     [[x, 0.5 * ex[1]] for x in np.linspace(0.4, 0.6, 7) * ex[0]])
    run = GpuRun(sw, case, variant=1, tz=16)  # 2 x 3 blocks of 512 x 16 points per launch
    lib = run.ctx.lib
    before = run.forward([shot])[0]
    run.ctx.check(lib.sw_wavesim_set_wait_test(run.h, 20_000_000, 3), "set_wait_test")
    with pytest.raises(sw._lib.SwError) as e:
        run.forward([shot])
    assert e.value.code == SW_ERR_TIMEOUT
    run.ctx.check(lib.sw_wavesim_set_wait_test(run.h, 4_000_000_000, -1), "set_wait_test")
    after = run.forward([shot])[0]
    run.close()
    assert np.array_equal(after, before)
    assert np.abs(before).max() > 0


def test_wait_test_rejects_bad_arguments(sw):
    vp = smooth_model((64, 40), 1500.0, 2800.0, 3)
    case = Case(vp=vp, h=(5.0, 5.0), dt=stable_dt(vp, (5.0, 5.0)), halo=4, freetop=False)
    run = GpuRun(sw, case)
    lib = run.ctx.lib
    assert lib.sw_wavesim_set_wait_test(run.h, 10, -1) != 0
    assert lib.sw_wavesim_set_wait_test(run.h, 20_000_000, -2) != 0
    assert lib.sw_wavesim_set_wait_test(None, 20_000_000, -1) != 0
    run.close()
