"""The seeded workload generators (seismicwaves.jl_gb300/configs.py) produce
the configurations the benchmark quotes: grid, spacing, C-PML width, record
lengths, receiver layouts, source frequency, checkpoint period, the CFL
fraction of the time step and the value ranges of the models."""
import inspect
import math

import numpy as np
import pytest

import __graft_entry__

sw = __graft_entry__.load_package()
C = __import__(sw.__name__ + ".configs", fromlist=["configs"])


def _cfl(vp, dt, h):
    return float(np.max(vp)) * dt * math.sqrt(sum(1.0 / x ** 2 for x in h))


def test_acoustic2d_201_forward_case():
    """201 x 201, 5 m, 2000 m/s plus a +300 m/s Gaussian (sigma 100 m) at the
    centre, 20-point C-PML, dt = 0.6 CFL, 1000 steps, 12 Hz source at
    (500, 25) m, 101 receivers every 10 m at 20 m depth."""
    w = C.acoustic2d_201()
    assert w.vp.shape == (201, 201) and w.h == (5.0, 5.0) and w.halo == 20 and not w.freetop
    assert w.vp.min() == pytest.approx(2000.0, abs=1e-3) and w.vp.max() == pytest.approx(2300.0)
    assert w.vp[100, 100] == pytest.approx(2300.0) and w.vp[100 + 20, 100] == pytest.approx(
        2000.0 + 300.0 * math.exp(-0.5), rel=1e-12)
    assert _cfl(w.vp, w.dt, w.h) == pytest.approx(0.6)
    (s,) = w.shots
    assert s.nt == 1000 and s.f0 == 12.0 and np.allclose(s.src_pos, [[500.0, 25.0]])
    assert s.rec_pos.shape == (101, 2) and np.allclose(s.rec_pos[:, 1], 20.0)
    assert np.allclose(np.diff(s.rec_pos[:, 0]), 10.0) and s.rec_pos[0, 0] == 0.0


def test_acoustic2d_801_gradient_case():
    """801 x 801, 5 m, 1500-3500 m/s (linear trend plus 8 seeded blobs), the
    observed data from 1.05 vp, 3000 steps, 10 Hz, 401 receivers, K = 50."""
    w = C.acoustic2d_801()
    assert w.vp.shape == (801, 801) and w.h == (5.0, 5.0) and w.halo == 20 and w.check_freq == 50
    assert 1500.0 <= w.vp.min() and w.vp.max() <= 3500.0
    np.testing.assert_allclose(w.vp_observed, 1.05 * w.vp)
    assert _cfl(w.vp, w.dt, w.h) == pytest.approx(0.6)
    (s,) = w.shots
    assert s.nt == 3000 and s.f0 == 10.0 and s.rec_pos.shape == (401, 2)


def test_acoustic2d_2001x801_batch():
    """2001 x 801, 10 m, 12 layers from 1500 to 4500 m/s with 3 % smoothed
    noise, 64 shots evenly spaced at 20 m depth, 50-300 receivers and
    2000-4000 steps per shot, 8 Hz, K = 50; observed data from a second noise
    realisation."""
    w = C.acoustic2d_2001x801()
    assert w.vp.shape == (2001, 801) and w.h == (10.0, 10.0) and w.halo == 20 and w.check_freq == 50
    assert len(w.shots) == 64
    assert all(50 <= s.rec_pos.shape[0] <= 300 and 2000 <= s.nt <= 4000 and s.f0 == 8.0 for s in w.shots)
    assert all(np.allclose(s.src_pos[:, 1], 20.0) and np.allclose(s.rec_pos[:, 1], 20.0) for s in w.shots)
    xs = np.array([s.src_pos[0, 0] for s in w.shots])
    assert np.allclose(np.diff(xs), np.diff(xs)[0])
    assert len({s.nt for s in w.shots}) > 32 and len({s.rec_pos.shape[0] for s in w.shots}) > 32
    assert 1400.0 <= w.vp.min() < 1600.0 and 4400.0 < w.vp.max() <= 4700.0
    assert not np.array_equal(w.vp, w.vp_observed)
    assert _cfl(np.maximum(w.vp, w.vp_observed), w.dt, w.h) == pytest.approx(0.6)


def test_acoustic3d_400_defaults_and_layout():
    """400^3, 10 m, 1800-4000 m/s smooth random model, 16 shots on a 4 x 4
    surface grid with a 40 x 40 receiver patch each, 2000 steps, 10 Hz, K = 100
    (the layout is checked on a 60^3 instance of the same generator)."""
    d = {k: v.default for k, v in inspect.signature(C.acoustic3d_400).parameters.items()}
    assert (d["n"], d["nshots_side"], d["patch"], d["nt"]) == (400, 4, 40, 2000)
    w = C.acoustic3d_400(n=60)
    assert w.vp.shape == (60, 60, 60) and w.h == (10.0, 10.0, 10.0) and w.halo == 20 and w.check_freq == 100
    assert w.vp.min() == pytest.approx(1800.0) and w.vp.max() == pytest.approx(4000.0)
    assert len(w.shots) == 16 and all(s.rec_pos.shape == (1600, 3) and s.f0 == 10.0 for s in w.shots)
    assert len({tuple(s.src_pos[0, :2]) for s in w.shots}) == 16


def test_elastic2d_1200x600_batch():
    """1200 x 600, 5 m, vp 2000-4500, vs = vp / sqrt(3) * (0.9-1.0), rho
    1800-2700 from seeded smooth fields, 32 explosive sources, 300 receivers,
    4000 steps, 15 Hz, K = 50, CFL 0.6 with the 7/6 factor of the 4th-order
    stencil."""
    w = C.elastic2d_1200x600()
    assert w.lam.shape == (1200, 600) and w.h == (5.0, 5.0) and w.halo == 20 and w.check_freq == 50
    vp = w.vp
    vs = np.sqrt(w.mu / w.rho)
    assert vp.min() == pytest.approx(2000.0) and vp.max() == pytest.approx(4500.0)
    r = vs / vp * math.sqrt(3.0)
    assert r.min() == pytest.approx(0.9) and r.max() == pytest.approx(1.0)
    assert w.rho.min() == pytest.approx(1800.0) and w.rho.max() == pytest.approx(2700.0)
    assert w.momtens == (1.0, 1.0, 0.0)
    assert len(w.shots) == 32 and all(s.rec_pos.shape == (300, 2) and s.nt == 4000 and s.f0 == 15.0
                                      for s in w.shots)
    lam_o, mu_o, rho_o = w.observed_model
    vmax = max(float(vp.max()), float(np.sqrt((lam_o + 2 * mu_o) / rho_o).max()))
    assert vmax * w.dt * math.sqrt(2.0 / 25.0) * 7 / 6 == pytest.approx(0.6)
