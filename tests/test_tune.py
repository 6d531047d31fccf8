"""Host logic of the autotuner (tune.py) on the CPU, against a fake library:
every candidate is installed and timed on shots capped at `steps`, the
callers' record lengths come back afterwards (also when a trial fails), the
fastest candidate is installed last, and a second call for the same key
re-installs the cached choice without timing again.  Gradient trials run
checkpointed gradients of 2 K + 2 steps and choose each stencil kind's band
height from that kind's own (fake) event timing."""
import ctypes

import pytest

import __graft_entry__

sw = __graft_entry__.load_package()
T = __import__(sw.__name__ + ".tune", fromlist=["tune"])


class _Shot(ctypes.Structure):
    _fields_ = [("nt", ctypes.c_int32)]


class _FakeLib:
    def __init__(self, fastest, fail_on=None):
        self.current = None
        self.calls = []
        self.fastest, self.fail_on = fastest, fail_on
        self.clock = 0.0
        self.nts = []

    def sw_wavesim_set_tuning(self, h, tz, v):
        self.current = (v, tz)
        self.calls.append(("set", v, tz))
        return 0

    def sw_wavesim_set_band_heights(self, h, f, r, a):
        self.bands = (f, r, a)
        self.calls.append(("bands", f, r, a))
        return 0

    def sw_acoustic_forward(self, h, n, shots, on_device):
        self.nts.append([shots[k].nt for k in range(n)])
        if self.current == self.fail_on:
            return 3
        self.clock += 1.0 if self.current == self.fastest else 2.0
        return 0


class _FakeCtx:
    def __init__(self, lib):
        self.lib = lib

    def check(self, rc, what):
        if rc != 0:
            raise RuntimeError(what)

    def profile(self, on):
        self.lib.prof_on = on

    def profile_read(self, kind):
        return self.lib.kind_ms[kind], 1, 0.0


class _GradLib(_FakeLib):
    """Gradient trials whose per-kind times depend on each kind's band height:
    forward fastest at 4 rows, recompute at 8, adjoint at 16; variant 2 is
    slower everywhere."""
    BEST = {0: 4, 4: 8, 1: 16}

    def __init__(self):
        super().__init__(fastest=None)
        self.bands = (0, 0, 0)
        self.kind_ms = {}
        self.prof_on = False

    def sw_acoustic_gradient(self, h, n, shots, on_device, g, m):
        self.nts.append([shots[k].nt for k in range(n)])
        v, tz = self.current
        self.kind_ms = {}
        for kind, slot in ((0, 0), (4, 1), (1, 2)):
            t = self.bands[slot] or tz or 8
            self.kind_ms[kind] = (1.0 if t == self.BEST[kind] else 1.5) * (2.0 if v == 2 else 1.0)
        self.clock += sum(self.kind_ms.values())
        return 0


@pytest.fixture(autouse=True)
def _fresh(monkeypatch):
    monkeypatch.setattr(T, "_cache", {})


def _shots(nts):
    arr = (_Shot * len(nts))()
    for k, nt in enumerate(nts):
        arr[k].nt = nt
    return arr


def test_autotune_picks_the_fastest_and_restores_nt(monkeypatch):
    lib = _FakeLib(fastest=(512, 8))
    monkeypatch.setattr(T.time, "perf_counter", lambda: lib.clock)
    shots = _shots([3000, 10, 2500])
    r = T.autotune(_FakeCtx(lib), None, ("g",), shots, 3, 2, steps=24)
    assert (r["variant"], r["tz"], r["band_heights"]) == (512, 8, None)
    assert set(r["trial_s"]) == set(T.CANDIDATES_2D)
    assert lib.calls[-2:] == [("set", 512, 8), ("bands", 0, 0, 0)]
    assert all(nts == [24, 10, 24] for nts in lib.nts)  # trials run on capped records
    assert [s.nt for s in shots] == [3000, 10, 2500]
    # cached: the choice is installed again, nothing is timed
    n = len(lib.nts)
    again = T.autotune(_FakeCtx(lib), None, ("g",), shots, 3, 2)
    assert again is r and len(lib.nts) == n and lib.calls[-2:] == [("set", 512, 8), ("bands", 0, 0, 0)]


def test_autotune_3d_candidates(monkeypatch):
    lib = _FakeLib(fastest=(0, 32))
    monkeypatch.setattr(T.time, "perf_counter", lambda: lib.clock)
    r = T.autotune(_FakeCtx(lib), None, ("g3",), _shots([100]), 1, 3)
    assert (r["variant"], r["tz"]) == (0, 32) and set(r["trial_s"]) == set(T.CANDIDATES_3D)


def test_autotune_restores_nt_when_a_trial_fails(monkeypatch):
    lib = _FakeLib(fastest=(0, 4), fail_on=(2, 8))
    monkeypatch.setattr(T.time, "perf_counter", lambda: lib.clock)
    shots = _shots([900, 700])
    with pytest.raises(RuntimeError):
        T.autotune(_FakeCtx(lib), None, ("g",), shots, 2, 2, steps=16)
    assert [s.nt for s in shots] == [900, 700]
    assert T._cache == {}


def test_autotune_gradient_picks_band_heights_per_kind(monkeypatch):
    lib = _GradLib()
    monkeypatch.setattr(T.time, "perf_counter", lambda: lib.clock)
    shots = _shots([3000, 1500])
    r = T.autotune(_FakeCtx(lib), None, ("gg",), shots, 2, 2, gradient_out=(0, 0), check_freq=20,
                   candidates=[(0, 4), (0, 8), (2, 8)])
    assert all(nts == [42, 42] for nts in lib.nts)  # 2 K + 2 steps
    assert [s.nt for s in shots] == [3000, 1500]
    assert r["variant"] == 0 and r["band_heights"] == (4, 8, 16) and r["tz"] == 0
    assert set(r["per_kind_ms"]) == {(0, 4), (0, 8), (2, 8)}
    assert set(r["band_ms"]) == set(T.TZ_KIND_2D)
    assert lib.calls[-2:] == [("set", 0, 0), ("bands", 4, 8, 16)]
    assert not lib.prof_on


def test_autotune_gradient_falls_back_to_forwards_on_short_records(monkeypatch):
    lib = _FakeLib(fastest=(0, 8))
    monkeypatch.setattr(T.time, "perf_counter", lambda: lib.clock)
    shots = _shots([30, 900])
    r = T.autotune(_FakeCtx(lib), None, ("gs",), shots, 2, 2, gradient_out=(0, 0), check_freq=50)
    assert r["variant"] == 0 and r["tz"] == 8 and r["band_heights"] is None and r["per_kind_ms"] == {}
    assert all(nts == [24, 24] for nts in lib.nts)
    assert [s.nt for s in shots] == [30, 900]
