"""Host logic of the autotuner (tune.py) on the CPU, against a fake library:
every candidate is installed and timed on shots capped at `steps`, the
callers' record lengths come back afterwards (also when a trial fails), the
fastest candidate is installed last, and a second call for the same key
re-installs the cached choice without timing again."""
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
    choice, timings = T.autotune(_FakeCtx(lib), None, ("g",), shots, 3, 2, steps=24)
    assert choice == (512, 8)
    assert set(timings) == set(T.CANDIDATES_2D)
    assert lib.calls[-1] == ("set", 512, 8)
    assert all(nts == [24, 10, 24] for nts in lib.nts)  # trials run on capped records
    assert [s.nt for s in shots] == [3000, 10, 2500]
    # cached: the choice is installed again, nothing is timed
    n = len(lib.nts)
    again = T.autotune(_FakeCtx(lib), None, ("g",), shots, 3, 2)
    assert again[0] == (512, 8) and len(lib.nts) == n and lib.calls[-1] == ("set", 512, 8)


def test_autotune_3d_candidates(monkeypatch):
    lib = _FakeLib(fastest=(0, 32))
    monkeypatch.setattr(T.time, "perf_counter", lambda: lib.clock)
    choice, timings = T.autotune(_FakeCtx(lib), None, ("g3",), _shots([100]), 1, 3)
    assert choice == (0, 32) and set(timings) == set(T.CANDIDATES_3D)


def test_autotune_restores_nt_when_a_trial_fails(monkeypatch):
    lib = _FakeLib(fastest=(0, 4), fail_on=(2, 8))
    monkeypatch.setattr(T.time, "perf_counter", lambda: lib.clock)
    shots = _shots([900, 700])
    with pytest.raises(RuntimeError):
        T.autotune(_FakeCtx(lib), None, ("g",), shots, 2, 2, steps=16)
    assert [s.nt for s in shots] == [900, 700]
    assert T._cache == {}
