"""Host logic of the reverse-mode rule (rrules.py) on the CPU: swgradient is
replaced by a fake that returns known fields, so the sign per physics, the
keys, the misfit fallback and the torch adapter are checked without a GPU."""
import numpy as np
import pytest

import __graft_entry__

sw = __graft_entry__.load_package()
R = __import__(sw.__name__ + ".rrules", fromlist=["rrules"])

SHAPE = (7, 5)


def _fields(seed, keys):
    rng = np.random.default_rng(seed)
    return {k: np.asfortranarray(rng.standard_normal(SHAPE)) for k in keys}


class _FakeMisfit:
    def __init__(self, value):
        self.value = value

    def calcmisfit(self, recs):
        return self.value


class _Shot:
    recs = None


def _install(monkeypatch, grads, chi, seen):
    def fake(params_or_wavesim, matprop, shots, misfit, *, runparams=None, gradparams=None):
        seen.append((matprop, gradparams))
        return (grads, chi) if chi is not None else grads
    monkeypatch.setattr(R._api, "swgradient", fake)


def _materials():
    base = 2000.0 + np.zeros(SHAPE)
    return {
        "cd": (sw.VpAcousticCDMaterialProperties(np.asfortranarray(base)), ["vp"], -1.0),
        "vd": (sw.VpRhoAcousticVDMaterialProperties(np.asfortranarray(base), np.asfortranarray(base + 300)),
               ["vp", "rho"], -1.0),
        "elastic": (sw.ElasticIsoMaterialProperties(np.asfortranarray(base * 1e6), np.asfortranarray(base * 5e5),
                                                    np.asfortranarray(base)), ["lambda", "mu", "rho"], 1.0),
    }


@pytest.mark.parametrize("kind", ["cd", "vd", "elastic"])
def test_pullback_sign_and_keys(monkeypatch, kind):
    matprop, keys, sign = _materials()[kind]
    grads = _fields(1, keys)
    seen = []
    _install(monkeypatch, grads, 3.25, seen)
    chi, pb = R.rrule_swmisfit(None, matprop, [_Shot()], [_FakeMisfit(0.0)])
    assert chi == 3.25
    assert seen[0][1].compute_misfit is True
    t = pb(2.0)
    assert list(t) == keys
    for k in keys:
        np.testing.assert_array_equal(t[k], sign * 2.0 * grads[k])


def test_misfit_summed_when_gradient_run_has_none(monkeypatch):
    matprop, keys, _ = _materials()["cd"]
    _install(monkeypatch, _fields(2, keys), None, [])
    chi, _ = R.rrule_swmisfit(None, matprop, [_Shot(), _Shot()], [_FakeMisfit(1.5), _FakeMisfit(0.25)])
    assert chi == 1.75


def test_missing_gradient_key_is_an_error(monkeypatch):
    matprop, _, _ = _materials()["vd"]
    _install(monkeypatch, _fields(3, ["vp"]), 1.0, [])
    with pytest.raises(KeyError):
        R.rrule_swmisfit(None, matprop, [_Shot()], [_FakeMisfit(0.0)])


def test_with_fields_replaces_by_key_and_checks_shapes():
    matprop, _, _ = _materials()["elastic"]
    new = np.ones(SHAPE)
    m2 = R.with_fields(matprop, {"mu": new})
    assert m2.μ.flags.f_contiguous and np.array_equal(m2.μ, new)
    assert m2.λ is matprop.λ and matprop.μ is not m2.μ
    with pytest.raises(ValueError):
        R.with_fields(matprop, {"mu": np.ones((3, 3))})
    with pytest.raises(KeyError):
        R.with_fields(matprop, {"vp": new})
    with pytest.raises(TypeError):
        R.material_fields(object())


@pytest.mark.parametrize("kind", ["cd", "vd", "elastic"])
@pytest.mark.parametrize("dtype", ["float64", "float32"])
def test_torch_function_backward(monkeypatch, kind, dtype):
    torch = pytest.importorskip("torch")
    matprop, keys, sign = _materials()[kind]
    grads = _fields(4, keys)
    seen = []
    _install(monkeypatch, grads, 0.5, seen)
    chi = R.misfit_function(None, matprop, [_Shot()], [_FakeMisfit(0.0)])
    td = getattr(torch, dtype)
    ts = {k: torch.tensor(np.asarray(getattr(matprop, a)) + 1.0, dtype=td, requires_grad=True)
          for k, a in R.material_fields(matprop)}
    y = chi(**ts)
    assert y.dtype == torch.float64 and float(y.detach()) == 0.5
    # the simulation saw the tensors' values, in the model's (Fortran) layout
    mp = seen[0][0]
    for k, a in R.material_fields(matprop):
        np.testing.assert_allclose(getattr(mp, a), np.asarray(getattr(matprop, a)) + 1.0)
        assert getattr(mp, a).flags.f_contiguous
    (3.0 * y).backward()
    for k in keys:
        assert ts[k].grad.dtype == td
        np.testing.assert_allclose(ts[k].grad.numpy(), (sign * 3.0 * grads[k]).astype(dtype), rtol=1e-6)


def test_torch_function_subset_of_fields(monkeypatch):
    torch = pytest.importorskip("torch")
    matprop, _, _ = _materials()["vd"]
    grads = _fields(5, ["vp", "rho"])
    seen = []
    _install(monkeypatch, grads, 1.0, seen)
    chi = R.misfit_function(None, matprop, [_Shot()], [_FakeMisfit(0.0)])
    rho = torch.tensor(np.asarray(matprop.rho), requires_grad=True)
    chi(rho=rho).backward()
    np.testing.assert_array_equal(rho.grad.numpy(), -grads["rho"])
    assert seen[0][0].vp is matprop.vp
    with pytest.raises(KeyError):
        chi(mu=rho)
    with pytest.raises(ValueError):
        chi()
