"""Reverse-mode rule for the misfit of a simulation: the ChainRulesCore
``rrule(swmisfit!, ...)`` that the GB300 extension adds around ``swgradient!``
(SeismicWaves.jl itself defines no AD rules), and the same rule as a
``torch.autograd.Function``.

One ``swgradient`` call (src/apis/gradient.jl:31-136) gives both the misfit
and the adjoint gradient; the pullback only scales the stored gradient.

Sign.  ``swgradient`` returns the reference's gradients as they are.  Central
differences of the misfit show that these are

  * ``-dchi/dm`` on the acoustic paths: ``dchi/du = C^-1 r``
    (L2Misfit.jl:64-77) is negated into the adjoint source
    (``adjointsource = .-dchi_du``, acou_gradient.jl:48 and :142), and the chain rules ``2/vp^3`` (acou_gradient.jl:4-95)
    and ``-2/(vp^3 rho)``, ``-1/(vp^2 rho^2)`` (acou_gradient.jl:146-201) keep
    that sign -- the returned field is a descent direction;
  * ``+dchi/dm`` on the elastic path (ela_gradient.jl:4-187), whose correlation
    kernels (correlate_gradient_xPU.jl:1-83) carry the opposite sign.

A pullback must return the derivative itself, so it multiplies by the sign of
the physics (``GRADIENT_SIGN``): the tangent of ``vp`` on the acoustic paths is
``-dchi * swgradient(...)["vp"]``.
"""
from __future__ import annotations

import copy
import dataclasses
from typing import Callable, Sequence

import numpy as np

from . import api as _api

GRADIENT_SIGN = {"acoustic": -1.0, "elastic": 1.0}


def _physics(matprop) -> str:
    from . import elastic as E
    return "elastic" if isinstance(matprop, E.ElasticIsoMaterialProperties) else "acoustic"


def material_fields(matprop) -> list[tuple[str, str]]:
    """(gradient key, material attribute) pairs of the differentiable fields of ``matprop``, in the order
    of the reference's gradient dictionaries."""
    from . import elastic as E
    from . import vd as V
    if isinstance(matprop, E.ElasticIsoMaterialProperties):
        return [("lambda", "λ"), ("mu", "μ"), ("rho", "ρ")]
    if isinstance(matprop, V.VpRhoAcousticVDMaterialProperties):
        return [("vp", "vp"), ("rho", "rho")]
    if isinstance(matprop, _api.VpAcousticCDMaterialProperties):
        return [("vp", "vp")]
    raise TypeError(f"no reverse rule for material properties of type {type(matprop).__name__}")


def rrule_swmisfit(params_or_wavesim, matprop, shots: Sequence, misfit: Sequence, *,
                   runparams: _api.RunParameters | None = None,
                   gradparams: _api.GradParameters | None = None) -> tuple[float, Callable]:
    """``rrule(swmisfit!, params_or_wavesim, matprop, shots, misfit)``: returns the summed misfit chi and
    ``pullback(dchi) -> {key: dchi * dchi/dm}`` keyed like ``swgradient``'s dictionary.

    A prebuilt wavesim must have been built with ``gradient=True``; when its GradParameters do not ask for
    the misfit, chi is summed from the misfit objects over the seismograms the gradient run recorded
    (``run_swmisfit!``, src/apis/misfit.jl:85-104).
    """
    gp = dataclasses.replace(gradparams or _api.GradParameters(), compute_misfit=True)
    out = _api.swgradient(params_or_wavesim, matprop, shots, misfit, runparams=runparams, gradparams=gp)
    if isinstance(out, tuple):
        grads, chi = out
    else:
        grads = out
        chi = float(sum(m.calcmisfit(s.recs) for s, m in zip(shots, misfit)))
    sign = GRADIENT_SIGN[_physics(matprop)]
    keys = [k for k, _ in material_fields(matprop)]
    missing = [k for k in keys if k not in grads]
    if missing:
        raise KeyError(f"swgradient returned no gradient for {missing}")
    derivs = {k: sign * np.asarray(grads[k], dtype=np.float64) for k in keys}

    def pullback(dchi):
        d = float(dchi)
        return {k: d * v for k, v in derivs.items()}

    return float(chi), pullback


def with_fields(matprop, values: dict):
    """Copy of ``matprop`` with the differentiable fields named by gradient key replaced by ``values``
    (Fortran-ordered float64 arrays of the model's shape)."""
    attrs = dict(material_fields(matprop))
    unknown = set(values) - set(attrs)
    if unknown:
        raise KeyError(f"{type(matprop).__name__} has no differentiable fields {sorted(unknown)}")
    out = copy.copy(matprop)
    for k, v in values.items():
        ref = np.asarray(getattr(matprop, attrs[k]))
        arr = np.asfortranarray(np.asarray(v, dtype=np.float64))
        if arr.shape != ref.shape:
            raise ValueError(f"{k}: shape {arr.shape} does not match the model's {ref.shape}")
        setattr(out, attrs[k], arr)
    return out


def misfit_function(params_or_wavesim, matprop, shots: Sequence, misfit: Sequence, *,
                    runparams: _api.RunParameters | None = None,
                    gradparams: _api.GradParameters | None = None):
    """The misfit as a differentiable torch function of the material fields.

    Returns ``chi(**fields) -> 0-d float64 tensor``; each keyword (a gradient key of ``matprop``: "vp",
    "rho", "lambda", "mu") takes a tensor of the model's shape, the fields not given keep ``matprop``'s
    values, and ``chi(...).backward()`` leaves ``dchi/dm`` in the tensors' ``.grad``.  Every call runs one
    ``swgradient`` on the GPU.
    """
    import torch

    class _SWMisfit(torch.autograd.Function):
        @staticmethod
        def forward(ctx, keys, *tensors):
            values = {k: t.detach().to("cpu", torch.float64).numpy() for k, t in zip(keys, tensors)}
            chi, pullback = rrule_swmisfit(params_or_wavesim, with_fields(matprop, values), shots, misfit,
                                           runparams=runparams, gradparams=gradparams)
            tang = pullback(1.0)
            ctx.save_for_backward(*[torch.from_numpy(np.ascontiguousarray(tang[k])).to(t)
                                    for k, t in zip(keys, tensors)])
            return torch.tensor(chi, dtype=torch.float64, device=tensors[0].device)

        @staticmethod
        def backward(ctx, dchi):
            return (None,) + tuple(dchi.to(t) * t for t in ctx.saved_tensors)

    keys_all = [k for k, _ in material_fields(matprop)]

    def chi(**fields):
        if not fields:
            raise ValueError(f"give at least one of {keys_all}")
        keys = tuple(k for k in keys_all if k in fields)
        unknown = set(fields) - set(keys_all)
        if unknown:
            raise KeyError(f"{type(matprop).__name__} has no differentiable fields {sorted(unknown)}")
        return _SWMisfit.apply(keys, *[fields[k] for k in keys])

    return chi
