"""Rebuilds the seeded cases stored in tests/golden/*.npz (made by
tests/golden/make_golden.py): the inputs as the test drivers' case and shot
objects, and the oracle's FP64 outputs."""
from __future__ import annotations

from pathlib import Path

import numpy as np

GOLDEN = Path(__file__).resolve().parent / "golden"


def _load(name):
    with np.load(GOLDEN / f"{name}.npz") as z:
        return {k: z[k] for k in z.files}


def acoustic_cd2d():
    """(Case, Shot with observed, check_freq, expected dict(traces, misfit, grad))."""
    from cases import Case, Shot
    d = _load("acoustic_cd2d")
    case = Case(vp=np.asfortranarray(d["vp"]), h=tuple(float(x) for x in d["h"]), dt=float(d["dt"]),
                halo=int(d["halo"]), freetop=bool(d["freetop"]), rcoef=float(d["rcoef"]))
    shot = Shot(src_pos=d["src_pos"], rec_pos=d["rec_pos"], tf=np.asfortranarray(d["tf"]), f0=float(d["f0"]),
                nt=int(d["nt"]), observed=np.asfortranarray(d["observed"]))
    return case, shot, int(d["check_freq"]), dict(traces=d["traces"], misfit=float(d["misfit"]), grad=d["grad_vp"])


def acoustic_vd2d():
    """(VDCase, VDShot, observed, check_freq, expected dict(traces, misfit, vp, rho))."""
    from vd_cases import VDCase, VDShot
    d = _load("acoustic_vd2d")
    shot = VDShot(d["src"], d["rec"], np.asfortranarray(d["tf"]), float(d["f0"]))
    case = VDCase(np.asfortranarray(d["vp"]), np.asfortranarray(d["rho"]), float(d["h"]), float(d["dt"]),
                  int(d["halo"]), freetop=bool(d["freetop"]), interp=int(d["interp"]), rcoef=float(d["rcoef"]),
                  shots=[shot])
    exp = dict(traces=d["traces"], misfit=float(d["misfit"]), vp=d["grad_vp"], rho=d["grad_rho"])
    return case, shot, np.asfortranarray(d["observed"]), int(d["check_freq"]), exp


def elastic2d():
    """(ElCase, ElShot, observed, check_freq, expected dict(traces, misfit, rho, lambda, mu))."""
    from elastic_cases import ElCase, ElShot
    d = _load("elastic2d")
    shot = ElShot("mt", d["src"], d["rec"], int(d["nt"]), float(d["f0"]),
                  momtens=[tuple(float(x) for x in row) for row in np.atleast_2d(d["momtens"])])
    case = ElCase(d["lam"].shape[0], d["lam"].shape[1], float(d["h"]), float(d["dt"]), int(d["halo"]),
                  np.asfortranarray(d["lam"]), np.asfortranarray(d["mu"]), np.asfortranarray(d["rho"]), [shot],
                  freetop=bool(d["freetop"]), sinc=bool(d["sinc"]), interp_rho=int(d["interp_rho"]),
                  interp_mu=int(d["interp_mu"]), rcoef=float(d["rcoef"]))
    exp = dict(traces=d["traces"], misfit=float(d["misfit"]), rho=d["grad_rho"], **{"lambda": d["grad_lambda"]},
               mu=d["grad_mu"])
    return case, shot, np.asfortranarray(d["observed"]), int(d["check_freq"]), exp
