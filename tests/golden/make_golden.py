"""Generates the golden fixtures in tests/golden/ with the FP64 oracle.

Run from the repository root:  python tests/golden/make_golden.py

Each .npz file holds one seeded case: every input that the library and the
oracle take, and the oracle's FP64 outputs (traces, misfit, gradients).
tests/test_golden.py re-runs the oracle on the stored inputs (CPU: it pins the
oracle against regressions); tests/test_gpu_golden.py runs libswgb300 on them
and compares with the stored outputs, without running the oracle.

SeismicWaves.jl ships no golden vectors and cannot run here (it is a Julia
package), so these outputs come from the oracle, which is itself pinned by
the reference's known-answer tests (tests/test_oracle_*.py).
"""
from __future__ import annotations

import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
sys.path.insert(0, str(HERE.parent))
sys.path.insert(0, str(HERE.parents[1]))


def acoustic_cd2d():
    import oracle
    import __graft_entry__
    from cases import Case, make_shot, oracle_forward, oracle_gradient, smooth_model, stable_dt
    sw = __graft_entry__.load_package()
    vp = smooth_model((81, 71), 1500.0, 3000.0, seed=11)
    h = (8.0, 8.0)
    case = Case(vp=vp, h=h, dt=stable_dt(vp, h, 0.6), halo=10, freetop=True)
    ex = [hh * (n - 1) for n, hh in zip(vp.shape, h)]
    recx = np.linspace(0.1 * ex[0], 0.9 * ex[0], 7)
    shot = make_shot(h, ex, 300, case.dt, 14.0, [[0.4 * ex[0], 0.3 * ex[1]]],
                     np.stack([recx, np.full_like(recx, 0.2 * ex[1])], 1))
    pert = Case(vp=np.asfortranarray(vp * 1.05), h=h, dt=case.dt, halo=case.halo, freetop=case.freetop)
    shot.observed = oracle_forward(oracle, sw, pert, shot)
    g, m, tr = oracle_gradient(oracle, sw, case, shot, check_freq=9)
    return dict(vp=vp, h=np.array(h), dt=case.dt, halo=case.halo, freetop=int(case.freetop), rcoef=case.rcoef,
                src_pos=shot.src_pos, rec_pos=shot.rec_pos, tf=shot.tf, f0=shot.f0, nt=shot.nt, check_freq=9,
                observed=shot.observed, traces=tr, misfit=m, grad_vp=g)


def acoustic_vd2d():
    from vd_cases import VDCase, oracle_forward, oracle_gradient, small_case
    case = small_case(nt=300, seed=5, interp=1, freetop=True, nx=70, nz=60, halo=8)
    shot = case.shots[0]
    pert = VDCase(np.asfortranarray(case.vp * 1.05), np.asfortranarray(case.rho * 0.97), case.h, case.dt,
                  case.halo, freetop=case.freetop, interp=case.interp, shots=[shot])
    obs = oracle_forward(pert, shot)
    g, m, tr = oracle_gradient(case, shot, obs, check_freq=7)
    return dict(vp=case.vp, rho=case.rho, h=case.h, dt=case.dt, halo=case.halo, freetop=int(case.freetop),
                interp=case.interp, rcoef=case.rcoef, src=shot.src, rec=shot.rec, tf=shot.tf, f0=shot.f0,
                check_freq=7, observed=obs, traces=tr, misfit=m, grad_vp=g["vp"], grad_rho=g["rho"])


def elastic2d():
    import copy
    from elastic_cases import oracle_forward, oracle_gradient, small_case
    case = small_case("mt", freetop=True, nt=300, nx=70, nz=60, halo=8)
    shot = case.shots[0]
    pert = copy.deepcopy(case)
    pert.lam, pert.mu, pert.rho = case.lam * 1.3, case.mu * 0.88, case.rho * 0.92
    obs = oracle_forward(pert, shot)
    g, m, tr = oracle_gradient(case, shot, obs, check_freq=7)
    return dict(lam=case.lam, mu=case.mu, rho=case.rho, h=case.h, dt=case.dt, halo=case.halo,
                freetop=int(case.freetop), sinc=int(case.sinc), interp_rho=case.interp_rho,
                interp_mu=case.interp_mu, rcoef=case.rcoef, src=shot.src, rec=shot.rec, nt=shot.nt, f0=shot.f0,
                momtens=np.array(shot.momtens, dtype=np.float64), check_freq=7, observed=obs, traces=tr,
                misfit=m, grad_rho=g["rho"], grad_lambda=g["lambda"], grad_mu=g["mu"])


CASES = {"acoustic_cd2d": acoustic_cd2d, "acoustic_vd2d": acoustic_vd2d, "elastic2d": elastic2d}


def main():
    for name, fn in CASES.items():
        d = fn()
        np.savez_compressed(HERE / f"{name}.npz", **{k: np.asarray(v) for k, v in d.items()})
        print(f"{name}.npz: misfit {float(d['misfit']):.6e}")


if __name__ == "__main__":
    main()
