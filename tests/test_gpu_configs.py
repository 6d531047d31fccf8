"""Parity at the sizes of the benchmark configurations that the FP64 oracle
finishes in seconds to a minute: the 201 x 201 forward and the 801 x 801
forward + L2 misfit + adjoint gradient with checkpoint period 50."""
import numpy as np
import pytest

from cases import Case, GpuRun, Shot, oracle_forward, oracle_gradient, rel_l2

pytestmark = pytest.mark.gpu

TRACE_TOL = 1e-5     # traces, relative L2 against the FP64 oracle
MISFIT_TOL = 1e-6    # misfit, relative
GRAD_TOL = 1e-5      # gradient (FP32 checkpoints), relative L2


def _case(w):
    shots = [Shot(src_pos=s.src_pos, rec_pos=s.rec_pos, tf=np.asfortranarray(s.stf(w.dt)), f0=s.f0, nt=s.nt)
             for s in w.shots]
    return Case(vp=w.vp, h=w.h, dt=w.dt, halo=w.halo, freetop=w.freetop, shots=shots)


def test_acoustic2d_201_forward(sw, oracle):
    from seismicwaves_gb300 import configs
    case = _case(configs.acoustic2d_201())
    run = GpuRun(sw, case)
    tr = run.forward(case.shots)[0]
    run.close()
    assert rel_l2(tr, oracle_forward(oracle, sw, case, case.shots[0])) < TRACE_TOL


def test_acoustic2d_801_gradient(sw, oracle):
    from seismicwaves_gb300 import configs
    w = configs.acoustic2d_801()
    case = _case(w)
    shot = case.shots[0]
    obs_case = Case(vp=w.vp_observed, h=w.h, dt=w.dt, halo=w.halo, freetop=w.freetop)
    shot.observed = oracle_forward(oracle, sw, obs_case, shot)
    run = GpuRun(sw, case, gradient=True, check_freq=w.check_freq)
    g, msf, tr = run.gradient([shot])
    run.close()
    gref, mref, tref = oracle_gradient(oracle, sw, case, shot, check_freq=w.check_freq)
    errs = (rel_l2(tr[0], tref), abs(msf - mref) / mref, rel_l2(g, gref))
    print(f"acoustic2d_801: traces {errs[0]:.3e}  misfit {errs[1]:.3e}  gradient {errs[2]:.3e}")
    assert errs[0] < TRACE_TOL
    assert errs[1] < MISFIT_TOL
    assert errs[2] < GRAD_TOL
