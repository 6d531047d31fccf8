"""Snapshots of forward runs (RunParameters.snapevery): the fields the
reference's LinearSnapshotter keeps (src/utils/snapshotter.jl:1-41) -- p[it]
for the acoustic path, ucur and sigma for the elastic one -- against the FP64
oracle, through the C ABI (sw_*_forward_snapshots)."""
import ctypes

import numpy as np
import pytest

import oracle as O
from cases import GpuRun, make_shot, oracle_cpml, prepared, rel_l2, smooth_model, stable_dt, Case
from elastic_cases import GpuElastic, oracle_shot, cpml as el_cpml, small_case, sw

pytestmark = pytest.mark.gpu

TOL = 1e-5


def _acoustic_case(shape, h, halo):
    vp = smooth_model(shape, 1500.0, 3000.0, 11)
    return Case(vp=vp, h=(h,) * len(shape), dt=stable_dt(vp, (h,) * len(shape), 0.6), halo=halo, freetop=False)


@pytest.mark.parametrize("shape", [(120, 97), (40, 36, 34)])
def test_acoustic_snapshots_match_oracle(sw, oracle, shape):
    case = _acoustic_case(shape, 8.0, 6)
    ex = [case.h[d] * (shape[d] - 1) for d in range(len(shape))]
    src = [[0.4 * e for e in ex]]
    rec = [[0.6 * e for e in ex]]
    shot = make_shot(case.h, ex, 120, case.dt, 15.0, src, rec)
    run = GpuRun(sw, case)
    arr, keep, outs = run._structs([shot], False)
    snapevery = 25
    npts = int(np.prod(shape))
    buf = np.zeros((shot.nt // snapevery) * npts, np.float32)
    ptrs = (ctypes.c_void_p * 1)(buf.ctypes.data)
    run.ctx.check(run.ctx.lib.sw_acoustic_forward_snapshots(run.h, 1, arr, 0, snapevery, ptrs), "snapshots")
    run.close()
    si, ri, tf, _ = prepared(sw, case, shot)
    tr_ref, snaps_ref = O.acoustic_forward_snapshots(case.vp, case.h, case.dt, case.halo,
                                                     oracle_cpml(oracle, case, shot.f0), tf.astype(np.float64), si,
                                                     ri, snapevery)
    snaps = buf.reshape(-1, npts)
    assert snaps.shape[0] == snaps_ref.shape[0] == shot.nt // snapevery
    for q in range(snaps.shape[0]):
        ref = snaps_ref[q].reshape(-1, order="F")
        assert rel_l2(snaps[q], ref) < TOL, q
    assert rel_l2(outs[0], tr_ref) < TOL


def test_elastic_snapshots_match_oracle():
    case = small_case("mt", nt=200)
    shot = case.shots[0]
    ctx = sw._lib.Context(0)
    run = GpuElastic(ctx, case)
    structs, keep = run._structs([shot])
    snapevery = 40
    nx, nz = case.nx, case.nz
    B = (nx - 1) * nz + nx * (nz - 1) + 2 * nx * nz + (nx - 1) * (nz - 1)
    buf = np.zeros((shot.nt // snapevery) * B, np.float32)
    ptrs = (ctypes.c_void_p * 1)(buf.ctypes.data)
    ctx.check(ctx.lib.sw_elastic_forward_snapshots(run.h, 1, structs, 0, snapevery, ptrs), "snapshots")
    run.close()
    tr_ref, snaps_ref = O.elastic_forward_snapshots(case.lam, case.mu, case.rho, (case.h, case.h), case.dt, case.halo,
                                                    case.freetop, el_cpml(case, shot), oracle_shot(case, shot),
                                                    snapevery)
    snaps = buf.reshape(-1, B)
    for q in range(snaps.shape[0]):
        assert rel_l2(snaps[q], snaps_ref[q]) < TOL, q
    assert rel_l2(keep[0][0], tr_ref) < TOL
    ctx.close()
