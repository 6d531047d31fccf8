"""sw_acoustic2d_forward_noalloc against the regular forward entry point.

The no-allocation entry point serves callers that cannot let a library call
cudaMalloc (code living in another runtime's device memory pool, fixed
device-memory budgets, pipelines that cannot take the synchronisation an
allocation may impose): it keeps all of its working memory in a fixed 64 MiB
array inside the library.  It must give the same traces as sw_acoustic_forward
on two calls in a row (the second call starts from the first call's leftovers
in that shared array), and refuse grids that do not fit.  This file is
collected last so a failure here leaves every other test already run.
"""
import ctypes

import numpy as np
import pytest

from cases import Case, GpuRun, make_shot, prepared, rel_l2, smooth_model, stable_dt

pytestmark = pytest.mark.gpu

TRACE_TOL = 1e-5  # same bound as the forward parity tests


def _params(L, case, n=None):
    prm = L.SwAcousticParams()
    prm.ndim = 2
    for d in range(2):
        prm.n[d] = (n or case.vp.shape)[d]
        prm.h[d] = case.h[d]
    prm.dt, prm.halo, prm.rcoef, prm.freetop = case.dt, case.halo, case.rcoef, int(case.freetop)
    return prm


def _noalloc_case(kind):
    """Two layouts: damped grid with an interior source pair and a receiver on
    the free surface; and halo = 0 (no memory variables) with a source on the
    grid's outermost line, whose node keeps the 3-value ring in the shared
    array -- the state most exposed to a previous call's leftovers."""
    vp = smooth_model((203, 157), 1600.0, 3200.0, seed=21)
    if kind == "damped":
        case = Case(vp=vp, h=(6.0, 6.0), dt=stable_dt(vp, (6.0, 6.0)), halo=15, freetop=True)
    else:
        case = Case(vp=vp, h=(6.0, 6.0), dt=stable_dt(vp, (6.0, 6.0)), halo=0, freetop=False)
    ex = [h * (n - 1) for n, h in zip(vp.shape, case.h)]
    recx = np.linspace(0.05 * ex[0], 0.95 * ex[0], 23)
    rec = np.stack([recx, np.full_like(recx, 0.08 * ex[1])], 1)
    if kind == "damped":
        rec[0, 1] = 0.0  # one receiver on the free surface
        src = [[0.4 * ex[0], 0.3 * ex[1]], [0.4 * ex[0], 0.3 * ex[1]], [0.6 * ex[0], 0.5 * ex[1]]]
    else:
        src = [[0.0, 0.3 * ex[1]], [0.6 * ex[0], 0.5 * ex[1]]]  # first source on the line i = 1
        rec[1] = [0.0, 0.3 * ex[1]]  # a receiver on that boundary node
    shot = make_shot(case.h, ex, 700, case.dt, 12.0, src, rec)
    return case, shot


@pytest.mark.parametrize("kind", ["damped", "edge_source_no_halo"])
def test_noalloc_forward_matches_regular_entry_point(sw, kind):
    torch = pytest.importorskip("torch")
    L = sw._lib
    lib = L.load()
    case, shot = _noalloc_case(kind)
    vp = case.vp
    run = GpuRun(sw, case)
    ref = run.forward([shot])[0]
    run.close()

    si, ri, scal, cp = prepared(sw, case, shot)
    dev = torch.device("cuda", 0)
    vp_d = torch.from_numpy(np.ascontiguousarray(vp.ravel(order="F"), dtype=np.float32)).to(dev)
    tf_d = torch.from_numpy(np.ascontiguousarray(scal[: shot.nt].ravel(order="F"))).to(dev)
    tr_d = torch.empty(shot.nt * ri.shape[0], dtype=torch.float32, device=dev)
    prm = _params(L, case)
    st = L.SwAcousticShot()
    st.nt, st.nsrc, st.nrec = shot.nt, si.shape[0], ri.shape[0]
    st.src_idx, st.rec_idx, st.cpml = si.ctypes.data, ri.ctypes.data, cp.ctypes.data
    st.srctf, st.traces = tf_d.data_ptr(), tr_d.data_ptr()
    for call in range(2):
        tr_d.fill_(float("nan"))
        torch.cuda.synchronize(dev)
        rc = lib.sw_acoustic2d_forward_noalloc(ctypes.byref(prm), vp_d.data_ptr(), ctypes.byref(st), None)
        assert rc == L.SW_OK, f"call {call}: status {rc}"
        out = tr_d.cpu().numpy().reshape(ri.shape[0], shot.nt).T
        assert np.all(np.isfinite(out))
        assert rel_l2(out, ref) < TRACE_TOL, f"call {call}"


def test_noalloc_rejects_grids_beyond_its_scratch(sw):
    torch = pytest.importorskip("torch")
    L = sw._lib
    lib = L.load()
    vp = np.full((64, 64), 2000.0, order="F")
    case = Case(vp=vp, h=(5.0, 5.0), dt=1e-3, halo=5, freetop=False)
    prm = _params(L, case, n=(4000, 4000))  # 16 M points: four fields alone exceed 64 MiB
    si = np.array([[10, 10]], dtype=np.int32, order="F")
    ri = np.array([[20, 20]], dtype=np.int32, order="F")
    cp = np.zeros(2 * (4 * 5 + 4 + 4 * 5), np.float32)
    dev = torch.device("cuda", 0)
    vp_d = torch.zeros(16, dtype=torch.float32, device=dev)
    buf = torch.zeros(16, dtype=torch.float32, device=dev)
    st = L.SwAcousticShot()
    st.nt, st.nsrc, st.nrec = 10, 1, 1
    st.src_idx, st.rec_idx, st.cpml = si.ctypes.data, ri.ctypes.data, cp.ctypes.data
    st.srctf, st.traces = buf.data_ptr(), buf.data_ptr()
    rc = lib.sw_acoustic2d_forward_noalloc(ctypes.byref(prm), vp_d.data_ptr(), ctypes.byref(st), None)
    assert rc == L.SW_ERR_CAPACITY
