"""ctypes binding of libswgb300.so (the C ABI of include/swgb300.h).

The shared library is built in-tree (``build.py``).  Loading fails loudly when
it is missing: there is no CPU fallback behind this module.
"""
from __future__ import annotations

import ctypes
from pathlib import Path

HERE = Path(__file__).resolve().parent
LIB_PATH = HERE / "libswgb300.so"

(SW_OK, SW_ERR_ARG, SW_ERR_OOM, SW_ERR_CUDA, SW_ERR_TIMEOUT, SW_ERR_STATE, SW_ERR_UNSUPPORTED,
 SW_ERR_CAPACITY) = range(8)
STATUS_NAMES = {
    SW_ERR_ARG: "SW_ERR_ARG", SW_ERR_OOM: "SW_ERR_OOM", SW_ERR_CUDA: "SW_ERR_CUDA",
    SW_ERR_TIMEOUT: "SW_ERR_TIMEOUT", SW_ERR_STATE: "SW_ERR_STATE", SW_ERR_UNSUPPORTED: "SW_ERR_UNSUPPORTED",
    SW_ERR_CAPACITY: "SW_ERR_CAPACITY",
}

# Every function declared in include/swgb300.h (checked by the test-suite).
EXPORTS = [
    "sw_version", "sw_ctx_create", "sw_ctx_destroy", "sw_ctx_last_error", "sw_ctx_stream",
    "sw_cpml_coefficients", "sw_cpml_coefficients64", "sw_wavesim_create", "sw_wavesim_destroy", "sw_wavesim_set_vp",
    "sw_acoustic_forward", "sw_acoustic_gradient", "sw_wavesim_set_tuning", "sw_wavesim_set_band_heights",
    "sw_wavesim_set_precision", "sw_wavesim_set_vp64",
    "sw_wavesim_set_wait_test",
    "sw_profile_enable",
    "sw_profile_read", "sw_profile_read_kernels", "sw_acoustic2d_forward_noalloc", "sw_elastic_create", "sw_elastic_destroy",
    "sw_elastic_set_material", "sw_elastic_forward", "sw_elastic_gradient", "sw_elastic_set_tuning",
    "sw_wavesim_use_graphs", "sw_acoustic_forward_snapshots", "sw_elastic_forward_snapshots",
    "sw_acoustic_vd_create", "sw_acoustic_vd_destroy", "sw_acoustic_vd_set_material", "sw_acoustic_vd_forward",
    "sw_acoustic_vd_forward_snapshots", "sw_acoustic_vd_gradient", "sw_acoustic_vd_set_tuning",
    "sw_acoustic_vd_set_precision", "sw_acoustic_vd_set_material64",
]

i32, f64, vp_ = ctypes.c_int32, ctypes.c_double, ctypes.c_void_p


class SwAcousticParams(ctypes.Structure):
    _fields_ = [("ndim", i32), ("n", i32 * 3), ("h", f64 * 3), ("dt", f64), ("halo", i32),
                ("rcoef", f64), ("freetop", i32)]


class SwAcousticShot(ctypes.Structure):
    _fields_ = [("nt", i32), ("nsrc", i32), ("src_idx", vp_), ("srctf", vp_), ("nrec", i32),
                ("rec_idx", vp_), ("traces", vp_), ("cpml", vp_), ("observed", vp_),
                ("invcov_diag", vp_), ("nwin", i32), ("windows", vp_), ("src_pos", vp_), ("rec_pos", vp_),
                ("invcov", vp_), ("misfit_kind", i32), ("misfit_dt", f64), ("cpml64", vp_)]


class SwGradParams(ctypes.Structure):
    _fields_ = [("check_freq", i32), ("mute_radius_src", i32), ("mute_radius_rec", i32),
                ("compute_misfit", i32), ("snapshot_bf16", i32)]


class SwElasticParams(ctypes.Structure):
    _fields_ = [("n", i32 * 2), ("h", f64 * 2), ("dt", f64), ("halo", i32), ("rcoef", f64), ("freetop", i32),
                ("interp_rho", i32), ("interp_mu", i32)]


class SwPointTable(ctypes.Structure):
    _fields_ = [("offsets", vp_), ("ij", vp_), ("coef", vp_)]


class SwElasticShot(ctypes.Structure):
    _fields_ = [("nt", i32), ("kind", i32), ("nsrc", i32), ("srctf", vp_), ("momtens", vp_),
                ("src", SwPointTable * 2), ("nrec", i32), ("rec", SwPointTable * 2), ("traces", vp_),
                ("cpml", vp_), ("observed", vp_), ("invcov_diag", vp_), ("nwin", i32), ("windows", vp_),
                ("src_pos", vp_), ("rec_pos", vp_), ("invcov", vp_), ("misfit_kind", i32), ("misfit_dt", f64)]


class SwError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"{STATUS_NAMES.get(code, code)}: {msg}")
        self.code = code
        self.msg = msg


_lib = None


def load() -> ctypes.CDLL:
    """Load libswgb300.so (raises if it has not been built)."""
    global _lib
    if _lib is not None:
        return _lib
    if not LIB_PATH.exists():
        raise RuntimeError(f"{LIB_PATH} is missing: build it with seismicwaves.jl_gb300/build.py "
                           "(or __graft_entry__.build()); there is no CPU fallback")
    lib = ctypes.CDLL(str(LIB_PATH))
    P = ctypes.POINTER
    lib.sw_version.restype = ctypes.c_int
    lib.sw_ctx_create.argtypes = [ctypes.c_int, vp_, P(vp_)]
    lib.sw_ctx_destroy.argtypes = [vp_]
    lib.sw_ctx_last_error.argtypes = [vp_]
    lib.sw_ctx_last_error.restype = ctypes.c_char_p
    lib.sw_ctx_stream.argtypes = [vp_]
    lib.sw_ctx_stream.restype = vp_
    lib.sw_cpml_coefficients.argtypes = [f64, f64, i32, f64, f64, f64, i32, vp_, vp_, vp_, vp_]
    lib.sw_cpml_coefficients64.argtypes = [f64, f64, i32, f64, f64, f64, i32, vp_, vp_, vp_, vp_]
    lib.sw_wavesim_create.argtypes = [vp_, P(SwAcousticParams), i32, P(SwGradParams), P(vp_)]
    lib.sw_wavesim_destroy.argtypes = [vp_]
    lib.sw_wavesim_set_vp.argtypes = [vp_, vp_, i32]
    lib.sw_acoustic_forward.argtypes = [vp_, i32, P(SwAcousticShot), i32]
    lib.sw_acoustic_gradient.argtypes = [vp_, i32, P(SwAcousticShot), i32, vp_, vp_]
    lib.sw_wavesim_set_tuning.argtypes = [vp_, i32, i32]
    lib.sw_wavesim_set_band_heights.argtypes = [vp_, i32, i32, i32]
    lib.sw_wavesim_set_precision.argtypes = [vp_, i32]
    lib.sw_wavesim_set_vp64.argtypes = [vp_, vp_, i32]
    lib.sw_wavesim_set_wait_test.argtypes = [vp_, ctypes.c_int64, i32]
    lib.sw_profile_enable.argtypes = [vp_, i32]
    lib.sw_profile_read.argtypes = [vp_, i32, P(f64), P(ctypes.c_int64), P(f64)]
    lib.sw_profile_read_kernels.argtypes = [vp_, i32, P(ctypes.c_int64)]
    lib.sw_acoustic2d_forward_noalloc.argtypes = [P(SwAcousticParams), vp_, P(SwAcousticShot), vp_]
    lib.sw_elastic_create.argtypes = [vp_, P(SwElasticParams), i32, P(SwGradParams), P(vp_)]
    lib.sw_elastic_destroy.argtypes = [vp_]
    lib.sw_elastic_set_material.argtypes = [vp_, vp_, vp_, vp_]
    lib.sw_elastic_forward.argtypes = [vp_, i32, P(SwElasticShot), i32]
    lib.sw_elastic_gradient.argtypes = [vp_, i32, P(SwElasticShot), i32, vp_, vp_, vp_, vp_]
    lib.sw_elastic_set_tuning.argtypes = [vp_, i32]
    lib.sw_wavesim_use_graphs.argtypes = [vp_, i32]
    lib.sw_acoustic_forward_snapshots.argtypes = [vp_, i32, P(SwAcousticShot), i32, i32, P(vp_)]
    lib.sw_elastic_forward_snapshots.argtypes = [vp_, i32, P(SwElasticShot), i32, i32, P(vp_)]
    lib.sw_acoustic_vd_create.argtypes = [vp_, P(SwAcousticParams), i32, i32, P(SwGradParams), P(vp_)]
    lib.sw_acoustic_vd_destroy.argtypes = [vp_]
    lib.sw_acoustic_vd_set_material.argtypes = [vp_, vp_, vp_]
    lib.sw_acoustic_vd_forward.argtypes = [vp_, i32, P(SwAcousticShot), i32]
    lib.sw_acoustic_vd_forward_snapshots.argtypes = [vp_, i32, P(SwAcousticShot), i32, i32, P(vp_)]
    lib.sw_acoustic_vd_gradient.argtypes = [vp_, i32, P(SwAcousticShot), i32, vp_, vp_, vp_]
    lib.sw_acoustic_vd_set_tuning.argtypes = [vp_, i32]
    lib.sw_acoustic_vd_set_precision.argtypes = [vp_, i32]
    lib.sw_acoustic_vd_set_material64.argtypes = [vp_, vp_, vp_]
    _lib = lib
    return lib


class Context:
    """sw_ctx: one device, one stream."""

    def __init__(self, device: int = 0, stream: int | None = None):
        self.lib = load()
        self.h = vp_()
        rc = self.lib.sw_ctx_create(int(device), vp_(stream) if stream else None, ctypes.byref(self.h))
        if rc != SW_OK:
            raise SwError(rc, f"sw_ctx_create(device={device}) failed (no usable CUDA device?)")

    def check(self, rc: int, what: str):
        if rc != SW_OK:
            raise SwError(rc, f"{what}: {self.lib.sw_ctx_last_error(self.h).decode()}")

    @property
    def stream(self) -> int:
        return int(self.lib.sw_ctx_stream(self.h) or 0)

    def profile(self, on: bool):
        self.check(self.lib.sw_profile_enable(self.h, int(on)), "sw_profile_enable")

    def profile_read(self, kind: int):
        ms, n, b = f64(), ctypes.c_int64(), f64()
        self.check(self.lib.sw_profile_read(self.h, kind, ctypes.byref(ms), ctypes.byref(n), ctypes.byref(b)),
                   "sw_profile_read")
        return ms.value, n.value, b.value

    def profile_kernels(self, kind: int) -> int:
        """Kernel launches inside the timed brackets of `kind`."""
        n = ctypes.c_int64()
        self.check(self.lib.sw_profile_read_kernels(self.h, kind, ctypes.byref(n)), "sw_profile_read_kernels")
        return n.value

    def close(self):
        if self.h:
            self.lib.sw_ctx_destroy(self.h)
            self.h = vp_()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def cpml_coefficients64(vel_max, dt, halo, rcoef, h, f0, freetop_axis):
    """sw_cpml_coefficients64 -> (a, a_h, b, b_h) float64 arrays."""
    import numpy as np
    lib = load()
    a = np.zeros(2 * (halo + 1))
    b = np.zeros(2 * (halo + 1))
    ah = np.zeros(max(2 * halo, 1))
    bh = np.zeros(max(2 * halo, 1))
    rc = lib.sw_cpml_coefficients64(float(vel_max), float(dt), int(halo), float(rcoef), float(h), float(f0),
                                    int(bool(freetop_axis)), a.ctypes.data, ah.ctypes.data, b.ctypes.data,
                                    bh.ctypes.data)
    if rc != SW_OK:
        raise SwError(rc, "sw_cpml_coefficients64: invalid arguments")
    return a, ah[: 2 * halo], b, bh[: 2 * halo]


def cpml_coefficients(vel_max, dt, halo, rcoef, h, f0, freetop_axis):
    """sw_cpml_coefficients -> (a, a_h, b, b_h) float32 arrays."""
    import numpy as np
    lib = load()
    a = np.zeros(2 * (halo + 1), np.float32)
    b = np.zeros(2 * (halo + 1), np.float32)
    ah = np.zeros(max(2 * halo, 1), np.float32)
    bh = np.zeros(max(2 * halo, 1), np.float32)
    rc = lib.sw_cpml_coefficients(float(vel_max), float(dt), int(halo), float(rcoef), float(h), float(f0),
                                  int(bool(freetop_axis)), a.ctypes.data, ah.ctypes.data, b.ctypes.data,
                                  bh.ctypes.data)
    if rc != SW_OK:
        raise SwError(rc, "sw_cpml_coefficients: invalid arguments")
    return a, ah[: 2 * halo], b, bh[: 2 * halo]
