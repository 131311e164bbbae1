"""ctypes binding of liblbm_gb300.so, the C ABI declared in include/lbm_gb300.h.

There is no fallback: if the library is missing and cannot be built, or the
GPU cannot be used, every call raises ``LbmError``.
"""

import ctypes
import os
import threading

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "liblbm_gb300.so")

OK, ERR_ARG, ERR_CUDA, ERR_NONFINITE, ERR_STATE = range(5)
BGK, TRT, LES = 0, 1, 2
NO_OBSTACLE, CYLINDER, SPHERE, BOX, HEATSINK = 0, 1, 2, 3, 4
PERIODIC, SLIP, LID = 0, 1, 2
F32, F16, BF16, F64 = 0, 1, 2, 3
HOST, DEVICE = 0, 1
FLAG_SIMT = 1
FLAG_BULKCOPY = 2
FLAG_SLOT_POINTERS = 4
FIELDS = ("ux", "uy", "uz", "p", "vmag", "r_rho", "r_ux", "r_uy", "r_uz", "r_ke", "fx", "fy", "fz")
MONITORS = ("continuity", "momentum_x", "momentum_y", "momentum_z", "energy", "drag", "lift")
STORAGE = {"f32": F32, "f16": F16, "bf16": BF16, "f64": F64}
COLLISION = {"bgk": BGK, "trt": TRT, "les": LES}
OBSTACLE = {"none": NO_OBSTACLE, "cylinder": CYLINDER, "sphere": SPHERE, "box": BOX, "heatsink": HEATSINK}
HEAT_FIELDS = ("t_solid", "q_solid", "temp")
OUT_TEMP = 5
SIDE = {"periodic": PERIODIC, "slip": SLIP, "lid": LID}


class LbmError(RuntimeError):
    """A failed C-ABI call; ``status`` is the lbm_status code."""

    def __init__(self, status, message):
        super().__init__(message)
        self.status = status


class Config(ctypes.Structure):
    """struct lbm_config."""

    _fields_ = [
        ("nx", ctypes.c_int32), ("ny", ctypes.c_int32), ("nz", ctypes.c_int32),
        ("collision", ctypes.c_int32), ("obstacle", ctypes.c_int32),
        ("lateral", ctypes.c_int32), ("vertical", ctypes.c_int32), ("storage", ctypes.c_int32),
        ("nu", ctypes.c_double), ("cs", ctypes.c_double), ("magic", ctypes.c_double),
        ("ox", ctypes.c_double), ("oy", ctypes.c_double), ("oz", ctypes.c_double),
        ("r", ctypes.c_double), ("hx", ctypes.c_double), ("hy", ctypes.c_double), ("hz", ctypes.c_double),
        ("u0", ctypes.c_double), ("sponge_start", ctypes.c_double), ("sponge_strength", ctypes.c_double),
        ("u_lid", ctypes.c_double), ("omega_rot", ctypes.c_double),
        ("device", ctypes.c_int32), ("flags", ctypes.c_int32),
        ("sink", ctypes.c_double * 8),
        ("heat", ctypes.c_int32), ("reserved", ctypes.c_int32),
        ("alpha", ctypes.c_double), ("heat_nu", ctypes.c_double),
    ]


class AdjConfig(ctypes.Structure):
    """struct lbm_adj_config."""

    _fields_ = [
        ("nx", ctypes.c_int32), ("ny", ctypes.c_int32), ("nz", ctypes.c_int32),
        ("precision", ctypes.c_int32), ("steps", ctypes.c_int32), ("loss_start", ctypes.c_int32),
        ("checkpoint", ctypes.c_int32), ("device", ctypes.c_int32),
        ("u0", ctypes.c_double), ("tau0", ctypes.c_double), ("cs", ctypes.c_double), ("r", ctypes.c_double),
        ("ox", ctypes.c_double), ("oy", ctypes.c_double), ("width", ctypes.c_double),
        ("diameter", ctypes.c_double), ("sponge_start", ctypes.c_double),
        ("sponge_strength", ctypes.c_double), ("seed_amp", ctypes.c_double),
    ]


class WingConfig(ctypes.Structure):
    """struct lbm_wing_config."""

    _fields_ = [
        ("nx", ctypes.c_int32), ("ny", ctypes.c_int32), ("nz", ctypes.c_int32), ("collision", ctypes.c_int32),
        ("nu", ctypes.c_double), ("cs", ctypes.c_double), ("magic", ctypes.c_double),
        ("chord", ctypes.c_double), ("x_ea", ctypes.c_double), ("y_ea", ctypes.c_double), ("ea", ctypes.c_double),
        ("u0", ctypes.c_double), ("sponge_start", ctypes.c_double), ("sponge_strength", ctypes.c_double),
        ("device", ctypes.c_int32), ("reserved", ctypes.c_int32),
    ]


class FsiConfig(ctypes.Structure):
    """struct lbm_fsi_config."""

    _fields_ = [
        ("nx", ctypes.c_int32), ("ny", ctypes.c_int32), ("nz", ctypes.c_int32), ("collision", ctypes.c_int32),
        ("nu", ctypes.c_double), ("cs", ctypes.c_double), ("magic", ctypes.c_double),
        ("chord", ctypes.c_double), ("x_ea", ctypes.c_double), ("y_ea", ctypes.c_double), ("ea", ctypes.c_double),
        ("span", ctypes.c_double), ("u0", ctypes.c_double), ("sponge_start", ctypes.c_double),
        ("sponge_strength", ctypes.c_double), ("device", ctypes.c_int32), ("reserved", ctypes.c_int32),
    ]


_D4 = ctypes.POINTER(ctypes.c_double)
_SIGNATURES = {
    "lbm_abi_version": (ctypes.c_int32, []),
    "lbm_last_error": (ctypes.c_char_p, []),
    "lbm_create": (ctypes.c_int, [ctypes.POINTER(Config), ctypes.POINTER(ctypes.c_void_p)]),
    "lbm_destroy": (ctypes.c_int, [ctypes.c_void_p]),
    "lbm_init": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_double]),
    "lbm_init_random": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_double, ctypes.c_double, ctypes.c_uint64]),
    "lbm_step": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int32, ctypes.c_void_p]),
    "lbm_run": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int32, ctypes.c_int32, ctypes.c_void_p]),
    "lbm_monitors": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int32, ctypes.c_double,
                                    ctypes.POINTER(ctypes.c_double)]),
    "lbm_field_sums": (ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(ctypes.c_double)]),
    "lbm_field": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int32, ctypes.POINTER(ctypes.c_void_p)]),
    "lbm_set_field": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int32, ctypes.c_void_p]),
    "lbm_set_physics": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int32, ctypes.c_double, ctypes.c_double]),
    "lbm_set_obstacle": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int32, ctypes.POINTER(ctypes.c_double)]),
    "lbm_set_actuation": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_double]),
    "lbm_get_actuation": (ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(ctypes.c_double)]),
    "lbm_set_sponge": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_double, ctypes.c_double]),
    "lbm_set_populations": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int32, ctypes.c_int32]),
    "lbm_get_populations": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int32, ctypes.c_int32]),
    "lbm_mask": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p]),
    "lbm_set_output_stride": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int32]),
    "lbm_output": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int32, ctypes.POINTER(ctypes.c_void_p),
                                  ctypes.POINTER(ctypes.c_int64)]),
    "lbm_update_output": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p]),
    "lbm_step_count": (ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(ctypes.c_int64)]),
    "lbm_memory": (ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(ctypes.c_int64)]),
    "lbm_sync": (ctypes.c_int, [ctypes.c_void_p]),
    "lbm_test_bulkcopy_stall": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int64]),
    "lbm_timing": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int32]),
    "lbm_timing_read": (ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(ctypes.c_double)]),
    "lbm_field_sums_static": (ctypes.c_int, [ctypes.POINTER(ctypes.c_void_p), ctypes.c_int64,
                                             ctypes.c_void_p, ctypes.c_void_p]),
    "lbm_managed_alloc": (ctypes.c_int, [ctypes.c_int64, ctypes.POINTER(ctypes.c_void_p)]),
    "lbm_managed_free": (ctypes.c_int, [ctypes.c_void_p]),
    "lbm_velocity_gradient": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_double, ctypes.c_void_p]),
    "lbm_vorticity_q": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p,
                                       ctypes.c_int32, ctypes.c_void_p]),
    "lbm_vorticity_q_direct": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_double, ctypes.c_void_p, ctypes.c_void_p,
                                              ctypes.c_int32, ctypes.c_void_p]),
    "lbm_run_timed": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int32, ctypes.c_int32, ctypes.c_void_p,
                                     ctypes.POINTER(ctypes.c_double)]),
    "lbm_read_output": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int32, ctypes.c_void_p, ctypes.c_void_p]),
    "lbm_set_sink": (ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(ctypes.c_double)]),
    "lbm_heat_field": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int32, ctypes.POINTER(ctypes.c_void_p)]),
    "lbm_set_heat_populations": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int32,
                                                ctypes.c_int32]),
    "lbm_get_heat_populations": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int32,
                                                ctypes.c_int32]),
    "lbm_wing_create": (ctypes.c_int, [ctypes.POINTER(WingConfig), ctypes.POINTER(ctypes.c_void_p)]),
    "lbm_wing_destroy": (ctypes.c_int, [ctypes.c_void_p]),
    "lbm_wing_init": (ctypes.c_int, [ctypes.c_void_p, _D4]),
    "lbm_wing_step": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int32, _D4, _D4]),
    "lbm_wing_set_physics": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int32, ctypes.c_double]),
    "lbm_wing_field": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int32, ctypes.POINTER(ctypes.c_void_p)]),
    "lbm_wing_populations": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int32]),
    "lbm_wing_mask": (ctypes.c_int, [ctypes.c_void_p, _D4, ctypes.c_void_p]),
    "lbm_wing_set_output_stride": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int32]),
    "lbm_wing_output": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int32, ctypes.POINTER(ctypes.c_void_p),
                                       ctypes.POINTER(ctypes.c_int64)]),
    "lbm_wing_update_output": (ctypes.c_int, [ctypes.c_void_p]),
    "lbm_fsi_create": (ctypes.c_int, [ctypes.POINTER(FsiConfig), ctypes.POINTER(ctypes.c_void_p)]),
    "lbm_fsi_destroy": (ctypes.c_int, [ctypes.c_void_p]),
    "lbm_fsi_init": (ctypes.c_int, [ctypes.c_void_p, _D4]),
    "lbm_fsi_step": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int32, _D4, _D4]),
    "lbm_fsi_set_physics": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int32, ctypes.c_double]),
    "lbm_fsi_field": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int32, ctypes.POINTER(ctypes.c_void_p)]),
    "lbm_fsi_populations": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int32]),
    "lbm_fsi_mask": (ctypes.c_int, [ctypes.c_void_p, _D4, ctypes.c_void_p]),
    "lbm_fsi_set_output_stride": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int32]),
    "lbm_fsi_output": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int32, ctypes.POINTER(ctypes.c_void_p),
                                      ctypes.POINTER(ctypes.c_int64)]),
    "lbm_fsi_update_output": (ctypes.c_int, [ctypes.c_void_p]),
    "lbm_adj_create": (ctypes.c_int, [ctypes.POINTER(AdjConfig), ctypes.POINTER(ctypes.c_void_p)]),
    "lbm_adj_destroy": (ctypes.c_int, [ctypes.c_void_p]),
    "lbm_adj_set_params": (ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(ctypes.c_double)]),
    "lbm_adj_forward": (ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(ctypes.c_double)]),
    "lbm_adj_backward": (ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(ctypes.c_double)]),
    "lbm_adj_state": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int32, ctypes.c_void_p]),
    "lbm_adj_info": (ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(ctypes.c_double)]),
}

_lib = None
_lock = threading.Lock()


def load(build=True):
    """Load (building first if needed) the native library."""
    global _lib
    with _lock:
        if _lib is not None:
            return _lib
        if build:
            import importlib.util
            spec = importlib.util.spec_from_file_location("lbm_build_native", os.path.join(HERE, "build_native.py"))
            mod = importlib.util.module_from_spec(spec)
            spec.loader.exec_module(mod)
            mod.build()
        if not os.path.exists(LIB_PATH):
            raise LbmError(ERR_STATE, f"{LIB_PATH} is missing; build it with build_native.py")
        lib = ctypes.CDLL(LIB_PATH)
        for name, (res, args) in _SIGNATURES.items():
            fn = getattr(lib, name)
            fn.restype = res
            fn.argtypes = args
        _lib = lib
        return lib


def check(status, allow=()):
    if status != OK and status not in allow:
        msg = _lib.lbm_last_error().decode(errors="replace") if _lib is not None else ""
        raise LbmError(status, msg or f"lbm status {status}")
    return status


class Handle:
    """Owns one native solver; destroyed with the last reference."""

    def __init__(self, cfg):
        self.lib = load()
        self.cfg = cfg
        ptr = ctypes.c_void_p()
        check(self.lib.lbm_create(ctypes.byref(cfg), ctypes.byref(ptr)))
        self.ptr = ptr

    def __del__(self):
        ptr, self.ptr = getattr(self, "ptr", None), None
        if ptr and _lib is not None:
            _lib.lbm_destroy(ptr)

    def call(self, name, *args, allow=()):
        return check(getattr(self.lib, name)(self.ptr, *args), allow)
