"""ctypes binding of ``libpfgb300.so`` (declared in ``include/pf_gb300.h``).

The structs below mirror the C structs field for field; ``load()`` checks
their sizes against ``pfg_struct_size`` so a mismatch fails at load time.
There is no CPU fallback: if the library is missing, every entry point
raises.
"""
import ctypes
import os

from . import _build

MAX_ORIS = 64
MAX_SEGMENTS = 16
BC_NEUMANN, BC_PERIODIC = 0, 1
LAYOUT_ZYX, LAYOUT_XYZ = 0, 1

STATUS = {
    0: "PFG_OK", 1: "PFG_ERR_SHAPE", 2: "PFG_ERR_NULL", 3: "PFG_ERR_ALIGN", 4: "PFG_ERR_PARAM",
    5: "PFG_ERR_LAUNCH", 6: "PFG_ERR_TIMEOUT", 7: "PFG_ERR_CAPACITY", 8: "PFG_ERR_NO_DEVICE",
}


class PfParams(ctypes.Structure):
    _fields_ = [
        ("nx", ctypes.c_int32), ("ny", ctypes.c_int32), ("nz", ctypes.c_int32),
        ("num_oris", ctypes.c_int32),
        ("h_x", ctypes.c_float), ("h_y", ctypes.c_float), ("h_z", ctypes.c_float),
        ("T_liquidus", ctypes.c_float), ("gas_const", ctypes.c_float), ("Qg", ctypes.c_float),
        ("L0", ctypes.c_float), ("kappa_g", ctypes.c_float), ("m_g", ctypes.c_float),
        ("anisotropy", ctypes.c_float), ("ad_hoc", ctypes.c_float),
        ("bc_x", ctypes.c_int32), ("bc_y", ctypes.c_int32), ("bc_z", ctypes.c_int32),
        ("force_liquid_zero", ctypes.c_int32), ("liquid_shift", ctypes.c_float),
        ("grain_dirs", ctypes.c_float * (3 * MAX_ORIS * 3)),
    ]


class Segment(ctypes.Structure):
    _fields_ = [(k, ctypes.c_float) for k in ("t0", "t1", "x0", "y0", "x1", "y1", "power",
                                             "reserved")]


class HeatParams(ctypes.Structure):
    _fields_ = [
        ("nx", ctypes.c_int32), ("ny", ctypes.c_int32), ("nz", ctypes.c_int32),
        ("dx", ctypes.c_float), ("dy", ctypes.c_float), ("dz", ctypes.c_float),
        ("rho", ctypes.c_float), ("h_conv", ctypes.c_float), ("emissivity", ctypes.c_float),
        ("sigma_sb", ctypes.c_float), ("T0", ctypes.c_float), ("Ts", ctypes.c_float),
        ("Tl", ctypes.c_float), ("latent", ctypes.c_float), ("absorptivity", ctypes.c_float),
        ("beam_radius", ctypes.c_float), ("x_first", ctypes.c_float),
        ("y_first", ctypes.c_float), ("layout", ctypes.c_int32),
        ("num_segments", ctypes.c_int32), ("path", Segment * MAX_SEGMENTS),
    ]


class Clock(ctypes.Structure):
    _fields_ = [("t", ctypes.c_double), ("step", ctypes.c_int64)]


class Quench(ctypes.Structure):
    _fields_ = [(k, ctypes.c_double) for k in ("T_base", "grad", "vel", "z0", "z_first")]


class BatchJob(ctypes.Structure):
    _fields_ = [("params", PfParams), ("quench", Quench), ("eta", ctypes.c_void_p * 2),
                ("t0", ctypes.c_double), ("dt", ctypes.c_float), ("reserved", ctypes.c_int32),
                ("base_step", ctypes.c_int64), ("target_steps", ctypes.c_int64)]


class Diag(ctypes.Structure):
    _fields_ = [("energy", ctypes.c_double), ("max_T", ctypes.c_double),
                ("n_cells", ctypes.c_int64), ("n_ori_changed", ctypes.c_int64),
                ("n_liquid", ctypes.c_int64), ("n_nonfinite", ctypes.c_int64),
                ("mass", ctypes.c_double * MAX_ORIS)]


class PointSourceRecord(ctypes.Structure):
    _fields_ = [("t", ctypes.c_double)] + [(k, ctypes.c_float) for k in
                                           ("x", "y", "z", "ux", "uy", "uz", "Q", "vel")]


class PointSources(ctypes.Structure):
    _fields_ = [(k, ctypes.c_float) for k in ("T_ambient", "alpha", "kappa", "T_clip", "x_first",
                                               "y_first", "z_first")] + [
        ("reserved", ctypes.c_int32), ("table", ctypes.c_void_p), ("num_records", ctypes.c_int64)]


class Interp(ctypes.Structure):
    _fields_ = [("t_future", ctypes.c_double), ("dt_coarse", ctypes.c_double)]


class Grain(ctypes.Structure):
    _fields_ = [("first_cell", ctypes.c_int64), ("ori", ctypes.c_int32),
                ("reserved", ctypes.c_int32), ("cells", ctypes.c_int64),
                ("sum", ctypes.c_int64 * 3), ("sum2", ctypes.c_int64 * 6)]


class CfdGrid(ctypes.Structure):
    _fields_ = [("nx", ctypes.c_int32), ("ny", ctypes.c_int32), ("nz", ctypes.c_int32),
                ("pad", ctypes.c_int32)] + [(k, ctypes.c_double) for k in
                                            ("dx", "dy", "dz", "lx", "ly", "lz")]


class LinClipC(ctypes.Structure):
    _fields_ = [(k, ctypes.c_double) for k in ("a", "b", "lo", "hi")]


class CfdEnergy(ctypes.Structure):
    _fields_ = ([("cp", LinClipC), ("k", LinClipC)]
                + [(k, ctypes.c_double) for k in ("rho", "latent_heat", "Ts", "Tl", "dt", "T_ref",
                                                  "h_conv", "emissivity", "sigma")]
                + [("heat_source", ctypes.c_int32), ("max_newton", ctypes.c_int32)]
                + [(k, ctypes.c_double) for k in ("P", "eta", "rb", "phi", "speed", "xl", "yl",
                                                  "zl", "newton_tol")])


class CfdFlow(ctypes.Structure):
    _fields_ = ([(k, ctypes.c_double) for k in ("rho", "visco", "dt", "marangoni", "Ts", "Tl")]
                + [(k, ctypes.c_int32) for k in ("x0", "y0", "z0", "pad")])


class CfdStats(ctypes.Structure):
    _fields_ = [("newton_iters", ctypes.c_int32), ("pad", ctypes.c_int32),
                ("energy_krylov", ctypes.c_int64), ("momentum_krylov", ctypes.c_int64 * 3),
                ("pressure_krylov", ctypes.c_int64)]


_P = ctypes.c_void_p
_I = ctypes.c_int
_F = ctypes.c_float
_PROTOS = {
    "pfg_abi_version": (_I, []),
    "pfg_status_string": (ctypes.c_char_p, [_I]),
    "pfg_last_cuda_error": (ctypes.c_char_p, []),
    "pfg_struct_size": (ctypes.c_int64, [_I]),
    "pfg_set_kernel_variant": (_I, [_I]),
    "pfg_device_error": (_I, [_I]),
    "pfg_tune": (_I, [_I, _I]),
    "pfg_describe_plan": (_I, [ctypes.POINTER(PfParams), _P]),
    "pfg_fixed_plan": (_I, [ctypes.POINTER(PfParams)]),
    "pfg_pf_step": (_I, [ctypes.POINTER(PfParams), _P, _P, _P, _F, _P]),
    "pfg_pf_step_quench": (_I, [ctypes.POINTER(PfParams), ctypes.POINTER(Quench), _P, _P, _P, _P,
                                _F, _P]),
    "pfg_heat_step": (_I, [ctypes.POINTER(HeatParams), _P, _P, _F, _F, _F, _F, _P]),
    "pfg_heat_pf_step": (_I, [ctypes.POINTER(PfParams), ctypes.POINTER(HeatParams), _P, _P, _P,
                              _P, _P, _P, _F, _P]),
    "pfg_heat_pf_step_comp": (_I, [ctypes.POINTER(PfParams), ctypes.POINTER(HeatParams), _P, _P,
                                   _P, _P, _P, _P, _P, _P, _F, _P]),
    "pfg_heat_pf_step_comp_supported": (_I, [ctypes.POINTER(PfParams)]),
    "pfg_batch_table_bytes": (ctypes.c_int64, [_I]),
    "pfg_batch_encode": (_I, [ctypes.POINTER(BatchJob), _I, _P, ctypes.c_int64,
                              ctypes.POINTER(ctypes.c_int64)]),
    "pfg_batch_step": (_I, [_P, _I, _P]),
    "pfg_batch_advance": (_I, [_P, _I, _P]),
    "pfg_adjoint_scratch_bytes": (ctypes.c_int64, [ctypes.POINTER(PfParams)]),
    "pfg_adjoint_step": (_I, [ctypes.POINTER(PfParams), ctypes.POINTER(HeatParams), _P, _P,
                              ctypes.c_double, _F, _P, _P, _P, _P, _P, ctypes.c_int64, _P, _F,
                              _P]),
    "pfg_objective": (_I, [ctypes.POINTER(PfParams), _P, _P, _P, _P, _P]),
    "pfg_pf_diag_scratch_bytes": (ctypes.c_int64, [ctypes.POINTER(PfParams)]),
    "pfg_pf_diag": (_I, [ctypes.POINTER(PfParams), _P, _P, _I, _P, _P, _P, ctypes.c_int64, _P,
                         _P]),
    "pfg_pf_diag_noalloc": (_I, [ctypes.POINTER(PfParams), _P, _P, _I, _P, _P, _P, _P]),
    "pfg_pf_inspect": (_I, [ctypes.POINTER(PfParams), _P, _P, _I, _P, _P, _P, ctypes.c_int64,
                            _P, _P]),
    "pfg_pf_step_point_source": (_I, [ctypes.POINTER(PfParams), ctypes.POINTER(PointSources), _P,
                                      _P, _P, _P, _F, _P]),
    "pfg_pf_step_interp": (_I, [ctypes.POINTER(PfParams), ctypes.POINTER(Interp), _P, _P, _P, _P,
                                _P, _P, _F, _P]),
    "pfg_transpose_xyz": (_I, [ctypes.c_int32, ctypes.c_int32, ctypes.c_int32, _P, _P, _P]),
    "pfg_cfd_workspace_bytes": (ctypes.c_int64, [ctypes.POINTER(CfdGrid), ctypes.POINTER(CfdGrid)]),
    "pfg_cfd_energy_solve": (_I, [ctypes.POINTER(CfdGrid), ctypes.POINTER(CfdEnergy), _P, _P, _P,
                                  _P, ctypes.c_int64, ctypes.POINTER(CfdStats), _P]),
    "pfg_cfd_solid_update": (_I, [ctypes.POINTER(CfdGrid), ctypes.c_double, ctypes.c_double, _P,
                                  _P, _P]),
    "pfg_cfd_flow_step": (_I, [ctypes.POINTER(CfdGrid), ctypes.POINTER(CfdGrid),
                               ctypes.POINTER(CfdFlow), _P, _P, _P, _P, _P, _P, ctypes.c_int64,
                               ctypes.POINTER(CfdStats), _P]),
    "pfg_point_source_T": (_I, [ctypes.POINTER(PfParams), ctypes.POINTER(PointSources), _P, _P,
                                _P]),
    "pfg_grain_scratch_bytes": (ctypes.c_int64, [ctypes.POINTER(PfParams)]),
    "pfg_grains": (_I, [ctypes.POINTER(PfParams), _P, _P, _I, _P, _P, ctypes.c_int64, _P, _P,
                        ctypes.c_int64, _P]),
}
_STRUCTS = [(0, PfParams), (1, Segment), (2, HeatParams), (3, Clock), (4, Diag), (5, Quench),
            (6, BatchJob), (7, Grain), (8, PointSourceRecord), (9, PointSources),
            (10, Interp), (11, CfdGrid), (12, LinClipC), (13, CfdEnergy), (14, CfdFlow),
            (15, CfdStats)]

_lib = None


class PFGError(RuntimeError):
    """A library call returned a failure status."""


def load():
    """Load the CUDA library; raises if it has not been built."""
    global _lib
    if _lib is not None:
        return _lib
    path = _build.LIB
    if not os.path.exists(path):
        raise RuntimeError(
            f"{path} is missing: build it with `python -c 'import __graft_entry__ as g; g.build()'` "
            "(needs nvcc).  jax_am_gb300 has no CPU fallback.")
    lib = ctypes.CDLL(path)
    for name, (res, args) in _PROTOS.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    for which, cls in _STRUCTS:
        got = lib.pfg_struct_size(which)
        if got != ctypes.sizeof(cls):
            raise RuntimeError(f"ABI mismatch: sizeof({cls.__name__}) is {ctypes.sizeof(cls)} "
                               f"in Python but {got} in the library")
    _lib = lib
    return lib


def check(status, what):
    """Raise the Python error that matches the reference's behaviour."""
    if status == 0:
        return
    lib = load()
    msg = lib.pfg_status_string(status).decode()
    if status == 5:
        msg += ": " + lib.pfg_last_cuda_error().decode()
    text = f"{what} failed ({STATUS.get(status, status)}): {msg}"
    if status in (1, 2, 3, 4):
        raise ValueError(text)
    raise PFGError(text)


def ptr(t):
    """Device address of a tensor (None -> NULL)."""
    return None if t is None else ctypes.c_void_p(t.data_ptr())


PLAN_FIELDS = ("kernel", "vec", "lanes_per_cell", "tile_x", "tile_y", "warps_x", "rows_per_warp",
               "slots", "planes_per_unit", "ctas", "smem_bytes", "sm_count")


def describe_plan(params):
    """The launch plan of a step with ``params`` on the current device."""
    out = (ctypes.c_int32 * 12)()
    check(load().pfg_describe_plan(ctypes.byref(params), out), "pfg_describe_plan")
    plan = dict(zip(PLAN_FIELDS, list(out)))
    fixed = load().pfg_fixed_plan(ctypes.byref(params))
    if fixed < 0:
        check(-fixed, "pfg_fixed_plan")
    plan["fixed"] = fixed  # compile-time tile plan of the TMA-fed kernel (0: none)
    return plan


def device_error(clear=True):
    """0, or PFG_ERR_TIMEOUT (6) if a bounded device-side wait ran out since
    the last call (the affected step's output is invalid)."""
    v = load().pfg_device_error(int(clear))
    if v < 0 or v in (5, 8):
        check(v if v > 0 else 5, "pfg_device_error")
    return v
