"""ctypes binding of libhyperflow_gpu.so (the C ABI in include/hyperflow_gpu.h).

The library is built in-tree by ``hyperflow_gb300.build`` (``__graft_entry__.build()``).
There is no fallback: if the library is missing or fails to load, importing the
GPU entry points raises.
"""
import ctypes
import os

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libhyperflow_gpu.so")

HF_OK, HF_ERR_INADMISSIBLE, HF_ERR_CHEM_FAIL, HF_ERR_MAXSTEPS, HF_ERR_ARG, HF_ERR_CUDA, HF_ERR_TIMEOUT, \
    HF_ERR_NEGATIVE, HF_ERR_FACE, HF_ERR_COMBINE = range(10)
STATUS_NAMES = {0: "HF_OK", 1: "HF_ERR_INADMISSIBLE", 2: "HF_ERR_CHEM_FAIL", 3: "HF_ERR_MAXSTEPS", 4: "HF_ERR_ARG",
                5: "HF_ERR_CUDA", 6: "HF_ERR_TIMEOUT", 7: "HF_ERR_NEGATIVE", 8: "HF_ERR_FACE", 9: "HF_ERR_COMBINE"}
HF_BC_REFLECTING, HF_BC_TRANSMISSIVE, HF_BC_INFLOW, HF_BC_WEDGE = range(4)
HF_CHEM_PLAIN, HF_CHEM_PERSISTENT = 0, 1
HF_FLUX_PLAIN, HF_FLUX_FUSED = 0, 1

_d = ctypes.c_double
_dp = ctypes.POINTER(ctypes.c_double)
_vp = ctypes.c_void_p
_i64 = ctypes.c_int64
_i32 = ctypes.c_int32


class Level(ctypes.Structure):
    _fields_ = [("nx", _i32), ("ny", _i32), ("dx", _d), ("dy", _d), ("xlo", _d), ("ylo", _d),
                ("periodic", _i32 * 2), ("bc_lo", _i32 * 2), ("bc_hi", _i32 * 2), ("inlet", _d * 13),
                ("wedge_start", _d)]


class Patch(ctypes.Structure):
    _fields_ = [("ilo", _i32), ("jlo", _i32), ("nx", _i32), ("ny", _i32), ("ng", _i32), ("pad_", _i32),
                ("pitch", _i64), ("comp_stride", _i64), ("offset", _i64)]


class Counters(ctypes.Structure):
    _fields_ = [("first_order_stages", _i64), ("roundoff_repairs", _i64), ("retries", _i64),
                ("chem_cell_calls", _i64), ("chem_steps", _i64), ("kernel_launches", _i64),
                ("chem_coop_cells", _i64)]


class ChemHistory(ctypes.Structure):
    _fields_ = [("h", _vp), ("cost", _vp)]


class AdjointOpts(ctypes.Structure):
    _fields_ = [("objective", _i32), ("checkpoint_every", _i32), ("ignition_dT", _d), ("rtol", _d), ("atol", _d)]


HF_OBJ_IGNITION_DELAY, HF_OBJ_PEAK_PRESSURE, HF_OBJ_FINAL_T = range(3)


class TagCriteria(ctypes.Structure):
    _fields_ = [("pressure_tag", _d), ("temperature_tag", _d), ("fuel_rate_tag", _d), ("density_tag", _d),
                ("chemistry", _i32), ("box_only", _i32), ("has_box", _i32), ("pad_", _i32), ("box", _d * 4),
                ("velocity", _d * 2)]


class AmrOpts(ctypes.Structure):
    _fields_ = [("max_level", _i32), ("block", _i32), ("tag_buffer", _i32), ("regrid_interval", _i32),
                ("chemistry", _i32), ("chem_form", _i32), ("rtol", _d), ("atol", _d), ("tags", TagCriteria)]


# (name, restype, argtypes) for every entry point of the header
SIGNATURES = [
    ("hf_init", _i32, [ctypes.c_char_p, ctypes.c_int, ctypes.POINTER(_vp)]),
    ("hf_destroy", None, [_vp]),
    ("hf_nspecies", ctypes.c_int, [_vp]),
    ("hf_last_error", ctypes.c_char_p, [_vp]),
    ("hf_get_counters", None, [_vp, ctypes.POINTER(Counters)]),
    ("hf_set_rate_scale", _i32, [_vp, _dp]),
    ("hf_set_timing", None, [_vp, ctypes.c_int]),
    ("hf_get_timing", None, [_vp, _dp, ctypes.POINTER(_i64)]),
    ("hf_properties", _i32, [_vp, _vp, _i64, _i64, _vp, _vp, _vp, _vp, _vp]),
    ("hf_hllc", _i32, [_vp, _vp, _vp, _vp, _vp, _i64, _i64, ctypes.c_int, _vp, _vp]),
    ("hf_fill_ghosts", _i32, [_vp, ctypes.POINTER(Level), ctypes.POINTER(Patch), ctypes.c_int, _vp, _vp]),
    ("hf_interp_coarse_to_fine", _i32, [_vp, ctypes.POINTER(Patch), _vp, ctypes.POINTER(Patch), _vp,
                                        ctypes.POINTER(_i32), _vp]),
    ("hf_flux_update", _i32, [_vp, ctypes.POINTER(Level), ctypes.POINTER(Patch), ctypes.c_int, _vp, _vp, _vp, _vp,
                              _vp, _d, ctypes.c_int, ctypes.c_int, ctypes.POINTER(_i64), _vp]),
    ("hf_chem_advance", _i32, [_vp, _vp, _i64, _vp, _i64, _d, _vp, _d, _d, ctypes.c_int, ctypes.POINTER(_i64), _vp]),
    ("hf_chem_advance_batched", _i32, [_vp, _vp, _i64, _vp, _i64, _d, _vp, _d, _d, _vp, ctypes.POINTER(_i64), _vp]),
    ("hf_fp64_peak", _i32, [_vp, _dp, _vp]),
    ("hf_fastmath_eval", _i32, [_vp, _i64, _vp, _vp, _vp, _vp, _vp]),
    ("hf_amr_create", _i32, [_vp, ctypes.POINTER(Level), _vp, ctypes.POINTER(AmrOpts), ctypes.POINTER(_vp), _vp]),
    ("hf_amr_destroy", None, [_vp]),
    ("hf_amr_create_levels", _i32, [_vp, ctypes.POINTER(Level), ctypes.POINTER(_vp), ctypes.c_int,
                                    ctypes.POINTER(AmrOpts), ctypes.POINTER(_vp), _vp]),
    ("hf_amr_step", _i32, [_vp, _d, _dp, _vp]),
    ("hf_amr_cfl_dt", _i32, [_vp, _d, _dp, _vp]),
    ("hf_amr_regrid", _i32, [_vp, _vp]),
    ("hf_amr_info", _i32, [_vp, ctypes.c_int, ctypes.POINTER(_i32), ctypes.POINTER(_i32), ctypes.POINTER(_i32),
                           ctypes.POINTER(_i32), ctypes.POINTER(_i32), ctypes.POINTER(_i64)]),
    ("hf_amr_get_level", _i32, [_vp, ctypes.c_int, _vp, _vp, _vp]),
    ("hf_amr_totals", _i32, [_vp, _dp, _vp]),
    ("hf_amr_time", _d, [_vp]),
    ("hf_amr_set_graph", None, [_vp, ctypes.c_int]),
    ("hf_amr_stats", None, [_vp, ctypes.POINTER(_i64), ctypes.POINTER(_i64)]),
    ("hf_flow_record", _i32, [_vp, ctypes.POINTER(Level), _vp, _i32, _vp, _d, _i32, ctypes.c_int, _d, _d, _vp, _vp,
                              ctypes.POINTER(_vp), _vp]),
    ("hf_flow_adjoint", _i32, [_vp, _vp, _vp, _vp, _vp]),
    ("hf_flow_tape_destroy", None, [_vp]),
    ("hf_flux_adjoint", _i32, [_vp, ctypes.POINTER(Level), ctypes.POINTER(Patch), _vp, _vp, _d, ctypes.c_int, _vp,
                               _vp]),
    ("hf_chem_objective", _i32, [_vp, _vp, _i64, _i64, _d, _i32, ctypes.POINTER(AdjointOpts), _vp,
                                 ctypes.POINTER(_i64), _vp]),
    ("hf_chem_adjoint", _i32, [_vp, _vp, _i64, _i64, _d, _i32, ctypes.POINTER(AdjointOpts), _vp, _vp, _vp,
                               ctypes.POINTER(_i64), _vp]),
    ("hf_chem_advance_noalloc", _i32, [ctypes.c_int, _vp, _i64, _vp, _i64, _d, _vp, _d, _d, ctypes.POINTER(_i64), _vp]),
    ("hf_totals", _i32, [_vp, ctypes.POINTER(Patch), ctypes.c_int, _vp, _vp, _d, ctypes.c_int, _dp, _vp]),
    ("hf_average_down", _i32, [_vp, ctypes.POINTER(Patch), ctypes.c_int, _vp, ctypes.POINTER(Patch), ctypes.c_int,
                               _vp, _vp]),
    ("hf_reflux", _i32, [_vp, ctypes.POINTER(Level), ctypes.POINTER(Patch), ctypes.c_int, _vp, _vp, _vp,
                         ctypes.POINTER(Patch), ctypes.c_int, _vp, _vp, _d, _vp]),
    ("hf_tag_cells", _i32, [_vp, ctypes.POINTER(Level), ctypes.POINTER(Patch), ctypes.c_int, _vp, _d,
                            ctypes.POINTER(TagCriteria), _vp, _vp]),
    ("hf_cfl_dt", _i32, [_vp, ctypes.POINTER(Level), ctypes.POINTER(Patch), ctypes.c_int, _vp, _d, _dp, _vp]),
    ("hf_validate", _i32, [_vp, ctypes.POINTER(Level), ctypes.POINTER(Patch), ctypes.c_int, _vp,
                           ctypes.POINTER(_i64), _vp]),
    ("hf_set_chem_tuning", _i32, [_i32, _i32]),
    ("hf_get_chem_tuning", None, [ctypes.POINTER(_i32), ctypes.POINTER(_i32)]),
    ("hf_repair_roundoff", _i32, [_vp, ctypes.c_int, ctypes.POINTER(Level), ctypes.POINTER(ctypes.POINTER(Patch)),
                                  ctypes.POINTER(ctypes.c_int), ctypes.POINTER(_vp), ctypes.POINTER(_vp),
                                  ctypes.POINTER(_i64), _vp]),
    ("hf_stepper_create", _i32, [_vp, ctypes.POINTER(Level), _vp, ctypes.c_int, _d, _d, ctypes.c_int, ctypes.c_int,
                                 ctypes.POINTER(_vp)]),
    ("hf_stepper_destroy", None, [_vp]),
    ("hf_stepper_step", _i32, [_vp, _d, _dp, _vp]),
    ("hf_stepper_run", _i32, [_vp, _i32, _d, ctypes.POINTER(_i32), _vp]),
    ("hf_stepper_get", _i32, [_vp, _vp, _vp]),
    ("hf_stepper_set_host", _i32, [_vp, _vp, _vp]),
    ("hf_stepper_get_host", _i32, [_vp, _vp, _vp]),
    ("hf_stepper_time", _d, [_vp]),
    ("hf_stepper_cfl_dt", _i32, [_vp, _d, _dp, _vp]),
    ("hf_stepper_stats", None, [_vp, ctypes.POINTER(_i64), ctypes.POINTER(_i64)]),
    ("hf_stepper_set_graph", None, [_vp, ctypes.c_int]),
    ("hf_stepper_graph_info", None, [_vp, ctypes.POINTER(ctypes.c_uint32), ctypes.POINTER(_i32),
                                     ctypes.POINTER(ctypes.c_uint32)]),
]

_lib = None


def load():
    """Load the library (raises OSError if it is missing or does not load)."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise OSError("libhyperflow_gpu.so is not built: run hyperflow_gb300.build.build() "
                          "(__graft_entry__.build()) first")
        lib = ctypes.CDLL(LIB_PATH)
        for name, res, args in SIGNATURES:
            f = getattr(lib, name)
            f.restype = res
            f.argtypes = args
        _lib = lib
    return _lib
