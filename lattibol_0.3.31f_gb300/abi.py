"""ctypes mirror of the C ABI declared in include/lattibol.h and include/lbgb300.h.

``DataD2Q9`` / ``DataD3Q19`` are the reference's per-device state structs
(reference src/lattibol.h:29-97): the same member order, so a struct filled
here can be handed to the reference's own kernels or to this library's
drop-in entry points alike.
"""
import ctypes
import os

_fp = ctypes.POINTER(ctypes.c_float)
_bp = ctypes.c_void_p  # bool*

LIB_DIR = os.path.join(os.path.dirname(os.path.abspath(__file__)), "lib")
LIB_PATH = os.path.join(LIB_DIR, "liblbgb300.so")


class dim3(ctypes.Structure):
    _fields_ = [("x", ctypes.c_uint), ("y", ctypes.c_uint), ("z", ctypes.c_uint)]


def _floats(*names):
    return [(n, ctypes.c_void_p) for n in names]


class DataD2Q9(ctypes.Structure):
    _fields_ = (_floats("ux", "uy", "rho") + [("solid", _bp), ("solid_bound", _bp)]
                + _floats(*["f%d" % k for k in range(9)])
                + _floats("border_f1", "border_f5", "border_f8", "border_f3", "border_f6",
                          "border_f7")
                + _floats("nb_border_f1", "nb_border_f5", "nb_border_f8", "nb_border_f3",
                          "nb_border_f6", "nb_border_f7")
                + [("width", ctypes.c_int), ("height", ctypes.c_int),
                   ("deviceCount", ctypes.c_int), ("dev", ctypes.c_int)]
                + _floats("plotBuffer", "valueCur") + [("stream", ctypes.c_void_p)]
                + _floats("psi", "ueq_x", "ueq_y"))

    POP = ["f%d" % k for k in range(9)]
    BORDER = ["border_f1", "border_f5", "border_f8", "border_f3", "border_f6", "border_f7"]
    NB_BORDER = ["nb_" + b for b in BORDER]


class DataD3Q19(ctypes.Structure):
    _fields_ = (_floats("ux", "uy", "uz", "rho") + [("solid", _bp), ("solid_bound", _bp)]
                + _floats(*["f%d" % k for k in range(19)])
                + _floats("border_f1", "border_f7", "border_f8", "border_f9", "border_f10",
                          "border_f2", "border_f11", "border_f12", "border_f13", "border_f14")
                + _floats("nb_border_f1", "nb_border_f7", "nb_border_f8", "nb_border_f9",
                          "nb_border_f10", "nb_border_f2", "nb_border_f11", "nb_border_f12",
                          "nb_border_f13", "nb_border_f14")
                + [("width", ctypes.c_int), ("height", ctypes.c_int), ("depth", ctypes.c_int),
                   ("deviceCount", ctypes.c_int), ("dev", ctypes.c_int)]
                + _floats("plotBuffer", "valueCur") + [("stream", ctypes.c_void_p)])

    POP = ["f%d" % k for k in range(19)]
    BORDER = ["border_f1", "border_f7", "border_f8", "border_f9", "border_f10", "border_f2",
              "border_f11", "border_f12", "border_f13", "border_f14"]
    NB_BORDER = ["nb_" + b for b in BORDER]


class lb_config(ctypes.Structure):
    _fields_ = [("lattice", ctypes.c_int), ("nx", ctypes.c_int), ("ny", ctypes.c_int),
                ("nz", ctypes.c_int), ("mode", ctypes.c_int), ("storage", ctypes.c_int),
                ("tau_inv", ctypes.c_float), ("force", ctypes.c_float * 3),
                ("u_in", ctypes.c_float * 3), ("rho_out", ctypes.c_float),
                ("wall_u", ctypes.c_float * 3), ("G", ctypes.c_float), ("G_ads", ctypes.c_float),
                ("psi_form", ctypes.c_int), ("graph_steps", ctypes.c_int),
                ("tuning", ctypes.c_int), ("rho_ref", ctypes.c_float)]


class lb_run_params_d3q19(ctypes.Structure):
    _fields_ = [(n, ctypes.c_float) for n in ("w0", "w1", "w7", "tau_inv", "ux_in", "uy_in",
                                              "uz_in", "rho_out")] + [("cursor", ctypes.c_int * 3)]


class lb_case_params(ctypes.Structure):
    """The parameter file of a case (reference src/input.cpp:51-94)."""
    _fields_ = [("device_count", ctypes.c_int), ("max_dim", ctypes.c_int),
                ("ux", ctypes.c_float), ("uy", ctypes.c_float), ("uz", ctypes.c_float),
                ("rho", ctypes.c_float), ("viscosity", ctypes.c_float),
                ("update_steps", ctypes.c_int), ("ext_f", ctypes.c_float * 3),
                ("G", ctypes.c_float), ("G_ads", ctypes.c_float), ("tau_inv", ctypes.c_float),
                ("min_u", ctypes.c_float), ("max_u", ctypes.c_float),
                ("min_rho", ctypes.c_float), ("max_rho", ctypes.c_float)]


# constants of lbgb300.h
LB_OK, LB_ERR_ARG, LB_ERR_CUDA, LB_ERR_STATE, LB_ERR_NOMEM, LB_ERR_DEVICE = 0, -1, -2, -3, -4, -5
LB_ERR_IO = -6
LB_D2Q9, LB_D3Q19 = 9, 19
LB_MODE_REFERENCE, LB_MODE_NATIVE = 0, 1
LB_STORE_F32, LB_STORE_F16, LB_STORE_BF16 = 0, 1, 2
LB_PSI_REF, LB_PSI_EXP1 = 0, 1
LB_CELL_FLUID, LB_CELL_WALL, LB_CELL_MOVING = 0, 1, 2
LB_ABI_STANDALONE, LB_ABI_FUSED = 0, 1
LB_TUNE_DEFAULT, LB_TUNE_EXPLICIT, LB_TUNE_REVERSE = 0, 0x100, 0x001
LB_TUNE_PDL = 0x008
LB_TUNE_TBLOCK = 0x020
LB_TUNE_SC_STAGED = 0x040
LB_TUNE_SC_NO_TMA = 0x080


def LB_TUNE_TBLOCK_SHAPE(n):
    return n << 12


_c = ctypes
# (name, restype, argtypes) of every exported C symbol declared in include/lbgb300.h
PROTOTYPES = [
    ("streaming_d2q9", None, [_c.POINTER(DataD2Q9), dim3, dim3]),
    ("streaming_d3q19", None, [_c.POINTER(DataD3Q19), dim3, dim3]),
    ("collision_d2q9", None, [_c.c_void_p, _c.POINTER(DataD2Q9)] + [_c.c_float] * 11
     + [dim3, dim3] + [_c.c_float] * 4),
    ("collision_d3q19", None, [_c.c_void_p, _c.POINTER(DataD3Q19)] + [_c.c_float] * 12
     + [dim3, dim3]),
    ("get_border_d2q9", None, [_c.POINTER(DataD2Q9), dim3, dim3]),
    ("get_border_d3q19", None, [_c.POINTER(DataD3Q19), dim3, dim3]),
    ("apply_border_d2q9", None, [_c.POINTER(DataD2Q9), dim3, dim3]),
    ("apply_border_d3q19", None, [_c.POINTER(DataD3Q19), dim3, dim3]),
    ("read_value_2d", None, [_c.c_void_p, _c.POINTER(DataD2Q9), _c.c_int, _c.c_int, _c.c_int]),
    ("read_value_3d", None, [_c.c_void_p, _c.POINTER(DataD3Q19), _c.c_int, _c.c_int, _c.c_int]),
    ("copy_border_devices_d2q9", None, [_c.c_void_p] * 12 + [_c.c_int, _c.c_void_p]),
    ("lb_copy_border_devices_d3q19", None, [_c.c_void_p, _c.c_void_p, _c.c_int, _c.c_int,
                                            _c.c_void_p]),
    ("lb_abi_set_mode", _c.c_int, [_c.c_int]),
    ("lb_abi_get_mode", _c.c_int, []),
    ("lb_abi_release_d2q9", _c.c_int, [_c.POINTER(DataD2Q9)]),
    ("lb_abi_release_d3q19", _c.c_int, [_c.POINTER(DataD3Q19)]),
    ("lb_reduce_d2q9", _c.c_int, [_c.POINTER(DataD2Q9), _c.POINTER(_c.c_double)]),
    ("lb_reduce_d3q19", _c.c_int, [_c.POINTER(DataD3Q19), _c.POINTER(_c.c_double)]),
    ("lb_reduce_d3q19_noalloc", _c.c_int, [_c.POINTER(DataD3Q19), _c.POINTER(_c.c_double)]),
    ("lb_run_lbm_d3q19", _c.c_int, [_c.POINTER(DataD3Q19), _c.c_void_p,
                                    _c.POINTER(lb_run_params_d3q19), _c.c_int, _c.c_void_p]),
    ("lb_abi_last_error", _c.c_char_p, []),
    ("lb_abi_clear_error", _c.c_int, []),
    ("lb_config_default", _c.c_int, [_c.POINTER(lb_config), _c.c_int, _c.c_int, _c.c_int,
                                     _c.c_int]),
    ("lb_create", _c.c_int, [_c.POINTER(lb_config), _c.POINTER(_c.c_void_p)]),
    ("lb_destroy", _c.c_int, [_c.c_void_p]),
    ("lb_error", _c.c_char_p, [_c.c_void_p]),
    ("lb_set_flags", _c.c_int, [_c.c_void_p, _c.c_void_p]),
    ("lb_set_populations", _c.c_int, [_c.c_void_p, _c.c_void_p]),
    ("lb_get_populations", _c.c_int, [_c.c_void_p, _c.c_void_p]),
    ("lb_init_equilibrium", _c.c_int, [_c.c_void_p] * 5),
    ("lb_step", _c.c_int, [_c.c_void_p, _c.c_int]),
    ("lb_get_moments", _c.c_int, [_c.c_void_p] * 5),
    ("lb_reduce", _c.c_int, [_c.c_void_p, _c.POINTER(_c.c_double)]),
    ("lb_synchronize", _c.c_int, [_c.c_void_p]),
    ("lb_probe", _c.c_int, [_c.c_void_p, _c.c_int, _c.c_int, _c.c_int, _c.c_void_p]),
    ("lb_run_probe", _c.c_int, [_c.c_void_p, _c.c_int, _c.c_int, _c.c_int, _c.c_int,
                                _c.c_void_p]),
    ("lb_time_steps", _c.c_int, [_c.c_void_p, _c.c_int, _c.POINTER(_c.c_float)]),
    ("lb_launch_count", _c.c_int64, [_c.c_void_p]),
    ("lb_wall_correction", _c.c_int, [_c.c_void_p, _c.c_void_p]),
    ("lb_ensemble_create", _c.c_int, [_c.c_int, _c.c_void_p, _c.c_void_p, _c.c_void_p,
                                      _c.c_void_p, _c.c_int, _c.POINTER(_c.c_void_p)]),
    ("lb_ensemble_destroy", _c.c_int, [_c.c_void_p]),
    ("lb_ensemble_error", _c.c_char_p, [_c.c_void_p]),
    ("lb_ensemble_nodes", _c.c_long, [_c.c_void_p]),
    ("lb_ensemble_offset", _c.c_long, [_c.c_void_p, _c.c_int]),
    ("lb_ensemble_set_populations", _c.c_int, [_c.c_void_p, _c.c_void_p]),
    ("lb_ensemble_get_populations", _c.c_int, [_c.c_void_p, _c.c_void_p]),
    ("lb_ensemble_init_equilibrium", _c.c_int, [_c.c_void_p, _c.c_void_p]),
    ("lb_ensemble_step", _c.c_int, [_c.c_void_p, _c.c_int]),
    ("lb_ensemble_time_steps", _c.c_int, [_c.c_void_p, _c.c_int, _c.POINTER(_c.c_float)]),
    ("lb_ensemble_get_moments", _c.c_int, [_c.c_void_p] * 4),
    ("lb_ensemble_set_launch", _c.c_int, [_c.c_void_p, _c.c_int, _c.c_int, _c.c_int]),
    ("lb_ensemble_get_launch", _c.c_int, [_c.c_void_p, _c.c_void_p]),
    ("lb_ensemble_autotune", _c.c_int, [_c.c_void_p, _c.c_int, _c.c_void_p]),
    ("lb_ensemble_launch_count", _c.c_int64, [_c.c_void_p]),
    ("lb_mlp_create", _c.c_int, [_c.c_uint64, _c.POINTER(_c.c_void_p)]),
    ("lb_mlp_destroy", _c.c_int, [_c.c_void_p]),
    ("lb_mlp_error", _c.c_char_p, [_c.c_void_p]),
    ("lb_mlp_num_params", _c.c_int, []),
    ("lb_mlp_set_params", _c.c_int, [_c.c_void_p, _c.c_void_p]),
    ("lb_mlp_get_params", _c.c_int, [_c.c_void_p, _c.c_void_p]),
    ("lb_mlp_forward", _c.c_int, [_c.c_void_p, _c.c_void_p, _c.c_void_p, _c.c_long]),
    ("lb_mlp_grad", _c.c_int, [_c.c_void_p, _c.c_void_p, _c.c_void_p, _c.c_long, _c.c_void_p,
                               _c.POINTER(_c.c_double)]),
    ("lb_mlp_train", _c.c_int, [_c.c_void_p, _c.c_void_p, _c.c_void_p, _c.c_long, _c.c_int,
                                _c.c_int, _c.c_float, _c.c_uint64, _c.c_void_p]),
    ("lb_closure_enable", _c.c_int, [_c.c_void_p, _c.c_void_p, _c.c_float, _c.c_float,
                                     _c.c_float, _c.c_void_p]),
    ("lb_closure_sample", _c.c_int, [_c.c_void_p, _c.c_int, _c.c_float, _c.c_float, _c.c_float,
                                     _c.c_void_p, _c.c_void_p, _c.POINTER(_c.c_double)]),
    ("lb_closure_sample_avg", _c.c_int, [_c.c_void_p, _c.c_int, _c.c_float, _c.c_float,
                                         _c.c_float, _c.c_int, _c.c_void_p, _c.c_void_p,
                                         _c.POINTER(_c.c_double)]),
    ("lb_device_fields", _c.c_int, [_c.c_void_p] + [_c.POINTER(_c.c_void_p)] * 4),
    ("lb_extents", _c.c_int, [_c.c_void_p] + [_c.POINTER(_c.c_int)] * 3),
    ("lb_tcgen05_selftest", _c.c_int, [_c.c_void_p, _c.POINTER(_c.c_int)]),
    ("lb_wait_selftest", _c.c_int, [_c.c_int, _c.POINTER(_c.c_int)]),
    ("lb_case_load_parameters", _c.c_int, [_c.c_char_p, _c.POINTER(lb_case_params)]),
    ("lb_case_load_solids_bmp", _c.c_int, [_c.c_char_p, _c.POINTER(_c.c_int),
                                           _c.POINTER(_c.c_int), _c.c_void_p, _c.c_size_t]),
    ("lb_stl_read", _c.c_int, [_c.c_char_p, _c.POINTER(_c.c_int64), _c.c_void_p, _c.c_size_t]),
    ("lb_voxelize", _c.c_int, [_c.c_void_p, _c.c_int64, _c.c_int, _c.POINTER(_c.c_int),
                               _c.c_void_p, _c.c_size_t, _c.POINTER(_c.c_int)]),
    ("lb_case_load_solids_stl", _c.c_int, [_c.c_char_p, _c.c_int] + [_c.POINTER(_c.c_int)] * 3
     + [_c.c_void_p, _c.c_size_t]),
    ("lb_case_init_d2q9", _c.c_int, [_c.POINTER(lb_case_params), _c.c_int, _c.c_int]
     + [_c.c_void_p] * 9),
    ("lb_case_init_d3q19", _c.c_int, [_c.POINTER(lb_case_params), _c.c_int, _c.c_int, _c.c_int]
     + [_c.c_void_p] * 7),
    ("lb_vtk_save", _c.c_int, [_c.c_char_p] + [_c.c_int] * 5 + [_c.c_void_p] * 4),
    ("lb_vtk_save_parallel", _c.c_int, [_c.c_char_p] + [_c.c_int] * 5),
    ("lb_vtk_save_ctx", _c.c_int, [_c.c_void_p, _c.c_char_p, _c.c_int]),
    ("lb_checkpoint_save", _c.c_int, [_c.c_void_p, _c.c_char_p]),
    ("lb_checkpoint_load", _c.c_int, [_c.c_void_p, _c.c_char_p]),
    ("lb_checkpoint_create", _c.c_int, [_c.c_char_p, _c.POINTER(_c.c_void_p)]),
    ("lb_checkpoint_info", _c.c_int, [_c.c_char_p, _c.POINTER(lb_config),
                                      _c.POINTER(_c.c_int64)]),
    ("lb_steps_done", _c.c_int64, [_c.c_void_p]),
    ("lb_slab_create", _c.c_int, [_c.POINTER(lb_config), _c.c_int, _c.c_int,
                                  _c.POINTER(_c.c_void_p)]),
    ("lb_slab_info", _c.c_int, [_c.c_void_p] + [_c.POINTER(_c.c_int)] * 3
     + [_c.POINTER(_c.c_size_t)]),
    ("lb_stream", _c.c_void_p, [_c.c_void_p]),
    ("lb_slab_pack", _c.c_int, [_c.c_void_p, _c.c_void_p, _c.c_void_p]),
    ("lb_slab_step", _c.c_int, [_c.c_void_p, _c.c_int, _c.c_void_p, _c.c_void_p]),
    ("lb_slab_unpack", _c.c_int, [_c.c_void_p, _c.c_void_p, _c.c_void_p]),
    ("lb_slab_group_step", _c.c_int, [_c.POINTER(_c.c_void_p), _c.c_int, _c.c_int]),
    ("lb_slab_group_time", _c.c_int, [_c.POINTER(_c.c_void_p), _c.c_int, _c.c_int,
                                      _c.POINTER(_c.c_float)]),
    ("lb_device_count", _c.c_int, [_c.POINTER(_c.c_int)]),
    ("lb_set_device", _c.c_int, [_c.c_int]),
    ("lb_malloc", _c.c_int, [_c.POINTER(_c.c_void_p), _c.c_size_t]),
    ("lb_free", _c.c_int, [_c.c_void_p]),
    ("lb_malloc_host", _c.c_int, [_c.POINTER(_c.c_void_p), _c.c_size_t]),
    ("lb_free_host", _c.c_int, [_c.c_void_p]),
    ("lb_memcpy_h2d", _c.c_int, [_c.c_void_p, _c.c_void_p, _c.c_size_t]),
    ("lb_memcpy_d2h", _c.c_int, [_c.c_void_p, _c.c_void_p, _c.c_size_t]),
    ("lb_memset", _c.c_int, [_c.c_void_p, _c.c_int, _c.c_size_t]),
    ("lb_device_synchronize", _c.c_int, []),
    ("lb_version", _c.c_char_p, []),
]

# the reference's C++-linkage copy_border_devices_d3q19 (Itanium mangling of
# void(float* x20, int, int, CUstream_st*&))
CXX_SYMBOLS = ["_Z25copy_border_devices_d3q19PfS_S_S_S_S_S_S_S_S_S_S_S_S_S_S_S_S_S_S_iiRP11CUstream_st"]


def load(path=LIB_PATH):
    """Load liblbgb300.so and attach prototypes.  Raises if it is missing:
    there is no CPU fallback."""
    if not os.path.exists(path):
        raise RuntimeError("liblbgb300.so not built (%s); run __graft_entry__.build()" % path)
    lib = ctypes.CDLL(path)
    for name, res, args in PROTOTYPES:
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    return lib
