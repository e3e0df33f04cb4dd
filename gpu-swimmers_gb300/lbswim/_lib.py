"""ctypes binding of liblbswim's C ABI (include/lbswim_c.h).

The shared library is built in-tree by gpu-swimmers_gb300/build.py.  There is
no fallback: if the library is missing or cannot be loaded, importing lbswim
raises ImportError.
"""
import ctypes as C
import os

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "_liblbswim.so")

F64, F32, BF16, F16 = 0, 1, 2, 3
PRECISIONS = {"f64": F64, "float64": F64, "double": F64, "f32": F32, "float32": F32,
              "float": F32, "bf16": BF16, "bfloat16": BF16, "f16": F16, "float16": F16,
              "half": F16}
PRECISION_NAMES = {F64: "f64", F32: "f32", BF16: "bf16", F16: "f16"}

FIELD_RHO, FIELD_U, FIELD_FORCE, FIELD_FOLD, FIELD_FNEW = range(5)
FIELD_COMPONENTS = {FIELD_RHO: 1, FIELD_U: 3, FIELD_FORCE: 3, FIELD_FOLD: 15, FIELD_FNEW: 15}
SW_R, SW_V, SW_N = 0, 1, 2
TR_R, TR_S, TR_V = 0, 1, 2
COMPAT_INIT_SXZ, COMPAT_SYNC_STEP, COMPAT_EXACT_F64, COMPAT_WIDE_INDEX = 1, 2, 4, 8
COMPAT_EAGER_FIELDS, COMPAT_BULK_COPY = 16, 32
STATUS_NONFINITE, STATUS_PARTICLE_OUTSIDE, STATUS_COPY_TIMEOUT = 1, 2, 4

ERRORS = {-1: "invalid argument", -2: "CUDA error", -3: "out of memory", -4: "invalid state",
          -5: "not supported"}


class LbswimError(RuntimeError):
    def __init__(self, code, message):
        super().__init__("%s (%d): %s" % (ERRORS.get(code, "error"), code, message))
        self.code = code


class LBParamsStruct(C.Structure):
    _fields_ = [("cs2", C.c_double), ("w", C.c_double * 15), ("xi", (C.c_double * 3) * 15),
                ("ci", (C.c_int * 3) * 15), ("Q", ((C.c_double * 3) * 3) * 15),
                ("complement", C.c_int * 15), ("norms", C.c_double * 15),
                ("mm", (C.c_double * 15) * 15), ("mmi", (C.c_double * 15) * 15),
                ("tau_s", C.c_double), ("tau_b", C.c_double)]


class AddressingStruct(C.Structure):
    _fields_ = [("size", C.c_int * 3), ("strides", C.c_int * 3), ("n", C.c_int)]


class CommonParamsStruct(C.Structure):
    _fields_ = [("P", C.c_double), ("l", C.c_double), ("alpha", C.c_double),
                ("mobility", C.c_double), ("translational_advection_off", C.c_int),
                ("rotational_advection_off", C.c_int), ("seed", C.c_ulonglong)]


_VP = C.c_void_p
_D = C.POINTER(C.c_double)

_PROTOS = {
    "lbswim_last_error": (C.c_char_p, []),
    "lbswim_version": (C.c_char_p, []),
    "lbswim_kernel_launches": (C.c_int, [C.POINTER(C.c_ulonglong)]),
    "lbswim_host_alloc": (C.c_int, [C.c_size_t, C.POINTER(_VP)]),
    "lbswim_host_free": (C.c_int, [_VP]),
    "lbswim_lattice_create": (C.c_int, [C.c_int, C.c_int, C.c_int, C.c_double, C.c_double,
                                        C.c_int, C.POINTER(_VP)]),
    "lbswim_lattice_destroy": (C.c_int, [_VP]),
    "lbswim_lattice_step": (C.c_int, [_VP]),
    "lbswim_lattice_calc_hydro": (C.c_int, [_VP]),
    "lbswim_lattice_init_from_hydro": (C.c_int, [_VP]),
    "lbswim_lattice_zero_force": (C.c_int, [_VP]),
    "lbswim_lattice_h2d": (C.c_int, [_VP, C.c_int, _D]),
    "lbswim_lattice_d2h": (C.c_int, [_VP, C.c_int, _D]),
    "lbswim_lattice_get_params": (C.c_int, [_VP, C.POINTER(LBParamsStruct)]),
    "lbswim_lattice_get_addressing": (C.c_int, [_VP, C.POINTER(AddressingStruct)]),
    "lbswim_lattice_get_time_step": (C.c_int, [_VP, C.POINTER(C.c_int)]),
    "lbswim_lattice_set_time_step": (C.c_int, [_VP, C.c_int]),
    "lbswim_lattice_get_precision": (C.c_int, [_VP, C.POINTER(C.c_int)]),
    "lbswim_lattice_set_compat": (C.c_int, [_VP, C.c_int]),
    "lbswim_lattice_set_stream": (C.c_int, [_VP, _VP]),
    "lbswim_lattice_synchronize": (C.c_int, [_VP]),
    "lbswim_lattice_join": (C.c_int, [_VP]),
    "lbswim_lattice_get_tile": (C.c_int, [_VP, C.POINTER(C.c_int)]),
    "lbswim_lattice_conservation": (C.c_int, [_VP, _D]),
    "lbswim_lattice_get_rho0": (C.c_int, [_VP, _D]),
    "lbswim_lattice_init_random": (C.c_int, [_VP, C.c_ulonglong, C.c_double]),
    "lbswim_swimmers_init_random": (C.c_int, [_VP, _VP, C.c_ulonglong]),
    "lbswim_tracers_init_random": (C.c_int, [_VP, _VP, C.c_ulonglong]),
    "lbswim_lattice_set_tau": (C.c_int, [_VP, C.c_double, C.c_double]),
    "lbswim_lattice_set_tile": (C.c_int, [_VP, C.c_int]),
    "lbswim_ensemble_create": (C.c_int, [C.POINTER(_VP)]),
    "lbswim_ensemble_destroy": (C.c_int, [_VP]),
    "lbswim_ensemble_set_members": (C.c_int, [_VP, C.POINTER(_VP), C.POINTER(_VP),
                                              C.POINTER(_VP), C.c_int]),
    "lbswim_ensemble_step": (C.c_int, [_VP, C.c_int]),
    "lbswim_ensemble_step_limited": (C.c_int, [_VP, C.c_int, C.POINTER(C.c_int)]),
    "lbswim_ensemble_autotune": (C.c_int, [_VP]),
    "lbswim_lattice_device_ptr": (C.c_int, [_VP, C.c_int, C.POINTER(_VP), C.POINTER(C.c_int)]),
    "lbswim_lattice_set_timing": (C.c_int, [_VP, C.c_int]),
    "lbswim_lattice_get_timing": (C.c_int, [_VP, C.POINTER(C.c_double), C.POINTER(C.c_int)]),
    "lbswim_swimmers_create": (C.c_int, [C.c_int, C.POINTER(CommonParamsStruct), C.POINTER(_VP)]),
    "lbswim_swimmers_destroy": (C.c_int, [_VP]),
    "lbswim_swimmers_set_common": (C.c_int, [_VP, C.POINTER(CommonParamsStruct)]),
    "lbswim_swimmers_get_common": (C.c_int, [_VP, C.POINTER(CommonParamsStruct)]),
    "lbswim_swimmers_get_num": (C.c_int, [_VP, C.POINTER(C.c_int)]),
    "lbswim_swimmers_add_forces": (C.c_int, [_VP, _VP]),
    "lbswim_swimmers_move": (C.c_int, [_VP, _VP]),
    "lbswim_swimmers_h2d": (C.c_int, [_VP, C.c_int, _D]),
    "lbswim_swimmers_d2h": (C.c_int, [_VP, C.c_int, _D]),
    "lbswim_swimmers_d2h_all": (C.c_int, [_VP, _D, _D, _D]),
    "lbswim_swimmers_get_rng": (C.c_int, [_VP, C.POINTER(C.c_ulonglong), C.POINTER(C.c_ulonglong)]),
    "lbswim_swimmers_set_rng": (C.c_int, [_VP, C.c_ulonglong, C.c_ulonglong]),
    "lbswim_lattice_interp_velocity": (C.c_int, [_VP, C.c_int, _D, _D]),
    "lbswim_rng_draws": (C.c_int, [C.c_ulonglong, C.c_int, C.c_ulonglong,
                                   C.POINTER(C.c_float), _D]),
    "lbswim_spread_forces_noalloc": (C.c_int, [_VP, _VP, C.c_int, C.c_double, C.c_double,
                                               C.c_int, C.c_int, C.c_int, _VP, C.c_int, _VP]),
    "lbswim_tracers_create": (C.c_int, [C.c_int, C.POINTER(_VP)]),
    "lbswim_tracers_destroy": (C.c_int, [_VP]),
    "lbswim_tracers_get_num": (C.c_int, [_VP, C.POINTER(C.c_int)]),
    "lbswim_tracers_move": (C.c_int, [_VP, _VP]),
    "lbswim_tracers_h2d": (C.c_int, [_VP, C.c_int, _D]),
    "lbswim_tracers_d2h": (C.c_int, [_VP, C.c_int, _D]),
    "lbswim_system_step": (C.c_int, [_VP, C.POINTER(_VP), C.c_int, C.POINTER(_VP), C.c_int,
                                     C.c_int]),
    "lbswim_lattice_get_status": (C.c_int, [_VP, C.POINTER(C.c_uint), C.c_int]),
    "lbswim_device_alloc": (C.c_int, [C.c_size_t, C.POINTER(_VP)]),
    "lbswim_device_free": (C.c_int, [_VP]),
    "lbswim_memcpy_h2d": (C.c_int, [_VP, _VP, C.c_size_t]),
    "lbswim_memcpy_d2h": (C.c_int, [_VP, _VP, C.c_size_t]),
    "lbswim_lbparams_fill": (C.c_int, [C.POINTER(LBParamsStruct)]),
    "lbswim_lattice_device_buffers": (C.c_int, [_VP, C.POINTER(_VP)]),
    "lbswim_swimmers_device_ptr": (C.c_int, [_VP, C.c_int, C.POINTER(_VP)]),
    "lbswim_tracers_device_ptr": (C.c_int, [_VP, C.c_int, C.POINTER(_VP)]),
}


def _load():
    if not os.path.exists(LIB_PATH):
        raise ImportError("liblbswim is not built (%s missing); run "
                          "`python gpu-swimmers_gb300/build.py`" % LIB_PATH)
    lib = C.CDLL(LIB_PATH)
    for name, (res, args) in _PROTOS.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    return lib


lib = _load()


def check(status):
    if status != 0:
        msg = lib.lbswim_last_error()
        raise LbswimError(status, msg.decode() if msg else "")
    return status


def dptr(a):
    """Pointer to the data of a C-contiguous float64 numpy array."""
    if a.dtype.char != "d" or not a.flags.c_contiguous:
        raise TypeError("expected a C-contiguous float64 array")
    return a.ctypes.data_as(_D)


class _PinnedBlock:
    """Page-locked host memory from lbswim_host_alloc, freed with the block."""

    def __init__(self, nbytes):
        self.ptr = _VP()
        check(lib.lbswim_host_alloc(max(int(nbytes), 8), C.byref(self.ptr)))

    def __del__(self):
        ptr, self.ptr = getattr(self, "ptr", None), None
        if ptr and lib is not None:
            try:
                lib.lbswim_host_free(ptr)
            except Exception:
                pass


def pinned_zeros(n):
    """A zeroed float64 numpy array of n elements in page-locked host memory.
    The memory lives as long as any array or view made from it."""
    n = int(n)
    block = _PinnedBlock(8 * n)
    cbuf = (C.c_double * max(n, 1)).from_address(block.ptr.value)
    cbuf._block = block  # views of the array keep cbuf, and cbuf the block
    a = np.ctypeslib.as_array(cbuf)[:n]
    a[:] = 0.0
    return a


def kernel_launches():
    out = C.c_ulonglong()
    check(lib.lbswim_kernel_launches(C.byref(out)))
    return out.value


def rng_draws(seed, n, step):
    """Device-side draws of the swimmer random stream: (uniform[n], normal[3, n])."""
    import numpy as np
    u = np.zeros(n, dtype=np.float32)
    g = np.zeros((3, n), dtype=np.float64)
    check(lib.lbswim_rng_draws(int(seed), int(n), int(step),
                               u.ctypes.data_as(C.POINTER(C.c_float)), dptr(g)))
    return u, g


def version():
    return lib.lbswim_version().decode()
