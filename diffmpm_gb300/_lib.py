"""ctypes binding of ``libdiffmpm_gb300.so`` (the C ABI in include/diffmpm_gb300.h).

The library must exist (``python -m diffmpm_gb300.build`` or
``__graft_entry__.build()``); importing this module without it raises, and there
is no CPU fallback.
"""
from __future__ import annotations

import ctypes as C
from pathlib import Path

import numpy as np

LIB_PATH = Path(__file__).resolve().parent / "libdiffmpm_gb300.so"

MPM_OK = 0
STATUS_NAMES = {
    1: "MPM_ERR_INVALID", 2: "MPM_ERR_CUDA", 3: "MPM_ERR_OUT_OF_MESH", 4: "MPM_ERR_CFL",
    5: "MPM_ERR_UNSUPPORTED", 6: "MPM_ERR_STATE", 7: "MPM_ERR_NOMEM",
}

LINEAR_ELASTIC, SIMPLE, NEWTONIAN = 0, 1, 2
USF, USL = 0, 1

FIELD = {
    "loc": 0, "velocity": 1, "stress": 2, "strain": 3, "density": 4, "volume": 5,
    "mass": 6, "volumetric_strain_centroid": 7, "material_id": 8, "youngs_modulus": 9,
    "element_ids": 10, "momentum": 11,
}
NODAL_FIELD = {"mass": 0, "velocity": 1, "acceleration": 2, "momentum": 3}
PHASE = {"nodal_kinematics": 0, "forces": 1, "particle_kinematics": 2}


class MpmError(RuntimeError):
    """A non-zero MpmStatus from the library."""

    def __init__(self, code, message):
        super().__init__(f"{STATUS_NAMES.get(code, code)}: {message}")
        self.code = code


class OutOfMeshError(MpmError, ValueError):
    pass


class MpmMaterial(C.Structure):
    _fields_ = [("type", C.c_int), ("density", C.c_double), ("youngs_modulus", C.c_double),
                ("poisson_ratio", C.c_double), ("E", C.c_double), ("bulk_modulus", C.c_double),
                ("dynamic_viscosity", C.c_double)]


class MpmDesc(C.Structure):
    _fields_ = [
        ("ndim", C.c_int), ("nelements", C.c_int * 2), ("el_len", C.c_double * 2),
        ("scheme", C.c_int), ("velocity_update", C.c_int), ("reinit_each_step", C.c_int),
        ("dt", C.c_double), ("gravity", C.c_double * 2),
        ("n_constraints", C.c_int), ("constraint_node", C.POINTER(C.c_int32)),
        ("constraint_dir", C.POINTER(C.c_int32)), ("constraint_velocity", C.POINTER(C.c_double)),
        ("n_functions", C.c_int), ("function_npoints", C.POINTER(C.c_int32)),
        ("function_x", C.POINTER(C.c_double)), ("function_y", C.POINTER(C.c_double)),
        ("n_nodal_forces", C.c_int), ("nodal_force_node", C.POINTER(C.c_int32)),
        ("nodal_force_dir", C.POINTER(C.c_int32)), ("nodal_force_value", C.POINTER(C.c_double)),
        ("nodal_force_function", C.POINTER(C.c_int32)),
        ("n_materials", C.c_int), ("materials", C.POINTER(MpmMaterial)),
    ]


class MpmTuning(C.Structure):
    _fields_ = [("block_steps", C.c_int32), ("resort_every", C.c_int32), ("nk_ctas", C.c_int32),
                ("g2p_ctas", C.c_int32), ("forces_lpc", C.c_int32), ("ms_per_step", C.c_float)]


# (name, restype, argtypes) of every exported entry point
_VP = C.c_void_p
SIGNATURES = [
    ("mpm_abi_version", C.c_int, []),
    ("mpm_create", C.c_int, [C.POINTER(MpmDesc), C.POINTER(_VP)]),
    ("mpm_destroy", C.c_int, [_VP]),
    ("mpm_last_error", C.c_char_p, [_VP]),
    ("mpm_set_particles", C.c_int, [_VP, C.c_int64, _VP, _VP, C.c_int, _VP]),
    ("mpm_write_field", C.c_int, [_VP, C.c_int, _VP, C.c_int, _VP]),
    ("mpm_read_field", C.c_int, [_VP, C.c_int, _VP, C.c_int, _VP]),
    ("mpm_output_enqueue", C.c_int, [_VP, C.c_int, _VP, _VP, C.c_size_t, _VP, C.POINTER(C.c_int64)]),
    ("mpm_output_wait", C.c_int, [_VP, C.c_int64]),
    ("mpm_host_alloc", C.c_int, [C.c_size_t, C.POINTER(_VP)]),
    ("mpm_host_free", C.c_int, [_VP]),
    ("mpm_set_tractions", C.c_int, [_VP, C.c_int, _VP, _VP, _VP, _VP, _VP]),
    ("mpm_set_particle_velocity_constraints", C.c_int, [_VP, C.c_int, _VP, _VP, _VP, _VP]),
    ("mpm_read_nodal_field", C.c_int, [_VP, C.c_int, _VP, C.c_int, _VP]),
    ("mpm_write_nodal_field", C.c_int, [_VP, C.c_int, _VP, C.c_int, _VP]),
    ("mpm_initialize", C.c_int, [_VP, _VP]),
    ("mpm_step", C.c_int, [_VP, C.c_int, _VP]),
    ("mpm_get_step", C.c_int, [_VP, C.POINTER(C.c_int64)]),
    ("mpm_set_step", C.c_int, [_VP, C.c_int64]),
    ("mpm_run_phase", C.c_int, [_VP, C.c_int, _VP]),
    ("mpm_time_phases", C.c_int, [_VP, C.c_int, _VP, _VP]),
    ("mpm_set_block_steps", C.c_int, [_VP, C.c_int]),
    ("mpm_set_kernel_variant", C.c_int, [_VP, C.c_int, C.c_int, C.c_int]),
    ("mpm_set_empty_split", C.c_int, [_VP, C.c_int]),
    ("mpm_device_name", C.c_int, [C.c_int, C.c_char_p, C.c_int]),
    ("mpm_get_counters", C.c_int, [_VP, C.POINTER(C.c_int64), C.POINTER(C.c_int64)]),
    ("mpm_set_gravity", C.c_int, [_VP, C.c_double, C.c_double]),
    ("mpm_record", C.c_int, [_VP, C.c_int, C.c_int, _VP]),
    ("mpm_adjoint", C.c_int, [_VP, _VP, _VP, _VP, _VP, _VP, C.c_int, _VP]),
    ("mpm_batch_create", C.c_int, [C.POINTER(_VP), C.c_int, C.POINTER(_VP)]),
    ("mpm_batch_destroy", C.c_int, [_VP]),
    ("mpm_batch_last_error", C.c_char_p, [_VP]),
    ("mpm_batch_size", C.c_int, [_VP, C.POINTER(C.c_int), C.POINTER(C.c_int)]),
    ("mpm_batch_step", C.c_int, [_VP, C.c_int, _VP]),
    ("mpm_batch_write_field", C.c_int, [_VP, C.c_int, _VP, C.c_int, _VP]),
    ("mpm_batch_read_field", C.c_int, [_VP, C.c_int, _VP, C.c_int, _VP]),
    ("mpm_batch_write_nodal_field", C.c_int, [_VP, C.c_int, _VP, C.c_int, _VP]),
    ("mpm_batch_restart", C.c_int, [_VP, _VP]),
    ("mpm_batch_set_block_steps", C.c_int, [_VP, C.c_int]),
    ("mpm_batch_autotune", C.c_int, [_VP, C.c_int, C.POINTER(MpmTuning), _VP]),
    ("mpm_batch_set_tuning", C.c_int, [_VP, C.POINTER(MpmTuning)]),
    ("mpm_batch_get_tuning", C.c_int, [_VP, C.POINTER(MpmTuning)]),
    ("mpm_batch_record", C.c_int, [_VP, C.c_int, C.c_int, _VP]),
    ("mpm_batch_adjoint", C.c_int, [_VP, C.POINTER(_VP), C.POINTER(_VP), C.POINTER(_VP),
                                    C.POINTER(_VP), C.POINTER(_VP), C.c_int, _VP]),
    ("mpm_volume_setup_noalloc", C.c_int, [C.c_int, C.c_int, C.c_double, C.c_double, C.c_int64,
                                           _VP, _VP, _VP, _VP, _VP, _VP]),
]

_lib = None


def load():
    """Load the shared library (raises if it was not built)."""
    global _lib
    if _lib is None:
        if not LIB_PATH.exists():
            raise ImportError(
                f"{LIB_PATH.name} is missing: build it with __graft_entry__.build() or "
                "python -m diffmpm_gb300.build (there is no CPU fallback)")
        lib = C.CDLL(str(LIB_PATH))
        for name, res, args in SIGNATURES:
            fn = getattr(lib, name)
            fn.restype = res
            fn.argtypes = args
        _lib = lib
    return _lib


def check(code, handle=None):
    if code != MPM_OK:
        msg = load().mpm_last_error(handle).decode(errors="replace")
        if code == 3:
            raise OutOfMeshError(code, msg)
        raise MpmError(code, msg)


def check_batch(code, batch=None):
    if code != MPM_OK:
        msg = load().mpm_batch_last_error(batch).decode(errors="replace")
        if code == 3:
            raise OutOfMeshError(code, msg)
        raise MpmError(code, msg)


def ptr(a):
    """Pointer of a contiguous numpy array (or None)."""
    if a is None:
        return None
    return a.ctypes.data_as(C.c_void_p)
